// Sliced-BF16 tensor-core complex GEMM (zgemm_tc.cu).
#pragma once

#include <cuda_bf16.h>

#include "negf_internal.cuh"

namespace negf {

// An operand cut into integer BF16 slices, K-major: for slice p of item b, `rows` rows of
// 2K BF16 values at data + ((b*slices + p)*rows + r)*2K, with one power-of-two exponent
// per row in exps[b*rows_logical + r] (rows_logical = rows for A, rows/2 for B).
struct SlicedOperand {
  __nv_bfloat16* data = nullptr;
  int* exps = nullptr;
  int rows = 0, k = 0, slices = 0, batch = 0;
  size_t data_bytes = 0;     // capacity of data; slice_a/slice_b refuse anything larger
  size_t exps_count = 0;     // capacity of exps (ints)
};

bool tc_supported_slices(int s);
// K padded to a multiple of 4 (TMA rows must be a multiple of 16 bytes)
int padded_k(int k);
// bytes of the slice planes for `rows` x K complex operands (A: rows = M; B: rows = 2N);
// pass padded_k(K)
size_t sliced_bytes(int rows, int k, int slices, int batch);
// A operand: M x K complex, column-major (lda, batch stride sA)
int slice_a(const double2* A, int lda, long long sA, int m, int k, int batch, int slices, SlicedOperand& out,
            cudaStream_t st);
// B operand: K x N complex, column-major
int slice_b(const double2* B, int ldb, long long sB, int k, int n, int batch, int slices, SlicedOperand& out,
            cudaStream_t st);
// C = alpha A B + beta C (C column-major, ldc, batch stride sC); err: optional device flag.
// slices = 0 uses every plane (A and B must have the same count); slices > 0 uses the
// leading `slices` planes of each operand, which may have been sliced finer.
int zgemm_tc(const SlicedOperand& A, const SlicedOperand& B, double2 alpha, double2 beta, double2* C, int ldc,
             long long sC, int* err, cudaStream_t st, int slices = 0);

}  // namespace negf
