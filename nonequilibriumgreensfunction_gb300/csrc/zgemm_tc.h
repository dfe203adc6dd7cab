// Sliced-BF16 tensor-core complex GEMM (zgemm_tc.cu).
#pragma once

#include <cuda_bf16.h>

#include "negf_internal.cuh"

namespace negf {

// An operand cut into integer BF16 slices, K-major: for slice p of item b, `rows` rows of
// 2K BF16 values at data + ((b*slices + p)*rows + r)*2K.  A (M x K complex) has rows = 2M:
// row 2i = [Ar(i,:), -Ai(i,:)], row 2i+1 = [Ai(i,:), Ar(i,:)]; B (K x N complex) has
// rows = N: row j = [Br(:,j), Bi(:,j)].  One power-of-two exponent per complex row of A
// (exps[b*M + i]) or column of B (exps[b*N + j]).
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
// bytes of the slice planes of `rows` K-major rows of 2K values; pass padded_k(K)
size_t sliced_bytes(int rows, int k, int slices, int batch);
// the same for an M x K complex A operand (2M rows) and a K x N complex B operand (N rows)
size_t sliced_bytes_a(int m, int k, int slices, int batch);
size_t sliced_bytes_b(int n, int k, int slices, int batch);
// A operand: M x K complex, column-major (lda, batch stride sA)
int slice_a(const double2* A, int lda, long long sA, int m, int k, int batch, int slices, SlicedOperand& out,
            cudaStream_t st);
// B operand: K x N complex, column-major
int slice_b(const double2* B, int ldb, long long sB, int k, int n, int batch, int slices, SlicedOperand& out,
            cudaStream_t st);
// C = alpha A B + beta C (C column-major, ldc, batch stride sC); err: optional device flag.
// slices = 0 uses every plane (A and B must have the same count); slices > 0 uses the
// leading `slices` planes of each operand, which may have been sliced finer.
// tune_c: optional scratch of ldc * n * batch complex values.  With it, the first call of a
// shape with beta != 0 is also tuned: the variants are timed with beta = 0 writing into the
// scratch (C itself is never touched by the timings), then the chosen one computes C.
int zgemm_tc(const SlicedOperand& A, const SlicedOperand& B, double2 alpha, double2 beta, double2* C, int ldc,
             long long sC, int* err, cudaStream_t st, int slices = 0, double2* tune_c = nullptr);

}  // namespace negf
