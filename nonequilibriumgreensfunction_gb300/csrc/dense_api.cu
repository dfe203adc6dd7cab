// Stateless dense entry points: the reference's ZGEMM calls and Invert_Matrix
// (Source/MKL_Routines_Cluster.F90:2-33) on host arrays, running on the current device.
#include <vector>

#include "engine.h"
#include "zgemm_tc.h"

namespace {

struct DevBuf {
  void* p = nullptr;
  ~DevBuf() { if (p) cudaFree(p); }
  int alloc(size_t bytes) { return cudaMalloc(&p, bytes) == cudaSuccess ? NEGF_OK : NEGF_ENOMEM; }
};

}  // namespace

extern "C" {

int negf_zgemm(int32_t slices, int32_t m, int32_t n, int32_t k, const double* alpha, const double* A, int32_t lda,
               const double* B, int32_t ldb, const double* beta, double* C, int32_t ldc, int32_t batch) {
  using namespace negf;
  if (m <= 0 || n <= 0 || k <= 0 || batch <= 0 || !alpha || !beta || !A || !B || !C) return NEGF_EINVAL;
  if (lda < m || ldb < k || ldc < m) return NEGF_EINVAL;
  if (slices != 0 && !tc_supported_slices(slices)) return NEGF_EINVAL;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return NEGF_ENODEV;
  const size_t sA = (size_t)lda * k, sB = (size_t)ldb * n, sC = (size_t)ldc * n;
  DevBuf dA, dB, dC, dErr;
  NEGF_TRY(dA.alloc(sizeof(double2) * sA * batch));
  NEGF_TRY(dB.alloc(sizeof(double2) * sB * batch));
  NEGF_TRY(dC.alloc(sizeof(double2) * sC * batch));
  NEGF_TRY(dErr.alloc(sizeof(int)));
  NEGF_CUDA_TRY(cudaMemcpy(dA.p, A, sizeof(double2) * sA * batch, cudaMemcpyHostToDevice));
  NEGF_CUDA_TRY(cudaMemcpy(dB.p, B, sizeof(double2) * sB * batch, cudaMemcpyHostToDevice));
  NEGF_CUDA_TRY(cudaMemcpy(dC.p, C, sizeof(double2) * sC * batch, cudaMemcpyHostToDevice));
  NEGF_CUDA_TRY(cudaMemset(dErr.p, 0, sizeof(int)));
  const double2 al = make_double2(alpha[0], alpha[1]), be = make_double2(beta[0], beta[1]);
  cudaStream_t st = 0;
  if (slices == 0) {
    GemmBatch g{};
    g.m = m; g.n = n; g.k = k; g.alpha = al; g.beta = be;
    g.A = (const double2*)dA.p; g.lda = lda; g.sA = (long long)sA; g.opA = OP_N;
    g.B = (const double2*)dB.p; g.ldb = ldb; g.sB = (long long)sB; g.opB = OP_N;
    g.C = (double2*)dC.p; g.ldc = ldc; g.sC = (long long)sC; g.batch = batch;
    NEGF_TRY(zgemm_f64(g, st));
  } else {
    const int kp = padded_k(k);
    DevBuf sa, sb, ea, fb;
    NEGF_TRY(sa.alloc(sliced_bytes_a(m, kp, slices, batch)));
    NEGF_TRY(sb.alloc(sliced_bytes_b(n, kp, slices, batch)));
    NEGF_TRY(ea.alloc(sizeof(int) * (size_t)m * batch));
    NEGF_TRY(fb.alloc(sizeof(int) * (size_t)n * batch));
    SlicedOperand oa, ob;
    oa.data = (__nv_bfloat16*)sa.p; oa.exps = (int*)ea.p;
    ob.data = (__nv_bfloat16*)sb.p; ob.exps = (int*)fb.p;
    oa.data_bytes = sliced_bytes_a(m, kp, slices, batch); oa.exps_count = (size_t)m * batch;
    ob.data_bytes = sliced_bytes_b(n, kp, slices, batch); ob.exps_count = (size_t)n * batch;
    NEGF_TRY(slice_a((const double2*)dA.p, lda, (long long)sA, m, k, batch, slices, oa, st));
    NEGF_TRY(slice_b((const double2*)dB.p, ldb, (long long)sB, k, n, batch, slices, ob, st));
    NEGF_TRY(zgemm_tc(oa, ob, al, be, (double2*)dC.p, ldc, (long long)sC, (int*)dErr.p, st));
  }
  NEGF_CUDA_TRY(cudaStreamSynchronize(st));
  int err = 0;
  NEGF_CUDA_TRY(cudaMemcpy(&err, dErr.p, sizeof(int), cudaMemcpyDeviceToHost));
  if (err) return NEGF_ETIMEDOUT;
  NEGF_CUDA_TRY(cudaMemcpy(C, dC.p, sizeof(double2) * sC * batch, cudaMemcpyDeviceToHost));
  return NEGF_OK;
}

int negf_zinv(int32_t n, const double* G, double* invG, int32_t batch) {
  using namespace negf;
  if (n <= 0 || batch <= 0 || !G || !invG) return NEGF_EINVAL;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return NEGF_ENODEV;
  const size_t nn = (size_t)n * n;
  DevBuf dA, dS;
  NEGF_TRY(dA.alloc(sizeof(double2) * nn * batch));
  NEGF_TRY(dS.alloc(sizeof(int) * batch));
  NEGF_CUDA_TRY(cudaMemcpy(dA.p, G, sizeof(double2) * nn * batch, cudaMemcpyHostToDevice));
  NEGF_CUDA_TRY(cudaMemset(dS.p, 0, sizeof(int) * batch));
  InvWork w;
  int st = inv_work_alloc(w, n, batch);
  if (st == NEGF_OK) st = zinv_f64((double2*)dA.p, (long long)nn, n, batch, w, 0);
  if (st == NEGF_OK) st = merge_info_kernel_launch(batch, w.info, (int*)dS.p, 0);
  std::vector<int> info(batch, 0);
  if (st == NEGF_OK && cudaDeviceSynchronize() != cudaSuccess) st = NEGF_ECUDA;
  if (st == NEGF_OK && cudaMemcpy(info.data(), dS.p, sizeof(int) * batch, cudaMemcpyDeviceToHost) != cudaSuccess)
    st = NEGF_ECUDA;
  if (st == NEGF_OK && cudaMemcpy(invG, dA.p, sizeof(double2) * nn * batch, cudaMemcpyDeviceToHost) != cudaSuccess)
    st = NEGF_ECUDA;
  inv_work_free(w);
  if (st != NEGF_OK) return st;
  for (int b = 0; b < batch; ++b)
    if (info[b]) return info[b];
  return NEGF_OK;
}

}  // extern "C"
