// Batched complex FP64 GEMM on the DFMA pipe.
//
// GB300 (sm_103) executes about two FP64 fused multiply-adds per clock per SM: cuBLAS
// ZGEMM measures 1.10 TFLOP/s on the whole part, and this kernel 1.00 TFLOP/s with its FP64
// pipe busy on 97.6% of its active cycles (ncu).  The FP64 form is therefore bound by that
// pipe, and this kernel only has to keep it busy: 64x64 complex output tiles, K steps of 8
// staged through double-buffered shared memory, 4x4 complex accumulators per thread
// (4 DFMA per complex multiply-add).  Replaces the ZGEMM calls of
// Source/Recursive_Greens.F90, Source/Contact_Self_Energy.F90 and the zgemm-equivalent
// loops of Source/Calculate_Gnp.F90 / Source/Calculate_Observables.F90.
#include "negf_internal.cuh"

namespace negf {

namespace {

constexpr int BM = 64, BN = 64, BK = 8, NT = 256;

template <int OP, typename T>
__device__ __forceinline__ T opval(T v) {
  if (OP == OP_C) return cconj(v);
  return v;
}

// op(A)(i, k) for column-major A
template <int OP, typename T>
__device__ __forceinline__ T load_a(const T* __restrict__ A, int lda, int m, int k, int i, int kk) {
  if (i >= m || kk >= k) return CplxTraits<T>::make(0, 0);
  if (OP == OP_N) return A[(long long)kk * lda + i];
  return opval<OP>(A[(long long)i * lda + kk]);
}
// op(B)(kk, j)
template <int OP, typename T>
__device__ __forceinline__ T load_b(const T* __restrict__ B, int ldb, int n, int k, int kk, int j) {
  if (j >= n || kk >= k) return CplxTraits<T>::make(0, 0);
  if (OP == OP_N) return B[(long long)j * ldb + kk];
  return opval<OP>(B[(long long)kk * ldb + j]);
}

template <int OPA, int OPB, typename T>
__global__ void __launch_bounds__(NT) zgemm_kernel(GemmBatchT<T> g) {
  __shared__ T As[2][BK][BM];
  __shared__ T Bs[2][BK][BN];
  const int b = blockIdx.z;
  const T* __restrict__ A = g.A + (long long)b * g.sA;
  const T* __restrict__ B = g.B + (long long)b * g.sB;
  T* __restrict__ C = g.C + (long long)b * g.sC;
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
  const int t = threadIdx.x;
  const int tx = t & 15, ty = t >> 4;

  // load coordinates (two elements per thread per operand)
  int ai[2], ak[2], bk[2], bj[2];
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    int e = t + r * NT;  // 0..511
    if (OPA == OP_N) { ai[r] = e & (BM - 1); ak[r] = e >> 6; }
    else { ak[r] = e & (BK - 1); ai[r] = e >> 3; }
    if (OPB == OP_N) { bk[r] = e & (BK - 1); bj[r] = e >> 3; }
    else { bj[r] = e & (BN - 1); bk[r] = e >> 6; }
  }

  T acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = CplxTraits<T>::make(0, 0);

  T ra[2], rb[2];
  const int ktiles = (g.k + BK - 1) / BK;
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    ra[r] = load_a<OPA, T>(A, g.lda, g.m, g.k, m0 + ai[r], ak[r]);
    rb[r] = load_b<OPB, T>(B, g.ldb, g.n, g.k, bk[r], n0 + bj[r]);
  }
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    As[0][ak[r]][ai[r]] = ra[r];
    Bs[0][bk[r]][bj[r]] = rb[r];
  }
  __syncthreads();

  for (int kt = 0; kt < ktiles; ++kt) {
    const int cur = kt & 1;
    const bool more = (kt + 1) < ktiles;
    if (more) {
      const int k0 = (kt + 1) * BK;
#pragma unroll
      for (int r = 0; r < 2; ++r) {
        ra[r] = load_a<OPA, T>(A, g.lda, g.m, g.k, m0 + ai[r], k0 + ak[r]);
        rb[r] = load_b<OPB, T>(B, g.ldb, g.n, g.k, k0 + bk[r], n0 + bj[r]);
      }
    }
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      T av[4], bv[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) av[i] = As[cur][kk][tx + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) bv[j] = Bs[cur][kk][ty + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) cfma(acc[i][j], av[i], bv[j]);
    }
    if (more) {
#pragma unroll
      for (int r = 0; r < 2; ++r) {
        As[cur ^ 1][ak[r]][ai[r]] = ra[r];
        Bs[cur ^ 1][bk[r]][bj[r]] = rb[r];
      }
    }
    __syncthreads();
  }

  const bool beta0 = (g.beta.x == 0.0 && g.beta.y == 0.0);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int row = m0 + tx + 16 * i;
    if (row >= g.m) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int col = n0 + ty + 16 * j;
      if (col >= g.n) continue;
      T* cp = C + (long long)col * g.ldc + row;
      T v = cmul(g.alpha, acc[i][j]);
      if (!beta0) v = cadd(v, cmul(g.beta, *cp));
      *cp = v;
    }
  }
}

template <int OPA, int OPB, typename T>
void launch(const GemmBatchT<T>& g, cudaStream_t st) {
  dim3 grid((g.m + BM - 1) / BM, (g.n + BN - 1) / BN, g.batch);
  zgemm_kernel<OPA, OPB, T><<<grid, NT, 0, st>>>(g);
}

}  // namespace

int zgemm_f64(const GemmBatch& g, cudaStream_t st) {
  if (g.m <= 0 || g.n <= 0 || g.batch <= 0) return NEGF_OK;
  if (g.batch > 65535) return NEGF_EINVAL;
#define NEGF_GEMM_CASE(a, b) \
  if (g.opA == a && g.opB == b) {                                                            \
    cudaEvent_t ev;                                                                          \
    timed_begin(st, TK_GEMM, 8.0 * g.m * g.n * (double)g.k * g.batch, &ev);                  \
    launch<a, b, double2>(g, st);                                                            \
    NEGF_CUDA_TRY(cudaGetLastError());                                                       \
    timed_end(st, TK_GEMM, ev);                                                              \
    count_launch();                                                                          \
    return NEGF_OK;                                                                          \
  }
  NEGF_GEMM_CASE(OP_N, OP_N)
  NEGF_GEMM_CASE(OP_N, OP_C)
  NEGF_GEMM_CASE(OP_C, OP_N)
  NEGF_GEMM_CASE(OP_N, OP_T)
  NEGF_GEMM_CASE(OP_T, OP_N)
  NEGF_GEMM_CASE(OP_C, OP_C)
#undef NEGF_GEMM_CASE
  return NEGF_EINVAL;
}

}  // namespace negf

namespace negf {

int cgemm_f32(const GemmBatchT<float2>& g, cudaStream_t st) {
  if (g.m <= 0 || g.n <= 0 || g.batch <= 0) return NEGF_OK;
  if (g.batch > 65535 || g.opA != OP_N || g.opB != OP_N) return NEGF_EINVAL;
  cudaEvent_t ev;
  timed_begin(st, TK_F32, 8.0 * g.m * g.n * (double)g.k * g.batch, &ev);
  launch<OP_N, OP_N, float2>(g, st);
  NEGF_CUDA_TRY(cudaGetLastError());
  timed_end(st, TK_F32, ev);
  count_launch();
  return NEGF_OK;
}

}  // namespace negf
