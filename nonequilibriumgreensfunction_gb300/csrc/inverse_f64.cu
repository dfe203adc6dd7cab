// Batched in-place complex FP64 matrix inverse: blocked Gauss-Jordan elimination with
// partial row pivoting.
//
// Replaces Invert_Matrix (Source/MKL_Routines_Cluster.F90:2-33, ZGETRF + ZGETRI).  Both
// are 8n^3 real flops; Gauss-Jordan is chosen because every panel step after the panel
// factorisation is ONE rank-nb update of the whole matrix (a GEMM), with no triangular
// solves, which keeps the FP64 pipe of all SMs busy across a batch of matrices.
//
// Per panel K = [k0, k0+nb):
//   1. gj_panel:   one CTA per matrix factorises the n x nb panel in shared memory
//                  (pivot = first max of |re|+|im| over rows >= k, as LAPACK izamax).
//   2. gj_swap:    applies the panel's row interchanges to the other columns, copies
//                  their rows K into R (nb x n) and zeroes them.
//   3. zgemm:      A(:, not K) += P * R(:, not K), P = A(:, K) (the factorised panel).
// After the last panel, gj_colswap undoes the row pivoting as column interchanges.
// INFO follows ZGETRF: the 1-based index of the first exactly-zero pivot (0 if none).
#include "negf_internal.cuh"

namespace negf {

namespace {

constexpr int PANEL_THREADS = 512;
constexpr size_t kPanelSmemMax = 200 * 1024;

__device__ __forceinline__ void argmax_combine(double& v, int& i, double v2, int i2) {
  // larger value wins; on ties the lower row index wins (izamax returns the first max)
  if (v2 > v || (v2 == v && i2 < i)) { v = v2; i = i2; }
}

// Panel stored column-major in shared memory: Ps[c * n + i], c in [0, kb), i in [0, n).
__global__ void __launch_bounds__(PANEL_THREADS) gj_panel_kernel(double2* A, long long sA, int n, int k0, int kb,
                                                                 int* ipiv, int* info) {
  extern __shared__ double2 Ps[];
  __shared__ double red_v[PANEL_THREADS / 32];
  __shared__ int red_i[PANEL_THREADS / 32];
  __shared__ int s_piv;
  __shared__ double2 s_d;
  const int b = blockIdx.x;
  double2* Ab = A + (long long)b * sA;
  int* ip = ipiv + (long long)b * n;
  const int t = threadIdx.x;
  const int lane = t & 31, warp = t >> 5;

  const double2* src = Ab + (long long)k0 * n;
  for (int e = t; e < n * kb; e += PANEL_THREADS) Ps[e] = src[e];
  __syncthreads();

  for (int c = 0; c < kb; ++c) {
    const int r = k0 + c;
    double2* col = Ps + (long long)c * n;
    // ---- pivot search over rows r..n-1
    double bv = -1.0;
    int bi = n;
    for (int i = r + t; i < n; i += PANEL_THREADS) argmax_combine(bv, bi, cabs1(col[i]), i);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      double ov = __shfl_down_sync(0xffffffffu, bv, off);
      int oi = __shfl_down_sync(0xffffffffu, bi, off);
      argmax_combine(bv, bi, ov, oi);
    }
    if (lane == 0) { red_v[warp] = bv; red_i[warp] = bi; }
    __syncthreads();
    if (t == 0) {
      double v = red_v[0];
      int i = red_i[0];
      for (int w = 1; w < PANEL_THREADS / 32; ++w) argmax_combine(v, i, red_v[w], red_i[w]);
      if (i >= n) i = r;
      s_piv = i;
      ip[r] = i;
      double2 pv = col[i];
      if (pv.x == 0.0 && pv.y == 0.0) {
        if (info[b] == 0) info[b] = r + 1;
        s_d = make_double2(0.0, 0.0);
      } else {
        s_d = crcp(pv);
      }
    }
    __syncthreads();
    const int p = s_piv;
    const double2 d = s_d;
    const bool singular = (d.x == 0.0 && d.y == 0.0);
    // ---- interchange rows r and p inside the panel, scale the pivot row
    if (t < kb) {
      double2* cj = Ps + (long long)t * n;
      double2 vr = cj[r], vp = cj[p];
      if (p != r) { cj[p] = vr; }
      // new pivot-row value is the old row p
      cj[r] = (t == c) ? (singular ? vp : d) : (singular ? vp : cmul(vp, d));
    }
    __syncthreads();
    if (singular) continue;
    // ---- eliminate column c from every other row; row i is owned by one thread
    for (int i = t; i < n; i += PANEL_THREADS) {
      if (i == r) continue;
      const double2 f = col[i];
      for (int j = 0; j < kb; ++j) {
        if (j == c) continue;
        double2* cj = Ps + (long long)j * n;
        const double2 rv = cj[r];
        double2 v = cj[i];
        v.x = fma(-f.x, rv.x, v.x);
        v.x = fma(f.y, rv.y, v.x);
        v.y = fma(-f.x, rv.y, v.y);
        v.y = fma(-f.y, rv.x, v.y);
        cj[i] = v;
      }
      col[i] = cmul(make_double2(-f.x, -f.y), d);
    }
    __syncthreads();
  }
  double2* dst = Ab + (long long)k0 * n;
  for (int e = t; e < n * kb; e += PANEL_THREADS) dst[e] = Ps[e];
}

// One thread per column j outside the panel: apply the nb row interchanges in order, copy
// rows K to R (kb x n, column-major) and zero them in A.  Panel columns get R = 0.
__global__ void gj_swap_kernel(double2* A, long long sA, int n, int k0, int kb, const int* ipiv, double2* R,
                               long long sR) {
  const int b = blockIdx.y;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  double2* Ab = A + (long long)b * sA;
  const int* ip = ipiv + (long long)b * n;
  double2* Rb = R + (long long)b * sR;
  if (j >= k0 && j < k0 + kb) {
    for (int c = 0; c < kb; ++c) Rb[(long long)j * kb + c] = make_double2(0.0, 0.0);
    return;
  }
  double2* colj = Ab + (long long)j * n;
  for (int c = 0; c < kb; ++c) {
    const int r = k0 + c, p = ip[r];
    if (p != r) {
      double2 tmp = colj[r];
      colj[r] = colj[p];
      colj[p] = tmp;
    }
  }
  for (int c = 0; c < kb; ++c) {
    Rb[(long long)j * kb + c] = colj[k0 + c];
    colj[k0 + c] = make_double2(0.0, 0.0);
  }
}

// One thread per row: column interchanges in reverse pivot order.
__global__ void gj_colswap_kernel(double2* A, long long sA, int n, const int* ipiv) {
  const int b = blockIdx.y;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double2* Ab = A + (long long)b * sA;
  const int* ip = ipiv + (long long)b * n;
  for (int k = n - 1; k >= 0; --k) {
    const int p = ip[k];
    if (p != k) {
      double2 tmp = Ab[(long long)k * n + i];
      Ab[(long long)k * n + i] = Ab[(long long)p * n + i];
      Ab[(long long)p * n + i] = tmp;
    }
  }
}

}  // namespace

int panel_width(int n) {
  // the panel (n x nb complex) must fit the 227 KB opt-in shared memory of a CTA
  const long long limit = kPanelSmemMax;
  int nb = 32;
  while (nb > 4 && (long long)n * nb * (long long)sizeof(double2) > limit) nb >>= 1;
  return nb;
}

int inv_work_alloc(InvWork& w, int n, int batch) {
  if (w.n_cap >= n && w.batch_cap >= batch && w.rbuf) return NEGF_OK;
  inv_work_free(w);
  w.nb = panel_width(n);
  if (cudaMalloc(&w.rbuf, sizeof(double2) * (size_t)batch * w.nb * n) != cudaSuccess) return NEGF_ENOMEM;
  if (cudaMalloc(&w.ipiv, sizeof(int) * (size_t)batch * n) != cudaSuccess) return NEGF_ENOMEM;
  if (cudaMalloc(&w.info, sizeof(int) * (size_t)batch) != cudaSuccess) return NEGF_ENOMEM;
  w.n_cap = n;
  w.batch_cap = batch;
  return NEGF_OK;
}

void inv_work_free(InvWork& w) {
  if (w.rbuf) cudaFree(w.rbuf);
  if (w.ipiv) cudaFree(w.ipiv);
  if (w.info) cudaFree(w.info);
  w = InvWork{};
}

int zinv_f64(double2* A, long long sA, int n, int batch, InvWork& w, cudaStream_t st) {
  if (batch <= 0 || n <= 0) return NEGF_OK;
  if (n > w.n_cap || batch > w.batch_cap) return NEGF_EINVAL;
  const int nb = panel_width(n);
  const size_t smem = sizeof(double2) * (size_t)n * nb;
  if (smem > kPanelSmemMax) return NEGF_EINVAL;
  NEGF_CUDA_TRY(cudaFuncSetAttribute(gj_panel_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kPanelSmemMax));
  NEGF_CUDA_TRY(cudaMemsetAsync(w.info, 0, sizeof(int) * batch, st));
  const long long sR = (long long)nb * n;
  for (int k0 = 0; k0 < n; k0 += nb) {
    const int kb = (n - k0 < nb) ? (n - k0) : nb;
    cudaEvent_t ev;
    timed_begin(st, TK_PANEL, 8.0 * n * (double)kb * kb * batch, &ev);
    gj_panel_kernel<<<batch, PANEL_THREADS, smem, st>>>(A, sA, n, k0, kb, w.ipiv, w.info);
    NEGF_CUDA_TRY(cudaGetLastError());
    timed_end(st, TK_PANEL, ev);
    dim3 g2((n + 127) / 128, batch);
    gj_swap_kernel<<<g2, 128, 0, st>>>(A, sA, n, k0, kb, w.ipiv, w.rbuf, sR);
    NEGF_CUDA_TRY(cudaGetLastError());
    count_launch(2);
    // A(:, 0:k0) += P R(:, 0:k0);  A(:, k0+kb:n) += P R(:, k0+kb:n)
    GemmBatch g{};
    g.m = n; g.k = kb; g.alpha = make_double2(1.0, 0.0); g.beta = make_double2(1.0, 0.0);
    g.A = A + (long long)k0 * n; g.lda = n; g.sA = sA; g.opA = OP_N;
    g.ldb = kb; g.sB = sR; g.opB = OP_N;
    g.ldc = n; g.sC = sA; g.batch = batch;
    if (k0 > 0) {
      g.n = k0; g.B = w.rbuf; g.C = A;
      NEGF_TRY(zgemm_f64(g, st));
    }
    if (k0 + kb < n) {
      g.n = n - k0 - kb; g.B = w.rbuf + (long long)(k0 + kb) * kb; g.C = A + (long long)(k0 + kb) * n;
      NEGF_TRY(zgemm_f64(g, st));
    }
  }
  dim3 g3((n + 127) / 128, batch);
  gj_colswap_kernel<<<g3, 128, 0, st>>>(A, sA, n, w.ipiv);
  NEGF_CUDA_TRY(cudaGetLastError());
  count_launch();
  return NEGF_OK;
}

}  // namespace negf
