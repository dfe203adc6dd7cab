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
//   3. gj_update:  A(:, not K) += P * R(:, not K), P = A(:, K) (the factorised panel).
// After the last panel, gj_colswap undoes the row pivoting as column interchanges.
// INFO follows ZGETRF: the 1-based index of the first exactly-zero pivot (0 if none).
#include "negf_internal.cuh"

namespace negf {

namespace {

constexpr int PANEL_THREADS = 512;
constexpr size_t kPanelSmemMax = 200 * 1024;

// V is the real type of the matrix: the FP32 inverse compares floats, so its pivot search
// stays off the FP64 pipe (comparing the floats orders them as their doubles would)
template <typename V>
__device__ __forceinline__ void argmax_combine(V& v, int& i, V v2, int i2) {
  // larger value wins; on ties the lower row index wins (izamax returns the first max)
  if (v2 > v || (v2 == v && i2 < i)) { v = v2; i = i2; }
}

// Factorisation of one n x kb panel held column-major in shared memory, Ps[c * n + i],
// c in [0, kb), i in [0, n), by the whole CTA (blockDim.x a multiple of 32 and >= kb).
// The pivot of each column is the first maximum of |re|+|im| (exact comparisons with the
// lowest index winning ties), and every row is eliminated by one thread with the same
// operations whatever the thread count, so the result does not depend on blockDim.
// red_v / red_i hold one entry per warp.  Ends after a barrier.
template <typename T>
__device__ __forceinline__ void panel_factor(T* Ps, int n, int k0, int kb, int* ip, int* info_b,
                                             typename CplxTraits<T>::R* red_v, int* red_i, int* s_piv, T* s_d) {
  using R = typename CplxTraits<T>::R;
  const int t = threadIdx.x, nth = blockDim.x;
  const int lane = t & 31, warp = t >> 5, nwarps = nth >> 5;
  for (int c = 0; c < kb; ++c) {
    const int r = k0 + c;
    T* col = Ps + (long long)c * n;
    // ---- pivot search over rows r..n-1
    R bv = -1;
    int bi = n;
    for (int i = r + t; i < n; i += nth) argmax_combine(bv, bi, (R)cabs1(col[i]), i);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      R ov = __shfl_down_sync(0xffffffffu, bv, off);
      int oi = __shfl_down_sync(0xffffffffu, bi, off);
      argmax_combine(bv, bi, ov, oi);
    }
    if (lane == 0) { red_v[warp] = bv; red_i[warp] = bi; }
    __syncthreads();
    // second level by warp 0 with shuffles (the maximum under "larger value, then lower
    // index" does not depend on the order of the comparisons)
    if (warp == 0) {
      R v = lane < nwarps ? red_v[lane] : (R)-1;
      int i = lane < nwarps ? red_i[lane] : n;
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        R ov = __shfl_down_sync(0xffffffffu, v, off);
        int oi = __shfl_down_sync(0xffffffffu, i, off);
        argmax_combine(v, i, ov, oi);
      }
      if (lane == 0) {
        if (i >= n) i = r;
        *s_piv = i;
        ip[r] = i;
        T pv = col[i];
        if (pv.x == 0 && pv.y == 0) {
          if (*info_b == 0) *info_b = r + 1;
          *s_d = CplxTraits<T>::make(0, 0);
        } else {
          *s_d = crcp(pv);
        }
      }
    }
    __syncthreads();
    const int p = *s_piv;
    const T d = *s_d;
    const bool singular = (d.x == 0 && d.y == 0);
    // ---- interchange rows r and p inside the panel, scale the pivot row
    if (t < kb) {
      T* cj = Ps + (long long)t * n;
      T vr = cj[r], vp = cj[p];
      if (p != r) { cj[p] = vr; }
      // new pivot-row value is the old row p
      cj[r] = (t == c) ? (singular ? vp : d) : (singular ? vp : cmul(vp, d));
    }
    __syncthreads();
    if (singular) continue;
    // ---- eliminate column c from every other row; row i is owned by one thread, which
    // loads EU columns of its row and of the pivot row before any arithmetic or store (the
    // row's elements are independent, so this only removes the wait on each load)
    constexpr int EU = 8;
    for (int i = t; i < n; i += nth) {
      if (i == r) continue;
      const T f = col[i];
      int j0 = 0;
      for (; j0 + EU <= kb; j0 += EU) {
        T rv[EU], v[EU];
#pragma unroll
        for (int q = 0; q < EU; ++q) {
          const T* cj = Ps + (long long)(j0 + q) * n;
          rv[q] = cj[r];
          v[q] = cj[i];
        }
#pragma unroll
        for (int q = 0; q < EU; ++q) {
          if (j0 + q == c) continue;
          v[q].x = fma((R)-f.x, rv[q].x, v[q].x);
          v[q].x = fma(f.y, rv[q].y, v[q].x);
          v[q].y = fma((R)-f.x, rv[q].y, v[q].y);
          v[q].y = fma((R)-f.y, rv[q].x, v[q].y);
          Ps[(long long)(j0 + q) * n + i] = v[q];
        }
      }
      for (int j = j0; j < kb; ++j) {
        if (j == c) continue;
        T* cj = Ps + (long long)j * n;
        const T rv = cj[r];
        T v = cj[i];
        v.x = fma((R)-f.x, rv.x, v.x);
        v.x = fma(f.y, rv.y, v.x);
        v.y = fma((R)-f.x, rv.y, v.y);
        v.y = fma((R)-f.y, rv.x, v.y);
        cj[i] = v;
      }
      col[i] = cmul(CplxTraits<T>::make(-f.x, -f.y), d);
    }
    __syncthreads();
  }
}

// One CTA per matrix: the panel [k0, k0 + kb) factorised in shared memory.
template <typename T>
__global__ void __launch_bounds__(PANEL_THREADS) gj_panel_kernel(T* A, long long sA, int n, int k0, int kb,
                                                                 int* ipiv, int* info) {
  extern __shared__ __align__(16) unsigned char panel_raw[];
  T* Ps = reinterpret_cast<T*>(panel_raw);
  using R = typename CplxTraits<T>::R;
  __shared__ R red_v[PANEL_THREADS / 32];
  __shared__ int red_i[PANEL_THREADS / 32];
  __shared__ int s_piv;
  __shared__ T s_d;
  const int b = blockIdx.x;
  T* Ab = A + (long long)b * sA;
  const int t = threadIdx.x;
  const T* src = Ab + (long long)k0 * n;
  for (int e = t; e < n * kb; e += PANEL_THREADS) Ps[e] = src[e];
  __syncthreads();
  panel_factor<T>(Ps, n, k0, kb, ipiv + (long long)b * n, info + b, red_v, red_i, &s_piv, &s_d);
  T* dst = Ab + (long long)k0 * n;
  for (int e = t; e < n * kb; e += PANEL_THREADS) dst[e] = Ps[e];
}

// Row interchanges of one panel for the columns outside it, and the copy of rows K into R.
// The kb interchanges (r, ip[r]) of the panel touch at most 2 kb rows.  Thread 0 of each
// CTA composes them once into a gather list over the touched rows (row trow[t] receives the
// value of row torig[t]); then one warp per column loads its touched values (all loads
// before any store, so the gather is a simultaneous permutation), writes rows K to R
// (kb x n, column-major) with zeros in A, and the other touched rows back in place.
// Panel columns get R = 0.
constexpr int SWAP_WARPS = 8;
template <typename T>
__global__ void __launch_bounds__(SWAP_WARPS * 32) gj_swap_kernel(T* A, long long sA, int n, int k0, int kb,
                                                                  const int* ipiv, T* R, long long sR) {
  __shared__ int trow[64], torig[64];
  __shared__ int s_nt;
  const int b = blockIdx.y;
  T* Ab = A + (long long)b * sA;
  const int* ip = ipiv + (long long)b * n;
  T* Rb = R + (long long)b * sR;
  if (threadIdx.x == 0) {
    int nt = kb;
    for (int c = 0; c < kb; ++c) { trow[c] = k0 + c; torig[c] = k0 + c; }
    for (int c = 0; c < kb; ++c) {
      const int r = k0 + c, p = ip[r];
      if (p == r) continue;
      int ip_ = -1;
      for (int t = 0; t < nt; ++t)
        if (trow[t] == p) { ip_ = t; break; }
      if (ip_ < 0) { ip_ = nt; trow[nt] = p; torig[nt] = p; ++nt; }
      const int tmp = torig[c];   // row r sits at index c
      torig[c] = torig[ip_];
      torig[ip_] = tmp;
    }
    s_nt = nt;
  }
  __syncthreads();
  const int nt = s_nt;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int j = blockIdx.x * SWAP_WARPS + warp;
  if (j >= n) return;
  if (j >= k0 && j < k0 + kb) {
    for (int c = lane; c < kb; c += 32) Rb[(long long)j * kb + c] = CplxTraits<T>::make(0, 0);
    return;
  }
  T* colj = Ab + (long long)j * n;
  T v0 = CplxTraits<T>::make(0, 0), v1 = CplxTraits<T>::make(0, 0);
  if (lane < nt) v0 = colj[torig[lane]];
  if (lane + 32 < nt) v1 = colj[torig[lane + 32]];
  __syncwarp();
  if (lane < nt) {
    const int r = trow[lane];
    if (r >= k0 && r < k0 + kb) { Rb[(long long)j * kb + (r - k0)] = v0; colj[r] = CplxTraits<T>::make(0, 0); }
    else colj[r] = v0;
  }
  if (lane + 32 < nt) {
    const int r = trow[lane + 32];
    if (r >= k0 && r < k0 + kb) { Rb[(long long)j * kb + (r - k0)] = v1; colj[r] = CplxTraits<T>::make(0, 0); }
    else colj[r] = v1;
  }
}

// The rank-kb update of one panel step: A(:, j) += P R(:, j) for every column j outside the
// panel [k0, k0 + kb), P = A(:, k0:k0+kb) (n x kb), R (kb x n) from gj_swap.  K = kb <= 32,
// so each CTA stages its whole P and R slabs in shared memory with one barrier and then
// runs the kb rank-1 steps from there: 80 x 80 output tiles, 256 threads of 5 x 5 complex
// accumulators (25 FMAs per 10 shared loads).  The R slab's rows are padded to 81 entries:
// its loads walk k fastest, and an 80-entry stride would put every thread of a warp on the
// same bank.  In the FP32 form the 25 values of A a thread updates are loaded before the k
// loop, so their latency overlaps the slab loads and the FMAs instead of serialising 25
// load/store round trips at the end (the FP64 form, with twice the registers per value,
// loads them a column of five at a time).  The k order and the final A + sum equal those of
// the general GEMM kernel, so results are bitwise the same.
constexpr int UPD_T = 80, UPD_R = 5, UPD_RS = UPD_T + 1;
template <typename T>
__global__ void __launch_bounds__(256, sizeof(T) == 8 ? 2 : 1) gj_update_kernel(T* A, long long sA, int n, int k0, int kb, const T* R,
                                                        long long sR) {
  extern __shared__ __align__(16) unsigned char upd_raw[];
  T* Ps = reinterpret_cast<T*>(upd_raw);              // [kb][UPD_T]
  T* Rs = Ps + 32 * UPD_T;                              // [kb][UPD_RS]
  constexpr bool kPrefetch = sizeof(T) == 8;            // float2
  const int b = blockIdx.z;
  const int m0 = blockIdx.x * UPD_T, n0 = blockIdx.y * UPD_T;
  if (n0 >= k0 && n0 + UPD_T <= k0 + kb) return;        // tile inside the panel columns
  T* Ab = A + (long long)b * sA;
  const T* Rb = R + (long long)b * sR;
  const int t = threadIdx.x;
  const int tx = t & 15, ty = t >> 4;
  auto updated = [&](int i, int j) -> T* {              // nullptr: outside A or in the panel
    const int row = m0 + tx + 16 * i, col = n0 + ty + 16 * j;
    if (row >= n || col >= n || (col >= k0 && col < k0 + kb)) return nullptr;
    return Ab + (long long)col * n + row;
  };
  T cin[kPrefetch ? UPD_R : 1][kPrefetch ? UPD_R : 1];
  if constexpr (kPrefetch) {
#pragma unroll
    for (int j = 0; j < UPD_R; ++j)
#pragma unroll
      for (int i = 0; i < UPD_R; ++i) {
        const T* cp = updated(i, j);
        cin[i][j] = cp ? *cp : CplxTraits<T>::make(0, 0);
      }
  }
  for (int e = t; e < kb * UPD_T; e += 256) {
    const int k = e / UPD_T, i = e % UPD_T;
    Ps[k * UPD_T + i] = (m0 + i < n) ? Ab[(long long)(k0 + k) * n + m0 + i] : CplxTraits<T>::make(0, 0);
    const int j = e / kb, kk = e % kb;                  // R slab: contiguous kb x UPD_T
    Rs[kk * UPD_RS + j] = (n0 + j < n) ? Rb[(long long)(n0 + j) * kb + kk] : CplxTraits<T>::make(0, 0);
  }
  __syncthreads();
  T acc[UPD_R][UPD_R];
#pragma unroll
  for (int i = 0; i < UPD_R; ++i)
#pragma unroll
    for (int j = 0; j < UPD_R; ++j) acc[i][j] = CplxTraits<T>::make(0, 0);
  for (int k = 0; k < kb; ++k) {
    T av[UPD_R], bv[UPD_R];
#pragma unroll
    for (int i = 0; i < UPD_R; ++i) av[i] = Ps[k * UPD_T + tx + 16 * i];
#pragma unroll
    for (int j = 0; j < UPD_R; ++j) bv[j] = Rs[k * UPD_RS + ty + 16 * j];
#pragma unroll
    for (int i = 0; i < UPD_R; ++i)
#pragma unroll
      for (int j = 0; j < UPD_R; ++j) cfma(acc[i][j], av[i], bv[j]);
  }
#pragma unroll
  for (int j = 0; j < UPD_R; ++j) {
    T c[UPD_R];
    if constexpr (!kPrefetch) {   // the column's five loads before its five stores
#pragma unroll
      for (int i = 0; i < UPD_R; ++i) {
        const T* cp = updated(i, j);
        c[i] = cp ? *cp : CplxTraits<T>::make(0, 0);
      }
    }
#pragma unroll
    for (int i = 0; i < UPD_R; ++i) {
      T* cp = updated(i, j);
      if (!cp) continue;
      if constexpr (kPrefetch) *cp = cadd(acc[i][j], cin[i][j]);
      else *cp = cadd(acc[i][j], c[i]);
    }
  }
}

// The FP32 rank-kb update as a persistent, software-pipelined kernel (two CTAs per SM, each
// walking output tiles of 80 x 80).  While a CTA computes one tile, cp.async copies the P
// and R slabs of its next tile into the other half of a double buffer, and the tile's C
// values load into registers behind the k loop; the one-tile-per-CTA form above ran its
// load, compute and store phases back to back with two CTAs per SM to overlap them.  Each
// output element is formed by exactly the operations of gj_update_kernel (the same k order
// of fused multiply-adds from the same slabs, then A + sum), so results are bitwise equal.
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem, int src_bytes) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"((uint32_t)__cvta_generic_to_shared(smem)),
               "l"(gmem), "r"(src_bytes)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

constexpr int UPD_SLABS = 32 * UPD_T + 32 * UPD_RS;   // float2 of one buffer: P slab, then R slab

__global__ void __launch_bounds__(256, 2) gj_update_f32_pipelined(float2* A, long long sA, int n, int k0, int kb,
                                                                  const float2* R, long long sR, int ntm, int ntn,
                                                                  long long ntiles) {
  extern __shared__ __align__(16) unsigned char upp_raw[];
  float2* bufs = reinterpret_cast<float2*>(upp_raw);   // [2][UPD_SLABS]
  const int t = threadIdx.x;
  const int tx = t & 15, ty = t >> 4;
  const long long per_item = (long long)ntm * ntn;
  // copies of tile q's slabs into buffer Ps (P slab [kb][UPD_T], R slab [kb][UPD_RS]);
  // entries outside A are zero-filled without a read
  auto issue = [&](long long q, float2* Ps) {
    const int b = (int)(q / per_item);
    const int r = (int)(q % per_item);
    const int m0 = (r / ntn) * UPD_T, n0 = (r % ntn) * UPD_T;
    const float2* Ab = A + (long long)b * sA;
    const float2* Rb = R + (long long)b * sR;
    float2* Rs = Ps + 32 * UPD_T;
    for (int e = t; e < kb * UPD_T; e += 256) {
      const int k = e / UPD_T, i = e % UPD_T;
      const bool okp = m0 + i < n;
      cp_async8(&Ps[k * UPD_T + i], okp ? (const void*)&Ab[(long long)(k0 + k) * n + m0 + i] : (const void*)Ab,
                okp ? 8 : 0);
      const int j = e / kb, kk = e % kb;
      const bool okr = n0 + j < n;
      cp_async8(&Rs[kk * UPD_RS + j], okr ? (const void*)&Rb[(long long)(n0 + j) * kb + kk] : (const void*)Rb,
                okr ? 8 : 0);
    }
    cp_async_commit();
  };
  long long q = blockIdx.x;
  if (q < ntiles) issue(q, bufs);
  for (int it = 0; q < ntiles; q += gridDim.x, ++it) {
    const float2* Ps = bufs + (it & 1) * UPD_SLABS;
    const float2* Rs = Ps + 32 * UPD_T;
    const int b = (int)(q / per_item);
    const int r = (int)(q % per_item);
    const int m0 = (r / ntn) * UPD_T, n0 = (r % ntn) * UPD_T;
    float2* Ab = A + (long long)b * sA;
    auto updated = [&](int i, int j) -> float2* {   // nullptr: outside A or in the panel
      const int row = m0 + tx + 16 * i, col = n0 + ty + 16 * j;
      if (row >= n || col >= n || (col >= k0 && col < k0 + kb)) return nullptr;
      return Ab + (long long)col * n + row;
    };
    float2 cin[UPD_R][UPD_R];
#pragma unroll
    for (int j = 0; j < UPD_R; ++j)
#pragma unroll
      for (int i = 0; i < UPD_R; ++i) {
        const float2* cp = updated(i, j);
        cin[i][j] = cp ? *cp : make_float2(0.0f, 0.0f);
      }
    // the next tile's slabs go into the other buffer, which every thread finished reading
    // before the barrier that ended the previous iteration
    if (q + gridDim.x < ntiles) issue(q + gridDim.x, bufs + ((it + 1) & 1) * UPD_SLABS);
    else cp_async_commit();   // an empty group keeps the count: wait_group 1 below = this tile
    cp_async_wait<1>();
    __syncthreads();
    float2 acc[UPD_R][UPD_R];
#pragma unroll
    for (int i = 0; i < UPD_R; ++i)
#pragma unroll
      for (int j = 0; j < UPD_R; ++j) acc[i][j] = make_float2(0.0f, 0.0f);
    for (int k = 0; k < kb; ++k) {
      float2 av[UPD_R], bv[UPD_R];
#pragma unroll
      for (int i = 0; i < UPD_R; ++i) av[i] = Ps[k * UPD_T + tx + 16 * i];
#pragma unroll
      for (int j = 0; j < UPD_R; ++j) bv[j] = Rs[k * UPD_RS + ty + 16 * j];
#pragma unroll
      for (int i = 0; i < UPD_R; ++i)
#pragma unroll
        for (int j = 0; j < UPD_R; ++j) cfma(acc[i][j], av[i], bv[j]);
    }
#pragma unroll
    for (int j = 0; j < UPD_R; ++j)
#pragma unroll
      for (int i = 0; i < UPD_R; ++i) {
        float2* cp = updated(i, j);
        if (cp) *cp = cadd(acc[i][j], cin[i][j]);
      }
    __syncthreads();   // this buffer is free for the tile after next
  }
  cp_async_wait<0>();
}

// One thread per row: column interchanges in reverse pivot order.
template <typename T>
__global__ void gj_colswap_kernel(T* A, long long sA, int n, const int* ipiv) {
  const int b = blockIdx.y;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  T* Ab = A + (long long)b * sA;
  const int* ip = ipiv + (long long)b * n;
  for (int k = n - 1; k >= 0; --k) {
    const int p = ip[k];
    if (p != k) {
      T tmp = Ab[(long long)k * n + i];
      Ab[(long long)k * n + i] = Ab[(long long)p * n + i];
      Ab[(long long)p * n + i] = tmp;
    }
  }
}

// The whole FP32 Gauss-Jordan of one matrix in one CTA: for every panel, the panel
// factorisation, its row interchanges and its rank-kb update, in the same order and with
// the same operations per element as gj_panel + gj_swap + gj_update, so the inverse is
// bitwise the same as the three-launch form's (the update's k order, its fused multiply-
// adds and the final A + sum are those of gj_update_kernel).  It replaces 3 launches per
// panel by one per inverse and keeps the panel in shared memory across its update.
//   - the panel (n x 32 float2, up to 100 KB at n = 400) stays in shared memory;
//   - the other columns are processed in chunks of 32: one warp per column applies the
//     panel's interchanges (the same gather list as gj_swap) and moves rows K into the
//     chunk's R slab (32 x 32 in shared memory), then all 256 threads update the chunk,
//     each thread 4 rows x 8 columns of accumulators;
//   - two CTAs share an SM, so one's serial panel steps overlap the other's updates.
// Offered when the batch has at least one matrix per SM (below that the three-launch form
// spreads a matrix over many SMs and always finishes first); the engine times both forms
// on its first inverse of a shape and keeps the faster.  The column interchanges that end
// the inverse stay a separate launch (gj_colswap_kernel).
constexpr int FUSED_THREADS = 256, FUSED_JC = 32, FUSED_RS = FUSED_JC + 1, FUSED_MAX_N = 400;
__global__ void __launch_bounds__(FUSED_THREADS, 2) gj_fused_f32_kernel(float2* A, long long sA, int n, int* ipiv,
                                                                        int* info) {
  extern __shared__ __align__(16) unsigned char fused_raw[];
  float2* Ps = reinterpret_cast<float2*>(fused_raw);   // [32][n]: the panel, column-major
  float2* Rs = Ps + 32 * n;                             // [32][FUSED_RS]: rows K of a chunk
  __shared__ float red_v[FUSED_THREADS / 32];
  __shared__ int red_i[FUSED_THREADS / 32];
  __shared__ int s_piv, s_nt;
  __shared__ float2 s_d;
  __shared__ int trow[64], torig[64];
  const int b = blockIdx.x;
  float2* Ab = A + (long long)b * sA;
  int* ip = ipiv + (long long)b * n;
  const int t = threadIdx.x;
  const int warp = t >> 5, lane = t & 31;
  const int rg = t & 63, cg = t >> 6;                   // update: row group, column group
  const float2 zero = make_float2(0.f, 0.f);
  for (int k0 = 0; k0 < n; k0 += FUSED_JC) {
    const int kb = n - k0 < FUSED_JC ? n - k0 : FUSED_JC;
    const float2* src = Ab + (long long)k0 * n;
    for (int e = t; e < n * kb; e += FUSED_THREADS) Ps[e] = src[e];
    __syncthreads();
    panel_factor<float2>(Ps, n, k0, kb, ip, info + b, red_v, red_i, &s_piv, &s_d);
    float2* dst = Ab + (long long)k0 * n;
    for (int e = t; e < n * kb; e += FUSED_THREADS) dst[e] = Ps[e];
    if (t == 0) {   // the panel's interchanges as one gather over the touched rows (gj_swap)
      int nt = kb;
      for (int c = 0; c < kb; ++c) { trow[c] = k0 + c; torig[c] = k0 + c; }
      for (int c = 0; c < kb; ++c) {
        const int r = k0 + c, p = ip[r];
        if (p == r) continue;
        int ip_ = -1;
        for (int q = 0; q < nt; ++q)
          if (trow[q] == p) { ip_ = q; break; }
        if (ip_ < 0) { ip_ = nt; trow[nt] = p; torig[nt] = p; ++nt; }
        const int tmp = torig[c];
        torig[c] = torig[ip_];
        torig[ip_] = tmp;
      }
      s_nt = nt;
    }
    __syncthreads();
    const int nt = s_nt;
    for (int j0 = 0; j0 < n; j0 += FUSED_JC) {
      if (j0 == k0) continue;                           // the panel's own columns
      // interchanges of the chunk's columns; rows K go to R and become zero in A
      for (int jj = warp; jj < FUSED_JC; jj += FUSED_THREADS / 32) {
        const int j = j0 + jj;
        if (j >= n) break;
        float2* colj = Ab + (long long)j * n;
        float2 v0 = zero, v1 = zero;
        if (lane < nt) v0 = colj[torig[lane]];
        if (lane + 32 < nt) v1 = colj[torig[lane + 32]];
        __syncwarp();
        if (lane < nt) {
          const int r = trow[lane];
          if (r >= k0 && r < k0 + kb) { Rs[(r - k0) * FUSED_RS + jj] = v0; colj[r] = zero; }
          else colj[r] = v0;
        }
        if (lane + 32 < nt) {
          const int r = trow[lane + 32];
          if (r >= k0 && r < k0 + kb) { Rs[(r - k0) * FUSED_RS + jj] = v1; colj[r] = zero; }
          else colj[r] = v1;
        }
      }
      __syncthreads();
      // A(:, j) += P R(:, j) for the chunk's columns: rows rg + 64 q (+ 256 per pass),
      // columns j0 + 8 cg + c
      for (int i0 = 0; i0 < n; i0 += 256) {
        float2 acc[4][8];
#pragma unroll
        for (int q = 0; q < 4; ++q)
#pragma unroll
          for (int c = 0; c < 8; ++c) acc[q][c] = zero;
        for (int k = 0; k < kb; ++k) {
          float2 pv[4], rv[8];
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const int i = i0 + rg + 64 * q;
            pv[q] = i < n ? Ps[k * n + i] : zero;
          }
#pragma unroll
          for (int c = 0; c < 8; ++c) rv[c] = Rs[k * FUSED_RS + 8 * cg + c];
#pragma unroll
          for (int q = 0; q < 4; ++q)
#pragma unroll
            for (int c = 0; c < 8; ++c) cfma(acc[q][c], pv[q], rv[c]);
        }
#pragma unroll
        for (int c = 0; c < 8; ++c) {
          const int j = j0 + 8 * cg + c;
          if (j >= n) break;
          float2* colj = Ab + (long long)j * n;
          float2 cin[4];
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const int i = i0 + rg + 64 * q;
            cin[q] = i < n ? colj[i] : zero;
          }
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const int i = i0 + rg + 64 * q;
            if (i < n) colj[i] = cadd(acc[q][c], cin[q]);
          }
        }
      }
      __syncthreads();   // the chunk's A and R are done before the next chunk's interchanges
    }
  }
}

}  // namespace

size_t gj_fused_smem(int n) { return sizeof(float2) * ((size_t)32 * n + 32 * FUSED_RS); }

int panel_width(int n, int elem_bytes) {
  // the panel (n x nb complex) must fit the 227 KB opt-in shared memory of a CTA.  The
  // panel's work grows with nb (n*nb^2 per panel, n^2*nb per inverse) while its rank-nb
  // updates are cheap, so both forms use nb = 32.
  const long long limit = kPanelSmemMax;
  int nb = 32;
  (void)elem_bytes;
  while (nb > 4 && (long long)n * nb * (long long)elem_bytes > limit) nb >>= 1;
  return nb;
}

int inv_work_alloc(InvWork& w, int n, int batch, cudaMemPool_t pool, cudaStream_t st) {
  if (w.n_cap >= n && w.batch_cap >= batch && w.rbuf) return NEGF_OK;
  inv_work_free(w, st);
  w.nb = panel_width(n);
  w.pooled = pool != nullptr;
  auto get = [&](void** p, size_t bytes) {
    return (pool ? cudaMallocFromPoolAsync(p, bytes, pool, st) : cudaMalloc(p, bytes)) == cudaSuccess;
  };
  // R buffer: nb x n complex per matrix, large enough for both forms (FP64 nb, FP32 2nb)
  if (!get((void**)&w.rbuf, sizeof(double2) * (size_t)batch * w.nb * n)) return NEGF_ENOMEM;
  if (!get((void**)&w.ipiv, sizeof(int) * (size_t)batch * n)) return NEGF_ENOMEM;
  if (!get((void**)&w.info, sizeof(int) * (size_t)batch)) return NEGF_ENOMEM;
  w.n_cap = n;
  w.batch_cap = batch;
  return NEGF_OK;
}

void inv_work_free(InvWork& w, cudaStream_t st) {
  for (void* p : {(void*)w.rbuf, (void*)w.ipiv, (void*)w.info})
    if (p) {
      if (w.pooled) cudaFreeAsync(p, st);
      else cudaFree(p);
    }
  w = InvWork{};
}

namespace {


int sm_count_cached() {
  static int n = 0;
  if (n == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 148;
  }
  return n;
}

// FP32 inverse as one fused launch per batch (plus the column interchanges)
int gj_invert_fused_f32(float2* A, long long sA, int n, int batch, InvWork& w, cudaStream_t st) {
  const size_t smem = gj_fused_smem(n);
  NEGF_CUDA_TRY(cudaFuncSetAttribute(gj_fused_f32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  NEGF_CUDA_TRY(cudaMemsetAsync(w.info, 0, sizeof(int) * batch, st));
  cudaEvent_t ev;
  timed_begin(st, TK_F32, 8.0 * (double)n * n * n * batch, &ev);
  gj_fused_f32_kernel<<<batch, FUSED_THREADS, smem, st>>>(A, sA, n, w.ipiv, w.info);
  NEGF_CUDA_TRY(cudaGetLastError());
  timed_end(st, TK_F32, ev);
  dim3 g3((n + 127) / 128, batch);
  gj_colswap_kernel<float2><<<g3, 128, 0, st>>>(A, sA, n, w.ipiv);
  NEGF_CUDA_TRY(cudaGetLastError());
  count_launch(2);
  return NEGF_OK;
}

template <typename T>
int gj_invert(T* A, long long sA, int n, int batch, InvWork& w, cudaStream_t st) {
  if (batch <= 0 || n <= 0) return NEGF_OK;
  if (n > w.n_cap || batch > w.batch_cap) return NEGF_EINVAL;
  const int nb = panel_width(n, (int)sizeof(T));
  const size_t smem = sizeof(T) * (size_t)n * nb;
  if (smem > kPanelSmemMax) return NEGF_EINVAL;
  NEGF_CUDA_TRY(cudaFuncSetAttribute(gj_panel_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kPanelSmemMax));
  const size_t upd_smem = sizeof(T) * 32 * (UPD_T + UPD_RS);
  NEGF_CUDA_TRY(cudaFuncSetAttribute(gj_update_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)upd_smem));
  const size_t upp_smem = sizeof(float2) * 2 * (size_t)UPD_SLABS;
  if constexpr (sizeof(T) == 8)
    NEGF_CUDA_TRY(cudaFuncSetAttribute(gj_update_f32_pipelined, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)upp_smem));
  if (nb > 32 || batch > 65535) return NEGF_EINVAL;
  NEGF_CUDA_TRY(cudaMemsetAsync(w.info, 0, sizeof(int) * batch, st));
  T* rbuf = reinterpret_cast<T*>(w.rbuf);
  const long long sR = (long long)nb * n;
  for (int k0 = 0; k0 < n; k0 += nb) {
    const int kb = (n - k0 < nb) ? (n - k0) : nb;
    cudaEvent_t ev;
    timed_begin(st, TK_PANEL, 8.0 * n * (double)kb * kb * batch, &ev);
    gj_panel_kernel<T><<<batch, PANEL_THREADS, smem, st>>>(A, sA, n, k0, kb, w.ipiv, w.info);
    NEGF_CUDA_TRY(cudaGetLastError());
    timed_end(st, TK_PANEL, ev);
    dim3 g2((n + SWAP_WARPS - 1) / SWAP_WARPS, batch);
    gj_swap_kernel<T><<<g2, SWAP_WARPS * 32, 0, st>>>(A, sA, n, k0, kb, w.ipiv, rbuf, sR);
    NEGF_CUDA_TRY(cudaGetLastError());
    count_launch(2);
    // A(:, j) += P R(:, j) for the columns outside the panel
    {
      cudaEvent_t eu;
      timed_begin(st, sizeof(T) == 8 ? TK_F32 : TK_GEMM, 8.0 * n * (double)(n - kb) * kb * batch, &eu);
      const int nt = (n + UPD_T - 1) / UPD_T;
      if constexpr (sizeof(T) == 8) {
        const long long ntiles = (long long)nt * nt * batch;
        const int grid = (int)std::min<long long>(ntiles, 2LL * sm_count_cached());
        gj_update_f32_pipelined<<<grid, 256, upp_smem, st>>>(reinterpret_cast<float2*>(A), sA, n, k0, kb,
                                                             reinterpret_cast<const float2*>(rbuf), sR, nt, nt,
                                                             ntiles);
      } else {
        dim3 gu(nt, nt, batch);
        gj_update_kernel<T><<<gu, 256, upd_smem, st>>>(A, sA, n, k0, kb, rbuf, sR);
      }
      NEGF_CUDA_TRY(cudaGetLastError());
      timed_end(st, sizeof(T) == 8 ? TK_F32 : TK_GEMM, eu);
      count_launch();
    }
  }
  dim3 g3((n + 127) / 128, batch);
  gj_colswap_kernel<T><<<g3, 128, 0, st>>>(A, sA, n, w.ipiv);
  NEGF_CUDA_TRY(cudaGetLastError());
  count_launch();
  return NEGF_OK;
}

}  // namespace

int zinv_f64(double2* A, long long sA, int n, int batch, InvWork& w, cudaStream_t st) {
  return gj_invert<double2>(A, sA, n, batch, w, st);
}

bool cinv_f32_fused_ok(int n, int batch) { return n <= FUSED_MAX_N && batch >= sm_count_cached(); }

int cinv_f32(float2* A, long long sA, int n, int batch, InvWork& w, cudaStream_t st, int form) {
  if (form == 1) {
    if (!cinv_f32_fused_ok(n, batch)) return NEGF_EINVAL;
    if (batch <= 0) return NEGF_OK;
    if (n > w.n_cap || batch > w.batch_cap) return NEGF_EINVAL;
    return gj_invert_fused_f32(A, sA, n, batch, w, st);
  }
  return gj_invert<float2>(A, sA, n, batch, w, st);
}

}  // namespace negf
