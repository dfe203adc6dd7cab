// Structured and element-wise kernels of the FP64 solve: assembly of the matrices to
// invert, block-diagonal hopping products, the site blocks of Gn/Gp, traces and the
// density / spin reductions.  All are O(n^2) per block; the O(n^3) work is in
// gemm_f64.cu and inverse_f64.cu.
#include <algorithm>

#include "negf_internal.cuh"

namespace negf {

namespace {

constexpr int EW_THREADS = 256;

inline dim3 ew_grid(long long elems, int batch) {
  long long bx = (elems + EW_THREADS - 1) / EW_THREADS;
  if (bx > 65535) bx = 65535;
  return dim3((unsigned)bx, (unsigned)batch);
}

// hop block element: H(s*no + a, s*no + c)
__device__ __forceinline__ double2 hbe(const HopBD& h, int s, int a, int c) {
  return h.hb[((long long)s * h.norb + a) * h.norb + c];
}

// ---- W assembly (Energy_Sweep.F90:31-38 + Recursive_Greens.F90:18-20 / :70-72) ----------
__global__ void form_w_kernel(FormW a) {
  const int b = blockIdx.y;
  const int n = a.n;
  const long long nn = (long long)n * n;
  const Item it = a.items[b];
  const double2* Hx = a.Hall + ((long long)it.slot * a.npx + a.x) * nn;
  const double2* gp = a.gprev ? a.gprev + (long long)b * a.sG : nullptr;
  const double2* zs = a.zsub ? a.zsub + (long long)b * a.sZ : nullptr;
  const double2* sl = (a.x == 0 && a.sigL) ? a.sigL + (long long)b * a.sSig : nullptr;
  const double2* sr = (a.x == a.npx - 1 && a.sigR) ? a.sigR + (long long)b * a.sSig : nullptr;
  double2* W = a.W + (long long)b * a.sW;
  const int no = a.hop.norb;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nn; e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e % n), j = (int)(e / n);
    double2 v = make_double2(-Hx[e].x, -Hx[e].y);
    if (i == j) { v.x += it.energy; v.y += a.eta; }
    if (sl) v = csub(v, sl[e]);
    if (sr) v = csub(v, sr[e]);
    if (zs) v = csub(v, zs[e]);
    if (gp && a.hop.hb) {
      // sum_{p in site(i), q in site(j)} L(i,p) g(p,q) R(q,j)
      const int si = i / no, ai = i % no, sj = j / no, aj = j % no;
      double2 acc = make_double2(0.0, 0.0);
      for (int pa = 0; pa < no; ++pa) {
        // side 0: L = H^H -> L(i,p) = conj(H(p,i));  side 1: L = H -> H(i,p)
        const double2 l = a.side == 0 ? cconj(hbe(a.hop, si, pa, ai)) : hbe(a.hop, si, ai, pa);
        double2 row = make_double2(0.0, 0.0);
        const int p = si * no + pa;
        for (int qa = 0; qa < no; ++qa) {
          // side 0: R = H -> H(q,j);  side 1: R = H^H -> conj(H(j,q))
          const double2 r = a.side == 0 ? hbe(a.hop, sj, qa, aj) : cconj(hbe(a.hop, sj, aj, qa));
          const int q = sj * no + qa;
          cfma(row, gp[(long long)q * n + p], r);
        }
        cfma(acc, l, row);
      }
      v = csub(v, acc);
    }
    W[e] = v;
  }
}

// acc += x c (right) or c x (left) for one compact hop term of the given kind
__device__ __forceinline__ void term_fma(double2& acc, double2 x, double2 c, int kind, bool c_left) {
  if (kind == 0) {
    acc.x = fma(c.x, x.x, acc.x);
    acc.y = fma(c.x, x.y, acc.y);
  } else if (kind == 1) {
    acc.x = fma(-c.y, x.y, acc.x);
    acc.y = fma(c.y, x.x, acc.y);
  } else if (c_left) {
    cfma(acc, c, x);
  } else {
    cfma(acc, x, c);
  }
}

// W with the coupling term from the compact terms of a hop block shared by every site:
// W(i, j) -= sum_p L(a, p) sum_q G(4 si + p, 4 sj + q) R(q, c) over the nonzero terms only
// (i = 4 si + a, j = 4 sj + c), the nesting of form_w_blocks_kernel.  Lanes of a warp share
// j and take the same kinds of terms, so they branch together; the G elements come from L1.
__global__ void form_w_rows_kernel(FormW a) {
  const int b = blockIdx.y;
  const int n = a.n;
  const long long nn = (long long)n * n;
  const Item it = a.items[b];
  const double2* Hx = a.Hall + ((long long)it.slot * a.npx + a.x) * nn;
  const double2* gp = a.gprev + (long long)b * a.sG;
  const double2* sl = (a.x == 0 && a.sigL) ? a.sigL + (long long)b * a.sSig : nullptr;
  const double2* sr = (a.x == a.npx - 1 && a.sigR) ? a.sigR + (long long)b * a.sSig : nullptr;
  double2* W = a.W + (long long)b * a.sW;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nn; e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e % n), j = (int)(e / n);
    double2 v = make_double2(-Hx[e].x, -Hx[e].y);
    if (i == j) { v.x += it.energy; v.y += a.eta; }
    if (sl) v = csub(v, sl[e]);
    if (sr) v = csub(v, sr[e]);
    const int ra = i & 3, ca = j & 3;
    const double2* gb = gp + (long long)(j - ca) * n + (i - ra);   // G(4 si + p, 4 sj + q) = gb[q n + p]
    double2 acc = make_double2(0.0, 0.0);
    for (int tl = 0; tl < a.lrow.cnt[ra]; ++tl) {
      const int p = a.lrow.p[ra][tl];
      double2 t = make_double2(0.0, 0.0);
      for (int tr = 0; tr < a.rrow.cnt[ca]; ++tr)
        term_fma(t, gb[(long long)a.rrow.p[ca][tr] * n + p], a.rrow.c[ca][tr], a.rrow.kind[ca][tr], false);
      term_fma(acc, t, a.lrow.c[ra][tl], a.lrow.kind[ra][tl], true);
    }
    W[e] = csub(v, acc);
  }
}

// The same W when HopX is block diagonal with 4 x 4 site blocks: one thread per 4 x 4 site
// block (si, sj) of W.  The coupling term of the block is L_si G(si, sj) R_sj (side 0:
// L = H^H, R = H; side 1: L = H, R = H^H), formed as T = G R and then L T: 8 complex FMAs
// per element instead of the 20 of the element-wise form.  GB300's FP64 pipe runs at 1/64
// of its FP32 rate, so this FP64 arithmetic, not memory, bounds the kernel.  Used when the
// sites' blocks differ; a block shared by every site takes form_w_rows_kernel.  Each thread
// reads and writes its block as four 64-byte column pieces; consecutive threads take
// consecutive row blocks, so a warp's accesses to a column are contiguous.
__global__ void form_w_blocks_kernel(FormW a) {
  const int b = blockIdx.y;
  const int n = a.n, ns = n / 4;
  const long long nblk = (long long)ns * ns;
  const Item it = a.items[b];
  const double2* Hx = a.Hall + ((long long)it.slot * a.npx + a.x) * ((long long)n * n);
  const double2* gp = a.gprev + (long long)b * a.sG;
  const double2* sl = (a.x == 0 && a.sigL) ? a.sigL + (long long)b * a.sSig : nullptr;
  const double2* sr = (a.x == a.npx - 1 && a.sigR) ? a.sigR + (long long)b * a.sSig : nullptr;
  double2* W = a.W + (long long)b * a.sW;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nblk; t += (long long)gridDim.x * blockDim.x) {
    const int si = (int)(t % ns), sj = (int)(t / ns);
    double2 g[4][4];                       // g[r][c] = G(4 si + r, 4 sj + c)
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const double2* col = gp + (long long)(4 * sj + c) * n + 4 * si;
#pragma unroll
      for (int r = 0; r < 4; ++r) g[r][c] = col[r];
    }
    // T = G R, one column of R(q, j) at a time (side 0: R = H, side 1: R = H^H)
    double2 tm[4][4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      double2 rc[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) rc[q] = a.side == 0 ? hbe(a.hop, sj, q, c) : cconj(hbe(a.hop, sj, c, q));
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        double2 acc = make_double2(0.0, 0.0);
#pragma unroll
        for (int q = 0; q < 4; ++q) cfma(acc, g[r][q], rc[q]);
        tm[r][c] = acc;
      }
    }
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const long long e0 = (long long)(4 * sj + c) * n + 4 * si;
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        double2 acc = make_double2(0.0, 0.0);
#pragma unroll
        for (int p = 0; p < 4; ++p)   // L(r, p): side 0: L = H^H, side 1: L = H
          cfma(acc, a.side == 0 ? cconj(hbe(a.hop, si, p, r)) : hbe(a.hop, si, r, p), tm[p][c]);
        const long long e = e0 + r;
        double2 v = make_double2(-Hx[e].x, -Hx[e].y);
        if (si == sj && r == c) { v.x += it.energy; v.y += a.eta; }
        if (sl) v = csub(v, sl[e]);
        if (sr) v = csub(v, sr[e]);
        W[e] = csub(v, acc);
      }
    }
  }
}

// ---- Y = op(H) X  or  X op(H), H block diagonal ------------------------------------
__global__ void hop_apply_kernel(HopBD h, int n, int left, int op, const double2* X, long long sX, double2* Y,
                                 long long sY) {
  const int b = blockIdx.y;
  const long long nn = (long long)n * n;
  const double2* Xb = X + (long long)b * sX;
  double2* Yb = Y + (long long)b * sY;
  const int no = h.norb;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nn; e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e % n), j = (int)(e / n);
    double2 acc = make_double2(0.0, 0.0);
    if (left) {
      // Y(i,j) = sum_p op(H)(i,p) X(p,j), p in site(i)
      const int s = i / no, ai = i % no;
      for (int pa = 0; pa < no; ++pa) {
        const double2 hv = (op == OP_C) ? cconj(hbe(h, s, pa, ai)) : hbe(h, s, ai, pa);
        cfma(acc, hv, Xb[(long long)j * n + s * no + pa]);
      }
    } else {
      // Y(i,j) = sum_q X(i,q) op(H)(q,j), q in site(j)
      const int s = j / no, aj = j % no;
      for (int qa = 0; qa < no; ++qa) {
        const double2 hv = (op == OP_C) ? cconj(hbe(h, s, aj, qa)) : hbe(h, s, qa, aj);
        cfma(acc, Xb[(long long)(s * no + qa) * n + i], hv);
      }
    }
    Yb[e] = acc;
  }
}

// The same products when every site shares one 4 x 4 block, from its compact terms: the
// wire models' HopX blocks are half zeros with purely real or imaginary nonzeros, so each
// output takes two terms of two FP64 fmas instead of four complex fmas (16 fmas).  The term
// lists are kernel parameters sorted by kind, so every lane runs the same kinds of terms;
// the skipped terms are exact zeros of hop_apply_kernel's sequence.
__global__ void hop_rows_kernel(HopRows r, int n, int left, const double2* X, long long sX, double2* Y, long long sY) {
  const int b = blockIdx.y;
  const long long nn = (long long)n * n;
  const double2* Xb = X + (long long)b * sX;
  double2* Yb = Y + (long long)b * sY;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nn; e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e % n), j = (int)(e / n);
    // left: x_p = X(4s + p, j), a = i % 4; right: x_p = X(i, 4s + p), a = j % 4
    const int a = left ? (i & 3) : (j & 3);
    const double2* xb = left ? Xb + (long long)j * n + (i - a) : Xb + (long long)(j - a) * n + i;
    const long long xs = left ? 1 : n;
    double2 acc = make_double2(0.0, 0.0);
    for (int t = 0; t < r.cnt[a]; ++t) {
      const double2 x = xb[r.p[a][t] * xs];
      const double2 c = r.c[a][t];
      const int k = r.kind[a][t];
      if (k == 0) {
        acc.x = fma(c.x, x.x, acc.x);
        acc.y = fma(c.x, x.y, acc.y);
      } else if (k == 1) {
        acc.x = fma(-c.y, x.y, acc.x);
        acc.y = fma(c.y, x.x, acc.y);
      } else if (left) {
        cfma(acc, c, x);
      } else {
        cfma(acc, x, c);
      }
    }
    Yb[e] = acc;
  }
}

// ---- site blocks of X Gamma X^H ------------------------------------------------------
// P[r][a] = sum_k Y(r,k) conj(X(site(r)*no + a, k)); one thread per row r, the k loop is
// split over KSPLIT groups of threads and reduced in shared memory (fixed order).
constexpr int SB_ROWS = 64, SB_KSPLIT = 4;
// NOM bounds the orbitals per site (4, or 8 for the BdG form); no <= NOM
template <int NOM>
__global__ void __launch_bounds__(SB_ROWS* SB_KSPLIT) site_blocks_kernel(int n, int no, const double2* Y, long long sY,
                                                                         const double2* X, long long sX, double2* P,
                                                                         long long sP) {
  __shared__ double2 part[SB_KSPLIT][SB_ROWS][NOM];
  const int b = blockIdx.y;
  const int lr = threadIdx.x % SB_ROWS, kg = threadIdx.x / SB_ROWS;
  const int r = blockIdx.x * SB_ROWS + lr;
  const double2* Yb = Y + (long long)b * sY;
  const double2* Xb = X + (long long)b * sX;
  double2 acc[NOM];
  for (int a = 0; a < NOM; ++a) acc[a] = make_double2(0, 0);
  if (r < n) {
    const int base = (r / no) * no;
    const int k_per = (n + SB_KSPLIT - 1) / SB_KSPLIT;
    const int k_lo = kg * k_per, k_hi = min(n, k_lo + k_per);
    for (int k = k_lo; k < k_hi; ++k) {
      const double2 y = Yb[(long long)k * n + r];
      for (int a = 0; a < no && a < NOM; ++a) cfma(acc[a], y, cconj(Xb[(long long)k * n + base + a]));
    }
  }
  for (int a = 0; a < NOM; ++a) part[kg][lr][a] = acc[a];
  __syncthreads();
  if (kg == 0 && r < n) {
    for (int a = 0; a < no && a < NOM; ++a) {
      double2 s = part[0][lr][a];
      for (int q = 1; q < SB_KSPLIT; ++q) s = cadd(s, part[q][lr][a]);
      P[(long long)b * sP + (long long)r * no + a] = s;
    }
  }
}

// ---- in-slice neighbour blocks ------------------------------------------------------
// For the row r of site s = r / no (s = y + z*npy):
//   P0[r][a] = sum_k Y(r,k) conj(X(s*no + a, k))            (the site itself)
//   P1[r][a] = same with site s + 1    (next y; zero when y = npy - 1)
//   P2[r][a] = same with site s + npy  (next z; zero when z = npz - 1)
// One pass over Y serves all three; the k split is reduced in shared memory per output in a
// fixed order, so P0 equals what site_blocks_kernel writes.
template <int NOM>
__global__ void __launch_bounds__(SB_ROWS* SB_KSPLIT) site_pairs_kernel(int n, int no, int npy, int npz,
                                                                        const double2* Y, long long sY,
                                                                        const double2* X, long long sX, double2* P0,
                                                                        double2* P1, double2* P2, long long sP) {
  __shared__ double2 part[SB_KSPLIT][SB_ROWS][NOM];
  const int b = blockIdx.y;
  const int lr = threadIdx.x % SB_ROWS, kg = threadIdx.x / SB_ROWS;
  const int r = blockIdx.x * SB_ROWS + lr;
  const double2* Yb = Y + (long long)b * sY;
  const double2* Xb = X + (long long)b * sX;
  double2 acc[3][NOM];
  for (int d = 0; d < 3; ++d)
    for (int a = 0; a < NOM; ++a) acc[d][a] = make_double2(0, 0);
  int base[3] = {-1, -1, -1};
  if (r < n) {
    const int s = r / no;
    const int y = s % npy, z = s / npy;
    base[0] = s * no;
    if (y < npy - 1) base[1] = (s + 1) * no;
    if (z < npz - 1) base[2] = (s + npy) * no;
    const int k_per = (n + SB_KSPLIT - 1) / SB_KSPLIT;
    const int k_lo = kg * k_per, k_hi = min(n, k_lo + k_per);
    for (int k = k_lo; k < k_hi; ++k) {
      const double2 yv = Yb[(long long)k * n + r];
      const double2* xk = Xb + (long long)k * n;
      for (int d = 0; d < 3; ++d) {
        if (base[d] < 0) continue;
        for (int a = 0; a < no && a < NOM; ++a) cfma(acc[d][a], yv, cconj(xk[base[d] + a]));
      }
    }
  }
  double2* outs[3] = {P0, P1, P2};
  for (int d = 0; d < 3; ++d) {
    for (int a = 0; a < NOM; ++a) part[kg][lr][a] = acc[d][a];
    __syncthreads();
    if (kg == 0 && r < n) {
      for (int a = 0; a < no && a < NOM; ++a) {
        double2 v = part[0][lr][a];
        for (int q = 1; q < SB_KSPLIT; ++q) v = cadd(v, part[q][lr][a]);
        outs[d][(long long)b * sP + (long long)r * no + a] = v;
      }
    }
    __syncthreads();
  }
}

// ---- Re sum Q .* conj(X) (one CTA per item, fixed reduction order) -------------------
__global__ void trace_dot_kernel(int n, const double2* Q, long long sQ, const double2* X, long long sX, double* out,
                                 int out_stride) {
  __shared__ double red[EW_THREADS];
  const int b = blockIdx.x;
  const long long nn = (long long)n * n;
  const double2* Qb = Q + (long long)b * sQ;
  const double2* Xb = X + (long long)b * sX;
  double s = 0.0;
  for (long long e = threadIdx.x; e < nn; e += EW_THREADS) {
    const double2 q = Qb[e], x = Xb[e];
    s = fma(q.x, x.x, s);
    s = fma(q.y, x.y, s);
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = EW_THREADS / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[(long long)b * out_stride] = red[0];
}

__global__ void gather_kernel(int n, const double2* src, const int* idx, int idx_stride, double2* dst, long long sDst) {
  const int b = blockIdx.y;
  const long long nn = (long long)n * n;
  const double2* s = src + (long long)idx[(long long)b * idx_stride] * nn;
  double2* d = dst + (long long)b * sDst;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nn; e += (long long)gridDim.x * blockDim.x)
    d[e] = s[e];
}

__global__ void copy_kernel(int n, const double2* src, long long sSrc, double2* dst, long long sDst) {
  const int b = blockIdx.y;
  const long long nn = (long long)n * n;
  const double2* s = src + (long long)b * sSrc;
  double2* d = dst + (long long)b * sDst;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nn; e += (long long)gridDim.x * blockDim.x)
    d[e] = s[e];
}

__global__ void identity_kernel(int n, double2* A, long long sA) {
  const int b = blockIdx.y;
  const long long nn = (long long)n * n;
  double2* d = A + (long long)b * sA;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nn; e += (long long)gridDim.x * blockDim.x)
    d[e] = make_double2((e % n) == (e / n) ? 1.0 : 0.0, 0.0);
}

// ---- Sancho-Rubio pieces (Contact_Self_Energy.F90:110-223) ---------------------------
__global__ void form_alpha_kernel(int n, const double* energies, const double2* const* hend, double eta, double extra,
                                  double2* A, long long sA) {
  const int b = blockIdx.y;
  const long long nn = (long long)n * n;
  const double2* H = hend[b];
  double2* d = A + (long long)b * sA;
  const double e0 = energies[b];
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nn; e += (long long)gridDim.x * blockDim.x) {
    double2 v = make_double2(-H[e].x, -H[e].y);
    if ((e % n) == (e / n)) { v.x += e0; v.y += eta + extra; }
    d[e] = v;
  }
}

// T += change (if active); cmax[b] = max |change| (as the bit pattern of a non-negative
// double, combined with atomicMax across CTAs; a NaN is recorded as a positive NaN, whose
// pattern exceeds every finite one).  cmax must be zeroed before the launch.
__global__ void sr_accumulate_kernel(int n, const int* active, const double2* change, long long sC, double2* T,
                                     long long sT, unsigned long long* cmax) {
  __shared__ double red[EW_THREADS];
  const int b = blockIdx.y;
  const long long nn = (long long)n * n;
  const double2* c = change + (long long)b * sC;
  double2* t = T + (long long)b * sT;
  const bool act = active[b] != 0;
  double m = 0.0;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nn; e += (long long)gridDim.x * blockDim.x) {
    const double2 v = c[e];
    double a = hypot(v.x, v.y);
    if (isnan(a)) a = __longlong_as_double(0x7FF8000000000000LL);
    m = (isnan(a) || isnan(m)) ? a : fmax(m, a);
    if (act) t[e] = cadd(t[e], v);
  }
  red[threadIdx.x] = m;
  __syncthreads();
  for (int w = EW_THREADS / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      const double o = red[threadIdx.x + w];
      red[threadIdx.x] = (isnan(o) || isnan(red[threadIdx.x])) ? __longlong_as_double(0x7FF8000000000000LL)
                                                                : fmax(red[threadIdx.x], o);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) atomicMax(cmax + b, (unsigned long long)__double_as_longlong(red[0]));
}

// W = alpha - L T with L = H^H (lead 0) or H (lead 1), H block diagonal
__global__ void sr_form_final_kernel(HopBD h, int n, int lead, const double2* alpha, long long sA, const double2* T,
                                     long long sT, double2* W, long long sW) {
  const int b = blockIdx.y;
  const long long nn = (long long)n * n;
  const double2* al = alpha + (long long)b * sA;
  const double2* Tb = T + (long long)b * sT;
  double2* Wb = W + (long long)b * sW;
  const int no = h.norb;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nn; e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e % n), j = (int)(e / n);
    const int s = i / no, ai = i % no;
    double2 acc = make_double2(0.0, 0.0);
    for (int pa = 0; pa < no; ++pa) {
      const double2 l = lead == 0 ? cconj(hbe(h, s, pa, ai)) : hbe(h, s, ai, pa);
      cfma(acc, l, Tb[(long long)j * n + s * no + pa]);
    }
    Wb[e] = csub(al[e], acc);
  }
}

// Sigma = L g R; lead 0: H^H g H; lead 1: H g H^H.  Gamma = i (Sigma - Sigma^H).
__global__ void sr_sigma_kernel(HopBD h, int n, int lead, const double2* g, long long sg, double2* sig, long long sS) {
  const int b = blockIdx.y;
  const long long nn = (long long)n * n;
  const double2* gb = g + (long long)b * sg;
  double2* Sb = sig + (long long)b * sS;
  const int no = h.norb;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nn; e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e % n), j = (int)(e / n);
    const int si = i / no, ai = i % no, sj = j / no, aj = j % no;
    double2 acc = make_double2(0.0, 0.0);
    for (int pa = 0; pa < no; ++pa) {
      const double2 l = lead == 0 ? cconj(hbe(h, si, pa, ai)) : hbe(h, si, ai, pa);
      double2 row = make_double2(0.0, 0.0);
      const int p = si * no + pa;
      for (int qa = 0; qa < no; ++qa) {
        const double2 r = lead == 0 ? hbe(h, sj, qa, aj) : cconj(hbe(h, sj, aj, qa));
        cfma(row, gb[(long long)(sj * no + qa) * n + p], r);
      }
      cfma(acc, l, row);
    }
    Sb[e] = acc;
  }
}

__global__ void gamma_dos_kernel(int n, const double2* sig, long long sS, double2* gam, long long sG, double* dos) {
  __shared__ double red[EW_THREADS];
  const int b = blockIdx.x;
  const long long nn = (long long)n * n;
  const double2* Sb = sig + (long long)b * sS;
  double2* Gb = gam + (long long)b * sG;
  for (long long e = threadIdx.x; e < nn; e += EW_THREADS) {
    const int i = (int)(e % n), j = (int)(e / n);
    const double2 s = Sb[e], st = Sb[(long long)i * n + j];
    // i (S - S^H): S^H(i,j) = conj(S(j,i))
    const double2 d = make_double2(s.x - st.x, s.y + st.y);
    Gb[e] = make_double2(-d.y, d.x);
  }
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += EW_THREADS) s += Sb[(long long)i * n + i].y;
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = EW_THREADS / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) dos[b] = -red[0] / 3.14159265358979323846;
}

// ---- densities and spin from the site blocks (Calculate_Gnp.F90:117-124,
//      Calculate_Observables.F90:10-43) -------------------------------------------------
// One thread per (item, x, site).  Gn_site = f1 P1 + f2 P2, Gp_site = (1-f1) P1 + (1-f2) P2.
__global__ void density_spin_kernel(DensityArgs a) {
  const int b = blockIdx.y;
  const int nsite = a.npy * a.npz;
  const int total = a.npx * nsite;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  const int no = a.norb;
  const Item it = a.items[b];
  const double w = it.dE / (2.0 * 3.14159265358979323846);
  double e_n = 0.0, e_p = 0.0;
  if (idx < total) {
    const int x = idx / nsite, s = idx % nsite;          // s = y + z*npy (orbital index order)
    const int y = s % a.npy, z = s / a.npy;
    const double2* p1 = a.P1 + (long long)b * a.sP + ((long long)x * a.n + (long long)s * no) * no;
    const double2* p2 = a.P2 + (long long)b * a.sP + ((long long)x * a.n + (long long)s * no) * no;
    double rn = 0.0, rp = 0.0, en = 0.0, ep = 0.0;
    double sp[3] = {0.0, 0.0, 0.0};
    for (int ia = 0; ia < no; ++ia) {
      const double2 q1 = p1[ia * no + ia], q2 = p2[ia * no + ia];
      rn += it.f1 * q1.x + it.f2 * q2.x;
      rp += (1.0 - it.f1) * q1.x + (1.0 - it.f2) * q2.x;
      if (ia == a.nh - 1) { en = rn; ep = rp; }   // EDensity/HDensity: electron orbitals only
    }
    if (a.calc_spin) {
      // Re sum_{ia,ib} Gn(ia,ib) gM(ib,ia), P stored as P[row ia][col ib]
      for (int j = 0; j < 3; ++j) {
        const double2* gm = a.spin_ops + j * no * no;
        double acc = 0.0;
        for (int ia = 0; ia < no; ++ia)
          for (int ib = 0; ib < no; ++ib) {
            const double2 q1 = p1[ia * no + ib], q2 = p2[ia * no + ib];
            const double2 gn = make_double2(it.f1 * q1.x + it.f2 * q2.x, it.f1 * q1.y + it.f2 * q2.y);
            const double2 g = gm[ib * no + ia];
            acc += gn.x * g.x - gn.y * g.y;
          }
        sp[j] = acc;
      }
    }
    // site arrays are (x, y, z) column-major: x fastest
    const long long o = (long long)x + (long long)a.npx * (y + (long long)a.npy * z);
    double* so = a.site_out + (long long)b * a.nf * total;
    so[o] = rn * w;
    so[total + o] = rp * w;
    so[2 * total + o] = sp[0] * w;
    so[3 * total + o] = sp[1] * w;
    so[4 * total + o] = sp[2] * w;
    e_n = en;
    e_p = ep;
  }
  // per-item EDensity/HDensity partial sums: written per thread block, summed by host-ordered kernel
  __shared__ double red_n[256], red_p[256];
  red_n[threadIdx.x] = e_n;
  red_p[threadIdx.x] = e_p;
  __syncthreads();
  for (int s2 = blockDim.x / 2; s2 > 0; s2 >>= 1) {
    if (threadIdx.x < s2) {
      red_n[threadIdx.x] += red_n[threadIdx.x + s2];
      red_p[threadIdx.x] += red_p[threadIdx.x + s2];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    // partials[b][blockIdx.x][2]
    a.sums[((long long)b * gridDim.x + blockIdx.x) * 2 + 0] = red_n[0];
    a.sums[((long long)b * gridDim.x + blockIdx.x) * 2 + 1] = red_p[0];
  }
}

// ---- bond currents, Source/Calculate_Observables.F90:110-169 -----------------------------
// One thread per site (x, y, z) of one item.  With Gn = f1 P1 + f2 P2, Gp = (1-f1) P1 +
// (1-f2) P2 and the Hermitian symmetry Gn(b,a) = conj(Gn(a,b)), each orbital pair (i, j)
// of a bond a -> b contributes
//   dumVar = REAL(4)( Re( i q^2/hbar (H(a,b) Gn(b,a) - Gn(a,b) H(b,a) - H(a,b) Gp(b,a)
//                                    + Gp(a,b) H(b,a)) ) )
// and J += dumVar dE/(2 pi) in REAL(8), as the reference's dumVar (:7) is REAL(4).  The x
// bond couples the same site of slices x and x+1 through HopX(a,a) and its conjugate
// (:150-156).  Writes site_out fields 5, 6, 7 = Jx, Jy, Jz.
// dumVar of one orbital pair: the two lead blocks of P at (a_i, b_j) and H(a_i, b_j),
// H(b_j, a_i), rounded to REAL(4)
__device__ __forceinline__ float bond_dum(double2 p1, double2 p2, double2 hab, double2 hba, double f1, double f2,
                                          double pref) {
  const double2 gn = make_double2(f1 * p1.x + f2 * p2.x, f1 * p1.y + f2 * p2.y);
  const double2 gp = make_double2((1.0 - f1) * p1.x + (1.0 - f2) * p2.x, (1.0 - f1) * p1.y + (1.0 - f2) * p2.y);
  double2 v = csub(cmul(hab, cconj(gn)), cmul(gn, hba));
  v = csub(v, cmul(hab, cconj(gp)));
  v = cadd(v, cmul(gp, hba));
  return __double2float_rn(-pref * v.y);   // Re(i c v) = -c Im v
}

// bond d (0: +x, 1: +y, 2: +z) leaving site (x, y, z) stays inside the grid
__device__ __forceinline__ bool bond_inside(const CurrentArgs& a, int d, int x, int y, int z) {
  return d == 0 ? x < a.npx - 1 : (d == 1 ? y < a.npy - 1 : z < a.npz - 1);
}

// operands of orbital pair (ii, jj) of an inside bond d leaving site s = y + z npy of slice
// x; H is the slice's Htotd block, prow the item's site-block row of (x, s)
__device__ __forceinline__ void bond_pair(const CurrentArgs& a, const double2* H, long long prow, int d, int s, int ii,
                                          int jj, double2& p1, double2& p2, double2& hab, double2& hba) {
  const int no = a.norb;
  const long long n = a.n;
  const long long q = prow + ii * no + jj;
  if (d == 0) {
    const long long ri = (long long)s * no + ii, rj = (long long)s * no + jj;
    const double2 hx = a.Hop[rj * n + ri];
    p1 = a.Px1[q]; p2 = a.Px2[q]; hab = hx; hba = cconj(hx);
    return;
  }
  const long long nb = d == 1 ? s + 1 : s + a.npy;
  const long long ra = (long long)s * no + ii, rb = nb * no + jj;
  p1 = (d == 1 ? a.Py1 : a.Pz1)[q];
  p2 = (d == 1 ? a.Py2 : a.Pz2)[q];
  hab = H[rb * n + ra];
  hba = H[ra * n + rb];
}

__global__ void bond_currents_kernel(CurrentArgs a) {
  const int b = blockIdx.y;
  const int nsite = a.npy * a.npz;
  const int total = a.npx * nsite;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= total) return;
  const int no = a.norb;
  const Item it = a.items[b];
  const double w = it.dE / (2.0 * 3.14159265358979323846);
  const int x = idx / nsite, s = idx % nsite;
  const int y = s % a.npy, z = s / a.npy;
  const long long n = a.n;
  const double2* H = a.Hall + ((long long)it.slot * a.npx + x) * n * n;
  const long long prow = (long long)b * a.sP + ((long long)x * n + (long long)s * no) * no;
  double j[3] = {0.0, 0.0, 0.0}, ju[3] = {0.0, 0.0, 0.0};
  for (int d = 0; d < 3; ++d) {
    if (!bond_inside(a, d, x, y, z)) continue;
    for (int ii = 0; ii < a.nh; ++ii)
      for (int jj = 0; jj < a.nh; ++jj) {
        double2 p1, p2, hab, hba;
        bond_pair(a, H, prow, d, s, ii, jj, p1, p2, hab, hba);
        const double dum = (double)bond_dum(p1, p2, hab, hba, it.f1, it.f2, a.q2_over_hbar);
        j[d] += dum * w;
        ju[d] += dum;
      }
  }
  const long long o = (long long)x + (long long)a.npx * (y + (long long)a.npy * z);
  double* so = a.site_out + (long long)b * a.nf * total;
  so[5LL * total + o] = j[0];
  so[6LL * total + o] = j[1];
  so[7LL * total + o] = j[2];
  if (a.er_out) {
    // energy-resolved fields (Calculate_Observables.F90:124-157, Calculate_Gnp.F90:125-127):
    // the unweighted bond sums and sum over orbitals of Re Gn(i,i) - Re Gp(i,i)
    double rho = 0.0;
    for (int ii = 0; ii < no; ++ii) {
      const double2 q1 = a.P1[prow + ii * no + ii], q2 = a.P2[prow + ii * no + ii];
      rho += (it.f1 * q1.x + it.f2 * q2.x) - ((1.0 - it.f1) * q1.x + (1.0 - it.f2) * q2.x);
    }
    double* eo = a.er_out + (long long)b * 4 * total;
    eo[o] = ju[0];
    eo[total + o] = ju[1];
    eo[2LL * total + o] = ju[2];
    eo[3LL * total + o] = rho;
  }
}

// Orbital-resolved bond currents and densities (ORJx/y/z of Calculate_Observables.F90:127-160,
// ORRhon of Calculate_Gnp.F90:127-129), summed over the items of each slot in item order.
// One thread per (slot, site, q): q < 3 norb^2 is orbital pair (ii, jj), ii*norb + jj =
// q % norb^2, of bond direction q / norb^2 (x, y, z); q >= 3 norb^2 is orbital q - 3 norb^2
// of the density.  or_acc[slot][q][site] += sum_b dE_b/(2 pi) value_b, q fastest across
// threads so that a warp reads whole site blocks.
__global__ void orbital_resolved_kernel(CurrentArgs a) {
  const int no = a.norb, nq = 3 * no * no + no;
  const int nsite = a.npy * a.npz;
  const int total = a.npx * nsite;
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= (long long)total * nq) return;
  const int slot = blockIdx.y;
  const int q = (int)(idx % nq);
  const int site = (int)(idx / nq);
  const int x = site / nsite, s = site % nsite;
  const int y = s % a.npy, z = s / a.npy;
  const long long n = a.n;
  double acc = 0.0;
  if (q < 3 * no * no) {
    const int d = q / (no * no), ii = (q % (no * no)) / no, jj = q % no;
    if (ii < a.nh && jj < a.nh && bond_inside(a, d, x, y, z)) {
      for (int b = 0; b < a.batch; ++b) {
        const Item it = a.items[b];
        if (it.slot != slot) continue;
        const double w = it.dE / (2.0 * 3.14159265358979323846);
        const double2* H = a.Hall + ((long long)it.slot * a.npx + x) * n * n;
        const long long prow = (long long)b * a.sP + ((long long)x * n + (long long)s * no) * no;
        double2 p1, p2, hab, hba;
        bond_pair(a, H, prow, d, s, ii, jj, p1, p2, hab, hba);
        acc += (double)bond_dum(p1, p2, hab, hba, it.f1, it.f2, a.q2_over_hbar) * w;
      }
    }
  } else {
    const int ii = q - 3 * no * no;
    for (int b = 0; b < a.batch; ++b) {
      const Item it = a.items[b];
      if (it.slot != slot) continue;
      const double w = it.dE / (2.0 * 3.14159265358979323846);
      const long long pd = (long long)b * a.sP + ((long long)x * n + (long long)s * no) * no + ii * no + ii;
      acc += (it.f1 * a.P1[pd].x + it.f2 * a.P2[pd].x) * w;
    }
  }
  const long long o = (long long)x + (long long)a.npx * (y + (long long)a.npy * z);
  a.or_acc[((long long)slot * nq + q) * total + o] += acc;
}

// ---- model contacts (Contact_Self_Energy.F90:19-67) ---------------------------------
// Sigma of job s, lead l: coef[s][l] = (diag, up, lo).  Types 1/2: diag on the first ndiag
// orbitals.  Type 3: the same norb x norb block on every site, diag on both nh x nh
// diagonal blocks, up * gds in the electron-hole block, lo * gds in the hole-electron one.
__global__ void contact_fill_kernel(int n, int no, int nh, int type, int ndiag, const double2* coef, ContactGds g,
                                    double2* sigL, double2* sigR, long long sS) {
  const int job = blockIdx.y;
  const long long nn = (long long)n * n;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < 2 * nn;
       e += (long long)gridDim.x * blockDim.x) {
    const int lead = (int)(e / nn);
    const long long f = e % nn;
    const int i = (int)(f % n), j = (int)(f / n);
    const double2* c = coef + ((long long)job * 2 + lead) * 3;
    double2 v = make_double2(0.0, 0.0);
    if (type != 3) {
      if (i == j && i < ndiag) v = c[0];
    } else if (i / no == j / no) {
      const int ai = i % no, aj = j % no;
      const bool ei = ai < nh, ej = aj < nh;
      if (ei == ej) {
        if (ai == aj) v = c[0];
      } else if (ei) {
        v = cmul(c[1], g.m[ai][aj - nh]);
      } else {
        v = cmul(c[2], g.m[ai - nh][aj]);
      }
    }
    (lead == 0 ? sigL : sigR)[(long long)job * sS + f] = v;
  }
}

// out[b][r][a] = X[b](r, site(r)*no + a): the diagonal site blocks of a column-major block
__global__ void site_diag_kernel(int n, int no, const double2* X, long long sX, double2* out, long long sO) {
  const int b = blockIdx.y;
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= (long long)n * no) return;
  const int r = (int)(e / no), a = (int)(e % no);
  out[(long long)b * sO + e] = X[(long long)b * sX + (long long)((r / no) * no + a) * n + r];
}

// Supercurrent transmission of Calculate_Observables.F90:60-81 for site-block-diagonal
// SigmaL / GammaL: T = sum_r sz(r) Re[(i Gn11 SigmaL^H)(r,r) - (G11 GammaL)(r,r)], sz = +1
// on electron orbitals, with Gn11 = f1 P1 + f2 P2 on slice 1 and G11 its diagonal site
// blocks.  One CTA per item, fixed reduction order.
__global__ void josephson_kernel(int n, int no, const Item* items, const double2* P1, const double2* P2, long long sP,
                                 const double2* G11, long long sG, const double2* sig, const double2* gam,
                                 long long sS, double* out) {
  __shared__ double red[EW_THREADS];
  const int b = blockIdx.x;
  const Item it = items[b];
  double t = 0.0;
  for (int r = threadIdx.x; r < n; r += blockDim.x) {
    const int base = (r / no) * no;
    double2 s1 = make_double2(0.0, 0.0), s2 = make_double2(0.0, 0.0);
    for (int a = 0; a < no; ++a) {
      const long long q = (long long)r * no + a;
      const double2 p1 = P1[(long long)b * sP + q], p2 = P2[(long long)b * sP + q];
      const double2 gn = make_double2(it.f1 * p1.x + it.f2 * p2.x, it.f1 * p1.y + it.f2 * p2.y);
      const long long c = (long long)(base + a);
      cfma(s1, gn, cconj(sig[(long long)b * sS + c * n + r]));           // Gn(r,c) conj(Sigma(r,c))
      cfma(s2, G11[(long long)b * sG + q], gam[(long long)b * sS + (long long)r * n + c]);  // G(r,c) Gamma(c,r)
    }
    const double v = -s1.y - s2.x;                                       // Re(i s1) - Re(s2)
    t += (r % no < no / 2) ? v : -v;
  }
  red[threadIdx.x] = t;
  __syncthreads();
  for (int k = blockDim.x / 2; k > 0; k >>= 1) {
    if (threadIdx.x < k) red[threadIdx.x] += red[threadIdx.x + k];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[b] = red[0];
}

__global__ void reduce_sites_kernel(int batch, int total, int nf, int nslots, const Item* items,
                                    const double* site_out, double* acc) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long per_slot = (long long)nf * total;
  if (i >= per_slot * nslots) return;
  const int slot = (int)(i / per_slot);
  const long long f = i % per_slot;
  double s = acc[i];
  for (int b = 0; b < batch; ++b)
    if (items[b].slot == slot) s += site_out[(long long)b * per_slot + f];
  acc[i] = s;
}

}  // namespace

// =====================================================================================
int form_w(const FormW& a, cudaStream_t st) {
  if (a.gprev && a.use_rows && a.hop.norb == 4 && !a.zsub && a.n % 4 == 0) {
    form_w_rows_kernel<<<ew_grid((long long)a.n * a.n, a.batch), EW_THREADS, 0, st>>>(a);
    NEGF_CUDA_TRY(cudaGetLastError());
    count_launch();
    return NEGF_OK;
  }
  if (a.gprev && a.hop.hb && a.hop.norb == 4 && !a.zsub && a.n % 4 == 0) {
    const long long nblk = (long long)(a.n / 4) * (a.n / 4);
    form_w_blocks_kernel<<<ew_grid(nblk, a.batch), 128, 0, st>>>(a);
    NEGF_CUDA_TRY(cudaGetLastError());
    count_launch();
    return NEGF_OK;
  }
  form_w_kernel<<<ew_grid((long long)a.n * a.n, a.batch), EW_THREADS, 0, st>>>(a);
  NEGF_CUDA_TRY(cudaGetLastError());
  count_launch();
  return NEGF_OK;
}

int hop_apply(const HopBD& h, const HopRows* rows, int n, int batch, int left, Op op, const double2* X, long long sX,
              double2* Y, long long sY, cudaStream_t st) {
  if (rows && h.norb == 4 && n % 4 == 0 && X != Y) {
    hop_rows_kernel<<<ew_grid((long long)n * n, batch), EW_THREADS, 0, st>>>(*rows, n, left, X, sX, Y, sY);
    NEGF_CUDA_TRY(cudaGetLastError());
    count_launch();
    return NEGF_OK;
  }
  hop_apply_kernel<<<ew_grid((long long)n * n, batch), EW_THREADS, 0, st>>>(h, n, left, (int)op, X, sX, Y, sY);
  NEGF_CUDA_TRY(cudaGetLastError());
  count_launch();
  return NEGF_OK;
}

int site_blocks(int n, int norb, int batch, const double2* Y, long long sY, const double2* X, long long sX, double2* P,
                long long sP, cudaStream_t st) {
  if (norb < 1 || norb > 8) return NEGF_EINVAL;
  dim3 grid((n + SB_ROWS - 1) / SB_ROWS, batch);
  if (norb <= 4)
    site_blocks_kernel<4><<<grid, SB_ROWS * SB_KSPLIT, 0, st>>>(n, norb, Y, sY, X, sX, P, sP);
  else
    site_blocks_kernel<8><<<grid, SB_ROWS * SB_KSPLIT, 0, st>>>(n, norb, Y, sY, X, sX, P, sP);
  NEGF_CUDA_TRY(cudaGetLastError());
  count_launch();
  return NEGF_OK;
}

int site_pairs(int n, int norb, int npy, int npz, int batch, const double2* Y, long long sY, const double2* X,
               long long sX, double2* P, double2* Py, double2* Pz, long long sP, cudaStream_t st) {
  if (norb < 1 || norb > 8 || n != norb * npy * npz) return NEGF_EINVAL;
  dim3 grid((n + SB_ROWS - 1) / SB_ROWS, batch);
  if (norb <= 4)
    site_pairs_kernel<4><<<grid, SB_ROWS * SB_KSPLIT, 0, st>>>(n, norb, npy, npz, Y, sY, X, sX, P, Py, Pz, sP);
  else
    site_pairs_kernel<8><<<grid, SB_ROWS * SB_KSPLIT, 0, st>>>(n, norb, npy, npz, Y, sY, X, sX, P, Py, Pz, sP);
  NEGF_CUDA_TRY(cudaGetLastError());
  count_launch();
  return NEGF_OK;
}

int bond_currents(const CurrentArgs& a, cudaStream_t st) {
  if (a.norb > 8 || a.nh < 1 || a.nh > a.norb || a.nf < 8) return NEGF_EINVAL;
  const int total = a.npx * a.npy * a.npz;
  dim3 grid((total + 127) / 128, a.batch);
  bond_currents_kernel<<<grid, 128, 0, st>>>(a);
  NEGF_CUDA_TRY(cudaGetLastError());
  count_launch();
  return NEGF_OK;
}

int orbital_resolved(const CurrentArgs& a, int nslots, cudaStream_t st) {
  if (a.norb > 8 || a.nh < 1 || a.nh > a.norb || !a.or_acc || nslots < 1) return NEGF_EINVAL;
  const long long work = (long long)a.npx * a.npy * a.npz * (3 * a.norb * a.norb + a.norb);
  dim3 grid((unsigned)((work + 255) / 256), nslots);
  orbital_resolved_kernel<<<grid, 256, 0, st>>>(a);
  NEGF_CUDA_TRY(cudaGetLastError());
  count_launch();
  return NEGF_OK;
}

int contact_fill(int n, int no, int nh, int type, int ndiag, int njobs, const double2* coef, const ContactGds& g,
                 double2* sigL, double2* sigR, long long sS, cudaStream_t st) {
  if (njobs < 1) return NEGF_OK;
  contact_fill_kernel<<<ew_grid(2LL * n * n, njobs), EW_THREADS, 0, st>>>(n, no, nh, type, ndiag, coef, g, sigL, sigR,
                                                                          sS);
  NEGF_CUDA_TRY(cudaGetLastError());
  count_launch();
  return NEGF_OK;
}

int site_diag(int n, int no, int batch, const double2* X, long long sX, double2* out, long long sO, cudaStream_t st) {
  const long long work = (long long)n * no;
  site_diag_kernel<<<dim3((unsigned)((work + 255) / 256), batch), 256, 0, st>>>(n, no, X, sX, out, sO);
  NEGF_CUDA_TRY(cudaGetLastError());
  count_launch();
  return NEGF_OK;
}

int josephson(int n, int no, int batch, const Item* items, const double2* P1, const double2* P2, long long sP,
              const double2* G11, long long sG, const double2* sig, const double2* gam, long long sS, double* out,
              cudaStream_t st) {
  josephson_kernel<<<batch, EW_THREADS, 0, st>>>(n, no, items, P1, P2, sP, G11, sG, sig, gam, sS, out);
  NEGF_CUDA_TRY(cudaGetLastError());
  count_launch();
  return NEGF_OK;
}

int trace_dot(int n, int batch, const double2* Q, long long sQ, const double2* X, long long sX, double* out,
              int out_stride, cudaStream_t st) {
  trace_dot_kernel<<<batch, EW_THREADS, 0, st>>>(n, Q, sQ, X, sX, out, out_stride);
  NEGF_CUDA_TRY(cudaGetLastError());
  count_launch();
  return NEGF_OK;
}

int gather_blocks(int n, int batch, const double2* src, const int* idx, int idx_stride, double2* dst, long long sDst,
                  cudaStream_t st) {
  gather_kernel<<<ew_grid((long long)n * n, batch), EW_THREADS, 0, st>>>(n, src, idx, idx_stride, dst, sDst);
  NEGF_CUDA_TRY(cudaGetLastError());
  count_launch();
  return NEGF_OK;
}

int copy_blocks(int n, int batch, const double2* src, long long sSrc, double2* dst, long long sDst, cudaStream_t st) {
  copy_kernel<<<ew_grid((long long)n * n, batch), EW_THREADS, 0, st>>>(n, src, sSrc, dst, sDst);
  NEGF_CUDA_TRY(cudaGetLastError());
  count_launch();
  return NEGF_OK;
}

int set_identity(int n, int batch, double2* A, long long sA, cudaStream_t st) {
  identity_kernel<<<ew_grid((long long)n * n, batch), EW_THREADS, 0, st>>>(n, A, sA);
  NEGF_CUDA_TRY(cudaGetLastError());
  count_launch();
  return NEGF_OK;
}

int form_alpha(int n, int nprob, const double* energies, const double2* const* hend, double eta, double extra_eta,
               double2* A, long long sA, cudaStream_t st) {
  form_alpha_kernel<<<ew_grid((long long)n * n, nprob), EW_THREADS, 0, st>>>(n, energies, hend, eta, extra_eta, A, sA);
  NEGF_CUDA_TRY(cudaGetLastError());
  count_launch();
  return NEGF_OK;
}

int sr_accumulate(int n, int nprob, const int* active, const double2* change, long long sC, double2* T, long long sT,
                  double* cmax, cudaStream_t st) {
  unsigned long long* bits = reinterpret_cast<unsigned long long*>(cmax);
  NEGF_CUDA_TRY(cudaMemsetAsync(bits, 0, sizeof(unsigned long long) * nprob, st));
  const long long nn = (long long)n * n;
  const int per = (int)std::min<long long>((nn + EW_THREADS * 16 - 1) / (EW_THREADS * 16), 64);
  sr_accumulate_kernel<<<dim3(per, nprob), EW_THREADS, 0, st>>>(n, active, change, sC, T, sT, bits);
  NEGF_CUDA_TRY(cudaGetLastError());
  count_launch();
  return NEGF_OK;
}

int sr_form_final(const HopBD& h, int n, int nprob, int lead, const double2* alpha, long long sA, const double2* T,
                  long long sT, double2* W, long long sW, cudaStream_t st) {
  sr_form_final_kernel<<<ew_grid((long long)n * n, nprob), EW_THREADS, 0, st>>>(h, n, lead, alpha, sA, T, sT, W, sW);
  NEGF_CUDA_TRY(cudaGetLastError());
  count_launch();
  return NEGF_OK;
}

int sr_sigma(const HopBD& h, int n, int nprob, int lead, const double2* g, long long sg, double2* sig, long long sSig,
             double2* gam, long long sGam, double* dos, cudaStream_t st) {
  if (lead >= 0) {  // lead < 0: sig already formed (dense HopX), only Gamma and DOS
    sr_sigma_kernel<<<ew_grid((long long)n * n, nprob), EW_THREADS, 0, st>>>(h, n, lead, g, sg, sig, sSig);
    NEGF_CUDA_TRY(cudaGetLastError());
    count_launch();
  }
  gamma_dos_kernel<<<nprob, EW_THREADS, 0, st>>>(n, sig, sSig, gam, sGam, dos);
  NEGF_CUDA_TRY(cudaGetLastError());
  count_launch();
  return NEGF_OK;
}

int density_spin(const DensityArgs& a, cudaStream_t st) {
  const int total = a.npx * a.npy * a.npz;
  dim3 grid((total + 255) / 256, a.batch);
  density_spin_kernel<<<grid, 256, 0, st>>>(a);
  NEGF_CUDA_TRY(cudaGetLastError());
  count_launch();
  return NEGF_OK;
}

int reduce_sites(int batch, int nsite_total, int nf, int nslots, const Item* items, const double* site_out,
                 double* acc, cudaStream_t st) {
  const long long n = (long long)nf * nsite_total * nslots;
  reduce_sites_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(batch, nsite_total, nf, nslots, items, site_out,
                                                                   acc);
  NEGF_CUDA_TRY(cudaGetLastError());
  count_launch();
  return NEGF_OK;
}

}  // namespace negf

// =====================================================================================
// mixed-form helpers: precision conversion and the Newton-Schulz residual
// =====================================================================================
namespace negf {

namespace {

__global__ void to_f32_kernel(int n, const double2* src, long long sS, float2* dst, long long sD) {
  const int b = blockIdx.y;
  const long long nn = (long long)n * n;
  const double2* s = src + (long long)b * sS;
  float2* d = dst + (long long)b * sD;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nn; e += (long long)gridDim.x * blockDim.x)
    d[e] = make_float2((float)s[e].x, (float)s[e].y);
}

// one read of the matrix to invert: its FP64 copy (kept for the residual) and FP32 copy
__global__ void split_copy_kernel(int n, const double2* src, long long sS, double2* d64, long long s64, float2* d32,
                                  long long s32) {
  const int b = blockIdx.y;
  const long long nn = (long long)n * n;
  const double2* s = src + (long long)b * sS;
  double2* a = d64 + (long long)b * s64;
  float2* c = d32 + (long long)b * s32;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nn; e += (long long)gridDim.x * blockDim.x) {
    const double2 v = s[e];
    a[e] = v;
    c[e] = make_float2((float)v.x, (float)v.y);
  }
}

__global__ void to_f64_kernel(int n, const float2* src, long long sS, double2* dst, long long sD) {
  const int b = blockIdx.y;
  const long long nn = (long long)n * n;
  const float2* s = src + (long long)b * sS;
  double2* d = dst + (long long)b * sD;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nn; e += (long long)gridDim.x * blockDim.x)
    d[e] = make_double2((double)s[e].x, (double)s[e].y);
}

// R = I - T in place; rnorm[b] = max over rows of sum_j |R_ij| (the infinity norm, the
// Newton-Schulz contraction factor).  A CTA covers 32 rows; its 8 thread rows stride over
// the columns (coalesced) and the row sums are reduced in shared memory in fixed order.
// |x| of a double as a float, truncated, from its bits with integer operations (below
// the float range -> 0, above -> inf, NaN -> NaN): the residual norm only decides whether
// a matrix takes more steps or an FP64 inverse, so float accuracy is enough, and the
// conversion instruction would run on the FP64 pipe
__device__ __forceinline__ float abs_to_float(double x) {
  const unsigned long long a = (unsigned long long)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFULL;
  const int E = (int)(a >> 52) - 1023 + 127;
  const unsigned int m = (unsigned int)(a >> 29) & 0x7FFFFFu;
  if ((a >> 52) == 0x7FF) return __uint_as_float(0x7F800000u | (m ? 0x400000u : 0u));
  if (E <= 0) return 0.0f;
  if (E >= 255) return __uint_as_float(0x7F800000u);
  return __uint_as_float(((unsigned int)E << 23) | m);
}

__global__ void ns_residual_kernel(int n, double2* T, long long sT, unsigned long long* rnorm) {
  __shared__ float part[8][32];
  const int b = blockIdx.y;
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int i = blockIdx.x * 32 + tx;
  float s = 0.0f;
  if (i < n) {
    double2* Tb = T + (long long)b * sT;
    for (int j = ty; j < n; j += 8) {
      double2 v = Tb[(long long)j * n + i];
      // R = I - T: a subtraction on the diagonal only, a sign flip elsewhere
      const double re = i == j ? 1.0 - v.x : __longlong_as_double(__double_as_longlong(v.x) ^ (long long)(1ULL << 63));
      v = make_double2(re, __longlong_as_double(__double_as_longlong(v.y) ^ (long long)(1ULL << 63)));
      Tb[(long long)j * n + i] = v;
      s += abs_to_float(v.x) + abs_to_float(v.y);
    }
  }
  part[ty][tx] = s;
  __syncthreads();
  if (ty == 0) {
    for (int q = 1; q < 8; ++q) s += part[q][tx];
    if (isnan(s)) s = 1e30f;
    // warp max, then one atomicMax per CTA on the bit pattern of the double (non-negative
    // doubles order as integers)
    for (int off = 16; off > 0; off >>= 1) s = fmaxf(s, __shfl_xor_sync(0xffffffffu, s, off));
    if (tx == 0) atomicMax(rnorm + b, (unsigned long long)__double_as_longlong((double)s));
  }
}

}  // namespace

int to_f32(int n, int batch, const double2* src, long long sS, float2* dst, long long sD, cudaStream_t st) {
  to_f32_kernel<<<ew_grid((long long)n * n, batch), EW_THREADS, 0, st>>>(n, src, sS, dst, sD);
  NEGF_CUDA_TRY(cudaGetLastError());
  count_launch();
  return NEGF_OK;
}

int split_copy(int n, int batch, const double2* src, long long sS, double2* d64, long long s64, float2* d32,
               long long s32, cudaStream_t st) {
  split_copy_kernel<<<ew_grid((long long)n * n, batch), EW_THREADS, 0, st>>>(n, src, sS, d64, s64, d32, s32);
  NEGF_CUDA_TRY(cudaGetLastError());
  count_launch();
  return NEGF_OK;
}

int to_f64(int n, int batch, const float2* src, long long sS, double2* dst, long long sD, cudaStream_t st) {
  to_f64_kernel<<<ew_grid((long long)n * n, batch), EW_THREADS, 0, st>>>(n, src, sS, dst, sD);
  NEGF_CUDA_TRY(cudaGetLastError());
  count_launch();
  return NEGF_OK;
}

namespace {
__global__ void gather_strided_kernel(int n, const double2* src, long long sSrc, const int* idx, double2* dst,
                                      long long sDst, int scatter) {
  const int i = blockIdx.y;
  const long long nn = (long long)n * n;
  const double2* s_ = scatter ? src + (long long)i * sSrc : src + (long long)idx[i] * sSrc;
  double2* d = scatter ? dst + (long long)idx[i] * sDst : dst + (long long)i * sDst;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nn; e += (long long)gridDim.x * blockDim.x)
    d[e] = s_[e];
}
}  // namespace

int gather_strided(int n, int count, const double2* src, long long sSrc, const int* idx, double2* dst, long long sDst,
                   cudaStream_t st) {
  if (count <= 0) return NEGF_OK;
  gather_strided_kernel<<<ew_grid((long long)n * n, count), EW_THREADS, 0, st>>>(n, src, sSrc, idx, dst, sDst, 0);
  NEGF_CUDA_TRY(cudaGetLastError());
  count_launch();
  return NEGF_OK;
}

int scatter_strided(int n, int count, const double2* src, long long sSrc, const int* idx, double2* dst,
                    long long sDst, cudaStream_t st) {
  if (count <= 0) return NEGF_OK;
  gather_strided_kernel<<<ew_grid((long long)n * n, count), EW_THREADS, 0, st>>>(n, src, sSrc, idx, dst, sDst, 1);
  NEGF_CUDA_TRY(cudaGetLastError());
  count_launch();
  return NEGF_OK;
}


int ns_residual(int n, int batch, double2* T, long long sT, unsigned long long* rnorm, cudaStream_t st) {
  dim3 grid((n + 31) / 32, batch);
  ns_residual_kernel<<<grid, dim3(32, 8), 0, st>>>(n, T, sT, rnorm);
  NEGF_CUDA_TRY(cudaGetLastError());
  count_launch();
  return NEGF_OK;
}

}  // namespace negf
