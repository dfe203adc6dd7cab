// Internal declarations shared by the translation units of libnegf_gb300.so.
//
// Device layout: every M x M complex block is column-major, interleaved double2
// (the memory layout of the reference's COMPLEX(8) arrays, Source/NEGF_Module.F90:56-75),
// so blocks cross the C ABI with a plain memcpy.
#pragma once

#include <cuda_runtime.h>
#include <atomic>
#include <cstdint>
#include <cstdio>
#include <mutex>
#include <vector>

#include "../../include/negf.h"

namespace negf {

// physical constants of Source/Constants.F90:4-6
constexpr double kQ = 1.602e-19;
constexpr double kH = 6.626e-34;
constexpr double kHbar = kH / (2.0 * 3.14159265358979323846);

// ----------------------------------------------------------------------------------
// complex helpers (double2 = (re, im))
// ----------------------------------------------------------------------------------
__host__ __device__ __forceinline__ double2 cmake(double r, double i) { return make_double2(r, i); }
__host__ __device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ __forceinline__ double2 cconj(double2 a) { return make_double2(a.x, -a.y); }
__host__ __device__ __forceinline__ double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
// acc += a * b
__host__ __device__ __forceinline__ void cfma(double2& acc, double2 a, double2 b) {
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(a.y, b.x, acc.y);
}
// 1 / a, scaled to avoid overflow in |a|^2
__host__ __device__ __forceinline__ double2 crcp(double2 a) {
  double s = fmax(fabs(a.x), fabs(a.y));
  if (s == 0.0) return make_double2(1.0 / 0.0, 0.0);
  double ar = a.x / s, ai = a.y / s;
  double d = s * (ar * ar + ai * ai);
  return make_double2(ar / d, -ai / d);
}
// |re| + |im|, the pivot measure of LAPACK izamax/dcabs1
__host__ __device__ __forceinline__ double cabs1(double2 a) { return fabs(a.x) + fabs(a.y); }

// single-precision twins (FP32 form of the inverse)
__host__ __device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
__host__ __device__ __forceinline__ void cfma(float2& acc, float2 a, float2 b) {
  acc.x = fmaf(a.x, b.x, acc.x);
  acc.x = fmaf(-a.y, b.y, acc.x);
  acc.y = fmaf(a.x, b.y, acc.y);
  acc.y = fmaf(a.y, b.x, acc.y);
}
__host__ __device__ __forceinline__ float2 crcp(float2 a) {
  float s = fmaxf(fabsf(a.x), fabsf(a.y));
  if (s == 0.0f) return make_float2(1.0f / 0.0f, 0.0f);
  float ar = a.x / s, ai = a.y / s;
  float d = s * (ar * ar + ai * ai);
  return make_float2(ar / d, -ai / d);
}
__host__ __device__ __forceinline__ float cabs1(float2 a) { return fabsf(a.x) + fabsf(a.y); }

template <typename T> struct CplxTraits;
template <> struct CplxTraits<double2> { using R = double; static __host__ __device__ double2 make(double r, double i) { return make_double2(r, i); } };
template <> struct CplxTraits<float2> { using R = float; static __host__ __device__ float2 make(float r, float i) { return make_float2(r, i); } };

// ----------------------------------------------------------------------------------
// error handling
// ----------------------------------------------------------------------------------
#define NEGF_CUDA_TRY(expr)                                                                 \
  do {                                                                                      \
    cudaError_t _e = (expr);                                                                \
    if (_e != cudaSuccess) {                                                                \
      ::negf::record_cuda_error(_e, #expr, __FILE__, __LINE__);                             \
      return NEGF_ECUDA;                                                                    \
    }                                                                                       \
  } while (0)

#define NEGF_TRY(expr)                                                                      \
  do {                                                                                      \
    int _s = (expr);                                                                        \
    if (_s < 0) return _s;                                                                  \
  } while (0)

void record_cuda_error(cudaError_t e, const char* what, const char* file, int line);
const char* last_cuda_error_text();

// ----------------------------------------------------------------------------------
// instrumentation (process-wide, shared by all handles and server workers: counters are
// atomic, the flop sums and the event bookkeeping are under `mu`)
// ----------------------------------------------------------------------------------
// kinds timed per launch (kernels) or per phase (PH_*), only while profiling is on
enum TimedKind {
  TK_GEMM = 0, TK_PANEL = 1, TK_TC = 2, TK_F32 = 3, TK_SLICE = 4,
  TK_PH_SR = 5, TK_PH_RGF = 6, TK_PH_INV = 7, TK_PH_DENS = 8, TK_COUNT = 9
};
struct Instrument {
  std::atomic<long long> launches{0};
  std::atomic<long long> kind_launches[TK_COUNT];
  std::mutex mu;
  double kind_flops[TK_COUNT] = {};
  std::atomic<bool> timing{false};
  struct Rec { cudaEvent_t a, b; int kind; };
  std::vector<Rec> pending;
  double kind_ms[TK_COUNT] = {};
  double tc_complex_flops = 0;
  std::vector<cudaEvent_t> pool;
  Instrument() { for (auto& k : kind_launches) k.store(0); }
};
Instrument& instrument();
inline void count_launch(int n = 1) { instrument().launches.fetch_add(n, std::memory_order_relaxed); }
void add_tc_complex_flops(double f);
// start/stop a timed region on `st` around one launch of `kind`
void timed_begin(cudaStream_t st, int kind, double flops, cudaEvent_t* a);
void timed_end(cudaStream_t st, int kind, cudaEvent_t a);
void instrument_resolve();   // accumulate the elapsed times of finished event pairs

// ----------------------------------------------------------------------------------
// GEMM: C = alpha * op(A) * op(B) + beta * C, strided batch (FP64 complex, SIMT DFMA)
// ----------------------------------------------------------------------------------
enum Op : int { OP_N = 0, OP_T = 1, OP_C = 2 };

template <typename T>
struct GemmBatchT {
  int m, n, k;
  T alpha, beta;
  const T* A; int lda; long long sA; Op opA;
  const T* B; int ldb; long long sB; Op opB;
  T* C; int ldc; long long sC;
  int batch;
};
using GemmBatch = GemmBatchT<double2>;
int zgemm_f64(const GemmBatch& g, cudaStream_t st);
int cgemm_f32(const GemmBatchT<float2>& g, cudaStream_t st);   // FP32 twin (inverse updates)

// ----------------------------------------------------------------------------------
// Batched in-place inverse (blocked Gauss-Jordan with partial row pivoting)
// ----------------------------------------------------------------------------------
struct InvWork {
  double2* rbuf = nullptr;   // batch * nb * n (FP64; reused as float2 storage by the FP32 form)
  int* ipiv = nullptr;       // batch * n
  int* info = nullptr;       // batch
  int n_cap = 0, batch_cap = 0, nb = 0;
  bool pooled = false;       // allocated stream-ordered from a memory pool
};
// pool = nullptr: plain cudaMalloc / cudaFree; otherwise stream-ordered on `st` from `pool`
int inv_work_alloc(InvWork& w, int n, int batch, cudaMemPool_t pool = nullptr, cudaStream_t st = 0);
void inv_work_free(InvWork& w, cudaStream_t st = 0);
int panel_width(int n, int elem_bytes = 16);
// A: batch matrices of n x n, column-major, consecutive at stride sA.  On return A holds
// the inverses; w.info[b] (device) holds the LAPACK-style INFO of each matrix.
int zinv_f64(double2* A, long long sA, int n, int batch, InvWork& w, cudaStream_t st);
// FP32 twin (the first guess of the mixed-form inverse).  form 0: panel / interchange /
// update launches per 32-column panel; form 1: one fused launch with a CTA per matrix (needs
// cinv_f32_fused_ok).  Both give bitwise the same result.
int cinv_f32(float2* A, long long sA, int n, int batch, InvWork& w, cudaStream_t st, int form = 0);
bool cinv_f32_fused_ok(int n, int batch);

// ----------------------------------------------------------------------------------
// per-item description of a batch (uploaded once per batch)
// ----------------------------------------------------------------------------------
struct Item {
  double energy;
  double f1, f2, dE;
  int slot;      // Hamiltonian slot
  int sr_l;      // Sancho-Rubio problem giving Sigma_L
  int sr_r;      // Sancho-Rubio problem giving Sigma_R
  int pad;
};

// ----------------------------------------------------------------------------------
// element-wise / structured kernels (ops.cu)
// ----------------------------------------------------------------------------------
// Block-diagonal hopping matrix, compact form: nsite blocks of norb x norb (row-major
// per block: hb[s*norb*norb + a*norb + b] = H(s*norb+a, s*norb+b)).
struct HopBD {
  const double2* hb = nullptr;
  int norb = 4, nsite = 0;
};

// W[b] = (E_b + i eta) I - Hslice[b] - (x==0 ? SigL[b] : 0) - (x==N-1 ? SigR[b] : 0)
//        - coupling term, where the coupling term is, if gprev != nullptr:
//          side 0:  H^H gprev[b] H    (left-connected sweep, Recursive_Greens.F90:18-20)
//          side 1:  H gprev[b] H^H    (right-connected sweep, Recursive_Greens.F90:70-72)
//        using the block-diagonal H, or, if zsub != nullptr, zsub[b] (dense path).
// A 4 x 4 hop block shared by every site, as compact terms per output index a: cnt[a]
// terms (p[a][t], c[a][t]) with Y_a = sum_t c x_p (left: c = op(H)(a, p); right:
// Y(i, a) = sum_t x_p c with c = op(H)(p, a)); kind 0 = real c, 1 = imaginary c,
// 2 = general.  Each list is sorted by kind, so that lanes of different rows take the same
// branches; the order of two terms can then differ from the dense fma sequence, which moves
// the last bit of a sum at most.
struct HopRows {
  int cnt[4];
  int p[4][4];
  int kind[4][4];
  double2 c[4][4];
};

struct FormW {
  int n, batch, npx, x;
  double eta;
  const Item* items;
  const double2* Hall;       // slots * npx * n*n
  const double2* sigL; long long sSig;   // per item, may be null
  const double2* sigR;
  const double2* gprev; long long sG;   // per item
  int side;
  HopBD hop;
  const double2* zsub; long long sZ;
  double2* W; long long sW;
  // every site shares one 4 x 4 hop block: the coupling term L G R from compact terms,
  // lrow = L by rows (left form), rrow = R by columns (right form)
  int use_rows = 0;
  HopRows lrow{}, rrow{};
};
int form_w(const FormW& a, cudaStream_t st);

// Y[b] = op(H) X[b] (left == 1) or X[b] op(H) (left == 0), H block diagonal; op in {N, C}.
// rows (may be null): the compact form of op(H) for that side when every site has the same
// 4 x 4 block.
int hop_apply(const HopBD& h, const HopRows* rows, int n, int batch, int left, Op op, const double2* X, long long sX,
              double2* Y, long long sY, cudaStream_t st);

// Site blocks of P = X Gamma X^H: P[b][r][a] = sum_k Y[b](r,k) conj(X[b](site(r)*norb + a, k)),
// with Y = X Gamma (precomputed).  Output stride per item sP (n*norb elements per slice).
int site_blocks(int n, int norb, int batch, const double2* Y, long long sY, const double2* X, long long sX,
                double2* P, long long sP, cudaStream_t st);

// site_blocks for the site itself (P), its +y neighbour (Py) and its +z neighbour (Pz) in one
// pass: Py[b][r][a] = sum_k Y[b](r,k) conj(X[b]((site(r)+1)*norb + a, k)), Pz with site + npy;
// zero where the neighbour is outside the slice.  Same layout and stride as site_blocks.
int site_pairs(int n, int norb, int npy, int npz, int batch, const double2* Y, long long sY, const double2* X,
               long long sX, double2* P, double2* Py, double2* Pz, long long sP, cudaStream_t st);

// out[b] = Re sum_ij Q[b](i,j) conj(X[b](i,j))   (trace of Q X^H), one value per item.
int trace_dot(int n, int batch, const double2* Q, long long sQ, const double2* X, long long sX,
              double* out, int out_stride, cudaStream_t st);

// gather per-item copies: dst[b] = src[idx[b]] (M x M blocks)
int gather_blocks(int n, int batch, const double2* src, const int* idx_dev, int idx_stride,
                  double2* dst, long long sDst, cudaStream_t st);

int copy_blocks(int n, int batch, const double2* src, long long sSrc, double2* dst, long long sDst, cudaStream_t st);
int set_identity(int n, int batch, double2* A, long long sA, cudaStream_t st);

// Sancho-Rubio helpers
struct SrProblem {
  double energy;
  const double2* h_end;  // the end slice H_1 (left) or H_N (right) used for alpha
  int want_l, want_r;
};
// A[s] = (E_s + i*(eta + extra_eta)) I - Hend[s]
int form_alpha(int n, int nprob, const double* energies, const double2* const* hend, double eta,
               double extra_eta, double2* A, long long sA, cudaStream_t st);
// T += (active[s] ? change : 0); cmax[s] = max |change| (NaN -> NaN)
int sr_accumulate(int n, int nprob, const int* active, const double2* change, long long sC, double2* T,
                  long long sT, double* cmax, cudaStream_t st);
// W = alpha - H^H T  (lead 0)   or  alpha - H T (lead 1) with block-diagonal H
int sr_form_final(const HopBD& h, int n, int nprob, int lead, const double2* alpha, long long sA,
                  const double2* T, long long sT, double2* W, long long sW, cudaStream_t st);
// Sigma = H^H g H (lead 0) or H g H^H (lead 1); Gamma = i (Sigma - Sigma^H); dos = -Im Tr Sigma / pi
int sr_sigma(const HopBD& h, int n, int nprob, int lead, const double2* g, long long sg, double2* sig,
             long long sSig, double2* gam, long long sGam, double* dos, cudaStream_t st);

// density / spin from the site blocks of both leads.  P1, P2: [item][x][n][norb].
// site_out: [item][nf][npx*npy*npz], fields 0..4 = (RhoN, RhoP, SigX, SigY, SigZ) already
// weighted by dE/(2 pi) (fields 5..7 = Jx, Jy, Jz when nf = 8, bond_currents);
// sums: [item][2] = (EDensity, HDensity).
struct DensityArgs {
  int n, norb, npx, npy, npz, batch, calc_spin, nf;
  int nh;                   // electron orbitals per site: EDensity/HDensity sum over them
  const Item* items;
  const double2* P1; const double2* P2; long long sP;
  const double2* spin_ops;  // 3 * norb*norb (row-major)
  double* site_out;         // batch * 5 * nsite_total
  double* sums;             // batch * 2
};
int density_spin(const DensityArgs& a, cudaStream_t st);

// bond currents into site_out fields 5..7 (Jx, Jy, Jz), dE/(2 pi)-weighted, from the
// neighbour blocks of both leads: Px[item][x][n][norb] = P(x, x+1; r, site(r)*norb + a),
// Py/Pz as site_pairs writes them; Hall as FormW, Hop = HopX (dense, column-major).
struct CurrentArgs {
  int n, norb, npx, npy, npz, batch, nf;
  int nh;                   // bond sums run over orbital pairs ii, jj < nh (electrons)
  const Item* items;
  const double2* Hall;
  const double2* Hop;
  const double2 *Px1, *Py1, *Pz1, *Px2, *Py2, *Pz2;
  long long sP;
  double q2_over_hbar;
  double* site_out;
  // energy- and orbital-resolved outputs (optional): er_out [item][4][npx*npy*npz] =
  // unweighted (ERJx, ERJy, ERJz, ERRhon); or_acc [slot][3 norb^2 + norb][npx*npy*npz] =
  // dE/(2 pi)-weighted (ORJx, ORJy, ORJz pairs ii*norb + jj, then ORRhon per orbital).
  // Both read the diagonal site blocks P1, P2 ([item][x][n][norb]).
  const double2 *P1 = nullptr, *P2 = nullptr;
  double* er_out = nullptr;
  double* or_acc = nullptr;
};
int bond_currents(const CurrentArgs& a, cudaStream_t st);
// or_acc[slot] += this batch's orbital-resolved sums for slots 0..nslots-1
int orbital_resolved(const CurrentArgs& a, int nslots, cudaStream_t st);

// model contacts: coef[job][lead][3] = (diag, up, lo), gds the nh x nh pairing structure
struct ContactGds {
  double2 m[4][4];
};
int contact_fill(int n, int no, int nh, int type, int ndiag, int njobs, const double2* coef, const ContactGds& g,
                 double2* sigL, double2* sigR, long long sS, cudaStream_t st);
// out[b][r][a] = X[b](r, site(r)*no + a)
int site_diag(int n, int no, int batch, const double2* X, long long sX, double2* out, long long sO, cudaStream_t st);
// supercurrent transmission per item (Calculate_Observables.F90:60-81), site-block-diagonal Sigma_L
int josephson(int n, int no, int batch, const Item* items, const double2* P1, const double2* P2, long long sP,
              const double2* G11, long long sG, const double2* sig, const double2* gam, long long sS, double* out,
              cudaStream_t st);

// acc[slot][f][i] += sum over items b with items[b].slot == slot (in order) of
// site_out[b][f][i], f < nf
int reduce_sites(int batch, int nsite_total, int nf, int nslots, const Item* items, const double* site_out,
                 double* acc, cudaStream_t st);

// mixed form: precision conversion and the Newton-Schulz residual R = I - T (in place),
// rnorm[b] = atomic max of the row-sum norm of R as the bit pattern of a double
int to_f32(int n, int batch, const double2* src, long long sS, float2* dst, long long sD, cudaStream_t st);
int to_f64(int n, int batch, const float2* src, long long sS, double2* dst, long long sD, cudaStream_t st);
int split_copy(int n, int batch, const double2* src, long long sS, double2* d64, long long s64, float2* d32,
               long long s32, cudaStream_t st);
int ns_residual(int n, int batch, double2* T, long long sT, unsigned long long* rnorm, cudaStream_t st);
// dst[i] = src[idx[i]] (gather) / dst[idx[i]] = src[i] (scatter) for i < count, n x n
// blocks at the given strides, idx on the device
int gather_strided(int n, int count, const double2* src, long long sSrc, const int* idx, double2* dst, long long sDst,
                   cudaStream_t st);
int scatter_strided(int n, int count, const double2* src, long long sSrc, const int* idx, double2* dst,
                    long long sDst, cudaStream_t st);

}  // namespace negf
