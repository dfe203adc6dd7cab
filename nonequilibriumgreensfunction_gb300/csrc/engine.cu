// Host orchestration of the per-energy NEGF solve (FP64 form).
//
// Mapping to the reference (all paths relative to the reference project):
//   solve_sr   - Contact_Self_Energy / Sancho_Rubio, Source/Contact_Self_Energy.F90:68-101,110-223
//   solve_rgf  - Energy_Sweep InvGRd assembly (Source/Energy_Sweep.F90:31-38) and
//                Get_Retarded_Greens (Source/Recursive_Greens.F90:2-107), fused with the
//                G Gamma G^H products of Calculate_Gnp (Source/Calculate_Gnp.F90:10-114)
//                and the trace of Calculate_Observables (Source/Calculate_Observables.F90:46-100)
//   densities  - Calculate_Gnp.F90:117-124 and Calculate_Observables.F90:10-43
//   batch_solve- the energy loop of Source/NEGF_Main.F90:21-27 and the MPI sums of
//                Source/MPI_Routines.F90:33-90, as one device pass per chunk of requests
//
// Algorithmic differences from the reference, all exact in exact arithmetic:
//  * Only the two block columns G(:,1), G(:,N) are formed; the backward GRd/GRu/GRl
//    recursion (Recursive_Greens.F90:37-51) is not needed because G(1,1) = gR_1 and
//    G(x+1,1) = gR_{x+1} H^H G(x,1) (the reference obtains G(2,1) from GRl(1) and then
//    overwrites it with the same recursion, :88-96).
//  * The right-connected sweep runs first and its blocks are overwritten in place by
//    the left-connected ones, so one Npx*M^2 block store per energy suffices.
//  * Gn/Gp are formed as P_c = G(:,c) Gamma_c G(:,c)^H restricted to the site blocks the
//    reductions read (diagonal norb x norb site blocks), Gn = f1 P_1 + f2 P_2 and
//    Gp = (1-f1) P_1 + (1-f2) P_2 (Calculate_Gnp.F90:10-114 with the scalars pulled out).
//  * When H_1 == H_N the two leads share one decimation: the right-lead recursion is the
//    left one with t and t~ exchanged (Contact_Self_Energy.F90:75,87), so the products
//    that involve only t, t~ are shared and each lead keeps its own T and stop test.
//  * HopX that is block diagonal in norb x norb site blocks (every channel built by
//    Source/Build_Hamiltonian.F90:59-64) is applied as a site-local operator.
#include "engine.h"

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstddef>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <utility>

namespace negf {

namespace {

constexpr int kSrBlocks = 13;
enum SrRole { SR_ALPHA = 0, SR_T, SR_TT, SR_TOLDL, SR_TOLDR, SR_TL, SR_TR, SR_TMP, SR_W1, SR_TN, SR_TTN, SR_CHG, SR_W2 };

__global__ void merge_info_k(int batch, const int* info, int* status) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < batch && status[b] == 0 && info[b] != 0) status[b] = info[b];
}

// Engines allocate from a library-private stream-ordered memory pool per device, with an
// unlimited release threshold: a freed engine's blocks stay in the pool and the next
// engine takes them without a new device allocation, and freeing (cudaFreeAsync) does not
// synchronise the device the way cudaFree does -- the serving layer creates and releases
// engines while other engines run.  negf_destroy trims the pool, so a plain handle returns
// its memory to the device.
std::mutex g_pool_mu;
cudaMemPool_t g_pool[64] = {};

int pool_for(int device, cudaMemPool_t* out) {
  if (device < 0 || device >= 64) return NEGF_EINVAL;
  std::lock_guard<std::mutex> g(g_pool_mu);
  if (!g_pool[device]) {
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    NEGF_CUDA_TRY(cudaMemPoolCreate(&g_pool[device], &props));
    uint64_t keep = ~0ULL;
    NEGF_CUDA_TRY(cudaMemPoolSetAttribute(g_pool[device], cudaMemPoolAttrReleaseThreshold, &keep));
  }
  *out = g_pool[device];
  return NEGF_OK;
}

// Pinned host staging buffers are kept for reuse as well (cudaFreeHost synchronises the
// device); a buffer of at least the requested size is taken from the free list.
std::mutex g_pin_mu;
std::multimap<size_t, void*> g_pin_free;
int pinned_take(size_t bytes, double** out, size_t* got) {
  {
    std::lock_guard<std::mutex> g(g_pin_mu);
    auto it = g_pin_free.lower_bound(bytes);
    if (it != g_pin_free.end()) {
      *out = static_cast<double*>(it->second);
      *got = it->first;
      g_pin_free.erase(it);
      return NEGF_OK;
    }
  }
  NEGF_CUDA_TRY(cudaMallocHost((void**)out, bytes));
  *got = bytes;
  return NEGF_OK;
}
void pinned_give(double* p, size_t bytes) {
  if (!p) return;
  std::lock_guard<std::mutex> g(g_pin_mu);
  g_pin_free.insert({bytes, p});
}

// device allocation of `count` T on stream `st` from `pool`, added to `bytes`; with `dry`
// only the bytes are counted
template <typename T>
int dalloc(T** p, size_t count, long long& bytes, bool dry, cudaMemPool_t pool, cudaStream_t st) {
  if (dry) { *p = nullptr; bytes += (long long)(sizeof(T) * count); return NEGF_OK; }
  if (count == 0) { *p = nullptr; return NEGF_OK; }
  if (cudaMallocFromPoolAsync((void**)p, sizeof(T) * count, pool, st) != cudaSuccess) {
    *p = nullptr;
    return NEGF_ENOMEM;
  }
  bytes += (long long)(sizeof(T) * count);
  return NEGF_OK;
}
template <typename T>
void dfree(T*& p, cudaStream_t st) {
  if (p) cudaFreeAsync((void*)p, st);
  p = nullptr;
}

bool blocks_equal(const double2* a, const double2* b, size_t n) { return std::memcmp(a, b, n * sizeof(double2)) == 0; }

double __longlong_as_double_host(unsigned long long v) {
  double d;
  std::memcpy(&d, &v, sizeof(d));
  return d;
}

}  // namespace

int merge_info_kernel_launch(int batch, const int* info, int* status, cudaStream_t st) {
  merge_info_k<<<(batch + 127) / 128, 128, 0, st>>>(batch, info, status);
  NEGF_CUDA_TRY(cudaGetLastError());
  count_launch();
  return NEGF_OK;
}

Engine::~Engine() {
  if (!own_st_) return;   // never initialised (or only sized by estimate_bytes)
  cudaSetDevice(p_.device);
  // nothing of this engine may still run when its blocks go back to the pool
  if (st_ && st_ != own_st_) cudaStreamSynchronize(st_);
  cudaStreamSynchronize(own_st_);
  cudaStream_t s = own_st_;
  dfree(dH_, s); dfree(dHop_, s); dfree(dHopBD_, s); dfree(dSpin_, s); dfree(dHtab_, s); dfree(dVext_, s);
  dfree(dG_, s); dfree(dC1_, s); dfree(dCN_, s); dfree(dZ_, s); dfree(dY_, s); dfree(dQ_, s);
  dfree(dSigL_, s); dfree(dSigR_, s); dfree(dGamL_, s); dfree(dGamR_, s);
  dfree(dP1_, s); dfree(dP2_, s); dfree(dCol1_, s); dfree(dColN_, s);
  dfree(dPx1_, s); dfree(dPy1_, s); dfree(dPz1_, s); dfree(dPx2_, s); dfree(dPy2_, s); dfree(dPz2_, s);
  if (currents_) { dfree(dYalt_, s); dfree(dCNalt_, s); }
  dfree(dEr_, s); dfree(dOrAcc_, s); dfree(dContactCoef_, s); dfree(dG11_, s); dfree(dTrJ_, s);
  dfree(dSite_, s); dfree(dSums_, s); dfree(dTr_, s); dfree(dAcc_, s); dfree(dStatus_, s); dfree(dItems_, s);
  dfree(dSr_, s); dfree(dSrSigL_, s); dfree(dSrSigR_, s); dfree(dSrGamL_, s); dfree(dSrGamR_, s);
  dfree(dSrCmax_, s); dfree(dSrDos_, s); dfree(dSrActive_, s); dfree(dSrE_, s); dfree(dSrHend_, s);
  dfree(dSrStatus_, s);
  inv_work_free(inv_, s);
  dfree(dWinv_, s); dfree(dW32_, s); dfree(dT_, s); dfree(sa_.data, s); dfree(sb_.data, s); dfree(sa_.exps, s);
  dfree(sb_.exps, s); dfree(sw_.data, s); dfree(sw_.exps, s); dfree(sgl_.data, s); dfree(sgl_.exps, s);
  dfree(sgr_.data, s); dfree(sgr_.exps, s);
  dfree(dRnorm_, s); dfree(dNsIdx_, s); dfree(dNsX_, s); dfree(dNsW_, s); dfree(dTcErr_, s);
  cudaStreamSynchronize(own_st_);   // the frees have run: the blocks are back in the pool
  pinned_give(hPin_, hPinBytes_);
  cudaStreamDestroy(own_st_);
}

int pool_trim(int device) {
  cudaMemPool_t pool;
  NEGF_TRY(pool_for(device, &pool));
  NEGF_CUDA_TRY(cudaMemPoolTrimTo(pool, 0));
  return NEGF_OK;
}

int Engine::configure(const negf_params& p) {
  if (p.npx < 2 || p.npy < 1 || p.npz < 1 || p.norb < 1 || p.norb > 8) return NEGF_EINVAL;
  if (p.contact_type < NEGF_CONTACT_LEADS || p.contact_type > NEGF_CONTACT_SC || p.reserved1 != 0) return NEGF_EINVAL;
  for (int i = 0; i < 8; ++i)
    if (p.reserved2[i] != 0) return NEGF_EINVAL;
  // SC contacts act on a BdG Hamiltonian: nh electron orbitals, then their holes
  const int nh = p.contact_type == NEGF_CONTACT_SC ? p.norb / 2 : p.norb;
  if (p.contact_type == NEGF_CONTACT_SC && (p.norb % 2 != 0 || nh > 4)) return NEGF_EINVAL;
  if (p.calc_spin && nh > 4) return NEGF_EINVAL;
  if (!(p.tunneling_rate >= 0.0) || !std::isfinite(p.delta_sc[0]) || !std::isfinite(p.delta_sc[1]) ||
      !std::isfinite(p.chi_lr))
    return NEGF_EINVAL;
  if (p.n_hamiltonians < 1 || p.max_batch < 1 || p.max_batch > 4096) return NEGF_EINVAL;
  if (!(p.eta >= 0.0) || !(p.sr_tol > 0.0) || p.sr_max_iter < 1) return NEGF_EINVAL;
  if (p.precision != NEGF_PREC_FP64 && p.precision != NEGF_PREC_MIXED) return NEGF_EINVAL;
  if (p.precision == NEGF_PREC_MIXED && p.mixed_slices != 0 && !tc_supported_slices(p.mixed_slices))
    return NEGF_EINVAL;
  // the tensor-core products keep exact accumulators up to K' = 2 M = 1600
  if (p.precision == NEGF_PREC_MIXED && 2 * padded_k(p.norb * p.npy * p.npz) > 1600) return NEGF_EINVAL;
  p_ = p;
  M_ = p.norb * p.npy * p.npz;
  MM_ = (long long)M_ * M_;
  nsite_ = p.npy * p.npz;
  B_ = p.max_batch;
  S_ = 2 * p.max_batch;
  keep_columns_ = p.keep_g_columns != 0;
  currents_ = p.calc_currents != 0;
  nh_ = nh;
  nf_ = currents_ ? 8 : 5;
  mixed_ = p.precision == NEGF_PREC_MIXED;
  if (mixed_ && p.mixed_slices != 0) s_rgf_ = p.mixed_slices;
  if (mixed_ && p.sr_slices != 0) {
    if (p.sr_slices < 5 || p.sr_slices > 8) return NEGF_EINVAL;
    s_sr_ = p.sr_slices;
  }
  if (mixed_ && p.residual_slices != 0) {
    if (p.residual_slices < 5 || p.residual_slices > 8) return NEGF_EINVAL;
    s_res_ = p.residual_slices;
  }
  return NEGF_OK;
}

long long Engine::estimate_bytes(const negf_params& p) {
  Engine e;
  if (e.configure(p) != NEGF_OK) return -1;
  e.dry_ = true;
  if (e.alloc() != NEGF_OK) return -1;
  return e.bytes_;
}

int Engine::init(const negf_params& p) {
  NEGF_TRY(configure(p));
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return NEGF_ENODEV;
  if (p.device < 0 || p.device >= ndev) return NEGF_EINVAL;
  NEGF_CUDA_TRY(cudaSetDevice(p.device));
  NEGF_CUDA_TRY(cudaStreamCreateWithFlags(&own_st_, cudaStreamNonBlocking));
  st_ = own_st_;
  slot_set_.assign(p.n_hamiltonians, 0);
  slot_rep_.assign(p.n_hamiltonians, 0);
  slot_joint_.assign(p.n_hamiltonians, 0);
  end_h1_.assign(p.n_hamiltonians, {});
  end_hn_.assign(p.n_hamiltonians, {});
  return alloc();
}

int Engine::alloc() {
  if (!dry_) NEGF_TRY(pool_for(p_.device, &pool_));
  const long long N = p_.npx;
  const long long total = nsite_total();
  NEGF_TRY(dalloc(&dH_, (size_t)(p_.n_hamiltonians * N * MM_), bytes_, dry_, pool_, own_st_));
  NEGF_TRY(dalloc(&dHop_, (size_t)MM_, bytes_, dry_, pool_, own_st_));
  NEGF_TRY(dalloc(&dHopBD_, (size_t)nsite_ * p_.norb * p_.norb, bytes_, dry_, pool_, own_st_));
  NEGF_TRY(dalloc(&dSpin_, (size_t)3 * p_.norb * p_.norb, bytes_, dry_, pool_, own_st_));
  NEGF_TRY(dalloc(&dHtab_, (size_t)16 * (2 + p_.npz), bytes_, dry_, pool_, own_st_));
  NEGF_TRY(dalloc(&dVext_, (size_t)total, bytes_, dry_, pool_, own_st_));
  NEGF_TRY(dalloc(&dG_, (size_t)(B_ * N * MM_), bytes_, dry_, pool_, own_st_));
  double2** bufs[] = {&dC1_, &dCN_, &dZ_, &dY_, &dQ_, &dSigL_, &dSigR_, &dGamL_, &dGamR_};
  for (double2** b : bufs) NEGF_TRY(dalloc(b, (size_t)(B_ * MM_), bytes_, dry_, pool_, own_st_));
  NEGF_TRY(dalloc(&dP1_, (size_t)(B_ * N * M_ * p_.norb), bytes_, dry_, pool_, own_st_));
  NEGF_TRY(dalloc(&dP2_, (size_t)(B_ * N * M_ * p_.norb), bytes_, dry_, pool_, own_st_));
  if (keep_columns_) {
    NEGF_TRY(dalloc(&dCol1_, (size_t)(N * MM_), bytes_, dry_, pool_, own_st_));
    NEGF_TRY(dalloc(&dColN_, (size_t)(N * MM_), bytes_, dry_, pool_, own_st_));
  }
  if (currents_) {
    double2** pb[] = {&dPx1_, &dPy1_, &dPz1_, &dPx2_, &dPy2_, &dPz2_};
    for (double2** b : pb) NEGF_TRY(dalloc(b, (size_t)(B_ * N * M_ * p_.norb), bytes_, dry_, pool_, own_st_));
    NEGF_TRY(dalloc(&dYalt_, (size_t)(B_ * MM_), bytes_, dry_, pool_, own_st_));
    NEGF_TRY(dalloc(&dCNalt_, (size_t)(B_ * MM_), bytes_, dry_, pool_, own_st_));
    // the x bond of the last slice does not exist: its blocks stay zero
    if (!dry_)
      for (double2* b : {dPx1_, dPx2_})
        NEGF_CUDA_TRY(cudaMemsetAsync(b, 0, sizeof(double2) * (size_t)(B_ * N * M_ * p_.norb), own_st_));
  } else {
    dYalt_ = dY_;
    dCNalt_ = dCN_;
  }
  sums_blocks_ = (int)((total + 255) / 256);
  if (p_.contact_type != NEGF_CONTACT_LEADS) NEGF_TRY(dalloc(&dContactCoef_, (size_t)S_ * 6, bytes_, dry_, pool_, own_st_));
  if (sc_()) {
    NEGF_TRY(dalloc(&dG11_, (size_t)B_ * M_ * p_.norb, bytes_, dry_, pool_, own_st_));
    NEGF_TRY(dalloc(&dTrJ_, (size_t)B_, bytes_, dry_, pool_, own_st_));
  }
  NEGF_TRY(dalloc(&dSite_, (size_t)(B_ * nf_ * total), bytes_, dry_, pool_, own_st_));
  NEGF_TRY(dalloc(&dSums_, (size_t)B_ * sums_blocks_ * 2, bytes_, dry_, pool_, own_st_));
  NEGF_TRY(dalloc(&dTr_, (size_t)B_ * 4, bytes_, dry_, pool_, own_st_));
  NEGF_TRY(dalloc(&dAcc_, (size_t)(p_.n_hamiltonians * nf_ * total), bytes_, dry_, pool_, own_st_));
  NEGF_TRY(dalloc(&dStatus_, (size_t)B_, bytes_, dry_, pool_, own_st_));
  NEGF_TRY(dalloc(&dItems_, (size_t)B_, bytes_, dry_, pool_, own_st_));
  NEGF_TRY(dalloc(&dSr_, (size_t)(kSrBlocks * S_ * MM_), bytes_, dry_, pool_, own_st_));
  double2** srb[] = {&dSrSigL_, &dSrSigR_, &dSrGamL_, &dSrGamR_};
  for (double2** b : srb) NEGF_TRY(dalloc(b, (size_t)(S_ * MM_), bytes_, dry_, pool_, own_st_));
  NEGF_TRY(dalloc(&dSrCmax_, (size_t)2 * S_, bytes_, dry_, pool_, own_st_));
  NEGF_TRY(dalloc(&dSrDos_, (size_t)2 * S_, bytes_, dry_, pool_, own_st_));
  NEGF_TRY(dalloc(&dSrActive_, (size_t)2 * S_, bytes_, dry_, pool_, own_st_));
  NEGF_TRY(dalloc(&dSrE_, (size_t)S_, bytes_, dry_, pool_, own_st_));
  NEGF_TRY(dalloc(&dSrHend_, (size_t)S_, bytes_, dry_, pool_, own_st_));
  NEGF_TRY(dalloc(&dSrStatus_, (size_t)S_, bytes_, dry_, pool_, own_st_));
  {   // inv_work_alloc: R buffer, pivots, INFO
    const long long cap = std::max(B_, S_);
    if (!dry_) NEGF_TRY(inv_work_alloc(inv_, M_, (int)cap, pool_, own_st_));
    bytes_ += 16LL * cap * panel_width(M_) * M_ + 4LL * cap * M_ + 4LL * cap;
  }
  if (mixed_) {
    const int cap = std::max(B_, S_);
    const int smax = 8;   // every slice count a phase may use (RGF, Sancho-Rubio, residual: <= 8)
    NEGF_TRY(dalloc(&dWinv_, (size_t)(cap * MM_), bytes_, dry_, pool_, own_st_));
    NEGF_TRY(dalloc(&dW32_, (size_t)(cap * MM_), bytes_, dry_, pool_, own_st_));
    NEGF_TRY(dalloc(&dT_, (size_t)(cap * MM_), bytes_, dry_, pool_, own_st_));
    const int kp = padded_k(M_);
    NEGF_TRY(dalloc(reinterpret_cast<char**>(&sa_.data), sliced_bytes_a(M_, kp, smax, cap), bytes_, dry_, pool_, own_st_));
    NEGF_TRY(dalloc(reinterpret_cast<char**>(&sb_.data), sliced_bytes_b(M_, kp, smax, cap), bytes_, dry_, pool_, own_st_));
    NEGF_TRY(dalloc(reinterpret_cast<char**>(&sw_.data), sliced_bytes_a(M_, kp, smax, cap), bytes_, dry_, pool_, own_st_));
    NEGF_TRY(dalloc(&sw_.exps, (size_t)cap * M_, bytes_, dry_, pool_, own_st_));
    NEGF_TRY(dalloc(&sa_.exps, (size_t)cap * M_, bytes_, dry_, pool_, own_st_));
    NEGF_TRY(dalloc(&sb_.exps, (size_t)cap * M_, bytes_, dry_, pool_, own_st_));
    NEGF_TRY(dalloc(reinterpret_cast<char**>(&sgl_.data), sliced_bytes_b(M_, kp, s_rgf_, B_), bytes_, dry_, pool_, own_st_));
    NEGF_TRY(dalloc(reinterpret_cast<char**>(&sgr_.data), sliced_bytes_b(M_, kp, s_rgf_, B_), bytes_, dry_, pool_, own_st_));
    NEGF_TRY(dalloc(&sgl_.exps, (size_t)B_ * M_, bytes_, dry_, pool_, own_st_));
    NEGF_TRY(dalloc(&sgr_.exps, (size_t)B_ * M_, bytes_, dry_, pool_, own_st_));
    sgl_.data_bytes = sgr_.data_bytes = sliced_bytes_b(M_, kp, s_rgf_, B_);
    sgl_.exps_count = sgr_.exps_count = (size_t)B_ * M_;
    sa_.data_bytes = sw_.data_bytes = sliced_bytes_a(M_, kp, smax, cap);
    sb_.data_bytes = sliced_bytes_b(M_, kp, smax, cap);
    sa_.exps_count = sb_.exps_count = sw_.exps_count = (size_t)cap * M_;
    NEGF_TRY(dalloc(&dRnorm_, (size_t)cap, bytes_, dry_, pool_, own_st_));
    NEGF_TRY(dalloc(&dNsIdx_, (size_t)cap, bytes_, dry_, pool_, own_st_));
    NEGF_TRY(dalloc(&dNsX_, (size_t)cap * MM_, bytes_, dry_, pool_, own_st_));
    NEGF_TRY(dalloc(&dNsW_, (size_t)cap * MM_, bytes_, dry_, pool_, own_st_));
    NEGF_TRY(dalloc(&dTcErr_, (size_t)1, bytes_, dry_, pool_, own_st_));
    if (!dry_) NEGF_CUDA_TRY(cudaMemsetAsync(dTcErr_, 0, sizeof(int), own_st_));
  }
  if (dry_) return NEGF_OK;   // estimate_bytes: device bytes only
  hPinBytes_ = sizeof(double) * (size_t)std::max<long long>(
                   {(long long)B_ * sums_blocks_ * 2, (long long)B_ * 4, 4LL * S_,
                    (long long)p_.n_hamiltonians * nf_ * total, (long long)nf_ * total, 64});
  NEGF_TRY(pinned_take(hPinBytes_, &hPin_, &hPinBytes_));
  // the allocations are ordered on the engine's stream; after this they are usable from
  // any stream (the caller's, through negf_set_stream) and by the synchronous copies below
  NEGF_CUDA_TRY(cudaStreamSynchronize(own_st_));
  // spin operators, by default those of Source/Read_In_Allocate.F90 for nh electron orbitals:
  // tau0 (x) sigma_j for nh = 4 (:183-196), the Pauli matrices for nh = 2 (:205-216), zero
  // otherwise (:151-159)
  std::vector<double2> spin(3 * p_.norb * p_.norb, make_double2(0.0, 0.0));
  bool any = false;
  for (int j = 0; j < 3; ++j)
    for (int r = 0; r < 4; ++r)
      for (int c = 0; c < 4; ++c)
        if (p_.spin_ops[j][r][c][0] != 0.0 || p_.spin_ops[j][r][c][1] != 0.0) any = true;
  // the operators act on the nh electron orbitals of a site (Calculate_Observables.F90:14-15);
  // with SC contacts the hole block of the BdG site stays zero
  const int no = p_.norb, ne = nh_;
  if (any) {
    for (int j = 0; j < 3; ++j)
      for (int r = 0; r < ne; ++r)
        for (int c = 0; c < ne; ++c)
          spin[(j * no + r) * no + c] = make_double2(p_.spin_ops[j][r][c][0], p_.spin_ops[j][r][c][1]);
  } else if (ne == 4) {
    // sigma_x, sigma_y, sigma_z on the spin index (orbital = 2*tau + sigma)
    const double2 one = make_double2(1, 0), mi = make_double2(0, -1), pi_ = make_double2(0, 1), m1 = make_double2(-1, 0);
    auto at = [&](int j, int r, int c) -> double2& { return spin[(j * no + r) * no + c]; };
    for (int blk = 0; blk < 2; ++blk) {
      const int o = 2 * blk;
      at(0, o, o + 1) = one; at(0, o + 1, o) = one;
      at(1, o, o + 1) = mi;  at(1, o + 1, o) = pi_;
      at(2, o, o) = one;     at(2, o + 1, o + 1) = m1;
    }
  } else if (ne == 2) {
    const double2 one = make_double2(1, 0), mi = make_double2(0, -1), pi_ = make_double2(0, 1), m1 = make_double2(-1, 0);
    auto at = [&](int j, int r, int c) -> double2& { return spin[(j * no + r) * no + c]; };
    at(0, 0, 1) = one; at(0, 1, 0) = one;
    at(1, 0, 1) = mi;  at(1, 1, 0) = pi_;
    at(2, 0, 0) = one; at(2, 1, 1) = m1;
  }
  NEGF_CUDA_TRY(cudaMemcpy(dSpin_, spin.data(), sizeof(double2) * spin.size(), cudaMemcpyHostToDevice));
  return NEGF_OK;
}

int Engine::set_hopx(const double2* hx) {
  if (hop_set_) {
    std::vector<double2> cur(MM_);
    NEGF_CUDA_TRY(cudaMemcpy(cur.data(), dHop_, sizeof(double2) * MM_, cudaMemcpyDeviceToHost));
    // a different HopX invalidates every slot uploaded with the old one
    if (!blocks_equal(cur.data(), hx, MM_)) std::fill(slot_set_.begin(), slot_set_.end(), 0);
  }
  NEGF_CUDA_TRY(cudaMemcpy(dHop_, hx, sizeof(double2) * MM_, cudaMemcpyHostToDevice));
  // block-diagonal detection (site blocks of norb x norb)
  const int no = p_.norb;
  bool bd = true;
  for (int j = 0; j < M_ && bd; ++j)
    for (int i = 0; i < M_; ++i) {
      if (i / no == j / no) continue;
      const double2 v = hx[(long long)j * M_ + i];
      if (v.x != 0.0 || v.y != 0.0) { bd = false; break; }
    }
  hop_bd_ = bd;
  if (bd) {
    std::vector<double2> hb((size_t)nsite_ * no * no);
    for (int s = 0; s < nsite_; ++s)
      for (int a = 0; a < no; ++a)
        for (int c = 0; c < no; ++c) hb[((size_t)s * no + a) * no + c] = hx[(long long)(s * no + c) * M_ + s * no + a];
    NEGF_CUDA_TRY(cudaMemcpy(dHopBD_, hb.data(), sizeof(double2) * hb.size(), cudaMemcpyHostToDevice));
    hop_uniform_ = no == 4;
    for (size_t e = 16; e < hb.size() && hop_uniform_; ++e)
      if (hb[e].x != hb[e % 16].x || hb[e].y != hb[e % 16].y) hop_uniform_ = false;
    if (hop_uniform_) {
      // op(H)(a, p) from the site block H(a, p) = hb[a * 4 + p]
      auto opH = [&](int opc, int a, int p) {
        const double2 v = opc ? hb[p * 4 + a] : hb[a * 4 + p];
        return opc ? make_double2(v.x, -v.y) : v;
      };
      for (int left = 0; left < 2; ++left)
        for (int opc = 0; opc < 2; ++opc) {
          HopRows& r = hop_rows_[left][opc];
          for (int a = 0; a < 4; ++a) {
            int cnt = 0;
            for (int kind = 0; kind < 3; ++kind)
              for (int p = 0; p < 4; ++p) {
                // left: Y_a = sum_p op(H)(a, p) x_p; right: Y_a = sum_p x_p op(H)(p, a)
                const double2 c = left ? opH(opc, a, p) : opH(opc, p, a);
                const int k = (c.x != 0.0 && c.y != 0.0) ? 2 : (c.x != 0.0 ? 0 : (c.y != 0.0 ? 1 : -1));
                if (k != kind) continue;
                r.p[a][cnt] = p; r.kind[a][cnt] = k; r.c[a][cnt] = c; ++cnt;
              }
            r.cnt[a] = cnt;
          }
        }
    }
  } else {
    hop_uniform_ = false;
  }
  hop_set_ = true;
  return NEGF_OK;
}

int Engine::set_hamiltonian(int slot, const double* Htotd, const double* HopX) {
  if (slot < 0 || slot >= p_.n_hamiltonians || !Htotd) return NEGF_EINVAL;
  if (!hop_set_ && !HopX) return NEGF_EINVAL;
  NEGF_CUDA_TRY(cudaSetDevice(p_.device));
  const double2* h = reinterpret_cast<const double2*>(Htotd);
  const long long N = p_.npx;
  if (HopX) NEGF_TRY(set_hopx(reinterpret_cast<const double2*>(HopX)));
  NEGF_CUDA_TRY(cudaMemcpy(dH_ + (long long)slot * N * MM_, h, sizeof(double2) * N * MM_, cudaMemcpyHostToDevice));
  end_h1_[slot].assign(h, h + MM_);
  end_hn_[slot].assign(h + (N - 1) * MM_, h + N * MM_);
  slot_set_[slot] = 1;
  recompute_lead_classes();
  sr_valid_ = rgf_valid_ = dens_valid_ = false;
  return NEGF_OK;
}

void Engine::recompute_lead_classes() {
  const int ns = p_.n_hamiltonians;
  for (int s = 0; s < ns; ++s) {
    slot_rep_[s] = s;
    slot_joint_[s] = 0;
    if (!slot_set_[s]) continue;
    slot_joint_[s] = blocks_equal(end_h1_[s].data(), end_hn_[s].data(), MM_) ? 1 : 0;
    for (int r = 0; r < s; ++r) {
      if (!slot_set_[r] || slot_rep_[r] != r) continue;
      if (blocks_equal(end_h1_[r].data(), end_h1_[s].data(), MM_) &&
          blocks_equal(end_hn_[r].data(), end_hn_[s].data(), MM_)) {
        slot_rep_[s] = r;
        break;
      }
    }
  }
}

int Engine::gemm_tc_nn(int batch, const double2* A, long long sA, const double2* B, long long sB, double2* C,
                       long long sC, double2 alpha, double2 beta, int slices) {
  NEGF_TRY(slice_a(A, M_, sA, M_, M_, batch, slices, sa_, st_));
  NEGF_TRY(slice_b(B, M_, sB, M_, M_, batch, slices, sb_, st_));
  return zgemm_tc(sa_, sb_, alpha, beta, C, M_, sC, dTcErr_, st_);
}

// C = A G with G's B-operand slicing made once per sweep (Gamma_L, Gamma_R); FP64 form:
// a plain product with G itself
int Engine::gemm_gamma(int batch, const double2* A, long long sA, const double2* G, const SlicedOperand& sg,
                       double2* C, long long sC) {
  const double2 one = make_double2(1, 0), zero = make_double2(0, 0);
  if (!mixed_) return gemm(batch, OP_N, A, sA, OP_N, G, MM_, C, sC, one, zero);
  NEGF_TRY(slice_a(A, M_, sA, M_, M_, batch, s_rgf_, sa_, st_));
  return zgemm_tc(sa_, sg, one, zero, C, M_, sC, dTcErr_, st_);
}

int Engine::gemm(int batch, Op opA, const double2* A, long long sA, Op opB, const double2* B, long long sB, double2* C,
                 long long sC, double2 alpha, double2 beta) {
  if (mixed_ && opA == OP_N && opB == OP_N && sA != 0 && sB != 0)
    return gemm_tc_nn(batch, A, sA, B, sB, C, sC, alpha, beta, cur_slices_);
  GemmBatch g{};
  g.m = M_; g.n = M_; g.k = M_;
  g.alpha = alpha; g.beta = beta;
  g.A = A; g.lda = M_; g.sA = sA; g.opA = opA;
  g.B = B; g.ldb = M_; g.sB = sB; g.opB = opB;
  g.C = C; g.ldc = M_; g.sC = sC;
  g.batch = batch;
  return zgemm_f64(g, st_);
}

int Engine::hop_mul(int left, Op op, const double2* X, long long sX, double2* Y, long long sY, int batch) {
  if (hop_bd_)
    return hop_apply(hop(), hop_uniform_ ? &hop_rows_[left ? 1 : 0][op == OP_C ? 1 : 0] : nullptr, M_, batch, left, op,
                     X, sX, Y, sY, st_);
  const double2 one = make_double2(1, 0), zero = make_double2(0, 0);
  if (left) return gemm(batch, op, dHop_, 0, OP_N, X, sX, Y, sY, one, zero);
  return gemm(batch, OP_N, X, sX, op, dHop_, 0, Y, sY, one, zero);
}

int Engine::merge_info(int batch) { return merge_info_kernel_launch(batch, inv_.info, dStatus_, st_); }

// In-place inverse of `batch` matrices at stride sA; INFO of singular ones merged into
// status_dev.  FP64 form: blocked Gauss-Jordan.  Mixed form: FP32 Gauss-Jordan, then
// ns_steps_ Newton-Schulz steps X <- X + X (I - W X) with W X formed at s_res_ slices
// (FP64-class) and X R at s_upd_ slices, and up to ns_max_steps_ in all for a matrix whose
// residual norm before its last update is above ns_tol_.  A matrix is inverted again in
// FP64 when its first residual norm is above ns_accept_, its FP32 factorisation met a zero
// pivot, or it is still above ns_tol_ after ns_max_steps_ steps.
int Engine::invert(double2* A, long long sA, int batch, int* status_dev) {
  cudaEvent_t ph;
  timed_begin(st_, TK_PH_INV, 0.0, &ph);
  const int rc = invert_impl(A, sA, batch, status_dev);
  timed_end(st_, TK_PH_INV, ph);
  return rc;
}

int Engine::invert_impl(double2* A, long long sA, int batch, int* status_dev) {
  if (!mixed_) {
    NEGF_TRY(zinv_f64(A, sA, M_, batch, inv_, st_));
    return merge_info_kernel_launch(batch, inv_.info, status_dev, st_);
  }
  const double2 one = make_double2(1, 0), zero = make_double2(0, 0);
  NEGF_TRY(split_copy(M_, batch, A, sA, dWinv_, MM_, dW32_, MM_, st_));
  NEGF_TRY(invert_f32(batch));
  NEGF_TRY(to_f64(M_, batch, dW32_, MM_, A, sA, st_));
  std::vector<int> info32(batch);
  NEGF_CUDA_TRY(cudaMemcpyAsync(info32.data(), inv_.info, sizeof(int) * batch, cudaMemcpyDeviceToHost, st_));
  NEGF_CUDA_TRY(cudaMemsetAsync(dRnorm_, 0, sizeof(unsigned long long) * batch, st_));
  NEGF_TRY(slice_a(dWinv_, M_, MM_, M_, M_, batch, s_res_, sw_, st_));
  std::vector<unsigned long long> r0(batch), rk(batch);
  // ns_steps_ steps for the whole batch
  for (int step = 0; step < ns_steps_; ++step) {
    if (step > 0) NEGF_CUDA_TRY(cudaMemsetAsync(dRnorm_, 0, sizeof(unsigned long long) * batch, st_));
    // the first residual only has to be good to the square root of the target (the next
    // step squares the error), so it takes s_res0_ slices: the leading planes of W's slicing
    const int sr = (step == 0 && ns_steps_ > 1) ? s_res0_ : s_res_;
    NEGF_TRY(slice_b(A, M_, sA, M_, M_, batch, sr, sb_, st_));
    NEGF_TRY(zgemm_tc(sw_, sb_, one, zero, dT_, M_, MM_, dTcErr_, st_, sr));    // T = W X
    NEGF_TRY(ns_residual(M_, batch, dT_, MM_, dRnorm_, st_));                     // R = I - T
    if (step == 0)
      NEGF_CUDA_TRY(cudaMemcpyAsync(r0.data(), dRnorm_, sizeof(unsigned long long) * batch, cudaMemcpyDeviceToHost, st_));
    if (step == ns_steps_ - 1)
      NEGF_CUDA_TRY(cudaMemcpyAsync(rk.data(), dRnorm_, sizeof(unsigned long long) * batch, cudaMemcpyDeviceToHost, st_));
    NEGF_TRY(slice_a(A, M_, sA, M_, M_, batch, s_upd_, sa_, st_));
    NEGF_TRY(slice_b(dT_, M_, MM_, M_, M_, batch, s_upd_, sb_, st_));
    // X += X R; dT_ (R, already sliced) lends itself as the autotuner's scratch output
    NEGF_TRY(zgemm_tc(sa_, sb_, one, one, A, M_, sA, dTcErr_, st_, 0, dT_));
  }
  NEGF_CUDA_TRY(cudaStreamSynchronize(st_));
  // Further steps only for the matrices whose residual norm before the last update was
  // above ns_tol_ (that update squared it), gathered into a compact batch: the work is
  // proportional to the matrices that need it, and each matrix's result depends only on
  // its own residuals, never on the rest of the batch.
  std::vector<int> act;
  // rlast[b]: matrix b's residual norm before its last update (the update squares it)
  std::vector<double> rlast(batch);
  for (int b = 0; b < batch; ++b) {
    rlast[b] = __longlong_as_double_host(rk[b]);
    const double r = __longlong_as_double_host(r0[b]);
    if (info32[b] != 0 || !(r <= ns_accept_)) continue;     // redone in FP64 below
    if (!(rlast[b] <= ns_tol_)) act.push_back(b);
  }
  for (int step = ns_steps_; step < ns_max_steps_ && !act.empty(); ++step) {
    const int na = (int)act.size();
    ns_extra_ += na;
    NEGF_CUDA_TRY(cudaMemcpyAsync(dNsIdx_, act.data(), sizeof(int) * na, cudaMemcpyHostToDevice, st_));
    NEGF_TRY(gather_strided(M_, na, A, sA, dNsIdx_, dNsX_, MM_, st_));
    NEGF_TRY(gather_strided(M_, na, dWinv_, MM_, dNsIdx_, dNsW_, MM_, st_));
    NEGF_CUDA_TRY(cudaMemsetAsync(dRnorm_, 0, sizeof(unsigned long long) * na, st_));
    NEGF_TRY(slice_a(dNsW_, M_, MM_, M_, M_, na, s_res_, sa_, st_));
    NEGF_TRY(slice_b(dNsX_, M_, MM_, M_, M_, na, s_res_, sb_, st_));
    NEGF_TRY(zgemm_tc(sa_, sb_, one, zero, dT_, M_, MM_, dTcErr_, st_));            // T = W X
    NEGF_TRY(ns_residual(M_, na, dT_, MM_, dRnorm_, st_));                           // R = I - T
    NEGF_CUDA_TRY(cudaMemcpyAsync(rk.data(), dRnorm_, sizeof(unsigned long long) * na, cudaMemcpyDeviceToHost, st_));
    NEGF_TRY(slice_a(dNsX_, M_, MM_, M_, M_, na, s_upd_, sa_, st_));
    NEGF_TRY(slice_b(dT_, M_, MM_, M_, M_, na, s_upd_, sb_, st_));
    NEGF_TRY(zgemm_tc(sa_, sb_, one, one, dNsX_, M_, MM_, dTcErr_, st_, 0, dT_));  // X += X R
    NEGF_TRY(scatter_strided(M_, na, dNsX_, MM_, dNsIdx_, A, sA, st_));
    NEGF_CUDA_TRY(cudaStreamSynchronize(st_));
    std::vector<int> next;
    for (int i = 0; i < na; ++i) {
      rlast[act[i]] = __longlong_as_double_host(rk[i]);
      if (!(rlast[act[i]] <= ns_tol_)) next.push_back(act[i]);
    }
    act.swap(next);
  }
  NEGF_CUDA_TRY(cudaStreamSynchronize(st_));
  // A matrix still in `act` took ns_max_steps_ steps and its residual norm before the last
  // update stayed above ns_tol_: its inverse is not FP64-class, so it joins the FP64 redo
  // with the matrices that failed the first test, and never leaves this call unflagged.
  std::vector<char> unconv(batch, 0);
  for (int b : act) unconv[b] = 1;
  ns_unconverged_ += (long long)act.size();
  double worst = 0.0, worst_last = 0.0;
  std::vector<int> bad;
  for (int b = 0; b < batch; ++b) {
    const double r = __longlong_as_double_host(r0[b]);
    if (info32[b] != 0 || !(r <= ns_accept_) || unconv[b]) {
      bad.push_back(b);
    } else {
      worst = std::max(worst, r);
      worst_last = std::max(worst_last, rlast[b]);
    }
  }
  if (!bad.empty()) {
    // FP64 inverses of the saved matrices, all failures of this call in one batched call
    const int nb = (int)bad.size();
    for (int i = 0; i < nb; ++i)
      NEGF_CUDA_TRY(cudaMemcpyAsync(dT_ + (long long)i * MM_, dWinv_ + (long long)bad[i] * MM_,
                                    sizeof(double2) * MM_, cudaMemcpyDeviceToDevice, st_));
    NEGF_TRY(zinv_f64(dT_, MM_, M_, nb, inv_, st_));
    for (int i = 0; i < nb; ++i) {
      NEGF_CUDA_TRY(cudaMemcpyAsync(A + (long long)bad[i] * sA, dT_ + (long long)i * MM_, sizeof(double2) * MM_,
                                    cudaMemcpyDeviceToDevice, st_));
      NEGF_TRY(merge_info_kernel_launch(1, inv_.info + i, status_dev + bad[i], st_));
    }
    fallbacks_ += nb;
  }
  last_rnorm_max_ = std::max(last_rnorm_max_, worst);
  last_rk_max_ = std::max(last_rk_max_, worst_last);
  return NEGF_OK;
}

// The FP32 inverse of the dW32_ batch in the faster of the two Gauss-Jordan forms.  Both
// give bitwise the same inverse, so the choice never changes a result: the first call of a
// batch size that admits the fused form runs the three-launch form, restores dW32_ from
// the saved FP64 matrices, runs the fused form and keeps the faster (timed with events on
// the engine's stream).
int Engine::invert_f32(int batch) {
  if (!cinv_f32_fused_ok(M_, batch)) return cinv_f32(dW32_, MM_, M_, batch, inv_, st_, 0);
  // NEGF_GJ_FORM = 0 or 1 runs that form instead of the timed choice (to compare or profile
  // the forms; both give bitwise the same inverse)
  if (const char* ev = std::getenv("NEGF_GJ_FORM"))
    if (ev[0] == '0' || ev[0] == '1') return cinv_f32(dW32_, MM_, M_, batch, inv_, st_, ev[0] - '0');
  int bb = 1;
  while (bb < batch) bb <<= 1;
  auto it = gj_form_.find(bb);
  if (it != gj_form_.end()) return cinv_f32(dW32_, MM_, M_, batch, inv_, st_, it->second);
  cudaEvent_t ev[4];
  for (int i = 0; i < 4; ++i)
    if (cudaEventCreate(&ev[i]) != cudaSuccess) {
      for (int j = 0; j < i; ++j) cudaEventDestroy(ev[j]);
      return NEGF_ECUDA;
    }
  int rc = NEGF_OK;
  float t0 = 0.f, t1 = 0.f;
  cudaEventRecord(ev[0], st_);
  rc = cinv_f32(dW32_, MM_, M_, batch, inv_, st_, 0);
  cudaEventRecord(ev[1], st_);
  if (rc == NEGF_OK) rc = to_f32(M_, batch, dWinv_, MM_, dW32_, MM_, st_);   // the same FP32 copy again
  cudaEventRecord(ev[2], st_);
  if (rc == NEGF_OK) rc = cinv_f32(dW32_, MM_, M_, batch, inv_, st_, 1);
  cudaEventRecord(ev[3], st_);
  if (rc == NEGF_OK && cudaEventSynchronize(ev[3]) == cudaSuccess && cudaEventElapsedTime(&t0, ev[0], ev[1]) ==
      cudaSuccess && cudaEventElapsedTime(&t1, ev[2], ev[3]) == cudaSuccess)
    gj_form_[bb] = t1 < t0 ? 1 : 0;
  for (int i = 0; i < 4; ++i) cudaEventDestroy(ev[i]);
  return rc;
}

int Engine::set_refinement(int max_steps, double tol, double accept) {
  if (!mixed_) return NEGF_ESTATE;
  // the two fixed steps stay; at most 16 in all.  A residual norm below 1 is what makes
  // the Newton-Schulz iteration converge, so the acceptance bound must stay below it.
  const int ms = max_steps <= 0 ? 4 : max_steps;
  const double t = tol <= 0.0 ? 1e-5 : tol;
  const double a = accept <= 0.0 ? 0.5 : accept;
  if (ms < ns_steps_ || ms > 16 || !(t < 1.0) || !(a < 1.0)) return NEGF_EINVAL;
  ns_max_steps_ = ms;
  ns_tol_ = t;
  ns_accept_ = a;
  return NEGF_OK;
}

// -------------------------------------------------------------------------------------
// Sancho-Rubio (Source/Contact_Self_Energy.F90:110-223), batched over problems
// -------------------------------------------------------------------------------------
int Engine::solve_sr(const std::vector<SrJob>& jobs, std::vector<int>& status, std::vector<int>& iters) {
  cudaEvent_t ph;
  timed_begin(st_, TK_PH_SR, 0.0, &ph);
  const int rc = p_.contact_type == NEGF_CONTACT_LEADS ? solve_sr_impl(jobs, status, iters)
                                                       : solve_contact_model(jobs, status, iters);
  timed_end(st_, TK_PH_SR, ph);
  return rc;
}

int Engine::solve_sr_impl(const std::vector<SrJob>& jobs, std::vector<int>& status, std::vector<int>& iters) {
  const int S = (int)jobs.size();
  if (S == 0) return NEGF_OK;
  if (S > S_) return NEGF_EINVAL;
  const long long N = p_.npx;
  const double2 one = make_double2(1, 0), zero = make_double2(0, 0), mone = make_double2(-1, 0);
  std::vector<double> e(S);
  std::vector<const double2*> hend(S);
  for (int s = 0; s < S; ++s) {
    e[s] = jobs[s].energy;
    const int slot = jobs[s].slot;
    if (slot < 0 || !slot_set_[slot]) return NEGF_ENOHAM;
    hend[s] = dH_ + ((long long)slot * N + (jobs[s].use_last ? N - 1 : 0)) * MM_;
  }
  NEGF_CUDA_TRY(cudaMemcpyAsync(dSrE_, e.data(), sizeof(double) * S, cudaMemcpyHostToDevice, st_));
  NEGF_CUDA_TRY(cudaMemcpyAsync(dSrHend_, hend.data(), sizeof(void*) * S, cudaMemcpyHostToDevice, st_));
  NEGF_CUDA_TRY(cudaMemsetAsync(dSrStatus_, 0, sizeof(int) * S, st_));
  int role[kSrBlocks];
  for (int r = 0; r < kSrBlocks; ++r) role[r] = r;
  auto buf = [&](int r) { return dSr_ + (long long)role[r] * S_ * MM_; };
  const long long sM = MM_;
  auto inv_merge = [&](double2* A) -> int { return invert(A, sM, S, dSrStatus_); };
  cur_slices_ = s_sr_;
  // Each lead's own products run over the contiguous range of problems that want that
  // lead (batch_solve orders problems left-only, joint, right-only); a problem inside a
  // range that does not want the lead only computes values nobody reads.
  int lo[2] = {S, S}, hi[2] = {0, 0};
  for (int q = 0; q < S; ++q) {
    if (jobs[q].want_l) { lo[0] = std::min(lo[0], q); hi[0] = q + 1; }
    if (jobs[q].want_r) { lo[1] = std::min(lo[1], q); hi[1] = q + 1; }
  }
  auto at = [&](int r, int lead) { return buf(r) + (long long)lo[lead] * sM; };
  auto nlead = [&](int lead) { return hi[lead] > lo[lead] ? hi[lead] - lo[lead] : 0; };

  // alpha = (E + i eta) I - H_end (:71-74 / :83-86)
  NEGF_TRY(form_alpha(M_, S, dSrE_, dSrHend_, p_.eta, 0.0, buf(SR_ALPHA), sM, st_));
  // g0 = inv(alpha + i eta I) (:141)
  NEGF_TRY(form_alpha(M_, S, dSrE_, dSrHend_, p_.eta, p_.eta, buf(SR_TMP), sM, st_));
  NEGF_TRY(inv_merge(buf(SR_TMP)));
  // left lead beta = -H^H:  t = -g0 beta^H = g0 H,  t~ = -g0 beta = g0 H^H (:147-149)
  NEGF_TRY(hop_mul(0, OP_N, buf(SR_TMP), sM, buf(SR_T), sM, S));
  NEGF_TRY(hop_mul(0, OP_C, buf(SR_TMP), sM, buf(SR_TT), sM, S));
  // T_L = t; the right lead (beta = -H) starts from t_R = t~, so T_R = t~ (:151)
  NEGF_TRY(copy_blocks(M_, S, buf(SR_T), sM, buf(SR_TL), sM, st_));
  NEGF_TRY(copy_blocks(M_, S, buf(SR_TT), sM, buf(SR_TR), sM, st_));
  NEGF_TRY(set_identity(M_, S, buf(SR_TOLDL), sM, st_));
  NEGF_TRY(set_identity(M_, S, buf(SR_TOLDR), sM, st_));

  std::vector<int> act(2 * S);
  for (int s = 0; s < S; ++s) { act[s] = jobs[s].want_l; act[S + s] = jobs[s].want_r; }
  iters.assign(2 * S, 0);
  status.assign(S, 0);
  NEGF_CUDA_TRY(cudaMemcpyAsync(dSrActive_, act.data(), sizeof(int) * 2 * S, cudaMemcpyHostToDevice, st_));
  int it = 0;
  auto any_active = [&]() { return std::any_of(act.begin(), act.end(), [](int a) { return a != 0; }); };
  while (any_active() && it < p_.sr_max_iter) {
    ++it;
    // Told_L <- Told_L t~ ; Told_R <- Told_R t  (:157-158, with t <-> t~ for the right lead),
    // each over its lead's problems; W1 then takes the old Told's role, and the problems
    // outside the range keep their (unread) values in the swapped buffers
    if (nlead(0))
      NEGF_TRY(gemm(nlead(0), OP_N, at(SR_TOLDL, 0), sM, OP_N, at(SR_TT, 0), sM, at(SR_W1, 0), sM, one, zero));
    std::swap(role[SR_TOLDL], role[SR_W1]);
    if (nlead(1))
      NEGF_TRY(gemm(nlead(1), OP_N, at(SR_TOLDR, 1), sM, OP_N, at(SR_T, 1), sM, at(SR_W1, 1), sM, one, zero));
    std::swap(role[SR_TOLDR], role[SR_W1]);
    // tmp = inv(I - t t~ - t~ t) (:160-163)
    NEGF_TRY(set_identity(M_, S, buf(SR_TMP), sM, st_));
    NEGF_TRY(gemm(S, OP_N, buf(SR_T), sM, OP_N, buf(SR_TT), sM, buf(SR_TMP), sM, mone, one));
    NEGF_TRY(gemm(S, OP_N, buf(SR_TT), sM, OP_N, buf(SR_T), sM, buf(SR_TMP), sM, mone, one));
    NEGF_TRY(inv_merge(buf(SR_TMP)));
    // t <- tmp t t ; t~ <- tmp t~ t~ (:170-176)
    NEGF_TRY(gemm(S, OP_N, buf(SR_TMP), sM, OP_N, buf(SR_T), sM, buf(SR_W1), sM, one, zero));
    NEGF_TRY(gemm(S, OP_N, buf(SR_W1), sM, OP_N, buf(SR_T), sM, buf(SR_TN), sM, one, zero));
    NEGF_TRY(gemm(S, OP_N, buf(SR_TMP), sM, OP_N, buf(SR_TT), sM, buf(SR_W1), sM, one, zero));
    NEGF_TRY(gemm(S, OP_N, buf(SR_W1), sM, OP_N, buf(SR_TT), sM, buf(SR_TTN), sM, one, zero));
    // change = Told t ; T += change (:178-180), each over its lead's problems
    if (nlead(0)) {
      NEGF_TRY(gemm(nlead(0), OP_N, at(SR_TOLDL, 0), sM, OP_N, at(SR_TN, 0), sM, at(SR_CHG, 0), sM, one, zero));
      NEGF_TRY(sr_accumulate(M_, nlead(0), dSrActive_ + lo[0], at(SR_CHG, 0), sM, at(SR_TL, 0), sM,
                             dSrCmax_ + lo[0], st_));
    }
    if (nlead(1)) {
      NEGF_TRY(gemm(nlead(1), OP_N, at(SR_TOLDR, 1), sM, OP_N, at(SR_TTN, 1), sM, at(SR_CHG, 1), sM, one, zero));
      NEGF_TRY(sr_accumulate(M_, nlead(1), dSrActive_ + S + lo[1], at(SR_CHG, 1), sM, at(SR_TR, 1), sM,
                             dSrCmax_ + S + lo[1], st_));
    }
    std::swap(role[SR_T], role[SR_TN]);
    std::swap(role[SR_TT], role[SR_TTN]);
    NEGF_CUDA_TRY(cudaMemcpyAsync(hPin_, dSrCmax_, sizeof(double) * 2 * S, cudaMemcpyDeviceToHost, st_));
    NEGF_CUDA_TRY(cudaStreamSynchronize(st_));
    bool changed = false;
    for (int q = 0; q < 2 * S; ++q) {
      if (!act[q]) continue;
      const double c = hPin_[q];
      if (std::isnan(c)) {               // :182-191
        status[q % S] = NEGF_ENAN;
        act[q] = 0; iters[q] = it; changed = true;
      } else if (!(c > p_.sr_tol)) {     // loop test of :154
        act[q] = 0; iters[q] = it; changed = true;
      }
    }
    if (changed)
      NEGF_CUDA_TRY(cudaMemcpyAsync(dSrActive_, act.data(), sizeof(int) * 2 * S, cudaMemcpyHostToDevice, st_));
  }
  for (int q = 0; q < 2 * S; ++q)
    if (act[q]) { iters[q] = it; if (status[q % S] == 0) status[q % S] = NEGF_ESR_NOCONV; }

  // g = inv(alpha + beta T), Sigma = beta g beta^H (:195-209) for each lead, over the
  // problems that want it
  for (int lead = 0; lead < 2; ++lead) {
    const int n = nlead(lead), a = lo[lead];
    if (n == 0) continue;
    const long long off = (long long)a * sM;
    double2* T = buf(lead == 0 ? SR_TL : SR_TR) + off;
    double2* W = buf(SR_TMP) + off;
    if (hop_bd_) {
      NEGF_TRY(sr_form_final(hop(), M_, n, lead, buf(SR_ALPHA) + off, sM, T, sM, W, sM, st_));
    } else {
      NEGF_TRY(copy_blocks(M_, n, buf(SR_ALPHA) + off, sM, W, sM, st_));
      NEGF_TRY(gemm(n, lead == 0 ? OP_C : OP_N, dHop_, 0, OP_N, T, sM, W, sM, mone, one));
    }
    NEGF_TRY(invert(W, sM, n, dSrStatus_ + a));
    double2* sig = (lead == 0 ? dSrSigL_ : dSrSigR_) + off;
    double2* gam = (lead == 0 ? dSrGamL_ : dSrGamR_) + off;
    if (hop_bd_) {
      NEGF_TRY(sr_sigma(hop(), M_, n, lead, W, sM, sig, sM, gam, sM, dSrDos_ + lead * S + a, st_));
    } else {
      // lead 0: H^H g H ; lead 1: H g H^H
      NEGF_TRY(gemm(n, lead == 0 ? OP_C : OP_N, dHop_, 0, OP_N, W, sM, buf(SR_W1) + off, sM, one, zero));
      NEGF_TRY(gemm(n, OP_N, buf(SR_W1) + off, sM, lead == 0 ? OP_N : OP_C, dHop_, 0, sig, sM, one, zero));
      NEGF_TRY(sr_sigma(HopBD{}, M_, n, -1, nullptr, 0, sig, sM, gam, sM, dSrDos_ + lead * S + a, st_));
    }
  }
  std::vector<int> st(S);
  NEGF_CUDA_TRY(cudaMemcpyAsync(st.data(), dSrStatus_, sizeof(int) * S, cudaMemcpyDeviceToHost, st_));
  NEGF_CUDA_TRY(cudaStreamSynchronize(st_));
  for (int s = 0; s < S; ++s)
    if (status[s] == 0 && st[s] != 0) status[s] = st[s];
  return NEGF_OK;
}

// Contacts with a closed-form self-energy (Source/Contact_Self_Energy.F90:19-67): the
// per-energy scalars are formed here, the blocks on the device; Gamma and the contact DOS
// follow from Sigma as for the decimated leads (:94-101).
int Engine::solve_contact_model(const std::vector<SrJob>& jobs, std::vector<int>& status, std::vector<int>& iters) {
  const int S = (int)jobs.size();
  status.assign(S, 0);
  iters.assign(2 * S, 0);
  if (S == 0) return NEGF_OK;
  if (S > S_) return NEGF_EINVAL;
  const double rate = p_.tunneling_rate == 0.0 ? 1.0 : p_.tunneling_rate;   // :10
  std::vector<double2> coef((size_t)S * 6, make_double2(0.0, 0.0));
  for (int s = 0; s < S; ++s) {
    double2* c = coef.data() + (size_t)s * 6;
    if (p_.contact_type != NEGF_CONTACT_SC) {                 // :19-28, Sigma_R = Sigma_L
      c[0] = c[3] = make_double2(0.0, -rate);
      continue;
    }
    // :29-59: omega = 1/sqrt(DeltaSCL^2 - ce^2) for both contacts (the right one also uses
    // DeltaSCL at :49), ce = E + i eta (:16)
    const std::complex<double> ce(jobs[s].energy, p_.eta);
    const std::complex<double> omega = 1.0 / std::sqrt(p_.delta_sc[0] * p_.delta_sc[0] - ce * ce);
    const std::complex<double> m_alpha = -rate * omega * ce;
    const std::complex<double> ph = std::exp(std::complex<double>(0.0, p_.chi_lr));
    for (int lead = 0; lead < 2; ++lead) {
      const std::complex<double> up = rate * omega * p_.delta_sc[lead];
      const std::complex<double> lo = rate * omega * (-p_.delta_sc[lead]);
      const std::complex<double> u = lead == 0 ? up * ph : up, l = lead == 0 ? lo * std::conj(ph) : lo;
      c[lead * 3 + 0] = make_double2(m_alpha.real(), m_alpha.imag());
      c[lead * 3 + 1] = make_double2(u.real(), u.imag());
      c[lead * 3 + 2] = make_double2(l.real(), l.imag());
    }
  }
  ContactGds g{};
  bool any = false;
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) {
      g.m[r][c] = make_double2(p_.gds[r][c][0], p_.gds[r][c][1]);
      if (p_.gds[r][c][0] != 0.0 || p_.gds[r][c][1] != 0.0) any = true;
    }
  if (!any && nh_ == 4) {   // the four-orbital models' gDS (Source/Read_In_Allocate.F90:199-202)
    g.m[0][1] = make_double2(1, 0); g.m[1][0] = make_double2(-1, 0);
    g.m[2][3] = make_double2(1, 0); g.m[3][2] = make_double2(-1, 0);
  } else if (!any && nh_ == 2) {   // :214-215
    g.m[0][1] = make_double2(1, 0); g.m[1][0] = make_double2(-1, 0);
  }
  NEGF_CUDA_TRY(cudaMemcpyAsync(dContactCoef_, coef.data(), sizeof(double2) * coef.size(), cudaMemcpyHostToDevice, st_));
  const int ndiag = p_.contact_type == NEGF_CONTACT_PSMALL ? p_.npy * p_.norb : M_;   // :24-28: NN orbitals
  const long long sM = MM_;
  NEGF_TRY(contact_fill(M_, p_.norb, nh_, p_.contact_type, ndiag, S, dContactCoef_, g, dSrSigL_, dSrSigR_, sM, st_));
  for (int lead = 0; lead < 2; ++lead)
    NEGF_TRY(sr_sigma(HopBD{}, M_, S, -1, nullptr, 0, lead == 0 ? dSrSigL_ : dSrSigR_, sM,
                      lead == 0 ? dSrGamL_ : dSrGamR_, sM, dSrDos_ + lead * S, st_));
  return NEGF_OK;
}

// -------------------------------------------------------------------------------------
// RGF sweep with the Gn site blocks and the end-block traces, batched over items
// -------------------------------------------------------------------------------------
int Engine::solve_rgf(const std::vector<Item>& items, bool keep_columns) {
  cudaEvent_t ph;
  timed_begin(st_, TK_PH_RGF, 0.0, &ph);
  const int rc = solve_rgf_impl(items, keep_columns);
  timed_end(st_, TK_PH_RGF, ph);
  return rc;
}

int Engine::solve_rgf_impl(const std::vector<Item>& items, bool keep_columns) {
  const int B = (int)items.size();
  if (B == 0) return NEGF_OK;
  if (B > B_) return NEGF_EINVAL;
  for (const Item& it : items)
    if (it.slot < 0 || it.slot >= p_.n_hamiltonians || !slot_set_[it.slot]) return NEGF_ENOHAM;
  const int N = p_.npx;
  const long long sM = MM_, sG = (long long)N * MM_;
  const long long sP = (long long)N * M_ * p_.norb;
  const double2 one = make_double2(1, 0), zero = make_double2(0, 0);
  NEGF_CUDA_TRY(cudaMemcpyAsync(dItems_, items.data(), sizeof(Item) * B, cudaMemcpyHostToDevice, st_));
  NEGF_CUDA_TRY(cudaMemsetAsync(dStatus_, 0, sizeof(int) * B, st_));
  const int istride = (int)(sizeof(Item) / sizeof(int));
  const int* idx_l = reinterpret_cast<const int*>(reinterpret_cast<const char*>(dItems_) + offsetof(Item, sr_l));
  const int* idx_r = reinterpret_cast<const int*>(reinterpret_cast<const char*>(dItems_) + offsetof(Item, sr_r));
  NEGF_TRY(gather_blocks(M_, B, dSrSigL_, idx_l, istride, dSigL_, sM, st_));
  NEGF_TRY(gather_blocks(M_, B, dSrSigR_, idx_r, istride, dSigR_, sM, st_));
  NEGF_TRY(gather_blocks(M_, B, dSrGamL_, idx_l, istride, dGamL_, sM, st_));
  NEGF_TRY(gather_blocks(M_, B, dSrGamR_, idx_r, istride, dGamR_, sM, st_));
  if (mixed_) {   // Gamma is the right factor of every G(:,c) Gamma_c product of the sweep
    NEGF_TRY(slice_b(dGamL_, M_, sM, M_, M_, B, s_rgf_, sgl_, st_));
    NEGF_TRY(slice_b(dGamR_, M_, sM, M_, M_, B, s_rgf_, sgr_, st_));
  }

  auto form = [&](int x, int side, const double2* gprev) -> int {
    FormW fw{};
    fw.n = M_; fw.batch = B; fw.npx = N; fw.x = x; fw.eta = p_.eta;
    fw.items = dItems_; fw.Hall = dH_;
    fw.sigL = dSigL_; fw.sigR = dSigR_; fw.sSig = sM;
    fw.side = side; fw.sG = sG; fw.sZ = sM;
    fw.W = dG_ + (long long)x * MM_; fw.sW = sG;
    if (gprev) {
      if (hop_bd_) {
        fw.gprev = gprev;
        fw.hop = hop();
        if (hop_uniform_) {   // side 0: L = H^H, R = H; side 1: L = H, R = H^H
          fw.use_rows = 1;
          fw.lrow = hop_rows_[1][side == 0 ? 1 : 0];
          fw.rrow = hop_rows_[0][side == 0 ? 0 : 1];
        }
      } else {
        // side 0: H^H g H ; side 1: H g H^H  (dense HopX)
        NEGF_TRY(hop_mul(1, side == 0 ? OP_C : OP_N, gprev, sG, dZ_, sM, B));
        NEGF_TRY(hop_mul(0, side == 0 ? OP_N : OP_C, dZ_, sM, dQ_, sM, B));
        fw.zsub = dQ_;
      }
    }
    NEGF_TRY(form_w(fw, st_));
    return invert(dG_ + (long long)x * MM_, sG, B, dStatus_);
  };
  cur_slices_ = s_rgf_;

  // right-connected sweep gR_x = inv(A_x - H gR_{x+1} H^H), x = N..1 (Recursive_Greens.F90:67-86)
  for (int x = N - 1; x >= 0; --x) NEGF_TRY(form(x, 1, x < N - 1 ? dG_ + (long long)(x + 1) * MM_ : nullptr));

  // forward: column 1 from gR, then the left-connected gL_x into the same slot.  With
  // currents, Y alternates between two buffers so that Y(x-1) = G(x-1,1) Gamma_L is still
  // there when G(x,1) is formed: P1(x-1, x) = Y(x-1) G(x,1)^H on the site blocks.
  const long long sl = (long long)M_ * p_.norb;   // one slice of site blocks
  for (int x = 0; x < N; ++x) {
    double2* Gx = dG_ + (long long)x * MM_;
    double2* Y = (x & 1) ? dYalt_ : dY_;
    double2* Yprev = (x & 1) ? dY_ : dYalt_;
    if (x == 0) {
      NEGF_TRY(copy_blocks(M_, B, Gx, sG, dC1_, sM, st_));                     // G(1,1) = gR_1
      if (sc_()) NEGF_TRY(site_diag(M_, p_.norb, B, dC1_, sM, dG11_, (long long)M_ * p_.norb, st_));
    } else {
      NEGF_TRY(hop_mul(1, OP_C, dC1_, sM, dZ_, sM, B));                          // H^H G(x-1,1)
      NEGF_TRY(gemm(B, OP_N, Gx, sG, OP_N, dZ_, sM, dC1_, sM, one, zero));       // gR_x H^H G(x-1,1)
      if (currents_)
        NEGF_TRY(site_blocks(M_, p_.norb, B, Yprev, sM, dC1_, sM, dPx1_ + (x - 1) * sl, sP, st_));
    }
    if (keep_columns && dCol1_) NEGF_TRY(copy_blocks(M_, 1, dC1_, sM, dCol1_ + (long long)x * MM_, sM, st_));
    NEGF_TRY(gemm_gamma(B, dC1_, sM, dGamL_, sgl_, Y, sM));                        // G(x,1) Gamma_L
    if (currents_)
      NEGF_TRY(site_pairs(M_, p_.norb, p_.npy, p_.npz, B, Y, sM, dC1_, sM, dP1_ + x * sl, dPy1_ + x * sl,
                          dPz1_ + x * sl, sP, st_));
    else
      NEGF_TRY(site_blocks(M_, p_.norb, B, Y, sM, dC1_, sM, dP1_ + x * sl, sP, st_));
    if (x == 0) {
      NEGF_TRY(gemm(B, OP_N, dGamL_, sM, OP_N, Y, sM, dQ_, sM, one, zero));
      NEGF_TRY(trace_dot(M_, B, dQ_, sM, dC1_, sM, dTr_ + 0, 4, st_));
    }
    if (x == N - 1) {
      NEGF_TRY(gemm(B, OP_N, dGamR_, sM, OP_N, Y, sM, dQ_, sM, one, zero));
      NEGF_TRY(trace_dot(M_, B, dQ_, sM, dC1_, sM, dTr_ + 2, 4, st_));
    }
    // gL_x = inv(A_x - H^H gL_{x-1} H) (Recursive_Greens.F90:16-34)
    NEGF_TRY(form(x, 0, x > 0 ? dG_ + (long long)(x - 1) * MM_ : nullptr));
  }

  // backward: column N, G(x,N) = gL_x H G(x+1,N) (Recursive_Greens.F90:53-63).  With
  // currents, G(:,N) alternates between two buffers so that G(x+1,N) is still there for
  // P2(x, x+1) = Y(x) G(x+1,N)^H on the site blocks.
  for (int x = N - 1; x >= 0; --x) {
    double2* Gx = dG_ + (long long)x * MM_;
    double2* CN = ((N - 1 - x) & 1) ? dCNalt_ : dCN_;
    double2* CNprev = ((N - 1 - x) & 1) ? dCN_ : dCNalt_;
    if (x == N - 1) {
      NEGF_TRY(copy_blocks(M_, B, Gx, sG, CN, sM, st_));
    } else {
      NEGF_TRY(hop_mul(1, OP_N, CNprev, sM, dZ_, sM, B));
      NEGF_TRY(gemm(B, OP_N, Gx, sG, OP_N, dZ_, sM, CN, sM, one, zero));
    }
    if (keep_columns && dColN_) NEGF_TRY(copy_blocks(M_, 1, CN, sM, dColN_ + (long long)x * MM_, sM, st_));
    NEGF_TRY(gemm_gamma(B, CN, sM, dGamR_, sgr_, dY_, sM));                         // G(x,N) Gamma_R
    if (currents_) {
      NEGF_TRY(site_pairs(M_, p_.norb, p_.npy, p_.npz, B, dY_, sM, CN, sM, dP2_ + x * sl, dPy2_ + x * sl,
                          dPz2_ + x * sl, sP, st_));
      if (x < N - 1) NEGF_TRY(site_blocks(M_, p_.norb, B, dY_, sM, CNprev, sM, dPx2_ + x * sl, sP, st_));
    } else {
      NEGF_TRY(site_blocks(M_, p_.norb, B, dY_, sM, CN, sM, dP2_ + x * sl, sP, st_));
    }
    if (x == 0) {   // T12 = Re Tr[Gamma_L G(1,N) Gamma_R G(1,N)^H] (Calculate_Observables.F90:85-100)
      NEGF_TRY(gemm(B, OP_N, dGamL_, sM, OP_N, dY_, sM, dQ_, sM, one, zero));
      NEGF_TRY(trace_dot(M_, B, dQ_, sM, CN, sM, dTr_ + 1, 4, st_));
    }
    if (x == N - 1) {
      NEGF_TRY(gemm(B, OP_N, dGamR_, sM, OP_N, dY_, sM, dQ_, sM, one, zero));
      NEGF_TRY(trace_dot(M_, B, dQ_, sM, CN, sM, dTr_ + 3, 4, st_));
    }
  }
  return NEGF_OK;
}

int Engine::densities(const std::vector<Item>& items, std::vector<double>& edens, std::vector<double>& hdens) {
  cudaEvent_t ph;
  timed_begin(st_, TK_PH_DENS, 0.0, &ph);
  const int rc = densities_impl(items, edens, hdens);
  timed_end(st_, TK_PH_DENS, ph);
  return rc;
}

int Engine::densities_impl(const std::vector<Item>& items, std::vector<double>& edens, std::vector<double>& hdens) {
  const int B = (int)items.size();
  NEGF_CUDA_TRY(cudaMemcpyAsync(dItems_, items.data(), sizeof(Item) * B, cudaMemcpyHostToDevice, st_));
  DensityArgs a{};
  a.n = M_; a.norb = p_.norb; a.npx = p_.npx; a.npy = p_.npy; a.npz = p_.npz; a.batch = B;
  a.calc_spin = p_.calc_spin; a.nf = nf_; a.items = dItems_; a.nh = nh_;
  a.P1 = dP1_; a.P2 = dP2_; a.sP = (long long)p_.npx * M_ * p_.norb;
  a.spin_ops = dSpin_; a.site_out = dSite_; a.sums = dSums_;
  NEGF_TRY(density_spin(a, st_));
  if (currents_) {
    CurrentArgs c{};
    c.n = M_; c.norb = p_.norb; c.npx = p_.npx; c.npy = p_.npy; c.npz = p_.npz; c.batch = B; c.nf = nf_;
    c.nh = nh_;
    c.items = dItems_; c.Hall = dH_; c.Hop = dHop_;
    c.Px1 = dPx1_; c.Py1 = dPy1_; c.Pz1 = dPz1_; c.Px2 = dPx2_; c.Py2 = dPy2_; c.Pz2 = dPz2_;
    c.sP = a.sP;
    c.q2_over_hbar = kQ * kQ / kHbar;
    c.site_out = dSite_;
    c.P1 = dP1_; c.P2 = dP2_;
    NEGF_TRY(bond_currents(c, st_));
  }
  if (sc_())   // supercurrent transmission from slice 1 (Calculate_Observables.F90:60-81)
    NEGF_TRY(josephson(M_, p_.norb, B, dItems_, dP1_, dP2_, a.sP, dG11_, (long long)M_ * p_.norb, dSigL_, dGamL_, MM_,
                       dTrJ_, st_));
  const size_t np = (size_t)B * sums_blocks_ * 2;
  NEGF_CUDA_TRY(cudaMemcpyAsync(hPin_, dSums_, sizeof(double) * np, cudaMemcpyDeviceToHost, st_));
  NEGF_CUDA_TRY(cudaStreamSynchronize(st_));
  edens.assign(B, 0.0);
  hdens.assign(B, 0.0);
  const double inv2pi = 1.0 / (2.0 * 3.14159265358979323846);
  for (int b = 0; b < B; ++b) {
    double sn = 0.0, sp = 0.0;
    for (int k = 0; k < sums_blocks_; ++k) {
      sn += hPin_[((size_t)b * sums_blocks_ + k) * 2 + 0];
      sp += hPin_[((size_t)b * sums_blocks_ + k) * 2 + 1];
    }
    edens[b] = sn * inv2pi;
    hdens[b] = sp * inv2pi;
  }
  return NEGF_OK;
}

int Engine::ensure_resolved() {
  if (!currents_) return NEGF_ESTATE;
  const long long total = nsite_total();
  if (!dEr_ || !dOrAcc_) {
    if (!dEr_) NEGF_TRY(dalloc(&dEr_, (size_t)B_ * 4 * total, bytes_, false, pool_, own_st_));
    if (!dOrAcc_)
      NEGF_TRY(dalloc(&dOrAcc_, (size_t)p_.n_hamiltonians * n_or_fields() * total, bytes_, false, pool_, own_st_));
    NEGF_CUDA_TRY(cudaStreamSynchronize(own_st_));
  }
  return NEGF_OK;
}

int Engine::resolved(int batch, bool er, bool orb, int nslots) {
  NEGF_TRY(ensure_resolved());
  CurrentArgs c{};
  c.n = M_; c.norb = p_.norb; c.npx = p_.npx; c.npy = p_.npy; c.npz = p_.npz; c.batch = batch; c.nf = nf_;
  c.nh = nh_;
  c.items = dItems_; c.Hall = dH_; c.Hop = dHop_;
  c.Px1 = dPx1_; c.Py1 = dPy1_; c.Pz1 = dPz1_; c.Px2 = dPx2_; c.Py2 = dPy2_; c.Pz2 = dPz2_;
  c.sP = (long long)p_.npx * M_ * p_.norb;
  c.q2_over_hbar = kQ * kQ / kHbar;
  c.site_out = dSite_;
  c.P1 = dP1_; c.P2 = dP2_;
  if (er) {
    c.er_out = dEr_;
    NEGF_TRY(bond_currents(c, st_));   // rewrites the J fields with the same values
    c.er_out = nullptr;
  }
  if (orb) {
    c.or_acc = dOrAcc_;
    NEGF_TRY(orbital_resolved(c, nslots, st_));
  }
  return NEGF_OK;
}

// -------------------------------------------------------------------------------------
// Batched solve
// -------------------------------------------------------------------------------------
int Engine::batch_solve(const negf_request* req, int n, negf_result* res, double* const* outs,
                        double* site_items, const ResolvedOut* ro) {
  if (n < 0 || (n > 0 && (!req || !res))) return NEGF_EINVAL;
  NEGF_CUDA_TRY(cudaSetDevice(p_.device));
  const long long total = nsite_total();
  const int nslots = p_.n_hamiltonians;
  for (int i = 0; i < n; ++i) {
    const int s = req[i].slot;
    if (s < 0 || s >= nslots) return NEGF_EINVAL;
    if (!slot_set_[s]) return NEGF_ENOHAM;
  }
  const bool want_er = ro && ro->any_er(), want_or = ro && ro->any_or();
  if (want_er || want_or) {
    NEGF_TRY(ensure_resolved());
    if (want_or)
      NEGF_CUDA_TRY(cudaMemsetAsync(dOrAcc_, 0, sizeof(double) * nslots * n_or_fields() * total, st_));
  }
  std::vector<double> er_host(want_er ? (size_t)B_ * 4 * total : 0);
  NEGF_CUDA_TRY(cudaMemsetAsync(dAcc_, 0, sizeof(double) * nslots * nf_ * total, st_));
  for (int c0 = 0; c0 < n; c0 += B_) {
    const int nb = std::min(B_, n - c0);
    // Sancho-Rubio problems: one per (energy, lead class) when H_1 == H_N, otherwise a
    // left-only and a right-only one.  They are ordered left-only, joint, right-only, so
    // the problems that need each lead's products form one contiguous range.
    std::vector<SrJob> jl_only, joint, jr_only;
    std::map<std::pair<double, int>, std::pair<int, int>> key2job;   // (list, index) codes
    std::vector<Item> items(nb);
    std::vector<std::pair<int, int>> item_jobs(nb);
    for (int i = 0; i < nb; ++i) {
      const negf_request& r = req[c0 + i];
      // model contacts do not depend on the Hamiltonian: one problem per energy
      const bool model = p_.contact_type != NEGF_CONTACT_LEADS;
      const int rep = model ? 0 : slot_rep_[r.slot];
      auto key = std::make_pair(r.energy, rep);
      auto itk = key2job.find(key);
      std::pair<int, int> code;   // list * 2^20 + index, for the left and the right lead
      if (itk == key2job.end()) {
        if (model || slot_joint_[rep]) {
          joint.push_back(SrJob{r.energy, rep, 0, 1, 1});
          const int c = (1 << 20) + (int)joint.size() - 1;
          code = {c, c};
        } else {
          jl_only.push_back(SrJob{r.energy, rep, 0, 1, 0});
          jr_only.push_back(SrJob{r.energy, rep, 1, 0, 1});
          code = {(int)jl_only.size() - 1, (2 << 20) + (int)jr_only.size() - 1};
        }
        key2job[key] = code;
      } else {
        code = itk->second;
      }
      item_jobs[i] = code;
    }
    std::vector<SrJob> jobs(jl_only);
    jobs.insert(jobs.end(), joint.begin(), joint.end());
    jobs.insert(jobs.end(), jr_only.begin(), jr_only.end());
    const int base[3] = {0, (int)jl_only.size(), (int)(jl_only.size() + joint.size())};
    for (int i = 0; i < nb; ++i) {
      const negf_request& r = req[c0 + i];
      Item& it = items[i];
      it.energy = r.energy; it.f1 = r.f1; it.f2 = r.f2; it.dE = r.dE; it.slot = r.slot;
      it.sr_l = base[item_jobs[i].first >> 20] + (item_jobs[i].first & ((1 << 20) - 1));
      it.sr_r = base[item_jobs[i].second >> 20] + (item_jobs[i].second & ((1 << 20) - 1));
      it.pad = 0;
    }
    std::vector<int> sr_status, sr_iters;
    NEGF_TRY(solve_sr(jobs, sr_status, sr_iters));
    const int S = (int)jobs.size();
    std::vector<double> dos(2 * S);
    NEGF_CUDA_TRY(cudaMemcpyAsync(dos.data(), dSrDos_, sizeof(double) * S, cudaMemcpyDeviceToHost, st_));
    NEGF_CUDA_TRY(cudaMemcpyAsync(dos.data() + S, dSrDos_ + S, sizeof(double) * S, cudaMemcpyDeviceToHost, st_));
    NEGF_TRY(solve_rgf(items, false));
    std::vector<double> ed, hd;
    NEGF_TRY(densities(items, ed, hd));
    NEGF_TRY(reduce_sites(nb, (int)total, nf_, nslots, dItems_, dSite_, dAcc_, st_));
    if (want_er || want_or) NEGF_TRY(resolved(nb, want_er, want_or, nslots));
    if (want_er)
      NEGF_CUDA_TRY(cudaMemcpyAsync(er_host.data(), dEr_, sizeof(double) * 4 * total * nb, cudaMemcpyDeviceToHost,
                                    st_));
    if (site_items)
      NEGF_CUDA_TRY(cudaMemcpyAsync(site_items + (size_t)c0 * nf_ * total, dSite_,
                                    sizeof(double) * nf_ * total * nb, cudaMemcpyDeviceToHost, st_));
    std::vector<double> tr(4 * (size_t)nb), trj(sc_() ? nb : 0);
    std::vector<int> rst(nb);
    NEGF_CUDA_TRY(cudaMemcpyAsync(tr.data(), dTr_, sizeof(double) * 4 * nb, cudaMemcpyDeviceToHost, st_));
    if (sc_()) NEGF_CUDA_TRY(cudaMemcpyAsync(trj.data(), dTrJ_, sizeof(double) * nb, cudaMemcpyDeviceToHost, st_));
    NEGF_CUDA_TRY(cudaMemcpyAsync(rst.data(), dStatus_, sizeof(int) * nb, cudaMemcpyDeviceToHost, st_));
    NEGF_CUDA_TRY(cudaStreamSynchronize(st_));
    for (int i = 0; i < nb; ++i) {
      negf_result& o = res[c0 + i];
      const Item& it = items[i];
      o.T12 = sc_() ? trj[i] : tr[4 * i + 1];
      o.modes[0] = tr[4 * i + 0] + tr[4 * i + 1];
      o.modes[1] = tr[4 * i + 2] + tr[4 * i + 3];
      o.EDensity = ed[i];
      o.HDensity = hd[i];
      o.dosc[0] = dos[it.sr_l];
      o.dosc[1] = dos[S + it.sr_r];
      int stv = sr_status[it.sr_l] ? sr_status[it.sr_l] : sr_status[it.sr_r];
      if (stv == 0) stv = rst[i];
      o.status = stv;
      o.sr_iters = std::max(sr_iters[it.sr_l], sr_iters[S + it.sr_r]);
    }
    if (want_er)   // request c0 + i -> column c0 + i of each energy-resolved array
      for (int f = 0; f < 4; ++f) {
        if (!ro->er[f]) continue;
        for (int i = 0; i < nb; ++i) {
          double* dst = ro->er[f] + (size_t)(c0 + i) * total;
          const double* src = er_host.data() + ((size_t)i * 4 + f) * total;
          for (long long k = 0; k < total; ++k) dst[k] += src[k];
        }
      }
  }
  if (want_or) {
    const int nq = n_or_fields(), no2 = p_.norb * p_.norb;
    std::vector<double> orh((size_t)nslots * nq * total);
    NEGF_CUDA_TRY(cudaMemcpyAsync(orh.data(), dOrAcc_, sizeof(double) * orh.size(), cudaMemcpyDeviceToHost, st_));
    NEGF_CUDA_TRY(cudaStreamSynchronize(st_));
    for (int s = 0; s < nslots; ++s)
      for (int q = 0; q < nq; ++q) {
        double* dst;
        if (q < 3 * no2) {
          if (!ro->orj[q / no2]) continue;
          dst = ro->orj[q / no2] + ((size_t)s * no2 + q % no2) * total;
        } else {
          if (!ro->orrho) continue;
          dst = ro->orrho + ((size_t)s * p_.norb + (q - 3 * no2)) * total;
        }
        const double* src = orh.data() + ((size_t)s * nq + q) * total;
        for (long long k = 0; k < total; ++k) dst[k] += src[k];
      }
  }
  // add the slot-resolved site sums into the caller's arrays
  const size_t acc_n = (size_t)nslots * nf_ * total;
  NEGF_CUDA_TRY(cudaMemcpyAsync(hPin_, dAcc_, sizeof(double) * acc_n, cudaMemcpyDeviceToHost, st_));
  NEGF_CUDA_TRY(cudaStreamSynchronize(st_));
  for (int f = 0; f < nf_; ++f) {
    if (!outs || !outs[f]) continue;
    if (f >= 2 && f < 5 && !p_.calc_spin) continue;
    for (int s = 0; s < nslots; ++s)
      for (long long i = 0; i < total; ++i)
        outs[f][(size_t)s * total + i] += hPin_[((size_t)s * nf_ + f) * total + i];
  }
  return NEGF_OK;   // per-request failures are reported in res[i].status
}

}  // namespace negf
