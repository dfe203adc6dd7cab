// extern "C" entry points of libnegf_gb300.so (declared in include/negf.h).
#include <cstring>
#include <new>
#include <string>

#include "engine.h"

namespace negf {

namespace {
thread_local std::string g_last_cuda_error;
}  // namespace

void record_cuda_error(cudaError_t e, const char* what, const char* file, int line) {
  g_last_cuda_error = std::string(cudaGetErrorString(e)) + " in " + what + " (" + file + ":" + std::to_string(line) + ")";
}
const char* last_cuda_error_text() { return g_last_cuda_error.c_str(); }

Instrument& instrument() {
  static Instrument g;
  return g;
}

namespace {
void resolve_locked() {
  Instrument& I = instrument();
  for (const Instrument::Rec& r : I.pending) {
    float ms = 0.f;
    if (cudaEventSynchronize(r.b) == cudaSuccess && cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess)
      I.kind_ms[r.kind] += ms;
    I.pool.push_back(r.a);
    I.pool.push_back(r.b);
  }
  I.pending.clear();
}

cudaEvent_t pooled_event() {
  Instrument& I = instrument();
  if (!I.pool.empty()) {
    cudaEvent_t e = I.pool.back();
    I.pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
  return e;
}
}  // namespace

void add_tc_complex_flops(double f) {
  Instrument& I = instrument();
  std::lock_guard<std::mutex> g(I.mu);
  I.tc_complex_flops += f;
}

void timed_begin(cudaStream_t st, int kind, double flops, cudaEvent_t* a) {
  Instrument& I = instrument();
  I.kind_launches[kind].fetch_add(1, std::memory_order_relaxed);
  *a = nullptr;
  std::lock_guard<std::mutex> g(I.mu);
  I.kind_flops[kind] += flops;
  if (!I.timing.load()) return;
  *a = pooled_event();
  if (*a) cudaEventRecord(*a, st);
}

void timed_end(cudaStream_t st, int kind, cudaEvent_t a) {
  Instrument& I = instrument();
  if (!a) return;
  std::lock_guard<std::mutex> g(I.mu);
  cudaEvent_t b = pooled_event();
  if (!b) { I.pool.push_back(a); return; }
  cudaEventRecord(b, st);
  I.pending.push_back(Instrument::Rec{a, b, kind});
  if (I.pending.size() >= 8192) resolve_locked();
}

void instrument_resolve() {
  Instrument& I = instrument();
  std::lock_guard<std::mutex> g(I.mu);
  resolve_locked();
}

}  // namespace negf

struct negf_handle {
  negf::Engine eng;
  // per-energy interface: Sancho-Rubio problems of the current energy
  int sr_l = 0, sr_r = 0;
  int sr_status = 0, sr_iters = 0;
};

using negf::Engine;

extern "C" {

int negf_create(const negf_params* p, negf_handle** out) {
  if (!p || !out) return NEGF_EINVAL;
  *out = nullptr;
  for (int i = 0; i < 3; ++i)
    if (p->reserved[i] != 0) return NEGF_EINVAL;
  negf_handle* h = new (std::nothrow) negf_handle();
  if (!h) return NEGF_ENOMEM;
  const int st = h->eng.init(*p);
  if (st != NEGF_OK) {
    delete h;
    return st;
  }
  *out = h;
  return NEGF_OK;
}

int negf_destroy(negf_handle* h) {
  if (!h) return NEGF_OK;
  const bool inited = h->eng.own_st_ != nullptr;
  const int dev = h->eng.p_.device;
  delete h;
  // the engine's blocks went back to the library's pool: return them to the device
  if (inited) negf::pool_trim(dev);
  return NEGF_OK;
}

const char* negf_strerror(int code) {
  if (code > 0) return "singular matrix: exactly-zero pivot in an inverse (LAPACK INFO > 0)";
  switch (code) {
    case NEGF_OK: return "ok";
    case NEGF_EINVAL: return "invalid argument";
    case NEGF_ENOMEM: return "device allocation failed";
    case NEGF_ECUDA: return negf::last_cuda_error_text()[0] ? negf::last_cuda_error_text() : "CUDA error";
    case NEGF_ESR_NOCONV: return "Sancho-Rubio did not converge within sr_max_iter";
    case NEGF_ENAN: return "NaN in the Sancho-Rubio update";
    case NEGF_ESTATE: return "call order violated";
    case NEGF_EADMIT: return "request exceeds the admission budget";
    case NEGF_ETIMEDOUT: return "bounded device wait timed out";
    case NEGF_EREFINE: return "refinement residual above bound";
    case NEGF_ENODEV: return "no CUDA device";
    case NEGF_ENOHAM: return "Hamiltonian slot not set";
    case NEGF_ESCRATCH: return "sizes exceed the static scratch of negf_zgemm_noalloc (m, n, k <= 512)";
    default: return "unknown error";
  }
}

int negf_device_bytes(const negf_handle* h, int64_t* bytes) {
  if (!h || !bytes) return NEGF_EINVAL;
  *bytes = h->eng.bytes();
  return NEGF_OK;
}

int negf_estimate_device_bytes(const negf_params* p, int64_t* bytes) {
  if (!p || !bytes) return NEGF_EINVAL;
  for (int i = 0; i < 3; ++i)
    if (p->reserved[i] != 0) return NEGF_EINVAL;
  const long long b = Engine::estimate_bytes(*p);
  if (b < 0) return NEGF_EINVAL;
  *bytes = b;
  return NEGF_OK;
}

int negf_set_stream(negf_handle* h, void* stream) {
  if (!h) return NEGF_EINVAL;
  Engine& e = h->eng;
  NEGF_CUDA_TRY(cudaSetDevice(e.p_.device));
  NEGF_CUDA_TRY(cudaStreamSynchronize(e.st_));
  e.st_ = stream ? static_cast<cudaStream_t>(stream) : e.own_st_;
  return NEGF_OK;
}

int negf_profile(negf_handle* h, int enable) {
  if (!h) return NEGF_EINVAL;
  NEGF_CUDA_TRY(cudaSetDevice(h->eng.p_.device));
  negf::instrument_resolve();
  negf::Instrument& I = negf::instrument();
  {
    std::lock_guard<std::mutex> g(I.mu);
    I.launches.store(0);
    for (int k = 0; k < negf::TK_COUNT; ++k) { I.kind_launches[k].store(0); I.kind_flops[k] = 0; I.kind_ms[k] = 0; }
    I.tc_complex_flops = 0;
    I.timing.store(enable != 0);
  }
  h->eng.fallbacks_ = 0;
  h->eng.ns_extra_ = 0;
  h->eng.ns_unconverged_ = 0;
  h->eng.last_rnorm_max_ = 0.0;
  h->eng.last_rk_max_ = 0.0;
  return NEGF_OK;
}

int negf_set_refinement(negf_handle* h, int32_t ns_max_steps, double ns_tol, double ns_accept) {
  if (!h) return NEGF_EINVAL;
  return h->eng.set_refinement(ns_max_steps, ns_tol, ns_accept);
}

int negf_get_stats(negf_handle* h, negf_stats* out) {
  if (!h || !out) return NEGF_EINVAL;
  NEGF_CUDA_TRY(cudaSetDevice(h->eng.p_.device));
  negf::instrument_resolve();
  negf::Instrument& I = negf::instrument();
  std::lock_guard<std::mutex> g(I.mu);
  out->launches = I.launches.load();
  out->gemm_launches = I.kind_launches[negf::TK_GEMM].load();
  out->gemm_ms = I.kind_ms[negf::TK_GEMM];
  out->gemm_flops = I.kind_flops[negf::TK_GEMM];
  out->panel_launches = I.kind_launches[negf::TK_PANEL].load();
  out->panel_ms = I.kind_ms[negf::TK_PANEL];
  out->tc_launches = I.kind_launches[negf::TK_TC].load();
  out->tc_ms = I.kind_ms[negf::TK_TC];
  out->tc_flops = I.kind_flops[negf::TK_TC];
  out->tc_complex_flops = I.tc_complex_flops;
  out->f32_gemm_ms = I.kind_ms[negf::TK_F32];
  out->slice_ms = I.kind_ms[negf::TK_SLICE];
  out->phase_sr_ms = I.kind_ms[negf::TK_PH_SR];
  out->phase_rgf_ms = I.kind_ms[negf::TK_PH_RGF];
  out->phase_inv_ms = I.kind_ms[negf::TK_PH_INV];
  out->phase_dens_ms = I.kind_ms[negf::TK_PH_DENS];
  out->fallbacks = h->eng.fallbacks_;
  out->ns_residual_max = h->eng.last_rnorm_max_;
  out->ns_extra_steps = h->eng.ns_extra_;
  out->ns_unconverged = h->eng.ns_unconverged_;
  out->ns_final_residual_max = h->eng.last_rk_max_;
  return NEGF_OK;
}

int negf_set_hamiltonian(negf_handle* h, int32_t slot, const double* Htotd, const double* HopX) {
  if (!h) return NEGF_EINVAL;
  return h->eng.set_hamiltonian(slot, Htotd, HopX);
}

int negf_build_hamiltonian(negf_handle* h, int32_t slot, const negf_wire_model* model) {
  if (!h || !model) return NEGF_EINVAL;
  return h->eng.build_hamiltonian(slot, *model);
}

int negf_contact_self_energy(negf_handle* h, double energy, double* SigmaL, double* SigmaR, double* GammaL,
                             double* GammaR, double* dosc) {
  if (!h) return NEGF_EINVAL;
  Engine& e = h->eng;
  if (!e.slot_set_[0]) return NEGF_ENOHAM;
  NEGF_CUDA_TRY(cudaSetDevice(e.p_.device));
  std::vector<negf::SrJob> jobs;
  const int rep = e.slot_rep_[0];
  if (e.slot_joint_[rep] || e.p_.contact_type != NEGF_CONTACT_LEADS) {
    jobs.push_back(negf::SrJob{energy, rep, 0, 1, 1});
    h->sr_l = h->sr_r = 0;
  } else {
    jobs.push_back(negf::SrJob{energy, rep, 0, 1, 0});
    jobs.push_back(negf::SrJob{energy, rep, 1, 0, 1});
    h->sr_l = 0;
    h->sr_r = 1;
  }
  std::vector<int> status, iters;
  e.sr_valid_ = e.rgf_valid_ = e.dens_valid_ = false;
  NEGF_TRY(e.solve_sr(jobs, status, iters));
  const int S = (int)jobs.size();
  const size_t bytes = sizeof(double2) * (size_t)e.MM_;
  struct Out { double* dst; const double2* src; } outs[4] = {
      {SigmaL, e.dSrSigL_ + (long long)h->sr_l * e.MM_}, {SigmaR, e.dSrSigR_ + (long long)h->sr_r * e.MM_},
      {GammaL, e.dSrGamL_ + (long long)h->sr_l * e.MM_}, {GammaR, e.dSrGamR_ + (long long)h->sr_r * e.MM_}};
  for (const Out& o : outs)
    if (o.dst) NEGF_CUDA_TRY(cudaMemcpyAsync(o.dst, o.src, bytes, cudaMemcpyDeviceToHost, e.st_));
  double dos[2];
  NEGF_CUDA_TRY(cudaMemcpyAsync(&dos[0], e.dSrDos_ + h->sr_l, sizeof(double), cudaMemcpyDeviceToHost, e.st_));
  NEGF_CUDA_TRY(cudaMemcpyAsync(&dos[1], e.dSrDos_ + S + h->sr_r, sizeof(double), cudaMemcpyDeviceToHost, e.st_));
  NEGF_CUDA_TRY(cudaStreamSynchronize(e.st_));
  if (dosc) { dosc[0] = dos[0]; dosc[1] = dos[1]; }
  h->sr_status = status[h->sr_l] ? status[h->sr_l] : status[h->sr_r];
  h->sr_iters = std::max(iters[h->sr_l], iters[S + h->sr_r]);
  e.cur_energy_ = energy;
  e.sr_valid_ = true;
  return h->sr_status;
}

int negf_get_retarded_greens(negf_handle* h) {
  if (!h) return NEGF_EINVAL;
  Engine& e = h->eng;
  if (!e.sr_valid_) return NEGF_ESTATE;
  NEGF_CUDA_TRY(cudaSetDevice(e.p_.device));
  std::vector<negf::Item> items(1);
  items[0] = negf::Item{e.cur_energy_, 0.0, 0.0, 0.0, 0, h->sr_l, h->sr_r, 0};
  e.rgf_valid_ = e.dens_valid_ = false;
  NEGF_TRY(e.solve_rgf(items, e.keep_columns_));
  int st = 0;
  NEGF_CUDA_TRY(cudaMemcpyAsync(&st, e.dStatus_, sizeof(int), cudaMemcpyDeviceToHost, e.st_));
  NEGF_CUDA_TRY(cudaStreamSynchronize(e.st_));
  e.cur_rgf_status_ = st;
  e.rgf_valid_ = true;
  return st;
}

int negf_copy_g_columns(negf_handle* h, double* GRLef, double* GRRgt) {
  if (!h) return NEGF_EINVAL;
  Engine& e = h->eng;
  if (!e.rgf_valid_ || !e.dCol1_) return NEGF_ESTATE;
  NEGF_CUDA_TRY(cudaSetDevice(e.p_.device));
  const int M = e.M_, N = e.p_.npx;
  const size_t ntot = (size_t)N * M;
  double* dsts[2] = {GRLef, GRRgt};
  const double2* srcs[2] = {e.dCol1_, e.dColN_};
  for (int c = 0; c < 2; ++c) {
    if (!dsts[c]) continue;
    for (int x = 0; x < N; ++x) {
      // block x (M x M, ld M) -> rows x*M.. of an Ntot x M column-major array (ld Ntot)
      NEGF_CUDA_TRY(cudaMemcpy2DAsync(dsts[c] + 2 * (size_t)x * M, ntot * sizeof(double2), srcs[c] + (size_t)x * e.MM_,
                                      M * sizeof(double2), M * sizeof(double2), M, cudaMemcpyDeviceToHost, e.st_));
    }
  }
  NEGF_CUDA_TRY(cudaStreamSynchronize(e.st_));
  return NEGF_OK;
}

int negf_calculate_gnp(negf_handle* h, double f1, double f2, double dE, double* RhoN, double* RhoP) {
  if (!h) return NEGF_EINVAL;
  Engine& e = h->eng;
  if (!e.rgf_valid_) return NEGF_ESTATE;
  NEGF_CUDA_TRY(cudaSetDevice(e.p_.device));
  std::vector<negf::Item> items(1);
  items[0] = negf::Item{e.cur_energy_, f1, f2, dE, 0, h->sr_l, h->sr_r, 0};
  std::vector<double> ed, hd;
  NEGF_TRY(e.densities(items, ed, hd));
  const long long total = e.nsite_total();
  e.last_site_.resize((size_t)e.nf_ * total);
  NEGF_CUDA_TRY(cudaMemcpyAsync(e.last_site_.data(), e.dSite_, sizeof(double) * e.nf_ * total,
                                cudaMemcpyDeviceToHost, e.st_));
  NEGF_CUDA_TRY(cudaStreamSynchronize(e.st_));
  for (long long i = 0; i < total; ++i) {
    if (RhoN) RhoN[i] += e.last_site_[i];
    if (RhoP) RhoP[i] += e.last_site_[total + i];
  }
  e.last_edens_ = ed[0];
  e.last_hdens_ = hd[0];
  e.dens_valid_ = true;
  return NEGF_OK;
}

int negf_calculate_observables(negf_handle* h, double dE, double f1, double f2, double* T12, double* EDensity,
                               double* HDensity, double* modes, double* contact_current, double* SigX, double* SigY,
                               double* SigZ) {
  if (!h) return NEGF_EINVAL;
  Engine& e = h->eng;
  if (!e.dens_valid_) return NEGF_ESTATE;
  NEGF_CUDA_TRY(cudaSetDevice(e.p_.device));
  double tr[4], trj = 0.0;
  NEGF_CUDA_TRY(cudaMemcpyAsync(tr, e.dTr_, sizeof(tr), cudaMemcpyDeviceToHost, e.st_));
  if (e.sc_()) NEGF_CUDA_TRY(cudaMemcpyAsync(&trj, e.dTrJ_, sizeof(double), cudaMemcpyDeviceToHost, e.st_));
  NEGF_CUDA_TRY(cudaStreamSynchronize(e.st_));
  const double t12 = e.sc_() ? trj : tr[1];
  if (T12) *T12 = t12;
  if (EDensity) *EDensity = e.last_edens_;
  if (HDensity) *HDensity = e.last_hdens_;
  if (modes) { modes[0] = tr[0] + tr[1]; modes[1] = tr[2] + tr[3]; }
  if (contact_current && e.sc_()) {   // supercurrent, Source/Calculate_Observables.F90:79-80
    contact_current[0] += negf::kQ * dE / negf::kH * t12;
    contact_current[1] += negf::kQ * dE / negf::kH * (-t12);
  } else if (contact_current) {   // Source/Calculate_Observables.F90:102-103
    contact_current[0] += negf::kQ * dE / negf::kH * (t12 * (f2 - f1));
    contact_current[1] += negf::kQ * dE / negf::kH * (t12 * (f1 - f2));
  }
  if (e.p_.calc_spin) {
    const long long total = e.nsite_total();
    double* outs[3] = {SigX, SigY, SigZ};
    for (int j = 0; j < 3; ++j)
      if (outs[j])
        for (long long i = 0; i < total; ++i) outs[j][i] += e.last_site_[(2 + j) * total + i];
  }
  return NEGF_OK;
}

int negf_calculate_currents(negf_handle* h, double* Jx, double* Jy, double* Jz) {
  if (!h) return NEGF_EINVAL;
  Engine& e = h->eng;
  if (!e.currents_ || !e.dens_valid_) return NEGF_ESTATE;
  const long long total = e.nsite_total();
  double* outs[3] = {Jx, Jy, Jz};
  for (int j = 0; j < 3; ++j)
    if (outs[j])
      for (long long i = 0; i < total; ++i) outs[j][i] += e.last_site_[(5 + j) * total + i];
  return NEGF_OK;
}

int negf_calculate_resolved(negf_handle* h, double* ERJx, double* ERJy, double* ERJz, double* ERRhon, double* ORJx,
                            double* ORJy, double* ORJz, double* ORRhon) {
  if (!h) return NEGF_EINVAL;
  Engine& e = h->eng;
  if (!e.currents_ || !e.dens_valid_) return NEGF_ESTATE;
  NEGF_CUDA_TRY(cudaSetDevice(e.p_.device));
  const bool er = ERJx || ERJy || ERJz || ERRhon, orb = ORJx || ORJy || ORJz || ORRhon;
  if (!er && !orb) return NEGF_OK;
  NEGF_TRY(e.ensure_resolved());
  const long long total = e.nsite_total();
  const int nq = e.n_or_fields(), no = e.p_.norb, no2 = no * no;
  if (orb) NEGF_CUDA_TRY(cudaMemsetAsync(e.dOrAcc_, 0, sizeof(double) * nq * total, e.st_));
  // the item of the last negf_calculate_gnp call is still in the handle's item list (slot 0)
  NEGF_TRY(e.resolved(1, er, orb, 1));
  std::vector<double> erh(er ? 4 * total : 0), orh(orb ? (size_t)nq * total : 0);
  if (er) NEGF_CUDA_TRY(cudaMemcpyAsync(erh.data(), e.dEr_, sizeof(double) * erh.size(), cudaMemcpyDeviceToHost, e.st_));
  if (orb)
    NEGF_CUDA_TRY(cudaMemcpyAsync(orh.data(), e.dOrAcc_, sizeof(double) * orh.size(), cudaMemcpyDeviceToHost, e.st_));
  NEGF_CUDA_TRY(cudaStreamSynchronize(e.st_));
  double* ero[4] = {ERJx, ERJy, ERJz, ERRhon};
  for (int f = 0; f < 4; ++f)
    if (ero[f])
      for (long long i = 0; i < total; ++i) ero[f][i] += erh[(size_t)f * total + i];
  double* oro[3] = {ORJx, ORJy, ORJz};
  for (int q = 0; q < nq; ++q) {
    double* dst = q < 3 * no2 ? (oro[q / no2] ? oro[q / no2] + (size_t)(q % no2) * total : nullptr)
                              : (ORRhon ? ORRhon + (size_t)(q - 3 * no2) * total : nullptr);
    if (!dst) continue;
    for (long long i = 0; i < total; ++i) dst[i] += orh[(size_t)q * total + i];
  }
  return NEGF_OK;
}

int negf_solve_batch(negf_handle* h, const negf_request* req, int32_t n, negf_result* res, double* RhoN, double* RhoP,
                     double* SigX, double* SigY, double* SigZ) {
  if (!h) return NEGF_EINVAL;
  double* outs[8] = {RhoN, RhoP, SigX, SigY, SigZ, nullptr, nullptr, nullptr};
  return h->eng.batch_solve(req, n, res, outs);
}

int negf_solve_batch_ex(negf_handle* h, const negf_request* req, int32_t n, negf_result* res,
                        const negf_batch_outputs* out) {
  if (!h) return NEGF_EINVAL;
  double* outs[8] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  if (out) {
    for (int i = 0; i < 8; ++i)
      if (out->reserved[i]) return NEGF_EINVAL;
    negf::ResolvedOut ro;
    ro.er[0] = out->ERJx; ro.er[1] = out->ERJy; ro.er[2] = out->ERJz; ro.er[3] = out->ERRhon;
    ro.orj[0] = out->ORJx; ro.orj[1] = out->ORJy; ro.orj[2] = out->ORJz; ro.orrho = out->ORRhon;
    if ((out->Jx || out->Jy || out->Jz || ro.any_er() || ro.any_or()) && !h->eng.currents_) return NEGF_ESTATE;
    double* o[8] = {out->RhoN, out->RhoP, out->SigX, out->SigY, out->SigZ, out->Jx, out->Jy, out->Jz};
    for (int i = 0; i < 8; ++i) outs[i] = o[i];
    return h->eng.batch_solve(req, n, res, outs, nullptr, &ro);
  }
  return h->eng.batch_solve(req, n, res, outs);
}

}  // extern "C"
