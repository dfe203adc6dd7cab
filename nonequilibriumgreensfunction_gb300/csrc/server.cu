// Request server (negf_server_*), with each request's state kept on the device (host
// worker threads drive the batches): replaces the MPI master/worker energy
// sweep of Source/NEGF_Main.F90:21-27 with continuous batching on one GPU.
//
// Requests (a wire's Htotd/HopX and a list of energy points) are queued by submit().
// Admission assigns a request to the worker of its geometry (npx, npy, npz, norb, HopX)
// once that worker has a free Hamiltonian slot; a worker (an Engine with its own CUDA
// stream and host thread) is created when the HBM budget has room for its block store
// (max_batch * Npx * M^2 * 16 bytes plus its slots and work buffers) and idle workers are
// destroyed to make room.  Each worker repeatedly packs the pending energy points of all
// its admitted requests, oldest first, into one batch of up to max_batch points, so
// requests that arrive while a batch runs join the next one.  Workers of different
// geometries run concurrently.  Per-point arithmetic never mixes batch items, so a
// request's results are independent of what it was batched with.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <tuple>
#include <vector>

#include "engine.h"

namespace {

using Clock = std::chrono::steady_clock;

struct GeomKey {
  int npx, npy, npz, norb;
  size_t hop_hash;
  bool operator<(const GeomKey& o) const {
    return std::tie(npx, npy, npz, norb, hop_hash) < std::tie(o.npx, o.npy, o.npz, o.norb, o.hop_hash);
  }
};

struct Worker;

struct Request {
  int64_t id = 0;
  GeomKey key{};
  std::vector<double2> H, hop;
  bool has_model = false;       // generate H on the device from `model` (and V)
  negf_wire_model model{};
  std::vector<double> V;
  std::vector<double> e, f1, f2, dE;
  std::vector<double> res7;   // 7 per energy
  std::vector<double> rho;    // RhoN then RhoP, npx*npy*npz each
  int next = 0, n_done = 0, status = 0, slot = -1;
  bool uploaded = false, done = false;
  double t_submit = 0, t_admit = -1, t_done = -1;
  Worker* w = nullptr;
};

struct Worker {
  GeomKey key{};
  std::unique_ptr<negf::Engine> eng;
  std::vector<Request*> slot_owner;
  std::deque<Request*> active;    // admitted (slot assigned), energy points pending or in flight
  std::thread th;
  long long bytes = 0;
  bool busy = false;
  bool quit = false;
  // true only while the worker's thread is blocked in its wait on work_cv: the one state in
  // which another thread may evict it (its thread runs none of the worker's code then, and
  // wakes on `quit`).  A worker that has just finished a batch may release the server lock
  // inside admit_locked; it must not be evicted from under itself there.
  bool waiting = false;
};

size_t hash_bytes(const void* p, size_t n) {
  // FNV-1a over the bytes of HopX
  const unsigned char* c = static_cast<const unsigned char*>(p);
  size_t h = 1469598103934665603ull;
  for (size_t i = 0; i < n; ++i) { h ^= c[i]; h *= 1099511628211ull; }
  return h;
}

}  // namespace

struct negf_server {
  negf_serve_params p{};
  std::mutex mu;
  std::condition_variable work_cv, done_cv;
  std::deque<Request*> pending;
  std::map<int64_t, std::unique_ptr<Request>> reqs;
  std::map<GeomKey, std::unique_ptr<Worker>> workers;
  int64_t next_id = 1;
  long long budget = 0, used = 0;
  // engine churn: engines created and released, and the host seconds spent in their
  // allocation (negf_create's work) and release (their device frees)
  long long n_created = 0, n_released = 0;
  double t_create = 0.0, t_release = 0.0;
  Clock::time_point t0 = Clock::now();

  double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }

  negf_params engine_params(const GeomKey& k) const {
    negf_params ep;
    std::memset(&ep, 0, sizeof(ep));
    ep.npx = k.npx; ep.npy = k.npy; ep.npz = k.npz; ep.norb = k.norb;
    ep.n_hamiltonians = p.slots_per_geometry;
    ep.max_batch = p.max_batch;
    ep.eta = p.eta; ep.sr_tol = p.sr_tol; ep.sr_max_iter = p.sr_max_iter;
    ep.calc_spin = p.calc_spin; ep.precision = p.precision; ep.device = p.device;
    ep.mixed_slices = p.mixed_slices;
    return ep;
  }

  // an engine's device bytes: Engine::alloc counted without allocating, plus 64 MB for the
  // allocator's rounding and the library's per-context state
  long long estimate(const GeomKey& k) const {
    const long long b = negf::Engine::estimate_bytes(engine_params(k));
    return b < 0 ? b : b + (64LL << 20);
  }

  // Destroy idle workers (no admitted requests, not running a batch) until `need` bytes
  // fit the budget.  `self` (the calling worker, if any) is never chosen.
  bool evict_idle_locked(long long need, Worker* self) {
    std::vector<std::unique_ptr<Worker>> dead;
    long long freed = 0;
    for (auto it = workers.begin(); it != workers.end() && budget - used + freed < need;) {
      Worker* w = it->second.get();
      const bool idle = w != self && w->waiting && !w->busy && w->active.empty() &&
                        std::all_of(w->slot_owner.begin(), w->slot_owner.end(), [](Request* r) { return r == nullptr; });
      if (idle) {
        w->quit = true;
        freed += w->bytes;
        dead.push_back(std::move(it->second));
        it = workers.erase(it);
      } else {
        ++it;
      }
    }
    if (!dead.empty()) {
      work_cv.notify_all();
      mu.unlock();
      double t_rel = 0.0;
      for (auto& w : dead) {
        if (w->th.joinable()) w->th.join();
        const double t0 = now();
        w.reset();   // frees the engine's device memory
        t_rel += now() - t0;
      }
      mu.lock();
      used -= freed;
      n_released += (long long)dead.size();
      t_release += t_rel;
    }
    return budget - used >= need;
  }

  // Admit pending requests (oldest first) whose geometry has a worker with a free slot,
  // creating workers within the HBM budget.  Called with `mu` held; may release it while
  // idle workers are joined, so the pending list is re-scanned from the front afterwards.
  void admit_locked(Worker* self) {
    for (auto it = pending.begin(); it != pending.end();) {
      Request* r = *it;
      Worker* w = nullptr;
      auto wi = workers.find(r->key);
      if (wi != workers.end()) {
        w = wi->second.get();
      } else {
        const long long need = estimate(r->key);
        if (need < 0 || need > budget) {
          // a geometry no engine accepts (e.g. M > 800 in the mixed form), or one whose
          // engine alone exceeds the whole budget: it would never be admitted
          r->status = need < 0 ? NEGF_EINVAL : NEGF_EADMIT;
          r->done = true;
          r->t_done = now();
          it = pending.erase(it);
          done_cv.notify_all();
          continue;
        }
        if (budget - used < need) {
          const bool ok = evict_idle_locked(need, self);
          it = std::find(pending.begin(), pending.end(), r);   // the lock may have been released
          if (it == pending.end()) { it = pending.begin(); continue; }
          if (!ok) { ++it; continue; }
        }
        wi = workers.find(r->key);
        if (wi != workers.end()) {
          w = wi->second.get();
        } else {
          auto nw = std::make_unique<Worker>();
          nw->key = r->key;
          nw->eng = std::make_unique<negf::Engine>();
          const double t0 = now();
          int irc = nw->eng->init(engine_params(r->key));
          if (irc == NEGF_ENOMEM) {
            // the library's pool keeps released engines' blocks for reuse; when they do not
            // fit this engine's buffers, give them back to the device and try once more
            nw->eng = std::make_unique<negf::Engine>();
            negf::pool_trim(p.device);
            irc = nw->eng->init(engine_params(r->key));
          }
          t_create += now() - t0;
          if (irc != NEGF_OK) {
            r->status = NEGF_ENOMEM;
            r->done = true;
            r->t_done = now();
            it = pending.erase(it);
            done_cv.notify_all();
            continue;
          }
          nw->bytes = nw->eng->bytes();
          used += nw->bytes;
          ++n_created;
          nw->slot_owner.assign(p.slots_per_geometry, nullptr);
          w = nw.get();
          workers[r->key] = std::move(nw);
          w->th = std::thread([this, w] { worker_loop(w); });
        }
      }
      auto free_slot = std::find(w->slot_owner.begin(), w->slot_owner.end(), nullptr);
      if (free_slot == w->slot_owner.end()) { ++it; continue; }
      r->slot = (int)(free_slot - w->slot_owner.begin());
      *free_slot = r;
      r->w = w;
      w->active.push_back(r);
      it = pending.erase(it);
      work_cv.notify_all();
    }
  }

  void worker_loop(Worker* w) {
    cudaSetDevice(p.device);
    negf::Engine& eng = *w->eng;
    const long long total = (long long)w->key.npx * w->key.npy * w->key.npz;
    const int nf = eng.nf_;
    std::vector<double> items((size_t)nf * total * (size_t)p.max_batch);
    std::unique_lock<std::mutex> lk(mu);
    for (;;) {
      w->waiting = true;
      work_cv.wait(lk, [&] {
        if (w->quit) return true;
        for (Request* r : w->active)
          if (!r->uploaded || r->next < (int)r->e.size()) return true;
        return false;
      });
      w->waiting = false;
      if (w->quit) return;
      w->busy = true;
      // uploads of newly admitted requests
      std::vector<Request*> up;
      for (Request* r : w->active)
        if (!r->uploaded) up.push_back(r);
      if (!up.empty()) {
        lk.unlock();
        std::vector<int> st(up.size());
        for (size_t i = 0; i < up.size(); ++i) {
          Request* r = up[i];
          if (r->has_model) {
            r->model.V = r->V.empty() ? nullptr : r->V.data();
            st[i] = eng.build_hamiltonian(r->slot, r->model);
          } else {
            st[i] = eng.set_hamiltonian(r->slot, reinterpret_cast<const double*>(r->H.data()),
                                        reinterpret_cast<const double*>(r->hop.data()));
          }
        }
        lk.lock();
        const double t = now();
        for (size_t i = 0; i < up.size(); ++i) {
          up[i]->uploaded = true;
          up[i]->t_admit = t;
          if (st[i] != NEGF_OK) { up[i]->status = st[i]; up[i]->next = (int)up[i]->e.size(); }
        }
      }
      // pack the next batch: oldest admitted requests first
      std::vector<negf_request> batch;
      std::vector<std::pair<Request*, int>> owner;
      for (Request* r : w->active) {
        while (r->uploaded && r->next < (int)r->e.size() && (int)batch.size() < p.max_batch) {
          const int i = r->next++;
          negf_request q{};
          q.energy = r->e[i]; q.f1 = r->f1[i]; q.f2 = r->f2[i]; q.dE = r->dE[i]; q.slot = r->slot;
          batch.push_back(q);
          owner.emplace_back(r, i);
        }
        if ((int)batch.size() >= p.max_batch) break;
      }
      std::vector<negf_result> res(batch.size());
      int rc = NEGF_OK;
      if (!batch.empty()) {
        lk.unlock();
        rc = eng.batch_solve(batch.data(), (int)batch.size(), res.data(), nullptr, items.data());
        lk.lock();
      }
      // scatter results; each energy's densities are added to its request in energy order
      // (the order a single batch over the whole request uses), so sums do not depend on
      // how the request's energies were split into batches
      std::vector<Request*> touched;
      for (size_t i = 0; i < owner.size(); ++i) {
        Request* r = owner[i].first;
        const int k = owner[i].second;
        const negf_result& o = res[i];
        double* d = r->res7.data() + 7 * (size_t)k;
        d[0] = o.T12; d[1] = o.EDensity; d[2] = o.HDensity; d[3] = o.modes[0]; d[4] = o.modes[1];
        d[5] = o.dosc[0]; d[6] = o.dosc[1];
        const int stv = rc != NEGF_OK ? rc : o.status;
        if (stv != 0 && r->status == 0) r->status = stv;
        r->n_done++;
        const double* si = items.data() + i * nf * (size_t)total;
        for (long long j = 0; j < total; ++j) {
          r->rho[j] += si[j];
          r->rho[total + j] += si[total + j];
        }
        if (std::find(touched.begin(), touched.end(), r) == touched.end()) touched.push_back(r);
      }
      for (Request* r : touched) {
        if (r->n_done == (int)r->e.size()) {
          r->done = true;
          r->t_done = now();
          w->slot_owner[r->slot] = nullptr;
          w->active.erase(std::find(w->active.begin(), w->active.end(), r));
        }
      }
      w->busy = false;
      admit_locked(w);
      done_cv.notify_all();
      const bool idle = w->active.empty() &&
                        std::all_of(w->slot_owner.begin(), w->slot_owner.end(), [](Request* r) { return r == nullptr; });
      auto it = workers.find(w->key);
      if (idle && !pending.empty() && it != workers.end() && it->second.get() == w) {
        // requests of other geometries wait for memory: release this idle engine and exit
        std::unique_ptr<Worker> self = std::move(it->second);
        workers.erase(it);
        const long long freed = self->bytes;
        lk.unlock();
        const double t0 = now();
        self->eng.reset();
        const double t_rel = now() - t0;
        lk.lock();
        used -= freed;
        ++n_released;
        t_release += t_rel;
        admit_locked(nullptr);
        done_cv.notify_all();
        self->th.detach();
        return;
      }
    }
  }
};

extern "C" {

int negf_server_create(const negf_serve_params* p, negf_server** out) {
  if (!p || !out) return NEGF_EINVAL;
  *out = nullptr;
  if (p->max_batch < 1 || p->slots_per_geometry < 1 || !(p->sr_tol > 0) || p->sr_max_iter < 1) return NEGF_EINVAL;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return NEGF_ENODEV;
  if (p->device < 0 || p->device >= ndev) return NEGF_EINVAL;
  auto s = std::make_unique<negf_server>();
  s->p = *p;
  NEGF_CUDA_TRY(cudaSetDevice(p->device));
  size_t fr = 0, tot = 0;
  NEGF_CUDA_TRY(cudaMemGetInfo(&fr, &tot));
  s->budget = p->hbm_budget_bytes > 0 ? p->hbm_budget_bytes : (long long)(0.8 * (double)fr);
  *out = s.release();
  return NEGF_OK;
}

int negf_server_submit(negf_server* s, const negf_wire_request* r, int64_t* id) {
  if (!s || !r || !id || r->n_energies < 1 || !r->energies || !r->f1 || !r->f2 || !r->dE) return NEGF_EINVAL;
  if (r->model ? (r->Htotd || r->HopX || r->norb != 4) : (!r->Htotd || !r->HopX)) return NEGF_EINVAL;
  if (r->npx < 2 || r->npy < 1 || r->npz < 1 || r->norb < 1 || r->norb > 4) return NEGF_EINVAL;
  auto q = std::make_unique<Request>();
  const long long m = (long long)r->norb * r->npy * r->npz, mm = m * m;
  const double2* x = reinterpret_cast<const double2*>(r->HopX);
  std::vector<double2> hop_model;
  if (r->model) {
    for (int i = 0; i < 8; ++i)
      if (r->model->reserved[i] != 0) return NEGF_EINVAL;
    q->has_model = true;
    q->model = *r->model;
    if (r->model->V) q->V.assign(r->model->V, r->model->V + (size_t)r->npx * r->npy * r->npz);
    // the dense HopX the device build produces keys the geometry, so model and uploaded
    // wires with the same HopX share a worker
    hop_model.assign(mm, make_double2(0.0, 0.0));
    for (long long st = 0; st < m / 4; ++st)
      for (int a = 0; a < 4; ++a)
        for (int b = 0; b < 4; ++b)
          hop_model[(st * 4 + b) * m + st * 4 + a] = make_double2(r->model->hop[0][a][b][0], r->model->hop[0][a][b][1]);
    x = hop_model.data();
  } else {
    const double2* h = reinterpret_cast<const double2*>(r->Htotd);
    q->H.assign(h, h + r->npx * mm);
    q->hop.assign(x, x + mm);
  }
  q->e.assign(r->energies, r->energies + r->n_energies);
  q->f1.assign(r->f1, r->f1 + r->n_energies);
  q->f2.assign(r->f2, r->f2 + r->n_energies);
  q->dE.assign(r->dE, r->dE + r->n_energies);
  q->res7.assign(7 * (size_t)r->n_energies, 0.0);
  q->rho.assign(2 * (size_t)r->npx * r->npy * r->npz, 0.0);
  q->key = GeomKey{r->npx, r->npy, r->npz, r->norb, hash_bytes(x, sizeof(double2) * mm)};
  std::lock_guard<std::mutex> g(s->mu);
  q->id = s->next_id++;
  q->t_submit = s->now();
  *id = q->id;
  Request* raw = q.get();
  s->reqs[q->id] = std::move(q);
  s->pending.push_back(raw);
  s->admit_locked(nullptr);
  return NEGF_OK;
}

int negf_server_poll(negf_server* s, int64_t id, negf_wire_status* st, double* res7, double* rho, int32_t release) {
  if (!s) return NEGF_EINVAL;
  std::lock_guard<std::mutex> g(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) return NEGF_EINVAL;
  Request* r = it->second.get();
  if (st) {
    st->done = r->done ? 1 : 0;
    st->status = r->status;
    st->n_done = r->n_done;
    st->t_submit = r->t_submit;
    st->t_admit = r->t_admit;
    st->t_done = r->t_done;
  }
  if (r->done) {
    if (res7) std::memcpy(res7, r->res7.data(), sizeof(double) * r->res7.size());
    if (rho) std::memcpy(rho, r->rho.data(), sizeof(double) * r->rho.size());
    if (release) s->reqs.erase(it);
  }
  return NEGF_OK;
}

int negf_server_wait(negf_server* s, int64_t id, double timeout_s) {
  if (!s) return NEGF_EINVAL;
  std::unique_lock<std::mutex> lk(s->mu);
  auto pred = [&] {
    auto it = s->reqs.find(id);
    return it == s->reqs.end() || it->second->done;
  };
  if (!s->done_cv.wait_for(lk, std::chrono::duration<double>(timeout_s), pred)) return NEGF_ETIMEDOUT;
  return s->reqs.count(id) ? NEGF_OK : NEGF_EINVAL;
}

double negf_server_clock(const negf_server* s) { return s ? s->now() : 0.0; }

int negf_server_get_stats(negf_server* s, negf_server_stats* out) {
  if (!s || !out) return NEGF_EINVAL;
  std::lock_guard<std::mutex> g(s->mu);
  std::memset(out, 0, sizeof(*out));
  out->engines_created = s->n_created;
  out->engines_released = s->n_released;
  out->create_s = s->t_create;
  out->release_s = s->t_release;
  out->engines_live = (int64_t)s->workers.size();
  out->bytes_used = s->used;
  out->bytes_budget = s->budget;
  return NEGF_OK;
}

int negf_server_destroy(negf_server* s) {
  if (!s) return NEGF_EINVAL;
  std::vector<std::unique_ptr<Worker>> ws;
  {
    std::lock_guard<std::mutex> g(s->mu);
    for (auto& kv : s->workers) kv.second->quit = true;
    s->work_cv.notify_all();
    for (auto& kv : s->workers) ws.push_back(std::move(kv.second));
    s->workers.clear();
  }
  for (auto& w : ws)
    if (w->th.joinable()) w->th.join();
  ws.clear();
  const int dev = s->p.device;
  delete s;
  negf::pool_trim(dev);   // the released engines' blocks go back to the device
  return NEGF_OK;
}

}  // extern "C"
