"""Benchmark: energy-point solves/s of the per-energy NEGF solve at M = 400.

Workload ("ti_wire_M400_Npx100"): the 4-band TI nanowire with Npy = Npz = 10 (M = 400),
Npx = 100, axial flux 0.5 Phi_0 (Peierls phases on the y hops), Zeeman 0.01 eV, Anderson
disorder W = 0.1 eV with 4 seeds (4 Hamiltonian slots, 1 GB of complex128 on the device),
eta = 1e-5, Sancho-Rubio tolerance 1e-10, kT = 0.025 eV, mu_L - mu_R = 0.01 eV, energies
from the 512-point grid in [-0.3, 0.3] eV.  Synthetic, seeded inputs of the stated
shapes (no dataset exists for this workload).

One step = one batch of --batch requests (consecutive grid energies, seeds round-robin),
solved through negf_solve_batch with the Hamiltonians resident in HBM.  `value` is
solves/s over K steps timed with CUDA events on the stream the library launches on.
`e2e` repeats the steps through the public API with host buffers: every step uploads the
4 Hamiltonians from pinned host memory and reads the results back.

--impl reference times the CPU restatement of the reference algorithm (oracle/) on this
host's cores on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

import numpy as np  # noqa: E402

WORKLOAD = "ti_wire_M400_Npx100"
NPX, NPY, NPZ = 100, 10, 10
SEEDS = 4
N_E = 512
ETA, SR_TOL, KT = 1e-5, 1e-10, 0.025
MU = (0.005, -0.005)
FLUX, ZEEMAN, W = 0.5, 0.01, 0.1
METRIC = "energy-point solves/s at M=400 (mixed vs FP64, T err<=1e-6)"


def energy_grid():
    return np.linspace(-0.3, 0.3, N_E)


def fermi(e, mu, kt):
    x = (e - mu) / kt
    return 0.0 if x > 700 else 1.0 / (1.0 + math.exp(x))


def step_requests(step, batch, rank, world):
    """Requests of one step: batch/4 consecutive grid energies, each for all 4 disorder
    seeds (the config's 512 energies x 4 seeds, walked energy-major), so the seeds of one
    energy share its lead decimation; ranks take disjoint energies (the units are
    independent, no exchange between ranks)."""
    grid = energy_grid()
    ne = max(1, batch // SEEDS)
    idx = [((step * world + rank) * ne + i // SEEDS) % N_E for i in range(batch)]
    e = grid[idx]
    slots = np.array([i % SEEDS for i in range(batch)], dtype=np.int32)
    f1 = np.array([fermi(x, MU[0], KT) for x in e])
    f2 = np.array([fermi(x, MU[1], KT) for x in e])
    return e, f1, f2, slots


def max_over_ranks(value, dist, device):
    """The slowest rank's time (the job finishes when it does): an all-reduce MAX of one
    scalar; `device` is the rank's GPU under NCCL, the CPU under gloo."""
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def scope_flops_per_solve(m, npx, n_sr, n_leads=2):
    """The work model of the hot-path scope table (real flops per energy point):
    F = 96 M^3 Npx + n_leads (72 n_SR + 56) M^3 + 16 M^3 -- per slice 12 complex M^3
    products or inverses of 8 M^3 each (both sweeps, both column propagations, the two
    G Gamma products), per decimation iteration 8 products and 1 inverse per lead, the
    transmission's 2 products.  It counts dense HopX products that the site-local HopX
    of these wires makes O(M^2) and does not share the decimation between seeds."""
    m3 = float(m) ** 3
    return 96.0 * m3 * npx + n_leads * (72.0 * n_sr + 56.0) * m3 + 16.0 * m3


def algorithmic_flops_per_solve(m, npx, n_sr, n_seeds_sharing=SEEDS):
    """Work model of the solve (real flops), per energy point:
    RGF: per slice 2 inverses + 4 complex GEMMs (column 1, column N, G Gamma_L, G Gamma_R),
    each 8 M^3 -> 48 M^3 per slice (HopX products are site-local, O(M^2));
    Sancho-Rubio: per iteration 10 GEMMs + 1 inverse (both leads share t, t~) = 88 M^3,
    plus 3 inverses at set-up/final = 24 M^3, shared by the seeds at one energy;
    traces: 4 GEMMs = 32 M^3."""
    m3 = float(m) ** 3
    rgf = 48.0 * m3 * npx
    sr = (88.0 * n_sr + 24.0) * m3 / n_seeds_sharing
    return rgf + sr + 32.0 * m3


class ClockSampler:
    def __init__(self, path):
        self.path = path
        self.proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + q, "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self, device_index):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": []}
        try:
            rows = [ln.split(",") for ln in open(self.path).read().strip().splitlines()]
        except Exception:
            return out
        rows = [[c.strip() for c in r] for r in rows if len(r) >= 9 and r[0].strip() == str(device_index)]
        if not rows:
            return out
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in rows:
            for name, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        out["sm_mhz"] = statistics.median(sm) if sm else None
        out["sm_max_mhz"] = max(mx) if mx else None
        out["reasons"] = sorted(reasons)
        out["samples"] = len(rows)
        return out


def measured_peaks():
    try:
        return json.load(open(os.path.join(REPO, "MEASURED_PEAKS.json")))
    except Exception:
        return {}


def fp64_zgemm_peak_tflops(torch, device):
    """FP64 denominator for the FP64 form: cuBLAS ZGEMM (complex128, 4096^3) measured live."""
    n = 4096
    a = torch.randn(n, n, dtype=torch.complex128, device=device)
    b = torch.randn(n, n, dtype=torch.complex128, device=device)
    for _ in range(2):
        torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 0.0
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = max(best, 8.0 * n ** 3 / (e0.elapsed_time(e1) * 1e-3) / 1e12)
    del a, b
    torch.cuda.empty_cache()
    return best


def build_hamiltonians():
    from nonequilibriumgreensfunction_gb300 import hamiltonian as HB
    hams = []
    for seed in range(SEEDS):
        h, x = HB.ti_wire(NPX, NPY, NPZ, zeeman=ZEEMAN, flux=FLUX, W=W, seed=seed)
        hams.append((h, x))
    return hams


def cpu_sample(n_energies=1):
    """The oracle (CPU restatement of the reference algorithm) on a bounded sample: the
    first n_energies requests of step 0 at full size.  Returns (solves/s, threads, text)."""
    from oracle import negf_oracle as O
    from nonequilibriumgreensfunction_gb300 import hamiltonian as HB
    e, f1, f2, slots = step_requests(0, n_energies, 0, 1)
    opt = O.SolveOptions(eta=ETA, sr_tol=SR_TOL, kT=KT, calc_spin=True)
    hams = {s: HB.ti_wire(NPX, NPY, NPZ, zeeman=ZEEMAN, flux=FLUX, W=W, seed=s) for s in set(int(v) for v in slots)}
    t0 = time.perf_counter()
    for i in range(n_energies):
        h, x = hams[int(slots[i])]
        O.energy_sweep(h, x, float(e[i]), MU, 0.6 / (N_E - 1), NPY, NPZ, opt)
    dt = time.perf_counter() - t0
    threads = os.cpu_count() or 1
    return n_energies / dt, threads, ("%d energy point(s) of the workload at full size (M=400, Npx=100), "
                                      "NumPy/OpenBLAS on all host threads" % n_energies)


SERVING_XS = (6, 8, 10)            # Npy = Npz of the served wires (M = 144, 256, 400)
SERVING_NPX = (50, 75, 100)
SERVING_E = (8, 64)                # energies per request, log-uniform
# the serving configuration as stated: Npy = Npz in {6, 8, 10, 12, 14} (M up to 784), Npx
# uniform in [50, 200], energies per request log-uniform in [64, 1024] (scaled by
# --serving-energy-scale to bound the run)
C4_XS = (6, 8, 10, 12, 14)
C4_NPX = (50, 200)
C4_E = (64, 1024)


def serving_request(rng, mix="reduced", e_scale=1.0):
    """One request of the serving mix: a wire given as a model (its Hamiltonian is built on
    the device), per-request disorder seed, W ~ U[0, 0.2] eV and flux ~ U[0, 1] Phi_0.
    mix "reduced": the bench's default mix; "c4": the serving configuration's cross-sections,
    Npx in [50, 200] and [64, 1024] energies times e_scale."""
    from nonequilibriumgreensfunction_gb300 import hamiltonian as HB
    if mix == "c4":
        n = int(rng.choice(C4_XS))
        npx = int(rng.integers(C4_NPX[0], C4_NPX[1] + 1))
        lo, hi = C4_E[0] * e_scale, C4_E[1] * e_scale
    else:
        n = int(rng.choice(SERVING_XS))
        npx = int(rng.choice(SERVING_NPX))
        lo, hi = SERVING_E
    ne = max(1, int(round(math.exp(rng.uniform(math.log(lo), math.log(hi))))))
    e = np.sort(rng.choice(energy_grid(), size=ne, replace=False))
    model = HB.wire_model(W=float(rng.uniform(0.0, 0.2)), seed=int(rng.integers(1 << 62)),
                          flux=float(rng.uniform(0.0, 1.0)), zeeman=ZEEMAN)
    f1 = np.array([fermi(x, MU[0], KT) for x in e])
    f2 = np.array([fermi(x, MU[1], KT) for x in e])
    return dict(shape=(npx, n, n), model=model, energies=e, f1=f1, f2=f2, dE=0.6 / (N_E - 1))


def serving_bench(seconds, device, form="mixed", mix="reduced", e_scale=1.0, burst_n=24):
    """p50/p99 latency under Poisson arrivals at 80% of the measured capacity.  mix
    "reduced" (the default bench run): cross-sections {6, 8, 10}, Npx in {50, 75, 100},
    8-64 energies per request instead of {6..14}, [50, 200] and 64-1024; mix "c4": the
    serving configuration's wires with the energies per request scaled by e_scale."""
    from nonequilibriumgreensfunction_gb300.serving import Server, run_poisson_load
    rng = np.random.default_rng(4)
    mk = lambda g: serving_request(g, mix, e_scale)  # noqa: E731
    slots = 8 if mix == "reduced" else 2
    with Server(precision=form, max_batch=32, slots_per_geometry=slots, eta=ETA, sr_tol=SR_TOL,
                device=device) as srv:
        # capacity: a closed burst (also creates the engines of the geometries)
        burst = [mk(rng) for _ in range(burst_n)]
        t0 = time.perf_counter()
        ids = [srv.submit_model(*r["shape"], r["model"], r["energies"], r["f1"], r["f2"], r["dE"]) for r in burst]
        for rid in ids:
            srv.wait(rid, timeout=1800.0)
            srv.result(rid)
        cap_wall = time.perf_counter() - t0
        cap_solves = sum(r["energies"].size for r in burst)
        capacity = cap_solves / cap_wall
        mean_e = float(np.mean([r["energies"].size for r in burst]))
        rate = 0.8 * capacity / mean_e
        lat, solves, wall = run_poisson_load(srv, mk, rate, seconds, rng)
        churn = srv.stats()
    if mix == "c4":
        load = ("Poisson arrivals at 0.8 x measured capacity; Npy=Npz in {6,8,10,12,14} (M up to 784), "
                "Npx ~ U[50,200], %g-%g energies/request (log-uniform; the configuration's 64-1024 x %g), "
                "W~U[0,0.2] eV, flux~U[0,1] Phi0, per-request seed; wires sent as models and built on the "
                "device" % (C4_E[0] * e_scale, C4_E[1] * e_scale, e_scale))
    else:
        load = ("Poisson arrivals at 0.8 x measured capacity; Npy=Npz in {6,8,10}, Npx in {50,75,100}, "
                "8-64 energies/request (log-uniform), W~U[0,0.2] eV, flux~U[0,1] Phi0, per-request seed; "
                "wires sent as models and built on the device")
    return {"p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "p90_s": float(np.percentile(lat, 90)), "mean_s": float(np.mean(lat)),
            "solves_per_s": solves / wall, "capacity_solves_per_s": capacity, "arrival_rate_req_per_s": rate,
            "requests": int(lat.size), "seconds": seconds, "wall_s": wall, "form": form, "mix": mix,
            "engines": churn, "load": load}


def run_serving_bench(args):
    """The serving leg on its own (--workload serving): one JSON line with a result per form."""
    forms = ["mixed", "fp64"] if args.serving_form == "both" else [args.serving_form]
    out = {"metric": "serving p50/p99 latency (s) and solves/s under Poisson arrivals at 80% of capacity",
           "workload": "serving_%s" % args.serving_config, "data": "synthetic", "results": []}
    for f in forms:
        secs = args.serving_seconds if f == "mixed" or args.serving_fp64_seconds <= 0 else args.serving_fp64_seconds
        scale = args.serving_energy_scale if f == "mixed" else args.serving_fp64_energy_scale
        out["results"].append(serving_bench(secs, 0, form=f, mix=args.serving_config, e_scale=scale,
                                            burst_n=args.serving_burst))
    print(json.dumps(out), flush=True)


def run_scf_bench(args):
    """Self-consistent bias point at the config-5 geometry: Npx = 60, Npy = Npz = 12 (M = 576),
    W = 0.1 eV, mu_L - mu_R = 0.05 eV, eps_r = 100, a 0.1 eV gate on the wire surface, linear
    mixing 0.3 for 10 iterations, mixed form.  The sample is --scf-energies energies x
    --scf-seeds disorder seeds per iteration (the configuration names 1024 x 8), stated in
    the output.  The mixed solve is then compared with the FP64 solve on the converged
    potential: T(E) at 16 energies."""
    from nonequilibriumgreensfunction_gb300 import Solver, scf
    from nonequilibriumgreensfunction_gb300 import hamiltonian as HB
    npx, npy, npz, n_iter = 60, 12, 12, 10
    n_seeds, n_e = args.scf_seeds, args.scf_energies
    mu_l, mu_r = 0.025, -0.025
    models = [HB.wire_model(W=0.1, seed=s, zeeman=ZEEMAN) for s in range(n_seeds)]
    energies = np.linspace(-0.3, 0.3, n_e)
    de = energies[1] - energies[0]
    with Solver(npx, npy, npz, n_hamiltonians=n_seeds, max_batch=min(n_e * n_seeds, 256), eta=ETA, sr_tol=SR_TOL,
                precision="mixed") as s:
        t0 = time.perf_counter()
        out = scf.run_scf(s, models, energies, de, mu_l, mu_r, KT, eps_r=100.0, u_gate=0.1, beta=0.3,
                          n_iter=n_iter)
        wall = time.perf_counter() - t0
    sub = np.linspace(0, n_e - 1, 16).astype(int)
    e_sub = energies[sub]
    f1 = np.array([scf.occupation(e, mu_l, KT) for e in e_sub])
    f2 = np.array([scf.occupation(e, mu_r, KT) for e in e_sub])
    t = {}
    for prec in ("mixed", "fp64"):
        with Solver(npx, npy, npz, max_batch=16, eta=ETA, sr_tol=SR_TOL, precision=prec) as s:
            m = dict(models[0])
            m["V"] = out["U"][..., 0]
            s.build_hamiltonian(m)
            t[prec] = s.solve_batch(e_sub, f1, f2, de)["T12"]
    rel = np.abs(t["mixed"] - t["fp64"]) / np.maximum(np.abs(t["fp64"]), 1e-3)
    solves = n_iter * n_e * n_seeds
    line = {"metric": "self-consistent bias point: wall time per outer iteration", "workload": "scf_M576_Npx60",
            "value": wall / n_iter, "unit": "s/iteration", "higher_is_better": False,
            "solves_per_s": solves / wall, "iterations": n_iter,
            "history_max_change_eV": [h["max_change"] for h in out["history"]],
            "history_rel_change": [h["rel_change"] for h in out["history"]],
            "poisson_iters": [h["poisson_iters"] for h in out["history"]],
            "t_rel_err_max_on_converged_potential": float(rel.max()), "t_err_gate": 1e-6,
            "config": {"npx": npx, "npy": npy, "npz": npz, "M": 4 * npy * npz, "seeds": n_seeds,
                       "energies_per_iteration": n_e, "eps_r": 100.0, "gate_eV": 0.1, "mixing": 0.3,
                       "mu_l": mu_l, "mu_r": mu_r, "kT": KT,
                       "sample": "%d energies x %d seeds per iteration (config: 1024 x 8)" % (n_e, n_seeds)},
            "data": "synthetic"}
    print(json.dumps(line), flush=True)


def run_reference(args, rank, world):
    if rank != 0:
        return
    from oracle import negf_oracle as O
    from nonequilibriumgreensfunction_gb300 import hamiltonian as HB
    opt = O.SolveOptions(eta=ETA, sr_tol=SR_TOL, kT=KT, calc_spin=True)
    hams = {}
    times = []
    per_step = 1
    # warm-up steps exercise the same code on a 4-slice wire (a CPU path has nothing to
    # warm but its caches); timed steps solve full-size energy points
    hw, xw = HB.ti_wire(4, NPY, NPZ, zeeman=ZEEMAN, flux=FLUX, W=W, seed=0)
    for step in range(args.warmup):
        O.energy_sweep(hw, xw, float(energy_grid()[step % N_E]), MU, 0.6 / (N_E - 1), NPY, NPZ, opt)
    for step in range(args.steps):
        e, f1, f2, slots = step_requests(step, per_step, 0, 1)
        for s in set(int(v) for v in slots):
            if s not in hams:
                hams[s] = HB.ti_wire(NPX, NPY, NPZ, zeeman=ZEEMAN, flux=FLUX, W=W, seed=s)
        t0 = time.perf_counter()
        for i in range(per_step):
            h, x = hams[int(slots[i])]
            O.energy_sweep(h, x, float(e[i]), MU, 0.6 / (N_E - 1), NPY, NPZ, opt)
        times.append(time.perf_counter() - t0)
    total = sum(times)
    value = per_step * len(times) / total
    threads = os.cpu_count() or 1
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * total / len(times), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "c128", "data": "synthetic",
        "config": {"workload": WORKLOAD, "batch": per_step, "form": "cpu-oracle"},
        "cpu_baseline": {"value": value, "unit": "solves/s", "cores": threads, "kind": "port",
                         "sample": "%d energy point per step at full size (M=400, Npx=100), NumPy/OpenBLAS "
                                   "restatement of the reference algorithm on all host threads" % per_step},
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    global NPX, WORKLOAD
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--form", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--batch", type=int, default=256)
    ap.add_argument("--slices", type=int, default=0, help="mixed form: BF16 slices of the RGF products (0 = default)")
    ap.add_argument("--residual-slices", type=int, default=0, help="mixed form: slices of the Newton-Schulz residual")
    ap.add_argument("--sr-slices", type=int, default=0, help="mixed form: slices of the Sancho-Rubio products")
    ap.add_argument("--fp64-steps", type=int, default=1,
                    help="mixed form: timed FP64 steps on the same requests (T error and FP64 rate)")
    ap.add_argument("--fp64-batch", type=int, default=0,
                    help="mixed form: requests of each compared step solved in FP64 (a prefix of the "
                         "step; 0 = the whole step)")
    ap.add_argument("--e2e-steps", type=int, default=5,
                    help="steps of the end-to-end leg (each re-uploads the Hamiltonians); at most --steps")
    ap.add_argument("--npx", type=int, default=NPX,
                    help="slices of the wire; the benchmark workload is 100, shorter wires only for profiling")
    ap.add_argument("--workload", default="wire", choices=["wire", "scf", "serving"],
                    help="wire: the solves/s benchmark; scf: the self-consistent bias point (config 5 geometry); "
                         "serving: the serving leg alone")
    ap.add_argument("--serving-config", default="reduced", choices=["reduced", "c4"],
                    help="--workload serving: the bench's reduced mix or the serving configuration's wires")
    ap.add_argument("--serving-form", default="mixed", choices=["mixed", "fp64", "both"])
    ap.add_argument("--serving-energy-scale", type=float, default=1.0 / 16,
                    help="c4 mix: energies per request are log-uniform in [64, 1024] x this")
    ap.add_argument("--serving-fp64-energy-scale", type=float, default=1.0 / 64,
                    help="c4 mix, FP64 form: the same scale for the FP64 server")
    ap.add_argument("--serving-fp64-seconds", type=float, default=0.0,
                    help="--workload serving: Poisson seconds of the FP64 form (0 = --serving-seconds)")
    ap.add_argument("--serving-burst", type=int, default=24, help="requests of the closed capacity burst")
    ap.add_argument("--scf-energies", type=int, default=64, help="--workload scf: energies per iteration")
    ap.add_argument("--scf-seeds", type=int, default=2, help="--workload scf: disorder seeds per iteration")
    ap.add_argument("--kernel-case", default="none", choices=["none", "gemm_tc"],
                    help="profiling aid: run only one kernel case (gemm_tc: 16 complex 400^3 products at "
                         "--slices slices, twice) and exit")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--clocks-csv", default=None,
                    help="where the nvidia-smi samples of the timed region go (%%d = rank); "
                         "default: the temporary directory")
    ap.add_argument("--serving-seconds", type=float, default=30.0,
                    help="length of the Poisson-arrival serving run (0 = skip); rank 0 of a 1-GPU run only")
    args = ap.parse_args()

    if args.npx != NPX:
        NPX = args.npx
        WORKLOAD = "ti_wire_M400_Npx%d" % NPX
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if args.workload == "scf":
        run_scf_bench(args)
        return
    if args.workload == "serving":
        run_serving_bench(args)
        return
    if args.kernel_case == "gemm_tc":
        from nonequilibriumgreensfunction_gb300 import capi
        rng = np.random.default_rng(0)
        a = rng.standard_normal((16, 400, 400)) + 1j * rng.standard_normal((16, 400, 400))
        b = rng.standard_normal((16, 400, 400)) + 1j * rng.standard_normal((16, 400, 400))
        for _ in range(2):
            c = capi.zgemm(a, b, slices=args.slices or 5)
        print(json.dumps({"kernel_case": "gemm_tc", "slices": args.slices or 5,
                          "max_abs_err": float(np.abs(c - a @ b).max())}))
        return

    import torch
    import torch.distributed as dist
    from nonequilibriumgreensfunction_gb300 import Solver

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    if world > 1:
        dist.init_process_group("nccl", device_id=dev)

    hams = build_hamiltonians()
    m = 4 * NPY * NPZ
    solver = Solver(NPX, NPY, NPZ, n_hamiltonians=SEEDS, max_batch=args.batch, eta=ETA, sr_tol=SR_TOL,
                    calc_spin=True, precision=args.form, device=local_rank, mixed_slices=args.slices,
                    residual_slices=args.residual_slices, sr_slices=args.sr_slices)
    stream = torch.cuda.Stream(dev)          # a real stream handle, so events bracket the work
    torch.cuda.set_stream(stream)
    solver.set_stream(stream.cuda_stream)
    # pinned host copies of the inputs in the reference's memory layout (for e2e)
    pinned = []
    for h, x in hams:
        hf = torch.empty((NPX, m, m), dtype=torch.complex128, pin_memory=True).numpy()
        hf[...] = h.transpose(0, 2, 1)
        xf = np.asfortranarray(x)
        pinned.append((hf, xf))
    for k, (hf, xf) in enumerate(pinned):
        solver.set_hamiltonian_fortran(hf, xf, slot=k)

    nsites = NPX * NPY * NPZ
    rho_n = np.zeros((NPX, NPY, NPZ, SEEDS), order="F")
    rho_p = np.zeros_like(rho_n)
    spin = [np.zeros_like(rho_n) for _ in range(3)]

    def one_step(step):
        e, f1, f2, slots = step_requests(step, args.batch, rank, world)
        return solver.solve_batch(e, f1, f2, 0.6 / (N_E - 1), slots=slots, rho_n=rho_n, rho_p=rho_p, spin=spin)

    for s in range(args.warmup):
        r = one_step(s)
        assert (r["status"] == 0).all(), r["status"]
    sr_iters = int(np.max(r["sr_iters"]))
    timed_results = []

    clocks_path = (args.clocks_csv.replace("%d", str(rank))) if args.clocks_csv else os.path.join(
        tempfile.gettempdir(), "negf_bench_clocks_rank%d.csv" % rank)
    os.makedirs(os.path.dirname(os.path.abspath(clocks_path)), exist_ok=True)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    solver.profile(True)
    with ClockSampler(clocks_path) as clk:
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for s in range(args.steps):
            r = one_step(args.warmup + s)
            timed_results.append(r)
        ev1.record(stream)
        torch.cuda.synchronize()
    st = solver.stats()
    solver.profile(False)
    elapsed = ev0.elapsed_time(ev1) * 1e-3
    if world > 1:
        elapsed = max_over_ranks(elapsed, dist, dev)
        dist.barrier()
    solves = args.batch * args.steps * world
    value = solves / elapsed

    # e2e: through the public API with host buffers, upload + solve + readback each step
    e2e = None
    if not args.no_e2e:
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        n_e2e = max(1, min(args.e2e_steps, args.steps))
        ev2, ev3 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev2.record(stream)
        for s in range(n_e2e):
            for k, (hf, xf) in enumerate(pinned):
                solver.set_hamiltonian_fortran(hf, xf, slot=k)
            one_step(args.warmup + s)
        ev3.record(stream)
        torch.cuda.synchronize()
        el2 = ev2.elapsed_time(ev3) * 1e-3
        if world > 1:
            el2 = max_over_ranks(el2, dist, dev)
        h2d = sum(hf.nbytes + xf.nbytes for hf, xf in pinned) + args.batch * 40
        d2h = args.batch * 64 + 5 * nsites * SEEDS * 8
        e2e = {"value": args.batch * n_e2e * world / el2, "unit": "solves/s",
               "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h), "steps": n_e2e}

    # FP64 form on the same requests: its rate, and the T error of the mixed form
    fp64 = None
    if args.form == "mixed" and args.fp64_steps > 0:
        st_mixed = st
        solver.close()
        nfb = args.batch if args.fp64_batch <= 0 else max(SEEDS, min(args.fp64_batch, args.batch))
        ref = Solver(NPX, NPY, NPZ, n_hamiltonians=SEEDS, max_batch=nfb, eta=ETA, sr_tol=SR_TOL,
                     calc_spin=True, precision="fp64", device=local_rank)
        ref.set_stream(stream.cuda_stream)
        ref.profile(True)
        for k, (hf, xf) in enumerate(pinned):
            ref.set_hamiltonian_fortran(hf, xf, slot=k)
        n_fp = min(args.fp64_steps, args.steps)
        rn64 = np.zeros_like(rho_n)
        ev4, ev5 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        ev4.record(stream)
        outs = []
        for s in range(n_fp):
            e, f1, f2, slots = step_requests(args.warmup + s, args.batch, rank, world)
            outs.append(ref.solve_batch(e[:nfb], f1[:nfb], f2[:nfb], 0.6 / (N_E - 1), slots=slots[:nfb], rho_n=rn64))
        ev5.record(stream)
        torch.cuda.synchronize()
        el64 = ev4.elapsed_time(ev5) * 1e-3
        st64 = ref.stats()
        t_err = 0.0
        rho_err = 0.0
        worst = []
        for s_i, (a, b) in enumerate(zip(timed_results[:n_fp], outs)):
            rel = np.abs(a["T12"][:nfb] - b["T12"]) / np.maximum(np.abs(b["T12"]), 1e-3)
            t_err = max(t_err, float(np.max(rel)))
            for k in ("EDensity", "HDensity"):
                den = np.maximum(np.abs(b[k]), 1e-3 * np.abs(b[k]).max())
                rho_err = max(rho_err, float(np.max(np.abs(a[k][:nfb] - b[k]) / den)))
            e_s, _, _, sl_s = step_requests(args.warmup + s_i, args.batch, rank, world)
            for i in np.argsort(rel)[-3:]:
                worst.append((float(rel[i]), float(e_s[i]), int(sl_s[i]), float(b["T12"][i]), float(a["T12"][i])))
        worst = sorted(worst)[-3:]
        fp64_peak = fp64_zgemm_peak_tflops(torch, dev)
        gemm_tf = st64["gemm_flops"] / (st64["gemm_ms"] * 1e-3) / 1e12 if st64["gemm_ms"] > 0 else None
        fp64 = {"value": nfb * n_fp / el64, "unit": "solves/s", "steps": n_fp, "batch": nfb,
                "compared_solves": nfb * n_fp, "t_rel_err_max": t_err, "t_err_gate": 1e-6,
                "gate_ok": t_err <= 1e-6, "t_err_floor": "denominator max(|T_fp64|, 1e-3)",
                "density_rel_err_max": rho_err,
                "density_err_floor": "EDensity/HDensity, denominator max(|x|, 1e-3 max|x|)",
                "worst": [{"rel": w[0], "E": w[1], "seed": w[2], "T_fp64": w[3], "T_mixed": w[4]} for w in worst],
                "roofline": {"bound": "fp64", "kernel": "zgemm_kernel<double2> (FP64 complex GEMM, DFMA)",
                             "achieved": gemm_tf, "peak": fp64_peak, "unit": "TFLOP/s",
                             "frac": (gemm_tf / fp64_peak) if gemm_tf else None,
                             "peak_source": "cuBLAS ZGEMM 4096^3 complex128 measured live (of measured)",
                             "launches": st64["gemm_launches"], "gemm_s": st64["gemm_ms"] * 1e-3,
                             "gauss_jordan_panel_s": st64["panel_ms"] * 1e-3, "step_s": el64 / n_fp}}
        ref.close()
        solver = None
        st = st_mixed

    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return

    peaks = measured_peaks()
    if args.form == "fp64":
        fp64_peak = fp64_zgemm_peak_tflops(torch, dev)
        gemm_tf = st["gemm_flops"] / (st["gemm_ms"] * 1e-3) / 1e12 if st["gemm_ms"] > 0 else None
        roofline = {
            "bound": "tensor", "kernel": "zgemm_kernel (FP64 complex GEMM, DFMA)",
            "achieved": gemm_tf, "peak": fp64_peak, "unit": "TFLOP/s",
            "frac": (gemm_tf / fp64_peak) if gemm_tf else None, "traffic": None,
            "peak_source": "cuBLAS ZGEMM 4096^3 complex128 measured live (of measured)",
            "launches": st["gemm_launches"], "share_of_step": st["gemm_ms"] * 1e-3 / elapsed,
        }
    else:
        # tensor work actually issued: the slice-pair products, counted from the stats'
        # complex-equivalent flops; achieved = issued BF16 tensor flops / kernel time
        # achieved: the algorithmic work of the scope table's convention, 3 BF16 MMAs per
        # split real product, i.e. 3 x 8 m n k real flops per complex product the launches
        # compute; issued: every slice-pair MMA the kernel actually runs, S (S + 1) / 2 of
        # them per real product (the precision cost of the integer slicing)
        tc_issued = st.get("tc_flops") or None
        tc_tf = (3.0 * st["tc_complex_flops"] / (st["tc_ms"] * 1e-3) / 1e12) if st["tc_ms"] > 0 else None
        issued_tf = (tc_issued / (st["tc_ms"] * 1e-3) / 1e12) if (tc_issued and st["tc_ms"] > 0) else None
        bf16_peak = peaks.get("bf16_tflops")
        # DRAM traffic of one 5-slice RGF product launch (M = 400): an ncu capture of 16
        # products by the persistent kernel the autotuner picks at this shape
        # (dram__bytes_read.sum + dram__bytes_write.sum = 153.8 + 23.8 MB) scaled to the
        # step's 256 (the operands are per product, so the bytes grow in proportion), beside
        # the launch's algorithmic bytes: each product's A and B slice planes read once
        # (800 x 800 and 400 x 800 BF16 values per plane, 5 planes) and C written once
        traffic = (153.795840e6 + 23.783168e6) * (args.batch / 16)
        algo_bytes = args.batch * (800 * 800 * 5 * 2 + 400 * 800 * 5 * 2 + 400 * 400 * 16)
        roofline = {
            "bound": "tensor", "kernel": "zgemm_tc_persistent / zgemm_tc_kernel (tcgen05 sliced-BF16 complex GEMM)",
            "achieved": tc_tf, "peak": bf16_peak, "unit": "TFLOP/s",
            "frac": (tc_tf / bf16_peak) if (tc_tf and bf16_peak) else None, "traffic": traffic,
            "traffic_unit": "bytes per 5-slice product launch of the step's batch",
            "traffic_source": "ncu capture of 16 products, scaled in proportion to the batch",
            "traffic_algorithmic_bytes": algo_bytes,
            "peak_source": "MEASURED_PEAKS.json bf16_tflops (of measured, burst)",
            "achieved_convention": "3 BF16 MMAs (3 x 8 m n k flops) per complex product computed",
            "issued_tflops": issued_tf, "issued_frac": (issued_tf / bf16_peak) if (issued_tf and bf16_peak) else None,
            "launches": st["tc_launches"], "share_of_step": st["tc_ms"] * 1e-3 / elapsed,
            "complex_equiv_tflops": (st["tc_complex_flops"] / (st["tc_ms"] * 1e-3) / 1e12) if st["tc_ms"] > 0 else None,
            "fallbacks": st["fallbacks"], "ns_residual_max": st["ns_residual_max"],
            "ns_extra_steps": st["ns_extra_steps"], "ns_unconverged": st["ns_unconverged"],
            "ns_final_residual_max": st["ns_final_residual_max"],
        }
    roofline["breakdown_s_per_step"] = {
        k: st[k] * 1e-3 / args.steps for k in ("phase_sr_ms", "phase_rgf_ms", "phase_inv_ms", "phase_dens_ms",
                                               "tc_ms", "gemm_ms", "panel_ms", "f32_gemm_ms", "slice_ms")}
    flops_solve = algorithmic_flops_per_solve(m, NPX, sr_iters)
    flops_scope = scope_flops_per_solve(m, NPX, sr_iters)
    serving = None
    if args.serving_seconds > 0 and world == 1:
        if solver is not None:
            solver.close()
            solver = None
        serving = serving_bench(args.serving_seconds, local_rank)
    cpu = None
    if not args.no_cpu_baseline and world == 1:
        v, cores, sample = cpu_sample(1)
        cpu = {"value": v, "unit": "solves/s", "cores": cores, "kind": "port", "sample": sample}
    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * elapsed / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c128" if args.form == "fp64" else "bf16-sliced/c128",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "M": m, "npx": NPX, "seeds": SEEDS, "batch_per_gpu": args.batch,
                   "form": args.form, "eta": ETA, "sr_tol": SR_TOL, "l2": "inputs larger than L2 (1 GB H, "
                   "%.1f GB block store)" % (args.batch * NPX * m * m * 16 / 1e9), "parallelism": "energy-sharded x%d" % world},
        "roofline": roofline,
        "solve_tflops": flops_solve * value / 1e12 / world,
        "algorithmic_flops_per_solve": flops_solve,
        "algorithmic_model": "48 M^3 Npx + (88 n_SR + 24) M^3 / seeds + 32 M^3 (the work this solver "
                             "does: site-local HopX, decimation shared by the seeds of an energy)",
        "solve_tflops_scope_model": flops_scope * value / 1e12 / world,
        "scope_flops_per_solve": flops_scope,
        "sr_iters": sr_iters,
        "cpu_baseline": cpu,
        "fp64_form": fp64,
        "e2e": e2e,
        "serving": serving,
        "gpu_launches": st["launches"],
        "clocks": clk.summary(local_rank),
        "peaks_file": {k: peaks.get(k) for k in ("hbm_gbs", "bf16_tflops", "bf16_tflops_sustained")},
    }
    print(json.dumps(line), flush=True)
    if solver is not None:
        solver.close()
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
