"""Generate the golden vectors in tests/golden/*.npz from the CPU oracle.

The reference publishes no test vectors and cannot be built here (Fortran + MKL + MPI,
no Fortran compiler), so the golden vectors are the oracle's output on fixed, seeded
inputs; tests/test_oracle.py pins the oracle itself against a dense inverse and physics
invariants.  Each fixture stores its inputs' parameters and a SHA-256 of the Hamiltonian
so that a consumer that rebuilds the input can prove it is the same one.

    python tests/golden/make_golden.py            # all cases
    python tests/golden/make_golden.py c1         # one case
"""
from __future__ import annotations

import hashlib
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from oracle import negf_oracle as O  # noqa: E402
from nonequilibriumgreensfunction_gb300 import hamiltonian as HB  # noqa: E402


def h_digest(htotd, hopx):
    m = hashlib.sha256()
    m.update(np.ascontiguousarray(htotd).tobytes())
    m.update(np.ascontiguousarray(hopx).tobytes())
    return m.hexdigest()


# -- case definitions (also imported by the tests) -------------------------------------
CASES = {
    # The reference's default run (Source/Read_In_Allocate.F90:29-50): 4x3x3 wire, its own
    # Dirac basis, mu = (-0.1, 0), T = 0 steps, eta = 1e-4, Sancho-Rubio tolerance 1e-8.
    "ref_debug": dict(npx=4, npy=3, npz=3, basis="reference", zeeman=0.0, flux=0.0, W=0.0, seed=0,
                      eta=1e-4, sr_tol=1e-8, kT=0.0, mu_lead=(0.1, 0.0),
                      energies=[-1e-10, 0.02, 0.05, 0.08, 0.1, 0.35, 0.6], dE=0.1 / 599, calc_spin=True),
    # BASELINE config 1: M = 64, Npx = 20, W = 0.1 eV, eta = 1e-5, SR tol 1e-10,
    # kT = 0.025, muL - muR = 0.01 eV, 64 energies in [-0.3, 0.3].
    "c1": dict(npx=20, npy=4, npz=4, basis="tau_sigma", zeeman=0.0, flux=0.0, W=0.1, seed=0,
               eta=1e-5, sr_tol=1e-10, kT=0.025, mu_lead=(0.005, -0.005),
               energies=list(np.linspace(-0.3, 0.3, 64)), dE=0.6 / 63, calc_spin=True),
    # flux + Zeeman + disorder on a small wire (the config-2 Hamiltonian terms)
    "flux_zeeman": dict(npx=6, npy=3, npz=3, basis="tau_sigma", zeeman=0.01, flux=0.5, W=0.1, seed=3,
                        eta=1e-5, sr_tol=1e-10, kT=0.025, mu_lead=(0.005, -0.005),
                        energies=[-0.25, -0.05, 0.0, 0.12, 0.29], dE=0.6 / 511, calc_spin=True),
    # BASELINE config 2 geometry (M = 400, Npx = 100), two energies of seed 1
    "c2_sub": dict(npx=100, npy=10, npz=10, basis="tau_sigma", zeeman=0.01, flux=0.5, W=0.1, seed=1,
                   eta=1e-5, sr_tol=1e-10, kT=0.025, mu_lead=(0.005, -0.005),
                   energies=[-0.1, 0.0037], dE=0.6 / 511, calc_spin=True),
    # BASELINE config 5 cross-section (Npy = Npz = 12, M = 576) on a short wire: products
    # with K' = 2M = 1152 > 800, where the tensor-core GEMM splits its accumulators along K
    "m576": dict(npx=8, npy=12, npz=12, basis="tau_sigma", zeeman=0.01, flux=0.5, W=0.1, seed=5,
                 eta=1e-5, sr_tol=1e-10, kT=0.025, mu_lead=(0.025, -0.025),
                 energies=[-0.262, 0.0021, 0.147], dE=0.6 / 1023, calc_spin=True),
    # the largest cross-section of BASELINE config 4 (Npy = Npz = 14, M = 784, K' = 1568),
    # the strongest disorder and flux of that mix
    "m784": dict(npx=6, npy=14, npz=14, basis="tau_sigma", zeeman=0.01, flux=1.0, W=0.2, seed=7,
                 eta=1e-5, sr_tol=1e-10, kT=0.025, mu_lead=(0.005, -0.005),
                 energies=[-0.213, 0.0513], dE=0.6 / 1023, calc_spin=True),
}


def build_inputs(case):
    c = CASES[case]
    htotd, hopx = HB.ti_wire(c["npx"], c["npy"], c["npz"], zeeman=c["zeeman"], flux=c["flux"], W=c["W"],
                             seed=c["seed"], basis=c["basis"])
    return htotd, hopx


def run_case(case):
    c = CASES[case]
    htotd, hopx = build_inputs(case)
    opt = O.SolveOptions(eta=c["eta"], sr_tol=c["sr_tol"], kT=c["kT"], calc_spin=c["calc_spin"])
    keys = ["T12", "Modec1", "Modec2", "EDensity", "HDensity"]
    out = {k: [] for k in keys}
    out.update(DOSc=[], RhoN=[], RhoP=[], SigExp=[], f1=[], f2=[], sr_iters=[])
    t0 = time.time()
    for e in c["energies"]:
        r = O.energy_sweep(htotd, hopx, float(e), c["mu_lead"], c["dE"], c["npy"], c["npz"], opt)
        for k in keys:
            out[k].append(r[k])
        out["DOSc"].append(r["dosc"])
        out["RhoN"].append(r["RhoN"])
        out["RhoP"].append(r["RhoP"])
        out["SigExp"].append(r["SigExp"])
        out["f1"].append(r["f1"])
        out["f2"].append(r["f2"])
        out["sr_iters"].append(r["sr_iters"])
    arrs = {k: np.asarray(v) for k, v in out.items()}
    # site arrays: the energy sum (what the reference accumulates, Calculate_Gnp.F90:123-124)
    # plus per-energy values on a subset of at most 8 energies
    n_e = len(c["energies"])
    site_idx = np.unique(np.linspace(0, n_e - 1, min(n_e, 8)).round().astype(int))
    for k in ("RhoN", "RhoP", "SigExp"):
        arrs[k + "_sum"] = arrs[k].sum(axis=0)
        arrs[k] = arrs[k][site_idx]
    arrs["site_idx"] = site_idx
    arrs["energies"] = np.asarray(c["energies"], dtype=np.float64)
    arrs["h_sha256"] = np.array(h_digest(htotd, hopx))
    arrs["params"] = np.array(json.dumps({k: (list(v) if isinstance(v, tuple) else v)
                                          for k, v in c.items() if k != "energies"}))
    path = os.path.join(HERE, case + ".npz")
    np.savez_compressed(path, **arrs)
    print("%s: %d energies in %.1f s -> %s" % (case, len(c["energies"]), time.time() - t0, path))


if __name__ == "__main__":
    for name in (sys.argv[1:] or list(CASES)):
        run_case(name)
