"""Mixed form (tcgen05 sliced-BF16 products, FP32 Gauss-Jordan + Newton-Schulz inverses
with FP64-class residuals): accuracy against the FP64 oracle.

Stated tolerance of the mixed form: transmission and site density within 1e-6 relative
of the FP64 result (T floored at 1e-3 channels, density at 1e-3 of its maximum)."""
import importlib.util
import os

import numpy as np
import pytest

from conftest import GOLDEN
from oracle import negf_oracle as O
from nonequilibriumgreensfunction_gb300 import Solver
from nonequilibriumgreensfunction_gb300 import hamiltonian as HB

pytestmark = pytest.mark.gpu

MIXED_RTOL = 1e-6


def rel_err(a, b, floor):
    a, b = np.asarray(a), np.asarray(b)
    return float((np.abs(a - b) / np.maximum(np.abs(b), floor)).max())


@pytest.mark.parametrize("slices", [4, 5])
def test_mixed_matches_oracle_small(need_gpu, slices):
    npx, npy, npz = 10, 3, 3
    htotd, hopx = HB.ti_wire(npx, npy, npz, W=0.1, seed=2, flux=0.5, zeeman=0.01)
    opt = O.SolveOptions(eta=1e-5, sr_tol=1e-10, kT=0.025, calc_spin=True)
    mu = (0.005, -0.005)
    es = np.array([-0.27, -0.1, 0.0013, 0.08, 0.22])
    f1 = [O.fermi(e, mu[0], opt.kT) for e in es]
    f2 = [O.fermi(e, mu[1], opt.kT) for e in es]
    with Solver(npx, npy, npz, eta=opt.eta, sr_tol=opt.sr_tol, calc_spin=True, max_batch=5, precision="mixed",
                mixed_slices=slices) as s:
        s.set_hamiltonian(htotd, hopx)
        rn = s.new_site_array(1)
        r = s.solve_batch(es, f1, f2, 1e-3, rho_n=rn)
    assert (r["status"] == 0).all()
    want = np.zeros((npx, npy, npz))
    for i, e in enumerate(es):
        ref = O.energy_sweep(htotd, hopx, float(e), mu, 1e-3, npy, npz, opt)
        assert rel_err(r["T12"][i], ref["T12"], 1e-3) <= MIXED_RTOL, (e, r["T12"][i], ref["T12"])
        assert rel_err(r["Modec1"][i], ref["Modec1"], 1e-3) <= MIXED_RTOL
        assert rel_err(r["DOSc1"][i], ref["dosc"][0], 1e-3) <= MIXED_RTOL
        want += ref["RhoN"]
    assert rel_err(rn[..., 0], want, 1e-3 * np.abs(want).max()) <= MIXED_RTOL


def test_mixed_full_size_matches_golden(need_gpu):
    """M = 400, Npx = 100: the mixed form against the FP64 golden vectors."""
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    c = mg.CASES["c2_sub"]
    g = np.load(os.path.join(GOLDEN, "c2_sub.npz"))
    htotd, hopx = mg.build_inputs("c2_sub")
    with Solver(c["npx"], c["npy"], c["npz"], eta=c["eta"], sr_tol=c["sr_tol"], calc_spin=True, max_batch=2,
                precision="mixed") as s:
        s.set_hamiltonian(htotd, hopx)
        rn = s.new_site_array(1)
        r = s.solve_batch(np.asarray(c["energies"]), g["f1"], g["f2"], c["dE"], rho_n=rn)
        st = s.stats()
    assert (r["status"] == 0).all()
    for k in ("T12", "Modec1", "Modec2"):
        assert rel_err(r[k], g[k], 1e-3) <= MIXED_RTOL, (k, r[k], g[k])
    assert rel_err(rn[..., 0], g["RhoN_sum"], 1e-3 * np.abs(g["RhoN_sum"]).max()) <= MIXED_RTOL
    assert st["tc_launches"] > 0
