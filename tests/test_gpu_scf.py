"""Self-consistent bias point on the GPU against the oracle: the device Poisson solver
(conjugate gradients) against the restated SIP / a direct solve, and the whole
Poisson <-> NEGF loop against the oracle's loop (FP64 at 1e-9; the mixed form against the
FP64 loop at 1e-6)."""
import numpy as np
import pytest

from oracle import negf_oracle as O
from oracle import poisson_oracle as P
from nonequilibriumgreensfunction_gb300 import Solver, capi, scf
from nonequilibriumgreensfunction_gb300 import hamiltonian as HB

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("shape,n", [((60, 12, 12), 1), ((9, 3, 4), 3), ((200, 14, 14), 1)])
def test_device_poisson_matches_direct_solve(need_gpu, shape, n):
    rng = np.random.default_rng(n)
    rho = rng.uniform(-0.02, 0.02, shape + (n,))
    bc = (0.025, -0.025, 0.1)
    kap = P.kappa(100.0)
    u, iters = scf.poisson_solve(rho, bc, kap, tol=1e-13)
    assert iters > 0
    for g in range(n):
        want = P.direct_solve(P.poisson_rhs(rho[..., g], kap, bc))
        assert np.abs(u[..., g] - want).max() <= 1e-10 * np.abs(want).max()


def test_device_poisson_reports_non_convergence(need_gpu):
    rho = np.random.default_rng(0).uniform(-0.02, 0.02, (30, 6, 6))
    with pytest.raises(capi.NegfError) as ei:
        scf.poisson_solve(rho, (0.0, 0.0, 0.1), 0.18, tol=1e-14, max_iter=3)
    assert ei.value.code == capi.NEGF_EREFINE


def _small_case():
    npx, npy, npz = 8, 3, 3
    models = [HB.wire_model(W=0.1, seed=s, zeeman=0.01, flux=0.2) for s in (1, 2)]
    energies = np.linspace(-0.3, 0.3, 12)
    return npx, npy, npz, models, energies, energies[1] - energies[0]


def test_scf_loop_matches_oracle_fp64(need_gpu):
    npx, npy, npz, models, energies, de = _small_case()
    opt = O.SolveOptions(eta=1e-5, sr_tol=1e-10, kT=0.025)
    us, hist, t_last = P.scf_loop(npx, npy, npz, models, energies, de, 0.025, -0.025, opt, n_iter=3)
    with Solver(npx, npy, npz, n_hamiltonians=2, max_batch=8, eta=1e-5, sr_tol=1e-10) as s:
        out = scf.run_scf(s, models, energies, de, 0.025, -0.025, 0.025, n_iter=3)
    # compare the charge-induced part of U (U minus the charge-free Laplace solution)
    u0, _ = scf.poisson_solve(np.zeros((npx, npy, npz)), (0.025, -0.025, 0.1), P.kappa(100.0), tol=1e-13)
    scale = max(np.abs(u - u0).max() for u in us)
    assert scale > 1e-6
    for k in range(2):
        assert np.abs(out["U"][..., k] - us[k]).max() <= 1e-9 * scale
        t = out["last"]["T12"][k * energies.size:(k + 1) * energies.size]
        assert np.abs(t - t_last[k]).max() <= 1e-9 * max(np.abs(t_last[k]).max(), 1.0)
    for a, b in zip(out["history"], hist):
        assert abs(a["max_change"] - b) <= 1e-6 * b + 1e-12


def test_scf_mixed_form_matches_fp64(need_gpu):
    npx, npy, npz = 20, 6, 6
    models = [HB.wire_model(W=0.1, seed=s, zeeman=0.01) for s in (3, 4)]
    energies = np.linspace(-0.3, 0.3, 16)
    de = energies[1] - energies[0]
    res = {}
    for prec in ("fp64", "mixed"):
        with Solver(npx, npy, npz, n_hamiltonians=2, max_batch=32, eta=1e-5, sr_tol=1e-10, precision=prec) as s:
            res[prec] = scf.run_scf(s, models, energies, de, 0.025, -0.025, 0.025, n_iter=4)
    a, b = res["fp64"], res["mixed"]
    u0, _ = scf.poisson_solve(np.zeros((npx, npy, npz)), (0.025, -0.025, 0.1), P.kappa(100.0), tol=1e-13)
    charge_part = np.abs(a["U"] - u0[..., None]).max()
    assert np.abs(a["U"] - b["U"]).max() <= 1e-6 * charge_part
    ta, tb = a["last"]["T12"], b["last"]["T12"]
    assert (np.abs(ta - tb) / np.maximum(np.abs(ta), 1e-3)).max() <= 1e-6
    # the loop contracts: the Poisson update shrinks from the first to the last iteration
    assert a["history"][-1]["max_change"] < a["history"][0]["max_change"]
