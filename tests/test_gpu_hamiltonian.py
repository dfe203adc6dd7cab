"""negf_build_hamiltonian: Htotd generated in HBM (Build_Hamiltonian.F90 on the device)
must be the host twin's array element for element.  The solve is deterministic, so a
device-built slot and an uploaded copy of build_from_model give bitwise equal results."""
import numpy as np
import pytest

from oracle import negf_oracle as O
from nonequilibriumgreensfunction_gb300 import Solver, capi
from nonequilibriumgreensfunction_gb300 import hamiltonian as HB

pytestmark = pytest.mark.gpu


def _solve(s, slots, energies):
    n = len(energies)
    rho = np.zeros((s.npx, s.npy, s.npz, s.n_hamiltonians), order="F")
    sp = [np.zeros_like(rho) for _ in range(3)]
    out = s.solve_batch(energies, 0.9, 0.2, 0.01, slots=slots, rho_n=rho, spin=sp)
    return out, rho, sp


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_device_build_equals_uploaded_host_twin(need_gpu, precision):
    npx, npy, npz = 7, 3, 4
    models = [HB.wire_model(W=0.2, seed=s, flux=0.5, zeeman=0.01) for s in (7, 8)]
    energies = np.array([-0.21, 0.03, 0.19, 0.03])
    slots = np.array([0, 1, 1, 0])
    kw = dict(n_hamiltonians=2, max_batch=4, eta=1e-5, sr_tol=1e-10, calc_spin=True, precision=precision)
    with Solver(npx, npy, npz, **kw) as up, Solver(npx, npy, npz, **kw) as dev:
        for slot, m in enumerate(models):
            h, x = HB.build_from_model(npx, npy, npz, m)
            up.set_hamiltonian(h, x, slot=slot)
            dev.build_hamiltonian(m, slot=slot)
        a, ra, sa = _solve(up, slots, energies)
        b, rb, sb = _solve(dev, slots, energies)
    for k in ("T12", "EDensity", "HDensity", "Modec1", "Modec2", "DOSc1", "DOSc2"):
        assert np.array_equal(a[k], b[k]), k
    assert np.array_equal(ra, rb)
    for x, y in zip(sa, sb):
        assert np.array_equal(x, y)


def test_device_build_matches_oracle_and_explicit_potential(need_gpu):
    npx, npy, npz = 5, 2, 3
    v = np.random.default_rng(4).uniform(-0.05, 0.05, (npx, npy, npz))
    m = HB.wire_model(flux=0.3, V=v)
    h, x = HB.build_from_model(npx, npy, npz, m)
    opt = O.SolveOptions(eta=1e-5, sr_tol=1e-10)
    with Solver(npx, npy, npz, eta=1e-5, sr_tol=1e-10) as s:
        s.build_hamiltonian(m)
        for e in (-0.15, 0.07):
            ref = O.energy_sweep(h, x, e, (0.5, -0.5), 0.01, npy, npz, opt)
            got = s.energy_sweep(e, 1.0, 0.0, 0.01)
            assert abs(got["T12"] - ref["T12"]) <= 1e-9 * max(abs(ref["T12"]), 1e-6)


def test_full_size_device_build(need_gpu):
    """M = 400, Npx = 100: the 256 MB slot is generated on the device; results equal the
    uploaded host twin's."""
    npx, npy, npz = 100, 10, 10
    m = HB.wire_model(W=0.1, seed=0, flux=0.5, zeeman=0.01)
    h, x = HB.build_from_model(npx, npy, npz, m)
    kw = dict(max_batch=1, eta=1e-5, sr_tol=1e-10, precision="mixed")
    with Solver(npx, npy, npz, **kw) as up, Solver(npx, npy, npz, **kw) as dev:
        up.set_hamiltonian(h, x)
        dev.build_hamiltonian(m)
        a = up.solve_batch([-0.2], 1.0, 0.0, 0.01)
        b = dev.solve_batch([-0.2], 1.0, 0.0, 0.01)
    assert np.array_equal(a["T12"], b["T12"])


def test_build_rejects_bad_arguments(need_gpu):
    with Solver(4, 2, 2) as s:
        with pytest.raises(capi.NegfError):
            s.build_hamiltonian(HB.wire_model(), slot=3)
    with Solver(4, 2, 2, norb=2) as s:
        with pytest.raises(capi.NegfError):
            s.build_hamiltonian(HB.wire_model())
