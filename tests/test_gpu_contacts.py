"""Contacts with a closed-form self-energy (Source/Contact_Self_Energy.F90:19-67) and the
superconducting (BdG) branch of Calculate_Observables (:60-81) on the GPU, through the C ABI,
against the oracle.  FP64 form: 1e-9 relative, with quantities that can cancel to ~0 compared
against 1e-3 of their largest value (as in test_gpu_parity.py); bond currents against their
largest value at 1e-6 (REAL(4) terms)."""
import numpy as np
import pytest

from oracle import negf_oracle as O
from nonequilibriumgreensfunction_gb300 import Solver
from nonequilibriumgreensfunction_gb300 import hamiltonian as HB

pytestmark = pytest.mark.gpu
RTOL = 1e-9
SCALARS = ("T12", "EDensity", "HDensity", "Modec1", "Modec2")


def assert_close(a, b, what, rtol=RTOL):
    a = np.asarray(a, dtype=float)
    b = np.asarray(b, dtype=float)
    den = np.maximum(np.abs(b), max(1e-3 * np.abs(b).max(), 1e-300))
    err = (np.abs(a - b) / den).max()
    assert err <= rtol, "%s: max rel err %.3e > %.1e" % (what, err, rtol)


def assert_currents_close(got, want, what, rtol=1e-6):
    err = np.abs(np.asarray(got) - want).max() / max(np.abs(want).max(), 1e-300)
    assert err <= rtol, "%s: max err %.3e of max|J| > %.1e" % (what, err, rtol)


def _zeros(npx, npy, npz, n=None):
    return np.zeros((npx, npy, npz) if n is None else (npx, npy, npz, n), order="F")


def _bdg_wire(npx, npy, npz, seed=1):
    h, x = HB.ti_wire(npx, npy, npz, W=0.1, seed=seed)
    h = h - 0.12 * np.eye(h.shape[1])[None]            # Fermi level inside the surface band
    return HB.bdg(h, x, npy, npz)


def _check_per_energy(s, h, x, energies, opt, mu, de, npy, npz, currents):
    npx = h.shape[0]
    for e in energies:
        ref = O.energy_sweep(h, x, float(e), mu, de, npy, npz, opt, calc_currents=currents)
        rn, rp = _zeros(npx, npy, npz), _zeros(npx, npy, npz)
        sp = [_zeros(npx, npy, npz) for _ in range(3)]
        j = [_zeros(npx, npy, npz) for _ in range(3)] if currents else None
        cc = np.zeros(2)
        cse = s.contact_self_energy(float(e), want_matrices=False)
        s.get_retarded_greens()
        s.calculate_gnp(ref["f1"], ref["f2"], de, rn, rp)
        obs = s.calculate_observables(de, ref["f1"], ref["f2"], cc, sp)
        if currents:
            s.calculate_currents(j)
        for k in SCALARS:
            assert_close(obs[k], ref[k], "%s(E=%g)" % (k, e))
        assert_close(cse["dosc"], ref["dosc"], "dosc(E=%g)" % e)
        assert_close(cc, ref["ContactCurrent"], "ContactCurrent(E=%g)" % e)
        assert_close(rn, ref["RhoN"], "RhoN(E=%g)" % e)
        assert_close(rp, ref["RhoP"], "RhoP(E=%g)" % e)
        if opt.calc_spin:
            scale = max(np.abs(ref["RhoN"]).max(), np.abs(ref["RhoP"]).max())
            for i in range(3):
                assert np.abs(sp[i] - ref["SigExp"][i]).max() <= RTOL * scale, ("spin", i, e)
        if currents:
            for i, k in enumerate(("Jx", "Jy", "Jz")):
                assert_currents_close(j[i], ref[k], "%s(E=%g)" % (k, e))


@pytest.mark.parametrize("contact_type", [1, 2])
def test_phenomenological_contacts_match_oracle(need_gpu, contact_type):
    npx, npy, npz = 5, 3, 2
    h, x = HB.ti_wire(npx, npy, npz, W=0.2, seed=3, flux=0.3, zeeman=0.01)
    opt = O.SolveOptions(eta=1e-4, kT=0.025, calc_spin=True, contact_type=contact_type, tunneling_rate=0.6)
    mu, de = (0.005, -0.005), 0.01
    energies = np.array([-0.2, 0.01, 0.15])
    kw = dict(eta=1e-4, calc_spin=True, contact_type=contact_type, tunneling_rate=0.6)
    with Solver(npx, npy, npz, **kw) as s:
        s.set_hamiltonian(h, x)
        _check_per_energy(s, h, x, energies, opt, mu, de, npy, npz, currents=False)
    refs = [O.energy_sweep(h, x, float(e), mu, de, npy, npz, opt) for e in energies]
    rn = _zeros(npx, npy, npz, 1)
    with Solver(npx, npy, npz, max_batch=2, **kw) as s:
        s.set_hamiltonian(h, x)
        out = s.solve_batch(energies, [r["f1"] for r in refs], [r["f2"] for r in refs], de, rho_n=rn)
    assert (out["status"] == 0).all() and (out["sr_iters"] == 0).all()
    for k in SCALARS:
        assert_close(out[k], [r[k] for r in refs], k)
    assert_close(out["DOSc1"], [r["dosc"][0] for r in refs], "DOSc1")
    assert_close(rn[..., 0], sum(r["RhoN"] for r in refs), "RhoN")


def test_superconducting_contacts_match_oracle(need_gpu):
    """BdG wire (norb = 8) between superconducting contacts with phase difference 0.8:
    the supercurrent transmission, the electron-only densities, spin and bond currents,
    per energy and batched over two slots."""
    npx, npy, npz = 5, 2, 2
    opt = O.SolveOptions(eta=1e-4, norb=8, contact_type=3, chi_lr=0.8, calc_spin=True)
    mu, de = (0.0, 0.0), 2.2e-3 / 6
    energies = np.linspace(-1.1e-3, 1.1e-3, 7)
    hs = [_bdg_wire(npx, npy, npz, seed=s) for s in (1, 2)]
    kw = dict(norb=8, eta=1e-4, contact_type=3, chi_lr=0.8, delta_sc=(1e-3, 1e-3), calc_spin=True,
              calc_currents=True)
    with Solver(npx, npy, npz, **kw) as s:
        s.set_hamiltonian(*hs[0])
        _check_per_energy(s, hs[0][0], hs[0][1], energies[::2], opt, mu, de, npy, npz, currents=True)
    refs = [[O.energy_sweep(h, x, float(e), mu, de, npy, npz, opt, calc_currents=True) for e in energies]
            for h, x in hs]
    n = energies.size
    e_all = np.tile(energies, 2)
    f_all = np.array([r["f1"] for rs in refs for r in rs])
    slots = np.repeat([0, 1], n)
    rn = _zeros(npx, npy, npz, 2)
    j = [_zeros(npx, npy, npz, 2) for _ in range(3)]
    with Solver(npx, npy, npz, n_hamiltonians=2, max_batch=4, **kw) as s:
        for slot, (h, x) in enumerate(hs):
            s.set_hamiltonian(h, x, slot=slot)
        out = s.solve_batch(e_all, f_all, f_all, de, slots=slots, rho_n=rn, currents=j)
    assert (out["status"] == 0).all()
    for k in SCALARS:
        assert_close(out[k], [r[k] for rs in refs for r in rs], k)
    for slot in range(2):
        assert_close(rn[..., slot], sum(r["RhoN"] for r in refs[slot]), "RhoN slot %d" % slot)
        for i, k in enumerate(("Jx", "Jy", "Jz")):
            assert_currents_close(j[i][..., slot], sum(r[k] for r in refs[slot]), "%s slot %d" % (k, slot))


def test_superconducting_contacts_mixed_form(need_gpu):
    """Tensor-core form on a larger BdG wire (M = 72): the supercurrent transmission within
    1e-6 of its largest value over the window."""
    npx, npy, npz = 12, 3, 3
    h, x = _bdg_wire(npx, npy, npz, seed=4)
    opt = O.SolveOptions(eta=1e-4, norb=8, contact_type=3, chi_lr=0.8)
    energies = np.linspace(-1.1e-3, 1.1e-3, 6)
    refs = [O.energy_sweep(h, x, float(e), (0.0, 0.0), 1e-4, npy, npz, opt) for e in energies]
    with Solver(npx, npy, npz, norb=8, max_batch=6, eta=1e-4, contact_type=3, chi_lr=0.8, precision="mixed") as s:
        s.set_hamiltonian(h, x)
        out = s.solve_batch(energies, [r["f1"] for r in refs], [r["f2"] for r in refs], 1e-4)
    assert (out["status"] == 0).all()
    t_ref = np.array([r["T12"] for r in refs])
    assert np.abs(out["T12"] - t_ref).max() <= 1e-6 * np.abs(t_ref).max()
