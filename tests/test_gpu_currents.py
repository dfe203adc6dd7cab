"""Bond currents Jx/Jy/Jz (Source/Calculate_Observables.F90:110-169) on the GPU, through
the C ABI, against the oracle.

The reference forms each orbital-pair term in REAL(4) (dumVar, :7) and adds it, weighted by
dE/(2 pi), into REAL(8) arrays.  Both sides round each term to float32 the same way, so the
arrays agree far inside the float32 resolution; the tolerance is 1e-6 of the array's largest
|J| (natural scale: a bond with no current is compared against the flowing ones)."""
import numpy as np
import pytest

from oracle import negf_oracle as O
from nonequilibriumgreensfunction_gb300 import Solver, capi
from nonequilibriumgreensfunction_gb300 import hamiltonian as HB

pytestmark = pytest.mark.gpu
J_RTOL = 1e-6
KEYS = ("Jx", "Jy", "Jz")


def assert_currents_close(got, want, what, rtol=J_RTOL):
    scale = max(np.abs(want).max(), 1e-300)
    err = np.abs(np.asarray(got) - want).max() / scale
    assert err <= rtol, "%s: max err %.3e of max|J| > %.1e" % (what, err, rtol)


def _site(npx, npy, npz, n=None):
    shape = (npx, npy, npz) if n is None else (npx, npy, npz, n)
    return np.zeros(shape, order="F")


def test_per_energy_currents_match_oracle(need_gpu):
    npx, npy, npz = 5, 3, 2
    htotd, hopx = HB.ti_wire(npx, npy, npz, W=0.1, seed=3, flux=0.3, zeeman=0.01)
    opt = O.SolveOptions(eta=1e-5, sr_tol=1e-10, kT=0.025)
    mu = (0.005, -0.005)
    de = 0.6 / 63
    with Solver(npx, npy, npz, eta=1e-5, sr_tol=1e-10, calc_currents=True) as s:
        s.set_hamiltonian(htotd, hopx)
        for e in (-0.2, 0.004, 0.13):
            ref = O.energy_sweep(htotd, hopx, e, mu, de, npy, npz, opt, calc_currents=True)
            j = [_site(npx, npy, npz) for _ in range(3)]
            s.energy_sweep(e, ref["f1"], ref["f2"], de, currents=j)
            for k, got in zip(KEYS, j):
                assert_currents_close(got, ref[k], "%s(E=%g)" % (k, e))


def test_batch_currents_match_oracle_per_slot(need_gpu):
    """Two disorder seeds, energies chunked over several device batches; the J arrays of
    each slot are the sums over that slot's energies, as the MPI reduction gives them."""
    npx, npy, npz = 6, 2, 3
    hs = [HB.ti_wire(npx, npy, npz, W=0.2, seed=s, flux=0.5, zeeman=0.01) for s in (0, 1)]
    opt = O.SolveOptions(eta=1e-5, sr_tol=1e-10, kT=0.025)
    mu = (0.005, -0.005)
    energies = np.linspace(-0.25, 0.25, 5)
    de = energies[1] - energies[0]
    want = [[np.zeros((npx, npy, npz)) for _ in KEYS] for _ in hs]
    reqs = []
    for slot, (h, x) in enumerate(hs):
        for e in energies:
            ref = O.energy_sweep(h, x, float(e), mu, de, npy, npz, opt, calc_currents=True)
            for i, k in enumerate(KEYS):
                want[slot][i] += ref[k]
            reqs.append((e, ref["f1"], ref["f2"], slot))
    e, f1, f2, slots = (np.array(v) for v in zip(*reqs))
    j = [_site(npx, npy, npz, 2) for _ in KEYS]
    rho = _site(npx, npy, npz, 2)
    with Solver(npx, npy, npz, n_hamiltonians=2, max_batch=4, eta=1e-5, sr_tol=1e-10, calc_currents=True) as s:
        for slot, (h, x) in enumerate(hs):
            s.set_hamiltonian(h, x, slot=slot)
        out = s.solve_batch(e, f1, f2, de, slots=slots, rho_n=rho, currents=j)
    assert (out["status"] == 0).all()
    for slot in range(2):
        for i, k in enumerate(KEYS):
            assert_currents_close(j[i][..., slot], want[slot][i], "%s slot %d" % (k, slot))


def test_mixed_form_currents(need_gpu):
    """Tensor-core form: J within 1e-6 of the largest current, like the densities."""
    npx, npy, npz = 8, 4, 4
    htotd, hopx = HB.ti_wire(npx, npy, npz, W=0.1, seed=2, flux=0.5, zeeman=0.01)
    opt = O.SolveOptions(eta=1e-5, sr_tol=1e-10, kT=0.025)
    mu = (0.005, -0.005)
    energies = np.array([-0.21, 0.0, 0.17])
    de = 0.01
    want = [np.zeros((npx, npy, npz)) for _ in KEYS]
    f1s, f2s = [], []
    for e in energies:
        ref = O.energy_sweep(htotd, hopx, float(e), mu, de, npy, npz, opt, calc_currents=True)
        for i, k in enumerate(KEYS):
            want[i] += ref[k]
        f1s.append(ref["f1"])
        f2s.append(ref["f2"])
    j = [_site(npx, npy, npz, 1) for _ in KEYS]
    with Solver(npx, npy, npz, max_batch=3, eta=1e-5, sr_tol=1e-10, precision="mixed", calc_currents=True) as s:
        s.set_hamiltonian(htotd, hopx)
        s.solve_batch(energies, f1s, f2s, de, currents=j)
    for i, k in enumerate(KEYS):
        assert_currents_close(j[i][..., 0], want[i], k)


def test_full_size_currents_conserved(need_gpu):
    """M = 400, Npx = 100 wire (flux 0.5, Zeeman 0.01, W = 0.1): the current through every
    cross-section is the same, and equals 2 T12 (f1 - f2) q^2/h at each energy."""
    npx, npy, npz = 100, 10, 10
    htotd, hopx = HB.ti_wire(npx, npy, npz, W=0.1, seed=0, flux=0.5, zeeman=0.01)
    energies = np.array([-0.2, 0.15])
    unit = O.Q_E ** 2 / O.HBAR / (2.0 * O.PI)
    with Solver(npx, npy, npz, max_batch=1, eta=1e-7, sr_tol=1e-10, precision="mixed", calc_currents=True) as s:
        s.set_hamiltonian(htotd, hopx)
        for e in energies:
            j = [_site(npx, npy, npz, 1) for _ in KEYS]
            out = s.solve_batch([e], 1.0, 0.0, 1.0, currents=j)
            through = j[0][:-1, :, :, 0].sum(axis=(1, 2)) / unit
            assert np.ptp(through) <= 1e-5 * np.abs(through).max(), (e, np.ptp(through))
            assert abs(through.mean() - 2.0 * out["T12"][0]) <= 1e-3 * abs(through.mean())


def test_currents_need_the_flag(need_gpu):
    htotd, hopx = HB.ti_wire(4, 2, 2)
    with Solver(4, 2, 2) as s:
        s.set_hamiltonian(htotd, hopx)
        s.energy_sweep(0.1, 1.0, 0.0, 0.01)
        with pytest.raises(capi.NegfError) as ei:
            s.calculate_currents([_site(4, 2, 2)] * 3)
        assert ei.value.code == capi.NEGF_ESTATE
        with pytest.raises(capi.NegfError) as ei:
            s.solve_batch([0.1], 1.0, 0.0, 0.01, currents=[_site(4, 2, 2, 1)] * 3)
        assert ei.value.code == capi.NEGF_ESTATE


ER_KEYS = ("ERJx", "ERJy", "ERJz")
OR_KEYS = ("ORJx", "ORJy", "ORJz")


def _assert_density_close(got, want, what, rtol=1e-9):
    scale = max(np.abs(want).max(), 1e-300)
    err = np.abs(np.asarray(got) - want).max() / scale
    assert err <= rtol, "%s: max err %.3e of max > %.1e" % (what, err, rtol)


def test_per_energy_resolved_match_oracle(need_gpu):
    """erCD/orCD arrays of one energy through negf_calculate_resolved."""
    npx, npy, npz = 5, 3, 2
    htotd, hopx = HB.ti_wire(npx, npy, npz, W=0.1, seed=5, flux=0.3, zeeman=0.01)
    opt = O.SolveOptions(eta=1e-5, sr_tol=1e-10, kT=0.025)
    mu = (0.005, -0.005)
    de = 0.6 / 63
    with Solver(npx, npy, npz, eta=1e-5, sr_tol=1e-10, calc_currents=True) as s:
        s.set_hamiltonian(htotd, hopx)
        for e in (-0.17, 0.002):
            ref = O.energy_sweep(htotd, hopx, e, mu, de, npy, npz, opt, calc_currents=True, calc_resolved=True)
            s.energy_sweep(e, ref["f1"], ref["f2"], de)
            er = [_site(npx, npy, npz) for _ in range(4)]
            orb = [np.zeros((npx, npy, npz, 16), order="F") for _ in range(3)] + \
                [np.zeros((npx, npy, npz, 4), order="F")]
            s.calculate_resolved(er=er, orb=orb)
            for k, got in zip(ER_KEYS, er):
                assert_currents_close(got, ref[k], "%s(E=%g)" % (k, e))
            _assert_density_close(er[3], ref["ERRhon"], "ERRhon(E=%g)" % e)
            for k, got in zip(OR_KEYS, orb):
                assert_currents_close(got, ref[k], "%s(E=%g)" % (k, e))
            _assert_density_close(orb[3], ref["ORRhon"], "ORRhon(E=%g)" % e)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_resolved_match_oracle(need_gpu, precision):
    """Two slots over several device batches: ERJ columns per request, ORJ/ORRhon summed
    per slot, and the totals unchanged by asking for them."""
    npx, npy, npz = 5, 2, 3
    hs = [HB.ti_wire(npx, npy, npz, W=0.2, seed=s, flux=0.5, zeeman=0.01) for s in (7, 8)]
    opt = O.SolveOptions(eta=1e-5, sr_tol=1e-10, kT=0.025)
    mu = (0.005, -0.005)
    energies = np.linspace(-0.22, 0.22, 4)
    de = energies[1] - energies[0]
    refs, reqs = [], []
    for slot, (h, x) in enumerate(hs):
        for e in energies:
            ref = O.energy_sweep(h, x, float(e), mu, de, npy, npz, opt, calc_currents=True, calc_resolved=True)
            refs.append((slot, ref))
            reqs.append((e, ref["f1"], ref["f2"], slot))
    e, f1, f2, slots = (np.array(v) for v in zip(*reqs))
    n = e.size
    er = [_site(npx, npy, npz, n) for _ in range(4)]
    orb = [np.zeros((npx, npy, npz, 16, 2), order="F") for _ in range(3)] + \
        [np.zeros((npx, npy, npz, 4, 2), order="F")]
    j = [_site(npx, npy, npz, 2) for _ in KEYS]
    j_plain = [_site(npx, npy, npz, 2) for _ in KEYS]
    kw = dict(n_hamiltonians=2, max_batch=3, eta=1e-5, sr_tol=1e-10, calc_currents=True, precision=precision)
    with Solver(npx, npy, npz, **kw) as s:
        for slot, (h, x) in enumerate(hs):
            s.set_hamiltonian(h, x, slot=slot)
        s.solve_batch(e, f1, f2, de, slots=slots, currents=j_plain)
        out = s.solve_batch(e, f1, f2, de, slots=slots, currents=j, er=er, orb=orb)
    assert (out["status"] == 0).all()
    for a, b in zip(j, j_plain):
        assert np.array_equal(a, b)
    rtol_d = 1e-9 if precision == "fp64" else 1e-6
    for i, (slot, ref) in enumerate(refs):
        for k, got in zip(ER_KEYS, er):
            assert_currents_close(got[..., i], ref[k], "%s request %d" % (k, i))
        _assert_density_close(er[3][..., i], ref["ERRhon"], "ERRhon request %d" % i, rtol_d)
    for slot in range(2):
        mine = [ref for s_, ref in refs if s_ == slot]
        for k, got in zip(OR_KEYS, orb):
            assert_currents_close(got[..., slot], sum(r[k] for r in mine), "%s slot %d" % (k, slot))
        _assert_density_close(orb[3][..., slot], sum(r["ORRhon"] for r in mine), "ORRhon slot %d" % slot, rtol_d)
        for i, k in enumerate(KEYS):
            assert np.abs(orb[i][..., slot].sum(axis=3) - j[i][..., slot]).max() <= \
                1e-12 * np.abs(j[i][..., slot]).max()


def test_resolved_need_the_flag(need_gpu):
    htotd, hopx = HB.ti_wire(4, 2, 2)
    with Solver(4, 2, 2) as s:
        s.set_hamiltonian(htotd, hopx)
        s.energy_sweep(0.1, 1.0, 0.0, 0.01)
        with pytest.raises(capi.NegfError) as ei:
            s.calculate_resolved(er=[_site(4, 2, 2)] * 4)
        assert ei.value.code == capi.NEGF_ESTATE
        with pytest.raises(capi.NegfError) as ei:
            s.solve_batch([0.1], 1.0, 0.0, 0.01, er=[_site(4, 2, 2, 1)] * 4)
        assert ei.value.code == capi.NEGF_ESTATE
