"""GPU parity: the CUDA path (through the C ABI) against the CPU oracle and the committed
golden vectors.  Tolerance for the FP64 form: 1e-9 relative.  Quantities that can cancel
to ~0 (in-gap transmission and density, spin of an unpolarised wire) are compared
relative to their natural scale: T and the modes to 1e-6 (their scale is O(1) channels),
spin to the largest site density of the same energy window (spin is a difference of
spin-resolved densities)."""
import importlib.util
import os

import numpy as np
import pytest

from conftest import GOLDEN
from oracle import negf_oracle as O
from nonequilibriumgreensfunction_gb300 import Solver, capi
from nonequilibriumgreensfunction_gb300 import hamiltonian as HB

pytestmark = pytest.mark.gpu

RTOL = 1e-9


def _mg():
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    return mg


def close(a, b, rtol=RTOL, floor=None):
    """|a - b| <= rtol * max(|b|, floor); floor defaults to 1e-3 of max|b| and is the
    natural scale of the quantity where its value can cancel to ~0."""
    a = np.asarray(a, dtype=complex)
    b = np.asarray(b, dtype=complex)
    if floor is None:
        floor = 1e-3 * np.abs(b).max()
    den = np.maximum(np.abs(b), max(floor, 1e-300))
    err = (np.abs(a - b) / den).max() if a.size else 0.0
    return err <= rtol, err


def assert_close(a, b, what, rtol=RTOL, floor=None):
    ok, err = close(a, b, rtol, floor)
    assert ok, "%s: max rel err %.3e > %.1e" % (what, err, rtol)


def assert_currents_close(got, want, what, rtol=1e-6):
    """Bond currents: each term is REAL(4) in the reference (Calculate_Observables.F90:7),
    so they are compared against the largest |J| of the array."""
    err = np.abs(got - want).max() / max(np.abs(want).max(), 1e-300)
    assert err <= rtol, "%s: max err %.3e of max|J| > %.1e" % (what, err, rtol)


def test_per_energy_interface_matches_oracle(need_gpu):
    """Contact_Self_Energy -> Get_Retarded_Greens -> Calculate_Gnp -> Calculate_Observables
    at the reference's default size (4x3x3, its Dirac basis, eta = 1e-4, T = 0)."""
    htotd, hopx = HB.ti_wire(4, 3, 3, basis="reference", W=0.1, seed=5)
    opt = O.SolveOptions(eta=1e-4, sr_tol=1e-8, calc_spin=True)
    mu = (0.1, 0.0)
    de = 0.1 / 599
    with Solver(4, 3, 3, eta=1e-4, sr_tol=1e-8, calc_spin=True, keep_g_columns=True) as s:
        s.set_hamiltonian(htotd, hopx)
        for e in (0.0123, 0.05, 0.35, 0.61):
            ref = O.energy_sweep(htotd, hopx, e, mu, de, 3, 3, opt, keep_blocks=True)
            cse = s.contact_self_energy(e)
            assert cse["status"] == 0
            # matrices: normwise (relative to the largest element)
            for k in ("SigmaL", "SigmaR", "GammaL", "GammaR"):
                assert_close(cse[k], ref[k], k, floor=np.abs(ref[k]).max())
            assert_close(cse["dosc"], ref["dosc"], "dosc")
            assert s.get_retarded_greens() == 0
            g1, gn = s.g_columns()
            assert_close(g1, ref["GRLef"], "GRLef", floor=np.abs(ref["GRLef"]).max())
            assert_close(gn, ref["GRRgt"], "GRRgt", floor=np.abs(ref["GRRgt"]).max())
            rn, rp = s.new_site_array(), s.new_site_array()
            s.calculate_gnp(ref["f1"], ref["f2"], de, rn, rp)
            assert_close(rn, ref["RhoN"], "RhoN")
            assert_close(rp, ref["RhoP"], "RhoP")
            cc = np.zeros(2)
            spin = [s.new_site_array() for _ in range(3)]
            obs = s.calculate_observables(de, ref["f1"], ref["f2"], cc, spin)
            for k in ("T12", "Modec1", "Modec2", "EDensity", "HDensity"):
                assert_close(obs[k], ref[k], k, floor=1e-6)
            assert_close(cc, ref["ContactCurrent"], "ContactCurrent", floor=1e-30)
            assert_close(np.stack(spin), ref["SigExp"], "spin", floor=np.abs(ref["RhoN"]).max())


@pytest.mark.parametrize("case", ["ref_debug", "flux_zeeman", "c1", "m576", "m784"])
def test_batch_matches_golden(case, need_gpu):
    mg = _mg()
    c = mg.CASES[case]
    g = np.load(os.path.join(GOLDEN, case + ".npz"))
    htotd, hopx = mg.build_inputs(case)
    assert str(g["h_sha256"]) == mg.h_digest(htotd, hopx)
    e = np.asarray(c["energies"])
    with Solver(c["npx"], c["npy"], c["npz"], eta=c["eta"], sr_tol=c["sr_tol"], calc_spin=True,
                max_batch=min(16, len(e))) as s:
        s.set_hamiltonian(htotd, hopx)
        rn, rp = s.new_site_array(1), s.new_site_array(1)
        spin = [s.new_site_array(1) for _ in range(3)]
        r = s.solve_batch(e, g["f1"], g["f2"], c["dE"], rho_n=rn, rho_p=rp, spin=spin)
    assert (r["status"] == 0).all()
    for k in ("T12", "Modec1", "Modec2", "EDensity", "HDensity"):
        assert_close(r[k], g[k], "%s/%s" % (case, k))
    assert_close(np.stack([r["DOSc1"], r["DOSc2"]], 1), g["DOSc"], "DOSc")
    assert_close(rn[..., 0], g["RhoN_sum"], "RhoN_sum")
    assert_close(rp[..., 0], g["RhoP_sum"], "RhoP_sum")
    assert_close(np.stack([a[..., 0] for a in spin]), g["SigExp_sum"], "spin_sum", floor=np.abs(g["RhoN_sum"]).max())
    # Sancho-Rubio stops at the same iteration as the oracle
    assert (r["sr_iters"] == g["sr_iters"].max(axis=1)).all()


def test_full_size_geometry_matches_golden(need_gpu):
    """M = 400, Npx = 100 (the config-2 wire with flux, Zeeman and disorder)."""
    path = os.path.join(GOLDEN, "c2_sub.npz")
    if not os.path.exists(path):
        pytest.skip("c2_sub golden not generated")
    mg = _mg()
    c = mg.CASES["c2_sub"]
    g = np.load(path)
    htotd, hopx = mg.build_inputs("c2_sub")
    assert str(g["h_sha256"]) == mg.h_digest(htotd, hopx)
    with Solver(c["npx"], c["npy"], c["npz"], eta=c["eta"], sr_tol=c["sr_tol"], calc_spin=True, max_batch=2) as s:
        s.set_hamiltonian(htotd, hopx)
        rn, rp = s.new_site_array(1), s.new_site_array(1)
        spin = [s.new_site_array(1) for _ in range(3)]
        r = s.solve_batch(np.asarray(c["energies"]), g["f1"], g["f2"], c["dE"], rho_n=rn, rho_p=rp, spin=spin)
    assert (r["status"] == 0).all()
    for k in ("T12", "Modec1", "Modec2", "EDensity", "HDensity"):
        assert_close(r[k], g[k], "c2/%s" % k)
    assert_close(rn[..., 0], g["RhoN_sum"], "RhoN_sum")
    assert_close(np.stack([a[..., 0] for a in spin]), g["SigExp_sum"], "spin_sum", floor=np.abs(g["RhoN_sum"]).max())


def test_multi_slot_batch_matches_oracle(need_gpu):
    """Disorder seeds in separate Hamiltonian slots, mixed in one batch; the leads are
    shared, so one decimation per energy serves every slot."""
    npx, npy, npz = 6, 3, 2
    opt = O.SolveOptions(eta=1e-5, sr_tol=1e-10, kT=0.025, calc_spin=True)
    mu = (0.005, -0.005)
    hams = [HB.ti_wire(npx, npy, npz, W=0.15, seed=sd, flux=0.4, zeeman=0.01) for sd in range(3)]
    energies = np.array([-0.2, 0.05, 0.05, 0.21, -0.2, 0.13])
    slots = np.array([0, 1, 2, 2, 1, 0])
    de = 1e-3
    f1 = np.array([O.fermi(x, mu[0], opt.kT) for x in energies])
    f2 = np.array([O.fermi(x, mu[1], opt.kT) for x in energies])
    with Solver(npx, npy, npz, n_hamiltonians=3, max_batch=4, eta=opt.eta, sr_tol=opt.sr_tol, calc_spin=True) as s:
        for k, (h, x) in enumerate(hams):
            s.set_hamiltonian(h, x, slot=k)
        rn = s.new_site_array(3)
        r = s.solve_batch(energies, f1, f2, de, slots=slots, rho_n=rn)
    want_rn = np.zeros((npx, npy, npz, 3))
    for i, (e, sl) in enumerate(zip(energies, slots)):
        h, x = hams[sl]
        ref = O.energy_sweep(h, x, float(e), mu, de, npy, npz, opt)
        assert_close(r["T12"][i], ref["T12"], "T12[%d]" % i, floor=1e-6)
        assert_close(r["EDensity"][i], ref["EDensity"], "EDensity[%d]" % i)
        want_rn[..., sl] += ref["RhoN"]
    assert_close(rn, want_rn, "RhoN per slot")


def test_dense_hopx_and_asymmetric_leads(need_gpu):
    """A HopX that is not site-block-diagonal takes the dense-product path, and end slices
    that differ (H_1 != H_N) need one decimation per lead."""
    npx, npy, npz = 5, 2, 2
    htotd, hopx = HB.ti_wire(npx, npy, npz, W=0.1, seed=1)
    rng = np.random.default_rng(0)
    m = hopx.shape[0]
    hopx = hopx + 0.05 * (rng.standard_normal((m, m)) + 1j * rng.standard_normal((m, m)))
    htotd = htotd.copy()
    d = 0.03 * rng.standard_normal(m)
    htotd[0] = htotd[0] + np.diag(d)        # left end slice differs from the right one
    opt = O.SolveOptions(eta=1e-5, sr_tol=1e-10, kT=0.025, calc_spin=True)
    mu = (0.05, -0.05)
    with Solver(npx, npy, npz, eta=opt.eta, sr_tol=opt.sr_tol, calc_spin=True, max_batch=3) as s:
        s.set_hamiltonian(htotd, hopx)
        es = np.array([-0.15, 0.02, 0.3])
        f1 = [O.fermi(x, mu[0], opt.kT) for x in es]
        f2 = [O.fermi(x, mu[1], opt.kT) for x in es]
        rn = s.new_site_array(1)
        r = s.solve_batch(es, f1, f2, 1e-3, rho_n=rn)
    want = np.zeros((npx, npy, npz))
    for i, e in enumerate(es):
        ref = O.energy_sweep(htotd, hopx, float(e), mu, 1e-3, npy, npz, opt)
        for k in ("T12", "Modec1", "Modec2", "EDensity", "HDensity"):
            assert_close(r[k][i], ref[k], "%s[%d]" % (k, i), floor=1e-6)
        assert_close([r["DOSc1"][i], r["DOSc2"][i]], ref["dosc"], "dosc[%d]" % i)
        want += ref["RhoN"]
    assert_close(rn[..., 0], want, "RhoN")


@pytest.mark.parametrize("precision,rtol", [("fp64", RTOL), ("mixed", 1e-6)])
def test_joint_and_one_sided_decimations_in_one_batch(need_gpu, precision, rtol):
    """Two slots in one batch: slot 0 has equal end slices (one decimation serves both
    leads), slot 1 a right end slice shifted by a potential (a left-only and a right-only
    decimation).  The problems are ordered left-only, joint, right-only, and each lead's
    products run over its own range; every request must match the oracle."""
    npx, npy, npz = 6, 3, 3
    h0, hopx = HB.ti_wire(npx, npy, npz, W=0.1, seed=7, flux=0.4, zeeman=0.01)
    h1, _ = HB.ti_wire(npx, npy, npz, W=0.1, seed=8, flux=0.4, zeeman=0.01)
    h1 = h1.copy()
    h1[-1] = h1[-1] + 0.02 * np.eye(h1.shape[1])
    opt = O.SolveOptions(eta=1e-5, sr_tol=1e-10, kT=0.025)
    mu = (0.005, -0.005)
    es = np.array([-0.22, -0.05, 0.011, 0.17])
    e_all = np.concatenate([es, es])
    slots = np.repeat([1, 0], es.size)            # the one-sided slot first in the batch
    f1 = [O.fermi(x, mu[0], opt.kT) for x in e_all]
    f2 = [O.fermi(x, mu[1], opt.kT) for x in e_all]
    with Solver(npx, npy, npz, n_hamiltonians=2, eta=opt.eta, sr_tol=opt.sr_tol, max_batch=e_all.size,
                precision=precision) as s:
        s.set_hamiltonian(h0, hopx, slot=0)
        s.set_hamiltonian(h1, hopx, slot=1)
        r = s.solve_batch(e_all, f1, f2, 1e-3, slots=slots)
    assert (r["status"] == 0).all()
    for i, (e, sl) in enumerate(zip(e_all, slots)):
        ref = O.energy_sweep(h1 if sl else h0, hopx, float(e), mu, 1e-3, npy, npz, opt)
        for k in ("T12", "Modec1", "Modec2"):
            assert_close(r[k][i], ref[k], "%s[%d]" % (k, i), rtol=rtol, floor=1e-3)
        assert_close([r["DOSc1"][i], r["DOSc2"][i]], ref["dosc"], "dosc[%d]" % i, rtol=rtol)
        if precision == "fp64":
            assert r["sr_iters"][i] == max(ref["sr_iters"])


@pytest.mark.parametrize("precision,rtol,rho_rtol", [("fp64", RTOL, RTOL), ("mixed", 1e-6, 5e-6)])
def test_uniform_hop_block_with_general_entries(need_gpu, precision, rtol, rho_rtol):
    """Every site shares one HopX block whose nonzeros are general complex numbers, with
    rows of different kinds (one real extra entry): the compact term lists of the HopX
    products and of the W assembly take their general and mixed branches.  The mixed form
    keeps T, the modes and EDensity/HDensity within 1e-6; its site densities measured 2.1e-6
    at one site of this 2 x 2 cross-section near a band edge, so they are held to 5e-6."""
    npx, npy, npz = 6, 2, 2
    htotd, hopx = HB.ti_wire(npx, npy, npz, W=0.1, seed=4, flux=0.3)
    blk = hopx[:4, :4] * np.exp(0.3j)
    blk[0, 1] = 0.04                                # a real entry beside general ones
    nsite = npy * npz
    hopx = np.kron(np.eye(nsite), blk)
    opt = O.SolveOptions(eta=1e-5, sr_tol=1e-10, kT=0.025, calc_spin=True)
    mu = (0.05, -0.05)
    es = np.array([-0.6, -0.4, 0.45])               # in the bands of the 2 x 2 cross-section
    f1 = [O.fermi(x, mu[0], opt.kT) for x in es]
    f2 = [O.fermi(x, mu[1], opt.kT) for x in es]
    with Solver(npx, npy, npz, eta=opt.eta, sr_tol=opt.sr_tol, calc_spin=True, max_batch=3,
                precision=precision) as s:
        s.set_hamiltonian(htotd, hopx)
        rn = s.new_site_array(1)
        r = s.solve_batch(es, f1, f2, 1e-3, rho_n=rn)
    assert (r["status"] == 0).all()
    want = np.zeros((npx, npy, npz))
    for i, e in enumerate(es):
        ref = O.energy_sweep(htotd, hopx, float(e), mu, 1e-3, npy, npz, opt)
        for k in ("T12", "Modec1", "EDensity", "HDensity"):
            assert_close(r[k][i], ref[k], "%s[%d]" % (k, i), rtol=rtol, floor=1e-6)
        want += ref["RhoN"]
    assert_close(rn[..., 0], want, "RhoN", rtol=rho_rtol)


def test_result_is_the_same_alone_and_in_a_batch(need_gpu):
    """Each item's arithmetic is independent of what else is in the batch: bitwise equal."""
    npx, npy, npz = 8, 3, 3
    htotd, hopx = HB.ti_wire(npx, npy, npz, W=0.1, seed=9, flux=0.5, zeeman=0.01)
    es = np.linspace(-0.25, 0.25, 7)
    with Solver(npx, npy, npz, eta=1e-5, sr_tol=1e-10, max_batch=7) as s:
        s.set_hamiltonian(htotd, hopx)
        full = s.solve_batch(es, 0.7, 0.2, 1e-3)
        for i in (0, 3, 6):
            one = s.solve_batch(es[i:i + 1], 0.7, 0.2, 1e-3)
            for k in ("T12", "EDensity", "Modec1", "DOSc1"):
                assert one[k][0] == full[k][i], (k, i)


def test_sancho_rubio_cap_reports_no_convergence(need_gpu):
    htotd, hopx = HB.ti_wire(4, 2, 2)
    with Solver(4, 2, 2, eta=1e-5, sr_tol=1e-10, sr_max_iter=1) as s:
        s.set_hamiltonian(htotd, hopx)
        r = s.solve_batch([0.1], 1.0, 0.0, 1e-3)
        assert r["status"][0] == capi.NEGF_ESR_NOCONV
        assert r["sr_iters"][0] == 1


def test_singular_block_reports_info_and_handle_stays_usable(need_gpu):
    """A vacancy (zeroed rows/columns of Htotd and HopX, the pattern of Insert_Vacancy,
    Build_Hamiltonian.F90:170-182) at E = 0 with eta = 0 makes an RGF block exactly singular:
    the solve reports LAPACK-style INFO > 0 and the next solve on the handle is normal."""
    npx, npy, npz = 4, 2, 2
    htotd, hopx = HB.ti_wire(npx, npy, npz)
    htotd = htotd.copy()
    hopx = hopx.copy()
    r0 = 4  # orbitals of site 1
    htotd[1, r0:r0 + 4, :] = 0
    htotd[1, :, r0:r0 + 4] = 0
    hopx[r0:r0 + 4, :] = 0
    hopx[:, r0:r0 + 4] = 0
    good_h, good_x = HB.ti_wire(npx, npy, npz)
    with Solver(npx, npy, npz, eta=0.0, sr_tol=1e-10, n_hamiltonians=2, max_batch=1) as s:
        s.set_hamiltonian(htotd, hopx, slot=0)
        r = s.solve_batch([0.0], 1.0, 0.0, 1e-3)
        assert r["status"][0] > 0
        s.set_hamiltonian(good_h, good_x, slot=1)     # a new HopX: slot 0 is invalidated
        r2 = s.solve_batch([0.0], 1.0, 0.0, 1e-3, slots=[1])
        assert r2["status"][0] == 0
        with pytest.raises(capi.NegfError) as ei:
            s.solve_batch([0.0], 1.0, 0.0, 1e-3, slots=[0])
        assert ei.value.code == capi.NEGF_ENOHAM
    ref = O.energy_sweep(good_h, good_x, 0.0, (0.0, 0.0), 1e-3, npy, npz, O.SolveOptions(eta=0.0, sr_tol=1e-10))
    assert_close(r2["T12"][0], ref["T12"], "T12 after singular", floor=1e-6)
    assert_close(r2["EDensity"][0], ref["EDensity"], "EDensity after singular", floor=1e-6)


def test_bad_arguments_are_rejected(need_gpu):
    with pytest.raises(capi.NegfError) as ei:
        Solver(1, 2, 2)   # Npx = 1 is not a valid RGF chain (Recursive_Greens.F90:55 indexes GRu(:,:,0))
    assert ei.value.code == capi.NEGF_EINVAL
    with Solver(3, 2, 2) as s:
        with pytest.raises(capi.NegfError) as ei:
            s.solve_batch([0.1], 1.0, 0.0, 1e-3)      # no Hamiltonian yet
        assert ei.value.code == capi.NEGF_ENOHAM
        with pytest.raises(capi.NegfError):
            s.get_retarded_greens()                    # before contact_self_energy


def test_c_driver_energy_loop_matches_oracle(need_gpu, tmp_path):
    """A C caller making Energy_Sweep's calls in the reference's order (the sequence the
    Fortran ISO_C_BINDING shim makes), on arrays in the reference's memory layout."""
    import subprocess
    from conftest import REPO
    npx, npy, npz = 4, 3, 3
    htotd, hopx = HB.ti_wire(npx, npy, npz, basis="reference", W=0.05, seed=2)
    m = htotd.shape[1]
    hf = np.ascontiguousarray(htotd.transpose(0, 2, 1))       # Htotd(M, M, npx) memory
    xf = np.asfortranarray(hopx)
    (tmp_path / "h.bin").write_bytes(hf.tobytes())
    (tmp_path / "x.bin").write_bytes(xf.tobytes(order="F"))
    libdir = os.path.dirname(capi.library_path())
    exe = str(tmp_path / "drv")
    subprocess.run(["gcc", "-O1", "-I", os.path.join(REPO, "include"),
                    os.path.join(REPO, "nonequilibriumgreensfunction_gb300", "fortran", "energy_sweep_driver.c"),
                    "-o", exe, "-L", libdir, "-lnegf_gb300", "-Wl,-rpath," + libdir], check=True)
    mu1, mu2, n_e = 0.1, 0.0, 12
    e_min, e_max = -1e-10, 0.1 + 1e-10
    out = tmp_path / "out.bin"
    subprocess.run([exe, str(npx), str(npy), str(npz), str(tmp_path / "h.bin"), str(tmp_path / "x.bin"),
                    "1e-4", "1e-8", repr(mu1), repr(mu2), str(n_e), repr(e_min), repr(e_max), str(out)], check=True)
    vals = np.fromfile(out, dtype=np.float64)
    nsites = npx * npy * npz
    per_e = vals[:7 * n_e].reshape(n_e, 7)
    rhon = vals[7 * n_e:7 * n_e + nsites].reshape((npx, npy, npz), order="F")
    j0 = 7 * n_e + 2 * nsites + 2
    jgot = [vals[j0 + i * nsites:j0 + (i + 1) * nsites].reshape((npx, npy, npz), order="F") for i in range(3)]
    opt = O.SolveOptions(eta=1e-4, sr_tol=1e-8)
    eaxis = e_min + (e_max - e_min) / (n_e - 1) * np.arange(n_e)
    w = O.energy_weights(eaxis, (e_max - e_min) / (n_e - 1))
    want_rn = np.zeros((npx, npy, npz))
    want_j = [np.zeros((npx, npy, npz)) for _ in range(3)]
    for k, e in enumerate(eaxis):
        ref = O.energy_sweep(htotd, hopx, float(e), (mu1, mu2), w[k], npy, npz, opt, calc_currents=True)
        for i, key in enumerate(("Jx", "Jy", "Jz")):
            want_j[i] += ref[key]
        got = dict(zip(["T12", "EDensity", "HDensity", "Modec1", "Modec2"], per_e[k, :5]))
        for key, v in got.items():
            assert_close(v, ref[key], "%s[%d]" % (key, k), floor=1e-6)
        assert_close(per_e[k, 5:7], ref["dosc"], "dosc[%d]" % k)
        want_rn += ref["RhoN"]
    assert_close(rhon, want_rn, "RhoN")
    for i, key in enumerate(("Jx", "Jy", "Jz")):
        assert_currents_close(jgot[i], want_j[i], key)
