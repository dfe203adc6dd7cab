"""Mixed form (tcgen05 sliced-BF16 products, FP32 Gauss-Jordan + Newton-Schulz inverses
with FP64-class residuals): accuracy against the FP64 oracle and the FP64 GPU form.

Stated tolerance of the mixed form: transmission, the modes and site density within 1e-6
relative of the FP64 result (T and modes floored at 1e-3 channels, density at 1e-3 of its
maximum); spin within 1e-6 of the largest site density of the same energies (spin is a
difference of spin-resolved densities and cancels to ~0 in an unpolarised wire)."""
import importlib.util
import os

import numpy as np
import pytest

from conftest import GOLDEN
from oracle import negf_oracle as O
from nonequilibriumgreensfunction_gb300 import Solver, capi
from nonequilibriumgreensfunction_gb300 import hamiltonian as HB

pytestmark = pytest.mark.gpu

MIXED_RTOL = 1e-6


def rel_err(a, b, floor):
    a, b = np.asarray(a), np.asarray(b)
    return float((np.abs(a - b) / np.maximum(np.abs(b), floor)).max())


def _mg():
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    return mg


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
        spin = [s.new_site_array(1) for _ in range(3)]
        r = s.solve_batch(es, f1, f2, 1e-3, rho_n=rn, spin=spin)
    assert (r["status"] == 0).all()
    want = np.zeros((npx, npy, npz))
    want_spin = np.zeros((3, npx, npy, npz))
    for i, e in enumerate(es):
        ref = O.energy_sweep(htotd, hopx, float(e), mu, 1e-3, npy, npz, opt)
        assert rel_err(r["T12"][i], ref["T12"], 1e-3) <= MIXED_RTOL, (e, r["T12"][i], ref["T12"])
        assert rel_err(r["Modec1"][i], ref["Modec1"], 1e-3) <= MIXED_RTOL
        assert rel_err(r["DOSc1"][i], ref["dosc"][0], 1e-3) <= MIXED_RTOL
        want += ref["RhoN"]
        want_spin += ref["SigExp"]
    assert rel_err(rn[..., 0], want, 1e-3 * np.abs(want).max()) <= MIXED_RTOL
    got_spin = np.stack([a[..., 0] for a in spin])
    assert np.abs(got_spin - want_spin).max() <= MIXED_RTOL * np.abs(want).max()


def _check_against_golden(case, max_batch):
    mg = _mg()
    c = mg.CASES[case]
    g = np.load(os.path.join(GOLDEN, case + ".npz"))
    htotd, hopx = mg.build_inputs(case)
    assert str(g["h_sha256"]) == mg.h_digest(htotd, hopx)
    with Solver(c["npx"], c["npy"], c["npz"], eta=c["eta"], sr_tol=c["sr_tol"], calc_spin=True,
                max_batch=max_batch, precision="mixed") as s:
        s.set_hamiltonian(htotd, hopx)
        s.profile(True)
        rn, rp = s.new_site_array(1), s.new_site_array(1)
        spin = [s.new_site_array(1) for _ in range(3)]
        r = s.solve_batch(np.asarray(c["energies"]), g["f1"], g["f2"], c["dE"], rho_n=rn, rho_p=rp, spin=spin)
        st = s.stats()
    assert (r["status"] == 0).all(), r["status"]
    for k in ("T12", "Modec1", "Modec2"):
        assert rel_err(r[k], g[k], 1e-3) <= MIXED_RTOL, (case, k, r[k], g[k])
    for k in ("EDensity", "HDensity"):
        assert rel_err(r[k], g[k], 1e-3 * np.abs(g[k]).max()) <= MIXED_RTOL, (case, k)
    assert rel_err(np.stack([r["DOSc1"], r["DOSc2"]], 1), g["DOSc"], 1e-3 * np.abs(g["DOSc"]).max()) <= MIXED_RTOL
    scale = np.abs(g["RhoN_sum"]).max()
    assert rel_err(rn[..., 0], g["RhoN_sum"], 1e-3 * scale) <= MIXED_RTOL
    assert rel_err(rp[..., 0], g["RhoP_sum"], 1e-3 * np.abs(g["RhoP_sum"]).max()) <= MIXED_RTOL
    got_spin = np.stack([a[..., 0] for a in spin])
    assert np.abs(got_spin - g["SigExp_sum"]).max() <= MIXED_RTOL * scale
    # the products ran on the tensor cores, and every inverse kept in the mixed form was
    # certified (residual norm before its last update <= ns_tol = 1e-5)
    assert st["tc_launches"] > 0 and st["ns_final_residual_max"] <= 1e-5
    return st


def test_mixed_full_size_matches_golden(need_gpu):
    """M = 400, Npx = 100: the mixed form against the FP64 golden vectors."""
    _check_against_golden("c2_sub", 2)


@pytest.mark.parametrize("case", ["m576", "m784"])
def test_mixed_large_cross_sections_match_golden(need_gpu, case):
    """M = 576 and M = 784 (the config-5 and the largest config-4 cross-sections): every
    product has K' = 2M > 800, so the tensor-core GEMM accumulates each half of K in its
    own set of exact accumulators; T, modes, DOS, densities and spin against the oracle."""
    _check_against_golden(case, 3)


def test_mixed_sixteen_seed_batch_matches_fp64(need_gpu):
    """A config-3 style batch: M = 400, Npx = 100, 16 disorder seeds with W_s ~ U[0, 0.2]
    eV drawn from seed s, at an energy near the bulk band edge and one mid-gap, all 32
    solves in one mixed batch, against the FP64 GPU form (itself pinned to the oracle at
    1e-9 by test_gpu_parity) on the same device-built wires."""
    npx, npy, npz, n_seeds = 100, 10, 10, 16
    es = np.repeat([-0.248, 0.0037], n_seeds)
    slots = np.tile(np.arange(n_seeds), 2)
    mu = (0.005, -0.005)
    f1 = [O.fermi(e, mu[0], 0.025) for e in es]
    f2 = [O.fermi(e, mu[1], 0.025) for e in es]
    models = [HB.wire_model(W=float(np.random.default_rng(s).uniform(0.0, 0.2)), seed=s, flux=0.5, zeeman=0.01)
              for s in range(n_seeds)]
    out = {}
    for prec in ("mixed", "fp64"):
        with Solver(npx, npy, npz, n_hamiltonians=n_seeds, max_batch=es.size, eta=1e-5, sr_tol=1e-10,
                    calc_spin=True, precision=prec) as s:
            for k, m in enumerate(models):
                s.build_hamiltonian(m, slot=k)
            s.profile(True)
            rn = s.new_site_array(n_seeds)
            spin = [s.new_site_array(n_seeds) for _ in range(3)]
            r = s.solve_batch(es, f1, f2, 0.6 / 2047, slots=slots, rho_n=rn, spin=spin)
            out[prec] = (r, rn, np.stack(spin), s.stats())
    (rm, rnm, spm, stm), (rf, rnf, spf, _) = out["mixed"], out["fp64"]
    assert (rm["status"] == 0).all() and (rf["status"] == 0).all()
    assert rel_err(rm["T12"], rf["T12"], 1e-3) <= MIXED_RTOL
    assert rel_err(rm["Modec1"], rf["Modec1"], 1e-3) <= MIXED_RTOL
    for k in range(n_seeds):
        scale = np.abs(rnf[..., k]).max()
        assert rel_err(rnm[..., k], rnf[..., k], 1e-3 * scale) <= MIXED_RTOL, k
        assert np.abs(spm[..., k] - spf[..., k]).max() <= MIXED_RTOL * scale, k
    # every inverse kept in the mixed form was certified: its residual norm before the last
    # update was at most ns_tol (1e-5), so that update left an error of order 1e-10 or less;
    # the others (ns_unconverged, fallbacks) were redone in FP64
    assert stm["ns_final_residual_max"] <= 1e-5


def test_newton_schulz_cap_sends_unconverged_inverses_to_fp64(need_gpu):
    """The refinement cap is never a silent exit.  With the cap at the two fixed steps and
    a tolerance no residual can meet, every inverse is left unconverged: each must be
    redone in FP64 (counted in ns_unconverged and fallbacks), no request may fail, and the
    results must match the oracle."""
    npx, npy, npz = 8, 3, 3
    htotd, hopx = HB.ti_wire(npx, npy, npz, W=0.1, seed=4, flux=0.5, zeeman=0.01)
    opt = O.SolveOptions(eta=1e-5, sr_tol=1e-10, kT=0.025, calc_spin=True)
    mu = (0.005, -0.005)
    es = np.array([-0.2481, 0.0013, 0.19])
    f1 = [O.fermi(e, mu[0], opt.kT) for e in es]
    f2 = [O.fermi(e, mu[1], opt.kT) for e in es]
    with Solver(npx, npy, npz, eta=opt.eta, sr_tol=opt.sr_tol, calc_spin=True, max_batch=3,
                precision="mixed") as s:
        s.set_hamiltonian(htotd, hopx)
        s.set_refinement(ns_max_steps=2, ns_tol=1e-30)
        s.profile(True)
        rn = s.new_site_array(1)
        r = s.solve_batch(es, f1, f2, 1e-3, rho_n=rn)
        st = s.stats()
        # the defaults again: the same solve certifies its inverses without redoing any
        s.set_refinement()
        s.profile(True)
        r2 = s.solve_batch(es, f1, f2, 1e-3)
        st2 = s.stats()
    assert (r["status"] == 0).all()
    # every RGF inverse (2 per slice per energy) at least, plus the decimation's
    assert st["ns_unconverged"] >= 2 * npx * es.size
    assert st["fallbacks"] >= st["ns_unconverged"]
    assert st2["ns_unconverged"] == 0 and st2["ns_final_residual_max"] <= 1e-5
    want = np.zeros((npx, npy, npz))
    for i, e in enumerate(es):
        ref = O.energy_sweep(htotd, hopx, float(e), mu, 1e-3, npy, npz, opt)
        assert rel_err(r["T12"][i], ref["T12"], 1e-3) <= MIXED_RTOL
        assert rel_err(r2["T12"][i], ref["T12"], 1e-3) <= MIXED_RTOL
        want += ref["RhoN"]
    assert rel_err(rn[..., 0], want, 1e-3 * np.abs(want).max()) <= MIXED_RTOL


def test_set_refinement_validates_its_arguments(need_gpu):
    with Solver(4, 3, 3, precision="mixed") as s:
        for bad in (dict(ns_max_steps=1), dict(ns_max_steps=17), dict(ns_tol=1.0), dict(ns_accept=1.5)):
            with pytest.raises(capi.NegfError) as ei:
                s.set_refinement(**bad)
            assert ei.value.code == capi.NEGF_EINVAL
        s.set_refinement(ns_max_steps=6, ns_tol=1e-8, ns_accept=0.25)
    with Solver(4, 3, 3, precision="fp64") as s:
        with pytest.raises(capi.NegfError) as ei:
            s.set_refinement(ns_max_steps=3)
        assert ei.value.code == capi.NEGF_ESTATE


def test_fused_gauss_jordan_gives_the_same_bits_as_the_three_launch_form(need_gpu):
    """A batch with at least one matrix per SM inverts its FP32 blocks with the fused
    one-CTA-per-matrix Gauss-Jordan kernel; smaller batches use the panel / interchange /
    update launches.  Both run the same operations in the same order, so a request's
    results are bitwise the same in a batch of 160 and in batches of 8."""
    npx, npy, npz = 6, 3, 3
    htotd, hopx = HB.ti_wire(npx, npy, npz, W=0.1, seed=6, flux=0.5, zeeman=0.01)
    es = np.linspace(-0.29, 0.29, 160)
    f1 = np.full(es.size, 0.7)
    f2 = np.full(es.size, 0.2)
    out = []
    for mb in (160, 8):
        with Solver(npx, npy, npz, eta=1e-5, sr_tol=1e-10, calc_spin=True, max_batch=mb, precision="mixed") as s:
            s.set_hamiltonian(htotd, hopx)
            rn = s.new_site_array(1)
            r = s.solve_batch(es, f1, f2, 1e-3, rho_n=rn)
            out.append((r, rn))
    (ra, rna), (rb, rnb) = out
    assert (ra["status"] == 0).all() and (rb["status"] == 0).all()
    for k in ("T12", "Modec1", "Modec2", "EDensity", "HDensity", "DOSc1"):
        assert np.array_equal(ra[k], rb[k]), k
