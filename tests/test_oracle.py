"""Pinning the CPU oracle (no GPU): the reference publishes no test vectors and cannot be
built here, so the oracle is checked against a dense inverse of the full block-tridiagonal
matrix and against physics invariants, and the committed golden vectors are checked to be
the oracle's own output."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN
from oracle import negf_oracle as O
from nonequilibriumgreensfunction_gb300 import hamiltonian as HB


def _wire(npx=5, npy=3, npz=2, **kw):
    return HB.ti_wire(npx, npy, npz, **kw)


@pytest.mark.parametrize("energy", [-0.2, 0.0, 0.13, 0.4])
@pytest.mark.parametrize("basis", ["tau_sigma", "reference"])
def test_rgf_columns_equal_dense_inverse(energy, basis):
    htotd, hopx = _wire(basis=basis, W=0.2, seed=7, flux=0.3, zeeman=0.02)
    opt = O.SolveOptions(eta=1e-4)
    r = O.energy_sweep(htotd, hopx, energy, (0.05, -0.05), 1e-3, 3, 2, opt, keep_blocks=True)
    g = O.dense_retarded_greens(htotd, hopx, r["SigmaL"], r["SigmaR"], energy, opt.eta)
    m = htotd.shape[1]
    npx = htotd.shape[0]
    scale = np.abs(g).max()
    for x in range(npx):
        assert np.abs(g[x * m:(x + 1) * m, :m] - r["GRLef"][x]).max() < 1e-11 * scale
        assert np.abs(g[x * m:(x + 1) * m, -m:] - r["GRRgt"][x]).max() < 1e-11 * scale
        assert np.abs(g[x * m:(x + 1) * m, x * m:(x + 1) * m] - r["GRd"][x]).max() < 1e-11 * scale


def test_transmission_reciprocity_and_sum_rule():
    htotd, hopx = _wire(W=0.3, seed=2, zeeman=0.01)
    opt = O.SolveOptions(eta=1e-5, sr_tol=1e-10)
    e = 0.11
    r = O.energy_sweep(htotd, hopx, e, (0.1, -0.1), 1e-3, 3, 2, opt, keep_blocks=True, calc_currents=True)
    g = O.dense_retarded_greens(htotd, hopx, r["SigmaL"], r["SigmaR"], e, opt.eta)
    m = htotd.shape[1]
    g1n, gn1 = g[:m, -m:], g[-m:, :m]
    t_lr = np.real(np.trace(r["GammaL"] @ g1n @ r["GammaR"] @ g1n.conj().T))
    t_rl = np.real(np.trace(r["GammaR"] @ gn1 @ r["GammaL"] @ gn1.conj().T))
    assert abs(t_lr - r["T12"]) < 1e-12 * max(1.0, abs(t_lr))
    # L <-> R reciprocity holds up to the eta-broadening of the device
    assert abs(t_lr - t_rl) < 1e-6
    # sum rule i(G - G^H) = G (Gamma_L + Gamma_R + 2 eta) G^H on every diagonal block
    a_full = 1j * (g - g.conj().T)
    gam = np.zeros_like(g)
    gam[:m, :m] = r["GammaL"]
    gam[-m:, -m:] = r["GammaR"]
    rhs = g @ (gam + 2 * opt.eta * np.eye(g.shape[0])) @ g.conj().T
    assert np.abs(a_full - rhs).max() < 1e-9 * np.abs(a_full).max()
    # and Gn + Gp of the reference equals the contact part of the spectral function
    contact = g @ gam @ g.conj().T
    for x in range(htotd.shape[0]):
        blk = slice(x * m, (x + 1) * m)
        assert np.abs(r["Gnd"][x] + r["Gpd"][x] - contact[blk, blk]).max() < 1e-10 * np.abs(contact).max()


def test_clean_wire_has_integer_transmission():
    htotd, hopx = _wire(npx=6, npy=3, npz=3)
    opt = O.SolveOptions(eta=1e-7, sr_tol=1e-12)
    for e in (0.05, 0.25, 0.45):
        r = O.energy_sweep(htotd, hopx, e, (0.0, 0.0), 1e-3, 3, 3, opt)
        assert abs(r["T12"] - round(r["T12"])) < 1e-3, (e, r["T12"])
        assert abs(r["Modec1"] - r["Modec2"]) < 1e-3


def test_self_energy_satisfies_surface_dyson_equation():
    # Sigma_L = H^H (alpha - Sigma_L)^-1 H, Sigma_R = H (alpha - Sigma_R)^-1 H^H, alpha = (E + i eta) - H_1.
    # The reference seeds the decimation with inv(alpha + i eta) (an extra i eta,
    # Contact_Self_Energy.F90:141) while the final g uses alpha, so the equation holds up to
    # O(eta): the residual must shrink in proportion to eta.
    htotd, hopx = _wire(npx=3, W=0.0)
    m = htotd.shape[1]
    for e in (-0.1, 0.2):
        rel = []
        for eta in (1e-5, 1e-7):
            opt = O.SolveOptions(eta=eta, sr_tol=1e-13)
            cse = O.contact_self_energy(htotd, hopx, e, opt)
            alpha = complex(e, eta) * np.eye(m) - htotd[0]
            sl, sr = cse["SigmaL"], cse["SigmaR"]
            res_l = sl - hopx.conj().T @ np.linalg.inv(alpha - sl) @ hopx
            res_r = sr - hopx @ np.linalg.inv(alpha - sr) @ hopx.conj().T
            r = max(np.abs(res_l).max() / np.abs(sl).max(), np.abs(res_r).max() / np.abs(sr).max())
            assert r < 20 * eta, (e, eta, r)
            rel.append(r)
            for gam in (cse["GammaL"], cse["GammaR"]):   # Hermitian, positive semi-definite
                assert np.abs(gam - gam.conj().T).max() < 1e-12
                assert np.linalg.eigvalsh(gam).min() > -1e-9
        assert rel[1] < rel[0] / 20


def test_gauge_and_basis_invariance():
    # T and density do not depend on the Dirac basis choice (tau_sigma vs the reference's)
    kw = dict(npx=4, npy=3, npz=2, M0=0.3, B=0.25, A=0.5)
    h1, x1 = HB.ti_wire(**kw, basis="tau_sigma")
    opt = O.SolveOptions(eta=1e-5, sr_tol=1e-11)
    r1 = O.energy_sweep(h1, x1, 0.07, (0.1, -0.1), 1e-3, 3, 2, opt)
    # a unitary site rotation U: H -> U H U^H on every site leaves T and site density invariant
    rng = np.random.default_rng(5)
    q, _ = np.linalg.qr(rng.standard_normal((4, 4)) + 1j * rng.standard_normal((4, 4)))
    u = np.kron(np.eye(h1.shape[1] // 4), q)
    h2 = np.einsum("ij,xjk,lk->xil", u, h1, u.conj())
    x2 = u @ x1 @ u.conj().T
    r2 = O.energy_sweep(h2, x2, 0.07, (0.1, -0.1), 1e-3, 3, 2, opt)
    assert abs(r1["T12"] - r2["T12"]) < 1e-9
    assert np.abs(r1["RhoN"] - r2["RhoN"]).max() < 1e-9 * np.abs(r1["RhoN"]).max()


def test_reference_builder_matches_package_builder():
    # oracle's literal Build_Hamiltonian restatement == the package's builder in the reference basis
    dis = HB.disorder_potential(5, 3, 4, 0.2, 11)
    h_o, x_o = O.build_hamiltonian_reference(5, 3, 4, ab_phi=0.35, disorder=dis)
    h_p, x_p = HB.ti_wire(5, 3, 4, basis="reference", flux=0.35, disorder=dis)
    assert np.abs(h_o - h_p).max() < 1e-15
    assert np.abs(x_o - x_p).max() == 0.0
    # and with the tau_sigma blocks passed explicitly
    onsite, hx, hy, hz = HB.site_blocks(0.3, 0.25, 0.5, 0.01)
    h_o, x_o = O.build_hamiltonian_reference(4, 2, 3, ab_phi=0.5, onsite_blocks=onsite, hops=(hx, hy, hz))
    h_p, x_p = HB.ti_wire(4, 2, 3, zeeman=0.01, flux=0.5)
    assert np.abs(h_o - h_p).max() < 1e-15
    assert np.abs(x_o - x_p).max() == 0.0


def test_hamiltonian_is_hermitian_and_leads_match_end_slices():
    h, x = HB.ti_wire(6, 3, 3, W=0.2, seed=4, flux=0.5, zeeman=0.01)
    for s in h:
        assert np.abs(s - s.conj().T).max() < 1e-15
    assert np.array_equal(h[0], h[-1])      # disorder only on slices 2..npx-1
    assert not np.array_equal(h[1], h[0])


def test_sancho_rubio_iteration_cap_and_quirks():
    htotd, hopx = _wire(npx=3)
    opt = O.SolveOptions(eta=1e-5, sr_tol=1e-10, sr_max_iter=1)
    cse = O.contact_self_energy(htotd, hopx, 0.1, opt)
    assert list(cse["sr_iters"]) == [1, 1]


def test_saved_sancho_rubio_counter_caps_the_whole_process():
    """The reference's SAVEd counter (Contact_Self_Energy.F90:119,154-155): calls sharing it
    add up their iterations; once the sum passes 20000 a call does no decimation at all and
    its Sigma comes from the first term alone, while a fresh per-call counter converges."""
    htotd, hopx = _wire(npx=3)
    per_call = O.SolveOptions(eta=1e-5, sr_tol=1e-10)
    ref = O.contact_self_energy(htotd, hopx, 0.1, per_call)
    n = int(ref["sr_iters"][0])
    assert n > 3
    # a fresh process: the shared counter gives the same result as the per-call one and
    # advances by both leads' iterations
    st = O.SrCounter()
    shared = O.SolveOptions(eta=1e-5, sr_tol=1e-10, sr_counter=st)
    a = O.contact_self_energy(htotd, hopx, 0.1, shared)
    assert np.array_equal(a["SigmaL"], ref["SigmaL"]) and np.array_equal(a["SigmaR"], ref["SigmaR"])
    assert st.value == 1 + int(ref["sr_iters"].sum())
    # late in a long single-process run: the left lead gets 2 iterations, the right none
    st.value = 20000 - 1
    b = O.contact_self_energy(htotd, hopx, 0.1, shared)
    assert list(b["sr_iters"]) == [2, 0] and st.value == 20001
    err = np.abs(b["SigmaR"] - ref["SigmaR"]).max() / np.abs(ref["SigmaR"]).max()
    assert err > 1e-3          # Sigma from CapT = t alone, far from the converged one
    c = O.contact_self_energy(htotd, hopx, 0.1, shared)
    assert list(c["sr_iters"]) == [0, 0]
    assert np.array_equal(c["SigmaR"], b["SigmaR"])


def test_energy_weights_follow_energy_sweep():
    eaxis, de0 = O.energy_axis_reference((-0.1, 0.0), 0.0, 600)
    w = O.energy_weights(eaxis, de0)
    assert np.allclose(w[:-1], np.diff(eaxis))
    assert w[-1] == w[-2]


@pytest.mark.parametrize("case", ["ref_debug", "flux_zeeman", "c1"])
def test_golden_vectors_are_oracle_output(case):
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    g = np.load(os.path.join(GOLDEN, case + ".npz"))
    c = mg.CASES[case]
    htotd, hopx = mg.build_inputs(case)
    assert str(g["h_sha256"]) == mg.h_digest(htotd, hopx)
    opt = O.SolveOptions(eta=c["eta"], sr_tol=c["sr_tol"], kT=c["kT"], calc_spin=c["calc_spin"])
    idx = [0, len(c["energies"]) - 1]
    for i in idx:
        r = O.energy_sweep(htotd, hopx, float(c["energies"][i]), c["mu_lead"], c["dE"], c["npy"], c["npz"], opt)
        assert abs(r["T12"] - g["T12"][i]) <= 1e-12 * max(1.0, abs(g["T12"][i]))
        assert abs(r["EDensity"] - g["EDensity"][i]) <= 1e-12 * max(1.0, abs(g["EDensity"][i]))
    p = json.loads(str(g["params"]))
    assert p["npx"] == c["npx"]


def test_bond_currents_obey_kirchhoff_and_landauer():
    """Pins the restatement of Calculate_Observables.F90:110-169: with eta -> 0 the bond
    currents are divergence-free at every interior site (x, y and z bonds together, so their
    signs and orbital index order must agree), and the +x current through any cross-section
    is 2 T12 (f1 - f2) q^2/h (the Gn - Gp difference counts both leads).  The reference's
    REAL(4) terms bound the agreement at ~1e-7 of the largest current."""
    htotd, hopx = HB.ti_wire(6, 3, 3, W=0.2, seed=1, flux=0.3, zeeman=0.01)
    opt = O.SolveOptions(eta=1e-7, sr_tol=1e-10, kT=0.0)
    unit = O.Q_E ** 2 / O.HBAR / (2.0 * O.PI)
    for e in (-0.2, 0.21):
        r = O.energy_sweep(htotd, hopx, e, (0.5, -0.5), 1.0, 3, 3, opt, calc_currents=True)
        jx, jy, jz = r["Jx"] / unit, r["Jy"] / unit, r["Jz"] / unit
        scale = max(np.abs(jx).max(), np.abs(jy).max(), np.abs(jz).max())
        div = jx.copy()
        div[1:] -= jx[:-1]
        div += jy
        div[:, 1:] -= jy[:, :-1]
        div += jz
        div[:, :, 1:] -= jz[:, :, :-1]
        assert np.abs(div[1:-1]).max() <= 1e-6 * scale
        through = jx[:-1].sum(axis=(1, 2))
        assert np.ptp(through) <= 1e-6 * np.abs(through).max()
        assert abs(through.mean() - 2.0 * r["T12"] * (r["f1"] - r["f2"])) <= 1e-3 * abs(through.mean())


def test_resolved_currents_decompose_the_totals():
    """The energy- and orbital-resolved arrays of the restatement (erCD/orCD,
    Calculate_Observables.F90:124-160, Calculate_Gnp.F90:125-129) are decompositions of the
    totals: ERJ dE/(2 pi) = J, the ORJ pairs sum to J, the ORRhon orbitals sum to RhoN and
    ERRhon dE/(2 pi) = RhoN - RhoP."""
    npx, npy, npz = 4, 2, 3
    htotd, hopx = HB.ti_wire(npx, npy, npz, W=0.2, seed=4, flux=0.4, zeeman=0.01)
    opt = O.SolveOptions(eta=1e-5, sr_tol=1e-10, kT=0.025)
    de = 0.013
    w = de / (2.0 * O.PI)
    r = O.energy_sweep(htotd, hopx, 0.07, (0.005, -0.005), de, npy, npz, opt, calc_currents=True,
                       calc_resolved=True)
    for d in "xyz":
        j = r["J" + d]
        scale = np.abs(j).max()
        assert r["ORJ" + d].shape == (npx, npy, npz, 16)
        assert np.abs(r["ERJ" + d] * w - j).max() <= 1e-13 * scale
        assert np.abs(r["ORJ" + d].sum(axis=3) - j).max() <= 1e-13 * scale
    assert r["ORRhon"].shape == (npx, npy, npz, 4)
    assert np.abs(r["ORRhon"].sum(axis=3) - r["RhoN"]).max() <= 1e-13 * np.abs(r["RhoN"]).max()
    diff = r["RhoN"] - r["RhoP"]
    assert np.abs(r["ERRhon"] * w - diff).max() <= 1e-12 * np.abs(diff).max()


def test_bdg_builders_agree():
    """The package's BdG conversion equals the oracle's restatement of the reference's BdG
    blocks (Build_Hamiltonian.F90:52-56, 162-163, 199-200) on a disordered flux wire."""
    npx, npy, npz = 3, 3, 2
    h, x = HB.ti_wire(npx, npy, npz, W=0.3, seed=2, flux=0.4, zeeman=0.02)
    hb, xb = HB.bdg(h, x, npy, npz)
    ho, xo = O.bdg_hamiltonian(h, x, npy, npz, 4)
    assert hb.shape == (npx, 8 * npy * npz, 8 * npy * npz)
    assert np.array_equal(hb, ho) and np.array_equal(xb, xo)
    assert np.abs(hb - hb.conj().transpose(0, 2, 1)).max() == 0.0


def test_model_contact_self_energies():
    """Contact types 1-3 (Contact_Self_Energy.F90:19-67): the phenomenological contacts give
    -Im Tr Sigma / pi = rate x (number of contacted orbitals), and the superconducting
    contacts give the BCS density of states rate M |E| / (pi sqrt(E^2 - Delta^2)) outside the
    gap, a positive semidefinite Gamma, and Sigma_L = Sigma_R at chi = 0."""
    npx, npy, npz = 2, 3, 2
    h, x = HB.ti_wire(npx, npy, npz)
    m = h.shape[1]
    for ct, k in ((1, m), (2, npy * 4)):
        c = O.contact_self_energy(h, x, 0.05, O.SolveOptions(contact_type=ct, tunneling_rate=0.7), npy=npy)
        assert np.allclose(c["dosc"], 0.7 * k / O.PI, rtol=1e-14)
        assert np.allclose(np.diag(c["GammaL"])[:k], 1.4) and np.all(np.diag(c["GammaL"])[k:] == 0)
    hb, xb = O.bdg_hamiltonian(h, x, npy, npz, 4)
    mb = hb.shape[1]
    delta = 1e-3
    for e in (-3e-3, -1.5e-3, 1.2e-3, 4e-3):
        opt = O.SolveOptions(norb=8, contact_type=3, eta=1e-9, delta_sc=(delta, delta), chi_lr=0.8)
        c = O.contact_self_energy(hb, xb, e, opt)
        want = mb * abs(e) / (O.PI * np.sqrt(e * e - delta * delta))
        assert np.allclose(c["dosc"], want, rtol=1e-6), (e, c["dosc"], want)
        for g in (c["GammaL"], c["GammaR"]):
            assert np.linalg.eigvalsh(g).min() >= -1e-9 * np.abs(g).max()
    c = O.contact_self_energy(hb, xb, 0.4e-3, O.SolveOptions(norb=8, contact_type=3, chi_lr=0.0, eta=1e-9))
    assert np.array_equal(c["SigmaL"], c["SigmaR"])
    assert abs(c["dosc"][0]) < 1e-3 * mb                     # inside the gap: eta-broadened only


# channel models 1-4 (Build_Hamiltonian.F90:19-47) with the sizes Read_In_Allocate.F90:51-60 forces
CHANNEL_WIRES = {0: (5, 3, 2), 1: (5, 2, 2), 2: (5, 3, 2), 3: (5, 4, 1), 4: (5, 1, 1)}


@pytest.mark.parametrize("ct", sorted(CHANNEL_WIRES))
def test_channel_models_host_twin_equals_oracle_builder(ct):
    """The package's host twin of the device builder (hamiltonian.channel_model) equals the
    oracle's Build_Hamiltonian restatement, with disorder and (where the model has a 2-D
    cross-section) the Aharonov-Bohm phase; every slice is Hermitian."""
    npx, npy, npz = CHANNEL_WIRES[ct]
    flux = 0.3 if npy > 1 and npz > 1 else 0.0
    m = HB.channel_model(ct, mu_t=0.05, flux=flux, W=0.3, seed=7)
    h, x = HB.build_from_model(npx, npy, npz, m)
    dis = HB.anderson_counter(npx, npy, npz, 0.3, 7)
    ho, xo = O.build_hamiltonian_reference(npx, npy, npz, mu_t=0.05, ab_phi=flux, disorder=dis, channel_type=ct)
    assert h.shape[1] == O.channel_norb(ct) * npy * npz == HB.CHANNEL_NORB[ct] * npy * npz
    assert np.abs(h - ho).max() <= 1e-15 * max(1.0, np.abs(ho).max())
    assert np.array_equal(x, xo)
    for s in ho:
        assert np.abs(s - s.conj().T).max() <= 1e-15 * np.abs(s).max()


def test_channel_models_refuse_sizes_the_reference_forces():
    with pytest.raises(ValueError):
        O.build_hamiltonian_reference(4, 3, 2, channel_type=3)
    with pytest.raises(ValueError):
        O.build_hamiltonian_reference(4, 2, 1, channel_type=4)


def test_one_band_metal_transmission_counts_open_modes():
    """Clean one-band metal (channelType 2): E = 6t + e_y + e_z - 2t cos kx with the open
    chains' transverse levels e = -2t cos(pi m / (n + 1)); T equals the number of
    transverse modes with |E - 6 - e_y - e_z| < 2."""
    npx, npy, npz = 5, 3, 2
    h, x = O.build_hamiltonian_reference(npx, npy, npz, channel_type=2)
    opt = O.SolveOptions(eta=1e-7, sr_tol=1e-12, norb=1)
    ey = -2.0 * np.cos(np.pi * np.arange(1, npy + 1) / (npy + 1))
    ez = -2.0 * np.cos(np.pi * np.arange(1, npz + 1) / (npz + 1))
    for e in (2.0, 3.7, 5.1, 6.3, 9.5):
        n_open = int(np.sum(np.abs(e - 6.0 - ey[:, None] - ez[None, :]) < 2.0))
        r = O.energy_sweep(h, x, e, (0.0, 0.0), 1e-3, npy, npz, opt)
        assert abs(r["T12"] - n_open) < 1e-4, (e, r["T12"], n_open)


def test_spin_orbit_wire_and_surface_models_conduct_integer_channels():
    """The 1-D spin-orbit wire (channelType 4, H(k) = -mu + sin(k) sigma_y) has two
    channels for |E + mu| < 1 and none outside; the clean TI surface strip (3), the Bi2Se3
    wire (1) and the toy TI (0) carry an integer number of channels."""
    h, x = O.build_hamiltonian_reference(5, 1, 1, channel_type=4, mu_t=0.1)
    opt = O.SolveOptions(eta=1e-7, sr_tol=1e-12, norb=2)
    for e, want in ((-0.9, 2), (0.3, 2), (0.7, 2), (1.3, 0), (-1.4, 0)):
        r = O.energy_sweep(h, x, e, (0.0, 0.0), 1e-3, 1, 1, opt)
        assert abs(r["T12"] - want) < 1e-4, (e, r["T12"])
    for ct, (npy, npz), es in ((3, (4, 1), (-0.6, 0.8)), (1, (2, 2), (-20.0,)), (0, (3, 2), (0.4,))):
        h, x = O.build_hamiltonian_reference(5, npy, npz, channel_type=ct)
        opt = O.SolveOptions(eta=1e-7, sr_tol=1e-12, norb=O.channel_norb(ct))
        for e in es:
            t = O.energy_sweep(h, x, e, (0.0, 0.0), 1e-3, npy, npz, opt)["T12"]
            assert t > 0.5 and abs(t - round(t)) < 1e-4, (ct, e, t)


def test_spin_and_pairing_matrices_follow_the_orbital_count():
    """Read_In_Allocate.F90: Nh = 2 uses the Pauli matrices for gMx, gMy, gMz and
    [[0, 1], [-1, 0]] for gDS; Nh = 1 leaves them zero."""
    sx, sy, sz = O.reference_spin_matrices(2)
    assert np.array_equal(sx @ sy - sy @ sx, 2j * sz)
    assert all(not g.any() for g in O.reference_spin_matrices(1))
    assert np.array_equal(O.reference_gds(2), np.array([[0, 1], [-1, 0]], dtype=complex))
    assert np.array_equal(O.reference_spin_matrices(4)[0], O.reference_gamma_matrices()[4])


def test_surface_model_josephson_current_is_odd_in_the_phase():
    """Superconducting contacts on the two-orbital TI surface (channelType 3, BdG with
    Nh = 2: gDS = [[0, 1], [-1, 0]], Read_In_Allocate.F90:214-215): the spectral supercurrent
    of Calculate_Observables.F90:60-81 vanishes at chi = 0 and pi and is odd in chi."""
    h, x = O.build_hamiltonian_reference(6, 3, 1, channel_type=3)
    hb, xb = O.bdg_hamiltonian(h, x, 3, 1, nh=2)

    def t12(chi, e):
        opt = O.SolveOptions(eta=1e-5, sr_tol=1e-10, norb=4, contact_type=3, chi_lr=chi)
        return O.energy_sweep(hb, xb, e, (0.0, 0.0), 1e-4, 3, 1, opt)["T12"]

    for e in (-5e-4, 7e-4):
        plus, minus = t12(0.3, e), t12(-0.3, e)
        assert abs(plus) > 1e-5
        assert abs(plus + minus) <= 1e-9 * abs(plus)
        assert abs(t12(0.0, e)) <= 1e-12 and abs(t12(np.pi, e)) <= 1e-12
