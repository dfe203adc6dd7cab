"""Model-0 topological-insulator nanowire Hamiltonian (the solve's input producer).

The reference builds Htotd (M x M x Npx) and HopX (M x M) in Build_Hamiltonian
(Source/Build_Hamiltonian.F90:13-18,59-100) on the MPI root.  This module builds the same
arrays on the host with NumPy for the wire the benchmarks use:

    on-site  (M0 - 6B) tau_z sigma_0 + V_i + Z tau_0 sigma_z
    hop_j    B tau_z sigma_0 - (i A / 2) tau_x sigma_j        (j = x, y, z)

in the tau (x) sigma basis (orbital = 2*tau + sigma), or, with ``basis="reference"``,
the reference's own Dirac matrices g0..g3 (Source/Read_In_Allocate.F90:161-181) with
AA = (MM - 3/a0^2) g0 and Hop_j = (g0/a0^2 - i g_j/a0)/2.

Layout conventions follow the reference: in-slice orbital index
orb + y*norb + z*norb*npy (Source/Build_Hamiltonian.F90:160); the y-hop carries the
Aharonov-Bohm phase exp(i 2 pi z Phi / ((npy-1)(npz-1))) (Landau gauge,
Source/Build_Hamiltonian.F90:186-207); Anderson disorder is added on slices 2..npx-1
only (Source/Build_Hamiltonian.F90:279-296), so the end slices equal the leads.
Arrays are returned slice-first: htotd[x, row, col], hopx[row, col].
"""
from __future__ import annotations

import math

import numpy as np

NORB = 4

_s0 = np.eye(2, dtype=complex)
_sx = np.array([[0, 1], [1, 0]], dtype=complex)
_sy = np.array([[0, -1j], [1j, 0]], dtype=complex)
_sz = np.array([[1, 0], [0, -1]], dtype=complex)


# the reference's Dirac matrices g0..g3 for four orbitals (Source/Read_In_Allocate.F90:161-181)
_G0 = np.diag([1.0, 1.0, -1.0, -1.0]).astype(complex)
_G1 = np.array([[0, 0, 0, -1j], [0, 0, 1j, 0], [0, -1j, 0, 0], [1j, 0, 0, 0]], dtype=complex)
_G2 = np.array([[0, 0, 0, -1], [0, 0, -1, 0], [0, -1, 0, 0], [-1, 0, 0, 0]], dtype=complex)
_G3 = np.array([[0, 0, -1j, 0], [0, 0, 0, -1j], [1j, 0, 0, 0], [0, 1j, 0, 0]], dtype=complex)


def tau_sigma(t, s):
    return np.kron(t, s)


def spin_operators():
    """tau_0 sigma_{x,y,z}: the spin operators gMx, gMy, gMz (Source/Read_In_Allocate.F90:183-196)."""
    return tau_sigma(_s0, _sx), tau_sigma(_s0, _sy), tau_sigma(_s0, _sz)


def site_blocks(M0=0.3, B=0.25, A=0.5, zeeman=0.0, basis="tau_sigma"):
    """(onsite, hop_x, hop_y, hop_z) 4x4 blocks."""
    if basis == "tau_sigma":
        tz = tau_sigma(_sz, _s0)
        onsite = (M0 - 6.0 * B) * tz + zeeman * tau_sigma(_s0, _sz)
        hops = [B * tz - 0.5j * A * tau_sigma(_sx, s) for s in (_sx, _sy, _sz)]
        return onsite, hops[0], hops[1], hops[2]
    if basis == "reference":
        mm, a0 = 1.5, 1.0
        onsite = (mm - 3.0 / (a0 * a0)) * _G0 + zeeman * tau_sigma(_s0, _sz)
        hops = [0.5 * (_G0 / (a0 * a0) - 1j / a0 * g) for g in (_G1, _G2, _G3)]
        return onsite, hops[0], hops[1], hops[2]
    raise ValueError("basis must be 'tau_sigma' or 'reference'")


# Bi2Se3 parameters (Source/NEGF_Module.F90:10-17, in eV, Angstrom).  The reference declares
# them REAL(8) but writes them as default-kind literals, so they hold the single-precision
# values of these decimals; the same values are used here.
BI2SE3 = {k: float(np.float32(v)) for k, v in
          dict(A1="2.26", A2="3.33", C="-0.0083", D1="5.74", D2="30.4", M="0.28", B1="6.86", B2="44.5").items()}

# orbitals per site of each channel model (Source/Read_In_Allocate.F90:51-65)
CHANNEL_NORB = {0: 4, 1: 4, 2: 1, 3: 2, 4: 2}


def channel_blocks(channel_type, a0=1.0, mu_t=0.0, t_met=1.0):
    """(onsite, hop_x, hop_y, hop_z) site blocks of the reference's channel models
    (Source/Build_Hamiltonian.F90:13-47), norb x norb with norb = CHANNEL_NORB[channel_type]:

        0  toy 3-D TI (norb 4):  (1.5 - 3/a0^2) g0 - mu_t,  hop_j = (g0/a0^2 - i g_j/a0) / 2
        1  Bi2Se3 (norb 4):      (C + (2 D1 + 4 D2)/a0^2) + (M - (2 B1 + 4 B2)/a0^2) g0,
                                 hop_x,y = i A2/(2 a0) g_1,2 - D2/a0^2 + B2/a0^2 g0,
                                 hop_z   = i A1/(2 a0) g3    - D1/a0^2 + B1/a0^2 g0
        2  one-band metal (1):   6 t,  hop_j = -t
        3  TI surface (2):       0,  hop_x = -i sigma_y / 2,  hop_y = i sigma_x / 2,  hop_z = 0
        4  1-D SOC wire (2):     -mu_t,  hop_x = -i sigma_y / 2,  hop_y = hop_z = 0

    g0..g3 are the reference's Dirac matrices for norb 4 (Source/Read_In_Allocate.F90:161-181);
    for norb 2 its g1, g2, g3 are the Pauli matrices (:205-213).  Model 3 needs npz = 1 and
    model 4 npy = npz = 1 (Source/Read_In_Allocate.F90:53-60)."""
    if channel_type not in CHANNEL_NORB:
        raise ValueError("channel_type must be 0..4")
    n = CHANNEL_NORB[channel_type]
    ident = np.eye(n, dtype=complex)
    zero = np.zeros((n, n), dtype=complex)
    g0, g1, g2, g3 = _G0, _G1, _G2, _G3
    if channel_type == 0:
        onsite = (1.5 - 3.0 / (a0 * a0)) * g0 - mu_t * ident
        hx, hy, hz = (0.5 * (g0 / (a0 * a0) - 1j / a0 * g) for g in (g1, g2, g3))
        return onsite, hx, hy, hz
    if channel_type == 1:
        p = BI2SE3
        onsite = (p["C"] + (2.0 * p["D1"] + 4.0 * p["D2"]) / (a0 * a0)) * ident \
            + (p["M"] - (2.0 * p["B1"] + 4.0 * p["B2"]) / (a0 * a0)) * g0
        hy = p["A2"] / (2.0 * a0) * 1j * g2 - p["D2"] / (a0 * a0) * ident + p["B2"] / (a0 * a0) * g0
        hz = p["A1"] / (2.0 * a0) * 1j * g3 - p["D1"] / (a0 * a0) * ident + p["B1"] / (a0 * a0) * g0
        hx = p["A2"] / (2.0 * a0) * 1j * g1 - p["D2"] / (a0 * a0) * ident + p["B2"] / (a0 * a0) * g0
        return onsite, hx, hy, hz
    if channel_type == 2:
        return 6.0 * t_met * ident, -t_met * ident, -t_met * ident, -t_met * ident
    if channel_type == 3:
        return zero, -0.5j * _sy, 0.5j * _sx, zero.copy()
    return -mu_t * ident, -0.5j * _sy, zero, zero.copy()


def channel_model(channel_type, a0=1.0, mu_t=0.0, t_met=1.0, flux=0.0, W=0.0, seed=0, V=None):
    """negf_build_hamiltonian parameters of channel model ``channel_type`` (channel_blocks);
    build the handle with norb = CHANNEL_NORB[channel_type]."""
    onsite, hx, hy, hz = channel_blocks(channel_type, a0, mu_t, t_met)
    return dict(onsite=onsite, hops=(hx, hy, hz), flux=float(flux), W=float(W), seed=int(seed), V=V)


def disorder_potential(npx, npy, npz, W, seed):
    """Uniform V in [-W/2, W/2] per site on slices 2..npx-1 (zero on the end slices),
    drawn in (x, y, z) order from numpy's PCG64 seeded with ``seed``."""
    v = np.zeros((npx, npy, npz))
    if W != 0.0 and npx > 2:
        rng = np.random.Generator(np.random.PCG64(seed))
        v[1:npx - 1] = (rng.random((npx - 2, npy, npz)) - 0.5) * W
    return v


def ti_wire(npx, npy, npz, M0=0.3, B=0.25, A=0.5, zeeman=0.0, flux=0.0, W=0.0, seed=0,
            basis="tau_sigma", disorder=None):
    """Build (htotd[npx, M, M], hopx[M, M]) complex128 for an open-boundary wire.

    ``flux`` is the Aharonov-Bohm flux through the cross-section in units of Phi_0;
    ``W``/``seed`` give Anderson disorder unless an explicit ``disorder`` array
    (npx, npy, npz) is passed.
    """
    onsite, hx, hy, hz = site_blocks(M0, B, A, zeeman, basis)
    nsite = npy * npz
    m = NORB * nsite
    h = np.zeros((m, m), dtype=complex)
    hopx = np.zeros((m, m), dtype=complex)

    def sl(y, z):
        i = (y + z * npy) * NORB
        return slice(i, i + NORB)

    for z in range(npz):
        for y in range(npy):
            s = sl(y, z)
            h[s, s] = onsite
            hopx[s, s] = hx
            if y + 1 < npy:
                t = sl(y + 1, z)
                blk = hy
                if flux != 0.0 and npy > 1 and npz > 1:
                    blk = hy * np.exp(1j * 2.0 * np.pi * z * flux / ((npy - 1) * (npz - 1)))
                h[s, t] = blk
                h[t, s] = blk.conj().T
            if z + 1 < npz:
                t = sl(y, z + 1)
                h[s, t] = hz
                h[t, s] = hz.conj().T
    htotd = np.repeat(h[None], npx, axis=0)
    if disorder is None:
        disorder = disorder_potential(npx, npy, npz, W, seed)
    if np.any(disorder != 0.0):
        # v[x, y, z] on the diagonal of site (y, z): orbital index (y + z*npy)*NORB + orb
        diag = np.repeat(disorder.transpose(0, 2, 1).reshape(npx, nsite), NORB, axis=1)
        idx = np.arange(m)
        htotd[:, idx, idx] += diag
    return htotd, hopx


# ---------------------------------------------------------------------------------------
# Counter-based wire model: the form negf_build_hamiltonian generates on the device
# ---------------------------------------------------------------------------------------
_GOLDEN_GAMMA = np.uint64(0x9E3779B97F4A7C15)
_MIX1 = np.uint64(0xBF58476D1CE4E5B9)
_MIX2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed, i):
    """Output ``i`` (array) of SplitMix64 seeded with ``seed`` (Steele, Lea, Flood 2014)."""
    with np.errstate(over="ignore"):
        z = np.uint64(seed) + np.asarray(i, dtype=np.uint64) * _GOLDEN_GAMMA
        z = (z ^ (z >> np.uint64(30))) * _MIX1
        z = (z ^ (z >> np.uint64(27))) * _MIX2
        return z ^ (z >> np.uint64(31))


def anderson_counter(npx, npy, npz, W, seed):
    """Anderson potential (u - 1/2) W on slices 2..npx-1 with u = (s >> 11) 2^-53, s the
    output x + npx (y + npy z) + 1 of SplitMix64(seed): the device's disorder stream."""
    x, y, z = np.meshgrid(np.arange(npx), np.arange(npy), np.arange(npz), indexing="ij")
    i = (x + npx * (y + npy * z)).astype(np.uint64) + np.uint64(1)
    u = (splitmix64(seed, i) >> np.uint64(11)).astype(np.float64) * 2.0 ** -53
    v = (u - 0.5) * W
    v[0] = 0.0
    v[npx - 1] = 0.0
    return v


def wire_model(M0=0.3, B=0.25, A=0.5, zeeman=0.0, flux=0.0, W=0.0, seed=0, basis="tau_sigma", V=None):
    """Parameters of negf_build_hamiltonian: the 4x4 site blocks plus flux, disorder
    (W, seed) and an optional site potential V (npx, npy, npz) added to the disorder."""
    onsite, hx, hy, hz = site_blocks(M0, B, A, zeeman, basis)
    return dict(onsite=onsite, hops=(hx, hy, hz), flux=float(flux), W=float(W), seed=int(seed), V=V)


def build_from_model(npx, npy, npz, model):
    """Host twin of negf_build_hamiltonian: (htotd[npx, M, M], hopx[M, M]) with the same
    arithmetic as the device path (the y-hop phase and its product with the block in plain
    float operations, the potential added once to the on-site diagonal), so the two are
    equal element for element.  The blocks are norb x norb (norb <= 4)."""
    onsite = np.asarray(model["onsite"], dtype=complex)
    hx, hy, hz = (np.asarray(h, dtype=complex) for h in model["hops"])
    norb = onsite.shape[0]
    nsite = npy * npz
    m = norb * nsite
    flux = model["flux"]
    phased = flux != 0.0 and npy > 1 and npz > 1
    hy_z = []
    for z in range(npz):
        if not phased:
            hy_z.append(hy.copy())
            continue
        th = 2.0 * math.pi * z * flux / ((npy - 1) * (npz - 1))
        c, s = math.cos(th), math.sin(th)
        blk = np.empty((norb, norb), dtype=complex)
        for a in range(norb):
            for b in range(norb):
                hr, hi = float(hy[a, b].real), float(hy[a, b].imag)
                blk[a, b] = complex(hr * c - hi * s, hr * s + hi * c)
        hy_z.append(blk)
    h = np.zeros((m, m), dtype=complex)
    hopx = np.zeros((m, m), dtype=complex)
    for z in range(npz):
        for y in range(npy):
            i = (y + z * npy) * norb
            s = slice(i, i + norb)
            h[s, s] = onsite
            hopx[s, s] = hx
            if y + 1 < npy:
                t = slice(i + norb, i + 2 * norb)
                h[s, t] = hy_z[z]
                h[t, s] = hy_z[z].conj().T
            if z + 1 < npz:
                t = slice(i + norb * npy, i + norb * npy + norb)
                h[s, t] = hz
                h[t, s] = hz.conj().T
    v = anderson_counter(npx, npy, npz, model["W"], model["seed"])
    if model.get("V") is not None:
        v = np.asarray(model["V"], dtype=np.float64) + v      # the device adds V + disorder
    htotd = np.repeat(h[None], npx, axis=0)
    diag = np.repeat(np.asarray(v).transpose(0, 2, 1).reshape(npx, nsite), norb, axis=1)
    idx = np.arange(m)
    htotd[:, idx, idx] = (htotd[:, idx, idx].real + diag) + 1j * htotd[:, idx, idx].imag
    return htotd, hopx


def bdg(htotd, hopx, npy, npz, nh=NORB):
    """BdG form of a wire for superconducting contacts: every nh x nh site-pair block H_e
    of Htotd and HopX becomes [[H_e, 0], [0, -conj(H_e)]] on 2 nh orbitals per site, electron
    orbitals first (Source/Read_In_Allocate.F90:69-71, Build_Hamiltonian.F90:52-56,
    162-163, 199-200).  Returns (htotd[npx, 2M, 2M], hopx[2M, 2M])."""
    htotd = np.asarray(htotd, dtype=np.complex128)
    hopx = np.asarray(hopx, dtype=np.complex128)
    nsite = npy * npz
    no = 2 * nh
    e_idx = (np.arange(nsite)[:, None] * no + np.arange(nh)[None, :]).ravel()   # electron rows
    h_idx = e_idx + nh                                                           # their holes
    m2 = nsite * no

    def one(blk):
        out = np.zeros((m2, m2), dtype=np.complex128)
        out[np.ix_(e_idx, e_idx)] = blk
        out[np.ix_(h_idx, h_idx)] = -np.conj(blk)
        return out
    return np.stack([one(b) for b in htotd]), one(hopx)
