"""CPU oracle for the per-energy NEGF solve.

TEST INFRASTRUCTURE ONLY.  Nothing in the product path imports this module; it is the
checker that the CUDA path is compared against (tests/, ``__graft_entry__.smoke()`` and
the ``cpu_baseline`` / ``--impl reference`` legs of ``bench.py``).

It restates, in NumPy complex128 with LAPACK ``zgetrf``/``zgetri`` (the routines the
reference calls through MKL), the reference's per-energy path:

    Source/Energy_Sweep.F90:1-46            energy_sweep()
    Source/Contact_Self_Energy.F90:1-106    contact_self_energy()
    Source/Contact_Self_Energy.F90:110-223  sancho_rubio()
    Source/MKL_Routines_Cluster.F90:2-33    invert_matrix()
    Source/Recursive_Greens.F90:2-107       get_retarded_greens()
    Source/Calculate_Gnp.F90:1-136          calculate_gnp()
    Source/Calculate_Observables.F90:2-169  calculate_observables()
    Source/Build_Hamiltonian.F90:1-207      build_hamiltonian_reference() (channel models 0-4)
    Source/Build_Hamiltonian.F90:13-47      channel_blocks(); Read_In_Allocate.F90:51-65 channel_norb()
    Source/NEGF_Module.F90:7,10-17          Bi2Se3 parameters and tMet
    Source/Build_Hamiltonian.F90:52-56,162-163,199-200   bdg_hamiltonian()
    Source/Read_In_Allocate.F90:151-216     gamma, spin and pairing matrices for Nh = 4, 2, 1

The algorithm follows the reference step by step: the backward GRd/GRu/GRl recursion
is kept, Gn/Gp are formed as full blocks, and the same zgemm products are taken in
the same order.  The reference's naive quadruple loops in Calculate_Gnp are written
here as matrix products of the same operands, so results differ from a literal loop
only by floating-point summation order.

Parity status: UNPINNED against the reference executable.  The reference is Fortran 90
+ MKL + MPI; no Fortran compiler exists in the build container or on the GPU host, and
the reference ships no tests, golden vectors or fixtures.  The oracle is pinned instead
by (i) a dense inversion of the full (Npx*M)^2 matrix, (ii) physics invariants (integer
transmission of a clean wire, the exact open-mode count of the one-band metal and the two
channels of the 1-D spin-orbit wire, L<->R reciprocity, the A = Gn + Gp sum rule, the
surface Dyson equation of the lead self-energy, a Josephson current odd in the phase) and
(iii) committed golden vectors it generated (tests/golden/make_golden.py).

Reference quirks are exposed as parameters of ``SolveOptions``; the defaults are the
reference's own values (eta = 1e-4, Sancho-Rubio tolerance 1e-8, T=0 step occupations).
"""
from __future__ import annotations

import dataclasses
import math
from typing import Optional

import numpy as np
from scipy.linalg import lapack

# Source/Constants.F90:3-7
Q_E = 1.602e-19
H_PLANCK = 6.626e-34
PI = 4.0 * math.atan(1.0)
HBAR = H_PLANCK / (2.0 * PI)
ETA_SIGMA_REFERENCE = 1e-4


# ---------------------------------------------------------------------------
# Gamma / spin matrices, Source/Read_In_Allocate.F90:161-197 (Nh == 4)
# ---------------------------------------------------------------------------
def reference_gamma_matrices():
    """Return (g0, g1, g2, g3, gMx, gMy, gMz) exactly as Read_In_Allocate.F90:161-197."""
    c0, c1, ci = 0j, 1 + 0j, 1j
    g1 = np.array([[c0, c0, c0, -ci], [c0, c0, ci, c0], [c0, -ci, c0, c0], [ci, c0, c0, c0]])
    g2 = np.array([[c0, c0, c0, -c1], [c0, c0, -c1, c0], [c0, -c1, c0, c0], [-c1, c0, c0, c0]])
    g3 = np.array([[c0, c0, -ci, c0], [c0, c0, c0, -ci], [ci, c0, c0, c0], [c0, ci, c0, c0]])
    g0 = np.diag([c1, c1, -c1, -c1])
    gMx = np.array([[c0, c1, c0, c0], [c1, c0, c0, c0], [c0, c0, c0, c1], [c0, c0, c1, c0]])
    gMy = np.array([[c0, -ci, c0, c0], [ci, c0, c0, c0], [c0, c0, c0, -ci], [c0, c0, ci, c0]])
    gMz = np.diag([c1, -c1, c1, -c1])
    return g0, g1, g2, g3, gMx, gMy, gMz


def reference_spin_matrices(nh=4):
    """(gMx, gMy, gMz) for Nh electron orbitals per site: the Nh == 4 matrices of
    Read_In_Allocate.F90:183-196, the Pauli matrices g1, g2, g3 for Nh == 2 (:205-216), and
    for any other Nh the zero matrices the arrays are allocated as (:151-159)."""
    if nh == 4:
        return reference_gamma_matrices()[4:]
    if nh == 2:
        c0, c1, ci = 0j, 1 + 0j, 1j
        return (np.array([[c0, c1], [c1, c0]]), np.array([[c0, -ci], [ci, c0]]), np.array([[c1, c0], [c0, -c1]]))
    return tuple(np.zeros((nh, nh), dtype=complex) for _ in range(3))


def reference_gds(nh=4):
    """gDS, the pairing structure of the superconducting contacts: Read_In_Allocate.F90:199-202
    for Nh == 4, :214-215 for Nh == 2, zero otherwise."""
    c0, c1 = 0j, 1 + 0j
    if nh == 4:
        return np.array([[c0, c1, c0, c0], [-c1, c0, c0, c0], [c0, c0, c0, c1], [c0, c0, -c1, c0]])
    if nh == 2:
        return np.array([[c0, c1], [-c1, c0]])
    return np.zeros((nh, nh), dtype=complex)


# Bi2Se3 parameters, NEGF_Module.F90:10-17.  They are REAL(8) PARAMETERs initialised from
# default-kind (single precision) literals, so their values are the nearest floats of the
# decimals, widened to double.
MP_A1, MP_A2, MP_C, MP_D1, MP_D2, MP_M, MP_B1, MP_B2 = (
    float(np.float32(v)) for v in ("2.26", "3.33", "-0.0083", "5.74", "30.4", "0.28", "6.86", "44.5"))
T_MET = 1.0   # NEGF_Module.F90:7, tMet = 1D0


def channel_norb(channel_type):
    """Orbitals per site of a channel model, Read_In_Allocate.F90:51-65."""
    return {0: 4, 1: 4, 2: 1, 3: 2, 4: 2}[channel_type]


def channel_blocks(channel_type, a0=1.0, mu_t=0.0, t_met=T_MET):
    """(AA, HopX, HopY, HopZ) site blocks, Nh x Nh, of the channel models of
    Build_Hamiltonian.F90:13-47: 0 the toy TI, 1 Bi2Se3, 2 the one-band metal, 3 the TI
    surface state, 4 the 1-D wire with spin-orbit coupling.  Blocks the reference leaves
    unset stay at their zero initialisation (:8-11).  The Dirac matrices are those of
    Read_In_Allocate.F90 for the model's Nh (g0 = 0 and g1..g3 the Pauli matrices when
    Nh == 2, all zero when Nh == 1)."""
    nh = channel_norb(channel_type)
    c1, ci = 1 + 0j, 1j
    ident = np.eye(nh, dtype=complex)
    if nh == 4:
        g0, g1, g2, g3 = reference_gamma_matrices()[:4]
    else:
        g0 = np.zeros((nh, nh), dtype=complex)
        g1, g2, g3 = reference_spin_matrices(nh)   # Read_In_Allocate.F90:205-213: g1, g2, g3
    z = np.zeros((nh, nh), dtype=complex)
    if channel_type == 0:                                              # :13-18
        mm = 1.5
        aa = (mm - 3.0 / (a0 * a0)) * g0 - mu_t * ident
        hx = 0.5 * (c1 / (a0 * a0) * g0 - ci / a0 * g1)
        hy = 0.5 * (c1 / (a0 * a0) * g0 - ci / a0 * g2)
        hz = 0.5 * (c1 / (a0 * a0) * g0 - ci / a0 * g3)
    elif channel_type == 1:                                            # :19-33
        aa = (MP_C + (2.0 * MP_D1 + 4.0 * MP_D2) / (a0 * a0)) * ident \
            + (MP_M - (2.0 * MP_B1 + 4.0 * MP_B2) / (a0 * a0)) * g0
        hy = MP_A2 / (2.0 * a0) * ci * g2 - MP_D2 / (a0 * a0) * ident + MP_B2 / (a0 * a0) * g0
        hz = MP_A1 / (2.0 * a0) * ci * g3 - MP_D1 / (a0 * a0) * ident + MP_B1 / (a0 * a0) * g0
        hx = MP_A2 / (2.0 * a0) * ci * g1 - MP_D2 / (a0 * a0) * ident + MP_B2 / (a0 * a0) * g0
    elif channel_type == 2:                                            # :34-38
        aa = np.full((1, 1), 6.0 * t_met, dtype=complex)
        hx = hy = hz = np.full((1, 1), -t_met, dtype=complex)
    elif channel_type == 3:                                            # :39-43
        aa, hz = z, z
        hy = 0.5 * ci * g1
        hx = -0.5 * ci * g2
    elif channel_type == 4:                                            # :44-47
        aa = (-mu_t) * ident
        hx = -ci * 0.5 * g2
        hy = hz = z
    else:
        raise ValueError("channelType must be in 0..4")
    return aa, hx, hy, hz


# ---------------------------------------------------------------------------
# Hamiltonian, model 0 (channelType == 0), Source/Build_Hamiltonian.F90
# ---------------------------------------------------------------------------
def build_hamiltonian_reference(npx, npy, npz, a0=1.0, mu_t=0.0, ab_phi=0.0, bcy=0, bcz=0,
                                disorder=None, onsite_blocks=None, hops=None, channel_type=0):
    """Slice Hamiltonian of channel model ``channel_type`` (``channel_blocks``), following
    Build_Hamiltonian.F90:13-47,59-100,154-207.  Read_In_Allocate.F90:53-60 forces Npz = 1
    for model 3 and Npy = Npz = 1 for model 4 (and open boundaries); they are required here.

    ``disorder`` is an optional real array (npx, npy, npz) of on-site potentials added by
    Insert_Impurity (Build_Hamiltonian.F90:154-165); the reference only fills slices
    2..npx-1 (Build_Hamiltonian.F90:279-296) and the caller is expected to do the same.
    ``onsite_blocks``/``hops`` override the 4x4 AA and (HopX, HopY, HopZ) blocks; by
    default they are the reference's own (MM = 1.5, Build_Hamiltonian.F90:14-18).
    Returns (Htotd[npx, M, M], HopX[M, M]) as complex128, slice index first.
    """
    norb = channel_norb(channel_type)
    if (channel_type == 3 and npz != 1) or (channel_type == 4 and (npy != 1 or npz != 1)):
        raise ValueError("channel model %d needs Npz = 1 (3) or Npy = Npz = 1 (4)" % channel_type)
    ident = np.eye(norb, dtype=complex)
    aa, hx, hy, hz = channel_blocks(channel_type, a0, mu_t)
    if onsite_blocks is not None:
        aa = np.asarray(onsite_blocks, dtype=complex)
    if hops is not None:
        hx, hy, hz = (np.asarray(h, dtype=complex) for h in hops)
    nn = npy * norb
    m = npz * nn
    # Build_Hamiltonian.F90:59-64: HopZ is block diagonal over y, HopX over (y, z)
    hopz_full = np.zeros((nn, nn), dtype=complex)
    for yy in range(npy):
        hopz_full[yy * norb:(yy + 1) * norb, yy * norb:(yy + 1) * norb] = hz
    hopx = np.zeros((m, m), dtype=complex)
    for s in range(npy * npz):
        hopx[s * norb:(s + 1) * norb, s * norb:(s + 1) * norb] = hx
    # :66-79 intraslice y chain
    hh1d = np.zeros((nn, nn), dtype=complex)
    for yy in range(npy - 1):
        hh1d[norb * yy:norb * (yy + 1), norb * yy:norb * (yy + 1)] = aa
        hh1d[norb * yy:norb * (yy + 1), norb * (yy + 1):norb * (yy + 2)] = hy
        hh1d[norb * (yy + 1):norb * (yy + 2), norb * yy:norb * (yy + 1)] = hy.conj().T
    hh1d[nn - norb:nn, nn - norb:nn] = aa
    if bcy == 1:
        hh1d[0:norb, nn - norb:nn] = hy.conj().T
        hh1d[nn - norb:nn, 0:norb] = hy
    # :82-94 z stacking
    hh2d = np.zeros((m, m), dtype=complex)
    for zz in range(npz - 1):
        hh2d[zz * nn:(zz + 1) * nn, zz * nn:(zz + 1) * nn] = hh1d
        hh2d[zz * nn:(zz + 1) * nn, (zz + 1) * nn:(zz + 2) * nn] = hopz_full
        hh2d[(zz + 1) * nn:(zz + 2) * nn, zz * nn:(zz + 1) * nn] = hopz_full.conj().T
    hh2d[m - nn:m, m - nn:m] = hh1d
    if bcz == 1:
        hh2d[0:nn, nn * (npz - 1):nn * npz] = hopz_full.conj().T
        hh2d[nn * (npz - 1):nn * npz, 0:nn] = hopz_full
    htotd = np.repeat(hh2d[None, :, :], npx, axis=0)
    # :186-207 Aharonov-Bohm phase on the y hops (Landau gauge)
    if ab_phi > 1e-10:
        for zz in range(1, npz + 1):
            phase = np.exp(1j * 2.0 * PI * float(zz - 1) * ab_phi / float(npy - 1) / float(npz - 1))
            for xx in range(npx):
                for yy in range(1, npy):
                    idx = (yy - 1) * norb + (zz - 1) * nn
                    blk = htotd[xx, idx:idx + norb, idx + norb:idx + 2 * norb] * phase
                    htotd[xx, idx:idx + norb, idx + norb:idx + 2 * norb] = blk
                    htotd[xx, idx + norb:idx + 2 * norb, idx:idx + norb] = blk.conj().T
    # :154-165 Insert_Impurity (on-site potential times identity on the site block)
    if disorder is not None:
        for xx in range(npx):
            for yy in range(npy):
                for zz in range(npz):
                    v = disorder[xx, yy, zz]
                    if v != 0.0:
                        idx = yy * norb + zz * nn
                        htotd[xx, idx:idx + norb, idx:idx + norb] += v * ident
    return htotd, hopx


def bdg_hamiltonian(htotd, hopx, npy, npz, nh=4):
    """The BdG form of an Nh-orbital Hamiltonian for superconducting contacts
    (Read_In_Allocate.F90:69-71: Norb = 2 Nh): every Nh x Nh site-pair block H_e of Htotd
    and HopX becomes the Norb x Norb block [[H_e, 0], [0, -conj(H_e)]]
    (Build_Hamiltonian.F90:52-56 for the unit-cell blocks, :162-163 after an impurity,
    :199-200 after the Aharonov-Bohm phase).  Site blocks keep the in-slice order
    orb + y Norb + z Npy Norb with the electron orbitals first."""
    nsite = npy * npz
    no = 2 * nh

    def conv(blk):
        e = blk.reshape(nsite, nh, nsite, nh)
        out = np.zeros((nsite, no, nsite, no), dtype=complex)
        out[:, :nh, :, :nh] = e
        out[:, nh:, :, nh:] = -np.conj(e)
        return out.reshape(nsite * no, nsite * no)
    return np.stack([conv(b) for b in htotd]), conv(hopx)


# ---------------------------------------------------------------------------
# Options (reference quirks as switches)
# ---------------------------------------------------------------------------
@dataclasses.dataclass
class SolveOptions:
    """Per-run switches.  Defaults are the reference's own values."""
    eta: float = ETA_SIGMA_REFERENCE        # Source/Constants.F90:7
    sr_tol: float = 1e-8                     # Source/Contact_Self_Energy.F90:154
    sr_max_iter: int = 20000                 # Source/Contact_Self_Energy.F90:154,202
    kT: float = 0.0                          # 0 -> T=0 step, Source/Energy_Sweep.F90:11-21
    calc_spin: bool = False                  # calcSigExp, Source/Read_In_Allocate.F90:93
    norb: int = 4
    # contactType (Source/Read_In_Allocate.F90:19): 0 semi-infinite leads, 1/2 phenomenological
    # (Contact_Self_Energy.F90:19-28), 3 superconducting with a BdG Hamiltonian (:29-67)
    contact_type: int = 0
    tunneling_rate: float = 1.0              # Contact_Self_Energy.F90:10
    delta_sc: tuple = (1e-3, 1e-3)           # DeltaSCL, DeltaSCR, Read_In_Allocate.F90:74-75
    chi_lr: float = 0.8                      # Read_In_Allocate.F90:72
    gds: Optional[np.ndarray] = None         # None -> reference_gds()
    # The reference's Sancho-Rubio iteration counter is an implicitly SAVEd local,
    # ``INTEGER(4) :: counter=1`` (Contact_Self_Energy.F90:119): it is initialised once per
    # process and every iteration of every call increments it (:155), so the loop test
    # ``counter <= 20000`` (:154) caps the iterations of the whole process, not of one call.
    # None (default): a counter per call, the cap sr_max_iter per call.  An SrCounter:
    # the reference's process-wide counter, shared by every call given the same object.
    sr_counter: Optional["SrCounter"] = None

    @property
    def nh(self) -> int:
        """Electron orbitals per site: Norb, or half of it for the BdG Hamiltonian
        (Read_In_Allocate.F90:67-71)."""
        return self.norb // 2 if self.contact_type == 3 else self.norb


@dataclasses.dataclass
class SrCounter:
    """The reference's SAVEd Sancho-Rubio counter (Contact_Self_Energy.F90:119,154-155).

    ``value`` starts at 1 as in the reference and keeps its value between calls.  Once the
    iterations of all calls so far have taken it past 20000, the loop body of every later
    call is skipped: CapT stays t (the first term of Eq. 16, :151) and Sigma is formed from
    it without decimation.  A single-process run reaches this after about 20000 / (2 n_SR)
    energies (about 400-500 at n_SR = 20-25); the reference's 72-rank production run gives
    each rank about 9 energies and never does.  The cap test ``counter == 20000`` (:202)
    can fire only when a call converges exactly at that count."""
    value: int = 1


def fermi(energy: float, mu_c: float, kT: float) -> float:
    """Occupation of a lead.  kT == 0 is the reference's step ``energy <= mu_c``
    (Source/Energy_Sweep.F90:11-21, with mu_c = muT - mu(c)); kT > 0 is Fermi-Dirac."""
    if kT <= 0.0:
        return 1.0 if energy <= mu_c else 0.0
    x = (energy - mu_c) / kT
    if x > 700:
        return 0.0
    return 1.0 / (1.0 + math.exp(x))


# ---------------------------------------------------------------------------
# Dense LA, Source/MKL_Routines_Cluster.F90:2-33
# ---------------------------------------------------------------------------
def invert_matrix(g: np.ndarray):
    """ZGETRF then, if INFO == 0, ZGETRI.  Returns (inverse, info)."""
    lu, piv, info = lapack.zgetrf(np.asfortranarray(g))
    if info != 0:
        return lu, int(info)
    inv, info2 = lapack.zgetri(lu, piv)
    return inv, int(info2)


# ---------------------------------------------------------------------------
# Sancho-Rubio, Source/Contact_Self_Energy.F90:110-223
# ---------------------------------------------------------------------------
def sancho_rubio(alpha: np.ndarray, beta: np.ndarray, eta: float, tol: float, max_iter: int,
                 counter_state: Optional[SrCounter] = None):
    """Lopez-Sancho/Rubio decimation.  Returns (Sigma, error_flag, iterations).

    Without ``counter_state`` the iteration counter is local to the call and max_iter caps
    each call.  With it, the counter is the reference's SAVEd one (Contact_Self_Energy.F90:
    119): it starts from ``counter_state.value``, is stored back at the end, and the cap
    max_iter applies to the sum over all calls sharing the state (see SrCounter).
    """
    nn = alpha.shape[0]
    ident = np.eye(nn, dtype=complex)
    betad = beta.conj().T
    # :141 tmp = inv(alpha + i*eta) (an extra i*eta on top of the one in alpha)
    tmp, err = invert_matrix(alpha + ident * complex(0.0, eta))
    t = -tmp @ betad                    # :147
    tt = -tmp @ beta                    # :149
    cap_t = t.copy()                    # :151
    toldt = ident.copy()                # :152
    change_max = 1.0                    # change initialised to c1, :135
    counter = 1 if counter_state is None else counter_state.value
    counter0 = counter
    while counter <= max_iter and change_max > tol:       # :154
        counter += 1
        toldt = toldt @ tt                                  # :157-158
        cmat1 = ident - t @ tt - tt @ t                     # :160-162
        tmp, err = invert_matrix(cmat1)                     # :163
        if err:
            raise RuntimeError("Sancho_Rubio: singular inv(Id - t*tt - tt*t)")  # :164-167 STOP
        t = (tmp @ t) @ t                                   # :170-172
        tt = (tmp @ tt) @ tt                                # :174-176
        change = toldt @ t                                  # :178
        cap_t = cap_t + change                              # :180
        abs_change = np.abs(change)
        if np.isnan(abs_change).any():                      # :182-191
            if counter_state is not None:
                counter_state.value = counter
            return None, 1, counter - counter0
        change_max = float(abs_change.max())
    if counter_state is not None:
        counter_state.value = counter
    cmat1 = beta @ cap_t + alpha                            # :195-196
    gfinal, err = invert_matrix(cmat1)                      # :197
    if counter == max_iter:                                 # :202-205
        err = 1
    sigma = (beta @ gfinal) @ beta.conj().T                 # :208-209
    return sigma, err, counter - counter0


# ---------------------------------------------------------------------------
# Contact_Self_Energy (contactType 0), Source/Contact_Self_Energy.F90:1-106
# ---------------------------------------------------------------------------
def contact_self_energy(htotd, hopx, energy, opt: SolveOptions, npy=None):
    """Returns dict with SigmaL, SigmaR, GammaL, GammaR, dosc (2,), sr_err (2,), sr_iters (2,).
    ``npy`` is needed by contact type 2 only."""
    npx, m, _ = htotd.shape
    ident = np.eye(m, dtype=complex)
    ce = complex(energy, opt.eta)                           # :16
    if opt.contact_type in (1, 2, 3):
        if opt.contact_type == 2 and npy is None:
            raise ValueError("contact type 2 needs npy")
        sig_l, sig_r = model_contact_self_energy(m, npy, ce, opt)
        return _finish_contacts(sig_l, sig_r, np.zeros(2, dtype=int), np.zeros(2, dtype=int))
    alpha = -htotd[0] + ident * ce                          # :71-74
    sig_l, err_l, it_l = sancho_rubio(alpha, -hopx.conj().T, opt.eta, opt.sr_tol, opt.sr_max_iter,
                                      opt.sr_counter)
    alpha = -htotd[npx - 1] + ident * ce                    # :83-86
    sig_r, err_r, it_r = sancho_rubio(alpha, -hopx, opt.eta, opt.sr_tol, opt.sr_max_iter, opt.sr_counter)
    if sig_l is None or sig_r is None:
        raise FloatingPointError("Sancho_Rubio produced NaN")
    return _finish_contacts(sig_l, sig_r, np.array([err_l, err_r]), np.array([it_l, it_r]))


def _finish_contacts(sig_l, sig_r, err, iters):
    dosc = np.array([-np.imag(np.trace(sig_l)) / PI, -np.imag(np.trace(sig_r)) / PI])  # :94-97
    gam_l = 1j * (sig_l - sig_l.conj().T)                   # :100
    gam_r = 1j * (sig_r - sig_r.conj().T)                   # :101
    return dict(SigmaL=sig_l, SigmaR=sig_r, GammaL=gam_l, GammaR=gam_r, dosc=dosc, sr_err=err, sr_iters=iters)


def model_contact_self_energy(m, npy, ce, opt: SolveOptions):
    """Self-energies of the contact models that need no decimation
    (Contact_Self_Energy.F90:19-67); ce = E + i eta_sigma (:16).
      1: -i rate on every orbital of the end slice (:19-23);
      2: the same on the first NN = Npy*Norb orbitals only (:24-28);
      3: superconducting contacts on a BdG Hamiltonian, the same Norb x Norb block on every
         site (:29-67): omega = 1/sqrt(DeltaSCL^2 - ce^2) (the right contact also uses
         DeltaSCL here, :49), -rate omega ce on both diagonal Nh x Nh blocks,
         rate omega (+-Delta) gDS off the diagonal, times exp(+-i chi) on the left contact
         only."""
    rate = opt.tunneling_rate
    if opt.contact_type in (1, 2):
        sig = np.zeros((m, m), dtype=complex)
        k = m if opt.contact_type == 1 else npy * opt.norb
        sig[np.arange(k), np.arange(k)] = -1j * rate
        return sig, sig.copy()
    nh, no = opt.nh, opt.norb
    gds = reference_gds(opt.nh) if opt.gds is None else np.asarray(opt.gds, dtype=complex)
    ident = np.eye(nh, dtype=complex)
    out = []
    for side in (0, 1):
        omega = 1.0 / np.sqrt(complex(opt.delta_sc[0]) ** 2 - ce ** 2)      # :33, :49
        m_alpha = -rate * omega * ce                                         # :35, :51
        d_up = rate * omega * opt.delta_sc[side]                             # :36, :52
        d_lo = rate * omega * (-opt.delta_sc[side])                          # :37, :53
        ph = np.exp(1j * opt.chi_lr) if side == 0 else 1.0                   # :43-44
        blk = np.zeros((no, no), dtype=complex)
        blk[:nh, :nh] = m_alpha * ident                                      # :40-41
        blk[nh:, nh:] = m_alpha * ident
        blk[:nh, nh:] = d_up * gds * ph                                      # :43
        blk[nh:, :nh] = d_lo * gds * np.conj(ph)                             # :44
        out.append(np.kron(np.eye(m // no), blk))                            # :63-67
    return out[0], out[1]


# ---------------------------------------------------------------------------
# Get_Retarded_Greens, Source/Recursive_Greens.F90:2-107
# ---------------------------------------------------------------------------
def get_retarded_greens(inv_grd, hopx):
    """inv_grd: (npx, M, M).  Returns dict with GRLef (npx, M, M) = G_{x,1},
    GRRgt (npx, M, M) = G_{x,N}, GRd, GRu, GRl and the error flags of the inverses."""
    npx, m, _ = inv_grd.shape
    mh = -hopx
    mhd = mh.conj().T
    ident = np.eye(m, dtype=complex)
    infos = []
    glr = np.empty_like(inv_grd)
    for i in range(npx):                                    # :16-34
        if i > 0:
            cmat1 = inv_grd[i] - (mhd @ glr[i - 1]) @ mh    # :18-20
        else:
            cmat1 = inv_grd[i]
        glr[i], info = invert_matrix(cmat1)                 # :26
        infos.append(info)
    grd = np.empty_like(inv_grd)
    gru = np.empty((max(npx - 1, 0), m, m), dtype=complex)
    grl = np.empty((max(npx - 1, 0), m, m), dtype=complex)
    grd[npx - 1] = glr[npx - 1]                             # :37
    for i in range(npx - 2, -1, -1):                        # :38-51
        grl[i] = (-(grd[i + 1] @ mhd)) @ glr[i]             # :40-41
        gru[i] = (-(glr[i] @ mh)) @ grd[i + 1]              # :43-44
        cmat1 = -(mh @ grl[i]) + ident                      # :46-49
        grd[i] = glr[i] @ cmat1                             # :50
    grrgt = np.zeros_like(inv_grd)                          # :53-63
    grrgt[npx - 1] = grd[npx - 1]
    if npx >= 2:
        grrgt[npx - 2] = gru[npx - 2]
    for ii in range(1, npx - 1):
        jj = npx - 1 - ii                                   # 1-based jj; block jj-1 <- block jj
        grrgt[jj - 1] = (-(glr[jj - 1] @ mh)) @ grrgt[jj]
    grr = np.empty_like(inv_grd)                            # :67-86
    for i in range(npx - 1, -1, -1):
        if i < npx - 1:
            cmat1 = inv_grd[i] - (mh @ grr[i + 1]) @ mhd
        else:
            cmat1 = inv_grd[i]
        grr[i], info = invert_matrix(cmat1)
        infos.append(info)
    grlef = np.zeros_like(inv_grd)                          # :88-96
    grlef[0] = grd[0]
    if npx >= 2:
        grlef[1] = grl[0]
    for i in range(0, npx - 1):
        grlef[i + 1] = (-(grr[i + 1] @ mhd)) @ grlef[i]     # :92-96 (the first pass overwrites GRl(1))
    return dict(GRLef=grlef, GRRgt=grrgt, GRd=grd, GRu=gru, GRl=grl, infos=np.array(infos))


# ---------------------------------------------------------------------------
# Calculate_Gnp, Source/Calculate_Gnp.F90:1-136
# ---------------------------------------------------------------------------
def calculate_gnp(grlef, grrgt, gam_l, gam_r, f1, f2, with_offdiag=True):
    """Gn/Gp diagonal (npx, M, M) and, optionally, the +-1 blocks (npx-1, M, M)."""
    npx = grlef.shape[0]
    out = {}
    for name, fa, fb in (("n", f1, f2), ("p", 1.0 - f1, 1.0 - f2)):
        c_l = fa * (grlef @ gam_l)                          # :12-18 / :64-70
        c_r = fb * (grrgt @ gam_r)                          # :37-43 / :90-96
        d = c_l @ grlef.conj().transpose(0, 2, 1) + c_r @ grrgt.conj().transpose(0, 2, 1)
        out["G%sd" % name] = d                              # :20-35 diagonal blocks
        if with_offdiag and npx > 1:
            out["G%su" % name] = (c_l[:-1] @ grlef[1:].conj().transpose(0, 2, 1)
                                  + c_r[:-1] @ grrgt[1:].conj().transpose(0, 2, 1))
            out["G%sl" % name] = (c_l[1:] @ grlef[:-1].conj().transpose(0, 2, 1)
                                  + c_r[1:] @ grrgt[:-1].conj().transpose(0, 2, 1))
    return out


def site_density(gd, npy, npz, norb=4):
    """Re diag(G?d) summed over the orbitals of each site -> (npx, npy, npz);
    index ii+(yy-1)*Norb+(zz-1)*NN as Calculate_Gnp.F90:118-124."""
    npx = gd.shape[0]
    diag = np.real(np.diagonal(gd, axis1=1, axis2=2))       # (npx, M)
    per_site = diag.reshape(npx, npz, npy, norb).sum(axis=3)  # in-slice index (orb, y, z), z slowest
    return per_site.transpose(0, 2, 1)                      # -> (x, y, z)


# ---------------------------------------------------------------------------
# Calculate_Observables, Source/Calculate_Observables.F90:2-169
# ---------------------------------------------------------------------------
def calculate_observables(gnp, grrgt, gam_l, gam_r, htotd, hopx, f1, f2, de, npy, npz,
                          calc_spin=False, calc_currents=True, norb=4, calc_resolved=False, nh=None,
                          bdg=False, sig_l=None, grd1=None):
    """``nh``: electron orbitals per site (Norb, or Norb/2 on a BdG Hamiltonian); the spin,
    EDensity/HDensity and current sums run over them only, as the reference's loops do.
    ``bdg``: the supercurrent transmission (:60-81) from Gnd(:,:,1), SigmaL, GRd(:,:,1) =
    ``grd1`` and GammaL instead of the Landauer trace."""
    npx = htotd.shape[0]
    nn = npy * norb
    nh = norb if nh is None else nh
    nsite = npy * npz
    res = {}
    gnd, gpd = gnp["Gnd"], gnp["Gpd"]
    gmx, gmy, gmz = reference_spin_matrices(nh)
    if calc_spin:                                           # :10-30
        # site blocks Gnd(idx+ii, idx+jj), ii, jj <= Nh, idx = y*Norb + z*NN, against gM(jj, ii)
        blocks = gnd.reshape(npx, nsite, norb, nsite, norb)
        diag_blocks = blocks[:, np.arange(nsite), :nh, np.arange(nsite), :nh]   # (nsite, npx, nh, nh)
        sig = np.zeros((3, npx, npy, npz))
        for j, gm in enumerate((gmx, gmy, gmz)):
            v = de / (2.0 * PI) * np.real(np.einsum("sxab,ba->xs", diag_blocks, gm[:nh, :nh]))
            sig[j] = v.reshape(npx, npz, npy).transpose(0, 2, 1)
        res["SigExp"] = sig
    # :33-43 electron/hole DOS at this energy (orbitals ii <= Nh of every site)
    dn = np.real(np.diagonal(gnd, axis1=1, axis2=2)).reshape(npx, nsite, norb)[:, :, :nh]
    dp = np.real(np.diagonal(gpd, axis1=1, axis2=2)).reshape(npx, nsite, norb)[:, :, :nh]
    res["EDensity"] = float(dn.sum() / (2.0 * PI))
    res["HDensity"] = float(dp.sum() / (2.0 * PI))
    # :46-53 injected modes
    res["Modec1"] = float(np.real(np.sum(gam_l * (gnd[0] + gpd[0]).T)))
    res["Modec2"] = float(np.real(np.sum(gam_r * (gnd[npx - 1] + gpd[npx - 1]).T)))
    if bdg:
        # :60-81 supercurrent transmission, PRB 62, 648 (2000) Eq. 14:
        # cmat1 = (i Gnd(:,:,1)) SigmaL^H, cmat2 = GRd(:,:,1) (-GammaL),
        # T12 = sum_ii sigma_z(ii) Re (cmat1 + cmat2)(ii, ii), +1 on electron orbitals
        cmat1 = (1j * gnd[0]) @ sig_l.conj().T
        cmat2 = grd1 @ (-gam_l)
        sz = np.where(np.arange(gnd.shape[1]) % norb < norb // 2, 1.0, -1.0)
        t12 = float(np.sum(sz * np.real(np.diagonal(cmat1 + cmat2))))
        res["T12"] = t12
        res["ContactCurrent"] = np.array([Q_E * de / H_PLANCK * t12, Q_E * de / H_PLANCK * (-t12)])  # :79-80
    else:
        # :85-100 transmission
        g1n = grrgt[0]
        cmat1 = gam_l @ g1n
        cmat2 = gam_r @ g1n.conj().T
        t12 = float(np.real(np.sum(cmat1 * cmat2.T)))
        res["T12"] = t12
        res["ContactCurrent"] = np.array([Q_E * de / H_PLANCK * (t12 * (f2 - f1)),
                                          Q_E * de / H_PLANCK * (t12 * (f1 - f2))])  # :102-103
    if calc_currents and "Gnu" in gnp:                      # :110-169, dumVar is REAL(4)
        j = np.zeros((3, npx, npy, npz))                    # Jx, Jy, Jz
        er = np.zeros((3, npx, npy, npz))                   # ERJx/y/z at this energy (:124-157)
        orj = np.zeros((3, npx, npy, npz, norb * norb))     # ORJx/y/z, pair (ii-1)*Norb+jj (:127-160)
        gnu, gnl, gpu_, gpl = gnp["Gnu"], gnp["Gnl"], gnp["Gpu"], gnp["Gpl"]
        pref = 1j * Q_E * Q_E / HBAR
        w = de / (2.0 * PI)
        for xx in range(npx):
            h = htotd[xx]
            for yy in range(npy):
                for zz in range(npz):
                    idx = yy * norb + zz * nn
                    a = slice(idx, idx + nh)                # orbitals ii <= Nh (:114-115)
                    terms = [None, None, None]
                    if yy < npy - 1:
                        b = slice(idx + norb, idx + norb + nh)
                        terms[1] = (h[a, b] * gnd[xx][b, a].T - gnd[xx][a, b] * h[b, a].T
                                    - h[a, b] * gpd[xx][b, a].T + gpd[xx][a, b] * h[b, a].T)
                    if zz < npz - 1:
                        b = slice(idx + nn, idx + nn + nh)
                        terms[2] = (h[a, b] * gnd[xx][b, a].T - gnd[xx][a, b] * h[b, a].T
                                    - h[a, b] * gpd[xx][b, a].T + gpd[xx][a, b] * h[b, a].T)
                    if xx < npx - 1:
                        hx = hopx[a, a]
                        terms[0] = (hx * gnl[xx][a, a].T - gnu[xx][a, a] * np.conj(hx)
                                    - hx * gpl[xx][a, a].T + gpu_[xx][a, a] * np.conj(hx))
                    for d, v in enumerate(terms):
                        if v is None:
                            continue
                        dum = np.float32(np.real(pref * v)).astype(np.float64)   # [ii, jj]
                        j[d, xx, yy, zz] = np.sum(dum * w)
                        er[d, xx, yy, zz] = np.sum(dum)
                        pairs = np.zeros((norb, norb))
                        pairs[:nh, :nh] = dum * w
                        orj[d, xx, yy, zz] = pairs.ravel()
        res["Jx"], res["Jy"], res["Jz"] = j
        if calc_resolved:
            res["ERJx"], res["ERJy"], res["ERJz"] = er
            res["ORJx"], res["ORJy"], res["ORJz"] = orj
    return res


def orbital_density(gd, npy, npz, norb=4):
    """Re diag(G?d) per orbital of each site -> (npx, npy, npz, norb) (ORRhon before its
    dE/(2 pi) weight, Calculate_Gnp.F90:128-129)."""
    npx = gd.shape[0]
    diag = np.real(np.diagonal(gd, axis1=1, axis2=2))       # (npx, M)
    return diag.reshape(npx, npz, npy, norb).transpose(0, 2, 1, 3)


# ---------------------------------------------------------------------------
# Energy_Sweep, Source/Energy_Sweep.F90:1-46
# ---------------------------------------------------------------------------
def energy_sweep(htotd, hopx, energy, mu_lead, de, npy, npz, opt: SolveOptions,
                 calc_currents=False, keep_blocks=False, calc_resolved=False):
    """One energy point.  ``mu_lead`` = (muT - mu(1), muT - mu(2)), the lead
    electrochemical potentials.  Returns a dict of per-energy results, with RhoN/RhoP
    and spin already weighted by dE/(2 pi) as the reference accumulates them."""
    npx, m, _ = htotd.shape
    f1 = fermi(energy, mu_lead[0], opt.kT)
    f2 = fermi(energy, mu_lead[1], opt.kT)
    cse = contact_self_energy(htotd, hopx, energy, opt, npy=npy)
    ident = np.eye(m, dtype=complex)
    inv_grd = -htotd + ident[None] * complex(energy, opt.eta)   # :31-36
    inv_grd[0] = inv_grd[0] - cse["SigmaL"]                     # :37
    inv_grd[npx - 1] = inv_grd[npx - 1] - cse["SigmaR"]         # :38
    rg = get_retarded_greens(inv_grd, hopx)
    gnp = calculate_gnp(rg["GRLef"], rg["GRRgt"], cse["GammaL"], cse["GammaR"], f1, f2,
                        with_offdiag=calc_currents)
    out = dict(energy=energy, f1=f1, f2=f2, dosc=cse["dosc"], sr_iters=cse["sr_iters"],
               sr_err=cse["sr_err"], rgf_infos=rg["infos"])
    out["RhoN"] = site_density(gnp["Gnd"], npy, npz, opt.norb) * (de / (2.0 * PI))
    out["RhoP"] = site_density(gnp["Gpd"], npy, npz, opt.norb) * (de / (2.0 * PI))
    obs = calculate_observables(gnp, rg["GRRgt"], cse["GammaL"], cse["GammaR"], htotd, hopx,
                                f1, f2, de, npy, npz, calc_spin=opt.calc_spin,
                                calc_currents=calc_currents, norb=opt.norb, calc_resolved=calc_resolved,
                                nh=opt.nh, bdg=opt.contact_type == 3, sig_l=cse["SigmaL"], grd1=rg["GRd"][0])
    out.update(obs)
    if calc_resolved:                                           # Calculate_Gnp.F90:125-129
        on = orbital_density(gnp["Gnd"], npy, npz, opt.norb)
        op = orbital_density(gnp["Gpd"], npy, npz, opt.norb)
        out["ERRhon"] = (on - op).sum(axis=3)
        out["ORRhon"] = on * (de / (2.0 * PI))
    if keep_blocks:
        out.update(cse)
        out.update(rg)
        out.update(gnp)
    return out


def energy_axis_reference(mu, mu_t, n_e=600):
    """Source/Read_In_Allocate.F90:248-259 (no Poisson, normal contacts)."""
    e_min = mu_t - max(mu) - 1e-10
    e_max = mu_t - min(mu) + 1e-10
    de = (e_max - e_min) / (n_e - 1)
    return e_min + de * np.arange(n_e), de


def energy_weights(eaxis, de0):
    """dE used at each energy: EAxis(e+1)-EAxis(e), except the last point which keeps
    the previous value (Source/Energy_Sweep.F90:7-9; deltaE is a module variable that
    starts at (eMax-eMin)/(eStpnum-1), Source/Read_In_Allocate.F90:255)."""
    n = len(eaxis)
    w = np.empty(n)
    prev = de0
    for e in range(n):
        if e != n - 1:
            prev = eaxis[e + 1] - eaxis[e]
        w[e] = prev
    return w


# ---------------------------------------------------------------------------
# Dense cross-check (not the reference algorithm): full (npx*M)^2 inverse
# ---------------------------------------------------------------------------
def dense_retarded_greens(htotd, hopx, sig_l, sig_r, energy, eta):
    npx, m, _ = htotd.shape
    n = npx * m
    a = np.zeros((n, n), dtype=complex)
    for x in range(npx):
        a[x * m:(x + 1) * m, x * m:(x + 1) * m] = complex(energy, eta) * np.eye(m) - htotd[x]
        if x + 1 < npx:
            a[x * m:(x + 1) * m, (x + 1) * m:(x + 2) * m] = -hopx
            a[(x + 1) * m:(x + 2) * m, x * m:(x + 1) * m] = -hopx.conj().T
    a[0:m, 0:m] -= sig_l
    a[n - m:n, n - m:n] -= sig_r
    return np.linalg.inv(a)
