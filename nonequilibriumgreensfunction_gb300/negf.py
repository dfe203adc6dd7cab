"""Host-side mirror of the reference's per-energy interface, on top of the C ABI.

The reference's hot path is Energy_Sweep (Source/Energy_Sweep.F90:1-46) calling four
subroutines that share NEGF_Module globals.  ``Solver`` keeps their names and argument
meaning, with the globals made explicit:

    Solver.contact_self_energy(energy)        Contact_Self_Energy   (Contact_Self_Energy.F90:1-106)
    Solver.get_retarded_greens()              Get_Retarded_Greens   (Recursive_Greens.F90:2-107)
    Solver.calculate_gnp(f1, f2, dE, ...)     Calculate_Gnp         (Calculate_Gnp.F90:1-136)
    Solver.calculate_observables(dE, f1, f2)  Calculate_Observables (Calculate_Observables.F90:2-169)
    Solver.energy_sweep(energy, ...)          Energy_Sweep          (Energy_Sweep.F90:1-46)
    Solver.solve_batch(...)                   the energy loop of NEGF_Main.F90:21-27 + MPI sums

Errors follow the reference's errorFlag convention: LAPACK INFO > 0 is returned as a
status (the reference prints and continues, Recursive_Greens.F90:28-33), library errors
(< 0) raise ``NegfError``.  Every call runs on the GPU; there is no CPU path.

Array conventions (NumPy side): Hamiltonians are slice-first ``htotd[x, row, col]``,
site arrays are ``(npx, npy, npz)`` Fortran-ordered (the reference's RhoN layout).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import capi
from .capi import NegfParams, NegfRequest, NegfResult, check

_dp = ctypes.POINTER(ctypes.c_double)


def _ptr(a):
    if a is None:
        return None
    return a.ctypes.data_as(_dp)


def _to_fortran_blocks(htotd):
    """(npx, row, col) -> memory of Fortran Htotd(M, M, npx)."""
    return np.ascontiguousarray(np.asarray(htotd, dtype=np.complex128).transpose(0, 2, 1))


class Solver:
    def __init__(self, npx, npy, npz, norb=4, n_hamiltonians=1, max_batch=1, eta=1e-4, sr_tol=1e-8,
                 sr_max_iter=20000, calc_spin=False, precision="fp64", device=0, keep_g_columns=False,
                 spin_ops=None, mixed_slices=0, residual_slices=0, sr_slices=0, calc_currents=False,
                 contact_type=0, tunneling_rate=1.0, delta_sc=(1e-3, 1e-3), chi_lr=0.8, gds=None):
        """``contact_type`` is the reference's contactType: 0 semi-infinite leads, 1 / 2
        phenomenological contacts, 3 superconducting contacts on a BdG Hamiltonian (norb =
        2 x the electron orbitals; see hamiltonian.bdg).  ``tunneling_rate``, ``delta_sc``
        (DeltaSCL, DeltaSCR), ``chi_lr`` and ``gds`` (None = the four-orbital model's) are
        the contact parameters of Read_In_Allocate.F90:69-76,199-202."""
        self.lib = capi.load()
        p = NegfParams()
        p.npx, p.npy, p.npz, p.norb = npx, npy, npz, norb
        p.n_hamiltonians, p.max_batch = n_hamiltonians, max_batch
        p.eta, p.sr_tol, p.sr_max_iter = eta, sr_tol, sr_max_iter
        p.calc_spin = 1 if calc_spin else 0
        p.precision = {"fp64": capi.NEGF_PREC_FP64, "mixed": capi.NEGF_PREC_MIXED}[precision]
        p.device = device
        p.mixed_slices = mixed_slices
        p.residual_slices = residual_slices
        p.sr_slices = sr_slices
        p.keep_g_columns = 1 if keep_g_columns else 0
        p.calc_currents = 1 if calc_currents else 0
        nh = norb // 2 if contact_type == capi.NEGF_CONTACT_SC else norb
        if spin_ops is not None:
            ops = np.asarray(spin_ops, dtype=np.complex128)
            buf = np.zeros((3, 4, 4, 2))
            buf[:, :nh, :nh, 0] = ops.real
            buf[:, :nh, :nh, 1] = ops.imag
            for i, v in enumerate(buf.ravel()):
                p.spin_ops[i] = v
        p.contact_type = contact_type
        p.tunneling_rate = tunneling_rate
        p.delta_sc[0], p.delta_sc[1] = delta_sc
        p.chi_lr = chi_lr
        if gds is not None:
            g = np.asarray(gds, dtype=np.complex128)
            buf = np.zeros((4, 4, 2))
            buf[:g.shape[0], :g.shape[1], 0] = g.real
            buf[:g.shape[0], :g.shape[1], 1] = g.imag
            for i, v in enumerate(buf.ravel()):
                p.gds[i] = v
        self.params = p
        self.npx, self.npy, self.npz, self.norb = npx, npy, npz, norb
        self.M = norb * npy * npz
        self.max_batch = max_batch
        self.n_hamiltonians = n_hamiltonians
        self.calc_spin = bool(calc_spin)
        self.calc_currents = bool(calc_currents)
        self.contact_type = contact_type
        self.nh = nh
        h = ctypes.c_void_p()
        check(self.lib.negf_create(ctypes.byref(p), ctypes.byref(h)), "negf_create")
        self._h = h

    # -- lifetime --------------------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            self.lib.negf_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def device_bytes(self) -> int:
        v = ctypes.c_int64()
        check(self.lib.negf_device_bytes(self._h, ctypes.byref(v)), "negf_device_bytes")
        return int(v.value)

    def set_stream(self, stream_handle):
        """Run on a caller-owned cudaStream_t (an int handle, e.g. torch's
        ``torch.cuda.current_stream().cuda_stream``); None restores the handle's stream."""
        check(self.lib.negf_set_stream(self._h, ctypes.c_void_p(stream_handle) if stream_handle else None),
              "negf_set_stream")

    def profile(self, enable=True):
        check(self.lib.negf_profile(self._h, 1 if enable else 0), "negf_profile")

    def set_refinement(self, ns_max_steps=0, ns_tol=0.0, ns_accept=0.0):
        """Newton-Schulz policy of the mixed form (negf_set_refinement): at most
        ``ns_max_steps`` refinement steps per inverse, more than the two fixed ones while
        the residual norm before the latest update is above ``ns_tol``; an inverse whose
        first residual norm is above ``ns_accept``, or that is still above ``ns_tol`` after
        the last step, is redone in FP64.  0 selects a default (4, 1e-5, 0.5)."""
        check(self.lib.negf_set_refinement(self._h, int(ns_max_steps), float(ns_tol), float(ns_accept)),
              "negf_set_refinement")

    def stats(self):
        st = capi.NegfStats()
        check(self.lib.negf_get_stats(self._h, ctypes.byref(st)), "negf_get_stats")
        return {k: getattr(st, k) for k, _ in capi.NegfStats._fields_}

    # -- Hamiltonian -----------------------------------------------------------------
    def set_hamiltonian(self, htotd, hopx=None, slot=0):
        hf = _to_fortran_blocks(htotd)
        if hf.shape != (self.npx, self.M, self.M):
            raise ValueError("htotd must be (npx, M, M) = %s" % ((self.npx, self.M, self.M),))
        xf = None if hopx is None else np.asfortranarray(np.asarray(hopx, dtype=np.complex128))
        check(self.lib.negf_set_hamiltonian(self._h, slot, _ptr(hf),
                                            None if xf is None else _ptr(xf)),
              "negf_set_hamiltonian")

    def set_hamiltonian_fortran(self, htotd_f, hopx_f=None, slot=0):
        """Upload arrays that already have the reference's memory layout: ``htotd_f`` is
        the contiguous memory of Htotd(M, M, npx) (NumPy shape (npx, M, M) indexed
        [x, col, row]) and ``hopx_f`` a Fortran-ordered (M, M) array; no host copy is made
        (pinned buffers upload at full PCIe/C2C speed)."""
        if htotd_f.dtype != np.complex128 or not htotd_f.flags.c_contiguous or htotd_f.size != self.npx * self.M ** 2:
            raise ValueError("htotd_f must be contiguous complex128 with npx*M*M elements")
        if hopx_f is not None and (hopx_f.dtype != np.complex128 or not hopx_f.flags.f_contiguous):
            raise ValueError("hopx_f must be Fortran-ordered complex128")
        check(self.lib.negf_set_hamiltonian(self._h, slot, _ptr(htotd_f),
                                            None if hopx_f is None else _ptr(hopx_f)),
              "negf_set_hamiltonian")

    def build_hamiltonian(self, model, slot=0):
        """Generate slot ``slot``'s Htotd (and HopX) on the device from a wire model
        (``hamiltonian.wire_model``): Build_Hamiltonian.F90 without the host-to-device copy.
        ``hamiltonian.build_from_model`` gives the identical arrays on the host."""
        m, keep = capi.wire_model_struct(model, (self.npx, self.npy, self.npz))
        check(self.lib.negf_build_hamiltonian(self._h, slot, ctypes.byref(m)), "negf_build_hamiltonian")
        del keep

    # -- the reference's four subroutines --------------------------------------------
    def contact_self_energy(self, energy, want_matrices=True):
        m = self.M
        mats = [np.zeros((m, m), dtype=np.complex128, order="F") for _ in range(4)] if want_matrices else [None] * 4
        dosc = np.zeros(2)
        st = check(self.lib.negf_contact_self_energy(
            self._h, float(energy), *[None if a is None else _ptr(a) for a in mats],
            _ptr(dosc)), "negf_contact_self_energy")
        out = dict(dosc=dosc, status=st)
        if want_matrices:
            out.update(SigmaL=mats[0], SigmaR=mats[1], GammaL=mats[2], GammaR=mats[3])
        return out

    def get_retarded_greens(self):
        return check(self.lib.negf_get_retarded_greens(self._h), "negf_get_retarded_greens")

    def g_columns(self):
        """(GRLef, GRRgt) as (npx, M, M) block arrays; needs keep_g_columns=True."""
        ntot = self.npx * self.M
        a = np.zeros((ntot, self.M), dtype=np.complex128, order="F")
        b = np.zeros((ntot, self.M), dtype=np.complex128, order="F")
        check(self.lib.negf_copy_g_columns(self._h, _ptr(a), _ptr(b)),
              "negf_copy_g_columns")
        return a.reshape(self.npx, self.M, self.M), b.reshape(self.npx, self.M, self.M)

    def new_site_array(self, n_slots=None):
        shape = (self.npx, self.npy, self.npz) if n_slots is None else (self.npx, self.npy, self.npz, n_slots)
        return np.zeros(shape, order="F")

    def calculate_gnp(self, f1, f2, dE, rho_n=None, rho_p=None):
        for a in (rho_n, rho_p):
            if a is not None and not (a.flags.f_contiguous and a.dtype == np.float64):
                raise ValueError("site arrays must be Fortran-ordered float64")
        check(self.lib.negf_calculate_gnp(self._h, float(f1), float(f2), float(dE), _ptr(rho_n), _ptr(rho_p)),
              "negf_calculate_gnp")

    def calculate_observables(self, dE, f1, f2, contact_current=None, spin=None):
        t12, ed, hd = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        modes = np.zeros(2)
        cc = contact_current if contact_current is not None else np.zeros(2)
        sx = sy = sz = None
        if spin is not None:
            sx, sy, sz = spin
        check(self.lib.negf_calculate_observables(
            self._h, float(dE), float(f1), float(f2), ctypes.byref(t12), ctypes.byref(ed), ctypes.byref(hd),
            _ptr(modes), _ptr(cc), _ptr(sx), _ptr(sy), _ptr(sz)), "negf_calculate_observables")
        return dict(T12=t12.value, EDensity=ed.value, HDensity=hd.value, Modec1=modes[0], Modec2=modes[1])

    def calculate_currents(self, currents):
        """Bond currents of Calculate_Observables.F90:110-169 for the energy of the last
        calculate_gnp call, added into ``currents`` = (Jx, Jy, Jz), Fortran-ordered
        (npx, npy, npz) float64 arrays (None entries are skipped)."""
        jx, jy, jz = currents
        for a in (jx, jy, jz):
            if a is not None and not (a.flags.f_contiguous and a.dtype == np.float64):
                raise ValueError("site arrays must be Fortran-ordered float64")
        check(self.lib.negf_calculate_currents(self._h, _ptr(jx), _ptr(jy), _ptr(jz)), "negf_calculate_currents")

    def calculate_resolved(self, er=None, orb=None):
        """Energy- and orbital-resolved current densities (erCD/orCD,
        Calculate_Observables.F90:124-160, Calculate_Gnp.F90:125-129) of the energy of the
        last calculate_gnp call.  ``er`` = (ERJx, ERJy, ERJz, ERRhon), (npx, npy, npz) arrays
        the unweighted values are added to; ``orb`` = (ORJx, ORJy, ORJz) of shape (npx, npy,
        npz, norb**2) and ORRhon of shape (npx, npy, npz, norb), dE/(2 pi)-weighted.  All
        Fortran-ordered float64; None entries are skipped."""
        arrs = tuple(er if er is not None else (None,) * 4) + tuple(orb if orb is not None else (None,) * 4)
        for a in arrs:
            if a is not None and not (a.flags.f_contiguous and a.dtype == np.float64):
                raise ValueError("site arrays must be Fortran-ordered float64")
        check(self.lib.negf_calculate_resolved(self._h, *(_ptr(a) for a in arrs)), "negf_calculate_resolved")

    def energy_sweep(self, energy, f1, f2, dE, rho_n=None, rho_p=None, contact_current=None, spin=None,
                     currents=None):
        """Energy_Sweep.F90:28-46 for one energy; returns the per-energy observables."""
        cse = self.contact_self_energy(energy, want_matrices=False)
        st = self.get_retarded_greens()
        self.calculate_gnp(f1, f2, dE, rho_n, rho_p)
        obs = self.calculate_observables(dE, f1, f2, contact_current, spin)
        if currents is not None:
            self.calculate_currents(currents)
        obs.update(dosc=cse["dosc"], sr_status=cse["status"], rgf_status=st)
        return obs

    # -- batched ---------------------------------------------------------------------
    def solve_batch(self, energies, f1, f2, dE, slots=None, rho_n=None, rho_p=None, spin=None, currents=None,
                    er=None, orb=None):
        """Solve len(energies) energy points (chunked by max_batch on the device).

        ``rho_n``/``rho_p``/``spin``/``currents`` (if given) are (npx, npy, npz,
        n_hamiltonians) Fortran-ordered arrays the dE-weighted densities, spin densities
        (SigX, SigY, SigZ) and bond currents (Jx, Jy, Jz) are added to.  ``er`` =
        (ERJx, ERJy, ERJz, ERRhon), each (npx, npy, npz, n): the unweighted energy-resolved
        values of request i are added to [..., i].  ``orb`` = (ORJx, ORJy, ORJz) of shape
        (npx, npy, npz, norb**2, n_hamiltonians) and ORRhon (npx, npy, npz, norb,
        n_hamiltonians): the dE-weighted orbital-resolved sums.  Returns a dict of
        per-request arrays."""
        energies = np.asarray(energies, dtype=np.float64)
        n = energies.size
        f1 = np.broadcast_to(np.asarray(f1, dtype=np.float64), (n,))
        f2 = np.broadcast_to(np.asarray(f2, dtype=np.float64), (n,))
        dE = np.broadcast_to(np.asarray(dE, dtype=np.float64), (n,))
        slots = np.zeros(n, dtype=np.int32) if slots is None else np.broadcast_to(np.asarray(slots, np.int32), (n,))
        req = (NegfRequest * n)()
        for i in range(n):
            req[i].energy, req[i].f1, req[i].f2, req[i].dE = energies[i], f1[i], f2[i], dE[i]
            req[i].slot = int(slots[i])
            req[i].flags = 0
        res = (NegfResult * n)()
        sx = sy = sz = None
        if spin is not None:
            sx, sy, sz = spin
        if currents is None and er is None and orb is None:
            rc = self.lib.negf_solve_batch(self._h, req, n, res, _ptr(rho_n), _ptr(rho_p), _ptr(sx), _ptr(sy),
                                           _ptr(sz))
            check(rc, "negf_solve_batch")
        else:
            outs = capi.NegfBatchOutputs()
            arrs = ((rho_n, rho_p, sx, sy, sz) + tuple(currents if currents is not None else (None,) * 3)
                    + tuple(er if er is not None else (None,) * 4) + tuple(orb if orb is not None else (None,) * 4))
            for name, a in zip(("RhoN", "RhoP", "SigX", "SigY", "SigZ", "Jx", "Jy", "Jz",
                                "ERJx", "ERJy", "ERJz", "ERRhon", "ORJx", "ORJy", "ORJz", "ORRhon"), arrs):
                if a is not None and not (a.flags.f_contiguous and a.dtype == np.float64):
                    raise ValueError("site arrays must be Fortran-ordered float64")
                setattr(outs, name, None if a is None else a.ctypes.data)
            check(self.lib.negf_solve_batch_ex(self._h, req, n, res, ctypes.byref(outs)), "negf_solve_batch_ex")
        out = dict(
            T12=np.array([r.T12 for r in res]),
            EDensity=np.array([r.EDensity for r in res]),
            HDensity=np.array([r.HDensity for r in res]),
            Modec1=np.array([r.modes[0] for r in res]),
            Modec2=np.array([r.modes[1] for r in res]),
            DOSc1=np.array([r.dosc[0] for r in res]),
            DOSc2=np.array([r.dosc[1] for r in res]),
            status=np.array([r.status for r in res], dtype=np.int32),
            sr_iters=np.array([r.sr_iters for r in res], dtype=np.int32),
        )
        return out
