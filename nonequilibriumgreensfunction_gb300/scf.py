"""Self-consistent bias point: the Poisson <-> NEGF loop of Source/NEGF_Main.F90:7-38.

Each outer iteration builds every disorder sample's Hamiltonian on the device with the
current electron potential energy U on its sites (Build_Hamiltonian with the Poisson
potential, Source/Build_Hamiltonian.F90:104-112), runs the whole energy sweep of all
samples as one batched device solve, and solves the 7-point Poisson problem for the new
potential on the device (negf_poisson_solve, the role of SIP_V1 in
Source/SIP_Solver.F90).  The potential is mixed linearly, U <- U + beta (U_poisson - U),
for a fixed number of iterations; the history records max |U_poisson - U| and the
reference's relative-change test max |dU| / (1e-10 + |U|) (Source/SIP_Solver.F90:185-189).

Electrostatics (the configuration's choices; the reference's own Poisson setup differs and
is documented with the oracle):
  - rho = n - p per site: electrons n are RhoN of the energies at or above the mid-gap
    energy e_mid, holes p are RhoP of the energies below it.  Each carrier is counted on its
    own side of the gap, where the other occupation vanishes at the window's ends, so a
    potential shift that moves states across the fixed ends of the energy window does not
    show up as charge (the reference, Source/Read_In_Allocate.F90:242-244, integrates only
    over the bias window for the same reason);
  - kappa = q / (eps0 eps_r a) with a = 1 nm, so a unit of site charge raises U by kappa eV;
  - Dirichlet values: U = mu_L on the plane x = -1, U = mu_R on x = npx (contacts whose
    bands follow their electrochemical potential) and U = u_gate on every y and z face.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from . import capi
from .capi import check

Q = 1.602e-19                 # Source/Constants.F90:4
EPS0 = 8.85418782e-12         # Source/Constants.F90:5
LATTICE_M = 1e-9


def kappa(eps_r: float) -> float:
    return Q / (EPS0 * eps_r * LATTICE_M)


def occupation(energy: float, mu: float, kT: float) -> float:
    """Lead occupation: the step [E <= mu] for kT = 0 (Source/Energy_Sweep.F90:11-21),
    Fermi-Dirac otherwise."""
    if kT <= 0.0:
        return 1.0 if energy <= mu else 0.0
    x = (energy - mu) / kT
    if x > 700:
        return 0.0
    return 1.0 / (1.0 + math.exp(x))


def poisson_solve(rho, bc, kap, u0=None, tol=1e-12, max_iter=100000):
    """Solve the Poisson problem on the device for one grid (npx, npy, npz) or a stack
    (npx, npy, npz, n).  bc = (U_left, U_right, U_gate).  Returns (U, iterations)."""
    lib = capi.load()
    rho = np.asarray(rho, dtype=np.float64)
    single = rho.ndim == 3
    r4 = rho[..., None] if single else rho
    npx, npy, npz, n = r4.shape
    rf = np.asfortranarray(r4)
    # a private copy: the library writes the solution into it
    u = np.zeros(r4.shape, order="F") if u0 is None else np.array(
        np.asarray(u0, dtype=np.float64).reshape(r4.shape), order="F", copy=True)
    b = np.asarray(bc, dtype=np.float64)
    iters = ctypes.c_int32()
    check(lib.negf_poisson_solve(npx, npy, npz, n, rf.ctypes.data_as(capi._dp), b.ctypes.data_as(capi._dp),
                                 float(kap), u.ctypes.data_as(capi._dp), float(tol), int(max_iter),
                                 ctypes.byref(iters)), "negf_poisson_solve")
    return (u[..., 0] if single else u), iters.value


def run_scf(solver, models, energies, dE, mu_l, mu_r, kT, eps_r=100.0, u_gate=0.1, beta=0.3, n_iter=10,
            u0=None, poisson_tol=1e-12, e_mid=0.0):
    """Run ``n_iter`` outer iterations on ``solver`` (a Solver with n_hamiltonians >=
    len(models); one slot per disorder sample).  ``models`` are hamiltonian.wire_model
    dicts.  Returns dict(U=(npx, npy, npz, n) final potential, history=[...],
    last=the per-request results of the last iteration (slot-major, energies in the given
    order), rho_n/rho_p = the electron and hole densities of it)."""
    npx, npy, npz = solver.npx, solver.npy, solver.npz
    ns = len(models)
    energies = np.asarray(energies, dtype=np.float64)
    kap = kappa(eps_r)
    bc = (mu_l, mu_r, u_gate)
    if u0 is None:
        lap, _ = poisson_solve(np.zeros((npx, npy, npz, 1)), bc, kap, tol=poisson_tol)
        u = np.asfortranarray(np.repeat(lap, ns, axis=3))
    else:
        u = np.asfortranarray(np.array(u0, dtype=np.float64).reshape(npx, npy, npz, ns))
    f1 = np.array([occupation(e, mu_l, kT) for e in energies])
    f2 = np.array([occupation(e, mu_r, kT) for e in energies])
    ne = energies.size
    e_all = np.tile(energies, ns)
    f1_all, f2_all = np.tile(f1, ns), np.tile(f2, ns)
    slots = np.repeat(np.arange(ns, dtype=np.int32), ne)
    upper = e_all >= e_mid
    history = []
    last = None
    rn = rp = None
    for _ in range(n_iter):
        for s, m in enumerate(models):
            mm = dict(m)
            mm["V"] = u[..., s] if m.get("V") is None else u[..., s] + np.asarray(m["V"])
            solver.build_hamiltonian(mm, slot=s)
        rn = np.zeros((npx, npy, npz, solver.n_hamiltonians), order="F")
        rp = np.zeros_like(rn)
        parts = []
        for sel, kw in ((upper, dict(rho_n=rn)), (~upper, dict(rho_p=rp))):
            if sel.any():
                parts.append((sel, solver.solve_batch(e_all[sel], f1_all[sel], f2_all[sel], dE, slots=slots[sel],
                                                      **kw)))
        last = {}
        for key, v in parts[0][1].items():
            out = np.zeros(e_all.size, dtype=v.dtype)
            for sel, res in parts:
                out[sel] = res[key]
            last[key] = out
        un, iters = poisson_solve(rn[..., :ns] - rp[..., :ns], bc, kap, u0=u, tol=poisson_tol)
        du = un - u
        history.append(dict(max_change=float(np.abs(du).max()),
                            rel_change=float((np.abs(du) / (1e-10 + np.abs(u))).max()),
                            poisson_iters=iters, status=int(np.abs(last["status"]).max())))
        u = np.asfortranarray(u + beta * du)
    return dict(U=u, history=history, last=last, rho_n=rn, rho_p=rp)
