"""CPU oracle for the self-consistent bias point (Poisson <-> NEGF).

TEST INFRASTRUCTURE ONLY.  Nothing in the product path imports this module; it is the
checker the device Poisson solver and the self-consistent loop are compared against.

What it restates:

    Source/SIP_Solver.F90:36-201    sip_iteration()  Stone's strongly implicit procedure, both
                                                      sweep orders (odd/even outer iteration)
    Source/SIP_Module.F90:47-49     SIP_ALPHAS       the relaxation parameters cycled by iteration
    Source/SIP_Solver.F90:185-190   the update Phi += PhiDelta and the relative-change test
    Source/NEGF_Main.F90:7-38       scf_loop()       Poisson -> Build_Hamiltonian -> energy loop

The electrostatic problem is the one of the self-consistent configuration (7-point
Laplacian, uniform eps_r, Dirichlet values on the planes outside the site grid: the two
contacts at x = -1 and x = npx, a gate on every y and z face), written for the electron
potential energy U (eV) on each site:

    sum_{6 neighbours j} (U_i - U_j) = kappa * rho_i,    rho = n - p,
    kappa = q / (eps0 eps_r a)   (a = 1 nm; q, eps0 of Source/Constants.F90)

so that electrons raise their own potential energy.  The reference's Poisson differs and
this restatement says where: it normalises eps by the Bi2Se3 value and has no kappa
(Source/SIP_Coefficients.F90), shifts the SIP diagonal by -ro as a linearisation of its
nonlinear problem (Source/SIP_Solver.F90:62-67), takes one SIP sweep per outer iteration
with Phi += PhiDelta, and adds Phi to the on-site energy with the opposite sign convention
(Source/Build_Hamiltonian.F90:104-112).  Here each outer iteration solves the linear
problem to convergence with the same SIP recurrences and mixes linearly:
U <- U + beta (U_poisson - U).

Parity status: the SIP restatement is pinned against a sparse direct solve of the same
system (tests/test_poisson_oracle.py); the reference's own Poisson path cannot be run
(Fortran, no compiler here).
"""
from __future__ import annotations

import numpy as np

from oracle import negf_oracle as O

EPS0 = 8.85418782e-12          # Source/Constants.F90:5
LATTICE_M = 1e-9               # lattice constant a = 1 nm
SIP_ALPHAS = (0.25, 0.35, 0.45, 0.35, 0.25, 0.15)   # Source/SIP_Module.F90:47-49


def kappa(eps_r: float) -> float:
    """Potential energy (eV) per unit of site charge density: q / (eps0 eps_r a)."""
    return O.Q_E / (EPS0 * eps_r * LATTICE_M)


def poisson_rhs(rho, kap, bc):
    """b = kappa rho + the Dirichlet values of the neighbours outside the grid.
    bc = (U_left, U_right, U_gate); rho is (npx, npy, npz)."""
    b = kap * np.asarray(rho, dtype=np.float64)
    b = b.copy()
    b[0] += bc[0]
    b[-1] += bc[1]
    b[:, 0] += bc[2]
    b[:, -1] += bc[2]
    b[:, :, 0] += bc[2]
    b[:, :, -1] += bc[2]
    return b


def apply_operator(u):
    """(A u)_i = 6 u_i - sum of the in-grid neighbours (zero outside)."""
    au = 6.0 * u
    au[1:] -= u[:-1]
    au[:-1] -= u[1:]
    au[:, 1:] -= u[:, :-1]
    au[:, :-1] -= u[:, 1:]
    au[:, :, 1:] -= u[:, :, :-1]
    au[:, :, :-1] -= u[:, :, 1:]
    return au


def direct_solve(b):
    """Sparse direct solve of A u = b (the pin for the SIP restatement)."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spl
    nx, ny, nz = b.shape

    def lap(n):
        return sp.diags([-np.ones(n - 1), 2.0 * np.ones(n), -np.ones(n - 1)], [-1, 0, 1])
    ix, iy, iz = sp.identity(nx), sp.identity(ny), sp.identity(nz)
    # x fastest (column-major), matching b.ravel(order="F")
    a = (sp.kron(sp.kron(iz, iy), lap(nx)) + sp.kron(sp.kron(iz, lap(ny)), ix)
         + sp.kron(sp.kron(lap(nz), iy), ix)).tocsc()
    return spl.spsolve(a, b.ravel(order="F")).reshape(b.shape, order="F")


def _hyperplanes(shape):
    nx, ny, nz = shape
    i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    s = (i + j + k).ravel()
    order = np.argsort(s, kind="stable")
    bounds = np.searchsorted(s[order], np.arange(nx + ny + nz - 1))
    planes = []
    for t in range(nx + ny + nz - 2):
        sel = order[bounds[t]:bounds[t + 1]]
        planes.append((i.ravel()[sel], j.ravel()[sel], k.ravel()[sel]))
    return planes


def _sip_sweep(coef, rhs_res, alpha, planes):
    """One SIP correction in the first sweep order of Source/SIP_Solver.F90:59-117 on a
    grid whose unknowns are ordered i fastest, then j, then k.  coef = (B, C, D, E, F, G, H)
    are the couplings to (k-1, j-1, i-1, self, i+1, j+1, k+1); rhs_res is the residual R.
    Points of one hyperplane i+j+k = s depend only on the plane before (forward) or after
    (backward), so each plane is evaluated at once; every point's arithmetic is the
    reference's recurrence."""
    B, C, D, E, F, G, H = coef
    nx, ny, nz = E.shape
    shp = (nx + 2, ny + 2, nz + 2)        # one zero ghost layer on each side (index + 1)
    a, b, c, d, e, f, g, v, dl = (np.zeros(shp) for _ in range(9))
    for (i, j, k) in planes:
        I, J, K = i + 1, j + 1, k + 1
        a[I, J, K] = B[i, j, k] / (1.0 + alpha * (e[I, J, K - 1] + f[I, J, K - 1]))
        b[I, J, K] = C[i, j, k] / (1.0 + alpha * (e[I, J - 1, K] + g[I, J - 1, K]))
        c[I, J, K] = D[i, j, k] / (1.0 + alpha * (g[I - 1, J, K] + f[I - 1, J, K]))
        d[I, J, K] = (E[i, j, k]
                      - c[I, J, K] * (e[I - 1, J, K] - alpha * g[I - 1, J, K] - alpha * f[I - 1, J, K])
                      - b[I, J, K] * (f[I, J - 1, K] - alpha * e[I, J - 1, K] - alpha * g[I, J - 1, K])
                      - a[I, J, K] * (g[I, J, K - 1] - alpha * e[I, J, K - 1] - alpha * f[I, J, K - 1]))
        e[I, J, K] = (F[i, j, k] - alpha * (a[I, J, K] * e[I, J, K - 1] + b[I, J, K] * e[I, J - 1, K])) / d[I, J, K]
        f[I, J, K] = (G[i, j, k] - alpha * (c[I, J, K] * f[I - 1, J, K] + a[I, J, K] * f[I, J, K - 1])) / d[I, J, K]
        g[I, J, K] = (H[i, j, k] - alpha * (c[I, J, K] * g[I - 1, J, K] + b[I, J, K] * g[I, J - 1, K])) / d[I, J, K]
    for (i, j, k) in planes:                                   # :95-106
        I, J, K = i + 1, j + 1, k + 1
        v[I, J, K] = (rhs_res[i, j, k] - a[I, J, K] * v[I, J, K - 1] - b[I, J, K] * v[I, J - 1, K]
                      - c[I, J, K] * v[I - 1, J, K]) / d[I, J, K]
    for (i, j, k) in reversed(planes):                         # :108-116
        I, J, K = i + 1, j + 1, k + 1
        dl[I, J, K] = v[I, J, K] - e[I, J, K] * dl[I + 1, J, K] - f[I, J, K] * dl[I, J + 1, K] \
            - g[I, J, K] * dl[I, J, K + 1]
    return dl[1:-1, 1:-1, 1:-1]


def sip_iteration(u, b, it, planes):
    """One outer SIP iteration (Source/SIP_Solver.F90:36-190) on A u = b written as the
    reference's 7-point form  B u(k-1) + C u(j-1) + D u(i-1) + E u + F u(i+1) + G u(j+1)
    + H u(k+1) = ro  with B..H = 1, E = -6 and ro = -b.  Even iterations use the first sweep
    order; odd ones reverse j and k (the second sweep, :120-181), which is the first sweep
    on the grid flipped in j and k with (B, C, G, H) -> (H, G, C, B).  alpha cycles through
    SIP_ALPHAS (:16).  Returns u + PhiDelta and max |PhiDelta|."""
    one = np.ones_like(u)
    coef = (one, one, one, -6.0 * one, one, one, one)
    # R = ro - (stencil) u with ro = -b: the reference's residual, zero neighbours outside
    res = -b + apply_operator(u)
    alpha = SIP_ALPHAS[it % len(SIP_ALPHAS)]
    if it % 2 == 0:
        delta = _sip_sweep(coef, res, alpha, planes)
    else:
        fl = (slice(None), slice(None, None, -1), slice(None, None, -1))
        B, C, D, E, F, G, H = (x[fl] for x in coef)
        delta = _sip_sweep((H, G, D, E, F, C, B), res[fl], alpha, planes)[fl]
    return u + delta, float(np.abs(delta).max())


def sip_solve(b, u0=None, tol=1e-13, max_iter=2000):
    """Iterate SIP outer iterations until ||A u - b|| <= tol ||b||."""
    u = np.zeros_like(b) if u0 is None else np.array(u0, dtype=np.float64)
    planes = _hyperplanes(b.shape)
    nb = np.linalg.norm(b)
    for it in range(max_iter):
        if np.linalg.norm(apply_operator(u) - b) <= tol * nb:
            return u, it
        u, _ = sip_iteration(u, b, it, planes)
    raise RuntimeError("SIP did not converge in %d iterations" % max_iter)


def scf_loop(npx, npy, npz, models, energies, dE, mu_l, mu_r, opt, eps_r=100.0, u_gate=0.1, beta=0.3,
             n_iter=3, e_mid=0.0):
    """Self-consistent bias point in the order of Source/NEGF_Main.F90:7-38: for each
    outer iteration and each disorder sample (model), build the Hamiltonian with the
    current potential U on every site, run the energy loop, form rho = n - p, solve
    Poisson and mix.  Electrons n are RhoN of the energies at or above the mid-gap energy
    e_mid, holes p are RhoP of those below it (each carrier on its own side of the gap, so
    the fixed ends of the energy window, where Gn or Gp vanish, do not contribute).  U
    starts from the charge-free (Laplace) solution.  Returns the final U per sample, the
    history of max |U_poisson - U| and the per-energy T12 of the last iteration's
    Hamiltonians."""
    from nonequilibriumgreensfunction_gb300 import hamiltonian as HB
    kap = kappa(eps_r)
    bc = (mu_l, mu_r, u_gate)
    u0, _ = sip_solve(poisson_rhs(np.zeros((npx, npy, npz)), kap, bc))
    us = [u0.copy() for _ in models]
    hist = []
    t_last = None
    for _ in range(n_iter):
        worst = 0.0
        t_last = []
        for s, m in enumerate(models):
            mm = dict(m)
            mm["V"] = us[s] if m.get("V") is None else us[s] + m["V"]
            h, x = HB.build_from_model(npx, npy, npz, mm)
            rn = np.zeros((npx, npy, npz))
            rp = np.zeros((npx, npy, npz))
            ts = []
            for e in energies:
                r = O.energy_sweep(h, x, float(e), (mu_l, mu_r), dE, npy, npz, opt)
                if e >= e_mid:
                    rn += r["RhoN"]
                else:
                    rp += r["RhoP"]
                ts.append(r["T12"])
            t_last.append(np.array(ts))
            un, _ = sip_solve(poisson_rhs(rn - rp, kap, bc), u0=us[s])
            worst = max(worst, float(np.abs(un - us[s]).max()))
            us[s] = us[s] + beta * (un - us[s])
        hist.append(worst)
    return us, hist, t_last
