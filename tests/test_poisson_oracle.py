"""The Poisson oracle: the restatement of Stone's strongly implicit procedure
(Source/SIP_Solver.F90:36-201) is pinned against a sparse direct solve of the same
7-point system.  CPU only."""
import numpy as np
import pytest

from oracle import poisson_oracle as P


def test_kappa_value():
    # q / (eps0 * 100 * 1 nm) with Source/Constants.F90's q and eps0
    assert abs(P.kappa(100.0) - 1.602e-19 / (8.85418782e-12 * 100.0 * 1e-9)) < 1e-15
    assert 0.18 < P.kappa(100.0) < 0.182


@pytest.mark.parametrize("shape", [(10, 4, 4), (7, 3, 5), (24, 6, 6)])
def test_sip_matches_direct_solve(shape):
    rng = np.random.default_rng(sum(shape))
    rho = rng.uniform(-0.02, 0.02, shape)
    b = P.poisson_rhs(rho, P.kappa(100.0), (0.025, -0.025, 0.1))
    u, it = P.sip_solve(b, tol=1e-13)
    ud = P.direct_solve(b)
    assert it > 2                                  # both sweep orders took part
    assert np.abs(u - ud).max() <= 1e-11 * np.abs(ud).max()


def test_single_sip_iteration_reduces_the_error_in_both_orders():
    shape = (12, 5, 4)
    rng = np.random.default_rng(3)
    b = P.poisson_rhs(rng.uniform(-0.01, 0.01, shape), P.kappa(100.0), (0.0, 0.0, 0.1))
    ud = P.direct_solve(b)
    planes = P._hyperplanes(shape)
    u = np.zeros(shape)
    err = np.abs(u - ud).max()
    for it in range(4):
        u, _ = P.sip_iteration(u, b, it, planes)
        e2 = np.abs(u - ud).max()
        assert e2 < err
        err = e2


def test_laplace_solution_is_bounded_by_boundary_values():
    b = P.poisson_rhs(np.zeros((9, 4, 4)), P.kappa(100.0), (0.025, -0.025, 0.1))
    u, _ = P.sip_solve(b)
    assert u.max() < 0.1 and u.min() > -0.025
