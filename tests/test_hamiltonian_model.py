"""The counter-based wire model (hamiltonian.wire_model / build_from_model), the host twin
of negf_build_hamiltonian (Build_Hamiltonian.F90 on the device).  CPU only."""
import numpy as np

from nonequilibriumgreensfunction_gb300 import hamiltonian as HB


def test_splitmix64_known_answers():
    # the published SplitMix64 sequence for seed 1234567 (Steele, Lea, Flood 2014 generator)
    got = HB.splitmix64(1234567, np.arange(1, 6))
    assert list(got) == [6457827717110365317, 3203168211198807973, 9817491932198370423,
                         4593380528125082431, 16408922859458223821]


def test_anderson_counter_range_and_leads():
    v = HB.anderson_counter(50, 7, 5, 0.2, 11)
    assert v.shape == (50, 7, 5)
    assert (v[0] == 0).all() and (v[-1] == 0).all()            # Build_Hamiltonian.F90:279-296
    inner = v[1:-1]
    assert inner.min() >= -0.1 and inner.max() < 0.1
    assert abs(inner.mean()) < 0.01 and abs(inner.std() - 0.2 / np.sqrt(12)) < 0.005
    assert not np.array_equal(v, HB.anderson_counter(50, 7, 5, 0.2, 12))
    assert np.array_equal(v, HB.anderson_counter(50, 7, 5, 0.2, 11))


def test_model_build_equals_reference_layout_builder():
    """Same wire as ti_wire (the layout of Build_Hamiltonian.F90:154-207) given the same
    potential: equal without flux, and to rounding with the Landau-gauge phase."""
    v = HB.anderson_counter(6, 3, 4, 0.1, 3)
    for flux, tol in ((0.0, 0.0), (0.5, 1e-15)):
        a, ax = HB.build_from_model(6, 3, 4, HB.wire_model(W=0.1, seed=3, flux=flux, zeeman=0.01))
        b, bx = HB.ti_wire(6, 3, 4, flux=flux, zeeman=0.01, disorder=v)
        assert np.abs(a - b).max() <= tol
        assert np.array_equal(ax, bx)
        assert np.allclose(a, a.conj().transpose(0, 2, 1), rtol=0, atol=0)


def test_explicit_potential_adds_to_disorder():
    v = np.random.default_rng(0).random((5, 2, 3))
    a, _ = HB.build_from_model(5, 2, 3, HB.wire_model(W=0.3, seed=9, V=v))
    b, _ = HB.ti_wire(5, 2, 3, disorder=v + HB.anderson_counter(5, 2, 3, 0.3, 9))
    assert np.array_equal(a, b)
    c, _ = HB.build_from_model(5, 2, 3, HB.wire_model(V=v))
    d, _ = HB.ti_wire(5, 2, 3, disorder=v)
    assert np.array_equal(c, d)
