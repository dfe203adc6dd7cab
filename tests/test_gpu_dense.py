"""GPU tests of the dense kernels through the C ABI: the FP64 DFMA GEMM, the tcgen05
sliced-BF16 GEMM and the Gauss-Jordan inverse, against NumPy FP64.

Error bound of the sliced GEMM with S slices of 7 bits (row scale of A, column scale of B):
    |C - C_ref|_ij <= c * 2^(-7 S) * k * max_l |A_il| * max_l |B_lj|
checked with c = 8 (the truncation of both operands, both parts of the complex product)."""
import numpy as np
import pytest

from nonequilibriumgreensfunction_gb300 import capi

pytestmark = pytest.mark.gpu


def _rand(rng, *shape, spread=0.0):
    a = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    if spread:
        a = a * np.exp(spread * rng.standard_normal(shape[:-1]))[..., None]
    return a


def _bound(A, B, S):
    ra = np.abs(A).max(axis=-1)                       # (batch, m)
    cb = np.abs(B).max(axis=-2)                       # (batch, n)
    k = A.shape[-1]
    return 8.0 * 2.0 ** (-7 * S) * k * ra[..., :, None] * cb[..., None, :]


@pytest.mark.parametrize("shape", [(64, 64, 64), (37, 53, 12), (130, 200, 256), (400, 400, 400)])
@pytest.mark.parametrize("S", [3, 4, 5, 6, 7, 8])
def test_sliced_gemm_error_bound(need_gpu, shape, S):
    rng = np.random.default_rng(S * 1000 + shape[0])
    m, n, k = shape
    A = _rand(rng, 2, m, k, spread=2.0)
    B = _rand(rng, 2, k, n)
    ref = A @ B
    got = capi.zgemm(A, B, slices=S)
    err = np.abs(got - ref)
    assert (err <= _bound(A, B, S) + 1e-300).all(), (S, shape, (err / _bound(A, B, S)).max())


def test_sliced_gemm_alpha_beta_and_fp64_path(need_gpu):
    rng = np.random.default_rng(3)
    A, B, C = _rand(rng, 3, 96, 80), _rand(rng, 3, 80, 72), _rand(rng, 3, 96, 72)
    al, be = 0.5 - 2j, -1.25 + 0.5j
    ref = al * (A @ B) + be * C
    for S in (0, 7):
        got = capi.zgemm(A, B, C, alpha=al, beta=be, slices=S)
        assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max(), S


def test_sliced_gemm_zero_rows_and_wide_exponents(need_gpu):
    rng = np.random.default_rng(4)
    A = _rand(rng, 1, 128, 64)
    A[0, 5, :] = 0.0
    A[0, 7, :] *= 1e-200
    A[0, 9, :] *= 1e150
    B = _rand(rng, 1, 64, 128)
    B[0, :, 3] = 0.0
    ref = A @ B
    got = capi.zgemm(A, B, slices=7)
    assert np.all(got[0, 5, :] == 0.0) and np.all(got[0, :, 3] == 0.0)
    rel = np.abs(got - ref) / np.maximum(np.abs(A).max(axis=-1)[..., None] * np.abs(B).max(axis=-2)[:, None, :], 1e-300)
    assert rel.max() < 8 * 2.0 ** -49 * A.shape[-1]


def test_inverse_matches_lapack(need_gpu):
    rng = np.random.default_rng(5)
    for n in (36, 64, 400):
        G = _rand(rng, 3, n, n) + 4 * np.eye(n)
        inv, info = capi.zinv(G)
        assert info == 0
        ref = np.linalg.inv(G)
        assert np.abs(inv - ref).max() <= 1e-11 * np.abs(ref).max()
    S = np.eye(8, dtype=complex)
    S[3, :] = 0
    S[:, 3] = 0
    _, info = capi.zinv(S)
    assert info == 4          # LAPACK INFO: 1-based index of the first zero pivot


def test_tensor_core_variant_choice_does_not_change_results(need_gpu, monkeypatch):
    """The first product of a shape times the two per-tile tcgen05 kernels (different N
    tiles) and the persistent one and keeps the fastest; all issue each output's MMAs in
    the same K order into exact accumulators, so every variant, the tuning call and the
    later (cached-choice) calls give bitwise equal results.  NEGF_TC_VARIANT forces one."""
    rng = np.random.default_rng(11)
    for s in (3, 4, 5, 6, 7, 8):
        for shape in ((6, 96, 96, 96), (3, 144, 144, 144), (2, 400, 400, 400)):
            nb, m, n, k = shape
            a = rng.standard_normal((nb, m, k)) + 1j * rng.standard_normal((nb, m, k))
            b = rng.standard_normal((nb, k, n)) + 1j * rng.standard_normal((nb, k, n))
            monkeypatch.delenv("NEGF_TC_VARIANT", raising=False)
            first = capi.zgemm(a, b, slices=s)
            again = capi.zgemm(a, b, slices=s)
            assert np.array_equal(first, again), (s, shape)
            for v in ("0", "1", "2"):
                monkeypatch.setenv("NEGF_TC_VARIANT", v)
                assert np.array_equal(capi.zgemm(a, b, slices=s), first), (s, shape, v)
            assert (np.abs(first - a @ b) <= _bound(a, b, s)).all(), (s, shape)
    monkeypatch.delenv("NEGF_TC_VARIANT", raising=False)


@pytest.mark.parametrize("S", [3, 5, 7, 8])
def test_sliced_gemm_split_k_accumulators(need_gpu, S):
    """K' = 2k > 800: the K blocks are split in two halves with their own exact
    accumulators (k = 576 and 784, the config-5 and largest config-4 cross-sections, and
    an odd k = 613); the error bound is the same, alpha and beta are applied once."""
    rng = np.random.default_rng(100 + S)
    for (m, n, k) in ((576, 576, 576), (784, 160, 784), (200, 136, 613)):
        A = _rand(rng, 1, m, k, spread=1.0)
        B = _rand(rng, 1, k, n)
        C = _rand(rng, 1, m, n)
        al, be = 0.5 + 0.25j, 1.0
        got = capi.zgemm(A, B, C, alpha=al, beta=be, slices=S)
        ref = al * (A @ B) + be * C
        assert (np.abs(got - ref) <= abs(al) * _bound(A, B, S) + 1e-12 * np.abs(C)).all(), (S, m, n, k)


def test_sliced_gemm_refuses_k_beyond_its_exact_accumulators(need_gpu):
    A = np.zeros((1, 16, 801), dtype=complex)
    B = np.zeros((1, 801, 16), dtype=complex)
    with pytest.raises(capi.NegfError) as ei:
        capi.zgemm(A, B, slices=5)
    assert ei.value.code == capi.NEGF_EINVAL
