"""negf_zgemm_noalloc: the tensor-core sliced GEMM for callers that cannot allocate device
memory (their device memory belongs to another allocator, or their loop cannot absorb
the device-wide synchronisation of cudaMalloc/cudaFree).  Its scratch is a static device
array shared by all calls, so this test makes two calls in a row with different operands
and sizes and checks each against negf_zgemm (which allocates its own scratch) on the
same inputs, within the sliced-GEMM error bound used by test_gpu_dense.py; it also checks
the size limit.  Runs last so that a failure here never hides another test's result."""
import ctypes

import numpy as np
import pytest

from nonequilibriumgreensfunction_gb300 import capi

pytestmark = pytest.mark.gpu


def _bound(A, B, S):
    return 8.0 * 2.0 ** (-7 * S) * A.shape[-1] * np.abs(A).max(axis=-1)[:, None] * np.abs(B).max(axis=-2)[None, :]


def _noalloc(lib, torch, S, A, B, C, alpha, beta):
    # column-major device copies: a contiguous (cols, rows) tensor is the column-major matrix
    dA = torch.from_numpy(np.ascontiguousarray(A.T)).cuda()
    dB = torch.from_numpy(np.ascontiguousarray(B.T)).cuda()
    dC = torch.from_numpy(np.ascontiguousarray(C.T)).cuda()
    al = np.array([alpha.real, alpha.imag])
    be = np.array([beta.real, beta.imag])
    m, k = A.shape
    n = B.shape[1]
    torch.cuda.synchronize()
    rc = lib.negf_zgemm_noalloc(S, m, n, k, al.ctypes.data_as(capi._dp), ctypes.c_void_p(dA.data_ptr()), m,
                                ctypes.c_void_p(dB.data_ptr()), k, be.ctypes.data_as(capi._dp),
                                ctypes.c_void_p(dC.data_ptr()), m, None)
    return rc, dC.cpu().numpy().T


def test_noalloc_matches_allocating_gemm_on_two_calls(need_gpu):
    torch = pytest.importorskip("torch")
    lib = capi.load()
    rng = np.random.default_rng(21)
    cases = [(7, (400, 400, 400)), (5, (130, 77, 256))]   # two calls in a row, second smaller
    for S, (m, n, k) in cases:
        A = rng.standard_normal((m, k)) + 1j * rng.standard_normal((m, k))
        B = rng.standard_normal((k, n)) + 1j * rng.standard_normal((k, n))
        C = rng.standard_normal((m, n)) + 1j * rng.standard_normal((m, n))
        alpha, beta = 0.75 - 0.5j, 1.0 + 0.0j
        want = capi.zgemm(A, B, C, alpha=alpha, beta=beta, slices=S)
        rc, got = _noalloc(lib, torch, S, A, B, C, alpha, beta)
        assert rc == capi.NEGF_OK, capi.strerror(rc)
        tol = abs(alpha) * _bound(A, B, S)
        assert (np.abs(got - want) <= tol).all()
        assert (np.abs(got - (alpha * (A @ B) + beta * C)) <= tol).all()


def test_noalloc_first_beta_zero_call_of_a_shape_and_device_memory(need_gpu):
    """beta = 0 on a shape no call has used yet: the first such call of a shape times the
    kernel variants on the shared scratch before it keeps one, so two calls in a row (the
    tuning call and a tuned one) must both match negf_zgemm and alpha A B.  Free device
    memory must not move across a call: the entry point allocates nothing."""
    torch = pytest.importorskip("torch")
    lib = capi.load()
    rng = np.random.default_rng(33)
    m, n, k, S = 96, 200, 64, 7
    alpha, beta = 1.0 - 0.25j, 0.0 + 0.0j
    for rep in range(2):
        A = rng.standard_normal((m, k)) + 1j * rng.standard_normal((m, k))
        B = rng.standard_normal((k, n)) + 1j * rng.standard_normal((k, n))
        C = np.full((m, n), np.nan + 0j)          # beta = 0: C is never read
        rc, got = _noalloc(lib, torch, S, A, B, C, alpha, beta)   # first: the tuning call
        assert rc == capi.NEGF_OK, capi.strerror(rc)
        want = capi.zgemm(A, B, alpha=alpha, slices=S)
        tol = abs(alpha) * _bound(A, B, S)
        assert np.isfinite(got).all()
        assert (np.abs(got - want) <= tol).all(), rep
        assert (np.abs(got - alpha * (A @ B)) <= tol).all(), rep
    # device buffers first, then free memory around two more calls of the same shape
    dA = torch.from_numpy(np.ascontiguousarray(A.T)).cuda()
    dB = torch.from_numpy(np.ascontiguousarray(B.T)).cuda()
    dC = torch.zeros((n, m), dtype=torch.complex128, device="cuda")
    al = np.array([alpha.real, alpha.imag])
    be = np.array([0.0, 0.0])
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(2):
        rc = lib.negf_zgemm_noalloc(S, m, n, k, al.ctypes.data_as(capi._dp), ctypes.c_void_p(dA.data_ptr()), m,
                                    ctypes.c_void_p(dB.data_ptr()), k, be.ctypes.data_as(capi._dp),
                                    ctypes.c_void_p(dC.data_ptr()), m, None)
        assert rc == capi.NEGF_OK
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0


def test_noalloc_rejects_sizes_beyond_its_scratch(need_gpu):
    torch = pytest.importorskip("torch")
    lib = capi.load()
    A = np.zeros((513, 8), dtype=complex)
    B = np.zeros((8, 8), dtype=complex)
    C = np.zeros((513, 8), dtype=complex)
    rc, _ = _noalloc(lib, torch, 4, A, B, C, 1.0 + 0j, 0.0 + 0j)
    assert rc == capi.NEGF_ESCRATCH
    assert "512" in capi.strerror(rc)
