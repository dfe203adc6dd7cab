"""ctypes binding of include/negf.h (libnegf_gb300.so).

This is the same binding a Python caller of the reference-side C ABI would write; the
Fortran ISO_C_BINDING interface in fortran/negf_gpu_shim.F90 binds the same symbols.
Loading never falls back to a CPU path: a missing or unbuildable library raises.
"""
from __future__ import annotations

import ctypes
import os
from ctypes import POINTER, c_char_p, c_double, c_int, c_int32, c_int64, c_uint64, c_void_p

from . import _build

NEGF_OK = 0
NEGF_EINVAL = -1
NEGF_ENOMEM = -2
NEGF_ECUDA = -3
NEGF_ESR_NOCONV = -4
NEGF_ENAN = -5
NEGF_ESTATE = -6
NEGF_EADMIT = -7
NEGF_ETIMEDOUT = -8
NEGF_EREFINE = -9
NEGF_ENODEV = -10
NEGF_ENOHAM = -11
NEGF_ESCRATCH = -12

NEGF_PREC_FP64 = 0
NEGF_PREC_MIXED = 1
NEGF_CONTACT_LEADS, NEGF_CONTACT_PBIG, NEGF_CONTACT_PSMALL, NEGF_CONTACT_SC = 0, 1, 2, 3

# every symbol include/negf.h declares
EXPORTED_SYMBOLS = (
    "negf_create", "negf_destroy", "negf_strerror", "negf_device_bytes", "negf_estimate_device_bytes",
    "negf_set_stream", "negf_profile", "negf_get_stats", "negf_set_refinement",
    "negf_set_hamiltonian", "negf_build_hamiltonian", "negf_contact_self_energy", "negf_get_retarded_greens",
    "negf_copy_g_columns", "negf_calculate_gnp", "negf_calculate_observables",
    "negf_calculate_currents", "negf_calculate_resolved", "negf_solve_batch", "negf_solve_batch_ex",
    "negf_zgemm", "negf_zinv", "negf_zgemm_noalloc", "negf_poisson_solve",
    "negf_server_create", "negf_server_submit", "negf_server_poll", "negf_server_wait",
    "negf_server_clock", "negf_server_get_stats", "negf_server_destroy",
)


class NegfParams(ctypes.Structure):
    _fields_ = [
        ("npx", c_int32), ("npy", c_int32), ("npz", c_int32), ("norb", c_int32),
        ("n_hamiltonians", c_int32), ("max_batch", c_int32),
        ("eta", c_double), ("sr_tol", c_double),
        ("sr_max_iter", c_int32), ("calc_spin", c_int32), ("precision", c_int32),
        ("device", c_int32), ("mixed_slices", c_int32), ("keep_g_columns", c_int32),
        ("residual_slices", c_int32), ("sr_slices", c_int32), ("calc_currents", c_int32),
        ("reserved", c_int32 * 3),
        ("spin_ops", c_double * (3 * 4 * 4 * 2)),
        ("contact_type", c_int32), ("reserved1", c_int32),
        ("tunneling_rate", c_double), ("delta_sc", c_double * 2), ("chi_lr", c_double),
        ("gds", c_double * (4 * 4 * 2)),
        ("reserved2", c_int32 * 8),
    ]


class NegfRequest(ctypes.Structure):
    _fields_ = [("energy", c_double), ("f1", c_double), ("f2", c_double), ("dE", c_double),
                ("slot", c_int32), ("flags", c_int32)]


class NegfResult(ctypes.Structure):
    _fields_ = [("T12", c_double), ("EDensity", c_double), ("HDensity", c_double),
                ("modes", c_double * 2), ("dosc", c_double * 2),
                ("status", c_int32), ("sr_iters", c_int32)]


class NegfWireModel(ctypes.Structure):
    _fields_ = [("onsite", c_double * 32), ("hop", c_double * 96), ("flux", c_double), ("W", c_double),
                ("seed", c_uint64), ("V", c_void_p), ("reserved", c_int32 * 8)]


def wire_model_struct(model, shape):
    """NegfWireModel from a ``hamiltonian.wire_model`` dict; returns (struct, V array kept
    alive by the caller for as long as the struct is used).  ``shape`` = (npx, npy, npz)."""
    import numpy as np
    m = NegfWireModel()
    blocks = [np.asarray(model["onsite"], dtype=complex)] + [np.asarray(h, dtype=complex) for h in model["hops"]]
    n = blocks[0].shape[0]
    if n > 4 or any(b.shape != (n, n) for b in blocks):
        raise ValueError("site blocks must be norb x norb with norb <= 4")
    padded = []
    for b in blocks:                        # norb x norb in the leading corner of 4 x 4
        q = np.zeros((4, 4), dtype=complex)
        q[:n, :n] = b
        padded.append(q)
    flat = [np.stack([b.real, b.imag], axis=-1).ravel() for b in padded]
    for i, v in enumerate(flat[0]):
        m.onsite[i] = v
    for j in range(3):
        for i, v in enumerate(flat[1 + j]):
            m.hop[32 * j + i] = v
    m.flux, m.W, m.seed = float(model["flux"]), float(model["W"]), int(model["seed"]) & (2 ** 64 - 1)
    keep = None
    if model.get("V") is not None:
        keep = np.asfortranarray(np.asarray(model["V"], dtype=np.float64))
        if keep.shape != tuple(shape):
            raise ValueError("V must be (npx, npy, npz) = %s" % (tuple(shape),))
        m.V = keep.ctypes.data
    return m, keep


class NegfBatchOutputs(ctypes.Structure):
    _fields_ = [("RhoN", c_void_p), ("RhoP", c_void_p), ("SigX", c_void_p), ("SigY", c_void_p),
                ("SigZ", c_void_p), ("Jx", c_void_p), ("Jy", c_void_p), ("Jz", c_void_p),
                ("ERJx", c_void_p), ("ERJy", c_void_p), ("ERJz", c_void_p), ("ERRhon", c_void_p),
                ("ORJx", c_void_p), ("ORJy", c_void_p), ("ORJz", c_void_p), ("ORRhon", c_void_p),
                ("reserved", c_void_p * 8)]


class NegfStats(ctypes.Structure):
    _fields_ = [("launches", c_int64), ("gemm_launches", c_int64), ("gemm_ms", c_double),
                ("gemm_flops", c_double), ("panel_launches", c_int64), ("panel_ms", c_double),
                ("tc_launches", c_int64), ("tc_ms", c_double), ("tc_flops", c_double),
                ("tc_complex_flops", c_double),
                ("fallbacks", c_int64), ("ns_residual_max", c_double), ("f32_gemm_ms", c_double),
                ("slice_ms", c_double), ("phase_sr_ms", c_double), ("phase_rgf_ms", c_double),
                ("phase_inv_ms", c_double), ("phase_dens_ms", c_double), ("ns_extra_steps", c_int64),
                ("ns_unconverged", c_int64), ("ns_final_residual_max", c_double)]


class NegfServeParams(ctypes.Structure):
    _fields_ = [("device", c_int32), ("precision", c_int32), ("mixed_slices", c_int32), ("max_batch", c_int32),
                ("slots_per_geometry", c_int32), ("calc_spin", c_int32), ("eta", c_double), ("sr_tol", c_double),
                ("sr_max_iter", c_int32), ("reserved0", c_int32), ("hbm_budget_bytes", c_int64),
                ("reserved", c_int32 * 8)]


class NegfWireRequest(ctypes.Structure):
    _fields_ = [("npx", c_int32), ("npy", c_int32), ("npz", c_int32), ("norb", c_int32),
                ("Htotd", c_void_p), ("HopX", c_void_p), ("n_energies", c_int32), ("reserved0", c_int32),
                ("energies", c_void_p), ("f1", c_void_p), ("f2", c_void_p), ("dE", c_void_p),
                ("model", c_void_p)]


class NegfWireStatus(ctypes.Structure):
    _fields_ = [("done", c_int32), ("status", c_int32), ("n_done", c_int32), ("reserved0", c_int32),
                ("t_submit", c_double), ("t_admit", c_double), ("t_done", c_double)]


class NegfServerStats(ctypes.Structure):
    _fields_ = [("engines_created", c_int64), ("engines_released", c_int64), ("engines_live", c_int64),
                ("create_s", c_double), ("release_s", c_double), ("bytes_used", c_int64), ("bytes_budget", c_int64),
                ("reserved", c_int64 * 4)]


class NegfError(RuntimeError):
    def __init__(self, code: int, where: str):
        self.code = code
        super().__init__("%s failed: %s (%d)" % (where, strerror(code), code))


_lib = None
_dp = POINTER(c_double)


def _declare(lib):
    h = c_void_p
    sig = {
        "negf_create": (c_int, [POINTER(NegfParams), POINTER(c_void_p)]),
        "negf_destroy": (c_int, [h]),
        "negf_strerror": (c_char_p, [c_int]),
        "negf_device_bytes": (c_int, [h, POINTER(c_int64)]),
        "negf_estimate_device_bytes": (c_int, [POINTER(NegfParams), POINTER(c_int64)]),
        "negf_set_stream": (c_int, [h, c_void_p]),
        "negf_profile": (c_int, [h, c_int]),
        "negf_get_stats": (c_int, [h, POINTER(NegfStats)]),
        "negf_set_refinement": (c_int, [h, c_int32, c_double, c_double]),
        "negf_set_hamiltonian": (c_int, [h, c_int32, _dp, _dp]),
        "negf_build_hamiltonian": (c_int, [h, c_int32, POINTER(NegfWireModel)]),
        "negf_contact_self_energy": (c_int, [h, c_double, _dp, _dp, _dp, _dp, _dp]),
        "negf_get_retarded_greens": (c_int, [h]),
        "negf_copy_g_columns": (c_int, [h, _dp, _dp]),
        "negf_calculate_gnp": (c_int, [h, c_double, c_double, c_double, _dp, _dp]),
        "negf_calculate_observables": (c_int, [h, c_double, c_double, c_double, _dp, _dp, _dp, _dp,
                                               _dp, _dp, _dp, _dp]),
        "negf_calculate_currents": (c_int, [h, _dp, _dp, _dp]),
        "negf_calculate_resolved": (c_int, [h, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp]),
        "negf_zgemm": (c_int, [c_int32, c_int32, c_int32, c_int32, _dp, _dp, c_int32, _dp, c_int32, _dp, _dp,
                               c_int32, c_int32]),
        "negf_zinv": (c_int, [c_int32, _dp, _dp, c_int32]),
        "negf_poisson_solve": (c_int, [c_int32, c_int32, c_int32, c_int32, _dp, _dp, c_double, _dp, c_double,
                                       c_int32, POINTER(c_int32)]),
        "negf_zgemm_noalloc": (c_int, [c_int32, c_int32, c_int32, c_int32, _dp, c_void_p, c_int32, c_void_p, c_int32,
                                       _dp, c_void_p, c_int32, c_void_p]),
        "negf_server_create": (c_int, [POINTER(NegfServeParams), POINTER(c_void_p)]),
        "negf_server_submit": (c_int, [h, POINTER(NegfWireRequest), POINTER(c_int64)]),
        "negf_server_poll": (c_int, [h, c_int64, POINTER(NegfWireStatus), _dp, _dp, c_int32]),
        "negf_server_wait": (c_int, [h, c_int64, c_double]),
        "negf_server_clock": (c_double, [h]),
        "negf_server_get_stats": (c_int, [h, POINTER(NegfServerStats)]),
        "negf_server_destroy": (c_int, [h]),
        "negf_solve_batch": (c_int, [h, POINTER(NegfRequest), c_int32, POINTER(NegfResult),
                                     _dp, _dp, _dp, _dp, _dp]),
        "negf_solve_batch_ex": (c_int, [h, POINTER(NegfRequest), c_int32, POINTER(NegfResult),
                                        POINTER(NegfBatchOutputs)]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args


def library_path() -> str:
    return _build.LIB_PATH


def load(build_if_missing: bool = True):
    """Load libnegf_gb300.so (building it with nvcc when absent or stale)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB_PATH
    if build_if_missing and (not os.path.exists(path) or _build.needs_build()):
        _build.build()
    if not os.path.exists(path):
        raise RuntimeError("libnegf_gb300.so is missing and could not be built")
    lib = ctypes.CDLL(path)
    _declare(lib)
    _lib = lib
    return lib


def strerror(code: int) -> str:
    if _lib is None:
        return "error %d" % code
    return _lib.negf_strerror(code).decode()


def check(code: int, where: str) -> int:
    if code < 0:
        raise NegfError(code, where)
    return code


def _p(a):
    import numpy as np  # noqa: F401
    return a.ctypes.data_as(_dp)


def zgemm(A, B, C=None, alpha=1.0, beta=0.0, slices=0):
    """C = alpha A B + beta C on the GPU for batches of complex matrices.

    A: (batch, m, k) or (m, k); B: (batch, k, n) or (k, n).  slices = 0 uses the FP64
    DFMA kernel, slices in {3, 4, 5, 7} the tcgen05 sliced-BF16 kernel."""
    import numpy as np
    lib = load()
    A = np.asarray(A, dtype=np.complex128)
    B = np.asarray(B, dtype=np.complex128)
    squeeze = A.ndim == 2
    if squeeze:
        A, B = A[None], B[None]
    batch, m, k = A.shape
    n = B.shape[2]
    af = np.ascontiguousarray(A.transpose(0, 2, 1))     # column-major blocks
    bf = np.ascontiguousarray(B.transpose(0, 2, 1))
    if C is None:
        cf = np.zeros((batch, n, m), dtype=np.complex128)
    else:
        Cc = np.asarray(C, dtype=np.complex128)
        cf = np.ascontiguousarray((Cc[None] if squeeze else Cc).transpose(0, 2, 1))
    al = np.array([complex(alpha).real, complex(alpha).imag])
    be = np.array([complex(beta).real, complex(beta).imag])
    check(lib.negf_zgemm(slices, m, n, k, _p(al), _p(af), m, _p(bf), k, _p(be), _p(cf), m, batch), "negf_zgemm")
    out = cf.transpose(0, 2, 1)
    return out[0] if squeeze else out


def zinv(G):
    """Batched inverse (Invert_Matrix); returns (inverse, info)."""
    import numpy as np
    lib = load()
    G = np.asarray(G, dtype=np.complex128)
    squeeze = G.ndim == 2
    if squeeze:
        G = G[None]
    batch, n, _ = G.shape
    gf = np.ascontiguousarray(G.transpose(0, 2, 1))
    out = np.zeros_like(gf)
    info = check(lib.negf_zinv(n, _p(gf), _p(out), batch), "negf_zinv")
    inv = out.transpose(0, 2, 1)
    return (inv[0] if squeeze else inv), info
