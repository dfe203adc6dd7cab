"""C ABI checks that need no GPU: the library builds, loads and exports every symbol
include/negf.h declares; the ctypes structures match the C layout; without a device the
library refuses to run (there is no CPU fallback)."""
import ctypes
import os
import re
import subprocess
import tempfile

import pytest

from conftest import REPO, gpu_available
from nonequilibriumgreensfunction_gb300 import capi

HEADER = os.path.join(REPO, "include", "negf.h")


def declared_symbols():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"NEGF_API\s+[a-z_ ]+\**\s*(negf_[a-z_]+)\s*\(", txt)))


def test_header_declarations_match_binding_list():
    assert declared_symbols() == sorted(capi.EXPORTED_SYMBOLS)


def test_library_exports_every_declared_symbol():
    capi.load()
    out = subprocess.run(["nm", "-D", "--defined-only", capi.library_path()], capture_output=True, text=True,
                         check=True).stdout
    exported = set(re.findall(r"\bT\s+(negf_\w+)", out))
    missing = [s for s in declared_symbols() if s not in exported]
    assert not missing, missing
    lib = ctypes.CDLL(capi.library_path())
    for s in declared_symbols():
        assert hasattr(lib, s)


def test_struct_layout_matches_header():
    src = r"""
#include <stdio.h>
#include <stddef.h>
#include "negf.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\n", sizeof(negf_params), offsetof(negf_params, eta),
         offsetof(negf_params, spin_ops), offsetof(negf_params, keep_g_columns), sizeof(negf_request),
         sizeof(negf_result), offsetof(negf_result, status), sizeof(negf_stats), sizeof(negf_wire_model),
         sizeof(negf_batch_outputs), sizeof(negf_wire_request));
  return 0;
}
"""
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        exe = os.path.join(d, "t")
        open(c, "w").write(src)
        subprocess.run(["gcc", "-I", os.path.join(REPO, "include"), c, "-o", exe], check=True)
        vals = [int(v) for v in subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()]
    want = [ctypes.sizeof(capi.NegfParams), capi.NegfParams.eta.offset, capi.NegfParams.spin_ops.offset,
            capi.NegfParams.keep_g_columns.offset, ctypes.sizeof(capi.NegfRequest), ctypes.sizeof(capi.NegfResult),
            capi.NegfResult.status.offset, ctypes.sizeof(capi.NegfStats), ctypes.sizeof(capi.NegfWireModel),
            ctypes.sizeof(capi.NegfBatchOutputs), ctypes.sizeof(capi.NegfWireRequest)]
    assert vals == want


def test_field_offsets_match_header():
    """Every field of the parameter and output structures the bindings fill sits where the C
    compiler puts it (contact parameters, resolved-output pointers, stats counters)."""
    structs = {
        "negf_params": capi.NegfParams, "negf_batch_outputs": capi.NegfBatchOutputs,
        "negf_stats": capi.NegfStats, "negf_result": capi.NegfResult, "negf_request": capi.NegfRequest,
        "negf_wire_model": capi.NegfWireModel, "negf_serve_params": capi.NegfServeParams,
        "negf_wire_request": capi.NegfWireRequest, "negf_wire_status": capi.NegfWireStatus,
        "negf_server_stats": capi.NegfServerStats,
    }
    lines = []
    for cname, cls in structs.items():
        for fname, _ in cls._fields_:
            lines.append('  printf("%%s.%%s %%zu\\n", "%s", "%s", offsetof(%s, %s));' % (cname, fname, cname, fname))
    src = "#include <stdio.h>\n#include <stddef.h>\n#include \"negf.h\"\nint main(void) {\n" + "\n".join(lines) + \
        "\n  return 0;\n}\n"
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        exe = os.path.join(d, "t")
        open(c, "w").write(src)
        subprocess.run(["gcc", "-I", os.path.join(REPO, "include"), c, "-o", exe], check=True)
        got = dict(line.split() for line in subprocess.run([exe], capture_output=True, text=True,
                                                           check=True).stdout.splitlines())
    for cname, cls in structs.items():
        for fname, _ in cls._fields_:
            assert int(got["%s.%s" % (cname, fname)]) == getattr(cls, fname).offset, (cname, fname)


def test_strerror_covers_codes():
    capi.load()
    for code in range(-12, 1):
        assert capi.strerror(code) not in ("", "unknown error")
    assert "pivot" in capi.strerror(3)


@pytest.mark.skipif(gpu_available(), reason="checks the no-device path")
def test_no_device_fails_loudly():
    from nonequilibriumgreensfunction_gb300 import Solver
    with pytest.raises(capi.NegfError) as ei:
        Solver(4, 3, 3)
    assert ei.value.code == capi.NEGF_ENODEV


def test_c_driver_compiles_against_header():
    """The reference-side caller: a C translation of Energy_Sweep's call sequence
    compiles and links against the library (it is run on the GPU by the gpu tests)."""
    drv = os.path.join(REPO, "nonequilibriumgreensfunction_gb300", "fortran", "energy_sweep_driver.c")
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "drv")
        subprocess.run(["gcc", "-O1", "-I", os.path.join(REPO, "include"), drv, "-o", exe,
                        "-L", os.path.dirname(capi.library_path()), "-lnegf_gb300", "-lm"], check=True)


def test_fortran_shim_params_type_matches_header():
    """The shim's BIND(C) negf_params_t (no Fortran compiler here) lays out like negf_params:
    its fields, parsed from the source and placed with C alignment, have the header's
    offsets and total size."""
    shim = os.path.join(REPO, "nonequilibriumgreensfunction_gb300", "fortran", "negf_gpu_shim.F90")
    txt = open(shim).read()
    body = txt[txt.index("TYPE, BIND(C) :: negf_params_t"):txt.index("END TYPE")]
    sizes = {"INTEGER(C_INT32_T)": 4, "REAL(C_DOUBLE)": 8}
    fields, off = [], 0
    for line in body.splitlines()[1:]:
        line = line.split("!")[0].strip()
        if not line:
            continue
        kind, names = [p.strip() for p in line.split("::")]
        size = sizes[kind]
        for m in re.finditer(r"(\w+)(?:\(([\d,\s]+)\))?", names):
            count = 1
            if m.group(2):
                for d in m.group(2).split(","):
                    count *= int(d)
            off = (off + size - 1) // size * size
            fields.append((m.group(1), off))
            off += size * count
    total = (off + 7) // 8 * 8
    src = "#include <stdio.h>\n#include <stddef.h>\n#include \"negf.h\"\nint main(void) {\n"
    src += "\n".join('  printf("%%zu\\n", offsetof(negf_params, %s));' % f for f, _ in fields)
    src += '\n  printf("%zu\\n", sizeof(negf_params));\n  return 0;\n}\n'
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        exe = os.path.join(d, "t")
        open(c, "w").write(src)
        subprocess.run(["gcc", "-I", os.path.join(REPO, "include"), c, "-o", exe], check=True)
        vals = [int(v) for v in subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()]
    assert vals[:-1] == [o for _, o in fields], list(zip([f for f, _ in fields], vals, [o for _, o in fields]))
    assert vals[-1] == total


def test_device_bytes_estimate_needs_no_device():
    """negf_estimate_device_bytes counts the allocation of negf_create on the host: it grows
    with the batch by the Npx*M^2*16-byte block store per entry, the mixed form adds its
    slice planes, and parameters negf_create refuses are refused."""
    lib = capi.load()

    def est(**kw):
        p = capi.NegfParams()
        p.npx, p.npy, p.npz, p.norb = kw.get("npx", 100), kw.get("npy", 10), kw.get("npz", 10), 4
        p.n_hamiltonians, p.max_batch = kw.get("slots", 4), kw.get("batch", 256)
        p.eta, p.sr_tol, p.sr_max_iter = 1e-5, 1e-10, 20000
        p.precision = kw.get("precision", capi.NEGF_PREC_MIXED)
        v = ctypes.c_int64()
        rc = lib.negf_estimate_device_bytes(ctypes.byref(p), ctypes.byref(v))
        return rc, v.value

    rc, b256 = est()
    assert rc == capi.NEGF_OK
    m2 = 400 * 400
    assert b256 > (256 + 4) * 100 * m2 * 16                 # block store + slots
    rc, b255 = est(batch=255)
    assert rc == capi.NEGF_OK and b256 - b255 >= 100 * m2 * 16
    rc, f64 = est(precision=capi.NEGF_PREC_FP64)
    assert rc == capi.NEGF_OK and f64 < b256
    assert est(npy=15, npz=14)[0] == capi.NEGF_EINVAL         # M = 840 > 800 in the mixed form
    assert est(npy=15, npz=14, precision=capi.NEGF_PREC_FP64)[0] == capi.NEGF_OK
    assert est(batch=0)[0] == capi.NEGF_EINVAL


def test_wire_model_struct_pads_smaller_site_blocks():
    """negf_wire_model holds 4 x 4 blocks; a channel model of norb < 4 goes into their leading
    norb x norb corner (row-major [row][col][re, im]) with zeros elsewhere, which the device
    builder requires."""
    import numpy as np
    from nonequilibriumgreensfunction_gb300 import capi
    from nonequilibriumgreensfunction_gb300 import hamiltonian as HB
    for ct in (2, 3, 4):
        model = HB.channel_model(ct, mu_t=0.2, W=0.1, seed=3)
        n = HB.CHANNEL_NORB[ct]
        m, keep = capi.wire_model_struct(model, (4, 1, 1))
        onsite = np.array(m.onsite[:]).reshape(4, 4, 2)
        hops = np.array(m.hop[:]).reshape(3, 4, 4, 2)
        want = np.asarray(model["onsite"])
        assert np.array_equal(onsite[:n, :n, 0], want.real) and np.array_equal(onsite[:n, :n, 1], want.imag)
        for j in range(3):
            hj = np.asarray(model["hops"][j])
            assert np.array_equal(hops[j, :n, :n, 0], hj.real) and np.array_equal(hops[j, :n, :n, 1], hj.imag)
        mask = np.ones((4, 4), dtype=bool)
        mask[:n, :n] = False
        assert not onsite[mask].any() and not hops[:, mask].any()
        assert m.W == 0.1 and m.seed == 3 and keep is None
    with pytest.raises(ValueError):
        capi.wire_model_struct(dict(onsite=np.eye(5), hops=(np.eye(5),) * 3, flux=0.0, W=0.0, seed=0), (4, 1, 1))
