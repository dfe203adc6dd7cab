"""Serving: continuous batching of wires of different cross-sections.  Each request's
results equal those of the same wire solved alone (the batch composition never enters
a request's arithmetic), and admission under a small HBM budget queues requests until
memory frees up instead of failing."""
import numpy as np
import pytest

from nonequilibriumgreensfunction_gb300 import Solver
from nonequilibriumgreensfunction_gb300 import hamiltonian as HB
from nonequilibriumgreensfunction_gb300.serving import Server

pytestmark = pytest.mark.gpu


def _wire(n, npx, seed):
    h, x = HB.ti_wire(npx, n, n, W=0.1, seed=seed, flux=0.3, zeeman=0.01)
    return h, x


def _alone(h, x, npx, n, es, f1, f2, de, precision):
    with Solver(npx, n, n, eta=1e-5, sr_tol=1e-10, max_batch=len(es), precision=precision) as s:
        s.set_hamiltonian(h, x)
        rn = s.new_site_array(1)
        r = s.solve_batch(es, f1, f2, de, rho_n=rn)
    return r, rn[..., 0]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_server_results_same_alone_and_in_the_mix(need_gpu, precision):
    rng = np.random.default_rng(0)
    wires = [(2, 6, 0), (3, 5, 1), (2, 6, 2), (3, 7, 3), (2, 6, 4)]   # (cross-section, npx, seed)
    reqs = []
    with Server(precision=precision, max_batch=4, slots_per_geometry=2) as srv:
        for n, npx, seed in wires:
            h, x = _wire(n, npx, seed)
            es = np.sort(rng.uniform(-0.25, 0.25, size=int(rng.integers(3, 9))))
            f1 = rng.uniform(0, 1, es.size)
            f2 = rng.uniform(0, 1, es.size)
            rid = srv.submit(h, x, es, f1, f2, 1e-3)
            reqs.append((rid, h, x, n, npx, es, f1, f2))
        for rid, h, x, n, npx, es, f1, f2 in reqs:
            srv.wait(rid, timeout=300)
            got = srv.result(rid)
            assert got["status"] == 0
            want, rn = _alone(h, x, npx, n, es, f1, f2, 1e-3, precision)
            for k in ("T12", "EDensity", "HDensity", "Modec1", "Modec2", "DOSc1", "DOSc2"):
                assert np.array_equal(got[k], want[k]), (k, got[k], want[k])
            assert np.array_equal(got["RhoN"], rn)
            assert got["t_submit"] <= got["t_admit"] <= got["t_done"]


def test_server_admission_under_small_budget(need_gpu):
    """A budget that holds one geometry's engine at a time: requests of the other geometry
    wait for the idle engine to be released, and every request completes."""
    rng = np.random.default_rng(1)
    with Server(precision="fp64", max_batch=2, slots_per_geometry=1, hbm_budget_bytes=100 << 20) as srv:
        ids = []
        for i in range(4):
            n, npx = (2, 6) if i % 2 == 0 else (3, 5)
            h, x = _wire(n, npx, i)
            es = rng.uniform(-0.2, 0.2, 3)
            ids.append((srv.submit(h, x, es, 1.0, 0.0, 1e-3), h, x, n, npx, es))
        for rid, h, x, n, npx, es in ids:
            srv.wait(rid, timeout=300)
            got = srv.result(rid)
            assert got["status"] == 0
            want, _ = _alone(h, x, npx, n, es, 1.0, 0.0, 1e-3, "fp64")
            assert np.array_equal(got["T12"], want["T12"])


def test_server_model_requests_match_uploaded_wires(need_gpu):
    """Wires submitted as models (generated on the device) mix with uploaded wires of the
    same geometry and give the results of the uploaded host twin solved alone."""
    rng = np.random.default_rng(5)
    with Server(precision="mixed", max_batch=4, slots_per_geometry=2) as srv:
        reqs = []
        for i in range(4):
            m = HB.wire_model(W=0.15, seed=100 + i, flux=0.25 * i, zeeman=0.01)
            h, x = HB.build_from_model(6, 3, 3, m)
            es = np.sort(rng.uniform(-0.25, 0.25, size=5))
            if i % 2 == 0:
                rid = srv.submit_model(6, 3, 3, m, es, 0.8, 0.1, 1e-3)
            else:
                rid = srv.submit(h, x, es, 0.8, 0.1, 1e-3)
            reqs.append((rid, h, x, es))
        for rid, h, x, es in reqs:
            srv.wait(rid, timeout=300)
            got = srv.result(rid)
            assert got["status"] == 0
            want, rn = _alone(h, x, 6, 3, es, 0.8, 0.1, 1e-3, "mixed")
            assert np.array_equal(got["T12"], want["T12"])
            assert np.array_equal(got["RhoN"], rn)


@pytest.mark.parametrize("precision,currents", [("fp64", False), ("mixed", False), ("mixed", True)])
def test_admission_estimate_equals_the_engine_allocation(need_gpu, precision, currents):
    """The serving layer admits engines by negf_estimate_device_bytes; it must be the bytes
    negf_create actually allocates (mixed form: slice planes, Newton-Schulz buffers)."""
    import ctypes
    from nonequilibriumgreensfunction_gb300 import capi
    for (npx, n, batch) in ((12, 6, 8), (5, 14, 3)):
        with Solver(npx, n, n, max_batch=batch, n_hamiltonians=2, precision=precision,
                    calc_currents=currents) as s:
            v = ctypes.c_int64()
            assert s.lib.negf_estimate_device_bytes(ctypes.byref(s.params), ctypes.byref(v)) == capi.NEGF_OK
            assert v.value == s.device_bytes(), (npx, n, batch)


def test_eviction_churn_with_many_geometries(need_gpu):
    """The serving configuration's regime: many geometries and an HBM budget that holds
    about two engines, so workers are evicted and re-created continually while others run
    (a worker that has just finished a batch, and may release the server lock while it
    admits, is never evicted from under itself).  Every request finishes with the results
    it has alone."""
    import ctypes
    from nonequilibriumgreensfunction_gb300 import capi
    geoms = [(2, 5), (3, 5), (2, 6), (3, 6), (2, 7), (3, 7)]      # (cross-section, npx)
    with Solver(7, 3, 3, max_batch=3, n_hamiltonians=1, precision="mixed") as s:
        v = ctypes.c_int64()
        assert s.lib.negf_estimate_device_bytes(ctypes.byref(s.params), ctypes.byref(v)) == capi.NEGF_OK
        big = v.value
    rng = np.random.default_rng(9)
    reqs = []
    # admission asks for an engine's bytes plus 64 MB: this budget holds two engines
    with Server(precision="mixed", max_batch=3, slots_per_geometry=1,
                hbm_budget_bytes=int(2.3 * big) + (64 << 20)) as srv:
        for i in range(30):
            n, npx = geoms[int(rng.integers(len(geoms)))]
            h, x = _wire(n, npx, 200 + i)
            es = np.sort(rng.uniform(-0.25, 0.25, size=int(rng.integers(2, 7))))
            reqs.append((srv.submit(h, x, es, 0.7, 0.2, 1e-3), h, x, n, npx, es))
        for rid, h, x, n, npx, es in reqs:
            srv.wait(rid, timeout=600)
            got = srv.result(rid)
            assert got["status"] == 0
            want, _ = _alone(h, x, npx, n, es, 0.7, 0.2, 1e-3, "mixed")
            assert np.array_equal(got["T12"], want["T12"])
        st = srv.stats()
    # the budget forced engines to be released and created again
    assert st["engines_created"] > len(geoms) // 2 and st["engines_released"] >= 1
    assert st["engines_created"] - st["engines_released"] == st["engines_live"]
    assert st["bytes_used"] <= st["bytes_budget"]


def test_request_larger_than_the_budget_fails_at_once(need_gpu):
    """A request whose engine alone exceeds the server's HBM budget can never be admitted:
    it finishes at once with NEGF_EADMIT instead of waiting, and the server keeps serving."""
    from nonequilibriumgreensfunction_gb300 import capi
    with Server(precision="fp64", max_batch=2, slots_per_geometry=1, hbm_budget_bytes=80 << 20) as srv:
        hb, xb = _wire(8, 20, 1)                        # M = 256, Npx = 20: an engine of ~150 MB
        big = srv.submit(hb, xb, [0.01], 1.0, 0.0, 1e-3)
        h, x = _wire(2, 5, 2)
        small = srv.submit(h, x, [0.02, 0.1], 1.0, 0.0, 1e-3)
        srv.wait(big, timeout=60)
        assert srv.result(big)["status"] == capi.NEGF_EADMIT
        srv.wait(small, timeout=300)
        assert srv.result(small)["status"] == 0
