"""Python side of the request server (negf_server_* in include/negf.h), whose requests keep
their state on the device, and the Poisson-arrival load generator used to measure serving
latency.

The server replaces the MPI master/worker energy sweep (Source/NEGF_Main.F90:21-27):
wires of different cross-sections arrive as requests, are admitted by their HBM
footprint, and their energy points are continuously batched with those of other
requests of the same geometry."""
from __future__ import annotations

import ctypes
import math
import time

import numpy as np

from . import capi
from .capi import NegfServeParams, NegfWireRequest, NegfWireStatus, check


class Server:
    def __init__(self, precision="mixed", max_batch=16, slots_per_geometry=8, eta=1e-5, sr_tol=1e-10,
                 sr_max_iter=20000, calc_spin=False, hbm_budget_bytes=0, device=0, mixed_slices=0):
        self.lib = capi.load()
        p = NegfServeParams()
        p.device = device
        p.precision = {"fp64": capi.NEGF_PREC_FP64, "mixed": capi.NEGF_PREC_MIXED}[precision]
        p.mixed_slices = mixed_slices
        p.max_batch = max_batch
        p.slots_per_geometry = slots_per_geometry
        p.calc_spin = 1 if calc_spin else 0
        p.eta, p.sr_tol, p.sr_max_iter = eta, sr_tol, sr_max_iter
        p.hbm_budget_bytes = int(hbm_budget_bytes)
        h = ctypes.c_void_p()
        check(self.lib.negf_server_create(ctypes.byref(p), ctypes.byref(h)), "negf_server_create")
        self._h = h
        self._meta = {}

    def close(self):
        if getattr(self, "_h", None):
            self.lib.negf_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def clock(self) -> float:
        return float(self.lib.negf_server_clock(self._h))

    def submit(self, htotd, hopx, energies, f1, f2, dE):
        """Queue one wire: htotd[x, row, col] (npx, M, M), hopx (M, M), per-energy f1/f2/dE."""
        htotd = np.asarray(htotd, dtype=np.complex128)
        npx, m, _ = htotd.shape
        hf = np.ascontiguousarray(htotd.transpose(0, 2, 1))
        xf = np.asfortranarray(np.asarray(hopx, dtype=np.complex128))
        e = np.ascontiguousarray(energies, dtype=np.float64)
        n = e.size
        arrs = [np.ascontiguousarray(np.broadcast_to(np.asarray(v, dtype=np.float64), (n,))) for v in (f1, f2, dE)]
        nsite = m // 4
        npy = self._infer_npy(nsite)
        r = NegfWireRequest()
        r.npx, r.npy, r.npz, r.norb = npx, npy, nsite // npy, 4
        r.Htotd, r.HopX = hf.ctypes.data, xf.ctypes.data
        r.n_energies = n
        r.energies, r.f1, r.f2, r.dE = e.ctypes.data, arrs[0].ctypes.data, arrs[1].ctypes.data, arrs[2].ctypes.data
        rid = ctypes.c_int64()
        check(self.lib.negf_server_submit(self._h, ctypes.byref(r), ctypes.byref(rid)), "negf_server_submit")
        self._meta[rid.value] = (n, npx, r.npy, r.npz)
        return rid.value

    def submit_model(self, npx, npy, npz, model, energies, f1, f2, dE):
        """Queue one wire given as a model (``hamiltonian.wire_model``): the server
        generates its Htotd on the device, so only the model crosses to the GPU."""
        e = np.ascontiguousarray(energies, dtype=np.float64)
        n = e.size
        arrs = [np.ascontiguousarray(np.broadcast_to(np.asarray(v, dtype=np.float64), (n,))) for v in (f1, f2, dE)]
        m, keep = capi.wire_model_struct(model, (npx, npy, npz))
        r = NegfWireRequest()
        r.npx, r.npy, r.npz, r.norb = npx, npy, npz, 4
        r.n_energies = n
        r.energies, r.f1, r.f2, r.dE = e.ctypes.data, arrs[0].ctypes.data, arrs[1].ctypes.data, arrs[2].ctypes.data
        r.model = ctypes.addressof(m)
        rid = ctypes.c_int64()
        check(self.lib.negf_server_submit(self._h, ctypes.byref(r), ctypes.byref(rid)), "negf_server_submit")
        del keep
        self._meta[rid.value] = (n, npx, npy, npz)
        return rid.value

    def _infer_npy(self, nsite):
        # wires here are square in cross-section unless set explicitly
        s = int(round(math.sqrt(nsite)))
        return s if s * s == nsite else nsite

    def set_geometry_hint(self, npy):
        self._infer_npy = lambda nsite, npy=npy: npy

    def stats(self):
        """Engine churn: engines created / released / live, host seconds spent creating and
        releasing them, and the bytes in use against the budget."""
        st = capi.NegfServerStats()
        check(self.lib.negf_server_get_stats(self._h, ctypes.byref(st)), "negf_server_get_stats")
        return {k: getattr(st, k) for k, _ in capi.NegfServerStats._fields_ if k != "reserved"}

    def status(self, rid):
        st = NegfWireStatus()
        check(self.lib.negf_server_poll(self._h, rid, ctypes.byref(st), None, None, 0), "negf_server_poll")
        return st

    def result(self, rid, release=True):
        n, npx, npy, npz = self._meta[rid]
        res7 = np.zeros((n, 7))
        rho = np.zeros(2 * npx * npy * npz)
        st = NegfWireStatus()
        check(self.lib.negf_server_poll(self._h, rid, ctypes.byref(st), res7.ctypes.data_as(capi._dp),
                                        rho.ctypes.data_as(capi._dp), 1 if release else 0), "negf_server_poll")
        if not st.done:
            return None
        if release:
            self._meta.pop(rid, None)
        keys = ["T12", "EDensity", "HDensity", "Modec1", "Modec2", "DOSc1", "DOSc2"]
        out = {k: res7[:, i].copy() for i, k in enumerate(keys)}
        out["RhoN"] = rho[:npx * npy * npz].reshape((npx, npy, npz), order="F")
        out["RhoP"] = rho[npx * npy * npz:].reshape((npx, npy, npz), order="F")
        out["status"] = st.status
        out["latency"] = st.t_done - st.t_submit
        out["t_submit"], out["t_admit"], out["t_done"] = st.t_submit, st.t_admit, st.t_done
        return out

    def wait(self, rid, timeout=600.0):
        rc = self.lib.negf_server_wait(self._h, rid, float(timeout))
        if rc == capi.NEGF_ETIMEDOUT:
            raise TimeoutError("request %d not done after %.0f s" % (rid, timeout))
        check(rc, "negf_server_wait")


def run_poisson_load(server, make_request, rate_hz, duration_s, rng, max_outstanding=64):
    """Submit requests as a Poisson stream of `rate_hz` for `duration_s`, then drain.
    `make_request(rng)` returns (htotd, hopx, energies, f1, f2, dE), or a dict with keys
    shape=(npx, npy, npz), model, energies, f1, f2, dE for a wire generated on the device.
    Returns per-request latency (s), solves, and wall time."""
    t0 = time.perf_counter()
    ids, solves = [], 0
    t_next = 0.0
    while True:
        now = time.perf_counter() - t0
        if now >= duration_s:
            break
        if now < t_next:
            time.sleep(min(t_next - now, 0.05))
            continue
        req = make_request(rng)
        if isinstance(req, dict):
            e = req["energies"]
            ids.append(server.submit_model(*req["shape"], req["model"], e, req["f1"], req["f2"], req["dE"]))
        else:
            h, x, e, f1, f2, de = req
            ids.append(server.submit(h, x, e, f1, f2, de))
        solves += len(e)
        t_next += rng.exponential(1.0 / rate_hz)
    lat = []
    for rid in ids:
        server.wait(rid, timeout=1800.0)
        r = server.result(rid)
        lat.append(r["latency"])
    wall = time.perf_counter() - t0
    return np.asarray(lat), solves, wall
