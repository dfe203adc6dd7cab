"""Host-side pieces of bench.py (no GPU): the script compiles, the request schedule is the
config's energy x seed walk with disjoint energies per rank, the work model is stated."""
import importlib.util
import os
import py_compile

import numpy as np

from conftest import REPO


def _bench():
    py_compile.compile(os.path.join(REPO, "bench.py"), doraise=True)
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(REPO, "bench.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def test_step_requests_walk_energies_times_seeds():
    b = _bench()
    e, f1, f2, slots = b.step_requests(0, 16, 0, 1)
    assert list(slots) == [0, 1, 2, 3] * 4
    assert len(set(np.round(e, 12))) == 4          # 4 energies, each for all 4 seeds
    assert np.all((f1 >= 0) & (f1 <= 1)) and np.all(f2 <= f1 + 1e-15)
    # ranks take disjoint energies
    seen = set()
    for r in range(4):
        er, _, _, _ = b.step_requests(3, 16, r, 4)
        s = set(np.round(er, 12))
        assert not (s & seen)
        seen |= s


def test_work_model_matches_statement():
    b = _bench()
    m, npx, nsr = 400, 100, 18
    assert b.algorithmic_flops_per_solve(m, npx, nsr) == 48.0 * m ** 3 * npx + (88.0 * nsr + 24.0) * m ** 3 / 4 + 32.0 * m ** 3


def _gloo_rank(rank, world, port, out_q):
    import torch.distributed as dist
    b = _bench()
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    try:
        e, _, _, slots = b.step_requests(2, 16, rank, world)
        units = sorted(zip(np.round(e, 12).tolist(), slots.tolist()))
        gathered = [None] * world
        dist.all_gather_object(gathered, units)
        t = b.max_over_ranks(0.5 + rank, dist, "cpu")
        out_q.put((rank, gathered, t))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_shard_disjointly_and_time_the_slowest():
    """The N > 1 path of bench.py on two CPU ranks (gloo): each rank's (energy, seed) units
    are disjoint from the other's, and the step time is the slowest rank's."""
    import multiprocessing as mp
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_gloo_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, gathered, t in res:
        assert t == 1.5
        a, b = set(map(tuple, gathered[0])), set(map(tuple, gathered[1]))
        assert len(a) == 16 and len(b) == 16 and not (a & b)
