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
