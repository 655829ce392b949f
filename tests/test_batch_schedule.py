"""The batch's assignment of problems to worker streams (csrc/pdt_schedule.h, built on the host as the C ABI
builds it): longest problems first, each to the least-loaded stream. Checked against a restatement, for its
bound (the most loaded stream within 4/3 of the best assignment, found by exhaustive search on small
cases) and for the cases a batch meets (fewer problems than streams, equal costs)."""
import ctypes
import itertools
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def emu(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("schedule") / "schedule_emu.so")
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-o", out,
                           os.path.join(HERE, "native", "schedule_emu.cpp")])
    lib = ctypes.CDLL(out)
    lib.emu_assign.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
    return lib


def _assign(emu, cost, P):
    c = np.ascontiguousarray(cost, dtype=np.uint64)
    o = np.zeros(len(c), dtype=np.uint64)
    emu.emu_assign(c.ctypes.data, len(c), P, o.ctypes.data)
    return o.astype(np.int64)


def _restated(cost, P):
    order = sorted(range(len(cost)), key=lambda i: -cost[i])  # stable: ties by index
    load, owner = [0] * P, [0] * len(cost)
    for i in order:
        w = min(range(P), key=lambda k: (load[k], k))
        owner[i] = w
        load[w] += cost[i]
    return owner


def _makespan(cost, owner, P):
    load = np.zeros(P, dtype=np.int64)
    np.add.at(load, owner, cost)
    return int(load.max())


def test_matches_restatement(emu):
    rng = np.random.default_rng(5)
    for _ in range(200):
        n, P = int(rng.integers(1, 80)), int(rng.integers(1, 40))
        cost = rng.integers(1, 10 ** 7, n)
        assert list(_assign(emu, cost, P)) == _restated(list(cost), P)


def test_within_four_thirds_of_best(emu):
    rng = np.random.default_rng(6)
    for _ in range(60):
        n, P = int(rng.integers(2, 9)), int(rng.integers(2, 4))
        cost = rng.integers(1, 100, n)
        best = min(_makespan(cost, np.array(a), P) for a in itertools.product(range(P), repeat=n))
        got = _makespan(cost, _assign(emu, cost, P), P)
        assert got * 3 * P <= best * (4 * P - 1), (cost, P, got, best)


def test_batch_shapes(emu):
    # fewer problems than streams: every problem has a stream of its own
    cost = [640 * 368 * 15, 192 * 192 * 8, 320 * 320 * 21, 256 * 256 * 12]
    assert sorted(_assign(emu, cost, 32)) == [0, 1, 2, 3]
    # equal costs: round robin in index order
    assert list(_assign(emu, [7] * 6, 3)) == [0, 1, 2, 0, 1, 2]
    # two large problems never share a stream while others are light
    cost = [100, 100, 1, 1, 1, 1]
    o = _assign(emu, cost, 2)
    assert o[0] != o[1]
    # no streams or no problems
    assert list(_assign(emu, [3, 4], 0)) == [0, 0]
    assert len(_assign(emu, [], 4)) == 0
