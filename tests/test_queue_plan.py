"""CPU: the work-queue plan of the batched launch (achr.cu_gb300/csrc/achr_queue_plan.h), compiled
here with the host C++ compiler: every chain exactly once, longest chain time first, each tile at
most its share of the work queued from it on, and single chains at the end."""
from __future__ import annotations

import ctypes as C
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

CSRC = Path(__file__).resolve().parents[1] / "achr.cu_gb300" / "csrc"

WRAPPER = r"""
#include "achr_queue_plan.h"
extern "C" int plan(int n_models, const int *models, const int *n_points, const double *chain_time, int ctas,
                    int tiles, int *out, int cap) {
    std::vector<int> m(models, models + n_models);
    const std::vector<achr::QueueItem> items = achr::plan_queue(m, n_points, chain_time, ctas, tiles);
    int k = 0;
    for (const achr::QueueItem &q : items) {
        if (k < cap) {
            out[3 * k] = q.model;
            out[3 * k + 1] = q.p0;
            out[3 * k + 2] = q.p1;
        }
        ++k;
    }
    return k;
}
"""


@pytest.fixture(scope="module")
def planner(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    d = tmp_path_factory.mktemp("plan")
    (d / "plan.cpp").write_text(WRAPPER)
    so = d / "libplan.so"
    subprocess.run([cxx, "-O2", "-std=c++17", "-shared", "-fPIC", "-I", str(CSRC), str(d / "plan.cpp"), "-o", str(so)],
                   check=True)
    lib = C.CDLL(str(so))
    lib.plan.restype = C.c_int
    lib.plan.argtypes = [C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_double), C.c_int, C.c_int,
                         C.POINTER(C.c_int), C.c_int]

    def run(n_points, chain_time, ctas, tiles, models=None):
        n_points = np.ascontiguousarray(n_points, dtype=np.int32)
        chain_time = np.ascontiguousarray(chain_time, dtype=np.float64)
        models = np.ascontiguousarray(np.arange(len(n_points)) if models is None else models, dtype=np.int32)
        cap = int(n_points.sum()) + 8
        out = np.zeros(3 * cap, dtype=np.int32)
        k = lib.plan(len(models), models.ctypes.data_as(C.POINTER(C.c_int)), n_points.ctypes.data_as(C.POINTER(C.c_int)),
                     chain_time.ctypes.data_as(C.POINTER(C.c_double)), ctas, tiles,
                     out.ctypes.data_as(C.POINTER(C.c_int)), cap)
        return out[:3 * k].reshape(k, 3)
    return run


def _check(items, n_points, chain_time, ctas, tiles):
    # every chain of every model exactly once, each model's tiles contiguous and in order
    for k, P in enumerate(n_points):
        mine = items[items[:, 0] == k]
        if P == 0:
            assert len(mine) == 0
            continue
        assert mine[0, 1] == 0 and mine[-1, 2] == P
        assert np.all(mine[1:, 1] == mine[:-1, 2]) and np.all(mine[:, 2] > mine[:, 1])
    # models longest chain time first
    order = [int(m) for i, m in enumerate(items[:, 0]) if i == 0 or items[i - 1, 0] != m]
    assert len(order) == len(set(order))
    assert all(chain_time[a] >= chain_time[b] for a, b in zip(order, order[1:]))
    # a tile holds at most its share (1 / (tiles x ctas)) of the work queued from it on, or one
    # chain; so the tiles shrink towards the end of the queue, which ends with single chains
    work = (items[:, 2] - items[:, 1]) * np.asarray(chain_time)[items[:, 0]]
    behind = np.cumsum(work[::-1])[::-1]  # work queued from each item to the end
    single = items[:, 2] - items[:, 1] == 1
    assert np.all(single | (work <= behind / (tiles * ctas) * (1 + 1e-9)))
    if sum(n_points) >= tiles * ctas:
        assert single[-1]


@pytest.mark.parametrize("tiles", [1, 4, 16])
def test_plan_covers_every_chain_in_shrinking_tiles(planner, tiles):
    rng = np.random.default_rng(tiles)
    sizes = np.exp(rng.uniform(np.log(95), np.log(7440), size=12))
    n_points = np.floor(262144 * sizes / sizes.sum()).astype(int)  # the batch64 workload's chain count
    n_points[3] = 0  # a model without chains
    chain_time = sizes * 1000 * 1e-9
    items = planner(n_points, chain_time, 304, tiles)
    _check(items, n_points, chain_time, 304, tiles)
    # guided self-scheduling: O(tiles x ctas x log(chains)) queue operations, not one per chain
    assert len(items) <= tiles * 304 * (np.log(n_points.sum()) + 2) < n_points.sum()


def test_plan_of_one_small_model_is_one_chain_per_item(planner):
    items = planner([10], [1e-6], 304, 4)
    assert items.tolist() == [[0, p, p + 1] for p in range(10)]


def test_plan_uses_only_the_given_models(planner):
    n_points = np.array([100, 200, 300])
    items = planner(n_points, [3e-6, 2e-6, 1e-6], 8, 4, models=[2, 0])
    assert set(items[:, 0]) == {0, 2} and items[0, 0] == 0
    _check(items[items[:, 0] != 1], np.array([100, 0, 300]), [3e-6, 2e-6, 1e-6], 8, 4)
