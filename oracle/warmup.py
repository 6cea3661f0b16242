"""Warmup points by restating VFWarmup/createWarmupPtsGLPK.c with scipy's HiGHS.

TEST FIXTURE TOOLING, not product code: the sampler takes warmup points as an
input, and the LP warmup is deliberately not ported to the GPU.  GLPK and MPI
are absent here, so this restatement produces the fixture CSVs for small
models.  It follows the reference's procedure:

  * nPts = max(nPts, 2n)                                   createWarmupPtsGLPK.c:238-245
  * for i in [0, nPts/2): objective e_i for i < n, else U(-0.5, 0.5) per
    coefficient; solve max (column 2i+1) and min (column 2i)  :100-114, :168-173
  * clip the LP solution to [lb, ub]                          :166 (movePtsBds :36-46)
  * centre = mean of the points; every point -> 0.33 x + 0.67 centre  :283-284, :48-65
  * written with "%f", values separated by ',' (one line per reaction)  :286-298

HiGHS and GLPK return different optimal vertices when an LP has several, so
the points are equivalent in role, not identical to GLPK's.
"""
from __future__ import annotations

import numpy as np


def _solve_pair(job):
    """Max and min of one objective over {S v = 0, lb <= v <= ub}, clipped to the box."""
    from scipy.optimize import linprog

    S, lb, ub, obj = job
    m, n = S.shape
    bounds = [(None if np.isinf(l) else l, None if np.isinf(u) else u) for l, u in zip(lb, ub)]
    out = []
    for j in (+1, -1):
        # linprog minimises: maximise obj.v as minimise -obj.v
        res = linprog(-j * obj, A_eq=S, b_eq=np.zeros(m), bounds=bounds, method="highs-ds")
        x = res.x if res.status == 0 else np.zeros(n)
        out.append(np.minimum(np.maximum(x, lb), ub))
    return out  # [max, min]


def lp_warmup(S, lb, ub, n_pts, seed=0, workers=1):
    """workers > 1 solves the LPs in a spawned process pool (same points, any order)."""
    import scipy.sparse as sp

    S = sp.csr_matrix(np.asarray(S.todense() if hasattr(S, "todense") else S, dtype=np.float64))
    lb = np.asarray(lb, dtype=np.float64)
    ub = np.asarray(ub, dtype=np.float64)
    m, n = S.shape
    n_pts = max(int(n_pts), 2 * n)
    half = n_pts // 2
    rng = np.random.default_rng(seed)
    objs = []
    for i in range(half):
        if i < n:
            obj = np.zeros(n)
            obj[i] = 1.0
        else:
            obj = rng.random(n) - 0.5
        objs.append(obj)
    jobs = [(S, lb, ub, o) for o in objs]
    if workers > 1:
        import multiprocessing as mp

        with mp.get_context("spawn").Pool(workers) as pool:
            pairs = pool.map(_solve_pair, jobs, chunksize=8)
    else:
        pairs = [_solve_pair(j) for j in jobs]
    flux = np.zeros((n, n_pts))
    for i, (xmax, xmin) in enumerate(pairs):
        flux[:, 2 * i + 1] = xmax
        flux[:, 2 * i] = xmin
    centre = flux.mean(axis=1)
    return flux * 0.33 + 0.67 * centre[:, None]


def write_csv(path, warmup):
    """%f text, one line per reaction, as createWarmupPtsGLPK.c:289-297 writes it."""
    with open(path, "w") as f:
        for row in np.asarray(warmup):
            f.write(",".join("%f" % v for v in row))
            f.write("\n")
