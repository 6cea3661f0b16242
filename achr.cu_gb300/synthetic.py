"""Seeded synthetic metabolic models and warmup points for tests and benchmarks.

Model law (a stand-in for the E. coli core / Recon2-scale models the
reference's paper uses, which are not available): every reaction touches 2-6
distinct metabolites (uniform) with integer coefficients drawn uniformly from
{-2, -1, 1, 2}; a fraction of the non-exchange reactions is irreversible
(lb = 0, ub = 1000), the rest have lb = -1000, ub = 1000; n_exchange reactions
are bounded +-exchange_bound.  v = 0 is feasible, so the polytope
{S v = 0, lb <= v <= ub} is bounded and non-empty.

Files are written in the fixed-MPS layout of the reference's own MPS writer
(VFWarmup/test_fva_validation.py:49-90): rows EQ<i>, columns X<j>, bounds
LO/UP/FX, empty RHS.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np


@dataclass
class SyntheticSpec:
    n_rxns: int
    n_mets: int
    irreversible_frac: float
    n_exchange: int
    exchange_bound: float
    seed: int


# The two single-model workloads of the benchmark plan: a 72 x 95 model sampled
# with 1000 chains x 1000 steps, and a genome-scale 2766 x 3742 model sampled
# with 100,000 chains x 2000 steps.
SMALL = SyntheticSpec(n_rxns=95, n_mets=72, irreversible_frac=0.25, n_exchange=20, exchange_bound=10.0, seed=1)
GENOME = SyntheticSpec(n_rxns=3742, n_mets=2766, irreversible_frac=0.30, n_exchange=150, exchange_bound=20.0, seed=2)
# The 5063 x 7440 model of the mixed-precision reprojection and learned-
# preconditioner workloads (262,144 chains x 5000 steps), same law as GENOME.
LARGE = SyntheticSpec(n_rxns=7440, n_mets=5063, irreversible_frac=0.30, n_exchange=150, exchange_bound=20.0, seed=4)


def make_model(spec: SyntheticSpec):
    """Return (row, col, val, lb, ub) of the seeded model."""
    rng = np.random.default_rng(spec.seed)
    n, m = spec.n_rxns, spec.n_mets
    rows, cols, vals = [], [], []
    coef = np.array([-2.0, -1.0, 1.0, 2.0])
    for j in range(n):
        k = int(rng.integers(2, 7))
        k = min(k, m)
        mets = rng.choice(m, size=k, replace=False)
        for r in np.sort(mets):
            rows.append(int(r))
            cols.append(j)
            vals.append(float(coef[rng.integers(0, 4)]))
    lb = np.full(n, -1000.0)
    ub = np.full(n, 1000.0)
    perm = rng.permutation(n)
    ex = perm[: spec.n_exchange]
    rest = perm[spec.n_exchange:]
    n_irr = int(round(spec.irreversible_frac * len(rest)))
    irr = rest[:n_irr]
    lb[irr] = 0.0
    lb[ex] = -spec.exchange_bound
    ub[ex] = spec.exchange_bound
    return (np.array(rows, dtype=np.int32), np.array(cols, dtype=np.int32), np.array(vals), lb, ub)


def host_model(spec: SyntheticSpec):
    from . import HostModel  # noqa: WPS433 (package-relative import)

    row, col, val, lb, ub = make_model(spec)
    return HostModel(spec.n_rxns, spec.n_mets, row, col, val, lb, ub)


def dense(n_mets, n_rxns, row, col, val):
    S = np.zeros((n_mets, n_rxns))
    np.add.at(S, (row, col), val)
    return S


def write_mps(path, n_mets, n_rxns, row, col, val, lb, ub, name="synthetic"):
    """Fixed-format MPS in the layout of VFWarmup/test_fva_validation.py:49-90."""
    order = np.lexsort((row, col))
    with open(path, "w") as f:
        f.write(f"{'NAME':<14}{name}\n")
        f.write("ROWS\n")
        f.write(" N  COST\n")
        for i in range(n_mets):
            f.write(f" E  EQ{i + 1}\n")
        f.write("COLUMNS\n")
        for q in order:
            cname = f"X{int(col[q]) + 1}"
            rname = f"EQ{int(row[q]) + 1}"
            f.write(f"    {cname:<10}{rname:<10}{val[q]:<12g}\n")
        f.write("RHS\n")
        f.write("BOUNDS\n")
        for j in range(n_rxns):
            cname = f"X{j + 1}"
            lo, up = lb[j], ub[j]
            if lo == 0 and up == 0:
                f.write(f" FX BOUND     {cname:<10}{0:<12g}\n")
            else:
                if lo != 0:
                    f.write(f" LO BOUND     {cname:<10}{lo:<12g}\n")
                f.write(f" UP BOUND     {cname:<10}{up:<12g}\n")
        f.write("ENDATA\n")


def interior_point(S, lb, ub, cap=50.0):
    """A feasible point with slack >= 1 on every reaction that can have it.

    One LP (HiGHS interior point): maximise sum(y) subject to S v = 0,
    y_i <= v_i - lb_i, y_i <= ub_i - v_i, 0 <= y_i <= cap.  Reactions left with
    y_i = 0 cannot leave their bound (blocked).  The LP solution is then moved
    back onto {S v = 0} with the blocked reactions held fixed (LSQR on S).
    Returns (v0, blocked_mask).
    """
    import scipy.sparse as sp
    from scipy.optimize import linprog
    from scipy.sparse.linalg import lsqr

    S = sp.csr_matrix(S)
    m, n = S.shape
    eye = sp.identity(n, format="csr")
    A_ub = sp.vstack([sp.hstack([-eye, eye]), sp.hstack([eye, eye])]).tocsr()
    b_ub = np.concatenate([-lb, ub])
    A_eq = sp.hstack([S, sp.csr_matrix((m, n))]).tocsr()
    bounds = [(lo, up) for lo, up in zip(lb, ub)] + [(0.0, cap)] * n
    c = np.concatenate([np.zeros(n), -np.ones(n)])
    res = linprog(c, A_ub=A_ub, b_ub=b_ub, A_eq=A_eq, b_eq=np.zeros(m), bounds=bounds, method="highs-ipm")
    if res.status != 0:
        raise RuntimeError(f"interior-point LP failed: {res.message}")
    v0 = res.x[:n].copy()
    blocked = res.x[n:] < 0.5e-3 * cap
    v0[blocked] = np.where(np.abs(v0[blocked] - lb[blocked]) <= np.abs(v0[blocked] - ub[blocked]), lb[blocked],
                           ub[blocked])
    free = ~blocked
    SF = S[:, free].tocsr()
    for _ in range(3):
        r = S @ v0
        delta = lsqr(SF, r, atol=1e-15, btol=1e-15, iter_lim=20000)[0]
        v0[free] -= delta
    v0 = np.minimum(np.maximum(v0, lb), ub)
    return v0, blocked


def interior_chord_warmup(S, lb, ub, n_pts, seed=0, null_space=None, interior=None):
    """Warmup points for genome-scale models (stand-in for createWarmupPtsGLPK).

    The reference generates one LP solution per warmup point (FVA extremes,
    VFWarmup/createWarmupPtsGLPK.c:100-173); at 3742 reactions one LP takes
    about 5 s here, so 7484 of them are out of reach.  Instead: from the
    interior point v0 (one LP), follow random directions P_F g (g ~ N(0, I),
    P_F the orthogonal projector onto the null space of S restricted to the
    non-blocked reactions) to where each chord leaves the box, alternating the
    far and near end as the reference alternates max and min; clip, and shrink
    toward the mean with 0.33 x + 0.67 centre (createWarmupPtsGLPK.c:283-284).
    The points satisfy S w = 0 to FP64 rounding.  null_space(S_F) -> basis
    may be supplied; the default uses numpy's symmetric eigensolver.  interior
    = (v0, blocked) from interior_point() may be supplied to skip the LP.
    """
    S = np.asarray(S.todense() if hasattr(S, "todense") else S, dtype=np.float64)
    lb = np.asarray(lb, dtype=np.float64)
    ub = np.asarray(ub, dtype=np.float64)
    v0, blocked = interior if interior is not None else interior_point(S, lb, ub)
    free = np.flatnonzero(~blocked)
    SF = S[:, free]
    if null_space is None:
        lam, V = np.linalg.eigh(SF.T @ SF)
        tol = len(free) * max(abs(lam).max(), 0.0) * 2.2204e-16
        NF = V[:, np.abs(lam) < tol]
    else:
        NF = null_space(SF)
    rng = np.random.default_rng(seed)
    n = S.shape[1]
    pts = np.empty((n, n_pts))
    lbF, ubF, vF = lb[free], ub[free], v0[free]
    block = 1024
    for j0 in range(0, n_pts, block):
        j1 = min(n_pts, j0 + block)
        G = rng.standard_normal((len(free), j1 - j0))
        D = NF @ (NF.T @ G)
        with np.errstate(divide="ignore", invalid="ignore"):
            up = np.where(D > 0, (ubF - vF)[:, None] / D, np.where(D < 0, (lbF - vF)[:, None] / D, np.inf))
            lo = np.where(D > 0, (lbF - vF)[:, None] / D, np.where(D < 0, (ubF - vF)[:, None] / D, -np.inf))
        tmax = np.min(up, axis=0)
        tmin = np.max(lo, axis=0)
        far = (np.arange(j0, j1) % 2) == 1
        t = np.where(far, tmax, tmin)
        t = np.where(np.isfinite(t), t, 0.0)
        pts[:, j0:j1] = v0[:, None]
        pts[free, j0:j1] = vF[:, None] + D * t[None, :]
    pts = np.minimum(np.maximum(pts, lb[:, None]), ub[:, None])
    centre = pts.mean(axis=1)
    return pts * 0.33 + 0.67 * centre[:, None]


def batch_spec(k: int, n: int) -> SyntheticSpec:
    """Model k of the 64-model batch workload: n reactions, 0.7 n metabolites."""
    return SyntheticSpec(n_rxns=n, n_mets=max(2, int(round(0.7 * n))), irreversible_frac=0.3,
                         n_exchange=max(2, n // 25), exchange_bound=20.0, seed=1000 + k)


def batch_interior(args):
    """(k, n) -> (k, v0, blocked) for the batch workload; runs in a worker process."""
    k, n = args
    spec = batch_spec(k, n)
    row, col, val, lb, ub = make_model(spec)
    v0, blocked = interior_point(dense(spec.n_mets, n, row, col, val), lb, ub)
    return k, v0, blocked


def ideal_bytes_per_chain_step(n: int) -> int:
    """Algorithmic HBM bytes of one plain chain-step: w_r read, x and c read+write (5 n doubles)."""
    return 40 * n


def log_uniform_sizes(count, lo, hi, seed):
    rng = np.random.default_rng(seed)
    return [int(round(math.exp(v))) for v in rng.uniform(math.log(lo), math.log(hi), size=count)]
