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


def chord_warmup(lb, ub, N, n_pts, seed=0):
    """Warmup points for models too large for the LP restatement.

    Stand-in for createWarmupPtsGLPK at genome scale: for random directions
    N z (z ~ N(0, I)) through the feasible point 0, take the point where the
    chord leaves the box (alternately at its far and near end, as the LP
    warmup alternates max and min), then shrink every point toward the mean as
    createWarmupPtsGLPK.c:283-284 does (0.33 x + 0.67 centre).  The points lie
    in null(S) to FP64 rounding.
    """
    rng = np.random.default_rng(seed)
    n, d = N.shape
    pts = np.zeros((n, n_pts))
    block = 512
    for j0 in range(0, n_pts, block):
        j1 = min(n_pts, j0 + block)
        Z = rng.standard_normal((d, j1 - j0))
        D = N @ Z  # n x b directions
        with np.errstate(divide="ignore", invalid="ignore"):
            up = np.where(D > 0, ub[:, None] / D, np.where(D < 0, lb[:, None] / D, np.inf))
            lo = np.where(D > 0, lb[:, None] / D, np.where(D < 0, ub[:, None] / D, -np.inf))
        tmax = np.min(up, axis=0)
        tmin = np.max(lo, axis=0)
        sign = np.where((np.arange(j0, j1) % 2) == 1, 1.0, 0.0)
        t = sign * tmax + (1.0 - sign) * tmin
        t = np.where(np.isfinite(t), t, 0.0)
        pts[:, j0:j1] = D * t[None, :]
    pts = np.minimum(np.maximum(pts, lb[:, None]), ub[:, None])
    centre = pts.mean(axis=1)
    return pts * 0.33 + 0.67 * centre[:, None]


def ideal_bytes_per_chain_step(n: int) -> int:
    """Algorithmic HBM bytes of one plain chain-step: w_r read, x and c read+write (5 n doubles)."""
    return 40 * n


def log_uniform_sizes(count, lo, hi, seed):
    rng = np.random.default_rng(seed)
    return [int(round(math.exp(v))) for v in rng.uniform(math.log(lo), math.log(hi), size=count)]
