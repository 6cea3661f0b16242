"""Pure-Python restatement of the reference sampler -- TEST INFRASTRUCTURE ONLY.

An implementation independent of achr_oracle.c (own Philox, own loops), used
to cross-check the C oracle and to generate the committed golden fixtures.
Slow: for small models and few chains only.

Follows marouenbg/ACHR.cu:
  computeKernelCuda   ACHRcu/ACHRCuda.cu:436-502 (SVD of S^T S, cutoff n*sigma0*2.2204e-16)
  createCenterPt      ACHRcu/ACHRCuda.cu:414-434
  step loop           ACHRcu/ACHRCuda.cu:193-385 (see achr_oracle.c for the line map)
with the counter-based random stream of the GPU build instead of cuRAND XORWOW.
"""
from __future__ import annotations

import math

import numpy as np

MASK = 0xFFFFFFFF
EPSILON = 2.2204e-16  # ACHRCuda.cu:41


def philox4x32_10(ctr, key):
    """Philox4x32-10 (Salmon et al., SC'11)."""
    c0, c1, c2, c3 = (int(x) & MASK for x in ctr)
    k0, k1 = (int(x) & MASK for x in key)
    for _ in range(10):
        p0 = 0xD2511F53 * c0
        p1 = 0xCD9E8D57 * c2
        c0, c1, c2, c3 = ((p1 >> 32) ^ c1 ^ k0) & MASK, p1 & MASK, ((p0 >> 32) ^ c3 ^ k1) & MASK, p0 & MASK
        k0 = (k0 + 0x9E3779B9) & MASK
        k1 = (k1 + 0xBB67AE85) & MASK
    return [c0, c1, c2, c3]


def draw(seed, chain, step, attempt):
    return philox4x32_10([step, attempt, chain & MASK, chain >> 32], [seed & MASK, seed >> 32])


def warmup_index(seed, chain, step, attempt, W):
    return (draw(seed, chain, step, attempt)[0] * W) >> 32


def step_uniform(seed, chain, step):
    w = draw(seed, chain, step, 0)
    bits = (w[2] << 32) | w[3]
    return ((bits >> 12) + 0.5) * 2.0 ** -52


def null_space_sts(S):
    """N from the SVD of S^T S with the reference's cutoff (ACHRCuda.cu:459-489)."""
    S = np.asarray(S, dtype=np.float64)
    n = S.shape[1]
    StS = S.T @ S
    _, sv, vh = np.linalg.svd(StS)
    tol = n * sv[0] * EPSILON
    istart = 0
    for i in range(n):
        if sv[i] < tol:
            istart = i
            break
    return vh.T[:, istart:].copy()


def centre(warmup):
    w = np.asarray(warmup, dtype=np.float64)
    alpha = 1.0 / w.shape[1]
    return np.array([alpha * math.fsum(row) for row in w])


def sample_chain(S_rows, lb, ub, warmup, N, c0, seed, chain, T, check_period=10, max_attempts=100000,
                 centre_offset=0, residual_tol=1e-9, max_min_tol=1e-9, u_tol=1e-9, d_tol=1e-14):
    """One chain.  S_rows: list of (cols, vals) per metabolite.  Returns (x, n_rejected)."""
    n, W = warmup.shape
    c = [float(v) for v in c0]
    prev = list(c)
    x = [0.0] * n
    rejected = 0
    for s in range(T):
        U = step_uniform(seed, chain, s)
        att = 0
        while True:
            if att >= max_attempts:
                return np.array(x), rejected, True
            r = warmup_index(seed, chain, s, att, W)
            att += 1
            w = warmup[:, r]
            u = [float(w[i]) - c[i] for i in range(n)]
            ss = 0.0
            for v in u:
                ss += v * v
            norm = math.sqrt(ss)
            k = 0
            mn_best = mx_best = 0.0
            for i in range(n):
                u[i] = u[i] / norm if norm != 0.0 else float("nan")
                dub = ub[i] - prev[i]
                dlb = prev[i] - lb[i]
                if dub > d_tol and dlb > d_tol:
                    if u[i] > u_tol:
                        mn, mx = -dlb / u[i], dub / u[i]
                    elif u[i] < -u_tol:
                        mn, mx = dub / u[i], -dlb / u[i]
                    else:
                        continue
                    if k == 0 or mn > mn_best:
                        mn_best = mn
                    if k == 0 or mx < mx_best:
                        mx_best = mx
                    k += 1
            if k == 0 or (abs(mn_best) < max_min_tol and abs(mx_best) < max_min_tol) or mn_best > mx_best:
                rejected += 1
                continue
            t = U * (mx_best - mn_best) + mn_best
            x = [prev[i] + t * u[i] for i in range(n)]
            if s % check_period == 0:
                res = 0.0
                for cols, vals in S_rows:
                    acc = 0.0
                    for cc, vv in zip(cols, vals):
                        acc += vv * x[cc]
                    res = max(res, abs(acc))
                if res > residual_tol:
                    xv = np.array(x)
                    tmp = [float(np.dot(N[:, j], xv)) for j in range(N.shape[1])]
                    x = [float(np.dot(N[i, :], tmp)) for i in range(n)]
            tc = s + centre_offset
            alpha = (W + tc) / (W + tc + 1.0)
            beta = 1.0 / (W + tc + 1.0)
            for i in range(n):
                if x[i] > ub[i]:
                    x[i] = float(ub[i])
                elif x[i] < lb[i]:
                    x[i] = float(lb[i])
                prev[i] = x[i]
                c[i] = alpha * c[i] + beta * x[i]
            break
    return np.array(x), rejected, False


def rows_of(n_mets, row, col, val):
    acc = {}
    for r, c, v in zip(np.asarray(row).tolist(), np.asarray(col).tolist(), np.asarray(val).tolist()):
        acc[(r, c)] = acc.get((r, c), 0.0) + v
    rows = [([], []) for _ in range(n_mets)]
    for (r, c) in sorted(acc):
        if acc[(r, c)] != 0.0:
            rows[r][0].append(c)
            rows[r][1].append(acc[(r, c)])
    return rows
