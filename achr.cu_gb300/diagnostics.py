"""Convergence diagnostics of sampler traces: rank-normalised split-R-hat and bulk ESS.

Definitions follow Vehtari, Gelman, Simpson, Carpenter and Buerkner, "Rank-
normalization, folding, and localization: an improved R-hat for assessing
convergence of MCMC" (Bayesian Analysis, 2021):

* every chain is split into two halves;
* draws are replaced by the normal scores of their pooled fractional ranks,
  Phi^-1((r - 3/8) / (S + 1/4)), ties sharing their average rank;
* split-R-hat = sqrt(var+ / W) with W the mean within-chain variance, B / n the
  variance of the chain means and var+ = (n - 1) / n W + B / n; the reported
  R-hat is the larger of the bulk value and the value on the folded draws
  |x - median|;
* bulk ESS = S / tau with tau = -1 + 2 sum_k P_k, where P_k = rho_2k + rho_2k+1
  are sums of the combined autocorrelation estimates
  rho_t = 1 - (W - mean_j acov_j(t)) / var+, truncated at the first negative P_k
  and made monotone non-increasing (Geyer's initial monotone sequence).

Arrays are (chains, draws, parameters); everything is vectorised over the
parameters.  The sampler produces the traces (achr_sample_resume segments);
this module only evaluates them.
"""
from __future__ import annotations

import numpy as np
from scipy.special import ndtri
from scipy.stats import rankdata


def _split(x: np.ndarray) -> np.ndarray:
    m, n, p = x.shape
    h = n // 2
    return np.concatenate([x[:, :h], x[:, n - h:]], axis=0)


def _rank_normal(x: np.ndarray) -> np.ndarray:
    m, n, p = x.shape
    flat = x.reshape(m * n, p)
    r = rankdata(flat, axis=0, method="average")
    z = ndtri((r - 0.375) / (m * n + 0.25))
    return z.reshape(m, n, p)


def _rhat_core(z: np.ndarray) -> np.ndarray:
    m, n, _ = z.shape
    means = z.mean(axis=1)
    w = z.var(axis=1, ddof=1).mean(axis=0)
    b_over_n = means.var(axis=0, ddof=1)
    var_plus = (n - 1) / n * w + b_over_n
    with np.errstate(divide="ignore", invalid="ignore"):
        return np.sqrt(var_plus / w)


def split_rhat(draws: np.ndarray) -> np.ndarray:
    """Rank-normalised split-R-hat, max of bulk and folded, per parameter."""
    x = _split(np.asarray(draws, dtype=np.float64))
    bulk = _rhat_core(_rank_normal(x))
    folded = _rhat_core(_rank_normal(np.abs(x - np.median(x.reshape(-1, x.shape[2]), axis=0))))
    return np.fmax(bulk, folded)


def _autocov(z: np.ndarray) -> np.ndarray:
    """Biased autocovariance of every chain and parameter, lags 0..n-1 (FFT)."""
    m, n, p = z.shape
    zc = z - z.mean(axis=1, keepdims=True)
    size = 1 << int(np.ceil(np.log2(2 * n)))
    f = np.fft.rfft(zc, n=size, axis=1)
    ac = np.fft.irfft(f * np.conj(f), n=size, axis=1)[:, :n] / n
    return ac


def bulk_ess(draws: np.ndarray) -> np.ndarray:
    """Bulk effective sample size per parameter (rank-normalised split chains)."""
    z = _rank_normal(_split(np.asarray(draws, dtype=np.float64)))
    m, n, p = z.shape
    acov = _autocov(z)
    w = z.var(axis=1, ddof=1).mean(axis=0)
    b_over_n = z.mean(axis=1).var(axis=0, ddof=1)
    var_plus = (n - 1) / n * w + b_over_n
    with np.errstate(divide="ignore", invalid="ignore"):
        rho = 1.0 - (w[None, :] - acov.mean(axis=0) * n / (n - 1)) / var_plus[None, :]  # (lags, p)
    rho[0] = 1.0
    npairs = n // 2
    pairs = rho[: 2 * npairs].reshape(npairs, 2, p).sum(axis=1)  # P_k
    # truncate at the first negative pair sum, then force monotone non-increasing
    neg = pairs < 0
    first_neg = np.where(neg.any(axis=0), neg.argmax(axis=0), npairs)
    keep = np.arange(npairs)[:, None] < first_neg[None, :]
    pairs = np.where(keep, pairs, 0.0)
    pairs = np.minimum.accumulate(np.where(keep, pairs, np.inf), axis=0)
    pairs = np.where(keep, pairs, 0.0)
    tau = -1.0 + 2.0 * pairs.sum(axis=0)
    tau = np.maximum(tau, 1.0 / np.log10(m * n))  # the published lower cap on tau
    return m * n / tau


def summarize(draws: np.ndarray, frozen_tol: float = 1e-9, exclude=None) -> dict:
    """min ESS, max R-hat and their parameters; draws (chains, draws, params).

    A parameter whose draws all lie within frozen_tol * max(1, |median|) of
    each other is frozen (a blocked reaction, or one pinned by the constraints
    and moving only by rounding): it has no meaningful ESS or R-hat and is
    counted separately.  exclude (boolean per parameter) marks parameters known
    to be pinned -- for fluxes, those with one value in every warmup point --
    which are left out even when rounding drift over a long run moves them
    past frozen_tol."""
    x = np.asarray(draws, dtype=np.float64)
    flat = x.reshape(-1, x.shape[2])
    spread = flat.max(axis=0) - flat.min(axis=0)
    moving = spread > frozen_tol * np.maximum(1.0, np.abs(np.median(flat, axis=0)))
    if exclude is not None:
        moving &= ~np.asarray(exclude, dtype=bool)
    ess = np.full(x.shape[2], np.nan)
    rhat = np.full(x.shape[2], np.nan)
    if moving.any():
        ess[moving] = bulk_ess(x[:, :, moving])
        rhat[moving] = split_rhat(x[:, :, moving])
    finite = np.isfinite(ess) & np.isfinite(rhat)
    if not finite.any():
        return {"min_ess": float("nan"), "max_rhat": float("nan"), "params": 0}
    e = np.where(finite, ess, np.inf)
    r = np.where(finite, rhat, -np.inf)
    rf = rhat[finite]
    return {"min_ess": float(e.min()), "argmin_ess": int(e.argmin()), "max_rhat": float(r.max()),
            "argmax_rhat": int(r.argmax()), "median_rhat": float(np.median(rf)),
            "rhat_q99": float(np.quantile(rf, 0.99)), "median_ess": float(np.median(ess[finite])),
            "params": int(finite.sum()), "frozen_params": int((~finite).sum())}
