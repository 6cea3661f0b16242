"""CPU: the FP64 oracle of the preconditioner's loss and gradients against finite differences."""
from __future__ import annotations

import numpy as np

from oracle import precond


def _problem(seed=0, d=12, r=3, B=40):
    rng = np.random.default_rng(seed)
    s = 0.3 * rng.standard_normal(d)
    U = 0.5 * rng.standard_normal((d, r))
    Y = rng.standard_normal((d, B)) * np.exp(rng.uniform(-1, 1, (d, 1)))
    return s, U, Y


def test_gradients_match_finite_differences():
    s, U, Y = _problem()
    val, gs, gU = precond.loss_grad(s, U, Y)
    assert np.isclose(val, precond.loss(s, U, Y))
    h = 1e-6
    for i in range(len(s)):
        e = np.zeros_like(s)
        e[i] = h
        fd = (precond.loss(s + e, U, Y) - precond.loss(s - e, U, Y)) / (2 * h)
        assert abs(fd - gs[i]) <= 1e-6 * max(1.0, abs(fd))
    for i in range(U.shape[0]):
        for j in range(U.shape[1]):
            E = np.zeros_like(U)
            E[i, j] = h
            fd = (precond.loss(s, U + E, Y) - precond.loss(s, U - E, Y)) / (2 * h)
            assert abs(fd - gU[i, j]) <= 1e-6 * max(1.0, abs(fd))


def test_loss_is_minimised_by_the_sample_covariance():
    """At C = Sigma the KL is zero and the gradient vanishes (full-rank model)."""
    rng = np.random.default_rng(3)
    d, B = 6, 4000
    A = rng.standard_normal((d, d))
    Y = A @ rng.standard_normal((d, B))
    Sig = Y @ Y.T / B
    # represent Sigma exactly: diagonal part exp(2 s) = delta below its smallest
    # eigenvalue and U = chol(Sigma - delta I)
    delta = 0.5 * np.linalg.eigvalsh(Sig).min()
    s = np.full(d, 0.5 * np.log(delta))
    U = np.linalg.cholesky(Sig - delta * np.eye(d))
    assert abs(precond.kl_to_sample_covariance(s, U, Y)) < 1e-10
    _, gs, gU = precond.loss_grad(s, U, Y)
    assert np.abs(gs).max() < 1e-9 and np.abs(gU).max() < 1e-9
