"""FP64 numpy oracle of the learned direction preconditioner -- TEST INFRASTRUCTURE ONLY.

Only tests/, smoke() and bench.py's baseline legs may import this module; the
product (the CUDA library) never does.  The preconditioner has no reference
counterpart (the reference's only direction rule is ACHR's, ACHRcu/ACHRCuda.cu:
260-264), so this restates the model directly from its definition:

    C = diag(exp(2 s)) + U U^T                     (direction covariance, d x d)
    loss(s, U; Y) = 1/2 tr(C^-1 Y Y^T / B) + 1/2 log det C

for a minibatch Y (d x B) of centred null-space coordinates.  Gradients are
computed from the dense matrices (C^-1 explicitly), independently of the
Woodbury form the GPU kernels use, and are themselves checked against central
finite differences in tests/test_precond_oracle.py.
"""
from __future__ import annotations

import numpy as np


def covariance(s, U):
    s = np.asarray(s, dtype=np.float64)
    U = np.asarray(U, dtype=np.float64)
    return np.diag(np.exp(2.0 * s)) + U @ U.T


def loss(s, U, Y):
    Y = np.asarray(Y, dtype=np.float64)
    C = covariance(s, U)
    sign, logdet = np.linalg.slogdet(C)
    Ci = np.linalg.inv(C)
    B = Y.shape[1]
    return 0.5 * np.trace(Ci @ (Y @ Y.T)) / B + 0.5 * logdet


def loss_grad(s, U, Y):
    """(loss, d loss / d s, d loss / d U), all FP64."""
    s = np.asarray(s, dtype=np.float64)
    U = np.asarray(U, dtype=np.float64)
    Y = np.asarray(Y, dtype=np.float64)
    B = Y.shape[1]
    C = covariance(s, U)
    Ci = np.linalg.inv(C)
    Sig = Y @ Y.T / B
    G = 0.5 * (Ci - Ci @ Sig @ Ci)  # d loss / d C (symmetric)
    gU = 2.0 * G @ U
    gs = 2.0 * np.exp(2.0 * s) * np.diag(G)
    sign, logdet = np.linalg.slogdet(C)
    val = 0.5 * np.trace(Ci @ Sig) + 0.5 * logdet
    return val, gs, gU


def kl_to_sample_covariance(s, U, Y):
    """KL( N(0, Sigma) || N(0, C) ) with Sigma = Y Y^T / B."""
    Y = np.asarray(Y, dtype=np.float64)
    d, B = Y.shape
    Sig = Y @ Y.T / B
    C = covariance(s, U)
    _, ld_c = np.linalg.slogdet(C)
    _, ld_s = np.linalg.slogdet(Sig)
    return 0.5 * (np.trace(np.linalg.solve(C, Sig)) - d + ld_c - ld_s)
