"""Test inputs in the reference's own input form at the sizes the benchmark runs.

The reference reads its warmup points from the CSV that
VFWarmup/createWarmupPtsGLPK.c writes with "%f" (:289-297), read back at
ACHRcu/ACHRCuda.cu:675-689.  Six decimals leave |S w| near 1e-6, so the
reference's 10-step residual check (ACHRCuda.cu:325-343) reprojects nearly
every time it runs.  These helpers build seeded generator-law models (the
benchmark's law, achr_gb300.synthetic) and pass their warmup points through
the library's own %f writer and CSV reader, so the GPU and the oracle see
exactly the values a drop-in user's CSV would hold.
"""
from __future__ import annotations

import importlib

import numpy as np


def gpu_null_space_fn(pkg):
    """Null-space basis of a dense matrix through the library (cuSOLVER), for the chord warmups."""
    def null_space(SF):
        r, c = np.nonzero(SF)
        m = pkg.HostModel(SF.shape[1], SF.shape[0], r, c, SF[r, c], np.full(SF.shape[1], -1.0),
                          np.full(SF.shape[1], 1.0))
        with pkg.Sampler(m, np.zeros((SF.shape[1], 1))) as tmp:
            return tmp.null_space()
    return null_space


def percent_f_roundtrip(pkg, warm, tmp_dir, name="warmup.csv"):
    """Write an (n, W) warmup matrix as the reference's CSV (%f, one line per reaction) and read it back."""
    path = tmp_dir / name
    pkg.write_points_csv(path, warm)
    return pkg.read_warmup_csv(path, warm.shape[0])


def reference_form_case(pkg, spec, n_warmup, tmp_dir, seed=17):
    """(model, %f-rounded warmups) of a seeded generator-law model."""
    synth = importlib.import_module("achr_gb300.synthetic")
    row, col, val, lb, ub = synth.make_model(spec)
    S = synth.dense(spec.n_mets, spec.n_rxns, row, col, val)
    warm = synth.interior_chord_warmup(S, lb, ub, n_warmup, seed=spec.seed + seed, null_space=gpu_null_space_fn(pkg))
    model = pkg.HostModel(spec.n_rxns, spec.n_mets, row, col, val, lb, ub)
    return model, percent_f_roundtrip(pkg, warm, tmp_dir, f"warmup_{spec.n_rxns}.csv")


def rel_err(a, b):
    """Largest difference relative to max(1, max|b|), the parity tests' measure."""
    return float(np.abs(a - b).max() / max(1.0, np.abs(b).max()))


def refined_null_space(S, N):
    """N with its component in the row space of S removed, re-orthonormalised.

    A null-space basis from an FP64 factorisation is orthogonal to the rows of S
    only to a few 1e-15 (the small fixture's: 4.6e-15).  The deferred
    reprojection removes the row-space part of x itself, x - S^T (S S^T)^+ S x,
    while the oracle applies N (N^T x), so that residue separates the two, and
    a later hit-and-run step bounded by a tiny direction component can
    multiply it a thousandfold.  One application of the projector and a QR
    (signs fixed so the columns keep their direction) bring it to 6e-16.
    """
    S = np.asarray(S, dtype=np.float64)
    N1 = N - S.T @ (np.linalg.pinv(S @ S.T) @ (S @ N))
    Q, R = np.linalg.qr(N1)
    return np.ascontiguousarray(Q * np.sign(np.diag(R))[None, :])
