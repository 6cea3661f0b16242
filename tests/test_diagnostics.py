"""CPU: R-hat and ESS on draws with known answers."""
from __future__ import annotations

import importlib

import numpy as np
import pytest


@pytest.fixture(scope="module")
def diag(pkg):
    return importlib.import_module("achr_gb300.diagnostics")


def test_iid_draws(diag):
    rng = np.random.default_rng(0)
    x = rng.standard_normal((8, 1000, 5))
    r = diag.split_rhat(x)
    e = diag.bulk_ess(x)
    assert np.all(np.abs(r - 1.0) < 0.01)
    assert np.all(np.abs(e / 8000 - 1.0) < 0.15)


def test_ar1_ess(diag):
    """AR(1) with coefficient phi: ESS / S -> (1 - phi) / (1 + phi)."""
    rng = np.random.default_rng(1)
    phi, m, n = 0.8, 8, 4000
    x = np.zeros((m, n, 3))
    x[:, 0] = rng.standard_normal((m, 3)) / np.sqrt(1 - phi * phi)
    for t in range(1, n):
        x[:, t] = phi * x[:, t - 1] + rng.standard_normal((m, 3))
    e = diag.bulk_ess(x) / (m * n)
    assert np.all(np.abs(e - (1 - phi) / (1 + phi)) < 0.03)
    assert np.all(diag.split_rhat(x) < 1.01)


def test_shifted_chain_detected(diag):
    rng = np.random.default_rng(2)
    x = rng.standard_normal((4, 500, 2))
    x[0, :, 0] += 3.0  # one chain elsewhere in parameter 0
    r = diag.split_rhat(x)
    assert r[0] > 1.1 and r[1] < 1.02


def test_scale_mismatch_detected_by_folding(diag):
    rng = np.random.default_rng(3)
    x = rng.standard_normal((4, 2000, 1))
    x[0] *= 4.0  # same centre, wider spread: the folded R-hat sees it
    assert diag.split_rhat(x)[0] > 1.05


def test_frozen_parameter_excluded(diag):
    rng = np.random.default_rng(4)
    x = rng.standard_normal((4, 200, 3))
    x[:, :, 1] = 7.0
    s = diag.summarize(x)
    assert s["params"] == 2 and s["frozen_params"] == 1


def test_excluded_parameters_are_left_out(diag):
    rng = np.random.default_rng(6)
    x = rng.standard_normal((4, 300, 3))
    x[0, :, 2] += 1e-6 * np.arange(300)  # a "pinned" flux drifting by rounding in one chain
    s_all = diag.summarize(x)
    s_ex = diag.summarize(x, exclude=[False, False, True])
    assert s_all["params"] == 3 and s_ex["params"] == 2 and s_ex["frozen_params"] == 1
    assert s_ex["max_rhat"] <= s_all["max_rhat"]
