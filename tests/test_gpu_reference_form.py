"""GPU parity in the configurations the benchmark times, on the reference's input form.

The bench runs the default chain-kernel configuration for its model size
(384 threads x 10 reactions per thread for 2049-3840 reactions, 512 x 15 for
6145-7680) on generator-law models; the reference's warmup CSV is written with
"%f" (VFWarmup/createWarmupPtsGLPK.c:292), so its residual check
(ACHRcu/ACHRCuda.cu:325-343) reprojects at nearly every check.  Here the GPU
runs exactly that: generator-law models at 2766 x 3742 and 5063 x 7440 and the
reference's own P_Putida model (911 x 1060, non-integer coefficients), warmup
points passed through the library's %f writer and CSV reader, and every
reprojection form.  Bar: points within 1e-10 of the oracle (relative to
max(1, max|x|)) with equal accepted, rejected, check and reprojection counts,
and reprojections > 0.
"""
from __future__ import annotations

import importlib

import numpy as np
import pytest

from cases import reference_form_case, rel_err

pytestmark = pytest.mark.gpu

REL_TOL = 1e-10


@pytest.fixture(scope="module")
def synth(pkg):
    return importlib.import_module("achr_gb300.synthetic")


@pytest.fixture(scope="module")
def genome_case(pkg, native, synth, tmp_path_factory):
    model, warm = reference_form_case(pkg, synth.GENOME, 1024, tmp_path_factory.mktemp("genome"))
    with pkg.Sampler(model, warm) as s:
        N = s.null_space()
    return model, warm, N


@pytest.fixture(scope="module")
def large_case(pkg, native, synth, tmp_path_factory):
    model, warm = reference_form_case(pkg, synth.LARGE, 1024, tmp_path_factory.mktemp("large"))
    with pkg.Sampler(model, warm) as s:
        N = s.null_space()
    return model, warm, N


def _check(pkg, oracle_mod, model, warm, N, P, T, seed, **opts):
    with pkg.Sampler(model, warm, **opts) as s:
        s.set_null_space(N)
        pts, st = s.sample(P, T, seed=seed)
    ref, rst = oracle_mod.sample(model, warm, N, seed, P, T)
    err = rel_err(pts, ref)
    assert err <= REL_TOL, err
    assert st["accepted"] == rst["accepted"] == P * T
    assert st["rejected"] == rst["rejected"]
    assert st["checks"] == rst["checks"] > 0
    assert st["reprojections"] == rst["reprojections"] > 0
    assert (pts >= model.lb[:, None] - 1e-9).all() and (pts <= model.ub[:, None] + 1e-9).all()
    return st


def test_genome_warmups_carry_the_percent_f_residual(genome_case):
    model, warm, _ = genome_case
    r = np.abs(model.dense() @ warm).max()
    assert 1e-7 < r < 1e-4  # %f leaves |S w| far above the 1e-9 trigger


@pytest.mark.parametrize("form", [0, 2], ids=["default_fp64_projector", "residual_form"])
def test_genome_384x10_matches_oracle(pkg, oracle_mod, genome_case, form):
    """2766 x 3742, the bench's model and configuration (384 x 10, merged brackets, padding skip,
    sliced-ELL residual checks); 32 chains x 50 steps."""
    model, warm, N = genome_case
    assert model.n_rxns == 3742 and N.shape[1] * model.n_rxns < 4e6  # default: N (N^T x) in FP64
    _check(pkg, oracle_mod, model, warm, N, 32, 50, seed=4242, reproject_form=form)


def test_genome_384x10_separate_bracket_pass(pkg, oracle_mod, genome_case):
    model, warm, N = genome_case
    _check(pkg, oracle_mod, model, warm, N, 16, 30, seed=77, bracket_pass=1)


@pytest.mark.parametrize("form", [0, 1], ids=["default_residual_form", "fp64_projector"])
def test_large_512x15_matches_oracle(pkg, oracle_mod, large_case, form):
    """5063 x 7440 (512 x 15, one CTA per SM); 16 chains x 30 steps."""
    model, warm, N = large_case
    assert model.n_rxns == 7440 and N.shape[1] * model.n_rxns >= 4e6  # default: the residual form
    _check(pkg, oracle_mod, model, warm, N, 16, 30, seed=515, reproject_form=form)


def test_putida_matches_oracle(pkg, native, oracle_mod, putida_files):
    """The reference's own model and a 2n %f warmup CSV made from it; 64 chains x 50 steps."""
    mps, csv = putida_files
    model = pkg.read_mps(mps)
    warm = pkg.read_warmup_csv(csv, model.n_rxns)
    with pkg.Sampler(model, warm) as s:
        N = s.null_space()
    st = _check(pkg, oracle_mod, model, warm, N, 64, 50, seed=2024)
    assert st["reprojections"] >= 64 * 4  # every chain reprojects at most of its 5 checks


def _z_scores(a, b):
    """z of the mean and of the standard-deviation difference per flux (rows), chains in columns."""
    na, nb = a.shape[1], b.shape[1]
    ma, mb = a.mean(axis=1), b.mean(axis=1)
    va, vb = a.var(axis=1, ddof=1), b.var(axis=1, ddof=1)
    moving = (va > 1e-18) | (vb > 1e-18)
    se_m = np.sqrt(va / na + vb / nb)
    sa, sb = np.sqrt(va), np.sqrt(vb)

    def se_sd(x, s, nx):
        k = ((x - x.mean(axis=1, keepdims=True)) ** 4).mean(axis=1) / np.maximum(s ** 4, 1e-300)
        return s * np.sqrt(np.maximum(k - 1.0, 1e-12) / (4.0 * nx))

    se_s = np.sqrt(se_sd(a, sa, na) ** 2 + se_sd(b, sb, nb) ** 2)
    zm = np.where(moving, (ma - mb) / np.where(moving, se_m, 1.0), 0.0)
    zs = np.where(moving, (sa - sb) / np.where(moving, se_s, 1.0), 0.0)
    return zm, zs, moving


def test_genome_flux_moments_match_oracle_within_3_se(pkg, oracle_mod, genome_case):
    """Independent chains (disjoint chain ids): per-flux means and standard deviations of 2000
    GPU chains and 2000 oracle chains after 60 steps agree within 3 standard errors.  Over
    k ~ 3500 moving fluxes about 0.27 % exceed 3 by chance (fluxes are correlated, so the count
    varies more than binomially): at most 1 % may, and none may exceed 5.5."""
    model, warm, N = genome_case
    P, T = 2000, 60
    with pkg.Sampler(model, warm) as s:
        s.set_null_space(N)
        gpu, _ = s.sample(P, T, seed=8)
    cpu, _ = oracle_mod.sample(model, warm, N, 8, P, T, chain_offset=10 ** 6)
    zm, zs, moving = _z_scores(gpu, cpu)
    k = int(moving.sum())
    assert k > 3000
    for z in (zm, zs):
        assert np.abs(z).max() <= 5.5, np.sort(np.abs(z))[-5:]
        assert int((np.abs(z) > 3).sum()) <= 0.01 * k, int((np.abs(z) > 3).sum())
