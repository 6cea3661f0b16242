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


def _check(pkg, oracle_mod, model, warm, N, P, T, seed, tol=REL_TOL, oracle_opts=None, **opts):
    with pkg.Sampler(model, warm, **opts) as s:
        s.set_null_space(N)
        pts, st = s.sample(P, T, seed=seed)
    ref, rst = oracle_mod.sample(model, warm, N, seed, P, T, **(oracle_opts or {}))
    err = rel_err(pts, ref)
    counts = {k: (st[k], rst[k]) for k in ("accepted", "rejected", "checks", "reprojections")}
    assert st["accepted"] == rst["accepted"] == P * T, counts
    assert st["rejected"] == rst["rejected"], counts
    assert st["checks"] == rst["checks"] > 0, counts
    assert st["reprojections"] == rst["reprojections"] > 0, counts
    assert err <= tol, (err, counts)
    assert (pts >= model.lb[:, None] - 1e-9).all() and (pts <= model.ub[:, None] + 1e-9).all()
    return st


def test_genome_warmups_carry_the_percent_f_residual(genome_case):
    model, warm, _ = genome_case
    r = np.abs(model.dense() @ warm).max()
    assert 1e-7 < r < 1e-4  # %f leaves |S w| far above the 1e-9 trigger


GENOME_FORMS = [
    ({"reproject_form": 0}, True),   # chosen by the inputs: %f warmups at this size -> deferred
    ({"reproject_form": 1}, False),  # N (N^T x) in FP64 inside the chain kernel
    ({"reproject_form": 2}, False),  # residual form inside the chain kernel
    ({"reproject_form": 3, "reprojection_passes": 4}, True),
    ({"reproject_form": 3, "reprojection_passes": 8}, True),
]


@pytest.mark.parametrize("opts,deferred", GENOME_FORMS,
                         ids=["auto_deferred", "fp64_projector", "residual_form", "deferred_4pass", "deferred_8pass"])
def test_genome_384x10_matches_oracle(pkg, oracle_mod, genome_case, opts, deferred):
    """2766 x 3742, the bench's model and configuration (384 x 10, merged brackets, padding skip,
    sliced-ELL residual checks); 32 chains x 50 steps, every reprojection form."""
    model, warm, N = genome_case
    assert model.n_rxns == 3742
    st = _check(pkg, oracle_mod, model, warm, N, 32, 50, seed=4242, **opts)
    assert (st["segments"] > 0) == deferred


def test_genome_384x10_separate_bracket_pass(pkg, oracle_mod, genome_case):
    model, warm, N = genome_case
    _check(pkg, oracle_mod, model, warm, N, 16, 30, seed=77, bracket_pass=1)


@pytest.mark.parametrize("form,deferred", [(0, True), (1, False), (2, False)],
                         ids=["auto_deferred", "fp64_projector", "residual_form"])
def test_large_512x15_matches_oracle(pkg, oracle_mod, large_case, form, deferred):
    """5063 x 7440 (512 x 15, one CTA per SM); 16 chains x 30 steps."""
    model, warm, N = large_case
    assert model.n_rxns == 7440
    st = _check(pkg, oracle_mod, model, warm, N, 16, 30, seed=515, reproject_form=form)
    assert (st["segments"] > 0) == deferred


@pytest.fixture(scope="module")
def putida_case(pkg, native, putida_files):
    mps, csv = putida_files
    model = pkg.read_mps(mps)
    warm = pkg.read_warmup_csv(csv, model.n_rxns)
    with pkg.Sampler(model, warm) as s:
        N = s.null_space()
    return model, warm, N


def _oracle_sensitivity(oracle_mod, model, warm, N, P, T, seed, **kw):
    """How far the oracle's own points move when N is perturbed by 1e-15 relative (a rounding-
    level change): the spread any FP64 evaluation order can show on this model."""
    rng = np.random.default_rng(0)
    a, _ = oracle_mod.sample(model, warm, N, seed, P, T, **kw)
    b, _ = oracle_mod.sample(model, warm, N * (1.0 + 1e-15 * rng.standard_normal(N.shape)), seed, P, T, **kw)
    return rel_err(a, b)


@pytest.mark.parametrize("form", [0, 1], ids=["auto", "fp64_projector"])
def test_putida_matches_oracle_well_conditioned(pkg, oracle_mod, putida_case, form):
    """The reference's own model with a 2n %f warmup CSV made from it, 64 chains x 50 steps, at
    u_tol = 1e-4: ratio-test candidates then have |u_i| > 1e-4, the oracle is insensitive to
    rounding (a 1e-15 change of N moves its points by ~1e-11), and the bar is the usual 1e-10."""
    model, warm, N = putida_case
    assert _oracle_sensitivity(oracle_mod, model, warm, N, 64, 50, 2024, u_tol=1e-4) < 1e-10
    _check(pkg, oracle_mod, model, warm, N, 64, 50, seed=2024, oracle_opts={"u_tol": 1e-4}, u_tol=1e-4,
           reproject_form=form)


@pytest.mark.parametrize("form", [0, 1], ids=["auto", "fp64_projector"])
def test_putida_matches_oracle_reference_tolerances(pkg, oracle_mod, putida_case, form):
    """Same at the reference's u_tol = 1e-9 (ACHRCuda.cu:508).  There a coordinate with |u_i|
    just above 1e-9 (reactions with coefficients like 5e-5) can bound the step, t = dist / |u_i|,
    which multiplies rounding differences in x by up to ~1e8: the oracle's own points move by
    ~2e-8 under a 1e-15 change of N.  The GPU must take the same steps (equal counts) and stay
    within that spread; the well-conditioned test above pins the arithmetic."""
    model, warm, N = putida_case
    spread = _oracle_sensitivity(oracle_mod, model, warm, N, 64, 50, 2024)
    assert spread > 1e-10  # the model really is this sensitive at the reference's tolerance
    _check(pkg, oracle_mod, model, warm, N, 64, 50, seed=2024, tol=max(REL_TOL, 10 * spread), reproject_form=form)


def test_putida_keeps_reprojection_in_the_chain_kernel(pkg, putida_case):
    """S S^T of P_Putida has a condition number near 1e8 (coefficients from 5e-5 to 45): the
    BF16-split passes of the deferred reprojection would not converge, so the automatic choice
    reprojects in the chain kernel (FP64) and an explicit request for the deferred form is refused."""
    model, warm, N = putida_case
    with pkg.Sampler(model, warm) as s:
        _, st = s.sample(8, 12, seed=1)
        assert st["reprojections"] > 0 and st["segments"] == 0
    with pkg.Sampler(model, warm, reproject_form=3) as s:
        with pytest.raises(pkg.AchrError) as e:
            s.sample(8, 12, seed=1)
        assert e.value.status == 8


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
