"""GPU: the tensor-core GEMM against PyTorch FP32, and the batched reprojection
against an FP64 projection of the same points."""
from __future__ import annotations

import importlib

import numpy as np
import pytest

from conftest import dense_S

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _gemm(pkg, A, B, A1=None, B1=None):
    M, K = A.shape
    N = B.shape[0]
    C = torch.full((M, N), float("nan"), dtype=torch.float32, device="cuda")
    pkg.gemm_bf16(M, N, K, A.data_ptr(), B.data_ptr(), C.data_ptr(), K, K, N,
                  A1=A1.data_ptr() if A1 is not None else 0, B1=B1.data_ptr() if B1 is not None else 0)
    return C


@pytest.mark.parametrize("M,N,K", [(128, 256, 64), (300, 520, 192), (1000, 257, 1024), (64, 40, 640)])
def test_gemm_bf16_matches_torch_fp32(pkg, M, N, K):
    g = torch.Generator(device="cuda").manual_seed(M * 7 + N)
    A = torch.randn(M, K, device="cuda", generator=g).to(torch.bfloat16)
    B = torch.randn(N, K, device="cuda", generator=g).to(torch.bfloat16)
    C = _gemm(pkg, A, B)
    ref = A.float() @ B.float().T  # BF16 products are exact in FP32; only the summation order differs
    scale = A.float().abs() @ B.float().abs().T
    assert torch.isfinite(C).all()
    err = (C - ref).abs()
    assert (err <= 1e-5 * scale + 1e-30).all(), float((err / scale).max())


def test_gemm_three_split_products_reach_fp32_accuracy(pkg):
    """A0 B0^T + A0 B1^T + A1 B0^T with hi/lo BF16 splits of FP64 data: relative error near 2^-16."""
    rng = np.random.default_rng(5)
    M, N, K = 256, 512, 448
    A = rng.standard_normal((M, K))
    B = rng.standard_normal((N, K)) * np.exp(rng.uniform(-3, 3, (N, 1)))  # rows of very different scale
    tA = torch.from_numpy(A).cuda()
    tB = torch.from_numpy(B).cuda()
    Ah = tA.to(torch.bfloat16)
    Al = (tA - Ah.double()).to(torch.bfloat16)
    Bh = tB.to(torch.bfloat16)
    Bl = (tB - Bh.double()).to(torch.bfloat16)
    C = _gemm(pkg, Ah, Bh, A1=Al, B1=Bl).double().cpu().numpy()
    ref = A @ B.T
    scale = np.abs(A) @ np.abs(B).T
    rel = np.abs(C - ref) / scale
    assert rel.max() < 3e-5
    # one BF16 product alone is far worse: the split terms are doing the work
    C1 = _gemm(pkg, Ah, Bh).double().cpu().numpy()
    assert (np.abs(C1 - ref) / scale).max() > 4 * rel.max()


def test_gemm_rejects_bad_shapes(pkg):
    A = torch.zeros(128, 64, dtype=torch.bfloat16, device="cuda")
    C = torch.zeros(128, 128, dtype=torch.float32, device="cuda")
    with pytest.raises(pkg.AchrError):
        pkg.gemm_bf16(128, 128, 60, A.data_ptr(), A.data_ptr(), C.data_ptr(), 64, 64, 128)  # K not a multiple of 64
    with pytest.raises(pkg.AchrError):
        pkg.gemm_bf16(128, 128, 64, A.data_ptr(), A.data_ptr(), C.data_ptr(), 60, 64, 128)  # lda not a multiple of 8


def _fp64_reprojection(S, lb, ub, X):
    """The oracle: x <- clip(N N^T x) with N N^T = I - S^T (S S^T)^+ S, all FP64 (numpy)."""
    B = np.linalg.pinv(S @ S.T, rcond=S.shape[0] * 2.2204e-16, hermitian=True)
    Y = X - S.T @ (B @ (S @ X))
    return np.clip(Y, lb[:, None], ub[:, None])


def _perturbed_points(sampler, model, P, T, noise, seed):
    """Sampled points with relative noise on the coordinates that are not at a
    bound (so that the projection's clip stays inactive and the FP64 oracle's
    result is itself feasible)."""
    pts, _ = sampler.sample(P, T, seed=seed)
    rng = np.random.default_rng(seed)
    lb, ub = np.asarray(model.lb)[:, None], np.asarray(model.ub)[:, None]
    room = np.minimum(pts - lb, ub - pts) > 1e-3 * (1.0 + np.abs(pts))
    return pts + room * noise * rng.standard_normal(pts.shape) * (1.0 + np.abs(pts))


@pytest.fixture(scope="module")
def small(pkg, small_model, golden):
    s = pkg.Sampler(small_model, golden["warmup"])
    s.set_null_space(golden["N"])
    yield s, small_model, dense_S(small_model)
    s.close()


def _kappa(S):
    lam = np.linalg.eigvalsh(S @ S.T)
    lam = lam[lam > S.shape[0] * lam.max() * 2.2204e-16]
    return lam.max() / lam.min()


# One pass moves x by the FP64 correction d = S^T (S S^T)^+ S x up to an error
# of about eps * kappa(S S^T) |d|, eps ~ 1.1e-5 for the three BF16 split
# products (each operand split to 16 significant bits, the lo*lo term dropped).
EPS3 = 1.2e-5


@pytest.mark.parametrize("P", [100, 70000])
def test_reproject_matches_fp64_projection(pkg, small, P):
    s, model, S = small
    X = _perturbed_points(s, model, min(P, 500), 30, 2e-11, seed=21)
    if P > X.shape[1]:  # tile to the chain count: more than one 65,536-chain GEMM
        X = np.tile(X, (1, (P + X.shape[1] - 1) // X.shape[1]))[:, :P].copy()
    ref = _fp64_reprojection(S, model.lb, model.ub, X)
    d = torch.from_numpy(X).cuda()
    acc = torch.zeros_like(d)
    st = s.reproject(P, d.data_ptr(), P, d_centre_acc=acc.data_ptr())
    got = d.cpu().numpy()
    moved = np.abs(ref - X).max()
    tol = 2 * EPS3 * _kappa(S)
    assert st["residual_before"] > 1e-8 and st["rounds"] == 1
    assert np.abs(got - ref).max() <= tol * moved + 1e-13 * np.abs(X).max()
    assert st["residual_after"] <= tol * st["residual_before"]
    assert np.abs(S @ got).max() <= 1e-8
    assert np.all(got >= model.lb[:, None] - 1e-9) and np.all(got <= model.ub[:, None] + 1e-9)
    assert np.array_equal(acc.cpu().numpy(), got - X) or np.abs(acc.cpu().numpy() - (got - X)).max() < 1e-15
    assert st["rank"] == np.linalg.matrix_rank(S)
    assert st["gemm_flops"] > 0 and st["gemm_ms"] > 0


def test_reproject_agrees_with_null_space_form(pkg, small, golden):
    """The S-residual form equals N (N^T x) of the FP64 null-space basis."""
    s, model, S = small
    X = _perturbed_points(s, model, 64, 20, 1e-10, seed=4)
    N = golden["N"]
    ref = np.clip(N @ (N.T @ X), model.lb[:, None], model.ub[:, None])
    d = torch.from_numpy(X).cuda()
    s.reproject(64, d.data_ptr(), 64)
    moved = np.abs(ref - X).max()
    assert np.abs(d.cpu().numpy() - ref).max() <= 2 * EPS3 * _kappa(S) * moved + 1e-12


def test_reproject_larger_model_several_tiles(pkg):
    """m = 210 metabolites: two M tiles, four K blocks per split product."""
    synth = importlib.import_module("achr_gb300.synthetic")
    from oracle import reference_py
    spec = synth.SyntheticSpec(300, 210, 0.3, 30, 20.0, seed=11)
    row, col, val, lb, ub = synth.make_model(spec)
    m = pkg.HostModel(spec.n_rxns, spec.n_mets, row, col, val, lb, ub)
    S = dense_S(m)
    warm = synth.interior_chord_warmup(S, lb, ub, 2 * spec.n_rxns, seed=spec.seed)
    with pkg.Sampler(m, warm) as s:
        s.set_null_space(reference_py.null_space_sts(S))
        X = _perturbed_points(s, m, 700, 25, 2e-11, seed=9)
        ref = _fp64_reprojection(S, lb, ub, X)
        d = torch.from_numpy(X).cuda()
        st = s.reproject(700, d.data_ptr(), 700)
        got = d.cpu().numpy()
    tol = 2 * EPS3 * _kappa(S)
    assert np.abs(got - ref).max() <= tol * np.abs(ref - X).max() + 1e-13 * np.abs(X).max()
    # Coordinates sitting exactly at a bound are clipped back after the
    # correction (as the reference clips after reprojecting), which leaves a
    # residual of the correction's size in the FP64 oracle's result as well.
    res_ref = np.abs(S @ ref).max()
    assert np.abs(S @ got).max() <= max(1e-8, 1.01 * res_ref + 1e-12)
    assert st["residual_after"] <= max(tol * st["residual_before"], 1.01 * res_ref + 1e-12)


def test_reproject_rounds_converge_and_stop(pkg, small):
    """Several passes drive a large residual below residual_tol; later passes find
    nothing to do and leave the points bitwise unchanged."""
    s, model, S = small
    X = _perturbed_points(s, model, 200, 10, 1e-6, seed=3)
    d = torch.from_numpy(X).cuda()
    st = s.reproject(200, d.data_ptr(), 200, max_rounds=6)
    assert st["residual_before"] > 1e-5 and st["residual_after"] <= 1e-9
    assert 2 <= st["rounds"] < 6
    snap = d.clone()
    st2 = s.reproject(200, d.data_ptr(), 200, max_rounds=3)
    assert st2["rounds"] == 0 and torch.equal(snap, d)


def test_periodic_sampling(pkg, small_model, golden):
    """Segments of `period` steps, each followed by the batched reprojection; no per-chain checks."""
    S = dense_S(small_model)
    P, T, period = 256, 60, 20
    with pkg.Sampler(small_model, golden["warmup"], check_period=0) as s:
        s.set_null_space(golden["N"])
        x = torch.zeros((s.n, P), dtype=torch.float64, device="cuda")
        a = torch.zeros_like(x)
        st, rs = s.sample_periodic(P, T, period, x.data_ptr(), a.data_ptr(), P, seed=8)
        pts = x.cpu().numpy()
        assert st["accepted"] == P * T and st["checks"] == 0 and st["stuck_chains"] == 0
        assert rs["rounds"] == T // period and rs["residual_after"] <= 1e-8
        assert np.abs(S @ pts).max() <= 1e-8
        assert np.all(pts >= small_model.lb[:, None] - 1e-9) and np.all(pts <= small_model.ub[:, None] + 1e-9)
        # the first segment is plain sampling followed by one reprojection
        x1 = torch.zeros_like(x)
        a1 = torch.zeros_like(x)
        s.sample_resume(P, 0, period, False, x1.data_ptr(), a1.data_ptr(), P, seed=8)
        s.reproject(P, x1.data_ptr(), P, d_centre_acc=a1.data_ptr())
        x2 = torch.zeros_like(x)
        a2 = torch.zeros_like(x)
        s.sample_periodic(P, period, period, x2.data_ptr(), a2.data_ptr(), P, seed=8)
        assert torch.equal(x1, x2) and torch.equal(a1, a2)
