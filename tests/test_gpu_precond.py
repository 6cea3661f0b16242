"""GPU: hit-and-run along a direction pool against the oracle, the preconditioner's
loss/gradient kernels against the FP64 oracle, its training, the null-space
coordinates and the learned direction pool."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import dense_S

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

REL_TOL = 1e-10


@pytest.fixture(scope="module")
def sampler(pkg, small_model, golden):
    s = pkg.Sampler(small_model, golden["warmup"])
    s.set_null_space(golden["N"])
    yield s
    s.close()


def _pool(N, K, seed):
    rng = np.random.default_rng(seed)
    return N @ rng.standard_normal((N.shape[1], K))


@pytest.mark.parametrize("steps", [1, 20, 50])
def test_hit_and_run_matches_oracle(pkg, small_model, golden, oracle_mod, steps):
    N = golden["N"]
    D = _pool(N, 60, seed=7)
    with pkg.Sampler(small_model, golden["warmup"]) as s:
        s.set_null_space(N)
        s.set_directions(D)
        assert np.array_equal(s.directions(), D)
        pts, st = s.sample(64, steps, seed=42)
        centre = s.centre()
    prob = oracle_mod.Problem(small_model, D, N, centre_point=centre)
    ref, rst = prob.sample(42, 64, steps, hit_and_run=True)
    assert np.abs(pts - ref).max() <= REL_TOL * max(1.0, np.abs(ref).max())
    assert st["accepted"] == rst["accepted"] and st["rejected"] == rst["rejected"]
    assert st["reprojections"] == rst["reprojections"]


def test_directions_cleared_returns_to_achr(pkg, small_model, golden):
    with pkg.Sampler(small_model, golden["warmup"]) as s:
        s.set_null_space(golden["N"])
        a, _ = s.sample(16, 10, seed=3)
        s.set_directions(_pool(golden["N"], 30, seed=1))
        b, _ = s.sample(16, 10, seed=3)
        s.set_directions(None)
        c, _ = s.sample(16, 10, seed=3)
    assert not np.array_equal(a, b) and np.array_equal(a, c)


def _dev(a, dtype=torch.float32):
    return torch.from_numpy(np.ascontiguousarray(a)).to(device="cuda", dtype=dtype)


def test_loss_grad_matches_fp64_oracle(pkg):
    from oracle import precond
    rng = np.random.default_rng(11)
    d, r, B = 50, 8, 200
    s = 0.3 * rng.standard_normal(d)
    U = 0.4 * rng.standard_normal((d, r))
    Y = rng.standard_normal((d, 3 * B)) * np.exp(rng.uniform(-1, 1, (d, 1)))
    ds, dU, dY = _dev(s), _dev(U), _dev(Y)
    gs = torch.zeros(d, device="cuda")
    gU = torch.zeros((d, r), device="cuda")
    # minibatch = columns [B, 2B) of a wider Y: exercises the leading dimension
    loss = pkg.precond_loss_grad(d, r, B, ds.data_ptr(), dU.data_ptr(), dY.data_ptr() + 4 * B, 3 * B,
                                 gs.data_ptr(), gU.data_ptr())
    val, gs_ref, gU_ref = precond.loss_grad(s.astype(np.float32), U.astype(np.float32),
                                            Y.astype(np.float32)[:, B:2 * B])
    assert abs(loss - val) <= 1e-4 * max(1.0, abs(val))
    assert np.abs(gs.cpu().numpy() - gs_ref).max() <= 2e-4 * max(1.0, np.abs(gs_ref).max())
    assert np.abs(gU.cpu().numpy() - gU_ref).max() <= 2e-4 * max(1.0, np.abs(gU_ref).max())


def test_training_fits_a_known_covariance(pkg):
    from oracle import precond
    rng = np.random.default_rng(5)
    d, r, n = 64, 4, 32768
    s_true = np.log(rng.uniform(0.2, 2.0, d))
    U_true = rng.standard_normal((d, r)) * 1.5
    C = precond.covariance(s_true, U_true)
    Y = np.linalg.cholesky(C) @ rng.standard_normal((d, n))
    s0 = 0.5 * np.log(Y.var(axis=1))
    U0 = 0.01 * rng.standard_normal((d, r))
    ds, dU, dY = _dev(s0), _dev(U0), _dev(Y)
    st = pkg.precond_train(d, r, n, dY.data_ptr(), n, ds.data_ptr(), dU.data_ptr(), iterations=1500, batch=2048,
                           learning_rate=0.02, init=0, full_batch=0)
    assert st["iterations"] == 1500 and st["loss_last"] < st["loss_first"]
    s_fit, U_fit = ds.cpu().numpy().astype(np.float64), dU.cpu().numpy().astype(np.float64)
    kl_fit = precond.kl_to_sample_covariance(s_fit, U_fit, Y)
    kl_init = precond.kl_to_sample_covariance(s0, U0, Y)
    kl_true = precond.kl_to_sample_covariance(s_true, U_true, Y)
    # minibatch noise keeps Adam near, not at, the optimum
    assert kl_fit < 0.05 * kl_init and kl_fit < kl_true + 0.2


def test_full_batch_training_reaches_the_optimum(pkg):
    """Full-batch steps (the samples replaced by their covariance's square root): from the
    probabilistic-PCA start the exact loss falls, and the fit ends at least as close to the sample
    covariance as the true parameters (which lie in the model family) and closer than the start."""
    from oracle import precond
    rng = np.random.default_rng(6)
    d, r, n = 64, 4, 32768
    s_true = np.log(rng.uniform(0.2, 2.0, d))
    U_true = rng.standard_normal((d, r)) * 1.5
    Y = np.linalg.cholesky(precond.covariance(s_true, U_true)) @ rng.standard_normal((d, n))
    ds, dU, dY = _dev(np.zeros(d)), _dev(np.zeros((d, r))), _dev(Y)
    pkg.precond_train(d, r, n, dY.data_ptr(), n, ds.data_ptr(), dU.data_ptr(), iterations=0, init=1)
    s_p, U_p = ds.cpu().numpy().astype(np.float64), dU.cpu().numpy().astype(np.float64)
    st = pkg.precond_train(d, r, n, dY.data_ptr(), n, ds.data_ptr(), dU.data_ptr(), iterations=1500,
                           learning_rate=0.01, init=1, full_batch=1)
    s_fit, U_fit = ds.cpu().numpy().astype(np.float64), dU.cpu().numpy().astype(np.float64)
    kl_pca = precond.kl_to_sample_covariance(s_p, U_p, Y)
    kl_fit = precond.kl_to_sample_covariance(s_fit, U_fit, Y)
    kl_true = precond.kl_to_sample_covariance(s_true, U_true, Y)
    assert st["loss_last"] < st["loss_first"]
    # the full-sample loss of the fit, from the FP64 oracle, equals what the GPU reports (training runs
    # in coordinates scaled to unit RMS, which shifts the loss by -sum(log rms))
    rms = np.sqrt((Y ** 2).mean(axis=1))
    want = precond.loss(s_fit, U_fit, Y) - np.log(rms).sum()
    assert abs(want - st["loss_last"]) <= 1e-3 * abs(want) + 1e-3, (want, st["loss_last"])
    assert kl_fit < kl_pca and kl_fit <= kl_true + 0.01, (kl_fit, kl_pca, kl_true)


def test_precond_basis_spans_the_affine_hull(pkg, sampler, small_model, golden):
    S = dense_S(small_model)
    warm = golden["warmup"]
    frozen = np.ptp(warm, axis=1) <= 1e-9 * np.maximum(1.0, np.abs(warm).max(axis=1))
    d, nf = sampler.precond_dim()
    B = sampler.precond_basis()
    assert nf == int(frozen.sum()) and B.shape == (small_model.n_rxns, d)
    assert np.abs(S @ B).max() <= 1e-12 and np.abs(B[frozen]).max() <= 1e-12
    assert np.abs(B.T @ B - np.eye(d)).max() <= 1e-12
    A = np.vstack([S, np.eye(S.shape[1])[frozen]])
    lam, V = np.linalg.eigh(A.T @ A)
    ref = V[:, lam < A.shape[1] * lam.max() * 2.2204e-16]
    assert ref.shape[1] == d
    assert np.abs(B @ B.T - ref @ ref.T).max() <= 1e-10  # same subspace


def test_training_start_options(pkg):
    """Zero steps: a given start comes back unchanged through the standardisation; the
    probabilistic-PCA start is the maximum-likelihood sigma^2 I + U U^T of the samples."""
    from oracle import precond
    rng = np.random.default_rng(8)
    d, r, n = 40, 3, 8192
    Y = (rng.standard_normal((d, r)) @ rng.standard_normal((r, n)) * 3.0 + 0.5 * rng.standard_normal((d, n)))
    Y *= np.exp(rng.uniform(-2, 2, (d, 1)))
    s0 = 0.2 * rng.standard_normal(d)
    U0 = rng.standard_normal((d, r))
    ds, dU, dY = _dev(s0), _dev(U0), _dev(Y)
    pkg.precond_train(d, r, n, dY.data_ptr(), n, ds.data_ptr(), dU.data_ptr(), iterations=0, batch=256, init=0,
                      standardize=1)
    assert np.allclose(ds.cpu().numpy(), s0, atol=1e-5) and np.allclose(dU.cpu().numpy(), U0, rtol=1e-5, atol=1e-5)
    pkg.precond_train(d, r, n, dY.data_ptr(), n, ds.data_ptr(), dU.data_ptr(), iterations=0, batch=256, init=1,
                      standardize=1)
    s_p, U_p = ds.cpu().numpy().astype(np.float64), dU.cpu().numpy().astype(np.float64)
    # reference PPCA in standardised coordinates, mapped back
    sig = np.sqrt((Y ** 2).mean(axis=1))
    Z = Y / sig[:, None]
    lam, V = np.linalg.eigh(Z @ Z.T / n)
    s2 = lam[: d - r].mean()
    C_ref = np.diag(sig) @ (s2 * np.eye(d) + (V[:, d - r:] * (lam[d - r:] - s2)) @ V[:, d - r:].T) @ np.diag(sig)
    C_got = precond.covariance(s_p, U_p)
    assert np.abs(C_got - C_ref).max() <= 1e-3 * np.abs(C_ref).max()


def test_null_coords_match_numpy(pkg, sampler, golden):
    P = 300
    pts, _ = sampler.sample(P, 25, seed=9)
    mu = pts.mean(axis=1)
    X = _dev(pts, torch.float64)
    dmu = _dev(mu, torch.float64)
    Bas = sampler.precond_basis()
    d = Bas.shape[1]
    Y = torch.full((d, P + 4), float("nan"), device="cuda")
    sampler.null_coords(P, X.data_ptr(), P, Y.data_ptr(), P + 4, d_mu=dmu.data_ptr())
    ref = Bas.T @ (pts - mu[:, None])
    got = Y[:, :P].double().cpu().numpy()
    assert np.abs(got - ref).max() <= 1e-4 * np.abs(ref).max()


def test_learned_pool_directions_lie_in_null_space(pkg, small_model, golden):
    S = dense_S(small_model)
    rng = np.random.default_rng(2)
    with pkg.Sampler(small_model, golden["warmup"]) as s:
        s.set_null_space(golden["N"])
        d, _ = s.precond_dim()
        Bas = s.precond_basis()
        r = 4
        ds = _dev(0.1 * rng.standard_normal(d))
        dU = _dev(0.5 * rng.standard_normal((d, r)))
        s.precond_pool(r, ds.data_ptr(), dU.data_ptr(), 500, seed=17)
        G = s.directions()
        assert G.shape == (s.n, 500)
        assert np.abs(S @ G).max() <= 1e-12 * np.abs(G).max()
        # the pool's covariance in the basis coordinates approaches exp(2 s) + U U^T
        Yc = Bas.T @ G
        emp = Yc @ Yc.T / 500
        from oracle import precond
        C = precond.covariance(ds.cpu().numpy(), dU.cpu().numpy())
        assert np.abs(emp - C).max() < 0.35 * np.abs(C).max()
        pts, st = s.sample(128, 40, seed=1)
    assert st["accepted"] == 128 * 40 and st["stuck_chains"] == 0
    assert np.abs(S @ pts).max() <= 1e-8
    assert np.all(pts >= small_model.lb[:, None] - 1e-9) and np.all(pts <= small_model.ub[:, None] + 1e-9)


def test_check_directions_falls_back_to_plain_achr(pkg, small_model, golden):
    """A pool that cannot mix (one direction: every chain stays on its own line through its
    starting warmup point) fails the split-R-hat check and is removed; a pool of the warmup
    points' own spread (differences from their centre, in the null space) passes and stays."""
    with pkg.Sampler(small_model, golden["warmup"]) as s:
        s.set_null_space(golden["N"])
        Bas = s.precond_basis()
        s.set_directions(Bas[:, :1])
        chk = s.check_directions(chains=128, burnin=2000, draws=40, gap=50, seed=3)
        assert chk["kept"] == 0 and chk["rhat_max"] >= 1.01 and chk["fluxes"] > 0
        assert s.directions().shape[1] == 0  # back to ACHR
        W = golden["warmup"]
        pool = Bas @ (Bas.T @ (W - W.mean(axis=1, keepdims=True)))
        s.set_directions(pool)
        chk = s.check_directions(chains=256, burnin=50000, draws=100, gap=500, seed=3, rhat_limit=1.1)
        assert chk["kept"] == 1 and chk["rhat_max"] < 1.1, chk
        assert s.directions().shape[1] == W.shape[1]


def test_check_directions_needs_a_pool(pkg, sampler):
    with pytest.raises(pkg.AchrError) as e:
        sampler.check_directions()
    assert e.value.status == 1


def _ess_draws(s, M, B, K, L, seed, starts):
    """(chains, draws, fluxes) after B burn-in steps, then K draws L steps apart (resumed launches)."""
    n = s.n
    pts = starts[0].clone()
    acc = starts[1].clone()
    stream = torch.cuda.current_stream().cuda_stream
    s.sample_resume(M, 0, B, True, pts.data_ptr(), acc.data_ptr(), M, stream=stream, seed=seed)
    trace = torch.empty((K, n, M), dtype=torch.float64, device="cuda")
    for k in range(K):
        s.sample_resume(M, B + k * L, L, True, pts.data_ptr(), acc.data_ptr(), M, stream=stream, seed=seed)
        trace[k].copy_(pts)
    torch.cuda.synchronize()
    return trace.permute(2, 0, 1).cpu().numpy()


def test_learned_directions_beat_the_ablations_on_an_elongated_polytope(pkg):
    """Where the polytope is anisotropic the training earns its place: a 200 x 2 x 2 x 2 box (one
    reaction 100 times wider than the others, plus a coupled pair v4 = v5).  Hit-and-run along
    isotropic directions in the same basis moves along the long reaction by about the box's width
    per step, so it mixes there slowly; the trained map puts its directions along it.  Same chains,
    starts, seed and schedule for every sampler: the learned map's min-ESS is at least 3x the
    isotropic ablation's, and at least that of the untrained (PCA-start) map."""
    diag = pytest.importorskip("achr_gb300.diagnostics")
    n = 6
    row, col, val = np.array([0, 0]), np.array([4, 5]), np.array([1.0, -1.0])
    lb = np.array([-100.0, -1.0, -1.0, -1.0, -1.0, -1.0])
    ub = -lb
    model = pkg.HostModel(n, 1, row, col, val, lb, ub)
    rng = np.random.default_rng(5)
    W = 2 * n
    warm = rng.uniform(lb[:, None] * 0.9, ub[:, None] * 0.9, size=(n, W))
    warm[5] = warm[4]
    with pkg.Sampler(model, warm) as s:
        d, _ = s.precond_dim()
        assert d == 5
        r = 2
        # training samples from plain ACHR, in the preconditioner's coordinates
        Pt, Tb, Ks, Lg = 2048, 500, 4, 50
        stream = torch.cuda.current_stream().cuda_stream
        x = torch.zeros((n, Pt), dtype=torch.float64, device="cuda")
        a = torch.zeros_like(x)
        mu = torch.from_numpy(s.centre()).cuda()
        Y = torch.empty((d, Pt * Ks), dtype=torch.float32, device="cuda")
        s.sample_resume(Pt, 0, Tb, False, x.data_ptr(), a.data_ptr(), Pt, stream=stream, seed=11)
        for k in range(Ks):
            s.sample_resume(Pt, Tb + k * Lg, Lg, True, x.data_ptr(), a.data_ptr(), Pt, stream=stream, seed=11)
            s.null_coords(Pt, x.data_ptr(), Pt, Y.data_ptr() + 4 * k * Pt, Pt * Ks, d_mu=mu.data_ptr(),
                          stream=stream)
        Y -= Y.mean(dim=1, keepdim=True)
        ns = Pt * Ks
        maps = {}
        for name, iters in (("pca", 0), ("learned", 1000)):
            sv = torch.zeros(d, dtype=torch.float32, device="cuda")
            Uv = torch.zeros((d, r), dtype=torch.float32, device="cuda")
            pkg.precond_train(d, r, ns, Y.data_ptr(), ns, sv.data_ptr(), Uv.data_ptr(), stream=stream,
                              iterations=iters, batch=ns, learning_rate=0.01, seed=3, init=1, full_batch=1)
            maps[name] = (sv, Uv)
        maps["isotropic"] = (torch.zeros(d, dtype=torch.float32, device="cuda"),
                             torch.zeros((d, r), dtype=torch.float32, device="cuda"))
        M, B, K, L = 256, 200, 100, 10
        idx = torch.from_numpy(rng.integers(0, W, size=M)).cuda()
        wt = torch.from_numpy(np.ascontiguousarray(warm)).cuda()
        starts = (wt[:, idx].contiguous(), (float(W) * wt.mean(dim=1, keepdim=True)).expand(-1, M).contiguous())
        ess = {}
        for name, (sv, Uv) in maps.items():
            s.precond_pool(r, sv.data_ptr(), Uv.data_ptr(), 4096, seed=21)
            ess[name] = diag.summarize(_ess_draws(s, M, B, K, L, 99, starts))["min_ess"]
        s.set_directions(None)
    assert ess["learned"] >= 3.0 * ess["isotropic"], ess
    assert ess["learned"] >= ess["pca"] * 0.95, ess
