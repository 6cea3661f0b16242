"""GPU: achr_sample_noalloc, the entry point for callers that cannot allocate.

Callers inside another framework's memory pool, with device memory reserved up
front, or on a repeated path that must not allocate, pass the model and the
output as their own device buffers; the library keeps its working data in a
fixed device array.  This file is collected last so that a failure here never
hides the other tests.  The points must match those of the allocating entry
point (a context with the same null space, seed, chains and options) to the
parity tolerance, on two calls in a row (the second call reuses the array the
first one left behind), and a call must leave the device's free memory as it
found it.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import dense_S

pytestmark = pytest.mark.gpu

REL_TOL = 1e-10


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _csr(model):
    S = dense_S(model)
    rp, ci, vv = [0], [], []
    for r in range(model.n_mets):
        nz = np.flatnonzero(S[r])
        ci.extend(nz.tolist())
        vv.extend(S[r, nz].tolist())
        rp.append(len(ci))
    return np.array(rp), np.array(ci), np.array(vv)


def _device_model(pkg, torch, model, warmup, N, keep, col_idx=None):
    n, W = warmup.shape
    ld = n + (n & 1)
    wpad = np.zeros((W, ld))
    wpad[:, :n] = warmup.T  # column j of the ld x W column-major matrix = row j here
    rp, ci, vv = _csr(model)
    if col_idx is not None:
        ci = col_idx
    tensors = {
        "warmup": torch.tensor(wpad, dtype=torch.float64, device="cuda"),
        "lb": torch.tensor(np.asarray(model.lb, dtype=np.float64), device="cuda"),
        "ub": torch.tensor(np.asarray(model.ub, dtype=np.float64), device="cuda"),
        "row_ptr": torch.tensor(rp, dtype=torch.int32, device="cuda"),
        "col_idx": torch.tensor(ci, dtype=torch.int32, device="cuda"),
        "val": torch.tensor(vv, dtype=torch.float64, device="cuda"),
        "N": torch.tensor(np.asfortranarray(N).T.copy(), dtype=torch.float64, device="cuda"),
    }
    keep.update(tensors)
    return pkg.DeviceModel(n, model.n_mets, W, N.shape[1], ld,
                           *(tensors[k].data_ptr() for k in ("warmup", "lb", "ub", "row_ptr", "col_idx", "val", "N")),
                           len(ci))


def _free_bytes(torch):
    torch.cuda.synchronize()
    return torch.cuda.mem_get_info()[0]


def _infinite_bounds_case(pkg):
    """A 12-reaction model with one free lower and one free upper bound (as in the parity tests)."""
    from oracle import reference_py

    rng = np.random.default_rng(0)
    n, m = 12, 4
    row = np.repeat(np.arange(m), 3)
    col = rng.choice(n, size=row.size)
    val = rng.choice([-1.0, 1.0, 2.0], size=row.size)
    lb = np.full(n, -10.0)
    ub = np.full(n, 10.0)
    lb[0] = -np.inf
    ub[1] = np.inf
    model = pkg.HostModel(n, m, row, col, val, lb, ub)
    N = reference_py.null_space_sts(dense_S(model))
    warm = np.clip((N @ rng.standard_normal((N.shape[1], 30))) * 0.5, -5, 5)
    return model, N @ (N.T @ warm), N


# (label, options for both entry points, warmup transform)
CASES = [
    ("reference", {}, None),
    ("no_checks", {"check_period": 0}, None),
    ("check_every_step", {"check_period": 1}, None),
    ("threads_64", {"threads_per_chain": 64}, None),
    ("separate_brackets", {"bracket_pass": 1}, None),
    ("feasible", {"mode": 1}, "project"),
]


@pytest.mark.parametrize("label,opts,transform", CASES, ids=[c[0] for c in CASES])
def test_noalloc_matches_allocating_entry_point(pkg, native, small_model, golden, label, opts, transform):
    torch = _torch()
    N = golden["N"]
    warm = golden["warmup"]
    if transform == "project":  # FEASIBLE mode: the no-alloc call uses the warmup points as given
        warm = N @ (N.T @ warm)
    keep = {}
    dm = _device_model(pkg, torch, small_model, warm, N, keep)
    n = small_model.n_rxns
    o = pkg.default_options()
    for k, v in opts.items():
        setattr(o, k, v)
    with pkg.Sampler(small_model, warm, **opts) as s:
        s.set_null_space(N)
        for call, (seed, P, T) in enumerate(((1234, 64, 50), (99, 40, 23))):
            ref, rst = s.sample(P, T, seed=seed)
            out = torch.zeros((n, P), dtype=torch.float64, device="cuda")
            stream = torch.cuda.current_stream().cuda_stream
            before = _free_bytes(torch)
            st = pkg.sample_noalloc(dm, P, T, out.data_ptr(), P, stream, seed=seed, options=o)
            after = _free_bytes(torch)
            if call == 1:  # the first call of the process may load the module's code
                assert after == before, f"device free memory changed by {before - after} bytes"
            got = out.cpu().numpy()
            assert np.abs(got - ref).max() <= REL_TOL * max(1.0, np.abs(ref).max())
            assert st["accepted"] == rst["accepted"] == P * T
            assert st["rejected"] == rst["rejected"]
            assert st["checks"] == rst["checks"] and st["reprojections"] == rst["reprojections"]
            if transform == "project":
                assert np.abs(dense_S(small_model) @ got).max() <= 1e-8


def test_noalloc_infinite_bounds(pkg, native):
    torch = _torch()
    model, warm, N = _infinite_bounds_case(pkg)
    keep = {}
    dm = _device_model(pkg, torch, model, warm, N, keep)
    with pkg.Sampler(model, warm) as s:
        s.set_null_space(N)
        for seed in (2, 3):
            ref, _ = s.sample(16, 30, seed=seed)
            out = torch.zeros((model.n_rxns, 16), dtype=torch.float64, device="cuda")
            pkg.sample_noalloc(dm, 16, 30, out.data_ptr(), 16, torch.cuda.current_stream().cuda_stream, seed=seed)
            assert np.abs(out.cpu().numpy() - ref).max() <= REL_TOL * max(1.0, np.abs(ref).max())


def test_noalloc_rejects_bad_column_index(pkg, native, small_model, golden):
    """A column index outside [0, n) is caught by the device-side check before the chain kernel runs."""
    torch = _torch()
    _, ci, _ = _csr(small_model)
    bad = ci.copy()
    bad[len(bad) // 2] = small_model.n_rxns + 7
    keep = {}
    dm = _device_model(pkg, torch, small_model, golden["warmup"], golden["N"], keep, col_idx=bad)
    out = torch.zeros((small_model.n_rxns, 4), dtype=torch.float64, device="cuda")
    with pytest.raises(pkg.AchrError) as e:
        pkg.sample_noalloc(dm, 4, 5, out.data_ptr(), 4, torch.cuda.current_stream().cuda_stream)
    assert e.value.status == 1 and "column" in str(e.value)
    # the device is still usable: the same call with the right indices samples
    dm2 = _device_model(pkg, torch, small_model, golden["warmup"], golden["N"], keep)
    st = pkg.sample_noalloc(dm2, 4, 5, out.data_ptr(), 4, torch.cuda.current_stream().cuda_stream)
    assert st["accepted"] == 20


def test_noalloc_rejects_residual_form(pkg, native, small_model, golden):
    torch = _torch()
    keep = {}
    dm = _device_model(pkg, torch, small_model, golden["warmup"], golden["N"], keep)
    o = pkg.default_options()
    o.reproject_form = 2
    with pytest.raises(pkg.AchrError) as e:
        pkg.sample_noalloc(dm, 4, 5, 16, 4, options=o)
    assert e.value.status == 8


def test_noalloc_rejects_models_beyond_its_array(pkg, native):
    dm = pkg.DeviceModel(pkg.NOALLOC_MAX_RXNS + 1, 1, 2, 1, pkg.NOALLOC_MAX_RXNS + 2, 16, 16, 16, 16, 16, 16, 16, 1)
    with pytest.raises(pkg.AchrError) as e:
        pkg.sample_noalloc(dm, 1, 1, 16, 1)
    assert e.value.status == 8 and "at most" in str(e.value)
