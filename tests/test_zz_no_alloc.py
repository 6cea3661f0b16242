"""GPU: achr_sample_noalloc, the entry point for callers that cannot allocate.

Callers inside another framework's memory pool, with device memory reserved up
front, or on a repeated path that must not allocate, pass the model and the
output as their own device buffers; the library keeps its working data in a
fixed device array.  This file is collected last so that a failure here never
hides the other tests.  The points must match those of the allocating entry
point (achr_sample, same seed and chains) to the parity tolerance, on two calls
in a row (the second call reuses the array the first one left behind).
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL_TOL = 1e-10


def _device_model(pkg, torch, model, warmup, N, keep):
    n, W = warmup.shape
    ld = n + (n & 1)
    wpad = np.zeros((W, ld))
    wpad[:, :n] = warmup.T  # column j of the ld x W column-major matrix = row j here
    rp, ci, vv = _csr(model)
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
    return pkg.DeviceModel(n, model.n_mets, W, N.shape[1], ld, *(tensors[k].data_ptr() for k in
                                                                  ("warmup", "lb", "ub", "row_ptr", "col_idx", "val", "N")))


def _csr(model):
    S = np.zeros((model.n_mets, model.n_rxns))
    np.add.at(S, (np.asarray(model.row), np.asarray(model.col)), np.asarray(model.val))
    rp, ci, vv = [0], [], []
    for r in range(model.n_mets):
        nz = np.flatnonzero(S[r])
        ci.extend(nz.tolist())
        vv.extend(S[r, nz].tolist())
        rp.append(len(ci))
    return np.array(rp), np.array(ci), np.array(vv)


def test_noalloc_matches_allocating_entry_point(pkg, native, small_model, golden):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    keep = {}
    dm = _device_model(pkg, torch, small_model, golden["warmup"], golden["N"], keep)
    n = small_model.n_rxns
    with pkg.Sampler(small_model, golden["warmup"]) as s:
        s.set_null_space(golden["N"])
        for seed, P, T in ((1234, 64, 50), (99, 40, 23)):
            ref, rst = s.sample(P, T, seed=seed)
            out = torch.zeros((n, P), dtype=torch.float64, device="cuda")
            st = pkg.sample_noalloc(dm, P, T, out.data_ptr(), P, torch.cuda.current_stream().cuda_stream, seed=seed)
            got = out.cpu().numpy()
            assert np.abs(got - ref).max() <= REL_TOL * max(1.0, np.abs(ref).max())
            assert st["accepted"] == rst["accepted"] == P * T
            assert st["rejected"] == rst["rejected"]


def test_noalloc_rejects_models_beyond_its_array(pkg, native):
    dm = pkg.DeviceModel(pkg.NOALLOC_MAX_RXNS + 1, 1, 2, 1, pkg.NOALLOC_MAX_RXNS + 2, 16, 16, 16, 16, 16, 16, 16)
    with pytest.raises(pkg.AchrError) as e:
        pkg.sample_noalloc(dm, 1, 1, 16, 1)
    assert e.value.status == 8 and "at most" in str(e.value)
