"""CPU: the C-ABI library loads and exports every symbol include/achr.h declares."""
from __future__ import annotations

import ctypes as C
import re
import subprocess

from conftest import ROOT


def test_header_symbols_exported(native, pkg):
    names = pkg.exported_symbols()
    assert "achr_create" in names and "achr_sample" in names
    for name in names:
        assert hasattr(native, name), name


def test_bound_signatures_cover_header(pkg):
    assert set(pkg.exported_symbols()) == set(pkg._SIGNATURES)


def test_nm_dynamic_exports(native, pkg):
    out = subprocess.run(["nm", "-D", "--defined-only", str(pkg.library_path())], capture_output=True, text=True)
    exported = set(re.findall(r"\bT (achr_\w+)", out.stdout))
    assert set(pkg.exported_symbols()) <= exported


def test_default_options_are_reference_constants(native, pkg):
    o = pkg.default_options()
    # ACHRCuda.cu:325, 338, 505, 508, 512
    assert (o.check_period, o.residual_tol, o.max_min_tol, o.u_tol, o.d_tol) == (10, 1e-9, 1e-9, 1e-9, 1e-14)
    assert o.mode == pkg.MODE_REFERENCE and o.centre_offset == 0


def test_version_and_error_string(native):
    assert native.achr_version() >= 100
    assert isinstance(native.achr_last_error(), bytes)


def test_create_rejects_bad_arguments_without_gpu_work(native, pkg):
    ctx = C.c_void_p()
    assert native.achr_create(None, None, 0, None, C.byref(ctx)) == 1
    assert b"NULL" in native.achr_last_error()


def test_header_compiles_as_c(tmp_path):
    src = tmp_path / "t.c"
    src.write_text('#include "achr.h"\nint main(void){achr_options o; achr_default_options(&o); return 0;}\n')
    res = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-fsyntax-only", "-I", str(ROOT / "include"),
                          str(src)], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr


def _model_struct(pkg, n=3, m=1, lb=(-1.0, -1.0, -1.0), ub=(1.0, 1.0, 1.0)):
    import numpy as np
    row = np.zeros(n, dtype=np.int32)
    col = np.arange(n, dtype=np.int32)
    val = np.array([1.0, -1.0, 1.0][:n] + [1.0] * max(0, n - 3))
    lbv = np.asarray(lb, dtype=np.float64)
    ubv = np.asarray(ub, dtype=np.float64)
    keep = (row, col, val, lbv, ubv)
    mdl = pkg.Model(n, m, n, row.ctypes.data_as(C.POINTER(C.c_int32)), col.ctypes.data_as(C.POINTER(C.c_int32)),
                    val.ctypes.data_as(C.POINTER(C.c_double)), lbv.ctypes.data_as(C.POINTER(C.c_double)),
                    ubv.ctypes.data_as(C.POINTER(C.c_double)))
    return mdl, keep


def test_create_validates_before_gpu_work(native, pkg):
    """Argument and option errors are reported before any device work (no GPU needed)."""
    import numpy as np
    mdl, keep = _model_struct(pkg)
    warm = np.zeros(3)
    wp = warm.ctypes.data_as(C.POINTER(C.c_double))
    ctx = C.c_void_p()
    for field, value in (("check_period", -1), ("reproject_form", 4), ("reprojection_passes", 9), ("threads_per_chain", 100),
                         ("max_attempts", 0), ("centre_offset", 2), ("mode", 7), ("bracket_pass", 2)):
        o = pkg.default_options()
        setattr(o, field, value)
        assert native.achr_create(C.byref(mdl), wp, 1, C.byref(o), C.byref(ctx)) == 1, field
    o = pkg.default_options()
    assert native.achr_create(C.byref(mdl), wp, 0, C.byref(o), C.byref(ctx)) == 1  # no warmup points
    big, keep2 = _model_struct(pkg)
    big.n_rxns = 20000
    assert native.achr_create(C.byref(big), wp, 1, C.byref(o), C.byref(ctx)) == 8  # UNSUPPORTED: n > 16384
    bad, keep3 = _model_struct(pkg, lb=(-1.0, 2.0, -1.0))
    assert native.achr_create(C.byref(bad), wp, 1, C.byref(o), C.byref(ctx)) == 1
    assert b"lb > ub" in native.achr_last_error()


def test_other_entry_points_reject_bad_arguments(native, pkg):
    assert native.achr_reproject_batch(None, 1, None, None, 1, 1, None, None) == 1
    assert native.achr_sample_periodic(None, 0, 0, 1, 1, 0, 1, None, None, 1, None, None, None) == 1
    assert native.achr_set_directions(None, None, 0, 0) == 1
    assert native.achr_gemm_bf16(128, 128, 60, 1, None, None, 64, None, None, 64, None, 128, None) == 1
    assert b"multiple of 64" in native.achr_last_error()
    assert native.achr_precond_loss_grad(0, 1, 1, None, None, None, 1, None, None, None, None) == 1
    opt = pkg.precond_options()
    assert native.achr_precond_train(4, 8, 16, None, 16, C.byref(opt), None, None, None, None) == 1
