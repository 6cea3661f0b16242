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
