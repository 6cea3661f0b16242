"""GB300-native ACHR sampler: Python mirror of the reference's ACHRCuda flow.

The product is the C-ABI library ``_build/libachr_gb300.so`` (CUDA kernels for
sm_103a plus host set-up and I/O) and the ``ACHRCuda`` command line built
beside it.  This module binds that ABI with ctypes for tests, benchmarks and
Python users; it performs no sampling work itself and has no CPU fallback.

The directory name contains a dot, so it is loaded by file path and
registered as the module ``achr_gb300`` (see ``load_package`` in
``__graft_entry__``).
"""
from __future__ import annotations

import ctypes as C
import math
import os
from dataclasses import dataclass
from pathlib import Path
from typing import Optional

import numpy as np

PKG_DIR = Path(__file__).resolve().parent
INCLUDE_HEADER = PKG_DIR.parent / "include" / "achr.h"

MODE_REFERENCE = 0
MODE_FEASIBLE = 1
NULL_SVD_STS = 0
NULL_SVD_S = 1
NULL_FIXED = 2

STATUS_NAMES = {
    0: "ACHR_OK", 1: "ACHR_ERR_INVALID", 2: "ACHR_ERR_CUDA", 3: "ACHR_ERR_NOMEM", 4: "ACHR_ERR_IO",
    5: "ACHR_ERR_PARSE", 6: "ACHR_ERR_NUMERIC", 7: "ACHR_ERR_TIMEOUT", 8: "ACHR_ERR_UNSUPPORTED",
}


class AchrError(RuntimeError):
    """A call through the C ABI returned a non-zero achr_status."""

    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class Model(C.Structure):
    _fields_ = [
        ("n_rxns", C.c_int32), ("n_mets", C.c_int32), ("nnz", C.c_int64),
        ("row", C.POINTER(C.c_int32)), ("col", C.POINTER(C.c_int32)), ("val", C.POINTER(C.c_double)),
        ("lb", C.POINTER(C.c_double)), ("ub", C.POINTER(C.c_double)),
    ]


class ModelBuf(C.Structure):
    _fields_ = [
        ("model", Model),
        ("row_buf", C.POINTER(C.c_int32)), ("col_buf", C.POINTER(C.c_int32)),
        ("val_buf", C.POINTER(C.c_double)), ("lb_buf", C.POINTER(C.c_double)), ("ub_buf", C.POINTER(C.c_double)),
    ]


class Options(C.Structure):
    _fields_ = [
        ("mode", C.c_int32), ("null_space", C.c_int32), ("check_period", C.c_int32), ("max_attempts", C.c_int32),
        ("centre_offset", C.c_int32), ("exact_ratio", C.c_int32), ("threads_per_chain", C.c_int32),
        ("reproject_form", C.c_int32),
        ("residual_tol", C.c_double), ("max_min_tol", C.c_double), ("u_tol", C.c_double), ("d_tol", C.c_double),
        ("feasibility_tol", C.c_double), ("wait_limit_ns", C.c_int32), ("bracket_pass", C.c_int32),
        ("reprojection_passes", C.c_int32),
    ]


class Stats(C.Structure):
    _fields_ = [
        ("accepted", C.c_int64), ("rejected", C.c_int64), ("checks", C.c_int64), ("reprojections", C.c_int64),
        ("stuck_chains", C.c_int64), ("exact_evals", C.c_int64), ("final_projections", C.c_int64),
        ("max_residual", C.c_double), ("max_bound_violation", C.c_double), ("kernel_ms", C.c_double),
        ("segments", C.c_int64), ("reprojection_passes", C.c_int64), ("reprojection_gemms", C.c_int64),
        ("chain_ms", C.c_double), ("reprojection_ms", C.c_double), ("reprojection_flops", C.c_double),
        ("kernel_launches", C.c_int64),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class DeviceModel(C.Structure):
    """achr_device_model: a model already in device memory (pointers are device addresses)."""
    _fields_ = [
        ("n_rxns", C.c_int32), ("n_mets", C.c_int32), ("n_warmup", C.c_int32), ("null_dim", C.c_int32),
        ("ld_warmup", C.c_int64), ("warmup", C.c_void_p), ("lb", C.c_void_p), ("ub", C.c_void_p),
        ("row_ptr", C.c_void_p), ("col_idx", C.c_void_p), ("val", C.c_void_p), ("N", C.c_void_p),
        ("nnz", C.c_int64),
    ]


NOALLOC_MAX_RXNS = 8192


class BatchStats(C.Structure):
    _fields_ = [
        ("graph_ms", C.c_double), ("load_imbalance", C.c_double), ("accepted", C.c_int64), ("rejected", C.c_int64),
        ("reprojections", C.c_int64), ("stuck_chains", C.c_int64), ("max_residual", C.c_double),
        ("max_bound_violation", C.c_double),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class ReprojStats(C.Structure):
    _fields_ = [
        ("residual_before", C.c_double), ("residual_after", C.c_double), ("gemm_ms", C.c_double),
        ("total_ms", C.c_double), ("gemm_flops", C.c_double), ("rounds", C.c_int32), ("rank", C.c_int32),
        ("lambda_min", C.c_double), ("lambda_max", C.c_double),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class DirectionCheck(C.Structure):
    _fields_ = [("rhat_max", C.c_double), ("fluxes", C.c_int32), ("kept", C.c_int32), ("sampling_ms", C.c_double)]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class PrecondOptions(C.Structure):
    _fields_ = [
        ("iterations", C.c_int32), ("batch", C.c_int32), ("learning_rate", C.c_float), ("beta1", C.c_float),
        ("beta2", C.c_float), ("eps", C.c_float), ("seed", C.c_uint64), ("init", C.c_int32),
        ("standardize", C.c_int32), ("full_batch", C.c_int32),
    ]


class PrecondStats(C.Structure):
    _fields_ = [("loss_first", C.c_double), ("loss_last", C.c_double), ("train_ms", C.c_double),
                ("iterations", C.c_int32)]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


# Every symbol include/achr.h declares, with its ctypes signature.
_SIGNATURES = {
    "achr_default_options": (None, [C.POINTER(Options)]),
    "achr_create": (C.c_int, [C.POINTER(Model), C.POINTER(C.c_double), C.c_int32, C.POINTER(Options),
                              C.POINTER(C.c_void_p)]),
    "achr_set_null_space": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.c_int32]),
    "achr_get_null_space_dim": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32)]),
    "achr_get_null_space": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "achr_get_centre": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "achr_sample": (C.c_int, [C.c_void_p, C.c_uint64, C.c_uint64, C.c_int32, C.c_int32, C.POINTER(C.c_double),
                              C.POINTER(Stats)]),
    "achr_sample_device": (C.c_int, [C.c_void_p, C.c_uint64, C.c_uint64, C.c_int32, C.c_int32, C.c_void_p,
                                     C.c_int64, C.c_void_p, C.POINTER(Stats)]),
    "achr_destroy": (None, [C.c_void_p]),
    "achr_sample_resume": (C.c_int, [C.c_void_p, C.c_uint64, C.c_uint64, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                     C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.POINTER(Stats)]),
    "achr_autotune": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32)]),
    "achr_sample_batch": (C.c_int, [C.POINTER(C.c_void_p), C.c_int32, C.POINTER(C.c_int32), C.c_int32, C.c_uint64,
                                    C.POINTER(C.c_void_p), C.POINTER(C.c_int64), C.c_void_p, C.POINTER(BatchStats),
                                    C.POINTER(C.c_double)]),
    "achr_set_batch_tiles": (C.c_int, [C.c_int32]),
    "achr_get_batch_tiles": (C.c_int32, []),
    "achr_autotune_batch": (C.c_int, [C.POINTER(C.c_void_p), C.c_int32, C.POINTER(C.c_int32), C.c_int32, C.c_uint64,
                                      C.POINTER(C.c_void_p), C.POINTER(C.c_int64), C.c_void_p,
                                      C.POINTER(C.c_int32)]),
    "achr_sample_noalloc": (C.c_int, [C.POINTER(DeviceModel), C.POINTER(Options), C.c_uint64, C.c_uint64, C.c_int32,
                                      C.c_int32, C.c_void_p, C.c_int64, C.c_void_p, C.POINTER(Stats)]),
    "achr_set_directions": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_int32]),
    "achr_get_n_directions": (C.c_int32, [C.c_void_p]),
    "achr_get_directions": (C.c_int, [C.c_void_p, C.c_void_p]),
    "achr_check_directions": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_uint64,
                                        C.c_double, C.POINTER(DirectionCheck)]),
    "achr_precond_default_options": (None, [C.POINTER(PrecondOptions)]),
    "achr_precond_dim": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "achr_get_precond_basis": (C.c_int, [C.c_void_p, C.c_void_p]),
    "achr_null_coords": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_int64,
                                   C.c_void_p]),
    "achr_precond_loss_grad": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p,
                                         C.c_int64, C.POINTER(C.c_float), C.c_void_p, C.c_void_p, C.c_void_p]),
    "achr_precond_train": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_int64,
                                     C.POINTER(PrecondOptions), C.c_void_p, C.c_void_p, C.c_void_p,
                                     C.POINTER(PrecondStats)]),
    "achr_precond_pool": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_int32, C.c_uint64]),
    "achr_reproject_batch": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_int64, C.c_int32,
                                       C.c_void_p, C.POINTER(ReprojStats)]),
    "achr_sample_periodic": (C.c_int, [C.c_void_p, C.c_uint64, C.c_uint64, C.c_int32, C.c_int32, C.c_int32,
                                       C.c_int32, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.POINTER(Stats),
                                       C.POINTER(ReprojStats)]),
    "achr_gemm_bf16": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_int64,
                                 C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_void_p]),
    "achr_read_mps": (C.c_int, [C.c_char_p, C.POINTER(ModelBuf)]),
    "achr_free_model": (None, [C.POINTER(ModelBuf)]),
    "achr_read_warmup_csv": (C.c_int, [C.c_char_p, C.c_int32, C.POINTER(C.POINTER(C.c_double)),
                                       C.POINTER(C.c_int32)]),
    "achr_write_points_csv": (C.c_int, [C.c_char_p, C.POINTER(C.c_double), C.c_int32, C.c_int32, C.c_int32]),
    "achr_format_f": (C.c_int32, [C.c_double, C.c_char_p]),
    "achr_free": (None, [C.c_void_p]),
    "achr_last_error": (C.c_char_p, []),
    "achr_version": (C.c_int32, []),
}

_lib: Optional[C.CDLL] = None


def library_path() -> Path:
    return PKG_DIR / "_build" / "libachr_gb300.so"


def cli_path() -> Path:
    return PKG_DIR / "_build" / "ACHRCuda"


def lib() -> C.CDLL:
    """Load the native library; raises if it has not been built (no fallback)."""
    global _lib
    if _lib is None:
        path = library_path()
        if not path.exists():
            raise ImportError(f"native library {path} is missing: run __graft_entry__.build() first")
        handle = C.CDLL(str(path))
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(handle, name)
            fn.restype = res
            fn.argtypes = args
        _lib = handle
    return _lib


def _check(status: int) -> None:
    if status != 0:
        msg = lib().achr_last_error()
        raise AchrError(status, msg.decode() if msg else "")


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _iptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


def default_options(**overrides) -> Options:
    opt = Options()
    lib().achr_default_options(C.byref(opt))
    for k, v in overrides.items():
        if not hasattr(opt, k):
            raise KeyError(k)
        setattr(opt, k, v)
    return opt


@dataclass
class HostModel:
    """S as COO triplets plus bounds, the part of an MPS model the sampler uses."""
    n_rxns: int
    n_mets: int
    row: np.ndarray
    col: np.ndarray
    val: np.ndarray
    lb: np.ndarray
    ub: np.ndarray

    def dense(self) -> np.ndarray:
        S = np.zeros((self.n_mets, self.n_rxns))
        np.add.at(S, (self.row, self.col), self.val)
        return S

    def _as_struct(self):
        keep = (np.ascontiguousarray(self.row, dtype=np.int32), np.ascontiguousarray(self.col, dtype=np.int32),
                np.ascontiguousarray(self.val, dtype=np.float64), np.ascontiguousarray(self.lb, dtype=np.float64),
                np.ascontiguousarray(self.ub, dtype=np.float64))
        m = Model(self.n_rxns, self.n_mets, len(keep[0]), _iptr(keep[0]), _iptr(keep[1]), _dptr(keep[2]),
                  _dptr(keep[3]), _dptr(keep[4]))
        return m, keep


def read_mps(path: str | os.PathLike) -> HostModel:
    """Read a fixed-format MPS file through the library's reader."""
    mb = ModelBuf()
    _check(lib().achr_read_mps(str(path).encode(), C.byref(mb)))
    try:
        m = mb.model
        nnz = m.nnz
        hm = HostModel(m.n_rxns, m.n_mets,
                       np.ctypeslib.as_array(m.row, (nnz,)).copy() if nnz else np.zeros(0, np.int32),
                       np.ctypeslib.as_array(m.col, (nnz,)).copy() if nnz else np.zeros(0, np.int32),
                       np.ctypeslib.as_array(m.val, (nnz,)).copy() if nnz else np.zeros(0),
                       np.ctypeslib.as_array(m.lb, (m.n_rxns,)).copy(),
                       np.ctypeslib.as_array(m.ub, (m.n_rxns,)).copy())
    finally:
        lib().achr_free_model(C.byref(mb))
    return hm


def read_warmup_csv(path: str | os.PathLike, n_rxns: int) -> np.ndarray:
    """Read a warmup CSV into an (n, W) array (column j = warmup point j)."""
    ptr = C.POINTER(C.c_double)()
    W = C.c_int32()
    _check(lib().achr_read_warmup_csv(str(path).encode(), n_rxns, C.byref(ptr), C.byref(W)))
    try:
        flat = np.ctypeslib.as_array(ptr, (W.value * n_rxns,)).copy()
    finally:
        lib().achr_free(ptr)
    return flat.reshape(W.value, n_rxns).T.copy()


def write_points_csv(path: str | os.PathLike, points: np.ndarray, threads: int = 0) -> None:
    """Write an (n, P) array as the reference's File<ii>."""
    pts = np.ascontiguousarray(points, dtype=np.float64)
    n, P = pts.shape
    _check(lib().achr_write_points_csv(str(path).encode(), _dptr(pts), n, P, threads))


def format_f(v: float) -> str:
    buf = C.create_string_buffer(400)
    k = lib().achr_format_f(float(v), buf)
    return buf.raw[:k].decode()


class Sampler:
    """One model and its warmup points resident on the GPU.

    Mirrors the reference program's flow (ACHRcu/ACHRCuda.cu:504-802): set-up
    (null space, centre) once, then one ``sample`` call per output file.
    """

    def __init__(self, model: HostModel, warmup: np.ndarray, options: Optional[Options] = None, **overrides):
        self.model = model
        self.n = model.n_rxns
        w = np.asarray(warmup, dtype=np.float64)
        if w.ndim != 2 or w.shape[0] != self.n:
            raise ValueError("warmup must be an (n_rxns, W) array")
        self.W = w.shape[1]
        wcol = np.asfortranarray(w)  # column j contiguous
        opt = options if options is not None else default_options(**overrides)
        self.options = opt
        m, keep = model._as_struct()
        ctx = C.c_void_p()
        _check(lib().achr_create(C.byref(m), wcol.ctypes.data_as(C.POINTER(C.c_double)), self.W, C.byref(opt),
                                 C.byref(ctx)))
        del keep
        self._ctx = ctx

    def close(self) -> None:
        if getattr(self, "_ctx", None):
            lib().achr_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def null_dim(self) -> int:
        d = C.c_int32()
        _check(lib().achr_get_null_space_dim(self._ctx, C.byref(d)))
        return d.value

    def null_space(self) -> np.ndarray:
        d = self.null_dim
        out = np.zeros(self.n * d)
        if d:
            _check(lib().achr_get_null_space(self._ctx, _dptr(out)))
        return out.reshape(d, self.n).T.copy()

    def set_null_space(self, N: np.ndarray) -> None:
        Nf = np.asfortranarray(np.asarray(N, dtype=np.float64))
        if Nf.shape[0] != self.n:
            raise ValueError("N must have n_rxns rows")
        _check(lib().achr_set_null_space(self._ctx, Nf.ctypes.data_as(C.POINTER(C.c_double)), Nf.shape[1]))

    def centre(self) -> np.ndarray:
        out = np.zeros(self.n)
        _check(lib().achr_get_centre(self._ctx, _dptr(out)))
        return out

    def sample(self, n_points: int, n_steps: int, seed: int = 0, chain_offset: int = 0,
               out: Optional[np.ndarray] = None) -> tuple[np.ndarray, dict]:
        """Run n_points chains of n_steps; returns ((n, P) points, stats)."""
        if out is None:
            out = np.empty((self.n, n_points))
        if out.shape != (self.n, n_points) or out.dtype != np.float64 or not out.flags.c_contiguous:
            raise ValueError("out must be a C-contiguous float64 (n_rxns, n_points) array")
        st = Stats()
        _check(lib().achr_sample(self._ctx, seed, chain_offset, n_points, n_steps, _dptr(out), C.byref(st)))
        return out, st.as_dict()

    def sample_resume(self, n_points: int, step0: int, n_steps: int, resume: bool, d_points: int, d_centre_acc: int,
                      ld: int, stream: int = 0, seed: int = 0, chain_offset: int = 0,
                      with_stats: bool = False) -> Optional[dict]:
        """Start or continue chains in place on device state buffers (achr_sample_resume)."""
        st = Stats() if with_stats else None
        _check(lib().achr_sample_resume(self._ctx, seed, chain_offset, n_points, step0, n_steps, int(resume),
                                        C.c_void_p(d_points), C.c_void_p(d_centre_acc), ld, C.c_void_p(stream),
                                        C.byref(st) if st is not None else None))
        return st.as_dict() if st is not None else None

    def set_directions(self, dirs=None, d_dirs: int = 0, ld: int = 0, n_dirs: int = 0) -> None:
        """Hit-and-run along a pool of directions (achr_set_directions): a host (n, K)
        array, or a device pointer with leading dimension ld; None / 0 returns to ACHR."""
        if dirs is not None:
            D = np.asfortranarray(np.asarray(dirs, dtype=np.float64))
            if D.shape[0] != self.n:
                raise ValueError(f"directions must be ({self.n}, K)")
            _check(lib().achr_set_directions(self._ctx, D.ctypes.data_as(C.c_void_p), self.n, D.shape[1]))
        else:
            _check(lib().achr_set_directions(self._ctx, C.c_void_p(d_dirs or None), ld, n_dirs))

    def directions(self) -> np.ndarray:
        """The installed hit-and-run direction pool, (n, K); empty in ACHR mode."""
        k = lib().achr_get_n_directions(self._ctx)
        out = np.zeros((self.n, k), order="F")
        if k:
            _check(lib().achr_get_directions(self._ctx, out.ctypes.data_as(C.c_void_p)))
        return out

    def check_directions(self, chains: int = 256, burnin: int = 20000, draws: int = 100, gap: int = 200,
                         seed: int = 0, rhat_limit: float = 1.01) -> dict:
        """Pilot of the installed pool; removes it (back to plain ACHR) when max split-R-hat >= rhat_limit."""
        out = DirectionCheck()
        _check(lib().achr_check_directions(self._ctx, chains, burnin, draws, gap, seed, rhat_limit, C.byref(out)))
        return out.as_dict()

    def precond_dim(self) -> tuple[int, int]:
        """(dimension of the preconditioner's basis, reactions pinned across all warmup points)."""
        d, f = C.c_int32(), C.c_int32()
        _check(lib().achr_precond_dim(self._ctx, C.byref(d), C.byref(f)))
        return d.value, f.value

    def precond_basis(self) -> np.ndarray:
        d, _ = self.precond_dim()
        out = np.zeros((self.n, d), order="F")
        if d:
            _check(lib().achr_get_precond_basis(self._ctx, out.ctypes.data_as(C.c_void_p)))
        return out

    def null_coords(self, n_points: int, d_points: int, ld: int, d_Y: int, ldy: int, d_mu: int = 0,
                    stream: int = 0) -> None:
        """Y (d x P FP32, device) = N^T (x - mu) for an n x ld device block of points."""
        _check(lib().achr_null_coords(self._ctx, n_points, C.c_void_p(d_points), ld, C.c_void_p(d_mu or None),
                                      C.c_void_p(d_Y), ldy, C.c_void_p(stream)))

    def precond_pool(self, rank: int, d_s: int, d_U: int, n_dirs: int, seed: int = 0) -> None:
        """Install a pool of n_dirs directions N (exp(s) z1 + U z2) (achr_precond_pool)."""
        _check(lib().achr_precond_pool(self._ctx, rank, C.c_void_p(d_s), C.c_void_p(d_U or None), n_dirs, seed))

    def reproject(self, n_points: int, d_points: int, ld: int, d_centre_acc: int = 0, max_rounds: int = 1,
                  stream: int = 0, with_stats: bool = True) -> Optional[dict]:
        """Reproject chains 0..P-1 of an n x ld device block in place (achr_reproject_batch)."""
        st = ReprojStats() if with_stats else None
        _check(lib().achr_reproject_batch(self._ctx, n_points, C.c_void_p(d_points), C.c_void_p(d_centre_acc or None),
                                          ld, max_rounds, C.c_void_p(stream), C.byref(st) if st is not None else None))
        return st.as_dict() if st is not None else None

    def sample_periodic(self, n_points: int, n_steps: int, period: int, d_points: int, d_centre_acc: int, ld: int,
                        stream: int = 0, seed: int = 0, chain_offset: int = 0, max_rounds: int = 4):
        """T steps in segments of `period`, each followed by a batched reprojection
        (achr_sample_periodic).  Returns (sampling stats, reprojection stats)."""
        st, rs = Stats(), ReprojStats()
        _check(lib().achr_sample_periodic(self._ctx, seed, chain_offset, n_points, n_steps, period, max_rounds,
                                          C.c_void_p(d_points), C.c_void_p(d_centre_acc), ld, C.c_void_p(stream),
                                          C.byref(st), C.byref(rs)))
        return st.as_dict(), rs.as_dict()

    def autotune(self) -> int:
        """Pick the fastest chain-kernel configuration for this model; returns threads per chain."""
        t = C.c_int32()
        _check(lib().achr_autotune(self._ctx, C.byref(t)))
        self.options.threads_per_chain = t.value
        return t.value

    def sample_device(self, n_points: int, n_steps: int, d_out: int, ld_out: int, stream: int = 0, seed: int = 0,
                      chain_offset: int = 0, with_stats: bool = False) -> Optional[dict]:
        """Queue sampling into device memory d_out (n x ld_out row-major) on a CUDA stream."""
        st = Stats() if with_stats else None
        _check(lib().achr_sample_device(self._ctx, seed, chain_offset, n_points, n_steps, C.c_void_p(d_out), ld_out,
                                        C.c_void_p(stream), C.byref(st) if st is not None else None))
        return st.as_dict() if st is not None else None


def sample_noalloc(model: DeviceModel, n_points: int, n_steps: int, d_out: int, ld_out: int, stream: int = 0,
                   seed: int = 0, chain_offset: int = 0, options: Optional[Options] = None) -> dict:
    """Sample through achr_sample_noalloc (no allocation by the library); returns the stats."""
    st = Stats()
    opt = options if options is not None else default_options()
    _check(lib().achr_sample_noalloc(C.byref(model), C.byref(opt), seed, chain_offset, n_points, n_steps,
                                     C.c_void_p(d_out), ld_out, C.c_void_p(stream), C.byref(st)))
    return st.as_dict()


def sample_batch(samplers, n_points, n_steps: int, d_outs, ld_outs, stream: int = 0, seed: int = 0):
    """Sample several models in one CUDA-graph launch (achr_sample_batch).
    Returns (batch stats dict, per-model finish times in ms)."""
    k = len(samplers)
    ctxs = (C.c_void_p * k)(*[s._ctx for s in samplers])
    pts = (C.c_int32 * k)(*n_points)
    outs = (C.c_void_p * k)(*d_outs)
    lds = (C.c_int64 * k)(*ld_outs)
    ms = (C.c_double * k)()
    st = BatchStats()
    _check(lib().achr_sample_batch(ctxs, k, pts, n_steps, seed, outs, lds, C.c_void_p(stream), C.byref(st), ms))
    return st.as_dict(), list(ms)


def set_batch_tiles(tiles: int) -> None:
    """Tile size of the batched work queues (achr_set_batch_tiles): an item holds the work queued
    behind it divided by tiles x the queue's CTAs."""
    _check(lib().achr_set_batch_tiles(tiles))


def batch_tiles() -> int:
    return int(lib().achr_get_batch_tiles())


def autotune_batch(samplers, n_points, n_steps: int, d_outs, ld_outs, stream: int = 0, seed: int = 0) -> int:
    """Time a short batched run with each tile setting (achr_autotune_batch) and keep the fastest."""
    k = len(samplers)
    ctxs = (C.c_void_p * k)(*[s._ctx for s in samplers])
    pts = (C.c_int32 * k)(*n_points)
    outs = (C.c_void_p * k)(*d_outs)
    lds = (C.c_int64 * k)(*ld_outs)
    best = C.c_int32()
    _check(lib().achr_autotune_batch(ctxs, k, pts, n_steps, seed, outs, lds, C.c_void_p(stream), C.byref(best)))
    return best.value


def gemm_bf16(M: int, N: int, K: int, A0: int, B0: int, C_out: int, lda: int, ldb: int, ldc: int,
              A1: int = 0, B1: int = 0, stream: int = 0) -> None:
    """Tensor-core GEMM on device pointers (achr_gemm_bf16): C = A0 B0^T, or with A1/B1
    given the three hi/lo split products A0 B0^T + A0 B1^T + A1 B0^T."""
    nsplit = 3 if (A1 and B1) else 1
    _check(lib().achr_gemm_bf16(M, N, K, nsplit, C.c_void_p(A0), C.c_void_p(A1 or None), lda, C.c_void_p(B0),
                                C.c_void_p(B1 or None), ldb, C.c_void_p(C_out), ldc, C.c_void_p(stream)))


def precond_options(**overrides) -> PrecondOptions:
    o = PrecondOptions()
    lib().achr_precond_default_options(C.byref(o))
    for k, v in overrides.items():
        setattr(o, k, v)
    return o


def precond_loss_grad(d: int, r: int, B: int, d_s: int, d_U: int, d_Y: int, ldy: int, d_gs: int, d_gU: int,
                      stream: int = 0) -> float:
    """Loss and gradients of the preconditioner on one minibatch (device pointers)."""
    loss = C.c_float()
    _check(lib().achr_precond_loss_grad(d, r, B, C.c_void_p(d_s), C.c_void_p(d_U), C.c_void_p(d_Y), ldy,
                                        C.byref(loss), C.c_void_p(d_gs), C.c_void_p(d_gU), C.c_void_p(stream)))
    return loss.value


def precond_train(d: int, r: int, n_samples: int, d_Y: int, ldy: int, d_s: int, d_U: int, stream: int = 0,
                  **options) -> dict:
    """Fit s, U (device, updated in place) to the samples Y (achr_precond_train)."""
    opt = precond_options(**options)
    st = PrecondStats()
    _check(lib().achr_precond_train(d, r, n_samples, C.c_void_p(d_Y), ldy, C.byref(opt), C.c_void_p(d_s),
                                    C.c_void_p(d_U), C.c_void_p(stream), C.byref(st)))
    return st.as_dict()


def exported_symbols() -> list[str]:
    """Function names declared in include/achr.h."""
    import re
    text = INCLUDE_HEADER.read_text()
    names = re.findall(r"^\s*(?:const\s+)?[\w\s\*]+?\b(achr_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))
