"""CPU oracle of the ACHR sampling step -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline and
reference arms may import this package, and only as the checker or as the
timed CPU reference.  The product (the CUDA library and the ACHRCuda CLI)
never calls into it.

PARITY UNPINNED: the reference sampler (ACHRcu/ACHRCuda.cu) cannot be built
here (CUDA 13 rejects its device-side cudaDeviceSynchronize(), sm_37 is gone,
GLPK and GSL are absent) and ships no golden outputs or known-answer tests.
The restatement is pinned by the published Philox4x32-10 known-answer
vectors, by an independent pure-Python restatement (tests/golden/make_golden.py)
whose outputs are committed as fixtures, and by invariants.

Contents:
  achr_oracle.c      FP64 C restatement of the step loop (ACHRcu/ACHRCuda.cu:193-385)
  reference_py.py    pure-Python/numpy restatement of the same loop and of
                     computeKernelCuda / createCenterPt (:414-502)
  warmup.py          restatement of VFWarmup/createWarmupPtsGLPK.c with scipy HiGHS
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD_DIR = HERE / "_build"
LIB_PATH = BUILD_DIR / "liboracle.so"


def build(force: bool = False) -> Path:
    """Compile achr_oracle.c into _build/liboracle.so (gcc, OpenMP, no FP contraction)."""
    src = HERE / "achr_oracle.c"
    if not force and LIB_PATH.exists() and LIB_PATH.stat().st_mtime > src.stat().st_mtime:
        return LIB_PATH
    BUILD_DIR.mkdir(exist_ok=True)
    cc = os.environ.get("CC", "gcc")
    cmd = [cc, "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-std=c11", str(src), "-o",
           str(LIB_PATH), "-lm"]
    res = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed: {' '.join(cmd)}\n{res.stdout}")
    return LIB_PATH


class _Problem(C.Structure):
    _fields_ = [
        ("n", C.c_int32), ("m", C.c_int32), ("n_warmup", C.c_int32),
        ("warmup", C.POINTER(C.c_double)), ("lb", C.POINTER(C.c_double)), ("ub", C.POINTER(C.c_double)),
        ("row_ptr", C.POINTER(C.c_int32)), ("col_idx", C.POINTER(C.c_int32)), ("val", C.POINTER(C.c_double)),
        ("d", C.c_int32), ("N", C.POINTER(C.c_double)), ("centre", C.POINTER(C.c_double)),
    ]


class _Options(C.Structure):
    _fields_ = [
        ("check_period", C.c_int32), ("max_attempts", C.c_int32), ("centre_offset", C.c_int32),
        ("threads", C.c_int32), ("hit_and_run", C.c_int32), ("reserved", C.c_int32),
        ("residual_tol", C.c_double), ("max_min_tol", C.c_double), ("u_tol", C.c_double), ("d_tol", C.c_double),
    ]


class _Stats(C.Structure):
    _fields_ = [("accepted", C.c_int64), ("rejected", C.c_int64), ("checks", C.c_int64),
                ("reprojections", C.c_int64), ("stuck_chains", C.c_int64)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build()
        h = C.CDLL(str(path))
        h.oracle_philox4x32_10.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
        h.oracle_philox4x32_10.restype = None
        h.oracle_warmup_index.argtypes = [C.c_uint64, C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32]
        h.oracle_warmup_index.restype = C.c_uint32
        h.oracle_step_uniform.argtypes = [C.c_uint64, C.c_uint64, C.c_uint32]
        h.oracle_step_uniform.restype = C.c_double
        h.oracle_sample.argtypes = [C.POINTER(_Problem), C.POINTER(_Options), C.c_uint64, C.c_uint64, C.c_int32,
                                    C.c_int32, C.POINTER(C.c_double), C.POINTER(_Stats)]
        h.oracle_sample.restype = C.c_int
        h.oracle_centre.argtypes = [C.c_int32, C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        h.oracle_centre.restype = None
        _lib = h
    return _lib


def philox(ctr, key):
    c = (C.c_uint32 * 4)(*[int(x) & 0xFFFFFFFF for x in ctr])
    k = (C.c_uint32 * 2)(*[int(x) & 0xFFFFFFFF for x in key])
    o = (C.c_uint32 * 4)()
    lib().oracle_philox4x32_10(c, k, o)
    return [int(x) for x in o]


def warmup_index(seed, chain, step, attempt, W):
    return int(lib().oracle_warmup_index(seed, chain, step, attempt, W))


def step_uniform(seed, chain, step):
    return float(lib().oracle_step_uniform(seed, chain, step))


def csr(n_mets, row, col, val):
    """CSR of S from COO (duplicates summed, zeros dropped), rows then columns ascending."""
    row = np.asarray(row, dtype=np.int64)
    col = np.asarray(col, dtype=np.int64)
    val = np.asarray(val, dtype=np.float64)
    n_cols = int(col.max()) + 1 if col.size else 1
    key = row * n_cols + col
    uk, inv = np.unique(key, return_inverse=True)
    sums = np.zeros(uk.size)
    np.add.at(sums, inv, val)
    keep = sums != 0.0
    uk, sums = uk[keep], sums[keep]
    r = (uk // n_cols).astype(np.int64)
    row_ptr = np.zeros(n_mets + 1, dtype=np.int32)
    np.add.at(row_ptr, r + 1, 1)
    row_ptr = np.cumsum(row_ptr).astype(np.int32)
    return row_ptr, (uk % n_cols).astype(np.int32), sums


def centre(warmup):
    w = np.asfortranarray(np.asarray(warmup, dtype=np.float64))
    n, W = w.shape
    out = np.zeros(n)
    lib().oracle_centre(n, W, w.ctypes.data_as(C.POINTER(C.c_double)), out.ctypes.data_as(C.POINTER(C.c_double)))
    return out


class Problem:
    """A model, its warmup points and a null-space basis prepared once for the C oracle."""

    def __init__(self, model, warmup, N, centre_point=None):
        n = model.n_rxns
        self.n = n
        self.w = np.asfortranarray(np.asarray(warmup, dtype=np.float64))
        self.N = np.asfortranarray(np.asarray(N, dtype=np.float64).reshape(n, -1))
        self.rp, self.ci, self.vv = csr(model.n_mets, model.row, model.col, model.val)
        self.lb = np.ascontiguousarray(model.lb, dtype=np.float64)
        self.ub = np.ascontiguousarray(model.ub, dtype=np.float64)
        self.c0 = centre(self.w) if centre_point is None else np.ascontiguousarray(centre_point, dtype=np.float64)
        dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))  # noqa: E731
        ip = lambda a: a.ctypes.data_as(C.POINTER(C.c_int32))  # noqa: E731
        self.pb = _Problem(n, model.n_mets, self.w.shape[1], dp(self.w), dp(self.lb), dp(self.ub), ip(self.rp),
                           ip(self.ci), dp(self.vv), self.N.shape[1], dp(self.N), dp(self.c0))

    def sample(self, seed, n_points, n_steps, chain_offset=0, check_period=10, max_attempts=100000, centre_offset=0,
               threads=0, residual_tol=1e-9, max_min_tol=1e-9, u_tol=1e-9, d_tol=1e-14, hit_and_run=False):
        """Returns ((n, P) points, stats dict).  hit_and_run: the warmup matrix holds
        directions (u = w_r / |w_r|, no centre) and chains start at centre_point."""
        op = _Options(check_period, max_attempts, centre_offset, threads, int(hit_and_run), 0, residual_tol,
                      max_min_tol, u_tol, d_tol)
        out = np.zeros((self.n, n_points))
        st = _Stats()
        rc = lib().oracle_sample(C.byref(self.pb), C.byref(op), seed, chain_offset, n_points, n_steps,
                                 out.ctypes.data_as(C.POINTER(C.c_double)), C.byref(st))
        if rc != 0:
            raise RuntimeError(f"oracle_sample failed ({rc})")
        return out, {k: getattr(st, k) for k, _ in st._fields_}


def sample(model, warmup, N, seed, n_points, n_steps, chain_offset=0, check_period=10, max_attempts=100000,
           centre_offset=0, threads=0, residual_tol=1e-9, max_min_tol=1e-9, u_tol=1e-9, d_tol=1e-14,
           centre_point=None):
    """Run the C oracle.  model: object with n_rxns, n_mets, row, col, val, lb, ub.
    warmup: (n, W); N: (n, d).  Returns ((n, P) points, stats dict)."""
    return Problem(model, warmup, N, centre_point).sample(
        seed, n_points, n_steps, chain_offset=chain_offset, check_period=check_period, max_attempts=max_attempts,
        centre_offset=centre_offset, threads=threads, residual_tol=residual_tol, max_min_tol=max_min_tol,
        u_tol=u_tol, d_tol=d_tol)
