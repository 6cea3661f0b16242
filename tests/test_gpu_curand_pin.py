"""GPU: the sampler's Philox4x32-10 (oracle C code and the CUDA header shared by
the kernels) against cuRAND's device Philox4_32_10 on random counters and keys."""
from __future__ import annotations

import ctypes as C
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = Path(__file__).resolve().parent


@pytest.fixture(scope="module")
def curand_lib(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    out = tmp_path_factory.mktemp("curand") / "libcurand_philox.so"
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-shared", "-Xcompiler", "-fPIC",
                    str(HERE / "cuda" / "curand_philox.cu"), "-o", str(out)], check=True)
    lib = C.CDLL(str(out))
    u64p = C.POINTER(C.c_uint64)
    lib.curand_philox_batch.argtypes = [C.c_int, u64p, u64p, u64p, C.POINTER(C.c_uint32)]
    lib.curand_philox_batch.restype = C.c_int
    return lib


def test_philox_matches_curand(curand_lib, oracle_mod):
    rng = np.random.default_rng(2026)
    n = 4096
    ctr = rng.integers(0, 2 ** 32, size=(n, 4), dtype=np.uint64)
    ctr[:, 1] >>= np.uint64(2)  # the offset argument is 4 x (c1:c0) in 64 bits: c1 < 2^30
    key = rng.integers(0, 2 ** 32, size=(n, 2), dtype=np.uint64)
    ctr[:8] = 0  # include the all-zero counter and small counters
    ctr[8:16, 0] = np.arange(8)
    seed = np.ascontiguousarray(key[:, 0] | (key[:, 1] << np.uint64(32)))
    subseq = np.ascontiguousarray(ctr[:, 2] | (ctr[:, 3] << np.uint64(32)))
    offset = np.ascontiguousarray((ctr[:, 0] | (ctr[:, 1] << np.uint64(32))) * np.uint64(4))
    out = np.zeros((n, 4), dtype=np.uint32)
    u64p = C.POINTER(C.c_uint64)
    rc = curand_lib.curand_philox_batch(n, seed.ctypes.data_as(u64p), subseq.ctypes.data_as(u64p),
                                        offset.ctypes.data_as(u64p), out.ctypes.data_as(C.POINTER(C.c_uint32)))
    assert rc == 0
    ours = np.array([oracle_mod.philox([int(c) for c in ctr[i]], [int(k) for k in key[i]]) for i in range(n)],
                    dtype=np.uint32)
    assert np.array_equal(ours, out)
