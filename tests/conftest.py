"""Shared fixtures.  GPU tests are marked `gpu`; everything else runs on CPU."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = Path(__file__).resolve().parent / "golden"
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

import __graft_entry__ as graft_entry  # noqa: E402

PKG = graft_entry.load_package()


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built native library")


@pytest.fixture(scope="session")
def pkg():
    return PKG


@pytest.fixture(scope="session")
def native(pkg):
    """The built C-ABI library (built on demand; tests never fall back to Python)."""
    try:
        return pkg.lib()
    except ImportError:
        graft_entry._load_builder().build()
        return pkg.lib()


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle

    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def golden():
    z = np.load(GOLDEN / "small_golden.npz")
    return {k: z[k] for k in z.files}


@pytest.fixture(scope="session")
def small_model(pkg, golden):
    g = golden
    return pkg.HostModel(int(g["n_rxns"]), int(g["n_mets"]), g["row"], g["col"], g["val"], g["lb"], g["ub"])


@pytest.fixture(scope="session")
def putida_files(tmp_path_factory):
    """The reference's P_Putida model and its 2n %f warmup CSV, unpacked from tests/golden/."""
    import gzip
    import shutil

    d = tmp_path_factory.mktemp("putida")
    out = []
    for name in ("P_Putida.mps", "putida_warmup.csv"):
        with gzip.open(GOLDEN / (name + ".gz"), "rb") as f, open(d / name, "wb") as g:
            shutil.copyfileobj(f, g)
        out.append(d / name)
    return tuple(out)


def dense_S(model):
    S = np.zeros((model.n_mets, model.n_rxns))
    np.add.at(S, (np.asarray(model.row), np.asarray(model.col)), np.asarray(model.val))
    return S


def have_gpu() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:  # pragma: no cover
        return False
