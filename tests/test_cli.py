"""The ACHRCuda command line: the reference's five positional arguments and File<ii> output."""
from __future__ import annotations

import json
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN


def _run(pkg, args, cwd):
    return subprocess.run([str(pkg.cli_path()), *map(str, args)], cwd=cwd, capture_output=True, text=True,
                          timeout=600)


def test_cli_usage_error(native, pkg, tmp_path):
    r = _run(pkg, ["only", "two"], tmp_path)
    assert r.returncode == 2 and "usage" in r.stderr


def test_cli_unreadable_model_exit_code(native, pkg, tmp_path):
    """The reference returns 1 when the MPS file cannot be read (ACHRCuda.cu:563-566)."""
    r = _run(pkg, [tmp_path / "missing.mps", GOLDEN / "small_warmup.csv", 1, 2, 2], tmp_path)
    assert r.returncode == 1 and "Error reading MPS file" in r.stdout


def test_cli_bad_numbers(native, pkg, tmp_path):
    r = _run(pkg, [GOLDEN / "small.mps", GOLDEN / "small_warmup.csv", 1, "x", 2], tmp_path)
    assert r.returncode == 2


@pytest.mark.parametrize("flags", [["--reproject", "fast"], ["--check-period", "-1"], ["--mode", "x"],
                                   ["--bracket-pass", "both"], ["--seed"], ["--bogus", "1"]])
def test_cli_bad_flags(native, pkg, tmp_path, flags):
    r = _run(pkg, [GOLDEN / "small.mps", GOLDEN / "small_warmup.csv", 1, 2, 2, *flags], tmp_path)
    assert r.returncode == 2


def test_cli_truncated_warmup(native, pkg, tmp_path):
    bad = tmp_path / "w.csv"
    bad.write_text("\n".join((GOLDEN / "small_warmup.csv").read_text().splitlines()[:10]) + "\n")
    r = _run(pkg, [GOLDEN / "small.mps", bad, 1, 2, 2], tmp_path)
    assert r.returncode == 2 and "lines" in r.stderr


@pytest.mark.gpu
def test_cli_end_to_end_matches_oracle(native, pkg, oracle_mod, tmp_path):
    """Two files of 12 chains x 30 steps: File<ii> has n lines of 12 "%f" values,
    chain ids ii*12.., and equals the oracle's points (same seed, same basis N)
    formatted with "%f"."""
    model = pkg.read_mps(GOLDEN / "small.mps")
    warm = pkg.read_warmup_csv(GOLDEN / "small_warmup.csv", model.n_rxns)
    r = _run(pkg, [GOLDEN / "small.mps", GOLDEN / "small_warmup.csv", 2, 12, 30, "--seed", 4242, "--report",
                   "rep.json"], tmp_path)
    assert r.returncode == 0, r.stdout + r.stderr
    for line in ("Null space done in", "File 0", "File 1", "Sampling done in", "nWrmup egale a 190"):
        assert line in r.stdout
    rep = json.loads((tmp_path / "rep.json").read_text())
    assert rep["accepted"] == 2 * 12 * 30 and rep["stuck_chains"] == 0
    with pkg.Sampler(model, warm) as s:  # the same set-up the CLI ran: same basis
        N = s.null_space()
    for ii in range(2):
        text = (tmp_path / f"File{ii}").read_text()
        lines = text.split("\n")
        assert lines[-1] == "" and len(lines) == model.n_rxns + 1
        assert all(len(ln.split(",")) == 12 for ln in lines[:-1])
        ref, _ = oracle_mod.sample(model, warm, N, 4242, 12, 30, chain_offset=ii * 12)
        want = "".join(",".join("%f" % v for v in row) + "\n" for row in ref)
        if text != want:  # a value within 1e-12 of a rounding boundary may print either way
            got = np.array([[float(t) for t in ln.split(",")] for ln in lines[:-1]])
            assert np.abs(got - ref).max() <= 5e-7 + 1e-9 * np.abs(ref).max()
