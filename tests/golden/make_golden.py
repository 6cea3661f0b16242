"""Generate the committed golden fixtures of the test suite.

Run from the repository root:  python tests/golden/make_golden.py

Writes into tests/golden/:
  small.mps           seeded 72 x 95 synthetic model (fixed MPS, the layout of
                      VFWarmup/test_fva_validation.py:49-90)
  small_warmup.csv    190 = 2n warmup points from the LP restatement of
                      VFWarmup/createWarmupPtsGLPK.c (scipy HiGHS), "%f" text
  small_golden.npz    the model arrays, the parsed warmup, a null-space basis
                      from the SVD of S^T S (ACHRCuda.cu:436-502) and the final
                      points of 6 chains x 60 steps from the pure-Python
                      restatement (oracle/reference_py.py), seed 1234
  philox_kat.json     Philox4x32-10 known-answer vectors published with
                      Random123 (Salmon et al., SC'11)

The C oracle is checked against these in tests/test_oracle.py; the GPU kernel
against the C oracle in tests/test_gpu_parity.py.
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import __graft_entry__ as ge  # noqa: E402

ge.load_package()
from achr_gb300 import synthetic  # noqa: E402
from oracle import reference_py, warmup  # noqa: E402

OUT = Path(__file__).resolve().parent
SEED = 1234
CHAINS = 6
STEPS = 60

PHILOX_KAT = [
    {"ctr": ["00000000", "00000000", "00000000", "00000000"], "key": ["00000000", "00000000"],
     "out": ["6627e8d5", "e169c58d", "bc57ac4c", "9b00dbd8"]},
    {"ctr": ["ffffffff", "ffffffff", "ffffffff", "ffffffff"], "key": ["ffffffff", "ffffffff"],
     "out": ["408f276d", "41c83b0e", "a20bc7c6", "6d5451fd"]},
    {"ctr": ["243f6a88", "85a308d3", "13198a2e", "03707344"], "key": ["a4093822", "299f31d0"],
     "out": ["d16cfe09", "94fdcceb", "5001e420", "24126ea1"]},
]


def parse_csv(path, n):
    rows = [line for line in Path(path).read_text().splitlines() if line.strip()]
    assert len(rows) == n
    return np.array([[float(t) for t in r.split(",")] for r in rows])


def main():
    spec = synthetic.SMALL
    row, col, val, lb, ub = synthetic.make_model(spec)
    synthetic.write_mps(OUT / "small.mps", spec.n_mets, spec.n_rxns, row, col, val, lb, ub, name="SMALL")
    S = synthetic.dense(spec.n_mets, spec.n_rxns, row, col, val)
    wu = warmup.lp_warmup(S, lb, ub, 2 * spec.n_rxns, seed=5)
    warmup.write_csv(OUT / "small_warmup.csv", wu)
    W = parse_csv(OUT / "small_warmup.csv", spec.n_rxns)
    N = reference_py.null_space_sts(S)
    c0 = reference_py.centre(W)
    rows = reference_py.rows_of(spec.n_mets, row, col, val)
    pts = np.zeros((spec.n_rxns, CHAINS))
    rejected = 0
    for p in range(CHAINS):
        x, rej, stuck = reference_py.sample_chain(rows, lb, ub, W, N, c0, SEED, p, STEPS)
        assert not stuck
        pts[:, p] = x
        rejected += rej
    np.savez_compressed(OUT / "small_golden.npz", row=row, col=col, val=val, lb=lb, ub=ub, n_mets=spec.n_mets,
                        n_rxns=spec.n_rxns, warmup=W, N=N, centre=c0, seed=SEED, chains=CHAINS, steps=STEPS,
                        points=pts, rejected=rejected)
    (OUT / "philox_kat.json").write_text(json.dumps(PHILOX_KAT, indent=1) + "\n")
    print(f"n={spec.n_rxns} m={spec.n_mets} W={W.shape[1]} d={N.shape[1]} rejected={rejected}")
    print(f"max |S w| of parsed warmup: {np.abs(S @ W).max():.3e}")


if __name__ == "__main__":
    main()
