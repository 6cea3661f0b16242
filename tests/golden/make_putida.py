"""Fixture of the reference's own model: VFWarmup/lib/P_Putida.mps (911 x 1060).

Writes, next to this script:
  P_Putida.mps.gz            the reference's model file, gzipped, unchanged
  putida_warmup.csv.gz       2n = 2120 warmup points made from it by
                             oracle/warmup.py (the restatement of
                             VFWarmup/createWarmupPtsGLPK.c with HiGHS), written
                             with "%f" as that program writes them (one line
                             per reaction, comma-separated), gzipped

The model has non-integer coefficients (e.g. -5E-05, 45.5608), 19 fixed
reactions and bounds of several magnitudes, none of which the synthetic
generator produces.  Run where a checkout of the reference exists:

    ACHR_REFERENCE_DIR=<checkout> python tests/golden/make_putida.py
"""
from __future__ import annotations

import gzip
import os
import shutil
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))


def main() -> None:
    ref = Path(os.environ.get("ACHR_REFERENCE_DIR", "/root/reference"))
    src = ref / "VFWarmup" / "lib" / "P_Putida.mps"
    with open(src, "rb") as f, gzip.GzipFile(HERE / "P_Putida.mps.gz", "wb", mtime=0) as g:
        shutil.copyfileobj(f, g)

    import __graft_entry__ as ge
    from oracle import warmup

    pkg = ge.load_package()
    m = pkg.read_mps(src)
    warm = warmup.lp_warmup(m.dense(), m.lb, m.ub, 2 * m.n_rxns, seed=0, workers=os.cpu_count() or 1)
    tmp = HERE / "putida_warmup.csv"
    warmup.write_csv(tmp, warm)
    with open(tmp, "rb") as f, gzip.GzipFile(HERE / "putida_warmup.csv.gz", "wb", mtime=0) as g:
        shutil.copyfileobj(f, g)
    tmp.unlink()
    print(f"wrote {m.n_mets} x {m.n_rxns} model and {warm.shape[1]} warmup points")


if __name__ == "__main__":
    main()
