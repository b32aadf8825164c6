"""Regenerates tests/golden/oracle_regression.npz: outputs of the FP64 oracle
(reference lookup-table mode) for small seeded sets of columns.  The fixtures
freeze the oracle: tests/test_oracle.py checks that it still reproduces them.
They are regression vectors of the restatement, not outputs of the reference
(which cannot be run here).

    python tests/golden/make_golden.py
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from mima_gb300 import atmosphere as A  # noqa: E402
from mima_gb300 import tables  # noqa: E402
from oracle import oracle as orc  # noqa: E402

CASES = {"l40": dict(ncol=8, nlay=40, seed=101, ts_sigma=2.0, rh_random=False),
         "l60": dict(ncol=6, nlay=60, seed=202, ts_sigma=5.0, rh_random=True)}


def compute():
    orc.build()
    orc.load(tables.ensure_blob())
    orc.set_table_mode(True)
    out = {}
    for name, c in CASES.items():
        atm = A.small_atmosphere(c["ncol"], c["nlay"], seed=c["seed"], ts_sigma=c["ts_sigma"],
                                 rh_random=c["rh_random"])
        lw, sw = orc.rrtmg_lw(atm, idrv=1), orc.rrtmg_sw(atm)
        for k in ("uflx", "dflx", "hr", "duflx_dt"):
            out[f"{name}_{k}"] = lw[k]
        for k in ("swuflx", "swdflx", "swhr"):
            out[f"{name}_{k}"] = sw[k]
    blob = Path(tables.ensure_blob()).read_bytes()
    out["blob_checksum"] = np.array([tables.blob_checksum(blob)], dtype=np.uint64)
    return out


if __name__ == "__main__":
    np.savez_compressed(Path(__file__).with_name("oracle_regression.npz"), **compute())
    print("wrote", Path(__file__).with_name("oracle_regression.npz"))
