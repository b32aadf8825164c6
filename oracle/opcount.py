"""Algorithmic FLOP count of the clear-sky LW and SW path -- TEST
INFRASTRUCTURE ONLY.

Runs the oracle's FLOP-count build (``make -C oracle opcount``: the same C++
restatement with ``double`` mapped onto the counting scalar of opcount.hpp,
results bit for bit those of the normal build) with one thread, in the
analytic-transcendental form (exp and the tau transition function evaluated,
not looked up), after the table initialisation, and returns the operations
per column by kind: add / sub, mul, div, sqrt, exp, log, pow, trigonometric,
comparisons.  The reference's redundant second SW two-stream pass (the "total"
stream, identical to the clear one in clear sky) is left out of the count.
FLOPs = add + mul + div + sqrt + exp + log + pow (every operation 1; FMA is
never formed, so a multiply-add counts 2).
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

from . import oracle as O

HERE = Path(__file__).resolve().parent
LIB = HERE / "build" / "liboracle_opcount.so"
KINDS = ("add", "mul", "div", "sqrt", "exp", "log", "pow", "trig", "cmp")
FLOP_KINDS = ("add", "mul", "div", "sqrt", "exp", "log", "pow")

_lib = None


def load(blob_path, cpdair: float = 1004.64):
    global _lib
    if _lib is None:
        subprocess.run(["make", "-s", "-C", str(HERE), "opcount"], check=True)
        lib = C.CDLL(str(LIB))
        lib.orc_init.argtypes = [C.c_char_p, C.c_double]
        lib.orc_set_table_mode.argtypes = [C.c_int]
        lib.orc_opcount_get.argtypes = [C.POINTER(C.c_ulonglong)]
        if lib.orc_init(str(blob_path).encode(), C.c_double(cpdair)) != 0:
            raise RuntimeError(f"counting oracle init failed for {blob_path}")
        lib.orc_set_table_mode(0)
        _lib = lib
    return _lib


def _counted(fn, *args, **kw):
    """Run an oracle wrapper of oracle.py on the counting library, one thread."""
    saved = O._lib
    O._lib = _lib
    try:
        _lib.orc_opcount_reset()
        out = fn(*args, nthreads=1, **kw)
        buf = (C.c_ulonglong * len(KINDS))()
        _lib.orc_opcount_get(buf)
    finally:
        O._lib = saved
    return out, dict(zip(KINDS, (int(x) for x in buf)))


def count(atm):
    """(lw, sw, counts_lw, counts_sw): outputs and operation counts per column."""
    lw, cl = _counted(O.rrtmg_lw, atm)
    sw, cs = _counted(O.rrtmg_sw, atm)
    per = lambda c: {k: v / atm.ncol for k, v in c.items()}
    return lw, sw, per(cl), per(cs)


def count_clouds(atm, lw_cloud, sw_cloud, lw_icld: int = 2):
    """Operation counts per column of a cloudy LW call (overlap ``lw_icld``)
    and a cloudy SW call on ``atm``: the cloud physics, the cloudy solver
    branches and the SW total-sky pass (work of its own in a call with
    clouds) counted.  Returns (counts_lw, counts_sw)."""
    _, cl = _counted(O.rrtmg_lw, atm, cloud=lw_cloud, icld=lw_icld)
    _, cs = _counted(O.rrtmg_sw, atm, cloud=sw_cloud)
    per = lambda c: {k: v / atm.ncol for k, v in c.items()}
    return per(cl), per(cs)


def flops(c) -> float:
    return float(sum(c[k] for k in FLOP_KINDS))


LW_PHASES = ("inatm", "setcoef", "taumol", "rtrnmr")
SW_PHASES = ("inatm_sw", "setcoef_sw", "taumol_sw", "spcvrt_sw")


def phase_flops(atm):
    """FLOPs per column of each phase of the clear-sky LW and SW path (SW over
    the sunlit columns), as two dicts keyed by LW_PHASES / SW_PHASES."""
    nk = len(KINDS)
    buf = (C.c_ulonglong * (4 * nk))()
    f = lambda a: np.ascontiguousarray(a, dtype=np.float64)
    p = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    lw = [f(a) for a in (atm.play, atm.plev, atm.tlay, atm.tlev, atm.tsfc, atm.h2o, atm.o3, atm.co2, atm.ch4,
                         atm.n2o, atm.o2, atm.cfc11, atm.cfc12, atm.cfc22, atm.ccl4, atm.emis)]
    _lib.orc_lw_phase_counts(C.c_int(atm.ncol), C.c_int(atm.nlay), *[p(a) for a in lw], buf)
    per = lambda n: [flops(dict(zip(KINDS, (buf[ph * nk + k] / n for k in range(nk))))) for ph in range(4)]
    out_lw = dict(zip(LW_PHASES, per(atm.ncol)))
    sw = [f(a) for a in (atm.play, atm.plev, atm.tlay, atm.tlev, atm.tsfc, atm.h2o, atm.o3, atm.co2, atm.ch4,
                         atm.n2o, atm.o2, atm.asdir, atm.asdif, atm.aldir, atm.aldif, atm.coszen)]
    _lib.orc_sw_phase_counts(C.c_int(atm.ncol), C.c_int(atm.nlay), *[p(a) for a in sw], C.c_double(atm.adjes),
                             C.c_int(atm.dyofyr), C.c_double(atm.scon), buf)
    lit = max(1, int((np.asarray(atm.coszen) >= 1e-10).sum()))
    return out_lw, dict(zip(SW_PHASES, per(lit)))


def table(blob_path, layers=(20, 40, 60, 80), ncol: int = 8, seed: int = 11):
    """FLOPs per column of LW and SW for each layer count, and the least-squares
    line a + b L through them."""
    load(blob_path)
    rows = []
    for L in layers:
        from mima_gb300 import atmosphere as A
        atm = A.small_atmosphere(ncol, L, seed=seed, rh_random=False)
        _, _, cl, cs = count(atm)
        rows.append((L, flops(cl), flops(cs), cl, cs))
    Ls = np.array([r[0] for r in rows], dtype=float)
    fit = lambda y: np.polyfit(Ls, np.array(y), 1)
    return rows, fit([r[1] for r in rows]), fit([r[2] for r in rows])
