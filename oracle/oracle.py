"""ctypes front end of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use
this module, as the checker.  It builds ``oracle/build/liboracle.so`` (the C++
FP64 restatement of the reference's RRTMG path -- clear sky, the non-McICA
cloudy paths and McICA with its stochastic cloud generator; see the .cpp files
for the file:line each function follows) with ``make`` when it is missing.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "build" / "liboracle.so"

_lib = None
_blob = None

_dp = C.POINTER(C.c_double)


def build(force: bool = False) -> Path:
    if force or not LIB.exists() or any(
            p.stat().st_mtime > LIB.stat().st_mtime for p in HERE.glob("oracle_*")):
        subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB


def _p(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def load(blob_path, cpdair: float = 1004.64):
    """Load the oracle with the given table blob (idempotent per blob)."""
    global _lib, _blob
    if _lib is None:
        build()
        _lib = C.CDLL(str(LIB))
        _lib.orc_init.argtypes = [C.c_char_p, C.c_double]
        _lib.orc_set_table_mode.argtypes = [C.c_int]
        _lib.orc_table.argtypes = [C.c_char_p, C.c_char_p, _dp, C.c_int]
        _lib.orc_max_threads.restype = C.c_int
    key = (str(blob_path), cpdair)
    if _blob != key:
        rc = _lib.orc_init(str(blob_path).encode(), C.c_double(cpdair))
        if rc != 0:
            raise RuntimeError(f"oracle init failed ({rc}) for {blob_path}")
        _blob = key
    return _lib


def set_table_mode(use_tables: bool) -> None:
    _lib.orc_set_table_mode(1 if use_tables else 0)


def max_threads() -> int:
    return int(_lib.orc_max_threads())


def _f(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class CloudRangeError(RuntimeError):
    """A cloud effective radius outside the range of its parameterisation's
    table: the reference's cldprop / cldprop_sw stop."""


def rrtmg_lw(atm, idrv: int = 0, tauaer=None, nthreads: int = 0, cloud=None, icld: int = 1):
    """rrtmg_lw on ``atm``; returns dict of (nlev, ncol) arrays.  Clear sky, or
    with ``cloud`` = dict(cldfr=(nlay, ncol), taucld=(nlay, ncol, 16) [Fortran
    (16, ncol, nlay)], cicewp / cliqwp (nlay, ncol), and for the cloud physics
    inflag (0: optical depths given, 1: abscld1 x water path, 2: ice and
    liquid parameterisations), iceflag, liqflag, reice / reliq (nlay, ncol)):
    random overlap (``icld`` = 1, rtrn) or maximum/random overlap (``icld`` =
    2 or 3, rtrnmr)."""
    n, L = atm.ncol, atm.nlay
    out = {k: np.zeros((L + 1, n)) for k in ("uflx", "dflx", "uflxc", "dflxc", "duflx_dt", "duflxc_dt")}
    out.update({k: np.zeros((L, n)) for k in ("hr", "hrc")})
    args = [_f(atm.play), _f(atm.plev), _f(atm.tlay), _f(atm.tlev), _f(atm.tsfc), _f(atm.h2o),
            _f(atm.o3), _f(atm.co2), _f(atm.ch4), _f(atm.n2o), _f(atm.o2), _f(atm.cfc11),
            _f(atm.cfc12), _f(atm.cfc22), _f(atm.ccl4), _f(atm.emis),
            None if tauaer is None else _f(tauaer)]
    cl = cloud or {}
    carg = [None if cl.get(k) is None else _f(cl[k]) for k in ("cldfr", "taucld", "cicewp", "cliqwp")]
    rad = [None if cl.get(k) is None else _f(cl[k]) for k in ("reice", "reliq")]
    flags = [C.c_int(int(cl.get(k, 0))) for k in ("inflag", "iceflag", "liqflag")]
    rc = _lib.orc_rrtmg_lw(C.c_int(n), C.c_int(L), C.c_int(icld if cloud else 0), C.c_int(idrv),
                           *[_p(a) for a in args],
                           _p(out["uflx"]), _p(out["dflx"]), _p(out["hr"]), _p(out["uflxc"]),
                           _p(out["dflxc"]), _p(out["hrc"]), _p(out["duflx_dt"]), _p(out["duflxc_dt"]),
                           C.c_int(nthreads), *[_p(a) for a in carg], *flags, *[_p(a) for a in rad])
    if rc == 5:
        raise CloudRangeError("an effective radius is outside its parameterisation's range (cldprop stops)")
    if rc != 0:
        raise RuntimeError(f"orc_rrtmg_lw failed ({rc})")
    return out


def rrtmg_lw_bands(atm, idrv: int = 0):
    """Per-band clear-sky LW fluxes: dict of (16, nlev, ncol) arrays "uflx",
    "dflx" and (idrv = 1) "duflx_dt", one column at a time, W/m2."""
    n, L = atm.ncol, atm.nlay
    out = {k: np.zeros((16, L + 1, n)) for k in ("uflx", "dflx", "duflx_dt")}
    args = [_f(atm.play), _f(atm.plev), _f(atm.tlay), _f(atm.tlev), _f(atm.tsfc), _f(atm.h2o),
            _f(atm.o3), _f(atm.co2), _f(atm.ch4), _f(atm.n2o), _f(atm.o2), _f(atm.cfc11),
            _f(atm.cfc12), _f(atm.cfc22), _f(atm.ccl4), _f(atm.emis)]
    rc = _lib.orc_rrtmg_lw_bands(C.c_int(n), C.c_int(L), C.c_int(idrv), *[_p(a) for a in args],
                                 _p(out["uflx"]), _p(out["dflx"]), _p(out["duflx_dt"]))
    if rc != 0:
        raise RuntimeError(f"orc_rrtmg_lw_bands failed ({rc})")
    return out


LW_PHASES = ("inatm", "setcoef", "taumol", "rtrnmr")
SW_PHASES = ("inatm_sw", "setcoef_sw", "taumol_sw", "spcvrt_sw")


def phase_times(atm):
    """Where the time goes on the CPU: seconds per column of each phase of the
    clear-sky LW and SW path (one thread; SW over the sunlit columns), as two
    dicts keyed by LW_PHASES / SW_PHASES.  spcvrt_sw holds the reference's two
    two-stream passes (the clear and the "total" one) and the heating rates."""
    ns = (C.c_longlong * 4)()
    lw = [_f(a) for a in (atm.play, atm.plev, atm.tlay, atm.tlev, atm.tsfc, atm.h2o, atm.o3, atm.co2, atm.ch4,
                          atm.n2o, atm.o2, atm.cfc11, atm.cfc12, atm.cfc22, atm.ccl4, atm.emis)]
    if _lib.orc_lw_phase_times(C.c_int(atm.ncol), C.c_int(atm.nlay), *[_p(a) for a in lw], ns) != 0:
        raise RuntimeError("orc_lw_phase_times failed")
    out_lw = {k: v * 1e-9 / atm.ncol for k, v in zip(LW_PHASES, ns)}
    sw = [_f(a) for a in (atm.play, atm.plev, atm.tlay, atm.tlev, atm.tsfc, atm.h2o, atm.o3, atm.co2, atm.ch4,
                          atm.n2o, atm.o2, atm.asdir, atm.asdif, atm.aldir, atm.aldif, atm.coszen)]
    if _lib.orc_sw_phase_times(C.c_int(atm.ncol), C.c_int(atm.nlay), *[_p(a) for a in sw],
                               C.c_double(atm.adjes), C.c_int(atm.dyofyr), C.c_double(atm.scon), ns) != 0:
        raise RuntimeError("orc_sw_phase_times failed")
    lit = max(1, int((np.asarray(atm.coszen) >= 1e-10).sum()))
    out_sw = {k: v * 1e-9 / lit for k, v in zip(SW_PHASES, ns)}
    return out_lw, out_sw


class PartialCloud(RuntimeError):
    """A partly cloudy layer in a SW call with clouds: the reference's
    non-McICA SW stops (rrtmg_sw_rad.nomcica.f90:533-538)."""


def rrtmg_sw(atm, iaer: int = 0, tauaer=None, ssaaer=None, asmaer=None, nthreads: int = 0, cloud=None):
    """rrtmg_sw on ``atm``.  ``cloud`` = dict(cldfr (nlay, ncol), taucld, ssacld,
    asmcld, fsfcld (nlay, ncol, 14) [Fortran (14, ncol, nlay)], optional cicewp
    / cliqwp (nlay, ncol)): icld = 1, cloud optics given (inflgsw = 0); or
    with inflag = 2, iceflag (1..3), liqflag (1), cicewp / cliqwp and reice /
    reliq (nlay, ncol): the optics from the ice and liquid parameterisations."""
    n, L = atm.ncol, atm.nlay
    out = {k: np.zeros((L + 1, n)) for k in ("swuflx", "swdflx", "swuflxc", "swdflxc")}
    out.update({k: np.zeros((L, n)) for k in ("swhr", "swhrc")})
    args = [_f(atm.play), _f(atm.plev), _f(atm.tlay), _f(atm.tlev), _f(atm.tsfc), _f(atm.h2o),
            _f(atm.o3), _f(atm.co2), _f(atm.ch4), _f(atm.n2o), _f(atm.o2), _f(atm.asdir),
            _f(atm.asdif), _f(atm.aldir), _f(atm.aldif), _f(atm.coszen)]
    aer = [None if a is None else _f(a) for a in (tauaer, ssaaer, asmaer)]
    cl = cloud or {}
    carg = [None if cl.get(k) is None else _f(cl[k])
            for k in ("cldfr", "taucld", "ssacld", "asmcld", "fsfcld", "cicewp", "cliqwp")]
    rad = [None if cl.get(k) is None else _f(cl[k]) for k in ("reice", "reliq")]
    flags = [C.c_int(int(cl.get(k, 0))) for k in ("inflag", "iceflag", "liqflag")]
    rc = _lib.orc_rrtmg_sw(C.c_int(n), C.c_int(L), C.c_int(1 if cloud else 0), C.c_int(iaer),
                           *[_p(a) for a in args],
                           C.c_double(atm.adjes), C.c_int(atm.dyofyr), C.c_double(atm.scon),
                           *[_p(a) for a in aer],
                           _p(out["swuflx"]), _p(out["swdflx"]), _p(out["swhr"]), _p(out["swuflxc"]),
                           _p(out["swdflxc"]), _p(out["swhrc"]), C.c_int(nthreads), *[_p(a) for a in carg],
                           *flags, *[_p(a) for a in rad])
    if rc == 5:
        raise CloudRangeError("an effective size is outside its parameterisation's range (cldprop_sw stops)")
    if rc == 4:
        raise PartialCloud("a layer is partly cloudy (0 < cldfr < 1): not computed without McICA")
    if rc != 0:
        raise RuntimeError(f"orc_rrtmg_sw failed ({rc})")
    return out


def lw_optics(atm):
    n, L = atm.ncol, atm.nlay
    taug = np.zeros((140, L, n))
    fracs = np.zeros((140, L, n))
    laytrop = np.zeros(n, dtype=np.int32)
    args = [_f(atm.play), _f(atm.plev), _f(atm.tlay), _f(atm.tlev), _f(atm.tsfc), _f(atm.h2o),
            _f(atm.o3), _f(atm.co2), _f(atm.ch4), _f(atm.n2o), _f(atm.o2)]
    rc = _lib.orc_lw_optics(C.c_int(n), C.c_int(L), *[_p(a) for a in args], _p(taug), _p(fracs),
                            laytrop.ctypes.data_as(C.POINTER(C.c_int)))
    if rc != 0:
        raise RuntimeError("orc_lw_optics failed")
    return taug, fracs, laytrop


def sw_optics(atm):
    n, L = atm.ncol, atm.nlay
    taug = np.zeros((112, L, n))
    taur = np.zeros((112, L, n))
    sfz = np.zeros((112, n))
    args = [_f(atm.play), _f(atm.plev), _f(atm.tlay), _f(atm.tlev), _f(atm.tsfc), _f(atm.h2o),
            _f(atm.o3), _f(atm.co2), _f(atm.ch4), _f(atm.n2o), _f(atm.o2)]
    rc = _lib.orc_sw_optics(C.c_int(n), C.c_int(L), *[_p(a) for a in args], _p(taug), _p(taur), _p(sfz))
    if rc != 0:
        raise RuntimeError("orc_sw_optics failed")
    return taug, taur, sfz


def table(key: str, name: str) -> np.ndarray:
    buf = np.zeros(1 << 16)
    n = _lib.orc_table(key.encode(), name.encode(), _p(buf), C.c_int(buf.size))
    if n < 0:
        raise KeyError((key, name))
    if n > buf.size:
        buf = np.zeros(n)
        _lib.orc_table(key.encode(), name.encode(), _p(buf), C.c_int(n))
    return buf[:n].copy()


def mt_ints(seed: int, n: int) -> np.ndarray:
    """The first n tempered 32-bit draws of the reference's Mersenne Twister
    (mcica_random_numbers.f90) seeded with ``seed``."""
    out = np.zeros(n, dtype=np.uint32)
    _lib.orc_mt_ints(C.c_int32(seed), C.c_int(n), out.ctypes.data_as(C.POINTER(C.c_uint32)))
    return out


def mcica_subcol(side, atm, cloud, icld: int = 2, irng: int = 1, permuteseed: int = 1):
    """McICA's stochastic sub-columns (mcica_subcol_lw / mcica_subcol_sw): the
    cloud fields of ``cloud`` (cldfr, cicewp, cliqwp (nlay, ncol); LW taucld
    (nlay, ncol, 16); SW taucld, ssacld, asmcld, fsfcld (nlay, ncol, 14))
    drawn onto one binary cloud mask per g-point (140 LW, 112 SW) and layer,
    with overlap ``icld`` (1 random, 2 maximum/random, 3 maximum) from the
    reference's generator ``irng`` (0 kissvec, 1 Mersenne Twister) and
    ``permuteseed``.  Returns dict of (nlay, ncol, ng) arrays: cldfr, cicewp,
    cliqwp and the band optics of the cloudy sub-columns."""
    from mima_gb300 import tables
    n, L = atm.ncol, atm.nlay
    blob = tables.read_blob(tables.ensure_blob())
    ngb = np.asarray(blob[f"{side}.ngb"][0], dtype=np.int64)
    band = (ngb - ngb[0]).astype(np.int32)
    nsub, nband = band.size, (16 if side == "lw" else 14)
    names = ["taucld"] if side == "lw" else ["taucld", "ssacld", "asmcld", "fsfcld"]
    clear = np.array([0.0] if side == "lw" else [0.0, 1.0, 0.0, 0.0])
    fields = np.ascontiguousarray(np.stack([np.broadcast_to(cloud[k], (L, n, nband)) for k in names]),
                                  dtype=np.float64)
    out = {k: np.zeros((L, n, nsub)) for k in ("cldfr", "cicewp", "cliqwp")}
    fo = np.zeros((len(names), L, n, nsub))
    rc = _lib.orc_mcica_subcol(C.c_int(n), C.c_int(L), C.c_int(nsub), C.c_int(icld), C.c_int(irng),
                               C.c_int(permuteseed), _p(_f(atm.play)), _p(_f(cloud["cldfr"])),
                               _p(_f(cloud["cicewp"])), _p(_f(cloud["cliqwp"])), C.c_int(nband),
                               band.ctypes.data_as(C.POINTER(C.c_int)), C.c_int(len(names)), _p(fields),
                               _p(clear), _p(out["cldfr"]), _p(out["cicewp"]), _p(out["cliqwp"]), _p(fo))
    if rc != 0:
        raise RuntimeError(f"orc_mcica_subcol failed ({rc})")
    out.update({k: fo[j] for j, k in enumerate(names)})
    return out


def rrtmg_lw_mcica(atm, sub, idrv: int = 0, tauaer=None, nthreads: int = 0, inflag: int = 0, iceflag: int = 0,
                   liqflag: int = 0, reice=None, reliq=None):
    """McICA rrtmg_lw (rrtmg_lw_rad.f90) on ``atm`` with the sub-column clouds
    ``sub`` (as mcica_subcol("lw", ...) returns: cldfr, taucld, cicewp,
    cliqwp (nlay, ncol, 140)), cldprmc's ``inflag`` (0 depths given, 2 the
    parameterisations with ``reice`` / ``reliq`` (nlay, ncol)) and rtrnmc.
    Returns the dict of rrtmg_lw."""
    n, L = atm.ncol, atm.nlay
    out = {k: np.zeros((L + 1, n)) for k in ("uflx", "dflx", "uflxc", "dflxc", "duflx_dt", "duflxc_dt")}
    out.update({k: np.zeros((L, n)) for k in ("hr", "hrc")})
    args = [_f(atm.play), _f(atm.plev), _f(atm.tlay), _f(atm.tlev), _f(atm.tsfc), _f(atm.h2o),
            _f(atm.o3), _f(atm.co2), _f(atm.ch4), _f(atm.n2o), _f(atm.o2), _f(atm.cfc11),
            _f(atm.cfc12), _f(atm.cfc22), _f(atm.ccl4), _f(atm.emis)]
    cl = [_f(sub[k]) for k in ("cldfr", "taucld", "cicewp", "cliqwp")]
    rad = [None if a is None else _f(a) for a in (reice, reliq)]
    rc = _lib.orc_rrtmg_lw_mcica(C.c_int(n), C.c_int(L), C.c_int(1), C.c_int(idrv), *[_p(a) for a in args],
                                 C.c_int(inflag), C.c_int(iceflag), C.c_int(liqflag), *[_p(a) for a in cl],
                                 *[_p(a) for a in rad], _p(None if tauaer is None else _f(tauaer)),
                                 _p(out["uflx"]), _p(out["dflx"]), _p(out["hr"]), _p(out["uflxc"]),
                                 _p(out["dflxc"]), _p(out["hrc"]), _p(out["duflx_dt"]), _p(out["duflxc_dt"]),
                                 C.c_int(nthreads))
    if rc == 5:
        raise CloudRangeError("cldprmc stops (inflag 1, or a size outside its table)")
    if rc != 0:
        raise RuntimeError(f"orc_rrtmg_lw_mcica failed ({rc})")
    return out


def rrtmg_sw_mcica(atm, sub, iaer: int = 0, tauaer=None, ssaaer=None, asmaer=None, nthreads: int = 0,
                   inflag: int = 0, iceflag: int = 0, liqflag: int = 0, reice=None, reliq=None):
    """McICA rrtmg_sw (rrtmg_sw_rad.f90) on ``atm`` with the sub-column clouds
    ``sub`` (as mcica_subcol("sw", ...) returns: cldfr, taucld, ssacld,
    asmcld, fsfcld, cicewp, cliqwp (nlay, ncol, 112)), cldprmc_sw's ``inflag``
    (0 optics given, 2 the parameterisations with ``reice`` / ``reliq``
    (nlay, ncol)) and spcvmc_sw.  Every column is computed, dark ones with
    cos(zenith) clamped to 1e-10 as the McICA driver does.  Returns the dict
    of rrtmg_sw."""
    n, L = atm.ncol, atm.nlay
    out = {k: np.zeros((L + 1, n)) for k in ("swuflx", "swdflx", "swuflxc", "swdflxc")}
    out.update({k: np.zeros((L, n)) for k in ("swhr", "swhrc")})
    args = [_f(atm.play), _f(atm.plev), _f(atm.tlay), _f(atm.tlev), _f(atm.tsfc), _f(atm.h2o),
            _f(atm.o3), _f(atm.co2), _f(atm.ch4), _f(atm.n2o), _f(atm.o2), _f(atm.asdir),
            _f(atm.asdif), _f(atm.aldir), _f(atm.aldif), _f(atm.coszen)]
    cl = [None if sub.get(k) is None else _f(sub[k])
          for k in ("cldfr", "taucld", "ssacld", "asmcld", "fsfcld", "cicewp", "cliqwp")]
    rad = [None if a is None else _f(a) for a in (reice, reliq)]
    aer = [None if a is None else _f(a) for a in (tauaer, ssaaer, asmaer)]
    rc = _lib.orc_rrtmg_sw_mcica(C.c_int(n), C.c_int(L), C.c_int(1), C.c_int(iaer), *[_p(a) for a in args],
                                 C.c_double(atm.adjes), C.c_int(atm.dyofyr), C.c_double(atm.scon),
                                 C.c_int(inflag), C.c_int(iceflag), C.c_int(liqflag), *[_p(a) for a in cl],
                                 *[_p(a) for a in rad], *[_p(a) for a in aer],
                                 _p(out["swuflx"]), _p(out["swdflx"]), _p(out["swhr"]), _p(out["swuflxc"]),
                                 _p(out["swdflxc"]), _p(out["swhrc"]), C.c_int(nthreads))
    if rc == 5:
        raise CloudRangeError("cldprmc_sw stops (inflag 1, or a size outside its table)")
    if rc != 0:
        raise RuntimeError(f"orc_rrtmg_sw_mcica failed ({rc})")
    return out


def mt_jump_ints(seed: int, jump: int, n: int):
    """The n Mersenne Twister draws after the first ``jump`` ones, by the
    F2-linear jump-ahead (no draw of the first ``jump`` is made); and the
    degree of the characteristic polynomial found."""
    out = np.zeros(n, dtype=np.uint32)
    _lib.orc_mt_jump_ints.restype = C.c_int
    deg = _lib.orc_mt_jump_ints(C.c_int32(seed), C.c_uint64(jump), C.c_int(n),
                                out.ctypes.data_as(C.POINTER(C.c_uint32)))
    return out, deg


def mt_subcol_starts(seed: int, stride: int, nsub: int, n: int):
    """The first n draws of nsub Mersenne Twister streams starting ``stride``
    words apart, the starts reached by one jump polynomial applied in a chain:
    (nsub, n) uint32."""
    out = np.zeros((nsub, n), dtype=np.uint32)
    _lib.orc_mt_subcol_starts(C.c_int32(seed), C.c_uint64(stride), C.c_int(nsub), C.c_int(n),
                              out.ctypes.data_as(C.POINTER(C.c_uint32)))
    return out
