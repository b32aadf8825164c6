"""Python mirror of MiMA's ``rrtmg_lw`` / ``rrtmg_sw`` calls over the C-ABI.

The reference calls (``rrtmg_lw_rad.nomcica.f90:80-89``,
``rrtmg_sw_rad.nomcica.f90:78-88``) become methods of :class:`RRTMG` with the
same argument names and meaning; every array is passed straight to
``librrtmg_gpu.so`` (include/rrtmg_gpu.h).  Host numpy arrays go through
``rrtmg_lw_c`` / ``rrtmg_sw_c``; device arrays (anything exposing
``data_ptr()``, e.g. torch CUDA tensors) through ``rrtmg_lw_dev`` /
``rrtmg_sw_dev`` on a given stream.

There is no CPU fallback: constructing :class:`RRTMG` raises if the shared
library is missing or the GPU cannot be initialised.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

from . import tables

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "lib" / "librrtmg_gpu.so"

RRTMG_OK = 0
RRTMG_ERR_ARG = 1
RRTMG_ERR_UNSUPPORTED = 2
RRTMG_ERR_CUDA = 3
RRTMG_ERR_TABLES = 4
RRTMG_ERR_INPUT = 5
RRTMG_ERR_NOMEM = 6
PREC = {"fp64": 0, "split": 1}
STATIC_SCRATCH_BYTES = 64 * 1024 * 1024  # RRTMG_GPU_STATIC_SCRATCH_BYTES
TRANS = {"table": 0, "analytic": 1}

# Every symbol include/rrtmg_gpu.h and include/rrtmg_run.h declare.
EXPORTED = ("rrtmg_gpu_init", "rrtmg_gpu_finalize", "rrtmg_gpu_set_precision", "rrtmg_gpu_error_string",
            "rrtmg_gpu_last_error", "rrtmg_gpu_launch_count", "rrtmg_lw_c", "rrtmg_sw_c", "rrtmg_lw_dev",
            "rrtmg_sw_dev", "rrtmg_gpu_reserve", "rrtmg_gpu_sync_status", "rrtmg_lw_dev_static",
            "rrtmg_gpu_set_transcendentals", "rrtmg_jacobian_dev", "rrtmg_vjp_dev", "rrtmg_gpu_set_profiling",
            "rrtmg_gpu_profile", "rrtmg_step_dev",
            # include/rrtmg_run.h
            "rrtmg_run_params_default", "rrtmg_run_dev", "rrtmg_run_c")
KERNELS = ("lw_prep", "lw_gpoint", "lw_finalize", "sw_prep", "sw_gpoint", "sw_finalize")

_lib = None
_dp = C.POINTER(C.c_double)


class RunParams(C.Structure):
    """``rrtmg_run_params`` (include/rrtmg_run.h): the rrtm_radiation_nml and
    astro_nml values MiMA's run_rrtmg reads (rrtm_radiation.f90:106-198,
    astro.f90:22-31).  Build one with :func:`run_params`."""
    _fields_ = [(n, C.c_int) for n in (
        "lonstep", "do_zm_tracers", "do_zm_rad", "do_fixed_water", "include_secondary_gases", "do_precip_albedo",
        "num_precip", "use_dyofyr", "solday", "dt_rad_avg")] + [(n, C.c_double) for n in (
            "h2o_lower_limit", "temp_lower_limit", "temp_upper_limit", "co2ppmv", "o3_val", "fixed_water",
            "fixed_water_pres", "fixed_water_lat", "ch4_val", "n2o_val", "o2_val", "cfc11_val", "cfc12_val",
            "cfc22_val", "ccl4_val", "precip_albedo", "precip_lat", "slowdown_rad", "obliq", "solr_cnst", "solrad",
            "equinox_day")]


def run_params(**kw) -> RunParams:
    """The reference's namelist defaults (rrtmg_run_params_default), then ``kw``."""
    p = RunParams()
    rc = load_library().rrtmg_run_params_default(C.byref(p))
    if rc != RRTMG_OK:
        raise RRTMGError(rc, "rrtmg_run_params_default")
    for k, v in kw.items():
        if not hasattr(p, k):
            raise AttributeError(f"rrtmg_run_params has no field {k}")
        setattr(p, k, v)
    return p


# run_rrtmg arguments: inputs and outputs in the order of rrtmg_run_dev / rrtmg_run_c.
RUN_IN = ("lat", "lon", "p_full", "p_half", "z_full", "z_half", "t", "q", "o3", "t_surf_rad", "albedo", "rrtm_precip")
RUN_OUT = ("tdt", "coszen", "flux_sw", "flux_lw", "t_half", "tdt_rad", "tdt_sw", "tdt_lw", "olr", "isr")


class RRTMGError(RuntimeError):
    def __init__(self, code: int, detail: str = ""):
        self.code = code
        msg = _lib.rrtmg_gpu_error_string(code).decode() if _lib else f"status {code}"
        super().__init__(f"{msg} ({code}){': ' + detail if detail else ''}")


def load_library(path: Path | str | None = None) -> C.CDLL:
    """Load librrtmg_gpu.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path or os.environ.get("RRTMG_GPU_LIB", LIB_PATH))
    if not p.exists():
        raise RuntimeError(f"{p} not found; build it with `python -m mima_gb300.build` (no CPU fallback exists)")
    lib = C.CDLL(str(p))
    vp = C.c_void_p
    lib.rrtmg_gpu_init.argtypes = [C.c_double, C.c_char_p, C.c_int, C.POINTER(vp)]
    lib.rrtmg_gpu_finalize.argtypes = [vp]
    lib.rrtmg_gpu_set_precision.argtypes = [vp, C.c_int]
    lib.rrtmg_gpu_error_string.argtypes = [C.c_int]
    lib.rrtmg_gpu_error_string.restype = C.c_char_p
    lib.rrtmg_gpu_last_error.argtypes = [vp]
    lib.rrtmg_gpu_last_error.restype = C.c_char_p
    lib.rrtmg_gpu_launch_count.argtypes = [vp]
    lib.rrtmg_gpu_launch_count.restype = C.c_longlong
    lib.rrtmg_gpu_reserve.argtypes = [vp, C.c_int, C.c_int]
    lib.rrtmg_gpu_sync_status.argtypes = [vp, vp]
    lib.rrtmg_run_params_default.argtypes = [C.POINTER(RunParams)]
    _lib = lib
    return lib


def _host(a):
    if a is None:
        return None
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a


def _hp(a):
    return None if a is None else a.ctypes.data_as(_dp)


def _dptr(t, n=None, name="array", device=None):
    """Device pointer of a CUDA float64 tensor, checked first: a tensor of
    another type, layout, device or a smaller size would make the kernels read
    or write outside it.  ``n``: elements the call reads or writes."""
    if t is None:
        return None
    if not (getattr(t, "is_cuda", False) and str(t.dtype) == "torch.float64" and t.is_contiguous()):
        raise ValueError(f"{name} must be a contiguous float64 CUDA tensor")
    if device is not None and t.device.index is not None and t.device.index != device:
        raise ValueError(f"{name} is on cuda:{t.device.index}, the handle on cuda:{device}")
    if n is not None and t.numel() < n:
        raise ValueError(f"{name} has {t.numel()} elements; the call needs {n}")
    return C.cast(C.c_void_p(int(t.data_ptr())), _dp)


_LOOKUP = object()  # the argument's tensor is looked up by name

_PER_LAYER = ("play", "tlay", "h2ovmr", "o3vmr", "co2vmr", "ch4vmr", "n2ovmr", "o2vmr", "cfc11vmr", "cfc12vmr",
              "cfc22vmr", "ccl4vmr", "hr", "hrc", "swhr", "swhrc")
_PER_LEVEL = ("plev", "tlev", "uflx", "dflx", "uflxc", "dflxc", "duflx_dt", "duflxc_dt", "swuflx", "swdflx",
              "swuflxc", "swdflxc")
_PER_COLUMN = ("tsfc", "asdir", "asdif", "aldir", "aldif", "coszen")


def array_sizes(ncol, nlay):
    """Elements of every rrtmg_lw / rrtmg_sw array by argument name, (rows,
    ncol) column-fastest; ``tauaer`` is the SW one (14 bands), ``tauaer_lw``
    the LW one (16 bands)."""
    n = {k: nlay * ncol for k in _PER_LAYER}
    n.update({k: (nlay + 1) * ncol for k in _PER_LEVEL})
    n.update({k: ncol for k in _PER_COLUMN})
    n.update(emis=16 * ncol, tauaer_lw=16 * nlay * ncol, tauaer=14 * nlay * ncol, ssaaer=14 * nlay * ncol,
             asmaer=14 * nlay * ncol)
    # clouds: cldfr, cicewp, cliqwp, reice, reliq (nlay, ncol); LW taucld
    # Fortran (16, ncol, nlay); SW taucld ("taucld_sw"), ssacld, asmcld, fsfcld
    # Fortran (14, ncol, nlay)
    n.update(cldfr=nlay * ncol, cicewp=nlay * ncol, cliqwp=nlay * ncol, taucld=16 * nlay * ncol,
             reice=nlay * ncol, reliq=nlay * ncol)
    n.update({k: 14 * nlay * ncol for k in ("taucld_sw", "ssacld", "asmcld", "fsfcld")})
    return n


def run_array_sizes(si, sj, sk):
    """Elements of every run_rrtmg array by name (the GCM slab's shapes)."""
    P = si * sj
    full, half = P * sk, P * (sk + 1)
    n = dict(lat=P, lon=P, p_full=full, p_half=half, z_full=full, z_half=half, t=full, q=full, o3=full,
             t_surf_rad=P, albedo=P, rrtm_precip=P)
    n.update(tdt=full, coszen=P, flux_sw=P, flux_lw=P, t_half=half, tdt_rad=full, tdt_sw=full, tdt_lw=full,
             olr=P, isr=P)
    return n


def _outputs(given, shapes, ncol):
    """Output arrays (rows, ncol): the caller's where given (checked), else new."""
    out = {}
    for k, rows in shapes.items():
        a = None if given is None else given.get(k)
        if a is None:
            a = np.empty((rows, ncol))
        elif a.dtype != np.float64 or a.shape != (rows, ncol) or not a.flags["C_CONTIGUOUS"]:
            raise ValueError(f"output {k} must be a C-contiguous float64 array of shape {(rows, ncol)}")
        out[k] = a
    return out


class RRTMG:
    """One GPU handle: tables loaded once (rrtmg_lw_ini/rrtmg_sw_ini)."""

    def __init__(self, blob=None, cpdair: float = 1004.64, device: int = 0, precision: str = "fp64"):
        lib = load_library()
        blob = Path(blob) if blob else tables.ensure_blob()
        h = C.c_void_p()
        rc = lib.rrtmg_gpu_init(C.c_double(cpdair), str(blob).encode(), C.c_int(device), C.byref(h))
        if rc != RRTMG_OK:
            raise RRTMGError(rc, f"rrtmg_gpu_init({blob})")
        self._h = h
        self.lib = lib
        self.device = device
        self.set_precision(precision)

    def close(self):
        if getattr(self, "_h", None):
            self.lib.rrtmg_gpu_finalize(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_precision(self, precision: str) -> None:
        rc = self.lib.rrtmg_gpu_set_precision(self._h, PREC[precision])
        self._check(rc)
        self.precision = precision

    def launch_count(self) -> int:
        return int(self.lib.rrtmg_gpu_launch_count(self._h))

    def reserve(self, ncol: int, nlay: int) -> None:
        self._check(self.lib.rrtmg_gpu_reserve(self._h, ncol, nlay))

    def sync_status(self, stream=None) -> int:
        return int(self.lib.rrtmg_gpu_sync_status(self._h, C.c_void_p(stream or 0)))

    def _check(self, rc):
        if rc != RRTMG_OK:
            raise RRTMGError(rc, self.last_error())

    def last_error(self) -> str:
        """The message of the handle's last failed call."""
        return self.lib.rrtmg_gpu_last_error(self._h).decode()

    # ---------------- host-array drop-ins ----------------
    def rrtmg_lw(self, ncol, nlay, icld, idrv, play, plev, tlay, tlev, tsfc, h2ovmr, o3vmr, co2vmr,
                 ch4vmr=None, n2ovmr=None, o2vmr=None, cfc11vmr=None, cfc12vmr=None, cfc22vmr=None,
                 ccl4vmr=None, emis=None, tauaer=None, check=True, out=None, inflglw=0, cldfr=None, taucld=None,
                 cicewp=None, cliqwp=None, iceflglw=0, liqflglw=0, reice=None, reliq=None):
        """rrtmg_lw on host arrays; returns uflx, dflx, hr, uflxc, dflxc, hrc (+ duflx_dt, duflxc_dt).
        ``out`` optionally supplies the output arrays (float64, C-contiguous;
        page-locked arrays let the library overlap copies with kernels).
        Clouds (icld = 1 random overlap, 2 / 3 maximum/random overlap):
        cldfr, cicewp, cliqwp (nlay, ncol), and with inflglw = 0 taucld
        (nlay, ncol, 16) = Fortran (16, ncol, nlay); inflglw = 1 forms the
        depths from the water paths, inflglw = 2 from the ice (iceflglw 0-3)
        and liquid (liqflglw 0-1) parameterisations with the effective sizes
        reice, reliq (nlay, ncol)."""
        L, N = nlay, ncol
        ins = [_host(a) for a in (play, plev, tlay, tlev, tsfc, h2ovmr, o3vmr, co2vmr, ch4vmr, n2ovmr, o2vmr,
                                  cfc11vmr, cfc12vmr, cfc22vmr, ccl4vmr, emis)]
        shapes = {"uflx": L + 1, "dflx": L + 1, "uflxc": L + 1, "dflxc": L + 1, "hr": L, "hrc": L}
        if idrv == 1:
            shapes.update(duflx_dt=L + 1, duflxc_dt=L + 1)
        out = _outputs(out, shapes, N)
        ta = _host(tauaer)
        cl = [_host(a) for a in (cldfr, taucld, cicewp, cliqwp, reice, reliq)]
        rc = self.lib.rrtmg_lw_c(
            self._h, C.c_int(N), C.c_int(L), C.c_int(icld), C.c_int(idrv), *[_hp(a) for a in ins],
            C.c_int(inflglw), C.c_int(iceflglw), C.c_int(liqflglw), *[_hp(a) for a in cl], _hp(ta),
            _hp(out["uflx"]), _hp(out["dflx"]), _hp(out["hr"]), _hp(out["uflxc"]), _hp(out["dflxc"]),
            _hp(out["hrc"]), _hp(out.get("duflx_dt")), _hp(out.get("duflxc_dt")))
        out["status"] = rc
        if check:
            self._check(rc)
        return out

    def rrtmg_sw(self, ncol, nlay, icld, iaer, play, plev, tlay, tlev, tsfc, h2ovmr, o3vmr, co2vmr, ch4vmr,
                 n2ovmr, o2vmr, asdir, asdif, aldir, aldif, coszen, adjes, dyofyr, scon, tauaer=None,
                 ssaaer=None, asmaer=None, check=True, out=None, inflgsw=0, cldfr=None, taucld=None, ssacld=None,
                 asmcld=None, fsfcld=None, cicewp=None, cliqwp=None, iceflgsw=0, liqflgsw=0, reice=None,
                 reliq=None):
        """rrtmg_sw on host arrays; returns swuflx, swdflx, swhr, swuflxc,
        swdflxc, swhrc.  Clouds (icld >= 1; every sunlit layer clear or
        overcast): cldfr, cicewp, cliqwp (nlay, ncol); with inflgsw = 0 taucld,
        ssacld, asmcld, fsfcld (nlay, ncol, 14) = Fortran (14, ncol, nlay);
        inflgsw = 2 forms the optics from the ice (iceflgsw 1-3) and liquid
        (liqflgsw 1) parameterisations with the effective sizes reice, reliq
        (nlay, ncol)."""
        L, N = nlay, ncol
        ins = [_host(a) for a in (play, plev, tlay, tlev, tsfc, h2ovmr, o3vmr, co2vmr, ch4vmr, n2ovmr, o2vmr,
                                  asdir, asdif, aldir, aldif, coszen)]
        aer = [_host(a) for a in (tauaer, ssaaer, asmaer)]
        cl = [_host(a) for a in (cldfr, taucld, ssacld, asmcld, fsfcld, cicewp, cliqwp, reice, reliq)]
        out = _outputs(out, {"swuflx": L + 1, "swdflx": L + 1, "swuflxc": L + 1, "swdflxc": L + 1, "swhr": L,
                             "swhrc": L}, N)
        rc = self.lib.rrtmg_sw_c(
            self._h, C.c_int(N), C.c_int(L), C.c_int(icld), C.c_int(iaer), *[_hp(a) for a in ins],
            C.c_double(adjes), C.c_int(dyofyr), C.c_double(scon), C.c_int(inflgsw), C.c_int(iceflgsw),
            C.c_int(liqflgsw), *[_hp(a) for a in cl], *[_hp(a) for a in aer], None,
            _hp(out["swuflx"]), _hp(out["swdflx"]), _hp(out["swhr"]), _hp(out["swuflxc"]),
            _hp(out["swdflxc"]), _hp(out["swhrc"]))
        out["status"] = rc
        if check:
            self._check(rc)
        return out

    # Convenience: whole Atmosphere objects (mima_gb300.atmosphere)
    def lw(self, atm, idrv=0, tauaer=None, check=True, cloud=None, icld=1):
        """``cloud``: dict(cldfr, taucld[, cicewp, cliqwp]) (given cloud optical
        depths, as rrtmg_lw's arguments), or with ``inflag`` 1 / 2 (and
        ``iceflag``, ``liqflag``, ``reice``, ``reliq``) the cloud physics, with
        overlap ``icld`` (1 random, 2 / 3 maximum/random)."""
        cl = cloud or {}
        return self.rrtmg_lw(atm.ncol, atm.nlay, icld if cloud else 0, idrv, atm.play, atm.plev, atm.tlay, atm.tlev,
                             atm.tsfc, atm.h2o, atm.o3, atm.co2, atm.ch4, atm.n2o, atm.o2, atm.cfc11, atm.cfc12,
                             atm.cfc22, atm.ccl4, atm.emis, tauaer, check=check, cldfr=cl.get("cldfr"),
                             taucld=cl.get("taucld"), cicewp=cl.get("cicewp"), cliqwp=cl.get("cliqwp"),
                             inflglw=int(cl.get("inflag", 0)), iceflglw=int(cl.get("iceflag", 0)),
                             liqflglw=int(cl.get("liqflag", 0)), reice=cl.get("reice"), reliq=cl.get("reliq"))

    def sw(self, atm, iaer=0, tauaer=None, ssaaer=None, asmaer=None, check=True, cloud=None):
        """``cloud``: dict(cldfr, taucld, ssacld, asmcld, fsfcld[, cicewp,
        cliqwp]) for icld = 1 (given cloud optics), as rrtmg_sw's arguments, or
        dict(cldfr, cicewp, cliqwp, reice, reliq, inflag=2, iceflag, liqflag)
        (cloud physics)."""
        cl = cloud or {}
        return self.rrtmg_sw(atm.ncol, atm.nlay, 1 if cloud else 0, iaer, atm.play, atm.plev, atm.tlay, atm.tlev,
                             atm.tsfc, atm.h2o, atm.o3, atm.co2, atm.ch4, atm.n2o, atm.o2, atm.asdir, atm.asdif,
                             atm.aldir, atm.aldif, atm.coszen, atm.adjes, atm.dyofyr, atm.scon,
                             tauaer, ssaaer, asmaer, check=check, inflgsw=int(cl.get("inflag", 0)),
                             iceflgsw=int(cl.get("iceflag", 0)), liqflgsw=int(cl.get("liqflag", 0)),
                             **{k: cl.get(k) for k in ("cldfr", "taucld", "ssacld", "asmcld", "fsfcld", "cicewp",
                                                       "cliqwp", "reice", "reliq")})

    # ---------------- device-array entry points ----------------
    def _ptrs(self, ncol, nlay, *dicts):
        """Checked device pointers: ``p(name)`` of the array of that name in
        ``dicts`` (the first that has it), ``p(name, tensor)`` of a tensor
        passed as its own argument (None stays NULL)."""
        n = array_sizes(ncol, nlay)

        def p(k, t=_LOOKUP):
            if t is _LOOKUP:
                t = next((dct[k] for dct in dicts if dct is not None and dct.get(k) is not None), None)
            return _dptr(t, n[k], k, self.device)
        return p

    def rrtmg_lw_dev(self, stream, ncol, nlay, icld, idrv, d, out, tauaer=None, inflglw=0, iceflglw=0,
                     liqflglw=0):
        """``d``/``out``: dicts of CUDA tensors with the argument names of
        rrtmg_lw (clouds: cldfr, taucld, cicewp, cliqwp, reice, reliq)."""
        g = self._ptrs(ncol, nlay, d)
        o = self._ptrs(ncol, nlay, out)
        rc = self.lib.rrtmg_lw_dev(
            self._h, C.c_void_p(stream or 0), C.c_int(ncol), C.c_int(nlay), C.c_int(icld), C.c_int(idrv),
            g("play"), g("plev"), g("tlay"), g("tlev"), g("tsfc"), g("h2ovmr"), g("o3vmr"), g("co2vmr"),
            g("ch4vmr"), g("n2ovmr"), g("o2vmr"), g("cfc11vmr"), g("cfc12vmr"), g("cfc22vmr"), g("ccl4vmr"),
            g("emis"), C.c_int(inflglw), C.c_int(iceflglw), C.c_int(liqflglw), g("cldfr"), g("taucld"),
            g("cicewp"), g("cliqwp"), g("reice"), g("reliq"), g("tauaer_lw", tauaer), o("uflx"), o("dflx"),
            o("hr"), o("uflxc"), o("dflxc"), o("hrc"), o("duflx_dt"), o("duflxc_dt"))
        self._check(rc)

    def set_profiling(self, on: bool):
        self._check(self.lib.rrtmg_gpu_set_profiling(self._h, int(bool(on))))

    def profile(self) -> dict:
        """Durations (ms) of the six kernels of the last profiled LW and SW call."""
        ms = (C.c_float * 6)()
        self._check(self.lib.rrtmg_gpu_profile(self._h, ms))
        return dict(zip(KERNELS, [float(v) for v in ms]))

    def set_transcendentals(self, mode: str):
        """"table" (the reference's lookup tables, default) or "analytic"."""
        self._check(self.lib.rrtmg_gpu_set_transcendentals(self._h, TRANS[mode]))

    def _adjoint(self, fn, stream, ncol, nlay, d, extra, adjes, dyofyr, scon, iaer=0, tauaer_lw=None,
                 tauaer_sw=None, ssaaer=None, asmaer=None):
        g = self._ptrs(ncol, nlay, d)
        nx, ny = adjoint_shape(nlay)
        # extra: (jac,) of nx * ny * ncol, or (cot, grad) of ny * ncol and nx * ncol
        sizes = [nx * ny * ncol] if len(extra) == 1 else [ny * ncol, nx * ncol]
        names = ["jac"] if len(extra) == 1 else ["cot", "grad"]
        rc = fn(self._h, C.c_void_p(stream or 0), C.c_int(ncol), C.c_int(nlay),
                g("play"), g("plev"), g("tlay"), g("tlev"), g("tsfc"), g("h2ovmr"), g("o3vmr"), g("co2vmr"),
                g("ch4vmr"), g("n2ovmr"), g("o2vmr"), g("cfc11vmr"), g("cfc12vmr"), g("cfc22vmr"), g("ccl4vmr"),
                g("emis"), g("tauaer_lw", tauaer_lw), g("asdir"), g("asdif"), g("aldir"), g("aldif"), g("coszen"),
                C.c_double(adjes), C.c_int(dyofyr), C.c_double(scon), C.c_int(iaer), g("tauaer", tauaer_sw),
                g("ssaaer", ssaaer), g("asmaer", asmaer),
                *[_dptr(t, n, k, self.device) for t, n, k in zip(extra, sizes, names)])
        self._check(rc)

    def jacobian(self, atm):
        """Host convenience: Jacobians (nx, ny, ncol) of ``atm`` (numpy)."""
        import torch
        nx, ny = adjoint_shape(atm.nlay)
        d = atm_device_inputs(atm)
        jac = torch.empty((nx, ny, atm.ncol), dtype=torch.float64, device="cuda")
        s = torch.cuda.current_stream()
        self.jacobian_dev(s.cuda_stream, atm.ncol, atm.nlay, d, jac, atm.adjes, atm.dyofyr, atm.scon)
        s.synchronize()
        return jac.cpu().numpy()

    def vjp(self, atm, cot):
        """Host convenience: cot (ny, ncol) -> grad (nx, ncol)."""
        import torch
        nx, ny = adjoint_shape(atm.nlay)
        d = atm_device_inputs(atm)
        c = torch.from_numpy(np.ascontiguousarray(cot, dtype=np.float64)).cuda()
        grad = torch.empty((nx, atm.ncol), dtype=torch.float64, device="cuda")
        s = torch.cuda.current_stream()
        self.vjp_dev(s.cuda_stream, atm.ncol, atm.nlay, d, c, grad, atm.adjes, atm.dyofyr, atm.scon)
        s.synchronize()
        return grad.cpu().numpy()

    def jacobian_dev(self, stream, ncol, nlay, d, jac, adjes, dyofyr, scon, **kw):
        """Jacobians into ``jac`` (CUDA float64 tensor of shape (nx, ny, ncol),
        nx = 3 nlay + 2 inputs, ny = 2 nlay + 3 rows; see include/rrtmg_gpu.h)."""
        self._adjoint(self.lib.rrtmg_jacobian_dev, stream, ncol, nlay, d, [jac], adjes, dyofyr, scon, **kw)

    def vjp_dev(self, stream, ncol, nlay, d, cot, grad, adjes, dyofyr, scon, **kw):
        """grad (nx, ncol) = cot (ny, ncol) contracted with the Jacobian."""
        self._adjoint(self.lib.rrtmg_vjp_dev, stream, ncol, nlay, d, [cot, grad], adjes, dyofyr, scon, **kw)

    def rrtmg_lw_dev_static(self, stream, ncol, nlay, icld, idrv, d, out, tauaer=None):
        """As :meth:`rrtmg_lw_dev`, through the allocation-free entry point
        (scratch in the library's static device array)."""
        g = self._ptrs(ncol, nlay, d)
        o = self._ptrs(ncol, nlay, out)
        rc = self.lib.rrtmg_lw_dev_static(
            self._h, C.c_void_p(stream or 0), C.c_int(ncol), C.c_int(nlay), C.c_int(icld), C.c_int(idrv),
            g("play"), g("plev"), g("tlay"), g("tlev"), g("tsfc"), g("h2ovmr"), g("o3vmr"), g("co2vmr"),
            g("ch4vmr"), g("n2ovmr"), g("o2vmr"), g("cfc11vmr"), g("cfc12vmr"), g("cfc22vmr"), g("ccl4vmr"),
            g("emis"), C.c_int(0), C.c_int(0), C.c_int(0), None, None, None, None, None, None,
            g("tauaer_lw", tauaer), o("uflx"), o("dflx"), o("hr"), o("uflxc"), o("dflxc"), o("hrc"), o("duflx_dt"),
            o("duflxc_dt"))
        self._check(rc)

    def rrtmg_sw_dev(self, stream, ncol, nlay, icld, iaer, d, out, adjes, dyofyr, scon, cloud=None):
        """``d``/``out``: dicts of CUDA tensors with the argument names of
        rrtmg_sw; ``cloud`` (icld >= 1): dict of CUDA tensors cldfr, taucld,
        ssacld, asmcld, fsfcld[, cicewp, cliqwp] (shapes as rrtmg_sw's), or for
        the cloud physics cldfr, cicewp, cliqwp, reice, reliq with the ints
        inflag = 2, iceflag, liqflag."""
        g = self._ptrs(ncol, nlay, d)
        o = self._ptrs(ncol, nlay, out)
        cl = cloud or {}
        c = [g(k, cl.get(k)) for k in ("cldfr",)] + [g(k + "_sw" if k == "taucld" else k, cl.get(k))
                                                     for k in ("taucld", "ssacld", "asmcld", "fsfcld")]
        c += [g(k, cl.get(k)) for k in ("cicewp", "cliqwp", "reice", "reliq")]
        fl = [C.c_int(int(cl.get(k, 0))) for k in ("inflag", "iceflag", "liqflag")]
        rc = self.lib.rrtmg_sw_dev(
            self._h, C.c_void_p(stream or 0), C.c_int(ncol), C.c_int(nlay), C.c_int(icld), C.c_int(iaer),
            g("play"), g("plev"), g("tlay"), g("tlev"), g("tsfc"), g("h2ovmr"), g("o3vmr"), g("co2vmr"),
            g("ch4vmr"), g("n2ovmr"), g("o2vmr"), g("asdir"), g("asdif"), g("aldir"), g("aldif"),
            g("coszen"), C.c_double(adjes), C.c_int(dyofyr), C.c_double(scon), *fl, *c, g("tauaer"), g("ssaaer"),
            g("asmaer"), None, o("swuflx"), o("swdflx"), o("swhr"), o("swuflxc"), o("swdflxc"), o("swhrc"))
        self._check(rc)


    def rrtmg_step_dev(self, stream, ncol, nlay, d, olw, osw, adjes, dyofyr, scon, idrv=0, iaer=0, tauaer_lw=None):
        """Fused LW + SW step on device arrays (rrtmg_step_dev): ``d`` holds
        the inputs by rrtmg_lw / rrtmg_sw argument name (plus ``tauaer``,
        ``ssaaer``, ``asmaer`` for iaer = 10), ``olw`` / ``osw`` the outputs."""
        g = self._ptrs(ncol, nlay, d)
        o = self._ptrs(ncol, nlay, olw)
        q = self._ptrs(ncol, nlay, osw)
        rc = self.lib.rrtmg_step_dev(
            self._h, C.c_void_p(stream or 0), C.c_int(ncol), C.c_int(nlay), C.c_int(idrv), C.c_int(iaer),
            g("play"), g("plev"), g("tlay"), g("tlev"), g("tsfc"), g("h2ovmr"), g("o3vmr"), g("co2vmr"),
            g("ch4vmr"), g("n2ovmr"), g("o2vmr"), g("cfc11vmr"), g("cfc12vmr"), g("cfc22vmr"), g("ccl4vmr"),
            g("emis"), g("tauaer_lw", tauaer_lw), g("asdir"), g("asdif"), g("aldir"), g("aldif"), g("coszen"),
            C.c_double(adjes), C.c_int(dyofyr), C.c_double(scon), g("tauaer"), g("ssaaer"), g("asmaer"),
            o("uflx"), o("dflx"), o("hr"), o("uflxc"), o("dflxc"), o("hrc"), o("duflx_dt"), o("duflxc_dt"),
            q("swuflx"), q("swdflx"), q("swhr"), q("swuflxc"), q("swdflxc"), q("swhrc"))
        self._check(rc)

    def run_rrtmg(self, prm, slab, seconds, days, days_per_year=365, tdt=None, diagnostics=True, out=None):
        """run_rrtmg on host arrays (rrtmg_run_c).  ``slab`` holds the GCM
        arrays of :data:`RUN_IN` as C-ordered (sk[+1], sj, si) / (sj, si)
        numpy arrays (Fortran (si, sj, sk) order); returns the outputs of
        :data:`RUN_OUT` (tdt = the given tendency plus the radiative one).
        ``out``: optional caller arrays for the outputs (e.g. page-locked ones;
        ``out["tdt"]`` holds the tendency before radiation and is updated)."""
        si, sj, sk = slab.si, slab.sj, slab.sk
        shapes = {"tdt": (sk, sj, si), "coszen": (sj, si), "flux_sw": (sj, si), "flux_lw": (sj, si),
                  "t_half": (sk + 1, sj, si), "tdt_rad": (sk, sj, si), "tdt_sw": (sk, sj, si),
                  "tdt_lw": (sk, sj, si), "olr": (sj, si), "isr": (sj, si)}
        if out is not None:
            for k, a in out.items():
                if a.shape != shapes[k] or a.dtype != np.float64 or not a.flags.c_contiguous:
                    raise ValueError(f"out[{k!r}] must be a C-contiguous float64 array of shape {shapes[k]}")
        else:
            keep = RUN_OUT if diagnostics else ("tdt", "coszen", "flux_sw", "flux_lw")
            out = {k: np.empty(shapes[k]) for k in keep}
            out["tdt"] = np.array(slab.tdt if tdt is None else tdt, dtype=np.float64, order="C", copy=True)
        ins = [_host(getattr(slab, k)) for k in RUN_IN]
        rc = self.lib.rrtmg_run_c(self._h, C.byref(prm), C.c_int(si), C.c_int(sj), C.c_int(sk), C.c_int(seconds),
                                  C.c_int(days), C.c_int(days_per_year), *[_hp(a) for a in ins],
                                  *[_hp(out.get(k)) for k in RUN_OUT])
        self._check(rc)
        return out

    def run_rrtmg_dev(self, stream, prm, si, sj, sk, seconds, days, days_per_year, d, out):
        """run_rrtmg on device arrays (rrtmg_run_dev): ``d`` maps the names
        of :data:`RUN_IN`, ``out`` those of :data:`RUN_OUT` to CUDA tensors
        (missing optional ones are NULL)."""
        n = run_array_sizes(si, sj, sk)
        rc = self.lib.rrtmg_run_dev(self._h, C.c_void_p(stream or 0), C.byref(prm), C.c_int(si), C.c_int(sj),
                                    C.c_int(sk), C.c_int(seconds), C.c_int(days), C.c_int(days_per_year),
                                    *[_dptr(d.get(k), n[k], k, self.device) for k in RUN_IN],
                                    *[_dptr(out.get(k), n[k], k, self.device) for k in RUN_OUT])
        self._check(rc)


def adjoint_shape(nlay):
    """(nx, ny) of the adjoint entry points: inputs tlay, q, tlev, tsfc; rows
    LW heating, OLR, LW surface net, SW heating, SW surface net."""
    return 3 * nlay + 2, 2 * nlay + 3


def output_rows(lw, sw):
    """The adjoint's output rows (ny, ncol) formed from forward outputs."""
    L = lw["hr"].shape[0]
    return np.concatenate([lw["hr"], lw["uflx"][L:L + 1], lw["uflx"][0:1] - lw["dflx"][0:1], sw["swhr"],
                           sw["swdflx"][0:1] - sw["swuflx"][0:1]])


def atm_device_inputs(atm, device="cuda"):
    """Copy an Atmosphere to CUDA tensors keyed by the rrtmg_lw/rrtmg_sw argument names."""
    import torch
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).to(device)
    return {
        "play": t(atm.play), "plev": t(atm.plev), "tlay": t(atm.tlay), "tlev": t(atm.tlev),
        "tsfc": t(atm.tsfc), "h2ovmr": t(atm.h2o), "o3vmr": t(atm.o3), "co2vmr": t(atm.co2),
        "ch4vmr": t(atm.ch4), "n2ovmr": t(atm.n2o), "o2vmr": t(atm.o2), "cfc11vmr": t(atm.cfc11),
        "cfc12vmr": t(atm.cfc12), "cfc22vmr": t(atm.cfc22), "ccl4vmr": t(atm.ccl4), "emis": t(atm.emis),
        "asdir": t(atm.asdir), "asdif": t(atm.asdif), "aldir": t(atm.aldir), "aldif": t(atm.aldif),
        "coszen": t(atm.coszen),
    }


def device_outputs(ncol, nlay, device="cuda", idrv=0):
    import torch
    e = lambda n: torch.empty((n, ncol), dtype=torch.float64, device=device)
    lw = {"uflx": e(nlay + 1), "dflx": e(nlay + 1), "hr": e(nlay), "uflxc": e(nlay + 1), "dflxc": e(nlay + 1),
          "hrc": e(nlay)}
    if idrv == 1:
        lw["duflx_dt"] = e(nlay + 1)
        lw["duflxc_dt"] = e(nlay + 1)
    sw = {"swuflx": e(nlay + 1), "swdflx": e(nlay + 1), "swhr": e(nlay), "swuflxc": e(nlay + 1),
          "swdflxc": e(nlay + 1), "swhrc": e(nlay)}
    return lw, sw
