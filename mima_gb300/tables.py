"""Coefficient tables for the RRTMG clear-sky LW/SW column-radiation path.

The reference model keeps its absorption-coefficient tables as Fortran data
statements (``name(section) = (/ values /)``) compiled into the model:

* SW: ``rrtmg_sw/gcm_model/src/rrtmg_sw_k_g.f90`` (``sw_kgb16..29``), the
  reference atmosphere ``swatmref`` (``rrtmg_sw_setcoef.f90:289-343``), the
  g-point maps ``swcmbdat`` and band data ``swdatinit``
  (``rrtmg_sw_init.f90:157-367``).
* LW: Planck tables ``lwavplank``/``lwavplankderiv``
  (``rrtmg_lw_setcoef.f90:581-1990``), reference atmosphere ``lwatmref``
  (``rrtmg_lw_setcoef.f90:418-578``), g-point maps ``lwcmbdat`` and band data
  ``lwdatinit`` (``rrtmg_lw_init.f90:178-363``).

The LW absorption coefficients (``rrtmg_lw_k_g.f90`` / ``rrtmg_lw.nc``) are not
part of the MiMA distribution, so this module generates *synthetic* LW
k-distributions: seeded, log-spread, increasing with g, with exactly the shapes
the ``rrlw_kgNN`` modules declare, so they pass through the same 256 -> 140
g-point reduction as real data would.  Every LW result built on them is a
synthetic-k-distribution result.  Where a ``rrtmg_lw_k_g.f90`` is at hand (the
AER RRTMG_LW distribution's data file), ``build_blob(..., lw_kg=path)`` (or
``--lw-kg`` on the command line) parses the real LW k-distribution from it
instead, with the parser of the SW data; ``lw_nc=`` / ``--lw-nc`` reads it from
the netCDF form ``rrtmg_lw.nc`` the way the reference's
``rrtmg_lw_read_nc.f90`` does.  The kernels then compute the reference's
physical LW fluxes.

Nothing here is used at run time by the kernels: the output is one binary
"table blob" (format below) that the C-ABI's ``rrtmg_gpu_init`` reads, reduces
(``cmbgb*``) and uploads.  The blob holds the *unreduced* 16-g tables so that the
reduction itself is part of the checked path.

Blob format (little endian)::

    char[8]  magic "RRTMGTB1"
    u32      version (1), u32 count
    count x  entry {char name[48]; u32 dtype (0=f64,1=i32); u32 ndim;
                    i32 lbound[4]; u32 dims[4]; u64 offset; u64 nbytes}
    data     arrays in Fortran (first-index-fastest) order, 64-byte aligned
    u64      checksum of everything before it (see ``blob_checksum``)
"""
from __future__ import annotations

import os
import re
import struct
from pathlib import Path

import numpy as np

MAGIC = b"RRTMGTB1"
VERSION = 1
NAME_LEN = 48

# Location of the RRTMG sources inside a MiMA checkout.
RRTM_SUBDIR = Path("src/atmos_param/rrtm_radiation")

DEFAULT_BLOB = Path(__file__).resolve().parent / "data" / "rrtmg_tables.bin"
DEFAULT_LW_SEED = 20240601


# --------------------------------------------------------------------------
# Fortran source scanning
# --------------------------------------------------------------------------

def _statements(path: Path):
    """Yield (routine, statement) pairs with comments and continuations removed."""
    routine = None
    buf = ""
    with open(path, "r", errors="replace") as fh:
        for raw in fh:
            line = raw.split("!", 1)[0].rstrip()
            if not line.strip():
                continue
            s = line.strip()
            if s.startswith("&"):
                s = s[1:]
            if s.endswith("&"):
                buf += s[:-1] + " "
                continue
            stmt = (buf + s).strip()
            buf = ""
            m = re.match(r"(?i)^(end\s+)?subroutine\s+(\w+)", stmt)
            if m:
                routine = None if m.group(1) else m.group(2).lower()
                continue
            yield routine, stmt


def _int_params(paths):
    """Integer named constants (``integer, parameter :: a = 1, b = 2``)."""
    params = {}
    for p in paths:
        for _, st in _statements(p):
            if re.match(r"(?i)^\s*integer.*parameter", st):
                rhs = st.split("::", 1)[1]
                for part in rhs.split(","):
                    if "=" in part:
                        k, v = part.split("=", 1)
                        try:
                            params[k.strip().lower()] = int(v.strip())
                        except ValueError:
                            pass
    return params


def _split_top(s: str):
    """Split on commas that are not inside parentheses."""
    out, depth, cur = [], 0, ""
    for ch in s:
        if ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        if ch == "," and depth == 0:
            out.append(cur)
            cur = ""
        else:
            cur += ch
    if cur.strip():
        out.append(cur)
    return out


def _dim(spec: str, params):
    spec = spec.strip().lower()
    if ":" in spec:
        lo, hi = spec.split(":")
        return _ival(lo, params), _ival(hi, params)
    return 1, _ival(spec, params)


def _ival(s, params):
    s = s.strip().lower()
    if "*" in s:
        a, b = s.split("*", 1)
        return _ival(a, params) * _ival(b, params)
    return params[s] if s in params else int(s)


def _decls(path: Path, params):
    """Real array declarations -> {name: (lbounds, shape)}; scalars get ()."""
    out = {}
    for _, st in _statements(path):
        m = re.match(r"(?i)^\s*real\s*\(\s*kind\s*=\s*\w+\s*\)\s*(,\s*dimension\s*\(([^)]*)\))?\s*::(.*)$", st)
        if not m:
            continue
        common = m.group(2)
        for item in _split_top(m.group(3)):
            item = item.strip()
            mm = re.match(r"(\w+)\s*(\((.*)\))?$", item)
            if not mm:
                continue
            name = mm.group(1).lower()
            dims = mm.group(3) if mm.group(3) else common
            if dims is None:
                out[name] = ((), ())
            else:
                ds = [_dim(d, params) for d in _split_top(dims)]
                out[name] = (tuple(d[0] for d in ds), tuple(d[1] - d[0] + 1 for d in ds))
    return out


_NUM = re.compile(r"_(rb|im|r8|kind_rb)$", re.I)


def _num(tok: str):
    tok = tok.strip()
    if "*" in tok:
        n, v = tok.split("*", 1)
        return [_num(v)[0]] * int(n)
    tok = _NUM.sub("", tok).replace("d", "e").replace("D", "e")
    return [float(tok)]


def _values(rhs: str):
    rhs = rhs.strip()
    if rhs.startswith("(/"):
        body = rhs[2:rhs.rindex("/)")]
        vals = []
        for tok in body.split(","):
            if tok.strip():
                vals.extend(_num(tok))
        return vals
    return _num(rhs)


def _assign(arrays, decl, name, section, vals):
    lb, shape = decl
    arr = arrays.setdefault(name, np.full(shape if shape else (), np.nan, dtype=np.float64))
    if not shape:
        assert len(vals) == 1, name
        arrays[name] = np.float64(vals[0])
        return
    if section is None:
        idx = tuple(slice(None) for _ in shape)
    else:
        parts = _split_top(section)
        assert len(parts) == len(shape), (name, section)
        idx = []
        for p, lo, n in zip(parts, lb, shape):
            p = p.strip()
            if p == ":":
                idx.append(slice(None))
            elif ":" in p:
                a, b = (int(x) for x in p.split(":"))
                idx.append(slice(a - lo, b - lo + 1))
            else:
                idx.append(int(p) - lo)
        idx = tuple(idx)
    target = arr[idx]
    tshape = np.shape(target)
    v = np.asarray(vals, dtype=np.float64)
    assert v.size == int(np.prod(tshape)), (name, section, v.size, tshape)
    arr[idx] = v.reshape(tshape, order="F")


def _data_from(path: Path, decls, routines=None, by_routine=False):
    """Collect ``name(section) = values`` data assignments from ``path``."""
    result = {}
    for routine, st in _statements(path):
        if routines is not None and routine not in routines:
            continue
        m = re.match(r"^(\w+)\s*(\(([^=]*)\))?\s*=\s*(.+)$", st)
        if not m:
            continue
        name = m.group(1).lower()
        if name not in decls:
            continue
        key = routine if by_routine else None
        arrays = result.setdefault(key, {})
        _assign(arrays, decls[name], name, m.group(3), _values(m.group(4)))
    return result if by_routine else result.get(None, {})


def _sw_kg_data(path: Path, decls_by_band):
    """One pass over ``rrtmg_sw_k_g.f90``; routine ``sw_kgbNN`` fills band NN."""
    return _kg_data(path, "sw_kgb", decls_by_band)


def _kg_data(path: Path, prefix: str, decls_by_band):
    """One pass over a k-distribution data file (``rrtmg_sw_k_g.f90``,
    ``rrtmg_lw_k_g.f90``): the data assignments of routine ``<prefix>NN`` fill
    band NN's arrays declared in ``decls_by_band[NN]``."""
    result = {b: {} for b in decls_by_band}
    for routine, st in _statements(path):
        if not routine or not routine.startswith(prefix):
            continue
        try:
            b = int(routine[len(prefix):])
        except ValueError:
            continue
        if b not in decls_by_band:
            continue
        m = re.match(r"^(\w+)\s*(\(([^=]*)\))?\s*=\s*(.+)$", st)
        if not m:
            continue
        name = m.group(1).lower()
        if name not in decls_by_band[b]:
            continue
        _assign(result[b], decls_by_band[b][name], name, m.group(3), _values(m.group(4)))
    return result


def _int_data_from(path: Path, routine: str, names):
    """Integer / real 1-D ``name(:) = (/ ... /)`` lists inside ``routine``."""
    out = {}
    for r, st in _statements(path):
        if r != routine:
            continue
        m = re.match(r"^(\w+)\s*(\(:\))?\s*=\s*(\(/.+/\))$", st)
        if m and m.group(1).lower() in names:
            out[m.group(1).lower()] = np.asarray(_values(m.group(3)))
    return out


# --------------------------------------------------------------------------
# Reference (SW, LW support) tables
# --------------------------------------------------------------------------

def _paths(root: Path):
    rr = Path(root) / RRTM_SUBDIR
    return {
        "lw_src": rr / "rrtmg_lw/gcm_model/src",
        "lw_mod": rr / "rrtmg_lw/gcm_model/modules",
        "sw_src": rr / "rrtmg_sw/gcm_model/src",
        "sw_mod": rr / "rrtmg_sw/gcm_model/modules",
    }


def _as_struct(name, v):
    v = np.asarray(v)
    if name in ("wt", "wavenum1", "wavenum2", "delwave"):
        return v.astype(np.float64)
    assert np.all(v == np.round(v)), name
    return v.astype(np.int32)


STRUCT_NAMES = ("ngc", "ngs", "ngm", "ngn", "ngb", "wt", "wavenum1", "wavenum2",
                "delwave", "ng", "nspa", "nspb")


def reference_tables(root) -> dict:
    """Parse every reference table the path needs; returns {blob_name: array}."""
    P = _paths(root)
    out = {}

    # ---- SW absorption data, per band (rrtmg_sw_k_g.f90 sw_kgbNN) ----------
    sw_params = _int_params([P["sw_mod"] / "parrrsw.f90"] +
                            sorted(P["sw_mod"].glob("rrsw_kg*.f90")))
    sw_decls = {}
    for b in range(16, 30):
        sw_decls[b] = _decls(P["sw_mod"] / f"rrsw_kg{b}.f90", sw_params)
    per_routine = _sw_kg_data(P["sw_src"] / "rrtmg_sw_k_g.f90", sw_decls)
    for b, arrays in per_routine.items():
        for name, arr in arrays.items():
            a = np.asarray(arr, dtype=np.float64)
            if np.isnan(a).any():
                raise ValueError(f"SW band {b} table {name} incompletely assigned")
            out[f"sw{b}.{name}"] = (a, sw_decls[b][name][0])

    # ---- SW reference atmosphere (swatmref) --------------------------------
    ref_decl = _decls(P["sw_mod"] / "rrsw_ref.f90", sw_params)
    atm = _data_from(P["sw_src"] / "rrtmg_sw_setcoef.f90", ref_decl, routines={"swatmref"})
    for k in ("pref", "preflog", "tref"):
        out[f"sw.{k}"] = (atm[k], (1,))

    # ---- SW band structure (swdatinit, swcmbdat) ---------------------------
    sinit = P["sw_src"] / "rrtmg_sw_init.f90"
    st = _int_data_from(sinit, "swcmbdat", STRUCT_NAMES)
    st.update(_int_data_from(sinit, "swdatinit", STRUCT_NAMES))
    for k, v in st.items():
        out[f"sw.{k}"] = (_as_struct(k, v), (1,))

    # ---- LW reference atmosphere and Planck tables -------------------------
    lw_params = _int_params([P["lw_mod"] / "parrrtm.f90"] +
                            sorted(P["lw_mod"].glob("rrlw_kg*.f90")))
    lref = _decls(P["lw_mod"] / "rrlw_ref.f90", lw_params)
    lwvn = _decls(P["lw_mod"] / "rrlw_wvn.f90", lw_params)
    lsc = P["lw_src"] / "rrtmg_lw_setcoef.f90"
    atm = _data_from(lsc, lref, routines={"lwatmref"})
    for k in ("pref", "preflog", "tref", "chi_mls"):
        out[f"lw.{k}"] = (atm[k], (1,) * atm[k].ndim)
    planck = _data_from(lsc, lwvn, routines={"lwavplank", "lwavplankderiv"})
    for k in ("totplnk", "totplk16", "totplnkderiv", "totplk16deriv"):
        a = planck[k]
        if np.isnan(a).any():
            raise ValueError(f"LW Planck table {k} incompletely assigned")
        out[f"lw.{k}"] = (a, (1,) * a.ndim)

    linit = P["lw_src"] / "rrtmg_lw_init.f90"
    st = _int_data_from(linit, "lwcmbdat", STRUCT_NAMES)
    st.update(_int_data_from(linit, "lwdatinit", STRUCT_NAMES))
    for k, v in st.items():
        out[f"lw.{k}"] = (_as_struct(k, v), (1,))

    # ---- cloud optical properties (lwcldpr, swcldpr): cldprop / cldprop_sw ---
    for src, mod, routine, prefix, prm in ((linit, P["lw_mod"] / "rrlw_cld.f90", "lwcldpr", "lwcld", lw_params),
                                          (sinit, P["sw_mod"] / "rrsw_cld.f90", "swcldpr", "swcld", sw_params)):
        decl = _decls(mod, prm)
        data = _data_from(src, decl, routines={routine})
        for k, (lb, _shape) in decl.items():
            a = np.asarray(data.get(k, np.nan), dtype=np.float64)
            if np.isnan(a).any():
                raise ValueError(f"cloud table {k} incompletely assigned")
            out[f"{prefix}.{k}"] = (np.atleast_1d(a), lb if lb else (1,))

    # ---- LW table shapes (for the synthetic generator) ----------------------
    shapes = {}
    for b in range(1, 17):
        d = _decls(P["lw_mod"] / f"rrlw_kg{b:02d}.f90", lw_params)
        shapes[b] = {k: v for k, v in d.items() if _is_original_lw_table(k)}
    return out, shapes


_LW_ORIGINAL = ("fracrefao", "fracrefbo", "selfrefo", "forrefo",
                "ccl4o", "cfc11adjo", "cfc12o", "cfc22adjo")


def _is_original_lw_table(name: str) -> bool:
    """16-g (unreduced) LW table names as declared in ``rrlw_kgNN``."""
    return name in _LW_ORIGINAL or name.startswith("kao") or name.startswith("kbo")


# --------------------------------------------------------------------------
# Synthetic LW k-distribution
# --------------------------------------------------------------------------

# log10 range (lowest g, highest g) of the key-species coefficients per band,
# lower / upper atmosphere.  Chosen so that per-layer optical depths span about
# 1e-6 .. 1e3 and the band strengths follow the broad shape of the real LW
# spectrum (strong H2O rotation and CO2 15 um bands, weak window bands).
_LW_STRENGTH = {
    1: ((-3.0, 2.0), (-3.0, 1.5)),   2: ((-3.5, 1.5), (-3.5, 1.0)),
    3: ((-3.0, 2.5), (-2.5, 2.5)),   4: ((-2.0, 3.0), (-1.5, 3.0)),
    5: ((-3.0, 2.0), (-2.0, 2.0)),   6: ((-4.5, -0.5), (-4.5, -0.5)),
    7: ((-4.0, 1.0), (-2.0, 2.0)),   8: ((-4.5, 0.0), (-3.0, 1.5)),
    9: ((-3.5, 1.5), (-3.0, 1.0)),  10: ((-3.0, 2.0), (-3.0, 1.5)),
    11: ((-3.0, 2.0), (-3.0, 1.5)), 12: ((-4.0, 0.5), (-4.0, 0.5)),
    13: ((-4.0, 0.5), (-4.0, 0.5)), 14: ((-2.0, 3.0), (-2.0, 3.0)),
    15: ((-4.0, 0.5), (-4.0, 0.5)), 16: ((-4.0, 0.5), (-3.5, 0.5)),
}


def synthetic_lw_tables(shapes: dict, seed: int = DEFAULT_LW_SEED) -> dict:
    """Seeded synthetic 16-g LW tables with the declared ``rrlw_kgNN`` shapes."""
    rng = np.random.default_rng(seed)
    out = {}
    g = np.arange(16) / 15.0
    for b in range(1, 17):
        (alo, ahi), (blo, bhi) = _LW_STRENGTH[b]
        for name in sorted(shapes[b]):
            lb, shape = shapes[b][name]
            if name.startswith("fracref"):
                # (16,) or (16, J): positive Planck fractions summing to 1 over g.
                J = shape[1] if len(shape) > 1 else 1
                base = np.exp(-2.2 * g) + 0.02
                fr = base[:, None] * (1.0 + 0.3 * rng.uniform(-1, 1, size=(16, J)))
                fr *= (1.0 + 0.15 * np.sin(np.linspace(0, np.pi, J)))[None, :] * np.linspace(1.0, 0.8, 16)[:, None] ** np.arange(J)[None, :] ** 0.3
                fr /= fr.sum(axis=0, keepdims=True)
                a = fr.reshape(shape)
            elif name in ("kao", "kbo"):
                lo, hi = (alo, ahi) if name == "kao" else (blo, bhi)
                a = _log_table(rng, shape, lo, hi)
            elif "_m" in name:
                lo, hi = (-6.5, -2.5) if name.startswith("ka") else (-7.0, -3.0)
                a = _log_table(rng, shape, lo, hi)
            elif name == "selfrefo":
                a = _log_table(rng, shape, -3.0, -0.5, tslope=-0.06)
            elif name == "forrefo":
                a = _log_table(rng, shape, -4.0, -1.5, tslope=0.02)
            else:
                # CFC / CCl4 cross sections (cm2 * 1e20 per molecule).
                a = _log_table(rng, shape, 1.0, 2.5)
            out[f"lw{b:02d}.{name}"] = (np.ascontiguousarray(a, dtype=np.float64), lb)
    return out


def lw_kg_tables(path, shapes: dict) -> dict:
    """The real LW k-distribution from a ``rrtmg_lw_k_g.f90`` (the reference's
    data statements, routines ``lw_kgb01..16``; rrtmg_lw_init.f90 calls them
    before the g-point reduction) for every 16-g table ``shapes`` declares
    (the ``rrlw_kgNN`` modules): {blob_name: (array, lbounds)}, the form of
    :func:`synthetic_lw_tables`.  A table that the file leaves unassigned or
    only partly assigned is an error."""
    per_band = _kg_data(Path(path), "lw_kgb", shapes)
    out = {}
    for b in range(1, 17):
        for name, (lb, shape) in sorted(shapes[b].items()):
            a = per_band[b].get(name)
            if a is None:
                raise ValueError(f"{path}: LW band {b} table {name} is not assigned")
            a = np.asarray(a, dtype=np.float64)
            if a.shape != tuple(shape) or np.isnan(a).any():
                raise ValueError(f"{path}: LW band {b} table {name} incompletely assigned")
            out[f"lw{b:02d}.{name}"] = (np.ascontiguousarray(a), lb)
    return out


def lw_nc_reads(reader_src, params) -> list:
    """The reads that the reference's netCDF reader of the LW data
    (``rrtmg_lw_read_nc.f90``, routines ``lw_kgb01..16``) performs, in order:
    [(band, target table, target section or None, netCDF variable, Fortran
    start, Fortran count)], the
    start and count vectors evaluated from the routine's parameters
    (bandNumber, numGPoints, gPointSetNumber), ``rrlw_ncpar``'s dimension
    constants and the absorber index ``getAbsorberIndex`` set (1-based position
    in ``AbsorberNames``).  ``params``: integer constants of parrrtm /
    rrlw_ncpar; the absorber names are read from ``rrlw_ncpar.f90``'s
    directory."""
    src = Path(reader_src)
    names_src = (src.parent.parent / "modules" / "rrlw_ncpar.f90").read_text()
    m = re.search(r"AbsorberNames\s*=\s*\(/(.*?)/\)", names_src.replace("&", " "), re.S)
    absorbers = [a.strip().upper() for a in re.findall(r"'([^']*)'", m.group(1))]
    reads, local, var = [], {}, None
    for routine, st in _statements(src):
        if not routine or not routine.startswith("lw_kgb"):
            local, var = {}, None
            continue
        band = int(routine[6:])
        pm = re.match(r"(?i)^integer.*parameter\s*::(.*)$", st)
        if pm:
            for part in _split_top(pm.group(1)):
                k, v = part.split("=", 1)
                v = v.strip().lower()
                local[k.strip().lower()] = int(v) if v.lstrip("-").isdigit() else params[v]
            continue
        am = re.match(r"(?i)^call\s+getabsorberindex\s*\(\s*'(\w+)'\s*,\s*(\w+)\s*\)", st)
        if am:
            local[am.group(2).lower()] = absorbers.index(am.group(1).upper()) + 1
            continue
        vm = re.search(r'(?i)nf90_inq_varid\s*\(\s*ncid\s*,\s*"(\w+)"', st)
        if vm:
            var = vm.group(1)
            continue
        gm = re.search(r"(?i)nf90_get_var\s*\(\s*ncid\s*,\s*varid\s*,\s*(\w+)\s*(\(([^)]*)\))?\s*,"
                       r"\s*start\s*=\s*\(/(.*?)/\)\s*,\s*count\s*=\s*\(/(.*?)/\)\s*\)", st)
        if gm:
            ev = lambda t: int(t) if t.strip().isdigit() else {**params, **local}[t.strip().lower()]
            start = [ev(t) for t in gm.group(4).split(",")]
            count = [ev(t) for t in gm.group(5).split(",")]
            reads.append((band, gm.group(1).lower(), gm.group(3), var, start, count))
    return reads


def lw_nc_tables(nc_path, reader_src, params, shapes: dict) -> dict:
    """The real LW k-distribution from the netCDF form of the data
    (``rrtmg_lw.nc``), read as the reference's reader reads it
    (:func:`lw_nc_reads`): every hyperslab in Fortran element order into its
    16-g table.  netCDF-3 files only (scipy); a table that ``shapes`` declares
    but no read fills is an error."""
    from scipy.io import netcdf_file
    with open(nc_path, "rb") as fh:
        magic = fh.read(4)
    if magic.startswith(b"\x89HDF"):
        raise ValueError(f"{nc_path}: a netCDF-4 (HDF5) file; convert it to netCDF-3 (nccopy -k classic)")
    out = {}
    filled = {}
    with netcdf_file(str(nc_path), "r", mmap=False) as f:
        for band, name, section, var, start, count in lw_nc_reads(reader_src, params):
            if name not in shapes.get(band, {}):
                continue
            if var not in f.variables:
                raise ValueError(f"{nc_path}: no variable {var}")
            a = np.asarray(f.variables[var].data, dtype=np.float64).transpose()  # Fortran axis order
            if a.ndim != len(start) or any(s < 1 or s - 1 + c > n for s, c, n in zip(start, count, a.shape)):
                raise ValueError(f"{nc_path}: {var} {a.shape} does not hold the hyperslab {start} + {count}")
            hs = a[tuple(slice(s - 1, s - 1 + c) for s, c in zip(start, count))]
            # nf90_get_var fills the target (or its section) in Fortran element order
            try:
                _assign(filled.setdefault(band, {}), shapes[band][name], name, section,
                        list(hs.flatten(order="F")))
            except AssertionError:
                raise ValueError(f"{nc_path}: {var} for LW band {band} table {name}: {hs.size} values do not "
                                 f"fill {section or 'the table'}") from None
    out = {}
    for b in range(1, 17):
        for name, (lb, shape) in sorted(shapes[b].items()):
            arr = filled.get(b, {}).get(name)
            if arr is None or np.isnan(arr).any():
                raise ValueError(f"{nc_path}: LW band {b} table {name} is not read in full from the file")
            out[f"lw{b:02d}.{name}"] = (np.ascontiguousarray(arr), lb)
    return out


def _log_table(rng, shape, lo, hi, tslope=0.0):
    """log10-spread table increasing along the trailing g axis.

    Leading axes get smooth variation (so interpolation in eta, T, p is
    meaningful) and 3% seeded noise.
    """
    shape = tuple(shape)
    gaxis = np.linspace(lo, hi, shape[-1])
    lead = shape[:-1]
    smooth = np.zeros(lead)
    for ax, n in enumerate(lead):
        x = np.linspace(-1.0, 1.0, n)
        bshape = [1] * len(lead)
        bshape[ax] = n
        amp = [0.25, 0.1, 0.3, 0.1][ax % 4]
        smooth = smooth + amp * np.sin(1.3 * x + 0.4 * ax).reshape(bshape)
        if ax == 0 and tslope:
            smooth = smooth + (tslope * np.arange(n)).reshape(bshape)
    logk = smooth[..., None] + gaxis + 0.03 * rng.standard_normal(shape)
    return 10.0 ** logk


# --------------------------------------------------------------------------
# Blob I/O
# --------------------------------------------------------------------------

def blob_checksum(data: bytes) -> int:
    """Position-weighted sum of the little-endian u64 words of ``data``.

    ``sum_i w_i * (2 i + 1) mod 2**64`` over the zero-padded words, XOR the byte
    length.  The C readers compute the same definition.
    """
    n = len(data)
    pad = (-n) % 8
    w = np.frombuffer(data + b"\0" * pad, dtype="<u8")
    k = np.arange(w.size, dtype=np.uint64) * np.uint64(2) + np.uint64(1)
    with np.errstate(over="ignore"):
        s = int(np.sum(w * k, dtype=np.uint64))
    return (s ^ n) & 0xFFFFFFFFFFFFFFFF


def write_blob(path, tables: dict) -> None:
    """Write ``{name: (array, lbounds)}`` to the blob format described above."""
    path = Path(path)
    path.parent.mkdir(parents=True, exist_ok=True)
    names = sorted(tables)
    header_size = 8 + 8 + len(names) * (NAME_LEN + 4 + 4 + 16 + 16 + 8 + 8)
    off = (header_size + 63) // 64 * 64
    entries, blobs = [], []
    for n in names:
        arr, lb = tables[n]
        arr = np.asarray(arr)
        if arr.dtype.kind in "iu":
            dtype, raw = 1, np.asarray(arr, dtype="<i4").flatten(order="F").tobytes()
        else:
            dtype, raw = 0, np.asarray(arr, dtype="<f8").flatten(order="F").tobytes()
        dims = list(arr.shape) + [1] * (4 - arr.ndim)
        lbs = list(lb) + [1] * (4 - len(lb))
        entries.append((n, dtype, arr.ndim, lbs, dims, off, len(raw)))
        blobs.append((off, raw))
        off = (off + len(raw) + 63) // 64 * 64
    buf = bytearray(off)
    struct.pack_into("<8sII", buf, 0, MAGIC, VERSION, len(names))
    p = 16
    for (n, dtype, ndim, lbs, dims, o, nb) in entries:
        nm = n.encode()
        assert len(nm) < NAME_LEN, n
        struct.pack_into(f"<{NAME_LEN}sII4i4IQQ", buf, p, nm, dtype, ndim, *lbs, *dims, o, nb)
        p += NAME_LEN + 8 + 16 + 16 + 16
    for o, raw in blobs:
        buf[o:o + len(raw)] = raw
    csum = blob_checksum(bytes(buf))
    with open(path, "wb") as fh:
        fh.write(buf)
        fh.write(struct.pack("<Q", csum))


def read_blob(path) -> dict:
    """Read a blob back into ``{name: (array (Fortran order), lbounds)}``."""
    data = Path(path).read_bytes()
    magic, ver, count = struct.unpack_from("<8sII", data, 0)
    if magic != MAGIC or ver != VERSION:
        raise ValueError(f"{path}: not an RRTMG table blob")
    out = {}
    p = 16
    for _ in range(count):
        f = struct.unpack_from(f"<{NAME_LEN}sII4i4IQQ", data, p)
        p += NAME_LEN + 8 + 16 + 16 + 16
        name = f[0].split(b"\0", 1)[0].decode()
        dtype, ndim = f[1], f[2]
        lbs, dims, off, nb = f[3:3 + ndim], f[7:7 + ndim], f[11], f[12]
        dt = "<i4" if dtype == 1 else "<f8"
        arr = np.frombuffer(data, dtype=dt, count=nb // np.dtype(dt).itemsize, offset=off)
        out[name] = (arr.reshape(dims, order="F"), tuple(lbs))
    return out


def lw_nc_params(reference_root) -> dict:
    """Integer constants the netCDF reader's start / count vectors use
    (parrrtm, rrlw_ncpar, rrlw_kgNN)."""
    P = _paths(reference_root)
    return _int_params([P["lw_mod"] / "parrrtm.f90", P["lw_mod"] / "rrlw_ncpar.f90"] +
                       sorted(P["lw_mod"].glob("rrlw_kg*.f90")))


def build_blob(reference_root, out_path=DEFAULT_BLOB, lw_seed: int = DEFAULT_LW_SEED, lw_kg=None,
               lw_nc=None) -> Path:
    """Parse the reference tables and write the blob.  The LW k-distribution
    is the real one of ``lw_kg`` (a ``rrtmg_lw_k_g.f90``) or ``lw_nc`` (a
    netCDF-3 ``rrtmg_lw.nc``, read as ``rrtmg_lw_read_nc.f90`` reads it) when
    given, else the seeded synthetic one (the MiMA tree does not ship the LW
    data)."""
    tables, shapes = reference_tables(reference_root)
    if lw_kg is not None and lw_nc is not None:
        raise ValueError("give the LW data as rrtmg_lw_k_g.f90 or as rrtmg_lw.nc, not both")
    if lw_kg is not None or lw_nc is not None:
        if lw_kg is not None:
            tables.update(lw_kg_tables(lw_kg, shapes))
        else:
            reader = _paths(reference_root)["lw_src"] / "rrtmg_lw_read_nc.f90"
            tables.update(lw_nc_tables(lw_nc, reader, lw_nc_params(reference_root), shapes))
        tables["meta.lw_real_kdist"] = (np.asarray([1], dtype=np.int32), (1,))
    else:
        tables.update(synthetic_lw_tables(shapes, lw_seed))
        tables["meta.lw_synthetic_seed"] = (np.asarray([lw_seed], dtype=np.int32), (1,))
    write_blob(out_path, tables)
    return Path(out_path)


def ensure_blob(reference_root=None, out_path=DEFAULT_BLOB) -> Path:
    """Return the blob path, building it from a MiMA checkout if it is missing."""
    out_path = Path(os.environ.get("RRTMG_TABLE_BLOB", out_path))
    if out_path.exists():
        return out_path
    root = reference_root or os.environ.get("MIMA_ROOT")
    if root is None or not (Path(root) / RRTM_SUBDIR).exists():
        raise FileNotFoundError(
            f"RRTMG table blob {out_path} is missing and no MiMA source tree was given "
            "(set MIMA_ROOT to a MiMA checkout, or RRTMG_TABLE_BLOB to an existing blob)")
    return build_blob(root, out_path)


if __name__ == "__main__":
    import argparse
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("mima_root")
    ap.add_argument("-o", "--out", default=str(DEFAULT_BLOB))
    ap.add_argument("--lw-seed", type=int, default=DEFAULT_LW_SEED)
    ap.add_argument("--lw-kg", default=None,
                    help="rrtmg_lw_k_g.f90 holding the real LW k-distribution (default: synthetic)")
    ap.add_argument("--lw-nc", default=None,
                    help="rrtmg_lw.nc (netCDF-3) holding the real LW k-distribution (default: synthetic)")
    a = ap.parse_args()
    print(build_blob(a.mima_root, a.out, a.lw_seed, a.lw_kg, a.lw_nc))
