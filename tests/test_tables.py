"""Coefficient tables: Fortran data parsing, blob format, synthetic LW data,
and the g-point reduction restated in numpy against the oracle's C++ one."""
import numpy as np
import pytest

from mima_gb300 import tables


def test_blob_roundtrip_and_checksum(tmp_path):
    t = {"a.x": (np.arange(12.0).reshape(3, 4, order="F"), (1, 13)),
         "a.n": (np.array([1, 2, 3], dtype=np.int32), (1,))}
    p = tmp_path / "b.bin"
    tables.write_blob(p, t)
    back = tables.read_blob(p)
    assert np.array_equal(back["a.x"][0], t["a.x"][0]) and back["a.x"][1] == (1, 13)
    assert back["a.n"][0].dtype == np.int32
    raw = bytearray(p.read_bytes())
    raw[100] ^= 1
    p.write_bytes(bytes(raw))
    data = bytes(raw)
    assert tables.blob_checksum(data[:-8]) != int.from_bytes(data[-8:], "little")


def test_blob_contents(blob):
    d = tables.read_blob(blob)
    # band structure of the 140 / 112 g-point models (parrrtm.f90, parrrsw.f90)
    assert d["lw.ngc"][0].tolist() == [10, 12, 16, 14, 16, 8, 12, 8, 12, 6, 8, 8, 4, 2, 2, 2]
    assert d["sw.ngc"][0].tolist() == [6, 12, 8, 8, 10, 10, 2, 10, 8, 6, 6, 8, 6, 12]
    assert d["lw.ngn"][0].sum() == 256 and d["sw.ngn"][0].sum() == 224
    # SW absorption data fully assigned, declared shapes (rrsw_kgNN)
    assert d["sw17.kao"][0].shape == (9, 5, 13, 16)
    assert d["sw17.kbo"][0].shape == (5, 5, 47, 16) and d["sw17.kbo"][1] == (1, 1, 13, 1)
    assert d["sw24.raylao"][0].shape == (16, 9)
    for k, (a, _) in d.items():
        if a.dtype.kind == "f":
            assert np.all(np.isfinite(a)), k
    assert d["lw.totplnk"][0].shape == (181, 16)
    assert d["lw.chi_mls"][0].shape == (7, 59)


def test_synthetic_lw_planck_fractions_sum_to_one(blob):
    d = tables.read_blob(blob)
    for b in range(1, 17):
        for nm in ("fracrefao", "fracrefbo"):
            k = f"lw{b:02d}.{nm}"
            if k in d:
                s = d[k][0].sum(axis=0)
                assert np.allclose(s, 1.0, atol=1e-12), k
    assert int(d["meta.lw_synthetic_seed"][0][0]) == tables.DEFAULT_LW_SEED


def _np_reduce(orig, gaxis, ngc, ngn, rw, weighted):
    a = np.moveaxis(orig, gaxis, -1)
    out = np.zeros(a.shape[:-1] + (ngc,))
    src = 0
    for igc in range(ngc):
        acc = np.zeros(a.shape[:-1])
        for _ in range(ngn[igc]):
            acc = acc + (a[..., src] * rw[src] if weighted else a[..., src])
            src += 1
        out[..., igc] = acc
    return np.moveaxis(out, -1, gaxis)


def _rwgt(ngc, ngn, ngm, wt):
    rw = np.zeros(len(ngc) * 16)
    igcsm = 0
    for b in range(len(ngc)):
        if ngc[b] < 16:
            wtsm = np.zeros(16)
            ip = 0
            for igc in range(ngc[b]):
                s = 0.0
                for _ in range(ngn[igcsm]):
                    s = s + wt[ip]
                    ip += 1
                wtsm[igc] = s
                igcsm += 1
            for ig in range(16):
                rw[b * 16 + ig] = wt[ig] / wtsm[ngm[b * 16 + ig] - 1]
        else:
            rw[b * 16:(b + 1) * 16] = 1.0
            igcsm += 16
    return rw


@pytest.mark.parametrize("band,name,red", [(3, "kao", "ka"), (5, "fracrefao", "fracrefa"),
                                           (13, "kao_mco", "ka_mco"), (1, "kbo", "kb")])
def test_lw_reduction_numpy_vs_oracle(blob, orc, band, name, red):
    d = tables.read_blob(blob)
    ngc, ngn, ngm = d["lw.ngc"][0], d["lw.ngn"][0], d["lw.ngm"][0]
    rw = _rwgt(ngc, ngn, ngm, d["lw.wt"][0])
    goff = int(ngc[:band - 1].sum())
    orig = d[f"lw{band:02d}.{name}"][0]
    gaxis = 0 if name.startswith("fracref") else orig.ndim - 1
    mine = _np_reduce(orig, gaxis, int(ngc[band - 1]), ngn[goff:], rw[(band - 1) * 16:], not name.startswith("fracref"))
    theirs = orc.table(f"lw{band:02d}", red)
    assert np.array_equal(mine.flatten(order="F"), theirs)


@pytest.mark.parametrize("band,name,red", [(16, "kao", "ka"), (24, "raylao", "rayla"),
                                           (17, "sfluxrefo", "sfluxref"), (29, "absco2o", "absco2")])
def test_sw_reduction_numpy_vs_oracle(blob, orc, band, name, red):
    d = tables.read_blob(blob)
    ngc, ngn, ngm = d["sw.ngc"][0], d["sw.ngn"][0], d["sw.ngm"][0]
    rw = _rwgt(ngc, ngn, ngm, d["sw.wt"][0])
    ib = band - 16
    goff = int(ngc[:ib].sum())
    orig = d[f"sw{band}.{name}"][0]
    plain = name.startswith("sfluxref")
    gaxis = 0 if (plain or name == "raylao") else orig.ndim - 1
    mine = _np_reduce(orig, gaxis, int(ngc[ib]), ngn[goff:], rw[ib * 16:], not plain)
    assert np.array_equal(mine.flatten(order="F"), orc.table(f"sw{band}", red))


def test_kurucz_solar_source_totals(orc):
    """The reduced SW solar source sums to RRTMG's internal solar constant,
    rrsw_scon = 1368.22 W/m2 (parrrsw.f90), at every eta of the mixed bands."""
    total = 0.0
    for b in range(16, 30):
        sf = orc.table(f"sw{b}", "sfluxref")
        ng = [6, 12, 8, 8, 10, 10, 2, 10, 8, 6, 6, 8, 6, 12][b - 16]
        sf = sf.reshape(ng, -1, order="F")
        col = sf[:, 0].sum()
        assert np.allclose(sf.sum(axis=0), col, rtol=2e-3), b
        total += col * (50.15 / 48.37 if b == 27 else 1.0)
    assert abs(total - 1368.22) < 1.5, total


# ---- real LW k-distribution ingestion (rrtmg_lw_k_g.f90) -------------------

def _lw_band_tables(blob):
    """The blob's 16-g LW tables {band: {name: (array, lbounds)}}."""
    import re
    out = {}
    for k, v in tables.read_blob(blob).items():
        m = re.match(r"^lw(\d\d)\.(\w+)$", k)
        if m:
            out.setdefault(int(m.group(1)), {})[m.group(2)] = v
    return out


def _write_lw_kg(path, bands, drop=None):
    """A data file in the layout of the reference's k-distribution files
    (routines lw_kgbNN; ``name(:, j, k) = (/ & ... /)`` column sections, five
    values per continuation line, ``_rb`` kinds), full precision.  ``drop`` =
    (band, name, section index) leaves one section out."""
    lines = []
    for b in sorted(bands):
        lines += [f"      subroutine lw_kgb{b:02d}", f"      use rrlw_kg{b:02d}"]
        for name in sorted(bands[b]):
            a, lb = bands[b][name]
            cols = [((), a)] if a.ndim == 1 else [(ix, a[(slice(None),) + ix]) for ix in np.ndindex(*a.shape[1:])]
            for n, (ix, col) in enumerate(cols):
                if drop == (b, name, n):
                    continue
                sec = ", ".join([":"] + [str(i + lo) for i, lo in zip(ix, lb[1:])])
                lines.append(f"      {name}({sec}) = (/ &")
                vals = [f"{v:.17e}_rb" for v in col]
                for i in range(0, len(vals), 5):
                    lines.append("        & " + ",".join(vals[i:i + 5]) + (" /)" if i + 5 >= len(vals) else ", &"))
        lines.append(f"      end subroutine lw_kgb{b:02d}")
    path.write_text("\n".join(lines) + "\n")


def test_lw_kg_file_round_trip(blob, tmp_path):
    bands = _lw_band_tables(blob)
    assert sorted(bands) == list(range(1, 17))
    shapes = {b: {n: (lb, a.shape) for n, (a, lb) in t.items()} for b, t in bands.items()}
    p = tmp_path / "rrtmg_lw_k_g.f90"
    _write_lw_kg(p, bands)
    got = tables.lw_kg_tables(p, shapes)
    assert len(got) == sum(len(t) for t in bands.values())
    for b, t in bands.items():
        for n, (a, lb) in t.items():
            g, glb = got[f"lw{b:02d}.{n}"]
            assert glb == lb and np.array_equal(g, a), (b, n)


def test_lw_kg_file_incomplete_is_an_error(blob, tmp_path):
    bands = _lw_band_tables(blob)
    shapes = {b: {n: (lb, a.shape) for n, (a, lb) in t.items()} for b, t in bands.items()}
    p = tmp_path / "partial.f90"
    _write_lw_kg(p, bands, drop=(5, "kao", 7))
    with pytest.raises(ValueError, match="band 5 table kao incompletely assigned"):
        tables.lw_kg_tables(p, shapes)
    missing = {b: dict(t) for b, t in bands.items()}
    del missing[9]["selfrefo"]
    _write_lw_kg(p, missing)
    with pytest.raises(ValueError, match="band 9 table selfrefo is not assigned"):
        tables.lw_kg_tables(p, shapes)


def test_blob_from_lw_kg_file(blob, tmp_path):
    """build_blob(lw_kg=...) puts the file's LW tables in the blob in place of
    the synthetic ones; everything else is unchanged."""
    import __graft_entry__ as ge
    root = ge._reference_root()
    if root is None:
        pytest.skip("no MiMA source tree")
    p = tmp_path / "rrtmg_lw_k_g.f90"
    _write_lw_kg(p, _lw_band_tables(blob))
    out = tables.build_blob(root, tmp_path / "real.bin", lw_kg=p)
    a, b = tables.read_blob(blob), tables.read_blob(out)
    assert "meta.lw_real_kdist" in b and "meta.lw_synthetic_seed" not in b
    assert set(a) - {"meta.lw_synthetic_seed"} == set(b) - {"meta.lw_real_kdist"}
    for k in set(a) & set(b):
        assert np.array_equal(a[k][0], b[k][0]) and a[k][1] == b[k][1], k


# ---- the netCDF form (rrtmg_lw.nc, read as rrtmg_lw_read_nc.f90 reads it) --

def _reference_root_or_skip():
    import __graft_entry__ as ge
    root = ge._reference_root()
    if root is None:
        pytest.skip("no MiMA source tree")
    return root


def _nc_reads(root):
    reader = tables._paths(root)["lw_src"] / "rrtmg_lw_read_nc.f90"
    return reader, tables.lw_nc_reads(reader, tables.lw_nc_params(root))


def _section(a, lb, sec):
    if sec is None:
        return a
    idx = []
    for p, lo in zip(sec.split(","), lb):
        p = p.strip()
        if p == ":":
            idx.append(slice(None))
        elif ":" in p:
            x, y = (int(v) for v in p.split(":"))
            idx.append(slice(x - lo, y - lo + 1))
        else:
            idx.append(int(p) - lo)
    return a[tuple(idx)]


def _write_lw_nc(path, bands, reads, skip_var=None):
    """A netCDF-3 file holding ``bands``' tables where the reads find them:
    each variable as large as its reads reach, dimensions in the file's
    (reversed Fortran) order."""
    from scipy.io import netcdf_file
    ext = {}
    for _, _, _, var, start, count in reads:
        e = ext.setdefault(var, [1] * len(start))
        for i, (s0, c) in enumerate(zip(start, count)):
            e[i] = max(e[i], s0 - 1 + c)
    arrays = {v: np.zeros(e) for v, e in ext.items()}
    for b, name, sec, var, start, count in reads:
        a, lb = bands[b][name]
        vals = np.asarray(_section(a, lb, sec)).flatten(order="F")
        arrays[var][tuple(slice(s0 - 1, s0 - 1 + c) for s0, c in zip(start, count))] = vals.reshape(count, order="F")
    with netcdf_file(str(path), "w") as f:
        for v, a in arrays.items():
            if v == skip_var:
                continue
            dims = []
            for i, n in enumerate(reversed(a.shape)):
                dims.append(f"{v}_{i}")
                f.createDimension(dims[-1], n)
            f.createVariable(v, "d", tuple(dims))[:] = a.transpose()


def test_lw_nc_reader_parse_covers_every_table(blob):
    root = _reference_root_or_skip()
    _, reads = _nc_reads(root)
    bands = _lw_band_tables(blob)
    assert len(reads) == 115
    assert {(b, n) for b, n, *_ in reads} == {(b, n) for b, t in bands.items() for n in t}
    for b, name, sec, var, start, count in reads:
        a, lb = bands[b][name]
        assert int(np.prod(count)) == np.asarray(_section(a, lb, sec)).size, (b, name)
        assert start[-2] == b and start[-1] == 1  # band, g-point set 1


def test_lw_nc_round_trip(blob, tmp_path):
    root = _reference_root_or_skip()
    reader, reads = _nc_reads(root)
    bands = _lw_band_tables(blob)
    shapes = {b: {n: (lb, a.shape) for n, (a, lb) in t.items()} for b, t in bands.items()}
    p = tmp_path / "rrtmg_lw.nc"
    _write_lw_nc(p, bands, reads)
    got = tables.lw_nc_tables(p, reader, tables.lw_nc_params(root), shapes)
    for b, t in bands.items():
        for n, (a, lb) in t.items():
            g, glb = got[f"lw{b:02d}.{n}"]
            assert glb == lb and np.array_equal(g, a), (b, n)
    out = tables.build_blob(root, tmp_path / "nc.bin", lw_nc=p)
    x, y = tables.read_blob(blob), tables.read_blob(out)
    assert "meta.lw_real_kdist" in y and set(x) - {"meta.lw_synthetic_seed"} == set(y) - {"meta.lw_real_kdist"}
    for k in set(x) & set(y):
        assert np.array_equal(x[k][0], y[k][0]), k


def test_lw_nc_refuses_what_it_can_not_read(blob, tmp_path):
    root = _reference_root_or_skip()
    reader, reads = _nc_reads(root)
    bands = _lw_band_tables(blob)
    shapes = {b: {n: (lb, a.shape) for n, (a, lb) in t.items()} for b, t in bands.items()}
    p = tmp_path / "partial.nc"
    _write_lw_nc(p, bands, reads, skip_var="H20SelfAbsorptionCoefficients")
    with pytest.raises(ValueError, match="no variable H20SelfAbsorptionCoefficients"):
        tables.lw_nc_tables(p, reader, tables.lw_nc_params(root), shapes)
    h5 = tmp_path / "hdf5.nc"
    h5.write_bytes(b"\x89HDF\r\n\x1a\n" + b"\0" * 64)
    with pytest.raises(ValueError, match="netCDF-4"):
        tables.lw_nc_tables(h5, reader, tables.lw_nc_params(root), shapes)
    with pytest.raises(ValueError, match="not both"):
        tables.build_blob(root, tmp_path / "x.bin", lw_kg=p, lw_nc=p)
