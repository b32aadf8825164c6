"""Known answers from the reference's own standalone RRTMG_LW runs
(doc_rrtm/runs_std_atm, extracted by tests/golden/make_rrtm_std_atm.py): the
upward LW flux at the surface of every run, total and per band.

With surface emissivity 1 that flux is, per band, fluxfac * wtdiff *
delwave * plankbnd(tsfc) * (sum of the band's Planck fractions) -- the Planck
tables, their interpolation in setcoef, the band widths and the flux factors
of the reference, with no absorption coefficient involved -- so it pins those
parts of the LW path although the LW k-distribution is not in the MiMA tree.
The idrv = 1 run prints the fluxes at tsfc + DTBOUND extrapolated with the
surface-temperature derivative, which pins the Planck-derivative tables.
Tolerances: the runs print 4 decimals, and the real Planck fractions sum to 1
per band only to about 1e-5.  No GPU."""
import json
from pathlib import Path

import numpy as np
import pytest

from mima_gb300 import atmosphere as A
from mima_gb300 import tables

FIX = json.loads((Path(__file__).resolve().parent / "golden" / "rrtm_lw_std_atm.json").read_text())
RUNS = FIX["runs"]


def column(tbound, nlay=40):
    atm = A.small_atmosphere(1, nlay, seed=3)
    atm.tsfc = np.full(1, float(tbound))
    atm.emis = np.ones_like(atm.emis)
    return atm


@pytest.mark.parametrize("name", sorted(RUNS))
def test_surface_upward_total(orc, name):
    r = RUNS[name]
    idrv = 1 if "dtbound" in r else 0
    out = orc.rrtmg_lw(column(r["tbound"]), idrv=idrv)
    up = out["uflx"][0, 0] + (r["dtbound"] * out["duflx_dt"][0, 0] if idrv else 0.0)
    lo, hi, ref = r["surface_up"][0]
    assert (lo, hi) == (10.0, 3250.0)
    assert abs(up - ref) <= 1e-5 * ref, (name, up, ref)


# Runs printing the 16 band blocks.  The cloudy McICA run's band blocks are
# left out: they add up to 429.02 W/m2 against its own printed total of
# 424.80 (the other runs' blocks add up to their totals), so they are no
# known answer for the band fluxes.
PER_BAND = [n for n in sorted(RUNS) if len(RUNS[n]["surface_up"]) == 17 and "imca1" not in n]


@pytest.mark.parametrize("name", PER_BAND)
def test_surface_upward_per_band(orc, blob, name):
    r = RUNS[name]
    idrv = 1 if "dtbound" in r else 0
    b = orc.rrtmg_lw_bands(column(r["tbound"]), idrv=idrv)
    up = b["uflx"][:, 0, 0] + (r["dtbound"] * b["duflx_dt"][:, 0, 0] if idrv else 0.0)
    ref = np.array([v[2] for v in r["surface_up"][1:]])
    wn = np.array([v[:2] for v in r["surface_up"][1:]])
    t = tables.read_blob(blob)
    np.testing.assert_array_equal(wn[:, 0], t["lw.wavenum1"][0].ravel())
    np.testing.assert_array_equal(wn[:, 1], t["lw.wavenum2"][0].ravel())
    # the bands' own fluxes add up to the total flux of the same call
    full = orc.rrtmg_lw(column(r["tbound"]), idrv=idrv)
    tot = full["uflx"][0, 0] + (r["dtbound"] * full["duflx_dt"][0, 0] if idrv else 0.0)
    assert abs(up.sum() - tot) <= 1e-9 * tot
    # bands 1-15: the reference's printed band blocks
    err = np.abs(up[:15] - ref[:15])
    assert (err <= 6e-5 + 1.5e-5 * ref[:15]).all(), list(zip(up[:15], ref[:15]))
    # band 16: the printed block is a single-band run (istart = 16,
    # rrtmg_lw_setcoef.f90:215-232), whose Planck table totplk16 stops at
    # 3250 cm-1; the full-spectrum call (MiMA's, istart = 1) uses totplnk(:, 16),
    # which reaches to infinity, and the printed total holds that value
    total_ref = r["surface_up"][0][2]
    assert abs(up[15] - (total_ref - ref[:15].sum())) <= 6e-4
    assert abs(up[15] - ref[15]) > 0.05 * ref[15]


def test_band16_single_band_planck(blob):
    """The printed band-16 block of the 294.2 K runs is the istart = 16 Planck
    integral: fluxfac * wtdiff * delwave(16) * totplk16 interpolated at TBOUND
    (plus DTBOUND times totplk16deriv in the idrv = 1 run)."""
    t = tables.read_blob(blob)
    p16 = np.asarray(t["lw.totplk16"][0]).ravel()
    d16 = np.asarray(t["lw.totplk16deriv"][0]).ravel()
    fac = np.pi * 1.0e4 * (3250.0 - 2600.0)  # fluxfac * wtdiff = 2 pi 1e4 * 0.5
    for name in ("MLS-clr", "MLS-clr-idrv1"):
        r = RUNS[name]
        tb = r["tbound"]
        i = int(tb - 159.0)  # setcoef's indbound: 1-based, the table's first entry at 160 K
        f = tb - int(tb)  # tbndfrac; p16[i - 1] is totplk16(indbound)
        v = p16[i - 1] + f * (p16[i] - p16[i - 1])
        if "dtbound" in r:
            v += r["dtbound"] * (d16[i - 1] + f * (d16[i] - d16[i - 1]))
        assert abs(fac * v - r["surface_up"][16][2]) <= 6e-5 + 1.5e-5 * r["surface_up"][16][2], (name, fac * v)


# ---- the standard-atmosphere profiles --------------------------------------
# Runs with layer input (IATM = 0) and no aerosols, clouds or cross-sections:
# the fixture holds their profiles (TAPE5 records 2.1-2.1.2) and the printed
# full-spectrum fluxes by level.

AMDW, AMDO = 1.607793, 0.603428  # dry-air / H2O and dry-air / O3 molecular-weight ratios (inatm)
PROFILES = [n for n in sorted(RUNS) if "profile" in RUNS[n]]


def std_atm_column(r):
    """One column of the library's inputs from a run's profile: layer and
    level pressures and temperatures as given; the molecular amounts as
    mixing ratios relative to dry air (given as such, or column densities over
    the dry-air column WBROADL + the other gases); H2O passed as specific
    humidity and O3 as mass mixing ratio, the quantities MiMA's rrtmg_lw
    arguments carry; emissivity 1.  CO has no argument in MiMA's rrtmg_lw and
    is dropped.  The library then recomputes the dry-air column from the
    pressure levels (hydrostatic, inatm), which differs from the run's by a
    median 0.4-0.9 % and by up to 6 % in single layers."""
    pr = r["profile"]
    L = len(pr["pave"])
    wkl = np.array(pr["wkl"]).T
    wb = np.array(pr["wbroadl"])
    vmr = wkl / (wb + wkl[1:].sum(axis=0)) if (wkl > 1.0).any() else wkl
    atm = A.small_atmosphere(1, L, seed=0)
    col = lambda v: np.ascontiguousarray(np.asarray(v, dtype=np.float64)[:, None])
    atm.play, atm.plev = col(pr["pave"]), col(pr["pz"])
    atm.tlay, atm.tlev = col(pr["tave"]), col(pr["tz"])
    atm.tsfc = np.full(1, float(r["tbound"]))
    atm.h2o = col(vmr[0] / (AMDW + vmr[0]))
    atm.o3 = col(vmr[2] / AMDO)
    atm.co2, atm.n2o, atm.ch4, atm.o2 = col(vmr[1]), col(vmr[3]), col(vmr[5]), col(vmr[6])
    atm.emis = np.ones_like(atm.emis)
    return atm


def test_profiles_present():
    assert PROFILES == ["MLS-clr", "MLS-clr-idrv1", "MLW-clr", "SAW-clr", "TROP-clr"]


@pytest.mark.parametrize("name", PROFILES)
def test_profile_reader_matches_printed_levels(name):
    """The profile reader's level pressures are the levels the run printed
    (to its 4-5 significant digits); layers lie between their levels."""
    r = RUNS[name]
    pr, lv = r["profile"], r["levels"]
    L = len(pr["pave"])
    assert len(pr["pz"]) == len(pr["tz"]) == len(lv["p"]) == len(lv["up"]) == L + 1
    np.testing.assert_allclose(pr["pz"], lv["p"], rtol=5e-4)
    pz, pave = np.array(pr["pz"]), np.array(pr["pave"])
    assert (np.diff(pz) < 0).all() and ((pave < pz[:-1]) & (pave > pz[1:])).all()
    assert pr["tz"][0] == r["tbound"]
    assert lv["hr"][-1] == 0.0 and lv["down"][-1] == 0.0


@pytest.mark.parametrize("name", PROFILES)
def test_std_atm_profiles_through_the_oracle(orc, name):
    """Each standard atmosphere runs through the oracle's LW path (finite
    fluxes), and its surface emission is the run's printed level-0 upward flux."""
    r = RUNS[name]
    idrv = 1 if "dtbound" in r else 0
    out = orc.rrtmg_lw(std_atm_column(r), idrv=idrv)
    for k, v in out.items():
        assert np.isfinite(v).all(), k
    up0 = out["uflx"][0, 0] + (r["dtbound"] * out["duflx_dt"][0, 0] if idrv else 0.0)
    assert abs(up0 - r["levels"]["up"][0]) <= 1e-5 * r["levels"]["up"][0]


@pytest.mark.parametrize("name", PROFILES)
def test_std_atm_fluxes_with_real_lw_data(orc, blob, name):
    """Tolerance check of the LW path with the real LW k-distribution (a blob
    built with ``--lw-kg rrtmg_lw_k_g.f90``): the oracle's fluxes on the
    standard atmospheres against the standalone's printed ones, within 2 W/m2
    at every level, and the heating rates of the layers below 1 hPa within
    0.3 K/day (idrv = 0 runs).  The bounds allow for the dry-air columns, which
    the library recomputes from the pressure levels.  Skipped with the synthetic
    LW k-distribution, whose fluxes are not RRTMG's."""
    if "meta.lw_real_kdist" not in tables.read_blob(blob):
        pytest.skip("the table blob carries the synthetic LW k-distribution")
    r = RUNS[name]
    lv = r["levels"]
    idrv = 1 if "dtbound" in r else 0
    out = orc.rrtmg_lw(std_atm_column(r), idrv=idrv)
    up = out["uflx"][:, 0] + (r["dtbound"] * out["duflx_dt"][:, 0] if idrv else 0.0)
    assert np.abs(up - np.array(lv["up"])).max() <= 2.0
    assert np.abs(out["dflx"][:, 0] - np.array(lv["down"])).max() <= 2.0
    if not idrv:
        below = np.array(lv["p"][:-1]) > 1.0
        assert np.abs(out["hr"][:, 0] - np.array(lv["hr"][:-1]))[below].max() <= 0.3
