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

FIX = json.loads((Path(__file__).resolve().parent / "golden" / "rrtm_lw_std_atm_surface.json").read_text())
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
