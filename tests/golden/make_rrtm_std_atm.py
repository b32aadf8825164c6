"""Extracts known answers for the LW path from the reference's own standalone
RRTMG_LW runs (MiMA ``doc_rrtm/runs_std_atm``: ``input_rrtm_*`` /
``output_rrtm_*``) into ``rrtm_lw_std_atm.json``.

With surface emissivity 1 (record 1.4 IEMIS = 0 in every run) the upward LW
flux at the surface is, per band, fluxfac * wtdiff * delwave(band) *
plankbnd(band) * (the band's Planck fractions summed over its g-points)
(rrtmg_lw_rtrnmr.f90 rad0 and the band sums; plankbnd from
rrtmg_lw_setcoef.f90): it needs the Planck tables and the band constants, not
the absorption coefficients.  The fixture keeps, for each run, the surface
temperature TBOUND (and DTBOUND of the idrv = 1 run, whose printed upward
fluxes are those at TBOUND + DTBOUND extrapolated with the derivative), and
the level-0 upward flux of every printed spectral block (the 10-3250 cm-1
total and, where printed, the 16 bands).

For the runs that read layer input (record 1.2 IATM = 0) with no aerosols,
clouds or cross-sections, it also keeps the profile (records 2.1-2.1.2: layer
pressure and temperature, level pressure and temperature, the 7 molecular
amounts and the broadening-gas column of every layer) and the printed
full-spectrum fluxes and heating rates by level, for tolerance checks of the LW
path with the real LW k-distribution.

Usage: python tests/golden/make_rrtm_std_atm.py [MiMA source tree]
"""
from __future__ import annotations

import json
import os
import re
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "rrtm_lw_std_atm.json"

# output run name -> input file suffix (the cloudy runs share inputs)
INPUT_OF = {"MLS-cld5-icld2-imca0": "MLS-cld-imca0", "MLS-cld5-icld2-imca1": "MLS-cld-imca1",
            "MLS-cld5-icld2-imca1_bnds": "MLS-cld-imca1"}


def read_input(path: Path) -> dict:
    """TBOUND and IEMIS of record 1.4 (the line after record 1.2, which carries
    the HI= flags) and DTBOUND of record 1.4.1 for idrv = 1 runs."""
    lines = path.read_text().splitlines()
    i = next(k for k, s in enumerate(lines) if "HI=" in s)
    rec = lines[i + 1]
    tbound = float(rec[0:10])
    iemis = rec[11:12].strip()
    out = {"tbound": tbound, "iemis": int(iemis) if iemis else 0}
    if "idrv1" in path.name:
        out["dtbound"] = float(lines[i + 2].split()[0])
    return out


def read_output(path: Path) -> list:
    """[(wavenumber low, high, level-0 upward flux)] of every spectral block."""
    blocks, rng = [], None
    for s in path.read_text().splitlines():
        m = re.search(r"Wavenumbers:\s*([\d.]+)\s*-\s*([\d.]+)\s*cm", s)
        if m:
            rng = (float(m.group(1)), float(m.group(2)))
            continue
        f = s.split()
        if rng is not None and len(f) >= 6 and f[0] == "0":
            blocks.append([rng[0], rng[1], float(f[2])])
            rng = None
    return blocks


def read_flags(path: Path) -> dict:
    """Record 1.2 flags by column (IAER 19-20, IATM 50, IXSECT 70, IOUT 88-90,
    IDRV 92, IMCA 94, ICLD 95)."""
    lines = path.read_text().splitlines()
    rec = next(s for s in lines if "HI=" in s).ljust(95)
    field = lambda a, b: int(rec[a - 1:b].strip() or 0)
    return {"iaer": field(19, 20), "iatm": field(50, 50), "ixsect": field(70, 70), "iout": field(88, 90),
            "idrv": field(92, 92), "imca": field(94, 94), "icld": field(95, 95)}


def read_profile(path: Path) -> dict:
    """Records 2.1-2.1.2 of a layer-input run: IFORM, NLAYRS, NMOL; per layer
    PAVE, TAVE (and for the first layer PZ, TZ of its bottom), PZ, TZ of its
    top, WKL(1..7), WBROADL (fixed columns; the IFORM = 1 widths)."""
    lines = path.read_text().splitlines()
    i = next(k for k, s in enumerate(lines) if "HI=" in s) + 2
    if "idrv1" in path.name:
        i += 1
    rec = lines[i]
    iform, nlay, nmol = int(rec[1:2]), int(rec[2:5]), int(rec[5:10])
    if iform != 1 or nmol != 7:
        raise ValueError(f"{path}: IFORM {iform}, NMOL {nmol} not handled")
    prof = {"pave": [], "tave": [], "pz": [], "tz": [], "wkl": [], "wbroadl": []}
    k = i + 1
    for lay in range(nlay):
        a = lines[k].ljust(90)
        prof["pave"].append(float(a[0:15]))
        prof["tave"].append(float(a[15:25]))
        if lay == 0:
            prof["pz"].append(float(a[48:56]))
            prof["tz"].append(float(a[56:63]))
        prof["pz"].append(float(a[70:78]))
        prof["tz"].append(float(a[78:85]))
        b = lines[k + 1].ljust(120)
        v = [float(b[15 * j:15 * j + 15]) for j in range(8)]
        prof["wkl"].append(v[:7])
        prof["wbroadl"].append(v[7])
        k += 2
    return prof


def read_levels(path: Path) -> dict:
    """The first (10-3250 cm-1) block by level, surface first: pressure (hPa),
    upward, downward flux (W/m2), and the heating rate (K/day) printed on the
    level's row, htr(lev): the layer between this level and the next one up
    (0 on the top level)."""
    out = {"p": [], "up": [], "down": [], "hr": []}
    started = False
    for s in path.read_text().splitlines():
        if "Wavenumbers:" in s:
            if started:
                break
            started = True
            continue
        f = s.split()
        if started and len(f) == 6 and f[0].isdigit():
            for key, v in zip(("p", "up", "down", "hr"), (f[1], f[2], f[3], f[5])):
                out[key].append(float(v))
    return {k: v[::-1] for k, v in out.items()}


def main(root: Path) -> None:
    runs = root / "doc_rrtm" / "runs_std_atm"
    fixture = {"source": "doc_rrtm/runs_std_atm (standalone RRTMG_LW outputs shipped with MiMA)", "runs": {}}
    for p in sorted(runs.glob("output_rrtm_*")):
        name = p.name[len("output_rrtm_"):]
        src = runs / ("input_rrtm_" + INPUT_OF.get(name, name))
        inp = read_input(src)
        run = {**inp, "surface_up": read_output(p), "flags": read_flags(src)}
        fl = run["flags"]
        if fl["iatm"] == 0 and fl["iaer"] == 0 and fl["ixsect"] == 0 and fl["icld"] == 0:
            run["profile"] = read_profile(src)
            run["levels"] = read_levels(p)
        fixture["runs"][name] = run
    OUT.write_text(json.dumps(fixture, indent=1) + "\n")
    print(f"wrote {OUT} ({len(fixture['runs'])} runs)")


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("MIMA_ROOT")
    if not root:
        sys.exit("usage: make_rrtm_std_atm.py MIMA_ROOT  (a MiMA checkout; or set MIMA_ROOT)")
    main(Path(root))
