"""Extracts known answers for the LW path from the reference's own standalone
RRTMG_LW runs (MiMA ``doc_rrtm/runs_std_atm``: ``input_rrtm_*`` /
``output_rrtm_*``) into ``rrtm_lw_std_atm_surface.json``.

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

Usage: python tests/golden/make_rrtm_std_atm.py [MiMA source tree]
"""
from __future__ import annotations

import json
import re
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "rrtm_lw_std_atm_surface.json"

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


def main(root: Path) -> None:
    runs = root / "doc_rrtm" / "runs_std_atm"
    fixture = {"source": "doc_rrtm/runs_std_atm (standalone RRTMG_LW outputs shipped with MiMA)", "runs": {}}
    for p in sorted(runs.glob("output_rrtm_*")):
        name = p.name[len("output_rrtm_"):]
        inp = read_input(runs / ("input_rrtm_" + INPUT_OF.get(name, name)))
        fixture["runs"][name] = {**inp, "surface_up": read_output(p)}
    OUT.write_text(json.dumps(fixture, indent=1) + "\n")
    print(f"wrote {OUT} ({len(fixture['runs'])} runs)")


if __name__ == "__main__":
    main(Path(sys.argv[1]) if len(sys.argv) > 1 else Path("/root/reference"))
