"""Cloud optical properties from water paths and effective sizes, restated in
numpy for the tests (a second statement beside the oracle's C++ one):

* ``lw_taucloud``: cldprop, inflag = 2 (rrtmg_lw_cldprop.f90:185-270), per
  layer the 16 cloud-band optical depths of a layer whose optics are formed,
  for parameterisations that give all 16 bands (ice iceflag 2 / 3, or iceflag
  1 together with liquid liqflag 1, and liqflag 1);
* ``sw_cloud``: cldprop_sw, inflag = 2 (rrtmg_sw_cldprop.f90:158-340), per
  layer the 14 bands' delta-scaled optical depth, single-scattering albedo
  and asymmetry.

Both read the reference's tables from the table blob (``lwcld.*``,
``swcld.*``).  Sizes outside a parameterisation's range are the caller's to
avoid.
"""
import numpy as np

from mima_gb300 import tables

# icb (rrtmg_lw_cldprop.f90:120-122): cloud band -> coefficient band of the
# 5-band ice parameterisation (iceflag 1)
ICB5 = np.array([1, 2, 3, 3, 3, 4, 4, 4, 5, 5, 5, 5, 5, 5, 5, 5])


def _tab(blob):
    return {k: a for k, (a, lb) in tables.read_blob(blob).items()}


def _interp(tab, factor, index):
    """table(index) + fint * (table(index + 1) - table(index)), 1-based rows."""
    fint = factor - index
    lo, hi = tab[index - 1], tab[index]
    return lo + fint[:, None] * (hi - lo)


def lw_taucloud(blob, ciwp, clwp, reice, reliq, iceflag):
    """(n, 16) optical depths of n layers with liquid liqflag = 1."""
    T = _tab(blob)
    ciwp, clwp, reice, reliq = (np.asarray(a, dtype=np.float64).ravel() for a in (ciwp, clwp, reice, reliq))
    n = ciwp.size
    if iceflag == 1:
        ice = T["lwcld.absice1"][0][None, :] + T["lwcld.absice1"][1][None, :] / reice[:, None]
        ice = ice[:, ICB5 - 1]
    else:
        factor = (reice - 2.0) / 3.0
        index = factor.astype(np.int64)
        index[index == (43 if iceflag == 2 else 46)] -= 1
        ice = _interp(T["lwcld.absice2" if iceflag == 2 else "lwcld.absice3"], factor, index)
    ice = np.where(ciwp[:, None] == 0.0, 0.0, ice)
    index = (reliq - 1.5).astype(np.int64)
    index[index == 0] = 1
    index[index == 58] = 57
    liq = _interp(T["lwcld.absliq1"], reliq - 1.5, index)
    liq = np.where(clwp[:, None] == 0.0, 0.0, liq)
    return ciwp[:, None] * ice + clwp[:, None] * liq


def sw_cloud(blob, ciwp, clwp, reice, reliq, iceflag):
    """(tau, ssa, asm), each (n, 14), of n layers with liquid liqflag = 1."""
    T = _tab(blob)
    ciwp, clwp, reice, reliq = (np.asarray(a, dtype=np.float64).ravel() for a in (ciwp, clwp, reice, reliq))
    if iceflag == 1:
        wn = T["sw.wavenum2"]
        icx = np.select([wn > 1.43e4, wn > 7.7e3, wn > 5.3e3, wn > 4.0e3], [1, 2, 3, 4], 5) - 1
        ext = T["swcld.abari"][icx][None, :] + T["swcld.bbari"][icx][None, :] / reice[:, None]
        ssa = 1.0 - T["swcld.cbari"][icx][None, :] - T["swcld.dbari"][icx][None, :] * reice[:, None]
        g = T["swcld.ebari"][icx][None, :] + T["swcld.fbari"][icx][None, :] * reice[:, None]
        g = np.where(g >= 1.0, 1.0 - 1e-6, g)
        fw = g * g
    else:
        sfx = "2" if iceflag == 2 else "3"
        factor = (reice - 2.0) / 3.0
        index = factor.astype(np.int64)
        index[index == (43 if iceflag == 2 else 46)] -= 1
        ext = _interp(T["swcld.extice" + sfx], factor, index)
        ssa = _interp(T["swcld.ssaice" + sfx], factor, index)
        g = _interp(T["swcld.asyice" + sfx], factor, index)
        if iceflag == 2:
            fw = g * g
        else:
            fw = np.minimum(_interp(T["swcld.fdlice3"], factor, index) + 0.5 / ssa, g)
    none = ciwp[:, None] == 0.0
    ext, ssa, g, fw = (np.where(none, 0.0, a) for a in (ext, ssa, g, fw))
    index = (reliq - 1.5).astype(np.int64)
    index[index == 0] = 1
    index[index == 58] = 57
    fint = reliq - 1.5 - index
    extl = _interp(T["swcld.extliq1"], reliq - 1.5, index)
    ssal = _interp(T["swcld.ssaliq1"], reliq - 1.5, index)
    ssal = np.where((fint[:, None] < 0.0) & (ssal > 1.0), T["swcld.ssaliq1"][index - 1], ssal)
    gl = _interp(T["swcld.asyliq1"], reliq - 1.5, index)
    fl = gl * gl
    noliq = clwp[:, None] == 0.0
    extl, ssal, gl, fl = (np.where(noliq, 0.0, a) for a in (extl, ssal, gl, fl))
    tauliq0, tauice0 = clwp[:, None] * extl, ciwp[:, None] * ext
    ssaliq = ssal * (1.0 - fl) / (1.0 - fl * ssal)
    tauliq = (1.0 - fl * ssal) * tauliq0
    ssaice = ssa * (1.0 - fw) / (1.0 - fw * ssa)
    tauice = (1.0 - fw * ssa) * tauice0
    scatliq = ssaliq * tauliq
    scatice = ssaice * tauice
    tau = tauliq + tauice
    tau = np.where(tau == 0.0, 1e-20, tau)
    scatice = np.where(scatice == 0.0, 1e-20, scatice)
    ssac = (scatliq + scatice) / tau
    asm = (scatliq * (gl - fl) / (1.0 - fl) + scatice * (g - fw) / (1.0 - fw)) / (scatliq + scatice)
    return tau, ssac, asm
