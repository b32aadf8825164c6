// CPU oracle, longwave: data structures.  TEST INFRASTRUCTURE ONLY.
#pragma once
#include <map>
#include <string>
#include <vector>

#include "oracle_tables.hpp"

namespace orc {

extern int g_table_mode;

struct LwTables {
  std::map<std::string, FArr> t[17];  // reduced per-band tables ("ka", "kb", "selfref", ...)
  FArr pref, preflog, tref, chi_mls, totplnk, totplk16, totplnkderiv, totplk16deriv;
  double delwave[17];
  int ngc[17], ngs[17], nspa[17], nspb[17];
  double tau_tbl[10001], exp_tbl[10001], tfn_tbl[10001];
  double bpade, heatfac, fluxfac, oneminus, grav, avogad;
  // cloud optical properties (rrlw_cld: lwcldpr, rrtmg_lw_init.f90:2018-2656)
  FArr absice0, absice1, absice2, absice3, absliq1;
  double abscld1 = 0.0, absliq0 = 0.0;
};
extern LwTables g_lw;

// Arguments of rrtmg_lw (rrtmg_lw_rad.nomcica.f90:80-89), column-major with
// the column index fastest; optional gases may be null (treated as zero).
struct LwInput {
  int ncol, nlay;
  const double *play, *plev, *tlay, *tlev, *tsfc, *h2ovmr, *o3vmr, *co2vmr, *ch4vmr, *n2ovmr,
      *o2vmr, *cfc11vmr, *cfc12vmr, *cfc22vmr, *ccl4vmr, *emis, *tauaer;
  // Clouds (icld = 1, inflglw = 0): cldfr (ncol, nlay), taucld (16, ncol, nlay),
  // cicewp / cliqwp (ncol, nlay) or null.
  int icld = 0;
  const double *cldfr = nullptr, *taucld = nullptr, *cicewp = nullptr, *cliqwp = nullptr;
  // cloud physics (inflag = 1: abscld1 x water path; 2: ice and liquid
  // parameterisations selected by iceflag / liqflag, radii reice / reliq)
  int inflag = 0, iceflag = 0, liqflag = 0;
  const double *reice = nullptr, *reliq = nullptr;
  // McICA (rrtmg_lw_rad.f90): per-g-point sub-column clouds cldfmcl,
  // taucmcl, ciwpmcl, clwpmcl (140, ncol, nlay), sizes reicmcl / relqmcl
  // (ncol, nlay); with mcica set the solver is rtrnmc
  bool mcica = false;
  const double *cldfmcl = nullptr, *taucmcl = nullptr, *ciwpmcl = nullptr, *clwpmcl = nullptr;
  const double *reicmcl = nullptr, *relqmcl = nullptr;
};

struct LwColumn {
  int nlayers = 0, laytrop = 0;
  double tbound = 0, pwvcm = 0;
  std::vector<double> pavel, tavel, pz, tz, coldry, wbrodl;
  std::vector<double> wkl[8], wx[5], taua[17];
  double semiss[17], plankbnd[17], dplankbnd_dt[17];
  std::vector<double> planklay[17], planklev[17];
  std::vector<int> jp, jt, jt1, indself, indfor, indminor;
  std::vector<double> colh2o, colco2, colo3, coln2o, colco, colch4, colo2, colbrd;
  std::vector<double> fac00, fac01, fac10, fac11, selffac, selffrac, forfac, forfrac;
  std::vector<double> minorfrac, scaleminor, scaleminorn2;
  std::vector<double> rat_h2oco2, rat_h2oco2_1, rat_h2oo3, rat_h2oo3_1, rat_h2on2o, rat_h2on2o_1,
      rat_h2och4, rat_h2och4_1, rat_n2oco2, rat_n2oco2_1, rat_o3co2, rat_o3co2_1;
  std::vector<double> taug[141], fracs[141], taut[141];
  std::vector<double> cldfrac, taucloud[17];  // icld >= 1: layer cloud fraction, cldprop's cloud optical depth
  int ncbands = 1;        // cldprop's number of cloud bands (1, 5 or 16), the last value it set
  bool cld_error = false;  // cldprop stopped (an effective radius out of its table's range)
  // McICA: cloud cover and depth of each g-point and layer, [g - 1][layer]
  bool mcica = false;
  std::vector<double> cldfmc, taucmc;

  void resize(int nl) {
    auto r = [&](std::vector<double>& v) { v.assign(nl + 2, 0.0); };
    auto ri = [&](std::vector<int>& v) { v.assign(nl + 2, 0); };
    r(pavel); r(tavel); r(pz); r(tz); r(coldry); r(wbrodl);
    for (auto& v : wkl) r(v);
    for (auto& v : wx) r(v);
    for (auto& v : taua) r(v);
    for (auto& v : planklay) r(v);
    for (auto& v : planklev) r(v);
    ri(jp); ri(jt); ri(jt1); ri(indself); ri(indfor); ri(indminor);
    r(colh2o); r(colco2); r(colo3); r(coln2o); r(colco); r(colch4); r(colo2); r(colbrd);
    r(fac00); r(fac01); r(fac10); r(fac11); r(selffac); r(selffrac); r(forfac); r(forfrac);
    r(minorfrac); r(scaleminor); r(scaleminorn2);
    r(rat_h2oco2); r(rat_h2oco2_1); r(rat_h2oo3); r(rat_h2oo3_1); r(rat_h2on2o); r(rat_h2on2o_1);
    r(rat_h2och4); r(rat_h2och4_1); r(rat_n2oco2); r(rat_n2oco2_1); r(rat_o3co2); r(rat_o3co2_1);
    for (auto& v : taug) r(v);
    for (auto& v : fracs) r(v);
    for (auto& v : taut) r(v);
    r(cldfrac);
    for (auto& v : taucloud) r(v);
    for (int b = 0; b < 17; ++b) semiss[b] = plankbnd[b] = dplankbnd_dt[b] = 0.0;
  }
};

struct LwOut {
  std::vector<double> totu, totd, htr, dtotu_dt;  // levels 0..nlay (htr: layers 0..nlay-1, top 0)
  std::vector<double> totuc, totdc, htrc, dtotuc_dt;  // clear-sky stream (rtrn, icld = 1)
  // Per-band fluxes, filled only when want_bands is set (sized 16 * (nlay + 1)
  // by the caller, band-major): upward, downward, d(upward)/d(tsfc) (idrv = 1).
  bool want_bands = false;
  std::vector<double> bandu, bandd, dbandu_dt;
};

void lw_init(const Blob& blob, double cpdair);
void lw_inatm(const LwInput& in, int iplon, LwColumn& c);
void lw_setcoef(LwColumn& c, int idrv);
void lw_taumol(LwColumn& c);
void lw_rtrnmr(LwColumn& c, int idrv, LwOut& out);
void lw_rtrn(LwColumn& c, int idrv, LwOut& out);
void lw_column(const LwInput& in, int iplon, int idrv, LwColumn& c, LwOut& out);

}  // namespace orc
