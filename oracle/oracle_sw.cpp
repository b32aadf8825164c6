// CPU oracle, shortwave -- TEST INFRASTRUCTURE ONLY (the checker, never the
// product).  FP64 restatement of the reference's RRTMG_SW path (clear sky, and
// clear or overcast layers with given cloud optics: icld = 1, inflgsw = 0 --
// cldprop_sw rrtmg_sw_cldprop.f90:118-156, the clear / cloudy combination of
// spcvrt_sw):
//   inatm_sw    rrtmg_sw_rad.nomcica.f90:761-1101
//   driver      rrtmg_sw_rad.nomcica.f90:78-731 (coszen skip :502-510,
//               albedo bands :566-578, heating :712-726)
//   setcoef_sw  rrtmg_sw_setcoef.f90:30-286
//   taumol_sw   rrtmg_sw_taumol.f90:31-1538 (taumol16..29)
//   spcvrt_sw   rrtmg_sw_spcvrt.f90:12-626 (both the "clear" and the "total"
//               streams, exactly as the reference runs them)
//   reftra_sw   rrtmg_sw_reftra.f90:29-305 (kmodts = 2)
//   vrtqdr_sw   rrtmg_sw_vrtqdr.f90:28-152
// Build with -ffp-contract=off.
#include "oracle_sw.hpp"

// Markers of the FLOP-count build (opcount.hpp): the work between them is the
// reference's second ("total") two-stream pass, which in clear sky repeats the
// clear pass, and is left out of the algorithmic count.  No-ops otherwise.
#ifndef OPC_PAUSE
#define OPC_PAUSE() ((void)0)
#define OPC_RESUME() ((void)0)
#endif

#include <cmath>

namespace orc {

SwTables g_sw;

void sw_init(const Blob& blob, double cpdair) {
  SwTables& T = g_sw;
  const int nbnd = 14;
  std::vector<int> ngc = blob.i("sw.ngc"), ngn = blob.i("sw.ngn"), ngm = blob.i("sw.ngm"),
                   ngs = blob.i("sw.ngs"), nspa = blob.i("sw.nspa"), nspb = blob.i("sw.nspb");
  std::vector<double> rwgt = make_rwgt(nbnd, ngc, ngn, ngm, blob.r("sw.wt"));
  int ngs_prev = 0;
  for (int b = 16; b <= 29; ++b) {
    int ib = b - 15;
    T.ngc[b] = ngc[ib - 1];
    T.ngs[b] = ngs[ib - 1];
    T.nspa[b] = nspa[ib - 1];
    T.nspb[b] = nspb[ib - 1];
    char pre[8];
    std::snprintf(pre, sizeof pre, "sw%02d.", b);
    std::string prefix(pre);
    for (const auto& kv : blob.real) {
      if (kv.first.rfind(prefix, 0) != 0) continue;
      std::string nm = kv.first.substr(prefix.size());
      if (nm.back() != 'o') {  // band scalars (rayl)
        T.t[b][nm] = kv.second;
        continue;
      }
      std::string red = nm.rfind("kao", 0) == 0 ? "ka" : nm.rfind("kbo", 0) == 0 ? "kb" : nm.substr(0, nm.size() - 1);
      bool plain = nm.rfind("sfluxref", 0) == 0;
      bool gfirst = plain || nm.rfind("rayla", 0) == 0;
      int gpos = gfirst ? 0 : kv.second.ndim - 1;
      T.t[b][red] = reduce_g(kv.second, gpos, ngc[ib - 1], &ngn[ngs_prev], &rwgt[(size_t)(ib - 1) * 16], !plain);
    }
    ngs_prev = ngs[ib - 1];
  }
  T.preflog = blob.r("sw.preflog");
  T.tref = blob.r("sw.tref");
  // rrtmg_sw_init.f90:96-104
  const int ntbl = 10000;
  const double pade = 0.278, expeps = 1.e-20;
  T.exp_tbl[0] = 1.0;
  T.exp_tbl[ntbl] = expeps;
  T.bpade = 1.0 / pade;
  for (int itr = 1; itr <= ntbl - 1; ++itr) {
    double tfn = (double)itr / (double)ntbl;
    double tau_tbl = T.bpade * tfn / (1. - tfn);
    T.exp_tbl[itr] = std::exp(-tau_tbl);
    if (T.exp_tbl[itr] <= expeps) T.exp_tbl[itr] = expeps;
  }
  // swdatinit, rrtmg_sw_init.f90:157-241
  T.grav = 9.8066;
  T.avogad = 6.02214199e+23;
  T.heatfac = T.grav * 8.6400e4 / (cpdair * 1.e2);
  T.oneminus = 1.0 - 1.e-06;
  T.pi = 2. * std::asin(1.);
  for (auto [f, name] : {std::pair<FArr*, const char*>{&T.extliq1, "extliq1"}, {&T.ssaliq1, "ssaliq1"},
                         {&T.asyliq1, "asyliq1"}, {&T.extice2, "extice2"}, {&T.ssaice2, "ssaice2"},
                         {&T.asyice2, "asyice2"}, {&T.extice3, "extice3"}, {&T.ssaice3, "ssaice3"},
                         {&T.asyice3, "asyice3"}, {&T.fdlice3, "fdlice3"}, {&T.abari, "abari"},
                         {&T.bbari, "bbari"}, {&T.cbari, "cbari"}, {&T.dbari, "dbari"}, {&T.ebari, "ebari"},
                         {&T.fbari, "fbari"}})
    *f = blob.r(std::string("swcld.") + name);
  T.wavenum2 = blob.r("sw.wavenum2");
}

// exp(-x) through the SW lookup table with the reference's small-x series
// (od_lo = 0.06), used for every transmittance in reftra/spcvrt.
static inline double sw_exp(double ze1) {
  if (ze1 <= 0.06) return 1. - ze1 + 0.5 * ze1 * ze1;
  if (!g_table_mode) return std::exp(-ze1);
  double tblind = ze1 / (g_sw.bpade + ze1);
  int itind = (int)(10000.0 * tblind + 0.5);
  return g_sw.exp_tbl[itind];
}

// ---------------------------------------------------------------------------
void sw_inatm(const SwInput& in, int iplon, SwColumn& c) {
  const double amd = 28.9660, amw = 18.0160, amdw = 1.607793, amdo = 0.603428;
  const int nlay = in.nlay, ncol = in.ncol;
  auto A = [&](const double* p, int l) { return p[(size_t)iplon + (size_t)ncol * (size_t)(l - 1)]; };
  c.nlayers = nlay;
  c.resize(nlay);
  double adjflx = in.adjes;
  if (in.dyofyr > 0) {
    double gamma = 2. * g_sw.pi * (in.dyofyr - 1) / 365.;
    adjflx = 1.000110 + .034221 * std::cos(gamma) + .001289 * std::sin(gamma) +
             .000719 * std::cos(2. * gamma) + .000077 * std::sin(2. * gamma);
  }
  for (int ib = 16; ib <= 29; ++ib) {
    double solvar = in.scon / 1.36822e+03;
    c.adjflux[ib] = adjflx * solvar;
  }
  c.tbound = in.tsfc[iplon];
  c.pz[0] = A(in.plev, 1);
  c.tz[0] = A(in.tlev, 1);
  for (int l = 1; l <= nlay; ++l) {
    c.pavel[l] = A(in.play, l);
    c.tavel[l] = A(in.tlay, l);
    c.pz[l] = A(in.plev, l + 1);
    c.tz[l] = A(in.tlev, l + 1);
    c.pdp[l] = c.pz[l - 1] - c.pz[l];
    double h2o = A(in.h2ovmr, l);
    c.wkl[1][l] = (h2o / (1. - h2o)) * amdw;
    c.wkl[2][l] = A(in.co2vmr, l);
    c.wkl[3][l] = A(in.o3vmr, l) * amdo;
    c.wkl[4][l] = in.n2ovmr ? A(in.n2ovmr, l) : 0.0;
    c.wkl[5][l] = 0.0;
    c.wkl[6][l] = in.ch4vmr ? A(in.ch4vmr, l) : 0.0;
    c.wkl[7][l] = in.o2vmr ? A(in.o2vmr, l) : 0.0;
    double amm = (1. - c.wkl[1][l]) * amd + c.wkl[1][l] * amw;
    c.coldry[l] = (c.pz[l - 1] - c.pz[l]) * 1.e3 * g_sw.avogad / (1.e2 * g_sw.grav * amm * (1. + c.wkl[1][l]));
  }
  for (int l = 1; l <= nlay; ++l)
    for (int imol = 1; imol <= 7; ++imol) c.wkl[imol][l] = c.coldry[l] * c.wkl[imol][l];
  for (int l = 1; l <= nlay; ++l)
    for (int ib = 1; ib <= 14; ++ib) {
      size_t o = (size_t)iplon + (size_t)ncol * ((size_t)(l - 1) + (size_t)nlay * (size_t)(ib - 1));
      bool aer = in.iaer >= 1 && in.tauaer;
      c.taua[ib][l] = aer ? in.tauaer[o] : 0.0;
      c.ssaa[ib][l] = aer ? in.ssaaer[o] : 1.0;
      c.asma[ib][l] = aer ? in.asmaer[o] : 0.0;
    }
}

// ---------------------------------------------------------------------------
void sw_setcoef(SwColumn& c) {
  const SwTables& T = g_sw;
  const double stpfac = 296. / 1013.;
  c.laytrop = 0;
  c.laylow = 0;
  for (int lay = 1; lay <= c.nlayers; ++lay) {
    double plog = std::log(c.pavel[lay]);
    int jp = (int)(36. - 5 * (plog + 0.04));
    if (jp < 1) jp = 1; else if (jp > 58) jp = 58;
    c.jp[lay] = jp;
    int jp1 = jp + 1;
    double fp = 5. * (T.preflog(jp) - plog);
    int jt = (int)(3. + (c.tavel[lay] - T.tref(jp)) / 15.);
    if (jt < 1) jt = 1; else if (jt > 4) jt = 4;
    c.jt[lay] = jt;
    double ft = ((c.tavel[lay] - T.tref(jp)) / 15.) - (double)(jt - 3);
    int jt1 = (int)(3. + (c.tavel[lay] - T.tref(jp1)) / 15.);
    if (jt1 < 1) jt1 = 1; else if (jt1 > 4) jt1 = 4;
    c.jt1[lay] = jt1;
    double ft1 = ((c.tavel[lay] - T.tref(jp1)) / 15.) - (double)(jt1 - 3);
    double water = c.wkl[1][lay] / c.coldry[lay];
    double scalefac = c.pavel[lay] * stpfac / c.tavel[lay];
    auto cols = [&]() {
      c.colh2o[lay] = 1.e-20 * c.wkl[1][lay];
      c.colco2[lay] = 1.e-20 * c.wkl[2][lay];
      c.colo3[lay] = 1.e-20 * c.wkl[3][lay];
      c.coln2o[lay] = 1.e-20 * c.wkl[4][lay];
      c.colch4[lay] = 1.e-20 * c.wkl[6][lay];
      c.colo2[lay] = 1.e-20 * c.wkl[7][lay];
      c.colmol[lay] = 1.e-20 * c.coldry[lay] + c.colh2o[lay];
      if (c.colco2[lay] == 0.) c.colco2[lay] = 1.e-32 * c.coldry[lay];
      if (c.coln2o[lay] == 0.) c.coln2o[lay] = 1.e-32 * c.coldry[lay];
      if (c.colch4[lay] == 0.) c.colch4[lay] = 1.e-32 * c.coldry[lay];
      if (c.colo2[lay] == 0.) c.colo2[lay] = 1.e-32 * c.coldry[lay];
    };
    if (plog > 4.56) {
      c.laytrop = c.laytrop + 1;
      if (plog >= 6.62) c.laylow = c.laylow + 1;
      c.forfac[lay] = scalefac / (1. + water);
      double factor = (332.0 - c.tavel[lay]) / 36.0;
      c.indfor[lay] = std::min(2, std::max(1, (int)factor));
      c.forfrac[lay] = factor - (double)c.indfor[lay];
      c.selffac[lay] = water * c.forfac[lay];
      factor = (c.tavel[lay] - 188.0) / 7.2;
      c.indself[lay] = std::min(9, std::max(1, (int)factor - 7));
      c.selffrac[lay] = factor - (double)(c.indself[lay] + 7);
      cols();
    } else {
      c.forfac[lay] = scalefac / (1. + water);
      double factor = (c.tavel[lay] - 188.0) / 36.0;
      c.indfor[lay] = 3;
      c.forfrac[lay] = factor - 1.0;
      cols();
      c.selffac[lay] = 0.;
      c.selffrac[lay] = 0.;
      c.indself[lay] = 0;
    }
    double compfp = 1. - fp;
    c.fac10[lay] = compfp * ft;
    c.fac00[lay] = compfp * (1. - ft);
    c.fac11[lay] = fp * ft1;
    c.fac01[lay] = fp * (1. - ft1);
  }
  // Explicit pads for the reference's jp(0) / jp(nlay+1) reads (taumol_sw
  // lower loops read jp(lay+1) at lay = laytrop; upper loops read jp(lay-1)).
  c.jp[0] = 0;
  c.jp[c.nlayers + 1] = 0;
}

// ---------------------------------------------------------------------------
// taumol_sw helpers
// ---------------------------------------------------------------------------
struct SwEta {
  double speccomb, fs;
  int js;
};
static inline SwEta sw_eta(double a, double strrat_b, double mult) {
  SwEta e;
  e.speccomb = a + strrat_b;
  double specparm = a / e.speccomb;
  if (specparm >= g_sw.oneminus) specparm = g_sw.oneminus;
  double specmult = mult * (specparm);
  e.js = 1 + (int)specmult;
  e.fs = std::fmod(specmult, 1.);
  return e;
}

// speccomb * (8-term eta/T/p interpolation); stride 9 (lower) or 5 (upper).
static inline double major8(const FArr& abs, const SwColumn& c, int lay, const SwEta& e, int ind0, int ind1,
                            int s, int ig) {
  double fs = e.fs;
  double fac000 = (1. - fs) * c.fac00[lay];
  double fac010 = (1. - fs) * c.fac10[lay];
  double fac100 = fs * c.fac00[lay];
  double fac110 = fs * c.fac10[lay];
  double fac001 = (1. - fs) * c.fac01[lay];
  double fac011 = (1. - fs) * c.fac11[lay];
  double fac101 = fs * c.fac01[lay];
  double fac111 = fs * c.fac11[lay];
  return e.speccomb * (fac000 * abs.flat(ind0, ig) + fac100 * abs.flat(ind0 + 1, ig) +
                       fac010 * abs.flat(ind0 + s, ig) + fac110 * abs.flat(ind0 + s + 1, ig) +
                       fac001 * abs.flat(ind1, ig) + fac101 * abs.flat(ind1 + 1, ig) +
                       fac011 * abs.flat(ind1 + s, ig) + fac111 * abs.flat(ind1 + s + 1, ig));
}
static inline double interp4s(const FArr& k, const SwColumn& c, int lay, int ind0, int ind1, int ig) {
  return c.fac00[lay] * k.flat(ind0, ig) + c.fac10[lay] * k.flat(ind0 + 1, ig) +
         c.fac01[lay] * k.flat(ind1, ig) + c.fac11[lay] * k.flat(ind1 + 1, ig);
}
// selffac*(self interp) + forfac*(for interp)
static inline double selfplusfor(const FArr& selfref, const FArr& forref, const SwColumn& c, int lay, int ig) {
  int inds = c.indself[lay], indf = c.indfor[lay];
  return c.selffac[lay] * (selfref(inds, ig) + c.selffrac[lay] * (selfref(inds + 1, ig) - selfref(inds, ig))) +
         c.forfac[lay] * (forref(indf, ig) + c.forfrac[lay] * (forref(indf + 1, ig) - forref(indf, ig)));
}
static inline double selfonly(const FArr& selfref, const SwColumn& c, int lay, int ig) {
  int inds = c.indself[lay];
  return c.selffac[lay] * (selfref(inds, ig) + c.selffrac[lay] * (selfref(inds + 1, ig) - selfref(inds, ig)));
}
// forref(indf,ig) + forfrac*(forref(indf+1,ig) - forref(indf,ig)); the upper
// loops of taumol17/21 multiply it by colh2o*forfac (rrtmg_sw_taumol.f90:450-454, 858-862).
static inline double forinterp(const FArr& forref, const SwColumn& c, int lay, int ig) {
  int indf = c.indfor[lay];
  return forref(indf, ig) + c.forfrac[lay] * (forref(indf + 1, ig) - forref(indf, ig));
}
static inline double foronly(const FArr& forref, const SwColumn& c, int lay, int ig) {
  int indf = c.indfor[lay];
  return c.forfac[lay] * (forref(indf, ig) + c.forfrac[lay] * (forref(indf + 1, ig) - forref(indf, ig)));
}
static inline int ind_lo(const SwColumn& c, int lay, int nsp, int js, bool one) {
  return ((c.jp[lay] - 1) * 5 + (c.jt[lay] - 1)) * nsp + (one ? 1 : js);
}
static inline int ind_lo1(const SwColumn& c, int lay, int nsp, int js, bool one) {
  return (c.jp[lay] * 5 + (c.jt1[lay] - 1)) * nsp + (one ? 1 : js);
}
static inline int ind_up(const SwColumn& c, int lay, int nsp, int js, bool one) {
  return ((c.jp[lay] - 13) * 5 + (c.jt[lay] - 1)) * nsp + (one ? 1 : js);
}
static inline int ind_up1(const SwColumn& c, int lay, int nsp, int js, bool one) {
  return ((c.jp[lay] - 12) * 5 + (c.jt1[lay] - 1)) * nsp + (one ? 1 : js);
}
static inline double sfl_eta(const FArr& sf, int ig, const SwEta& e) {
  return sf(ig, e.js) + e.fs * (sf(ig, e.js + 1) - sf(ig, e.js));
}

// Lower-loop solar-source layer: laysolfr = laytrop, moved to min(lay+1,
// laytrop) where jp crosses layreffr (e.g. taumol18 :548-552).
static inline int laysolfr_lower(const SwColumn& c, int layreffr, int lay, int cur) {
  if (c.jp[lay] < layreffr && c.jp[lay + 1] >= layreffr) return std::min(lay + 1, c.laytrop);
  return cur;
}

// ---------------------------------------------------------------------------
void sw_taumol(SwColumn& c) {
  const SwTables& T = g_sw;
  const int nl = c.nlayers, lt = c.laytrop;
  auto& taug = c.taug;
  auto& taur = c.taur;
  auto& sfz = c.sfluxzen;
  // ---- band 16 (:245-363)
  {
    auto& t = T.t[16];
    const FArr &absa = t.at("ka"), &absb = t.at("kb"), &selfref = t.at("selfref"), &forref = t.at("forref"),
               &sflux = t.at("sfluxref");
    double rayl = t.at("rayl").v[0];
    double strrat1 = 252.131;
    int layreffr = 18;
    for (int lay = 1; lay <= lt; ++lay) {
      SwEta e = sw_eta(c.colh2o[lay], strrat1 * c.colch4[lay], 8.);
      int ind0 = ind_lo(c, lay, T.nspa[16], e.js, false), ind1 = ind_lo1(c, lay, T.nspa[16], e.js, false);
      double tauray = c.colmol[lay] * rayl;
      for (int ig = 1; ig <= T.ngc[16]; ++ig) {
        taug[ig][lay] = major8(absa, c, lay, e, ind0, ind1, 9, ig) + c.colh2o[lay] * selfplusfor(selfref, forref, c, lay, ig);
        taur[ig][lay] = tauray;
      }
    }
    int laysolfr = nl;
    for (int lay = lt + 1; lay <= nl; ++lay) {
      if (c.jp[lay - 1] < layreffr && c.jp[lay] >= layreffr) laysolfr = lay;
      int ind0 = ind_up(c, lay, T.nspb[16], 1, true), ind1 = ind_up1(c, lay, T.nspb[16], 1, true);
      double tauray = c.colmol[lay] * rayl;
      for (int ig = 1; ig <= T.ngc[16]; ++ig) {
        taug[ig][lay] = c.colch4[lay] * interp4s(absb, c, lay, ind0, ind1, ig);
        if (lay == laysolfr) sfz[ig] = sflux(ig);
        taur[ig][lay] = tauray;
      }
    }
  }
  // ---- band 17 (:366-484)
  {
    auto& t = T.t[17];
    const int o = T.ngs[16];
    const FArr &absa = t.at("ka"), &absb = t.at("kb"), &selfref = t.at("selfref"), &forref = t.at("forref"),
               &sflux = t.at("sfluxref");
    double rayl = t.at("rayl").v[0];
    double strrat = 0.364641;
    int layreffr = 30;
    for (int lay = 1; lay <= lt; ++lay) {
      SwEta e = sw_eta(c.colh2o[lay], strrat * c.colco2[lay], 8.);
      int ind0 = ind_lo(c, lay, T.nspa[17], e.js, false), ind1 = ind_lo1(c, lay, T.nspa[17], e.js, false);
      double tauray = c.colmol[lay] * rayl;
      for (int ig = 1; ig <= T.ngc[17]; ++ig) {
        taug[o + ig][lay] = major8(absa, c, lay, e, ind0, ind1, 9, ig) + c.colh2o[lay] * selfplusfor(selfref, forref, c, lay, ig);
        taur[o + ig][lay] = tauray;
      }
    }
    int laysolfr = nl;
    for (int lay = lt + 1; lay <= nl; ++lay) {
      if (c.jp[lay - 1] < layreffr && c.jp[lay] >= layreffr) laysolfr = lay;
      SwEta e = sw_eta(c.colh2o[lay], strrat * c.colco2[lay], 4.);
      int ind0 = ind_up(c, lay, T.nspb[17], e.js, false), ind1 = ind_up1(c, lay, T.nspb[17], e.js, false);
      double tauray = c.colmol[lay] * rayl;
      for (int ig = 1; ig <= T.ngc[17]; ++ig) {
        taug[o + ig][lay] = major8(absb, c, lay, e, ind0, ind1, 5, ig) + c.colh2o[lay] * c.forfac[lay] * forinterp(forref, c, lay, ig);
        if (lay == laysolfr) sfz[o + ig] = sfl_eta(sflux, ig, e);
        taur[o + ig][lay] = tauray;
      }
    }
  }
  // ---- bands 18, 19, 21 (lower eta-mixed with self/for; solar source in the lower loop)
  auto lower_eta_band = [&](int b, double strrat, int layreffr, const std::vector<double>& colb) {
    auto& t = T.t[b];
    const int o = T.ngs[b - 1];
    const FArr &absa = t.at("ka"), &selfref = t.at("selfref"), &forref = t.at("forref"), &sflux = t.at("sfluxref");
    double rayl = t.at("rayl").v[0];
    int laysolfr = lt;
    for (int lay = 1; lay <= lt; ++lay) {
      laysolfr = laysolfr_lower(c, layreffr, lay, laysolfr);
      SwEta e = sw_eta(c.colh2o[lay], strrat * colb[lay], 8.);
      int ind0 = ind_lo(c, lay, T.nspa[b], e.js, false), ind1 = ind_lo1(c, lay, T.nspa[b], e.js, false);
      double tauray = c.colmol[lay] * rayl;
      for (int ig = 1; ig <= T.ngc[b]; ++ig) {
        taug[o + ig][lay] = major8(absa, c, lay, e, ind0, ind1, 9, ig) + c.colh2o[lay] * selfplusfor(selfref, forref, c, lay, ig);
        if (lay == laysolfr) sfz[o + ig] = sfl_eta(sflux, ig, e);
        taur[o + ig][lay] = tauray;
      }
    }
  };
  // band 18 (:487-600): lower h2o/ch4, upper ch4
  lower_eta_band(18, 38.9589, 6, c.colch4);
  {
    auto& t = T.t[18];
    const int o = T.ngs[17];
    const FArr& absb = t.at("kb");
    double rayl = t.at("rayl").v[0];
    for (int lay = lt + 1; lay <= nl; ++lay) {
      int ind0 = ind_up(c, lay, T.nspb[18], 1, true), ind1 = ind_up1(c, lay, T.nspb[18], 1, true);
      double tauray = c.colmol[lay] * rayl;
      for (int ig = 1; ig <= T.ngc[18]; ++ig) {
        taug[o + ig][lay] = c.colch4[lay] * interp4s(absb, c, lay, ind0, ind1, ig);
        taur[o + ig][lay] = tauray;
      }
    }
  }
  // band 19 (:603-715): lower h2o/co2, upper co2
  lower_eta_band(19, 5.49281, 3, c.colco2);
  {
    auto& t = T.t[19];
    const int o = T.ngs[18];
    const FArr& absb = t.at("kb");
    double rayl = t.at("rayl").v[0];
    for (int lay = lt + 1; lay <= nl; ++lay) {
      int ind0 = ind_up(c, lay, T.nspb[19], 1, true), ind1 = ind_up1(c, lay, T.nspb[19], 1, true);
      double tauray = c.colmol[lay] * rayl;
      for (int ig = 1; ig <= T.ngc[19]; ++ig) {
        taug[o + ig][lay] = c.colco2[lay] * interp4s(absb, c, lay, ind0, ind1, ig);
        taur[o + ig][lay] = tauray;
      }
    }
  }
  // ---- band 20 (:718-818): h2o + ch4
  {
    auto& t = T.t[20];
    const int o = T.ngs[19];
    const FArr &absa = t.at("ka"), &absb = t.at("kb"), &selfref = t.at("selfref"), &forref = t.at("forref"),
               &sflux = t.at("sfluxref"), &absch4 = t.at("absch4");
    double rayl = t.at("rayl").v[0];
    int layreffr = 3, laysolfr = lt;
    for (int lay = 1; lay <= lt; ++lay) {
      laysolfr = laysolfr_lower(c, layreffr, lay, laysolfr);
      int ind0 = ind_lo(c, lay, T.nspa[20], 1, true), ind1 = ind_lo1(c, lay, T.nspa[20], 1, true);
      double tauray = c.colmol[lay] * rayl;
      for (int ig = 1; ig <= T.ngc[20]; ++ig) {
        taug[o + ig][lay] = c.colh2o[lay] * (interp4s(absa, c, lay, ind0, ind1, ig) + selfonly(selfref, c, lay, ig) +
                                             foronly(forref, c, lay, ig)) +
                            c.colch4[lay] * absch4(ig);
        taur[o + ig][lay] = tauray;
        if (lay == laysolfr) sfz[o + ig] = sflux(ig);
      }
    }
    for (int lay = lt + 1; lay <= nl; ++lay) {
      int ind0 = ind_up(c, lay, T.nspb[20], 1, true), ind1 = ind_up1(c, lay, T.nspb[20], 1, true);
      double tauray = c.colmol[lay] * rayl;
      for (int ig = 1; ig <= T.ngc[20]; ++ig) {
        // (fac00*absb + ... + fac11*absb(ind1+1) + forfac*(...)) in one sum (:800-806)
        taug[o + ig][lay] = c.colh2o[lay] * (interp4s(absb, c, lay, ind0, ind1, ig) + foronly(forref, c, lay, ig)) +
                            c.colch4[lay] * absch4(ig);
        taur[o + ig][lay] = tauray;
      }
    }
  }
  // ---- band 21 (:821-964): h2o/co2 both regions
  lower_eta_band(21, 0.0045321, 8, c.colco2);
  {
    auto& t = T.t[21];
    const int o = T.ngs[20];
    const FArr &absb = t.at("kb"), &forref = t.at("forref");
    double rayl = t.at("rayl").v[0];
    double strrat = 0.0045321;
    for (int lay = lt + 1; lay <= nl; ++lay) {
      SwEta e = sw_eta(c.colh2o[lay], strrat * c.colco2[lay], 4.);
      int ind0 = ind_up(c, lay, T.nspb[21], e.js, false), ind1 = ind_up1(c, lay, T.nspb[21], e.js, false);
      double tauray = c.colmol[lay] * rayl;
      for (int ig = 1; ig <= T.ngc[21]; ++ig) {
        taug[o + ig][lay] = major8(absb, c, lay, e, ind0, ind1, 5, ig) + c.colh2o[lay] * c.forfac[lay] * forinterp(forref, c, lay, ig);
        taur[o + ig][lay] = tauray;
      }
    }
  }
  // ---- band 22 (:967-1066): h2o/o2 + o2 continuum
  {
    auto& t = T.t[22];
    const int o = T.ngs[21];
    const FArr &absa = t.at("ka"), &absb = t.at("kb"), &selfref = t.at("selfref"), &forref = t.at("forref"),
               &sflux = t.at("sfluxref");
    double rayl = t.at("rayl").v[0];
    double o2adj = 1.6, strrat = 0.022708;
    int layreffr = 2, laysolfr = lt;
    for (int lay = 1; lay <= lt; ++lay) {
      laysolfr = laysolfr_lower(c, layreffr, lay, laysolfr);
      double o2cont = 4.35e-4 * c.colo2[lay] / (350.0 * 2.0);
      SwEta e = sw_eta(c.colh2o[lay], o2adj * strrat * c.colo2[lay], 8.);
      int ind0 = ind_lo(c, lay, T.nspa[22], e.js, false), ind1 = ind_lo1(c, lay, T.nspa[22], e.js, false);
      double tauray = c.colmol[lay] * rayl;
      for (int ig = 1; ig <= T.ngc[22]; ++ig) {
        taug[o + ig][lay] = major8(absa, c, lay, e, ind0, ind1, 9, ig) + c.colh2o[lay] * selfplusfor(selfref, forref, c, lay, ig) + o2cont;
        if (lay == laysolfr) sfz[o + ig] = sfl_eta(sflux, ig, e);
        taur[o + ig][lay] = tauray;
      }
    }
    for (int lay = lt + 1; lay <= nl; ++lay) {
      double o2cont = 4.35e-4 * c.colo2[lay] / (350.0 * 2.0);
      int ind0 = ind_up(c, lay, T.nspb[22], 1, true), ind1 = ind_up1(c, lay, T.nspb[22], 1, true);
      double tauray = c.colmol[lay] * rayl;
      for (int ig = 1; ig <= T.ngc[22]; ++ig) {
        taug[o + ig][lay] = c.colo2[lay] * o2adj * interp4s(absb, c, lay, ind0, ind1, ig) + o2cont;
        taur[o + ig][lay] = tauray;
      }
    }
  }
  // ---- band 23 (:1069-1138): h2o, g-dependent Rayleigh
  {
    auto& t = T.t[23];
    const int o = T.ngs[22];
    const FArr &absa = t.at("ka"), &selfref = t.at("selfref"), &forref = t.at("forref"), &sflux = t.at("sfluxref"),
               &rayl = t.at("rayl");
    double givfac = 1.029;
    int layreffr = 6, laysolfr = lt;
    for (int lay = 1; lay <= lt; ++lay) {
      laysolfr = laysolfr_lower(c, layreffr, lay, laysolfr);
      int ind0 = ind_lo(c, lay, T.nspa[23], 1, true), ind1 = ind_lo1(c, lay, T.nspa[23], 1, true);
      for (int ig = 1; ig <= T.ngc[23]; ++ig) {
        double tauray = c.colmol[lay] * rayl(ig);
        taug[o + ig][lay] = c.colh2o[lay] * (givfac * interp4s(absa, c, lay, ind0, ind1, ig) + selfonly(selfref, c, lay, ig) +
                                             foronly(forref, c, lay, ig));
        if (lay == laysolfr) sfz[o + ig] = sflux(ig);
        taur[o + ig][lay] = tauray;
      }
    }
    for (int lay = lt + 1; lay <= nl; ++lay)
      for (int ig = 1; ig <= T.ngc[23]; ++ig) {
        taug[o + ig][lay] = 0.;
        taur[o + ig][lay] = c.colmol[lay] * rayl(ig);
      }
  }
  // ---- band 24 (:1141-1259): h2o/o2 + o3, eta-dependent Rayleigh
  {
    auto& t = T.t[24];
    const int o = T.ngs[23];
    const FArr &absa = t.at("ka"), &absb = t.at("kb"), &selfref = t.at("selfref"), &forref = t.at("forref"),
               &sflux = t.at("sfluxref"), &abso3a = t.at("abso3a"), &abso3b = t.at("abso3b"),
               &rayla = t.at("rayla"), &raylb = t.at("raylb");
    double strrat = 0.124692;
    int layreffr = 1, laysolfr = lt;
    for (int lay = 1; lay <= lt; ++lay) {
      laysolfr = laysolfr_lower(c, layreffr, lay, laysolfr);
      SwEta e = sw_eta(c.colh2o[lay], strrat * c.colo2[lay], 8.);
      int ind0 = ind_lo(c, lay, T.nspa[24], e.js, false), ind1 = ind_lo1(c, lay, T.nspa[24], e.js, false);
      for (int ig = 1; ig <= T.ngc[24]; ++ig) {
        double tauray = c.colmol[lay] * (rayla(ig, e.js) + e.fs * (rayla(ig, e.js + 1) - rayla(ig, e.js)));
        taug[o + ig][lay] = major8(absa, c, lay, e, ind0, ind1, 9, ig) + c.colo3[lay] * abso3a(ig) +
                            c.colh2o[lay] * selfplusfor(selfref, forref, c, lay, ig);
        if (lay == laysolfr) sfz[o + ig] = sfl_eta(sflux, ig, e);
        taur[o + ig][lay] = tauray;
      }
    }
    for (int lay = lt + 1; lay <= nl; ++lay) {
      int ind0 = ind_up(c, lay, T.nspb[24], 1, true), ind1 = ind_up1(c, lay, T.nspb[24], 1, true);
      for (int ig = 1; ig <= T.ngc[24]; ++ig) {
        double tauray = c.colmol[lay] * raylb(ig);
        taug[o + ig][lay] = c.colo2[lay] * interp4s(absb, c, lay, ind0, ind1, ig) + c.colo3[lay] * abso3b(ig);
        taur[o + ig][lay] = tauray;
      }
    }
  }
  // ---- band 25 (:1262-1322): h2o + o3
  {
    auto& t = T.t[25];
    const int o = T.ngs[24];
    const FArr &absa = t.at("ka"), &sflux = t.at("sfluxref"), &abso3a = t.at("abso3a"), &abso3b = t.at("abso3b"),
               &rayl = t.at("rayl");
    int layreffr = 2, laysolfr = lt;
    for (int lay = 1; lay <= lt; ++lay) {
      laysolfr = laysolfr_lower(c, layreffr, lay, laysolfr);
      int ind0 = ind_lo(c, lay, T.nspa[25], 1, true), ind1 = ind_lo1(c, lay, T.nspa[25], 1, true);
      for (int ig = 1; ig <= T.ngc[25]; ++ig) {
        double tauray = c.colmol[lay] * rayl(ig);
        taug[o + ig][lay] = c.colh2o[lay] * interp4s(absa, c, lay, ind0, ind1, ig) + c.colo3[lay] * abso3a(ig);
        if (lay == laysolfr) sfz[o + ig] = sflux(ig);
        taur[o + ig][lay] = tauray;
      }
    }
    for (int lay = lt + 1; lay <= nl; ++lay)
      for (int ig = 1; ig <= T.ngc[25]; ++ig) {
        double tauray = c.colmol[lay] * rayl(ig);
        taug[o + ig][lay] = c.colo3[lay] * abso3b(ig);
        taur[o + ig][lay] = tauray;
      }
  }
  // ---- band 26 (:1325-1368): Rayleigh only
  {
    auto& t = T.t[26];
    const int o = T.ngs[25];
    const FArr &sflux = t.at("sfluxref"), &rayl = t.at("rayl");
    int laysolfr = lt;
    for (int lay = 1; lay <= lt; ++lay)
      for (int ig = 1; ig <= T.ngc[26]; ++ig) {
        if (lay == laysolfr) sfz[o + ig] = sflux(ig);
        taug[o + ig][lay] = 0.;
        taur[o + ig][lay] = c.colmol[lay] * rayl(ig);
      }
    for (int lay = lt + 1; lay <= nl; ++lay)
      for (int ig = 1; ig <= T.ngc[26]; ++ig) {
        taug[o + ig][lay] = 0.;
        taur[o + ig][lay] = c.colmol[lay] * rayl(ig);
      }
  }
  // ---- band 27 (:1371-1434): o3
  {
    auto& t = T.t[27];
    const int o = T.ngs[26];
    const FArr &absa = t.at("ka"), &absb = t.at("kb"), &sflux = t.at("sfluxref"), &rayl = t.at("rayl");
    double scalekur = 50.15 / 48.37;
    int layreffr = 32;
    for (int lay = 1; lay <= lt; ++lay) {
      int ind0 = ind_lo(c, lay, T.nspa[27], 1, true), ind1 = ind_lo1(c, lay, T.nspa[27], 1, true);
      for (int ig = 1; ig <= T.ngc[27]; ++ig) {
        double tauray = c.colmol[lay] * rayl(ig);
        taug[o + ig][lay] = c.colo3[lay] * interp4s(absa, c, lay, ind0, ind1, ig);
        taur[o + ig][lay] = tauray;
      }
    }
    int laysolfr = nl;
    for (int lay = lt + 1; lay <= nl; ++lay) {
      if (c.jp[lay - 1] < layreffr && c.jp[lay] >= layreffr) laysolfr = lay;
      int ind0 = ind_up(c, lay, T.nspb[27], 1, true), ind1 = ind_up1(c, lay, T.nspb[27], 1, true);
      for (int ig = 1; ig <= T.ngc[27]; ++ig) {
        double tauray = c.colmol[lay] * rayl(ig);
        taug[o + ig][lay] = c.colo3[lay] * interp4s(absb, c, lay, ind0, ind1, ig);
        if (lay == laysolfr) sfz[o + ig] = scalekur * sflux(ig);
        taur[o + ig][lay] = tauray;
      }
    }
  }
  // ---- band 28 (:1437-1534): o3/o2
  {
    auto& t = T.t[28];
    const int o = T.ngs[27];
    const FArr &absa = t.at("ka"), &absb = t.at("kb"), &sflux = t.at("sfluxref");
    double rayl = t.at("rayl").v[0];
    double strrat = 6.67029e-07;
    int layreffr = 58;
    for (int lay = 1; lay <= lt; ++lay) {
      SwEta e = sw_eta(c.colo3[lay], strrat * c.colo2[lay], 8.);
      int ind0 = ind_lo(c, lay, T.nspa[28], e.js, false), ind1 = ind_lo1(c, lay, T.nspa[28], e.js, false);
      double tauray = c.colmol[lay] * rayl;
      for (int ig = 1; ig <= T.ngc[28]; ++ig) {
        taug[o + ig][lay] = major8(absa, c, lay, e, ind0, ind1, 9, ig);
        taur[o + ig][lay] = tauray;
      }
    }
    int laysolfr = nl;
    for (int lay = lt + 1; lay <= nl; ++lay) {
      if (c.jp[lay - 1] < layreffr && c.jp[lay] >= layreffr) laysolfr = lay;
      SwEta e = sw_eta(c.colo3[lay], strrat * c.colo2[lay], 4.);
      int ind0 = ind_up(c, lay, T.nspb[28], e.js, false), ind1 = ind_up1(c, lay, T.nspb[28], e.js, false);
      double tauray = c.colmol[lay] * rayl;
      for (int ig = 1; ig <= T.ngc[28]; ++ig) {
        taug[o + ig][lay] = major8(absb, c, lay, e, ind0, ind1, 5, ig);
        if (lay == laysolfr) sfz[o + ig] = sfl_eta(sflux, ig, e);
        taur[o + ig][lay] = tauray;
      }
    }
  }
  // ---- band 29 (:1537-1636): h2o + co2
  {
    auto& t = T.t[29];
    const int o = T.ngs[28];
    const FArr &absa = t.at("ka"), &absb = t.at("kb"), &selfref = t.at("selfref"), &forref = t.at("forref"),
               &sflux = t.at("sfluxref"), &absh2o = t.at("absh2o"), &absco2 = t.at("absco2");
    double rayl = t.at("rayl").v[0];
    int layreffr = 49;
    for (int lay = 1; lay <= lt; ++lay) {
      int ind0 = ind_lo(c, lay, T.nspa[29], 1, true), ind1 = ind_lo1(c, lay, T.nspa[29], 1, true);
      double tauray = c.colmol[lay] * rayl;
      for (int ig = 1; ig <= T.ngc[29]; ++ig) {
        taug[o + ig][lay] = c.colh2o[lay] * (interp4s(absa, c, lay, ind0, ind1, ig) + selfonly(selfref, c, lay, ig) +
                                             foronly(forref, c, lay, ig)) +
                            c.colco2[lay] * absco2(ig);
        taur[o + ig][lay] = tauray;
      }
    }
    int laysolfr = nl;
    for (int lay = lt + 1; lay <= nl; ++lay) {
      if (c.jp[lay - 1] < layreffr && c.jp[lay] >= layreffr) laysolfr = lay;
      int ind0 = ind_up(c, lay, T.nspb[29], 1, true), ind1 = ind_up1(c, lay, T.nspb[29], 1, true);
      double tauray = c.colmol[lay] * rayl;
      for (int ig = 1; ig <= T.ngc[29]; ++ig) {
        taug[o + ig][lay] = c.colco2[lay] * interp4s(absb, c, lay, ind0, ind1, ig) + c.colh2o[lay] * absh2o(ig);
        if (lay == laysolfr) sfz[o + ig] = sflux(ig);
        taur[o + ig][lay] = tauray;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// reftra_sw (kmodts = 2), arrays indexed 1..klev (top-down)
// ---------------------------------------------------------------------------
static void reftra(int nlayers, const std::vector<char>& lrtchk, const std::vector<double>& pgg, double prmuz,
                   const std::vector<double>& ptau, const std::vector<double>& pw, std::vector<double>& pref,
                   std::vector<double>& prefd, std::vector<double>& ptra, std::vector<double>& ptrad) {
  const double eps = 1.e-08, zwcrit = 0.9999995;
  for (int jk = 1; jk <= nlayers; ++jk) {
    if (!lrtchk[jk]) {
      pref[jk] = 0.;
      ptra[jk] = 1.;
      prefd[jk] = 0.;
      ptrad[jk] = 1.;
      continue;
    }
    double zto1 = ptau[jk], zw = pw[jk], zg = pgg[jk];
    double zg3 = 3. * zg;
    double zgamma1 = (8. - zw * (5. + zg3)) * 0.25;
    double zgamma2 = 3. * (zw * (1. - zg)) * 0.25;
    double zgamma3 = (2. - zg3 * prmuz) * 0.25;
    double zgamma4 = 1. - zgamma3;
    double r = zg / (1. - zg);
    double zwo = zw / (1. - (1. - zw) * (r * r));
    if (zwo >= zwcrit) {
      double za = zgamma1 * prmuz;
      double za1 = za - zgamma3;
      double zgt = zgamma1 * zto1;
      double ze1 = std::min(zto1 / prmuz, 500.);
      double ze2 = sw_exp(ze1);
      pref[jk] = (zgt - za1 * (1. - ze2)) / (1. + zgt);
      ptra[jk] = 1. - pref[jk];
      prefd[jk] = zgt / (1. + zgt);
      ptrad[jk] = 1. - prefd[jk];
      if (ze2 == 1.0) {
        pref[jk] = 0.0;
        ptra[jk] = 1.0;
        prefd[jk] = 0.0;
        ptrad[jk] = 1.0;
      }
    } else {
      double za1 = zgamma1 * zgamma4 + zgamma2 * zgamma3;
      double za2 = zgamma1 * zgamma3 + zgamma2 * zgamma4;
      double zrk = std::sqrt(zgamma1 * zgamma1 - zgamma2 * zgamma2);
      double zrp = zrk * prmuz;
      double zrp1 = 1. + zrp;
      double zrm1 = 1. - zrp;
      double zrk2 = 2. * zrk;
      double zrpp = 1. - zrp * zrp;
      double zrkg = zrk + zgamma1;
      double zr1 = zrm1 * (za2 + zrk * zgamma3);
      double zr2 = zrp1 * (za2 - zrk * zgamma3);
      double zr3 = zrk2 * (zgamma3 - za2 * prmuz);
      double zr4 = zrpp * zrkg;
      double zr5 = zrpp * (zrk - zgamma1);
      double zt1 = zrp1 * (za1 + zrk * zgamma4);
      double zt2 = zrm1 * (za1 - zrk * zgamma4);
      double zt3 = zrk2 * (zgamma4 + za1 * prmuz);
      double zt4 = zr4;
      double zt5 = zr5;
      double zbeta = (zgamma1 - zrk) / zrkg;
      double ze1 = std::min(zrk * zto1, 500.);
      double ze2 = std::min(zto1 / prmuz, 500.);
      double zem1 = sw_exp(ze1);
      double zep1 = 1. / zem1;
      double zem2 = sw_exp(ze2);
      double zep2 = 1. / zem2;
      double zdenr = zr4 * zep1 + zr5 * zem1;
      double zdent = zt4 * zep1 + zt5 * zem1;
      if (zdenr >= -eps && zdenr <= eps) {
        pref[jk] = eps;
        ptra[jk] = zem2;
      } else {
        pref[jk] = zw * (zr1 * zep1 - zr2 * zem1 - zr3 * zem2) / zdenr;
        ptra[jk] = zem2 - zem2 * zw * (zt1 * zep1 - zt2 * zem1 - zt3 * zep2) / zdent;
      }
      double zemm = zem1 * zem1;
      double zdend = 1. / ((1. - zbeta * zemm) * zrkg);
      prefd[jk] = zgamma2 * (1. - zemm) * zdend;
      ptrad[jk] = zrk2 * zem1 * zdend;
    }
  }
}

// vrtqdr_sw: adding method, levels 1..klev+1 (top-down)
static void vrtqdr(int klev, const std::vector<double>& pref, const std::vector<double>& prefd,
                   const std::vector<double>& ptra, const std::vector<double>& ptrad, const std::vector<double>& pdbt,
                   const std::vector<double>& ptdbt, std::vector<double>& pfd, std::vector<double>& pfu) {
  std::vector<double> prup(klev + 2), prupd(klev + 2), prdnd(klev + 2), ztdn(klev + 2);
  // spcvrt sets zrup(klev+1) = palbp, zrupd(klev+1) = palbd (rrtmg_sw_spcvrt.f90:350-351, 370-371),
  // the same values it stores in zref(klev+1), zrefd(klev+1).
  prup[klev + 1] = pref[klev + 1];
  prupd[klev + 1] = prefd[klev + 1];
  double zreflect = 1. / (1. - prefd[klev + 1] * prefd[klev]);
  prup[klev] = pref[klev] + (ptrad[klev] * ((ptra[klev] - pdbt[klev]) * prefd[klev + 1] + pdbt[klev] * pref[klev + 1])) * zreflect;
  prupd[klev] = prefd[klev] + ptrad[klev] * ptrad[klev] * prefd[klev + 1] * zreflect;
  for (int jk = 1; jk <= klev - 1; ++jk) {
    int ikp = klev + 1 - jk, ikx = ikp - 1;
    zreflect = 1. / (1. - prupd[ikp] * prefd[ikx]);
    prup[ikx] = pref[ikx] + (ptrad[ikx] * ((ptra[ikx] - pdbt[ikx]) * prupd[ikp] + pdbt[ikx] * prup[ikp])) * zreflect;
    prupd[ikx] = prefd[ikx] + ptrad[ikx] * ptrad[ikx] * prupd[ikp] * zreflect;
  }
  ztdn[1] = 1.;
  prdnd[1] = 0.;
  ztdn[2] = ptra[1];
  prdnd[2] = prefd[1];
  for (int jk = 2; jk <= klev; ++jk) {
    int ikp = jk + 1;
    zreflect = 1. / (1. - prefd[jk] * prdnd[jk]);
    ztdn[ikp] = ptdbt[jk] * ptra[jk] + (ptrad[jk] * ((ztdn[jk] - ptdbt[jk]) + ptdbt[jk] * pref[jk] * prdnd[jk])) * zreflect;
    prdnd[ikp] = prefd[jk] + ptrad[jk] * ptrad[jk] * prdnd[jk] * zreflect;
  }
  for (int jk = 1; jk <= klev + 1; ++jk) {
    zreflect = 1. / (1. - prdnd[jk] * prupd[jk]);
    pfu[jk] = (ptdbt[jk] * prup[jk] + (ztdn[jk] - ptdbt[jk]) * prupd[jk]) * zreflect;
    pfd[jk] = ptdbt[jk] + (ztdn[jk] - ptdbt[jk] + ptdbt[jk] * prup[jk] * prdnd[jk]) * zreflect;
  }
}

// ---------------------------------------------------------------------------
// spcvrt_sw / spcvmc_sw, icpr = 1, idelm = 1: the clear pass, and the total
// pass combined with it by the cover, per band (non-McICA) or per g-point
// (McICA); clear sky has cover 0 and cloud optics 0 / 1 / 0
// ---------------------------------------------------------------------------
void sw_spcvrt(SwColumn& c, double prmu0, const double* albdir, const double* albdif, SwOut& out, bool run_taumol) {
  const SwTables& T = g_sw;
  const int klev = c.nlayers;
  out.fu.assign(klev + 2, 0.);
  out.fd.assign(klev + 2, 0.);
  out.cu.assign(klev + 2, 0.);
  out.cd.assign(klev + 2, 0.);
  if (run_taumol) sw_taumol(c);
  const int K = klev + 2;
  std::vector<double> ztauc(K), zomcc(K), zgcc(K), ztauo(K), zomco(K), zgco(K);
  std::vector<double> zrefc(K), zrefdc(K), ztrac(K), ztradc(K), zrefo(K), zrefdo(K), ztrao(K), ztrado(K);
  std::vector<double> zref(K), zrefd(K), ztra(K), ztrad(K), zdbtc(K), ztdbtc(K), zdbt(K), ztdbt(K);
  std::vector<double> zcd(K), zcu(K), zfd(K), zfu(K);
  std::vector<char> lrtchkclr(K, 1), lrtchkcld(K, 0);
  int iw = 0;
  for (int jb = 16; jb <= 29; ++jb) {
    int ibm = jb - 15;
    for (int jg = 1; jg <= T.ngc[jb]; ++jg) {
      iw = iw + 1;
      // spcvmc_sw (rrtmg_sw_spcvmc.f90:388, 412-413, 462-474, 504-505): the
      // g-point's own cover and cloud optics in place of the band's
      const size_t gk = (size_t)(iw - 1) * (size_t)K;
      auto CF = [&](int lay) { return c.mcica ? c.cldfmc[gk + lay] : c.pclfr[lay]; };
      auto TC = [&](int lay) { return c.mcica ? c.taucmc[gk + lay] : c.ptauc[ibm][lay]; };
      auto OC = [&](int lay) { return c.mcica ? c.ssacmc[gk + lay] : c.pomgc[ibm][lay]; };
      auto AC = [&](int lay) { return c.mcica ? c.asmcmc[gk + lay] : c.pasyc[ibm][lay]; };
      double zincflx = c.adjflux[jb] * c.sfluxzen[iw] * prmu0;
      ztdbtc[1] = 1.0;
      zdbtc[klev + 1] = 0.0;
      ztrac[klev + 1] = 0.0;
      ztradc[klev + 1] = 0.0;
      zrefc[klev + 1] = albdir[ibm];
      zrefdc[klev + 1] = albdif[ibm];
      ztrao[klev + 1] = 0.0;
      ztrado[klev + 1] = 0.0;
      zrefo[klev + 1] = albdir[ibm];
      zrefdo[klev + 1] = albdif[ibm];
      ztdbt[1] = 1.0;
      zdbt[klev + 1] = 0.0;
      ztra[klev + 1] = 0.0;
      ztrad[klev + 1] = 0.0;
      zref[klev + 1] = albdir[ibm];
      zrefd[klev + 1] = albdif[ibm];
      for (int jk = 1; jk <= klev; ++jk) {
        int ikl = klev + 1 - jk;
        lrtchkclr[jk] = 1;
        lrtchkcld[jk] = CF(ikl) > 1.e-12;  // pclfr > repclc (:263, :388)
        double taua = c.taua[ibm][ikl], omga = c.ssaa[ibm][ikl], asya = c.asma[ibm][ikl];
        ztauc[jk] = c.taur[iw][ikl] + c.taug[iw][ikl] + taua;
        zomcc[jk] = c.taur[iw][ikl] * 1.0 + taua * omga;
        zgcc[jk] = asya * omga * taua / zomcc[jk];
        zomcc[jk] = zomcc[jk] / ztauc[jk];
        double zf = zgcc[jk] * zgcc[jk];
        double zwf = zomcc[jk] * zf;
        ztauc[jk] = (1.0 - zwf) * ztauc[jk];
        zomcc[jk] = (zomcc[jk] - zwf) / (1.0 - zwf);
        zgcc[jk] = (zgcc[jk] - zf) / (1.0 - zf);
        // icpr >= 1 (:459-464); clear sky: ptauc = 0, pomgc = 1, pasyc = 0
        if (!c.total_pass) OPC_PAUSE();
        const double ptauc = TC(ikl), pomgc = OC(ikl), pasyc = AC(ikl);
        ztauo[jk] = ztauc[jk] + ptauc;
        zomco[jk] = ztauc[jk] * zomcc[jk] + ptauc * pomgc;
        zgco[jk] = (ptauc * pomgc * pasyc + ztauc[jk] * zomcc[jk] * zgcc[jk]) / zomco[jk];
        zomco[jk] = zomco[jk] / ztauo[jk];
        if (!c.total_pass) OPC_RESUME();
      }
      reftra(klev, lrtchkclr, zgcc, prmu0, ztauc, zomcc, zrefc, zrefdc, ztrac, ztradc);
      if (!c.total_pass) OPC_PAUSE();
      reftra(klev, lrtchkcld, zgco, prmu0, ztauo, zomco, zrefo, zrefdo, ztrao, ztrado);
      if (!c.total_pass) OPC_RESUME();
      for (int jk = 1; jk <= klev; ++jk) {
        if (!c.total_pass) OPC_PAUSE();
        const int ikl = klev + 1 - jk;
        const double zclear = 1.0 - CF(ikl), zcloud = CF(ikl);
        zref[jk] = zclear * zrefc[jk] + zcloud * zrefo[jk];
        zrefd[jk] = zclear * zrefdc[jk] + zcloud * zrefdo[jk];
        ztra[jk] = zclear * ztrac[jk] + zcloud * ztrao[jk];
        ztrad[jk] = zclear * ztradc[jk] + zcloud * ztrado[jk];
        if (!c.total_pass) OPC_RESUME();
        double zdbtmc = sw_exp(ztauc[jk] / prmu0);
        zdbtc[jk] = zdbtmc;
        ztdbtc[jk + 1] = zdbtc[jk] * ztdbtc[jk];
        if (!c.total_pass) OPC_PAUSE();
        double zdbtmo = sw_exp(ztauo[jk] / prmu0);
        zdbt[jk] = zclear * zdbtmc + zcloud * zdbtmo;
        ztdbt[jk + 1] = zdbt[jk] * ztdbt[jk];
        if (!c.total_pass) OPC_RESUME();
      }
      vrtqdr(klev, zrefc, zrefdc, ztrac, ztradc, zdbtc, ztdbtc, zcd, zcu);
      if (!c.total_pass) OPC_PAUSE();
      vrtqdr(klev, zref, zrefd, ztra, ztrad, zdbt, ztdbt, zfd, zfu);
      if (!c.total_pass) OPC_RESUME();
      for (int jk = 1; jk <= klev + 1; ++jk) {
        int ikl = klev + 2 - jk;
        if (!c.total_pass) OPC_PAUSE();
        out.fu[ikl] = out.fu[ikl] + zincflx * zfu[jk];
        out.fd[ikl] = out.fd[ikl] + zincflx * zfd[jk];
        if (!c.total_pass) OPC_RESUME();
        out.cu[ikl] = out.cu[ikl] + zincflx * zcu[jk];
        out.cd[ikl] = out.cd[ikl] + zincflx * zcd[jk];
      }
    }
  }
}

// cldprop_sw, inflag = 2 (rrtmg_sw_cldprop.f90:158-340) for one layer whose
// optics are formed: ice (Ebert-Curry coefficients by band limit, iceflag 1;
// the STREAMER table, 2; Fu's table with its delta fractions, 3) and liquid
// (Hu-Stamnes table, liqflag 1) extinction, single-scattering albedo and
// asymmetry, each delta-M scaled, combined into the layer's delta-scaled
// optics.  Returns false where the reference stops.  band = 0: the 14 bands
// (cldprop_sw); band = 16..29: that band alone, as cldprmc_sw forms one
// g-point's optics on its band ngb(ig) (rrtmg_sw_cldprmc.f90:150-320), its
// stops taken on that band only.
static bool sw_cldprop_phys(const SwInput& in, double ciwp, double clwp, double radice, double radliq,
                            double* taucloud, double* ssacloud, double* asmcloud, int band = 0) {
  const SwTables& T = g_sw;
  const int lo = band ? band : 16, hi = band ? band : 29;
  const double eps = 1.e-06, cldmin = 1.e-20;
  double extcoice[30], ssacoice[30], gice[30], forwice[30], extcoliq[30], ssacoliq[30], gliq[30], forwliq[30];
  auto ice_ok = [&](int ib) {
    return !(extcoice[ib] < 0.0 || ssacoice[ib] > 1.0 || ssacoice[ib] < 0.0 || gice[ib] > 1.0 || gice[ib] < 0.0);
  };
  if (ciwp == 0.0) {
    for (int ib = lo; ib <= hi; ++ib) extcoice[ib] = ssacoice[ib] = gice[ib] = forwice[ib] = 0.0;
  } else if (in.iceflag == 1) {
    if (radice < 13.0 || radice > 130.) return false;
    for (int ib = lo; ib <= hi; ++ib) {
      const double wn = T.wavenum2(ib - 15);
      int icx = 5;
      if (wn > 1.43e04) icx = 1;
      else if (wn > 7.7e03) icx = 2;
      else if (wn > 5.3e03) icx = 3;
      else if (wn > 4.0e03) icx = 4;
      extcoice[ib] = T.abari(icx) + T.bbari(icx) / radice;
      ssacoice[ib] = 1. - T.cbari(icx) - T.dbari(icx) * radice;
      gice[ib] = T.ebari(icx) + T.fbari(icx) * radice;
      if (gice[ib] >= 1.0) gice[ib] = 1.0 - eps;
      forwice[ib] = gice[ib] * gice[ib];
      if (!ice_ok(ib)) return false;
    }
  } else if (in.iceflag == 2) {
    if (radice < 5.0 || radice > 131.0) return false;
    const double factor = (radice - 2.) / 3.;
    int index = (int)factor;
    if (index == 43) index = 42;
    const double fint = factor - (double)index;
    for (int ib = lo; ib <= hi; ++ib) {
      extcoice[ib] = T.extice2(index, ib) + fint * (T.extice2(index + 1, ib) - T.extice2(index, ib));
      ssacoice[ib] = T.ssaice2(index, ib) + fint * (T.ssaice2(index + 1, ib) - T.ssaice2(index, ib));
      gice[ib] = T.asyice2(index, ib) + fint * (T.asyice2(index + 1, ib) - T.asyice2(index, ib));
      forwice[ib] = gice[ib] * gice[ib];
      if (!ice_ok(ib)) return false;
    }
  } else {
    if (radice < 5.0 || radice > 140.0) return false;
    const double factor = (radice - 2.) / 3.;
    int index = (int)factor;
    if (index == 46) index = 45;
    const double fint = factor - (double)index;
    for (int ib = lo; ib <= hi; ++ib) {
      extcoice[ib] = T.extice3(index, ib) + fint * (T.extice3(index + 1, ib) - T.extice3(index, ib));
      ssacoice[ib] = T.ssaice3(index, ib) + fint * (T.ssaice3(index + 1, ib) - T.ssaice3(index, ib));
      gice[ib] = T.asyice3(index, ib) + fint * (T.asyice3(index + 1, ib) - T.asyice3(index, ib));
      const double fdelta = T.fdlice3(index, ib) + fint * (T.fdlice3(index + 1, ib) - T.fdlice3(index, ib));
      if (fdelta < 0.0 || fdelta > 1.0) return false;
      forwice[ib] = fdelta + 0.5 / ssacoice[ib];
      if (forwice[ib] > gice[ib]) forwice[ib] = gice[ib];
      if (!ice_ok(ib)) return false;
    }
  }
  if (clwp == 0.0) {
    for (int ib = lo; ib <= hi; ++ib) extcoliq[ib] = ssacoliq[ib] = gliq[ib] = forwliq[ib] = 0.0;
  } else {
    if (radliq < 2.5 || radliq > 60.) return false;
    int index = (int)(radliq - 1.5);
    if (index == 0) index = 1;
    if (index == 58) index = 57;
    const double fint = radliq - 1.5 - (double)index;
    for (int ib = lo; ib <= hi; ++ib) {
      extcoliq[ib] = T.extliq1(index, ib) + fint * (T.extliq1(index + 1, ib) - T.extliq1(index, ib));
      ssacoliq[ib] = T.ssaliq1(index, ib) + fint * (T.ssaliq1(index + 1, ib) - T.ssaliq1(index, ib));
      if (fint < 0. && ssacoliq[ib] > 1.) ssacoliq[ib] = T.ssaliq1(index, ib);
      gliq[ib] = T.asyliq1(index, ib) + fint * (T.asyliq1(index + 1, ib) - T.asyliq1(index, ib));
      forwliq[ib] = gliq[ib] * gliq[ib];
      if (extcoliq[ib] < 0.0 || ssacoliq[ib] > 1.0 || ssacoliq[ib] < 0.0 || gliq[ib] > 1.0 || gliq[ib] < 0.0)
        return false;
    }
  }
  for (int ib = lo; ib <= hi; ++ib) {
    const double tauliqorig = clwp * extcoliq[ib];
    const double tauiceorig = ciwp * extcoice[ib];
    const double ssaliq = ssacoliq[ib] * (1.0 - forwliq[ib]) / (1.0 - forwliq[ib] * ssacoliq[ib]);
    const double tauliq = (1.0 - forwliq[ib] * ssacoliq[ib]) * tauliqorig;
    const double ssaice = ssacoice[ib] * (1.0 - forwice[ib]) / (1.0 - forwice[ib] * ssacoice[ib]);
    const double tauice = (1.0 - forwice[ib] * ssacoice[ib]) * tauiceorig;
    const double scatliq = ssaliq * tauliq;
    double scatice = ssaice * tauice;
    double tc = tauliq + tauice;
    if (tc == 0.0) tc = cldmin;
    if (scatice == 0.0) scatice = cldmin;
    taucloud[ib - 16] = tc;
    ssacloud[ib - 16] = (scatliq + scatice) / tc;
    if (in.iceflag == 3)
      asmcloud[ib - 16] = (1.0 / (scatliq + scatice)) *
                          (scatliq * (gliq[ib] - forwliq[ib]) / (1.0 - forwliq[ib]) +
                           scatice * ((gice[ib] - forwice[ib]) / (1.0 - forwice[ib])));
    else
      asmcloud[ib - 16] = (scatliq * (gliq[ib] - forwliq[ib]) / (1.0 - forwliq[ib]) +
                           scatice * (gice[ib] - forwice[ib]) / (1.0 - forwice[ib])) /
                          (scatliq + scatice);
  }
  return true;
}

// cldprop_sw (rrtmg_sw_cldprop.f90:118-340): the optics of a layer whose
// cover is >= cldmin and whose water path or band-summed depth is >= cldmin
// (1e-20) are formed -- with inflag = 0 the given optics delta-M scaled with
// the forward-scattering fraction, with inflag = 2 by sw_cldprop_phys; other
// layers keep taucloud = 0, ssacloud = 1, asmcloud = 0.  Returns false where
// the reference stops.
static bool sw_cldprop(const SwInput& in, int iplon, SwColumn& c) {
  const int nl = in.nlay, ncol = in.ncol;
  const double cldmin = 1.e-20;
  for (int lay = 1; lay <= nl; ++lay) {
    const size_t o = (size_t)iplon + (size_t)ncol * (size_t)(lay - 1);
    c.pclfr[lay] = in.cldfr[o];
    double tauctot = 0.0;
    for (int n = 0; n < 14; ++n) tauctot = tauctot + (in.taucld ? in.taucld[(size_t)n + 14 * o] : 0.0);
    const double ciwp = in.cicewp ? in.cicewp[o] : 0.0, clwp = in.cliqwp ? in.cliqwp[o] : 0.0;
    const double cwp = ciwp + clwp;
    for (int ibm = 1; ibm <= 14; ++ibm) {
      c.ptauc[ibm][lay] = 0.0;
      c.pomgc[ibm][lay] = 1.0;
      c.pasyc[ibm][lay] = 0.0;
    }
    if (c.pclfr[lay] >= cldmin && (cwp >= cldmin || tauctot >= cldmin) && in.inflag == 2) {
      double tc[14], ssa[14], asm_[14];
      if (!sw_cldprop_phys(in, ciwp, clwp, in.reice ? in.reice[o] : 0.0, in.reliq ? in.reliq[o] : 0.0, tc, ssa,
                           asm_))
        return false;
      for (int ibm = 1; ibm <= 14; ++ibm) {
        c.ptauc[ibm][lay] = tc[ibm - 1];
        c.pomgc[ibm][lay] = ssa[ibm - 1];
        c.pasyc[ibm][lay] = asm_[ibm - 1];
      }
    } else if (c.pclfr[lay] >= cldmin && (cwp >= cldmin || tauctot >= cldmin)) {
      for (int ibm = 1; ibm <= 14; ++ibm) {
        const size_t q = (size_t)(ibm - 1) + 14 * o;
        const double taucldorig_a = in.taucld[q];
        const double ffp = in.fsfcld[q];
        const double ffp1 = 1.0 - ffp;
        const double ffpssa = 1.0 - ffp * in.ssacld[q];
        c.pomgc[ibm][lay] = ffp1 * in.ssacld[q] / ffpssa;
        c.ptauc[ibm][lay] = ffpssa * taucldorig_a;
        c.pasyc[ibm][lay] = (in.asmcld[q] - ffp) / (ffp1);
      }
    }
  }
  return true;
}

// McICA's cloud inputs (inatm_sw, rrtmg_sw_rad.f90:1084-1099) and cldprmc_sw
// (rrtmg_sw_cldprmc.f90:112-328): per g-point iw and layer, a sub-column whose
// cover is >= cldmin and whose water path or own depth is >= cldmin (1e-20)
// gets its optics formed -- inflag = 0 the given ones delta-M scaled with the
// forward-scattering fraction, inflag = 2 the parameterisations on its band
// ngb(iw); other sub-columns keep the optics given.  inflag = 1 stops (not
// available with McICA), as does a size or optical property out of range.
static bool sw_cldprmc(const SwInput& in, int iplon, SwColumn& c) {
  const int nl = in.nlay, ncol = in.ncol, L2 = nl + 2;
  const double cldmin = 1.e-20;
  c.cldfmc.assign((size_t)112 * L2, 0.0);
  c.taucmc.assign((size_t)112 * L2, 0.0);
  c.ssacmc.assign((size_t)112 * L2, 1.0);
  c.asmcmc.assign((size_t)112 * L2, 0.0);
  for (int lay = 1; lay <= nl; ++lay) {
    const size_t o = (size_t)iplon + (size_t)ncol * (size_t)(lay - 1);
    int iw = 0;
    for (int jb = 16; jb <= 29; ++jb)
      for (int jg = 1; jg <= g_sw.ngc[jb]; ++jg) {
        iw = iw + 1;
        const size_t q = (size_t)(iw - 1) + 112 * o, k = (size_t)(iw - 1) * L2 + lay;
        const double cf = in.cldfmcl[q];
        double tau = in.taucmcl ? in.taucmcl[q] : 0.0;
        double ssa = in.ssacmcl ? in.ssacmcl[q] : 1.0;
        double asy = in.asmcmcl ? in.asmcmcl[q] : 0.0;
        const double ciwp = in.ciwpmcl ? in.ciwpmcl[q] : 0.0, clwp = in.clwpmcl ? in.clwpmcl[q] : 0.0;
        const double cwp = ciwp + clwp;
        if (cf >= cldmin && (cwp >= cldmin || tau >= cldmin)) {
          if (in.inflag == 0) {
            const double ffp = in.fsfcmcl[q];
            const double ffp1 = 1.0 - ffp;
            const double ffpssa = 1.0 - ffp * ssa;
            const double ssacloud_a = ffp1 * ssa / ffpssa;
            tau = ffpssa * tau;
            ssa = ssacloud_a;
            asy = (asy - ffp) / (ffp1);
          } else if (in.inflag == 1) {
            return false;
          } else if (in.inflag == 2) {
            double tc[14], sc[14], ac[14];
            if (!sw_cldprop_phys(in, ciwp, clwp, in.reice ? in.reice[o] : 0.0, in.reliq ? in.reliq[o] : 0.0, tc,
                                 sc, ac, jb))
              return false;
            tau = tc[jb - 16];
            ssa = sc[jb - 16];
            asy = ac[jb - 16];
          }
        }
        c.cldfmc[k] = cf;
        c.taucmc[k] = tau;
        c.ssacmc[k] = ssa;
        c.asmcmc[k] = asy;
      }
  }
  return true;
}

bool sw_column(const SwInput& in, int iplon, SwColumn& c, SwOut& out, bool* partial, bool* stopped) {
  const double zepzen = 1.e-10;
  int nl = in.nlay;
  if (partial) *partial = false;
  if (stopped) *stopped = false;
  if (!in.mcica && in.coszen[iplon] < zepzen) {
    out.fu.assign(nl + 2, 0.);
    out.fd.assign(nl + 2, 0.);
    out.cu.assign(nl + 2, 0.);
    out.cd.assign(nl + 2, 0.);
    out.hr.assign(nl + 1, 0.);
    out.hrc.assign(nl + 1, 0.);
    return false;
  }
  sw_inatm(in, iplon, c);
  c.total_pass = in.icld >= 1;
  c.mcica = in.mcica && in.icld >= 1;
  if (c.mcica) {
    if (!sw_cldprmc(in, iplon, c) && stopped) *stopped = true;
  } else if (in.icld >= 1) {
    // without McICA the SW computes clear or overcast layers only (:533-538)
    const double zepsec = 1.e-06, oneminus = 1.0 - zepsec;
    for (int i = 1; i <= nl; ++i) {
      const double f = in.cldfr[(size_t)iplon + (size_t)in.ncol * (size_t)(i - 1)];
      if (f > zepsec && f < oneminus && partial) *partial = true;
    }
    if (!sw_cldprop(in, iplon, c) && stopped) *stopped = true;
  }
  sw_setcoef(c);
  double cossza = in.coszen[iplon];
  if (cossza < zepzen) cossza = zepzen;
  double albdir[15], albdif[15];
  for (int ib = 1; ib <= 9; ++ib) {
    albdir[ib] = in.aldir[iplon];
    albdif[ib] = in.aldif[iplon];
  }
  albdir[14] = in.aldir[iplon];
  albdif[14] = in.aldif[iplon];
  for (int ib = 10; ib <= 13; ++ib) {
    albdir[ib] = in.asdir[iplon];
    albdif[ib] = in.asdif[iplon];
  }
  sw_spcvrt(c, cossza, albdir, albdif, out);
  out.hr.assign(nl + 1, 0.);
  out.hrc.assign(nl + 1, 0.);
  for (int i = 1; i <= nl; ++i) {
    double zdpgcp = g_sw.heatfac / c.pdp[i];
    double nc1 = out.cd[i + 1] - out.cu[i + 1], nc0 = out.cd[i] - out.cu[i];
    double nf1 = out.fd[i + 1] - out.fu[i + 1], nf0 = out.fd[i] - out.fu[i];
    out.hrc[i] = (nc1 - nc0) * zdpgcp;
    out.hr[i] = (nf1 - nf0) * zdpgcp;
  }
  out.hrc[nl] = 0.;
  out.hr[nl] = 0.;
  return true;
}

}  // namespace orc
