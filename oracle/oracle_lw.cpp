// CPU oracle, longwave -- TEST INFRASTRUCTURE ONLY (the checker, never the
// product).  FP64 restatement of the reference's RRTMG_LW path (clear sky,
// and clouds with given cloud optical depths, inflglw = 0 -- cldprop
// rrtmg_lw_cldprop.f90:155-174 -- with random overlap, icld = 1, rtrn
// rrtmg_lw_rtrn.f90, or maximum/random overlap, icld = 2 / 3, rtrnmr's cloudy
// branches rrtmg_lw_rtrnmr.f90:300-705):
//   inatm    rrtmg_lw_rad.nomcica.f90:572-901
//   setcoef  rrtmg_lw_setcoef.f90:31-415
//   taumol   rrtmg_lw_taumol.f90:31-3149 (taugb1..16)
//   rtrnmr   rrtmg_lw_rtrnmr.f90:32-779 (clear-layer branch :589-616,
//            upward :649-713, band sums :720-746, heating :752-776)
//   driver   rrtmg_lw_rad.nomcica.f90:80-569 (taut = taug + taua, :508-520)
// Expressions keep the reference's operation order; build with
// -ffp-contract=off so no multiply-add is fused.
#include "oracle_lw.hpp"

#include <algorithm>
#include <cmath>

namespace orc {

LwTables g_lw;
int g_table_mode = 1;  // 1: reference lookup tables; 0: analytic exp / tfn

static std::string reduced_name(const std::string& o) {
  // kao -> ka, kbo_mn2 -> kb_mn2, fracrefao -> fracrefa, ccl4o -> ccl4
  if (o.rfind("kao", 0) == 0) return "ka" + o.substr(3);
  if (o.rfind("kbo", 0) == 0) return "kb" + o.substr(3);
  return o.substr(0, o.size() - 1);
}

void lw_init(const Blob& blob, double cpdair) {
  LwTables& T = g_lw;
  const int nbnd = 16;
  std::vector<int> ngc = blob.i("lw.ngc"), ngn = blob.i("lw.ngn"), ngm = blob.i("lw.ngm"),
                   ngs = blob.i("lw.ngs"), nspa = blob.i("lw.nspa"), nspb = blob.i("lw.nspb");
  std::vector<double> rwgt = make_rwgt(nbnd, ngc, ngn, ngm, blob.r("lw.wt"));
  const FArr& dw = blob.r("lw.delwave");
  int ngs_prev = 0;
  for (int b = 1; b <= nbnd; ++b) {
    T.ngc[b] = ngc[b - 1];
    T.ngs[b] = ngs[b - 1];
    T.nspa[b] = nspa[b - 1];
    T.nspb[b] = nspb[b - 1];
    T.delwave[b] = dw(b);
    char pre[8];
    std::snprintf(pre, sizeof pre, "lw%02d.", b);
    std::string prefix(pre);
    for (const auto& kv : blob.real) {
      if (kv.first.rfind(prefix, 0) != 0) continue;
      std::string nm = kv.first.substr(prefix.size());
      bool planckfrac = nm.rfind("fracref", 0) == 0;
      int gpos = planckfrac ? 0 : kv.second.ndim - 1;
      T.t[b][reduced_name(nm)] =
          reduce_g(kv.second, gpos, ngc[b - 1], &ngn[ngs_prev], &rwgt[(size_t)(b - 1) * 16], !planckfrac);
    }
    ngs_prev = ngs[b - 1];
  }
  T.pref = blob.r("lw.pref");
  T.preflog = blob.r("lw.preflog");
  T.tref = blob.r("lw.tref");
  T.chi_mls = blob.r("lw.chi_mls");
  T.totplnk = blob.r("lw.totplnk");
  T.totplk16 = blob.r("lw.totplk16");
  T.totplnkderiv = blob.r("lw.totplnkderiv");
  T.totplk16deriv = blob.r("lw.totplk16deriv");
  T.absice0 = blob.r("lwcld.absice0");
  T.absice1 = blob.r("lwcld.absice1");
  T.absice2 = blob.r("lwcld.absice2");
  T.absice3 = blob.r("lwcld.absice3");
  T.absliq1 = blob.r("lwcld.absliq1");
  T.abscld1 = blob.r("lwcld.abscld1").v.at(0);
  T.absliq0 = blob.r("lwcld.absliq0").v.at(0);

  // rrtmg_lw_init.f90:106-124
  const int ntbl = 10000;
  const double pade = 0.278, expeps = 1.e-20;
  T.tau_tbl[0] = 0.0;
  T.tau_tbl[ntbl] = 1.e10;
  T.exp_tbl[0] = 1.0;
  T.exp_tbl[ntbl] = expeps;
  T.tfn_tbl[0] = 0.0;
  T.tfn_tbl[ntbl] = 1.0;
  T.bpade = 1.0 / pade;
  for (int itr = 1; itr <= ntbl - 1; ++itr) {
    double tfn = (double)itr / (double)ntbl;
    T.tau_tbl[itr] = T.bpade * tfn / (1.0 - tfn);
    T.exp_tbl[itr] = std::exp(-T.tau_tbl[itr]);
    if (T.exp_tbl[itr] <= expeps) T.exp_tbl[itr] = expeps;
    if (T.tau_tbl[itr] < 0.06)
      T.tfn_tbl[itr] = T.tau_tbl[itr] / 6.0;
    else
      T.tfn_tbl[itr] = 1.0 - 2.0 * ((1.0 / T.tau_tbl[itr]) - (T.exp_tbl[itr] / (1. - T.exp_tbl[itr])));
  }
  // lwdatinit, rrtmg_lw_init.f90:178-279
  T.grav = 9.8066;
  T.avogad = 6.02214199e+23;
  T.heatfac = T.grav * 8.6400e4 / (cpdair * 1.e2);
  // rrtmg_lw_rad.nomcica.f90:419-421
  T.oneminus = 1.0 - 1.e-6;
  T.fluxfac = (2.0 * std::asin(1.0)) * 2.e4;
}

// ---------------------------------------------------------------------------
// cldprop with separate ice and liquid parameterisations (inflag = 2),
// rrtmg_lw_cldprop.f90:185-270, for one layer whose optics are formed.
// Sets the layer's taucloud for cloud bands 1..ncbands, with ncbands the
// running value the reference keeps across its layer loop (1 at the start; 5
// after an iceflag = 1 ice cloud; 16 after an iceflag 2 / 3 ice cloud or a
// liqflag = 1 liquid cloud).  icb maps the 16 (or 5) cloud bands onto the
// coefficient bands of the parameterisation in use.  Returns false where the
// reference stops (an effective radius outside its table's range).
// ---------------------------------------------------------------------------
static const int kIpat[16][3] = {{1, 1, 1},  {1, 2, 2},  {1, 3, 3},  {1, 3, 4},  {1, 3, 5},  {1, 4, 6},
                                 {1, 4, 7},  {1, 4, 8},  {1, 5, 9},  {1, 5, 10}, {1, 5, 11}, {1, 5, 12},
                                 {1, 5, 13}, {1, 5, 14}, {1, 5, 15}, {1, 5, 16}};  // ipat = icb (16, 0:2)

int lw_cloud_band(int iband, int ncbands) { return kIpat[iband - 1][ncbands == 1 ? 0 : ncbands == 5 ? 1 : 2]; }

bool lw_cldprop_phys(const LwInput& in, double ciwp, double clwp, double radice, double radliq, LwColumn& c,
                     int lay) {
  const LwTables& T = g_lw;
  double abscoice[17] = {0}, abscoliq[17] = {0};
  int iceind = 0, liqind = 0;
  if (ciwp == 0.0) {
    abscoice[1] = 0.0;
    iceind = 0;
  } else if (in.iceflag == 0) {
    if (radice < 10.0) return false;
    abscoice[1] = T.absice0(1) + T.absice0(2) / radice;
    iceind = 0;
  } else if (in.iceflag == 1) {
    if (radice < 13.0 || radice > 130.) return false;
    c.ncbands = 5;
    for (int ib = 1; ib <= 5; ++ib) abscoice[ib] = T.absice1(1, ib) + T.absice1(2, ib) / radice;
    iceind = 1;
  } else if (in.iceflag == 2) {
    if (radice < 5.0 || radice > 131.0) return false;
    c.ncbands = 16;
    const double factor = (radice - 2.) / 3.;
    int index = (int)factor;
    if (index == 43) index = 42;
    const double fint = factor - (double)index;
    for (int ib = 1; ib <= 16; ++ib)
      abscoice[ib] = T.absice2(index, ib) + fint * (T.absice2(index + 1, ib) - (T.absice2(index, ib)));
    iceind = 2;
  } else {
    if (radice < 5.0 || radice > 140.0) return false;
    c.ncbands = 16;
    const double factor = (radice - 2.) / 3.;
    int index = (int)factor;
    if (index == 46) index = 45;
    const double fint = factor - (double)index;
    for (int ib = 1; ib <= 16; ++ib)
      abscoice[ib] = T.absice3(index, ib) + fint * (T.absice3(index + 1, ib) - (T.absice3(index, ib)));
    iceind = 2;
  }
  if (clwp == 0.0) {
    abscoliq[1] = 0.0;
    liqind = 0;
    if (iceind == 1) iceind = 2;
  } else if (in.liqflag == 0) {
    abscoliq[1] = T.absliq0;
    liqind = 0;
    if (iceind == 1) iceind = 2;
  } else {
    if (radliq < 2.5 || radliq > 60.) return false;
    int index = (int)(radliq - 1.5);
    if (index == 0) index = 1;
    if (index == 58) index = 57;
    const double fint = radliq - 1.5 - (double)index;
    c.ncbands = 16;
    for (int ib = 1; ib <= 16; ++ib)
      abscoliq[ib] = T.absliq1(index, ib) + fint * (T.absliq1(index + 1, ib) - (T.absliq1(index, ib)));
    liqind = 2;
  }
  for (int ib = 1; ib <= c.ncbands; ++ib)
    c.taucloud[ib][lay] = ciwp * abscoice[kIpat[ib - 1][iceind]] + clwp * abscoliq[kIpat[ib - 1][liqind]];
  return true;
}

// ---------------------------------------------------------------------------
// McICA's cloud inputs and cldprmc (rrtmg_lw_rad.f90 inatm :882-891,
// rrtmg_lw_cldprmc.f90): each g-point's sub-column cover, depth, ice and
// liquid water paths of a layer; with inflag = 2 the depth formed from the
// water paths by the parameterisations at the g-point's band ngb(ig) (the
// 5-band ice fit at icb(ngb(ig)) for iceflag = 1) where cover >= cldmin and
// water path or depth >= cldmin; inflag = 0 keeps the given depths; inflag
// = 1 stops (not available with McICA), as does a size outside its table.
// ---------------------------------------------------------------------------
static void lw_cldprmc(const LwInput& in, int iplon, LwColumn& c) {
  const LwTables& T = g_lw;
  const int nl = c.nlayers, L1 = nl + 1;
  const size_t N = (size_t)in.ncol;
  c.cldfmc.assign((size_t)140 * L1, 0.0);
  c.taucmc.assign((size_t)140 * L1, 0.0);
  int bandof[141];
  for (int b = 1, ig = 1; b <= 16; ++b)
    for (; ig <= T.ngs[b]; ++ig) bandof[ig] = b;
  const double cldmin = 1.e-20;
  for (int l = 1; l <= nl; ++l) {
    const size_t ol = (size_t)iplon + N * (size_t)(l - 1);
    const double radice = in.reicmcl ? in.reicmcl[ol] : 0.0, radliq = in.relqmcl ? in.relqmcl[ol] : 0.0;
    for (int ig = 1; ig <= 140; ++ig) {
      const size_t q = (size_t)(ig - 1) + 140 * ol;
      const double cf = in.cldfmcl[q], tau = in.taucmcl ? in.taucmcl[q] : 0.0;
      const double ciwp = in.ciwpmcl ? in.ciwpmcl[q] : 0.0, clwp = in.clwpmcl ? in.clwpmcl[q] : 0.0;
      const size_t k = (size_t)(ig - 1) * L1 + l;
      c.cldfmc[k] = cf;
      c.taucmc[k] = tau;
      if (!(cf >= cldmin && (ciwp + clwp >= cldmin || tau >= cldmin))) continue;
      if (in.inflag == 0) continue;
      if (in.inflag == 1) {
        c.cld_error = true;
        continue;
      }
      const int nb = bandof[ig];
      double abscoice = 0.0, abscoliq = 0.0;
      if (ciwp == 0.0) {
        abscoice = 0.0;
      } else if (in.iceflag == 0) {
        if (radice < 10.0) c.cld_error = true;
        abscoice = T.absice0(1) + T.absice0(2) / radice;
      } else if (in.iceflag == 1) {
        if (radice < 13.0 || radice > 130.) {
          c.cld_error = true;
          continue;
        }
        const int ib = kIpat[nb - 1][1];
        abscoice = T.absice1(1, ib) + T.absice1(2, ib) / radice;
      } else {
        const bool two = in.iceflag == 2;
        if (radice < 5.0 || radice > (two ? 131.0 : 140.0)) {
          c.cld_error = true;
          continue;
        }
        const double factor = (radice - 2.) / 3.;
        int index = (int)factor;
        if (index == (two ? 43 : 46)) index = two ? 42 : 45;
        const double fint = factor - (double)index;
        const FArr& t = two ? T.absice2 : T.absice3;
        abscoice = t(index, nb) + fint * (t(index + 1, nb) - (t(index, nb)));
      }
      if (clwp == 0.0) {
        abscoliq = 0.0;
      } else if (in.liqflag == 0) {
        abscoliq = T.absliq0;
      } else {
        if (radliq < 2.5 || radliq > 60.) {
          c.cld_error = true;
          continue;
        }
        int index = (int)(radliq - 1.5);
        if (index == 0) index = 1;
        if (index == 58) index = 57;
        const double fint = radliq - 1.5 - (double)index;
        abscoliq = T.absliq1(index, nb) + fint * (T.absliq1(index + 1, nb) - (T.absliq1(index, nb)));
      }
      c.taucmc[k] = ciwp * abscoice + clwp * abscoliq;
    }
  }
}

// ---------------------------------------------------------------------------
// inatm: rrtmg_lw_rad.nomcica.f90:572-901 (MiMA: h2ovmr carries specific
// humidity, o3vmr carries the O3 mass mixing ratio, :775-778)
// ---------------------------------------------------------------------------
void lw_inatm(const LwInput& in, int iplon, LwColumn& c) {
  const double amd = 28.9660, amw = 18.0160, amdw = 1.607793, amdo = 0.603428;
  const int nlay = in.nlay, ncol = in.ncol;
  auto A = [&](const double* p, int l) { return p[(size_t)iplon + (size_t)ncol * (size_t)(l - 1)]; };
  c.nlayers = nlay;
  c.resize(nlay);
  double amttl = 0.0, wvttl = 0.0;
  c.tbound = in.tsfc[iplon];
  c.pz[0] = A(in.plev, 1);
  c.tz[0] = A(in.tlev, 1);
  for (int l = 1; l <= nlay; ++l) {
    c.pavel[l] = A(in.play, l);
    c.tavel[l] = A(in.tlay, l);
    c.pz[l] = A(in.plev, l + 1);
    c.tz[l] = A(in.tlev, l + 1);
    double h2o = A(in.h2ovmr, l);
    c.wkl[1][l] = (h2o / (1.0 - h2o)) * amdw;
    c.wkl[2][l] = A(in.co2vmr, l);
    c.wkl[3][l] = A(in.o3vmr, l) * amdo;
    c.wkl[4][l] = in.n2ovmr ? A(in.n2ovmr, l) : 0.0;
    c.wkl[5][l] = 0.0;
    c.wkl[6][l] = in.ch4vmr ? A(in.ch4vmr, l) : 0.0;
    c.wkl[7][l] = in.o2vmr ? A(in.o2vmr, l) : 0.0;
    double amm = (1.0 - c.wkl[1][l]) * amd + c.wkl[1][l] * amw;
    c.coldry[l] = (c.pz[l - 1] - c.pz[l]) * 1.e3 * g_lw.avogad /
                  (1.e2 * g_lw.grav * amm * (1.0 + c.wkl[1][l]));
  }
  for (int l = 1; l <= nlay; ++l) {
    c.wx[1][l] = in.ccl4vmr ? A(in.ccl4vmr, l) : 0.0;
    c.wx[2][l] = in.cfc11vmr ? A(in.cfc11vmr, l) : 0.0;
    c.wx[3][l] = in.cfc12vmr ? A(in.cfc12vmr, l) : 0.0;
    c.wx[4][l] = in.cfc22vmr ? A(in.cfc22vmr, l) : 0.0;
  }
  for (int l = 1; l <= nlay; ++l) {
    double summol = 0.0;
    for (int imol = 2; imol <= 7; ++imol) summol = summol + c.wkl[imol][l];
    c.wbrodl[l] = c.coldry[l] * (1.0 - summol);
    for (int imol = 1; imol <= 7; ++imol) c.wkl[imol][l] = c.coldry[l] * c.wkl[imol][l];
    amttl = amttl + c.coldry[l] + c.wkl[1][l];
    wvttl = wvttl + c.wkl[1][l];
    for (int ix = 1; ix <= 4; ++ix)  // ixindx(ix) = ix (lwdatinit)
      c.wx[ix][l] = c.coldry[l] * c.wx[ix][l] * 1.e-20;
  }
  double wvsh = (amw * wvttl) / (amd * amttl);
  c.pwvcm = wvsh * (1.e3 * c.pz[0]) / (1.e2 * g_lw.grav);
  for (int n = 1; n <= 16; ++n) c.semiss[n] = in.emis ? in.emis[(size_t)iplon + (size_t)ncol * (size_t)(n - 1)] : 1.0;
  for (int l = 1; l <= nlay; ++l)
    for (int ib = 1; ib <= 16; ++ib)
      c.taua[ib][l] = in.tauaer ? in.tauaer[(size_t)iplon + (size_t)ncol * ((size_t)(l - 1) + (size_t)nlay * (size_t)(ib - 1))] : 0.0;
  // Clouds (:866-888): cldfrac(l) = cldfr(iplon,l), tauc(n,l) = taucld(n,iplon,l);
  // then cldprop (rrtmg_lw_cldprop.f90:155-270): a layer's cloud optical
  // depths are formed when cldfrac >= cldmin and the condensed water path or
  // the band-summed optical depth is >= cldmin (1e-20), else they are 0.
  c.ncbands = 1;
  c.cld_error = false;
  c.mcica = in.mcica && in.icld >= 1;
  if (c.mcica) {
    lw_cldprmc(in, iplon, c);
  } else if (in.icld >= 1) {
    const double cldmin = 1.e-20;
    for (int l = 1; l <= nlay; ++l) {
      const size_t o = (size_t)iplon + (size_t)ncol * (size_t)(l - 1);
      c.cldfrac[l] = in.cldfr[o];
      double tauctot = 0.0;
      for (int ib = 1; ib <= 16; ++ib) tauctot = tauctot + (in.taucld ? in.taucld[(size_t)(ib - 1) + 16 * o] : 0.0);
      const double ciwp = in.cicewp ? in.cicewp[o] : 0.0, clwp = in.cliqwp ? in.cliqwp[o] : 0.0;
      const double cwp = ciwp + clwp;
      for (int ib = 1; ib <= 16; ++ib) c.taucloud[ib][l] = 0.0;
      if (!(c.cldfrac[l] >= cldmin && (cwp >= cldmin || tauctot >= cldmin))) continue;
      if (in.inflag == 0) {
        c.ncbands = 16;
        for (int ib = 1; ib <= 16; ++ib) c.taucloud[ib][l] = in.taucld[(size_t)(ib - 1) + 16 * o];
      } else if (in.inflag == 1) {
        c.ncbands = 16;
        for (int ib = 1; ib <= 16; ++ib) c.taucloud[ib][l] = g_lw.abscld1 * cwp;
      } else {
        if (!lw_cldprop_phys(in, ciwp, clwp, in.reice ? in.reice[o] : 0.0, in.reliq ? in.reliq[o] : 0.0, c, l))
          c.cld_error = true;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// setcoef: rrtmg_lw_setcoef.f90:31-415 (istart = 1)
// ---------------------------------------------------------------------------
static inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

void lw_setcoef(LwColumn& c, int idrv) {
  const LwTables& T = g_lw;
  const double stpfac = 296. / 1013.;
  int indbound = (int)(c.tbound - 159.);
  indbound = clampi(indbound, 1, 180);
  double tbndfrac = c.tbound - 159. - (double)indbound;
  int indlev0 = (int)(c.tz[0] - 159.);
  indlev0 = clampi(indlev0, 1, 180);
  double t0frac = c.tz[0] - 159. - (double)indlev0;
  c.laytrop = 0;
  for (int lay = 1; lay <= c.nlayers; ++lay) {
    int indlay = clampi((int)(c.tavel[lay] - 159.), 1, 180);
    double tlayfrac = c.tavel[lay] - 159. - (double)indlay;
    int indlev = clampi((int)(c.tz[lay] - 159.), 1, 180);
    double tlevfrac = c.tz[lay] - 159. - (double)indlev;
    for (int iband = 1; iband <= 15; ++iband) {
      if (lay == 1) {
        double dbdtlev = T.totplnk(indbound + 1, iband) - T.totplnk(indbound, iband);
        c.plankbnd[iband] = c.semiss[iband] * (T.totplnk(indbound, iband) + tbndfrac * dbdtlev);
        dbdtlev = T.totplnk(indlev0 + 1, iband) - T.totplnk(indlev0, iband);
        c.planklev[iband][0] = T.totplnk(indlev0, iband) + t0frac * dbdtlev;
        if (idrv == 1) {
          dbdtlev = T.totplnkderiv(indbound + 1, iband) - T.totplnkderiv(indbound, iband);
          c.dplankbnd_dt[iband] = c.semiss[iband] * (T.totplnkderiv(indbound, iband) + tbndfrac * dbdtlev);
        }
      }
      double dbdtlev = T.totplnk(indlev + 1, iband) - T.totplnk(indlev, iband);
      double dbdtlay = T.totplnk(indlay + 1, iband) - T.totplnk(indlay, iband);
      c.planklay[iband][lay] = T.totplnk(indlay, iband) + tlayfrac * dbdtlay;
      c.planklev[iband][lay] = T.totplnk(indlev, iband) + tlevfrac * dbdtlev;
    }
    // band 16, istart /= 16 branch (:214-231)
    {
      const int iband = 16;
      if (lay == 1) {
        double dbdtlev = T.totplnk(indbound + 1, iband) - T.totplnk(indbound, iband);
        c.plankbnd[iband] = c.semiss[iband] * (T.totplnk(indbound, iband) + tbndfrac * dbdtlev);
        if (idrv == 1) {
          dbdtlev = T.totplnkderiv(indbound + 1, iband) - T.totplnkderiv(indbound, iband);
          c.dplankbnd_dt[iband] = c.semiss[iband] * (T.totplnkderiv(indbound, iband) + tbndfrac * dbdtlev);
        }
        dbdtlev = T.totplnk(indlev0 + 1, iband) - T.totplnk(indlev0, iband);
        c.planklev[iband][0] = T.totplnk(indlev0, iband) + t0frac * dbdtlev;
      }
      double dbdtlev = T.totplnk(indlev + 1, iband) - T.totplnk(indlev, iband);
      double dbdtlay = T.totplnk(indlay + 1, iband) - T.totplnk(indlay, iband);
      c.planklay[iband][lay] = T.totplnk(indlay, iband) + tlayfrac * dbdtlay;
      c.planklev[iband][lay] = T.totplnk(indlev, iband) + tlevfrac * dbdtlev;
    }

    double plog = std::log(c.pavel[lay]);
    int jp = (int)(36. - 5 * (plog + 0.04));
    jp = clampi(jp, 1, 58);
    c.jp[lay] = jp;
    int jp1 = jp + 1;
    double fp = 5. * (T.preflog(jp) - plog);
    int jt = clampi((int)(3. + (c.tavel[lay] - T.tref(jp)) / 15.), 1, 4);
    c.jt[lay] = jt;
    double ft = ((c.tavel[lay] - T.tref(jp)) / 15.) - (double)(jt - 3);
    int jt1 = clampi((int)(3. + (c.tavel[lay] - T.tref(jp1)) / 15.), 1, 4);
    c.jt1[lay] = jt1;
    double ft1 = ((c.tavel[lay] - T.tref(jp1)) / 15.) - (double)(jt1 - 3);
    double water = c.wkl[1][lay] / c.coldry[lay];
    double scalefac = c.pavel[lay] * stpfac / c.tavel[lay];

    auto cols = [&]() {
      c.colh2o[lay] = 1.e-20 * c.wkl[1][lay];
      c.colco2[lay] = 1.e-20 * c.wkl[2][lay];
      c.colo3[lay] = 1.e-20 * c.wkl[3][lay];
      c.coln2o[lay] = 1.e-20 * c.wkl[4][lay];
      c.colco[lay] = 1.e-20 * c.wkl[5][lay];
      c.colch4[lay] = 1.e-20 * c.wkl[6][lay];
      c.colo2[lay] = 1.e-20 * c.wkl[7][lay];
      if (c.colco2[lay] == 0.) c.colco2[lay] = 1.e-32 * c.coldry[lay];
      if (c.colo3[lay] == 0.) c.colo3[lay] = 1.e-32 * c.coldry[lay];
      if (c.coln2o[lay] == 0.) c.coln2o[lay] = 1.e-32 * c.coldry[lay];
      if (c.colco[lay] == 0.) c.colco[lay] = 1.e-32 * c.coldry[lay];
      if (c.colch4[lay] == 0.) c.colch4[lay] = 1.e-32 * c.coldry[lay];
      c.colbrd[lay] = 1.e-20 * c.wbrodl[lay];
    };
    const FArr& chi = T.chi_mls;
    if (plog > 4.56) {
      c.laytrop = c.laytrop + 1;
      c.forfac[lay] = scalefac / (1. + water);
      double factor = (332.0 - c.tavel[lay]) / 36.0;
      c.indfor[lay] = std::min(2, std::max(1, (int)factor));
      c.forfrac[lay] = factor - (double)c.indfor[lay];
      c.selffac[lay] = water * c.forfac[lay];
      factor = (c.tavel[lay] - 188.0) / 7.2;
      c.indself[lay] = std::min(9, std::max(1, (int)factor - 7));
      c.selffrac[lay] = factor - (double)(c.indself[lay] + 7);
      c.scaleminor[lay] = c.pavel[lay] / c.tavel[lay];
      c.scaleminorn2[lay] = (c.pavel[lay] / c.tavel[lay]) * (c.wbrodl[lay] / (c.coldry[lay] + c.wkl[1][lay]));
      factor = (c.tavel[lay] - 180.8) / 7.2;
      c.indminor[lay] = std::min(18, std::max(1, (int)factor));
      c.minorfrac[lay] = factor - (double)c.indminor[lay];
      c.rat_h2oco2[lay] = chi(1, jp) / chi(2, jp);
      c.rat_h2oco2_1[lay] = chi(1, jp + 1) / chi(2, jp + 1);
      c.rat_h2oo3[lay] = chi(1, jp) / chi(3, jp);
      c.rat_h2oo3_1[lay] = chi(1, jp + 1) / chi(3, jp + 1);
      c.rat_h2on2o[lay] = chi(1, jp) / chi(4, jp);
      c.rat_h2on2o_1[lay] = chi(1, jp + 1) / chi(4, jp + 1);
      c.rat_h2och4[lay] = chi(1, jp) / chi(6, jp);
      c.rat_h2och4_1[lay] = chi(1, jp + 1) / chi(6, jp + 1);
      c.rat_n2oco2[lay] = chi(4, jp) / chi(2, jp);
      c.rat_n2oco2_1[lay] = chi(4, jp + 1) / chi(2, jp + 1);
      cols();
    } else {
      c.forfac[lay] = scalefac / (1. + water);
      double factor = (c.tavel[lay] - 188.0) / 36.0;
      c.indfor[lay] = 3;
      c.forfrac[lay] = factor - 1.0;
      c.selffac[lay] = water * c.forfac[lay];
      c.scaleminor[lay] = c.pavel[lay] / c.tavel[lay];
      c.scaleminorn2[lay] = (c.pavel[lay] / c.tavel[lay]) * (c.wbrodl[lay] / (c.coldry[lay] + c.wkl[1][lay]));
      factor = (c.tavel[lay] - 180.8) / 7.2;
      c.indminor[lay] = std::min(18, std::max(1, (int)factor));
      c.minorfrac[lay] = factor - (double)c.indminor[lay];
      c.rat_h2oco2[lay] = chi(1, jp) / chi(2, jp);
      c.rat_h2oco2_1[lay] = chi(1, jp + 1) / chi(2, jp + 1);
      c.rat_o3co2[lay] = chi(3, jp) / chi(2, jp);
      c.rat_o3co2_1[lay] = chi(3, jp + 1) / chi(2, jp + 1);
      cols();
    }
    double compfp = 1. - fp;
    c.fac10[lay] = compfp * ft;
    c.fac00[lay] = compfp * (1. - ft);
    c.fac11[lay] = fp * ft1;
    c.fac01[lay] = fp * (1. - ft1);
    c.selffac[lay] = c.colh2o[lay] * c.selffac[lay];
    c.forfac[lay] = c.colh2o[lay] * c.forfac[lay];
  }
}

// ---------------------------------------------------------------------------
// taumol helpers (shared arithmetic of taugb3/4/5/7/9/12/13/15/16 lower loops)
// ---------------------------------------------------------------------------
struct Eta {
  double speccomb, specparm, fs;
  int js;
};

static inline Eta eta(double a, double ratb, double b, double mult) {
  Eta e;
  e.speccomb = a + ratb * b;
  e.specparm = a / e.speccomb;
  if (e.specparm >= g_lw.oneminus) e.specparm = g_lw.oneminus;
  double specmult = mult * (e.specparm);
  e.js = 1 + (int)specmult;
  e.fs = std::fmod(specmult, 1.0);
  return e;
}

// fac000..fac210 (or fac001..fac211) for one of the two pressure levels,
// taugb3 lower loop :560-620 pattern.
struct Fac3 {
  double f0a, f1a, f2a;  // x fac00 (or fac01)
  double f0b, f1b, f2b;  // x fac10 (or fac11)
};

static inline Fac3 fac3(double specparm, double fs, double facA, double facB) {
  Fac3 f{0, 0, 0, 0, 0, 0};
  if (specparm < 0.125) {
    double p = fs - 1;
    double p4 = (p * p) * (p * p);
    double fk0 = p4, fk1 = 1 - p - 2.0 * p4, fk2 = p + p4;
    f.f0a = fk0 * facA; f.f1a = fk1 * facA; f.f2a = fk2 * facA;
    f.f0b = fk0 * facB; f.f1b = fk1 * facB; f.f2b = fk2 * facB;
  } else if (specparm > 0.875) {
    double p = -fs;
    double p4 = (p * p) * (p * p);
    double fk0 = p4, fk1 = 1 - p - 2.0 * p4, fk2 = p + p4;
    f.f0a = fk0 * facA; f.f1a = fk1 * facA; f.f2a = fk2 * facA;
    f.f0b = fk0 * facB; f.f1b = fk1 * facB; f.f2b = fk2 * facB;
  } else {
    f.f0a = (1. - fs) * facA;
    f.f0b = (1. - fs) * facB;
    f.f1a = fs * facA;
    f.f1b = fs * facB;
  }
  return f;
}

// tau_major term for one pressure level (:641-690).
static inline double tau_major3(const FArr& absa, double specparm, double speccomb, int ind, int ig,
                                const Fac3& f) {
  if (specparm < 0.125) {
    return speccomb * (f.f0a * absa.flat(ind, ig) + f.f1a * absa.flat(ind + 1, ig) +
                       f.f2a * absa.flat(ind + 2, ig) + f.f0b * absa.flat(ind + 9, ig) +
                       f.f1b * absa.flat(ind + 10, ig) + f.f2b * absa.flat(ind + 11, ig));
  } else if (specparm > 0.875) {
    return speccomb * (f.f2a * absa.flat(ind - 1, ig) + f.f1a * absa.flat(ind, ig) +
                       f.f0a * absa.flat(ind + 1, ig) + f.f2b * absa.flat(ind + 8, ig) +
                       f.f1b * absa.flat(ind + 9, ig) + f.f0b * absa.flat(ind + 10, ig));
  }
  return speccomb * (f.f0a * absa.flat(ind, ig) + f.f1a * absa.flat(ind + 1, ig) +
                     f.f0b * absa.flat(ind + 9, ig) + f.f1b * absa.flat(ind + 10, ig));
}

// Upper-atmosphere eta-mixed major term (taugb3 :747-756 pattern, 5 eta levels).
static inline double tau_major_upper(const FArr& absb, double speccomb, double fs, int ind0,
                                     double speccomb1, double fs1, int ind1, const LwColumn& c,
                                     int lay, int ig) {
  double fac000 = (1. - fs) * c.fac00[lay];
  double fac010 = (1. - fs) * c.fac10[lay];
  double fac100 = fs * c.fac00[lay];
  double fac110 = fs * c.fac10[lay];
  double fac001 = (1. - fs1) * c.fac01[lay];
  double fac011 = (1. - fs1) * c.fac11[lay];
  double fac101 = fs1 * c.fac01[lay];
  double fac111 = fs1 * c.fac11[lay];
  return speccomb * (fac000 * absb.flat(ind0, ig) + fac100 * absb.flat(ind0 + 1, ig) +
                     fac010 * absb.flat(ind0 + 5, ig) + fac110 * absb.flat(ind0 + 6, ig)) +
         speccomb1 * (fac001 * absb.flat(ind1, ig) + fac101 * absb.flat(ind1 + 1, ig) +
                      fac011 * absb.flat(ind1 + 5, ig) + fac111 * absb.flat(ind1 + 6, ig));
}

static inline double interp4(const FArr& k, const LwColumn& c, int lay, int ind0, int ind1, int ig) {
  return c.fac00[lay] * k.flat(ind0, ig) + c.fac10[lay] * k.flat(ind0 + 1, ig) +
         c.fac01[lay] * k.flat(ind1, ig) + c.fac11[lay] * k.flat(ind1 + 1, ig);
}

static inline double tself(const FArr& selfref, const LwColumn& c, int lay, int ig) {
  int inds = c.indself[lay];
  return c.selffac[lay] * (selfref(inds, ig) + c.selffrac[lay] * (selfref(inds + 1, ig) - selfref(inds, ig)));
}
static inline double tfor(const FArr& forref, const LwColumn& c, int lay, int ig) {
  int indf = c.indfor[lay];
  return c.forfac[lay] * (forref(indf, ig) + c.forfrac[lay] * (forref(indf + 1, ig) - forref(indf, ig)));
}
// minor table interpolated in T only: k(indm,ig) + minorfrac*(k(indm+1,ig)-k(indm,ig))
static inline double minor1(const FArr& k, const LwColumn& c, int lay, int ig) {
  int indm = c.indminor[lay];
  return k(indm, ig) + c.minorfrac[lay] * (k(indm + 1, ig) - k(indm, ig));
}
// minor table interpolated in eta and T (taugb3 :624-629 pattern)
static inline double minor2(const FArr& k, int jm, double fm, const LwColumn& c, int lay, int ig) {
  int indm = c.indminor[lay];
  double m1 = k(jm, indm, ig) + fm * (k(jm + 1, indm, ig) - k(jm, indm, ig));
  double m2 = k(jm, indm + 1, ig) + fm * (k(jm + 1, indm + 1, ig) - k(jm, indm + 1, ig));
  return m1 + c.minorfrac[lay] * (m2 - m1);
}
static inline double fracs_eta(const FArr& fr, int jpl, double fpl, int ig) {
  return fr(ig, jpl) + fpl * (fr(ig, jpl + 1) - fr(ig, jpl));
}

// ---------------------------------------------------------------------------
// taumol: rrtmg_lw_taumol.f90 taugb1..16.  taug/fracs indexed [ig][lay]
// with ig the global g-point 1..140.
// ---------------------------------------------------------------------------
void lw_taumol(LwColumn& c) {
  const LwTables& T = g_lw;
  const FArr& chi = T.chi_mls;
  const int nl = c.nlayers, lt = c.laytrop;
  auto& taug = c.taug;
  auto& fracs = c.fracs;

  // ---- band 1 (:280-372)
  {
    auto& t = T.t[1];
    const FArr &absa = t.at("ka"), &absb = t.at("kb"), &selfref = t.at("selfref"),
               &forref = t.at("forref"), &kamn2 = t.at("ka_mn2"), &kbmn2 = t.at("kb_mn2"),
               &fra = t.at("fracrefa"), &frb = t.at("fracrefb");
    for (int lay = 1; lay <= lt; ++lay) {
      int ind0 = ((c.jp[lay] - 1) * 5 + (c.jt[lay] - 1)) * T.nspa[1] + 1;
      int ind1 = (c.jp[lay] * 5 + (c.jt1[lay] - 1)) * T.nspa[1] + 1;
      double pp = c.pavel[lay];
      double corradj = 1.;
      if (pp < 250.) corradj = 1. - 0.15 * (250. - pp) / 154.4;
      double scalen2 = c.colbrd[lay] * c.scaleminorn2[lay];
      for (int ig = 1; ig <= T.ngc[1]; ++ig) {
        double tauself = tself(selfref, c, lay, ig);
        double taufor = tfor(forref, c, lay, ig);
        double taun2 = scalen2 * minor1(kamn2, c, lay, ig);
        taug[ig][lay] = corradj * (c.colh2o[lay] * interp4(absa, c, lay, ind0, ind1, ig) + tauself + taufor + taun2);
        fracs[ig][lay] = fra(ig);
      }
    }
    for (int lay = lt + 1; lay <= nl; ++lay) {
      int ind0 = ((c.jp[lay] - 13) * 5 + (c.jt[lay] - 1)) * T.nspb[1] + 1;
      int ind1 = ((c.jp[lay] - 12) * 5 + (c.jt1[lay] - 1)) * T.nspb[1] + 1;
      double pp = c.pavel[lay];
      double corradj = 1. - 0.15 * (pp / 95.6);
      double scalen2 = c.colbrd[lay] * c.scaleminorn2[lay];
      for (int ig = 1; ig <= T.ngc[1]; ++ig) {
        double taufor = tfor(forref, c, lay, ig);
        double taun2 = scalen2 * minor1(kbmn2, c, lay, ig);
        taug[ig][lay] = corradj * (c.colh2o[lay] * interp4(absb, c, lay, ind0, ind1, ig) + taufor + taun2);
        fracs[ig][lay] = frb(ig);
      }
    }
  }
  // ---- band 2 (:375-450)
  {
    auto& t = T.t[2];
    const int o = T.ngs[1];
    const FArr &absa = t.at("ka"), &absb = t.at("kb"), &selfref = t.at("selfref"),
               &forref = t.at("forref"), &fra = t.at("fracrefa"), &frb = t.at("fracrefb");
    for (int lay = 1; lay <= lt; ++lay) {
      int ind0 = ((c.jp[lay] - 1) * 5 + (c.jt[lay] - 1)) * T.nspa[2] + 1;
      int ind1 = (c.jp[lay] * 5 + (c.jt1[lay] - 1)) * T.nspa[2] + 1;
      double pp = c.pavel[lay];
      double corradj = 1. - .05 * (pp - 100.) / 900.;
      for (int ig = 1; ig <= T.ngc[2]; ++ig) {
        double tauself = tself(selfref, c, lay, ig);
        double taufor = tfor(forref, c, lay, ig);
        taug[o + ig][lay] = corradj * (c.colh2o[lay] * interp4(absa, c, lay, ind0, ind1, ig) + tauself + taufor);
        fracs[o + ig][lay] = fra(ig);
      }
    }
    for (int lay = lt + 1; lay <= nl; ++lay) {
      int ind0 = ((c.jp[lay] - 13) * 5 + (c.jt[lay] - 1)) * T.nspb[2] + 1;
      int ind1 = ((c.jp[lay] - 12) * 5 + (c.jt1[lay] - 1)) * T.nspb[2] + 1;
      for (int ig = 1; ig <= T.ngc[2]; ++ig) {
        double taufor = tfor(forref, c, lay, ig);
        taug[o + ig][lay] = c.colh2o[lay] * interp4(absb, c, lay, ind0, ind1, ig) + taufor;
        fracs[o + ig][lay] = frb(ig);
      }
    }
  }
  // ---- band 3 (:453-771): h2o/co2, minor n2o
  {
    auto& t = T.t[3];
    const int o = T.ngs[2];
    const FArr &absa = t.at("ka"), &absb = t.at("kb"), &selfref = t.at("selfref"),
               &forref = t.at("forref"), &kamn2o = t.at("ka_mn2o"), &kbmn2o = t.at("kb_mn2o"),
               &fra = t.at("fracrefa"), &frb = t.at("fracrefb");
    double refrat_planck_a = chi(1, 9) / chi(2, 9);
    double refrat_planck_b = chi(1, 13) / chi(2, 13);
    double refrat_m_a = chi(1, 3) / chi(2, 3);
    double refrat_m_b = chi(1, 13) / chi(2, 13);
    for (int lay = 1; lay <= lt; ++lay) {
      Eta e = eta(c.colh2o[lay], c.rat_h2oco2[lay], c.colco2[lay], 8.);
      Eta e1 = eta(c.colh2o[lay], c.rat_h2oco2_1[lay], c.colco2[lay], 8.);
      Eta em = eta(c.colh2o[lay], refrat_m_a, c.colco2[lay], 8.);
      double chi_n2o = c.coln2o[lay] / c.coldry[lay];
      double ratn2o = 1.e20 * chi_n2o / chi(4, c.jp[lay] + 1);
      double adjcoln2o;
      if (ratn2o > 1.5) {
        double adjfac = 0.5 + std::pow(ratn2o - 0.5, 0.65);
        adjcoln2o = adjfac * chi(4, c.jp[lay] + 1) * c.coldry[lay] * 1.e-20;
      } else {
        adjcoln2o = c.coln2o[lay];
      }
      Eta ep = eta(c.colh2o[lay], refrat_planck_a, c.colco2[lay], 8.);
      int ind0 = ((c.jp[lay] - 1) * 5 + (c.jt[lay] - 1)) * T.nspa[3] + e.js;
      int ind1 = (c.jp[lay] * 5 + (c.jt1[lay] - 1)) * T.nspa[3] + e1.js;
      Fac3 f0 = fac3(e.specparm, e.fs, c.fac00[lay], c.fac10[lay]);
      Fac3 f1 = fac3(e1.specparm, e1.fs, c.fac01[lay], c.fac11[lay]);
      for (int ig = 1; ig <= T.ngc[3]; ++ig) {
        double tauself = tself(selfref, c, lay, ig);
        double taufor = tfor(forref, c, lay, ig);
        double absn2o = minor2(kamn2o, em.js, em.fs, c, lay, ig);
        double tau_major = tau_major3(absa, e.specparm, e.speccomb, ind0, ig, f0);
        double tau_major1 = tau_major3(absa, e1.specparm, e1.speccomb, ind1, ig, f1);
        taug[o + ig][lay] = tau_major + tau_major1 + tauself + taufor + adjcoln2o * absn2o;
        fracs[o + ig][lay] = fracs_eta(fra, ep.js, ep.fs, ig);
      }
    }
    for (int lay = lt + 1; lay <= nl; ++lay) {
      Eta e = eta(c.colh2o[lay], c.rat_h2oco2[lay], c.colco2[lay], 4.);
      Eta e1 = eta(c.colh2o[lay], c.rat_h2oco2_1[lay], c.colco2[lay], 4.);
      Eta em = eta(c.colh2o[lay], refrat_m_b, c.colco2[lay], 4.);
      double chi_n2o = c.coln2o[lay] / c.coldry[lay];
      double ratn2o = 1.e20 * chi_n2o / chi(4, c.jp[lay] + 1);
      double adjcoln2o;
      if (ratn2o > 1.5) {
        double adjfac = 0.5 + std::pow(ratn2o - 0.5, 0.65);
        adjcoln2o = adjfac * chi(4, c.jp[lay] + 1) * c.coldry[lay] * 1.e-20;
      } else {
        adjcoln2o = c.coln2o[lay];
      }
      Eta ep = eta(c.colh2o[lay], refrat_planck_b, c.colco2[lay], 4.);
      int ind0 = ((c.jp[lay] - 13) * 5 + (c.jt[lay] - 1)) * T.nspb[3] + e.js;
      int ind1 = ((c.jp[lay] - 12) * 5 + (c.jt1[lay] - 1)) * T.nspb[3] + e1.js;
      for (int ig = 1; ig <= T.ngc[3]; ++ig) {
        double taufor = tfor(forref, c, lay, ig);
        double absn2o = minor2(kbmn2o, em.js, em.fs, c, lay, ig);
        taug[o + ig][lay] = tau_major_upper(absb, e.speccomb, e.fs, ind0, e1.speccomb, e1.fs, ind1, c, lay, ig) +
                            taufor + adjcoln2o * absn2o;
        fracs[o + ig][lay] = fracs_eta(frb, ep.js, ep.fs, ig);
      }
    }
  }
  // ---- band 4 (:774-1002): lower h2o/co2, upper o3/co2
  {
    auto& t = T.t[4];
    const int o = T.ngs[3];
    const FArr &absa = t.at("ka"), &absb = t.at("kb"), &selfref = t.at("selfref"),
               &forref = t.at("forref"), &fra = t.at("fracrefa"), &frb = t.at("fracrefb");
    double refrat_planck_a = chi(1, 11) / chi(2, 11);
    double refrat_planck_b = chi(3, 13) / chi(2, 13);
    for (int lay = 1; lay <= lt; ++lay) {
      Eta e = eta(c.colh2o[lay], c.rat_h2oco2[lay], c.colco2[lay], 8.);
      Eta e1 = eta(c.colh2o[lay], c.rat_h2oco2_1[lay], c.colco2[lay], 8.);
      Eta ep = eta(c.colh2o[lay], refrat_planck_a, c.colco2[lay], 8.);
      int ind0 = ((c.jp[lay] - 1) * 5 + (c.jt[lay] - 1)) * T.nspa[4] + e.js;
      int ind1 = (c.jp[lay] * 5 + (c.jt1[lay] - 1)) * T.nspa[4] + e1.js;
      Fac3 f0 = fac3(e.specparm, e.fs, c.fac00[lay], c.fac10[lay]);
      Fac3 f1 = fac3(e1.specparm, e1.fs, c.fac01[lay], c.fac11[lay]);
      for (int ig = 1; ig <= T.ngc[4]; ++ig) {
        double tauself = tself(selfref, c, lay, ig);
        double taufor = tfor(forref, c, lay, ig);
        double tau_major = tau_major3(absa, e.specparm, e.speccomb, ind0, ig, f0);
        double tau_major1 = tau_major3(absa, e1.specparm, e1.speccomb, ind1, ig, f1);
        taug[o + ig][lay] = tau_major + tau_major1 + tauself + taufor;
        fracs[o + ig][lay] = fracs_eta(fra, ep.js, ep.fs, ig);
      }
    }
    for (int lay = lt + 1; lay <= nl; ++lay) {
      Eta e = eta(c.colo3[lay], c.rat_o3co2[lay], c.colco2[lay], 4.);
      Eta e1 = eta(c.colo3[lay], c.rat_o3co2_1[lay], c.colco2[lay], 4.);
      Eta ep = eta(c.colo3[lay], refrat_planck_b, c.colco2[lay], 4.);
      int ind0 = ((c.jp[lay] - 13) * 5 + (c.jt[lay] - 1)) * T.nspb[4] + e.js;
      int ind1 = ((c.jp[lay] - 12) * 5 + (c.jt1[lay] - 1)) * T.nspb[4] + e1.js;
      for (int ig = 1; ig <= T.ngc[4]; ++ig) {
        taug[o + ig][lay] = tau_major_upper(absb, e.speccomb, e.fs, ind0, e1.speccomb, e1.fs, ind1, c, lay, ig);
        fracs[o + ig][lay] = fracs_eta(frb, ep.js, ep.fs, ig);
      }
      // Empirical upper-atmosphere scalings (:994-1000)
      taug[o + 8][lay] = taug[o + 8][lay] * 0.92;
      taug[o + 9][lay] = taug[o + 9][lay] * 0.88;
      taug[o + 10][lay] = taug[o + 10][lay] * 1.07;
      taug[o + 11][lay] = taug[o + 11][lay] * 1.1;
      taug[o + 12][lay] = taug[o + 12][lay] * 0.99;
      taug[o + 13][lay] = taug[o + 13][lay] * 0.88;
      taug[o + 14][lay] = taug[o + 14][lay] * 0.943;
    }
  }
  // ---- band 5 (:1005-1293): lower h2o/co2 + minor o3 + ccl4, upper o3/co2 + ccl4
  {
    auto& t = T.t[5];
    const int o = T.ngs[4];
    const FArr &absa = t.at("ka"), &absb = t.at("kb"), &selfref = t.at("selfref"),
               &forref = t.at("forref"), &kamo3 = t.at("ka_mo3"), &ccl4 = t.at("ccl4"),
               &fra = t.at("fracrefa"), &frb = t.at("fracrefb");
    double refrat_planck_a = chi(1, 5) / chi(2, 5);
    double refrat_planck_b = chi(3, 43) / chi(2, 43);
    double refrat_m_a = chi(1, 7) / chi(2, 7);
    for (int lay = 1; lay <= lt; ++lay) {
      Eta e = eta(c.colh2o[lay], c.rat_h2oco2[lay], c.colco2[lay], 8.);
      Eta e1 = eta(c.colh2o[lay], c.rat_h2oco2_1[lay], c.colco2[lay], 8.);
      Eta em = eta(c.colh2o[lay], refrat_m_a, c.colco2[lay], 8.);
      Eta ep = eta(c.colh2o[lay], refrat_planck_a, c.colco2[lay], 8.);
      int ind0 = ((c.jp[lay] - 1) * 5 + (c.jt[lay] - 1)) * T.nspa[5] + e.js;
      int ind1 = (c.jp[lay] * 5 + (c.jt1[lay] - 1)) * T.nspa[5] + e1.js;
      Fac3 f0 = fac3(e.specparm, e.fs, c.fac00[lay], c.fac10[lay]);
      Fac3 f1 = fac3(e1.specparm, e1.fs, c.fac01[lay], c.fac11[lay]);
      for (int ig = 1; ig <= T.ngc[5]; ++ig) {
        double tauself = tself(selfref, c, lay, ig);
        double taufor = tfor(forref, c, lay, ig);
        double abso3 = minor2(kamo3, em.js, em.fs, c, lay, ig);
        double tau_major = tau_major3(absa, e.specparm, e.speccomb, ind0, ig, f0);
        double tau_major1 = tau_major3(absa, e1.specparm, e1.speccomb, ind1, ig, f1);
        taug[o + ig][lay] = tau_major + tau_major1 + tauself + taufor + abso3 * c.colo3[lay] + c.wx[1][lay] * ccl4(ig);
        fracs[o + ig][lay] = fracs_eta(fra, ep.js, ep.fs, ig);
      }
    }
    for (int lay = lt + 1; lay <= nl; ++lay) {
      Eta e = eta(c.colo3[lay], c.rat_o3co2[lay], c.colco2[lay], 4.);
      Eta e1 = eta(c.colo3[lay], c.rat_o3co2_1[lay], c.colco2[lay], 4.);
      Eta ep = eta(c.colo3[lay], refrat_planck_b, c.colco2[lay], 4.);
      int ind0 = ((c.jp[lay] - 13) * 5 + (c.jt[lay] - 1)) * T.nspb[5] + e.js;
      int ind1 = ((c.jp[lay] - 12) * 5 + (c.jt1[lay] - 1)) * T.nspb[5] + e1.js;
      for (int ig = 1; ig <= T.ngc[5]; ++ig) {
        taug[o + ig][lay] = tau_major_upper(absb, e.speccomb, e.fs, ind0, e1.speccomb, e1.fs, ind1, c, lay, ig) +
                            c.wx[1][lay] * ccl4(ig);
        fracs[o + ig][lay] = fracs_eta(frb, ep.js, ep.fs, ig);
      }
    }
  }
  // ---- band 6 (:1296-1371): h2o + minor co2 + cfc11/cfc12
  {
    auto& t = T.t[6];
    const int o = T.ngs[5];
    const FArr &absa = t.at("ka"), &selfref = t.at("selfref"), &forref = t.at("forref"),
               &kamco2 = t.at("ka_mco2"), &cfc11adj = t.at("cfc11adj"), &cfc12 = t.at("cfc12"),
               &fra = t.at("fracrefa");
    for (int lay = 1; lay <= lt; ++lay) {
      double chi_co2 = c.colco2[lay] / (c.coldry[lay]);
      double ratco2 = 1.e20 * chi_co2 / chi(2, c.jp[lay] + 1);
      double adjcolco2;
      if (ratco2 > 3.0) {
        double adjfac = 2.0 + std::pow(ratco2 - 2.0, 0.77);
        adjcolco2 = adjfac * chi(2, c.jp[lay] + 1) * c.coldry[lay] * 1.e-20;
      } else {
        adjcolco2 = c.colco2[lay];
      }
      int ind0 = ((c.jp[lay] - 1) * 5 + (c.jt[lay] - 1)) * T.nspa[6] + 1;
      int ind1 = (c.jp[lay] * 5 + (c.jt1[lay] - 1)) * T.nspa[6] + 1;
      for (int ig = 1; ig <= T.ngc[6]; ++ig) {
        double tauself = tself(selfref, c, lay, ig);
        double taufor = tfor(forref, c, lay, ig);
        double absco2 = (minor1(kamco2, c, lay, ig));
        taug[o + ig][lay] = c.colh2o[lay] * interp4(absa, c, lay, ind0, ind1, ig) + tauself + taufor +
                            adjcolco2 * absco2 + c.wx[2][lay] * cfc11adj(ig) + c.wx[3][lay] * cfc12(ig);
        fracs[o + ig][lay] = fra(ig);
      }
    }
    for (int lay = lt + 1; lay <= nl; ++lay) {
      for (int ig = 1; ig <= T.ngc[6]; ++ig) {
        taug[o + ig][lay] = 0.0 + c.wx[2][lay] * cfc11adj(ig) + c.wx[3][lay] * cfc12(ig);
        fracs[o + ig][lay] = fra(ig);
      }
    }
  }
  // ---- band 7 (:1374-1604): lower h2o/o3 + minor co2, upper o3 + minor co2
  {
    auto& t = T.t[7];
    const int o = T.ngs[6];
    const FArr &absa = t.at("ka"), &absb = t.at("kb"), &selfref = t.at("selfref"),
               &forref = t.at("forref"), &kamco2 = t.at("ka_mco2"), &kbmco2 = t.at("kb_mco2"),
               &fra = t.at("fracrefa"), &frb = t.at("fracrefb");
    double refrat_planck_a = chi(1, 3) / chi(3, 3);
    double refrat_m_a = chi(1, 3) / chi(3, 3);
    for (int lay = 1; lay <= lt; ++lay) {
      Eta e = eta(c.colh2o[lay], c.rat_h2oo3[lay], c.colo3[lay], 8.);
      Eta e1 = eta(c.colh2o[lay], c.rat_h2oo3_1[lay], c.colo3[lay], 8.);
      Eta em = eta(c.colh2o[lay], refrat_m_a, c.colo3[lay], 8.);
      double chi_co2 = c.colco2[lay] / (c.coldry[lay]);
      double ratco2 = 1.e20 * chi_co2 / chi(2, c.jp[lay] + 1);
      double adjcolco2;
      if (ratco2 > 3.0) {
        double adjfac = 3.0 + std::pow(ratco2 - 3.0, 0.79);
        adjcolco2 = adjfac * chi(2, c.jp[lay] + 1) * c.coldry[lay] * 1.e-20;
      } else {
        adjcolco2 = c.colco2[lay];
      }
      Eta ep = eta(c.colh2o[lay], refrat_planck_a, c.colo3[lay], 8.);
      int ind0 = ((c.jp[lay] - 1) * 5 + (c.jt[lay] - 1)) * T.nspa[7] + e.js;
      int ind1 = (c.jp[lay] * 5 + (c.jt1[lay] - 1)) * T.nspa[7] + e1.js;
      Fac3 f0 = fac3(e.specparm, e.fs, c.fac00[lay], c.fac10[lay]);
      Fac3 f1 = fac3(e1.specparm, e1.fs, c.fac01[lay], c.fac11[lay]);
      for (int ig = 1; ig <= T.ngc[7]; ++ig) {
        double tauself = tself(selfref, c, lay, ig);
        double taufor = tfor(forref, c, lay, ig);
        double absco2 = minor2(kamco2, em.js, em.fs, c, lay, ig);
        double tau_major = tau_major3(absa, e.specparm, e.speccomb, ind0, ig, f0);
        double tau_major1 = tau_major3(absa, e1.specparm, e1.speccomb, ind1, ig, f1);
        taug[o + ig][lay] = tau_major + tau_major1 + tauself + taufor + adjcolco2 * absco2;
        fracs[o + ig][lay] = fracs_eta(fra, ep.js, ep.fs, ig);
      }
    }
    for (int lay = lt + 1; lay <= nl; ++lay) {
      double chi_co2 = c.colco2[lay] / (c.coldry[lay]);
      double ratco2 = 1.e20 * chi_co2 / chi(2, c.jp[lay] + 1);
      double adjcolco2;
      if (ratco2 > 3.0) {
        double adjfac = 2.0 + std::pow(ratco2 - 2.0, 0.79);
        adjcolco2 = adjfac * chi(2, c.jp[lay] + 1) * c.coldry[lay] * 1.e-20;
      } else {
        adjcolco2 = c.colco2[lay];
      }
      int ind0 = ((c.jp[lay] - 13) * 5 + (c.jt[lay] - 1)) * T.nspb[7] + 1;
      int ind1 = ((c.jp[lay] - 12) * 5 + (c.jt1[lay] - 1)) * T.nspb[7] + 1;
      for (int ig = 1; ig <= T.ngc[7]; ++ig) {
        double absco2 = minor1(kbmco2, c, lay, ig);
        taug[o + ig][lay] = c.colo3[lay] * interp4(absb, c, lay, ind0, ind1, ig) + adjcolco2 * absco2;
        fracs[o + ig][lay] = frb(ig);
      }
      taug[o + 6][lay] = taug[o + 6][lay] * 0.92;
      taug[o + 7][lay] = taug[o + 7][lay] * 0.88;
      taug[o + 8][lay] = taug[o + 8][lay] * 1.07;
      taug[o + 9][lay] = taug[o + 9][lay] * 1.1;
      taug[o + 10][lay] = taug[o + 10][lay] * 0.99;
      taug[o + 11][lay] = taug[o + 11][lay] * 0.855;
    }
  }
  // ---- band 8 (:1607-1721): h2o, minors co2/o3/n2o, cfc12/cfc22
  {
    auto& t = T.t[8];
    const int o = T.ngs[7];
    const FArr &absa = t.at("ka"), &absb = t.at("kb"), &selfref = t.at("selfref"),
               &forref = t.at("forref"), &kamco2 = t.at("ka_mco2"), &kamo3 = t.at("ka_mo3"),
               &kamn2o = t.at("ka_mn2o"), &kbmco2 = t.at("kb_mco2"), &kbmn2o = t.at("kb_mn2o"),
               &cfc12 = t.at("cfc12"), &cfc22adj = t.at("cfc22adj"), &fra = t.at("fracrefa"),
               &frb = t.at("fracrefb");
    for (int lay = 1; lay <= lt; ++lay) {
      double chi_co2 = c.colco2[lay] / (c.coldry[lay]);
      double ratco2 = 1.e20 * chi_co2 / chi(2, c.jp[lay] + 1);
      double adjcolco2;
      if (ratco2 > 3.0) {
        double adjfac = 2.0 + std::pow(ratco2 - 2.0, 0.65);
        adjcolco2 = adjfac * chi(2, c.jp[lay] + 1) * c.coldry[lay] * 1.e-20;
      } else {
        adjcolco2 = c.colco2[lay];
      }
      int ind0 = ((c.jp[lay] - 1) * 5 + (c.jt[lay] - 1)) * T.nspa[8] + 1;
      int ind1 = (c.jp[lay] * 5 + (c.jt1[lay] - 1)) * T.nspa[8] + 1;
      for (int ig = 1; ig <= T.ngc[8]; ++ig) {
        double tauself = tself(selfref, c, lay, ig);
        double taufor = tfor(forref, c, lay, ig);
        double absco2 = (minor1(kamco2, c, lay, ig));
        double abso3 = (minor1(kamo3, c, lay, ig));
        double absn2o = (minor1(kamn2o, c, lay, ig));
        taug[o + ig][lay] = c.colh2o[lay] * interp4(absa, c, lay, ind0, ind1, ig) + tauself + taufor +
                            adjcolco2 * absco2 + c.colo3[lay] * abso3 + c.coln2o[lay] * absn2o +
                            c.wx[3][lay] * cfc12(ig) + c.wx[4][lay] * cfc22adj(ig);
        fracs[o + ig][lay] = fra(ig);
      }
    }
    for (int lay = lt + 1; lay <= nl; ++lay) {
      double chi_co2 = c.colco2[lay] / c.coldry[lay];
      double ratco2 = 1.e20 * chi_co2 / chi(2, c.jp[lay] + 1);
      double adjcolco2;
      if (ratco2 > 3.0) {
        double adjfac = 2.0 + std::pow(ratco2 - 2.0, 0.65);
        adjcolco2 = adjfac * chi(2, c.jp[lay] + 1) * c.coldry[lay] * 1.e-20;
      } else {
        adjcolco2 = c.colco2[lay];
      }
      int ind0 = ((c.jp[lay] - 13) * 5 + (c.jt[lay] - 1)) * T.nspb[8] + 1;
      int ind1 = ((c.jp[lay] - 12) * 5 + (c.jt1[lay] - 1)) * T.nspb[8] + 1;
      for (int ig = 1; ig <= T.ngc[8]; ++ig) {
        double absco2 = (minor1(kbmco2, c, lay, ig));
        double absn2o = (minor1(kbmn2o, c, lay, ig));
        taug[o + ig][lay] = c.colo3[lay] * interp4(absb, c, lay, ind0, ind1, ig) + adjcolco2 * absco2 +
                            c.coln2o[lay] * absn2o + c.wx[3][lay] * cfc12(ig) + c.wx[4][lay] * cfc22adj(ig);
        fracs[o + ig][lay] = frb(ig);
      }
    }
  }
  // ---- band 9 (:1724-1995): lower h2o/ch4 + minor n2o, upper ch4 + minor n2o
  {
    auto& t = T.t[9];
    const int o = T.ngs[8];
    const FArr &absa = t.at("ka"), &absb = t.at("kb"), &selfref = t.at("selfref"),
               &forref = t.at("forref"), &kamn2o = t.at("ka_mn2o"), &kbmn2o = t.at("kb_mn2o"),
               &fra = t.at("fracrefa"), &frb = t.at("fracrefb");
    double refrat_planck_a = chi(1, 9) / chi(6, 9);
    double refrat_m_a = chi(1, 3) / chi(6, 3);
    for (int lay = 1; lay <= lt; ++lay) {
      Eta e = eta(c.colh2o[lay], c.rat_h2och4[lay], c.colch4[lay], 8.);
      Eta e1 = eta(c.colh2o[lay], c.rat_h2och4_1[lay], c.colch4[lay], 8.);
      Eta em = eta(c.colh2o[lay], refrat_m_a, c.colch4[lay], 8.);
      double chi_n2o = c.coln2o[lay] / (c.coldry[lay]);
      double ratn2o = 1.e20 * chi_n2o / chi(4, c.jp[lay] + 1);
      double adjcoln2o;
      if (ratn2o > 1.5) {
        double adjfac = 0.5 + std::pow(ratn2o - 0.5, 0.65);
        adjcoln2o = adjfac * chi(4, c.jp[lay] + 1) * c.coldry[lay] * 1.e-20;
      } else {
        adjcoln2o = c.coln2o[lay];
      }
      Eta ep = eta(c.colh2o[lay], refrat_planck_a, c.colch4[lay], 8.);
      int ind0 = ((c.jp[lay] - 1) * 5 + (c.jt[lay] - 1)) * T.nspa[9] + e.js;
      int ind1 = (c.jp[lay] * 5 + (c.jt1[lay] - 1)) * T.nspa[9] + e1.js;
      Fac3 f0 = fac3(e.specparm, e.fs, c.fac00[lay], c.fac10[lay]);
      Fac3 f1 = fac3(e1.specparm, e1.fs, c.fac01[lay], c.fac11[lay]);
      for (int ig = 1; ig <= T.ngc[9]; ++ig) {
        double tauself = tself(selfref, c, lay, ig);
        double taufor = tfor(forref, c, lay, ig);
        double absn2o = minor2(kamn2o, em.js, em.fs, c, lay, ig);
        double tau_major = tau_major3(absa, e.specparm, e.speccomb, ind0, ig, f0);
        double tau_major1 = tau_major3(absa, e1.specparm, e1.speccomb, ind1, ig, f1);
        taug[o + ig][lay] = tau_major + tau_major1 + tauself + taufor + adjcoln2o * absn2o;
        fracs[o + ig][lay] = fracs_eta(fra, ep.js, ep.fs, ig);
      }
    }
    for (int lay = lt + 1; lay <= nl; ++lay) {
      double chi_n2o = c.coln2o[lay] / (c.coldry[lay]);
      double ratn2o = 1.e20 * chi_n2o / chi(4, c.jp[lay] + 1);
      double adjcoln2o;
      if (ratn2o > 1.5) {
        double adjfac = 0.5 + std::pow(ratn2o - 0.5, 0.65);
        adjcoln2o = adjfac * chi(4, c.jp[lay] + 1) * c.coldry[lay] * 1.e-20;
      } else {
        adjcoln2o = c.coln2o[lay];
      }
      int ind0 = ((c.jp[lay] - 13) * 5 + (c.jt[lay] - 1)) * T.nspb[9] + 1;
      int ind1 = ((c.jp[lay] - 12) * 5 + (c.jt1[lay] - 1)) * T.nspb[9] + 1;
      for (int ig = 1; ig <= T.ngc[9]; ++ig) {
        double absn2o = minor1(kbmn2o, c, lay, ig);
        taug[o + ig][lay] = c.colch4[lay] * interp4(absb, c, lay, ind0, ind1, ig) + adjcoln2o * absn2o;
        fracs[o + ig][lay] = frb(ig);
      }
    }
  }
  // ---- band 10 (:1998-2056): h2o
  {
    auto& t = T.t[10];
    const int o = T.ngs[9];
    const FArr &absa = t.at("ka"), &absb = t.at("kb"), &selfref = t.at("selfref"),
               &forref = t.at("forref"), &fra = t.at("fracrefa"), &frb = t.at("fracrefb");
    for (int lay = 1; lay <= lt; ++lay) {
      int ind0 = ((c.jp[lay] - 1) * 5 + (c.jt[lay] - 1)) * T.nspa[10] + 1;
      int ind1 = (c.jp[lay] * 5 + (c.jt1[lay] - 1)) * T.nspa[10] + 1;
      for (int ig = 1; ig <= T.ngc[10]; ++ig) {
        double tauself = tself(selfref, c, lay, ig);
        double taufor = tfor(forref, c, lay, ig);
        taug[o + ig][lay] = c.colh2o[lay] * interp4(absa, c, lay, ind0, ind1, ig) + tauself + taufor;
        fracs[o + ig][lay] = fra(ig);
      }
    }
    for (int lay = lt + 1; lay <= nl; ++lay) {
      int ind0 = ((c.jp[lay] - 13) * 5 + (c.jt[lay] - 1)) * T.nspb[10] + 1;
      int ind1 = ((c.jp[lay] - 12) * 5 + (c.jt1[lay] - 1)) * T.nspb[10] + 1;
      for (int ig = 1; ig <= T.ngc[10]; ++ig) {
        double taufor = tfor(forref, c, lay, ig);
        taug[o + ig][lay] = c.colh2o[lay] * interp4(absb, c, lay, ind0, ind1, ig) + taufor;
        fracs[o + ig][lay] = frb(ig);
      }
    }
  }
  // ---- band 11 (:2059-2135): h2o + minor o2
  {
    auto& t = T.t[11];
    const int o = T.ngs[10];
    const FArr &absa = t.at("ka"), &absb = t.at("kb"), &selfref = t.at("selfref"),
               &forref = t.at("forref"), &kamo2 = t.at("ka_mo2"), &kbmo2 = t.at("kb_mo2"),
               &fra = t.at("fracrefa"), &frb = t.at("fracrefb");
    for (int lay = 1; lay <= lt; ++lay) {
      int ind0 = ((c.jp[lay] - 1) * 5 + (c.jt[lay] - 1)) * T.nspa[11] + 1;
      int ind1 = (c.jp[lay] * 5 + (c.jt1[lay] - 1)) * T.nspa[11] + 1;
      double scaleo2 = c.colo2[lay] * c.scaleminor[lay];
      for (int ig = 1; ig <= T.ngc[11]; ++ig) {
        double tauself = tself(selfref, c, lay, ig);
        double taufor = tfor(forref, c, lay, ig);
        double tauo2 = scaleo2 * minor1(kamo2, c, lay, ig);
        taug[o + ig][lay] = c.colh2o[lay] * interp4(absa, c, lay, ind0, ind1, ig) + tauself + taufor + tauo2;
        fracs[o + ig][lay] = fra(ig);
      }
    }
    for (int lay = lt + 1; lay <= nl; ++lay) {
      int ind0 = ((c.jp[lay] - 13) * 5 + (c.jt[lay] - 1)) * T.nspb[11] + 1;
      int ind1 = ((c.jp[lay] - 12) * 5 + (c.jt1[lay] - 1)) * T.nspb[11] + 1;
      double scaleo2 = c.colo2[lay] * c.scaleminor[lay];
      for (int ig = 1; ig <= T.ngc[11]; ++ig) {
        double taufor = tfor(forref, c, lay, ig);
        double tauo2 = scaleo2 * minor1(kbmo2, c, lay, ig);
        taug[o + ig][lay] = c.colh2o[lay] * interp4(absb, c, lay, ind0, ind1, ig) + taufor + tauo2;
        fracs[o + ig][lay] = frb(ig);
      }
    }
  }
  // ---- band 12 (:2138-2313): lower h2o/co2, upper zero
  {
    auto& t = T.t[12];
    const int o = T.ngs[11];
    const FArr &absa = t.at("ka"), &selfref = t.at("selfref"), &forref = t.at("forref"),
               &fra = t.at("fracrefa");
    double refrat_planck_a = chi(1, 10) / chi(2, 10);
    for (int lay = 1; lay <= lt; ++lay) {
      Eta e = eta(c.colh2o[lay], c.rat_h2oco2[lay], c.colco2[lay], 8.);
      Eta e1 = eta(c.colh2o[lay], c.rat_h2oco2_1[lay], c.colco2[lay], 8.);
      Eta ep = eta(c.colh2o[lay], refrat_planck_a, c.colco2[lay], 8.);
      int ind0 = ((c.jp[lay] - 1) * 5 + (c.jt[lay] - 1)) * T.nspa[12] + e.js;
      int ind1 = (c.jp[lay] * 5 + (c.jt1[lay] - 1)) * T.nspa[12] + e1.js;
      Fac3 f0 = fac3(e.specparm, e.fs, c.fac00[lay], c.fac10[lay]);
      Fac3 f1 = fac3(e1.specparm, e1.fs, c.fac01[lay], c.fac11[lay]);
      for (int ig = 1; ig <= T.ngc[12]; ++ig) {
        double tauself = tself(selfref, c, lay, ig);
        double taufor = tfor(forref, c, lay, ig);
        double tau_major = tau_major3(absa, e.specparm, e.speccomb, ind0, ig, f0);
        double tau_major1 = tau_major3(absa, e1.specparm, e1.speccomb, ind1, ig, f1);
        taug[o + ig][lay] = tau_major + tau_major1 + tauself + taufor;
        fracs[o + ig][lay] = fracs_eta(fra, ep.js, ep.fs, ig);
      }
    }
    if (lt < nl)
      for (int lay = lt + 1; lay <= nl; ++lay)
        for (int ig = 1; ig <= T.ngc[12]; ++ig) {
          taug[o + ig][lay] = 0.0;
          fracs[o + ig][lay] = 0.0;
        }
  }
  // ---- band 13 (:2316-2584): lower h2o/n2o + minors co2, co; upper minor o3
  {
    auto& t = T.t[13];
    const int o = T.ngs[12];
    const FArr &absa = t.at("ka"), &selfref = t.at("selfref"), &forref = t.at("forref"),
               &kamco2 = t.at("ka_mco2"), &kamco = t.at("ka_mco"), &kbmo3 = t.at("kb_mo3"),
               &fra = t.at("fracrefa"), &frb = t.at("fracrefb");
    double refrat_planck_a = chi(1, 5) / chi(4, 5);
    double refrat_m_a = chi(1, 1) / chi(4, 1);
    double refrat_m_a3 = chi(1, 3) / chi(4, 3);
    for (int lay = 1; lay <= lt; ++lay) {
      Eta e = eta(c.colh2o[lay], c.rat_h2on2o[lay], c.coln2o[lay], 8.);
      Eta e1 = eta(c.colh2o[lay], c.rat_h2on2o_1[lay], c.coln2o[lay], 8.);
      Eta emc = eta(c.colh2o[lay], refrat_m_a, c.coln2o[lay], 8.);
      double chi_co2 = c.colco2[lay] / (c.coldry[lay]);
      double ratco2 = 1.e20 * chi_co2 / 3.55e-4;
      double adjcolco2;
      if (ratco2 > 3.0) {
        double adjfac = 2.0 + std::pow(ratco2 - 2.0, 0.68);
        adjcolco2 = adjfac * 3.55e-4 * c.coldry[lay] * 1.e-20;
      } else {
        adjcolco2 = c.colco2[lay];
      }
      Eta emo = eta(c.colh2o[lay], refrat_m_a3, c.coln2o[lay], 8.);
      Eta ep = eta(c.colh2o[lay], refrat_planck_a, c.coln2o[lay], 8.);
      int ind0 = ((c.jp[lay] - 1) * 5 + (c.jt[lay] - 1)) * T.nspa[13] + e.js;
      int ind1 = (c.jp[lay] * 5 + (c.jt1[lay] - 1)) * T.nspa[13] + e1.js;
      Fac3 f0 = fac3(e.specparm, e.fs, c.fac00[lay], c.fac10[lay]);
      Fac3 f1 = fac3(e1.specparm, e1.fs, c.fac01[lay], c.fac11[lay]);
      for (int ig = 1; ig <= T.ngc[13]; ++ig) {
        double tauself = tself(selfref, c, lay, ig);
        double taufor = tfor(forref, c, lay, ig);
        double absco2 = minor2(kamco2, emc.js, emc.fs, c, lay, ig);
        double absco = minor2(kamco, emo.js, emo.fs, c, lay, ig);
        double tau_major = tau_major3(absa, e.specparm, e.speccomb, ind0, ig, f0);
        double tau_major1 = tau_major3(absa, e1.specparm, e1.speccomb, ind1, ig, f1);
        taug[o + ig][lay] = tau_major + tau_major1 + tauself + taufor + adjcolco2 * absco2 + c.colco[lay] * absco;
        fracs[o + ig][lay] = fracs_eta(fra, ep.js, ep.fs, ig);
      }
    }
    for (int lay = lt + 1; lay <= nl; ++lay) {
      for (int ig = 1; ig <= T.ngc[13]; ++ig) {
        double abso3 = minor1(kbmo3, c, lay, ig);
        taug[o + ig][lay] = c.colo3[lay] * abso3;
        fracs[o + ig][lay] = frb(ig);
      }
    }
  }
  // ---- band 14 (:2587-2645): co2
  {
    auto& t = T.t[14];
    const int o = T.ngs[13];
    const FArr &absa = t.at("ka"), &absb = t.at("kb"), &selfref = t.at("selfref"),
               &forref = t.at("forref"), &fra = t.at("fracrefa"), &frb = t.at("fracrefb");
    for (int lay = 1; lay <= lt; ++lay) {
      int ind0 = ((c.jp[lay] - 1) * 5 + (c.jt[lay] - 1)) * T.nspa[14] + 1;
      int ind1 = (c.jp[lay] * 5 + (c.jt1[lay] - 1)) * T.nspa[14] + 1;
      for (int ig = 1; ig <= T.ngc[14]; ++ig) {
        double tauself = tself(selfref, c, lay, ig);
        double taufor = tfor(forref, c, lay, ig);
        taug[o + ig][lay] = c.colco2[lay] * interp4(absa, c, lay, ind0, ind1, ig) + tauself + taufor;
        fracs[o + ig][lay] = fra(ig);
      }
    }
    for (int lay = lt + 1; lay <= nl; ++lay) {
      int ind0 = ((c.jp[lay] - 13) * 5 + (c.jt[lay] - 1)) * T.nspb[14] + 1;
      int ind1 = ((c.jp[lay] - 12) * 5 + (c.jt1[lay] - 1)) * T.nspb[14] + 1;
      for (int ig = 1; ig <= T.ngc[14]; ++ig) {
        taug[o + ig][lay] = c.colco2[lay] * interp4(absb, c, lay, ind0, ind1, ig);
        fracs[o + ig][lay] = frb(ig);
      }
    }
  }
  // ---- band 15 (:2648-2836): lower n2o/co2 + minor n2, upper zero
  {
    auto& t = T.t[15];
    const int o = T.ngs[14];
    const FArr &absa = t.at("ka"), &selfref = t.at("selfref"), &forref = t.at("forref"),
               &kamn2 = t.at("ka_mn2"), &fra = t.at("fracrefa");
    double refrat_planck_a = chi(4, 1) / chi(2, 1);
    double refrat_m_a = chi(4, 1) / chi(2, 1);
    for (int lay = 1; lay <= lt; ++lay) {
      Eta e = eta(c.coln2o[lay], c.rat_n2oco2[lay], c.colco2[lay], 8.);
      Eta e1 = eta(c.coln2o[lay], c.rat_n2oco2_1[lay], c.colco2[lay], 8.);
      Eta em = eta(c.coln2o[lay], refrat_m_a, c.colco2[lay], 8.);
      Eta ep = eta(c.coln2o[lay], refrat_planck_a, c.colco2[lay], 8.);
      int ind0 = ((c.jp[lay] - 1) * 5 + (c.jt[lay] - 1)) * T.nspa[15] + e.js;
      int ind1 = (c.jp[lay] * 5 + (c.jt1[lay] - 1)) * T.nspa[15] + e1.js;
      double scalen2 = c.colbrd[lay] * c.scaleminor[lay];
      Fac3 f0 = fac3(e.specparm, e.fs, c.fac00[lay], c.fac10[lay]);
      Fac3 f1 = fac3(e1.specparm, e1.fs, c.fac01[lay], c.fac11[lay]);
      for (int ig = 1; ig <= T.ngc[15]; ++ig) {
        double tauself = tself(selfref, c, lay, ig);
        double taufor = tfor(forref, c, lay, ig);
        double taun2 = scalen2 * minor2(kamn2, em.js, em.fs, c, lay, ig);
        double tau_major = tau_major3(absa, e.specparm, e.speccomb, ind0, ig, f0);
        double tau_major1 = tau_major3(absa, e1.specparm, e1.speccomb, ind1, ig, f1);
        taug[o + ig][lay] = tau_major + tau_major1 + tauself + taufor + taun2;
        fracs[o + ig][lay] = fracs_eta(fra, ep.js, ep.fs, ig);
      }
    }
    for (int lay = lt + 1; lay <= nl; ++lay)
      for (int ig = 1; ig <= T.ngc[15]; ++ig) {
        taug[o + ig][lay] = 0.0;
        fracs[o + ig][lay] = 0.0;
      }
  }
  // ---- band 16 (:2839-3147): lower h2o/ch4, upper ch4
  {
    auto& t = T.t[16];
    const int o = T.ngs[15];
    const FArr &absa = t.at("ka"), &absb = t.at("kb"), &selfref = t.at("selfref"),
               &forref = t.at("forref"), &fra = t.at("fracrefa"), &frb = t.at("fracrefb");
    double refrat_planck_a = chi(1, 6) / chi(6, 6);
    for (int lay = 1; lay <= lt; ++lay) {
      Eta e = eta(c.colh2o[lay], c.rat_h2och4[lay], c.colch4[lay], 8.);
      Eta e1 = eta(c.colh2o[lay], c.rat_h2och4_1[lay], c.colch4[lay], 8.);
      Eta ep = eta(c.colh2o[lay], refrat_planck_a, c.colch4[lay], 8.);
      int ind0 = ((c.jp[lay] - 1) * 5 + (c.jt[lay] - 1)) * T.nspa[16] + e.js;
      int ind1 = (c.jp[lay] * 5 + (c.jt1[lay] - 1)) * T.nspa[16] + e1.js;
      Fac3 f0 = fac3(e.specparm, e.fs, c.fac00[lay], c.fac10[lay]);
      Fac3 f1 = fac3(e1.specparm, e1.fs, c.fac01[lay], c.fac11[lay]);
      for (int ig = 1; ig <= T.ngc[16]; ++ig) {
        double tauself = tself(selfref, c, lay, ig);
        double taufor = tfor(forref, c, lay, ig);
        double tau_major = tau_major3(absa, e.specparm, e.speccomb, ind0, ig, f0);
        double tau_major1 = tau_major3(absa, e1.specparm, e1.speccomb, ind1, ig, f1);
        taug[o + ig][lay] = tau_major + tau_major1 + tauself + taufor;
        fracs[o + ig][lay] = fracs_eta(fra, ep.js, ep.fs, ig);
      }
    }
    for (int lay = lt + 1; lay <= nl; ++lay) {
      int ind0 = ((c.jp[lay] - 13) * 5 + (c.jt[lay] - 1)) * T.nspb[16] + 1;
      int ind1 = ((c.jp[lay] - 12) * 5 + (c.jt1[lay] - 1)) * T.nspb[16] + 1;
      for (int ig = 1; ig <= T.ngc[16]; ++ig) {
        taug[o + ig][lay] = c.colch4[lay] * interp4(absb, c, lay, ind0, ind1, ig);
        fracs[o + ig][lay] = frb(ig);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// rtrnmr, clear sky (icld = 0: every layer takes the clear branch and the
// clear-sky stream equals the total stream, :603-616, :697-705).
// ---------------------------------------------------------------------------
void lw_rtrnmr(LwColumn& c, int idrv, LwOut& out) {
  const LwTables& T = g_lw;
  const int nl = c.nlayers;
  const double wtdiff = 0.5, rec_6 = 0.166667;
  static const double a0[17] = {0, 1.66, 1.55, 1.58, 1.66, 1.54, 1.454, 1.89, 1.33, 1.668, 1.66, 1.66, 1.66, 1.66, 1.66, 1.66, 1.66};
  static const double a1[17] = {0, 0.00, 0.25, 0.22, 0.00, 0.13, 0.446, -0.10, 0.40, -0.006, 0.00, 0.00, 0.00, 0.00, 0.00, 0.00, 0.00};
  static const double a2[17] = {0, 0.00, -12.0, -11.7, 0.00, -0.72, -0.243, 0.19, -0.062, 0.414, 0.00, 0.00, 0.00, 0.00, 0.00, 0.00, 0.00};
  double secdiff[17];
  for (int ibnd = 1; ibnd <= 16; ++ibnd) {
    if (ibnd == 1 || ibnd == 4 || ibnd >= 10) {
      secdiff[ibnd] = 1.66;
    } else {
      secdiff[ibnd] = a0[ibnd] + a1[ibnd] * std::exp(a2[ibnd] * c.pwvcm);
      if (secdiff[ibnd] > 1.80) secdiff[ibnd] = 1.80;
      if (secdiff[ibnd] < 1.50) secdiff[ibnd] = 1.50;
    }
  }
  std::vector<double> urad(nl + 1, 0.0), drad(nl + 1, 0.0), totu(nl + 1, 0.0), totd(nl + 1, 0.0);
  std::vector<double> d_urad(nl + 1, 0.0), dtotu_dt(nl + 1, 0.0);
  std::vector<double> atrans(nl + 1), bbugas(nl + 1);
  int igc = 1;
  for (int iband = 1; iband <= 16; ++iband) {
    for (; igc <= T.ngs[iband]; ++igc) {
      double radld = 0.;
      for (int lev = nl; lev >= 1; --lev) {
        double plfrac = c.fracs[igc][lev];
        double blay = c.planklay[iband][lev];
        double dplankup = c.planklev[iband][lev] - blay;
        double dplankdn = c.planklev[iband][lev - 1] - blay;
        double odepth = secdiff[iband] * c.taut[igc][lev];
        if (odepth < 0.0) odepth = 0.0;
        double bbd;
        if (odepth <= 0.06) {
          atrans[lev] = odepth - 0.5 * odepth * odepth;
          odepth = rec_6 * odepth;
          bbd = plfrac * (blay + dplankdn * odepth);
          bbugas[lev] = plfrac * (blay + dplankup * odepth);
        } else if (g_table_mode) {
          double tblind = odepth / (T.bpade + odepth);
          int itr = (int)(10000.0 * tblind + 0.5);
          double transc = T.exp_tbl[itr];
          atrans[lev] = 1. - transc;
          double tausfac = T.tfn_tbl[itr];
          bbd = plfrac * (blay + tausfac * dplankdn);
          bbugas[lev] = plfrac * (blay + tausfac * dplankup);
        } else {
          // Analytic transmittance and tau transition function (the functions
          // the tables sample, rrtmg_lw_init.f90:115-122).
          double transc = std::exp(-odepth);
          atrans[lev] = 1. - transc;
          double tausfac = 1. - 2. * ((1. / odepth) - (transc / (1. - transc)));
          bbd = plfrac * (blay + tausfac * dplankdn);
          bbugas[lev] = plfrac * (blay + tausfac * dplankup);
        }
        radld = radld + (bbd - radld) * atrans[lev];
        drad[lev - 1] = drad[lev - 1] + radld;
      }
      double rad0 = c.fracs[igc][1] * c.plankbnd[iband];
      double reflect = 1. - c.semiss[iband];
      double radlu = rad0 + reflect * radld;
      urad[0] = urad[0] + radlu;
      double d_radlu_dt = 0.0;
      if (idrv == 1) {
        d_radlu_dt = c.fracs[igc][1] * c.dplankbnd_dt[iband];
        d_urad[0] = d_urad[0] + d_radlu_dt;
      }
      for (int lev = 1; lev <= nl; ++lev) {
        radlu = radlu + (bbugas[lev] - radlu) * atrans[lev];
        urad[lev] = urad[lev] + radlu;
        if (idrv == 1) {
          d_radlu_dt = d_radlu_dt * (1.0 - atrans[lev]);
          d_urad[lev] = d_urad[lev] + d_radlu_dt;
        }
      }
    }
    for (int lev = nl; lev >= 0; --lev) {
      double uflux = urad[lev] * wtdiff;
      double dflux = drad[lev] * wtdiff;
      urad[lev] = 0.0;
      drad[lev] = 0.0;
      totu[lev] = totu[lev] + uflux * T.delwave[iband];
      totd[lev] = totd[lev] + dflux * T.delwave[iband];
      if (out.want_bands) {  // the band's own fluxes (W/m2), as the standalone RRTMG_LW prints them
        out.bandu[(size_t)(iband - 1) * (nl + 1) + lev] = uflux * T.delwave[iband] * T.fluxfac;
        out.bandd[(size_t)(iband - 1) * (nl + 1) + lev] = dflux * T.delwave[iband] * T.fluxfac;
      }
    }
    if (idrv == 1) {
      for (int lev = nl; lev >= 0; --lev) {
        double duflux_dt = d_urad[lev] * wtdiff;
        d_urad[lev] = 0.0;
        dtotu_dt[lev] = dtotu_dt[lev] + duflux_dt * T.delwave[iband] * T.fluxfac;
        if (out.want_bands) out.dbandu_dt[(size_t)(iband - 1) * (nl + 1) + lev] = duflux_dt * T.delwave[iband] * T.fluxfac;
      }
    }
  }
  std::vector<double> fnet(nl + 1);
  totu[0] = totu[0] * T.fluxfac;
  totd[0] = totd[0] * T.fluxfac;
  fnet[0] = totu[0] - totd[0];
  out.htr.assign(nl + 1, 0.0);
  for (int lev = 1; lev <= nl; ++lev) {
    totu[lev] = totu[lev] * T.fluxfac;
    totd[lev] = totd[lev] * T.fluxfac;
    fnet[lev] = totu[lev] - totd[lev];
    int l = lev - 1;
    out.htr[l] = T.heatfac * (fnet[l] - fnet[lev]) / (c.pz[l] - c.pz[lev]);
  }
  out.htr[nl] = 0.0;
  out.totu = totu;
  out.totd = totd;
  out.dtotu_dt = dtotu_dt;
}

// ---------------------------------------------------------------------------
// rtrn: random cloud overlap (icld = 1), rrtmg_lw_rtrn.f90:32-590.  A layer
// is cloudy when cldfrac >= 1e-6 (:302-315); its cloud optical depth
// secdiff * taucloud gives the effective cloud fraction (1 - e^{-odcld})
// cldfrac.  The clear-sky stream follows the total stream until the first
// cloudy layer from the top (iclddn, :441-448) and is computed on its own
// everywhere above the surface once a column holds a cloud (:500-512).
// ---------------------------------------------------------------------------
void lw_rtrn(LwColumn& c, int idrv, LwOut& out) {
  const LwTables& T = g_lw;
  const int nl = c.nlayers;
  const double wtdiff = 0.5, rec_6 = 0.166667;
  static const double a0[17] = {0, 1.66, 1.55, 1.58, 1.66, 1.54, 1.454, 1.89, 1.33, 1.668, 1.66, 1.66, 1.66, 1.66, 1.66, 1.66, 1.66};
  static const double a1[17] = {0, 0.00, 0.25, 0.22, 0.00, 0.13, 0.446, -0.10, 0.40, -0.006, 0.00, 0.00, 0.00, 0.00, 0.00, 0.00, 0.00};
  static const double a2[17] = {0, 0.00, -12.0, -11.7, 0.00, -0.72, -0.243, 0.19, -0.062, 0.414, 0.00, 0.00, 0.00, 0.00, 0.00, 0.00, 0.00};
  double secdiff[17];
  for (int ibnd = 1; ibnd <= 16; ++ibnd) {
    if (ibnd == 1 || ibnd == 4 || ibnd >= 10) {
      secdiff[ibnd] = 1.66;
    } else {
      secdiff[ibnd] = a0[ibnd] + a1[ibnd] * std::exp(a2[ibnd] * c.pwvcm);
      if (secdiff[ibnd] > 1.80) secdiff[ibnd] = 1.80;
      if (secdiff[ibnd] < 1.50) secdiff[ibnd] = 1.50;
    }
  }
  // cloud optical depth and effective cloud fraction per layer and band (:302-315)
  std::vector<int> icldlyr(nl + 1, 0);
  std::vector<double> odcld[17], efclfrac[17];
  for (int ib = 1; ib <= 16; ++ib) {
    odcld[ib].assign(nl + 1, 0.0);
    efclfrac[ib].assign(nl + 1, 0.0);
  }
  // McICA (rtrnmc, rrtmg_lw_rtrnmc.f90:279-310): per g-point, a sub-column is
  // cloudy where its cover is 1, its depth secdiff(ngb(ig)) x taucmc; a layer
  // takes the cloudy branch for all its g-points when any of them is cloudy
  const int L1 = nl + 1;
  std::vector<double> odg, efg;
  if (c.mcica) {
    odg.assign((size_t)140 * L1, 0.0);
    efg.assign((size_t)140 * L1, 0.0);
    for (int lay = 1; lay <= nl; ++lay) {
      icldlyr[lay] = 0;
      for (int b = 1, ig = 1; b <= 16; ++b)
        for (; ig <= T.ngs[b]; ++ig) {
          const size_t k = (size_t)(ig - 1) * L1 + lay;
          if (c.cldfmc[k] == 1.0) {
            odg[k] = secdiff[b] * c.taucmc[k];
            const double transcld = std::exp(-odg[k]);
            efg[k] = (1.0 - transcld) * c.cldfmc[k];
            icldlyr[lay] = 1;
          }
        }
    }
  }
  for (int lay = 1; lay <= nl && !c.mcica; ++lay)
    for (int ib = 1; ib <= 16; ++ib) {
      if (c.cldfrac[lay] >= 1.e-6) {
        odcld[ib][lay] = secdiff[ib] * c.taucloud[ib][lay];
        const double transcld = std::exp(-odcld[ib][lay]);
        const double abscld = 1. - transcld;
        efclfrac[ib][lay] = abscld * c.cldfrac[lay];
        icldlyr[lay] = 1;
      } else {
        icldlyr[lay] = 0;
      }
    }
  // the transmittance function and the optical depth of a table entry, or
  // (analytic mode) of the optical depth itself
  auto tbl = [&](double od, double& trans, double& tfn, double& odq) {
    if (g_table_mode) {
      const double tblind = od / (T.bpade + od);
      const int it = (int)(10000.0 * tblind + 0.5);
      trans = T.exp_tbl[it];
      tfn = T.tfn_tbl[it];
      odq = T.tau_tbl[it];
    } else {
      trans = std::exp(-od);
      tfn = 1. - 2. * ((1. / od) - (trans / (1. - trans)));
      odq = od;
    }
  };
  std::vector<double> urad(nl + 1, 0.0), drad(nl + 1, 0.0), totu(nl + 1, 0.0), totd(nl + 1, 0.0);
  std::vector<double> clru(nl + 1, 0.0), clrd(nl + 1, 0.0), totuc(nl + 1, 0.0), totdc(nl + 1, 0.0);
  std::vector<double> d_urad(nl + 1, 0.0), d_clru(nl + 1, 0.0), dtotu_dt(nl + 1, 0.0), dtotuc_dt(nl + 1, 0.0);
  std::vector<double> atrans(nl + 1), bbugas(nl + 1), atot(nl + 1), bbutot(nl + 1);
  int igc = 1;
  for (int iband = 1; iband <= 16; ++iband) {
    const int ib = lw_cloud_band(iband, c.ncbands);  // ipat(iband, ...) (rrtmg_lw_rtrn.f90:324-330)
    for (; igc <= T.ngs[iband]; ++igc) {
      // the cloud depth, effective cover and cover of layer lev for this g-point
      auto OD = [&](int lev) { return c.mcica ? odg[(size_t)(igc - 1) * L1 + lev] : odcld[ib][lev]; };
      auto EF = [&](int lev) { return c.mcica ? efg[(size_t)(igc - 1) * L1 + lev] : efclfrac[ib][lev]; };
      auto CF = [&](int lev) { return c.mcica ? c.cldfmc[(size_t)(igc - 1) * L1 + lev] : c.cldfrac[lev]; };
      double radld = 0., radclrd = 0.;
      int iclddn = 0;
      for (int lev = nl; lev >= 1; --lev) {
        const double plfrac = c.fracs[igc][lev];
        const double blay = c.planklay[iband][lev];
        const double dplankup = c.planklev[iband][lev] - blay;
        const double dplankdn = c.planklev[iband][lev - 1] - blay;
        double odepth = secdiff[iband] * c.taut[igc][lev];
        if (odepth < 0.0) odepth = 0.0;
        double bbd;
        if (icldlyr[lev] == 1) {  // :350-416
          iclddn = 1;
          double odtot = odepth + OD(lev);
          double gassrc, bbdtot;
          if (odtot < 0.06) {
            atrans[lev] = odepth - 0.5 * odepth * odepth;
            const double odepth_rec = rec_6 * odepth;
            gassrc = plfrac * (blay + dplankdn * odepth_rec) * atrans[lev];
            atot[lev] = odtot - 0.5 * odtot * odtot;
            const double odtot_rec = rec_6 * odtot;
            bbdtot = plfrac * (blay + dplankdn * odtot_rec);
            bbd = plfrac * (blay + dplankdn * odepth_rec);
            bbugas[lev] = plfrac * (blay + dplankup * odepth_rec);
            bbutot[lev] = plfrac * (blay + dplankup * odtot_rec);
          } else if (odepth <= 0.06) {
            atrans[lev] = odepth - 0.5 * odepth * odepth;
            const double odepth_rec = rec_6 * odepth;
            gassrc = plfrac * (blay + dplankdn * odepth_rec) * atrans[lev];
            odtot = odepth + OD(lev);
            double ttot, tfactot, odq;
            tbl(odtot, ttot, tfactot, odq);
            bbdtot = plfrac * (blay + tfactot * dplankdn);
            bbd = plfrac * (blay + dplankdn * odepth_rec);
            atot[lev] = 1. - ttot;
            bbugas[lev] = plfrac * (blay + dplankup * odepth_rec);
            bbutot[lev] = plfrac * (blay + tfactot * dplankup);
          } else {
            double tgas, tfacgas, odq;
            tbl(odepth, tgas, tfacgas, odq);
            odepth = odq;  // odepth = tau_tbl(itgas)
            atrans[lev] = 1. - tgas;
            gassrc = atrans[lev] * plfrac * (blay + tfacgas * dplankdn);
            odtot = odepth + OD(lev);
            double ttot, tfactot, odq2;
            tbl(odtot, ttot, tfactot, odq2);
            bbdtot = plfrac * (blay + tfactot * dplankdn);
            bbd = plfrac * (blay + tfacgas * dplankdn);
            atot[lev] = 1. - ttot;
            bbugas[lev] = plfrac * (blay + tfacgas * dplankup);
            bbutot[lev] = plfrac * (blay + tfactot * dplankup);
          }
          radld = radld - radld * (atrans[lev] + EF(lev) * (1. - atrans[lev])) + gassrc +
                  CF(lev) * (bbdtot * atot[lev] - gassrc);
          drad[lev - 1] = drad[lev - 1] + radld;
        } else {  // clear layer (:418-436), as rtrnmr
          if (odepth <= 0.06) {
            atrans[lev] = odepth - 0.5 * odepth * odepth;
            odepth = rec_6 * odepth;
            bbd = plfrac * (blay + dplankdn * odepth);
            bbugas[lev] = plfrac * (blay + dplankup * odepth);
          } else {
            double transc, tausfac, odq;
            tbl(odepth, transc, tausfac, odq);
            atrans[lev] = 1. - transc;
            bbd = plfrac * (blay + tausfac * dplankdn);
            bbugas[lev] = plfrac * (blay + tausfac * dplankup);
          }
          radld = radld + (bbd - radld) * atrans[lev];
          drad[lev - 1] = drad[lev - 1] + radld;
        }
        if (iclddn == 1) {  // :441-448
          radclrd = radclrd + (bbd - radclrd) * atrans[lev];
          clrd[lev - 1] = clrd[lev - 1] + radclrd;
        } else {
          radclrd = radld;
          clrd[lev - 1] = drad[lev - 1];
        }
      }
      const double rad0 = c.fracs[igc][1] * c.plankbnd[iband];
      const double reflect = 1. - c.semiss[iband];
      double radlu = rad0 + reflect * radld;
      double radclru = rad0 + reflect * radclrd;
      urad[0] = urad[0] + radlu;
      clru[0] = clru[0] + radclru;
      double d_radlu_dt = 0.0, d_radclru_dt = 0.0;
      if (idrv == 1) {
        const double d_rad0_dt = c.fracs[igc][1] * c.dplankbnd_dt[iband];
        d_radlu_dt = d_rad0_dt;
        d_urad[0] = d_urad[0] + d_radlu_dt;
        d_radclru_dt = d_rad0_dt;
        d_clru[0] = d_clru[0] + d_radclru_dt;
      }
      for (int lev = 1; lev <= nl; ++lev) {  // :478-520
        if (icldlyr[lev] == 1) {
          const double gassrc = bbugas[lev] * atrans[lev];
          radlu = radlu - radlu * (atrans[lev] + EF(lev) * (1. - atrans[lev])) + gassrc +
                  CF(lev) * (bbutot[lev] * atot[lev] - gassrc);
          urad[lev] = urad[lev] + radlu;
          if (idrv == 1) {
            d_radlu_dt = d_radlu_dt * CF(lev) * (1.0 - atot[lev]) +
                         d_radlu_dt * (1.0 - CF(lev)) * (1.0 - atrans[lev]);
            d_urad[lev] = d_urad[lev] + d_radlu_dt;
          }
        } else {
          radlu = radlu + (bbugas[lev] - radlu) * atrans[lev];
          urad[lev] = urad[lev] + radlu;
          if (idrv == 1) {
            d_radlu_dt = d_radlu_dt * (1.0 - atrans[lev]);
            d_urad[lev] = d_urad[lev] + d_radlu_dt;
          }
        }
        if (iclddn == 1) {
          radclru = radclru + (bbugas[lev] - radclru) * atrans[lev];
          clru[lev] = clru[lev] + radclru;
        } else {
          radclru = radlu;
          clru[lev] = urad[lev];
        }
        if (idrv == 1) {
          if (iclddn == 1) {
            d_radclru_dt = d_radclru_dt * (1.0 - atrans[lev]);
            d_clru[lev] = d_clru[lev] + d_radclru_dt;
          } else {
            d_radclru_dt = d_radlu_dt;
            d_clru[lev] = d_urad[lev];
          }
        }
      }
    }
    for (int lev = nl; lev >= 0; --lev) {  // :526-543
      const double uflux = urad[lev] * wtdiff, dflux = drad[lev] * wtdiff;
      urad[lev] = 0.0;
      drad[lev] = 0.0;
      totu[lev] = totu[lev] + uflux * T.delwave[iband];
      totd[lev] = totd[lev] + dflux * T.delwave[iband];
      const double uclfl = clru[lev] * wtdiff, dclfl = clrd[lev] * wtdiff;
      clru[lev] = 0.0;
      clrd[lev] = 0.0;
      totuc[lev] = totuc[lev] + uclfl * T.delwave[iband];
      totdc[lev] = totdc[lev] + dclfl * T.delwave[iband];
    }
    if (idrv == 1) {
      for (int lev = nl; lev >= 0; --lev) {
        const double duflux_dt = d_urad[lev] * wtdiff;
        d_urad[lev] = 0.0;
        dtotu_dt[lev] = dtotu_dt[lev] + duflux_dt * T.delwave[iband] * T.fluxfac;
        const double duclfl_dt = d_clru[lev] * wtdiff;
        d_clru[lev] = 0.0;
        dtotuc_dt[lev] = dtotuc_dt[lev] + duclfl_dt * T.delwave[iband] * T.fluxfac;
      }
    }
  }
  std::vector<double> fnet(nl + 1), fnetc(nl + 1);
  totu[0] = totu[0] * T.fluxfac;
  totd[0] = totd[0] * T.fluxfac;
  fnet[0] = totu[0] - totd[0];
  totuc[0] = totuc[0] * T.fluxfac;
  totdc[0] = totdc[0] * T.fluxfac;
  fnetc[0] = totuc[0] - totdc[0];
  out.htr.assign(nl + 1, 0.0);
  out.htrc.assign(nl + 1, 0.0);
  for (int lev = 1; lev <= nl; ++lev) {
    totu[lev] = totu[lev] * T.fluxfac;
    totd[lev] = totd[lev] * T.fluxfac;
    fnet[lev] = totu[lev] - totd[lev];
    totuc[lev] = totuc[lev] * T.fluxfac;
    totdc[lev] = totdc[lev] * T.fluxfac;
    fnetc[lev] = totuc[lev] - totdc[lev];
    const int l = lev - 1;
    out.htr[l] = T.heatfac * (fnet[l] - fnet[lev]) / (c.pz[l] - c.pz[lev]);
    out.htrc[l] = T.heatfac * (fnetc[l] - fnetc[lev]) / (c.pz[l] - c.pz[lev]);
  }
  out.totu = totu;
  out.totd = totd;
  out.dtotu_dt = dtotu_dt;
  out.totuc = totuc;
  out.totdc = totdc;
  out.dtotuc_dt = dtotuc_dt;
}

// ---------------------------------------------------------------------------
// rtrnmr with clouds: maximum/random overlap (icld = 2, 3 in the non-McICA
// driver, rrtmg_lw_rad.nomcica.f90:527-541), rrtmg_lw_rtrnmr.f90:300-705.
// Each cloudy layer carries a cloudy and a clear radiance; the overlap
// factors move radiance between them at the layer's lower (upward pass) or
// upper (downward pass) boundary, from the cloud fractions of the layer and
// its two neighbours (:326-475).  cldfrac(0) (read as 0 x value at the lowest
// layer, :400-401) is taken as 0; cldfrac(nlayers + 1) is the driver's zero.
// ---------------------------------------------------------------------------
struct MrOverlap {
  // upward factors indexed lev + 1 (1..nl+1), downward ones lev - 1 (0..nl-1)
  std::vector<double> faccld1, faccld2, facclr1, facclr2, faccmb1, faccmb2;
  std::vector<double> faccld1d, faccld2d, facclr1d, facclr2d, faccmb1d, faccmb2d;
  std::vector<int> istcld, istcldd;
};

static void lw_mr_overlap(const std::vector<double>& cf, const std::vector<int>& icldlyr, int nl, MrOverlap& o) {
  for (auto* v : {&o.faccld1, &o.faccld2, &o.facclr1, &o.facclr2, &o.faccmb1, &o.faccmb2, &o.faccld1d, &o.faccld2d,
                  &o.facclr1d, &o.facclr2d, &o.faccmb1d, &o.faccmb2d})
    v->assign(nl + 2, 0.0);
  o.istcld.assign(nl + 2, 0);
  o.istcldd.assign(nl + 2, 0);
  double rat1 = 0.0, rat2 = 0.0;
  // upward (:326-403)
  o.istcld[1] = 1;
  o.istcldd[nl] = 1;
  for (int lev = 1; lev <= nl; ++lev) {
    if (icldlyr[lev] != 1) {
      o.istcld[lev + 1] = 1;
      continue;
    }
    o.istcld[lev + 1] = 0;
    if (lev == nl) {
      o.faccld1[lev + 1] = o.faccld2[lev + 1] = o.facclr1[lev + 1] = 0.;
      o.facclr2[lev + 1] = o.faccmb1[lev + 1] = o.faccmb2[lev + 1] = 0.;
    } else if (cf[lev + 1] >= cf[lev]) {
      o.faccld1[lev + 1] = 0.;
      o.faccld2[lev + 1] = 0.;
      if (o.istcld[lev] == 1) {
        o.facclr1[lev + 1] = 0.;
        o.facclr2[lev + 1] = 0.;
        if (cf[lev] < 1.) o.facclr2[lev + 1] = (cf[lev + 1] - cf[lev]) / (1. - cf[lev]);
        o.facclr2[lev] = 0.;
        o.faccld2[lev] = 0.;
      } else {
        const double fmax = std::max(cf[lev], cf[lev - 1]);
        if (cf[lev + 1] > fmax) {
          o.facclr1[lev + 1] = rat2;
          o.facclr2[lev + 1] = (cf[lev + 1] - fmax) / (1. - fmax);
        } else if (cf[lev + 1] < fmax) {
          o.facclr1[lev + 1] = (cf[lev + 1] - cf[lev]) / (cf[lev - 1] - cf[lev]);
          o.facclr2[lev + 1] = 0.;
        } else {
          o.facclr1[lev + 1] = rat2;
          o.facclr2[lev + 1] = 0.;
        }
      }
      if (o.facclr1[lev + 1] > 0. || o.facclr2[lev + 1] > 0.) {
        rat1 = 1.;
        rat2 = 0.;
      } else {
        rat1 = 0.;
        rat2 = 0.;
      }
    } else {
      o.facclr1[lev + 1] = 0.;
      o.facclr2[lev + 1] = 0.;
      if (o.istcld[lev] == 1) {
        o.faccld1[lev + 1] = 0.;
        o.faccld2[lev + 1] = (cf[lev] - cf[lev + 1]) / cf[lev];
        o.facclr2[lev] = 0.;
        o.faccld2[lev] = 0.;
      } else {
        const double fmin = std::min(cf[lev], cf[lev - 1]);
        if (cf[lev + 1] <= fmin) {
          o.faccld1[lev + 1] = rat1;
          o.faccld2[lev + 1] = (fmin - cf[lev + 1]) / fmin;
        } else {
          o.faccld1[lev + 1] = (cf[lev] - cf[lev + 1]) / (cf[lev] - fmin);
          o.faccld2[lev + 1] = 0.;
        }
      }
      if (o.faccld1[lev + 1] > 0. || o.faccld2[lev + 1] > 0.) {
        rat1 = 0.;
        rat2 = 1.;
      } else {
        rat1 = 0.;
        rat2 = 0.;
      }
    }
    o.faccmb1[lev + 1] = o.facclr1[lev + 1] * o.faccld2[lev] * cf[lev - 1];
    o.faccmb2[lev + 1] = o.faccld1[lev + 1] * o.facclr2[lev] * (1. - cf[lev - 1]);
  }
  // downward (:405-475)
  for (int lev = nl; lev >= 1; --lev) {
    if (icldlyr[lev] != 1) {
      o.istcldd[lev - 1] = 1;
      continue;
    }
    o.istcldd[lev - 1] = 0;
    if (lev == 1) {
      o.faccld1d[lev - 1] = o.faccld2d[lev - 1] = o.facclr1d[lev - 1] = 0.;
      o.facclr2d[lev - 1] = o.faccmb1d[lev - 1] = o.faccmb2d[lev - 1] = 0.;
    } else if (cf[lev - 1] >= cf[lev]) {
      o.faccld1d[lev - 1] = 0.;
      o.faccld2d[lev - 1] = 0.;
      if (o.istcldd[lev] == 1) {
        o.facclr1d[lev - 1] = 0.;
        o.facclr2d[lev - 1] = 0.;
        if (cf[lev] < 1.) o.facclr2d[lev - 1] = (cf[lev - 1] - cf[lev]) / (1. - cf[lev]);
        o.facclr2d[lev] = 0.;
        o.faccld2d[lev] = 0.;
      } else {
        const double fmax = std::max(cf[lev], cf[lev + 1]);
        if (cf[lev - 1] > fmax) {
          o.facclr1d[lev - 1] = rat2;
          o.facclr2d[lev - 1] = (cf[lev - 1] - fmax) / (1. - fmax);
        } else if (cf[lev - 1] < fmax) {
          o.facclr1d[lev - 1] = (cf[lev - 1] - cf[lev]) / (cf[lev + 1] - cf[lev]);
          o.facclr2d[lev - 1] = 0.;
        } else {
          o.facclr1d[lev - 1] = rat2;
          o.facclr2d[lev - 1] = 0.;
        }
      }
      if (o.facclr1d[lev - 1] > 0. || o.facclr2d[lev - 1] > 0.) {
        rat1 = 1.;
        rat2 = 0.;
      } else {
        rat1 = 0.;
        rat2 = 0.;
      }
    } else {
      o.facclr1d[lev - 1] = 0.;
      o.facclr2d[lev - 1] = 0.;
      if (o.istcldd[lev] == 1) {
        o.faccld1d[lev - 1] = 0.;
        o.faccld2d[lev - 1] = (cf[lev] - cf[lev - 1]) / cf[lev];
        o.facclr2d[lev] = 0.;
        o.faccld2d[lev] = 0.;
      } else {
        const double fmin = std::min(cf[lev], cf[lev + 1]);
        if (cf[lev - 1] <= fmin) {
          o.faccld1d[lev - 1] = rat1;
          o.faccld2d[lev - 1] = (fmin - cf[lev - 1]) / fmin;
        } else {
          o.faccld1d[lev - 1] = (cf[lev] - cf[lev - 1]) / (cf[lev] - fmin);
          o.faccld2d[lev - 1] = 0.;
        }
      }
      if (o.faccld1d[lev - 1] > 0. || o.faccld2d[lev - 1] > 0.) {
        rat1 = 0.;
        rat2 = 1.;
      } else {
        rat1 = 0.;
        rat2 = 0.;
      }
    }
    o.faccmb1d[lev - 1] = o.facclr1d[lev - 1] * o.faccld2d[lev] * cf[lev + 1];
    o.faccmb2d[lev - 1] = o.faccld1d[lev - 1] * o.facclr2d[lev] * (1. - cf[lev + 1]);
  }
}

void lw_rtrnmr_cld(LwColumn& c, int idrv, LwOut& out) {
  const LwTables& T = g_lw;
  const int nl = c.nlayers;
  const double wtdiff = 0.5, rec_6 = 0.166667;
  static const double a0[17] = {0, 1.66, 1.55, 1.58, 1.66, 1.54, 1.454, 1.89, 1.33, 1.668, 1.66, 1.66, 1.66, 1.66, 1.66, 1.66, 1.66};
  static const double a1[17] = {0, 0.00, 0.25, 0.22, 0.00, 0.13, 0.446, -0.10, 0.40, -0.006, 0.00, 0.00, 0.00, 0.00, 0.00, 0.00, 0.00};
  static const double a2[17] = {0, 0.00, -12.0, -11.7, 0.00, -0.72, -0.243, 0.19, -0.062, 0.414, 0.00, 0.00, 0.00, 0.00, 0.00, 0.00, 0.00};
  double secdiff[17];
  for (int ibnd = 1; ibnd <= 16; ++ibnd) {
    if (ibnd == 1 || ibnd == 4 || ibnd >= 10) {
      secdiff[ibnd] = 1.66;
    } else {
      secdiff[ibnd] = a0[ibnd] + a1[ibnd] * std::exp(a2[ibnd] * c.pwvcm);
      if (secdiff[ibnd] > 1.80) secdiff[ibnd] = 1.80;
      if (secdiff[ibnd] < 1.50) secdiff[ibnd] = 1.50;
    }
  }
  // cloudy layers and their cloud optical depths (:315-323)
  std::vector<int> icldlyr(nl + 2, 0);
  std::vector<double> odcld[17];
  for (int ib = 1; ib <= 16; ++ib) odcld[ib].assign(nl + 1, 0.0);
  for (int lay = 1; lay <= nl; ++lay)
    for (int ib = 1; ib <= 16; ++ib) {
      if (c.cldfrac[lay] >= 1.e-6) {
        odcld[ib][lay] = secdiff[ib] * c.taucloud[ib][lay];
        icldlyr[lay] = 1;
      } else {
        odcld[ib][lay] = 0.0;
        icldlyr[lay] = 0;
      }
    }
  MrOverlap ov;
  lw_mr_overlap(c.cldfrac, icldlyr, nl, ov);
  const std::vector<double>& cf = c.cldfrac;
  auto tbl = [&](double od, double& trans, double& tfn, double& odq) {
    if (g_table_mode) {
      const double tblind = od / (T.bpade + od);
      const int it = (int)(10000.0 * tblind + 0.5);
      trans = T.exp_tbl[it];
      tfn = T.tfn_tbl[it];
      odq = T.tau_tbl[it];
    } else {
      trans = std::exp(-od);
      tfn = 1. - 2. * ((1. / od) - (trans / (1. - trans)));
      odq = od;
    }
  };
  std::vector<double> urad(nl + 1, 0.0), drad(nl + 1, 0.0), totu(nl + 1, 0.0), totd(nl + 1, 0.0);
  std::vector<double> clru(nl + 1, 0.0), clrd(nl + 1, 0.0), totuc(nl + 1, 0.0), totdc(nl + 1, 0.0);
  std::vector<double> d_urad(nl + 1, 0.0), d_clru(nl + 1, 0.0), dtotu_dt(nl + 1, 0.0), dtotuc_dt(nl + 1, 0.0);
  std::vector<double> atrans(nl + 1), bbugas(nl + 1), atot(nl + 1), bbutot(nl + 1);
  int igc = 1;
  for (int iband = 1; iband <= 16; ++iband) {
    const int ib = lw_cloud_band(iband, c.ncbands);  // ipat(iband, ...) (rrtmg_lw_rtrn.f90:324-330)
    for (; igc <= T.ngs[iband]; ++igc) {
      double radld = 0., radclrd = 0.;
      double cldradd = 0., clrradd = 0., rad = 0.;
      int iclddn = 0;
      for (int lev = nl; lev >= 1; --lev) {  // :500-617
        const double plfrac = c.fracs[igc][lev];
        const double blay = c.planklay[iband][lev];
        const double dplankup = c.planklev[iband][lev] - blay;
        const double dplankdn = c.planklev[iband][lev - 1] - blay;
        double odepth = secdiff[iband] * c.taut[igc][lev];
        if (odepth < 0.0) odepth = 0.0;
        double bbd;
        if (icldlyr[lev] == 1) {
          iclddn = 1;
          double odtot = odepth + odcld[ib][lev];
          double gassrc, bbdtot;
          if (odtot < 0.06) {
            atrans[lev] = odepth - 0.5 * odepth * odepth;
            const double odepth_rec = rec_6 * odepth;
            gassrc = plfrac * (blay + dplankdn * odepth_rec) * atrans[lev];
            atot[lev] = odtot - 0.5 * odtot * odtot;
            const double odtot_rec = rec_6 * odtot;
            bbdtot = plfrac * (blay + dplankdn * odtot_rec);
            bbd = plfrac * (blay + dplankdn * odepth_rec);
            bbugas[lev] = plfrac * (blay + dplankup * odepth_rec);
            bbutot[lev] = plfrac * (blay + dplankup * odtot_rec);
          } else if (odepth <= 0.06) {
            atrans[lev] = odepth - 0.5 * odepth * odepth;
            const double odepth_rec = rec_6 * odepth;
            gassrc = plfrac * (blay + dplankdn * odepth_rec) * atrans[lev];
            odtot = odepth + odcld[ib][lev];
            double ttot, tfactot, odq;
            tbl(odtot, ttot, tfactot, odq);
            bbdtot = plfrac * (blay + tfactot * dplankdn);
            bbd = plfrac * (blay + dplankdn * odepth_rec);
            atot[lev] = 1. - ttot;
            bbugas[lev] = plfrac * (blay + dplankup * odepth_rec);
            bbutot[lev] = plfrac * (blay + tfactot * dplankup);
          } else {
            double tgas, tfacgas, odq;
            tbl(odepth, tgas, tfacgas, odq);
            odepth = odq;  // odepth = tau_tbl(itgas)
            atrans[lev] = 1. - tgas;
            gassrc = atrans[lev] * plfrac * (blay + tfacgas * dplankdn);
            odtot = odepth + odcld[ib][lev];
            double ttot, tfactot, odq2;
            tbl(odtot, ttot, tfactot, odq2);
            bbdtot = plfrac * (blay + tfactot * dplankdn);
            bbd = plfrac * (blay + tfacgas * dplankdn);
            atot[lev] = 1. - ttot;
            bbugas[lev] = plfrac * (blay + tfacgas * dplankup);
            bbutot[lev] = plfrac * (blay + tfactot * dplankup);
          }
          if (ov.istcldd[lev] == 1) {
            cldradd = cf[lev] * radld;
            clrradd = radld - cldradd;
            rad = 0.;
          }
          const double ttot = 1. - atot[lev];
          const double cldsrc = bbdtot * atot[lev];
          cldradd = cldradd * ttot + cf[lev] * cldsrc;
          clrradd = clrradd * (1. - atrans[lev]) + (1. - cf[lev]) * gassrc;
          radld = cldradd + clrradd;
          drad[lev - 1] = drad[lev - 1] + radld;
          const double radmod = rad * (ov.facclr1d[lev - 1] * (1. - atrans[lev]) + ov.faccld1d[lev - 1] * ttot) -
                                ov.faccmb1d[lev - 1] * gassrc + ov.faccmb2d[lev - 1] * cldsrc;
          const double oldcld = cldradd - radmod;
          const double oldclr = clrradd + radmod;
          rad = -radmod + ov.facclr2d[lev - 1] * oldclr - ov.faccld2d[lev - 1] * oldcld;
          cldradd = cldradd + rad;
          clrradd = clrradd - rad;
        } else {
          if (odepth <= 0.06) {
            atrans[lev] = odepth - 0.5 * odepth * odepth;
            odepth = rec_6 * odepth;
            bbd = plfrac * (blay + dplankdn * odepth);
            bbugas[lev] = plfrac * (blay + dplankup * odepth);
          } else {
            double transc, tausfac, odq;
            tbl(odepth, transc, tausfac, odq);
            atrans[lev] = 1. - transc;
            bbd = plfrac * (blay + tausfac * dplankdn);
            bbugas[lev] = plfrac * (blay + tausfac * dplankup);
          }
          radld = radld + (bbd - radld) * atrans[lev];
          drad[lev - 1] = drad[lev - 1] + radld;
        }
        if (iclddn == 1) {  // :606-614
          radclrd = radclrd + (bbd - radclrd) * atrans[lev];
          clrd[lev - 1] = clrd[lev - 1] + radclrd;
        } else {
          radclrd = radld;
          clrd[lev - 1] = drad[lev - 1];
        }
      }
      const double rad0 = c.fracs[igc][1] * c.plankbnd[iband];
      const double reflect = 1. - c.semiss[iband];
      double radlu = rad0 + reflect * radld;
      double radclru = rad0 + reflect * radclrd;
      urad[0] = urad[0] + radlu;
      clru[0] = clru[0] + radclru;
      double d_radlu_dt = 0.0, d_radclru_dt = 0.0;
      if (idrv == 1) {
        const double d_rad0_dt = c.fracs[igc][1] * c.dplankbnd_dt[iband];
        d_radlu_dt = d_rad0_dt;
        d_urad[0] = d_urad[0] + d_radlu_dt;
        d_radclru_dt = d_rad0_dt;
        d_clru[0] = d_clru[0] + d_radclru_dt;
      }
      double cldradu = 0., clrradu = 0.;
      rad = 0.;
      for (int lev = 1; lev <= nl; ++lev) {  // :649-705
        if (icldlyr[lev] == 1) {
          const double gassrc = bbugas[lev] * atrans[lev];
          if (ov.istcld[lev] == 1) {
            cldradu = cf[lev] * radlu;
            clrradu = radlu - cldradu;
            rad = 0.;
          }
          const double ttot = 1. - atot[lev];
          const double cldsrc = bbutot[lev] * atot[lev];
          cldradu = cldradu * ttot + cf[lev] * cldsrc;
          clrradu = clrradu * (1.0 - atrans[lev]) + (1. - cf[lev]) * gassrc;
          radlu = cldradu + clrradu;
          urad[lev] = urad[lev] + radlu;
          const double radmod = rad * (ov.facclr1[lev + 1] * (1.0 - atrans[lev]) + ov.faccld1[lev + 1] * ttot) -
                                ov.faccmb1[lev + 1] * gassrc + ov.faccmb2[lev + 1] * cldsrc;
          const double oldcld = cldradu - radmod;
          const double oldclr = clrradu + radmod;
          rad = -radmod + ov.facclr2[lev + 1] * oldclr - ov.faccld2[lev + 1] * oldcld;
          cldradu = cldradu + rad;
          clrradu = clrradu - rad;
          if (idrv == 1) {
            d_radlu_dt = d_radlu_dt * cf[lev] * (1.0 - atot[lev]) + d_radlu_dt * (1.0 - cf[lev]) * (1.0 - atrans[lev]);
            d_urad[lev] = d_urad[lev] + d_radlu_dt;
          }
        } else {
          radlu = radlu + (bbugas[lev] - radlu) * atrans[lev];
          urad[lev] = urad[lev] + radlu;
          if (idrv == 1) {
            d_radlu_dt = d_radlu_dt * (1.0 - atrans[lev]);
            d_urad[lev] = d_urad[lev] + d_radlu_dt;
          }
        }
        if (iclddn == 1) {
          radclru = radclru + (bbugas[lev] - radclru) * atrans[lev];
          clru[lev] = clru[lev] + radclru;
        } else {
          radclru = radlu;
          clru[lev] = urad[lev];
        }
        if (idrv == 1) {
          if (iclddn == 1) {
            d_radclru_dt = d_radclru_dt * (1.0 - atrans[lev]);
            d_clru[lev] = d_clru[lev] + d_radclru_dt;
          } else {
            d_radclru_dt = d_radlu_dt;
            d_clru[lev] = d_urad[lev];
          }
        }
      }
    }
    for (int lev = nl; lev >= 0; --lev) {  // :711-726
      const double uflux = urad[lev] * wtdiff, dflux = drad[lev] * wtdiff;
      urad[lev] = 0.0;
      drad[lev] = 0.0;
      totu[lev] = totu[lev] + uflux * T.delwave[iband];
      totd[lev] = totd[lev] + dflux * T.delwave[iband];
      const double uclfl = clru[lev] * wtdiff, dclfl = clrd[lev] * wtdiff;
      clru[lev] = 0.0;
      clrd[lev] = 0.0;
      totuc[lev] = totuc[lev] + uclfl * T.delwave[iband];
      totdc[lev] = totdc[lev] + dclfl * T.delwave[iband];
    }
    if (idrv == 1) {
      for (int lev = nl; lev >= 0; --lev) {
        const double duflux_dt = d_urad[lev] * wtdiff;
        d_urad[lev] = 0.0;
        dtotu_dt[lev] = dtotu_dt[lev] + duflux_dt * T.delwave[iband] * T.fluxfac;
        const double duclfl_dt = d_clru[lev] * wtdiff;
        d_clru[lev] = 0.0;
        dtotuc_dt[lev] = dtotuc_dt[lev] + duclfl_dt * T.delwave[iband] * T.fluxfac;
      }
    }
  }
  std::vector<double> fnet(nl + 1), fnetc(nl + 1);
  totu[0] = totu[0] * T.fluxfac;
  totd[0] = totd[0] * T.fluxfac;
  fnet[0] = totu[0] - totd[0];
  totuc[0] = totuc[0] * T.fluxfac;
  totdc[0] = totdc[0] * T.fluxfac;
  fnetc[0] = totuc[0] - totdc[0];
  out.htr.assign(nl + 1, 0.0);
  out.htrc.assign(nl + 1, 0.0);
  for (int lev = 1; lev <= nl; ++lev) {
    totu[lev] = totu[lev] * T.fluxfac;
    totd[lev] = totd[lev] * T.fluxfac;
    fnet[lev] = totu[lev] - totd[lev];
    totuc[lev] = totuc[lev] * T.fluxfac;
    totdc[lev] = totdc[lev] * T.fluxfac;
    fnetc[lev] = totuc[lev] - totdc[lev];
    const int l = lev - 1;
    out.htr[l] = T.heatfac * (fnet[l] - fnet[lev]) / (c.pz[l] - c.pz[lev]);
    out.htrc[l] = T.heatfac * (fnetc[l] - fnetc[lev]) / (c.pz[l] - c.pz[lev]);
  }
  out.totu = totu;
  out.totd = totd;
  out.dtotu_dt = dtotu_dt;
  out.totuc = totuc;
  out.totdc = totdc;
  out.dtotuc_dt = dtotuc_dt;
}

void lw_column(const LwInput& in, int iplon, int idrv, LwColumn& c, LwOut& out) {
  lw_inatm(in, iplon, c);
  lw_setcoef(c, idrv);
  lw_taumol(c);
  // iaer = 10: taut = taug + taua(ngb(ig))  (:508-520)
  int ig = 1;
  for (int b = 1; b <= 16; ++b)
    for (; ig <= g_lw.ngs[b]; ++ig)
      for (int k = 1; k <= c.nlayers; ++k) c.taut[ig][k] = c.taug[ig][k] + c.taua[b][k];
  // icld = 1: rtrn (random overlap); icld = 2, 3: rtrnmr with clouds
  // (maximum/random overlap); clear sky: rtrnmr (:527-541)
  // McICA: rtrnmc whatever the overlap (rrtmg_lw_rad.f90:543), the overlap
  // being in the sub-columns already
  if (c.mcica || in.icld == 1) {
    lw_rtrn(c, idrv, out);
  } else if (in.icld >= 2) {
    lw_rtrnmr_cld(c, idrv, out);
  } else {
    lw_rtrnmr(c, idrv, out);
    out.totuc = out.totu;
    out.totdc = out.totd;
    out.htrc = out.htr;
    out.dtotuc_dt = out.dtotu_dt;
  }
}

}  // namespace orc
