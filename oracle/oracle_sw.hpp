// CPU oracle, shortwave: data structures.  TEST INFRASTRUCTURE ONLY.
#pragma once
#include <map>
#include <string>
#include <vector>

#include "oracle_tables.hpp"

namespace orc {

extern int g_table_mode;

struct SwTables {
  std::map<std::string, FArr> t[30];  // reduced per-band tables, bands 16..29
  FArr preflog, tref;
  int ngc[30], ngs[30], nspa[30], nspb[30];
  double exp_tbl[10001];
  double bpade, heatfac, oneminus, grav, avogad, pi;
  // cloud optical properties (rrsw_cld: swcldpr, rrtmg_sw_init.f90:1519-3341)
  // and the band limits (wavenum2) that select the Ebert-Curry coefficients
  FArr extliq1, ssaliq1, asyliq1, extice2, ssaice2, asyice2, extice3, ssaice3, asyice3, fdlice3;
  FArr abari, bbari, cbari, dbari, ebari, fbari, wavenum2;
};
extern SwTables g_sw;

// Arguments of rrtmg_sw (rrtmg_sw_rad.nomcica.f90:78-88); aerosol arrays are
// (ncol, nlay, 14) and used when iaer = 10.
struct SwInput {
  int ncol, nlay, iaer, dyofyr;
  double adjes, scon;
  const double *play, *plev, *tlay, *tlev, *tsfc, *h2ovmr, *o3vmr, *co2vmr, *ch4vmr, *n2ovmr, *o2vmr;
  const double *asdir, *asdif, *aldir, *aldif, *coszen;
  const double *tauaer, *ssaaer, *asmaer;
  // Clouds (icld = 1, inflgsw = 0): cldfr (ncol, nlay); taucld, ssacld, asmcld,
  // fsfcld (14, ncol, nlay); cicewp / cliqwp (ncol, nlay) or null.
  int icld = 0;
  const double *cldfr = nullptr, *taucld = nullptr, *ssacld = nullptr, *asmcld = nullptr, *fsfcld = nullptr,
               *cicewp = nullptr, *cliqwp = nullptr;
  // cloud physics (inflag = 2: ice and liquid parameterisations selected by
  // iceflag (1..3) and liqflag (1), effective sizes reice / reliq)
  int inflag = 0, iceflag = 0, liqflag = 0;
  const double *reice = nullptr, *reliq = nullptr;
  // McICA (rrtmg_sw_rad.f90:80-90): sub-column clouds, one per g-point, in
  // place of cldfr / taucld / ... -- cldfmcl, taucmcl, ssacmcl, asmcmcl,
  // fsfcmcl, ciwpmcl, clwpmcl (112, ncol, nlay); reice / reliq as above.
  bool mcica = false;
  const double *cldfmcl = nullptr, *taucmcl = nullptr, *ssacmcl = nullptr, *asmcmcl = nullptr,
               *fsfcmcl = nullptr, *ciwpmcl = nullptr, *clwpmcl = nullptr;
};

struct SwColumn {
  int nlayers = 0, laytrop = 0, laylow = 0;
  double tbound = 0;
  double adjflux[30];
  std::vector<double> pavel, tavel, pz, tz, pdp, coldry;
  std::vector<double> wkl[8], taua[15], ssaa[15], asma[15];
  std::vector<int> jp, jt, jt1, indself, indfor;
  std::vector<double> colh2o, colco2, colo3, coln2o, colch4, colo2, colmol;
  std::vector<double> fac00, fac01, fac10, fac11, selffac, selffrac, forfac, forfrac;
  std::vector<double> taug[113], taur[113];
  // clouds: cover and cldprop_sw's delta-scaled cloud optics per band (ibm 1..14)
  std::vector<double> pclfr, ptauc[15], pomgc[15], pasyc[15];
  // McICA: cover and cldprmc_sw's delta-scaled optics per g-point,
  // [(iw - 1) * (nlayers + 2) + lay]
  bool mcica = false;
  std::vector<double> cldfmc, taucmc, ssacmc, asmcmc;
  // a call with clouds: its total-sky two-stream pass is work of its own
  // (the op-counting build counts it; in clear sky it repeats the clear pass)
  bool total_pass = false;
  double sfluxzen[113];

  void resize(int nl) {
    auto r = [&](std::vector<double>& v) { v.assign(nl + 2, 0.0); };
    auto ri = [&](std::vector<int>& v) { v.assign(nl + 2, 0); };
    r(pavel); r(tavel); r(pz); r(tz); r(pdp); r(coldry);
    for (auto& v : wkl) r(v);
    for (auto& v : taua) r(v);
    for (auto& v : ssaa) r(v);
    for (auto& v : asma) r(v);
    ri(jp); ri(jt); ri(jt1); ri(indself); ri(indfor);
    r(colh2o); r(colco2); r(colo3); r(coln2o); r(colch4); r(colo2); r(colmol);
    r(fac00); r(fac01); r(fac10); r(fac11); r(selffac); r(selffrac); r(forfac); r(forfrac);
    for (auto& v : taug) r(v);
    for (auto& v : taur) r(v);
    r(pclfr);
    for (int b = 0; b < 15; ++b) {
      r(ptauc[b]);
      pomgc[b].assign(nl + 2, 1.0);
      r(pasyc[b]);
    }
    for (int g = 0; g < 113; ++g) sfluxzen[g] = 0.0;
    for (int b = 0; b < 30; ++b) adjflux[b] = 0.0;
  }
};

struct SwOut {
  std::vector<double> fu, fd, cu, cd;  // levels 1..nlay+1 (surface first)
  std::vector<double> hr, hrc;         // layers 1..nlay
};

void sw_init(const Blob& blob, double cpdair);
void sw_inatm(const SwInput& in, int iplon, SwColumn& c);
void sw_setcoef(SwColumn& c);
void sw_taumol(SwColumn& c);
// run_taumol = false: the caller has already run sw_taumol on c (the phase
// timing of the oracle); the results are the same.
void sw_spcvrt(SwColumn& c, double prmu0, const double* albdir, const double* albdif, SwOut& out,
               bool run_taumol = true);
// Returns false for a dark column (no SW); sets *partial when the column holds
// a partly cloudy layer, which the reference's non-McICA SW refuses
// (rrtmg_sw_rad.nomcica.f90:533-538).  With in.mcica the McICA driver
// (rrtmg_sw_rad.f90): cldprmc_sw and spcvmc_sw, every column computed (the
// McICA driver has no dark-column skip: cos(zenith) is clamped to 1e-10),
// partial covers allowed.
// *stopped: cldprop_sw stopped for this column (a size out of range or an
// optical property out of its physical range).
bool sw_column(const SwInput& in, int iplon, SwColumn& c, SwOut& out, bool* partial = nullptr,
               bool* stopped = nullptr);

}  // namespace orc
