// FLOP-count build of the oracle only (make opcount) -- TEST INFRASTRUCTURE
// ONLY.  Reads and clears the calling thread's operation counters of
// opcount.hpp; run the counted calls with one thread.
#include "oracle_lw.hpp"
#include "oracle_sw.hpp"

using namespace orc;

namespace {

// Adds the counters' growth since `before` to acc[0..NKIND) and moves
// `before` to the current counts.
void take(unsigned long long* acc, unsigned long long* before) {
  for (int k = 0; k < opc::NKIND; ++k) {
    acc[k] += opc::g_count[k] - before[k];
    before[k] = opc::g_count[k];
  }
}

}  // namespace

extern "C" {

void orc_opcount_reset() {
  for (int k = 0; k < opc::NKIND; ++k) opc::g_count[k] = 0;
}

void orc_opcount_get(unsigned long long* out) {
  for (int k = 0; k < opc::NKIND; ++k) out[k] = opc::g_count[k];
}

// Operations by phase, summed over the columns, out[phase * NKIND + kind]:
// LW phases inatm, setcoef, taumol (with the aerosol add), rtrnmr -- the
// phases of rrtmg_lw's column loop (rrtmg_lw_rad.nomcica.f90:453-570).
int orc_lw_phase_counts(int ncol, int nlay, const double* play, const double* plev, const double* tlay,
                        const double* tlev, const double* tsfc, const double* h2ovmr, const double* o3vmr,
                        const double* co2vmr, const double* ch4vmr, const double* n2ovmr, const double* o2vmr,
                        const double* cfc11vmr, const double* cfc12vmr, const double* cfc22vmr,
                        const double* ccl4vmr, const double* emis, unsigned long long* out) {
  LwInput in{ncol, nlay, play, plev, tlay, tlev, tsfc, h2ovmr, o3vmr, co2vmr, ch4vmr, n2ovmr, o2vmr,
             cfc11vmr, cfc12vmr, cfc22vmr, ccl4vmr, emis, nullptr};
  for (int k = 0; k < 4 * opc::NKIND; ++k) out[k] = 0;
  LwColumn c;
  LwOut o;
  unsigned long long before[opc::NKIND];
  for (int iplon = 0; iplon < ncol; ++iplon) {
    for (int k = 0; k < opc::NKIND; ++k) before[k] = opc::g_count[k];
    lw_inatm(in, iplon, c);
    take(out + 0 * opc::NKIND, before);
    lw_setcoef(c, 0);
    take(out + 1 * opc::NKIND, before);
    lw_taumol(c);
    int ig = 1;
    for (int b = 1; b <= 16; ++b)
      for (; ig <= g_lw.ngs[b]; ++ig)
        for (int k = 1; k <= c.nlayers; ++k) c.taut[ig][k] = c.taug[ig][k] + c.taua[b][k];
    take(out + 2 * opc::NKIND, before);
    lw_rtrnmr(c, 0, o);
    take(out + 3 * opc::NKIND, before);
  }
  return 0;
}

// SW phases inatm_sw, setcoef_sw, taumol_sw, spcvrt_sw (one two-stream pass:
// the reference's second, "total" pass is not counted, as in the whole-path
// count) with the heating rates; dark columns are skipped, as in rrtmg_sw.
int orc_sw_phase_counts(int ncol, int nlay, const double* play, const double* plev, const double* tlay,
                        const double* tlev, const double* tsfc, const double* h2ovmr, const double* o3vmr,
                        const double* co2vmr, const double* ch4vmr, const double* n2ovmr, const double* o2vmr,
                        const double* asdir, const double* asdif, const double* aldir, const double* aldif,
                        const double* coszen, double adjes, int dyofyr, double scon, unsigned long long* out) {
  SwInput in{ncol, nlay, 0, dyofyr, adjes, scon, play, plev, tlay, tlev, tsfc, h2ovmr, o3vmr, co2vmr,
             ch4vmr, n2ovmr, o2vmr, asdir, asdif, aldir, aldif, coszen, nullptr, nullptr, nullptr};
  for (int k = 0; k < 4 * opc::NKIND; ++k) out[k] = 0;
  SwColumn c;
  SwOut o;
  unsigned long long before[opc::NKIND];
  for (int iplon = 0; iplon < ncol; ++iplon) {
    if (coszen[iplon] < 1.e-10) continue;
    for (int k = 0; k < opc::NKIND; ++k) before[k] = opc::g_count[k];
    sw_inatm(in, iplon, c);
    take(out + 0 * opc::NKIND, before);
    sw_setcoef(c);
    take(out + 1 * opc::NKIND, before);
    sw_taumol(c);
    take(out + 2 * opc::NKIND, before);
    double albdir[15], albdif[15];
    for (int ib = 1; ib <= 14; ++ib) {
      const bool vis = ib >= 10 && ib <= 13;
      albdir[ib] = vis ? asdir[iplon] : aldir[iplon];
      albdif[ib] = vis ? asdif[iplon] : aldif[iplon];
    }
    sw_spcvrt(c, coszen[iplon], albdir, albdif, o, false);
    o.hr.assign(nlay + 1, 0.);
    for (int i = 1; i < nlay; ++i) o.hr[i] = (o.fd[i + 1] - o.fu[i + 1] - (o.fd[i] - o.fu[i])) * (g_sw.heatfac / c.pdp[i]);
    take(out + 3 * opc::NKIND, before);
  }
  return 0;
}

}  // extern "C"
