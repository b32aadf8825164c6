// CPU oracle, C entry points -- TEST INFRASTRUCTURE ONLY.  Called (via
// ctypes) by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg.
// The argument lists follow rrtmg_lw (rrtmg_lw_rad.nomcica.f90:80-89) and
// rrtmg_sw (rrtmg_sw_rad.nomcica.f90:78-88), and for the McICA entry points
// the McICA drivers' (rrtmg_lw_rad.f90:80-276, rrtmg_sw_rad.f90:80-90); arrays
// are column-major with the column index fastest.  Columns run in parallel
// with OpenMP (the reference loops over them serially, :453 / :500).
#include <chrono>
#include <cstdio>
#include <exception>

#include "oracle_lw.hpp"
#include "oracle_sw.hpp"

#ifdef _OPENMP
#include <omp.h>
#endif

using namespace orc;

static Blob g_blob;
static int g_ready = 0;

extern "C" int orc_max_threads();

// Every column of an LW call, in parallel; true where cldprop / cldprmc
// stopped in some column.
static int lw_columns(const LwInput& in, int idrv, double* uflx, double* dflx, double* hr, double* uflxc,
                      double* dflxc, double* hrc, double* duflx_dt, double* duflxc_dt, int nthreads) {
  const int ncol = in.ncol, nlay = in.nlay;
  int stopped = 0;
#pragma omp parallel num_threads(nthreads > 0 ? nthreads : orc_max_threads()) reduction(| : stopped)
  {
    LwColumn c;
    LwOut o;
#pragma omp for schedule(dynamic, 16)
    for (int iplon = 0; iplon < ncol; ++iplon) {
      lw_column(in, iplon, idrv, c, o);
      if (c.cld_error) stopped = 1;
      for (int k = 0; k <= nlay; ++k) {
        size_t ix = (size_t)iplon + (size_t)ncol * (size_t)k;
        uflx[ix] = o.totu[k];
        dflx[ix] = o.totd[k];
        uflxc[ix] = o.totuc[k];
        dflxc[ix] = o.totdc[k];
        if (idrv == 1 && duflx_dt) {
          duflx_dt[ix] = o.dtotu_dt[k];
          if (duflxc_dt) duflxc_dt[ix] = o.dtotuc_dt[k];
        }
      }
      for (int k = 0; k < nlay; ++k) {
        size_t ix = (size_t)iplon + (size_t)ncol * (size_t)k;
        hr[ix] = o.htr[k];
        hrc[ix] = o.htrc[k];
      }
    }
  }
  return stopped;
}

// Every column of an SW call, in parallel; *partial / *stopped as sw_column
// reports them for some column.
static void sw_columns(const SwInput& in, double* swuflx, double* swdflx, double* swhr, double* swuflxc,
                       double* swdflxc, double* swhrc, int nthreads, int* partial_out, int* stopped_out) {
  const int ncol = in.ncol, nlay = in.nlay;
  int partial = 0, stopped = 0;
#pragma omp parallel num_threads(nthreads > 0 ? nthreads : orc_max_threads()) reduction(| : partial, stopped)
  {
    SwColumn c;
    SwOut o;
#pragma omp for schedule(dynamic, 16)
    for (int iplon = 0; iplon < ncol; ++iplon) {
      bool part = false, stop = false;
      sw_column(in, iplon, c, o, &part, &stop);
      if (part) partial = 1;
      if (stop) stopped = 1;
      for (int k = 1; k <= nlay + 1; ++k) {
        size_t ix = (size_t)iplon + (size_t)ncol * (size_t)(k - 1);
        swuflx[ix] = o.fu[k];
        swdflx[ix] = o.fd[k];
        swuflxc[ix] = o.cu[k];
        swdflxc[ix] = o.cd[k];
      }
      for (int k = 1; k <= nlay; ++k) {
        size_t ix = (size_t)iplon + (size_t)ncol * (size_t)(k - 1);
        swhr[ix] = o.hr[k];
        swhrc[ix] = o.hrc[k];
      }
    }
  }
  *partial_out = partial;
  *stopped_out = stopped;
}

extern "C" {

int orc_init(const char* blob_path, double cpdair) {
  try {
    g_blob = Blob();
    g_blob.load(blob_path);
    lw_init(g_blob, cpdair);
    sw_init(g_blob, cpdair);
    g_ready = 1;
    return 0;
  } catch (const std::exception& e) {
    std::fprintf(stderr, "orc_init: %s\n", e.what());
    return 1;
  }
}

void orc_set_table_mode(int use_tables) { g_table_mode = use_tables ? 1 : 0; }

int orc_max_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

int orc_rrtmg_lw(int ncol, int nlay, int icld, int idrv, const double* play, const double* plev,
                 const double* tlay, const double* tlev, const double* tsfc, const double* h2ovmr,
                 const double* o3vmr, const double* co2vmr, const double* ch4vmr, const double* n2ovmr,
                 const double* o2vmr, const double* cfc11vmr, const double* cfc12vmr, const double* cfc22vmr,
                 const double* ccl4vmr, const double* emis, const double* tauaer, double* uflx, double* dflx,
                 double* hr, double* uflxc, double* dflxc, double* hrc, double* duflx_dt, double* duflxc_dt,
                 int nthreads, const double* cldfr, const double* taucld, const double* cicewp,
                 const double* cliqwp, int inflag, int iceflag, int liqflag, const double* reice,
                 const double* reliq) {
  if (!g_ready) return 2;
  if (icld != 0 && !(icld >= 1 && icld <= 3 && cldfr)) return 3;
  if (icld != 0 && inflag == 0 && !taucld) return 3;
  if (icld != 0 && inflag >= 1 && !(cicewp && cliqwp)) return 3;
  if (icld != 0 && inflag == 2 && !(iceflag >= 0 && iceflag <= 3 && liqflag >= 0 && liqflag <= 1 && reice && reliq))
    return 3;
  LwInput in{ncol, nlay, play, plev, tlay, tlev, tsfc, h2ovmr, o3vmr, co2vmr, ch4vmr, n2ovmr, o2vmr,
             cfc11vmr, cfc12vmr, cfc22vmr, ccl4vmr, emis, tauaer};
  in.icld = icld;
  in.cldfr = cldfr;
  in.taucld = taucld;
  in.cicewp = cicewp;
  in.cliqwp = cliqwp;
  in.inflag = inflag;
  in.iceflag = iceflag;
  in.liqflag = liqflag;
  in.reice = reice;
  in.reliq = reliq;
  const int stopped = lw_columns(in, idrv, uflx, dflx, hr, uflxc, dflxc, hrc, duflx_dt, duflxc_dt, nthreads);
  return stopped ? 5 : 0;  // 5: cldprop stopped (an effective radius out of range)
}

// McICA rrtmg_lw (rrtmg_lw_rad.f90:80-276): the clear-sky inputs of
// orc_rrtmg_lw with the sub-column clouds cldfmcl, taucmcl, ciwpmcl, clwpmcl
// (140, ncol, nlay), reicmcl / relqmcl (ncol, nlay), cldprmc's inflag 0 / 2
// (1 stops) and rtrnmc.  Returns 3 for a bad argument, 5 where cldprmc stops.
int orc_rrtmg_lw_mcica(int ncol, int nlay, int icld, int idrv, const double* play, const double* plev,
                       const double* tlay, const double* tlev, const double* tsfc, const double* h2ovmr,
                       const double* o3vmr, const double* co2vmr, const double* ch4vmr, const double* n2ovmr,
                       const double* o2vmr, const double* cfc11vmr, const double* cfc12vmr,
                       const double* cfc22vmr, const double* ccl4vmr, const double* emis, int inflag, int iceflag,
                       int liqflag, const double* cldfmcl, const double* taucmcl, const double* ciwpmcl,
                       const double* clwpmcl, const double* reicmcl, const double* relqmcl, const double* tauaer,
                       double* uflx, double* dflx, double* hr, double* uflxc, double* dflxc, double* hrc,
                       double* duflx_dt, double* duflxc_dt, int nthreads) {
  if (!g_ready) return 2;
  if (icld != 0 && !cldfmcl) return 3;
  LwInput in{ncol, nlay, play, plev, tlay, tlev, tsfc, h2ovmr, o3vmr, co2vmr, ch4vmr, n2ovmr, o2vmr,
             cfc11vmr, cfc12vmr, cfc22vmr, ccl4vmr, emis, tauaer};
  in.icld = icld;
  in.inflag = inflag;
  in.iceflag = iceflag;
  in.liqflag = liqflag;
  in.mcica = true;
  in.cldfmcl = cldfmcl;
  in.taucmcl = taucmcl;
  in.ciwpmcl = ciwpmcl;
  in.clwpmcl = clwpmcl;
  in.reicmcl = reicmcl;
  in.relqmcl = relqmcl;
  const int stopped = lw_columns(in, idrv, uflx, dflx, hr, uflxc, dflxc, hrc, duflx_dt, duflxc_dt, nthreads);
  return stopped ? 5 : 0;
}

int orc_rrtmg_sw(int ncol, int nlay, int icld, int iaer, const double* play, const double* plev,
                 const double* tlay, const double* tlev, const double* tsfc, const double* h2ovmr,
                 const double* o3vmr, const double* co2vmr, const double* ch4vmr, const double* n2ovmr,
                 const double* o2vmr, const double* asdir, const double* asdif, const double* aldir,
                 const double* aldif, const double* coszen, double adjes, int dyofyr, double scon,
                 const double* tauaer, const double* ssaaer, const double* asmaer, double* swuflx,
                 double* swdflx, double* swhr, double* swuflxc, double* swdflxc, double* swhrc, int nthreads,
                 const double* cldfr, const double* taucld, const double* ssacld, const double* asmcld,
                 const double* fsfcld, const double* cicewp, const double* cliqwp, int inflag, int iceflag,
                 int liqflag, const double* reice, const double* reliq) {
  if (!g_ready) return 2;
  if (icld != 0 && !(icld == 1 && cldfr)) return 3;
  if (icld != 0 && inflag == 0 && !(taucld && ssacld && asmcld && fsfcld)) return 3;
  if (icld != 0 && inflag == 2 &&
      !(iceflag >= 1 && iceflag <= 3 && liqflag == 1 && cicewp && cliqwp && reice && reliq))
    return 3;
  if (icld != 0 && inflag != 0 && inflag != 2) return 3;
  if (iaer != 0 && iaer != 10) return 3;
  SwInput in{ncol, nlay, iaer, dyofyr, adjes, scon, play, plev, tlay, tlev, tsfc, h2ovmr, o3vmr, co2vmr,
             ch4vmr, n2ovmr, o2vmr, asdir, asdif, aldir, aldif, coszen, tauaer, ssaaer, asmaer};
  in.icld = icld;
  in.cldfr = cldfr;
  in.taucld = taucld;
  in.ssacld = ssacld;
  in.asmcld = asmcld;
  in.fsfcld = fsfcld;
  in.cicewp = cicewp;
  in.cliqwp = cliqwp;
  in.inflag = inflag;
  in.iceflag = iceflag;
  in.liqflag = liqflag;
  in.reice = reice;
  in.reliq = reliq;
  int partial = 0, stopped = 0;
  sw_columns(in, swuflx, swdflx, swhr, swuflxc, swdflxc, swhrc, nthreads, &partial, &stopped);
  // 5: cldprop_sw stopped (a size out of its range); 4: a partly cloudy
  // layer (the reference's non-McICA SW stops)
  return stopped ? 5 : partial ? 4 : 0;
}

// McICA rrtmg_sw (rrtmg_sw_rad.f90:80-90): the argument list of orc_rrtmg_sw
// with the sub-column clouds cldfmcl, taucmcl, ssacmcl, asmcmcl, fsfcmcl,
// ciwpmcl, clwpmcl (112, ncol, nlay) in place of the layer clouds, reicmcl /
// relqmcl (ncol, nlay); cldprmc_sw's inflag 0 (optics given) or 2 (iceflag
// 1..3, liqflag 1).  Returns 3 for missing or invalid inputs, 5 where
// cldprmc_sw stops.
int orc_rrtmg_sw_mcica(int ncol, int nlay, int icld, int iaer, const double* play, const double* plev,
                       const double* tlay, const double* tlev, const double* tsfc, const double* h2ovmr,
                       const double* o3vmr, const double* co2vmr, const double* ch4vmr, const double* n2ovmr,
                       const double* o2vmr, const double* asdir, const double* asdif, const double* aldir,
                       const double* aldif, const double* coszen, double adjes, int dyofyr, double scon,
                       int inflag, int iceflag, int liqflag, const double* cldfmcl, const double* taucmcl,
                       const double* ssacmcl, const double* asmcmcl, const double* fsfcmcl,
                       const double* ciwpmcl, const double* clwpmcl, const double* reicmcl,
                       const double* relqmcl, const double* tauaer, const double* ssaaer, const double* asmaer,
                       double* swuflx, double* swdflx, double* swhr, double* swuflxc, double* swdflxc,
                       double* swhrc, int nthreads) {
  if (!g_ready) return 2;
  if (icld != 0 && !cldfmcl) return 3;
  if (icld != 0 && inflag == 0 && !(taucmcl && ssacmcl && asmcmcl && fsfcmcl)) return 3;
  if (icld != 0 && inflag == 2 &&
      !(iceflag >= 1 && iceflag <= 3 && liqflag == 1 && ciwpmcl && clwpmcl && reicmcl && relqmcl))
    return 3;
  if (iaer != 0 && iaer != 10) return 3;
  SwInput in{ncol, nlay, iaer, dyofyr, adjes, scon, play, plev, tlay, tlev, tsfc, h2ovmr, o3vmr, co2vmr,
             ch4vmr, n2ovmr, o2vmr, asdir, asdif, aldir, aldif, coszen, tauaer, ssaaer, asmaer};
  in.icld = icld;
  in.inflag = inflag;
  in.iceflag = iceflag;
  in.liqflag = liqflag;
  in.reice = reicmcl;
  in.reliq = relqmcl;
  in.mcica = true;
  in.cldfmcl = cldfmcl;
  in.taucmcl = taucmcl;
  in.ssacmcl = ssacmcl;
  in.asmcmcl = asmcmcl;
  in.fsfcmcl = fsfcmcl;
  in.ciwpmcl = ciwpmcl;
  in.clwpmcl = clwpmcl;
  int partial = 0, stopped = 0;
  sw_columns(in, swuflx, swdflx, swhr, swuflxc, swdflxc, swhrc, nthreads, &partial, &stopped);
  return stopped ? 5 : 0;
}

// Clear-sky rrtmg_lw per band: bandu/bandd/dbandu_dt (ncol, nlay+1, 16) are the
// 16 bands' upward and downward fluxes and d(upward)/d(tsfc) (written when
// idrv = 1), in W/m2, the per-band blocks the standalone RRTMG_LW prints.
int orc_rrtmg_lw_bands(int ncol, int nlay, int idrv, const double* play, const double* plev, const double* tlay,
                       const double* tlev, const double* tsfc, const double* h2ovmr, const double* o3vmr,
                       const double* co2vmr, const double* ch4vmr, const double* n2ovmr, const double* o2vmr,
                       const double* cfc11vmr, const double* cfc12vmr, const double* cfc22vmr,
                       const double* ccl4vmr, const double* emis, double* bandu, double* bandd,
                       double* dbandu_dt) {
  if (!g_ready) return 2;
  LwInput in{ncol, nlay, play, plev, tlay, tlev, tsfc, h2ovmr, o3vmr, co2vmr, ch4vmr, n2ovmr, o2vmr,
             cfc11vmr, cfc12vmr, cfc22vmr, ccl4vmr, emis, nullptr};
  const size_t nlev = (size_t)nlay + 1;
  for (int iplon = 0; iplon < ncol; ++iplon) {
    LwColumn c;
    LwOut o;
    o.want_bands = true;
    o.bandu.assign(16 * nlev, 0.0);
    o.bandd.assign(16 * nlev, 0.0);
    o.dbandu_dt.assign(16 * nlev, 0.0);
    lw_column(in, iplon, idrv, c, o);
    for (size_t b = 0; b < 16; ++b)
      for (size_t k = 0; k < nlev; ++k) {
        size_t ix = (size_t)iplon + (size_t)ncol * (k + nlev * b);
        bandu[ix] = o.bandu[b * nlev + k];
        bandd[ix] = o.bandd[b * nlev + k];
        if (idrv == 1 && dbandu_dt) dbandu_dt[ix] = o.dbandu_dt[b * nlev + k];
      }
  }
  return 0;
}

// Where the time goes: the clear-sky path's phases timed separately, one
// thread, summed over the columns, in nanoseconds (integer clock ticks, so
// that the FLOP-count build compiles the same code).  LW: ns[0..3] = inatm,
// setcoef, taumol (with the aerosol add), rtrnmr.  SW: ns[0..3] = inatm_sw,
// setcoef_sw, taumol_sw, spcvrt_sw without its taumol call plus the heating
// rates; dark columns are skipped, as in rrtmg_sw.
static long long ticks(std::chrono::steady_clock::time_point a, std::chrono::steady_clock::time_point b) {
  return (long long)std::chrono::duration_cast<std::chrono::nanoseconds>(b - a).count();
}

int orc_lw_phase_times(int ncol, int nlay, const double* play, const double* plev, const double* tlay,
                       const double* tlev, const double* tsfc, const double* h2ovmr, const double* o3vmr,
                       const double* co2vmr, const double* ch4vmr, const double* n2ovmr, const double* o2vmr,
                       const double* cfc11vmr, const double* cfc12vmr, const double* cfc22vmr,
                       const double* ccl4vmr, const double* emis, long long* ns) {
  if (!g_ready) return 2;
  LwInput in{ncol, nlay, play, plev, tlay, tlev, tsfc, h2ovmr, o3vmr, co2vmr, ch4vmr, n2ovmr, o2vmr,
             cfc11vmr, cfc12vmr, cfc22vmr, ccl4vmr, emis, nullptr};
  for (int k = 0; k < 4; ++k) ns[k] = 0;
  LwColumn c;
  LwOut o;
  using clk = std::chrono::steady_clock;
  for (int iplon = 0; iplon < ncol; ++iplon) {
    const auto t0 = clk::now();
    lw_inatm(in, iplon, c);
    const auto t1 = clk::now();
    lw_setcoef(c, 0);
    const auto t2 = clk::now();
    lw_taumol(c);
    int ig = 1;
    for (int b = 1; b <= 16; ++b)
      for (; ig <= g_lw.ngs[b]; ++ig)
        for (int k = 1; k <= c.nlayers; ++k) c.taut[ig][k] = c.taug[ig][k] + c.taua[b][k];
    const auto t3 = clk::now();
    lw_rtrnmr(c, 0, o);
    const auto t4 = clk::now();
    ns[0] += ticks(t0, t1);
    ns[1] += ticks(t1, t2);
    ns[2] += ticks(t2, t3);
    ns[3] += ticks(t3, t4);
  }
  return 0;
}

int orc_sw_phase_times(int ncol, int nlay, const double* play, const double* plev, const double* tlay,
                       const double* tlev, const double* tsfc, const double* h2ovmr, const double* o3vmr,
                       const double* co2vmr, const double* ch4vmr, const double* n2ovmr, const double* o2vmr,
                       const double* asdir, const double* asdif, const double* aldir, const double* aldif,
                       const double* coszen, double adjes, int dyofyr, double scon, long long* ns) {
  if (!g_ready) return 2;
  SwInput in{ncol, nlay, 0, dyofyr, adjes, scon, play, plev, tlay, tlev, tsfc, h2ovmr, o3vmr, co2vmr,
             ch4vmr, n2ovmr, o2vmr, asdir, asdif, aldir, aldif, coszen, nullptr, nullptr, nullptr};
  for (int k = 0; k < 4; ++k) ns[k] = 0;
  SwColumn c;
  SwOut o;
  using clk = std::chrono::steady_clock;
  for (int iplon = 0; iplon < ncol; ++iplon) {
    if (in.coszen[iplon] < 1.e-10) continue;
    const auto t0 = clk::now();
    sw_inatm(in, iplon, c);
    const auto t1 = clk::now();
    sw_setcoef(c);
    const auto t2 = clk::now();
    sw_taumol(c);
    const auto t3 = clk::now();
    double albdir[15], albdif[15];
    for (int ib = 1; ib <= 14; ++ib) {
      const bool vis = ib >= 10 && ib <= 13;
      albdir[ib] = vis ? in.asdir[iplon] : in.aldir[iplon];
      albdif[ib] = vis ? in.asdif[iplon] : in.aldif[iplon];
    }
    sw_spcvrt(c, in.coszen[iplon], albdir, albdif, o, false);
    o.hr.assign(nlay + 1, 0.);
    for (int i = 1; i < nlay; ++i) o.hr[i] = (o.fd[i + 1] - o.fu[i + 1] - (o.fd[i] - o.fu[i])) * (g_sw.heatfac / c.pdp[i]);
    const auto t4 = clk::now();
    ns[0] += ticks(t0, t1);
    ns[1] += ticks(t1, t2);
    ns[2] += ticks(t2, t3);
    ns[3] += ticks(t3, t4);
  }
  return 0;
}

// Gas optics only (stage parity): taug/fracs (ncol, nlay, 140), laytrop (ncol).
int orc_lw_optics(int ncol, int nlay, const double* play, const double* plev, const double* tlay,
                  const double* tlev, const double* tsfc, const double* h2ovmr, const double* o3vmr,
                  const double* co2vmr, const double* ch4vmr, const double* n2ovmr, const double* o2vmr,
                  double* taug, double* fracs, int* laytrop) {
  if (!g_ready) return 2;
  LwInput in{ncol, nlay, play, plev, tlay, tlev, tsfc, h2ovmr, o3vmr, co2vmr, ch4vmr, n2ovmr, o2vmr,
             nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
#pragma omp parallel
  {
    LwColumn c;
#pragma omp for
    for (int iplon = 0; iplon < ncol; ++iplon) {
      lw_inatm(in, iplon, c);
      lw_setcoef(c, 0);
      lw_taumol(c);
      laytrop[iplon] = c.laytrop;
      for (int g = 1; g <= 140; ++g)
        for (int k = 1; k <= nlay; ++k) {
          size_t ix = (size_t)iplon + (size_t)ncol * ((size_t)(k - 1) + (size_t)nlay * (size_t)(g - 1));
          taug[ix] = c.taug[g][k];
          fracs[ix] = c.fracs[g][k];
        }
    }
  }
  return 0;
}

// Gas optics only: taug/taur (ncol, nlay, 112), sfluxzen (ncol, 112).
int orc_sw_optics(int ncol, int nlay, const double* play, const double* plev, const double* tlay,
                  const double* tlev, const double* tsfc, const double* h2ovmr, const double* o3vmr,
                  const double* co2vmr, const double* ch4vmr, const double* n2ovmr, const double* o2vmr,
                  double* taug, double* taur, double* sfluxzen) {
  if (!g_ready) return 2;
  SwInput in{ncol, nlay, 0, 0, 1.0, 1368.22, play, plev, tlay, tlev, tsfc, h2ovmr, o3vmr, co2vmr,
             ch4vmr, n2ovmr, o2vmr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
#pragma omp parallel
  {
    SwColumn c;
#pragma omp for
    for (int iplon = 0; iplon < ncol; ++iplon) {
      sw_inatm(in, iplon, c);
      sw_setcoef(c);
      sw_taumol(c);
      for (int g = 1; g <= 112; ++g) {
        sfluxzen[(size_t)iplon + (size_t)ncol * (size_t)(g - 1)] = c.sfluxzen[g];
        for (int k = 1; k <= nlay; ++k) {
          size_t ix = (size_t)iplon + (size_t)ncol * ((size_t)(k - 1) + (size_t)nlay * (size_t)(g - 1));
          taug[ix] = c.taug[g][k];
          taur[ix] = c.taur[g][k];
        }
      }
    }
  }
  return 0;
}

// Reduced table access: key like "lw03" / "sw24", name like "ka", "fracrefa".
// Returns the element count (copies at most n values), or -1.
int orc_table(const char* key, const char* name, double* out, int n) {
  if (!g_ready) return -1;
  std::string k(key), nm(name);
  const FArr* a = nullptr;
  int b = std::atoi(k.c_str() + 2);
  if (k.rfind("lw", 0) == 0 && b >= 1 && b <= 16) {
    auto it = g_lw.t[b].find(nm);
    if (it != g_lw.t[b].end()) a = &it->second;
  } else if (k.rfind("sw", 0) == 0 && b >= 16 && b <= 29) {
    auto it = g_sw.t[b].find(nm);
    if (it != g_sw.t[b].end()) a = &it->second;
  }
  if (!a) return -1;
  int m = (int)a->v.size();
  for (int i = 0; i < m && i < n; ++i) out[i] = a->v[i];
  return m;
}

}  // extern "C"
