// Device side of MiMA's radiation driver run_rrtmg
// (src/atmos_param/rrtm_radiation/rrtm_radiation.f90:464-834) with the
// half-level temperature of interp_temp (:420-460) and the zenith angle of
// compute_zenith (astro.f90:59-248): kernels that turn the GCM state of one
// slab into RRTM columns and the RRTM results back into GCM tendencies and
// surface fluxes (driver.cu).
#pragma once
#include <cuda_runtime.h>

namespace rrtmg {

// GCM arrays are Fortran (si, sj[, sk or sk+1]) with the longitude index
// fastest; level k = 1 is the model top.
struct RunGcm {
  const double *lat, *lon;                    // (si, sj) radians
  const double *p_full, *p_half;              // Pa
  const double *z_full, *z_half;              // m (interp_temp)
  const double *t, *q, *o3;                   // K, kg/kg, O3 mmr (o3 may be null: o3_val)
  const double *t_surf, *albedo, *precip;     // (si, sj); precip may be null
};

// RRTM columns: (ncol, nlay) / (ncol, nlay+1) / (ncol) / (ncol, 16), column
// index fastest, layer 1 at the surface.
struct RunCols {
  double *play, *plev, *tlay, *tlev, *tsfc, *h2o, *o3, *co2, *emis, *alb, *cosz;
  double* gas[7];  // ch4, n2o, o2, cfc11, cfc12, cfc22, ccl4 (null when zero)
};

struct RunRad {
  const double *uflx, *dflx, *hr, *swuflx, *swdflx, *swhr;
};

struct RunOut {
  double *tdt, *coszen, *flux_sw, *flux_lw, *t_half, *tdt_rad, *tdt_sw, *tdt_lw, *olr, *isr;
};

struct RunScalars {
  int si, sj, sk, lonstep, nsub, ncol;
  // compute_zenith
  double radsec, dt_pi, dec_sin, dec_cos, dec_tan, radpersec;
  int zen_dt;
  // input preparation
  int zm_tracers, fixed_water, secondary, precip_albedo, zm_rad;
  double h2o_lo, t_lo, t_hi, co2, o3_val, fixed_water_val, fixed_water_pres, fixed_water_lat;
  double precip_albedo_val, precip_lat;
  int num_precip;
  double gas_val[7];
};

// Zenith angle of every GCM point; per latitude the zonal sums of q
// (do_zm_tracers) and of precipitation (do_precip_albedo); the top-interface
// flag (some top p_half <= 0).  zq (sj, sk), zp (sj) and flag are scratch.
void launch_run_zonal(const RunScalars& s, const RunGcm& g, double* coszen, double* zq, double* zp, unsigned* flag,
                      cudaStream_t st);
// GCM slab -> RRTM columns (lonstep subsampling, flip, hPa, top fix, clamps).
void launch_run_prep(const RunScalars& s, const RunGcm& g, const double* coszen, const double* zq,
                     const double* zp, const unsigned* flag, const RunCols& c, cudaStream_t st);
// interp_temp on the whole slab (the t_half output).
void launch_run_thalf(const RunScalars& s, const RunGcm& g, double* t_half, cudaStream_t st);
// do_zm_rad: zonal means of the heating (sj, sk) and surface fluxes (sj).
void launch_run_zonal_rad(const RunScalars& s, const RunRad& r, double* zt, double* zsw, double* zlw,
                          cudaStream_t st);
// RRTM results -> GCM tendencies (tdt += ...), surface fluxes, diagnostics.
void launch_run_post(const RunScalars& s, const RunRad& r, const double* zt, const double* zsw, const double* zlw,
                     const RunOut& o, cudaStream_t st);

}  // namespace rrtmg
