/*
 * rrtmg_run.h -- MiMA's radiation driver step on the GPU: the C-ABI that
 * replaces run_rrtmg (src/atmos_param/rrtm_radiation/rrtm_radiation.f90:464-834)
 * together with the interp_temp call that precedes it in the physics driver
 * (src/atmos_param/physics_driver/physics_driver.f90:1289-1290).
 *
 * One call takes the GCM state of one slab (si longitudes x sj latitudes x sk
 * levels, the arrays run_rrtmg receives) and performs, on the device:
 *   - interp_temp (rrtm_radiation.f90:420-460): half-level temperatures;
 *   - compute_zenith (src/atmos_param/rrtm_radiation/astro.f90:59-248);
 *   - the input preparation of run_rrtmg (:596-677): do_precip_albedo,
 *     do_zm_tracers, do_fixed_water, subsampling every lonstep-th longitude,
 *     reversal to surface-first RRTM order, Pa -> hPa, the top-interface fix
 *     and the h2o / temperature clamps;
 *   - rrtmg_sw and rrtmg_lw (clear sky, iaer = 0, idrv = 0; the handle's
 *     precision and transcendental mode);
 *   - the output side (:715-815): heating in K/s interpolated back to every
 *     longitude (closed toroidally) or zonally averaged (do_zm_rad),
 *     tdt += tdt_rrtm, the surface fluxes and the diagnostics.
 *
 * Arrays are Fortran column-major with the longitude index fastest:
 * (si,sj) / (si,sj,sk) / (si,sj,sk+1); level 1 is the model top; pressures in
 * Pa, heights in m, q in kg/kg, O3 as mass mixing ratio, lat/lon in radians.
 * si must be a multiple of lonstep.
 *
 * Not on the device (left to the caller, as host control flow): the radiation
 * alarm (dt_rad, :527-547), store_intermediate_rad, the netCDF interpolators
 * (do_read_ozone, do_read_h2o, do_read_radiation, do_read_*_flux; a caller
 * that reads ozone passes the interpolated, scaled and clamped field as o3),
 * resetting rrtm_precip / num_precip after a do_precip_albedo step, and
 * write_diag_rrtm.
 */
#ifndef RRTMG_RUN_H
#define RRTMG_RUN_H

#include "rrtmg_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Namelist values run_rrtmg reads: rrtm_radiation_nml
 * (rrtm_radiation.f90:106-198) and astro_nml (astro.f90:22-31).
 * rrtmg_run_params_default fills the reference's defaults (in brackets). */
typedef struct rrtmg_run_params {
  int lonstep;                  /* [1] radiation on every lonstep-th longitude */
  int do_zm_tracers;            /* [0] zonal-mean q into the radiation */
  int do_zm_rad;                /* [0] zonal-mean heating and surface fluxes */
  int do_fixed_water;           /* [0] q = fixed_water where p_full <= fixed_water_pres*100
                                       and |lat| <= fixed_water_lat (both as the reference compares them) */
  int include_secondary_gases;  /* [0] ch4 ... ccl4 = *_val (else 0) */
  int do_precip_albedo;         /* [0] albedo from the zonal-mean precipitation in rrtm_precip */
  int num_precip;               /* [0] number of sums in rrtm_precip (caller state; 0 disables) */
  int use_dyofyr;               /* [0] Earth-Sun distance from the day of year */
  int solday;                   /* [0] > 0: perpetual day of year */
  int dt_rad_avg;               /* [86400] zenith-angle averaging interval in s (do_rad_time_avg;
                                       0 = instantaneous) */
  double h2o_lower_limit;       /* [2e-7] */
  double temp_lower_limit;      /* [100] */
  double temp_upper_limit;      /* [370] */
  double co2ppmv;               /* [300] */
  double o3_val;                /* [0] O3 mmr when no o3 field is passed */
  double fixed_water;           /* [2e-6] kg/kg */
  double fixed_water_pres;      /* [100e2] */
  double fixed_water_lat;       /* [90] */
  double ch4_val, n2o_val, o2_val, cfc11_val, cfc12_val, cfc22_val, ccl4_val; /* [0] vmr */
  double precip_albedo;         /* [0.35] */
  double precip_lat;            /* [0] degrees */
  double slowdown_rad;          /* [1] */
  double obliq;                 /* [23.439] degrees */
  double solr_cnst;             /* [1368.22] W/m2 */
  double solrad;                /* [1] Earth-Sun distance factor (adjes) */
  double equinox_day;           /* [0.25] */
} rrtmg_run_params;

int rrtmg_run_params_default(rrtmg_run_params* p);

/* run_rrtmg on device arrays, enqueued on `stream`.
 *   seconds, days: get_time(Time) of the model time; days_per_year: the days
 *     of length_of_year() of the calendar.
 *   inputs: lat, lon (si,sj); p_full, z_full, t, q (si,sj,sk); p_half, z_half
 *     (si,sj,sk+1); t_surf_rad, albedo (si,sj); o3 (si,sj,sk) or NULL
 *     (o3_val); rrtm_precip (si,sj), needed when do_precip_albedo and
 *     num_precip > 0.
 *   tdt (si,sj,sk) K/s: the radiative tendency is added.
 *   coszen (si,sj): written.
 *   flux_sw (net downward SW), flux_lw (downward LW) at the surface (si,sj):
 *     both or neither.
 *   optional outputs (NULL = not wanted): t_half (si,sj,sk+1), tdt_rad,
 *     tdt_sw, tdt_lw (si,sj,sk) K/s, olr, isr (si,sj) W/m2.
 * The call allocates device workspace on the first use of a slab size only
 * (rrtmg_gpu_reserve does not cover it): make one call of that size before
 * capturing the call in a CUDA graph.  Input validation is reported by
 * rrtmg_gpu_sync_status. */
int rrtmg_run_dev(rrtmg_gpu_handle h, void* stream, const rrtmg_run_params* prm, int si, int sj, int sk,
                  int seconds, int days, int days_per_year, const double* lat, const double* lon,
                  const double* p_full, const double* p_half, const double* z_full, const double* z_half,
                  const double* t, const double* q, const double* o3, const double* t_surf_rad,
                  const double* albedo, const double* rrtm_precip, double* tdt, double* coszen, double* flux_sw,
                  double* flux_lw, double* t_half, double* tdt_rad, double* tdt_sw, double* tdt_lw, double* olr,
                  double* isr);

/* The same with host arrays (the call MiMA's Fortran makes): inputs are
 * copied in, tdt is read and written back, outputs are copied out; the call
 * returns when the results are in the host arrays. */
int rrtmg_run_c(rrtmg_gpu_handle h, const rrtmg_run_params* prm, int si, int sj, int sk, int seconds, int days,
                int days_per_year, const double* lat, const double* lon, const double* p_full,
                const double* p_half, const double* z_full, const double* z_half, const double* t, const double* q,
                const double* o3, const double* t_surf_rad, const double* albedo, const double* rrtm_precip,
                double* tdt, double* coszen, double* flux_sw, double* flux_lw, double* t_half, double* tdt_rad,
                double* tdt_sw, double* tdt_lw, double* olr, double* isr);

#ifdef __cplusplus
}
#endif
#endif /* RRTMG_RUN_H */
