/*
 * rrtmg_gpu.h -- C-ABI of the GB300 (sm_103a) implementation of RRTMG clear-sky
 * longwave and shortwave column radiation, the radiation hot path of MiMA.
 *
 * Drop-in boundary.  MiMA's radiation driver calls
 *     rrtmg_lw(...)   src/atmos_param/rrtm_radiation/rrtmg_lw/gcm_model/src/rrtmg_lw_rad.nomcica.f90:80-89
 *     rrtmg_sw(...)   src/atmos_param/rrtm_radiation/rrtmg_sw/gcm_model/src/rrtmg_sw_rad.nomcica.f90:78-88
 *     rrtmg_lw_ini / rrtmg_sw_ini(cpdair)   rrtmg_lw_init.f90:28, rrtmg_sw_init.f90:28
 * from run_rrtmg (src/atmos_param/rrtm_radiation/rrtm_radiation.f90:686-748).
 * rrtmg_lw_c / rrtmg_sw_c below take the same arguments in the same order and
 * with the same meaning, plus the handle and the two array extents the Fortran
 * assumed-shape arrays carry implicitly.
 *
 * Conventions
 *   - Arrays are Fortran column-major with the column index fastest:
 *     (ncol,nlay), (ncol,nlay+1), (ncol), emis (ncol,16), tauaer (ncol,nlay,nbnd).
 *     RRTM layer 1 is the surface layer; pressures in hPa.
 *   - As in MiMA, the h2ovmr argument carries specific humidity (kg/kg) and
 *     o3vmr the O3 mass mixing ratio; both are converted as in inatm
 *     (rrtmg_lw_rad.nomcica.f90:775-778, rrtmg_sw_rad.nomcica.f90:1004-1007).
 *   - Outputs are fully overwritten.  Heating rates are K/day.  The SW rate of
 *     the top layer is 0 (MiMA's change, rrtmg_sw_rad.nomcica.f90:725-726);
 *     the LW rate of the top layer is computed (rrtmg_lw_rtrnmr.f90:774-775
 *     zeroes htr(nlayers), which lies above the last output layer).
 *   - Optional gas arrays (ch4, n2o, o2, cfc*) and tauaer may be NULL (= 0).
 *   - Clouds: rrtmg_lw_c / rrtmg_lw_dev compute icld = 1 (random overlap,
 *     rrtmg_lw_rtrn.f90) and icld = 2 / 3 (maximum/random overlap,
 *     rrtmg_lw_rtrnmr.f90, where the non-McICA driver sends both,
 *     rrtmg_lw_rad.nomcica.f90:527-541) with cldprop's options
 *     (rrtmg_lw_cldprop.f90:155-270): inflglw = 0 cloud optical depths
 *     given, taucld (16,ncol,nlay); 1 abscld1 x (cicewp + cliqwp); 2 the ice
 *     (iceflglw 0-3) and liquid (liqflglw 0-1) parameterisations with the
 *     effective sizes reice / reliq (ncol,nlay, microns).  cldfr (ncol,nlay)
 *     always; cicewp / cliqwp (ncol,nlay, g/m2) required for inflglw 1 / 2,
 *     else NULL or given (they decide, with the band sum of taucld, whether a
 *     layer's optics are formed).  rrtmg_sw_c / rrtmg_sw_dev compute icld = 1,
 *     2, 3 (identical without McICA) with cldprop_sw's options
 *     (rrtmg_sw_cldprop.f90:118-340): inflgsw = 0 cloud optics given, taucld,
 *     ssacld, asmcld, fsfcld (14,ncol,nlay); 2 the ice (iceflgsw 1-3) and
 *     liquid (liqflgsw 1) parameterisations with cicewp / cliqwp and reice /
 *     reliq.  As the reference's non-McICA SW (rrtmg_sw_rad.nomcica.f90:
 *     533-538), every layer of a sunlit column must be clear or overcast
 *     (cldfr <= 1e-6 or >= 1 - 1e-6): a partly cloudy one is reported as
 *     RRTMG_ERR_INPUT, where the reference stops the program; so is an
 *     effective size outside its parameterisation's table (or not a number)
 *     or a cloud optical property outside its physical range in a layer whose
 *     optics are formed (cldprop / cldprop_sw stop).  Every other entry point
 *     is clear sky (icld = 0).  The reference coerces icld and iaer silently
 *     (:437, :471-479); this library returns RRTMG_ERR_UNSUPPORTED for any
 *     configuration it does not compute (icld outside 0..3, inflglw outside
 *     0..2, inflgsw other than 0 / 2, SW cloud physics with iceflgsw outside
 *     1..3 or liqflgsw other than 1) and never falls back to a CPU path.
 *   - Every entry point returns a status (0 = success).  A handle is not
 *     thread-safe; use one handle per host thread.
 */
#ifndef RRTMG_GPU_H
#define RRTMG_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct rrtmg_gpu_state* rrtmg_gpu_handle;

enum rrtmg_gpu_status {
  RRTMG_OK = 0,
  RRTMG_ERR_ARG = 1,          /* bad dimension, null required pointer, bad handle */
  RRTMG_ERR_UNSUPPORTED = 2,  /* icld not in 0..3, a cloud option not computed (inflglw not in 0..2, inflgsw
                                 not 0 / 2, SW iceflgsw / liqflgsw), iaer not in {0,10}, idrv not in {0,1} */
  RRTMG_ERR_CUDA = 3,         /* CUDA runtime error (see rrtmg_gpu_last_error) */
  RRTMG_ERR_TABLES = 4,       /* table blob missing, malformed or checksum mismatch */
  RRTMG_ERR_INPUT = 5,        /* device-side validation flagged a non-finite or out-of-range input, a
                                 partly cloudy sunlit layer in a SW call with clouds, or a cloud size or
                                 optical property outside its parameterisation's range */
  RRTMG_ERR_NOMEM = 6         /* device workspace allocation failed */
};

enum rrtmg_gpu_precision {
  RRTMG_PREC_FP64 = 0,  /* FP64 everywhere; bit-level parity target vs the FP64 reference path */
  RRTMG_PREC_SPLIT = 1  /* FP32 setcoef, gas optics, transmittances and per-g recursions;
                           g-point sums to FP64 accuracy (compensated FP32), FP64 band sums
                           and heating-rate differencing */
};

/* Maximum number of layers (parrrtm.f90 / parrrsw.f90 mxlay). */
#define RRTMG_GPU_MAX_LAYERS 203

/* Transcendental evaluation of the solvers: the reference's lookup tables
 * (exp_tbl / tfn_tbl, 10001 entries, the default) or the analytic functions
 * they sample.  The analytic form is the smooth forward whose derivatives the
 * adjoint entry points compute. */
enum { RRTMG_TRANS_TABLE = 0, RRTMG_TRANS_ANALYTIC = 1 };

/* Replaces rrtmg_lw_ini(cpdair) + rrtmg_sw_ini(cpdair) (rrtmg_lw_init.f90:28-175,
 * rrtmg_sw_init.f90:28-154): reads the unreduced coefficient tables from
 * table_blob, performs the 256->140 / 224->112 g-point reduction, builds the
 * transmittance tables and uploads everything to `device`. */
int rrtmg_gpu_init(double cpdair, const char* table_blob, int device, rrtmg_gpu_handle* out);
/* No counterpart in the reference (whose tables live until the program ends):
 * waits for the handle's streams and frees its device state. */
int rrtmg_gpu_finalize(rrtmg_gpu_handle h);

/* No counterpart in the reference (FP64 throughout, -r8).  Selects
 * RRTMG_PREC_FP64 (default) or RRTMG_PREC_SPLIT for later calls. */
int rrtmg_gpu_set_precision(rrtmg_gpu_handle h, int precision);

/* No counterpart in the reference, which returns no status (errors stop the
 * program): the meaning of a status code. */
const char* rrtmg_gpu_error_string(int status);
/* Detail of the last failure on this handle ("" if none). */
const char* rrtmg_gpu_last_error(rrtmg_gpu_handle h);
/* No counterpart in the reference.  Number of kernel launches issued by this
 * handle since init. */
long long rrtmg_gpu_launch_count(rrtmg_gpu_handle h);

/* rrtmg_lw (rrtmg_lw_rad.nomcica.f90:80-89), host arrays.  tauaer (ncol,nlay,16)
 * is always added to the gas optical depth (the reference forces iaer = 10,
 * :442).  duflx_dt/duflxc_dt (ncol,nlay+1) are written when idrv = 1.  With
 * clouds (icld >= 1) the clear-sky outputs (uflxc, dflxc, hrc, duflxc_dt) are
 * the solver's clear-sky stream, else they equal the total ones. */
int rrtmg_lw_c(rrtmg_gpu_handle h, int ncol, int nlay, int icld, int idrv,
               const double* play, const double* plev, const double* tlay, const double* tlev,
               const double* tsfc, const double* h2ovmr, const double* o3vmr, const double* co2vmr,
               const double* ch4vmr, const double* n2ovmr, const double* o2vmr,
               const double* cfc11vmr, const double* cfc12vmr, const double* cfc22vmr,
               const double* ccl4vmr, const double* emis, int inflglw, int iceflglw, int liqflglw,
               const double* cldfr, const double* taucld, const double* cicewp, const double* cliqwp,
               const double* reice, const double* reliq, const double* tauaer,
               double* uflx, double* dflx, double* hr, double* uflxc, double* dflxc, double* hrc,
               double* duflx_dt, double* duflxc_dt);

/* rrtmg_sw (rrtmg_sw_rad.nomcica.f90:78-88), host arrays.  Columns with
 * coszen < 1e-10 get zero fluxes and heating (MiMA's skip, :502-510).
 * iaer = 10 uses tauaer/ssaaer/asmaer (ncol,nlay,14); ecaer is ignored.  With
 * clouds (icld >= 1) the clear-sky outputs (swuflxc, swdflxc, swhrc) are the
 * clear pass of spcvrt_sw, else they equal the total ones. */
int rrtmg_sw_c(rrtmg_gpu_handle h, int ncol, int nlay, int icld, int iaer,
               const double* play, const double* plev, const double* tlay, const double* tlev,
               const double* tsfc, const double* h2ovmr, const double* o3vmr, const double* co2vmr,
               const double* ch4vmr, const double* n2ovmr, const double* o2vmr,
               const double* asdir, const double* asdif, const double* aldir, const double* aldif,
               const double* coszen, double adjes, int dyofyr, double scon,
               int inflgsw, int iceflgsw, int liqflgsw, const double* cldfr, const double* taucld,
               const double* ssacld, const double* asmcld, const double* fsfcld,
               const double* cicewp, const double* cliqwp, const double* reice, const double* reliq,
               const double* tauaer, const double* ssaaer, const double* asmaer, const double* ecaer,
               double* swuflx, double* swdflx, double* swhr, double* swuflxc, double* swdflxc,
               double* swhrc);

/* Device-pointer variants: identical arguments, every array is a device
 * pointer, work is enqueued on `stream` (a cudaStream_t, NULL = default) and
 * the call returns without synchronising.  Input validation results are
 * collected on the device; rrtmg_gpu_sync_status() waits for the stream and
 * returns RRTMG_ERR_INPUT if any enqueued call saw invalid input.  After a
 * first call with the same (ncol, nlay) the calls allocate nothing and may be
 * captured in a CUDA graph. */
int rrtmg_lw_dev(rrtmg_gpu_handle h, void* stream, int ncol, int nlay, int icld, int idrv,
                 const double* play, const double* plev, const double* tlay, const double* tlev,
                 const double* tsfc, const double* h2ovmr, const double* o3vmr, const double* co2vmr,
                 const double* ch4vmr, const double* n2ovmr, const double* o2vmr,
                 const double* cfc11vmr, const double* cfc12vmr, const double* cfc22vmr,
                 const double* ccl4vmr, const double* emis, int inflglw, int iceflglw, int liqflglw,
                 const double* cldfr, const double* taucld, const double* cicewp, const double* cliqwp,
                 const double* reice, const double* reliq, const double* tauaer,
                 double* uflx, double* dflx, double* hr, double* uflxc, double* dflxc, double* hrc,
                 double* duflx_dt, double* duflxc_dt);

int rrtmg_sw_dev(rrtmg_gpu_handle h, void* stream, int ncol, int nlay, int icld, int iaer,
                 const double* play, const double* plev, const double* tlay, const double* tlev,
                 const double* tsfc, const double* h2ovmr, const double* o3vmr, const double* co2vmr,
                 const double* ch4vmr, const double* n2ovmr, const double* o2vmr,
                 const double* asdir, const double* asdif, const double* aldir, const double* aldif,
                 const double* coszen, double adjes, int dyofyr, double scon,
                 int inflgsw, int iceflgsw, int liqflgsw, const double* cldfr, const double* taucld,
                 const double* ssacld, const double* asmcld, const double* fsfcld,
                 const double* cicewp, const double* cliqwp, const double* reice, const double* reliq,
                 const double* tauaer, const double* ssaaer, const double* asmaer, const double* ecaer,
                 double* swuflx, double* swdflx, double* swhr, double* swuflxc, double* swdflxc,
                 double* swhrc);

/* Fused LW + SW step on device arrays (no single counterpart in the
 * reference, whose run_rrtmg calls rrtmg_sw and then rrtmg_lw,
 * rrtm_radiation.f90:686-748): the arguments of rrtmg_lw_dev and
 * rrtmg_sw_dev merged, clear sky (icld = 0, the cloud arguments omitted), LW
 * aerosols tauaer_lw (ncol,nlay,16) optional, SW aerosols when iaer = 10.  The
 * results equal those of the two separate calls bit for bit.  The SW call
 * runs on a second stream of the handle, forked from `stream` and joined back
 * into it by events, so that the two calls overlap on the GPU; everything is
 * complete when `stream` reaches the end of the call's work, and the call can
 * be captured in a CUDA graph (as two parallel branches).  Calls on one
 * handle share its workspaces: order them on one stream. */
int rrtmg_step_dev(rrtmg_gpu_handle h, void* stream, int ncol, int nlay, int idrv, int iaer,
                   const double* play, const double* plev, const double* tlay, const double* tlev,
                   const double* tsfc, const double* h2ovmr, const double* o3vmr, const double* co2vmr,
                   const double* ch4vmr, const double* n2ovmr, const double* o2vmr,
                   const double* cfc11vmr, const double* cfc12vmr, const double* cfc22vmr,
                   const double* ccl4vmr, const double* emis, const double* tauaer_lw,
                   const double* asdir, const double* asdif, const double* aldir, const double* aldif,
                   const double* coszen, double adjes, int dyofyr, double scon,
                   const double* tauaer_sw, const double* ssaaer, const double* asmaer,
                   double* uflx, double* dflx, double* hr, double* uflxc, double* dflxc, double* hrc,
                   double* duflx_dt, double* duflxc_dt,
                   double* swuflx, double* swdflx, double* swhr, double* swuflxc, double* swdflxc,
                   double* swhrc);

/* No counterpart in the reference.  Kernel timing: while enabled, the LW and
 * SW calls record CUDA events around each of their three kernels (prep,
 * g-point solver, finalize) on the call's stream (not while the stream is
 * being captured).  rrtmg_gpu_profile waits for the events and writes the
 * six durations of the last LW and SW call in ms: LW prep, LW g-point, LW
 * finalize, SW prep, SW g-point, SW finalize. */
int rrtmg_gpu_set_profiling(rrtmg_gpu_handle h, int on);
int rrtmg_gpu_profile(rrtmg_gpu_handle h, float* ms);

/* No counterpart in the reference (which always uses its tables).  Selects
 * RRTMG_TRANS_TABLE or RRTMG_TRANS_ANALYTIC for later calls on the handle. */
int rrtmg_gpu_set_transcendentals(rrtmg_gpu_handle h, int mode);

/* No counterpart in the reference.  Reserves device workspace for clear-sky
 * LW, SW and fused calls of up to ncol columns and nlay layers, so that later
 * such device calls allocate nothing (e.g. before graph capture).  A call with
 * clouds needs more (cloud fields, the clear-sky partials, overlap factors,
 * formed cloud optics): its first call of a size grows the workspace, and
 * later calls of that size and configuration allocate nothing. */
int rrtmg_gpu_reserve(rrtmg_gpu_handle h, int ncol, int nlay);

/* No counterpart in the reference (which does not validate its inputs).
 * Waits for `stream` and reports RRTMG_ERR_INPUT if an enqueued call flagged
 * invalid input (the flag is then cleared). */
int rrtmg_gpu_sync_status(rrtmg_gpu_handle h, void* stream);

/* Adjoint of the clear-sky LW + SW radiation: Jacobians of
 *   rows (ny = 2*nlay + 3): LW heating rate of layers 1..nlay (K/day), OLR
 *     (upward LW at the top level, W/m2), LW surface net flux (up - down),
 *     SW heating rate of layers 1..nlay, SW surface net flux (down - up);
 * with respect to
 *   inputs (nx = 3*nlay + 2): tlay of layers 1..nlay, h2ovmr (specific
 *     humidity) of layers 1..nlay, tlev of levels 0..nlay, tsfc.
 * The differentiated forward is RRTMG_TRANS_ANALYTIC (the reference's
 * transmittance tables are piecewise constant in optical depth), in FP64, or
 * with RRTMG_PREC_SPLIT in FP32 with FP64-accurate g-point sums and FP64 band
 * sums; no counterpart
 * in the reference, which has only the LW surface-temperature derivative
 * (idrv = 1, rrtmg_lw_rtrnmr.f90:628-745).  The reverse sweeps of rtrnmr and
 * spcvrt run per g-point with the layer optics recomputed from checkpointed
 * per-layer setcoef inputs.  Arguments are those of rrtmg_lw_dev and
 * rrtmg_sw_dev (device arrays, clear sky; tauaer_lw (ncol,nlay,16) optional,
 * SW aerosols when iaer = 10).
 *   jac  (ncol, ny, nx), column index fastest: jac[(x*ny + r)*ncol + c].
 * Workspace: about 16*(nlay+2)*(3*nlay+3)*8 bytes per column (661 KB at
 * 40 layers); split large column counts into several calls. */
int rrtmg_jacobian_dev(rrtmg_gpu_handle h, void* stream, int ncol, int nlay,
                       const double* play, const double* plev, const double* tlay, const double* tlev,
                       const double* tsfc, const double* h2ovmr, const double* o3vmr, const double* co2vmr,
                       const double* ch4vmr, const double* n2ovmr, const double* o2vmr,
                       const double* cfc11vmr, const double* cfc12vmr, const double* cfc22vmr,
                       const double* ccl4vmr, const double* emis, const double* tauaer_lw,
                       const double* asdir, const double* asdif, const double* aldir, const double* aldif,
                       const double* coszen, double adjes, int dyofyr, double scon, int iaer,
                       const double* tauaer_sw, const double* ssaaer, const double* asmaer, double* jac);

/* Vector-Jacobian product (one reverse sweep per g-point): given cotangents
 * cot (ncol, ny) of the rows above, writes grad (ncol, nx) = cot^T J per
 * column: grad[x*ncol + c].  Same arguments as rrtmg_jacobian_dev otherwise;
 * no counterpart in the reference. */
int rrtmg_vjp_dev(rrtmg_gpu_handle h, void* stream, int ncol, int nlay,
                  const double* play, const double* plev, const double* tlay, const double* tlev,
                  const double* tsfc, const double* h2ovmr, const double* o3vmr, const double* co2vmr,
                  const double* ch4vmr, const double* n2ovmr, const double* o2vmr,
                  const double* cfc11vmr, const double* cfc12vmr, const double* cfc22vmr,
                  const double* ccl4vmr, const double* emis, const double* tauaer_lw,
                  const double* asdir, const double* asdif, const double* aldir, const double* aldif,
                  const double* coszen, double adjes, int dyofyr, double scon, int iaer,
                  const double* tauaer_sw, const double* ssaaer, const double* asmaer,
                  const double* cot, double* grad);

/* Size of the library's static LW device scratch (64 MiB), held by every GPU
 * that loads the library until process exit.  At nlay = 40 a call needs about
 * 39.2 KB per column, so up to about 1700 columns fit; at nlay = 60, about 1150. */
#define RRTMG_GPU_STATIC_SCRATCH_BYTES (64u * 1024u * 1024u)

/* No counterpart in the reference.  Same arguments and results as
 * rrtmg_lw_dev, but the call allocates nothing: its scratch is the library's
 * static device array of RRTMG_GPU_STATIC_SCRATCH_BYTES, not the handle's
 * workspace (no cudaMalloc or cudaFree, no allocating library routine).
 * A call whose (ncol, nlay) needs more scratch than that returns
 * RRTMG_ERR_ARG with the byte counts in rrtmg_gpu_last_error().  The first call
 * on a device looks up the array's device address (cudaGetSymbolAddress) with
 * that device current; make that first call before any stream capture.  All
 * calls on a device share the one array and it keeps the last call's
 * contents, so calls that overlap on the GPU (different streams, or different
 * handles on one device) race: order them on one stream or with events.
 * The array's device address is kept for the life of the process, so do not
 * reset the device (cudaDeviceReset) while the library is loaded: a later
 * call would write through the old context's address. */
int rrtmg_lw_dev_static(rrtmg_gpu_handle h, void* stream, int ncol, int nlay, int icld, int idrv,
                        const double* play, const double* plev, const double* tlay, const double* tlev,
                        const double* tsfc, const double* h2ovmr, const double* o3vmr, const double* co2vmr,
                        const double* ch4vmr, const double* n2ovmr, const double* o2vmr,
                        const double* cfc11vmr, const double* cfc12vmr, const double* cfc22vmr,
                        const double* ccl4vmr, const double* emis, int inflglw, int iceflglw, int liqflglw,
                        const double* cldfr, const double* taucld, const double* cicewp, const double* cliqwp,
                        const double* reice, const double* reliq, const double* tauaer,
                        double* uflx, double* dflx, double* hr, double* uflxc, double* dflxc, double* hrc,
                        double* duflx_dt, double* duflxc_dt);

#ifdef __cplusplus
}
#endif
#endif /* RRTMG_GPU_H */
