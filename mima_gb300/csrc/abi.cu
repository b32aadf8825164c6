// C-ABI of the GB300 RRTMG path (declared in include/rrtmg_gpu.h).
//
// A handle owns: the device coefficient tables (FP64 and FP32 copies), two
// internal streams for the host-pointer entry points (column chunks alternate
// between them), a device flag word for input validation, and device
// workspaces grown on demand: LW scratch, SW scratch (kept separate so an LW
// and an SW call may run concurrently on different streams), the adjoint's,
// and per-stream staging and scratch for the host-pointer entry points.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>

#include <cmath>

#include "adjoint.h"
#include "common.cuh"
#include "driver.h"
#include "launch.h"
#include "rrtmg_gpu.h"
#include "rrtmg_run.h"
#include "tables_host.h"

using namespace rrtmg;

namespace {

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
};

}  // namespace

struct rrtmg_gpu_state {
  int device = 0;
  int precision = RRTMG_PREC_FP64;
  int analytic = 0;  // 1: exp/tfn evaluated instead of looked up
  cudaStream_t stream = nullptr;
  HostTables host;
  double *lw_tab64 = nullptr, *sw_tab64 = nullptr, *lw_exp64 = nullptr, *lw_tfn64 = nullptr, *sw_exp64 = nullptr;
  double* lw_tau64 = nullptr;
  float* lw_tau32 = nullptr;
  double *totplnk = nullptr, *totplnkderiv = nullptr;
  float *totplnk32 = nullptr, *totplnkderiv32 = nullptr;  // FP32 copies (split prep)
  float *lw_tab32 = nullptr, *sw_tab32 = nullptr, *lw_exp32 = nullptr, *lw_tfn32 = nullptr, *sw_exp32 = nullptr;
  // FP32 LW transmittance and tau transition function side by side (one
  // gather per table lookup in the split LW solver)
  float2* lw_exptfn32 = nullptr;
  double* cldtab = nullptr;  // cloud optical property tables (ct:: offsets)
  float* cldtab32 = nullptr;  // their FP32 copy (split LW cloud physics)
  unsigned* flags = nullptr;
  DevBuf lw_ws, sw_ws, adj_ws;
  // host-pointer calls: a second stream and per-stream staging and scratch, so
  // that column chunks alternate between the streams
  cudaStream_t stream2 = nullptr;
  DevBuf hio[2], hws[2];
  // run_rrtmg calls: RRTM columns, results, zonal scratch and the LW and SW
  // scratch (device entry point); host-array calls: per latitude-chunk stream
  // staging and workspace
  DevBuf run_ws, run_cio[2], run_cws[2];
  // fused LW+SW calls: the SW call runs on `side`, forked from and joined back
  // into the caller's stream with these events; host-array run_rrtmg chunks on
  // stream2 fork onto side2
  cudaStream_t side = nullptr, side2 = nullptr;
  cudaEvent_t fork_ev = nullptr, join_ev = nullptr, fork_ev2 = nullptr, join_ev2 = nullptr;
  long long launches = 0;
  std::string err;
  // Optional per-kernel timing: events around every launch of the last LW
  // and SW call (prep, g-point, finalize), outside stream capture only.
  bool profiling = false;
  cudaEvent_t ev[2][4] = {};
};

namespace {

int fail(rrtmg_gpu_state* h, int code, const std::string& msg) {
  if (h) h->err = msg;
  return code;
}

int cuda_fail(rrtmg_gpu_state* h, cudaError_t e, const char* where) {
  return fail(h, RRTMG_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

template <class T>
cudaError_t upload(T** dst, const std::vector<T>& src) {
  cudaError_t e = cudaMalloc((void**)dst, src.size() * sizeof(T) + 16);
  if (e != cudaSuccess) return e;
  return cudaMemcpy(*dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice);
}

std::vector<float> to_f32(const std::vector<double>& v) {
  std::vector<float> f(v.size());
  for (size_t i = 0; i < v.size(); ++i) f[i] = (float)v[i];
  return f;
}

std::vector<float2> interleave_f32(const std::vector<double>& a, const std::vector<double>& b) {
  std::vector<float2> f(a.size());
  for (size_t i = 0; i < a.size(); ++i) f[i] = make_float2((float)a[i], (float)b[i]);
  return f;
}

size_t align256(size_t n) { return (n + 255) & ~(size_t)255; }

// Failure injection for tests, on the host (no GPU fault): with
// RRTMG_GPU_FAIL_ALLOC=1 in the environment every workspace allocation fails
// as cudaMalloc reports an exhausted device.
bool alloc_failure_injected() {
  const char* v = std::getenv("RRTMG_GPU_FAIL_ALLOC");
  return v != nullptr && v[0] == '1';
}

// Grow a workspace; refuses while the stream is being captured.
int ensure(rrtmg_gpu_state* h, DevBuf& b, size_t need, cudaStream_t s) {
  if (b.bytes >= need) return RRTMG_OK;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (s != nullptr && cudaStreamIsCapturing(s, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone)
    return fail(h, RRTMG_ERR_NOMEM,
                "workspace too small during stream capture: make one call of this size before capturing "
                "(rrtmg_gpu_reserve covers the LW and SW calls)");
  if (b.p) cudaFree(b.p);
  b.p = nullptr;
  b.bytes = 0;
  cudaError_t e = alloc_failure_injected() ? cudaErrorMemoryAllocation : cudaMalloc(&b.p, need);
  if (e != cudaSuccess) {
    b.p = nullptr;
    return fail(h, RRTMG_ERR_NOMEM, std::string("device workspace allocation failed: ") + cudaGetErrorString(e));
  }
  b.bytes = need;
  return RRTMG_OK;
}

struct Carver {
  char* base;
  size_t off = 0;
  template <class T>
  T* take(size_t n) {
    T* p = (T*)(base ? base + off : nullptr);
    off += align256(n * sizeof(T));
    return p;
  }
};

// cloudy: also the per-layer cloud fields and the clear-sky band partials
// (icld >= 1), with maximum/random overlap (icld = 2, 3) the overlap factors,
// and with cloud physics (inflag 1 / 2) the formed cloud depths; clear-sky
// calls carve none of them.
LwWork carve_lw(void* base, int ncol, int nlay, size_t* bytes, bool cloudy = false, bool maxrand = false,
                bool phys = false) {
  Carver c{(char*)base};
  const size_t N = (size_t)ncol, L = (size_t)nlay;
  LwWork w{};
  w.idx = c.take<uint32_t>(L * N);
  w.f = c.take<double>((size_t)LF_N * L * N);
  w.planklay = c.take<double>(16 * L * N);
  w.planklev = c.take<double>(16 * (L + 1) * N);
  w.plankbnd = c.take<double>(16 * N);
  w.dplankbnd = c.take<double>(16 * N);
  w.secdiff = c.take<double>(16 * N);
  w.laytrop = c.take<int>(N);
  w.bu = c.take<double>(kLwSlots * (L + 1) * N);
  w.bd = c.take<double>(kLwSlots * (L + 1) * N);
  w.bdu = c.take<double>(kLwSlots * (L + 1) * N);
  w.colsum = c.take<double>(2 * L * N);
  if (cloudy) {
    w.cld = c.take<double>(2 * L * N);
    w.buc = c.take<double>(kLwSlots * (L + 1) * N);
    w.bdc = c.take<double>(kLwSlots * (L + 1) * N);
    w.bduc = c.take<double>(kLwSlots * (L + 1) * N);
    if (maxrand) w.ovl = c.take<double>(12 * L * N);
    if (phys) w.odc = c.take<double>(16 * L * N);
  }
  if (bytes) *bytes = c.off;
  return w;
}

// cloudy: the per-layer cloud fields and the clear-pass band partials, and on
// the split path (split) the total-sky pass's cloud optics; with cloud
// physics on the FP64 path (phys) the formed optics.
SwWork carve_sw(void* base, int ncol, int nlay, size_t* bytes, bool cloudy = false, bool phys = false,
                bool split = false) {
  Carver c{(char*)base};
  const size_t N = (size_t)ncol, L = (size_t)nlay;
  SwWork w{};
  w.idx = c.take<uint32_t>(L * N);
  w.f = c.take<double>((size_t)SF_N * L * N);
  w.laytrop = c.take<int>(N);
  w.laysolfr = c.take<int>(14 * N);
  w.su = c.take<double>(kSwSlots * (L + 1) * N);
  w.sd = c.take<double>(kSwSlots * (L + 1) * N);
  if (cloudy) {
    w.cld = c.take<double>(2 * L * N);
    w.suc = c.take<double>(kSwSlots * (L + 1) * N);
    w.sdc = c.take<double>(kSwSlots * (L + 1) * N);
    if (phys && !split) w.cldopt = c.take<double>(3 * 14 * L * N);
    if (split) w.cldq = c.take<float4>(14 * L * N);
  }
  if (bytes) *bytes = c.off;
  return w;
}

bool valid_handle(rrtmg_gpu_state* h) { return h != nullptr && h->lw_tab64 != nullptr; }

int check_dims(rrtmg_gpu_state* h, int ncol, int nlay) {
  if (ncol < 1) return fail(h, RRTMG_ERR_ARG, "ncol must be >= 1");
  if (nlay < 2 || nlay > RRTMG_GPU_MAX_LAYERS) return fail(h, RRTMG_ERR_ARG, "nlay must be in [2, 203]");
  if ((long long)ncol * (long long)(nlay + 1) * 16 > (1LL << 31) - 1)
    return fail(h, RRTMG_ERR_ARG, "ncol * (nlay+1) too large for one call; split the columns");
  return RRTMG_OK;
}

// The split path stores the per-layer fields as float in the same carving.
template <class F>
LwWorkT<F> work_as(const LwWork& w) {
  return LwWorkT<F>{w.idx, (F*)w.f, (F*)w.planklay, (F*)w.planklev, (F*)w.plankbnd, (F*)w.dplankbnd, (F*)w.secdiff,
                    w.laytrop, w.bu, w.bd, w.bdu, w.colsum, (F*)w.cld, w.buc, w.bdc, w.bduc, (F*)w.ovl, w.odc};
}
template <class F>
SwWorkT<F> work_as(const SwWork& w) {
  return SwWorkT<F>{w.idx, (F*)w.f, w.laytrop, w.laysolfr, w.su, w.sd, (F*)w.cld, w.suc, w.sdc, w.cldopt, w.cldq};
}
template <class F>
LwPrepT<F> prep_of(const LwWorkT<F>& w) {
  return LwPrepT<F>{w.idx, w.f, w.planklay, w.planklev, w.plankbnd, w.dplankbnd, w.secdiff, w.laytrop};
}
template <class F>
SwPrepT<F> prep_of(const SwWorkT<F>& w) {
  return SwPrepT<F>{w.idx, w.f, w.laytrop, w.laysolfr};
}

// ---------------------------------------------------------------------------
// Enqueue one LW radiation call on stream s (all pointers on the device) with
// its scratch carved from `base` (carve_lw bytes).
// ---------------------------------------------------------------------------
// Records profiling event k of family fam (0 LW, 1 SW) on s when enabled.
void mark(rrtmg_gpu_state* h, int fam, int k, cudaStream_t s) {
  if (!h->profiling) return;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone) return;
  cudaEventRecord(h->ev[fam][k], s);
}

int lw_enqueue(rrtmg_gpu_state* h, cudaStream_t s, void* base, int ncol, int nlay, int idrv, const LwIn& in,
               double* uflx, double* dflx, double* hr, double* uflxc, double* dflxc, double* hrc, double* duflx_dt,
               double* duflxc_dt) {
  // clouds (icld >= 1): the call carries cloud arrays; icld = 2, 3:
  // maximum/random overlap with its overlap factors
  const bool cloudy = in.cldfr != nullptr, maxrand = cloudy && in.icld >= 2;
  // cloud physics (inflag 1 / 2): the depths are formed on the device, after
  // prep (they carry secdiff), and handed to the solver in place of taucld
  const bool phys = cloudy && in.inflag != 0;
  LwWork w = carve_lw(base, ncol, nlay, nullptr, cloudy, maxrand, phys);
  const double* taucld = phys ? w.odc : in.taucld;
  mark(h, 0, 0, s);
  const int nb = h->precision == RRTMG_PREC_SPLIT ? lw_slot_blocks(ncol) : lw_gpoint_blocks(h->host.lw, ncol);
  if (h->precision == RRTMG_PREC_SPLIT) {
    const LwWorkT<float> w32 = work_as<float>(w);
    launch_lw_prep_split(in, w32, h->totplnk32, h->totplnkderiv32, ncol, nlay, idrv, h->flags, s);
    if (phys)
      launch_lw_cldphys_split(in, w32.secdiff, h->cldtab32, w32.cld, w.odc, ncol, nlay, h->flags, s);
    else if (cloudy)
      launch_lw_cloud_split(in, w32.cld, ncol, nlay, s);
    if (maxrand) launch_lw_overlap_split(in.cldfr, w32.ovl, ncol, nlay, s);
    mark(h, 0, 1, s);
    if (cloudy)
      launch_lw_gpoint_cld_split(prep_of(w32), w32.cld, taucld, in.emis, in.tauaer, h->lw_tab32, h->lw_exp32,
                                 h->lw_tfn32, h->lw_tau32, w.bu, w.bd, w.bdu, w.buc, w.bdc, w.bduc, ncol, nlay, idrv,
                                 nb, h->analytic, s, w32.ovl, phys);
    else
      launch_lw_gpoint_split(prep_of(w32), in.emis, in.tauaer, h->lw_tab32, h->lw_exptfn32, w.bu, w.bd,
                             w.bdu, ncol, nlay, idrv, nb, h->analytic, s);
  } else {
    launch_lw_prep(in, w, h->totplnk, h->totplnkderiv, ncol, nlay, idrv, h->flags, s);
    if (phys)
      launch_lw_cldphys(in, w.secdiff, h->cldtab, w.cld, w.odc, ncol, nlay, h->flags, s);
    else if (cloudy)
      launch_lw_cloud(in, w.cld, ncol, nlay, s);
    if (maxrand) launch_lw_overlap(in.cldfr, w.ovl, ncol, nlay, s);
    mark(h, 0, 1, s);
    if (cloudy)
      launch_lw_gpoint_cld_fp64(prep_of(w), w.cld, taucld, in.emis, in.tauaer, h->lw_tab64, h->lw_exp64,
                                h->lw_tfn64, h->lw_tau64, w.bu, w.bd, w.bdu, w.buc, w.bdc, w.bduc, ncol, nlay, idrv,
                                nb, h->analytic, s, w.ovl, phys);
    else
      launch_lw_gpoint_fp64(prep_of(w), in.emis, in.tauaer, h->lw_tab64, h->lw_exp64, h->lw_tfn64, w.bu, w.bd, w.bdu,
                            ncol, nlay, idrv, nb, h->analytic, s);
  }
  mark(h, 0, 2, s);
  if (h->precision == RRTMG_PREC_SPLIT)
    launch_lw_finalize_split(w.bu, w.bd, w.bdu, in.plev, ncol, nlay, idrv, uflx, dflx, hr, uflxc, dflxc, hrc,
                             duflx_dt, duflxc_dt, s, w.buc, w.bdc, w.bduc);
  else
    launch_lw_finalize(w.bu, w.bd, w.bdu, in.plev, ncol, nlay, idrv, uflx, dflx, hr, uflxc, dflxc, hrc, duflx_dt,
                       duflxc_dt, s, w.buc, w.bdc, w.bduc);
  mark(h, 0, 3, s);
  h->launches += 4 + (cloudy ? 1 : 0) + (maxrand ? 1 : 0);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(h, e, "LW kernel launch");
  return RRTMG_OK;
}

int lw_run(rrtmg_gpu_state* h, cudaStream_t s, int ncol, int nlay, int idrv, const LwIn& in, double* uflx,
           double* dflx, double* hr, double* uflxc, double* dflxc, double* hrc, double* duflx_dt, double* duflxc_dt) {
  size_t need;
  carve_lw(nullptr, ncol, nlay, &need, in.cldfr != nullptr, in.cldfr != nullptr && in.icld >= 2,
           in.cldfr != nullptr && in.inflag != 0);
  int rc = ensure(h, h->lw_ws, need, s);
  if (rc) return rc;
  return lw_enqueue(h, s, h->lw_ws.p, ncol, nlay, idrv, in, uflx, dflx, hr, uflxc, dflxc, hrc, duflx_dt, duflxc_dt);
}

// Cloud arguments of the LW calls: icld = 0 (clear sky), or clouds with
// icld = 1 random overlap (rrtmg_lw_rtrn.f90), icld = 2 / 3 maximum/random
// overlap (rrtmg_lw_rtrnmr.f90; the non-McICA driver routes both there,
// rrtmg_lw_rad.nomcica.f90:527-541).  cldprop's options
// (rrtmg_lw_cldprop.f90:155-270): inflglw = 0 optical depths given (taucld);
// 1 abscld1 x water path (cicewp, cliqwp); 2 ice (iceflglw 0-3) and liquid
// (liqflglw 0-1) parameterisations with the water paths and effective sizes
// (reice, reliq).
int lw_cloud_args(rrtmg_gpu_state* h, int icld, int inflglw, int iceflglw, int liqflglw, const double* cldfr,
                  const double* taucld, const double* cicewp, const double* cliqwp, const double* reice,
                  const double* reliq) {
  if (icld == 0) return RRTMG_OK;
  if (icld < 0 || icld > 3) return fail(h, RRTMG_ERR_UNSUPPORTED, "icld must be in [0, 3]");
  if (inflglw < 0 || inflglw > 2) return fail(h, RRTMG_ERR_UNSUPPORTED, "inflglw must be in [0, 2]");
  if (inflglw == 2 && (iceflglw < 0 || iceflglw > 3 || liqflglw < 0 || liqflglw > 1))
    return fail(h, RRTMG_ERR_UNSUPPORTED, "LW cloud physics: iceflglw must be in [0, 3] and liqflglw in [0, 1]");
  if (!cldfr) return fail(h, RRTMG_ERR_ARG, "LW clouds need cldfr");
  if (inflglw == 0 && !taucld) return fail(h, RRTMG_ERR_ARG, "LW clouds with inflglw = 0 need taucld");
  if (inflglw >= 1 && (!cicewp || !cliqwp))
    return fail(h, RRTMG_ERR_ARG, "LW cloud physics needs cicewp and cliqwp");
  if (inflglw == 2 && (!reice || !reliq)) return fail(h, RRTMG_ERR_ARG, "LW cloud physics needs reice and reliq");
  return RRTMG_OK;
}

// Cloud arguments of the SW calls: icld = 0 (clear sky), or icld = 1 with the
// cloud optics given (inflgsw = 0, rrtmg_sw_cldprop.f90:142-156).  Without
// McICA the reference computes clear and overcast layers only (a partly
// cloudy layer stops it, rrtmg_sw_rad.nomcica.f90:533-538): icld = 1, 2 and 3
// are the same there, so all three are taken; such a layer is reported by the
// kernels as invalid input.  cldprop_sw's options (rrtmg_sw_cldprop.f90:40,
// 118-340): inflgsw = 0 optics given; 2 ice (iceflgsw 1-3) and liquid
// (liqflgsw 1) parameterisations with the water paths and effective sizes.
// The reference's cldprop_sw has no branch for the others (inflgsw = 1 leaves
// its layers without cloud optics); they are refused.
int sw_cloud_args(rrtmg_gpu_state* h, int icld, int inflgsw, int iceflgsw, int liqflgsw, const double* cldfr,
                  const double* taucld, const double* ssacld, const double* asmcld, const double* fsfcld,
                  const double* cicewp, const double* cliqwp, const double* reice, const double* reliq) {
  if (icld == 0) return RRTMG_OK;
  if (icld < 0 || icld > 3) return fail(h, RRTMG_ERR_UNSUPPORTED, "icld must be in [0, 3]");
  if (inflgsw != 0 && inflgsw != 2) return fail(h, RRTMG_ERR_UNSUPPORTED, "inflgsw must be 0 or 2");
  if (inflgsw == 2 && (iceflgsw < 1 || iceflgsw > 3 || liqflgsw != 1))
    return fail(h, RRTMG_ERR_UNSUPPORTED, "SW cloud physics: iceflgsw must be in [1, 3] and liqflgsw 1");
  if (!cldfr) return fail(h, RRTMG_ERR_ARG, "SW clouds need cldfr");
  if (inflgsw == 0 && (!taucld || !ssacld || !asmcld || !fsfcld))
    return fail(h, RRTMG_ERR_ARG, "SW clouds with inflgsw = 0 need taucld, ssacld, asmcld and fsfcld");
  if (inflgsw == 2 && (!cicewp || !cliqwp || !reice || !reliq))
    return fail(h, RRTMG_ERR_ARG, "SW cloud physics needs cicewp, cliqwp, reice and reliq");
  return RRTMG_OK;
}

// Incident-flux scaling (inatm_sw, rrtmg_sw_rad.nomcica.f90:953-972): the
// GCM's Earth-Sun factor, or Iqbal's day-of-year formula, times scon/1368.22.
double adjflux_of(const rrtmg_gpu_state* h, double adjes, int dyofyr, double scon) {
  double adjflx = adjes;
  if (dyofyr > 0) {
    const double gamma = 2. * h->host.sw.pi * (dyofyr - 1) / 365.;
    adjflx = 1.000110 + .034221 * std::cos(gamma) + .001289 * std::sin(gamma) + .000719 * std::cos(2. * gamma) +
             .000077 * std::sin(2. * gamma);
  }
  return adjflx * (scon / 1.36822e+03);
}

int sw_enqueue(rrtmg_gpu_state* h, cudaStream_t s, void* base, int ncol, int nlay, int iaer, double adjes,
               int dyofyr, double scon, const SwIn& in, double* swuflx, double* swdflx, double* swhr, double* swuflxc,
               double* swdflxc, double* swhrc) {
  // clouds (icld = 1): a clear-sky pass into the clear partials (suc, sdc) and
  // a total-sky pass into su, sd, as the reference's two two-stream passes
  const bool cloudy = in.cldfr != nullptr;
  // cloud physics (inflag = 2): the cloud kernel forms the optics, which the
  // total-sky pass reads in place of the given ones (no forward fraction: they
  // are delta-scaled already)
  const bool phys = cloudy && in.inflag == 2;
  const bool split = h->precision == RRTMG_PREC_SPLIT;
  SwWork w = carve_sw(base, ncol, nlay, nullptr, cloudy, phys, split);
  SwIn tin = in;
  if (split) {
    tin.cldq = w.cldq;
  } else if (phys) {
    const size_t S = (size_t)14 * nlay * ncol;
    tin.taucld = w.cldopt;
    tin.ssacld = w.cldopt + S;
    tin.asmcld = w.cldopt + 2 * S;
    tin.fsfcld = nullptr;
  }
  const double adjflux = adjflux_of(h, adjes, dyofyr, scon);
  const int nb = h->precision == RRTMG_PREC_SPLIT ? sw_slot_blocks(ncol) : sw_gpoint_blocks(h->host.sw, ncol);
  double* cu = cloudy ? w.suc : w.su;
  double* cd = cloudy ? w.sdc : w.sd;
  mark(h, 1, 0, s);
  if (h->precision == RRTMG_PREC_SPLIT) {
    const SwWorkT<float> w32 = work_as<float>(w);
    launch_sw_prep_split(in, w32, ncol, nlay, h->flags, s);
    if (cloudy) launch_sw_cloud_split(in, w32.cld, ncol, nlay, h->flags, s, h->cldtab, w.cldq);
    mark(h, 1, 1, s);
    launch_sw_gpoint_split(prep_of(w32), in, adjflux, iaer, h->sw_tab32, h->sw_tab64, h->sw_exp32, cu, cd, ncol,
                           nlay, nb, h->analytic, s);
    if (cloudy)
      launch_sw_gpoint_split(prep_of(w32), tin, adjflux, iaer, h->sw_tab32, h->sw_tab64, h->sw_exp32, w.su, w.sd,
                             ncol, nlay, nb, h->analytic, s, w32.cld);
  } else {
    launch_sw_prep(in, w, ncol, nlay, h->flags, s);
    if (cloudy) launch_sw_cloud(in, w.cld, ncol, nlay, h->flags, s, h->cldtab, w.cldopt);
    mark(h, 1, 1, s);
    launch_sw_gpoint_fp64(prep_of(w), in, adjflux, iaer, h->sw_tab64, h->sw_exp64, cu, cd, ncol, nlay, nb,
                          h->analytic, s);
    if (cloudy)
      launch_sw_gpoint_fp64(prep_of(w), tin, adjflux, iaer, h->sw_tab64, h->sw_exp64, w.su, w.sd, ncol, nlay, nb,
                            h->analytic, s, w.cld);
  }
  mark(h, 1, 2, s);
  if (h->precision == RRTMG_PREC_SPLIT)
    launch_sw_finalize_split(w.su, w.sd, in.plev, in.coszen, ncol, nlay, swuflx, swdflx, swhr, swuflxc, swdflxc,
                             swhrc, s, w.suc, w.sdc);
  else
    launch_sw_finalize(w.su, w.sd, in.plev, in.coszen, ncol, nlay, swuflx, swdflx, swhr, swuflxc, swdflxc, swhrc, s,
                       w.suc, w.sdc);
  mark(h, 1, 3, s);
  h->launches += cloudy ? 6 : 4;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(h, e, "SW kernel launch");
  return RRTMG_OK;
}

int sw_run(rrtmg_gpu_state* h, cudaStream_t s, int ncol, int nlay, int iaer, double adjes, int dyofyr, double scon,
           const SwIn& in, double* swuflx, double* swdflx, double* swhr, double* swuflxc, double* swdflxc,
           double* swhrc) {
  size_t need;
  carve_sw(nullptr, ncol, nlay, &need, in.cldfr != nullptr, in.cldfr != nullptr && in.inflag == 2,
           h->precision == RRTMG_PREC_SPLIT);
  int rc = ensure(h, h->sw_ws, need, s);
  if (rc) return rc;
  return sw_enqueue(h, s, h->sw_ws.p, ncol, nlay, iaer, adjes, dyofyr, scon, in, swuflx, swdflx, swhr, swuflxc,
                    swdflxc, swhrc);
}

// Runs sw(side) on the handle's side stream and lw(st) on st, the side stream
// forked from st and joined back into it by events (a pattern that stream
// capture records as two parallel graph branches).  The join is enqueued even
// when a launch failed, so that a capture stays well formed.
struct Fork {
  cudaStream_t side;
  cudaEvent_t fork, join;
};
Fork default_fork(rrtmg_gpu_state* h) { return Fork{h->side, h->fork_ev, h->join_ev}; }

template <class LwF, class SwF>
int fork_lw_sw(rrtmg_gpu_state* h, cudaStream_t st, const Fork& fk, LwF&& lw, SwF&& sw) {
  cudaError_t e = cudaEventRecord(fk.fork, st);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(fk.side, fk.fork, 0);
  if (e != cudaSuccess) return cuda_fail(h, e, "fork onto the side stream");
  const int rs = sw(fk.side);
  const int rl = lw(st);
  e = cudaEventRecord(fk.join, fk.side);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(st, fk.join, 0);
  if (rs) return rs;
  if (rl) return rl;
  if (e != cudaSuccess) return cuda_fail(h, e, "join the side stream");
  return RRTMG_OK;
}

// ---------------------------------------------------------------------------
// Host-pointer calls.  Every caller array is (ncol, rows) with the column
// index fastest.  The columns are processed in chunks that alternate between
// the handle's two streams: per chunk, pitched copies of the chunk's columns of
// every input into contiguous (nc, rows) staging arrays, the kernels, and
// pitched copies of the outputs back into the caller's arrays, so that the
// copies of one chunk overlap the kernels of the other.
// ---------------------------------------------------------------------------
struct HostIn {
  const double* p;  // may be null (optional array)
  size_t rows;
  size_t per = 1;   // values per column in a row (taucld: 16, band fastest)
};
struct HostOut {
  double* p;  // may be null (not requested)
  size_t rows;
};
#ifndef RRTMG_HOST_CHUNK
#define RRTMG_HOST_CHUNK 16384
#endif
// Minimum columns per chunk and the largest chunk count of a host-array call.
// LW + SW host calls at 32768 columns (page-locked arrays) took 9.43 ms in one
// chunk, 8.78 in 2 or 3, 9.17 in 4, 9.89 in 8.
constexpr int kChunkMin = RRTMG_HOST_CHUNK, kMaxChunks = 16;
// Most input and output arrays of one host-array call (rrtmg_sw_c: 26 / 6).
constexpr int kMaxHostIn = 28, kMaxHostOut = 12;

int read_flags(rrtmg_gpu_state* h, cudaStream_t s);

// True when p is page-locked host memory (allocated or registered with CUDA).
bool pinned(const void* p) {
  if (!p) return true;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}

template <class Need, class Enqueue>
int host_call(rrtmg_gpu_state* h, int ncol, const HostIn* in, int nin, const HostOut* out, int nout, Need&& ws_need,
              Enqueue&& enqueue, const char* what) {
  if (nin > kMaxHostIn || nout > kMaxHostOut) return fail(h, RRTMG_ERR_ARG, "too many arrays for one host call");
  // On a failure after copies were enqueued, wait for them: they read and
  // write the caller's arrays, which the caller may free once the call returns.
  auto drain = [h]() {
    cudaStreamSynchronize(h->stream);
    cudaStreamSynchronize(h->stream2);
  };
  // Chunks only for page-locked arrays: pitched copies of pageable memory are
  // staged by the driver row by row; pageable arrays move in one piece.
  bool all_pinned = true;
  for (int k = 0; k < nin && all_pinned; ++k) all_pinned = pinned(in[k].p);
  for (int k = 0; k < nout && all_pinned; ++k) all_pinned = pinned(out[k].p);
  const int nchunk = (all_pinned && ncol >= 2 * kChunkMin) ? std::min(kMaxChunks, ncol / kChunkMin) : 1;
  int csize = (ncol + nchunk - 1) / nchunk;
  csize = std::min(ncol, (csize + 31) / 32 * 32);
  // staging and scratch per stream, sized for the largest chunk
  size_t stage = 0;
  for (int k = 0; k < nin; ++k)
    if (in[k].p) stage += align256((size_t)csize * in[k].per * in[k].rows * sizeof(double));
  for (int k = 0; k < nout; ++k)
    if (out[k].p) stage += align256((size_t)csize * out[k].rows * sizeof(double));
  cudaStream_t st[2] = {h->stream, h->stream2};
  for (int i = 0; i < 2 && i < nchunk; ++i) {
    int rc = ensure(h, h->hio[i], stage, nullptr);
    if (!rc) rc = ensure(h, h->hws[i], ws_need(csize), nullptr);
    if (rc) return rc;
  }
  const size_t pitch = (size_t)ncol * sizeof(double);
  cudaError_t e = cudaSuccess;
  const double* din[kMaxHostIn];
  double* dout[kMaxHostOut];
  for (int c = 0; c < nchunk && e == cudaSuccess; ++c) {
    const int c0 = c * csize;
    const int nc = std::min(csize, ncol - c0);
    if (nc <= 0) break;
    cudaStream_t s = st[c % 2];
    Carver cv{(char*)h->hio[c % 2].p};
    const size_t w = (size_t)nc * sizeof(double);
    for (int k = 0; k < nin; ++k) {
      din[k] = nullptr;
      if (!in[k].p) continue;
      const size_t pk = in[k].per;
      double* d = cv.take<double>((size_t)nc * pk * in[k].rows);
      if (e == cudaSuccess)
        e = nchunk == 1 ? cudaMemcpyAsync(d, in[k].p, w * pk * in[k].rows, cudaMemcpyHostToDevice, s)
                        : cudaMemcpy2DAsync(d, w * pk, in[k].p + c0 * pk, pitch * pk, w * pk, in[k].rows,
                                            cudaMemcpyHostToDevice, s);
      din[k] = d;
    }
    for (int k = 0; k < nout; ++k) dout[k] = out[k].p ? cv.take<double>((size_t)nc * out[k].rows) : nullptr;
    if (e != cudaSuccess) break;
    int rc = enqueue(s, h->hws[c % 2].p, nc, din, dout);
    if (rc) {
      drain();
      return rc;
    }
    for (int k = 0; k < nout && e == cudaSuccess; ++k)
      if (out[k].p)
        e = nchunk == 1 ? cudaMemcpyAsync(out[k].p, dout[k], w * out[k].rows, cudaMemcpyDeviceToHost, s)
                        : cudaMemcpy2DAsync(out[k].p + c0, pitch, dout[k], w, w, out[k].rows, cudaMemcpyDeviceToHost, s);
  }
  if (e != cudaSuccess) {
    drain();
    return cuda_fail(h, e, what);
  }
  e = cudaStreamSynchronize(h->stream2);
  if (e != cudaSuccess) return cuda_fail(h, e, "synchronise");
  return read_flags(h, h->stream);
}

// Adjoint workspace: dual prep fields and band partial gradients.
void carve_adj(void* base, int ncol, int nlay, int nseed_lw, int nseed_sw, AdjLwWork* lw, AdjSwWork* sw,
               size_t* bytes) {
  Carver c{(char*)base};
  const size_t N = (size_t)ncol, L = (size_t)nlay;
  AdjLwWork a;
  a.idx = c.take<uint32_t>(L * N);
  a.laytrop = c.take<int>(N);
  a.fv = c.take<double>((size_t)LF_N * L * N);
  a.ft = c.take<double>((size_t)LF_N * L * N);
  a.fq = c.take<double>((size_t)LF_N * L * N);
  a.play_v = c.take<double>(16 * L * N);
  a.play_t = c.take<double>(16 * L * N);
  a.plev_v = c.take<double>(16 * (L + 1) * N);
  a.plev_t = c.take<double>(16 * (L + 1) * N);
  a.pbnd_v = c.take<double>(16 * N);
  a.pbnd_t = c.take<double>(16 * N);
  a.secdiff = c.take<double>(16 * N);
  a.dsec = c.take<double>(16 * L * N);
  a.hs = c.take<double>(L * N);
  a.part = c.take<double>((size_t)kLwBands * nseed_lw * adj_lw_entries(nlay) * N);
  AdjSwWork b;
  b.idx = c.take<uint32_t>(L * N);
  b.laytrop = c.take<int>(N);
  b.laysolfr = c.take<int>(14 * N);
  b.fv = c.take<double>((size_t)SF_N * L * N);
  b.ft = c.take<double>((size_t)SF_N * L * N);
  b.fq = c.take<double>((size_t)SF_N * L * N);
  b.hs = c.take<double>(L * N);
  b.part = c.take<double>((size_t)kSwBands * nseed_sw * adj_sw_entries(nlay) * N);
  if (lw) *lw = a;
  if (sw) *sw = b;
  if (bytes) *bytes = c.off;
}

// Jacobians (cot == nullptr) or vector-Jacobian products of the analytic
// FP64 forward, enqueued on s.
int adj_run(rrtmg_gpu_state* h, cudaStream_t s, int ncol, int nlay, const LwIn& lin, const SwIn& sin, int iaer,
            double adjflux, const double* cot, double* out) {
  const int nseed_lw = cot ? 1 : nlay + 2, nseed_sw = cot ? 1 : nlay + 1;
  size_t need;
  carve_adj(nullptr, ncol, nlay, nseed_lw, nseed_sw, nullptr, nullptr, &need);
  int rc = ensure(h, h->adj_ws, need, s);
  if (rc) return rc;
  AdjLwWork lw;
  AdjSwWork sw;
  carve_adj(h->adj_ws.p, ncol, nlay, nseed_lw, nseed_sw, &lw, &sw, nullptr);
  const bool split = h->precision == RRTMG_PREC_SPLIT;
  const int nbl = lw_gpoint_blocks(h->host.lw, ncol, split), nbs = sw_gpoint_blocks(h->host.sw, ncol, split);
  if (h->precision == RRTMG_PREC_SPLIT) {
    // FP32 checkpoints in the same carving (they take half the room)
    const AdjLwWorkT<float> l32{lw.idx, lw.laytrop, (float*)lw.fv, (float*)lw.ft, (float*)lw.fq, (float*)lw.play_v,
                                (float*)lw.play_t, (float*)lw.plev_v, (float*)lw.plev_t, (float*)lw.pbnd_v,
                                (float*)lw.pbnd_t, (float*)lw.secdiff, lw.dsec, lw.hs, lw.part};
    const AdjSwWorkT<float> s32{sw.idx, sw.laytrop, sw.laysolfr, (float*)sw.fv, (float*)sw.ft, (float*)sw.fq, sw.hs,
                                sw.part};
    launch_adj_lw_split(lin, l32, h->totplnk32, h->lw_tab32, cot, nseed_lw, ncol, nlay, nbl, s);
    launch_adj_sw_split(sin, s32, adjflux, iaer, h->sw_tab32, h->sw_tab64, cot, nseed_sw, ncol, nlay, nbs, s);
  } else {
    launch_adj_lw(lin, lw, h->totplnk, h->lw_tab64, cot, nseed_lw, ncol, nlay, nbl, s);
    launch_adj_sw(sin, sw, adjflux, iaer, h->sw_tab64, cot, nseed_sw, ncol, nlay, nbs, s);
  }
  launch_adj_finalize(lw, sw, lin.plev, sin.coszen, nseed_lw, nseed_sw, ncol, nlay, out, cot != nullptr, s);
  h->launches += 5;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(h, e, "adjoint kernel launch");
  return RRTMG_OK;
}

int read_flags(rrtmg_gpu_state* h, cudaStream_t s) {
  unsigned f = 0;
  cudaError_t e = cudaMemcpyAsync(&f, h->flags, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(h, e, "synchronise");
  if (f) {
    cudaMemsetAsync(h->flags, 0, sizeof(unsigned), s);
    cudaStreamSynchronize(s);
    if (f & 1u)
      return fail(h, RRTMG_ERR_INPUT, "non-finite or out-of-range input (pressure <= 0, T <= 0, q outside [0,1), NaN/Inf)");
    if (f & 4u)
      return fail(h, RRTMG_ERR_INPUT,
                  "clouds: an effective size outside its parameterisation's range, or a cloud optical property "
                  "outside its physical range (cldprop / cldprop_sw stop)");
    return fail(h, RRTMG_ERR_INPUT, "SW clouds: a partly cloudy layer (1e-6 < cldfr < 1 - 1e-6) needs McICA");
  }
  return RRTMG_OK;
}


}  // namespace

extern "C" {

const char* rrtmg_gpu_error_string(int status) {
  switch (status) {
    case RRTMG_OK: return "success";
    case RRTMG_ERR_ARG: return "invalid argument";
    case RRTMG_ERR_UNSUPPORTED:
      return "unsupported configuration (icld 0-3; LW inflglw 0-2, iceflglw 0-3, liqflglw 0-1; SW inflgsw 0 or 2, "
             "iceflgsw 1-3, liqflgsw 1, clear or overcast layers; iaer 0/10; idrv 0/1)";
    case RRTMG_ERR_CUDA: return "CUDA error";
    case RRTMG_ERR_TABLES: return "coefficient table blob missing or invalid";
    case RRTMG_ERR_INPUT: return "invalid input values";
    case RRTMG_ERR_NOMEM: return "device memory allocation failed";
    default: return "unknown status";
  }
}

const char* rrtmg_gpu_last_error(rrtmg_gpu_handle h) { return h ? h->err.c_str() : "null handle"; }

long long rrtmg_gpu_launch_count(rrtmg_gpu_handle h) { return h ? h->launches : 0; }

int rrtmg_gpu_init(double cpdair, const char* table_blob, int device, rrtmg_gpu_handle* out) {
  if (!out) return RRTMG_ERR_ARG;
  *out = nullptr;
  if (!(cpdair > 0.0)) return RRTMG_ERR_ARG;
  rrtmg_gpu_state* h = new (std::nothrow) rrtmg_gpu_state();
  if (!h) return RRTMG_ERR_NOMEM;
  std::string err = build_host_tables(table_blob, cpdair, h->host);
  if (!err.empty()) {
    std::fprintf(stderr, "rrtmg_gpu_init: %s\n", err.c_str());
    delete h;
    return RRTMG_ERR_TABLES;
  }
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->stream2, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->side, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->side2, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->fork_ev, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->join_ev, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->fork_ev2, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->join_ev2, cudaEventDisableTiming);
  if (e == cudaSuccess) e = upload(&h->lw_tab64, h->host.lw_tab);
  if (e == cudaSuccess) e = upload(&h->sw_tab64, h->host.sw_tab);
  if (e == cudaSuccess) e = upload(&h->lw_exp64, h->host.lw_exp);
  if (e == cudaSuccess) e = upload(&h->lw_tfn64, h->host.lw_tfn);
  if (e == cudaSuccess) e = upload(&h->lw_tau64, h->host.lw_tau);
  if (e == cudaSuccess) e = upload(&h->lw_tau32, to_f32(h->host.lw_tau));
  if (e == cudaSuccess) e = upload(&h->sw_exp64, h->host.sw_exp);
  if (e == cudaSuccess) e = upload(&h->totplnk, h->host.totplnk);
  if (e == cudaSuccess) e = upload(&h->totplnkderiv, h->host.totplnkderiv);
  if (e == cudaSuccess) e = upload(&h->totplnk32, to_f32(h->host.totplnk));
  if (e == cudaSuccess) e = upload(&h->totplnkderiv32, to_f32(h->host.totplnkderiv));
  if (e == cudaSuccess) e = upload(&h->lw_tab32, to_f32(h->host.lw_tab));
  if (e == cudaSuccess) e = upload(&h->sw_tab32, to_f32(h->host.sw_tab));
  if (e == cudaSuccess) e = upload(&h->lw_exp32, to_f32(h->host.lw_exp));
  if (e == cudaSuccess) e = upload(&h->lw_tfn32, to_f32(h->host.lw_tfn));
  if (e == cudaSuccess) e = upload(&h->lw_exptfn32, interleave_f32(h->host.lw_exp, h->host.lw_tfn));
  if (e == cudaSuccess) e = upload(&h->sw_exp32, to_f32(h->host.sw_exp));
  if (e == cudaSuccess) e = upload(&h->cldtab, h->host.cld);
  if (e == cudaSuccess) e = upload(&h->cldtab32, to_f32(h->host.cld));
  if (e == cudaSuccess) e = cudaMalloc((void**)&h->flags, sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMemset(h->flags, 0, sizeof(unsigned));
  if (e == cudaSuccess) e = upload_constants_fp64(h->host.lw, h->host.sw);
  if (e == cudaSuccess) e = upload_constants_split(h->host.lw, h->host.sw);
  if (e == cudaSuccess) e = upload_constants_adjoint(h->host.lw, h->host.sw);
  if (e != cudaSuccess) {
    std::fprintf(stderr, "rrtmg_gpu_init: %s\n", cudaGetErrorString(e));
    h->device = device;
    rrtmg_gpu_finalize(h);
    return RRTMG_ERR_CUDA;
  }
  h->device = device;
  *out = h;
  return RRTMG_OK;
}

int rrtmg_gpu_finalize(rrtmg_gpu_handle h) {
  if (!h) return RRTMG_ERR_ARG;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  if (h->stream2) cudaStreamSynchronize(h->stream2);
  if (h->side) cudaStreamSynchronize(h->side);
  if (h->side2) cudaStreamSynchronize(h->side2);
  void* ptrs[] = {h->lw_tab64, h->sw_tab64, h->lw_exp64, h->lw_tfn64, h->sw_exp64, h->totplnk, h->totplnkderiv,
                  h->lw_tau64, h->lw_tau32,
                  h->totplnk32, h->totplnkderiv32,
                  h->lw_tab32, h->sw_tab32, h->lw_exp32, h->lw_tfn32, h->lw_exptfn32, h->sw_exp32, h->cldtab, h->cldtab32, h->flags,
                  h->lw_ws.p,
                  h->sw_ws.p, h->adj_ws.p, h->hio[0].p, h->hio[1].p, h->hws[0].p, h->hws[1].p, h->run_ws.p,
                  h->run_cio[0].p, h->run_cio[1].p, h->run_cws[0].p, h->run_cws[1].p};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (h->stream) cudaStreamDestroy(h->stream);
  if (h->stream2) cudaStreamDestroy(h->stream2);
  if (h->side) cudaStreamDestroy(h->side);
  if (h->side2) cudaStreamDestroy(h->side2);
  for (cudaEvent_t ev : {h->fork_ev, h->join_ev, h->fork_ev2, h->join_ev2})
    if (ev) cudaEventDestroy(ev);
  for (auto& fam : h->ev)
    for (auto& e : fam)
      if (e) cudaEventDestroy(e);
  delete h;
  return RRTMG_OK;
}

int rrtmg_gpu_set_precision(rrtmg_gpu_handle h, int precision) {
  if (!valid_handle(h)) return RRTMG_ERR_ARG;
  if (precision != RRTMG_PREC_FP64 && precision != RRTMG_PREC_SPLIT)
    return fail(h, RRTMG_ERR_ARG, "precision must be RRTMG_PREC_FP64 or RRTMG_PREC_SPLIT");
  h->precision = precision;
  return RRTMG_OK;
}

int rrtmg_gpu_set_transcendentals(rrtmg_gpu_handle h, int mode) {
  if (!valid_handle(h)) return RRTMG_ERR_ARG;
  if (mode != RRTMG_TRANS_TABLE && mode != RRTMG_TRANS_ANALYTIC)
    return fail(h, RRTMG_ERR_ARG, "mode must be RRTMG_TRANS_TABLE or RRTMG_TRANS_ANALYTIC");
  h->analytic = mode == RRTMG_TRANS_ANALYTIC;
  return RRTMG_OK;
}

int rrtmg_gpu_set_profiling(rrtmg_gpu_handle h, int on) {
  if (!valid_handle(h)) return RRTMG_ERR_ARG;
  cudaSetDevice(h->device);
  if (on && !h->ev[0][0]) {
    for (auto& fam : h->ev)
      for (auto& e : fam) {
        cudaError_t r = cudaEventCreate(&e);
        if (r != cudaSuccess) return cuda_fail(h, r, "create profiling events");
      }
  }
  h->profiling = on != 0;
  return RRTMG_OK;
}

int rrtmg_gpu_profile(rrtmg_gpu_handle h, float* ms) {
  if (!valid_handle(h) || !ms) return RRTMG_ERR_ARG;
  if (!h->ev[0][0]) return fail(h, RRTMG_ERR_ARG, "profiling was never enabled on this handle");
  for (int f = 0; f < 2; ++f)
    for (int k = 0; k < 3; ++k) {
      cudaError_t r = cudaEventSynchronize(h->ev[f][k + 1]);
      if (r == cudaSuccess) r = cudaEventElapsedTime(&ms[3 * f + k], h->ev[f][k], h->ev[f][k + 1]);
      if (r != cudaSuccess) return cuda_fail(h, r, "read profiling events");
    }
  return RRTMG_OK;
}

int rrtmg_gpu_reserve(rrtmg_gpu_handle h, int ncol, int nlay) {
  if (!valid_handle(h)) return RRTMG_ERR_ARG;
  int rc = check_dims(h, ncol, nlay);
  if (rc) return rc;
  cudaSetDevice(h->device);
  size_t a, b;
  carve_lw(nullptr, ncol, nlay, &a);
  carve_sw(nullptr, ncol, nlay, &b);
  rc = ensure(h, h->lw_ws, a, nullptr);
  if (rc) return rc;
  return ensure(h, h->sw_ws, b, nullptr);
}

int rrtmg_gpu_sync_status(rrtmg_gpu_handle h, void* stream) {
  if (!valid_handle(h)) return RRTMG_ERR_ARG;
  return read_flags(h, (cudaStream_t)stream);
}

int rrtmg_lw_dev(rrtmg_gpu_handle h, void* stream, int ncol, int nlay, int icld, int idrv, const double* play,
                 const double* plev, const double* tlay, const double* tlev, const double* tsfc, const double* h2ovmr,
                 const double* o3vmr, const double* co2vmr, const double* ch4vmr, const double* n2ovmr,
                 const double* o2vmr, const double* cfc11vmr, const double* cfc12vmr, const double* cfc22vmr,
                 const double* ccl4vmr, const double* emis, int inflglw, int iceflglw, int liqflglw,
                 const double* cldfr, const double* taucld, const double* cicewp, const double* cliqwp,
                 const double* reice, const double* reliq, const double* tauaer, double* uflx, double* dflx,
                 double* hr, double* uflxc, double* dflxc, double* hrc, double* duflx_dt, double* duflxc_dt) {
  if (!valid_handle(h)) return RRTMG_ERR_ARG;
  int rc = check_dims(h, ncol, nlay);
  if (rc) return rc;
  rc = lw_cloud_args(h, icld, inflglw, iceflglw, liqflglw, cldfr, taucld, cicewp, cliqwp, reice, reliq);
  if (rc) return rc;
  if (idrv != 0 && idrv != 1) return fail(h, RRTMG_ERR_UNSUPPORTED, "idrv must be 0 or 1");
  if (!play || !plev || !tlay || !tlev || !tsfc || !h2ovmr || !o3vmr || !co2vmr || !uflx || !dflx || !hr ||
      !uflxc || !dflxc || !hrc)
    return fail(h, RRTMG_ERR_ARG, "a required array pointer is null");
  if (idrv == 1 && !duflx_dt) return fail(h, RRTMG_ERR_ARG, "idrv = 1 needs duflx_dt");
  cudaSetDevice(h->device);
  LwIn in{play, plev, tlay, tlev, tsfc, h2ovmr, o3vmr, co2vmr, ch4vmr, n2ovmr, o2vmr, cfc11vmr, cfc12vmr,
          cfc22vmr, ccl4vmr, emis, tauaer};
  if (icld != 0) {
    in.cldfr = cldfr;
    in.taucld = taucld;
    in.cicewp = cicewp;
    in.cliqwp = cliqwp;
    in.icld = icld;
    in.inflag = inflglw;
    in.iceflag = iceflglw;
    in.liqflag = liqflglw;
    in.reice = reice;
    in.reliq = reliq;
  }
  return lw_run(h, (cudaStream_t)stream, ncol, nlay, idrv, in, uflx, dflx, hr, uflxc, dflxc, hrc, duflx_dt,
                duflxc_dt);
}

int rrtmg_sw_dev(rrtmg_gpu_handle h, void* stream, int ncol, int nlay, int icld, int iaer, const double* play,
                 const double* plev, const double* tlay, const double* tlev, const double* tsfc, const double* h2ovmr,
                 const double* o3vmr, const double* co2vmr, const double* ch4vmr, const double* n2ovmr,
                 const double* o2vmr, const double* asdir, const double* asdif, const double* aldir,
                 const double* aldif, const double* coszen, double adjes, int dyofyr, double scon, int inflgsw,
                 int iceflgsw, int liqflgsw, const double* cldfr, const double* taucld, const double* ssacld,
                 const double* asmcld, const double* fsfcld, const double* cicewp, const double* cliqwp,
                 const double* reice, const double* reliq, const double* tauaer, const double* ssaaer,
                 const double* asmaer, const double* ecaer, double* swuflx, double* swdflx, double* swhr,
                 double* swuflxc, double* swdflxc, double* swhrc) {
  (void)ecaer;
  if (!valid_handle(h)) return RRTMG_ERR_ARG;
  int rc = check_dims(h, ncol, nlay);
  if (rc) return rc;
  rc = sw_cloud_args(h, icld, inflgsw, iceflgsw, liqflgsw, cldfr, taucld, ssacld, asmcld, fsfcld, cicewp, cliqwp,
                     reice, reliq);
  if (rc) return rc;
  if (iaer != 0 && iaer != 10) return fail(h, RRTMG_ERR_UNSUPPORTED, "iaer must be 0 or 10");
  if (!play || !plev || !tlay || !tlev || !tsfc || !h2ovmr || !o3vmr || !co2vmr || !asdir || !asdif || !aldir ||
      !aldif || !coszen || !swuflx || !swdflx || !swhr || !swuflxc || !swdflxc || !swhrc)
    return fail(h, RRTMG_ERR_ARG, "a required array pointer is null");
  if (iaer == 10 && (!tauaer || !ssaaer || !asmaer)) return fail(h, RRTMG_ERR_ARG, "iaer = 10 needs tauaer/ssaaer/asmaer");
  if (!(scon > 0.0)) return fail(h, RRTMG_ERR_ARG, "scon must be positive");
  cudaSetDevice(h->device);
  SwIn in{play, plev, tlay, tlev, tsfc, h2ovmr, o3vmr, co2vmr, ch4vmr, n2ovmr, o2vmr, asdir, asdif, aldir, aldif,
          coszen, tauaer, ssaaer, asmaer};
  if (icld != 0) {
    in.cldfr = cldfr;
    in.taucld = taucld;
    in.ssacld = ssacld;
    in.asmcld = asmcld;
    in.fsfcld = fsfcld;
    in.cicewp = cicewp;
    in.cliqwp = cliqwp;
    in.inflag = inflgsw;
    in.iceflag = iceflgsw;
    in.liqflag = liqflgsw;
    in.reice = reice;
    in.reliq = reliq;
  }
  return sw_run(h, (cudaStream_t)stream, ncol, nlay, iaer, adjes, dyofyr, scon, in, swuflx, swdflx, swhr, swuflxc,
                swdflxc, swhrc);
}

int rrtmg_step_dev(rrtmg_gpu_handle h, void* stream, int ncol, int nlay, int idrv, int iaer, const double* play,
                   const double* plev, const double* tlay, const double* tlev, const double* tsfc,
                   const double* h2ovmr, const double* o3vmr, const double* co2vmr, const double* ch4vmr,
                   const double* n2ovmr, const double* o2vmr, const double* cfc11vmr, const double* cfc12vmr,
                   const double* cfc22vmr, const double* ccl4vmr, const double* emis, const double* tauaer_lw,
                   const double* asdir, const double* asdif, const double* aldir, const double* aldif,
                   const double* coszen, double adjes, int dyofyr, double scon, const double* tauaer_sw,
                   const double* ssaaer, const double* asmaer, double* uflx, double* dflx, double* hr,
                   double* uflxc, double* dflxc, double* hrc, double* duflx_dt, double* duflxc_dt,
                   double* swuflx, double* swdflx, double* swhr, double* swuflxc, double* swdflxc,
                   double* swhrc) {
  if (!valid_handle(h)) return RRTMG_ERR_ARG;
  int rc = check_dims(h, ncol, nlay);
  if (rc) return rc;
  if (idrv != 0 && idrv != 1) return fail(h, RRTMG_ERR_UNSUPPORTED, "idrv must be 0 or 1");
  if (iaer != 0 && iaer != 10) return fail(h, RRTMG_ERR_UNSUPPORTED, "iaer must be 0 or 10");
  if (!play || !plev || !tlay || !tlev || !tsfc || !h2ovmr || !o3vmr || !co2vmr || !asdir || !asdif || !aldir ||
      !aldif || !coszen || !uflx || !dflx || !hr || !uflxc || !dflxc || !hrc || !swuflx || !swdflx || !swhr ||
      !swuflxc || !swdflxc || !swhrc)
    return fail(h, RRTMG_ERR_ARG, "a required array pointer is null");
  if (idrv == 1 && !duflx_dt) return fail(h, RRTMG_ERR_ARG, "idrv = 1 needs duflx_dt");
  if (iaer == 10 && (!tauaer_sw || !ssaaer || !asmaer))
    return fail(h, RRTMG_ERR_ARG, "iaer = 10 needs tauaer/ssaaer/asmaer");
  if (!(scon > 0.0)) return fail(h, RRTMG_ERR_ARG, "scon must be positive");
  cudaSetDevice(h->device);
  const LwIn lin{play, plev, tlay, tlev, tsfc, h2ovmr, o3vmr, co2vmr, ch4vmr, n2ovmr, o2vmr, cfc11vmr, cfc12vmr,
                 cfc22vmr, ccl4vmr, emis, tauaer_lw};
  const SwIn sin{play, plev, tlay, tlev, tsfc, h2ovmr, o3vmr, co2vmr, ch4vmr, n2ovmr, o2vmr, asdir, asdif, aldir,
                 aldif, coszen, tauaer_sw, ssaaer, asmaer};
  return fork_lw_sw(
      h, (cudaStream_t)stream, default_fork(h),
      [&](cudaStream_t s) {
        return lw_run(h, s, ncol, nlay, idrv, lin, uflx, dflx, hr, uflxc, dflxc, hrc, duflx_dt, duflxc_dt);
      },
      [&](cudaStream_t s) {
        return sw_run(h, s, ncol, nlay, iaer, adjes, dyofyr, scon, sin, swuflx, swdflx, swhr, swuflxc, swdflxc,
                      swhrc);
      });
}

static int adjoint_entry(rrtmg_gpu_handle h, void* stream, int ncol, int nlay, const double* play,
                         const double* plev, const double* tlay, const double* tlev, const double* tsfc,
                         const double* h2ovmr, const double* o3vmr, const double* co2vmr, const double* ch4vmr,
                         const double* n2ovmr, const double* o2vmr, const double* cfc11vmr,
                         const double* cfc12vmr, const double* cfc22vmr, const double* ccl4vmr,
                         const double* emis, const double* tauaer_lw, const double* asdir, const double* asdif,
                         const double* aldir, const double* aldif, const double* coszen, double adjes, int dyofyr,
                         double scon, int iaer, const double* tauaer_sw, const double* ssaaer,
                         const double* asmaer, const double* cot, double* out) {
  if (!valid_handle(h)) return RRTMG_ERR_ARG;
  int rc = check_dims(h, ncol, nlay);
  if (rc) return rc;
  if (iaer != 0 && iaer != 10) return fail(h, RRTMG_ERR_UNSUPPORTED, "iaer must be 0 or 10");
  if (!play || !plev || !tlay || !tlev || !tsfc || !h2ovmr || !o3vmr || !co2vmr || !asdir || !asdif || !aldir ||
      !aldif || !coszen || !out)
    return fail(h, RRTMG_ERR_ARG, "a required array pointer is null");
  if (iaer == 10 && (!tauaer_sw || !ssaaer || !asmaer))
    return fail(h, RRTMG_ERR_ARG, "iaer = 10 needs tauaer/ssaaer/asmaer");
  if (!(scon > 0.0)) return fail(h, RRTMG_ERR_ARG, "scon must be positive");
  if ((long long)kLwBands * (nlay + 2) * (3LL * nlay + 3) * ncol > (1LL << 40))
    return fail(h, RRTMG_ERR_ARG, "too many columns for one Jacobian call; split the columns");
  cudaSetDevice(h->device);
  LwIn lin{play, plev, tlay, tlev, tsfc, h2ovmr, o3vmr, co2vmr, ch4vmr, n2ovmr, o2vmr, cfc11vmr, cfc12vmr,
           cfc22vmr, ccl4vmr, emis, tauaer_lw};
  SwIn sin{play, plev, tlay, tlev, tsfc, h2ovmr, o3vmr, co2vmr, ch4vmr, n2ovmr, o2vmr, asdir, asdif, aldir, aldif,
           coszen, tauaer_sw, ssaaer, asmaer};
  return adj_run(h, (cudaStream_t)stream, ncol, nlay, lin, sin, iaer, adjflux_of(h, adjes, dyofyr, scon), cot, out);
}

int rrtmg_jacobian_dev(rrtmg_gpu_handle h, void* stream, int ncol, int nlay, const double* play, const double* plev,
                       const double* tlay, const double* tlev, const double* tsfc, const double* h2ovmr,
                       const double* o3vmr, const double* co2vmr, const double* ch4vmr, const double* n2ovmr,
                       const double* o2vmr, const double* cfc11vmr, const double* cfc12vmr, const double* cfc22vmr,
                       const double* ccl4vmr, const double* emis, const double* tauaer_lw, const double* asdir,
                       const double* asdif, const double* aldir, const double* aldif, const double* coszen,
                       double adjes, int dyofyr, double scon, int iaer, const double* tauaer_sw,
                       const double* ssaaer, const double* asmaer, double* jac) {
  return adjoint_entry(h, stream, ncol, nlay, play, plev, tlay, tlev, tsfc, h2ovmr, o3vmr, co2vmr, ch4vmr, n2ovmr,
                       o2vmr, cfc11vmr, cfc12vmr, cfc22vmr, ccl4vmr, emis, tauaer_lw, asdir, asdif, aldir, aldif,
                       coszen, adjes, dyofyr, scon, iaer, tauaer_sw, ssaaer, asmaer, nullptr, jac);
}

int rrtmg_vjp_dev(rrtmg_gpu_handle h, void* stream, int ncol, int nlay, const double* play, const double* plev,
                  const double* tlay, const double* tlev, const double* tsfc, const double* h2ovmr,
                  const double* o3vmr, const double* co2vmr, const double* ch4vmr, const double* n2ovmr,
                  const double* o2vmr, const double* cfc11vmr, const double* cfc12vmr, const double* cfc22vmr,
                  const double* ccl4vmr, const double* emis, const double* tauaer_lw, const double* asdir,
                  const double* asdif, const double* aldir, const double* aldif, const double* coszen,
                  double adjes, int dyofyr, double scon, int iaer, const double* tauaer_sw, const double* ssaaer,
                  const double* asmaer, const double* cot, double* grad) {
  if (!cot) return fail(h, RRTMG_ERR_ARG, "rrtmg_vjp_dev needs cotangents");
  return adjoint_entry(h, stream, ncol, nlay, play, plev, tlay, tlev, tsfc, h2ovmr, o3vmr, co2vmr, ch4vmr, n2ovmr,
                       o2vmr, cfc11vmr, cfc12vmr, cfc22vmr, ccl4vmr, emis, tauaer_lw, asdir, asdif, aldir, aldif,
                       coszen, adjes, dyofyr, scon, iaer, tauaer_sw, ssaaer, asmaer, cot, grad);
}

int rrtmg_lw_c(rrtmg_gpu_handle h, int ncol, int nlay, int icld, int idrv, const double* play, const double* plev,
               const double* tlay, const double* tlev, const double* tsfc, const double* h2ovmr, const double* o3vmr,
               const double* co2vmr, const double* ch4vmr, const double* n2ovmr, const double* o2vmr,
               const double* cfc11vmr, const double* cfc12vmr, const double* cfc22vmr, const double* ccl4vmr,
               const double* emis, int inflglw, int iceflglw, int liqflglw, const double* cldfr, const double* taucld,
               const double* cicewp, const double* cliqwp, const double* reice, const double* reliq,
               const double* tauaer, double* uflx, double* dflx, double* hr, double* uflxc, double* dflxc,
               double* hrc, double* duflx_dt, double* duflxc_dt) {
  if (!valid_handle(h)) return RRTMG_ERR_ARG;
  int rc = check_dims(h, ncol, nlay);
  if (rc) return rc;
  rc = lw_cloud_args(h, icld, inflglw, iceflglw, liqflglw, cldfr, taucld, cicewp, cliqwp, reice, reliq);
  if (rc) return rc;
  if (idrv != 0 && idrv != 1) return fail(h, RRTMG_ERR_UNSUPPORTED, "idrv must be 0 or 1");
  if (!play || !plev || !tlay || !tlev || !tsfc || !h2ovmr || !o3vmr || !co2vmr || !uflx || !dflx || !hr ||
      !uflxc || !dflxc || !hrc)
    return fail(h, RRTMG_ERR_ARG, "a required array pointer is null");
  if (idrv == 1 && !duflx_dt) return fail(h, RRTMG_ERR_ARG, "idrv = 1 needs duflx_dt");
  cudaSetDevice(h->device);
  const bool cloudy = icld != 0, phys2 = cloudy && inflglw == 2;
  const size_t L = nlay, Lv = nlay + 1;
  const HostIn in[23] = {{play, L}, {plev, Lv}, {tlay, L}, {tlev, Lv}, {tsfc, 1}, {h2ovmr, L}, {o3vmr, L},
                         {co2vmr, L}, {ch4vmr, L}, {n2ovmr, L}, {o2vmr, L}, {cfc11vmr, L}, {cfc12vmr, L},
                         {cfc22vmr, L}, {ccl4vmr, L}, {emis, 16}, {tauaer, 16 * L},
                         {cloudy ? cldfr : nullptr, L}, {cloudy ? taucld : nullptr, L, 16},
                         {cloudy ? cicewp : nullptr, L}, {cloudy ? cliqwp : nullptr, L},
                         {phys2 ? reice : nullptr, L}, {phys2 ? reliq : nullptr, L}};
  const HostOut out[8] = {{uflx, Lv}, {dflx, Lv}, {hr, L}, {uflxc, Lv}, {dflxc, Lv}, {hrc, L},
                          {idrv == 1 ? duflx_dt : nullptr, Lv}, {idrv == 1 ? duflxc_dt : nullptr, Lv}};
  auto need = [&](int nc) {
    size_t b;
    carve_lw(nullptr, nc, nlay, &b, cloudy, icld >= 2, cloudy && inflglw != 0);
    return b;
  };
  auto enq = [&](cudaStream_t s, void* ws, int nc, const double* const* d, double* const* o) {
    LwIn li{d[0],  d[1],  d[2],  d[3],  d[4],  d[5],  d[6],  d[7],  d[8],  d[9], d[10],
            d[11], d[12], d[13], d[14], d[15], d[16], d[17], d[18], d[19], d[20], icld};
    if (cloudy) {
      li.inflag = inflglw;
      li.iceflag = iceflglw;
      li.liqflag = liqflglw;
      li.reice = d[21];
      li.reliq = d[22];
    }
    return lw_enqueue(h, s, ws, nc, nlay, idrv, li, o[0], o[1], o[2], o[3], o[4], o[5], o[6], o[7]);
  };
  return host_call(h, ncol, in, 23, out, 8, need, enq, "copy LW arrays");
}

int rrtmg_sw_c(rrtmg_gpu_handle h, int ncol, int nlay, int icld, int iaer, const double* play, const double* plev,
               const double* tlay, const double* tlev, const double* tsfc, const double* h2ovmr, const double* o3vmr,
               const double* co2vmr, const double* ch4vmr, const double* n2ovmr, const double* o2vmr,
               const double* asdir, const double* asdif, const double* aldir, const double* aldif,
               const double* coszen, double adjes, int dyofyr, double scon, int inflgsw, int iceflgsw,
               int liqflgsw, const double* cldfr, const double* taucld, const double* ssacld, const double* asmcld,
               const double* fsfcld, const double* cicewp, const double* cliqwp, const double* reice,
               const double* reliq, const double* tauaer, const double* ssaaer, const double* asmaer,
               const double* ecaer, double* swuflx, double* swdflx, double* swhr, double* swuflxc, double* swdflxc,
               double* swhrc) {
  (void)ecaer;
  if (!valid_handle(h)) return RRTMG_ERR_ARG;
  int rc = check_dims(h, ncol, nlay);
  if (rc) return rc;
  rc = sw_cloud_args(h, icld, inflgsw, iceflgsw, liqflgsw, cldfr, taucld, ssacld, asmcld, fsfcld, cicewp, cliqwp,
                     reice, reliq);
  if (rc) return rc;
  if (iaer != 0 && iaer != 10) return fail(h, RRTMG_ERR_UNSUPPORTED, "iaer must be 0 or 10");
  if (!play || !plev || !tlay || !tlev || !tsfc || !h2ovmr || !o3vmr || !co2vmr || !asdir || !asdif || !aldir ||
      !aldif || !coszen || !swuflx || !swdflx || !swhr || !swuflxc || !swdflxc || !swhrc)
    return fail(h, RRTMG_ERR_ARG, "a required array pointer is null");
  if (iaer == 10 && (!tauaer || !ssaaer || !asmaer)) return fail(h, RRTMG_ERR_ARG, "iaer = 10 needs tauaer/ssaaer/asmaer");
  if (!(scon > 0.0)) return fail(h, RRTMG_ERR_ARG, "scon must be positive");
  cudaSetDevice(h->device);
  const size_t L = nlay, Lv = nlay + 1;
  const bool aer = iaer == 10, cloudy = icld != 0, phys = cloudy && inflgsw == 2;
  auto cl = [&](const double* a) { return cloudy ? a : nullptr; };
  auto ph = [&](const double* a) { return phys ? a : nullptr; };
  const HostIn in[28] = {{play, L}, {plev, Lv}, {tlay, L}, {tlev, Lv}, {tsfc, 1}, {h2ovmr, L}, {o3vmr, L},
                         {co2vmr, L}, {ch4vmr, L}, {n2ovmr, L}, {o2vmr, L}, {asdir, 1}, {asdif, 1}, {aldir, 1},
                         {aldif, 1}, {coszen, 1}, {aer ? tauaer : nullptr, 14 * L}, {aer ? ssaaer : nullptr, 14 * L},
                         {aer ? asmaer : nullptr, 14 * L}, {cl(cldfr), L}, {cl(taucld), L, 14}, {cl(ssacld), L, 14},
                         {cl(asmcld), L, 14}, {cl(fsfcld), L, 14}, {cl(cicewp), L}, {cl(cliqwp), L},
                         {ph(reice), L}, {ph(reliq), L}};
  const HostOut out[6] = {{swuflx, Lv}, {swdflx, Lv}, {swhr, L}, {swuflxc, Lv}, {swdflxc, Lv}, {swhrc, L}};
  auto need = [&](int nc) {
    size_t b;
    carve_sw(nullptr, nc, nlay, &b, cloudy, phys, h->precision == RRTMG_PREC_SPLIT);
    return b;
  };
  auto enq = [&](cudaStream_t s, void* ws, int nc, const double* const* d, double* const* o) {
    SwIn si{d[0],  d[1],  d[2],  d[3],  d[4],  d[5],  d[6],  d[7],  d[8],  d[9],  d[10], d[11], d[12],
            d[13], d[14], d[15], d[16], d[17], d[18], d[19], d[20], d[21], d[22], d[23], d[24], d[25]};
    if (cloudy) {
      si.inflag = inflgsw;
      si.iceflag = iceflgsw;
      si.liqflag = liqflgsw;
      si.reice = d[26];
      si.reliq = d[27];
    }
    return sw_enqueue(h, s, ws, nc, nlay, iaer, adjes, dyofyr, scon, si, o[0], o[1], o[2], o[3], o[4], o[5]);
  };
  return host_call(h, ncol, in, 28, out, 6, need, enq, "copy SW arrays");
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free LW device call (rrtmg_lw_dev_static).
//
// The LW scratch (per-layer optics, Planck terms, band partial fluxes) lives in
// one file-scope device array of RRTMG_GPU_STATIC_SCRATCH_BYTES that every
// device loading this library holds until process exit.  In host code
// `g_lw_static_scratch` is only a stand-in for the symbol; its device address
// is looked up once per device with cudaGetSymbolAddress, with that device
// current, on the first call made on that device.  Every scratch word a call
// reads is written earlier by the same call (prep writes all per-layer fields,
// the g-point kernel writes every level of every band partial, including the
// zero downward flux at the top), so no clearing is needed; the validation
// flag word is the handle's.  All calls on a device share the array, so calls
// that overlap on the GPU race.
// ---------------------------------------------------------------------------
#include <mutex>

static __device__ __align__(256) unsigned char g_lw_static_scratch[RRTMG_GPU_STATIC_SCRATCH_BYTES];

namespace {

constexpr int kMaxStaticDevices = 64;
std::mutex g_static_mu;
void* g_static_ptr[kMaxStaticDevices] = {};

// Device address of g_lw_static_scratch on `device` (current), looked up once.
cudaError_t static_scratch(int device, void** out) {
  std::lock_guard<std::mutex> lock(g_static_mu);
  if (!g_static_ptr[device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_lw_static_scratch);
    if (e != cudaSuccess) return e;
    g_static_ptr[device] = p;
  }
  *out = g_static_ptr[device];
  return cudaSuccess;
}

}  // namespace

extern "C" int rrtmg_lw_dev_static(rrtmg_gpu_handle h, void* stream, int ncol, int nlay, int icld, int idrv,
                                   const double* play, const double* plev, const double* tlay, const double* tlev,
                                   const double* tsfc, const double* h2ovmr, const double* o3vmr,
                                   const double* co2vmr, const double* ch4vmr, const double* n2ovmr,
                                   const double* o2vmr, const double* cfc11vmr, const double* cfc12vmr,
                                   const double* cfc22vmr, const double* ccl4vmr, const double* emis, int inflglw,
                                   int iceflglw, int liqflglw, const double* cldfr, const double* taucld,
                                   const double* cicewp, const double* cliqwp, const double* reice,
                                   const double* reliq, const double* tauaer, double* uflx, double* dflx,
                                   double* hr, double* uflxc, double* dflxc, double* hrc, double* duflx_dt,
                                   double* duflxc_dt) {
  (void)inflglw; (void)iceflglw; (void)liqflglw; (void)cldfr; (void)taucld; (void)cicewp; (void)cliqwp;
  (void)reice; (void)reliq;
  if (!valid_handle(h)) return RRTMG_ERR_ARG;
  int rc = check_dims(h, ncol, nlay);
  if (rc) return rc;
  if (icld != 0) return fail(h, RRTMG_ERR_UNSUPPORTED, "only clear sky (icld = 0) is computed");
  if (idrv != 0 && idrv != 1) return fail(h, RRTMG_ERR_UNSUPPORTED, "idrv must be 0 or 1");
  if (!play || !plev || !tlay || !tlev || !tsfc || !h2ovmr || !o3vmr || !co2vmr || !uflx || !dflx || !hr ||
      !uflxc || !dflxc || !hrc)
    return fail(h, RRTMG_ERR_ARG, "a required array pointer is null");
  if (idrv == 1 && !duflx_dt) return fail(h, RRTMG_ERR_ARG, "idrv = 1 needs duflx_dt");
  size_t need;
  carve_lw(nullptr, ncol, nlay, &need);
  if (need > (size_t)RRTMG_GPU_STATIC_SCRATCH_BYTES)
    return fail(h, RRTMG_ERR_ARG,
                "rrtmg_lw_dev_static: " + std::to_string(ncol) + " columns x " + std::to_string(nlay) +
                    " layers need " + std::to_string(need) + " bytes of scratch, more than the static limit of " +
                    std::to_string((size_t)RRTMG_GPU_STATIC_SCRATCH_BYTES) + " bytes; split the columns");
  if (h->device < 0 || h->device >= kMaxStaticDevices)
    return fail(h, RRTMG_ERR_ARG, "rrtmg_lw_dev_static: device ordinal out of range");
  cudaError_t e = cudaSetDevice(h->device);
  if (e != cudaSuccess) return cuda_fail(h, e, "rrtmg_lw_dev_static: set device");
  void* base = nullptr;
  e = static_scratch(h->device, &base);
  if (e != cudaSuccess) return cuda_fail(h, e, "rrtmg_lw_dev_static: cudaGetSymbolAddress");
  LwIn in{play, plev, tlay, tlev, tsfc, h2ovmr, o3vmr, co2vmr, ch4vmr, n2ovmr, o2vmr, cfc11vmr, cfc12vmr,
          cfc22vmr, ccl4vmr, emis, tauaer};
  return lw_enqueue(h, (cudaStream_t)stream, base, ncol, nlay, idrv, in, uflx, dflx, hr, uflxc, dflxc, hrc,
                    duflx_dt, duflxc_dt);
}

// ---------------------------------------------------------------------------
// run_rrtmg on the device (include/rrtmg_run.h): GCM slab -> RRTM columns ->
// rrtmg_sw + rrtmg_lw -> GCM tendencies, all on one stream.
// ---------------------------------------------------------------------------
namespace {

struct RunWork {
  RunCols c;
  double *uflx, *dflx, *hr, *uflxc, *dflxc, *hrc;
  double *swuflx, *swdflx, *swhr, *swuflxc, *swdflxc, *swhrc;
  double *zq, *zp, *zt, *zsw, *zlw;
  unsigned* flag;
};

RunWork carve_run(void* base, int sj, int sk, int ncol, bool secondary, size_t* bytes) {
  Carver cv{(char*)base};
  const size_t N = (size_t)ncol, L = (size_t)sk, Lv = L + 1;
  RunWork w;
  w.c.play = cv.take<double>(L * N);
  w.c.plev = cv.take<double>(Lv * N);
  w.c.tlay = cv.take<double>(L * N);
  w.c.tlev = cv.take<double>(Lv * N);
  w.c.tsfc = cv.take<double>(N);
  w.c.h2o = cv.take<double>(L * N);
  w.c.o3 = cv.take<double>(L * N);
  w.c.co2 = cv.take<double>(L * N);
  w.c.emis = cv.take<double>(16 * N);
  w.c.alb = cv.take<double>(N);
  w.c.cosz = cv.take<double>(N);
  for (int m = 0; m < 7; ++m) w.c.gas[m] = secondary ? cv.take<double>(L * N) : nullptr;
  double** lev[] = {&w.uflx, &w.dflx, &w.uflxc, &w.dflxc, &w.swuflx, &w.swdflx, &w.swuflxc, &w.swdflxc};
  for (double** p : lev) *p = cv.take<double>(Lv * N);
  double** lay[] = {&w.hr, &w.hrc, &w.swhr, &w.swhrc};
  for (double** p : lay) *p = cv.take<double>(L * N);
  w.zq = cv.take<double>((size_t)sj * L);
  w.zt = cv.take<double>((size_t)sj * L);
  w.zp = cv.take<double>(sj);
  w.zsw = cv.take<double>(sj);
  w.zlw = cv.take<double>(sj);
  w.flag = cv.take<unsigned>(1);
  if (bytes) *bytes = cv.off;
  return w;
}

struct RunArgs {
  int si, sj, sk, seconds, days, days_per_year;
  RunGcm g;
  RunOut o;
};

// Argument checks shared by the device and host entry points.
int run_check(rrtmg_gpu_state* h, const rrtmg_run_params* p, const RunArgs& a) {
  if (!valid_handle(h)) return RRTMG_ERR_ARG;
  if (!p) return fail(h, RRTMG_ERR_ARG, "null rrtmg_run_params");
  if (a.si < 1 || a.sj < 1) return fail(h, RRTMG_ERR_ARG, "si and sj must be >= 1");
  if (p->lonstep < 1 || a.si % p->lonstep != 0) return fail(h, RRTMG_ERR_ARG, "si must be a multiple of lonstep >= 1");
  if (a.days_per_year < 1) return fail(h, RRTMG_ERR_ARG, "days_per_year must be >= 1");
  if (p->dt_rad_avg < 0) return fail(h, RRTMG_ERR_ARG, "dt_rad_avg must be >= 0 (resolve dt_rad_avg < 0 to dt_rad)");
  int rc = check_dims(h, a.si / p->lonstep * a.sj, a.sk);
  if (rc) return rc;
  const RunGcm& g = a.g;
  if (!g.lat || !g.lon || !g.p_full || !g.p_half || !g.z_full || !g.z_half || !g.t || !g.q || !g.t_surf ||
      !g.albedo || !a.o.tdt || !a.o.coszen)
    return fail(h, RRTMG_ERR_ARG, "a required array pointer is null");
  if ((a.o.flux_sw == nullptr) != (a.o.flux_lw == nullptr))
    return fail(h, RRTMG_ERR_ARG, "flux_sw and flux_lw: both or neither");
  if (p->do_precip_albedo && p->num_precip > 0 && !g.precip)
    return fail(h, RRTMG_ERR_ARG, "do_precip_albedo with num_precip > 0 needs rrtm_precip");
  if (!(p->solr_cnst > 0.0)) return fail(h, RRTMG_ERR_ARG, "solr_cnst must be positive");
  return RRTMG_OK;
}

// Model time of the radiation (rrtm_radiation.f90:550-558) and the
// declination terms of compute_zenith (astro.f90:98-137).
RunScalars run_scalars(const rrtmg_run_params& p, const RunArgs& a, int* dyofyr) {
  const double pi = 3.14159265358979323846;
  long long sec = a.seconds, days = a.days;
  if (p.solday > 0) {
    days = p.solday;
  } else if (p.slowdown_rad != 1.0) {
    const long long t = (long long)((double)(days * 86400 + sec) * p.slowdown_rad);
    days = t / 86400;
    sec = t % 86400;
  }
  RunScalars s{};
  s.si = a.si;
  s.sj = a.sj;
  s.sk = a.sk;
  s.lonstep = p.lonstep;
  s.nsub = a.si / p.lonstep;
  s.ncol = s.nsub * a.sj;
  const int dpy = a.days_per_year;
  s.radpersec = 2 * pi / 86400.;
  const double radperday = 2 * pi / dpy;
  s.radsec = (double)sec * s.radpersec;
  s.zen_dt = p.dt_rad_avg;
  s.dt_pi = (double)p.dt_rad_avg * s.radpersec;
  long long d = days - (long long)(p.equinox_day * dpy);
  d %= dpy;
  if (d < 0) d += dpy;
  const double radday = (double)d * radperday;
  s.dec_sin = std::sin(p.obliq * (pi / 180.)) * std::sin(radday);
  const double dec = std::asin(s.dec_sin);
  s.dec_cos = std::cos(dec);
  s.dec_tan = std::tan(dec);
  *dyofyr = p.use_dyofyr ? (int)d : 0;  // rrtm_radiation.f90:598
  s.zm_tracers = p.do_zm_tracers != 0;
  s.fixed_water = p.do_fixed_water != 0;
  s.secondary = p.include_secondary_gases != 0;
  s.precip_albedo = p.do_precip_albedo != 0 && p.num_precip > 0;
  s.zm_rad = p.do_zm_rad != 0;
  s.h2o_lo = p.h2o_lower_limit;
  s.t_lo = p.temp_lower_limit;
  s.t_hi = p.temp_upper_limit;
  s.co2 = p.co2ppmv * 1.e-6;
  s.o3_val = p.o3_val;
  s.fixed_water_val = p.fixed_water;
  s.fixed_water_pres = p.fixed_water_pres;
  s.fixed_water_lat = p.fixed_water_lat;
  s.precip_albedo_val = p.precip_albedo;
  s.precip_lat = p.precip_lat;
  s.num_precip = p.num_precip;
  const double gv[7] = {p.ch4_val, p.n2o_val, p.o2_val, p.cfc11_val, p.cfc12_val, p.cfc22_val, p.ccl4_val};
  for (int m = 0; m < 7; ++m) s.gas_val[m] = gv[m];
  return s;
}

// Enqueues run_rrtmg on stream st.  Scratch (RRTM columns, results, zonal sums,
// the LW and SW scratch) is carved from ws; the SW call is forked onto fk.side.
// top: -1 to find on the device whether some top interface is at 0 Pa (the
// whole slab is in the call), else the host's answer for the whole slab (the
// call is a latitude chunk of it).
int run_enqueue(rrtmg_gpu_state* h, cudaStream_t st, const rrtmg_run_params& p, const RunArgs& a, DevBuf& ws,
                const Fork& fk, int top) {
  int dyofyr = 0;
  const RunScalars s = run_scalars(p, a, &dyofyr);
  size_t nrun, nlw, nsw;
  carve_run(nullptr, a.sj, a.sk, s.ncol, s.secondary, &nrun);
  carve_lw(nullptr, s.ncol, a.sk, &nlw);
  carve_sw(nullptr, s.ncol, a.sk, &nsw);
  int rc = ensure(h, ws, nrun + nlw + nsw, st);
  if (rc) return rc;
  const RunWork w = carve_run(ws.p, a.sj, a.sk, s.ncol, s.secondary, nullptr);
  void* lw_base = (char*)ws.p + nrun;
  void* sw_base = (char*)lw_base + nlw;
  // the flag is read as zero / nonzero
  cudaError_t e = cudaMemsetAsync(w.flag, top > 0 ? 1 : 0, sizeof(unsigned), st);
  if (e != cudaSuccess) return cuda_fail(h, e, "run_rrtmg: clear flag");
  launch_run_zonal(s, a.g, a.o.coszen, w.zq, w.zp, w.flag, st);
  if (a.o.t_half) launch_run_thalf(s, a.g, a.o.t_half, st);
  launch_run_prep(s, a.g, a.o.coszen, w.zq, w.zp, w.flag, w.c, st);
  h->launches += a.o.t_half ? 3 : 2;
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(h, e, "run_rrtmg: input kernels");
  const RunCols& c = w.c;
  // rrtm_radiation.f90:683-713 (SW) and :718-749 (LW), clear sky, iaer = idrv = 0;
  // the two calls are independent and run concurrently
  const SwIn sin{c.play, c.plev, c.tlay, c.tlev, c.tsfc, c.h2o, c.o3, c.co2, c.gas[0], c.gas[1], c.gas[2],
                 c.alb, c.alb, c.alb, c.alb, c.cosz, nullptr, nullptr, nullptr};
  const LwIn lin{c.play, c.plev, c.tlay, c.tlev, c.tsfc, c.h2o, c.o3, c.co2, c.gas[0], c.gas[1], c.gas[2],
                 c.gas[3], c.gas[4], c.gas[5], c.gas[6], c.emis, nullptr};
  rc = fork_lw_sw(
      h, st, fk,
      [&](cudaStream_t ls) {
        return lw_enqueue(h, ls, lw_base, s.ncol, a.sk, 0, lin, w.uflx, w.dflx, w.hr, w.uflxc, w.dflxc, w.hrc,
                          nullptr, nullptr);
      },
      [&](cudaStream_t ss) {
        return sw_enqueue(h, ss, sw_base, s.ncol, a.sk, 0, p.solrad, dyofyr, p.solr_cnst, sin, w.swuflx, w.swdflx,
                          w.swhr, w.swuflxc, w.swdflxc, w.swhrc);
      });
  if (rc) return rc;
  const RunRad r{w.uflx, w.dflx, w.hr, w.swuflx, w.swdflx, w.swhr};
  if (s.zm_rad) {
    launch_run_zonal_rad(s, r, w.zt, w.zsw, w.zlw, st);
    h->launches += 1;
  }
  launch_run_post(s, r, w.zt, w.zsw, w.zlw, a.o, st);
  h->launches += 1;
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(h, e, "run_rrtmg: output kernels");
  return RRTMG_OK;
}

RunArgs run_args(int si, int sj, int sk, int seconds, int days, int days_per_year, const double* lat,
                 const double* lon, const double* p_full, const double* p_half, const double* z_full,
                 const double* z_half, const double* t, const double* q, const double* o3, const double* t_surf_rad,
                 const double* albedo, const double* rrtm_precip, double* tdt, double* coszen, double* flux_sw,
                 double* flux_lw, double* t_half, double* tdt_rad, double* tdt_sw, double* tdt_lw, double* olr,
                 double* isr) {
  RunArgs a;
  a.si = si;
  a.sj = sj;
  a.sk = sk;
  a.seconds = seconds;
  a.days = days;
  a.days_per_year = days_per_year;
  a.g = RunGcm{lat, lon, p_full, p_half, z_full, z_half, t, q, o3, t_surf_rad, albedo, rrtm_precip};
  a.o = RunOut{tdt, coszen, flux_sw, flux_lw, t_half, tdt_rad, tdt_sw, tdt_lw, olr, isr};
  return a;
}

}  // namespace

extern "C" {

int rrtmg_run_params_default(rrtmg_run_params* p) {
  if (!p) return RRTMG_ERR_ARG;
  std::memset(p, 0, sizeof(*p));
  p->lonstep = 1;
  p->dt_rad_avg = 86400;
  p->h2o_lower_limit = 2.e-7;
  p->temp_lower_limit = 100.;
  p->temp_upper_limit = 370.;
  p->co2ppmv = 300.;
  p->fixed_water = 2.e-06;
  p->fixed_water_pres = 100.e02;
  p->fixed_water_lat = 90.;
  p->precip_albedo = 0.35;
  p->slowdown_rad = 1.0;
  p->obliq = 23.439;
  p->solr_cnst = 1368.22;
  p->solrad = 1.0;
  p->equinox_day = 0.25;
  return RRTMG_OK;
}

int rrtmg_run_dev(rrtmg_gpu_handle h, void* stream, const rrtmg_run_params* prm, int si, int sj, int sk,
                  int seconds, int days, int days_per_year, const double* lat, const double* lon,
                  const double* p_full, const double* p_half, const double* z_full, const double* z_half,
                  const double* t, const double* q, const double* o3, const double* t_surf_rad,
                  const double* albedo, const double* rrtm_precip, double* tdt, double* coszen, double* flux_sw,
                  double* flux_lw, double* t_half, double* tdt_rad, double* tdt_sw, double* tdt_lw, double* olr,
                  double* isr) {
  const RunArgs a = run_args(si, sj, sk, seconds, days, days_per_year, lat, lon, p_full, p_half, z_full, z_half, t,
                             q, o3, t_surf_rad, albedo, rrtm_precip, tdt, coszen, flux_sw, flux_lw, t_half, tdt_rad,
                             tdt_sw, tdt_lw, olr, isr);
  int rc = run_check(h, prm, a);
  if (rc) return rc;
  cudaSetDevice(h->device);
  return run_enqueue(h, (cudaStream_t)stream, *prm, a, h->run_ws, default_fork(h), -1);
}

int rrtmg_run_c(rrtmg_gpu_handle h, const rrtmg_run_params* prm, int si, int sj, int sk, int seconds, int days,
                int days_per_year, const double* lat, const double* lon, const double* p_full,
                const double* p_half, const double* z_full, const double* z_half, const double* t, const double* q,
                const double* o3, const double* t_surf_rad, const double* albedo, const double* rrtm_precip,
                double* tdt, double* coszen, double* flux_sw, double* flux_lw, double* t_half, double* tdt_rad,
                double* tdt_sw, double* tdt_lw, double* olr, double* isr) {
  RunArgs a = run_args(si, sj, sk, seconds, days, days_per_year, lat, lon, p_full, p_half, z_full, z_half, t, q, o3,
                       t_surf_rad, albedo, rrtm_precip, tdt, coszen, flux_sw, flux_lw, t_half, tdt_rad, tdt_sw,
                       tdt_lw, olr, isr);
  int rc = run_check(h, prm, a);
  if (rc) return rc;
  cudaSetDevice(h->device);
  // Arrays are (level, latitude, longitude), longitude fastest: a block of
  // latitude rows is `planes` strided runs of si * rows values.  On
  // page-locked arrays the slab is processed in latitude chunks that alternate
  // between the handle's two streams (each with its own staging, workspace
  // and SW side stream), so that the copies of one chunk overlap the kernels
  // of the other; every step of run_rrtmg works within a latitude row except
  // the top-interface test, which the host makes for the whole slab.
  const size_t plane = (size_t)si * sj;
  const double** ins[] = {&a.g.lat, &a.g.lon, &a.g.p_full, &a.g.p_half, &a.g.z_full, &a.g.z_half, &a.g.t,
                          &a.g.q, &a.g.o3, &a.g.t_surf, &a.g.albedo, &a.g.precip};
  const int in_planes[] = {1, 1, sk, sk + 1, sk, sk + 1, sk, sk, sk, 1, 1, 1};
  double** outs[] = {&a.o.tdt, &a.o.coszen, &a.o.flux_sw, &a.o.flux_lw, &a.o.t_half, &a.o.tdt_rad,
                     &a.o.tdt_sw, &a.o.tdt_lw, &a.o.olr, &a.o.isr};
  const int out_planes[] = {sk, 1, 1, 1, sk + 1, sk, sk, sk, 1, 1};
  // whether some top interface of the RRTM columns is at 0 Pa
  // (rrtm_radiation.f90:655-656), over the whole slab, as the zonal kernel
  // finds it: p_half(i, j, 1) * 0.01 <= 0 at the columns kept by lonstep
  int top = 0;
  for (int j = 0; j < sj && !top; ++j)
    for (int i = 0; i < si; i += prm->lonstep)
      if (a.g.p_half[(size_t)si * j + i] * 0.01 <= 0.0) {
        top = 1;
        break;
      }
  bool all_pinned = true;
  for (int k = 0; k < 12 && all_pinned; ++k) all_pinned = pinned(*ins[k]);
  for (int k = 0; k < 10 && all_pinned; ++k) all_pinned = pinned(*outs[k]);
  const int ncol = si / prm->lonstep * sj;
  int nchunk = (all_pinned && ncol >= 2 * kChunkMin) ? std::min(kMaxChunks, ncol / kChunkMin) : 1;
  nchunk = std::min(nchunk, sj);
  const int rows = (sj + nchunk - 1) / nchunk;
  size_t stage = 0;
  for (int k = 0; k < 12; ++k)
    if (*ins[k]) stage += align256((size_t)si * rows * in_planes[k] * sizeof(double));
  for (int k = 0; k < 10; ++k)
    if (*outs[k]) stage += align256((size_t)si * rows * out_planes[k] * sizeof(double));
  for (int i = 0; i < 2 && i < nchunk; ++i) {
    rc = ensure(h, h->run_cio[i], stage, nullptr);
    if (rc) return rc;
  }
  cudaStream_t sts[2] = {h->stream, h->stream2};
  const Fork fks[2] = {default_fork(h), Fork{h->side2, h->fork_ev2, h->join_ev2}};
  auto drain = [h]() {
    cudaStreamSynchronize(h->stream);
    cudaStreamSynchronize(h->stream2);
  };
  cudaError_t e = cudaSuccess;
  for (int c = 0; c < nchunk; ++c) {
    const int j0 = c * rows, nr = std::min(rows, sj - j0);
    if (nr <= 0) break;
    cudaStream_t st = sts[c % 2];
    Carver cv{(char*)h->run_cio[c % 2].p};
    const size_t off = (size_t)si * j0, w = (size_t)si * nr * sizeof(double);
    RunArgs ac = a;
    ac.sj = nr;
    // copy of `planes` runs of w bytes between the slab and the chunk
    auto copy = [&](void* dst, size_t dpitch, const void* src, size_t spitch, int planes, cudaMemcpyKind kind) {
      return planes == 1 ? cudaMemcpyAsync(dst, src, w, kind, st)
                         : cudaMemcpy2DAsync(dst, dpitch, src, spitch, w, planes, kind, st);
    };
    const double** cin[] = {&ac.g.lat, &ac.g.lon, &ac.g.p_full, &ac.g.p_half, &ac.g.z_full, &ac.g.z_half,
                            &ac.g.t, &ac.g.q, &ac.g.o3, &ac.g.t_surf, &ac.g.albedo, &ac.g.precip};
    for (int k = 0; k < 12 && e == cudaSuccess; ++k) {
      if (!*ins[k]) continue;
      double* d = cv.take<double>((size_t)si * nr * in_planes[k]);
      e = copy(d, w, *ins[k] + off, plane * sizeof(double), in_planes[k], cudaMemcpyHostToDevice);
      *cin[k] = d;
    }
    double** cout[] = {&ac.o.tdt, &ac.o.coszen, &ac.o.flux_sw, &ac.o.flux_lw, &ac.o.t_half, &ac.o.tdt_rad,
                       &ac.o.tdt_sw, &ac.o.tdt_lw, &ac.o.olr, &ac.o.isr};
    for (int k = 0; k < 10 && e == cudaSuccess; ++k) {
      if (!*outs[k]) continue;
      double* d = cv.take<double>((size_t)si * nr * out_planes[k]);
      // tdt is read (the tendency before radiation) and written
      if (k == 0) e = copy(d, w, *outs[0] + off, plane * sizeof(double), out_planes[0], cudaMemcpyHostToDevice);
      *cout[k] = d;
    }
    // On a failure after copies were enqueued, wait for them before returning:
    // they read and write the caller's arrays.  The SW work of run_enqueue is
    // joined back into st, so the two streams cover it.
    if (e != cudaSuccess) {
      drain();
      return cuda_fail(h, e, "run_rrtmg: copy inputs");
    }
    rc = run_enqueue(h, st, *prm, ac, h->run_cws[c % 2], fks[c % 2], top);
    if (rc) {
      drain();
      return rc;
    }
    for (int k = 0; k < 10 && e == cudaSuccess; ++k)
      if (*outs[k])
        e = copy(*outs[k] + off, plane * sizeof(double), *cout[k], w, out_planes[k], cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
      drain();
      return cuda_fail(h, e, "run_rrtmg: copy outputs");
    }
  }
  e = cudaStreamSynchronize(h->stream2);
  if (e != cudaSuccess) return cuda_fail(h, e, "synchronise");
  return read_flags(h, h->stream);
}

}  // extern "C"
