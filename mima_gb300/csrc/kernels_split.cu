// FP32-split instantiation of the g-point solvers: gas optics, transmittance
// lookups and per-g recursions in FP32 (multiply-add contraction allowed);
// g-point sums to FP64 accuracy, band partials and the finalize kernels below
// in FP64.
#include "kernels.cuh"
#include "launch.h"

namespace rrtmg {

// LW band weight of the broadband sums per slot (sub-band): wtdiff *
// delwave(band) * fluxfac (rrtmg_lw_rtrnmr.f90:720-746), folded into one
// factor and split into two floats (w = hi + lo to 2^-48) for the compensated
// FP32 band sums.
__constant__ float2 c_lw_bandw[kLwSlots];

cudaError_t upload_constants_split(const LwConst& lw, const SwConst& sw) {
  cudaError_t e = cudaMemcpyToSymbol(c_lw, &lw, sizeof(LwConst));
  if (e != cudaSuccess) return e;
  const LwConstF f = make_lwconstf(lw);
  e = cudaMemcpyToSymbol(c_lwf, &f, sizeof(LwConstF));
  if (e != cudaSuccess) return e;
  float2 bw[kLwSlots];
  for (int k = 0; k < kLwSlots; ++k) {
    const double w = 0.5 * lw.band[lw_slot(k).band - 1].delwave * lw.fluxfac;
    bw[k].x = (float)w;
    bw[k].y = (float)(w - (double)bw[k].x);
  }
  e = cudaMemcpyToSymbol(c_lw_bandw, bw, sizeof(bw));
  if (e != cudaSuccess) return e;
  return cudaMemcpyToSymbol(c_sw, &sw, sizeof(SwConst));
}

// ---------------------------------------------------------------------------
// Finalize kernels of the split path.  The same fluxes and heating rates as
// the FP64 finalize kernels (rrtmg_lw_rtrnmr.f90:720-776; rrtmg_sw_rad
// .nomcica.f90:712-726 with MiMA's zero top layer), from the band partials
// (compensated FP32 pairs, s + c): the bands are summed by compensated FP32
// arithmetic (Knuth's TwoSum per addition, an FMA recovering each product's
// rounding error, the error terms gathered in a second float), within about
// 2^-44 of the exact sum of the partials, and only the broadband flux (the
// pair's value) and the heating-rate difference are formed in FP64.  A thread
// walks kLevChunk consecutive levels of one column, forming every level's
// band sums once and carrying the level below for the heating rate.  Measured
// at T85 x 40 (GB300): one level per thread, which re-forms the level below,
// LW 0.084 ms and SW 0.092 ms; two levels 0.244 / 0.141, four 0.225 / 0.129,
// eight 0.239 / 0.133 ms (identical outputs): the loads of one thread's levels
// issue one after the other, so the parallelism of a thread per level wins.
// ---------------------------------------------------------------------------
#ifndef RRTMG_FINALIZE_LEVELS
#define RRTMG_FINALIZE_LEVELS 1
#endif
constexpr int kLevChunk = RRTMG_FINALIZE_LEVELS;

// Compensated FP32 sum; explicitly rounded operations, so that contraction
// cannot merge the error terms.
struct CSum {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float x) {
    const float t = __fadd_rn(s, x), bv = __fsub_rn(t, s);
    c = __fadd_rn(c, __fadd_rn(__fsub_rn(s, __fsub_rn(t, bv)), __fsub_rn(x, bv)));
    s = t;
  }
  // a band partial (s + c)
  __device__ __forceinline__ void add(float2 p) {
    add(p.x);
    c = __fadd_rn(c, p.y);
  }
  // a band partial times a weight (w.x + w.y)
  __device__ __forceinline__ void add(float2 p, float2 w) {
    const float pr = __fmul_rn(p.x, w.x);
    c = __fadd_rn(c, __fmaf_rn(p.x, w.x, -pr));
    c = __fadd_rn(c, __fmaf_rn(p.x, w.y, __fmul_rn(p.y, w.x)));
    add(pr);
  }
  __device__ __forceinline__ double value() const { return (double)s + (double)c; }
};

// buc, bdc, bduc: the clear-sky band partials of a cloudy call, else null.
__global__ void __launch_bounds__(128) lw_finalize_split_kernel(const double* __restrict__ bu,
                                                                const double* __restrict__ bd,
                                                                const double* __restrict__ bdu,
                                                                const double* __restrict__ plev, int ncol, int nlay,
                                                                int idrv, double* uflx, double* dflx, double* hr,
                                                                double* uflxc, double* dflxc, double* hrc,
                                                                double* duflx_dt, double* duflxc_dt,
                                                                const double* __restrict__ buc,
                                                                const double* __restrict__ bdc,
                                                                const double* __restrict__ bduc) {
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= ncol) return;
  const int lev0 = blockIdx.y * kLevChunk, lev1 = min(nlay, lev0 + kLevChunk - 1);
  const size_t N = (size_t)ncol, bs = (size_t)(nlay + 1) * N;
  auto sums = [&](const double* a, const double* b, int lv, double& x, double& y) {
    CSum sx, sy;
    const size_t o = (size_t)lv * N + col;
#pragma unroll
    for (int k = 0; k < kLwSlots; ++k) {
      sx.add(__ldg(as_pair(a) + k * bs + o), c_lw_bandw[k]);
      sy.add(__ldg(as_pair(b) + k * bs + o), c_lw_bandw[k]);
    }
    x = sx.value();
    y = sy.value();
  };
  auto sum1 = [&](const double* a, int lv) {
    CSum sx;
    const size_t o = (size_t)lv * N + col;
#pragma unroll
    for (int k = 0; k < kLwSlots; ++k) sx.add(__ldg(as_pair(a) + k * bs + o), c_lw_bandw[k]);
    return sx.value();
  };
  const bool clear_own = buc != nullptr;
  double tu0 = 0.0, td0 = 0.0, tuc0 = 0.0, tdc0 = 0.0;
  if (lev0 >= 1) {
    sums(bu, bd, lev0 - 1, tu0, td0);
    if (clear_own) sums(buc, bdc, lev0 - 1, tuc0, tdc0);
  }
  for (int lev = lev0; lev <= lev1; ++lev) {
    double tu, td, tuc, tdc;
    sums(bu, bd, lev, tu, td);
    if (clear_own) sums(buc, bdc, lev, tuc, tdc);
    else tuc = tu, tdc = td;
    const size_t oo = (size_t)lev * N + col;
    uflx[oo] = tu;
    dflx[oo] = td;
    uflxc[oo] = tuc;
    dflxc[oo] = tdc;
    if (idrv == 1) {
      const double tdu = sum1(bdu, lev);
      if (duflx_dt) duflx_dt[oo] = tdu;
      if (duflxc_dt) duflxc_dt[oo] = clear_own ? sum1(bduc, lev) : tdu;
    }
    if (lev >= 1) {
      const double dp = __ldg(plev + oo - N) - __ldg(plev + oo);
      const double h = c_lw.heatfac * ((tu0 - td0) - (tu - td)) / dp;
      hr[oo - N] = h;
      hrc[oo - N] = clear_own ? c_lw.heatfac * ((tuc0 - tdc0) - (tuc - tdc)) / dp : h;
    }
    tu0 = tu;
    td0 = td;
    tuc0 = tuc;
    tdc0 = tdc;
  }
}

// suc, sdc: the clear-sky band partials of a cloudy call, else null.
__global__ void __launch_bounds__(128) sw_finalize_split_kernel(const double* __restrict__ su,
                                                                const double* __restrict__ sd,
                                                                const double* __restrict__ plev,
                                                                const double* __restrict__ coszen, int ncol, int nlay,
                                                                double* swuflx, double* swdflx, double* swhr,
                                                                double* swuflxc, double* swdflxc, double* swhrc,
                                                                const double* __restrict__ suc,
                                                                const double* __restrict__ sdc) {
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= ncol) return;
  const int lev0 = blockIdx.y * kLevChunk, lev1 = min(nlay, lev0 + kLevChunk - 1);
  const size_t N = (size_t)ncol, bs = (size_t)(nlay + 1) * N;
  const bool lit = __ldg(coszen + col) >= 1.e-10;
  auto sums = [&](const double* u, const double* d, int lv, double& fu, double& fd) {
    fu = 0.0;
    fd = 0.0;
    if (!lit) return;
    CSum su_, sd_;
    const size_t o = (size_t)lv * N + col;
#pragma unroll
    for (int k = 0; k < kSwSlots; ++k) {
      su_.add(__ldg(as_pair(u) + k * bs + o));
      sd_.add(__ldg(as_pair(d) + k * bs + o));
    }
    fu = su_.value();
    fd = sd_.value();
  };
  const bool clear_own = suc != nullptr;
  double fu0 = 0.0, fd0 = 0.0, fuc0 = 0.0, fdc0 = 0.0;
  if (lev0 >= 1) {
    sums(su, sd, lev0 - 1, fu0, fd0);
    if (clear_own) sums(suc, sdc, lev0 - 1, fuc0, fdc0);
  }
  for (int lev = lev0; lev <= lev1; ++lev) {
    double fu, fd, fuc, fdc;
    sums(su, sd, lev, fu, fd);
    if (clear_own) sums(suc, sdc, lev, fuc, fdc);
    else fuc = fu, fdc = fd;
    const size_t oo = (size_t)lev * N + col;
    swuflx[oo] = fu;
    swdflx[oo] = fd;
    swuflxc[oo] = fuc;
    swdflxc[oo] = fdc;
    if (lev >= 1) {
      double h = 0.0, hc = 0.0;
      if (lit && lev < nlay) {
        const double zdpgcp = c_sw.heatfac / (__ldg(plev + oo - N) - __ldg(plev + oo));
        h = ((fd - fu) - (fd0 - fu0)) * zdpgcp;
        hc = clear_own ? ((fdc - fuc) - (fdc0 - fuc0)) * zdpgcp : h;
      }
      swhr[oo - N] = h;
      swhrc[oo - N] = hc;
    }
    fu0 = fu;
    fd0 = fd;
    fuc0 = fuc;
    fdc0 = fdc;
  }
}

void launch_lw_finalize_split(const double* bu, const double* bd, const double* bdu, const double* plev, int ncol,
                              int nlay, int idrv, double* uflx, double* dflx, double* hr, double* uflxc,
                              double* dflxc, double* hrc, double* duflx_dt, double* duflxc_dt, cudaStream_t s,
                              const double* buc, const double* bdc, const double* bduc) {
  const dim3 g((ncol + 127) / 128, (nlay + 1 + kLevChunk - 1) / kLevChunk);
  lw_finalize_split_kernel<<<g, 128, 0, s>>>(bu, bd, bdu, plev, ncol, nlay, idrv, uflx, dflx, hr, uflxc, dflxc, hrc,
                                             duflx_dt, duflxc_dt, buc, bdc, bduc);
}

void launch_sw_finalize_split(const double* su, const double* sd, const double* plev, const double* coszen, int ncol,
                              int nlay, double* swuflx, double* swdflx, double* swhr, double* swuflxc,
                              double* swdflxc, double* swhrc, cudaStream_t s, const double* suc, const double* sdc) {
  const dim3 g((ncol + 127) / 128, (nlay + 1 + kLevChunk - 1) / kLevChunk);
  sw_finalize_split_kernel<<<g, 128, 0, s>>>(su, sd, plev, coszen, ncol, nlay, swuflx, swdflx, swhr, swuflxc, swdflxc,
                                             swhrc, suc, sdc);
}

// The split solvers are instantiated per (analytic, idrv / aerosol) flag pair.
template <int MAXL>
static void lw_split_flags(int fl, int nb, cudaStream_t s, const LwPrepT<float>& p, const double* emis,
                           const double* tauaer, const float* tab, const float2* exptfn, double* bu, double* bd,
                           double* bdu, int ncol, int nlay, int idrv, int analytic) {
  auto k = fl == 0 ? lw_gpoint_kernel<float, MAXL, 0>
         : fl == 1 ? lw_gpoint_kernel<float, MAXL, 1>
         : fl == 2 ? lw_gpoint_kernel<float, MAXL, 2>
                   : lw_gpoint_kernel<float, MAXL, 3>;
  k<<<nb, kBlock, 0, s>>>(p, emis, tauaer, tab, nullptr, nullptr, bu, bd, bdu, ncol, nlay, idrv, analytic, exptfn);
}

void launch_lw_gpoint_split(const LwPrepT<float>& p, const double* emis, const double* tauaer, const float* tab,
                            const float2* exptfn, double* bu, double* bd, double* bdu, int ncol, int nlay, int idrv,
                            int nb, int analytic, cudaStream_t s) {
  const int fl = (analytic ? 1 : 0) | (idrv == 1 ? 2 : 0);
  if (maxl_for(nlay) == 64)
    lw_split_flags<64>(fl, nb, s, p, emis, tauaer, tab, exptfn, bu, bd, bdu, ncol, nlay, idrv, analytic);
  else
    lw_split_flags<208>(fl, nb, s, p, emis, tauaer, tab, exptfn, bu, bd, bdu, ncol, nlay, idrv, analytic);
}

// Cloudy LW (icld = 1, 2, 3): instantiated per (analytic, idrv) flag pair;
// the overlap (ovl null: random) is chosen at run time.
template <int MAXL>
static void lw_split_cld_flags(int fl, int nb, cudaStream_t s, const LwPrepT<float>& p, const float* cld,
                               const double* taucld, const double* emis, const double* tauaer, const float* tab,
                               const float* exptbl, const float* tfntbl, const float* tautbl, double* bu, double* bd,
                               double* bdu, double* buc, double* bdc, double* bduc, int ncol, int nlay,
                               const float* ovl, bool scaled) {
  auto k = fl == 0 ? lw_gpoint_cld_kernel<float, MAXL, 0>
         : fl == 1 ? lw_gpoint_cld_kernel<float, MAXL, 1>
         : fl == 2 ? lw_gpoint_cld_kernel<float, MAXL, 2>
                   : lw_gpoint_cld_kernel<float, MAXL, 3>;
  k<<<nb, kBlock, 0, s>>>(p, cld, taucld, emis, tauaer, tab, exptbl, tfntbl, tautbl, bu, bd, bdu, buc, bdc, bduc, ncol,
                          nlay, 0, 0, ovl, scaled ? 1 : 0);
}

void launch_lw_gpoint_cld_split(const LwPrepT<float>& p, const float* cld, const double* taucld, const double* emis,
                                const double* tauaer, const float* tab, const float* exptbl, const float* tfntbl,
                                const float* tautbl, double* bu, double* bd, double* bdu, double* buc, double* bdc,
                                double* bduc, int ncol, int nlay, int idrv, int nb, int analytic, cudaStream_t s,
                                const float* ovl, bool scaled) {
  const int fl = (analytic ? 1 : 0) | (idrv == 1 ? 2 : 0);
  if (maxl_for(nlay) == 64)
    lw_split_cld_flags<64>(fl, nb, s, p, cld, taucld, emis, tauaer, tab, exptbl, tfntbl, tautbl, bu, bd, bdu, buc,
                           bdc, bduc, ncol, nlay, ovl, scaled);
  else
    lw_split_cld_flags<208>(fl, nb, s, p, cld, taucld, emis, tauaer, tab, exptbl, tfntbl, tautbl, bu, bd, bdu, buc,
                            bdc, bduc, ncol, nlay, ovl, scaled);
}

template <int MAXL, bool TOT>
static void sw_split_flags(int fl, int nb, cudaStream_t s, const SwPrepT<float>& p, const SwIn& in, double adjflux,
                           int iaer, const float* tab, const double* tab64, const float* exptbl, double* su,
                           double* sd, int ncol, int nlay, int analytic, const float* cld) {
  auto k = fl == 0 ? sw_gpoint_kernel<float, MAXL, 0, TOT>
         : fl == 1 ? sw_gpoint_kernel<float, MAXL, 1, TOT>
         : fl == 2 ? sw_gpoint_kernel<float, MAXL, 2, TOT>
                   : sw_gpoint_kernel<float, MAXL, 3, TOT>;
  k<<<nb, kBlock, 0, s>>>(p, in, adjflux, iaer, tab, tab64, exptbl, su, sd, ncol, nlay, analytic, cld);
}

void launch_sw_gpoint_split(const SwPrepT<float>& p, const SwIn& in, double adjflux, int iaer, const float* tab,
                            const double* tab64, const float* exptbl, double* su, double* sd, int ncol, int nlay,
                            int nb, int analytic, cudaStream_t s, const float* cld) {
  const int fl = (analytic ? 1 : 0) | (iaer == 10 ? 2 : 0);
  const bool big = maxl_for(nlay) != 64;
  if (cld) {
    if (!big) sw_split_flags<64, true>(fl, nb, s, p, in, adjflux, iaer, tab, tab64, exptbl, su, sd, ncol, nlay, analytic, cld);
    else sw_split_flags<208, true>(fl, nb, s, p, in, adjflux, iaer, tab, tab64, exptbl, su, sd, ncol, nlay, analytic, cld);
  } else {
    if (!big) sw_split_flags<64, false>(fl, nb, s, p, in, adjflux, iaer, tab, tab64, exptbl, su, sd, ncol, nlay, analytic, nullptr);
    else sw_split_flags<208, false>(fl, nb, s, p, in, adjflux, iaer, tab, tab64, exptbl, su, sd, ncol, nlay, analytic, nullptr);
  }
}

}  // namespace rrtmg
