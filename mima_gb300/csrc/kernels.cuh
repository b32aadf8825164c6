// RRTMG clear-sky LW/SW column-radiation kernels for sm_103a.
//
// Work decomposition (per radiation call, LW and SW alike):
//   1. prep    one thread per (column, layer): inatm + setcoef of the layer,
//              then one thread per column for the column sums, laytrop,
//              secdiff and the surface Planck terms (LW) or the solar-source
//              layers (SW).  FP64 on the FP64 path, FP32 on the split path.
//   2. gpoint  one thread per (column, g-point).  A warp holds the g-points
//              of a single band for several columns (lanes per column: the
//              next power of two >= the band's g count on the FP64 path, the
//              g count itself on the split path), so every warp runs one
//              band's straight-line gas-optics code and its table loads for
//              one column are contiguous.  Each thread evaluates taumol for
//              its g-point layer by layer and runs that g-point's vertical
//              recursions in registers/local memory; at every level the
//              g-point contributions of a column are summed (FP64 warp
//              shuffles on the FP64 path, shared-memory staging with
//              compensated FP32 sums on the split path) into FP64 band
//              partials.
//   3. finalize the band partials summed in band order (FP64), flux outputs,
//              heating-rate differencing (FP64).
// The column kernels (prep, FP64 finalize) are defined only in the
// translation unit that defines RRTMG_DEFINE_COLUMN_KERNELS.  Real = double
// gives the FP64 path; Real = float the FP32-split path.
#pragma once
#include <math.h>

#include "sw_optics.cuh"

namespace rrtmg {

// Constant memory: one copy per translation unit, filled by upload_constants().
static __constant__ LwConst c_lw;
static __constant__ SwConst c_sw;
static __constant__ LwConstF c_lwf;  // uploaded by the FP32-split unit only

// FP32 copies of the per-layer LW constants (host side, for the upload of
// c_lwf in every translation unit that runs FP32 gas optics).
inline LwConstF make_lwconstf(const LwConst& lw) {
  LwConstF f{};
  for (int k = 0; k < 7 * 60; ++k) f.chi[k] = (float)lw.chi[k];
  for (int j = 0; j < 61; ++j) {
    f.r_h2oco2[j] = (float)lw.r_h2oco2[j];
    f.r_h2oo3[j] = (float)lw.r_h2oo3[j];
    f.r_h2on2o[j] = (float)lw.r_h2on2o[j];
    f.r_h2och4[j] = (float)lw.r_h2och4[j];
    f.r_n2oco2[j] = (float)lw.r_n2oco2[j];
    f.r_o3co2[j] = (float)lw.r_o3co2[j];
  }
  for (int b = 0; b < kLwBands; ++b)
    for (int k = 0; k < 4; ++k) f.refrat[b][k] = (float)lw.refrat[b][k];
  f.oneminus = (float)lw.oneminus;
  return f;
}

// Per-layer LW constants in the solver's arithmetic type.
template <class R>
__device__ __forceinline__ const auto& lw_rconst() {
  if constexpr (sizeof(R) == 4)
    return c_lwf;
  else
    return c_lw;
}

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

template <int W>
__device__ __forceinline__ double seg_sum(double v) {
#pragma unroll
  for (int o = W / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ bool bad(double x) { return !isfinite(x); }

// g-point sums of the FP32-split solvers, to FP64 accuracy without FP64
// arithmetic per g-point.  Each lane of a warp holds one (column, g-point)
// value per level; NB value streams are staged in FP32 in shared memory for
// up to W levels, then every lane forms one (column, level) sum and hands it
// to the store as a double.  The sum runs in g order as a compensated FP32
// sum: Knuth's TwoSum splits every addition into the rounded sum and its exact
// rounding error, and with per-g weights `wt` (the SW incident fluxes, FP32)
// an FMA recovers the exact error of each product; the errors accumulate in a
// second float; the pair (s, c) is stored as is (a float2 band partial), its
// value s + c within about NG^2 u^2 (u = 2^-24) of the exact sum -- the
// accuracy of the FP64 sum it replaces, with no FP64 operation in the solver
// (GB300's FP64 rate is a small fraction of its FP32 rate; the finalize
// kernels add the pairs of all bands by the same compensated summation).  Explicitly rounded intrinsics keep
// the compiler from contracting the error terms.  Rows are 33 floats wide so
// that the staging stores and the per-lane row reads are free of bank
// conflicts.  A warp stages at most kStageRows rows: W levels of one stream
// or half as many of two, so that the buffers of a block take 8.4 KB of shared
// memory and a smaller shared-memory carve-out leaves L1 room for the solvers'
// per-thread arrays.  All lanes of the warp must call put/next/flush
// uniformly (the level loops are warp-uniform).
constexpr int kRow = 33;
#ifndef RRTMG_STAGE_ROWS
#define RRTMG_STAGE_ROWS 16
#endif
constexpr int kStageRows = RRTMG_STAGE_ROWS;
// The clear-sky LW solver stages 4 rows: more L1 for its per-thread arrays
// (measured at T85 x 40: LW 2.738 ms at 16 rows, 2.713 at 8; 2.752 at 8 and
// 2.731 at 4 on another GB300; the SW solver, 2.283 -> 2.344 ms at 8 rows,
// keeps 16).
#ifndef RRTMG_LW_STAGE_ROWS
#define RRTMG_LW_STAGE_ROWS 4
#endif
constexpr int kLwStageRows = RRTMG_LW_STAGE_ROWS;
template <int W, int NG, int NB, bool WEIGHTED, int ROWS = kStageRows>
struct GSum {
  float* buf;          // this warp's [kStageRows][kRow]
  const float* wt;     // this warp's [32] per-lane weights (WEIGHTED only)
  int lane, n, first, dir;
  int nb;              // streams in use (<= NB)
  // levels staged per flush
  __device__ __forceinline__ int cap() const { return W < ROWS / nb ? W : ROWS / nb; }
  // streams beyond nb are not staged (the LW solver offers its idrv stream always)
  __device__ __forceinline__ void put(int b, float v) {
    if (b < nb) buf[(b * cap() + n) * kRow + lane] = v;
  }
  template <class Store>
  __device__ __forceinline__ void flush(Store&& st) {
    __syncwarp();
    const int sl = lane % W, cs = lane / W;
    if (sl < n && cs < 32 / W) {
#pragma unroll
      for (int b = 0; b < NB; ++b) {
        if (b >= nb) break;
        const float* row = buf + (b * cap() + sl) * kRow + cs * W;
        float s = 0.f, c = 0.f;
#pragma unroll 2
        for (int g = 0; g < NG; ++g) {
          float x = row[g];
          if constexpr (WEIGHTED) {
            const float wf = wt[cs * W + g];
            const float pr = __fmul_rn(wf, x);
            c = __fadd_rn(c, __fmaf_rn(wf, x, -pr));
            x = pr;
          }
          const float t = __fadd_rn(s, x), bv = __fsub_rn(t, s);
          c = __fadd_rn(c, __fadd_rn(__fsub_rn(s, __fsub_rn(t, bv)), __fsub_rn(x, bv)));
          s = t;
        }
        st(b, first + dir * sl, cs, s, c);
      }
    }
    __syncwarp();
    first += dir * n;
    n = 0;
  }
  template <class Store>
  __device__ __forceinline__ void next(Store&& st) {
    if (++n == cap()) flush(st);
  }
};
// Lanes per column of a band with ng g-points: the next power of two on the
// FP64 path (whose warp-shuffle sums need power-of-two groups) and in the
// adjoint; on the split path ng itself where that fits more columns into a
// warp (ng = 6: 5 columns instead of 4; ng = 10: 3 instead of 2; the tail
// lanes of the warp idle), else the power of two.  Measured at 32768 columns:
// SW solver 4.55 -> 4.1 ms, LW 3.36 -> 3.35 ms (ng for every band: LW 3.44 ms).
__host__ __device__ constexpr int split_lanes(int ng, bool split) {
  return (split && 32 / ng > 32 / pow2ceil(ng)) ? ng : pow2ceil(ng);
}

// Sub-bands of the split path ("slots"): the bands of 12 g-points, whose
// warps would idle 4 of every 16 lanes, run as groups of 8 + 4 g-points, each
// group with its own lanes per column and its own band partial; every other
// band is one slot.  The finalize kernels sum the slots.  Measured at T85 x 40
// (GB300): SW solver 2.46 -> 2.28 ms; LW solver 2.99 -> 2.86 ms (finalize
// 0.08 -> 0.11 ms) with its 12-g-point bands split, and 2.90 -> 2.78 ms with
// its band of 14 g-points as 8 + 6 (a 6-lane group packs 5 columns in a
// warp); as 8 + 4 + 2 it took 3.43 ms (a 2-lane group spreads each table
// gather over 16 columns).  RRTMG_LW_SUBBANDS=0 builds the LW solver with one
// slot per band.
struct SubBand {
  int band, g0, ng;  // band (LW 1..16, SW 16..29), first g-point in the band, g-points
};
#if RRTMG_LW_SUBBANDS
__host__ __device__ constexpr SubBand lw_slot(int s) {
  constexpr SubBand t[kLwSlots] = {{1, 0, 10}, {2, 0, 8},  {2, 8, 4},  {3, 0, 16}, {4, 0, 8},  {4, 8, 6},  {5, 0, 16},
                                   {6, 0, 8},  {7, 0, 8},  {7, 8, 4},  {8, 0, 8},  {9, 0, 8},  {9, 8, 4},  {10, 0, 6},
                                   {11, 0, 8}, {12, 0, 8}, {13, 0, 4}, {14, 0, 2}, {15, 0, 2}, {16, 0, 2}};
  return t[s];
}
#else
__host__ __device__ constexpr SubBand lw_slot(int s) { return SubBand{s + 1, 0, lw_ng(s + 1)}; }
#endif
__host__ __device__ constexpr SubBand sw_slot(int s) {
  constexpr SubBand t[kSwSlots] = {{16, 0, 6}, {17, 0, 8}, {17, 8, 4}, {18, 0, 8}, {19, 0, 8}, {20, 0, 10},
                                   {21, 0, 10}, {22, 0, 2}, {23, 0, 10}, {24, 0, 8}, {25, 0, 6}, {26, 0, 6},
                                   {27, 0, 8}, {28, 0, 6}, {29, 0, 8}, {29, 8, 4}};
  return t[s];
}

// Shared-memory floats of the staging buffers of one 128-thread block.
constexpr int kGSumFloats = (kBlock / 32) * kStageRows * kRow;
constexpr int kLwGSumFloats = (kBlock / 32) * kLwStageRows * kRow;

// The split path's band partials: a double slot of the band-partial arrays
// holds one compensated pair (s, c) of the g-point sum (8 bytes either way).
__device__ __forceinline__ float2* as_pair(double* p) { return reinterpret_cast<float2*>(p); }
__device__ __forceinline__ const float2* as_pair(const double* p) { return reinterpret_cast<const float2*>(p); }

// Per-thread layer state that one sweep writes together and the other reads
// together, kept side by side so that each layer's store and load is one wide
// local-memory access instead of two or four.
template <class R>
struct __align__(2 * sizeof(R)) Pair2 {
  R a, b;
};
template <class R>
struct __align__(4 * sizeof(R)) Quad {
  R a, b, c, d;
};

#ifdef RRTMG_DEFINE_COLUMN_KERNELS
// ---------------------------------------------------------------------------
// LW prep: inatm (rrtmg_lw_rad.nomcica.f90:572-901) + setcoef
// (rrtmg_lw_setcoef.f90:31-415) + secdiff (rrtmg_lw_rtrnmr.f90:271-279), in two
// launches: one thread per (column, layer) for everything that depends on one
// layer, then one thread per column for the column sums (amttl, wvttl, in
// layer order as the reference accumulates them), laytrop, the surface and
// bottom-level Planck terms and secdiff.  Each value is the same expression as
// in the reference's layer loop.
// totplnk / totplnkderiv: device tables [(ind-1) + 181*(band-1)].
// ---------------------------------------------------------------------------
// F is both the storage and the arithmetic type: the FP64 path computes in
// double, the FP32-split path (whose prepared fields are FP32) in float, with
// the same expressions in the same order; the inputs are validated in double.
template <class F>
__global__ void __launch_bounds__(128) lw_prep_layer_kernel(LwIn in, LwWorkT<F> w, const F* __restrict__ totplnk,
                                                            int ncol, int nlay, unsigned* __restrict__ flags) {
  using T = F;
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= ncol) return;
  const int l = blockIdx.y + 1;
  const LwConst& C = c_lw;
  const T amd = (T)28.9660, amw = (T)18.0160, amdw = (T)1.607793, amdo = (T)0.603428;
  const T stpfac = (T)(296. / 1013.);
  const size_t N = (size_t)ncol;
  const size_t fstride = (size_t)nlay * N;
  auto A = [&](const double* p, int ll) { return __ldg(p + (size_t)col + N * (size_t)(ll - 1)); };
  auto P = [&](int ind, int b) { return __ldg(totplnk + (ind - 1) + 181 * (b - 1)); };
  (void)amw;
  unsigned flag = 0;
  {
    const double pv = A(in.play, l), tv = A(in.tlay, l), pz = A(in.plev, l + 1), tz = A(in.tlev, l + 1);
    const double q = A(in.h2o, l);
    if (bad(pv) || bad(tv) || bad(pz) || bad(tz) || bad(q) || pv <= 0. || tv <= 0. || q < 0. || q >= 1. || pz < 0.)
      flag = 1;
  }
  const T pz_prev = (T)A(in.plev, l);
  const T pavel = (T)A(in.play, l), tavel = (T)A(in.tlay, l);
  const T pz_l = (T)A(in.plev, l + 1), tz_l = (T)A(in.tlev, l + 1);
  const T h2o = (T)A(in.h2o, l);
  T wk1 = (h2o / ((T)1. - h2o)) * amdw;
  T wk2 = (T)A(in.co2, l);
  T wk3 = (T)A(in.o3, l) * amdo;
  T wk4 = in.n2o ? (T)A(in.n2o, l) : (T)0.0;
  T wk6 = in.ch4 ? (T)A(in.ch4, l) : (T)0.0;
  T wk7 = in.o2 ? (T)A(in.o2, l) : (T)0.0;
  T amm = ((T)1. - wk1) * amd + wk1 * amw;
  T coldry = (pz_prev - pz_l) * (T)1.e3 * (T)C.avogad / ((T)1.e2 * (T)C.grav * amm * ((T)1. + wk1));
  T summol = (T)0.0;
  summol = summol + wk2;
  summol = summol + wk3;
  summol = summol + wk4;
  summol = summol + (T)0.0;
  summol = summol + wk6;
  summol = summol + wk7;
  T wbrodl = coldry * ((T)1. - summol);
  wk1 = coldry * wk1;
  wk2 = coldry * wk2;
  wk3 = coldry * wk3;
  wk4 = coldry * wk4;
  T wk5 = coldry * (T)0.0;
  wk6 = coldry * wk6;
  wk7 = coldry * wk7;
  // column sums of inatm (amttl, wvttl), formed in layer order by the column kernel
  w.colsum[(size_t)(l - 1) * N + col] = coldry;
  w.colsum[fstride + (size_t)(l - 1) * N + col] = wk1;
  const T e20 = (T)1.e-20;
  T wx1 = in.ccl4 ? coldry * (T)A(in.ccl4, l) * e20 : coldry * (T)0.0 * e20;
  T wx2 = in.cfc11 ? coldry * (T)A(in.cfc11, l) * e20 : coldry * (T)0.0 * e20;
  T wx3 = in.cfc12 ? coldry * (T)A(in.cfc12, l) * e20 : coldry * (T)0.0 * e20;
  T wx4 = in.cfc22 ? coldry * (T)A(in.cfc22, l) * e20 : coldry * (T)0.0 * e20;

  // Planck functions of the layer and its upper interface
  const int indlay = clampi((int)(tavel - (T)159.), 1, 180);
  const T tlayfrac = tavel - (T)159. - (T)indlay;
  const int indlev = clampi((int)(tz_l - (T)159.), 1, 180);
  const T tlevfrac = tz_l - (T)159. - (T)indlev;
  for (int b = 1; b <= 16; ++b) {
    T dbdtlev = P(indlev + 1, b) - P(indlev, b);
    T dbdtlay = P(indlay + 1, b) - P(indlay, b);
    w.planklay[((size_t)(b - 1) * nlay + (l - 1)) * N + col] = P(indlay, b) + tlayfrac * dbdtlay;
    w.planklev[((size_t)(b - 1) * (nlay + 1) + l) * N + col] = P(indlev, b) + tlevfrac * dbdtlev;
  }

  const T plog = log(pavel);
  const int jp = clampi((int)((T)36. - (T)5 * (plog + (T)0.04)), 1, 58);
  const int jp1 = jp + 1;
  const T fp = (T)5. * ((T)C.preflog[jp - 1] - plog);
  const int jt = clampi((int)((T)3. + (tavel - (T)C.tref[jp - 1]) / (T)15.), 1, 4);
  const T ft = ((tavel - (T)C.tref[jp - 1]) / (T)15.) - (T)(jt - 3);
  const int jt1 = clampi((int)((T)3. + (tavel - (T)C.tref[jp1 - 1]) / (T)15.), 1, 4);
  const T ft1 = ((tavel - (T)C.tref[jp1 - 1]) / (T)15.) - (T)(jt1 - 3);
  const T water = wk1 / coldry;
  const T scalefac = pavel * stpfac / tavel;
  T forfac, forfrac, selffac, selffrac = (T)0.0, minorfrac, factor;
  int indfor, indself = 1, indminor;
  if (plog > (T)4.56) {
    forfac = scalefac / ((T)1. + water);
    factor = ((T)332.0 - tavel) / (T)36.0;
    indfor = min(2, max(1, (int)factor));
    forfrac = factor - (T)indfor;
    selffac = water * forfac;
    factor = (tavel - (T)188.0) / (T)7.2;
    indself = min(9, max(1, (int)factor - 7));
    selffrac = factor - (T)(indself + 7);
  } else {
    forfac = scalefac / ((T)1. + water);
    factor = (tavel - (T)188.0) / (T)36.0;
    indfor = 3;
    forfrac = factor - (T)1.0;
    selffac = water * forfac;
  }
  const T scaleminor = pavel / tavel;
  const T scaleminorn2 = (pavel / tavel) * (wbrodl / (coldry + wk1));
  factor = (tavel - (T)180.8) / (T)7.2;
  indminor = min(18, max(1, (int)factor));
  minorfrac = factor - (T)indminor;

  T colh2o = e20 * wk1, colco2 = e20 * wk2, colo3 = e20 * wk3, coln2o = e20 * wk4;
  T colco = e20 * wk5, colch4 = e20 * wk6, colo2 = e20 * wk7;
  const T e32 = (T)1.e-32;
  if (colco2 == (T)0.) colco2 = e32 * coldry;
  if (colo3 == (T)0.) colo3 = e32 * coldry;
  if (coln2o == (T)0.) coln2o = e32 * coldry;
  if (colco == (T)0.) colco = e32 * coldry;
  if (colch4 == (T)0.) colch4 = e32 * coldry;
  const T colbrd = e20 * wbrodl;
  const T compfp = (T)1. - fp;
  const size_t o = (size_t)(l - 1) * N + col;
  F* f = w.f;
  f[LF_PAVEL * fstride + o] = pavel;
  f[LF_COLDRY * fstride + o] = coldry;
  f[LF_COLH2O * fstride + o] = colh2o;
  f[LF_COLCO2 * fstride + o] = colco2;
  f[LF_COLO3 * fstride + o] = colo3;
  f[LF_COLN2O * fstride + o] = coln2o;
  f[LF_COLCO * fstride + o] = colco;
  f[LF_COLCH4 * fstride + o] = colch4;
  f[LF_COLO2 * fstride + o] = colo2;
  f[LF_COLBRD * fstride + o] = colbrd;
  f[LF_FAC10 * fstride + o] = compfp * ft;
  f[LF_FAC00 * fstride + o] = compfp * ((T)1. - ft);
  f[LF_FAC11 * fstride + o] = fp * ft1;
  f[LF_FAC01 * fstride + o] = fp * ((T)1. - ft1);
  f[LF_SELFFAC * fstride + o] = colh2o * selffac;
  f[LF_SELFFRAC * fstride + o] = selffrac;
  f[LF_FORFAC * fstride + o] = colh2o * forfac;
  f[LF_FORFRAC * fstride + o] = forfrac;
  f[LF_MINORFRAC * fstride + o] = minorfrac;
  f[LF_SCALEMINOR * fstride + o] = scaleminor;
  f[LF_SCALEMINORN2 * fstride + o] = scaleminorn2;
  f[LF_WX1 * fstride + o] = wx1;
  f[LF_WX2 * fstride + o] = wx2;
  f[LF_WX3 * fstride + o] = wx3;
  f[LF_WX4 * fstride + o] = wx4;
  w.idx[o] = pack_idx(jp, jt, jt1, indself, indfor, indminor);
  if (flag) atomicOr(flags, 1u);
}

template <class F>
__global__ void __launch_bounds__(128) lw_prep_column_kernel(LwIn in, LwWorkT<F> w, const F* __restrict__ totplnk,
                                                             const F* __restrict__ totplnkderiv, int ncol,
                                                             int nlay, int idrv, unsigned* __restrict__ flags) {
  using T = F;
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= ncol) return;
  const LwConst& C = c_lw;
  const T amd = (T)28.9660, amw = (T)18.0160;
  const size_t N = (size_t)ncol;
  const size_t fstride = (size_t)nlay * N;
  auto A = [&](const double* p, int l) { return __ldg(p + (size_t)col + N * (size_t)(l - 1)); };
  auto P = [&](int ind, int b) { return __ldg(totplnk + (ind - 1) + 181 * (b - 1)); };
  auto PD = [&](int ind, int b) { return __ldg(totplnkderiv + (ind - 1) + 181 * (b - 1)); };
  unsigned flag = 0;
  {
    const double tb = __ldg(in.tsfc + col), pz = A(in.plev, 1), tz = A(in.tlev, 1);
    if (bad(tb) || bad(pz) || bad(tz) || tb <= 0. || tz <= 0.) flag = 1;
  }
  const T tbound = (T)__ldg(in.tsfc + col);
  const T pz0 = (T)A(in.plev, 1);
  const T tz0 = (T)A(in.tlev, 1);
  const int indbound = clampi((int)(tbound - (T)159.), 1, 180);
  const T tbndfrac = tbound - (T)159. - (T)indbound;
  const int indlev0 = clampi((int)(tz0 - (T)159.), 1, 180);
  const T t0frac = tz0 - (T)159. - (T)indlev0;
  for (int b = 1; b <= 16; ++b) {
    T semiss = in.emis ? (T)__ldg(in.emis + col + N * (b - 1)) : (T)1.0;
    T dbdtlev = P(indbound + 1, b) - P(indbound, b);
    w.plankbnd[(b - 1) * N + col] = semiss * (P(indbound, b) + tbndfrac * dbdtlev);
    dbdtlev = P(indlev0 + 1, b) - P(indlev0, b);
    w.planklev[((size_t)(b - 1) * (nlay + 1)) * N + col] = P(indlev0, b) + t0frac * dbdtlev;
    if (idrv == 1) {
      dbdtlev = PD(indbound + 1, b) - PD(indbound, b);
      w.dplankbnd[(b - 1) * N + col] = semiss * (PD(indbound, b) + tbndfrac * dbdtlev);
    }
  }
  T amttl = (T)0.0, wvttl = (T)0.0;
  int laytrop = 0;
  for (int l = 1; l <= nlay; ++l) {
    const T coldry = (T)w.colsum[(size_t)(l - 1) * N + col];
    const T wk1 = (T)w.colsum[fstride + (size_t)(l - 1) * N + col];
    amttl = amttl + coldry + wk1;
    wvttl = wvttl + wk1;
    // the same test on the same value as the layer kernel's branch
    if (log((T)A(in.play, l)) > (T)4.56) laytrop = laytrop + 1;
  }
  w.laytrop[col] = laytrop;
  const T wvsh = (amw * wvttl) / (amd * amttl);
  const T pwvcm = wvsh * ((T)1.e3 * pz0) / ((T)1.e2 * (T)C.grav);
  const T a0[16] = {(T)1.66, (T)1.55, (T)1.58, (T)1.66, (T)1.54, (T)1.454, (T)1.89, (T)1.33,
                    (T)1.668, (T)1.66, (T)1.66, (T)1.66, (T)1.66, (T)1.66, (T)1.66, (T)1.66};
  const T a1[16] = {(T)0.00, (T)0.25, (T)0.22, (T)0.00, (T)0.13, (T)0.446, (T)-0.10, (T)0.40,
                    (T)-0.006, 0, 0, 0, 0, 0, 0, 0};
  const T a2[16] = {(T)0.00, (T)-12.0, (T)-11.7, (T)0.00, (T)-0.72, (T)-0.243, (T)0.19, (T)-0.062,
                    (T)0.414, 0, 0, 0, 0, 0, 0, 0};
  for (int b = 1; b <= 16; ++b) {
    T s;
    if (b == 1 || b == 4 || b >= 10) {
      s = (T)1.66;
    } else {
      s = a0[b - 1] + a1[b - 1] * exp(a2[b - 1] * pwvcm);
      if (s > (T)1.80) s = (T)1.80;
      if (s < (T)1.50) s = (T)1.50;
    }
    w.secdiff[(b - 1) * N + col] = s;
  }
  if (flag) atomicOr(flags, 1u);
}

#endif  // RRTMG_DEFINE_COLUMN_KERNELS

// ---------------------------------------------------------------------------
// LW g-point solver: taumol + rtrnmr clear-sky branch
// (rrtmg_lw_rtrnmr.f90:505-616 downward, :628-713 upward) for one g-point.
// ---------------------------------------------------------------------------
// Split path: the two table lookups of a layer are one gather of exptfn
// (exp_tbl and tfn_tbl interleaved); FP64 path: exptbl and tfntbl.
// G0, NS: the g-points [G0, G0 + NS) of the band that this call computes
// (a sub-band of the split path, else the whole band); SLOT: its band-partial
// index.
template <int B, class R, int MAXL, int G0 = 0, int NS = lw_ng(B), int SLOT = B - 1>
__device__ __forceinline__ void lw_band(const LwPrepT<R>& p, const double* __restrict__ emis,
                                        const double* __restrict__ tauaer, const R* __restrict__ tab,
                                        const R* __restrict__ exptbl, const R* __restrict__ tfntbl,
                                        double* __restrict__ bu, double* __restrict__ bd, double* __restrict__ bdu,
                                        int ncol, int nlay, int idrv, bool analytic, int blk, float* sbuf,
                                        const float2* __restrict__ exptfn) {
  const bool IDRV = idrv == 1;
  constexpr bool SPLIT = sizeof(R) == 4;
  constexpr int NG = NS;
  constexpr int W = split_lanes(NG, SPLIT);
  constexpr int CPW = 32 / W;
  constexpr int CPB = (kBlock / 32) * CPW;
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int lane_col = wib * CPW + lane / W, g = lane % W;
  const int col = blk * CPB + lane_col;
  const bool valid = lane < CPW * W && col < ncol;
  const bool active = valid && g < NG;
  const int c = valid ? col : (col < ncol ? col : ncol - 1);
  const int gg = G0 + (g < NG ? g : NG - 1);
  const size_t N = (size_t)ncol;
  const int lt = p.laytrop[c];
  const R secdiff = p.secdiff[(B - 1) * N + c];
  const R bpade = (R)c_lw.bpade;
  const R rec_6 = (R)0.166667;
  const size_t fstride = (size_t)nlay * N;
  Pair2<R> ab[MAXL];  // {atrans, bbugas} of each layer
  R radld = (R)0., fracs1 = (R)0.;
  double* bdp = bd + (size_t)SLOT * (nlay + 1) * N + col;
  double* bup = bu + (size_t)SLOT * (nlay + 1) * N + col;
  double* bdup = IDRV ? bdu + (size_t)SLOT * (nlay + 1) * N + col : nullptr;
  // Split path: band sums through the warp's staging buffers; the summing
  // lane of column sub-index cs writes column wcol0 + cs.
  const int wcol0 = blk * CPB + wib * CPW;
  GSum<W, NG, 2, false, kLwStageRows> gs{sbuf + (SPLIT ? wib * kLwStageRows * kRow : 0), nullptr, lane, 0,
                                          nlay - 1, -1,
                           1};
  auto store_dn = [&](int b, int lev, int cs, float s, float cmp) {
    const int cc = wcol0 + cs;
    if (cc < ncol) as_pair(bd)[((size_t)SLOT * (nlay + 1) + lev) * N + cc] = make_float2(s, cmp);
  };
  auto store_up = [&](int b, int lev, int cs, float s, float cmp) {
    const int cc = wcol0 + cs;
    if (cc >= ncol) return;
    if (b == 0)
      as_pair(bu)[((size_t)SLOT * (nlay + 1) + lev) * N + cc] = make_float2(s, cmp);
    else if (IDRV)
      as_pair(bdu)[((size_t)SLOT * (nlay + 1) + lev) * N + cc] = make_float2(s, cmp);
  };
  // No downward radiance enters at the top (drad(nlayers) stays 0,
  // rrtmg_lw_rtrnmr.f90:290-300).
  if (g == 0 && valid) bdp[(size_t)nlay * N] = 0.0;
  // the packed table indices of the next layer are loaded one layer ahead;
  // a level's Planck term is loaded once, as the lower level of the layer
  // above and the upper level of the layer below
  uint32_t idx_next = __ldg(p.idx + (size_t)(nlay - 1) * N + c);
  const R* plev_b = p.planklev + (size_t)(B - 1) * (nlay + 1) * N + c;
  R plev_up = __ldg(plev_b + (size_t)nlay * N);
  for (int lev = nlay; lev >= 1; --lev) {
    const size_t o = (size_t)(lev - 1) * N + c;
    const Idx ix = unpack_idx(idx_next);
    if (lev > 1) idx_next = __ldg(p.idx + o - N);
    LwLayerView<R> L{p.f, fstride, o};
    R taug, fracs;
    lw_gas<B, R>(c_lw, lw_rconst<R>(), L, ix, lev <= lt, gg, tab, taug, fracs);
    R taut = taug;
    if (tauaer) taut = taug + (R)__ldg(tauaer + c + N * ((size_t)(lev - 1) + (size_t)nlay * (B - 1)));
    const R plfrac = fracs;
    const R blay = __ldg(p.planklay + ((size_t)(B - 1) * nlay + (lev - 1)) * N + c);
    const R plev_dn = __ldg(plev_b + (size_t)(lev - 1) * N);
    const R dplankup = plev_up - blay;
    const R dplankdn = plev_dn - blay;
    plev_up = plev_dn;
    R odepth = secdiff * taut;
    if (odepth < (R)0.0) odepth = (R)0.0;
    R atr, bbd, bbu;
    if (odepth <= (R)0.06) {
      atr = odepth - (R)0.5 * odepth * odepth;
      odepth = rec_6 * odepth;
      bbd = plfrac * (blay + dplankdn * odepth);
      bbu = plfrac * (blay + dplankup * odepth);
    } else if (analytic) {
      // The functions the tables sample (rrtmg_lw_init.f90:115-122).
      const R transc = exp(-odepth);
      atr = (R)1. - transc;
      const R tausfac = (R)1. - (R)2. * (((R)1. / odepth) - (transc / ((R)1. - transc)));
      bbd = plfrac * (blay + tausfac * dplankdn);
      bbu = plfrac * (blay + tausfac * dplankup);
    } else {
      const R tblind = odepth / (bpade + odepth);
      int itr = (int)((R)10000.0 * tblind + (R)0.5);
      itr = itr < 0 ? 0 : (itr > kNTbl ? kNTbl : itr);  // in range for any odepth >= 0; guards NaN input
      R transc, tausfac;
      if constexpr (SPLIT) {
        const float2 et = __ldg(exptfn + itr);
        transc = et.x;
        tausfac = et.y;
      } else {
        transc = tld(exptbl + itr);
        tausfac = tld(tfntbl + itr);
      }
      atr = (R)1. - transc;
      bbd = plfrac * (blay + tausfac * dplankdn);
      bbu = plfrac * (blay + tausfac * dplankup);
    }
    ab[lev - 1] = Pair2<R>{atr, bbu};
    radld = radld + (bbd - radld) * atr;
    if constexpr (SPLIT) {
      gs.put(0, radld);
      gs.next(store_dn);
    } else {
      const double s = seg_sum<W>(active ? (double)radld : 0.0);
      if (g == 0 && valid) bdp[(size_t)(lev - 1) * N] = s;
    }
    if (lev == 1) fracs1 = fracs;
  }
  if constexpr (SPLIT) {
    if (gs.n) gs.flush(store_dn);
    gs.first = 0;
    gs.dir = 1;
    gs.nb = IDRV ? 2 : 1;
  }
  const R semiss = emis ? (R)__ldg(emis + c + N * (B - 1)) : (R)1.0;
  const R rad0 = fracs1 * __ldg(p.plankbnd + (B - 1) * N + c);
  const R reflect = (R)1. - semiss;
  R radlu = rad0 + reflect * radld;
  R dlu = (R)0.;
  if (IDRV) dlu = fracs1 * __ldg(p.dplankbnd + (B - 1) * N + c);
  if constexpr (SPLIT) {
    gs.put(0, radlu);
    gs.put(1, dlu);
    gs.next(store_up);
  } else {
    double s = seg_sum<W>(active ? (double)radlu : 0.0);
    if (g == 0 && valid) bup[0] = s;
    if (IDRV) {
      s = seg_sum<W>(active ? (double)dlu : 0.0);
      if (g == 0 && valid) bdup[0] = s;
    }
  }
  for (int lev = 1; lev <= nlay; ++lev) {
    const Pair2<R> l = ab[lev - 1];
    radlu = radlu + (l.b - radlu) * l.a;
    if (IDRV) dlu = dlu * ((R)1.0 - l.a);
    if constexpr (SPLIT) {
      gs.put(0, radlu);
      gs.put(1, dlu);
      gs.next(store_up);
    } else {
      double s = seg_sum<W>(active ? (double)radlu : 0.0);
      if (g == 0 && valid) bup[(size_t)lev * N] = s;
      if (IDRV) {
        s = seg_sum<W>(active ? (double)dlu : 0.0);
        if (g == 0 && valid) bdup[(size_t)lev * N] = s;
      }
    }
  }
  if constexpr (SPLIT) {
    if (gs.n) gs.flush(store_up);
  }
}

// ---------------------------------------------------------------------------
// LW g-point solver with clouds, random overlap (icld = 1, cloud optical
// depths given): rrtmg_lw_rtrn.f90:302-520 for one g-point.  A layer is
// cloudy when its cloud fraction is >= 1e-6 (cld[0] holds it, 0 otherwise);
// its cloud optical depth is secdiff * taucld where cldprop keeps taucld
// (cld[1] = 1, rrtmg_lw_cldprop.f90:167-174), else 0.  The clear-sky stream
// follows the total stream until the first cloudy layer from the top and is
// computed on its own above the surface once the column holds a cloud.
// Total and clear-sky level radiances are summed over the band's g-points
// into their own band partials.
// scaled (cloud physics): taucld holds lw_cldphys_kernel's depths, already
// along the diffusivity angle of their cloud band.
// With ovl (icld = 2, 3): maximum/random overlap, rrtmg_lw_rtrnmr.f90:
// 500-705.  Through a block of adjacent cloudy layers the radiance is carried
// as a cloudy and a clear part; at each cloudy layer's far boundary the
// overlap factors of lw_overlap_kernel move radiance between the two.
// ---------------------------------------------------------------------------
template <int B, class R, int MAXL, int G0 = 0, int NS = lw_ng(B), int SLOT = B - 1>
__device__ __forceinline__ void lw_band_cld(const LwPrepT<R>& p, const R* __restrict__ cld,
                                            const double* __restrict__ taucld, const double* __restrict__ emis,
                                            const double* __restrict__ tauaer, const R* __restrict__ tab,
                                            const R* __restrict__ exptbl, const R* __restrict__ tfntbl,
                                            const R* __restrict__ tautbl, double* __restrict__ bu,
                                            double* __restrict__ bd, double* __restrict__ bdu,
                                            double* __restrict__ buc, double* __restrict__ bdc,
                                            double* __restrict__ bduc, int ncol, int nlay, int idrv, bool analytic,
                                            int blk, float* sbuf, const R* __restrict__ ovl, bool scaled) {
  const bool IDRV = idrv == 1;
  constexpr bool SPLIT = sizeof(R) == 4;
  constexpr int NG = NS;
  constexpr int W = split_lanes(NG, SPLIT);
  constexpr int CPW = 32 / W;
  constexpr int CPB = (kBlock / 32) * CPW;
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int lane_col = wib * CPW + lane / W, g = lane % W;
  const int col = blk * CPB + lane_col;
  const bool valid = lane < CPW * W && col < ncol;
  const bool active = valid && g < NG;
  const int c = valid ? col : (col < ncol ? col : ncol - 1);
  const int gg = G0 + (g < NG ? g : NG - 1);
  const size_t N = (size_t)ncol;
  const int lt = p.laytrop[c];
  const R secdiff = p.secdiff[(B - 1) * N + c];
  const R seccld = scaled ? (R)1. : secdiff;
  const R bpade = (R)c_lw.bpade;
  const R rec_6 = (R)0.166667;
  const size_t fstride = (size_t)nlay * N;
  // {atrans, bbugas} of each layer and {atot, bbutot} of each cloudy one: a
  // clear layer moves half the bytes of a cloudy one through local memory
  Pair2<R> lq[MAXL], lqc[MAXL];
  R efcl[MAXL];
  // transmittance, tau transition function and the optical depth of a table
  // entry (exp_tbl, tfn_tbl, tau_tbl), or with the analytic functions, of od
  auto tbl = [&](R od, R& trans, R& tfn, R& odq) {
    if (analytic) {
      trans = exp(-od);
      tfn = (R)1. - (R)2. * (((R)1. / od) - (trans / ((R)1. - trans)));
      odq = od;
    } else {
      const R tblind = od / (bpade + od);
      int it = (int)((R)10000.0 * tblind + (R)0.5);
      it = it < 0 ? 0 : (it > kNTbl ? kNTbl : it);
      trans = tld(exptbl + it);
      tfn = tld(tfntbl + it);
      odq = tld(tautbl + it);
    }
  };
  const size_t bo = (size_t)SLOT * (nlay + 1) * N;
  // streams: downward 0 total, 1 clear; upward 0 total, 1 clear, 2 / 3 their
  // surface-temperature derivatives (idrv = 1)
  double* dst_dn[2] = {bd + bo, bdc + bo};
  double* dst_up[4] = {bu + bo, buc + bo, IDRV ? bdu + bo : nullptr, IDRV ? bduc + bo : nullptr};
  const int wcol0 = blk * CPB + wib * CPW;
  GSum<W, NG, 4, false> gs{sbuf + (SPLIT ? wib * kStageRows * kRow : 0), nullptr, lane, 0, nlay - 1, -1, 2};
  auto store_dn = [&](int b, int lev, int cs, float s, float cmp) {
    const int cc = wcol0 + cs;
    if (cc < ncol) as_pair(dst_dn[b])[(size_t)lev * N + cc] = make_float2(s, cmp);
  };
  auto store_up = [&](int b, int lev, int cs, float s, float cmp) {
    const int cc = wcol0 + cs;
    if (cc < ncol && dst_up[b]) as_pair(dst_up[b])[(size_t)lev * N + cc] = make_float2(s, cmp);
  };
  // FP64 path: the band's level sums by warp shuffles
  auto sum_dn = [&](int b, int lev, R v) {
    const double s = seg_sum<W>(active ? (double)v : 0.0);
    if (g == 0 && valid) dst_dn[b][(size_t)lev * N + col] = s;
  };
  auto sum_up = [&](int b, int lev, R v) {
    const double s = seg_sum<W>(active ? (double)v : 0.0);
    if (g == 0 && valid && dst_up[b]) dst_up[b][(size_t)lev * N + col] = s;
  };
  // no downward radiance enters at the top
  if (g == 0 && valid) {
    dst_dn[0][(size_t)nlay * N + col] = 0.0;
    dst_dn[1][(size_t)nlay * N + col] = 0.0;
  }
  R radld = (R)0., radclrd = (R)0., fracs1 = (R)0.;
  bool iclddn = false;
  // maximum/random overlap: the cloudy and clear parts and the radiance
  // moved between them; whether the layer above was cloudy (istcldd = 0)
  R cldrad = (R)0., clrrad = (R)0., rad = (R)0.;
  bool above_cloudy = false;
  const size_t ostride = (size_t)nlay * N;  // one overlap factor's stride
  uint32_t idx_next = __ldg(p.idx + (size_t)(nlay - 1) * N + c);
  for (int lev = nlay; lev >= 1; --lev) {
    const size_t o = (size_t)(lev - 1) * N + c;
    const Idx ix = unpack_idx(idx_next);
    if (lev > 1) idx_next = __ldg(p.idx + o - N);
    LwLayerView<R> L{p.f, fstride, o};
    R taug, fracs;
    lw_gas<B, R>(c_lw, lw_rconst<R>(), L, ix, lev <= lt, gg, tab, taug, fracs);
    R taut = taug;
    if (tauaer) taut = taug + (R)__ldg(tauaer + c + N * ((size_t)(lev - 1) + (size_t)nlay * (B - 1)));
    const R plfrac = fracs;
    const R blay = __ldg(p.planklay + ((size_t)(B - 1) * nlay + (lev - 1)) * N + c);
    const R dplankup = __ldg(p.planklev + ((size_t)(B - 1) * (nlay + 1) + lev) * N + c) - blay;
    const R dplankdn = __ldg(p.planklev + ((size_t)(B - 1) * (nlay + 1) + lev - 1) * N + c) - blay;
    R odepth = secdiff * taut;
    if (odepth < (R)0.0) odepth = (R)0.0;
    const R cf = __ldg(cld + o);
    R atr, bbd, bbu, at = (R)0., bbut = (R)0., ef = (R)0.;
    if (cf > (R)0.) {  // cloudy layer (rtrn :350-416)
      iclddn = true;
      const R odcld = seccld * (__ldg(cld + fstride + o) * (R)__ldg(taucld + (B - 1) + 16 * o));
      if (!ovl) ef = ((R)1. - exp(-odcld)) * cf;
      R odtot = odepth + odcld;
      R gassrc, bbdtot;
      if (odtot < (R)0.06) {
        atr = odepth - (R)0.5 * odepth * odepth;
        const R odepth_rec = rec_6 * odepth;
        gassrc = plfrac * (blay + dplankdn * odepth_rec) * atr;
        at = odtot - (R)0.5 * odtot * odtot;
        const R odtot_rec = rec_6 * odtot;
        bbdtot = plfrac * (blay + dplankdn * odtot_rec);
        bbd = plfrac * (blay + dplankdn * odepth_rec);
        bbu = plfrac * (blay + dplankup * odepth_rec);
        bbut = plfrac * (blay + dplankup * odtot_rec);
      } else if (odepth <= (R)0.06) {
        atr = odepth - (R)0.5 * odepth * odepth;
        const R odepth_rec = rec_6 * odepth;
        gassrc = plfrac * (blay + dplankdn * odepth_rec) * atr;
        R ttot, tfactot, odq;
        tbl(odtot, ttot, tfactot, odq);
        bbdtot = plfrac * (blay + tfactot * dplankdn);
        bbd = plfrac * (blay + dplankdn * odepth_rec);
        at = (R)1. - ttot;
        bbu = plfrac * (blay + dplankup * odepth_rec);
        bbut = plfrac * (blay + tfactot * dplankup);
      } else {
        R tgas, tfacgas, odq;
        tbl(odepth, tgas, tfacgas, odq);
        odepth = odq;  // tau_tbl(itgas)
        atr = (R)1. - tgas;
        gassrc = atr * plfrac * (blay + tfacgas * dplankdn);
        odtot = odepth + odcld;
        R ttot, tfactot, odq2;
        tbl(odtot, ttot, tfactot, odq2);
        bbdtot = plfrac * (blay + tfactot * dplankdn);
        bbd = plfrac * (blay + tfacgas * dplankdn);
        at = (R)1. - ttot;
        bbu = plfrac * (blay + tfacgas * dplankup);
        bbut = plfrac * (blay + tfactot * dplankup);
      }
      if (ovl) {  // rtrnmr :561-588
        if (!above_cloudy) {
          cldrad = cf * radld;
          clrrad = radld - cldrad;
          rad = (R)0.;
        }
        const R ttot = (R)1. - at;
        const R cldsrc = bbdtot * at;
        cldrad = cldrad * ttot + cf * cldsrc;
        clrrad = clrrad * ((R)1. - atr) + ((R)1. - cf) * gassrc;
        radld = cldrad + clrrad;
        const R* od = ovl + 6 * ostride + o;  // facclr1d, faccld1d, faccmb1d, faccmb2d, facclr2d, faccld2d
        const R radmod = rad * (__ldg(od) * ((R)1. - atr) + __ldg(od + ostride) * ttot) -
                         __ldg(od + 2 * ostride) * gassrc + __ldg(od + 3 * ostride) * cldsrc;
        const R oldcld = cldrad - radmod;
        const R oldclr = clrrad + radmod;
        rad = -radmod + __ldg(od + 4 * ostride) * oldclr - __ldg(od + 5 * ostride) * oldcld;
        cldrad = cldrad + rad;
        clrrad = clrrad - rad;
      } else {
        radld = radld - radld * (atr + ef * ((R)1. - atr)) + gassrc + cf * (bbdtot * at - gassrc);
      }
    } else {  // clear layer (rtrn :418-436)
      if (odepth <= (R)0.06) {
        atr = odepth - (R)0.5 * odepth * odepth;
        odepth = rec_6 * odepth;
        bbd = plfrac * (blay + dplankdn * odepth);
        bbu = plfrac * (blay + dplankup * odepth);
      } else {
        R transc, tausfac, odq;
        tbl(odepth, transc, tausfac, odq);
        atr = (R)1. - transc;
        bbd = plfrac * (blay + tausfac * dplankdn);
        bbu = plfrac * (blay + tausfac * dplankup);
      }
      radld = radld + (bbd - radld) * atr;
    }
    above_cloudy = cf > (R)0.;
    lq[lev - 1] = Pair2<R>{atr, bbu};
    if (cf > (R)0.) lqc[lev - 1] = Pair2<R>{at, bbut};
    if (!ovl) efcl[lev - 1] = ef;  // read by random overlap only
    // clear-sky stream (:441-448)
    if (iclddn)
      radclrd = radclrd + (bbd - radclrd) * atr;
    else
      radclrd = radld;
    if constexpr (SPLIT) {
      gs.put(0, radld);
      gs.put(1, radclrd);
      gs.next(store_dn);
    } else {
      sum_dn(0, lev - 1, radld);
      sum_dn(1, lev - 1, radclrd);
    }
    if (lev == 1) fracs1 = fracs;
  }
  if constexpr (SPLIT) {
    if (gs.n) gs.flush(store_dn);
    gs.first = 0;
    gs.dir = 1;
    gs.nb = IDRV ? 4 : 2;
  }
  const R semiss = emis ? (R)__ldg(emis + c + N * (B - 1)) : (R)1.0;
  const R rad0 = fracs1 * __ldg(p.plankbnd + (B - 1) * N + c);
  const R reflect = (R)1. - semiss;
  R radlu = rad0 + reflect * radld;
  R radclru = rad0 + reflect * radclrd;
  R dlu = (R)0., dluc = (R)0.;
  if (IDRV) {
    dlu = fracs1 * __ldg(p.dplankbnd + (B - 1) * N + c);
    dluc = dlu;
  }
  auto emit = [&](int lev) {
    if constexpr (SPLIT) {
      gs.put(0, radlu);
      gs.put(1, radclru);
      gs.put(2, dlu);
      gs.put(3, dluc);
      gs.next(store_up);
    } else {
      sum_up(0, lev, radlu);
      sum_up(1, lev, radclru);
      if (IDRV) {
        sum_up(2, lev, dlu);
        sum_up(3, lev, dluc);
      }
    }
  };
  emit(0);
  bool below_cloudy = false;  // maximum/random overlap: istcld = 0
  rad = (R)0.;
  for (int lev = 1; lev <= nlay; ++lev) {  // rtrn :478-520, rtrnmr :649-705
    const Pair2<R> l = lq[lev - 1];
    const R atr = l.a, bbugas = l.b;
    const size_t o = (size_t)(lev - 1) * N + c;
    const R cf = __ldg(cld + o);
    if (cf > (R)0.) {
      const R gassrc = bbugas * atr;
      const Pair2<R> lc = lqc[lev - 1];
      const R at = lc.a, bbutot = lc.b;
      if (ovl) {
        if (!below_cloudy) {
          cldrad = cf * radlu;
          clrrad = radlu - cldrad;
          rad = (R)0.;
        }
        const R ttot = (R)1. - at;
        const R cldsrc = bbutot * at;
        cldrad = cldrad * ttot + cf * cldsrc;
        clrrad = clrrad * ((R)1.0 - atr) + ((R)1. - cf) * gassrc;
        radlu = cldrad + clrrad;
        const R* ou = ovl + o;  // facclr1, faccld1, faccmb1, faccmb2, facclr2, faccld2 (index lev + 1)
        const R radmod = rad * (__ldg(ou) * ((R)1.0 - atr) + __ldg(ou + ostride) * ttot) -
                         __ldg(ou + 2 * ostride) * gassrc + __ldg(ou + 3 * ostride) * cldsrc;
        const R oldcld = cldrad - radmod;
        const R oldclr = clrrad + radmod;
        rad = -radmod + __ldg(ou + 4 * ostride) * oldclr - __ldg(ou + 5 * ostride) * oldcld;
        cldrad = cldrad + rad;
        clrrad = clrrad - rad;
      } else {
        radlu = radlu - radlu * (atr + efcl[lev - 1] * ((R)1. - atr)) + gassrc + cf * (bbutot * at - gassrc);
      }
      if (IDRV) dlu = dlu * cf * ((R)1.0 - at) + dlu * ((R)1.0 - cf) * ((R)1.0 - atr);
    } else {
      radlu = radlu + (bbugas - radlu) * atr;
      if (IDRV) dlu = dlu * ((R)1.0 - atr);
    }
    below_cloudy = cf > (R)0.;
    if (iclddn) {
      radclru = radclru + (bbugas - radclru) * atr;
      if (IDRV) dluc = dluc * ((R)1.0 - atr);
    } else {
      radclru = radlu;
      dluc = dlu;
    }
    emit(lev);
  }
  if constexpr (SPLIT) {
    if (gs.n) gs.flush(store_up);
  }
}

// Blocks of a band for `lanes` lanes per column: 32 / lanes columns per warp.
__host__ __device__ inline int lw_blocks_for_band(int lanes, int ncol) {
  const int cpb = (kBlock / 32) * (32 / lanes);
  return (ncol + cpb - 1) / cpb;
}

// The g-point grids enumerate their units -- the slots on the split path, the
// bands on the FP64 path -- then the column blocks of each: the unit of grid
// block blk, blk becoming the block's index within the unit (a past-the-end
// unit for blocks beyond the grid's work).
template <bool SPLIT>
__device__ __forceinline__ int lw_unit_of_block(int& blk, int ncol) {
  int u = 0;
  for (; u < (SPLIT ? kLwSlots : kLwBands); ++u) {
    const int nb = lw_blocks_for_band(SPLIT ? split_lanes(lw_slot(u).ng, true) : split_lanes(c_lw.band[u].ng, false),
                                      ncol);
    if (blk < nb) break;
    blk -= nb;
  }
  return u;
}
template <bool SPLIT>
__device__ __forceinline__ int sw_unit_of_block(int& blk, int ncol) {
  int u = 0;
  for (; u < (SPLIT ? kSwSlots : kSwBands); ++u) {
    const int nb = lw_blocks_for_band(SPLIT ? split_lanes(sw_slot(u).ng, true) : split_lanes(c_sw.band[u].ng, false),
                                      ncol);
    if (blk < nb) break;
    blk -= nb;
  }
  return u;
}

// Minimum resident blocks per SM asked of the register allocator for the
// FP32-split solvers.  They are latency-bound (table gathers, local-memory
// column arrays), so occupancy pays even at the price of spills: on GB300 at
// 32768 columns x 40 layers, 12/12 (40 registers) first ran the LW+SW split
// step in 11.1 ms against 19.0 ms at 1/1 (105 registers).  Re-measured with
// the flag-specialised solvers: LW 3.11 ms at 12, 3.27 at 10; SW 3.65 ms at
// 12, 3.58 at 14 (32 registers); with the SW layer state in packed records:
// SW 2.46 ms at 12 (40 registers), 2.51 at 14 and 16, 2.55 at 10; with the LW
// layer state packed and the exp / tfn gather merged: LW 3.17 ms at 12 and 11,
// 3.29 at 10, 2.99-3.04 at 13, 14 and 16.  FP64 solvers: 1.
#ifndef RRTMG_SPLIT_LW_MINB
#define RRTMG_SPLIT_LW_MINB 13
#endif
#ifndef RRTMG_SPLIT_SW_MINB
#define RRTMG_SPLIT_SW_MINB 12
#endif

// FL < 0: analytic and idrv as passed; FL >= 0: compile-time flags (bit 0
// analytic, bit 1 idrv = 1), so that the code of the unused branches folds
// away (the split path instantiates all four).
template <class R, int MAXL, int FL = -1>
__global__ void __launch_bounds__(kBlock, sizeof(R) == 4 ? RRTMG_SPLIT_LW_MINB : 1) lw_gpoint_kernel(LwPrepT<R> p, const double* __restrict__ emis,
                                                           const double* __restrict__ tauaer,
                                                           const R* __restrict__ tab, const R* __restrict__ exptbl,
                                                           const R* __restrict__ tfntbl, double* bu, double* bd,
                                                           double* bdu, int ncol, int nlay, int idrv,
                                                           int analytic, const float2* __restrict__ exptfn = nullptr) {
  __shared__ float sbuf[sizeof(R) == 4 ? kLwGSumFloats : 1];
  constexpr bool SPLIT = sizeof(R) == 4;
  int blk = blockIdx.x;
  const int unit = lw_unit_of_block<SPLIT>(blk, ncol);  // slot (split) or band (FP64)
  const int band = SPLIT ? (unit < kLwSlots ? lw_slot(unit).band - 1 : kLwBands) : unit;
  if (threadIdx.x == 0 && band < kLwBands) prefetch_band_l2(tab, c_lw.band[band]);
  const bool an = FL < 0 ? analytic != 0 : (FL & 1) != 0;
  const int idv = FL < 0 ? idrv : ((FL & 2) ? 1 : 0);
  if constexpr (SPLIT) {
#define RRTMG_LW_SLOT(s)                                                                                           \
  case s:                                                                                                          \
    lw_band<lw_slot(s).band, R, MAXL, lw_slot(s).g0, lw_slot(s).ng, s>(p, emis, tauaer, tab, exptbl, tfntbl, bu, bd, \
                                                                       bdu, ncol, nlay, idv, an, blk, sbuf, exptfn); \
    break;
    switch (unit) {
      RRTMG_LW_SLOT(0) RRTMG_LW_SLOT(1) RRTMG_LW_SLOT(2) RRTMG_LW_SLOT(3) RRTMG_LW_SLOT(4) RRTMG_LW_SLOT(5)
      RRTMG_LW_SLOT(6) RRTMG_LW_SLOT(7) RRTMG_LW_SLOT(8) RRTMG_LW_SLOT(9) RRTMG_LW_SLOT(10) RRTMG_LW_SLOT(11)
      RRTMG_LW_SLOT(12) RRTMG_LW_SLOT(13) RRTMG_LW_SLOT(14) RRTMG_LW_SLOT(15)
#if RRTMG_LW_SUBBANDS
      RRTMG_LW_SLOT(16) RRTMG_LW_SLOT(17) RRTMG_LW_SLOT(18) RRTMG_LW_SLOT(19)
#endif
      default: break;
    }
#undef RRTMG_LW_SLOT
  } else {
#define RRTMG_LW_CASE(b) \
  case b - 1: lw_band<b, R, MAXL>(p, emis, tauaer, tab, exptbl, tfntbl, bu, bd, bdu, ncol, nlay, idv, an, blk, sbuf, exptfn); break;
    switch (unit) {
      RRTMG_LW_CASE(1) RRTMG_LW_CASE(2) RRTMG_LW_CASE(3) RRTMG_LW_CASE(4) RRTMG_LW_CASE(5) RRTMG_LW_CASE(6)
      RRTMG_LW_CASE(7) RRTMG_LW_CASE(8) RRTMG_LW_CASE(9) RRTMG_LW_CASE(10) RRTMG_LW_CASE(11) RRTMG_LW_CASE(12)
      RRTMG_LW_CASE(13) RRTMG_LW_CASE(14) RRTMG_LW_CASE(15) RRTMG_LW_CASE(16)
      default: break;
    }
#undef RRTMG_LW_CASE
  }
}

// Cloudy LW g-point kernel (icld = 1, 2, 3): as lw_gpoint_kernel, with
// lw_band_cld (ovl null: random overlap, else maximum/random).  FL < 0:
// analytic and idrv as passed (FP64 path); FL >= 0: compile-time flags (bit
// 0 analytic, bit 1 idrv; split path).
template <class R, int MAXL, int FL>
__global__ void __launch_bounds__(kBlock, sizeof(R) == 4 ? RRTMG_SPLIT_LW_MINB : 1)
    lw_gpoint_cld_kernel(LwPrepT<R> p, const R* __restrict__ cld, const double* __restrict__ taucld,
                         const double* __restrict__ emis, const double* __restrict__ tauaer,
                         const R* __restrict__ tab, const R* __restrict__ exptbl, const R* __restrict__ tfntbl,
                         const R* __restrict__ tautbl, double* bu, double* bd, double* bdu, double* buc, double* bdc,
                         double* bduc, int ncol, int nlay, int idrv, int analytic, const R* __restrict__ ovl,
                         int scaled) {
  __shared__ float sbuf[sizeof(R) == 4 ? kGSumFloats : 1];
  constexpr bool SPLIT = sizeof(R) == 4;
  int blk = blockIdx.x;
  const int unit = lw_unit_of_block<SPLIT>(blk, ncol);  // slot (split) or band (FP64)
  const int band = SPLIT ? (unit < kLwSlots ? lw_slot(unit).band - 1 : kLwBands) : unit;
  if (threadIdx.x == 0 && band < kLwBands) prefetch_band_l2(tab, c_lw.band[band]);
  const bool an = FL < 0 ? analytic != 0 : (FL & 1) != 0;
  const int idv = FL < 0 ? idrv : ((FL & 2) ? 1 : 0);
  if constexpr (SPLIT) {
#define RRTMG_LW_SLOT(s)                                                                                          \
  case s:                                                                                                         \
    lw_band_cld<lw_slot(s).band, R, MAXL, lw_slot(s).g0, lw_slot(s).ng, s>(                                      \
        p, cld, taucld, emis, tauaer, tab, exptbl, tfntbl, tautbl, bu, bd, bdu, buc, bdc, bduc, ncol, nlay, idv, an, \
        blk, sbuf, ovl, scaled != 0);                                                                             \
    break;
    switch (unit) {
      RRTMG_LW_SLOT(0) RRTMG_LW_SLOT(1) RRTMG_LW_SLOT(2) RRTMG_LW_SLOT(3) RRTMG_LW_SLOT(4) RRTMG_LW_SLOT(5)
      RRTMG_LW_SLOT(6) RRTMG_LW_SLOT(7) RRTMG_LW_SLOT(8) RRTMG_LW_SLOT(9) RRTMG_LW_SLOT(10) RRTMG_LW_SLOT(11)
      RRTMG_LW_SLOT(12) RRTMG_LW_SLOT(13) RRTMG_LW_SLOT(14) RRTMG_LW_SLOT(15)
#if RRTMG_LW_SUBBANDS
      RRTMG_LW_SLOT(16) RRTMG_LW_SLOT(17) RRTMG_LW_SLOT(18) RRTMG_LW_SLOT(19)
#endif
      default: break;
    }
#undef RRTMG_LW_SLOT
  } else {
#define RRTMG_LW_CASE(b)                                                                                            \
  case b - 1:                                                                                                      \
    lw_band_cld<b, R, MAXL>(p, cld, taucld, emis, tauaer, tab, exptbl, tfntbl, tautbl, bu, bd, bdu, buc, bdc, bduc, \
                            ncol, nlay, idv, an, blk, sbuf, ovl, scaled != 0);                                     \
    break;
    switch (unit) {
      RRTMG_LW_CASE(1) RRTMG_LW_CASE(2) RRTMG_LW_CASE(3) RRTMG_LW_CASE(4) RRTMG_LW_CASE(5) RRTMG_LW_CASE(6)
      RRTMG_LW_CASE(7) RRTMG_LW_CASE(8) RRTMG_LW_CASE(9) RRTMG_LW_CASE(10) RRTMG_LW_CASE(11) RRTMG_LW_CASE(12)
      RRTMG_LW_CASE(13) RRTMG_LW_CASE(14) RRTMG_LW_CASE(15) RRTMG_LW_CASE(16)
      default: break;
    }
#undef RRTMG_LW_CASE
  }
}

#ifdef RRTMG_DEFINE_COLUMN_KERNELS
// ---------------------------------------------------------------------------
// Clouds of the LW call (icld = 1, cloud optical depths given), one thread per
// (column, layer): inatm's cldfrac / tauc (rrtmg_lw_rad.nomcica.f90:866-888),
// rtrn's cloudy-layer test cldfrac >= 1e-6 (rrtmg_lw_rtrn.f90:302-315) and
// cldprop's rule for keeping the optical depths, cldfrac >= cldmin and
// (ciwp + clwp >= cldmin or the band-summed depth >= cldmin), cldmin = 1e-20
// (rrtmg_lw_cldprop.f90:155-174).  cld[0][lay][col]: the cloud fraction of a
// cloudy layer, else 0; cld[1][lay][col]: 1 where the depths are kept, else 0.
// ---------------------------------------------------------------------------
template <class F>
__global__ void __launch_bounds__(128) lw_cloud_kernel(LwIn in, F* __restrict__ cld, int ncol, int nlay) {
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= ncol) return;
  const size_t o = (size_t)blockIdx.y * ncol + col;
  const double cf = __ldg(in.cldfr + o);
  double tauctot = 0.0;
  for (int ib = 0; ib < kLwBands; ++ib) tauctot = tauctot + __ldg(in.taucld + ib + 16 * o);
  const double cwp = (in.cicewp ? __ldg(in.cicewp + o) : 0.0) + (in.cliqwp ? __ldg(in.cliqwp + o) : 0.0);
  const double cldmin = 1.e-20;
  const bool kept = cf >= cldmin && (cwp >= cldmin || tauctot >= cldmin);
  cld[o] = cf >= 1.e-6 ? (F)cf : (F)0;
  cld[(size_t)nlay * ncol + o] = kept ? (F)1 : (F)0;
}

// ---------------------------------------------------------------------------
// LW cloud physics (cldprop with inflag = 1 or 2, rrtmg_lw_cldprop.f90:
// 155-270, and rtrn / rtrnmr's cloud depths along the diffusivity angle,
// rrtmg_lw_rtrn.f90:302-330).
//
// cldprop keeps a count of cloud bands, ncbands, across its layer loop
// (bottom to top): 1 at the start, 16 after a layer with given depths or
// inflag = 1, after an iceflag 2 / 3 ice cloud or a liqflag = 1 liquid cloud,
// 5 after an iceflag = 1 ice cloud; a layer fills cloud bands 1..ncbands as
// the count stands after it.  The radiative transfer then takes band iband's
// cloud depth from cloud band ipat(iband, final count) -- so an ice-only
// iceflag = 1 layer at the top of a column leaves every layer of that column
// with 5 cloud bands.
// ---------------------------------------------------------------------------
// Cloud band of band iband (1..16) with ncb cloud bands (ipat, icb).
__device__ __forceinline__ int lw_cloud_band(int iband, int ncb) {
  if (ncb == 1) return 1;
  if (ncb == 5) return iband <= 2 ? iband : iband <= 5 ? 3 : iband <= 8 ? 4 : 5;
  return iband;
}
// Whether a layer's optics are formed: cover >= cldmin and water path or
// band-summed given depth >= cldmin (cldmin = 1e-20).
__device__ __forceinline__ bool lw_cloud_kept(const LwIn& in, size_t o, double& cf, double& ciwp, double& clwp) {
  cf = __ldg(in.cldfr + o);
  ciwp = in.cicewp ? __ldg(in.cicewp + o) : 0.0;
  clwp = in.cliqwp ? __ldg(in.cliqwp + o) : 0.0;
  double tauctot = 0.0;
  if (in.taucld)
    for (int ib = 0; ib < kLwBands; ++ib) tauctot = tauctot + __ldg(in.taucld + ib + 16 * o);
  const double cwp = ciwp + clwp, cldmin = 1.e-20;
  return cf >= cldmin && (cwp >= cldmin || tauctot >= cldmin);
}
// One formed layer: advances ncb, gives the icb columns of the ice and liquid
// coefficients (0: one value, 1: 5 ice bands, 2: per band); false where the
// reference stops (a size outside its table; not-a-number sizes too).
__device__ __forceinline__ bool lw_cloud_layer(const LwIn& in, double ciwp, double clwp, double radice,
                                               double radliq, int& ncb, int& iceind, int& liqind) {
  iceind = 0;
  liqind = 0;
  if (in.inflag == 1) {
    ncb = 16;
    return true;
  }
  bool ok = true;
  if (ciwp != 0.0) {
    if (in.iceflag == 0) {
      ok = radice >= 10.0;
    } else if (in.iceflag == 1) {
      ok = radice >= 13.0 && radice <= 130.0;
      ncb = 5;
      iceind = 1;
    } else {
      ok = radice >= 5.0 && radice <= (in.iceflag == 2 ? 131.0 : 140.0);
      ncb = 16;
      iceind = 2;
    }
  }
  if (clwp == 0.0 || in.liqflag == 0) {
    if (iceind == 1) iceind = 2;
  } else {
    ok = ok && radliq >= 2.5 && radliq <= 60.0;
    ncb = 16;
    liqind = 2;
  }
  return ok;
}
// Interpolation in a (rows, bands) table at a 1-based row and fraction.
template <class A>
__device__ __forceinline__ A cld_interp(const A* t, int rows, int index, A fint, int col) {
  const A a = __ldg(t + (index - 1) + rows * col), b = __ldg(t + index + rows * col);
  return a + fint * (b - a);
}
// Ice and liquid absorption coefficients (m2/g) of coefficient band k, in
// the arithmetic A of the tables T (FP64; FP32 on the split path, whose
// g-point solver takes the depths in FP32).  The table rows are chosen in
// FP64 on both paths.
template <class A>
__device__ __forceinline__ A lw_absice(const LwIn& in, const A* T, double ciwp, double radice, int k) {
  if (ciwp == 0.0) return (A)0.;
  if (in.iceflag == 0) return __ldg(T + ct::ABSICE0) + __ldg(T + ct::ABSICE0 + 1) / (A)radice;
  if (in.iceflag == 1)
    return __ldg(T + ct::ABSICE1 + 2 * (k - 1)) + __ldg(T + ct::ABSICE1 + 1 + 2 * (k - 1)) / (A)radice;
  const int rows = in.iceflag == 2 ? 43 : 46;
  const double factor = (radice - 2.) / 3.;
  int index = (int)factor;
  if (index == rows) index = rows - 1;
  return cld_interp<A>(T + (in.iceflag == 2 ? ct::ABSICE2 : ct::ABSICE3), rows, index, (A)(factor - (double)index),
                       k - 1);
}
template <class A>
__device__ __forceinline__ A lw_absliq(const LwIn& in, const A* T, double clwp, double radliq, int k) {
  if (clwp == 0.0) return (A)0.;
  if (in.liqflag == 0) return __ldg(T + ct::ABSLIQ0);
  int index = (int)(radliq - 1.5);
  if (index == 0) index = 1;
  if (index == 58) index = 57;
  return cld_interp<A>(T + ct::ABSLIQ1, 58, index, (A)(radliq - 1.5 - (double)index), k - 1);
}

// One thread per (column, band), the 16 band threads of a column adjacent:
// the cover and formed-layer mask of every layer (band 1's thread, as
// lw_cloud_kernel) and odc[lay][col][iband] = secdiff(ib) x taucloud(lay, ib),
// ib = ipat(iband, ncbands), the cloud depth rtrn / rtrnmr use (0 for a layer
// whose optics are not formed or that filled fewer cloud bands).  Every band
// thread scans the column's layers for the final count of cloud bands, then
// walks them again with the running count.  A size outside its table sets
// flag bit 2 (reported as invalid input) and leaves the column's depths 0.
template <class F>
__global__ void __launch_bounds__(128) lw_cldphys_kernel(LwIn in, const F* __restrict__ secdiff,
                                                         const F* __restrict__ T, F* __restrict__ cld,
                                                         double* __restrict__ odc, int ncol, int nlay,
                                                         unsigned* __restrict__ flags) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)ncol * kLwBands) return;
  const int col = (int)(t / kLwBands), iband = (int)(t % kLwBands) + 1;
  const bool lead = iband == 1;
  const size_t N = (size_t)ncol, S = (size_t)nlay * N;
  int ncb = 1;
  bool ok = true;
  for (int l = 0; l < nlay; ++l) {
    const size_t o = (size_t)l * N + col;
    double cf, ciwp, clwp;
    const bool kept = lw_cloud_kept(in, o, cf, ciwp, clwp);
    if (lead) {
      cld[o] = cf >= 1.e-6 ? (F)cf : (F)0;
      cld[S + o] = kept ? (F)1 : (F)0;
    }
    int ii, li;
    if (kept && !lw_cloud_layer(in, ciwp, clwp, in.reice ? __ldg(in.reice + o) : 0.0,
                                in.reliq ? __ldg(in.reliq + o) : 0.0, ncb, ii, li))
      ok = false;
  }
  if (!ok && lead) atomicOr(flags, 4u);
  const int ib = lw_cloud_band(iband, ncb);
  const F sec = secdiff[(size_t)(ib - 1) * N + col];
  int run = 1;
  for (int l = 0; l < nlay; ++l) {
    const size_t o = (size_t)l * N + col;
    double cf, ciwp, clwp;
    const bool kept = lw_cloud_kept(in, o, cf, ciwp, clwp);
    F tc = (F)0.;
    if (ok && kept) {
      const double radice = in.reice ? __ldg(in.reice + o) : 0.0, radliq = in.reliq ? __ldg(in.reliq + o) : 0.0;
      int iceind, liqind;
      lw_cloud_layer(in, ciwp, clwp, radice, radliq, run, iceind, liqind);
      if (ib <= run) {
        if (in.inflag == 1) {
          tc = __ldg(T + ct::ABSCLD1) * (F)(ciwp + clwp);
        } else {
          const int ki = lw_cloud_band(ib, iceind == 0 ? 1 : iceind == 1 ? 5 : 16);
          const int kl = lw_cloud_band(ib, liqind == 0 ? 1 : 16);
          tc = (F)ciwp * lw_absice<F>(in, T, ciwp, radice, ki) + (F)clwp * lw_absliq<F>(in, T, clwp, radliq, kl);
        }
      }
    }
    odc[16 * o + (iband - 1)] = ok && kept ? (double)(sec * tc) : 0.0;
  }
}

// The split path's LW cloud physics: as lw_cldphys_kernel, with the layer
// tests (cldprop's keep rule, the size ranges, the count of cloud bands a
// layer leaves, the table rows and fractions of its sizes) taken once per
// layer, in FP64 as the reference takes them, by the column's 16 band threads
// together -- each a sixteenth of the layers -- and shared through shared
// memory; the depths then follow in FP32.  Dynamic shared memory: 8 columns x
// nlay layers of LwCldLay.
struct LwCldLay {
  float ciwp, clwp, rice, ifint, lfint;
  unsigned char iidx, lidx;  // table rows (1-based)
  // bit 0 kept, bits 1-2 the count the layer leaves (0 unchanged, 1: 5, 2: 16),
  // bits 3-4 iceind, bit 5 liqind = 2, bit 6 ice present, bit 7 liquid present
  unsigned char code;
};
static_assert(sizeof(LwCldLay) == 24, "LwCldLay: 24 bytes (39 KB of shared memory at 203 layers)");
__global__ void __launch_bounds__(128) lw_cldphys_split_kernel(LwIn in, const float* __restrict__ secdiff,
                                                               const float* __restrict__ T, float* __restrict__ cld,
                                                               double* __restrict__ odc, int ncol, int nlay,
                                                               unsigned* __restrict__ flags) {
  extern __shared__ LwCldLay slay[];
  __shared__ int sbad[kBlock / kLwBands];
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = t < (long long)ncol * kLwBands;
  const int cib = threadIdx.x / kLwBands, iband = threadIdx.x % kLwBands + 1;
  const int col = valid ? (int)(t / kLwBands) : 0;
  const size_t N = (size_t)ncol, S = (size_t)nlay * N;
  LwCldLay* L = slay + (size_t)cib * nlay;
  if (iband == 1) sbad[cib] = 0;
  __syncthreads();
  if (valid) {
    for (int l = iband - 1; l < nlay; l += kLwBands) {
      const size_t o = (size_t)l * N + col;
      double cf, ciwp, clwp;
      const bool kept = lw_cloud_kept(in, o, cf, ciwp, clwp);
      cld[o] = cf >= 1.e-6 ? (float)cf : 0.f;
      cld[S + o] = kept ? 1.f : 0.f;
      LwCldLay r{};
      r.code = kept ? 1 : 0;
      if (kept) {
        const double radice = in.reice ? __ldg(in.reice + o) : 0.0, radliq = in.reliq ? __ldg(in.reliq + o) : 0.0;
        int ncb = 0, ii, li;
        if (!lw_cloud_layer(in, ciwp, clwp, radice, radliq, ncb, ii, li)) sbad[cib] = 1;
        r.code |= (unsigned char)(((ncb == 5 ? 1 : ncb == 16 ? 2 : 0) << 1) | (ii << 3) | (li == 2 ? 32 : 0) |
                                  (ciwp != 0.0 ? 64 : 0) | (clwp != 0.0 ? 128 : 0));
        r.ciwp = (float)ciwp;
        r.clwp = (float)clwp;
        r.rice = (float)radice;
        if (in.inflag == 2 && ciwp != 0.0 && in.iceflag >= 2 && radice >= 5.0 && radice <= 140.0) {
          const int rows = in.iceflag == 2 ? 43 : 46;
          const double factor = (radice - 2.) / 3.;
          int index = (int)factor;
          if (index == rows) index = rows - 1;
          r.iidx = (unsigned char)index;
          r.ifint = (float)(factor - (double)index);
        }
        if (in.inflag == 2 && clwp != 0.0 && in.liqflag == 1 && radliq >= 2.5 && radliq <= 60.0) {
          int index = (int)(radliq - 1.5);
          if (index == 0) index = 1;
          if (index == 58) index = 57;
          r.lidx = (unsigned char)index;
          r.lfint = (float)(radliq - 1.5 - (double)index);
        }
      }
      L[l] = r;
    }
  }
  __syncthreads();
  if (!valid) return;
  const bool ok = sbad[cib] == 0;
  if (!ok && iband == 1) atomicOr(flags, 4u);
  int ncb = 1;
  for (int l = 0; l < nlay; ++l) {
    const int set = (L[l].code >> 1) & 3;
    if (set) ncb = set == 1 ? 5 : 16;
  }
  const int ib = lw_cloud_band(iband, ncb);
  const float sec = secdiff[(size_t)(ib - 1) * N + col];
  int run = 1;
  for (int l = 0; l < nlay; ++l) {
    const LwCldLay r = L[l];
    const bool kept = r.code & 1;
    float tc = 0.f;
    if (ok && kept) {
      const int set = (r.code >> 1) & 3;
      if (set) run = set == 1 ? 5 : 16;
      if (ib <= run) {
        if (in.inflag == 1) {
          tc = __ldg(T + ct::ABSCLD1) * (r.ciwp + r.clwp);
        } else {
          const int iceind = (r.code >> 3) & 3, liqind = (r.code & 32) ? 2 : 0;
          const int ki = lw_cloud_band(ib, iceind == 0 ? 1 : iceind == 1 ? 5 : 16);
          const int kl = lw_cloud_band(ib, liqind == 0 ? 1 : 16);
          float ai = 0.f, al = 0.f;
          if (r.code & 64) {
            if (in.iceflag == 0)
              ai = __ldg(T + ct::ABSICE0) + __ldg(T + ct::ABSICE0 + 1) / r.rice;
            else if (in.iceflag == 1)
              ai = __ldg(T + ct::ABSICE1 + 2 * (ki - 1)) + __ldg(T + ct::ABSICE1 + 1 + 2 * (ki - 1)) / r.rice;
            else
              ai = cld_interp<float>(T + (in.iceflag == 2 ? ct::ABSICE2 : ct::ABSICE3), in.iceflag == 2 ? 43 : 46,
                                     r.iidx, r.ifint, ki - 1);
          }
          if (r.code & 128) al = in.liqflag == 0 ? __ldg(T + ct::ABSLIQ0) : cld_interp<float>(T + ct::ABSLIQ1, 58, r.lidx, r.lfint, kl - 1);
          tc = r.ciwp * ai + r.clwp * al;
        }
      }
    }
    odc[16 * ((size_t)l * N + col) + (iband - 1)] = ok && kept ? (double)(sec * tc) : 0.0;
  }
}

// ---------------------------------------------------------------------------
// Overlap factors of maximum/random cloud overlap (icld = 2, 3), one thread
// per column: rrtmg_lw_rtrnmr.f90:326-475, an upward and a downward scan over
// the layers that carry the rat1 / rat2 state from one cloudy layer to the
// next (and from the upward scan into the downward one).  A cloudy layer has
// cldfrac >= 1e-6; the factors use the raw cloud fractions of the layer and
// its neighbours, cldfrac(0) and cldfrac(nlay + 1) taken as 0 (the reference
// multiplies its out-of-range cldfrac(0) by a zero factor).  A factor the
// reference zeroes at a layer below / above a clear one is the 0 that the
// scan carries out of the clear layer.  ovl[j][lay][col], j = 0..5: facclr1,
// faccld1, faccmb1, faccmb2, facclr2, faccld2 at index lay + 1 (read by the
// upward pass through layer lay); j = 6..11: the same *d factors at index
// lay - 1 (downward pass); 0 for clear layers.
// ---------------------------------------------------------------------------
template <class F>
__global__ void __launch_bounds__(128) lw_overlap_kernel(const double* __restrict__ cldfr, F* __restrict__ ovl,
                                                         int ncol, int nlay) {
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= ncol) return;
  const size_t N = (size_t)ncol, S = (size_t)nlay * N;
  auto cfa = [&](int lev) { return lev < 1 || lev > nlay ? 0.0 : __ldg(cldfr + (size_t)(lev - 1) * N + col); };
  auto cloudy = [&](int lev) { return lev >= 1 && lev <= nlay && cfa(lev) >= 1.e-6; };
  double rat1 = 0.0, rat2 = 0.0;
  double c2clr = 0.0, c2cld = 0.0;  // facclr2 / faccld2 at the current index, carried
  for (int lev = 1; lev <= nlay; ++lev) {
    F* o = ovl + (size_t)(lev - 1) * N + col;
    if (!cloudy(lev)) {
      for (int j = 0; j < 6; ++j) o[j * S] = (F)0;
      c2clr = c2cld = 0.0;
      continue;
    }
    const bool ist = !cloudy(lev - 1);
    const double cm = cfa(lev - 1), c0 = cfa(lev), cp = cfa(lev + 1);
    double clr1 = 0., clr2 = 0., cld1 = 0., cld2 = 0.;
    if (lev == nlay) {
    } else if (cp >= c0) {
      if (ist) {
        if (c0 < 1.) clr2 = (cp - c0) / (1. - c0);
      } else {
        const double fmx = c0 > cm ? c0 : cm;
        if (cp > fmx) {
          clr1 = rat2;
          clr2 = (cp - fmx) / (1. - fmx);
        } else if (cp < fmx) {
          clr1 = (cp - c0) / (cm - c0);
        } else {
          clr1 = rat2;
        }
      }
      rat1 = (clr1 > 0. || clr2 > 0.) ? 1. : 0.;
      rat2 = 0.;
    } else {
      if (ist) {
        cld2 = (c0 - cp) / c0;
      } else {
        const double fmn = c0 < cm ? c0 : cm;
        if (cp <= fmn) {
          cld1 = rat1;
          cld2 = (fmn - cp) / fmn;
        } else {
          cld1 = (c0 - cp) / (c0 - fmn);
        }
      }
      rat1 = 0.;
      rat2 = (cld1 > 0. || cld2 > 0.) ? 1. : 0.;
    }
    const double cmb1 = clr1 * c2cld * cm, cmb2 = cld1 * c2clr * (1. - cm);
    o[0] = (F)clr1;
    o[S] = (F)cld1;
    o[2 * S] = (F)cmb1;
    o[3 * S] = (F)cmb2;
    o[4 * S] = (F)clr2;
    o[5 * S] = (F)cld2;
    c2clr = clr2;
    c2cld = cld2;
  }
  c2clr = c2cld = 0.0;
  for (int lev = nlay; lev >= 1; --lev) {
    F* o = ovl + 6 * S + (size_t)(lev - 1) * N + col;
    if (!cloudy(lev)) {
      for (int j = 0; j < 6; ++j) o[j * S] = (F)0;
      c2clr = c2cld = 0.0;
      continue;
    }
    const bool ist = !cloudy(lev + 1);
    const double cm = cfa(lev - 1), c0 = cfa(lev), cp = cfa(lev + 1);
    double clr1 = 0., clr2 = 0., cld1 = 0., cld2 = 0.;
    if (lev == 1) {
    } else if (cm >= c0) {
      if (ist) {
        if (c0 < 1.) clr2 = (cm - c0) / (1. - c0);
      } else {
        const double fmx = c0 > cp ? c0 : cp;
        if (cm > fmx) {
          clr1 = rat2;
          clr2 = (cm - fmx) / (1. - fmx);
        } else if (cm < fmx) {
          clr1 = (cm - c0) / (cp - c0);
        } else {
          clr1 = rat2;
        }
      }
      rat1 = (clr1 > 0. || clr2 > 0.) ? 1. : 0.;
      rat2 = 0.;
    } else {
      if (ist) {
        cld2 = (c0 - cm) / c0;
      } else {
        const double fmn = c0 < cp ? c0 : cp;
        if (cm <= fmn) {
          cld1 = rat1;
          cld2 = (fmn - cm) / fmn;
        } else {
          cld1 = (c0 - cm) / (c0 - fmn);
        }
      }
      rat1 = 0.;
      rat2 = (cld1 > 0. || cld2 > 0.) ? 1. : 0.;
    }
    const double cmb1 = clr1 * c2cld * cp, cmb2 = cld1 * c2clr * (1. - cp);
    o[0] = (F)clr1;
    o[S] = (F)cld1;
    o[2 * S] = (F)cmb1;
    o[3 * S] = (F)cmb2;
    o[4 * S] = (F)clr2;
    o[5 * S] = (F)cld2;
    c2clr = clr2;
    c2cld = cld2;
  }
}

// ---------------------------------------------------------------------------
// LW finalize: band sums (rrtmg_lw_rtrnmr.f90:720-746), fluxes and heating
// (:752-776); clear-sky outputs equal the total ones in clear sky.
// ---------------------------------------------------------------------------
// buc, bdc, bduc: the clear-sky band partials of a cloudy call (rtrn's clear
// stream), else null (clear sky: the clear-sky outputs are the total ones).
__global__ void __launch_bounds__(128) lw_finalize_kernel(const double* __restrict__ bu, const double* __restrict__ bd,
                                                          const double* __restrict__ bdu,
                                                          const double* __restrict__ plev, int ncol, int nlay,
                                                          int idrv, double* uflx, double* dflx, double* hr,
                                                          double* uflxc, double* dflxc, double* hrc,
                                                          double* duflx_dt, double* duflxc_dt,
                                                          const double* __restrict__ buc = nullptr,
                                                          const double* __restrict__ bdc = nullptr,
                                                          const double* __restrict__ bduc = nullptr) {
  // one thread per (column, level); the heating of the layer below the level
  // re-forms the band sums of the level below (same order, same rounding)
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= ncol) return;
  const int lev = blockIdx.y;
  const LwConst& C = c_lw;
  const size_t N = (size_t)ncol;
  const double wtdiff = 0.5;
  auto sums = [&](const double* u, const double* d, int lv, double& tu, double& td) {
    tu = 0.0;
    td = 0.0;
    for (int b = 0; b < kLwBands; ++b) {
      const size_t o = ((size_t)b * (nlay + 1) + lv) * N + col;
      tu = tu + (__ldg(u + o) * wtdiff) * C.band[b].delwave;
      td = td + (__ldg(d + o) * wtdiff) * C.band[b].delwave;
    }
    tu = tu * C.fluxfac;
    td = td * C.fluxfac;
  };
  auto dsum = [&](const double* du) {
    double tdu = 0.0;
    for (int b = 0; b < kLwBands; ++b) {
      const size_t o = ((size_t)b * (nlay + 1) + lev) * N + col;
      tdu = tdu + (__ldg(du + o) * wtdiff) * C.band[b].delwave * C.fluxfac;
    }
    return tdu;
  };
  const bool clear_own = buc != nullptr;
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
    const double tdu = dsum(bdu);
    if (duflx_dt) duflx_dt[oo] = tdu;
    if (duflxc_dt) duflxc_dt[oo] = clear_own ? dsum(bduc) : tdu;
  }
  if (lev >= 1) {
    const double dp = __ldg(plev + oo - N) - __ldg(plev + oo);
    double tu0, td0;
    sums(bu, bd, lev - 1, tu0, td0);
    const double h = C.heatfac * ((tu0 - td0) - (tu - td)) / dp;
    const size_t oh = (size_t)(lev - 1) * N + col;
    hr[oh] = h;
    if (clear_own) {
      double tuc0, tdc0;
      sums(buc, bdc, lev - 1, tuc0, tdc0);
      hrc[oh] = C.heatfac * ((tuc0 - tdc0) - (tuc - tdc)) / dp;
    } else {
      hrc[oh] = h;
    }
  }
}

#endif  // RRTMG_DEFINE_COLUMN_KERNELS

// ---------------------------------------------------------------------------
// SW prep: inatm_sw (rrtmg_sw_rad.nomcica.f90:761-1101) + setcoef_sw
// (rrtmg_sw_setcoef.f90:30-286) + the solar-source layer of every band
// (laysolfr logic of taumol16..29).
// ---------------------------------------------------------------------------
__device__ __forceinline__ int sw_layreffr(int b) {
  switch (b) {
    case 16: return 18; case 17: return 30; case 18: return 6; case 19: return 3; case 20: return 3;
    case 21: return 8; case 22: return 2; case 23: return 6; case 24: return 1; case 25: return 2;
    case 27: return 32; case 28: return 58; case 29: return 49; default: return 0;
  }
}
// Bands whose solar source is taken in the upper-atmosphere loop.
__host__ __device__ constexpr bool sw_upper_source(int b) { return b == 16 || b == 17 || b == 27 || b == 28 || b == 29; }

#ifdef RRTMG_DEFINE_COLUMN_KERNELS
// Two launches as for LW: one thread per (column, layer), then one thread per
// column for laytrop and the solar-source layer of every band.
// F is the storage and the arithmetic type, as for the LW prep kernels.
template <class F>
__global__ void __launch_bounds__(128) sw_prep_layer_kernel(SwIn in, SwWorkT<F> w, int ncol, int nlay,
                                                            unsigned* __restrict__ flags) {
  using T = F;
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= ncol) return;
  const int l = blockIdx.y + 1;
  const SwConst& C = c_sw;
  const T amd = (T)28.9660, amw = (T)18.0160, amdw = (T)1.607793, amdo = (T)0.603428;
  const T stpfac = (T)(296. / 1013.);
  const size_t N = (size_t)ncol;
  const size_t fstride = (size_t)nlay * N;
  auto A = [&](const double* p, int ll) { return __ldg(p + (size_t)col + N * (size_t)(ll - 1)); };
  unsigned flag = 0;
  {
    const double pv = A(in.play, l), tv = A(in.tlay, l), pz = A(in.plev, l + 1), q = A(in.h2o, l);
    if (bad(pv) || bad(tv) || bad(pz) || bad(q) || pv <= 0. || tv <= 0. || q < 0. || q >= 1. || pz < 0.) flag = 1;
  }
  const T pz_prev = (T)A(in.plev, l);
  const T pavel = (T)A(in.play, l), tavel = (T)A(in.tlay, l);
  const T pz_l = (T)A(in.plev, l + 1);
  const T h2o = (T)A(in.h2o, l);
  T wk1 = (h2o / ((T)1. - h2o)) * amdw;
  T wk2 = (T)A(in.co2, l);
  T wk3 = (T)A(in.o3, l) * amdo;
  T wk4 = in.n2o ? (T)A(in.n2o, l) : (T)0.0;
  T wk6 = in.ch4 ? (T)A(in.ch4, l) : (T)0.0;
  T wk7 = in.o2 ? (T)A(in.o2, l) : (T)0.0;
  T amm = ((T)1. - wk1) * amd + wk1 * amw;
  T coldry = (pz_prev - pz_l) * (T)1.e3 * (T)C.avogad / ((T)1.e2 * (T)C.grav * amm * ((T)1. + wk1));
  wk1 = coldry * wk1;
  wk2 = coldry * wk2;
  wk3 = coldry * wk3;
  wk4 = coldry * wk4;
  wk6 = coldry * wk6;
  wk7 = coldry * wk7;

  const T plog = log(pavel);
  const int jp = clampi((int)((T)36. - (T)5 * (plog + (T)0.04)), 1, 58);
  const int jp1 = jp + 1;
  const T fp = (T)5. * ((T)C.preflog[jp - 1] - plog);
  const int jt = clampi((int)((T)3. + (tavel - (T)C.tref[jp - 1]) / (T)15.), 1, 4);
  const T ft = ((tavel - (T)C.tref[jp - 1]) / (T)15.) - (T)(jt - 3);
  const int jt1 = clampi((int)((T)3. + (tavel - (T)C.tref[jp1 - 1]) / (T)15.), 1, 4);
  const T ft1 = ((tavel - (T)C.tref[jp1 - 1]) / (T)15.) - (T)(jt1 - 3);
  const T water = wk1 / coldry;
  const T scalefac = pavel * stpfac / tavel;
  T forfac, forfrac, selffac, selffrac, factor;
  int indfor, indself;
  const bool lower = plog > (T)4.56;
  if (lower) {
    forfac = scalefac / ((T)1. + water);
    factor = ((T)332.0 - tavel) / (T)36.0;
    indfor = min(2, max(1, (int)factor));
    forfrac = factor - (T)indfor;
    selffac = water * forfac;
    factor = (tavel - (T)188.0) / (T)7.2;
    indself = min(9, max(1, (int)factor - 7));
    selffrac = factor - (T)(indself + 7);
  } else {
    forfac = scalefac / ((T)1. + water);
    factor = (tavel - (T)188.0) / (T)36.0;
    indfor = 3;
    forfrac = factor - (T)1.0;
    selffac = (T)0.;
    selffrac = (T)0.;
    indself = 0;
  }
  const T e20 = (T)1.e-20, e32 = (T)1.e-32;
  T colh2o = e20 * wk1, colco2 = e20 * wk2, colo3 = e20 * wk3, coln2o = e20 * wk4;
  T colch4 = e20 * wk6, colo2 = e20 * wk7;
  const T colmol = e20 * coldry + colh2o;
  if (colco2 == (T)0.) colco2 = e32 * coldry;
  if (coln2o == (T)0.) coln2o = e32 * coldry;
  if (colch4 == (T)0.) colch4 = e32 * coldry;
  if (colo2 == (T)0.) colo2 = e32 * coldry;
  const T compfp = (T)1. - fp;
  const size_t o = (size_t)(l - 1) * N + col;
  F* f = w.f;
  f[SF_COLH2O * fstride + o] = colh2o;
  f[SF_COLCO2 * fstride + o] = colco2;
  f[SF_COLO3 * fstride + o] = colo3;
  f[SF_COLCH4 * fstride + o] = colch4;
  f[SF_COLO2 * fstride + o] = colo2;
  f[SF_COLMOL * fstride + o] = colmol;
  f[SF_FAC10 * fstride + o] = compfp * ft;
  f[SF_FAC00 * fstride + o] = compfp * ((T)1. - ft);
  f[SF_FAC11 * fstride + o] = fp * ft1;
  f[SF_FAC01 * fstride + o] = fp * ((T)1. - ft1);
  f[SF_SELFFAC * fstride + o] = selffac;
  f[SF_SELFFRAC * fstride + o] = selffrac;
  f[SF_FORFAC * fstride + o] = forfac;
  f[SF_FORFRAC * fstride + o] = forfrac;
  w.idx[o] = pack_idx(jp, jt, jt1, indself, indfor, 1);

  if (flag) atomicOr(flags, 1u);
}

template <class F>
__global__ void __launch_bounds__(128) sw_prep_column_kernel(SwIn in, SwWorkT<F> w, int ncol, int nlay,
                                                             unsigned* __restrict__ flags) {
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= ncol) return;
  const size_t N = (size_t)ncol;
  auto A = [&](const double* p, int l) { return __ldg(p + (size_t)col + N * (size_t)(l - 1)); };
  unsigned flag = 0;
  if (bad(__ldg(in.coszen + col))) flag = 1;
  int laytrop = 0;
  for (int l = 1; l <= nlay; ++l)
    if (log((F)A(in.play, l)) > (F)4.56) laytrop = laytrop + 1;  // the layer kernel's test, in F
  w.laytrop[col] = laytrop;
  // Solar-source layer of every band, as the taumol16..29 loops select it:
  //   upper-loop bands (16, 17, 27, 28, 29): laysolfr = nlay, replaced by the
  //     last lay in laytrop+1..nlay with jp(lay-1) < layreffr <= jp(lay);
  //   lower-loop bands (18..25): laysolfr = laytrop, replaced by
  //     min(lay+1, laytrop) for the last lay in 1..laytrop with
  //     jp(lay) < layreffr <= jp(lay+1);
  //   band 26: laytrop.
  // jp(0) and jp(nlay+1) read as 0.  0 means "no source layer" (empty loop).
  auto jpat = [&](int lay) -> int {
    if (lay < 1 || lay > nlay) return 0;
    return unpack_idx(w.idx[(size_t)(lay - 1) * N + col]).jp;
  };
  for (int bi = 0; bi < kSwBands; ++bi) {
    const int b = bi + 16;
    const int ref = sw_layreffr(b);
    int ls;
    if (b == 26) {
      ls = laytrop;
    } else if (sw_upper_source(b)) {
      ls = (laytrop < nlay) ? nlay : 0;
      for (int lay = laytrop + 1; lay <= nlay; ++lay)
        if (jpat(lay - 1) < ref && jpat(lay) >= ref) ls = lay;
    } else {
      ls = laytrop;
      for (int lay = 1; lay <= laytrop; ++lay)
        if (jpat(lay) < ref && jpat(lay + 1) >= ref) ls = min(lay + 1, laytrop);
    }
    w.laysolfr[bi * N + col] = ls;
  }
  if (flag) atomicOr(flags, 1u);
}

#endif  // RRTMG_DEFINE_COLUMN_KERNELS

// ---------------------------------------------------------------------------
// SW g-point solver: taumol_sw, delta-scaling and reftra_sw, direct beam, the
// two vrtqdr_sw sweeps, for one g-point (rrtmg_sw_spcvrt.f90:296-618,
// rrtmg_sw_reftra.f90, rrtmg_sw_vrtqdr.f90).  In clear sky the reference's
// "total" stream is bit-identical to its "clear" stream (cloud weights 0/1),
// so one stream is computed and written to both outputs.
// ---------------------------------------------------------------------------
template <class R, class TT>
__device__ __forceinline__ R sw_exp_tbl(R ze1, R bpade, const TT* __restrict__ exptbl, bool analytic) {
  if (ze1 <= (R)0.06) return (R)1. - ze1 + (R)0.5 * ze1 * ze1;
  if (analytic) return exp(-ze1);
  const R tblind = ze1 / (bpade + ze1);
  int itind = (int)((R)10000.0 * tblind + (R)0.5);
  itind = itind < 0 ? 0 : (itind > kNTbl ? kNTbl : itind);  // guards NaN / negative optical depths
  return (R)tld(exptbl + itind);
}

// delta-Eddington layer reflectance/transmittance, kmodts = 2 (rrtmg_sw_reftra.f90:143-300)
template <class R, class TT>
__device__ __forceinline__ void reftra1(R zto1, R zw, R zg, R prmuz, R bpade, const TT* __restrict__ exptbl,
                                        bool analytic, R& pref, R& prefd, R& ptra, R& ptrad) {
  const R eps = (R)1.e-08, zwcrit = (R)0.9999995;
  const R zg3 = (R)3. * zg;
  const R zgamma1 = ((R)8. - zw * ((R)5. + zg3)) * (R)0.25;
  const R zgamma2 = (R)3. * (zw * ((R)1. - zg)) * (R)0.25;
  const R zgamma3 = ((R)2. - zg3 * prmuz) * (R)0.25;
  const R zgamma4 = (R)1. - zgamma3;
  const R r = zg / ((R)1. - zg);
  const R zwo = zw / ((R)1. - ((R)1. - zw) * (r * r));
  if (zwo >= zwcrit) {
    const R za = zgamma1 * prmuz;
    const R za1 = za - zgamma3;
    const R zgt = zgamma1 * zto1;
    const R ze1 = fmin(zto1 / prmuz, (R)500.);
    const R ze2 = sw_exp_tbl<R, TT>(ze1, bpade, exptbl, analytic);
    pref = (zgt - za1 * ((R)1. - ze2)) / ((R)1. + zgt);
    ptra = (R)1. - pref;
    prefd = zgt / ((R)1. + zgt);
    ptrad = (R)1. - prefd;
    if (ze2 == (R)1.0) {
      pref = (R)0.0;
      ptra = (R)1.0;
      prefd = (R)0.0;
      ptrad = (R)1.0;
    }
  } else {
    const R za1 = zgamma1 * zgamma4 + zgamma2 * zgamma3;
    const R za2 = zgamma1 * zgamma3 + zgamma2 * zgamma4;
    const R zrk = sqrt(zgamma1 * zgamma1 - zgamma2 * zgamma2);
    const R zrp = zrk * prmuz;
    const R zrp1 = (R)1. + zrp;
    const R zrm1 = (R)1. - zrp;
    const R zrk2 = (R)2. * zrk;
    const R zrpp = (R)1. - zrp * zrp;
    const R zrkg = zrk + zgamma1;
    const R zr1 = zrm1 * (za2 + zrk * zgamma3);
    const R zr2 = zrp1 * (za2 - zrk * zgamma3);
    const R zr3 = zrk2 * (zgamma3 - za2 * prmuz);
    const R zr4 = zrpp * zrkg;
    const R zr5 = zrpp * (zrk - zgamma1);
    const R zt1 = zrp1 * (za1 + zrk * zgamma4);
    const R zt2 = zrm1 * (za1 - zrk * zgamma4);
    const R zt3 = zrk2 * (zgamma4 + za1 * prmuz);
    const R zbeta = (zgamma1 - zrk) / zrkg;
    const R ze1 = fmin(zrk * zto1, (R)500.);
    const R ze2 = fmin(zto1 / prmuz, (R)500.);
    const R zem1 = sw_exp_tbl<R, TT>(ze1, bpade, exptbl, analytic);
    const R zep1 = (R)1. / zem1;
    const R zem2 = sw_exp_tbl<R, TT>(ze2, bpade, exptbl, analytic);
    const R zep2 = (R)1. / zem2;
    const R zdenr = zr4 * zep1 + zr5 * zem1;
    const R zt4 = zr4, zt5 = zr5;
    const R zdent = zt4 * zep1 + zt5 * zem1;
    if (zdenr >= -eps && zdenr <= eps) {
      pref = eps;
      ptra = zem2;
    } else {
      pref = zw * (zr1 * zep1 - zr2 * zem1 - zr3 * zem2) / zdenr;
      ptra = zem2 - zem2 * zw * (zt1 * zep1 - zt2 * zem1 - zt3 * zep2) / zdent;
    }
    const R zemm = zem1 * zem1;
    const R zdend = (R)1. / (((R)1. - zbeta * zemm) * zrkg);
    prefd = zgamma2 * ((R)1. - zemm) * zdend;
    ptrad = zrk2 * zem1 * zdend;
  }
}

// exp(-x) from the SW table / series together with exp(-x) - 1, the latter
// formed without cancellation (series: -x + x^2/2; table: tbl - 1).
// R: float, or a dual number of floats (the split adjoint).
template <class R>
__device__ __forceinline__ void sw_exp_pair(R ze1, R bpade, const float* __restrict__ exptbl, bool analytic, R& e,
                                            R& em1) {
  if (ze1 <= (R)0.06) {
    em1 = -ze1 + (R)0.5 * ze1 * ze1;
    e = (R)1. - ze1 + (R)0.5 * ze1 * ze1;
    return;
  }
  if (analytic) {
    e = exp(-ze1);
    em1 = expm1(-ze1);
    return;
  }
  const R tblind = ze1 / (bpade + ze1);
  int itind = (int)((R)10000.0 * tblind + (R)0.5);
  itind = itind < 0 ? 0 : (itind > kNTbl ? kNTbl : itind);
  e = (R)tld(exptbl + itind);
  em1 = e - (R)1.;
}

// FP32 delta-Eddington layer solution (same model as reftra1, kmodts = 2),
// rearranged so that no O(1) terms cancel for optically thin or nearly
// conservative layers, where FP32 would otherwise lose the layer absorptance,
// and so that no e^{+kt} is formed (scaled by e^{-kt}, see below):
//   * the numerators zr1 e^{kt} - zr2 e^{-kt} - zr3 e^{-t/mu} (and the zt
//     analogue) have zr1 - zr2 - zr3 = 0, so they are evaluated on the
//     complements e - 1;
//   * k = sqrt(g1^2 - g2^2) = sqrt(2 (1 - w) (g1 + g2)) since g1 - g2 = 2(1 - w);
//   * (1 - beta e^{-2kt}) (k + g1) = 2k + (g1 - k)(1 - e^{-2kt});
//   * zr4 e^{kt} + zr5 e^{-kt} = zrpp (k (e^{kt} + e^{-kt}) + g1 (e^{kt} - e^{-kt})).
// Exponentials are the same table / series values as the reference uses.
// zg_zero: the asymmetry factor is identically 0 (no aerosol), so r = 0 and
// zwo = zw without the two divisions.  pdbt (optional): e^{-t/mu}, the value
// the direct-beam lookup of spcvrt_sw (rrtmg_sw_spcvrt.f90:496-507) takes for
// the same argument (its missing 500 cap changes nothing in FP32, where both
// table ends are 0).  cw (optional, >= 0): the co-albedo 1 - zw formed
// without cancellation by the caller.  An FP32 albedo within 1e-5 of 1 holds
// its co-albedo to a few per cent only, and the absorptance of an optically
// thick, nearly conservative layer (a cloud) scales with it; with cw the
// conservative-branch test is made on the co-albedo of zwo, 1 - zwo =
// cw (1 - r^2) / (1 - cw r^2), as the reference's FP64 test resolves it.
template <class R>
__device__ __forceinline__ void reftra_split(R zto1, R zw, R zg, R prmuz, R bpade, const float* __restrict__ exptbl,
                                             bool analytic, R& pref, R& prefd, R& ptra, R& ptrad,
                                             bool zg_zero = false, R* pdbt = nullptr, R cw = (R)-1.) {
  const R eps = (R)1.e-08, zwcrit = (R)0.9999995;
  const R zg3 = (R)3. * zg;
  const R zgamma1 = ((R)8. - zw * ((R)5. + zg3)) * (R)0.25;
  const R zgamma2 = (R)3. * (zw * ((R)1. - zg)) * (R)0.25;
  const R zgamma3 = ((R)2. - zg3 * prmuz) * (R)0.25;
  const R zgamma4 = (R)1. - zgamma3;
  const bool own_cw = cw >= (R)0.;
  if (!own_cw) cw = (R)1. - zw;
  bool conservative;
  if (own_cw) {
    // zwo = zw / den: a negative den makes zwo negative, a zero one infinite
    const R r2 = zg_zero ? (R)0. : (zg / ((R)1. - zg)) * (zg / ((R)1. - zg));
    const R den = (R)1. - cw * r2;
    conservative = den > (R)0. ? cw * ((R)1. - r2) <= (R)(1. - 0.9999995) * den : den == (R)0.;
  } else {
    R zwo = zw;
    if (!zg_zero) {
      const R r = zg / ((R)1. - zg);
      zwo = zw / ((R)1. - cw * (r * r));
    }
    conservative = zwo >= zwcrit;
  }
  if (conservative) {
    const R za1 = zgamma1 * prmuz - zgamma3;
    const R zgt = zgamma1 * zto1;
    R ze2, m2;
    sw_exp_pair(fmin(zto1 / prmuz, (R)500.), bpade, exptbl, analytic, ze2, m2);
    if (pdbt) *pdbt = ze2;
    pref = (zgt + za1 * m2) / ((R)1. + zgt);
    ptra = (R)1. - pref;
    prefd = zgt / ((R)1. + zgt);
    ptrad = (R)1. - prefd;
    if (m2 == (R)0.) {
      pref = (R)0.;
      ptra = (R)1.;
      prefd = (R)0.;
      ptrad = (R)1.;
    }
  } else {
    const R za1 = zgamma1 * zgamma4 + zgamma2 * zgamma3;
    const R za2 = zgamma1 * zgamma3 + zgamma2 * zgamma4;
    const R zrk = sqrt(((R)2. * cw) * (zgamma1 + zgamma2));
    const R zrp = zrk * prmuz;
    const R zrp1 = (R)1. + zrp, zrm1 = (R)1. - zrp, zrk2 = (R)2. * zrk, zrpp = (R)1. - zrp * zrp;
    const R zr1 = zrm1 * (za2 + zrk * zgamma3);
    const R zr2 = zrp1 * (za2 - zrk * zgamma3);
    const R zr3 = zrk2 * (zgamma3 - za2 * prmuz);
    const R zt1 = zrp1 * (za1 + zrk * zgamma4);
    const R zt2 = zrm1 * (za1 - zrk * zgamma4);
    const R zt3 = zrk2 * (zgamma4 + za1 * prmuz);
    R zem1, m1, zem2, m2;
    sw_exp_pair(fmin(zrk * zto1, (R)500.), bpade, exptbl, analytic, zem1, m1);
    sw_exp_pair(fmin(zto1 / prmuz, (R)500.), bpade, exptbl, analytic, zem2, m2);
    if (pdbt) *pdbt = zem2;
    // Numerators and denominator multiplied by E = e^{-kt} (= zem1), so that
    // only e^{-kt}, e^{-t/mu} and their complements appear: e^{+kt} would
    // overflow FP32 in thick layers (and its derivative already beyond kt = 44).
    //   (e^{kt} - 1) E = -m1,  (e^{kt} + e^{-kt}) E = 1 + E^2,  (e^{kt} - e^{-kt}) E = 1 - E^2,
    //   (e^{t/mu} - 1) e^{-t/mu} = -m2.
    const R E = zem1;
    const R zden = zrpp * (zrk * ((R)1. + E * E) + zgamma1 * (-m1 * ((R)2. + m1)));
    if (zden >= -eps && zden <= eps) {
      pref = eps;
      ptra = zem2;
    } else {
      const R wz = zw / zden;
      pref = wz * (-m1 * (zr1 + zr2 * E) - zr3 * m2 * E);
      ptra = zem2 - wz * (-m1 * zem2 * (zt1 + zt2 * E) + zt3 * m2 * E);
    }
    const R omm = -m1 * ((R)2. + m1);  // 1 - e^{-2kt}
    const R zdend = (R)1. / (zrk2 + (zgamma1 - zrk) * omm);
    prefd = zgamma2 * omm * zdend;
    ptrad = zrk2 * zem1 * zdend;
  }
}

// TOT: the total-sky pass of a cloudy call (icld = 1): every layer's clear
// optics combined with its cloud optics by the cover (spcvrt_sw :459-525);
// cld: [cover][cldprop mask] per layer.  Otherwise the clear-sky pass.
template <int B, class R, int MAXL, bool TOT = false, int G0 = 0, int NS = sw_ng(B), int SLOT = B - 16>
__device__ __forceinline__ void sw_band(const SwPrepT<R>& p, const SwIn& in, double adjflux, int iaer,
                                        const R* __restrict__ tab, const double* __restrict__ tab64,
                                        const R* __restrict__ exptbl, double* __restrict__ su,
                                        double* __restrict__ sd, int ncol, int nlay, bool analytic, int blk, float* sbuf,
                                        float* swt, const R* __restrict__ cld = nullptr) {
  constexpr bool SPLIT = sizeof(R) == 4;
  constexpr int NG = NS;
  constexpr int W = split_lanes(NG, SPLIT);
  constexpr int CPW = 32 / W;
  constexpr int CPB = (kBlock / 32) * CPW;
  constexpr int ibm = B - 15;  // 1..14
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int lane_col = wib * CPW + lane / W, g = lane % W;
  const int col = blk * CPB + lane_col;
  const bool valid = lane < CPW * W && col < ncol;
  const int c = valid ? col : (col < ncol ? col : ncol - 1);
  const int gg = G0 + (g < NG ? g : NG - 1);
  const size_t N = (size_t)ncol;
  const size_t fstride = (size_t)nlay * N;
  const double coszen = __ldg(in.coszen + c);
  const bool lit = coszen >= 1.e-10;
  const bool active = valid && g < NG && lit;
  const R prmu0 = lit ? (R)coszen : (R)1.0;
  const R bpade = (R)c_sw.bpade;
  const int lt = p.laytrop[c];
  const int klev = nlay;

  // Solar source and incident flux of this g-point.
  double zincflx = 0.0;
  {
    const int ls = p.laysolfr[(size_t)(B - 16) * N + c];
    if (ls >= 1) {
      SwLayerView<double, R> L{p.f, fstride, (size_t)(ls - 1) * N + c};
      const double sfz = sw_sfluxzen<B>(c_sw, L, ls <= lt, gg, tab64);
      zincflx = adjflux * sfz * (lit ? coszen : 1.0);
    }
  }
  const R albdir = (R)__ldg(((ibm >= 10 && ibm <= 13) ? in.asdir : in.aldir) + c);
  const R albdif = (R)__ldg(((ibm >= 10 && ibm <= 13) ? in.asdif : in.aldif) + c);

  // Layer and level state, top-down (jk = 1..klev, + surface klev+1):
  // lay[k] = {pref, prefd, ptra, ptrad} of layer k (0-based);
  // lvl[j] = {ptdbt, ztdn, prdnd} of level j and pdbt of layer j.  The level
  // above the current layer is carried in registers (tdbt1, tdn1, rdnd1).
  Quad<R> lay[MAXL + 1], lvl[MAXL + 2];
  R tdbt1 = (R)1.0, tdn1 = (R)1.0, rdnd1 = (R)0.0;
  // the packed table indices of the next layer are loaded one layer ahead
  uint32_t idx_next = __ldg(p.idx + (size_t)(klev - 1) * N + c);
  for (int jk = 1; jk <= klev; ++jk) {
    const int ikl = klev + 1 - jk;
    const size_t o = (size_t)(ikl - 1) * N + c;
    const Idx ix = unpack_idx(idx_next);
    if (ikl > 1) idx_next = __ldg(p.idx + o - N);
    SwLayerView<R> L{p.f, fstride, o};
    R taug, taur;
    sw_gas<B, R>(c_sw, L, ix, ikl <= lt, gg, tab, taug, taur);
    R taua = (R)0., omga = (R)1., asya = (R)0.;
    R cwa = (R)0.;  // the aerosol co-albedo 1 - omga, formed in FP64 (cloudy split pass)
    if (iaer == 10) {
      const size_t oa = c + N * ((size_t)(ikl - 1) + (size_t)nlay * (ibm - 1));
      taua = (R)__ldg(in.tauaer + oa);
      const double ssaa = __ldg(in.ssaaer + oa);
      omga = (R)ssaa;
      if constexpr (TOT && sizeof(R) == 4) cwa = (R)(1.0 - ssaa);
      asya = (R)__ldg(in.asmaer + oa);
    }
    R ztauc = taur + taug + taua;
    R zomcc = taur * (R)1.0 + taua * omga;
    R zgcc = asya * omga * taua / zomcc;
    zomcc = zomcc / ztauc;
    const R zf = zgcc * zgcc;
    const R zwf = zomcc * zf;
    ztauc = ((R)1.0 - zwf) * ztauc;
    zomcc = (zomcc - zwf) / ((R)1.0 - zwf);
    zgcc = (zgcc - zf) / ((R)1.0 - zf);
    R rf, rfd, tr, trd, zdbtmc;
    if constexpr (sizeof(R) == 4) {
      reftra_split(ztauc, zomcc, zgcc, prmu0, bpade, exptbl, analytic, rf, rfd, tr, trd, iaer != 10, &zdbtmc);
    } else {
      reftra1<R, R>(ztauc, zomcc, zgcc, prmu0, bpade, exptbl, analytic, rf, rfd, tr, trd);
      zdbtmc = sw_exp_tbl<R, R>(ztauc / prmu0, bpade, exptbl, analytic);
    }
    if constexpr (TOT) {
      // A layer without cover keeps its clear optics: the reference's cover-weighted
      // combination below gives them back exactly (1 x clear + 0 x total), so the
      // total-sky optics of such a layer are skipped.
      // cldprop_sw, inflag = 0 (rrtmg_sw_cldprop.f90:142-156): delta-M scaled
      // cloud optics where the mask keeps them, else tau 0, ssa 1, g 0
      const R pclfr = __ldg(cld + o);
      if (pclfr > (R)0.) {
        R ptauc = (R)0., pomgc = (R)1., pasyc = (R)0.;
        R pcw = (R)0.;  // split path: the cloud's delta-scaled co-albedo 1 - pomgc
        if (sizeof(R) == 4 && __ldg(cld + fstride + o) > (R)0.) {
          // split path: the band's optics as sw_cloud_kernel formed them
          const float4 qv = __ldg(in.cldq + (size_t)(ibm - 1) + 14 * o);
          ptauc = (R)qv.x;
          pomgc = (R)qv.y;
          pasyc = (R)qv.z;
          pcw = (R)qv.w;
        } else if (__ldg(cld + fstride + o) > (R)0.) {
          const size_t q = (size_t)(ibm - 1) + 14 * o;
          const R taucldorig = (R)__ldg(in.taucld + q), ffp = in.fsfcld ? (R)__ldg(in.fsfcld + q) : (R)0.;
          const R ssac = (R)__ldg(in.ssacld + q), asmc = (R)__ldg(in.asmcld + q);
          const R ffp1 = (R)1.0 - ffp;
          const R ffpssa = (R)1.0 - ffp * ssac;
          pomgc = ffp1 * ssac / ffpssa;
          ptauc = ffpssa * taucldorig;
          pasyc = (asmc - ffp) / (ffp1);
        }
        // total-sky optics (spcvrt_sw :459-464), reftra only for cloudy layers
        // (pclfr > repclc = 1e-12, :388; reftra gives 0, 1, 0, 1 otherwise)
        const R ztauo = ztauc + ptauc;
        R zomco = ztauc * zomcc + ptauc * pomgc;
        const R zgco = (ptauc * pomgc * pasyc + ztauc * zomcc * zgcc) / zomco;
        zomco = zomco / ztauo;
        R rfo = (R)0., rfdo = (R)0., tro = (R)1., trdo = (R)1.;
        if (pclfr > (R)1.e-12) {
          if constexpr (sizeof(R) == 4) {
            // the total co-albedo from the clear one (gas absorption and aerosol
            // co-albedo over the depth, through the delta-M scaling: 1 - w' =
            // (1 - w) / (1 - f w)) and the cloud's, without cancellation
            const R cwc = (taug + taua * cwa) / ((taur + taug + taua) * ((R)1.0 - zwf));
            const R cwo = (ztauc * cwc + ptauc * pcw) / ztauo;
            reftra_split(ztauo, zomco, zgco, prmu0, bpade, exptbl, analytic, rfo, rfdo, tro, trdo, false, (R*)nullptr,
                         cwo);
          } else {
            reftra1<R, R>(ztauo, zomco, zgco, prmu0, bpade, exptbl, analytic, rfo, rfdo, tro, trdo);
          }
        }
        const R zdbtmo = sw_exp_tbl<R, R>(ztauo / prmu0, bpade, exptbl, analytic);
        const R zclear = (R)1.0 - pclfr, zcloud = pclfr;
        rf = zclear * rf + zcloud * rfo;
        rfd = zclear * rfd + zcloud * rfdo;
        tr = zclear * tr + zcloud * tro;
        trd = zclear * trd + zcloud * trdo;
        zdbtmc = zclear * zdbtmc + zcloud * zdbtmo;
      }
    }
    lay[jk - 1] = Quad<R>{rf, rfd, tr, trd};
    lvl[jk - 1] = Quad<R>{tdbt1, tdn1, rdnd1, zdbtmc};
    // Downward adding sweep of vrtqdr_sw (:127-139), fused with the layer loop
    // (level 0: ptdbt = ztdn = 1, prdnd = 0).
    const R tdbt = zdbtmc * tdbt1;
    if (jk == 1) {
      tdn1 = tr;
      rdnd1 = rfd;
    } else {
      const R zreflect = (R)1. / ((R)1. - rfd * rdnd1);
      const R tdn = tdbt1 * tr + (trd * ((tdn1 - tdbt1) + tdbt1 * rf * rdnd1)) * zreflect;
      rdnd1 = rfd + trd * trd * rdnd1 * zreflect;
      tdn1 = tdn;
    }
    tdbt1 = tdbt;
  }
  lvl[klev] = Quad<R>{tdbt1, tdn1, rdnd1, (R)0.};
  // Upward sweep (vrtqdr_sw :104-124) from the surface, with the level fluxes
  // (:141-149) as soon as each level's upward reflectances are known.
  double* sup = su + (size_t)SLOT * (nlay + 1) * N + col;
  double* sdp = sd + (size_t)SLOT * (nlay + 1) * N + col;
  // Split path: incident-flux-weighted band sums through the warp's staging
  // buffers (levels surface first); the summing lane of column sub-index cs
  // writes column wcol0 + cs.
  const int wcol0 = blk * CPB + wib * CPW;
  GSum<W, NG, 2, true> gs{sbuf + (SPLIT ? wib * kStageRows * kRow : 0), swt + (SPLIT ? wib * 32 : 0), lane, 0, 0, 1, 2};
  if constexpr (SPLIT) swt[wib * 32 + lane] = active ? (float)zincflx : 0.f;
  auto store = [&](int b, int lev, int cs, float s, float cmp) {
    const int cc = wcol0 + cs;
    if (cc < ncol) as_pair(b == 0 ? su : sd)[((size_t)SLOT * (nlay + 1) + lev) * N + cc] = make_float2(s, cmp);
  };
  R prup = albdir, prupd = albdif;  // level klev+1 (surface)
  for (int jk = klev + 1; jk >= 1; --jk) {
    const Quad<R> lv = lvl[jk - 1];  // level jk-1, and the direct beam of layer jk-1
    if (jk <= klev) {
      const Quad<R> ly = lay[jk - 1];
      const R pref = ly.a, prefd = ly.b, ptra = ly.c, ptrad = ly.d, pdbt = lv.d;
      if (jk == klev) {
        const R zreflect = (R)1. / ((R)1. - albdif * prefd);
        const R nup = pref + (ptrad * ((ptra - pdbt) * albdif + pdbt * albdir)) * zreflect;
        const R nupd = prefd + ptrad * ptrad * albdif * zreflect;
        prup = nup;
        prupd = nupd;
      } else {
        const R zreflect = (R)1. / ((R)1. - prupd * prefd);
        const R nup = pref + (ptrad * ((ptra - pdbt) * prupd + pdbt * prup)) * zreflect;
        const R nupd = prefd + ptrad * ptrad * prupd * zreflect;
        prup = nup;
        prupd = nupd;
      }
    }
    const R tdbt = lv.a, tdn = lv.b, rdnd = lv.c;
    const R zreflect = (R)1. / ((R)1. - rdnd * prupd);
    const R pfu = (tdbt * prup + (tdn - tdbt) * prupd) * zreflect;
    const R pfd = tdbt + (tdn - tdbt + tdbt * prup * rdnd) * zreflect;
    // output level (surface first) ikl = klev + 2 - jk  ->  0-based klev + 1 - jk
    if constexpr (SPLIT) {
      gs.put(0, pfu);
      gs.put(1, pfd);
      gs.next(store);
    } else {
      const double su_s = seg_sum<W>(active ? zincflx * (double)pfu : 0.0);
      const double sd_s = seg_sum<W>(active ? zincflx * (double)pfd : 0.0);
      if (g == 0 && valid) {
        sup[(size_t)(klev + 1 - jk) * N] = su_s;
        sdp[(size_t)(klev + 1 - jk) * N] = sd_s;
      }
    }
  }
  if constexpr (SPLIT) {
    if (gs.n) gs.flush(store);
  }
}

// FL < 0: analytic and iaer as passed; FL >= 0: compile-time flags (bit 0
// analytic, bit 1 iaer = 10), as for the LW kernel.  TOT: the total-sky pass
// of a cloudy call (cld: per-layer cover and cldprop mask), else clear sky.
template <class R, int MAXL, int FL = -1, bool TOT = false>
__global__ void __launch_bounds__(kBlock, sizeof(R) == 4 ? RRTMG_SPLIT_SW_MINB : 1) sw_gpoint_kernel(SwPrepT<R> p, SwIn in, double adjflux, int iaer,
                                                           const R* __restrict__ tab, const double* __restrict__ tab64,
                                                           const R* __restrict__ exptbl, double* su, double* sd,
                                                           int ncol, int nlay, int analytic, const R* __restrict__ cld) {
  __shared__ float sbuf[sizeof(R) == 4 ? kGSumFloats : 1];
  __shared__ float swt[sizeof(R) == 4 ? kBlock : 1];
  constexpr bool SPLIT = sizeof(R) == 4;
  int blk = blockIdx.x;
  const int unit = sw_unit_of_block<SPLIT>(blk, ncol);  // slot (split) or band (FP64)
  const int band = SPLIT ? (unit < kSwSlots ? sw_slot(unit).band - 16 : kSwBands) : unit;
  if (threadIdx.x == 0 && band < kSwBands) prefetch_band_l2(tab, c_sw.band[band]);
  const bool an = FL < 0 ? analytic != 0 : (FL & 1) != 0;
  const int ia = FL < 0 ? iaer : ((FL & 2) ? 10 : 0);
  if constexpr (SPLIT) {
#define RRTMG_SW_SLOT(s)                                                                                         \
  case s:                                                                                                        \
    sw_band<sw_slot(s).band, R, MAXL, TOT, sw_slot(s).g0, sw_slot(s).ng, s>(p, in, adjflux, ia, tab, tab64, exptbl, \
                                                                          su, sd, ncol, nlay, an, blk, sbuf, swt,  \
                                                                          cld);                                    \
    break;
    switch (unit) {
      RRTMG_SW_SLOT(0) RRTMG_SW_SLOT(1) RRTMG_SW_SLOT(2) RRTMG_SW_SLOT(3) RRTMG_SW_SLOT(4) RRTMG_SW_SLOT(5)
      RRTMG_SW_SLOT(6) RRTMG_SW_SLOT(7) RRTMG_SW_SLOT(8) RRTMG_SW_SLOT(9) RRTMG_SW_SLOT(10) RRTMG_SW_SLOT(11)
      RRTMG_SW_SLOT(12) RRTMG_SW_SLOT(13) RRTMG_SW_SLOT(14) RRTMG_SW_SLOT(15)
      default: break;
    }
#undef RRTMG_SW_SLOT
  } else {
#define RRTMG_SW_CASE(b) \
  case b - 16: sw_band<b, R, MAXL, TOT>(p, in, adjflux, ia, tab, tab64, exptbl, su, sd, ncol, nlay, an, blk, sbuf, swt, cld); break;
    switch (unit) {
      RRTMG_SW_CASE(16) RRTMG_SW_CASE(17) RRTMG_SW_CASE(18) RRTMG_SW_CASE(19) RRTMG_SW_CASE(20) RRTMG_SW_CASE(21)
      RRTMG_SW_CASE(22) RRTMG_SW_CASE(23) RRTMG_SW_CASE(24) RRTMG_SW_CASE(25) RRTMG_SW_CASE(26) RRTMG_SW_CASE(27)
      RRTMG_SW_CASE(28) RRTMG_SW_CASE(29)
      default: break;
    }
#undef RRTMG_SW_CASE
  }
}

#ifdef RRTMG_DEFINE_COLUMN_KERNELS
// ---------------------------------------------------------------------------
// SW cloud physics of one band k (band 16 + k) of one formed layer
// (cldprop_sw, inflag = 2, rrtmg_sw_cldprop.f90:158-340): the ice extinction
// (m2/g), single-scattering albedo, asymmetry and forward fraction of Ebert
// and Curry's fit (iceflag 1; its five spectral intervals chosen by the band's
// upper limit wavenum2), of Key's Streamer table (2) or of Fu's table with its
// delta fractions (3), and those of Hu and Stamnes' liquid table (liqflag 1);
// each delta-M scaled and combined into the band's delta-scaled depth tau,
// albedo ssa and asymmetry g.  A zero depth or ice scattering becomes cldmin =
// 1e-20.  Returns false (nothing written) where the reference stops: a size
// outside its table (not-a-number sizes too), or a coefficient outside its
// physical range.
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool sw_cloud_band_optics(const SwIn& in, const double* __restrict__ T, double ciwp,
                                                     double clwp, double radice, double radliq, int k, double& tau,
                                                     double& ssa, double& g) {
  const double eps = 1.e-06, cldmin = 1.e-20;
  double ext_i = 0.0, ssa_i = 0.0, g_i = 0.0, fw_i = 0.0;
  if (ciwp != 0.0) {
    if (in.iceflag == 1) {
      if (!(radice >= 13.0 && radice <= 130.0)) return false;
      const double wn = __ldg(T + ct::WAVENUM2 + k);
      const int icx = wn > 1.43e04 ? 0 : wn > 7.7e03 ? 1 : wn > 5.3e03 ? 2 : wn > 4.0e03 ? 3 : 4;
      const double* c = T + ct::ABARI + icx;
      ext_i = __ldg(c) + __ldg(c + 5) / radice;
      ssa_i = 1. - __ldg(c + 10) - __ldg(c + 15) * radice;
      g_i = __ldg(c + 20) + __ldg(c + 25) * radice;
      if (g_i >= 1.0) g_i = 1.0 - eps;
      fw_i = g_i * g_i;
    } else {
      const int rows = in.iceflag == 2 ? 43 : 46;
      if (!(radice >= 5.0 && radice <= (in.iceflag == 2 ? 131.0 : 140.0))) return false;
      const double factor = (radice - 2.) / 3.;
      int index = (int)factor;
      if (index == rows) index = rows - 1;
      const double fint = factor - (double)index;
      if (in.iceflag == 2) {
        ext_i = cld_interp(T + ct::EXTICE2, 43, index, fint, k);
        ssa_i = cld_interp(T + ct::SSAICE2, 43, index, fint, k);
        g_i = cld_interp(T + ct::ASYICE2, 43, index, fint, k);
        fw_i = g_i * g_i;
      } else {
        ext_i = cld_interp(T + ct::EXTICE3, 46, index, fint, k);
        ssa_i = cld_interp(T + ct::SSAICE3, 46, index, fint, k);
        g_i = cld_interp(T + ct::ASYICE3, 46, index, fint, k);
        const double fdelta = cld_interp(T + ct::FDLICE3, 46, index, fint, k);
        if (fdelta < 0.0 || fdelta > 1.0) return false;
        fw_i = fdelta + 0.5 / ssa_i;
        if (fw_i > g_i) fw_i = g_i;
      }
    }
    if (ext_i < 0.0 || ssa_i > 1.0 || ssa_i < 0.0 || g_i > 1.0 || g_i < 0.0) return false;
  }
  double ext_l = 0.0, ssa_l = 0.0, g_l = 0.0, fw_l = 0.0;
  if (clwp != 0.0) {
    if (!(radliq >= 2.5 && radliq <= 60.0)) return false;
    int index = (int)(radliq - 1.5);
    if (index == 0) index = 1;
    if (index == 58) index = 57;
    const double fint = radliq - 1.5 - (double)index;
    ext_l = cld_interp(T + ct::EXTLIQ1, 58, index, fint, k);
    ssa_l = cld_interp(T + ct::SSALIQ1, 58, index, fint, k);
    if (fint < 0. && ssa_l > 1.) ssa_l = __ldg(T + ct::SSALIQ1 + (index - 1) + 58 * k);
    g_l = cld_interp(T + ct::ASYLIQ1, 58, index, fint, k);
    fw_l = g_l * g_l;
    if (ext_l < 0.0 || ssa_l > 1.0 || ssa_l < 0.0 || g_l > 1.0 || g_l < 0.0) return false;
  }
  const double tauliqorig = clwp * ext_l, tauiceorig = ciwp * ext_i;
  const double ssaliq = ssa_l * (1.0 - fw_l) / (1.0 - fw_l * ssa_l);
  const double tauliq = (1.0 - fw_l * ssa_l) * tauliqorig;
  const double ssaice = ssa_i * (1.0 - fw_i) / (1.0 - fw_i * ssa_i);
  const double tauice = (1.0 - fw_i * ssa_i) * tauiceorig;
  const double scatliq = ssaliq * tauliq;
  double scatice = ssaice * tauice;
  double t = tauliq + tauice;
  if (t == 0.0) t = cldmin;
  if (scatice == 0.0) scatice = cldmin;
  tau = t;
  ssa = (scatliq + scatice) / t;
  if (in.iceflag == 3)
    g = (1.0 / (scatliq + scatice)) *
        (scatliq * (g_l - fw_l) / (1.0 - fw_l) + scatice * ((g_i - fw_i) / (1.0 - fw_i)));
  else
    g = (scatliq * (g_l - fw_l) / (1.0 - fw_l) + scatice * (g_i - fw_i) / (1.0 - fw_i)) / (scatliq + scatice);
  return true;
}

// ---------------------------------------------------------------------------
// Clouds of the SW call (icld = 1, cloud optics given), one thread per
// (column, layer): inatm_sw's cldfrac (rrtmg_sw_rad.nomcica.f90:1065-1083);
// the non-McICA SW computes clear or overcast layers only and stops on a
// cover in (zepsec, 1 - zepsec), zepsec = 1e-6 (:533-538): such a layer of a
// sunlit column sets flag bit 1 (reported as invalid input); cldprop_sw keeps a layer's optics
// when cover >= cldmin and (ciwp + clwp >= cldmin or the band-summed depth >=
// cldmin), cldmin = 1e-20 (rrtmg_sw_cldprop.f90:120-141).  cld[0][lay][col]:
// the cover; cld[1][lay][col]: 1 where the optics are kept, else 0.
// ---------------------------------------------------------------------------
// With cloud physics (inflag = 2), a sunlit layer whose optics are formed
// gets them from sw_cloud_band_optics into opt ([tau, ssa, g][lay][col]
// [band]); a size or optical property that stops the reference sets flag bit
// 2.  On the split path (quads) every formed layer's band optics go, as the
// total-sky pass takes them, into quads[lay][col][band] = {delta-scaled depth,
// albedo, asymmetry, co-albedo}, formed in FP64 once per band instead of once
// per g-point: with given optics, cldprop_sw's delta-M scaling
// (rrtmg_sw_cldprop.f90:142-156) and 1 - w' = (1 - ssa) / (1 - f ssa); with
// the physics, its outputs and 1 - ssa.  Formed layers are few and
// scattered, so the warp computes them two at a time with a lane per band,
// instead of a lane per layer idling the others.
template <class F>
__global__ void __launch_bounds__(128) sw_cloud_kernel(SwIn in, F* __restrict__ cld, int ncol, int nlay,
                                                       unsigned* __restrict__ flags, const double* __restrict__ T,
                                                       double* __restrict__ opt, float4* __restrict__ quads) {
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  const bool here = col < ncol;  // every lane stays for the warp's shuffles
  const size_t S = (size_t)nlay * ncol;
  const size_t o = (size_t)blockIdx.y * ncol + (here ? col : 0);
  double cf = 0.0, ciwp = 0.0, clwp = 0.0;
  bool kept = false, lit = false;
  if (here) {
    cf = __ldg(in.cldfr + o);
    double tauctot = 0.0;
    if (in.taucld)
      for (int ib = 0; ib < kSwBands; ++ib) tauctot = tauctot + __ldg(in.taucld + ib + 14 * o);
    ciwp = in.cicewp ? __ldg(in.cicewp + o) : 0.0;
    clwp = in.cliqwp ? __ldg(in.cliqwp + o) : 0.0;
    const double cwp = ciwp + clwp;
    const double cldmin = 1.e-20, zepsec = 1.e-06;
    // the checks run in sunlit columns only: the reference skips the others (:500-509)
    lit = __ldg(in.coszen + col) >= 1.e-10;
    if (cf > zepsec && cf < 1.0 - zepsec && lit) atomicOr(flags, 2u);
    kept = cf >= cldmin && (cwp >= cldmin || tauctot >= cldmin);
    // unlit columns (whose outputs are zeros) keep no optics, so that the
    // total-sky pass reads only optics written here
    if (in.inflag == 2 && !lit) kept = false;
  }
  if (in.inflag == 2 || quads) {
    const int lane = threadIdx.x & 31;
    const double radice = here && in.reice ? __ldg(in.reice + o) : 0.0;
    const double radliq = here && in.reliq ? __ldg(in.reliq + o) : 0.0;
    bool failed = false;
    // two layers per pass: lanes 0-15 take the first, 16-31 the second, a
    // lane per band
    const int half = lane >> 4, band = lane & 15;
    for (unsigned todo = __ballot_sync(0xffffffffu, kept); todo;) {
      const int src0 = __ffs(todo) - 1;
      todo &= todo - 1;
      const int src1 = todo ? __ffs(todo) - 1 : -1;
      if (todo) todo &= todo - 1;
      const int src = half ? src1 : src0;
      const int from = src < 0 ? src0 : src;
      const double ci = __shfl_sync(0xffffffffu, ciwp, from), cl = __shfl_sync(0xffffffffu, clwp, from);
      const double ri = __shfl_sync(0xffffffffu, radice, from), rl = __shfl_sync(0xffffffffu, radliq, from);
      const size_t os = __shfl_sync(0xffffffffu, (unsigned long long)o, from);
      bool ok = true;
      if (src >= 0 && band < kSwBands) {
        const size_t q = 14 * os + band;
        double tau, ssa, g, cw;
        if (in.inflag == 2) {
          ok = sw_cloud_band_optics(in, T, ci, cl, ri, rl, band, tau, ssa, g);
          cw = 1.0 - ssa;
        } else {
          const double tc = __ldg(in.taucld + q), ffp = in.fsfcld ? __ldg(in.fsfcld + q) : 0.0;
          const double ssac = __ldg(in.ssacld + q), asmc = __ldg(in.asmcld + q);
          const double ffp1 = 1.0 - ffp, ffpssa = 1.0 - ffp * ssac;
          tau = ffpssa * tc;
          ssa = ffp1 * ssac / ffpssa;
          g = (asmc - ffp) / ffp1;
          cw = (1.0 - ssac) / ffpssa;
        }
        if (ok && quads) {
          quads[q] = make_float4((float)tau, (float)ssa, (float)g, (float)cw);
        } else if (ok) {
          opt[q] = tau;
          opt[14 * S + q] = ssa;
          opt[28 * S + q] = g;
        }
      }
      const unsigned bad = __ballot_sync(0xffffffffu, !ok);
      if ((lane == src0 && (bad & 0xffffu)) || (lane == src1 && (bad >> 16))) failed = true;
    }
    if (failed) {
      atomicOr(flags, 4u);
      kept = false;
    }
  }
  if (here) {
    cld[o] = (F)cf;
    cld[S + o] = kept ? (F)1 : (F)0;
  }
}

// SW finalize: band sums, outputs, heating (rrtmg_sw_rad.nomcica.f90:688-726);
// dark columns (coszen < 1e-10) get zeros (:502-510).
// suc, sdc: the clear-sky band partials of a cloudy call (its clear pass),
// else null (clear sky: the clear-sky outputs are the total ones).
__global__ void __launch_bounds__(128) sw_finalize_kernel(const double* __restrict__ su, const double* __restrict__ sd,
                                                          const double* __restrict__ plev,
                                                          const double* __restrict__ coszen, int ncol, int nlay,
                                                          double* swuflx, double* swdflx, double* swhr,
                                                          double* swuflxc, double* swdflxc, double* swhrc,
                                                          const double* __restrict__ suc = nullptr,
                                                          const double* __restrict__ sdc = nullptr) {
  // one thread per (column, level), as the LW finalize
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= ncol) return;
  const int k = blockIdx.y;
  const size_t N = (size_t)ncol;
  const bool lit = __ldg(coszen + col) >= 1.e-10;
  auto sums = [&](const double* u, const double* d, int lv, double& fu, double& fd) {
    fu = 0.0;
    fd = 0.0;
    if (!lit) return;
    for (int b = 0; b < kSwBands; ++b) {
      const size_t o = ((size_t)b * (nlay + 1) + lv) * N + col;
      fu = fu + __ldg(u + o);
      fd = fd + __ldg(d + o);
    }
  };
  const bool clear_own = suc != nullptr;
  double fu, fd, fuc, fdc;
  sums(su, sd, k, fu, fd);
  if (clear_own) sums(suc, sdc, k, fuc, fdc);
  else fuc = fu, fdc = fd;
  const size_t oo = (size_t)k * N + col;
  swuflx[oo] = fu;
  swdflx[oo] = fd;
  swuflxc[oo] = fuc;
  swdflxc[oo] = fdc;
  if (k >= 1) {
    const size_t oh = (size_t)(k - 1) * N + col;
    double h = 0.0, hc = 0.0;
    if (lit && k < nlay) {
      const double zdpgcp = c_sw.heatfac / (__ldg(plev + oo - N) - __ldg(plev + oo));
      double fu0, fd0;
      sums(su, sd, k - 1, fu0, fd0);
      h = ((fd - fu) - (fd0 - fu0)) * zdpgcp;
      if (clear_own) {
        double fuc0, fdc0;
        sums(suc, sdc, k - 1, fuc0, fdc0);
        hc = ((fdc - fuc) - (fdc0 - fuc0)) * zdpgcp;
      } else {
        hc = h;
      }
    }
    swhr[oh] = h;
    swhrc[oh] = hc;
  }
}

#endif  // RRTMG_DEFINE_COLUMN_KERNELS

}  // namespace rrtmg
