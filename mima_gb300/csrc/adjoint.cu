// Adjoint (reverse-mode) kernels of the clear-sky LW and SW paths: Jacobians
// of the heating rates, OLR and surface net fluxes with respect to layer
// temperature, specific humidity, level temperature and surface temperature,
// or vector-Jacobian products with caller cotangents.
//
// The differentiated forward is the analytic-transcendental variant of the
// FP64 path (exp / tau-transition function evaluated instead of looked up in
// the 10001-entry tables, which are piecewise constant in the optical depth).
// Per (column, g-point) thread:
//   1. the layer optics are recomputed from checkpointed per-layer inputs (the
//      setcoef fields with their d/dT and d/dq tangents, written once per
//      column by the dual prep kernels below), through the same templated gas
//      optics the forward runs, instantiated on dual numbers;
//   2. the forward recursions (rtrnmr clear branch; spcvrt adding method)
//      run once and keep their level states;
//   3. for every cotangent seed the recursions are reversed (rtrnmr: two
//      first-order sweeps; spcvrt: the reverse of the upward reflectance and
//      of the downward transmission sweeps) and the layer gradients are
//      contracted with the local tangents;
//   4. gradients are summed over the band's g-points (shared-memory staging,
//      one (column, entry) sum per lane; FP64 sums, or compensated FP32 sums
//      in the split adjoint) into FP64 per-band partials, which a finalize
//      kernel weights and sums over bands.
#include <cuda_runtime.h>

#include "adjoint.h"
#include "dual.cuh"
#include "kernels.cuh"
#include "launch.h"

namespace rrtmg {

using D2 = Dual<double>;

// ---------------------------------------------------------------------------
// LW dual prep: inatm + setcoef (rrtmg_lw_rad.nomcica.f90:572-901,
// rrtmg_lw_setcoef.f90:31-415) per layer with tangents d/dtlay and d/dq of the
// same layer; Planck functions with their temperature slopes; secdiff
// (rrtmg_lw_rtrnmr.f90:271-279) with d secdiff / d q of every layer through
// the column water vapour pwvcm.
// ---------------------------------------------------------------------------
// F is the checkpoint type and the arithmetic type (duals Dual<F>): the FP64
// adjoint computes in double, the split adjoint in float, with the same
// expressions in the same order.
template <class F>
__global__ void __launch_bounds__(128) adj_lw_prep_kernel(LwIn in, AdjLwWorkT<F> w, const F* __restrict__ totplnk,
                                                          int ncol, int nlay) {
  using T = F;
  using DT = Dual<T>;
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= ncol) return;
  const LwConst& C = c_lw;
  const T amd = (T)28.9660, amw = (T)18.0160, amdw = (T)1.607793, amdo = (T)0.603428;
  const T stpfac = (T)(296. / 1013.);
  const T one = (T)1., e20 = (T)1.e-20, e32 = (T)1.e-32, zero = (T)0.;
  const size_t N = (size_t)ncol;
  const size_t fstride = (size_t)nlay * N;
  auto A = [&](const double* p, int l) { return (T)__ldg(p + (size_t)col + N * (size_t)(l - 1)); };
  auto P = [&](int ind, int b) { return __ldg(totplnk + (ind - 1) + 181 * (b - 1)); };

  const T tbound = (T)__ldg(in.tsfc + col);
  T pz_prev = A(in.plev, 1);
  const T pz0 = pz_prev;
  const T tz0 = A(in.tlev, 1);
  const int indbound = clampi((int)(tbound - (T)159.), 1, 180);
  const T tbndfrac = tbound - (T)159. - (T)indbound;
  const int indlev0 = clampi((int)(tz0 - (T)159.), 1, 180);
  const T t0frac = tz0 - (T)159. - (T)indlev0;
  for (int b = 1; b <= 16; ++b) {
    const T semiss = in.emis ? (T)__ldg(in.emis + col + N * (b - 1)) : one;
    T slope = P(indbound + 1, b) - P(indbound, b);
    w.pbnd_v[(b - 1) * N + col] = semiss * (P(indbound, b) + tbndfrac * slope);
    w.pbnd_t[(b - 1) * N + col] = semiss * slope;
    slope = P(indlev0 + 1, b) - P(indlev0, b);
    w.plev_v[((size_t)(b - 1) * (nlay + 1)) * N + col] = P(indlev0, b) + t0frac * slope;
    w.plev_t[((size_t)(b - 1) * (nlay + 1)) * N + col] = slope;
  }

  T amttl = zero, wvttl = zero;
  int laytrop = 0;
  for (int l = 1; l <= nlay; ++l) {
    const T pavel = A(in.play, l);
    const DT tavel(A(in.tlay, l), one, zero);
    const T pz_l = A(in.plev, l + 1), tz_l = A(in.tlev, l + 1);
    const DT h2o(A(in.h2o, l), zero, one);
    DT wk1 = (h2o / (one - h2o)) * amdw;
    const T wk2 = A(in.co2, l);
    const T wk3 = A(in.o3, l) * amdo;
    const T wk4 = in.n2o ? A(in.n2o, l) : zero;
    const T wk6 = in.ch4 ? A(in.ch4, l) : zero;
    const T wk7 = in.o2 ? A(in.o2, l) : zero;
    const DT amm = (one - wk1) * amd + wk1 * amw;
    const DT coldry = (pz_prev - pz_l) * (T)1.e3 * (T)C.avogad / ((T)1.e2 * (T)C.grav * amm * (one + wk1));
    const T summol = wk2 + wk3 + wk4 + zero + wk6 + wk7;
    const DT wbrodl = coldry * (one - summol);
    wk1 = coldry * wk1;
    const DT cwk2 = coldry * wk2, cwk3 = coldry * wk3, cwk4 = coldry * wk4, cwk6 = coldry * wk6,
             cwk7 = coldry * wk7;
    amttl = amttl + coldry.v + wk1.v;
    wvttl = wvttl + wk1.v;
    // d(wvttl)/dq_l and d(amttl)/dq_l, for d pwvcm / dq_l below
    w.dsec[(size_t)(l - 1) * N + col] = wk1.q;
    w.dsec[fstride + (size_t)(l - 1) * N + col] = coldry.q + wk1.q;
    const DT wx1 = in.ccl4 ? coldry * A(in.ccl4, l) * e20 : coldry * zero;
    const DT wx2 = in.cfc11 ? coldry * A(in.cfc11, l) * e20 : coldry * zero;
    const DT wx3 = in.cfc12 ? coldry * A(in.cfc12, l) * e20 : coldry * zero;
    const DT wx4 = in.cfc22 ? coldry * A(in.cfc22, l) * e20 : coldry * zero;

    const int indlay = clampi((int)(tavel.v - (T)159.), 1, 180);
    const T tlayfrac = tavel.v - (T)159. - (T)indlay;
    const int indlev = clampi((int)(tz_l - (T)159.), 1, 180);
    const T tlevfrac = tz_l - (T)159. - (T)indlev;
    for (int b = 1; b <= 16; ++b) {
      const T sl = P(indlay + 1, b) - P(indlay, b);
      const T sv = P(indlev + 1, b) - P(indlev, b);
      w.play_v[((size_t)(b - 1) * nlay + (l - 1)) * N + col] = P(indlay, b) + tlayfrac * sl;
      w.play_t[((size_t)(b - 1) * nlay + (l - 1)) * N + col] = sl;
      w.plev_v[((size_t)(b - 1) * (nlay + 1) + l) * N + col] = P(indlev, b) + tlevfrac * sv;
      w.plev_t[((size_t)(b - 1) * (nlay + 1) + l) * N + col] = sv;
    }

    const T plog = log(pavel);
    const int jp = clampi((int)((T)36. - (T)5 * (plog + (T)0.04)), 1, 58);
    const int jp1 = jp + 1;
    const T fp = (T)5. * ((T)C.preflog[jp - 1] - plog);
    const int jt = clampi((int)((T)3. + (tavel.v - (T)C.tref[jp - 1]) / (T)15.), 1, 4);
    const DT ft = ((tavel - (T)C.tref[jp - 1]) / (T)15.) - (T)(jt - 3);
    const int jt1 = clampi((int)((T)3. + (tavel.v - (T)C.tref[jp1 - 1]) / (T)15.), 1, 4);
    const DT ft1 = ((tavel - (T)C.tref[jp1 - 1]) / (T)15.) - (T)(jt1 - 3);
    const DT water = wk1 / coldry;
    const DT scalefac = (pavel * stpfac) / tavel;
    DT forfac, forfrac, selffac, selffrac(zero), minorfrac, factor;
    int indfor, indself = 1, indminor;
    if (plog > (T)4.56) {
      laytrop = laytrop + 1;
      forfac = scalefac / (one + water);
      factor = ((T)332.0 - tavel) / (T)36.0;
      indfor = min(2, max(1, (int)factor.v));
      forfrac = factor - (T)indfor;
      selffac = water * forfac;
      factor = (tavel - (T)188.0) / (T)7.2;
      indself = min(9, max(1, (int)factor.v - 7));
      selffrac = factor - (T)(indself + 7);
    } else {
      forfac = scalefac / (one + water);
      factor = (tavel - (T)188.0) / (T)36.0;
      indfor = 3;
      forfrac = factor - one;
      selffac = water * forfac;
    }
    const DT scaleminor = pavel / tavel;
    const DT scaleminorn2 = (pavel / tavel) * (wbrodl / (coldry + wk1));
    factor = (tavel - (T)180.8) / (T)7.2;
    indminor = min(18, max(1, (int)factor.v));
    minorfrac = factor - (T)indminor;

    const DT colh2o = e20 * wk1;
    DT colco2 = e20 * cwk2, colo3 = e20 * cwk3, coln2o = e20 * cwk4;
    DT colco = coldry * zero, colch4 = e20 * cwk6;
    const DT colo2 = e20 * cwk7;
    if (colco2.v == zero) colco2 = e32 * coldry;
    if (colo3.v == zero) colo3 = e32 * coldry;
    if (coln2o.v == zero) coln2o = e32 * coldry;
    if (colco.v == zero) colco = e32 * coldry;
    if (colch4.v == zero) colch4 = e32 * coldry;
    const DT colbrd = e20 * wbrodl;
    const T compfp = one - fp;
    const size_t o = (size_t)(l - 1) * N + col;
    auto put = [&](int fld, const DT& x) {
      const size_t i = (size_t)fld * fstride + o;
      w.fv[i] = x.v;
      w.ft[i] = x.t;
      w.fq[i] = x.q;
    };
    put(LF_PAVEL, DT(pavel));
    put(LF_COLDRY, coldry);
    put(LF_COLH2O, colh2o);
    put(LF_COLCO2, colco2);
    put(LF_COLO3, colo3);
    put(LF_COLN2O, coln2o);
    put(LF_COLCO, colco);
    put(LF_COLCH4, colch4);
    put(LF_COLO2, colo2);
    put(LF_COLBRD, colbrd);
    put(LF_FAC10, compfp * ft);
    put(LF_FAC00, compfp * (one - ft));
    put(LF_FAC11, fp * ft1);
    put(LF_FAC01, fp * (one - ft1));
    put(LF_SELFFAC, colh2o * selffac);
    put(LF_SELFFRAC, selffrac);
    put(LF_FORFAC, colh2o * forfac);
    put(LF_FORFRAC, forfrac);
    put(LF_MINORFRAC, minorfrac);
    put(LF_SCALEMINOR, scaleminor);
    put(LF_SCALEMINORN2, scaleminorn2);
    put(LF_WX1, wx1);
    put(LF_WX2, wx2);
    put(LF_WX3, wx3);
    put(LF_WX4, wx4);
    w.idx[o] = pack_idx(jp, jt, jt1, indself, indfor, indminor);
    w.hs[o] = (double)((T)C.heatfac / (pz_prev - pz_l));
    pz_prev = pz_l;
  }
  w.laytrop[col] = laytrop;
  // secdiff(pwvcm) and d secdiff / d q_l = secdiff'(pwvcm) pwvcm (dwv_l / wvttl - dam_l / amttl)
  const T wvsh = (amw * wvttl) / (amd * amttl);
  const T pwvcm = wvsh * ((T)1.e3 * pz0) / ((T)1.e2 * (T)C.grav);
  const T a0[16] = {(T)1.66, (T)1.55, (T)1.58, (T)1.66, (T)1.54, (T)1.454, (T)1.89, (T)1.33,
                    (T)1.668, (T)1.66, (T)1.66, (T)1.66, (T)1.66, (T)1.66, (T)1.66, (T)1.66};
  const T a1[16] = {(T)0.00, (T)0.25, (T)0.22, (T)0.00, (T)0.13, (T)0.446, (T)-0.10, (T)0.40,
                    (T)-0.006, 0, 0, 0, 0, 0, 0, 0};
  const T a2[16] = {(T)0.00, (T)-12.0, (T)-11.7, (T)0.00, (T)-0.72, (T)-0.243, (T)0.19, (T)-0.062,
                    (T)0.414, 0, 0, 0, 0, 0, 0, 0};
  T dsdp[16];
  for (int b = 1; b <= 16; ++b) {
    T sv, d = zero;
    if (b == 1 || b == 4 || b >= 10) {
      sv = (T)1.66;
    } else {
      const T e = exp(a2[b - 1] * pwvcm);
      sv = a0[b - 1] + a1[b - 1] * e;
      d = a1[b - 1] * a2[b - 1] * e;
      if (sv > (T)1.80) { sv = (T)1.80; d = zero; }
      if (sv < (T)1.50) { sv = (T)1.50; d = zero; }
    }
    w.secdiff[(b - 1) * N + col] = sv;
    dsdp[b - 1] = d;
  }
  // dsec currently holds dwv_l (rows 0..nlay-1) and dam_l (rows nlay..2nlay-1)
  // in its first two band planes; overwrite band by band from the top band
  // down so that the two source planes are read before band 1 and 2 reuse them.
  for (int l = 1; l <= nlay; ++l) {
    const size_t o = (size_t)(l - 1) * N + col;
    const T dp = pwvcm * ((T)w.dsec[o] / wvttl - (T)w.dsec[fstride + o] / amttl);
    for (int b = 16; b >= 1; --b) w.dsec[(size_t)(b - 1) * fstride + o] = dsdp[b - 1] * dp;
  }
}

// ---------------------------------------------------------------------------
// Sums over the g-points of a band of per-lane gradient entries: entries are
// staged in shared memory W at a time (rows padded to kRow), then lane
// (cs, sl) sums entry sl of column sub-index cs over the band's NG lanes in g
// order.  FP64 entries are summed in FP64; FP32 entries (split adjoint) with
// the compensated TwoSum accumulation of the forward solvers' GSum, to FP64
// accuracy on the FP32 pipe.  Warp-uniform calls only.
// ---------------------------------------------------------------------------
template <int W, int NG, class TS = double>
struct GRed {
  TS* buf;  // this warp's [W][kRow]
  int lane, n, first;
  __device__ __forceinline__ void put(TS v) { buf[n * kRow + lane] = v; }
  template <class Store>
  __device__ __forceinline__ void flush(Store&& st) {
    __syncwarp();
    const int sl = lane % W, cs = lane / W;
    if (sl < n && cs < 32 / W) {
      const TS* row = buf + sl * kRow + cs * W;
      if constexpr (sizeof(TS) == 4) {
        float s = 0.f, c = 0.f;
#pragma unroll 2
        for (int g = 0; g < NG; ++g) {
          const float x = row[g], t = __fadd_rn(s, x), bv = __fsub_rn(t, s);
          c = __fadd_rn(c, __fadd_rn(__fsub_rn(s, __fsub_rn(t, bv)), __fsub_rn(x, bv)));
          s = t;
        }
        st(first + sl, cs, (double)s + (double)c);
      } else {
        double acc = 0.0;
#pragma unroll
        for (int g = 0; g < NG; ++g) acc += (double)row[g];
        st(first + sl, cs, acc);
      }
    }
    __syncwarp();
    first += n;
    n = 0;
  }
  template <class Store>
  __device__ __forceinline__ void next(Store&& st) {
    if (++n == W) flush(st);
  }
};
constexpr int kRedDoubles = (kBlock / 32) * 16 * kRow;

// Dual view of the checkpointed setcoef fields of one (layer, column).
template <class R>
struct LwDualView {
  const R *fv, *ft, *fq;
  size_t fstride, o;
  __device__ __forceinline__ Dual<R> operator()(int fld) const {
    const size_t i = (size_t)fld * fstride + o;
    return Dual<R>(__ldg(fv + i), __ldg(ft + i), __ldg(fq + i));
  }
};

// ---------------------------------------------------------------------------
// LW reverse sweep of one g-point (rrtmg_lw_rtrnmr.f90:505-616 downward,
// :628-713 upward, clear branch, analytic transcendentals).
//   Recursions per g:  D_{l-1} = t_l D_l + sd_l,  U_l = t_l U_{l-1} + su_l,
//   U_0 = fracs_1 * emis * B(tsfc) + (1 - emis) D_0,  t = 1 - atr,
//   sd = atr * bbd, su = atr * bbu.
//   Outputs per band (weight wtdiff * delwave * fluxfac applied at finalize):
//   div_k = (U_{k-1} - U_k) - (D_{k-1} - D_k) for the heating of layer k,
//   OLR = U_nlay, surface net = U_0 - D_0.
//   Seed c: Phi = sum_k c_k div_k + c_olr U_nlay + c_sfc (U_0 - D_0).
//   Adjoints: lamU_nlay = aU_nlay, lamU_m = aU_m + t_{m+1} lamU_{m+1};
//             lamD_0 = aD_0 + (1 - emis) lamU_0, lamD_m = aD_m + t_m lamD_{m-1};
//   dPhi/dt_l = lamU_l U_{l-1} + lamD_{l-1} D_l, dPhi/dsd_l = lamD_{l-1},
//   dPhi/dsu_l = lamU_l, dPhi/drad0 = lamU_0, then the chain rule through the
//   layer tangents (tlay, q, secdiff, tlev below / above).
// ---------------------------------------------------------------------------
template <int B, class R, int MAXL>
__device__ __forceinline__ void lw_adj_band(const LwIn& in, const AdjLwWorkT<R>& w, const R* __restrict__ tab,
                                            const double* __restrict__ cot, int nseed, int ncol, int nlay, int blk,
                                            double* sred) {
  using DR = Dual<R>;
  constexpr int NG = lw_ng(B);
  // lanes per column as in the forward solvers (packed on the split path)
  constexpr int W = split_lanes(NG, sizeof(R) == 4);
  constexpr int CPW = 32 / W;
  constexpr int CPB = (kBlock / 32) * CPW;
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int lane_col = wib * CPW + lane / W, g = lane % W;
  const int col = blk * CPB + lane_col;
  const bool valid = lane < CPW * W && col < ncol;
  const int c = valid ? col : (col < ncol ? col : ncol - 1);
  const int gg = g < NG ? g : NG - 1;
  const size_t N = (size_t)ncol;
  const size_t fstride = (size_t)nlay * N;
  const int lt = w.laytrop[c];
  const R secdiff = w.secdiff[(B - 1) * N + c];
  const R rec_6 = (R)0.166667;
  const int E = 3 * nlay + 3;

  // Layer state (index l-1) and level radiances.  The tangents of a layer
  // are written together and read together, so they sit side by side in
  // records (one wide local access each):
  //   tq[k].T = {t, sd, su}/dtlay and dsd/dtlev below,
  //   tq[k].Q = {t, sd, su}/dq and dsu/dtlev above,
  //   ts[k]   = {t, sd, su}/dsecdiff.
  struct TQ {
    Quad<R> T, Q;
  };
  Pair2<R> ab[MAXL];  // {atr, bbu}
  TQ tq[MAXL];
  Quad<R> ts[MAXL];
  R Dl[MAXL + 1], Ul[MAXL + 1], nu[MAXL + 1];
  R ck[MAXL + 1];                  // seed cotangents of the layer divergences (index k = 1..nlay; ck[0] = 0)

  // 1. layer optics with tangents (recomputed from the checkpointed fields) and
  //    the downward recursion
  R radld = (R)0;
  Dl[nlay] = (R)0;
  DR fr1;
  for (int lev = nlay; lev >= 1; --lev) {
    const int k = lev - 1;
    const size_t o = (size_t)k * N + c;
    const Idx ix = unpack_idx(__ldg(w.idx + o));
    LwDualView<R> L{w.fv, w.ft, w.fq, fstride, o};
    DR taug, fracs;
    lw_gas<B, DR>(c_lw, lw_rconst<R>(), L, ix, lev <= lt, gg, tab, taug, fracs);
    const R ta = in.tauaer ? (R)__ldg(in.tauaer + c + N * ((size_t)k + (size_t)nlay * (B - 1))) : (R)0;
    const R taut = taug.v + ta;
    R od = secdiff * taut, odT = secdiff * taug.t, odQ = secdiff * taug.q, odS = taut;
    if (od < (R)0) od = odT = odQ = odS = (R)0;
    R a, a_d, tf, tf_d;
    if (od <= (R)0.06) {
      a = od - (R)0.5 * od * od;
      a_d = (R)1 - od;
      tf = rec_6 * od;
      tf_d = rec_6;
    } else {
      const R e = exp(-od), om = (R)1 - e;
      a = om;
      a_d = e;
      if (sizeof(R) == 4 && od < (R)1) {
        // tf = 1 - 2 (1/od - 1/(e^od - 1)) by its Bernoulli series: the closed
        // form cancels to a few digits in FP32 for small od
        const R x2 = od * od;
        tf = od * ((R)(1. / 6) - x2 * ((R)(1. / 360) - x2 * ((R)(1. / 15120) - x2 * (R)(1. / 604800))));
        tf_d = (R)(1. / 6) - x2 * ((R)(1. / 120) - x2 * ((R)(1. / 3024) - x2 * (R)(1. / 86400)));
      } else {
        const R iod = (R)1 / od, iom = (R)1 / om;
        tf = (R)1 - (R)2 * (iod - e * iom);
        tf_d = (R)2 * (iod * iod) - (R)2 * e * (iom * iom);
      }
    }
    const R plf = fracs.v;
    const size_t ol = ((size_t)(B - 1) * nlay + k) * N + c;
    const R blay = __ldg(w.play_v + ol), blay_t = __ldg(w.play_t + ol);
    const size_t ou = ((size_t)(B - 1) * (nlay + 1) + lev) * N + c, od_ = ou - N;
    const R pup = __ldg(w.plev_v + ou), pup_t = __ldg(w.plev_t + ou);
    const R pdn = __ldg(w.plev_v + od_), pdn_t = __ldg(w.plev_t + od_);
    const R dpup = pup - blay, dpdn = pdn - blay;
    const R bd = plf * (blay + tf * dpdn), bu = plf * (blay + tf * dpup);
    ab[k] = Pair2<R>{a, bu};
    auto tang = [&](R odx, R dplf, R dbl, R& ot, R& osd, R& osu) {
      const R da = a_d * odx, dtf = tf_d * odx;
      const R dbd = dplf * (blay + tf * dpdn) + plf * (dbl + dtf * dpdn - tf * dbl);
      const R dbu = dplf * (blay + tf * dpup) + plf * (dbl + dtf * dpup - tf * dbl);
      ot = -da;
      osd = da * bd + a * dbd;
      osu = da * bu + a * dbu;
    };
    TQ r;
    Quad<R> rs;
    tang(odT, fracs.t, blay_t, r.T.a, r.T.b, r.T.c);
    tang(odQ, fracs.q, (R)0, r.Q.a, r.Q.b, r.Q.c);
    tang(odS, (R)0, (R)0, rs.a, rs.b, rs.c);
    r.T.d = a * plf * tf * pdn_t;
    r.Q.d = a * plf * tf * pup_t;
    rs.d = (R)0;
    tq[k] = r;
    ts[k] = rs;
    radld = radld + (bd - radld) * a;
    Dl[k] = radld;
    if (lev == 1) fr1 = fracs;
  }
  // 2. upward recursion
  const R pb = __ldg(w.pbnd_v + (B - 1) * N + c), pb_t = __ldg(w.pbnd_t + (B - 1) * N + c);
  const R semiss = in.emis ? (R)__ldg(in.emis + c + N * (B - 1)) : (R)1;
  const R reflect = (R)1 - semiss;
  Ul[0] = fr1.v * pb + reflect * Dl[0];
  for (int l = 1; l <= nlay; ++l) {
    const Pair2<R> x = ab[l - 1];
    Ul[l] = Ul[l - 1] + (x.b - Ul[l - 1]) * x.a;
  }

  // 3. reverse sweeps, one cotangent seed at a time.  With c_k the cotangent of
  //    div_k (c_0 = c_{nlay+1} = 0) the adjoints are carried as
  //      nu_m  = lamU_m + c_m:  nu_nlay = c_olr,
  //              nu_m = atr_{m+1} c_{m+1} + t_{m+1} nu_{m+1} (+ c_sfc at m = 0);
  //      rho_m = lamD_m + c_{m+1}: rho_0 = -c_sfc + (1 - emis) lamU_0,
  //              rho_m = atr_m c_m + t_m rho_{m-1};
  //    the same recursions as for lamU, lamD without the cancellation of
  //    c_{m+1} - t_{m+1} c_{m+1} (which costs FP32 its digits for thin layers).
  const int wcol0 = blk * CPB + wib * CPW;
  for (int s = 0; s < nseed; ++s) {
    ck[0] = (R)0;
    for (int kk = 1; kk <= nlay; ++kk) {
      const double hs = __ldg(w.hs + (size_t)(kk - 1) * N + c);
      ck[kk] = (R)(cot ? __ldg(cot + (size_t)(kk - 1) * N + c) * hs : (s == kk - 1 ? hs : 0.0));
    }
    const R colr = (R)(cot ? __ldg(cot + (size_t)nlay * N + c) : (s == nlay ? 1.0 : 0.0));
    const R csfc = (R)(cot ? __ldg(cot + (size_t)(nlay + 1) * N + c) : (s == nlay + 1 ? 1.0 : 0.0));
    nu[nlay] = colr;
    for (int m = nlay - 1; m >= 0; --m) {
      const R am = ab[m].a;
      nu[m] = am * ck[m + 1] + ((R)1 - am) * nu[m + 1] + (m == 0 ? csfc : (R)0);
    }
    GRed<W, NG, R> red{(R*)sred + wib * W * kRow, (int)(threadIdx.x & 31), 0, 0};
    auto store = [&](int e, int cs, double v) {
      const int cc = wcol0 + cs;
      if (cc < ncol) w.part[(((size_t)(B - 1) * nseed + s) * E + e) * N + cc] = v;
    };
    const R lamU0 = nu[0] - ck[0];
    R rho = -csfc + reflect * lamU0;  // rho_0
    R gS = (R)0, accLev = (R)0;
    for (int l = 1; l <= nlay; ++l) {
      const int k = l - 1;
      const R lamU = nu[l] - ck[l];
      const R lamD = rho - ck[l];  // lamD_{l-1} = rho_{l-1} - c_l
      const R gt = lamU * Ul[l - 1] + lamD * Dl[l];
      const R gsd = lamD, gsu = lamU;
      const TQ r = tq[k];
      const Quad<R> rs = ts[k];
      R gT = gt * r.T.a + gsd * r.T.b + gsu * r.T.c;
      R gQ = gt * r.Q.a + gsd * r.Q.b + gsu * r.Q.c;
      if (l == 1) {
        gT += lamU0 * fr1.t * pb;
        gQ += lamU0 * fr1.q * pb;
      }
      gS += gt * rs.a + gsd * rs.b + gsu * rs.c;
      const R gLev = accLev + gsd * r.T.d;
      accLev = gsu * r.Q.d;
      red.put(gT);
      red.next(store);
      red.put(gQ);
      red.next(store);
      red.put(gLev);
      red.next(store);
      const R ak = ab[k].a;
      rho = ak * ck[l] + ((R)1 - ak) * rho;  // rho_l
    }
    red.put(accLev);
    red.next(store);
    red.put(lamU0 * fr1.v * pb_t);
    red.next(store);
    red.put(gS);
    red.next(store);
    if (red.n) red.flush(store);
  }
}

// Minimum resident blocks per SM asked of the register allocator for the
// FP32/FP64-split adjoint kernels (a VJP at 32768 columns x 40 layers on
// GB300 with packed lanes: 28.1 ms at 6, 24.0 ms at 8, 23.1 ms at 10,
// 25.7 ms at 12); the FP64 ones: 1.
#ifndef RRTMG_SPLIT_ADJ_MINB
#define RRTMG_SPLIT_ADJ_MINB 10
#endif
#ifndef RRTMG_SPLIT_ADJ_LW_MINB
#define RRTMG_SPLIT_ADJ_LW_MINB RRTMG_SPLIT_ADJ_MINB
#endif
#ifndef RRTMG_SPLIT_ADJ_SW_MINB
#define RRTMG_SPLIT_ADJ_SW_MINB RRTMG_SPLIT_ADJ_MINB
#endif

template <class R, int MAXL>
__global__ void __launch_bounds__(kBlock, sizeof(R) == 4 ? RRTMG_SPLIT_ADJ_LW_MINB : 1) lw_adj_kernel(LwIn in, AdjLwWorkT<R> w, const R* __restrict__ tab,
                                                        const double* __restrict__ cot, int nseed, int ncol,
                                                        int nlay) {
  // FP32 entries take half the staging room: a smaller shared-memory carve-out
  // leaves the split kernels more L1 for their per-thread arrays
  __shared__ double sred[sizeof(R) == 4 ? kRedDoubles / 2 : kRedDoubles];
  int blk = blockIdx.x, band = 0;
  for (; band < kLwBands; ++band) {
    const int nb = lw_blocks_for_band(split_lanes(c_lw.band[band].ng, sizeof(R) == 4), ncol);
    if (blk < nb) break;
    blk -= nb;
  }
#define RRTMG_LW_ADJ_CASE(b) \
  case b - 1: lw_adj_band<b, R, MAXL>(in, w, tab, cot, nseed, ncol, nlay, blk, sred); break;
  switch (band) {
    RRTMG_LW_ADJ_CASE(1) RRTMG_LW_ADJ_CASE(2) RRTMG_LW_ADJ_CASE(3) RRTMG_LW_ADJ_CASE(4) RRTMG_LW_ADJ_CASE(5)
    RRTMG_LW_ADJ_CASE(6) RRTMG_LW_ADJ_CASE(7) RRTMG_LW_ADJ_CASE(8) RRTMG_LW_ADJ_CASE(9) RRTMG_LW_ADJ_CASE(10)
    RRTMG_LW_ADJ_CASE(11) RRTMG_LW_ADJ_CASE(12) RRTMG_LW_ADJ_CASE(13) RRTMG_LW_ADJ_CASE(14) RRTMG_LW_ADJ_CASE(15)
    RRTMG_LW_ADJ_CASE(16)
    default: break;
  }
#undef RRTMG_LW_ADJ_CASE
}

// ---------------------------------------------------------------------------
// SW dual prep: inatm_sw + setcoef_sw (rrtmg_sw_rad.nomcica.f90:761-1101,
// rrtmg_sw_setcoef.f90:30-286) per layer with tangents d/dtlay and d/dq of the
// same layer, and the solar-source layer of every band (as the forward prep).
// ---------------------------------------------------------------------------
template <class F>
__global__ void __launch_bounds__(128) adj_sw_prep_kernel(SwIn in, AdjSwWorkT<F> w, int ncol, int nlay) {
  // F is the checkpoint and the arithmetic type, as in adj_lw_prep_kernel
  using T = F;
  using DT = Dual<T>;
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= ncol) return;
  const SwConst& C = c_sw;
  const T amd = (T)28.9660, amw = (T)18.0160, amdw = (T)1.607793, amdo = (T)0.603428;
  const T stpfac = (T)(296. / 1013.);
  const T one = (T)1., e20 = (T)1.e-20, e32 = (T)1.e-32, zero = (T)0.;
  const size_t N = (size_t)ncol;
  const size_t fstride = (size_t)nlay * N;
  auto A = [&](const double* p, int l) { return (T)__ldg(p + (size_t)col + N * (size_t)(l - 1)); };
  T pz_prev = A(in.plev, 1);
  int laytrop = 0;
  for (int l = 1; l <= nlay; ++l) {
    const T pavel = A(in.play, l);
    const DT tavel(A(in.tlay, l), one, zero);
    const T pz_l = A(in.plev, l + 1);
    const DT h2o(A(in.h2o, l), zero, one);
    DT wk1 = (h2o / (one - h2o)) * amdw;
    const T wk2 = A(in.co2, l);
    const T wk3 = A(in.o3, l) * amdo;
    const T wk4 = in.n2o ? A(in.n2o, l) : zero;
    const T wk6 = in.ch4 ? A(in.ch4, l) : zero;
    const T wk7 = in.o2 ? A(in.o2, l) : zero;
    const DT amm = (one - wk1) * amd + wk1 * amw;
    const DT coldry = (pz_prev - pz_l) * (T)1.e3 * (T)C.avogad / ((T)1.e2 * (T)C.grav * amm * (one + wk1));
    wk1 = coldry * wk1;
    const DT cwk2 = coldry * wk2, cwk3 = coldry * wk3, cwk4 = coldry * wk4, cwk6 = coldry * wk6,
             cwk7 = coldry * wk7;
    const T plog = log(pavel);
    const int jp = clampi((int)((T)36. - (T)5 * (plog + (T)0.04)), 1, 58);
    const int jp1 = jp + 1;
    const T fp = (T)5. * ((T)C.preflog[jp - 1] - plog);
    const int jt = clampi((int)((T)3. + (tavel.v - (T)C.tref[jp - 1]) / (T)15.), 1, 4);
    const DT ft = ((tavel - (T)C.tref[jp - 1]) / (T)15.) - (T)(jt - 3);
    const int jt1 = clampi((int)((T)3. + (tavel.v - (T)C.tref[jp1 - 1]) / (T)15.), 1, 4);
    const DT ft1 = ((tavel - (T)C.tref[jp1 - 1]) / (T)15.) - (T)(jt1 - 3);
    const DT water = wk1 / coldry;
    const DT scalefac = (pavel * stpfac) / tavel;
    DT forfac, forfrac, selffac(zero), selffrac(zero), factor;
    int indfor, indself = 0;
    if (plog > (T)4.56) {
      laytrop = laytrop + 1;
      forfac = scalefac / (one + water);
      factor = ((T)332.0 - tavel) / (T)36.0;
      indfor = min(2, max(1, (int)factor.v));
      forfrac = factor - (T)indfor;
      selffac = water * forfac;
      factor = (tavel - (T)188.0) / (T)7.2;
      indself = min(9, max(1, (int)factor.v - 7));
      selffrac = factor - (T)(indself + 7);
    } else {
      forfac = scalefac / (one + water);
      factor = (tavel - (T)188.0) / (T)36.0;
      indfor = 3;
      forfrac = factor - one;
    }
    const DT colh2o = e20 * wk1;
    DT colco2 = e20 * cwk2, colch4 = e20 * cwk6, colo2 = e20 * cwk7, coln2o = e20 * cwk4;
    const DT colo3 = e20 * cwk3;
    const DT colmol = e20 * coldry + colh2o;
    if (colco2.v == zero) colco2 = e32 * coldry;
    if (coln2o.v == zero) coln2o = e32 * coldry;
    if (colch4.v == zero) colch4 = e32 * coldry;
    if (colo2.v == zero) colo2 = e32 * coldry;
    const T compfp = one - fp;
    const size_t o = (size_t)(l - 1) * N + col;
    auto put = [&](int fld, const DT& x) {
      const size_t i = (size_t)fld * fstride + o;
      w.fv[i] = x.v;
      w.ft[i] = x.t;
      w.fq[i] = x.q;
    };
    put(SF_COLH2O, colh2o);
    put(SF_COLCO2, colco2);
    put(SF_COLO3, colo3);
    put(SF_COLCH4, colch4);
    put(SF_COLO2, colo2);
    put(SF_COLMOL, colmol);
    put(SF_FAC10, compfp * ft);
    put(SF_FAC00, compfp * (one - ft));
    put(SF_FAC11, fp * ft1);
    put(SF_FAC01, fp * (one - ft1));
    put(SF_SELFFAC, selffac);
    put(SF_SELFFRAC, selffrac);
    put(SF_FORFAC, forfac);
    put(SF_FORFRAC, forfrac);
    w.idx[o] = pack_idx(jp, jt, jt1, indself, indfor, 1);
    w.hs[o] = (double)((T)C.heatfac / (pz_prev - pz_l));
    pz_prev = pz_l;
  }
  w.laytrop[col] = laytrop;
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
}

template <class R>
struct SwDualView {
  const R *fv, *ft, *fq;
  size_t fstride, o;
  __device__ __forceinline__ Dual<R> operator()(int fld) const {
    const size_t i = (size_t)fld * fstride + o;
    return Dual<R>(__ldg(fv + i), __ldg(ft + i), __ldg(fq + i));
  }
};

// ---------------------------------------------------------------------------
// SW reverse sweep of one g-point (spcvrt_sw clear stream,
// rrtmg_sw_spcvrt.f90:296-618, reftra_sw and vrtqdr_sw, analytic
// transcendentals).  Top-down index j (0 = top of atmosphere, klev = surface):
//   layer j: reflectance R, diffuse Rd, transmittance T, diffuse Td, direct Tx;
//   downward:  tb_{j+1} = Tx_j tb_j,  z = 1 / (1 - Rd_j rn_j),
//              tn_{j+1} = tb_j T_j + Td_j ((tn_j - tb_j) + tb_j R_j rn_j) z,
//              rn_{j+1} = Rd_j + Td_j^2 rn_j z            (tb_0 = tn_0 = 1, rn_0 = 0);
//   upward:    z = 1 / (1 - pd_{j+1} Rd_j),
//              pu_j = R_j + Td_j ((T_j - Tx_j) pd_{j+1} + Tx_j pu_{j+1}) z,
//              pd_j = Rd_j + Td_j^2 pd_{j+1} z           (pu, pd at the surface: albedos);
//   fluxes:    z = 1 / (1 - rn pd),  fu = (tb pu + (tn - tb) pd) z,
//              fd = tb + (tn - tb + tb pu rn) z,  net = zinc (fd - fu).
// The reverse carries the adjoints of (pu, pd) downward from the top and of
// (tb, tn, rn) upward from the surface, collecting d Phi / d(R, Rd, T, Td, Tx)
// of every layer, then contracts them with the layer tangents.
// ---------------------------------------------------------------------------
template <int B, class R, int MAXL>
__device__ __forceinline__ void sw_adj_band(const SwIn& in, const AdjSwWorkT<R>& w, double adjflux, int iaer,
                                            const R* __restrict__ tab, const double* __restrict__ tab64,
                                            const double* __restrict__ cot, int nseed, int ncol, int nlay, int blk,
                                            double* sred) {
  using DR = Dual<R>;
  constexpr int NG = sw_ng(B);
  constexpr int W = split_lanes(NG, sizeof(R) == 4);
  constexpr int CPW = 32 / W;
  constexpr int CPB = (kBlock / 32) * CPW;
  constexpr int ibm = B - 15;
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int lane_col = wib * CPW + lane / W, g = lane % W;
  const int col = blk * CPB + lane_col;
  const bool valid = lane < CPW * W && col < ncol;
  const int c = valid ? col : (col < ncol ? col : ncol - 1);
  const int gg = g < NG ? g : NG - 1;
  const size_t N = (size_t)ncol;
  const size_t fstride = (size_t)nlay * N;
  const double coszen = __ldg(in.coszen + c);
  const bool lit = coszen >= 1.e-10;
  const R prmu0 = (R)(lit ? coszen : 1.0);
  const R bpade = (R)c_sw.bpade;
  const int lt = w.laytrop[c];
  const int klev = nlay;
  const int E = 2 * nlay;

  DR zinc((R)0);
  const int ls = w.laysolfr[(size_t)(B - 16) * N + c];
  if (ls >= 1) {
    SwDualView<R> L{w.fv, w.ft, w.fq, fstride, (size_t)(ls - 1) * N + c};
    const DR sfz = sw_sfluxzen<B>(c_sw, L, ls <= lt, gg, tab64);
    zinc = ((R)adjflux * sfz) * (R)(lit ? coszen : 1.0);
  }
  const R albdir = (R)__ldg(((ibm >= 10 && ibm <= 13) ? in.asdir : in.aldir) + c);
  const R albdif = (R)__ldg(((ibm >= 10 && ibm <= 13) ? in.asdif : in.aldif) + c);

  // layer properties (value, d/dtlay, d/dq) and level states, top-down index
  R Rv[MAXL], Rt[MAXL], Rq[MAXL], Dv[MAXL], Dt[MAXL], Dq[MAXL], Tv[MAXL], Tt[MAXL], Tq[MAXL];
  R Sv[MAXL], St[MAXL], Sq[MAXL], Xv[MAXL], Xt[MAXL], Xq[MAXL];
  R tb[MAXL + 1], tn[MAXL + 1], rn[MAXL + 1], pu[MAXL + 1], pd[MAXL + 1];
  R zf[MAXL + 1], dn[MAXL + 1];  // 1/(1 - rn pd) and fd - fu per level
  R zu[MAXL], zd[MAXL];          // reciprocals of the upward / downward recursions per layer
  R gR[MAXL], gD[MAXL], gT[MAXL], gS[MAXL], gX[MAXL];
  R an[MAXL + 1];                // seed cotangents of net flux per bottom-up level
  R gtl[MAXL], gql[MAXL];         // FP32: layer gradients contracted as the sweeps go
  R lb[MAXL + 1], ln[MAXL + 1], lr[MAXL + 1];  // local cotangents of tb, tn, rn per level
  for (int j = 0; j < klev; ++j) {
    const int ikl = klev - j;
    const size_t o = (size_t)(ikl - 1) * N + c;
    const Idx ix = unpack_idx(__ldg(w.idx + o));
    SwDualView<R> L{w.fv, w.ft, w.fq, fstride, o};
    DR taug, taur;
    sw_gas<B, DR>(c_sw, L, ix, ikl <= lt, gg, tab, taug, taur);
    DR ztauc, zomcc, zgcc;
    if (iaer == 10) {
      const size_t oa = c + N * ((size_t)(ikl - 1) + (size_t)nlay * (ibm - 1));
      const R taua = (R)__ldg(in.tauaer + oa);
      const R omga = (R)__ldg(in.ssaaer + oa);
      const R asya = (R)__ldg(in.asmaer + oa);
      ztauc = taur + taug + taua;
      zomcc = taur * (R)1 + taua * omga;
      zgcc = (asya * omga * taua) / zomcc;
      zomcc = zomcc / ztauc;
      const DR zf = zgcc * zgcc;
      const DR zwf = zomcc * zf;
      ztauc = ((R)1 - zwf) * ztauc;
      zomcc = (zomcc - zwf) / ((R)1 - zwf);
      zgcc = (zgcc - zf) / ((R)1 - zf);
    } else {
      // without aerosol the delta scaling is the identity (asymmetry 0)
      ztauc = taur + taug;
      zomcc = taur / ztauc;
      zgcc = DR((R)0);
    }
    // the delta-Eddington solution in its cancellation-free form (the same
    // function as reftra_sw, fewer divisions), in FP64 or FP32
    DR rf, rfd, tr, trd;
    reftra_split(ztauc, zomcc, zgcc, DR(prmu0), DR(bpade), (const float*)nullptr, true, rf, rfd, tr, trd, iaer != 10);
    const DR tx = sw_exp_tbl<DR, R>(ztauc / prmu0, DR(bpade), (const R*)nullptr, true);
    Rv[j] = rf.v; Rt[j] = rf.t; Rq[j] = rf.q;
    Dv[j] = rfd.v; Dt[j] = rfd.t; Dq[j] = rfd.q;
    Tv[j] = tr.v; Tt[j] = tr.t; Tq[j] = tr.q;
    Sv[j] = trd.v; St[j] = trd.t; Sq[j] = trd.q;
    Xv[j] = tx.v; Xt[j] = tx.t; Xq[j] = tx.q;
  }
  tb[0] = (R)1.0; tn[0] = (R)1.0; rn[0] = (R)0.0;
  for (int j = 0; j < klev; ++j) {
    tb[j + 1] = Xv[j] * tb[j];
    const R z = (R)1.0 / ((R)1.0 - Dv[j] * rn[j]);
    if constexpr (sizeof(R) == 8) zd[j] = z;
    tn[j + 1] = tb[j] * Tv[j] + Sv[j] * ((tn[j] - tb[j]) + tb[j] * Rv[j] * rn[j]) * z;
    rn[j + 1] = Dv[j] + Sv[j] * Sv[j] * rn[j] * z;
  }
  pu[klev] = albdir; pd[klev] = albdif;
  for (int j = klev - 1; j >= 0; --j) {
    const R z = (R)1.0 / ((R)1.0 - pd[j + 1] * Dv[j]);
    if constexpr (sizeof(R) == 8) zu[j] = z;
    pu[j] = Rv[j] + Sv[j] * ((Tv[j] - Xv[j]) * pd[j + 1] + Xv[j] * pu[j + 1]) * z;
    pd[j] = Dv[j] + Sv[j] * Sv[j] * pd[j + 1] * z;
  }
  // FP64: reciprocals and flux differences kept per level (FP64 divides are
  // expensive); FP32 recomputes them (local-memory traffic is what costs)
  if constexpr (sizeof(R) == 8) {
    for (int j = 0; j <= klev; ++j) {
      const R z = (R)1.0 / ((R)1.0 - rn[j] * pd[j]);
      zf[j] = z;
      const R fu = (tb[j] * pu[j] + (tn[j] - tb[j]) * pd[j]) * z;
      const R fd = tb[j] + (tn[j] - tb[j] + tb[j] * pu[j] * rn[j]) * z;
      dn[j] = fd - fu;
    }
  }

  const int wcol0 = blk * CPB + wib * CPW;
  const double gate = lit ? 1.0 : 0.0;  // dark columns have zero SW outputs
  for (int s = 0; s < nseed; ++s) {
    // cotangent of net at every bottom-up level m (an[m]); layers 1..nlay-1 carry
    // heating cotangents (the top layer's rate is 0)
    const double csfc = cot ? __ldg(cot + (size_t)(2 * nlay + 2) * N + c) : (s == nlay ? 1.0 : 0.0);
    double cprev = 0.0;  // cdiv(m)
    for (int m = 0; m <= nlay; ++m) {
      double cnext = 0.0;  // cdiv(m + 1)
      const int kk = m + 1;
      if (kk <= nlay - 1) {
        const double hs = __ldg(w.hs + (size_t)(kk - 1) * N + c);
        cnext = cot ? __ldg(cot + (size_t)(nlay + 2 + kk - 1) * N + c) * hs : (s == kk - 1 ? hs : 0.0);
      }
      an[m] = (R)(gate * (cprev - cnext + (m == 0 ? csfc : 0.0)));
      cprev = cnext;
    }
    auto anet = [&](int m) { return an[m]; };
    // local cotangents of the level states at top-down level j from the fluxes there
    auto local = [&](int j, R& ltb, R& ltn, R& lrn, R& lpu, R& lpd) {
      const R a = zinc.v * anet(klev - j);
      R z;
      if constexpr (sizeof(R) == 8)
        z = zf[j];
      else
        z = (R)1.0 / ((R)1.0 - rn[j] * pd[j]);
      const R Af = tb[j] * pu[j] + (tn[j] - tb[j]) * pd[j];
      const R Bf = tn[j] - tb[j] + tb[j] * pu[j] * rn[j];
      // fu = Af z (cotangent -a), fd = tb + Bf z (cotangent a)
      ltb = -a * (pu[j] - pd[j]) * z + a * ((R)1.0 + (-(R)1.0 + pu[j] * rn[j]) * z);
      ltn = -a * pd[j] * z + a * z;
      lpu = -a * tb[j] * z + a * tb[j] * rn[j] * z;
      lpd = -a * ((tn[j] - tb[j]) * z + Af * z * z * rn[j]) + a * Bf * z * z * rn[j];
      lrn = -a * Af * z * z * pd[j] + a * (tb[j] * pu[j] * z + Bf * z * z * pd[j]);
    };
    R lzinc = (R)0.0;
    if constexpr (sizeof(R) == 8) {
      for (int j = 0; j <= klev; ++j) lzinc += anet(klev - j) * dn[j];
      for (int j = 0; j < klev; ++j) gR[j] = gD[j] = gT[j] = gS[j] = gX[j] = (R)0.0;
      // reverse of the upward sweep, carried from the top down; the local
      // cotangents of (tb, tn, rn) are kept for the second sweep
      R Lu = (R)0.0, Ld = (R)0.0;
      {
        R lpu, lpd;
        local(klev, lb[klev], ln[klev], lr[klev], lpu, lpd);
      }
      for (int j = 0; j < klev; ++j) {
        R lpu, lpd;
        local(j, lb[j], ln[j], lr[j], lpu, lpd);
        Lu += lpu;
        Ld += lpd;
        const R z = zu[j];
        const R Xx = (Tv[j] - Xv[j]) * pd[j + 1] + Xv[j] * pu[j + 1];
        const R Td = Sv[j];
        gR[j] += Lu;
        gS[j] += Lu * Xx * z + Ld * (R)2.0 * Td * pd[j + 1] * z;
        gT[j] += Lu * Td * pd[j + 1] * z;
        gX[j] += Lu * Td * (pu[j + 1] - pd[j + 1]) * z;
        gD[j] += Ld * ((R)1.0 + Td * Td * pd[j + 1] * z * z * pd[j + 1]) + Lu * Td * Xx * z * z * pd[j + 1];
        const R nLu = Lu * Td * Xv[j] * z;
        const R nLd = Lu * (Td * (Tv[j] - Xv[j]) * z + Td * Xx * z * z * Dv[j]) +
                           Ld * (Td * Td * z + Td * Td * pd[j + 1] * z * z * Dv[j]);
        Lu = nLu;
        Ld = nLd;
      }
      // reverse of the downward sweep, carried from the surface up
      R Lb = (R)0.0, Ln = (R)0.0, Lr = (R)0.0;
      for (int j = klev; j >= 1; --j) {
        Lb += lb[j];
        Ln += ln[j];
        Lr += lr[j];
        const int q = j - 1;
        const R z = zd[q];
        const R Y = (tn[q] - tb[q]) + tb[q] * Rv[q] * rn[q];
        const R Td = Sv[q];
        gX[q] += Lb * tb[q];
        gT[q] += Ln * tb[q];
        gS[q] += Ln * Y * z + Lr * (R)2.0 * Td * rn[q] * z;
        gR[q] += Ln * Td * tb[q] * rn[q] * z;
        gD[q] += Ln * Td * Y * z * z * rn[q] + Lr * ((R)1.0 + Td * Td * rn[q] * z * z * rn[q]);
        const R nLb = Lb * Xv[q] + Ln * (Tv[q] + Td * (-(R)1.0 + Rv[q] * rn[q]) * z);
        const R nLn = Ln * Td * z;
        const R nLr = Ln * (Td * tb[q] * Rv[q] * z + Td * Y * z * z * Dv[q]) +
                           Lr * (Td * Td * z + Td * Td * rn[q] * z * z * Dv[q]);
        Lb = nLb;
        Ln = nLn;
        Lr = nLr;
      }
    } else {
      for (int j = 0; j <= klev; ++j) {
        const R z = (R)1.0 / ((R)1.0 - rn[j] * pd[j]);
        const R fu = (tb[j] * pu[j] + (tn[j] - tb[j]) * pd[j]) * z;
        const R fd = tb[j] + (tn[j] - tb[j] + tb[j] * pu[j] * rn[j]) * z;
        lzinc += anet(klev - j) * (fd - fu);
      }
      for (int j = 0; j < klev; ++j) gtl[j] = gql[j] = (R)0.0;
      auto contract = [&](int j, R dR, R dD, R dT, R dS, R dX) {
        gtl[j] += dR * Rt[j] + dD * Dt[j] + dT * Tt[j] + dS * St[j] + dX * Xt[j];
        gql[j] += dR * Rq[j] + dD * Dq[j] + dT * Tq[j] + dS * Sq[j] + dX * Xq[j];
      };
      // reverse of the upward sweep, carried from the top down
      R Lu = (R)0.0, Ld = (R)0.0;
      for (int j = 0; j < klev; ++j) {
        R ltb, ltn, lrn, lpu, lpd;
        local(j, ltb, ltn, lrn, lpu, lpd);
        Lu += lpu;
        Ld += lpd;
        const R z = (R)1.0 / ((R)1.0 - pd[j + 1] * Dv[j]);
        const R Xx = (Tv[j] - Xv[j]) * pd[j + 1] + Xv[j] * pu[j + 1];
        const R Td = Sv[j];
        contract(j, Lu, Ld * ((R)1.0 + Td * Td * pd[j + 1] * z * z * pd[j + 1]) + Lu * Td * Xx * z * z * pd[j + 1],
                 Lu * Td * pd[j + 1] * z, Lu * Xx * z + Ld * (R)2.0 * Td * pd[j + 1] * z,
                 Lu * Td * (pu[j + 1] - pd[j + 1]) * z);
        const R nLu = Lu * Td * Xv[j] * z;
        const R nLd = Lu * (Td * (Tv[j] - Xv[j]) * z + Td * Xx * z * z * Dv[j]) +
                      Ld * (Td * Td * z + Td * Td * pd[j + 1] * z * z * Dv[j]);
        Lu = nLu;
        Ld = nLd;
      }
      // reverse of the downward sweep, carried from the surface up
      R Lb = (R)0.0, Ln = (R)0.0, Lr = (R)0.0;
      for (int j = klev; j >= 1; --j) {
        R ltb, ltn, lrn, lpu, lpd;
        local(j, ltb, ltn, lrn, lpu, lpd);
        Lb += ltb;
        Ln += ltn;
        Lr += lrn;
        const int q = j - 1;
        const R z = (R)1.0 / ((R)1.0 - Dv[q] * rn[q]);
        const R Y = (tn[q] - tb[q]) + tb[q] * Rv[q] * rn[q];
        const R Td = Sv[q];
        contract(q, Ln * Td * tb[q] * rn[q] * z,
                 Ln * Td * Y * z * z * rn[q] + Lr * ((R)1.0 + Td * Td * rn[q] * z * z * rn[q]), Ln * tb[q],
                 Ln * Y * z + Lr * (R)2.0 * Td * rn[q] * z, Lb * tb[q]);
        const R nLb = Lb * Xv[q] + Ln * (Tv[q] + Td * (-(R)1.0 + Rv[q] * rn[q]) * z);
        const R nLn = Ln * Td * z;
        const R nLr = Ln * (Td * tb[q] * Rv[q] * z + Td * Y * z * z * Dv[q]) +
                      Lr * (Td * Td * z + Td * Td * rn[q] * z * z * Dv[q]);
        Lb = nLb;
        Ln = nLn;
        Lr = nLr;
      }
    }
    GRed<W, NG, R> red{(R*)sred + wib * W * kRow, (int)(threadIdx.x & 31), 0, 0};
    auto store = [&](int e, int cs, double v) {
      const int cc = wcol0 + cs;
      if (cc < ncol) w.part[(((size_t)(B - 16) * nseed + s) * E + e) * N + cc] = v;
    };
    for (int l = 1; l <= nlay; ++l) {
      const int j = klev - l;
      R gt, gq;
      if constexpr (sizeof(R) == 8) {
        gt = gR[j] * Rt[j] + gD[j] * Dt[j] + gT[j] * Tt[j] + gS[j] * St[j] + gX[j] * Xt[j];
        gq = gR[j] * Rq[j] + gD[j] * Dq[j] + gT[j] * Tq[j] + gS[j] * Sq[j] + gX[j] * Xq[j];
      } else {
        gt = gtl[j];
        gq = gql[j];
      }
      if (l == ls) {
        gt += lzinc * zinc.t;
        gq += lzinc * zinc.q;
      }
      red.put(gt);
      red.next(store);
      red.put(gq);
      red.next(store);
    }
    if (red.n) red.flush(store);
  }
}

// AER < 0: iaer as passed; 0 / 1: compile-time aerosol flag (the split adjoint
// instantiates both, so that the aerosol code folds away without aerosols).
template <class R, int MAXL, int AER = -1>
__global__ void __launch_bounds__(kBlock, sizeof(R) == 4 ? RRTMG_SPLIT_ADJ_SW_MINB : 1) sw_adj_kernel(SwIn in, AdjSwWorkT<R> w, double adjflux, int iaer,
                                                        const R* __restrict__ tab, const double* __restrict__ tab64,
                                                        const double* __restrict__ cot, int nseed, int ncol,
                                                        int nlay) {
  // FP32 entries take half the staging room: a smaller shared-memory carve-out
  // leaves the split kernels more L1 for their per-thread arrays
  __shared__ double sred[sizeof(R) == 4 ? kRedDoubles / 2 : kRedDoubles];
  int blk = blockIdx.x, band = 0;
  for (; band < kSwBands; ++band) {
    const int nb = lw_blocks_for_band(split_lanes(c_sw.band[band].ng, sizeof(R) == 4), ncol);
    if (blk < nb) break;
    blk -= nb;
  }
  const int ia = AER < 0 ? iaer : (AER ? 10 : 0);
#define RRTMG_SW_ADJ_CASE(b) \
  case b - 16: sw_adj_band<b, R, MAXL>(in, w, adjflux, ia, tab, tab64, cot, nseed, ncol, nlay, blk, sred); break;
  switch (band) {
    RRTMG_SW_ADJ_CASE(16) RRTMG_SW_ADJ_CASE(17) RRTMG_SW_ADJ_CASE(18) RRTMG_SW_ADJ_CASE(19) RRTMG_SW_ADJ_CASE(20)
    RRTMG_SW_ADJ_CASE(21) RRTMG_SW_ADJ_CASE(22) RRTMG_SW_ADJ_CASE(23) RRTMG_SW_ADJ_CASE(24) RRTMG_SW_ADJ_CASE(25)
    RRTMG_SW_ADJ_CASE(26) RRTMG_SW_ADJ_CASE(27) RRTMG_SW_ADJ_CASE(28) RRTMG_SW_ADJ_CASE(29)
    default: break;
  }
#undef RRTMG_SW_ADJ_CASE
}

// ---------------------------------------------------------------------------
// Band sums.  LW partials are weighted by wtdiff * delwave * fluxfac
// (rrtmg_lw_rtrnmr.f90:720-746); the secdiff entry is chained to every
// layer's q through d secdiff / d q.  SW partials are already in W/m2.
// Jacobian: one thread per (column, output row); VJP: one per column.
// ---------------------------------------------------------------------------
// Thread per (column, output row, chunk of kAdjXChunk inputs).
constexpr int kAdjXChunk = 8;
__global__ void __launch_bounds__(128) adj_finalize_kernel(AdjLwWork lw, AdjSwWork sw, int nseed_lw, int nseed_sw,
                                                           int ncol, int nlay, double* __restrict__ out, int vjp) {
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= ncol) return;
  const size_t N = (size_t)ncol;
  const int L = nlay, ny = 2 * L + 3, nx = 3 * L + 2;
  const int nxc = (nx + kAdjXChunk - 1) / kAdjXChunk;
  const int r = blockIdx.y / nxc;  // output row (Jacobian) or 0 (VJP)
  const int x0 = (blockIdx.y % nxc) * kAdjXChunk, x1 = min(nx, x0 + kAdjXChunk);
  const int Elw = 3 * L + 3, Esw = 2 * L;
  const double wtdiff = 0.5;
  auto lwp = [&](int b, int s, int e) { return __ldg(lw.part + (((size_t)b * nseed_lw + s) * Elw + e) * N + col); };
  auto swp = [&](int b, int s, int e) { return __ldg(sw.part + (((size_t)b * nseed_sw + s) * Esw + e) * N + col); };
  double wb[kLwBands];
#pragma unroll
  for (int b = 0; b < kLwBands; ++b) wb[b] = wtdiff * c_lw.band[b].delwave * c_lw.fluxfac;
  const bool do_lw = vjp || r < L + 2;
  const bool do_sw = vjp || r >= L + 2;
  const int slw = vjp ? 0 : r, ssw = vjp ? 0 : r - (L + 2);
  for (int x = x0; x < x1; ++x) {
    double v = 0.0;
    if (do_lw) {
      int e;
      if (x < L) e = 3 * x;                          // tlay
      else if (x < 2 * L) e = 3 * (x - L) + 1;       // q
      else if (x < 3 * L) e = 3 * (x - 2 * L) + 2;   // tlev 0..nlay-1
      else if (x == 3 * L) e = 3 * L;                // tlev nlay
      else e = 3 * L + 1;                            // tsfc
#pragma unroll
      for (int b = 0; b < kLwBands; ++b) {
        double t = lwp(b, slw, e);
        if (x >= L && x < 2 * L) t += lwp(b, slw, 3 * L + 2) * __ldg(lw.dsec + ((size_t)b * L + (x - L)) * N + col);
        v += wb[b] * t;
      }
    }
    if (do_sw && x < 2 * L) {
      const int e = x < L ? 2 * x : 2 * (x - L) + 1;
      for (int b = 0; b < kSwBands; ++b) v += swp(b, ssw, e);
    }
    if (vjp)
      out[(size_t)x * N + col] = v;
    else
      out[((size_t)x * ny + r) * N + col] = v;
  }
}

// ---------------------------------------------------------------------------
// Host side.
// ---------------------------------------------------------------------------
cudaError_t upload_constants_adjoint(const LwConst& lw, const SwConst& sw) {
  cudaError_t e = cudaMemcpyToSymbol(c_lw, &lw, sizeof(LwConst));
  if (e != cudaSuccess) return e;
  const LwConstF f = make_lwconstf(lw);
  e = cudaMemcpyToSymbol(c_lwf, &f, sizeof(LwConstF));
  if (e != cudaSuccess) return e;
  return cudaMemcpyToSymbol(c_sw, &sw, sizeof(SwConst));
}

void launch_adj_lw(const LwIn& in, const AdjLwWork& w, const double* totplnk, const double* tab,
                   const double* cot, int nseed, int ncol, int nlay, int nb, cudaStream_t s) {
  adj_lw_prep_kernel<double><<<(ncol + 127) / 128, 128, 0, s>>>(in, w, totplnk, ncol, nlay);
  if (maxl_for(nlay) == 64)
    lw_adj_kernel<double, 64><<<nb, kBlock, 0, s>>>(in, w, tab, cot, nseed, ncol, nlay);
  else
    lw_adj_kernel<double, 208><<<nb, kBlock, 0, s>>>(in, w, tab, cot, nseed, ncol, nlay);
}

void launch_adj_lw_split(const LwIn& in, const AdjLwWorkT<float>& w, const float* totplnk, const float* tab,
                         const double* cot, int nseed, int ncol, int nlay, int nb, cudaStream_t s) {
  adj_lw_prep_kernel<float><<<(ncol + 127) / 128, 128, 0, s>>>(in, w, totplnk, ncol, nlay);
  if (maxl_for(nlay) == 64)
    lw_adj_kernel<float, 64><<<nb, kBlock, 0, s>>>(in, w, tab, cot, nseed, ncol, nlay);
  else
    lw_adj_kernel<float, 208><<<nb, kBlock, 0, s>>>(in, w, tab, cot, nseed, ncol, nlay);
}

void launch_adj_sw(const SwIn& in, const AdjSwWork& w, double adjflux, int iaer, const double* tab,
                   const double* cot, int nseed, int ncol, int nlay, int nb, cudaStream_t s) {
  adj_sw_prep_kernel<double><<<(ncol + 127) / 128, 128, 0, s>>>(in, w, ncol, nlay);
  if (maxl_for(nlay) == 64)
    sw_adj_kernel<double, 64><<<nb, kBlock, 0, s>>>(in, w, adjflux, iaer, tab, tab, cot, nseed, ncol, nlay);
  else
    sw_adj_kernel<double, 208><<<nb, kBlock, 0, s>>>(in, w, adjflux, iaer, tab, tab, cot, nseed, ncol, nlay);
}

void launch_adj_sw_split(const SwIn& in, const AdjSwWorkT<float>& w, double adjflux, int iaer, const float* tab,
                         const double* tab64, const double* cot, int nseed, int ncol, int nlay, int nb,
                         cudaStream_t s) {
  adj_sw_prep_kernel<float><<<(ncol + 127) / 128, 128, 0, s>>>(in, w, ncol, nlay);
  if (maxl_for(nlay) == 64)
    (iaer == 10 ? sw_adj_kernel<float, 64, 1> : sw_adj_kernel<float, 64, 0>)<<<nb, kBlock, 0, s>>>(
        in, w, adjflux, iaer, tab, tab64, cot, nseed, ncol, nlay);
  else
    (iaer == 10 ? sw_adj_kernel<float, 208, 1> : sw_adj_kernel<float, 208, 0>)<<<nb, kBlock, 0, s>>>(
        in, w, adjflux, iaer, tab, tab64, cot, nseed, ncol, nlay);
}

void launch_adj_finalize(const AdjLwWork& lw, const AdjSwWork& sw, const double* plev, const double* coszen,
                         int nseed_lw, int nseed_sw, int ncol, int nlay, double* out, bool vjp, cudaStream_t s) {
  (void)plev;
  (void)coszen;
  const int nxc = (adj_nx(nlay) + kAdjXChunk - 1) / kAdjXChunk;
  dim3 grid((ncol + 127) / 128, (vjp ? 1 : adj_ny(nlay)) * nxc);
  adj_finalize_kernel<<<grid, 128, 0, s>>>(lw, sw, nseed_lw, nseed_sw, ncol, nlay, out, vjp ? 1 : 0);
}

}  // namespace rrtmg
