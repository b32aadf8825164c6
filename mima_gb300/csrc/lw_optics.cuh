// LW gas optics for one (layer, g-point): optical depth taug and Planck
// fraction fracs.  One device function per band, selected at compile time, so
// a warp (which always holds g-points of a single band) runs straight-line
// code.  The arithmetic is the reference's taugb1..16
// (rrtmg_lw_taumol.f90:280-3147) evaluated for a single (layer, g):
//   * key species: 4-point (p, T) interpolation, or the eta-mixed 9-level
//     (lower) / 5-level (upper) form with the 3-point treatment near eta = 0
//     and 1 (specparm < 0.125 / > 0.875);
//   * water-vapour self / foreign continua, minor gases (T- or (eta, T)-
//     interpolated), cross sections;
//   * Planck fractions, eta-interpolated in the mixed bands.
// The sum association of every expression follows the reference so that the
// FP64 instantiation is bit-reproducible against a literal restatement.
#pragma once
#include <type_traits>

#include "common.cuh"
#include "dual.cuh"

namespace rrtmg {

// Compile-time g-point counts per band (parrrtm.f90 ng1..ng16).
__host__ __device__ constexpr int lw_ng(int b) {
  return b == 1 ? 10 : b == 2 ? 12 : b == 3 ? 16 : b == 4 ? 14 : b == 5 ? 16 : b == 6 ? 8 : b == 7 ? 12
       : b == 8 ? 8 : b == 9 ? 12 : b == 10 ? 6 : b == 11 ? 8 : b == 12 ? 8 : b == 13 ? 4 : 2;
}
__host__ __device__ constexpr int pow2ceil(int n) { return n <= 2 ? 2 : n <= 4 ? 4 : n <= 8 ? 8 : n <= 16 ? 16 : 32; }

// Layer-state accessor: fields of one (layer, column) of the prep output.
template <class R>
struct LwLayerView {
  const R* __restrict__ f;  // per-layer fields stored in the solver's type
  size_t fstride;           // nlay * ncol
  size_t o;                 // (lay-1) * ncol + col
  __device__ __forceinline__ R operator()(int fld) const { return fld_ld(f + (size_t)fld * fstride + o); }
};

template <class R>
struct EtaV {
  R speccomb, specparm, fs;
  int js;
};

template <class R>
__device__ __forceinline__ EtaV<R> eta_mix(R a, R ratb, R b, R mult, R oneminus) {
  EtaV<R> e;
  e.speccomb = a + ratb * b;
  e.specparm = a / e.speccomb;
  if (e.specparm >= oneminus) e.specparm = oneminus;
  R specmult = mult * (e.specparm);
  int ip = (int)specmult;
  e.fs = specmult - (R)ip;  // mod(specmult, 1) for specmult >= 0
  // For valid inputs 0 <= specparm <= oneminus, so 0 <= ip < mult; the clamp
  // only keeps table reads in bounds for non-finite or negative inputs (which
  // the prep kernels flag as invalid).
  const int top = (int)mult - 1;
  ip = ip < 0 ? 0 : (ip > top ? top : ip);
  e.js = 1 + ip;
  return e;
}

// Interpolation weights of one pressure level of the 9-level eta form.
template <class R>
struct W3 {
  R a0, a1, a2, b0, b1, b2;
};
template <class R>
__device__ __forceinline__ W3<R> w3(R specparm, R fs, R facA, R facB) {
  W3<R> w;
  if (specparm < (R)0.125) {
    R p = fs - (R)1;
    R p4 = (p * p) * (p * p);
    R fk0 = p4, fk1 = (R)1 - p - (R)2.0 * p4, fk2 = p + p4;
    w.a0 = fk0 * facA; w.a1 = fk1 * facA; w.a2 = fk2 * facA;
    w.b0 = fk0 * facB; w.b1 = fk1 * facB; w.b2 = fk2 * facB;
  } else if (specparm > (R)0.875) {
    R p = -fs;
    R p4 = (p * p) * (p * p);
    R fk0 = p4, fk1 = (R)1 - p - (R)2.0 * p4, fk2 = p + p4;
    w.a0 = fk0 * facA; w.a1 = fk1 * facA; w.a2 = fk2 * facA;
    w.b0 = fk0 * facB; w.b1 = fk1 * facB; w.b2 = fk2 * facB;
  } else {
    w.a0 = ((R)1. - fs) * facA;
    w.b0 = ((R)1. - fs) * facB;
    w.a1 = fs * facA;
    w.b1 = fs * facB;
    w.a2 = (R)0;
    w.b2 = (R)0;
  }
  return w;
}

// tab points at the band's key-species table (absa); rows are ind-1, g fastest.
template <class R, int NG, class TT>
__device__ __forceinline__ R major9(const TT* __restrict__ ka, R specparm, R speccomb, int ind, int g,
                                    const W3<R>& w) {
  auto K = [&](int i) { return tld(ka + (size_t)(i - 1) * NG + g); };
  if (specparm < (R)0.125)
    return speccomb * (w.a0 * K(ind) + w.a1 * K(ind + 1) + w.a2 * K(ind + 2) + w.b0 * K(ind + 9) +
                       w.b1 * K(ind + 10) + w.b2 * K(ind + 11));
  if (specparm > (R)0.875)
    return speccomb * (w.a2 * K(ind - 1) + w.a1 * K(ind) + w.a0 * K(ind + 1) + w.b2 * K(ind + 8) +
                       w.b1 * K(ind + 9) + w.b0 * K(ind + 10));
  return speccomb * (w.a0 * K(ind) + w.a1 * K(ind + 1) + w.b0 * K(ind + 9) + w.b1 * K(ind + 10));
}

template <class R, int NG, class TT>
__device__ __forceinline__ R interp4(const TT* __restrict__ k, R f00, R f10, R f01, R f11, int i0, int i1, int g) {
  auto K = [&](int i) { return tld(k + (size_t)(i - 1) * NG + g); };
  return f00 * K(i0) + f10 * K(i0 + 1) + f01 * K(i1) + f11 * K(i1 + 1);
}

// Upper-atmosphere 5-level eta form (two pressure levels summed).
template <class R, int NG, class TT>
__device__ __forceinline__ R major5(const TT* __restrict__ kb, R sc, R fs, int i0, R sc1, R fs1, int i1, R f00,
                                    R f10, R f01, R f11, int g) {
  auto K = [&](int i) { return tld(kb + (size_t)(i - 1) * NG + g); };
  R fac000 = ((R)1. - fs) * f00, fac010 = ((R)1. - fs) * f10, fac100 = fs * f00, fac110 = fs * f10;
  R fac001 = ((R)1. - fs1) * f01, fac011 = ((R)1. - fs1) * f11, fac101 = fs1 * f01, fac111 = fs1 * f11;
  return sc * (fac000 * K(i0) + fac100 * K(i0 + 1) + fac010 * K(i0 + 5) + fac110 * K(i0 + 6)) +
         sc1 * (fac001 * K(i1) + fac101 * K(i1 + 1) + fac011 * K(i1 + 5) + fac111 * K(i1 + 6));
}

// k(row, g) + frac * (k(row+1, g) - k(row, g))
template <class R, int NG, class TT>
__device__ __forceinline__ R lin(const TT* __restrict__ k, int row1, R frac, int g) {
  R a = (R)tld(k + (size_t)(row1 - 1) * NG + g), b = (R)tld(k + (size_t)row1 * NG + g);
  return a + frac * (b - a);
}
// Minor table k(j, indm, g) with nj rows in eta: eta- then T-interpolated.
template <class R, int NG, class TT>
__device__ __forceinline__ R minor_eta(const TT* __restrict__ k, int nj, int jm, R fm, int indm, R minorfrac, int g) {
  auto K = [&](int j, int m) { return tld(k + ((size_t)(m - 1) * nj + (j - 1)) * NG + g); };
  R m1 = K(jm, indm) + fm * (K(jm + 1, indm) - K(jm, indm));
  R m2 = K(jm, indm + 1) + fm * (K(jm + 1, indm + 1) - K(jm, indm + 1));
  return m1 + minorfrac * (m2 - m1);
}

// x^e for the minor-gas column adjustments: the FP64/FP32 forms evaluate pow
// in FP64 as written; the dual form carries the derivative.
template <class R>
__device__ __forceinline__ R rpow(R x, double e) {
  return (R)pow((double)x, e);
}
template <class R>
__device__ __forceinline__ Dual<R> rpow(Dual<R> x, double e) {
  return pow(x, (R)e);
}

template <class R>
__device__ __forceinline__ R adj_col(R col, R coldry, R chiref, R thresh, R base, double expo) {
  // Empirical adjustment of a minor column that exceeds the reference
  // profile, e.g. rrtmg_lw_taumol.f90:528-535.
  R chi_x = col / (coldry);
  R ratx = (R)1.e20 * chi_x / chiref;
  if (ratx > thresh) {
    R adjfac = base + rpow(ratx - base, expo);
    return adjfac * chiref * coldry * (R)1.e-20;
  }
  return col;
}

struct LwBandCtx {
  const BandDesc* bd;
  const LwConst* cst;
};

// taug / fracs of band B for g (0-based in band) at one layer.
// C: band layout and FP64 constants; CR: the per-layer constants in type R
// (C itself for FP64, its FP32 copy for the split path).
// V: layer-field accessor returning R; TT: table element type (R itself, or
// the value type of a dual R).
template <int B, class R, class RC, class V, class TT>
__device__ __forceinline__ void lw_gas(const LwConst& C, const RC& CR, const V& L, const Idx& ix, bool lower, int g,
                                       const TT* __restrict__ tab, R& taug, R& fracs) {
  constexpr int NG = lw_ng(B);
  const BandDesc& bd = C.band[B - 1];
  const TT* ka = tab + bd.off[LW_KA];
  const TT* kb = tab + bd.off[LW_KB];
  const TT* self = tab + bd.off[LW_SELF];
  const TT* forr = tab + bd.off[LW_FOR];
  const TT* fra = tab + bd.off[LW_FRA];
  const TT* frb = tab + bd.off[LW_FRB];
  using CT = std::remove_cv_t<std::remove_reference_t<decltype(CR.oneminus)>>;  // double or float
  const R one_m = (R)CR.oneminus;
  const int jp = ix.jp;
  auto i_lo = [&](int js) { return ((jp - 1) * 5 + (ix.jt - 1)) * bd.nspa + js; };
  auto i_lo1 = [&](int js) { return (jp * 5 + (ix.jt1 - 1)) * bd.nspa + js; };
  auto i_up = [&](int js) { return ((jp - 13) * 5 + (ix.jt - 1)) * bd.nspb + js; };
  auto i_up1 = [&](int js) { return ((jp - 12) * 5 + (ix.jt1 - 1)) * bd.nspb + js; };
  auto tself = [&]() { return L(LF_SELFFAC) * lin<R, NG>(self, ix.inds, L(LF_SELFFRAC), g); };
  auto tfor = [&]() { return L(LF_FORFAC) * lin<R, NG>(forr, ix.indf, L(LF_FORFRAC), g); };
  auto fr1 = [&](const TT* fr) { return (R)tld(fr + g); };
  auto fr_eta = [&](const TT* fr, const EtaV<R>& e) { return lin<R, NG>(fr, e.js, e.fs, g); };
  auto i4 = [&](const TT* k, int i0, int i1) {
    return interp4<R, NG>(k, L(LF_FAC00), L(LF_FAC10), L(LF_FAC01), L(LF_FAC11), i0, i1, g);
  };
  auto rat = [&](const auto* r, int j) { return (R)r[j]; };
  auto chi = [&](int i, int j) { return (R)CR.chi[(j - 1) * 7 + (i - 1)]; };

  if constexpr (B == 1) {
    if (lower) {
      R pp = L(LF_PAVEL);
      R corradj = (R)1.;
      if (pp < (R)250.) corradj = (R)1. - (R)0.15 * ((R)250. - pp) / (R)154.4;
      R scalen2 = L(LF_COLBRD) * L(LF_SCALEMINORN2);
      R tauself = tself(), taufor = tfor();
      R taun2 = scalen2 * lin<R, NG>(tab + bd.off[LW_MA1], ix.indm, L(LF_MINORFRAC), g);
      taug = corradj * (L(LF_COLH2O) * i4(ka, i_lo(1), i_lo1(1)) + tauself + taufor + taun2);
      fracs = fr1(fra);
    } else {
      R pp = L(LF_PAVEL);
      R corradj = (R)1. - (R)0.15 * (pp / (R)95.6);
      R scalen2 = L(LF_COLBRD) * L(LF_SCALEMINORN2);
      R taufor = tfor();
      R taun2 = scalen2 * lin<R, NG>(tab + bd.off[LW_MB1], ix.indm, L(LF_MINORFRAC), g);
      taug = corradj * (L(LF_COLH2O) * i4(kb, i_up(1), i_up1(1)) + taufor + taun2);
      fracs = fr1(frb);
    }
  } else if constexpr (B == 2) {
    if (lower) {
      R pp = L(LF_PAVEL);
      R corradj = (R)1. - (R).05 * (pp - (R)100.) / (R)900.;
      R tauself = tself(), taufor = tfor();
      taug = corradj * (L(LF_COLH2O) * i4(ka, i_lo(1), i_lo1(1)) + tauself + taufor);
      fracs = fr1(fra);
    } else {
      R taufor = tfor();
      taug = L(LF_COLH2O) * i4(kb, i_up(1), i_up1(1)) + taufor;
      fracs = fr1(frb);
    }
  } else if constexpr (B == 3 || B == 5 || B == 7 || B == 9 || B == 13 || B == 15) {
    // Lower: eta-mixed key species + minor gas with its own eta.
    // Keys: 3: h2o/co2 (minor n2o), 5: h2o/co2 (minor o3, ccl4), 7: h2o/o3
    // (minor co2), 9: h2o/ch4 (minor n2o), 13: h2o/n2o (minors co2, co),
    // 15: n2o/co2 (minor n2).
    if (lower) {
      R a, b;
      const CT *r0, *r1;
      if constexpr (B == 3 || B == 5) { a = L(LF_COLH2O); b = L(LF_COLCO2); r0 = CR.r_h2oco2; }
      else if constexpr (B == 7) { a = L(LF_COLH2O); b = L(LF_COLO3); r0 = CR.r_h2oo3; }
      else if constexpr (B == 9) { a = L(LF_COLH2O); b = L(LF_COLCH4); r0 = CR.r_h2och4; }
      else if constexpr (B == 13) { a = L(LF_COLH2O); b = L(LF_COLN2O); r0 = CR.r_h2on2o; }
      else { a = L(LF_COLN2O); b = L(LF_COLCO2); r0 = CR.r_n2oco2; }
      r1 = r0;
      EtaV<R> e = eta_mix<R>(a, rat(r0, jp), b, (R)8., one_m);
      EtaV<R> e1 = eta_mix<R>(a, rat(r1, jp + 1), b, (R)8., one_m);
      EtaV<R> em = eta_mix<R>(a, (R)CR.refrat[B - 1][2], b, (R)8., one_m);
      R extra, extra2 = (R)0;
      if constexpr (B == 3 || B == 9) {
        R adjcoln2o = adj_col<R>(L(LF_COLN2O), L(LF_COLDRY), chi(4, jp + 1), (R)1.5, (R)0.5, 0.65);
        R absn2o = minor_eta<R, NG>(tab + bd.off[LW_MA1], 9, em.js, em.fs, ix.indm, L(LF_MINORFRAC), g);
        extra = adjcoln2o * absn2o;
      } else if constexpr (B == 5) {
        R abso3 = minor_eta<R, NG>(tab + bd.off[LW_MA1], 9, em.js, em.fs, ix.indm, L(LF_MINORFRAC), g);
        extra = abso3 * L(LF_COLO3);
      } else if constexpr (B == 7) {
        R adjcolco2 = adj_col<R>(L(LF_COLCO2), L(LF_COLDRY), chi(2, jp + 1), (R)3.0, (R)3.0, 0.79);
        R absco2 = minor_eta<R, NG>(tab + bd.off[LW_MA1], 9, em.js, em.fs, ix.indm, L(LF_MINORFRAC), g);
        extra = adjcolco2 * absco2;
      } else if constexpr (B == 13) {
        // ratco2 against a fixed 3.55e-4 reference (rrtmg_lw_taumol.f90:2404-2410)
        R chi_co2 = L(LF_COLCO2) / (L(LF_COLDRY));
        R ratco2 = (R)1.e20 * chi_co2 / (R)3.55e-4;
        R adjcolco2;
        if (ratco2 > (R)3.0) {
          R adjfac = (R)2.0 + rpow(ratco2 - (R)2.0, 0.68);
          adjcolco2 = adjfac * (R)3.55e-4 * L(LF_COLDRY) * (R)1.e-20;
        } else {
          adjcolco2 = L(LF_COLCO2);
        }
        EtaV<R> emo = eta_mix<R>(a, (R)CR.refrat[B - 1][3], b, (R)8., one_m);
        R absco2 = minor_eta<R, NG>(tab + bd.off[LW_MA1], 9, em.js, em.fs, ix.indm, L(LF_MINORFRAC), g);
        R absco = minor_eta<R, NG>(tab + bd.off[LW_MA2], 9, emo.js, emo.fs, ix.indm, L(LF_MINORFRAC), g);
        extra = adjcolco2 * absco2;
        extra2 = L(LF_COLCO) * absco;
      } else {  // B == 15
        R scalen2 = L(LF_COLBRD) * L(LF_SCALEMINOR);
        extra = scalen2 * minor_eta<R, NG>(tab + bd.off[LW_MA1], 9, em.js, em.fs, ix.indm, L(LF_MINORFRAC), g);
      }
      EtaV<R> ep = eta_mix<R>(a, (R)CR.refrat[B - 1][0], b, (R)8., one_m);
      int ind0 = i_lo(e.js), ind1 = i_lo1(e1.js);
      W3<R> w0 = w3<R>(e.specparm, e.fs, L(LF_FAC00), L(LF_FAC10));
      W3<R> w1 = w3<R>(e1.specparm, e1.fs, L(LF_FAC01), L(LF_FAC11));
      R tauself = tself(), taufor = tfor();
      R tau_major = major9<R, NG>(ka, e.specparm, e.speccomb, ind0, g, w0);
      R tau_major1 = major9<R, NG>(ka, e1.specparm, e1.speccomb, ind1, g, w1);
      if constexpr (B == 5) {
        taug = tau_major + tau_major1 + tauself + taufor + extra + L(LF_WX1) * tld(tab + bd.off[LW_X1] + g);
      } else if constexpr (B == 13) {
        taug = tau_major + tau_major1 + tauself + taufor + extra + extra2;
      } else {
        taug = tau_major + tau_major1 + tauself + taufor + extra;
      }
      fracs = fr_eta(fra, ep);
    } else {
      if constexpr (B == 3 || B == 5) {
        R a = (B == 3) ? L(LF_COLH2O) : L(LF_COLO3);
        const auto* r0 = (B == 3) ? CR.r_h2oco2 : CR.r_o3co2;
        R b = L(LF_COLCO2);
        EtaV<R> e = eta_mix<R>(a, rat(r0, jp), b, (R)4., one_m);
        EtaV<R> e1 = eta_mix<R>(a, rat(r0, jp + 1), b, (R)4., one_m);
        EtaV<R> ep = eta_mix<R>(a, (R)CR.refrat[B - 1][1], b, (R)4., one_m);
        int ind0 = i_up(e.js), ind1 = i_up1(e1.js);
        R maj = major5<R, NG>(kb, e.speccomb, e.fs, ind0, e1.speccomb, e1.fs, ind1, L(LF_FAC00), L(LF_FAC10),
                              L(LF_FAC01), L(LF_FAC11), g);
        if constexpr (B == 3) {
          EtaV<R> em = eta_mix<R>(a, (R)CR.refrat[B - 1][3], b, (R)4., one_m);
          R adjcoln2o = adj_col<R>(L(LF_COLN2O), L(LF_COLDRY), chi(4, jp + 1), (R)1.5, (R)0.5, 0.65);
          R taufor = tfor();
          R absn2o = minor_eta<R, NG>(tab + bd.off[LW_MB1], 5, em.js, em.fs, ix.indm, L(LF_MINORFRAC), g);
          taug = maj + taufor + adjcoln2o * absn2o;
        } else {
          taug = maj + L(LF_WX1) * tld(tab + bd.off[LW_X1] + g);
        }
        fracs = fr_eta(frb, ep);
      } else if constexpr (B == 7) {
        R adjcolco2 = adj_col<R>(L(LF_COLCO2), L(LF_COLDRY), chi(2, jp + 1), (R)3.0, (R)2.0, 0.79);
        R absco2 = lin<R, NG>(tab + bd.off[LW_MB1], ix.indm, L(LF_MINORFRAC), g);
        R t = L(LF_COLO3) * i4(kb, i_up(1), i_up1(1)) + adjcolco2 * absco2;
        constexpr double sc[12] = {1, 1, 1, 1, 1, 0.92, 0.88, 1.07, 1.1, 0.99, 0.855, 1};
        if (g >= 5 && g <= 10) t = t * (R)sc[g];
        taug = t;
        fracs = fr1(frb);
      } else if constexpr (B == 9) {
        R adjcoln2o = adj_col<R>(L(LF_COLN2O), L(LF_COLDRY), chi(4, jp + 1), (R)1.5, (R)0.5, 0.65);
        R absn2o = lin<R, NG>(tab + bd.off[LW_MB1], ix.indm, L(LF_MINORFRAC), g);
        taug = L(LF_COLCH4) * i4(kb, i_up(1), i_up1(1)) + adjcoln2o * absn2o;
        fracs = fr1(frb);
      } else if constexpr (B == 13) {
        R abso3 = lin<R, NG>(tab + bd.off[LW_MB1], ix.indm, L(LF_MINORFRAC), g);
        taug = L(LF_COLO3) * abso3;
        fracs = fr1(frb);
      } else {  // 15
        taug = (R)0.0;
        fracs = (R)0.0;
      }
    }
  } else if constexpr (B == 4 || B == 12 || B == 16) {
    // Lower: eta-mixed key species only (4: h2o/co2, 12: h2o/co2, 16: h2o/ch4)
    if (lower) {
      R a = L(LF_COLH2O);
      R b = (B == 16) ? L(LF_COLCH4) : L(LF_COLCO2);
      const auto* r0 = (B == 16) ? CR.r_h2och4 : CR.r_h2oco2;
      EtaV<R> e = eta_mix<R>(a, rat(r0, jp), b, (R)8., one_m);
      EtaV<R> e1 = eta_mix<R>(a, rat(r0, jp + 1), b, (R)8., one_m);
      EtaV<R> ep = eta_mix<R>(a, (R)CR.refrat[B - 1][0], b, (R)8., one_m);
      int ind0 = i_lo(e.js), ind1 = i_lo1(e1.js);
      W3<R> w0 = w3<R>(e.specparm, e.fs, L(LF_FAC00), L(LF_FAC10));
      W3<R> w1 = w3<R>(e1.specparm, e1.fs, L(LF_FAC01), L(LF_FAC11));
      R tauself = tself(), taufor = tfor();
      R tau_major = major9<R, NG>(ka, e.specparm, e.speccomb, ind0, g, w0);
      R tau_major1 = major9<R, NG>(ka, e1.specparm, e1.speccomb, ind1, g, w1);
      taug = tau_major + tau_major1 + tauself + taufor;
      fracs = fr_eta(fra, ep);
    } else {
      if constexpr (B == 4) {
        R a = L(LF_COLO3), b = L(LF_COLCO2);
        EtaV<R> e = eta_mix<R>(a, rat(CR.r_o3co2, jp), b, (R)4., one_m);
        EtaV<R> e1 = eta_mix<R>(a, rat(CR.r_o3co2, jp + 1), b, (R)4., one_m);
        EtaV<R> ep = eta_mix<R>(a, (R)CR.refrat[B - 1][1], b, (R)4., one_m);
        int ind0 = i_up(e.js), ind1 = i_up1(e1.js);
        R t = major5<R, NG>(kb, e.speccomb, e.fs, ind0, e1.speccomb, e1.fs, ind1, L(LF_FAC00), L(LF_FAC10),
                            L(LF_FAC01), L(LF_FAC11), g);
        constexpr double sc[14] = {1, 1, 1, 1, 1, 1, 1, 0.92, 0.88, 1.07, 1.1, 0.99, 0.88, 0.943};
        if (g >= 7) t = t * (R)sc[g];
        taug = t;
        fracs = fr_eta(frb, ep);
      } else if constexpr (B == 12) {
        taug = (R)0.0;
        fracs = (R)0.0;
      } else {  // 16
        taug = L(LF_COLCH4) * i4(kb, i_up(1), i_up1(1));
        fracs = fr1(frb);
      }
    }
  } else if constexpr (B == 6) {
    if (lower) {
      R adjcolco2 = adj_col<R>(L(LF_COLCO2), L(LF_COLDRY), chi(2, jp + 1), (R)3.0, (R)2.0, 0.77);
      R tauself = tself(), taufor = tfor();
      R absco2 = (lin<R, NG>(tab + bd.off[LW_MA1], ix.indm, L(LF_MINORFRAC), g));
      taug = L(LF_COLH2O) * i4(ka, i_lo(1), i_lo1(1)) + tauself + taufor + adjcolco2 * absco2 +
             L(LF_WX2) * tld(tab + bd.off[LW_X1] + g) + L(LF_WX3) * tld(tab + bd.off[LW_X2] + g);
    } else {
      taug = (R)0.0 + L(LF_WX2) * tld(tab + bd.off[LW_X1] + g) + L(LF_WX3) * tld(tab + bd.off[LW_X2] + g);
    }
    fracs = fr1(fra);
  } else if constexpr (B == 8) {
    R adjcolco2 = adj_col<R>(L(LF_COLCO2), L(LF_COLDRY), chi(2, jp + 1), (R)3.0, (R)2.0, 0.65);
    R x12 = L(LF_WX3) * tld(tab + bd.off[LW_X1] + g);
    if (lower) {
      R tauself = tself(), taufor = tfor();
      R absco2 = (lin<R, NG>(tab + bd.off[LW_MA1], ix.indm, L(LF_MINORFRAC), g));
      R abso3 = (lin<R, NG>(tab + bd.off[LW_MA2], ix.indm, L(LF_MINORFRAC), g));
      R absn2o = (lin<R, NG>(tab + bd.off[LW_MA3], ix.indm, L(LF_MINORFRAC), g));
      taug = L(LF_COLH2O) * i4(ka, i_lo(1), i_lo1(1)) + tauself + taufor + adjcolco2 * absco2 +
             L(LF_COLO3) * abso3 + L(LF_COLN2O) * absn2o + x12 + L(LF_WX4) * tld(tab + bd.off[LW_X2] + g);
      fracs = fr1(fra);
    } else {
      R absco2 = (lin<R, NG>(tab + bd.off[LW_MB1], ix.indm, L(LF_MINORFRAC), g));
      R absn2o = (lin<R, NG>(tab + bd.off[LW_MB2], ix.indm, L(LF_MINORFRAC), g));
      taug = L(LF_COLO3) * i4(kb, i_up(1), i_up1(1)) + adjcolco2 * absco2 + L(LF_COLN2O) * absn2o + x12 +
             L(LF_WX4) * tld(tab + bd.off[LW_X2] + g);
      fracs = fr1(frb);
    }
  } else if constexpr (B == 10) {
    if (lower) {
      R tauself = tself(), taufor = tfor();
      taug = L(LF_COLH2O) * i4(ka, i_lo(1), i_lo1(1)) + tauself + taufor;
      fracs = fr1(fra);
    } else {
      R taufor = tfor();
      taug = L(LF_COLH2O) * i4(kb, i_up(1), i_up1(1)) + taufor;
      fracs = fr1(frb);
    }
  } else if constexpr (B == 11) {
    R scaleo2 = L(LF_COLO2) * L(LF_SCALEMINOR);
    if (lower) {
      R tauself = tself(), taufor = tfor();
      R tauo2 = scaleo2 * lin<R, NG>(tab + bd.off[LW_MA1], ix.indm, L(LF_MINORFRAC), g);
      taug = L(LF_COLH2O) * i4(ka, i_lo(1), i_lo1(1)) + tauself + taufor + tauo2;
      fracs = fr1(fra);
    } else {
      R taufor = tfor();
      R tauo2 = scaleo2 * lin<R, NG>(tab + bd.off[LW_MB1], ix.indm, L(LF_MINORFRAC), g);
      taug = L(LF_COLH2O) * i4(kb, i_up(1), i_up1(1)) + taufor + tauo2;
      fracs = fr1(frb);
    }
  } else if constexpr (B == 14) {
    if (lower) {
      R tauself = tself(), taufor = tfor();
      taug = L(LF_COLCO2) * i4(ka, i_lo(1), i_lo1(1)) + tauself + taufor;
      fracs = fr1(fra);
    } else {
      taug = L(LF_COLCO2) * i4(kb, i_up(1), i_up1(1));
      fracs = fr1(frb);
    }
  }
}

}  // namespace rrtmg
