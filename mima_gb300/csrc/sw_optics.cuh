// SW gas optics for one (layer, g-point): gaseous optical depth taug and
// Rayleigh optical depth taur, plus the solar source sfluxzen of a g-point.
// Band B is a template argument (16..29); the arithmetic is the reference's
// taumol16..29 (rrtmg_sw_taumol.f90:243-1536) for a single (layer, g), with the
// reference's sum association.
#pragma once
#include "lw_optics.cuh"

namespace rrtmg {

// Compile-time g-point counts per band (parrrsw.f90 ng16..ng29).
__host__ __device__ constexpr int sw_ng(int b) {
  return b == 16 ? 6 : b == 17 ? 12 : b == 18 ? 8 : b == 19 ? 8 : b == 20 ? 10 : b == 21 ? 10 : b == 22 ? 2
       : b == 23 ? 10 : b == 24 ? 8 : b == 25 ? 6 : b == 26 ? 6 : b == 27 ? 8 : b == 28 ? 6 : 12;
}

// Band constants of taumol16..29.
__host__ __device__ constexpr double sw_strrat(int b) {
  return b == 16 ? 252.131 : b == 17 ? 0.364641 : b == 18 ? 38.9589 : b == 19 ? 5.49281 : b == 21 ? 0.0045321
       : b == 22 ? 0.022708 : b == 24 ? 0.124692 : b == 28 ? 6.67029e-07 : 0.0;
}

// Per-layer fields stored as F (the solver's type), read as R.
template <class R, class F = R>
struct SwLayerView {
  const F* __restrict__ f;
  size_t fstride, o;
  __device__ __forceinline__ R operator()(int fld) const { return (R)fld_ld(f + (size_t)fld * fstride + o); }
};

// Eta of the band's key-species pair at one layer; mult 8 (lower) or 4 (upper).
template <int B, class R, class V>
__device__ __forceinline__ EtaV<R> sw_band_eta(const V& L, R mult, R one_m) {
  constexpr double s = sw_strrat(B);
  if constexpr (B == 16 || B == 18) return eta_mix<R>(L(SF_COLH2O), (R)s, L(SF_COLCH4), mult, one_m);
  else if constexpr (B == 17 || B == 19 || B == 21) return eta_mix<R>(L(SF_COLH2O), (R)s, L(SF_COLCO2), mult, one_m);
  else if constexpr (B == 22) return eta_mix<R>(L(SF_COLH2O), (R)(1.6 * s), L(SF_COLO2), mult, one_m);
  else if constexpr (B == 24) return eta_mix<R>(L(SF_COLH2O), (R)s, L(SF_COLO2), mult, one_m);
  else return eta_mix<R>(L(SF_COLO3), (R)s, L(SF_COLO2), mult, one_m);  // 28
}

// speccomb * (8-term eta / T / p interpolation); stride 9 (lower) or 5 (upper).
template <class R, int NG, class TT>
__device__ __forceinline__ R sw_major8(const TT* __restrict__ k, const EtaV<R>& e, R f00, R f10, R f01, R f11,
                                       int i0, int i1, int s, int g) {
  auto K = [&](int i) { return tld(k + (size_t)(i - 1) * NG + g); };
  R fs = e.fs;
  R fac000 = ((R)1. - fs) * f00, fac010 = ((R)1. - fs) * f10, fac100 = fs * f00, fac110 = fs * f10;
  R fac001 = ((R)1. - fs) * f01, fac011 = ((R)1. - fs) * f11, fac101 = fs * f01, fac111 = fs * f11;
  return e.speccomb * (fac000 * K(i0) + fac100 * K(i0 + 1) + fac010 * K(i0 + s) + fac110 * K(i0 + s + 1) +
                       fac001 * K(i1) + fac101 * K(i1 + 1) + fac011 * K(i1 + s) + fac111 * K(i1 + s + 1));
}

template <int B, class R, class V, class TT>
__device__ __forceinline__ void sw_gas(const SwConst& C, const V& L, const Idx& ix, bool lower, int g,
                                       const TT* __restrict__ tab, R& taug, R& taur) {
  constexpr int NG = sw_ng(B);
  const BandDesc& bd = C.band[B - 16];
  const TT* ka = tab + bd.off[SW_KA];
  const TT* kb = tab + bd.off[SW_KB];
  const TT* self = tab + bd.off[SW_SELF];
  const TT* forr = tab + bd.off[SW_FOR];
  const TT* rayl = tab + bd.off[SW_RAYL];
  const R one_m = (R)C.oneminus;
  const int jp = ix.jp;
  auto i_lo = [&](int js) { return ((jp - 1) * 5 + (ix.jt - 1)) * bd.nspa + js; };
  auto i_lo1 = [&](int js) { return (jp * 5 + (ix.jt1 - 1)) * bd.nspa + js; };
  auto i_up = [&](int js) { return ((jp - 13) * 5 + (ix.jt - 1)) * bd.nspb + js; };
  auto i_up1 = [&](int js) { return ((jp - 12) * 5 + (ix.jt1 - 1)) * bd.nspb + js; };
  auto i4 = [&](const TT* k, int i0, int i1) {
    return interp4<R, NG>(k, L(SF_FAC00), L(SF_FAC10), L(SF_FAC01), L(SF_FAC11), i0, i1, g);
  };
  auto selft = [&]() { return L(SF_SELFFAC) * lin<R, NG>(self, ix.inds, L(SF_SELFFRAC), g); };
  auto fort = [&]() { return L(SF_FORFAC) * lin<R, NG>(forr, ix.indf, L(SF_FORFRAC), g); };
  auto m8 = [&](const TT* k, const EtaV<R>& e, int i0, int i1, int s) {
    return sw_major8<R, NG>(k, e, L(SF_FAC00), L(SF_FAC10), L(SF_FAC01), L(SF_FAC11), i0, i1, s, g);
  };
  auto E = [&](int role) { return (R)tld(tab + bd.off[role] + g); };
  const R colmol = L(SF_COLMOL);

  if constexpr (B == 16 || B == 18 || B == 19 || B == 21 || B == 22 || B == 17) {
    const R rs = tld(rayl);
    if (lower) {
      EtaV<R> e = sw_band_eta<B, R>(L, (R)8., one_m);
      R t = m8(ka, e, i_lo(e.js), i_lo1(e.js), 9) + L(SF_COLH2O) * (selft() + fort());
      if constexpr (B == 22) t = t + (R)4.35e-4 * L(SF_COLO2) / (R)(350.0 * 2.0);
      taug = t;
    } else {
      if constexpr (B == 16) taug = L(SF_COLCH4) * i4(kb, i_up(1), i_up1(1));
      else if constexpr (B == 18) taug = L(SF_COLCH4) * i4(kb, i_up(1), i_up1(1));
      else if constexpr (B == 19) taug = L(SF_COLCO2) * i4(kb, i_up(1), i_up1(1));
      else if constexpr (B == 22)
        taug = L(SF_COLO2) * (R)1.6 * i4(kb, i_up(1), i_up1(1)) + (R)4.35e-4 * L(SF_COLO2) / (R)(350.0 * 2.0);
      else {  // 17, 21: eta-mixed upper with foreign continuum
        EtaV<R> e = sw_band_eta<B, R>(L, (R)4., one_m);
        taug = m8(kb, e, i_up(e.js), i_up1(e.js), 5) +
               L(SF_COLH2O) * L(SF_FORFAC) * lin<R, NG>(forr, ix.indf, L(SF_FORFRAC), g);
      }
    }
    taur = colmol * rs;
  } else if constexpr (B == 20) {
    const R rs = tld(rayl);
    if (lower)
      taug = L(SF_COLH2O) * (i4(ka, i_lo(1), i_lo1(1)) + selft() + fort()) + L(SF_COLCH4) * E(SW_E1);
    else
      taug = L(SF_COLH2O) * (i4(kb, i_up(1), i_up1(1)) + fort()) + L(SF_COLCH4) * E(SW_E1);
    taur = colmol * rs;
  } else if constexpr (B == 23) {
    if (lower) taug = L(SF_COLH2O) * ((R)1.029 * i4(ka, i_lo(1), i_lo1(1)) + selft() + fort());
    else taug = (R)0.;
    taur = colmol * tld(rayl + g);
  } else if constexpr (B == 24) {
    if (lower) {
      EtaV<R> e = sw_band_eta<B, R>(L, (R)8., one_m);
      taur = colmol * lin<R, NG>(rayl, e.js, e.fs, g);
      taug = m8(ka, e, i_lo(e.js), i_lo1(e.js), 9) + L(SF_COLO3) * E(SW_E2) + L(SF_COLH2O) * (selft() + fort());
    } else {
      taur = colmol * E(SW_E1);
      taug = L(SF_COLO2) * i4(kb, i_up(1), i_up1(1)) + L(SF_COLO3) * E(SW_E3);
    }
  } else if constexpr (B == 25) {
    if (lower) taug = L(SF_COLH2O) * i4(ka, i_lo(1), i_lo1(1)) + L(SF_COLO3) * E(SW_E2);
    else taug = L(SF_COLO3) * E(SW_E3);
    taur = colmol * tld(rayl + g);
  } else if constexpr (B == 26) {
    taug = (R)0.;
    taur = colmol * tld(rayl + g);
  } else if constexpr (B == 27) {
    if (lower) taug = L(SF_COLO3) * i4(ka, i_lo(1), i_lo1(1));
    else taug = L(SF_COLO3) * i4(kb, i_up(1), i_up1(1));
    taur = colmol * tld(rayl + g);
  } else if constexpr (B == 28) {
    EtaV<R> e = sw_band_eta<B, R>(L, lower ? (R)8. : (R)4., one_m);
    if (lower) taug = m8(ka, e, i_lo(e.js), i_lo1(e.js), 9);
    else taug = m8(kb, e, i_up(e.js), i_up1(e.js), 5);
    taur = colmol * tld(rayl);
  } else {  // 29
    if (lower)
      taug = L(SF_COLH2O) * (i4(ka, i_lo(1), i_lo1(1)) + selft() + fort()) + L(SF_COLCO2) * E(SW_E2);
    else
      taug = L(SF_COLCO2) * i4(kb, i_up(1), i_up1(1)) + L(SF_COLH2O) * E(SW_E1);
    taur = colmol * tld(rayl);
  }
}

// Solar source of g-point g of band B, taken at the band's reference layer
// (laysolfr, computed by the prep kernel exactly as the taumol loops do).
// Bands whose sfluxref depends on eta interpolate it with that layer's eta.
// The result has the view's type (double, or a dual for the adjoint).
template <int B, class V>
__device__ __forceinline__ auto sw_sfluxzen(const SwConst& C, const V& L, bool lower, int g,
                                            const double* __restrict__ tab) {
  using R = decltype(L(0));
  constexpr int NG = sw_ng(B);
  const BandDesc& bd = C.band[B - 16];
  const double* sf = tab + bd.off[SW_SFLUX];
  if constexpr (B == 17 || B == 28) {
    EtaV<R> e = sw_band_eta<B, R>(L, (R)4., (R)C.oneminus);
    return lin<R, NG>(sf, e.js, e.fs, g);
  } else if constexpr (B == 18 || B == 19 || B == 21 || B == 22 || B == 24) {
    EtaV<R> e = sw_band_eta<B, R>(L, (R)8., (R)C.oneminus);
    return lin<R, NG>(sf, e.js, e.fs, g);
  } else if constexpr (B == 27) {
    return (R)((50.15 / 48.37) * tld(sf + g));
  } else {
    return (R)tld(sf + g);
  }
}

}  // namespace rrtmg
