// Shared definitions of the GB300 RRTMG column-radiation kernels.
//
// Data layout in HBM (all column-fastest so that a warp of consecutive
// columns, or of the g-points of one column, touches contiguous memory):
//   * inputs/outputs: the caller's Fortran (ncol, nlev) arrays as is;
//   * per-layer gas state from the prep kernels: field-major SoA
//     [field][layer][column];
//   * coefficient tables: one buffer per precision, every reduced table
//     stored with the g-point index fastest, [..non-g indices..][g], so the
//     lanes that hold the g-points of one column read one contiguous run;
//   * band partial fluxes: [band][level][column] (FP64), summed over bands
//     in a fixed order by the finalize kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace rrtmg {

constexpr int kMaxLay = 203;
constexpr int kLwBands = 16;
constexpr int kLwG = 140;
constexpr int kSwBands = 14;
// Sub-bands (slots) of the split path's g-point grids (kernels.cuh lw_slot /
// sw_slot): rows of the band-partial arrays.
#ifndef RRTMG_LW_SUBBANDS
#define RRTMG_LW_SUBBANDS 1
#endif
constexpr int kLwSlots = RRTMG_LW_SUBBANDS ? 20 : 16, kSwSlots = 16;
constexpr int kSwG = 112;
constexpr int kBlock = 128;  // threads per block in the g-point kernels
constexpr int kNTbl = 10000;

// Table roles (slots in BandDesc::off).  LW: key-species tables, continua,
// Planck fractions, up to three lower / two upper minor-gas tables and two
// cross-section tables.  SW: key species, continua, solar source, Rayleigh and
// four band-specific extras.
enum LwRole { LW_KA = 0, LW_KB, LW_SELF, LW_FOR, LW_FRA, LW_FRB, LW_MA1, LW_MA2, LW_MA3, LW_MB1, LW_MB2,
              LW_X1, LW_X2, LW_NROLE };
enum SwRole { SW_KA = 0, SW_KB, SW_SELF, SW_FOR, SW_SFLUX, SW_RAYL, SW_E1, SW_E2, SW_E3, SW_E4, SW_NROLE };

struct BandDesc {
  int ng;      // reduced g-points of the band
  int ngpad;   // lanes per column: power of two >= ng
  int goff;    // first g-point of the band in the 140 / 112 ordering
  int nspa, nspb;
  int off[16];     // element offset of each role's table, -1 if the band has none
  int nrow[16];    // extent of the first non-g index of 2-/3-d tables (row stride helper)
  int tbeg, tend;  // element range of all the band's tables (multiples of 4: 16-byte aligned)
  double delwave;
};

// LW per-layer fields written by the prep kernel ([field][layer][column]).
enum LwField {
  LF_PAVEL = 0, LF_COLDRY, LF_COLH2O, LF_COLCO2, LF_COLO3, LF_COLN2O, LF_COLCO, LF_COLCH4, LF_COLO2,
  LF_COLBRD, LF_FAC00, LF_FAC01, LF_FAC10, LF_FAC11, LF_SELFFAC, LF_SELFFRAC, LF_FORFAC, LF_FORFRAC,
  LF_MINORFRAC, LF_SCALEMINOR, LF_SCALEMINORN2, LF_WX1, LF_WX2, LF_WX3, LF_WX4, LF_N
};
enum SwField {
  SF_COLH2O = 0, SF_COLCO2, SF_COLO3, SF_COLCH4, SF_COLO2, SF_COLMOL, SF_FAC00, SF_FAC01, SF_FAC10,
  SF_FAC11, SF_SELFFAC, SF_SELFFRAC, SF_FORFAC, SF_FORFRAC, SF_N
};

// Table gather (k-distribution and transmittance tables: read-only and reused
// by every cell of a band) and per-layer prep-field load: the read-only path.
// L1 eviction-priority variants of both (tables evict-last, fields
// evict-first) were measured on GB300 and changed neither solver's time.
template <class T>
__device__ __forceinline__ T tld(const T* p) {
  return __ldg(p);
}
template <class T>
__device__ __forceinline__ T fld_ld(const T* p) {
  return __ldg(p);
}

// Stages a band's k-distribution tables into L2 through the bulk-copy (TMA)
// unit: one cp.async.bulk.prefetch.L2 of the band's table range, whose start
// and length are multiples of 16 bytes (BandDesc::tbeg / tend).  Issued by
// one thread of each g-point block before its first gather; a hint, it
// neither waits nor changes any result.
#ifndef RRTMG_TABLE_PREFETCH_L2
#define RRTMG_TABLE_PREFETCH_L2 1
#endif
template <class T>
__device__ __forceinline__ void prefetch_band_l2(const T* tab, const BandDesc& bd) {
  const unsigned bytes = (unsigned)((bd.tend - bd.tbeg) * (int)sizeof(T));
  if (!RRTMG_TABLE_PREFETCH_L2 || bytes == 0) return;
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(tab + bd.tbeg), "r"(bytes) : "memory");
}

// Packed integer interpolation indices of one layer.
__host__ __device__ inline uint32_t pack_idx(int jp, int jt, int jt1, int inds, int indf, int indm) {
  return (uint32_t)jp | ((uint32_t)jt << 6) | ((uint32_t)jt1 << 9) | ((uint32_t)inds << 12) |
         ((uint32_t)indf << 16) | ((uint32_t)indm << 18);
}
struct Idx {
  int jp, jt, jt1, inds, indf, indm;
};
__host__ __device__ inline Idx unpack_idx(uint32_t v) {
  Idx i;
  i.jp = (int)(v & 63u);
  i.jt = (int)((v >> 6) & 7u);
  i.jt1 = (int)((v >> 9) & 7u);
  i.inds = (int)((v >> 12) & 15u);
  i.indf = (int)((v >> 16) & 3u);
  i.indm = (int)((v >> 18) & 31u);
  return i;
}

// Constants of the LW path (constant memory in every kernel translation unit).
struct LwConst {
  BandDesc band[kLwBands];
  double chi[7 * 60];      // chi_mls(i, jp) at [(jp-1)*7 + (i-1)], jp = 1..59 (+ pad)
  double preflog[60], tref[60];
  // chi_mls ratios per reference level, identical to setcoef's per-layer
  // divisions (rrtmg_lw_setcoef.f90:323-336, 370-374)
  double r_h2oco2[61], r_h2oo3[61], r_h2on2o[61], r_h2och4[61], r_n2oco2[61], r_o3co2[61];
  double refrat[kLwBands][4];  // band constants refrat_planck_a/b, refrat_m_a/b (or m_a3)
  double heatfac, fluxfac, oneminus, bpade, grav, avogad;
};

// FP32 copies of the LW constants the gas optics reads per layer, for the
// FP32-split solvers (same member names as in LwConst).
struct LwConstF {
  float chi[7 * 60];
  float r_h2oco2[61], r_h2oo3[61], r_h2on2o[61], r_h2och4[61], r_n2oco2[61], r_o3co2[61];
  float refrat[kLwBands][4];
  float oneminus;
};

struct SwConst {
  BandDesc band[kSwBands];
  double preflog[60], tref[60];
  double heatfac, oneminus, bpade, grav, avogad, pi;
};

// Per-call view of the LW prep output.
// Per-layer inputs of the g-point solvers, stored in the solver's arithmetic
// type F (double for the FP64 path, float for the FP32-split path; the prep
// kernels compute in FP64 either way and round on store).
template <class F>
struct LwPrepT {
  const uint32_t* idx;  // [lay][col]
  const F* f;           // [LF_N][lay][col]
  const F* planklay;    // [band][lay][col]
  const F* planklev;    // [band][lev 0..nlay][col]
  const F* plankbnd;    // [band][col]
  const F* dplankbnd;   // [band][col]
  const F* secdiff;     // [band][col]
  const int* laytrop;   // [col]
};
using LwPrep = LwPrepT<double>;

template <class F>
struct SwPrepT {
  const uint32_t* idx;  // [lay][col]
  const F* f;           // [SF_N][lay][col]
  const int* laytrop;   // [col]
  const int* laysolfr;  // [band][col], 0 = no solar-source layer
};
using SwPrep = SwPrepT<double>;

// ---------------------------------------------------------------------------
// Device pointers of one call (inputs as passed by the caller) and of its
// scratch workspace.
// ---------------------------------------------------------------------------
struct LwIn {
  const double *play, *plev, *tlay, *tlev, *tsfc, *h2o, *o3, *co2, *ch4, *n2o, *o2, *cfc11, *cfc12, *cfc22, *ccl4,
      *emis, *tauaer;
  // clouds (icld = 1, 2, 3), null in clear sky: cldfr (ncol, nlay), taucld
  // (16, ncol, nlay; may be null with inflag 1 / 2), cicewp / cliqwp (ncol,
  // nlay) or null
  const double *cldfr, *taucld, *cicewp, *cliqwp;
  // cloud overlap with clouds: 1 random (rtrn), 2 or 3 maximum/random (rtrnmr)
  int icld;
  // cldprop's choice (0: depths given; 1: abscld1 x water path; 2: ice and
  // liquid parameterisations iceflag 0-3, liqflag 0-1 with the effective
  // sizes reice / reliq (ncol, nlay))
  int inflag, iceflag, liqflag;
  const double *reice, *reliq;
};
template <class F>
struct LwWorkT {
  uint32_t* idx;
  F *f, *planklay, *planklev, *plankbnd, *dplankbnd, *secdiff;
  int* laytrop;
  double *bu, *bd, *bdu;  // band partials [band][lev][col]
  double* colsum;         // per-layer coldry and wk1 [2][lay][col] for the column sums
  // clouds only (null in clear sky): per layer [cloud fraction of a cloudy
  // layer, else 0][cldprop's 0/1 optical-depth mask] and the clear-sky band
  // partials
  F* cld;
  double *buc, *bdc, *bduc;
  // maximum/random overlap only: rtrnmr's overlap factors per layer,
  // [12][lay][col] (lw_overlap_kernel)
  F* ovl;
  // cloud physics (inflag 1 / 2) only: the cloud optical depth of each band
  // already along the diffusivity angle, secdiff(ib) x taucloud(ib) with ib
  // the band's cloud band (16 bands fastest, per layer and column)
  double* odc;
};
using LwWork = LwWorkT<double>;
struct SwIn {
  const double *play, *plev, *tlay, *tlev, *tsfc, *h2o, *o3, *co2, *ch4, *n2o, *o2, *asdir, *asdif, *aldir, *aldif,
      *coszen, *tauaer, *ssaaer, *asmaer;
  // clouds (icld = 1), null in clear sky: cldfr (ncol, nlay); taucld,
  // ssacld, asmcld, fsfcld (14, ncol, nlay); cicewp / cliqwp or null.  The
  // total-sky pass reads fsfcld = null as no forward fraction.
  const double *cldfr, *taucld, *ssacld, *asmcld, *fsfcld, *cicewp, *cliqwp;
  // cldprop_sw's choice (0: optics given; 2: ice iceflag 1-3 and liquid
  // liqflag 1 parameterisations with the effective sizes reice / reliq)
  int inflag, iceflag, liqflag;
  const double *reice, *reliq;
  // split path, total-sky pass only (a workspace array, not a caller input):
  // per layer and band {delta-scaled cloud depth, albedo, asymmetry,
  // co-albedo}, formed in FP64 by sw_cloud_kernel
  const float4* cldq;
};
// ---------------------------------------------------------------------------
// Cloud optical property tables (rrlw_cld and rrsw_cld, filled by lwcldpr /
// swcldpr, rrtmg_lw_init.f90 and rrtmg_sw_init.f90) in one FP64 array, each
// table in Fortran order at its offset below, with the SW band limits
// wavenum2 (rrsw_wvn) that select the Ebert-Curry coefficients.
// ---------------------------------------------------------------------------
namespace ct {
constexpr int ABSICE0 = 0;                   // (2)
constexpr int ABSICE1 = ABSICE0 + 2;         // (2, 5)
constexpr int ABSICE2 = ABSICE1 + 10;        // (43, 16)
constexpr int ABSICE3 = ABSICE2 + 43 * 16;   // (46, 16)
constexpr int ABSLIQ0 = ABSICE3 + 46 * 16;   // scalar
constexpr int ABSLIQ1 = ABSLIQ0 + 1;         // (58, 16)
constexpr int ABSCLD1 = ABSLIQ1 + 58 * 16;   // scalar
constexpr int EXTLIQ1 = ABSCLD1 + 1;         // (58, 16:29), then ssaliq1, asyliq1
constexpr int SSALIQ1 = EXTLIQ1 + 58 * 14;
constexpr int ASYLIQ1 = SSALIQ1 + 58 * 14;
constexpr int EXTICE2 = ASYLIQ1 + 58 * 14;   // (43, 16:29), then ssaice2, asyice2
constexpr int SSAICE2 = EXTICE2 + 43 * 14;
constexpr int ASYICE2 = SSAICE2 + 43 * 14;
constexpr int EXTICE3 = ASYICE2 + 43 * 14;   // (46, 16:29), then ssaice3, asyice3, fdlice3
constexpr int SSAICE3 = EXTICE3 + 46 * 14;
constexpr int ASYICE3 = SSAICE3 + 46 * 14;
constexpr int FDLICE3 = ASYICE3 + 46 * 14;
constexpr int ABARI = FDLICE3 + 46 * 14;     // (5) each: abari, bbari, cbari, dbari, ebari, fbari
constexpr int WAVENUM2 = ABARI + 6 * 5;      // (16:29)
constexpr int SIZE = WAVENUM2 + 14;
}  // namespace ct

template <class F>
struct SwWorkT {
  uint32_t* idx;
  F* f;
  int *laytrop, *laysolfr;
  double *su, *sd;  // band partials [band][lev][col]
  // clouds only (null in clear sky): per layer [cover][cldprop's 0/1 mask]
  // and the clear-sky band partials
  F* cld;
  double *suc, *sdc;
  // cloud physics (inflag = 2), FP64 path only: cldprop_sw's delta-scaled
  // optics, [tau, ssa, g][14 bands fastest, per layer and column]
  double* cldopt;
  // clouds, split path only: the cloud optics of the total-sky pass (SwIn::cldq)
  float4* cldq;
};
using SwWork = SwWorkT<double>;

}  // namespace rrtmg
