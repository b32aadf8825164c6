// Device workspaces and host launchers of the adjoint translation unit
// (adjoint.cu).
#pragma once
#include <cuda_runtime.h>

#include "common.cuh"

namespace rrtmg {

// Output layout of the adjoint entry points, per column:
//   rows (ny = 2 nlay + 3): LW heating of layers 1..nlay (K/day), OLR (W/m2,
//     upward), LW surface net flux (up - down, W/m2), SW heating of layers
//     1..nlay, SW surface net flux (down - up);
//   inputs (nx = 3 nlay + 2): tlay of layers 1..nlay, h2ovmr (specific
//     humidity) of layers 1..nlay, tlev of levels 0..nlay, tsfc.
inline int adj_ny(int nlay) { return 2 * nlay + 3; }
inline int adj_nx(int nlay) { return 3 * nlay + 2; }
// Per-seed gradient entries of one g-point: LW (tlay_l, q_l, tlev_{l-1}) for
// l = 1..nlay, then tlev_nlay, tsfc, secdiff; SW (tlay_l, q_l).
inline int adj_lw_entries(int nlay) { return 3 * nlay + 3; }
inline int adj_sw_entries(int nlay) { return 2 * nlay; }

// F: the type of the checkpointed per-layer values (double for the FP64
// adjoint, float for the FP32/FP64-split adjoint); band partials stay FP64.
template <class F>
struct AdjLwWorkT {
  uint32_t* idx;
  int* laytrop;
  F *fv, *ft, *fq;               // setcoef fields [LF_N][lay][col]: value, d/dtlay, d/dq
  F *play_v, *play_t;            // planklay [band][lay][col] and d/dtlay
  F *plev_v, *plev_t;            // planklev [band][lev][col] and d/dtlev
  F *pbnd_v, *pbnd_t;            // emissivity * plankbnd [band][col] and d/dtsfc
  F* secdiff;                    // [band][col]
  double* dsec;                  // d secdiff / d q [band][lay][col]
  double* hs;                    // heatfac / (plev(l-1) - plev(l)) [lay][col]
  double* part;                  // band partial gradients [band][seed][entry][col]
};
using AdjLwWork = AdjLwWorkT<double>;

template <class F>
struct AdjSwWorkT {
  uint32_t* idx;
  int *laytrop, *laysolfr;
  F *fv, *ft, *fq;               // setcoef fields [SF_N][lay][col]: value, d/dtlay, d/dq
  double* hs;                    // heatfac / (plev(l-1) - plev(l)) [lay][col]
  double* part;                  // band partial gradients [band][seed][entry][col]
};
using AdjSwWork = AdjSwWorkT<double>;

cudaError_t upload_constants_adjoint(const LwConst& lw, const SwConst& sw);

// cot: NULL for full Jacobians (one unit seed per output row), else the
// cotangents (ncol, ny) of a vector-Jacobian product.
// tab: the k-tables in the adjoint's type; tab64 the FP64 tables (SW solar source).
void launch_adj_lw(const LwIn& in, const AdjLwWork& w, const double* totplnk, const double* tab,
                   const double* cot, int nseed, int ncol, int nlay, int nb, cudaStream_t s);
void launch_adj_sw(const SwIn& in, const AdjSwWork& w, double adjflux, int iaer, const double* tab,
                   const double* cot, int nseed, int ncol, int nlay, int nb, cudaStream_t s);
// FP32/FP64-split adjoint: FP32 dual numbers and reverse sweeps, g-point sums
// to FP64 accuracy, FP64 band sums.
void launch_adj_lw_split(const LwIn& in, const AdjLwWorkT<float>& w, const float* totplnk, const float* tab,
                         const double* cot, int nseed, int ncol, int nlay, int nb, cudaStream_t s);
void launch_adj_sw_split(const SwIn& in, const AdjSwWorkT<float>& w, double adjflux, int iaer, const float* tab,
                         const double* tab64, const double* cot, int nseed, int ncol, int nlay, int nb,
                         cudaStream_t s);
// Weighted band sums into jac (ny, nx per column) or grad (nx per column).
void launch_adj_finalize(const AdjLwWork& lw, const AdjSwWork& sw, const double* plev, const double* coszen,
                         int nseed_lw, int nseed_sw, int ncol, int nlay, double* out, bool vjp, cudaStream_t s);

}  // namespace rrtmg
