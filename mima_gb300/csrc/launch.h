// Host-side launch wrappers of the kernel translation units (kernels_fp64.cu,
// compiled without multiply-add contraction for bit-reproducible FP64, and
// kernels_split.cu, the FP32-split path).  Each translation unit owns a copy
// of the constant-memory tables and uploads it in upload_constants_*().
#pragma once
#include <cuda_runtime.h>

#include "common.cuh"

namespace rrtmg {

// Choice of the compiled per-thread column depth (local-memory arrays).
inline int maxl_for(int nlay) { return nlay <= 64 ? 64 : 208; }

cudaError_t upload_constants_fp64(const LwConst& lw, const SwConst& sw);
cudaError_t upload_constants_split(const LwConst& lw, const SwConst& sw);

// FP64 translation unit: prep (FP64 and FP32), FP64 g-point solvers, FP64 finalize.
void launch_lw_prep(const LwIn& in, const LwWork& w, const double* totplnk, const double* totplnkderiv, int ncol,
                    int nlay, int idrv, unsigned* flags, cudaStream_t s);
void launch_lw_gpoint_fp64(const LwPrep& p, const double* emis, const double* tauaer, const double* tab,
                           const double* exptbl, const double* tfntbl, double* bu, double* bd, double* bdu, int ncol,
                           int nlay, int idrv, int nb, int analytic, cudaStream_t s);
// buc, bdc, bduc: clear-sky band partials of a cloudy call, or null (clear sky).
void launch_lw_finalize(const double* bu, const double* bd, const double* bdu, const double* plev, int ncol, int nlay,
                        int idrv, double* uflx, double* dflx, double* hr, double* uflxc, double* dflxc, double* hrc,
                        double* duflx_dt, double* duflxc_dt, cudaStream_t s, const double* buc = nullptr,
                        const double* bdc = nullptr, const double* bduc = nullptr);
// Clouds (icld = 1): per-layer cloud fields, FP64 and FP32 storage.
void launch_lw_cloud(const LwIn& in, double* cld, int ncol, int nlay, cudaStream_t s);
void launch_lw_cloud_split(const LwIn& in, float* cld, int ncol, int nlay, cudaStream_t s);
// Cloud physics (inflag 1 / 2): the cloud fields of launch_lw_cloud and the
// cloud depths along the diffusivity angle (odc); cldtab: ct:: tables (FP32
// copy on the split path).
void launch_lw_cldphys(const LwIn& in, const double* secdiff, const double* cldtab, double* cld, double* odc, int ncol,
                       int nlay, unsigned* flags, cudaStream_t s);
void launch_lw_cldphys_split(const LwIn& in, const float* secdiff, const float* cldtab, float* cld, double* odc,
                             int ncol, int nlay, unsigned* flags, cudaStream_t s);
// Maximum/random overlap (icld = 2, 3): rtrnmr's overlap factors per layer.
void launch_lw_overlap(const double* cldfr, double* ovl, int ncol, int nlay, cudaStream_t s);
void launch_lw_overlap_split(const double* cldfr, float* ovl, int ncol, int nlay, cudaStream_t s);
// ovl: the overlap factors of maximum/random overlap, or null (random overlap).
// scaled: taucld is launch_lw_cldphys's odc (depths along the diffusivity angle).
void launch_lw_gpoint_cld_fp64(const LwPrep& p, const double* cld, const double* taucld, const double* emis,
                               const double* tauaer, const double* tab, const double* exptbl, const double* tfntbl,
                               const double* tautbl, double* bu, double* bd, double* bdu, double* buc, double* bdc,
                               double* bduc, int ncol, int nlay, int idrv, int nb, int analytic, cudaStream_t s,
                               const double* ovl = nullptr, bool scaled = false);
void launch_lw_gpoint_cld_split(const LwPrepT<float>& p, const float* cld, const double* taucld, const double* emis,
                                const double* tauaer, const float* tab, const float* exptbl, const float* tfntbl,
                                const float* tautbl, double* bu, double* bd, double* bdu, double* buc, double* bdc,
                                double* bduc, int ncol, int nlay, int idrv, int nb, int analytic, cudaStream_t s,
                                const float* ovl = nullptr, bool scaled = false);
void launch_sw_prep(const SwIn& in, const SwWork& w, int ncol, int nlay, unsigned* flags, cudaStream_t s);
// Prep for the FP32-split solvers: the same steps in FP32 arithmetic (FP32 Planck
// tables), fields stored as float.
void launch_lw_prep_split(const LwIn& in, const LwWorkT<float>& w, const float* totplnk, const float* totplnkderiv,
                          int ncol, int nlay, int idrv, unsigned* flags, cudaStream_t s);
void launch_sw_prep_split(const SwIn& in, const SwWorkT<float>& w, int ncol, int nlay, unsigned* flags,
                          cudaStream_t s);
// cld: per-layer cover and cldprop mask of a cloudy call's total-sky pass, or
// null (a clear-sky pass).
void launch_sw_gpoint_fp64(const SwPrep& p, const SwIn& in, double adjflux, int iaer, const double* tab,
                           const double* exptbl, double* su, double* sd, int ncol, int nlay, int nb, int analytic,
                           cudaStream_t s, const double* cld = nullptr);
// SW clouds (icld = 1): per-layer cover and cldprop mask; flags a partly cloudy
// layer.  With cloud physics (in.inflag = 2) also the optics of formed layers
// into opt ([tau, ssa, g][lay][col][band]) from the ct:: tables cldtab; on the
// split path the total-sky pass's cloud optics of every formed layer into
// quads (SwIn::cldq).
void launch_sw_cloud(const SwIn& in, double* cld, int ncol, int nlay, unsigned* flags, cudaStream_t s,
                     const double* cldtab = nullptr, double* opt = nullptr);
void launch_sw_cloud_split(const SwIn& in, float* cld, int ncol, int nlay, unsigned* flags, cudaStream_t s,
                           const double* cldtab, float4* quads);
void launch_sw_finalize(const double* su, const double* sd, const double* plev, const double* coszen, int ncol,
                        int nlay, double* swuflx, double* swdflx, double* swhr, double* swuflxc, double* swdflxc,
                        double* swhrc, cudaStream_t s, const double* suc = nullptr, const double* sdc = nullptr);
// Split-path finalize: the same outputs with fewer FP64 operations (kernels_split.cu).
void launch_lw_finalize_split(const double* bu, const double* bd, const double* bdu, const double* plev, int ncol,
                              int nlay, int idrv, double* uflx, double* dflx, double* hr, double* uflxc,
                              double* dflxc, double* hrc, double* duflx_dt, double* duflxc_dt, cudaStream_t s,
                              const double* buc = nullptr, const double* bdc = nullptr, const double* bduc = nullptr);
void launch_sw_finalize_split(const double* su, const double* sd, const double* plev, const double* coszen, int ncol,
                              int nlay, double* swuflx, double* swdflx, double* swhr, double* swuflxc,
                              double* swdflxc, double* swhrc, cudaStream_t s, const double* suc = nullptr,
                              const double* sdc = nullptr);

// FP32-split translation unit.
// exptfn: the FP32 transmittance and tau transition tables interleaved.
void launch_lw_gpoint_split(const LwPrepT<float>& p, const double* emis, const double* tauaer, const float* tab,
                            const float2* exptfn, double* bu, double* bd, double* bdu, int ncol,
                            int nlay, int idrv, int nb, int analytic, cudaStream_t s);
void launch_sw_gpoint_split(const SwPrepT<float>& p, const SwIn& in, double adjflux, int iaer, const float* tab,
                            const double* tab64, const float* exptbl, double* su, double* sd, int ncol, int nlay,
                            int nb, int analytic, cudaStream_t s, const float* cld = nullptr);

// Number of blocks of the g-point grids: the sum over bands of the band's
// blocks (4 warps of 32 / lanes columns; lanes = split_lanes(ng, split)).
int lw_gpoint_blocks(const LwConst& c, int ncol, bool split = false);
int sw_gpoint_blocks(const SwConst& c, int ncol, bool split = false);
// Blocks of the split forward grids, which enumerate the slots (sub-bands).
int lw_slot_blocks(int ncol);
int sw_slot_blocks(int ncol);

}  // namespace rrtmg
