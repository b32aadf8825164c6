// FP64 instantiation of the RRTMG kernels.  Built with --fmad=false: every
// multiply and add is rounded separately, as written, so the FP64 path
// reproduces a literal FP64 restatement of the reference bit for bit apart
// from transcendental functions (log/exp) and the order of g-point sums.
#define RRTMG_DEFINE_COLUMN_KERNELS
#include "kernels.cuh"
#include "launch.h"

namespace rrtmg {

cudaError_t upload_constants_fp64(const LwConst& lw, const SwConst& sw) {
  cudaError_t e = cudaMemcpyToSymbol(c_lw, &lw, sizeof(LwConst));
  if (e != cudaSuccess) return e;
  return cudaMemcpyToSymbol(c_sw, &sw, sizeof(SwConst));
}

int lw_gpoint_blocks(const LwConst& c, int ncol, bool split) {
  int n = 0;
  for (int b = 0; b < kLwBands; ++b) n += lw_blocks_for_band(split_lanes(c.band[b].ng, split), ncol);
  return n;
}
int sw_gpoint_blocks(const SwConst& c, int ncol, bool split) {
  int n = 0;
  for (int b = 0; b < kSwBands; ++b) n += lw_blocks_for_band(split_lanes(c.band[b].ng, split), ncol);
  return n;
}
int lw_slot_blocks(int ncol) {
  int n = 0;
  for (int s = 0; s < kLwSlots; ++s) n += lw_blocks_for_band(split_lanes(lw_slot(s).ng, true), ncol);
  return n;
}
int sw_slot_blocks(int ncol) {
  int n = 0;
  for (int s = 0; s < kSwSlots; ++s) n += lw_blocks_for_band(split_lanes(sw_slot(s).ng, true), ncol);
  return n;
}

void launch_lw_prep(const LwIn& in, const LwWork& w, const double* totplnk, const double* totplnkderiv, int ncol,
                    int nlay, int idrv, unsigned* flags, cudaStream_t s) {
  const dim3 g((ncol + 127) / 128, nlay);
  lw_prep_layer_kernel<double><<<g, 128, 0, s>>>(in, w, totplnk, ncol, nlay, flags);
  lw_prep_column_kernel<double><<<(ncol + 127) / 128, 128, 0, s>>>(in, w, totplnk, totplnkderiv, ncol, nlay, idrv,
                                                                  flags);
}

void launch_lw_prep_split(const LwIn& in, const LwWorkT<float>& w, const float* totplnk, const float* totplnkderiv,
                          int ncol, int nlay, int idrv, unsigned* flags, cudaStream_t s) {
  const dim3 g((ncol + 127) / 128, nlay);
  lw_prep_layer_kernel<float><<<g, 128, 0, s>>>(in, w, totplnk, ncol, nlay, flags);
  lw_prep_column_kernel<float><<<(ncol + 127) / 128, 128, 0, s>>>(in, w, totplnk, totplnkderiv, ncol, nlay, idrv,
                                                                 flags);
}

void launch_lw_gpoint_fp64(const LwPrep& p, const double* emis, const double* tauaer, const double* tab,
                           const double* exptbl, const double* tfntbl, double* bu, double* bd, double* bdu, int ncol,
                           int nlay, int idrv, int nb, int analytic, cudaStream_t s) {
  if (maxl_for(nlay) == 64)
    lw_gpoint_kernel<double, 64><<<nb, kBlock, 0, s>>>(p, emis, tauaer, tab, exptbl, tfntbl, bu, bd, bdu, ncol, nlay, idrv, analytic);
  else
    lw_gpoint_kernel<double, 208><<<nb, kBlock, 0, s>>>(p, emis, tauaer, tab, exptbl, tfntbl, bu, bd, bdu, ncol, nlay, idrv, analytic);
}

void launch_lw_gpoint_cld_fp64(const LwPrep& p, const double* cld, const double* taucld, const double* emis,
                               const double* tauaer, const double* tab, const double* exptbl, const double* tfntbl,
                               const double* tautbl, double* bu, double* bd, double* bdu, double* buc, double* bdc,
                               double* bduc, int ncol, int nlay, int idrv, int nb, int analytic, cudaStream_t s,
                               const double* ovl, bool scaled) {
  if (maxl_for(nlay) == 64)
    lw_gpoint_cld_kernel<double, 64, -1><<<nb, kBlock, 0, s>>>(p, cld, taucld, emis, tauaer, tab, exptbl, tfntbl, tautbl,
                                                              bu, bd, bdu, buc, bdc, bduc, ncol, nlay, idrv, analytic,
                                                              ovl, scaled ? 1 : 0);
  else
    lw_gpoint_cld_kernel<double, 208, -1><<<nb, kBlock, 0, s>>>(p, cld, taucld, emis, tauaer, tab, exptbl, tfntbl,
                                                               tautbl, bu, bd, bdu, buc, bdc, bduc, ncol, nlay, idrv,
                                                               analytic, ovl, scaled ? 1 : 0);
}

void launch_lw_cloud(const LwIn& in, double* cld, int ncol, int nlay, cudaStream_t s) {
  lw_cloud_kernel<double><<<dim3((ncol + 127) / 128, nlay), 128, 0, s>>>(in, cld, ncol, nlay);
}
void launch_lw_cloud_split(const LwIn& in, float* cld, int ncol, int nlay, cudaStream_t s) {
  lw_cloud_kernel<float><<<dim3((ncol + 127) / 128, nlay), 128, 0, s>>>(in, cld, ncol, nlay);
}
void launch_lw_cldphys(const LwIn& in, const double* secdiff, const double* cldtab, double* cld, double* odc, int ncol,
                       int nlay, unsigned* flags, cudaStream_t s) {
  lw_cldphys_kernel<double><<<(unsigned)(((long long)ncol * kLwBands + 127) / 128), 128, 0, s>>>(in, secdiff, cldtab, cld, odc, ncol, nlay, flags);
}
void launch_lw_cldphys_split(const LwIn& in, const float* secdiff, const float* cldtab, float* cld, double* odc,
                             int ncol, int nlay, unsigned* flags, cudaStream_t s) {
  // 8 columns x nlay layer records of 24 bytes: at most 39 KB at 203 layers
  const size_t smem = (size_t)(kBlock / kLwBands) * nlay * sizeof(LwCldLay);
  lw_cldphys_split_kernel<<<(unsigned)(((long long)ncol * kLwBands + 127) / 128), 128, smem, s>>>(
      in, secdiff, cldtab, cld, odc, ncol, nlay, flags);
}
void launch_lw_overlap(const double* cldfr, double* ovl, int ncol, int nlay, cudaStream_t s) {
  lw_overlap_kernel<double><<<(ncol + 127) / 128, 128, 0, s>>>(cldfr, ovl, ncol, nlay);
}
void launch_lw_overlap_split(const double* cldfr, float* ovl, int ncol, int nlay, cudaStream_t s) {
  lw_overlap_kernel<float><<<(ncol + 127) / 128, 128, 0, s>>>(cldfr, ovl, ncol, nlay);
}

void launch_lw_finalize(const double* bu, const double* bd, const double* bdu, const double* plev, int ncol, int nlay,
                        int idrv, double* uflx, double* dflx, double* hr, double* uflxc, double* dflxc, double* hrc,
                        double* duflx_dt, double* duflxc_dt, cudaStream_t s, const double* buc, const double* bdc,
                        const double* bduc) {
  lw_finalize_kernel<<<dim3((ncol + 127) / 128, nlay + 1), 128, 0, s>>>(bu, bd, bdu, plev, ncol, nlay, idrv, uflx, dflx, hr, uflxc,
                                                        dflxc, hrc, duflx_dt, duflxc_dt, buc, bdc, bduc);
}

void launch_sw_prep(const SwIn& in, const SwWork& w, int ncol, int nlay, unsigned* flags, cudaStream_t s) {
  sw_prep_layer_kernel<double><<<dim3((ncol + 127) / 128, nlay), 128, 0, s>>>(in, w, ncol, nlay, flags);
  sw_prep_column_kernel<double><<<(ncol + 127) / 128, 128, 0, s>>>(in, w, ncol, nlay, flags);
}

void launch_sw_prep_split(const SwIn& in, const SwWorkT<float>& w, int ncol, int nlay, unsigned* flags,
                          cudaStream_t s) {
  sw_prep_layer_kernel<float><<<dim3((ncol + 127) / 128, nlay), 128, 0, s>>>(in, w, ncol, nlay, flags);
  sw_prep_column_kernel<float><<<(ncol + 127) / 128, 128, 0, s>>>(in, w, ncol, nlay, flags);
}

void launch_sw_gpoint_fp64(const SwPrep& p, const SwIn& in, double adjflux, int iaer, const double* tab,
                           const double* exptbl, double* su, double* sd, int ncol, int nlay, int nb, int analytic,
                           cudaStream_t s, const double* cld) {
  if (cld) {
    if (maxl_for(nlay) == 64)
      sw_gpoint_kernel<double, 64, -1, true><<<nb, kBlock, 0, s>>>(p, in, adjflux, iaer, tab, tab, exptbl, su, sd, ncol,
                                                                  nlay, analytic, cld);
    else
      sw_gpoint_kernel<double, 208, -1, true><<<nb, kBlock, 0, s>>>(p, in, adjflux, iaer, tab, tab, exptbl, su, sd, ncol,
                                                                   nlay, analytic, cld);
    return;
  }
  if (maxl_for(nlay) == 64)
    sw_gpoint_kernel<double, 64><<<nb, kBlock, 0, s>>>(p, in, adjflux, iaer, tab, tab, exptbl, su, sd, ncol, nlay, analytic, nullptr);
  else
    sw_gpoint_kernel<double, 208><<<nb, kBlock, 0, s>>>(p, in, adjflux, iaer, tab, tab, exptbl, su, sd, ncol, nlay, analytic, nullptr);
}

void launch_sw_cloud(const SwIn& in, double* cld, int ncol, int nlay, unsigned* flags, cudaStream_t s,
                     const double* cldtab, double* opt) {
  sw_cloud_kernel<double><<<dim3((ncol + 127) / 128, nlay), 128, 0, s>>>(in, cld, ncol, nlay, flags, cldtab, opt,
                                                                        nullptr);
}
void launch_sw_cloud_split(const SwIn& in, float* cld, int ncol, int nlay, unsigned* flags, cudaStream_t s,
                           const double* cldtab, float4* quads) {
  sw_cloud_kernel<float><<<dim3((ncol + 127) / 128, nlay), 128, 0, s>>>(in, cld, ncol, nlay, flags, cldtab, nullptr,
                                                                       quads);
}

void launch_sw_finalize(const double* su, const double* sd, const double* plev, const double* coszen, int ncol,
                        int nlay, double* swuflx, double* swdflx, double* swhr, double* swuflxc, double* swdflxc,
                        double* swhrc, cudaStream_t s, const double* suc, const double* sdc) {
  sw_finalize_kernel<<<dim3((ncol + 127) / 128, nlay + 1), 128, 0, s>>>(su, sd, plev, coszen, ncol, nlay, swuflx, swdflx, swhr,
                                                        swuflxc, swdflxc, swhrc, suc, sdc);
}

}  // namespace rrtmg
