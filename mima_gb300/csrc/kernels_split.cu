// FP32-split instantiation of the g-point solvers: gas optics, transmittance
// lookups and per-g recursions in FP32 (multiply-add contraction allowed);
// g-point sums, band partials and everything downstream stay FP64.
#include "kernels.cuh"
#include "launch.h"

namespace rrtmg {

cudaError_t upload_constants_split(const LwConst& lw, const SwConst& sw) {
  cudaError_t e = cudaMemcpyToSymbol(c_lw, &lw, sizeof(LwConst));
  if (e != cudaSuccess) return e;
  const LwConstF f = make_lwconstf(lw);
  e = cudaMemcpyToSymbol(c_lwf, &f, sizeof(LwConstF));
  if (e != cudaSuccess) return e;
  return cudaMemcpyToSymbol(c_sw, &sw, sizeof(SwConst));
}

void launch_lw_gpoint_split(const LwPrepT<float>& p, const double* emis, const double* tauaer, const float* tab,
                            const float* exptbl, const float* tfntbl, double* bu, double* bd, double* bdu, int ncol,
                            int nlay, int idrv, int nb, int analytic, cudaStream_t s) {
  if (maxl_for(nlay) == 64)
    lw_gpoint_kernel<float, 64><<<nb, kBlock, 0, s>>>(p, emis, tauaer, tab, exptbl, tfntbl, bu, bd, bdu, ncol, nlay, idrv, analytic);
  else
    lw_gpoint_kernel<float, 208><<<nb, kBlock, 0, s>>>(p, emis, tauaer, tab, exptbl, tfntbl, bu, bd, bdu, ncol, nlay, idrv, analytic);
}

void launch_sw_gpoint_split(const SwPrepT<float>& p, const SwIn& in, double adjflux, int iaer, const float* tab,
                            const double* tab64, const float* exptbl, double* su, double* sd, int ncol, int nlay,
                            int nb, int analytic, cudaStream_t s) {
  if (maxl_for(nlay) == 64)
    sw_gpoint_kernel<float, 64><<<nb, kBlock, 0, s>>>(p, in, adjflux, iaer, tab, tab64, exptbl, su, sd, ncol, nlay, analytic);
  else
    sw_gpoint_kernel<float, 208><<<nb, kBlock, 0, s>>>(p, in, adjflux, iaer, tab, tab64, exptbl, su, sd, ncol, nlay, analytic);
}

}  // namespace rrtmg
