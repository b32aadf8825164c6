// GCM-side kernels of the radiation driver: MiMA's run_rrtmg
// (src/atmos_param/rrtm_radiation/rrtm_radiation.f90:464-834), interp_temp
// (:420-460) and compute_zenith (src/atmos_param/rrtm_radiation/astro.f90:59-248)
// on the device, so that a GCM slab goes to RRTM columns and back without
// leaving HBM.
//
// Everything here is O(points x levels) data movement with a few FP64
// operations per element (HBM-bound, microseconds at T85).  The arithmetic
// uses explicitly rounded operations (no contraction into FMA) in the
// reference's evaluation order, so that the results are bit-identical to an
// IEEE restatement of the Fortran; only sin/cos/tan/acos of the zenith angle
// are the CUDA library's.
#include <cuda_runtime.h>

#include "driver.h"

namespace rrtmg {
namespace {

constexpr double kPi = 3.14159265358979323846;  // FMS constants_mod PI
constexpr double kDayPerSec = 1.0 / 86400.0;    // daypersec (rrtm_radiation.f90:104)

__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dvd(double a, double b) { return __ddiv_rn(a, b); }
// a*x + b*y as two products and a sum (the reference's interpolations)
__device__ __forceinline__ double lin2(double a, double x, double b, double y) { return add(mul(a, x), mul(b, y)); }

// compute_zenith (astro.f90:120-246) at one point; radsec, dt_pi and the
// declination terms are the host's (astro.f90:113-137).
__device__ double zenith(const RunScalars& s, double lat, double lon) {
  const double twopi = mul(2.0, kPi);
  // local time in [-pi, pi) (:121-126): Fortran modulo(x, 2 pi)
  double tp = fmod(add(s.radsec, lon), twopi);
  if (tp < 0.0) tp = add(tp, twopi);
  tp = sub(tp, kPi);
  if (tp >= kPi) tp = sub(tp, twopi);
  if (tp < -kPi) tp = add(tp, twopi);
  // half-day length (:140-147)
  double lat_h = lat;
  if (lat_h == mul(0.5, kPi)) lat_h = sub(lat, 1.0e-5);
  if (lat_h == -mul(0.5, kPi)) lat_h = add(lat, 1.0e-5);
  const double cos_h = mul(-tan(lat_h), s.dec_tan);
  double h;
  if (cos_h <= -1.0)
    h = kPi;
  else if (cos_h >= 1.0)
    h = 0.0;
  else
    h = acos(cos_h);
  const double aa = mul(sin(lat), s.dec_sin), bb = mul(cos(lat), s.dec_cos);
  double cosz;
  const int dt = s.zen_dt;
  if (dt > 0 && dt < 86400) {
    // mean over [t, t + dt] (:156-227): the reference's eight cases in order
    const double tt = add(tp, s.dt_pi), st = sin(tp), stt = sin(tt), sh = sin(h);
    const double ddt = (double)dt;
    cosz = 0.0;
    if (add(tt, h) != 0.0 && tp < -h && fabs(tt) <= h) cosz = add(aa, dvd(mul(bb, add(stt, sh)), add(tt, h)));
    if (tp < -h && h != 0.0 && h < tt) cosz = add(aa, dvd(mul(bb, add(sh, sh)), add(h, h)));
    if (fabs(tp) <= h && fabs(tt) <= h) cosz = add(aa, dvd(mul(bb, sub(stt, st)), sub(tt, tp)));
    if (sub(h, tp) != 0.0 && fabs(tp) <= h && h < tt) cosz = add(aa, dvd(mul(bb, sub(sh, st)), sub(h, tp)));
    const double tth = sub(add(tt, h), twopi);
    if (sub(twopi, h) < tt && tth != 0.0 && tp <= h)
      cosz = dvd(add(mul(cosz, sub(h, tp)), add(mul(aa, tth), mul(bb, add(stt, sh)))), add(sub(h, tp), tth));
    if (h < tp && sub(twopi, h) >= tt) cosz = 0.0;
    if (h < tp && sub(twopi, h) < tt) cosz = add(aa, dvd(mul(bb, add(stt, sh)), tth));
    // fraction of the interval with the sun up (:221-227)
    double fr = 0.0;
    if (tp < -h && tt < -h) fr = 0.0;
    if (tp < -h && fabs(tt) <= h) fr = dvd(add(tt, h), ddt);
    if (tp < -h && h < tt) fr = dvd(add(h, h), ddt);
    if (fabs(tp) <= h && fabs(tt) <= h) fr = dvd(sub(tt, tp), ddt);
    if (fabs(tp) <= h && h < tt) fr = dvd(sub(h, tp), ddt);
    if (h < tp) fr = 0.0;
    if (sub(twopi, h) < tt) fr = add(fr, dvd(tth, ddt));
    cosz = dvd(mul(cosz, fr), s.radpersec);
  } else if (dt >= 86400) {
    cosz = dvd(add(mul(aa, h), mul(bb, sin(h))), kPi);  // daily mean (:233)
  } else {
    cosz = fabs(tp) <= h ? add(aa, mul(bb, cos(tp))) : 0.0;  // instantaneous (:238-243)
  }
  return cosz > 0.0 ? cosz : 0.0;  // max(0, cosz) (:246)
}

// t_half of interp_temp (rrtm_radiation.f90:430-457) at half level kh
// (0 = model top, sk = surface) of point p.
__device__ __forceinline__ double thalf_at(const RunGcm& g, size_t p, size_t plane, int kh, int sk) {
  if (kh == 0) return mul(0.5, sub(mul(3.0, g.t[p]), g.t[p + plane]));
  if (kh == sk) return g.t_surf[p];
  const double zf0 = g.z_full[p + plane * (kh - 1)], zf1 = g.z_full[p + plane * kh];
  const double zh = g.z_half[p + plane * kh];
  const double dzk2 = dvd(1.0, sub(zf0, zf1));
  const double dzk = mul(sub(zh, zf1), dzk2), dzk1 = mul(sub(zf0, zh), dzk2);
  return lin2(g.t[p + plane * kh], dzk1, g.t[p + plane * (kh - 1)], dzk);
}

// max(x, lo) then min(x, hi) of rrtm_radiation.f90:673-677; a NaN passes
// through (and is then flagged by the RRTM input validation).
__device__ __forceinline__ double clamp(double x, double lo, double hi) {
  x = x < lo ? lo : x;
  return x > hi ? hi : x;
}

// One block per latitude.
__global__ void run_zonal_kernel(RunScalars s, RunGcm g, double* __restrict__ coszen, double* __restrict__ zq,
                                 double* __restrict__ zp, unsigned* __restrict__ flag) {
  const int j = blockIdx.x;
  const size_t plane = (size_t)s.si * s.sj, row = (size_t)s.si * j;
  for (int i = threadIdx.x; i < s.si; i += blockDim.x) coszen[row + i] = zenith(s, g.lat[row + i], g.lon[row + i]);
  // top interface of the RRTM columns (:655-656): is some p_half(:,:,1) * 0.01 <= 0?
  for (int i = threadIdx.x; i < s.nsub; i += blockDim.x)
    if (mul(g.p_half[row + (size_t)i * s.lonstep], 0.01) <= 0.0) atomicOr(flag, 1u);
  // do_zm_tracers (:613-617): sum(q, 1) / size(q, 1), summed in index order
  if (s.zm_tracers)
    for (int k = threadIdx.x; k < s.sk; k += blockDim.x) {
      const double* q = g.q + row + plane * k;
      double acc = 0.0;
      for (int i = 0; i < s.si; ++i) acc = add(acc, q[i]);
      zq[j + (size_t)s.sj * k] = dvd(acc, (double)s.si);
    }
  // do_precip_albedo (:604-611): zonal sum of rrtm_precip, zeroed equatorward of precip_lat
  if (s.precip_albedo && threadIdx.x == 0) {
    const double lim = dvd(mul(s.precip_lat, 3.14159265), 180.0);
    double acc = 0.0;
    for (int i = 0; i < s.si; ++i) acc = add(acc, fabs(g.lat[row + i]) < lim ? 0.0 : g.precip[row + i]);
    zp[j] = acc;
  }
}

// Thread (column, row): row l < sk prepares layer l, every row l <= sk level l.
__global__ void run_prep_kernel(RunScalars s, RunGcm g, const double* __restrict__ coszen,
                                const double* __restrict__ zq, const double* __restrict__ zp,
                                const unsigned* __restrict__ flag, RunCols c) {
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= s.ncol) return;
  const int l = blockIdx.y, sk = s.sk;
  const int isub = col % s.nsub, j = col / s.nsub;
  const size_t N = s.ncol, plane = (size_t)s.si * s.sj;
  const size_t p = (size_t)isub * s.lonstep + (size_t)s.si * j;
  if (l < sk) {
    // layer l <- GCM full level sk-1-l (:652-660, :673-677)
    const int k = sk - 1 - l;
    const size_t gi = p + plane * k, o = (size_t)l * N + col;
    const double pf = g.p_full[gi];
    c.play[o] = mul(pf, 0.01);
    c.tlay[o] = clamp(g.t[gi], s.t_lo, s.t_hi);
    double q = s.zm_tracers ? zq[j + (size_t)s.sj * k] : g.q[gi];
    // do_fixed_water (:631-641)
    if (s.fixed_water && fabs(g.lat[p]) <= s.fixed_water_lat && pf <= mul(s.fixed_water_pres, 100.0))
      q = s.fixed_water_val;
    c.h2o[o] = q < s.h2o_lo ? s.h2o_lo : q;
    c.o3[o] = g.o3 ? g.o3[gi] : s.o3_val;
    c.co2[o] = s.co2;
    if (s.secondary)
      for (int m = 0; m < 7; ++m) c.gas[m][o] = s.gas_val[m];
  }
  {
    // level l <- GCM half level sk-l (:653-658); top fix pfull(:,sk) * 0.5
    const int kh = sk - l;
    const size_t o = (size_t)l * N + col;
    c.plev[o] = (l == sk && *flag) ? mul(mul(g.p_full[p], 0.01), 0.5) : mul(g.p_half[p + plane * kh], 0.01);
    c.tlev[o] = clamp(thalf_at(g, p, plane, kh, sk), s.t_lo, s.t_hi);
  }
  if (l == 0) {
    c.tsfc[col] = g.t_surf[p];
    c.cosz[col] = coszen[p];
    double a = g.albedo[p];
    if (s.precip_albedo)  // albedo + (precip_albedo - albedo) * sum / size / num_precip
      a = add(a, dvd(dvd(mul(sub(s.precip_albedo_val, a), zp[j]), (double)s.si), (double)s.num_precip));
    c.alb[col] = a;
    for (int b = 0; b < 16; ++b) c.emis[(size_t)b * N + col] = 1.0;
  }
}

__global__ void run_thalf_kernel(RunScalars s, RunGcm g, double* __restrict__ t_half) {
  const size_t plane = (size_t)s.si * s.sj;
  const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= plane) return;
  const int kh = blockIdx.y;
  t_half[p + plane * kh] = thalf_at(g, p, plane, kh, s.sk);
}

// Thread per (latitude, level) and per latitude (k == sk): do_zm_rad means
// (:768-769, :801-803), summed in index order.
__global__ void run_zonal_rad_kernel(RunScalars s, RunRad r, double* __restrict__ zt, double* __restrict__ zsw,
                                     double* __restrict__ zlw) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= s.sj * (s.sk + 1)) return;
  const int j = t % s.sj, k = t / s.sj;
  const size_t N = s.ncol, c0 = (size_t)s.nsub * j;
  const double n = (double)(s.nsub > 1 ? s.nsub : 1);
  if (k < s.sk) {
    const size_t o = (size_t)(s.sk - 1 - k) * N + c0;
    double acc = 0.0;
    for (int i = 0; i < s.nsub; ++i) acc = add(acc, add(mul(r.swhr[o + i], kDayPerSec), mul(r.hr[o + i], kDayPerSec)));
    zt[j + (size_t)s.sj * k] = dvd(acc, n);
  } else {
    double a = 0.0, b = 0.0;
    for (int i = 0; i < s.nsub; ++i) {
      a = add(a, sub(r.swdflx[c0 + i], r.swuflx[c0 + i]));
      b = add(b, r.dflx[c0 + i]);
    }
    zsw[j] = dvd(a, n);
    zlw[j] = dvd(b, n);
  }
}

// Thread (GCM point, row): row k < sk is full level k, row sk the surface
// and top-of-atmosphere fields (:715-716, :751-815).
__global__ void run_post_kernel(RunScalars s, RunRad r, const double* __restrict__ zt,
                                const double* __restrict__ zsw, const double* __restrict__ zlw, RunOut o) {
  const size_t plane = (size_t)s.si * s.sj;
  const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= plane) return;
  const int k = blockIdx.y;
  const int i = (int)(p % s.si), j = (int)(p / s.si);
  // lonstep interpolation, closed toroidally (:760-771)
  const int isub = i / s.lonstep, isub1 = isub + 1 < s.nsub ? isub + 1 : 0;
  const double di = mul((double)(i % s.lonstep), dvd(1.0, (double)s.lonstep)), omd = sub(1.0, di);
  const size_t N = s.ncol, c0 = isub + (size_t)s.nsub * j, c1 = isub1 + (size_t)s.nsub * j;
  if (k < s.sk) {
    const size_t l = (size_t)(s.sk - 1 - k) * N;
    const double sw0 = mul(r.swhr[l + c0], kDayPerSec), sw1 = mul(r.swhr[l + c1], kDayPerSec);
    const double lw0 = mul(r.hr[l + c0], kDayPerSec), lw1 = mul(r.hr[l + c1], kDayPerSec);
    const double td = s.zm_rad ? zt[j + (size_t)s.sj * k] : lin2(di, add(sw1, lw1), omd, add(sw0, lw0));
    const size_t gi = p + plane * k;
    o.tdt[gi] = add(o.tdt[gi], td);
    if (o.tdt_rad) o.tdt_rad[gi] = td;
    if (o.tdt_sw) o.tdt_sw[gi] = lin2(di, sw1, omd, sw0);
    if (o.tdt_lw) o.tdt_lw[gi] = lin2(di, lw1, omd, lw0);
    return;
  }
  const size_t top = (size_t)s.sk * N;
  if (o.olr) o.olr[p] = lin2(di, r.uflx[top + c1], omd, r.uflx[top + c0]);
  if (o.isr)
    o.isr[p] = lin2(di, sub(r.swdflx[top + c1], r.swuflx[top + c1]), omd, sub(r.swdflx[top + c0], r.swuflx[top + c0]));
  if (o.flux_sw)
    o.flux_sw[p] = s.zm_rad ? zsw[j] : lin2(di, sub(r.swdflx[c1], r.swuflx[c1]), omd, sub(r.swdflx[c0], r.swuflx[c0]));
  if (o.flux_lw) o.flux_lw[p] = s.zm_rad ? zlw[j] : lin2(di, r.dflx[c1], omd, r.dflx[c0]);
}

}  // namespace

void launch_run_zonal(const RunScalars& s, const RunGcm& g, double* coszen, double* zq, double* zp, unsigned* flag,
                      cudaStream_t st) {
  run_zonal_kernel<<<s.sj, 128, 0, st>>>(s, g, coszen, zq, zp, flag);
}

void launch_run_prep(const RunScalars& s, const RunGcm& g, const double* coszen, const double* zq,
                     const double* zp, const unsigned* flag, const RunCols& c, cudaStream_t st) {
  run_prep_kernel<<<dim3((s.ncol + 127) / 128, s.sk + 1), 128, 0, st>>>(s, g, coszen, zq, zp, flag, c);
}

void launch_run_thalf(const RunScalars& s, const RunGcm& g, double* t_half, cudaStream_t st) {
  const size_t plane = (size_t)s.si * s.sj;
  run_thalf_kernel<<<dim3((unsigned)((plane + 127) / 128), s.sk + 1), 128, 0, st>>>(s, g, t_half);
}

void launch_run_zonal_rad(const RunScalars& s, const RunRad& r, double* zt, double* zsw, double* zlw,
                          cudaStream_t st) {
  const int n = s.sj * (s.sk + 1);
  run_zonal_rad_kernel<<<(n + 127) / 128, 128, 0, st>>>(s, r, zt, zsw, zlw);
}

void launch_run_post(const RunScalars& s, const RunRad& r, const double* zt, const double* zsw, const double* zlw,
                     const RunOut& o, cudaStream_t st) {
  const size_t plane = (size_t)s.si * s.sj;
  run_post_kernel<<<dim3((unsigned)((plane + 127) / 128), s.sk + 1), 128, 0, st>>>(s, r, zt, zsw, zlw, o);
}

}  // namespace rrtmg
