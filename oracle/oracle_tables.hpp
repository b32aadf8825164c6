// CPU oracle for the RRTMG clear-sky column-radiation path -- TEST
// INFRASTRUCTURE ONLY.  Nothing in the product links or calls this code; only
// tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg do, as the
// checker.
//
// This header: the coefficient-table store of the oracle.  It reads the
// unreduced (16 g-points per band) tables from the table blob written by
// mima_gb300/tables.py and performs the reference's initialisation steps:
//   * rwgt from wt/ngc/ngn/ngm      rrtmg_lw_init.f90:130-155, rrtmg_sw_init.f90:108-134
//   * g-point reduction cmbgb*      rrtmg_lw_init.f90:366-2015 (cmbgb1..16),
//                                   rrtmg_sw_init.f90:473-1516 (cmbgb16s..29):
//       k-type tables   reduced(..., igc) = sum_ipr orig(..., iprsm) * rwgt(iprsm + off)
//       fracref*/sfluxref*          plain sums (no weights)
//   * lookup tables                 rrtmg_lw_init.f90:106-124, rrtmg_sw_init.f90:96-104
//
// Parity status: the oracle is a restatement; the reference Fortran cannot be
// compiled here (no Fortran compiler), and the reference ships no golden
// vectors for this path, so parity of the oracle itself is unpinned.
#pragma once
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

namespace orc {

// Fortran-style array: column-major, explicit lower bounds, 1..4 dims.
struct FArr {
  std::vector<double> v;
  int ndim = 0;
  int lb[4] = {1, 1, 1, 1};
  int n[4] = {1, 1, 1, 1};
  size_t size() const { return v.size(); }
  size_t off(int i, int j = 0, int k = 0, int l = 0) const {
    size_t o = (size_t)(i - lb[0]);
    if (ndim > 1) o += (size_t)n[0] * (size_t)(j - lb[1]);
    if (ndim > 2) o += (size_t)n[0] * n[1] * (size_t)(k - lb[2]);
    if (ndim > 3) o += (size_t)n[0] * n[1] * n[2] * (size_t)(l - lb[3]);
    return o;
  }
  double operator()(int i) const { return v[off(i)]; }
  double operator()(int i, int j) const { return v[off(i, j)]; }
  double operator()(int i, int j, int k) const { return v[off(i, j, k)]; }
  double operator()(int i, int j, int k, int l) const { return v[off(i, j, k, l)]; }
  double& at(int i, int j = 0, int k = 0, int l = 0) { return v[off(i, j, k, l)]; }
  // Fortran EQUIVALENCE of ka(..,ng) with absa(prod(..), ng): 2-D flat view.
  double flat(int ind, int ig) const {
    size_t inner = v.size() / (size_t)n[ndim - 1];
    return v[(size_t)(ind - 1) + inner * (size_t)(ig - 1)];
  }
};

struct Blob {
  std::map<std::string, FArr> real;
  std::map<std::string, std::vector<int>> ints;

  static uint64_t checksum(const unsigned char* p, size_t nbytes) {
    uint64_t s = 0;
    size_t nw = (nbytes + 7) / 8;
    for (size_t w = 0; w < nw; ++w) {
      uint64_t word = 0;
      for (int b = 0; b < 8; ++b) {
        size_t i = w * 8 + b;
        if (i < nbytes) word |= (uint64_t)p[i] << (8 * b);
      }
      s += word * (uint64_t)(2 * w + 1);
    }
    return s ^ (uint64_t)nbytes;
  }

  void load(const char* path) {
    FILE* f = std::fopen(path, "rb");
    if (!f) throw std::runtime_error(std::string("cannot open table blob ") + path);
    std::fseek(f, 0, SEEK_END);
    long sz = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    std::vector<unsigned char> d((size_t)sz);
    if (std::fread(d.data(), 1, d.size(), f) != d.size()) {
      std::fclose(f);
      throw std::runtime_error("short read on table blob");
    }
    std::fclose(f);
    if (sz < 24 || std::memcmp(d.data(), "RRTMGTB1", 8) != 0)
      throw std::runtime_error("not an RRTMG table blob");
    uint64_t stored;
    std::memcpy(&stored, d.data() + sz - 8, 8);
    if (checksum(d.data(), (size_t)sz - 8) != stored)
      throw std::runtime_error("table blob checksum mismatch");
    uint32_t count;
    std::memcpy(&count, d.data() + 12, 4);
    size_t p = 16;
    for (uint32_t e = 0; e < count; ++e) {
      char name[49] = {0};
      std::memcpy(name, d.data() + p, 48);
      uint32_t dtype, ndim;
      int32_t lbs[4];
      uint32_t dims[4];
      uint64_t off, nb;
      std::memcpy(&dtype, d.data() + p + 48, 4);
      std::memcpy(&ndim, d.data() + p + 52, 4);
      std::memcpy(lbs, d.data() + p + 56, 16);
      std::memcpy(dims, d.data() + p + 72, 16);
      std::memcpy(&off, d.data() + p + 88, 8);
      std::memcpy(&nb, d.data() + p + 96, 8);
      p += 104;
      if (dtype == 1) {
        std::vector<int> iv(nb / 4);
        std::memcpy(iv.data(), d.data() + off, nb);
        ints[name] = iv;
      } else {
        FArr a;
        a.ndim = (int)ndim;
        for (int k = 0; k < 4; ++k) {
          a.lb[k] = lbs[k];
          a.n[k] = (int)dims[k];
        }
        a.v.resize(nb / 8);
        std::memcpy(a.v.data(), d.data() + off, nb);
        if (a.ndim == 0) a.ndim = 1;
        real[name] = a;
      }
    }
  }
  const FArr& r(const std::string& k) const {
    auto it = real.find(k);
    if (it == real.end()) throw std::runtime_error("table missing from blob: " + k);
    return it->second;
  }
  bool has(const std::string& k) const { return real.count(k) != 0; }
  const std::vector<int>& i(const std::string& k) const {
    auto it = ints.find(k);
    if (it == ints.end()) throw std::runtime_error("int table missing from blob: " + k);
    return it->second;
  }
};

// g-point reduction of one table.  gpos = index of the g dimension (0 = first,
// ndim-1 = last).  Follows the cmbgb loops: for every fixed non-g index, for
// igc = 1..ngc(band): sum over the ngn(ngs(band-1)+igc) original g-points.
inline FArr reduce_g(const FArr& o, int gpos, int ngc, const int* ngn_band,
                     const double* rwgt_band, bool weighted) {
  FArr r = o;
  r.n[gpos] = ngc;
  size_t total = 1;
  for (int k = 0; k < r.ndim; ++k) total *= (size_t)r.n[k];
  r.v.assign(total, 0.0);
  // Strides of the original array.
  size_t so[4], sr[4];
  so[0] = sr[0] = 1;
  for (int k = 1; k < 4; ++k) {
    so[k] = so[k - 1] * (size_t)o.n[k - 1];
    sr[k] = sr[k - 1] * (size_t)r.n[k - 1];
  }
  // Iterate over all non-g index tuples.
  int cnt[4] = {0, 0, 0, 0};
  int lim[4];
  for (int k = 0; k < 4; ++k) lim[k] = (k == gpos || k >= o.ndim) ? 1 : o.n[k];
  for (cnt[3] = 0; cnt[3] < lim[3]; ++cnt[3])
    for (cnt[2] = 0; cnt[2] < lim[2]; ++cnt[2])
      for (cnt[1] = 0; cnt[1] < lim[1]; ++cnt[1])
        for (cnt[0] = 0; cnt[0] < lim[0]; ++cnt[0]) {
          size_t bo = 0, br = 0;
          for (int k = 0; k < 4; ++k) {
            bo += so[k] * (size_t)cnt[k];
            br += sr[k] * (size_t)cnt[k];
          }
          int iprsm = 0;
          for (int igc = 0; igc < ngc; ++igc) {
            double sum = 0.0;
            for (int ipr = 0; ipr < ngn_band[igc]; ++ipr) {
              ++iprsm;
              double val = o.v[bo + so[gpos] * (size_t)(iprsm - 1)];
              if (weighted)
                sum = sum + val * rwgt_band[iprsm - 1];
              else
                sum = sum + val;
            }
            r.v[br + sr[gpos] * (size_t)igc] = sum;
          }
        }
  return r;
}

// rwgt for all bands: rrtmg_lw_init.f90:130-155 / rrtmg_sw_init.f90:108-134.
inline std::vector<double> make_rwgt(int nbnd, const std::vector<int>& ngc,
                                     const std::vector<int>& ngn,
                                     const std::vector<int>& ngm,
                                     const FArr& wt) {
  const int mg = 16;
  std::vector<double> rwgt((size_t)nbnd * mg, 0.0);
  int igcsm = 0;
  for (int ibnd = 1; ibnd <= nbnd; ++ibnd) {
    int iprsm = 0;
    double wtsm[16];
    if (ngc[ibnd - 1] < mg) {
      for (int igc = 1; igc <= ngc[ibnd - 1]; ++igc) {
        igcsm = igcsm + 1;
        double wtsum = 0.0;
        for (int ipr = 1; ipr <= ngn[igcsm - 1]; ++ipr) {
          iprsm = iprsm + 1;
          wtsum = wtsum + wt(iprsm);
        }
        wtsm[igc - 1] = wtsum;
      }
      for (int ig = 1; ig <= mg; ++ig) {
        int ind = (ibnd - 1) * mg + ig;
        rwgt[ind - 1] = wt(ig) / wtsm[ngm[ind - 1] - 1];
      }
    } else {
      for (int ig = 1; ig <= mg; ++ig) {
        igcsm = igcsm + 1;
        int ind = (ibnd - 1) * mg + ig;
        rwgt[ind - 1] = 1.0;
      }
    }
  }
  return rwgt;
}

}  // namespace orc
