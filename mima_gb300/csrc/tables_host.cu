// Host-side construction of the device coefficient tables.
//
// Reads the unreduced 16-g tables from the table blob (format documented in
// mima_gb300/tables.py), computes the reduction weights rwgt
// (rrtmg_lw_init.f90:130-155, rrtmg_sw_init.f90:108-134), reduces every table
// to the 140 / 112 g-point sets following cmbgb1..16 / cmbgb16s..29
// (k-type tables weighted by rwgt, Planck fractions and solar source summed
// plainly), and lays each reduced table out for the device with the g-point
// index fastest: element (non-g indices in Fortran order, g) at
// nong_flat * ng + g.  Also builds the transmittance / tau-transition lookup
// tables (rrtmg_lw_init.f90:106-124, rrtmg_sw_init.f90:96-104) and the
// constant-memory blocks.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>

#include "lw_optics.cuh"
#include "sw_optics.cuh"
#include "tables_host.h"

namespace rrtmg {
namespace {

struct Arr {
  bool is_int = false;
  std::vector<double> d;
  std::vector<int> iv;
  std::vector<int> dims;
};

using ArrMap = std::map<std::string, Arr>;

uint64_t blob_checksum(const unsigned char* p, size_t n) {
  uint64_t s = 0;
  const size_t nw = (n + 7) / 8;
  for (size_t w = 0; w < nw; ++w) {
    uint64_t word = 0;
    const size_t base = w * 8;
    const size_t take = (base + 8 <= n) ? 8 : n - base;
    std::memcpy(&word, p + base, take);  // little-endian host
    s += word * (uint64_t)(2 * w + 1);
  }
  return s ^ (uint64_t)n;
}

std::string read_blob(const char* path, ArrMap& out) {
  if (!path) return "table blob path is null";
  FILE* f = std::fopen(path, "rb");
  if (!f) return std::string("cannot open table blob: ") + path;
  std::vector<unsigned char> buf;
  unsigned char tmp[1 << 16];
  size_t got;
  while ((got = std::fread(tmp, 1, sizeof tmp, f)) > 0) buf.insert(buf.end(), tmp, tmp + got);
  std::fclose(f);
  if (buf.size() < 24 || std::memcmp(buf.data(), "RRTMGTB1", 8) != 0) return "not an RRTMG table blob";
  uint64_t stored;
  std::memcpy(&stored, buf.data() + buf.size() - 8, 8);
  if (blob_checksum(buf.data(), buf.size() - 8) != stored) return "table blob checksum mismatch";
  uint32_t count;
  std::memcpy(&count, buf.data() + 12, 4);
  const size_t rec = 48 + 4 + 4 + 16 + 16 + 8 + 8;
  if (16 + (size_t)count * rec > buf.size()) return "table blob header truncated";
  for (uint32_t e = 0; e < count; ++e) {
    const unsigned char* r = buf.data() + 16 + (size_t)e * rec;
    char name[49];
    std::memcpy(name, r, 48);
    name[48] = 0;
    uint32_t dtype, ndim, dims[4];
    uint64_t off, nb;
    std::memcpy(&dtype, r + 48, 4);
    std::memcpy(&ndim, r + 52, 4);
    std::memcpy(dims, r + 72, 16);
    std::memcpy(&off, r + 88, 8);
    std::memcpy(&nb, r + 96, 8);
    // every entry: a known type, at most 4 dimensions, its bytes inside the
    // file, a whole number of elements, and as many elements as its dimensions
    const uint64_t esz = dtype == 1 ? 4 : 8;
    if ((dtype != 0 && dtype != 1) || ndim > 4 || off > buf.size() || nb > buf.size() - off || nb % esz != 0)
      return std::string("table blob entry out of range: ") + name;
    uint64_t n = 1;
    bool fits = true;
    for (uint32_t k = 0; k < ndim && fits; ++k) {
      fits = dims[k] <= 0x7fffffffu && (dims[k] == 0 || n <= (nb / esz) / dims[k]);
      n *= dims[k];
    }
    if (!fits || n != nb / esz) return std::string("table blob entry size does not match its dimensions: ") + name;
    Arr a;
    for (uint32_t k = 0; k < ndim; ++k) a.dims.push_back((int)dims[k]);
    if (dtype == 1) {
      a.is_int = true;
      a.iv.resize(nb / 4);
      std::memcpy(a.iv.data(), buf.data() + off, nb);
    } else {
      a.d.resize(nb / 8);
      std::memcpy(a.d.data(), buf.data() + off, nb);
    }
    out[name] = a;
  }
  return "";
}

// Reduction weights for nbnd bands of 16 original g-points each.
std::vector<double> reduction_weights(int nbnd, const std::vector<int>& ngc, const std::vector<int>& ngn,
                                      const std::vector<int>& ngm, const std::vector<double>& wt) {
  std::vector<double> rwgt((size_t)nbnd * 16);
  int igcsm = 0;
  for (int b = 0; b < nbnd; ++b) {
    double wtsm[16] = {0};
    int iprsm = 0;
    if (ngc[b] < 16) {
      for (int igc = 0; igc < ngc[b]; ++igc) {
        double wtsum = 0.0;
        for (int ipr = 0; ipr < ngn[igcsm]; ++ipr) wtsum = wtsum + wt[iprsm++];
        wtsm[igc] = wtsum;
        ++igcsm;
      }
      for (int ig = 0; ig < 16; ++ig) rwgt[(size_t)b * 16 + ig] = wt[ig] / wtsm[ngm[(size_t)b * 16 + ig] - 1];
    } else {
      for (int ig = 0; ig < 16; ++ig) rwgt[(size_t)b * 16 + ig] = 1.0;
      igcsm += 16;
    }
  }
  return rwgt;
}

// Pads a table to a multiple of 4 elements, so that the next band's tables
// start 16-byte aligned in FP32 and FP64 (the bulk-copy unit's alignment).
void pad4(std::vector<double>& v) {
  while (v.size() % 4) v.push_back(0.0);
}

// Reduce one table along axis gaxis to ngc g-points and append it to dst in
// device layout.  Returns the element offset.
int reduce_append(const Arr& a, int gaxis, int ngc, const int* ngn, const double* rw, bool weighted,
                  std::vector<double>& dst) {
  const int nd = (int)a.dims.size();
  size_t stride[4] = {1, 1, 1, 1};
  for (int k = 1; k < nd; ++k) stride[k] = stride[k - 1] * (size_t)a.dims[k - 1];
  size_t nong = 1;
  for (int k = 0; k < nd; ++k)
    if (k != gaxis) nong *= (size_t)a.dims[k];
  const int off = (int)dst.size();
  dst.resize(dst.size() + nong * (size_t)ngc);
  // enumerate non-g index tuples in Fortran order
  std::vector<int> ix(nd, 0);
  for (size_t r = 0; r < nong; ++r) {
    size_t base = 0;
    for (int k = 0; k < nd; ++k)
      if (k != gaxis) base += stride[k] * (size_t)ix[k];
    int src = 0;
    for (int igc = 0; igc < ngc; ++igc) {
      double sum = 0.0;
      for (int ipr = 0; ipr < ngn[igc]; ++ipr, ++src) {
        const double v = a.d[base + stride[gaxis] * (size_t)src];
        sum = weighted ? sum + v * rw[src] : sum + v;
      }
      dst[off + r * (size_t)ngc + igc] = sum;
    }
    for (int k = 0; k < nd; ++k) {  // increment the tuple, skipping gaxis
      if (k == gaxis) continue;
      if (++ix[k] < a.dims[k]) break;
      ix[k] = 0;
    }
  }
  return off;
}

const Arr* find(const ArrMap& m, const std::string& k) {
  auto it = m.find(k);
  return it == m.end() ? nullptr : &it->second;
}

std::vector<int> ints(const ArrMap& m, const std::string& k, std::string& err) {
  const Arr* a = find(m, k);
  if (!a || !a->is_int) {
    err = "table blob lacks " + k;
    return {};
  }
  return a->iv;
}
std::vector<double> reals(const ArrMap& m, const std::string& k, std::string& err) {
  const Arr* a = find(m, k);
  if (!a || a->is_int) {
    err = "table blob lacks " + k;
    return {};
  }
  return a->d;
}

// Table role of an unreduced LW table name in band b.
int lw_role(int b, const std::string& n) {
  if (n == "kao") return LW_KA;
  if (n == "kbo") return LW_KB;
  if (n == "selfrefo") return LW_SELF;
  if (n == "forrefo") return LW_FOR;
  if (n == "fracrefao") return LW_FRA;
  if (n == "fracrefbo") return LW_FRB;
  switch (b) {
    case 8:
      if (n == "kao_mco2") return LW_MA1;
      if (n == "kao_mo3") return LW_MA2;
      if (n == "kao_mn2o") return LW_MA3;
      if (n == "kbo_mco2") return LW_MB1;
      if (n == "kbo_mn2o") return LW_MB2;
      if (n == "cfc12o") return LW_X1;
      if (n == "cfc22adjo") return LW_X2;
      break;
    case 13:
      if (n == "kao_mco2") return LW_MA1;
      if (n == "kao_mco") return LW_MA2;
      if (n == "kbo_mo3") return LW_MB1;
      break;
    case 6:
      if (n == "kao_mco2") return LW_MA1;
      if (n == "cfc11adjo") return LW_X1;
      if (n == "cfc12o") return LW_X2;
      break;
    case 5:
      if (n == "kao_mo3") return LW_MA1;
      if (n == "ccl4o") return LW_X1;
      break;
    default:
      if (n.rfind("kao_m", 0) == 0) return LW_MA1;
      if (n.rfind("kbo_m", 0) == 0) return LW_MB1;
      break;
  }
  return -1;
}

int sw_role(int b, const std::string& n) {
  if (n == "kao") return SW_KA;
  if (n == "kbo") return SW_KB;
  if (n == "selfrefo") return SW_SELF;
  if (n == "forrefo") return SW_FOR;
  if (n == "sfluxrefo") return SW_SFLUX;
  if (n == "rayl" || n == "raylo" || n == "raylao") return SW_RAYL;
  if (b == 20 && n == "absch4o") return SW_E1;
  if (b == 24 && n == "raylbo") return SW_E1;
  if ((b == 24 || b == 25) && n == "abso3ao") return SW_E2;
  if ((b == 24 || b == 25) && n == "abso3bo") return SW_E3;
  if (b == 29 && n == "absh2oo") return SW_E1;
  if (b == 29 && n == "absco2o") return SW_E2;
  return -1;
}

void lookup_tables(std::vector<double>& expt, std::vector<double>* tfnt, double bpade) {
  const int ntbl = kNTbl;
  const double expeps = 1.e-20;
  expt.assign(ntbl + 1, 0.0);
  if (tfnt) tfnt->assign(ntbl + 1, 0.0);
  expt[0] = 1.0;
  expt[ntbl] = expeps;
  if (tfnt) {
    (*tfnt)[0] = 0.0;
    (*tfnt)[ntbl] = 1.0;
  }
  for (int itr = 1; itr < ntbl; ++itr) {
    const double tfn = (double)itr / (double)ntbl;
    const double tau = bpade * tfn / (1.0 - tfn);
    double e = std::exp(-tau);
    if (e <= expeps) e = expeps;
    expt[itr] = e;
    if (tfnt) (*tfnt)[itr] = (tau < 0.06) ? tau / 6.0 : 1.0 - 2.0 * ((1.0 / tau) - (e / (1. - e)));
  }
}

}  // namespace

std::string build_host_tables(const char* blob_path, double cpdair, HostTables& T) {
  ArrMap m;
  std::string err = read_blob(blob_path, m);
  if (!err.empty()) return err;
  std::memset(&T.lw, 0, sizeof(LwConst));
  std::memset(&T.sw, 0, sizeof(SwConst));
  T.lw_tab.clear();
  T.sw_tab.clear();

  // ---------------- LW ----------------
  {
    auto ngc = ints(m, "lw.ngc", err), ngn = ints(m, "lw.ngn", err), ngm = ints(m, "lw.ngm", err),
         nspa = ints(m, "lw.nspa", err), nspb = ints(m, "lw.nspb", err);
    auto wt = reals(m, "lw.wt", err), delwave = reals(m, "lw.delwave", err);
    if (!err.empty()) return err;
    if (ngc.size() != 16 || ngn.size() != (size_t)kLwG || ngm.size() != 256) return "LW g-point maps malformed";
    auto rwgt = reduction_weights(16, ngc, ngn, ngm, wt);
    int goff = 0;
    for (int b = 1; b <= 16; ++b) {
      BandDesc& bd = T.lw.band[b - 1];
      if (ngc[b - 1] != lw_ng(b)) return "LW band g-point count differs from the compiled layout";
      bd.ng = ngc[b - 1];
      bd.ngpad = pow2ceil(bd.ng);
      bd.goff = goff;
      bd.nspa = nspa[b - 1];
      bd.nspb = nspb[b - 1];
      bd.delwave = delwave[b - 1];
      for (int r = 0; r < 16; ++r) bd.off[r] = -1;
      pad4(T.lw_tab);
      bd.tbeg = (int)T.lw_tab.size();
      char pre[8];
      std::snprintf(pre, sizeof pre, "lw%02d.", b);
      for (const auto& kv : m) {
        if (kv.first.rfind(pre, 0) != 0) continue;
        const std::string nm = kv.first.substr(5);
        const int role = lw_role(b, nm);
        if (role < 0) return "unrecognised LW table " + kv.first;
        const bool planck = nm.rfind("fracref", 0) == 0;
        const int gaxis = planck ? 0 : (int)kv.second.dims.size() - 1;
        if (kv.second.dims[gaxis] != 16) return "LW table without 16 g-points: " + kv.first;
        bd.off[role] = reduce_append(kv.second, gaxis, bd.ng, &ngn[goff], &rwgt[(size_t)(b - 1) * 16], !planck,
                                     T.lw_tab);
        bd.nrow[role] = kv.second.dims[0];
      }
      for (int r : {LW_KA, LW_SELF, LW_FOR, LW_FRA})
        if (bd.off[r] < 0) return "LW band lacks a key table";
      pad4(T.lw_tab);
      bd.tend = (int)T.lw_tab.size();
      goff += bd.ng;
    }
    // Bands without an upper key table still get a valid pointer.
    for (int b = 0; b < 16; ++b)
      for (int r = 0; r < LW_NROLE; ++r)
        if (T.lw.band[b].off[r] < 0) T.lw.band[b].off[r] = 0;
    auto chi = reals(m, "lw.chi_mls", err), preflog = reals(m, "lw.preflog", err), tref = reals(m, "lw.tref", err);
    T.totplnk = reals(m, "lw.totplnk", err);
    T.totplnkderiv = reals(m, "lw.totplnkderiv", err);
    if (!err.empty()) return err;
    if (chi.size() != 7 * 59 || preflog.size() != 59 || T.totplnk.size() != 181 * 16) return "LW reference data malformed";
    for (size_t k = 0; k < chi.size(); ++k) T.lw.chi[k] = chi[k];
    for (int j = 0; j < 59; ++j) {
      T.lw.preflog[j] = preflog[j];
      T.lw.tref[j] = tref[j];
    }
    auto C = [&](int i, int j) { return chi[(size_t)(j - 1) * 7 + (i - 1)]; };
    for (int jp = 1; jp <= 59; ++jp) {
      T.lw.r_h2oco2[jp] = C(1, jp) / C(2, jp);
      T.lw.r_h2oo3[jp] = C(1, jp) / C(3, jp);
      T.lw.r_h2on2o[jp] = C(1, jp) / C(4, jp);
      T.lw.r_h2och4[jp] = C(1, jp) / C(6, jp);
      T.lw.r_n2oco2[jp] = C(4, jp) / C(2, jp);
      T.lw.r_o3co2[jp] = C(3, jp) / C(2, jp);
    }
    // refrat_planck_a / _b, refrat_m_a / _b (or _a3) of each band
    // (rrtmg_lw_taumol.f90 taugb3..16 preambles).
    auto R = [&](int b, int k, double v) { T.lw.refrat[b - 1][k] = v; };
    R(3, 0, C(1, 9) / C(2, 9)); R(3, 1, C(1, 13) / C(2, 13)); R(3, 2, C(1, 3) / C(2, 3)); R(3, 3, C(1, 13) / C(2, 13));
    R(4, 0, C(1, 11) / C(2, 11)); R(4, 1, C(3, 13) / C(2, 13));
    R(5, 0, C(1, 5) / C(2, 5)); R(5, 1, C(3, 43) / C(2, 43)); R(5, 2, C(1, 7) / C(2, 7));
    R(7, 0, C(1, 3) / C(3, 3)); R(7, 2, C(1, 3) / C(3, 3));
    R(9, 0, C(1, 9) / C(6, 9)); R(9, 2, C(1, 3) / C(6, 3));
    R(12, 0, C(1, 10) / C(2, 10));
    R(13, 0, C(1, 5) / C(4, 5)); R(13, 2, C(1, 1) / C(4, 1)); R(13, 3, C(1, 3) / C(4, 3));
    R(15, 0, C(4, 1) / C(2, 1)); R(15, 2, C(4, 1) / C(2, 1));
    R(16, 0, C(1, 6) / C(6, 6));
    T.lw.grav = 9.8066;
    T.lw.avogad = 6.02214199e+23;
    T.lw.heatfac = T.lw.grav * 8.6400e4 / (cpdair * 1.e2);
    T.lw.oneminus = 1.0 - 1.e-6;
    T.lw.fluxfac = (2.0 * std::asin(1.0)) * 2.e4;
    T.lw.bpade = 1.0 / 0.278;
    lookup_tables(T.lw_exp, &T.lw_tfn, T.lw.bpade);
    // tau_tbl: the optical depth each entry stands for (0 and 1e10 at the ends)
    T.lw_tau.assign(kNTbl + 1, 0.0);
    T.lw_tau[kNTbl] = 1.e10;
    for (int itr = 1; itr < kNTbl; ++itr) {
      const double tfn = (double)itr / (double)kNTbl;
      T.lw_tau[itr] = T.lw.bpade * tfn / (1.0 - tfn);
    }
  }

  // ---------------- SW ----------------
  {
    auto ngc = ints(m, "sw.ngc", err), ngn = ints(m, "sw.ngn", err), ngm = ints(m, "sw.ngm", err),
         nspa = ints(m, "sw.nspa", err), nspb = ints(m, "sw.nspb", err);
    auto wt = reals(m, "sw.wt", err), delwave = reals(m, "sw.delwave", err);
    auto preflog = reals(m, "sw.preflog", err), tref = reals(m, "sw.tref", err);
    if (!err.empty()) return err;
    if (ngc.size() != 14 || ngn.size() != (size_t)kSwG || ngm.size() != 224) return "SW g-point maps malformed";
    auto rwgt = reduction_weights(14, ngc, ngn, ngm, wt);
    int goff = 0;
    for (int b = 16; b <= 29; ++b) {
      const int ib = b - 16;
      BandDesc& bd = T.sw.band[ib];
      if (ngc[ib] != sw_ng(b)) return "SW band g-point count differs from the compiled layout";
      bd.ng = ngc[ib];
      bd.ngpad = pow2ceil(bd.ng);
      bd.goff = goff;
      bd.nspa = nspa[ib];
      bd.nspb = nspb[ib];
      bd.delwave = delwave[ib];
      for (int r = 0; r < 16; ++r) bd.off[r] = -1;
      pad4(T.sw_tab);
      bd.tbeg = (int)T.sw_tab.size();
      char pre[8];
      std::snprintf(pre, sizeof pre, "sw%02d.", b);
      for (const auto& kv : m) {
        if (kv.first.rfind(pre, 0) != 0) continue;
        const std::string nm = kv.first.substr(5);
        const int role = sw_role(b, nm);
        if (role < 0) return "unrecognised SW table " + kv.first;
        if (nm == "rayl") {  // band scalar, not reduced
          bd.off[role] = (int)T.sw_tab.size();
          T.sw_tab.push_back(kv.second.d.at(0));
          continue;
        }
        const bool plain = nm.rfind("sfluxref", 0) == 0;
        const bool gfirst = plain || nm == "raylao";
        const int gaxis = gfirst ? 0 : (int)kv.second.dims.size() - 1;
        if (kv.second.dims[gaxis] != 16) return "SW table without 16 g-points: " + kv.first;
        bd.off[role] = reduce_append(kv.second, gaxis, bd.ng, &ngn[goff], &rwgt[(size_t)ib * 16], !plain, T.sw_tab);
        bd.nrow[role] = kv.second.dims[0];
      }
      if (bd.off[SW_SFLUX] < 0 || bd.off[SW_RAYL] < 0) return "SW band lacks solar source or Rayleigh table";
      pad4(T.sw_tab);
      bd.tend = (int)T.sw_tab.size();
      goff += bd.ng;
    }
    for (int b = 0; b < 14; ++b)
      for (int r = 0; r < SW_NROLE; ++r)
        if (T.sw.band[b].off[r] < 0) T.sw.band[b].off[r] = 0;
    for (int j = 0; j < 59; ++j) {
      T.sw.preflog[j] = preflog[j];
      T.sw.tref[j] = tref[j];
    }
    T.sw.grav = 9.8066;
    T.sw.avogad = 6.02214199e+23;
    T.sw.heatfac = T.sw.grav * 8.6400e4 / (cpdair * 1.e2);
    T.sw.oneminus = 1.0 - 1.e-06;
    T.sw.pi = 2. * std::asin(1.);
    T.sw.bpade = 1.0 / 0.278;
    lookup_tables(T.sw_exp, nullptr, T.sw.bpade);
  }

  // ---------------- cloud optical properties ----------------
  {
    T.cld.assign(ct::SIZE, 0.0);
    struct Part {
      const char* name;
      int off;
      size_t n;
    };
    const Part parts[] = {
        {"lwcld.absice0", ct::ABSICE0, 2},        {"lwcld.absice1", ct::ABSICE1, 10},
        {"lwcld.absice2", ct::ABSICE2, 43 * 16},  {"lwcld.absice3", ct::ABSICE3, 46 * 16},
        {"lwcld.absliq0", ct::ABSLIQ0, 1},        {"lwcld.absliq1", ct::ABSLIQ1, 58 * 16},
        {"lwcld.abscld1", ct::ABSCLD1, 1},        {"swcld.extliq1", ct::EXTLIQ1, 58 * 14},
        {"swcld.ssaliq1", ct::SSALIQ1, 58 * 14},  {"swcld.asyliq1", ct::ASYLIQ1, 58 * 14},
        {"swcld.extice2", ct::EXTICE2, 43 * 14},  {"swcld.ssaice2", ct::SSAICE2, 43 * 14},
        {"swcld.asyice2", ct::ASYICE2, 43 * 14},  {"swcld.extice3", ct::EXTICE3, 46 * 14},
        {"swcld.ssaice3", ct::SSAICE3, 46 * 14},  {"swcld.asyice3", ct::ASYICE3, 46 * 14},
        {"swcld.fdlice3", ct::FDLICE3, 46 * 14},  {"swcld.abari", ct::ABARI, 5},
        {"swcld.bbari", ct::ABARI + 5, 5},        {"swcld.cbari", ct::ABARI + 10, 5},
        {"swcld.dbari", ct::ABARI + 15, 5},       {"swcld.ebari", ct::ABARI + 20, 5},
        {"swcld.fbari", ct::ABARI + 25, 5},       {"sw.wavenum2", ct::WAVENUM2, 14}};
    for (const Part& p : parts) {
      auto v = reals(m, p.name, err);
      if (!err.empty()) return err;
      if (v.size() != p.n) return std::string("cloud table malformed: ") + p.name;
      std::copy(v.begin(), v.end(), T.cld.begin() + p.off);
    }
  }
  return "";
}

}  // namespace rrtmg
