// Host-side construction of the device coefficient tables (replaces
// rrtmg_lw_ini / rrtmg_sw_ini, rrtmg_lw_init.f90:28-175, rrtmg_sw_init.f90:28-154).
#pragma once
#include <string>
#include <vector>

#include "common.cuh"

namespace rrtmg {

struct HostTables {
  std::vector<double> lw_tab, sw_tab;           // reduced band tables, g fastest
  std::vector<double> lw_exp, lw_tfn, sw_exp;   // 0..10000 lookup tables
  std::vector<double> lw_tau;                   // optical depth of each LW table entry (rrtmg_lw_init.f90:115-122)
  std::vector<double> totplnk, totplnkderiv;    // (181, 16) Fortran order
  std::vector<double> cld;                      // cloud optical property tables, ct:: offsets
  LwConst lw;
  SwConst sw;
};

// Returns "" on success, else a message.
std::string build_host_tables(const char* blob_path, double cpdair, HostTables& out);

}  // namespace rrtmg
