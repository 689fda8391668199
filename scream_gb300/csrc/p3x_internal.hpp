/* Internal declarations shared by the host translation units of libp3x. */
#ifndef P3X_INTERNAL_HPP
#define P3X_INTERNAL_HPP

#include <cstdint>
#include <vector>

#include "p3x.h"

namespace p3x {

/* P3 table dimensions, physics/p3/p3_functions.hpp:31-46 and
 * physics/share/physics_constants.hpp:90-92. */
constexpr int kDensize = 5, kRimsize = 4, kIsize = 50, kIceCols = 12, kRcollsize = 30,
              kCollCols = 2, kVT0 = 300, kVT1 = 10, kMuRDim = 150, kDnuDim = 16;
constexpr int kIceTableSize = kDensize * kRimsize * kIsize * kIceCols;             /* 12000 */
constexpr int kCollTableSize = kDensize * kRimsize * kIsize * kRcollsize * kCollCols; /* 60000 */
constexpr int kVTableSize = kVT0 * kVT1;                                           /* 3000 */

struct HostTables {
  std::vector<double> ice, collect, vn, vm, revap, mu_r, dnu;
};

void build_rain_tables(HostTables& T, double mu_r_constant);
int build_ice_tables(HostTables& T);
int read_ice_table_file(const char* path, const char* expect_version, HostTables& T);
int write_ice_table_file(const char* path, const char* version);
double incomplete_gamma_q(double a, double x);

/* Murphy-Koop saturation vapour pressures over liquid (first kSvpIntervals
 * rows) and ice (next kSvpIntervals rows) as cubic polynomials in the
 * position u in [0,1) inside each 1/64 K interval from 150 K: row i holds
 * c0..c3 with e(T) = c0 + u (c1 + u (c2 + u c3)). */
constexpr double kSvpT0 = 150.0, kSvpInvH = 64.0;
constexpr int kSvpIntervals = 12800;
void build_svp_table(std::vector<double>& coef);

/* Size of the static hand-over scratch of p3x_main_fixed_scratch. */
constexpr size_t kFixedScratchBytes = size_t(64) << 20;

/* Synthetic workload, p3x_workload.cpp */
int workload_generate(int kind, uint64_t seed, int col0, int ncol, int nlev, double* const* fields,
                      int64_t ld);

}  // namespace p3x

#endif
