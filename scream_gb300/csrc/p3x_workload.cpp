/*
 * Synthetic P3 workloads (host C++).
 *
 * kind 0/1: seeded standard-atmosphere columns.  Surface pressure
 *   1000 hPa + N(0, 5 hPa); nlev+1 hybrid interfaces to a 2 hPa top with
 *   eta_k = (k/nlev)^1.5, B_k = max(0, (eta_k - 0.2)/0.8); heights from the
 *   ISA (288.15 K, 6.5 K/km to 11 km, isothermal 216.65 K above) plus a
 *   per-level N(0, 2 K) temperature perturbation; qv = RH * qsat_liquid
 *   (Murphy-Koop, share/physics_saturation_impl.hpp:67-79,155-156) with RH ~
 *   U(0.3, 1.05) (kind 1: U(0.9, 1.05) in even-indexed columns); one cloud
 *   layer 1-4 km thick with its base uniform in [1, 10 - thickness] km
 *   holding qc, qr, qi ~ 10^U(-7,-3) kg/kg, nc ~ U(5e7, 2e8), nr ~ U(1e3, 1e5),
 *   ni ~ U(1e3, 1e6) /kg, qm = U(0, 0.5) qi, bm = qm / U(100, 900).
 *   Cloud fractions are 1 inside the layer and 0 outside, floored to 1e-4 and
 *   with the rain fraction max-overlapped with the level above, as the P3
 *   interface does (physics/p3/eamxx_p3_process_interface.hpp:108-126,132).
 *   inv_exner, theta and dz follow share/util/
 *   scream_common_physics_functions_impl.hpp:88-97,115-117,214-223,400-409.
 * kind 2: the reference's "mixed" test case, physics/p3/p3_ic_cases.cpp:11-120.
 *
 * Column i draws from its own mt19937_64 stream keyed by (seed, i), so any
 * contiguous column range can be generated independently (and in parallel).
 * Uniform and normal deviates are formed from the raw 64-bit draws here
 * (53-bit mantissa; Box-Muller), so results do not depend on the C++
 * library's distribution classes.
 */
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <random>
#include <vector>

#include "p3x_internal.hpp"

namespace p3x {

namespace {

constexpr double kRd = 287.042, kCp = 1004.64, kG = 9.80616, kP0 = 100000.0;
constexpr double kEp2 = 18.016 / 28.966;
constexpr double kPi = 3.14159265358979323;

uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

struct Rng {
  std::mt19937_64 g;
  explicit Rng(uint64_t s) : g(s) {}
  double uniform() { return double(g() >> 11) * (1.0 / 9007199254740992.0); } /* [0,1) */
  double uniform(double a, double b) { return a + (b - a) * uniform(); }
  double normal(double mean, double sd) {
    const double u1 = 1.0 - uniform(); /* (0,1] */
    const double u2 = uniform();
    return mean + sd * std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * kPi * u2);
  }
};

double qsat_liq(double T, double p) {
  const double logt = std::log(T);
  const double e = std::exp(54.842763 - (6763.22 / T) - (4.210 * logt) + (0.000367 * T) +
                            (std::tanh(0.0415 * (T - 218.8)) *
                             (53.878 - (1331.22 / T) - (9.44523 * logt) + 0.014025 * T)));
  return kEp2 * e / std::max(p, 1.e-3);
}

void gen_atmosphere_column(int kind, uint64_t seed, int64_t gi, int nlev, double* const* f, int64_t off) {
  Rng rng(splitmix64(seed ^ splitmix64(uint64_t(gi) + 0x1234567ull)));
  const double p_top = 200.0;
  const double ps = kP0 + rng.normal(0.0, 500.0);
  std::vector<double> pint(nlev + 1);
  for (int k = 0; k <= nlev; ++k) {
    const double eta = std::pow(double(k) / nlev, 1.5);
    const double pref = p_top + (kP0 - p_top) * eta;
    const double B = std::max(0.0, (eta - 0.2) / 0.8);
    pint[k] = pref + B * (ps - kP0);
  }
  pint[0] = p_top;
  pint[nlev] = ps;

  const double Ts = 288.15, L = 6.5e-3, T11 = 216.65;
  const double expo = kG / (kRd * L);
  const double p11 = ps * std::pow(T11 / Ts, expo);
  auto z_of_p = [&](double p) {
    if (p >= p11) return (Ts / L) * (1.0 - std::pow(p / ps, 1.0 / expo));
    return 11000.0 + (kRd * T11 / kG) * std::log(p11 / p);
  };
  auto T_isa = [&](double z) { return z <= 11000.0 ? Ts - L * z : T11; };

  const bool wide_rh = (kind == 1) && (gi % 2 == 0);
  std::vector<double> zmid(nlev), T(nlev);
  for (int k = 0; k < nlev; ++k) {
    const double pmid = 0.5 * (pint[k] + pint[k + 1]);
    const double dp = pint[k + 1] - pint[k];
    zmid[k] = z_of_p(pmid);
    T[k] = T_isa(zmid[k]) + rng.normal(0.0, 2.0);
    const double rh = wide_rh ? rng.uniform(0.9, 1.05) : rng.uniform(0.3, 1.05);
    const double qv = rh * qsat_liq(T[k], pmid);
    const double exner = std::pow(pmid / kP0, kRd * (1.0 / kCp));
    const double c1 = -1.0 + 1.0 / kEp2;
    const double Tv = T[k] * (1.0 + c1 * qv);
    f[P3X_F_PRES][off + k] = pmid;
    f[P3X_F_DPRES][off + k] = dp;
    f[P3X_F_INV_EXNER][off + k] = 1.0 / exner;
    f[P3X_F_TH][off + k] = T[k] / exner;
    f[P3X_F_QV][off + k] = qv;
    f[P3X_F_DZ][off + k] = (kRd / kG) * dp * Tv / pmid;
    f[P3X_F_QV_PREV][off + k] = qv;
    f[P3X_F_T_PREV][off + k] = T[k];
    f[P3X_F_INV_QC_RELVAR][off + k] = 1.0;
    f[P3X_F_NCCN][off + k] = 1.0e8;
    f[P3X_F_NI_ACTIVATED][off + k] = 0.0;
    f[P3X_F_NC_NUCEAT_TEND][off + k] = 0.0;
  }

  const double thick = rng.uniform(1000.0, 4000.0);
  const double base = rng.uniform(1000.0, 10000.0 - thick);
  std::vector<double> cld(nlev);
  for (int k = 0; k < nlev; ++k) {
    const bool in = zmid[k] >= base && zmid[k] <= base + thick;
    cld[k] = in ? 1.0 : 0.0;
    double qc = 0, qr = 0, qi = 0, nc = 0, nr = 0, ni = 0, qm = 0, bm = 0;
    if (in) {
      qc = std::pow(10.0, rng.uniform(-7.0, -3.0));
      qr = std::pow(10.0, rng.uniform(-7.0, -3.0));
      qi = std::pow(10.0, rng.uniform(-7.0, -3.0));
      nc = rng.uniform(5.0e7, 2.0e8);
      nr = rng.uniform(1.0e3, 1.0e5);
      ni = rng.uniform(1.0e3, 1.0e6);
      qm = rng.uniform(0.0, 0.5) * qi;
      bm = qm / rng.uniform(100.0, 900.0);
    }
    f[P3X_F_QC][off + k] = qc;
    f[P3X_F_QR][off + k] = qr;
    f[P3X_F_QI][off + k] = qi;
    f[P3X_F_NC][off + k] = nc;
    f[P3X_F_NR][off + k] = nr;
    f[P3X_F_NI][off + k] = ni;
    f[P3X_F_QM][off + k] = qm;
    f[P3X_F_BM][off + k] = bm;
  }
  const double mincld = 0.0001;
  for (int k = 0; k < nlev; ++k) {
    const double c = std::max(cld[k], mincld);
    f[P3X_F_CLD_FRAC_L][off + k] = c;
    f[P3X_F_CLD_FRAC_I][off + k] = c;
    double cr = c;
    if (k != 0) cr = cld[k - 1] > cr ? cld[k - 1] : cr;
    f[P3X_F_CLD_FRAC_R][off + k] = cr;
  }
}

/* physics/p3/p3_ic_cases.cpp:11-120 ("mixed"), column index i. */
void gen_mixed_column(int64_t i, int nk, double* const* f, int64_t off) {
  auto at = [&](int fld, int k) -> double& { return f[fld][off + k]; };
  for (int fld = 0; fld < P3X_NUM_INPUTS; ++fld)
    for (int k = 0; k < nk; ++k) at(fld, k) = 0.0;
  for (int k = 0; k < nk; ++k) at(P3X_F_NCCN, k) = (100.0 + 0 - 0) * 1e6; /* i/ncol, k/nk: integer 0 */
  for (int k = 0; k < 15; ++k) at(P3X_F_QC, nk - 20 + k) = 1e-4 * (1 - double(k) / 14);
  for (int k = 0; k < nk; ++k) at(P3X_F_NC, k) = 1e6;
  for (int k = 0; k < 20; ++k) at(P3X_F_QR, nk - 20 + k) = 1e-5 * (1 - double(k) / 19);
  for (int k = 0; k < nk; ++k) at(P3X_F_NR, k) = 1e6;
  for (int k = 0; k < 15; ++k) at(P3X_F_QI, nk - 20 + k) = 1e-4;
  for (int k = 0; k < nk; ++k) at(P3X_F_NI, k) = 1e6;
  for (int k = 0; k < 15; ++k) at(P3X_F_QM, nk - 20 + k) = 1e-4 * (1 - double(k) / 14);
  for (int k = 0; k < 15; ++k) at(P3X_F_BM, nk - 20 + k) = 1e-2;
  for (int k = 0; k < nk; ++k) {
    const double tmp = -5e-4 + 1e-3 / double(nk) * k;
    at(P3X_F_QV, k) = tmp > 0 ? tmp : 0;
  }
  for (int k = 0; k < 15; ++k) at(P3X_F_QV, nk - 20 + k) = 5e-3;
  for (int k = 0; k < nk; ++k) at(P3X_F_PRES, k) = 100 + 1e5 / double(nk) * k;
  for (int k = 0; k < nk; ++k) at(P3X_F_DPRES, k) = 1e5 / double(nk);
  for (int k = 0; k < nk; ++k) at(P3X_F_INV_EXNER, k) = std::pow((1e5 / at(P3X_F_PRES, k)), (287.15 / 1005.0));
  for (int k = 0; k < nk; ++k) {
    at(P3X_F_CLD_FRAC_I, k) = 1.0;
    at(P3X_F_CLD_FRAC_L, k) = 1.0;
    at(P3X_F_CLD_FRAC_R, k) = 1.0;
    at(P3X_F_INV_QC_RELVAR, k) = 1.0;
  }
  std::vector<double> T(nk);
  for (int k = 0; k < nk; ++k) {
    T[k] = 150 + 150 / double(nk) * k;
    if (i > 0) T[k] += ((i % 3) - 0.5) / double(nk) * k;
    at(P3X_F_TH, k) = T[k] * std::pow(kP0 / at(P3X_F_PRES, k), kRd / kCp);
  }
  at(P3X_F_QI, nk - 1) = 1e-9;
  at(P3X_F_QV, nk - 1) = 5e-2;
  at(P3X_F_QR, nk - 1) = 1e-6;
  at(P3X_F_QC, nk - 1) = 1e-6;
  at(P3X_F_QI, nk - 25) = 5e-8;
  at(P3X_F_QC, 35) = 1e-7;
  at(P3X_F_QV, 35) = 1e-6;
  at(P3X_F_QV, 33) = 1e-4;
  for (int k = 0; k < nk; ++k) {
    at(P3X_F_QV_PREV, k) = at(P3X_F_QV, k);
    at(P3X_F_T_PREV, k) = T[k];
  }
  const double g = 9.8;
  for (int k = 0; k < nk; ++k) {
    double plo, phi;
    plo = (k == 0) ? std::max<double>(double(i), at(P3X_F_PRES, 0) - 0.5 * (at(P3X_F_PRES, 1) - at(P3X_F_PRES, 0)) / (1 - 0))
                   : 0.5 * (at(P3X_F_PRES, k - 1) + at(P3X_F_PRES, k));
    phi = (k == nk - 1) ? at(P3X_F_PRES, nk - 1) + 0.5 * (at(P3X_F_PRES, nk - 1) - at(P3X_F_PRES, nk - 2)) / (1 - 0)
                        : 0.5 * (at(P3X_F_PRES, k) + at(P3X_F_PRES, k + 1));
    const double dpres = phi - plo;
    at(P3X_F_DZ, k) = kRd * T[k] / (g * at(P3X_F_PRES, k)) * dpres;
  }
}

}  // namespace

int workload_generate(int kind, uint64_t seed, int col0, int ncol, int nlev, double* const* fields,
                      int64_t ld) {
  if (ncol < 0 || nlev < 1 || ld < nlev || !fields) return P3X_EINVAL;
  for (int fld = 0; fld < P3X_NUM_INPUTS; ++fld)
    if (!fields[fld]) return P3X_EINVAL;
  if (kind == 2 && nlev < 36) return P3X_EINVAL;
  if (kind < 0 || kind > 2) return P3X_EINVAL;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
  for (int c = 0; c < ncol; ++c) {
    const int64_t gi = int64_t(col0) + c;
    if (kind == 2) {
      gen_mixed_column(gi, nlev, fields, int64_t(c) * ld);
    } else {
      gen_atmosphere_column(kind, seed, gi, nlev, fields, int64_t(c) * ld);
    }
  }
  return P3X_OK;
}

}  // namespace p3x
