/*
 * CPU oracle for P3 `p3_main` -- TEST INFRASTRUCTURE ONLY (see p3_oracle.h).
 *
 * Every function below restates one reference routine, scalar (pack size 1),
 * FP64, in the same evaluation order, keeping the reference's quirks.  The
 * file:line citations are relative to components/eamxx/src/physics/ unless
 * stated otherwise.
 *
 * The one deliberate difference: the reference zero-initialises only the
 * first nlev entries of the (nlev+1)-long precip_liq_flux / precip_ice_flux
 * with pack size 1 (p3/impl/p3_main_impl.hpp:200-203 via p3_main_init's
 * zero_init loop over nk_pack); the Fortran p3_main zeroes all nlev+1
 * (eam/src/physics/p3/scream/micro_p3.F90:1312-1313).  The oracle follows the
 * Fortran statement so the surface interface does not carry stale data.
 */
#include "p3_oracle.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

using Real = double;

/* share/physics_constants.hpp:27-102 */
namespace C {
constexpr Real Cpair = 1004.64;
constexpr Real Rair = 287.042;
constexpr Real RH2O = 461.505;
constexpr Real RV = RH2O;
constexpr Real RHO_H2O = 1000.0;
constexpr Real INV_RHO_H2O = 1.0 / RHO_H2O;
constexpr Real MWH2O = 18.016;
constexpr Real MWdry = 28.966;
constexpr Real ep_2 = MWH2O / MWdry;
constexpr Real gravit = 9.80616;
constexpr Real LatVap = 2501000.0;
constexpr Real LatIce = 333700.0;
constexpr Real CpLiq = 4188.0;
constexpr Real Tmelt = 273.15;
constexpr Real T_zerodegc = Tmelt;
constexpr Real T_homogfrz = Tmelt - 40;
constexpr Real T_rainfrz = Tmelt - 4;
constexpr Real Pi = 3.14159265358979323;
constexpr Real RHOW = RHO_H2O;
constexpr Real INV_RHO_RIMEMAX = 1.0 / 900.0;
constexpr Real THIRD = 1.0 / 3.0;
constexpr Real SXTH = 1.0 / 6.0;
constexpr Real PIOV3 = Pi * THIRD;
constexpr Real PIOV6 = Pi * SXTH;
constexpr Real BIMM = 2.0;
constexpr Real CONS1 = PIOV6 * RHOW;
constexpr Real CONS2 = 4. * PIOV3 * RHOW;
constexpr Real CONS3 = 1.0 / (CONS2 * 1.562500000000000e-14);
constexpr Real CONS5 = PIOV6 * BIMM;
constexpr Real CONS6 = PIOV6 * PIOV6 * RHOW * BIMM;
constexpr Real QSMALL = 1.e-14;
constexpr Real QTENDSMALL = 1e-20;
constexpr Real BSMALL = 1.e-15;
constexpr Real NSMALL = 1.e-16;
constexpr Real P0 = 100000.0;
constexpr Real RD = Rair;
constexpr Real RHO_1000MB = P0 / (RD * Tmelt);
constexpr Real RHO_600MB = 60000 / (RD * 253.15);
constexpr Real CP = Cpair;
constexpr Real INV_CP = 1.0 / CP;
constexpr Real dt_left_tol = 1.e-4;
constexpr Real bcn = 2.;
constexpr Real dropmass = 5.2e-7;
constexpr Real NCCNST = 200.0e+6;
constexpr Real incloud_limit = 5.1e-3;
constexpr Real precip_limit = 1.0e-2;
constexpr Real f1r = 0.78;
constexpr Real f2r = 0.32;
constexpr Real nmltratio = 1.0;
}  // namespace C

/* p3/p3_functions.hpp:31-48 */
constexpr int densize = 5, rimsize = 4, isize = 50, ice_table_size = 12,
              rcollsize = 30, collect_table_size = 2;
constexpr Real lookup_table_1a_dum1_c = 4.135985029041767e+00;
constexpr int VT0 = 300, VT1 = 10;

/* A hard cap on CFL substeps; the reference loop is unbounded
 * (p3/impl/p3_cloud_sed_impl.hpp:62).  Hitting it is reported, not silent. */
constexpr int kMaxSubsteps = 100000;

struct Err {
  int bits = 0;
};

inline Real square(Real x) { return x * x; }
inline Real cube(Real x) { return x * x * x; }

/* ---------------------------------------------------------------------- */
/* Saturation: share/physics_saturation_impl.hpp                          */
/* ---------------------------------------------------------------------- */

/* check_temperature: physics_saturation_impl.hpp:14-36 (device abort there;
 * an error bit here). */
inline void check_temperature(Real t, Err& e) {
  if (!(t > 0)) e.bits |= P3O_ENUMERIC;
}

/* MurphyKoop_svp: physics_saturation_impl.hpp:38-81 */
Real MurphyKoop_svp(Real t, bool ice, Err& e) {
  check_temperature(t, e);
  if (t < C::Tmelt && ice) {
    return std::exp(9.550426 - (5723.265 / t) + (3.53068 * std::log(t)) - (0.00728332 * t));
  }
  const Real logt = std::log(t);
  return std::exp(54.842763 - (6763.22 / t) - (4.210 * logt) + (0.000367 * t) +
                  (std::tanh(0.0415 * (t - 218.8)) *
                   (53.878 - (1331.22 / t) - (9.44523 * logt) + 0.014025 * t)));
}

/* qv_sat_dry with the MurphyKoop choice: physics_saturation_impl.hpp:126-157 */
Real qv_sat_dry(Real t, Real p, bool ice, Err& e) {
  const Real e_pres = MurphyKoop_svp(t, ice, e);
  return C::ep_2 * e_pres / std::max(p, 1.e-3);
}

/* ---------------------------------------------------------------------- */
/* Table lookups: p3/impl/p3_table_ice_impl.hpp, p3/impl/p3_table3_impl.hpp */
/* ---------------------------------------------------------------------- */

struct TableIce {
  int dumi, dumjj, dumii;
  Real dum1, dum4, dum5;
};
struct TableRain {
  int dumj;
  Real dum3;
};
struct Table3 {
  int dumii, dumjj;
  Real rdumii, rdumjj;
};

inline Real ice_at(const p3o_tables* t, int jj, int ii, int i, int idx) {
  return t->ice[((jj * rimsize + ii) * isize + i) * ice_table_size + idx];
}
inline Real coll_at(const p3o_tables* t, int jj, int ii, int i, int j, int idx) {
  return t->collect[(((jj * rimsize + ii) * isize + i) * rcollsize + j) * collect_table_size + idx];
}
inline Real t2_at(const double* tab, int i, int j) { return tab[i * VT1 + j]; }

/* lookup_ice: p3_table_ice_impl.hpp:80-138 */
void lookup_ice(Real qi, Real ni, Real qm, Real rhop, TableIce& tab) {
  tab.dum1 = (std::log10(qi / ni) + 18) * lookup_table_1a_dum1_c - 10;
  tab.dumi = static_cast<int>(tab.dum1);
  tab.dum1 = std::min(tab.dum1, static_cast<Real>(isize));
  tab.dum1 = std::max(tab.dum1, 1.);
  tab.dumi = std::max(1, tab.dumi);
  tab.dumi = std::min(isize - 1, tab.dumi);
  tab.dum4 = (qm / qi) * 3 + 1;
  tab.dumii = static_cast<int>(tab.dum4);
  tab.dum4 = std::min(tab.dum4, static_cast<Real>(rimsize));
  tab.dum4 = std::max(tab.dum4, 1.);
  tab.dumii = std::max(1, tab.dumii);
  tab.dumii = std::min(rimsize - 1, tab.dumii);
  if (rhop <= 650) {
    tab.dum5 = (rhop - 50) * 0.005 + 1;
  } else {
    tab.dum5 = (rhop - 650) * 0.004 + 4;
  }
  tab.dumjj = static_cast<int>(tab.dum5);
  tab.dum5 = std::min(tab.dum5, static_cast<Real>(densize));
  tab.dum5 = std::max(tab.dum5, 1.);
  tab.dumjj = std::max(1, tab.dumjj);
  tab.dumjj = std::min(densize - 1, tab.dumjj);
  tab.dumi -= 1;
  tab.dumjj -= 1;
  tab.dumii -= 1;
}

/* lookup_rain: p3_table_ice_impl.hpp:140-173 */
void lookup_rain(Real qr, Real nr, TableRain& tab) {
  const bool gt_small = qr > C::QSMALL && nr > 0.0;
  Real dumlr = 1;
  if (gt_small) dumlr = std::cbrt(qr / (C::Pi * C::RHO_H2O * nr));
  tab.dum3 = (std::log10(1 * dumlr) + 5) * 10.70415;
  tab.dumj = static_cast<int>(tab.dum3);
  tab.dum3 = std::min(tab.dum3, static_cast<Real>(rcollsize));
  tab.dum3 = std::max(tab.dum3, 1.);
  tab.dumj = std::max(1, tab.dumj);
  tab.dumj = std::min(rcollsize - 1, tab.dumj);
  if (!gt_small) {
    tab.dumj = 1;
    tab.dum3 = 1;
  }
  tab.dumj -= 1;
}

/* apply_table_ice: p3_table_ice_impl.hpp:175-212 */
Real apply_table_ice(int idx, const p3o_tables* t, const TableIce& tab) {
  const Real w1 = tab.dum1 - Real(tab.dumi) - 1;
  const Real w4 = tab.dum4 - Real(tab.dumii) - 1;
  const Real w5 = tab.dum5 - Real(tab.dumjj) - 1;
  Real iproc1 = ice_at(t, tab.dumjj, tab.dumii, tab.dumi, idx) +
                w1 * (ice_at(t, tab.dumjj, tab.dumii, tab.dumi + 1, idx) -
                      ice_at(t, tab.dumjj, tab.dumii, tab.dumi, idx));
  Real gproc1 = ice_at(t, tab.dumjj, tab.dumii + 1, tab.dumi, idx) +
                w1 * (ice_at(t, tab.dumjj, tab.dumii + 1, tab.dumi + 1, idx) -
                      ice_at(t, tab.dumjj, tab.dumii + 1, tab.dumi, idx));
  const Real tmp1 = iproc1 + w4 * (gproc1 - iproc1);
  iproc1 = ice_at(t, tab.dumjj + 1, tab.dumii, tab.dumi, idx) +
           w1 * (ice_at(t, tab.dumjj + 1, tab.dumii, tab.dumi + 1, idx) -
                 ice_at(t, tab.dumjj + 1, tab.dumii, tab.dumi, idx));
  gproc1 = ice_at(t, tab.dumjj + 1, tab.dumii + 1, tab.dumi, idx) +
           w1 * (ice_at(t, tab.dumjj + 1, tab.dumii + 1, tab.dumi + 1, idx) -
                 ice_at(t, tab.dumjj + 1, tab.dumii + 1, tab.dumi, idx));
  const Real tmp2 = iproc1 + w4 * (gproc1 - iproc1);
  return tmp1 + w5 * (tmp2 - tmp1);
}

/* apply_table_coll: p3_table_ice_impl.hpp:214-297 */
Real apply_table_coll(int idx, const p3o_tables* t, const TableIce& ti, const TableRain& tr) {
  const Real w1 = ti.dum1 - Real(ti.dumi) - 1;
  const Real w3 = tr.dum3 - Real(tr.dumj) - 1;
  const Real w4 = ti.dum4 - Real(ti.dumii) - 1;
  const Real w5 = ti.dum5 - Real(ti.dumjj) - 1;
  auto c = [&](int jj, int ii, int i, int j) { return coll_at(t, jj, ii, i, j, idx); };
  Real dproc1 = c(ti.dumjj, ti.dumii, ti.dumi, tr.dumj) +
                w1 * (c(ti.dumjj, ti.dumii, ti.dumi + 1, tr.dumj) - c(ti.dumjj, ti.dumii, ti.dumi, tr.dumj));
  Real dproc2 = c(ti.dumjj, ti.dumii, ti.dumi, tr.dumj + 1) +
                w1 * (c(ti.dumjj, ti.dumii, ti.dumi + 1, tr.dumj + 1) - c(ti.dumjj, ti.dumii, ti.dumi, tr.dumj + 1));
  Real iproc1 = dproc1 + w3 * (dproc2 - dproc1);
  dproc1 = c(ti.dumjj, ti.dumii + 1, ti.dumi, tr.dumj) +
           w1 * (c(ti.dumjj, ti.dumii + 1, ti.dumi + 1, tr.dumj) - c(ti.dumjj, ti.dumii + 1, ti.dumi, tr.dumj));
  dproc2 = c(ti.dumjj, ti.dumii + 1, ti.dumi, tr.dumj + 1) +
           w1 * (c(ti.dumjj, ti.dumii + 1, ti.dumi + 1, tr.dumj + 1) - c(ti.dumjj, ti.dumii + 1, ti.dumi, tr.dumj + 1));
  Real gproc1 = dproc1 + w3 * (dproc2 - dproc1);
  const Real tmp1 = iproc1 + w4 * (gproc1 - iproc1);
  dproc1 = c(ti.dumjj + 1, ti.dumii, ti.dumi, tr.dumj) +
           w1 * (c(ti.dumjj + 1, ti.dumii, ti.dumi + 1, tr.dumj) - c(ti.dumjj + 1, ti.dumii, ti.dumi, tr.dumj));
  dproc2 = c(ti.dumjj + 1, ti.dumii, ti.dumi, tr.dumj + 1) +
           w1 * (c(ti.dumjj + 1, ti.dumii, ti.dumi + 1, tr.dumj + 1) - c(ti.dumjj + 1, ti.dumii, ti.dumi, tr.dumj + 1));
  iproc1 = dproc1 + w3 * (dproc2 - dproc1);
  dproc1 = c(ti.dumjj + 1, ti.dumii + 1, ti.dumi, tr.dumj) +
           w1 * (c(ti.dumjj + 1, ti.dumii + 1, ti.dumi + 1, tr.dumj) - c(ti.dumjj + 1, ti.dumii + 1, ti.dumi, tr.dumj));
  dproc2 = c(ti.dumjj + 1, ti.dumii + 1, ti.dumi, tr.dumj + 1) +
           w1 * (c(ti.dumjj + 1, ti.dumii + 1, ti.dumi + 1, tr.dumj + 1) - c(ti.dumjj + 1, ti.dumii + 1, ti.dumi, tr.dumj + 1));
  gproc1 = dproc1 + w3 * (dproc2 - dproc1);
  const Real tmp2 = iproc1 + w4 * (gproc1 - iproc1);
  return tmp1 + w5 * (tmp2 - tmp1);
}

/* lookup (Table3): p3_table3_impl.hpp:14-64 */
void lookup3(Real mu_r, Real lamr, Table3& tab) {
  const Real dum1 = (mu_r + 1) / lamr;
  if (dum1 <= 195.e-6) {
    const Real inv_dum3 = 0.1;
    Real rdumii = (dum1 * 1.e6 + 5) * inv_dum3;
    rdumii = std::max(rdumii, 1.0);
    rdumii = std::min(rdumii, 20.0);
    int dumii = static_cast<int>(rdumii);
    dumii = std::max(dumii, 1);
    dumii = std::min(dumii, 20);
    tab.rdumii = rdumii;
    tab.dumii = dumii;
  } else {
    const Real inv_dum3 = C::THIRD * 0.1;
    Real rdumii = (dum1 * 1.e+6 - 195) * inv_dum3 + 20;
    rdumii = std::max(rdumii, 20.0);
    rdumii = std::min(rdumii, 300.0);
    int dumii = static_cast<int>(rdumii);
    dumii = std::max(dumii, 20);
    dumii = std::min(dumii, 299);
    tab.rdumii = rdumii;
    tab.dumii = dumii;
  }
  Real rdumjj = mu_r + 1;
  rdumjj = std::max(rdumjj, 1.);
  rdumjj = std::min(rdumjj, 10.);
  int dumjj = static_cast<int>(rdumjj);
  dumjj = std::max(dumjj, 1);
  dumjj = std::min(dumjj, 9);
  tab.rdumjj = rdumjj;
  tab.dumjj = dumjj;
}

/* apply_table (Table3): p3_table3_impl.hpp:66-83 */
Real apply_table3(const double* table, const Table3& t3) {
  const Real rdumii_m_dumii = t3.rdumii - Real(t3.dumii);
  const Real t_im1_jm1 = t2_at(table, t3.dumii - 1, t3.dumjj - 1);
  const Real dum1 = (t_im1_jm1 + rdumii_m_dumii * (t2_at(table, t3.dumii, t3.dumjj - 1) - t_im1_jm1));
  const Real t_im1_j = t2_at(table, t3.dumii - 1, t3.dumjj);
  const Real dum2 = (t_im1_j + rdumii_m_dumii * (t2_at(table, t3.dumii, t3.dumjj) - t_im1_j));
  return dum1 + (t3.rdumjj - Real(t3.dumjj)) * (dum2 - dum1);
}

/* ---------------------------------------------------------------------- */
/* Process routines (p3/impl/*_impl.hpp)                                  */
/* ---------------------------------------------------------------------- */

/* calculate_incloud_mixingratios: p3_incloud_mixingratios_impl.hpp:12-69
 * Quirk kept: bm_incld uses inv_cld_frac_l (line 49). */
void calculate_incloud_mixingratios(Real qc, Real qr, Real qi, Real qm, Real nc, Real nr, Real ni,
                                    Real bm, Real inv_cld_frac_l, Real inv_cld_frac_i,
                                    Real inv_cld_frac_r, Real& qc_incld, Real& qr_incld,
                                    Real& qi_incld, Real& qm_incld, Real& nc_incld, Real& nr_incld,
                                    Real& ni_incld, Real& bm_incld) {
  if (qc >= C::QSMALL) {
    qc_incld = qc * inv_cld_frac_l;
    nc_incld = std::max(nc * inv_cld_frac_l, 0.);
  } else {
    qc_incld = 0;
    nc_incld = 0;
  }
  if (qi >= C::QSMALL) {
    qi_incld = qi * inv_cld_frac_i;
    ni_incld = std::max(ni * inv_cld_frac_i, 0.);
  } else {
    qi_incld = 0;
    ni_incld = 0;
  }
  if (qi >= C::QSMALL && qm >= C::QSMALL) {
    qm_incld = qm * inv_cld_frac_i;
    bm_incld = std::max(bm * inv_cld_frac_l, 0.);
  } else {
    qm_incld = 0;
    bm_incld = 0;
  }
  if (qr >= C::QSMALL) {
    qr_incld = qr * inv_cld_frac_r;
    nr_incld = std::max(nr * inv_cld_frac_r, 0.);
  } else {
    qr_incld = 0;
    nr_incld = 0;
  }
  if (qc_incld > C::incloud_limit || qi_incld > C::incloud_limit || qr_incld > C::precip_limit ||
      bm_incld > C::incloud_limit) {
    qc_incld = std::min(qc_incld, C::incloud_limit);
    qi_incld = std::min(qi_incld, C::incloud_limit);
    bm_incld = std::min(bm_incld, C::incloud_limit);
    qr_incld = std::min(qr_incld, C::precip_limit);
  }
}

/* get_time_space_phys_variables: p3_get_time_space_phys_variables_impl.hpp:12-45 */
void get_time_space_phys_variables(Real T_atm, Real pres, Real rho, Real qv_sat_l, Real qv_sat_i,
                                   Real& mu, Real& dv, Real& sc, Real& dqsdt, Real& dqsidt, Real& ab,
                                   Real& abi, Real& kap, Real& eii) {
  mu = 1.496e-6 * std::pow(T_atm, 1.5) / (T_atm + 120);
  dv = 8.794e-5 * std::pow(T_atm, 1.81) / pres;
  sc = mu / (rho * dv);
  const Real dum = 1 / (C::RV * square(T_atm));
  dqsdt = C::LatVap * qv_sat_l * dum;
  dqsidt = (C::LatVap + C::LatIce) * qv_sat_i * dum;
  ab = 1 + dqsdt * C::LatVap * C::INV_CP;
  abi = 1 + dqsidt * (C::LatVap + C::LatIce) * C::INV_CP;
  kap = 1.414e+3 * mu;
  const Real tval1 = 253.15, tval2 = 273.15, dtval = 20;
  if (T_atm < tval1) {
    eii = 0.001;
  } else if (T_atm < tval2) {
    eii = 0.001 + (T_atm - tval1) * (0.3 - 0.001) / dtval;
  } else {
    eii = 0.3;
  }
}

/* get_cloud_dsd2: p3_dsd2_impl.hpp:14-74 (iparam = 3, so the dnu branch is inactive) */
void get_cloud_dsd2(Real qc, Real& nc, Real& mu_c, Real rho, Real& nu, Real& lamc, Real& cdist,
                    Real& cdist1) {
  lamc = 0;
  cdist = 0;
  cdist1 = 0;
  nu = 0;
  mu_c = 0;
  if (qc >= C::QSMALL) {
    nc = std::max(nc, C::NSMALL);
    Real mu_c_local = 0.0005714 * (nc * 1.e-6 * rho) + 0.2714;
    mu_c_local = 1 / (mu_c_local * mu_c_local) - 1;
    mu_c_local = std::max(mu_c_local, 2.);
    mu_c_local = std::min(mu_c_local, 15.);
    mu_c = mu_c_local;
    lamc = std::cbrt(C::CONS1 * nc * (mu_c + 3) * (mu_c + 2) * (mu_c + 1) / qc);
    const Real lammin = (mu_c + 1) * 2.5e+4;
    const Real lammax = (mu_c + 1) * 1.e+6;
    const bool lt = lamc < lammin, gt = lamc > lammax;
    if (lt) lamc = lammin;
    if (gt) lamc = lammax;
    if (lt || gt) {
      nc = 6 * (lamc * lamc * lamc) * qc / (C::Pi * C::RHO_H2O * (mu_c + 3) * (mu_c + 2) * (mu_c + 1));
    }
    cdist = nc * (mu_c + 1) / lamc;
    cdist1 = nc / std::tgamma(mu_c + 1);
  }
}

/* get_rain_dsd2: p3_dsd2_impl.hpp:76-126 */
void get_rain_dsd2(Real qr, Real& nr, Real& mu_r, Real& lamr, const p3o_runtime& rt) {
  lamr = 0;
  if (qr >= C::QSMALL) {
    const Real nr_lim = std::max(nr, C::NSMALL);
    mu_r = rt.constant_mu_rain;
    const Real mass_to_d3_factor = C::CONS1 * (mu_r + 3) * (mu_r + 2) * (mu_r + 1);
    lamr = std::cbrt(mass_to_d3_factor * nr_lim / qr);
    const Real lammax = (mu_r + 1.) * 1.e+5;
    const Real lammin = (mu_r + 1.) * 500;
    const bool lt = lamr < lammin, gt = lamr > lammax;
    nr = nr_lim;
    if (lt || gt) {
      if (lt) lamr = lammin;
      if (gt) lamr = lammax;
      nr = lamr * lamr * lamr * qr / mass_to_d3_factor;
    }
  }
}

/* get_cdistr_logn0r: p3_dsd2_impl.hpp:128-148 */
void get_cdistr_logn0r(Real qr, Real nr, Real mu_r, Real lamr, Real& cdistr, Real& logn0r) {
  cdistr = 0;
  logn0r = 0;
  if (qr >= C::QSMALL) {
    cdistr = nr / std::tgamma(mu_r + 1);
    logn0r = std::log10(cdistr) + (mu_r + 1) * std::log10(lamr);
  }
}

/* impose_max_total_ni: p3_impose_max_total_ni_impl.hpp:9-27 */
void impose_max_total_ni(Real& ni_local, Real max_total_ni, Real inv_rho_local) {
  if (ni_local >= 1e-20) {
    ni_local = ni_local * std::min(max_total_ni * inv_rho_local / ni_local, 1.);
  }
}

/* calc_bulk_rho_rime: p3_ice_sed_impl.hpp:14-64 */
Real calc_bulk_rho_rime(Real qi_tot, Real& qi_rim, Real& bi_rim, const p3o_runtime& rt) {
  Real rho_rime = 0;
  const bool gt = bi_rim >= C::BSMALL;
  const bool lt = bi_rim < C::BSMALL;
  if (gt) rho_rime = qi_rim / bi_rim;
  const bool rr_lt_min = rho_rime < rt.min_rime_rho;
  const bool rr_gt_max = rho_rime > rt.max_rime_rho;
  if (gt && rr_lt_min) rho_rime = rt.min_rime_rho;
  if (gt && rr_gt_max) rho_rime = rt.max_rime_rho;
  if (gt && (rr_gt_max || rr_lt_min)) bi_rim = qi_rim / rho_rime;
  if (lt) {
    qi_rim = 0;
    bi_rim = 0;
    rho_rime = 0;
  }
  if (qi_rim > qi_tot && rho_rime > 0) {
    qi_rim = qi_tot;
    bi_rim = qi_rim / rho_rime;
  }
  if (qi_rim < C::QSMALL) {
    qi_rim = 0;
    bi_rim = 0;
  }
  return rho_rime;
}

/* ice_cldliq_collection: p3_ice_collection_impl.hpp:9-52 */
void ice_cldliq_collection(Real rho, Real temp, Real rhofaci, Real table_val_qc2qi_collect,
                           Real qi_incld, Real qc_incld, Real ni_incld, Real nc_incld,
                           Real& qc2qi_collect_tend, Real& nc_collect_tend,
                           Real& qc2qr_ice_shed_tend, Real& ncshdc, const p3o_runtime& rt) {
  const bool t_is_negative = temp <= C::Tmelt;
  const bool both = qi_incld >= C::QSMALL && qc_incld >= C::QSMALL;
  const Real f = rt.cldliq_to_ice_collection_factor;
  if (both && t_is_negative)
    qc2qi_collect_tend = rhofaci * table_val_qc2qi_collect * qc_incld * f * rho * ni_incld;
  if (both) nc_collect_tend = rhofaci * table_val_qc2qi_collect * nc_incld * f * rho * ni_incld;
  if (both && !t_is_negative) {
    qc2qr_ice_shed_tend = rhofaci * table_val_qc2qi_collect * qc_incld * f * rho * ni_incld;
    nc_collect_tend = rhofaci * table_val_qc2qi_collect * nc_incld * f * rho * ni_incld;
    ncshdc = qc2qr_ice_shed_tend * (1.0 / C::dropmass);
  }
}

/* ice_rain_collection: p3_ice_collection_impl.hpp:54-101 */
void ice_rain_collection(Real rho, Real temp, Real rhofaci, Real logn0r, Real table_val_nr_collect,
                         Real table_val_qr2qi_collect, Real qi_incld, Real ni_incld, Real qr_incld,
                         Real& qr2qi_collect_tend, Real& nr_collect_tend, const p3o_runtime& rt) {
  const bool t_is_negative = temp <= C::Tmelt;
  const bool both = qi_incld >= C::QSMALL && qr_incld >= C::QSMALL;
  const Real f = rt.rain_to_ice_collection_factor;
  const Real ten = 10.0;
  if (both && t_is_negative) {
    qr2qi_collect_tend = std::pow(ten, table_val_qr2qi_collect + logn0r) * rho * rhofaci * f * ni_incld;
    nr_collect_tend = std::pow(ten, table_val_nr_collect + logn0r) * rho * rhofaci * f * ni_incld;
  }
  if (both && !t_is_negative) {
    nr_collect_tend = std::pow(ten, table_val_nr_collect + logn0r) * rho * rhofaci * f * ni_incld;
  }
}

/* ice_self_collection: p3_ice_collection_impl.hpp:103-152 */
void ice_self_collection(Real rho, Real rhofaci, Real table_val_ni_self_collect, Real eii,
                         Real qm_incld, Real qi_incld, Real ni_incld, Real& ni_selfcollect_tend) {
  const bool qm_pos = qm_incld > 0;
  if (qi_incld >= C::QSMALL) {
    Real tmp1 = 0.0;
    if (qm_pos) tmp1 = qm_incld / qi_incld;
    Real Eii_fact = 0.0;
    if (tmp1 < 0.6 && qm_pos) Eii_fact = 1;
    if (tmp1 >= 0.6 && tmp1 < 0.9 && qm_pos) Eii_fact = 1 - (tmp1 - 0.6) / 0.3;
    if (tmp1 >= 0.9 && qm_pos) Eii_fact = 0;
    if (!qm_pos) Eii_fact = 1;
    ni_selfcollect_tend = table_val_ni_self_collect * rho * eii * Eii_fact * rhofaci * ni_incld * ni_incld;
  }
}

/* ice_melting: p3_ice_melting_impl.hpp:10-53.  Quirk kept: the max(...,0) is
 * applied to qi2qr_melt_tend unconditionally inside the branch (line 47). */
void ice_melting(Real rho, Real T_atm, Real pres, Real rhofaci, Real table_val_qi2qr_melting,
                 Real table_val_qi2qr_vent_melt, Real dv, Real sc, Real mu, Real kap, Real qv,
                 Real qi_incld, Real ni_incld, Real& qi2qr_melt_tend, Real& ni2nr_melt_tend,
                 Err& e) {
  const bool has_melt_qi = qi_incld >= C::QSMALL && T_atm > C::Tmelt;
  if (has_melt_qi) {
    const Real qsat0 = qv_sat_dry(C::Tmelt, pres, false, e);
    qi2qr_melt_tend = ((table_val_qi2qr_melting +
                        table_val_qi2qr_vent_melt * std::cbrt(sc) * std::sqrt(rhofaci * rho / mu)) *
                       ((T_atm - C::Tmelt) * kap - rho * C::LatVap * dv * (qsat0 - qv)) * 2 * C::Pi /
                       C::LatIce) *
                      ni_incld;
    qi2qr_melt_tend = std::max(qi2qr_melt_tend, 0.);
    ni2nr_melt_tend = qi2qr_melt_tend * (ni_incld / qi_incld);
  }
}

/* ice_cldliq_wet_growth: p3_ice_cldliq_wet_growth_impl.hpp:12-80 */
void ice_cldliq_wet_growth(Real rho, Real temp, Real pres, Real rhofaci, Real table_val_qi2qr_melting,
                           Real table_val_qi2qr_vent_melt, Real dv, Real kap, Real mu, Real sc,
                           Real qv, Real qc_incld, Real qi_incld, Real ni_incld, Real qr_incld,
                           bool& log_wetgrowth, Real& qr2qi_collect_tend, Real& qc2qi_collect_tend,
                           Real& qc_growth_rate, Real& nr_ice_shed_tend, Real& qc2qr_ice_shed_tend,
                           Err& e) {
  const bool t_is_negative = temp < C::Tmelt;
  const bool any_if = qi_incld >= C::QSMALL && (qc_incld + qr_incld) >= 1.0e-6 && t_is_negative;
  const bool any_if_col = any_if && (qc2qi_collect_tend + qr2qi_collect_tend) >= 1.0e-10;
  if (any_if) {
    const Real qsat0 = qv_sat_dry(C::Tmelt, pres, false, e);
    qc_growth_rate = ((table_val_qi2qr_melting +
                       table_val_qi2qr_vent_melt * std::cbrt(sc) * std::sqrt(rhofaci * rho / mu)) *
                      (C::Pi * 2) * (rho * C::LatVap * dv * (qsat0 - qv) - (temp - C::Tmelt) * kap) /
                      (C::LatIce + C::CpLiq * (temp - C::Tmelt))) *
                     ni_incld;
    qc_growth_rate = std::max(qc_growth_rate, 0.);
    const Real dum = std::max(0., (qc2qi_collect_tend + qr2qi_collect_tend) - qc_growth_rate);
    const bool dum_ge_small = dum >= 1.0e-10;
    if (dum_ge_small) {
      nr_ice_shed_tend = nr_ice_shed_tend + dum * 1.923e+6;
      const Real dum1 = 1.0 / (qc2qi_collect_tend + qr2qi_collect_tend);
      if (any_if_col) {
        qc2qr_ice_shed_tend = qc2qr_ice_shed_tend + dum * qc2qi_collect_tend * dum1;
        qc2qi_collect_tend = std::max(0., qc2qi_collect_tend - dum * qc2qi_collect_tend * dum1);
        qr2qi_collect_tend = std::max(0., qr2qi_collect_tend - dum * qr2qi_collect_tend * dum1);
      }
    }
    log_wetgrowth = dum_ge_small;
  }
}

/* ice_relaxation_timescale: p3_ice_relaxation_timescale_impl.hpp:9-37 */
void ice_relaxation_timescale(Real rho, Real temp, Real rhofaci, Real table_val_qi2qr_melting,
                              Real table_val_qi2qr_vent_melt, Real dv, Real mu, Real sc,
                              Real qi_incld, Real ni_incld, Real& epsi, Real& epsi_tot) {
  const bool any_if = qi_incld >= C::QSMALL && temp < C::Tmelt;
  if (any_if) {
    epsi = ((table_val_qi2qr_melting + table_val_qi2qr_vent_melt * std::cbrt(sc) * std::sqrt(rhofaci * rho / mu)) *
            2.0 * C::Pi * rho * dv) *
           ni_incld;
    epsi_tot = epsi_tot + epsi;
  } else {
    epsi = 0;
  }
}

/* calc_rime_density: p3_calc_rime_density_impl.hpp:13-70 */
void calc_rime_density(Real T_atm, Real rhofaci, Real table_val_qi_fallspd, Real acn, Real lamc,
                       Real mu_c, Real qc_incld, Real qc2qi_collect_tend, Real& vtrmi1,
                       Real& rho_qm_cloud) {
  const bool act = qc2qi_collect_tend >= C::QSMALL && T_atm < C::T_zerodegc;
  if (act) {
    vtrmi1 = table_val_qi_fallspd * rhofaci;
    if (qc_incld >= C::QSMALL) {
      const Real Vt_qc = acn * std::tgamma(4 + C::bcn + mu_c) / (std::pow(lamc, C::bcn) * std::tgamma(4 + mu_c));
      const Real D_c = (4 + mu_c) / lamc;
      const Real V_impact = std::fabs(vtrmi1 - Vt_qc);
      const Real inv_Tc = 1 / std::min(-0.001, T_atm - C::T_zerodegc);
      const Real Ri = std::max(1., std::min(-0.5e+6 * D_c * V_impact * inv_Tc, 12.));
      if (Ri <= 8.0) {
        rho_qm_cloud = (0.051 + 0.114 * Ri - 0.0055 * square(Ri)) * 1000;
      } else {
        rho_qm_cloud = 611. + 72.25 * (Ri - 8);
      }
    } else {
      rho_qm_cloud = 400;
    }
  } else {
    vtrmi1 = 0;
    rho_qm_cloud = 400;
  }
}

/* cldliq_immersion_freezing: p3_cldliq_imm_freezing_impl.hpp:13-50 (sgs_var_coef = 1) */
void cldliq_immersion_freezing(Real T_atm, Real lamc, Real mu_c, Real cdist1, Real qc_incld,
                               Real& qc2qi_hetero_freeze_tend, Real& nc2ni_immers_freeze_tend,
                               const p3o_runtime& rt) {
  if (qc_incld >= C::QSMALL && T_atm <= C::T_rainfrz) {
    const Real expAimmDt = std::exp(rt.immersion_freezing_exponent * (C::T_zerodegc - T_atm));
    const Real inv_lamc3 = cube(1 / lamc);
    const Real sgs_var_coef = 1;
    qc2qi_hetero_freeze_tend = sgs_var_coef * C::CONS6 * cdist1 * std::tgamma(7 + mu_c) * expAimmDt * square(inv_lamc3);
    nc2ni_immers_freeze_tend = C::CONS5 * cdist1 * std::tgamma(4.0 + mu_c) * expAimmDt * inv_lamc3;
  }
}

/* rain_immersion_freezing: p3_rain_imm_freezing_impl.hpp:13-44 */
void rain_immersion_freezing(Real T_atm, Real lamr, Real mu_r, Real cdistr, Real qr_incld,
                             Real& qr2qi_immers_freeze_tend, Real& nr2ni_immers_freeze_tend,
                             const p3o_runtime& rt) {
  if (qr_incld >= C::QSMALL && T_atm <= C::T_rainfrz) {
    qr2qi_immers_freeze_tend =
        C::CONS6 * std::exp(std::log(cdistr) + std::log(std::tgamma(7. + mu_r)) - 6. * std::log(lamr)) *
        std::exp(rt.immersion_freezing_exponent * (C::T_zerodegc - T_atm));
    nr2ni_immers_freeze_tend =
        C::CONS5 * std::exp(std::log(cdistr) + std::log(std::tgamma(4. + mu_r)) - 3. * std::log(lamr)) *
        std::exp(rt.immersion_freezing_exponent * (C::T_zerodegc - T_atm));
  }
}

/* calc_liq_relaxation_timescale: p3_calc_liq_relaxation_timescale_impl.hpp:13-43 */
void calc_liq_relaxation_timescale(const p3o_tables* tab, Real rho, Real f1r, Real f2r, Real dv,
                                   Real mu, Real sc, Real mu_r, Real lamr, Real cdistr, Real cdist,
                                   Real qr_incld, Real qc_incld, Real& epsr, Real& epsc) {
  epsr = 0;
  if (qr_incld >= C::QSMALL) {
    Table3 t3;
    lookup3(mu_r, lamr, t3);
    epsr = 2 * C::Pi * cdistr * rho * dv *
           (f1r * std::tgamma(mu_r + 2) / lamr + f2r * std::sqrt(rho / mu) * std::cbrt(sc) * apply_table3(tab->revap, t3));
  }
  if (qc_incld >= C::QSMALL) {
    epsc = 2 * C::Pi * rho * dv * cdist;
  } else {
    epsc = 0;
  }
}

/* evaporate_rain (+ tscale_weight / equilib_tend / instant_tend):
 * p3_evaporate_rain_impl.hpp:9-203 */
void evaporate_rain(Real qr_incld, Real qc_incld, Real nr_incld, Real qi_incld, Real cld_frac_l,
                    Real cld_frac_r, Real qv, Real qv_prev, Real qv_sat_l, Real qv_sat_i, Real ab,
                    Real abi, Real epsr, Real epsi_tot, Real t_atm, Real t_atm_prev, Real dqsdt,
                    Real dt, Real& qr2qv_evap_tend, Real& nr_evap_tend) {
  qr2qv_evap_tend = 0;
  nr_evap_tend = 0;
  const Real inv_dt = 1 / dt;
  const Real inv_cp = 1 / C::Cpair;
  const Real ssat_r = qv - qv_sat_l;
  Real cld_frac;
  if ((qc_incld + qi_incld) < 1.e-6) {
    cld_frac = 0;
  } else {
    cld_frac = cld_frac_l;
  }
  const bool is_rain_evap = qr_incld >= C::QSMALL && ssat_r < 0 && cld_frac_r > cld_frac;
  if (is_rain_evap) {
    const Real tau_r = 1 / epsr;
    Real eps_eff, A_c;
    if (t_atm < C::Tmelt) {
      eps_eff = epsr + epsi_tot * (1 + (C::LatVap + C::LatIce) * inv_cp * dqsdt) / abi;
      A_c = (qv - qv_prev) * inv_dt - dqsdt * (t_atm - t_atm_prev) * inv_dt -
            (qv_sat_l - qv_sat_i) * (1 + (C::LatVap + C::LatIce) * inv_cp * dqsdt) / abi * epsi_tot;
    } else {
      eps_eff = epsr;
      A_c = (qv - qv_prev) * inv_dt - dqsdt * (t_atm - t_atm_prev) * inv_dt;
    }
    if (eps_eff < 1e-20) eps_eff = 1e-20;
    const Real tau_eff = 1 / eps_eff;
    const bool is_qr_tiny = qr_incld < 1e-12 && qv / qv_sat_l < 0.999;
    if (is_qr_tiny) {
      qr2qv_evap_tend = qr_incld * inv_dt;
    } else {
      const Real dt_over_tau = dt / tau_eff;
      const Real tscale_weight = -std::expm1(-dt_over_tau) / dt_over_tau;
      const Real equilib_tend = -A_c / ab * tau_eff / tau_r;
      const Real instant_tend = -ssat_r / (ab * tau_r);
      qr2qv_evap_tend = instant_tend * tscale_weight + equilib_tend * (1 - tscale_weight);
    }
    if (qr2qv_evap_tend > -ssat_r * inv_dt / ab) qr2qv_evap_tend = -ssat_r * inv_dt / ab;
    if (qr2qv_evap_tend < 0) qr2qv_evap_tend = 0;
    if (qr2qv_evap_tend > qr_incld * inv_dt) qr2qv_evap_tend = qr_incld * inv_dt;
    qr2qv_evap_tend = qr2qv_evap_tend * (cld_frac_r - cld_frac) / cld_frac_r;
    nr_evap_tend = qr2qv_evap_tend * (nr_incld / qr_incld);
  }
}

/* ice_deposition_sublimation: p3_ice_deposition_sublimation_impl.hpp:9-65 */
void ice_deposition_sublimation(Real qi_incld, Real ni_incld, Real T_atm, Real qv_sat_l,
                                Real qv_sat_i, Real epsi, Real abi, Real qv, Real inv_dt,
                                Real& qv2qi_vapdep_tend, Real& qi2qv_sublim_tend,
                                Real& ni_sublim_tend, Real& qc2qi_berg_tend) {
  qc2qi_berg_tend = 0;
  qv2qi_vapdep_tend = 0;
  qi2qv_sublim_tend = 0;
  ni_sublim_tend = 0;
  if (qi_incld > C::QSMALL) {
    const Real qi_tend = std::min(epsi / abi, inv_dt) * (qv - qv_sat_i);
    const bool neg = qi_tend < 0;
    if (neg) {
      qi2qv_sublim_tend = -qi_tend;
      ni_sublim_tend = qi2qv_sublim_tend * (ni_incld / qi_incld);
    }
    const bool T_lt_frz = T_atm < C::T_zerodegc;
    if (T_lt_frz && !neg) qv2qi_vapdep_tend = qi_tend;
    if (T_lt_frz) qc2qi_berg_tend = std::max(epsi / abi * (qv_sat_l - qv_sat_i), 0.);
  }
}

/* ice_nucleation: p3_ice_nucleation_impl.hpp:9-61 */
void ice_nucleation(Real temp, Real inv_rho, Real ni, Real ni_activated, Real qv_supersat_i,
                    Real inv_dt, bool do_predict_nc, bool do_prescribed_CCN,
                    Real& qv2qi_nucleat_tend, Real& ni_nucleat_tend, const p3o_runtime& rt) {
  const Real T_icenuc = C::Tmelt - 15.0;
  const Real mi0 = 4.0 * C::PIOV3 * 900.0 * 1.e-18;
  const bool do_log = (!do_predict_nc || do_prescribed_CCN);
  const bool base = temp < T_icenuc && qv_supersat_i >= 0.05;
  const bool any_if_log = base && !do_log;
  const bool any_if_not_log = base && do_log;
  if (any_if_not_log) {
    Real dum = 0.005 * std::exp(rt.deposition_nucleation_exponent * (C::Tmelt - temp)) * 1.0e3 * inv_rho;
    dum = std::min(dum, 1.0e5 * inv_rho);
    const Real N_nuc = std::max(0., (dum - ni) * inv_dt);
    if (N_nuc >= C::NSMALL) {
      const Real Q_nuc = std::max(0., (dum - ni) * mi0 * inv_dt);
      qv2qi_nucleat_tend = Q_nuc;
      ni_nucleat_tend = N_nuc;
    }
  } else if (any_if_log) {
    ni_nucleat_tend = std::max(0., (ni_activated - ni) * inv_dt);
    qv2qi_nucleat_tend = ni_nucleat_tend * mi0;
  }
}

/* cloud_water_autoconversion: p3_autoconversion_impl.hpp:9-58 (CONS3 quirk kept) */
void cloud_water_autoconversion(Real rho, Real qc_incld, Real nc_incld, Real& qc2qr_autoconv_tend,
                                Real& nc2nr_autoconv_tend, Real& ncautr, const p3o_runtime& rt) {
  Real CONS3;
  if (rt.autoconversion_radius == 25.0e-6) {
    CONS3 = C::CONS3;
  } else {
    CONS3 = 1.0 / (C::CONS2 * std::pow(rt.autoconversion_radius, 3.0));
  }
  if (qc_incld >= 1e-8) {
    const Real sgs_var_coef = 1;
    qc2qr_autoconv_tend = sgs_var_coef * rt.autoconversion_prefactor *
                          std::pow(qc_incld, rt.autoconversion_qc_exponent) *
                          std::pow(nc_incld * 1.e-6 * rho, -rt.autoconversion_nc_exponent);
    ncautr = qc2qr_autoconv_tend * CONS3;
    nc2nr_autoconv_tend = qc2qr_autoconv_tend * nc_incld / qc_incld;
  }
  if (qc2qr_autoconv_tend == 0) nc2nr_autoconv_tend = 0;
  if (nc2nr_autoconv_tend == 0) qc2qr_autoconv_tend = 0;
}

/* droplet_self_collection: p3_droplet_self_coll_impl.hpp:14-30 */
void droplet_self_collection(Real qc_incld, Real& nc_selfcollect_tend) {
  if (qc_incld >= C::QSMALL) nc_selfcollect_tend = 0;
}

/* cloud_rain_accretion: p3_cloud_rain_acc_impl.hpp:14-55 */
void cloud_rain_accretion(Real qc_incld, Real nc_incld, Real qr_incld, Real& qc2qr_accret_tend,
                          Real& nc_accret_tend, const p3o_runtime& rt) {
  const Real sgs_var_coef = 1;
  if (qr_incld >= C::QSMALL && qc_incld >= C::QSMALL) {
    if (rt.accretion_qc_exponent == rt.accretion_qr_exponent) {
      qc2qr_accret_tend = sgs_var_coef * rt.accretion_prefactor * std::pow(qc_incld * qr_incld, rt.accretion_qr_exponent);
    } else {
      qc2qr_accret_tend = sgs_var_coef * rt.accretion_prefactor * std::pow(qc_incld, rt.accretion_qc_exponent) *
                          std::pow(qr_incld, rt.accretion_qr_exponent);
    }
    nc_accret_tend = qc2qr_accret_tend * nc_incld / qc_incld;
    if (nc_accret_tend == 0) qc2qr_accret_tend = 0;
    if (qc2qr_accret_tend == 0) nc_accret_tend = 0;
  }
}

/* rain_self_collection: p3_rain_self_collection_impl.hpp:9-56 */
void rain_self_collection(Real rho, Real qr_incld, Real nr_incld, Real& nr_selfcollect_tend,
                          const p3o_runtime& rt) {
  if (qr_incld >= C::QSMALL) {
    const Real dum2 = std::cbrt((qr_incld) / (C::Pi * C::RHO_H2O * nr_incld));
    Real dum;
    if (dum2 < rt.rain_selfcollection_breakup_diameter) {
      dum = 1;
    } else {
      dum = 2 - std::exp(2300 * (dum2 - rt.rain_selfcollection_breakup_diameter));
    }
    nr_selfcollect_tend = dum * rt.rain_selfcollection_prefactor * nr_incld * qr_incld * rho;
  }
}

struct Rates {
  Real qc2qr_accret_tend = 0, qr2qv_evap_tend = 0, qc2qr_autoconv_tend = 0, nc_accret_tend = 0,
       nc_selfcollect_tend = 0, nc2nr_autoconv_tend = 0, nr_selfcollect_tend = 0, nr_evap_tend = 0,
       ncautr = 0, qi2qv_sublim_tend = 0, nr_ice_shed_tend = 0, qc2qi_hetero_freeze_tend = 0,
       qr2qi_collect_tend = 0, qc2qr_ice_shed_tend = 0, qi2qr_melt_tend = 0, qc2qi_collect_tend = 0,
       qr2qi_immers_freeze_tend = 0, qv2qi_nucleat_tend = 0, ni2nr_melt_tend = 0, nc_collect_tend = 0,
       ncshdc = 0, nc2ni_immers_freeze_tend = 0, nr_collect_tend = 0, ni_selfcollect_tend = 0,
       ni_nucleat_tend = 0, qv2qi_vapdep_tend = 0, qc2qi_berg_tend = 0, nr2ni_immers_freeze_tend = 0,
       ni_sublim_tend = 0, qc_growth_rate = 0;
};

/* back_to_cell_average: p3_back_to_cell_average_impl.hpp:14-77 */
void back_to_cell_average(Real cld_frac_l, Real cld_frac_r, Real cld_frac_i, Rates& r) {
  const Real ir_cldm = std::min(cld_frac_i, cld_frac_r);
  const Real il_cldm = std::min(cld_frac_i, cld_frac_l);
  const Real lr_cldm = std::min(cld_frac_l, cld_frac_r);
  r.qc2qr_accret_tend *= lr_cldm;
  r.qr2qv_evap_tend *= cld_frac_r;
  r.qc2qr_autoconv_tend *= cld_frac_l;
  r.nc_accret_tend *= lr_cldm;
  r.nc_selfcollect_tend *= cld_frac_l;
  r.nc2nr_autoconv_tend *= cld_frac_l;
  r.nr_selfcollect_tend *= cld_frac_r;
  r.nr_evap_tend *= cld_frac_r;
  r.ncautr *= lr_cldm;
  r.qi2qv_sublim_tend *= cld_frac_i;
  r.nr_ice_shed_tend *= il_cldm;
  r.qc2qi_hetero_freeze_tend *= il_cldm;
  r.qr2qi_collect_tend *= ir_cldm;
  r.qc2qr_ice_shed_tend *= il_cldm;
  r.qi2qr_melt_tend *= cld_frac_i;
  r.qc2qi_collect_tend *= il_cldm;
  r.qr2qi_immers_freeze_tend *= cld_frac_r;
  r.ni2nr_melt_tend *= cld_frac_i;
  r.nc_collect_tend *= il_cldm;
  r.ncshdc *= il_cldm;
  r.nc2ni_immers_freeze_tend *= cld_frac_l;
  r.nr_collect_tend *= ir_cldm;
  r.ni_selfcollect_tend *= cld_frac_i;
  r.qv2qi_vapdep_tend *= cld_frac_i;
  r.nr2ni_immers_freeze_tend *= cld_frac_r;
  r.ni_sublim_tend *= cld_frac_i;
  r.qc2qi_berg_tend *= il_cldm;
}

/* cloud_water_conservation: p3_conservation_impl.hpp:9-52 */
void cloud_water_conservation(Real qc, Real dt, Real& qc2qr_autoconv_tend, Real& qc2qr_accret_tend,
                              Real& qc2qi_collect_tend, Real& qc2qi_hetero_freeze_tend,
                              Real& qc2qr_ice_shed_tend, Real& qc2qi_berg_tend,
                              Real& qi2qv_sublim_tend, Real& qv2qi_vapdep_tend) {
  const Real sinks = (qc2qr_autoconv_tend + qc2qr_accret_tend + qc2qi_collect_tend +
                      qc2qi_hetero_freeze_tend + qc2qr_ice_shed_tend + qc2qi_berg_tend) * dt;
  const Real sources = qc;
  Real ratio;
  const bool enforce = sinks > sources && sinks >= C::QTENDSMALL;
  if (enforce) {
    ratio = sources / sinks;
    qc2qr_autoconv_tend *= ratio;
    qc2qr_accret_tend *= ratio;
    qc2qi_collect_tend *= ratio;
    qc2qi_hetero_freeze_tend *= ratio;
    qc2qr_ice_shed_tend *= ratio;
    qc2qi_berg_tend *= ratio;
  } else {
    ratio = 1;
  }
  if (sources > C::QTENDSMALL) {
    qv2qi_vapdep_tend *= (1 - ratio);
    qi2qv_sublim_tend *= (1 - ratio);
  }
}

/* rain_water_conservation: p3_conservation_impl.hpp:54-76 */
void rain_water_conservation(Real qr, Real qc2qr_autoconv_tend, Real qc2qr_accret_tend,
                             Real qi2qr_melt_tend, Real qc2qr_ice_shed_tend, Real dt,
                             Real& qr2qv_evap_tend, Real& qr2qi_collect_tend,
                             Real& qr2qi_immers_freeze_tend) {
  const Real sinks = (qr2qv_evap_tend + qr2qi_collect_tend + qr2qi_immers_freeze_tend) * dt;
  const Real sources = qr + (qc2qr_autoconv_tend + qc2qr_accret_tend + qi2qr_melt_tend + qc2qr_ice_shed_tend) * dt;
  if (sinks > sources && sinks >= C::QTENDSMALL) {
    const Real ratio = sources / sinks;
    qr2qv_evap_tend *= ratio;
    qr2qi_collect_tend *= ratio;
    qr2qi_immers_freeze_tend *= ratio;
  }
}

/* ice_water_conservation: p3_conservation_impl.hpp:78-98 */
void ice_water_conservation(Real qi, Real qv2qi_vapdep_tend, Real qv2qi_nucleat_tend,
                            Real qc2qi_berg_tend, Real qr2qi_collect_tend, Real qc2qi_collect_tend,
                            Real qr2qi_immers_freeze_tend, Real qc2qi_hetero_freeze_tend, Real dt,
                            Real& qi2qv_sublim_tend, Real& qi2qr_melt_tend) {
  const Real sinks = (qi2qv_sublim_tend + qi2qr_melt_tend) * dt;
  const Real sources = qi + (qv2qi_vapdep_tend + qv2qi_nucleat_tend + qr2qi_collect_tend + qc2qi_collect_tend +
                             qr2qi_immers_freeze_tend + qc2qi_hetero_freeze_tend + qc2qi_berg_tend) * dt;
  if (sinks > sources && sinks >= C::QTENDSMALL) {
    const Real ratio = sources / sinks;
    qi2qv_sublim_tend *= ratio;
    qi2qr_melt_tend *= ratio;
  }
}

/* nc_conservation: p3_nc_conservation_impl.hpp:12-25 */
void nc_conservation(Real nc, Real nc_selfcollect_tend, Real dt, Real& nc_collect_tend,
                     Real& nc2ni_immers_freeze_tend, Real& nc_accret_tend, Real& nc2nr_autoconv_tend) {
  const Real sink_nc = (nc_collect_tend + nc2ni_immers_freeze_tend + nc_accret_tend + nc2nr_autoconv_tend) * dt;
  const Real source_nc = nc + nc_selfcollect_tend * dt;
  if (sink_nc > source_nc) {
    const Real ratio = source_nc / sink_nc;
    nc_collect_tend *= ratio;
    nc2ni_immers_freeze_tend *= ratio;
    nc_accret_tend *= ratio;
    nc2nr_autoconv_tend *= ratio;
  }
}

/* nr_conservation: p3_nr_conservation_impl.hpp:12-25 */
void nr_conservation(Real nr, Real ni2nr_melt_tend, Real nr_ice_shed_tend, Real ncshdc,
                     Real nc2nr_autoconv_tend, Real dt, Real nmltratio, Real& nr_collect_tend,
                     Real& nr2ni_immers_freeze_tend, Real& nr_selfcollect_tend, Real& nr_evap_tend) {
  const Real sink_nr = (nr_collect_tend + nr2ni_immers_freeze_tend + nr_selfcollect_tend + nr_evap_tend) * dt;
  const Real source_nr = nr + (ni2nr_melt_tend * nmltratio + nr_ice_shed_tend + ncshdc + nc2nr_autoconv_tend) * dt;
  if (sink_nr > source_nr) {
    const Real ratio = source_nr / sink_nr;
    nr_collect_tend *= ratio;
    nr2ni_immers_freeze_tend *= ratio;
    nr_selfcollect_tend *= ratio;
    nr_evap_tend *= ratio;
  }
}

/* ni_conservation: p3_ni_conservation_impl.hpp:12-24 */
void ni_conservation(Real ni, Real ni_nucleat_tend, Real nr2ni_immers_freeze_tend,
                     Real nc2ni_immers_freeze_tend, Real dt, Real& ni2nr_melt_tend,
                     Real& ni_sublim_tend, Real& ni_selfcollect_tend) {
  const Real sink_ni = (ni2nr_melt_tend + ni_sublim_tend + ni_selfcollect_tend) * dt;
  const Real source_ni = ni + (ni_nucleat_tend + nr2ni_immers_freeze_tend + nc2ni_immers_freeze_tend) * dt;
  if (sink_ni > source_ni) {
    const Real ratio = source_ni / sink_ni;
    ni2nr_melt_tend *= ratio;
    ni_sublim_tend *= ratio;
    ni_selfcollect_tend *= ratio;
  }
}

/* ice_supersat_conservation: p3_ice_supersat_conservation_impl.hpp:12-40 */
void ice_supersat_conservation(Real& qv2qi_vapdep_tend, Real& qv2qi_nucleat_tend, Real cld_frac_i,
                               Real qv, Real qv_sat_i, Real t_atm, Real dt, Real qi2qv_sublim_tend,
                               Real qr2qv_evap_tend) {
  const Real latsublim2 = (C::LatVap + C::LatIce) * (C::LatVap + C::LatIce);
  const Real qv_sink = qv2qi_vapdep_tend + qv2qi_nucleat_tend;
  if (qv_sink > C::QSMALL && cld_frac_i > 1e-20) {
    Real qv_avail = (qv + (qi2qv_sublim_tend + qr2qv_evap_tend) * dt - qv_sat_i) /
                    (1 + latsublim2 * qv_sat_i / (C::CP * C::RH2O * square(t_atm))) / dt;
    qv_avail = std::max(qv_avail, 0.);
    if (qv_sink > qv_avail) {
      const Real fract = qv_avail / qv_sink;
      qv2qi_nucleat_tend *= fract;
      qv2qi_vapdep_tend *= fract;
    }
  }
}

/* prevent_liq_supersaturation: p3_prevent_liq_supersaturation_impl.hpp:12-79 */
void prevent_liq_supersaturation(Real pres, Real t_atm, Real qv, Real dt, Real qv2qi_vapdep_tend,
                                 Real qinuc, Real& qi2qv_sublim_tend, Real& qr2qv_evap_tend, Err& e) {
  const Real qv_sources = qi2qv_sublim_tend + qr2qv_evap_tend;
  if (!(qv_sources >= C::QSMALL)) return;
  const Real qv_sinks = qv2qi_vapdep_tend + qinuc;
  const Real qv_endstep = qv - qv_sinks * dt + qv_sources * dt;
  const Real T_endstep = t_atm + ((qv_sinks - qi2qv_sublim_tend) * (C::LatVap + C::LatIce) * C::INV_CP -
                                  qr2qv_evap_tend * C::LatVap * C::INV_CP) * dt;
  (void)qv_endstep;
  const Real qsl = qv_sat_dry(T_endstep, pres, false, e);
  const Real A = C::LatVap * qsl * dt * C::INV_CP / (C::RV * T_endstep * T_endstep) *
                 ((C::LatVap + C::LatIce) * qi2qv_sublim_tend + C::LatVap * qr2qv_evap_tend);
  Real frac = (qsl - qv + qv_sinks * dt + A) / (qv_sources * dt + A);
  frac = std::max(0., frac);
  frac = std::min(1., frac);
  qi2qv_sublim_tend = frac * qi2qv_sublim_tend;
  qr2qv_evap_tend = frac * qr2qv_evap_tend;
}

/* update_prognostic_ice: p3_update_prognostics_impl.hpp:9-79 */
void update_prognostic_ice(const Rates& r, Real inv_exner, bool do_predict_nc, bool log_wetgrowth,
                           Real dt, Real nmltratio, Real rho_qm_cloud, Real& th_atm, Real& qv,
                           Real& qi, Real& ni, Real& qm, Real& bm, Real& qc, Real& nc, Real& qr, Real& nr) {
  qc = qc + (-r.qc2qi_hetero_freeze_tend - r.qc2qi_collect_tend - r.qc2qr_ice_shed_tend - r.qc2qi_berg_tend) * dt;
  if (do_predict_nc) nc = nc + (-r.nc_collect_tend - r.nc2ni_immers_freeze_tend) * dt;
  qr = qr + (-r.qr2qi_collect_tend + r.qi2qr_melt_tend - r.qr2qi_immers_freeze_tend + r.qc2qr_ice_shed_tend) * dt;
  nr = nr + (-r.nr_collect_tend - r.nr2ni_immers_freeze_tend + nmltratio * r.ni2nr_melt_tend + r.nr_ice_shed_tend + r.ncshdc) * dt;
  if (qi >= C::QSMALL) {
    bm = bm - ((r.qi2qv_sublim_tend + r.qi2qr_melt_tend) / qi) * dt * bm;
    qm = qm - ((r.qi2qv_sublim_tend + r.qi2qr_melt_tend) * qm / qi) * dt;
    qi = qi - (r.qi2qv_sublim_tend + r.qi2qr_melt_tend) * dt;
  }
  const Real dum = (r.qr2qi_collect_tend + r.qc2qi_collect_tend + r.qr2qi_immers_freeze_tend + r.qc2qi_hetero_freeze_tend) * dt;
  qi = qi + (r.qv2qi_vapdep_tend + r.qv2qi_nucleat_tend + r.qc2qi_berg_tend) * dt + dum;
  qm = qm + dum;
  bm = bm + (r.qr2qi_collect_tend * C::INV_RHO_RIMEMAX + r.qc2qi_collect_tend / rho_qm_cloud +
             (r.qr2qi_immers_freeze_tend + r.qc2qi_hetero_freeze_tend) * C::INV_RHO_RIMEMAX) * dt;
  ni = ni + (r.ni_nucleat_tend - r.ni2nr_melt_tend - r.ni_sublim_tend - r.ni_selfcollect_tend +
             r.nr2ni_immers_freeze_tend + r.nc2ni_immers_freeze_tend) * dt;
  if (qm < 0) {
    qm = 0;
    bm = 0;
  }
  if (log_wetgrowth) {
    qm = qi;
    bm = qm * C::INV_RHO_RIMEMAX;
  }
  qv = qv + (-r.qv2qi_vapdep_tend + r.qi2qv_sublim_tend - r.qv2qi_nucleat_tend) * dt;
  th_atm = th_atm + inv_exner * ((r.qv2qi_vapdep_tend - r.qi2qv_sublim_tend + r.qv2qi_nucleat_tend) * (C::LatVap + C::LatIce) * C::INV_CP +
                                 (r.qr2qi_collect_tend + r.qc2qi_collect_tend + r.qc2qi_hetero_freeze_tend + r.qr2qi_immers_freeze_tend -
                                  r.qi2qr_melt_tend + r.qc2qi_berg_tend) * C::LatIce * C::INV_CP) * dt;
}

/* update_prognostic_liquid: p3_update_prognostics_impl.hpp:81-123 (IPARAM = 3) */
void update_prognostic_liquid(const Rates& r, bool do_predict_nc, bool do_prescribed_CCN, Real inv_rho,
                              Real inv_exner, Real dt, Real& th_atm, Real& qv, Real& qc, Real& nc,
                              Real& qr, Real& nr) {
  qc = qc + (-r.qc2qr_accret_tend - r.qc2qr_autoconv_tend) * dt;
  qr = qr + (r.qc2qr_accret_tend + r.qc2qr_autoconv_tend - r.qr2qv_evap_tend) * dt;
  if (do_predict_nc || do_prescribed_CCN) {
    nc = nc + (-r.nc_accret_tend - r.nc2nr_autoconv_tend + r.nc_selfcollect_tend) * dt;
  } else {
    nc = C::NCCNST * inv_rho;
  }
  nr = nr + (r.ncautr - r.nr_selfcollect_tend - r.nr_evap_tend) * dt;
  qv = qv + r.qr2qv_evap_tend * dt;
  th_atm = th_atm + inv_exner * (-r.qr2qv_evap_tend * C::LatVap * C::INV_CP) * dt;
}

/* ---------------------------------------------------------------------- */
/* Sedimentation: p3/impl/p3_upwind_impl.hpp, p3_find_impl.hpp,             */
/* p3_cloud_sed_impl.hpp, p3_rain_sed_impl.hpp, p3_ice_sed_impl.hpp          */
/* ---------------------------------------------------------------------- */

/* find_bottom / find_top (serial branch): p3_find_impl.hpp:14-92 */
int find_bottom(const Real* v, Real small, int kbot, int ktop, int kdir, bool& present) {
  present = false;
  int k_xbot = 0;
  for (int k = kbot; k != ktop + kdir; k += kdir) {
    if (v[k] < small) continue;
    k_xbot = k;
    present = true;
    break;
  }
  return k_xbot;
}
int find_top(const Real* v, Real small, int kbot, int ktop, int kdir, bool& present) {
  present = false;
  int k_xtop = 0;
  for (int k = ktop; k != kbot - kdir; k -= kdir) {
    if (v[k] < small) continue;
    k_xtop = k;
    present = true;
    break;
  }
  return k_xtop;
}

/* calc_first_order_upwind_step: p3_upwind_impl.hpp:14-80 (pack size 1).
 * Fluxes are formed from start-of-substep values, then every cell in
 * [k_top, k_bot] (kdir = -1) or [k_bot, k_top] (kdir = +1) is updated; the
 * top cell has zero inflow. */
void upwind_step(const Real* rho, const Real* inv_rho, const Real* inv_dz, int k_bot, int k_top,
                 int kdir, Real dt_sub, int nfield, Real* const* flux, Real* const* V, Real* const* r) {
  const int kmin = (kdir == 1 ? k_bot : k_top);
  const int kmax = (kdir == 1 ? k_top : k_bot);
  for (int k = kmin; k <= kmax; ++k)
    for (int f = 0; f < nfield; ++f) flux[f][k] = V[f][k] * r[f][k] * rho[k];
  {
    const int k = k_top;
    for (int f = 0; f < nfield; ++f) {
      const Real fluxdiv = (0 - flux[f][k]) * inv_dz[k];
      r[f][k] += fluxdiv * dt_sub * inv_rho[k];
    }
  }
  int lo = kmin, hi = kmax;
  if (kdir == 1) --hi; else ++lo;
  for (int k = lo; k <= hi; ++k) {
    for (int f = 0; f < nfield; ++f) {
      const Real flux_pkdir = flux[f][k + kdir];
      const Real fluxdiv = (flux_pkdir - flux[f][k]) * inv_dz[k];
      r[f][k] += fluxdiv * dt_sub * inv_rho[k];
    }
  }
}

/* generalized_sedimentation: p3_upwind_impl.hpp:82-116 */
void generalized_sedimentation(const Real* rho, const Real* inv_rho, const Real* inv_dz, int k_qxtop,
                               int& k_qxbot, int kbot, int kdir, Real Co_max, Real& dt_left,
                               Real& prt_accum, int nfield, Real* const* fluxes, Real* const* Vs,
                               Real* const* rs) {
  const int tmpint1 = static_cast<int>(Co_max + 1);
  const Real dt_sub = dt_left / tmpint1;
  const int k_temp = (k_qxbot == kbot) ? k_qxbot : k_qxbot - kdir;
  upwind_step(rho, inv_rho, inv_dz, k_temp, k_qxtop, kdir, dt_sub, nfield, fluxes, Vs, rs);
  if (k_qxbot == kbot) {
    prt_accum += fluxes[0][kbot] * dt_sub;
  } else {
    k_qxbot -= kdir;
  }
  dt_left -= dt_sub;
}

/* Per-column workspace, mirroring the 44 workspace slots of
 * p3_main_impl.hpp:126-163 that carry information between stages. */
struct Work {
  std::vector<Real> mu_r, T_atm, lamr, logn0r, nu, cdist, cdist1, cdistr, inv_cld_frac_i,
      inv_cld_frac_l, inv_cld_frac_r, qc_incld, qr_incld, qi_incld, qm_incld, nc_incld, nr_incld,
      ni_incld, bm_incld, inv_dz, inv_rho, rho, rhofacr, rhofaci, acn, qv_sat_l, qv_sat_i,
      qv_supersat_i, exner, mu_c, lamc;
  std::vector<Real> V1, V2, F1, F2, F3, F4;
  void resize(int nk) {
    for (auto* v : {&mu_r, &T_atm, &lamr, &logn0r, &nu, &cdist, &cdist1, &cdistr, &inv_cld_frac_i,
                    &inv_cld_frac_l, &inv_cld_frac_r, &qc_incld, &qr_incld, &qi_incld, &qm_incld,
                    &nc_incld, &nr_incld, &ni_incld, &bm_incld, &inv_dz, &inv_rho, &rho, &rhofacr,
                    &rhofaci, &acn, &qv_sat_l, &qv_sat_i, &qv_supersat_i, &exner, &mu_c, &lamc, &V1,
                    &V2, &F1, &F2, &F3, &F4})
      v->assign(nk, 0.0);
  }
};

/* One column.  Stage order, early exits and argument flow follow
 * p3_main_internal (p3_main_impl.hpp:108-325). */
struct Col {
  Real *qc, *nc, *qr, *nr, *qi, *qm, *ni, *bm, *qv, *th;
  const Real *nc_nuceat_tend, *nccn, *ni_activated, *inv_qc_relvar, *cld_frac_i, *cld_frac_l,
      *cld_frac_r, *pres, *dz, *dpres, *inv_exner, *qv_prev, *t_prev;
  Real *qv2qi_depos_tend, *precip_liq_surf, *precip_ice_surf, *diag_eff_radius_qc,
      *diag_eff_radius_qi, *diag_eff_radius_qr, *rho_qi, *precip_liq_flux, *precip_ice_flux,
      *precip_total_tend, *nevapr, *liq_ice_exchange, *vap_liq_exchange, *vap_ice_exchange;
};

/* p3_main_init, p3_main_part1 and p3_main_part2 of one column.  Returns
 * false when the column takes one of the two early exits of
 * p3_main_internal (p3_main_impl.hpp:237-239 after part1, :260 after part2),
 * which skip everything after them. */
bool p3_column_part12(const Col& c, int nk, Real dt, bool predictNc, bool prescribedCCN,
                      const p3o_runtime& rt, const p3o_tables* tab, Work& w, Err& e) {
  const Real inv_dt = 1 / dt;
  const bool do_ice_production = rt.do_ice_production != 0;

  /* p3_main_init: p3_main_impl.hpp:18-72 */
  *c.precip_liq_surf = 0;
  *c.precip_ice_surf = 0;
  for (int k = 0; k < nk; ++k) {
    c.diag_eff_radius_qc[k] = 10.e-6;
    c.diag_eff_radius_qi[k] = 25.e-6;
    c.diag_eff_radius_qr[k] = 500.e-6;
    w.inv_cld_frac_i[k] = 1 / c.cld_frac_i[k];
    w.inv_cld_frac_l[k] = 1 / c.cld_frac_l[k];
    w.inv_cld_frac_r[k] = 1 / c.cld_frac_r[k];
    w.exner[k] = 1 / c.inv_exner[k];
    w.T_atm[k] = c.th[k] * w.exner[k];
    c.qv[k] = std::max(c.qv[k], 0.);
    w.inv_dz[k] = 1 / c.dz[k];
    c.rho_qi[k] = 0;
    c.qv2qi_depos_tend[k] = 0;
    c.precip_total_tend[k] = 0;
    c.nevapr[k] = 0;
    /* history fields are zero-filled by the caller in the reference
     * (eamxx_p3_run.cpp:27-29); done here so the step is self-contained. */
    c.liq_ice_exchange[k] = 0;
    c.vap_liq_exchange[k] = 0;
    c.vap_ice_exchange[k] = 0;
  }
  for (int k = 0; k <= nk; ++k) {
    c.precip_liq_flux[k] = 0;
    c.precip_ice_flux[k] = 0;
  }
  for (auto* v : {&w.mu_r, &w.lamr, &w.logn0r, &w.nu, &w.cdist, &w.cdist1, &w.cdistr, &w.qc_incld,
                  &w.qr_incld, &w.qi_incld, &w.qm_incld, &w.nc_incld, &w.nr_incld, &w.ni_incld,
                  &w.bm_incld, &w.inv_rho, &w.rho, &w.rhofacr, &w.rhofaci, &w.acn, &w.qv_sat_l,
                  &w.qv_sat_i, &w.qv_supersat_i, &w.mu_c, &w.lamc})
    std::fill(v->begin(), v->end(), 0.0);

  /* p3_main_part1: p3_main_impl_part1.hpp:18-185 */
  bool nucleationPossible = false, hydrometeorsPresent = false;
  for (int k = 0; k < nk; ++k) {
    w.rho[k] = c.dpres[k] / c.dz[k] / C::gravit;
    w.inv_rho[k] = 1 / w.rho[k];
    w.qv_sat_l[k] = qv_sat_dry(w.T_atm[k], c.pres[k], false, e);
    w.qv_sat_i[k] = qv_sat_dry(w.T_atm[k], c.pres[k], true, e);
    w.qv_supersat_i[k] = c.qv[k] / w.qv_sat_i[k] - 1;
    w.rhofacr[k] = std::pow(C::RHO_1000MB * w.inv_rho[k], .54);
    w.rhofaci[k] = std::pow(C::RHO_600MB * w.inv_rho[k], .54);
    const Real dum = 1.496e-6 * std::pow(w.T_atm[k], 1.5) / (w.T_atm[k] + 120);
    w.acn[k] = C::gravit * C::RHO_H2O / (18 * dum);
    if (w.T_atm[k] < C::T_zerodegc && w.qv_supersat_i[k] >= -0.05) nucleationPossible = true;

    if (c.qc[k] < C::QSMALL) {
      c.qv[k] = c.qv[k] + c.qc[k];
      c.th[k] = c.th[k] - c.inv_exner[k] * c.qc[k] * C::LatVap * C::INV_CP;
      c.qc[k] = 0;
      c.nc[k] = 0;
    } else {
      hydrometeorsPresent = true;
      if (prescribedCCN) {
        c.nc[k] = std::max(c.nc[k], rt.spa_ccn_to_nc_factor * c.nccn[k] / w.inv_cld_frac_l[k]);
      } else if (predictNc) {
        c.nc[k] = std::max(c.nc[k] + c.nc_nuceat_tend[k] * dt, 0.0);
      } else {
        c.nc[k] = C::NCCNST * w.inv_rho[k];
      }
    }
    if (c.qr[k] < C::QSMALL) {
      c.qv[k] = c.qv[k] + c.qr[k];
      c.th[k] = c.th[k] - c.inv_exner[k] * c.qr[k] * C::LatVap * C::INV_CP;
      c.qr[k] = 0;
      c.nr[k] = 0;
    } else {
      hydrometeorsPresent = true;
    }
    if (c.qi[k] < C::QSMALL || (c.qi[k] < 1.e-8 && w.qv_supersat_i[k] < -0.1)) {
      c.qv[k] = c.qv[k] + c.qi[k];
      c.th[k] = c.th[k] - c.inv_exner[k] * c.qi[k] * (C::LatVap + C::LatIce) * C::INV_CP;
      c.qi[k] = 0;
      c.ni[k] = 0;
      c.qm[k] = 0;
      c.bm[k] = 0;
    } else {
      hydrometeorsPresent = true;
    }
    if (c.qi[k] >= C::QSMALL && c.qi[k] < 1.e-8 && w.T_atm[k] >= C::T_zerodegc) {
      c.qr[k] = c.qr[k] + c.qi[k];
      c.th[k] = c.th[k] - c.inv_exner[k] * c.qi[k] * C::LatIce * C::INV_CP;
      c.qi[k] = 0;
      c.ni[k] = 0;
      c.qm[k] = 0;
      c.bm[k] = 0;
    }
    w.T_atm[k] = c.th[k] * w.exner[k];
    calculate_incloud_mixingratios(c.qc[k], c.qr[k], c.qi[k], c.qm[k], c.nc[k], c.nr[k], c.ni[k], c.bm[k],
                                   w.inv_cld_frac_l[k], w.inv_cld_frac_i[k], w.inv_cld_frac_r[k],
                                   w.qc_incld[k], w.qr_incld[k], w.qi_incld[k], w.qm_incld[k],
                                   w.nc_incld[k], w.nr_incld[k], w.ni_incld[k], w.bm_incld[k]);
  }

  if (!(nucleationPossible || hydrometeorsPresent)) return false;

  /* p3_main_part2: p3_main_impl_part2.hpp:18-526 */
  hydrometeorsPresent = false;
  for (int k = 0; k < nk; ++k) {
    const bool skip_all = (c.qc[k] < C::QSMALL && c.qr[k] < C::QSMALL && c.qi[k] < C::QSMALL &&
                           w.T_atm[k] < C::T_zerodegc && w.qv_supersat_i[k] < -0.05);
    if (skip_all) continue;

    Rates r;
    Real mu = 0, dv = 0, sc = 0, dqsdt = 0, dqsidt = 0, ab = 0, abi = 0, kap = 0, eii = 0;
    Real table_val_qi_fallspd = 0, table_val_ni_self_collect = 0, table_val_qc2qi_collect = 0,
         table_val_qi2qr_melting = 0, table_val_nr_collect = 0, table_val_qr2qi_collect = 0,
         table_val_ni_lammax = 0, table_val_ni_lammin = 0, table_val_qi2qr_vent_melt = 0;
    Real vtrmi1 = 0, rho_qm_cloud = 400, epsi = 0, epsr = 0, epsc = 0, epsi_tot = 0;
    bool wetgrowth = false;

    const bool skip_micro = !(w.qc_incld[k] >= C::QSMALL || w.qr_incld[k] >= C::QSMALL || w.qi_incld[k] >= C::QSMALL);
    if (!skip_micro) {
      get_time_space_phys_variables(w.T_atm[k], c.pres[k], w.rho[k], w.qv_sat_l[k], w.qv_sat_i[k], mu, dv,
                                    sc, dqsdt, dqsidt, ab, abi, kap, eii);
      get_cloud_dsd2(w.qc_incld[k], w.nc_incld[k], w.mu_c[k], w.rho[k], w.nu[k], w.lamc[k], w.cdist[k], w.cdist1[k]);
      c.nc[k] = w.nc_incld[k] * c.cld_frac_l[k];
      get_rain_dsd2(w.qr_incld[k], w.nr_incld[k], w.mu_r[k], w.lamr[k], rt);
      get_cdistr_logn0r(w.qr_incld[k], w.nr_incld[k], w.mu_r[k], w.lamr[k], w.cdistr[k], w.logn0r[k]);
      c.nr[k] = w.nr_incld[k] * c.cld_frac_r[k];
      impose_max_total_ni(w.ni_incld[k], rt.max_total_ni, w.inv_rho[k]);

      if (w.qi_incld[k] >= C::QSMALL) {
        w.ni_incld[k] = std::max(w.ni_incld[k], C::NSMALL);
        w.nr_incld[k] = std::max(w.nr_incld[k], C::NSMALL);
        const Real rhop = calc_bulk_rho_rime(w.qi_incld[k], w.qm_incld[k], w.bm_incld[k], rt);
        c.qm[k] = w.qm_incld[k] * c.cld_frac_i[k];
        c.bm[k] = w.bm_incld[k] * c.cld_frac_i[k];
        TableIce ti;
        lookup_ice(w.qi_incld[k], w.ni_incld[k], w.qm_incld[k], rhop, ti);
        TableRain tr;
        lookup_rain(w.qr_incld[k], w.nr_incld[k], tr);
        table_val_qi_fallspd = apply_table_ice(1, tab, ti);
        table_val_ni_self_collect = apply_table_ice(2, tab, ti);
        table_val_qc2qi_collect = apply_table_ice(3, tab, ti);
        table_val_qi2qr_melting = apply_table_ice(4, tab, ti);
        table_val_ni_lammax = apply_table_ice(6, tab, ti);
        table_val_ni_lammin = apply_table_ice(7, tab, ti);
        table_val_qi2qr_vent_melt = apply_table_ice(9, tab, ti);
        if (w.qr_incld[k] >= C::QSMALL) {
          table_val_nr_collect = apply_table_coll(0, tab, ti, tr);
          table_val_qr2qi_collect = apply_table_coll(1, tab, ti, tr);
        }
        w.ni_incld[k] = std::min(w.ni_incld[k], table_val_ni_lammax * w.ni_incld[k]);
        w.ni_incld[k] = std::max(w.ni_incld[k], table_val_ni_lammin * w.ni_incld[k]);
      }

      if (do_ice_production) {
        ice_cldliq_collection(w.rho[k], w.T_atm[k], w.rhofaci[k], table_val_qc2qi_collect, w.qi_incld[k],
                              w.qc_incld[k], w.ni_incld[k], w.nc_incld[k], r.qc2qi_collect_tend,
                              r.nc_collect_tend, r.qc2qr_ice_shed_tend, r.ncshdc, rt);
        ice_rain_collection(w.rho[k], w.T_atm[k], w.rhofaci[k], w.logn0r[k], table_val_nr_collect,
                            table_val_qr2qi_collect, w.qi_incld[k], w.ni_incld[k], w.qr_incld[k],
                            r.qr2qi_collect_tend, r.nr_collect_tend, rt);
        ice_self_collection(w.rho[k], w.rhofaci[k], table_val_ni_self_collect, eii, w.qm_incld[k],
                            w.qi_incld[k], w.ni_incld[k], r.ni_selfcollect_tend);
      }
      ice_melting(w.rho[k], w.T_atm[k], c.pres[k], w.rhofaci[k], table_val_qi2qr_melting,
                  table_val_qi2qr_vent_melt, dv, sc, mu, kap, c.qv[k], w.qi_incld[k], w.ni_incld[k],
                  r.qi2qr_melt_tend, r.ni2nr_melt_tend, e);
      if (do_ice_production) {
        ice_cldliq_wet_growth(w.rho[k], w.T_atm[k], c.pres[k], w.rhofaci[k], table_val_qi2qr_melting,
                              table_val_qi2qr_vent_melt, dv, kap, mu, sc, c.qv[k], w.qc_incld[k],
                              w.qi_incld[k], w.ni_incld[k], w.qr_incld[k], wetgrowth,
                              r.qr2qi_collect_tend, r.qc2qi_collect_tend, r.qc_growth_rate,
                              r.nr_ice_shed_tend, r.qc2qr_ice_shed_tend, e);
      }
      ice_relaxation_timescale(w.rho[k], w.T_atm[k], w.rhofaci[k], table_val_qi2qr_melting,
                               table_val_qi2qr_vent_melt, dv, mu, sc, w.qi_incld[k], w.ni_incld[k],
                               epsi, epsi_tot);
      calc_rime_density(w.T_atm[k], w.rhofaci[k], table_val_qi_fallspd, w.acn[k], w.lamc[k], w.mu_c[k],
                        w.qc_incld[k], r.qc2qi_collect_tend, vtrmi1, rho_qm_cloud);
      if (do_ice_production) {
        cldliq_immersion_freezing(w.T_atm[k], w.lamc[k], w.mu_c[k], w.cdist1[k], w.qc_incld[k],
                                  r.qc2qi_hetero_freeze_tend, r.nc2ni_immers_freeze_tend, rt);
        rain_immersion_freezing(w.T_atm[k], w.lamr[k], w.mu_r[k], w.cdistr[k], w.qr_incld[k],
                                r.qr2qi_immers_freeze_tend, r.nr2ni_immers_freeze_tend, rt);
      }
      calc_liq_relaxation_timescale(tab, w.rho[k], C::f1r, C::f2r, dv, mu, sc, w.mu_r[k], w.lamr[k],
                                    w.cdistr[k], w.cdist[k], w.qr_incld[k], w.qc_incld[k], epsr, epsc);
      evaporate_rain(w.qr_incld[k], w.qc_incld[k], w.nr_incld[k], w.qi_incld[k], c.cld_frac_l[k],
                     c.cld_frac_r[k], c.qv[k], c.qv_prev[k], w.qv_sat_l[k], w.qv_sat_i[k], ab, abi, epsr,
                     epsi_tot, w.T_atm[k], c.t_prev[k], dqsdt, dt, r.qr2qv_evap_tend, r.nr_evap_tend);
      if (do_ice_production) {
        ice_deposition_sublimation(w.qi_incld[k], w.ni_incld[k], w.T_atm[k], w.qv_sat_l[k], w.qv_sat_i[k],
                                   epsi, abi, c.qv[k], inv_dt, r.qv2qi_vapdep_tend, r.qi2qv_sublim_tend,
                                   r.ni_sublim_tend, r.qc2qi_berg_tend);
      }
    }

    if (do_ice_production) {
      ice_nucleation(w.T_atm[k], w.inv_rho[k], c.ni[k], c.ni_activated[k], w.qv_supersat_i[k], inv_dt,
                     predictNc, prescribedCCN, r.qv2qi_nucleat_tend, r.ni_nucleat_tend, rt);
    }
    cloud_water_autoconversion(w.rho[k], w.qc_incld[k], w.nc_incld[k], r.qc2qr_autoconv_tend,
                               r.nc2nr_autoconv_tend, r.ncautr, rt);
    droplet_self_collection(w.qc_incld[k], r.nc_selfcollect_tend);
    cloud_rain_accretion(w.qc_incld[k], w.nc_incld[k], w.qr_incld[k], r.qc2qr_accret_tend,
                         r.nc_accret_tend, rt);
    rain_self_collection(w.rho[k], w.qr_incld[k], w.nr_incld[k], r.nr_selfcollect_tend, rt);
    back_to_cell_average(c.cld_frac_l[k], c.cld_frac_r[k], c.cld_frac_i[k], r);

    cloud_water_conservation(c.qc[k], dt, r.qc2qr_autoconv_tend, r.qc2qr_accret_tend, r.qc2qi_collect_tend,
                             r.qc2qi_hetero_freeze_tend, r.qc2qr_ice_shed_tend, r.qc2qi_berg_tend,
                             r.qi2qv_sublim_tend, r.qv2qi_vapdep_tend);
    rain_water_conservation(c.qr[k], r.qc2qr_autoconv_tend, r.qc2qr_accret_tend, r.qi2qr_melt_tend,
                            r.qc2qr_ice_shed_tend, dt, r.qr2qv_evap_tend, r.qr2qi_collect_tend,
                            r.qr2qi_immers_freeze_tend);
    ice_water_conservation(c.qi[k], r.qv2qi_vapdep_tend, r.qv2qi_nucleat_tend, r.qc2qi_berg_tend,
                           r.qr2qi_collect_tend, r.qc2qi_collect_tend, r.qr2qi_immers_freeze_tend,
                           r.qc2qi_hetero_freeze_tend, dt, r.qi2qv_sublim_tend, r.qi2qr_melt_tend);
    nc_conservation(c.nc[k], r.nc_selfcollect_tend, dt, r.nc_collect_tend, r.nc2ni_immers_freeze_tend,
                    r.nc_accret_tend, r.nc2nr_autoconv_tend);
    nr_conservation(c.nr[k], r.ni2nr_melt_tend, r.nr_ice_shed_tend, r.ncshdc, r.nc2nr_autoconv_tend, dt,
                    C::nmltratio, r.nr_collect_tend, r.nr2ni_immers_freeze_tend, r.nr_selfcollect_tend,
                    r.nr_evap_tend);
    ni_conservation(c.ni[k], r.ni_nucleat_tend, r.nr2ni_immers_freeze_tend, r.nc2ni_immers_freeze_tend, dt,
                    r.ni2nr_melt_tend, r.ni_sublim_tend, r.ni_selfcollect_tend);
    ice_supersat_conservation(r.qv2qi_vapdep_tend, r.qv2qi_nucleat_tend, c.cld_frac_i[k], c.qv[k],
                              w.qv_sat_i[k], c.th[k] / c.inv_exner[k], dt, r.qi2qv_sublim_tend,
                              r.qr2qv_evap_tend);
    prevent_liq_supersaturation(c.pres[k], w.T_atm[k], c.qv[k], dt, r.qv2qi_vapdep_tend,
                                r.qv2qi_nucleat_tend, r.qi2qv_sublim_tend, r.qr2qv_evap_tend, e);

    update_prognostic_ice(r, c.inv_exner[k], predictNc, wetgrowth, dt, C::nmltratio, rho_qm_cloud, c.th[k],
                          c.qv[k], c.qi[k], c.ni[k], c.qm[k], c.bm[k], c.qc[k], c.nc[k], c.qr[k], c.nr[k]);
    update_prognostic_liquid(r, predictNc, prescribedCCN, w.inv_rho[k], c.inv_exner[k], dt, c.th[k], c.qv[k],
                             c.qc[k], c.nc[k], c.qr[k], c.nr[k]);

    c.qv2qi_depos_tend[k] = r.qv2qi_vapdep_tend - r.qi2qv_sublim_tend + r.qv2qi_nucleat_tend;
    c.precip_total_tend[k] = r.qc2qr_accret_tend + r.qc2qr_autoconv_tend + r.qc2qr_ice_shed_tend + r.qc2qi_collect_tend;
    c.nevapr[k] = r.qi2qv_sublim_tend + r.qr2qv_evap_tend;
    c.vap_ice_exchange[k] = r.qv2qi_vapdep_tend - r.qi2qv_sublim_tend + r.qv2qi_nucleat_tend;
    c.vap_liq_exchange[k] = -r.qr2qv_evap_tend;
    c.liq_ice_exchange[k] = r.qc2qi_hetero_freeze_tend + r.qr2qi_immers_freeze_tend - r.qi2qr_melt_tend +
                            r.qc2qi_berg_tend + r.qc2qi_collect_tend + r.qr2qi_collect_tend;

    if (c.qc[k] < C::QSMALL) {
      c.qv[k] = c.qv[k] + c.qc[k];
      c.th[k] = c.th[k] - c.inv_exner[k] * c.qc[k] * C::LatVap * C::INV_CP;
      c.qc[k] = 0;
      c.nc[k] = 0;
    } else {
      hydrometeorsPresent = true;
    }
    if (c.qr[k] < C::QSMALL) {
      c.qv[k] = c.qv[k] + c.qr[k];
      c.th[k] = c.th[k] - c.inv_exner[k] * c.qr[k] * C::LatVap * C::INV_CP;
      c.qr[k] = 0;
      c.nr[k] = 0;
    } else {
      hydrometeorsPresent = true;
    }
    if (c.qi[k] < C::QSMALL) {
      c.qv[k] = c.qv[k] + c.qi[k];
      c.th[k] = c.th[k] - c.inv_exner[k] * c.qi[k] * (C::LatVap + C::LatIce) * C::INV_CP;
      c.qi[k] = 0;
      c.ni[k] = 0;
      c.qm[k] = 0;
      c.bm[k] = 0;
    } else {
      hydrometeorsPresent = true;
    }

    w.ni_incld[k] = c.ni[k] / c.cld_frac_i[k];
    impose_max_total_ni(w.ni_incld[k], rt.max_total_ni, w.inv_rho[k]);
    c.ni[k] = w.ni_incld[k] * c.cld_frac_i[k];
    calculate_incloud_mixingratios(c.qc[k], c.qr[k], c.qi[k], c.qm[k], c.nc[k], c.nr[k], c.ni[k], c.bm[k],
                                   w.inv_cld_frac_l[k], w.inv_cld_frac_i[k], w.inv_cld_frac_r[k],
                                   w.qc_incld[k], w.qr_incld[k], w.qi_incld[k], w.qm_incld[k],
                                   w.nc_incld[k], w.nr_incld[k], w.ni_incld[k], w.bm_incld[k]);
  }

  return hydrometeorsPresent;
}

/* Cloud, rain and ice sedimentation, homogeneous freezing and
 * p3_main_part3 of a column that went on past part2
 * (p3_main_impl.hpp:262-325).  Reads from the workspace the per-level
 * density, its inverse, 1/dz, the fall-speed factors (rhofacr, rhofaci,
 * acn), the temperature after part1 (homogeneous freezing uses it) and the
 * in-cloud mixing ratios of the state left by part2. */
void p3_column_sed_part3(const Col& c, int nk, Real dt, bool predictNc, const p3o_runtime& rt,
                         const p3o_tables* tab, Work& w, Err& e) {
  const Real inv_dt = 1 / dt;
  const int kdir = -1, ktop = 0, kbot = nk - 1;
  const bool do_ice_production = rt.do_ice_production != 0;
  const Real* rho = w.rho.data();
  const Real* inv_rho = w.inv_rho.data();
  const Real* inv_dz = w.inv_dz.data();

  /* cloud_sedimentation: p3_cloud_sed_impl.hpp:14-147 */
  {
    bool present;
    const int k_qxtop = find_top(c.qc, C::QSMALL, kbot, ktop, kdir, present);
    if (present) {
      Real dt_left = dt, prt_accum = 0.0;
      int k_qxbot = find_bottom(c.qc, C::QSMALL, kbot, k_qxtop, kdir, present);
      int nsub = 0;
      while (dt_left > C::dt_left_tol) {
        if (++nsub > kMaxSubsteps) { e.bits |= P3O_ESUBSTEP; break; }
        Real Co_max = 0.0;
        std::fill(w.V1.begin(), w.V1.end(), 0.0);
        if (predictNc) std::fill(w.V2.begin(), w.V2.end(), 0.0);
        for (int k = k_qxtop; k <= k_qxbot; ++k) {
          if (w.qc_incld[k] > C::QSMALL) {
            Real nu, cdist, cdist1;
            get_cloud_dsd2(w.qc_incld[k], w.nc_incld[k], w.mu_c[k], rho[k], nu, w.lamc[k], cdist, cdist1);
            c.nc[k] = w.nc_incld[k] * c.cld_frac_l[k];
            const Real dum = 1 / std::pow(w.lamc[k], C::bcn);
            w.V1[k] = w.acn[k] * std::tgamma(4 + C::bcn + w.mu_c[k]) * dum / std::tgamma(w.mu_c[k] + 4);
            if (predictNc) w.V2[k] = w.acn[k] * std::tgamma(1 + C::bcn + w.mu_c[k]) * dum / std::tgamma(w.mu_c[k] + 1);
            Co_max = std::max(Co_max, w.V1[k] * dt_left * inv_dz[k]);
          }
        }
        if (!(Co_max >= 0)) { e.bits |= P3O_ENUMERIC; break; }
        Real* fl[2] = {w.F1.data(), w.F2.data()};
        Real* vs[2] = {w.V1.data(), w.V2.data()};
        Real* rs[2] = {c.qc, c.nc};
        generalized_sedimentation(rho, inv_rho, inv_dz, k_qxtop, k_qxbot, kbot, kdir, Co_max, dt_left,
                                  prt_accum, predictNc ? 2 : 1, fl, vs, rs);
        for (int k = 0; k < nk; ++k) {
          w.qc_incld[k] = c.qc[k] / c.cld_frac_l[k];
          w.nc_incld[k] = c.nc[k] / c.cld_frac_l[k];
        }
      }
      *c.precip_liq_surf = prt_accum * C::INV_RHO_H2O * inv_dt;
    }
  }

  /* rain_sedimentation: p3_rain_sed_impl.hpp:38-170 */
  {
    bool present;
    const int k_qxtop = find_top(c.qr, C::QSMALL, kbot, ktop, kdir, present);
    if (present) {
      Real dt_left = dt, prt_accum = 0.0;
      int k_qxbot = find_bottom(c.qr, C::QSMALL, kbot, k_qxtop, kdir, present);
      int nsub = 0;
      while (dt_left > C::dt_left_tol) {
        if (++nsub > kMaxSubsteps) { e.bits |= P3O_ESUBSTEP; break; }
        Real Co_max = 0.0;
        std::fill(w.V1.begin(), w.V1.end(), 0.0);
        std::fill(w.V2.begin(), w.V2.end(), 0.0);
        for (int k = k_qxtop; k <= k_qxbot; ++k) {
          if (w.qr_incld[k] > C::QSMALL) {
            /* compute_rain_fall_velocity: p3_rain_sed_impl.hpp:14-36 */
            get_rain_dsd2(w.qr_incld[k], w.nr_incld[k], w.mu_r[k], w.lamr[k], rt);
            Table3 t3;
            lookup3(w.mu_r[k], w.lamr[k], t3);
            w.V1[k] = apply_table3(tab->vm, t3) * w.rhofacr[k];
            w.V2[k] = apply_table3(tab->vn, t3) * w.rhofacr[k];
            c.nr[k] = w.nr_incld[k] * c.cld_frac_r[k];
            Co_max = std::max(Co_max, w.V1[k] * dt_left * inv_dz[k]);
          }
        }
        if (!(Co_max >= 0)) { e.bits |= P3O_ENUMERIC; break; }
        Real* fl[2] = {w.F1.data(), w.F2.data()};
        Real* vs[2] = {w.V1.data(), w.V2.data()};
        Real* rs[2] = {c.qr, c.nr};
        generalized_sedimentation(rho, inv_rho, inv_dz, k_qxtop, k_qxbot, kbot, kdir, Co_max, dt_left,
                                  prt_accum, 2, fl, vs, rs);
        for (int k = 0; k < nk; ++k) {
          w.qr_incld[k] = c.qr[k] / c.cld_frac_r[k];
          w.nr_incld[k] = c.nr[k] / c.cld_frac_r[k];
        }
        /* precip_liq_flux accumulation (p3_rain_sed_impl.hpp:139-153): the
         * interface below level k receives flux_qx(k) every substep. */
        for (int k = k_qxtop + 1; k <= k_qxbot + 1; ++k) {
          c.precip_liq_flux[k] = c.precip_liq_flux[k] + w.F1[k - 1];
        }
      }
      *c.precip_liq_surf += prt_accum * C::INV_RHO_H2O * inv_dt;
    }
  }

  /* ice_sedimentation: p3_ice_sed_impl.hpp:66-205 */
  {
    bool present;
    const int k_qxtop = find_top(c.qi, C::QSMALL, kbot, ktop, kdir, present);
    if (present) {
      Real dt_left = dt, prt_accum = 0.0;
      int k_qxbot = find_bottom(c.qi, C::QSMALL, kbot, k_qxtop, kdir, present);
      int nsub = 0;
      while (dt_left > C::dt_left_tol) {
        if (++nsub > kMaxSubsteps) { e.bits |= P3O_ESUBSTEP; break; }
        Real Co_max = 0.0;
        std::fill(w.V1.begin(), w.V1.end(), 0.0);
        std::fill(w.V2.begin(), w.V2.end(), 0.0);
        for (int k = k_qxtop; k <= k_qxbot; ++k) {
          if (w.qi_incld[k] > C::QSMALL) {
            w.ni_incld[k] = std::max(w.ni_incld[k], C::NSMALL);
            const Real rhop = calc_bulk_rho_rime(w.qi_incld[k], w.qm_incld[k], w.bm_incld[k], rt);
            c.qm[k] = w.qm_incld[k] * c.cld_frac_i[k];
            c.bm[k] = w.bm_incld[k] * c.cld_frac_i[k];
            TableIce ti;
            lookup_ice(w.qi_incld[k], w.ni_incld[k], w.qm_incld[k], rhop, ti);
            const Real table_val_ni_fallspd = apply_table_ice(0, tab, ti);
            const Real table_val_qi_fallspd = apply_table_ice(1, tab, ti);
            const Real table_val_ni_lammax = apply_table_ice(6, tab, ti);
            const Real table_val_ni_lammin = apply_table_ice(7, tab, ti);
            w.ni_incld[k] = std::min(w.ni_incld[k], table_val_ni_lammax * w.ni_incld[k]);
            w.ni_incld[k] = std::max(w.ni_incld[k], table_val_ni_lammin * w.ni_incld[k]);
            c.ni[k] = w.ni_incld[k] * c.cld_frac_i[k];
            w.V1[k] = rt.ice_sedimentation_factor * table_val_qi_fallspd * w.rhofaci[k];
            w.V2[k] = rt.ice_sedimentation_factor * table_val_ni_fallspd * w.rhofaci[k];
            Co_max = std::max(Co_max, w.V1[k] * dt_left * inv_dz[k]);
          }
        }
        if (!(Co_max >= 0)) { e.bits |= P3O_ENUMERIC; break; }
        Real* fl[4] = {w.F1.data(), w.F2.data(), w.F3.data(), w.F4.data()};
        Real* vs[4] = {w.V1.data(), w.V2.data(), w.V1.data(), w.V1.data()};
        Real* rs[4] = {c.qi, c.ni, c.qm, c.bm};
        generalized_sedimentation(rho, inv_rho, inv_dz, k_qxtop, k_qxbot, kbot, kdir, Co_max, dt_left,
                                  prt_accum, 4, fl, vs, rs);
        for (int k = 0; k < nk; ++k) {
          w.qi_incld[k] = c.qi[k] / c.cld_frac_i[k];
          w.ni_incld[k] = c.ni[k] / c.cld_frac_i[k];
          w.qm_incld[k] = c.qm[k] / c.cld_frac_i[k];
          w.bm_incld[k] = c.bm[k] / c.cld_frac_i[k];
        }
      }
      *c.precip_ice_surf += prt_accum * C::INV_RHO_H2O * inv_dt;
    }
  }

  /* homogeneous_freezing: p3_ice_sed_impl.hpp:207-270 (T_atm from the start of the step) */
  if (do_ice_production) {
    for (int k = 0; k < nk; ++k) {
      const bool t_lt = w.T_atm[k] < C::T_homogfrz;
      const bool qc_ge = t_lt && c.qc[k] >= C::QSMALL;
      const bool qr_ge = t_lt && c.qr[k] >= C::QSMALL;
      const Real Qc_nuc = c.qc[k], Qr_nuc = c.qr[k];
      const Real Nc_nuc = std::max(c.nc[k], C::NSMALL), Nr_nuc = std::max(c.nr[k], C::NSMALL);
      if (qc_ge) {
        c.qm[k] = c.qm[k] + Qc_nuc;
        c.qi[k] = c.qi[k] + Qc_nuc;
        c.bm[k] = c.bm[k] + Qc_nuc * C::INV_RHO_RIMEMAX;
        c.ni[k] = c.ni[k] + Nc_nuc;
        c.th[k] = c.th[k] + c.inv_exner[k] * Qc_nuc * C::LatIce * C::INV_CP;
      }
      if (qr_ge) {
        c.qm[k] = c.qm[k] + Qr_nuc;
        c.qi[k] = c.qi[k] + Qr_nuc;
        c.bm[k] = c.bm[k] + Qr_nuc * C::INV_RHO_RIMEMAX;
        c.ni[k] = c.ni[k] + Nr_nuc;
        c.th[k] = c.th[k] + c.inv_exner[k] * Qr_nuc * C::LatIce * C::INV_CP;
      }
      if (qc_ge) { c.qc[k] = 0; c.nc[k] = 0; }
      if (qr_ge) { c.qr[k] = 0; c.nr[k] = 0; }
    }
  }

  /* p3_main_part3: p3_main_impl_part3.hpp:18-204 */
  for (int k = 0; k < nk; ++k) {
    /* cloud */
    {
      const bool qc_gt_small = c.qc[k] >= C::QSMALL;
      const Real qc_incld = c.qc[k] / c.cld_frac_l[k];
      Real nc_incld = c.nc[k] / c.cld_frac_l[k];
      if (qc_gt_small) {
        Real ig1, ig2;
        get_cloud_dsd2(qc_incld, nc_incld, w.mu_c[k], rho[k], w.nu[k], w.lamc[k], ig1, ig2);
        c.nc[k] = nc_incld * c.cld_frac_l[k];
        c.diag_eff_radius_qc[k] = 0.5 * (w.mu_c[k] + 3) / w.lamc[k];
      } else {
        c.qv[k] = c.qv[k] + c.qc[k];
        c.th[k] = c.th[k] - c.inv_exner[k] * c.qc[k] * C::LatVap * C::INV_CP;
        c.vap_liq_exchange[k] = c.vap_liq_exchange[k] - c.qc[k];
        c.qc[k] = 0;
        c.nc[k] = 0;
      }
    }
    /* rain */
    {
      const bool qr_gt_small = c.qr[k] >= C::QSMALL;
      const Real qr_incld = c.qr[k] / c.cld_frac_r[k];
      Real nr_incld = c.nr[k] / c.cld_frac_r[k];
      if (qr_gt_small) {
        get_rain_dsd2(qr_incld, nr_incld, w.mu_r[k], w.lamr[k], rt);
        c.nr[k] = nr_incld * c.cld_frac_r[k];
        c.diag_eff_radius_qr[k] = 1.5 / w.lamr[k];
      } else {
        c.qv[k] = c.qv[k] + c.qr[k];
        c.th[k] = c.th[k] - c.inv_exner[k] * c.qr[k] * C::LatVap * C::INV_CP;
        c.vap_liq_exchange[k] = c.vap_liq_exchange[k] - c.qr[k];
        c.qr[k] = 0;
        c.nr[k] = 0;
      }
    }
    /* ice */
    {
      const bool qi_gt_small = c.qi[k] >= C::QSMALL;
      c.ni[k] = std::max(c.ni[k], C::NSMALL);
      const Real qi_incld = c.qi[k] / c.cld_frac_i[k];
      Real ni_incld = c.ni[k] / c.cld_frac_i[k];
      Real qm_incld = c.qm[k] / c.cld_frac_i[k];
      Real bm_incld = c.bm[k] / c.cld_frac_i[k];
      Real rhop = 0;
      if (qi_gt_small) {
        rhop = calc_bulk_rho_rime(qi_incld, qm_incld, bm_incld, rt);
        c.qm[k] = qm_incld * c.cld_frac_i[k];
        c.bm[k] = bm_incld * c.cld_frac_i[k];
      }
      impose_max_total_ni(ni_incld, rt.max_total_ni, inv_rho[k]);
      Real table_val_ice_eff_radius = 0, table_val_ni_lammax = 0, table_val_ni_lammin = 0,
           table_val_ice_bulk_dens = 0;
      if (qi_gt_small) {
        TableIce ti;
        lookup_ice(qi_incld, ni_incld, qm_incld, rhop, ti);
        table_val_ice_eff_radius = apply_table_ice(5, tab, ti);
        table_val_ni_lammax = apply_table_ice(6, tab, ti);
        table_val_ni_lammin = apply_table_ice(7, tab, ti);
        table_val_ice_bulk_dens = apply_table_ice(11, tab, ti);
        ni_incld = std::min(ni_incld, table_val_ni_lammax * ni_incld);
        ni_incld = std::max(ni_incld, table_val_ni_lammin * ni_incld);
      }
      c.ni[k] = ni_incld * c.cld_frac_i[k];
      if (c.qm[k] < C::QSMALL && qi_gt_small) {
        c.qm[k] = 0;
        c.bm[k] = 0;
      }
      if (qi_gt_small) {
        c.diag_eff_radius_qi[k] = table_val_ice_eff_radius;
        c.rho_qi[k] = table_val_ice_bulk_dens;
      } else {
        c.qv[k] = c.qv[k] + c.qi[k];
        c.th[k] = c.th[k] - c.inv_exner[k] * c.qi[k] * (C::LatVap + C::LatIce) * C::INV_CP;
        c.qi[k] = 0;
        c.ni[k] = 0;
        c.qm[k] = 0;
        c.bm[k] = 0;
      }
    }
    if (c.qr[k] < C::QSMALL) c.nr[k] = 0;
  }
}

/* One column, in the stage order of p3_main_internal (p3_main_impl.hpp:108-325). */
void p3_column(const Col& c, int nk, Real dt, bool predictNc, bool prescribedCCN,
               const p3o_runtime& rt, const p3o_tables* tab, Work& w, Err& e) {
  if (p3_column_part12(c, nk, dt, predictNc, prescribedCCN, rt, tab, w, e))
    p3_column_sed_part3(c, nk, dt, predictNc, rt, tab, w, e);
}

/* Field pointers of column i. */
Col column_of(const p3o_fields* f, int i, int64_t ld, int64_t li) {
  Col c;
  const int64_t o = i * ld, oi = i * li;
  c.qc = f->qc + o; c.nc = f->nc + o; c.qr = f->qr + o; c.nr = f->nr + o;
  c.qi = f->qi + o; c.qm = f->qm + o; c.ni = f->ni + o; c.bm = f->bm + o;
  c.qv = f->qv + o; c.th = f->th + o;
  c.nc_nuceat_tend = f->nc_nuceat_tend + o; c.nccn = f->nccn + o;
  c.ni_activated = f->ni_activated + o; c.inv_qc_relvar = f->inv_qc_relvar + o;
  c.cld_frac_i = f->cld_frac_i + o; c.cld_frac_l = f->cld_frac_l + o;
  c.cld_frac_r = f->cld_frac_r + o; c.pres = f->pres + o; c.dz = f->dz + o;
  c.dpres = f->dpres + o; c.inv_exner = f->inv_exner + o; c.qv_prev = f->qv_prev + o;
  c.t_prev = f->t_prev + o;
  c.qv2qi_depos_tend = f->qv2qi_depos_tend + o;
  c.precip_liq_surf = f->precip_liq_surf + i; c.precip_ice_surf = f->precip_ice_surf + i;
  c.diag_eff_radius_qc = f->diag_eff_radius_qc + o; c.diag_eff_radius_qi = f->diag_eff_radius_qi + o;
  c.diag_eff_radius_qr = f->diag_eff_radius_qr + o; c.rho_qi = f->rho_qi + o;
  c.precip_liq_flux = f->precip_liq_flux + oi; c.precip_ice_flux = f->precip_ice_flux + oi;
  c.precip_total_tend = f->precip_total_tend + o; c.nevapr = f->nevapr + o;
  c.liq_ice_exchange = f->liq_ice_exchange + o; c.vap_liq_exchange = f->vap_liq_exchange + o;
  c.vap_ice_exchange = f->vap_ice_exchange + o;
  return c;
}

/* The hand-over rows of the staged entry points, [kHandover][ncol][ld]. */
enum { H_TATM = 0, H_RHO, H_RHOFACR, H_RHOFACI, H_ACN, kHandover };

}  // namespace

extern "C" {

void p3o_runtime_defaults(p3o_runtime* rt) {
  rt->max_total_ni = 740.0e3;
  rt->autoconversion_prefactor = 1350.0;
  rt->autoconversion_qc_exponent = 2.47;
  rt->autoconversion_nc_exponent = 1.79;
  rt->autoconversion_radius = 25.0e-6;
  rt->accretion_prefactor = 67.0;
  rt->accretion_qc_exponent = 1.15;
  rt->accretion_qr_exponent = 1.15;
  rt->rain_selfcollection_prefactor = 5.78;
  rt->rain_selfcollection_breakup_diameter = 0.00028;
  rt->constant_mu_rain = 1.0;
  rt->spa_ccn_to_nc_factor = 1.0;
  rt->cldliq_to_ice_collection_factor = 0.5;
  rt->rain_to_ice_collection_factor = 1.0;
  rt->min_rime_rho = 50.0;
  rt->max_rime_rho = 900.0;
  rt->immersion_freezing_exponent = 0.65;
  rt->deposition_nucleation_exponent = 0.304;
  rt->ice_sedimentation_factor = 1.0;
  rt->do_ice_production = 1;
  rt->pad_ = 0;
}

int p3o_main(const p3o_call* call, const p3o_runtime* rt, const p3o_tables* tab,
             const p3o_fields* f, double* elapsed_us) {
  const int ncol = call->ncol, nk = call->nlev;
  const int64_t ld = call->ld, li = call->ld_int;
  int err = 0;
  const auto t0 = std::chrono::steady_clock::now();
#ifdef _OPENMP
  const int nthr = call->nthreads > 0 ? call->nthreads : omp_get_max_threads();
#pragma omp parallel num_threads(nthr) reduction(| : err)
#endif
  {
    Work w;
    w.resize(nk);
    Err e;
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 16)
#endif
    for (int i = 0; i < ncol; ++i) {
      const Col c = column_of(f, i, ld, li);
      p3_column(c, nk, call->dt, call->predictNc != 0, call->prescribedCCN != 0, *rt, tab, w, e);
    }
    err |= e.bits;
  }
  const auto t1 = std::chrono::steady_clock::now();
  if (elapsed_us) *elapsed_us = std::chrono::duration<double, std::micro>(t1 - t0).count();
  return err;
}

int p3o_main_part12(const p3o_call* call, const p3o_runtime* rt, const p3o_tables* tab, const p3o_fields* f,
                    double* handover, int32_t* cflag) {
  const int ncol = call->ncol, nk = call->nlev;
  const int64_t ld = call->ld, li = call->ld_int;
  int err = 0;
#ifdef _OPENMP
  const int nthr = call->nthreads > 0 ? call->nthreads : omp_get_max_threads();
#pragma omp parallel num_threads(nthr) reduction(| : err)
#endif
  {
    Work w;
    w.resize(nk);
    Err e;
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 16)
#endif
    for (int i = 0; i < ncol; ++i) {
      const Col c = column_of(f, i, ld, li);
      const bool go_on = p3_column_part12(c, nk, call->dt, call->predictNc != 0, call->prescribedCCN != 0, *rt,
                                          tab, w, e);
      cflag[i] = go_on ? 1 : 0;
      if (!go_on) continue;
      const std::vector<Real>* rows[kHandover] = {&w.T_atm, &w.rho, &w.rhofacr, &w.rhofaci, &w.acn};
      for (int h = 0; h < kHandover; ++h) {
        double* dst = handover + (int64_t(h) * ncol + i) * ld;
        for (int k = 0; k < nk; ++k) dst[k] = (*rows[h])[k];
      }
    }
    err |= e.bits;
  }
  return err;
}

int p3o_main_sed_part3(const p3o_call* call, const p3o_runtime* rt, const p3o_tables* tab, const p3o_fields* f,
                       const double* handover, const int32_t* cflag) {
  const int ncol = call->ncol, nk = call->nlev;
  const int64_t ld = call->ld, li = call->ld_int;
  int err = 0;
#ifdef _OPENMP
  const int nthr = call->nthreads > 0 ? call->nthreads : omp_get_max_threads();
#pragma omp parallel num_threads(nthr) reduction(| : err)
#endif
  {
    Work w;
    w.resize(nk);
    Err e;
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 16)
#endif
    for (int i = 0; i < ncol; ++i) {
      if (!cflag[i]) continue;
      const Col c = column_of(f, i, ld, li);
      w.resize(nk); /* nothing of the previous column is carried over */
      std::vector<Real>* rows[kHandover] = {&w.T_atm, &w.rho, &w.rhofacr, &w.rhofaci, &w.acn};
      for (int h = 0; h < kHandover; ++h) {
        const double* src = handover + (int64_t(h) * ncol + i) * ld;
        for (int k = 0; k < nk; ++k) (*rows[h])[k] = src[k];
      }
      /* what part1 and part2 leave in the workspace for the later stages
       * (p3_main_impl_part1.hpp, p3_main_impl_part2.hpp:516-523): 1/rho,
       * 1/dz and the in-cloud values of the state */
      for (int k = 0; k < nk; ++k) {
        w.inv_rho[k] = 1 / w.rho[k];
        w.inv_dz[k] = 1 / c.dz[k];
        w.inv_cld_frac_l[k] = 1 / c.cld_frac_l[k];
        w.inv_cld_frac_i[k] = 1 / c.cld_frac_i[k];
        w.inv_cld_frac_r[k] = 1 / c.cld_frac_r[k];
        calculate_incloud_mixingratios(c.qc[k], c.qr[k], c.qi[k], c.qm[k], c.nc[k], c.nr[k], c.ni[k], c.bm[k],
                                       w.inv_cld_frac_l[k], w.inv_cld_frac_i[k], w.inv_cld_frac_r[k],
                                       w.qc_incld[k], w.qr_incld[k], w.qi_incld[k], w.qm_incld[k],
                                       w.nc_incld[k], w.nr_incld[k], w.ni_incld[k], w.bm_incld[k]);
      }
      p3_column_sed_part3(c, nk, call->dt, call->predictNc != 0, *rt, tab, w, e);
    }
    err |= e.bits;
  }
  return err;
}

void p3o_calc_first_order_upwind_step(int nk, int k_bot, int k_top, int kdir, double dt_sub,
                                      const double* rho, const double* inv_rho, const double* inv_dz,
                                      int nfield, double* const* flux, double* const* V,
                                      double* const* r) {
  (void)nk;
  upwind_step(rho, inv_rho, inv_dz, k_bot, k_top, kdir, dt_sub, nfield, flux, V, r);
}

int p3o_find_top(const double* v, double small, int kbot, int ktop, int kdir, int* present) {
  bool p;
  const int k = find_top(v, small, kbot, ktop, kdir, p);
  *present = p ? 1 : 0;
  return k;
}

int p3o_find_bottom(const double* v, double small, int kbot, int ktop, int kdir, int* present) {
  bool p;
  const int k = find_bottom(v, small, kbot, ktop, kdir, p);
  *present = p ? 1 : 0;
  return k;
}

void p3o_table3_lookup_apply(const p3o_tables* tab, int which, int n, const double* mu_r,
                             const double* lamr, double* out) {
  const double* t = which == 0 ? tab->vn : (which == 1 ? tab->vm : tab->revap);
  for (int i = 0; i < n; ++i) {
    Table3 t3;
    lookup3(mu_r[i], lamr[i], t3);
    out[i] = apply_table3(t, t3);
  }
}

/* tend8 = {qc2qr_autoconv, qc2qr_accret, qc2qi_collect, qc2qi_hetero_freeze,
 *          qc2qr_ice_shed, qc2qi_berg, qi2qv_sublim, qv2qi_vapdep} */
void p3o_cloud_water_conservation(double qc, double dt, double* t) {
  cloud_water_conservation(qc, dt, t[0], t[1], t[2], t[3], t[4], t[5], t[6], t[7]);
}
/* tend7 = {qc2qr_autoconv, qc2qr_accret, qi2qr_melt, qc2qr_ice_shed,
 *          qr2qv_evap, qr2qi_collect, qr2qi_immers_freeze} */
void p3o_rain_water_conservation(double qr, double dt, double* t) {
  rain_water_conservation(qr, t[0], t[1], t[2], t[3], dt, t[4], t[5], t[6]);
}
/* tend9 = {qv2qi_vapdep, qv2qi_nucleat, qc2qi_berg, qr2qi_collect, qc2qi_collect,
 *          qr2qi_immers_freeze, qc2qi_hetero_freeze, qi2qv_sublim, qi2qr_melt} */
void p3o_ice_water_conservation(double qi, double dt, double* t) {
  ice_water_conservation(qi, t[0], t[1], t[2], t[3], t[4], t[5], t[6], dt, t[7], t[8]);
}

double p3o_qv_sat_dry(double t, double p, int ice) {
  Err e;
  return qv_sat_dry(t, p, ice != 0, e);
}

}  // extern "C"
