/*
 * P3 lookup-table pipeline (host C++, shared by every precision form).
 *
 * - Rain tables vn / vm / revap [300][10] and mu_r [150]: numerical
 *   quadrature over a 10,000-bin gamma PSD, restating the Fortran p3_init_b
 *   (components/eam/src/physics/p3/scream/micro_p3.F90:218-341) with
 *   mu_r = 1 (micro_p3_utils.F90:33).
 * - dnu [16]: the literal table of p3/impl/p3_table3_impl.hpp:120-135.
 * - Ice table [5][4][50][12] and ice-rain collection table [5][4][50][30][2]:
 *   restating the offline generator
 *   components/eam/tools/create_p3_lookupTable/create_p3_lookupTable_1.f90-v4.1
 *   (v4.1): lambda search on a 9000-point grid (:504-600), lambda-limiter
 *   bounds (:648-690), fall-speed / reflectivity / mean-size / density moments
 *   (:731-808), self-aggregation (:809-928), droplet collection (:929-1009),
 *   rain collection (:1010-1205), deposition / ventilation (:1207-1279) and
 *   effective radius (:1281-1356).  The regularised upper incomplete gamma
 *   function Q(a,x) is evaluated with the series of Abramowitz & Stegun
 *   6.5.29 for x < a+1 and otherwise with Legendre's continued fraction
 *   (A&S 6.5.31) summed by the modified Lentz method (Lentz 1976; Thompson &
 *   Barnett 1986).  The generator's own constants are kept (pi = 3.14159,
 *   g = 9.861, 600 hPa / 253.15 K reference air, mu_r = 0 for rain).  Its
 *   particle-2 area quirk in the aggregation loop (the mass interpolation
 *   fraction is taken at particle 1's diameter, :872-884) is kept too.
 *   Sums that the generator evaluates as 1000 x 1000 double loops are
 *   factored into per-bin partial sums; this reorders floating-point
 *   additions only.
 * - Text format: the official "p3_lookup_table_1.dat-v4.1.1" layout read by
 *   p3/impl/p3_table_ice_impl.hpp:33-71 (a "VERSION x.y.z" header, then per
 *   (rime density, rime fraction) 50 rows of 2 ints + 15 reals followed by
 *   1500 rows of 2 ints + 6 reals).  Generated values are rounded to the
 *   generator's e15.5 output precision so that the in-memory tables equal a
 *   write/read round trip, and a real v4.1.1 file can be dropped in instead.
 */
#include "p3x_internal.hpp"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace p3x {

namespace {

constexpr int n_rhor = 5, n_Fr = 4, n_Qnorm = 50, n_Drscale = 30;
constexpr int kIceRawCols = 15, kCollRawCols = 6;

/* ------------------------------------------------------------------ */
/* Regularised upper incomplete gamma Q(a, x)                          */
/* ------------------------------------------------------------------ */
double inc_gamma_upper_reg(double a, double x) {
  if (!(x > 0.0)) return 1.0;
  const double log_pref = -x + a * std::log(x) - std::log(std::tgamma(a));
  if (x < a + 1.0) {
    /* P(a,x) = x^a e^-x / Gamma(a+1) * sum_n x^n / ((a+1)...(a+n)) */
    double term = 1.0 / a, sum = term;
    for (int n = 1; n < 100000; ++n) {
      term *= x / (a + n);
      sum += term;
      if (std::fabs(term) < std::fabs(sum) * 1e-16) break;
    }
    const double P = std::exp(log_pref) * sum;
    return 1.0 - P;
  }
  /* Gamma(a,x) e^x x^-a = 1/(b0 + a1/(b1 + a2/(b2 + ...))),
   * b_n = x + 2n + 1 - a, a_n = -n (n - a).  Modified Lentz. */
  const double tiny = 1e-300;
  double f = x + 1.0 - a;
  if (f == 0.0) f = tiny;
  double Cc = f, D = 0.0;
  for (int n = 1; n < 100000; ++n) {
    const double an = -n * (n - a);
    const double bn = x + 2.0 * n + 1.0 - a;
    D = bn + an * D;
    if (D == 0.0) D = tiny;
    Cc = bn + an / Cc;
    if (Cc == 0.0) Cc = tiny;
    D = 1.0 / D;
    const double delta = Cc * D;
    f *= delta;
    if (std::fabs(delta - 1.0) < 1e-16) break;
  }
  return std::exp(log_pref) / f;
}

/* Round to the generator's e15.5 output precision (5 significant digits). */
double round_e155(double v) {
  if (v == 0.0 || !std::isfinite(v)) return v;
  char buf[64];
  std::snprintf(buf, sizeof buf, "%.4e", v);
  return std::strtod(buf, nullptr);
}

/* Generator constants, create_p3_lookupTable_1.f90-v4.1:55-160 */
struct Gen {
  double pi = 3.14159, g = 9.861, p = 60000., t = 253.15;
  double rho, mu, c0 = 0.6, del0 = 5.83, c1, c2;
  double ds = 1.9, cs = 0.0121, dg = 3., bas = 1.88, aas, bag = 2., aag, dcrit;
  double thrd = 1. / 3., sxth = 1. / 6.;
  double Dm_max = 2000.e-6, Dm_min = 2.e-6;
  double mu_r_gen = 0.;
  Gen() {
    rho = p / (287.15 * t);
    mu = 1.496E-6 * std::pow(t, 1.5) / (t + 120.) / rho;
    c1 = 4. / (del0 * del0 * std::pow(c0, 0.5));
    c2 = del0 * del0 / 4.;
    aas = 0.2285 * std::pow(100., bas) / (100. * 100.);
    aag = pi * 0.25;
    dcrit = std::pow(pi / (6. * cs) * 900., 1. / (ds - 3.));
  }
};

/* Per (rime density, rime fraction) regime of the mass- and area-size
 * relations, :250-314 (partial-riming iteration for the critical sizes). */
struct Regime {
  double Fr, cgp, dcrits, dcritr, csr, dsr;
  bool unrimed;  /* i_Fr == 1 */
};

Regime make_regime(const Gen& G, int i_rhor, int i_Fr) {
  static const double rime_rho[n_rhor] = {50., 250., 450., 650., 900.};
  static const double Fr_vals[n_Fr] = {0., 0.333, 0.667, 1.};
  Regime R;
  R.Fr = Fr_vals[i_Fr];
  const double crp = rime_rho[i_rhor] * G.pi * G.sxth;
  R.cgp = crp;
  R.unrimed = (i_Fr == 0);
  if (i_Fr == 0) {
    R.dcrits = 1.e+6;
    R.dcritr = R.dcrits;
    R.csr = G.cs;
    R.dsr = G.ds;
  } else if (i_Fr == 1 || i_Fr == 2) {
    for (int it = 0; it < 10000; ++it) {
      R.dcrits = std::pow(G.cs / R.cgp, 1. / (G.dg - G.ds));
      R.dcritr = std::pow((1. + R.Fr / (1. - R.Fr)) * G.cs / R.cgp, 1. / (G.dg - G.ds));
      R.csr = G.cs * (1. + R.Fr / (1. - R.Fr));
      R.dsr = G.ds;
      const double rhodep = 1. / (R.dcritr - R.dcrits) * 6. * G.cs / (G.pi * (G.ds - 2.)) *
                            (std::pow(R.dcritr, G.ds - 2.) - std::pow(R.dcrits, G.ds - 2.));
      const double cgpold = R.cgp;
      R.cgp = crp * R.Fr + rhodep * (1. - R.Fr) * G.pi * G.sxth;
      if (std::fabs((R.cgp - cgpold) / R.cgp) < 0.01) break;
    }
  } else {
    R.dcrits = std::pow(G.cs / R.cgp, 1. / (G.dg - G.ds));
    R.dcritr = 1.e+6;
    R.csr = R.cgp;
    R.dsr = G.dg;
  }
  return R;
}

/* Mass (cs1, ds1) and projected area (aas1, bas1) at diameter d, :333-370. */
struct MA {
  double cs1, ds1, aas1, bas1;
};
MA mass_area(const Gen& G, const Regime& R, double d) {
  MA m;
  if (d <= G.dcrit) {
    m.cs1 = G.pi * G.sxth * 900.;
    m.ds1 = 3.;
    m.bas1 = 2.;
    m.aas1 = G.pi / 4.;
  } else if (d <= R.dcrits) {
    m.cs1 = G.cs;
    m.ds1 = G.ds;
    m.bas1 = G.bas;
    m.aas1 = G.aas;
  } else if (d <= R.dcritr) {
    m.cs1 = R.cgp;
    m.ds1 = G.dg;
    m.bas1 = G.bag;
    m.aas1 = G.aag;
  } else {
    m.cs1 = R.csr;
    m.ds1 = R.dsr;
    if (R.unrimed) {
      m.aas1 = G.aas;
      m.bas1 = G.bas;
    } else {
      m.bas1 = G.bas;
      const double dum1 = G.aas * std::pow(d, G.bas);
      const double dum2 = G.aag * std::pow(d, G.bag);
      const double m1 = m.cs1 * std::pow(d, m.ds1);
      const double m2 = G.cs * std::pow(d, G.ds);
      const double m3 = R.cgp * std::pow(d, G.dg);
      const double dum3 = dum1 + (m1 - m2) * (dum2 - dum1) / (m3 - m2);
      m.aas1 = dum3 / std::pow(d, G.bas);
    }
  }
  return m;
}

/* Mitchell & Heymsfield (2005) fall speed, :372-392 (turbulence terms a0 = b0 = 0). */
double fall_speed(const Gen& G, const MA& m, double d) {
  const double xx = 2. * m.cs1 * G.g * G.rho * std::pow(d, m.ds1 + 2. - m.bas1) /
                    (m.aas1 * (G.mu * G.rho) * (G.mu * G.rho));
  const double sx = std::pow(xx, 0.5);
  const double q = std::pow(1. + G.c1 * sx, 0.5);
  const double b1 = G.c1 * sx / (2. * (q - 1.) * q);
  const double a1 = (G.c2 * (q - 1.) * (q - 1.)) / std::pow(xx, b1);
  return a1 * std::pow(G.mu, 1. - 2. * b1) * std::pow(2. * m.cs1 * G.g / (G.rho * m.aas1), b1) *
         std::pow(d, b1 * (m.ds1 - m.bas1 + 2.) - 1.);
}

/* Rain drop fall speed for the collection integrals, :440-466. */
double rain_fall_speed(const Gen& G, double dia) {
  double amg = G.pi * G.sxth * 997. * dia * dia * dia;
  amg = amg * 1000.;
  double dum2;
  if (dia <= 134.43e-6) {
    dum2 = 4.5795e5 * std::pow(amg, 2. * G.thrd);
  } else if (dia < 1511.64e-6) {
    dum2 = 4.962e3 * std::pow(amg, G.thrd);
  } else if (dia < 3477.84e-6) {
    dum2 = 1.732e3 * std::pow(amg, G.sxth);
  } else {
    dum2 = 917.;
  }
  return dum2 * 1.e-2;
}

double mu_of_lam(double lam) {
  double mu_i = 0.076 * std::pow(lam / 100., 0.8) - 2.;
  mu_i = std::max(mu_i, 0.);
  mu_i = std::min(mu_i, 6.);
  return mu_i;
}

/* Mass integral over the four PSD regions divided by n0, :576-596. */
double mass_moment(const Gen& G, const Regime& R, double lam, double mu_i, bool clip) {
  const double cs1 = G.pi * G.sxth * 900., ds1 = 3.;
  const double dum1 = std::pow(lam, -ds1 - mu_i - 1.) * std::tgamma(mu_i + ds1 + 1.) *
                      (1. - inc_gamma_upper_reg(mu_i + ds1 + 1., G.dcrit * lam));
  double dum2 = std::pow(lam, -G.ds - mu_i - 1.) * std::tgamma(mu_i + G.ds + 1.) *
                inc_gamma_upper_reg(mu_i + G.ds + 1., G.dcrit * lam);
  double dum = std::pow(lam, -G.ds - mu_i - 1.) * std::tgamma(mu_i + G.ds + 1.) *
               inc_gamma_upper_reg(mu_i + G.ds + 1., R.dcrits * lam);
  dum2 = dum2 - dum;
  if (clip) dum2 = std::max(dum2, 0.);
  double dum3 = std::pow(lam, -G.dg - mu_i - 1.) * std::tgamma(mu_i + G.dg + 1.) *
                inc_gamma_upper_reg(mu_i + G.dg + 1., R.dcrits * lam);
  dum = std::pow(lam, -G.dg - mu_i - 1.) * std::tgamma(mu_i + G.dg + 1.) *
        inc_gamma_upper_reg(mu_i + G.dg + 1., R.dcritr * lam);
  dum3 = dum3 - dum;
  if (clip) dum3 = std::max(dum3, 0.);
  const double dum4 = std::pow(lam, -R.dsr - mu_i - 1.) * std::tgamma(mu_i + R.dsr + 1.) *
                      inc_gamma_upper_reg(mu_i + R.dsr + 1., R.dcritr * lam);
  return cs1 * dum1 + G.cs * dum2 + R.cgp * dum3 + R.csr * dum4;
}

/* One (rime density, rime fraction) slab of the raw generator output. */
void generate_slab(const Gen& G, int i_rhor, int i_Fr, double* ice_raw /* [50][15] */,
                   double* coll_raw /* [50][30][6] */) {
  const Regime R = make_regime(G, i_rhor, i_Fr);

  /* fall1 on the 2-um grid, fall2 / fallr on the 20-um grid (:320-470) */
  std::vector<double> fall1(10000), fall2(1000), fallr(1000);
  for (int jj = 1; jj <= 10000; ++jj) {
    const double d1 = double(jj) * 2. * 1.e-6 - 1.e-6;
    fall1[jj - 1] = fall_speed(G, mass_area(G, R, d1), d1);
  }
  for (int jj = 1; jj <= 1000; ++jj) {
    const double d1 = double(jj) * 20. * 1.e-6 - 10.e-6;
    fall2[jj - 1] = fall_speed(G, mass_area(G, R, d1), d1);
    fallr[jj - 1] = rain_fall_speed(G, d1);
  }

  /* lambda search table: mass moment for each of the 9000 candidate lambdas
   * (independent of the normalised mass being matched) */
  std::vector<double> lam_grid(9000), qn_grid(9000);
  for (int ii = 1; ii <= 9000; ++ii) {
    double lam = std::pow(1.0013, ii) * 100.;
    const double mu_i = mu_of_lam(lam);
    lam = std::max(lam, (mu_i + 1.) / G.Dm_max);
    lam = std::min(lam, (mu_i + 1.) / G.Dm_min);
    const double n0 = std::pow(lam, mu_i + 1.) / std::tgamma(mu_i + 1.);
    lam_grid[ii - 1] = lam;
    qn_grid[ii - 1] = n0 * mass_moment(G, R, lam, mu_i, true);
  }

  /* 20-um grid geometry that does not depend on the PSD */
  std::vector<double> d20(1000), area20(1000), mass20(1000);
  for (int jj = 1; jj <= 1000; ++jj) {
    const double d1 = double(jj) * 20. * 1.e-6 - 10.e-6;
    MA m = mass_area(G, R, d1);
    if (d1 <= G.dcrit) m.aas1 = G.pi * 0.25;
    d20[jj - 1] = d1;
    area20[jj - 1] = m.aas1 * std::pow(d1, m.bas1);
    mass20[jj - 1] = m.cs1 * std::pow(d1, m.ds1);
  }

  /* Rain-collection kernels per rain size class (:1010-1205), factored:
   * sum_k (A_j + B_k) |F2_j - FR_k| w_k = A_j G0_j + G1_j. */
  std::vector<double> G0(n_Drscale * 1000), G1(n_Drscale * 1000), H0(n_Drscale * 1000),
      H1(n_Drscale * 1000), lamrs(n_Drscale);
  for (int i_Dr = 1; i_Dr <= n_Drscale; ++i_Dr) {
    const double dum = std::pow(1.24, i_Dr) * 10.e-6;
    const double lamv = 1. / dum;
    lamrs[i_Dr - 1] = lamv;
    const double mu_r = G.mu_r_gen;
    double lamr = lamv * std::pow(std::tgamma(mu_r + 4.) / (6. * std::tgamma(mu_r + 1.)), G.thrd);
    const double lammax = (mu_r + 1.) * 1.e+5;
    const double lammin = (mu_r + 1.) * 200.;
    lamr = std::min(lamr, lammax);
    lamr = std::max(lamr, lammin);
    const double dd = 20.e-6;
    std::vector<double> num(1000), B(1000), M(1000);
    for (int kk = 0; kk < 1000; ++kk) {
      const double d2 = d20[kk];
      num[kk] = std::pow(d2, mu_r) * std::exp(-lamr * d2) * dd;
      B[kk] = G.pi * 0.25 * d2 * d2;
      M[kk] = G.pi * G.sxth * 997. * d2 * d2 * d2;
    }
    for (int jj = 0; jj < 1000; ++jj) {
      double g0 = 0, g1 = 0, h0 = 0, h1 = 0;
      const double f2 = fall2[jj];
      for (int kk = 0; kk < 1000; ++kk) {
        const double w = std::fabs(f2 - fallr[kk]) * num[kk];
        g0 += w;
        g1 += B[kk] * w;
        h0 += w * M[kk];
        h1 += B[kk] * w * M[kk];
      }
      G0[(i_Dr - 1) * 1000 + jj] = g0;
      G1[(i_Dr - 1) * 1000 + jj] = g1;
      H0[(i_Dr - 1) * 1000 + jj] = h0;
      H1[(i_Dr - 1) * 1000 + jj] = h1;
    }
  }

  /* particle-2 area in the aggregation loop (:850-886): the standard rule,
   * except above dcritr where the mass interpolation fraction is evaluated
   * at particle 1's diameter (generator quirk kept). */
  std::vector<double> frac_d1(1000, 0.0), a_d(1000), b_d(1000), powbas(1000);
  for (int jj = 0; jj < 1000; ++jj) {
    const double d = d20[jj];
    a_d[jj] = G.aas * std::pow(d, G.bas);
    b_d[jj] = G.aag * std::pow(d, G.bag);
    powbas[jj] = std::pow(d, G.bas);
    const double m1 = R.csr * std::pow(d, R.dsr);
    const double m2 = G.cs * std::pow(d, G.ds);
    const double m3 = R.cgp * std::pow(d, G.dg);
    frac_d1[jj] = (m1 - m2) / (m3 - m2);
    (void)frac_d1;
  }
  std::vector<double> m1d(1000), m2d(1000), m3d(1000);
  for (int jj = 0; jj < 1000; ++jj) {
    const double d = d20[jj];
    m1d[jj] = R.csr * std::pow(d, R.dsr);
    m2d[jj] = G.cs * std::pow(d, G.ds);
    m3d[jj] = R.cgp * std::pow(d, G.dg);
  }

  for (int i_Q = 1; i_Q <= n_Qnorm; ++i_Q) {
    const double q = std::pow(261.7, (i_Q + 10) * 0.1) * 1.e-18;

    /* lambda with the smallest |q - qdum| (first minimum wins), :504-560 */
    double qerror = std::fabs(q - qn_grid[0]);
    double lamf = lam_grid[0];
    for (int ii = 1; ii < 9000; ++ii) {
      const double e = std::fabs(q - qn_grid[ii]);
      if (e < qerror) {
        lamf = lam_grid[ii];
        qerror = e;
      }
    }
    const double lam = lamf;
    const double mu_i = mu_of_lam(lam);
    const double n0 = q / mass_moment(G, R, lam, mu_i, false);

    /* lambda-limiter normalised number bounds, :648-690 */
    double duml = (mu_i + 1.) / G.Dm_min;
    double n0dum = q / mass_moment(G, R, duml, mu_i, false);
    const double nlarge = n0dum / (std::pow(duml, mu_i + 1.) / std::tgamma(mu_i + 1.));
    duml = (mu_i + 1.) / G.Dm_max;
    n0dum = q / mass_moment(G, R, duml, mu_i, false);
    const double nsmall = n0dum / (std::pow(duml, mu_i + 1.) / std::tgamma(mu_i + 1.));

    /* moments on the 2-um grid, :731-808; droplet collection :929-1009;
     * deposition :1207-1279; effective radius :1281-1356 */
    double sum1 = 0, sum2 = 0, sum3 = 0, sum4 = 0, sum5 = 0, sum6 = 0, sum7 = 0;
    double nrwat = 0, vdep = 0, vdep1 = 0, eff1 = 0, eff2 = 0;
    {
      const double dd = 2.e-6;
      for (int ii = 1; ii <= 10000; ++ii) {
        const double dum = double(ii) * dd - 1.e-6;
        const double d1 = double(ii) * 2. * 1.e-6 - 1.e-6;
        MA m = mass_area(G, R, dum);
        const double e = std::exp(-lam * dum);
        const double f1 = fall1[ii - 1];
        sum1 += f1 * std::pow(dum, mu_i) * e * dd;
        sum2 += f1 * m.cs1 * std::pow(dum, m.ds1 + mu_i) * e * dd;
        sum3 += std::pow(dum, mu_i) * e * dd;
        sum4 += m.cs1 * std::pow(dum, m.ds1 + mu_i) * e * dd;
        sum5 += n0 * (m.cs1 / 917.) * (m.cs1 / 917.) * (6. / G.pi) * (6. / G.pi) *
                std::pow(dum, 2. * m.ds1 + mu_i) * e * dd;
        sum6 += m.cs1 * std::pow(dum, m.ds1 + mu_i + 1.) * e * dd;
        sum7 += (m.cs1 * std::pow(dum, m.ds1)) * (m.cs1 * std::pow(dum, m.ds1)) /
                (G.pi * G.sxth * dum * dum * dum) * std::pow(dum, mu_i) * e * dd;

        MA ma = mass_area(G, R, d1);
        if (d1 <= G.dcrit) ma.aas1 = G.pi * 0.25;
        const double e1 = std::exp(-lam * d1);
        if (d1 >= 100.e-6) {
          nrwat += ma.aas1 * std::pow(d1, ma.bas1) * f1 * n0 * std::pow(d1, mu_i) * e1 * dd;
        }
        double cap;
        if (d1 <= G.dcrit) {
          cap = 1.;
        } else if (d1 <= R.dcrits) {
          cap = 0.48;
        } else if (d1 <= R.dcritr) {
          cap = 1.;
        } else {
          if (R.unrimed) {
            cap = 0.48;
          } else {
            const double m1 = R.csr * std::pow(d1, R.dsr);
            const double m2 = G.cs * std::pow(d1, G.ds);
            const double m3 = R.cgp * std::pow(d1, G.dg);
            cap = 0.48 + (m1 - m2) * (1. - 0.48) / (m3 - m2);
          }
        }
        const double vent = std::pow(f1 * d1, 0.5);
        const double pw = std::pow(d1, mu_i + 1.) * e1 * dd;
        if (d1 < 100.e-6) {
          vdep += cap * n0 * pw;
        } else {
          vdep += cap * n0 * 0.65 * pw;
          vdep1 += cap * n0 * 0.44 * vent * pw;
        }
        eff1 += ma.cs1 * std::pow(d1, ma.ds1) * std::pow(d1, mu_i) * e1 * dd;
        eff2 += ma.aas1 * std::pow(d1, ma.bas1) * std::pow(d1, mu_i) * e1 * dd;
      }
    }

    /* self-aggregation, :809-928 */
    double nagg = 0;
    {
      const double dd = 20.e-6;
      std::vector<double> num(1000);
      for (int jj = 1000; jj >= 1; --jj) {
        const double d1 = double(jj) * dd - 10.e-6;
        num[jj - 1] = n0 * std::pow(d1, mu_i) * std::exp(-lam * d1) * dd;
      }
      for (int jj = 1000; jj >= 1; --jj) {
        const double A1 = area20[jj - 1];
        const double d1 = d20[jj - 1];
        const bool p1_above = d1 > R.dcritr;
        for (int kk = 1; kk <= jj - 1; ++kk) {
          const double d2 = d20[kk - 1];
          double A2;
          if (d2 > R.dcritr && !R.unrimed && p1_above) {
            const double dum1 = a_d[kk - 1], dum2 = b_d[kk - 1];
            const double dum3 = dum1 + (m1d[jj - 1] - m2d[jj - 1]) * (dum2 - dum1) / (m3d[jj - 1] - m2d[jj - 1]);
            A2 = (dum3 / powbas[kk - 1]) * std::pow(d2, G.bas);
          } else {
            A2 = area20[kk - 1];
          }
          const double delu = std::fabs(fall2[jj - 1] - fall2[kk - 1]);
          nagg += (A1 + A2) * delu * num[jj - 1] * num[kk - 1];
        }
      }
    }

    /* ice-rain collection, :1010-1205 (factored double sum) */
    for (int i_Dr = 0; i_Dr < n_Drscale; ++i_Dr) {
      double s1 = 0, s2 = 0, s6 = 0;
      const double dd = 20.e-6;
      for (int jj = 0; jj < 1000; ++jj) {
        const double d1 = d20[jj];
        const double X = n0 * std::pow(d1, mu_i) * std::exp(-lam * d1) * dd;
        const double A = area20[jj];
        const double g0 = G0[i_Dr * 1000 + jj], g1 = G1[i_Dr * 1000 + jj];
        s1 += X * (A * g0 + g1);
        s2 += X * (A * H0[i_Dr * 1000 + jj] + H1[i_Dr * 1000 + jj]);
        s6 += X * mass20[jj] * (A * g0 + g1);
      }
      double* row = coll_raw + ((i_Q - 1) * n_Drscale + i_Dr) * kCollRawCols;
      row[0] = q;
      row[1] = 1.;
      row[2] = lamrs[i_Dr];
      row[3] = s1;
      row[4] = s2;
      row[5] = s6;
    }

    double* row = ice_raw + (i_Q - 1) * kIceRawCols;
    row[0] = q;            /* qsave  */
    row[1] = 1.;           /* nsave  */
    row[2] = sum1 / sum3;  /* uns    */
    row[3] = sum2 / sum4;  /* ums    */
    row[4] = nagg;         /* nagg   */
    row[5] = nrwat;        /* nrwat  */
    row[6] = vdep;         /* vdep   */
    row[7] = 3. * eff1 / (4. * eff2 * 916.7); /* eff */
    row[8] = nlarge;       /* nlarge */
    row[9] = nsmall;       /* nsmall */
    row[10] = lam;         /* lsave  */
    row[11] = sum5;        /* refl   */
    row[12] = vdep1;       /* vdep1  */
    row[13] = sum6 / sum4; /* dmm    */
    row[14] = sum7 / sum4; /* rhomm  */
  }
}

void finish_raw(std::vector<double>& v) {
  for (auto& x : v) {
    if (x < 1.e-99) x = 0.;
    x = round_e155(x);
  }
}

/* raw generator rows -> P3 tables (p3_table_ice_impl.hpp:46-67) */
void select_tables(const std::vector<double>& ice_raw, const std::vector<double>& coll_raw,
                   HostTables& T) {
  T.ice.assign(size_t(n_rhor) * n_Fr * n_Qnorm * kIceCols, 0.0);
  T.collect.assign(size_t(n_rhor) * n_Fr * n_Qnorm * n_Drscale * kCollCols, 0.0);
  for (int s = 0; s < n_rhor * n_Fr; ++s) {
    for (int i = 0; i < n_Qnorm; ++i) {
      const double* r = &ice_raw[(size_t(s) * n_Qnorm + i) * kIceRawCols];
      int j_idx = 0;
      for (int j = 0; j < kIceRawCols; ++j) {
        if (j > 1 && j != 10) T.ice[(size_t(s) * n_Qnorm + i) * kIceCols + j_idx++] = r[j];
      }
      for (int j = 0; j < n_Drscale; ++j) {
        const double* c = &coll_raw[((size_t(s) * n_Qnorm + i) * n_Drscale + j) * kCollRawCols];
        T.collect[((size_t(s) * n_Qnorm + i) * n_Drscale + j) * kCollCols + 0] = std::log10(c[3]);
        T.collect[((size_t(s) * n_Qnorm + i) * n_Drscale + j) * kCollCols + 1] = std::log10(c[4]);
      }
    }
  }
}

}  // namespace

double incomplete_gamma_q(double a, double x) { return inc_gamma_upper_reg(a, x); }

/* p3_init_b restatement (micro_p3.F90:218-341). */
void build_rain_tables(HostTables& T, double mu_r_constant) {
  const double pi = 3.14159265358979323, sxth = 1. / 6., thrd = 1. / 3.;
  const double piov6 = pi * sxth;
  T.mu_r.assign(kMuRDim, mu_r_constant);
  T.vn.assign(size_t(kVT0) * kVT1, 0.0);
  T.vm.assign(size_t(kVT0) * kVT1, 0.0);
  T.revap.assign(size_t(kVT0) * kVT1, 0.0);
  std::vector<double> vn1(kVT0), vm1(kVT0), re1(kVT0);
  const double mu_r = mu_r_constant; /* the same for all 10 mu columns */
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 4)
#endif
  for (int jj = 1; jj <= kVT0; ++jj) {
    double dm;
    if (jj <= 20) {
      dm = (double(jj) * 10. - 5.) * 1.e-6;
    } else {
      dm = (double(jj - 20) * 30. + 195.) * 1.e-6;
    }
    const double lamr = (mu_r + 1.) / dm;
    double dum1 = 0, dum2 = 0, dum3 = 0, dum4 = 0, dum5 = 0;
    const double dd = 2.;
    for (int kk = 1; kk <= 10000; ++kk) {
      const double dia = (double(kk) * dd - dd * 0.5) * 1.e-6;
      double amg = piov6 * 997. * std::pow(dia, 3.);
      amg = amg * 1000.;
      double vt;
      if (dia * 1.e+6 <= 134.43) {
        vt = 4.5795e+3 * std::pow(amg, 2. * thrd);
      } else if (dia * 1.e+6 < 1511.64) {
        vt = 4.962e+1 * std::pow(amg, thrd);
      } else if (dia * 1.e+6 < 3477.84) {
        vt = 1.732e+1 * std::pow(amg, sxth);
      } else {
        vt = 9.17;
      }
      const double e = std::exp(-lamr * dia);
      const double w0 = std::pow(10., mu_r * std::log10(dia) + 4. * mu_r) * e * dd * 1.e-6;
      const double w3 = std::pow(10., (mu_r + 3.) * std::log10(dia) + 4. * mu_r) * e * dd * 1.e-6;
      dum1 += vt * w0;
      dum2 += w0;
      dum3 += vt * w3;
      dum4 += w3;
      dum5 += std::pow(vt * dia, 0.5) * std::pow(10., (mu_r + 1.) * std::log10(dia) + 3. * mu_r) * e * dd * 1.e-6;
    }
    dum2 = std::max(dum2, 1.e-30);
    dum4 = std::max(dum4, 1.e-30);
    dum5 = std::max(dum5, 1.e-30);
    vn1[jj - 1] = dum1 / dum2;
    vm1[jj - 1] = dum3 / dum4;
    re1[jj - 1] = std::pow(10., std::log10(dum5) + (mu_r + 1.) * std::log10(lamr) - (3. * mu_r));
  }
  for (int jj = 0; jj < kVT0; ++jj) {
    for (int ii = 0; ii < kVT1; ++ii) {
      T.vn[size_t(jj) * kVT1 + ii] = vn1[jj];
      T.vm[size_t(jj) * kVT1 + ii] = vm1[jj];
      T.revap[size_t(jj) * kVT1 + ii] = re1[jj];
    }
  }
  /* p3_table3_impl.hpp:120-135 */
  static const double dnu[kDnuDim] = {0.000,  -0.557, -0.430, -0.307, -0.186, -0.067,
                                      -0.050, -0.167, -0.282, -0.397, -0.512, -0.626,
                                      -0.739, -0.853, -0.966, -0.966};
  T.dnu.assign(dnu, dnu + kDnuDim);
}

int generate_ice_raw(std::vector<double>& ice_raw, std::vector<double>& coll_raw) {
  const Gen G;
  ice_raw.assign(size_t(n_rhor) * n_Fr * n_Qnorm * kIceRawCols, 0.0);
  coll_raw.assign(size_t(n_rhor) * n_Fr * n_Qnorm * n_Drscale * kCollRawCols, 0.0);
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1)
#endif
  for (int s = 0; s < n_rhor * n_Fr; ++s) {
    const int i_rhor = s / n_Fr, i_Fr = s % n_Fr;
    generate_slab(G, i_rhor, i_Fr, &ice_raw[size_t(s) * n_Qnorm * kIceRawCols],
                  &coll_raw[size_t(s) * n_Qnorm * n_Drscale * kCollRawCols]);
  }
  finish_raw(ice_raw);
  finish_raw(coll_raw);
  return 0;
}

int build_ice_tables(HostTables& T) {
  std::vector<double> ice_raw, coll_raw;
  const int rc = generate_ice_raw(ice_raw, coll_raw);
  if (rc) return rc;
  select_tables(ice_raw, coll_raw, T);
  return 0;
}

int write_ice_table_file(const char* path, const char* version) {
  std::vector<double> ice_raw, coll_raw;
  generate_ice_raw(ice_raw, coll_raw);
  FILE* fp = std::fopen(path, "w");
  if (!fp) return -1;
  std::fprintf(fp, "VERSION %s\n", version);
  for (int s = 0; s < n_rhor * n_Fr; ++s) {
    const int i_rhor = s / n_Fr + 1, i_Fr = s % n_Fr + 1;
    for (int i = 0; i < n_Qnorm; ++i) {
      std::fprintf(fp, "%5d%5d", i_rhor, i_Fr);
      for (int j = 0; j < kIceRawCols; ++j)
        std::fprintf(fp, "%15.4E", ice_raw[(size_t(s) * n_Qnorm + i) * kIceRawCols + j]);
      std::fprintf(fp, "\n");
    }
    for (int i = 0; i < n_Qnorm; ++i) {
      for (int j = 0; j < n_Drscale; ++j) {
        std::fprintf(fp, "%5d%5d", i_rhor, i_Fr);
        for (int k = 0; k < kCollRawCols; ++k)
          std::fprintf(fp, "%15.4E", coll_raw[((size_t(s) * n_Qnorm + i) * n_Drscale + j) * kCollRawCols + k]);
        std::fprintf(fp, "\n");
      }
    }
  }
  std::fclose(fp);
  return 0;
}

/* Reader for the official text format, p3_table_ice_impl.hpp:33-71.
 * Returns 0, or -1 (cannot open), -2 (bad header), -3 (version mismatch),
 * -4 (truncated file). */
int read_ice_table_file(const char* path, const char* expect_version, HostTables& T) {
  std::ifstream in(path);
  if (!in) return -1;
  std::string tag, ver;
  in >> tag >> ver;
  if (tag != "VERSION") return -2;
  if (expect_version && ver != expect_version) return -3;
  T.ice.assign(size_t(n_rhor) * n_Fr * n_Qnorm * kIceCols, 0.0);
  T.collect.assign(size_t(n_rhor) * n_Fr * n_Qnorm * n_Drscale * kCollCols, 0.0);
  double dum_s;
  int dum_i;
  for (int jj = 0; jj < n_rhor; ++jj) {
    for (int ii = 0; ii < n_Fr; ++ii) {
      const size_t s = size_t(jj) * n_Fr + ii;
      for (int i = 0; i < n_Qnorm; ++i) {
        if (!(in >> dum_i >> dum_i)) return -4;
        int j_idx = 0;
        for (int j = 0; j < kIceRawCols; ++j) {
          if (!(in >> dum_s)) return -4;
          if (j > 1 && j != 10) T.ice[(s * n_Qnorm + i) * kIceCols + j_idx++] = dum_s;
        }
      }
      for (int i = 0; i < n_Qnorm; ++i) {
        for (int j = 0; j < n_Drscale; ++j) {
          if (!(in >> dum_i >> dum_i)) return -4;
          int k_idx = 0;
          for (int k = 0; k < kCollRawCols; ++k) {
            if (!(in >> dum_s)) return -4;
            if (k == 3 || k == 4)
              T.collect[((s * n_Qnorm + i) * n_Drscale + j) * kCollCols + k_idx++] = std::log10(dum_s);
          }
        }
      }
    }
  }
  return 0;
}

/* Saturation table of the FP32-bulk form.  Cubic Hermite interpolants of the
 * Murphy-Koop vapour pressures (share/physics_saturation_impl.hpp:38-81) and
 * their analytic temperature derivatives, evaluated in long double, on a
 * 1/64 K grid: the interpolation error is below 1e-12 relative at 150 K and
 * below 1e-13 above 200 K. */
namespace {
void mk_log_svp(long double T, bool ice, long double& lnf, long double& dlnf) {
  if (ice) {
    lnf = 9.550426L - 5723.265L / T + 3.53068L * std::log(T) - 0.00728332L * T;
    dlnf = 5723.265L / (T * T) + 3.53068L / T - 0.00728332L;
    return;
  }
  const long double th = std::tanh(0.0415L * (T - 218.8L));
  const long double B = 53.878L - 1331.22L / T - 9.44523L * std::log(T) + 0.014025L * T;
  const long double dB = 1331.22L / (T * T) - 9.44523L / T + 0.014025L;
  lnf = 54.842763L - 6763.22L / T - 4.210L * std::log(T) + 0.000367L * T + th * B;
  dlnf = 6763.22L / (T * T) - 4.210L / T + 0.000367L + 0.0415L * (1 - th * th) * B + th * dB;
}
}  // namespace

void build_svp_table(std::vector<double>& coef) {
  coef.assign(size_t(2) * kSvpIntervals * 4, 0.0);
  const long double h = 1.0L / kSvpInvH;
  for (int phase = 0; phase < 2; ++phase) {
    for (int i = 0; i < kSvpIntervals; ++i) {
      const long double Ta = kSvpT0 + i * h, Tb = Ta + h;
      long double la, da, lb, db;
      mk_log_svp(Ta, phase == 1, la, da);
      mk_log_svp(Tb, phase == 1, lb, db);
      const long double fa = std::exp(la), fb = std::exp(lb);
      const long double ga = h * fa * da, gb = h * fb * db; /* d e / d u */
      double* r = &coef[(size_t(phase) * kSvpIntervals + i) * 4];
      r[0] = double(fa);
      r[1] = double(ga);
      r[2] = double(3 * (fb - fa) - 2 * ga - gb);
      r[3] = double(2 * (fa - fb) + ga + gb);
    }
  }
}

}  // namespace p3x
