/*
 * Device physics of the P3 step, templated on the process-rate type TR
 * (double: plain form; float: FP32-bulk form).  State (mixing ratios,
 * numbers, theta, qv), saturation residuals, conservation limiters and the
 * prognostic updates are always FP64.
 *
 * Each routine states the same formula as the reference routine it names
 * (paths relative to components/eamxx/src/physics/), in the same order of
 * operations, so the FP64 form differs from the CPU reference only by the
 * rounding of the math library and fused multiply-adds.
 */
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace p3x {
namespace dev {

/* share/physics_constants.hpp:27-102 */
namespace C {
constexpr double Cpair = 1004.64, Rair = 287.042, RH2O = 461.505, RV = RH2O;
constexpr double RHO_H2O = 1000.0, INV_RHO_H2O = 1.0 / RHO_H2O;
constexpr double ep_2 = 18.016 / 28.966;
constexpr double gravit = 9.80616, LatVap = 2501000.0, LatIce = 333700.0, CpLiq = 4188.0;
constexpr double Tmelt = 273.15, T_zerodegc = Tmelt, T_homogfrz = Tmelt - 40, T_rainfrz = Tmelt - 4;
constexpr double Pi = 3.14159265358979323;
constexpr double INV_RHO_RIMEMAX = 1.0 / 900.0;
constexpr double THIRD = 1.0 / 3.0, SXTH = 1.0 / 6.0, PIOV3 = Pi * THIRD, PIOV6 = Pi * SXTH;
constexpr double BIMM = 2.0, CONS1 = PIOV6 * RHO_H2O, CONS2 = 4. * PIOV3 * RHO_H2O;
constexpr double CONS3 = 1.0 / (CONS2 * 1.562500000000000e-14);
constexpr double CONS5 = PIOV6 * BIMM, CONS6 = PIOV6 * PIOV6 * RHO_H2O * BIMM;
constexpr double QSMALL = 1.e-14, QTENDSMALL = 1e-20, BSMALL = 1.e-15, NSMALL = 1.e-16;
constexpr double P0 = 100000.0, RD = Rair;
constexpr double RHO_1000MB = P0 / (RD * Tmelt), RHO_600MB = 60000 / (RD * 253.15);
constexpr double CP = Cpair, INV_CP = 1.0 / CP;
constexpr double dt_left_tol = 1.e-4, bcn = 2., dropmass = 5.2e-7, NCCNST = 200.0e+6;
constexpr double incloud_limit = 5.1e-3, precip_limit = 1.0e-2, f1r = 0.78, f2r = 0.32;
constexpr double nmltratio = 1.0;
constexpr double lookup_table_1a_dum1_c = 4.135985029041767e+00;
}  // namespace C

constexpr int kDensize = 5, kRimsize = 4, kIsize = 50, kIceCols = 12, kRcollsize = 30,
              kCollCols = 2, kVT1 = 10;

/* status bits accumulated on the device */
enum : uint32_t { kErrNumeric = 1u, kErrSubstep = 2u, kErrWait = 4u, kErrRange = 8u };

/* Runtime options, P3Runtime (p3/p3_functions.hpp:112-133). */
struct RuntimeDev {
  double max_total_ni, autoconversion_prefactor, autoconversion_qc_exponent,
      autoconversion_nc_exponent, autoconversion_radius, accretion_prefactor,
      accretion_qc_exponent, accretion_qr_exponent, rain_selfcollection_prefactor,
      rain_selfcollection_breakup_diameter, constant_mu_rain, spa_ccn_to_nc_factor,
      cldliq_to_ice_collection_factor, rain_to_ice_collection_factor, min_rime_rho, max_rime_rho,
      immersion_freezing_exponent, deposition_nucleation_exponent, ice_sedimentation_factor;
  int do_ice_production;
  /* derived once on the host */
  double cons3;       /* autoconversion CONS3 (p3_autoconversion_impl.hpp:27-32) */
  int t3_dumjj;       /* Table3 mu index for the constant mu_r (p3_table3_impl.hpp:52-62) */
  double t3_rdumjj;
  /* Gamma function of the constant rain shape parameter mu_r */
  double g_mur1;      /* Gamma(mu_r + 1)       */
  double g_mur2;      /* Gamma(mu_r + 2)       */
  double lg_mur4;     /* log Gamma(mu_r + 4)   */
  double lg_mur7;     /* log Gamma(mu_r + 7)   */
  /* FP32-bulk saturation table (layout of build_svp_table) */
  const double* svp_tab;
  /* accretion_qc_exponent == accretion_qr_exponent (the single-power form) */
  int accretion_same_exponent;
  /* float copies (rounded to nearest on the host) of the parameters the
   * FP32-bulk rates read, so no kernel converts them */
  struct F32 {
    float max_total_ni, autoconversion_prefactor, autoconversion_qc_exponent, autoconversion_nc_exponent,
        accretion_prefactor, accretion_qc_exponent, accretion_qr_exponent, rain_selfcollection_prefactor,
        rain_selfcollection_breakup_diameter, constant_mu_rain, cldliq_to_ice_collection_factor,
        rain_to_ice_collection_factor, min_rime_rho, max_rime_rho, immersion_freezing_exponent,
        deposition_nucleation_exponent, ice_sedimentation_factor, cons3, t3_rdumjj, g_mur1, g_mur2, lg_mur4,
        lg_mur7;
  } f;
};

/* a runtime parameter in the rate type: the FP64 value, or its float copy */
template <class TR>
__device__ __forceinline__ TR rtp(double d, float f) {
  if constexpr (sizeof(TR) == sizeof(float)) {
    return f;
  } else {
    return d;
  }
}
#define P3X_RTP(TR, name) rtp<TR>(rt.name, rt.f.name)

/* ------------------------------------------------------------------ */
/* math wrappers (explicit precision)                                  */
/* ------------------------------------------------------------------ */
/* The FP64 forms go through one out-of-line copy each: the FP64 kernels'
 * dozens of inlined exp/log/pow/tanh/tgamma expansions overflowed the
 * instruction cache (part1+2's top stall was no_instruction); one copy per
 * function made the FP64 step 5 % faster with bitwise the same results.  The
 * FP32 forms stay inline. */
static __device__ __noinline__ double m_exp_nl(double x) { return exp(x); }
__device__ __forceinline__ double m_exp(double x) { return m_exp_nl(x); }
__device__ __forceinline__ float m_exp(float x) { return expf(x); }
static __device__ __noinline__ double m_log_nl(double x) { return log(x); }
__device__ __forceinline__ double m_log(double x) { return m_log_nl(x); }
__device__ __forceinline__ float m_log(float x) { return logf(x); }
static __device__ __noinline__ double m_log10_nl(double x) { return log10(x); }
__device__ __forceinline__ double m_log10(double x) { return m_log10_nl(x); }
__device__ __forceinline__ float m_log10(float x) { return log10f(x); }
static __device__ __noinline__ double m_pow_nl(double x, double y) { return pow(x, y); }
__device__ __forceinline__ double m_pow(double x, double y) { return m_pow_nl(x, y); }
__device__ __forceinline__ float m_pow(float x, float y) { return powf(x, y); }
static __device__ __noinline__ double m_cbrt_nl(double x) { return cbrt(x); }
__device__ __forceinline__ double m_cbrt(double x) { return m_cbrt_nl(x); }
__device__ __forceinline__ float m_cbrt(float x) { return cbrtf(x); }
static __device__ __noinline__ double m_sqrt_nl(double x) { return sqrt(x); }
__device__ __forceinline__ double m_sqrt(double x) { return m_sqrt_nl(x); }
__device__ __forceinline__ float m_sqrt(float x) { return sqrtf(x); }
static __device__ __noinline__ double m_tgamma_nl(double x) { return tgamma(x); }
__device__ __forceinline__ double m_tgamma(double x) { return m_tgamma_nl(x); }
__device__ __forceinline__ float m_tgamma(float x) { return tgammaf(x); }
static __device__ __noinline__ double m_expm1_nl(double x) { return expm1(x); }
__device__ __forceinline__ double m_expm1(double x) { return m_expm1_nl(x); }
__device__ __forceinline__ float m_expm1(float x) { return expm1f(x); }
static __device__ __noinline__ double m_tanh_nl(double x) { return tanh(x); }
__device__ __forceinline__ double m_tanh(double x) { return m_tanh_nl(x); }
__device__ __forceinline__ float m_tanh(float x) { return tanhf(x); }
__device__ __forceinline__ double m_fabs(double x) { return fabs(x); }
__device__ __forceinline__ float m_fabs(float x) { return fabsf(x); }

/* Exact float -> double conversion on the integer pipes: a normal float's
 * exponent is re-biased (+896) and its 23-bit significand shifted into the
 * double's 52-bit field; signed zeros map to signed zeros.  Subnormals,
 * infinities and NaNs take the hardware conversion.  For kernels bound by
 * the FP64 pipe, which also executes the hardware conversion, while their
 * integer pipes are nearly idle (the FP32-bulk part3; the selftest checks it
 * against the hardware for every float). */
__device__ __forceinline__ double f2d_int(float x) {
  const uint32_t u = __float_as_uint(x);
  const uint32_t e = (u >> 23) & 0xffu;
  const uint32_t mag = u & 0x7fffffffu;
  if ((e - 1u) >= 254u && mag != 0u) return double(x);
  const uint32_t m = u & 0x7fffffu;
  const uint32_t hi = (u & 0x80000000u) | (mag ? (((e + 896u) << 20) | (m >> 3)) : 0u);
  const uint32_t lo = (m & 7u) << 29;
  return __hiloint2double(int(hi), int(lo));
}

/* Float -> double where the instruction footprint limits the kernel more than
 * the FP64 pipe: the FP32-bulk part1+2 and sedimentation kernels are larger
 * than the SM's instruction cache (instruction fetch is part1+2's top stall at
 * 65,536 columns), and the hardware conversion is one instruction where
 * f2d_int inlines a dozen and a branch at each of some 80 call sites.  The
 * FP64-pipe-bound part3 keeps f2d_int.  Both are exact. */
__device__ __forceinline__ double f2d(float x) { return double(x); }

/* 1/x for the FP32-bulk form by Newton-Raphson from the FP32 reciprocal:
 * each step r <- r + r (1 - x r) squares the relative error (~2^-22 from
 * the FP32 seed, ~2^-44 after one step, below the FP64 rounding after two),
 * so the result is within an ulp or two of 1/x.  Four FP64 FMAs replace the
 * FP64 division sequence.  For positive normal x inside the float range
 * (pressures, Exner factors, layer thicknesses). */
__device__ __forceinline__ double rcp_newton(double x) {
  double r = f2d(__fdividef(1.0f, float(x)));
  r = fma(r, fma(-x, r, 1.0), r);
  r = fma(r, fma(-x, r, 1.0), r);
  return r;
}
/* One step only: relative error ~2^-44 (~1e-14), used where that is below
 * the other errors of the quantity (the saturation table's 1e-12). */
__device__ __forceinline__ double rcp_newton1(double x) {
  const double r = f2d(__fdividef(1.0f, float(x)));
  return fma(r, fma(-x, r, 1.0), r);
}

/* Double -> float on the integer pipes, rounding toward zero.  The top 23
 * significand bits are funnel-shifted under the re-biased exponent
 * (exponent - 896, taken mod 2^9 in the 32-bit word); |x| below 2^-126
 * becomes a signed zero, and |x| >= 2^128, infinities and NaN take the
 * hardware conversion.  Truncation is monotone and exact on integers, so
 * floor(d2f_rz(x)) = floor(x) for 0 <= x < 2^22: the saturation table's
 * interval index uses it.  (As a general narrowing of state values it was
 * slower than the hardware conversion, and its one-sided rounding biased the
 * sedimentation's substep counts.) */
__device__ __forceinline__ float d2f_rz(double x) {
  const uint32_t hi = uint32_t(__double2hiint(x)), lo = uint32_t(__double2loint(x));
  const uint32_t ahi = hi & 0x7fffffffu;
  if (ahi >= 0x47f00000u) return float(x);
  const uint32_t m = __funnelshift_l(lo, ahi, 3) - (896u << 23);
  return __uint_as_float((ahi < 0x38100000u ? 0u : m) | (hi & 0x80000000u));
}

/* Float <-> small integer on the FP32 and integer pipes (the hardware
 * conversions execute on the FP64 pipe on this part).  Magic-number method:
 * adding 1.5 * 2^23 with rounding toward minus infinity leaves floor(x) in
 * the low significand bits for |x| < 2^22; the reverse subtraction gives the
 * exact float of an integer |i| < 2^22. */
__device__ __forceinline__ int ffloor_small(float x) {
  return __float_as_int(__fadd_rd(x, 12582912.0f)) - 0x4B400000;
}
__device__ __forceinline__ float i2f_small(int i) { return __int_as_float(i + 0x4B400000) - 12582912.0f; }

/* Table index of a coordinate: the reference truncates to int and then
 * clamps the index to [1, hi - 1] (or a narrower range); truncating x
 * clamped to [0, hi] gives the same index for every x, NaN included (0, as
 * the hardware conversion gives).  The FP64 form keeps the conversion. */
__device__ __forceinline__ int table_index(float x, int hi) {
  return ffloor_small(fminf(fmaxf(x, 0.0f), float(hi)));
}
__device__ __forceinline__ int table_index(double x, int) { return static_cast<int>(x); }
/* a table index as the rate type */
__device__ __forceinline__ void index_value(int i, float& v) { v = i2f_small(i); }
__device__ __forceinline__ void index_value(int i, double& v) { v = double(i); }
template <class TR>
__device__ __forceinline__ TR ival(int i) {
  TR v;
  index_value(i, v);
  return v;
}

/* widen(x): exact conversion to double (identity for doubles) */
__device__ __forceinline__ double widen(double x) { return x; }
__device__ __forceinline__ double widen(float x) { return f2d(x); }

/* Threshold tests of a double against a constant, on the integer pipes.
 * For c > 0 the IEEE order of x against c is the signed order of the two
 * bit patterns for every x that is not NaN: a negative x (or -0) has the sign
 * bit set and compares below any positive pattern.  For c < 0 and x < 0 the
 * signed order of the patterns is the reverse of the order of the values.
 * A NaN compares by its bit pattern; only an already invalid state holds
 * one, and the saturation step reports that separately. */
__device__ __forceinline__ long long dbits(double x) { return __double_as_longlong(x); }
/* x < c, x >= c, x > c, x <= c for a constant c > 0 */
__device__ __forceinline__ bool dlt(double x, double c) { return dbits(x) < dbits(c); }
__device__ __forceinline__ bool dge(double x, double c) { return dbits(x) >= dbits(c); }
__device__ __forceinline__ bool dgt(double x, double c) { return dbits(x) > dbits(c); }
__device__ __forceinline__ bool dle(double x, double c) { return dbits(x) <= dbits(c); }
/* x >= c and x < c for a constant c < 0 */
__device__ __forceinline__ bool dge_neg(double x, double c) { return dbits(x) >= 0 || dbits(x) <= dbits(c); }
__device__ __forceinline__ bool dlt_neg(double x, double c) { return !dge_neg(x, c); }
/* x < 0 (false for -0) */
__device__ __forceinline__ bool dneg(double x) {
  return static_cast<unsigned long long>(dbits(x)) > 0x8000000000000000ull;
}
/* vmax(x, c) = (x < c) ? c : x and vmin(x, c) = (c < x) ? c : x, c > 0 */
__device__ __forceinline__ double dmax_c(double x, double c) { return dlt(x, c) ? c : x; }
__device__ __forceinline__ double dmin_c(double x, double c) { return dgt(x, c) ? c : x; }
/* x > 0 */
__device__ __forceinline__ bool dpos(double x) { return dbits(x) > 0; }
/* vmax(a, b) = (a < b) ? b : a for non-negative a and b (Courant numbers): the
 * bit patterns order as the values; a NaN b propagates (it would be dropped by
 * the IEEE form) and is then caught by the Courant check */
__device__ __forceinline__ double dmax_nn(double a, double b) { return dbits(a) < dbits(b) ? b : a; }
/* x is not +0 (adding or subtracting it may change a value) */
__device__ __forceinline__ bool dnz(double x) { return dbits(x) != 0; }
/* vmax(x, 0.) = (x < 0) ? 0 : x, and vmax(0., x) = (0 < x) ? x : 0 (+0 for -0) */
__device__ __forceinline__ double dmax0(double x) { return dneg(x) ? 0.0 : x; }
__device__ __forceinline__ double dmax_0x(double x) { return dpos(x) ? x : 0.0; }

/* Double-float accumulators on the FP32 pipe: a value is the unevaluated sum
 * hi + lo of two floats with |lo| <= ulp(hi) / 2 (about 48 significant bits).
 * Additions use Knuth's TwoSum followed by Dekker's Fast2Sum renormalisation;
 * the product of two floats is made exact with the FMA error-free product.
 * Every step is a correctly rounded FP32 operation written with the _rn
 * intrinsics, so the compiler can neither contract nor reorder it.  One update
 * costs ~14 FP32 instructions, against one FP64 FMA that occupies the FP64
 * pipe for the issue time of ~64 FP32 instructions on this part. */
/* exact value as a double: |lo| <= ulp(hi)/2, so hi + lo spans <= 48 bits */
__device__ __forceinline__ double dfloat_value(float2 g) { return f2d(g.x) + f2d(g.y); }

__device__ __forceinline__ float2 dfloat_renorm(float s, float e) {
  const float hi = __fadd_rn(s, e);
  return make_float2(hi, __fsub_rn(e, __fsub_rn(hi, s)));
}

/* g += a */
__device__ __forceinline__ void dfloat_add(float2& g, float a) {
  const float s = __fadd_rn(g.x, a);
  const float bb = __fsub_rn(s, g.x);
  const float e = __fadd_rn(__fsub_rn(g.x, __fsub_rn(s, bb)), __fsub_rn(a, bb));
  g = dfloat_renorm(s, __fadd_rn(e, g.y));
}

/* g += a * t, with the product a * t formed exactly (ph + pl) */
__device__ __forceinline__ void dfloat_add_prod(float2& g, float a, float t) {
  const float ph = __fmul_rn(a, t);
  const float pl = __fmaf_rn(a, t, -ph);
  const float s = __fadd_rn(g.x, ph);
  const float bb = __fsub_rn(s, g.x);
  const float e = __fadd_rn(__fsub_rn(g.x, __fsub_rn(s, bb)), __fsub_rn(ph, bb));
  g = dfloat_renorm(s, __fadd_rn(e, __fadd_rn(g.y, pl)));
}

/* Packed FP32 (Blackwell FFMA2/FADD2/FMUL2): two correctly rounded FP32
 * operations per lane and instruction, each component exactly the scalar
 * operation. */
__device__ __forceinline__ float2 f2neg(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 f2splat(float a) { return make_float2(a, a); }
/* a + w (b - a), as the scalar code evaluates it: fma(w, b - a, a) */
__device__ __forceinline__ float2 lerp2(float2 a, float2 b, float2 w) {
  return __ffma2_rn(w, __fadd2_rn(b, f2neg(a)), a);
}

/* Two double-floats side by side, g = {hi0, hi1, lo0, lo1}: g += a * t per
 * component, with the same steps as dfloat_add_prod. */
__device__ __forceinline__ void dfloat2_add_prod(float4& g, float2 a, float t) {
  const float2 tt = f2splat(t);
  const float2 hi = make_float2(g.x, g.y), lo = make_float2(g.z, g.w);
  const float2 ph = __fmul2_rn(a, tt);
  const float2 pl = __ffma2_rn(a, tt, f2neg(ph));
  const float2 s = __fadd2_rn(hi, ph);
  const float2 bb = __fadd2_rn(s, f2neg(hi));
  const float2 e = __fadd2_rn(__fadd2_rn(hi, f2neg(__fadd2_rn(s, f2neg(bb)))), __fadd2_rn(ph, f2neg(bb)));
  const float2 e2 = __fadd2_rn(e, __fadd2_rn(lo, pl));
  const float2 nh = __fadd2_rn(s, e2);
  const float2 nl = __fadd2_rn(e2, f2neg(__fadd2_rn(nh, f2neg(s))));
  g = make_float4(nh.x, nh.y, nl.x, nl.y);
}

/* std::max / std::min semantics ((a < b) ? b : a), as the CPU reference. */
template <class T> __device__ __forceinline__ T vmax(T a, T b) { return (a < b) ? b : a; }
template <class T> __device__ __forceinline__ T vmin(T a, T b) { return (b < a) ? b : a; }
template <class T> __device__ __forceinline__ T sq(T x) { return x * x; }

/* ------------------------------------------------------------------ */
/* Saturation (share/physics_saturation_impl.hpp)                      */
/* ------------------------------------------------------------------ */

/* MurphyKoop_svp, physics_saturation_impl.hpp:38-81.  T <= 0 or NaN sets the
 * numeric status bit (the reference aborts the kernel there). */
template <class TR>
__device__ __forceinline__ TR murphy_koop_svp(TR t, bool ice, uint32_t& err) {
  if (!(t > TR(0))) err |= kErrNumeric;
  if (t < TR(C::Tmelt) && ice) {
    return m_exp(TR(9.550426) - (TR(5723.265) / t) + (TR(3.53068) * m_log(t)) - (TR(0.00728332) * t));
  }
  const TR logt = m_log(t);
  return m_exp(TR(54.842763) - (TR(6763.22) / t) - (TR(4.210) * logt) + (TR(0.000367) * t) +
               (m_tanh(TR(0.0415) * (t - TR(218.8))) *
                (TR(53.878) - (TR(1331.22) / t) - (TR(9.44523) * logt) + TR(0.014025) * t)));
}

/* Murphy-Koop vapour pressure from the FP64 saturation table of the
 * FP32-bulk form: one cubic per 1/64 K interval from 150 K (interpolation
 * error < 1e-12 relative), the formula outside the tabulated range. */
constexpr double kSvpT0 = 150.0, kSvpInvH = 64.0;
constexpr int kSvpIntervals = 12800;
/* The formula outside the table, out of line: it is rarely reached, and its
 * FP64 divisions would otherwise be inlined at every table call site (about
 * 6 KB of code each in the FP32-bulk part1+2 kernel, which is larger than the
 * instruction cache).  The status bits come back with the value. */
struct SvpValue {
  double v;
  uint32_t err;
};
static __device__ __noinline__ SvpValue svp_out_of_table(double t, bool ice) {
  uint32_t e = 0;
  const double v = murphy_koop_svp<double>(t, ice, e);
  return SvpValue{v, e};
}

__device__ __forceinline__ double svp_tabulated(const double* tab, double t, bool ice, uint32_t& err) {
  const double x = fma(t, kSvpInvH, -kSvpT0 * kSvpInvH); /* = (t - T0) * 64, both exact here */
  if (!(!dneg(x) && dlt(x, double(kSvpIntervals)))) {
    const SvpValue r = svp_out_of_table(t, ice);
    err |= r.err;
    return r.v;
  }
  /* floor(x) through the truncated float (exact, see d2f_rz) and its exact
   * double, off the FP64 pipe */
  const int i = ffloor_small(d2f_rz(x));
  const double u = x - f2d(i2f_small(i));
  const int row = (ice && dlt(t, C::Tmelt)) ? kSvpIntervals + i : i;
  const double2* c = reinterpret_cast<const double2*>(tab) + size_t(row) * 2;
  const double2 c01 = __ldg(c), c23 = __ldg(c + 1);
  return c01.x + u * (c01.y + u * (c23.x + u * c23.y));
}

/* qv_sat_dry (MurphyKoop), physics_saturation_impl.hpp:126-157, as the
 * plain form evaluates it (the FP32-bulk form reads svp_tabulated). */
__device__ __forceinline__ double qv_sat_dry(double t, double p, bool ice, uint32_t& err) {
  const double e_pres = murphy_koop_svp<double>(t, ice, err);
  return C::ep_2 * e_pres / vmax(p, 1.e-3);
}

/* ------------------------------------------------------------------ */
/* Tables                                                              */
/* ------------------------------------------------------------------ */
/* Table pointers (global or staged shared memory; generic addresses).
 * t3 tables may be the full [300][10] arrays (t3_stride = 10, t3_j0 = 0) or
 * a staged two-column slice (t3_stride = 2, t3_j0 = first staged column). */
template <class TR>
struct Tabs {
  const TR* ice;
  const TR* collect;
  const TR* vn;
  const TR* vm;
  const TR* revap;
  int t3_stride, t3_j0;
};

/* Device order of the 12 ice-table columns: slot s holds reference column
 * kIceSlotCol[s].  Slots 0-3 are the columns ice sedimentation needs (0,1,6,7),
 * slots 4-7 the rest of part2's (2,3,4,9), slots 8-11 the rest of part3's
 * (5,11,8,10), so each stage reads a table corner with one or two 16-byte
 * vector loads instead of one scalar load per column. */
constexpr int kIceSlotCol[kIceCols] = {0, 1, 6, 7, 2, 3, 4, 9, 5, 11, 8, 10};
constexpr int kIceSedCols = 4;

__device__ __forceinline__ void ld4(const float* p, float o[4]) {
  const float4 v = *reinterpret_cast<const float4*>(p);
  o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
}
__device__ __forceinline__ void ld4(const double* p, double o[4]) {
  const double2 a = reinterpret_cast<const double2*>(p)[0];
  const double2 b = reinterpret_cast<const double2*>(p)[1];
  o[0] = a.x; o[1] = a.y; o[2] = b.x; o[3] = b.y;
}
template <class TR>
__device__ __forceinline__ const TR* ice_row(const Tabs<TR>& t, int jj, int ii, int i) {
  return t.ice + ((jj * kRimsize + ii) * kIsize + i) * kIceCols;
}
template <class TR>
__device__ __forceinline__ TR coll_at(const Tabs<TR>& t, int jj, int ii, int i, int j, int idx) {
  return __ldg(&t.collect[(((jj * kRimsize + ii) * kIsize + i) * kRcollsize + j) * kCollCols + idx]);
}
template <class TR>
__device__ __forceinline__ TR t3_at(const Tabs<TR>& t, const TR* tab, int i, int j) {
  return tab[i * t.t3_stride + (j - t.t3_j0)];
}

template <class TR>
struct TableIce {
  int dumi, dumjj, dumii;
  TR dum1, dum4, dum5;
};
template <class TR>
struct TableRain {
  int dumj;
  TR dum3;
};
template <class TR>
struct Table3 {
  int dumii, dumjj;
  TR rdumii, rdumjj;
};

/* lookup_ice, p3/impl/p3_table_ice_impl.hpp:80-138 */
template <class TR>
__device__ __forceinline__ void lookup_ice(TR qi, TR ni, TR qm, TR rhop, TableIce<TR>& tab) {
  tab.dum1 = (m_log10(qi / ni) + TR(18)) * TR(C::lookup_table_1a_dum1_c) - TR(10);
  tab.dumi = table_index(tab.dum1, kIsize);
  tab.dum1 = vmin(tab.dum1, TR(kIsize));
  tab.dum1 = vmax(tab.dum1, TR(1.));
  tab.dumi = max(1, tab.dumi);
  tab.dumi = min(kIsize - 1, tab.dumi);
  tab.dum4 = (qm / qi) * TR(3) + TR(1);
  tab.dumii = table_index(tab.dum4, kRimsize);
  tab.dum4 = vmin(tab.dum4, TR(kRimsize));
  tab.dum4 = vmax(tab.dum4, TR(1.));
  tab.dumii = max(1, tab.dumii);
  tab.dumii = min(kRimsize - 1, tab.dumii);
  if (rhop <= TR(650)) {
    tab.dum5 = (rhop - TR(50)) * TR(0.005) + TR(1);
  } else {
    tab.dum5 = (rhop - TR(650)) * TR(0.004) + TR(4);
  }
  tab.dumjj = table_index(tab.dum5, kDensize);
  tab.dum5 = vmin(tab.dum5, TR(kDensize));
  tab.dum5 = vmax(tab.dum5, TR(1.));
  tab.dumjj = max(1, tab.dumjj);
  tab.dumjj = min(kDensize - 1, tab.dumjj);
  tab.dumi -= 1;
  tab.dumjj -= 1;
  tab.dumii -= 1;
}

/* lookup_rain, p3_table_ice_impl.hpp:140-173 */
template <class TR>
__device__ __forceinline__ void lookup_rain(TR qr, TR nr, TableRain<TR>& tab) {
  const bool gt_small = qr > TR(C::QSMALL) && nr > TR(0.0);
  TR dumlr = TR(1);
  if (gt_small) dumlr = m_cbrt(qr / (TR(C::Pi) * TR(C::RHO_H2O) * nr));
  tab.dum3 = (m_log10(TR(1) * dumlr) + TR(5)) * TR(10.70415);
  tab.dumj = table_index(tab.dum3, kRcollsize);
  tab.dum3 = vmin(tab.dum3, TR(kRcollsize));
  tab.dum3 = vmax(tab.dum3, TR(1));
  tab.dumj = max(1, tab.dumj);
  tab.dumj = min(kRcollsize - 1, tab.dumj);
  if (!gt_small) {
    tab.dumj = 1;
    tab.dum3 = TR(1);
  }
  tab.dumj -= 1;
}

/* apply_table_ice, p3_table_ice_impl.hpp:175-212, for the four device slots
 * s0..s0+3 at once (s0 a multiple of 4); each value is interpolated with the
 * reference's order of operations. */
template <class TR>
__device__ __forceinline__ void apply_table_ice4(const Tabs<TR>& t, const TableIce<TR>& tab, int s0, TR out[4]) {
  const TR w1 = tab.dum1 - ival<TR>(tab.dumi) - TR(1);
  const TR w4 = tab.dum4 - ival<TR>(tab.dumii) - TR(1);
  const TR w5 = tab.dum5 - ival<TR>(tab.dumjj) - TR(1);
  TR a00[4], a01[4], a10[4], a11[4], b00[4], b01[4], b10[4], b11[4];
  ld4(ice_row(t, tab.dumjj, tab.dumii, tab.dumi) + s0, a00);
  ld4(ice_row(t, tab.dumjj, tab.dumii, tab.dumi + 1) + s0, a01);
  ld4(ice_row(t, tab.dumjj, tab.dumii + 1, tab.dumi) + s0, a10);
  ld4(ice_row(t, tab.dumjj, tab.dumii + 1, tab.dumi + 1) + s0, a11);
  ld4(ice_row(t, tab.dumjj + 1, tab.dumii, tab.dumi) + s0, b00);
  ld4(ice_row(t, tab.dumjj + 1, tab.dumii, tab.dumi + 1) + s0, b01);
  ld4(ice_row(t, tab.dumjj + 1, tab.dumii + 1, tab.dumi) + s0, b10);
  ld4(ice_row(t, tab.dumjj + 1, tab.dumii + 1, tab.dumi + 1) + s0, b11);
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    TR iproc1 = a00[c] + w1 * (a01[c] - a00[c]);
    TR gproc1 = a10[c] + w1 * (a11[c] - a10[c]);
    const TR tmp1 = iproc1 + w4 * (gproc1 - iproc1);
    iproc1 = b00[c] + w1 * (b01[c] - b00[c]);
    gproc1 = b10[c] + w1 * (b11[c] - b10[c]);
    const TR tmp2 = iproc1 + w4 * (gproc1 - iproc1);
    out[c] = tmp1 + w5 * (tmp2 - tmp1);
  }
}

/* The FP32 form of apply_table_ice4 on packed pairs of columns (s0..s0+1
 * and s0+2..s0+3): the same interpolations in the same order.  STRIDE is
 * the row length of the table copy read (kIceCols, or kIceSedCols for the
 * packed sedimentation copy), a constant so that the eight corners are one
 * address plus immediate offsets. */
template <int STRIDE>
__device__ __forceinline__ void ice_table4_f32(const float* ice, const TableIce<float>& tab, int s0, float out[4]) {
  const float w1 = tab.dum1 - ival<float>(tab.dumi) - 1.0f;
  const float w4 = tab.dum4 - ival<float>(tab.dumii) - 1.0f;
  const float w5 = tab.dum5 - ival<float>(tab.dumjj) - 1.0f;
  const float2 W1 = f2splat(w1), W4 = f2splat(w4), W5 = f2splat(w5);
  const float* const r = ice + ((tab.dumjj * kRimsize + tab.dumii) * kIsize + tab.dumi) * STRIDE + s0;
  constexpr int dI = STRIDE, dR = kIsize * STRIDE, dD = kRimsize * kIsize * STRIDE;
  auto at = [&](int off) { return *reinterpret_cast<const float4*>(r + off); };
  const float4 a00 = at(0), a01 = at(dI), a10 = at(dR), a11 = at(dR + dI);
  const float4 b00 = at(dD), b01 = at(dD + dI), b10 = at(dD + dR), b11 = at(dD + dR + dI);
  auto lo = [](float4 v) { return make_float2(v.x, v.y); };
  auto hi = [](float4 v) { return make_float2(v.z, v.w); };
  const float2 t1l = lerp2(lerp2(lo(a00), lo(a01), W1), lerp2(lo(a10), lo(a11), W1), W4);
  const float2 t2l = lerp2(lerp2(lo(b00), lo(b01), W1), lerp2(lo(b10), lo(b11), W1), W4);
  const float2 t1h = lerp2(lerp2(hi(a00), hi(a01), W1), lerp2(hi(a10), hi(a11), W1), W4);
  const float2 t2h = lerp2(lerp2(hi(b00), hi(b01), W1), lerp2(hi(b10), hi(b11), W1), W4);
  const float2 rl = lerp2(t1l, t2l, W5), rh = lerp2(t1h, t2h, W5);
  out[0] = rl.x; out[1] = rl.y; out[2] = rh.x; out[3] = rh.y;
}
template <>
__device__ __forceinline__ void apply_table_ice4<float>(const Tabs<float>& t, const TableIce<float>& tab, int s0,
                                                       float out[4]) {
  ice_table4_f32<kIceCols>(t.ice, tab, s0, out);
}

/* apply_table_coll, p3_table_ice_impl.hpp:214-297 */
template <class TR>
__device__ __forceinline__ TR apply_table_coll(int idx, const Tabs<TR>& t, const TableIce<TR>& ti,
                                               const TableRain<TR>& tr) {
  const TR w1 = ti.dum1 - ival<TR>(ti.dumi) - TR(1);
  const TR w3 = tr.dum3 - ival<TR>(tr.dumj) - TR(1);
  const TR w4 = ti.dum4 - ival<TR>(ti.dumii) - TR(1);
  const TR w5 = ti.dum5 - ival<TR>(ti.dumjj) - TR(1);
  TR tmp[2];
#pragma unroll
  for (int dj = 0; dj < 2; ++dj) {
    const int jj = ti.dumjj + dj;
    TR v[2];
#pragma unroll
    for (int di = 0; di < 2; ++di) {
      const int ii = ti.dumii + di;
      const TR c00 = coll_at(t, jj, ii, ti.dumi, tr.dumj, idx);
      const TR c10 = coll_at(t, jj, ii, ti.dumi + 1, tr.dumj, idx);
      const TR c01 = coll_at(t, jj, ii, ti.dumi, tr.dumj + 1, idx);
      const TR c11 = coll_at(t, jj, ii, ti.dumi + 1, tr.dumj + 1, idx);
      const TR dproc1 = c00 + w1 * (c10 - c00);
      const TR dproc2 = c01 + w1 * (c11 - c01);
      v[di] = dproc1 + w3 * (dproc2 - dproc1);
    }
    tmp[dj] = v[0] + w4 * (v[1] - v[0]);
  }
  return tmp[0] + w5 * (tmp[1] - tmp[0]);
}

/* lookup (Table3), p3_table3_impl.hpp:14-64.  The mu index is fixed by the
 * constant rain shape parameter and precomputed (rt.t3_dumjj/t3_rdumjj). */
template <class TR>
__device__ __forceinline__ void lookup3(TR mu_r, TR lamr, const RuntimeDev& rt, Table3<TR>& tab) {
  const TR dum1 = (mu_r + TR(1)) / lamr;
  if (dum1 <= TR(195.e-6)) {
    const TR inv_dum3 = TR(0.1);
    TR rdumii = (dum1 * TR(1.e6) + TR(5)) * inv_dum3;
    rdumii = vmax(rdumii, TR(1.0));
    rdumii = vmin(rdumii, TR(20.0));
    int dumii = table_index(rdumii, 20);
    dumii = max(dumii, 1);
    dumii = min(dumii, 20);
    tab.rdumii = rdumii;
    tab.dumii = dumii;
  } else {
    const TR inv_dum3 = TR(C::THIRD * 0.1);
    TR rdumii = (dum1 * TR(1.e+6) - TR(195)) * inv_dum3 + TR(20);
    rdumii = vmax(rdumii, TR(20.0));
    rdumii = vmin(rdumii, TR(300.0));
    int dumii = table_index(rdumii, 300);
    dumii = max(dumii, 20);
    dumii = min(dumii, 299);
    tab.rdumii = rdumii;
    tab.dumii = dumii;
  }
  tab.rdumjj = P3X_RTP(TR, t3_rdumjj);
  tab.dumjj = rt.t3_dumjj;
}

/* apply_table (Table3), p3_table3_impl.hpp:66-83 */
template <class TR>
__device__ __forceinline__ TR apply_table3(const Tabs<TR>& t, const TR* table, const Table3<TR>& t3) {
  const TR rdumii_m_dumii = t3.rdumii - ival<TR>(t3.dumii);
  const TR t_im1_jm1 = t3_at(t, table, t3.dumii - 1, t3.dumjj - 1);
  const TR dum1 = (t_im1_jm1 + rdumii_m_dumii * (t3_at(t, table, t3.dumii, t3.dumjj - 1) - t_im1_jm1));
  const TR t_im1_j = t3_at(t, table, t3.dumii - 1, t3.dumjj);
  const TR dum2 = (t_im1_j + rdumii_m_dumii * (t3_at(t, table, t3.dumii, t3.dumjj) - t_im1_j));
  return dum1 + (t3.rdumjj - ival<TR>(t3.dumjj)) * (dum2 - dum1);
}

/* ------------------------------------------------------------------ */
/* In-cloud values and DSD                                              */
/* ------------------------------------------------------------------ */

/* calculate_incloud_mixingratios, p3/impl/p3_incloud_mixingratios_impl.hpp:12-69
 * (bm_incld uses inv_cld_frac_l, line 49).  FP64. */
struct Incld {
  double qc, qr, qi, qm, nc, nr, ni, bm;
};
__device__ __forceinline__ void calc_incloud(double qc, double qr, double qi, double qm, double nc,
                                             double nr, double ni, double bm, double inv_cld_l,
                                             double inv_cld_i, double inv_cld_r, Incld& o) {
  if (dge(qc, C::QSMALL)) { o.qc = qc * inv_cld_l; o.nc = dmax0(nc * inv_cld_l); }
  else { o.qc = 0; o.nc = 0; }
  if (dge(qi, C::QSMALL)) { o.qi = qi * inv_cld_i; o.ni = dmax0(ni * inv_cld_i); }
  else { o.qi = 0; o.ni = 0; }
  if (dge(qi, C::QSMALL) && dge(qm, C::QSMALL)) { o.qm = qm * inv_cld_i; o.bm = dmax0(bm * inv_cld_l); }
  else { o.qm = 0; o.bm = 0; }
  if (dge(qr, C::QSMALL)) { o.qr = qr * inv_cld_r; o.nr = dmax0(nr * inv_cld_r); }
  else { o.qr = 0; o.nr = 0; }
  if (dgt(o.qc, C::incloud_limit) || dgt(o.qi, C::incloud_limit) || dgt(o.qr, C::precip_limit) ||
      dgt(o.bm, C::incloud_limit)) {
    o.qc = dmin_c(o.qc, C::incloud_limit);
    o.qi = dmin_c(o.qi, C::incloud_limit);
    o.bm = dmin_c(o.bm, C::incloud_limit);
    o.qr = dmin_c(o.qr, C::precip_limit);
  }
}

/* get_cloud_dsd2, p3/impl/p3_dsd2_impl.hpp:14-74 (iparam = 3).  The
 * spectral moments cdist (used only by the inactive cloud relaxation time
 * epsc) and cdist1 = nc/Gamma(mu_c+1) (immersion freezing, evaluated there
 * with the Gamma recurrence) are not needed by any output. */
template <class TR>
__device__ __forceinline__ void get_cloud_dsd2(TR qc, TR& nc, TR& mu_c, TR rho, TR& lamc) {
  lamc = 0; mu_c = 0;
  if (qc >= TR(C::QSMALL)) {
    nc = vmax(nc, TR(C::NSMALL));
    TR mu = TR(0.0005714) * (nc * TR(1.e-6) * rho) + TR(0.2714);
    mu = TR(1) / (mu * mu) - TR(1);
    mu = vmax(mu, TR(2.));
    mu = vmin(mu, TR(15.));
    mu_c = mu;
    lamc = m_cbrt(TR(C::CONS1) * nc * (mu_c + TR(3)) * (mu_c + TR(2)) * (mu_c + TR(1)) / qc);
    const TR lammin = (mu_c + TR(1)) * TR(2.5e+4);
    const TR lammax = (mu_c + TR(1)) * TR(1.e+6);
    const bool lt = lamc < lammin, gt = lamc > lammax;
    if (lt) lamc = lammin;
    if (gt) lamc = lammax;
    if (lt || gt) {
      nc = TR(6) * (lamc * lamc * lamc) * qc /
           (TR(C::Pi) * TR(C::RHO_H2O) * (mu_c + TR(3)) * (mu_c + TR(2)) * (mu_c + TR(1)));
    }
  }
}

/* get_rain_dsd2, p3_dsd2_impl.hpp:76-126 */
template <class TR>
__device__ __forceinline__ void get_rain_dsd2(TR qr, TR& nr, TR& mu_r, TR& lamr, const RuntimeDev& rt) {
  lamr = 0;
  if (qr >= TR(C::QSMALL)) {
    const TR nr_lim = vmax(nr, TR(C::NSMALL));
    mu_r = P3X_RTP(TR, constant_mu_rain);
    const TR f = TR(C::CONS1) * (mu_r + TR(3)) * (mu_r + TR(2)) * (mu_r + TR(1));
    lamr = m_cbrt(f * nr_lim / qr);
    const TR lammax = (mu_r + TR(1.)) * TR(1.e+5);
    const TR lammin = (mu_r + TR(1.)) * TR(500);
    const bool lt = lamr < lammin, gt = lamr > lammax;
    nr = nr_lim;
    if (lt || gt) {
      if (lt) lamr = lammin;
      if (gt) lamr = lammax;
      nr = lamr * lamr * lamr * qr / f;
    }
  }
}

/* impose_max_total_ni, p3_impose_max_total_ni_impl.hpp:9-27 */
template <class T>
__device__ __forceinline__ void impose_max_total_ni(T& ni_local, T max_total_ni, T inv_rho_local) {
  if (ni_local >= T(1e-20)) ni_local = ni_local * vmin(max_total_ni * inv_rho_local / ni_local, T(1.));
}

/* calc_bulk_rho_rime, p3/impl/p3_ice_sed_impl.hpp:14-64 */
template <class T>
__device__ __forceinline__ T calc_bulk_rho_rime(T qi_tot, T& qi_rim, T& bi_rim, const RuntimeDev& rt) {
  T rho_rime = 0;
  const bool gt = bi_rim >= T(C::BSMALL);
  const bool lt = bi_rim < T(C::BSMALL);
  if (gt) rho_rime = qi_rim / bi_rim;
  const bool rr_lt_min = rho_rime < P3X_RTP(T, min_rime_rho);
  const bool rr_gt_max = rho_rime > P3X_RTP(T, max_rime_rho);
  if (gt && rr_lt_min) rho_rime = P3X_RTP(T, min_rime_rho);
  if (gt && rr_gt_max) rho_rime = P3X_RTP(T, max_rime_rho);
  if (gt && (rr_gt_max || rr_lt_min)) bi_rim = qi_rim / rho_rime;
  if (lt) { qi_rim = 0; bi_rim = 0; rho_rime = 0; }
  if (qi_rim > qi_tot && rho_rime > T(0)) { qi_rim = qi_tot; bi_rim = qi_rim / rho_rime; }
  if (qi_rim < T(C::QSMALL)) { qi_rim = 0; bi_rim = 0; }
  return rho_rime;
}

/* ------------------------------------------------------------------ */
/* Process rates (all in-cloud, TR)                                    */
/* ------------------------------------------------------------------ */
template <class TR>
struct Rates {
  TR qc2qr_accret_tend, qr2qv_evap_tend, qc2qr_autoconv_tend, nc_accret_tend, nc_selfcollect_tend,
      nc2nr_autoconv_tend, nr_selfcollect_tend, nr_evap_tend, ncautr, qi2qv_sublim_tend,
      nr_ice_shed_tend, qc2qi_hetero_freeze_tend, qr2qi_collect_tend, qc2qr_ice_shed_tend,
      qi2qr_melt_tend, qc2qi_collect_tend, qr2qi_immers_freeze_tend, qv2qi_nucleat_tend,
      ni2nr_melt_tend, nc_collect_tend, ncshdc, nc2ni_immers_freeze_tend, nr_collect_tend,
      ni_selfcollect_tend, ni_nucleat_tend, qv2qi_vapdep_tend, qc2qi_berg_tend,
      nr2ni_immers_freeze_tend, ni_sublim_tend;
  __device__ __forceinline__ void zero() {
    qc2qr_accret_tend = qr2qv_evap_tend = qc2qr_autoconv_tend = nc_accret_tend = nc_selfcollect_tend =
        nc2nr_autoconv_tend = nr_selfcollect_tend = nr_evap_tend = ncautr = qi2qv_sublim_tend =
            nr_ice_shed_tend = qc2qi_hetero_freeze_tend = qr2qi_collect_tend = qc2qr_ice_shed_tend =
                qi2qr_melt_tend = qc2qi_collect_tend = qr2qi_immers_freeze_tend = qv2qi_nucleat_tend =
                    ni2nr_melt_tend = nc_collect_tend = ncshdc = nc2ni_immers_freeze_tend =
                        nr_collect_tend = ni_selfcollect_tend = ni_nucleat_tend = qv2qi_vapdep_tend =
                            qc2qi_berg_tend = nr2ni_immers_freeze_tend = ni_sublim_tend = TR(0);
  }
};

/* get_time_space_phys_variables, p3_get_time_space_phys_variables_impl.hpp:12-45 */
template <class TR>
struct PhysVars {
  TR mu, dv, sc, dqsdt, dqsidt, ab, abi, kap, eii;
};
template <class TR>
__device__ __forceinline__ void get_time_space_phys_variables(TR T_atm, TR pres, TR rho, TR qv_sat_l,
                                                              TR qv_sat_i, PhysVars<TR>& v) {
  v.mu = TR(1.496e-6) * m_pow(T_atm, TR(1.5)) / (T_atm + TR(120));
  v.dv = TR(8.794e-5) * m_pow(T_atm, TR(1.81)) / pres;
  v.sc = v.mu / (rho * v.dv);
  const TR dum = TR(1) / (TR(C::RV) * sq(T_atm));
  v.dqsdt = TR(C::LatVap) * qv_sat_l * dum;
  v.dqsidt = TR(C::LatVap + C::LatIce) * qv_sat_i * dum;
  v.ab = TR(1) + v.dqsdt * TR(C::LatVap) * TR(C::INV_CP);
  v.abi = TR(1) + v.dqsidt * TR(C::LatVap + C::LatIce) * TR(C::INV_CP);
  v.kap = TR(1.414e+3) * v.mu;
  if (T_atm < TR(253.15)) {
    v.eii = TR(0.001);
  } else if (T_atm < TR(273.15)) {
    v.eii = TR(0.001) + (T_atm - TR(253.15)) * (TR(0.3) - TR(0.001)) / TR(20);
  } else {
    v.eii = TR(0.3);
  }
}

/* ice_cldliq_collection, p3/impl/p3_ice_collection_impl.hpp:9-52 */
template <class TR>
__device__ __forceinline__ void ice_cldliq_collection(TR rho, double temp, TR rhofaci, TR tv, TR qi_incld,
                                                      TR qc_incld, TR ni_incld, TR nc_incld,
                                                      Rates<TR>& r, const RuntimeDev& rt) {
  const bool t_neg = dle(temp, C::Tmelt);
  const bool both = qi_incld >= TR(C::QSMALL) && qc_incld >= TR(C::QSMALL);
  const TR f = P3X_RTP(TR, cldliq_to_ice_collection_factor);
  if (both && t_neg) r.qc2qi_collect_tend = rhofaci * tv * qc_incld * f * rho * ni_incld;
  if (both) r.nc_collect_tend = rhofaci * tv * nc_incld * f * rho * ni_incld;
  if (both && !t_neg) {
    r.qc2qr_ice_shed_tend = rhofaci * tv * qc_incld * f * rho * ni_incld;
    r.nc_collect_tend = rhofaci * tv * nc_incld * f * rho * ni_incld;
    r.ncshdc = r.qc2qr_ice_shed_tend * TR(1.0 / C::dropmass);
  }
}

/* ice_rain_collection, p3_ice_collection_impl.hpp:54-101 */
template <class TR>
__device__ __forceinline__ void ice_rain_collection(TR rho, double temp, TR rhofaci, TR logn0r, TR tv_nr,
                                                    TR tv_qr, TR qi_incld, TR ni_incld, TR qr_incld,
                                                    Rates<TR>& r, const RuntimeDev& rt) {
  const bool t_neg = dle(temp, C::Tmelt);
  const bool both = qi_incld >= TR(C::QSMALL) && qr_incld >= TR(C::QSMALL);
  const TR f = P3X_RTP(TR, rain_to_ice_collection_factor);
  if (both && t_neg) {
    r.qr2qi_collect_tend = m_pow(TR(10.0), tv_qr + logn0r) * rho * rhofaci * f * ni_incld;
    r.nr_collect_tend = m_pow(TR(10.0), tv_nr + logn0r) * rho * rhofaci * f * ni_incld;
  }
  if (both && !t_neg) r.nr_collect_tend = m_pow(TR(10.0), tv_nr + logn0r) * rho * rhofaci * f * ni_incld;
}

/* ice_self_collection, p3_ice_collection_impl.hpp:103-152 */
template <class TR>
__device__ __forceinline__ void ice_self_collection(TR rho, TR rhofaci, TR tv, TR eii, TR qm_incld,
                                                    TR qi_incld, TR ni_incld, Rates<TR>& r) {
  const bool qm_pos = qm_incld > TR(0);
  if (qi_incld >= TR(C::QSMALL)) {
    TR tmp1 = 0;
    if (qm_pos) tmp1 = qm_incld / qi_incld;
    TR Eii_fact = 0;
    if (tmp1 < TR(0.6) && qm_pos) Eii_fact = TR(1);
    if (tmp1 >= TR(0.6) && tmp1 < TR(0.9) && qm_pos) Eii_fact = TR(1) - (tmp1 - TR(0.6)) / TR(0.3);
    if (tmp1 >= TR(0.9) && qm_pos) Eii_fact = TR(0);
    if (!qm_pos) Eii_fact = TR(1);
    r.ni_selfcollect_tend = tv * rho * eii * Eii_fact * rhofaci * ni_incld * ni_incld;
  }
}

/* ice_melting, p3/impl/p3_ice_melting_impl.hpp:10-53 (max(...,0) inside the branch) */
/* The departures dT0 = T - T_0C and dqv0 = qsat(T_0C) - qv are formed in FP64
 * by the caller (small differences of large numbers near the melting point). */
template <class TR>
__device__ __forceinline__ void ice_melting(TR rho, double dT0, double dqv0, TR rhofaci, TR tv_melt,
                                            TR tv_vent, const PhysVars<TR>& v, TR qi_incld,
                                            TR ni_incld, Rates<TR>& r) {
  if (qi_incld >= TR(C::QSMALL) && dpos(dT0)) {
    TR t = ((tv_melt + tv_vent * m_cbrt(v.sc) * m_sqrt(rhofaci * rho / v.mu)) *
            (TR(dT0) * v.kap - rho * TR(C::LatVap) * v.dv * TR(dqv0)) * TR(2) *
            TR(C::Pi) / TR(C::LatIce)) *
           ni_incld;
    t = vmax(t, TR(0.));
    r.qi2qr_melt_tend = t;
    r.ni2nr_melt_tend = t * (ni_incld / qi_incld);
  }
}

/* ice_cldliq_wet_growth, p3/impl/p3_ice_cldliq_wet_growth_impl.hpp:12-80 */
template <class TR>
__device__ __forceinline__ bool ice_cldliq_wet_growth(TR rho, double dT0, double dqv0, TR rhofaci, TR tv_melt,
                                                      TR tv_vent, const PhysVars<TR>& v,
                                                      TR qc_incld, TR qi_incld, TR ni_incld, TR qr_incld,
                                                      Rates<TR>& r) {
  const bool t_neg = dneg(dT0);
  const bool any_if = qi_incld >= TR(C::QSMALL) && (qc_incld + qr_incld) >= TR(1.0e-6) && t_neg;
  const bool any_if_col = any_if && (r.qc2qi_collect_tend + r.qr2qi_collect_tend) >= TR(1.0e-10);
  bool wet = false;
  if (any_if) {
    TR g = ((tv_melt + tv_vent * m_cbrt(v.sc) * m_sqrt(rhofaci * rho / v.mu)) * TR(C::Pi * 2) *
            (rho * TR(C::LatVap) * v.dv * TR(dqv0) - TR(dT0) * v.kap) /
            (TR(C::LatIce) + TR(C::CpLiq) * TR(dT0))) *
           ni_incld;
    g = vmax(g, TR(0.));
    /* The shed excess dum = collection - g and the collection that remains,
     * c - dum * c / (qc2qi + qr2qi), cancel almost completely when the
     * collection rate exceeds the wet-growth limit by orders of magnitude;
     * they are evaluated in FP64 (the FP64 form is unchanged by this). */
    const double qc2qi = widen(r.qc2qi_collect_tend), qr2qi = widen(r.qr2qi_collect_tend);
    const double dum = dmax_0x((qc2qi + qr2qi) - widen(g));
    const bool dum_ge_small = dge(dum, 1.0e-10);
    if (dum_ge_small) {
      r.nr_ice_shed_tend = TR(widen(r.nr_ice_shed_tend) + dum * 1.923e+6);
      const double dum1 = 1.0 / (qc2qi + qr2qi);
      if (any_if_col) {
        r.qc2qr_ice_shed_tend = TR(widen(r.qc2qr_ice_shed_tend) + dum * qc2qi * dum1);
        r.qc2qi_collect_tend = TR(dmax_0x(qc2qi - dum * qc2qi * dum1));
        r.qr2qi_collect_tend = TR(dmax_0x(qr2qi - dum * qr2qi * dum1));
      }
    }
    wet = dum_ge_small;
  }
  return wet;
}

/* calc_rime_density, p3/impl/p3_calc_rime_density_impl.hpp:13-70 */
template <class TR>
__device__ __forceinline__ TR calc_rime_density(TR T_atm, TR rhofaci, TR tv_fallspd, TR acn, TR lamc,
                                                TR mu_c, TR qc_incld, TR qc2qi_collect_tend) {
  TR rho_qm_cloud = TR(400);
  if (qc2qi_collect_tend >= TR(C::QSMALL) && T_atm < TR(C::T_zerodegc)) {
    const TR vtrmi1 = tv_fallspd * rhofaci;
    if (qc_incld >= TR(C::QSMALL)) {
      /* Gamma(4+bcn+mu_c)/Gamma(4+mu_c) = (5+mu_c)(4+mu_c) for bcn = 2 */
      const TR Vt_qc = acn * ((TR(5) + mu_c) * (TR(4) + mu_c)) / (lamc * lamc);
      const TR D_c = (TR(4) + mu_c) / lamc;
      const TR V_impact = m_fabs(vtrmi1 - Vt_qc);
      const TR inv_Tc = TR(1) / vmin(TR(-0.001), T_atm - TR(C::T_zerodegc));
      const TR Ri = vmax(TR(1.), vmin(TR(-0.5e+6) * D_c * V_impact * inv_Tc, TR(12.)));
      if (Ri <= TR(8.0)) {
        rho_qm_cloud = (TR(0.051) + TR(0.114) * Ri - TR(0.0055) * sq(Ri)) * TR(1000);
      } else {
        rho_qm_cloud = TR(611.) + TR(72.25) * (Ri - TR(8));
      }
    }
  }
  return rho_qm_cloud;
}

/* cldliq_immersion_freezing, p3/impl/p3_cldliq_imm_freezing_impl.hpp:13-50.
 * cdist1 * Gamma(7+mu_c) and cdist1 * Gamma(4+mu_c), with cdist1 =
 * nc/Gamma(mu_c+1) (p3_dsd2_impl.hpp:72), are evaluated as nc times the
 * rising products (1+mu)...(6+mu) and (1+mu)(2+mu)(3+mu). */
template <class TR>
__device__ __forceinline__ void cldliq_immersion_freezing(TR T_atm, TR lamc, TR mu_c, TR nc_incld, TR qc_incld,
                                                          Rates<TR>& r, const RuntimeDev& rt) {
  if (qc_incld >= TR(C::QSMALL) && T_atm <= TR(C::T_rainfrz)) {
    const TR expAimmDt = m_exp(P3X_RTP(TR, immersion_freezing_exponent) * (TR(C::T_zerodegc) - T_atm));
    const TR inv_lamc = TR(1) / lamc;
    const TR inv_lamc3 = inv_lamc * inv_lamc * inv_lamc;
    const TR p3 = (TR(1) + mu_c) * (TR(2) + mu_c) * (TR(3) + mu_c);
    const TR p6 = p3 * ((TR(4) + mu_c) * (TR(5) + mu_c) * (TR(6) + mu_c));
    if constexpr (sizeof(TR) == sizeof(double)) {
      r.qc2qi_hetero_freeze_tend = TR(C::CONS6) * (nc_incld * p6) * expAimmDt * sq(inv_lamc3);
    } else {
      /* (1/lamc)^6 underflows single precision: multiply it in twice */
      r.qc2qi_hetero_freeze_tend = TR(C::CONS6) * (nc_incld * p6) * expAimmDt * inv_lamc3 * inv_lamc3;
    }
    r.nc2ni_immers_freeze_tend = TR(C::CONS5) * (nc_incld * p3) * expAimmDt * inv_lamc3;
  }
}

/* rain_immersion_freezing, p3/impl/p3_rain_imm_freezing_impl.hpp:13-44 */
template <class TR>
__device__ __forceinline__ void rain_immersion_freezing(TR T_atm, TR lamr, TR mu_r, TR cdistr, TR qr_incld,
                                                        Rates<TR>& r, const RuntimeDev& rt) {
  if (qr_incld >= TR(C::QSMALL) && T_atm <= TR(C::T_rainfrz)) {
    const TR e = m_exp(P3X_RTP(TR, immersion_freezing_exponent) * (TR(C::T_zerodegc) - T_atm));
    /* mu_r is the runtime constant here: log(Gamma(7+mu_r)) and
     * log(Gamma(4+mu_r)) are precomputed on the host */
    (void)mu_r;
    r.qr2qi_immers_freeze_tend =
        TR(C::CONS6) * m_exp(m_log(cdistr) + P3X_RTP(TR, lg_mur7) - TR(6.) * m_log(lamr)) * e;
    r.nr2ni_immers_freeze_tend =
        TR(C::CONS5) * m_exp(m_log(cdistr) + P3X_RTP(TR, lg_mur4) - TR(3.) * m_log(lamr)) * e;
  }
}

/* ice_nucleation, p3/impl/p3_ice_nucleation_impl.hpp:9-61 */
template <class TR>
__device__ __forceinline__ void ice_nucleation(TR temp, TR inv_rho, TR ni, TR ni_activated, double qv_supersat_i,
                                               TR inv_dt, bool do_predict_nc, bool do_prescribed_CCN,
                                               Rates<TR>& r, const RuntimeDev& rt) {
  const TR mi0 = TR(4.0 * C::PIOV3 * 900.0 * 1.e-18);
  const bool do_log = (!do_predict_nc || do_prescribed_CCN);
  const bool base = temp < TR(C::Tmelt - 15.0) && qv_supersat_i >= 0.05;
  if (base && do_log) {
    TR dum = TR(0.005) * m_exp(P3X_RTP(TR, deposition_nucleation_exponent) * (TR(C::Tmelt) - temp)) * TR(1.0e3) * inv_rho;
    dum = vmin(dum, TR(1.0e5) * inv_rho);
    const TR N_nuc = vmax(TR(0.), (dum - ni) * inv_dt);
    if (N_nuc >= TR(C::NSMALL)) {
      const TR Q_nuc = vmax(TR(0.), (dum - ni) * mi0 * inv_dt);
      r.qv2qi_nucleat_tend = Q_nuc;
      r.ni_nucleat_tend = N_nuc;
    }
  } else if (base && !do_log) {
    r.ni_nucleat_tend = vmax(TR(0.), (ni_activated - ni) * inv_dt);
    r.qv2qi_nucleat_tend = r.ni_nucleat_tend * mi0;
  }
}

/* cloud_water_autoconversion, p3/impl/p3_autoconversion_impl.hpp:9-58 */
template <class TR>
__device__ __forceinline__ void cloud_water_autoconversion(TR rho, TR qc_incld, TR nc_incld, Rates<TR>& r,
                                                           const RuntimeDev& rt) {
  if (qc_incld >= TR(1e-8)) {
    r.qc2qr_autoconv_tend = P3X_RTP(TR, autoconversion_prefactor) * m_pow(qc_incld, P3X_RTP(TR, autoconversion_qc_exponent)) *
                            m_pow(nc_incld * TR(1.e-6) * rho, (-P3X_RTP(TR, autoconversion_nc_exponent)));
    r.ncautr = r.qc2qr_autoconv_tend * P3X_RTP(TR, cons3);
    r.nc2nr_autoconv_tend = r.qc2qr_autoconv_tend * nc_incld / qc_incld;
  }
  if (r.qc2qr_autoconv_tend == TR(0)) r.nc2nr_autoconv_tend = 0;
  if (r.nc2nr_autoconv_tend == TR(0)) r.qc2qr_autoconv_tend = 0;
}

/* cloud_rain_accretion, p3/impl/p3_cloud_rain_acc_impl.hpp:14-55 */
template <class TR>
__device__ __forceinline__ void cloud_rain_accretion(TR qc_incld, TR nc_incld, TR qr_incld, Rates<TR>& r,
                                                     const RuntimeDev& rt) {
  if (qr_incld >= TR(C::QSMALL) && qc_incld >= TR(C::QSMALL)) {
    if (rt.accretion_same_exponent) {
      r.qc2qr_accret_tend = P3X_RTP(TR, accretion_prefactor) * m_pow(qc_incld * qr_incld, P3X_RTP(TR, accretion_qr_exponent));
    } else {
      r.qc2qr_accret_tend = P3X_RTP(TR, accretion_prefactor) * m_pow(qc_incld, P3X_RTP(TR, accretion_qc_exponent)) *
                            m_pow(qr_incld, P3X_RTP(TR, accretion_qr_exponent));
    }
    r.nc_accret_tend = r.qc2qr_accret_tend * nc_incld / qc_incld;
    if (r.nc_accret_tend == TR(0)) r.qc2qr_accret_tend = 0;
    if (r.qc2qr_accret_tend == TR(0)) r.nc_accret_tend = 0;
  }
}

/* rain_self_collection, p3/impl/p3_rain_self_collection_impl.hpp:9-56 */
template <class TR>
__device__ __forceinline__ void rain_self_collection(TR rho, TR qr_incld, TR nr_incld, Rates<TR>& r,
                                                     const RuntimeDev& rt) {
  if (qr_incld >= TR(C::QSMALL)) {
    const TR dum2 = m_cbrt((qr_incld) / (TR(C::Pi) * TR(C::RHO_H2O) * nr_incld));
    const TR dbr = P3X_RTP(TR, rain_selfcollection_breakup_diameter);
    const TR dum = (dum2 < dbr) ? TR(1) : TR(2) - m_exp(TR(2300) * (dum2 - dbr));
    r.nr_selfcollect_tend = dum * P3X_RTP(TR, rain_selfcollection_prefactor) * nr_incld * qr_incld * rho;
  }
}

/* back_to_cell_average, p3/impl/p3_back_to_cell_average_impl.hpp:14-77 */
template <class TR>
__device__ __forceinline__ void back_to_cell_average(TR cld_l, TR cld_r, TR cld_i, Rates<TR>& r) {
  const TR ir = vmin(cld_i, cld_r), il = vmin(cld_i, cld_l), lr = vmin(cld_l, cld_r);
  r.qc2qr_accret_tend *= lr;
  r.qr2qv_evap_tend *= cld_r;
  r.qc2qr_autoconv_tend *= cld_l;
  r.nc_accret_tend *= lr;
  r.nc_selfcollect_tend *= cld_l;
  r.nc2nr_autoconv_tend *= cld_l;
  r.nr_selfcollect_tend *= cld_r;
  r.nr_evap_tend *= cld_r;
  r.ncautr *= lr;
  r.qi2qv_sublim_tend *= cld_i;
  r.nr_ice_shed_tend *= il;
  r.qc2qi_hetero_freeze_tend *= il;
  r.qr2qi_collect_tend *= ir;
  r.qc2qr_ice_shed_tend *= il;
  r.qi2qr_melt_tend *= cld_i;
  r.qc2qi_collect_tend *= il;
  r.qr2qi_immers_freeze_tend *= cld_r;
  r.ni2nr_melt_tend *= cld_i;
  r.nc_collect_tend *= il;
  r.ncshdc *= il;
  r.nc2ni_immers_freeze_tend *= cld_l;
  r.nr_collect_tend *= ir;
  r.ni_selfcollect_tend *= cld_i;
  r.qv2qi_vapdep_tend *= cld_i;
  r.nr2ni_immers_freeze_tend *= cld_r;
  r.ni_sublim_tend *= cld_i;
  r.qc2qi_berg_tend *= il;
}


/* ------------------------------------------------------------------ */
/* FP64 residual routines                                               */
/* ------------------------------------------------------------------ */

/* evaporate_rain, p3/impl/p3_evaporate_rain_impl.hpp:9-203.  The
 * supersaturation residual and the A_c source term are FP64; the
 * relaxation coefficients come in from the rate precision. */
__device__ __forceinline__ void evaporate_rain(double qr_incld, double qc_incld, double nr_incld,
                                               double qi_incld, double cld_frac_l, double cld_frac_r,
                                               double qv, double qv_prev, double qv_sat_l, double qv_sat_i,
                                               double ab, double abi, double epsr, double epsi_tot,
                                               double t_atm, double t_atm_prev, double dqsdt, double dt,
                                               double& qr2qv_evap_tend, double& nr_evap_tend) {
  qr2qv_evap_tend = 0;
  nr_evap_tend = 0;
  const double inv_dt = 1 / dt;
  const double inv_cp = 1 / C::Cpair;
  const double ssat_r = qv - qv_sat_l;
  const double cld_frac = ((qc_incld + qi_incld) < 1.e-6) ? 0.0 : cld_frac_l;
  if (qr_incld >= C::QSMALL && ssat_r < 0 && cld_frac_r > cld_frac) {
    const double tau_r = 1 / epsr;
    double eps_eff, A_c;
    if (t_atm < C::Tmelt) {
      eps_eff = epsr + epsi_tot * (1 + (C::LatVap + C::LatIce) * inv_cp * dqsdt) / abi;
      A_c = (qv - qv_prev) * inv_dt - dqsdt * (t_atm - t_atm_prev) * inv_dt -
            (qv_sat_l - qv_sat_i) * (1 + (C::LatVap + C::LatIce) * inv_cp * dqsdt) / abi * epsi_tot;
    } else {
      eps_eff = epsr;
      A_c = (qv - qv_prev) * inv_dt - dqsdt * (t_atm - t_atm_prev) * inv_dt;
    }
    if (eps_eff < 1e-20) eps_eff = 1e-20;
    const double tau_eff = 1 / eps_eff;
    if (qr_incld < 1e-12 && qv / qv_sat_l < 0.999) {
      qr2qv_evap_tend = qr_incld * inv_dt;
    } else {
      const double dt_over_tau = dt / tau_eff;
      const double w = -expm1(-dt_over_tau) / dt_over_tau;
      const double equilib = -A_c / ab * tau_eff / tau_r;
      const double instant = -ssat_r / (ab * tau_r);
      qr2qv_evap_tend = instant * w + equilib * (1 - w);
    }
    if (qr2qv_evap_tend > -ssat_r * inv_dt / ab) qr2qv_evap_tend = -ssat_r * inv_dt / ab;
    if (qr2qv_evap_tend < 0) qr2qv_evap_tend = 0;
    if (qr2qv_evap_tend > qr_incld * inv_dt) qr2qv_evap_tend = qr_incld * inv_dt;
    qr2qv_evap_tend = qr2qv_evap_tend * (cld_frac_r - cld_frac) / cld_frac_r;
    nr_evap_tend = qr2qv_evap_tend * (nr_incld / qr_incld);
  }
}

/* evaporate_rain of the FP32-bulk form: the supersaturation residual
 * ssat_r = qv - qv_sat_l and the A_c source term (differences of the state
 * against the previous step) are formed in FP64; the in-cloud values, the
 * relaxation weights, the equilibrium / instantaneous tendencies and the
 * limits are rate arithmetic in FP32.  Same formulas and branch order as
 * evaporate_rain. */
__device__ __forceinline__ void evaporate_rain_bulk(float qr_incld, float qc_incld, float nr_incld,
                                                    float qi_incld, float cld_frac_l, float cld_frac_r,
                                                    double qv, double qv_prev, double qv_sat_l, double qv_sat_i,
                                                    float ab, float abi, float epsr, float epsi_tot,
                                                    double t_atm, double t_atm_prev, float dqsdt, float dtf,
                                                    float inv_dt, double inv_dt_d, float& qr2qv_evap_tend,
                                                    float& nr_evap_tend) {
  qr2qv_evap_tend = 0;
  nr_evap_tend = 0;
  const double ssat_r_d = qv - qv_sat_l;
  const float cld_frac = ((qc_incld + qi_incld) < 1.e-6f) ? 0.0f : cld_frac_l;
  if (qr_incld >= float(C::QSMALL) && dneg(ssat_r_d) && cld_frac_r > cld_frac) {
    const float ssat_r = float(ssat_r_d);
    const float tau_r = 1.0f / epsr;
    const float lat_fac = 1.0f + float((C::LatVap + C::LatIce) / C::Cpair) * dqsdt;
    float eps_eff;
    double A_c_d = (qv - qv_prev) * inv_dt_d - f2d(dqsdt) * (t_atm - t_atm_prev) * inv_dt_d;
    if (dlt(t_atm, C::Tmelt)) {
      eps_eff = epsr + epsi_tot * lat_fac / abi;
      A_c_d -= (qv_sat_l - qv_sat_i) * f2d(lat_fac / abi * epsi_tot);
    } else {
      eps_eff = epsr;
    }
    const float A_c = float(A_c_d);
    if (eps_eff < 1e-20f) eps_eff = 1e-20f;
    const float tau_eff = 1.0f / eps_eff;
    float evap;
    if (qr_incld < 1e-12f && qv < 0.999 * qv_sat_l) {
      evap = qr_incld * inv_dt;
    } else {
      const float dt_over_tau = dtf / tau_eff;
      const float w = -expm1f(-dt_over_tau) / dt_over_tau;
      const float equilib = -A_c / ab * tau_eff / tau_r;
      const float instant = -ssat_r / (ab * tau_r);
      evap = instant * w + equilib * (1.0f - w);
    }
    const float lim = -ssat_r * inv_dt / ab;
    if (evap > lim) evap = lim;
    if (evap < 0.0f) evap = 0.0f;
    const float qlim = qr_incld * inv_dt;
    if (evap > qlim) evap = qlim;
    evap = evap * ((cld_frac_r - cld_frac) / cld_frac_r);
    qr2qv_evap_tend = evap;
    nr_evap_tend = evap * (nr_incld / qr_incld);
  }
}

/* ice_deposition_sublimation of the FP32-bulk form: the vapour residuals
 * qv - qv_sat_i and qv_sat_l - qv_sat_i are FP64, the in-cloud values and the
 * relaxation coefficient FP32. */
__device__ __forceinline__ void ice_deposition_sublimation_bulk(float qi_incld, float ni_incld, double T_atm,
                                                                double qv_sat_l, double qv_sat_i, float epsi,
                                                                float abi, double qv, float inv_dt,
                                                                float& vapdep, float& sublim, float& ni_sublim,
                                                                float& berg) {
  berg = 0; vapdep = 0; sublim = 0; ni_sublim = 0;
  if (qi_incld > float(C::QSMALL)) {
    const float coef = vmin(epsi / abi, inv_dt);
    const float qi_tend = coef * float(qv - qv_sat_i);
    const bool neg = qi_tend < 0;
    if (neg) {
      sublim = -qi_tend;
      ni_sublim = sublim * (ni_incld / qi_incld);
    }
    const bool T_lt_frz = dlt(T_atm, C::T_zerodegc);
    if (T_lt_frz && !neg) vapdep = qi_tend;
    if (T_lt_frz) berg = vmax(epsi / abi * float(qv_sat_l - qv_sat_i), 0.0f);
  }
}

/* ice_deposition_sublimation, p3/impl/p3_ice_deposition_sublimation_impl.hpp:9-65
 * (the vapour residual qv - qv_sat is FP64). */
__device__ __forceinline__ void ice_deposition_sublimation(double qi_incld, double ni_incld, double T_atm,
                                                           double qv_sat_l, double qv_sat_i, double epsi,
                                                           double abi, double qv, double inv_dt,
                                                           double& vapdep, double& sublim, double& ni_sublim,
                                                           double& berg) {
  berg = 0; vapdep = 0; sublim = 0; ni_sublim = 0;
  if (dgt(qi_incld, C::QSMALL)) {
    const double qi_tend = vmin(epsi / abi, inv_dt) * (qv - qv_sat_i);
    const bool neg = dneg(qi_tend);
    if (neg) {
      sublim = -qi_tend;
      ni_sublim = sublim * (ni_incld / qi_incld);
    }
    const bool T_lt_frz = dlt(T_atm, C::T_zerodegc);
    if (T_lt_frz && !neg) vapdep = qi_tend;
    if (T_lt_frz) berg = dmax0(epsi / abi * (qv_sat_l - qv_sat_i));
  }
}

/* cloud/rain/ice water conservation, p3/impl/p3_conservation_impl.hpp:9-98
 * (T = double in the plain form; float in the FP32-bulk form, where the
 * limiters only scale rates and the state update stays water-conserving). */
template <class T>
__device__ __forceinline__ int water_conservation(T qc, T qr, T qi, T dt, Rates<T>& r) {
  int limited = 0;
  {
    const T sinks = (r.qc2qr_autoconv_tend + r.qc2qr_accret_tend + r.qc2qi_collect_tend +
                          r.qc2qi_hetero_freeze_tend + r.qc2qr_ice_shed_tend + r.qc2qi_berg_tend) * dt;
    const T sources = qc;
    T ratio;
    if (sinks > sources && sinks >= T(C::QTENDSMALL)) {
      limited |= 1;
      ratio = sources / sinks;
      r.qc2qr_autoconv_tend *= ratio;
      r.qc2qr_accret_tend *= ratio;
      r.qc2qi_collect_tend *= ratio;
      r.qc2qi_hetero_freeze_tend *= ratio;
      r.qc2qr_ice_shed_tend *= ratio;
      r.qc2qi_berg_tend *= ratio;
    } else {
      ratio = T(1);
    }
    if (sources > T(C::QTENDSMALL)) {
      r.qv2qi_vapdep_tend *= (T(1) - ratio);
      r.qi2qv_sublim_tend *= (T(1) - ratio);
    }
  }
  {
    const T sinks = (r.qr2qv_evap_tend + r.qr2qi_collect_tend + r.qr2qi_immers_freeze_tend) * dt;
    const T sources = qr + (r.qc2qr_autoconv_tend + r.qc2qr_accret_tend + r.qi2qr_melt_tend +
                                 r.qc2qr_ice_shed_tend) * dt;
    if (sinks > sources && sinks >= T(C::QTENDSMALL)) {
      limited |= 2;
      const T ratio = sources / sinks;
      r.qr2qv_evap_tend *= ratio;
      r.qr2qi_collect_tend *= ratio;
      r.qr2qi_immers_freeze_tend *= ratio;
    }
  }
  {
    const T sinks = (r.qi2qv_sublim_tend + r.qi2qr_melt_tend) * dt;
    const T sources = qi + (r.qv2qi_vapdep_tend + r.qv2qi_nucleat_tend + r.qr2qi_collect_tend +
                                 r.qc2qi_collect_tend + r.qr2qi_immers_freeze_tend +
                                 r.qc2qi_hetero_freeze_tend + r.qc2qi_berg_tend) * dt;
    if (sinks > sources && sinks >= T(C::QTENDSMALL)) {
      limited |= 4;
      const T ratio = sources / sinks;
      r.qi2qv_sublim_tend *= ratio;
      r.qi2qr_melt_tend *= ratio;
    }
  }
  return limited;
}

/* nc/nr/ni conservation, p3/impl/p3_{nc,nr,ni}_conservation_impl.hpp */
template <class T>
__device__ __forceinline__ int number_conservation(T nc, T nr, T ni, T dt, Rates<T>& r) {
  int limited = 0;
  {
    const T sink = (r.nc_collect_tend + r.nc2ni_immers_freeze_tend + r.nc_accret_tend + r.nc2nr_autoconv_tend) * dt;
    const T source = nc + r.nc_selfcollect_tend * dt;
    if (sink > source) {
      limited |= 1;
      const T ratio = source / sink;
      r.nc_collect_tend *= ratio;
      r.nc2ni_immers_freeze_tend *= ratio;
      r.nc_accret_tend *= ratio;
      r.nc2nr_autoconv_tend *= ratio;
    }
  }
  {
    const T sink = (r.nr_collect_tend + r.nr2ni_immers_freeze_tend + r.nr_selfcollect_tend + r.nr_evap_tend) * dt;
    const T source = nr + (r.ni2nr_melt_tend * T(C::nmltratio) + r.nr_ice_shed_tend + r.ncshdc + r.nc2nr_autoconv_tend) * dt;
    if (sink > source) {
      limited |= 2;
      const T ratio = source / sink;
      r.nr_collect_tend *= ratio;
      r.nr2ni_immers_freeze_tend *= ratio;
      r.nr_selfcollect_tend *= ratio;
      r.nr_evap_tend *= ratio;
    }
  }
  {
    const T sink = (r.ni2nr_melt_tend + r.ni_sublim_tend + r.ni_selfcollect_tend) * dt;
    const T source = ni + (r.ni_nucleat_tend + r.nr2ni_immers_freeze_tend + r.nc2ni_immers_freeze_tend) * dt;
    if (sink > source) {
      limited |= 4;
      const T ratio = source / sink;
      r.ni2nr_melt_tend *= ratio;
      r.ni_sublim_tend *= ratio;
      r.ni_selfcollect_tend *= ratio;
    }
  }
  return limited;
}

/* ice_supersat_conservation, p3/impl/p3_ice_supersat_conservation_impl.hpp:12-40 */
__device__ __forceinline__ void ice_supersat_conservation(Rates<double>& r, double cld_frac_i, double qv,
                                                          double qv_sat_i, double t_atm, double dt) {
  const double latsublim2 = (C::LatVap + C::LatIce) * (C::LatVap + C::LatIce);
  const double qv_sink = r.qv2qi_vapdep_tend + r.qv2qi_nucleat_tend;
  if (dgt(qv_sink, C::QSMALL) && dgt(cld_frac_i, 1e-20)) {
    double qv_avail = (qv + (r.qi2qv_sublim_tend + r.qr2qv_evap_tend) * dt - qv_sat_i) /
                      (1 + latsublim2 * qv_sat_i / (C::CP * C::RH2O * sq(t_atm))) / dt;
    qv_avail = dmax0(qv_avail);
    if (qv_sink > qv_avail) {
      const double fract = qv_avail / qv_sink;
      r.qv2qi_nucleat_tend *= fract;
      r.qv2qi_vapdep_tend *= fract;
    }
  }
}

/* prevent_liq_supersaturation, p3/impl/p3_prevent_liq_supersaturation_impl.hpp:12-79 */
__device__ __forceinline__ void prevent_liq_supersaturation(double pres, double t_atm, double qv, double dt,
                                                            Rates<double>& r, uint32_t& err) {
  const double qv_sources = r.qi2qv_sublim_tend + r.qr2qv_evap_tend;
  if (!(qv_sources >= C::QSMALL)) return;
  const double qv_sinks = r.qv2qi_vapdep_tend + r.qv2qi_nucleat_tend;
  const double T_endstep = t_atm + ((qv_sinks - r.qi2qv_sublim_tend) * (C::LatVap + C::LatIce) * C::INV_CP -
                                    r.qr2qv_evap_tend * C::LatVap * C::INV_CP) * dt;
  const double qsl = qv_sat_dry(T_endstep, pres, false, err);
  const double A = C::LatVap * qsl * dt * C::INV_CP / (C::RV * T_endstep * T_endstep) *
                   ((C::LatVap + C::LatIce) * r.qi2qv_sublim_tend + C::LatVap * r.qr2qv_evap_tend);
  double frac = (qsl - qv + qv_sinks * dt + A) / (qv_sources * dt + A);
  frac = dmax_0x(frac);
  frac = dlt(frac, 1.) ? frac : 1.;
  r.qi2qv_sublim_tend = frac * r.qi2qv_sublim_tend;
  r.qr2qv_evap_tend = frac * r.qr2qv_evap_tend;
}

/* ice_supersat_conservation and prevent_liq_supersaturation of the FP32-bulk
 * form: the vapour residuals (qv + sources dt - qv_sat) are FP64, the
 * limiting fractions FP32. */
__device__ __forceinline__ void ice_supersat_conservation_bulk(Rates<float>& r, double cld_frac_i, double qv,
                                                               double qv_sat_i, float qv_sat_i_f, float tf,
                                                               float dtf) {
  const float qv_sink = r.qv2qi_vapdep_tend + r.qv2qi_nucleat_tend;
  if (qv_sink > float(C::QSMALL) && dgt(cld_frac_i, 1e-20)) {
    const double resid = qv + f2d((r.qi2qv_sublim_tend + r.qr2qv_evap_tend) * dtf) - qv_sat_i;
    constexpr float latsublim2 = float((C::LatVap + C::LatIce) * (C::LatVap + C::LatIce) / (C::CP * C::RH2O));
    float qv_avail = float(resid) / (1.0f + latsublim2 * qv_sat_i_f / (tf * tf)) / dtf;
    qv_avail = vmax(qv_avail, 0.0f);
    if (qv_sink > qv_avail) {
      const float fract = qv_avail / qv_sink;
      r.qv2qi_nucleat_tend *= fract;
      r.qv2qi_vapdep_tend *= fract;
    }
  }
}

__device__ __forceinline__ bool prevent_liq_supersaturation_bulk(double ep_inv_p, double t_atm, double qv, float dtf,
                                                                 Rates<float>& r, const RuntimeDev& rt,
                                                                 uint32_t& err) {
  const float qv_sources = r.qi2qv_sublim_tend + r.qr2qv_evap_tend;
  if (!(qv_sources >= float(C::QSMALL))) return false;
  const float qv_sinks = r.qv2qi_vapdep_tend + r.qv2qi_nucleat_tend;
  constexpr float lvs = float((C::LatVap + C::LatIce) * C::INV_CP), lv = float(C::LatVap * C::INV_CP);
  const double T_endstep = t_atm + f2d(((qv_sinks - r.qi2qv_sublim_tend) * lvs - r.qr2qv_evap_tend * lv) * dtf);
  const double qsl = svp_tabulated(rt.svp_tab, T_endstep, false, err) * ep_inv_p; /* ep_2 / max(p, 1e-3) */
  const float te = float(T_endstep);
  const float A = float(C::LatVap * C::INV_CP / C::RV) * float(qsl) * dtf / (te * te) *
                  (float(C::LatVap + C::LatIce) * r.qi2qv_sublim_tend + float(C::LatVap) * r.qr2qv_evap_tend);
  const double resid = qsl - qv + f2d(qv_sinks * dtf);
  float frac = (float(resid) + A) / (qv_sources * dtf + A);
  frac = vmax(0.0f, frac);
  frac = vmin(1.0f, frac);
  r.qi2qv_sublim_tend = frac * r.qi2qv_sublim_tend;
  r.qr2qv_evap_tend = frac * r.qr2qv_evap_tend;
  return frac < 1.0f; /* sublimation / evaporation were rescaled */
}

/* update_prognostic_ice / update_prognostic_liquid,
 * p3/impl/p3_update_prognostics_impl.hpp:9-123 (IPARAM = 3). */
struct State {
  double qc, nc, qr, nr, qi, qm, ni, bm, qv, th;
};
__device__ __forceinline__ void update_prognostics(const Rates<double>& r, double inv_exner, bool predictNc,
                                                   bool prescribedCCN, bool log_wetgrowth, double dt,
                                                   double rho_qm_cloud, double inv_rho, State& s) {
  s.qc = s.qc + (-r.qc2qi_hetero_freeze_tend - r.qc2qi_collect_tend - r.qc2qr_ice_shed_tend - r.qc2qi_berg_tend) * dt;
  if (predictNc) s.nc = s.nc + (-r.nc_collect_tend - r.nc2ni_immers_freeze_tend) * dt;
  s.qr = s.qr + (-r.qr2qi_collect_tend + r.qi2qr_melt_tend - r.qr2qi_immers_freeze_tend + r.qc2qr_ice_shed_tend) * dt;
  s.nr = s.nr + (-r.nr_collect_tend - r.nr2ni_immers_freeze_tend + C::nmltratio * r.ni2nr_melt_tend +
                 r.nr_ice_shed_tend + r.ncshdc) * dt;
  if (dge(s.qi, C::QSMALL)) {
    s.bm = s.bm - ((r.qi2qv_sublim_tend + r.qi2qr_melt_tend) / s.qi) * dt * s.bm;
    s.qm = s.qm - ((r.qi2qv_sublim_tend + r.qi2qr_melt_tend) * s.qm / s.qi) * dt;
    s.qi = s.qi - (r.qi2qv_sublim_tend + r.qi2qr_melt_tend) * dt;
  }
  const double dum = (r.qr2qi_collect_tend + r.qc2qi_collect_tend + r.qr2qi_immers_freeze_tend +
                      r.qc2qi_hetero_freeze_tend) * dt;
  s.qi = s.qi + (r.qv2qi_vapdep_tend + r.qv2qi_nucleat_tend + r.qc2qi_berg_tend) * dt + dum;
  s.qm = s.qm + dum;
  s.bm = s.bm + (r.qr2qi_collect_tend * C::INV_RHO_RIMEMAX + r.qc2qi_collect_tend / rho_qm_cloud +
                 (r.qr2qi_immers_freeze_tend + r.qc2qi_hetero_freeze_tend) * C::INV_RHO_RIMEMAX) * dt;
  s.ni = s.ni + (r.ni_nucleat_tend - r.ni2nr_melt_tend - r.ni_sublim_tend - r.ni_selfcollect_tend +
                 r.nr2ni_immers_freeze_tend + r.nc2ni_immers_freeze_tend) * dt;
  if (dneg(s.qm)) { s.qm = 0; s.bm = 0; }
  if (log_wetgrowth) { s.qm = s.qi; s.bm = s.qm * C::INV_RHO_RIMEMAX; }
  s.qv = s.qv + (-r.qv2qi_vapdep_tend + r.qi2qv_sublim_tend - r.qv2qi_nucleat_tend) * dt;
  s.th = s.th + inv_exner * ((r.qv2qi_vapdep_tend - r.qi2qv_sublim_tend + r.qv2qi_nucleat_tend) *
                                 (C::LatVap + C::LatIce) * C::INV_CP +
                             (r.qr2qi_collect_tend + r.qc2qi_collect_tend + r.qc2qi_hetero_freeze_tend +
                              r.qr2qi_immers_freeze_tend - r.qi2qr_melt_tend + r.qc2qi_berg_tend) *
                                 C::LatIce * C::INV_CP) * dt;
  /* liquid */
  s.qc = s.qc + (-r.qc2qr_accret_tend - r.qc2qr_autoconv_tend) * dt;
  s.qr = s.qr + (r.qc2qr_accret_tend + r.qc2qr_autoconv_tend - r.qr2qv_evap_tend) * dt;
  if (predictNc || prescribedCCN) {
    s.nc = s.nc + (-r.nc_accret_tend - r.nc2nr_autoconv_tend + r.nc_selfcollect_tend) * dt;
  } else {
    s.nc = C::NCCNST * inv_rho;
  }
  s.nr = s.nr + (r.ncautr - r.nr_selfcollect_tend - r.nr_evap_tend) * dt;
  s.qv = s.qv + r.qr2qv_evap_tend * dt;
  s.th = s.th + inv_exner * (-r.qr2qv_evap_tend * C::LatVap * C::INV_CP) * dt;
}

/* update_prognostic_ice / update_prognostic_liquid of the FP32-bulk form:
 * each prognostic's tendency is summed in FP32 from the FP32 rates (same
 * terms as update_prognostics) and applied to the FP64 state once; the
 * vapour change is minus the condensate changes, formed in FP64, so the
 * water of every cell is conserved to FP64 round-off.  qi_f, qm_f, bm_f are
 * the FP32 shadows of the current s.qi, s.qm, s.bm. */
__device__ __forceinline__ void update_prognostics_bulk(const Rates<float>& r, double inv_exner, bool predictNc,
                                                        bool prescribedCCN, bool log_wetgrowth, float dtf,
                                                        float rho_qm_cloud, double inv_rho, int wlim, int nlim,
                                                        const Rates<float>& r_lim, float qi_f, float qm_f,
                                                        float bm_f, State& s) {
  const float sink_i = r.qi2qv_sublim_tend + r.qi2qr_melt_tend;
  float dqi = 0, dqm = 0, dbm = 0;
  if (dge(s.qi, C::QSMALL)) {
    const float frac = sink_i * dtf / qi_f;
    dbm = -frac * bm_f;
    dqm = -frac * qm_f;
    dqi = -sink_i * dtf;
  }
  const float dum = (r.qr2qi_collect_tend + r.qc2qi_collect_tend + r.qr2qi_immers_freeze_tend +
                     r.qc2qi_hetero_freeze_tend) * dtf;
  dqi += (r.qv2qi_vapdep_tend + r.qv2qi_nucleat_tend + r.qc2qi_berg_tend) * dtf + dum;
  dqm += dum;
  dbm += (r.qr2qi_collect_tend * float(C::INV_RHO_RIMEMAX) + r.qc2qi_collect_tend / rho_qm_cloud +
          (r.qr2qi_immers_freeze_tend + r.qc2qi_hetero_freeze_tend) * float(C::INV_RHO_RIMEMAX)) * dtf;
  const float dni = (r.ni_nucleat_tend - r.ni2nr_melt_tend - r.ni_sublim_tend - r.ni_selfcollect_tend +
                     r.nr2ni_immers_freeze_tend + r.nc2ni_immers_freeze_tend) * dtf;
  const float dqc = (-r.qc2qi_hetero_freeze_tend - r.qc2qi_collect_tend - r.qc2qr_ice_shed_tend -
                     r.qc2qi_berg_tend - r.qc2qr_accret_tend - r.qc2qr_autoconv_tend) * dtf;
  const float dqr = (-r.qr2qi_collect_tend + r.qi2qr_melt_tend - r.qr2qi_immers_freeze_tend +
                     r.qc2qr_ice_shed_tend + r.qc2qr_accret_tend + r.qc2qr_autoconv_tend - r.qr2qv_evap_tend) * dtf;
  const float dnr = (-r.nr_collect_tend - r.nr2ni_immers_freeze_tend + float(C::nmltratio) * r.ni2nr_melt_tend +
                     r.nr_ice_shed_tend + r.ncshdc + r.ncautr - r.nr_selfcollect_tend - r.nr_evap_tend) * dtf;
  /* A reservoir whose conservation limiter engaged has limited sinks equal to
   * its sources, so its new value is exactly the change that later limiters
   * made to its rates (r_lim: the rates right after the conservation
   * limiters): rain evaporation and ice sublimation, deposition and
   * nucleation.  The FP64 update reaches this up to a round-off residue
   * (< qsmall, clipped to zero); an FP32 sum of the cancelling terms would
   * leave ~1e-7 of the sources instead.  The same holds for ni and, when
   * predicted, nc, whose limiters count exactly the update's terms.  The nr
   * limiter (p3_nr_conservation_impl.hpp:12-25) counts nc2nr_autoconv among
   * the sources where the update (p3_update_prognostics_impl.hpp) adds
   * ncautr, and no later limiter changes a rain-number rate, so a limited nr
   * becomes exactly (ncautr - nc2nr_autoconv) dt.  Near the melting level,
   * where shedding and collection both reach ~1e7 /kg/s, the FP32 sum of the
   * cancelling terms (~1e10 /kg, FP32 spacing ~1e3) would otherwise leave a
   * residue of ~1e3 /kg in place of that value, and rain sedimentation turns
   * it into a different drop size and fall speed. */
  const double Dqc = (wlim & 1) ? -s.qc : f2d(dqc);
  const double Dqr = (wlim & 2) ? -s.qr + f2d((r_lim.qr2qv_evap_tend - r.qr2qv_evap_tend) * dtf) : f2d(dqr);
  const double Dqi = ((wlim & 4) && dge(s.qi, C::QSMALL))
                         ? -s.qi + f2d(((r.qv2qi_vapdep_tend - r_lim.qv2qi_vapdep_tend) +
                                        (r.qv2qi_nucleat_tend - r_lim.qv2qi_nucleat_tend) -
                                        (r.qi2qv_sublim_tend - r_lim.qi2qv_sublim_tend)) * dtf)
                         : f2d(dqi);
  s.qi = s.qi + Dqi;
  s.qm = s.qm + f2d(dqm);
  s.bm = s.bm + f2d(dbm);
  s.ni = (nlim & 4) ? 0.0 : s.ni + f2d(dni);
  if (dneg(s.qm)) { s.qm = 0; s.bm = 0; }
  if (log_wetgrowth) { s.qm = s.qi; s.bm = s.qm * C::INV_RHO_RIMEMAX; }
  s.qc = s.qc + Dqc;
  s.qr = s.qr + Dqr;
  s.qv = s.qv - (Dqc + Dqr + Dqi);
  /* Latent heating from the FP64 condensate changes.  The reference heats by
   * (Lv+Lf)/cp per vapour -> ice, Lf/cp per liquid -> ice and -Lv/cp per
   * liquid -> vapour (p3_update_prognostics_impl.hpp); with vapour changing
   * by minus the condensate changes that sum equals
   * (Lv (Dqc + Dqr) + (Lv+Lf) Dqi) / cp in exact arithmetic.  Formed from the
   * same FP64 changes as the vapour, the column's energy
   * cp T + (Lv+Lf) qv + Lf (qc+qr) then closes to FP64 round-off. */
  s.th = s.th + inv_exner * ((C::LatVap * C::INV_CP) * (Dqc + Dqr) + ((C::LatVap + C::LatIce) * C::INV_CP) * Dqi);
  if (predictNc || prescribedCCN) {
    float dnc = (-r.nc_accret_tend - r.nc2nr_autoconv_tend + r.nc_selfcollect_tend) * dtf;
    if (predictNc) dnc += (-r.nc_collect_tend - r.nc2ni_immers_freeze_tend) * dtf;
    s.nc = ((nlim & 1) && predictNc) ? 0.0 : s.nc + f2d(dnc);
  } else {
    s.nc = C::NCCNST * inv_rho;
  }
  s.nr = (nlim & 2) ? f2d((r.ncautr - r.nc2nr_autoconv_tend) * dtf) : s.nr + f2d(dnr);
}

}  // namespace dev
}  // namespace p3x
