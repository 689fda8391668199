/*
 * The P3 step as three column kernels.
 *
 * One group of LANES threads (8, 16 or 32; a warp or part of one) owns one
 * column at a time; lane l owns levels l, l+LANES, l+2*LANES, ...  Inputs
 * are level-contiguous (EAMxx layout), so a group's loads of one field are
 * coalesced.  The reference's stage order (p3/impl/p3_main_impl.hpp:108-325)
 * is kept across three launches on one stream:
 *
 *   K1 p3_part12_kernel: p3_main_init + p3_main_part1 and p3_main_part2
 *      (level-parallel), with the two column-wide early exits of
 *      p3_main_impl.hpp:237-239 and :260 as group ballots.  It hands the
 *      per-level start-of-step temperature, density and fall-speed factors
 *      to K2/K3 through a scratch array and marks each column that goes on.
 *   K2 p3_sed_kernel: cloud, rain and ice sedimentation: CFL substeps with
 *      the Courant maximum as a group shuffle reduction and the upwind flux
 *      divergence walked down the levels chunk by chunk with a shuffle-up and
 *      a carry (p3_upwind_impl.hpp:14-116).  Substep loops are capped.
 *   K3 p3_part3_kernel: homogeneous freezing + p3_main_part3.
 *
 * Splitting lets each kernel keep its own register and shared-memory
 * footprint: part2's ~45 rates no longer limit the occupancy of the
 * latency-bound sedimentation walk.  Per-level temporaries of a phase live
 * in shared memory (9 FP64 arrays per column in K1, 11 in K2).  Lookup
 * tables are read from global memory (L1/L2) or, in K1, staged into shared
 * memory once per CTA with cp.async.bulk + mbarrier (Table3 slices for the
 * runtime's constant rain shape parameter, plus the whole ice table).
 */
#pragma once

#include <type_traits>

#include "p3x_physics.cuh"

namespace p3x {
namespace dev {

/* Arguments of one instance (device pointers, (ncol, nlev) row-major). */
struct Inst {
  double *qc, *nc, *qr, *nr, *qi, *qm, *ni, *bm, *qv, *th;
  const double *nc_nuceat_tend, *nccn, *ni_activated, *inv_qc_relvar, *cld_frac_i, *cld_frac_l,
      *cld_frac_r, *pres, *dz, *dpres, *inv_exner, *qv_prev, *t_prev;
  double *qv2qi_depos_tend, *precip_liq_surf, *precip_ice_surf, *diag_eff_radius_qc,
      *diag_eff_radius_qi, *diag_eff_radius_qr, *rho_qi, *precip_liq_flux, *precip_ice_flux,
      *precip_total_tend, *nevapr;
  double *liq_ice_exchange, *vap_liq_exchange, *vap_ice_exchange;
  /* hand-over from K1 to K2/K3: [kScrFields][ncol][ld] doubles, and one
   * continue flag per column (0: the column took an early exit) */
  double* scr;
  int32_t* cflag;
  int64_t ld, ld_int;
  int32_t ncol, nlev;
  double dt;
  int32_t predictNc, prescribedCCN, precision, pad_;
};

/* Work item of the batched form: (instance, column). */
struct WorkItem {
  int32_t inst, col;
};

template <class TR>
struct KParams {
  RuntimeDev rt;
  /* global tables in the rate precision */
  const TR* ice;
  const TR* ice_sed; /* FP32-bulk: slots 0-3 of every ice-table row, packed */
  const TR* collect;
  const TR* vn;
  const TR* vm;
  const TR* revap;
  const TR* t3slice; /* [3][300][2] = vn, vm, revap columns (t3_dumjj-1, t3_dumjj) */
  int staged;        /* stage ice table + Table3 slices into shared memory */
  int sm_stride;     /* doubles per per-level shared array (>= nlev_max + 1, even) */
  int groups_per_block;
  int nwork;         /* number of columns (single) or work items (batched) */
  const WorkItem* work;
  const Inst* insts;
  uint32_t* err;
  /* kWorkCounters zeroed counters: groups take work items from them as they
   * finish the last ones.  Null: groups stride the list statically. */
  uint32_t* wctr;
  /* check_values after part3 (null: off): kCheckWords words of CheckWord */
  unsigned long long* check;
  int check_fail; /* a temperature out of range also sets kErrRange */
};

/* check_values (p3_check_values_impl.hpp): counts of levels with T outside
 * (173, 323) K and with qv outside (0, 0.04), and the smallest packed
 * (instance, column, level) key of each kind. */
enum CheckWord { kChkTCount = 0, kChkQvCount, kChkTFirst, kChkQvFirst, kCheckWords };
__host__ __device__ inline unsigned long long check_key(int inst, int col, int k) {
  return (static_cast<unsigned long long>(inst) << 40) | (static_cast<unsigned long long>(col) << 16) |
         static_cast<unsigned long long>(k);
}

constexpr int kIceTableElems = kDensize * kRimsize * kIsize * kIceCols; /* 12000 */
constexpr int kT3SliceElems = 3 * 300 * 2;
constexpr int kMaxSubsteps = 100000;
constexpr long long kWaitSpinLimit = 1ll << 26;
constexpr uint64_t kWaitNanosLimit = 2000000000ull; /* 2 s */

/* shared arrays of one column group in K1 */
enum { A_TATM = 0, A_RHO, A_RHOFACR, A_RHOFACI, A_ACN, A_QVSL, A_QVSI, A_QVSSI, A_EPINVP, A_NARR };
/* shared arrays of one column group in K2; FAC is the fall-speed factor of
 * the species being sedimented (acn, rhofacr or rhofaci), the rain flux
 * accumulator re-uses R2 (rain has two fields) */
enum { B_RHO = 0, B_INVRHO, B_INVDZ, B_FAC, B_CLD, B_V1, B_V2, B_R0, B_R1, B_R2, B_R3, B_NARR };
/* slots (of S doubles) of one column group in K2: B_NARR in the FP64 form,
 * kSedBulkSlots in the FP32-bulk form (p3_sed_bulk) */
constexpr int kSedBulkSlots = 10;
template <class TR>
__host__ __device__ constexpr int sed_slots() {
  return sizeof(TR) == sizeof(float) ? kSedBulkSlots : B_NARR;
}
/* hand-over fields K1 -> K2/K3 */
enum { S_TATM = 0, S_RHO, S_RHOFACR, S_RHOFACI, S_ACN, kScrFields };

__device__ __forceinline__ double* scr_at(const Inst& in, int f, int col) {
  return in.scr + (int64_t(f) * in.ncol + col) * in.ld;
}
/* FP32-bulk: the float-valued hand-over fields (rho, fall-speed factors,
 * acn) hold floats in the first half of each column's row */
__device__ __forceinline__ float* scr_f(const Inst& in, int f, int col) {
  return reinterpret_cast<float*>(scr_at(in, f, col));
}

/* Launch-wide work counters of one step (K1, K2, K3, spare), zeroed on the
 * stream before K1.  They follow the hand-over doubles and the flags in an
 * instance's scratch. */
constexpr int kWorkCounters = 4;
__host__ __device__ inline size_t work_counter_offset(int ncol, int64_t ld) {
  const size_t d = size_t(kScrFields) * size_t(ncol) * size_t(ld) * sizeof(double);
  return ((d + size_t(ncol) * sizeof(int32_t) + 15) / 16) * 16;
}
/* bytes of the K1->K2/K3 scratch of an instance (doubles, flags, counters) */
__host__ __device__ inline size_t scratch_bytes(int ncol, int64_t ld) {
  return ((work_counter_offset(ncol, ld) + kWorkCounters * sizeof(uint32_t) + 255) / 256) * 256;
}

template <class TR>
__host__ __device__ constexpr size_t table_smem_bytes() {
  return ((sizeof(TR) * (kIceTableElems + kT3SliceElems) + 15) / 16) * 16 + 16;
}

/* ------------------------------------------------------------------ */
/* group primitives                                                    */
/* ------------------------------------------------------------------ */
template <int LANES>
__device__ __forceinline__ unsigned group_mask() {
  if (LANES == 32) return 0xffffffffu;
  const unsigned lw = threadIdx.x & 31u;
  return (0xffffffffu >> (32 - LANES)) << (lw & ~unsigned(LANES - 1));
}
template <int LANES>
__device__ __forceinline__ bool group_any(unsigned mask, bool p) {
  return __ballot_sync(mask, p) != 0u;
}
/* Maxima and minima over the group with the warp-reduction instruction
 * (redux.sync), one instruction instead of log2(LANES) dependent shuffles.
 * Non-negative floats and doubles order as their bit patterns (as unsigned
 * integers), so their maximum is the maximum of the patterns; a NaN (a
 * pattern above +inf) wins and reaches the caller's Courant check. */
/* maximum over the group of non-negative doubles (dmax_nn): the largest high
 * word, then the largest low word among the lanes holding it */
template <int LANES>
__device__ __forceinline__ double group_max_nn(unsigned mask, double v) {
  const unsigned hi = unsigned(__double2hiint(v)), lo = unsigned(__double2loint(v));
  const unsigned mhi = __reduce_max_sync(mask, hi);
  const unsigned mlo = __reduce_max_sync(mask, hi == mhi ? lo : 0u);
  return __hiloint2double(int(mhi), int(mlo));
}
/* maximum over the group of non-negative floats (Courant numbers) */
template <int LANES>
__device__ __forceinline__ float group_max_nn(unsigned mask, float v) {
  return __uint_as_float(__reduce_max_sync(mask, __float_as_uint(v)));
}
template <int LANES>
__device__ __forceinline__ int group_min_int(unsigned mask, int v) {
  return __reduce_min_sync(mask, v);
}
template <int LANES>
__device__ __forceinline__ int group_max_int(unsigned mask, int v) {
  return __reduce_max_sync(mask, v);
}

/* ------------------------------------------------------------------ */
/* bulk copy of the tables into shared memory                          */
/* ------------------------------------------------------------------ */
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

/* Thread 0 arms an mbarrier with the byte count and issues the bulk copies;
 * every thread then waits on the barrier's phase with a bounded spin.
 * Returns false (and sets kErrWait) if the wait gave up. */
template <class TR>
__device__ bool stage_tables(const KParams<TR>& kp, TR* s_ice, TR* s_t3, uint64_t* mbar, uint32_t& err) {
  const uint32_t bar = smem_u32(mbar);
  const uint32_t ice_bytes = uint32_t(sizeof(TR) * kIceTableElems);
  const uint32_t t3_bytes = uint32_t(sizeof(TR) * kT3SliceElems);
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(1) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar),
                 "r"(ice_bytes + t3_bytes)
                 : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(s_ice)),
        "l"(kp.ice), "r"(ice_bytes), "r"(bar)
        : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(s_t3)),
        "l"(kp.t3slice), "r"(t3_bytes), "r"(bar)
        : "memory");
  }
  bool done = false;
  uint64_t t0;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
  for (long long spin = 0; spin < kWaitSpinLimit; ++spin) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(0)
        : "memory");
    if (ok) {
      done = true;
      break;
    }
    uint64_t t1;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t1));
    if (t1 - t0 > kWaitNanosLimit) break;
  }
  if (!done) err |= kErrWait;
  return done;
}

/* Applies a rate-precision DSD adjustment of a number concentration to the
 * FP64 value only when the DSD routine changed it (exact for FP64). */
template <class TR>
__device__ __forceinline__ void apply_n_adjust(double& n_d, TR n_in, TR n_out) {
  if (n_out != n_in) n_d = double(n_out);
}

/* The end of p3_main_part2 (p3_main_part2_impl.hpp, after update_prognostics):
 * a species below qsmall goes to vapour and its latent heat to theta; a +0
 * moves nothing, so its FP64 updates are skipped (bitwise the same result).
 * Returns whether any species remains. */
__device__ __forceinline__ bool clip_to_vapour(State& s, double inv_exner) {
  bool hydro = false;
  if (dlt(s.qc, C::QSMALL)) {
    if (dnz(s.qc)) {
      s.qv = s.qv + s.qc;
      s.th = s.th - inv_exner * s.qc * C::LatVap * C::INV_CP;
    }
    s.qc = 0;
    s.nc = 0;
  } else {
    hydro = true;
  }
  if (dlt(s.qr, C::QSMALL)) {
    if (dnz(s.qr)) {
      s.qv = s.qv + s.qr;
      s.th = s.th - inv_exner * s.qr * C::LatVap * C::INV_CP;
    }
    s.qr = 0;
    s.nr = 0;
  } else {
    hydro = true;
  }
  if (dlt(s.qi, C::QSMALL)) {
    if (dnz(s.qi)) {
      s.qv = s.qv + s.qi;
      s.th = s.th - inv_exner * s.qi * (C::LatVap + C::LatIce) * C::INV_CP;
    }
    s.qi = 0; s.ni = 0; s.qm = 0; s.bm = 0;
  } else {
    hydro = true;
  }
  return hydro;
}

/* p3_main_part2 of one level in the FP32-bulk form (p3_main_part2_impl.hpp,
 * same order of processes).  The FP64 state is read once and shadowed in
 * FP32; the in-cloud values, DSDs, table lookups, process rates and limiter
 * ratios are FP32, while the thresholds test the FP64 state.  The vapour
 * residuals, the melting / wet-growth departures and the state update are
 * FP64.  A DSD or rime limiter that changes an in-cloud value rewrites the
 * FP64 state and its shadow.  sm / S: the K1 shared arrays of the column. */
__device__ __forceinline__ void part2_level_bulk(const Inst& in, const int64_t o, const int k,
                                                 double* __restrict__ sm, const int S, const KParams<float>& kp,
                                                 const Tabs<float>& tb, const double esat0, const float dtf,
                                                 const float inv_dtf, bool& hydro, uint32_t& err) {
  const RuntimeDev& rt = kp.rt;
  const bool predictNc = in.predictNc != 0, prescribedCCN = in.prescribedCCN != 0;
  const bool do_ice = rt.do_ice_production != 0;
  const double inv_dt_d = f2d(inv_dtf);
  const float* const smf_rho = reinterpret_cast<const float*>(&sm[A_RHO * S]);
  const float* const smf_rhofaci = reinterpret_cast<const float*>(&sm[A_RHOFACI * S]);
  const float* const smf_acn = reinterpret_cast<const float*>(&sm[A_ACN * S]);
  State s;
  s.qc = in.qc[o]; s.nc = in.nc[o]; s.qr = in.qr[o]; s.nr = in.nr[o];
  s.qi = in.qi[o]; s.qm = in.qm[o]; s.ni = in.ni[o]; s.bm = in.bm[o];
  s.qv = in.qv[o]; s.th = in.th[o];
  const double T = sm[A_TATM * S + k];
  const double qvssi = sm[A_QVSSI * S + k];
  const bool dry = dlt(s.qc, C::QSMALL) && dlt(s.qr, C::QSMALL) && dlt(s.qi, C::QSMALL);
  if (dry && dlt(T, C::T_zerodegc) && dlt_neg(qvssi, -0.05)) return;
  /* A level without hydrometeors where ice cannot nucleate (nucleation
   * needs T < Tmelt - 15 and qv_supersat_i >= 0.05; the test below leaves a
   * margin for the float temperature) has no process rate, so the level keeps
   * its state and every tendency output is the +0 that part1 wrote, except
   * vap_liq_exchange = -(+0).  With nc diagnosed (neither predicted nor
   * prescribed) the update resets nc, so that case goes the whole way. */
  if (dry && (predictNc || prescribedCCN) && !(dlt(T, C::Tmelt - 14.0) && dge(qvssi, 0.04))) {
    in.vap_liq_exchange[o] = -0.0;
    return;
  }

  const double cld_i = in.cld_frac_i[o], cld_l = in.cld_frac_l[o], cld_r = in.cld_frac_r[o];
  const double inv_exner = in.inv_exner[o];
  const double qvsl = sm[A_QVSL * S + k], qvsi = sm[A_QVSI * S + k];
  const double ep_inv_p = sm[A_EPINVP * S + k]; /* ep_2 / max(p, 1e-3) */
  const float rho = smf_rho[k], inv_rho = 1.0f / rho, rhofaci = smf_rhofaci[k], acn = smf_acn[k];
  const float T_r = float(T), qvsi_r = float(qvsi);
  const float cl = float(cld_l), ci = float(cld_i), cr = float(cld_r);
  const float icl = 1.0f / cl, ici = 1.0f / ci, icr = 1.0f / cr;
  /* FP32 shadows of the state (kept equal to float(s.x) where s.x changes) */
  const float qc0 = float(s.qc), qr0 = float(s.qr), qi0 = float(s.qi), ni0 = float(s.ni);
  float nc0 = float(s.nc), nr0 = float(s.nr), qm0 = float(s.qm), bm0 = float(s.bm);
  constexpr float QS = float(C::QSMALL);

  /* calculate_incloud_mixingratios (bm uses 1/cld_frac_l, p3_incloud_mixingratios_impl.hpp:49) */
  float qc_in = 0, nc_in = 0, qr_in = 0, nr_in = 0, qi_in = 0, ni_in = 0, qm_in = 0, bm_in = 0;
  if (dge(s.qc, C::QSMALL)) { qc_in = qc0 * icl; nc_in = vmax(nc0 * icl, 0.0f); }
  if (dge(s.qi, C::QSMALL)) { qi_in = qi0 * ici; ni_in = vmax(ni0 * ici, 0.0f); }
  if (dge(s.qi, C::QSMALL) && dge(s.qm, C::QSMALL)) { qm_in = qm0 * ici; bm_in = vmax(bm0 * icl, 0.0f); }
  if (dge(s.qr, C::QSMALL)) { qr_in = qr0 * icr; nr_in = vmax(nr0 * icr, 0.0f); }
  {
    constexpr float il = float(C::incloud_limit), pl = float(C::precip_limit);
    if (qc_in > il || qi_in > il || qr_in > pl || bm_in > il) {
      qc_in = vmin(qc_in, il);
      qi_in = vmin(qi_in, il);
      bm_in = vmin(bm_in, il);
      qr_in = vmin(qr_in, pl);
    }
  }

  Rates<float> r;
  r.zero();
  PhysVars<float> v;
  v.mu = v.dv = v.sc = v.dqsdt = v.dqsidt = v.ab = v.abi = v.kap = v.eii = 0.0f;
  float tv_fallspd = 0, tv_selfcol = 0, tv_qc2qi = 0, tv_melt = 0, tv_nr = 0, tv_qr2qi = 0, tv_lammax = 0,
        tv_lammin = 0, tv_vent = 0;
  float mu_c = 0, lamc = 0, mu_r = 0, lamr = 0, cdistr = 0, logn0r = 0;
  float epsi = 0, epsr = 0, epsi_tot = 0;
  float rho_qm_cloud = 400.0f;
  bool wet = false;

  if (qc_in >= QS || qr_in >= QS || qi_in >= QS) {
    get_time_space_phys_variables<float>(T_r, float(in.pres[o]), rho, float(qvsl), qvsi_r, v);
    {
      float n_out = nc_in;
      get_cloud_dsd2<float>(qc_in, n_out, mu_c, rho, lamc);
      if (n_out != nc_in) {
        nc_in = n_out;
        s.nc = f2d(n_out) * cld_l;
        nc0 = float(s.nc);
      }
    }
    {
      float n_out = nr_in;
      get_rain_dsd2<float>(qr_in, n_out, mu_r, lamr, rt);
      const bool changed = n_out != nr_in;
      nr_in = n_out;
      if (qr_in >= QS) {
        cdistr = nr_in / rt.f.g_mur1;
        logn0r = m_log10(cdistr) + (mu_r + 1.0f) * m_log10(lamr);
      }
      if (changed) {
        s.nr = f2d(n_out) * cld_r;
        nr0 = float(s.nr);
      }
    }
    impose_max_total_ni(ni_in, rt.f.max_total_ni, inv_rho);
    if (qi_in >= QS) {
      ni_in = vmax(ni_in, float(C::NSMALL));
      nr_in = vmax(nr_in, float(C::NSMALL));
      float qm_f = qm_in, bm_f = bm_in;
      const float rhop = calc_bulk_rho_rime<float>(qi_in, qm_f, bm_f, rt);
      if (qm_f != qm_in) {
        qm_in = qm_f;
        s.qm = f2d(qm_f) * cld_i;
        qm0 = float(s.qm);
      }
      if (bm_f != bm_in) {
        bm_in = bm_f;
        s.bm = f2d(bm_f) * cld_i;
        bm0 = float(s.bm);
      }
      TableIce<float> ti;
      lookup_ice<float>(qi_in, ni_in, qm_in, rhop, ti);
      TableRain<float> trn;
      lookup_rain<float>(qr_in, nr_in, trn);
      float ta[4], tc[4];
      apply_table_ice4<float>(tb, ti, 0, ta); /* columns 0, 1, 6, 7 */
      apply_table_ice4<float>(tb, ti, 4, tc); /* columns 2, 3, 4, 9 */
      tv_fallspd = ta[1];
      tv_selfcol = tc[0];
      tv_qc2qi = tc[1];
      tv_melt = tc[2];
      tv_lammax = ta[2];
      tv_lammin = ta[3];
      tv_vent = tc[3];
      if (qr_in >= QS) {
        tv_nr = apply_table_coll<float>(0, tb, ti, trn);
        tv_qr2qi = apply_table_coll<float>(1, tb, ti, trn);
      }
      ni_in = vmin(ni_in, tv_lammax * ni_in);
      ni_in = vmax(ni_in, tv_lammin * ni_in);
    }
    const double dT0 = T - C::Tmelt;
    const double dqv0 = esat0 * ep_inv_p - s.qv;
    if (do_ice) {
      ice_cldliq_collection<float>(rho, T, rhofaci, tv_qc2qi, qi_in, qc_in, ni_in, nc_in, r, rt);
      ice_rain_collection<float>(rho, T, rhofaci, logn0r, tv_nr, tv_qr2qi, qi_in, ni_in, qr_in, r, rt);
      ice_self_collection<float>(rho, rhofaci, tv_selfcol, v.eii, qm_in, qi_in, ni_in, r);
    }
    ice_melting<float>(rho, dT0, dqv0, rhofaci, tv_melt, tv_vent, v, qi_in, ni_in, r);
    if (do_ice) {
      wet = ice_cldliq_wet_growth<float>(rho, dT0, dqv0, rhofaci, tv_melt, tv_vent, v, qc_in, qi_in, ni_in, qr_in,
                                         r);
    }
    /* ice_relaxation_timescale, p3_ice_relaxation_timescale_impl.hpp:9-37 */
    if (qi_in >= QS && dlt(T, C::Tmelt)) {
      epsi = ((tv_melt + tv_vent * m_cbrt(v.sc) * m_sqrt(rhofaci * rho / v.mu)) * 2.0f * float(C::Pi) * rho *
              v.dv) * ni_in;
      epsi_tot = epsi_tot + epsi;
    }
    rho_qm_cloud = calc_rime_density<float>(T_r, rhofaci, tv_fallspd, acn, lamc, mu_c, qc_in,
                                            r.qc2qi_collect_tend);
    if (do_ice) {
      cldliq_immersion_freezing<float>(T_r, lamc, mu_c, nc_in, qc_in, r, rt);
      rain_immersion_freezing<float>(T_r, lamr, mu_r, cdistr, qr_in, r, rt);
    }
    /* calc_liq_relaxation_timescale, p3_calc_liq_relaxation_timescale_impl.hpp:13-43 */
    if (qr_in >= QS) {
      Table3<float> t3;
      lookup3<float>(mu_r, lamr, rt, t3);
      epsr = 2.0f * float(C::Pi) * cdistr * rho * v.dv *
             (float(C::f1r) * rt.f.g_mur2 / lamr +
              float(C::f2r) * m_sqrt(rho / v.mu) * m_cbrt(v.sc) * apply_table3<float>(tb, tb.revap, t3));
    }
    evaporate_rain_bulk(qr_in, qc_in, nr_in, qi_in, cl, cr, s.qv, in.qv_prev[o], qvsl, qvsi, v.ab, v.abi, epsr,
                        epsi_tot, T, in.t_prev[o], v.dqsdt, dtf, inv_dtf, inv_dt_d, r.qr2qv_evap_tend,
                        r.nr_evap_tend);
    if (do_ice) {
      ice_deposition_sublimation_bulk(qi_in, ni_in, T, qvsl, qvsi, epsi, v.abi, s.qv, inv_dtf, r.qv2qi_vapdep_tend,
                                      r.qi2qv_sublim_tend, r.ni_sublim_tend, r.qc2qi_berg_tend);
    }
  }
  if (do_ice) {
    ice_nucleation<float>(T_r, inv_rho, ni0, float(in.ni_activated[o]), qvssi, inv_dtf, predictNc, prescribedCCN,
                          r, rt);
  }
  cloud_water_autoconversion<float>(rho, qc_in, nc_in, r, rt);
  if (qc_in >= QS) r.nc_selfcollect_tend = 0.0f;
  cloud_rain_accretion<float>(qc_in, nc_in, qr_in, r, rt);
  rain_self_collection<float>(rho, qr_in, nr_in, r, rt);
  back_to_cell_average<float>(cl, cr, ci, r);

  /* limiters on the FP32 rates (FP64 vapour residuals), one FP64
   * application of each prognostic's FP32 tendency */
  const int wlim = water_conservation<float>(qc0, qr0, qi0, dtf, r);
  const int nlim = number_conservation<float>(nc0, nr0, ni0, dtf, r);
  const Rates<float> r_lim = r;
  ice_supersat_conservation_bulk(r, cld_i, s.qv, qvsi, qvsi_r, T_r, dtf);
  prevent_liq_supersaturation_bulk(ep_inv_p, T, s.qv, dtf, r, rt, err);
  update_prognostics_bulk(r, inv_exner, predictNc, prescribedCCN, wet, dtf, rho_qm_cloud, f2d(inv_rho), wlim, nlim,
                          r_lim, qi0, qm0, bm0, s);

  in.qv2qi_depos_tend[o] = f2d(r.qv2qi_vapdep_tend - r.qi2qv_sublim_tend + r.qv2qi_nucleat_tend);
  in.precip_total_tend[o] = f2d(r.qc2qr_accret_tend + r.qc2qr_autoconv_tend + r.qc2qr_ice_shed_tend +
                                r.qc2qi_collect_tend);
  in.nevapr[o] = f2d(r.qi2qv_sublim_tend + r.qr2qv_evap_tend);
  in.vap_ice_exchange[o] = f2d(r.qv2qi_vapdep_tend - r.qi2qv_sublim_tend + r.qv2qi_nucleat_tend);
  in.vap_liq_exchange[o] = f2d(-r.qr2qv_evap_tend);
  in.liq_ice_exchange[o] = f2d(r.qc2qi_hetero_freeze_tend + r.qr2qi_immers_freeze_tend - r.qi2qr_melt_tend +
                               r.qc2qi_berg_tend + r.qc2qi_collect_tend + r.qr2qi_collect_tend);

  hydro |= clip_to_vapour(s, inv_exner);
  if (dge(s.ni, 1e-20)) {
    /* impose_max_total_ni as a factor applied only when it limits */
    const float f = vmin(rt.f.max_total_ni * inv_rho * ci / float(s.ni), 1.0f);
    if (f < 1.0f) s.ni = s.ni * f2d(f);
  }
  in.qc[o] = s.qc; in.nc[o] = s.nc; in.qr[o] = s.qr; in.nr[o] = s.nr;
  in.qi[o] = s.qi; in.qm[o] = s.qm; in.ni[o] = s.ni; in.bm[o] = s.bm;
  in.qv[o] = s.qv; in.th[o] = s.th;
}

/* ------------------------------------------------------------------ */
/* one column                                                          */
/* ------------------------------------------------------------------ */
/* K1: p3_main_init, p3_main_part1, p3_main_part2 of one column. */
template <class TR, int LANES>
__device__ void p3_part12(const Inst& in, const int col, const KParams<TR>& kp, const Tabs<TR>& tb,
                          double* __restrict__ sm, const double esat0, uint32_t& err) {
  constexpr bool kF64 = sizeof(TR) == sizeof(double);
  const RuntimeDev& rt = kp.rt;
  const unsigned mask = group_mask<LANES>();
  const int lane = threadIdx.x & (LANES - 1);
  const int nk = in.nlev;
  const int S = kp.sm_stride;
  const int64_t co = int64_t(col) * in.ld;
  const int64_t ci = int64_t(col) * in.ld_int;
  const double dt = in.dt;
  const double inv_dt = 1 / dt;
  const bool predictNc = in.predictNc != 0, prescribedCCN = in.prescribedCCN != 0;
  const bool do_ice = rt.do_ice_production != 0;
#define SMA(a, k) sm[(a)*S + (k)]
  /* FP32-bulk: the float-valued slots (rho, fall-speed factors, acn) hold
   * floats in the first half of their slot */
#define SMF(a) reinterpret_cast<float*>(&sm[(a)*S])

  /* ---------------- phase 1: p3_main_init + p3_main_part1 ---------------- */
  bool nucl = false, hydro = false;
  for (int k = lane; k < nk; k += LANES) {
    const int64_t o = co + k;
    const double cld_l = in.cld_frac_l[o];
    const double inv_exner = in.inv_exner[o];
    double th = in.th[o];
    const double dz = in.dz[o];
    double qv = in.qv[o];
    const double pres = in.pres[o];
    const double dpres = in.dpres[o];
    double qc = in.qc[o], nc = in.nc[o], qr = in.qr[o], nr = in.nr[o];
    double qi = in.qi[o], ni = in.ni[o], qm = in.qm[o], bm = in.bm[o];

    in.diag_eff_radius_qc[o] = 10.e-6;
    in.diag_eff_radius_qi[o] = 25.e-6;
    in.diag_eff_radius_qr[o] = 500.e-6;
    in.rho_qi[o] = 0;
    in.qv2qi_depos_tend[o] = 0;
    in.precip_total_tend[o] = 0;
    in.nevapr[o] = 0;
    in.liq_ice_exchange[o] = 0;
    in.vap_liq_exchange[o] = 0;
    in.vap_ice_exchange[o] = 0;

    double rho, inv_rho, qvsl, qvsi, qvssi, ccn_nc;
    TR rho_t, inv_rho_t;
    const double exner = kF64 ? 1 / inv_exner : rcp_newton1(inv_exner);
    double T = th * exner;
    qv = dmax0(qv);
    if constexpr (kF64) {
      const double inv_cld_l = 1 / cld_l;
      rho = dpres / dz / C::gravit;
      inv_rho = 1 / rho;
      rho_t = rho;
      inv_rho_t = inv_rho;
      qvsl = qv_sat_dry(T, pres, false, err);
      qvsi = qv_sat_dry(T, pres, true, err);
      qvssi = qv / qvsi - 1;
      ccn_nc = rt.spa_ccn_to_nc_factor * in.nccn[o] / inv_cld_l;
    } else {
      /* FP32-bulk: rho and 1/rho only feed rates, fall speeds and fluxes
       * (the sedimentation's FP64 coefficient is g / dpres), so they are
       * FP32 and kept as floats in the shared slots and the hand-over; one
       * Newton reciprocal of the pressure, times ep_2, shared by both
       * saturation ratios (and kept for part2's melting departure and
       * supersaturation limiter); the supersaturation ratio (threshold and
       * rate input) in FP32 */
      const float rho_f = float(dpres) / (float(dz) * float(C::gravit));
      rho_t = rho_f;
      rho = f2d(rho_f);
      inv_rho_t = 1.0f / rho_f;
      inv_rho = f2d(inv_rho_t);
      const double ep_inv_p = C::ep_2 * rcp_newton1(dmax_c(pres, 1.e-3));
      SMA(A_EPINVP, k) = ep_inv_p;
      qvsl = svp_tabulated(rt.svp_tab, T, false, err) * ep_inv_p;
      qvsi = svp_tabulated(rt.svp_tab, T, true, err) * ep_inv_p;
      qvssi = f2d(float(qv) / float(qvsi) - 1.0f);
      ccn_nc = rt.spa_ccn_to_nc_factor * in.nccn[o] * cld_l;
    }
    const TR rhofacr = m_pow(TR(C::RHO_1000MB) * inv_rho_t, TR(.54));
    const TR rhofaci = m_pow(TR(C::RHO_600MB) * inv_rho_t, TR(.54));
    const TR dum = TR(1.496e-6) * m_pow(TR(T), TR(1.5)) / (TR(T) + TR(120));
    const TR acn = TR(C::gravit) * TR(C::RHO_H2O) / (TR(18) * dum);
    if (dlt(T, C::T_zerodegc) && dge_neg(qvssi, -0.05)) nucl = true;

    /* A species below qsmall goes to vapour; a +0 moves nothing, so its FP64
     * updates are skipped (bitwise the same result). */
    bool th_changed = false;
    if (dlt(qc, C::QSMALL)) {
      if (dnz(qc)) {
        qv = qv + qc;
        th = th - inv_exner * qc * C::LatVap * C::INV_CP;
        th_changed = true;
      }
      qc = 0;
      nc = 0;
    } else {
      hydro = true;
      if (prescribedCCN) {
        nc = vmax(nc, ccn_nc);
      } else if (predictNc) {
        nc = dmax0(nc + in.nc_nuceat_tend[o] * dt);
      } else {
        nc = C::NCCNST * inv_rho;
      }
    }
    if (dlt(qr, C::QSMALL)) {
      if (dnz(qr)) {
        qv = qv + qr;
        th = th - inv_exner * qr * C::LatVap * C::INV_CP;
        th_changed = true;
      }
      qr = 0;
      nr = 0;
    } else {
      hydro = true;
    }
    if (dlt(qi, C::QSMALL) || (dlt(qi, 1.e-8) && dlt_neg(qvssi, -0.1))) {
      if (dnz(qi)) {
        qv = qv + qi;
        th = th - inv_exner * qi * (C::LatVap + C::LatIce) * C::INV_CP;
        th_changed = true;
      }
      qi = 0; ni = 0; qm = 0; bm = 0;
    } else {
      hydro = true;
    }
    if (dge(qi, C::QSMALL) && dlt(qi, 1.e-8) && dge(T, C::T_zerodegc)) {
      qr = qr + qi;
      th = th - inv_exner * qi * C::LatIce * C::INV_CP;
      th_changed = true;
      qi = 0; ni = 0; qm = 0; bm = 0;
    }
    if (th_changed) T = th * exner;

    in.qc[o] = qc; in.nc[o] = nc; in.qr[o] = qr; in.nr[o] = nr;
    in.qi[o] = qi; in.ni[o] = ni; in.qm[o] = qm; in.bm[o] = bm;
    in.qv[o] = qv; in.th[o] = th;
    SMA(A_TATM, k) = T;
    if constexpr (kF64) {
      SMA(A_RHO, k) = rho;
      SMA(A_RHOFACR, k) = rhofacr;
      SMA(A_RHOFACI, k) = rhofaci;
      SMA(A_ACN, k) = acn;
    } else {
      SMF(A_RHO)[k] = rho_t;
      SMF(A_RHOFACR)[k] = rhofacr;
      SMF(A_RHOFACI)[k] = rhofaci;
      SMF(A_ACN)[k] = acn;
    }
    SMA(A_QVSL, k) = qvsl;
    SMA(A_QVSI, k) = qvsi;
    SMA(A_QVSSI, k) = qvssi;
  }
  for (int k = lane; k <= nk; k += LANES) {
    in.precip_liq_flux[ci + k] = 0;
    in.precip_ice_flux[ci + k] = 0;
  }
  if (lane == 0) {
    in.precip_liq_surf[col] = 0;
    in.precip_ice_surf[col] = 0;
  }
  if (!group_any<LANES>(mask, nucl || hydro)) {
    if (lane == 0) in.cflag[col] = 0;
    return;
  }

  /* ---------------- phase 2: p3_main_part2 ---------------- */
  hydro = false;
  if constexpr (!kF64) {
    const float dtf = float(dt), inv_dtf = float(inv_dt);
    for (int k = lane; k < nk; k += LANES)
      part2_level_bulk(in, co + k, k, sm, S, kp, tb, esat0, dtf, inv_dtf, hydro, err);
  } else {
  for (int k = lane; k < nk; k += LANES) {
    const int64_t o = co + k;
    State s;
    s.qc = in.qc[o]; s.nc = in.nc[o]; s.qr = in.qr[o]; s.nr = in.nr[o];
    s.qi = in.qi[o]; s.qm = in.qm[o]; s.ni = in.ni[o]; s.bm = in.bm[o];
    s.qv = in.qv[o]; s.th = in.th[o];
    const double T = SMA(A_TATM, k);
    const double qvssi = SMA(A_QVSSI, k);
    if (dlt(s.qc, C::QSMALL) && dlt(s.qr, C::QSMALL) && dlt(s.qi, C::QSMALL) && dlt(T, C::T_zerodegc) &&
        dlt_neg(qvssi, -0.05))
      continue;

    const double pres = in.pres[o];
    const double cld_i = in.cld_frac_i[o], cld_l = in.cld_frac_l[o], cld_r = in.cld_frac_r[o];
    const double inv_exner = in.inv_exner[o];
    const double qvsl = SMA(A_QVSL, k), qvsi = SMA(A_QVSI, k);
    const double rho = SMA(A_RHO, k);
    const double inv_rho = 1 / rho;
    const double rhofaci = SMA(A_RHOFACI, k);
    const double acn = SMA(A_ACN, k);
    Incld inc;
    calc_incloud(s.qc, s.qr, s.qi, s.qm, s.nc, s.nr, s.ni, s.bm, 1 / cld_l, 1 / cld_i, 1 / cld_r, inc);

    Rates<TR> r;
    r.zero();
    PhysVars<TR> v;
    v.mu = v.dv = v.sc = v.dqsdt = v.dqsidt = v.ab = v.abi = v.kap = v.eii = TR(0);
    TR tv_fallspd = 0, tv_selfcol = 0, tv_qc2qi = 0, tv_melt = 0, tv_nr = 0, tv_qr2qi = 0,
       tv_lammax = 0, tv_lammin = 0, tv_vent = 0;
    TR mu_c = 0, lamc = 0, mu_r = 0, lamr = 0, cdistr = 0, logn0r = 0;
    TR epsi = 0, epsr = 0, epsi_tot = 0;
    TR rho_qm_cloud = TR(400);
    bool wet = false;

    const bool skip_micro = !(dge(inc.qc, C::QSMALL) || dge(inc.qr, C::QSMALL) || dge(inc.qi, C::QSMALL));
    if (!skip_micro) {
      get_time_space_phys_variables<TR>(T, pres, rho, qvsl, qvsi, v);
      {
        const TR n_in = TR(inc.nc);
        TR n_out = n_in;
        get_cloud_dsd2<TR>(TR(inc.qc), n_out, mu_c, rho, lamc);
        apply_n_adjust(inc.nc, n_in, n_out);
        s.nc = inc.nc * cld_l;
      }
      {
        const TR n_in = TR(inc.nr);
        TR n_out = n_in;
        get_rain_dsd2<TR>(TR(inc.qr), n_out, mu_r, lamr, rt);
        apply_n_adjust(inc.nr, n_in, n_out);
        if (dge(inc.qr, C::QSMALL)) {
          cdistr = TR(inc.nr) / TR(rt.g_mur1);
          logn0r = m_log10(cdistr) + (mu_r + TR(1)) * m_log10(lamr);
        }
        s.nr = inc.nr * cld_r;
      }
      impose_max_total_ni(inc.ni, rt.max_total_ni, inv_rho);
      if (dge(inc.qi, C::QSMALL)) {
        inc.ni = dmax_c(inc.ni, C::NSMALL);
        inc.nr = dmax_c(inc.nr, C::NSMALL);
        const TR rhop = calc_bulk_rho_rime(inc.qi, inc.qm, inc.bm, rt);
        s.qm = inc.qm * cld_i;
        s.bm = inc.bm * cld_i;
        TableIce<TR> ti;
        lookup_ice<TR>(TR(inc.qi), TR(inc.ni), TR(inc.qm), rhop, ti);
        TableRain<TR> trn;
        lookup_rain<TR>(TR(inc.qr), TR(inc.nr), trn);
        TR ta[4], tc[4];
        apply_table_ice4<TR>(tb, ti, 0, ta); /* columns 0, 1, 6, 7 */
        apply_table_ice4<TR>(tb, ti, 4, tc); /* columns 2, 3, 4, 9 */
        tv_fallspd = ta[1];
        tv_selfcol = tc[0];
        tv_qc2qi = tc[1];
        tv_melt = tc[2];
        tv_lammax = ta[2];
        tv_lammin = ta[3];
        tv_vent = tc[3];
        if (dge(inc.qr, C::QSMALL)) {
          tv_nr = apply_table_coll<TR>(0, tb, ti, trn);
          tv_qr2qi = apply_table_coll<TR>(1, tb, ti, trn);
        }
        inc.ni = vmin(inc.ni, tv_lammax * inc.ni);
        inc.ni = vmax(inc.ni, tv_lammin * inc.ni);
      }
      const TR qi_r = inc.qi, qc_r = inc.qc, ni_r = inc.ni, nc_r = inc.nc, qr_r = inc.qr;
      const double dT0 = T - C::Tmelt;
      const double dqv0 = C::ep_2 * esat0 / vmax(pres, 1.e-3) - s.qv;
      if (do_ice) {
        ice_cldliq_collection<TR>(rho, T, rhofaci, tv_qc2qi, qi_r, qc_r, ni_r, nc_r, r, rt);
        ice_rain_collection<TR>(rho, T, rhofaci, logn0r, tv_nr, tv_qr2qi, qi_r, ni_r, qr_r, r, rt);
        ice_self_collection<TR>(rho, rhofaci, tv_selfcol, v.eii, TR(inc.qm), qi_r, ni_r, r);
      }
      ice_melting<TR>(rho, dT0, dqv0, rhofaci, tv_melt, tv_vent, v, qi_r, ni_r, r);
      if (do_ice) {
        wet = ice_cldliq_wet_growth<TR>(rho, dT0, dqv0, rhofaci, tv_melt, tv_vent, v, qc_r, qi_r, ni_r, qr_r, r);
      }
      /* ice_relaxation_timescale, p3_ice_relaxation_timescale_impl.hpp:9-37 */
      if (dge(inc.qi, C::QSMALL) && dlt(T, C::Tmelt)) {
        epsi = ((tv_melt + tv_vent * m_cbrt(v.sc) * m_sqrt(rhofaci * rho / v.mu)) * TR(2.0) * TR(C::Pi) * rho *
                v.dv) * ni_r;
        epsi_tot = epsi_tot + epsi;
      } else {
        epsi = TR(0);
      }
      rho_qm_cloud = calc_rime_density<TR>(T, rhofaci, tv_fallspd, acn, lamc, mu_c, qc_r, r.qc2qi_collect_tend);
      if (do_ice) {
        cldliq_immersion_freezing<TR>(T, lamc, mu_c, nc_r, qc_r, r, rt);
        rain_immersion_freezing<TR>(T, lamr, mu_r, cdistr, qr_r, r, rt);
      }
      /* calc_liq_relaxation_timescale, p3_calc_liq_relaxation_timescale_impl.hpp:13-43 */
      if (dge(inc.qr, C::QSMALL)) {
        Table3<TR> t3;
        lookup3<TR>(mu_r, lamr, rt, t3);
        epsr = TR(2) * TR(C::Pi) * cdistr * rho * v.dv *
               (TR(C::f1r) * TR(rt.g_mur2) / lamr +
                TR(C::f2r) * m_sqrt(rho / v.mu) * m_cbrt(v.sc) * apply_table3<TR>(tb, tb.revap, t3));
      }
      evaporate_rain(inc.qr, inc.qc, inc.nr, inc.qi, cld_l, cld_r, s.qv, in.qv_prev[o], qvsl, qvsi, v.ab, v.abi,
                     epsr, epsi_tot, T, in.t_prev[o], v.dqsdt, dt, r.qr2qv_evap_tend, r.nr_evap_tend);
      if (do_ice) {
        ice_deposition_sublimation(inc.qi, inc.ni, T, qvsl, qvsi, epsi, v.abi, s.qv, inv_dt, r.qv2qi_vapdep_tend,
                                   r.qi2qv_sublim_tend, r.ni_sublim_tend, r.qc2qi_berg_tend);
      }
    }
    if (do_ice) {
      ice_nucleation<TR>(T, inv_rho, s.ni, in.ni_activated[o], qvssi, inv_dt, predictNc, prescribedCCN, r, rt);
    }
    cloud_water_autoconversion<TR>(rho, inc.qc, inc.nc, r, rt);
    if (dge(inc.qc, C::QSMALL)) r.nc_selfcollect_tend = TR(0);
    cloud_rain_accretion<TR>(inc.qc, inc.nc, inc.qr, r, rt);
    rain_self_collection<TR>(rho, inc.qr, inc.nr, r, rt);
    back_to_cell_average<TR>(cld_l, cld_r, cld_i, r);

    water_conservation<double>(s.qc, s.qr, s.qi, dt, r);
    number_conservation<double>(s.nc, s.nr, s.ni, dt, r);
    ice_supersat_conservation(r, cld_i, s.qv, qvsi, s.th / inv_exner, dt);
    prevent_liq_supersaturation(pres, T, s.qv, dt, r, err);
    update_prognostics(r, inv_exner, predictNc, prescribedCCN, wet, dt, rho_qm_cloud, inv_rho, s);

    in.qv2qi_depos_tend[o] = r.qv2qi_vapdep_tend - r.qi2qv_sublim_tend + r.qv2qi_nucleat_tend;
    in.precip_total_tend[o] = r.qc2qr_accret_tend + r.qc2qr_autoconv_tend + r.qc2qr_ice_shed_tend + r.qc2qi_collect_tend;
    in.nevapr[o] = r.qi2qv_sublim_tend + r.qr2qv_evap_tend;
    in.vap_ice_exchange[o] = r.qv2qi_vapdep_tend - r.qi2qv_sublim_tend + r.qv2qi_nucleat_tend;
    in.vap_liq_exchange[o] = -r.qr2qv_evap_tend;
    in.liq_ice_exchange[o] = r.qc2qi_hetero_freeze_tend + r.qr2qi_immers_freeze_tend - r.qi2qr_melt_tend +
                             r.qc2qi_berg_tend + r.qc2qi_collect_tend + r.qr2qi_collect_tend;

    hydro |= clip_to_vapour(s, inv_exner);
    double ni_incld = s.ni / cld_i;
    impose_max_total_ni(ni_incld, rt.max_total_ni, inv_rho);
    s.ni = ni_incld * cld_i;
    in.qc[o] = s.qc; in.nc[o] = s.nc; in.qr[o] = s.qr; in.nr[o] = s.nr;
    in.qi[o] = s.qi; in.qm[o] = s.qm; in.ni[o] = s.ni; in.bm[o] = s.bm;
    in.qv[o] = s.qv; in.th[o] = s.th;
  }
  }
  if (!group_any<LANES>(mask, hydro)) {
    if (lane == 0) in.cflag[col] = 0;
    return;
  }
  for (int k = lane; k < nk; k += LANES) {
    scr_at(in, S_TATM, col)[k] = SMA(A_TATM, k);
    if constexpr (kF64) {
      scr_at(in, S_RHO, col)[k] = SMA(A_RHO, k);
      scr_at(in, S_RHOFACR, col)[k] = SMA(A_RHOFACR, k);
      scr_at(in, S_RHOFACI, col)[k] = SMA(A_RHOFACI, k);
      scr_at(in, S_ACN, col)[k] = SMA(A_ACN, k);
    } else {
      scr_f(in, S_RHO, col)[k] = SMF(A_RHO)[k];
      scr_f(in, S_RHOFACR, col)[k] = SMF(A_RHOFACR)[k];
      scr_f(in, S_RHOFACI, col)[k] = SMF(A_RHOFACI)[k];
      scr_f(in, S_ACN, col)[k] = SMF(A_ACN)[k];
    }
  }
  if (lane == 0) in.cflag[col] = 1;
#undef SMA
#undef SMF
}

/* K2 (FP64 form): cloud, rain and ice sedimentation of one column that went
 * on past part2. */
template <class TR, int LANES>
__device__ void p3_sed(const Inst& in, const int col, const KParams<TR>& kp, const Tabs<TR>& tb,
                       double* __restrict__ sm, uint32_t& err) {
  static_assert(sizeof(TR) == sizeof(double), "the FP32-bulk sedimentation is p3_sed_bulk");
  if (in.cflag[col] == 0) return;
  const RuntimeDev& rt = kp.rt;
  const unsigned mask = group_mask<LANES>();
  const int lane = threadIdx.x & (LANES - 1);
  const int nk = in.nlev;
  const int S = kp.sm_stride;
  const int64_t co = int64_t(col) * in.ld;
  const int64_t ci = int64_t(col) * in.ld_int;
  const double dt = in.dt;
  const double inv_dt = 1 / dt;
  const bool predictNc = in.predictNc != 0;
  const int kbot = nk - 1;
#define SMA(a, k) sm[(a)*S + (k)]
  for (int k = lane; k < nk; k += LANES) {
    const double rho = scr_at(in, S_RHO, col)[k];
    SMA(B_RHO, k) = rho;
    SMA(B_INVRHO, k) = 1 / rho;
    SMA(B_INVDZ, k) = 1 / in.dz[co + k];
  }
  double precip_liq_surf = 0, precip_ice_surf = 0;

  /* ---------------- phase 3: sedimentation ---------------- */
  /* Shared arrays during sedimentation: V1/V2 fall speeds (re-using the
   * part2-only saturation arrays), R0..R3 the species state, CLD the
   * species' cloud fraction (cloud and ice re-use A_QVSSI; rain re-uses A_ACN,
   * free once cloud sedimentation is done), PF the rain flux accumulator. */
  double* const V1 = &SMA(B_V1, 0);
  double* const V2 = &SMA(B_V2, 0);
  double* const PF = &SMA(B_R2, 0);
  double* const R0 = &SMA(B_R0, 0);
  double* const R1 = &SMA(B_R1, 0);
  double* const R2 = &SMA(B_R2, 0);
  double* const R3 = &SMA(B_R3, 0);
  double* const CLD = &SMA(B_CLD, 0);
  double* const FAC = &SMA(B_FAC, 0);
  const double* const RHO = &SMA(B_RHO, 0);
  const double* const INVRHO = &SMA(B_INVRHO, 0);
  const double* const INVDZ = &SMA(B_INVDZ, 0);

#pragma unroll 1
  for (int sp = 0; sp < 3; ++sp) {
    double* g0 = sp == 0 ? in.qc : (sp == 1 ? in.qr : in.qi);
    double* g1 = sp == 0 ? in.nc : (sp == 1 ? in.nr : in.ni);
    const double* cldp = sp == 0 ? in.cld_frac_l : (sp == 1 ? in.cld_frac_r : in.cld_frac_i);
    const int sfac = sp == 0 ? S_ACN : (sp == 1 ? S_RHOFACR : S_RHOFACI);
    const double* const facp = scr_at(in, sfac, col);
    const int nfield = sp == 0 ? (predictNc ? 2 : 1) : (sp == 1 ? 2 : 4);

    /* load the species into shared memory; find top / bottom (p3_find_impl.hpp) */
    int my_top = 1 << 30, my_bot = -1;
    for (int k = lane; k < nk; k += LANES) {
      const double q = g0[co + k];
      R0[k] = q;
      R1[k] = g1[co + k];
      CLD[k] = cldp[co + k];
      FAC[k] = facp[k];
      if (sp == 2) {
        R2[k] = in.qm[co + k];
        R3[k] = in.bm[co + k];
      }
      if (dge(q, C::QSMALL)) {
        my_top = min(my_top, k);
        my_bot = max(my_bot, k);
      }
    }
    const int k_qxtop = group_min_int<LANES>(mask, my_top);
    int k_qxbot = group_max_int<LANES>(mask, my_bot);
    if (k_qxbot < 0) continue; /* species absent (group-uniform) */
    if (sp == 1) {
      for (int k = lane; k <= nk; k += LANES) PF[k] = 0;
    }
    __syncwarp(mask);

    /* From here on lane l owns levels k_qxtop + l + j*LANES in both the
     * fall-speed pass and the flux walk, so only shuffles cross lanes. */
    double dt_left = dt, prt_accum = 0.0;
    bool first = true;
    int nsub = 0;
    while (dgt(dt_left, C::dt_left_tol)) {
      if (++nsub > kMaxSubsteps) {
        err |= kErrSubstep;
        break;
      }
      /* fall speeds on [k_qxtop, k_qxbot] and the Courant maximum */
      double lmax = 0.0;
      for (int k = k_qxtop + lane; k <= k_qxbot; k += LANES) {
        const double cld = CLD[k];
        double v1 = 0, v2 = 0;
        if (sp == 0) {
          double qc_incld, nc_incld;
          if (first) {
            const double inv_cld = 1 / cld;
            if (dge(R0[k], C::QSMALL)) {
              qc_incld = R0[k] * inv_cld;
              nc_incld = dmax0(R1[k] * inv_cld);
            } else {
              qc_incld = 0;
              nc_incld = 0;
            }
            qc_incld = dmin_c(qc_incld, C::incloud_limit);
          } else {
            qc_incld = R0[k] / cld;
            nc_incld = R1[k] / cld;
          }
          if (dgt(qc_incld, C::QSMALL)) {
            TR mu_c, lamc;
            const TR n_in = TR(nc_incld);
            TR n_out = n_in;
            get_cloud_dsd2<TR>(TR(qc_incld), n_out, mu_c, TR(RHO[k]), lamc);
            R1[k] = double(n_out) * cld;
            /* Stokes fall speeds, p3_cloud_sed_impl.hpp:99-103, with
             * Gamma(6+mu)/Gamma(4+mu) = (5+mu)(4+mu) and
             * Gamma(3+mu)/Gamma(1+mu) = (2+mu)(1+mu) (bcn = 2) */
            const TR dum = TR(1) / (lamc * lamc);
            const TR acn = TR(FAC[k]);
            v1 = double(acn * ((TR(5) + mu_c) * (TR(4) + mu_c)) * dum);
            if (predictNc) v2 = double(acn * ((TR(2) + mu_c) * (TR(1) + mu_c)) * dum);
            lmax = dmax_nn(lmax, v1 * dt_left * INVDZ[k]);
          }
        } else if (sp == 1) {
          double qr_incld, nr_incld;
          if (first) {
            const double inv_cld = 1 / cld;
            if (dge(R0[k], C::QSMALL)) {
              qr_incld = R0[k] * inv_cld;
              nr_incld = dmax0(R1[k] * inv_cld);
            } else {
              qr_incld = 0;
              nr_incld = 0;
            }
            qr_incld = dmin_c(qr_incld, C::precip_limit);
          } else {
            qr_incld = R0[k] / cld;
            nr_incld = R1[k] / cld;
          }
          if (dgt(qr_incld, C::QSMALL)) {
            TR mu_r = 0, lamr;
            const TR n_in = TR(nr_incld);
            TR n_out = n_in;
            get_rain_dsd2<TR>(TR(qr_incld), n_out, mu_r, lamr, rt);
            Table3<TR> t3;
            lookup3<TR>(mu_r, lamr, rt, t3);
            const TR rhofacr = TR(FAC[k]);
            v1 = double(apply_table3<TR>(tb, tb.vm, t3) * rhofacr);
            v2 = double(apply_table3<TR>(tb, tb.vn, t3) * rhofacr);
            R1[k] = double(n_out) * cld;
            lmax = dmax_nn(lmax, v1 * dt_left * INVDZ[k]);
          }
        } else {
          {
            double qi_incld, ni_incld, qm_incld, bm_incld;
            if (first) {
              const double inv_cld = 1 / cld;
              if (dge(R0[k], C::QSMALL)) {
                qi_incld = R0[k] * inv_cld;
                ni_incld = dmax0(R1[k] * inv_cld);
              } else {
                qi_incld = 0;
                ni_incld = 0;
              }
              if (dge(R0[k], C::QSMALL) && dge(R2[k], C::QSMALL)) {
                qm_incld = R2[k] * inv_cld;
                bm_incld = dmax0(R3[k] * (1 / in.cld_frac_l[co + k]));
              } else {
                qm_incld = 0;
                bm_incld = 0;
              }
              qi_incld = dmin_c(qi_incld, C::incloud_limit);
              bm_incld = dmin_c(bm_incld, C::incloud_limit);
            } else {
              qi_incld = R0[k] / cld;
              ni_incld = R1[k] / cld;
              qm_incld = R2[k] / cld;
              bm_incld = R3[k] / cld;
            }
            if (dgt(qi_incld, C::QSMALL)) {
              ni_incld = dmax_c(ni_incld, C::NSMALL);
              const double rhop = calc_bulk_rho_rime(qi_incld, qm_incld, bm_incld, rt);
              R2[k] = qm_incld * cld;
              R3[k] = bm_incld * cld;
              TableIce<TR> ti;
              lookup_ice<TR>(TR(qi_incld), TR(ni_incld), TR(qm_incld), TR(rhop), ti);
              TR tv[4];
              apply_table_ice4<TR>(tb, ti, 0, tv); /* columns 0, 1, 6, 7 */
              ni_incld = vmin(ni_incld, double(tv[2]) * ni_incld);
              ni_incld = vmax(ni_incld, double(tv[3]) * ni_incld);
              R1[k] = ni_incld * cld;
              const TR rhofaci = TR(FAC[k]);
              v1 = double(TR(rt.ice_sedimentation_factor) * tv[1] * rhofaci);
              v2 = double(TR(rt.ice_sedimentation_factor) * tv[0] * rhofaci);
              lmax = dmax_nn(lmax, v1 * dt_left * INVDZ[k]);
            }
          }
        }
        V1[k] = v1;
        V2[k] = v2;
      }
      if (k_qxbot < kbot && lane == (k_qxbot + 1 - k_qxtop) % LANES) {
        V1[k_qxbot + 1] = 0; /* the cell receiving the leading edge has no fall speed */
        V2[k_qxbot + 1] = 0;
      }
      const double Co_max = group_max_nn<LANES>(mask, lmax);
      if (!(Co_max >= 0) || Co_max > 2.0e9) {
        err |= kErrNumeric;
        break;
      }

      /* generalized_sedimentation + calc_first_order_upwind_step (kdir = -1):
       * fluxes from start-of-substep values, inflow from the level above by a
       * shuffle (carried across chunks), zero inflow at k_qxtop. */
      const int tmpint1 = static_cast<int>(Co_max + 1);
      const double dt_sub = dt_left / tmpint1;
      const int k_temp = (k_qxbot == kbot) ? k_qxbot : k_qxbot + 1;
      double carry0 = 0, carry1 = 0, carry2 = 0, carry3 = 0, flux_bot = 0;
      for (int base = k_qxtop; base <= k_temp; base += LANES) {
        const int k = base + lane;
        const bool act = k <= k_temp;
        double f0 = 0, f1 = 0, f2 = 0, f3 = 0;
        if (act) {
          const double rho = RHO[k];
          const double v1 = V1[k];
          f0 = v1 * R0[k] * rho;
          if (nfield > 1) f1 = V2[k] * R1[k] * rho;
          if (nfield > 2) {
            f2 = v1 * R2[k] * rho;
            f3 = v1 * R3[k] * rho;
          }
        }
        double u0 = __shfl_up_sync(mask, f0, 1, LANES);
        double u1 = __shfl_up_sync(mask, f1, 1, LANES);
        double u2 = 0, u3 = 0;
        if (nfield > 2) {
          u2 = __shfl_up_sync(mask, f2, 1, LANES);
          u3 = __shfl_up_sync(mask, f3, 1, LANES);
        }
        if (lane == 0) {
          u0 = carry0; u1 = carry1; u2 = carry2; u3 = carry3;
        }
        if (act) {
          const double invdz = INVDZ[k], irho = INVRHO[k];
          R0[k] += ((u0 - f0) * invdz) * dt_sub * irho;
          if (nfield > 1) R1[k] += ((u1 - f1) * invdz) * dt_sub * irho;
          if (nfield > 2) {
            R2[k] += ((u2 - f2) * invdz) * dt_sub * irho;
            R3[k] += ((u3 - f3) * invdz) * dt_sub * irho;
          }
          if (sp == 1) PF[k + 1] += f0;
          if (k == kbot) flux_bot = f0;
        }
        carry0 = __shfl_sync(mask, f0, LANES - 1, LANES);
        carry1 = __shfl_sync(mask, f1, LANES - 1, LANES);
        if (nfield > 2) {
          carry2 = __shfl_sync(mask, f2, LANES - 1, LANES);
          carry3 = __shfl_sync(mask, f3, LANES - 1, LANES);
        }
      }
      if (k_qxbot == kbot) {
        const int owner = (kbot - k_qxtop) % LANES;
        prt_accum += __shfl_sync(mask, flux_bot, owner, LANES) * dt_sub;
      } else {
        k_qxbot += 1;
      }
      dt_left -= dt_sub;
      first = false;
    }
    if (sp == 0) precip_liq_surf = prt_accum * C::INV_RHO_H2O * inv_dt;
    else if (sp == 1) precip_liq_surf += prt_accum * C::INV_RHO_H2O * inv_dt;
    else precip_ice_surf += prt_accum * C::INV_RHO_H2O * inv_dt;

    __syncwarp(mask);
    for (int k = lane; k < nk; k += LANES) {
      g0[co + k] = R0[k];
      g1[co + k] = R1[k];
      if (sp == 2) {
        in.qm[co + k] = R2[k];
        in.bm[co + k] = R3[k];
      }
    }
    if (sp == 1) {
      for (int k = lane; k <= nk; k += LANES) in.precip_liq_flux[ci + k] = PF[k];
    }
    __syncwarp(mask);
  }
  if (lane == 0) {
    in.precip_liq_surf[col] = precip_liq_surf;
    in.precip_ice_surf[col] = precip_ice_surf;
  }

#undef SMA
}

/* K2 of the FP32-bulk form.  Same algorithm and order as p3_sed.  Fall
 * speeds, density, fall-speed factors, 1/dz and an FP32 shadow of each
 * species field live in FP32 shared arrays and drive the fluxes; the Courant
 * maximum is taken in FP32.
 *
 * The accumulation of the flux divergence is carried by time-integrated face
 * fluxes: G_k = sum over substeps of F_k dt_sub, the flux leaving level k
 * downward, kept as a double-float (~48 significant bits).  A level's FP64
 * state after any number of substeps is R_k = B_k + (g / dpres_k) (G_{k-1} -
 * G_k), with B_k its value at the start (kept in the species' global array).
 * So a substep costs one double-float multiply-add (FP32 instructions only)
 * per field and level; both neighbours of a face read the same G, so the
 * column's mass telescopes exactly, and the surface precipitation is the
 * bottom face's G.  Where a limiter rewrites a level's state to x during the
 * walk, B_k is reset so that R_k = x at that moment. */
template <int LANES>
__device__ void p3_sed_bulk(const Inst& in, const int col, const KParams<float>& kp, const Tabs<float>& tb,
                            double* __restrict__ sm, uint32_t& err) {
  if (in.cflag[col] == 0) return;
  const RuntimeDev& rt = kp.rt;
  const unsigned mask = group_mask<LANES>();
  const int lane = threadIdx.x & (LANES - 1);
  const int nk = in.nlev;
  const int S = kp.sm_stride;
  const int64_t co = int64_t(col) * in.ld;
  const int64_t ci = int64_t(col) * in.ld_int;
  const double dt = in.dt;
  const double inv_dt = 1 / dt;
  const bool predictNc = in.predictNc != 0;
  const int kbot = nk - 1;
#define SMA(a, k) sm[(a)*S + (k)]
  /* kSedBulkSlots slots of S doubles; two float arrays share a slot.  The
   * density is read from the hand-over row (a float per level, L1-resident
   * during the walk) rather than held in a slot. */
  const float* const RHOf = scr_f(in, S_RHO, col);
  float* const FACf = reinterpret_cast<float*>(&SMA(0, 0));
  float* const CLDf = FACf + S;
  double* const COEF = &SMA(1, 0); /* g / dpres */
  float* const INVDZf = reinterpret_cast<float*>(&SMA(2, 0));
  float* const COEFf = INVDZf + S;
  /* Fields in pairs for the packed FP32 instructions: FP32 shadows of
   * fields (0, 1) and (2, 3), the fall speeds (V1, V2), and the time-
   * integrated face fluxes of fields (0, 1) and (2, 3) as double-floats
   * {hi_a, hi_b, lo_a, lo_b} (two slots each). */
  float2* const R23 = reinterpret_cast<float2*>(&SMA(3, 0));
  float2* const V12 = reinterpret_cast<float2*>(&SMA(4, 0));
  float2* const R01 = reinterpret_cast<float2*>(&SMA(5, 0));
  float4* const G01 = reinterpret_cast<float4*>(&SMA(6, 0));
  float4* const G23 = reinterpret_cast<float4*>(&SMA(8, 0));
  float2* const PF = reinterpret_cast<float2*>(G23); /* rain flux sum (rain has two fields) */
  /* the double-float G of field f at level k, as a double */
  auto g_value = [&](int f, int k) -> double {
    const float4 g = (f < 2 ? G01 : G23)[k];
    return (f & 1) ? dfloat_value(make_float2(g.y, g.w)) : dfloat_value(make_float2(g.x, g.z));
  };
  auto r_set = [&](int f, int k, float v) {
    float2& r = (f < 2 ? R01 : R23)[k];
    if (f & 1) {
      r.y = v;
    } else {
      r.x = v;
    }
  };
  /* Top and bottom of the three species (p3_find_impl.hpp) in one pass on
   * the integer pipes.  A species only ever changes the levels from its top
   * down to its final leading edge, so conversions, flux coefficients and the
   * FP64 state rebuild are limited to those levels; the levels above the top
   * and below the leading edge keep their values. */
  int top_c = 1 << 30, top_r = 1 << 30, top_i = 1 << 30, bot_c = -1, bot_r = -1, bot_i = -1;
  for (int k = lane; k < nk; k += LANES) {
    if (dge(in.qc[co + k], C::QSMALL)) { top_c = min(top_c, k); bot_c = k; }
    if (dge(in.qr[co + k], C::QSMALL)) { top_r = min(top_r, k); bot_r = k; }
    if (dge(in.qi[co + k], C::QSMALL)) { top_i = min(top_i, k); bot_i = k; }
  }
  top_c = group_min_int<LANES>(mask, top_c);
  top_r = group_min_int<LANES>(mask, top_r);
  top_i = group_min_int<LANES>(mask, top_i);
  bot_c = group_max_int<LANES>(mask, bot_c);
  bot_r = group_max_int<LANES>(mask, bot_r);
  bot_i = group_max_int<LANES>(mask, bot_i);
  const int k_first = min(top_c, min(top_r, top_i));
  for (int k = k_first + lane; k < nk; k += LANES) {
    const double coef = C::gravit * rcp_newton(in.dpres[co + k]);
    INVDZf[k] = 1.0f / float(in.dz[co + k]);
    COEF[k] = coef;
    COEFf[k] = float(coef);
  }
  double precip_liq_surf = 0, precip_ice_surf = 0;

  /* The three species, each with its code specialised (field count, tables,
   * limiters) at compile time. */
  auto species = [&](auto sp_tag) {
    constexpr int sp = decltype(sp_tag)::value;
    double* const B0 = sp == 0 ? in.qc : (sp == 1 ? in.qr : in.qi);
    double* const B1 = sp == 0 ? in.nc : (sp == 1 ? in.nr : in.ni);
    double* const B2 = in.qm;
    double* const B3 = in.bm;
    double* const Bf[4] = {B0, B1, B2, B3};
    const double* cldp = sp == 0 ? in.cld_frac_l : (sp == 1 ? in.cld_frac_r : in.cld_frac_i);
    const int sfac = sp == 0 ? S_ACN : (sp == 1 ? S_RHOFACR : S_RHOFACI);
    const float* const facp = scr_f(in, sfac, col);
    const int nfield = sp == 0 ? (predictNc ? 2 : 1) : (sp == 1 ? 2 : 4);
    const int nstate = sp == 2 ? 4 : 2; /* fields that limiters may rewrite */
    /* R_k := x now (k owned by this lane; G_{k-1} belongs to the lane above
     * and is final for this substep after the warp barrier) */
    auto set_state = [&](int f, int k, double x) {
      const double gin = k > 0 ? g_value(f, k - 1) : 0.0;
      Bf[f][co + k] = x - COEF[k] * (gin - g_value(f, k));
      r_set(f, k, float(x));
    };

    const int k_qxtop = sp == 0 ? top_c : (sp == 1 ? top_r : top_i);
    int k_qxbot = sp == 0 ? bot_c : (sp == 1 ? bot_r : bot_i);
    if (k_qxbot < 0) return; /* species absent (group-uniform) */
    /* the walk and the rebuild read G one level above the top */
    for (int k = max(k_qxtop - 1, 0) + lane; k < nk; k += LANES) {
      G01[k] = make_float4(0.f, 0.f, 0.f, 0.f);
      if (sp == 2) G23[k] = make_float4(0.f, 0.f, 0.f, 0.f);
      if (k >= k_qxtop) {
        R01[k] = make_float2(float(B0[co + k]), float(B1[co + k]));
        CLDf[k] = float(cldp[co + k]);
        FACf[k] = facp[k];
        if (sp == 2) R23[k] = make_float2(float(B2[co + k]), float(B3[co + k]));
      }
    }
    if (sp == 1) {
      for (int k = k_qxtop + 1 + lane; k <= nk; k += LANES) PF[k] = make_float2(0.f, 0.f);
    }
    __syncwarp(mask);

    /* The substep schedule is FP32 scalar work: one dt_sub scales every face
     * flux of a substep alike, so its rounding only changes that substep's
     * length by ~1e-7 relative and leaves the mass budget exact. */
    float dt_left = float(dt);
    bool first = true;
    int nsub = 0;
    while (dt_left > float(C::dt_left_tol)) {
      if (++nsub > kMaxSubsteps) {
        err |= kErrSubstep;
        break;
      }
      float lmax = 0.0f; /* max of V / dz; the Courant number is that times dt_left */
      for (int k = k_qxtop + lane; k <= k_qxbot; k += LANES) {
        float v1 = 0, v2 = 0;
        bool fall = false;
        /* In-cloud values in FP32.  The first substep applies the reference's
         * thresholds and limits (and the bm quirk: bm_incld uses 1/cld_frac_l);
         * the FP64 state is rewritten wherever a limiter made an in-cloud value
         * differ from the plain one. */
        const float cldf = CLDf[k];
        const float icf = 1.0f / cldf;
        if (sp == 0) {
          const float2 r01 = R01[k];
          const float n_plain = r01.y * icf;
          float qc_f = r01.x * icf, n_in = n_plain;
          if (first) {
            if (dge(B0[co + k], C::QSMALL)) {
              n_in = vmax(n_in, 0.0f);
            } else {
              qc_f = 0;
              n_in = 0;
            }
            qc_f = vmin(qc_f, float(C::incloud_limit));
          }
          if (qc_f > float(C::QSMALL)) {
            float mu_c, lamc;
            float n_out = n_in;
            get_cloud_dsd2<float>(qc_f, n_out, mu_c, RHOf[k], lamc);
            if (n_out != n_plain) {
              set_state(1, k, f2d(n_out) * f2d(cldf));
            }
            const float dum = 1.0f / (lamc * lamc);
            v1 = FACf[k] * ((5.0f + mu_c) * (4.0f + mu_c)) * dum;
            if (predictNc) v2 = FACf[k] * ((2.0f + mu_c) * (1.0f + mu_c)) * dum;
            fall = true;
          }
        } else if (sp == 1) {
          const float2 r01 = R01[k];
          const float n_plain = r01.y * icf;
          float qr_f = r01.x * icf, n_in = n_plain;
          if (first) {
            if (dge(B0[co + k], C::QSMALL)) {
              n_in = vmax(n_in, 0.0f);
            } else {
              qr_f = 0;
              n_in = 0;
            }
            qr_f = vmin(qr_f, float(C::precip_limit));
          }
          if (qr_f > float(C::QSMALL)) {
            float mu_r = 0, lamr;
            float n_out = n_in;
            get_rain_dsd2<float>(qr_f, n_out, mu_r, lamr, rt);
            Table3<float> t3;
            lookup3<float>(mu_r, lamr, rt, t3);
            v1 = apply_table3<float>(tb, tb.vm, t3) * FACf[k];
            v2 = apply_table3<float>(tb, tb.vn, t3) * FACf[k];
            if (n_out != n_plain) {
              set_state(1, k, f2d(n_out) * f2d(cldf));
            }
            fall = true;
          }
        } else {
          const float2 r01 = R01[k], r23 = R23[k];
          const float ni_plain = r01.y * icf, qm_plain = r23.x * icf, bm_plain = r23.y * icf;
          float qi_f = r01.x * icf, ni_f = ni_plain, qm_f = qm_plain, bm_f = bm_plain;
          if (first) {
            if (dge(B0[co + k], C::QSMALL)) {
              ni_f = vmax(ni_f, 0.0f);
            } else {
              qi_f = 0;
              ni_f = 0;
            }
            if (dge(B0[co + k], C::QSMALL) && dge(B2[co + k], C::QSMALL)) {
              bm_f = vmax(r23.y * (1.0f / float(in.cld_frac_l[co + k])), 0.0f);
            } else {
              qm_f = 0;
              bm_f = 0;
            }
            qi_f = vmin(qi_f, float(C::incloud_limit));
            bm_f = vmin(bm_f, float(C::incloud_limit));
          }
          if (qi_f > float(C::QSMALL)) {
            const float ni_l = vmax(ni_f, float(C::NSMALL));
            const float rhop = calc_bulk_rho_rime<float>(qi_f, qm_f, bm_f, rt);
            if (qm_f != qm_plain) {
              set_state(2, k, f2d(qm_f) * f2d(cldf));
            }
            if (bm_f != bm_plain) {
              set_state(3, k, f2d(bm_f) * f2d(cldf));
            }
            TableIce<float> ti;
            lookup_ice<float>(qi_f, ni_l, qm_f, rhop, ti);
            float tv[4];
            ice_table4_f32<kIceSedCols>(tb.ice, ti, 0, tv); /* columns 0, 1, 6, 7, packed copy */
            float n2 = vmin(ni_l, tv[2] * ni_l);
            n2 = vmax(n2, tv[3] * n2);
            if (n2 != ni_plain) {
              set_state(1, k, f2d(n2) * f2d(cldf));
            }
            const float f = rt.f.ice_sedimentation_factor * FACf[k];
            v1 = f * tv[1];
            v2 = f * tv[0];
            fall = true;
          }
        }
        V12[k] = make_float2(v1, v2);
        if (fall) lmax = vmax(lmax, v1 * INVDZf[k]);
      }
      if (k_qxbot < kbot && lane == (k_qxbot + 1 - k_qxtop) % LANES) {
        V12[k_qxbot + 1] = make_float2(0.f, 0.f); /* the cell receiving the leading edge has no fall speed */
      }
      const float Co_max = group_max_nn<LANES>(mask, lmax) * dt_left;
      if (!(Co_max >= 0.0f) || Co_max > 2.0e9f) {
        err |= kErrNumeric;
        break;
      }
      const int tmpint1 = static_cast<int>(Co_max + 1.0f);
      const float dt_sub = dt_left / float(tmpint1);
      const int k_temp = (k_qxbot == kbot) ? k_qxbot : k_qxbot + 1;
      /* FP32 fluxes from the shadows; double-float time-integrated face
       * fluxes; the shadows follow with the FP32 flux divergence.  Fields go
       * in pairs through the packed FP32 instructions (same operations and
       * rounding as the scalar form). */
      float2 c01 = make_float2(0.f, 0.f), c23 = make_float2(0.f, 0.f);
      for (int base = k_qxtop; base <= k_temp; base += LANES) {
        const int k = base + lane;
        const bool act = k <= k_temp;
        float2 f01 = make_float2(0.f, 0.f), f23 = make_float2(0.f, 0.f);
        if (act) {
          const float2 rho2 = f2splat(RHOf[k]);
          const float2 v = V12[k];
          f01 = __fmul2_rn(__fmul2_rn(v, R01[k]), rho2);
          if (nfield < 2) f01.y = 0.f;
          if (nfield > 2) f23 = __fmul2_rn(__fmul2_rn(f2splat(v.x), R23[k]), rho2);
        }
        float2 u01, u23 = make_float2(0.f, 0.f);
        u01.x = __shfl_up_sync(mask, f01.x, 1, LANES);
        u01.y = nfield > 1 ? __shfl_up_sync(mask, f01.y, 1, LANES) : 0.f;
        if (nfield > 2) {
          u23.x = __shfl_up_sync(mask, f23.x, 1, LANES);
          u23.y = __shfl_up_sync(mask, f23.y, 1, LANES);
        }
        if (lane == 0) {
          u01 = c01;
          u23 = c23;
        }
        if (act) {
          const float2 coef2 = f2splat(COEFf[k] * dt_sub);
          dfloat2_add_prod(G01[k], f01, dt_sub);
          R01[k] = __ffma2_rn(__fadd2_rn(u01, f2neg(f01)), coef2, R01[k]);
          if (nfield > 2) {
            dfloat2_add_prod(G23[k], f23, dt_sub);
            R23[k] = __ffma2_rn(__fadd2_rn(u23, f2neg(f23)), coef2, R23[k]);
          }
          if (sp == 1) dfloat_add(PF[k + 1], f01.x);
        }
        c01.x = __shfl_sync(mask, f01.x, LANES - 1, LANES);
        c01.y = nfield > 1 ? __shfl_sync(mask, f01.y, LANES - 1, LANES) : 0.f;
        if (nfield > 2) {
          c23.x = __shfl_sync(mask, f23.x, LANES - 1, LANES);
          c23.y = __shfl_sync(mask, f23.y, LANES - 1, LANES);
        }
      }
      if (k_qxbot < kbot) k_qxbot += 1;
      dt_left -= dt_sub;
      first = false;
      __syncwarp(mask); /* G of the level above is read by set_state */
    }
    __syncwarp(mask);
    /* the bottom face's integral is what left the column: V is zero at the
     * leading edge, so G_kbot gains only in substeps where the species
     * reaches the surface */
    const double prt_accum = g_value(0, kbot);
    if (sp == 0) precip_liq_surf = prt_accum * C::INV_RHO_H2O * inv_dt;
    else if (sp == 1) precip_liq_surf += prt_accum * C::INV_RHO_H2O * inv_dt;
    else precip_ice_surf += prt_accum * C::INV_RHO_H2O * inv_dt;

    /* FP64 state: R_k = B_k + (g / dpres_k) (G_{k-1} - G_k), on the levels
     * from the top to the final leading edge (G is zero elsewhere) */
    /* G_{k-1} comes from the lane above (the same value that lane forms for
     * its own level); above the top it is zero: no flux enters there */
    double g_in[4] = {0.0, 0.0, 0.0, 0.0};
    for (int base = k_qxtop; base <= k_qxbot; base += LANES) {
      const int k = base + lane;
      const bool act = k <= k_qxbot;
#pragma unroll
      for (int f = 0; f < 4; ++f) {
        if (f < nstate) {
          const double g = act ? g_value(f, k) : 0.0;
          double gin = __shfl_up_sync(mask, g, 1, LANES);
          if (lane == 0) gin = g_in[f];
          if (act) Bf[f][co + k] = Bf[f][co + k] + COEF[k] * (gin - g);
          g_in[f] = __shfl_sync(mask, g, LANES - 1, LANES);
        }
      }
    }
    if (sp == 1) {
      /* interfaces above the top stay at part1's zero */
      for (int k = k_qxtop + 1 + lane; k <= nk; k += LANES) in.precip_liq_flux[ci + k] = dfloat_value(PF[k]);
    }
    __syncwarp(mask);
  };
  species(std::integral_constant<int, 0>{});
  species(std::integral_constant<int, 1>{});
  species(std::integral_constant<int, 2>{});
  if (lane == 0) {
    in.precip_liq_surf[col] = precip_liq_surf;
    in.precip_ice_surf[col] = precip_ice_surf;
  }
#undef SMA
}

/* K3: homogeneous freezing and p3_main_part3 of one column that went on past
 * part2. */
template <class TR, int LANES>
__device__ void p3_part3(const Inst& in, const int col, const KParams<TR>& kp, const Tabs<TR>& tb, const int inst_idx,
                         uint32_t& err) {
  if (in.cflag[col] == 0) return;
  const RuntimeDev& rt = kp.rt;
  const int lane = threadIdx.x & (LANES - 1);
  const int nk = in.nlev;
  const int64_t co = int64_t(col) * in.ld;
  const bool do_ice = rt.do_ice_production != 0;
  const double* const t_start = scr_at(in, S_TATM, col);
  constexpr bool kF64 = sizeof(TR) == sizeof(double);
  /* ---------------- phase 4: homogeneous freezing + p3_main_part3 ---------------- */
  for (int k = lane; k < nk; k += LANES) {
    const int64_t o = co + k;
    State s;
    s.qc = in.qc[o]; s.nc = in.nc[o]; s.qr = in.qr[o]; s.nr = in.nr[o];
    s.qi = in.qi[o]; s.qm = in.qm[o]; s.ni = in.ni[o]; s.bm = in.bm[o];
    s.qv = in.qv[o]; s.th = in.th[o];
    const double inv_exner = in.inv_exner[o];
    const double cld_l = in.cld_frac_l[o], cld_r = in.cld_frac_r[o], cld_i = in.cld_frac_i[o];
    /* rho: FP64 in the plain form, a float in the FP32-bulk hand-over */
    double rho = 0, inv_rho = 0;
    float rho_f = 0.f, inv_rho_f = 0.f;
    if constexpr (kF64) {
      rho = scr_at(in, S_RHO, col)[k];
      inv_rho = 1 / rho;
    } else {
      rho_f = scr_f(in, S_RHO, col)[k];
      inv_rho_f = 1.0f / rho_f;
    }
    double vap_liq = in.vap_liq_exchange[o];
    double eff_qc = in.diag_eff_radius_qc[o], eff_qr = in.diag_eff_radius_qr[o], eff_qi = in.diag_eff_radius_qi[o];
    double rho_qi = 0;

    /* homogeneous_freezing, p3/impl/p3_ice_sed_impl.hpp:207-270 */
    if (do_ice && dlt(t_start[k], C::T_homogfrz)) {
      const double Qc_nuc = s.qc, Qr_nuc = s.qr;
      const double Nc_nuc = dmax_c(s.nc, C::NSMALL), Nr_nuc = dmax_c(s.nr, C::NSMALL);
      const bool qc_ge = dge(s.qc, C::QSMALL), qr_ge = dge(s.qr, C::QSMALL);
      if (qc_ge) {
        s.qm = s.qm + Qc_nuc;
        s.qi = s.qi + Qc_nuc;
        s.bm = s.bm + Qc_nuc * C::INV_RHO_RIMEMAX;
        s.ni = s.ni + Nc_nuc;
        s.th = s.th + inv_exner * Qc_nuc * C::LatIce * C::INV_CP;
      }
      if (qr_ge) {
        s.qm = s.qm + Qr_nuc;
        s.qi = s.qi + Qr_nuc;
        s.bm = s.bm + Qr_nuc * C::INV_RHO_RIMEMAX;
        s.ni = s.ni + Nr_nuc;
        s.th = s.th + inv_exner * Qr_nuc * C::LatIce * C::INV_CP;
      }
      if (qc_ge) { s.qc = 0; s.nc = 0; }
      if (qr_ge) { s.qr = 0; s.nr = 0; }
    }

    if constexpr (sizeof(TR) == sizeof(double)) {
      /* part3: cloud */
      if (dge(s.qc, C::QSMALL)) {
        const double qc_incld = s.qc / cld_l;
        double nc_incld = s.nc / cld_l;
        TR mu_c, lamc;
        const TR n_in = TR(nc_incld);
        TR n_out = n_in;
        get_cloud_dsd2<TR>(TR(qc_incld), n_out, mu_c, TR(rho), lamc);
        apply_n_adjust(nc_incld, n_in, n_out);
        s.nc = nc_incld * cld_l;
        eff_qc = double(TR(0.5) * (mu_c + TR(3)) / lamc);
      } else {
        if (dnz(s.qc)) {
          s.qv = s.qv + s.qc;
          s.th = s.th - inv_exner * s.qc * C::LatVap * C::INV_CP;
          vap_liq = vap_liq - s.qc;
        }
        s.qc = 0;
        s.nc = 0;
      }
      /* part3: rain */
      if (dge(s.qr, C::QSMALL)) {
        const double qr_incld = s.qr / cld_r;
        double nr_incld = s.nr / cld_r;
        TR mu_r = 0, lamr;
        const TR n_in = TR(nr_incld);
        TR n_out = n_in;
        get_rain_dsd2<TR>(TR(qr_incld), n_out, mu_r, lamr, rt);
        apply_n_adjust(nr_incld, n_in, n_out);
        s.nr = nr_incld * cld_r;
        eff_qr = double(TR(1.5) / lamr);
      } else {
        if (dnz(s.qr)) {
          s.qv = s.qv + s.qr;
          s.th = s.th - inv_exner * s.qr * C::LatVap * C::INV_CP;
          vap_liq = vap_liq - s.qr;
        }
        s.qr = 0;
        s.nr = 0;
      }
      /* part3: ice */
      {
        const bool qi_gt_small = dge(s.qi, C::QSMALL);
        s.ni = dmax_c(s.ni, C::NSMALL);
        const double qi_incld = s.qi / cld_i;
        double ni_incld = s.ni / cld_i;
        double qm_incld = s.qm / cld_i;
        double bm_incld = s.bm / cld_i;
        double rhop = 0;
        if (qi_gt_small) {
          rhop = calc_bulk_rho_rime(qi_incld, qm_incld, bm_incld, rt);
          s.qm = qm_incld * cld_i;
          s.bm = bm_incld * cld_i;
        }
        impose_max_total_ni(ni_incld, rt.max_total_ni, inv_rho);
        if (qi_gt_small) {
          TableIce<TR> ti;
          lookup_ice<TR>(TR(qi_incld), TR(ni_incld), TR(qm_incld), TR(rhop), ti);
          TR ta[4], te[4];
          apply_table_ice4<TR>(tb, ti, 0, ta); /* columns 0, 1, 6, 7 */
          apply_table_ice4<TR>(tb, ti, 8, te); /* columns 5, 11, 8, 10 */
          const TR tv_eff = te[0];
          const TR tv_lmax = ta[2];
          const TR tv_lmin = ta[3];
          const TR tv_dens = te[1];
          ni_incld = vmin(ni_incld, double(tv_lmax) * ni_incld);
          ni_incld = vmax(ni_incld, double(tv_lmin) * ni_incld);
          eff_qi = double(tv_eff);
          rho_qi = double(tv_dens);
        }
        s.ni = ni_incld * cld_i;
        if (dlt(s.qm, C::QSMALL) && qi_gt_small) {
          s.qm = 0;
          s.bm = 0;
        }
        if (!qi_gt_small) {
          if (dnz(s.qi)) {
            s.qv = s.qv + s.qi;
            s.th = s.th - inv_exner * s.qi * (C::LatVap + C::LatIce) * C::INV_CP;
          }
          s.qi = 0; s.ni = 0; s.qm = 0; s.bm = 0;
        }
      }
    } else {
      /* FP32-bulk part3: in-cloud values, DSDs and the diagnostics in FP32; the
       * FP64 state is rewritten only where a limiter changed an in-cloud value */
      if (dge(s.qc, C::QSMALL)) {
        const float icl = 1.0f / float(cld_l);
        const float qc_f = float(s.qc) * icl;
        const float n_in = float(s.nc) * icl;
        float n_out = n_in, mu_c, lamc;
        get_cloud_dsd2<float>(qc_f, n_out, mu_c, rho_f, lamc);
        if (n_out != n_in) s.nc = f2d_int(n_out) * cld_l;
        eff_qc = f2d_int(0.5f * (mu_c + 3.0f) / lamc);
      } else {
        if (dnz(s.qc)) {
          s.qv = s.qv + s.qc;
          s.th = s.th - inv_exner * s.qc * C::LatVap * C::INV_CP;
          vap_liq = vap_liq - s.qc;
        }
        s.qc = 0;
        s.nc = 0;
      }
      if (dge(s.qr, C::QSMALL)) {
        const float icr = 1.0f / float(cld_r);
        const float qr_f = float(s.qr) * icr;
        const float n_in = float(s.nr) * icr;
        float n_out = n_in, mu_r = 0, lamr;
        get_rain_dsd2<float>(qr_f, n_out, mu_r, lamr, rt);
        if (n_out != n_in) s.nr = f2d_int(n_out) * cld_r;
        eff_qr = f2d_int(1.5f / lamr);
      } else {
        if (dnz(s.qr)) {
          s.qv = s.qv + s.qr;
          s.th = s.th - inv_exner * s.qr * C::LatVap * C::INV_CP;
          vap_liq = vap_liq - s.qr;
        }
        s.qr = 0;
        s.nr = 0;
      }
      {
        const bool qi_gt_small = dge(s.qi, C::QSMALL);
        s.ni = dmax_c(s.ni, C::NSMALL);
        if (qi_gt_small) {
          const float ici = 1.0f / float(cld_i);
          const float qi_f = float(s.qi) * ici;
          const float ni0 = float(s.ni) * ici;
          const float qm0 = float(s.qm) * ici, bm0 = float(s.bm) * ici;
          float qm_f = qm0, bm_f = bm0;
          const float rhop = calc_bulk_rho_rime<float>(qi_f, qm_f, bm_f, rt);
          if (qm_f != qm0) s.qm = f2d_int(qm_f) * cld_i;
          if (bm_f != bm0) s.bm = f2d_int(bm_f) * cld_i;
          float ni_f = ni0;
          impose_max_total_ni(ni_f, rt.f.max_total_ni, inv_rho_f);
          TableIce<float> ti;
          lookup_ice<float>(qi_f, ni_f, qm_f, rhop, ti);
          float ta[4], te[4];
          apply_table_ice4<float>(tb, ti, 0, ta); /* columns 0, 1, 6, 7 */
          apply_table_ice4<float>(tb, ti, 8, te); /* columns 5, 11, 8, 10 */
          ni_f = vmin(ni_f, ta[2] * ni_f);
          ni_f = vmax(ni_f, ta[3] * ni_f);
          eff_qi = f2d_int(te[0]);
          rho_qi = f2d_int(te[1]);
          if (ni_f != ni0) s.ni = f2d_int(ni_f) * cld_i;
          if (dlt(s.qm, C::QSMALL)) {
            s.qm = 0;
            s.bm = 0;
          }
        } else {
          if (dnz(s.qi)) {
            s.qv = s.qv + s.qi;
            s.th = s.th - inv_exner * s.qi * (C::LatVap + C::LatIce) * C::INV_CP;
          }
          s.qi = 0; s.ni = 0; s.qm = 0; s.bm = 0;
        }
      }
    }
    if (dlt(s.qr, C::QSMALL)) s.nr = 0;

    in.qc[o] = s.qc; in.nc[o] = s.nc; in.qr[o] = s.qr; in.nr[o] = s.nr;
    in.qi[o] = s.qi; in.qm[o] = s.qm; in.ni[o] = s.ni; in.bm[o] = s.bm;
    in.qv[o] = s.qv; in.th[o] = s.th;
    in.vap_liq_exchange[o] = vap_liq;
    in.diag_eff_radius_qc[o] = eff_qc;
    in.diag_eff_radius_qr[o] = eff_qr;
    in.diag_eff_radius_qi[o] = eff_qi;
    in.rho_qi[o] = rho_qi;
    if (kp.check) {
      /* check_values (p3_check_values_impl.hpp:26-81, called at
       * p3_main_impl.hpp:316-323 with T = th exner): T must lie in
       * (173, 323) K and qv in (0, 0.04); the reference traps only on T, and
       * only when its debug abort is on.  Recorded, never trapped. */
      const double T = s.th * (1 / inv_exner);
      const unsigned long long key = check_key(inst_idx, col, k);
      if (!(dgt(T, 173.0) && dlt(T, 323.0))) {
        atomicAdd(&kp.check[kChkTCount], 1ull);
        atomicMin(&kp.check[kChkTFirst], key);
        if (kp.check_fail) err |= kErrRange;
      }
      if (!(dpos(s.qv) && dlt(s.qv, 0.04))) {
        atomicAdd(&kp.check[kChkQvCount], 1ull);
        atomicMin(&kp.check[kChkQvFirst], key);
      }
    }
  }
}

/* ------------------------------------------------------------------ */
/* kernels                                                             */
/* ------------------------------------------------------------------ */

/* Table pointers of a CTA: staged into shared memory (K1, when kp.staged)
 * or the global copies.  Returns the first byte after the staged tables, or
 * nullptr when the staging wait gave up. */
template <class TR>
__device__ __forceinline__ unsigned char* setup_tables(const KParams<TR>& kp, bool stage, unsigned char* smem_raw,
                                                       Tabs<TR>& tb, uint32_t& err) {
  tb.collect = kp.collect;
  if (stage) {
    TR* s_ice = reinterpret_cast<TR*>(smem_raw);
    TR* s_t3 = s_ice + kIceTableElems;
    uint64_t* mbar = reinterpret_cast<uint64_t*>(smem_raw + table_smem_bytes<TR>() - 16);
    if (!stage_tables<TR>(kp, s_ice, s_t3, mbar, err)) return nullptr;
    tb.ice = s_ice;
    tb.vn = s_t3;
    tb.vm = s_t3 + 600;
    tb.revap = s_t3 + 1200;
    tb.t3_stride = 2;
    tb.t3_j0 = kp.rt.t3_dumjj - 1;
    return smem_raw + table_smem_bytes<TR>();
  }
  tb.ice = kp.ice;
  tb.vn = kp.vn;
  tb.vm = kp.vm;
  tb.revap = kp.revap;
  tb.t3_stride = kVT1;
  tb.t3_j0 = 0;
  return smem_raw;
}

/* Runs f(w) for the work items of this column group.  With a counter, a warp
 * takes the next 32/LANES items whenever it has finished its last ones, so a
 * warp that drew cheap columns takes more of them and no SM idles behind the
 * slowest column list (a static stride gives every warp a fixed share, and an
 * even stride gives it columns of one parity only).  Without one, groups
 * stride the list. */
template <int LANES, class F>
__device__ __forceinline__ void for_each_work(uint32_t* ctr, int nwork, int groups_per_block, F&& f) {
  if (ctr) {
    const int lane = threadIdx.x & 31;
    const int nthr = min(32, int(blockDim.x) - int(threadIdx.x & ~31u));
    const unsigned wmask = nthr == 32 ? 0xffffffffu : ((1u << nthr) - 1u);
    const uint32_t per_warp = uint32_t(nthr / LANES);
    const uint32_t g_in_warp = uint32_t(lane / LANES);
    for (;;) {
      uint32_t base = 0;
      if (lane == 0) base = atomicAdd(ctr, per_warp);
      base = __shfl_sync(wmask, base, 0);
      if (base >= uint32_t(nwork)) break;
      const uint32_t w = base + g_in_warp;
      if (w < uint32_t(nwork)) f(int(w));
    }
  } else {
    const int groups_total = gridDim.x * groups_per_block;
    for (int w = blockIdx.x * groups_per_block + int(threadIdx.x) / LANES; w < nwork; w += groups_total) f(w);
  }
}

/* Column of work item w (single instance or batched work list). */
template <class TR>
__device__ __forceinline__ const Inst& work_inst(const Inst& inst0, const KParams<TR>& kp, int w, int& col) {
  if (kp.work) {
    const WorkItem wi = kp.work[w];
    col = wi.col;
    return kp.insts[wi.inst];
  }
  col = w;
  return inst0;
}

/* The FP32-bulk instantiation is held to 128 registers (two CTAs of 256
 * threads per SM; a few dozen bytes spill), which measured 25 % faster than 176
 * registers at one CTA per SM. */
template <class TR, int LANES>
__global__ void __launch_bounds__(256, sizeof(TR) == sizeof(float) ? 2 : 1)
    p3_part12_kernel(const Inst inst0, const KParams<TR> kp) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  uint32_t err = 0;
  Tabs<TR> tb;
  unsigned char* base = setup_tables<TR>(kp, kp.staged != 0, smem_raw, tb, err);
  if (!base) {
    if (threadIdx.x == 0) atomicOr(kp.err, err);
    return;
  }
  const int g_in_block = threadIdx.x / LANES;
  double* sm = reinterpret_cast<double*>(base) + size_t(g_in_block) * A_NARR * kp.sm_stride;
  /* liquid saturation vapour pressure at 0 C (qsat0 of ice_melting and
   * ice_cldliq_wet_growth), evaluated once */
  const double esat0 = murphy_koop_svp<double>(C::Tmelt, false, err);
  for_each_work<LANES>(kp.wctr ? kp.wctr + 0 : nullptr, kp.nwork, kp.groups_per_block, [&](int w) {
    int col;
    const Inst& in = work_inst(inst0, kp, w, col);
    p3_part12<TR, LANES>(in, col, kp, tb, sm, esat0, err);
  });
  if (err) atomicOr(kp.err, err);
}

template <class TR, int LANES>
__global__ void __launch_bounds__(256) p3_sed_kernel(const Inst inst0, const KParams<TR> kp) {
  static_assert(sizeof(TR) == sizeof(double), "the FP32-bulk sedimentation kernel is p3_sed_bulk_kernel");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  uint32_t err = 0;
  Tabs<TR> tb;
  setup_tables<TR>(kp, false, smem_raw, tb, err);
  const int g_in_block = threadIdx.x / LANES;
  double* sm = reinterpret_cast<double*>(smem_raw) + size_t(g_in_block) * sed_slots<TR>() * kp.sm_stride;
  for_each_work<LANES>(kp.wctr ? kp.wctr + 1 : nullptr, kp.nwork, kp.groups_per_block, [&](int w) {
    int col;
    const Inst& in = work_inst(inst0, kp, w, col);
    p3_sed<TR, LANES>(in, col, kp, tb, sm, err);
  });
  if (err) atomicOr(kp.err, err);
}

/* K2 of the FP32-bulk form.  Held to 96 registers: with its 10 shared slots
 * per column that is five 4-column CTAs (20 warps) per SM, where the
 * latency-bound substep walk gains from every resident warp.  At most 256
 * threads per CTA (the launch checks it). */
template <int LANES>
__global__ void __maxnreg__(96) p3_sed_bulk_kernel(const Inst inst0, const KParams<float> kp) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  uint32_t err = 0;
  /* Compact tables, so that the lookups of the substep walk stay in the L1
   * data cache beside the CTAs' shared memory: the four ice-table columns of
   * sedimentation (16 KB) and the two-column Table3 slices of the rain
   * shape (2.4 KB each) rather than the full tables (48 KB and 12 KB). */
  Tabs<float> tb;
  tb.collect = kp.collect;
  tb.ice = kp.ice_sed;
  tb.vn = kp.t3slice;
  tb.vm = kp.t3slice + kT3SliceElems / 3;
  tb.revap = kp.t3slice + 2 * (kT3SliceElems / 3);
  tb.t3_stride = 2;
  tb.t3_j0 = kp.rt.t3_dumjj - 1;
  const int g_in_block = threadIdx.x / LANES;
  double* sm = reinterpret_cast<double*>(smem_raw) + size_t(g_in_block) * kSedBulkSlots * kp.sm_stride;
  for_each_work<LANES>(kp.wctr ? kp.wctr + 1 : nullptr, kp.nwork, kp.groups_per_block, [&](int w) {
    int col;
    const Inst& in = work_inst(inst0, kp, w, col);
    p3_sed_bulk<LANES>(in, col, kp, tb, sm, err);
  });
  if (err) atomicOr(kp.err, err);
}

template <class TR, int LANES>
__global__ void __launch_bounds__(256) p3_part3_kernel(const Inst inst0, const KParams<TR> kp) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  uint32_t err = 0;
  Tabs<TR> tb;
  setup_tables<TR>(kp, false, smem_raw, tb, err);
  for_each_work<LANES>(kp.wctr ? kp.wctr + 2 : nullptr, kp.nwork, kp.groups_per_block, [&](int w) {
    int col;
    const Inst& in = work_inst(inst0, kp, w, col);
    p3_part3<TR, LANES>(in, col, kp, tb, kp.work ? kp.work[w].inst : 0, err);
  });
  if (err) atomicOr(kp.err, err);
}

}  // namespace dev
}  // namespace p3x
