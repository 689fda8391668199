/* Host-side launch interface of the device kernels (internal to libp3x). */
#ifndef P3X_LAUNCH_HPP
#define P3X_LAUNCH_HPP

#include <cuda_runtime.h>

#include "p3x.h"
#include "p3x_column.cuh"

struct p3x_context;

namespace p3x {

struct LaunchSpec {
  int lanes;            /* 8, 16, 32 */
  int groups_per_block; /* columns per CTA */
  int staged;           /* tables in shared memory */
  int blocks_per_sm;    /* 0: as many as fit */
  cudaEvent_t* marks = nullptr; /* optional: 4 events recorded around K1, K2, K3 */
  double grid_frac = 1.0;       /* share of the resident-CTA capacity the persistent grid takes */
};

/* Shared-memory bytes of one CTA of K1 (part1+part2; staged tables plus the
 * per-level arrays) and of K2 (sedimentation).  K3 uses none. */
template <class TR>
inline size_t p3_smem_bytes(const LaunchSpec& ls, int sm_stride) {
  const size_t tables = ls.staged ? dev::table_smem_bytes<TR>() : 0;
  return tables + size_t(ls.groups_per_block) * dev::A_NARR * size_t(sm_stride) * sizeof(double);
}
template <class TR>
inline size_t sed_smem_bytes(const LaunchSpec& ls, int sm_stride) {
  return size_t(ls.groups_per_block) * dev::sed_slots<TR>() * size_t(sm_stride) * sizeof(double);
}

/* Launch shape of K2.  Sedimentation always runs 32 lanes per column,
 * whatever lane count K1 and K3 use: its substeps walk the levels chunk by
 * chunk, so a narrower group only lengthens the walk (measured at 65,536 x
 * 128 with 16 lanes: FP64 K2 +17 %, FP32-bulk K2 +95 %), while K1 in the
 * FP64 form runs 7 % faster at 16 lanes.  Columns per CTA as configured, at
 * most 8 (256 threads). */
inline LaunchSpec sed_spec(const LaunchSpec& ls) {
  LaunchSpec s = ls;
  s.lanes = 32;
  s.groups_per_block = ls.groups_per_block < 8 ? ls.groups_per_block : 8;
  s.staged = 0;
  return s;
}

/* CTAs of kernel `func` that fit on one SM with `threads` threads and `smem`
 * bytes of dynamic shared memory on the current device.  The first query of
 * a (device, kernel, threads, smem) shape raises the kernel's
 * dynamic-shared-memory limit as needed and asks the occupancy calculator;
 * later ones read the cache (p3x_api.cu). */
cudaError_t kernel_occupancy(const void* func, int threads, size_t smem, int* per_sm);

/* Kernel parts of one step, launched in order on one stream: K1
 * (part1+part2; zeroes the work counters first), K2 (sedimentation), K3
 * (part3). */
enum : int { kPartK1 = 1, kPartK2 = 2, kPartK3 = 4 };

/* Persistent launch of one part for one lane count (defined in
 * p3x_kernels_impl.cuh, instantiated in p3x_k_*.cu; K2 only for 32 lanes).
 * kp.nwork, kp.work, kp.insts and kp.sm_stride are set by the caller, and
 * every instance's scratch (Inst::scr, Inst::cflag) is bound. */
template <class TR, int LANES>
cudaError_t launch_p3_part(const dev::Inst& inst0, const dev::KParams<TR>& kp, const LaunchSpec& ls, int part,
                           int num_sms, cudaStream_t stream);

template <class TR>
inline cudaError_t launch_p3_part_lanes(const dev::Inst& inst0, const dev::KParams<TR>& kp, const LaunchSpec& ls,
                                        int part, int num_sms, cudaStream_t stream) {
  switch (ls.lanes) {
    case 8: return launch_p3_part<TR, 8>(inst0, kp, ls, part, num_sms, stream);
    case 16: return launch_p3_part<TR, 16>(inst0, kp, ls, part, num_sms, stream);
    case 32: return launch_p3_part<TR, 32>(inst0, kp, ls, part, num_sms, stream);
    default: return cudaErrorInvalidValue;
  }
}

/* The column kernels of one step in order on one stream: all three (K1, K2,
 * K3) by default, or the subset `parts` (kPartK* bits).  K1 zeroes the work
 * counters; a subset without K1 zeroes them here. */
template <class TR>
inline cudaError_t launch_p3(const dev::Inst& inst0, const dev::KParams<TR>& kp, const LaunchSpec& ls,
                             int num_sms, cudaStream_t stream, int parts = kPartK1 | kPartK2 | kPartK3) {
  cudaError_t e = cudaSuccess;
  if (parts & kPartK1) {
    e = launch_p3_part_lanes<TR>(inst0, kp, ls, kPartK1, num_sms, stream);
    if (e != cudaSuccess) return e;
  } else if (kp.wctr) {
    e = cudaMemsetAsync(kp.wctr, 0, dev::kWorkCounters * sizeof(uint32_t), stream);
    if (e != cudaSuccess) return e;
  }
  if (parts & kPartK2) {
    e = launch_p3_part<TR, 32>(inst0, kp, sed_spec(ls), kPartK2, num_sms, stream);
    if (e != cudaSuccess) return e;
  }
  if (parts & kPartK3) e = launch_p3_part_lanes<TR>(inst0, kp, ls, kPartK3, num_sms, stream);
  return e;
}

/* (nlev, ncol) column-fastest <-> (ncol, ld) level-contiguous transposes. */
cudaError_t launch_transpose_to_levels(const double* src, double* dst, int ncol, int nlev, int64_t ld,
                                       cudaStream_t st);
cudaError_t launch_transpose_to_columns(const double* src, double* dst, int ncol, int nlev, int64_t ld,
                                        cudaStream_t st);

/* One step of a work list of (instance, column) items whose instances all
 * have the given precision: K1, K2, K3 with the context's launch
 * configuration for that precision (p3x_api.cu).  Every instance's scratch
 * must be bound.  wctr: dev::kWorkCounters device words used by no other
 * launch in flight (zeroed on the stream), or null for a static stride. */
int launch_work(p3x_context* ctx, const p3x_runtime& rt, int precision, const dev::Inst* insts_d,
                const dev::WorkItem* work_d, int nwork, int nlev_max, uint32_t* wctr, cudaStream_t st,
                double grid_frac = 1.0);

/* The state hand-over of the P3 process interface between steps
 * (eamxx_p3_process_interface.hpp:218,237 with dry = wet mixing ratios):
 * qv_prev <- qv and t_prev <- th / inv_exner, for every work item. */
cudaError_t launch_postamble(const dev::Inst* insts_d, const dev::WorkItem* work_d, int nwork, cudaStream_t st);

/* Device pointers of the process-interface pre/postamble kernels. */
struct InterfacePtrs {
  const double *pmid, *pd, *pdd, *cld_t;
  double *T, *T_prev;
  double* q[9]; /* qc nc qr nr qi qm ni bm qv */
  double *th, *qv_prev, *inv_exner, *dz, *cld_l, *cld_i, *cld_r;
  double *eff_qc, *eff_qi, *eff_qr;
  const double *liq_surf, *ice_surf;
  double *liq_mass, *ice_mass, *vapor_flux, *water_flux, *ice_flux, *heat_flux;
};
cudaError_t launch_interface(const InterfacePtrs& p, int ncol, int nlev, int64_t ld, bool post, double dt,
                             cudaStream_t st);

/* Device pointers of the EAM driver's pre/post kernels (micro_p3_tend).
 * Constituent order of q, ptend_q and w: qv, cldliq, numliq, rain, numrain,
 * cldice, numice, cldrim, rimvol. */
struct EamPtrs {
  const double *pmid, *pmiddry, *pdel, *pdeldry, *zi, *t, *q[9], *ast, *npccn, *ni_act_in, *relvar, *cmeliq;
  double *t_prev, *qv_prev, *ptend_s, *ptend_q[9];
  double *qme, *rho, *icimrst, *icwmrst, *icinc, *icwnc, *rel, *rei, *dei, *mu, *lambdac, *nfice, *efcout, *ncout,
      *freql, *efiout, *niout, *freqi, *aqrain, *anrain, *freqr, *reff_rain, *deff_rain, *flxprc, *flxsnw;
  double *prec_pcw, *snow_pcw, *prec_str, *snow_str, *cdnumc;
  int subgrid, method;
  /* the P3 working arrays: prognostic state in constituent order, inputs */
  double* w[9];
  double *th, *pres, *dz, *dpres, *inv_exner, *cld_l, *cld_i, *cld_r, *nc_nuceat, *ni_act, *inv_relvar, *qv_prev_dry,
      *t_prev_p3;
  /* P3 outputs read by the post kernel */
  const double *eff_qc, *eff_qi, *eff_qr, *liq_surf, *ice_surf, *liq_flux, *ice_flux, *depos;
  double* vap_liq;
};
cudaError_t launch_eam(const EamPtrs& p, int ncol, int nlev, int64_t ld, int64_t ld_int, bool post, double dt,
                       cudaStream_t st);

cudaError_t launch_selftest(unsigned long long* mismatches_d, cudaStream_t st);

/* Fields of the column mass / energy conservation check (device pointers;
 * per-level (ncol, ld), winds (ncol, 2, ld), per-column (ncol)). */
struct ConsPtrs {
  const double *pd, *T, *qv, *qc, *qi, *qr, *winds, *ps, *phis;
  const double *vapor_flux, *water_flux, *ice_flux, *heat_flux;
  double *mass, *energy;                    /* column totals (may be null)   */
  const double *mass_before, *energy_before; /* null: totals only            */
  double *mass_err, *energy_err;            /* relative errors (with before) */
};
/* Column totals and, with the totals before, relative errors; with maxloc4
 * (4 doubles, device), also {max mass err, its column, max energy err, its
 * column}. */
cudaError_t launch_conservation(const ConsPtrs& p, int ncol, int nlev, int64_t ld, double dt, double* maxloc4,
                                cudaStream_t st);

cudaError_t launch_budgets(const double* qv, const double* qc, const double* qr, const double* qi,
                           const double* th, const double* dpres, const double* inv_exner, int ncol,
                           int nlev, int64_t ld, double* water, double* energy, cudaStream_t st);

}  // namespace p3x

#endif
