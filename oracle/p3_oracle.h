/*
 * CPU oracle for the P3 microphysics step -- TEST INFRASTRUCTURE ONLY.
 *
 * This is a scalar (pack size 1), FP64, OpenMP-over-columns restatement of
 * EAMxx's `scream::p3::Functions<Real,Device>::p3_main`
 * (components/eamxx/src/physics/p3/impl/p3_main_impl.hpp:74-372 and the
 * impl/*_impl.hpp files it calls).  It exists to check the GPU product and to
 * serve as the timed CPU baseline; nothing in the product library links it.
 *
 * Parity status: the reference itself cannot be compiled here (EKAT and
 * Kokkos submodules are empty, no Fortran compiler, lookup-table data files
 * absent), so absolute p3_main outputs are pinned only through the
 * reference's own invariant tests (conservation limiters, upwind mass
 * conservation and monotonicity, Table3 continuity, find_top/find_bottom)
 * and its mixed initial condition; full-step absolute parity is unpinned.
 *
 * Layout: every 2-D field is (ncol, nlev) row-major with a leading dimension
 * (elements between consecutive columns), i.e. EAMxx's view_2d<Spack> with a
 * pack size of 1.  Level 0 is the model top.  Interface fields (precip fluxes)
 * have nlev+1 entries per column and their own leading dimension.
 */
#ifndef P3_ORACLE_H
#define P3_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Mirrors P3Runtime (components/eamxx/src/physics/p3/p3_functions.hpp:112-133). */
typedef struct p3o_runtime {
  double max_total_ni;
  double autoconversion_prefactor;
  double autoconversion_qc_exponent;
  double autoconversion_nc_exponent;
  double autoconversion_radius;
  double accretion_prefactor;
  double accretion_qc_exponent;
  double accretion_qr_exponent;
  double rain_selfcollection_prefactor;
  double rain_selfcollection_breakup_diameter;
  double constant_mu_rain;
  double spa_ccn_to_nc_factor;
  double cldliq_to_ice_collection_factor;
  double rain_to_ice_collection_factor;
  double min_rime_rho;
  double max_rime_rho;
  double immersion_freezing_exponent;
  double deposition_nucleation_exponent;
  double ice_sedimentation_factor;
  int32_t do_ice_production;
  int32_t pad_;
} p3o_runtime;

/* Mirrors P3LookupTables (p3_functions.hpp:262-276). Row-major C arrays. */
typedef struct p3o_tables {
  const double* ice;      /* [5][4][50][12]      */
  const double* collect;  /* [5][4][50][30][2]   (log10 values) */
  const double* vn;       /* [300][10]           */
  const double* vm;       /* [300][10]           */
  const double* revap;    /* [300][10]           */
  const double* mu_r;     /* [150]               */
  const double* dnu;      /* [16]                */
} p3o_tables;

/* Mirrors P3PrognosticState / P3DiagnosticInputs / P3DiagnosticOutputs /
 * P3HistoryOnly (p3_functions.hpp:159-259). */
typedef struct p3o_fields {
  /* prognostic (in/out) */
  double *qc, *nc, *qr, *nr, *qi, *qm, *ni, *bm, *qv, *th;
  /* diagnostic inputs */
  const double *nc_nuceat_tend, *nccn, *ni_activated, *inv_qc_relvar,
               *cld_frac_i, *cld_frac_l, *cld_frac_r, *pres, *dz, *dpres,
               *inv_exner, *qv_prev, *t_prev;
  /* diagnostic outputs */
  double *qv2qi_depos_tend, *precip_liq_surf, *precip_ice_surf,
         *diag_eff_radius_qc, *diag_eff_radius_qi, *diag_eff_radius_qr,
         *rho_qi, *precip_liq_flux, *precip_ice_flux, *precip_total_tend,
         *nevapr;
  /* history only */
  double *liq_ice_exchange, *vap_liq_exchange, *vap_ice_exchange;
} p3o_fields;

typedef struct p3o_call {
  int32_t ncol, nlev;
  int64_t ld;      /* leading dimension of mid-level fields   */
  int64_t ld_int;  /* leading dimension of interface fields   */
  double dt;
  int32_t it;
  int32_t predictNc, prescribedCCN;
  int32_t nthreads; /* <=0: OpenMP default */
} p3o_call;

/* Error bits (same meaning as the product's status codes). */
enum { P3O_OK = 0, P3O_ENUMERIC = 1, P3O_ESUBSTEP = 2 };

void p3o_runtime_defaults(p3o_runtime* rt);

/* One P3 step on all columns, in place.  Returns the OR of error bits.
 * *elapsed_us receives the wall time of the column loop (init excluded),
 * like the reference's return value (p3_main_impl.hpp:104-105,328-330). */
int p3o_main(const p3o_call* call, const p3o_runtime* rt, const p3o_tables* tab,
             const p3o_fields* f, double* elapsed_us);

/* The step in two stages, for stage-by-stage parity checks.
 * p3o_main_part12 runs p3_main_init, part1 and part2 in place and writes,
 * for every column that goes on (cflag[i] = 1; 0 after an early exit), the
 * hand-over the later stages read: rows [5][ncol][ld] of the temperature
 * after part1, the density, rhofacr, rhofaci and acn.  p3o_main_sed_part3
 * runs sedimentation, homogeneous freezing and part3 in place on the columns
 * with cflag[i] = 1, from the given state and hand-over.  Both stages in a
 * row give exactly p3o_main.  Return the OR of error bits. */
int p3o_main_part12(const p3o_call* call, const p3o_runtime* rt, const p3o_tables* tab,
                    const p3o_fields* f, double* handover, int32_t* cflag);
int p3o_main_sed_part3(const p3o_call* call, const p3o_runtime* rt, const p3o_tables* tab,
                       const p3o_fields* f, const double* handover, const int32_t* cflag);

/* Single-function entry points used by the invariant tests. */
void p3o_calc_first_order_upwind_step(int nk, int k_bot, int k_top, int kdir,
                                      double dt_sub, const double* rho,
                                      const double* inv_rho, const double* inv_dz,
                                      int nfield, double* const* flux,
                                      double* const* V, double* const* r);
int p3o_find_top(const double* v, double small, int kbot, int ktop, int kdir, int* present);
int p3o_find_bottom(const double* v, double small, int kbot, int ktop, int kdir, int* present);
void p3o_table3_lookup_apply(const p3o_tables* tab, int which, int n,
                             const double* mu_r, const double* lamr, double* out);
void p3o_cloud_water_conservation(double qc, double dt, double* tend8);
void p3o_rain_water_conservation(double qr, double dt, double* tend7);
void p3o_ice_water_conservation(double qi, double dt, double* tend9);
double p3o_qv_sat_dry(double t, double p, int ice);

#ifdef __cplusplus
}
#endif

#endif
