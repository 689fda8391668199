/*
 * p3x -- GB300-native P3 microphysics step behind the EAMxx P3 call surface.
 *
 * C ABI (no C++ or torch types).  Every entry point returns P3X_OK (0) or a
 * negative status.  Unless stated otherwise, field pointers are DEVICE
 * pointers to FP64 arrays laid out (ncol, nlev) row-major: level k of
 * column i is at ptr[i*ld + k], level 0 is the model top.  This is EAMxx's
 * view_2d<Spack> with a pack size of 1, the layout the reference uses on GPU.
 * Interface fields (precip_liq_flux, precip_ice_flux) hold nlev+1 values per
 * column with their own leading dimension.
 *
 * Reference interfaces replaced (paths relative to components/eamxx/src/):
 *   p3x_runtime ............ P3Runtime              physics/p3/p3_functions.hpp:112-157
 *   p3x_prognostic_state ... P3PrognosticState      physics/p3/p3_functions.hpp:159-182
 *   p3x_diagnostic_inputs .. P3DiagnosticInputs     physics/p3/p3_functions.hpp:184-213
 *   p3x_diagnostic_outputs . P3DiagnosticOutputs    physics/p3/p3_functions.hpp:215-241
 *   p3x_infrastructure ..... P3Infrastructure       physics/p3/p3_functions.hpp:243-263
 *   p3x_history_only ....... P3HistoryOnly          physics/p3/p3_functions.hpp:265-275
 *   p3x_context_create ..... p3_init + P3LookupTables
 *                            physics/p3/p3_f90.cpp:103-113,
 *                            physics/p3/impl/p3_table_ice_impl.hpp:16-78,
 *                            physics/p3/impl/p3_table3_impl.hpp:85-148
 *   p3x_main ............... Functions<Real,Device>::p3_main
 *                            physics/p3/p3_functions.hpp:1355-1369,
 *                            physics/p3/impl/p3_main_impl.hpp:333-372
 *   p3x_main_f ............. p3_main_c (Fortran-callable, host arrays,
 *                            (its:ite,kts:kte) column-fastest layout)
 *                            physics/p3/p3_iso_c.f90:132-183,
 *                            physics/p3/p3_main_wrap.cpp:11-24
 */
#ifndef P3X_H
#define P3X_H

#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ */
/* Status codes                                                        */
/* ------------------------------------------------------------------ */
#define P3X_OK 0
#define P3X_EINVAL (-1)   /* bad argument (null pointer, nlev <= 0, dt <= 0, ...) */
#define P3X_ENOMEM (-2)   /* device allocation failed or budget exceeded          */
#define P3X_ENUMERIC (-3) /* T <= 0 or NaN met in a saturation evaluation          */
#define P3X_ETIMEOUT (-4) /* sedimentation substep cap or a bounded wait ran out   */
#define P3X_ECUDA (-5)    /* a CUDA runtime call failed                            */
#define P3X_ETABLE (-6)   /* lookup table file missing / malformed / wrong version */
#define P3X_ERANGE (-7)   /* check_values in fail mode: T outside (173, 323) K      */

/* p3_init info codes (physics/p3/p3_iso_c.f90:43-130 returns 0 or -1..-6). */

/* Precision forms. */
#define P3X_FP64 0      /* FP64 everywhere                                            */
#define P3X_FP32_BULK 1 /* process rates + table interpolation in FP32; saturation    */
                        /* residuals, state updates, sedimentation flux accumulation  */
                        /* and column budgets in FP64                                 */

/* P3Runtime, p3_functions.hpp:112-133 (same names, same defaults). */
typedef struct p3x_runtime {
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
} p3x_runtime;

/* P3PrognosticState, p3_functions.hpp:159-182 (in/out). */
typedef struct p3x_prognostic_state {
  double *qc, *nc, *qr, *nr, *qi, *qm, *ni, *bm, *qv, *th;
} p3x_prognostic_state;

/* P3DiagnosticInputs, p3_functions.hpp:184-213 (read only). */
typedef struct p3x_diagnostic_inputs {
  const double *nc_nuceat_tend, *nccn, *ni_activated, *inv_qc_relvar, *cld_frac_i,
      *cld_frac_l, *cld_frac_r, *pres, *dz, *dpres, *inv_exner, *qv_prev, *t_prev;
} p3x_diagnostic_inputs;

/* P3DiagnosticOutputs, p3_functions.hpp:215-241.  precip_liq_surf and
 * precip_ice_surf have one value per column; precip_liq_flux and
 * precip_ice_flux have nlev+1 per column. */
typedef struct p3x_diagnostic_outputs {
  double *qv2qi_depos_tend, *precip_liq_surf, *precip_ice_surf, *diag_eff_radius_qc,
      *diag_eff_radius_qi, *diag_eff_radius_qr, *rho_qi, *precip_liq_flux, *precip_ice_flux,
      *precip_total_tend, *nevapr;
} p3x_diagnostic_outputs;

/* P3Infrastructure, p3_functions.hpp:243-263.  its/ite/kts/kte are kept for
 * the Fortran-style entry; col_location may be NULL (debug output only). */
typedef struct p3x_infrastructure {
  double dt;
  int32_t it, its, ite, kts, kte;
  int32_t predictNc, prescribedCCN;
  const double* col_location;
} p3x_infrastructure;

/* P3HistoryOnly, p3_functions.hpp:265-275.  The reference requires the
 * caller to zero these before p3_main (eamxx_p3_run.cpp:27-29); p3x zeroes
 * them itself, so callers may but need not. */
typedef struct p3x_history_only {
  double *liq_ice_exchange, *vap_liq_exchange, *vap_ice_exchange;
} p3x_history_only;

/* Leading dimensions in elements; 0 selects the dense value (nlev, nlev+1). */
typedef struct p3x_layout {
  int64_t ld;
  int64_t ld_int;
} p3x_layout;

/* Launch configuration (chosen by p3x_autotune or set by hand). */
typedef struct p3x_launch_config {
  int32_t lanes_per_column;  /* 8, 16 or 32 (part1+2 and part3; sedimentation  */
                             /*    always runs 32 lanes per column)            */
  int32_t columns_per_block; /* columns handled concurrently by one CTA        */
  int32_t table_staging;     /* 0: tables read through L1/L2; 1: staged into   */
                             /*    shared memory by bulk copies (cp.async.bulk) */
  int32_t blocks_per_sm;     /* persistent grid = blocks_per_sm x SM count (0 = auto) */
} p3x_launch_config;

typedef struct p3x_context p3x_context;

void p3x_runtime_defaults(p3x_runtime* rt);

/* Creates the lookup tables (the official text file when table_file is not
 * NULL, otherwise generated in-process) and uploads them to the current
 * device.  *info receives 0 or the negative P3X_* code of the failure. */
int p3x_context_create(const char* table_file, p3x_context** out, int* info);
int p3x_context_destroy(p3x_context* ctx);

/* Host copies of the P3LookupTables of a context (for checking / oracles).
 * Sizes: ice 5*4*50*12, collect 5*4*50*30*2, vn/vm/revap 300*10, mu_r 150,
 * dnu 16.  Any pointer may be NULL. */
int p3x_context_get_tables(const p3x_context* ctx, double* ice, double* collect, double* vn,
                           double* vm, double* revap, double* mu_r, double* dnu);

/* Host-only: fills caller-provided HOST arrays with the generated
 * P3LookupTables (same sizes as p3x_context_get_tables); when table_file is
 * not NULL the ice / collection tables are read from it instead.  Touches no
 * GPU. */
int p3x_tables_generate(const char* table_file, double* ice, double* collect, double* vn, double* vm,
                        double* revap, double* mu_r, double* dnu);

/* Regularised upper incomplete gamma function Q(a, x) used by the ice-table
 * generator (series for x < a+1, Legendre continued fraction otherwise). */
double p3x_incomplete_gamma_q(double a, double x);

/* Host-only: the FP64 saturation table of the FP32-bulk form.  Murphy-Koop
 * vapour pressure (share/physics_saturation_impl.hpp:38-81) over liquid
 * (rows 0..n-1) and ice (rows n..2n-1) as one cubic per interval of width
 * 1/inv_h K starting at t0: e(T) = c0 + u (c1 + u (c2 + u c3)) with
 * u = (T - t0) inv_h - i.  coef (may be NULL) receives 2 n 4 doubles.  No
 * counterpart in the reference, which evaluates the formula. */
int p3x_saturation_table(double* coef, int32_t* intervals, double* t0, double* inv_h);

/* Writes the generated ice / collection table in the official text format. */
int p3x_write_ice_table(const char* path, const char* version);

/* Functions<Real,Device>::p3_main: one P3 step over nj columns of nk levels,
 * device pointers, synchronous on `stream` (a cudaStream_t, NULL = legacy
 * default stream).  *elapsed_us (may be NULL) receives the step time in
 * microseconds measured with CUDA events, like the reference's return value. */
int p3x_main(p3x_context* ctx, const p3x_runtime* rt, const p3x_prognostic_state* prog,
             const p3x_diagnostic_inputs* din, const p3x_diagnostic_outputs* dout,
             const p3x_infrastructure* infra, const p3x_history_only* hist, int32_t nj, int32_t nk,
             const p3x_layout* layout, int32_t precision, void* stream, double* elapsed_us);

/* Same step on HOST buffers: every pointer of prog / din / dout / hist is a
 * host array in the same (nj, ld) layout (page-locked memory for full
 * speed).  The columns are processed in chunks of chunk_cols (0: a sixteenth
 * of nj, at least 8192) through a ring of three device chunk buffers on the
 * context's own streams, so one chunk's upload, another's kernels and a
 * third's download run at once.  Uploads the prognostic state and the
 * diagnostic inputs, downloads the prognostic state, the diagnostic outputs
 * and the history fields.  Synchronous: returns when the host arrays hold
 * the results; *elapsed_us (may be NULL) receives the time from the first
 * upload to the last download.  Results are bitwise those of p3x_main on the
 * same data.  Calls on one context are serialised (they share its chunk
 * buffers); calls on different contexts run concurrently.  The reference's host drivers pass host views to p3_main
 * through its own deep copies; this entry is that path without them. */
int p3x_main_host(p3x_context* ctx, const p3x_runtime* rt, const p3x_prognostic_state* prog,
                  const p3x_diagnostic_inputs* din, const p3x_diagnostic_outputs* dout,
                  const p3x_infrastructure* infra, const p3x_history_only* hist, int32_t nj, int32_t nk,
                  const p3x_layout* layout, int32_t precision, int32_t chunk_cols, double* elapsed_us);

/* Same, stream-ordered and asynchronous: no host synchronisation.  The
 * per-step hand-over scratch between the three kernels (40 B per
 * column-level + 4 B per column + 16 B of work counters) is taken from and returned to the
 * context's stream-ordered memory pool on `stream`, so concurrent calls on
 * different streams do not share scratch.  Device-side error bits accumulate
 * in the context; read them with p3x_context_check. */
int p3x_main_async(p3x_context* ctx, const p3x_runtime* rt, const p3x_prognostic_state* prog,
                   const p3x_diagnostic_inputs* din, const p3x_diagnostic_outputs* dout,
                   const p3x_infrastructure* infra, const p3x_history_only* hist, int32_t nj,
                   int32_t nk, const p3x_layout* layout, int32_t precision, void* stream);

/* Same step as p3x_main_async, but the hand-over scratch between its three
 * kernels comes from one 64 MiB array of static device storage instead of
 * the context's memory pool, so the call allocates no device memory: for
 * hosts that reserve the device's memory for themselves at start-up and
 * cannot let a library allocate during their time loop.  No counterpart in
 * the reference.
 *   - Limit: 40 * ncol * ld + 4 * ncol + 16 bytes (rounded up) must fit in
 *     64 MiB, e.g. 13,000 columns of 128 levels; larger calls return
 *     P3X_ENOMEM and launch nothing.
 *   - The array is one per device and shared by every context: calls that
 *     overlap on the device (different streams or host threads) race on it
 *     and must be serialised by the caller.
 *   - p3x_context_create reserves the array on the context's device and
 *     looks its address up there (cudaGetSymbolAddress, once per device), so
 *     the reservation happens at start-up, before any stream capture.  Call
 *     this entry with the context's device current; otherwise it returns
 *     P3X_EINVAL.
 *   - Nothing in the array has to be zeroed (the step zeroes its work
 *     counters on the stream). */
int p3x_main_fixed_scratch(p3x_context* ctx, const p3x_runtime* rt, const p3x_prognostic_state* prog,
                           const p3x_diagnostic_inputs* din, const p3x_diagnostic_outputs* dout,
                           const p3x_infrastructure* infra, const p3x_history_only* hist, int32_t nj,
                           int32_t nk, const p3x_layout* layout, int32_t precision, void* stream);

/* Capacity in bytes of the static scratch of p3x_main_fixed_scratch, and
 * whether it is reserved on the context's device (1 once the context
 * exists).  No counterpart in the reference. */
int p3x_fixed_scratch_info(const p3x_context* ctx, int64_t* capacity_bytes, int32_t* reserved);

/* ------------------------------------------------------------------ */
/* Process interface around the step (P3Microphysics pre/postamble)    */
/* ------------------------------------------------------------------ */
/* Host-model fields of the P3 atmosphere process
 * (physics/p3/eamxx_p3_process_interface.hpp:63-353).  Device pointers;
 * per-level fields are (ncol, nlev) with the layout's ld, per-column fields
 * have ncol entries.  Per-column pointers may be NULL (skipped). */
typedef struct p3x_interface_fields {
  const double *pmid, *pseudo_density, *pseudo_density_dry, *cld_frac_t;
  double* T_atm;                /* preamble: in; postamble: in/out          */
  double* T_prev;               /* postamble: out                           */
  double *precip_liq_surf_mass, /* per column, accumulated by the postamble */
      *precip_ice_surf_mass;
  double *vapor_flux, *water_flux, *ice_flux, *heat_flux; /* per column, out */
} p3x_interface_fields;

/* p3_preamble (eamxx_p3_process_interface.hpp:63-132): dz from the wet
 * state, wet -> dry mixing ratios of the 9 prognostic species and qv_prev,
 * inv_exner and th from T_atm and pmid, cloud fractions floored at 1e-4 and
 * the rain fraction's maximum overlap with the level above.  Writes prog and
 * din's dz, inv_exner, cld_frac_l/i/r and qv_prev (which must be writable). */
int p3x_preamble(const p3x_interface_fields* f, const p3x_prognostic_state* prog,
                 const p3x_diagnostic_inputs* din, int32_t nj, int32_t nk, const p3x_layout* layout,
                 void* stream);

/* p3_postamble (eamxx_p3_process_interface.hpp:200-269): T_atm from th with
 * the dry/wet rescaled increment, T_prev, dry -> wet mixing ratios and
 * qv_prev, effective radii in microns, surface precipitation mass
 * accumulated over dt, and the mass/energy boundary fluxes. */
int p3x_postamble(const p3x_interface_fields* f, const p3x_prognostic_state* prog,
                  const p3x_diagnostic_inputs* din, const p3x_diagnostic_outputs* dout, int32_t nj,
                  int32_t nk, const p3x_layout* layout, double dt, void* stream);

/* ------------------------------------------------------------------ */
/* EAM driver around the step (micro_p3_tend)                          */
/* ------------------------------------------------------------------ */
/* Fields of EAM's P3 driver micro_p3_tend
 * (eam/src/physics/p3/scream/micro_p3_interface.F90:735-1484) on the
 * device: the physics state it reads, the physics-buffer fields it carries
 * between steps, the tendencies it returns and its diagnostics.  Per-level
 * fields are (ncol, nlev) with the layout's ld; zi, flxprc and flxsnw
 * (nlev+1 interfaces, top first) use ld_int; per-column fields have ncol
 * entries.  q and ptend_q hold the driver's nine constituents in this
 * order: qv, cldliq, numliq, rain, numrain, cldice, numice, cldrim, rimvol
 * (wet mixing ratios, as in state%q).  Diagnostic pointers may be NULL
 * (not computed); everything else is required. */
typedef struct p3x_eam_fields {
  /* physics state (read only) */
  const double *pmid, *pmiddry, *pdel, *pdeldry, *zi, *t;
  const double* q[9];
  /* physics buffer inputs (read only): cloud fraction, activation
   * tendencies, cloud-liquid relative variance, macrophysics condensation */
  const double *ast, *npccn, *ni_activated, *relvar, *cmeliq;
  /* physics buffer carried between steps (in/out): T and wet qv at the end
   * of the previous step */
  double *t_prev, *qv_prev;
  /* tendencies (out): dry static energy and the nine constituents */
  double* ptend_s;
  double* ptend_q[9];
  /* diagnostics (out, optional) */
  double *qme, *rho, *icimrst, *icwmrst, *icinc, *icwnc, *rel, *rei, *dei, *mu, *lambdac, *nfice, *efcout,
      *ncout, *freql, *efiout, *niout, *freqi, *aqrain, *anrain, *freqr, *reff_rain, *deff_rain;
  double *flxprc, *flxsnw;                                  /* interfaces */
  double *prec_pcw, *snow_pcw, *prec_str, *snow_str, *cdnumc; /* per column */
  int32_t subgrid_clouds;     /* micro_subgrid_cloud: 0 = all cloud fractions 1 */
  int32_t precip_frac_method; /* P3X_PRECIP_FRAC_MAX_OVERLAP (the driver's) or _IN_CLOUD */
} p3x_eam_fields;

#define P3X_PRECIP_FRAC_MAX_OVERLAP 0
#define P3X_PRECIP_FRAC_IN_CLOUD 1

/* The driver's preparation of the P3 inputs (micro_p3_interface.F90:
 * 982-1047, get_cloud_fraction :661-732): wet -> dry mixing ratios by
 * pdel / pdeldry into prog (qv, qc, nc, qr, nr, qi, ni, qm, bm) and qv_prev,
 * inv_exner = 1 / (pmid 1e-5)^(rair / cp), dz from zi, th = T inv_exner,
 * pres = pmiddry, dpres = pdeldry, the cloud fractions, nc_nuceat_tend =
 * npccn, ni_activated, inv_qc_relvar = relvar and t_prev, into din (whose
 * arrays must be writable; nccn is left to the caller). */
int p3x_eam_tend_pre(const p3x_eam_fields* e, const p3x_prognostic_state* prog,
                     const p3x_diagnostic_inputs* din, int32_t nj, int32_t nk, const p3x_layout* layout,
                     void* stream);

/* The driver's use of the P3 results (micro_p3_interface.F90:1182-1431):
 * dry -> wet by pdeldry / pdel, the enthalpy-rescaled temperature change,
 * ptend_s and ptend_q (of the non-negative wet values), t_prev and the wet
 * qv_prev, qme and vap_liq_exchange += cmeliq (hist), surface precipitation
 * for export, radiation and COSP diagnostics.  mu and lambdac: the
 * reference's Fortran p3_main returns the cloud-droplet shape and slope,
 * which the C++ p3_main replaced here does not; they are written as the
 * driver's initial values (0) except where ast < 1e-4, where the driver's
 * convective values apply. */
int p3x_eam_tend_post(const p3x_eam_fields* e, const p3x_prognostic_state* prog,
                      const p3x_diagnostic_inputs* din, const p3x_diagnostic_outputs* dout,
                      const p3x_history_only* hist, int32_t nj, int32_t nk, const p3x_layout* layout,
                      double dt, void* stream);

/* micro_p3_tend on the device: p3x_eam_tend_pre, the P3 step (p3x_main_async
 * with infra's dt, it, predictNc and prescribedCCN) and p3x_eam_tend_post on
 * `stream`, asynchronously.  prog, din, dout and hist are the driver's
 * working arrays (its local copies of the state).  The arguments of all three
 * parts are checked before the first launch: P3X_EINVAL leaves every array
 * as it was. */
int p3x_eam_micro_p3_tend(p3x_context* ctx, const p3x_runtime* rt, const p3x_eam_fields* e,
                          const p3x_prognostic_state* prog, const p3x_diagnostic_inputs* din,
                          const p3x_diagnostic_outputs* dout, const p3x_infrastructure* infra,
                          const p3x_history_only* hist, int32_t nj, int32_t nk, const p3x_layout* layout,
                          int32_t precision, void* stream);

/* ------------------------------------------------------------------ */
/* The step in stages (stage-by-stage checks against a CPU restatement) */
/* ------------------------------------------------------------------ */
/* No counterpart in the reference, whose p3_main runs its stages inside one
 * kernel (p3_main_impl.hpp:108-325).  The step is three kernels in a row:
 *   P3X_STAGE_PART12  p3_main_init + p3_main_part1 + p3_main_part2
 *   P3X_STAGE_SED     cloud, rain and ice sedimentation
 *   P3X_STAGE_PART3   homogeneous freezing + p3_main_part3
 * p3x_main_stages runs the subset `stages` (OR of the bits) in that order on
 * `stream`, asynchronously, with the hand-over between them in the caller's
 * DEVICE buffer `handover` (16-byte aligned, p3x_handover_bytes(nj, ld)
 * bytes) instead of the context's pool, so a caller can stop after part2,
 * inspect or replace the hand-over and the state, and resume.  All three
 * stages in one call give exactly p3x_main_async.  Hand-over layout (ld as in
 * the call's layout):
 *   doubles [5][nj][ld]: the temperature after part1 (homogeneous freezing
 *     reads it), the air density, rhofacr, rhofaci and acn; in the FP32-bulk
 *     form the last four hold floats in the first half of each column's row;
 *   then int32 [nj]: 1 where the column goes on past part2, 0 where it took
 *     one of the step's early exits (later stages skip it);
 *   then the stages' work counters (zeroed by the call).
 * Only the rows of columns that go on are written by P3X_STAGE_PART12. */
#define P3X_STAGE_PART12 1
#define P3X_STAGE_SED 2
#define P3X_STAGE_PART3 4
int p3x_handover_bytes(int32_t nj, int64_t ld, int64_t* bytes);
int p3x_main_stages(p3x_context* ctx, const p3x_runtime* rt, const p3x_prognostic_state* prog,
                    const p3x_diagnostic_inputs* din, const p3x_diagnostic_outputs* dout,
                    const p3x_infrastructure* infra, const p3x_history_only* hist, int32_t nj, int32_t nk,
                    const p3x_layout* layout, int32_t precision, int32_t stages, void* handover,
                    void* stream);

/* Device self-test of numeric building blocks (no counterpart in the
 * reference): for all 2^32 float bit patterns, compares the FP32-bulk form's
 * integer-pipe float -> double conversion with the hardware conversion and
 * its FP32-pipe table indices with the hardware truncation (after the table
 * lookups' clamps), and checks its small-integer floats; for 2^32 doubles
 * covering every high word, compares its integer-pipe narrowing toward zero
 * with the hardware conversion; *mismatches receives the number of
 * disagreements (0 expected). */
int p3x_selftest(uint64_t* mismatches);

/* Per-kernel timing of single-instance steps (no counterpart in the
 * reference, which times p3_main as a whole): while on, every p3x_main /
 * p3x_main_async records CUDA events around its three kernels (part1+part2,
 * sedimentation, part3); p3x_kernel_times waits for the latest such step and
 * returns the three durations in ms. */
int p3x_set_kernel_timing(p3x_context* ctx, int32_t on);
int p3x_kernel_times(p3x_context* ctx, float* ms3);

/* check_values (physics/p3/impl/p3_check_values_impl.hpp:26-81, called after
 * part3 at p3_main_impl.hpp:316-323 in the reference's debug builds only): a
 * range check of every level of every column that went on past part2, T =
 * th / inv_exner in (173, 323) K and qv in (0, 0.04) kg/kg.  Modes:
 *   P3X_CHECK_OFF     no check (default; the reference's release build);
 *   P3X_CHECK_RECORD  out-of-range levels are counted (the reference's debug
 *                     build, which prints them and goes on);
 *   P3X_CHECK_FAIL    also, a temperature out of range makes the step
 *                     return P3X_ERANGE (the reference's debug abort; qv out
 *                     of range is only counted there too).  Nothing traps.
 * The mode applies to steps launched after the call, including new batches,
 * served requests and graphs captured afterwards.  p3x_check_values_report
 * synchronises `stream`, returns the counts and the smallest (instance,
 * column, level) of each kind since the previous report (-1 when none;
 * instance is 0 for single-instance steps), and clears them. */
#define P3X_CHECK_OFF 0
#define P3X_CHECK_RECORD 1
#define P3X_CHECK_FAIL 2
typedef struct p3x_check_report {
  int64_t t_out_of_range;  /* levels with T not in (173, 323) K    */
  int64_t qv_out_of_range; /* levels with qv not in (0, 0.04) kg/kg */
  int32_t t_first_instance, t_first_column, t_first_level;
  int32_t qv_first_instance, qv_first_column, qv_first_level;
} p3x_check_report;
int p3x_set_check_values(p3x_context* ctx, int32_t mode);
int p3x_check_values_report(p3x_context* ctx, void* stream, p3x_check_report* out);

/* Synchronises `stream`, returns and clears the accumulated device status. */
int p3x_context_check(p3x_context* ctx, void* stream);

/* Overrides the launch configuration used by p3x_main (and the host and
 * fixed-scratch entries, new batches and served requests) for a precision
 * form.  Defaults:
 * FP64 {16, 4, 0, 0}, FP32-bulk {32, 4, 0, 0}. */
int p3x_set_launch_config(p3x_context* ctx, int32_t precision, const p3x_launch_config* cfg);
int p3x_get_launch_config(const p3x_context* ctx, int32_t precision, p3x_launch_config* cfg);

/* p3_main_c (physics/p3/p3_iso_c.f90:132-183), same argument order, types
 * and meaning: HOST arrays in the Fortran (its:ite, kts:kte) layout (column
 * index fastest), precip fluxes (its:ite, kts:kte+1); its/ite/kts/kte/it are
 * c_int and do_predict_nc/do_prescribed_CCN are logical(c_bool), all by
 * value.  Unlike the reference subroutine it returns a status.  Uses the
 * default context created by p3x_init.  Runs FP64 on the current device.
 * elapsed_s receives the step time in seconds. */
int p3x_init(const char* table_file, int* info);
int p3x_finalize(void);
int p3x_main_f(double* qc, double* nc, double* qr, double* nr, double* th_atm, double* qv,
               double dt, double* qi, double* qm, double* ni, double* bm, double* pres,
               double* dz, double* nc_nuceat_tend, double* nccn_prescribed, double* ni_activated,
               double* inv_qc_relvar, int32_t it, double* precip_liq_surf,
               double* precip_ice_surf, int32_t its, int32_t ite, int32_t kts, int32_t kte,
               double* diag_eff_radius_qc, double* diag_eff_radius_qi,
               double* diag_eff_radius_qr, double* rho_qi, bool do_predict_nc,
               bool do_prescribed_CCN, double* dpres, double* inv_exner,
               double* qv2qi_depos_tend, double* precip_liq_flux, double* precip_ice_flux,
               double* cld_frac_r, double* cld_frac_l, double* cld_frac_i,
               double* liq_ice_exchange, double* vap_liq_exchange, double* vap_ice_exchange,
               double* qv_prev, double* t_prev, double* elapsed_s);

/* ------------------------------------------------------------------ */
/* Batched form: many independent instances in one persistent launch   */
/* ------------------------------------------------------------------ */
typedef struct p3x_instance_desc {
  p3x_prognostic_state prog;
  p3x_diagnostic_inputs din;
  p3x_diagnostic_outputs dout;
  p3x_history_only hist;
  p3x_layout layout;
  int32_t ncol, nlev;
  double dt;
  int32_t it;
  int32_t predictNc, prescribedCCN;
  int32_t precision;
} p3x_instance_desc;

typedef struct p3x_batch p3x_batch;

/* Builds the device work list (one item per column of every instance,
 * heaviest first) for n instances.  Allocates once, here. */
int p3x_batch_create(p3x_context* ctx, const p3x_runtime* rt, const p3x_instance_desc* descs,
                     int32_t n, p3x_batch** out);
/* One persistent launch over the work list on `stream` (no host sync). */
int p3x_batch_run(p3x_batch* b, void* stream);
/* Captures the batch launch into a CUDA graph; later p3x_batch_run calls
 * replay the graph. */
int p3x_batch_capture_graph(p3x_batch* b, void* stream);
int p3x_batch_set_launch_config(p3x_batch* b, const p3x_launch_config* cfg);
int p3x_batch_destroy(p3x_batch* b);

/* Autotuner: times candidate launch configurations (lanes per column x
 * columns per CTA x table staging x blocks per SM) on the given batch and
 * stores the fastest in *best (and in the batch).  ms_best may be NULL. */
int p3x_autotune_batch(p3x_batch* b, void* stream, int32_t reps, p3x_launch_config* best,
                       double* ms_best);

/* ------------------------------------------------------------------ */
/* Synthetic workload (seeded standard-atmosphere columns)             */
/* ------------------------------------------------------------------ */
/* Field order of the 23 P3 inputs handled by the generator and the
 * serving loop: the 10 prognostic fields then the 13 diagnostic inputs. */
enum {
  P3X_F_QC = 0, P3X_F_NC, P3X_F_QR, P3X_F_NR, P3X_F_QI, P3X_F_QM, P3X_F_NI, P3X_F_BM,
  P3X_F_QV, P3X_F_TH, P3X_F_NC_NUCEAT_TEND, P3X_F_NCCN, P3X_F_NI_ACTIVATED,
  P3X_F_INV_QC_RELVAR, P3X_F_CLD_FRAC_I, P3X_F_CLD_FRAC_L, P3X_F_CLD_FRAC_R, P3X_F_PRES,
  P3X_F_DZ, P3X_F_DPRES, P3X_F_INV_EXNER, P3X_F_QV_PREV, P3X_F_T_PREV, P3X_NUM_INPUTS
};

/* Fills columns [col0, col0+ncol) of a workload (HOST arrays, (ncol, nlev)
 * row-major with leading dimension ld).  kind 0: RH ~ U(0.3, 1.05);
 * kind 1: RH ~ U(0.9, 1.05) in even-indexed columns (supersaturation
 * stress); kind 2: the reference's "mixed" test case
 * (physics/p3/p3_ic_cases.cpp:11-120).  Column i draws from its own stream
 * seeded by (seed, i), so any column range is reproducible on its own. */
int p3x_workload_generate(int32_t kind, uint64_t seed, int32_t col0, int32_t ncol, int32_t nlev,
                          double* const* fields, int64_t ld);

/* Column budgets in FP64 (share/property_checks/
 * mass_and_energy_column_conservation_check.cpp:281-347): total water
 * W = sum_k (qv+qc+qr+qi) dpres/g and energy-like
 * E = sum_k (cp T + (Lv+Lf) qv + Lf (qc+qr)) dpres/g, per column, device
 * arrays.  T is th/inv_exner.  Asynchronous on `stream`. */
int p3x_column_budgets(const p3x_prognostic_state* prog, const double* dpres,
                       const double* inv_exner, int32_t ncol, int32_t nlev, int64_t ld,
                       double* water_out, double* energy_out, void* stream);

/* Column mass and energy conservation check around the P3 process
 * (share/property_checks/mass_and_energy_column_conservation_check.cpp):
 * host-model fields after the process (device pointers; per-level
 * (ncol, nlev) with leading dimension ld, horiz_winds (ncol, 2, nlev) with
 * the same ld, per-column (ncol)).  horiz_winds, ps, phis and the fluxes may
 * be NULL (kinetic energy, phis ps / g and that flux are then left out). */
typedef struct p3x_conservation_fields {
  const double *pseudo_density, *T_mid, *qv, *qc, *qi, *qr;
  const double* horiz_winds;
  const double *ps, *phis;
  const double *vapor_flux, *water_flux, *ice_flux, *heat_flux;
} p3x_conservation_fields;

/* Column totals, device arrays of ncol (either may be NULL):
 * mass = sum_k (qv+qc+qi+qr) pseudo_density / g (:281-298), energy =
 * sum_k (cp T + (u^2+v^2)/2 + (Lv+Lf) qv + Lf (qc+qr)) pseudo_density / g
 * + phis ps / g (:314-347).  Call it before the process (the reference's
 * compute_current_mass / compute_current_energy).  Asynchronous. */
int p3x_column_mass_energy(const p3x_conservation_fields* f, int32_t ncol, int32_t nlev, int64_t ld, double* mass,
                           double* energy, void* stream);

/* The check (:110-208): per column the relative error of the mass against
 * mass_before + (vapor_flux - water_flux rho_w) dt and of the energy against
 * energy_before + (vapor_flux (Lv+Lf) - (water_flux - ice_flux) rho_w Lf
 * + heat_flux) dt, into the caller's device arrays mass_err / energy_err
 * (ncol each); then the largest of each with its column (the smallest
 * column among equal maxima) into *out, and pass = both below their
 * tolerances (the reference driver's defaults are 1e-10 for mass and 1e-14
 * for energy, atmosphere_driver.cpp:428-429).  Synchronises `stream`;
 * allocates nothing. */
typedef struct p3x_conservation_report {
  double max_mass_err, max_energy_err;
  int32_t mass_col, energy_col;
  int32_t pass, pad_;
} p3x_conservation_report;
int p3x_conservation_check(p3x_context* ctx, const p3x_conservation_fields* f, const double* mass_before,
                           const double* energy_before, int32_t ncol, int32_t nlev, int64_t ld, double dt,
                           double mass_tol, double energy_tol, double* mass_err, double* energy_err,
                           p3x_conservation_report* out, void* stream);

/* ------------------------------------------------------------------ */
/* Serving: continuous batching of P3 steps under a memory budget      */
/* ------------------------------------------------------------------ */
typedef struct p3x_server p3x_server;

typedef struct p3x_serve_stats {
  int64_t completed;
  int64_t rejected;        /* larger than the whole budget               */
  double p50_ms, p90_ms, p99_ms, max_ms, mean_ms;
  double wall_s;
  double column_levels_per_s;
  double offered_rate_hz;
  int64_t peak_bytes;
  int32_t peak_inflight;
  int32_t pad_;
  /* per size class, ncol in [1,10), [10,100), [100,1000), [1000,10000),
   * [10000, 65536]: completed requests and latency percentiles */
  int64_t class_count[5];
  double class_p50_ms[5], class_p99_ms[5];
  /* latency / isolated service time of the same request (0 until
   * p3x_server_calibrate has run) */
  double slowdown_p50, slowdown_p99;
  /* bytes copied host -> device (first-step state uploads) and device ->
   * host (every step's result) */
  int64_t h2d_bytes, d2h_bytes;
} p3x_serve_stats;

/* Requests carry data: an instance's first step uploads its 23 input fields
 * from page-locked host memory, and every step downloads its result (the 10
 * prognostic fields and the two surface precipitation rates) to page-locked
 * host memory before it completes; latency covers both copies.
 * budget_bytes: device memory the server may hold for resident instances.
 * max_inflight: concurrent steps (one CUDA stream each). */
int p3x_server_create(p3x_context* ctx, const p3x_runtime* rt, int64_t budget_bytes,
                      int32_t max_inflight, p3x_server** out);
int p3x_server_destroy(p3x_server* s);

/* Submits a request: instance `instance_id` (created on first use, nlev 72
 * or 128, ncol <= 65536) advances by one step.  Its initial state is columns
 * [c0, c0 + ncol) of the server's synthetic workload (standard-atmosphere columns,
 * workload seed 5000) with c0 = seed mod (65536 - ncol + 1).  The instance
 * stays resident, readable with p3x_server_read_field, until the server is
 * destroyed.  arrival_s is the request's arrival time on the server clock
 * (seconds since p3x_server_create).  Non-blocking: requests run in
 * p3x_server_drain.  Returns P3X_ENOMEM (and counts a rejection) when the
 * instance alone exceeds the budget. */
int p3x_server_submit(p3x_server* s, int64_t instance_id, int32_t ncol, int32_t nlev,
                      int32_t precision, int32_t total_steps, uint64_t seed, double dt,
                      double arrival_s);

/* Runs a Poisson load of n sessions drawn from a seeded generator (ncol
 * log-uniform in [1, max_ncol], nlev from {72,128}, FP64 / FP32-bulk 50/50,
 * 1..20 steps each).  Sessions arrive at rate_hz; a session's first step
 * request arrives with it, each further step request arrives when the
 * previous step completes, and its memory is released after its last step.
 * Blocks until every session has finished; stats cover this run only
 * (latency = completion - arrival of each step request). */
int p3x_server_run_poisson(p3x_server* s, double rate_hz, int32_t n_requests,
                           int32_t max_ncol, uint64_t seed, p3x_serve_stats* stats);

/* Copies one prognostic field (P3X_F_QC..P3X_F_TH) or a surface precip
 * field (-1: precip_liq_surf, -2: precip_ice_surf) of a resident instance to
 * host memory (for result checks). */
int p3x_server_read_field(p3x_server* s, int64_t instance_id, int32_t field, double* host_out,
                          int64_t n);
/* Waits until every submitted request has finished. */
int p3x_server_drain(p3x_server* s, p3x_serve_stats* stats);

/* Measures isolated service times: two-step sessions alone on an otherwise
 * idle server, ncol in {1, 8, 64, 512, 4096, 32768, 65536}, both level
 * counts and both precision forms, best of two; a first step (which uploads
 * the state) and a later step are timed separately.  Later statistics then
 * report the slowdown (latency over the isolated time of the same kind of
 * step, log-log interpolated in ncol).  Calibration runs each step as one
 * launch sequence on the whole device, whatever the SM partition and the
 * dispatch chunk.  p3x_server_isolated_ms returns that
 * interpolated time of a later step.  No counterpart in the reference. */
int p3x_server_calibrate(p3x_server* s);

/* Dispatch policy (no counterpart in the reference).  on = 1 (the default,
 * share 0.875): a dispatch holds requests of one size kind (small: at most
 * 2^19 column-levels); a dispatch of more than 2^20 column-levels takes
 * large_grid_share of the kernels' resident-block capacity, leaving room on
 * every SM for other slots; and the last slot (when there is more than one)
 * takes only small instances, on the highest-priority stream.  Small
 * requests then wait less behind large steps, at some cost in throughput.
 * on = 0: every ready request of a precision is packed together, on any
 * slot, at full capacity.  Waits for running work first. */
int p3x_server_set_latency_policy(p3x_server* s, int32_t on, double large_grid_share);

/* SM partition (no counterpart in the reference).  small_sms > 0 splits the
 * device's SMs into two green contexts: at least small_sms SMs (rounded up to
 * the device's partition granularity, 8 on this architecture) for the last
 * slot, the rest for the other slots.  The last slot then takes only
 * instances of at most small_max_cl column-levels and the other slots never
 * take those, so a small request never waits for SMs that a large step holds;
 * each dispatch's persistent grids are sized to its partition.  small_sms = 0
 * removes the partition.  Needs max_inflight >= 2.  P3X_ECUDA where the
 * driver offers no green contexts (the server is then left unpartitioned).
 * Waits for
 * running work first.  sms_out (optional, 2 int32): the SMs of the small
 * partition and of the rest, 0 when unpartitioned. */
int p3x_server_set_sm_partition(p3x_server* s, int32_t small_sms, int64_t small_max_cl, int32_t* sms_out);

/* Dispatch chunking (no counterpart in the reference): a dispatch of more
 * than max_cl column-levels runs as consecutive launches of at most max_cl
 * column-levels each, so other slots' kernels reach the SMs between them
 * instead of waiting for a whole large step's kernels; 0 launches every
 * dispatch at once.  Default 2^18 (2,048 columns of 128 levels).  Results do
 * not depend on it.  Waits for running work first. */
int p3x_server_set_dispatch_chunk(p3x_server* s, int64_t max_cl);
int p3x_server_isolated_ms(p3x_server* s, int32_t precision, int32_t nlev, int32_t ncol, double* ms);

/* Checkpoint / resume of a resident instance (no counterpart in the
 * reference's interface; its restart carries the same state, including
 * qv_prev and T_prev: eamxx_p3_process_interface.cpp:93-94).
 * export: copies the instance's 23 input fields, [P3X_NUM_INPUTS][ncol][nlev]
 * in P3X_F_* order (n >= 23 ncol nlev doubles), to host memory; the instance
 * must be idle (drained).  import: makes instance `instance_id` (which must
 * not exist) resident with that state; later p3x_server_submit calls step
 * it, bitwise as if it had never left.  Like an explicit instance after its
 * last step, an idle imported instance may be evicted when admission needs
 * its memory. */
int p3x_server_export_instance(p3x_server* s, int64_t instance_id, double* host_state, int64_t n);
int p3x_server_import_instance(p3x_server* s, int64_t instance_id, int32_t ncol, int32_t nlev, int32_t precision,
                               double dt, const double* host_state, int64_t n);

/* Version string of the library build. */
const char* p3x_version(void);

#ifdef __cplusplus
}
#endif

#endif /* P3X_H */
