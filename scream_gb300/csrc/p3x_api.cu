/*
 * C ABI of libp3x (declared in include/p3x.h): lookup-table contexts, the
 * p3_main drop-in (device pointers), the p3_main_c drop-in (host arrays in the
 * Fortran layout), the batched persistent form with CUDA-graph capture and
 * its autotuner, synthetic workloads and column budgets.
 */
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "p3x.h"
#include "p3x_internal.hpp"
#include "p3x_launch.hpp"

struct p3x_context {
  int device = 0;
  int num_sms = 0;
  p3x::HostTables host;
  /* device tables, FP64 and FP32 copies */
  double *d_ice = nullptr, *d_coll = nullptr, *d_vn = nullptr, *d_vm = nullptr, *d_revap = nullptr;
  float *f_ice = nullptr, *f_coll = nullptr, *f_vn = nullptr, *f_vm = nullptr, *f_revap = nullptr;
  /* FP32 ice-table columns of ice sedimentation only (slots 0-3, 16 bytes a
   * row): a third of the rows' cache footprint */
  float* f_ice_sed = nullptr;
  /* Table3 two-column slices for every possible mu index (1..9):
   * [9][3][300][2] */
  double* d_t3slices = nullptr;
  float* f_t3slices = nullptr;
  double* d_svp = nullptr; /* FP32-bulk saturation table */
  uint32_t* d_err = nullptr;
  /* check_values words (dev::kCheckWords) and mode (P3X_CHECK_*) */
  unsigned long long* d_check = nullptr;
  int check_mode = 0;
  /* conservation check: {max mass err, column, max energy err, column} */
  double* d_maxloc = nullptr;
  /* stream-ordered pool of the per-call K1->K2/K3 scratch (memory is kept
   * for reuse; released with the context) */
  cudaMemPool_t pool = nullptr;
  /* optional per-kernel timing of single-instance steps */
  int ktime = 0;
  cudaEvent_t kev[4] = {nullptr, nullptr, nullptr, nullptr};
  p3x_launch_config cfg[2];
  /* scratch of the Fortran-layout entry (grown on demand) */
  std::vector<double*> fbuf;
  int64_t fbuf_elems = 0;
  double* fstage = nullptr;
  int64_t fstage_elems = 0;
  /* host-buffer entry: a ring of device chunk buffers, one stream each
   * (grown on demand) */
  static constexpr int kHostRing = 3;
  cudaStream_t hstream[kHostRing] = {nullptr, nullptr, nullptr};
  double* hbuf[kHostRing] = {nullptr, nullptr, nullptr};
  size_t hbuf_bytes = 0;
  std::mutex hmu; /* one host-entry call at a time per context (the ring is shared) */
};

namespace p3x {
namespace {

int cuda_status(cudaError_t e) {
  if (e == cudaSuccess) return P3X_OK;
  if (e == cudaErrorMemoryAllocation) return P3X_ENOMEM;
  return P3X_ECUDA;
}
#define P3X_CUDA(x)                         \
  do {                                      \
    const cudaError_t e_ = (x);             \
    if (e_ != cudaSuccess) return cuda_status(e_); \
  } while (0)

int status_from_bits(uint32_t bits) {
  if (bits & dev::kErrNumeric) return P3X_ENUMERIC;
  if (bits & (dev::kErrSubstep | dev::kErrWait)) return P3X_ETIMEOUT;
  if (bits & dev::kErrRange) return P3X_ERANGE;
  return P3X_OK;
}

/* check_values words after a reset: counts 0, first keys "none" */
int reset_check_words(unsigned long long* d, cudaStream_t st) {
  const unsigned long long init[dev::kCheckWords] = {0ull, 0ull, ~0ull, ~0ull};
  return cuda_status(cudaMemcpyAsync(d, init, sizeof(init), cudaMemcpyHostToDevice, st));
}

std::mutex g_tables_mu;
std::unique_ptr<HostTables> g_generated;

/* Generated tables are built once per process (the ice-table generation
 * integrates ~1e9 PSD bins). */
const HostTables& generated_tables() {
  std::lock_guard<std::mutex> lk(g_tables_mu);
  if (!g_generated) {
    auto t = std::make_unique<HostTables>();
    build_rain_tables(*t, 1.0);
    build_ice_tables(*t);
    g_generated = std::move(t);
  }
  return *g_generated;
}

template <class T>
int upload(T** dst, const std::vector<double>& src) {
  std::vector<T> tmp(src.begin(), src.end());
  P3X_CUDA(cudaMalloc(reinterpret_cast<void**>(dst), sizeof(T) * tmp.size()));
  P3X_CUDA(cudaMemcpy(*dst, tmp.data(), sizeof(T) * tmp.size(), cudaMemcpyHostToDevice));
  return P3X_OK;
}

dev::RuntimeDev make_runtime(const p3x_runtime& r) {
  dev::RuntimeDev d;
  d.max_total_ni = r.max_total_ni;
  d.autoconversion_prefactor = r.autoconversion_prefactor;
  d.autoconversion_qc_exponent = r.autoconversion_qc_exponent;
  d.autoconversion_nc_exponent = r.autoconversion_nc_exponent;
  d.autoconversion_radius = r.autoconversion_radius;
  d.accretion_prefactor = r.accretion_prefactor;
  d.accretion_qc_exponent = r.accretion_qc_exponent;
  d.accretion_qr_exponent = r.accretion_qr_exponent;
  d.rain_selfcollection_prefactor = r.rain_selfcollection_prefactor;
  d.rain_selfcollection_breakup_diameter = r.rain_selfcollection_breakup_diameter;
  d.constant_mu_rain = r.constant_mu_rain;
  d.spa_ccn_to_nc_factor = r.spa_ccn_to_nc_factor;
  d.cldliq_to_ice_collection_factor = r.cldliq_to_ice_collection_factor;
  d.rain_to_ice_collection_factor = r.rain_to_ice_collection_factor;
  d.min_rime_rho = r.min_rime_rho;
  d.max_rime_rho = r.max_rime_rho;
  d.immersion_freezing_exponent = r.immersion_freezing_exponent;
  d.deposition_nucleation_exponent = r.deposition_nucleation_exponent;
  d.ice_sedimentation_factor = r.ice_sedimentation_factor;
  d.do_ice_production = r.do_ice_production;
  /* p3/impl/p3_autoconversion_impl.hpp:27-32 */
  if (r.autoconversion_radius == 25.0e-6) {
    d.cons3 = dev::C::CONS3;
  } else {
    d.cons3 = 1.0 / (dev::C::CONS2 * std::pow(r.autoconversion_radius, 3.0));
  }
  /* p3/impl/p3_table3_impl.hpp:52-62 with the constant mu_r */
  double rdumjj = r.constant_mu_rain + 1;
  rdumjj = std::max(rdumjj, 1.);
  rdumjj = std::min(rdumjj, 10.);
  int dumjj = static_cast<int>(rdumjj);
  dumjj = std::max(dumjj, 1);
  dumjj = std::min(dumjj, 9);
  d.t3_rdumjj = rdumjj;
  d.t3_dumjj = dumjj;
  const double mu_r = r.constant_mu_rain;
  d.g_mur1 = std::tgamma(mu_r + 1.0);
  d.g_mur2 = std::tgamma(mu_r + 2.0);
  d.lg_mur4 = std::log(std::tgamma(mu_r + 4.0));
  d.lg_mur7 = std::log(std::tgamma(mu_r + 7.0));
  d.accretion_same_exponent = r.accretion_qc_exponent == r.accretion_qr_exponent ? 1 : 0;
  /* float copies for the FP32-bulk rates (round to nearest, as a device
   * conversion gives) */
  d.f.max_total_ni = float(d.max_total_ni);
  d.f.autoconversion_prefactor = float(d.autoconversion_prefactor);
  d.f.autoconversion_qc_exponent = float(d.autoconversion_qc_exponent);
  d.f.autoconversion_nc_exponent = float(d.autoconversion_nc_exponent);
  d.f.accretion_prefactor = float(d.accretion_prefactor);
  d.f.accretion_qc_exponent = float(d.accretion_qc_exponent);
  d.f.accretion_qr_exponent = float(d.accretion_qr_exponent);
  d.f.rain_selfcollection_prefactor = float(d.rain_selfcollection_prefactor);
  d.f.rain_selfcollection_breakup_diameter = float(d.rain_selfcollection_breakup_diameter);
  d.f.constant_mu_rain = float(d.constant_mu_rain);
  d.f.cldliq_to_ice_collection_factor = float(d.cldliq_to_ice_collection_factor);
  d.f.rain_to_ice_collection_factor = float(d.rain_to_ice_collection_factor);
  d.f.min_rime_rho = float(d.min_rime_rho);
  d.f.max_rime_rho = float(d.max_rime_rho);
  d.f.immersion_freezing_exponent = float(d.immersion_freezing_exponent);
  d.f.deposition_nucleation_exponent = float(d.deposition_nucleation_exponent);
  d.f.ice_sedimentation_factor = float(d.ice_sedimentation_factor);
  d.f.cons3 = float(d.cons3);
  d.f.t3_rdumjj = float(d.t3_rdumjj);
  d.f.g_mur1 = float(d.g_mur1);
  d.f.g_mur2 = float(d.g_mur2);
  d.f.lg_mur4 = float(d.lg_mur4);
  d.f.lg_mur7 = float(d.lg_mur7);
  return d;
}

bool valid_runtime(const p3x_runtime& r) {
  return std::isfinite(r.constant_mu_rain) && r.max_rime_rho > 0 && r.min_rime_rho > 0 &&
         std::isfinite(r.max_total_ni) && r.autoconversion_radius > 0;
}

LaunchSpec spec_of(const p3x_launch_config& c) {
  LaunchSpec s;
  s.lanes = c.lanes_per_column;
  s.groups_per_block = c.columns_per_block;
  s.staged = c.table_staging;
  s.blocks_per_sm = c.blocks_per_sm;
  return s;
}

int sm_stride_for(int nlev_max) {
  int s = nlev_max + 1;
  return (s + 1) & ~1;
}

bool spec_fits(int precision, const LaunchSpec& ls, int stride) {
  if (ls.lanes != 8 && ls.lanes != 16 && ls.lanes != 32) return false;
  if (ls.groups_per_block <= 0 || ls.groups_per_block * ls.lanes > 256) return false;
  const bool f32 = precision == P3X_FP32_BULK;
  const size_t k1 = f32 ? p3_smem_bytes<float>(ls, stride) : p3_smem_bytes<double>(ls, stride);
  const LaunchSpec ls2 = sed_spec(ls);
  const size_t k2 = f32 ? sed_smem_bytes<float>(ls2, stride) : sed_smem_bytes<double>(ls2, stride);
  return k1 <= size_t(227 * 1024) && k2 <= size_t(227 * 1024);
}

/* Falls back to tables in global memory and then to fewer columns per CTA
 * when a configuration does not fit in shared memory (very deep columns). */
LaunchSpec fit_spec(int precision, LaunchSpec ls, int stride) {
  if (spec_fits(precision, ls, stride)) return ls;
  ls.staged = 0;
  while (ls.groups_per_block > 1 && !spec_fits(precision, ls, stride)) ls.groups_per_block /= 2;
  return ls;
}

template <class TR>
dev::KParams<TR> make_kparams(p3x_context* ctx, const dev::RuntimeDev& rtd);

template <>
dev::KParams<double> make_kparams<double>(p3x_context* ctx, const dev::RuntimeDev& rtd) {
  dev::KParams<double> kp{};
  kp.rt = rtd;
  kp.ice = ctx->d_ice;
  kp.collect = ctx->d_coll;
  kp.vn = ctx->d_vn;
  kp.vm = ctx->d_vm;
  kp.revap = ctx->d_revap;
  kp.t3slice = ctx->d_t3slices + size_t(rtd.t3_dumjj - 1) * dev::kT3SliceElems;
  kp.rt.svp_tab = ctx->d_svp;
  kp.err = ctx->d_err;
  kp.check = ctx->check_mode ? ctx->d_check : nullptr;
  kp.check_fail = ctx->check_mode == P3X_CHECK_FAIL ? 1 : 0;
  return kp;
}
template <>
dev::KParams<float> make_kparams<float>(p3x_context* ctx, const dev::RuntimeDev& rtd) {
  dev::KParams<float> kp{};
  kp.rt = rtd;
  kp.ice = ctx->f_ice;
  kp.ice_sed = ctx->f_ice_sed;
  kp.collect = ctx->f_coll;
  kp.vn = ctx->f_vn;
  kp.vm = ctx->f_vm;
  kp.revap = ctx->f_revap;
  kp.t3slice = ctx->f_t3slices + size_t(rtd.t3_dumjj - 1) * dev::kT3SliceElems;
  kp.rt.svp_tab = ctx->d_svp;
  kp.err = ctx->d_err;
  kp.check = ctx->check_mode ? ctx->d_check : nullptr;
  kp.check_fail = ctx->check_mode == P3X_CHECK_FAIL ? 1 : 0;
  return kp;
}

int fill_inst(const p3x_prognostic_state* prog, const p3x_diagnostic_inputs* din,
              const p3x_diagnostic_outputs* dout, const p3x_history_only* hist, const p3x_layout* layout,
              int32_t nj, int32_t nk, double dt, int predictNc, int prescribedCCN, int precision,
              dev::Inst& in) {
  if (!prog || !din || !dout || !hist) return P3X_EINVAL;
  if (nj < 0 || nk <= 0 || !(dt > 0)) return P3X_EINVAL;
  if (precision != P3X_FP64 && precision != P3X_FP32_BULK) return P3X_EINVAL;
  in.qc = prog->qc; in.nc = prog->nc; in.qr = prog->qr; in.nr = prog->nr; in.qi = prog->qi;
  in.qm = prog->qm; in.ni = prog->ni; in.bm = prog->bm; in.qv = prog->qv; in.th = prog->th;
  in.nc_nuceat_tend = din->nc_nuceat_tend; in.nccn = din->nccn; in.ni_activated = din->ni_activated;
  in.inv_qc_relvar = din->inv_qc_relvar; in.cld_frac_i = din->cld_frac_i; in.cld_frac_l = din->cld_frac_l;
  in.cld_frac_r = din->cld_frac_r; in.pres = din->pres; in.dz = din->dz; in.dpres = din->dpres;
  in.inv_exner = din->inv_exner; in.qv_prev = din->qv_prev; in.t_prev = din->t_prev;
  in.qv2qi_depos_tend = dout->qv2qi_depos_tend; in.precip_liq_surf = dout->precip_liq_surf;
  in.precip_ice_surf = dout->precip_ice_surf; in.diag_eff_radius_qc = dout->diag_eff_radius_qc;
  in.diag_eff_radius_qi = dout->diag_eff_radius_qi; in.diag_eff_radius_qr = dout->diag_eff_radius_qr;
  in.rho_qi = dout->rho_qi; in.precip_liq_flux = dout->precip_liq_flux; in.precip_ice_flux = dout->precip_ice_flux;
  in.precip_total_tend = dout->precip_total_tend; in.nevapr = dout->nevapr;
  in.liq_ice_exchange = hist->liq_ice_exchange; in.vap_liq_exchange = hist->vap_liq_exchange;
  in.vap_ice_exchange = hist->vap_ice_exchange;
  const void* ptrs[] = {in.qc, in.nc, in.qr, in.nr, in.qi, in.qm, in.ni, in.bm, in.qv, in.th,
                        in.nc_nuceat_tend, in.nccn, in.ni_activated, in.inv_qc_relvar, in.cld_frac_i,
                        in.cld_frac_l, in.cld_frac_r, in.pres, in.dz, in.dpres, in.inv_exner, in.qv_prev,
                        in.t_prev, in.qv2qi_depos_tend, in.precip_liq_surf, in.precip_ice_surf,
                        in.diag_eff_radius_qc, in.diag_eff_radius_qi, in.diag_eff_radius_qr, in.rho_qi,
                        in.precip_liq_flux, in.precip_ice_flux, in.precip_total_tend, in.nevapr,
                        in.liq_ice_exchange, in.vap_liq_exchange, in.vap_ice_exchange};
  if (nj > 0)
    for (const void* p : ptrs)
      if (!p) return P3X_EINVAL;
  in.ld = (layout && layout->ld > 0) ? layout->ld : nk;
  in.ld_int = (layout && layout->ld_int > 0) ? layout->ld_int : nk + 1;
  if (in.ld < nk || in.ld_int < nk + 1) return P3X_EINVAL;
  in.ncol = nj;
  in.nlev = nk;
  in.dt = dt;
  in.predictNc = predictNc ? 1 : 0;
  in.prescribedCCN = prescribedCCN ? 1 : 0;
  in.precision = precision;
  in.pad_ = 0;
  in.scr = nullptr;
  in.cflag = nullptr;
  return P3X_OK;
}

void bind_scratch(dev::Inst& in, unsigned char* base) {
  in.scr = reinterpret_cast<double*>(base);
  in.cflag = reinterpret_cast<int32_t*>(base + size_t(dev::kScrFields) * size_t(in.ncol) * size_t(in.ld) *
                                        sizeof(double));
}

uint32_t* work_counters(const dev::Inst& in) {
  return reinterpret_cast<uint32_t*>(reinterpret_cast<unsigned char*>(in.scr) +
                                     dev::work_counter_offset(in.ncol, in.ld));
}

int launch_kernels(p3x_context* ctx, const p3x_runtime* rt, const dev::Inst& in, cudaStream_t st,
                   bool marks = true, int parts = kPartK1 | kPartK2 | kPartK3) {
  const dev::RuntimeDev rtd = make_runtime(*rt);
  const int stride = sm_stride_for(in.nlev);
  LaunchSpec ls = fit_spec(in.precision, spec_of(ctx->cfg[in.precision]), stride);
  if (ctx->ktime && marks) ls.marks = ctx->kev;
  if (!spec_fits(in.precision, ls, stride)) return P3X_EINVAL;
  cudaError_t e;
  if (in.precision == P3X_FP32_BULK) {
    dev::KParams<float> kp = make_kparams<float>(ctx, rtd);
    kp.sm_stride = stride;
    kp.nwork = in.ncol;
    kp.work = nullptr;
    kp.insts = nullptr;
    kp.wctr = work_counters(in);
    e = launch_p3<float>(in, kp, ls, ctx->num_sms, st, parts);
  } else {
    dev::KParams<double> kp = make_kparams<double>(ctx, rtd);
    kp.sm_stride = stride;
    kp.nwork = in.ncol;
    kp.work = nullptr;
    kp.insts = nullptr;
    kp.wctr = work_counters(in);
    e = launch_p3<double>(in, kp, ls, ctx->num_sms, st, parts);
  }
  return cuda_status(e);
}

/* One step of one instance: the K1->K2/K3 scratch comes from the context's
 * stream-ordered pool and returns to it behind the three kernels. */
int launch_single(p3x_context* ctx, const p3x_runtime* rt, const dev::Inst& in_, cudaStream_t st,
                  bool marks = true) {
  if (in_.ncol == 0) return P3X_OK;
  dev::Inst in = in_;
  void* scr = nullptr;
  P3X_CUDA(cudaMallocFromPoolAsync(&scr, dev::scratch_bytes(in.ncol, in.ld), ctx->pool, st));
  bind_scratch(in, static_cast<unsigned char*>(scr));
  const int rc = launch_kernels(ctx, rt, in, st, marks);
  const cudaError_t fe = cudaFreeAsync(scr, st);
  if (rc) return rc;
  return cuda_status(fe);
}

int read_and_clear_err(p3x_context* ctx, cudaStream_t st) {
  uint32_t bits = 0;
  P3X_CUDA(cudaMemcpyAsync(&bits, ctx->d_err, sizeof(bits), cudaMemcpyDeviceToHost, st));
  P3X_CUDA(cudaStreamSynchronize(st));
  if (bits) P3X_CUDA(cudaMemsetAsync(ctx->d_err, 0, sizeof(uint32_t), st));
  P3X_CUDA(cudaStreamSynchronize(st));
  return status_from_bits(bits);
}

p3x_context* g_default_ctx = nullptr;

struct OccKey {
  int device;
  const void* func;
  int threads;
  size_t smem;
  bool operator<(const OccKey& o) const {
    if (device != o.device) return device < o.device;
    if (func != o.func) return func < o.func;
    if (threads != o.threads) return threads < o.threads;
    return smem < o.smem;
  }
};
std::mutex g_occ_mu;
std::map<OccKey, int> g_occ;
std::map<std::pair<int, const void*>, size_t> g_smem_limit;

}  // namespace

cudaError_t kernel_occupancy(const void* func, int threads, size_t smem, int* per_sm) {
  int device = 0;
  cudaError_t e = cudaGetDevice(&device);
  if (e != cudaSuccess) return e;
  const OccKey key{device, func, threads, smem};
  std::lock_guard<std::mutex> lk(g_occ_mu);
  const auto it = g_occ.find(key);
  if (it != g_occ.end()) {
    *per_sm = it->second;
    return cudaSuccess;
  }
  /* the limit only grows, so shapes cached earlier stay launchable */
  size_t& limit = g_smem_limit[{device, func}];
  if (smem > limit) {
    e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
    limit = smem;
  }
  int n = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, func, threads, smem);
  if (e != cudaSuccess) return e;
  g_occ[key] = n;
  *per_sm = n;
  return cudaSuccess;
}
}  // namespace p3x

using namespace p3x;

extern "C" {

const char* p3x_version(void) { return "p3x 0.1 (sm_103a)"; }

void p3x_runtime_defaults(p3x_runtime* rt) {
  if (!rt) return;
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

int p3x_tables_generate(const char* table_file, double* ice, double* collect, double* vn, double* vm,
                        double* revap, double* mu_r, double* dnu) {
  HostTables t;
  if (table_file) {
    if (read_ice_table_file(table_file, "4.1.1", t) != 0) return P3X_ETABLE;
    build_rain_tables(t, 1.0);
  } else {
    t = generated_tables();
  }
  if (ice) std::copy(t.ice.begin(), t.ice.end(), ice);
  if (collect) std::copy(t.collect.begin(), t.collect.end(), collect);
  if (vn) std::copy(t.vn.begin(), t.vn.end(), vn);
  if (vm) std::copy(t.vm.begin(), t.vm.end(), vm);
  if (revap) std::copy(t.revap.begin(), t.revap.end(), revap);
  if (mu_r) std::copy(t.mu_r.begin(), t.mu_r.end(), mu_r);
  if (dnu) std::copy(t.dnu.begin(), t.dnu.end(), dnu);
  return P3X_OK;
}

double p3x_incomplete_gamma_q(double a, double x) { return incomplete_gamma_q(a, x); }

static_assert(p3x::kSvpIntervals == dev::kSvpIntervals && p3x::kSvpT0 == dev::kSvpT0 &&
                  p3x::kSvpInvH == dev::kSvpInvH,
              "saturation table layout differs between host and device");

int p3x_saturation_table(double* coef, int32_t* intervals, double* t0, double* inv_h) {
  if (intervals) *intervals = kSvpIntervals;
  if (t0) *t0 = kSvpT0;
  if (inv_h) *inv_h = kSvpInvH;
  if (coef) {
    std::vector<double> v;
    build_svp_table(v);
    std::copy(v.begin(), v.end(), coef);
  }
  return P3X_OK;
}

int p3x_write_ice_table(const char* path, const char* version) {
  if (!path) return P3X_EINVAL;
  return write_ice_table_file(path, version ? version : "4.1.1") == 0 ? P3X_OK : P3X_ETABLE;
}

}  // extern "C"

/* ------------------------------------------------------------------ */
/* Fixed, pre-reserved hand-over scratch (p3x_main_fixed_scratch)     */
/* ------------------------------------------------------------------ */
/* Some hosts cannot let a library take device memory while their time loop
 * runs: a model that reserves nearly all of HBM for its own pool at
 * start-up, or one that must keep a fixed, audited device footprint for a
 * whole simulation, has no memory to give and no way to account for a pool
 * that grows behind its back.  For them the three kernels' hand-over scratch
 * (40 bytes per column-level, 4 bytes per column and 16 bytes of work
 * counters) lives in one array of static device storage.  This translation
 * unit holds no kernel, so with lazy module loading the array is only
 * reserved on a device when its address is first looked up; context
 * creation does that, on the context's device, so the reservation happens at
 * start-up and never inside a caller's time loop.  Nothing in the array needs
 * to start at zero: the step zeroes its work counters on the stream, and
 * part1+part2 writes every column's continue flag, and the hand-over values
 * of every column that goes on, before sedimentation and part3 read them. */
static __device__ __align__(256) unsigned char g_step_scratch[p3x::kFixedScratchBytes];

namespace p3x {
namespace {
constexpr int kMaxDevices = 64;
std::mutex g_step_scratch_mu;
void* g_step_scratch_ptr[kMaxDevices] = {};

/* Address of the array on `device`, which must be the current device (a
 * symbol's address is looked up on the current one).  Looked up once per
 * device; the lookup loads this module there and so reserves the array. */
int step_scratch_address(int device, void** out) {
  int cur = -1;
  P3X_CUDA(cudaGetDevice(&cur));
  if (device < 0 || device >= kMaxDevices || cur != device) return P3X_EINVAL;
  std::lock_guard<std::mutex> lk(g_step_scratch_mu);
  if (!g_step_scratch_ptr[device]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_step_scratch);
    if (e != cudaSuccess) return cuda_status(e);
    g_step_scratch_ptr[device] = p;
  }
  *out = g_step_scratch_ptr[device];
  return P3X_OK;
}

bool step_scratch_reserved(int device) {
  if (device < 0 || device >= kMaxDevices) return false;
  std::lock_guard<std::mutex> lk(g_step_scratch_mu);
  return g_step_scratch_ptr[device] != nullptr;
}
}  // namespace
}  // namespace p3x

extern "C" {

int p3x_context_create(const char* table_file, p3x_context** out, int* info) {
  if (info) *info = 0;
  if (!out) return P3X_EINVAL;
  *out = nullptr;
  auto ctx = std::make_unique<p3x_context>();
  if (table_file) {
    HostTables t;
    const int rc = read_ice_table_file(table_file, "4.1.1", t);
    if (rc != 0) {
      if (info) *info = P3X_ETABLE;
      return P3X_ETABLE;
    }
    build_rain_tables(t, 1.0);
    ctx->host = std::move(t);
  } else {
    ctx->host = generated_tables();
  }
  int st;
  if (cudaGetDevice(&ctx->device) != cudaSuccess) {
    if (info) *info = P3X_ECUDA;
    return P3X_ECUDA;
  }
  cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, ctx->device);
  const HostTables& H = ctx->host;
  /* device copies of the ice table hold its columns in slot order */
  std::vector<double> ice_slots(H.ice.size());
  for (size_t row = 0; row < H.ice.size() / dev::kIceCols; ++row)
    for (int s = 0; s < dev::kIceCols; ++s)
      ice_slots[row * dev::kIceCols + s] = H.ice[row * dev::kIceCols + dev::kIceSlotCol[s]];
  std::vector<double> ice_sed(H.ice.size() / dev::kIceCols * dev::kIceSedCols);
  for (size_t row = 0; row < H.ice.size() / dev::kIceCols; ++row)
    for (int s = 0; s < dev::kIceSedCols; ++s) ice_sed[row * dev::kIceSedCols + s] = ice_slots[row * dev::kIceCols + s];
  if ((st = upload(&ctx->d_ice, ice_slots)) || (st = upload(&ctx->f_ice_sed, ice_sed)) ||
      (st = upload(&ctx->d_coll, H.collect)) ||
      (st = upload(&ctx->d_vn, H.vn)) || (st = upload(&ctx->d_vm, H.vm)) ||
      (st = upload(&ctx->d_revap, H.revap)) || (st = upload(&ctx->f_ice, ice_slots)) ||
      (st = upload(&ctx->f_coll, H.collect)) || (st = upload(&ctx->f_vn, H.vn)) ||
      (st = upload(&ctx->f_vm, H.vm)) || (st = upload(&ctx->f_revap, H.revap))) {
    if (info) *info = st;
    p3x_context_destroy(ctx.release());
    return st;
  }
  /* Table3 slices for mu index j = 1..9: columns (j-1, j) of vn, vm, revap */
  std::vector<double> sl(size_t(9) * dev::kT3SliceElems);
  for (int j = 1; j <= 9; ++j) {
    double* s = &sl[size_t(j - 1) * dev::kT3SliceElems];
    const std::vector<double>* tabs[3] = {&H.vn, &H.vm, &H.revap};
    for (int t = 0; t < 3; ++t)
      for (int i = 0; i < kVT0; ++i)
        for (int c = 0; c < 2; ++c) s[t * 600 + i * 2 + c] = (*tabs[t])[size_t(i) * kVT1 + (j - 1 + c)];
  }
  std::vector<double> svp;
  build_svp_table(svp);
  if ((st = upload(&ctx->d_t3slices, sl)) || (st = upload(&ctx->f_t3slices, sl)) || (st = upload(&ctx->d_svp, svp))) {
    if (info) *info = st;
    p3x_context_destroy(ctx.release());
    return st;
  }
  if (cudaMalloc(&ctx->d_err, sizeof(uint32_t)) != cudaSuccess ||
      cudaMemset(ctx->d_err, 0, sizeof(uint32_t)) != cudaSuccess ||
      cudaMalloc(&ctx->d_check, dev::kCheckWords * sizeof(unsigned long long)) != cudaSuccess ||
      cudaMalloc(&ctx->d_maxloc, 4 * sizeof(double)) != cudaSuccess ||
      reset_check_words(ctx->d_check, nullptr) != P3X_OK || cudaDeviceSynchronize() != cudaSuccess) {
    if (info) *info = P3X_ENOMEM;
    p3x_context_destroy(ctx.release());
    return P3X_ENOMEM;
  }
  {
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = ctx->device;
    uint64_t keep = UINT64_MAX;
    if (cudaMemPoolCreate(&ctx->pool, &props) != cudaSuccess ||
        cudaMemPoolSetAttribute(ctx->pool, cudaMemPoolAttrReleaseThreshold, &keep) != cudaSuccess) {
      if (info) *info = P3X_ECUDA;
      p3x_context_destroy(ctx.release());
      return P3X_ECUDA;
    }
  }
  /* 4 columns per CTA with the tables read through L1: part1+part2 then fits
   * two CTAs per SM (staging the tables in shared memory leaves room for one),
   * measured faster in both forms; staging remains a launch option.  The FP64
   * part1+part2 (254 registers) keeps twice the columns in flight at 16 lanes
   * per column and ran 7 % faster there (sedimentation stays at 32). */
  ctx->cfg[P3X_FP64] = p3x_launch_config{16, 4, 0, 0};
  ctx->cfg[P3X_FP32_BULK] = p3x_launch_config{32, 4, 0, 0};
  /* reserve the fixed hand-over scratch of p3x_main_fixed_scratch on this
   * device now (see g_step_scratch) */
  {
    void* scr = nullptr;
    if ((st = step_scratch_address(ctx->device, &scr))) {
      if (info) *info = st;
      p3x_context_destroy(ctx.release());
      return st;
    }
  }
  *out = ctx.release();
  return P3X_OK;
}

int p3x_context_destroy(p3x_context* ctx) {
  if (!ctx) return P3X_EINVAL;
  void* ptrs[] = {ctx->d_ice, ctx->d_coll, ctx->d_vn, ctx->d_vm, ctx->d_revap, ctx->f_ice, ctx->f_ice_sed, ctx->f_coll,
                  ctx->f_vn, ctx->f_vm, ctx->f_revap, ctx->d_t3slices, ctx->f_t3slices, ctx->d_svp, ctx->d_err,
                  ctx->d_check, ctx->d_maxloc, ctx->fstage};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  for (double* p : ctx->fbuf)
    if (p) cudaFree(p);
  if (ctx->pool) {
    cudaDeviceSynchronize();
    cudaMemPoolDestroy(ctx->pool);
  }
  for (cudaEvent_t e : ctx->kev)
    if (e) cudaEventDestroy(e);
  for (int i = 0; i < p3x_context::kHostRing; ++i) {
    if (ctx->hbuf[i]) cudaFree(ctx->hbuf[i]);
    if (ctx->hstream[i]) cudaStreamDestroy(ctx->hstream[i]);
  }
  delete ctx;
  return P3X_OK;
}

int p3x_context_get_tables(const p3x_context* ctx, double* ice, double* collect, double* vn, double* vm,
                           double* revap, double* mu_r, double* dnu) {
  if (!ctx) return P3X_EINVAL;
  const HostTables& H = ctx->host;
  if (ice) std::copy(H.ice.begin(), H.ice.end(), ice);
  if (collect) std::copy(H.collect.begin(), H.collect.end(), collect);
  if (vn) std::copy(H.vn.begin(), H.vn.end(), vn);
  if (vm) std::copy(H.vm.begin(), H.vm.end(), vm);
  if (revap) std::copy(H.revap.begin(), H.revap.end(), revap);
  if (mu_r) std::copy(H.mu_r.begin(), H.mu_r.end(), mu_r);
  if (dnu) std::copy(H.dnu.begin(), H.dnu.end(), dnu);
  return P3X_OK;
}

int p3x_set_launch_config(p3x_context* ctx, int32_t precision, const p3x_launch_config* cfg) {
  if (!ctx || !cfg || (precision != P3X_FP64 && precision != P3X_FP32_BULK)) return P3X_EINVAL;
  const LaunchSpec ls = spec_of(*cfg);
  if (!spec_fits(precision, ls, sm_stride_for(1))) return P3X_EINVAL;
  ctx->cfg[precision] = *cfg;
  return P3X_OK;
}

int p3x_get_launch_config(const p3x_context* ctx, int32_t precision, p3x_launch_config* cfg) {
  if (!ctx || !cfg || (precision != P3X_FP64 && precision != P3X_FP32_BULK)) return P3X_EINVAL;
  *cfg = ctx->cfg[precision];
  return P3X_OK;
}

int p3x_main_async(p3x_context* ctx, const p3x_runtime* rt, const p3x_prognostic_state* prog,
                   const p3x_diagnostic_inputs* din, const p3x_diagnostic_outputs* dout,
                   const p3x_infrastructure* infra, const p3x_history_only* hist, int32_t nj, int32_t nk,
                   const p3x_layout* layout, int32_t precision, void* stream) {
  if (!ctx || !rt || !infra || !valid_runtime(*rt)) return P3X_EINVAL;
  dev::Inst in;
  const int st = fill_inst(prog, din, dout, hist, layout, nj, nk, infra->dt, infra->predictNc,
                           infra->prescribedCCN, precision, in);
  if (st) return st;
  return launch_single(ctx, rt, in, static_cast<cudaStream_t>(stream));
}

int p3x_set_check_values(p3x_context* ctx, int32_t mode) {
  if (!ctx || mode < P3X_CHECK_OFF || mode > P3X_CHECK_FAIL) return P3X_EINVAL;
  ctx->check_mode = mode;
  return P3X_OK;
}

int p3x_check_values_report(p3x_context* ctx, void* stream, p3x_check_report* out) {
  if (!ctx || !out) return P3X_EINVAL;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  unsigned long long w[dev::kCheckWords];
  P3X_CUDA(cudaMemcpyAsync(w, ctx->d_check, sizeof(w), cudaMemcpyDeviceToHost, st));
  P3X_CUDA(cudaStreamSynchronize(st));
  const int rc = reset_check_words(ctx->d_check, st);
  if (rc) return rc;
  P3X_CUDA(cudaStreamSynchronize(st));
  auto unpack = [](unsigned long long key, int32_t& inst, int32_t& col, int32_t& lev) {
    if (key == ~0ull) {
      inst = col = lev = -1;
    } else {
      inst = int32_t(key >> 40);
      col = int32_t((key >> 16) & 0xffffffull);
      lev = int32_t(key & 0xffffull);
    }
  };
  out->t_out_of_range = int64_t(w[dev::kChkTCount]);
  out->qv_out_of_range = int64_t(w[dev::kChkQvCount]);
  unpack(w[dev::kChkTFirst], out->t_first_instance, out->t_first_column, out->t_first_level);
  unpack(w[dev::kChkQvFirst], out->qv_first_instance, out->qv_first_column, out->qv_first_level);
  return P3X_OK;
}

int p3x_handover_bytes(int32_t nj, int64_t ld, int64_t* bytes) {
  if (nj < 0 || ld <= 0 || !bytes) return P3X_EINVAL;
  *bytes = int64_t(dev::scratch_bytes(nj, ld));
  return P3X_OK;
}

int p3x_main_stages(p3x_context* ctx, const p3x_runtime* rt, const p3x_prognostic_state* prog,
                    const p3x_diagnostic_inputs* din, const p3x_diagnostic_outputs* dout,
                    const p3x_infrastructure* infra, const p3x_history_only* hist, int32_t nj, int32_t nk,
                    const p3x_layout* layout, int32_t precision, int32_t stages, void* handover, void* stream) {
  if (!ctx || !rt || !infra || !valid_runtime(*rt)) return P3X_EINVAL;
  if (stages <= 0 || (stages & ~(kPartK1 | kPartK2 | kPartK3))) return P3X_EINVAL;
  dev::Inst in;
  const int st = fill_inst(prog, din, dout, hist, layout, nj, nk, infra->dt, infra->predictNc,
                           infra->prescribedCCN, precision, in);
  if (st) return st;
  if (in.ncol == 0) return P3X_OK;
  if (!handover || (reinterpret_cast<uintptr_t>(handover) & 15)) return P3X_EINVAL;
  bind_scratch(in, static_cast<unsigned char*>(handover));
  return launch_kernels(ctx, rt, in, static_cast<cudaStream_t>(stream), false, stages);
}

int p3x_selftest(uint64_t* mismatches) {
  if (!mismatches) return P3X_EINVAL;
  unsigned long long* d = nullptr;
  P3X_CUDA(cudaMalloc(&d, sizeof(*d)));
  cudaError_t e = cudaMemset(d, 0, sizeof(*d));
  if (e == cudaSuccess) e = launch_selftest(d, nullptr);
  unsigned long long h = 0;
  if (e == cudaSuccess) e = cudaMemcpy(&h, d, sizeof(h), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return cuda_status(e);
  *mismatches = uint64_t(h);
  return P3X_OK;
}

int p3x_set_kernel_timing(p3x_context* ctx, int32_t on) {
  if (!ctx) return P3X_EINVAL;
  if (on && !ctx->kev[0])
    for (cudaEvent_t& e : ctx->kev) P3X_CUDA(cudaEventCreate(&e));
  ctx->ktime = on ? 1 : 0;
  return P3X_OK;
}

int p3x_kernel_times(p3x_context* ctx, float* ms3) {
  if (!ctx || !ms3 || !ctx->kev[0]) return P3X_EINVAL;
  P3X_CUDA(cudaEventSynchronize(ctx->kev[3]));
  for (int i = 0; i < 3; ++i) P3X_CUDA(cudaEventElapsedTime(&ms3[i], ctx->kev[i], ctx->kev[i + 1]));
  return P3X_OK;
}

int p3x_context_check(p3x_context* ctx, void* stream) {
  if (!ctx) return P3X_EINVAL;
  return read_and_clear_err(ctx, static_cast<cudaStream_t>(stream));
}

int p3x_main(p3x_context* ctx, const p3x_runtime* rt, const p3x_prognostic_state* prog,
             const p3x_diagnostic_inputs* din, const p3x_diagnostic_outputs* dout,
             const p3x_infrastructure* infra, const p3x_history_only* hist, int32_t nj, int32_t nk,
             const p3x_layout* layout, int32_t precision, void* stream, double* elapsed_us) {
  if (!ctx || !rt || !infra || !valid_runtime(*rt)) return P3X_EINVAL;
  dev::Inst in;
  int st = fill_inst(prog, din, dout, hist, layout, nj, nk, infra->dt, infra->predictNc, infra->prescribedCCN,
                     precision, in);
  if (st) return st;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaEvent_t e0, e1;
  P3X_CUDA(cudaEventCreate(&e0));
  P3X_CUDA(cudaEventCreate(&e1));
  cudaEventRecord(e0, s);
  st = launch_single(ctx, rt, in, s);
  cudaEventRecord(e1, s);
  const cudaError_t se = cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st) return st;
  if (se != cudaSuccess) return cuda_status(se);
  if (elapsed_us) *elapsed_us = double(ms) * 1000.0;
  return read_and_clear_err(ctx, s);
}

/* ------------------------------------------------------------------ */
/* Host-buffer entry: chunked, copies overlapped with the kernels       */
/* ------------------------------------------------------------------ */
namespace {

/* The fields of one call in the order of dev::Inst, with their row length
 * (0: one value per column, 1: ld, 2: ld_int) and direction (1 = uploaded,
 * 2 = downloaded, 3 = both). */
struct HostField {
  int rows;
  int dir;
};
constexpr int kNumHostFields = 37;
constexpr HostField kHostFields[kNumHostFields] = {
    {1, 3}, {1, 3}, {1, 3}, {1, 3}, {1, 3}, {1, 3}, {1, 3}, {1, 3}, {1, 3}, {1, 3},  /* prognostic state */
    {1, 1}, {1, 1}, {1, 1}, {1, 1}, {1, 1}, {1, 1}, {1, 1}, {1, 1}, {1, 1}, {1, 1},  /* diagnostic inputs */
    {1, 1}, {1, 1}, {1, 1},
    {1, 2}, {0, 2}, {0, 2}, {1, 2}, {1, 2}, {1, 2}, {1, 2}, {2, 2}, {2, 2}, {1, 2},  /* diagnostic outputs */
    {1, 2},
    {1, 2}, {1, 2}, {1, 2}};                                                          /* history */

/* the addresses of an Inst's field pointers, in kHostFields order */
void field_addrs(dev::Inst& in, const double** a[kNumHostFields]) {
  const double** v[kNumHostFields] = {
      const_cast<const double**>(&in.qc), const_cast<const double**>(&in.nc),
      const_cast<const double**>(&in.qr), const_cast<const double**>(&in.nr),
      const_cast<const double**>(&in.qi), const_cast<const double**>(&in.qm),
      const_cast<const double**>(&in.ni), const_cast<const double**>(&in.bm),
      const_cast<const double**>(&in.qv), const_cast<const double**>(&in.th),
      &in.nc_nuceat_tend, &in.nccn, &in.ni_activated, &in.inv_qc_relvar, &in.cld_frac_i, &in.cld_frac_l,
      &in.cld_frac_r, &in.pres, &in.dz, &in.dpres, &in.inv_exner, &in.qv_prev, &in.t_prev,
      const_cast<const double**>(&in.qv2qi_depos_tend), const_cast<const double**>(&in.precip_liq_surf),
      const_cast<const double**>(&in.precip_ice_surf), const_cast<const double**>(&in.diag_eff_radius_qc),
      const_cast<const double**>(&in.diag_eff_radius_qi), const_cast<const double**>(&in.diag_eff_radius_qr),
      const_cast<const double**>(&in.rho_qi), const_cast<const double**>(&in.precip_liq_flux),
      const_cast<const double**>(&in.precip_ice_flux), const_cast<const double**>(&in.precip_total_tend),
      const_cast<const double**>(&in.nevapr), const_cast<const double**>(&in.liq_ice_exchange),
      const_cast<const double**>(&in.vap_liq_exchange), const_cast<const double**>(&in.vap_ice_exchange)};
  for (int i = 0; i < kNumHostFields; ++i) a[i] = v[i];
}

int64_t row_len(const dev::Inst& in, int rows) { return rows == 0 ? 1 : (rows == 1 ? in.ld : in.ld_int); }

/* doubles of one chunk of `cols` columns of every field */
size_t chunk_elems(const dev::Inst& in, int64_t cols) {
  size_t n = 0;
  for (const HostField& f : kHostFields) n += size_t(cols) * size_t(row_len(in, f.rows));
  return n;
}

}  // namespace

int p3x_main_host(p3x_context* ctx, const p3x_runtime* rt, const p3x_prognostic_state* prog,
                  const p3x_diagnostic_inputs* din, const p3x_diagnostic_outputs* dout,
                  const p3x_infrastructure* infra, const p3x_history_only* hist, int32_t nj, int32_t nk,
                  const p3x_layout* layout, int32_t precision, int32_t chunk_cols, double* elapsed_us) {
  if (!ctx || !rt || !infra || !valid_runtime(*rt) || chunk_cols < 0) return P3X_EINVAL;
  dev::Inst host;
  int st = fill_inst(prog, din, dout, hist, layout, nj, nk, infra->dt, infra->predictNc, infra->prescribedCCN,
                     precision, host);
  if (st) return st;
  if (nj == 0) {
    if (elapsed_us) *elapsed_us = 0;
    return P3X_OK;
  }
  std::lock_guard<std::mutex> lock(ctx->hmu);
  /* chunks: a sixteenth of the columns (at least 8192, and all of them when
   * fewer), so that three chunks in flight overlap upload, kernels and
   * download.  At 345,600 x 128 on GB300 the step is then bound by the
   * host link (15.9 GB moved at ~290 GB/s both ways): 54.2 ms per step for
   * 16 chunks, 54.8 for 12, 56.8 for 8; a ring of 4 or 6 buffers measured
   * the same as 3. */
  int64_t cols = chunk_cols > 0 ? chunk_cols : std::max<int64_t>((int64_t(nj) + 15) / 16, 8192);
  cols = std::min<int64_t>(cols, nj);
  const size_t slot_bytes = chunk_elems(host, cols) * sizeof(double);
  if (slot_bytes > ctx->hbuf_bytes) {
    for (int i = 0; i < p3x_context::kHostRing; ++i) {
      if (ctx->hstream[i]) P3X_CUDA(cudaStreamSynchronize(ctx->hstream[i]));
      if (ctx->hbuf[i]) {
        cudaFree(ctx->hbuf[i]);
        ctx->hbuf[i] = nullptr;
      }
    }
    ctx->hbuf_bytes = 0;
    for (int i = 0; i < p3x_context::kHostRing; ++i) {
      if (cudaMalloc(&ctx->hbuf[i], slot_bytes) != cudaSuccess) {
        cudaGetLastError();
        for (int j = 0; j <= i; ++j) {
          if (ctx->hbuf[j]) cudaFree(ctx->hbuf[j]);
          ctx->hbuf[j] = nullptr;
        }
        return P3X_ENOMEM;
      }
    }
    ctx->hbuf_bytes = slot_bytes;
  }
  for (int i = 0; i < p3x_context::kHostRing; ++i)
    if (!ctx->hstream[i]) P3X_CUDA(cudaStreamCreateWithFlags(&ctx->hstream[i], cudaStreamNonBlocking));

  cudaEvent_t e0, e1;
  P3X_CUDA(cudaEventCreate(&e0));
  P3X_CUDA(cudaEventCreate(&e1));
  cudaEventRecord(e0, ctx->hstream[0]);
  for (int i = 1; i < p3x_context::kHostRing; ++i) cudaStreamWaitEvent(ctx->hstream[i], e0, 0);
  int nchunk = 0;
  for (int64_t c0 = 0; c0 < nj && st == P3X_OK; c0 += cols, ++nchunk) {
    const int slot = nchunk % p3x_context::kHostRing;
    cudaStream_t s = ctx->hstream[slot];
    const int64_t n = std::min<int64_t>(cols, int64_t(nj) - c0);
    dev::Inst chunk = host;
    chunk.ncol = int32_t(n);
    const double** ha[kNumHostFields];
    const double** ca[kNumHostFields];
    field_addrs(host, ha);
    field_addrs(chunk, ca);
    double* d = ctx->hbuf[slot];
    for (int i = 0; i < kNumHostFields && st == P3X_OK; ++i) {
      const int64_t len = row_len(host, kHostFields[i].rows);
      *ca[i] = d;
      if (kHostFields[i].dir & 1) {
        const cudaError_t e = cudaMemcpyAsync(d, *ha[i] + c0 * len, size_t(n * len) * sizeof(double),
                                              cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) st = cuda_status(e);
      }
      d += size_t(cols) * size_t(len);
    }
    if (st == P3X_OK) st = launch_single(ctx, rt, chunk, s, false);
    for (int i = 0; i < kNumHostFields && st == P3X_OK; ++i) {
      if (!(kHostFields[i].dir & 2)) continue;
      const int64_t len = row_len(host, kHostFields[i].rows);
      const cudaError_t e = cudaMemcpyAsync(const_cast<double*>(*ha[i]) + c0 * len, *ca[i],
                                            size_t(n * len) * sizeof(double), cudaMemcpyDeviceToHost, s);
      if (e != cudaSuccess) st = cuda_status(e);
    }
  }
  for (int i = 1; i < p3x_context::kHostRing; ++i) {
    cudaEvent_t ei;
    if (cudaEventCreateWithFlags(&ei, cudaEventDisableTiming) == cudaSuccess) {
      cudaEventRecord(ei, ctx->hstream[i]);
      cudaStreamWaitEvent(ctx->hstream[0], ei, 0);
      cudaEventDestroy(ei);
    }
  }
  cudaEventRecord(e1, ctx->hstream[0]);
  const cudaError_t se = cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st) return st;
  if (se != cudaSuccess) return cuda_status(se);
  if (elapsed_us) *elapsed_us = double(ms) * 1000.0;
  return read_and_clear_err(ctx, ctx->hstream[0]);
}

/* ------------------------------------------------------------------ */
/* Fortran-layout entry (p3_main_c)                                    */
/* ------------------------------------------------------------------ */
int p3x_init(const char* table_file, int* info) {
  if (g_default_ctx) return P3X_OK;
  return p3x_context_create(table_file, &g_default_ctx, info);
}

int p3x_finalize(void) {
  if (!g_default_ctx) return P3X_OK;
  const int st = p3x_context_destroy(g_default_ctx);
  g_default_ctx = nullptr;
  return st;
}

int p3x_main_f(double* qc, double* nc, double* qr, double* nr, double* th_atm, double* qv, double dt,
               double* qi, double* qm, double* ni, double* bm, double* pres, double* dz,
               double* nc_nuceat_tend, double* nccn_prescribed, double* ni_activated, double* inv_qc_relvar,
               int32_t it, double* precip_liq_surf, double* precip_ice_surf, int32_t its, int32_t ite,
               int32_t kts, int32_t kte, double* diag_eff_radius_qc, double* diag_eff_radius_qi,
               double* diag_eff_radius_qr, double* rho_qi, bool do_predict_nc, bool do_prescribed_CCN,
               double* dpres, double* inv_exner, double* qv2qi_depos_tend, double* precip_liq_flux,
               double* precip_ice_flux, double* cld_frac_r, double* cld_frac_l, double* cld_frac_i,
               double* liq_ice_exchange, double* vap_liq_exchange, double* vap_ice_exchange, double* qv_prev,
               double* t_prev, double* elapsed_s) {
  (void)it;
  if (!g_default_ctx) {
    int info = 0;
    const int st = p3x_init(nullptr, &info);
    if (st) return st;
  }
  p3x_context* ctx = g_default_ctx;
  if (!(dt > 0) || ite < its || kte < kts) return P3X_EINVAL;
  const int ncol = ite - its + 1, nlev = kte - kts + 1;
  /* fields in order: 23 inputs (P3X_F_*), then outputs */
  double* host[] = {qc, nc, qr, nr, qi, qm, ni, bm, qv, th_atm, nc_nuceat_tend, nccn_prescribed, ni_activated,
                    inv_qc_relvar, cld_frac_i, cld_frac_l, cld_frac_r, pres, dz, dpres, inv_exner, qv_prev,
                    t_prev,
                    /* 23.. outputs (mid levels) */
                    qv2qi_depos_tend, diag_eff_radius_qc, diag_eff_radius_qi, diag_eff_radius_qr, rho_qi,
                    liq_ice_exchange, vap_liq_exchange, vap_ice_exchange};
  constexpr int nin = P3X_NUM_INPUTS, nmid = nin + 8;
  for (double* p : host)
    if (!p) return P3X_EINVAL;
  if (!precip_liq_surf || !precip_ice_surf || !precip_liq_flux || !precip_ice_flux) return P3X_EINVAL;
  /* device buffers: nmid mid-level fields + 2 hidden mid (precip_total_tend,
   * nevapr) + 2 interface fields + 2 surface fields */
  const int64_t ld = nlev, ldi = nlev + 1;
  const int64_t mid = int64_t(ncol) * ld, itf = int64_t(ncol) * ldi;
  const int nbuf = nmid + 2 + 2 + 2;
  const int64_t need = std::max<int64_t>(mid, itf);
  if (int64_t(ctx->fbuf.size()) != nbuf || ctx->fbuf_elems < need) {
    for (double* p : ctx->fbuf)
      if (p) cudaFree(p);
    ctx->fbuf.assign(nbuf, nullptr);
    for (int b = 0; b < nbuf; ++b) P3X_CUDA(cudaMalloc(&ctx->fbuf[b], sizeof(double) * need));
    ctx->fbuf_elems = need;
  }
  if (ctx->fstage_elems < need) {
    if (ctx->fstage) cudaFree(ctx->fstage);
    P3X_CUDA(cudaMalloc(&ctx->fstage, sizeof(double) * need));
    ctx->fstage_elems = need;
  }
  cudaStream_t s = 0;
  /* host (its:ite, kts:kte) column-fastest -> device (ncol, nlev) */
  for (int f = 0; f < nin; ++f) {
    P3X_CUDA(cudaMemcpyAsync(ctx->fstage, host[f], sizeof(double) * mid, cudaMemcpyHostToDevice, s));
    P3X_CUDA(launch_transpose_to_levels(ctx->fstage, ctx->fbuf[f], ncol, nlev, ld, s));
  }
  double** B = ctx->fbuf.data();
  p3x_prognostic_state prog{B[0], B[1], B[2], B[3], B[4], B[5], B[6], B[7], B[8], B[9]};
  p3x_diagnostic_inputs din{B[10], B[11], B[12], B[13], B[14], B[15], B[16], B[17], B[18], B[19], B[20], B[21], B[22]};
  p3x_diagnostic_outputs dout{B[23], B[nmid + 4], B[nmid + 5], B[24], B[25], B[26], B[27],
                              B[nmid + 2], B[nmid + 3], B[nmid], B[nmid + 1]};
  p3x_history_only hist{B[28], B[29], B[30]};
  p3x_infrastructure infra{dt, it, its, ite, kts, kte, do_predict_nc ? 1 : 0, do_prescribed_CCN ? 1 : 0, nullptr};
  p3x_layout lay{ld, ldi};
  p3x_runtime rt;
  p3x_runtime_defaults(&rt);
  double us = 0;
  int st = p3x_main(ctx, &rt, &prog, &din, &dout, &infra, &hist, ncol, nlev, &lay, P3X_FP64, s, &us);
  if (st) return st;
  if (elapsed_s) *elapsed_s = us * 1e-6;
  /* copy back in/out and out fields */
  auto back = [&](const double* dsrc, double* hdst, int nl, int64_t ldx) -> int {
    P3X_CUDA(launch_transpose_to_columns(dsrc, ctx->fstage, ncol, nl, ldx, s));
    P3X_CUDA(cudaMemcpyAsync(hdst, ctx->fstage, sizeof(double) * int64_t(ncol) * nl, cudaMemcpyDeviceToHost, s));
    return P3X_OK;
  };
  for (int f = 0; f < P3X_F_TH + 1; ++f)
    if ((st = back(B[f], host[f], nlev, ld))) return st;
  for (int f = nin; f < nmid; ++f)
    if ((st = back(B[f], host[f], nlev, ld))) return st;
  if ((st = back(B[nmid + 2], precip_liq_flux, nlev + 1, ldi))) return st;
  if ((st = back(B[nmid + 3], precip_ice_flux, nlev + 1, ldi))) return st;
  P3X_CUDA(cudaMemcpyAsync(precip_liq_surf, B[nmid + 4], sizeof(double) * ncol, cudaMemcpyDeviceToHost, s));
  P3X_CUDA(cudaMemcpyAsync(precip_ice_surf, B[nmid + 5], sizeof(double) * ncol, cudaMemcpyDeviceToHost, s));
  P3X_CUDA(cudaStreamSynchronize(s));
  return P3X_OK;
}

/* ------------------------------------------------------------------ */
/* process interface pre/postamble                                    */
/* ------------------------------------------------------------------ */
static int interface_ptrs(const p3x_interface_fields* f, const p3x_prognostic_state* prog,
                          const p3x_diagnostic_inputs* din, const p3x_diagnostic_outputs* dout, bool post,
                          p3x::InterfacePtrs& p) {
  if (!f || !prog || !din) return P3X_EINVAL;
  if (!f->pmid || !f->pseudo_density || !f->pseudo_density_dry || !f->T_atm) return P3X_EINVAL;
  p = p3x::InterfacePtrs{};
  p.pmid = f->pmid; p.pd = f->pseudo_density; p.pdd = f->pseudo_density_dry; p.cld_t = f->cld_frac_t;
  p.T = f->T_atm; p.T_prev = f->T_prev;
  double* q[9] = {prog->qc, prog->nc, prog->qr, prog->nr, prog->qi, prog->ni, prog->qm, prog->bm, prog->qv};
  for (int s = 0; s < 9; ++s) {
    if (!q[s]) return P3X_EINVAL;
    p.q[s] = q[s];
  }
  p.th = prog->th;
  p.qv_prev = const_cast<double*>(din->qv_prev);
  if (!p.th || !p.qv_prev) return P3X_EINVAL;
  if (!post) {
    if (!f->cld_frac_t || !din->inv_exner || !din->dz || !din->cld_frac_l || !din->cld_frac_i || !din->cld_frac_r)
      return P3X_EINVAL;
    p.inv_exner = const_cast<double*>(din->inv_exner);
    p.dz = const_cast<double*>(din->dz);
    p.cld_l = const_cast<double*>(din->cld_frac_l);
    p.cld_i = const_cast<double*>(din->cld_frac_i);
    p.cld_r = const_cast<double*>(din->cld_frac_r);
  } else {
    if (!dout || !f->T_prev || !dout->diag_eff_radius_qc || !dout->diag_eff_radius_qi || !dout->diag_eff_radius_qr ||
        !dout->precip_liq_surf || !dout->precip_ice_surf)
      return P3X_EINVAL;
    p.eff_qc = dout->diag_eff_radius_qc; p.eff_qi = dout->diag_eff_radius_qi; p.eff_qr = dout->diag_eff_radius_qr;
    p.liq_surf = dout->precip_liq_surf; p.ice_surf = dout->precip_ice_surf;
    p.liq_mass = f->precip_liq_surf_mass; p.ice_mass = f->precip_ice_surf_mass;
    p.vapor_flux = f->vapor_flux; p.water_flux = f->water_flux; p.ice_flux = f->ice_flux; p.heat_flux = f->heat_flux;
  }
  return P3X_OK;
}

int p3x_preamble(const p3x_interface_fields* f, const p3x_prognostic_state* prog, const p3x_diagnostic_inputs* din,
                 int32_t nj, int32_t nk, const p3x_layout* layout, void* stream) {
  if (nj < 0 || nk <= 0) return P3X_EINVAL;
  p3x::InterfacePtrs p;
  const int st = interface_ptrs(f, prog, din, nullptr, false, p);
  if (st) return st;
  const int64_t ld = (layout && layout->ld > 0) ? layout->ld : nk;
  if (ld < nk) return P3X_EINVAL;
  return cuda_status(p3x::launch_interface(p, nj, nk, ld, false, 0.0, static_cast<cudaStream_t>(stream)));
}

int p3x_postamble(const p3x_interface_fields* f, const p3x_prognostic_state* prog, const p3x_diagnostic_inputs* din,
                  const p3x_diagnostic_outputs* dout, int32_t nj, int32_t nk, const p3x_layout* layout, double dt,
                  void* stream) {
  if (nj < 0 || nk <= 0 || !(dt > 0)) return P3X_EINVAL;
  p3x::InterfacePtrs p;
  const int st = interface_ptrs(f, prog, din, dout, true, p);
  if (st) return st;
  const int64_t ld = (layout && layout->ld > 0) ? layout->ld : nk;
  if (ld < nk) return P3X_EINVAL;
  return cuda_status(p3x::launch_interface(p, nj, nk, ld, true, dt, static_cast<cudaStream_t>(stream)));
}

/* EAM driver (micro_p3_tend): pointer checks and the kernels' view. */
static int eam_ptrs(const p3x_eam_fields* e, const p3x_prognostic_state* prog, const p3x_diagnostic_inputs* din,
                    const p3x_diagnostic_outputs* dout, const p3x_history_only* hist, bool post,
                    p3x::EamPtrs& p) {
  if (!e || !prog || !din) return P3X_EINVAL;
  if (!e->pmid || !e->pmiddry || !e->pdel || !e->pdeldry || !e->zi || !e->t || !e->ast || !e->npccn ||
      !e->ni_activated || !e->relvar || !e->t_prev || !e->qv_prev)
    return P3X_EINVAL;
  if (e->precip_frac_method != P3X_PRECIP_FRAC_MAX_OVERLAP && e->precip_frac_method != P3X_PRECIP_FRAC_IN_CLOUD)
    return P3X_EINVAL;
  p = p3x::EamPtrs{};
  p.pmid = e->pmid; p.pmiddry = e->pmiddry; p.pdel = e->pdel; p.pdeldry = e->pdeldry; p.zi = e->zi; p.t = e->t;
  p.ast = e->ast; p.npccn = e->npccn; p.ni_act_in = e->ni_activated; p.relvar = e->relvar; p.cmeliq = e->cmeliq;
  p.t_prev = e->t_prev; p.qv_prev = e->qv_prev;
  p.subgrid = e->subgrid_clouds != 0;
  p.method = e->precip_frac_method;
  /* the driver's constituents and the P3 state that holds each of them */
  double* w[9] = {prog->qv, prog->qc, prog->nc, prog->qr, prog->nr, prog->qi, prog->ni, prog->qm, prog->bm};
  for (int s = 0; s < 9; ++s) {
    if (!e->q[s] || !w[s]) return P3X_EINVAL;
    p.q[s] = e->q[s];
    p.w[s] = w[s];
  }
  p.th = prog->th;
  p.inv_exner = const_cast<double*>(din->inv_exner);
  p.cld_l = const_cast<double*>(din->cld_frac_l);
  p.cld_i = const_cast<double*>(din->cld_frac_i);
  p.cld_r = const_cast<double*>(din->cld_frac_r);
  if (!p.th || !p.inv_exner || !p.cld_l || !p.cld_i || !p.cld_r) return P3X_EINVAL;
  if (!post) {
    p.pres = const_cast<double*>(din->pres);
    p.dz = const_cast<double*>(din->dz);
    p.dpres = const_cast<double*>(din->dpres);
    p.nc_nuceat = const_cast<double*>(din->nc_nuceat_tend);
    p.ni_act = const_cast<double*>(din->ni_activated);
    p.inv_relvar = const_cast<double*>(din->inv_qc_relvar);
    p.qv_prev_dry = const_cast<double*>(din->qv_prev);
    p.t_prev_p3 = const_cast<double*>(din->t_prev);
    if (!p.pres || !p.dz || !p.dpres || !p.nc_nuceat || !p.ni_act || !p.inv_relvar || !p.qv_prev_dry ||
        !p.t_prev_p3)
      return P3X_EINVAL;
    return P3X_OK;
  }
  if (!dout || !hist || !e->cmeliq || !e->ptend_s || !hist->vap_liq_exchange) return P3X_EINVAL;
  for (int s = 0; s < 9; ++s) {
    if (!e->ptend_q[s]) return P3X_EINVAL;
    p.ptend_q[s] = e->ptend_q[s];
  }
  p.ptend_s = e->ptend_s;
  p.eff_qc = dout->diag_eff_radius_qc; p.eff_qi = dout->diag_eff_radius_qi; p.eff_qr = dout->diag_eff_radius_qr;
  p.liq_surf = dout->precip_liq_surf; p.ice_surf = dout->precip_ice_surf;
  p.liq_flux = dout->precip_liq_flux; p.ice_flux = dout->precip_ice_flux; p.depos = dout->qv2qi_depos_tend;
  if (!p.eff_qc || !p.eff_qi || !p.eff_qr || !p.liq_surf || !p.ice_surf || !p.liq_flux || !p.ice_flux || !p.depos)
    return P3X_EINVAL;
  p.vap_liq = hist->vap_liq_exchange;
  p.qme = e->qme; p.rho = e->rho; p.icimrst = e->icimrst; p.icwmrst = e->icwmrst; p.icinc = e->icinc;
  p.icwnc = e->icwnc; p.rel = e->rel; p.rei = e->rei; p.dei = e->dei; p.mu = e->mu; p.lambdac = e->lambdac;
  p.nfice = e->nfice; p.efcout = e->efcout; p.ncout = e->ncout; p.freql = e->freql; p.efiout = e->efiout;
  p.niout = e->niout; p.freqi = e->freqi; p.aqrain = e->aqrain; p.anrain = e->anrain; p.freqr = e->freqr;
  p.reff_rain = e->reff_rain; p.deff_rain = e->deff_rain; p.flxprc = e->flxprc; p.flxsnw = e->flxsnw;
  p.prec_pcw = e->prec_pcw; p.snow_pcw = e->snow_pcw; p.prec_str = e->prec_str; p.snow_str = e->snow_str;
  p.cdnumc = e->cdnumc;
  return P3X_OK;
}

static int eam_layout(const p3x_layout* layout, int32_t nk, int64_t& ld, int64_t& ld_int) {
  ld = (layout && layout->ld > 0) ? layout->ld : nk;
  ld_int = (layout && layout->ld_int > 0) ? layout->ld_int : int64_t(nk) + 1;
  return (ld < nk || ld_int < int64_t(nk) + 1) ? P3X_EINVAL : P3X_OK;
}

int p3x_eam_tend_pre(const p3x_eam_fields* e, const p3x_prognostic_state* prog, const p3x_diagnostic_inputs* din,
                     int32_t nj, int32_t nk, const p3x_layout* layout, void* stream) {
  if (nj < 0 || nk <= 0) return P3X_EINVAL;
  p3x::EamPtrs p;
  int st = eam_ptrs(e, prog, din, nullptr, nullptr, false, p);
  if (st) return st;
  int64_t ld, ld_int;
  if ((st = eam_layout(layout, nk, ld, ld_int))) return st;
  return cuda_status(p3x::launch_eam(p, nj, nk, ld, ld_int, false, 0.0, static_cast<cudaStream_t>(stream)));
}

int p3x_eam_tend_post(const p3x_eam_fields* e, const p3x_prognostic_state* prog, const p3x_diagnostic_inputs* din,
                      const p3x_diagnostic_outputs* dout, const p3x_history_only* hist, int32_t nj, int32_t nk,
                      const p3x_layout* layout, double dt, void* stream) {
  if (nj < 0 || nk <= 0 || !(dt > 0)) return P3X_EINVAL;
  p3x::EamPtrs p;
  int st = eam_ptrs(e, prog, din, dout, hist, true, p);
  if (st) return st;
  int64_t ld, ld_int;
  if ((st = eam_layout(layout, nk, ld, ld_int))) return st;
  return cuda_status(p3x::launch_eam(p, nj, nk, ld, ld_int, true, dt, static_cast<cudaStream_t>(stream)));
}

int p3x_eam_micro_p3_tend(p3x_context* ctx, const p3x_runtime* rt, const p3x_eam_fields* e,
                          const p3x_prognostic_state* prog, const p3x_diagnostic_inputs* din,
                          const p3x_diagnostic_outputs* dout, const p3x_infrastructure* infra,
                          const p3x_history_only* hist, int32_t nj, int32_t nk, const p3x_layout* layout,
                          int32_t precision, void* stream) {
  if (!ctx || !rt || !infra || !valid_runtime(*rt)) return P3X_EINVAL;
  /* Everything is checked before anything is launched: the preparation
   * rewrites the state in place (wet to dry), so a call that failed after it
   * would return with the state half converted. */
  p3x::EamPtrs p;
  int st = eam_ptrs(e, prog, din, dout, hist, false, p);
  if (!st) st = eam_ptrs(e, prog, din, dout, hist, true, p);
  if (st) return st;
  {
    /* the step's arguments: sizes, dt, layout, precision, pointers */
    dev::Inst in;
    if ((st = fill_inst(prog, din, dout, hist, layout, nj, nk, infra->dt, infra->predictNc, infra->prescribedCCN,
                        precision, in)))
      return st;
  }
  if ((st = p3x_eam_tend_pre(e, prog, din, nj, nk, layout, stream))) return st;
  if ((st = p3x_main_async(ctx, rt, prog, din, dout, infra, hist, nj, nk, layout, precision, stream))) return st;
  return p3x_eam_tend_post(e, prog, din, dout, hist, nj, nk, layout, infra->dt, stream);
}

/* ------------------------------------------------------------------ */
/* workload / budgets                                                  */
/* ------------------------------------------------------------------ */
int p3x_workload_generate(int32_t kind, uint64_t seed, int32_t col0, int32_t ncol, int32_t nlev,
                          double* const* fields, int64_t ld) {
  return workload_generate(kind, seed, col0, ncol, nlev, fields, ld);
}

static int cons_ptrs(const p3x_conservation_fields* f, p3x::ConsPtrs& p) {
  if (!f || !f->pseudo_density || !f->T_mid || !f->qv || !f->qc || !f->qi || !f->qr) return P3X_EINVAL;
  p = p3x::ConsPtrs{};
  p.pd = f->pseudo_density; p.T = f->T_mid; p.qv = f->qv; p.qc = f->qc; p.qi = f->qi; p.qr = f->qr;
  p.winds = f->horiz_winds; p.ps = f->ps; p.phis = f->phis;
  p.vapor_flux = f->vapor_flux; p.water_flux = f->water_flux; p.ice_flux = f->ice_flux; p.heat_flux = f->heat_flux;
  return P3X_OK;
}

int p3x_column_mass_energy(const p3x_conservation_fields* f, int32_t ncol, int32_t nlev, int64_t ld, double* mass,
                           double* energy, void* stream) {
  if (ncol < 0 || nlev <= 0 || (!mass && !energy)) return P3X_EINVAL;
  if (ld <= 0) ld = nlev;
  if (ld < nlev) return P3X_EINVAL;
  p3x::ConsPtrs p;
  const int st = cons_ptrs(f, p);
  if (st) return st;
  p.mass = mass;
  p.energy = energy;
  return cuda_status(p3x::launch_conservation(p, ncol, nlev, ld, 0.0, nullptr, static_cast<cudaStream_t>(stream)));
}

int p3x_conservation_check(p3x_context* ctx, const p3x_conservation_fields* f, const double* mass_before,
                           const double* energy_before, int32_t ncol, int32_t nlev, int64_t ld, double dt,
                           double mass_tol, double energy_tol, double* mass_err, double* energy_err,
                           p3x_conservation_report* out, void* stream) {
  if (!ctx || !mass_before || !energy_before || !mass_err || !energy_err || !out || ncol <= 0 || nlev <= 0 ||
      !(dt > 0))
    return P3X_EINVAL;
  if (ld <= 0) ld = nlev;
  if (ld < nlev) return P3X_EINVAL;
  p3x::ConsPtrs p;
  const int st = cons_ptrs(f, p);
  if (st) return st;
  p.mass_before = mass_before;
  p.energy_before = energy_before;
  p.mass_err = mass_err;
  p.energy_err = energy_err;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  P3X_CUDA(p3x::launch_conservation(p, ncol, nlev, ld, dt, ctx->d_maxloc, s));
  double h[4];
  P3X_CUDA(cudaMemcpyAsync(h, ctx->d_maxloc, sizeof(h), cudaMemcpyDeviceToHost, s));
  P3X_CUDA(cudaStreamSynchronize(s));
  out->max_mass_err = h[0];
  out->mass_col = int32_t(h[1]);
  out->max_energy_err = h[2];
  out->energy_col = int32_t(h[3]);
  out->pass = (h[0] < mass_tol && h[2] < energy_tol) ? 1 : 0;
  out->pad_ = 0;
  return P3X_OK;
}

int p3x_column_budgets(const p3x_prognostic_state* prog, const double* dpres, const double* inv_exner,
                       int32_t ncol, int32_t nlev, int64_t ld, double* water_out, double* energy_out,
                       void* stream) {
  if (!prog || !dpres || !inv_exner || ncol < 0 || nlev <= 0) return P3X_EINVAL;
  if (ld <= 0) ld = nlev;
  return cuda_status(launch_budgets(prog->qv, prog->qc, prog->qr, prog->qi, prog->th, dpres, inv_exner, ncol,
                                    nlev, ld, water_out, energy_out, static_cast<cudaStream_t>(stream)));
}

}  // extern "C"

/* ------------------------------------------------------------------ */
/* batched form                                                        */
/* ------------------------------------------------------------------ */
struct p3x_batch {
  p3x_context* ctx = nullptr;
  dev::RuntimeDev rtd{};
  dev::Inst* insts_d = nullptr;
  void* scratch = nullptr; /* every instance's K1->K2/K3 scratch */
  uint32_t* ctr_d = nullptr; /* work counters, kWorkCounters per group */
  struct Group {
    int precision = 0;
    dev::WorkItem* work_d = nullptr;
    int nwork = 0;
    int nlev_max = 0;
    LaunchSpec ls{32, 8, 1, 0};
  } groups[2];
  int ngroups = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

namespace p3x {
namespace {
template <class TR>
int launch_work_t(p3x_context* ctx, const dev::RuntimeDev& rtd, const LaunchSpec& ls0, const dev::Inst* insts_d,
                  const dev::WorkItem* work_d, int nwork, int nlev_max, uint32_t* wctr, cudaStream_t st,
                  double grid_frac = 1.0) {
  if (nwork == 0) return P3X_OK;
  const int stride = sm_stride_for(nlev_max);
  const int prec = sizeof(TR) == sizeof(double) ? P3X_FP64 : P3X_FP32_BULK;
  LaunchSpec ls = fit_spec(prec, ls0, stride);
  ls.grid_frac = grid_frac;
  if (!spec_fits(prec, ls, stride)) return P3X_EINVAL;
  dev::KParams<TR> kp = make_kparams<TR>(ctx, rtd);
  kp.sm_stride = stride;
  kp.nwork = nwork;
  kp.work = work_d;
  kp.insts = insts_d;
  kp.wctr = wctr;
  dev::Inst dummy{};
  return cuda_status(launch_p3<TR>(dummy, kp, ls, ctx->num_sms, st));
}

int batch_launch(p3x_batch* b, cudaStream_t st) {
  for (int g = 0; g < b->ngroups; ++g) {
    auto& G = b->groups[g];
    uint32_t* ctr = b->ctr_d + size_t(g) * dev::kWorkCounters;
    const int rc =
        G.precision == P3X_FP32_BULK
            ? launch_work_t<float>(b->ctx, b->rtd, G.ls, b->insts_d, G.work_d, G.nwork, G.nlev_max, ctr, st)
            : launch_work_t<double>(b->ctx, b->rtd, G.ls, b->insts_d, G.work_d, G.nwork, G.nlev_max, ctr, st);
    if (rc) return rc;
  }
  return P3X_OK;
}
void drop_graph(p3x_batch* b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->exec = nullptr;
  b->graph = nullptr;
}
}  // namespace

int launch_work(p3x_context* ctx, const p3x_runtime& rt, int precision, const dev::Inst* insts_d,
                const dev::WorkItem* work_d, int nwork, int nlev_max, uint32_t* wctr, cudaStream_t st,
                double grid_frac) {
  if (!ctx || (precision != P3X_FP64 && precision != P3X_FP32_BULK)) return P3X_EINVAL;
  const dev::RuntimeDev rtd = make_runtime(rt);
  const LaunchSpec ls = spec_of(ctx->cfg[precision]);
  return precision == P3X_FP32_BULK
             ? launch_work_t<float>(ctx, rtd, ls, insts_d, work_d, nwork, nlev_max, wctr, st, grid_frac)
             : launch_work_t<double>(ctx, rtd, ls, insts_d, work_d, nwork, nlev_max, wctr, st, grid_frac);
}

}  // namespace p3x

extern "C" {

int p3x_batch_create(p3x_context* ctx, const p3x_runtime* rt, const p3x_instance_desc* descs, int32_t n,
                     p3x_batch** out) {
  if (!ctx || !rt || !descs || n <= 0 || !out || !valid_runtime(*rt)) return P3X_EINVAL;
  *out = nullptr;
  std::vector<dev::Inst> insts(n);
  for (int i = 0; i < n; ++i) {
    const p3x_instance_desc& d = descs[i];
    const int st = fill_inst(&d.prog, &d.din, &d.dout, &d.hist, &d.layout, d.ncol, d.nlev, d.dt, d.predictNc,
                             d.prescribedCCN, d.precision, insts[i]);
    if (st) return st;
  }
  auto b = std::make_unique<p3x_batch>();
  b->ctx = ctx;
  b->rtd = make_runtime(*rt);
  size_t scr_total = 0;
  for (int i = 0; i < n; ++i) scr_total += dev::scratch_bytes(insts[i].ncol, insts[i].ld);
  if (scr_total) P3X_CUDA(cudaMalloc(&b->scratch, scr_total));
  P3X_CUDA(cudaMalloc(&b->ctr_d, 2 * dev::kWorkCounters * sizeof(uint32_t)));
  {
    size_t off = 0;
    for (int i = 0; i < n; ++i) {
      bind_scratch(insts[i], static_cast<unsigned char*>(b->scratch) + off);
      off += dev::scratch_bytes(insts[i].ncol, insts[i].ld);
    }
  }
  P3X_CUDA(cudaMalloc(&b->insts_d, sizeof(dev::Inst) * n));
  P3X_CUDA(cudaMemcpy(b->insts_d, insts.data(), sizeof(dev::Inst) * n, cudaMemcpyHostToDevice));
  for (int p = 0; p < 2; ++p) {
    /* deeper columns first, then interleave instances so that neighbouring
     * work items belong to different instances */
    std::vector<int> idx;
    for (int i = 0; i < n; ++i)
      if (insts[i].precision == p) idx.push_back(i);
    if (idx.empty()) continue;
    std::stable_sort(idx.begin(), idx.end(), [&](int a, int c) { return insts[a].nlev > insts[c].nlev; });
    std::vector<dev::WorkItem> work;
    int nlev_max = 0;
    for (int i : idx) {
      nlev_max = std::max(nlev_max, insts[i].nlev);
      for (int c = 0; c < insts[i].ncol; ++c) work.push_back(dev::WorkItem{i, c});
    }
    auto& G = b->groups[b->ngroups++];
    G.precision = p;
    G.nwork = int(work.size());
    G.nlev_max = nlev_max;
    G.ls = spec_of(ctx->cfg[p]);
    if (!work.empty()) {
      P3X_CUDA(cudaMalloc(&G.work_d, sizeof(dev::WorkItem) * work.size()));
      P3X_CUDA(cudaMemcpy(G.work_d, work.data(), sizeof(dev::WorkItem) * work.size(), cudaMemcpyHostToDevice));
    }
  }
  *out = b.release();
  return P3X_OK;
}

int p3x_batch_run(p3x_batch* b, void* stream) {
  if (!b) return P3X_EINVAL;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (b->exec) return cuda_status(cudaGraphLaunch(b->exec, st));
  return batch_launch(b, st);
}

int p3x_batch_capture_graph(p3x_batch* b, void* stream) {
  if (!b) return P3X_EINVAL;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (st == nullptr) return P3X_EINVAL; /* the legacy stream cannot be captured */
  drop_graph(b);
  P3X_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  const int rc = batch_launch(b, st);
  cudaGraph_t g = nullptr;
  const cudaError_t e = cudaStreamEndCapture(st, &g);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return cuda_status(e);
  b->graph = g;
  P3X_CUDA(cudaGraphInstantiate(&b->exec, g, 0));
  return P3X_OK;
}

int p3x_batch_set_launch_config(p3x_batch* b, const p3x_launch_config* cfg) {
  if (!b || !cfg) return P3X_EINVAL;
  const LaunchSpec ls = spec_of(*cfg);
  /* every group must accept the configuration before any group takes it */
  for (int g = 0; g < b->ngroups; ++g)
    if (!spec_fits(b->groups[g].precision, ls, sm_stride_for(1))) return P3X_EINVAL;
  for (int g = 0; g < b->ngroups; ++g) b->groups[g].ls = ls;
  drop_graph(b);
  return P3X_OK;
}

int p3x_batch_destroy(p3x_batch* b) {
  if (!b) return P3X_EINVAL;
  drop_graph(b);
  if (b->insts_d) cudaFree(b->insts_d);
  if (b->scratch) cudaFree(b->scratch);
  if (b->ctr_d) cudaFree(b->ctr_d);
  for (int g = 0; g < b->ngroups; ++g)
    if (b->groups[g].work_d) cudaFree(b->groups[g].work_d);
  delete b;
  return P3X_OK;
}

/* Times every candidate configuration on the batch and keeps the fastest.
 * The sweep covers threads per column (8, 16, 32 lanes, i.e. nlev/8 .. nlev/32
 * levels per thread), columns per CTA and staging of the ice / Table3 tables
 * into shared memory.  Each timed run advances the batch's instances by one
 * step. */
int p3x_autotune_batch(p3x_batch* b, void* stream, int32_t reps, p3x_launch_config* best, double* ms_best) {
  if (!b || reps <= 0) return P3X_EINVAL;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  drop_graph(b);
  const int lanes_c[] = {8, 16, 32};
  const int groups_c[] = {2, 4, 8};
  const int staged_c[] = {0, 1};
  const int bps_c[] = {0};
  p3x_launch_config best_cfg{32, 8, 1, 0};
  double best_ms = 1e300;
  cudaEvent_t e0, e1;
  P3X_CUDA(cudaEventCreate(&e0));
  P3X_CUDA(cudaEventCreate(&e1));
  for (int L : lanes_c)
    for (int G : groups_c)
      for (int S : staged_c)
        for (int B : bps_c) {
          const int groups = G * (32 / L); /* keep the CTA size in warps comparable across lane counts */
          if (groups * L > 256) continue;
          p3x_launch_config c{L, groups, S, B};
          bool ok = true;
          for (int g = 0; g < b->ngroups; ++g) {
            const LaunchSpec ls = spec_of(c);
            if (!spec_fits(b->groups[g].precision, ls, sm_stride_for(b->groups[g].nlev_max))) ok = false;
          }
          if (!ok) continue;
          for (int g = 0; g < b->ngroups; ++g) b->groups[g].ls = spec_of(c);
          if (batch_launch(b, st) != P3X_OK) continue; /* warm-up */
          cudaEventRecord(e0, st);
          int rc = P3X_OK;
          for (int r = 0; r < reps && rc == P3X_OK; ++r) rc = batch_launch(b, st);
          cudaEventRecord(e1, st);
          if (cudaEventSynchronize(e1) != cudaSuccess || rc != P3X_OK) continue;
          float ms = 0;
          cudaEventElapsedTime(&ms, e0, e1);
          const double per = double(ms) / reps;
          if (per < best_ms) {
            best_ms = per;
            best_cfg = c;
          }
        }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  for (int g = 0; g < b->ngroups; ++g) b->groups[g].ls = spec_of(best_cfg);
  if (best) *best = best_cfg;
  if (ms_best) *ms_best = best_ms;
  const int st_err = read_and_clear_err(b->ctx, st);
  return best_ms < 1e300 ? st_err : P3X_ECUDA;
}

}  // extern "C"

extern "C" int p3x_fixed_scratch_info(const p3x_context* ctx, int64_t* capacity_bytes, int32_t* reserved) {
  if (!ctx) return P3X_EINVAL;
  if (capacity_bytes) *capacity_bytes = int64_t(kFixedScratchBytes);
  if (reserved) *reserved = step_scratch_reserved(ctx->device) ? 1 : 0;
  return P3X_OK;
}

extern "C" int p3x_main_fixed_scratch(p3x_context* ctx, const p3x_runtime* rt, const p3x_prognostic_state* prog,
                                      const p3x_diagnostic_inputs* din, const p3x_diagnostic_outputs* dout,
                                      const p3x_infrastructure* infra, const p3x_history_only* hist, int32_t nj,
                                      int32_t nk, const p3x_layout* layout, int32_t precision, void* stream) {
  if (!ctx || !rt || !infra || !valid_runtime(*rt)) return P3X_EINVAL;
  dev::Inst in;
  const int st = fill_inst(prog, din, dout, hist, layout, nj, nk, infra->dt, infra->predictNc,
                           infra->prescribedCCN, precision, in);
  if (st) return st;
  if (in.ncol == 0) return P3X_OK;
  if (dev::scratch_bytes(in.ncol, in.ld) > kFixedScratchBytes) return P3X_ENOMEM;
  void* scr = nullptr;
  /* the context reserved the array on its device; a call made while another
   * device is current is rejected (P3X_EINVAL) */
  const int rc = step_scratch_address(ctx->device, &scr);
  if (rc) return rc;
  bind_scratch(in, static_cast<unsigned char*>(scr));
  return launch_kernels(ctx, rt, in, static_cast<cudaStream_t>(stream));
}
