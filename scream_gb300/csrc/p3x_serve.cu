/*
 * Serving loop of libp3x: continuous batching of P3 steps under a
 * device-memory budget.
 *
 * A request advances one resident instance (its own ncol x nlev state, FP64
 * or FP32-bulk) by one P3 step.  A single host thread runs the loop:
 *
 *   arrivals   -> per-instance FIFO of step requests (steps of one instance
 *                 run in order, one at a time);
 *   admission  -> an instance's memory (fields + hand-over scratch) is taken
 *                 from a stream-ordered pool only while the resident total
 *                 stays within the budget; admission is first come, first
 *                 served, so a large instance is not starved by small ones;
 *   dispatch   -> whenever one of `max_inflight` slots (a CUDA stream each)
 *                 is free, every ready request of one precision (up to a
 *                 column cap) is packed into one work list and stepped by
 *                 the batched kernels (part1+2, sedimentation, part3) plus
 *                 the state hand-over, in launches of at most a chunk of
 *                 column-levels (p3x_server_set_dispatch_chunk) so that other
 *                 slots' kernels reach the SMs between them; slots overlap on
 *                 the device;
 *   completion -> an event per slot, polled; latency = completion - arrival
 *                 on the host clock; a Poisson session's memory returns to
 *                 the pool after its last step; an instance created by
 *                 p3x_server_submit stays resident (readable) after its last
 *                 step until admission needs the memory (oldest first).
 *
 * If nothing is running, nothing is due and the instance at the head of the
 * admission queue still does not fit (memory held by idle instances that
 * wait for further requests), that instance is rejected instead of waiting
 * for memory that cannot come free.
 *
 * Requests carry data.  Instance workloads are column slices of synthetic
 * templates (65536 standard-atmosphere columns, RH ~ U(0.3, 1.05), per level
 * count) generated once per server into page-locked HOST memory, as a
 * client's state would be: instance `seed` starts at template column seed
 * mod (65536 - ncol + 1).  An instance's first step uploads its 23 input
 * fields from there on the dispatching slot's stream, and every step
 * downloads its result (the 10 prognostic fields and the two surface
 * precipitation rates) into the slot's page-locked result buffer before the
 * slot's completion event, so both copies lie inside the measured latency.
 * The same instance has the same data alone and in a mix; columns are
 * independent, so an instance's result does not depend on what it was
 * batched with.
 *
 * SM partition (p3x_server_set_sm_partition): the device's SMs are split
 * into two green contexts.  The last slot's stream lives in the small one and
 * takes only small instances; the other slots' streams live in the rest and
 * never take those.  A large step's persistent blocks then never hold the SMs
 * a small request needs (blocks of different kernels do not fit into each
 * other's leftovers: an SM running three FP32-bulk part1+2 blocks has no room
 * for one FP64 part1+2 block).  The green-context calls are the driver's,
 * resolved through the runtime at run time.
 *
 * Checkpoint / resume: p3x_server_export_instance copies an idle instance's
 * 23 input fields (the whole state a later step reads) to the host, and
 * p3x_server_import_instance makes a resident instance from such a copy, so
 * a run can stop after step N and continue bitwise from N+1 in another
 * server (the reference carries the same state across restarts, including
 * qv_prev / T_prev: eamxx_p3_process_interface.cpp:93-94).
 */
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <random>
#include <thread>
#include <vector>

#include <cuda.h> /* driver types of the green-context calls (resolved at run time) */

#include "p3x.h"
#include "p3x_internal.hpp"
#include "p3x_launch.hpp"

namespace {

using Clock = std::chrono::steady_clock;
using p3x::dev::Inst;
using p3x::dev::WorkItem;

constexpr int kTemplateCols = 65536;
constexpr uint64_t kTemplateSeed = 5000;   /* seed of the serving workload's templates */
constexpr int kMidOutputs = 10;             /* 7 per-level diagnostics + 3 history fields */
constexpr int kBatchColumnCap = 1 << 18;    /* columns per dispatched work list */
/* Latency policy (the default; p3x_server_set_latency_policy): small
 * requests must not wait behind large steps (an FP64 step of 65,536 x 128
 * takes ~130 ms alone).  A dispatch holds requests of one size kind (small:
 * at most kSmallInstanceCl column-levels); a dispatch of more than
 * kLargeDispatchCl column-levels takes the policy's share of the
 * resident-CTA capacity, so every SM keeps room for other slots' launches;
 * and the last slot (when there is more than one) takes only small
 * instances, on a stream of the highest priority, so its blocks are
 * scheduled first as blocks of the large steps retire.  The throughput
 * policy packs every ready request of a precision together on any slot at
 * full capacity. */
constexpr double kLargeDispatchCl = double(1 << 20);
/* Default dispatch chunk (p3x_server_set_dispatch_chunk): measured at 80 %
 * load, chunks of 2^18 column-levels cut the slowdown p99 from 33-37 to 5
 * (2^19: 8-14, 2^20: 17-20, 2^21: 28-33) at unchanged saturated throughput. */
constexpr int64_t kDispatchChunkCl = int64_t(1) << 18;
constexpr double kLargeGridShare = 0.875;
constexpr int64_t kSmallInstanceCl = int64_t(1) << 19;

size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

struct Instance {
  int64_t id = 0;
  int32_t ncol = 0, nlev = 0, precision = 0, total_steps = 1, done = 0;
  double dt = 300.0;
  uint64_t seed = 0;
  size_t bytes = 0;
  void* mem = nullptr;
  bool admitted = false, busy = false, closed_loop = false;
  double retired_at = -1; /* explicit instance after its last step: evictable */
  std::deque<double> arrivals; /* arrival times of queued steps */
  Inst in{};
};

struct Slot {
  cudaStream_t st = nullptr;      /* the stream in use: st_full, or st_part under an SM partition */
  cudaStream_t st_full = nullptr; /* on the whole device */
  cudaStream_t st_part = nullptr; /* in the slot's green context */
  cudaEvent_t ev = nullptr;
  bool busy = false;
  std::vector<int64_t> ids;     /* instances stepped by this dispatch */
  std::vector<double> arrivals; /* their requests' arrival times */
  Inst* h_insts = nullptr;
  WorkItem* h_work = nullptr;
  Inst* d_insts = nullptr;
  WorkItem* d_work = nullptr;
  int cap_insts = 0, cap_work = 0;
  double* h_out = nullptr; /* page-locked results of the dispatch's requests */
  size_t cap_out = 0;      /* doubles */
};

/* One completed request: latency and size (for per-class statistics). */
struct LatRec {
  double ms;
  int32_t ncol, nlev, precision;
  int32_t first; /* the instance's first step (it uploads the state) */
};

/* Calibration grid of isolated service times. */
constexpr int kCalNcol[] = {1, 8, 64, 512, 4096, 32768, 65536};
constexpr int kCalPoints = int(sizeof(kCalNcol) / sizeof(kCalNcol[0]));
constexpr int kSizeClasses = 5; /* ncol in [1,10), [10,100), [100,1000), [1000,10000), [10000, 65536] */
constexpr int kResultFields = 10; /* prognostic fields downloaded per request, plus two surface rates */

}  // namespace

struct p3x_server {
  p3x_context* ctx = nullptr;
  p3x_runtime rt{};
  int64_t budget = 0;
  int64_t resident = 0, peak_resident = 0;
  int32_t peak_inflight = 0;
  cudaMemPool_t pool = nullptr;
  /* page-locked host templates, nlev 72, 128: [P3X_NUM_INPUTS][65536][nlev] */
  double* tmpl[2] = {nullptr, nullptr};
  std::vector<Slot> slots;
  std::map<int64_t, Instance> inst;
  std::deque<int64_t> admit_fifo;                 /* instances waiting for memory */
  std::multimap<double, int64_t> future;          /* arrivals not yet due: time -> instance */
  Clock::time_point t0;
  std::vector<LatRec> lat;
  int64_t completed = 0, rejected = 0;
  double cl_done = 0;
  double first_arrival = -1, last_done = 0;
  int64_t h2d_bytes = 0, d2h_bytes = 0;
  /* isolated service time (ms) [first step / later step][precision][nlev 72/128][kCalNcol] */
  double iso_ms[2][2][2][kCalPoints] = {};
  bool calibrated = false;
  bool latency_policy = true;
  double large_share = kLargeGridShare;
  /* SM partition: green contexts {small, rest}, their SM counts, the largest
   * instance (column-levels) the small one takes */
  int num_sms = 0;
  bool part = false;
  CUgreenCtx gctx[2] = {nullptr, nullptr};
  int part_sms[2] = {0, 0};
  int64_t part_small_cl = 0;
  /* a dispatch larger than this many column-levels runs as consecutive
   * launches of at most this size (0: one launch) */
  int64_t chunk_cl = kDispatchChunkCl;
};

namespace {

int cuda_rc(cudaError_t e) {
  if (e == cudaSuccess) return P3X_OK;
  return e == cudaErrorMemoryAllocation ? P3X_ENOMEM : P3X_ECUDA;
}
#define SRV_CUDA(x)                                 \
  do {                                              \
    const cudaError_t e_ = (x);                     \
    if (e_ != cudaSuccess) return cuda_rc(e_);      \
  } while (0)

double now_s(const p3x_server* s) { return std::chrono::duration<double>(Clock::now() - s->t0).count(); }

/* The driver's green-context calls, looked up through the runtime so that the
 * library does not link the driver library. */
struct GreenApi {
  CUresult (*device_get)(CUdevice*, int) = nullptr;
  CUresult (*get_resource)(CUdevice, CUdevResource*, CUdevResourceType) = nullptr;
  CUresult (*split)(CUdevResource*, unsigned int*, const CUdevResource*, CUdevResource*, unsigned int,
                    unsigned int) = nullptr;
  CUresult (*make_desc)(CUdevResourceDesc*, CUdevResource*, unsigned int) = nullptr;
  CUresult (*create)(CUgreenCtx*, CUdevResourceDesc, CUdevice, unsigned int) = nullptr;
  CUresult (*destroy)(CUgreenCtx) = nullptr;
  CUresult (*stream_create)(CUstream*, CUgreenCtx, unsigned int, int) = nullptr;
  bool ok = false;
};

template <class F>
bool driver_entry(const char* name, F& fn) {
  void* p = nullptr;
  cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
  if (cudaGetDriverEntryPointByVersion(name, &p, CUDA_VERSION, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess || !p)
    return false;
  fn = reinterpret_cast<F>(p);
  return true;
}

const GreenApi& green_api() {
  static const GreenApi api = [] {
    GreenApi g;
    g.ok = driver_entry("cuDeviceGet", g.device_get) && driver_entry("cuDeviceGetDevResource", g.get_resource) &&
           driver_entry("cuDevSmResourceSplitByCount", g.split) &&
           driver_entry("cuDevResourceGenerateDesc", g.make_desc) && driver_entry("cuGreenCtxCreate", g.create) &&
           driver_entry("cuGreenCtxDestroy", g.destroy) && driver_entry("cuGreenCtxStreamCreate", g.stream_create);
    return g;
  }();
  return api;
}

/* Removes the SM partition: every slot back on its whole-device stream.
 * The caller has drained the server. */
void drop_partition(p3x_server* s) {
  for (auto& sl : s->slots) {
    sl.st = sl.st_full;
    if (sl.st_part) cudaStreamDestroy(sl.st_part);
    sl.st_part = nullptr;
  }
  for (CUgreenCtx& g : s->gctx) {
    if (g && green_api().ok) green_api().destroy(g);
    g = nullptr;
  }
  s->part = false;
  s->part_sms[0] = s->part_sms[1] = 0;
}

/* Splits the device into a green context of at least small_sms SMs for the
 * last slot and one of the remaining SMs for the others. */
int make_partition(p3x_server* s, int small_sms) {
  const GreenApi& g = green_api();
  if (!g.ok) return P3X_ECUDA;
  int ord = 0;
  SRV_CUDA(cudaGetDevice(&ord));
  CUdevice dev;
  if (g.device_get(&dev, ord) != CUDA_SUCCESS) return P3X_ECUDA;
  CUdevResource all{}, small{}, rest{};
  if (g.get_resource(dev, &all, CU_DEV_RESOURCE_TYPE_SM) != CUDA_SUCCESS) return P3X_ECUDA;
  unsigned int groups = 1;
  if (g.split(&small, &groups, &all, &rest, 0, unsigned(small_sms)) != CUDA_SUCCESS || groups != 1 ||
      small.sm.smCount == 0 || rest.sm.smCount == 0)
    return P3X_EINVAL;
  CUdevResourceDesc desc[2];
  if (g.make_desc(&desc[0], &small, 1) != CUDA_SUCCESS || g.make_desc(&desc[1], &rest, 1) != CUDA_SUCCESS)
    return P3X_ECUDA;
  for (int i = 0; i < 2; ++i)
    if (g.create(&s->gctx[i], desc[i], dev, CU_GREEN_CTX_DEFAULT_STREAM) != CUDA_SUCCESS) return P3X_ECUDA;
  s->part_sms[0] = int(small.sm.smCount);
  s->part_sms[1] = int(rest.sm.smCount);
  int prio_least = 0, prio_greatest = 0;
  SRV_CUDA(cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest));
  for (auto& sl : s->slots) {
    const bool last = &sl == &s->slots.back();
    CUstream cs = nullptr;
    if (g.stream_create(&cs, s->gctx[last ? 0 : 1], CU_STREAM_NON_BLOCKING, last ? prio_greatest : prio_least) !=
        CUDA_SUCCESS)
      return P3X_ECUDA;
    sl.st_part = static_cast<cudaStream_t>(cs);
  }
  for (auto& sl : s->slots) sl.st = sl.st_part;
  s->part = true;
  return P3X_OK;
}

size_t instance_bytes(int ncol, int nlev) {
  const size_t mid = align256(size_t(ncol) * nlev * sizeof(double));
  const size_t itf = align256(size_t(ncol) * (nlev + 1) * sizeof(double));
  const size_t srf = align256(size_t(ncol) * sizeof(double));
  return size_t(P3X_NUM_INPUTS + kMidOutputs) * mid + 2 * itf + 2 * srf + p3x::dev::scratch_bytes(ncol, nlev);
}

/* Binds the device pointers of an instance laid out in one allocation. */
void bind_instance(Instance& I) {
  const int ncol = I.ncol, nlev = I.nlev;
  const size_t mid = align256(size_t(ncol) * nlev * sizeof(double));
  const size_t itf = align256(size_t(ncol) * (nlev + 1) * sizeof(double));
  const size_t srf = align256(size_t(ncol) * sizeof(double));
  unsigned char* p = static_cast<unsigned char*>(I.mem);
  double* f[P3X_NUM_INPUTS + kMidOutputs];
  for (int k = 0; k < P3X_NUM_INPUTS + kMidOutputs; ++k, p += mid) f[k] = reinterpret_cast<double*>(p);
  double* liq_flux = reinterpret_cast<double*>(p); p += itf;
  double* ice_flux = reinterpret_cast<double*>(p); p += itf;
  double* liq_surf = reinterpret_cast<double*>(p); p += srf;
  double* ice_surf = reinterpret_cast<double*>(p); p += srf;
  Inst& in = I.in;
  in = Inst{};
  in.qc = f[P3X_F_QC]; in.nc = f[P3X_F_NC]; in.qr = f[P3X_F_QR]; in.nr = f[P3X_F_NR];
  in.qi = f[P3X_F_QI]; in.qm = f[P3X_F_QM]; in.ni = f[P3X_F_NI]; in.bm = f[P3X_F_BM];
  in.qv = f[P3X_F_QV]; in.th = f[P3X_F_TH];
  in.nc_nuceat_tend = f[P3X_F_NC_NUCEAT_TEND]; in.nccn = f[P3X_F_NCCN]; in.ni_activated = f[P3X_F_NI_ACTIVATED];
  in.inv_qc_relvar = f[P3X_F_INV_QC_RELVAR]; in.cld_frac_i = f[P3X_F_CLD_FRAC_I];
  in.cld_frac_l = f[P3X_F_CLD_FRAC_L]; in.cld_frac_r = f[P3X_F_CLD_FRAC_R]; in.pres = f[P3X_F_PRES];
  in.dz = f[P3X_F_DZ]; in.dpres = f[P3X_F_DPRES]; in.inv_exner = f[P3X_F_INV_EXNER];
  in.qv_prev = f[P3X_F_QV_PREV]; in.t_prev = f[P3X_F_T_PREV];
  double** o = f + P3X_NUM_INPUTS;
  in.qv2qi_depos_tend = o[0]; in.precip_total_tend = o[1]; in.nevapr = o[2];
  in.diag_eff_radius_qc = o[3]; in.diag_eff_radius_qi = o[4]; in.diag_eff_radius_qr = o[5]; in.rho_qi = o[6];
  in.liq_ice_exchange = o[7]; in.vap_liq_exchange = o[8]; in.vap_ice_exchange = o[9];
  in.precip_liq_flux = liq_flux; in.precip_ice_flux = ice_flux;
  in.precip_liq_surf = liq_surf; in.precip_ice_surf = ice_surf;
  in.scr = reinterpret_cast<double*>(p);
  in.cflag = reinterpret_cast<int32_t*>(p + size_t(p3x::dev::kScrFields) * ncol * nlev * sizeof(double));
  in.ld = nlev;
  in.ld_int = nlev + 1;
  in.ncol = ncol;
  in.nlev = nlev;
  in.dt = I.dt;
  in.predictNc = 1;
  in.prescribedCCN = 1;
  in.precision = I.precision;
}

int template_index(int nlev) { return nlev == 72 ? 0 : (nlev == 128 ? 1 : -1); }

int build_template(p3x_server* s, int which, int nlev) {
  const size_t n = size_t(kTemplateCols) * nlev;
  SRV_CUDA(cudaMallocHost(&s->tmpl[which], size_t(P3X_NUM_INPUTS) * n * sizeof(double)));
  std::vector<double*> fields(P3X_NUM_INPUTS);
  for (int f = 0; f < P3X_NUM_INPUTS; ++f) fields[f] = s->tmpl[which] + size_t(f) * n;
  return p3x::workload_generate(0, kTemplateSeed, 0, kTemplateCols, nlev, fields.data(), nlev);
}

/* The 23 input fields of an instance, in P3X_F_* order (device pointers). */
void input_fields(const Instance& I, double* dst[P3X_NUM_INPUTS]) {
  double* d[P3X_NUM_INPUTS] = {I.in.qc, I.in.nc, I.in.qr, I.in.nr, I.in.qi, I.in.qm, I.in.ni, I.in.bm,
                               I.in.qv, I.in.th,
                               const_cast<double*>(I.in.nc_nuceat_tend), const_cast<double*>(I.in.nccn),
                               const_cast<double*>(I.in.ni_activated), const_cast<double*>(I.in.inv_qc_relvar),
                               const_cast<double*>(I.in.cld_frac_i), const_cast<double*>(I.in.cld_frac_l),
                               const_cast<double*>(I.in.cld_frac_r), const_cast<double*>(I.in.pres),
                               const_cast<double*>(I.in.dz), const_cast<double*>(I.in.dpres),
                               const_cast<double*>(I.in.inv_exner), const_cast<double*>(I.in.qv_prev),
                               const_cast<double*>(I.in.t_prev)};
  for (int f = 0; f < P3X_NUM_INPUTS; ++f) dst[f] = d[f];
}

/* Takes memory for the instance and uploads its initial state (the template
 * slice in page-locked host memory) on stream st.  Host-side budget
 * accounting happened already. */
int materialise(p3x_server* s, Instance& I, cudaStream_t st) {
  SRV_CUDA(cudaMallocFromPoolAsync(&I.mem, I.bytes, s->pool, st));
  bind_instance(I);
  const int w = template_index(I.nlev);
  const int64_t c0 = int64_t(I.seed % uint64_t(kTemplateCols - I.ncol + 1));
  const size_t n = size_t(kTemplateCols) * I.nlev;
  double* dst[P3X_NUM_INPUTS];
  input_fields(I, dst);
  const size_t bytes = size_t(I.ncol) * I.nlev * sizeof(double);
  for (int f = 0; f < P3X_NUM_INPUTS; ++f) {
    const double* src = s->tmpl[w] + size_t(f) * n + size_t(c0) * I.nlev;
    SRV_CUDA(cudaMemcpyAsync(dst[f], src, bytes, cudaMemcpyHostToDevice, st));
  }
  s->h2d_bytes += int64_t(P3X_NUM_INPUTS) * int64_t(bytes);
  return P3X_OK;
}

/* Doubles of one request's downloaded result. */
size_t result_doubles(const Instance& I) { return size_t(I.ncol) * (size_t(kResultFields) * I.nlev + 2); }

int ensure_capacity(Slot& sl, int ninst, int nwork, size_t nout) {
  if (nout > sl.cap_out) {
    if (sl.h_out) cudaFreeHost(sl.h_out);
    sl.h_out = nullptr;
    const size_t cap = std::max(nout, 2 * sl.cap_out);
    SRV_CUDA(cudaMallocHost(&sl.h_out, cap * sizeof(double)));
    sl.cap_out = cap;
  }
  if (ninst > sl.cap_insts) {
    if (sl.h_insts) cudaFreeHost(sl.h_insts);
    if (sl.d_insts) cudaFree(sl.d_insts);
    const int cap = std::max(ninst, 2 * sl.cap_insts);
    SRV_CUDA(cudaMallocHost(&sl.h_insts, sizeof(Inst) * cap));
    SRV_CUDA(cudaMalloc(&sl.d_insts, sizeof(Inst) * cap));
    sl.cap_insts = cap;
  }
  if (nwork > sl.cap_work) {
    if (sl.h_work) cudaFreeHost(sl.h_work);
    if (sl.d_work) cudaFree(sl.d_work);
    const int cap = std::max(nwork, 2 * sl.cap_work);
    SRV_CUDA(cudaMallocHost(&sl.h_work, sizeof(WorkItem) * cap));
    SRV_CUDA(cudaMalloc(&sl.d_work, sizeof(WorkItem) * cap));
    sl.cap_work = cap;
  }
  return P3X_OK;
}

/* Moves due arrivals into their instances' queues. */
void take_arrivals(p3x_server* s, double t) {
  while (!s->future.empty() && s->future.begin()->first <= t) {
    const double at = s->future.begin()->first;
    const int64_t id = s->future.begin()->second;
    s->future.erase(s->future.begin());
    Instance& I = s->inst.at(id);
    I.arrivals.push_back(at);
    if (s->first_arrival < 0 || at < s->first_arrival) s->first_arrival = at;
  }
}

/* Frees retired explicit instances, oldest first, until `need` more bytes
 * fit in the budget.  Returns whether they fit. */
bool evict_for(p3x_server* s, int64_t need) {
  while (s->resident + need > s->budget) {
    int64_t victim = -1;
    double oldest = 1e300;
    for (auto& kv : s->inst) {
      const Instance& I = kv.second;
      if (I.retired_at >= 0 && !I.busy && I.arrivals.empty() && I.mem && I.retired_at < oldest) {
        oldest = I.retired_at;
        victim = kv.first;
      }
    }
    if (victim < 0) return false;
    Instance& V = s->inst.at(victim);
    cudaFreeAsync(V.mem, s->slots[0].st);
    s->resident -= int64_t(V.bytes);
    s->inst.erase(victim);
  }
  return true;
}

/* First come, first served admission against the budget. */
void admit(p3x_server* s) {
  while (!s->admit_fifo.empty()) {
    Instance& I = s->inst.at(s->admit_fifo.front());
    if (I.arrivals.empty()) break; /* not arrived yet */
    if (!evict_for(s, int64_t(I.bytes))) break;
    s->resident += int64_t(I.bytes);
    s->peak_resident = std::max(s->peak_resident, s->resident);
    I.admitted = true;
    s->admit_fifo.pop_front();
  }
}

/* Which instances a slot takes: any; small ones only (the latency policy's
 * reserved slot); under an SM partition, those of at most part_small_cl
 * column-levels (the small partition's slot) or the others. */
enum Pick { kPickAny, kPickSmall, kPickPartSmall, kPickPartRest };

/* Packs the ready requests of the oldest ready request's precision and size
 * kind (small: at most kSmallInstanceCl column-levels) into one work list and
 * launches it on slot sl, so a small request never rides a large step; pick
 * limits the instances considered. */
int dispatch(p3x_server* s, Slot& sl, Pick pick) {
  const bool by_kind = s->latency_policy;
  auto is_small = [by_kind](const Instance& I) {
    return !by_kind || int64_t(I.ncol) * I.nlev <= kSmallInstanceCl;
  };
  auto picked = [&](const Instance& I) {
    const bool part_small = int64_t(I.ncol) * I.nlev <= s->part_small_cl;
    switch (pick) {
      case kPickSmall: return is_small(I);
      case kPickPartSmall: return part_small;
      case kPickPartRest: return !part_small;
      default: return true;
    }
  };
  auto ready_now = [&](const Instance& I) {
    return I.admitted && !I.busy && !I.arrivals.empty() && picked(I);
  };
  int prec = -1;
  bool small = true;
  double oldest = 1e300;
  for (auto& kv : s->inst) {
    const Instance& I = kv.second;
    if (ready_now(I) && I.arrivals.front() < oldest) {
      oldest = I.arrivals.front();
      prec = I.precision;
      small = is_small(I);
    }
  }
  auto eligible = [&](const Instance& I) { return ready_now(I) && is_small(I) == small; };
  if (prec < 0) return 1; /* nothing ready */
  std::vector<Instance*> take;
  int cols = 0, nlev_max = 1;
  /* oldest first */
  std::vector<std::pair<double, Instance*>> ready;
  for (auto& kv : s->inst) {
    Instance& I = kv.second;
    if (eligible(I) && I.precision == prec) ready.push_back({I.arrivals.front(), &I});
  }
  std::sort(ready.begin(), ready.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
  size_t nout = 0;
  double cl = 0;
  for (auto& r : ready) {
    if (!take.empty() && cols + r.second->ncol > kBatchColumnCap) break;
    take.push_back(r.second);
    cols += r.second->ncol;
    cl += double(r.second->ncol) * r.second->nlev;
    nlev_max = std::max(nlev_max, r.second->nlev);
    nout += result_doubles(*r.second);
  }
  int rc = ensure_capacity(sl, int(take.size()), cols, nout);
  if (rc) return rc;
  sl.ids.clear();
  sl.arrivals.clear();
  int w = 0;
  for (size_t i = 0; i < take.size(); ++i) {
    Instance& I = *take[i];
    if (!I.mem) {
      rc = materialise(s, I, sl.st);
      if (rc) return rc;
    }
    sl.h_insts[i] = I.in;
    for (int c = 0; c < I.ncol; ++c) sl.h_work[w++] = WorkItem{int32_t(i), c};
    sl.ids.push_back(I.id);
    sl.arrivals.push_back(I.arrivals.front());
    I.arrivals.pop_front();
    I.busy = true;
  }
  SRV_CUDA(cudaMemcpyAsync(sl.d_insts, sl.h_insts, sizeof(Inst) * take.size(), cudaMemcpyHostToDevice, sl.st));
  SRV_CUDA(cudaMemcpyAsync(sl.d_work, sl.h_work, sizeof(WorkItem) * w, cudaMemcpyHostToDevice, sl.st));
  /* Static stride, no work counters: a launch that hands out work from a
   * counter keeps every CTA resident until its whole list is done, so the
   * other slots' launches find no free SM until then (measured at 80 % load:
   * p50 1.4 -> 1.75 ms, p90 30 -> 47 ms for 2.5 % more capacity).  With a
   * static stride CTAs retire one by one and the slots interleave. */
  /* the persistent grids: sized to the slot's SM partition, or the latency
   * policy's share of the device for a large dispatch */
  double frac = 1.0;
  if (s->part && s->num_sms > 0)
    frac = double(s->part_sms[pick == kPickPartSmall ? 0 : 1]) / double(s->num_sms);
  else if (s->latency_policy && cl > kLargeDispatchCl)
    frac = s->large_share;
  /* In chunks: every kernel of a chunk ends before the next chunk's starts,
   * so other slots' kernels, launched meanwhile, reach the SMs between them
   * instead of waiting for a whole large step.  Columns are independent, so
   * the results are those of one launch. */
  int per = w;
  if (s->chunk_cl > 0 && cl > double(s->chunk_cl))
    per = int(std::max<int64_t>(1, s->chunk_cl / std::max(1, nlev_max)));
  for (int off = 0; off < w; off += per) {
    rc = p3x::launch_work(s->ctx, s->rt, prec, sl.d_insts, sl.d_work + off, std::min(per, w - off), nlev_max,
                          nullptr, sl.st, frac);
    if (rc) return rc;
  }
  SRV_CUDA(p3x::launch_postamble(sl.d_insts, sl.d_work, w, sl.st));
  /* each request's result to the host, before the completion event */
  double* out = sl.h_out;
  for (Instance* Ip : take) {
    const Instance& I = *Ip;
    const size_t nf = size_t(I.ncol) * I.nlev;
    const double* src[kResultFields] = {I.in.qc, I.in.nc, I.in.qr, I.in.nr, I.in.qi,
                                        I.in.qm, I.in.ni, I.in.bm, I.in.qv, I.in.th};
    for (int f = 0; f < kResultFields; ++f, out += nf)
      SRV_CUDA(cudaMemcpyAsync(out, src[f], nf * sizeof(double), cudaMemcpyDeviceToHost, sl.st));
    SRV_CUDA(cudaMemcpyAsync(out, I.in.precip_liq_surf, I.ncol * sizeof(double), cudaMemcpyDeviceToHost, sl.st));
    out += I.ncol;
    SRV_CUDA(cudaMemcpyAsync(out, I.in.precip_ice_surf, I.ncol * sizeof(double), cudaMemcpyDeviceToHost, sl.st));
    out += I.ncol;
    s->d2h_bytes += int64_t(result_doubles(I) * sizeof(double));
  }
  SRV_CUDA(cudaEventRecord(sl.ev, sl.st));
  sl.busy = true;
  return P3X_OK;
}

/* Retires a finished dispatch. */
int complete(p3x_server* s, Slot& sl, double t) {
  for (size_t i = 0; i < sl.ids.size(); ++i) {
    Instance& I = s->inst.at(sl.ids[i]);
    s->lat.push_back(LatRec{(t - sl.arrivals[i]) * 1e3, I.ncol, I.nlev, I.precision, I.done == 0 ? 1 : 0});
    s->completed += 1;
    s->cl_done += double(I.ncol) * I.nlev;
    I.busy = false;
    I.done += 1;
    if (I.closed_loop && I.done >= I.total_steps) {
      SRV_CUDA(cudaFreeAsync(I.mem, sl.st));
      I.mem = nullptr;
      s->resident -= int64_t(I.bytes);
      s->inst.erase(sl.ids[i]);
    } else if (I.closed_loop) {
      s->future.insert({t, I.id}); /* the next step of a session arrives on completion */
    } else if (I.done >= I.total_steps && I.arrivals.empty()) {
      I.retired_at = t;
    }
  }
  s->last_done = t;
  sl.busy = false;
  return P3X_OK;
}

bool idle(const p3x_server* s) {
  if (!s->future.empty()) return false;
  for (const auto& sl : s->slots)
    if (sl.busy) return false;
  for (const auto& kv : s->inst)
    if (!kv.second.arrivals.empty()) return false;
  return true;
}

/* Runs the loop until every submitted (and every closed-loop follow-up)
 * request has completed. */
int run_loop(p3x_server* s) {
  double last_progress = now_s(s);
  while (!idle(s)) {
    const double t = now_s(s);
    /* watchdog: a loop that makes no progress for a minute (nothing
     * completes, dispatches or arrives) ends with P3X_ETIMEOUT */
    if (t - last_progress > 60.0 && (s->future.empty() || s->future.begin()->first < t)) return P3X_ETIMEOUT;
    take_arrivals(s, t);
    bool progressed = false;
    int inflight = 0;
    for (auto& sl : s->slots) {
      if (!sl.busy) continue;
      const cudaError_t q = cudaEventQuery(sl.ev);
      if (q == cudaSuccess) {
        const int rc = complete(s, sl, now_s(s));
        if (rc) return rc;
        progressed = true;
      } else if (q != cudaErrorNotReady) {
        return cuda_rc(q);
      } else {
        ++inflight;
      }
    }
    admit(s);
    for (auto& sl : s->slots) {
      if (sl.busy) continue;
      const bool last = s->slots.size() > 1 && &sl == &s->slots.back();
      Pick pick = kPickAny;
      if (s->part)
        pick = last ? kPickPartSmall : kPickPartRest;
      else if (s->latency_policy && last)
        pick = kPickSmall;
      const int rc = dispatch(s, sl, pick);
      if (rc == 1) continue; /* nothing ready for this slot */
      if (rc) return rc;
      ++inflight;
      progressed = true;
    }
    s->peak_inflight = std::max(s->peak_inflight, inflight);
    if (progressed) last_progress = now_s(s);
    if (!progressed && inflight == 0 && s->future.empty() && !s->admit_fifo.empty()) {
      /* nothing can free memory for the head of the admission queue */
      bool dispatchable = false;
      for (const auto& kv : s->inst) {
        const Instance& I = kv.second;
        if (I.admitted && !I.busy && !I.arrivals.empty()) dispatchable = true;
      }
      if (!dispatchable) {
        const int64_t id = s->admit_fifo.front();
        s->admit_fifo.pop_front();
        Instance& I = s->inst.at(id);
        s->rejected += int64_t(I.arrivals.size());
        s->inst.erase(id);
        continue;
      }
    }
    if (!progressed) {
      /* wait for the next arrival or completion without burning a core */
      double wait = 50e-6;
      if (!s->future.empty()) wait = std::min(wait, std::max(0.0, s->future.begin()->first - now_s(s)));
      if (wait > 0) std::this_thread::sleep_for(std::chrono::duration<double>(wait));
    }
  }
  return P3X_OK;
}

double percentile(std::vector<double> v, double q) {
  if (v.empty()) return 0;
  std::sort(v.begin(), v.end());
  const double pos = q * (v.size() - 1);
  const size_t i = size_t(pos);
  const double f = pos - double(i);
  return i + 1 < v.size() ? v[i] * (1 - f) + v[i + 1] * f : v[i];
}

int size_class(int ncol) {
  int c = 0;
  for (int lim = 10; c < kSizeClasses - 1 && ncol >= lim; lim *= 10) ++c;
  return c;
}

/* Isolated service time of a request, log-log interpolated in ncol on the
 * calibration grid of its precision and level count. */
double iso_time(const p3x_server* s, const LatRec& r) {
  const double* t = s->iso_ms[r.first ? 0 : 1][r.precision][r.nlev == 72 ? 0 : 1];
  int j = 0;
  while (j + 2 < kCalPoints && r.ncol > kCalNcol[j + 1]) ++j;
  const double x0 = std::log(double(kCalNcol[j])), x1 = std::log(double(kCalNcol[j + 1]));
  const double y0 = std::log(t[j]), y1 = std::log(t[j + 1]);
  const double w = (std::log(double(r.ncol)) - x0) / (x1 - x0);
  return std::exp(y0 + w * (y1 - y0));
}

void fill_stats(p3x_server* s, p3x_serve_stats* st, double offered) {
  if (!st) return;
  std::memset(st, 0, sizeof(*st));
  std::vector<double> ms;
  ms.reserve(s->lat.size());
  for (const LatRec& r : s->lat) ms.push_back(r.ms);
  st->completed = s->completed;
  st->rejected = s->rejected;
  st->p50_ms = percentile(ms, 0.50);
  st->p90_ms = percentile(ms, 0.90);
  st->p99_ms = percentile(ms, 0.99);
  st->max_ms = ms.empty() ? 0 : *std::max_element(ms.begin(), ms.end());
  double sum = 0;
  for (double v : ms) sum += v;
  st->mean_ms = ms.empty() ? 0 : sum / ms.size();
  st->wall_s = s->first_arrival >= 0 ? s->last_done - s->first_arrival : 0;
  st->column_levels_per_s = st->wall_s > 0 ? s->cl_done / st->wall_s : 0;
  st->offered_rate_hz = offered;
  st->peak_bytes = s->peak_resident;
  st->peak_inflight = s->peak_inflight;
  std::vector<double> cls[kSizeClasses];
  for (const LatRec& r : s->lat) cls[size_class(r.ncol)].push_back(r.ms);
  for (int c = 0; c < kSizeClasses; ++c) {
    st->class_count[c] = int64_t(cls[c].size());
    st->class_p50_ms[c] = percentile(cls[c], 0.50);
    st->class_p99_ms[c] = percentile(cls[c], 0.99);
  }
  if (s->calibrated && !s->lat.empty()) {
    std::vector<double> slow;
    slow.reserve(s->lat.size());
    for (const LatRec& r : s->lat) slow.push_back(r.ms / iso_time(s, r));
    st->slowdown_p50 = percentile(slow, 0.50);
    st->slowdown_p99 = percentile(slow, 0.99);
  }
  st->h2d_bytes = s->h2d_bytes;
  st->d2h_bytes = s->d2h_bytes;
}

void reset_stats(p3x_server* s) {
  s->lat.clear();
  s->h2d_bytes = s->d2h_bytes = 0;
  s->completed = s->rejected = 0;
  s->cl_done = 0;
  s->first_arrival = -1;
  s->last_done = 0;
  s->peak_resident = s->resident;
  s->peak_inflight = 0;
}

/* Registers a step request; creates the instance record on first use. */
int enqueue(p3x_server* s, int64_t id, int32_t ncol, int32_t nlev, int32_t precision, int32_t total_steps,
            uint64_t seed, double dt, double arrival, bool closed_loop) {
  if (ncol <= 0 || ncol > kTemplateCols || template_index(nlev) < 0 || total_steps <= 0 || !(dt > 0) ||
      (precision != P3X_FP64 && precision != P3X_FP32_BULK))
    return P3X_EINVAL;
  auto it = s->inst.find(id);
  if (it == s->inst.end()) {
    const size_t bytes = instance_bytes(ncol, nlev);
    if (int64_t(bytes) > s->budget) {
      s->rejected += 1;
      return P3X_ENOMEM;
    }
    Instance I;
    I.id = id;
    I.ncol = ncol;
    I.nlev = nlev;
    I.precision = precision;
    I.total_steps = total_steps;
    I.seed = seed;
    I.dt = dt;
    I.bytes = bytes;
    I.closed_loop = closed_loop;
    s->inst.emplace(id, std::move(I));
    s->admit_fifo.push_back(id);
  } else {
    const Instance& I = it->second;
    if (I.ncol != ncol || I.nlev != nlev || I.precision != precision) return P3X_EINVAL;
  }
  s->future.insert({arrival, id});
  return P3X_OK;
}

/* The calibration sessions (p3x_server_calibrate). */
int calibrate_runs(p3x_server* s) {
  int rc;
  const std::vector<LatRec> keep_lat = s->lat;
  const int64_t keep_done = s->completed, keep_h2d = s->h2d_bytes, keep_d2h = s->d2h_bytes;
  const double keep_cl = s->cl_done, keep_first = s->first_arrival, keep_last = s->last_done;
  int64_t id = -1;
  for (int prec = 0; prec < 2; ++prec)
    for (int l = 0; l < 2; ++l)
      for (int j = 0; j < kCalPoints; ++j) {
        const int nlev = l == 0 ? 72 : 128;
        const int64_t bytes = int64_t(instance_bytes(kCalNcol[j], nlev));
        double best[2] = {1e300, 1e300};
        if (bytes > s->budget) {
          for (int w = 0; w < 2; ++w) s->iso_ms[w][prec][l][j] = j > 0 ? s->iso_ms[w][prec][l][j - 1] : 1.0;
          continue;
        }
        /* a fresh two-step session each time, alone on the server: its first
         * step includes the state upload, as a session's first request does,
         * and its second (arriving when the first completes) does not; the
         * best of two sessions */
        for (int rep = 0; rep < 2; ++rep, --id) {
          s->lat.clear();
          rc = enqueue(s, id, kCalNcol[j], nlev, prec, 2, kTemplateSeed + uint64_t(j), 300.0, now_s(s), true);
          if (rc) return rc;
          rc = run_loop(s);
          if (rc) return rc;
          for (const LatRec& r : s->lat) best[r.first ? 0 : 1] = std::min(best[r.first ? 0 : 1], r.ms);
        }
        for (int w = 0; w < 2; ++w) s->iso_ms[w][prec][l][j] = best[w] < 1e300 ? best[w] : 1.0;
      }
  s->lat = keep_lat;
  s->completed = keep_done;
  s->h2d_bytes = keep_h2d;
  s->d2h_bytes = keep_d2h;
  s->cl_done = keep_cl;
  s->first_arrival = keep_first;
  s->last_done = keep_last;
  s->calibrated = true;
  return P3X_OK;
}

}  // namespace

extern "C" {

int p3x_server_create(p3x_context* ctx, const p3x_runtime* rt, int64_t budget_bytes, int32_t max_inflight,
                      p3x_server** out) {
  if (!out) return P3X_EINVAL;
  *out = nullptr;
  if (!ctx || !rt || budget_bytes <= 0 || max_inflight <= 0 || max_inflight > 64) return P3X_EINVAL;
  auto s = std::make_unique<p3x_server>();
  s->ctx = ctx;
  s->rt = *rt;
  s->budget = budget_bytes;
  int dev = 0;
  SRV_CUDA(cudaGetDevice(&dev));
  cudaMemPoolProps props{};
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = dev;
  SRV_CUDA(cudaMemPoolCreate(&s->pool, &props));
  uint64_t keep = UINT64_MAX;
  SRV_CUDA(cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep));
  int rc;
  if ((rc = build_template(s.get(), 0, 72)) || (rc = build_template(s.get(), 1, 128))) {
    p3x_server_destroy(s.release());
    return rc;
  }
  s->slots.resize(max_inflight);
  int prio_least = 0, prio_greatest = 0;
  SRV_CUDA(cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest));
  for (auto& sl : s->slots) {
    const bool small_slot = s->slots.size() > 1 && &sl == &s->slots.back();
    SRV_CUDA(cudaStreamCreateWithPriority(&sl.st_full, cudaStreamNonBlocking,
                                          small_slot ? prio_greatest : prio_least));
    sl.st = sl.st_full;
    SRV_CUDA(cudaEventCreateWithFlags(&sl.ev, cudaEventDisableTiming));
  }
  SRV_CUDA(cudaDeviceGetAttribute(&s->num_sms, cudaDevAttrMultiProcessorCount, dev));
  s->t0 = Clock::now();
  *out = s.release();
  return P3X_OK;
}

int p3x_server_destroy(p3x_server* s) {
  if (!s) return P3X_EINVAL;
  cudaDeviceSynchronize();
  for (auto& kv : s->inst)
    if (kv.second.mem) cudaFreeAsync(kv.second.mem, nullptr);
  cudaDeviceSynchronize();
  drop_partition(s);
  for (auto& sl : s->slots) {
    if (sl.ev) cudaEventDestroy(sl.ev);
    if (sl.st_full) cudaStreamDestroy(sl.st_full);
    if (sl.h_insts) cudaFreeHost(sl.h_insts);
    if (sl.h_work) cudaFreeHost(sl.h_work);
    if (sl.h_out) cudaFreeHost(sl.h_out);
    if (sl.d_insts) cudaFree(sl.d_insts);
    if (sl.d_work) cudaFree(sl.d_work);
  }
  for (double* t : s->tmpl)
    if (t) cudaFreeHost(t);
  if (s->pool) cudaMemPoolDestroy(s->pool);
  delete s;
  return P3X_OK;
}

int p3x_server_submit(p3x_server* s, int64_t instance_id, int32_t ncol, int32_t nlev, int32_t precision,
                      int32_t total_steps, uint64_t seed, double dt, double arrival_s) {
  if (!s) return P3X_EINVAL;
  return enqueue(s, instance_id, ncol, nlev, precision, total_steps, seed, dt, arrival_s, false);
}

int p3x_server_drain(p3x_server* s, p3x_serve_stats* stats) {
  if (!s) return P3X_EINVAL;
  const int rc = run_loop(s);
  fill_stats(s, stats, 0.0);
  return rc;
}

int p3x_server_run_poisson(p3x_server* s, double rate_hz, int32_t n_requests, int32_t max_ncol, uint64_t seed,
                           p3x_serve_stats* stats) {
  if (!s || !(rate_hz > 0) || n_requests <= 0 || max_ncol <= 0 || max_ncol > kTemplateCols) return P3X_EINVAL;
  int rc = run_loop(s); /* finish earlier work first */
  if (rc) return rc;
  reset_stats(s);
  std::mt19937_64 gen(seed);
  std::exponential_distribution<double> gap(rate_hz);
  std::uniform_real_distribution<double> u01(0.0, 1.0);
  std::uniform_int_distribution<int> steps(1, 20);
  const double start = now_s(s);
  double t = start;
  int64_t id = int64_t(1) << 40;
  for (int i = 0; i < n_requests; ++i) {
    t += gap(gen);
    const int ncol = std::max(1, std::min(max_ncol, int(std::floor(std::exp(u01(gen) * std::log(double(max_ncol) + 1.0))))));
    const int nlev = u01(gen) < 0.5 ? 72 : 128;
    const int prec = u01(gen) < 0.5 ? P3X_FP64 : P3X_FP32_BULK;
    const int nsteps = steps(gen);
    const uint64_t iseed = kTemplateSeed + uint64_t(i);
    rc = enqueue(s, id + i, ncol, nlev, prec, nsteps, iseed, 300.0, t, true);
    if (rc && rc != P3X_ENOMEM) return rc;
  }
  rc = run_loop(s);
  fill_stats(s, stats, rate_hz);
  return rc;
}

int p3x_server_set_latency_policy(p3x_server* s, int32_t on, double large_grid_share) {
  if (!s || !(large_grid_share > 0 && large_grid_share <= 1)) return P3X_EINVAL;
  const int rc = run_loop(s);
  if (rc) return rc;
  s->latency_policy = on != 0;
  s->large_share = large_grid_share;
  return P3X_OK;
}

int p3x_server_set_sm_partition(p3x_server* s, int32_t small_sms, int64_t small_max_cl, int32_t* sms_out) {
  if (!s || small_sms < 0 || (small_sms > 0 && (small_max_cl <= 0 || s->slots.size() < 2))) return P3X_EINVAL;
  if (small_sms >= s->num_sms) return P3X_EINVAL;
  int rc = run_loop(s);
  if (rc) return rc;
  SRV_CUDA(cudaDeviceSynchronize());
  drop_partition(s);
  if (small_sms > 0) {
    rc = make_partition(s, small_sms);
    if (rc) {
      drop_partition(s);
      return rc;
    }
    s->part_small_cl = small_max_cl;
  }
  if (sms_out) {
    sms_out[0] = s->part_sms[0];
    sms_out[1] = s->part_sms[1];
  }
  return P3X_OK;
}

int p3x_server_set_dispatch_chunk(p3x_server* s, int64_t max_cl) {
  if (!s || max_cl < 0) return P3X_EINVAL;
  const int rc = run_loop(s);
  if (rc) return rc;
  s->chunk_cl = max_cl;
  return P3X_OK;
}

int p3x_server_calibrate(p3x_server* s) {
  if (!s) return P3X_EINVAL;
  int rc = run_loop(s);
  if (rc) return rc;
  /* isolated times are those of one launch sequence on the whole device,
   * whatever the SM partition and dispatch chunks of the measured runs */
  const bool part = s->part;
  const int64_t chunk = s->chunk_cl;
  for (auto& sl : s->slots) sl.st = sl.st_full;
  s->part = false;
  s->chunk_cl = 0;
  rc = calibrate_runs(s);
  for (auto& sl : s->slots) sl.st = part ? sl.st_part : sl.st_full;
  s->part = part;
  s->chunk_cl = chunk;
  return rc;
}

int p3x_server_isolated_ms(p3x_server* s, int32_t precision, int32_t nlev, int32_t ncol, double* ms) {
  if (!s || !ms || !s->calibrated || (precision != P3X_FP64 && precision != P3X_FP32_BULK) ||
      template_index(nlev) < 0 || ncol < 1 || ncol > kTemplateCols)
    return P3X_EINVAL;
  *ms = iso_time(s, LatRec{0.0, ncol, nlev, precision, 0});
  return P3X_OK;
}

int p3x_server_export_instance(p3x_server* s, int64_t instance_id, double* host_state, int64_t n) {
  if (!s || !host_state) return P3X_EINVAL;
  auto it = s->inst.find(instance_id);
  if (it == s->inst.end() || !it->second.mem || it->second.busy || !it->second.arrivals.empty())
    return P3X_EINVAL;
  const Instance& I = it->second;
  const size_t nf = size_t(I.ncol) * I.nlev;
  if (n < int64_t(P3X_NUM_INPUTS * nf)) return P3X_EINVAL;
  double* src[P3X_NUM_INPUTS];
  input_fields(I, src);
  SRV_CUDA(cudaDeviceSynchronize());
  for (int f = 0; f < P3X_NUM_INPUTS; ++f)
    SRV_CUDA(cudaMemcpy(host_state + size_t(f) * nf, src[f], nf * sizeof(double), cudaMemcpyDeviceToHost));
  return P3X_OK;
}

int p3x_server_import_instance(p3x_server* s, int64_t instance_id, int32_t ncol, int32_t nlev, int32_t precision,
                               double dt, const double* host_state, int64_t n) {
  if (!s || !host_state || ncol <= 0 || ncol > kTemplateCols || template_index(nlev) < 0 || !(dt > 0) ||
      (precision != P3X_FP64 && precision != P3X_FP32_BULK))
    return P3X_EINVAL;
  const size_t nf = size_t(ncol) * nlev;
  if (n < int64_t(P3X_NUM_INPUTS * nf)) return P3X_EINVAL;
  if (s->inst.count(instance_id)) return P3X_EINVAL;
  int rc = run_loop(s);
  if (rc) return rc;
  const size_t bytes = instance_bytes(ncol, nlev);
  if (int64_t(bytes) > s->budget || !evict_for(s, int64_t(bytes))) return P3X_ENOMEM;
  Instance I;
  I.id = instance_id;
  I.ncol = ncol;
  I.nlev = nlev;
  I.precision = precision;
  I.total_steps = 0; /* evictable when idle, like an explicit instance after its last step */
  I.dt = dt;
  I.bytes = bytes;
  I.admitted = true;
  cudaStream_t st = s->slots[0].st;
  SRV_CUDA(cudaMallocFromPoolAsync(&I.mem, I.bytes, s->pool, st));
  bind_instance(I);
  double* dst[P3X_NUM_INPUTS];
  input_fields(I, dst);
  for (int f = 0; f < P3X_NUM_INPUTS; ++f)
    SRV_CUDA(cudaMemcpyAsync(dst[f], host_state + size_t(f) * nf, nf * sizeof(double), cudaMemcpyHostToDevice, st));
  SRV_CUDA(cudaStreamSynchronize(st));
  s->resident += int64_t(bytes);
  s->peak_resident = std::max(s->peak_resident, s->resident);
  I.retired_at = now_s(s);
  s->inst.emplace(instance_id, std::move(I));
  return P3X_OK;
}

int p3x_server_read_field(p3x_server* s, int64_t instance_id, int32_t field, double* host_out, int64_t n) {
  if (!s || !host_out) return P3X_EINVAL;
  auto it = s->inst.find(instance_id);
  if (it == s->inst.end() || !it->second.mem) return P3X_EINVAL;
  const Instance& I = it->second;
  const double* src;
  int64_t count;
  if (field == -1 || field == -2) {
    src = field == -1 ? I.in.precip_liq_surf : I.in.precip_ice_surf;
    count = I.ncol;
  } else if (field >= P3X_F_QC && field <= P3X_F_TH) {
    const double* f[] = {I.in.qc, I.in.nc, I.in.qr, I.in.nr, I.in.qi, I.in.qm, I.in.ni, I.in.bm, I.in.qv, I.in.th};
    src = f[field];
    count = int64_t(I.ncol) * I.nlev;
  } else {
    return P3X_EINVAL;
  }
  if (n < count) return P3X_EINVAL;
  SRV_CUDA(cudaDeviceSynchronize());
  SRV_CUDA(cudaMemcpy(host_out, src, sizeof(double) * count, cudaMemcpyDeviceToHost));
  return P3X_OK;
}

}  // extern "C"
