/*
 * Auxiliary device kernels of libp3x: layout transposes for the
 * Fortran-layout entry point, and the FP64 column water / energy budgets
 * (share/property_checks/mass_and_energy_column_conservation_check.cpp:281-347).
 */
#include "p3x_launch.hpp"

namespace p3x {

namespace {

/* src[k*ncol + i] (column fastest) -> dst[i*ld + k] (level contiguous), via a
 * 32x33 shared tile so that both sides are coalesced. */
__global__ void transpose_to_levels(const double* __restrict__ src, double* __restrict__ dst, int ncol,
                                    int nlev, int64_t ld) {
  __shared__ double tile[32][33];
  const int i0 = blockIdx.x * 32, k0 = blockIdx.y * 32;
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int k = k0 + r, i = i0 + threadIdx.x;
    if (k < nlev && i < ncol) tile[r][threadIdx.x] = src[int64_t(k) * ncol + i];
  }
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int i = i0 + r, k = k0 + threadIdx.x;
    if (k < nlev && i < ncol) dst[int64_t(i) * ld + k] = tile[threadIdx.x][r];
  }
}

__global__ void transpose_to_columns(const double* __restrict__ src, double* __restrict__ dst, int ncol,
                                     int nlev, int64_t ld) {
  __shared__ double tile[32][33];
  const int i0 = blockIdx.x * 32, k0 = blockIdx.y * 32;
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int i = i0 + r, k = k0 + threadIdx.x;
    if (k < nlev && i < ncol) tile[r][threadIdx.x] = src[int64_t(i) * ld + k];
  }
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int k = k0 + r, i = i0 + threadIdx.x;
    if (k < nlev && i < ncol) dst[int64_t(k) * ncol + i] = tile[threadIdx.x][r];
  }
}

/* One warp per column; lanes stride the levels; shuffle reduction. */
__global__ void column_budgets(const double* __restrict__ qv, const double* __restrict__ qc,
                               const double* __restrict__ qr, const double* __restrict__ qi,
                               const double* __restrict__ th, const double* __restrict__ dpres,
                               const double* __restrict__ inv_exner, int ncol, int nlev, int64_t ld,
                               double* __restrict__ water, double* __restrict__ energy) {
  constexpr double g = 9.80616, cp = 1004.64, Lv = 2501000.0, Lf = 333700.0;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= ncol) return;
  const int64_t o = int64_t(warp) * ld;
  double w = 0, e = 0;
  for (int k = lane; k < nlev; k += 32) {
    const double dp = dpres[o + k];
    const double T = th[o + k] / inv_exner[o + k];
    w += (qv[o + k] + qc[o + k] + qi[o + k] + qr[o + k]) * dp / g;
    e += (T * cp + (Lv + Lf) * qv[o + k] + Lf * (qc[o + k] + qr[o + k])) * dp / g;
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    w += __shfl_xor_sync(0xffffffffu, w, off);
    e += __shfl_xor_sync(0xffffffffu, e, off);
  }
  if (lane == 0) {
    if (water) water[warp] = w;
    if (energy) energy[warp] = e;
  }
}

/* Column totals of the mass and energy conservation check
 * (share/property_checks/mass_and_energy_column_conservation_check.cpp:281-298
 * compute_total_mass_on_column, :314-347 compute_total_energy_on_column),
 * one warp per column; with the totals before the process, also the relative
 * errors against the totals expected from the boundary fluxes (:140-200,
 * :300-312, :349-363).  Kinetic energy is included when winds are given,
 * phis ps / g when both are given. */
__global__ void conservation_kernel(ConsPtrs p, int ncol, int nlev, int64_t ld, double dt) {
  constexpr double g = 9.80616, cp = 1004.64, Lv = 2501000.0, Lf = 333700.0, rho_w = 1000.0;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= ncol) return;
  const int64_t o = int64_t(warp) * ld;
  double m = 0, e = 0;
  for (int k = lane; k < nlev; k += 32) {
    const double pd = p.pd[o + k];
    m += (p.qv[o + k] + p.qc[o + k] + p.qi[o + k] + p.qr[o + k]) * pd / g;
    double ke = 0;
    if (p.winds) {
      const double u = p.winds[int64_t(warp) * 2 * ld + k], v = p.winds[int64_t(warp) * 2 * ld + ld + k];
      ke = 0.5 * (u * u + v * v);
    }
    e += (p.T[o + k] * cp + ke + (Lv + Lf) * p.qv[o + k] + Lf * (p.qc[o + k] + p.qr[o + k])) * pd / g;
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    m += __shfl_xor_sync(0xffffffffu, m, off);
    e += __shfl_xor_sync(0xffffffffu, e, off);
  }
  if (lane != 0) return;
  if (p.ps && p.phis) e += p.phis[warp] * p.ps[warp] / g;
  if (p.mass) p.mass[warp] = m;
  if (p.energy) p.energy[warp] = e;
  if (p.mass_before) {
    const double vf = p.vapor_flux ? p.vapor_flux[warp] : 0.0, wf = p.water_flux ? p.water_flux[warp] : 0.0;
    const double inf = p.ice_flux ? p.ice_flux[warp] : 0.0, hf = p.heat_flux ? p.heat_flux[warp] : 0.0;
    const double m0 = p.mass_before[warp], e0 = p.energy_before[warp];
    const double m_exp = m0 + (vf - wf * rho_w) * dt;
    const double e_exp = e0 + (vf * (Lv + Lf) - (wf - inf) * rho_w * Lf + hf) * dt;
    p.mass_err[warp] = fabs(m - m_exp) / m0;
    p.energy_err[warp] = fabs(e - e_exp) / e0;
  }
}

/* Largest relative error and its column (the smallest column among equal
 * maxima), one block; errors are non-negative, so their bit patterns order
 * as the values (a NaN error sorts above every number). */
__global__ void maxloc_kernel(const double* __restrict__ a, const double* __restrict__ b, int n,
                              double* __restrict__ out) {
  __shared__ unsigned long long best_a[32], best_b[32];
  __shared__ int loc_a[32], loc_b[32];
  unsigned long long va = 0, vb = 0;
  int la = -1, lb = -1;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const unsigned long long xa = __double_as_longlong(a[i]), xb = __double_as_longlong(b[i]);
    if (la < 0 || xa > va) { va = xa; la = i; }
    if (lb < 0 || xb > vb) { vb = xb; lb = i; }
  }
  for (int off = 16; off > 0; off >>= 1) {
    const unsigned long long oa = __shfl_down_sync(0xffffffffu, va, off), ob = __shfl_down_sync(0xffffffffu, vb, off);
    const int ola = __shfl_down_sync(0xffffffffu, la, off), olb = __shfl_down_sync(0xffffffffu, lb, off);
    if (ola >= 0 && (la < 0 || oa > va || (oa == va && ola < la))) { va = oa; la = ola; }
    if (olb >= 0 && (lb < 0 || ob > vb || (ob == vb && olb < lb))) { vb = ob; lb = olb; }
  }
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) { best_a[w] = va; loc_a[w] = la; best_b[w] = vb; loc_b[w] = lb; }
  __syncthreads();
  if (threadIdx.x == 0) {
    va = 0; vb = 0; la = -1; lb = -1;
    for (int i = 0; i < int(blockDim.x >> 5); ++i) {
      if (loc_a[i] >= 0 && (la < 0 || best_a[i] > va || (best_a[i] == va && loc_a[i] < la))) { va = best_a[i]; la = loc_a[i]; }
      if (loc_b[i] >= 0 && (lb < 0 || best_b[i] > vb || (best_b[i] == vb && loc_b[i] < lb))) { vb = best_b[i]; lb = loc_b[i]; }
    }
    out[0] = __longlong_as_double(va);
    out[1] = double(la);
    out[2] = __longlong_as_double(vb);
    out[3] = double(lb);
  }
}

}  // namespace

cudaError_t launch_conservation(const ConsPtrs& p, int ncol, int nlev, int64_t ld, double dt, double* maxloc4,
                                cudaStream_t st) {
  if (ncol <= 0) return cudaSuccess;
  const int threads = 256;
  const long long blocks = (int64_t(ncol) * 32 + threads - 1) / threads;
  conservation_kernel<<<unsigned(blocks), threads, 0, st>>>(p, ncol, nlev, ld, dt);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || !maxloc4) return e;
  maxloc_kernel<<<1, 1024, 0, st>>>(p.mass_err, p.energy_err, ncol, maxloc4);
  return cudaGetLastError();
}

__global__ void postamble_kernel(const dev::Inst* __restrict__ insts, const dev::WorkItem* __restrict__ work,
                                 int nwork) {
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for (int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < nwork; w += warps) {
    const dev::WorkItem wi = work[w];
    const dev::Inst& in = insts[wi.inst];
    const int64_t co = int64_t(wi.col) * in.ld;
    double* qv_prev = const_cast<double*>(in.qv_prev);
    double* t_prev = const_cast<double*>(in.t_prev);
    for (int k = lane; k < in.nlev; k += 32) {
      qv_prev[co + k] = in.qv[co + k];
      t_prev[co + k] = in.th[co + k] / in.inv_exner[co + k];
    }
  }
}

/* Process-interface preamble and postamble (eamxx_p3_process_interface.hpp:
 * 63-269; the physics helpers restate
 * share/util/scream_common_physics_functions_impl.hpp:88-426).  One warp per
 * column, lanes over its levels (coalesced, no index division).  The
 * wet <-> dry factor pseudo_density / pseudo_density_dry (or its inverse) is
 * formed once per level and multiplies the ten mixing ratios, where the
 * reference divides each of them (x * pd / pdd): one rounding apart, at most
 * ~2 ulp, for a tenth of the FP64 divisions, which set this kernel's cost
 * on a part whose FP64 pipe issues a warp instruction every 16 cycles. */
__global__ void interface_preamble_kernel(InterfacePtrs p, int ncol, int nlev, int64_t ld) {
  const int col = int((int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (col >= ncol) return;
  const double c1 = -1.0 + 1.0 / dev::C::ep_2;
  const double mincld = 0.0001;
  for (int k = lane; k < nlev; k += 32) {
    const int64_t o = int64_t(col) * ld + k;
    const double pd = p.pd[o], pdd = p.pdd[o], pmid = p.pmid[o], T = p.T[o];
    const double qv_wet = p.q[8][o];
    /* calculate_dz with the virtual temperature of the wet state */
    const double Tv = T * (1.0 + c1 * qv_wet);
    p.dz[o] = (dev::C::RD / dev::C::gravit) * pd * Tv / pmid;
    const double wet_to_dry = pd / pdd;
#pragma unroll
    for (int s = 0; s < 9; ++s) p.q[s][o] = p.q[s][o] * wet_to_dry;
    p.qv_prev[o] = p.qv_prev[o] * wet_to_dry;
    const double exner = pow(pmid / dev::C::P0, dev::C::RD * dev::C::INV_CP);
    p.inv_exner[o] = 1.0 / exner;
    p.th[o] = T / exner;
    const double ct = p.cld_t[o];
    const double cl = ct > mincld ? ct : mincld;
    p.cld_l[o] = cl;
    p.cld_i[o] = cl;
    double cr = cl;
    if (k > 0) {
      const double above = p.cld_t[o - 1];
      cr = above > cr ? above : cr;
    }
    p.cld_r[o] = cr;
  }
}

__global__ void interface_postamble_kernel(InterfacePtrs p, int ncol, int nlev, int64_t ld, double dt) {
  const int col = int((int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (col >= ncol) return;
  for (int k = lane; k < nlev; k += 32) {
    const int64_t o = int64_t(col) * ld + k;
    const double pd = p.pd[o], pdd = p.pdd[o], pmid = p.pmid[o];
    const double dry_to_wet = pdd / pd;
    const double T_before = p.T[o];
    const double exner = pow(pmid / dev::C::P0, dev::C::RD * dev::C::INV_CP);
    double T = (p.th[o] * exner - T_before) * dry_to_wet;
    T += T_before;
    p.T[o] = T;
    p.T_prev[o] = T;
#pragma unroll
    for (int s = 0; s < 9; ++s) p.q[s][o] = p.q[s][o] * dry_to_wet;
    p.qv_prev[o] = p.q[8][o];
    p.eff_qc[o] *= 1e6;
    p.eff_qi[o] *= 1e6;
    p.eff_qr[o] *= 1e6;
  }
  if (lane == 0) {
    const double liq = p.liq_surf[col], ice = p.ice_surf[col];
    if (p.liq_mass) p.liq_mass[col] += liq * dev::C::RHO_H2O * dt;
    if (p.ice_mass) p.ice_mass[col] += ice * dev::C::RHO_H2O * dt;
    if (p.vapor_flux) p.vapor_flux[col] = 0.0;
    if (p.water_flux) p.water_flux[col] = liq + ice;
    if (p.ice_flux) p.ice_flux[col] = ice;
    if (p.heat_flux) p.heat_flux[col] = 0.0;
  }
}

/* EAM's P3 driver micro_p3_tend (eam/src/physics/p3/scream/
 * micro_p3_interface.F90:661-1431) around the step, one warp per column.
 * EAM's own constants (share/util/shr_const_mod.F90 through physconst):
 * R_dry from the gas constant and the molecular weight of dry air, cp_dry
 * and g; the driver's literal 287.15 in the in-cloud number concentrations
 * is kept as written. */
namespace eam {
constexpr double kRgas = 6.02214e26 * 1.38065e-23;
constexpr double kRair = kRgas / 28.966, kCpair = 1.00464e3, kGravit = 9.80616;
constexpr double kMincld = 0.0001, kQsmall = 1.0e-14;
constexpr double kMucon = 5.3, kDcon = 25.e-6, kDeicon = 50.0;
__device__ __forceinline__ double fmax_(double a, double b) { return a > b ? a : b; } /* Fortran max for these ranges */
__device__ __forceinline__ double fmin_(double a, double b) { return a < b ? a : b; }
}  // namespace eam

/* Preparation of the P3 inputs (micro_p3_interface.F90:982-1047) and the
 * cloud fractions of get_cloud_fraction (:661-732).  The rain fraction's
 * recurrence down the column, r_k = c_k ? max(r_{k-1}, m_k) : m_k (m the
 * floored cloud fraction; c_k: rain or ice above (max overlap) or no cloud
 * here (in cloud)), is a segmented maximum: a warp scan over each 32-level
 * chunk with the chunk above carried in.  Same values as the sequential
 * loop (max is exact). */
__global__ void eam_pre_kernel(EamPtrs p, int ncol, int nlev, int64_t ld, int64_t ld_int) {
  const int col = int((int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (col >= ncol) return;
  const double kappa = eam::kRair * (1.0 / eam::kCpair);
  double carry = 0.0;
  for (int base = 0; base < nlev; base += 32) {
    const int k = base + lane;
    const bool act = k < nlev;
    double m = 1.0;
    bool reset = true;
    if (act) {
      const int64_t o = int64_t(col) * ld + k;
      const double ratio = p.pdel[o] / p.pdeldry[o];
#pragma unroll
      for (int s = 0; s < 9; ++s) p.w[s][o] = p.q[s][o] * ratio;
      p.qv_prev_dry[o] = p.qv_prev[o] * ratio;
      const double inv_exner = 1.0 / pow(p.pmid[o] * 1.e-5, kappa);
      p.inv_exner[o] = inv_exner;
      const int64_t oi = int64_t(col) * ld_int + k;
      p.dz[o] = p.zi[oi] - p.zi[oi + 1];
      p.th[o] = p.t[o] * inv_exner;
      p.pres[o] = p.pmiddry[o];
      p.dpres[o] = p.pdeldry[o];
      p.nc_nuceat[o] = p.npccn[o];
      p.ni_act[o] = p.ni_act_in[o];
      p.inv_relvar[o] = p.relvar[o];
      p.t_prev_p3[o] = p.t_prev[o];
      if (p.subgrid) {
        m = eam::fmax_(p.ast[o], eam::kMincld);
        if (k > 0) {
          if (p.method == P3X_PRECIP_FRAC_MAX_OVERLAP) {
            /* rain or ice mass in the level above (dry mixing ratios) */
            const double qr_up = p.q[3][o - 1] * (p.pdel[o - 1] / p.pdeldry[o - 1]);
            const double qi_up = p.q[5][o - 1] * (p.pdel[o - 1] / p.pdeldry[o - 1]);
            reset = !(qr_up >= eam::kQsmall || qi_up >= eam::kQsmall);
          } else {
            reset = !(p.w[1][o] < eam::kQsmall && p.w[5][o] < eam::kQsmall);
          }
        }
        p.cld_l[o] = m;
        p.cld_i[o] = m;
      } else {
        p.cld_l[o] = 1.0;
        p.cld_i[o] = 1.0;
        p.cld_r[o] = 1.0;
      }
    }
    if (!p.subgrid) continue;
    /* inclusive segmented maximum over the chunk: (value, segment closed) */
    double v = m;
    bool closed = reset;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const double vu = __shfl_up_sync(0xffffffffu, v, d);
      const bool cu = __shfl_up_sync(0xffffffffu, closed, d);
      if (lane >= d && !closed) {
        v = eam::fmax_(vu, v);
        closed = cu;
      }
    }
    if (!closed) v = eam::fmax_(carry, v);
    if (act) p.cld_r[int64_t(col) * ld + k] = v;
    carry = __shfl_sync(0xffffffffu, v, 31);
  }
}

/* Use of the P3 results (micro_p3_interface.F90:1182-1431). */
__global__ void eam_post_kernel(EamPtrs p, int ncol, int nlev, int64_t ld, int64_t ld_int, double dt) {
  const int col = int((int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (col >= ncol) return;
  double cdnumc = 0.0;
  for (int k = lane; k < nlev; k += 32) {
    const int64_t o = int64_t(col) * ld + k;
    const double ratio = p.pdeldry[o] / p.pdel[o];
    double w[9];
#pragma unroll
    for (int s = 0; s < 9; ++s) w[s] = p.w[s][o] * ratio;
    const double t = p.t[o];
    double dtemp = p.th[o] / p.inv_exner[o] - t;
    dtemp = __dmul_rn(dtemp, ratio); /* rounded before the sum, as the driver writes it (no fused multiply-add) */
    const double temp = dtemp + t;
    p.ptend_s[o] = eam::kCpair * (temp - t) / dt;
#pragma unroll
    for (int s = 0; s < 9; ++s) p.ptend_q[s][o] = (eam::fmax_(0.0, w[s]) - p.q[s][o]) / dt;
    p.t_prev[o] = temp;
    p.qv_prev[o] = w[0];
    const double cme = p.cmeliq[o];
    if (p.qme) p.qme[o] = cme + p.depos[o];
    p.vap_liq[o] = p.vap_liq[o] + cme;
    const double pmid = p.pmid[o];
    if (p.rho) p.rho[o] = pmid / (eam::kRair * temp);
    const double cl = p.cld_l[o], ci = p.cld_i[o], cr = p.cld_r[o];
    const double icimr = eam::fmin_(p.q[5][o] / eam::fmax_(eam::kMincld, ci), 0.005);
    const double icwmr = eam::fmin_(p.q[1][o] / eam::fmax_(eam::kMincld, cl), 0.005);
    const double icin = p.q[6][o] / eam::fmax_(eam::kMincld, ci) * pmid / (287.15 * t);
    const double icwn = p.q[2][o] / eam::fmax_(eam::kMincld, cl) * pmid / (287.15 * t);
    if (p.icimrst) p.icimrst[o] = icimr;
    if (p.icwmrst) p.icwmrst[o] = icwmr;
    if (p.icinc) p.icinc[o] = icin;
    if (p.icwnc) p.icwnc[o] = icwn;
    const double rel = p.eff_qc[o] * 1e6, rei = p.eff_qi[o] * 1e6;
    double dei = rei * 2.0, mu = 0.0, lambdac = 0.0;
    if (p.ast[o] < 1.e-4) {
      mu = eam::kMucon;
      lambdac = (eam::kMucon + 1.0) / eam::kDcon;
      dei = eam::kDeicon;
    }
    if (p.rel) p.rel[o] = rel;
    if (p.rei) p.rei[o] = rei;
    if (p.dei) p.dei[o] = dei;
    if (p.mu) p.mu[o] = mu;
    if (p.lambdac) p.lambdac[o] = lambdac;
    /* w: 1 cldliq, 2 numliq, 3 rain, 4 numrain, 5 cldice */
    const double tot = w[3] + w[5] + w[1];
    if (p.nfice) p.nfice[o] = (w[5] > eam::kQsmall && tot > eam::kQsmall) ? eam::fmin_(w[5] / tot, 1.0) : 0.0;
    cdnumc = cdnumc + w[2] * p.pdel[o] / eam::kGravit;
    const bool liq = cl > 0.01 && icwmr > 5.e-5, ice = ci > 0.01 && icimr > 1.e-6;
    if (p.efcout) p.efcout[o] = liq ? rel * cl : 0.0;
    if (p.ncout) p.ncout[o] = liq ? icwn * cl : 0.0;
    if (p.freql) p.freql[o] = liq ? cl : 0.0;
    if (p.efiout) p.efiout[o] = ice ? rei * ci : 0.0;
    if (p.niout) p.niout[o] = ice ? icin * ci : 0.0;
    if (p.freqi) p.freqi[o] = ice ? ci : 0.0;
    const double reff = p.eff_qr[o];
    if (p.deff_rain) p.deff_rain[o] = reff * 2.0 * 1.e6;
    const bool rain = w[3] >= 1.e-7;
    if (p.aqrain) p.aqrain[o] = rain ? w[3] * cr : 0.0;
    if (p.anrain) p.anrain[o] = rain ? w[4] * cr : 0.0;
    if (p.freqr) p.freqr[o] = rain ? cr : 0.0;
    if (p.reff_rain) p.reff_rain[o] = rain ? reff * 1.e6 : reff;
  }
  for (int k = lane; k <= nlev; k += 32) {
    const int64_t oi = int64_t(col) * ld_int + k;
    const double lf = p.liq_flux[oi], fi = p.ice_flux[oi];
    if (p.flxprc) p.flxprc[oi] = lf + fi;
    if (p.flxsnw) p.flxsnw[oi] = fi;
  }
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) cdnumc += __shfl_xor_sync(0xffffffffu, cdnumc, d);
  if (lane == 0) {
    const double liq = p.liq_surf[col], ice = p.ice_surf[col];
    const double pcw = liq + ice;
    if (p.prec_pcw) p.prec_pcw[col] = pcw;
    if (p.prec_str) p.prec_str[col] = pcw + 0.0;
    if (p.snow_pcw) p.snow_pcw[col] = ice;
    if (p.snow_str) p.snow_str[col] = ice + 0.0;
    if (p.cdnumc) p.cdnumc[col] = cdnumc;
  }
}

cudaError_t launch_eam(const EamPtrs& p, int ncol, int nlev, int64_t ld, int64_t ld_int, bool post, double dt,
                       cudaStream_t st) {
  if (ncol <= 0 || nlev <= 0) return cudaSuccess;
  const int threads = 256;
  const long long blocks = (int64_t(ncol) * 32 + threads - 1) / threads;
  if (post) {
    eam_post_kernel<<<unsigned(blocks), threads, 0, st>>>(p, ncol, nlev, ld, ld_int, dt);
  } else {
    eam_pre_kernel<<<unsigned(blocks), threads, 0, st>>>(p, ncol, nlev, ld, ld_int);
  }
  return cudaGetLastError();
}

cudaError_t launch_interface(const InterfacePtrs& p, int ncol, int nlev, int64_t ld, bool post, double dt,
                             cudaStream_t st) {
  if (ncol <= 0 || nlev <= 0) return cudaSuccess;
  const int threads = 256;
  const long long blocks = (int64_t(ncol) * 32 + threads - 1) / threads;
  if (post) {
    interface_postamble_kernel<<<unsigned(blocks), threads, 0, st>>>(p, ncol, nlev, ld, dt);
  } else {
    interface_preamble_kernel<<<unsigned(blocks), threads, 0, st>>>(p, ncol, nlev, ld);
  }
  return cudaGetLastError();
}

cudaError_t launch_postamble(const dev::Inst* insts_d, const dev::WorkItem* work_d, int nwork, cudaStream_t st) {
  if (nwork <= 0) return cudaSuccess;
  const int threads = 256, per_block = threads / 32;
  int blocks = (nwork + per_block - 1) / per_block;
  if (blocks > 4096) blocks = 4096;
  postamble_kernel<<<blocks, threads, 0, st>>>(insts_d, work_d, nwork);
  return cudaGetLastError();
}

/* Exhaustive check of the integer-pipe float -> double conversion against
 * the hardware conversion: every one of the 2^32 float bit patterns. */
/* Every float bit pattern: the integer-pipe float -> double conversion
 * against the hardware one, and the FP32-pipe table index against the
 * hardware truncation after the callers' clamps ([1, hi - 1] and [1, hi]);
 * every integer below 2^22 in magnitude: its float on the FP32 pipe; 2^32
 * doubles covering every high word: the integer-pipe narrowing toward zero
 * against the hardware conversion; 2^24 hashed operand sets: the packed
 * double-float accumulation against the scalar one. */
__global__ void f2d_selftest_kernel(unsigned long long* mismatches) {
  unsigned long long bad = 0;
  const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < (uint64_t(1) << 32); i += stride) {
    const float x = __uint_as_float(uint32_t(i));
    const double a = dev::f2d_int(x), b = double(x);
    if (__double_as_longlong(a) != __double_as_longlong(b)) ++bad;
    const int tz = __float2int_rz(x);
    for (const int hi : {4, 5, 20, 30, 50, 300}) {
      const int ti = dev::table_index(x, hi);
      if (min(hi - 1, max(1, ti)) != min(hi - 1, max(1, tz))) ++bad;
      if (min(hi, max(1, ti)) != min(hi, max(1, tz))) ++bad;
    }
    const int j = int(uint32_t(i));
    if (j > -(1 << 22) && j < (1 << 22) && dev::i2f_small(j) != __int2float_rn(j)) ++bad;
    /* a double with this pattern as its high word and a hashed low word:
     * every sign, exponent and leading significand */
    const double y = __hiloint2double(int(uint32_t(i)), int(uint32_t(i) * 2654435761u));
    const double ay = fabs(y);
    const float want = !(ay < 0x1p128) ? __double2float_rn(y)
                                        : (ay < 0x1p-126 ? (signbit(y) ? -0.0f : 0.0f) : __double2float_rz(y));
    const float got = dev::d2f_rz(y);
    if (__float_as_uint(got) != __float_as_uint(want) && !(isnan(got) && isnan(want))) ++bad;
    /* the packed double-float accumulation against two scalar ones, on
     * hashed operands spanning many magnitudes */
    if ((i & 255u) == 0u) {
      const uint32_t h1 = uint32_t(i) * 747796405u + 2891336453u, h2 = h1 * 277803737u + 1u;
      const float s1 = __uint_as_float(0x30000000u + (h1 >> 4)), s2 = __uint_as_float(0x30000000u + (h2 >> 4));
      const float lo1 = s1 * 1.0e-8f, lo2 = -s2 * 3.0e-8f;
      const float a1 = __uint_as_float(0x34000000u + (h2 >> 5)), a2 = __uint_as_float(0x36000000u + (h1 >> 5));
      const float tt = __uint_as_float(0x3f800000u + (h1 & 0x7fffffu)) * 37.0f;
      float4 g = make_float4(s1, s2, lo1, lo2);
      float2 g1 = make_float2(s1, lo1), g2 = make_float2(s2, lo2);
      dev::dfloat2_add_prod(g, make_float2(a1, a2), tt);
      dev::dfloat_add_prod(g1, a1, tt);
      dev::dfloat_add_prod(g2, a2, tt);
      if (__float_as_uint(g.x) != __float_as_uint(g1.x) || __float_as_uint(g.z) != __float_as_uint(g1.y) ||
          __float_as_uint(g.y) != __float_as_uint(g2.x) || __float_as_uint(g.w) != __float_as_uint(g2.y))
        ++bad;
    }
  }
  if (bad) atomicAdd(mismatches, bad);
}

cudaError_t launch_selftest(unsigned long long* mismatches_d, cudaStream_t st) {
  f2d_selftest_kernel<<<4096, 256, 0, st>>>(mismatches_d);
  return cudaGetLastError();
}

cudaError_t launch_transpose_to_levels(const double* src, double* dst, int ncol, int nlev, int64_t ld,
                                       cudaStream_t st) {
  if (ncol <= 0 || nlev <= 0) return cudaSuccess;
  dim3 grid((ncol + 31) / 32, (nlev + 31) / 32), block(32, 8);
  transpose_to_levels<<<grid, block, 0, st>>>(src, dst, ncol, nlev, ld);
  return cudaGetLastError();
}

cudaError_t launch_transpose_to_columns(const double* src, double* dst, int ncol, int nlev, int64_t ld,
                                        cudaStream_t st) {
  if (ncol <= 0 || nlev <= 0) return cudaSuccess;
  dim3 grid((ncol + 31) / 32, (nlev + 31) / 32), block(32, 8);
  transpose_to_columns<<<grid, block, 0, st>>>(src, dst, ncol, nlev, ld);
  return cudaGetLastError();
}

cudaError_t launch_budgets(const double* qv, const double* qc, const double* qr, const double* qi,
                           const double* th, const double* dpres, const double* inv_exner, int ncol,
                           int nlev, int64_t ld, double* water, double* energy, cudaStream_t st) {
  if (ncol <= 0) return cudaSuccess;
  const int threads = 256;
  const long long blocks = (int64_t(ncol) * 32 + threads - 1) / threads;
  column_budgets<<<unsigned(blocks), threads, 0, st>>>(qv, qc, qr, qi, th, dpres, inv_exner, ncol, nlev, ld,
                                                       water, energy);
  return cudaGetLastError();
}

}  // namespace p3x
