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
