/* Launch helpers of the column kernels (included by the per-variant TUs). */
#pragma once

#include "p3x_launch.hpp"

namespace p3x {

/* Persistent launch of one kernel: the grid is the number of CTAs that fit on
 * all SMs at once (capped by blocks_per_sm when given, and by the amount of
 * work); groups walk the work list with a grid stride.  The occupancy comes
 * from a per-device cache, so a launch makes no attribute or occupancy query
 * after the first one of its shape. */
template <class TR, class Kern>
cudaError_t launch_persistent(Kern kern, const dev::Inst& inst0, const dev::KParams<TR>& kp, int threads,
                              size_t smem, int blocks_per_sm, int num_sms, cudaStream_t stream,
                              double grid_frac = 1.0) {
  int per_sm = 0;
  cudaError_t e = kernel_occupancy(reinterpret_cast<const void*>(kern), threads, smem, &per_sm);
  if (e != cudaSuccess) return e;
  if (per_sm <= 0) return cudaErrorInvalidConfiguration;
  if (blocks_per_sm > 0) per_sm = per_sm < blocks_per_sm ? per_sm : blocks_per_sm;
  long long grid = (long long)per_sm * num_sms;
  /* a share of the capacity leaves room on every SM for other streams' launches */
  if (grid_frac > 0 && grid_frac < 1) {
    const long long share = (long long)(double(grid) * grid_frac);
    grid = share > 0 ? share : 1;
  }
  const long long need = (kp.nwork + kp.groups_per_block - 1) / kp.groups_per_block;
  if (need < grid) grid = need;
  if (grid <= 0) return cudaSuccess;
  kern<<<int(grid), threads, smem, stream>>>(inst0, kp);
  return cudaGetLastError();
}

template <class TR, int LANES>
cudaError_t launch_p3_part(const dev::Inst& inst0, const dev::KParams<TR>& kp_in, const LaunchSpec& ls, int part,
                           int num_sms, cudaStream_t stream) {
  dev::KParams<TR> kp = kp_in;
  kp.groups_per_block = ls.groups_per_block;
  kp.staged = ls.staged;
  const int threads = ls.groups_per_block * LANES;
  if (threads <= 0 || threads > 256) return cudaErrorInvalidValue;
  cudaError_t e = cudaErrorInvalidValue;
  if (part == kPartK1) {
    if (kp.wctr) {
      e = cudaMemsetAsync(kp.wctr, 0, dev::kWorkCounters * sizeof(uint32_t), stream);
      if (e != cudaSuccess) return e;
    }
    if (ls.marks) cudaEventRecord(ls.marks[0], stream);
    e = launch_persistent<TR>(dev::p3_part12_kernel<TR, LANES>, inst0, kp, threads,
                              p3_smem_bytes<TR>(ls, kp.sm_stride), ls.blocks_per_sm, num_sms, stream, ls.grid_frac);
    if (e == cudaSuccess && ls.marks) cudaEventRecord(ls.marks[1], stream);
  } else if (part == kPartK2) {
    if constexpr (LANES == 32) {
      if constexpr (sizeof(TR) == sizeof(float)) {
        e = launch_persistent<TR>(dev::p3_sed_bulk_kernel<LANES>, inst0, kp, threads,
                                  sed_smem_bytes<TR>(ls, kp.sm_stride), 0, num_sms, stream, ls.grid_frac);
      } else {
        e = launch_persistent<TR>(dev::p3_sed_kernel<TR, LANES>, inst0, kp, threads,
                                  sed_smem_bytes<TR>(ls, kp.sm_stride), 0, num_sms, stream, ls.grid_frac);
      }
      if (e == cudaSuccess && ls.marks) cudaEventRecord(ls.marks[2], stream);
    }
  } else if (part == kPartK3) {
    e = launch_persistent<TR>(dev::p3_part3_kernel<TR, LANES>, inst0, kp, threads, 0, 0, num_sms, stream,
                              ls.grid_frac);
    if (e == cudaSuccess && ls.marks) cudaEventRecord(ls.marks[3], stream);
  }
  return e;
}

}  // namespace p3x
