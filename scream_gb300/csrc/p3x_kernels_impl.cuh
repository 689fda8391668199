/* Launch helpers of the column kernel (included by the per-variant TUs). */
#pragma once

#include "p3x_launch.hpp"

namespace p3x {

/* Persistent launch of p3_main_kernel<TR, LANES>: the grid is the number of
 * CTAs that fit on all SMs at once (capped by blocks_per_sm when given, and by
 * the amount of work); groups walk the work list with a grid stride. */
template <class TR, int LANES>
cudaError_t launch_p3_lanes(const dev::Inst& inst0, const dev::KParams<TR>& kp_in, const LaunchSpec& ls,
                            int num_sms, cudaStream_t stream) {
  dev::KParams<TR> kp = kp_in;
  kp.groups_per_block = ls.groups_per_block;
  kp.staged = ls.staged;
  const int threads = ls.groups_per_block * LANES;
  if (threads <= 0 || threads > 256) return cudaErrorInvalidValue;
  const size_t smem = p3_smem_bytes<TR>(ls, kp.sm_stride);
  auto kern = dev::p3_main_kernel<TR, LANES>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem);
  if (e != cudaSuccess) return e;
  if (per_sm <= 0) return cudaErrorInvalidConfiguration;
  if (ls.blocks_per_sm > 0) per_sm = per_sm < ls.blocks_per_sm ? per_sm : ls.blocks_per_sm;
  long long grid = (long long)per_sm * num_sms;
  const long long need = (kp.nwork + ls.groups_per_block - 1) / ls.groups_per_block;
  if (need < grid) grid = need;
  if (grid <= 0) return cudaSuccess;
  kern<<<int(grid), threads, smem, stream>>>(inst0, kp);
  return cudaGetLastError();
}

}  // namespace p3x
