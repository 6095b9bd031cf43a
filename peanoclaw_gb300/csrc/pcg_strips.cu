// pcg_strips.cu -- warp-strip form of the batched sweep and update: one
// warp per strip item, grid-stride over the item list (the items themselves
// are in pcg_strip_ops.cuh).
#include "pcg_kernels.h"
#include "pcg_strip_ops.cuh"

namespace pcg {

template <int kWarps, int kMinBlocks>
__global__ void __launch_bounds__(kWarps * 32, kMinBlocks)
    k_sweep_strips(double *__restrict__ slab, const PatchDev *__restrict__ patches,
                   const StripItem *__restrict__ items, const StripGroup *__restrict__ groups,
                   int count, SweParamsDev prm, unsigned long long *__restrict__ patch_smax,
                   unsigned long long *__restrict__ group_dt, const int *__restrict__ group_active,
                   int *__restrict__ fin, const int *__restrict__ pact) {
  __shared__ strip::StripWarpSmem SM[kWarps];
  __shared__ strip::StripLaneSmem LS[kWarps];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const double dry = prm.dry_tol;
  const double halfg = __dmul_rn(0.5, prm.g);
  for (int it = blockIdx.x * kWarps + wid; it < count; it += gridDim.x * kWarps) {
    const StripItem I = items[it];
    strip::sweep_item<false>(slab, patches, I, groups, prm, dry, halfg, patch_smax, group_dt, group_active, fin,
                             pact, SM[wid], LS[wid], lane);
  }
}

// Update in strip order (same per-cell arithmetic as k_update_tiles).
template <int kWarps>
__global__ void __launch_bounds__(kWarps * 32)
    k_update_strips(double *__restrict__ slab, const PatchDev *__restrict__ patches,
                    PatchTimeDev *__restrict__ times, const StripItem *__restrict__ items,
                    const StripGroup *__restrict__ groups, int count, SweParamsDev prm,
                    const unsigned long long *__restrict__ patch_smax,
                    const unsigned long long *__restrict__ group_dt,
                    const int *__restrict__ group_active, int *__restrict__ fin,
                    const int *__restrict__ pact, const unsigned long long *__restrict__ pdt,
                    const UpdateBands ub) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int it = blockIdx.x * kWarps + wid; it < count; it += gridDim.x * kWarps) {
    const StripItem I = items[it];
    strip::update_item<false>(slab, patches, times, I, groups, prm, patch_smax, group_dt, group_active, fin, pact,
                              pdt, ub, lane);
  }
}

namespace {

template <int kWarps, int kMinBlocks>
cudaError_t sweep_strips_t(cudaStream_t st, int grid, double *slab, const PatchDev *patches,
                           const StripItem *items, const StripGroup *groups, int count,
                           const SweParamsDev &prm, unsigned long long *patch_smax,
                           unsigned long long *group_dt, const int *group_active, int *fin,
                           const int *pact) {
  if (count <= 0) return cudaSuccess;
  k_sweep_strips<kWarps, kMinBlocks><<<grid, kWarps * 32, 0, st>>>(slab, patches, items, groups, count,
                                                                   prm, patch_smax, group_dt,
                                                                   group_active, fin, pact);
  return cudaGetLastError();
}

}  // namespace

// Variants of the strip sweep (CTA size, minimum resident CTAs per SM).
const StripVariant kStripVariants[kNumStripVariants] = {
    {4, 4}, {4, 5}, {8, 2}, {8, 3}, {6, 3},
};

cudaError_t launch_sweep_strips(cudaStream_t st, int variant, int grid, double *slab,
                                const PatchDev *patches, const StripItem *items,
                                const StripGroup *groups, int count, const SweParamsDev &prm,
                                unsigned long long *patch_smax, unsigned long long *group_dt,
                                const int *group_active, int *fin, const int *pact) {
  switch (variant) {
    case 0: return sweep_strips_t<4, 4>(st, grid, slab, patches, items, groups, count, prm, patch_smax, group_dt, group_active, fin, pact);
    case 1: return sweep_strips_t<4, 5>(st, grid, slab, patches, items, groups, count, prm, patch_smax, group_dt, group_active, fin, pact);
    case 2: return sweep_strips_t<8, 2>(st, grid, slab, patches, items, groups, count, prm, patch_smax, group_dt, group_active, fin, pact);
    case 3: return sweep_strips_t<8, 3>(st, grid, slab, patches, items, groups, count, prm, patch_smax, group_dt, group_active, fin, pact);
    case 4: return sweep_strips_t<6, 3>(st, grid, slab, patches, items, groups, count, prm, patch_smax, group_dt, group_active, fin, pact);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t strip_occupancy(int variant, int *blocks_per_sm) {
  switch (variant) {
    case 0: return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_sweep_strips<4, 4>, 128, 0);
    case 1: return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_sweep_strips<4, 5>, 128, 0);
    case 2: return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_sweep_strips<8, 2>, 256, 0);
    case 3: return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_sweep_strips<8, 3>, 256, 0);
    case 4: return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_sweep_strips<6, 3>, 192, 0);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t update_strips_occupancy(int *blocks_per_sm) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_update_strips<8>, 256, 0);
}

cudaError_t launch_update_strips(cudaStream_t st, int grid, double *slab, const PatchDev *patches,
                                 PatchTimeDev *times, const StripItem *items, const StripGroup *groups,
                                 int count, const SweParamsDev &prm,
                                 const unsigned long long *patch_smax,
                                 const unsigned long long *group_dt, const int *group_active,
                                 int *fin, const int *pact, const unsigned long long *pdt,
                                 const UpdateBands &ub) {
  if (count <= 0) return cudaSuccess;
  k_update_strips<8><<<grid, 256, 0, st>>>(slab, patches, times, items, groups, count, prm, patch_smax,
                                           group_dt, group_active, fin, pact, pdt, ub);
  return cudaGetLastError();
}

}  // namespace pcg
