// pcg_pipeline.cu -- pipelined batched step.
//
// The batched step's phases have very different bounds on this GPU: the
// update (SWE_WaveAccumulationBlock::updateUnknowns) and the ghost fill move
// bytes and barely use the FP64 pipe, the f-wave sweep
// (computeNumericalFluxes) is FP64-bound with the memory system nearly idle.
// Run one after the other they add up; here one persistent kernel per step
// runs the update of step k - 1 and the ghost fill, walls and sweep of step
// k together, so that the update's and the fill's memory traffic hides under
// the sweep's FP64 work.
//
// Every warp takes work items in queue order (one atomic per item): strip
// updates (U), chunks of 32 ghost cells (G), wall patches (W) and strip
// sweeps (S).  The host orders the queue so that an item's prerequisites come
// before it; an item waits, on per-patch counters, only for those:
//   G (src -> dst):  U of src (its per-item time factor comes from
//                    k_pipeline_items, computed before the launch from the
//                    intervals the updates will leave);
//   W (patch p):     U of p, every G into p (corner cells);
//   S (item):        for each patch p of its lane groups: U of p, every G
//                    into p, every G reading from p (the sweep overwrites
//                    p's uOld interior with net updates), W of p.
// Since every prerequisite sits earlier in the queue it has been taken by a
// running warp, so the earliest unfinished item can always proceed.  Writers
// publish with a fence and an atomic add after their stores; readers poll
// with acquire loads and read patch data through L2 (ld.global.cg), never a
// stale L1 line.  A wait has a time limit: when it runs out the error word is
// set, every warp stops taking items and the host reports the step as failed.
//
// The arithmetic of every cell is that of the separate kernels (the same
// device functions: pcg_strip_ops.cuh, pcg_ghost_ops.cuh), so results are
// bit-identical to the unfused step.
#include "pcg_ghost_ops.cuh"
#include "pcg_kernels.h"
#include "pcg_strip_ops.cuh"

namespace pcg {

namespace {

// A wait for a counter gives up after 0.2 s (a step takes milliseconds).
constexpr unsigned long long kPipeWaitNs = 200000000ull;
// Columns an update item loads before storing: one keeps the update's
// registers within the sweep's budget (four, as in k_update_strips, spills
// about 200 bytes a thread in this kernel); its memory latency overlaps the
// other warps' sweeps.
constexpr int kPipeUpdateBatch = 1;

__device__ __forceinline__ int ld_acquire(const int *p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ int ld_volatile(const int *p) { return *(const volatile int *)p; }

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Until *cnt >= target; false once the time limit ran out here (the error
// word is then set) or the error word was set elsewhere.
__device__ bool pipe_wait(const int *cnt, int target, PipeCtl *ctl) {
  if (ld_acquire(cnt) >= target) return true;
  const unsigned long long t0 = global_ns();
  unsigned ns = 64;
  for (;;) {
    __nanosleep(ns);
    if (ld_acquire(cnt) >= target) return true;
    if (ld_volatile(&ctl->err)) return false;
    if (global_ns() - t0 > kPipeWaitNs) {
      atomicCAS(&ctl->err, 0, 1);
      return false;
    }
    if (ns < 2048) ns <<= 1;
  }
}

// After the calling warp's stores: make them visible at GPU scope before the
// counter moves (every lane fences, then one lane adds).
__device__ __forceinline__ void publish_fence() {
  __threadfence();
  __syncwarp();
}

}  // namespace

template <int kWarps, int kMinBlocks>
__global__ void __launch_bounds__(kWarps * 32, kMinBlocks) k_pipeline_step(const PipeDev A) {
  __shared__ strip::StripWarpSmem SM[kWarps];
  __shared__ strip::StripLaneSmem LS[kWarps];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  PipeCtl *ctl = A.ctl;
  const int k = ld_volatile(&ctl->k);
  const int steps = ld_volatile(&ctl->steps);
  const bool first = k == 0;     // nothing to update yet
  const bool last = k >= steps;  // nothing to sweep any more
  // counters and targets of patch p: [0] strip groups updated, [1] ghost
  // cells written into p, [2] ghost cells read from p, [3] walls filled
  // (computed where used: few registers stay live across the item loop)
#define PIPE_CNT(c, p) (A.cnt + (long long)(c) * A.n_patches + (p))
#define PIPE_NEED(c, p) (A.need[(long long)(c) * A.n_patches + (p)])

  for (;;) {
    int idx = 0;
    if (lane == 0) idx = atomicAdd(&ctl->head, 1);
    idx = __shfl_sync(0xffffffffu, idx, 0);
    if (idx >= A.n_queue || ld_volatile(&ctl->err)) break;
    const unsigned code = A.queue[idx];
    const unsigned kind = code >> kPipeKindShift;
    const int i = (int)(code & kPipeIndexMask);

    if (kind == kPipeUpdate) {
      if (first) continue;
      const StripItem I = A.items[i];
      strip::update_item<true, kPipeUpdateBatch>(A.slab, A.patches, A.times, I, A.groups, A.prm, A.cur_smax,
                                                  A.cur_dt, A.cur_active, A.fin, nullptr, nullptr, UpdateBands(),
                                                  lane);
      const int hs = I.hs, gi = lane / hs, j = lane - gi * hs;
      publish_fence();
      if (gi < I.ngroups && j == 0) atomicAdd(PIPE_CNT(0, A.groups[I.g0 + gi].pid), 1);
    } else if (kind == kPipeGhost) {
      if (last) continue;
      constexpr int kPer = kPipeGhostChunk / 32;  // entries per lane
      int src[kPer], dst[kPer];
      bool ok = true;
#pragma unroll
      for (int k = 0; k < kPer; k++) {
        const int e = i * kPipeGhostChunk + k * 32 + lane;
        src[k] = dst[k] = -1;
        if (e < A.n_ghost) {
          const int item = e < A.ncopy ? A.copy_plan[e].item : A.cells[e].item;
          src[k] = A.gitems[item].src;
          dst[k] = A.gitems[item].dst;
          if (!first) ok = ok && pipe_wait(PIPE_CNT(0, src[k]), PIPE_NEED(0, src[k]), ctl);
        }
      }
      if (__any_sync(0xffffffffu, !ok)) break;
      const auto step_of = [is = A.item_step](int item) { return is[item]; };
#pragma unroll
      for (int k = 0; k < kPer; k++)
        if (dst[k] >= 0)
          ghost_entry<true>(A.slab, A.patches, A.gitems, A.cells, A.ncopy, A.copy_plan, A.plan, step_of,
                            i * kPipeGhostChunk + k * 32 + lane, A.nxt_active, A.fin, nullptr);
      publish_fence();
      // one add per distinct patch and entry row of the chunk
#pragma unroll
      for (int k = 0; k < kPer; k++) {
        const unsigned md = __match_any_sync(0xffffffffu, dst[k]);
        if (dst[k] >= 0 && lane == __ffs(md) - 1) atomicAdd(PIPE_CNT(1, dst[k]), __popc(md));
        const unsigned ms = __match_any_sync(0xffffffffu, src[k]);
        if (src[k] >= 0 && lane == __ffs(ms) - 1) atomicAdd(PIPE_CNT(2, src[k]), __popc(ms));
      }
    } else if (kind == kPipeWall) {
      if (last) continue;
      const int p = A.wall_patches[i];
      bool ok = true;
      if (lane == 0)
        ok = (first || pipe_wait(PIPE_CNT(0, p), PIPE_NEED(0, p), ctl)) && pipe_wait(PIPE_CNT(1, p), PIPE_NEED(1, p), ctl);
      if (!__shfl_sync(0xffffffffu, (int)ok, 0)) break;
      const PatchDev P = A.patches[p];
      if (A.nxt_active[P.group]) {
        // SolveTimestep::fillBoundaryLayers order: (0,lower), (1,upper), (0,upper), (1,lower)
        const int order[4][2] = {{0, 0}, {1, 1}, {0, 1}, {1, 0}};
        for (int f = 0; f < 4; f++) {
          const int d = order[f][0], up = order[f][1];
          if (P.wall & (1 << (2 * d + up))) wall_face<true>(A.slab, P, d, up, true, lane, 32);
          __syncwarp();
        }
      }
      publish_fence();
      if (lane == 0) atomicAdd(PIPE_CNT(3, p), 1);
    } else {
      if (last) continue;
      const StripItem I = A.items[i];
      const int hs = I.hs, gi = lane / hs, j = lane - gi * hs;
      bool ok = true;
      if (gi < I.ngroups && j == 0) {
        const int p = A.groups[I.g0 + gi].pid;
        ok = (first || pipe_wait(PIPE_CNT(0, p), PIPE_NEED(0, p), ctl)) &&
             pipe_wait(PIPE_CNT(1, p), PIPE_NEED(1, p), ctl) && pipe_wait(PIPE_CNT(2, p), PIPE_NEED(2, p), ctl) &&
             pipe_wait(PIPE_CNT(3, p), PIPE_NEED(3, p), ctl);
      }
      if (__any_sync(0xffffffffu, !ok)) break;
      strip::sweep_item<true>(A.slab, A.patches, I, A.groups, A.prm, A.prm.dry_tol, __dmul_rn(0.5, A.prm.g),
                              A.nxt_smax, A.nxt_dt,
                              A.nxt_active, A.fin, nullptr, SM[wid], LS[wid], lane);
    }
  }
#undef PIPE_CNT
#undef PIPE_NEED
  // the last CTA to leave advances the launch index
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const int prev = atomicAdd(&ctl->exited, 1);
    if (prev == (int)gridDim.x - 1) {
      ctl->exited = 0;
      ctl->k = k + 1;
    }
  }
}

__global__ void k_pipeline_pre(const PipePreDev A) {
  const int k = A.ctl->k, steps = A.ctl->steps;
  const bool first = k == 0, last = k >= steps;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
  for (int g = tid; g < A.n_groups; g += stride) {
    if (!first) {
      // end of step k - 1 (as k_record_hist with the time advance)
      const unsigned long long dt = A.nxt_dt[g];
      const int act = A.nxt_active[g];
      A.cur_dt[g] = dt;
      A.cur_active[g] = act;
      if (k - 1 < A.hist_cap) A.hist[(long long)(k - 1) * A.n_groups + g] = bitsd(dt);
      if (act) A.group_time[g] = __dadd_rn(A.group_time[g], bitsd(dt));
    }
    if (!last) {
      // start of step k (as k_reset_step)
      const double rem = __dsub_rn(A.group_t_end[g], A.group_time[g]);
      const bool active = gt_nonneg(rem, 0.0);
      const double cap = active ? rem : 0.0;
      const double mx = A.group_max_dt[g];
      A.nxt_dt[g] = dbits(lt_ieee(cap, mx) ? cap : mx);
      A.nxt_active[g] = active ? 1 : 0;
    }
  }
  for (int p = tid; p < A.n_patches; p += stride) {
    if (!first) A.cur_smax[p] = A.nxt_smax[p];
    if (!last) A.nxt_smax[p] = 0ull;
  }
  for (int c = tid; c < 4 * A.n_patches; c += stride) A.cnt[c] = 0;
  if (tid == 0) A.ctl->head = 0;
}

__global__ void k_pipeline_items(const PipeItemsDev A) {
  const int k = A.ctl->k, steps = A.ctl->steps;
  if (k >= steps) return;  // the last launch fills no ghost cells
  const bool first = k == 0;
  // a patch's time interval after the update of step k - 1 (k_update_strips:
  // leaves of active groups whose dt > 0 move on by their previous dt)
  const auto after_update = [&](int p) {
    PatchTimeDev T = A.times[p];
    const PatchDev &P = A.patches[p];
    if (!first && is_leaf(P) && A.cur_active[P.group]) {
      const double dt = bitsd(A.cur_dt[P.group]);
      if (tl_greater(dt, 0.0)) {
        T.time = __dadd_rn(T.time, T.dt);
        T.dt = dt;
      }
    }
    return T;
  };
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < A.n_items; i += gridDim.x * blockDim.x) {
    const GhostItemDev it = A.items[i];
    const PatchDev &S = A.patches[it.src], &D = A.patches[it.dst];
    const PatchTimeDev ST = after_update(it.src), DT = after_update(it.dst);
    GhostItemStepDev r;
    r.tf = it.kind == 0 ? transfer_tf(S, ST, D, DT) : interp_tf(S, ST, D, DT, false, true);
    r.itf = __dsub_rn(1.0, r.tf);
    r.vn_src = (int)vol_new(S);
    r.vo_src = (int)vol_old(S);
    r.vo_dst = (int)vol_old(D);
    r.nq = it.kind == 0 ? S.nq : (D.nq < 3 ? D.nq : 3);
    A.item_step[i] = r;
  }
}

cudaError_t launch_pipeline_items(cudaStream_t st, const PipeItemsDev &A) {
  if (A.n_items <= 0) return cudaSuccess;
  int grid = (A.n_items + 255) / 256;
  if (grid > 152 * 8) grid = 152 * 8;
  k_pipeline_items<<<grid, 256, 0, st>>>(A);
  return cudaGetLastError();
}

cudaError_t launch_pipeline_pre(cudaStream_t st, const PipePreDev &A) {
  int n = std::max(A.n_groups, 4 * A.n_patches);
  int grid = (n + 255) / 256;
  if (grid < 1) grid = 1;
  if (grid > 152 * 4) grid = 152 * 4;
  k_pipeline_pre<<<grid, 256, 0, st>>>(A);
  return cudaGetLastError();
}

cudaError_t launch_pipeline_step(cudaStream_t st, int variant, int grid, const PipeDev &A) {
  switch (variant) {
    case 0: k_pipeline_step<4, 4><<<grid, 128, 0, st>>>(A); break;
    case 1: k_pipeline_step<4, 5><<<grid, 128, 0, st>>>(A); break;
    case 2: k_pipeline_step<8, 2><<<grid, 256, 0, st>>>(A); break;
    case 3: k_pipeline_step<8, 3><<<grid, 256, 0, st>>>(A); break;
    case 4: k_pipeline_step<6, 3><<<grid, 192, 0, st>>>(A); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t pipeline_occupancy(int variant, int *blocks_per_sm) {
  switch (variant) {
    case 0: return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_pipeline_step<4, 4>, 128, 0);
    case 1: return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_pipeline_step<4, 5>, 128, 0);
    case 2: return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_pipeline_step<8, 2>, 256, 0);
    case 3: return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_pipeline_step<8, 3>, 256, 0);
    case 4: return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_pipeline_step<6, 3>, 192, 0);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace pcg
