// pcg_kernels.h -- host-side launchers of the kernels in pcg_kernels.cu.
#pragma once

#include <cuda.h>

#include <cuda_runtime.h>

#include <string>

#include "pcg_device.cuh"

// Records the calling thread's last error (returned by pcg_last_error) and
// returns `code`.
int pcg_report_error(int code, const std::string &msg);

namespace pcg {

cudaError_t launch_sweep(cudaStream_t st, int grid, double *slab, const PatchDev *patches,
                         const TileItem *tiles, int first, int count, const SweParamsDev &prm,
                         unsigned long long *patch_smax, unsigned long long *group_dt,
                         const int *group_active, int *fin = nullptr, const int *pact = nullptr);
// TMA-staged tile sweep (tiles, variant 1): tensor maps per patch.
struct TileMaps {
  CUtensorMap unew, uold, b;
};
bool tma_tile_shape(const PatchDev &P);
cudaError_t encode_tile_maps(const PatchDev &P, double *slab, TileMaps *out);
cudaError_t launch_sweep_tma(cudaStream_t st, int grid, double *slab, const PatchDev *patches,
                             const TileMaps *maps, const TileItem *tiles, int first, int count,
                             const SweParamsDev &prm, unsigned long long *patch_smax, unsigned long long *group_dt,
                             const int *group_active, int *fin, const int *pact, int *err);
cudaError_t launch_update(cudaStream_t st, int grid, double *slab, const PatchDev *patches,
                          PatchTimeDev *times, const TileItem *tiles, int first, int count,
                          const SweParamsDev &prm, const unsigned long long *patch_smax,
                          const unsigned long long *group_dt, const int *group_active,
                          int *fin = nullptr, const int *pact = nullptr,
                          const unsigned long long *pdt = nullptr);
cudaError_t launch_reset(cudaStream_t st, int n_groups, const double *group_max_dt,
                         const double *group_t_end, const double *group_time,
                         unsigned long long *group_dt, int *group_active, int n_patches,
                         unsigned long long *patch_smax);
// Local time stepping phases: 0 = neighbour constraints and activity (before
// the ghost fill), 1 = per-leaf dt (after the sweep), 2 = group time and dt
// (after the update).
// (leaf, virtual) pairs that set the virtual patches' time intervals in
// local time stepping, the distinct virtual patches and two per-patch key
// arrays for the interval reduction.
struct LtsVirtualDev {
  const int2 *pairs = nullptr;
  int n_pairs = 0;
  const int *virtuals = nullptr;
  int n_virtual = 0;
  unsigned long long *start = nullptr, *end = nullptr;
};
cudaError_t launch_lts(cudaStream_t st, int phase, int n_patches, int n_groups, const PatchDev *patches,
                       PatchTimeDev *times, const GhostItemDev *items, int n_items,
                       const LtsVirtualDev &vt, unsigned long long *nbmin, unsigned long long *patch_smax,
                       unsigned long long *group_tmin, unsigned long long *group_dt,
                       const double *group_max_dt, const double *group_t_end, const int *group_active,
                       int *pact, double *pmaxdt, unsigned long long *pdt, double *group_time,
                       const SweParamsDev &prm, unsigned long long *cells = nullptr);
cudaError_t launch_group_advance(cudaStream_t st, int n_groups, const unsigned long long *group_dt,
                                 const int *group_active, double *group_time);
cudaError_t launch_record_dt(cudaStream_t st, int n_groups, const unsigned long long *group_dt,
                             double *out);
cudaError_t launch_ghost_items(cudaStream_t st, double *slab, const PatchDev *patches,
                               const PatchTimeDev *times, const GhostItemDev *items, int first,
                               int count, const int *group_active);
cudaError_t launch_build_interp_plan(cudaStream_t st, const PatchDev *patches,
                                     const GhostItemDev *items, const GhostCellDev *cells, int count,
                                     InterpPlanDev *plan);
cudaError_t launch_ghost_cells(cudaStream_t st, double *slab, const PatchDev *patches,
                               const GhostItemDev *items, const GhostCellDev *cells, int ncopy,
                               int ninterp, const CopyPlanDev *copy_plan, const InterpPlanDev *plan,
                               const GhostItemStepDev *item_step, const int *group_active,
                               const int *fin, const int *pact = nullptr);
cudaError_t launch_scan_fin(cudaStream_t st, const double *slab, const PatchDev *patches, int count,
                            int *fin);
cudaError_t launch_build_copy_plan(cudaStream_t st, const PatchDev *patches, const GhostItemDev *items,
                                   const GhostCellDev *cells, int count, CopyPlanDev *plan);
// Per patch the depths (x lower, x upper, y lower, y upper; band[4 * pid ..],
// zeroed before) of the uOld interior bands the batched ghost fill reads.
cudaError_t launch_build_bands(cudaStream_t st, const PatchDev *patches, const GhostItemDev *items,
                               const GhostCellDev *cells, int ncopy, int ninterp, const InterpPlanDev *plan,
                               int *band);
cudaError_t launch_reset_items(cudaStream_t st, int n_groups, const double *group_max_dt, const double *group_t_end,
                               const double *group_time, unsigned long long *group_dt, int *group_active,
                               int n_patches, unsigned long long *patch_smax, const PatchDev *patches,
                               const PatchTimeDev *times, const GhostItemDev *items, int count,
                               GhostItemStepDev *out);
cudaError_t launch_item_step(cudaStream_t st, const PatchDev *patches, const PatchTimeDev *times,
                             const GhostItemDev *items, int count, GhostItemStepDev *out);
// from_unew: interior cells read from uNew (the batched step, whose copy
// uNew -> uOld is implicit) or from uOld (the reference layout after a step).
cudaError_t launch_walls(cudaStream_t st, double *slab, const PatchDev *patches,
                         const int *wall_patches, int count, const int *group_active,
                         const int *pact = nullptr, int from_unew = 1);
cudaError_t launch_fill_patch(cudaStream_t st, double *slab, const PatchDev *patches,
                              const PatchTimeDev *times, const GhostItemDev *items, int first,
                              int count, int pid, const int *group_active = nullptr);
size_t solve_patch_smem(int nx, int ny);
cudaError_t sweep_occupancy(int *blocks_per_sm);
cudaError_t prepare_solve_patch(size_t max_dynamic_smem);
cudaError_t launch_solve_patch(cudaStream_t st, double *slab, const PatchDev *patches,
                               PatchTimeDev *times, int pid, int nx, int ny,
                               const SweParamsDev &prm, double max_dt, double *out);
cudaError_t launch_copy_unew_to_uold(cudaStream_t st, double *slab, const PatchDev *patches, int pid,
                                     int n);
cudaError_t launch_swap_unew_uold(cudaStream_t st, double *slab, const PatchDev *patches, int pid, int n);
cudaError_t launch_fill_boundary_layer(cudaStream_t st, double *slab, const PatchDev *patches,
                                       int pid, int dim, int up);
cudaError_t launch_transfer(cudaStream_t st, double *slab, const PatchDev *patches,
                            const PatchTimeDev *times, const GhostItemDev &it);
cudaError_t launch_interpolate_many(cudaStream_t st, double *slab, const PatchDev *patches,
                                    const PatchTimeDev *times, const GhostItemDev *items, int n, int to_uold,
                                    int to_current, int use_unew_uold, int swe);
cudaError_t launch_scatter_times(cudaStream_t st, const long long *ids, const PatchTimeDev *in, int n,
                                 PatchTimeDev *times);
cudaError_t launch_interpolate(cudaStream_t st, double *slab, const PatchDev *patches,
                               const PatchTimeDev *times, const GhostItemDev &it, int to_uold,
                               int to_current, int use_unew_uold, int swe);
cudaError_t launch_restrict(cudaStream_t st, double *slab, const PatchDev *patches,
                            const PatchTimeDev *times, int src, int dst, int only_overlapped, int swe);
// Per-item table of the batched restriction (regions mapped into the
// destination, time factors), built in shared memory by k_level_transfer.
constexpr int kRestrMaxItems = 128;
struct RestrItemTab {
  double tfo, tfn;
  int src, nr, swe, pad_;
  int doff[4][2], dsz[4][2], ro[4][2], rs[4][2];
};
// Work counters of k_level_transfer (its two queues, the finished flux
// destinations, the CTAs that left; zero between launches: the kernel's last
// CTA resets them) and its error word (1: a phase wait ran out).
struct TransferCtl {
  unsigned next, next_store, done_flux, exited;
  int err, pad_[3];
};
constexpr int kTransferThreads = 256;
// Interior cells of a restriction destination per work item of
// k_level_transfer (one item per destination up to 64 x 64 cells: splitting
// a destination's cells over several items measured slower, each item
// reloading the table).
constexpr int kRestrChunkCells = 4096;
// Grid of k_level_transfer: one CTA per work item, at most the resident CTAs.
int level_transfer_grid(int num_sms, int n_leaf, int n_flux, int n_restr);
// Region geometry of the restriction items of n_dst destinations (begin)
// into geo (indexed like the items) and geo_bad (per destination).
cudaError_t launch_restr_geometry(cudaStream_t st, const PatchDev *patches, const PatchTimeDev *times,
                                  const int4 *items, const int *begin, int n_dst, RestrItemTab *geo,
                                  int *geo_bad);
// Flux correction and restriction phases of a batched step in one launch:
// the face fluxes of leaf_ids[0, n_leaf) (n_leaf = 0: none), the flux items
// of n_flux destinations (flux_begin), then the restriction items of the
// destinations (restr_begin, region geometry from launch_restr_geometry) in
// n_restr chunks (restr_chunks: destination, chunk of kRestrChunkCells
// cells); pact (local time stepping, may be null) limits the restriction to
// destinations with an advancing source.  wait_bias (0 in a step) is added
// to the flux destinations the restriction items wait for: the self-test
// sets it so that no wait can end.
cudaError_t launch_level_transfer(cudaStream_t st, int grid, double *slab, const PatchDev *patches,
                                  const PatchTimeDev *times, const int *leaf_ids, int n_leaf, double gf,
                                  const int4 *flux_items, const int *flux_begin, int n_flux,
                                  const int4 *restr_items, const int *restr_begin,
                                  const RestrItemTab *restr_geo, const int *restr_geo_bad,
                                  const int2 *restr_chunks, int n_restr, const int *group_active,
                                  const int *pact, TransferCtl *ctl, int wait_bias = 0);
cudaError_t launch_post_process_restriction(cudaStream_t st, double *slab, const PatchDev *patches,
                                            const int *ids, int count,
                                            const int *group_active = nullptr, const int *dirty = nullptr);
cudaError_t launch_compute_fluxes(cudaStream_t st, double *slab, const PatchDev *patches,
                                  const int *ids, int count, double gf,
                                  const int *group_active = nullptr);
// The flat ghost-cell list from exp[0, n_items] (item, first list entry;
// exp[n_items].y = the list length).
cudaError_t launch_expand_gcells(cudaStream_t st, const int2 *exp, int n_items, GhostCellDev *out);
cudaError_t launch_gather_cells(cudaStream_t st, const double *slab, const PatchDev *patches,
                                const int *ids, const long long *out_off, int count, double *out);
cudaError_t launch_switch_to_leaf(cudaStream_t st, double *slab, const PatchDev *patches,
                                  const PatchTimeDev *times, int pid);
cudaError_t launch_refinement_indicator(cudaStream_t st, const double *slab, const PatchDev *patches,
                                        const int *ids, int count, int kind, double *out);
cudaError_t launch_clear_interior(cudaStream_t st, double *slab, const PatchDev *patches,
                                  const int *ids, int count, const int *group_active = nullptr,
                                  const int *dirty = nullptr);
cudaError_t launch_flux_correction(cudaStream_t st, double *slab, const PatchDev *patches,
                                   const PatchTimeDev *times, int src, int dst, int dim, int dir);

// Warp-strip sweep variants: warps per CTA and minimum resident CTAs per SM
// (the register budget the compiler is held to).
struct StripVariant {
  int warps, min_blocks;
};
constexpr int kNumStripVariants = 5;
extern const StripVariant kStripVariants[kNumStripVariants];
cudaError_t launch_sweep_strips(cudaStream_t st, int variant, int grid, double *slab,
                                const PatchDev *patches, const StripItem *items,
                                const StripGroup *groups, int count, const SweParamsDev &prm,
                                unsigned long long *patch_smax, unsigned long long *group_dt,
                                const int *group_active, int *fin, const int *pact = nullptr);
cudaError_t strip_occupancy(int variant, int *blocks_per_sm);
cudaError_t update_strips_occupancy(int *blocks_per_sm);
cudaError_t launch_update_strips(cudaStream_t st, int grid, double *slab, const PatchDev *patches,
                                 PatchTimeDev *times, const StripItem *items, const StripGroup *groups,
                                 int count, const SweParamsDev &prm,
                                 const unsigned long long *patch_smax,
                                 const unsigned long long *group_dt, const int *group_active,
                                 int *fin, const int *pact = nullptr,
                                 const unsigned long long *pdt = nullptr, const UpdateBands &ub = UpdateBands());

// ---- fused batched step (pcg_fused.cu)
// Everything the fused kernels read besides the work list: the slab and the
// shadow buffer, the patch table, per group the pending-update state (pend:
// the group's last step left an update pending; par: the set it wrote, 0 = A
// in the slab, 1 = B in the shadow; dt_prev: the dt of that update) and
// activity, the face / corner tables (per patch 2 (nx + ny) face codes from
// face_begin[pid], 4 corner codes: >= 0 copy plan, <= -2 interpolation plan
// -code - 2, -1 none) with their plans and the per-item step data.
struct FusedDev {
  double *slab, *shadow;
  const PatchDev *patches;
  const int *pend, *par, *active;
  const unsigned long long *dt_prev;
  const int *face_begin, *face, *corner;
  const FusedCopyDev *copies;
  const FusedInterpDev *interps;
  const GhostItemStepDev *item_step;
  SweParamsDev prm;
};
cudaError_t launch_fused_strips(cudaStream_t st, int variant, int grid, const FusedDev &F, const StripItem *items,
                                const StripGroup *groups, int count, unsigned long long *patch_smax,
                                unsigned long long *group_dt);
cudaError_t fused_occupancy(int variant, int *blocks_per_sm);
cudaError_t launch_fused_advance(cudaStream_t st, const FusedDev &F, const int *leaf_ids, int n_leaves,
                                 PatchTimeDev *times, const unsigned long long *patch_smax, int n_groups,
                                 const unsigned long long *group_dt, double *group_time, int *pend, int *par,
                                 unsigned long long *dt_prev, double *hist, int *counter, int capacity);
cudaError_t launch_fused_flush(cudaStream_t st, const FusedDev &F, const int *leaf_ids, int n_leaves);
cudaError_t launch_build_fused_ghosts(cudaStream_t st, const PatchDev *patches, const GhostItemDev *items,
                                      const GhostCellDev *cells, int ncopy, int ninterp, const InterpPlanDev *plan,
                                      const int *face_begin, int *face, int *corner, FusedCopyDev *copies,
                                      FusedInterpDev *interps);

// ---- pipelined batched step (pcg_pipeline.cu)
// A run of `steps` steps is steps + 1 launches of [k_pipeline_pre,
// k_pipeline_step]: launch k updates with the dt of step k - 1 (k > 0) and
// fills, walls and sweeps step k (k < steps), its work items taken in queue
// order by every warp and held back by per-patch counters until what they
// read is written.  The step index k lives in PipeCtl (set to 0 with `steps`
// by the host before the first launch; the kernel's last CTA advances it).
struct PipeCtl {
  int head;    // next queue entry
  int err;     // 1: a wait for a counter ran out
  int k;       // launch index within the run
  int steps;   // steps of the run
  int exited;  // CTAs that left the kernel (reset by the last one)
  int pad_[3];
};
// Queue entries: item kind in the top two bits, index below.
constexpr unsigned kPipeUpdate = 0, kPipeGhost = 1, kPipeWall = 2, kPipeSweep = 3;
constexpr int kPipeKindShift = 30;
constexpr unsigned kPipeIndexMask = (1u << kPipeKindShift) - 1;
// Ghost-cell entries per ghost work item (four per lane).
constexpr int kPipeGhostChunk = 128;
// Per-patch counters and their targets, four arrays of n_patches each:
// strip groups updated (target: the patch's strip groups), ghost cells written
// into the patch, ghost cells read from the patch (targets: the list's
// counts), walls filled (target 1 for a patch on the wall list, else 0).
struct PipeDev {
  double *slab;
  const PatchDev *patches;
  PatchTimeDev *times;
  const StripItem *items;
  const StripGroup *groups;
  const GhostItemDev *gitems;
  const GhostCellDev *cells;
  const CopyPlanDev *copy_plan;
  const InterpPlanDev *plan;
  int ncopy, n_ghost;
  const GhostItemStepDev *item_step;  // per ghost item, from k_pipeline_items
  const int *wall_patches;
  const unsigned *queue;
  int n_queue, n_patches;
  int *cnt;
  const int *need;
  // dt, activity and max speed of the step being updated (cur) and of the
  // step being swept (nxt)
  unsigned long long *cur_dt, *nxt_dt, *cur_smax, *nxt_smax;
  int *cur_active, *nxt_active;
  int *fin;
  SweParamsDev prm;
  PipeCtl *ctl;
};
// Group and patch bookkeeping between two pipelined launches: the swept
// step's dt, activity and max speeds become the updated step's, its dt is
// recorded (hist[(k - 1) * n_groups + g] while k - 1 < hist_cap) and the
// group times advance; the next step's dt caps, activity and max speeds are
// reset; counters and the queue head are zeroed.
struct PipePreDev {
  int n_groups, n_patches;
  const double *group_max_dt, *group_t_end;
  double *group_time;
  unsigned long long *cur_dt, *nxt_dt, *cur_smax, *nxt_smax;
  int *cur_active, *nxt_active;
  double *hist;
  int hist_cap;
  int *cnt;
  PipeCtl *ctl;
};
cudaError_t launch_pipeline_pre(cudaStream_t st, const PipePreDev &A);
// Per-item time factors and strides of the ghost fill of step k (k <
// steps), from the time intervals the update of step k - 1 will leave (a
// leaf of a group that advanced by dt > 0: time + previous dt, dt), the same
// arithmetic as the update's; launched after k_pipeline_pre.
struct PipeItemsDev {
  const PatchDev *patches;
  const PatchTimeDev *times;
  const GhostItemDev *items;
  int n_items;
  const unsigned long long *cur_dt;
  const int *cur_active;
  GhostItemStepDev *item_step;
  const PipeCtl *ctl;
};
cudaError_t launch_pipeline_items(cudaStream_t st, const PipeItemsDev &A);
cudaError_t launch_pipeline_step(cudaStream_t st, int variant, int grid, const PipeDev &A);
cudaError_t pipeline_occupancy(int variant, int *blocks_per_sm);

}  // namespace pcg
