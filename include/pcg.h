/*
 * pcg.h -- C ABI of the GB300 SWE patch-update library (libpcg.so).
 *
 * The library is a drop-in for PeanoClaw's SWE numerics plugin: the host-side
 * spacetree traversal keeps calling the peanoclaw::Numerics interface
 * (src/peanoclaw/Numerics.h:30-204 in the reference); each virtual of that
 * interface maps onto one entry point below, and every patch's data vector
 * (h, hu, hv + ghost layers, the bathymetry parameter b and the face fluxes,
 * in the reference's LinearizationZYXQ layout) stays resident in HBM.
 *
 * Conventions
 *  - Every function returns PCG_OK (0) or a negative PCG_E_* code; the text of
 *    the last error of the calling thread is returned by pcg_last_error().
 *    No C++ exception crosses this boundary.
 *  - Patches are named by the int32 id that pcg_patch_alloc returns.
 *  - All floating point data is IEEE double (FP64).
 *  - Work is issued on the context's CUDA stream; calls that return values to
 *    the host synchronise that stream.
 */
#ifndef PCG_H
#define PCG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PCG_OK 0
#define PCG_E_INVALID (-1)   /* bad argument, unknown id, unsupported shape */
#define PCG_E_NOMEM (-2)     /* device memory (slab) exhausted: admission refused */
#define PCG_E_CUDA (-3)      /* a CUDA runtime call failed */
#define PCG_E_TIMEOUT (-4)   /* a bounded device-side wait ran out */
#define PCG_E_STATE (-5)     /* call not allowed in the current state */
#define PCG_E_NUMERIC (-6)   /* NaN or negative water height detected */

typedef struct pcg_context pcg_context;

/* SWE solver parameters.  The reference block's constants
 * (tools/SWE_WaveAccumulationBlock.cpp:225-239,270-284) are cfl = 0.4,
 * dry_tol_update = 0.1, s_min = 1e-5, dt_inf = FLT_MAX. */
typedef struct pcg_swe_params {
  double g;
  double cfl;
  double dry_tol;        /* Riemann solver: a cell is wet iff h > dry_tol */
  double dry_tol_update; /* updateUnknowns: h < this zeroes hu and hv */
  double s_min;          /* max wave speed <= s_min gives dt = dt_inf */
  double dt_inf;
} pcg_swe_params;

typedef struct pcg_config {
  int32_t device;          /* CUDA device ordinal */
  int32_t max_patches;     /* capacity of the patch table */
  int32_t max_groups;      /* independent simulations advanced together */
  int32_t reserved_;
  int64_t slab_doubles;    /* HBM slab for all patch vectors, in doubles */
  pcg_swe_params params;
} pcg_config;

/* Geometry and layout of one patch (peanoclaw::Patch / CellDescription,
 * src/peanoclaw/Patch.cpp:201-280). */
typedef struct pcg_patch_desc {
  int32_t nx, ny;      /* subdivision factor */
  int32_t ghost;       /* ghost layer width */
  int32_t nq;          /* unknowns per subcell */
  int32_t np_wo;       /* parameter fields without ghost layer */
  int32_t np_w;        /* parameter fields with ghost layer */
  int32_t level;
  int32_t flags;       /* PCG_PATCH_LEAF | PCG_PATCH_VIRTUAL */
  double pos[2];
  double size[2];
} pcg_patch_desc;

#define PCG_PATCH_LEAF 1
#define PCG_PATCH_VIRTUAL 2

/* TimeIntervals state of one patch (src/peanoclaw/grid/TimeIntervals.cpp). */
typedef struct pcg_patch_time {
  double time;               /* current time (uOld time of a leaf) */
  double dt;                 /* size of the last step (uNew = time + dt) */
  double est_next;           /* estimated next timestep size (CFL) */
  double min_neighbor_time;  /* uOld time of a virtual patch */
  double max_neighbor_dt;    /* uNew - uOld of a virtual patch */
  double restr_lower[2];     /* neighbouring ghost-layer bounds used by */
  double restr_upper[2];     /* restrictSolution(onlyOverlapped)        */
} pcg_patch_time;

/* One ghost-layer transfer of a precomputed face-pair list: the arguments of
 * Numerics::transferGhostlayer (kind COPY) or of the SWE interpolateSolution
 * the compositor issues from a coarse leaf (kind INTERP: toUOld, not current
 * time, time of uNew/uOld), see GhostlayerCompositorFunctors.cpp:23-221. */
typedef struct pcg_ghost_item {
  int32_t kind;
  int32_t src, dst;
  int32_t size[2];
  int32_t src_offset[2];
  int32_t dst_offset[2];
} pcg_ghost_item;

#define PCG_GHOST_COPY 0
#define PCG_GHOST_INTERP 1

/* Execution forms of a synchronous grid step. */
#define PCG_MODE_PLAIN 0    /* one launch per patch (per phase in the unfused step form) */
#define PCG_MODE_BATCHED 1  /* all patches in shared launches, replayed from a CUDA graph */

/* ---------------------------------------------------------------- context */

/* Create a context on cfg->device; reserves the patch slab.
 * Replaces the construction through NumericsFactory::createSWENumerics
 * (src/peanoclaw/NumericsFactory.cpp:28-51). */
int pcg_create(const pcg_config *cfg, pcg_context **out);
int pcg_destroy(pcg_context *ctx);
const char *pcg_last_error(void);
/* Free and total bytes of the slab (for admission by free HBM). */
int pcg_slab_info(pcg_context *ctx, int64_t *free_doubles, int64_t *total_doubles);
int pcg_set_params(pcg_context *ctx, const pcg_swe_params *params);

/* ---------------------------------------------------------------- patches */

/* Allocate a patch vector in the slab, zero-filled like Patch::switchToVirtual
 * (src/peanoclaw/Patch.cpp:732-776).  Returns PCG_E_NOMEM when it does not fit. */
int pcg_patch_alloc(pcg_context *ctx, const pcg_patch_desc *desc, int32_t *id);
int pcg_patch_free(pcg_context *ctx, int32_t id);
/* Number of doubles of a patch vector in the reference layout. */
int64_t pcg_patch_vector_size(const pcg_patch_desc *desc);
/* Host <-> device copy of the whole patch vector (reference layout). */
int pcg_patch_upload(pcg_context *ctx, int32_t id, const double *vec, int64_t n);
int pcg_patch_download(pcg_context *ctx, int32_t id, double *vec, int64_t n);
/* Contiguous multi-patch copies: vecs holds the vectors of ids[0..n) back to back. */
int pcg_patches_upload(pcg_context *ctx, int32_t n, const int32_t *ids, const double *vecs);
int pcg_patches_download(pcg_context *ctx, int32_t n, const int32_t *ids, double *vecs);
int pcg_patch_set_desc_flags(pcg_context *ctx, int32_t id, int32_t flags);
int pcg_patch_set_time(pcg_context *ctx, int32_t id, const pcg_patch_time *t);
int pcg_patch_get_time(pcg_context *ctx, int32_t id, pcg_patch_time *t);
/* Domain-boundary faces of a patch: bit (2*dim + upper); filled as reflecting
 * walls in the order of SolveTimestep::fillBoundaryLayers
 * (src/peanoclaw/mappings/SolveTimestep.cpp:87-142). */
int pcg_patch_set_boundary(pcg_context *ctx, int32_t id, uint32_t wall_mask);
/* Group (independent simulation) the patch belongs to; default 0. */
int pcg_patch_set_group(pcg_context *ctx, int32_t id, int32_t group);

/* ------------------------------------------- Numerics virtuals, one launch each */

/* DefaultTransfer::copyUNewToUOld (DefaultTransfer.cpph:103-113). */
int pcg_copy_unew_to_uold(pcg_context *ctx, int32_t id);
/* DefaultTransfer::swapUNewAndUOld (DefaultTransfer.cpph:115-127): the
 * interior values of uNew and uOld trade places. */
int pcg_swap_unew_and_uold(pcg_context *ctx, int32_t id);
/* SWEKernel::fillBoundaryLayer (src/peanoclaw/native/SWEKernel.cpp:176-237). */
int pcg_fill_boundary_layer(pcg_context *ctx, int32_t id, int32_t dimension, int32_t set_upper);
/* SWEKernel::solveTimestep (src/peanoclaw/native/SWEKernel.cpp:125-167):
 * f-wave sweep on uOld(+ghost), dt = min(block dt, max_dt), update, swap,
 * time-interval update.  Synchronous: returns the dt used and the estimate. */
int pcg_solve_timestep(pcg_context *ctx, int32_t id, double max_dt, double *dt_used,
                       double *est_next);
/* Numerics::transferGhostlayer -> DefaultTransfer (DefaultTransfer.cpph:15-101). */
int pcg_transfer_ghostlayer(pcg_context *ctx, const int32_t size[2], const int32_t src_offset[2],
                            const int32_t dst_offset[2], int32_t src, int32_t dst);
/* SWEKernel::interpolateSolution (SWEKernel.cpp:239-286) over
 * DefaultInterpolation (DefaultInterpolation.cpph:29-270); swe = 0 gives the
 * plain Numerics::interpolateSolution. */
int pcg_interpolate_solution(pcg_context *ctx, const int32_t size[2], const int32_t dst_offset[2],
                             int32_t src, int32_t dst, int32_t to_uold, int32_t to_current_time,
                             int32_t use_time_unew_or_uold, int32_t swe);
/* n interpolations with the same flags in one launch: size[2k], dst_offset[2k]
 * and src[k] -> dst[k] as in pcg_interpolate_solution.  The destinations
 * must be distinct and none may be a source (the items run concurrently);
 * Remesh::createCell initialises every new fine patch this way
 * (Remesh.cpp:399-420). */
int pcg_interpolate_solution_many(pcg_context *ctx, int32_t n, const int32_t *src, const int32_t *dst,
                                  const int32_t *size, const int32_t *dst_offset, int32_t to_uold,
                                  int32_t to_current_time, int32_t use_time_unew_or_uold, int32_t swe);
/* SWEKernel::restrictSolution (SWEKernel.cpp:288-307) over DefaultRestriction
 * (DefaultRestriction.cpph:17-150); swe = 0 gives Numerics::restrictSolution. */
int pcg_restrict_solution(pcg_context *ctx, int32_t src, int32_t dst, int32_t only_overlapped,
                          int32_t swe);
/* SWEKernel::postProcessRestriction (SWEKernel.cpp:309-316). */
int pcg_post_process_restriction(pcg_context *ctx, int32_t dst);
/* Numerics::computeFluxes -> DefaultFluxCorrection::computeFluxes
 * (DefaultFluxCorrection.cpph:43-85); g_flux is the constant of
 * Numerics::computeFlux (1.0 in the reference, Numerics.h:198). */
int pcg_compute_fluxes(pcg_context *ctx, int32_t id, double g_flux);
/* Numerics::applyFluxCorrection -> DefaultFluxCorrection::applyCorrection
 * (DefaultFluxCorrection.cpph:87-164). */
int pcg_apply_flux_correction(pcg_context *ctx, int32_t src, int32_t dst, int32_t dimension,
                              int32_t direction);

/* ----------------------------------------------------------------- remesh */

/* Patch::getAccessor().clearRegion of uNew and the uOld interior (what
 * GridLevelTransfer::switchToAndAddVirtualSubgrid does to a virtual patch
 * before its children restrict into it); used before a full restriction when
 * a refined patch coarsens. */
int pcg_clear_subgrid(pcg_context *ctx, int32_t id);
/* Host-side list builder of an adaptive grid of n x n patches with 3x
 * refinement (level l: (base * 3^l)^2 slots on [0,1]^2; no device work).
 * The np slots (lvl, si, sj) in patch order (level, then i, then j ascending),
 * refined[k] != 0 for a virtual (refined) slot, give: the ghost face pairs
 * (items, up to 8 np rows of pcg_ghost_item fields: kind, src, dst, size,
 * src_offset, dst_offset; copies between slots of one level, interpolation
 * from the nearest existing coarser slot, GhostlayerCompositorFunctors.cpp),
 * the flux-correction pairs (flux, up to 4 np rows: fine leaf, coarse owner,
 * dim, dir), the restriction pairs (restr, up to levels np rows: leaf,
 * virtual ancestor whose ghost-layer bounds it overlaps, ordered by ancestor
 * then leaf, GridLevelTransfer::restrictToOverlappingVirtualSubgrids), the
 * bounds lower[2 np] / upper[2 np] of every virtual slot
 * (GhostLayerCompositor::updateLower/UpperGhostlayerBound) and the wall
 * mask of every leaf on the domain boundary. */
int pcg_amr_layout(int32_t base, int32_t n, int32_t levels, int32_t np, const int32_t *lvl,
                   const int32_t *si, const int32_t *sj, const uint8_t *refined, int32_t *items,
                   int32_t *n_items, int32_t *flux, int32_t *n_flux, int32_t *restr, int32_t *n_restr,
                   double *lower, double *upper, int32_t *walls);
/* Patch::switchToLeaf (src/peanoclaw/Patch.cpp:793-816): the patch becomes a
 * leaf and its interior, restricted as values at the times 0 and 1 (the
 * reference's virtual-patch convention), is re-evaluated at the patch's time
 * (uOld) and time + dt (uNew).  Set the time interval first. */
int pcg_switch_to_leaf(pcg_context *ctx, int32_t id);
/* The BreakingDam refinement criterion of every listed patch
 * (BreakingDamSWEScenario::computeDemandedMeshWidth,
 * native/scenarios/BreakingDam.cpp:85-139): out[k] = max over interior
 * forward differences of |grad h| on uNew.  The scenario refines where it
 * exceeds 0.1 and coarsens where it is below. */
int pcg_refinement_indicator(pcg_context *ctx, int32_t n, const int32_t *ids, double *out);
/* The refinement criterion `kind` of every listed patch, one double per
 * patch (the scenario compares it with its threshold):
 *   PCG_CRIT_DEPTH_GRADIENT: as pcg_refinement_indicator (BreakingDam);
 *   PCG_CRIT_SURFACE_DIFFERENCE: max over interior forward differences of
 *     the surface h + b, not divided by the mesh width (BowlOcean's wave-front
 *     criterion, native/scenarios/BowlOcean.cpp:91-123, threshold 0.05);
 *   PCG_CRIT_SURFACE_GRADIENT: the BreakingDam stencil on the surface h + b
 *     (forward differences divided by the subcell size): a still lake over
 *     any bathymetry gives 0, a wave or a wet/dry coastline does not.
 * The surface criteria read b (the first parameter with ghost layer). */
#define PCG_CRIT_DEPTH_GRADIENT 0
#define PCG_CRIT_SURFACE_DIFFERENCE 1
#define PCG_CRIT_SURFACE_GRADIENT 2
int pcg_refinement_criterion(pcg_context *ctx, int32_t n, const int32_t *ids, int32_t kind, double *out);

/* ----------------------------------------------------------------- output */

/* No counterpart in the reference (its plotters read the Peano heap on the
 * host).  Gathers, for every listed patch back to back, uNew (nq planes) and
 * the interior of the parameters with ghost layer (np_w planes), each plane
 * nx*ny values in the layout's x-major order, in one device pass and one copy
 * to `out`; out_len must be sum over the patches of (nq + np_w) * nx * ny. */
int pcg_gather_cells(pcg_context *ctx, int32_t n, const int32_t *ids, double *out, int64_t out_len);
/* Time intervals of the listed patches in one call. */
int pcg_patches_get_time(pcg_context *ctx, int32_t n, const int32_t *ids, pcg_patch_time *out);
/* Time records of the listed patches in one call (pcg_patch_set_time for
 * each); ids must be distinct. */
int pcg_patches_set_time(pcg_context *ctx, int32_t n, const int32_t *ids, const pcg_patch_time *in);
/* Neighbouring ghost-layer bounds (restr_lower / restr_upper of
 * pcg_patch_time) of the listed patches in one call: lower[2k], lower[2k+1],
 * upper[2k], upper[2k+1] for ids[k]; the other time fields are kept.  The
 * reference accumulates these bounds per virtual patch during the traversal
 * (GhostLayerCompositor::updateLower/UpperGhostlayerBound,
 * GhostLayerCompositor.cpp:177-259); ids must be distinct. */
int pcg_patches_set_restriction_bounds(pcg_context *ctx, int32_t n, const int32_t *ids, const double *lower,
                                       const double *upper);

/* ------------------------------------------------------ batched grid step */

/* Install the precomputed face-pair list used by every following grid step
 * (replaces the per-vertex GhostLayerCompositor traversal,
 * GhostLayerCompositor.cpp:280-320).  Items must write disjoint ghost cells. */
int pcg_set_ghost_items(pcg_context *ctx, const pcg_ghost_item *items, int32_t n);
/* Restriction into virtual (refined) patches, run after the update of every
 * grid step: each destination's uNew and uOld interior is cleared
 * (GridLevelTransfer::switchToAndAddVirtualSubgrid), then
 * SWEKernel::restrictSolution(src[k], dst[k], only_overlapped) runs in list
 * order per destination (GridLevelTransfer::restrictToOverlappingVirtualSubgrids,
 * GridLevelTransfer.cpp:140-210), then SWEKernel::postProcessRestriction on
 * every destination (finalizeVirtualSubgrid, :212-275). */
int pcg_set_restriction_items(pcg_context *ctx, int32_t n, const int32_t *src, const int32_t *dst,
                              int32_t only_overlapped);
/* Flux correction after the update of every grid step: computeFluxes of every
 * leaf of the groups that the list's patches belong to (g_flux as in
 * Numerics::computeFlux; a group without items is a simulation without flux
 * correction and its flux areas are not written), then
 * applyFluxCorrection(src[k], dst[k], dim[k], dir[k]) in list order per
 * destination (SolveTimestep.cpp:674-679, FluxCorrectionFunctor). */
int pcg_set_flux_correction_items(pcg_context *ctx, int32_t n, const int32_t *src, const int32_t *dst,
                                  const int32_t *dim, const int32_t *dir, double g_flux);
/* Run the restriction list once (fills the virtual patches at start-up). */
int pcg_restrict_all(pcg_context *ctx);
/* Upper bound for the dt of a group (maximumTimestepSize). */
int pcg_set_group_max_dt(pcg_context *ctx, int32_t group, double max_dt);
/* No counterpart in the reference (its driver stops evolveToTime at the end
 * time).  Sets the group's time to `time` and its end time to `t_end`
 * (+inf, the default, means none).  Every following step caps the group's dt
 * at max(0, t_end - time) and adds the dt taken to its time on the device; a
 * group whose time has reached t_end is inactive: ghost fill, walls, sweep,
 * update and the flux/restriction phases skip its patches and its state and
 * time intervals stay unchanged, so many steps can be replayed (pcg_run)
 * while groups finish at different steps. */
int pcg_set_group_end_time(pcg_context *ctx, int32_t group, double time, double t_end);
/* times[max_groups] receives every group's time (see pcg_set_group_end_time). */
int pcg_get_group_times(pcg_context *ctx, double *times);
/* One synchronous step of every leaf patch: fill ghost layers (items, then
 * walls), f-wave sweep with per-patch CFL, dt_g = min(max_dt_g, min over the
 * group's patches), update with dt_g, swap, time update.  dt_out (may be NULL)
 * receives max_groups values. */
int pcg_step(pcg_context *ctx, int32_t mode, double *dt_out);
/* `steps` synchronous steps; BATCHED mode replays a captured CUDA graph.  The
 * dt of every step and group is written to dt_hist[steps * max_groups] (may be NULL). */
int pcg_run(pcg_context *ctx, int32_t steps, int32_t mode, double *dt_hist);
/* No counterpart in the reference.  pcg_run in two halves: pcg_run_async
 * enqueues the run (steps >= 1) and returns; pcg_run_wait waits for it and
 * does what pcg_run does after its launches (the dt record, the error words
 * of bounded waits, the statistics).  In between the host may call the
 * other entry points: their device work is ordered after the run on the
 * context's stream (a call that reads device data waits for the run);
 * pcg_run, pcg_run_async, pcg_step, pcg_autotune, pcg_profile_step and
 * pcg_set_time_stepping return PCG_E_STATE until pcg_run_wait. */
int pcg_run_async(pcg_context *ctx, int32_t steps, int32_t mode);
int pcg_run_wait(pcg_context *ctx, double *dt_hist);
/* No counterpart in the reference (its block applies the update right after
 * the sweep).  Step forms of pcg_step / pcg_run:
 *   PCG_FORM_AUTO (default): the fused form wherever it applies -- the
 *     synchronous step without restriction or flux-correction lists, every
 *     ghost item between leaves with one ghost layer, and (BATCHED) the
 *     warp-strip schedule.  One kernel per step fills each strip's ghost
 *     cells from its neighbours, applies the previous step's update to every
 *     cell it reads, sweeps and reduces the CFL dt; two small launches
 *     advance the time intervals and prepare the next step (the PLAIN form:
 *     the fused kernel once per patch).  The update of the last step stays
 *     pending in device memory until a call that reads or changes patch data,
 *     lists or parameters applies it, so the reference layout a download
 *     returns is the same as after unfused steps, bit for bit.
 *   PCG_FORM_UNFUSED: separate launches for ghost fill, walls, sweep and update.
 * The form never changes results. */
#define PCG_FORM_AUTO 0
#define PCG_FORM_UNFUSED 1
int pcg_set_step_form(pcg_context *ctx, int32_t form);
/* *fused = 1 if a step of `mode` takes the fused form with the current lists. */
int pcg_get_step_form(pcg_context *ctx, int32_t mode, int32_t *fused);
/* No counterpart in the reference.  *launches = the kernel launches one
 * batched step issues: the kernel nodes of the CUDA graph that pcg_run last
 * captured (0 before the first batched pcg_run or after the lists changed). */
int pcg_get_step_launches(pcg_context *ctx, int32_t *launches);
/* Cumulative interior cell updates and device time of pcg_step / pcg_run;
 * under local time stepping the cells of the leaves that advanced. */
int pcg_stats(pcg_context *ctx, int64_t *cell_updates, double *device_ms);
/* Block until all work issued on the context has finished. */
int pcg_synchronize(pcg_context *ctx);

/* ----------------------------------------------------- local time stepping */

/* Replaces the reference's adaptive (local) time stepping of SolveTimestep:
 * a leaf advances in a grid iteration when its end time is not reached and
 * its uNew time does not lie ahead of the minimal uNew time of its ghost
 * sources by more than the time tolerance (TimeIntervals.cpp:24-99,
 * isAllowedToAdvanceInTime / isBlockedByNeighbors).  With PCG_TS_LOCAL every
 * BATCHED pcg_step / pcg_run iteration decides which leaves advance (on the
 * device, from the times before the iteration), fills the ghost layers of
 * those leaves only (time-interpolated from their sources,
 * DefaultTransfer.cpph:27-50), and solves each of them with its own dt =
 * min(block CFL dt, group max_dt, end time - uNew time) (SolveTimestep.cpp:
 * 591-700).  A source's time constraint is its time + dt
 * (TimeIntervals::getTimeConstraint); before the decision every virtual
 * patch of the pcg_set_virtual_time_items list takes the intersection of
 * its leaves' time intervals, and after the update the restriction list
 * (pcg_set_restriction_items) refills the virtual patches, so coarse leaves
 * next to a refined region wait for its finest leaves and read their data
 * through the virtual patches (GridLevelTransfer.cpp:108-275).  The recorded
 * dt of a group is the minimal dt taken by its leaves in the iteration (0 if
 * none advanced); its time (pcg_get_group_times) becomes the minimal uNew
 * time of its leaves.  The end time of pcg_set_group_end_time bounds every
 * leaf.  Local time stepping runs in the BATCHED form only and takes no
 * flux-correction list (PCG_E_STATE otherwise); PCG_TS_GLOBAL (default) is
 * the synchronous step. */
#define PCG_TS_GLOBAL 0
#define PCG_TS_LOCAL 1
int pcg_set_time_stepping(pcg_context *ctx, int32_t mode);
/* (leaf[k], virt[k]) pairs, each leaf against every virtual ancestor: in
 * local time stepping each listed virtual patch's time interval becomes,
 * before every iteration, time = the maximal time of its leaves and dt =
 * their minimal time + dt minus that time (GridLevelTransfer::stepUp,
 * GridLevelTransfer.cpp:408-431; TimeIntervals::updateMinimalFineGridTimeInterval,
 * TimeIntervals.cpp:214-231; Patch.cpp:388-397).  Unused by the synchronous
 * step.  PCG_E_STATE at the next step if a pair does not join a leaf to a
 * non-leaf patch. */
int pcg_set_virtual_time_items(pcg_context *ctx, int32_t n, const int32_t *leaf, const int32_t *virt);

/* --------------------------------------------- batched schedule + autotuner */

/* No counterpart in the reference (its block sweep is one loop nest).  How the
 * BATCHED sweep and update map patches onto the GPU; every schedule computes
 * bit-identical results.
 *   kind 0: one 16x16 tile of a patch per CTA iteration (256 threads);
 *           variant 0 stages the tile + halo with per-thread loads,
 *           variant 1 with tensor copies (TMA: cp.async.bulk.tensor of the
 *           uNew, uOld and bathymetry boxes, per-patch tensor maps); variant 1
 *           needs leaves of even size, ghost width 1, 3 unknowns and the
 *           bathymetry as the only parameter field (PCG_E_INVALID at the
 *           step otherwise);
 *   kind 1: warp strips: a warp marches strips of up to 32 rows and `chunk`
 *           columns (1..32) of one or more patches along x; `variant` picks
 *           the CTA size / register budget (0..4: 4 warps x 4 CTAs/SM,
 *           4 x 5, 8 x 2, 8 x 3, 6 x 3). */
typedef struct pcg_schedule {
  int32_t kind;
  int32_t variant;
  int32_t chunk;
  int32_t unfused;   /* strips: 1 = the unfused step form even where the fused one applies;
                        2 = pcg_run in the pipelined form where it applies (the synchronous
                        step without restriction or flux-correction lists, PCG_FORM_AUTO):
                        per step a bookkeeping launch, a launch of the ghost items' time
                        factors and one persistent kernel that updates step k - 1 and
                        fills, walls and sweeps step k, its work items ordered by
                        per-patch counters (waits limited to 0.2 s: PCG_E_CUDA and an
                        incomplete run if one runs out); a run of K steps is K + 1 such
                        launch triples; pcg_step takes the unfused form */
} pcg_schedule;
#define PCG_SCHED_TILES 0
#define PCG_SCHED_STRIPS 1
/* Fix the schedule of the context (overrides any tuned choice). */
int pcg_set_schedule(pcg_context *ctx, const pcg_schedule *s);
int pcg_get_schedule(pcg_context *ctx, pcg_schedule *s);
/* Autotuner: runs `reps` BATCHED steps with each candidate schedule (tiles,
 * also with TMA staging where the leaves allow it;
 * strips x 5 variants x chunk 32 / 16 and variants 0, 2 x chunk 10 / 8, in the fused step form where it
 * applies; then the fastest strip schedule in the unfused form, and in the
 * pipelined form as one run of `reps` steps), times each candidate's steps with
 * CUDA events, keeps the fastest for this context and caches it for the
 * process under the key (SM count, histogram of leaf patch shapes), so later
 * contexts with the same patch mix start with it.  The simulation advances by
 * reps x n_candidates steps (each group by its own dt, as in pcg_step); the
 * patch time intervals record them.  tried[cap] / ms[cap] (may be NULL)
 * receive the candidates and their mean step time; *n_tried their number. */
int pcg_autotune(pcg_context *ctx, int32_t reps, pcg_schedule *tried, double *ms, int32_t cap,
                 int32_t *n_tried);

/* ----------------------------------------------------------- diagnostics */

/* No counterpart in the reference.  One BATCHED step with CUDA events between
 * its phases on the context stream; ms[5] receives the device time of
 * reset, ghost items, walls, sweep and update.  In the fused form the ghost
 * fill, walls and update are inside the sweep launch: ms[1] = ms[2] = 0,
 * ms[3] is the fused kernel, ms[4] the time advance, ms[0] the reset and
 * item factors of the next step.  In the pipelined form (schedule field
 * unfused = 2) a run of two steps is timed: ms[3] its middle step kernel
 * (update of the first step, fill, walls and sweep of the second), ms[0]
 * the two launches before it, ms[1] the first step kernel (fill, walls and
 * sweep only), ms[2] the last (update only), ms[4] = 0; the simulation
 * advances by two steps. */
int pcg_profile_step(pcg_context *ctx, double *ms);
/* No counterpart in the reference.  Measures the FP64 FMA throughput of the
 * context's device (dependent-chain loop on every SM); returns TFLOP/s with an
 * FMA counted as two flops. */
int pcg_probe_fp64_peak(pcg_context *ctx, double *tflops);
/* No counterpart in the reference.  Self-test of the level transfer's bounded
 * waits (the wait of the restriction items for the flux corrections): runs
 * the restriction items once with a wait that nothing can satisfy; every
 * wait runs out after its spin limit (about 0.1 s), sets the error word and
 * skips its item, so no patch data changes.  Returns PCG_OK when the host
 * read the error back (and reset it), PCG_E_STATE otherwise; the context
 * stays usable.  Needs a restriction list (PCG_E_STATE without one). */
int pcg_selftest_transfer_wait(pcg_context *ctx);
/* No counterpart in the reference.  Compares the library's integer-pipe FP64
 * divide, reciprocal and square root with the hardware IEEE operations on `samples`
 * pseudo-random operand pairs; *mismatches receives the number of results
 * whose bits differ (0 expected). */
int pcg_check_ieee_emulation(pcg_context *ctx, int64_t samples, uint64_t seed, int64_t *mismatches);

/* ----------------------------------------------------- allocation-free solve */

/* No counterpart in the reference.  SWEKernel::solveTimestep for one patch
 * without a context and without any device allocation, for callers that cannot
 * call cudaMalloc (a thread working on a patch buffer owned by another
 * component, or a process whose device memory belongs to another framework's
 * pool).  d_vector is the patch vector in device memory (reference layout,
 * ghost width 1, 3 unknowns, b with ghost layer), nx*ny <= 16384 (128 x 128),
 * larger patches are rejected with PCG_E_INVALID.  dt_used / est_next (host,
 * may be NULL) receive the dt taken and the CFL estimate; the caller keeps the
 * time intervals.  stream: a cudaStream_t (NULL = default stream).
 * Scratch is a fixed 393 KB array inside the library, held by every GPU that
 * loads it until exit and shared by all calls: calls that overlap on the GPU
 * race.  The first call in a device's context resolves that array's device
 * address (a set-up done again after the context was destroyed and created
 * anew, e.g. by cudaDeviceReset); make that first call before any stream
 * capture (PCG_E_STATE otherwise).  Calls made while `stream` is being
 * captured must pass NULL for dt_used and est_next, whose read-back copies
 * and synchronises the stream (PCG_E_INVALID otherwise). */
int pcg_solve_timestep_noalloc(double *d_vector, int32_t nx, int32_t ny, const double size[2],
                               const pcg_swe_params *params, double max_dt, double *dt_used,
                               double *est_next, void *stream);

#ifdef __cplusplus
}
#endif
#endif
