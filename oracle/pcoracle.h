/*
 * pcoracle.h -- CPU restatement of PeanoClaw's SWE patch-update path (FP64).
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the oracle that the CUDA path is
 * checked against.  Only the test suite, the smoke check and the CPU-baseline
 * leg of the benchmark may load it; the product library never links it and
 * never falls back to it.
 *
 * Every function restates one piece of the reference (file:line given at the
 * definition).  Where the reference calls third-party code that is not in the
 * reference tree (the TUM SWE f-wave Riemann solver), the function restates the
 * published method instead and says so.
 *
 * Arithmetic contract: the oracle is compiled with -ffp-contract=off; every
 * fused multiply-add is an explicit fma() call.  The CUDA kernels issue the
 * same IEEE operations in the same order, so results agree bit for bit.
 */
#ifndef PCORACLE_H
#define PCORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* One subgrid ("patch"), mirroring peanoclaw::Patch + its CellDescription
 * fields that the hot path reads (src/peanoclaw/Patch.h:135-516,
 * src/peanoclaw/dastgen/CellDescription.def:11-200).  `u` points at the
 * patch's data vector in the reference layout
 * (src/peanoclaw/grid/LinearizationZYXQ.h:20-88):
 *   [uNew  nq*nx*ny][uOld+ghost nq*(nx+2g)*(ny+2g)][params w/o ghost np_wo*nx*ny]
 *   [params with ghost np_w*(nx+2g)*(ny+2g)][fluxes 2*nq*(nx+ny)]
 * with index (q, x, y) -> q*qStride + x*cellStrideX + y  (y fastest). */
typedef struct pco_patch {
  int32_t nx, ny;          /* subdivision factor */
  int32_t ghost;           /* ghost layer width */
  int32_t nq;              /* unknowns per subcell */
  int32_t np_wo, np_w;     /* parameter fields without / with ghost layer */
  int32_t level;
  int32_t is_leaf, is_virtual;
  int32_t pad_;
  double pos[2], size[2];
  double time, dt, est_next;               /* TimeIntervals of a leaf */
  double min_neighbor_time, max_neighbor_dt; /* TimeIntervals of a virtual patch */
  double restr_lower[2], restr_upper[2];   /* neighbouring ghost-layer bounds */
  double *u;
} pco_patch;

/* SWE solver parameters.  Defaults of the reference block
 * (tools/SWE_WaveAccumulationBlock.cpp:225-239,270-284): cfl 0.4,
 * dry_tol_update 0.1, s_min 1e-5, dt_inf = FLT_MAX. */
typedef struct pco_swe_params {
  double g;
  double cfl;
  double dry_tol;          /* Riemann solver: a cell is wet iff h > dry_tol */
  double dry_tol_update;   /* updateUnknowns: h < this zeroes momentum */
  double s_min;            /* wave speeds <= s_min give dt = dt_inf */
  double dt_inf;
} pco_swe_params;

/* One ghost-layer transfer between two patches, as issued by the
 * GhostLayerCompositor functors
 * (src/peanoclaw/interSubgridCommunication/GhostlayerCompositorFunctors.cpp:23-221). */
typedef struct pco_ghost_item {
  int32_t kind;            /* 0: transferGhostlayer, 1: SWE interpolateSolution(toUOld, !current, useTimeUNewOrUOld) */
  int32_t src, dst;
  int32_t size[2];
  int32_t src_offset[2];
  int32_t dst_offset[2];
} pco_ghost_item;

enum { PCO_GHOST_COPY = 0, PCO_GHOST_INTERP = 1 };

/* ---- layout ---- */
int64_t pco_patch_vector_size(const pco_patch *p);
int64_t pco_idx_unew(const pco_patch *p, int q, int x, int y);
int64_t pco_idx_uold(const pco_patch *p, int q, int x, int y);
int64_t pco_idx_param_w(const pco_patch *p, int k, int x, int y);
int64_t pco_idx_flux(const pco_patch *p, int q, int c, int dim, int dir);

/* ---- time intervals (src/peanoclaw/grid/TimeIntervals.cpp:102-133) ---- */
double pco_time_uold(const pco_patch *p);
double pco_time_unew(const pco_patch *p);

/* ---- the f-wave edge solve (published method; see pcoracle.c) ---- */
void pco_fwave_edge(const pco_swe_params *prm,
                    double hL, double huL, double bL,
                    double hR, double huR, double bR,
                    double out[5]);

/* ---- SWE kernel (src/peanoclaw/native/SWEKernel.cpp) ---- */
void pco_copy_unew_to_uold(pco_patch *p);
void pco_swap_unew_uold(pco_patch *p);
void pco_swe_fill_boundary_layer(pco_patch *p, int dimension, int set_upper);
/* computeNumericalFluxes on uOld(+ghost): fills net (3*(nx+2)*(ny+2), block
 * layout) and returns the block's maxTimestep. */
double pco_swe_compute_net_updates(const pco_patch *p, const pco_swe_params *prm,
                                   double *net, double *max_speed);
void pco_swe_update_unknowns(pco_patch *p, const pco_swe_params *prm,
                             const double *net, double dt);
/* SWEKernel::solveTimestep (uOld must already hold uNew + ghost layers). */
void pco_swe_solve_timestep(pco_patch *p, const pco_swe_params *prm,
                            double max_dt, double *dt_used, double *est_next);

/* ---- Default* strategies (generic number of unknowns) ---- */
void pco_transfer_ghostlayer(const int size[2], const int src_off[2], const int dst_off[2],
                             const pco_patch *src, pco_patch *dst);
void pco_interpolate(const int dst_size[2], const int dst_off[2],
                     const pco_patch *src, pco_patch *dst,
                     int to_uold, int to_current_time, int use_time_unew_or_uold,
                     int swe_absolute_height);
void pco_restrict(const pco_patch *src, pco_patch *dst, int only_overlapped,
                  int swe_absolute_height);
void pco_swe_post_process_restriction(pco_patch *dst);
/* Patch::switchToLeaf data conversion (src/peanoclaw/Patch.cpp:793-816 with
 * switchRegionToMinimalFineGridTimeInterval, :55-76): a virtual patch holds
 * its restricted values at the times 0 and 1; the interior is re-evaluated at
 * the patch's time (uOld) and time + dt (uNew); the patch becomes a leaf. */
void pco_switch_to_leaf(pco_patch *p);
void pco_compute_fluxes(pco_patch *p, double g_flux);
void pco_apply_flux_correction(const pco_patch *src, pco_patch *dst, int dim, int dir);

/* ---- geometry (src/peanoclaw/geometry/Region.cpp) ---- */
void pco_region_map_to_patch(const int off[2], const int size[2],
                             const pco_patch *src, const pco_patch *dst, double eps,
                             int out_off[2], int out_size[2]);
int pco_regions_overlapped_by_ghostlayers(const double lower[2], const double upper[2],
                                          const double src_pos[2], const double src_size[2],
                                          const double src_sub[2], const int n[2],
                                          int out_off[8], int out_size[8]);
double pco_overlap_area(const double p1[2], const double s1[2],
                        const double p2[2], const double s2[2]);

/* ---- synchronous grid step (the semantics of the batched GPU form) ----
 * fill ghost layers (items in order, then walls), compute every leaf patch's
 * net updates and own CFL dt, dt = min(max_dt, min over the patches of each
 * group), update every leaf patch with its group's dt.  wall_mask bit (2*dim+upper). */
/* One local-time-stepping grid iteration (see pcoracle.c). */
int pco_grid_step_lts(pco_patch **patches, int n_patches, const pco_ghost_item *items, int n_items,
                      const uint8_t *wall_mask, const pco_swe_params *prm, double max_dt,
                      double t_end, const int32_t *vt_leaf, const int32_t *vt_virt, int n_vt,
                      double *dt_out, int n_threads);
void pco_grid_step(pco_patch **patches, int n_patches,
                   const pco_ghost_item *items, int n_items,
                   const uint8_t *wall_mask, const int32_t *group, int n_groups,
                   const pco_swe_params *prm, const double *max_dt,
                   double *dt_out, int n_threads);
/* Ghost fill only (items in order, then walls in the reference order). */
void pco_grid_fill(pco_patch **patches, int n_patches,
                   const pco_ghost_item *items, int n_items,
                   const uint8_t *wall_mask);

/* Ghost items grouped by destination, in list order within each (counting
 * sort): *start_out receives n_patches + 1 offsets into the returned array of
 * item indices (both malloc'ed; the caller frees them).  NULL when some copy
 * item reads outside its source's interior: then an item may read cells that
 * another item writes, and only the list order is exact. */
int *pco_items_by_dst(pco_patch **patches, int n_patches, const pco_ghost_item *items, int n_items,
                      int **start_out);

/* ---- FP32 twin (pcoracle_f32.c): timing baseline at the reference's storage
 * precision, not a parity reference.  pco_grid_step for one group with float
 * patch vectors u[p] in the layout of patches[p] (whose own u is not used);
 * the time intervals in patches[p] are advanced; *dt_out = the dt taken. */
void pco32_grid_step(pco_patch **patches, float **u, int n_patches,
                     const pco_ghost_item *items, int n_items, const uint8_t *wall_mask,
                     const pco_swe_params *prm, double max_dt, double *dt_out, int n_threads);

#ifdef __cplusplus
}
#endif
#endif
