/*
 * pcoracle.c -- CPU restatement (FP64) of PeanoClaw's SWE patch-update path.
 *
 * TEST INFRASTRUCTURE ONLY: the oracle the CUDA kernels are checked against.
 * Compiled with -ffp-contract=off; fused multiply-adds are explicit fma().
 *
 * Citations are file:line within the reference project (www5sccs/peanoclaw).
 */
#include "pcoracle.h"

#include <float.h>
#include <limits.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* tarch::la comparison tolerance (Peano 3 tarch/la/Scalar.h, which is not part
 * of the reference tree: the value is not pinned by any file here). */
#define PCO_TARCH_EPS 1.0e-8

static int tl_greater(double a, double b) { return a - b > PCO_TARCH_EPS; }
static int tl_equals(double a, double b) { return fabs(a - b) <= PCO_TARCH_EPS; }
static int tl_greater_equals(double a, double b) { return a - b >= -PCO_TARCH_EPS; }

/* ------------------------------------------------------------------------ */
/* Layout: src/peanoclaw/grid/LinearizationZYXQ.h:20-88,                     */
/*         src/peanoclaw/grid/Linearization.h:125-200                        */
/* ------------------------------------------------------------------------ */
static int64_t vol_new(const pco_patch *p) { return (int64_t)p->nx * p->ny; }
static int64_t vol_old(const pco_patch *p) {
  return (int64_t)(p->nx + 2 * p->ghost) * (p->ny + 2 * p->ghost);
}
static int64_t base_uold(const pco_patch *p) { return p->nq * vol_new(p); }
static int64_t base_pwo(const pco_patch *p) { return base_uold(p) + p->nq * vol_old(p); }
static int64_t base_pw(const pco_patch *p) { return base_pwo(p) + p->np_wo * vol_new(p); }
static int64_t base_flux(const pco_patch *p) { return base_pw(p) + p->np_w * vol_old(p); }

int64_t pco_patch_vector_size(const pco_patch *p) {
  return base_flux(p) + 2LL * p->nq * (p->nx + p->ny);
}
int64_t pco_idx_unew(const pco_patch *p, int q, int x, int y) {
  return q * vol_new(p) + (int64_t)x * p->ny + y;
}
int64_t pco_idx_uold(const pco_patch *p, int q, int x, int y) {
  return base_uold(p) + q * vol_old(p) + (int64_t)(x + p->ghost) * (p->ny + 2 * p->ghost) + (y + p->ghost);
}
int64_t pco_idx_param_w(const pco_patch *p, int k, int x, int y) {
  return base_pw(p) + k * vol_old(p) + (int64_t)(x + p->ghost) * (p->ny + 2 * p->ghost) + (y + p->ghost);
}
/* Flux array of face (dim, dir): faceOffset[2*dim + (1+dir)/2] + c + q*qStrideFlux[dim],
 * qStrideFlux[0] = ny, qStrideFlux[1] = nx (LinearizationZYXQ.h:51-69). */
int64_t pco_idx_flux(const pco_patch *p, int q, int c, int dim, int dir) {
  int64_t qs0 = p->ny, qs1 = p->nx;
  int64_t face_off[4];
  face_off[0] = 0;
  face_off[1] = face_off[0] + qs0 * p->nq;
  face_off[2] = face_off[1] + qs0 * p->nq;
  face_off[3] = face_off[2] + qs1 * p->nq;
  return base_flux(p) + face_off[2 * dim + (1 + dir) / 2] + c + q * (dim == 0 ? qs0 : qs1);
}

#define UNEW(p, q, x, y) ((p)->u[pco_idx_unew((p), (q), (x), (y))])
#define UOLD(p, q, x, y) ((p)->u[pco_idx_uold((p), (q), (x), (y))])
#define PARW(p, k, x, y) ((p)->u[pco_idx_param_w((p), (k), (x), (y))])

static void subcell_size(const pco_patch *p, double h[2]) {
  /* Patch::fillCaches (src/peanoclaw/Patch.cpp:32-39): size / subdivision */
  h[0] = p->size[0] / (double)p->nx;
  h[1] = p->size[1] / (double)p->ny;
}
static void subcell_center(const pco_patch *p, int x, int y, double c[2]) {
  /* Patch::getSubcellCenter (src/peanoclaw/Patch.cpp:429-435):
   * position + subcellSize*index + subcellSize*0.5 */
  double h[2];
  subcell_size(p, h);
  c[0] = (p->pos[0] + h[0] * (double)x) + h[0] * 0.5;
  c[1] = (p->pos[1] + h[1] * (double)y) + h[1] * 0.5;
}
/* SubgridIterator::getCellPosition (src/peanoclaw/grid/SubgridAccessor.cpph:169-172):
 * position + index * (size * (1/subdivision)) */
static void iter_cell_position(const pco_patch *p, int x, int y, double c[2]) {
  double s0 = p->size[0] * (1.0 / (double)p->nx);
  double s1 = p->size[1] * (1.0 / (double)p->ny);
  c[0] = p->pos[0] + (double)x * s0;
  c[1] = p->pos[1] + (double)y * s1;
}

/* ------------------------------------------------------------------------ */
/* TimeIntervals (src/peanoclaw/grid/TimeIntervals.cpp:102-123)              */
/* ------------------------------------------------------------------------ */
double pco_time_uold(const pco_patch *p) {
  return p->is_leaf ? p->time : p->min_neighbor_time;
}
double pco_time_unew(const pco_patch *p) {
  return p->is_leaf ? p->time + p->dt : p->min_neighbor_time + p->max_neighbor_dt;
}

/* ------------------------------------------------------------------------ */
/* f-wave Riemann solve for one edge.                                        */
/*                                                                           */
/* The reference calls the TUM SWE f-wave solver                             */
/* (tools/SWE_WaveAccumulationBlock.cpp:154-159,193-198), whose source is    */
/* not part of the reference tree.  This restates the published f-wave       */
/* method for the shallow water equations with bathymetry (Bale, LeVeque,    */
/* Mitran & Rossmanith, SIAM J. Sci. Comput. 24(3), 2002; LeVeque, Finite    */
/* Volume Methods for Hyperbolic Problems, 2002, sec. 15.5): the flux jump    */
/* including the bathymetry source term is decomposed on the Roe-averaged    */
/* eigenvectors (1, ubar -+ cbar).                                           */
/*                                                                           */
/* Defined details (identical in the CUDA kernels):                          */
/*  - a cell is wet iff h > dry_tol; dry cells carry zero velocity, zero    */
/*    Roe weight (s = 0, p = 0, F = 0, hu = 0) and depth max(h, 0);          */
/*  - wet|dry edge where the wet surface h+b does not reach the dry cell's   */
/*    bathymetry: reflecting wall (dry side replaced by the mirrored wet     */
/*    state), and the update of the dry cell is dropped;                     */
/*  - otherwise (inundation) the dry side enters as (h, 0, b);               */
/*  - per cell: s = sqrt(h), p = hu * (1/s), F = p*p, surface eta = h + b,  */
/*    gh = g/2 h; per edge cbar^2 = gh_L + gh_R;                             */
/*  - momentum flux jump through the free-surface difference                 */
/*    df2 = (F_R - F_L) + g/2 (h_L+h_R) (eta_R - eta_L), so a lake at rest   */
/*    (equal eta) gives exactly zero;                                        */
/*  - wave strengths beta1 = (lambda2 df1 - df2) * (1 / (2 cbar)), with     */
/*    lambda2 - lambda1 = 2 cbar, and beta2 = df1 - beta1 (the first         */
/*    component of beta1 r1 + beta2 r2 = (df1, df2));                        */
/*  - waves with speed < 0 go left, all others go right; when both go to    */
/*    one side that side receives the whole flux jump (df1, df2), which      */
/*    beta1 r1 + beta2 r2 equals;                                            */
/* out = {hNetLeft, huNetLeft, hNetRight, huNetRight, maxEdgeSpeed}          */
/* ------------------------------------------------------------------------ */
typedef struct {
  double gh, hu, b, eta, s, p, F; /* gh = g/2 h */
  int wet;
} cellq;

static void cell_derived(const pco_swe_params *prm, double h, double hu, double b, cellq *c) {
  c->b = b;
  c->wet = h > prm->dry_tol;
  if (c->wet) {
    double s = sqrt(h);
    double rs = 1.0 / s;
    double p = hu * rs;
    c->s = s;
    c->p = p;
    c->F = p * p;
    c->hu = hu;
  } else {
    /* a dry cell enters with zero velocity and a non-negative depth (a ghost
     * value interpolated across a coastline can be negative) */
    h = h > 0.0 ? h : 0.0;
    c->s = 0.0;
    c->p = 0.0;
    c->F = 0.0;
    c->hu = 0.0;
  }
  c->eta = h + b;
  c->gh = (0.5 * prm->g) * h;
}

static void fwave_derived(const pco_swe_params *prm, cellq L, cellq R, double out[5]) {
  if (!L.wet && !R.wet) {
    out[0] = out[1] = out[2] = out[3] = out[4] = 0.0;
    return;
  }
  int wallR = L.wet && !R.wet && (L.eta <= R.b);
  int wallL = R.wet && !L.wet && (R.eta <= L.b);
  if (wallR) {
    R.gh = L.gh; R.hu = -L.hu; R.b = L.b; R.eta = L.eta; R.s = L.s; R.p = -L.p; R.F = L.F;
  }
  if (wallL) {
    L.gh = R.gh; L.hu = -R.hu; L.b = R.b; L.eta = R.eta; L.s = R.s; L.p = -R.p; L.F = R.F;
  }
  double a = L.gh + R.gh; /* g/2 (hL + hR) as g/2 hL + g/2 hR */
  double cb = sqrt(a);
  double ub = (L.p + R.p) / (L.s + R.s);
  double l1 = ub - cb;
  double l2 = ub + cb;
  double df1 = R.hu - L.hu;
  double deta = R.eta - L.eta;
  double df2 = fma(a, deta, R.F - L.F);
  double inv = 1.0 / (2.0 * cb);
  double b1 = fma(l2, df1, -df2) * inv;
  double b2 = df1 - b1;
  double z1 = b1 * l1;
  double z2 = b2 * l2;
  double Lh, Lhu, Rh, Rhu;
  /* both waves to one side: the whole flux jump (df1, df2) goes there */
  if (l1 < 0.0) {
    if (l2 < 0.0) {
      Lh = df1; Lhu = df2; Rh = 0.0; Rhu = 0.0;
    } else {
      Lh = b1; Lhu = z1; Rh = b2; Rhu = z2;
    }
  } else {
    Lh = 0.0; Lhu = 0.0; Rh = df1; Rhu = df2;
  }
  if (wallR) { Rh = 0.0; Rhu = 0.0; }
  if (wallL) { Lh = 0.0; Lhu = 0.0; }
  out[0] = Lh; out[1] = Lhu; out[2] = Rh; out[3] = Rhu;
  out[4] = fmax(fabs(l1), fabs(l2));
}

void pco_fwave_edge(const pco_swe_params *prm, double hL, double huL, double bL,
                    double hR, double huR, double bR, double out[5]) {
  cellq L, R;
  cell_derived(prm, hL, huL, bL, &L);
  cell_derived(prm, hR, huR, bR, &R);
  fwave_derived(prm, L, R, out);
}

/* ------------------------------------------------------------------------ */
/* DefaultTransfer::copyUNewToUOld / swapUOldAndUNew                         */
/* (src/peanoclaw/interSubgridCommunication/DefaultTransfer.cpph:103-127)    */
/* ------------------------------------------------------------------------ */
void pco_copy_unew_to_uold(pco_patch *p) {
  for (int x = 0; x < p->nx; x++)
    for (int y = 0; y < p->ny; y++)
      for (int q = 0; q < p->nq; q++) UOLD(p, q, x, y) = UNEW(p, q, x, y);
}
void pco_swap_unew_uold(pco_patch *p) {
  for (int x = 0; x < p->nx; x++)
    for (int y = 0; y < p->ny; y++)
      for (int q = 0; q < p->nq; q++) {
        double a = UNEW(p, q, x, y);
        UNEW(p, q, x, y) = UOLD(p, q, x, y);
        UOLD(p, q, x, y) = a;
      }
}

/* ------------------------------------------------------------------------ */
/* SWEKernel::fillBoundaryLayer: reflecting wall                             */
/* (src/peanoclaw/native/SWEKernel.cpp:176-237)                              */
/* ------------------------------------------------------------------------ */
void pco_swe_fill_boundary_layer(pco_patch *p, int dimension, int set_upper) {
  if (dimension == 0) {
    int xi = set_upper ? p->nx : -1;
    int sx = xi + (set_upper ? -1 : +1);
    for (int yi = -1; yi < p->ny + 1; yi++)
      for (int q = 0; q < p->nq; q++) {
        double v = UOLD(p, q, sx, yi);
        UOLD(p, q, xi, yi) = (q == dimension + 1) ? -v : v;
      }
  } else {
    int yi = set_upper ? p->ny : -1;
    int sy = yi + (set_upper ? -1 : +1);
    for (int xi = -1; xi < p->nx + 1; xi++)
      for (int q = 0; q < p->nq; q++) {
        double v = UOLD(p, q, xi, sy);
        UOLD(p, q, xi, yi) = (q == dimension + 1) ? -v : v;
      }
  }
}

/* Wall faces in the order SolveTimestep::fillBoundaryLayers visits them in 2D
 * (src/peanoclaw/mappings/SolveTimestep.cpp:87-142): (0,lower), (1,upper),
 * (0,upper), (1,lower).  mask bit = 2*dim + upper. */
static void fill_walls(pco_patch *p, uint8_t mask) {
  static const int order[4][2] = {{0, 0}, {1, 1}, {0, 1}, {1, 0}};
  for (int k = 0; k < 4; k++) {
    int d = order[k][0], up = order[k][1];
    if (mask & (1u << (2 * d + up))) pco_swe_fill_boundary_layer(p, d, up);
  }
}

/* ------------------------------------------------------------------------ */
/* SWE_WaveAccumulationBlock::computeNumericalFluxes                         */
/* (tools/SWE_WaveAccumulationBlock.cpp:84-240), on the uOld(+ghost) arrays  */
/* bound by SWEKernel::advanceBlockInTime (src/peanoclaw/native/             */
/* SWEKernel.cpp:57-63).  Block index (i, j) = patch cell (i-1, j-1).        */
/* net has 3 fields of (nx+2)*(ny+2), X[i][j] = X[i*(ny+2)+j].               */
/* ------------------------------------------------------------------------ */
double pco_swe_compute_net_updates(const pco_patch *p, const pco_swe_params *prm,
                                   double *net, double *max_speed) {
  const int nx = p->nx, ny = p->ny, S = ny + 2;
  const int64_t A = (int64_t)(nx + 2) * (ny + 2);
  double h[2];
  subcell_size(p, h);
  const double dx = h[0], dy = h[1];
  const double dx_inv = 1.0 / dx, dy_inv = 1.0 / dy;
  double *hN = net, *huN = net + A, *hvN = net + 2 * A;
  memset(net, 0, sizeof(double) * 3 * A);
  double smax = 0.0;
  double o[5];
  /* vertical edges: i in [1, nx+1], j in [1, ny] (:142-175) */
  for (int i = 1; i < nx + 2; i++)
    for (int j = 1; j < ny + 1; j++) {
      int xl = i - 2, xr = i - 1, y = j - 1;
      pco_fwave_edge(prm, UOLD(p, 0, xl, y), UOLD(p, 1, xl, y), PARW(p, 0, xl, y),
                     UOLD(p, 0, xr, y), UOLD(p, 1, xr, y), PARW(p, 0, xr, y), o);
      hN[(i - 1) * S + j] = fma(dx_inv, o[0], hN[(i - 1) * S + j]);
      huN[(i - 1) * S + j] = fma(dx_inv, o[1], huN[(i - 1) * S + j]);
      hN[i * S + j] = fma(dx_inv, o[2], hN[i * S + j]);
      huN[i * S + j] = fma(dx_inv, o[3], huN[i * S + j]);
      smax = fmax(smax, o[4]);
    }
  /* horizontal edges: i in [1, nx], j in [1, ny+1] (:182-214) */
  for (int i = 1; i < nx + 1; i++)
    for (int j = 1; j < ny + 2; j++) {
      int x = i - 1, yd = j - 2, yu = j - 1;
      pco_fwave_edge(prm, UOLD(p, 0, x, yd), UOLD(p, 2, x, yd), PARW(p, 0, x, yd),
                     UOLD(p, 0, x, yu), UOLD(p, 2, x, yu), PARW(p, 0, x, yu), o);
      hN[i * S + (j - 1)] = fma(dy_inv, o[0], hN[i * S + (j - 1)]);
      hvN[i * S + (j - 1)] = fma(dy_inv, o[1], hvN[i * S + (j - 1)]);
      hN[i * S + j] = fma(dy_inv, o[2], hN[i * S + j]);
      hvN[i * S + j] = fma(dy_inv, o[3], hvN[i * S + j]);
      smax = fmax(smax, o[4]);
    }
  if (max_speed) *max_speed = smax;
  /* CFL (:225-239): dt = cfl * min(dx/s, dy/s) if s > s_min else FLT_MAX */
  if (smax > prm->s_min) return prm->cfl * fmin(dx / smax, dy / smax);
  return prm->dt_inf;
}

/* SWE_WaveAccumulationBlock::updateUnknowns (:247-296) on uOld interior. */
void pco_swe_update_unknowns(pco_patch *p, const pco_swe_params *prm,
                             const double *net, double dt) {
  const int nx = p->nx, ny = p->ny, S = ny + 2;
  const int64_t A = (int64_t)(nx + 2) * (ny + 2);
  const double *hN = net, *huN = net + A, *hvN = net + 2 * A;
  for (int i = 1; i < nx + 1; i++)
    for (int j = 1; j < ny + 1; j++) {
      int x = i - 1, y = j - 1;
      double hh = fma(-dt, hN[i * S + j], UOLD(p, 0, x, y));
      double hu = fma(-dt, huN[i * S + j], UOLD(p, 1, x, y));
      double hv = fma(-dt, hvN[i * S + j], UOLD(p, 2, x, y));
      if (hh < prm->dry_tol_update) { hu = 0.0; hv = 0.0; }
      if (hh < 0.0) hh = 0.0;
      UOLD(p, 0, x, y) = hh;
      UOLD(p, 1, x, y) = hu;
      UOLD(p, 2, x, y) = hv;
    }
}

/* SWEKernel::solveTimestep -> advanceBlockInTime
 * (src/peanoclaw/native/SWEKernel.cpp:50-88,125-167). */
void pco_swe_solve_timestep(pco_patch *p, const pco_swe_params *prm,
                            double max_dt, double *dt_used, double *est_next) {
  int64_t A = (int64_t)(p->nx + 2) * (p->ny + 2);
  double *net = (double *)malloc(sizeof(double) * 3 * A);
  double block_dt = pco_swe_compute_net_updates(p, prm, net, NULL);
  double dt = fmin(block_dt, max_dt);
  pco_swe_update_unknowns(p, prm, net, dt);
  free(net);
  pco_swap_unew_uold(p);
  if (tl_greater(dt, 0.0)) {
    p->time = p->time + p->dt; /* TimeIntervals::advanceInTime */
    p->dt = dt;
  }
  p->est_next = block_dt;
  if (dt_used) *dt_used = dt;
  if (est_next) *est_next = block_dt;
}

/* ------------------------------------------------------------------------ */
/* DefaultTransferTemplate::transferGhostlayer                               */
/* (src/peanoclaw/interSubgridCommunication/DefaultTransfer.cpph:15-101),    */
/* without PEANOCLAW_USE_ASCEND_FOR_RESTRICTION.                             */
/* ------------------------------------------------------------------------ */
static double transfer_time_factor(const pco_patch *src, const pco_patch *dst) {
  double dtu = pco_time_unew(dst);
  if (src->is_virtual) return (dtu - 0.0) / 1.0;
  double su = pco_time_unew(src), so = pco_time_uold(src);
  if (tl_greater(su - so, 0.0)) return (dtu - so) / (su - so);
  return 1.0;
}

void pco_transfer_ghostlayer(const int size[2], const int src_off[2], const int dst_off[2],
                             const pco_patch *src, pco_patch *dst) {
  double tf = transfer_time_factor(src, dst);
  double itf = 1.0 - tf;
  for (int x = 0; x < size[0]; x++)
    for (int y = 0; y < size[1]; y++)
      for (int q = 0; q < src->nq; q++) {
        double vn = UNEW(src, q, src_off[0] + x, src_off[1] + y);
        double vo = UOLD(src, q, src_off[0] + x, src_off[1] + y);
        UOLD(dst, q, dst_off[0] + x, dst_off[1] + y) = vn * tf + vo * itf;
      }
}

/* ------------------------------------------------------------------------ */
/* DefaultInterpolationTemplate::interpolateSolution                         */
/* (src/peanoclaw/interSubgridCommunication/DefaultInterpolation.cpph:29-270)*/
/* wrapped, if swe_absolute_height, by SWEKernel::interpolateSolution        */
/* (src/peanoclaw/native/SWEKernel.cpp:239-286): the source water height is  */
/* read as h + b and the destination region gets h - b afterwards.  The      */
/* reference writes h + b into the source and subtracts b again afterwards,  */
/* which can move source values by rounding; here the source is left as is.  */
/* ------------------------------------------------------------------------ */
static double interp_time_factor(const pco_patch *src, const pco_patch *dst,
                                 int to_current_time, int use_time_unew_or_uold) {
  double tf;
  if (tl_equals(src->dt, 0.0)) {
    tf = 1.0;
  } else if (use_time_unew_or_uold) {
    double so = pco_time_uold(src), su = pco_time_unew(src);
    if (to_current_time) tf = (pco_time_uold(dst) - so) / (su - so);
    else tf = (pco_time_unew(dst) - so) / (su - so);
  } else {
    if (to_current_time) tf = (dst->time - src->time) / (src->time + src->dt - src->time);
    else tf = (dst->time + dst->dt - src->time) / (src->time + src->dt - src->time);
  }
  return fmax(0.0, fmin(1.0, tf));
}

void pco_interpolate(const int dst_size[2], const int dst_off[2],
                     const pco_patch *src, pco_patch *dst,
                     int to_uold, int to_current_time, int use_time_unew_or_uold,
                     int swe_absolute_height) {
  double tf = interp_time_factor(src, dst, to_current_time, use_time_unew_or_uold);
  double one_m_tf = 1.0 - tf;
  /* Clear the destination region in uOld (:78-83), even when writing uNew. */
  for (int x = 0; x < dst_size[0]; x++)
    for (int y = 0; y < dst_size[1]; y++)
      for (int q = 0; q < dst->nq; q++)
        UOLD(dst, q, dst_off[0] + x, dst_off[1] + y) = 0.0;
  double sh[2], inv[2];
  subcell_size(src, sh);
  inv[0] = 1.0 / sh[0];
  inv[1] = 1.0 / sh[1];
  double sbase[2] = {src->pos[0] + sh[0] * 0.5, src->pos[1] + sh[1] * 0.5};
  for (int x = 0; x < dst_size[0]; x++)
    for (int y = 0; y < dst_size[1]; y++) {
      int cx = dst_off[0] + x, cy = dst_off[1] + y;
      double c[2];
      subcell_center(dst, cx, cy, c);
      int bi[2];
      for (int d = 0; d < 2; d++) {
        double local = c[d] - sbase[d];
        bi[d] = (int)floor(local * inv[d]);
      }
      int n[2] = {src->nx, src->ny};
      for (int d = 0; d < 2; d++) {
        int v = bi[d] < n[d] - 2 ? bi[d] : n[d] - 2;
        bi[d] = v > 0 ? v : 0;
      }
      /* dfor2(offset): dimension 0 runs fastest */
      for (int k = 0; k < 4; k++) {
        int off[2] = {k & 1, (k >> 1) & 1};
        int nxi = bi[0] + off[0], nyi = bi[1] + off[1];
        double npos[2];
        subcell_center(src, nxi, nyi, npos);
        double sf = 1.0;
        for (int d = 0; d < 2; d++) {
          double sign = (double)(1 - 2 * off[d]);
          sf = sf * (1.0 - (sign * (c[d] - npos[d])) * inv[d]);
        }
        for (int q = 0; q < dst->nq; q++) {
          double so = UOLD(src, q, nxi, nyi);
          double sn = UNEW(src, q, nxi, nyi);
          if (swe_absolute_height && q == 0) {
            double bb = PARW(src, 0, nxi, nyi);
            so = so + bb;
            sn = sn + bb;
          }
          if (to_uold) {
            double *dv = &UOLD(dst, q, cx, cy);
            *dv = *dv + sf * (so * one_m_tf + sn * tf);
          } else {
            double *dv = &UNEW(dst, q, cx, cy);
            *dv = (*dv + (sf * so) * one_m_tf) + (sf * sn) * tf;
          }
        }
      }
    }
  if (swe_absolute_height) {
    for (int x = 0; x < dst_size[0]; x++)
      for (int y = 0; y < dst_size[1]; y++) {
        int cx = dst_off[0] + x, cy = dst_off[1] + y;
        double bb = PARW(dst, 0, cx, cy);
        if (to_uold) UOLD(dst, 0, cx, cy) = UOLD(dst, 0, cx, cy) + (-1.0) * bb;
        else UNEW(dst, 0, cx, cy) = UNEW(dst, 0, cx, cy) + (-1.0) * bb;
      }
  }
}

/* ------------------------------------------------------------------------ */
/* Region geometry (src/peanoclaw/geometry/Region.cpp:174-315)               */
/* ------------------------------------------------------------------------ */
void pco_region_map_to_patch(const int off[2], const int size[2],
                             const pco_patch *src, const pco_patch *dst, double eps,
                             int out_off[2], int out_size[2]) {
  double ss[2], ds[2];
  subcell_size(src, ss);
  subcell_size(dst, ds);
  for (int d = 0; d < 2; d++) {
    double position = ss[d] * (double)off[d];
    position = position + (src->pos[d] - dst->pos[d]);
    double offset_temp = (position + eps) / ds[d];
    out_off[d] = (int)offset_temp;
    double sz = ss[d] * (double)(off[d] + size[d]);
    sz = sz + (src->pos[d] - dst->pos[d]);
    double size_temp = (sz - eps) / ds[d];
    size_temp = size_temp - (double)out_off[d];
    size_temp = size_temp + 1.0;
    out_size[d] = (int)size_temp;
  }
}

static void region_map_cell_to_patch(const int roff[2], const int rsize[2],
                                     const double fine_pos[2], const double fine_sub[2],
                                     const double coarse_sub[2], const double coarse_pos[2],
                                     double eps, int out_off[2], int out_size[2]) {
  for (int d = 0; d < 2; d++) {
    double offset_temp = ((coarse_pos[d] - fine_pos[d]) + eps) / fine_sub[d];
    int off = (int)offset_temp;
    double size_temp = (((coarse_pos[d] + coarse_sub[d]) - fine_pos[d]) - eps) / fine_sub[d];
    size_temp = size_temp - offset_temp;
    size_temp = size_temp + 1.0;
    int sz = (int)size_temp;
    int upper = off + sz;
    int rupper = roff[d] + rsize[d];
    int o = off > roff[d] ? off : roff[d];
    int u = upper < rupper ? upper : rupper;
    out_off[d] = o;
    out_size[d] = u - o;
  }
}

int pco_regions_overlapped_by_ghostlayers(const double lower[2], const double upper[2],
                                          const double src_pos[2], const double src_size[2],
                                          const double src_sub[2], const int n[2],
                                          int out_off[8], int out_size[8]) {
  int one_greater = 0, one_greater_equals = 0, all_greater = 1;
  for (int d = 0; d < 2; d++) {
    if (tl_greater(upper[d] + src_sub[d], lower[d])) one_greater = 1;
    if (tl_greater_equals(upper[d], src_pos[d] + src_size[d])) one_greater_equals = 1;
    if (!tl_greater(lower[d], src_pos[d])) all_greater = 0;
  }
  if (one_greater || one_greater_equals || !all_greater) {
    for (int k = 0; k < 8; k++) { out_off[k] = 0; out_size[k] = 0; }
    out_size[0] = n[0];
    out_size[1] = n[1];
    return 1;
  }
  const double eps = 1e-12;
  int lo[2], up[2];
  for (int d = 0; d < 2; d++) {
    double dl = (lower[d] - src_pos[d]) * (1.0 / src_sub[d]) + eps;
    double du = (upper[d] - src_pos[d]) * (1.0 / src_sub[d]) - eps;
    dl = fmin((double)INT_MAX, dl);
    du = fmax((double)INT_MIN, du);
    int a = (int)floor(dl), b = (int)floor(du);
    a = a < n[d] ? a : n[d];
    b = b < n[d] ? b : n[d];
    lo[d] = a > -1 ? a : -1;
    up[d] = b > -1 ? b : -1;
  }
  /* regions[r] offset/size component i live at out_*[2*r + i] */
  for (int d = 0; d < 2; d++) {
    int r0 = 2 * d, r1 = 2 * d + 1;
    out_size[2 * r0 + d] = up[d] + 1;
    out_off[2 * r0 + d] = 0;
    out_size[2 * r1 + d] = n[d] - lo[d];
    out_off[2 * r1 + d] = lo[d];
    for (int i = 0; i < d; i++) {
      out_size[2 * r0 + i] = -up[i] - 1 + lo[i];
      out_off[2 * r0 + i] = up[i] + 1;
      out_size[2 * r1 + i] = out_size[2 * r0 + i];
      out_off[2 * r1 + i] = out_off[2 * r0 + i];
    }
    for (int i = d + 1; i < 2; i++) {
      out_size[2 * r0 + i] = n[i];
      out_off[2 * r0 + i] = 0;
      out_size[2 * r1 + i] = n[i];
      out_off[2 * r1 + i] = 0;
    }
  }
  return 4;
}

/* DefaultRestrictionTemplate::calculateOverlappingRegion
 * (src/peanoclaw/interSubgridCommunication/DefaultRestriction.h:44-62) */
double pco_overlap_area(const double p1[2], const double s1[2],
                        const double p2[2], const double s2[2]) {
  double region = 1.0;
  for (int d = 0; d < 2; d++) {
    double a = p1[d] + s1[d], b = p2[d] + s2[d];
    double lo = p1[d] > p2[d] ? p1[d] : p2[d];
    double ov = (a < b ? a : b) - lo;
    region = region * ov;
    region = fmax(region, 0.0);
  }
  return region;
}

/* Patch::switchToLeaf (src/peanoclaw/Patch.cpp:793-816): the reference maps
 * the virtual patch's interval to [0, 1] (time = 0, timestepSize = 1) and
 * re-evaluates uOld / uNew of the interior at the patch's own time and
 * time + dt (switchRegionToMinimalFineGridTimeInterval, :55-76). */
void pco_switch_to_leaf(pco_patch *p) {
  p->is_virtual = 0;
  p->is_leaf = 1;
  const double time = 0.0, timestep = 1.0;
  double fo = 1.0, fn = 1.0;
  if (!tl_equals(timestep, 0.0)) {
    fo = (p->time - time) / timestep;
    fn = (p->time + p->dt - time) / timestep;
  }
  for (int x = 0; x < p->nx; x++)
    for (int y = 0; y < p->ny; y++)
      for (int q = 0; q < p->nq; q++) {
        double vo = UOLD(p, q, x, y), vn = UNEW(p, q, x, y);
        UOLD(p, q, x, y) = vo * (1.0 - fo) + vn * fo;
        UNEW(p, q, x, y) = vo * (1.0 - fn) + vn * fn;
      }
}

/* ------------------------------------------------------------------------ */
/* DefaultRestrictionTemplate::restrictRegion / restrictSolution             */
/* (src/peanoclaw/interSubgridCommunication/DefaultRestriction.cpph:17-150), */
/* wrapped, if swe_absolute_height, by SWEKernel::restrictSolution           */
/* (src/peanoclaw/native/SWEKernel.cpp:288-307): source h is read as h + b.  */
/* ------------------------------------------------------------------------ */
static void restrict_region(const pco_patch *src, pco_patch *dst, const int roff[2],
                            const int rsize[2], int swe) {
  const double eps = 1e-12;
  const double dtuold = 0.0, dtunew = 1.0;
  double ssub[2] = {src->size[0] * (1.0 / (double)src->nx), src->size[1] * (1.0 / (double)src->ny)};
  double dsub[2] = {dst->size[0] * (1.0 / (double)dst->nx), dst->size[1] * (1.0 / (double)dst->ny)};
  double dvol = dsub[0] * dsub[1];
  double tfo = 1.0, tfn = 1.0;
  if (tl_greater(src->dt, 0.0)) {
    double so = pco_time_uold(src), su = pco_time_unew(src);
    tfo = (dtuold - so) / (su - so);
    tfn = (dtunew - so) / (su - so);
  }
  int doff[2], dsz[2];
  pco_region_map_to_patch(roff, rsize, src, dst, eps, doff, dsz);
  for (int x = doff[0]; x < doff[0] + dsz[0]; x++)
    for (int y = doff[1]; y < doff[1] + dsz[1]; y++) {
      double dpos[2];
      iter_cell_position(dst, x, y, dpos);
      int coff[2], csz[2];
      region_map_cell_to_patch(roff, rsize, src->pos, ssub, dsub, dpos, eps, coff, csz);
      for (int sx = coff[0]; sx < coff[0] + csz[0]; sx++)
        for (int sy = coff[1]; sy < coff[1] + csz[1]; sy++) {
          double spos[2];
          iter_cell_position(src, sx, sy, spos);
          double ov = pco_overlap_area(dpos, dsub, spos, ssub);
          for (int q = 0; q < dst->nq; q++) {
            double vo = UOLD(src, q, sx, sy);
            double vn = UNEW(src, q, sx, sy);
            if (swe && q == 0) {
              double bb = PARW(src, 0, sx, sy);
              vo = vo + bb;
              vn = vn + bb;
            }
            double d_o = ((vo * (1.0 - tfo) + vn * tfo) * ov) / dvol;
            double d_n = ((vo * (1.0 - tfn) + vn * tfn) * ov) / dvol;
            UOLD(dst, q, x, y) = UOLD(dst, q, x, y) + d_o;
            UNEW(dst, q, x, y) = UNEW(dst, q, x, y) + d_n;
          }
        }
    }
}

void pco_restrict(const pco_patch *src, pco_patch *dst, int only_overlapped, int swe) {
  if (only_overlapped) {
    int off[8], sz[8];
    double ssub[2];
    subcell_size(src, ssub);
    int n[2] = {src->nx, src->ny};
    int nr = pco_regions_overlapped_by_ghostlayers(dst->restr_lower, dst->restr_upper,
                                                   src->pos, src->size, ssub, n, off, sz);
    for (int r = 0; r < nr; r++) {
      if (sz[2 * r] > 0 && sz[2 * r + 1] > 0) restrict_region(src, dst, &off[2 * r], &sz[2 * r], swe);
    }
  } else {
    int off[2] = {0, 0}, sz[2] = {src->nx, src->ny};
    restrict_region(src, dst, off, sz, swe);
  }
}

/* SWEKernel::postProcessRestriction (src/peanoclaw/native/SWEKernel.cpp:309-316) */
void pco_swe_post_process_restriction(pco_patch *dst) {
  for (int x = 0; x < dst->nx; x++)
    for (int y = 0; y < dst->ny; y++) {
      double bb = PARW(dst, 0, x, y);
      UOLD(dst, 0, x, y) = UOLD(dst, 0, x, y) + (-1.0) * bb;
    }
  for (int x = 0; x < dst->nx; x++)
    for (int y = 0; y < dst->ny; y++) {
      double bb = PARW(dst, 0, x, y);
      UNEW(dst, 0, x, y) = UNEW(dst, 0, x, y) + (-1.0) * bb;
    }
}

/* ------------------------------------------------------------------------ */
/* Flux correction                                                           */
/* (src/peanoclaw/interSubgridCommunication/DefaultFluxCorrection.cpph)      */
/* ------------------------------------------------------------------------ */
/* Numerics::computeFlux (src/peanoclaw/Numerics.h:186-203), nq == 3, g = g_flux
 * (the reference hard-codes 1.0). */
static void compute_flux(int dim, const double u[3], double g_flux, double f[3]) {
  double m = u[1 + dim];
  f[0] = u[0] * m;
  f[1] = u[1] * m;
  f[2] = u[2] * m;
  f[1] = f[1] * u[0];
  f[2] = f[2] * u[0];
  double pr = ((0.5 * g_flux) * u[0]) * u[0];
  f[1 + dim] = f[1 + dim] + pr;
}

/* computeFluxes (:43-85).  The upwind term at :72 is a separate statement
 * without effect, so the stored flux is the central average. */
void pco_compute_fluxes(pco_patch *p, double g_flux) {
  int n[2] = {p->nx, p->ny};
  for (int dim = 0; dim < 2; dim++) {
    int other = 1 - dim;
    for (int dir = -1; dir < 2; dir += 2) {
      int inner = (dir == -1) ? 0 : n[dim] - 1;
      int ghost = (dir == -1) ? -1 : n[dim];
      for (int c = 0; c < n[other]; c++) {
        double gu[3], iu[3], gf[3], ifl[3];
        for (int q = 0; q < 3; q++) {
          int gx = dim == 0 ? ghost : c, gy = dim == 0 ? c : ghost;
          int ix = dim == 0 ? inner : c, iy = dim == 0 ? c : inner;
          gu[q] = UOLD(p, q, gx, gy);
          iu[q] = UOLD(p, q, ix, iy);
        }
        compute_flux(dim, gu, g_flux, gf);
        compute_flux(dim, iu, g_flux, ifl);
        for (int q = 0; q < 3; q++)
          p->u[pco_idx_flux(p, q, c, dim, dir)] = 0.5 * (gf[q] + ifl[q]);
      }
    }
  }
}

static const double HYPERPLANE_EPS = 1e-10; /* HyperplaneRegion.cpp:12 */

/* applyCorrection (:87-164) with HyperplaneRegion::getInterfaceRegion and
 * getInterfaceRegionForSubcell (src/peanoclaw/geometry/HyperplaneRegion.cpp:26-104).
 * getInterfaceRegionForSubcell takes the extent of the destination from its
 * subcell size (:77 reads getSubcellSize() into subgridSize); restated as is. */
void pco_apply_flux_correction(const pco_patch *src, pco_patch *dst, int dim, int dir) {
  double lo = fmax(src->time, dst->time);
  double hi = fmin(src->time + src->dt, dst->time + dst->dt);
  double tov = hi - lo;
  /* getInterfaceRegion(src, dst): only its dimension/direction are used */
  int rdim = 0, rdir = 0;
  for (int d = 0; d < 2; d++) {
    if (tl_greater(dst->pos[d], src->pos[d])) { rdim = d; rdir = 1; }
    else if (tl_greater(src->pos[d], dst->pos[d])) { rdim = d; rdir = -1; }
  }
  double ssub[2], dsub[2];
  subcell_size(src, ssub);
  subcell_size(dst, dsub);
  double dvol = dsub[0] * dsub[1];
  int sn[2] = {src->nx, src->ny}, dn[2] = {dst->nx, dst->ny};
  int other = 1 - dim;
  (void)rdir;
  for (int cs = 0; cs < sn[other]; cs++) {
    /* getInterfaceRegionForSubcell(dst, src, cs, rdim, rdir) */
    int po = 1 - rdim; /* face-parallel dimension of the projection */
    double npos = src->pos[po] + ssub[po] * (double)cs;
    double lb = fmax(dst->pos[po], npos);
    double ub = fmin(dst->pos[po] + dsub[po], npos + ssub[po]);
    int lbc = (int)((lb - dst->pos[po] + HYPERPLANE_EPS) / dsub[po]);
    int ubc = (int)ceil((ub - dst->pos[po] - HYPERPLANE_EPS) / dsub[po]);
    double sF[3];
    for (int q = 0; q < 3; q++) sF[q] = src->u[pco_idx_flux(src, q, cs, dim, dir)];
    int dinner = (-dir == -1) ? 0 : dn[dim] - 1;
    for (int cd = lbc; cd < ubc; cd++) {
      double dF[3];
      for (int q = 0; q < 3; q++) dF[q] = dst->u[pco_idx_flux(dst, q, cd, dim, -dir)];
      /* calculateOverlappingRegion over the face-parallel dimension (:13-41) */
      double a1 = src->pos[other] + ((double)cs + 1.0) * ssub[other];
      double a2 = dst->pos[other] + ((double)cd + 1.0) * dsub[other];
      double b1 = src->pos[other] + (double)cs * ssub[other];
      double b2 = dst->pos[other] + (double)cd * dsub[other];
      double area = 1.0 * ((a1 < a2 ? a1 : a2) - (b1 > b2 ? b1 : b2));
      if (area < 0.0) area = 0.0;
      int ux = dim == 0 ? dinner : cd, uy = dim == 0 ? cd : dinner;
      if (ux < 0 || uy < 0 || ux >= dst->nx || uy >= dst->ny) continue;
      for (int q = 0; q < 3; q++) {
        double corr = (((sF[q] - dF[q]) * tov) * area) / dvol;
        UNEW(dst, q, ux, uy) = UNEW(dst, q, ux, uy) + corr;
      }
    }
  }
}

/* ------------------------------------------------------------------------ */
/* Synchronous grid step: the semantics of the batched GPU form.             */
/* ------------------------------------------------------------------------ */
/* Ghost items grouped by destination (declared in pcoracle.h). */
int *pco_items_by_dst(pco_patch **patches, int n_patches, const pco_ghost_item *items, int n_items,
                      int **start_out) {
  for (int k = 0; k < n_items; k++) {
    const pco_ghost_item *it = &items[k];
    if (it->kind != PCO_GHOST_COPY) continue; /* interpolation reads cells [0, n-1] */
    const pco_patch *src = patches[it->src];
    const int n[2] = {src->nx, src->ny};
    for (int d = 0; d < 2; d++)
      if (it->src_offset[d] < 0 || it->src_offset[d] + it->size[d] > n[d]) return NULL;
  }
  int *start = (int *)calloc((size_t)n_patches + 1, sizeof(int));
  int *cur = (int *)malloc(sizeof(int) * ((size_t)n_patches + 1));
  int *ord = (int *)malloc(sizeof(int) * (size_t)(n_items > 0 ? n_items : 1));
  for (int k = 0; k < n_items; k++) start[items[k].dst + 1]++;
  for (int p = 0; p < n_patches; p++) start[p + 1] += start[p];
  memcpy(cur, start, sizeof(int) * ((size_t)n_patches + 1));
  for (int k = 0; k < n_items; k++) ord[cur[items[k].dst]++] = k;
  free(cur);
  *start_out = start;
  return ord;
}

static void fill_item(pco_patch **patches, const pco_ghost_item *it) {
  pco_patch *src = patches[it->src], *dst = patches[it->dst];
  if (it->kind == PCO_GHOST_COPY)
    pco_transfer_ghostlayer(it->size, it->src_offset, it->dst_offset, src, dst);
  else
    pco_interpolate(it->size, it->dst_offset, src, dst, 1, 0, 1, 1);
}

void pco_grid_fill(pco_patch **patches, int n_patches,
                   const pco_ghost_item *items, int n_items, const uint8_t *wall_mask) {
  /* SolveTimestep::enterCell copies uNew into uOld before filling the domain
   * boundary (src/peanoclaw/mappings/SolveTimestep.cpp:637-643); ghost layers
   * transferred by the compositor live in uOld's ghost region and survive the
   * copy.  The copy is done first here, which gives the same uOld.
   * An item writes only its destination's ghost layer and reads source
   * interiors, so the destinations are filled in parallel, each with its
   * items in list order: the same writes in the same order as one pass over
   * the list.  The interior copies, which overwrite the uOld interiors the
   * items read, come after every item. */
  int *start = NULL;
  int *ord = pco_items_by_dst(patches, n_patches, items, n_items, &start);
  if (ord) {
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 16)
#endif
    for (int p = 0; p < n_patches; p++)
      for (int q = start[p]; q < start[p + 1]; q++) fill_item(patches, &items[ord[q]]);
    free(ord);
    free(start);
  } else {
    for (int k = 0; k < n_items; k++) fill_item(patches, &items[k]);
  }
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 16)
#endif
  for (int p = 0; p < n_patches; p++) {
    if (!patches[p]->is_leaf) continue;
    pco_copy_unew_to_uold(patches[p]);
    fill_walls(patches[p], wall_mask ? wall_mask[p] : 0);
  }
}

void pco_grid_step(pco_patch **patches, int n_patches,
                   const pco_ghost_item *items, int n_items,
                   const uint8_t *wall_mask, const int32_t *group, int n_groups,
                   const pco_swe_params *prm, const double *max_dt,
                   double *dt_out, int n_threads) {
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
#endif
  pco_grid_fill(patches, n_patches, items, n_items, wall_mask);
  double *own = (double *)malloc(sizeof(double) * (size_t)n_patches);
  double **nets = (double **)calloc((size_t)n_patches, sizeof(double *));
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 16)
#endif
  for (int p = 0; p < n_patches; p++) {
    pco_patch *pp = patches[p];
    own[p] = prm->dt_inf;
    if (!pp->is_leaf) continue;
    int64_t A = (int64_t)(pp->nx + 2) * (pp->ny + 2);
    nets[p] = (double *)malloc(sizeof(double) * 3 * A);
    own[p] = pco_swe_compute_net_updates(pp, prm, nets[p], NULL);
  }
  for (int gi = 0; gi < n_groups; gi++) dt_out[gi] = max_dt[gi];
  for (int p = 0; p < n_patches; p++) {
    if (!patches[p]->is_leaf) continue;
    int gi = group ? group[p] : 0;
    dt_out[gi] = fmin(own[p], dt_out[gi]);
  }
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 16)
#endif
  for (int p = 0; p < n_patches; p++) {
    pco_patch *pp = patches[p];
    if (!pp->is_leaf) continue;
    int gi = group ? group[p] : 0;
    double dt = dt_out[gi];
    pco_swe_update_unknowns(pp, prm, nets[p], dt);
    pco_swap_unew_uold(pp);
    if (tl_greater(dt, 0.0)) {
      pp->time = pp->time + pp->dt;
      pp->dt = dt;
    }
    pp->est_next = own[p];
    free(nets[p]);
  }
  free(nets);
  free(own);
}

/* ------------------------------------------------------------------------ */
/* Local time stepping (the semantics of the batched GPU form with per-patch */
/* time steps), one grid iteration in two phases.  The reference decides per */
/* leaf in the traversal whether it may advance (TimeIntervals.cpp:24-99:    */
/* the global end time is not reached and the patch is not blocked by its    */
/* neighbours, i.e. time + dt does not exceed the minimal uNew time of the   */
/* neighbouring subgrids) and then solves with max_dt = end time - (time +   */
/* dt) (SolveTimestep.cpp:591-700).  Here every decision and every ghost     */
/* fill of an iteration uses the times at its start (fill all, then solve    */
/* all): a leaf's neighbours are the sources of its ghost items; the ghost   */
/* layers of the advancing leaves are filled with the time factors of their */
/* uNew time (DefaultTransfer / interpolation time interpolation); the       */
/* leaves then step with dt = min(block CFL dt, max_dt).                     */
/* A neighbour's time constraint is its time + dt (TimeIntervals::           */
/* getTimeConstraint).  Virtual patches first take the intersection of the   */
/* time intervals of their listed leaves (vt_leaf[k] -> vt_virt[k]): time =  */
/* the maximal leaf time, dt = the minimal leaf time + dt minus that time    */
/* (GridLevelTransfer::stepUp, GridLevelTransfer.cpp:408-431, with           */
/* updateMinimalFineGridTimeInterval, TimeIntervals.cpp:214-231, and         */
/* Patch::switchValuesAndTimeIntervalToMinimalFineGridTimeInterval,         */
/* Patch.cpp:388-397).                                                       */
/* dt_out[p] receives the dt taken (0 for a leaf that did not advance);      */
/* returns the number of leaves that advanced.                               */
/* ------------------------------------------------------------------------ */
int pco_grid_step_lts(pco_patch **patches, int n_patches, const pco_ghost_item *items, int n_items,
                      const uint8_t *wall_mask, const pco_swe_params *prm, double max_dt,
                      double t_end, const int32_t *vt_leaf, const int32_t *vt_virt, int n_vt,
                      double *dt_out, int n_threads) {
  double *nbmin = (double *)malloc(sizeof(double) * (size_t)n_patches);
  char *active = (char *)calloc((size_t)n_patches, 1);
  double *maxdt = (double *)malloc(sizeof(double) * (size_t)n_patches);
  double *vstart = (double *)malloc(sizeof(double) * (size_t)n_patches);
  double *vend = (double *)malloc(sizeof(double) * (size_t)n_patches);
  for (int p = 0; p < n_patches; p++) {
    nbmin[p] = INFINITY;
    vstart[p] = -INFINITY;
    vend[p] = INFINITY;
  }
  for (int k = 0; k < n_vt; k++) {
    const pco_patch *lf = patches[vt_leaf[k]];
    const double t = lf->time, e = lf->time + lf->dt;
    if (t > vstart[vt_virt[k]]) vstart[vt_virt[k]] = t;
    if (e < vend[vt_virt[k]]) vend[vt_virt[k]] = e;
  }
  for (int k = 0; k < n_vt; k++) {
    pco_patch *v = patches[vt_virt[k]];
    v->time = vstart[vt_virt[k]];
    v->dt = vend[vt_virt[k]] - v->time;
  }
  for (int k = 0; k < n_items; k++) {
    const pco_patch *src = patches[items[k].src];
    double tc = src->time + src->dt;
    if (tc < nbmin[items[k].dst]) nbmin[items[k].dst] = tc;
  }
  int n_active = 0;
  for (int p = 0; p < n_patches; p++) {
    pco_patch *pp = patches[p];
    dt_out[p] = 0.0;
    if (!pp->is_leaf) continue;
    double tu = pco_time_unew(pp);
    double rem = t_end - tu;
    maxdt[p] = rem < max_dt ? rem : max_dt;
    active[p] = tl_greater(maxdt[p], 0.0) && !tl_greater(tu, nbmin[p]);
    n_active += active[p];
  }
  for (int k = 0; k < n_items; k++) {
    const pco_ghost_item *it = &items[k];
    if (!active[it->dst]) continue;
    pco_patch *src = patches[it->src], *dst = patches[it->dst];
    if (it->kind == PCO_GHOST_COPY)
      pco_transfer_ghostlayer(it->size, it->src_offset, it->dst_offset, src, dst);
    else
      pco_interpolate(it->size, it->dst_offset, src, dst, 1, 0, 1, 1);
  }
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
#pragma omp parallel for schedule(dynamic, 16)
#endif
  for (int p = 0; p < n_patches; p++) {
    pco_patch *pp = patches[p];
    if (!active[p]) continue;
    pco_copy_unew_to_uold(pp);
    fill_walls(pp, wall_mask ? wall_mask[p] : 0);
    int64_t A = (int64_t)(pp->nx + 2) * (pp->ny + 2);
    double *net = (double *)malloc(sizeof(double) * 3 * A);
    double own = pco_swe_compute_net_updates(pp, prm, net, NULL);
    double dt = fmin(own, maxdt[p]);
    pco_swe_update_unknowns(pp, prm, net, dt);
    pco_swap_unew_uold(pp);
    if (tl_greater(dt, 0.0)) {
      pp->time = pp->time + pp->dt;
      pp->dt = dt;
    }
    pp->est_next = own;
    dt_out[p] = dt;
    free(net);
  }
  free(nbmin);
  free(active);
  free(maxdt);
  free(vstart);
  free(vend);
  return n_active;
}

