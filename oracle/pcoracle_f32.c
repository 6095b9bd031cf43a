/*
 * pcoracle_f32.c -- FP32 twin of the oracle's synchronous grid step.
 *
 * TEST INFRASTRUCTURE ONLY: a CPU timing baseline at the reference's own
 * storage precision.  PeanoClaw's SWE build stores patch data as float
 * (records/Data.h:16-18) and the SWE block computes in that type
 * (tools/SWE_WaveAccumulationBlock.cpp:84-296); the FP64 oracle in
 * pcoracle.c is what the CUDA path is checked against bit for bit, and this
 * file times the same work with float data:
 *   - ghost fill (DefaultTransfer.cpph:15-101, DefaultInterpolation.cpph:29-270
 *     with the SWE wrapping of SWEKernel.cpp:239-286): time factors,
 *     positions and weights in double (tarch vectors are double), values read
 *     from and stored to float arrays;
 *   - reflecting walls (SWEKernel.cpp:176-237);
 *   - computeNumericalFluxes / updateUnknowns (SWE_WaveAccumulationBlock.cpp:
 *     84-296) with the f-wave restatement of pcoracle.c in float arithmetic
 *     (sqrtf, fmaf, float divides).
 * Layout, item order, wall order and the group-dt reduction are those of
 * pco_grid_step.  Results agree with the FP64 oracle to float rounding, not
 * bit for bit.
 */
#include "pcoracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define PCO_TARCH_EPS 1.0e-8

/* Layout of one patch vector (same as pco_idx_*; kept local so that the
 * inner loops inline it). */
typedef struct {
  int64_t vol_new, vol_old, base_uold, base_pw, stride;
  int g;
} lay32;

static lay32 layout(const pco_patch *p) {
  lay32 L;
  L.g = p->ghost;
  L.vol_new = (int64_t)p->nx * p->ny;
  L.vol_old = (int64_t)(p->nx + 2 * p->ghost) * (p->ny + 2 * p->ghost);
  L.base_uold = p->nq * L.vol_new;
  L.base_pw = L.base_uold + p->nq * L.vol_old + p->np_wo * L.vol_new;
  L.stride = p->ny + 2 * p->ghost;
  return L;
}
static inline int64_t i_new(const lay32 *L, const pco_patch *p, int q, int x, int y) {
  return q * L->vol_new + (int64_t)x * p->ny + y;
}
static inline int64_t i_old(const lay32 *L, int q, int x, int y) {
  return L->base_uold + q * L->vol_old + (int64_t)(x + L->g) * L->stride + (y + L->g);
}
static inline int64_t i_pw(const lay32 *L, int x, int y) {
  return L->base_pw + (int64_t)(x + L->g) * L->stride + (y + L->g);
}

static double time_uold(const pco_patch *p) { return p->is_leaf ? p->time : p->min_neighbor_time; }
static double time_unew(const pco_patch *p) {
  return p->is_leaf ? p->time + p->dt : p->min_neighbor_time + p->max_neighbor_dt;
}

/* ---- ghost fill ---------------------------------------------------------- */
static void transfer32(const pco_ghost_item *it, const pco_patch *src, const float *us,
                       const pco_patch *dst, float *ud) {
  double dtu = time_unew(dst), tf = 1.0;
  if (src->is_virtual) {
    tf = dtu;
  } else {
    double su = time_unew(src), so = time_uold(src);
    if (su - so > PCO_TARCH_EPS) tf = (dtu - so) / (su - so);
  }
  const double itf = 1.0 - tf;
  lay32 Ls = layout(src), Ld = layout(dst);
  for (int x = 0; x < it->size[0]; x++)
    for (int y = 0; y < it->size[1]; y++)
      for (int q = 0; q < src->nq; q++) {
        int sx = it->src_offset[0] + x, sy = it->src_offset[1] + y;
        double vn = us[i_new(&Ls, src, q, sx, sy)], vo = us[i_old(&Ls, q, sx, sy)];
        ud[i_old(&Ld, q, it->dst_offset[0] + x, it->dst_offset[1] + y)] = (float)(vn * tf + vo * itf);
      }
}

/* SWE interpolateSolution(toUOld, !toCurrentTime, useTimeUNewOrUOld) of a
 * ghost item: source heights read as h + b, destination gets h - b. */
static void interpolate32(const pco_ghost_item *it, const pco_patch *src, const float *us,
                          const pco_patch *dst, float *ud) {
  double tf = 1.0;
  if (fabs(src->dt) > PCO_TARCH_EPS) {
    double so = time_uold(src), su = time_unew(src);
    tf = (time_unew(dst) - so) / (su - so);
  }
  tf = fmax(0.0, fmin(1.0, tf));
  const double one_m_tf = 1.0 - tf;
  lay32 Ls = layout(src), Ld = layout(dst);
  const int nq = dst->nq;
  double sh[2] = {src->size[0] / (double)src->nx, src->size[1] / (double)src->ny};
  double dh[2] = {dst->size[0] / (double)dst->nx, dst->size[1] / (double)dst->ny};
  double inv[2] = {1.0 / sh[0], 1.0 / sh[1]};
  double sbase[2] = {src->pos[0] + sh[0] * 0.5, src->pos[1] + sh[1] * 0.5};
  for (int x = 0; x < it->size[0]; x++)
    for (int y = 0; y < it->size[1]; y++) {
      int cx = it->dst_offset[0] + x, cy = it->dst_offset[1] + y;
      double c[2] = {(dst->pos[0] + dh[0] * (double)cx) + dh[0] * 0.5,
                     (dst->pos[1] + dh[1] * (double)cy) + dh[1] * 0.5};
      int bi[2], n[2] = {src->nx, src->ny};
      for (int d = 0; d < 2; d++) {
        int v = (int)floor((c[d] - sbase[d]) * inv[d]);
        v = v < n[d] - 2 ? v : n[d] - 2;
        bi[d] = v > 0 ? v : 0;
      }
      double acc[8] = {0.0};
      for (int k = 0; k < 4; k++) {
        int nxi = bi[0] + (k & 1), nyi = bi[1] + ((k >> 1) & 1);
        double np0 = (src->pos[0] + sh[0] * (double)nxi) + sh[0] * 0.5;
        double np1 = (src->pos[1] + sh[1] * (double)nyi) + sh[1] * 0.5;
        double s0 = (double)(1 - 2 * (k & 1)), s1 = (double)(1 - 2 * ((k >> 1) & 1));
        double sf = (1.0 - (s0 * (c[0] - np0)) * inv[0]) * (1.0 - (s1 * (c[1] - np1)) * inv[1]);
        for (int q = 0; q < nq && q < 8; q++) {
          double so = us[i_old(&Ls, q, nxi, nyi)], sn = us[i_new(&Ls, src, q, nxi, nyi)];
          if (q == 0) {
            double bb = us[i_pw(&Ls, nxi, nyi)];
            so += bb;
            sn += bb;
          }
          /* the destination is a float array: every accumulation is stored */
          acc[q] = (float)(acc[q] + sf * (so * one_m_tf + sn * tf));
        }
      }
      for (int q = 0; q < nq && q < 8; q++) {
        double v = acc[q];
        if (q == 0) v = v - (double)ud[i_pw(&Ld, cx, cy)];
        ud[i_old(&Ld, q, cx, cy)] = (float)v;
      }
    }
}

/* Wall faces in the order of SolveTimestep::fillBoundaryLayers
 * (SolveTimestep.cpp:87-142); mask bit = 2*dim + upper. */
static void walls32(const pco_patch *p, float *u, uint8_t mask) {
  static const int order[4][2] = {{0, 0}, {1, 1}, {0, 1}, {1, 0}};
  lay32 L = layout(p);
  for (int k = 0; k < 4; k++) {
    int d = order[k][0], up = order[k][1];
    if (!(mask & (1u << (2 * d + up)))) continue;
    if (d == 0) {
      int xi = up ? p->nx : -1, sx = xi + (up ? -1 : 1);
      for (int yi = -1; yi < p->ny + 1; yi++)
        for (int q = 0; q < p->nq; q++) {
          float v = u[i_old(&L, q, sx, yi)];
          u[i_old(&L, q, xi, yi)] = q == 1 ? -v : v;
        }
    } else {
      int yi = up ? p->ny : -1, sy = yi + (up ? -1 : 1);
      for (int xi = -1; xi < p->nx + 1; xi++)
        for (int q = 0; q < p->nq; q++) {
          float v = u[i_old(&L, q, xi, sy)];
          u[i_old(&L, q, xi, yi)] = q == 2 ? -v : v;
        }
    }
  }
}

/* ---- f-wave in float (the restatement documented in pcoracle.c) --------- */
typedef struct {
  float gh, hu, b, eta, s, p, F;
  int wet;
} cellq32;

typedef struct {
  float halfg, dry_tol, dry_tol_update, s_min, cfl, dt_inf;
} prm32;

static inline void cell32(const prm32 *P, float h, float hu, float b, cellq32 *c) {
  c->b = b;
  c->wet = h > P->dry_tol;
  if (c->wet) {
    float s = sqrtf(h), rs = 1.0f / s, p = hu * rs;
    c->s = s; c->p = p; c->F = p * p; c->hu = hu;
  } else {
    h = h > 0.0f ? h : 0.0f;
    c->s = 0.0f; c->p = 0.0f; c->F = 0.0f; c->hu = 0.0f;
  }
  c->eta = h + b;
  c->gh = P->halfg * h;
}

static inline void fwave32(cellq32 L, cellq32 R, float o[5]) {
  if (!L.wet && !R.wet) {
    o[0] = o[1] = o[2] = o[3] = o[4] = 0.0f;
    return;
  }
  int wallR = L.wet && !R.wet && (L.eta <= R.b);
  int wallL = R.wet && !L.wet && (R.eta <= L.b);
  if (wallR) { R = L; R.hu = -L.hu; R.p = -L.p; }
  if (wallL) { L = R; L.hu = -R.hu; L.p = -R.p; }
  float a = L.gh + R.gh;
  float cb = sqrtf(a);
  float ub = (L.p + R.p) / (L.s + R.s);
  float l1 = ub - cb, l2 = ub + cb;
  float df1 = R.hu - L.hu;
  float df2 = fmaf(a, R.eta - L.eta, R.F - L.F);
  float inv = 1.0f / (2.0f * cb);
  float b1 = fmaf(l2, df1, -df2) * inv;
  float b2 = df1 - b1;
  float Lh, Lhu, Rh, Rhu;
  if (l1 < 0.0f) {
    if (l2 < 0.0f) { Lh = df1; Lhu = df2; Rh = 0.0f; Rhu = 0.0f; }
    else { Lh = b1; Lhu = b1 * l1; Rh = b2; Rhu = b2 * l2; }
  } else {
    Lh = 0.0f; Lhu = 0.0f; Rh = df1; Rhu = df2;
  }
  if (wallR) { Rh = 0.0f; Rhu = 0.0f; }
  if (wallL) { Lh = 0.0f; Lhu = 0.0f; }
  o[0] = Lh; o[1] = Lhu; o[2] = Rh; o[3] = Rhu;
  o[4] = fmaxf(fabsf(l1), fabsf(l2));
}

/* computeNumericalFluxes on uOld(+ghost) into net (3 x (nx+2)(ny+2), block
 * layout); returns the block's maxTimestep. */
static float net_updates32(const pco_patch *p, const float *u, const prm32 *P, float *net) {
  const int nx = p->nx, ny = p->ny, S = ny + 2;
  const int64_t A = (int64_t)(nx + 2) * (ny + 2);
  lay32 L = layout(p);
  const float dx = (float)(p->size[0] / (double)nx), dy = (float)(p->size[1] / (double)ny);
  const float dxi = 1.0f / dx, dyi = 1.0f / dy;
  const float *h = u + i_old(&L, 0, 0, 0), *hu = u + i_old(&L, 1, 0, 0), *hv = u + i_old(&L, 2, 0, 0);
  const float *b = u + i_pw(&L, 0, 0);
  const int64_t st = L.stride;
  float *hN = net, *huN = net + A, *hvN = net + 2 * A;
  memset(net, 0, sizeof(float) * 3 * A);
  float smax = 0.0f, o[5];
  cellq32 cl, cr;
  for (int i = 1; i < nx + 2; i++)
    for (int j = 1; j < ny + 1; j++) {
      int64_t kl = (int64_t)(i - 2) * st + (j - 1), kr = kl + st;
      cell32(P, h[kl], hu[kl], b[kl], &cl);
      cell32(P, h[kr], hu[kr], b[kr], &cr);
      fwave32(cl, cr, o);
      hN[(i - 1) * S + j] = fmaf(dxi, o[0], hN[(i - 1) * S + j]);
      huN[(i - 1) * S + j] = fmaf(dxi, o[1], huN[(i - 1) * S + j]);
      hN[i * S + j] = fmaf(dxi, o[2], hN[i * S + j]);
      huN[i * S + j] = fmaf(dxi, o[3], huN[i * S + j]);
      smax = fmaxf(smax, o[4]);
    }
  for (int i = 1; i < nx + 1; i++)
    for (int j = 1; j < ny + 2; j++) {
      int64_t kd = (int64_t)(i - 1) * st + (j - 2), ku = kd + 1;
      cell32(P, h[kd], hv[kd], b[kd], &cl);
      cell32(P, h[ku], hv[ku], b[ku], &cr);
      fwave32(cl, cr, o);
      hN[i * S + (j - 1)] = fmaf(dyi, o[0], hN[i * S + (j - 1)]);
      hvN[i * S + (j - 1)] = fmaf(dyi, o[1], hvN[i * S + (j - 1)]);
      hN[i * S + j] = fmaf(dyi, o[2], hN[i * S + j]);
      hvN[i * S + j] = fmaf(dyi, o[3], hvN[i * S + j]);
      smax = fmaxf(smax, o[4]);
    }
  if (smax > P->s_min) return P->cfl * fminf(dx / smax, dy / smax);
  return P->dt_inf;
}

/* updateUnknowns on the uOld interior, then the uNew/uOld swap. */
static void update_swap32(const pco_patch *p, float *u, const prm32 *P, const float *net, float dt) {
  const int nx = p->nx, ny = p->ny, S = ny + 2;
  const int64_t A = (int64_t)(nx + 2) * (ny + 2);
  lay32 L = layout(p);
  for (int x = 0; x < nx; x++)
    for (int y = 0; y < ny; y++) {
      int64_t k = (int64_t)(x + 1) * S + (y + 1);
      float hh = fmaf(-dt, net[k], u[i_old(&L, 0, x, y)]);
      float hu = fmaf(-dt, net[A + k], u[i_old(&L, 1, x, y)]);
      float hv = fmaf(-dt, net[2 * A + k], u[i_old(&L, 2, x, y)]);
      if (hh < P->dry_tol_update) { hu = 0.0f; hv = 0.0f; }
      if (hh < 0.0f) hh = 0.0f;
      float nv[3] = {hh, hu, hv};
      for (int q = 0; q < 3; q++) {
        /* uOld interior <- old uNew, uNew <- the updated values */
        u[i_old(&L, q, x, y)] = u[i_new(&L, p, q, x, y)];
        u[i_new(&L, p, q, x, y)] = nv[q];
      }
    }
}

static void fill32(pco_patch **patches, float **u, const pco_ghost_item *it) {
  if (it->kind == PCO_GHOST_COPY)
    transfer32(it, patches[it->src], u[it->src], patches[it->dst], u[it->dst]);
  else
    interpolate32(it, patches[it->src], u[it->src], patches[it->dst], u[it->dst]);
}

void pco32_grid_step(pco_patch **patches, float **u, int n_patches,
                     const pco_ghost_item *items, int n_items, const uint8_t *wall_mask,
                     const pco_swe_params *prm, double max_dt, double *dt_out, int n_threads) {
  prm32 P = {(float)(0.5 * prm->g), (float)prm->dry_tol, (float)prm->dry_tol_update,
             (float)prm->s_min, (float)prm->cfl, (float)prm->dt_inf};
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
#endif
  /* destinations in parallel, each with its items in list order (as
   * pco_grid_fill); the interior copies follow in the solve loop */
  int *start = NULL;
  int *ord = pco_items_by_dst(patches, n_patches, items, n_items, &start);
  if (ord) {
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 16)
#endif
    for (int p = 0; p < n_patches; p++)
      for (int q = start[p]; q < start[p + 1]; q++) fill32(patches, u, &items[ord[q]]);
    free(ord);
    free(start);
  } else {
    for (int k = 0; k < n_items; k++) fill32(patches, u, &items[k]);
  }
  float *own = (float *)malloc(sizeof(float) * (size_t)(n_patches > 0 ? n_patches : 1));
  float **nets = (float **)calloc((size_t)(n_patches > 0 ? n_patches : 1), sizeof(float *));
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 16)
#endif
  for (int p = 0; p < n_patches; p++) {
    const pco_patch *pp = patches[p];
    own[p] = P.dt_inf;
    if (!pp->is_leaf) continue;
    /* copyUNewToUOld (interior), then the domain walls */
    lay32 L = layout(pp);
    for (int q = 0; q < pp->nq; q++)
      for (int x = 0; x < pp->nx; x++)
        for (int y = 0; y < pp->ny; y++) u[p][i_old(&L, q, x, y)] = u[p][i_new(&L, pp, q, x, y)];
    walls32(pp, u[p], wall_mask ? wall_mask[p] : 0);
    nets[p] = (float *)malloc(sizeof(float) * 3 * (size_t)(pp->nx + 2) * (size_t)(pp->ny + 2));
    own[p] = net_updates32(pp, u[p], &P, nets[p]);
  }
  float dt = (float)max_dt;
  for (int p = 0; p < n_patches; p++)
    if (patches[p]->is_leaf) dt = fminf(dt, own[p]);
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 16)
#endif
  for (int p = 0; p < n_patches; p++) {
    pco_patch *pp = patches[p];
    if (!pp->is_leaf) continue;
    update_swap32(pp, u[p], &P, nets[p], dt);
    if ((double)dt > PCO_TARCH_EPS) {
      pp->time = pp->time + pp->dt;
      pp->dt = (double)dt;
    }
    pp->est_next = (double)own[p];
    free(nets[p]);
  }
  free(nets);
  free(own);
  if (dt_out) *dt_out = (double)dt;
}
