// pcg_strip_ops.cuh -- work items of the warp-strip sweep and update.
//
// Same arithmetic as k_sweep_tiles / k_update_tiles (and so as
// SWE_WaveAccumulationBlock::computeNumericalFluxes + updateUnknowns,
// tools/SWE_WaveAccumulationBlock.cpp:84-296), with another work
// decomposition: a warp owns up to G "lane groups", each a strip of hs rows
// (one row per lane, hs <= 32) and w columns of one patch, and marches the
// strip along x.  The x-edge between two columns is solved with the previous
// column's cell quantities kept in a per-lane shared-memory slot, the y-edges
// of a column with the lower neighbour taken from the next lane down (warp
// shuffle).  No CTA barrier is involved: warps are independent and the FP64
// pipe is fed by whichever warp has work.  The two strip-boundary rows are
// handled per warp before the march: the cells just below each group
// (derived once, kept in shared memory) and the edges just above each group
// (solved once, their lower-cell parts kept in shared memory for the top
// lane).
//
// The items are device functions shared by the strip kernels (pcg_strips.cu)
// and the pipelined step (pcg_pipeline.cu); kL2 reads patch data through L2
// only (ldd).
#pragma once
#include "pcg_device.cuh"

namespace pcg {
namespace strip {

// Per-warp shared memory: one entry per (group, column), G * w <= 32.
struct StripWarpSmem {
  double gh[32], b[32], eta[32], hv[32], s[32], q[32], G[32];  // cell below the group's first row
  double top_h[32], top_hv[32], top_sp[32];            // edge above the group's last row
  unsigned char wet[32];
};

template <bool kL2>
__device__ __forceinline__ void load_state(const double *__restrict__ slab, const PatchDev &P, int x,
                                           int y, double &h, double &hu, double &hv, double &b) {
  const bool inside = x >= 0 && x < P.nx && y >= 0 && y < P.ny;
  if (inside) {
    h = ldd<kL2>(slab + idx_unew(P, 0, x, y));
    hu = ldd<kL2>(slab + idx_unew(P, 1, x, y));
    hv = ldd<kL2>(slab + idx_unew(P, 2, x, y));
  } else {
    h = ldd<kL2>(slab + idx_uold(P, 0, x, y));
    hu = ldd<kL2>(slab + idx_uold(P, 1, x, y));
    hv = ldd<kL2>(slab + idx_uold(P, 2, x, y));
  }
  b = slab[idx_pw(P, 0, x, y)];
}

// Per-lane slot for the x-direction quantities of the previous column's cell.
struct StripLaneSmem {
  double gh[32], hu[32], b[32], eta[32], s[32], p[32], F[32];
  unsigned char wet[32];
};

__device__ __forceinline__ void store_x(StripLaneSmem &L, int lane, const CellQ &c) {
  L.gh[lane] = c.gh; L.hu[lane] = c.hu; L.b[lane] = c.b; L.eta[lane] = c.eta; L.s[lane] = c.s; L.p[lane] = c.p;
  L.F[lane] = c.F; L.wet[lane] = c.wet ? 1 : 0;
}
__device__ __forceinline__ CellQ load_x(const StripLaneSmem &L, int lane) {
  CellQ c;
  c.gh = L.gh[lane]; c.hu = L.hu[lane]; c.b = L.b[lane]; c.eta = L.eta[lane]; c.s = L.s[lane]; c.p = L.p[lane];
  c.F = L.F[lane]; c.wet = L.wet[lane] != 0;
  return c;
}

__device__ __forceinline__ double shfl_up_d(double v, int d) {
  return __shfl_up_sync(0xffffffffu, v, d);
}
__device__ __forceinline__ double shfl_down_d(double v, int d) {
  return __shfl_down_sync(0xffffffffu, v, d);
}

// 1 / subcell size of a patch in dimension d, correctly rounded on the
// integer pipes (same value as 1.0 / (size / n) in IEEE arithmetic).
__device__ __forceinline__ double inv_subcell(const PatchDev &P, int d) {
  return ieee::rcp_rn(ieee::div_rn(P.size[d], (double)(d == 0 ? P.nx : P.ny)));
}

// Sweep of one strip item: f-wave edges of every cell of its lane groups,
// net updates into the uOld interior, per-patch max wave speed and per-group
// CFL dt (atomics).  S and L are the warp's shared-memory slots.
template <bool kL2>
__device__ __forceinline__ void sweep_item(double *__restrict__ slab, const PatchDev *__restrict__ patches,
                                           const StripItem &I, const StripGroup *__restrict__ groups,
                                           const SweParamsDev &prm, double dry, double halfg,
                                           unsigned long long *__restrict__ patch_smax,
                                           unsigned long long *__restrict__ group_dt,
                                           const int *__restrict__ group_active, int *__restrict__ fin,
                                           const int *__restrict__ pact, StripWarpSmem &S, StripLaneSmem &L,
                                           int lane) {
  const int hs = I.hs, w = I.w, G = I.ngroups;
  const int gi = lane / hs, j = lane - gi * hs;
  const bool in_group = gi < G;
  const StripGroup SG = groups[I.g0 + (in_group ? gi : 0)];
  const PatchDev P = patches[SG.pid];
  const bool act = in_group && (!group_active || group_active[P.group]) && (!pact || pact[SG.pid]);
  // an item without an advancing lane group writes nothing: skip it whole
  // (finished groups, leaves that wait under local time stepping)
  if (!__any_sync(0xffffffffu, act)) return;
  const int y = SG.y0 + j;

  // ---- boundary rows: lane l < G*w takes (group l / w, column l % w)
  if (lane < G * w) {
    const int gh = lane / w, c = lane - gh * w;
    const StripGroup HG = groups[I.g0 + gh];
    const PatchDev &PH = patches[HG.pid];
    const int x = HG.x0 + c;
    double h, hu, hv, b;
    CellQ cx, cy, ty, ay;
    load_state<kL2>(slab, PH, x, HG.y0 - 1, h, hu, hv, b);
    cell_derived(dry, halfg, h, hu, hv, b, cx, cy);
    S.gh[lane] = cy.gh; S.b[lane] = cy.b; S.eta[lane] = cy.eta; S.hv[lane] = cy.hu; S.s[lane] = cy.s;
    S.q[lane] = cy.p; S.G[lane] = cy.F; S.wet[lane] = cy.wet ? 1 : 0;
    load_state<kL2>(slab, PH, x, HG.y0 + hs - 1, h, hu, hv, b);
    cell_derived(dry, halfg, h, hu, hv, b, cx, ty);
    load_state<kL2>(slab, PH, x, HG.y0 + hs, h, hu, hv, b);
    cell_derived(dry, halfg, h, hu, hv, b, cx, ay);
    double Lh, Lhv, Rh, Rhv, sp;
    fwave_edge(ty, ay, Lh, Lhv, Rh, Rhv, sp);
    S.top_h[lane] = Lh; S.top_hv[lane] = Lhv; S.top_sp[lane] = sp;
  }
  __syncwarp();

  const double dxi = inv_subcell(P, 0), dyi = inv_subcell(P, 1);
  double smax = 0.0;
  double h = 0.0, hu = 0.0, hv = 0.0, b = 0.0;
  // x-direction quantities of the previous column's cell live in shared
  // memory (one slot per lane) to keep the register budget small
  {
    CellQ cx, cy;
    if (act) load_state<kL2>(slab, P, SG.x0 - 1, y, h, hu, hv, b);
    cell_derived(dry, halfg, h, hu, hv, b, cx, cy);
    store_x(L, lane, cx);
  }
  // partial sums of the previous column's cell, in the accumulation order
  // of computeNumericalFluxes (x-edges left then right, y-edges lower then
  // upper): a1 = dxi * (left edge part of h), u1 = dxi * (left edge part of
  // hu); the y parts of h are added after the right edge's
  double a1 = 0.0, u1 = 0.0, yrh = 0.0, ylh = 0.0;
  // the loads of column c + 1 are issued before column c is computed
  double fh = 0.0, fhu = 0.0, fhv = 0.0, fb = 0.0;
  if (act) load_state<kL2>(slab, P, SG.x0, y, fh, fhu, fhv, fb);
  for (int c = 0; c <= w; c++) {
    const int x = SG.x0 + c;
    h = fh; hu = fhu; hv = fhv; b = fb;
    if (act && c < w) load_state<kL2>(slab, P, x + 1, y, fh, fhu, fhv, fb);
    CellQ cx, cy;
    cell_derived(dry, halfg, h, hu, hv, b, cx, cy);
    double Lh, Lhu, Rh, Rhu, sp;
    fwave_edge(load_x(L, lane), cx, Lh, Lhu, Rh, Rhu, sp);
    smax = fmax_nonneg(smax, sp);
    if (c > 0 && act) {
      double a = __fma_rn(dxi, Lh, a1);
      a = __fma_rn(dyi, yrh, a);
      slab[idx_uold(P, 0, x - 1, y)] = __fma_rn(dyi, ylh, a);
      slab[idx_uold(P, 1, x - 1, y)] = __fma_rn(dxi, Lhu, u1);
    }
    if (c == w) break;
    a1 = __fma_rn(dxi, Rh, 0.0);
    u1 = __fma_rn(dxi, Rhu, 0.0);
    store_x(L, lane, cx);
    // y-edge below this lane's cell; the lower cell comes from the next
    // lane down, or from shared memory for a group's first row
    CellQ dn;
    dn.gh = shfl_up_d(cy.gh, 1);
    dn.b = shfl_up_d(cy.b, 1);
    dn.eta = shfl_up_d(cy.eta, 1);
    dn.hu = shfl_up_d(cy.hu, 1);
    dn.s = shfl_up_d(cy.s, 1);
    dn.p = shfl_up_d(cy.p, 1);
    dn.F = shfl_up_d(cy.F, 1);
    dn.wet = __shfl_up_sync(0xffffffffu, (int)cy.wet, 1) != 0;
    const int sl = gi * w + c;
    if (j == 0 && act) {
      dn.gh = S.gh[sl]; dn.b = S.b[sl]; dn.eta = S.eta[sl]; dn.hu = S.hv[sl]; dn.s = S.s[sl];
      dn.p = S.q[sl]; dn.F = S.G[sl]; dn.wet = S.wet[sl] != 0;
    }
    double yLh, yLhv, yRh, yRhv, sp2;
    fwave_edge(dn, cy, yLh, yLhv, yRh, yRhv, sp2);
    smax = fmax_nonneg(smax, sp2);
    double uh = shfl_down_d(yLh, 1), uhv = shfl_down_d(yLhv, 1);
    if (j == hs - 1 && act) {
      uh = S.top_h[sl];
      uhv = S.top_hv[sl];
      smax = fmax_nonneg(smax, S.top_sp[sl]);
    }
    yrh = yRh;
    ylh = uh;
    // hv only has y-edge parts: complete for this column already
    if (act) slab[idx_uold(P, 2, x, y)] = __fma_rn(dyi, uhv, __fma_rn(dyi, yRhv, 0.0));
  }
  __syncwarp();  // S is reused by the next item

  // ---- per-group max wave speed (speeds >= 0: bit patterns order like values)
  unsigned long long m = act ? dbits(smax) : 0ull;
  for (int o = 1; o < 32; o <<= 1) {
    unsigned long long other = __shfl_down_sync(0xffffffffu, m, o);
    if (j + o < hs) m = other > m ? other : m;
  }
  if (act && j == 0) {
    if (fin) atomicOr(&fin[SG.pid], kFinUOld);
    atomicMax(&patch_smax[SG.pid], m);
    const double dtc = cfl_dt(prm, bitsd(m), subcell(P, 0), subcell(P, 1));
    atomicMin(&group_dt[P.group], dbits(dtc));
  }
}

// Update of one strip item with its group's dt (or the patch's own dt under
// local time stepping): uNew <- uNew - dt * net update (dry clamps), uOld
// interior <- previous uNew (only the bands of ub, see UpdateBands), time
// interval and next CFL estimate of the patch.  kBatch columns are loaded
// before any of them is stored.
template <bool kL2, int kBatch = 4>
__device__ __forceinline__ void update_item(double *__restrict__ slab, const PatchDev *__restrict__ patches,
                                            PatchTimeDev *__restrict__ times, const StripItem &I,
                                            const StripGroup *__restrict__ groups, const SweParamsDev &prm,
                                            const unsigned long long *__restrict__ patch_smax,
                                            const unsigned long long *__restrict__ group_dt,
                                            const int *__restrict__ group_active, int *__restrict__ fin,
                                            const int *__restrict__ pact, const unsigned long long *__restrict__ pdt,
                                            const UpdateBands &ub, int lane) {
  const int hs = I.hs, w = I.w, G = I.ngroups;
  const int gi = lane / hs, j = lane - gi * hs;
  if (gi >= G) return;
  const StripGroup SG = groups[I.g0 + gi];
  const PatchDev P = patches[SG.pid];
  if (group_active && !group_active[P.group]) return;
  if (pact && !pact[SG.pid]) return;
  const double dt = bitsd(pdt ? pdt[SG.pid] : group_dt[P.group]);
  const int y = SG.y0 + j;
  const long long vn = vol_new(P), vo = vol_old(P);
  long long in0 = idx_unew(P, 0, SG.x0, y), io0 = idx_uold(P, 0, SG.x0, y);
  const int sn = P.ny, so = P.ny + 2 * P.g;
  // old-state writes: this lane's row and the columns of the x bands
  int bx0 = P.nx, bx1 = 0;
  bool row_old = true;
  if (ub.band && !*ub.full &&
      gt_nonneg(__dsub_rn(ub.group_t_end[P.group], __dadd_rn(ub.group_time[P.group], dt)), 0.0)) {
    const int4 bd = ub.band[SG.pid];
    bx0 = bd.x;
    bx1 = P.nx - bd.y;
    row_old = y < bd.z || y >= P.ny - bd.w;
  }
  // loads of kBatch columns are issued before their stores (loads and
  // stores go through the same pointer, so the compiler cannot reorder them)
  bool big = false;  // an old value written to uOld is 2^1022 or more (or NaN)
  for (int c0 = 0; c0 < w; c0 += kBatch) {
    double st[kBatch][3], nt[kBatch][3];
#pragma unroll
    for (int k = 0; k < kBatch; k++) {
      if (c0 + k < w) {
        const long long a = in0 + (long long)k * sn, o = io0 + (long long)k * so;
        st[k][0] = ldd<kL2>(slab + a); st[k][1] = ldd<kL2>(slab + a + vn); st[k][2] = ldd<kL2>(slab + a + 2 * vn);
        nt[k][0] = ldd<kL2>(slab + o); nt[k][1] = ldd<kL2>(slab + o + vo); nt[k][2] = ldd<kL2>(slab + o + 2 * vo);
      }
    }
#pragma unroll
    for (int k = 0; k < kBatch; k++) {
      if (c0 + k < w) {
        const long long a = in0 + (long long)k * sn, o = io0 + (long long)k * so;
        double nh = __fma_rn(-dt, nt[k][0], st[k][0]);
        double nhu = __fma_rn(-dt, nt[k][1], st[k][1]);
        double nhv = __fma_rn(-dt, nt[k][2], st[k][2]);
        if (lt_ieee(nh, prm.dry_tol_update)) { nhu = 0.0; nhv = 0.0; }
        if (lt_zero(nh)) nh = 0.0;
        const int x = SG.x0 + c0 + k;
        if (row_old || x < bx0 || x >= bx1) {
          slab[o] = st[k][0]; slab[o + vo] = st[k][1]; slab[o + 2 * vo] = st[k][2];
        }
        slab[a] = nh; slab[a + vn] = nhu; slab[a + 2 * vn] = nhv;
        big |= !(small_mag(st[k][0]) && small_mag(st[k][1]) && small_mag(st[k][2]));
      }
    }
    in0 += (long long)kBatch * sn;
    io0 += (long long)kBatch * so;
  }
  if (fin && big) atomicAnd(&fin[SG.pid], ~kFinUOld);
  if (j == 0 && SG.x0 == 0 && SG.y0 == 0) {
    PatchTimeDev &T = times[SG.pid];
    if (tl_greater(dt, 0.0)) {
      T.time = __dadd_rn(T.time, T.dt);
      T.dt = dt;
    }
    T.est_next = cfl_dt(prm, bitsd(patch_smax[SG.pid]), subcell(P, 0), subcell(P, 1));
  }
}

}  // namespace strip
}  // namespace pcg
