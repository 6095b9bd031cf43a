// pcg_fused.cu -- the fused form of the batched synchronous step.
//
// One kernel per timestep does, per warp-strip item, what the unfused step
// does in four launches: the ghost fill of the strip's faces (copies and
// coarse-fine interpolations from the neighbours, reflecting walls), the
// update of the previous step, the f-wave sweep with the accumulation of the
// net updates, and the CFL reduction
// (SWE_WaveAccumulationBlock::computeNumericalFluxes + updateUnknowns,
// tools/SWE_WaveAccumulationBlock.cpp:84-296, and the compositor's face
// functors, GhostlayerCompositorFunctors.cpp:23-221).
//
// Deferred update.  The update q <- q - dt dq of step s needs dt_s, the
// minimum over every patch of the group, which is known only after the whole
// sweep.  So the update of step s is applied when step s + 1 loads its cells:
// a patch keeps two state copies, A (its reference-layout uNew and uOld
// interior) and B (6 nx ny doubles in the context's shadow buffer), each
// holding a state Q and the net updates D computed from it.  Step s + 1 reads
// the set R written by step s and computes the current state upd(Q, D, dt_s)
// for every cell it touches (its own cells, its strip's halo, the source
// cells of its ghost layer), sweeps it, and writes the state and the new net
// updates to the other set W.  Reads and writes never meet, so warps need no
// ordering between patches or strips.  The reference layout (uNew = new
// state, uOld interior = previous state, ghost layer as filled) is produced
// on demand by k_fused_flush (same arithmetic as k_update_strips) plus the
// wall fill from the previous state.  Every operation is the one the unfused
// step issues, so states and dts agree bit for bit.
//
// Before the first fused step of a group (pend == 0) its state is in the
// reference layout: uNew is the state, the uOld interior the previous state.
// That is set A read as (state, old) instead of (Q, D).
#include "pcg_device.cuh"
#include "pcg_kernels.h"

namespace pcg {

namespace {

// One state set of a patch: Q (or uNew) and D (or uOld interior), each three
// planes at (q, x, y) -> base + q * plane + x * row + y.
struct SetView {
  double *q, *d;
  int qrow, qplane, drow, dplane;
};

__device__ __forceinline__ SetView set_view(double *slab, double *shadow, const PatchDev &P, int which) {
  SetView v;
  const int vn = P.nx * P.ny;
  v.qrow = P.ny;
  v.qplane = vn;
  if (which == 0) {
    v.q = slab + P.off;
    v.d = slab + idx_uold(P, 0, 0, 0);
    v.drow = P.ny + 2 * P.g;
    v.dplane = (P.nx + 2 * P.g) * (P.ny + 2 * P.g);
  } else {
    v.q = shadow + P.sh_off;
    v.d = v.q + 3 * vn;
    v.drow = P.ny;
    v.dplane = vn;
  }
  return v;
}

// The read side of a patch in the current step: its set R, the pending dt
// and whether an update is pending.
struct ReadView {
  SetView s;
  double dt;
  bool pend;
  int which;
};

__device__ __forceinline__ ReadView read_view(const FusedDev &F, const PatchDev &P) {
  ReadView r;
  const int g = P.group;
  r.pend = F.pend[g] != 0;
  r.which = r.pend ? F.par[g] : 0;
  r.s = set_view(F.slab, F.shadow, P, r.which);
  r.dt = bitsd(F.dt_prev[g]);
  return r;
}

// The read side of another patch of the same group (a ghost source).
__device__ __forceinline__ ReadView read_view_as(const FusedDev &F, const PatchDev &S, const ReadView &same) {
  ReadView r = same;
  r.s = set_view(F.slab, F.shadow, S, same.which);
  return r;
}

// Raw values of one cell of set R.
struct Raw {
  double q0, q1, q2, d0, d1, d2;
};

__device__ __forceinline__ void load_raw(const ReadView &R, int x, int y, Raw &r) {
  const double *q = R.s.q + x * R.s.qrow + y;
  const double *d = R.s.d + x * R.s.drow + y;
  r.q0 = q[0];
  r.q1 = q[R.s.qplane];
  r.q2 = q[2 * R.s.qplane];
  r.d0 = d[0];
  r.d1 = d[R.s.dplane];
  r.d2 = d[2 * R.s.dplane];
}

// updateUnknowns of one cell (tools/SWE_WaveAccumulationBlock.cpp:247-296):
// the same operations as k_update_strips.
__device__ __forceinline__ void update_cell(double dry_tol_update, double dt, double q0, double q1, double q2,
                                            double d0, double d1, double d2, double &h, double &hu,
                                            double &hv) {
  h = __fma_rn(-dt, d0, q0);
  hu = __fma_rn(-dt, d1, q1);
  hv = __fma_rn(-dt, d2, q2);
  if (lt_ieee(h, dry_tol_update)) { hu = 0.0; hv = 0.0; }
  if (lt_zero(h)) h = 0.0;
}

// Current state of a raw cell.
__device__ __forceinline__ void state_of(const ReadView &R, double dtu, const Raw &r, double &h, double &hu,
                                         double &hv) {
  if (R.pend) {
    update_cell(dtu, R.dt, r.q0, r.q1, r.q2, r.d0, r.d1, r.d2, h, hu, hv);
  } else {
    h = r.q0; hu = r.q1; hv = r.q2;
  }
}

// Previous state (what uOld holds in the reference layout during the fill).
__device__ __forceinline__ void old_of(const ReadView &R, const Raw &r, double &o0, double &o1, double &o2) {
  if (R.pend) { o0 = r.q0; o1 = r.q1; o2 = r.q2; }
  else { o0 = r.d0; o1 = r.d1; o2 = r.d2; }
}

// Current state of interior cell (x, y).
__device__ __forceinline__ void interior_state(const ReadView &R, double dtu, int x, int y, double &h, double &hu,
                                               double &hv) {
  Raw r;
  load_raw(R, x, y, r);
  state_of(R, dtu, r, h, hu, hv);
}

// Ghost cell (x, y) of patch D (id pid, read view RD): a face cell of a
// reflecting wall mirrors the adjacent interior cell's current state with the
// normal momentum negated (SWEKernel::fillBoundaryLayer,
// native/SWEKernel.cpp:176-237); otherwise the ghost item that writes the cell
// is evaluated with the arithmetic of k_ghost_cells on its source's current
// and previous states; a face cell no item writes keeps the ghost layer's
// value.  Written to the ghost layer (corners of walls are filled by the
// flush: the sweep does not read corners).
__device__ __forceinline__ void ghost_cell(const FusedDev &F, int pid, const PatchDev &D, const ReadView &RD, int x,
                                           int y, double &h, double &hu, double &hv) {
  const double dtu = F.prm.dry_tol_update;
  const bool ox = x < 0 || x >= D.nx, oy = y < 0 || y >= D.ny;
  int code;
  if (ox && oy) {
    code = F.corner[4 * pid + (x >= D.nx ? 1 : 0) + (y >= D.ny ? 2 : 0)];
    if (code == -1) return;
  } else {
    int face, off;
    if (x < 0) { face = 0; off = y; }
    else if (x >= D.nx) { face = 1; off = D.ny + y; }
    else if (y < 0) { face = 2; off = 2 * D.ny + x; }
    else { face = 3; off = 2 * D.ny + D.nx + x; }
    if (D.wall & (1 << face)) {
      const int ix = face == 0 ? 0 : (face == 1 ? D.nx - 1 : x);
      const int iy = face == 2 ? 0 : (face == 3 ? D.ny - 1 : y);
      interior_state(RD, dtu, ix, iy, h, hu, hv);
      if (face < 2) hu = neg(hu);
      else hv = neg(hv);
      code = -1;
    } else {
      code = F.face[D.face_begin + off];
      if (code == -1) {
        h = F.slab[idx_uold(D, 0, x, y)];
        hu = F.slab[idx_uold(D, 1, x, y)];
        hv = F.slab[idx_uold(D, 2, x, y)];
        return;
      }
    }
  }
  if (code >= 0) {
    const FusedCopyDev cp = F.copies[code];
    const GhostItemStepDev I = F.item_step[cp.item];
    const ReadView R = read_view_as(F, F.patches[cp.src], RD);
    Raw r;
    load_raw(R, cp.sx, cp.sy, r);
    double n0, n1, n2, o0, o1, o2;
    state_of(R, dtu, r, n0, n1, n2);
    old_of(R, r, o0, o1, o2);
    h = __dadd_rn(__dmul_rn(n0, I.tf), __dmul_rn(o0, I.itf));
    hu = __dadd_rn(__dmul_rn(n1, I.tf), __dmul_rn(o1, I.itf));
    hv = __dadd_rn(__dmul_rn(n2, I.tf), __dmul_rn(o2, I.itf));
  } else if (code <= -2) {
    const FusedInterpDev pl = F.interps[-code - 2];
    const GhostItemStepDev I = F.item_step[pl.item];
    const PatchDev S = F.patches[pl.src];
    const ReadView R = read_view_as(F, S, RD);
    const double tf = I.tf, one_m_tf = I.itf;
    // time factor 1: (old [+ b]) * 0 + (new [+ b]) * 1 is new [+ b] up to the
    // sign of a zero, which the accumulator (started at +0, never -0)
    // absorbs, as long as old [+ b] is finite (both below 2^1022 in
    // magnitude); otherwise (rare) the whole expression
    const bool one = dbits(tf) == 0x3FF0000000000000ull;
    bool fast = one;
    double a0 = 0.0, a1 = 0.0, a2 = 0.0;
#pragma unroll 1
    for (int pass = 0; pass < 2; pass++) {
      if (pass == 1) {
        if (fast) break;
        a0 = a1 = a2 = 0.0;
      }
#pragma unroll
      for (int kk = 0; kk < 4; kk++) {
        const int sx = pl.bx + (kk & 1), sy = pl.by + ((kk >> 1) & 1);
        Raw r;
        load_raw(R, sx, sy, r);
        const double bb = F.slab[idx_pw(S, 0, sx, sy)];
        double n0, n1, n2, o0, o1, o2;
        state_of(R, dtu, r, n0, n1, n2);
        old_of(R, r, o0, o1, o2);
        const double sf = pl.sf[kk];
        if (pass == 0) {
          fast = fast && small_mag(o0) && small_mag(o1) && small_mag(o2) && small_mag(bb);
          a0 = __dadd_rn(a0, __dmul_rn(sf, __dadd_rn(n0, bb)));
          a1 = __dadd_rn(a1, __dmul_rn(sf, n1));
          a2 = __dadd_rn(a2, __dmul_rn(sf, n2));
        } else {
          const double so0 = __dadd_rn(o0, bb), sn0 = __dadd_rn(n0, bb);
          a0 = __dadd_rn(a0, __dmul_rn(sf, __dadd_rn(__dmul_rn(so0, one_m_tf), __dmul_rn(sn0, tf))));
          a1 = __dadd_rn(a1, __dmul_rn(sf, __dadd_rn(__dmul_rn(o1, one_m_tf), __dmul_rn(n1, tf))));
          a2 = __dadd_rn(a2, __dmul_rn(sf, __dadd_rn(__dmul_rn(o2, one_m_tf), __dmul_rn(n2, tf))));
        }
      }
    }
    h = __dadd_rn(a0, __dmul_rn(-1.0, F.slab[idx_pw(D, 0, x, y)]));
    hu = a1;
    hv = a2;
  }
  F.slab[idx_uold(D, 0, x, y)] = h;
  F.slab[idx_uold(D, 1, x, y)] = hu;
  F.slab[idx_uold(D, 2, x, y)] = hv;
}

// Per-warp shared memory: the cells just outside each lane group's strip
// (derived), the edge just above it, and every lane's left / right face
// ghost.  Before the boundary rows are derived, the bottom / top face ghosts
// of a boundary lane wait in that lane's slots of hv, s, q / top_h, top_hv,
// top_sp.
struct FusedWarpSmem {
  double gh[32], b[32], eta[32], hv[32], s[32], q[32], G[32];
  double top_h[32], top_hv[32], top_sp[32];
  double gl[3][32], gr[3][32];
  unsigned char wet[32];
};

struct FusedLaneSmem {
  double gh[32], hu[32], b[32], eta[32], s[32], p[32], F[32];
  unsigned char wet[32];
};

__device__ __forceinline__ void store_x(FusedLaneSmem &L, int lane, const CellQ &c) {
  L.gh[lane] = c.gh; L.hu[lane] = c.hu; L.b[lane] = c.b; L.eta[lane] = c.eta; L.s[lane] = c.s; L.p[lane] = c.p;
  L.F[lane] = c.F; L.wet[lane] = c.wet ? 1 : 0;
}
__device__ __forceinline__ CellQ load_x(const FusedLaneSmem &L, int lane) {
  CellQ c;
  c.gh = L.gh[lane]; c.hu = L.hu[lane]; c.b = L.b[lane]; c.eta = L.eta[lane]; c.s = L.s[lane]; c.p = L.p[lane];
  c.F = L.F[lane]; c.wet = L.wet[lane] != 0;
  return c;
}

__device__ __forceinline__ double shfl_up_d(double v, int d) { return __shfl_up_sync(0xffffffffu, v, d); }
__device__ __forceinline__ double shfl_down_d(double v, int d) { return __shfl_down_sync(0xffffffffu, v, d); }

__device__ __forceinline__ double inv_subcell(const PatchDev &P, int d) {
  return ieee::rcp_rn(ieee::div_rn(P.size[d], (double)(d == 0 ? P.nx : P.ny)));
}

}  // namespace

template <int kWarps, int kMinBlocks>
__global__ void __launch_bounds__(kWarps * 32, kMinBlocks)
    k_fused_strips(FusedDev F, const StripItem *__restrict__ items, const StripGroup *__restrict__ groups,
                   int count, unsigned long long *__restrict__ patch_smax,
                   unsigned long long *__restrict__ group_dt) {
  __shared__ FusedWarpSmem SM[kWarps];
  __shared__ FusedLaneSmem LS[kWarps];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  FusedWarpSmem &S = SM[wid];
  const SweParamsDev &prm = F.prm;
  const double dry = prm.dry_tol, dtu = prm.dry_tol_update;
  const double halfg = __dmul_rn(0.5, prm.g);
  for (int it = blockIdx.x * kWarps + wid; it < count; it += gridDim.x * kWarps) {
    const StripItem I = items[it];
    const int hs = I.hs, w = I.w, G = I.ngroups;
    const int gi = lane / hs, j = lane - gi * hs;
    const bool in_group = gi < G;
    const StripGroup SG = groups[I.g0 + (in_group ? gi : 0)];
    const PatchDev P = F.patches[SG.pid];
    const bool act = in_group && F.active[P.group];
    if (!__any_sync(0xffffffffu, act)) continue;
    const int y = SG.y0 + j;

    // ---- ghost cells this lane evaluates, in one loop: 0 / 1 the left /
    // right face cell of its row, 2 / 3 the bottom / top face cell of its
    // boundary column (lane l < G*w takes group l / w, column l % w), 4 - 7
    // the corners of its boundary group (ghost layer only)
    const bool bl = lane < G * w;
    const int gh = bl ? lane / w : 0, c = bl ? lane - gh * w : 0;
    const StripGroup HG = groups[I.g0 + gh];
    const PatchDev PH = F.patches[HG.pid];
    const bool hact = bl && F.active[PH.group];
#pragma unroll 1
    for (int t = 0; t < 8; t++) {
      bool on;
      int x, yy;
      switch (t) {
        case 0: on = act && SG.x0 == 0; x = -1; yy = y; break;
        case 1: on = act && SG.x0 + w == P.nx; x = P.nx; yy = y; break;
        case 2: on = hact && HG.y0 == 0; x = HG.x0 + c; yy = -1; break;
        case 3: on = hact && HG.y0 + hs == PH.ny; x = HG.x0 + c; yy = PH.ny; break;
        case 4: on = hact && c == 0 && HG.x0 == 0 && HG.y0 == 0; x = -1; yy = -1; break;
        case 5: on = hact && c == 0 && HG.x0 == 0 && HG.y0 + hs == PH.ny; x = -1; yy = PH.ny; break;
        case 6: on = hact && c == w - 1 && HG.x0 + w == PH.nx && HG.y0 == 0; x = PH.nx; yy = -1; break;
        default: on = hact && c == w - 1 && HG.x0 + w == PH.nx && HG.y0 + hs == PH.ny; x = PH.nx; yy = PH.ny; break;
      }
      if (!__any_sync(0xffffffffu, on)) continue;
      if (on) {
        const bool own = t < 2;
        const int pid = own ? SG.pid : HG.pid;
        const PatchDev D = F.patches[pid];
        const ReadView RD = read_view(F, D);
        double h = 0.0, hu = 0.0, hv = 0.0;
        ghost_cell(F, pid, D, RD, x, yy, h, hu, hv);
        double *s0 = t == 0 ? S.gl[0] : t == 1 ? S.gr[0] : t == 2 ? S.hv : S.top_h;
        double *s1 = t == 0 ? S.gl[1] : t == 1 ? S.gr[1] : t == 2 ? S.s : S.top_hv;
        double *s2 = t == 0 ? S.gl[2] : t == 1 ? S.gr[2] : t == 2 ? S.q : S.top_sp;
        if (t < 4) { s0[lane] = h; s1[lane] = hu; s2[lane] = hv; }
      }
    }
    __syncwarp();

    // ---- boundary rows of the boundary lanes: the derived cell below each
    // group and the edge above it
    if (hact) {
      const ReadView RH = read_view(F, PH);
      const int x = HG.x0 + c;
      double h, hu, hv;
      CellQ cx, cy, ty, ay;
      if (HG.y0 == 0) { h = S.hv[lane]; hu = S.s[lane]; hv = S.q[lane]; }
      else interior_state(RH, dtu, x, HG.y0 - 1, h, hu, hv);
      cell_derived(dry, halfg, h, hu, hv, F.slab[idx_pw(PH, 0, x, HG.y0 - 1)], cx, cy);
      S.gh[lane] = cy.gh; S.b[lane] = cy.b; S.eta[lane] = cy.eta; S.hv[lane] = cy.hu; S.s[lane] = cy.s;
      S.q[lane] = cy.p; S.G[lane] = cy.F; S.wet[lane] = cy.wet ? 1 : 0;
      interior_state(RH, dtu, x, HG.y0 + hs - 1, h, hu, hv);
      cell_derived(dry, halfg, h, hu, hv, F.slab[idx_pw(PH, 0, x, HG.y0 + hs - 1)], cx, ty);
      if (HG.y0 + hs == PH.ny) { h = S.top_h[lane]; hu = S.top_hv[lane]; hv = S.top_sp[lane]; }
      else interior_state(RH, dtu, x, HG.y0 + hs, h, hu, hv);
      cell_derived(dry, halfg, h, hu, hv, F.slab[idx_pw(PH, 0, x, HG.y0 + hs)], cx, ay);
      double Lh, Lhv, Rh, Rhv, sp;
      fwave_edge(ty, ay, Lh, Lhv, Rh, Rhv, sp);
      S.top_h[lane] = Lh; S.top_hv[lane] = Lhv; S.top_sp[lane] = sp;
    }
    const ReadView R = read_view(F, P);
    __syncwarp();

    const SetView W = set_view(F.slab, F.shadow, P, R.pend ? 1 - F.par[P.group] : 1);
    const double dxi = inv_subcell(P, 0), dyi = inv_subcell(P, 1);
    double smax = 0.0;
    double h = 0.0, hu = 0.0, hv = 0.0, b = 0.0;
    FusedLaneSmem &L = LS[wid];
    {
      CellQ cx, cy;
      if (act) {
        if (SG.x0 == 0) { h = S.gl[0][lane]; hu = S.gl[1][lane]; hv = S.gl[2][lane]; }
        else interior_state(R, dtu, SG.x0 - 1, y, h, hu, hv);
        b = F.slab[idx_pw(P, 0, SG.x0 - 1, y)];
      }
      cell_derived(dry, halfg, h, hu, hv, b, cx, cy);
      store_x(L, lane, cx);
    }
    double a1 = 0.0, u1 = 0.0, yrh = 0.0, ylh = 0.0;
    // raw values of column c + 1 are loaded before column c is computed
    Raw fr{0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    double fb = 0.0;
    bool fghost = false;
    if (act) {
      load_raw(R, SG.x0, y, fr);
      fb = F.slab[idx_pw(P, 0, SG.x0, y)];
    }
    for (int c = 0; c <= w; c++) {
      const int x = SG.x0 + c;
      if (fghost) { h = fr.q0; hu = fr.q1; hv = fr.q2; }
      else state_of(R, dtu, fr, h, hu, hv);
      b = fb;
      // the state of an own cell is this step's Q of set W
      if (act && c < w) {
        double *wq = W.q + x * W.qrow + y;
        wq[0] = h; wq[W.qplane] = hu; wq[2 * W.qplane] = hv;
      }
      if (act && c < w) {
        if (c + 1 == w && SG.x0 + w == P.nx) {
          fr.q0 = S.gr[0][lane]; fr.q1 = S.gr[1][lane]; fr.q2 = S.gr[2][lane];
          fghost = true;
        } else {
          load_raw(R, x + 1, y, fr);
        }
        fb = F.slab[idx_pw(P, 0, x + 1, y)];
      }
      CellQ cx, cy;
      cell_derived(dry, halfg, h, hu, hv, b, cx, cy);
      double Lh, Lhu, Rh, Rhu, sp;
      fwave_edge(load_x(L, lane), cx, Lh, Lhu, Rh, Rhu, sp);
      smax = fmax_nonneg(smax, sp);
      if (c > 0 && act) {
        double a = __fma_rn(dxi, Lh, a1);
        a = __fma_rn(dyi, yrh, a);
        double *wd = W.d + (x - 1) * W.drow + y;
        wd[0] = __fma_rn(dyi, ylh, a);
        wd[W.dplane] = __fma_rn(dxi, Lhu, u1);
      }
      if (c == w) break;
      a1 = __fma_rn(dxi, Rh, 0.0);
      u1 = __fma_rn(dxi, Rhu, 0.0);
      store_x(L, lane, cx);
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
      if (act) W.d[x * W.drow + y + 2 * W.dplane] = __fma_rn(dyi, uhv, __fma_rn(dyi, yRhv, 0.0));
    }
    __syncwarp();  // S is reused by the next item

    // ---- per-group max wave speed (speeds >= 0: bit patterns order like values)
    unsigned long long m = act ? dbits(smax) : 0ull;
    for (int o = 1; o < 32; o <<= 1) {
      unsigned long long other = __shfl_down_sync(0xffffffffu, m, o);
      if (j + o < hs) m = other > m ? other : m;
    }
    if (act && j == 0) {
      atomicMax(&patch_smax[SG.pid], m);
      const double dtc = cfl_dt(prm, bitsd(m), subcell(P, 0), subcell(P, 1));
      atomicMin(&group_dt[P.group], dbits(dtc));
    }
  }
}

// End of a fused step: the time intervals of every leaf of an active group
// (time += dt, dt and the CFL estimate, as k_update_strips), and in block 0
// the dt record, the group time, the pending dt and which set the step wrote.
__global__ void k_fused_advance(FusedDev F, const int *__restrict__ leaf_ids, int n_leaves,
                                PatchTimeDev *__restrict__ times,
                                const unsigned long long *__restrict__ patch_smax, int n_groups,
                                const unsigned long long *__restrict__ group_dt, double *__restrict__ group_time,
                                int *__restrict__ pend, int *__restrict__ par,
                                unsigned long long *__restrict__ dt_prev, double *__restrict__ hist,
                                int *__restrict__ counter, int capacity) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n_leaves; k += gridDim.x * blockDim.x) {
    const int p = leaf_ids[k];
    const PatchDev P = F.patches[p];
    if (!F.active[P.group]) continue;
    const double dt = bitsd(group_dt[P.group]);
    PatchTimeDev &T = times[p];
    if (tl_greater(dt, 0.0)) {
      T.time = __dadd_rn(T.time, T.dt);
      T.dt = dt;
    }
    T.est_next = cfl_dt(F.prm, bitsd(patch_smax[p]), subcell(P, 0), subcell(P, 1));
  }
  if (blockIdx.x != 0) return;
  __shared__ int idx;
  if (threadIdx.x == 0) idx = *counter;
  __syncthreads();
  for (int g = threadIdx.x; g < n_groups; g += blockDim.x) {
    if (idx < capacity) hist[(long long)idx * n_groups + g] = bitsd(group_dt[g]);
    if (F.active[g]) {
      group_time[g] = __dadd_rn(group_time[g], bitsd(group_dt[g]));
      dt_prev[g] = group_dt[g];
      par[g] = pend[g] ? 1 - par[g] : 1;
      pend[g] = 1;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) *counter = idx + 1;
}

// The reference layout of every leaf of a group with a pending update:
// uNew <- upd(Q, D, dt), uOld interior <- Q (k_update_strips' arithmetic and
// its swap).  One CTA per leaf.
__global__ void k_fused_flush(FusedDev F, const int *__restrict__ leaf_ids, int n_leaves) {
  for (int k = blockIdx.x; k < n_leaves; k += gridDim.x) {
    const int p = leaf_ids[k];
    const PatchDev P = F.patches[p];
    if (!F.pend[P.group]) continue;
    const ReadView R = read_view(F, P);
    const SetView A = set_view(F.slab, F.shadow, P, 0);
    const int n = P.nx * P.ny;
    for (int c = threadIdx.x; c < n; c += blockDim.x) {
      const int x = c / P.ny, y = c - x * P.ny;
      Raw r;
      load_raw(R, x, y, r);
      double h, hu, hv;
      update_cell(F.prm.dry_tol_update, R.dt, r.q0, r.q1, r.q2, r.d0, r.d1, r.d2, h, hu, hv);
      double *o = A.d + x * A.drow + y;
      o[0] = r.q0; o[A.dplane] = r.q1; o[2 * A.dplane] = r.q2;
      double *u = A.q + x * A.qrow + y;
      u[0] = h; u[A.qplane] = hu; u[2 * A.qplane] = hv;
    }
  }
}

// Face / corner tables and evaluation plans of the fused step from the flat
// ghost-cell list (copies first) and the interpolation plan.
__global__ void k_build_fused_ghosts(const PatchDev *__restrict__ patches, const GhostItemDev *__restrict__ items,
                                     const GhostCellDev *__restrict__ cells, int ncopy, int ninterp,
                                     const InterpPlanDev *__restrict__ plan, const int *__restrict__ face_begin,
                                     int *__restrict__ face, int *__restrict__ corner,
                                     FusedCopyDev *__restrict__ copies, FusedInterpDev *__restrict__ interps) {
  const int total = ncopy + ninterp;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
    const GhostCellDev gc = cells[e];
    const GhostItemDev it = items[gc.item];
    const PatchDev D = patches[it.dst];
    const int kx = gc.k / it.size[1], ky = gc.k - kx * it.size[1];
    const int cx = it.dst_off[0] + kx, cy = it.dst_off[1] + ky;
    int code;
    if (e < ncopy) {
      FusedCopyDev cp;
      cp.item = gc.item;
      cp.src = it.src;
      cp.sx = (short)(it.src_off[0] + kx);
      cp.sy = (short)(it.src_off[1] + ky);
      cp.pad_ = 0;
      copies[e] = cp;
      code = e;
    } else {
      const InterpPlanDev pl = plan[e - ncopy];
      FusedInterpDev fi;
      fi.item = gc.item;
      fi.src = it.src;
      fi.bx = pl.bx;
      fi.by = pl.by;
      for (int k = 0; k < 4; k++) fi.sf[k] = pl.sf[k];
      interps[e - ncopy] = fi;
      code = -(e - ncopy) - 2;
    }
    const bool ox = cx < 0 || cx >= D.nx, oy = cy < 0 || cy >= D.ny;
    if (ox && oy) corner[4 * it.dst + (cx >= D.nx ? 1 : 0) + (cy >= D.ny ? 2 : 0)] = code;
    else if (ox) face[face_begin[it.dst] + (cx < 0 ? cy : D.ny + cy)] = code;
    else if (oy) face[face_begin[it.dst] + 2 * D.ny + (cy < 0 ? cx : D.nx + cx)] = code;
  }
}

namespace {

template <int kWarps, int kMinBlocks>
cudaError_t fused_t(cudaStream_t st, int grid, const FusedDev &F, const StripItem *items,
                    const StripGroup *groups, int count, unsigned long long *patch_smax,
                    unsigned long long *group_dt) {
  if (count <= 0) return cudaSuccess;
  k_fused_strips<kWarps, kMinBlocks><<<grid, kWarps * 32, 0, st>>>(F, items, groups, count, patch_smax, group_dt);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_fused_strips(cudaStream_t st, int variant, int grid, const FusedDev &F, const StripItem *items,
                                const StripGroup *groups, int count, unsigned long long *patch_smax,
                                unsigned long long *group_dt) {
  switch (variant) {
    case 0: return fused_t<4, 4>(st, grid, F, items, groups, count, patch_smax, group_dt);
    case 1: return fused_t<4, 5>(st, grid, F, items, groups, count, patch_smax, group_dt);
    case 2: return fused_t<8, 2>(st, grid, F, items, groups, count, patch_smax, group_dt);
    case 3: return fused_t<8, 3>(st, grid, F, items, groups, count, patch_smax, group_dt);
    case 4: return fused_t<6, 3>(st, grid, F, items, groups, count, patch_smax, group_dt);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t fused_occupancy(int variant, int *blocks_per_sm) {
  switch (variant) {
    case 0: return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_fused_strips<4, 4>, 128, 0);
    case 1: return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_fused_strips<4, 5>, 128, 0);
    case 2: return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_fused_strips<8, 2>, 256, 0);
    case 3: return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_fused_strips<8, 3>, 256, 0);
    case 4: return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_fused_strips<6, 3>, 192, 0);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_fused_advance(cudaStream_t st, const FusedDev &F, const int *leaf_ids, int n_leaves,
                                 PatchTimeDev *times, const unsigned long long *patch_smax, int n_groups,
                                 const unsigned long long *group_dt, double *group_time, int *pend, int *par,
                                 unsigned long long *dt_prev, double *hist, int *counter, int capacity) {
  int grid = (n_leaves + 255) / 256;
  if (grid > 152 * 8) grid = 152 * 8;
  if (grid < 1) grid = 1;
  k_fused_advance<<<grid, 256, 0, st>>>(F, leaf_ids, n_leaves, times, patch_smax, n_groups, group_dt, group_time,
                                        pend, par, dt_prev, hist, counter, capacity);
  return cudaGetLastError();
}

cudaError_t launch_fused_flush(cudaStream_t st, const FusedDev &F, const int *leaf_ids, int n_leaves) {
  if (n_leaves <= 0) return cudaSuccess;
  int grid = n_leaves < 152 * 16 ? n_leaves : 152 * 16;
  k_fused_flush<<<grid, 256, 0, st>>>(F, leaf_ids, n_leaves);
  return cudaGetLastError();
}

cudaError_t launch_build_fused_ghosts(cudaStream_t st, const PatchDev *patches, const GhostItemDev *items,
                                      const GhostCellDev *cells, int ncopy, int ninterp, const InterpPlanDev *plan,
                                      const int *face_begin, int *face, int *corner, FusedCopyDev *copies,
                                      FusedInterpDev *interps) {
  const int total = ncopy + ninterp;
  if (total <= 0) return cudaSuccess;
  int grid = (total + 255) / 256;
  if (grid > 152 * 16) grid = 152 * 16;
  k_build_fused_ghosts<<<grid, 256, 0, st>>>(patches, items, cells, ncopy, ninterp, plan, face_begin, face, corner,
                                             copies, interps);
  return cudaGetLastError();
}

}  // namespace pcg
