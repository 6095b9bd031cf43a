// pcg_device.cuh -- device-side data structures and arithmetic of the GB300
// SWE patch-update path.
//
// All FP64 arithmetic below is spelled with explicit round-to-nearest
// intrinsics (__dadd_rn, __dmul_rn, __fma_rn, ...) and the library is built
// with -fmad=false, so the compiler neither contracts nor reorders anything:
// every result is the IEEE result of the written operation sequence.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "pcg_ieee.cuh"

namespace pcg {

// Patch table entry.  `off` is the offset (in doubles) of the patch's data
// vector inside the slab; the vector uses the reference's LinearizationZYXQ
// layout (src/peanoclaw/grid/LinearizationZYXQ.h:20-88).
struct __align__(16) PatchDev {
  long long off;
  int nx, ny, g, nq;
  int np_wo, np_w, level, flags;
  int group, wall, tile_begin, tile_count;
  double pos[2];
  double size[2];
  // offset (in doubles) of the patch's second state copy in the context's
  // shadow buffer (fused batched step: state and net updates, 6 nx ny doubles)
  long long sh_off;
  // first entry of the patch's 2 (nx + ny) face-ghost codes (fused step)
  int face_begin, pad_;
};

struct __align__(16) PatchTimeDev {
  double time, dt, est_next, min_nb_time, max_nb_dt;
  double rl[2], ru[2];
  double pad_;
};

// One sweep/update work item: a tile of at most kTile x kTile cells of a patch.
struct __align__(16) TileItem {
  int pid;
  short x0, y0, tw, th;
  int pad_;
};

// Warp-strip work item of the batched sweep/update: `ngroups` lane groups,
// each a strip of `hs` rows and `w` columns of one patch (the StripGroup
// entries g0 .. g0 + ngroups - 1), with ngroups * hs <= 32 and
// ngroups * w <= 32.
struct __align__(8) StripItem {
  int g0;
  unsigned char ngroups, hs, w, pad_;
};

struct __align__(8) StripGroup {
  int pid;
  short x0, y0;
};

struct SweParamsDev {
  double g, cfl, dry_tol, dry_tol_update, s_min, dt_inf;
};

struct GhostItemDev {
  int kind, src, dst;
  int size[2];
  int src_off[2];
  int dst_off[2];
};

// One ghost cell of the precomputed face-pair list: item and the cell's
// linear index k inside the item's region.
struct GhostCellDev {
  int item, k;
};

// Static part of a coarse-to-fine interpolation of one ghost cell: base
// source cell and the four d-linear weights (DefaultInterpolation.cpph:107-151),
// computed once per grid change.
struct __align__(8) InterpPlanDev {
  int bx, by;
  double sf[4];
};

// Precomputed source/destination offsets of one ghost cell of a COPY item
// (offsets of unknown 0; the other unknowns follow at the item's strides).
struct __align__(16) CopyPlanDev {
  long long src_new, src_old, dst;
  int item, dst_pid;
};

// Per-step data of one ghost item: its time factor (and 1 - tf) and the
// unknown strides of its source (uNew, uOld) and destination (uOld).
struct __align__(16) GhostItemStepDev {
  double tf, itf;
  int vn_src, vo_src, vo_dst, nq;
};

// Face-ghost evaluation plans of the fused batched step (built once per grid
// change from the ghost-cell list): a COPY ghost cell reads source cell
// (sx, sy) of patch src, an INTERP ghost cell the d-linear stencil at base
// cell (bx, by) of patch src with weights sf; `item` indexes the per-step
// item data (time factor).
struct __align__(16) FusedCopyDev {
  int item, src;
  short sx, sy;
  int pad_;
};
struct __align__(16) FusedInterpDev {
  int item, src, bx, by;
  double sf[4];
};

// Bit pattern of a double and back through an opaque register move: the
// compiler cannot see integer tests on these bits as floating-point
// operations (it would otherwise turn sign tests, absolute values and
// maxima into FP64 instructions, which take FP64 pipe slots).
__device__ __forceinline__ unsigned long long obits(double x) {
  unsigned long long u;
  asm("mov.b64 %0, %1;" : "=l"(u) : "d"(x));
  return u;
}
__device__ __forceinline__ double ofrom(unsigned long long u) {
  double x;
  asm("mov.b64 %0, %1;" : "=d"(x) : "l"(u));
  return x;
}

// |x| < 2^1022 (so that x + y of two such values is finite); NaN fails.
__device__ __forceinline__ bool small_mag(double x) {
  return (obits(x) & 0x7FFFFFFFFFFFFFFFull) < 0x7FD0000000000000ull;
}
constexpr int kFinUOld = 1;  // patch finiteness flags (see k_scan_fin)
constexpr int kFinB = 2;

// Loads of patch data; kL2: through L2 only (ld.global.cg), for kernels in
// which other SMs write the data while the kernel runs (an SM's L1 is not
// coherent with those writes).
template <bool kL2>
__device__ __forceinline__ double ldd(const double *p) {
  if constexpr (kL2) return __ldcg(p);
  else return *p;
}
template <bool kL2>
__device__ __forceinline__ int ldi(const int *p) {
  if constexpr (kL2) return __ldcg(p);
  else return *p;
}

// Old-state writes of the strip update.  band: per patch the depths of the
// uOld interior bands the batched ghost fill reads (x lower, x upper, y
// lower, y upper); null: the whole interior.  A step writes only the bands
// unless *full is nonzero or the group reaches its end time with this step
// (t_end - (time + dt) not > 0), so that the reference layout holds after
// the last step of a run and of a group.
struct UpdateBands {
  const int4 *band = nullptr;
  const int *full = nullptr;
  const double *group_time = nullptr, *group_t_end = nullptr;
};

constexpr int kTile = 16;           // tile edge of the sweep
constexpr int kSweepThreads = 256;  // kTile * kTile
constexpr int kFlagLeaf = 1;
constexpr int kFlagVirtual = 2;
// tarch::la comparison tolerance (same constant as the oracle).
constexpr double kTarchEps = 1.0e-8;

__device__ __forceinline__ long long vol_new(const PatchDev &p) { return (long long)p.nx * p.ny; }
__device__ __forceinline__ long long vol_old(const PatchDev &p) {
  return (long long)(p.nx + 2 * p.g) * (p.ny + 2 * p.g);
}
__device__ __forceinline__ long long idx_unew(const PatchDev &p, int q, int x, int y) {
  return p.off + q * vol_new(p) + (long long)x * p.ny + y;
}
__device__ __forceinline__ long long idx_uold(const PatchDev &p, int q, int x, int y) {
  return p.off + p.nq * vol_new(p) + q * vol_old(p) + (long long)(x + p.g) * (p.ny + 2 * p.g) +
         (y + p.g);
}
__device__ __forceinline__ long long idx_pw(const PatchDev &p, int k, int x, int y) {
  return p.off + p.nq * vol_new(p) + p.nq * vol_old(p) + p.np_wo * vol_new(p) + k * vol_old(p) +
         (long long)(x + p.g) * (p.ny + 2 * p.g) + (y + p.g);
}
__device__ __forceinline__ long long idx_flux(const PatchDev &p, int q, int c, int dim, int dir) {
  long long base = p.off + p.nq * vol_new(p) + p.nq * vol_old(p) + p.np_wo * vol_new(p) +
                   p.np_w * vol_old(p);
  long long qs0 = p.ny, qs1 = p.nx;
  long long f1 = qs0 * p.nq, f2 = f1 + qs0 * p.nq, f3 = f2 + qs1 * p.nq;
  int k = 2 * dim + (1 + dir) / 2;
  long long fo = (k == 0) ? 0 : (k == 1) ? f1 : (k == 2) ? f2 : f3;
  return base + fo + c + q * (dim == 0 ? qs0 : qs1);
}

__device__ __forceinline__ bool is_leaf(const PatchDev &p) { return (p.flags & kFlagLeaf) != 0; }
__device__ __forceinline__ bool is_virtual(const PatchDev &p) { return (p.flags & kFlagVirtual) != 0; }

// TimeIntervals::getTimeUOld / getTimeUNew (src/peanoclaw/grid/TimeIntervals.cpp:102-123)
__device__ __forceinline__ double time_uold(const PatchDev &p, const PatchTimeDev &t) {
  return is_leaf(p) ? t.time : t.min_nb_time;
}
__device__ __forceinline__ double time_unew(const PatchDev &p, const PatchTimeDev &t) {
  return is_leaf(p) ? __dadd_rn(t.time, t.dt) : __dadd_rn(t.min_nb_time, t.max_nb_dt);
}
__device__ __forceinline__ bool tl_greater(double a, double b) { return __dsub_rn(a, b) > kTarchEps; }
__device__ __forceinline__ bool tl_equals(double a, double b) {
  return fabs(__dsub_rn(a, b)) <= kTarchEps;
}

// (the divides on the integer pipes: the IEEE quotients, without FP64-pipe
// Newton steps)
__device__ __forceinline__ double subcell(const PatchDev &p, int d) {
  return ieee::div_rn(p.size[d], (double)(d == 0 ? p.nx : p.ny));
}
// Patch::getSubcellCenter: (pos + h*i) + h*0.5
__device__ __forceinline__ double subcell_center(const PatchDev &p, int d, int i) {
  double h = subcell(p, d);
  return __dadd_rn(__dadd_rn(p.pos[d], __dmul_rn(h, (double)i)), __dmul_rn(h, 0.5));
}
// SubgridIterator::getCellPosition: pos + i * (size * (1/n))
__device__ __forceinline__ double iter_sub(const PatchDev &p, int d) {
  return __dmul_rn(p.size[d], ieee::rcp_rn((double)(d == 0 ? p.nx : p.ny)));
}
__device__ __forceinline__ double iter_pos(const PatchDev &p, int d, int i) {
  return __dadd_rn(p.pos[d], __dmul_rn((double)i, iter_sub(p, d)));
}

// Positive doubles order like their bit patterns; used for exact max/min
// reductions with integer atomics.
__device__ __forceinline__ unsigned long long dbits(double v) {
  return obits(v);
}
__device__ __forceinline__ double bitsd(unsigned long long b) {
  return ofrom(b);
}

// IEEE comparisons evaluated on the bit patterns (integer pipes); each one
// returns exactly what the FP64 comparison returns, NaN included.
constexpr unsigned long long kAbsMask = 0x7FFFFFFFFFFFFFFFull;
constexpr unsigned long long kInfBits = 0x7FF0000000000000ull;
// x < 0.0
__device__ __forceinline__ bool lt_zero(double x) {
  long long b = (long long)obits(x);
  unsigned long long m = (unsigned long long)b & kAbsMask;
  return b < 0 && m != 0ull && m <= kInfBits;
}
// a < b, the IEEE comparison (false if either is NaN; -0 == +0)
__device__ __forceinline__ bool lt_ieee(double a, double b) {
  const long long ia = (long long)obits(a), ib = (long long)obits(b);
  const unsigned long long ma = (unsigned long long)ia & kAbsMask, mb = (unsigned long long)ib & kAbsMask;
  if (ma > kInfBits || mb > kInfBits || (ma | mb) == 0ull) return false;
  // sign-magnitude -> order-preserving two's complement keys
  const long long ka = ia < 0 ? -(long long)ma : (long long)ma;
  const long long kb = ib < 0 ? -(long long)mb : (long long)mb;
  return ka < kb;
}
// x > c for a constant c >= +0.0 (not NaN)
__device__ __forceinline__ bool gt_nonneg(double x, double c) {
  long long b = (long long)obits(x);
  return b > (long long)obits(c) && ((unsigned long long)b & kAbsMask) <= kInfBits;
}
// fmax(fabs(a), fabs(b)) with fmax's NaN rule (a NaN operand is ignored)
__device__ __forceinline__ double fmax_abs(double a, double b) {
  unsigned long long ma = obits(a) & kAbsMask;
  unsigned long long mb = obits(b) & kAbsMask;
  unsigned long long r = ma > kInfBits ? mb : (mb > kInfBits ? ma : (ma > mb ? ma : mb));
  return ofrom(r);
}
// fmax(a, b) for a, b >= +0.0 or NaN
__device__ __forceinline__ double fmax_nonneg(double a, double b) {
  unsigned long long ua = obits(a);
  unsigned long long ub = obits(b);
  unsigned long long r = ua > kInfBits ? ub : (ub > kInfBits ? ua : (ua > ub ? ua : ub));
  return ofrom(r);
}

// ---------------------------------------------------------------------------
// f-wave edge solve (same operation sequence as the oracle's fwave_derived).
// Divides and square roots go through pcg_ieee.cuh (integer pipes, results
// identical to the IEEE operations).
// Cell quantities: gh = g/2 h, hu (normal momentum, zero for dry cells), b,
// surface eta = h + b, s = sqrt(h), p = hu / s, F = p*p; wet = h > dry_tol; a
// dry cell has h = max(h, 0).
// ---------------------------------------------------------------------------
struct CellQ {
  double gh, hu, b, eta, s, p, F;
  bool wet;
};

__device__ __forceinline__ void cell_derived(double dry_tol, double halfg, double h, double hu, double hv,
                                             double b, CellQ &cx, CellQ &cy) {
  bool wet = gt_nonneg(h, dry_tol);
  cx.b = b; cx.wet = wet;
  cy.b = b; cy.wet = wet;
  if (wet) {
    double s = ieee::sqrt_rn(h);
    double rs = ieee::rcp_rn(s);
    double p = __dmul_rn(hu, rs);
    double q = __dmul_rn(hv, rs);
    cx.s = s; cx.p = p; cx.F = __dmul_rn(p, p); cx.hu = hu;
    cy.s = s; cy.p = q; cy.F = __dmul_rn(q, q); cy.hu = hv;
  } else {
    // dry: zero velocity, depth clamped to >= 0 (interpolated ghosts can be negative)
    double hd = gt_nonneg(h, 0.0) ? h : 0.0;
    h = hd;
    cx.s = 0.0; cx.p = 0.0; cx.F = 0.0; cx.hu = 0.0;
    cy.s = 0.0; cy.p = 0.0; cy.F = 0.0; cy.hu = 0.0;
  }
  const double eta = __dadd_rn(h, b);
  cx.eta = eta; cy.eta = eta;
  const double gh = __dmul_rn(halfg, h);
  cx.gh = gh; cy.gh = gh;
}

// 2 x, the IEEE product for every x.  A normal x whose double stays finite
// gets its exponent field incremented on the integer pipe; zeros,
// subnormals, overflow, infinities and NaNs go to an out-of-line multiply
// (out of line so that it is not evaluated speculatively beside the fast
// path, where it would take an FP64 slot on every call).
static __device__ __noinline__ double twice_slow(double x) { return __dmul_rn(2.0, x); }
__device__ __forceinline__ double twice(double x) {
  const unsigned long long u = obits(x);
  const unsigned e = (unsigned)(u >> 52) & 0x7FFu;
  if (e - 1u < 0x7FDu) return ofrom(u + (1ull << 52));
  return twice_slow(x);
}

// IEEE negation as a sign-bit flip (a standalone FP64 negation would take an
// FP64 issue slot).
__device__ __forceinline__ double neg(double x) {
  return ofrom(obits(x) ^ 0x8000000000000000ull);
}

// Wet|dry edge: decide whether the dry side is a reflecting wall and, if so,
// replace it by the mirrored wet state.
__device__ __forceinline__ void coastline(CellQ &L, CellQ &R, bool &wallL, bool &wallR) {
  wallR = L.wet && (L.eta <= R.b);
  wallL = R.wet && (R.eta <= L.b);
  if (wallR) { R.gh = L.gh; R.hu = neg(L.hu); R.b = L.b; R.eta = L.eta; R.s = L.s; R.p = neg(L.p); R.F = L.F; }
  if (wallL) { L.gh = R.gh; L.hu = neg(R.hu); L.b = R.b; L.eta = R.eta; L.s = R.s; L.p = neg(R.p); L.F = R.F; }
}

// out: Lh, Lhu, Rh, Rhu (net updates of the left/right cell) and the edge's
// max wave speed.
__device__ __forceinline__ void fwave_edge(CellQ L, CellQ R, double &Lh,
                                           double &Lhu, double &Rh, double &Rhu, double &speed) {
  if (!L.wet && !R.wet) {
    Lh = Lhu = Rh = Rhu = speed = 0.0;
    return;
  }
  bool wallR = false, wallL = false;
  // coastline edges only; the branch is taken per warp (a vote), so warps
  // without a wet|dry edge skip its FP64 additions and nothing is spilled
  const bool coast = L.wet != R.wet;
  if (__any_sync(__activemask(), coast)) {
    if (coast) coastline(L, R, wallL, wallR);
  }
  // a = g/2 (hL + hR), as g/2 hL + g/2 hR from the cells
  double a = __dadd_rn(L.gh, R.gh);
  double cb = ieee::sqrt_rn(a);
  double ub = ieee::div_rn(__dadd_rn(L.p, R.p), __dadd_rn(L.s, R.s));
  double l1 = __dsub_rn(ub, cb);
  double l2 = __dadd_rn(ub, cb);
  double df1 = __dsub_rn(R.hu, L.hu);
  double deta = __dsub_rn(R.eta, L.eta);
  double df2 = __fma_rn(a, deta, __dsub_rn(R.F, L.F));
  // lambda2 - lambda1 = 2 cbar
  double inv = ieee::rcp_rn(twice(cb));
  double b1 = __dmul_rn(__fma_rn(l2, df1, -df2), inv);
  // beta1 + beta2 = df1 (first component of the flux jump)
  double b2 = __dsub_rn(df1, b1);
  double z1 = __dmul_rn(b1, l1);
  double z2 = __dmul_rn(b2, l2);
  // both waves to one side (supersonic edges): the whole flux jump
  // (df1, df2) = beta1 r1 + beta2 r2 goes to that side (selects only)
  const bool left1 = lt_zero(l1), split = left1 && !lt_zero(l2);
  Lh = b1; Lhu = z1; Rh = b2; Rhu = z2;
  if (!split) {
    if (left1) { Lh = df1; Lhu = df2; Rh = 0.0; Rhu = 0.0; }
    else { Lh = 0.0; Lhu = 0.0; Rh = df1; Rhu = df2; }
  }
  if (wallR) { Rh = 0.0; Rhu = 0.0; }
  if (wallL) { Lh = 0.0; Lhu = 0.0; }
  speed = fmax_abs(l1, l2);
}

// CFL timestep of a block whose maximum wave speed is s
// (tools/SWE_WaveAccumulationBlock.cpp:225-239).
__device__ __forceinline__ double cfl_dt(const SweParamsDev &prm, double s, double dx, double dy) {
  if (s > prm.s_min) return __dmul_rn(prm.cfl, fmin(__ddiv_rn(dx, s), __ddiv_rn(dy, s)));
  return prm.dt_inf;
}

}  // namespace pcg
