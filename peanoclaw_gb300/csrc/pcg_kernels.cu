// pcg_kernels.cu -- CUDA kernels (sm_103a) of the SWE patch-update path.
//
// Kernels and the reference code each one replaces:
//   k_sweep_tiles / k_update_tiles  SWE_WaveAccumulationBlock::computeNumericalFluxes
//                                    + updateUnknowns (tools/SWE_WaveAccumulationBlock.cpp:84-296)
//                                    + SWEKernel::advanceBlockInTime swap/time update
//                                    (src/peanoclaw/native/SWEKernel.cpp:50-88)
//   k_solve_patch                    SWEKernel::solveTimestep, fused, one CTA per patch
//   k_ghost_items / k_walls          GhostLayerCompositor face/corner functors ->
//                                    DefaultTransfer / SWE interpolation, SWEKernel::fillBoundaryLayer
//   k_restrict                       DefaultRestriction (+ SWE h+b wrapping)
//   k_compute_fluxes / k_flux_corr   DefaultFluxCorrection
#include "pcg_device.cuh"
#include "pcg_ghost_ops.cuh"
#include "pcg_kernels.h"

#include <cuda.h>

#include <algorithm>
#include <cstdint>

namespace pcg {

// ===========================================================================
// Sweep: one 16x16 (or smaller) tile per CTA iteration.
// ===========================================================================
struct SweepSmem {
  double gh[kTile + 2][kTile + 2];
  double b[kTile + 2][kTile + 2];
  double eta[kTile + 2][kTile + 2];
  double hu[kTile + 2][kTile + 2];
  double hv[kTile + 2][kTile + 2];
  double s[kTile + 2][kTile + 2];
  double p[kTile + 2][kTile + 2];
  double q[kTile + 2][kTile + 2];
  double F[kTile + 2][kTile + 2];
  double G[kTile + 2][kTile + 2];
  unsigned char wet[kTile + 2][kTile + 2];
  double xl_h[kTile][kTile], xl_hu[kTile][kTile];  // left-going parts of x-edges
  double yl_h[kTile][kTile], yl_hv[kTile][kTile];  // down-going parts of y-edges
  double red[kSweepThreads / 32];
  double dxi, dyi;  // 1 / subcell size of the tile's patch
};

__device__ __forceinline__ CellQ load_x(const SweepSmem &S, int i, int j) {
  CellQ c;
  c.gh = S.gh[i][j]; c.b = S.b[i][j]; c.eta = S.eta[i][j]; c.hu = S.hu[i][j]; c.s = S.s[i][j]; c.p = S.p[i][j];
  c.F = S.F[i][j]; c.wet = S.wet[i][j] != 0;
  return c;
}
__device__ __forceinline__ CellQ load_y(const SweepSmem &S, int i, int j) {
  CellQ c;
  c.gh = S.gh[i][j]; c.b = S.b[i][j]; c.eta = S.eta[i][j]; c.hu = S.hv[i][j]; c.s = S.s[i][j]; c.p = S.q[i][j];
  c.F = S.G[i][j]; c.wet = S.wet[i][j] != 0;
  return c;
}

// Computes the net updates of one tile.  The state is read from `interior`
// (uNew in the batched form, uOld in the fused solveTimestep form) for cells
// inside the patch and from uOld for the ghost ring.  Returns, in the calling
// thread, the accumulated net updates of its cell (valid iff t < tw*th) and
// the tile's max wave speed (valid in every thread).
// One staged cell of a tile: its derived quantities into the tile's arrays.
__device__ __forceinline__ void stage_cell(SweepSmem &S, int sx, int sy, double dry, double halfg, double h,
                                           double hu, double hv, double b) {
  CellQ qx, qy;
  cell_derived(dry, halfg, h, hu, hv, b, qx, qy);
  S.gh[sx][sy] = qx.gh; S.b[sx][sy] = b; S.eta[sx][sy] = qx.eta; S.hu[sx][sy] = qx.hu; S.hv[sx][sy] = qy.hu;
  S.s[sx][sy] = qx.s; S.p[sx][sy] = qx.p; S.q[sx][sy] = qy.p;
  S.F[sx][sy] = qx.F; S.G[sx][sy] = qy.F; S.wet[sx][sy] = qx.wet ? 1 : 0;
}

__device__ __forceinline__ double sweep_tile_staged(SweepSmem &S, int tw, int th, double &nh, double &nhu,
                                                    double &nhv);

__device__ __forceinline__ double sweep_tile(SweepSmem &S, const double *__restrict__ slab,
                                             const PatchDev &P, const SweParamsDev &prm,
                                             int x0, int y0, int tw, int th, bool interior_is_unew,
                                             double &nh, double &nhu, double &nhv) {
  const int t = threadIdx.x;
  const double dry = prm.dry_tol;
  const double halfg = __dmul_rn(0.5, prm.g);
  if (t == 0) {
    S.dxi = __ddiv_rn(1.0, subcell(P, 0));
    S.dyi = __ddiv_rn(1.0, subcell(P, 1));
  }
  // ---- stage tile + halo (corners skipped: the 5-point sweep never reads them)
  const int sw = tw + 2, sh = th + 2;
  for (int k = t; k < sw * sh; k += blockDim.x) {
    int sx = k / sh, sy = k - sx * sh;
    bool cx = (sx == 0 || sx == sw - 1), cy = (sy == 0 || sy == sh - 1);
    if (cx && cy) continue;
    int x = x0 - 1 + sx, y = y0 - 1 + sy;
    bool inside = (x >= 0 && x < P.nx && y >= 0 && y < P.ny);
    double h, hu, hv;
    if (inside && interior_is_unew) {
      h = slab[idx_unew(P, 0, x, y)];
      hu = slab[idx_unew(P, 1, x, y)];
      hv = slab[idx_unew(P, 2, x, y)];
    } else {
      h = slab[idx_uold(P, 0, x, y)];
      hu = slab[idx_uold(P, 1, x, y)];
      hv = slab[idx_uold(P, 2, x, y)];
    }
    stage_cell(S, sx, sy, dry, halfg, h, hu, hv, slab[idx_pw(P, 0, x, y)]);
  }
  __syncthreads();
  return sweep_tile_staged(S, tw, th, nh, nhu, nhv);
}

// The edges, the accumulation and the max wave speed of a staged tile.
__device__ __forceinline__ double sweep_tile_staged(SweepSmem &S, int tw, int th, double &nh, double &nhu,
                                                    double &nhv) {
  const int t = threadIdx.x;
  double smax = 0.0;
  double xr_h = 0.0, xr_hu = 0.0, yr_h = 0.0, yr_hv = 0.0;
  const bool active = t < tw * th;
  const int lx = active ? t / th : 0, ly = active ? t - (t / th) * th : 0;
  if (active) {
    double Lh, Lhu, Rh, Rhu, sp;
    // x-edge between (lx-1, ly) and (lx, ly)
    fwave_edge(load_x(S, lx, ly + 1), load_x(S, lx + 1, ly + 1), Lh, Lhu, Rh, Rhu, sp);
    smax = fmax_nonneg(smax, sp);
    xr_h = Rh; xr_hu = Rhu;
    if (lx >= 1) { S.xl_h[lx - 1][ly] = Lh; S.xl_hu[lx - 1][ly] = Lhu; }
    // y-edge between (lx, ly-1) and (lx, ly)
    fwave_edge(load_y(S, lx + 1, ly), load_y(S, lx + 1, ly + 1), Lh, Lhu, Rh, Rhu, sp);
    smax = fmax_nonneg(smax, sp);
    yr_h = Rh; yr_hv = Rhu;
    if (ly >= 1) { S.yl_h[lx][ly - 1] = Lh; S.yl_hv[lx][ly - 1] = Lhu; }
  }
  // closing edges on the upper x and y side of the tile, done by the last
  // threads (the first ones stage the second round of halo cells)
  const int ce = t - ((int)blockDim.x - (th + tw));
  if (ce >= 0) {
    double Lh, Lhu, Rh, Rhu, sp;
    if (ce < th) {
      int j = ce;
      fwave_edge(load_x(S, tw, j + 1), load_x(S, tw + 1, j + 1), Lh, Lhu, Rh, Rhu, sp);
      S.xl_h[tw - 1][j] = Lh; S.xl_hu[tw - 1][j] = Lhu;
    } else {
      int i = ce - th;
      fwave_edge(load_y(S, i + 1, th), load_y(S, i + 1, th + 1), Lh, Lhu, Rh, Rhu, sp);
      S.yl_h[i][th - 1] = Lh; S.yl_hv[i][th - 1] = Lhu;
    }
    smax = fmax_nonneg(smax, sp);
  }
  __syncthreads();
  if (active) {
    const double dxi = S.dxi, dyi = S.dyi;
    // accumulation order of computeNumericalFluxes: x-edges (own left edge,
    // then right edge), then y-edges (own lower edge, then upper edge)
    double a = __fma_rn(dxi, xr_h, 0.0);
    a = __fma_rn(dxi, S.xl_h[lx][ly], a);
    a = __fma_rn(dyi, yr_h, a);
    nh = __fma_rn(dyi, S.yl_h[lx][ly], a);
    double u = __fma_rn(dxi, xr_hu, 0.0);
    nhu = __fma_rn(dxi, S.xl_hu[lx][ly], u);
    double v = __fma_rn(dyi, yr_hv, 0.0);
    nhv = __fma_rn(dyi, S.yl_hv[lx][ly], v);
  }
  // ---- tile max wave speed (speeds are >= 0: bit patterns order like values)
  unsigned long long m = dbits(smax);
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long other = __shfl_xor_sync(0xffffffffu, m, o);
    m = other > m ? other : m;
  }
  if ((t & 31) == 0) S.red[t >> 5] = bitsd(m);
  __syncthreads();
  unsigned long long r = 0;
  for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
    unsigned long long v = dbits(S.red[w]);
    r = v > r ? v : r;
  }
  __syncthreads();  // S is reused by the next tile
  return bitsd(r);
}

// Batched sweep: tiles [first, first + count) of the work list, grid-strided.
// Net updates go to the uOld interior (free between the ghost fill and the
// update), the tile's max speed to the patch and its CFL dt to the group.
__global__ void __launch_bounds__(kSweepThreads, 4)
    k_sweep_tiles(double *__restrict__ slab, const PatchDev *__restrict__ patches,
                  const TileItem *__restrict__ tiles, int first, int count, SweParamsDev prm,
                  unsigned long long *__restrict__ patch_smax,
                  unsigned long long *__restrict__ group_dt, const int *__restrict__ group_active, int *__restrict__ fin,
                  const int *__restrict__ pact) {
  __shared__ SweepSmem S;
  for (int it = blockIdx.x; it < count; it += gridDim.x) {
    TileItem ti = tiles[first + it];
    PatchDev P = patches[ti.pid];
    if (group_active && !group_active[P.group]) continue;
    if (pact && !pact[ti.pid]) continue;
    double nh = 0, nhu = 0, nhv = 0;
    double smax = sweep_tile(S, slab, P, prm, ti.x0, ti.y0, ti.tw, ti.th, true, nh, nhu, nhv);
    int t = threadIdx.x;
    if (t < ti.tw * ti.th) {
      int x = ti.x0 + t / ti.th, y = ti.y0 + t % ti.th;
      slab[idx_uold(P, 0, x, y)] = nh;
      slab[idx_uold(P, 1, x, y)] = nhu;
      slab[idx_uold(P, 2, x, y)] = nhv;
    }
    if (t == 0) {
      if (fin) atomicOr(&fin[ti.pid], kFinUOld);
      atomicMax(&patch_smax[ti.pid], dbits(smax));
      double dtc = cfl_dt(prm, smax, subcell(P, 0), subcell(P, 1));
      atomicMin(&group_dt[P.group], dbits(dtc));
    }
  }
}

// ---------------------------------------------------------------------------
// TMA-staged tile sweep (schedule: tiles, variant 1).  The same tiles and
// arithmetic as k_sweep_tiles; the tile + halo is brought into shared memory
// by three tensor copies (cp.async.bulk.tensor) per tile instead of per-thread
// loads: the uNew box (interior cells), the uOld box (ghost ring) and the
// bathymetry box, completing on one mbarrier.  Tensor maps per patch
// (TileMaps, encoded on the host by encode_tile_maps): uNew as (ny, nx, 3),
// uOld as (ny+2, nx+2, 3), b as (ny+2, nx+2), y innermost.  The innermost
// start coordinate must be a multiple of 2 doubles (16 bytes): the uNew box
// starts at y0 - 2 (tiles start at multiples of 16), the ghosted boxes at y0
// (which is y0 - 1 in interior coordinates); boxes are min(16, n) + 4 resp.
// + 2 doubles wide in y (even for even n), so only patches of even size take
// this form.  Boxes reaching past the patch read zeros (out-of-bounds fill)
// and those cells are taken from the uOld box.
// ---------------------------------------------------------------------------
struct __align__(128) TmaRaw {
  __align__(128) double un[3 * (kTile + 2) * (kTile + 4)];
  __align__(128) double uo[3 * (kTile + 2) * (kTile + 2)];
  __align__(128) double bb[(kTile + 2) * (kTile + 2)];
};
constexpr int kTmaSpin = 1 << 22;

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t *m, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(m)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *m, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(m)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *m, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(m)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, uint64_t *m, int c0, int c1,
                                            int c2) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(smem_u32(dst)),
      "l"((uint64_t)map), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(m))
      : "memory");
}
__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, uint64_t *m, int c0, int c1) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          smem_u32(dst)),
      "l"((uint64_t)map), "r"(c0), "r"(c1), "r"(smem_u32(m))
      : "memory");
}

// All threads: wait for the tile's copies (bounded); false if they did not
// complete (the kernel then sets *err and stops).
__device__ __forceinline__ bool tma_wait(uint64_t *m, unsigned parity) {
  bool ok = false;
  for (int i = 0; i < kTmaSpin && !ok; i++) ok = mbar_try_wait(m, parity);
  return !__syncthreads_or(!ok);
}

// Issues the three copies of tile `ti` into R (by one thread).
__device__ __forceinline__ void tma_issue_tile(TmaRaw &R, uint64_t *mbar, const TileMaps *maps, const TileItem &ti,
                                               const PatchDev &P) {
  const int bx = (P.nx < kTile ? P.nx : kTile) + 2;
  const int byo = (P.ny < kTile ? P.ny : kTile) + 2, byn = byo + 2;
  const TileMaps *M = &maps[ti.pid];
  // earlier reads of R (generic proxy) are ordered before the copies (async
  // proxy) by the barrier that ended them and this fence
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  mbar_expect_tx(mbar, (unsigned)(8 * (3 * bx * byn + 3 * bx * byo + bx * byo)));
  tma_load_3d(R.un, &M->unew, mbar, ti.y0 - 2, ti.x0 - 1, 0);
  tma_load_3d(R.uo, &M->uold, mbar, ti.y0, ti.x0, 0);
  tma_load_2d(R.bb, &M->b, mbar, ti.y0, ti.x0);
}

// One raw buffer per CTA: a double-buffered form (the next tile's copies in
// flight during the current sweep) measured slower, 17.8 against 14.7 ms per
// step on the 50k mix, its 80 registers and 72 KB of shared memory leaving 3
// CTAs per SM instead of 4 for this FP64-latency-bound sweep.
__global__ void __launch_bounds__(kSweepThreads, 4)
    k_sweep_tiles_tma(double *__restrict__ slab, const PatchDev *__restrict__ patches,
                      const TileMaps *__restrict__ maps, const TileItem *__restrict__ tiles, int first, int count,
                      SweParamsDev prm, unsigned long long *__restrict__ patch_smax,
                      unsigned long long *__restrict__ group_dt, const int *__restrict__ group_active,
                      int *__restrict__ fin, const int *__restrict__ pact, int *__restrict__ err) {
  __shared__ SweepSmem S;
  __shared__ __align__(8) uint64_t mbar;
  extern __shared__ __align__(128) unsigned char tma_smem[];
  TmaRaw &R = *reinterpret_cast<TmaRaw *>(tma_smem);
  if (threadIdx.x == 0) mbar_init(&mbar, 1);
  __syncthreads();
  unsigned parity = 0;
  const double dry = prm.dry_tol;
  const double halfg = __dmul_rn(0.5, prm.g);
  for (int it = blockIdx.x; it < count; it += gridDim.x) {
    const TileItem ti = tiles[first + it];
    const PatchDev P = patches[ti.pid];
    if (group_active && !group_active[P.group]) continue;
    if (pact && !pact[ti.pid]) continue;
    const int bx = (P.nx < kTile ? P.nx : kTile) + 2;
    const int byo = (P.ny < kTile ? P.ny : kTile) + 2, byn = byo + 2;
    if (threadIdx.x == 0) {
      S.dxi = __ddiv_rn(1.0, subcell(P, 0));
      S.dyi = __ddiv_rn(1.0, subcell(P, 1));
      tma_issue_tile(R, &mbar, maps, ti, P);
    }
    if (!tma_wait(&mbar, parity)) {
      // the copies did not complete: wait once more (bounded) so that none is
      // left writing shared memory, report, and stop
      tma_wait(&mbar, parity);
      if (threadIdx.x == 0) atomicExch(err, 2);
      return;
    }
    parity ^= 1u;
    const int tw = ti.tw, th = ti.th, sw = tw + 2, sh = th + 2;
    for (int k = threadIdx.x; k < sw * sh; k += blockDim.x) {
      const int sx = k / sh, sy = k - sx * sh;
      const bool cx = (sx == 0 || sx == sw - 1), cy = (sy == 0 || sy == sh - 1);
      if (cx && cy) continue;
      const int x = ti.x0 - 1 + sx, y = ti.y0 - 1 + sy;
      const bool inside = (x >= 0 && x < P.nx && y >= 0 && y < P.ny);
      double h, hu, hv;
      if (inside) {
        h = R.un[(0 * bx + sx) * byn + sy + 1];
        hu = R.un[(1 * bx + sx) * byn + sy + 1];
        hv = R.un[(2 * bx + sx) * byn + sy + 1];
      } else {
        h = R.uo[(0 * bx + sx) * byo + sy];
        hu = R.uo[(1 * bx + sx) * byo + sy];
        hv = R.uo[(2 * bx + sx) * byo + sy];
      }
      stage_cell(S, sx, sy, dry, halfg, h, hu, hv, R.bb[sx * byo + sy]);
    }
    __syncthreads();
    double nh = 0, nhu = 0, nhv = 0;
    const double smax = sweep_tile_staged(S, tw, th, nh, nhu, nhv);
    const int t = threadIdx.x;
    if (t < tw * th) {
      const int x = ti.x0 + t / th, y = ti.y0 + t % th;
      slab[idx_uold(P, 0, x, y)] = nh;
      slab[idx_uold(P, 1, x, y)] = nhu;
      slab[idx_uold(P, 2, x, y)] = nhv;
    }
    if (t == 0) {
      if (fin) atomicOr(&fin[ti.pid], kFinUOld);
      atomicMax(&patch_smax[ti.pid], dbits(smax));
      const double dtc = cfl_dt(prm, smax, subcell(P, 0), subcell(P, 1));
      atomicMin(&group_dt[P.group], dbits(dtc));
    }
  }
}

// Batched update: q_new = q - dt * net (tools/SWE_WaveAccumulationBlock.cpp:247-296)
// with the dry clamps, then the swap (uOld interior <- old state, uNew <- new)
// and, once per patch, the time-interval update of advanceBlockInTime.
__global__ void __launch_bounds__(kSweepThreads)
    k_update_tiles(double *__restrict__ slab, const PatchDev *__restrict__ patches,
                   PatchTimeDev *__restrict__ times, const TileItem *__restrict__ tiles, int first,
                   int count, SweParamsDev prm, const unsigned long long *__restrict__ patch_smax,
                   const unsigned long long *__restrict__ group_dt,
                   const int *__restrict__ group_active, int *__restrict__ fin,
                   const int *__restrict__ pact,
                   const unsigned long long *__restrict__ pdt) {
  for (int it = blockIdx.x; it < count; it += gridDim.x) {
    TileItem ti = tiles[first + it];
    PatchDev P = patches[ti.pid];
    if (group_active && !group_active[P.group]) continue;
    if (pact && !pact[ti.pid]) continue;
    double dt = bitsd(pdt ? pdt[ti.pid] : group_dt[P.group]);
    int t = threadIdx.x;
    if (t < ti.tw * ti.th) {
      int x = ti.x0 + t / ti.th, y = ti.y0 + t % ti.th;
      long long io0 = idx_uold(P, 0, x, y), io1 = idx_uold(P, 1, x, y), io2 = idx_uold(P, 2, x, y);
      long long in0 = idx_unew(P, 0, x, y), in1 = idx_unew(P, 1, x, y), in2 = idx_unew(P, 2, x, y);
      double h = slab[in0], hu = slab[in1], hv = slab[in2];
      double nh = __fma_rn(-dt, slab[io0], h);
      double nhu = __fma_rn(-dt, slab[io1], hu);
      double nhv = __fma_rn(-dt, slab[io2], hv);
      if (lt_ieee(nh, prm.dry_tol_update)) { nhu = 0.0; nhv = 0.0; }
      if (lt_zero(nh)) nh = 0.0;
      slab[io0] = h; slab[io1] = hu; slab[io2] = hv;
      slab[in0] = nh; slab[in1] = nhu; slab[in2] = nhv;
      if (fin && !(small_mag(h) && small_mag(hu) && small_mag(hv))) atomicAnd(&fin[ti.pid], ~kFinUOld);
    }
    if (t == 0 && ti.x0 == 0 && ti.y0 == 0) {
      PatchTimeDev &T = times[ti.pid];
      if (tl_greater(dt, 0.0)) {
        T.time = __dadd_rn(T.time, T.dt);
        T.dt = dt;
      }
      T.est_next = cfl_dt(prm, bitsd(patch_smax[ti.pid]), subcell(P, 0), subcell(P, 1));
    }
  }
}

// Start of a step: group dt <- min(max_dt, max(0, t_end - t)) (t_end = +inf
// unless the group has an end time), group active iff t_end - t > 0, patch
// max speed <- 0.
__global__ void k_reset_step(int n_groups, const double *__restrict__ group_max_dt,
                             const double *__restrict__ group_t_end,
                             const double *__restrict__ group_time,
                             unsigned long long *__restrict__ group_dt, int *__restrict__ group_active,
                             int n_patches, unsigned long long *__restrict__ patch_smax) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n_groups) {
    const double rem = __dsub_rn(group_t_end[i], group_time[i]);
    const bool active = gt_nonneg(rem, 0.0);
    const double cap = active ? rem : 0.0;
    const double mx = group_max_dt[i];
    group_dt[i] = dbits(lt_ieee(cap, mx) ? cap : mx);
    group_active[i] = active ? 1 : 0;
  }
  for (int k = i; k < n_patches; k += gridDim.x * blockDim.x) patch_smax[k] = 0ull;
}

// End of a step: t += dt for the active groups.
__global__ void k_group_advance(int n_groups, const unsigned long long *__restrict__ group_dt,
                                const int *__restrict__ group_active, double *__restrict__ group_time) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n_groups && group_active[i]) group_time[i] = __dadd_rn(group_time[i], bitsd(group_dt[i]));
}

// ---------------------------------------------------------------------------
// Local time stepping (one grid iteration in two phases; see pcg.h):
// order-preserving keys of doubles for integer atomicMin over any sign.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long okey(double x) {
  const unsigned long long b = dbits(x);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double unokey(unsigned long long k) {
  return (k >> 63) ? bitsd(k & 0x7FFFFFFFFFFFFFFFull) : bitsd(~k);
}

__global__ void k_lts_begin(int n_patches, unsigned long long *__restrict__ nbmin,
                            unsigned long long *__restrict__ patch_smax, int n_groups,
                            unsigned long long *__restrict__ group_tmin,
                            unsigned long long *__restrict__ group_dt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  for (int k = i; k < n_patches; k += gridDim.x * blockDim.x) {
    nbmin[k] = okey(INFINITY);
    patch_smax[k] = 0ull;
  }
  if (i < n_groups) {
    group_tmin[i] = okey(INFINITY);
    group_dt[i] = dbits(INFINITY);
  }
}

// Time intervals of the virtual patches: the intersection of the intervals
// of their listed leaves (time = maximal leaf time, dt = minimal leaf
// time + dt minus that time; GridLevelTransfer::stepUp with
// updateMinimalFineGridTimeInterval and
// switchValuesAndTimeIntervalToMinimalFineGridTimeInterval).
__global__ void k_lts_vt_reset(const int *__restrict__ vdsts, int nv, unsigned long long *__restrict__ vstart,
                               unsigned long long *__restrict__ vend) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nv; k += gridDim.x * blockDim.x) {
    vstart[vdsts[k]] = okey(-INFINITY);
    vend[vdsts[k]] = okey(INFINITY);
  }
}
__global__ void k_lts_vt_pairs(const int2 *__restrict__ pairs, int n, const PatchTimeDev *__restrict__ times,
                               unsigned long long *__restrict__ vstart, unsigned long long *__restrict__ vend) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const int2 pr = pairs[k];
    const PatchTimeDev T = times[pr.x];
    atomicMax(&vstart[pr.y], okey(T.time));
    atomicMin(&vend[pr.y], okey(__dadd_rn(T.time, T.dt)));
  }
}
__global__ void k_lts_vt_set(const int *__restrict__ vdsts, int nv, const unsigned long long *__restrict__ vstart,
                             const unsigned long long *__restrict__ vend, PatchTimeDev *__restrict__ times) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nv; k += gridDim.x * blockDim.x) {
    const int v = vdsts[k];
    const double t = unokey(vstart[v]);
    times[v].time = t;
    times[v].dt = __dsub_rn(unokey(vend[v]), t);
  }
}

// Minimal time constraint (time + dt, TimeIntervals::getTimeConstraint) of
// the ghost-item sources of every destination.
__global__ void k_lts_nbmin(const GhostItemDev *__restrict__ items, int count,
                            const PatchTimeDev *__restrict__ times, unsigned long long *__restrict__ nbmin) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) {
    const GhostItemDev it = items[k];
    const PatchTimeDev T = times[it.src];
    atomicMin(&nbmin[it.dst], okey(__dadd_rn(T.time, T.dt)));
  }
}

// Which leaves advance: the end time is not reached (max_dt = min(group
// max_dt, end time - uNew time) > tarch eps) and uNew time does not exceed
// the neighbours' minimal uNew time by more than eps
// (TimeIntervals::isAllowedToAdvanceInTime / isBlockedByNeighbors).
__global__ void k_lts_activity(const PatchDev *__restrict__ patches, const PatchTimeDev *__restrict__ times,
                               int n_patches, const unsigned long long *__restrict__ nbmin,
                               const double *__restrict__ group_max_dt, const double *__restrict__ group_t_end,
                               const int *__restrict__ group_active, int *__restrict__ pact,
                               double *__restrict__ pmaxdt) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n_patches; p += gridDim.x * blockDim.x) {
    const PatchDev P = patches[p];
    if (P.nx <= 0 || !is_leaf(P)) {
      pact[p] = 0;
      continue;
    }
    const double tu = time_unew(P, times[p]);
    const double rem = __dsub_rn(group_t_end[P.group], tu);
    const double mx = group_max_dt[P.group];
    const double maxdt = rem < mx ? rem : mx;
    pact[p] = group_active[P.group] && tl_greater(maxdt, 0.0) && !tl_greater(tu, unokey(nbmin[p]));
    pmaxdt[p] = maxdt;
  }
}

// dt of every advancing leaf (min of its block CFL dt and its max_dt), the
// group's minimal dt taken and minimal uNew time after the step; the cells
// of the leaves that advance are added to *cells.
__global__ void k_lts_dt(const PatchDev *__restrict__ patches, const PatchTimeDev *__restrict__ times,
                         int n_patches, const int *__restrict__ pact, const double *__restrict__ pmaxdt,
                         const unsigned long long *__restrict__ patch_smax, SweParamsDev prm,
                         unsigned long long *__restrict__ pdt, unsigned long long *__restrict__ group_dt,
                         unsigned long long *__restrict__ group_tmin, unsigned long long *__restrict__ cells) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n_patches; p += gridDim.x * blockDim.x) {
    const PatchDev P = patches[p];
    if (P.nx <= 0 || !is_leaf(P)) continue;
    const PatchTimeDev T = times[p];
    double tnext = time_unew(P, T);
    if (pact[p]) {
      const double own = cfl_dt(prm, bitsd(patch_smax[p]), subcell(P, 0), subcell(P, 1));
      const double dt = fmin(own, pmaxdt[p]);
      pdt[p] = dbits(dt);
      atomicMin(&group_dt[P.group], dbits(dt));
      if (tl_greater(dt, 0.0)) {
        tnext = __dadd_rn(__dadd_rn(T.time, T.dt), dt);
        if (cells) atomicAdd(cells, (unsigned long long)P.nx * (unsigned long long)P.ny);
      }
    }
    atomicMin(&group_tmin[P.group], okey(tnext));
  }
}

// End of an iteration: group time = minimal uNew time of its leaves; the
// recorded dt of a group without an advancing leaf is 0.
__global__ void k_lts_end(int n_groups, const unsigned long long *__restrict__ group_tmin,
                          double *__restrict__ group_time, unsigned long long *__restrict__ group_dt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_groups) return;
  const double t = unokey(group_tmin[i]);
  if (t != INFINITY) group_time[i] = t;
  if (bitsd(group_dt[i]) == INFINITY) group_dt[i] = dbits(0.0);
}

// Record the dt of every group after a step.
__global__ void k_record_dt(int n_groups, const unsigned long long *__restrict__ group_dt,
                            double *__restrict__ out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n_groups) out[i] = bitsd(group_dt[i]);
}

// ===========================================================================
// Fused per-patch solve (SWEKernel::solveTimestep), one CTA per patch.
// Input state: uOld (+ghost).  Net updates live in dynamic shared memory.
// ===========================================================================
__global__ void __launch_bounds__(kSweepThreads)
    k_solve_patch(double *__restrict__ slab, const PatchDev *__restrict__ patches,
                  PatchTimeDev *__restrict__ times, int pid, SweParamsDev prm, double max_dt,
                  double *__restrict__ out) {
  __shared__ SweepSmem S;
  extern __shared__ double net[];  // 3 * nx * ny
  const PatchDev P = patches[pid];
  const int nx = P.nx, ny = P.ny;
  double smax = 0.0;
  for (int x0 = 0; x0 < nx; x0 += kTile)
    for (int y0 = 0; y0 < ny; y0 += kTile) {
      int tw = min(kTile, nx - x0), th = min(kTile, ny - y0);
      double nh = 0, nhu = 0, nhv = 0;
      double s = sweep_tile(S, slab, P, prm, x0, y0, tw, th, false, nh, nhu, nhv);
      smax = fmax(smax, s);
      int t = threadIdx.x;
      if (t < tw * th) {
        int x = x0 + t / th, y = y0 + t % th;
        long long c = (long long)x * ny + y;
        net[c] = nh;
        net[(long long)nx * ny + c] = nhu;
        net[2LL * nx * ny + c] = nhv;
      }
    }
  __syncthreads();
  double dx = subcell(P, 0), dy = subcell(P, 1);
  double block_dt = cfl_dt(prm, smax, dx, dy);
  double dt = fmin(block_dt, max_dt);
  for (int c = threadIdx.x; c < nx * ny; c += blockDim.x) {
    int x = c / ny, y = c - x * ny;
    long long io0 = idx_uold(P, 0, x, y), io1 = idx_uold(P, 1, x, y), io2 = idx_uold(P, 2, x, y);
    long long in0 = idx_unew(P, 0, x, y), in1 = idx_unew(P, 1, x, y), in2 = idx_unew(P, 2, x, y);
    double nh = __fma_rn(-dt, net[c], slab[io0]);
    double nhu = __fma_rn(-dt, net[(long long)nx * ny + c], slab[io1]);
    double nhv = __fma_rn(-dt, net[2LL * nx * ny + c], slab[io2]);
    if (lt_ieee(nh, prm.dry_tol_update)) { nhu = 0.0; nhv = 0.0; }
    if (lt_zero(nh)) nh = 0.0;
    // swapUNewAndUOld: uOld <- previous uNew, uNew <- updated values
    double o0 = slab[in0], o1 = slab[in1], o2 = slab[in2];
    slab[io0] = o0; slab[io1] = o1; slab[io2] = o2;
    slab[in0] = nh; slab[in1] = nhu; slab[in2] = nhv;
  }
  if (threadIdx.x == 0) {
    PatchTimeDev &T = times[pid];
    if (tl_greater(dt, 0.0)) {
      T.time = __dadd_rn(T.time, T.dt);
      T.dt = dt;
    }
    T.est_next = block_dt;
    out[0] = dt;
    out[1] = block_dt;
  }
}

// ===========================================================================
// Ghost layers
// ===========================================================================

// DefaultTransferTemplate::transferGhostlayer body for cell k of the region.
__device__ __forceinline__ void transfer_cell(double *slab, const PatchDev &S, const PatchDev &D,
                                              const int size[2], const int so[2], const int dof[2],
                                              double tf, double itf, int k) {
  int x = k / size[1], y = k - x * size[1];
  for (int q = 0; q < S.nq; q++) {
    double vn = slab[idx_unew(S, q, so[0] + x, so[1] + y)];
    double vo = slab[idx_uold(S, q, so[0] + x, so[1] + y)];
    slab[idx_uold(D, q, dof[0] + x, dof[1] + y)] = __dadd_rn(__dmul_rn(vn, tf), __dmul_rn(vo, itf));
  }
}

// DefaultInterpolationTemplate::interpolateSolution body for destination cell
// k of the region (clear uOld, d-linear stencil with time factor, SWE h+b wrap).
__device__ void interp_cell(double *slab, const PatchDev &S, const PatchDev &D, const int size[2],
                            const int dof[2], double tf, bool to_uold, bool swe, int k) {
  double one_m_tf = __dsub_rn(1.0, tf);
  int cx = dof[0] + k / size[1], cy = dof[1] + k % size[1];
  for (int q = 0; q < D.nq; q++) slab[idx_uold(D, q, cx, cy)] = 0.0;
  double sh[2] = {subcell(S, 0), subcell(S, 1)};
  double inv[2] = {__ddiv_rn(1.0, sh[0]), __ddiv_rn(1.0, sh[1])};
  double c[2] = {subcell_center(D, 0, cx), subcell_center(D, 1, cy)};
  int bi[2];
  int n[2] = {S.nx, S.ny};
  for (int d = 0; d < 2; d++) {
    double sbase = __dadd_rn(S.pos[d], __dmul_rn(sh[d], 0.5));
    double local = __dsub_rn(c[d], sbase);
    int v = (int)floor(__dmul_rn(local, inv[d]));
    v = v < n[d] - 2 ? v : n[d] - 2;
    bi[d] = v > 0 ? v : 0;
  }
  for (int kk = 0; kk < 4; kk++) {
    int off[2] = {kk & 1, (kk >> 1) & 1};
    int nxi = bi[0] + off[0], nyi = bi[1] + off[1];
    double npos[2] = {subcell_center(S, 0, nxi), subcell_center(S, 1, nyi)};
    double sf = 1.0;
    for (int d = 0; d < 2; d++) {
      double sign = (double)(1 - 2 * off[d]);
      sf = __dmul_rn(sf, __dsub_rn(1.0, __dmul_rn(__dmul_rn(sign, __dsub_rn(c[d], npos[d])), inv[d])));
    }
    for (int q = 0; q < D.nq; q++) {
      double so = slab[idx_uold(S, q, nxi, nyi)];
      double sn = slab[idx_unew(S, q, nxi, nyi)];
      if (swe && q == 0) {
        double bb = slab[idx_pw(S, 0, nxi, nyi)];
        so = __dadd_rn(so, bb);
        sn = __dadd_rn(sn, bb);
      }
      if (to_uold) {
        long long id = idx_uold(D, q, cx, cy);
        slab[id] = __dadd_rn(slab[id], __dmul_rn(sf, __dadd_rn(__dmul_rn(so, one_m_tf), __dmul_rn(sn, tf))));
      } else {
        long long id = idx_unew(D, q, cx, cy);
        slab[id] = __dadd_rn(__dadd_rn(slab[id], __dmul_rn(__dmul_rn(sf, so), one_m_tf)),
                             __dmul_rn(__dmul_rn(sf, sn), tf));
      }
    }
  }
  if (swe) {
    double bb = slab[idx_pw(D, 0, cx, cy)];
    long long id = to_uold ? idx_uold(D, 0, cx, cy) : idx_unew(D, 0, cx, cy);
    slab[id] = __dadd_rn(slab[id], __dmul_rn(-1.0, bb));
  }
}

// Static interpolation geometry of ghost cell k of an INTERP item: the same
// operations as interp_cell, evaluated once per grid change.
__device__ void interp_plan_cell(const PatchDev &S, const PatchDev &D, const int size[2],
                                 const int dof[2], int k, InterpPlanDev &pl) {
  int cx = dof[0] + k / size[1], cy = dof[1] + k % size[1];
  double sh[2] = {subcell(S, 0), subcell(S, 1)};
  double inv[2] = {__ddiv_rn(1.0, sh[0]), __ddiv_rn(1.0, sh[1])};
  double c[2] = {subcell_center(D, 0, cx), subcell_center(D, 1, cy)};
  int bi[2];
  int n[2] = {S.nx, S.ny};
  for (int d = 0; d < 2; d++) {
    double sbase = __dadd_rn(S.pos[d], __dmul_rn(sh[d], 0.5));
    double local = __dsub_rn(c[d], sbase);
    int v = (int)floor(__dmul_rn(local, inv[d]));
    v = v < n[d] - 2 ? v : n[d] - 2;
    bi[d] = v > 0 ? v : 0;
  }
  pl.bx = bi[0];
  pl.by = bi[1];
  for (int kk = 0; kk < 4; kk++) {
    int off[2] = {kk & 1, (kk >> 1) & 1};
    double npos[2] = {subcell_center(S, 0, bi[0] + off[0]), subcell_center(S, 1, bi[1] + off[1])};
    double sf = 1.0;
    for (int d = 0; d < 2; d++) {
      double sign = (double)(1 - 2 * off[d]);
      sf = __dmul_rn(sf, __dsub_rn(1.0, __dmul_rn(__dmul_rn(sign, __dsub_rn(c[d], npos[d])), inv[d])));
    }
    pl.sf[kk] = sf;
  }
}

__global__ void k_build_interp_plan(const PatchDev *__restrict__ patches,
                                    const GhostItemDev *__restrict__ items,
                                    const GhostCellDev *__restrict__ cells, int count,
                                    InterpPlanDev *__restrict__ plan) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < count; e += gridDim.x * blockDim.x) {
    GhostCellDev gc = cells[e];
    GhostItemDev it = items[gc.item];
    interp_plan_cell(patches[it.src], patches[it.dst], it.size, it.dst_off, gc.k, plan[e]);
  }
}

// uOld interior bands the batched ghost fill reads, per patch and face
// (x lower, x upper, y lower, y upper): every source cell of a copy or an
// interpolation entry is assigned to its nearest face, whose depth becomes
// at least one more than the cell's distance from it.  Cells outside every
// band are read by nothing but the next sweep, which overwrites them.
__device__ __forceinline__ void band_mark(const PatchDev &S, int pid, int sx, int sy, int *band) {
  if (sx < 0 || sx >= S.nx || sy < 0 || sy >= S.ny) return;
  const int d[4] = {sx, S.nx - 1 - sx, sy, S.ny - 1 - sy};
  int f = 0;
  for (int k = 1; k < 4; k++)
    if (d[k] < d[f]) f = k;
  atomicMax(&band[4 * pid + f], d[f] + 1);
}

__global__ void k_build_bands(const PatchDev *__restrict__ patches, const GhostItemDev *__restrict__ items,
                              const GhostCellDev *__restrict__ cells, int ncopy, int ninterp,
                              const InterpPlanDev *__restrict__ plan, int *__restrict__ band) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ncopy + ninterp; e += gridDim.x * blockDim.x) {
    const GhostCellDev gc = cells[e];
    const GhostItemDev it = items[gc.item];
    const PatchDev &S = patches[it.src];
    if (e < ncopy) {
      const int x = gc.k / it.size[1], y = gc.k - x * it.size[1];
      band_mark(S, it.src, it.src_off[0] + x, it.src_off[1] + y, band);
    } else {
      const InterpPlanDev pl = plan[e - ncopy];
      for (int kk = 0; kk < 4; kk++) band_mark(S, it.src, pl.bx + (kk & 1), pl.by + ((kk >> 1) & 1), band);
    }
  }
}

// Copy plan of the batched ghost fill: offsets of every COPY ghost cell,
// computed once per grid change.
__global__ void k_build_copy_plan(const PatchDev *__restrict__ patches,
                                  const GhostItemDev *__restrict__ items,
                                  const GhostCellDev *__restrict__ cells, int count,
                                  CopyPlanDev *__restrict__ plan) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < count; e += gridDim.x * blockDim.x) {
    const GhostCellDev gc = cells[e];
    const GhostItemDev it = items[gc.item];
    const PatchDev &S = patches[it.src], &D = patches[it.dst];
    const int x = gc.k / it.size[1], y = gc.k - x * it.size[1];
    CopyPlanDev pl;
    pl.src_new = idx_unew(S, 0, it.src_off[0] + x, it.src_off[1] + y);
    pl.src_old = idx_uold(S, 0, it.src_off[0] + x, it.src_off[1] + y);
    pl.dst = idx_uold(D, 0, it.dst_off[0] + x, it.dst_off[1] + y);
    pl.item = gc.item;
    pl.dst_pid = it.dst;
    plan[e] = pl;
  }
}

// Start of a batched fill: the time factor of every item (it is the same for
// all cells of the item) and its unknown strides.
__device__ __forceinline__ void item_step_one(const PatchDev *__restrict__ patches,
                                              const PatchTimeDev *__restrict__ times,
                                              const GhostItemDev *__restrict__ items, int i,
                                              GhostItemStepDev *__restrict__ out) {
  out[i] = item_step_value(patches, times, items, i);
}

__global__ void k_item_step(const PatchDev *__restrict__ patches,
                            const PatchTimeDev *__restrict__ times,
                            const GhostItemDev *__restrict__ items, int count,
                            GhostItemStepDev *__restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x)
    item_step_one(patches, times, items, i, out);
}

// Step start of the batched form in one launch: k_reset_step's per-group dt
// caps and activity and the per-item time factors of k_item_step (neither
// reads what the other writes).
__global__ void k_reset_items(int n_groups, const double *__restrict__ group_max_dt,
                              const double *__restrict__ group_t_end, const double *__restrict__ group_time,
                              unsigned long long *__restrict__ group_dt, int *__restrict__ group_active,
                              int n_patches, unsigned long long *__restrict__ patch_smax,
                              const PatchDev *__restrict__ patches, const PatchTimeDev *__restrict__ times,
                              const GhostItemDev *__restrict__ items, int count,
                              GhostItemStepDev *__restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int stride = gridDim.x * blockDim.x;
  if (i < n_groups) {
    const double rem = __dsub_rn(group_t_end[i], group_time[i]);
    const bool active = gt_nonneg(rem, 0.0);
    const double cap = active ? rem : 0.0;
    const double mx = group_max_dt[i];
    group_dt[i] = dbits(lt_ieee(cap, mx) ? cap : mx);
    group_active[i] = active ? 1 : 0;
  }
  for (int k = i; k < n_patches; k += stride) patch_smax[k] = 0ull;
  for (int k = i; k < count; k += stride) item_step_one(patches, times, items, k, out);
}


// Batched ghost fill over the flat ghost-cell list: entries [0, ncopy) copy
// (DefaultTransfer's time-interpolated copy, offsets from the copy plan),
// [ncopy, ncopy + ninterp) interpolate with their precomputed d-linear plan
// (SWE interpolation with the h+b wrap).  Items write disjoint ghost cells,
// one thread per ghost cell; three CTAs per SM (80 registers: the unrolled
// interpolation keeps its 16 source values in registers, the occupancy
// hides the load latency; 0.50 ms on the 50k mix against 0.53 ms at two
// CTAs and 0.60 ms with the loads interleaved with the sums).
__global__ void __launch_bounds__(256, 3)
    k_ghost_cells(double *__restrict__ slab, const PatchDev *__restrict__ patches,
                  const GhostItemDev *__restrict__ items, const GhostCellDev *__restrict__ cells,
                  int ncopy, int ninterp, const CopyPlanDev *__restrict__ copy_plan,
                  const InterpPlanDev *__restrict__ plan,
                  const GhostItemStepDev *__restrict__ item_step,
                  const int *__restrict__ group_active, const int *__restrict__ fin,
                  const int *__restrict__ pact) {
  const int total = ncopy + ninterp;
  const auto step = [item_step](int item) { return item_step[item]; };
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x)
    ghost_entry<false>(slab, patches, items, cells, ncopy, copy_plan, plan, step, e, group_active, fin, pact);
}

// Batched ghost fill: one warp per item.  Items write disjoint ghost cells.
__global__ void k_ghost_items(double *__restrict__ slab, const PatchDev *__restrict__ patches,
                              const PatchTimeDev *__restrict__ times,
                              const GhostItemDev *__restrict__ items, int first, int count,
                              const int *__restrict__ group_active) {
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int w = warp; w < count; w += nwarps) {
    GhostItemDev it = items[first + w];
    PatchDev S = patches[it.src], D = patches[it.dst];
    if (group_active && !group_active[D.group]) continue;
    PatchTimeDev ST = times[it.src], DT = times[it.dst];
    int ncell = it.size[0] * it.size[1];
    if (it.kind == 0) {
      double tf = transfer_tf(S, ST, D, DT);
      double itf = __dsub_rn(1.0, tf);
      for (int k = lane; k < ncell; k += 32) transfer_cell(slab, S, D, it.size, it.src_off, it.dst_off, tf, itf, k);
    } else {
      double tf = interp_tf(S, ST, D, DT, false, true);
      for (int k = lane; k < ncell; k += 32) interp_cell(slab, S, D, it.size, it.dst_off, tf, true, true, k);
    }
  }
}

// Walls of the listed patches in the order of SolveTimestep::fillBoundaryLayers:
// (0,lower), (1,upper), (0,upper), (1,lower).  One warp per patch.
__global__ void k_walls(double *__restrict__ slab, const PatchDev *__restrict__ patches,
                        const int *__restrict__ wall_patches, int count,
                        const int *__restrict__ group_active, const int *__restrict__ pact, int from_unew) {
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int order[4][2] = {{0, 0}, {1, 1}, {0, 1}, {1, 0}};
  for (int w = warp; w < count; w += nwarps) {
    PatchDev P = patches[wall_patches[w]];
    if (group_active && !group_active[P.group]) continue;
    if (pact && !pact[wall_patches[w]]) continue;
    for (int f = 0; f < 4; f++) {
      int d = order[f][0], up = order[f][1];
      if (P.wall & (1 << (2 * d + up))) wall_face<false>(slab, P, d, up, from_unew != 0, lane, 32);
      __syncwarp();
    }
  }
}

// Plain form, one launch per patch: the patch's ghost items, then its walls.
__global__ void k_fill_patch(double *__restrict__ slab, const PatchDev *__restrict__ patches,
                             const PatchTimeDev *__restrict__ times,
                             const GhostItemDev *__restrict__ items, int first, int count, int pid,
                             const int *__restrict__ group_active) {
  if (group_active && !group_active[patches[pid].group]) return;
  int lane = threadIdx.x;
  for (int w = 0; w < count; w++) {
    GhostItemDev it = items[first + w];
    PatchDev S = patches[it.src], D = patches[it.dst];
    PatchTimeDev ST = times[it.src], DT = times[it.dst];
    int ncell = it.size[0] * it.size[1];
    if (it.kind == 0) {
      double tf = transfer_tf(S, ST, D, DT);
      double itf = __dsub_rn(1.0, tf);
      for (int k = lane; k < ncell; k += blockDim.x) transfer_cell(slab, S, D, it.size, it.src_off, it.dst_off, tf, itf, k);
    } else {
      double tf = interp_tf(S, ST, D, DT, false, true);
      for (int k = lane; k < ncell; k += blockDim.x) interp_cell(slab, S, D, it.size, it.dst_off, tf, true, true, k);
    }
  }
  __syncthreads();
  PatchDev P = patches[pid];
  const int order[4][2] = {{0, 0}, {1, 1}, {0, 1}, {1, 0}};
  for (int f = 0; f < 4; f++) {
    int d = order[f][0], up = order[f][1];
    if (P.wall & (1 << (2 * d + up))) wall_face<false>(slab, P, d, up, true, lane, blockDim.x);
    __syncthreads();
  }
}

// ===========================================================================
// Single Numerics operations (one launch each)
// ===========================================================================
__global__ void k_copy_unew_to_uold(double *slab, const PatchDev *patches, int pid) {
  PatchDev P = patches[pid];
  int n = P.nq * P.nx * P.ny;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    int q = k / (P.nx * P.ny), r = k - q * P.nx * P.ny, x = r / P.ny, y = r - x * P.ny;
    slab[idx_uold(P, q, x, y)] = slab[idx_unew(P, q, x, y)];
  }
}

// DefaultTransfer::swapUNewAndUOld (DefaultTransfer.cpph:115-127): the
// interior values of uNew and uOld trade places.
__global__ void k_swap_unew_uold(double *slab, const PatchDev *patches, int pid) {
  PatchDev P = patches[pid];
  int n = P.nq * P.nx * P.ny;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    int q = k / (P.nx * P.ny), r = k - q * P.nx * P.ny, x = r / P.ny, y = r - x * P.ny;
    const long long in = idx_unew(P, q, x, y), io = idx_uold(P, q, x, y);
    const double vn = slab[in], vo = slab[io];
    slab[in] = vo;
    slab[io] = vn;
  }
}

__global__ void k_fill_boundary_layer(double *slab, const PatchDev *patches, int pid, int dim, int up) {
  PatchDev P = patches[pid];
  wall_face<false>(slab, P, dim, up, false, threadIdx.x, blockDim.x);
}

__global__ void k_transfer(double *slab, const PatchDev *patches, const PatchTimeDev *times,
                           GhostItemDev it) {
  PatchDev S = patches[it.src], D = patches[it.dst];
  double tf = transfer_tf(S, times[it.src], D, times[it.dst]);
  double itf = __dsub_rn(1.0, tf);
  int ncell = it.size[0] * it.size[1];
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < ncell; k += gridDim.x * blockDim.x)
    transfer_cell(slab, S, D, it.size, it.src_off, it.dst_off, tf, itf, k);
}

__global__ void k_interpolate(double *slab, const PatchDev *patches, const PatchTimeDev *times,
                              GhostItemDev it, int to_uold, int to_current, int use_unew_uold, int swe) {
  PatchDev S = patches[it.src], D = patches[it.dst];
  double tf = interp_tf(S, times[it.src], D, times[it.dst], to_current != 0, use_unew_uold != 0);
  int ncell = it.size[0] * it.size[1];
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < ncell; k += gridDim.x * blockDim.x)
    interp_cell(slab, S, D, it.size, it.dst_off, tf, to_uold != 0, swe != 0, k);
}

// ---------------------------------------------------------------------------
// Restriction
// ---------------------------------------------------------------------------
// Region::getRegionsOverlappedByNeighboringGhostlayers (Region.cpp:247-315)
__device__ int regions_overlapped(const double lower[2], const double upper[2], const double sp[2],
                                  const double ss[2], const double sub[2], const int n[2],
                                  int off[8], int sz[8]) {
  bool one_greater = false, one_ge = false, all_greater = true;
  for (int d = 0; d < 2; d++) {
    if (tl_greater(__dadd_rn(upper[d], sub[d]), lower[d])) one_greater = true;
    if (__dsub_rn(upper[d], __dadd_rn(sp[d], ss[d])) >= -kTarchEps) one_ge = true;
    if (!tl_greater(lower[d], sp[d])) all_greater = false;
  }
  if (one_greater || one_ge || !all_greater) {
    for (int k = 0; k < 8; k++) { off[k] = 0; sz[k] = 0; }
    sz[0] = n[0]; sz[1] = n[1];
    return 1;
  }
  const double eps = 1e-12;
  int lo[2], up[2];
  for (int d = 0; d < 2; d++) {
    const double isub = ieee::rcp_rn(sub[d]);
    double dl = __dadd_rn(__dmul_rn(__dsub_rn(lower[d], sp[d]), isub), eps);
    double du = __dsub_rn(__dmul_rn(__dsub_rn(upper[d], sp[d]), isub), eps);
    dl = fmin(2147483647.0, dl);
    du = fmax(-2147483648.0, du);
    int a = (int)floor(dl), b = (int)floor(du);
    a = a < n[d] ? a : n[d];
    b = b < n[d] ? b : n[d];
    lo[d] = a > -1 ? a : -1;
    up[d] = b > -1 ? b : -1;
  }
  for (int d = 0; d < 2; d++) {
    int r0 = 2 * d, r1 = 2 * d + 1;
    sz[2 * r0 + d] = up[d] + 1; off[2 * r0 + d] = 0;
    sz[2 * r1 + d] = n[d] - lo[d]; off[2 * r1 + d] = lo[d];
    for (int i = 0; i < d; i++) {
      sz[2 * r0 + i] = -up[i] - 1 + lo[i]; off[2 * r0 + i] = up[i] + 1;
      sz[2 * r1 + i] = sz[2 * r0 + i]; off[2 * r1 + i] = off[2 * r0 + i];
    }
    for (int i = d + 1; i < 2; i++) {
      sz[2 * r0 + i] = n[i]; off[2 * r0 + i] = 0;
      sz[2 * r1 + i] = n[i]; off[2 * r1 + i] = 0;
    }
  }
  return 4;
}

// Region::mapToPatch (Region.cpp:174-206)
__device__ void map_to_patch(const int roff[2], const int rsz[2], const PatchDev &S,
                             const PatchDev &D, double eps, int ooff[2], int osz[2]) {
  for (int d = 0; d < 2; d++) {
    double ss = subcell(S, d), ds = subcell(D, d);
    double position = __dmul_rn(ss, (double)roff[d]);
    position = __dadd_rn(position, __dsub_rn(S.pos[d], D.pos[d]));
    double ot = ieee::div_rn(__dadd_rn(position, eps), ds);
    ooff[d] = (int)ot;
    double size = __dmul_rn(ss, (double)(roff[d] + rsz[d]));
    size = __dadd_rn(size, __dsub_rn(S.pos[d], D.pos[d]));
    double st = ieee::div_rn(__dsub_rn(size, eps), ds);
    st = __dsub_rn(st, (double)ooff[d]);
    st = __dadd_rn(st, 1.0);
    osz[d] = (int)st;
  }
}

// One restriction of src into dst (DefaultRestrictionTemplate::restrictSolution),
// executed by the whole CTA; regions are processed in order.
__device__ void restrict_block(double *slab, const PatchDev &S, const PatchTimeDev &ST,
                               const PatchDev &D, const PatchTimeDev &DT, bool only_overlapped,
                               bool swe) {
  int roff[8], rsz[8], nr;
  int n[2] = {S.nx, S.ny};
  if (only_overlapped) {
    double sp[2] = {S.pos[0], S.pos[1]}, ss[2] = {S.size[0], S.size[1]};
    double sub[2] = {subcell(S, 0), subcell(S, 1)};
    nr = regions_overlapped(DT.rl, DT.ru, sp, ss, sub, n, roff, rsz);
  } else {
    nr = 1;
    roff[0] = 0; roff[1] = 0; rsz[0] = n[0]; rsz[1] = n[1];
  }
  const double eps = 1e-12;
  double ssub[2] = {iter_sub(S, 0), iter_sub(S, 1)};
  double dsub[2] = {iter_sub(D, 0), iter_sub(D, 1)};
  double dvol = __dmul_rn(dsub[0], dsub[1]);
  double tfo = 1.0, tfn = 1.0;
  if (tl_greater(ST.dt, 0.0)) {
    double so = time_uold(S, ST), su = time_unew(S, ST);
    tfo = __ddiv_rn(__dsub_rn(0.0, so), __dsub_rn(su, so));
    tfn = __ddiv_rn(__dsub_rn(1.0, so), __dsub_rn(su, so));
  }
  for (int r = 0; r < nr; r++) {
    const int *ro = &roff[2 * r], *rs = &rsz[2 * r];
    if (only_overlapped && !(rs[0] > 0 && rs[1] > 0)) continue;
    int doff[2], dsz[2];
    map_to_patch(ro, rs, S, D, eps, doff, dsz);
    int ncell = dsz[0] > 0 && dsz[1] > 0 ? dsz[0] * dsz[1] : 0;
    for (int k = threadIdx.x; k < ncell; k += blockDim.x) {
      int x = doff[0] + k / dsz[1], y = doff[1] + k % dsz[1];
      double dpos[2] = {iter_pos(D, 0, x), iter_pos(D, 1, y)};
      int coff[2], csz[2];
      for (int d = 0; d < 2; d++) {
        double ot = __ddiv_rn(__dadd_rn(__dsub_rn(dpos[d], S.pos[d]), eps), ssub[d]);
        int o = (int)ot;
        double st = __ddiv_rn(__dsub_rn(__dsub_rn(__dadd_rn(dpos[d], dsub[d]), S.pos[d]), eps), ssub[d]);
        st = __dsub_rn(st, ot);
        st = __dadd_rn(st, 1.0);
        int up = o + (int)st;
        int rup = ro[d] + rs[d];
        int oo = o > ro[d] ? o : ro[d];
        int uu = up < rup ? up : rup;
        coff[d] = oo;
        csz[d] = uu - oo;
      }
      for (int sx = coff[0]; sx < coff[0] + csz[0]; sx++)
        for (int sy = coff[1]; sy < coff[1] + csz[1]; sy++) {
          double spos[2] = {iter_pos(S, 0, sx), iter_pos(S, 1, sy)};
          double region = 1.0;
          for (int d = 0; d < 2; d++) {
            double a = __dadd_rn(dpos[d], dsub[d]), b = __dadd_rn(spos[d], ssub[d]);
            double lo = dpos[d] > spos[d] ? dpos[d] : spos[d];
            region = __dmul_rn(region, __dsub_rn(a < b ? a : b, lo));
            region = fmax(region, 0.0);
          }
          for (int q = 0; q < D.nq; q++) {
            double vo = slab[idx_uold(S, q, sx, sy)];
            double vn = slab[idx_unew(S, q, sx, sy)];
            if (swe && q == 0) {
              double bb = slab[idx_pw(S, 0, sx, sy)];
              vo = __dadd_rn(vo, bb);
              vn = __dadd_rn(vn, bb);
            }
            double d_o = __ddiv_rn(__dmul_rn(__dadd_rn(__dmul_rn(vo, __dsub_rn(1.0, tfo)), __dmul_rn(vn, tfo)), region), dvol);
            double d_n = __ddiv_rn(__dmul_rn(__dadd_rn(__dmul_rn(vo, __dsub_rn(1.0, tfn)), __dmul_rn(vn, tfn)), region), dvol);
            long long io = idx_uold(D, q, x, y), in = idx_unew(D, q, x, y);
            slab[io] = __dadd_rn(slab[io], d_o);
            slab[in] = __dadd_rn(slab[in], d_n);
          }
        }
    }
    __syncthreads();
  }
}

__global__ void k_restrict(double *slab, const PatchDev *patches, const PatchTimeDev *times,
                           int src, int dst, int only_overlapped, int swe) {
  restrict_block(slab, patches[src], times[src], patches[dst], times[dst], only_overlapped != 0, swe != 0);
}

// Restriction of the items [b0, b1) (one destination) in list order, and
// within an item its regions in order (the same sequence as restrict_block).
// One warp per destination cell of a region: the lanes evaluate the
// contributions of up to 32 source cells at a time, lane 0 adds them to the
// cell's uOld / uNew values in source-cell order.
__device__ void restrict_items_in_order(double *slab, const PatchDev *patches, const PatchTimeDev *times,
                                        const int4 *items, int b0, int b1, double (*W)[32][6]) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int k = b0; k < b1; k++) {
    const int4 it = items[k];  // src, dst, only_overlapped, swe
    const PatchDev S = patches[it.x], D = patches[it.y];
    const PatchTimeDev ST = times[it.x], DT = times[it.y];
    const bool only_overlapped = it.z != 0, swe = it.w != 0;
    if (D.nq > 3) {
      restrict_block(slab, S, ST, D, DT, only_overlapped, swe);
      __syncthreads();
      continue;
    }
    int roff[8], rsz[8], nr;
    int n[2] = {S.nx, S.ny};
    if (only_overlapped) {
      double sp[2] = {S.pos[0], S.pos[1]}, ss[2] = {S.size[0], S.size[1]};
      double sub[2] = {subcell(S, 0), subcell(S, 1)};
      nr = regions_overlapped(DT.rl, DT.ru, sp, ss, sub, n, roff, rsz);
    } else {
      nr = 1;
      roff[0] = 0; roff[1] = 0; rsz[0] = n[0]; rsz[1] = n[1];
    }
    const double eps = 1e-12;
    const double ssub[2] = {iter_sub(S, 0), iter_sub(S, 1)};
    const double dsub[2] = {iter_sub(D, 0), iter_sub(D, 1)};
    const double dvol = __dmul_rn(dsub[0], dsub[1]);
    double tfo = 1.0, tfn = 1.0;
    if (tl_greater(ST.dt, 0.0)) {
      double so = time_uold(S, ST), su = time_unew(S, ST);
      tfo = __ddiv_rn(__dsub_rn(0.0, so), __dsub_rn(su, so));
      tfn = __ddiv_rn(__dsub_rn(1.0, so), __dsub_rn(su, so));
    }
    const double itfo = __dsub_rn(1.0, tfo), itfn = __dsub_rn(1.0, tfn);
    for (int r = 0; r < nr; r++) {
      const int *ro = &roff[2 * r], *rs = &rsz[2 * r];
      if (only_overlapped && !(rs[0] > 0 && rs[1] > 0)) continue;
      int doff[2], dsz[2];
      map_to_patch(ro, rs, S, D, eps, doff, dsz);
      const int ncell = dsz[0] > 0 && dsz[1] > 0 ? dsz[0] * dsz[1] : 0;
      for (int c = wid; c < ncell; c += (int)(blockDim.x >> 5)) {
        const int x = doff[0] + c / dsz[1], y = doff[1] + c % dsz[1];
        const double dpos[2] = {iter_pos(D, 0, x), iter_pos(D, 1, y)};
        int coff[2], csz[2];
        for (int d = 0; d < 2; d++) {
          double ot = __ddiv_rn(__dadd_rn(__dsub_rn(dpos[d], S.pos[d]), eps), ssub[d]);
          int o = (int)ot;
          double st = __ddiv_rn(__dsub_rn(__dsub_rn(__dadd_rn(dpos[d], dsub[d]), S.pos[d]), eps), ssub[d]);
          st = __dsub_rn(st, ot);
          st = __dadd_rn(st, 1.0);
          int up = o + (int)st;
          int rup = ro[d] + rs[d];
          int oo = o > ro[d] ? o : ro[d];
          int uu = up < rup ? up : rup;
          coff[d] = oo;
          csz[d] = uu - oo;
        }
        const int nsrc = csz[0] > 0 && csz[1] > 0 ? csz[0] * csz[1] : 0;
        if (nsrc == 0) continue;
        double acc[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        if (lane == 0) {
#pragma unroll
          for (int q = 0; q < 3; q++)
            if (q < D.nq) {
              acc[q] = slab[idx_uold(D, q, x, y)];
              acc[3 + q] = slab[idx_unew(D, q, x, y)];
            }
        }
        for (int base = 0; base < nsrc; base += 32) {
          const int kk = base + lane;
          if (kk < nsrc) {
            const int sx = coff[0] + kk / csz[1], sy = coff[1] + kk % csz[1];
            const double spos[2] = {iter_pos(S, 0, sx), iter_pos(S, 1, sy)};
            double region = 1.0;
            for (int d = 0; d < 2; d++) {
              double a = __dadd_rn(dpos[d], dsub[d]), b = __dadd_rn(spos[d], ssub[d]);
              double lo = dpos[d] > spos[d] ? dpos[d] : spos[d];
              region = __dmul_rn(region, __dsub_rn(a < b ? a : b, lo));
              region = fmax(region, 0.0);
            }
#pragma unroll
            for (int q = 0; q < 3; q++) {
              if (q >= D.nq) break;
              double vo = slab[idx_uold(S, q, sx, sy)];
              double vn = slab[idx_unew(S, q, sx, sy)];
              if (swe && q == 0) {
                double bb = slab[idx_pw(S, 0, sx, sy)];
                vo = __dadd_rn(vo, bb);
                vn = __dadd_rn(vn, bb);
              }
              W[wid][lane][q] = __ddiv_rn(__dmul_rn(__dadd_rn(__dmul_rn(vo, itfo), __dmul_rn(vn, tfo)), region), dvol);
              W[wid][lane][3 + q] = __ddiv_rn(__dmul_rn(__dadd_rn(__dmul_rn(vo, itfn), __dmul_rn(vn, tfn)), region), dvol);
            }
          }
          __syncwarp();
          if (lane == 0) {
            const int m = nsrc - base < 32 ? nsrc - base : 32;
            for (int j = 0; j < m; j++) {
#pragma unroll
              for (int q = 0; q < 3; q++)
                if (q < D.nq) {
                  acc[q] = __dadd_rn(acc[q], W[wid][j][q]);
                  acc[3 + q] = __dadd_rn(acc[3 + q], W[wid][j][3 + q]);
                }
            }
          }
          __syncwarp();
        }
        if (lane == 0) {
#pragma unroll
          for (int q = 0; q < 3; q++)
            if (q < D.nq) {
              slab[idx_uold(D, q, x, y)] = acc[q];
              slab[idx_unew(D, q, x, y)] = acc[3 + q];
            }
        }
      }
      __syncthreads();
    }
    __syncthreads();
  }
}


// Batched restriction of one destination (the restriction phase of
// k_level_transfer): the table of its items, then each interior cell once.
//
// restr_table_entry: per item the source, the time factors of its uOld / uNew
// values at the virtual times 0 and 1, and its regions (item order, then
// region order) mapped into the destination; *bad is set when a region
// leaves the destination (the item-by-item form is taken then).
//
// restr_cell_pair: the restricted uOld and uNew values of unknown q of the
// destination cell (x, y) -- the sums that the reference's clear,
// restrictSolution over the items in list order and postProcessRestriction
// leave in the cell, each formed in exactly that order: from the cleared
// 0.0, for every region of every item that holds the cell the terms of its
// source cells in loop order, then h + (-1 b).  The two sums share the
// regions, bounds and loads; the three unknowns of a cell are separate tasks.
// Per item of a destination: its regions in the source (the first half of a
// table entry, one thread per item).
struct RestrItemPre {
  double tfo, tfn;
  int src, nr, swe, pad_;
  int roff[8], rsz[8];
};

// The time factors of a source's uOld / uNew values at the virtual times 0
// and 1 (the interpolation weights of DefaultRestriction).
__device__ __forceinline__ void restr_time_factors(const PatchDev &S, const PatchTimeDev &ST, double &tfo,
                                                   double &tfn) {
  tfo = 1.0;
  tfn = 1.0;
  if (tl_greater(ST.dt, 0.0)) {
    double so = time_uold(S, ST), su = time_unew(S, ST);
    tfo = ieee::div_rn(__dsub_rn(0.0, so), __dsub_rn(su, so));
    tfn = ieee::div_rn(__dsub_rn(1.0, so), __dsub_rn(su, so));
  }
}

__device__ void restr_item_pre(const PatchDev *patches, const PatchTimeDev *times, const int4 it,
                               RestrItemPre &E) {
  const PatchDev S = patches[it.x];
  const PatchTimeDev DT = times[it.y];
  int nn[2] = {S.nx, S.ny};
  int nr;
  if (it.z != 0) {
    double sp[2] = {S.pos[0], S.pos[1]}, ss[2] = {S.size[0], S.size[1]};
    double sub[2] = {subcell(S, 0), subcell(S, 1)};
    nr = regions_overlapped(DT.rl, DT.ru, sp, ss, sub, nn, E.roff, E.rsz);
  } else {
    nr = 1;
    for (int k = 0; k < 8; k++) { E.roff[k] = 0; E.rsz[k] = 0; }
    E.rsz[0] = nn[0]; E.rsz[1] = nn[1];
  }
  E.tfo = 1.0; E.tfn = 1.0; E.src = it.x; E.nr = nr; E.swe = it.w; E.pad_ = it.z;
}

// Region r of an item mapped into the destination (the second half, one
// thread per (item, region)); *bad is set when it leaves the destination.
__device__ void restr_item_region(const PatchDev *patches, const RestrItemPre &P, int r, const PatchDev &D,
                                  RestrItemTab &E, int *bad) {
  const double eps = 1e-12;
  const int nr = P.nr;
  int doff[2] = {0, 0}, dsz[2] = {0, 0};
  if (r < nr && !(P.pad_ != 0 && !(P.rsz[2 * r] > 0 && P.rsz[2 * r + 1] > 0))) {
    const PatchDev S = patches[P.src];
    map_to_patch(&P.roff[2 * r], &P.rsz[2 * r], S, D, eps, doff, dsz);
    if (dsz[0] > 0 && dsz[1] > 0 &&
        (doff[0] < 0 || doff[1] < 0 || doff[0] + dsz[0] > D.nx || doff[1] + dsz[1] > D.ny))
      atomicOr(bad, 1);
  }
  for (int d = 0; d < 2; d++) {
    E.doff[r][d] = doff[d];
    E.dsz[r][d] = dsz[d] > 0 ? dsz[d] : 0;
    E.ro[r][d] = r < nr ? P.roff[2 * r + d] : 0;
    E.rs[r][d] = r < nr ? P.rsz[2 * r + d] : 0;
  }
  if (r == 0) {
    E.tfo = P.tfo; E.tfn = P.tfn; E.src = P.src; E.nr = nr; E.swe = P.swe; E.pad_ = 0;
  }
}

__device__ __forceinline__ bool restr_covers(const RestrItemTab &E, int r, int x, int y) {
  return x >= E.doff[r][0] && x < E.doff[r][0] + E.dsz[r][0] && y >= E.doff[r][1] &&
         y < E.doff[r][1] + E.dsz[r][1];
}

constexpr int kRestrBatch = 3;
__device__ void restr_cell_pair(double *slab, const PatchDev *patches, const PatchDev &D,
                                const RestrItemTab *T, int ni, int x, int y, int q, const double dsub[2],
                                double dvol) {
  const double eps = 1e-12;
  const double dpos[2] = {iter_pos(D, 0, x), iter_pos(D, 1, y)};
  const double da[2] = {__dadd_rn(dpos[0], dsub[0]), __dadd_rn(dpos[1], dsub[1])};
  double acc0 = 0.0, acc1 = 0.0;  // the cleared uOld / uNew values
  for (int t = 0; t < ni; t++) {
    const int nr = T[t].nr < 4 ? T[t].nr : 4;
    for (int r = 0; r < nr; r++) {
      if (!restr_covers(T[t], r, x, y)) continue;
      const PatchDev S = patches[T[t].src];
      const double ssub[2] = {iter_sub(S, 0), iter_sub(S, 1)};
      int coff[2], csz[2];
      for (int d = 0; d < 2; d++) {
        double ot = ieee::div_rn(__dadd_rn(__dsub_rn(dpos[d], S.pos[d]), eps), ssub[d]);
        int o = (int)ot;
        double st = ieee::div_rn(__dsub_rn(__dsub_rn(da[d], S.pos[d]), eps), ssub[d]);
        st = __dsub_rn(st, ot);
        st = __dadd_rn(st, 1.0);
        int up = o + (int)st;
        int rup = T[t].ro[r][d] + T[t].rs[r][d];
        int oo = o > T[t].ro[r][d] ? o : T[t].ro[r][d];
        int uu = up < rup ? up : rup;
        coff[d] = oo;
        csz[d] = uu - oo;
      }
      if (!(csz[0] > 0 && csz[1] > 0)) continue;
      const double tfo = T[t].tfo, tfn = T[t].tfn;
      const double itfo = __dsub_rn(1.0, tfo), itfn = __dsub_rn(1.0, tfn);
      const bool addb = T[t].swe != 0 && q == 0;
      for (int sx = coff[0]; sx < coff[0] + csz[0]; sx++) {
        // the x factor of the overlap area, once per source column
        const double sp0 = __dadd_rn(S.pos[0], __dmul_rn((double)sx, ssub[0]));
        const double b0 = __dadd_rn(sp0, ssub[0]);
        const double lo0 = dpos[0] > sp0 ? dpos[0] : sp0;
        const double r0 = fmax(__dmul_rn(1.0, __dsub_rn(da[0] < b0 ? da[0] : b0, lo0)), 0.0);
        // the terms of up to kRestrBatch source cells of the column are
        // formed side by side (independent divide chains), then added in
        // source order
        const int sy_end = coff[1] + csz[1];
        for (int sy0 = coff[1]; sy0 < sy_end; sy0 += kRestrBatch) {
          double t0[kRestrBatch], t1[kRestrBatch];
#pragma unroll
          for (int u = 0; u < kRestrBatch; u++) {
            const int sy = sy0 + u < sy_end ? sy0 + u : sy_end - 1;
            const double sp1 = __dadd_rn(S.pos[1], __dmul_rn((double)sy, ssub[1]));
            const double b1 = __dadd_rn(sp1, ssub[1]);
            const double lo1 = dpos[1] > sp1 ? dpos[1] : sp1;
            const double region = fmax(__dmul_rn(r0, __dsub_rn(da[1] < b1 ? da[1] : b1, lo1)), 0.0);
            double vo = slab[idx_uold(S, q, sx, sy)];
            double vn = slab[idx_unew(S, q, sx, sy)];
            if (addb) {
              double bb = slab[idx_pw(S, 0, sx, sy)];
              vo = __dadd_rn(vo, bb);
              vn = __dadd_rn(vn, bb);
            }
            t0[u] = ieee::div_rn(__dmul_rn(__dadd_rn(__dmul_rn(vo, itfo), __dmul_rn(vn, tfo)), region), dvol);
            t1[u] = ieee::div_rn(__dmul_rn(__dadd_rn(__dmul_rn(vo, itfn), __dmul_rn(vn, tfn)), region), dvol);
          }
#pragma unroll
          for (int u = 0; u < kRestrBatch; u++)
            if (sy0 + u < sy_end) {
              acc0 = __dadd_rn(acc0, t0[u]);
              acc1 = __dadd_rn(acc1, t1[u]);
            }
        }
      }
    }
  }
  if (q == 0) {
    const double nb = __dmul_rn(-1.0, slab[idx_pw(D, 0, x, y)]);
    acc0 = __dadd_rn(acc0, nb);
    acc1 = __dadd_rn(acc1, nb);
  }
  slab[idx_uold(D, q, x, y)] = acc0;
  slab[idx_unew(D, q, x, y)] = acc1;
}

__global__ void k_post_process_restriction(double *slab, const PatchDev *patches, const int *ids, int count,
                                           const int *group_active, const int *dirty) {
  PatchDev P = patches[ids[blockIdx.x % count]];
  if ((int)blockIdx.x >= count) return;
  if (dirty && !dirty[blockIdx.x]) return;
  if (group_active && !group_active[P.group]) return;
  for (int c = threadIdx.x; c < P.nx * P.ny; c += blockDim.x) {
    int x = c / P.ny, y = c % P.ny;
    double bb = slab[idx_pw(P, 0, x, y)];
    long long io = idx_uold(P, 0, x, y), in = idx_unew(P, 0, x, y);
    slab[io] = __dadd_rn(slab[io], __dmul_rn(-1.0, bb));
    slab[in] = __dadd_rn(slab[in], __dmul_rn(-1.0, bb));
  }
}

// ---------------------------------------------------------------------------
// Flux correction
// ---------------------------------------------------------------------------
__device__ __forceinline__ void compute_flux(int dim, const double u[3], double gf, double f[3]) {
  double m = u[1 + dim];
  f[0] = __dmul_rn(u[0], m);
  f[1] = __dmul_rn(u[1], m);
  f[2] = __dmul_rn(u[2], m);
  f[1] = __dmul_rn(f[1], u[0]);
  f[2] = __dmul_rn(f[2], u[0]);
  double pr = __dmul_rn(__dmul_rn(__dmul_rn(0.5, gf), u[0]), u[0]);
  f[1 + dim] = __dadd_rn(f[1 + dim], pr);
}

// The face flux of face cell c of side (dim, dir) of a patch: the mean of
// the fluxes of its uOld ghost and boundary cells (Numerics::computeFluxes).
__device__ __forceinline__ void face_flux(const double *slab, const PatchDev &P, int c, int dim, int dir,
                                          double gf, double f[3]) {
  const int n[2] = {P.nx, P.ny};
  const int inner = (dir == -1) ? 0 : n[dim] - 1;
  const int ghost = (dir == -1) ? -1 : n[dim];
  double gu[3], iu[3], gfx[3], ifx[3];
  for (int q = 0; q < 3; q++) {
    int gx = dim == 0 ? ghost : c, gy = dim == 0 ? c : ghost;
    int ix = dim == 0 ? inner : c, iy = dim == 0 ? c : inner;
    gu[q] = slab[idx_uold(P, q, gx, gy)];
    iu[q] = slab[idx_uold(P, q, ix, iy)];
  }
  compute_flux(dim, gu, gf, gfx);
  compute_flux(dim, iu, gf, ifx);
  for (int q = 0; q < 3; q++) f[q] = __dmul_rn(0.5, __dadd_rn(gfx[q], ifx[q]));
}

// Face cell k of a patch's four sides in storage order: (dim, dir, c).
__device__ __forceinline__ void face_of(const PatchDev &P, int k, int &dim, int &dir, int &c) {
  if (k < 2 * P.ny) { dim = 0; dir = (k < P.ny) ? -1 : 1; c = k % P.ny; }
  else { int r = k - 2 * P.ny; dim = 1; dir = (r < P.nx) ? -1 : 1; c = r % P.nx; }
}

// Numerics::computeFluxes of one patch: the face fluxes stored in the
// patch's flux area, by all threads of the CTA.
__device__ void store_patch_fluxes(double *slab, const PatchDev &P, double gf) {
  const int total = 2 * (P.ny + P.nx);
  for (int k = threadIdx.x; k < total; k += blockDim.x) {
    int dim, dir, c;
    face_of(P, k, dim, dir, c);
    double f[3];
    face_flux(slab, P, c, dim, dir, gf, f);
    for (int q = 0; q < 3; q++) slab[idx_flux(P, q, c, dim, dir)] = f[q];
  }
}

__global__ void k_compute_fluxes(double *slab, const PatchDev *patches, const int *ids, int count, double gf,
                                 const int *group_active) {
  if ((int)blockIdx.x >= count) return;
  PatchDev P = patches[ids[blockIdx.x]];
  if (group_active && !group_active[P.group]) return;
  store_patch_fluxes(slab, P, gf);
}

// DefaultFluxCorrectionTemplate::applyCorrection; the corrections of several
// source cells can land in one destination cell, so a single thread applies
// them in the reference's order.
__device__ void flux_correction_one(double *slab, const PatchDev *patches, const PatchTimeDev *times,
                                    int src, int dst, int dim, int dir) {
  PatchDev S = patches[src], D = patches[dst];
  PatchTimeDev ST = times[src], DT = times[dst];
  double lo = fmax(ST.time, DT.time);
  double hi = fmin(__dadd_rn(ST.time, ST.dt), __dadd_rn(DT.time, DT.dt));
  double tov = __dsub_rn(hi, lo);
  int rdim = 0;
  for (int d = 0; d < 2; d++) {
    if (tl_greater(D.pos[d], S.pos[d])) rdim = d;
    else if (tl_greater(S.pos[d], D.pos[d])) rdim = d;
  }
  double ssub[2] = {subcell(S, 0), subcell(S, 1)}, dsub[2] = {subcell(D, 0), subcell(D, 1)};
  double dvol = __dmul_rn(dsub[0], dsub[1]);
  int sn[2] = {S.nx, S.ny}, dn[2] = {D.nx, D.ny};
  int other = 1 - dim;
  const double heps = 1e-10;
  for (int cs = 0; cs < sn[other]; cs++) {
    int po = 1 - rdim;
    double npos = __dadd_rn(S.pos[po], __dmul_rn(ssub[po], (double)cs));
    double lb = fmax(D.pos[po], npos);
    double ub = fmin(__dadd_rn(D.pos[po], dsub[po]), __dadd_rn(npos, ssub[po]));
    int lbc = (int)__ddiv_rn(__dadd_rn(__dsub_rn(lb, D.pos[po]), heps), dsub[po]);
    int ubc = (int)ceil(__ddiv_rn(__dsub_rn(__dsub_rn(ub, D.pos[po]), heps), dsub[po]));
    double sF[3];
    for (int q = 0; q < 3; q++) sF[q] = slab[idx_flux(S, q, cs, dim, dir)];
    int dinner = (-dir == -1) ? 0 : dn[dim] - 1;
    for (int cd = lbc; cd < ubc; cd++) {
      double dF[3];
      for (int q = 0; q < 3; q++) dF[q] = slab[idx_flux(D, q, cd, dim, -dir)];
      double a1 = __dadd_rn(S.pos[other], __dmul_rn(__dadd_rn((double)cs, 1.0), ssub[other]));
      double a2 = __dadd_rn(D.pos[other], __dmul_rn(__dadd_rn((double)cd, 1.0), dsub[other]));
      double b1 = __dadd_rn(S.pos[other], __dmul_rn((double)cs, ssub[other]));
      double b2 = __dadd_rn(D.pos[other], __dmul_rn((double)cd, dsub[other]));
      double area = __dmul_rn(1.0, __dsub_rn(a1 < a2 ? a1 : a2, b1 > b2 ? b1 : b2));
      if (area < 0.0) area = 0.0;
      int ux = dim == 0 ? dinner : cd, uy = dim == 0 ? cd : dinner;
      if (ux < 0 || uy < 0 || ux >= D.nx || uy >= D.ny) continue;
      for (int q = 0; q < 3; q++) {
        double corr = __ddiv_rn(__dmul_rn(__dmul_rn(__dsub_rn(sF[q], dF[q]), tov), area), dvol);
        long long id = idx_unew(D, q, ux, uy);
        slab[id] = __dadd_rn(slab[id], corr);
      }
    }
  }
}

__global__ void k_flux_correction(double *slab, const PatchDev *patches, const PatchTimeDev *times,
                                  int src, int dst, int dim, int dir) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  flux_correction_one(slab, patches, times, src, dst, dim, dir);
}

// Flux correction of one destination, item after item (the form of
// k_level_transfer's flux phase for destinations whose items exceed its
// shared-memory tables): the items [b0, b1) (all with the same destination)
// in list order, reading the stored face fluxes.  Within
// an item one thread owns each (destination face cell, unknown) and adds the
// corrections of the source face cells that overlap it in source order (the
// order of flux_correction_one; the three unknowns are separate sums); the
// source cells' destination ranges are computed once per item into shared
// memory (s_lb, s_ub: kFluxMaxCells each).  Called by all threads of a CTA
// of at least kFluxThreads threads.
constexpr int kFluxLanes = 32;                 // face cells per round
constexpr int kFluxThreads = 3 * kFluxLanes;   // x 3 unknowns
constexpr int kFluxMaxCells = 1024;
__device__ void flux_destination_seq(double *slab, const PatchDev *patches, const PatchTimeDev *times,
                                     const int4 *items, int b0, int b1, const int *group_active, int *s_lb,
                                     int *s_ub) {
  for (int k = b0; k < b1; k++) {
    const int4 it = items[k];  // src, dst, dim, dir
    if (group_active && !group_active[patches[it.y].group]) continue;
    const PatchDev S = patches[it.x], D = patches[it.y];
    const int dim = it.z, dir = it.w, other = 1 - dim;
    const int sno = other == 0 ? S.nx : S.ny, dno = other == 0 ? D.nx : D.ny, dnd = dim == 0 ? D.nx : D.ny;
    if (sno > kFluxMaxCells) {
      if (threadIdx.x == 0) flux_correction_one(slab, patches, times, it.x, it.y, dim, dir);
      __syncthreads();
      continue;
    }
    const PatchTimeDev ST = times[it.x], DT = times[it.y];
    const double lo = fmax(ST.time, DT.time);
    const double hi = fmin(__dadd_rn(ST.time, ST.dt), __dadd_rn(DT.time, DT.dt));
    const double tov = __dsub_rn(hi, lo);
    int rdim = 0;
    for (int d = 0; d < 2; d++) {
      if (tl_greater(D.pos[d], S.pos[d])) rdim = d;
      else if (tl_greater(S.pos[d], D.pos[d])) rdim = d;
    }
    const double ssub0 = subcell(S, 0), ssub1 = subcell(S, 1), dsub0 = subcell(D, 0), dsub1 = subcell(D, 1);
    const double dvol = __dmul_rn(dsub0, dsub1);
    const double heps = 1e-10;
    const int po = 1 - rdim;
    const double ssp = po == 0 ? ssub0 : ssub1, dsp = po == 0 ? dsub0 : dsub1;
    const double spp = po == 0 ? S.pos[0] : S.pos[1], dpp = po == 0 ? D.pos[0] : D.pos[1];
    const double sso = other == 0 ? ssub0 : ssub1, dso = other == 0 ? dsub0 : dsub1;
    const double spo = other == 0 ? S.pos[0] : S.pos[1], dpo = other == 0 ? D.pos[0] : D.pos[1];
    for (int cs = threadIdx.x; cs < sno; cs += blockDim.x) {
      double npos = __dadd_rn(spp, __dmul_rn(ssp, (double)cs));
      double lb = fmax(dpp, npos);
      double ub = fmin(__dadd_rn(dpp, dsp), __dadd_rn(npos, ssp));
      s_lb[cs] = (int)ieee::div_rn(__dadd_rn(__dsub_rn(lb, dpp), heps), dsp);
      s_ub[cs] = (int)ceil(ieee::div_rn(__dsub_rn(__dsub_rn(ub, dpp), heps), dsp));
    }
    __syncthreads();
    const int dinner = (-dir == -1) ? 0 : dnd - 1;
    if ((int)threadIdx.x < kFluxThreads) {
      const int q = (int)threadIdx.x / kFluxLanes;
      for (int cd = (int)threadIdx.x - q * kFluxLanes; cd < dno; cd += kFluxLanes) {
        const int ux = dim == 0 ? dinner : cd, uy = dim == 0 ? cd : dinner;
        if (ux < 0 || uy < 0 || ux >= D.nx || uy >= D.ny) continue;
        const double dF = slab[idx_flux(D, q, cd, dim, -dir)];
        const double a2 = __dadd_rn(dpo, __dmul_rn(__dadd_rn((double)cd, 1.0), dso));
        const double b2 = __dadd_rn(dpo, __dmul_rn((double)cd, dso));
        for (int cs = 0; cs < sno; cs++) {
          if (cd < s_lb[cs] || cd >= s_ub[cs]) continue;
          double a1 = __dadd_rn(spo, __dmul_rn(__dadd_rn((double)cs, 1.0), sso));
          double b1 = __dadd_rn(spo, __dmul_rn((double)cs, sso));
          double area = __dmul_rn(1.0, __dsub_rn(a1 < a2 ? a1 : a2, b1 > b2 ? b1 : b2));
          if (area < 0.0) area = 0.0;
          double sF = slab[idx_flux(S, q, cs, dim, dir)];
          double corr = ieee::div_rn(__dmul_rn(__dmul_rn(__dsub_rn(sF, dF), tov), area), dvol);
          long long id = idx_unew(D, q, ux, uy);
          slab[id] = __dadd_rn(slab[id], corr);
        }
      }
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Level transfer of the batched step in one launch: the face fluxes of every
// leaf (computeFluxes), the flux-correction list (applyCorrection) and the
// restriction list into the virtual patches (clear, restrictSolution over
// the items in list order, postProcessRestriction), the order in which
// SolveTimestep::enterCell and GridLevelTransfer run them.
//
// A persistent grid claims work items from two queues:
//   A: [0, F)     flux destinations, then
//      [F, F+R)   restriction destinations (their sources include corrected
//                 leaves: they wait until every flux destination is done)
//   B: [0, S)     storage: the face fluxes of kTransferLeaves leaves into
//                 their flux areas (the corrections compute the face fluxes
//                 they need themselves, so nothing waits for these)
// The first F CTAs (R when there is no flux list) start on queue A, the
// others on queue B, so that the storage runs beside the corrections; a CTA
// whose queue is empty takes from the other one.  The flux items were all
// claimed before any restriction item, by CTAs that are running and wait on
// nothing, so the wait ends; it is bounded all the same, and one that runs
// out sets ctl->err (read by the host after the step) and skips its item.
// The last CTA to leave resets the counters for the next launch.
//
// Flux destination: per item (one CTA thread each) its geometry; per source
// face cell its destination range and face flux and per destination face cell
// its face flux, all at once; then one thread per (destination face cell,
// unknown) -- the first item whose side holds the cell owns it -- adds the
// corrections of every item's overlapping source cells in list order, then
// source order (flux_correction_one's order).  A destination with more items
// or face cells than the tables hold stores the face fluxes of its patches
// and takes flux_destination_seq.
//
// Restriction destination: the table of its items (one thread per item, then
// per (item, region)); every interior cell that no mapped region holds gets
// the cleared and post-processed values (h = 0 + (-1 b), hu = hv = 0); the
// (cell, unknown) pairs that regions hold are listed and computed by
// restr_cell_pair over the CTA's threads.  A destination with more items
// than the table holds, more than 3 unknowns, a region leaving it or more
// pairs than the list holds takes the item-by-item form (clear,
// restrict_items_in_order, post-process).
// ---------------------------------------------------------------------------
constexpr int kTransferLeaves = 2;
constexpr int kTransferMaxPairs = 3 * kRestrChunkCells;
constexpr int kTransferSpin = 1 << 20;
constexpr int kTransferWarps = kTransferThreads / 32;
constexpr int kXferFluxItems = 32;
constexpr int kXferFluxCells = 512;

struct XferFluxItem {
  int src, dim, dir, sno, dno, so, dof, dinner;
  double tov, dvol, spo, sso, dpo, dso, spp, ssp, dpp, dsp;
};
struct XferFluxSmem {
  XferFluxItem it[kXferFluxItems];
  int lb[kXferFluxCells], ub[kXferFluxCells];
  double sF[3][kXferFluxCells], dF[3][kXferFluxCells];
  int ni, nsrc, ndst, bad;
};
struct XferRestrSmem {
  RestrItemTab T[kRestrMaxItems];
  union {
    int pairs[kTransferMaxPairs];
    double W[kTransferWarps][32][6];
  } u;
  int bad, npairs;
};
constexpr size_t kTransferSmem =
    sizeof(XferFluxSmem) > sizeof(XferRestrSmem) ? sizeof(XferFluxSmem) : sizeof(XferRestrSmem);

__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// All threads: every earlier write of the CTA is done; one release-ordered
// increment of `counter`.
__device__ __forceinline__ void transfer_done(unsigned *counter) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(counter, 1u);
  }
}

// All threads: wait until *counter reaches target (bounded); false when the
// wait ran out or another wait already did (ctl->err set).
__device__ bool transfer_wait(const unsigned *counter, unsigned target, TransferCtl *ctl, int *s_flag) {
  if (threadIdx.x == 0) {
    int ok = 0;
    for (int i = 0; i < kTransferSpin; i++) {
      if (ld_acquire_gpu(counter) >= target) { ok = 1; break; }
      if (*(volatile int *)&ctl->err) break;
      __nanosleep(64);
    }
    if (!ok) atomicCAS(&ctl->err, 0, 1);
    __threadfence();
    *s_flag = ok;
  }
  __syncthreads();
  const bool ok = *s_flag != 0;
  __syncthreads();
  return ok;
}

__device__ void flux_destination(double *slab, const PatchDev *patches, const PatchTimeDev *times,
                                 const int4 *items, int b0, int b1, const int *group_active, double gf,
                                 XferFluxSmem &M) {
  const int ni = b1 - b0;
  const PatchDev D = patches[items[b0].y];
  if (group_active && !group_active[D.group]) return;
  if (threadIdx.x == 0) M.bad = ni > kXferFluxItems ? 1 : 0;
  __syncthreads();
  if (!M.bad) {
    for (int t = threadIdx.x; t < ni; t += blockDim.x) {
      const int4 it = items[b0 + t];  // src, dst, dim, dir
      const PatchDev S = patches[it.x];
      const PatchTimeDev ST = times[it.x], DT = times[it.y];
      XferFluxItem &I = M.it[t];
      const int dim = it.z, dir = it.w, other = 1 - dim;
      I.src = it.x; I.dim = dim; I.dir = dir;
      I.sno = other == 0 ? S.nx : S.ny;
      I.dno = other == 0 ? D.nx : D.ny;
      I.dinner = (-dir == -1) ? 0 : (dim == 0 ? D.nx : D.ny) - 1;
      const double lo = fmax(ST.time, DT.time);
      const double hi = fmin(__dadd_rn(ST.time, ST.dt), __dadd_rn(DT.time, DT.dt));
      I.tov = __dsub_rn(hi, lo);
      int rdim = 0;
      for (int d = 0; d < 2; d++) {
        if (tl_greater(D.pos[d], S.pos[d])) rdim = d;
        else if (tl_greater(S.pos[d], D.pos[d])) rdim = d;
      }
      const double ssub0 = subcell(S, 0), ssub1 = subcell(S, 1), dsub0 = subcell(D, 0), dsub1 = subcell(D, 1);
      I.dvol = __dmul_rn(dsub0, dsub1);
      const int po = 1 - rdim;
      I.ssp = po == 0 ? ssub0 : ssub1; I.dsp = po == 0 ? dsub0 : dsub1;
      I.spp = po == 0 ? S.pos[0] : S.pos[1]; I.dpp = po == 0 ? D.pos[0] : D.pos[1];
      I.sso = other == 0 ? ssub0 : ssub1; I.dso = other == 0 ? dsub0 : dsub1;
      I.spo = other == 0 ? S.pos[0] : S.pos[1]; I.dpo = other == 0 ? D.pos[0] : D.pos[1];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      int so = 0, dof = 0;
      for (int t = 0; t < ni; t++) {
        M.it[t].so = so; M.it[t].dof = dof;
        so += M.it[t].sno; dof += M.it[t].dno;
      }
      M.nsrc = so; M.ndst = dof;
      if (so > kXferFluxCells || dof > kXferFluxCells) M.bad = 1;
    }
    __syncthreads();
  }
  if (M.bad) {
    // the item-by-item form reads the stored face fluxes: store those of
    // the destination and of every source first
    store_patch_fluxes(slab, D, gf);
    for (int k = b0; k < b1; k++) store_patch_fluxes(slab, patches[items[k].x], gf);
    __syncthreads();
    flux_destination_seq(slab, patches, times, items, b0, b1, group_active, &M.lb[0], &M.ub[0]);
    return;
  }
  // source cells: destination range and face flux; destination face cells:
  // face flux
  const double heps = 1e-10;
  for (int e = threadIdx.x; e < M.nsrc + M.ndst; e += blockDim.x) {
    const bool src = e < M.nsrc;
    const int f = src ? e : e - M.nsrc;
    int t = 0;
    while (t + 1 < ni && (src ? M.it[t + 1].so : M.it[t + 1].dof) <= f) t++;
    const XferFluxItem &I = M.it[t];
    double F[3];
    if (src) {
      const int cs = f - I.so;
      const PatchDev S = patches[I.src];
      double npos = __dadd_rn(I.spp, __dmul_rn(I.ssp, (double)cs));
      double lb = fmax(I.dpp, npos);
      double ub = fmin(__dadd_rn(I.dpp, I.dsp), __dadd_rn(npos, I.ssp));
      M.lb[f] = (int)ieee::div_rn(__dadd_rn(__dsub_rn(lb, I.dpp), heps), I.dsp);
      M.ub[f] = (int)ceil(ieee::div_rn(__dsub_rn(__dsub_rn(ub, I.dpp), heps), I.dsp));
      face_flux(slab, S, cs, I.dim, I.dir, gf, F);
      for (int q = 0; q < 3; q++) M.sF[q][f] = F[q];
    } else {
      const int cd = f - I.dof;
      face_flux(slab, D, cd, I.dim, -I.dir, gf, F);
      for (int q = 0; q < 3; q++) M.dF[q][f] = F[q];
    }
  }
  __syncthreads();
  // one thread per (destination face cell, unknown), owned by the first item
  // whose side holds the cell
  for (int task = threadIdx.x; task < 3 * M.ndst; task += blockDim.x) {
    const int j = task / 3, q = task - 3 * j;
    int k = 0;
    while (k + 1 < ni && M.it[k + 1].dof <= j) k++;
    const int cd0 = j - M.it[k].dof;
    const int ux = M.it[k].dim == 0 ? M.it[k].dinner : cd0, uy = M.it[k].dim == 0 ? cd0 : M.it[k].dinner;
    bool owner = true;
    for (int k2 = 0; k2 < k && owner; k2++) {
      const XferFluxItem &I = M.it[k2];
      if (I.dim == 0 ? (ux == I.dinner && uy < I.dno) : (uy == I.dinner && ux < I.dno)) owner = false;
    }
    if (!owner || ux < 0 || uy < 0 || ux >= D.nx || uy >= D.ny) continue;
    const long long id = idx_unew(D, q, ux, uy);
    double acc = 0.0;
    bool any = false;
    for (int k2 = k; k2 < ni; k2++) {
      const XferFluxItem &I = M.it[k2];
      if (!(I.dim == 0 ? (ux == I.dinner && uy < I.dno) : (uy == I.dinner && ux < I.dno))) continue;
      const int cd = I.dim == 0 ? uy : ux;
      const double dF = M.dF[q][I.dof + cd];
      const double a2 = __dadd_rn(I.dpo, __dmul_rn(__dadd_rn((double)cd, 1.0), I.dso));
      const double b2 = __dadd_rn(I.dpo, __dmul_rn((double)cd, I.dso));
      for (int cs = 0; cs < I.sno; cs++) {
        if (cd < M.lb[I.so + cs] || cd >= M.ub[I.so + cs]) continue;
        double a1 = __dadd_rn(I.spo, __dmul_rn(__dadd_rn((double)cs, 1.0), I.sso));
        double b1 = __dadd_rn(I.spo, __dmul_rn((double)cs, I.sso));
        double area = __dmul_rn(1.0, __dsub_rn(a1 < a2 ? a1 : a2, b1 > b2 ? b1 : b2));
        if (area < 0.0) area = 0.0;
        double corr = ieee::div_rn(__dmul_rn(__dmul_rn(__dsub_rn(M.sF[q][I.so + cs], dF), I.tov), area), I.dvol);
        if (!any) {
          acc = slab[id];
          any = true;
        }
        acc = __dadd_rn(acc, corr);
      }
    }
    if (any) slab[id] = acc;
  }
}

// The region geometry of every restriction item (regions in the source,
// mapped into the destination), one CTA per destination, into geo (indexed
// like the items) and geo_bad[b] (the destination takes the item-by-item
// form).  It depends on the patches' geometry and the destinations'
// restriction bounds only, so it is rebuilt when those change, not per step.
__global__ void __launch_bounds__(128)
    k_restr_geometry(const PatchDev *patches, const PatchTimeDev *times, const int4 *items, const int *begin,
                     int n_dst, RestrItemTab *geo, int *geo_bad) {
  __shared__ RestrItemPre pre[kRestrMaxItems];
  __shared__ int s_bad;
  const int b = blockIdx.x;
  if (b >= n_dst) return;
  const int b0 = begin[b], b1 = begin[b + 1], ni = b1 - b0;
  const PatchDev D = patches[items[b0].y];
  if (threadIdx.x == 0) s_bad = (ni > kRestrMaxItems || D.nq > 3) ? 1 : 0;
  __syncthreads();
  if (!s_bad) {
    for (int t = threadIdx.x; t < ni; t += blockDim.x) restr_item_pre(patches, times, items[b0 + t], pre[t]);
    __syncthreads();
    for (int e = threadIdx.x; e < 4 * ni; e += blockDim.x) {
      RestrItemTab E;
      restr_item_region(patches, pre[e >> 2], e & 3, D, E, &s_bad);
      // each thread writes its own region's fields; region 0 also the header
      RestrItemTab &G = geo[b0 + (e >> 2)];
      const int r = e & 3;
      for (int d = 0; d < 2; d++) {
        G.doff[r][d] = E.doff[r][d];
        G.dsz[r][d] = E.dsz[r][d];
        G.ro[r][d] = E.ro[r][d];
        G.rs[r][d] = E.rs[r][d];
      }
      if (r == 0) {
        G.tfo = E.tfo; G.tfn = E.tfn; G.src = E.src; G.nr = E.nr; G.swe = E.swe; G.pad_ = 0;
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) geo_bad[b] = s_bad;
}

// One chunk of a restriction destination: cells [c0, c1) of its interior.
__device__ void restrict_destination(double *slab, const PatchDev *patches, const PatchTimeDev *times,
                                     const int4 *items, int b0, int b1, const PatchDev &D,
                                     const RestrItemTab *geo, int bad, int c0, int c1, XferRestrSmem &M) {
  const int ni = b1 - b0;
  const int n = D.nx * D.ny;
  if (threadIdx.x == 0) {
    M.bad = bad;
    M.npairs = 0;
  }
  __syncthreads();
  if (M.bad) {
    // item-by-item form, by the destination's first chunk: clear, every item
    // in order, post-process
    if (c0 != 0) return;
    for (int k = threadIdx.x; k < D.nq * n; k += blockDim.x) {
      int q = k / n, c = k - q * n, x = c / D.ny, y = c - x * D.ny;
      slab[idx_unew(D, q, x, y)] = 0.0;
      slab[idx_uold(D, q, x, y)] = 0.0;
    }
    __syncthreads();
    restrict_items_in_order(slab, patches, times, items, b0, b1, M.u.W);
    __syncthreads();
    for (int c = threadIdx.x; c < n; c += blockDim.x) {
      int x = c / D.ny, y = c % D.ny;
      double bb = slab[idx_pw(D, 0, x, y)];
      long long io = idx_uold(D, 0, x, y), in = idx_unew(D, 0, x, y);
      slab[io] = __dadd_rn(slab[io], __dmul_rn(-1.0, bb));
      slab[in] = __dadd_rn(slab[in], __dmul_rn(-1.0, bb));
    }
    return;
  }
  // the items' table: geometry, and this step's time factors
  for (int t = threadIdx.x; t < ni; t += blockDim.x) {
    RestrItemTab E = geo[b0 + t];
    restr_time_factors(patches[E.src], times[E.src], E.tfo, E.tfn);
    M.T[t] = E;
  }
  __syncthreads();
  int *pairs = M.u.pairs;
  for (int c = c0 + (int)threadIdx.x; c < c1; c += blockDim.x) {
    const int x = c / D.ny, y = c - x * D.ny;
    bool held = false;
    for (int t = 0; t < ni && !held; t++) {
      const int nr = M.T[t].nr < 4 ? M.T[t].nr : 4;
      for (int r = 0; r < nr && !held; r++) held = restr_covers(M.T[t], r, x, y);
    }
    if (!held) {
      const double nb = __dmul_rn(-1.0, slab[idx_pw(D, 0, x, y)]);
      const double h = __dadd_rn(0.0, nb);
      slab[idx_uold(D, 0, x, y)] = h;
      slab[idx_unew(D, 0, x, y)] = h;
      for (int q = 1; q < D.nq; q++) {
        slab[idx_uold(D, q, x, y)] = 0.0;
        slab[idx_unew(D, q, x, y)] = 0.0;
      }
    } else {
      // at most 3 unknowns x kRestrChunkCells cells: the list always holds them
      const int k = atomicAdd(&M.npairs, D.nq);
      for (int q = 0; q < D.nq; q++) pairs[k + q] = c * 4 + q;
    }
  }
  __syncthreads();
  const double dsub[2] = {iter_sub(D, 0), iter_sub(D, 1)};
  const double dvol = __dmul_rn(dsub[0], dsub[1]);
  const int np = M.npairs;
  for (int k = threadIdx.x; k < np; k += blockDim.x) {
    const int c = pairs[k] >> 2, q = pairs[k] & 3;
    const int x = c / D.ny, y = c - x * D.ny;
    restr_cell_pair(slab, patches, D, M.T, ni, x, y, q, dsub, dvol);
  }
}

__global__ void __launch_bounds__(kTransferThreads, 1)
    k_level_transfer(double *slab, const PatchDev *patches, const PatchTimeDev *times, const int *leaf_ids,
                     int n_leaf, double gf, const int4 *flux_items, const int *flux_begin, int n_flux,
                     const int4 *restr_items, const int *restr_begin, const RestrItemTab *restr_geo,
                     const int *restr_geo_bad, const int2 *restr_chunks, int n_restr, const int *group_active,
                     const int *pact, int wait_bias, TransferCtl *ctl) {
  extern __shared__ __align__(16) unsigned char xfer_smem[];
  __shared__ int s_item, s_flag;
  const int n_store = (n_leaf + kTransferLeaves - 1) / kTransferLeaves;
  const int n_a = n_flux + n_restr;
  int g_a = n_flux > 0 ? n_flux : n_restr;
  bool on_a = (int)blockIdx.x < g_a || n_store == 0;  // thread 0's queue
  for (;;) {
    if (threadIdx.x == 0) {
      int it = -1;
      for (int tries = 0; tries < 2 && it < 0; tries++) {
        if (on_a) {
          const unsigned k = atomicAdd(&ctl->next, 1u);
          if ((int)k < n_a) it = (int)k;
          else on_a = false;
        } else {
          const unsigned k = atomicAdd(&ctl->next_store, 1u);
          if ((int)k < n_store) it = n_a + (int)k;
          else on_a = true;
        }
      }
      s_item = it;
    }
    __syncthreads();
    const int item = s_item;
    __syncthreads();
    if (item < 0) break;
    if (item < n_flux) {
      flux_destination(slab, patches, times, flux_items, flux_begin[item], flux_begin[item + 1], group_active, gf,
                       *reinterpret_cast<XferFluxSmem *>(xfer_smem));
      transfer_done(&ctl->done_flux);
    } else if (item < n_flux + n_restr) {
      if (!transfer_wait(&ctl->done_flux, (unsigned)(n_flux + wait_bias), ctl, &s_flag)) continue;
      const int2 ch = restr_chunks[item - n_flux];  // destination, chunk
      const int b = ch.x;
      const int b0 = restr_begin[b], b1 = restr_begin[b + 1];
      const PatchDev D = patches[restr_items[b0].y];
      if (group_active && !group_active[D.group]) continue;
      if (pact) {
        // local time stepping: only destinations with an advancing source
        int any = 0;
        for (int k = b0 + (int)threadIdx.x; k < b1; k += blockDim.x) any |= pact[restr_items[k].x] ? 1 : 0;
        if (!__syncthreads_or(any)) continue;
      }
      const int c0 = ch.y * kRestrChunkCells, n = D.nx * D.ny;
      restrict_destination(slab, patches, times, restr_items, b0, b1, D, restr_geo, restr_geo_bad[b], c0,
                           c0 + kRestrChunkCells < n ? c0 + kRestrChunkCells : n,
                           *reinterpret_cast<XferRestrSmem *>(xfer_smem));
      __syncthreads();
    } else {
      // the face fluxes of up to kTransferLeaves leaves, all their face cells at once
      const int l0 = (item - n_flux - n_restr) * kTransferLeaves;
      const int l1 = l0 + kTransferLeaves < n_leaf ? l0 + kTransferLeaves : n_leaf;
      int tot = 0;
      for (int l = l0; l < l1; l++) {
        const PatchDev &P = patches[leaf_ids[l]];
        tot += 2 * (P.nx + P.ny);
      }
      for (int k = threadIdx.x; k < tot; k += blockDim.x) {
        int l = l0, kk = k;
        while (true) {
          const PatchDev &P = patches[leaf_ids[l]];
          const int m = 2 * (P.nx + P.ny);
          if (kk < m || l + 1 >= l1) break;
          kk -= m;
          l++;
        }
        const PatchDev P = patches[leaf_ids[l]];
        if (group_active && !group_active[P.group]) continue;
        int dim, dir, c;
        face_of(P, kk, dim, dir, c);
        double f[3];
        face_flux(slab, P, c, dim, dir, gf, f);
        for (int q = 0; q < 3; q++) slab[idx_flux(P, q, c, dim, dir)] = f[q];
      }
      __syncthreads();
    }
  }
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(&ctl->exited, 1u) == gridDim.x - 1) {
      ctl->next = 0;
      ctl->next_store = 0;
      ctl->done_flux = 0;
      ctl->exited = 0;
      __threadfence();
    }
  }
}

// Clears uNew and the uOld interior of the listed (virtual) patches before
// the restriction accumulates into them (Patch accessor clearRegion, called
// from GridLevelTransfer::switchToAndAddVirtualSubgrid).
__global__ void k_clear_interior(double *slab, const PatchDev *patches, const int *ids, int count,
                                 const int *group_active, const int *dirty) {
  if ((int)blockIdx.x >= count) return;
  if (dirty && !dirty[blockIdx.x]) return;
  PatchDev P = patches[ids[blockIdx.x]];
  if (group_active && !group_active[P.group]) return;
  int n = P.nx * P.ny;
  for (int k = threadIdx.x; k < P.nq * n; k += blockDim.x) {
    int q = k / n, c = k - q * n, x = c / P.ny, y = c - x * P.ny;
    slab[idx_unew(P, q, x, y)] = 0.0;
    slab[idx_uold(P, q, x, y)] = 0.0;
  }
}

// Patch::switchToLeaf data conversion (Patch.cpp:793-816 with
// switchRegionToMinimalFineGridTimeInterval, :55-76): the restricted values of
// a virtual patch stand for the times 0 and 1; the interior is re-evaluated
// at the patch's time (uOld) and time + dt (uNew).  One CTA.
__global__ void k_switch_to_leaf(double *__restrict__ slab, const PatchDev *__restrict__ patches,
                                 const PatchTimeDev *__restrict__ times, int pid) {
  const PatchDev P = patches[pid];
  const PatchTimeDev T = times[pid];
  const double time = 0.0, timestep = 1.0;
  double fo = 1.0, fn = 1.0;
  if (!tl_equals(timestep, 0.0)) {
    fo = __ddiv_rn(__dsub_rn(T.time, time), timestep);
    fn = __ddiv_rn(__dsub_rn(__dadd_rn(T.time, T.dt), time), timestep);
  }
  const double ofo = __dsub_rn(1.0, fo), ofn = __dsub_rn(1.0, fn);
  for (int k = threadIdx.x; k < P.nx * P.ny * P.nq; k += blockDim.x) {
    const int q = k / (P.nx * P.ny), c = k - q * (P.nx * P.ny), x = c / P.ny, y = c - x * P.ny;
    const long long io = idx_uold(P, q, x, y), in = idx_unew(P, q, x, y);
    const double vo = slab[io], vn = slab[in];
    slab[io] = __dadd_rn(__dmul_rn(vo, ofo), __dmul_rn(vn, fo));
    slab[in] = __dadd_rn(__dmul_rn(vo, ofn), __dmul_rn(vn, fn));
  }
}

// Finiteness flags of every patch slot: kFinUOld if every uOld interior
// unknown and kFinB if every interior value of the first parameter with
// ghost layer (b) is below 2^1022 in magnitude.  One CTA per slot.
__global__ void k_scan_fin(const double *__restrict__ slab, const PatchDev *__restrict__ patches, int count,
                           int *__restrict__ fin) {
  if ((int)blockIdx.x >= count) return;
  const PatchDev P = patches[blockIdx.x];
  __shared__ int bad_u, bad_b;
  if (threadIdx.x == 0) { bad_u = 0; bad_b = 0; }
  __syncthreads();
  if (P.nx > 0 && P.ny > 0) {
    const int nc = P.nx * P.ny;
    int bu = 0, bb = 0;
    for (int k = threadIdx.x; k < P.nq * nc; k += blockDim.x) {
      const int q = k / nc, c = k - q * nc, x = c / P.ny, y = c - x * P.ny;
      if (!small_mag(slab[idx_uold(P, q, x, y)])) bu = 1;
    }
    for (int k = threadIdx.x; k < (P.np_w > 0 ? nc : 0); k += blockDim.x) {
      const int x = k / P.ny, y = k - x * P.ny;
      if (!small_mag(slab[idx_pw(P, 0, x, y)])) bb = 1;
    }
    if (bu) atomicOr(&bad_u, 1);
    if (bb) atomicOr(&bad_b, 1);
  }
  __syncthreads();
  if (threadIdx.x == 0)
    fin[blockIdx.x] = (P.nx > 0 && P.np_w > 0) ? ((bad_u ? 0 : kFinUOld) | (bad_b ? 0 : kFinB)) : 0;
}

// Output gather: uNew (nq planes) and the interior of the parameters with
// ghost layer (np_w planes) of every listed patch, back to back, x-major
// planes of nx*ny values.  One CTA per patch.
__global__ void k_gather_cells(const double *__restrict__ slab, const PatchDev *__restrict__ patches,
                               const int *__restrict__ ids, const long long *__restrict__ out_off,
                               int count, double *__restrict__ out) {
  if ((int)blockIdx.x >= count) return;
  const PatchDev P = patches[ids[blockIdx.x]];
  double *o = out + out_off[blockIdx.x];
  const int nc = P.nx * P.ny;
  for (int k = threadIdx.x; k < P.nq * nc; k += blockDim.x) o[k] = slab[P.off + k];
  for (int k = threadIdx.x; k < P.np_w * nc; k += blockDim.x) {
    const int q = k / nc, c = k - q * nc, x = c / P.ny, y = c - x * P.ny;
    o[P.nq * nc + k] = slab[idx_pw(P, q, x, y)];
  }
}

// BreakingDam refinement criterion (BreakingDamSWEScenario::computeDemandedMeshWidth,
// native/scenarios/BreakingDam.cpp:85-139): max over xi < nx-1, yi < ny-1 of
// sqrt(|gx| |gx| + |gy| |gy|), gx = (h[xi+1][yi] - h[xi][yi]) / dx,
// gy = (h[xi][yi+1] - h[xi][yi]) / dy on uNew; fmax keeps the non-NaN operand.
// One CTA per listed patch.
__global__ void k_refinement_indicator(const double *__restrict__ slab, const PatchDev *__restrict__ patches,
                                       const int *__restrict__ ids, int count, int kind,
                                       double *__restrict__ out) {
  if ((int)blockIdx.x >= count) return;
  const PatchDev P = patches[ids[blockIdx.x]];
  const double dx = subcell(P, 0), dy = subcell(P, 1);
  const int mx = P.nx - 1, my = P.ny - 1;
  // kind 0: depth h, differences / subcell size (BreakingDam.cpp:100-116);
  // kind 1: surface h + b, plain differences (BowlOcean.cpp:106-122);
  // kind 2: surface h + b, differences / subcell size
  const bool surface = kind != 0, divide = kind != 1;
  auto value = [&](int x, int y) {
    const double h = slab[idx_unew(P, 0, x, y)];
    return surface ? __dadd_rn(h, slab[idx_pw(P, 0, x, y)]) : h;
  };
  double m = 0.0;
  for (int k = threadIdx.x; k < mx * my; k += blockDim.x) {
    const int xi = k / my, yi = k - xi * my;
    const double q0 = value(xi, yi);
    double gx = __dsub_rn(value(xi + 1, yi), q0);
    double gy = __dsub_rn(value(xi, yi + 1), q0);
    if (divide) {
      gx = ieee::div_rn(gx, dx);
      gy = ieee::div_rn(gy, dy);
    }
    const double ax = fabs(gx), ay = fabs(gy);
    m = fmax_nonneg(m, ieee::sqrt_rn(__dadd_rn(__dmul_rn(ax, ax), __dmul_rn(ay, ay))));
  }
  __shared__ unsigned long long red[32];
  // values are >= 0 or NaN; fmax_nonneg ignores NaN, so reduce with it
  for (int o = 16; o > 0; o >>= 1) m = fmax_nonneg(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = dbits(m);
  __syncthreads();
  if (threadIdx.x == 0) {
    double r = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) r = fmax_nonneg(r, bitsd(red[w]));
    out[blockIdx.x] = r;
  }
}

// ===========================================================================
// Host-side launchers
// ===========================================================================
cudaError_t launch_sweep(cudaStream_t st, int grid, double *slab, const PatchDev *patches,
                         const TileItem *tiles, int first, int count, const SweParamsDev &prm,
                         unsigned long long *patch_smax, unsigned long long *group_dt,
                         const int *group_active, int *fin, const int *pact) {
  if (count <= 0) return cudaSuccess;
  k_sweep_tiles<<<grid, kSweepThreads, 0, st>>>(slab, patches, tiles, first, count, prm, patch_smax,
                                                group_dt, group_active, fin, pact);
  return cudaGetLastError();
}

cudaError_t launch_sweep_tma(cudaStream_t st, int grid, double *slab, const PatchDev *patches,
                             const TileMaps *maps, const TileItem *tiles, int first, int count,
                             const SweParamsDev &prm, unsigned long long *patch_smax, unsigned long long *group_dt,
                             const int *group_active, int *fin, const int *pact, int *err) {
  if (count <= 0) return cudaSuccess;
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k_sweep_tiles_tma, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)sizeof(TmaRaw));
    if (e != cudaSuccess) return e;
    attr = true;
  }
  k_sweep_tiles_tma<<<grid, kSweepThreads, sizeof(TmaRaw), st>>>(slab, patches, maps, tiles, first, count, prm,
                                                                 patch_smax, group_dt, group_active, fin, pact,
                                                                 err);
  return cudaGetLastError();
}

// Tensor maps of the TMA tile sweep for one patch of even size, ghost width 1,
// 3 unknowns and the bathymetry as the only parameter field with ghost layer.
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static EncodeTiledFn g_encode_tiled = nullptr;

cudaError_t encode_tile_maps(const PatchDev &P, double *slab, TileMaps *out) {
  if (!g_encode_tiled) {
    cudaDriverEntryPointQueryResult q;
    void *f = nullptr;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q);
    if (e != cudaSuccess) return e;
    if (q != cudaDriverEntryPointSuccess || !f) return cudaErrorSymbolNotFound;
    g_encode_tiled = (EncodeTiledFn)f;
  }
  const cuuint32_t bx = (cuuint32_t)((P.nx < kTile ? P.nx : kTile) + 2);
  const cuuint32_t byo = (cuuint32_t)((P.ny < kTile ? P.ny : kTile) + 2), byn = byo + 2;
  const cuuint64_t nx = (cuuint64_t)P.nx, ny = (cuuint64_t)P.ny;
  double *unew = slab + P.off;
  double *uold = unew + 3 * nx * ny;
  double *b = uold + 3 * (nx + 2) * (ny + 2);
  const cuuint32_t es[3] = {1, 1, 1};
  {
    const cuuint64_t dims[3] = {ny, nx, 3};
    const cuuint64_t strides[2] = {ny * 8, nx * ny * 8};
    const cuuint32_t box[3] = {byn, bx, 3};
    if (g_encode_tiled(&out->unew, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, unew, dims, strides, box, es,
                       CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                       CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return cudaErrorInvalidValue;
  }
  {
    const cuuint64_t dims[3] = {ny + 2, nx + 2, 3};
    const cuuint64_t strides[2] = {(ny + 2) * 8, (nx + 2) * (ny + 2) * 8};
    const cuuint32_t box[3] = {byo, bx, 3};
    if (g_encode_tiled(&out->uold, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, uold, dims, strides, box, es,
                       CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                       CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return cudaErrorInvalidValue;
  }
  {
    const cuuint64_t dims[2] = {ny + 2, nx + 2};
    const cuuint64_t strides[1] = {(ny + 2) * 8};
    const cuuint32_t box[2] = {byo, bx};
    if (g_encode_tiled(&out->b, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, b, dims, strides, box, es,
                       CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                       CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return cudaErrorInvalidValue;
  }
  return cudaSuccess;
}

bool tma_tile_shape(const PatchDev &P) {
  return P.nx >= 2 && P.ny >= 2 && P.nx % 2 == 0 && P.ny % 2 == 0 && P.g == 1 && P.nq == 3 && P.np_wo == 0 &&
         P.np_w == 1;
}

cudaError_t launch_update(cudaStream_t st, int grid, double *slab, const PatchDev *patches,
                          PatchTimeDev *times, const TileItem *tiles, int first, int count,
                          const SweParamsDev &prm, const unsigned long long *patch_smax,
                          const unsigned long long *group_dt, const int *group_active, int *fin,
                          const int *pact, const unsigned long long *pdt) {
  if (count <= 0) return cudaSuccess;
  k_update_tiles<<<grid, kSweepThreads, 0, st>>>(slab, patches, times, tiles, first, count, prm,
                                                 patch_smax, group_dt, group_active, fin, pact, pdt);
  return cudaGetLastError();
}

cudaError_t launch_reset(cudaStream_t st, int n_groups, const double *group_max_dt,
                         const double *group_t_end, const double *group_time,
                         unsigned long long *group_dt, int *group_active, int n_patches,
                         unsigned long long *patch_smax) {
  int n = n_groups > n_patches ? n_groups : n_patches;
  int grid = (n + 255) / 256;
  if (grid > 1024) grid = 1024;
  if (grid < 1) grid = 1;
  k_reset_step<<<grid, 256, 0, st>>>(n_groups, group_max_dt, group_t_end, group_time, group_dt,
                                     group_active, n_patches, patch_smax);
  return cudaGetLastError();
}

cudaError_t launch_lts(cudaStream_t st, int phase, int n_patches, int n_groups, const PatchDev *patches,
                       PatchTimeDev *times, const GhostItemDev *items, int n_items,
                       const LtsVirtualDev &vt, unsigned long long *nbmin, unsigned long long *patch_smax,
                       unsigned long long *group_tmin, unsigned long long *group_dt,
                       const double *group_max_dt, const double *group_t_end, const int *group_active,
                       int *pact, double *pmaxdt, unsigned long long *pdt, double *group_time,
                       const SweParamsDev &prm, unsigned long long *cells) {
  const int np = n_patches > 0 ? n_patches : 1;
  const int gp = (np + 255) / 256 < 1024 ? (np + 255) / 256 : 1024;
  auto grid_for = [](int n) { return (n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096; };
  switch (phase) {
    case 0:
      k_lts_begin<<<gp, 256, 0, st>>>(n_patches, nbmin, patch_smax, n_groups, group_tmin, group_dt);
      if (vt.n_pairs > 0 && vt.n_virtual > 0) {
        k_lts_vt_reset<<<grid_for(vt.n_virtual), 256, 0, st>>>(vt.virtuals, vt.n_virtual, vt.start, vt.end);
        k_lts_vt_pairs<<<grid_for(vt.n_pairs), 256, 0, st>>>(vt.pairs, vt.n_pairs, times, vt.start, vt.end);
        k_lts_vt_set<<<grid_for(vt.n_virtual), 256, 0, st>>>(vt.virtuals, vt.n_virtual, vt.start, vt.end,
                                                             times);
      }
      if (n_items > 0)
        k_lts_nbmin<<<grid_for(n_items), 256, 0, st>>>(items, n_items, times, nbmin);
      k_lts_activity<<<gp, 256, 0, st>>>(patches, times, n_patches, nbmin, group_max_dt, group_t_end,
                                         group_active, pact, pmaxdt);
      break;
    case 1:
      k_lts_dt<<<gp, 256, 0, st>>>(patches, times, n_patches, pact, pmaxdt, patch_smax, prm, pdt, group_dt,
                                   group_tmin, cells);
      break;
    default:
      k_lts_end<<<(n_groups + 127) / 128, 128, 0, st>>>(n_groups, group_tmin, group_time, group_dt);
      break;
  }
  return cudaGetLastError();
}

cudaError_t launch_group_advance(cudaStream_t st, int n_groups, const unsigned long long *group_dt,
                                 const int *group_active, double *group_time) {
  k_group_advance<<<(n_groups + 127) / 128, 128, 0, st>>>(n_groups, group_dt, group_active, group_time);
  return cudaGetLastError();
}

cudaError_t launch_record_dt(cudaStream_t st, int n_groups, const unsigned long long *group_dt,
                             double *out) {
  k_record_dt<<<(n_groups + 127) / 128, 128, 0, st>>>(n_groups, group_dt, out);
  return cudaGetLastError();
}

cudaError_t launch_ghost_items(cudaStream_t st, double *slab, const PatchDev *patches,
                               const PatchTimeDev *times, const GhostItemDev *items, int first,
                               int count, const int *group_active) {
  if (count <= 0) return cudaSuccess;
  int warps_per_block = 8;
  int grid = (count + warps_per_block - 1) / warps_per_block;
  if (grid > 152 * 16) grid = 152 * 16;
  k_ghost_items<<<grid, 32 * warps_per_block, 0, st>>>(slab, patches, times, items, first, count,
                                                       group_active);
  return cudaGetLastError();
}

cudaError_t launch_build_interp_plan(cudaStream_t st, const PatchDev *patches,
                                     const GhostItemDev *items, const GhostCellDev *cells, int count,
                                     InterpPlanDev *plan) {
  if (count <= 0) return cudaSuccess;
  int grid = (count + 255) / 256;
  if (grid > 152 * 32) grid = 152 * 32;
  k_build_interp_plan<<<grid, 256, 0, st>>>(patches, items, cells, count, plan);
  return cudaGetLastError();
}

cudaError_t launch_ghost_cells(cudaStream_t st, double *slab, const PatchDev *patches,
                               const GhostItemDev *items, const GhostCellDev *cells, int ncopy,
                               int ninterp, const CopyPlanDev *copy_plan, const InterpPlanDev *plan,
                               const GhostItemStepDev *item_step, const int *group_active,
                               const int *fin, const int *pact) {
  int total = ncopy + ninterp;
  if (total <= 0) return cudaSuccess;
  int grid = (total + 255) / 256;
  if (grid > 152 * 32) grid = 152 * 32;
  k_ghost_cells<<<grid, 256, 0, st>>>(slab, patches, items, cells, ncopy, ninterp, copy_plan, plan,
                                      item_step, group_active, fin, pact);
  return cudaGetLastError();
}

cudaError_t launch_build_copy_plan(cudaStream_t st, const PatchDev *patches, const GhostItemDev *items,
                                   const GhostCellDev *cells, int count, CopyPlanDev *plan) {
  if (count <= 0) return cudaSuccess;
  int grid = (count + 255) / 256;
  if (grid > 152 * 32) grid = 152 * 32;
  k_build_copy_plan<<<grid, 256, 0, st>>>(patches, items, cells, count, plan);
  return cudaGetLastError();
}

cudaError_t launch_build_bands(cudaStream_t st, const PatchDev *patches, const GhostItemDev *items,
                               const GhostCellDev *cells, int ncopy, int ninterp, const InterpPlanDev *plan,
                               int *band) {
  const int total = ncopy + ninterp;
  if (total <= 0) return cudaSuccess;
  int grid = (total + 255) / 256;
  if (grid > 152 * 32) grid = 152 * 32;
  k_build_bands<<<grid, 256, 0, st>>>(patches, items, cells, ncopy, ninterp, plan, band);
  return cudaGetLastError();
}

cudaError_t launch_reset_items(cudaStream_t st, int n_groups, const double *group_max_dt, const double *group_t_end,
                               const double *group_time, unsigned long long *group_dt, int *group_active,
                               int n_patches, unsigned long long *patch_smax, const PatchDev *patches,
                               const PatchTimeDev *times, const GhostItemDev *items, int count,
                               GhostItemStepDev *out) {
  int n = n_groups > n_patches ? n_groups : n_patches;
  if (count > n) n = count;
  int grid = (n + 255) / 256;
  if (grid > 152 * 32) grid = 152 * 32;
  if (grid < 1) grid = 1;
  k_reset_items<<<grid, 256, 0, st>>>(n_groups, group_max_dt, group_t_end, group_time, group_dt, group_active,
                                      n_patches, patch_smax, patches, times, items, count, out);
  return cudaGetLastError();
}

cudaError_t launch_item_step(cudaStream_t st, const PatchDev *patches, const PatchTimeDev *times,
                             const GhostItemDev *items, int count, GhostItemStepDev *out) {
  if (count <= 0) return cudaSuccess;
  int grid = (count + 255) / 256;
  if (grid > 152 * 32) grid = 152 * 32;
  k_item_step<<<grid, 256, 0, st>>>(patches, times, items, count, out);
  return cudaGetLastError();
}

cudaError_t launch_walls(cudaStream_t st, double *slab, const PatchDev *patches,
                         const int *wall_patches, int count, const int *group_active,
                         const int *pact, int from_unew) {
  if (count <= 0) return cudaSuccess;
  int grid = (count + 7) / 8;
  if (grid > 152 * 16) grid = 152 * 16;
  k_walls<<<grid, 256, 0, st>>>(slab, patches, wall_patches, count, group_active, pact, from_unew);
  return cudaGetLastError();
}

cudaError_t launch_fill_patch(cudaStream_t st, double *slab, const PatchDev *patches,
                              const PatchTimeDev *times, const GhostItemDev *items, int first,
                              int count, int pid, const int *group_active) {
  k_fill_patch<<<1, 128, 0, st>>>(slab, patches, times, items, first, count, pid, group_active);
  return cudaGetLastError();
}

cudaError_t sweep_occupancy(int *blocks_per_sm) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_sweep_tiles, kSweepThreads, 0);
}

size_t solve_patch_smem(int nx, int ny) { return sizeof(double) * 3 * (size_t)nx * ny; }

cudaError_t prepare_solve_patch(size_t max_dynamic_smem) {
  return cudaFuncSetAttribute(k_solve_patch, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)max_dynamic_smem);
}

cudaError_t launch_solve_patch(cudaStream_t st, double *slab, const PatchDev *patches,
                               PatchTimeDev *times, int pid, int nx, int ny,
                               const SweParamsDev &prm, double max_dt, double *out) {
  k_solve_patch<<<1, kSweepThreads, solve_patch_smem(nx, ny), st>>>(slab, patches, times, pid, prm,
                                                                    max_dt, out);
  return cudaGetLastError();
}

cudaError_t launch_copy_unew_to_uold(cudaStream_t st, double *slab, const PatchDev *patches, int pid,
                                     int n) {
  k_copy_unew_to_uold<<<(n + 255) / 256, 256, 0, st>>>(slab, patches, pid);
  return cudaGetLastError();
}

cudaError_t launch_swap_unew_uold(cudaStream_t st, double *slab, const PatchDev *patches, int pid, int n) {
  k_swap_unew_uold<<<(n + 255) / 256, 256, 0, st>>>(slab, patches, pid);
  return cudaGetLastError();
}

cudaError_t launch_fill_boundary_layer(cudaStream_t st, double *slab, const PatchDev *patches,
                                       int pid, int dim, int up) {
  k_fill_boundary_layer<<<1, 128, 0, st>>>(slab, patches, pid, dim, up);
  return cudaGetLastError();
}

cudaError_t launch_transfer(cudaStream_t st, double *slab, const PatchDev *patches,
                            const PatchTimeDev *times, const GhostItemDev &it) {
  int n = it.size[0] * it.size[1];
  k_transfer<<<(n + 127) / 128, 128, 0, st>>>(slab, patches, times, it);
  return cudaGetLastError();
}

// Interpolations of several (source, destination) items with distinct
// destinations: one CTA per item, the cells of k_interpolate.
__global__ void k_interpolate_many(double *slab, const PatchDev *patches, const PatchTimeDev *times,
                                   const GhostItemDev *items, int to_uold, int to_current, int use_unew_uold,
                                   int swe) {
  const GhostItemDev it = items[blockIdx.x];
  const PatchDev S = patches[it.src], D = patches[it.dst];
  const double tf = interp_tf(S, times[it.src], D, times[it.dst], to_current != 0, use_unew_uold != 0);
  const int ncell = it.size[0] * it.size[1];
  for (int k = threadIdx.x; k < ncell; k += blockDim.x)
    interp_cell(slab, S, D, it.size, it.dst_off, tf, to_uold != 0, swe != 0, k);
}

cudaError_t launch_interpolate_many(cudaStream_t st, double *slab, const PatchDev *patches,
                                    const PatchTimeDev *times, const GhostItemDev *items, int n, int to_uold,
                                    int to_current, int use_unew_uold, int swe) {
  if (n <= 0) return cudaSuccess;
  k_interpolate_many<<<n, 256, 0, st>>>(slab, patches, times, items, to_uold, to_current, use_unew_uold, swe);
  return cudaGetLastError();
}

// Time records of listed patches.
__global__ void k_scatter_times(const long long *__restrict__ ids, const PatchTimeDev *__restrict__ in, int n,
                                PatchTimeDev *__restrict__ times) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) times[ids[k]] = in[k];
}

cudaError_t launch_scatter_times(cudaStream_t st, const long long *ids, const PatchTimeDev *in, int n,
                                 PatchTimeDev *times) {
  if (n <= 0) return cudaSuccess;
  k_scatter_times<<<(n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024, 256, 0, st>>>(ids, in, n, times);
  return cudaGetLastError();
}

cudaError_t launch_interpolate(cudaStream_t st, double *slab, const PatchDev *patches,
                               const PatchTimeDev *times, const GhostItemDev &it, int to_uold,
                               int to_current, int use_unew_uold, int swe) {
  int n = it.size[0] * it.size[1];
  k_interpolate<<<(n + 127) / 128, 128, 0, st>>>(slab, patches, times, it, to_uold, to_current,
                                                 use_unew_uold, swe);
  return cudaGetLastError();
}

cudaError_t launch_restrict(cudaStream_t st, double *slab, const PatchDev *patches,
                            const PatchTimeDev *times, int src, int dst, int only_overlapped, int swe) {
  k_restrict<<<1, 256, 0, st>>>(slab, patches, times, src, dst, only_overlapped, swe);
  return cudaGetLastError();
}

cudaError_t launch_post_process_restriction(cudaStream_t st, double *slab, const PatchDev *patches,
                                            const int *ids, int count, const int *group_active,
                                            const int *dirty) {
  if (count <= 0) return cudaSuccess;
  k_post_process_restriction<<<count, 256, 0, st>>>(slab, patches, ids, count, group_active, dirty);
  return cudaGetLastError();
}

cudaError_t launch_compute_fluxes(cudaStream_t st, double *slab, const PatchDev *patches,
                                  const int *ids, int count, double gf, const int *group_active) {
  if (count <= 0) return cudaSuccess;
  k_compute_fluxes<<<count, 128, 0, st>>>(slab, patches, ids, count, gf, group_active);
  return cudaGetLastError();
}

static cudaError_t level_transfer_setup() {
  static bool done = false;
  if (done) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(k_level_transfer, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)kTransferSmem);
  if (e == cudaSuccess) done = true;
  return e;
}

cudaError_t launch_restr_geometry(cudaStream_t st, const PatchDev *patches, const PatchTimeDev *times,
                                  const int4 *items, const int *begin, int n_dst, RestrItemTab *geo,
                                  int *geo_bad) {
  if (n_dst <= 0) return cudaSuccess;
  k_restr_geometry<<<n_dst, 128, 0, st>>>(patches, times, items, begin, n_dst, geo, geo_bad);
  return cudaGetLastError();
}

int level_transfer_grid(int num_sms, int n_leaf, int n_flux, int n_restr) {
  const int items = (n_leaf + kTransferLeaves - 1) / kTransferLeaves + n_flux + n_restr;
  if (items <= 0) return 0;
  if (level_transfer_setup() != cudaSuccess) return 0;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_level_transfer, kTransferThreads, kTransferSmem) !=
          cudaSuccess ||
      per_sm < 1)
    per_sm = 1;
  const int cap = (num_sms > 0 ? num_sms : 1) * per_sm;
  return items < cap ? items : cap;
}

cudaError_t launch_level_transfer(cudaStream_t st, int grid, double *slab, const PatchDev *patches,
                                  const PatchTimeDev *times, const int *leaf_ids, int n_leaf, double gf,
                                  const int4 *flux_items, const int *flux_begin, int n_flux,
                                  const int4 *restr_items, const int *restr_begin,
                                  const RestrItemTab *restr_geo, const int *restr_geo_bad,
                                  const int2 *restr_chunks, int n_restr, const int *group_active,
                                  const int *pact, TransferCtl *ctl, int wait_bias) {
  if (grid <= 0) return cudaSuccess;
  cudaError_t e = level_transfer_setup();
  if (e != cudaSuccess) return e;
  k_level_transfer<<<grid, kTransferThreads, kTransferSmem, st>>>(slab, patches, times, leaf_ids, n_leaf, gf, flux_items,
                                                      flux_begin, n_flux, restr_items, restr_begin, restr_geo,
                                                      restr_geo_bad, restr_chunks, n_restr, group_active, pact,
                                                      wait_bias, ctl);
  return cudaGetLastError();
}

// The flat ghost-cell list: block b writes the cells of item exp[b].x, the
// (item, cell) pairs [exp[b].y, exp[b + 1].y) of the list.
__global__ void k_expand_gcells(const int2 *__restrict__ exp, GhostCellDev *__restrict__ out) {
  const int2 e = exp[blockIdx.x];
  const int count = exp[blockIdx.x + 1].y - e.y;
  for (int q = threadIdx.x; q < count; q += blockDim.x) out[e.y + q] = GhostCellDev{e.x, q};
}

cudaError_t launch_expand_gcells(cudaStream_t st, const int2 *exp, int n_items, GhostCellDev *out) {
  if (n_items <= 0) return cudaSuccess;
  k_expand_gcells<<<n_items, 64, 0, st>>>(exp, out);
  return cudaGetLastError();
}

cudaError_t launch_scan_fin(cudaStream_t st, const double *slab, const PatchDev *patches, int count,
                            int *fin) {
  if (count <= 0) return cudaSuccess;
  k_scan_fin<<<count, 128, 0, st>>>(slab, patches, count, fin);
  return cudaGetLastError();
}

cudaError_t launch_gather_cells(cudaStream_t st, const double *slab, const PatchDev *patches,
                                const int *ids, const long long *out_off, int count, double *out) {
  if (count <= 0) return cudaSuccess;
  k_gather_cells<<<count, 256, 0, st>>>(slab, patches, ids, out_off, count, out);
  return cudaGetLastError();
}

cudaError_t launch_switch_to_leaf(cudaStream_t st, double *slab, const PatchDev *patches,
                                  const PatchTimeDev *times, int pid) {
  k_switch_to_leaf<<<1, 256, 0, st>>>(slab, patches, times, pid);
  return cudaGetLastError();
}

cudaError_t launch_refinement_indicator(cudaStream_t st, const double *slab, const PatchDev *patches,
                                        const int *ids, int count, int kind, double *out) {
  if (count <= 0) return cudaSuccess;
  k_refinement_indicator<<<count, 256, 0, st>>>(slab, patches, ids, count, kind, out);
  return cudaGetLastError();
}

cudaError_t launch_clear_interior(cudaStream_t st, double *slab, const PatchDev *patches,
                                  const int *ids, int count, const int *group_active, const int *dirty) {
  if (count <= 0) return cudaSuccess;
  k_clear_interior<<<count, 256, 0, st>>>(slab, patches, ids, count, group_active, dirty);
  return cudaGetLastError();
}

cudaError_t launch_flux_correction(cudaStream_t st, double *slab, const PatchDev *patches,
                                   const PatchTimeDev *times, int src, int dst, int dim, int dir) {
  k_flux_correction<<<1, 32, 0, st>>>(slab, patches, times, src, dst, dim, dir);
  return cudaGetLastError();
}

}  // namespace pcg

// ===========================================================================
// Allocation-free single-patch solve (pcg_solve_timestep_noalloc).
//
// Some callers cannot call cudaMalloc: a traversal thread that works on a
// patch buffer owned by someone else and must not trigger the device-wide
// synchronisation of an allocation, or a process whose device memory is held
// by another framework's pool, so that a new allocation can fail at any time.
// They also cannot create a pcg_context, whose slab is allocated.  For them
// the solve below keeps its scratch (the net updates of one patch and the two
// result words) in a fixed array that is part of the library image.
// ===========================================================================

namespace pcg {

// Largest patch (interior cells) the allocation-free solve accepts: 128 x 128.
constexpr int kNoAllocMaxCells = 128 * 128;

// 3 net-update fields of up to kNoAllocMaxCells cells + {dt used, next dt}:
// 393,232 bytes that every GPU which loads this library holds until exit.
// All calls share it and it keeps the last call's contents; every element a
// call reads was written earlier by the same call, so nothing needs clearing.
// Calls whose kernels overlap on the GPU (different streams, no ordering)
// race on this array.
static __device__ __align__(256) double g_noalloc_scratch[3 * kNoAllocMaxCells + 2];

__global__ void __launch_bounds__(kSweepThreads)
    k_solve_patch_noalloc(double *__restrict__ vec, PatchDev P, SweParamsDev prm, double max_dt,
                          double *__restrict__ scratch) {
  __shared__ SweepSmem S;
  const int nx = P.nx, ny = P.ny;
  double *net = scratch;
  double smax = 0.0;
  for (int x0 = 0; x0 < nx; x0 += kTile)
    for (int y0 = 0; y0 < ny; y0 += kTile) {
      int tw = min(kTile, nx - x0), th = min(kTile, ny - y0);
      double nh = 0, nhu = 0, nhv = 0;
      double s = sweep_tile(S, vec, P, prm, x0, y0, tw, th, false, nh, nhu, nhv);
      smax = fmax(smax, s);
      int t = threadIdx.x;
      if (t < tw * th) {
        int x = x0 + t / th, y = y0 + t % th;
        long long c = (long long)x * ny + y;
        net[c] = nh;
        net[(long long)nx * ny + c] = nhu;
        net[2LL * nx * ny + c] = nhv;
      }
    }
  __syncthreads();
  double dx = subcell(P, 0), dy = subcell(P, 1);
  double block_dt = cfl_dt(prm, smax, dx, dy);
  double dt = fmin(block_dt, max_dt);
  for (int c = threadIdx.x; c < nx * ny; c += blockDim.x) {
    int x = c / ny, y = c - x * ny;
    long long io0 = idx_uold(P, 0, x, y), io1 = idx_uold(P, 1, x, y), io2 = idx_uold(P, 2, x, y);
    long long in0 = idx_unew(P, 0, x, y), in1 = idx_unew(P, 1, x, y), in2 = idx_unew(P, 2, x, y);
    double nh = __fma_rn(-dt, net[c], vec[io0]);
    double nhu = __fma_rn(-dt, net[(long long)nx * ny + c], vec[io1]);
    double nhv = __fma_rn(-dt, net[2LL * nx * ny + c], vec[io2]);
    if (lt_ieee(nh, prm.dry_tol_update)) { nhu = 0.0; nhv = 0.0; }
    if (lt_zero(nh)) nh = 0.0;
    double o0 = vec[in0], o1 = vec[in1], o2 = vec[in2];
    vec[io0] = o0; vec[io1] = o1; vec[io2] = o2;
    vec[in0] = nh; vec[in1] = nhu; vec[in2] = nhv;
  }
  if (threadIdx.x == 0) {
    scratch[3 * kNoAllocMaxCells] = dt;
    scratch[3 * kNoAllocMaxCells + 1] = block_dt;
  }
}

}  // namespace pcg

#include <cuda.h>

#include <mutex>

#include "../../include/pcg.h"

namespace {
std::mutex g_noalloc_mu;
constexpr int kNoAllocMaxDevices = 64;
// Device address of the scratch array per device ordinal, valid for the
// context whose id is stored beside it: a context that was destroyed and
// created again (cudaDeviceReset, or a framework that resets the device)
// loads the library's module again, possibly at another address.
struct NoAllocScratchAddr {
  unsigned long long ctx_id;
  double *ptr;
};
NoAllocScratchAddr g_noalloc_addr[kNoAllocMaxDevices] = {};

// cuCtxGetCurrent / cuCtxGetId through the runtime's driver entry points (the
// library does not link the driver library itself, so that it still loads on
// machines without a GPU driver).
typedef CUresult (*CtxGetCurrentFn)(CUcontext *);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long *);

// Id of the calling thread's current context, 0 if there is none yet.
cudaError_t current_context_id(unsigned long long *id) {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  if (!get_current || !get_id) {
    cudaDriverEntryPointQueryResult q1, q2;
    void *f1 = nullptr, *f2 = nullptr;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1);
    if (e == cudaSuccess)
      e = cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2);
    if (e != cudaSuccess) return e;
    if (q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
      return cudaErrorSymbolNotFound;
    get_current = (CtxGetCurrentFn)f1;
    get_id = (CtxGetIdFn)f2;
  }
  CUcontext ctx = nullptr;
  if (get_current(&ctx) != CUDA_SUCCESS) return cudaErrorContextIsDestroyed;
  *id = 0;
  if (ctx && get_id(ctx, id) != CUDA_SUCCESS) return cudaErrorContextIsDestroyed;
  return cudaSuccess;
}
}  // namespace

extern "C" int pcg_solve_timestep_noalloc(double *d_vector, int32_t nx, int32_t ny,
                                          const double size[2], const pcg_swe_params *params,
                                          double max_dt, double *dt_used, double *est_next,
                                          void *stream) {
  using namespace pcg;
  if (!d_vector || !size || !params)
    return pcg_report_error(PCG_E_INVALID, "pcg_solve_timestep_noalloc: null argument");
  if (nx < 1 || ny < 1 || (long long)nx * ny > kNoAllocMaxCells)
    return pcg_report_error(PCG_E_INVALID,
                            "pcg_solve_timestep_noalloc: patch must have 1..16384 (128 x 128) cells");
  if (!(size[0] > 0.0) || !(size[1] > 0.0))
    return pcg_report_error(PCG_E_INVALID, "pcg_solve_timestep_noalloc: patch size must be positive");
  if (((uintptr_t)d_vector & 7u) != 0)
    return pcg_report_error(PCG_E_INVALID, "pcg_solve_timestep_noalloc: vector must be 8-byte aligned");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return pcg_report_error(PCG_E_CUDA, cudaGetErrorString(e));
  if (dev < 0 || dev >= kNoAllocMaxDevices)
    return pcg_report_error(PCG_E_INVALID, "pcg_solve_timestep_noalloc: device ordinal too large");
  cudaStream_t st = (cudaStream_t)stream;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  e = cudaStreamIsCapturing(st, &cap);
  if (e != cudaSuccess) return pcg_report_error(PCG_E_CUDA, cudaGetErrorString(e));
  const bool capturing = cap != cudaStreamCaptureStatusNone;
  // dt_used / est_next are read back with a copy and a stream synchronisation,
  // neither of which a stream under capture allows
  if (capturing && (dt_used || est_next))
    return pcg_report_error(PCG_E_INVALID,
                            "pcg_solve_timestep_noalloc: dt_used and est_next must be NULL while the "
                            "stream is being captured");
  double *scratch;
  {
    // First call on a device (or in a new context of it): resolve the device
    // address of the scratch array with that device current (the host-side
    // name is not a device address).
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    unsigned long long id = 0;
    e = current_context_id(&id);
    if (e != cudaSuccess)
      return pcg_report_error(PCG_E_CUDA, std::string("current context: ") + cudaGetErrorString(e));
    NoAllocScratchAddr &A = g_noalloc_addr[dev];
    if (id == 0 || !A.ptr || A.ctx_id != id) {
      if (capturing)
        return pcg_report_error(PCG_E_STATE,
                                "pcg_solve_timestep_noalloc: the first call in a device context must "
                                "come before any stream capture");
      double *p = nullptr;
      e = cudaGetSymbolAddress((void **)&p, g_noalloc_scratch);
      if (e != cudaSuccess || !p)
        return pcg_report_error(PCG_E_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      // the context exists now (the call above initialises it if needed)
      e = current_context_id(&id);
      if (e != cudaSuccess || id == 0)
        return pcg_report_error(PCG_E_CUDA, std::string("current context: ") + cudaGetErrorString(e));
      A.ptr = p;
      A.ctx_id = id;
    }
    scratch = A.ptr;
  }
  PatchDev P{};
  P.off = 0;
  P.nx = nx; P.ny = ny; P.g = 1; P.nq = 3; P.np_wo = 0; P.np_w = 1;
  P.flags = kFlagLeaf;
  P.size[0] = size[0]; P.size[1] = size[1];
  SweParamsDev prm{params->g, params->cfl, params->dry_tol, params->dry_tol_update, params->s_min,
                   params->dt_inf};
  k_solve_patch_noalloc<<<1, kSweepThreads, 0, st>>>(d_vector, P, prm, max_dt, scratch);
  e = cudaGetLastError();
  if (e != cudaSuccess) return pcg_report_error(PCG_E_CUDA, cudaGetErrorString(e));
  if (dt_used || est_next) {
    double res[2];
    e = cudaMemcpyAsync(res, scratch + 3 * kNoAllocMaxCells, sizeof(res), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return pcg_report_error(PCG_E_CUDA, cudaGetErrorString(e));
    if (dt_used) *dt_used = res[0];
    if (est_next) *est_next = res[1];
  }
  return PCG_OK;
}
