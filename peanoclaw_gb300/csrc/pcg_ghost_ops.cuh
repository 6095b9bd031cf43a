// pcg_ghost_ops.cuh -- ghost-layer device functions shared by the batched
// ghost fill (pcg_kernels.cu) and the pipelined step (pcg_pipeline.cu):
// time factors of DefaultTransfer / DefaultInterpolation, one ghost cell of
// the flat ghost-cell list, one wall face of SWEKernel::fillBoundaryLayer.
// kL2 reads patch data through L2 only (ldd / ldi).
#pragma once
#include "pcg_device.cuh"

namespace pcg {

__device__ __forceinline__ double transfer_tf(const PatchDev &S, const PatchTimeDev &ST,
                                              const PatchDev &D, const PatchTimeDev &DT) {
  double dtu = time_unew(D, DT);
  if (is_virtual(S)) return ieee::div_rn(__dsub_rn(dtu, 0.0), 1.0);
  double su = time_unew(S, ST), so = time_uold(S, ST);
  if (tl_greater(__dsub_rn(su, so), 0.0)) return ieee::div_rn(__dsub_rn(dtu, so), __dsub_rn(su, so));
  return 1.0;
}

__device__ __forceinline__ double interp_tf(const PatchDev &S, const PatchTimeDev &ST,
                                            const PatchDev &D, const PatchTimeDev &DT,
                                            bool to_current, bool use_unew_uold) {
  double tf;
  if (tl_equals(ST.dt, 0.0)) {
    tf = 1.0;
  } else if (use_unew_uold) {
    double so = time_uold(S, ST), su = time_unew(S, ST);
    double num = to_current ? __dsub_rn(time_uold(D, DT), so) : __dsub_rn(time_unew(D, DT), so);
    tf = ieee::div_rn(num, __dsub_rn(su, so));
  } else {
    double den = __dsub_rn(__dadd_rn(ST.time, ST.dt), ST.time);
    double num = to_current ? __dsub_rn(DT.time, ST.time)
                            : __dsub_rn(__dadd_rn(DT.time, DT.dt), ST.time);
    tf = ieee::div_rn(num, den);
  }
  return fmax(0.0, fmin(1.0, tf));
}

// Per-step data of ghost item i: its time factor (and 1 - tf) from the two
// patches' time intervals, and the unknown strides.
__device__ __forceinline__ GhostItemStepDev item_step_value(const PatchDev *__restrict__ patches,
                                                            const PatchTimeDev *__restrict__ times,
                                                            const GhostItemDev *__restrict__ items, int i) {
  const GhostItemDev it = items[i];
  const PatchDev &S = patches[it.src], &D = patches[it.dst];
  const PatchTimeDev &ST = times[it.src], &DT = times[it.dst];
  GhostItemStepDev r;
  r.tf = it.kind == 0 ? transfer_tf(S, ST, D, DT) : interp_tf(S, ST, D, DT, false, true);
  r.itf = __dsub_rn(1.0, r.tf);
  r.vn_src = (int)vol_new(S);
  r.vo_src = (int)vol_old(S);
  r.vo_dst = (int)vol_old(D);
  r.nq = it.kind == 0 ? S.nq : (D.nq < 3 ? D.nq : 3);
  return r;
}

// Ghost cell e of the flat list: entries [0, ncopy) copy (DefaultTransfer's
// time-interpolated copy, offsets from the copy plan), the others interpolate
// with their precomputed d-linear plan (SWE interpolation with the h+b wrap).
// step(item) gives the item's per-step data.
template <bool kL2, class StepFn>
__device__ __forceinline__ void ghost_entry(double *__restrict__ slab, const PatchDev *__restrict__ patches,
                                            const GhostItemDev *__restrict__ items,
                                            const GhostCellDev *__restrict__ cells, int ncopy,
                                            const CopyPlanDev *__restrict__ copy_plan,
                                            const InterpPlanDev *__restrict__ plan, StepFn step, int e,
                                            const int *__restrict__ group_active, const int *__restrict__ fin,
                                            const int *__restrict__ pact) {
  if (e < ncopy) {
    const CopyPlanDev pl = copy_plan[e];
    if (group_active && !group_active[patches[pl.dst_pid].group]) return;
    if (pact && !pact[pl.dst_pid]) return;
    const GhostItemStepDev I = step(pl.item);
    double vn[3], vo[3];
    const int nq = I.nq < 3 ? I.nq : 3;
#pragma unroll
    for (int q = 0; q < 3; q++) {
      if (q < nq) {
        vn[q] = ldd<kL2>(slab + pl.src_new + (long long)q * I.vn_src);
        vo[q] = ldd<kL2>(slab + pl.src_old + (long long)q * I.vo_src);
      }
    }
#pragma unroll
    for (int q = 0; q < 3; q++)
      if (q < nq)
        slab[pl.dst + (long long)q * I.vo_dst] = __dadd_rn(__dmul_rn(vn[q], I.tf), __dmul_rn(vo[q], I.itf));
    for (int q = 3; q < I.nq; q++)  // more than three unknowns (not the SWE case)
      slab[pl.dst + (long long)q * I.vo_dst] =
          __dadd_rn(__dmul_rn(ldd<kL2>(slab + pl.src_new + (long long)q * I.vn_src), I.tf),
                    __dmul_rn(ldd<kL2>(slab + pl.src_old + (long long)q * I.vo_src), I.itf));
    return;
  }
  const GhostCellDev gc = cells[e];
  const GhostItemDev it = items[gc.item];
  const PatchDev S = patches[it.src], D = patches[it.dst];
  if (group_active && !group_active[D.group]) return;
  if (pact && !pact[it.dst]) return;
  const InterpPlanDev pl = plan[e - ncopy];
  const GhostItemStepDev I = step(gc.item);
  const double tf = I.tf, one_m_tf = I.itf;
  int cx = it.dst_off[0] + gc.k / it.size[1], cy = it.dst_off[1] + gc.k % it.size[1];
  double acc[3];
  const int nq = I.nq;
  for (int q = 0; q < nq; q++) acc[q] = 0.0;
  // time factor 1 with a leaf source whose uOld and b interior are below
  // 2^1022: (uOld [+ b]) * 0 + (uNew [+ b]) * 1 is exactly uNew [+ b] up to
  // the sign of a zero, which the accumulator (started at +0, never -0)
  // absorbs, so uOld is not needed
  if (fin && dbits(tf) == 0x3FF0000000000000ull && is_leaf(S) &&
      (ldi<kL2>(fin + it.src) & (kFinUOld | kFinB)) == (kFinUOld | kFinB)) {
    if (nq == 3) {
      // the SWE case: all 16 source values and the destination's b loaded
      // before the sums (in registers), then the same sums in the same order
      double h[4], hu[4], hv[4], bb[4];
#pragma unroll
      for (int kk = 0; kk < 4; kk++) {
        const int nxi = pl.bx + (kk & 1), nyi = pl.by + ((kk >> 1) & 1);
        bb[kk] = slab[idx_pw(S, 0, nxi, nyi)];
        h[kk] = ldd<kL2>(slab + idx_unew(S, 0, nxi, nyi));
        hu[kk] = ldd<kL2>(slab + idx_unew(S, 1, nxi, nyi));
        hv[kk] = ldd<kL2>(slab + idx_unew(S, 2, nxi, nyi));
      }
      const double bd = slab[idx_pw(D, 0, cx, cy)];
      double a0 = 0.0, a1 = 0.0, a2 = 0.0;
#pragma unroll
      for (int kk = 0; kk < 4; kk++) {
        const double sf = pl.sf[kk];
        a0 = __dadd_rn(a0, __dmul_rn(sf, __dadd_rn(h[kk], bb[kk])));
        a1 = __dadd_rn(a1, __dmul_rn(sf, hu[kk]));
        a2 = __dadd_rn(a2, __dmul_rn(sf, hv[kk]));
      }
      a0 = __dadd_rn(a0, __dmul_rn(-1.0, bd));
      slab[idx_uold(D, 0, cx, cy)] = a0;
      slab[idx_uold(D, 1, cx, cy)] = a1;
      slab[idx_uold(D, 2, cx, cy)] = a2;
      return;
    }
    for (int kk = 0; kk < 4; kk++) {
      const int nxi = pl.bx + (kk & 1), nyi = pl.by + ((kk >> 1) & 1);
      const double sf = pl.sf[kk];
      const double bb = slab[idx_pw(S, 0, nxi, nyi)];
      acc[0] = __dadd_rn(acc[0], __dmul_rn(sf, __dadd_rn(ldd<kL2>(slab + idx_unew(S, 0, nxi, nyi)), bb)));
      for (int q = 1; q < nq; q++) acc[q] = __dadd_rn(acc[q], __dmul_rn(sf, ldd<kL2>(slab + idx_unew(S, q, nxi, nyi))));
    }
    acc[0] = __dadd_rn(acc[0], __dmul_rn(-1.0, slab[idx_pw(D, 0, cx, cy)]));
    for (int q = 0; q < nq; q++) slab[idx_uold(D, q, cx, cy)] = acc[q];
    return;
  }
  for (int kk = 0; kk < 4; kk++) {
    int nxi = pl.bx + (kk & 1), nyi = pl.by + ((kk >> 1) & 1);
    double sf = pl.sf[kk];
    for (int q = 0; q < nq; q++) {
      double so = ldd<kL2>(slab + idx_uold(S, q, nxi, nyi));
      double sn = ldd<kL2>(slab + idx_unew(S, q, nxi, nyi));
      if (q == 0) {
        double bb = slab[idx_pw(S, 0, nxi, nyi)];
        so = __dadd_rn(so, bb);
        sn = __dadd_rn(sn, bb);
      }
      acc[q] = __dadd_rn(acc[q], __dmul_rn(sf, __dadd_rn(__dmul_rn(so, one_m_tf), __dmul_rn(sn, tf))));
    }
  }
  acc[0] = __dadd_rn(acc[0], __dmul_rn(-1.0, slab[idx_pw(D, 0, cx, cy)]));
  for (int q = 0; q < nq; q++) slab[idx_uold(D, q, cx, cy)] = acc[q];
}

// SWEKernel::fillBoundaryLayer for one face; reads interior cells from uNew
// when `interior_from_unew` (the copy uNew -> uOld of SolveTimestep is implicit
// in the batched form), ghost cells from uOld.
template <bool kL2>
__device__ __forceinline__ void wall_face(double *slab, const PatchDev &P, int dim, int up,
                                          bool interior_from_unew, int lane, int nl) {
  if (dim == 0) {
    int xi = up ? P.nx : -1;
    int sx = xi + (up ? -1 : 1);
    for (int k = lane; k < (P.ny + 2) * P.nq; k += nl) {
      int yi = k / P.nq - 1, q = k % P.nq;
      bool inside = yi >= 0 && yi < P.ny;
      double v = (interior_from_unew && inside) ? ldd<kL2>(slab + idx_unew(P, q, sx, yi)) : ldd<kL2>(slab + idx_uold(P, q, sx, yi));
      slab[idx_uold(P, q, xi, yi)] = (q == dim + 1) ? -v : v;
    }
  } else {
    int yi = up ? P.ny : -1;
    int sy = yi + (up ? -1 : 1);
    for (int k = lane; k < (P.nx + 2) * P.nq; k += nl) {
      int xi = k / P.nq - 1, q = k % P.nq;
      bool inside = xi >= 0 && xi < P.nx;
      double v = (interior_from_unew && inside) ? ldd<kL2>(slab + idx_unew(P, q, xi, sy)) : ldd<kL2>(slab + idx_uold(P, q, xi, sy));
      slab[idx_uold(P, q, xi, yi)] = (q == dim + 1) ? -v : v;
    }
  }
}

}  // namespace pcg
