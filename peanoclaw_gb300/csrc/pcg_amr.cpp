// pcg_amr.cpp -- host-side list builder of adaptive grids (pcg_amr_layout).
//
// For a hierarchy of n x n patches with 3x refinement (level l has
// (base * 3^l)^2 slots on [0,1]^2) this derives, per grid change, what the
// Peano traversal derives per grid iteration: the ghost face-pair list
// (same-level copies, coarse-to-fine interpolation from the nearest existing
// coarser slot; GhostlayerCompositorFunctors.cpp:23-148), the flux-correction
// list (fine leaf faces against a coarser owner), the neighbouring
// ghost-layer bounds of the virtual patches
// (GhostLayerCompositor::updateLower/UpperGhostlayerBound) and the
// restriction list (GridLevelTransfer::restrictToOverlappingVirtualSubgrids,
// a leaf against every virtual ancestor whose bounds it overlaps).
#include <algorithm>
#include <cfloat>
#include <cstdint>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/pcg.h"

int pcg_report_error(int code, const std::string &msg);

namespace {

inline int64_t slot_key(int l, int i, int j) {
  return ((int64_t)l << 52) | ((int64_t)(uint32_t)i << 26) | (int64_t)(uint32_t)j;
}

}  // namespace

extern "C" int pcg_amr_layout(int32_t base, int32_t n, int32_t levels, int32_t np, const int32_t *lvl,
                              const int32_t *si, const int32_t *sj, const uint8_t *refined,
                              int32_t *items, int32_t *n_items, int32_t *flux, int32_t *n_flux,
                              int32_t *restr, int32_t *n_restr, double *lower, double *upper,
                              int32_t *walls) {
  if (base < 1 || n < 1 || levels < 1 || levels > 20 || np < 0 || (np > 0 && (!lvl || !si || !sj || !refined)) ||
      !items || !n_items || !flux || !n_flux || !restr || !n_restr || !lower || !upper || !walls)
    return pcg_report_error(PCG_E_INVALID, "pcg_amr_layout: bad arguments");
  std::vector<int64_t> m(levels);
  int64_t e = base;
  for (int l = 0; l < levels; l++, e *= 3) m[l] = e;
  // slot keys pack i and j into 26 bits each
  if (m[levels - 1] > ((int64_t)1 << 26))
    return pcg_report_error(PCG_E_INVALID, "pcg_amr_layout: more than 2^26 slots per side on the finest level");
  std::unordered_map<int64_t, int32_t> index;
  index.reserve((size_t)np * 2);
  std::vector<double> px(np), py(np), sx(np), sy(np);
  for (int32_t k = 0; k < np; k++) {
    if (lvl[k] < 0 || lvl[k] >= levels || si[k] < 0 || sj[k] < 0 || si[k] >= m[lvl[k]] || sj[k] >= m[lvl[k]])
      return pcg_report_error(PCG_E_INVALID, "pcg_amr_layout: slot out of range");
    index[slot_key(lvl[k], si[k], sj[k])] = k;
    const double L = 1.0 / (double)m[lvl[k]];
    px[k] = (double)si[k] * L;
    py[k] = (double)sj[k] * L;
    sx[k] = L;
    sy[k] = L;
  }
  auto find = [&](int l, int i, int j) -> int32_t {
    auto it = index.find(slot_key(l, i, j));
    return it == index.end() ? -1 : it->second;
  };
  // walls of the leaves on the domain boundary
  for (int32_t k = 0; k < np; k++) {
    int w = 0;
    if (!refined[k]) {
      const int64_t mm = m[lvl[k]];
      if (si[k] == 0) w |= 1;
      if (si[k] == mm - 1) w |= 2;
      if (sj[k] == 0) w |= 4;
      if (sj[k] == mm - 1) w |= 8;
    }
    walls[k] = w;
  }
  // ghost face pairs and flux-correction pairs
  static const int dirs[8][2] = {{-1, 0}, {1, 0}, {0, -1}, {0, 1}, {-1, -1}, {1, -1}, {-1, 1}, {1, 1}};
  int32_t ni = 0, nf = 0;
  for (int32_t d = 0; d < np; d++) {
    if (refined[d]) continue;
    const int l = lvl[d];
    for (const auto &dv : dirs) {
      const int64_t tx = (int64_t)si[d] + dv[0], ty = (int64_t)sj[d] + dv[1];
      if (tx < 0 || tx >= m[l] || ty < 0 || ty >= m[l]) continue;
      int32_t s = -1;
      int ls = l;
      int64_t ox = tx, oy = ty;
      for (; ls >= 0; ls--, ox /= 3, oy /= 3) {
        s = find(ls, (int)ox, (int)oy);
        if (s >= 0) break;
      }
      if (s < 0) continue;
      const int vx = -dv[0], vy = -dv[1];
      const int32_t szx = vx == 0 ? n : 1, szy = vy == 0 ? n : 1;
      const int32_t dox = vx == 0 ? 0 : (vx == 1 ? -1 : n), doy = vy == 0 ? 0 : (vy == 1 ? -1 : n);
      int32_t *row = items + 9 * (size_t)ni++;
      row[1] = s;
      row[2] = d;
      row[3] = szx;
      row[4] = szy;
      row[7] = dox;
      row[8] = doy;
      if (ls == l) {
        row[0] = PCG_GHOST_COPY;
        row[5] = vx == 0 ? 0 : (vx == 1 ? n - 1 : 0);
        row[6] = vy == 0 ? 0 : (vy == 1 ? n - 1 : 0);
      } else {
        row[0] = PCG_GHOST_INTERP;
        row[5] = 0;
        row[6] = 0;
        if (dv[0] == 0 || dv[1] == 0) {
          int32_t *f = flux + 4 * (size_t)nf++;
          f[0] = d;
          f[1] = s;
          f[2] = dv[0] != 0 ? 0 : 1;
          f[3] = dv[0] != 0 ? dv[0] : dv[1];
        }
      }
    }
  }
  *n_items = ni;
  *n_flux = nf;
  // neighbouring ghost-layer bounds of the virtual patches
  for (int32_t v = 0; v < np; v++) {
    lower[2 * v] = lower[2 * v + 1] = DBL_MAX;
    upper[2 * v] = upper[2 * v + 1] = -DBL_MAX;
  }
  for (int32_t v = 0; v < np; v++) {
    if (!refined[v]) continue;
    for (int dim = 0; dim < 2; dim++)
      for (int step = -1; step <= 1; step += 2) {
        const int32_t nb = dim == 0 ? find(lvl[v], si[v] + step, sj[v]) : find(lvl[v], si[v], sj[v] + step);
        if (nb < 0 || refined[nb]) continue;
        const double pos = dim == 0 ? px[nb] : py[nb], size = dim == 0 ? sx[nb] : sy[nb];
        const double sub = size / (double)n;
        if (step < 0)
          upper[2 * v + dim] = std::max(upper[2 * v + dim], pos + size + sub);
        else
          lower[2 * v + dim] = std::min(lower[2 * v + dim], pos - sub);
      }
  }
  // restriction: every leaf against each virtual ancestor it overlaps,
  // ordered by (ancestor, leaf)
  std::vector<std::pair<int32_t, int32_t>> rl;
  for (int32_t s = 0; s < np; s++) {
    if (refined[s]) continue;
    int64_t f = 1;
    for (int l = lvl[s] - 1; l >= 0; l--) {
      f *= 3;
      const int32_t v = find(l, (int)(si[s] / f), (int)(sj[s] / f));
      if (v < 0) continue;
      const double *lo = lower + 2 * v, *up = upper + 2 * v;
      const double ps[2] = {px[s], py[s]}, ss[2] = {sx[s], sy[s]};
      const bool overlapped = (up[0] - ps[0] > 1e-8) || (up[1] - ps[1] > 1e-8) ||
                              (ps[0] + ss[0] - lo[0] > 1e-8) || (ps[1] + ss[1] - lo[1] > 1e-8);
      if (overlapped) rl.push_back({v, s});
    }
  }
  std::sort(rl.begin(), rl.end());
  for (size_t k = 0; k < rl.size(); k++) {
    restr[2 * k] = rl[k].second;
    restr[2 * k + 1] = rl[k].first;
  }
  *n_restr = (int32_t)rl.size();
  return PCG_OK;
}
