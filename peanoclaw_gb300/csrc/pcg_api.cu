// pcg_api.cu -- C ABI (include/pcg.h) of the GB300 SWE patch-update library.
//
// The context owns one HBM slab holding every patch vector (reference
// layout), the patch table, the precomputed face-pair list and the sweep
// work list; host calls only enqueue work on the context's stream.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/pcg.h"
#include "pcg_device.cuh"
#include "pcg_kernels.h"

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string &msg) {
  g_last_error = msg;
  return code;
}

#define PCG_CUDA(call)                                                                     \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess)                                                                 \
      return fail(PCG_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));         \
  } while (0)

__global__ void k_scatter(double *slab, const double *staging, const long long *dst_off,
                          const long long *src_off, const long long *len, int n, int to_slab) {
  for (int i = blockIdx.x; i < n; i += gridDim.x) {
    long long d = dst_off[i], s = src_off[i], l = len[i];
    for (long long k = threadIdx.x; k < l; k += blockDim.x) {
      if (to_slab) slab[d + k] = staging[s + k];
      else ((double *)staging)[s + k] = slab[d + k];
    }
  }
}

// Records every group's dt of a step; with `advance` it also ends the step
// (t += dt for the active groups, as k_group_advance) in the same launch.
__global__ void k_record_hist(int n_groups, const unsigned long long *group_dt, double *hist,
                              int *counter, int capacity, int advance, const int *group_active,
                              double *group_time) {
  __shared__ int idx;
  if (threadIdx.x == 0) idx = *counter;
  __syncthreads();
  if (idx < capacity)
    for (int g = threadIdx.x; g < n_groups; g += blockDim.x)
      hist[(long long)idx * n_groups + g] = __longlong_as_double((long long)group_dt[g]);
  if (advance)
    for (int g = threadIdx.x; g < n_groups; g += blockDim.x)
      if (group_active[g]) group_time[g] = __dadd_rn(group_time[g], __longlong_as_double((long long)group_dt[g]));
  __syncthreads();
  if (threadIdx.x == 0) *counter = idx + 1;
}

// FP64 FMA throughput probe: 8 independent dependent chains per thread.
__global__ void k_fp64_probe(double *out, int iters, double a, double b) {
  double x0 = threadIdx.x * 1e-3, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
  double x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; i++) {
    x0 = __fma_rn(x0, a, b); x1 = __fma_rn(x1, a, b); x2 = __fma_rn(x2, a, b); x3 = __fma_rn(x3, a, b);
    x4 = __fma_rn(x4, a, b); x5 = __fma_rn(x5, a, b); x6 = __fma_rn(x6, a, b); x7 = __fma_rn(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

// Restriction bounds (lower x, y, upper x, y) of listed patches.
__global__ void k_scatter_bounds(const long long *__restrict__ ids, const double *__restrict__ b, int n,
                                 pcg::PatchTimeDev *__restrict__ times) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    pcg::PatchTimeDev &T = times[ids[k]];
    T.rl[0] = b[4 * k]; T.rl[1] = b[4 * k + 1];
    T.ru[0] = b[4 * k + 2]; T.ru[1] = b[4 * k + 3];
  }
}

// Self-check of the integer-pipe divide / square root against the hardware
// IEEE operations on pseudo-random operands (splitmix64 of seed and index).
__device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

__global__ void k_check_ieee(long long n, unsigned long long seed, unsigned long long *bad) {
  using namespace pcg::ieee;
  unsigned long long local = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    uint64_t A = splitmix64(seed ^ (2 * (uint64_t)i)), B = splitmix64(seed ^ (2 * (uint64_t)i + 1));
    switch (i & 7) {
      case 0: break;  // any bit pattern (specials, subnormals included)
      case 1:  // moderate exponents
        A = (A & ~(0x7FFull << 52)) | ((uint64_t)(900 + (A >> 53) % 250) << 52);
        B = (B & ~(0x7FFull << 52)) | ((uint64_t)(900 + (B >> 53) % 250) << 52);
        break;
      case 2: B = (B & ~kFrac) | (B & 63); break;                 // divisor near a power of two
      case 3: B = (B & ~kFrac) | (kFrac - (B & 63)); break;       // divisor mantissa near all ones
      case 4: A = (A & ~kFrac) | (B & kFrac); break;              // equal mantissas
      case 5: A = (A & ~kFrac) | (A & 1023); B = (B & ~kFrac) | (B & 1023); break;
      case 6: A &= ~kSign; A = (A & ~(0x7FFull << 52)) | (1023ull << 52); break;  // [1,2)
      default: A = (A & ~(0x7FFull << 52)) | ((uint64_t)(1010 + (A >> 53) % 30) << 52); break;
    }
    double a = from_bits(A), b = from_bits(B);
    double q1 = div_rn(a, b), q2 = __ddiv_rn(a, b);
    bool qbad = bits(q1) != bits(q2) && !(q1 != q1 && q2 != q2);
    double c1 = rcp_rn(b), c2 = __ddiv_rn(1.0, b);
    bool cbad = bits(c1) != bits(c2) && !(c1 != c1 && c2 != c2);
    double r1 = sqrt_rn(fabs(a)), r2 = __dsqrt_rn(fabs(a));
    bool sbad = bits(r1) != bits(r2) && !(r1 != r1 && r2 != r2);
    local += (qbad ? 1 : 0) + (cbad ? 1 : 0) + (sbad ? 1 : 0);
  }
  if (local) atomicAdd(bad, local);
}

constexpr int64_t kAlign = 32;  // doubles (256 B)

int64_t vector_size(const pcg_patch_desc &d) {
  int64_t vn = (int64_t)d.nx * d.ny, vo = (int64_t)(d.nx + 2 * d.ghost) * (d.ny + 2 * d.ghost);
  return d.nq * vn + d.nq * vo + d.np_wo * vn + d.np_w * vo + 2LL * d.nq * (d.nx + d.ny);
}

}  // namespace

int pcg_report_error(int code, const std::string &msg) { return fail(code, msg); }

struct pcg_context {
  int device = 0;
  int num_sms = 152;
  cudaStream_t stream = nullptr;
  pcg::SweParamsDev prm{};
  std::mutex mu;

  double *slab = nullptr;
  int64_t slab_doubles = 0;
  std::map<int64_t, int64_t> free_list;  // offset -> length

  int max_patches = 0, max_groups = 1;
  int slot_hint = 0;
  int patch_hw = 0;  // ids in use are below this (the patch table uploads [0, patch_hw))
  std::vector<pcg::PatchDev> h_patches;
  std::vector<int64_t> h_len;
  std::vector<char> used;
  pcg::PatchDev *d_patches = nullptr;
  pcg::PatchTimeDev *d_times = nullptr;
  bool patches_dirty = true;
  bool topo_dirty = true;

  unsigned long long *d_patch_smax = nullptr, *d_group_dt = nullptr;
  double *d_group_max_dt = nullptr;
  double *d_group_t_end = nullptr, *d_group_time = nullptr;  // end time (+inf: none), time
  int *d_group_active = nullptr;
  // per patch: bit 0 = uOld interior unknowns all below 2^1022 in magnitude,
  // bit 1 = b interior too (lets the ghost interpolation use uNew alone when
  // the time factor is 1); rescanned when fin_dirty
  int *d_fin = nullptr;
  bool fin_dirty = true;
  // local time stepping (pcg_set_time_stepping): per-patch activity, max dt,
  // dt taken, neighbours' minimal uNew time (order-preserving keys); per
  // group minimal uNew time after the iteration
  bool ts_local = false;
  int *d_pact = nullptr;
  double *d_pmaxdt = nullptr;
  unsigned long long *d_pdt = nullptr, *d_nbmin = nullptr, *d_group_tmin = nullptr;
  // (leaf, virtual) pairs of pcg_set_virtual_time_items and the distinct
  // virtual patches; interval keys per patch
  std::vector<int2> vt_user, h_vt;
  std::vector<int> vt_virtuals;
  int2 *d_vt = nullptr;
  int *d_vt_virtuals = nullptr;
  size_t d_vt_cap = 0, d_vtv_cap = 0;
  unsigned long long *d_vstart = nullptr, *d_vend = nullptr;
  // cells of the leaves advanced by local-time-stepping iterations
  unsigned long long *d_lts_cells = nullptr;
  double *d_dt_out = nullptr;
  double *h_pinned = nullptr;  // pinned scratch for small D2H/H2D
  std::vector<double> h_group_max_dt;

  // face-pair list, sorted by destination for the plain form
  std::vector<pcg_ghost_item> items_user;
  std::vector<pcg::GhostItemDev> h_items;
  std::vector<int> item_first, item_count;  // per patch (plain form)
  pcg::GhostItemDev *d_items = nullptr;
  size_t d_items_cap = 0;
  // flat ghost-cell list of the batched fill (copies first) + interpolation plan
  std::vector<int2> h_gexp;   // (item, first ghost-cell entry) per item with cells, then (-1, total)
  int2 *d_gexp = nullptr;
  size_t d_gexp_cap = 0;
  int64_t n_gcells = 0;
  int n_copy_cells = 0, n_interp_cells = 0;
  pcg::GhostCellDev *d_gcells = nullptr;
  size_t d_gcells_cap = 0;
  pcg::InterpPlanDev *d_plan = nullptr;
  size_t d_plan_cap = 0;
  pcg::CopyPlanDev *d_copy_plan = nullptr;
  size_t d_copy_plan_cap = 0;
  pcg::GhostItemStepDev *d_item_step = nullptr;
  size_t d_item_step_cap = 0;
  // per patch the uOld interior bands the ghost fill reads (int4: x lower,
  // x upper, y lower, y upper) and the strip update's full-write flag: 0
  // inside a batched run but for its last step, else nonzero
  int4 *d_band = nullptr;
  int *d_upd_full = nullptr;

  std::vector<pcg::TileItem> h_tiles;
  pcg::TileItem *d_tiles = nullptr;
  size_t d_tiles_cap = 0;
  std::vector<int> h_wall;
  int *d_wall = nullptr;
  size_t d_wall_cap = 0;
  std::vector<int> leaf_ids;
  int64_t cells_per_step = 0;
  int sweep_grid = 0;

  // batched sweep/update schedule (pcg_schedule); warp-strip work list
  pcg_schedule sched{PCG_SCHED_STRIPS, 2, 32, 0};
  bool sched_fixed = false;          // set by pcg_set_schedule / pcg_autotune
  std::string shape_key;             // SM count + leaf shape histogram
  std::vector<pcg::StripItem> h_sitems;
  std::vector<pcg::StripGroup> h_sgroups;
  pcg::StripItem *d_sitems = nullptr;
  pcg::StripGroup *d_sgroups = nullptr;
  size_t d_sitems_cap = 0, d_sgroups_cap = 0;
  int strip_grid = 0, update_grid = 0;

  double *d_solve_out = nullptr;
  size_t solve_smem_set = 0;

  // restriction / flux-correction phases after the update (AMR)
  std::vector<int4> restr_user, flux_user;
  std::vector<int4> h_restr, h_flux;      // grouped by destination
  std::vector<int> restr_begin, flux_begin, restr_dsts;
  int4 *d_restr = nullptr, *d_flux = nullptr;
  int *d_restr_begin = nullptr, *d_flux_begin = nullptr, *d_restr_dsts = nullptr, *d_leaf_ids = nullptr;
  std::vector<int> flux_leaf_ids;  // leaves of the groups with flux-correction items
  int *d_flux_leaf_ids = nullptr;
  size_t d_fleaf_cap = 0;
  pcg::RestrItemTab *d_restr_geo = nullptr;  // region geometry per restriction item
  int *d_restr_geo_bad = nullptr;            // per destination: item-by-item form
  int2 *d_restr_chunks = nullptr;            // (destination, chunk) work items of the restriction
  std::vector<int2> h_restr_chunks;
  size_t d_rgeo_cap = 0, d_rgeob_cap = 0, d_rch_cap = 0;
  bool restr_geo_dirty = true;               // lists, geometry or restriction bounds changed
  pcg::TileMaps *d_tile_maps = nullptr;  // tensor maps of the TMA tile sweep, per patch id
  size_t d_tmaps_cap = 0;
  bool tma_ok = false;                   // every leaf has a shape the TMA tile staging takes
  bool tile_maps_valid = false;
  pcg::TransferCtl *d_xfer = nullptr;  // work counters and error word of k_level_transfer (and the TMA sweep)
  bool xfer_pending = false;           // a level transfer ran since its error word was read
  size_t d_restr_cap = 0, d_flux_cap = 0, d_rb_cap = 0, d_fb_cap = 0, d_rd_cap = 0, d_leaf_cap = 0;
  double g_flux = 1.0;

  // graph of one batched step
  cudaGraphExec_t graph = nullptr;
  bool graph_valid = false;
  double *d_hist = nullptr;
  int hist_cap = 0;
  int *d_counter = nullptr;

  // staging for multi-patch copies
  double *d_staging = nullptr;
  size_t staging_cap = 0;
  long long *d_copy_meta = nullptr;
  size_t copy_meta_cap = 0;

  // fused batched step (pcg_fused.cu): the step form (pcg_set_step_form);
  // whether the ghost list suits it (leaf sources, ring destinations, copies
  // from interiors); a group may hold a pending update (the reference layout
  // is stale until settle()); the next step's reset and item factors are
  // done; the form of the captured step graph
  int form = PCG_FORM_AUTO;
  bool fused_lists_ok = false;
  bool fused_pending = false;
  bool fused_ready = false;
  bool graph_fused = false;
  int graph_kernels = 0;  // kernel nodes of the captured step graph
  // second state set of every leaf (6 nx ny doubles at PatchDev::sh_off)
  double *d_shadow = nullptr;
  size_t shadow_cap = 0;
  int64_t shadow_need = 0;
  // per group: update pending, set written last, dt of the pending update
  int *d_pend = nullptr, *d_par = nullptr;
  unsigned long long *d_dt_prev = nullptr;
  // face / corner ghost tables and their evaluation plans
  std::vector<int> h_face_begin;
  int *d_face_begin = nullptr, *d_face = nullptr, *d_corner = nullptr;
  size_t d_face_cap = 0;
  pcg::FusedCopyDev *d_fcopies = nullptr;
  size_t d_fcopies_cap = 0;
  pcg::FusedInterpDev *d_finterps = nullptr;
  size_t d_finterps_cap = 0;
  int fused_grid = 0;
  // plain form of the fused step: strips of one patch per item, ranges per patch
  std::vector<pcg::StripItem> h_pitems;
  std::vector<pcg::StripGroup> h_pgroups;
  std::vector<int> pitem_first, pitem_count;
  pcg::StripItem *d_pitems = nullptr;
  pcg::StripGroup *d_pgroups = nullptr;
  size_t d_pitems_cap = 0, d_pgroups_cap = 0;

  // pipelined batched step (pcg_pipeline.cu): its work queue and per-patch
  // counter targets for the current lists and strip items (built when the
  // form first runs after a change), the counters, the control word, and
  // the swept step's dt, activity and max speeds (the updated step's are
  // d_group_dt, d_group_active, d_patch_smax); the form of the captured graph
  bool pipe_valid = false;
  bool graph_pipe = false;
  int n_pipe_queue = 0;
  int pipe_grid = 0;
  unsigned *d_pipe_queue = nullptr;
  size_t d_pipe_queue_cap = 0;
  int *d_pipe_need = nullptr, *d_pipe_cnt = nullptr;
  size_t d_pipe_need_cap = 0, d_pipe_cnt_cap = 0;
  pcg::PipeCtl *d_pipe_ctl = nullptr;
  unsigned long long *d_pipe_dt = nullptr, *d_pipe_smax = nullptr;
  int *d_pipe_active = nullptr;
  size_t d_pipe_dt_cap = 0, d_pipe_smax_cap = 0, d_pipe_active_cap = 0;
  size_t d_pipe_ctl_cap = 0;

  // a run enqueued by pcg_run_async, completed by pcg_run_wait
  bool run_pending = false;
  int32_t run_steps = 0, run_mode = 0;
  bool run_pipe = false;

  int64_t cell_updates = 0;
  double device_ms = 0.0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
};

namespace {

bool valid_id(pcg_context *c, int32_t id) {
  return c && id >= 0 && id < c->max_patches && c->used[id];
}

int slab_alloc(pcg_context *c, int64_t len, int64_t *off) {
  int64_t need = (len + kAlign - 1) / kAlign * kAlign;
  for (auto it = c->free_list.begin(); it != c->free_list.end(); ++it) {
    if (it->second >= need) {
      *off = it->first;
      int64_t rest = it->second - need;
      int64_t noff = it->first + need;
      c->free_list.erase(it);
      if (rest > 0) c->free_list[noff] = rest;
      return PCG_OK;
    }
  }
  return fail(PCG_E_NOMEM, "slab exhausted: patch vector of " + std::to_string(len) + " doubles does not fit");
}

void slab_free(pcg_context *c, int64_t off, int64_t len) {
  int64_t need = (len + kAlign - 1) / kAlign * kAlign;
  auto it = c->free_list.emplace(off, need).first;
  auto nx = std::next(it);
  if (nx != c->free_list.end() && it->first + it->second == nx->first) {
    it->second += nx->second;
    c->free_list.erase(nx);
  }
  if (it != c->free_list.begin()) {
    auto pv = std::prev(it);
    if (pv->first + pv->second == it->first) {
      pv->second += it->second;
      c->free_list.erase(it);
    }
  }
}

template <class T>
int ensure_device(pcg_context *c, T **ptr, size_t *cap, size_t n) {
  if (n <= *cap && *ptr) return PCG_OK;
  if (*ptr) PCG_CUDA(cudaFree(*ptr));
  *ptr = nullptr;
  size_t nc = std::max<size_t>(n, 16);
  PCG_CUDA(cudaMalloc((void **)ptr, nc * sizeof(T)));
  *cap = nc;
  return PCG_OK;
}

int upload_patches(pcg_context *c) {
  if (!c->patches_dirty) return PCG_OK;
  // entries from patch_hw on were never used: zero on the device since the
  // context was created
  if (c->patch_hw > 0)
    PCG_CUDA(cudaMemcpyAsync(c->d_patches, c->h_patches.data(), sizeof(pcg::PatchDev) * (size_t)c->patch_hw,
                             cudaMemcpyHostToDevice, c->stream));
  PCG_CUDA(cudaStreamSynchronize(c->stream));
  c->patches_dirty = false;
  return PCG_OK;
}

// Schedules picked by pcg_autotune, per (SM count, leaf shape histogram).
std::mutex g_tuned_mu;
std::map<std::string, pcg_schedule> g_tuned;

std::string shape_key(pcg_context *c) {
  std::map<std::pair<int, int>, int64_t> hist;
  for (int p : c->leaf_ids) hist[{c->h_patches[p].nx, c->h_patches[p].ny}]++;
  std::string k = "sm" + std::to_string(c->num_sms);
  for (auto &e : hist)
    k += ";" + std::to_string(e.first.first) + "x" + std::to_string(e.first.second) + ":" +
         std::to_string(e.second);
  return k;
}

// Warp-strip work list: every leaf patch is cut into strips of at most 32 rows
// (balanced heights) and `chunk` columns (balanced widths); strips of equal
// (rows, columns) are packed floor(32 / max(rows, columns)) to a warp item.
// Items are ordered by decreasing work so that grid-strided warps get an even
// mix.
void build_strips(pcg_context *c, int chunk) {
  std::map<std::pair<int, int>, std::vector<pcg::StripGroup>> cls;
  for (int p : c->leaf_ids) {
    const pcg::PatchDev &P = c->h_patches[p];
    const int nsy = (P.ny + 31) / 32;
    for (int ky = 0; ky < nsy; ky++) {
      const int y0 = (int)((int64_t)ky * P.ny / nsy), y1 = (int)((int64_t)(ky + 1) * P.ny / nsy);
      const int hs = y1 - y0;
      const int wcap = std::min(chunk, 32 / (32 / hs));
      const int nsx = (P.nx + wcap - 1) / wcap;
      for (int kx = 0; kx < nsx; kx++) {
        const int x0 = (int)((int64_t)kx * P.nx / nsx), x1 = (int)((int64_t)(kx + 1) * P.nx / nsx);
        cls[{hs, x1 - x0}].push_back(pcg::StripGroup{p, (short)x0, (short)y0});
      }
    }
  }
  std::vector<std::pair<int64_t, std::pair<int, int>>> order;
  for (auto &e : cls) {
    const int hs = e.first.first, w = e.first.second;
    const int G = std::max(1, std::min(32 / hs, 32 / w));
    order.push_back({(int64_t)G * hs * w, e.first});
  }
  std::sort(order.begin(), order.end(), [](const auto &a, const auto &b) { return a.first > b.first; });
  c->h_sitems.clear();
  c->h_sgroups.clear();
  for (auto &o : order) {
    const int hs = o.second.first, w = o.second.second;
    const int G = std::max(1, std::min(32 / hs, 32 / w));
    const std::vector<pcg::StripGroup> &gs = cls[o.second];
    for (size_t k = 0; k < gs.size(); k += G) {
      pcg::StripItem it;
      it.g0 = (int)c->h_sgroups.size();
      it.ngroups = (unsigned char)std::min<size_t>(G, gs.size() - k);
      it.hs = (unsigned char)hs;
      it.w = (unsigned char)w;
      it.pad_ = 0;
      for (int g = 0; g < it.ngroups; g++) c->h_sgroups.push_back(gs[k + g]);
      c->h_sitems.push_back(it);
    }
  }
}

// Schedule of a patch mix the autotuner has not seen: small grids (fewer cells
// than 4096 per SM) have more parallelism in 16x16 tiles (one thread per
// cell) than in strips (one warp per strip); larger ones use strips of 8
// warps per CTA with the widest chunk that gives every SM at least one and a
// half times the strip items its resident warps take at once (a last, nearly
// empty wave of items costs a whole item time: on 27² patches one item per
// patch fills 0.6 of the warps, two fill 1.1 waves, three 1.7).
void default_schedule(pcg_context *c) {
  if (c->cells_per_step < (int64_t)c->num_sms * 4096) {
    c->sched = pcg_schedule{PCG_SCHED_TILES, 0, 32, 0};
    return;
  }
  int chunk = 32;
  for (int ch : {32, 16, 10, 8, 4}) {
    chunk = ch;
    build_strips(c, chunk);
    if ((int64_t)c->h_sitems.size() * 2 >= (int64_t)c->num_sms * 16 * 3) break;
  }
  c->sched = pcg_schedule{PCG_SCHED_STRIPS, 2, chunk, 0};
}

// Upload the strip list of the current schedule and size its grids.
int apply_schedule(pcg_context *c) {
  build_strips(c, c->sched.chunk);
  int rc;
  if ((rc = ensure_device(c, &c->d_sitems, &c->d_sitems_cap, c->h_sitems.size())) != PCG_OK) return rc;
  if ((rc = ensure_device(c, &c->d_sgroups, &c->d_sgroups_cap, c->h_sgroups.size())) != PCG_OK) return rc;
  if (!c->h_sitems.empty())
    PCG_CUDA(cudaMemcpyAsync(c->d_sitems, c->h_sitems.data(), sizeof(pcg::StripItem) * c->h_sitems.size(),
                             cudaMemcpyHostToDevice, c->stream));
  if (!c->h_sgroups.empty())
    PCG_CUDA(cudaMemcpyAsync(c->d_sgroups, c->h_sgroups.data(),
                             sizeof(pcg::StripGroup) * c->h_sgroups.size(), cudaMemcpyHostToDevice,
                             c->stream));
  const int v = c->sched.variant;
  int per_sm = 0;
  PCG_CUDA(pcg::strip_occupancy(v, &per_sm));
  if (per_sm < 1) per_sm = 1;
  const int64_t warps = pcg::kStripVariants[v].warps;
  const int64_t need = std::max<int64_t>(1, ((int64_t)c->h_sitems.size() + warps - 1) / warps);
  c->strip_grid = (int)std::min<int64_t>((int64_t)c->num_sms * per_sm, need);
  int upd_sm = 0;
  PCG_CUDA(pcg::update_strips_occupancy(&upd_sm));
  if (upd_sm < 1) upd_sm = 1;
  c->update_grid = (int)std::min<int64_t>((int64_t)c->num_sms * upd_sm,
                                          std::max<int64_t>(1, ((int64_t)c->h_sitems.size() + 7) / 8));
  int fused_sm = 0;
  PCG_CUDA(pcg::fused_occupancy(v, &fused_sm));
  if (fused_sm < 1) fused_sm = 1;
  c->fused_grid = (int)std::min<int64_t>((int64_t)c->num_sms * fused_sm, need);
  int pipe_sm = 0;
  PCG_CUDA(pcg::pipeline_occupancy(v, &pipe_sm));
  if (pipe_sm < 1) pipe_sm = 1;
  c->pipe_grid = c->num_sms * pipe_sm;
  c->pipe_valid = false;
  c->graph_valid = false;
  return PCG_OK;
}

// Strips of one patch per item (the plain form of the fused step: one launch
// per patch), the strip cut of build_strips with 32-column chunks.
void build_patch_strips(pcg_context *c) {
  c->h_pitems.clear();
  c->h_pgroups.clear();
  c->pitem_first.assign(c->max_patches, 0);
  c->pitem_count.assign(c->max_patches, 0);
  for (int p : c->leaf_ids) {
    const pcg::PatchDev &P = c->h_patches[p];
    c->pitem_first[p] = (int)c->h_pitems.size();
    const int nsy = (P.ny + 31) / 32;
    for (int ky = 0; ky < nsy; ky++) {
      const int y0 = (int)((int64_t)ky * P.ny / nsy), y1 = (int)((int64_t)(ky + 1) * P.ny / nsy);
      const int nsx = (P.nx + 31) / 32;
      for (int kx = 0; kx < nsx; kx++) {
        const int x0 = (int)((int64_t)kx * P.nx / nsx), x1 = (int)((int64_t)(kx + 1) * P.nx / nsx);
        pcg::StripItem it;
        it.g0 = (int)c->h_pgroups.size();
        it.ngroups = 1;
        it.hs = (unsigned char)(y1 - y0);
        it.w = (unsigned char)(x1 - x0);
        it.pad_ = 0;
        c->h_pgroups.push_back(pcg::StripGroup{p, (short)x0, (short)y0});
        c->h_pitems.push_back(it);
      }
    }
    c->pitem_count[p] = (int)c->h_pitems.size() - c->pitem_first[p];
  }
}

// Whether the ghost list suits the fused step: every item joins two leaves
// with one ghost layer and three unknowns, writes only ghost-layer cells of
// its destination, and a copy reads only interior cells of its source.
bool fused_lists_fit(pcg_context *c) {
  for (const pcg::GhostItemDev &it : c->h_items) {
    const pcg::PatchDev &S = c->h_patches[it.src], &D = c->h_patches[it.dst];
    if (!(S.flags & pcg::kFlagLeaf) || (S.flags & pcg::kFlagVirtual) || !(D.flags & pcg::kFlagLeaf)) return false;
    if (S.group != D.group) return false;
    if (S.g != 1 || D.g != 1 || S.nq != 3 || D.nq != 3 || S.np_w < 1 || D.np_w < 1) return false;
    if (it.size[0] < 1 || it.size[1] < 1) return false;
    const int x0 = it.dst_off[0], x1 = it.dst_off[0] + it.size[0];
    const int y0 = it.dst_off[1], y1 = it.dst_off[1] + it.size[1];
    if (x0 < -1 || x1 > D.nx + 1 || y0 < -1 || y1 > D.ny + 1) return false;
    const bool x_in = x0 < D.nx && x1 > 0, y_in = y0 < D.ny && y1 > 0;
    if (x_in && y_in) return false;
    if (it.kind == PCG_GHOST_COPY) {
      if (it.src_off[0] < 0 || it.src_off[1] < 0 || it.src_off[0] + it.size[0] > S.nx ||
          it.src_off[1] + it.size[1] > S.ny)
        return false;
    }
  }
  return true;
}

// Face / corner tables of the fused step, the shadow offsets of the leaves
// and the per-patch strip lists (after the ghost-cell list and the
// interpolation plan are on the device).
int build_fused_tables(pcg_context *c) {
  // the fused form applies to the synchronous step without restriction or
  // flux-correction lists: otherwise its tables are not built (a change of
  // the lists, the form or the time stepping rebuilds the topology)
  if (c->form != PCG_FORM_AUTO || c->ts_local || !c->restr_user.empty() || !c->flux_user.empty()) {
    c->fused_lists_ok = false;
    c->shadow_need = 0;
    return PCG_OK;
  }
  c->fused_lists_ok = fused_lists_fit(c);
  c->h_face_begin.assign(c->max_patches, 0);
  int64_t nf = 0, sh = 0;
  for (int p : c->leaf_ids) {
    pcg::PatchDev &P = c->h_patches[p];
    c->h_face_begin[p] = (int)nf;
    P.face_begin = (int)std::min<int64_t>(nf, INT32_MAX);
    nf += 2LL * (P.nx + P.ny);
    P.sh_off = sh;
    sh += (6LL * P.nx * P.ny + kAlign - 1) / kAlign * kAlign;
  }
  if (nf > INT32_MAX) return fail(PCG_E_INVALID, "too many ghost-layer face cells for the fused step");
  c->shadow_need = sh;
  int rc;
  if ((rc = ensure_device(c, &c->d_face, &c->d_face_cap, (size_t)nf)) != PCG_OK) return rc;
  if ((rc = ensure_device(c, &c->d_fcopies, &c->d_fcopies_cap, (size_t)c->n_copy_cells)) != PCG_OK) return rc;
  if ((rc = ensure_device(c, &c->d_finterps, &c->d_finterps_cap, (size_t)c->n_interp_cells)) != PCG_OK) return rc;
  PCG_CUDA(cudaMemcpyAsync(c->d_face_begin, c->h_face_begin.data(), sizeof(int) * c->max_patches,
                           cudaMemcpyHostToDevice, c->stream));
  if (nf) PCG_CUDA(cudaMemsetAsync(c->d_face, 0xFF, sizeof(int) * (size_t)nf, c->stream));
  PCG_CUDA(cudaMemsetAsync(c->d_corner, 0xFF, sizeof(int) * 4 * (size_t)c->max_patches, c->stream));
  if (c->fused_lists_ok)
    PCG_CUDA(pcg::launch_build_fused_ghosts(c->stream, c->d_patches, c->d_items, c->d_gcells, c->n_copy_cells,
                                            c->n_interp_cells, c->d_plan, c->d_face_begin, c->d_face, c->d_corner,
                                            c->d_fcopies, c->d_finterps));
  build_patch_strips(c);
  if ((rc = ensure_device(c, &c->d_pitems, &c->d_pitems_cap, c->h_pitems.size())) != PCG_OK) return rc;
  if ((rc = ensure_device(c, &c->d_pgroups, &c->d_pgroups_cap, c->h_pgroups.size())) != PCG_OK) return rc;
  if (!c->h_pitems.empty())
    PCG_CUDA(cudaMemcpyAsync(c->d_pitems, c->h_pitems.data(), sizeof(pcg::StripItem) * c->h_pitems.size(),
                             cudaMemcpyHostToDevice, c->stream));
  if (!c->h_pgroups.empty())
    PCG_CUDA(cudaMemcpyAsync(c->d_pgroups, c->h_pgroups.data(), sizeof(pcg::StripGroup) * c->h_pgroups.size(),
                             cudaMemcpyHostToDevice, c->stream));
  return PCG_OK;
}

// Rebuild the sweep work list, the wall list and the per-patch item ranges.
int rebuild_topology(pcg_context *c) {
  if (!c->topo_dirty) return upload_patches(c);
  c->h_tiles.clear();
  c->h_wall.clear();
  c->leaf_ids.clear();
  c->tile_maps_valid = false;
  c->cells_per_step = 0;
  for (int p = 0; p < c->patch_hw; p++) {
    pcg::PatchDev &P = c->h_patches[p];
    P.tile_begin = 0;
    P.tile_count = 0;
    if (!c->used[p] || !(P.flags & pcg::kFlagLeaf)) continue;
    c->leaf_ids.push_back(p);
    c->cells_per_step += (int64_t)P.nx * P.ny;
    P.tile_begin = (int)c->h_tiles.size();
    for (int x0 = 0; x0 < P.nx; x0 += pcg::kTile)
      for (int y0 = 0; y0 < P.ny; y0 += pcg::kTile) {
        pcg::TileItem t;
        t.pid = p;
        t.x0 = (short)x0;
        t.y0 = (short)y0;
        t.tw = (short)std::min(pcg::kTile, P.nx - x0);
        t.th = (short)std::min(pcg::kTile, P.ny - y0);
        t.pad_ = 0;
        c->h_tiles.push_back(t);
      }
    P.tile_count = (int)c->h_tiles.size() - P.tile_begin;
    if (P.wall) c->h_wall.push_back(p);
  }
  c->tma_ok = !c->leaf_ids.empty();
  for (int p : c->leaf_ids) c->tma_ok = c->tma_ok && pcg::tma_tile_shape(c->h_patches[p]);
  // items: keep the user's order within each destination (plain form needs
  // per-destination ranges; the batched kernel relies on disjoint writes)
  c->h_items.clear();
  c->item_first.assign(c->max_patches, 0);
  c->item_count.assign(c->max_patches, 0);
  // counting sort of the items by destination (stable: user order within one)
  std::vector<int> dst_start(c->patch_hw + 1, 0), by_dst;
  for (size_t k = 0; k < c->items_user.size(); k++) {
    const pcg_ghost_item &u = c->items_user[k];
    if (valid_id(c, u.src) && valid_id(c, u.dst)) dst_start[u.dst + 1]++;
  }
  for (int p = 0; p < c->patch_hw; p++) dst_start[p + 1] += dst_start[p];
  by_dst.resize(dst_start[c->patch_hw]);
  {
    std::vector<int> fill(dst_start.begin(), dst_start.end() - 1);
    for (size_t k = 0; k < c->items_user.size(); k++) {
      const pcg_ghost_item &u = c->items_user[k];
      if (valid_id(c, u.src) && valid_id(c, u.dst)) by_dst[fill[u.dst]++] = (int)k;
    }
  }
  c->h_items.reserve(by_dst.size());
  for (int p = 0; p < c->patch_hw; p++) {
    c->item_first[p] = (int)c->h_items.size();
    for (int i = dst_start[p]; i < dst_start[p + 1]; i++) {
      const int k = by_dst[i];
      const pcg_ghost_item &u = c->items_user[k];
      pcg::GhostItemDev d;
      d.kind = u.kind; d.src = u.src; d.dst = u.dst;
      d.size[0] = u.size[0]; d.size[1] = u.size[1];
      d.src_off[0] = u.src_offset[0]; d.src_off[1] = u.src_offset[1];
      d.dst_off[0] = u.dst_offset[0]; d.dst_off[1] = u.dst_offset[1];
      c->h_items.push_back(d);
    }
    c->item_count[p] = (int)c->h_items.size() - c->item_first[p];
  }
  // flat ghost-cell list: every cell of every COPY item, then of every INTERP item
  // (expanded on the device from one (item, first entry) pair per item)
  c->h_gexp.clear();
  int64_t ncell = 0;
  for (int pass = 0; pass < 2; pass++) {
    for (size_t k = 0; k < c->h_items.size(); k++) {
      const pcg::GhostItemDev &it = c->h_items[k];
      if (it.kind != pass) continue;
      const int nc = it.size[0] * it.size[1];
      if (nc <= 0) continue;
      c->h_gexp.push_back(make_int2((int)k, (int)ncell));
      ncell += nc;
    }
    if (pass == 0) c->n_copy_cells = (int)ncell;
  }
  if (ncell > INT32_MAX) return fail(PCG_E_INVALID, "too many ghost cells");
  c->h_gexp.push_back(make_int2(-1, (int)ncell));
  c->n_gcells = ncell;
  c->n_interp_cells = (int)ncell - c->n_copy_cells;
  // restriction and flux-correction items grouped by destination, list order kept
  auto group_by_dst = [&](const std::vector<int4> &in, std::vector<int4> &out, std::vector<int> &begin,
                          std::vector<int> *dsts) {
    std::vector<int> order;
    std::map<int, std::vector<int>> by;
    for (size_t k = 0; k < in.size(); k++) {
      if (!valid_id(c, in[k].x) || !valid_id(c, in[k].y)) continue;
      if (!by.count(in[k].y)) order.push_back(in[k].y);
      by[in[k].y].push_back((int)k);
    }
    out.clear();
    begin.assign(1, 0);
    if (dsts) dsts->clear();
    for (int d : order) {
      for (int k : by[d]) out.push_back(in[k]);
      begin.push_back((int)out.size());
      if (dsts) dsts->push_back(d);
    }
  };
  group_by_dst(c->restr_user, c->h_restr, c->restr_begin, &c->restr_dsts);
  group_by_dst(c->flux_user, c->h_flux, c->flux_begin, nullptr);
  // computeFluxes runs for the leaves of the groups (simulations) that have
  // flux correction, so that one group's flux areas do not depend on the
  // lists of the others
  {
    std::vector<char> gflux(c->max_groups, 0);
    for (const int4 &f : c->h_flux) {
      gflux[c->h_patches[f.x].group] = 1;
      gflux[c->h_patches[f.y].group] = 1;
    }
    c->flux_leaf_ids.clear();
    for (int p : c->leaf_ids)
      if (gflux[c->h_patches[p].group]) c->flux_leaf_ids.push_back(p);
  }
  c->h_vt.clear();
  c->vt_virtuals.clear();
  {
    std::vector<char> seen(c->max_patches, 0);
    for (const int2 &pr : c->vt_user) {
      if (!valid_id(c, pr.x) || !valid_id(c, pr.y)) continue;
      c->h_vt.push_back(pr);
      if (!seen[pr.y]) {
        seen[pr.y] = 1;
        c->vt_virtuals.push_back(pr.y);
      }
    }
  }
  int rc;
  if ((rc = ensure_device(c, &c->d_vt, &c->d_vt_cap, c->h_vt.size())) != PCG_OK) return rc;
  if ((rc = ensure_device(c, &c->d_vt_virtuals, &c->d_vtv_cap, c->vt_virtuals.size())) != PCG_OK) return rc;
  if ((rc = ensure_device(c, &c->d_restr, &c->d_restr_cap, c->h_restr.size())) != PCG_OK) return rc;
  if ((rc = ensure_device(c, &c->d_flux, &c->d_flux_cap, c->h_flux.size())) != PCG_OK) return rc;
  if ((rc = ensure_device(c, &c->d_restr_begin, &c->d_rb_cap, c->restr_begin.size())) != PCG_OK) return rc;
  if ((rc = ensure_device(c, &c->d_flux_begin, &c->d_fb_cap, c->flux_begin.size())) != PCG_OK) return rc;
  if ((rc = ensure_device(c, &c->d_restr_dsts, &c->d_rd_cap, c->restr_dsts.size())) != PCG_OK) return rc;
  c->h_restr_chunks.clear();
  for (size_t b = 0; b < c->restr_dsts.size(); b++) {
    const pcg::PatchDev &D = c->h_patches[c->restr_dsts[b]];
    const int n = D.nx * D.ny;
    for (int k = 0; k * pcg::kRestrChunkCells < n; k++) c->h_restr_chunks.push_back(make_int2((int)b, k));
  }
  if ((rc = ensure_device(c, &c->d_restr_chunks, &c->d_rch_cap, c->h_restr_chunks.size())) != PCG_OK) return rc;
  if ((rc = ensure_device(c, &c->d_restr_geo, &c->d_rgeo_cap, c->h_restr.size())) != PCG_OK) return rc;
  if ((rc = ensure_device(c, &c->d_restr_geo_bad, &c->d_rgeob_cap, c->restr_dsts.size())) != PCG_OK) return rc;
  c->restr_geo_dirty = true;
  if ((rc = ensure_device(c, &c->d_leaf_ids, &c->d_leaf_cap, c->leaf_ids.size())) != PCG_OK) return rc;
  if ((rc = ensure_device(c, &c->d_flux_leaf_ids, &c->d_fleaf_cap, c->flux_leaf_ids.size())) != PCG_OK)
    return rc;
  auto up = [&](void *dst, const void *src, size_t bytes) -> cudaError_t {
    return bytes ? cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, c->stream) : cudaSuccess;
  };
  PCG_CUDA(up(c->d_restr, c->h_restr.data(), sizeof(int4) * c->h_restr.size()));
  PCG_CUDA(up(c->d_flux, c->h_flux.data(), sizeof(int4) * c->h_flux.size()));
  PCG_CUDA(up(c->d_restr_begin, c->restr_begin.data(), sizeof(int) * c->restr_begin.size()));
  PCG_CUDA(up(c->d_flux_begin, c->flux_begin.data(), sizeof(int) * c->flux_begin.size()));
  PCG_CUDA(up(c->d_restr_dsts, c->restr_dsts.data(), sizeof(int) * c->restr_dsts.size()));
  PCG_CUDA(up(c->d_restr_chunks, c->h_restr_chunks.data(), sizeof(int2) * c->h_restr_chunks.size()));
  PCG_CUDA(up(c->d_leaf_ids, c->leaf_ids.data(), sizeof(int) * c->leaf_ids.size()));
  PCG_CUDA(up(c->d_flux_leaf_ids, c->flux_leaf_ids.data(), sizeof(int) * c->flux_leaf_ids.size()));
  PCG_CUDA(up(c->d_vt, c->h_vt.data(), sizeof(int2) * c->h_vt.size()));
  PCG_CUDA(up(c->d_vt_virtuals, c->vt_virtuals.data(), sizeof(int) * c->vt_virtuals.size()));
  if ((rc = ensure_device(c, &c->d_gcells, &c->d_gcells_cap, (size_t)c->n_gcells)) != PCG_OK) return rc;
  if ((rc = ensure_device(c, &c->d_gexp, &c->d_gexp_cap, c->h_gexp.size())) != PCG_OK) return rc;
  if ((rc = ensure_device(c, &c->d_plan, &c->d_plan_cap, (size_t)c->n_interp_cells)) != PCG_OK) return rc;
  if ((rc = ensure_device(c, &c->d_copy_plan, &c->d_copy_plan_cap, (size_t)c->n_copy_cells)) != PCG_OK) return rc;
  if ((rc = ensure_device(c, &c->d_item_step, &c->d_item_step_cap, c->h_items.size())) != PCG_OK) return rc;
  if ((rc = ensure_device(c, &c->d_tiles, &c->d_tiles_cap, c->h_tiles.size())) != PCG_OK) return rc;
  if ((rc = ensure_device(c, &c->d_wall, &c->d_wall_cap, c->h_wall.size())) != PCG_OK) return rc;
  if ((rc = ensure_device(c, &c->d_items, &c->d_items_cap, c->h_items.size())) != PCG_OK) return rc;
  if (!c->h_tiles.empty())
    PCG_CUDA(cudaMemcpyAsync(c->d_tiles, c->h_tiles.data(), sizeof(pcg::TileItem) * c->h_tiles.size(),
                             cudaMemcpyHostToDevice, c->stream));
  if (!c->h_wall.empty())
    PCG_CUDA(cudaMemcpyAsync(c->d_wall, c->h_wall.data(), sizeof(int) * c->h_wall.size(),
                             cudaMemcpyHostToDevice, c->stream));
  if (!c->h_items.empty())
    PCG_CUDA(cudaMemcpyAsync(c->d_items, c->h_items.data(), sizeof(pcg::GhostItemDev) * c->h_items.size(),
                             cudaMemcpyHostToDevice, c->stream));
  PCG_CUDA(cudaMemcpyAsync(c->d_gexp, c->h_gexp.data(), sizeof(int2) * c->h_gexp.size(), cudaMemcpyHostToDevice,
                           c->stream));
  PCG_CUDA(pcg::launch_expand_gcells(c->stream, c->d_gexp, (int)c->h_gexp.size() - 1, c->d_gcells));
  c->patches_dirty = true;
  if ((rc = upload_patches(c)) != PCG_OK) return rc;
  PCG_CUDA(pcg::launch_build_interp_plan(c->stream, c->d_patches, c->d_items, c->d_gcells + c->n_copy_cells,
                                         c->n_interp_cells, c->d_plan));
  PCG_CUDA(pcg::launch_build_copy_plan(c->stream, c->d_patches, c->d_items, c->d_gcells, c->n_copy_cells,
                                       c->d_copy_plan));
  PCG_CUDA(cudaMemsetAsync(c->d_band, 0, sizeof(int4) * c->max_patches, c->stream));
  PCG_CUDA(pcg::launch_build_bands(c->stream, c->d_patches, c->d_items, c->d_gcells, c->n_copy_cells,
                                   c->n_interp_cells, c->d_plan, (int *)c->d_band));
  if ((rc = build_fused_tables(c)) != PCG_OK) return rc;
  int per_sm = 0;
  PCG_CUDA(pcg::sweep_occupancy(&per_sm));
  if (per_sm < 1) per_sm = 1;
  c->sweep_grid = (int)std::min<int64_t>((int64_t)c->num_sms * per_sm, std::max<int64_t>(1, (int64_t)c->h_tiles.size()));
  c->shape_key = shape_key(c);
  if (!c->sched_fixed) {
    std::lock_guard<std::mutex> lk(g_tuned_mu);
    auto it = g_tuned.find(c->shape_key);
    if (it != g_tuned.end()) c->sched = it->second;
    else default_schedule(c);
  }
  if ((rc = apply_schedule(c)) != PCG_OK) return rc;
  c->patches_dirty = true;
  c->topo_dirty = false;
  c->graph_valid = false;
  return upload_patches(c);
}

int upload_group_max_dt(pcg_context *c) {
  PCG_CUDA(cudaMemcpyAsync(c->d_group_max_dt, c->h_group_max_dt.data(), sizeof(double) * c->max_groups,
                           cudaMemcpyHostToDevice, c->stream));
  return PCG_OK;
}

// The region geometry of the restriction list, when the lists, the patches'
// geometry or the restriction bounds changed since it was built (called
// before a step graph is captured, so that a graph holds no rebuild).
int refresh_restr_geometry(pcg_context *c) {
  if (!c->restr_geo_dirty || c->h_restr.empty()) return PCG_OK;
  PCG_CUDA(pcg::launch_restr_geometry(c->stream, c->d_patches, c->d_times, c->d_restr, c->d_restr_begin,
                                      (int)c->restr_dsts.size(), c->d_restr_geo, c->d_restr_geo_bad));
  c->restr_geo_dirty = false;
  return PCG_OK;
}

// Flux correction (computeFluxes of every leaf, then the correction list) and
// restriction into the virtual patches (clear, restrict list, post-process),
// the order in which SolveTimestep::enterCell and Remesh::leaveCell run them,
// in one launch (k_level_transfer).
int enqueue_level_transfer(pcg_context *c, bool flux, bool restr, const int *group_active, const int *pact) {
  using namespace pcg;
  flux = flux && !c->h_flux.empty();
  restr = restr && !c->h_restr.empty();
  const int n_leaf = flux ? (int)c->flux_leaf_ids.size() : 0;
  const int n_flux = flux ? (int)c->flux_begin.size() - 1 : 0;
  const int n_restr = restr ? (int)c->h_restr_chunks.size() : 0;
  const int grid = level_transfer_grid(c->num_sms, n_leaf, n_flux, n_restr);
  if (grid <= 0) return PCG_OK;
  if (restr) {
    int rc = refresh_restr_geometry(c);
    if (rc != PCG_OK) return rc;
  }
  PCG_CUDA(launch_level_transfer(c->stream, grid, c->slab, c->d_patches, c->d_times, c->d_flux_leaf_ids, n_leaf,
                                 c->g_flux, c->d_flux, c->d_flux_begin, n_flux, c->d_restr, c->d_restr_begin,
                                 c->d_restr_geo, c->d_restr_geo_bad, c->d_restr_chunks, n_restr, group_active,
                                 pact, c->d_xfer));
  c->xfer_pending = true;
  return PCG_OK;
}

int enqueue_post_update(pcg_context *c) {
  return enqueue_level_transfer(c, true, true, c->d_group_active, c->ts_local ? c->d_pact : nullptr);
}

// After the stream has been synchronised: the error word of the level
// transfers since the last check (a phase wait that ran out).
int check_level_transfer(pcg_context *c) {
  if (!c->xfer_pending) return PCG_OK;
  c->xfer_pending = false;
  int err = 0;
  PCG_CUDA(cudaMemcpy(&err, &c->d_xfer->err, sizeof(int), cudaMemcpyDeviceToHost));
  if (err) {
    PCG_CUDA(cudaMemset(c->d_xfer, 0, sizeof(pcg::TransferCtl)));
    if (err == 2)
      return fail(PCG_E_CUDA, "TMA tile sweep: the staging copies of a tile did not complete in time; the step's "
                              "sweep is incomplete");
    return fail(PCG_E_CUDA, "level transfer: a wait between its phases ran out; the step's flux correction "
                            "and restriction are incomplete");
  }
  return PCG_OK;
}

// Rescan the finiteness flags of every patch (after anything but a batched
// step changed patch data).
int refresh_fin(pcg_context *c) {
  if (!c->fin_dirty) return PCG_OK;
  PCG_CUDA(pcg::launch_scan_fin(c->stream, c->slab, c->d_patches, c->max_patches, c->d_fin));
  c->fin_dirty = false;
  return PCG_OK;
}

// Tensor maps of the TMA tile sweep for every leaf (built when the variant
// first runs after a topology change; the patches' data do not move).
int ensure_tile_maps(pcg_context *c) {
  if (c->tile_maps_valid) return PCG_OK;
  if (!c->tma_ok) return fail(PCG_E_INVALID, "the TMA tile staging needs leaves of even size with ghost width 1, "
                                            "3 unknowns and the bathymetry field only");
  std::vector<pcg::TileMaps> h((size_t)std::max(1, c->patch_hw));
  for (int p : c->leaf_ids) {
    cudaError_t e = pcg::encode_tile_maps(c->h_patches[p], c->slab, &h[p]);
    if (e != cudaSuccess) return fail(PCG_E_CUDA, std::string("tensor map of patch ") + std::to_string(p) + ": " +
                                                      cudaGetErrorString(e));
  }
  int rc;
  if ((rc = ensure_device(c, &c->d_tile_maps, &c->d_tmaps_cap, h.size())) != PCG_OK) return rc;
  PCG_CUDA(cudaMemcpyAsync(c->d_tile_maps, h.data(), sizeof(pcg::TileMaps) * h.size(), cudaMemcpyHostToDevice,
                           c->stream));
  PCG_CUDA(cudaStreamSynchronize(c->stream));
  c->tile_maps_valid = true;
  return PCG_OK;
}

// Batched sweep and update with the context's schedule.
int enqueue_sweep(pcg_context *c) {
  using namespace pcg;
  if (c->sched.kind == PCG_SCHED_TILES && c->sched.variant == 1) {
    int rc = ensure_tile_maps(c);
    if (rc != PCG_OK) return rc;
    PCG_CUDA(launch_sweep_tma(c->stream, c->sweep_grid, c->slab, c->d_patches, c->d_tile_maps, c->d_tiles, 0,
                              (int)c->h_tiles.size(), c->prm, c->d_patch_smax, c->d_group_dt, c->d_group_active,
                              c->d_fin, c->ts_local ? c->d_pact : nullptr, &c->d_xfer->err));
    c->xfer_pending = true;
  } else if (c->sched.kind == PCG_SCHED_TILES)
    PCG_CUDA(launch_sweep(c->stream, c->sweep_grid, c->slab, c->d_patches, c->d_tiles, 0,
                          (int)c->h_tiles.size(), c->prm, c->d_patch_smax, c->d_group_dt,
                          c->d_group_active, c->d_fin, c->ts_local ? c->d_pact : nullptr));
  else
    PCG_CUDA(launch_sweep_strips(c->stream, c->sched.variant, c->strip_grid, c->slab, c->d_patches,
                                 c->d_sitems, c->d_sgroups, (int)c->h_sitems.size(), c->prm,
                                 c->d_patch_smax, c->d_group_dt, c->d_group_active, c->d_fin,
                                 c->ts_local ? c->d_pact : nullptr));
  return PCG_OK;
}

int enqueue_update(pcg_context *c) {
  using namespace pcg;
  if (c->sched.kind == PCG_SCHED_TILES) {
    PCG_CUDA(launch_update(c->stream, c->sweep_grid, c->slab, c->d_patches, c->d_times, c->d_tiles, 0,
                           (int)c->h_tiles.size(), c->prm, c->d_patch_smax, c->d_group_dt,
                           c->d_group_active, c->d_fin, c->ts_local ? c->d_pact : nullptr,
                           c->ts_local ? c->d_pdt : nullptr));
  } else {
    pcg::UpdateBands ub;
    ub.band = c->d_band;
    ub.full = c->d_upd_full;
    ub.group_time = c->d_group_time;
    ub.group_t_end = c->d_group_t_end;
    PCG_CUDA(launch_update_strips(c->stream, c->update_grid, c->slab, c->d_patches, c->d_times,
                                  c->d_sitems, c->d_sgroups, (int)c->h_sitems.size(), c->prm,
                                  c->d_patch_smax, c->d_group_dt, c->d_group_active, c->d_fin,
                                  c->ts_local ? c->d_pact : nullptr, c->ts_local ? c->d_pdt : nullptr, ub));
  }
  return PCG_OK;
}

// One local-time-stepping phase (0: activity, 1: dts, 2: group times).
int enqueue_lts(pcg_context *c, int phase) {
  pcg::LtsVirtualDev vt;
  vt.pairs = c->d_vt;
  vt.n_pairs = (int)c->h_vt.size();
  vt.virtuals = c->d_vt_virtuals;
  vt.n_virtual = (int)c->vt_virtuals.size();
  vt.start = c->d_vstart;
  vt.end = c->d_vend;
  PCG_CUDA(pcg::launch_lts(c->stream, phase, c->max_patches, c->max_groups, c->d_patches, c->d_times,
                           c->d_items, (int)c->h_items.size(), vt, c->d_nbmin, c->d_patch_smax,
                           c->d_group_tmin, c->d_group_dt, c->d_group_max_dt, c->d_group_t_end,
                           c->d_group_active, c->d_pact, c->d_pmaxdt, c->d_pdt, c->d_group_time, c->prm,
                           c->d_lts_cells));
  return PCG_OK;
}

// Enqueue one synchronous step (no synchronisation, capturable in BATCHED
// mode); with local time stepping one iteration in which only the leaves
// that may advance are filled and solved, each with its own dt.
int enqueue_step(pcg_context *c, int mode, bool advance = true) {
  using namespace pcg;
  int rc;
  if (mode == PCG_MODE_BATCHED) {
    // reset and per-item time factors in one launch (the time factors read
    // the times before the step, which neither the reset nor the first
    // local-time-stepping phase changes)
    PCG_CUDA(launch_reset_items(c->stream, c->max_groups, c->d_group_max_dt, c->d_group_t_end, c->d_group_time,
                                c->d_group_dt, c->d_group_active, c->max_patches, c->d_patch_smax, c->d_patches,
                                c->d_times, c->d_items, (int)c->h_items.size(), c->d_item_step));
    const int *pact = c->ts_local ? c->d_pact : nullptr;
    if (c->ts_local && (rc = enqueue_lts(c, 0)) != PCG_OK) return rc;
    PCG_CUDA(launch_ghost_cells(c->stream, c->slab, c->d_patches, c->d_items, c->d_gcells, c->n_copy_cells,
                                c->n_interp_cells, c->d_copy_plan, c->d_plan, c->d_item_step,
                                c->d_group_active, c->d_fin, pact));
    PCG_CUDA(launch_walls(c->stream, c->slab, c->d_patches, c->d_wall, (int)c->h_wall.size(),
                          c->d_group_active, pact));
    if ((rc = enqueue_sweep(c)) != PCG_OK) return rc;
    if (c->ts_local && (rc = enqueue_lts(c, 1)) != PCG_OK) return rc;
    if ((rc = enqueue_update(c)) != PCG_OK) return rc;
    if (c->ts_local) {
      if ((rc = enqueue_lts(c, 2)) != PCG_OK) return rc;
      return enqueue_post_update(c);
    }
  } else {
    PCG_CUDA(launch_reset(c->stream, c->max_groups, c->d_group_max_dt, c->d_group_t_end, c->d_group_time,
                          c->d_group_dt, c->d_group_active, c->max_patches, c->d_patch_smax));
    for (int p : c->leaf_ids)
      PCG_CUDA(launch_fill_patch(c->stream, c->slab, c->d_patches, c->d_times, c->d_items,
                                 c->item_first[p], c->item_count[p], p, c->d_group_active));
    for (int p : c->leaf_ids) {
      const PatchDev &P = c->h_patches[p];
      PCG_CUDA(launch_sweep(c->stream, P.tile_count, c->slab, c->d_patches, c->d_tiles, P.tile_begin,
                            P.tile_count, c->prm, c->d_patch_smax, c->d_group_dt, c->d_group_active,
                            nullptr));
    }
    for (int p : c->leaf_ids) {
      const PatchDev &P = c->h_patches[p];
      PCG_CUDA(launch_update(c->stream, P.tile_count, c->slab, c->d_patches, c->d_times, c->d_tiles,
                             P.tile_begin, P.tile_count, c->prm, c->d_patch_smax, c->d_group_dt,
                             c->d_group_active, nullptr));
    }
    c->fin_dirty = true;
  }
  rc = enqueue_post_update(c);
  if (rc != PCG_OK) return rc;
  if (advance)
    PCG_CUDA(launch_group_advance(c->stream, c->max_groups, c->d_group_dt, c->d_group_active,
                                  c->d_group_time));
  return PCG_OK;
}

// ---- fused step

pcg::FusedDev fused_dev(pcg_context *c) {
  pcg::FusedDev F;
  F.slab = c->slab;
  F.shadow = c->d_shadow;
  F.patches = c->d_patches;
  F.pend = c->d_pend;
  F.par = c->d_par;
  F.active = c->d_group_active;
  F.dt_prev = c->d_dt_prev;
  F.face_begin = c->d_face_begin;
  F.face = c->d_face;
  F.corner = c->d_corner;
  F.copies = c->d_fcopies;
  F.interps = c->d_finterps;
  F.item_step = c->d_item_step;
  F.prm = c->prm;
  return F;
}

// Whether a step of `mode` takes the fused form (after rebuild_topology).
bool use_fused(pcg_context *c, int mode) {
  if (c->form == PCG_FORM_UNFUSED || (mode == PCG_MODE_BATCHED && c->sched.unfused)) return false;
  return c->fused_lists_ok && !c->ts_local && c->h_restr.empty() && c->h_flux.empty() && !c->leaf_ids.empty() &&
         (mode == PCG_MODE_PLAIN || c->sched.kind == PCG_SCHED_STRIPS);
}

// Whether a batched run takes the pipelined form: the strip schedule asks
// for it (unfused = 2) and the step is the synchronous one without
// restriction or flux-correction lists.
bool use_pipeline(pcg_context *c, int mode) {
  return mode == PCG_MODE_BATCHED && c->form == PCG_FORM_AUTO && c->sched.kind == PCG_SCHED_STRIPS &&
         c->sched.unfused == 2 && !c->ts_local && c->h_restr.empty() && c->h_flux.empty() && !c->leaf_ids.empty();
}

// Work queue and counter targets of the pipelined step (pcg_pipeline.cu) for
// the current lists and strip items.  The strip updates are ranked in patch
// order; every item gets a key: the rank of the last strip update among its
// prerequisites (updates: their own rank); the queue holds, for key u in
// increasing order, update u, then the ghost chunks, the wall patches and the
// sweeps with key u.  An item's prerequisites then
// all come before it (their keys are at most its own, with an earlier kind).
int build_pipeline(pcg_context *c) {
  const int np = c->max_patches;
  const int n_upd = (int)c->h_sitems.size();
  const int64_t n_ghost = c->n_gcells;
  const int64_t n_chunks = (n_ghost + pcg::kPipeGhostChunk - 1) / pcg::kPipeGhostChunk;
  if (n_ghost > INT32_MAX || n_upd > (int)pcg::kPipeIndexMask || n_chunks > (int64_t)pcg::kPipeIndexMask)
    return fail(PCG_E_INVALID, "pipelined step: the strip or ghost-cell list is too long");
  std::vector<int> need(4 * (size_t)np, 0);
  std::vector<int> ukey(np, -1), ginkey(np, -1), goutkey(np, -1);
  // updates in patch order (the strip list is sorted by strip shape): a
  // patch's neighbours are then updated shortly before or after it, and its
  // sweep can follow soon after its own update
  std::vector<int> uorder(n_upd), urank(n_upd);
  {
    std::vector<int> first_pid(n_upd);
    for (int i = 0; i < n_upd; i++) {
      const pcg::StripItem &I = c->h_sitems[i];
      int m = INT32_MAX;
      for (int g = 0; g < I.ngroups; g++) m = std::min(m, c->h_sgroups[I.g0 + g].pid);
      first_pid[i] = m;
      uorder[i] = i;
    }
    std::stable_sort(uorder.begin(), uorder.end(), [&](int a, int b) { return first_pid[a] < first_pid[b]; });
    for (int r = 0; r < n_upd; r++) urank[uorder[r]] = r;
  }
  for (int i = 0; i < n_upd; i++) {
    const pcg::StripItem &I = c->h_sitems[i];
    for (int g = 0; g < I.ngroups; g++) {
      const int p = c->h_sgroups[I.g0 + g].pid;
      need[p]++;
      ukey[p] = std::max(ukey[p], urank[i]);
    }
  }
  // every level waits `lag` ranks more than its prerequisites need: about
  // half the resident warps' worth of queue entries, so that what an item
  // waits for has usually finished when a warp takes it
  const int lag = std::max(64, c->pipe_grid * pcg::kStripVariants[c->sched.variant].warps / 2);
  std::vector<int> gkey((size_t)n_chunks, -1);
  for (size_t r = 0; r + 1 < c->h_gexp.size(); r++) {
    const int64_t b = c->h_gexp[r].y, e = c->h_gexp[r + 1].y;
    if (e <= b) continue;
    const pcg::GhostItemDev &it = c->h_items[c->h_gexp[r].x];
    need[(size_t)np + it.dst] += (int)(e - b);
    need[2 * (size_t)np + it.src] += (int)(e - b);
    const int key = std::max(ukey[it.src], ukey[it.dst]) + lag;
    for (int64_t ch = b / pcg::kPipeGhostChunk; ch <= (e - 1) / pcg::kPipeGhostChunk; ch++)
      gkey[ch] = std::max(gkey[ch], key);
  }
  for (size_t r = 0; r + 1 < c->h_gexp.size(); r++) {
    const int64_t b = c->h_gexp[r].y, e = c->h_gexp[r + 1].y;
    if (e <= b) continue;
    const pcg::GhostItemDev &it = c->h_items[c->h_gexp[r].x];
    for (int64_t ch = b / pcg::kPipeGhostChunk; ch <= (e - 1) / pcg::kPipeGhostChunk; ch++) {
      ginkey[it.dst] = std::max(ginkey[it.dst], gkey[ch]);
      goutkey[it.src] = std::max(goutkey[it.src], gkey[ch]);
    }
  }
  std::vector<int> wkey(np, -1);
  for (int p : c->h_wall) {
    need[3 * (size_t)np + p] = 1;
    wkey[p] = std::max(ukey[p], ginkey[p]) + lag;
  }
  std::vector<int> skey(n_upd, -1);
  for (int i = 0; i < n_upd; i++) {
    const pcg::StripItem &I = c->h_sitems[i];
    int k = -1;
    for (int g = 0; g < I.ngroups; g++) {
      const int p = c->h_sgroups[I.g0 + g].pid;
      k = std::max({k, ukey[p], ginkey[p], goutkey[p], wkey[p]});
    }
    skey[i] = k + lag;
  }
  // bucket b = key + 1: counts per bucket and kind, then fill
  int max_key = n_upd - 1;
  for (int k : gkey) max_key = std::max(max_key, k);
  for (int p : c->h_wall) max_key = std::max(max_key, wkey[p]);
  for (int k : skey) max_key = std::max(max_key, k);
  const size_t nb = (size_t)max_key + 2;
  std::vector<int64_t> start(4 * nb + 1, 0);  // (bucket, kind) -> first queue position
  auto slot = [](int key, unsigned kind) { return (size_t)(key + 1) * 4 + kind; };
  for (int i = 0; i < n_upd; i++) start[slot(urank[i], pcg::kPipeUpdate) + 1]++;
  for (int64_t ch = 0; ch < n_chunks; ch++) start[slot(gkey[ch], pcg::kPipeGhost) + 1]++;
  for (int p : c->h_wall) start[slot(wkey[p], pcg::kPipeWall) + 1]++;
  for (int i = 0; i < n_upd; i++) start[slot(skey[i], pcg::kPipeSweep) + 1]++;
  for (size_t k = 1; k < start.size(); k++) start[k] += start[k - 1];
  const int64_t n_queue = start.back();
  std::vector<unsigned> queue((size_t)n_queue);
  auto put = [&](int key, unsigned kind, int64_t index) {
    queue[(size_t)start[slot(key, kind)]++] = (kind << pcg::kPipeKindShift) | (unsigned)index;
  };
  for (int i = 0; i < n_upd; i++) put(urank[i], pcg::kPipeUpdate, i);
  for (int64_t ch = 0; ch < n_chunks; ch++) put(gkey[ch], pcg::kPipeGhost, ch);
  for (size_t w = 0; w < c->h_wall.size(); w++) put(wkey[c->h_wall[w]], pcg::kPipeWall, (int64_t)w);
  for (int i = 0; i < n_upd; i++) put(skey[i], pcg::kPipeSweep, i);
  // the order the kernel relies on (every wait is for an earlier entry):
  // checked here rather than found out as a wait that runs out
  {
    std::vector<int64_t> last_u(np, -1), last_gin(np, -1), last_gout(np, -1), wall_pos(np, -1);
    std::vector<int64_t> chunk_pos((size_t)n_chunks, -1), sweep_pos(n_upd, -1);
    for (int64_t q = 0; q < n_queue; q++) {
      const unsigned kind = queue[(size_t)q] >> pcg::kPipeKindShift;
      const int64_t i = queue[(size_t)q] & pcg::kPipeIndexMask;
      if (kind == pcg::kPipeUpdate) {
        const pcg::StripItem &I = c->h_sitems[(size_t)i];
        for (int g = 0; g < I.ngroups; g++) last_u[c->h_sgroups[I.g0 + g].pid] = q;
      } else if (kind == pcg::kPipeGhost) {
        chunk_pos[(size_t)i] = q;
      } else if (kind == pcg::kPipeWall) {
        wall_pos[c->h_wall[(size_t)i]] = q;
      } else {
        sweep_pos[(size_t)i] = q;
      }
    }
    bool ok = true;
    for (size_t r = 0; r + 1 < c->h_gexp.size() && ok; r++) {
      const int64_t b = c->h_gexp[r].y, e = c->h_gexp[r + 1].y;
      if (e <= b) continue;
      const pcg::GhostItemDev &it = c->h_items[c->h_gexp[r].x];
      for (int64_t ch = b / pcg::kPipeGhostChunk; ch <= (e - 1) / pcg::kPipeGhostChunk; ch++) {
        const int64_t q = chunk_pos[(size_t)ch];
        ok = ok && q > last_u[it.src] && q > last_u[it.dst];
        last_gin[it.dst] = std::max(last_gin[it.dst], q);
        last_gout[it.src] = std::max(last_gout[it.src], q);
      }
    }
    for (int p : c->h_wall) ok = ok && wall_pos[p] > last_u[p] && wall_pos[p] > last_gin[p];
    for (int i = 0; i < n_upd && ok; i++) {
      const pcg::StripItem &I = c->h_sitems[i];
      for (int g = 0; g < I.ngroups; g++) {
        const int p = c->h_sgroups[I.g0 + g].pid;
        const int64_t q = sweep_pos[i];
        ok = ok && q > last_u[p] && q > last_gin[p] && q > last_gout[p] && q > wall_pos[p];
      }
    }
    if (!ok) return fail(PCG_E_STATE, "pipelined step: work queue out of order");
  }
  int rc;
  if ((rc = ensure_device(c, &c->d_pipe_queue, &c->d_pipe_queue_cap, queue.size())) != PCG_OK) return rc;
  if ((rc = ensure_device(c, &c->d_pipe_need, &c->d_pipe_need_cap, need.size())) != PCG_OK) return rc;
  if ((rc = ensure_device(c, &c->d_pipe_cnt, &c->d_pipe_cnt_cap, need.size())) != PCG_OK) return rc;
  if ((rc = ensure_device(c, &c->d_pipe_ctl, &c->d_pipe_ctl_cap, 1)) != PCG_OK) return rc;
  if ((rc = ensure_device(c, &c->d_pipe_dt, &c->d_pipe_dt_cap, (size_t)c->max_groups)) != PCG_OK) return rc;
  if ((rc = ensure_device(c, &c->d_pipe_active, &c->d_pipe_active_cap, (size_t)c->max_groups)) != PCG_OK) return rc;
  if ((rc = ensure_device(c, &c->d_pipe_smax, &c->d_pipe_smax_cap, (size_t)np)) != PCG_OK) return rc;
  if (!queue.empty())
    PCG_CUDA(cudaMemcpyAsync(c->d_pipe_queue, queue.data(), sizeof(unsigned) * queue.size(),
                             cudaMemcpyHostToDevice, c->stream));
  PCG_CUDA(cudaMemcpyAsync(c->d_pipe_need, need.data(), sizeof(int) * need.size(), cudaMemcpyHostToDevice,
                           c->stream));
  PCG_CUDA(cudaMemsetAsync(c->d_pipe_ctl, 0, sizeof(pcg::PipeCtl), c->stream));
  PCG_CUDA(cudaStreamSynchronize(c->stream));
  c->n_pipe_queue = (int)n_queue;
  c->pipe_valid = true;
  c->graph_valid = false;
  return PCG_OK;
}

pcg::PipeDev pipe_dev(pcg_context *c) {
  pcg::PipeDev A;
  A.slab = c->slab;
  A.patches = c->d_patches;
  A.times = c->d_times;
  A.items = c->d_sitems;
  A.groups = c->d_sgroups;
  A.gitems = c->d_items;
  A.cells = c->d_gcells;
  A.copy_plan = c->d_copy_plan;
  A.plan = c->d_plan;
  A.ncopy = c->n_copy_cells;
  A.n_ghost = (int)c->n_gcells;
  A.item_step = c->d_item_step;
  A.wall_patches = c->d_wall;
  A.queue = c->d_pipe_queue;
  A.n_queue = c->n_pipe_queue;
  A.n_patches = c->max_patches;
  A.cnt = c->d_pipe_cnt;
  A.need = c->d_pipe_need;
  A.cur_dt = c->d_group_dt;
  A.nxt_dt = c->d_pipe_dt;
  A.cur_smax = c->d_patch_smax;
  A.nxt_smax = c->d_pipe_smax;
  A.cur_active = c->d_group_active;
  A.nxt_active = c->d_pipe_active;
  A.fin = c->d_fin;
  A.prm = c->prm;
  A.ctl = c->d_pipe_ctl;
  return A;
}

pcg::PipePreDev pipe_pre_dev(pcg_context *c) {
  pcg::PipePreDev A;
  A.n_groups = c->max_groups;
  A.n_patches = c->max_patches;
  A.group_max_dt = c->d_group_max_dt;
  A.group_t_end = c->d_group_t_end;
  A.group_time = c->d_group_time;
  A.cur_dt = c->d_group_dt;
  A.nxt_dt = c->d_pipe_dt;
  A.cur_smax = c->d_patch_smax;
  A.nxt_smax = c->d_pipe_smax;
  A.cur_active = c->d_group_active;
  A.nxt_active = c->d_pipe_active;
  A.hist = c->d_hist;
  A.hist_cap = c->hist_cap;
  A.cnt = c->d_pipe_cnt;
  A.ctl = c->d_pipe_ctl;
  return A;
}

pcg::PipeItemsDev pipe_items_dev(pcg_context *c) {
  pcg::PipeItemsDev A;
  A.patches = c->d_patches;
  A.times = c->d_times;
  A.items = c->d_items;
  A.n_items = (int)c->h_items.size();
  A.cur_dt = c->d_group_dt;
  A.cur_active = c->d_group_active;
  A.item_step = c->d_item_step;
  A.ctl = c->d_pipe_ctl;
  return A;
}

// The bookkeeping and item launches before each pipelined step launch.
int enqueue_pipeline_prep(pcg_context *c) {
  PCG_CUDA(pcg::launch_pipeline_pre(c->stream, pipe_pre_dev(c)));
  PCG_CUDA(pcg::launch_pipeline_items(c->stream, pipe_items_dev(c)));
  return PCG_OK;
}

// One launch triple of a pipelined run (capturable).
int enqueue_pipeline_launch(pcg_context *c) {
  int rc = enqueue_pipeline_prep(c);
  if (rc != PCG_OK) return rc;
  PCG_CUDA(pcg::launch_pipeline_step(c->stream, c->sched.variant, c->pipe_grid, pipe_dev(c)));
  return PCG_OK;
}

// Start of a pipelined run of `steps` steps (steps + 1 launch pairs follow).
int start_pipeline_run(pcg_context *c, int steps) {
  pcg::PipeCtl h{};
  h.steps = steps;
  PCG_CUDA(cudaMemcpyAsync(c->d_pipe_ctl, &h, sizeof(h), cudaMemcpyHostToDevice, c->stream));
  return PCG_OK;
}

// After the stream has been synchronised: the error word of the last
// pipelined run (a wait that ran out).
int check_pipeline(pcg_context *c) {
  int err = 0;
  PCG_CUDA(cudaMemcpy(&err, &c->d_pipe_ctl->err, sizeof(int), cudaMemcpyDeviceToHost));
  if (!err) return PCG_OK;
  PCG_CUDA(cudaMemset(c->d_pipe_ctl, 0, sizeof(pcg::PipeCtl)));
  return fail(PCG_E_CUDA, "pipelined step: a wait for another work item ran out; the run is incomplete");
}

// Back to the reference layout: every group with a pending update gets it
// applied (uNew, uOld interior) and its walls filled from the previous state;
// called by every entry point that reads or changes patch data, lists or
// parameters.  The next fused step then starts with its own reset.
int settle(pcg_context *c) {
  c->fused_ready = false;
  if (!c->fused_pending) return PCG_OK;
  PCG_CUDA(cudaSetDevice(c->device));
  const pcg::FusedDev F = fused_dev(c);
  PCG_CUDA(pcg::launch_fused_flush(c->stream, F, c->d_leaf_ids, (int)c->leaf_ids.size()));
  PCG_CUDA(pcg::launch_walls(c->stream, c->slab, c->d_patches, c->d_wall, (int)c->h_wall.size(), c->d_pend,
                             nullptr, 0));
  PCG_CUDA(cudaMemsetAsync(c->d_pend, 0, sizeof(int) * c->max_groups, c->stream));
  c->fused_pending = false;
  c->fin_dirty = true;
  return PCG_OK;
}

#define PCG_SETTLE(c)                          \
  do {                                         \
    int src_ = settle(c);                      \
    if (src_ != PCG_OK) return src_;           \
  } while (0)

int ensure_shadow(pcg_context *c) {
  if (c->d_shadow && (int64_t)c->shadow_cap >= c->shadow_need) return PCG_OK;
  if (c->d_shadow) PCG_CUDA(cudaFree(c->d_shadow));
  c->d_shadow = nullptr;
  c->shadow_cap = 0;
  const size_t n = (size_t)std::max<int64_t>(c->shadow_need, kAlign);
  cudaError_t e = cudaMalloc(&c->d_shadow, sizeof(double) * n);
  if (e != cudaSuccess) {
    c->d_shadow = nullptr;
    return fail(e == cudaErrorMemoryAllocation ? PCG_E_NOMEM : PCG_E_CUDA,
                std::string("fused step state buffer: ") + cudaGetErrorString(e));
  }
  c->shadow_cap = n;
  return PCG_OK;
}

// The reset and per-item time factors that start a step.
int enqueue_reset_items(pcg_context *c) {
  PCG_CUDA(pcg::launch_reset_items(c->stream, c->max_groups, c->d_group_max_dt, c->d_group_t_end, c->d_group_time,
                                   c->d_group_dt, c->d_group_active, c->max_patches, c->d_patch_smax, c->d_patches,
                                   c->d_times, c->d_items, (int)c->h_items.size(), c->d_item_step));
  return PCG_OK;
}

// One fused step: the fused sweep (one launch, or one per patch in the plain
// form), the time advance with the dt record, and the reset and item factors
// of the next step (three launches in the batched form; capturable).
int enqueue_fused_step(pcg_context *c, int mode) {
  const pcg::FusedDev F = fused_dev(c);
  if (mode == PCG_MODE_BATCHED) {
    PCG_CUDA(pcg::launch_fused_strips(c->stream, c->sched.variant, c->fused_grid, F, c->d_sitems, c->d_sgroups,
                                      (int)c->h_sitems.size(), c->d_patch_smax, c->d_group_dt));
  } else {
    for (int p : c->leaf_ids) {
      const int n = c->pitem_count[p];
      PCG_CUDA(pcg::launch_fused_strips(c->stream, 2, (n + 7) / 8, F, c->d_pitems + c->pitem_first[p],
                                        c->d_pgroups, n, c->d_patch_smax, c->d_group_dt));
    }
  }
  PCG_CUDA(pcg::launch_fused_advance(c->stream, F, c->d_leaf_ids, (int)c->leaf_ids.size(), c->d_times,
                                     c->d_patch_smax, c->max_groups, c->d_group_dt, c->d_group_time, c->d_pend,
                                     c->d_par, c->d_dt_prev, c->d_hist, c->d_counter, c->hist_cap));
  return enqueue_reset_items(c);
}

// Before fused steps: the state buffer and, unless the previous fused step
// left it done, the reset of the first step.
int fused_prologue(pcg_context *c) {
  int rc = ensure_shadow(c);
  if (rc != PCG_OK) return rc;
  if (!c->fused_ready) {
    if ((rc = enqueue_reset_items(c)) != PCG_OK) return rc;
    c->fused_ready = true;
  }
  return PCG_OK;
}

int ensure_hist(pcg_context *c, int steps) {
  if (steps <= c->hist_cap) return PCG_OK;
  if (c->d_hist) PCG_CUDA(cudaFree(c->d_hist));
  c->d_hist = nullptr;
  PCG_CUDA(cudaMalloc(&c->d_hist, sizeof(double) * (size_t)steps * c->max_groups));
  c->hist_cap = steps;
  c->graph_valid = false;
  return PCG_OK;
}

int ensure_staging(pcg_context *c, size_t doubles, size_t metas) {
  int rc;
  if ((rc = ensure_device(c, &c->d_staging, &c->staging_cap, doubles)) != PCG_OK) return rc;
  if ((rc = ensure_device(c, &c->d_copy_meta, &c->copy_meta_cap, 3 * metas)) != PCG_OK) return rc;
  return PCG_OK;
}

int multi_copy(pcg_context *c, int32_t n, const int32_t *ids, double *vecs, bool upload) {
  if (n <= 0) return PCG_OK;
  std::vector<long long> meta(3 * (size_t)n);
  long long total = 0;
  for (int i = 0; i < n; i++) {
    if (!valid_id(c, ids[i])) return fail(PCG_E_INVALID, "unknown patch id " + std::to_string(ids[i]));
    meta[i] = c->h_patches[ids[i]].off;
    meta[n + i] = total;
    meta[2 * n + i] = c->h_len[ids[i]];
    total += c->h_len[ids[i]];
  }
  int rc = ensure_staging(c, (size_t)total, (size_t)n);
  if (rc != PCG_OK) return rc;
  PCG_CUDA(cudaMemcpyAsync(c->d_copy_meta, meta.data(), sizeof(long long) * meta.size(),
                           cudaMemcpyHostToDevice, c->stream));
  int grid = std::min(n, 152 * 8);
  if (upload) {
    PCG_CUDA(cudaMemcpyAsync(c->d_staging, vecs, sizeof(double) * total, cudaMemcpyHostToDevice, c->stream));
    k_scatter<<<grid, 256, 0, c->stream>>>(c->slab, c->d_staging, c->d_copy_meta, c->d_copy_meta + n,
                                           c->d_copy_meta + 2 * n, n, 1);
    PCG_CUDA(cudaGetLastError());
  } else {
    k_scatter<<<grid, 256, 0, c->stream>>>(c->slab, c->d_staging, c->d_copy_meta, c->d_copy_meta + n,
                                           c->d_copy_meta + 2 * n, n, 0);
    PCG_CUDA(cudaGetLastError());
    PCG_CUDA(cudaMemcpyAsync(vecs, c->d_staging, sizeof(double) * total, cudaMemcpyDeviceToHost, c->stream));
  }
  PCG_CUDA(cudaStreamSynchronize(c->stream));
  return PCG_OK;
}

pcg::GhostItemDev make_item(int kind, const int32_t size[2], const int32_t so[2], const int32_t dof[2],
                            int src, int dst) {
  pcg::GhostItemDev it;
  it.kind = kind; it.src = src; it.dst = dst;
  it.size[0] = size[0]; it.size[1] = size[1];
  it.src_off[0] = so ? so[0] : 0; it.src_off[1] = so ? so[1] : 0;
  it.dst_off[0] = dof[0]; it.dst_off[1] = dof[1];
  return it;
}

bool region_inside(const pcg::PatchDev &P, const int32_t off[2], const int32_t size[2], bool with_ghost) {
  int n[2] = {P.nx, P.ny};
  int g = with_ghost ? P.g : 0;
  for (int d = 0; d < 2; d++) {
    if (size[d] < 0 || off[d] < -g || off[d] + size[d] > n[d] + g) return false;
  }
  return true;
}

}  // namespace

extern "C" {

const char *pcg_last_error(void) { return g_last_error.c_str(); }

int64_t pcg_patch_vector_size(const pcg_patch_desc *desc) {
  if (!desc) return -1;
  return vector_size(*desc);
}

int pcg_create(const pcg_config *cfg, pcg_context **out) {
  if (!cfg || !out) return fail(PCG_E_INVALID, "null argument");
  if (cfg->max_patches <= 0 || cfg->max_groups <= 0 || cfg->slab_doubles <= 0)
    return fail(PCG_E_INVALID, "max_patches, max_groups and slab_doubles must be positive");
  int ndev = 0;
  PCG_CUDA(cudaGetDeviceCount(&ndev));
  if (cfg->device < 0 || cfg->device >= ndev) return fail(PCG_E_INVALID, "no such CUDA device");
  PCG_CUDA(cudaSetDevice(cfg->device));
  pcg_context *c = new pcg_context();
  c->device = cfg->device;
  cudaDeviceProp prop;
  cudaError_t e = cudaGetDeviceProperties(&prop, cfg->device);
  if (e != cudaSuccess) { delete c; return fail(PCG_E_CUDA, cudaGetErrorString(e)); }
  c->num_sms = prop.multiProcessorCount;
  c->prm = {cfg->params.g, cfg->params.cfl, cfg->params.dry_tol, cfg->params.dry_tol_update,
            cfg->params.s_min, cfg->params.dt_inf};
  c->max_patches = cfg->max_patches;
  c->max_groups = cfg->max_groups;
  c->slab_doubles = cfg->slab_doubles;
  c->h_patches.assign(c->max_patches, pcg::PatchDev{});
  c->h_len.assign(c->max_patches, 0);
  c->used.assign(c->max_patches, 0);
  c->h_group_max_dt.assign(c->max_groups, cfg->params.dt_inf);
  auto cleanup = [&](cudaError_t err) {
    pcg_destroy(c);
    return fail(PCG_E_CUDA, std::string("pcg_create: ") + cudaGetErrorString(err));
  };
#define CREATE_CK(x) do { cudaError_t err_ = (x); if (err_ != cudaSuccess) return cleanup(err_); } while (0)
  CREATE_CK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  CREATE_CK(cudaEventCreate(&c->ev0));
  CREATE_CK(cudaEventCreate(&c->ev1));
  CREATE_CK(cudaMalloc(&c->slab, sizeof(double) * c->slab_doubles));
  c->free_list[0] = c->slab_doubles / kAlign * kAlign;
  CREATE_CK(cudaMalloc(&c->d_patches, sizeof(pcg::PatchDev) * c->max_patches));
  CREATE_CK(cudaMemset(c->d_patches, 0, sizeof(pcg::PatchDev) * c->max_patches));
  CREATE_CK(cudaMalloc(&c->d_times, sizeof(pcg::PatchTimeDev) * c->max_patches));
  CREATE_CK(cudaMemset(c->d_times, 0, sizeof(pcg::PatchTimeDev) * c->max_patches));
  CREATE_CK(cudaMalloc(&c->d_patch_smax, sizeof(unsigned long long) * c->max_patches));
  CREATE_CK(cudaMalloc(&c->d_group_dt, sizeof(unsigned long long) * c->max_groups));
  CREATE_CK(cudaMalloc(&c->d_group_max_dt, sizeof(double) * c->max_groups));
  CREATE_CK(cudaMalloc(&c->d_group_t_end, sizeof(double) * c->max_groups));
  CREATE_CK(cudaMalloc(&c->d_group_time, sizeof(double) * c->max_groups));
  CREATE_CK(cudaMalloc(&c->d_group_active, sizeof(int) * c->max_groups));
  CREATE_CK(cudaMalloc(&c->d_fin, sizeof(int) * c->max_patches));
  CREATE_CK(cudaMemset(c->d_fin, 0, sizeof(int) * c->max_patches));
  CREATE_CK(cudaMalloc(&c->d_pact, sizeof(int) * c->max_patches));
  CREATE_CK(cudaMemset(c->d_pact, 0, sizeof(int) * c->max_patches));
  CREATE_CK(cudaMalloc(&c->d_pmaxdt, sizeof(double) * c->max_patches));
  CREATE_CK(cudaMalloc(&c->d_pdt, sizeof(unsigned long long) * c->max_patches));
  CREATE_CK(cudaMalloc(&c->d_nbmin, sizeof(unsigned long long) * c->max_patches));
  CREATE_CK(cudaMalloc(&c->d_group_tmin, sizeof(unsigned long long) * c->max_groups));
  CREATE_CK(cudaMalloc(&c->d_lts_cells, sizeof(unsigned long long)));
  CREATE_CK(cudaMemset(c->d_lts_cells, 0, sizeof(unsigned long long)));
  CREATE_CK(cudaMalloc(&c->d_vstart, sizeof(unsigned long long) * c->max_patches));
  CREATE_CK(cudaMalloc(&c->d_vend, sizeof(unsigned long long) * c->max_patches));
  {
    std::vector<double> inf(c->max_groups, HUGE_VAL), zero(c->max_groups, 0.0);
    CREATE_CK(cudaMemcpy(c->d_group_t_end, inf.data(), sizeof(double) * c->max_groups, cudaMemcpyHostToDevice));
    CREATE_CK(cudaMemcpy(c->d_group_time, zero.data(), sizeof(double) * c->max_groups, cudaMemcpyHostToDevice));
    CREATE_CK(cudaMemset(c->d_group_active, 0, sizeof(int) * c->max_groups));
  }
  CREATE_CK(cudaMalloc(&c->d_pend, sizeof(int) * c->max_groups));
  CREATE_CK(cudaMemset(c->d_pend, 0, sizeof(int) * c->max_groups));
  CREATE_CK(cudaMalloc(&c->d_par, sizeof(int) * c->max_groups));
  CREATE_CK(cudaMemset(c->d_par, 0, sizeof(int) * c->max_groups));
  CREATE_CK(cudaMalloc(&c->d_dt_prev, sizeof(unsigned long long) * c->max_groups));
  CREATE_CK(cudaMemset(c->d_dt_prev, 0, sizeof(unsigned long long) * c->max_groups));
  CREATE_CK(cudaMalloc(&c->d_face_begin, sizeof(int) * c->max_patches));
  CREATE_CK(cudaMalloc(&c->d_corner, sizeof(int) * 4 * (size_t)c->max_patches));
  CREATE_CK(cudaMalloc(&c->d_dt_out, sizeof(double) * c->max_groups));
  CREATE_CK(cudaMalloc(&c->d_solve_out, sizeof(double) * 2));
  CREATE_CK(cudaMalloc(&c->d_counter, sizeof(int)));
  CREATE_CK(cudaMalloc(&c->d_band, sizeof(int4) * c->max_patches));
  CREATE_CK(cudaMemset(c->d_band, 0, sizeof(int4) * c->max_patches));
  CREATE_CK(cudaMalloc(&c->d_upd_full, sizeof(int)));
  CREATE_CK(cudaMemset(c->d_upd_full, 1, sizeof(int)));
  CREATE_CK(cudaMalloc(&c->d_xfer, sizeof(pcg::TransferCtl)));
  CREATE_CK(cudaMemset(c->d_xfer, 0, sizeof(pcg::TransferCtl)));
  CREATE_CK(cudaMallocHost(&c->h_pinned, sizeof(double) * std::max(64, c->max_groups)));
#undef CREATE_CK
  *out = c;
  return PCG_OK;
}

int pcg_destroy(pcg_context *c) {
  if (!c) return PCG_OK;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->graph) cudaGraphExecDestroy(c->graph);
  cudaFree(c->slab);
  cudaFree(c->d_patches);
  cudaFree(c->d_times);
  cudaFree(c->d_patch_smax);
  cudaFree(c->d_group_dt);
  cudaFree(c->d_group_max_dt);
  cudaFree(c->d_group_t_end);
  cudaFree(c->d_group_time);
  cudaFree(c->d_group_active);
  cudaFree(c->d_fin);
  cudaFree(c->d_pact);
  cudaFree(c->d_pmaxdt);
  cudaFree(c->d_pdt);
  cudaFree(c->d_nbmin);
  cudaFree(c->d_group_tmin);
  cudaFree(c->d_vstart);
  cudaFree(c->d_lts_cells);
  cudaFree(c->d_vend);
  cudaFree(c->d_vt);
  cudaFree(c->d_vt_virtuals);
  cudaFree(c->d_dt_out);
  cudaFree(c->d_items);
  cudaFree(c->d_gcells);
  cudaFree(c->d_gexp);
  cudaFree(c->d_restr);
  cudaFree(c->d_flux);
  cudaFree(c->d_restr_begin);
  cudaFree(c->d_flux_begin);
  cudaFree(c->d_restr_dsts);
  cudaFree(c->d_xfer);
  cudaFree(c->d_tile_maps);
  cudaFree(c->d_restr_geo);
  cudaFree(c->d_restr_geo_bad);
  cudaFree(c->d_restr_chunks);
  cudaFree(c->d_flux_leaf_ids);
  cudaFree(c->d_leaf_ids);
  cudaFree(c->d_plan);
  cudaFree(c->d_copy_plan);
  cudaFree(c->d_item_step);
  cudaFree(c->d_tiles);
  cudaFree(c->d_sitems);
  cudaFree(c->d_sgroups);
  cudaFree(c->d_wall);
  cudaFree(c->d_solve_out);
  cudaFree(c->d_hist);
  cudaFree(c->d_counter);
  cudaFree(c->d_staging);
  cudaFree(c->d_copy_meta);
  cudaFree(c->d_shadow);
  cudaFree(c->d_pend);
  cudaFree(c->d_par);
  cudaFree(c->d_dt_prev);
  cudaFree(c->d_face_begin);
  cudaFree(c->d_face);
  cudaFree(c->d_corner);
  cudaFree(c->d_fcopies);
  cudaFree(c->d_finterps);
  cudaFree(c->d_pitems);
  cudaFree(c->d_pgroups);
  cudaFree(c->d_band);
  cudaFree(c->d_upd_full);
  cudaFree(c->d_pipe_queue);
  cudaFree(c->d_pipe_need);
  cudaFree(c->d_pipe_cnt);
  cudaFree(c->d_pipe_ctl);
  cudaFree(c->d_pipe_dt);
  cudaFree(c->d_pipe_smax);
  cudaFree(c->d_pipe_active);
  if (c->h_pinned) cudaFreeHost(c->h_pinned);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return PCG_OK;
}

int pcg_slab_info(pcg_context *c, int64_t *free_doubles, int64_t *total_doubles) {
  if (!c) return fail(PCG_E_INVALID, "null context");
  int64_t f = 0;
  for (auto &kv : c->free_list) f += kv.second;
  if (free_doubles) *free_doubles = f;
  if (total_doubles) *total_doubles = c->slab_doubles;
  return PCG_OK;
}

int pcg_set_params(pcg_context *c, const pcg_swe_params *p) {
  if (!c || !p) return fail(PCG_E_INVALID, "null argument");
  std::lock_guard<std::mutex> lk(c->mu);
  PCG_SETTLE(c);
  c->prm = {p->g, p->cfl, p->dry_tol, p->dry_tol_update, p->s_min, p->dt_inf};
  c->graph_valid = false;
  return PCG_OK;
}

int pcg_patch_alloc(pcg_context *c, const pcg_patch_desc *d, int32_t *id) {
  if (!c || !d || !id) return fail(PCG_E_INVALID, "null argument");
  if (d->nx <= 0 || d->ny <= 0 || d->ghost < 0 || d->nq <= 0 || d->np_wo < 0 || d->np_w < 0)
    return fail(PCG_E_INVALID, "invalid patch shape");
  if (!(d->size[0] > 0.0) || !(d->size[1] > 0.0)) return fail(PCG_E_INVALID, "patch size must be positive");
  std::lock_guard<std::mutex> lk(c->mu);
  PCG_SETTLE(c);
  c->fin_dirty = true;
  int slot = -1;
  for (int k = 0; k < c->max_patches; k++) {
    int p = (c->slot_hint + k) % c->max_patches;
    if (!c->used[p]) { slot = p; break; }
  }
  if (slot < 0) return fail(PCG_E_NOMEM, "patch table full");
  int64_t len = vector_size(*d), off = 0;
  int rc = slab_alloc(c, len, &off);
  if (rc != PCG_OK) return rc;
  PCG_CUDA(cudaSetDevice(c->device));
  PCG_CUDA(cudaMemsetAsync(c->slab + off, 0, sizeof(double) * len, c->stream));
  pcg::PatchDev &P = c->h_patches[slot];
  P = pcg::PatchDev{};
  P.off = off;
  P.nx = d->nx; P.ny = d->ny; P.g = d->ghost; P.nq = d->nq;
  P.np_wo = d->np_wo; P.np_w = d->np_w; P.level = d->level; P.flags = d->flags;
  P.group = 0; P.wall = 0;
  P.pos[0] = d->pos[0]; P.pos[1] = d->pos[1];
  P.size[0] = d->size[0]; P.size[1] = d->size[1];
  c->h_len[slot] = len;
  c->used[slot] = 1;
  pcg::PatchTimeDev t{};
  const double big = 1.7976931348623157e308;
  t.rl[0] = t.rl[1] = big;
  t.ru[0] = t.ru[1] = -big;
  // pageable source: the copy is staged before cudaMemcpyAsync returns
  PCG_CUDA(cudaMemcpyAsync(c->d_times + slot, &t, sizeof(t), cudaMemcpyHostToDevice, c->stream));
  c->patches_dirty = c->topo_dirty = true;
  c->slot_hint = slot + 1;
  if (slot + 1 > c->patch_hw) c->patch_hw = slot + 1;
  *id = slot;
  return PCG_OK;
}

int pcg_patch_free(pcg_context *c, int32_t id) {
  if (!valid_id(c, id)) return fail(PCG_E_INVALID, "unknown patch id");
  std::lock_guard<std::mutex> lk(c->mu);
  PCG_SETTLE(c);
  c->fin_dirty = true;
  PCG_CUDA(cudaStreamSynchronize(c->stream));
  slab_free(c, c->h_patches[id].off, c->h_len[id]);
  c->used[id] = 0;
  if (id < c->slot_hint) c->slot_hint = id;
  c->h_patches[id] = pcg::PatchDev{};
  c->patches_dirty = c->topo_dirty = true;
  return PCG_OK;
}

int pcg_patch_upload(pcg_context *c, int32_t id, const double *vec, int64_t n) {
  if (!valid_id(c, id) || !vec) return fail(PCG_E_INVALID, "unknown patch id or null vector");
  if (n != c->h_len[id]) return fail(PCG_E_INVALID, "vector length does not match the patch layout");
  std::lock_guard<std::mutex> lk(c->mu);
  PCG_SETTLE(c);
  c->fin_dirty = true;
  PCG_CUDA(cudaMemcpyAsync(c->slab + c->h_patches[id].off, vec, sizeof(double) * n,
                           cudaMemcpyHostToDevice, c->stream));
  PCG_CUDA(cudaStreamSynchronize(c->stream));
  return PCG_OK;
}

int pcg_patch_download(pcg_context *c, int32_t id, double *vec, int64_t n) {
  if (!valid_id(c, id) || !vec) return fail(PCG_E_INVALID, "unknown patch id or null vector");
  if (n != c->h_len[id]) return fail(PCG_E_INVALID, "vector length does not match the patch layout");
  std::lock_guard<std::mutex> lk(c->mu);
  PCG_SETTLE(c);
  PCG_CUDA(cudaMemcpyAsync(vec, c->slab + c->h_patches[id].off, sizeof(double) * n,
                           cudaMemcpyDeviceToHost, c->stream));
  PCG_CUDA(cudaStreamSynchronize(c->stream));
  return PCG_OK;
}

int pcg_patches_upload(pcg_context *c, int32_t n, const int32_t *ids, const double *vecs) {
  if (!c || (n > 0 && (!ids || !vecs))) return fail(PCG_E_INVALID, "null argument");
  std::lock_guard<std::mutex> lk(c->mu);
  PCG_SETTLE(c);
  c->fin_dirty = true;
  return multi_copy(c, n, ids, const_cast<double *>(vecs), true);
}

int pcg_patches_download(pcg_context *c, int32_t n, const int32_t *ids, double *vecs) {
  if (!c || (n > 0 && (!ids || !vecs))) return fail(PCG_E_INVALID, "null argument");
  std::lock_guard<std::mutex> lk(c->mu);
  PCG_SETTLE(c);
  return multi_copy(c, n, ids, vecs, false);
}

int pcg_patch_set_desc_flags(pcg_context *c, int32_t id, int32_t flags) {
  if (!valid_id(c, id)) return fail(PCG_E_INVALID, "unknown patch id");
  std::lock_guard<std::mutex> lk(c->mu);
  PCG_SETTLE(c);
  c->fin_dirty = true;
  c->h_patches[id].flags = flags;
  c->patches_dirty = c->topo_dirty = true;
  return PCG_OK;
}

int pcg_patch_set_time(pcg_context *c, int32_t id, const pcg_patch_time *t) {
  if (!valid_id(c, id) || !t) return fail(PCG_E_INVALID, "unknown patch id or null time");
  std::lock_guard<std::mutex> lk(c->mu);
  PCG_SETTLE(c);
  pcg::PatchTimeDev d{};
  d.time = t->time; d.dt = t->dt; d.est_next = t->est_next;
  d.min_nb_time = t->min_neighbor_time; d.max_nb_dt = t->max_neighbor_dt;
  d.rl[0] = t->restr_lower[0]; d.rl[1] = t->restr_lower[1];
  d.ru[0] = t->restr_upper[0]; d.ru[1] = t->restr_upper[1];
  PCG_CUDA(cudaMemcpyAsync(c->d_times + id, &d, sizeof(d), cudaMemcpyHostToDevice, c->stream));
  PCG_CUDA(cudaStreamSynchronize(c->stream));
  c->restr_geo_dirty = true;
  return PCG_OK;
}

int pcg_patch_get_time(pcg_context *c, int32_t id, pcg_patch_time *t) {
  if (!valid_id(c, id) || !t) return fail(PCG_E_INVALID, "unknown patch id or null time");
  pcg::PatchTimeDev d;
  PCG_CUDA(cudaMemcpyAsync(&d, c->d_times + id, sizeof(d), cudaMemcpyDeviceToHost, c->stream));
  PCG_CUDA(cudaStreamSynchronize(c->stream));
  t->time = d.time; t->dt = d.dt; t->est_next = d.est_next;
  t->min_neighbor_time = d.min_nb_time; t->max_neighbor_dt = d.max_nb_dt;
  t->restr_lower[0] = d.rl[0]; t->restr_lower[1] = d.rl[1];
  t->restr_upper[0] = d.ru[0]; t->restr_upper[1] = d.ru[1];
  return PCG_OK;
}

int pcg_patch_set_boundary(pcg_context *c, int32_t id, uint32_t wall_mask) {
  if (!valid_id(c, id)) return fail(PCG_E_INVALID, "unknown patch id");
  if (wall_mask > 15u) return fail(PCG_E_INVALID, "wall mask has 4 bits in 2D");
  std::lock_guard<std::mutex> lk(c->mu);
  PCG_SETTLE(c);
  c->h_patches[id].wall = (int)wall_mask;
  c->patches_dirty = c->topo_dirty = true;
  return PCG_OK;
}

int pcg_patch_set_group(pcg_context *c, int32_t id, int32_t group) {
  if (!valid_id(c, id)) return fail(PCG_E_INVALID, "unknown patch id");
  if (group < 0 || group >= c->max_groups) return fail(PCG_E_INVALID, "group out of range");
  std::lock_guard<std::mutex> lk(c->mu);
  PCG_SETTLE(c);
  c->h_patches[id].group = group;
  c->patches_dirty = c->topo_dirty = true;
  c->graph_valid = false;
  return PCG_OK;
}

// ---------------------------------------------------------------- single ops

int pcg_copy_unew_to_uold(pcg_context *c, int32_t id) {
  if (!valid_id(c, id)) return fail(PCG_E_INVALID, "unknown patch id");
  std::lock_guard<std::mutex> lk(c->mu);
  PCG_SETTLE(c);
  c->fin_dirty = true;
  int rc = upload_patches(c);
  if (rc != PCG_OK) return rc;
  const pcg::PatchDev &P = c->h_patches[id];
  PCG_CUDA(pcg::launch_copy_unew_to_uold(c->stream, c->slab, c->d_patches, id, P.nq * P.nx * P.ny));
  return PCG_OK;
}

int pcg_swap_unew_and_uold(pcg_context *c, int32_t id) {
  if (!valid_id(c, id)) return fail(PCG_E_INVALID, "unknown patch id");
  std::lock_guard<std::mutex> lk(c->mu);
  PCG_SETTLE(c);
  c->fin_dirty = true;
  int rc = upload_patches(c);
  if (rc != PCG_OK) return rc;
  const pcg::PatchDev &P = c->h_patches[id];
  PCG_CUDA(pcg::launch_swap_unew_uold(c->stream, c->slab, c->d_patches, id, P.nq * P.nx * P.ny));
  return PCG_OK;
}

int pcg_fill_boundary_layer(pcg_context *c, int32_t id, int32_t dimension, int32_t set_upper) {
  if (!valid_id(c, id) || dimension < 0 || dimension > 1) return fail(PCG_E_INVALID, "bad patch or dimension");
  if (c->h_patches[id].g != 1 || c->h_patches[id].nq < 3)
    return fail(PCG_E_INVALID, "SWE wall boundary needs ghost width 1 and 3 unknowns");
  std::lock_guard<std::mutex> lk(c->mu);
  PCG_SETTLE(c);
  c->fin_dirty = true;
  int rc = upload_patches(c);
  if (rc != PCG_OK) return rc;
  PCG_CUDA(pcg::launch_fill_boundary_layer(c->stream, c->slab, c->d_patches, id, dimension, set_upper ? 1 : 0));
  return PCG_OK;
}

int pcg_solve_timestep(pcg_context *c, int32_t id, double max_dt, double *dt_used, double *est_next) {
  if (!valid_id(c, id)) return fail(PCG_E_INVALID, "unknown patch id");
  const pcg::PatchDev &P = c->h_patches[id];
  if (P.g != 1 || P.nq != 3 || P.np_w < 1)
    return fail(PCG_E_INVALID, "SWE solve needs ghost width 1, 3 unknowns and the bathymetry parameter");
  size_t smem = pcg::solve_patch_smem(P.nx, P.ny);
  if (smem > 190 * 1024) return fail(PCG_E_INVALID, "patch too large for the fused per-patch solve");
  std::lock_guard<std::mutex> lk(c->mu);
  PCG_SETTLE(c);
  c->fin_dirty = true;
  int rc = upload_patches(c);
  if (rc != PCG_OK) return rc;
  if (smem > c->solve_smem_set) {
    PCG_CUDA(pcg::prepare_solve_patch(190 * 1024));
    c->solve_smem_set = 190 * 1024;
  }
  PCG_CUDA(pcg::launch_solve_patch(c->stream, c->slab, c->d_patches, c->d_times, id, P.nx, P.ny, c->prm,
                                   max_dt, c->d_solve_out));
  PCG_CUDA(cudaMemcpyAsync(c->h_pinned, c->d_solve_out, 2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  PCG_CUDA(cudaStreamSynchronize(c->stream));
  if (dt_used) *dt_used = c->h_pinned[0];
  if (est_next) *est_next = c->h_pinned[1];
  return PCG_OK;
}

int pcg_transfer_ghostlayer(pcg_context *c, const int32_t size[2], const int32_t so[2],
                            const int32_t dof[2], int32_t src, int32_t dst) {
  if (!valid_id(c, src) || !valid_id(c, dst) || !size || !so || !dof) return fail(PCG_E_INVALID, "bad argument");
  const pcg::PatchDev &S = c->h_patches[src], &D = c->h_patches[dst];
  if (S.nq != D.nq) return fail(PCG_E_INVALID, "unknowns per subcell differ");
  if (!region_inside(S, so, size, false) || !region_inside(D, dof, size, true))
    return fail(PCG_E_INVALID, "transfer region outside the patches");
  std::lock_guard<std::mutex> lk(c->mu);
  PCG_SETTLE(c);
  c->fin_dirty = true;
  int rc = upload_patches(c);
  if (rc != PCG_OK) return rc;
  PCG_CUDA(pcg::launch_transfer(c->stream, c->slab, c->d_patches, c->d_times,
                                make_item(0, size, so, dof, src, dst)));
  return PCG_OK;
}

int pcg_interpolate_solution(pcg_context *c, const int32_t size[2], const int32_t dof[2], int32_t src,
                             int32_t dst, int32_t to_uold, int32_t to_current_time,
                             int32_t use_time_unew_or_uold, int32_t swe) {
  if (!valid_id(c, src) || !valid_id(c, dst) || !size || !dof) return fail(PCG_E_INVALID, "bad argument");
  const pcg::PatchDev &S = c->h_patches[src], &D = c->h_patches[dst];
  if (S.nq != D.nq) return fail(PCG_E_INVALID, "unknowns per subcell differ");
  if (S.nx < 2 || S.ny < 2) return fail(PCG_E_INVALID, "source needs at least 2x2 cells");
  if (!region_inside(D, dof, size, to_uold != 0)) return fail(PCG_E_INVALID, "region outside the destination");
  if (swe && (S.np_w < 1 || D.np_w < 1)) return fail(PCG_E_INVALID, "SWE interpolation needs the bathymetry parameter");
  std::lock_guard<std::mutex> lk(c->mu);
  PCG_SETTLE(c);
  c->fin_dirty = true;
  int rc = upload_patches(c);
  if (rc != PCG_OK) return rc;
  PCG_CUDA(pcg::launch_interpolate(c->stream, c->slab, c->d_patches, c->d_times,
                                   make_item(1, size, nullptr, dof, src, dst), to_uold, to_current_time,
                                   use_time_unew_or_uold, swe));
  return PCG_OK;
}

int pcg_interpolate_solution_many(pcg_context *c, int32_t n, const int32_t *src, const int32_t *dst,
                                  const int32_t *size, const int32_t *dof, int32_t to_uold, int32_t to_current_time,
                                  int32_t use_time_unew_or_uold, int32_t swe) {
  if (!c || n < 0 || (n > 0 && (!src || !dst || !size || !dof))) return fail(PCG_E_INVALID, "bad arguments");
  if (n == 0) return PCG_OK;
  std::vector<pcg::GhostItemDev> items(n);
  std::vector<char> seen(c->max_patches, 0);
  for (int32_t k = 0; k < n; k++) {
    if (!valid_id(c, src[k]) || !valid_id(c, dst[k]))
      return fail(PCG_E_INVALID, "interpolation " + std::to_string(k) + ": unknown patch id");
    if (seen[dst[k]]) return fail(PCG_E_INVALID, "interpolation " + std::to_string(k) + ": destination listed twice");
    seen[dst[k]] = 1;
    const pcg::PatchDev &S = c->h_patches[src[k]], &D = c->h_patches[dst[k]];
    if (S.nq != D.nq) return fail(PCG_E_INVALID, "interpolation " + std::to_string(k) + ": unknowns differ");
    if (S.nx < 2 || S.ny < 2) return fail(PCG_E_INVALID, "interpolation " + std::to_string(k) + ": source below 2x2");
    if (!region_inside(D, &dof[2 * k], &size[2 * k], to_uold != 0))
      return fail(PCG_E_INVALID, "interpolation " + std::to_string(k) + ": region outside the destination");
    if (swe && (S.np_w < 1 || D.np_w < 1))
      return fail(PCG_E_INVALID, "interpolation " + std::to_string(k) + ": needs the bathymetry parameter");
    items[k] = make_item(1, &size[2 * k], nullptr, &dof[2 * k], src[k], dst[k]);
  }
  for (int32_t k = 0; k < n; k++)
    if (seen[src[k]]) return fail(PCG_E_INVALID, "a destination is also a source");
  std::lock_guard<std::mutex> lk(c->mu);
  PCG_SETTLE(c);
  c->fin_dirty = true;
  PCG_CUDA(cudaSetDevice(c->device));
  int rc = upload_patches(c);
  if (rc != PCG_OK) return rc;
  rc = ensure_staging(c, (sizeof(pcg::GhostItemDev) * (size_t)n + 7) / 8, 0);
  if (rc != PCG_OK) return rc;
  pcg::GhostItemDev *d_items = reinterpret_cast<pcg::GhostItemDev *>(c->d_staging);
  PCG_CUDA(cudaMemcpyAsync(d_items, items.data(), sizeof(pcg::GhostItemDev) * (size_t)n, cudaMemcpyHostToDevice,
                           c->stream));
  PCG_CUDA(pcg::launch_interpolate_many(c->stream, c->slab, c->d_patches, c->d_times, d_items, n, to_uold,
                                        to_current_time, use_time_unew_or_uold, swe));
  PCG_CUDA(cudaStreamSynchronize(c->stream));
  return PCG_OK;
}

int pcg_patches_set_time(pcg_context *c, int32_t n, const int32_t *ids, const pcg_patch_time *in) {
  if (!c || n < 0 || (n > 0 && (!ids || !in))) return fail(PCG_E_INVALID, "bad arguments");
  if (n == 0) return PCG_OK;
  std::lock_guard<std::mutex> lk(c->mu);
  PCG_SETTLE(c);
  std::vector<char> seen(c->max_patches, 0);
  std::vector<long long> meta(n);
  std::vector<pcg::PatchTimeDev> rec(n);
  for (int32_t k = 0; k < n; k++) {
    if (!valid_id(c, ids[k])) return fail(PCG_E_INVALID, "unknown patch id " + std::to_string(ids[k]));
    if (seen[ids[k]]) return fail(PCG_E_INVALID, "patch id " + std::to_string(ids[k]) + " listed twice");
    seen[ids[k]] = 1;
    meta[k] = ids[k];
    pcg::PatchTimeDev d{};
    d.time = in[k].time; d.dt = in[k].dt; d.est_next = in[k].est_next;
    d.min_nb_time = in[k].min_neighbor_time; d.max_nb_dt = in[k].max_neighbor_dt;
    d.rl[0] = in[k].restr_lower[0]; d.rl[1] = in[k].restr_lower[1];
    d.ru[0] = in[k].restr_upper[0]; d.ru[1] = in[k].restr_upper[1];
    rec[k] = d;
  }
  PCG_CUDA(cudaSetDevice(c->device));
  int rc = ensure_staging(c, (sizeof(pcg::PatchTimeDev) * (size_t)n + 7) / 8, (size_t)n);
  if (rc != PCG_OK) return rc;
  PCG_CUDA(cudaMemcpyAsync(c->d_copy_meta, meta.data(), sizeof(long long) * (size_t)n, cudaMemcpyHostToDevice,
                           c->stream));
  PCG_CUDA(cudaMemcpyAsync(c->d_staging, rec.data(), sizeof(pcg::PatchTimeDev) * (size_t)n,
                           cudaMemcpyHostToDevice, c->stream));
  PCG_CUDA(pcg::launch_scatter_times(c->stream, c->d_copy_meta,
                                     reinterpret_cast<const pcg::PatchTimeDev *>(c->d_staging), n, c->d_times));
  PCG_CUDA(cudaStreamSynchronize(c->stream));
  c->restr_geo_dirty = true;
  return PCG_OK;
}

int pcg_restrict_solution(pcg_context *c, int32_t src, int32_t dst, int32_t only_overlapped, int32_t swe) {
  if (!valid_id(c, src) || !valid_id(c, dst)) return fail(PCG_E_INVALID, "unknown patch id");
  const pcg::PatchDev &S = c->h_patches[src], &D = c->h_patches[dst];
  if (S.nq != D.nq) return fail(PCG_E_INVALID, "unknowns per subcell differ");
  if (swe && S.np_w < 1) return fail(PCG_E_INVALID, "SWE restriction needs the bathymetry parameter");
  std::lock_guard<std::mutex> lk(c->mu);
  PCG_SETTLE(c);
  c->fin_dirty = true;
  int rc = upload_patches(c);
  if (rc != PCG_OK) return rc;
  PCG_CUDA(pcg::launch_restrict(c->stream, c->slab, c->d_patches, c->d_times, src, dst, only_overlapped, swe));
  return PCG_OK;
}

int pcg_post_process_restriction(pcg_context *c, int32_t dst) {
  if (!valid_id(c, dst)) return fail(PCG_E_INVALID, "unknown patch id");
  if (c->h_patches[dst].np_w < 1) return fail(PCG_E_INVALID, "needs the bathymetry parameter");
  std::lock_guard<std::mutex> lk(c->mu);
  PCG_SETTLE(c);
  c->fin_dirty = true;
  int rc = upload_patches(c);
  if (rc != PCG_OK) return rc;
  int *ids = nullptr;
  size_t cap = 0;
  // one-element id list in the pinned-free path: reuse d_counter-sized scratch
  rc = ensure_device(c, &ids, &cap, 1);
  if (rc != PCG_OK) return rc;
  PCG_CUDA(cudaMemcpyAsync(ids, &dst, sizeof(int), cudaMemcpyHostToDevice, c->stream));
  PCG_CUDA(pcg::launch_post_process_restriction(c->stream, c->slab, c->d_patches, ids, 1));
  PCG_CUDA(cudaStreamSynchronize(c->stream));
  PCG_CUDA(cudaFree(ids));
  return PCG_OK;
}

int pcg_clear_subgrid(pcg_context *c, int32_t id) {
  if (!valid_id(c, id)) return fail(PCG_E_INVALID, "unknown patch id");
  std::lock_guard<std::mutex> lk(c->mu);
  PCG_SETTLE(c);
  c->fin_dirty = true;
  int rc = upload_patches(c);
  if (rc != PCG_OK) return rc;
  int *ids = nullptr;
  size_t cap = 0;
  rc = ensure_device(c, &ids, &cap, 1);
  if (rc != PCG_OK) return rc;
  PCG_CUDA(cudaMemcpyAsync(ids, &id, sizeof(int), cudaMemcpyHostToDevice, c->stream));
  PCG_CUDA(pcg::launch_clear_interior(c->stream, c->slab, c->d_patches, ids, 1));
  PCG_CUDA(cudaStreamSynchronize(c->stream));
  PCG_CUDA(cudaFree(ids));
  return PCG_OK;
}

int pcg_gather_cells(pcg_context *c, int32_t n, const int32_t *ids, double *out, int64_t out_len) {
  if (!c || n < 0 || (n > 0 && (!ids || !out))) return fail(PCG_E_INVALID, "bad arguments");
  std::vector<long long> off(n);
  int64_t total = 0;
  for (int32_t k = 0; k < n; k++) {
    if (!valid_id(c, ids[k])) return fail(PCG_E_INVALID, "unknown patch id " + std::to_string(ids[k]));
    const pcg::PatchDev &P = c->h_patches[ids[k]];
    off[k] = total;
    total += (int64_t)(P.nq + P.np_w) * P.nx * P.ny;
  }
  if (total != out_len) return fail(PCG_E_INVALID, "out_len must be " + std::to_string(total));
  if (n == 0) return PCG_OK;
  std::lock_guard<std::mutex> lk(c->mu);
  PCG_SETTLE(c);
  PCG_CUDA(cudaSetDevice(c->device));
  int rc = upload_patches(c);
  if (rc != PCG_OK) return rc;
  int *d_ids = nullptr;
  long long *d_off = nullptr;
  double *d_out = nullptr;
  cudaError_t e = cudaMalloc(&d_ids, sizeof(int) * n);
  if (e == cudaSuccess) e = cudaMalloc(&d_off, sizeof(long long) * n);
  if (e == cudaSuccess) e = cudaMalloc(&d_out, sizeof(double) * total);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_ids, ids, sizeof(int) * n, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_off, off.data(), sizeof(long long) * n, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = pcg::launch_gather_cells(c->stream, c->slab, c->d_patches, d_ids, d_off, n, d_out);
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, d_out, sizeof(double) * total, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  cudaFree(d_ids);
  cudaFree(d_off);
  cudaFree(d_out);
  if (e != cudaSuccess) return fail(PCG_E_CUDA, std::string("pcg_gather_cells: ") + cudaGetErrorString(e));
  return PCG_OK;
}

int pcg_patches_get_time(pcg_context *c, int32_t n, const int32_t *ids, pcg_patch_time *out) {
  if (!c || n < 0 || (n > 0 && (!ids || !out))) return fail(PCG_E_INVALID, "bad arguments");
  for (int32_t k = 0; k < n; k++)
    if (!valid_id(c, ids[k])) return fail(PCG_E_INVALID, "unknown patch id " + std::to_string(ids[k]));
  if (n == 0) return PCG_OK;
  std::lock_guard<std::mutex> lk(c->mu);
  PCG_CUDA(cudaSetDevice(c->device));
  // every listed id is in use, so below the high-water mark
  std::vector<pcg::PatchTimeDev> all(c->patch_hw);
  PCG_CUDA(cudaMemcpyAsync(all.data(), c->d_times, sizeof(pcg::PatchTimeDev) * (size_t)c->patch_hw,
                           cudaMemcpyDeviceToHost, c->stream));
  PCG_CUDA(cudaStreamSynchronize(c->stream));
  for (int32_t k = 0; k < n; k++) {
    const pcg::PatchTimeDev &T = all[ids[k]];
    out[k].time = T.time;
    out[k].dt = T.dt;
    out[k].est_next = T.est_next;
    out[k].min_neighbor_time = T.min_nb_time;
    out[k].max_neighbor_dt = T.max_nb_dt;
    out[k].restr_lower[0] = T.rl[0]; out[k].restr_lower[1] = T.rl[1];
    out[k].restr_upper[0] = T.ru[0]; out[k].restr_upper[1] = T.ru[1];
  }
  return PCG_OK;
}

int pcg_patches_set_restriction_bounds(pcg_context *c, int32_t n, const int32_t *ids, const double *lower,
                                       const double *upper) {
  if (!c || n < 0 || (n > 0 && (!ids || !lower || !upper))) return fail(PCG_E_INVALID, "bad arguments");
  if (n == 0) return PCG_OK;
  std::lock_guard<std::mutex> lk(c->mu);
  PCG_SETTLE(c);
  std::vector<char> seen(c->max_patches, 0);
  std::vector<long long> meta(n);
  std::vector<double> b(4 * (size_t)n);
  for (int32_t k = 0; k < n; k++) {
    if (!valid_id(c, ids[k])) return fail(PCG_E_INVALID, "unknown patch id " + std::to_string(ids[k]));
    if (seen[ids[k]]) return fail(PCG_E_INVALID, "patch id " + std::to_string(ids[k]) + " listed twice");
    seen[ids[k]] = 1;
    meta[k] = ids[k];
    b[4 * k] = lower[2 * k]; b[4 * k + 1] = lower[2 * k + 1];
    b[4 * k + 2] = upper[2 * k]; b[4 * k + 3] = upper[2 * k + 1];
  }
  PCG_CUDA(cudaSetDevice(c->device));
  int rc = ensure_staging(c, b.size(), (size_t)n);
  if (rc != PCG_OK) return rc;
  PCG_CUDA(cudaMemcpyAsync(c->d_copy_meta, meta.data(), sizeof(long long) * meta.size(), cudaMemcpyHostToDevice,
                           c->stream));
  PCG_CUDA(cudaMemcpyAsync(c->d_staging, b.data(), sizeof(double) * b.size(), cudaMemcpyHostToDevice, c->stream));
  k_scatter_bounds<<<std::min(1024, (n + 255) / 256), 256, 0, c->stream>>>(c->d_copy_meta, c->d_staging, n,
                                                                             c->d_times);
  PCG_CUDA(cudaGetLastError());
  PCG_CUDA(cudaStreamSynchronize(c->stream));
  c->restr_geo_dirty = true;
  return PCG_OK;
}

int pcg_switch_to_leaf(pcg_context *c, int32_t id) {
  if (!valid_id(c, id)) return fail(PCG_E_INVALID, "unknown patch id");
  std::lock_guard<std::mutex> lk(c->mu);
  PCG_SETTLE(c);
  c->fin_dirty = true;
  PCG_CUDA(cudaSetDevice(c->device));
  pcg::PatchDev &P = c->h_patches[id];
  P.flags = (P.flags & ~pcg::kFlagVirtual) | pcg::kFlagLeaf;
  c->patches_dirty = true;
  c->topo_dirty = true;
  c->graph_valid = false;
  int rc = upload_patches(c);
  if (rc != PCG_OK) return rc;
  PCG_CUDA(pcg::launch_switch_to_leaf(c->stream, c->slab, c->d_patches, c->d_times, id));
  PCG_CUDA(cudaStreamSynchronize(c->stream));
  return PCG_OK;
}

int pcg_refinement_indicator(pcg_context *c, int32_t n, const int32_t *ids, double *out) {
  return pcg_refinement_criterion(c, n, ids, PCG_CRIT_DEPTH_GRADIENT, out);
}

int pcg_refinement_criterion(pcg_context *c, int32_t n, const int32_t *ids, int32_t kind, double *out) {
  if (!c || n < 0 || (n > 0 && (!ids || !out))) return fail(PCG_E_INVALID, "bad arguments");
  if (kind != PCG_CRIT_DEPTH_GRADIENT && kind != PCG_CRIT_SURFACE_DIFFERENCE && kind != PCG_CRIT_SURFACE_GRADIENT)
    return fail(PCG_E_INVALID, "unknown refinement criterion " + std::to_string(kind));
  for (int32_t k = 0; k < n; k++) {
    if (!valid_id(c, ids[k])) return fail(PCG_E_INVALID, "unknown patch id " + std::to_string(ids[k]));
    if (c->h_patches[ids[k]].nq < 1) return fail(PCG_E_INVALID, "patch without unknowns");
    if (kind != PCG_CRIT_DEPTH_GRADIENT && c->h_patches[ids[k]].np_w < 1)
      return fail(PCG_E_INVALID, "the surface criteria need the bathymetry parameter");
  }
  if (n == 0) return PCG_OK;
  std::lock_guard<std::mutex> lk(c->mu);
  PCG_SETTLE(c);
  PCG_CUDA(cudaSetDevice(c->device));
  int rc = upload_patches(c);
  if (rc != PCG_OK) return rc;
  int *d_ids = nullptr;
  double *d_out = nullptr;
  PCG_CUDA(cudaMalloc(&d_ids, sizeof(int) * n));
  cudaError_t e = cudaMalloc(&d_out, sizeof(double) * n);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_ids, ids, sizeof(int) * n, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = pcg::launch_refinement_indicator(c->stream, c->slab, c->d_patches, d_ids, n, kind, d_out);
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, d_out, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  cudaFree(d_ids);
  cudaFree(d_out);
  if (e != cudaSuccess) return fail(PCG_E_CUDA, std::string("pcg_refinement_indicator: ") + cudaGetErrorString(e));
  return PCG_OK;
}

int pcg_compute_fluxes(pcg_context *c, int32_t id, double g_flux) {
  if (!valid_id(c, id)) return fail(PCG_E_INVALID, "unknown patch id");
  if (c->h_patches[id].nq != 3 || c->h_patches[id].g < 1)
    return fail(PCG_E_INVALID, "flux computation needs 3 unknowns and a ghost layer");
  std::lock_guard<std::mutex> lk(c->mu);
  PCG_SETTLE(c);
  c->fin_dirty = true;
  int rc = upload_patches(c);
  if (rc != PCG_OK) return rc;
  int *ids = nullptr;
  size_t cap = 0;
  rc = ensure_device(c, &ids, &cap, 1);
  if (rc != PCG_OK) return rc;
  PCG_CUDA(cudaMemcpyAsync(ids, &id, sizeof(int), cudaMemcpyHostToDevice, c->stream));
  PCG_CUDA(pcg::launch_compute_fluxes(c->stream, c->slab, c->d_patches, ids, 1, g_flux));
  PCG_CUDA(cudaStreamSynchronize(c->stream));
  PCG_CUDA(cudaFree(ids));
  return PCG_OK;
}

int pcg_apply_flux_correction(pcg_context *c, int32_t src, int32_t dst, int32_t dimension, int32_t direction) {
  if (!valid_id(c, src) || !valid_id(c, dst)) return fail(PCG_E_INVALID, "unknown patch id");
  if (dimension < 0 || dimension > 1 || (direction != 1 && direction != -1))
    return fail(PCG_E_INVALID, "bad dimension/direction");
  if (c->h_patches[src].nq != 3 || c->h_patches[dst].nq != 3) return fail(PCG_E_INVALID, "needs 3 unknowns");
  std::lock_guard<std::mutex> lk(c->mu);
  PCG_SETTLE(c);
  c->fin_dirty = true;
  int rc = upload_patches(c);
  if (rc != PCG_OK) return rc;
  PCG_CUDA(pcg::launch_flux_correction(c->stream, c->slab, c->d_patches, c->d_times, src, dst, dimension, direction));
  return PCG_OK;
}

// ---------------------------------------------------------------- batched

int pcg_set_ghost_items(pcg_context *c, const pcg_ghost_item *items, int32_t n) {
  if (!c || n < 0 || (n > 0 && !items)) return fail(PCG_E_INVALID, "bad item list");
  std::lock_guard<std::mutex> lk(c->mu);
  PCG_SETTLE(c);
  for (int k = 0; k < n; k++) {
    const pcg_ghost_item &it = items[k];
    if (!valid_id(c, it.src) || !valid_id(c, it.dst) || (it.kind != 0 && it.kind != 1))
      return fail(PCG_E_INVALID, "ghost item " + std::to_string(k) + ": bad ids or kind");
    const pcg::PatchDev &S = c->h_patches[it.src], &D = c->h_patches[it.dst];
    if (S.nq != D.nq) return fail(PCG_E_INVALID, "ghost item " + std::to_string(k) + ": unknowns differ");
    if (!region_inside(D, it.dst_offset, it.size, true) ||
        (it.kind == 0 && !region_inside(S, it.src_offset, it.size, false)))
      return fail(PCG_E_INVALID, "ghost item " + std::to_string(k) + ": region outside the patches");
    if (it.kind == 1 && (S.nx < 2 || S.ny < 2 || S.np_w < 1 || D.np_w < 1 || S.nq != 3))
      return fail(PCG_E_INVALID, "ghost item " + std::to_string(k) + ": interpolation source unsupported");
  }
  c->items_user.assign(items, items + n);
  c->topo_dirty = true;
  return PCG_OK;
}

int pcg_set_restriction_items(pcg_context *c, int32_t n, const int32_t *src, const int32_t *dst,
                              int32_t only_overlapped) {
  if (!c || n < 0 || (n > 0 && (!src || !dst))) return fail(PCG_E_INVALID, "bad restriction list");
  std::lock_guard<std::mutex> lk(c->mu);
  PCG_SETTLE(c);
  std::vector<int4> v;
  for (int k = 0; k < n; k++) {
    if (!valid_id(c, src[k]) || !valid_id(c, dst[k]) || src[k] == dst[k])
      return fail(PCG_E_INVALID, "restriction item " + std::to_string(k) + ": bad ids");
    const pcg::PatchDev &S = c->h_patches[src[k]], &D = c->h_patches[dst[k]];
    if (S.nq != D.nq || S.np_w < 1 || D.np_w < 1)
      return fail(PCG_E_INVALID, "restriction item " + std::to_string(k) + ": not SWE patches");
    v.push_back(make_int4(src[k], dst[k], only_overlapped ? 1 : 0, 1));
  }
  c->restr_user = v;
  c->topo_dirty = true;
  return PCG_OK;
}

int pcg_set_flux_correction_items(pcg_context *c, int32_t n, const int32_t *src, const int32_t *dst,
                                  const int32_t *dim, const int32_t *dir, double g_flux) {
  if (!c || n < 0 || (n > 0 && (!src || !dst || !dim || !dir))) return fail(PCG_E_INVALID, "bad flux list");
  std::lock_guard<std::mutex> lk(c->mu);
  PCG_SETTLE(c);
  std::vector<int4> v;
  for (int k = 0; k < n; k++) {
    if (!valid_id(c, src[k]) || !valid_id(c, dst[k]) || dim[k] < 0 || dim[k] > 1 || (dir[k] != 1 && dir[k] != -1))
      return fail(PCG_E_INVALID, "flux item " + std::to_string(k) + ": bad arguments");
    if (c->h_patches[src[k]].nq != 3 || c->h_patches[dst[k]].nq != 3)
      return fail(PCG_E_INVALID, "flux item " + std::to_string(k) + ": needs 3 unknowns");
    v.push_back(make_int4(src[k], dst[k], dim[k], dir[k]));
  }
  c->flux_user = v;
  c->g_flux = g_flux;
  c->topo_dirty = true;
  return PCG_OK;
}

int pcg_restrict_all(pcg_context *c) {
  if (!c) return fail(PCG_E_INVALID, "null context");
  std::lock_guard<std::mutex> lk(c->mu);
  PCG_SETTLE(c);
  c->fin_dirty = true;
  PCG_CUDA(cudaSetDevice(c->device));
  int rc = rebuild_topology(c);
  if (rc != PCG_OK) return rc;
  // every destination, whatever the groups' and leaves' state
  if ((rc = enqueue_level_transfer(c, false, true, nullptr, nullptr)) != PCG_OK) return rc;
  PCG_CUDA(cudaStreamSynchronize(c->stream));
  return check_level_transfer(c);
}

int pcg_set_group_end_time(pcg_context *c, int32_t group, double time, double t_end) {
  if (!c || group < 0 || group >= c->max_groups) return fail(PCG_E_INVALID, "group out of range");
  std::lock_guard<std::mutex> lk(c->mu);
  PCG_SETTLE(c);
  PCG_CUDA(cudaSetDevice(c->device));
  c->h_pinned[0] = time;
  c->h_pinned[1] = t_end;
  PCG_CUDA(cudaMemcpyAsync(c->d_group_time + group, c->h_pinned, sizeof(double), cudaMemcpyHostToDevice,
                           c->stream));
  PCG_CUDA(cudaMemcpyAsync(c->d_group_t_end + group, c->h_pinned + 1, sizeof(double),
                           cudaMemcpyHostToDevice, c->stream));
  PCG_CUDA(cudaStreamSynchronize(c->stream));
  return PCG_OK;
}

int pcg_get_group_times(pcg_context *c, double *times) {
  if (!c || !times) return fail(PCG_E_INVALID, "null argument");
  std::lock_guard<std::mutex> lk(c->mu);
  PCG_CUDA(cudaSetDevice(c->device));
  PCG_CUDA(cudaMemcpyAsync(times, c->d_group_time, sizeof(double) * c->max_groups, cudaMemcpyDeviceToHost,
                           c->stream));
  PCG_CUDA(cudaStreamSynchronize(c->stream));
  return PCG_OK;
}

int pcg_set_group_max_dt(pcg_context *c, int32_t group, double max_dt) {
  if (!c || group < 0 || group >= c->max_groups) return fail(PCG_E_INVALID, "group out of range");
  std::lock_guard<std::mutex> lk(c->mu);
  c->fused_ready = false;
  c->h_group_max_dt[group] = max_dt;
  return PCG_OK;
}

static int check_solvable(pcg_context *c) {
  for (int p : c->leaf_ids) {
    const pcg::PatchDev &P = c->h_patches[p];
    if (P.g != 1 || P.nq != 3 || P.np_w < 1)
      return fail(PCG_E_INVALID, "leaf patch " + std::to_string(p) + " is not an SWE patch (ghost 1, 3 unknowns, b)");
    if (P.nx > 32767 || P.ny > 32767)  // tile / strip coordinates are 16-bit
      return fail(PCG_E_INVALID, "leaf patch " + std::to_string(p) + " has more than 32767 cells per edge");
  }
  return PCG_OK;
}

// Local time stepping runs in the batched form only, without a
// flux-correction list; the virtual-time pairs must join a leaf to a
// non-leaf patch.
static int check_mode(pcg_context *c, int mode) {
  if (!c->ts_local) return PCG_OK;
  if (mode != PCG_MODE_BATCHED) return fail(PCG_E_STATE, "local time stepping runs in the batched form only");
  if (!c->h_flux.empty()) return fail(PCG_E_STATE, "local time stepping takes no flux-correction list");
  for (size_t k = 0; k < c->h_vt.size(); k++) {
    const int2 pr = c->h_vt[k];
    if (!(c->h_patches[pr.x].flags & pcg::kFlagLeaf) || (c->h_patches[pr.y].flags & pcg::kFlagLeaf))
      return fail(PCG_E_STATE, "virtual-time item " + std::to_string(k) + " does not join a leaf to a non-leaf patch");
  }
  return PCG_OK;
}

int pcg_set_virtual_time_items(pcg_context *c, int32_t n, const int32_t *leaf, const int32_t *virt) {
  if (!c || n < 0 || (n > 0 && (!leaf || !virt))) return fail(PCG_E_INVALID, "bad virtual-time list");
  std::lock_guard<std::mutex> lk(c->mu);
  PCG_SETTLE(c);
  std::vector<int2> v;
  v.reserve(n);
  for (int k = 0; k < n; k++) {
    if (!valid_id(c, leaf[k]) || !valid_id(c, virt[k]) || leaf[k] == virt[k])
      return fail(PCG_E_INVALID, "virtual-time item " + std::to_string(k) + ": bad ids");
    v.push_back(make_int2(leaf[k], virt[k]));
  }
  c->vt_user = v;
  c->topo_dirty = true;
  return PCG_OK;
}

int pcg_set_time_stepping(pcg_context *c, int32_t mode) {
  if (!c || (mode != PCG_TS_GLOBAL && mode != PCG_TS_LOCAL)) return fail(PCG_E_INVALID, "bad time-stepping mode");
  std::lock_guard<std::mutex> lk(c->mu);
  if (c->run_pending) return fail(PCG_E_STATE, "a run started by pcg_run_async is still pending");
  PCG_SETTLE(c);
  const bool local = mode == PCG_TS_LOCAL;
  if (local != c->ts_local) {
    c->ts_local = local;
    c->graph_valid = false;
    c->topo_dirty = true;  // the fused form's tables depend on it
  }
  return PCG_OK;
}

int pcg_step(pcg_context *c, int32_t mode, double *dt_out) {
  if (!c || (mode != PCG_MODE_PLAIN && mode != PCG_MODE_BATCHED)) return fail(PCG_E_INVALID, "bad mode");
  std::lock_guard<std::mutex> lk(c->mu);
  if (c->run_pending) return fail(PCG_E_STATE, "a run started by pcg_run_async is still pending");
  PCG_CUDA(cudaSetDevice(c->device));
  int rc = rebuild_topology(c);
  if (rc != PCG_OK) return rc;
  if ((rc = check_solvable(c)) != PCG_OK) return rc;
  if ((rc = check_mode(c, mode)) != PCG_OK) return rc;
  if ((rc = upload_group_max_dt(c)) != PCG_OK) return rc;
  const bool fused = use_fused(c, mode);
  if (fused) {
    if ((rc = ensure_hist(c, 1)) != PCG_OK) return rc;
    PCG_CUDA(cudaMemsetAsync(c->d_counter, 0, sizeof(int), c->stream));
    PCG_CUDA(cudaEventRecord(c->ev0, c->stream));
    if ((rc = fused_prologue(c)) != PCG_OK) return rc;
    rc = enqueue_fused_step(c, mode);
    c->fused_pending = true;
    if (rc != PCG_OK) return rc;
    PCG_CUDA(cudaEventRecord(c->ev1, c->stream));
    PCG_CUDA(cudaMemcpyAsync(c->h_pinned, c->d_hist, sizeof(double) * c->max_groups, cudaMemcpyDeviceToHost,
                             c->stream));
  } else {
    PCG_SETTLE(c);
    if ((rc = refresh_fin(c)) != PCG_OK) return rc;
    PCG_CUDA(cudaEventRecord(c->ev0, c->stream));
    if ((rc = enqueue_step(c, mode)) != PCG_OK) return rc;
    PCG_CUDA(cudaEventRecord(c->ev1, c->stream));
    PCG_CUDA(pcg::launch_record_dt(c->stream, c->max_groups, c->d_group_dt, c->d_dt_out));
    PCG_CUDA(cudaMemcpyAsync(c->h_pinned, c->d_dt_out, sizeof(double) * c->max_groups, cudaMemcpyDeviceToHost,
                             c->stream));
  }
  PCG_CUDA(cudaStreamSynchronize(c->stream));
  {
    const int xrc = check_level_transfer(c);
    if (xrc != PCG_OK) return xrc;
  }
  float ms = 0.f;
  PCG_CUDA(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
  c->device_ms += ms;
  if (!c->ts_local) c->cell_updates += c->cells_per_step;
  if (dt_out) std::memcpy(dt_out, c->h_pinned, sizeof(double) * c->max_groups);
  return PCG_OK;
}

// Kernel nodes of a captured graph (the launches one replay issues).
static int count_kernel_nodes(cudaGraph_t g) {
  size_t n = 0;
  if (cudaGraphGetNodes(g, nullptr, &n) != cudaSuccess || n == 0) return 0;
  std::vector<cudaGraphNode_t> nodes(n);
  if (cudaGraphGetNodes(g, nodes.data(), &n) != cudaSuccess) return 0;
  int k = 0;
  for (size_t i = 0; i < n; i++) {
    cudaGraphNodeType t;
    if (cudaGraphNodeGetType(nodes[i], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) k++;
  }
  return k;
}

namespace {

// The launches of a run of `steps` steps (caller holds the context lock);
// run_finish completes it.
int run_enqueue(pcg_context *c, int32_t steps, int32_t mode) {
  PCG_CUDA(cudaSetDevice(c->device));
  int rc = rebuild_topology(c);
  if (rc != PCG_OK) return rc;
  if ((rc = check_solvable(c)) != PCG_OK) return rc;
  if ((rc = check_mode(c, mode)) != PCG_OK) return rc;
  if ((rc = upload_group_max_dt(c)) != PCG_OK) return rc;
  const bool fused = use_fused(c, mode);
  const bool pipe = !fused && use_pipeline(c, mode);
  if (!fused) {
    PCG_SETTLE(c);
    if ((rc = refresh_fin(c)) != PCG_OK) return rc;
    if ((rc = refresh_restr_geometry(c)) != PCG_OK) return rc;
    // (built outside the graph capture: they allocate)
    if (c->sched.kind == PCG_SCHED_TILES && c->sched.variant == 1 && (rc = ensure_tile_maps(c)) != PCG_OK)
      return rc;
    if (pipe && !c->pipe_valid && (rc = build_pipeline(c)) != PCG_OK) return rc;
  }
  if ((rc = ensure_hist(c, steps)) != PCG_OK) return rc;
  PCG_CUDA(cudaMemsetAsync(c->d_counter, 0, sizeof(int), c->stream));
  int threads = std::min(1024, std::max(32, (c->max_groups + 31) / 32 * 32));
  if (fused) {
    PCG_CUDA(cudaEventRecord(c->ev0, c->stream));
    if ((rc = fused_prologue(c)) != PCG_OK) return rc;
    if (mode == PCG_MODE_BATCHED) {
      if (!c->graph_valid || !c->graph_fused) {
        if (c->graph) { cudaGraphExecDestroy(c->graph); c->graph = nullptr; }
        c->graph_valid = false;
        cudaGraph_t g;
        PCG_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        int erc = enqueue_fused_step(c, PCG_MODE_BATCHED);
        cudaError_t ce = cudaStreamEndCapture(c->stream, &g);
        if (erc != PCG_OK) return erc;
        if (ce != cudaSuccess) return fail(PCG_E_CUDA, std::string("graph capture: ") + cudaGetErrorString(ce));
        c->graph_kernels = count_kernel_nodes(g);
        cudaError_t ie = cudaGraphInstantiate(&c->graph, g, 0);
        cudaGraphDestroy(g);
        if (ie != cudaSuccess) return fail(PCG_E_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ie));
        c->graph_valid = true;
        c->graph_fused = true;
        c->graph_pipe = false;
      }
      for (int s = 0; s < steps; s++) PCG_CUDA(cudaGraphLaunch(c->graph, c->stream));
    } else {
      for (int s = 0; s < steps; s++) {
        rc = enqueue_fused_step(c, PCG_MODE_PLAIN);
        c->fused_pending = true;
        if (rc != PCG_OK) return rc;
      }
    }
    c->fused_pending = true;
    PCG_CUDA(cudaEventRecord(c->ev1, c->stream));
  } else if (pipe) {
    if (!c->graph_valid || c->graph_fused || !c->graph_pipe) {
      if (c->graph) { cudaGraphExecDestroy(c->graph); c->graph = nullptr; }
      c->graph_valid = false;
      cudaGraph_t g;
      PCG_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
      int erc = enqueue_pipeline_launch(c);
      cudaError_t ce = cudaStreamEndCapture(c->stream, &g);
      if (erc != PCG_OK) return erc;
      if (ce != cudaSuccess) return fail(PCG_E_CUDA, std::string("graph capture: ") + cudaGetErrorString(ce));
      c->graph_kernels = count_kernel_nodes(g);
      cudaError_t ie = cudaGraphInstantiate(&c->graph, g, 0);
      cudaGraphDestroy(g);
      if (ie != cudaSuccess) return fail(PCG_E_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ie));
      c->graph_valid = true;
      c->graph_fused = false;
      c->graph_pipe = true;
    }
    if ((rc = start_pipeline_run(c, steps)) != PCG_OK) return rc;
    PCG_CUDA(cudaEventRecord(c->ev0, c->stream));
    for (int s = 0; s <= steps; s++) PCG_CUDA(cudaGraphLaunch(c->graph, c->stream));
    PCG_CUDA(cudaEventRecord(c->ev1, c->stream));
  } else if (mode == PCG_MODE_BATCHED) {
    if (!c->graph_valid || c->graph_fused || c->graph_pipe) {
      if (c->graph) { cudaGraphExecDestroy(c->graph); c->graph = nullptr; }
      c->graph_valid = false;
      cudaGraph_t g;
      PCG_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
      // the history kernel also advances the group times (one launch less);
      // local time stepping sets them in its own last phase
      int erc = enqueue_step(c, PCG_MODE_BATCHED, false);
      k_record_hist<<<1, threads, 0, c->stream>>>(c->max_groups, c->d_group_dt, c->d_hist, c->d_counter,
                                                 c->hist_cap, c->ts_local ? 0 : 1, c->d_group_active,
                                                 c->d_group_time);
      cudaError_t le = cudaGetLastError();
      cudaError_t ce = cudaStreamEndCapture(c->stream, &g);
      if (erc != PCG_OK) return erc;
      if (le != cudaSuccess) return fail(PCG_E_CUDA, cudaGetErrorString(le));
      if (ce != cudaSuccess) return fail(PCG_E_CUDA, std::string("graph capture: ") + cudaGetErrorString(ce));
      c->graph_kernels = count_kernel_nodes(g);
      cudaError_t ie = cudaGraphInstantiate(&c->graph, g, 0);
      cudaGraphDestroy(g);
      if (ie != cudaSuccess) return fail(PCG_E_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ie));
      c->graph_valid = true;
      c->graph_fused = false;
      c->graph_pipe = false;
    }
    // strip updates write the old state only where the next ghost fill reads
    // it, except in the run's last step (only ghost fills and sweeps read
    // the uOld interior in between: no level transfers, no local time
    // stepping); after the run the flag is back to full writes
    const bool bands = c->sched.kind == PCG_SCHED_STRIPS && !c->ts_local && c->h_restr.empty() &&
                       c->h_flux.empty() && steps > 1;
    PCG_CUDA(cudaEventRecord(c->ev0, c->stream));
    if (bands) PCG_CUDA(cudaMemsetAsync(c->d_upd_full, 0, sizeof(int), c->stream));
    for (int s = 0; s < steps; s++) {
      if (bands && s == steps - 1) PCG_CUDA(cudaMemsetAsync(c->d_upd_full, 1, sizeof(int), c->stream));
      PCG_CUDA(cudaGraphLaunch(c->graph, c->stream));
    }
    PCG_CUDA(cudaEventRecord(c->ev1, c->stream));
  } else {
    PCG_CUDA(cudaEventRecord(c->ev0, c->stream));
    for (int s = 0; s < steps; s++) {
      if ((rc = enqueue_step(c, PCG_MODE_PLAIN, false)) != PCG_OK) return rc;
      k_record_hist<<<1, threads, 0, c->stream>>>(c->max_groups, c->d_group_dt, c->d_hist, c->d_counter,
                                                 c->hist_cap, 1, c->d_group_active, c->d_group_time);
      PCG_CUDA(cudaGetLastError());
    }
    PCG_CUDA(cudaEventRecord(c->ev1, c->stream));
  }
  c->run_steps = steps;
  c->run_mode = mode;
  c->run_pipe = pipe;
  return PCG_OK;
}

// After run_enqueue: the dt record, the wait for the stream, the error words
// of the run's bounded waits, the statistics.
int run_finish(pcg_context *c, double *dt_hist) {
  const int32_t steps = c->run_steps, mode = c->run_mode;
  const bool pipe = c->run_pipe;
  int rc;

  if (dt_hist)
    PCG_CUDA(cudaMemcpyAsync(dt_hist, c->d_hist, sizeof(double) * (size_t)steps * c->max_groups,
                             cudaMemcpyDeviceToHost, c->stream));
  PCG_CUDA(cudaStreamSynchronize(c->stream));
  {
    const int xrc = check_level_transfer(c);
    if (xrc != PCG_OK) return xrc;
  }
  if (pipe && (rc = check_pipeline(c)) != PCG_OK) return rc;
  float ms = 0.f;
  PCG_CUDA(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
  c->device_ms += ms;
  if (!c->ts_local || mode != PCG_MODE_BATCHED) c->cell_updates += c->cells_per_step * steps;
  return PCG_OK;
}

}  // namespace

int pcg_run(pcg_context *c, int32_t steps, int32_t mode, double *dt_hist) {
  if (!c || steps < 0 || (mode != PCG_MODE_PLAIN && mode != PCG_MODE_BATCHED))
    return fail(PCG_E_INVALID, "bad arguments");
  if (steps == 0) return PCG_OK;
  std::lock_guard<std::mutex> lk(c->mu);
  if (c->run_pending) return fail(PCG_E_STATE, "a run started by pcg_run_async is still pending");
  int rc = run_enqueue(c, steps, mode);
  if (rc != PCG_OK) return rc;
  return run_finish(c, dt_hist);
}

int pcg_run_async(pcg_context *c, int32_t steps, int32_t mode) {
  if (!c || steps < 1 || (mode != PCG_MODE_PLAIN && mode != PCG_MODE_BATCHED))
    return fail(PCG_E_INVALID, "bad arguments");
  std::lock_guard<std::mutex> lk(c->mu);
  if (c->run_pending) return fail(PCG_E_STATE, "a run started by pcg_run_async is still pending");
  int rc = run_enqueue(c, steps, mode);
  if (rc != PCG_OK) return rc;
  c->run_pending = true;
  return PCG_OK;
}

int pcg_run_wait(pcg_context *c, double *dt_hist) {
  if (!c) return fail(PCG_E_INVALID, "null context");
  std::lock_guard<std::mutex> lk(c->mu);
  if (!c->run_pending) return fail(PCG_E_STATE, "no run started by pcg_run_async is pending");
  c->run_pending = false;
  PCG_CUDA(cudaSetDevice(c->device));
  return run_finish(c, dt_hist);
}

int pcg_get_step_launches(pcg_context *c, int32_t *launches) {
  if (!c || !launches) return fail(PCG_E_INVALID, "bad arguments");
  std::lock_guard<std::mutex> lk(c->mu);
  *launches = c->graph_valid ? c->graph_kernels : 0;
  return PCG_OK;
}

int pcg_set_step_form(pcg_context *c, int32_t form) {
  if (!c || (form != PCG_FORM_AUTO && form != PCG_FORM_UNFUSED)) return fail(PCG_E_INVALID, "bad step form");
  std::lock_guard<std::mutex> lk(c->mu);
  PCG_SETTLE(c);
  if (c->form != form) {
    c->form = form;
    c->graph_valid = false;
    c->topo_dirty = true;  // the fused form's tables are built for PCG_FORM_AUTO only
  }
  return PCG_OK;
}

int pcg_get_step_form(pcg_context *c, int32_t mode, int32_t *fused) {
  if (!c || !fused || (mode != PCG_MODE_PLAIN && mode != PCG_MODE_BATCHED)) return fail(PCG_E_INVALID, "bad arguments");
  std::lock_guard<std::mutex> lk(c->mu);
  PCG_CUDA(cudaSetDevice(c->device));
  int rc = rebuild_topology(c);
  if (rc != PCG_OK) return rc;
  *fused = use_fused(c, mode) ? 1 : 0;
  return PCG_OK;
}

namespace {

int check_schedule(const pcg_schedule *s) {
  if (!s) return fail(PCG_E_INVALID, "null schedule");
  if (s->kind == PCG_SCHED_TILES) {
    if (s->variant != 0 && s->variant != 1)
      return fail(PCG_E_INVALID, "tile variant must be 0 (thread loads) or 1 (TMA staging)");
    return PCG_OK;
  }
  if (s->kind != PCG_SCHED_STRIPS) return fail(PCG_E_INVALID, "schedule kind must be 0 or 1");
  if (s->variant < 0 || s->variant >= pcg::kNumStripVariants)
    return fail(PCG_E_INVALID, "strip variant out of range");
  if (s->chunk < 1 || s->chunk > 32) return fail(PCG_E_INVALID, "strip chunk must be in 1..32");
  if (s->unfused < 0 || s->unfused > 2) return fail(PCG_E_INVALID, "schedule field unfused must be 0, 1 or 2");
  return PCG_OK;
}

}  // namespace

int pcg_set_schedule(pcg_context *c, const pcg_schedule *s) {
  if (!c) return fail(PCG_E_INVALID, "null context");
  int rc = check_schedule(s);
  if (rc != PCG_OK) return rc;
  std::lock_guard<std::mutex> lk(c->mu);
  PCG_SETTLE(c);
  PCG_CUDA(cudaSetDevice(c->device));
  c->sched = *s;
  if (c->sched.kind == PCG_SCHED_TILES) { c->sched.chunk = 32; c->sched.unfused = 0; }
  c->sched_fixed = true;
  c->graph_valid = false;
  if (!c->topo_dirty) return apply_schedule(c);
  return PCG_OK;
}

int pcg_get_schedule(pcg_context *c, pcg_schedule *s) {
  if (!c || !s) return fail(PCG_E_INVALID, "null argument");
  std::lock_guard<std::mutex> lk(c->mu);
  PCG_CUDA(cudaSetDevice(c->device));
  int rc = rebuild_topology(c);
  if (rc != PCG_OK) return rc;
  *s = c->sched;
  return PCG_OK;
}

int pcg_autotune(pcg_context *c, int32_t reps, pcg_schedule *tried, double *ms, int32_t cap,
                 int32_t *n_tried) {
  if (!c || reps < 1 || cap < 0) return fail(PCG_E_INVALID, "bad arguments");
  std::lock_guard<std::mutex> lk(c->mu);
  if (c->run_pending) return fail(PCG_E_STATE, "a run started by pcg_run_async is still pending");
  PCG_CUDA(cudaSetDevice(c->device));
  int rc = rebuild_topology(c);
  if (rc != PCG_OK) return rc;
  if ((rc = check_solvable(c)) != PCG_OK) return rc;
  if ((rc = check_mode(c, PCG_MODE_BATCHED)) != PCG_OK) return rc;
  if ((rc = upload_group_max_dt(c)) != PCG_OK) return rc;
  std::vector<pcg_schedule> cand;
  cand.push_back(pcg_schedule{PCG_SCHED_TILES, 0, 32, 0});
  if (c->tma_ok) cand.push_back(pcg_schedule{PCG_SCHED_TILES, 1, 32, 0});
  for (int chunk : {32, 16})
    for (int v = 0; v < pcg::kNumStripVariants; v++) cand.push_back(pcg_schedule{PCG_SCHED_STRIPS, v, chunk, 0});
  // narrower chunks for grids with few strips per SM (several items per
  // patch: on 27² patches three 9-column chunks beat one of 27 or two of 14)
  for (int chunk : {10, 8})
    for (int v : {0, 2}) cand.push_back(pcg_schedule{PCG_SCHED_STRIPS, v, chunk, 0});
  std::vector<double> t(cand.size(), 0.0);
  for (size_t k = 0; k < cand.size(); k++) {
    c->sched = cand[k];
    if ((rc = apply_schedule(c)) != PCG_OK) return rc;
    // host-side set-up of a candidate stays out of its timed steps
    if (c->sched.kind == PCG_SCHED_TILES && c->sched.variant == 1 && (rc = ensure_tile_maps(c)) != PCG_OK)
      return rc;
    // strip candidates run the fused step where it applies, tiles the unfused one
    const bool fused = use_fused(c, PCG_MODE_BATCHED);
    if (fused) {
      if ((rc = fused_prologue(c)) != PCG_OK) return rc;
    } else {
      PCG_SETTLE(c);
      if ((rc = refresh_fin(c)) != PCG_OK) return rc;
    }
    for (int r = 0; r < reps; r++) {
      PCG_CUDA(cudaEventRecord(c->ev0, c->stream));
      if (fused) {
        rc = enqueue_fused_step(c, PCG_MODE_BATCHED);
        c->fused_pending = true;
      } else {
        rc = enqueue_step(c, PCG_MODE_BATCHED);
      }
      if (rc != PCG_OK) return rc;
      PCG_CUDA(cudaEventRecord(c->ev1, c->stream));
      PCG_CUDA(cudaStreamSynchronize(c->stream));
      float e = 0.f;
      PCG_CUDA(cudaEventElapsedTime(&e, c->ev0, c->ev1));
      t[k] += e;
      c->device_ms += e;
      if (!c->ts_local) c->cell_updates += c->cells_per_step;
    }
    t[k] /= reps;
  }
  size_t best = 0;
  for (size_t k = 1; k < cand.size(); k++)
    if (t[k] < t[best]) best = k;
  // the fastest strip schedule in the unfused form too, where the fused one applied
  if (cand[best].kind == PCG_SCHED_STRIPS && use_fused(c, PCG_MODE_BATCHED)) {
    pcg_schedule u = cand[best];
    u.unfused = 1;
    cand.push_back(u);
    t.push_back(0.0);
    c->sched = u;
    if ((rc = apply_schedule(c)) != PCG_OK) return rc;
    PCG_SETTLE(c);
    if ((rc = refresh_fin(c)) != PCG_OK) return rc;
    for (int r = 0; r < reps; r++) {
      PCG_CUDA(cudaEventRecord(c->ev0, c->stream));
      if ((rc = enqueue_step(c, PCG_MODE_BATCHED)) != PCG_OK) return rc;
      PCG_CUDA(cudaEventRecord(c->ev1, c->stream));
      PCG_CUDA(cudaStreamSynchronize(c->stream));
      float e = 0.f;
      PCG_CUDA(cudaEventElapsedTime(&e, c->ev0, c->ev1));
      t.back() += e;
      c->device_ms += e;
      c->cell_updates += c->cells_per_step;
    }
    t.back() /= reps;
    if (t.back() < t[best]) best = cand.size() - 1;
  }
  // the fastest strip schedule in the pipelined form, where it applies: a run
  // of reps steps (reps + 1 launch pairs), timed as a whole
  if (cand[best].kind == PCG_SCHED_STRIPS) {
    pcg_schedule u = cand[best];
    u.unfused = 2;
    c->sched = u;
    if ((rc = apply_schedule(c)) != PCG_OK) return rc;
    if (use_pipeline(c, PCG_MODE_BATCHED)) {
      cand.push_back(u);
      t.push_back(0.0);
      PCG_SETTLE(c);
      if ((rc = refresh_fin(c)) != PCG_OK) return rc;
      if ((rc = build_pipeline(c)) != PCG_OK) return rc;
      if ((rc = ensure_hist(c, reps)) != PCG_OK) return rc;
      if ((rc = start_pipeline_run(c, reps)) != PCG_OK) return rc;
      PCG_CUDA(cudaEventRecord(c->ev0, c->stream));
      for (int r = 0; r <= reps; r++)
        if ((rc = enqueue_pipeline_launch(c)) != PCG_OK) return rc;
      PCG_CUDA(cudaEventRecord(c->ev1, c->stream));
      PCG_CUDA(cudaStreamSynchronize(c->stream));
      if ((rc = check_pipeline(c)) != PCG_OK) return rc;
      float e = 0.f;
      PCG_CUDA(cudaEventElapsedTime(&e, c->ev0, c->ev1));
      t.back() = e / reps;
      c->device_ms += e;
      c->cell_updates += c->cells_per_step * reps;
      if (t.back() < t[best]) best = cand.size() - 1;
    }
  }
  c->sched = cand[best];
  c->sched_fixed = true;
  if ((rc = apply_schedule(c)) != PCG_OK) return rc;
  {
    std::lock_guard<std::mutex> g(g_tuned_mu);
    g_tuned[c->shape_key] = c->sched;
  }
  const int32_t n = (int32_t)cand.size();
  for (int32_t k = 0; k < std::min(n, cap); k++) {
    if (tried) tried[k] = cand[k];
    if (ms) ms[k] = t[k];
  }
  if (n_tried) *n_tried = n;
  return PCG_OK;
}

int pcg_stats(pcg_context *c, int64_t *cell_updates, double *device_ms) {
  if (!c) return fail(PCG_E_INVALID, "null context");
  if (cell_updates) {
    std::lock_guard<std::mutex> lk(c->mu);
    PCG_CUDA(cudaSetDevice(c->device));
    unsigned long long lts = 0;
    PCG_CUDA(cudaMemcpyAsync(&lts, c->d_lts_cells, sizeof(lts), cudaMemcpyDeviceToHost, c->stream));
    PCG_CUDA(cudaStreamSynchronize(c->stream));
    *cell_updates = c->cell_updates + (int64_t)lts;
  }
  if (device_ms) *device_ms = c->device_ms;
  return PCG_OK;
}

int pcg_profile_step(pcg_context *c, double *ms) {
  if (!c || !ms) return fail(PCG_E_INVALID, "null argument");
  std::lock_guard<std::mutex> lk(c->mu);
  if (c->run_pending) return fail(PCG_E_STATE, "a run started by pcg_run_async is still pending");
  if (c->ts_local) return fail(PCG_E_STATE, "the phase profile times the global step only");
  PCG_CUDA(cudaSetDevice(c->device));
  int rc = rebuild_topology(c);
  if (rc != PCG_OK) return rc;
  if ((rc = check_solvable(c)) != PCG_OK) return rc;
  if ((rc = upload_group_max_dt(c)) != PCG_OK) return rc;
  if (use_fused(c, PCG_MODE_BATCHED)) {
    // the fused step's three launches: fused sweep, time advance, next reset
    if ((rc = fused_prologue(c)) != PCG_OK) return rc;
    cudaEvent_t ev[4];
    for (int i = 0; i < 4; i++) PCG_CUDA(cudaEventCreate(&ev[i]));
    const pcg::FusedDev F = fused_dev(c);
    PCG_CUDA(cudaEventRecord(ev[0], c->stream));
    PCG_CUDA(pcg::launch_fused_strips(c->stream, c->sched.variant, c->fused_grid, F, c->d_sitems, c->d_sgroups,
                                      (int)c->h_sitems.size(), c->d_patch_smax, c->d_group_dt));
    PCG_CUDA(cudaEventRecord(ev[1], c->stream));
    PCG_CUDA(pcg::launch_fused_advance(c->stream, F, c->d_leaf_ids, (int)c->leaf_ids.size(), c->d_times,
                                       c->d_patch_smax, c->max_groups, c->d_group_dt, c->d_group_time, c->d_pend,
                                       c->d_par, c->d_dt_prev, c->d_hist, c->d_counter, 0));
    PCG_CUDA(cudaEventRecord(ev[2], c->stream));
    rc = enqueue_reset_items(c);
    c->fused_pending = true;
    if (rc != PCG_OK) return rc;
    PCG_CUDA(cudaEventRecord(ev[3], c->stream));
    PCG_CUDA(cudaStreamSynchronize(c->stream));
    float t[3];
    for (int i = 0; i < 3; i++) PCG_CUDA(cudaEventElapsedTime(&t[i], ev[i], ev[i + 1]));
    ms[0] = t[2];
    ms[1] = 0.0;
    ms[2] = 0.0;
    ms[3] = t[0];
    ms[4] = t[1];
    for (int i = 0; i < 4; i++) cudaEventDestroy(ev[i]);
    c->cell_updates += c->cells_per_step;
    return PCG_OK;
  }
  if (use_pipeline(c, PCG_MODE_BATCHED)) {
    // a pipelined run of two steps; its middle launch pair (update of the
    // first step, fill, walls and sweep of the second) is the steady state
    PCG_SETTLE(c);
    if ((rc = refresh_fin(c)) != PCG_OK) return rc;
    if (!c->pipe_valid && (rc = build_pipeline(c)) != PCG_OK) return rc;
    if ((rc = ensure_hist(c, 2)) != PCG_OK) return rc;
    if ((rc = start_pipeline_run(c, 2)) != PCG_OK) return rc;
    cudaEvent_t ev[7];
    for (int i = 0; i < 7; i++) PCG_CUDA(cudaEventCreate(&ev[i]));
    const pcg::PipeDev pd = pipe_dev(c);
    PCG_CUDA(cudaEventRecord(ev[0], c->stream));
    for (int l = 0; l < 3; l++) {
      if ((rc = enqueue_pipeline_prep(c)) != PCG_OK) return rc;
      PCG_CUDA(cudaEventRecord(ev[2 * l + 1], c->stream));
      PCG_CUDA(pcg::launch_pipeline_step(c->stream, c->sched.variant, c->pipe_grid, pd));
      PCG_CUDA(cudaEventRecord(ev[2 * l + 2], c->stream));
    }
    PCG_CUDA(cudaStreamSynchronize(c->stream));
    float t_pre = 0.f, t_first = 0.f, t_step = 0.f, t_last = 0.f;
    PCG_CUDA(cudaEventElapsedTime(&t_first, ev[1], ev[2]));
    PCG_CUDA(cudaEventElapsedTime(&t_pre, ev[2], ev[3]));
    PCG_CUDA(cudaEventElapsedTime(&t_step, ev[3], ev[4]));
    PCG_CUDA(cudaEventElapsedTime(&t_last, ev[5], ev[6]));
    for (int i = 0; i < 7; i++) cudaEventDestroy(ev[i]);
    if ((rc = check_pipeline(c)) != PCG_OK) return rc;
    ms[0] = t_pre;
    ms[1] = t_first;
    ms[2] = t_last;
    ms[3] = t_step;
    ms[4] = 0.0;
    c->cell_updates += 2 * c->cells_per_step;
    return PCG_OK;
  }
  PCG_SETTLE(c);
  if ((rc = refresh_fin(c)) != PCG_OK) return rc;
  cudaEvent_t ev[6];
  for (int i = 0; i < 6; i++) PCG_CUDA(cudaEventCreate(&ev[i]));
  using namespace pcg;
  PCG_CUDA(cudaEventRecord(ev[0], c->stream));
  PCG_CUDA(launch_reset(c->stream, c->max_groups, c->d_group_max_dt, c->d_group_t_end, c->d_group_time,
                        c->d_group_dt, c->d_group_active, c->max_patches,
                        c->d_patch_smax));
  PCG_CUDA(cudaEventRecord(ev[1], c->stream));
  PCG_CUDA(launch_item_step(c->stream, c->d_patches, c->d_times, c->d_items, (int)c->h_items.size(),
                            c->d_item_step));
  PCG_CUDA(launch_ghost_cells(c->stream, c->slab, c->d_patches, c->d_items, c->d_gcells, c->n_copy_cells,
                              c->n_interp_cells, c->d_copy_plan, c->d_plan, c->d_item_step,
                                c->d_group_active, c->d_fin));
  PCG_CUDA(cudaEventRecord(ev[2], c->stream));
  PCG_CUDA(launch_walls(c->stream, c->slab, c->d_patches, c->d_wall, (int)c->h_wall.size(),
                        c->d_group_active));
  PCG_CUDA(cudaEventRecord(ev[3], c->stream));
  if ((rc = enqueue_sweep(c)) != PCG_OK) return rc;
  PCG_CUDA(cudaEventRecord(ev[4], c->stream));
  if ((rc = enqueue_update(c)) != PCG_OK) return rc;
  PCG_CUDA(cudaEventRecord(ev[5], c->stream));
  PCG_CUDA(cudaStreamSynchronize(c->stream));
  for (int i = 0; i < 5; i++) {
    float t = 0.f;
    PCG_CUDA(cudaEventElapsedTime(&t, ev[i], ev[i + 1]));
    ms[i] = t;
  }
  for (int i = 0; i < 6; i++) cudaEventDestroy(ev[i]);
  c->cell_updates += c->cells_per_step;
  return PCG_OK;
}

int pcg_probe_fp64_peak(pcg_context *c, double *tflops) {
  if (!c || !tflops) return fail(PCG_E_INVALID, "null argument");
  std::lock_guard<std::mutex> lk(c->mu);
  PCG_CUDA(cudaSetDevice(c->device));
  int blocks = c->num_sms * 8, threads = 256, iters = 4096;
  double *buf = nullptr;
  PCG_CUDA(cudaMalloc(&buf, sizeof(double) * (size_t)blocks * threads));
  k_fp64_probe<<<blocks, threads, 0, c->stream>>>(buf, 64, 1.0000001, 1e-9);
  PCG_CUDA(cudaGetLastError());
  float best = 1e30f;
  for (int r = 0; r < 3; r++) {
    PCG_CUDA(cudaEventRecord(c->ev0, c->stream));
    k_fp64_probe<<<blocks, threads, 0, c->stream>>>(buf, iters, 1.0000001, 1e-9);
    PCG_CUDA(cudaEventRecord(c->ev1, c->stream));
    PCG_CUDA(cudaEventSynchronize(c->ev1));
    float t = 0.f;
    PCG_CUDA(cudaEventElapsedTime(&t, c->ev0, c->ev1));
    best = std::min(best, t);
  }
  PCG_CUDA(cudaFree(buf));
  *tflops = 2.0 * 8.0 * iters * (double)blocks * threads / (best * 1e-3) / 1e12;
  return PCG_OK;
}

int pcg_selftest_transfer_wait(pcg_context *c) {
  if (!c) return fail(PCG_E_INVALID, "null context");
  std::lock_guard<std::mutex> lk(c->mu);
  PCG_SETTLE(c);
  PCG_CUDA(cudaSetDevice(c->device));
  int rc = rebuild_topology(c);
  if (rc != PCG_OK) return rc;
  if (c->h_restr.empty()) return fail(PCG_E_STATE, "the self-test needs a restriction list");
  if ((rc = refresh_restr_geometry(c)) != PCG_OK) return rc;
  PCG_CUDA(cudaStreamSynchronize(c->stream));
  if ((rc = check_level_transfer(c)) != PCG_OK) return rc;
  // restriction items only (no flux destinations, no face-flux storage), each
  // waiting for one finished flux destination: nothing sets that counter
  const int n_restr = (int)c->h_restr_chunks.size();
  const int grid = pcg::level_transfer_grid(c->num_sms, 0, 0, n_restr);
  PCG_CUDA(pcg::launch_level_transfer(c->stream, grid, c->slab, c->d_patches, c->d_times, c->d_flux_leaf_ids, 0,
                                      c->g_flux, c->d_flux, c->d_flux_begin, 0, c->d_restr, c->d_restr_begin,
                                      c->d_restr_geo, c->d_restr_geo_bad, c->d_restr_chunks, n_restr, nullptr,
                                      nullptr, c->d_xfer, 1));
  PCG_CUDA(cudaStreamSynchronize(c->stream));
  int err = 0;
  PCG_CUDA(cudaMemcpy(&err, &c->d_xfer->err, sizeof(int), cudaMemcpyDeviceToHost));
  PCG_CUDA(cudaMemset(c->d_xfer, 0, sizeof(pcg::TransferCtl)));
  if (err != 1) return fail(PCG_E_STATE, "the level transfer's bounded wait did not report running out");
  return PCG_OK;
}

int pcg_check_ieee_emulation(pcg_context *c, int64_t samples, uint64_t seed, int64_t *mismatches) {
  if (!c || !mismatches || samples < 0) return fail(PCG_E_INVALID, "bad argument");
  std::lock_guard<std::mutex> lk(c->mu);
  PCG_CUDA(cudaSetDevice(c->device));
  unsigned long long *d = nullptr;
  PCG_CUDA(cudaMalloc(&d, sizeof(unsigned long long)));
  PCG_CUDA(cudaMemsetAsync(d, 0, sizeof(unsigned long long), c->stream));
  k_check_ieee<<<c->num_sms * 8, 256, 0, c->stream>>>(samples, seed, d);
  PCG_CUDA(cudaGetLastError());
  unsigned long long h = 0;
  PCG_CUDA(cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  PCG_CUDA(cudaStreamSynchronize(c->stream));
  PCG_CUDA(cudaFree(d));
  *mismatches = (int64_t)h;
  return PCG_OK;
}

int pcg_synchronize(pcg_context *c) {
  if (!c) return fail(PCG_E_INVALID, "null context");
  PCG_CUDA(cudaStreamSynchronize(c->stream));
  return PCG_OK;
}

}  // extern "C"
