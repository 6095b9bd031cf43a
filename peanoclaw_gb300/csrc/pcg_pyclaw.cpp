// pcg_pyclaw.cpp -- PeanoClaw's PyClaw C interface (pyclaw_peano_*) on the
// GB300 SWE kernel.
//
// The reference's libpeano-claw exports pyclaw_peano_new / destroy /
// evolveToTime / gatherSolution / runTests / runWorker
// (src/peanoclaw/pyclaw/pyclawBindings.cpp:108-340); its Python package loads
// them with ctypes and passes ctypes callbacks that receive numpy arrays of a
// subgrid's data (PyClawState.cpp:13-58: q = uNew (nq, nx, ny), qbc = uOld
// with ghost layer (nq, nx+2g, ny+2g), aux (naux, nx, ny))
// (src/python/peanoclaw/peano.py:44-134).  These functions keep those
// signatures and callback conventions for shallow-water problems solved on
// the GPU:
//  - the grid is the uniform spacetree level whose cells are
//    initialMaximalMeshWidthScalar wide, each cell a subgrid of the given
//    subdivision factor, with reflecting walls on the domain boundary;
//  - the initialization callback fills q (h, hu, hv) and, with one aux field,
//    the bathymetry of every subgrid (its return value, the demanded mesh
//    width, is accepted; the grid stays uniform); the bathymetry of the ghost
//    layer comes from the neighbouring subgrids, at the domain boundary from
//    the boundary cell;
//  - the solver, boundary-condition, refinement and inter-patch callbacks
//    are not called: the GPU f-wave kernel advances every subgrid with one
//    global timestep (pcg_run), the walls are the SWE kernel's
//    fillBoundaryLayer;
//  - evolveToTime runs batched steps until the end time (a device-side end
//    time, so the last step lands on it);
//  - gatherSolution calls the addPatchToSolution callback per subgrid with
//    numpy arrays over the downloaded data and the subgrid's new time.
// The numpy arrays are made with the hosting interpreter's C API, resolved
// at run time (the library is loaded into that interpreter by ctypes), so no
// Python headers are needed to build it.
#include <dlfcn.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/pcg_pyclaw.h"

namespace {

typedef void *PyObj;

// The callback types of PyClawCallbacks.h with PyObject* as an opaque pointer.
typedef double (*InitializationCallback)(PyObj q, PyObj qbc, PyObj aux, int sx0, int sx1, int sx2, int unknowns,
                                         int auxFields, double sizeX, double sizeY, double sizeZ, double posX,
                                         double posY, double posZ, bool skipQInitialization);
typedef void (*AddPatchToSolutionCallback)(PyObj q, PyObj qbc, int ghostlayerWidth, double sizeX, double sizeY,
                                           double sizeZ, double posX, double posY, double posZ, double currentTime);

// The interpreter functions the arrays need (all in the stable ABI).
struct PyApi {
  int (*gil_ensure)() = nullptr;
  void (*gil_release)(int) = nullptr;
  PyObj (*import_module)(const char *) = nullptr;
  PyObj (*get_attr)(PyObj, const char *) = nullptr;
  PyObj (*memoryview)(char *, long, int) = nullptr;
  PyObj (*call_obj_args)(PyObj, ...) = nullptr;
  PyObj (*call_method)(PyObj, const char *, const char *, ...) = nullptr;
  void (*dec_ref)(PyObj) = nullptr;
  void (*err_print)() = nullptr;
  PyObj frombuffer = nullptr;
  bool ok = false;
};

PyApi g_py;
std::string g_error;

template <class F>
bool resolve(F &f, const char *name) {
  f = reinterpret_cast<F>(dlsym(RTLD_DEFAULT, name));
  return f != nullptr;
}

bool python_api() {
  if (g_py.ok) return true;
  if (!resolve(g_py.gil_ensure, "PyGILState_Ensure") || !resolve(g_py.gil_release, "PyGILState_Release") ||
      !resolve(g_py.import_module, "PyImport_ImportModule") || !resolve(g_py.get_attr, "PyObject_GetAttrString") ||
      !resolve(g_py.memoryview, "PyMemoryView_FromMemory") ||
      !resolve(g_py.call_obj_args, "PyObject_CallFunctionObjArgs") ||
      !resolve(g_py.call_method, "PyObject_CallMethod") || !resolve(g_py.dec_ref, "Py_DecRef") ||
      !resolve(g_py.err_print, "PyErr_Print")) {
    g_error = "the Python interpreter's C API is not in this process";
    return false;
  }
  const int st = g_py.gil_ensure();
  PyObj np = g_py.import_module("numpy");
  if (np) {
    g_py.frombuffer = g_py.get_attr(np, "frombuffer");
    g_py.dec_ref(np);
  }
  if (!g_py.frombuffer) g_py.err_print();
  g_py.gil_release(st);
  if (!g_py.frombuffer) {
    g_error = "numpy is not importable";
    return false;
  }
  g_py.ok = true;
  return true;
}

// A writable float64 numpy array of shape (a, b, c) over `data` (the GIL held).
PyObj array3(double *data, int a, int b, int c) {
  const long nbytes = (long)sizeof(double) * a * b * c;
  PyObj mv = g_py.memoryview(reinterpret_cast<char *>(data), nbytes, 0x200 /* PyBUF_WRITE */);
  if (!mv) return nullptr;
  PyObj flat = g_py.call_obj_args(g_py.frombuffer, mv, nullptr);
  g_py.dec_ref(mv);
  if (!flat) return nullptr;
  PyObj arr = g_py.call_method(flat, "reshape", "(iii)", a, b, c);
  g_py.dec_ref(flat);
  return arr;
}

struct Runner {
  pcg_context *ctx = nullptr;
  int n = 0, naux = 0, npx = 0, npy = 0;
  double lo[2] = {0, 0}, sub[2] = {0, 0};
  std::vector<int32_t> ids;
  std::vector<double> packed;  // every subgrid's vector, reference layout, back to back
  int64_t vlen = 0;
  double time = 0.0;
  AddPatchToSolutionCallback add_to_solution = nullptr;
};

int64_t vector_len(int n) {
  pcg_patch_desc d{};
  d.nx = d.ny = n;
  d.ghost = 1;
  d.nq = 3;
  d.np_w = 1;
  return pcg_patch_vector_size(&d);
}

bool fail_pcg(const char *what) {
  g_error = std::string(what) + ": " + pcg_last_error();
  return false;
}

// Face and corner transfers of a regular grid of equal subgrids (same-level
// copies; GhostlayerCompositorFunctors.cpp:23-72), per destination in the
// order left, right, bottom, top, then the four corners.
std::vector<pcg_ghost_item> grid_items(const Runner &R) {
  std::vector<pcg_ghost_item> items;
  const int n = R.n;
  const int dirs[8][2] = {{-1, 0}, {1, 0}, {0, -1}, {0, 1}, {-1, -1}, {1, -1}, {-1, 1}, {1, 1}};
  for (int i = 0; i < R.npx; i++)
    for (int j = 0; j < R.npy; j++)
      for (const auto &dd : dirs) {
        const int ti = i + dd[0], tj = j + dd[1];
        if (ti < 0 || ti >= R.npx || tj < 0 || tj >= R.npy) continue;
        pcg_ghost_item it;
        it.kind = PCG_GHOST_COPY;
        it.src = R.ids[(size_t)ti * R.npy + tj];
        it.dst = R.ids[(size_t)i * R.npy + j];
        for (int d = 0; d < 2; d++) {
          const int v = -dd[d];  // direction from the source to the destination
          it.size[d] = v == 0 ? n : 1;
          it.dst_offset[d] = v == 0 ? 0 : (v == 1 ? -1 : n);
          it.src_offset[d] = v == 0 ? 0 : (v == 1 ? n - 1 : 0);
        }
        items.push_back(it);
      }
  return items;
}

bool setup(Runner &R, double meshWidth, const double off[2], const double size[2], int sx0, int sx1, int unknowns,
           int auxFields, int ghost, double dt0, InitializationCallback init) {
  if (unknowns != 3 || (auxFields != 0 && auxFields != 1) || ghost != 1 || sx0 != sx1 || sx0 < 2 ||
      !(meshWidth > 0.0)) {
    g_error = "the GPU SWE kernel takes 3 unknowns, at most one aux field (bathymetry), ghost layer width 1 "
              "and square subgrids";
    return false;
  }
  if (!init) {
    g_error = "no initialization callback";
    return false;
  }
  if (!python_api()) return false;
  R.n = sx0;
  R.naux = auxFields;
  R.npx = std::max(1, (int)std::lround(size[0] / meshWidth));
  R.npy = std::max(1, (int)std::lround(size[1] / meshWidth));
  R.lo[0] = off[0];
  R.lo[1] = off[1];
  R.sub[0] = size[0] / R.npx;
  R.sub[1] = size[1] / R.npy;
  const int n = R.n, np = R.npx * R.npy;
  R.vlen = vector_len(n);
  R.packed.assign((size_t)R.vlen * np, 0.0);
  // initial state and bathymetry through the callback, subgrid by subgrid
  std::vector<double> B((size_t)R.npx * n * R.npy * n, 0.0);
  std::vector<double> aux((size_t)std::max(1, R.naux) * n * n);
  const int gst = g_py.gil_ensure();
  bool ok = true;
  for (int i = 0; i < R.npx && ok; i++)
    for (int j = 0; j < R.npy && ok; j++) {
      double *v = R.packed.data() + (size_t)(i * R.npy + j) * R.vlen;
      std::fill(aux.begin(), aux.end(), 0.0);
      PyObj q = array3(v, 3, n, n);
      PyObj qbc = array3(v + 3 * n * n, 3, n + 2, n + 2);
      PyObj a = array3(aux.data(), R.naux, n, n);
      if (!q || !qbc || !a) {
        g_py.err_print();
        g_error = "could not create the subgrid arrays";
        ok = false;
      } else {
        init(q, qbc, a, n, n, 0, 3, R.naux, R.sub[0], R.sub[1], 0.0, R.lo[0] + i * R.sub[0],
             R.lo[1] + j * R.sub[1], 0.0, false);
      }
      if (q) g_py.dec_ref(q);
      if (qbc) g_py.dec_ref(qbc);
      if (a) g_py.dec_ref(a);
      if (R.naux)
        for (int x = 0; x < n; x++)
          for (int y = 0; y < n; y++) B[((size_t)i * n + x) * R.npy * n + (size_t)j * n + y] = aux[x * n + y];
    }
  g_py.gil_release(gst);
  if (!ok) return false;
  // bathymetry with ghost layer: the neighbours' cells, at the domain
  // boundary the boundary cell (the mirror of a reflecting wall)
  const int W = R.npx * n, H = R.npy * n;
  for (int i = 0; i < R.npx; i++)
    for (int j = 0; j < R.npy; j++) {
      double *b = R.packed.data() + (size_t)(i * R.npy + j) * R.vlen + 3 * n * n + 3 * (n + 2) * (n + 2);
      for (int x = -1; x <= n; x++)
        for (int y = -1; y <= n; y++) {
          const int gx = std::min(W - 1, std::max(0, i * n + x)), gy = std::min(H - 1, std::max(0, j * n + y));
          b[(x + 1) * (n + 2) + (y + 1)] = B[(size_t)gx * H + gy];
        }
    }
  pcg_config cfg{};
  cfg.device = 0;
  cfg.max_patches = np + 8;
  cfg.max_groups = 1;
  cfg.slab_doubles = (int64_t)((double)R.vlen * np * 1.2) + 65536;
  cfg.params = pcg_swe_params{9.81, 0.5, 0.01, 0.1, 1e-5, 3.4028234663852886e38};
  if (pcg_create(&cfg, &R.ctx) != PCG_OK) return fail_pcg("pcg_create");
  for (int i = 0; i < R.npx; i++)
    for (int j = 0; j < R.npy; j++) {
      pcg_patch_desc d{};
      d.nx = d.ny = n;
      d.ghost = 1;
      d.nq = 3;
      d.np_w = 1;
      d.flags = PCG_PATCH_LEAF;
      d.pos[0] = R.lo[0] + i * R.sub[0];
      d.pos[1] = R.lo[1] + j * R.sub[1];
      d.size[0] = R.sub[0];
      d.size[1] = R.sub[1];
      int32_t id = -1;
      if (pcg_patch_alloc(R.ctx, &d, &id) != PCG_OK) return fail_pcg("pcg_patch_alloc");
      const uint32_t wall = (i == 0 ? 1u : 0u) | (i == R.npx - 1 ? 2u : 0u) | (j == 0 ? 4u : 0u) |
                            (j == R.npy - 1 ? 8u : 0u);
      if (pcg_patch_set_boundary(R.ctx, id, wall) != PCG_OK) return fail_pcg("pcg_patch_set_boundary");
      pcg_patch_time t{};
      t.est_next = dt0;
      t.restr_lower[0] = t.restr_lower[1] = 1.7976931348623157e308;
      t.restr_upper[0] = t.restr_upper[1] = -1.7976931348623157e308;
      if (pcg_patch_set_time(R.ctx, id, &t) != PCG_OK) return fail_pcg("pcg_patch_set_time");
      R.ids.push_back(id);
    }
  if (pcg_patches_upload(R.ctx, np, R.ids.data(), R.packed.data()) != PCG_OK) return fail_pcg("pcg_patches_upload");
  const std::vector<pcg_ghost_item> items = grid_items(R);
  if (pcg_set_ghost_items(R.ctx, items.data(), (int32_t)items.size()) != PCG_OK) return fail_pcg("pcg_set_ghost_items");
  if (pcg_set_group_max_dt(R.ctx, 0, HUGE_VAL) != PCG_OK) return fail_pcg("pcg_set_group_max_dt");
  return true;
}

}  // namespace

extern "C" {

void *pyclaw_peano_new(double initialMaximalMeshWidthScalar, double domainOffsetX0, double domainOffsetX1,
                       double domainOffsetX2, double domainSizeX0, double domainSizeX1, double domainSizeX2,
                       int subdivisionFactorX0, int subdivisionFactorX1, int subdivisionFactorX2,
                       int unknownsPerSubcell, int auxiliarFieldsPerSubcell, int ghostlayerWidth,
                       double initialTimestepSize, char *configurationFile, bool useDimensionalSplittingExtrapolation,
                       bool reduceReductions, void *initializationCallback, void *boundaryConditionCallback,
                       void *solverCallback, void *refinementCriterionCallback, void *addPatchToSolutionCallback,
                       void *interpolationCallback, void *restrictionCallback, void *fluxCorrectionCallback,
                       bool enablePeanoLogging, int forkLevelIncrement, int *rank) {
  (void)domainOffsetX2; (void)domainSizeX2; (void)subdivisionFactorX2; (void)configurationFile;
  (void)useDimensionalSplittingExtrapolation; (void)reduceReductions; (void)boundaryConditionCallback;
  (void)solverCallback; (void)refinementCriterionCallback; (void)interpolationCallback; (void)restrictionCallback;
  (void)fluxCorrectionCallback; (void)enablePeanoLogging; (void)forkLevelIncrement;
  Runner *R = new Runner();
  const double off[2] = {domainOffsetX0, domainOffsetX1}, size[2] = {domainSizeX0, domainSizeX1};
  if (!setup(*R, initialMaximalMeshWidthScalar, off, size, subdivisionFactorX0, subdivisionFactorX1,
             unknownsPerSubcell, auxiliarFieldsPerSubcell, ghostlayerWidth, initialTimestepSize,
             reinterpret_cast<InitializationCallback>(initializationCallback))) {
    std::fprintf(stderr, "pyclaw_peano_new: %s\n", g_error.c_str());
    if (R->ctx) pcg_destroy(R->ctx);
    delete R;
    return nullptr;
  }
  R->add_to_solution = reinterpret_cast<AddPatchToSolutionCallback>(addPatchToSolutionCallback);
  if (rank) *rank = 0;
  return R;
}

void pyclaw_peano_destroy(void *runner) {
  Runner *R = static_cast<Runner *>(runner);
  if (!R) return;
  if (R->ctx) pcg_destroy(R->ctx);
  delete R;
}

void pyclaw_peano_evolveToTime(double time, void *runner) {
  Runner *R = static_cast<Runner *>(runner);
  if (!R) return;
  if (pcg_set_group_end_time(R->ctx, 0, R->time, time) != PCG_OK) {
    std::fprintf(stderr, "pyclaw_peano_evolveToTime: %s\n", pcg_last_error());
    return;
  }
  double t = R->time;
  while (t < time) {
    if (pcg_run(R->ctx, 16, PCG_MODE_BATCHED, nullptr) != PCG_OK) {
      std::fprintf(stderr, "pyclaw_peano_evolveToTime: %s\n", pcg_last_error());
      return;
    }
    double tn = t;
    if (pcg_get_group_times(R->ctx, &tn) != PCG_OK) return;
    if (!(tn > t)) {
      std::fprintf(stderr, "pyclaw_peano_evolveToTime: no progress towards t = %g\n", time);
      return;
    }
    t = tn;
  }
  R->time = t;
}

void pyclaw_peano_gatherSolution(void *runner) {
  Runner *R = static_cast<Runner *>(runner);
  if (!R) return;
  const int np = (int)R->ids.size(), n = R->n;
  if (pcg_patches_download(R->ctx, np, R->ids.data(), R->packed.data()) != PCG_OK) {
    std::fprintf(stderr, "pyclaw_peano_gatherSolution: %s\n", pcg_last_error());
    return;
  }
  if (!R->add_to_solution) return;
  std::vector<pcg_patch_time> times(np);
  if (pcg_patches_get_time(R->ctx, np, R->ids.data(), times.data()) != PCG_OK) return;
  const int gst = g_py.gil_ensure();
  for (int k = 0; k < np; k++) {
    double *v = R->packed.data() + (size_t)k * R->vlen;
    PyObj q = array3(v, 3, n, n);
    PyObj qbc = array3(v + 3 * n * n, 3, n + 2, n + 2);
    if (q && qbc) {
      const int i = k / R->npy, j = k % R->npy;
      R->add_to_solution(q, qbc, 1, R->sub[0], R->sub[1], 0.0, R->lo[0] + i * R->sub[0], R->lo[1] + j * R->sub[1],
                         0.0, times[k].time + times[k].dt);
    } else {
      g_py.err_print();
    }
    if (q) g_py.dec_ref(q);
    if (qbc) g_py.dec_ref(qbc);
  }
  g_py.gil_release(gst);
}

// The reference runs Peano's registered unit tests here; this library's
// tests are the repository's test suite.
void pyclaw_peano_runTests() {}

// MPI workers in the reference; one process per GPU here, so a worker has
// nothing to do.
int pyclaw_peano_runWorker(void *runner) {
  (void)runner;
  return 0;
}

int pyclaw_peano_setSweParameters(void *runner, const pcg_swe_params *params) {
  Runner *R = static_cast<Runner *>(runner);
  if (!R || !params) return PCG_E_INVALID;
  return pcg_set_params(R->ctx, params);
}

const char *pyclaw_peano_lastError() { return g_error.c_str(); }

}  // extern "C"
