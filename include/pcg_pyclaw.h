/*
 * pcg_pyclaw.h -- PeanoClaw's PyClaw C interface on the GB300 SWE kernel
 * (libpcg_pyclaw.so, built on libpcg.so).
 *
 * The reference's libpeano-claw exports these functions
 * (src/peanoclaw/pyclaw/pyclawBindings.cpp:108-340) for its Python package,
 * which loads them with ctypes (src/python/peanoclaw/peano.py:44-134) and
 * passes ctypes callbacks that receive numpy arrays of a subgrid's data
 * (PyClawCallbacks.h:9-107, PyClawState.cpp:13-58).  The signatures and the
 * callback conventions are the reference's; the subgrids are solved by the
 * GPU SWE kernel:
 *  - uniform grid of subgrids initialMaximalMeshWidthScalar wide, reflecting
 *    walls on the domain boundary; 3 unknowns (h, hu, hv), at most one aux
 *    field (bathymetry), ghost layer width 1, square subgrids (NULL
 *    otherwise);
 *  - the initialization callback fills every subgrid's q and aux; the
 *    solver, boundary-condition, refinement and inter-patch callbacks are
 *    not called (the GPU f-wave kernel advances all subgrids with one global
 *    timestep, g = 9.81, CFL 0.5 unless pyclaw_peano_setSweParameters says
 *    otherwise);
 *  - the library must be loaded into a Python process with numpy (it builds
 *    the callbacks' arrays with that interpreter's C API).
 */
#ifndef PCG_PYCLAW_H
#define PCG_PYCLAW_H

#include <stdbool.h>

#include "pcg.h"

#ifdef __cplusplus
extern "C" {
#endif

/* pyclawBindings.cpp:108-236: creates the grid, initialises every subgrid
 * through initializationCallback and uploads it; returns the runner (NULL on
 * failure, reason on stderr and from pyclaw_peano_lastError).  *rank = 0.
 * The 3rd dimension's arguments are ignored (2D). */
void *pyclaw_peano_new(double initialMaximalMeshWidthScalar, double domainOffsetX0, double domainOffsetX1,
                       double domainOffsetX2, double domainSizeX0, double domainSizeX1, double domainSizeX2,
                       int subdivisionFactorX0, int subdivisionFactorX1, int subdivisionFactorX2,
                       int unknownsPerSubcell, int auxiliarFieldsPerSubcell, int ghostlayerWidth,
                       double initialTimestepSize, char *configurationFile, bool useDimensionalSplittingExtrapolation,
                       bool reduceReductions, void *initializationCallback, void *boundaryConditionCallback,
                       void *solverCallback, void *refinementCriterionCallback, void *addPatchToSolutionCallback,
                       void *interpolationCallback, void *restrictionCallback, void *fluxCorrectionCallback,
                       bool enablePeanoLogging, int forkLevelIncrement, int *rank);
/* pyclawBindings.cpp:256-273. */
void pyclaw_peano_destroy(void *runner);
/* pyclawBindings.cpp:275-300: every subgrid advances to `time`. */
void pyclaw_peano_evolveToTime(double time, void *runner);
/* pyclawBindings.cpp:302-324: addPatchToSolutionCallback(q, qbc, ghost
 * width, size, position, new time) for every subgrid. */
void pyclaw_peano_gatherSolution(void *runner);
/* pyclawBindings.cpp:238-254 (Peano's unit tests): nothing to run here. */
void pyclaw_peano_runTests(void);
/* pyclawBindings.cpp:326-340 (MPI workers): one process per GPU, returns 0. */
int pyclaw_peano_runWorker(void *runner);
/* No counterpart in the reference: the SWE parameters of the GPU solver. */
int pyclaw_peano_setSweParameters(void *runner, const pcg_swe_params *params);
/* No counterpart in the reference: the reason of the last failure. */
const char *pyclaw_peano_lastError(void);

#ifdef __cplusplus
}
#endif
#endif
