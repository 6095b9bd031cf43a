"""The GPU Numerics plugin (peanoclaw_gb300/shim/GpuSWEKernel.cpp) compiles
warning-free as C++11 and C++17 against headers that declare the reference's
Numerics interface with its exact virtual signatures (every override is
checked by the compiler), links against libpcg.so, and exports the plugin's
class; no GPU needed."""
import subprocess

import pytest

import shim_build


@pytest.mark.parametrize("std", ["c++11", "c++17"])
def test_plugin_compiles_against_the_numerics_interface(tmp_path, std):
    lib = shim_build.build(str(tmp_path), std=std)
    syms = subprocess.run(["nm", "-D", "-C", "--defined-only", lib], capture_output=True, text=True).stdout
    for name in ("vtable for peanoclaw::native::GpuSWEKernel",
                 "peanoclaw::native::GpuSWEKernel::solveTimestep",
                 "peanoclaw::native::GpuSWEKernel::fillBoundaryLayer",
                 "peanoclaw::native::GpuSWEKernel::interpolateSolution",
                 "peanoclaw::native::GpuSWEKernel::restrictSolution",
                 "peanoclaw::interSubgridCommunication::DefaultTransfer::copyUNewToUOld",
                 "peanoclaw::interSubgridCommunication::DefaultTransfer::swapUNewAndUOld",
                 "shim_drive_iterations"):
        assert name in syms, name
