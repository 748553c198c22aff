"""bemgpu -- GB300 (sm_103a) full-3D Helmholtz BEM behind AcousticScattering.jl's API.

The numerical work runs in libbemgpu.so (CUDA, C ABI in include/bemgpu.h); this package
is the host-side mirror of the reference's ``bem`` / ``scattering_amplitude`` /
``target_strength`` / ``diagnostics`` / sweep interface, plus the deterministic surface
generators of the benchmark workloads.
"""
from . import meshes
from ._lib import lib, LIB_PATH
from .api import (ArgumentError, BEMGPUError, BEMSolution, Context, Factor, FluidFilled,
                  FrequencySweep, GasFilled, Mesh, PressureRelease, Rigid, Server,
                  SweepResult,
                  assemble, bem, context, dense_solve, diagnostics, factor_batch,
                  frequency_sweep, hmatrix_apply, solve_batch,
                  incidence_angle_sweep, mesh, pressure, scattering_amplitude,
                  target_strength)

__all__ = ["ArgumentError", "BEMGPUError", "BEMSolution", "Context", "Factor", "FluidFilled",
           "FrequencySweep", "GasFilled", "Mesh", "PressureRelease", "Rigid", "Server",
           "SweepResult",
           "assemble", "bem", "context", "dense_solve", "diagnostics", "factor_batch",
           "frequency_sweep", "hmatrix_apply", "solve_batch",
           "incidence_angle_sweep", "mesh", "meshes", "pressure", "scattering_amplitude",
           "target_strength", "lib", "LIB_PATH"]
