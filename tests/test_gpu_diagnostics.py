"""The reference's factor diagnostics and options (solvers/bem/full.jl:364-409, 330-341):
condition_limit with SVD condition numbers of the system and of the equilibrated system,
conditioning = :svd / :not_computed, norm_floor, and derivative_evaluation."""
import math

import numpy as np
import pytest

import bemgpu
from bemgpu import meshes
from oracle import oracle as O

pytestmark = pytest.mark.gpu

G, H, K = 1.05, 1.02, 1.7


def _fluid_system(nodes, tris, formulation="muller"):
    return O.assemble_fluid(O.Panels(nodes, tris), K, G, H, formulation)


@pytest.mark.parametrize("precision", ["double", "mixed"])
def test_condition_numbers_match_numpy_svd(ctx, precision):
    nodes, tris = meshes.icosphere(1.0, 1)   # 80 panels: a 160 x 160 Mueller system
    surf = bemgpu.mesh(nodes, tris)
    sol = bemgpu.bem(surf, bemgpu.FluidFilled(G, H), K, incidence_angle=0.3, ctx=ctx,
                     precision=precision)
    d = sol.diagnostics()
    sol.close()
    A = _fluid_system(nodes, tris)
    _, _, S = O.equilibrate(A)
    assert d["conditioning"] == "svd" and d["condition_limit"] == 512
    # FP64 system: the singular values of the same matrix; mixed: the compact system
    # (FP32 regular pairs), within that assembly's 2e-6
    tol = 1e-9 if precision == "double" else 2e-5
    assert abs(d["condition_number"] / np.linalg.cond(A) - 1) < tol
    # the GPU's scales are FP32 maxima: the scaled matrix differs by a diagonal of 1 + 6e-8
    assert abs(d["scaled_condition_number"] / np.linalg.cond(S) - 1) < 2e-5


def test_conditioning_not_computed_above_the_limit(ctx):
    nodes, tris = meshes.icosphere(1.0, 1)
    surf = bemgpu.mesh(nodes, tris)
    sol = bemgpu.bem(surf, bemgpu.FluidFilled(G, H), K, ctx=ctx, condition_limit=100)
    d = sol.diagnostics()
    sol.close()
    assert d["conditioning"] == "not_computed"
    assert d["condition_number"] is None and d["scaled_condition_number"] is None
    with pytest.raises(bemgpu.ArgumentError):
        bemgpu.bem(surf, bemgpu.FluidFilled(G, H), K, ctx=ctx, condition_limit=-1)


def test_condition_number_of_a_rigid_system_and_without_equilibration(ctx):
    nodes, tris = meshes.icosphere(1.0, 2)   # 320 panels
    surf = bemgpu.mesh(nodes, tris)
    sol = bemgpu.bem(surf, bemgpu.Rigid(), 2.0, ctx=ctx, equilibrate=False)
    d = sol.diagnostics()
    sol.close()
    M1, _ = O.assemble_bm(O.Panels(nodes, tris), 2.0, True)
    assert abs(d["condition_number"] / np.linalg.cond(M1) - 1) < 1e-9
    assert d["scaled_condition_number"] == d["condition_number"]  # equilibrate=false
    assert d["derivative_evaluation"] is None


def test_norm_floor_bounds_the_scales(ctx):
    nodes, tris = meshes.icosphere(1.0, 1)
    surf = bemgpu.mesh(nodes, tris)
    A = _fluid_system(nodes, tris)
    rows = np.max(np.abs(A), axis=1)
    floor = float(np.median(rows))                 # raises half of the row scales
    sol = bemgpu.bem(surf, bemgpu.FluidFilled(G, H), K, incidence_angle=0.3, ctx=ctx,
                     norm_floor=floor)
    d = sol.diagnostics()
    f = bemgpu.scattering_amplitude(sol)
    sol.close()
    _, _, S = O.equilibrate(A, floor)
    assert abs(d["scaled_condition_number"] / np.linalg.cond(S) - 1) < 2e-5
    ref = O.solve(nodes, tris, "fluid", K, incidence_angle=0.3, g=G, h=H, norm_floor=floor)
    assert abs(f - ref["amplitudes"][0]) < 1e-9 * abs(ref["amplitudes"][0])
    with pytest.raises(bemgpu.ArgumentError):
        bemgpu.bem(surf, bemgpu.FluidFilled(G, H), K, ctx=ctx, precision="mixed",
                   norm_floor=floor)


@pytest.mark.parametrize("formulation", ["muller", "cbie"])
def test_derivative_evaluation(ctx, formulation):
    nodes, tris = meshes.icosphere(1.0, 1)
    surf = bemgpu.mesh(nodes, tris)
    sol = bemgpu.bem(surf, bemgpu.FluidFilled(G, H), K, ctx=ctx, formulation=formulation)
    d = sol.diagnostics()
    sol.close()
    if formulation == "muller":
        assert d["derivative_evaluation"] == {"exterior": "direct", "interior": "direct"}
    else:
        assert d["derivative_evaluation"] is None
    assert math.isfinite(d["condition_number"])
