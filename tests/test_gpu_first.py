"""First GPU parity checks of libbemgpu against the CPU oracle."""
import math

import numpy as np
import pytest

import bemgpu
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _sphere(sub=2, r=1.0):
    return bemgpu.meshes.icosphere(r, sub)


@pytest.mark.parametrize("boundary", ["rigid", "pressure_release"])
@pytest.mark.parametrize("formulation", ["burton_miller", "cbie"])
def test_bm_operators_match_oracle(ctx, boundary, formulation):
    nodes, tris = _sphere(1)
    k = 2.3
    surf = bemgpu.mesh(nodes, tris)
    bc = bemgpu.Rigid() if boundary == "rigid" else bemgpu.PressureRelease()
    M1, M2 = bemgpu.assemble(surf, bc, k, formulation=formulation, ctx=ctx)
    P = O.Panels(nodes, tris)
    R1, R2 = O.assemble_bm(P, k, formulation == "burton_miller")
    for a, b in ((M1, R1), (M2, R2)):
        err = np.max(np.abs(a - b)) / np.max(np.abs(b))
        assert err < 1e-12, err


@pytest.mark.parametrize("boundary", ["rigid", "pressure_release"])
def test_bm_solve_matches_oracle(ctx, boundary):
    nodes, tris = _sphere(2)
    k = 1.7
    surf = bemgpu.mesh(nodes, tris)
    bc = bemgpu.Rigid() if boundary == "rigid" else bemgpu.PressureRelease()
    sol = bemgpu.bem(surf, bc, k, incidence_angle=0.4, incidence_azimuth=0.3, ctx=ctx)
    f = bemgpu.scattering_amplitude(sol)
    ref = O.solve(nodes, tris, boundary, k, incidence_angle=0.4, incidence_azimuth=0.3)
    rel = abs(f - ref["amplitudes"][0]) / abs(ref["amplitudes"][0])
    assert rel < 1e-9, rel


@pytest.mark.parametrize("formulation", ["muller", "cbie"])
def test_fluid_solve_matches_oracle(ctx, formulation):
    nodes, tris = _sphere(2)
    k, g, h = 1.5, 1.04, 1.04
    surf = bemgpu.mesh(nodes, tris)
    sol = bemgpu.bem(surf, bemgpu.FluidFilled(g, h), k, incidence_angle=0.0,
                     formulation=formulation, ctx=ctx)
    f = bemgpu.scattering_amplitude(sol)
    ref = O.solve(nodes, tris, "fluid", k, incidence_angle=0.0, g=g, h=h,
                  formulation=formulation)
    rel = abs(f - ref["amplitudes"][0]) / abs(ref["amplitudes"][0])
    assert rel < 1e-9, rel


def test_mixed_refinement_contract(ctx):
    nodes, tris = _sphere(2)
    k = 1.5
    surf = bemgpu.mesh(nodes, tris)
    fl = bemgpu.FluidFilled(1.05, 1.02)
    dbl = bemgpu.bem(surf, fl, k, incidence_angle=0.4, ctx=ctx)
    mix = bemgpu.bem(surf, fl, k, incidence_angle=0.4, precision="mixed", assembly="double",
                     ctx=ctx)
    d = bemgpu.diagnostics(mix)
    assert d["factor_precision"] == "single"
    assert d["normwise_backward_error"] <= 1e-13
    assert d["componentwise_backward_error"] <= 1e-13
    a, b = bemgpu.scattering_amplitude(mix), bemgpu.scattering_amplitude(dbl)
    assert abs(a - b) / abs(b) < 1e-8
