"""pressure(sol, points; field) on the GPU against the oracle's layer potentials, and the
reference's own consistency contracts (fields/pressure.jl; sphere/full3d.jl:293-347)."""
import math

import numpy as np
import pytest

import bemgpu
from bemgpu import meshes
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _solve(boundary, **kw):
    nodes, tris = meshes.icosphere(1.0, 2)
    surf = bemgpu.mesh(nodes, tris)
    sol = bemgpu.bem(surf, boundary, 1.3, incidence_angle=math.pi / 3, incidence_azimuth=0.4,
                     **kw)
    return nodes, tris, sol


def _points():
    dirs = np.array([[1.0, 0, 0], [0.0, 0.6, 0.8], [-0.6, 0.0, 0.8]])
    return np.array([r * d for r in (1.001, 1.1, 2.0, 5.0) for d in dirs])


@pytest.mark.parametrize("bc", [bemgpu.Rigid(), bemgpu.PressureRelease(),
                                bemgpu.FluidFilled(1.2, 1.1)])
def test_scattered_pressure_matches_oracle(ctx, bc):
    nodes, tris, sol = _solve(bc, ctx=ctx)
    pts = _points()
    got = bemgpu.pressure(sol, pts, field="scattered")
    P = O.Panels(nodes, tris)
    d = O.incidence_direction(math.pi / 3, 0.4)
    p, q = sol.traces()
    fl = isinstance(bc, bemgpu.FluidFilled)
    want = O.pressure(P, 1.3, pts, p, q, d, field="scattered", fluid=fl)
    assert np.max(np.abs(got - want) / np.abs(want)) < 1e-9
    total = bemgpu.pressure(sol, pts)
    inc = bemgpu.pressure(sol, pts, field="incident")
    assert np.allclose(total, inc + got, rtol=1e-12, atol=1e-14)


def test_interior_pressure_matches_oracle(ctx):
    bc = bemgpu.FluidFilled(1.2, 1.1)
    nodes, tris, sol = _solve(bc, ctx=ctx)
    pts = np.array([[0.0, 0.0, 0.0], [0.3, 0.2, -0.1], [0.0, 0.6, 0.7]])
    got = bemgpu.pressure(sol, pts, field="interior")
    P = O.Panels(nodes, tris)
    d = O.incidence_direction(math.pi / 3, 0.4)
    p, q = sol.traces()
    want = O.pressure(P, 1.3, pts, p, q, d, field="interior", g=1.2, h=1.1, fluid=True)
    assert np.max(np.abs(got - want) / np.abs(want)) < 1e-9
    assert np.allclose(bemgpu.pressure(sol, pts), got, rtol=1e-12)


def test_far_pressure_is_the_scattering_amplitude(ctx):
    _, _, sol = _solve(bemgpu.Rigid(), ctx=ctx)
    direction, dist = np.array([0.36, 0.48, 0.8]), 1e6
    far = bemgpu.pressure(sol, dist * direction, field="scattered") * dist \
        * np.exp(-1j * sol.k * dist)
    amp = bemgpu.scattering_amplitude(sol, direction=direction)
    assert abs(far - amp) <= 1e-4 * abs(amp) + 1e-12


def test_pressure_argument_errors(ctx):
    _, _, sol = _solve(bemgpu.Rigid(), ctx=ctx)
    with pytest.raises(bemgpu.ArgumentError):
        bemgpu.pressure(sol, (0.0, 0.0, 0.0))          # inside a rigid body
    with pytest.raises(bemgpu.ArgumentError):
        bemgpu.pressure(sol, (math.nan, 0.0, 0.0))
    with pytest.raises(bemgpu.ArgumentError):
        bemgpu.pressure(sol, (2.0, 0.0, 0.0), field="interior")
    assert bemgpu.pressure(sol, np.zeros((0, 3))).size == 0
