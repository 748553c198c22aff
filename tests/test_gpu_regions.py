"""Coupled fluid regions (solvers/bem/regions.jl): several closed interfaces, nested or
side by side, each operator block evaluated in its region's medium; against the oracle's
restatement of the same block system."""
import math

import numpy as np
import pytest

import bemgpu
from bemgpu import meshes
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _solve_both(ctx, surfs, mats, parents, k, beta, formulation="muller", precision="double"):
    sm = [bemgpu.mesh(*s) for s in surfs]
    fl = [bemgpu.FluidFilled(*m) for m in mats]
    sol = bemgpu.bem(sm, fl, k, parents=parents, incidence_angle=beta, formulation=formulation,
                     precision=precision, ctx=ctx)
    ref = O.solve_regions(surfs, mats, parents, k, incidence_angle=beta,
                          formulation=formulation)
    return sol, ref


def test_single_interface_is_the_fluid_solve(ctx):
    s = meshes.icosphere(1.0, 2)
    surf = bemgpu.mesh(*s)
    fl = bemgpu.FluidFilled(1.07, 1.04)
    one = bemgpu.bem([surf], [fl], 1.4, incidence_angle=0.5, ctx=ctx)
    ref = bemgpu.bem(surf, fl, 1.4, incidence_angle=0.5, ctx=ctx)
    a, b = bemgpu.scattering_amplitude(one), bemgpu.scattering_amplitude(ref)
    assert abs(a - b) <= 1e-12 * abs(b)
    p1, q1 = one.traces()
    p2, q2 = ref.traces()
    assert np.max(np.abs(p1 - p2)) <= 1e-11 * np.max(np.abs(p2))


@pytest.mark.parametrize("formulation", ["muller", "cbie"])
def test_nested_interfaces_match_oracle(ctx, formulation):
    surfs = [meshes.icosphere(1.0, 2), meshes.icosphere(0.5, 1)]
    mats = [(1.05, 1.03), (1.3, 1.2)]
    sol, ref = _solve_both(ctx, surfs, mats, [0, 1], 1.2, 0.3, formulation)
    a = bemgpu.scattering_amplitude(sol)
    assert abs(a - ref["amplitude"]) <= 1e-9 * abs(ref["amplitude"])
    p, v = sol.region_traces()
    n = len(p)
    x = ref["x"]
    assert np.max(np.abs(p - x[:n])) <= 1e-9 * np.max(np.abs(x[:n]))
    assert np.max(np.abs(v - x[n:])) <= 1e-9 * np.max(np.abs(x[n:]))
    ps, _ = sol.traces()
    assert np.all(ps[len(ps) - 80:] == 0)  # inner interface: no far-field contribution


def test_side_by_side_interfaces_match_oracle(ctx):
    """Two bodies in the exterior, close enough for cross near pairs."""
    surfs = [meshes.icosphere(1.0, 1, center=(-1.5, 0.0, 0.0)),
             meshes.icosphere(0.8, 1, center=(1.3, 0.0, 0.0))]
    mats = [(1.1, 1.05), (0.9, 1.1)]
    sol, ref = _solve_both(ctx, surfs, mats, [0, 0], 1.0, 0.0)
    a = bemgpu.scattering_amplitude(sol)
    assert abs(a - ref["amplitude"]) <= 1e-9 * abs(ref["amplitude"])


def test_mixed_precision_regions(ctx):
    surfs = [meshes.icosphere(1.0, 2), meshes.icosphere(0.5, 2)]
    mats = [(1.05, 1.03), (1.3, 1.2)]
    sol, ref = _solve_both(ctx, surfs, mats, [0, 1], 1.2, 0.3, precision="mixed")
    d = bemgpu.diagnostics(sol)
    assert d["normwise_backward_error"] <= 1e-13
    a = bemgpu.scattering_amplitude(sol)
    # FP32 regular-pair quadrature: agreement with the FP64 oracle to 1e-5
    assert abs(a - ref["amplitude"]) <= 1e-5 * abs(ref["amplitude"])


def test_parents_must_match_containment(ctx):
    outer = bemgpu.mesh(*meshes.icosphere(1.0, 1))
    inner = bemgpu.mesh(*meshes.icosphere(0.5, 1))
    fl = [bemgpu.FluidFilled(1.1, 1.0), bemgpu.FluidFilled(1.2, 1.0)]
    with pytest.raises(bemgpu.ArgumentError):
        bemgpu.bem([outer, inner], fl, 1.0, parents=[0, 0], ctx=ctx)  # inner is inside
    with pytest.raises(bemgpu.ArgumentError):
        bemgpu.bem([outer, inner], fl, 1.0, parents=[0, 2], ctx=ctx)  # not an earlier region


@pytest.mark.parametrize("formulation", ["muller", "cbie"])
def test_region_pressure_matches_oracle(ctx, formulation):
    """pressure(sol, points; field, region) of a coupled-region solution
    (fields/regions.jl:1-65): points outside, between the shells and inside the core, every
    field, region selection; against the oracle's restatement on the oracle's solution."""
    surfs = [meshes.icosphere(1.0, 2), meshes.icosphere(0.5, 1)]
    mats = [(1.05, 1.03), (1.3, 1.2)]
    k, beta = 1.2, 0.3
    sol, ref = _solve_both(ctx, surfs, mats, [0, 1], k, beta, formulation)
    d = O.incidence_direction(beta, 0.0)
    rng = np.random.default_rng(3)

    def shell(r0, r1, m):
        v = rng.standard_normal((m, 3))
        return v / np.linalg.norm(v, axis=1)[:, None] * rng.uniform(r0, r1, m)[:, None]

    outside, between, core = shell(1.3, 2.5, 6), shell(0.7, 0.85, 6), shell(0.05, 0.3, 6)
    cases = [(outside, "total", None), (outside, "scattered", None), (outside, "incident", None),
             (between, "total", None), (between, "interior", None), (core, "total", None),
             (core, "interior", 2), (between, "total", 1)]
    for pts, field, region in cases:
        got = sol.pressure(pts, field=field, region=region)
        want = O.pressure_regions(surfs, mats, [0, 1], k, pts, ref["x"], d, field=field,
                                  region=region)
        assert np.max(np.abs(got - want)) <= 1e-8 * np.max(np.abs(want)), (field, region)
    with pytest.raises(bemgpu.ArgumentError):
        sol.pressure(between, field="scattered")
    with pytest.raises(bemgpu.ArgumentError):
        sol.pressure(outside, field="interior")
    with pytest.raises(bemgpu.ArgumentError):
        sol.pressure(core, field="total", region=1)
    with pytest.raises(bemgpu.ArgumentError):
        sol.pressure(core, field="total", region=5)


def _nystrom_both(ctx, surfs, mats, parents, k, beta, formulation="muller", precision="double"):
    from oracle import nystrom as NY
    sm = [bemgpu.mesh(*s) for s in surfs]
    fl = [bemgpu.FluidFilled(*m) for m in mats]
    sol = bemgpu.bem(sm, fl, k, parents=parents, incidence_angle=beta, formulation=formulation,
                     precision=precision, ctx=ctx, discretization="nystrom")
    ref = NY.solve_regions(surfs, mats, parents, k, incidence_angle=beta,
                           formulation=formulation)
    return sol, ref


def test_nystrom_single_interface_is_the_nystrom_fluid_solve(ctx):
    """One interface in the exterior: the region block system on the quadrature nodes is
    the single-surface Nyström fluid system."""
    s = meshes.icosphere(1.0, 1)
    surf = bemgpu.mesh(*s)
    fl = bemgpu.FluidFilled(1.07, 1.04)
    one = bemgpu.bem([surf], [fl], 1.4, incidence_angle=0.5, ctx=ctx, discretization="nystrom")
    ref = bemgpu.bem(surf, fl, 1.4, incidence_angle=0.5, ctx=ctx, discretization="nystrom")
    a, b = bemgpu.scattering_amplitude(one), bemgpu.scattering_amplitude(ref)
    assert abs(a - b) <= 1e-11 * abs(b)
    one.close()
    ref.close()


@pytest.mark.parametrize("formulation", ["muller", "cbie"])
def test_nystrom_nested_interfaces_match_oracle(ctx, formulation):
    """Nested interfaces on the quadrature nodes (each surface's own operators corrected at
    the wavenumbers of both its regions): = the oracle's node restatement
    (oracle/nystrom.py:assemble_regions) to 1e-9 in amplitude and unknowns."""
    surfs = [meshes.icosphere(1.0, 1), meshes.icosphere(0.5, 1)]
    mats = [(1.05, 1.03), (1.3, 1.2)]
    sol, ref = _nystrom_both(ctx, surfs, mats, [0, 1], 1.2, 0.3, formulation)
    a = bemgpu.scattering_amplitude(sol)
    assert abs(a - ref["amplitude"]) <= 1e-9 * abs(ref["amplitude"])
    p, v = sol.region_traces()
    n = len(p)
    x = ref["x"]
    assert n == 2 * 80 * 7
    assert np.max(np.abs(p - x[:n])) <= 1e-9 * np.max(np.abs(x[:n]))
    assert np.max(np.abs(v - x[n:])) <= 1e-9 * np.max(np.abs(x[n:]))
    sol.close()


def test_nystrom_side_by_side_and_mixed_precision(ctx):
    """Two bodies in the exterior on the nodes: FP64 = the oracle to 1e-9, mixed precision
    within 0.01 dB with the refinement's backward error at its 1e-13 acceptance."""
    surfs = [meshes.icosphere(1.0, 1, center=(-1.5, 0.0, 0.0)),
             meshes.icosphere(0.8, 1, center=(1.3, 0.0, 0.0))]
    mats = [(1.1, 1.05), (0.9, 1.1)]
    sol, ref = _nystrom_both(ctx, surfs, mats, [0, 0], 1.0, 0.0)
    a = bemgpu.scattering_amplitude(sol)
    assert abs(a - ref["amplitude"]) <= 1e-9 * abs(ref["amplitude"])
    sol.close()
    mix, _ = _nystrom_both(ctx, surfs, mats, [0, 0], 1.0, 0.0, precision="mixed")
    m = bemgpu.scattering_amplitude(mix)
    assert abs(20 * math.log10(abs(m) / abs(a))) < 0.01
    assert mix.diagnostics()["normwise_backward_error"] <= 1e-13
    mix.close()
