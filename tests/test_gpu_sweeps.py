"""Sweeps (postprocessing/sweeps.jl): many incidence angles from one factor as one
multi-right-hand-side batch, and frequency sweeps, against one-at-a-time solves."""
import math

import numpy as np
import pytest

import bemgpu

pytestmark = pytest.mark.gpu

ANGLES = np.linspace(0.1, math.pi - 0.1, 9)   # 9 rhs: groups of 4, 4 and 1


@pytest.mark.parametrize("precision", ["double", "mixed"])
@pytest.mark.parametrize("boundary", ["rigid", "fluid"])
def test_angle_sweep_matches_single_solves(ctx, precision, boundary):
    surf = bemgpu.mesh(*bemgpu.meshes.icosphere(0.01, 2))
    bc = bemgpu.Rigid() if boundary == "rigid" else bemgpu.FluidFilled(1.05, 1.03)
    k = 250.0
    sw = bemgpu.incidence_angle_sweep(surf, bc, k, ANGLES, precision=precision, ctx=ctx)
    assert sw.amplitudes.shape == (len(ANGLES),)
    for r, ang in enumerate(ANGLES):
        sol = bemgpu.bem(surf, bc, k, incidence_angle=ang, precision=precision, ctx=ctx)
        want = bemgpu.scattering_amplitude(sol)
        # same factor, same refinement path per rhs: agreement to the refinement contract
        assert abs(sw.amplitudes[r] - want) <= 1e-10 * abs(want), (r, sw.amplitudes[r], want)
    assert np.allclose(sw.target_strength, 20 * np.log10(np.abs(sw.amplitudes)))


def test_angle_sweep_symmetry_of_sphere(ctx):
    """Backscatter of a sphere does not depend on the incidence direction (to the mesh)."""
    surf = bemgpu.mesh(*bemgpu.meshes.icosphere(0.01, 3))
    sw = bemgpu.incidence_angle_sweep(surf, bemgpu.Rigid(), 300.0, ANGLES, ctx=ctx)
    ts = sw.target_strength
    assert np.max(ts) - np.min(ts) < 0.05


def test_frequency_sweep_batched_equals_loop(ctx):
    surf = bemgpu.mesh(*bemgpu.meshes.uv_spheroid(0.02, 0.008, 24, 12, jitter=0.02, seed=3))
    fl = bemgpu.FluidFilled(1.0357, 1.0279)
    freqs = np.array([20e3, 45e3, 70e3])
    c = 1500.0
    loop = bemgpu.frequency_sweep(
        lambda k: bemgpu.bem(surf, fl, k, precision="mixed", ctx=ctx), freqs, c)
    items = [(surf, fl, float(k), dict(precision="mixed")) for k in loop.k]
    fs = bemgpu.factor_batch(items, ctx)
    sols = bemgpu.solve_batch(fs, [[math.pi / 2]] * len(fs), [[0.0]] * len(fs))
    amps = np.array([bemgpu.scattering_amplitude(s) for s in sols])
    # one batch and one-at-a-time run the same arithmetic per instance
    assert np.array_equal(amps, loop.amplitudes)
