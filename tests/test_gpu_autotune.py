"""The launch-shape autotuner only picks among bit-identical launch shapes: results with
it off, on (measuring) and on (reusing its choices) are the same to the last bit."""
import numpy as np
import pytest

import bemgpu
from bemgpu import meshes

pytestmark = pytest.mark.gpu


def test_autotuned_shapes_give_identical_results(ctx):
    # uneven batch: 1280, 1020 and 810 panels (the last two end on a panel narrower than 32)
    surfs = [bemgpu.mesh(*meshes.uv_spheroid(0.02, 0.01, nu, nv, jitter=0.02, seed=1))
             for nu, nv in ((32, 20), (30, 17), (27, 15))]
    fl = bemgpu.FluidFilled(1.0357, 1.0279)
    items = [(s, fl, k, dict(precision="mixed")) for s in surfs for k in (300.0, 600.0)]

    def run():
        fs = bemgpu.factor_batch(items, ctx)
        sols = bemgpu.solve_batch(fs, [[1.2]] * len(fs))
        out = np.array([bemgpu.scattering_amplitude(s) for s in sols])
        for s in sols:
            s.close()
        for f in fs:
            f.close()
        return out

    try:
        ctx.set_autotune(False)
        fixed = run()
        ctx.set_autotune(True)
        measured = run()
        reused = run()
    finally:
        ctx.set_autotune(True)
    assert np.array_equal(fixed, measured)
    assert np.array_equal(measured, reused)


def test_captured_lu_graphs_replay_with_identical_results(ctx):
    """The batched LU's launch sequence is captured the second time a batch shape is met
    and replayed afterwards; graph and eager launches give the same bits."""
    surfs = [bemgpu.mesh(*meshes.uv_spheroid(0.02, 0.01, nu, nv, jitter=0.02, seed=2))
             for nu, nv in ((32, 20), (27, 15))]
    fl = bemgpu.FluidFilled(1.0357, 1.0279)

    def run(ks):
        items = [(s, fl, k, dict(precision="mixed")) for s in surfs for k in ks]
        fs = bemgpu.factor_batch(items, ctx)
        sols = bemgpu.solve_batch(fs, [[0.9]] * len(fs))
        out = np.array([bemgpu.scattering_amplitude(s) for s in sols])
        for s in sols:
            s.close()
        for f in fs:
            f.close()
        return out

    try:
        ctx.set_graphs(False)
        eager = run((310.0, 620.0))
        ctx.set_graphs(True)
        s0 = ctx.graph_stats()
        first = run((310.0, 620.0))      # seen once: eager
        second = run((310.0, 620.0))     # captured and launched
        other = run((280.0, 560.0))      # same shape, new matrices: replayed
        third = run((310.0, 620.0))      # replayed
        s1 = ctx.graph_stats()
        ctx.set_graphs(False)
        other_eager = run((280.0, 560.0))
    finally:
        ctx.set_graphs(True)
    assert s1["captures"] - s0["captures"] == 1
    assert s1["replays"] - s0["replays"] == 2
    for got in (first, second, third):
        assert np.array_equal(got, eager)
    assert np.array_equal(other, other_eager)
