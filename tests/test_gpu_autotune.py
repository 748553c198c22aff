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
