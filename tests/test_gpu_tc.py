"""Tensor-core (tcgen05, split-BF16) complex update and the mixed-precision LU built on it."""
import math

import numpy as np
import pytest

import bemgpu
from bemgpu import meshes
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("m,n,k", [(128, 128, 32), (200, 300, 64), (1000, 700, 128),
                                   (257, 129, 100), (64, 40, 7)])
def test_tc_cgemm_matches_numpy(ctx, m, n, k):
    rng = np.random.default_rng(m + n + k)
    A = (rng.standard_normal((m, k)) + 1j * rng.standard_normal((m, k))).astype(np.complex64)
    B = (rng.standard_normal((k, n)) + 1j * rng.standard_normal((k, n))).astype(np.complex64)
    C = (rng.standard_normal((m, n)) + 1j * rng.standard_normal((m, n))).astype(np.complex64)
    got = ctx.debug_cgemm(A, B, C)
    want = C.astype(np.complex128) - A.astype(np.complex128) @ B.astype(np.complex128)
    err = np.linalg.norm(got - want) / (np.linalg.norm(A) * np.linalg.norm(B) / math.sqrt(k))
    # split-BF16 (3 products) keeps ~16 mantissa bits per operand
    assert err < 5e-5, err


@pytest.mark.parametrize("tensor", [True, False])
def test_mixed_lu_paths_agree_with_fp64(ctx, tensor):
    nodes, tris = meshes.icosphere(1.0, 3)
    surf = bemgpu.mesh(nodes, tris)
    fl = bemgpu.FluidFilled(1.05, 1.02)
    k = 2.0
    dbl = bemgpu.bem(surf, fl, k, incidence_angle=0.4, ctx=ctx)
    ctx.set_tensor_lu(tensor)
    try:
        mix = bemgpu.bem(surf, fl, k, incidence_angle=0.4, precision="mixed",
                         assembly="double", ctx=ctx)
    finally:
        ctx.set_tensor_lu(True)
    d = bemgpu.diagnostics(mix)
    assert d["factor_precision"] == "single", d
    assert d["normwise_backward_error"] <= 1e-13
    assert d["componentwise_backward_error"] <= 1e-13
    a, b = bemgpu.scattering_amplitude(mix), bemgpu.scattering_amplitude(dbl)
    assert abs(a - b) / abs(b) < 1e-8


def test_mixed_rigid_tensor_lu_against_oracle(ctx):
    nodes, tris = meshes.icosphere(0.01, 3)
    k = 2 * math.pi * 38e3 / 1477.4
    surf = bemgpu.mesh(nodes, tris)
    sol = bemgpu.bem(surf, bemgpu.Rigid(), k, incidence_angle=math.pi / 2,
                     incidence_azimuth=math.pi / 2, precision="mixed", ctx=ctx)
    ref = O.solve(nodes, tris, "rigid", k, incidence_angle=math.pi / 2,
                  incidence_azimuth=math.pi / 2)["amplitudes"][0]
    f = bemgpu.scattering_amplitude(sol)
    assert abs(20 * math.log10(abs(f) / abs(ref))) < 0.01
    assert bemgpu.diagnostics(sol)["factor_precision"] == "single"
