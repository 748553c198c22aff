"""Compact mixed-precision storage of the system (complex64 values, exact for the FP32
regular-pair rule, plus FP64 corrections at the near pairs): the expanded matrix, the
residuals the refinement computes from it in FP32 pair arithmetic, and the solutions."""
import math

import numpy as np
import pytest

import bemgpu
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _fluid_case():
    nodes, tris = bemgpu.meshes.icosphere(1.0, 2)
    return nodes, tris, bemgpu.mesh(nodes, tris), 1.5, 1.05, 1.02


def test_compact_matrix_matches_oracle(ctx):
    nodes, tris, surf, k, g, h = _fluid_case()
    M = bemgpu.assemble(surf, bemgpu.FluidFilled(g, h), k, precision="mixed", ctx=ctx)
    R = O.assemble_fluid(O.Panels(nodes, tris), k, g, h)
    # FP32 quadrature of the regular pairs: relative 1e-6 of the largest entry
    assert np.max(np.abs(M - R)) / np.max(np.abs(R)) < 2e-6
    D = bemgpu.assemble(surf, bemgpu.FluidFilled(g, h), k, precision="mixed",
                        assembly="double", ctx=ctx)
    assert np.max(np.abs(D - R)) / np.max(np.abs(R)) < 1e-12


@pytest.mark.parametrize("formulation", ["muller", "cbie"])
def test_compact_refinement_solves_the_fp32_assembled_system(ctx, formulation):
    """The refined solution solves the expanded compact system to the FP64 contract."""
    nodes, tris, surf, k, g, h = _fluid_case()
    fl = bemgpu.FluidFilled(g, h)
    beta = 0.4
    sol = bemgpu.bem(surf, fl, k, incidence_angle=beta, precision="mixed",
                     formulation=formulation, ctx=ctx)
    d = bemgpu.diagnostics(sol)
    assert d["factor_precision"] == "single"
    assert d["normwise_backward_error"] <= 1e-13
    M = bemgpu.assemble(surf, fl, k, precision="mixed", formulation=formulation, ctx=ctx)
    P = O.Panels(nodes, tris)
    pinc, qinc = O.incident(P, k, O.incidence_direction(beta, 0.0))
    ps, qs = sol.traces()
    n = len(ps)
    if formulation == "muller":
        x = np.concatenate([ps + pinc, qs + qinc])
        b = np.concatenate([pinc, qinc])
        r = M @ x - b
        nw = np.max(np.abs(r)) / (np.max(np.abs(M).sum(axis=1)) * np.max(np.abs(x)) +
                                  np.max(np.abs(b)))
        assert nw < 1e-13, nw
    # and the amplitude agrees with the all-FP64 solve to the FP32 quadrature level
    dbl = bemgpu.bem(surf, fl, k, incidence_angle=beta, formulation=formulation, ctx=ctx)
    a, b_ = bemgpu.scattering_amplitude(sol), bemgpu.scattering_amplitude(dbl)
    assert abs(a - b_) / abs(b_) < 1e-5
    assert n == surf.n_panels


@pytest.mark.parametrize("boundary", ["rigid", "pressure_release"])
def test_compact_bm_matches_double(ctx, boundary):
    nodes, tris = bemgpu.meshes.icosphere(1.0, 2)
    surf = bemgpu.mesh(nodes, tris)
    bc = bemgpu.Rigid() if boundary == "rigid" else bemgpu.PressureRelease()
    k = 2.1
    mix = bemgpu.bem(surf, bc, k, incidence_angle=0.7, precision="mixed", ctx=ctx)
    dbl = bemgpu.bem(surf, bc, k, incidence_angle=0.7, ctx=ctx)
    d = bemgpu.diagnostics(mix)
    assert d["normwise_backward_error"] <= 1e-13
    a, b = bemgpu.scattering_amplitude(mix), bemgpu.scattering_amplitude(dbl)
    assert abs(a - b) / abs(b) < 1e-5
    M1, M2 = bemgpu.assemble(surf, bc, k, precision="mixed", ctx=ctx)
    R1, R2 = O.assemble_bm(O.Panels(nodes, tris), k, True)
    for A_, R_ in ((M1, R1), (M2, R2)):
        assert np.max(np.abs(A_ - R_)) / np.max(np.abs(R_)) < 2e-6


def test_compact_promotion_uses_exact_near_values(ctx):
    """A condition guard above 1 forces the FP64 fallback from the compact system; the
    promoted factor must reproduce the all-FP64 solve of the FP32-assembled matrix."""
    nodes, tris, surf, k, g, h = _fluid_case()
    fl = bemgpu.FluidFilled(g, h)
    sol = bemgpu.bem(surf, fl, k, incidence_angle=0.2, precision="mixed",
                     refinement=dict(condition_guard=2.0), ctx=ctx)
    d = bemgpu.diagnostics(sol)
    assert d["factor_precision"] == "double"
    M = bemgpu.assemble(surf, fl, k, precision="mixed", ctx=ctx)
    P = O.Panels(nodes, tris)
    pinc, qinc = O.incident(P, k, O.incidence_direction(0.2, 0.0))
    b = np.concatenate([pinc, qinc])
    x = np.linalg.solve(M, b)
    ps, qs = sol.traces()
    got = np.concatenate([ps + pinc, qs + qinc])
    assert np.max(np.abs(got - x)) / np.max(np.abs(x)) < 1e-11
