"""Nyström discretisation on the GPU against its CPU oracle (oracle/nystrom.py).

Operator entries after the element corrections within 1e-11 of the largest entry; FP64
traces and far field within 1e-9; the mixed factor with refinement within 0.01 dB and the
reference's backward-error contract (fluid_system.jl:172-309); many incidences from one
factor equal separate solves (sweeps.jl:680-701); the 1280-panel sphere within the
reference's 0.1 dB of the modal series; the field at points (nearest element recovered
by the fit) equal to the oracle's; unsupported combinations rejected.
"""
import math

import numpy as np
import pytest

import bemgpu
from bemgpu import meshes
from oracle import modal
from oracle import nystrom as NY
from oracle import oracle as O

pytestmark = pytest.mark.gpu

K38 = 2 * math.pi * 38e3 / 1477.4


def _bc(name):
    return bemgpu.Rigid() if name == "rigid" else bemgpu.PressureRelease()


@pytest.mark.parametrize("boundary", ["rigid", "pressure_release"])
@pytest.mark.parametrize("formulation", ["burton_miller", "cbie"])
def test_node_operators_match_oracle(ctx, boundary, formulation):
    nodes, tris = meshes.icosphere(0.01, 1)
    surf = bemgpu.mesh(nodes, tris)
    M1, M2 = bemgpu.assemble(surf, _bc(boundary), K38, formulation=formulation, ctx=ctx,
                             discretization="nystrom")
    R1, R2 = NY.assemble(O.Panels(nodes, tris), K38, formulation == "burton_miller")
    assert M1.shape == (7 * 80, 7 * 80)
    for a, b in ((M1, R1), (M2, R2)):
        err = np.max(np.abs(a - b)) / np.max(np.abs(b))
        assert err < 1e-11, err


@pytest.mark.parametrize("boundary", ["rigid", "pressure_release"])
@pytest.mark.parametrize("formulation", ["burton_miller", "cbie"])
def test_fp64_solve_matches_oracle(ctx, boundary, formulation):
    nodes, tris = meshes.icosphere(0.01, 2)
    surf = bemgpu.mesh(nodes, tris)
    beta, alpha = 0.7, 0.4
    sol = bemgpu.bem(surf, _bc(boundary), K38, incidence_angle=beta, incidence_azimuth=alpha,
                     formulation=formulation, ctx=ctx, discretization="nystrom")
    p, q = sol.traces()
    rp, rq, (y, ny, w) = NY.solve(nodes, tris, boundary, K38, beta, alpha, formulation)
    assert p.shape == (7 * 320,)
    for a, b in ((p, rp), (q, rq)):
        assert np.linalg.norm(a - b) <= 1e-9 * np.linalg.norm(b)
    d = O.incidence_direction(beta, alpha)
    for xh in (-d, d, np.array([0.0, 0.6, 0.8])):
        ref = NY.far_field(y, ny, w, K38, xh, rp, rq)
        got = sol.far_field(xh)[0]
        assert abs(got - ref) <= 1e-9 * abs(ref)
    diag = sol.diagnostics()
    assert diag["discretization"] == "nystrom"
    assert diag["unknown_count"] == 7 * 320
    sol.close()


def test_jittered_spheroid_matches_oracle(ctx):
    nodes, tris = meshes.uv_spheroid(0.02, 0.01, 16, 10, jitter=0.02, seed=5)
    surf = bemgpu.mesh(nodes, tris)
    k = 2 * math.pi * 70e3 / 1500.0
    sol = bemgpu.bem(surf, bemgpu.Rigid(), k, incidence_angle=1.1, ctx=ctx,
                     discretization="nystrom")
    rp, rq, (y, ny, w) = NY.solve(nodes, tris, "rigid", k, 1.1, 0.0)
    d = O.incidence_direction(1.1, 0.0)
    ref = NY.far_field(y, ny, w, k, -d, rp, rq)
    got = bemgpu.scattering_amplitude(sol)
    assert abs(got - ref) <= 1e-9 * abs(ref)
    sol.close()


@pytest.mark.parametrize("boundary", ["rigid", "pressure_release"])
def test_mixed_refinement_contract(ctx, boundary):
    nodes, tris = meshes.icosphere(0.01, 2)
    surf = bemgpu.mesh(nodes, tris)
    sd = bemgpu.bem(surf, _bc(boundary), K38, ctx=ctx, discretization="nystrom")
    sm = bemgpu.bem(surf, _bc(boundary), K38, ctx=ctx, discretization="nystrom",
                    precision="mixed")
    fd, fm = bemgpu.scattering_amplitude(sd), bemgpu.scattering_amplitude(sm)
    assert abs(20 * math.log10(abs(fm) / abs(fd))) < 0.01
    assert abs(fm - fd) <= 1e-8 * abs(fd)
    dm = sm.diagnostics()
    assert dm["normwise_backward_error"] <= 1e-13
    assert dm["componentwise_backward_error"] <= 1e-13
    sd.close()
    sm.close()


def test_sweep_equals_separate_solves(ctx):
    nodes, tris = meshes.icosphere(0.01, 2)
    surf = bemgpu.mesh(nodes, tris)
    angles = np.array([0.0, 0.9, 2.2, math.pi])
    sw = bemgpu.incidence_angle_sweep(surf, bemgpu.Rigid(), K38, angles, ctx=ctx,
                                      discretization="nystrom")
    for a, amp in zip(angles, sw.amplitudes):
        sol = bemgpu.bem(surf, bemgpu.Rigid(), K38, incidence_angle=a, ctx=ctx,
                         discretization="nystrom")
        one = bemgpu.scattering_amplitude(sol)
        assert abs(amp - one) <= 1e-12 * abs(one)
        sol.close()


@pytest.mark.parametrize("boundary", ["rigid", "pressure_release"])
def test_sphere_1280_panels_against_modal(ctx, boundary):
    a = 0.01
    nodes, tris = meshes.icosphere(a, 3)
    surf = bemgpu.mesh(nodes, tris)
    sol = bemgpu.bem(surf, _bc(boundary), K38, incidence_angle=math.pi / 2,
                     incidence_azimuth=math.pi / 2, ctx=ctx, discretization="nystrom")
    f = bemgpu.scattering_amplitude(sol)
    fm = modal.form_function(boundary, K38, a)
    assert abs(20 * math.log10(abs(f) / abs(fm))) < 0.1
    assert abs(f - fm) < 0.02 * abs(fm)
    sol.close()


@pytest.mark.parametrize("boundary", ["rigid", "pressure_release"])
def test_point_field_matches_oracle(ctx, boundary):
    a = 0.01
    nodes, tris = meshes.icosphere(a, 2)
    surf = bemgpu.mesh(nodes, tris)
    beta, alpha = 0.7, 0.4
    sol = bemgpu.bem(surf, _bc(boundary), K38, incidence_angle=beta, incidence_azimuth=alpha,
                     ctx=ctx, discretization="nystrom")
    p, q = sol.traces()
    d = O.incidence_direction(beta, alpha)
    dirs = np.array([[1.0, 0, 0], [0.0, 0.6, 0.8], [-0.6, 0.0, 0.8], [0.0, 0.0, -1.0]])
    pts = np.concatenate([rf * a * dirs for rf in (1.005, 1.05, 1.3, 3.0)])
    P = O.Panels(nodes, tris)
    got = bemgpu.pressure(sol, pts, field="scattered")
    want = NY.pressure(P, K38, pts, p, q, d, "scattered")
    assert np.max(np.abs(got - want) / np.abs(want)) < 1e-9
    inc = bemgpu.pressure(sol, pts, field="incident")
    assert np.allclose(inc, np.exp(1j * K38 * (pts @ d)), rtol=1e-14, atol=1e-15)
    assert np.allclose(bemgpu.pressure(sol, pts), inc + got, rtol=1e-12, atol=1e-15)
    with pytest.raises(bemgpu.ArgumentError):  # inside the body
        bemgpu.pressure(sol, np.zeros((1, 3)))
    far_dir, dist = np.array([0.36, 0.48, 0.8]), 1e4
    far = bemgpu.pressure(sol, dist * far_dir, field="scattered") * dist \
        * np.exp(-1j * K38 * dist)
    amp = bemgpu.scattering_amplitude(sol, direction=far_dir)
    assert abs(far - amp) <= 1e-3 * abs(amp)
    sol.close()


G_FL, H_FL = 1.0357, 1.0279


@pytest.mark.parametrize("formulation", ["muller", "cbie"])
def test_fluid_operators_match_oracle(ctx, formulation):
    nodes, tris = meshes.icosphere(0.01, 1)
    surf = bemgpu.mesh(nodes, tris)
    A = bemgpu.assemble(surf, bemgpu.FluidFilled(G_FL, H_FL), K38, formulation=formulation,
                        ctx=ctx, discretization="nystrom")
    R = NY.assemble_fluid(O.Panels(nodes, tris), K38, G_FL, H_FL, formulation)
    assert A.shape == (2 * 7 * 80, 2 * 7 * 80)
    assert np.max(np.abs(A - R)) / np.max(np.abs(R)) < 1e-11


@pytest.mark.parametrize("formulation", ["muller", "cbie"])
def test_fluid_solve_and_field_match_oracle(ctx, formulation):
    a = 0.01
    nodes, tris = meshes.icosphere(a, 2)
    surf = bemgpu.mesh(nodes, tris)
    beta, alpha = 0.7, 0.4
    bc = bemgpu.FluidFilled(G_FL, H_FL)
    sol = bemgpu.bem(surf, bc, K38, incidence_angle=beta, incidence_azimuth=alpha,
                     formulation=formulation, ctx=ctx, discretization="nystrom")
    p, q = sol.traces()
    rp, rq, (y, ny, w) = NY.solve(nodes, tris, "fluid", K38, beta, alpha, formulation,
                                  G_FL, H_FL)
    for u, v in ((p, rp), (q, rq)):
        assert np.linalg.norm(u - v) <= 1e-9 * np.linalg.norm(v)
    d = O.incidence_direction(beta, alpha)
    ref = NY.far_field(y, ny, w, K38, -d, rp, rq)
    assert abs(bemgpu.scattering_amplitude(sol) - ref) <= 1e-9 * abs(ref)
    P = O.Panels(nodes, tris)
    dirs = np.array([[1.0, 0, 0], [0.0, 0.6, 0.8], [-0.6, 0.0, 0.8]])
    cen = P.centroids[[3, 101, 250]]  # on the facets: just inside / outside the polyhedron
    outside = np.concatenate([1.003 * cen] + [rf * a * dirs for rf in (1.005, 1.3)])
    inside = np.concatenate([0.997 * cen] + [rf * a * dirs for rf in (0.9, 0.5)] +
                            [np.zeros((1, 3))])
    got = bemgpu.pressure(sol, outside, field="scattered")
    want = NY.pressure(P, K38, outside, p, q, d, "scattered", g=G_FL, h=H_FL)
    assert np.max(np.abs(got - want) / np.abs(want)) < 1e-9
    got = bemgpu.pressure(sol, inside, field="interior")
    want = NY.pressure(P, K38, inside, p, q, d, "interior", g=G_FL, h=H_FL)
    assert np.max(np.abs(got - want) / np.abs(want)) < 1e-9
    assert np.allclose(bemgpu.pressure(sol, inside), got, rtol=1e-12)
    with pytest.raises(bemgpu.ArgumentError):
        bemgpu.pressure(sol, outside, field="interior")
    sol.close()


def test_fluid_mixed_refinement_contract(ctx):
    nodes, tris = meshes.icosphere(0.01, 2)
    surf = bemgpu.mesh(nodes, tris)
    bc = bemgpu.FluidFilled(G_FL, H_FL)
    sd = bemgpu.bem(surf, bc, K38, ctx=ctx, discretization="nystrom")
    sm = bemgpu.bem(surf, bc, K38, ctx=ctx, discretization="nystrom", precision="mixed")
    fd, fm = bemgpu.scattering_amplitude(sd), bemgpu.scattering_amplitude(sm)
    assert abs(20 * math.log10(abs(fm) / abs(fd))) < 0.01
    dm = sm.diagnostics()
    assert dm["normwise_backward_error"] <= 1e-13
    sd.close()
    sm.close()


def test_compressed_node_operators_match_dense(ctx):
    """The reference's default configuration: Nyström nodes + compressed operators +
    GMRES.  At tol 1e-10 and reltol 1e-11 the solution equals the dense oracle's."""
    nodes, tris = meshes.icosphere(0.01, 2)
    surf = bemgpu.mesh(nodes, tris)
    beta, alpha = 0.7, 0.4
    sol = bemgpu.bem(surf, bemgpu.Rigid(), K38, incidence_angle=beta, incidence_azimuth=alpha,
                     ctx=ctx, discretization="nystrom",
                     compression=dict(method="hmatrix", tol=1e-10, leaf_size=32),
                     gmres_kwargs=dict(reltol=1e-11, restart=500, maxiter=4000))
    st = sol.hmatrix_stats()
    assert st["lowrank_blocks"] > 0 and st["gmres_converged"]
    p, q = sol.traces()
    rp, rq, (y, ny, w) = NY.solve(nodes, tris, "rigid", K38, beta, alpha)
    for u, v in ((p, rp), (q, rq)):
        assert np.linalg.norm(u - v) <= 1e-8 * np.linalg.norm(v)
    d = O.incidence_direction(beta, alpha)
    ref = NY.far_field(y, ny, w, K38, -d, rp, rq)
    assert abs(bemgpu.scattering_amplitude(sol) - ref) <= 1e-8 * abs(ref)
    sol.close()


def test_compressed_soft_gmres_is_block_preconditioned(ctx):
    """The Nyström soft system's eigenvalues straddle the imaginary axis, where restarted
    GMRES stalls (the oracle's GMRES on the dense matrix shows it); the compressed solve
    iterates on A P^-1, P the element blocks (right preconditioning: the residual stays
    b - A x), following the oracle's GMRES on the dense A P^-1 step by step to the dense
    solution."""
    nodes, tris = meshes.icosphere(0.01, 2)
    surf = bemgpu.mesh(nodes, tris)
    kw = dict(reltol=1e-10, restart=150, maxiter=300)
    sol = bemgpu.bem(surf, bemgpu.PressureRelease(), K38, incidence_angle=0.7,
                     incidence_azimuth=0.4, ctx=ctx, discretization="nystrom",
                     compression=dict(method="hmatrix", tol=1e-12, leaf_size=32),
                     gmres_kwargs=kw)
    P = O.Panels(nodes, tris)
    M1, M2 = NY.assemble(P, K38, True)
    y, ny, w = NY.nodes_of(P)
    d = O.incidence_direction(0.7, 0.4)
    b = M1 @ np.exp(1j * K38 * (y @ d))
    _, plain = O.gmres(M2, b, **kw)
    assert not plain["converged"]
    Pinv = np.zeros_like(M2)
    for e in range(M2.shape[0] // 7):
        c = slice(7 * e, 7 * e + 7)
        Pinv[c, c] = np.linalg.inv(M2[c, c])
    _, info = O.gmres(M2 @ Pinv, b, **kw)
    st = sol.hmatrix_stats()
    hist = sol.residual_history(0)
    assert info["converged"] and st["gmres_converged"]
    assert abs(st["gmres_iterations"] - info["iterations"]) <= 1
    m = min(len(hist), len(info["history"]))
    bn = np.linalg.norm(b)
    assert np.all(np.abs(hist[:m] - info["history"][:m]) <= 1e-6 * info["history"][:m] + 1e-11 * bn)
    p, q = sol.traces()
    rp, rq, _ = NY.solve(nodes, tris, "pressure_release", K38, 0.7, 0.4)
    assert np.linalg.norm(q - rq) <= 1e-8 * np.linalg.norm(rq)
    sol.close()


def test_compressed_rigid_gmres_is_schwarz_preconditioned(ctx):
    """The rigid node system's spectrum spreads as the mesh is refined (restarted GMRES:
    about 300 steps to 1e-6 at 320 panels, 630 at 1280, beyond 1200 at 5120); with
    `neighbours=48` the compressed solve iterates on A P^-1 with P^-1 the restricted
    additive Schwarz preconditioner over 48-element neighbourhoods.  Its step count
    follows the oracle's GMRES on the dense A P^-1 (whose local inverses are FP64 and
    whose same-element entries are exact, where the GPU's are FP32 and from the
    compressed defect products), and its solution is the dense solve's."""
    nodes, tris = meshes.icosphere(0.01, 2)
    surf = bemgpu.mesh(nodes, tris)
    kw = dict(reltol=1e-8, restart=150, maxiter=1200)
    sol = bemgpu.bem(surf, bemgpu.Rigid(), K38, incidence_angle=0.7, incidence_azimuth=0.4,
                     ctx=ctx, discretization="nystrom",
                     compression=dict(method="hmatrix", tol=1e-10, leaf_size=32,
                                      neighbours=48),
                     gmres_kwargs=kw)
    st = sol.hmatrix_stats()
    p, q = sol.traces()
    sol.close()
    P = O.Panels(nodes, tris)
    M1, M2 = NY.assemble(P, K38, True)
    y, ny, w = NY.nodes_of(P)
    d = O.incidence_direction(0.7, 0.4)
    b = M2 @ (1j * K38 * (ny @ d) * np.exp(1j * K38 * (y @ d)))
    _, plain = O.gmres(M1, b, **kw)
    Pinv = NY.ras_matrix(M1, NY.neighbourhoods(y))
    _, info = O.gmres(M1 @ Pinv, b, **kw)
    assert st["gmres_converged"] and info["converged"]
    assert info["iterations"] < plain["iterations"] / 5
    assert abs(st["gmres_iterations"] - info["iterations"]) <= max(3, 0.15 * info["iterations"])
    rp, rq, _ = NY.solve(nodes, tris, "rigid", K38, 0.7, 0.4)
    assert np.linalg.norm(p - rp) <= 1e-6 * np.linalg.norm(rp)


def test_compressed_rigid_nystrom_at_5120_panels(ctx):
    """The reference's default configuration (Nyström nodes, compression tol 1e-5, GMRES
    reltol 1e-4, restart 150, maxiter 1200, no preconditioner) on the 5120-panel sphere
    (35 840 nodes) at k a = 1.6: converged within the 1200 steps (about 720), within
    0.05 dB of the dense Nyström solve."""
    nodes, tris = meshes.icosphere(0.01, 4)
    surf = bemgpu.mesh(nodes, tris)
    kw = dict(incidence_angle=1.0, incidence_azimuth=0.3, ctx=ctx, discretization="nystrom",
              precision="mixed")
    sol = bemgpu.bem(surf, bemgpu.Rigid(), K38, compression=dict(method="hmatrix"), **kw)
    st = sol.hmatrix_stats()
    fh = bemgpu.scattering_amplitude(sol)
    sol.close()
    dense = bemgpu.bem(surf, bemgpu.Rigid(), K38, **kw)
    fd = bemgpu.scattering_amplitude(dense)
    dense.close()
    assert st["gmres_converged"], st
    assert st["gmres_iterations"] < 1200
    assert abs(20 * math.log10(abs(fh) / abs(fd))) < 0.05


@pytest.mark.parametrize("boundary,precision", [("rigid", "double"), ("rigid", "mixed"),
                                                ("pressure_release", "double"),
                                                ("pressure_release", "mixed")])
def test_compressed_node_operators_at_the_reference_defaults(ctx, boundary, precision):
    nodes, tris = meshes.icosphere(0.01, 3)
    surf = bemgpu.mesh(nodes, tris)
    dense = bemgpu.bem(surf, _bc(boundary), K38, ctx=ctx, discretization="nystrom")
    sol = bemgpu.bem(surf, _bc(boundary), K38, ctx=ctx, discretization="nystrom",
                     precision=precision, compression=dict(method="hmatrix", tol=1e-5))
    assert sol.hmatrix_stats()["gmres_converged"]
    fd, fh = bemgpu.scattering_amplitude(dense), bemgpu.scattering_amplitude(sol)
    assert abs(20 * math.log10(abs(fh) / abs(fd))) < 0.05
    assert sol.hmatrix_stats()["compression"] < 0.5
    pts = np.array([[0.0, 0.0, 0.013], [0.02, 0.0, 0.0]])
    ph, pd = bemgpu.pressure(sol, pts), bemgpu.pressure(dense, pts)
    assert np.all(np.abs(ph - pd) < 1e-3 * np.abs(pd))
    dense.close()
    sol.close()


def test_unsupported_combinations_are_rejected(ctx):
    nodes, tris = meshes.icosphere(0.01, 1)
    surf = bemgpu.mesh(nodes, tris)
    sol = bemgpu.bem([surf], [bemgpu.FluidFilled(1.03, 1.02)], K38, ctx=ctx,
                     discretization="nystrom")
    with pytest.raises(bemgpu.ArgumentError):  # field evaluation of Nyström regions
        sol.pressure(np.array([[0.0, 0.0, 0.02]]))
    sol.close()
    with pytest.raises(bemgpu.ArgumentError):
        bemgpu.bem(surf, bemgpu.FluidFilled(1.03, 1.02), K38, ctx=ctx, discretization="nystrom",
                   compression=dict(method="hmatrix"))


def _reference_amplitudes():
    import json
    import os
    path = os.path.join(os.path.dirname(__file__), "golden", "reference_amplitudes.json")
    with open(path) as f:
        return json.load(f)


def _check_amplitudes(got, refs, db, rel):
    for f, b in zip(got, refs):
        assert abs(20 * math.log10(abs(f) / abs(b))) < db, (f, b)
        assert abs(f - b) < rel * abs(b), (f, b, abs(f - b) / abs(b))


def test_reference_rigid_spheroid_amplitudes_collocation(ctx):
    """The amplitudes the reference's tests hard-code for a rigid spheroid
    (test/extended/bem/spheroid/full3d.jl:9-24) at the reference's own tolerance, 0.1 dB
    and 1 % (full3d.jl:21-22): the collocation discretisation on 11520 panels (96 x 60;
    the oracle's error there is 0.85 %), mixed precision."""
    s = _reference_amplitudes()["rigid_spheroid"]
    nodes, tris = meshes.uv_spheroid(s["a"], s["b"], 96, 60)
    sol = bemgpu.bem(bemgpu.mesh(nodes, tris), bemgpu.Rigid(), s["k"],
                     incidence_angle=s["incidence_angle"],
                     incidence_azimuth=s["incidence_azimuth"], ctx=ctx, precision="mixed")
    got = [sol.far_field(np.array(r["direction"]))[0] for r in s["references"]]
    sol.close()
    _check_amplitudes(got, [complex(*r["amplitude"]) for r in s["references"]], 0.1, 0.01)


def test_reference_rigid_spheroid_amplitudes(ctx):
    """The same amplitudes from the Nyström discretisation (the reference's own) on 5120
    panels (64 x 40, 35840 node unknowns): within the reference's 0.1 dB.  Its amplitude
    error falls slowly with the flat-facet mesh -- 1.96 %, 1.49 % and 1.23 % at 1280, 2880
    and 5120 panels (measured on a GB300) -- so 1 % needs about 10^4 panels (a 70 000-node
    dense system); 1.3 % is the bound asserted here."""
    s = _reference_amplitudes()["rigid_spheroid"]
    nodes, tris = meshes.uv_spheroid(s["a"], s["b"], 64, 40)
    surf = bemgpu.mesh(nodes, tris)
    sol = bemgpu.bem(surf, bemgpu.Rigid(), s["k"], incidence_angle=s["incidence_angle"],
                     incidence_azimuth=s["incidence_azimuth"], ctx=ctx,
                     discretization="nystrom", precision="mixed")
    got = [sol.far_field(np.array(r["direction"]))[0] for r in s["references"]]
    sol.close()
    _check_amplitudes(got, [complex(*r["amplitude"]) for r in s["references"]], 0.1, 0.013)


@pytest.mark.parametrize("heavy", [False, True])
def test_reference_fluid_sphere_amplitudes_collocation(ctx, heavy):
    """The reference's hard-coded amplitudes of the gas-filled (g 0.0012, h 0.23) and the
    heavy (g 1000, h 2) fluid sphere at k a = 1 (sphere/full3d.jl:209-234) at the
    reference's 0.1 dB and 1 %: the collocation discretisation on 1280 panels."""
    c = [c for c in _reference_amplitudes()["fluid_sphere"]
         if c["k"] == 1.0 and (c["g"] > 1) == heavy][0]
    nodes, tris = meshes.icosphere(1.0, 3)
    sol = bemgpu.bem(bemgpu.mesh(nodes, tris), bemgpu.FluidFilled(c["g"], c["h"]), c["k"],
                     incidence_angle=0.0, ctx=ctx, precision="mixed")
    got = sol.far_field(np.array(c["directions"]))
    sol.close()
    _check_amplitudes(got, [complex(x, y) for x, y in c["amplitudes"]], 0.1, 0.01)


def test_reference_gas_sphere_amplitudes(ctx):
    """The gas-filled sphere's amplitudes (g 0.0012, h 0.23, k a = 1) from the Nyström
    discretisation: 1.07 % / 0.053 dB at 1280 panels, 0.48 % / 0.024 dB at 2880 (measured
    on a GB300; the 2880-panel solve takes four minutes in FP64, to which the condition
    guard promotes this system), so 1280 panels with 1.2 % is asserted here."""
    c = [c for c in _reference_amplitudes()["fluid_sphere"] if c["k"] == 1.0 and c["g"] < 1][0]
    nodes, tris = meshes.icosphere(1.0, 3)
    surf = bemgpu.mesh(nodes, tris)
    sol = bemgpu.bem(surf, bemgpu.FluidFilled(c["g"], c["h"]), c["k"], incidence_angle=0.0,
                     ctx=ctx, discretization="nystrom", precision="mixed")
    got = sol.far_field(np.array(c["directions"]))
    sol.close()
    _check_amplitudes(got, [complex(x, y) for x, y in c["amplitudes"]], 0.1, 0.012)
