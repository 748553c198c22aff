"""Compressed operators + GMRES on the GPU (the reference's rigid/soft default
solve_full_bem(...; compression=(method=:hmatrix, tol), gmres_kwargs), full.jl:52-184)
against the oracle: products against the oracle's dense operators, solutions against the
oracle's direct solve, iteration counts and residual histories against the oracle's GMRES
restatement on the dense operators."""
import math

import numpy as np
import pytest

import bemgpu
from bemgpu import meshes
from oracle import oracle as O

pytestmark = pytest.mark.gpu

K0 = 2 * math.pi * 38e3 / 1477.4  # rigid sphere a = 1 cm at 38 kHz, ka = 1.6
HM = dict(method="hmatrix")


@pytest.fixture(scope="module")
def sphere():
    nodes, tris = meshes.icosphere(0.01, 3)
    return nodes, tris, bemgpu.mesh(nodes, tris), O.Panels(nodes, tris)


@pytest.fixture(scope="module")
def spheroid():
    nodes, tris = meshes.uv_spheroid(0.02, 0.01, 48, 30, jitter=0.02, seed=11)
    return nodes, tris, bemgpu.mesh(nodes, tris), O.Panels(nodes, tris)


@pytest.mark.parametrize("formulation", ["burton_miller", "cbie"])
@pytest.mark.parametrize("tol", [1e-5, 1e-9])
def test_compressed_products_match_oracle_operators(ctx, sphere, formulation, tol):
    nodes, tris, surf, P = sphere
    M1, M2 = O.assemble_bm(P, K0, formulation == "burton_miller")
    rng = np.random.default_rng(1)
    X = rng.standard_normal((P.n, 3)) + 1j * rng.standard_normal((P.n, 3))
    for op, M in ((0, M1), (1, M2)):
        Y, st = bemgpu.hmatrix_apply(surf, bemgpu.Rigid(), K0, X, op=op, formulation=formulation,
                                     tol=tol, ctx=ctx)
        ref = M @ X
        err = np.linalg.norm(Y - ref) / np.linalg.norm(ref)
        assert err <= 10 * tol, (op, err, st)
        assert st["lowrank_blocks"] + st["densified_blocks"] > 0
        if tol >= 1e-6:  # tighter: small blocks may need more rank than a full block holds
            assert st["lowrank_blocks"] > 0 and st["compression"] < 1.0


def test_full_blocks_reproduce_oracle_entries(ctx, spheroid):
    """With a tolerance at rounding level the compressed product is the dense product: the
    full blocks (regular + near rules into block storage) carry the oracle's entries."""
    nodes, tris, surf, P = spheroid
    k = 2 * math.pi * 60e3 / 1500.0
    M1, M2 = O.assemble_bm(P, k, True)
    rng = np.random.default_rng(2)
    X = rng.standard_normal(P.n) + 1j * rng.standard_normal(P.n)
    for op, M in ((0, M1), (1, M2)):
        Y, st = bemgpu.hmatrix_apply(surf, bemgpu.Rigid(), k, X, op=op, tol=1e-13, ctx=ctx)
        ref = M @ X
        assert np.linalg.norm(Y[:, 0] - ref) <= 1e-10 * np.linalg.norm(ref), st


@pytest.mark.parametrize("boundary", ["rigid", "pressure_release"])
def test_compressed_solve_matches_direct_oracle(ctx, sphere, boundary):
    nodes, tris, surf, P = sphere
    bc = bemgpu.Rigid() if boundary == "rigid" else bemgpu.PressureRelease()
    ref = O.solve(nodes, tris, boundary, K0, incidence_angle=math.pi / 2,
                  incidence_azimuth=math.pi / 2, panels=P)
    f0 = ref["amplitudes"][0]
    # tight: the compressed GMRES solve is the dense solution
    sol = bemgpu.bem(surf, bc, K0, incidence_angle=math.pi / 2, incidence_azimuth=math.pi / 2,
                     compression=dict(HM, tol=1e-11), gmres_kwargs=dict(reltol=1e-11), ctx=ctx)
    f = bemgpu.scattering_amplitude(sol)
    assert abs(f - f0) <= 1e-8 * abs(f0)
    p, q = sol.traces()
    assert np.linalg.norm(p - ref["p_scat"]) <= 1e-8 * np.linalg.norm(ref["p_scat"])
    assert np.linalg.norm(q - ref["dpdn_scat"]) <= 1e-8 * np.linalg.norm(ref["dpdn_scat"])
    d = sol.diagnostics()
    assert d["method"] == "gmres" and d["converged"] and d["relative_residual"] <= 1e-10
    sol.close()
    # the reference's defaults (tol 1e-5, reltol 1e-4): within 0.01 dB of the dense solve
    sol = bemgpu.bem(surf, bc, K0, incidence_angle=math.pi / 2, incidence_azimuth=math.pi / 2,
                     compression=HM, ctx=ctx)
    assert abs(bemgpu.target_strength(sol) - O.target_strength(f0)) <= 0.01
    sol.close()


def test_gmres_follows_the_oracle_restatement(ctx, sphere):
    """Restarted GMRES on the compressed operator (tol at rounding level) takes the oracle
    GMRES's steps on the dense operator: same count (+-1) and residual estimates."""
    nodes, tris, surf, P = sphere
    kw = dict(reltol=1e-9, restart=6, maxiter=1200)
    rep = O.solve_gmres(nodes, tris, "rigid", K0, incidence_angle=0.4, incidence_azimuth=1.1,
                        panels=P, **kw)
    sol = bemgpu.bem(surf, bemgpu.Rigid(), K0, incidence_angle=0.4, incidence_azimuth=1.1,
                     compression=dict(HM, tol=1e-13), gmres_kwargs=kw, ctx=ctx)
    d = sol.diagnostics()
    h = sol.residual_history(0)
    assert rep["converged"] and d["converged"]
    assert abs(d["iterations"] - rep["iterations"]) <= 1
    assert len(h) == d["iterations"]
    m = min(len(h), len(rep["history"]))
    bn = np.linalg.norm(rep["b"])
    assert np.all(np.abs(h[:m] - rep["history"][:m]) <= 1e-6 * rep["history"][:m] + 1e-11 * bn)
    f = bemgpu.scattering_amplitude(sol)
    assert abs(f - rep["amplitude"]) <= 1e-7 * abs(rep["amplitude"])
    sol.close()


def test_gmres_stops_at_maxiter_and_warns(ctx, sphere):
    nodes, tris, surf, P = sphere
    with pytest.warns(RuntimeWarning, match="GMRES did not converge"):
        sol = bemgpu.bem(surf, bemgpu.Rigid(), K0, compression=HM,
                         gmres_kwargs=dict(reltol=1e-14, maxiter=5), ctx=ctx)
    d = sol.diagnostics()
    assert not d["converged"] and d["iterations"] == 5
    assert len(sol.residual_history()) == 5
    sol.close()


@pytest.mark.parametrize("precision", ["double", "mixed"])
def test_batched_right_hand_sides_equal_single_solves(ctx, sphere, precision):
    """Right-hand sides iterate in lock step but independently, and the block products
    keep each one's summation order: a sweep returns exactly the amplitudes of separate
    solves."""
    nodes, tris, surf, P = sphere
    angles = [0.3, 1.2, 2.5, 0.7, 1.9]  # a group of 4 products per CTA plus a tail
    sw = bemgpu.incidence_angle_sweep(surf, bemgpu.Rigid(), K0, angles, compression=HM,
                                      precision=precision, ctx=ctx)
    single = []
    for a in angles:
        sol = bemgpu.bem(surf, bemgpu.Rigid(), K0, incidence_angle=a, incidence_azimuth=0.0,
                         compression=HM, precision=precision, ctx=ctx)
        single.append(bemgpu.scattering_amplitude(sol))
        sol.close()
    assert np.array_equal(sw.amplitudes, np.array(single))


def test_compressed_larger_body_within_reference_tolerance(ctx, spheroid):
    nodes, tris, surf, P = spheroid
    k = 2 * math.pi * 60e3 / 1500.0
    ref = O.solve(nodes, tris, "rigid", k, incidence_angle=1.0, incidence_azimuth=0.3, panels=P)
    sol = bemgpu.bem(surf, bemgpu.Rigid(), k, incidence_angle=1.0, incidence_azimuth=0.3,
                     compression=HM, ctx=ctx)
    st = sol.hmatrix_stats()
    assert st["compression"] < 0.6 and st["gmres_converged"]
    assert abs(bemgpu.target_strength(sol) - O.target_strength(ref["amplitudes"][0])) <= 0.01
    sol.close()


def test_compression_option_errors(ctx, sphere):
    nodes, tris, surf, P = sphere
    with pytest.raises(bemgpu.ArgumentError):
        bemgpu.bem(surf, bemgpu.Rigid(), K0, compression=dict(method="fmm"), ctx=ctx)
    with pytest.raises(bemgpu.ArgumentError):
        bemgpu.bem(surf, bemgpu.Rigid(), K0, compression=dict(HM, tol=2.0), ctx=ctx)
    with pytest.raises(bemgpu.ArgumentError):
        bemgpu.bem(surf, bemgpu.FluidFilled(1.03, 1.02), K0, compression=HM, ctx=ctx)
    with pytest.raises(bemgpu.ArgumentError):
        bemgpu.bem(surf, bemgpu.Rigid(), K0, compression=HM, gmres_kwargs=dict(restrt=3),
                   ctx=ctx)


@pytest.mark.parametrize("boundary", ["rigid", "pressure_release"])
def test_mixed_precision_operators(ctx, spheroid, boundary):
    """precision=mixed: complex64 operators with FP32 entries and products; products within
    FP32 + compression error of the oracle's, solutions within 0.01 dB of the direct solve."""
    nodes, tris, surf, P = spheroid
    k = 2 * math.pi * 60e3 / 1500.0
    M1, M2 = O.assemble_bm(P, k, True)
    rng = np.random.default_rng(4)
    X = rng.standard_normal(P.n) + 1j * rng.standard_normal(P.n)
    for op, M in ((0, M1), (1, M2)):
        Y, st = bemgpu.hmatrix_apply(surf, bemgpu.Rigid(), k, X, op=op, tol=1e-5,
                                     precision="mixed", ctx=ctx)
        ref = M @ X
        assert np.linalg.norm(Y[:, 0] - ref) <= 1e-4 * np.linalg.norm(ref), st
    bc = bemgpu.Rigid() if boundary == "rigid" else bemgpu.PressureRelease()
    ref = O.solve(nodes, tris, boundary, k, incidence_angle=0.7, incidence_azimuth=0.2, panels=P)
    sol = bemgpu.bem(surf, bc, k, incidence_angle=0.7, incidence_azimuth=0.2, compression=HM,
                     precision="mixed", ctx=ctx)
    d = sol.diagnostics()
    assert d["converged"] and d["factor_precision"] == "single"
    assert abs(bemgpu.target_strength(sol) - O.target_strength(ref["amplitudes"][0])) <= 0.01
    sol.close()


def test_queries_of_a_compressed_solution(ctx, sphere):
    """pressure() and far fields at many directions of a compressed-operator solution
    equal the dense solution's (tight tolerances)."""
    nodes, tris, surf, P = sphere
    kw = dict(incidence_angle=0.8, incidence_azimuth=0.4)
    dense = bemgpu.bem(surf, bemgpu.Rigid(), K0, ctx=ctx, **kw)
    comp = bemgpu.bem(surf, bemgpu.Rigid(), K0, compression=dict(HM, tol=1e-11),
                      gmres_kwargs=dict(reltol=1e-11), ctx=ctx, **kw)
    rng = np.random.default_rng(9)
    pts = rng.standard_normal((20, 3))
    pts *= (0.015 + 0.02 * rng.random(20))[:, None] / np.linalg.norm(pts, axis=1)[:, None]
    for field in ("total", "scattered"):
        a = dense.pressure(pts, field=field)
        b = comp.pressure(pts, field=field)
        assert np.linalg.norm(a - b) <= 1e-8 * np.linalg.norm(a)
    dirs = rng.standard_normal((7, 3))
    dirs /= np.linalg.norm(dirs, axis=1)[:, None]
    fa, fb = dense.far_field(dirs), comp.far_field(dirs)
    assert np.linalg.norm(fa - fb) <= 1e-8 * np.linalg.norm(fa)
    dense.close()
    comp.close()


def test_tiny_mesh_without_admissible_blocks(ctx):
    """A surface of one leaf: no compressed block, the full block and GMRES alone."""
    nodes, tris = meshes.icosphere(0.01, 0)
    surf = bemgpu.mesh(nodes, tris)
    ref = O.solve(nodes, tris, "rigid", K0, incidence_angle=0.9, incidence_azimuth=0.1)
    sol = bemgpu.bem(surf, bemgpu.Rigid(), K0, incidence_angle=0.9, incidence_azimuth=0.1,
                     compression=dict(HM, tol=1e-10), gmres_kwargs=dict(reltol=1e-12), ctx=ctx)
    st = sol.hmatrix_stats()
    assert st["lowrank_blocks"] == 0 and st["dense_blocks"] == 1
    f0 = ref["amplitudes"][0]
    assert abs(bemgpu.scattering_amplitude(sol) - f0) <= 1e-9 * abs(f0)
    sol.close()


def test_gmres_groups_under_a_small_budget(sphere):
    """With an HBM budget that holds the Krylov bases of only a few right-hand sides, GMRES
    runs them in groups; the results are those of one group."""
    nodes, tris, surf, P = sphere
    angles = np.linspace(0.1, 3.0, 12)
    kw = dict(compression=HM, gmres_kwargs=dict(restart=500, reltol=1e-8))
    big = bemgpu.Context(0)
    small = bemgpu.Context(0, 200 << 20)
    a = bemgpu.incidence_angle_sweep(bemgpu.mesh(nodes, tris), bemgpu.Rigid(), K0, angles,
                                     ctx=big, **kw)
    b = bemgpu.incidence_angle_sweep(bemgpu.mesh(nodes, tris), bemgpu.Rigid(), K0, angles,
                                     ctx=small, **kw)
    assert np.array_equal(a.amplitudes, b.amplitudes)
