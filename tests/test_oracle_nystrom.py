"""The Nyström oracle pinned before it is trusted (no GPU).

Pins: the corrected discrete Green identities hold for every interpolant (the defining
property of the density-interpolation correction, solvers/bem/quadrature/fluid.jl:124-149);
the sphere's modal series (solvers/modal/sphere.jl) at the reference's 0.1 dB; error
decreasing under refinement; the fit keeps full rank over five decades of k times the
panel size (no singular value reaches the 1e-13 cutoff, so every pseudo-inverse solution
is the unique minimum-norm one); argument checks of the host interface.
"""
import math

import numpy as np
import pytest

from bemgpu import meshes
from oracle import modal
from oracle import nystrom as NY
from oracle import oracle as O

K38 = 2 * math.pi * 38e3 / 1477.4  # rigid sphere a = 1 cm at 38 kHz, c = 1477.4 m/s


def _ts_error(boundary, sub, k=K38, a=0.01):
    nodes, tris = meshes.icosphere(a, sub)
    p, q, (y, ny, w) = NY.solve(nodes, tris, boundary, k, math.pi / 2, math.pi / 2)
    d = O.incidence_direction(math.pi / 2, math.pi / 2)
    f = NY.far_field(y, ny, w, k, -d, p, q)
    fm = modal.form_function(boundary, k, a)
    return 20 * math.log10(abs(f) / abs(fm)), abs(f - fm) / abs(fm)


def test_corrected_identities_hold_for_every_interpolant():
    nodes, tris = meshes.icosphere(0.01, 1)
    P = O.Panels(nodes, tris)
    (S, D, K, H), (y, ny, w) = NY.corrected_operators(P, K38)
    u, f = NY.traces(y, ny, K38)
    r1 = -0.5 * u + S @ f - D @ u
    r2 = -0.5 * f + K @ f - H @ u
    assert np.abs(r1).max() < 1e-11 * np.abs(u).max()
    assert np.abs(r2).max() < 1e-11 * np.abs(f).max()
    # and not before the correction
    S0, D0, K0, H0 = NY.operators(y, ny, w, K38)
    assert np.abs(-0.5 * u + S0 @ f - D0 @ u).max() > 1e-3 * np.abs(u).max()


@pytest.mark.parametrize("boundary", ["rigid", "pressure_release"])
def test_sphere_against_modal(boundary):
    db, rel = _ts_error(boundary, 2)
    assert abs(db) < 0.1, db
    assert rel < 0.06, rel


@pytest.mark.parametrize("boundary", ["rigid", "pressure_release"])
def test_point_field_against_modal_near_field(boundary):
    """Nearest-element exclusion + fit at points from 0.5 % to 200 % of the radius off the
    sphere: the modal scattered field within 5 % at 320 panels."""
    a = 0.01
    nodes, tris = meshes.icosphere(a, 2)
    P = O.Panels(nodes, tris)
    p, q, _ = NY.solve(nodes, tris, boundary, K38, math.pi / 2, math.pi / 2)
    d = O.incidence_direction(math.pi / 2, math.pi / 2)
    dirs = np.array([[1.0, 0, 0], [0.0, 0.6, 0.8], [-0.6, 0.0, 0.8], [0.0, 0.0, -1.0]])
    pts = np.concatenate([rf * a * dirs for rf in (1.005, 1.05, 1.3, 3.0)])
    got = NY.pressure(P, K38, pts, p, q, d, "scattered")
    want = np.array([modal.scattered_field(boundary, K38, a, np.linalg.norm(x),
                                           (x @ d) / np.linalg.norm(x)) for x in pts])
    assert np.max(np.abs(got - want)) < 0.05 * np.max(np.abs(want))
    with pytest.raises(ValueError):
        NY.pressure(P, K38, np.zeros((1, 3)), p, q, d, "total")


def test_modal_near_field_tends_to_the_form_function():
    a, r = 0.01, 1e5
    for b in ("rigid", "pressure_release"):
        near = modal.scattered_field(b, K38, a, r, -1.0) * r * np.exp(-1j * K38 * r)
        far = modal.form_function(b, K38, a)
        assert abs(near - far) < 1e-4 * abs(far)


G_FL, H_FL = 1.0357, 1.0279  # the fluid spheroid workload's contrasts


@pytest.mark.parametrize("formulation", ["muller", "cbie"])
def test_fluid_sphere_against_modal(formulation):
    a = 0.01
    nodes, tris = meshes.icosphere(a, 2)
    p, q, (y, ny, w) = NY.solve(nodes, tris, "fluid", K38, math.pi / 2, math.pi / 2,
                                formulation, G_FL, H_FL)
    d = O.incidence_direction(math.pi / 2, math.pi / 2)
    f = NY.far_field(y, ny, w, K38, -d, p, q)
    fm = modal.form_function("fluid", K38, a, g=G_FL, h=H_FL)
    assert abs(20 * math.log10(abs(f) / abs(fm))) < 0.1
    assert abs(f - fm) < 0.015 * abs(fm)


def test_fluid_pressure_is_continuous_across_the_surface():
    a = 0.01
    nodes, tris = meshes.icosphere(a, 2)
    P = O.Panels(nodes, tris)
    p, q, _ = NY.solve(nodes, tris, "fluid", K38, math.pi / 2, math.pi / 2, "muller",
                       G_FL, H_FL)
    d = O.incidence_direction(math.pi / 2, math.pi / 2)
    cen = P.centroids[[3, 101, 250]]  # facet centres: 0.3 % off the facet on either side
    assert not any(NY._inside(P, x) for x in 1.003 * cen)
    assert all(NY._inside(P, x) for x in 0.997 * cen)
    po = NY.pressure(P, K38, 1.003 * cen, p, q, d, "total", g=G_FL, h=H_FL)
    pi = NY.pressure(P, K38, 0.997 * cen, p, q, d, "total", g=G_FL, h=H_FL)
    assert np.all(np.abs(po - pi) < 0.03 * np.abs(po))


def test_refinement_reduces_error():
    e1 = _ts_error("rigid", 1)[1]
    e2 = _ts_error("rigid", 2)[1]
    assert e2 < 0.5 * e1, (e1, e2)


def test_fit_keeps_full_rank():
    nodes, tris = meshes.icosphere(0.01, 2)
    P = O.Panels(nodes, tris)
    y, ny, w = NY.nodes_of(P)
    h = math.sqrt(P.areas.mean())
    for kh in (0.005, 0.05, 0.5, 2.0, 10.0):
        u, f = NY.traces(y, ny, kh / h)
        _, dropped = NY.fit_weights(u, f, np.zeros_like(u))
        assert dropped == 0, kh


def test_directions_are_unit_and_distinct():
    d = NY.directions()
    assert d.shape == (9, 3)
    assert np.allclose((d * d).sum(1), 1.0, atol=1e-15)
    g = d @ d.T
    assert np.all(np.abs(g - np.eye(9)) < 0.97)  # no repeated or antipodal pair


def test_host_rejects_unsupported_nystrom_options():
    import bemgpu
    from bemgpu.api import _problem
    with pytest.raises(bemgpu.ArgumentError):
        _problem(bemgpu.Rigid(), 1.0, discretization="galerkin")
    p = _problem(bemgpu.PressureRelease(), 2.0, discretization="nystrom")
    assert p.discretization == 1


def test_oracle_schwarz_neighbourhoods_and_gmres():
    """The restricted additive Schwarz restatement: every neighbourhood starts with its own
    element and holds the 48 nearest elements (by centroid node); GMRES on A P^-1 of the
    320-panel rigid sphere needs a fraction of the plain steps and reaches the same
    solution."""
    import math
    nodes, tris = meshes.icosphere(0.01, 2)
    P = O.Panels(nodes, tris)
    k = 2 * math.pi * 38e3 / 1477.4
    M1, M2 = NY.assemble(P, k, True)
    y, ny, w = NY.nodes_of(P)
    nb = NY.neighbourhoods(y)
    cent = y[::7]
    for e in (0, 17, 319):
        assert nb[e][0] == e and len(nb[e]) == 48
        d = np.sqrt(((cent - cent[e]) ** 2).sum(1))
        assert d[nb[e]].max() <= np.sort(d)[47] + 1e-15
    d = O.incidence_direction(0.7, 0.4)
    b = M2 @ (1j * k * (ny @ d) * np.exp(1j * k * (y @ d)))
    kw = dict(reltol=1e-8, restart=150, maxiter=1200)
    x0, plain = O.gmres(M1, b, **kw)
    Pinv = NY.ras_matrix(M1, nb)
    yv, info = O.gmres(M1 @ Pinv, b, **kw)
    assert info["converged"] and info["iterations"] * 5 < plain["iterations"]
    assert np.linalg.norm(Pinv @ yv - x0) <= 1e-6 * np.linalg.norm(x0)


@pytest.mark.parametrize("sub,count", [(2, 48), (3, 48), (1, 100)])
def test_library_schwarz_neighbourhoods_match_oracle(sub, count):
    """The library's neighbourhood search (host, grid-accelerated) returns the oracle's
    neighbourhoods exactly, including a count above the number of elements."""
    import ctypes
    from bemgpu import _lib as C
    nodes, tris = meshes.icosphere(0.01, sub)
    m = tris.shape[1]
    cnt = min(count, m)
    out = np.zeros(m * cnt, dtype=np.int32)
    fn, ft = np.asfortranarray(nodes), np.asfortranarray(tris.astype(np.int64))
    st = C.lib().bemgpu_schwarz_neighbourhoods(
        C.dptr(fn), fn.shape[1], C.i64ptr(ft), m, count,
        out.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)))
    assert st == C.OK
    P = O.Panels(nodes, tris)
    y, _, _ = NY.nodes_of(P)
    ref = NY.neighbourhoods(y, count)
    assert np.array_equal(out.reshape(m, cnt), np.array(ref))
