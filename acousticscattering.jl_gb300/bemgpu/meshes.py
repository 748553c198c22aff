"""Deterministic flat-triangle surface generators for the BEM workloads.

The reference meshes through Gmsh (``geometry/canonical_mesh.jl:13-58``), which is not
part of this build.  These generators produce ``(nodes, triangles)`` pairs in the layout
of the reference's supplied-mesh entry point ``mesh(nodes::3xN, triangles::3xM)``
(``geometry/surface.jl:271-298``): ``nodes`` is a 3 x N float64 array (one column per
vertex), ``triangles`` a 3 x M int64 array of 1-based vertex indices, ordered so that
``(b - a) x (c - a)`` points out of the body.

Every coordinate is computed with correctly rounded IEEE operations only (+, -, *, /,
sqrt) and a fixed-order polynomial sine/cosine, and the jitter comes from a
counter-based SplitMix64 stream, so the same arguments give bit-identical arrays on
x86-64 and AArch64 hosts.  ``mesh_hash`` fingerprints a pair with SHA-256.
"""
from __future__ import annotations

import hashlib
import math

import numpy as np

_MASK64 = (1 << 64) - 1


def splitmix64(state: int) -> tuple[int, int]:
    """One SplitMix64 step: returns (new_state, output)."""
    state = (state + 0x9E3779B97F4A7C15) & _MASK64
    z = state
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _MASK64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _MASK64
    return state, z ^ (z >> 31)


def seed_for(master: int, index: int) -> int:
    """Per-instance seed derived from a master seed (SplitMix64 of master ^ index mix)."""
    _, out = splitmix64((master * 0x9E3779B97F4A7C15 + index) & _MASK64)
    return out


def uniform_stream(seed: int, count: int) -> np.ndarray:
    """``count`` doubles in [0, 1) from a SplitMix64 stream (53-bit mantissas)."""
    out = np.empty(count, dtype=np.float64)
    s = seed & _MASK64
    for i in range(count):
        s, z = splitmix64(s)
        out[i] = (z >> 11) * (1.0 / 9007199254740992.0)
    return out


_TWO_PI = 6.283185307179586
_HALF_PI = 1.5707963267948966


def det_sincos(theta: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """Platform-reproducible sine and cosine (abs. error ~1e-16 for |theta| < 1e3)."""
    theta = np.asarray(theta, dtype=np.float64)
    q = np.rint(theta / _HALF_PI)
    r = (theta - q * _HALF_PI) - q * 6.123233995736766e-17
    qi = q.astype(np.int64) & 3
    s = _sin_red(r)
    c = _cos_red(r)
    sin = np.where(qi == 0, s, np.where(qi == 1, c, np.where(qi == 2, -s, -c)))
    cos = np.where(qi == 0, c, np.where(qi == 1, -s, np.where(qi == 2, -c, s)))
    return sin, cos


def _sin_red(x: np.ndarray) -> np.ndarray:
    x2 = x * x
    s = np.full_like(x, -1.0 / 1307674368000.0)          # -1/15!
    for a in (1.0 / 6227020800.0, -1.0 / 39916800.0, 1.0 / 362880.0, -1.0 / 5040.0,
              1.0 / 120.0, -1.0 / 6.0):
        s = s * x2 + a
    return x + x * x2 * s


def _cos_red(x: np.ndarray) -> np.ndarray:
    x2 = x * x
    c = np.full_like(x, 1.0 / 20922789888000.0)          # 1/16!
    for a in (-1.0 / 87178291200.0, 1.0 / 479001600.0, -1.0 / 3628800.0, 1.0 / 40320.0,
              -1.0 / 720.0, 1.0 / 24.0, -0.5):
        c = c * x2 + a
    return 1.0 + x2 * c


def mesh_hash(nodes: np.ndarray, triangles: np.ndarray) -> str:
    """SHA-256 over (N, M, nodes column-major float64 LE, triangles int64 LE)."""
    nodes = np.asarray(nodes, dtype="<f8")
    tris = np.asarray(triangles, dtype="<i8")
    h = hashlib.sha256()
    h.update(np.array([nodes.shape[1], tris.shape[1]], dtype="<i8").tobytes())
    h.update(np.asfortranarray(nodes).tobytes(order="F"))
    h.update(np.asfortranarray(tris).tobytes(order="F"))
    return h.hexdigest()


def icosphere(radius: float = 1.0, subdivisions: int = 3,
              center=(0.0, 0.0, 0.0)) -> tuple[np.ndarray, np.ndarray]:
    """Icosahedron refined by ``subdivisions`` midpoint splits, projected to a sphere.

    ``subdivisions=3`` gives 1280 triangles and 642 vertices (20 * 4**3 faces,
    10 * 4**3 + 2 vertices), the sphere of the rigid 38 kHz workload.
    """
    if subdivisions < 0:
        raise ValueError("subdivisions must be nonnegative")
    t = (1.0 + math.sqrt(5.0)) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0),
         (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11),
             (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6), (7, 1, 8),
             (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9),
             (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    pts = [np.array(p, dtype=np.float64) for p in v]

    def unit(p):
        return p / math.sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2])

    pts = [unit(p) for p in pts]
    for _ in range(subdivisions):
        cache: dict[tuple[int, int], int] = {}

        def mid(a, b):
            key = (a, b) if a < b else (b, a)
            if key not in cache:
                pts.append(unit((pts[a] + pts[b]) * 0.5))
                cache[key] = len(pts) - 1
            return cache[key]

        nf = []
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    nodes = np.array(pts, dtype=np.float64).T * float(radius)
    nodes = nodes + np.asarray(center, dtype=np.float64).reshape(3, 1)
    tris = np.array(faces, dtype=np.int64).T + 1
    return np.ascontiguousarray(nodes), np.ascontiguousarray(tris)


def _revolution(profile, nlon: int, nrings: int):
    """Triangulate a surface of revolution about +x.

    ``profile(theta)`` returns (x, rho) arrays for polar angles theta in (0, pi); the
    poles sit at theta = 0 and pi.  Rings r = 1..nrings at theta = pi r / (nrings + 1),
    nlon vertices per ring.  Triangles: 2 * nlon * nrings.
    """
    if nlon < 3 or nrings < 1:
        raise ValueError("need nlon >= 3 and nrings >= 1")
    th = np.arange(1, nrings + 1, dtype=np.float64) * (math.pi / (nrings + 1))
    ph = np.arange(nlon, dtype=np.float64) * (_TWO_PI / nlon)
    sph, cph = det_sincos(ph)
    xr, rho = profile(th)
    x0, _ = profile(np.array([0.0]))
    x1, _ = profile(np.array([math.pi]))
    X = np.repeat(xr, nlon)
    Y = (rho[:, None] * cph[None, :]).reshape(-1)
    Z = (rho[:, None] * sph[None, :]).reshape(-1)
    nodes = np.empty((3, nrings * nlon + 2), dtype=np.float64)
    nodes[:, 0] = (x0[0], 0.0, 0.0)
    nodes[0, 1:-1], nodes[1, 1:-1], nodes[2, 1:-1] = X, Y, Z
    nodes[:, -1] = (x1[0], 0.0, 0.0)
    south = nodes.shape[1] - 1

    def vid(r, l):
        return 1 + r * nlon + (l % nlon)

    faces = []
    for l in range(nlon):  # cap at theta = 0 (+x pole)
        faces.append((0, vid(0, l + 1), vid(0, l)))
    for r in range(nrings - 1):
        for l in range(nlon):
            a, b = vid(r, l), vid(r, l + 1)
            c, d = vid(r + 1, l), vid(r + 1, l + 1)
            faces.append((a, b, d))
            faces.append((a, d, c))
    for l in range(nlon):  # cap at theta = pi (-x pole)
        faces.append((south, vid(nrings - 1, l), vid(nrings - 1, l + 1)))
    # the faces above wind clockwise seen from outside; swap two corners
    tris = np.array(faces, dtype=np.int64)[:, (0, 2, 1)].T + 1
    return nodes, np.ascontiguousarray(tris)


def _mean_edge(nodes: np.ndarray, tris: np.ndarray) -> float:
    t = tris - 1
    total = 0.0
    for a, b in ((0, 1), (1, 2), (2, 0)):
        d = nodes[:, t[b]] - nodes[:, t[a]]
        total += math.fsum(np.sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]).tolist())
    return total / (3 * t.shape[1])


def _jitter(nodes: np.ndarray, tris: np.ndarray, jitter: float, seed: int) -> np.ndarray:
    if jitter == 0.0:
        return nodes
    amp = jitter * _mean_edge(nodes, tris)
    u = uniform_stream(seed, nodes.size).reshape(nodes.shape[1], 3).T
    return nodes + (2.0 * u - 1.0) * amp


def uv_spheroid(a: float, b: float, nlon: int, nrings: int, jitter: float = 0.0,
                seed: int = 0) -> tuple[np.ndarray, np.ndarray]:
    """UV-mapped spheroid, semi-axis ``a`` along x (symmetry axis), ``b`` equatorial.

    Triangles: 2 * nlon * nrings (5120 for nlon=64, nrings=40; 20480 for 128 x 80).
    ``jitter`` displaces every vertex coordinate by U(-jitter, jitter) times the mean
    edge length, from the SplitMix64 stream of ``seed``.
    """
    def profile(th):
        s, c = det_sincos(th)
        return a * c, b * s

    nodes, tris = _revolution(profile, nlon, nrings)
    return np.ascontiguousarray(_jitter(nodes, tris, jitter, seed)), tris


def body_of_revolution(b: float, aspect: float, coeffs, nlon: int, nrings: int):
    """Spheroid radius profile r(theta) = b (1 + sum_m c_m cos(m theta)), stretched by
    ``aspect`` along the x (symmetry) axis: (aspect b cos t, b sin t cos p, b sin t sin p)
    scaled by the modulation factor."""
    coeffs = [float(c) for c in coeffs]

    def profile(th):
        s, c = det_sincos(th)
        mod = np.ones_like(th)
        for m, cm in enumerate(coeffs, start=1):
            _, cmth = det_sincos(m * th)
            mod = mod + cm * cmth
        return aspect * b * c * mod, b * s * mod

    return _revolution(profile, nlon, nrings)


def grid_for_panels(target: int, aspect: float) -> tuple[int, int]:
    """(nlon, nrings) with 2 * nlon * nrings close to ``target`` panels, rings denser
    along longer bodies."""
    ratio = min(max(aspect / 1.6, 0.6), 4.0)          # nrings / nlon
    nlon = max(8, int(round(math.sqrt(target / (2.0 * ratio)))))
    nrings = max(3, int(round(target / (2.0 * nlon))))
    return nlon, nrings


def random_body(master_seed: int, index: int, panel_range=(500, 12000)) -> dict:
    """One seeded instance of the uneven body-of-revolution workload.

    b ~ U(5, 20) mm, aspect ~ U(1.5, 6), c_1..c_4 ~ U(-0.05, 0.05), panel count
    log-uniform in ``panel_range``, frequency ~ U(10, 200) kHz, incidence uniform on
    the sphere, rigid or pressure release 50/50.
    """
    seed = seed_for(master_seed, index)
    u = uniform_stream(seed, 12)
    b = 0.005 + 0.015 * u[0]
    aspect = 1.5 + 4.5 * u[1]
    coeffs = [-0.05 + 0.1 * u[2 + m] for m in range(4)]
    lo, hi = panel_range
    target = int(round(math.exp(math.log(lo) + (math.log(hi) - math.log(lo)) * u[6])))
    freq = 10e3 + 190e3 * u[7]
    cos_beta = 2.0 * u[8] - 1.0
    beta = math.acos(cos_beta)
    alpha = _TWO_PI * u[9]
    boundary = "rigid" if u[10] < 0.5 else "pressure_release"
    nlon, nrings = grid_for_panels(target, aspect)
    return dict(seed=seed, b=b, aspect=aspect, coeffs=coeffs, target_panels=target,
                nlon=nlon, nrings=nrings, panels=2 * nlon * nrings, frequency=freq,
                incidence_angle=beta, incidence_azimuth=alpha, boundary=boundary)
