"""CPU FP64 oracle for the full-3D collocation BEM (test infrastructure only).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import this
module, always as the checker of the CUDA library, never as a product path.

Layers:
  * ``Panels``          -- ctypes view of the C restatement in ``bem_oracle.c``;
  * ``assemble_*``      -- dense system operators (reference block algebra,
                           solvers/bem/full.jl:68-128 and :289-346);
  * ``factor_fluid`` / ``solve_fluid`` -- equilibration + LAPACK LU
                           (full.jl:364-409, :422-440);
  * ``MixedRefinement`` -- complex64 LU with complex128 residual refinement and the
                           promotion state machine (solvers/bem/fluid_system.jl:172-309);
  * ``solve``           -- the ``bem`` call chain for one mesh, boundary and k
                           (full.jl:52-184, :273-495), returning scattered traces;
  * ``far_field``       -- full.jl:509-519;  ``target_strength`` -- target_strength.jl:8;
  * ``gmres`` / ``solve_gmres`` -- the reference's GMRES path for rigid/soft bodies
                           (full.jl:130-184) on dense operators: the checker of the
                           compressed-operator GPU path.
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess

import numpy as np
import scipy.linalg as sla

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

NEAR_ETA = 2.0


def build() -> str:
    """Compile liboracle.so in place (make); returns its path."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return os.path.join(_HERE, "liboracle.so")


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        dp, i64, vp = ctypes.POINTER(ctypes.c_double), ctypes.c_int64, ctypes.c_void_p
        L.oracle_panel_size.restype = ctypes.c_int
        L.oracle_panels.argtypes = [dp, i64, ctypes.POINTER(ctypes.c_int64), i64, vp]
        L.oracle_panels.restype = ctypes.c_int
        L.oracle_near_pairs.argtypes = [vp, i64, ctypes.c_double,
                                        ctypes.POINTER(ctypes.c_int64),
                                        ctypes.POINTER(ctypes.c_int64), i64]
        L.oracle_near_pairs.restype = ctypes.c_int64
        L.oracle_assemble_bm.argtypes = [vp, i64, ctypes.c_double, ctypes.c_double,
                                         ctypes.c_int, dp, dp]
        L.oracle_assemble_fluid.argtypes = [vp, i64, ctypes.c_double, ctypes.c_double,
                                            ctypes.c_double, ctypes.c_double,
                                            ctypes.c_int, dp]
        L.oracle_assemble_ops.argtypes = [vp, i64, ctypes.c_double, ctypes.c_double,
                                          dp, dp, dp, dp]
        L.oracle_incident.argtypes = [vp, i64, ctypes.c_double, dp, dp, dp]
        L.oracle_far_field.argtypes = [vp, i64, ctypes.c_double, dp, dp, dp, dp]
        L.oracle_pair_ops.argtypes = [vp, i64, i64, ctypes.c_int, ctypes.c_double, dp]
        L.oracle_laplace_parts.argtypes = [vp, dp, dp, ctypes.c_int, dp]
        L.oracle_layer_potentials.argtypes = [vp, i64, ctypes.c_double, dp, ctypes.c_double,
                                              dp, dp, ctypes.c_int, dp]
        L.oracle_solid_angle.argtypes = [vp, i64, dp]
        L.oracle_solid_angle.restype = ctypes.c_double
        _LIB = L
    return _LIB


def _dp(a):
    """Raw double* of a contiguous (C or Fortran order) float64 or complex128 array."""
    assert a.flags.c_contiguous or a.flags.f_contiguous
    return ctypes.cast(a.ctypes.data, ctypes.POINTER(ctypes.c_double))


class Panels:
    """Panel geometry of a validated (nodes 3xN, triangles 3xM 1-based) surface."""

    def __init__(self, nodes, triangles):
        L = lib()
        self.nodes = np.asfortranarray(nodes, dtype=np.float64)
        self.tris = np.asfortranarray(triangles, dtype=np.int64)
        self.n = self.tris.shape[1]
        self._buf = ctypes.create_string_buffer(L.oracle_panel_size() * self.n)
        rc = L.oracle_panels(_dp(self.nodes), self.nodes.shape[1],
                             self.tris.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                             self.n, self._buf)
        if rc != 0:
            raise ValueError(f"invalid surface (code {rc})")
        raw = np.frombuffer(self._buf, dtype=np.float64).reshape(self.n, -1)
        # record layout: v[3][3], c[3], n[3], area, diam, g[7][3]
        self.vertices = raw[:, 0:9].reshape(self.n, 3, 3)
        self.centroids = raw[:, 9:12]
        self.normals = raw[:, 12:15]
        self.areas = raw[:, 15]
        self.diams = raw[:, 16]
        self.gauss = raw[:, 17:38].reshape(self.n, 7, 3)

    @property
    def ptr(self):
        return self._buf

    def near_pairs(self, eta=NEAR_ETA):
        rowptr = np.zeros(self.n + 1, dtype=np.int64)
        cap = 64 * self.n
        while True:
            cols = np.zeros(cap, dtype=np.int64)
            cnt = lib().oracle_near_pairs(
                self._buf, self.n, eta,
                rowptr.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                cols.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), cap)
            if cnt >= 0:
                return rowptr, cols[:cnt].copy()
            cap *= 4

    def pair_ops(self, i, j, near, k):
        out = np.zeros(8)
        lib().oracle_pair_ops(self._buf, i, j, int(near), k, _dp(out))
        return out[0::2] + 1j * out[1::2]

    def laplace_parts(self, j, x, nx, self_panel=False):
        out = np.zeros(4)
        x = np.ascontiguousarray(x, dtype=np.float64)
        nx = np.ascontiguousarray(nx, dtype=np.float64)
        rec = ctypes.byref(self._buf, j * lib().oracle_panel_size())
        lib().oracle_laplace_parts(rec, _dp(x), _dp(nx), int(self_panel), _dp(out))
        return out


def incidence_direction(beta, alpha):
    """Polar angle from +x, azimuth from +y toward +z (solvers/bem/full.jl:14-18)."""
    return np.array([math.cos(beta), math.sin(beta) * math.cos(alpha),
                     math.sin(beta) * math.sin(alpha)])


def assemble_bm(P: Panels, k, burton_miller=True, eta=NEAR_ETA):
    n = P.n
    M1 = np.zeros((n, n), dtype=np.complex128, order="F")
    M2 = np.zeros((n, n), dtype=np.complex128, order="F")
    lib().oracle_assemble_bm(P.ptr, n, eta, float(k), int(burton_miller),
                             _dp(M1), _dp(M2))
    return M1, M2


def assemble_fluid(P: Panels, k, g, h, formulation="muller", eta=NEAR_ETA):
    n = P.n
    A = np.zeros((2 * n, 2 * n), dtype=np.complex128, order="F")
    lib().oracle_assemble_fluid(P.ptr, n, eta, float(k), float(g), float(h),
                                0 if formulation == "muller" else 1,
                                _dp(A))
    return A


def assemble_ops(P: Panels, k, eta=NEAR_ETA):
    """Raw S, D, K', H (n x n each) of all panel pairs at wavenumber k."""
    n = P.n
    out = [np.zeros((n, n), dtype=np.complex128, order="F") for _ in range(4)]
    lib().oracle_assemble_ops(P.ptr, n, eta, float(k), *[_dp(m) for m in out])
    return out


def combined_panels(surfaces):
    """One panel set over several closed surfaces (each (nodes, triangles), 1-based),
    panels in surface order; returns (Panels, panel offsets)."""
    nodes, tris, offs, base = [], [], [0], 0
    for nd, tr in surfaces:
        nodes.append(np.asarray(nd, dtype=np.float64))
        tris.append(np.asarray(tr, dtype=np.int64) + base)
        base += nd.shape[1]
        offs.append(offs[-1] + tr.shape[1])
    return Panels(np.concatenate(nodes, axis=1), np.concatenate(tris, axis=1)), offs


def assemble_regions(surfaces, materials, parents, k, formulation="muller", eta=NEAR_ETA):
    """Coupled fluid regions (solvers/bem/regions.jl:189-236): surface i (1-based) encloses
    region i, parents[i-1] is the region outside it (0 = exterior); materials[i-1] =
    (density, sound speed) contrasts of region i relative to the exterior.  Returns the
    2n x 2n system, the combined panels and the panel offsets."""
    P, offs = combined_panels(surfaces)
    n = P.n
    count = len(surfaces)
    dens = [1.0] + [float(m[0]) for m in materials]
    speeds = [1.0] + [float(m[1]) for m in materials]
    ops = {}

    def region_ops(r):
        if r not in ops:
            ops[r] = assemble_ops(P, k / speeds[r], eta)
        return ops[r]

    A = np.eye(2 * n, dtype=np.complex128) if formulation == "muller" else \
        np.zeros((2 * n, 2 * n), dtype=np.complex128)
    for i in range(1, count + 1):
        rows = np.arange(offs[i - 1], offs[i])
        for region in (i, parents[i - 1]):
            rho = dens[region]
            S, D, K, H = region_ops(region)
            eqs = rows + n if region == i else rows
            if formulation == "cbie":
                A[np.ix_(eqs, rows)] += 0.5 * np.eye(len(rows))
            for j in range(1, count + 1):
                if not (j == region or parents[j - 1] == region):
                    continue
                sign = 1.0 if j == region else -1.0
                cols = np.arange(offs[j - 1], offs[j])
                blk = np.ix_(rows, cols)
                if formulation == "cbie":
                    A[np.ix_(eqs, cols)] += sign * D[blk]
                    A[np.ix_(eqs, cols + n)] -= sign * rho * S[blk]
                    continue
                A[np.ix_(rows, cols)] += sign * D[blk]
                A[np.ix_(rows, cols + n)] -= sign * rho * S[blk]
                A[np.ix_(rows + n, cols)] += (sign / rho) * H[blk]
                A[np.ix_(rows + n, cols + n)] -= sign * K[blk]
    return A, P, offs


def solve_regions(surfaces, materials, parents, k, incidence_angle=math.pi / 2,
                  incidence_azimuth=0.0, formulation="muller", eta=NEAR_ETA):
    """FP64 dense solve of the coupled-region system with the exterior plane wave on the
    surfaces that border the exterior (regions.jl:240-253), and the backscatter amplitude
    summed over those surfaces (solvers/bem/postprocessing.jl:15-31)."""
    A, P, offs = assemble_regions(surfaces, materials, parents, k, formulation, eta)
    n = P.n
    d = incidence_direction(incidence_angle, incidence_azimuth)
    pinc, qinc = incident(P, k, d)
    b = np.zeros(2 * n, dtype=np.complex128)
    outer = np.zeros(n, dtype=bool)
    for i in range(1, len(surfaces) + 1):
        if parents[i - 1] == 0:
            sl = slice(offs[i - 1], offs[i])
            outer[sl] = True
            b[sl] = pinc[sl]
            if formulation == "muller":
                b[n + offs[i - 1]:n + offs[i]] = qinc[sl]
    x = np.linalg.solve(A, b)
    p_tot, v = x[:n], x[n:]
    ps = np.where(outer, p_tot - pinc, 0.0)
    qs = np.where(outer, v - qinc, 0.0)  # exterior density is 1
    amp = far_field(P, k, -d, ps, qs)
    return dict(A=A, b=b, x=x, amplitude=amp, p_scat=ps, dpdn_scat=qs, panels=P, offsets=offs)


def pressure_regions(surfaces, materials, parents, k, points, x, direction, field="total",
                     region=None, eta=NEAR_ETA):
    """Pressure of a coupled-region solution (fields/regions.jl:1-65): each point's region by
    the walk over the interfaces (an interface is tested when its parent is the region
    found so far: inside, on, or outside by its solid angle), then the interfaces bordering
    that region contribute S dp - D p (region inside them) or D p - S dp (outside), with the
    region's wavenumber, p the solved pressure and dp = density * v of the region's side;
    in the unbounded region the traces are the scattered ones and the total field adds
    the incident wave.  x = the solved [p; v] over the surfaces in order."""
    L = lib()
    count = len(surfaces)
    dens = [1.0] + [float(m[0]) for m in materials]
    speeds = [1.0] + [float(m[1]) for m in materials]
    Ps = [Panels(nd, tr) for nd, tr in surfaces]
    offs = np.cumsum([0] + [P_.n for P_ in Ps])
    n = int(offs[-1])
    d = np.asarray(direction, dtype=np.float64)
    out = []
    for xp in np.atleast_2d(np.asarray(points, dtype=np.float64)):
        xp = np.ascontiguousarray(xp)
        containing, adjacent = 0, None
        for i in range(1, count + 1):
            if parents[i - 1] != containing:
                continue
            om = L.oracle_solid_angle(Ps[i - 1].ptr, Ps[i - 1].n, _dp(xp))
            if abs(om - 2 * math.pi) < 1e-6 * 4 * math.pi:
                adjacent = (parents[i - 1], i)
                break
            if om > 2 * math.pi:
                containing = i
        if region is not None:
            ok = region == containing if adjacent is None else region in adjacent
            if not ok:
                raise ValueError("the point does not belong to the selected region")
            reg = region
        elif adjacent is not None:
            reg = adjacent[1] if field == "interior" else adjacent[0]
        else:
            reg = containing
        if field == "scattered" and reg != 0:
            raise ValueError("field=:scattered requires the unbounded exterior region")
        if field == "interior" and reg == 0:
            raise ValueError("field=:interior requires a bounded fluid region")
        inc = np.exp(1j * k * d @ xp)
        if field == "incident":
            out.append(inc)
            continue
        kr = k / speeds[reg]
        val = 0.0 + 0.0j
        for i in range(1, count + 1):
            inside = i == reg
            if not (inside or parents[i - 1] == reg):
                continue
            sl = slice(offs[i - 1], offs[i])
            p = np.array(x[sl], dtype=np.complex128)
            dp = (dens[i] if inside else dens[parents[i - 1]]) * np.array(x[n + offs[i - 1]:n + offs[i]])
            if reg == 0:
                pinc, qinc = incident(Ps[i - 1], k, d)
                p, dp = p - pinc, dp - qinc
            p, dp = np.ascontiguousarray(p), np.ascontiguousarray(dp)
            r = np.zeros(2)
            # oracle_layer_potentials: interior flag 1 -> S dp - D p, 0 -> D p - S dp
            L.oracle_layer_potentials(Ps[i - 1].ptr, Ps[i - 1].n, kr, _dp(xp), eta, _dp(p),
                                      _dp(dp), 1 if inside else 0, _dp(r))
            val += complex(r[0], r[1])
        if field == "total" and reg == 0:
            val += inc
        out.append(val)
    return np.array(out)


def incident(P: Panels, k, direction):
    d = np.ascontiguousarray(direction, dtype=np.float64)
    p = np.zeros(P.n, dtype=np.complex128)
    q = np.zeros(P.n, dtype=np.complex128)
    lib().oracle_incident(P.ptr, P.n, float(k), _dp(d), _dp(p),
                          _dp(q))
    return p, q


def far_field(P: Panels, k, xhat, p, q):
    out = np.zeros(2)
    xh = np.ascontiguousarray(xhat, dtype=np.float64)
    p = np.ascontiguousarray(p, dtype=np.complex128)
    q = np.ascontiguousarray(q, dtype=np.complex128)
    lib().oracle_far_field(P.ptr, P.n, float(k), _dp(xh), _dp(p),
                           _dp(q), _dp(out))
    return complex(out[0], out[1])


def pressure(P: Panels, k, points, p_scat, q_scat, direction, field="scattered", g=1.0,
             h=1.0, fluid=False, eta=NEAR_ETA):
    """Field at points from the scattered traces (fields/pressure.jl:404-471): exterior
    scattered D p - S q (plus the incident wave for "total"), interior S q_i - D p_i with
    p_i = p + p_inc, q_i = g (q + q_inc) at k / h."""
    L = lib()
    out = []
    p_inc, q_inc = incident(P, k, direction)
    for x in np.atleast_2d(np.asarray(points, dtype=np.float64)):
        x = np.ascontiguousarray(x)
        om = L.oracle_solid_angle(P.ptr, P.n, _dp(x))
        inside = om > 2 * math.pi
        if field == "incident":
            out.append(np.exp(1j * k * direction @ x))
            continue
        if inside:
            if not fluid or field == "scattered":
                raise ValueError("no exterior field inside the body")
            pi_, qi_ = np.ascontiguousarray(p_scat + p_inc), np.ascontiguousarray(g * (q_scat + q_inc))
            r = np.zeros(2)
            L.oracle_layer_potentials(P.ptr, P.n, k / h, _dp(x), eta, _dp(pi_), _dp(qi_), 1,
                                      _dp(r))
            out.append(complex(r[0], r[1]))
        else:
            if field == "interior":
                raise ValueError("interior field at an exterior point")
            ps, qs = np.ascontiguousarray(p_scat), np.ascontiguousarray(q_scat)
            r = np.zeros(2)
            L.oracle_layer_potentials(P.ptr, P.n, k, _dp(x), eta, _dp(ps), _dp(qs), 0, _dp(r))
            v = complex(r[0], r[1])
            if field == "total":
                v += np.exp(1j * k * direction @ x)
            out.append(v)
    return np.array(out)


def target_strength(f):
    """20 log10 |f| (postprocessing/target_strength.jl:8)."""
    return 20.0 * math.log10(abs(f))


# ---------------------------------------------------------------- GMRES
def gmres(A, b, reltol=1e-4, abstol=0.0, restart=150, maxiter=1200):
    """Restarted GMRES with the semantics of IterativeSolvers.gmres as the reference calls
    it for rigid/soft bodies (solvers/bem/full.jl:153-154, defaults full.jl:57): x0 = 0;
    stop when the residual estimate |g[j+1]| <= max(reltol |b|, abstol) or after maxiter
    Arnoldi steps; an explicit residual b - A x starts every restart cycle.  The Arnoldi
    vectors are orthogonalised by classical Gram-Schmidt with one reorthogonalisation and
    the Hessenberg matrix reduced by complex Givens rotations [c s; -conj(s) c].
    Returns x and dict(iterations, converged, history)."""
    b = np.asarray(b, dtype=np.complex128)
    n = b.size
    x = np.zeros(n, dtype=np.complex128)
    beta = float(np.linalg.norm(b))
    tol = max(reltol * beta, abstol)
    hist, iters, converged = [], 0, False
    r = b.copy()
    while True:
        if beta <= tol:
            converged = True
            break
        if iters >= maxiter:
            break
        V = np.zeros((n, restart + 1), dtype=np.complex128)
        H = np.zeros((restart + 1, restart), dtype=np.complex128)
        g = np.zeros(restart + 1, dtype=np.complex128)
        cs = np.zeros(restart)
        sn = np.zeros(restart, dtype=np.complex128)
        V[:, 0] = r / beta
        g[0] = beta
        kd = 0
        for j in range(restart):
            w = A @ V[:, j]
            for _ in range(2):
                h = V[:, :j + 1].conj().T @ w
                w = w - V[:, :j + 1] @ h
                H[:j + 1, j] += h
            hn = float(np.linalg.norm(w))
            H[j + 1, j] = hn
            V[:, j + 1] = w / hn if hn > 0 else 0.0
            for i in range(j):
                a, c2 = H[i, j], H[i + 1, j]
                H[i, j] = cs[i] * a + sn[i] * c2
                H[i + 1, j] = cs[i] * c2 - np.conj(sn[i]) * a
            a, c2 = H[j, j], H[j + 1, j]
            aa, bb = abs(a), abs(c2)
            if aa == 0.0:
                c, s, rr = 0.0, 1.0 + 0.0j, c2
            else:
                t = math.hypot(aa, bb)
                ph = a / aa
                c, s, rr = aa / t, ph * np.conj(c2) / t, ph * t
            cs[j], sn[j] = c, s
            H[j, j], H[j + 1, j] = rr, 0.0
            g[j + 1] = -np.conj(s) * g[j]
            g[j] = c * g[j]
            res = abs(g[j + 1])
            iters += 1
            hist.append(res)
            kd = j + 1
            if res <= tol:
                converged = True
                break
            if iters >= maxiter:
                break
        y = sla.solve_triangular(H[:kd, :kd], g[:kd], lower=False)
        x = x + V[:, :kd] @ y
        if converged or iters >= maxiter:
            break
        r = b - A @ x
        beta = float(np.linalg.norm(r))
    return x, dict(iterations=iters, converged=converged, history=np.array(hist))


def solve_gmres(nodes, triangles, boundary, k, incidence_angle=math.pi / 2,
                incidence_azimuth=0.0, formulation="burton_miller", eta=NEAR_ETA, panels=None,
                **gmres_kwargs):
    """The reference's rigid/soft path solve_full_bem (full.jl:52-184) with GMRES on the
    dense operators (compression=(method=:none,)): traces, backscatter and the GMRES
    report."""
    P = panels if panels is not None else Panels(nodes, triangles)
    d = incidence_direction(incidence_angle, incidence_azimuth)
    p_inc, q_inc = incident(P, k, d)
    M1, M2 = assemble_bm(P, k, formulation == "burton_miller", eta)
    if boundary == "rigid":
        A, b = M1, M2 @ q_inc
    elif boundary == "pressure_release":
        A, b = M2, M1 @ p_inc
    else:
        raise ValueError(f"unknown boundary {boundary!r}")
    x, rep = gmres(A, b, **gmres_kwargs)
    p_s, q_s = (x, -q_inc) if boundary == "rigid" else (-p_inc, x)
    amp = far_field(P, k, -d, p_s, q_s)
    rep.update(p_scat=p_s, dpdn_scat=q_s, amplitude=amp, A=A, b=b, x=x, panels=P)
    return rep


# ---------------------------------------------------------------- dense factor/solve
def equilibrate(A, norm_floor=0.0):
    """Row max, then column max of the row-scaled matrix, each bounded below by
    norm_floor (full.jl:388-394)."""
    rows = np.maximum(np.max(np.abs(A), axis=1), norm_floor)
    rows[rows == 0] = 1.0
    scaled = A / rows[:, None]
    cols = np.maximum(np.max(np.abs(scaled), axis=0), norm_floor)
    cols[cols == 0] = 1.0
    return rows, cols, scaled / cols[None, :]


class DoubleFactor:
    """Equilibrated complex128 LU (full.jl:364-409 with precision=:double)."""

    def __init__(self, A, equilibrate_rows=True, norm_floor=0.0):
        self.A = A
        if equilibrate_rows:
            self.rows, self.cols, S = equilibrate(A, norm_floor)
        else:
            self.rows = self.cols = None
            S = A.copy()
        self.lu = sla.lu_factor(S, check_finite=False)

    def solve(self, b):
        sb = b if self.rows is None else b / self.rows[:, None] if b.ndim == 2 else b / self.rows
        sx = sla.lu_solve(self.lu, sb, check_finite=False)
        if self.cols is None:
            return sx
        return sx / (self.cols[:, None] if sx.ndim == 2 else self.cols)


class MixedRefinement:
    """Guarded complex64 factorisation with complex128 residual refinement.

    Restates MixedRefinement in solvers/bem/fluid_system.jl:172-309: equilibration
    (:196-211), conversion check (:218), single LU + singular check (:219-221),
    infinity-norm reciprocal condition guard (:222-225), corrections (:229-239),
    backward errors (:241-262) and the accept / promote loop (:264-307).
    """

    def __init__(self, A, condition_guard=10 * np.finfo(np.float32).eps):
        n, m = A.shape
        if n != m or n == 0:
            raise ValueError("expected a nonempty square matrix")
        if not np.all(np.isfinite(A)):
            raise ValueError("matrix must be finite")
        self.A = A
        rows = np.max(np.abs(A), axis=1)
        rows[rows == 0] = 1.0
        cols = np.max(np.abs(A / rows[:, None]), axis=0)
        cols[cols == 0] = 1.0
        self.rows, self.cols = rows, cols
        self.matrix_norm = float(np.max(np.sum(np.abs(A), axis=1)))
        self.precision, self.reason = "single", "none"
        self.rcond = float("nan")
        with np.errstate(over="ignore", invalid="ignore"):
            low = (A / rows[:, None] / cols[None, :]).astype(np.complex64)
        if not np.all(np.isfinite(low)):
            self.promote("conversion")
            return
        anorm = float(np.max(np.sum(np.abs(low), axis=1)))
        lu, piv, info = sla.lapack.cgetrf(low)
        if info > 0:
            self.promote("single_singular")
            return
        self.lu = (lu, piv)
        rc, info = sla.lapack.cgecon(lu, anorm, norm="I")
        self.rcond = float(rc)
        if not math.isfinite(self.rcond) or self.rcond <= condition_guard:
            self.promote("condition")

    def promote(self, reason):
        scaled = self.A / self.rows[:, None] / self.cols[None, :]
        self.lu = sla.lu_factor(scaled, check_finite=False)
        self.precision, self.reason = "double", reason

    def correction(self, rhs):
        scaled = rhs / self.rows
        mag = float(np.max(np.abs(scaled))) if scaled.size else 0.0
        if not math.isfinite(mag):
            return np.full(rhs.shape, complex("nan"), dtype=np.complex128)
        if mag == 0.0:
            return np.zeros_like(rhs)
        work = scaled / mag
        if self.precision == "single":
            lu, piv = self.lu
            x, info = sla.lapack.cgetrs(lu, piv, work.astype(np.complex64))
            v = x.astype(np.complex128)
        else:
            v = sla.lu_solve(self.lu, work, check_finite=False)
        return v * mag / self.cols

    def backward_errors(self, x, b):
        residual = b - self.A @ x
        den = np.abs(b) + np.abs(self.A) @ np.abs(x)
        if not (np.all(np.isfinite(residual)) and np.all(np.isfinite(den))):
            return residual, math.inf, math.inf
        ar = np.abs(residual)
        with np.errstate(divide="ignore", invalid="ignore"):
            ratio = np.where(den == 0, np.where(ar == 0, 0.0, np.inf), ar / den)
        comp = float(np.max(ratio)) if ratio.size else 0.0
        scale = self.matrix_norm * float(np.max(np.abs(x))) + float(np.max(np.abs(b)))
        rn = float(np.max(ar))
        if not math.isfinite(scale):
            norm = math.inf
        elif scale == 0.0:
            norm = 0.0 if rn == 0.0 else math.inf
        else:
            norm = rn / scale
        return residual, norm, comp

    def solve(self, b, tolerance=1e-13, maxiter=8):
        x = self.correction(b)
        history = []
        corrections = attempts = stalls = 0
        previous = math.inf
        while True:
            residual, nw, cw = self.backward_errors(x, b)
            metric = max(nw, cw)
            history.append((self.precision, nw, cw))
            if math.isfinite(metric) and metric <= tolerance:
                return dict(x=x, precision=self.precision, reason=self.reason,
                            corrections=corrections, history=history, normwise=nw,
                            componentwise=cw)
            stalls = stalls + 1 if metric >= previous * 0.9 else 0
            reason = ("nonfinite" if not math.isfinite(metric) else
                      "iteration_limit" if attempts >= maxiter else
                      "stagnation" if stalls >= 2 else None)
            if reason is not None:
                if self.precision == "double":
                    raise RuntimeError(f"double-precision fallback failed: {reason}")
                self.promote(reason)
                x = self.correction(b)
                previous, attempts, stalls = math.inf, 0, 0
                continue
            updated = x + self.correction(residual)
            if np.array_equal(updated, x):
                if self.precision == "double":
                    raise RuntimeError("double-precision correction stagnated")
                self.promote("stagnation")
                x = self.correction(b)
                previous, attempts, stalls = math.inf, 0, 0
                continue
            x = updated
            previous = metric
            corrections += 1
            attempts += 1


# ---------------------------------------------------------------- the solve chain
def solve(nodes, triangles, boundary, k, incidence_angle=math.pi / 2,
          incidence_azimuth=0.0, formulation=None, g=1.0, h=1.0, precision="double",
          equilibrate_rows=True, directions=None, eta=NEAR_ETA, panels=None, norm_floor=0.0):
    """Scattered traces and far-field amplitudes for one (mesh, boundary, k, incidence).

    boundary: "rigid", "pressure_release" or "fluid".  Returns a dict with p_scat,
    dpdn_scat, the amplitudes at ``directions`` (default backscatter) and the panels.
    """
    if not (math.isfinite(k) and k > 0):
        raise ValueError("k must be finite and positive")
    P = panels if panels is not None else Panels(nodes, triangles)
    n = P.n
    d = incidence_direction(incidence_angle, incidence_azimuth)
    p_inc, q_inc = incident(P, k, d)
    info = {}
    if boundary in ("rigid", "pressure_release"):
        formulation = formulation or "burton_miller"
        M1, M2 = assemble_bm(P, k, formulation == "burton_miller", eta)
        if boundary == "rigid":
            A, b = M1, M2 @ q_inc
        else:
            A, b = M2, M1 @ p_inc
        F = DoubleFactor(A, equilibrate_rows, norm_floor)
        x = F.solve(b)
        if boundary == "rigid":
            p_s, q_s = x, -q_inc
        else:
            p_s, q_s = -p_inc, x
    elif boundary == "fluid":
        formulation = formulation or "muller"
        A = assemble_fluid(P, k, g, h, formulation, eta)
        if formulation == "muller":
            b = np.concatenate([p_inc, q_inc])
        else:
            b = np.zeros(2 * n, dtype=np.complex128)
            b[n:] = -(A[n:, :] @ np.concatenate([p_inc, q_inc]))
        if precision == "mixed":
            F = MixedRefinement(A)
            res = F.solve(b)
            x = res["x"]
            info.update(res)
        else:
            F = DoubleFactor(A, equilibrate_rows, norm_floor)
            x = F.solve(b)
        p_s, q_s = x[:n], x[n:]
        if formulation == "muller":
            p_s, q_s = p_s - p_inc, q_s - q_inc
    else:
        raise ValueError(f"unknown boundary {boundary!r}")
    if directions is None:
        directions = [-d]
    amps = np.array([far_field(P, k, xh, p_s, q_s) for xh in directions])
    info.update(p_scat=p_s, dpdn_scat=q_s, amplitudes=amps, panels=P, A=A, b=b, x=x)
    return info
