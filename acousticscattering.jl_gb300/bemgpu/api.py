"""Host-side mirror of AcousticScattering.jl's full-3D BEM interface over libbemgpu.

Names, arguments and error behaviour follow the reference:

  mesh(nodes, triangles)                        geometry/surface.jl:271-298 (validation
                                                 surface.jl:341-405)
  bem(surface, boundary, k; incidence_angle=pi/2, incidence_azimuth=0, ...)
                                                solvers/bem/surface.jl:10-23 with the
                                                 options of full.jl:52-58 and :273-279
  scattering_amplitude(sol; direction)          solvers/bem/postprocessing.jl:1-13
  target_strength(sol_or_f; direction)          postprocessing/target_strength.jl:8, 26
  diagnostics(sol)                              solvers/shared/postprocessing.jl:17
  incidence_angle_sweep(surface, boundary, k, angles)   postprocessing/sweeps.jl:626-701
  frequency_sweep(solve, frequencies, c)        postprocessing/sweeps.jl:103-110
  Rigid / PressureRelease / FluidFilled         core/materials.jl:16-76

Invalid arguments raise ArgumentError (a ValueError), as the reference's ArgumentError;
non-convergence of the double-precision fallback raises RuntimeError, as its error().
Every numerical operation runs in libbemgpu on the GPU; there is no CPU path.
"""
from __future__ import annotations

import ctypes
import math
import warnings
from dataclasses import dataclass, field

import numpy as np

from . import _lib as C


class ArgumentError(ValueError):
    """Invalid argument (the reference's ArgumentError)."""


class BEMGPUError(RuntimeError):
    """Device-side failure reported by libbemgpu."""


# ------------------------------------------------------------------ boundary conditions
class AbstractBoundaryCondition:
    pass


class Rigid(AbstractBoundaryCondition):
    """Zero total normal velocity (core/materials.jl:16)."""

    code = C.RIGID

    def __repr__(self):
        return "Rigid()"


class PressureRelease(AbstractBoundaryCondition):
    """Zero total pressure (core/materials.jl:23)."""

    code = C.PRESSURE_RELEASE

    def __repr__(self):
        return "PressureRelease()"


class FluidFilled(AbstractBoundaryCondition):
    """Homogeneous fluid interior: density_contrast g = rho_i/rho_e, soundspeed_contrast
    h = c_i/c_e (core/materials.jl:62-76)."""

    code = C.FLUID

    def __init__(self, density_contrast: float, soundspeed_contrast: float):
        self.density_contrast = float(density_contrast)
        self.soundspeed_contrast = float(soundspeed_contrast)

    def __repr__(self):
        return f"FluidFilled({self.density_contrast}, {self.soundspeed_contrast})"


GasFilled = FluidFilled

_FORMULATIONS = {None: C.FORMULATION_DEFAULT, "burton_miller": C.BURTON_MILLER,
                 "cbie": C.CBIE, "muller": C.MULLER}
_FORMULATION_NAMES = {C.BURTON_MILLER: "burton_miller", C.CBIE: "cbie", C.MULLER: "muller"}


# ------------------------------------------------------------------ errors / context
def _last_error(ctx=None) -> str:
    buf = ctypes.create_string_buffer(512)
    C.lib().bemgpu_last_error(ctx, buf, 512)
    return buf.value.decode(errors="replace")


def _check(status: int, ctx=None):
    if status == C.OK:
        return
    msg = _last_error(ctx)
    if status in (C.EINVAL, C.ETOPOLOGY):
        raise ArgumentError(msg)
    if status == C.ENOTCONVERGED:
        raise RuntimeError(msg)
    name = C.lib().bemgpu_status_string(status).decode()
    raise BEMGPUError(f"{name}: {msg}")


class Context:
    """One device context (stream, HBM budget, caching allocator)."""

    def __init__(self, device: int = 0, hbm_budget_bytes: int = 0):
        h = ctypes.c_void_p()
        _check(C.lib().bemgpu_ctx_create(device, hbm_budget_bytes, ctypes.byref(h)))
        self.handle = h
        self.device = device

    def memory(self):
        used, budget = ctypes.c_uint64(), ctypes.c_uint64()
        _check(C.lib().bemgpu_ctx_memory(self.handle, ctypes.byref(used), ctypes.byref(budget)),
               self.handle)
        return used.value, budget.value

    def synchronize(self):
        _check(C.lib().bemgpu_ctx_synchronize(self.handle), self.handle)

    def set_autotune(self, enable: bool = True):
        """Measured launch shapes (panel cluster size, residual rows per thread); every
        choice gives bit-identical results."""
        _check(C.lib().bemgpu_ctx_set_autotune(self.handle, int(enable)), self.handle)

    def profile(self, enable: bool = True):
        _check(C.lib().bemgpu_profile_enable(self.handle, int(enable)), self.handle)

    def profile_reset(self):
        _check(C.lib().bemgpu_profile_reset(self.handle), self.handle)

    def profile_read(self, family: str):
        n, ms = ctypes.c_int64(), ctypes.c_double()
        _check(C.lib().bemgpu_profile_read(self.handle, family.encode(), ctypes.byref(n),
                                           ctypes.byref(ms)), self.handle)
        return n.value, ms.value

    def set_graphs(self, enable: bool = True):
        """Capture and replay the batched LU's launch sequence as CUDA graphs (default on)."""
        _check(C.lib().bemgpu_ctx_set_graphs(self.handle, int(bool(enable))), self.handle)

    def inject_alloc_failures(self, count: int):
        """Test hook: the next ``count`` device allocations of this context and its lanes
        fail as if cudaMalloc had run out of memory (0 cancels)."""
        _check(C.lib().bemgpu_ctx_inject_alloc_failures(self.handle, int(count)), self.handle)

    def graph_stats(self) -> dict:
        """Batched-LU graphs captured and replayed so far."""
        cap, rep = ctypes.c_int64(), ctypes.c_int64()
        _check(C.lib().bemgpu_ctx_graph_stats(self.handle, ctypes.byref(cap), ctypes.byref(rep)),
               self.handle)
        return {"captures": cap.value, "replays": rep.value}

    def set_tensor_lu(self, enable: bool):
        """Complex64 LU trailing updates on the tensor cores (default) or CUDA cores."""
        _check(C.lib().bemgpu_ctx_set_tensor_lu(self.handle, int(enable)), self.handle)

    def debug_cgemm(self, A, B, C_):
        """C - A B through the split-BF16 tensor-core update (complex64 testing hook)."""
        A = np.asfortranarray(A, dtype=np.complex64)
        B = np.asfortranarray(B, dtype=np.complex64)
        out = np.asfortranarray(np.array(C_, dtype=np.complex64))
        m, k = A.shape
        n = B.shape[1]
        _check(C.lib().bemgpu_debug_cgemm(self.handle, m, n, k, C.fptr(A), C.fptr(B),
                                          C.fptr(out)), self.handle)
        return out

    def timer_start(self):
        _check(C.lib().bemgpu_timer_start(self.handle), self.handle)

    def timer_stop(self) -> float:
        ms = ctypes.c_double()
        _check(C.lib().bemgpu_timer_stop(self.handle, ctypes.byref(ms)), self.handle)
        return ms.value

    @staticmethod
    def launch_count() -> int:
        n = ctypes.c_int64()
        C.lib().bemgpu_launch_count(None, ctypes.byref(n))
        return n.value

    def close(self):
        if getattr(self, "handle", None):
            C.lib().bemgpu_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_DEFAULT: Context | None = None


def context() -> Context:
    """The process-wide default context on device 0 (created on first use)."""
    global _DEFAULT
    if _DEFAULT is None:
        _DEFAULT = Context(0)
    return _DEFAULT


# ------------------------------------------------------------------ surfaces
class Mesh:
    """A validated closed flat-triangle surface (the reference's Mesh of a supplied
    surface).  ``nodes`` 3 x N float64, ``triangles`` 3 x M int64 (1-based)."""

    def __init__(self, nodes, triangles, units: str = "m", provenance="supplied triangles"):
        nodes = np.asarray(nodes, dtype=np.float64)
        tris = np.asarray(triangles)
        if nodes.ndim != 2 or nodes.shape[0] != 3:
            raise ArgumentError("nodes must have three rows")
        if tris.ndim != 2 or tris.shape[0] != 3:
            raise ArgumentError("triangles must have 3 rows in Gmsh ordering (flat triangles)")
        if not np.issubdtype(tris.dtype, np.integer):
            raise ArgumentError("triangles must be integer node indices")
        scale = {"m": 1.0, "cm": 0.01, "mm": 0.001}.get(units)
        if scale is None:
            raise ArgumentError("units must be :m, :cm or :mm")
        self.nodes = np.asfortranarray(nodes * scale)
        self.triangles = np.asfortranarray(tris.astype(np.int64))
        if self.triangles.shape[1] == 0:
            raise ArgumentError("surface must contain triangles")
        res = ctypes.c_double()
        err = ctypes.create_string_buffer(256)
        st = C.lib().bemgpu_mesh_validate(C.dptr(self.nodes), self.nodes.shape[1],
                                          C.i64ptr(self.triangles), self.triangles.shape[1],
                                          ctypes.byref(res), err, 256)
        if st != C.OK:
            raise ArgumentError(err.value.decode())
        self.resolution = res.value
        h = ctypes.create_string_buffer(65)
        C.lib().bemgpu_mesh_hash(C.dptr(self.nodes), self.nodes.shape[1],
                                 C.i64ptr(self.triangles), self.triangles.shape[1], h)
        self.hash = h.value.decode()
        self.provenance = provenance
        self._handles: dict[int, ctypes.c_void_p] = {}

    @property
    def n_panels(self) -> int:
        return int(self.triangles.shape[1])

    def handle(self, ctx: Context):
        key = id(ctx)
        if key not in self._handles:
            h = ctypes.c_void_p()
            _check(C.lib().bemgpu_mesh_upload(ctx.handle, C.dptr(self.nodes), self.nodes.shape[1],
                                              C.i64ptr(self.triangles), self.triangles.shape[1],
                                              ctypes.byref(h)), ctx.handle)
            self._handles[key] = (ctx, h)
        return self._handles[key][1]

    def release(self):
        for ctx, h in self._handles.values():
            C.lib().bemgpu_mesh_destroy(h)
        self._handles.clear()

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass


def mesh(nodes, triangles, *, units: str = "m") -> Mesh:
    """Supplied closed surface (geometry/surface.jl:271-298)."""
    return Mesh(nodes, triangles, units=units)


# ------------------------------------------------------------------ problems
def _problem(boundary, k, formulation=None, precision="double", equilibrate=True,
             refinement=None, near_eta=2.0, assembly=None,
             discretization="collocation", condition_limit=512,
             norm_floor=0.0) -> C.Problem:
    if not isinstance(boundary, AbstractBoundaryCondition):
        raise ArgumentError("boundary must be Rigid(), PressureRelease() or FluidFilled(g, h)")
    if discretization not in C.DISCRETIZATION:
        raise ArgumentError("discretization must be :collocation or :nystrom")
    if formulation not in _FORMULATIONS:
        raise ArgumentError("formulation must be :burton_miller, :cbie or :muller")
    if precision not in ("double", "mixed"):
        raise ArgumentError("precision must be :double or :mixed")
    if assembly not in C.ASSEMBLY:
        raise ArgumentError("assembly must be :double or :single")
    refinement = dict(refinement or {})
    unknown = set(refinement) - {"tolerance", "maxiter", "condition_guard"}
    if unknown:
        raise ArgumentError("unknown refinement option")
    if refinement and precision != "mixed":
        raise ArgumentError("refinement options require precision=:mixed")
    maxiter = refinement.get("maxiter", 8)
    if not isinstance(maxiter, (int, np.integer)) or maxiter < 0:
        raise ArgumentError("maxiter must be a nonnegative integer")
    k = float(k)
    if not (math.isfinite(k) and k > 0):
        raise ArgumentError("k must be finite and positive")
    if precision == "mixed" and not equilibrate:
        raise ArgumentError("mixed precision requires equilibrate=true")
    if not isinstance(condition_limit, (int, np.integer)) or condition_limit < 0:
        raise ArgumentError("condition_limit must be nonnegative")
    norm_floor = float(norm_floor)
    if not (math.isfinite(norm_floor) and norm_floor >= 0):
        raise ArgumentError("norm_floor must be finite and nonnegative")
    if precision == "mixed" and norm_floor != 0.0:
        raise ArgumentError("mixed precision does not support norm_floor")
    tol = refinement.get("tolerance", 1e-13)
    if not (math.isfinite(tol) and 0 < tol < 1):
        raise ArgumentError("invalid refinement tolerance")
    guard = refinement.get("condition_guard", 10 * float(np.finfo(np.float32).eps))
    if not (math.isfinite(guard) and guard >= 0):
        raise ArgumentError("invalid condition guard")
    if isinstance(boundary, FluidFilled):
        g, h = boundary.density_contrast, boundary.soundspeed_contrast
        if not (math.isfinite(g) and g > 0 and math.isfinite(h) and h > 0):
            raise ArgumentError(
                "fluid density and soundspeed contrasts must be finite and positive")
        if formulation not in (None, "muller", "cbie"):
            raise ArgumentError("fluid formulation must be :muller or :cbie")
    elif formulation not in (None, "burton_miller", "cbie"):
        raise ArgumentError("formulation must be :cbie or :burton_miller")
    p = C.Problem()
    C.lib().bemgpu_problem_init(ctypes.byref(p))
    p.boundary = boundary.code
    p.formulation = _FORMULATIONS[formulation]
    p.precision = C.MIXED if precision == "mixed" else C.DOUBLE
    p.equilibrate = int(bool(equilibrate))
    p.k = float(k)
    if isinstance(boundary, FluidFilled):
        p.density_contrast = boundary.density_contrast
        p.soundspeed_contrast = boundary.soundspeed_contrast
    p.refine_tolerance = float(refinement.get("tolerance", 1e-13))
    p.refine_maxiter = int(maxiter)
    p.condition_guard = float(refinement.get("condition_guard", 10 * np.finfo(np.float32).eps))
    p.near_eta = float(near_eta)
    p.assembly = C.ASSEMBLY[assembly]
    p.discretization = C.DISCRETIZATION[discretization]
    p.condition_limit = int(condition_limit)
    p.norm_floor = norm_floor
    return p


def _discretization(problem) -> str:
    return "nystrom" if problem.discretization == C.DISCRETIZATION["nystrom"] else "collocation"


def _direction(beta, alpha):
    """Polar angle from +x, azimuth from +y toward +z (solvers/bem/full.jl:14-18)."""
    return np.array([math.cos(beta), math.sin(beta) * math.cos(alpha),
                     math.sin(beta) * math.sin(alpha)])


def _diag_dict(d: C.Diagnostics, extra=None) -> dict:
    out = {f: getattr(d, f) for f, _ in C.Diagnostics._fields_}
    out["formulation"] = _FORMULATION_NAMES.get(d.formulation, "cbie")
    out["precision"] = "mixed" if d.precision == C.MIXED else "double"
    out["factor_precision"] = "single" if d.factor_precision == 0 else "double"
    out["refinement_reason"] = C.REASONS[d.refinement_reason]
    out["coupling"] = complex(d.coupling_re, d.coupling_im)
    out["method"] = "mixed_refinement" if d.precision == C.MIXED else "direct"
    out["equilibrate"] = bool(d.equilibrate)
    # the reference's factor diagnostics (solvers/bem/full.jl:364-409, 330-341)
    svd = d.conditioning == 1
    out["conditioning"] = "svd" if svd else "not_computed"
    out["condition_number"] = d.condition_number if svd else None
    out["scaled_condition_number"] = d.scaled_condition_number if svd else None
    names = {0: "not_used", 1: "direct"}
    fluid_muller = out["formulation"] == "muller"
    out["derivative_evaluation"] = ({"exterior": names[d.derivative_exterior],
                                     "interior": names[d.derivative_interior]}
                                    if fluid_muller else None)
    for f_ in ("derivative_exterior", "derivative_interior"):
        out.pop(f_)
    if extra:
        out.update(extra)
    return out


# ------------------------------------------------------------------ factor / solution
class Factor:
    """Assembled and factored system of one (surface, boundary, k): serves any number
    of incidence directions (the reuse of incidence_angle_sweep, sweeps.jl:680-701)."""

    def __init__(self, surface: Mesh, boundary, k, ctx: Context | None = None, **options):
        self.problem = _problem(boundary, k, **options)
        self.ctx = ctx or context()
        self.surface, self.boundary, self.k = surface, boundary, float(k)
        h = ctypes.c_void_p()
        _check(C.lib().bemgpu_factor_create(self.ctx.handle, surface.handle(self.ctx),
                                            ctypes.byref(self.problem), ctypes.byref(h)),
               self.ctx.handle)
        self.handle = h

    @classmethod
    def _wrap(cls, ctx, handle, surface, boundary, k, problem):
        f = cls.__new__(cls)
        f.ctx, f.handle, f.surface, f.boundary, f.k, f.problem = (ctx, handle, surface,
                                                                  boundary, float(k), problem)
        return f

    def solve(self, angles, azimuths=0.0) -> "BEMSolution":
        angles = np.atleast_1d(np.asarray(angles, dtype=np.float64))
        az = np.broadcast_to(np.asarray(azimuths, dtype=np.float64), angles.shape)
        inc = np.ascontiguousarray(np.stack([angles, az], axis=1).reshape(-1))
        h = ctypes.c_void_p()
        _check(C.lib().bemgpu_factor_solve(self.handle, len(angles), C.dptr(inc),
                                           ctypes.byref(h)), self.ctx.handle)
        return BEMSolution(self.ctx, h, self.surface, self.boundary, self.k, angles, az,
                           discretization=_discretization(self.problem))

    def diagnostics(self) -> dict:
        d = C.Diagnostics()
        _check(C.lib().bemgpu_factor_diagnostics(self.handle, ctypes.byref(d)))
        return _diag_dict(d)

    def close(self):
        if getattr(self, "handle", None):
            C.lib().bemgpu_factor_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class BEMSolution:
    """Result of bem(): surface traces of one or more incidence directions
    (the reference's BEMSolution{_FullBEMSurfaceData}, solvers/bem/types.jl:2-36)."""

    method = "full"

    def __init__(self, ctx, handle, surface, boundary, k, angles, azimuths,
                 discretization="collocation"):
        self.ctx, self.handle = ctx, handle
        self.discretization = discretization
        self.body = surface
        self.boundary = boundary
        self.k = float(k)
        self.incidence_angles = np.asarray(angles, dtype=np.float64)
        self.incidence_azimuths = np.asarray(azimuths, dtype=np.float64)

    @property
    def incidence_angle(self):
        return float(self.incidence_angles[0])

    @property
    def incidence_azimuth(self):
        return float(self.incidence_azimuths[0])

    @property
    def nrhs(self):
        return len(self.incidence_angles)

    def far_field(self, directions=None, rhs: int = 0) -> np.ndarray:
        if directions is None:
            out = np.zeros(1, dtype=np.complex128)
            _check(C.lib().bemgpu_far_field(self.handle, rhs, 1, None, C.dptr(out)),
                   self.ctx.handle)
            return out
        d = np.ascontiguousarray(np.asarray(directions, dtype=np.float64).reshape(-1, 3))
        out = np.zeros(d.shape[0], dtype=np.complex128)
        _check(C.lib().bemgpu_far_field(self.handle, rhs, d.shape[0], C.dptr(d), C.dptr(out)),
               self.ctx.handle)
        return out

    @property
    def n_panels(self) -> int:
        if isinstance(self.body, (list, tuple)):
            return sum(s.n_panels for s in self.body)
        return self.body.n_panels

    def region_traces(self, rhs: int = 0):
        """Coupled regions: total pressure p and flux unknown v at every unknown location
        (panel, or quadrature node for the Nyström discretisation), surfaces in order (the
        interior normal derivative is density_i v)."""
        n = self.n_nodes
        p = np.zeros(n, dtype=np.complex128)
        v = np.zeros(n, dtype=np.complex128)
        _check(C.lib().bemgpu_region_traces(self.handle, rhs, C.dptr(p), C.dptr(v)),
               self.ctx.handle)
        return p, v

    @property
    def n_nodes(self) -> int:
        """Unknown locations: panel centroids (collocation) or quadrature nodes (Nyström,
        node q of panel t at index 7 t + q)."""
        return self.n_panels * C.NODES_PER_PANEL[self.discretization]

    def traces(self, rhs: int = 0):
        """Scattered pressure and normal derivative at every unknown location (n_nodes)."""
        n = self.n_nodes
        p = np.zeros(n, dtype=np.complex128)
        q = np.zeros(n, dtype=np.complex128)
        _check(C.lib().bemgpu_traces(self.handle, rhs, C.dptr(p), C.dptr(q)), self.ctx.handle)
        return p, q

    @property
    def p_scat(self):
        return self.traces(0)[0]

    @property
    def dpdn_scat(self):
        return self.traces(0)[1]

    def pressure(self, points, field: str = "total", rhs: int = 0, region=None) -> np.ndarray:
        """Field at points; region (coupled-region solutions only, fields/pressure.jl:42-53):
        None = each point's own region, else 0 (unbounded) or an interface index."""
        if field not in C.FIELDS:
            raise ArgumentError("field must be :total, :scattered, :incident or :interior")
        if region is not None and not (isinstance(region, (int, np.integer)) and region >= 0):
            raise ArgumentError("region must be zero or an interface index")
        pts = np.ascontiguousarray(np.asarray(points, dtype=np.float64).reshape(-1, 3))
        out = np.zeros(pts.shape[0], dtype=np.complex128)
        if pts.shape[0]:
            _check(C.lib().bemgpu_pressure_region(
                self.handle, rhs, pts.shape[0], C.dptr(pts), C.FIELDS[field],
                -1 if region is None else int(region), C.dptr(out)), self.ctx.handle)
        return out

    def hmatrix_stats(self) -> dict:
        """Compression and GMRES statistics (compressed-operator solutions)."""
        st = C.HmatrixStats()
        _check(C.lib().bemgpu_hmatrix_stats_get(self.handle, ctypes.byref(st)), self.ctx.handle)
        return {f: getattr(st, f) for f, _ in C.HmatrixStats._fields_ if f != "pad"}

    def residual_history(self, rhs: int = 0) -> np.ndarray:
        """GMRES residual estimates, one per Arnoldi step (compressed-operator solutions)."""
        cnt = ctypes.c_int32()
        _check(C.lib().bemgpu_gmres_history(self.handle, rhs, None, 0, ctypes.byref(cnt)),
               self.ctx.handle)
        out = np.zeros(max(1, cnt.value))
        _check(C.lib().bemgpu_gmres_history(self.handle, rhs, C.dptr(out), cnt.value,
                                            ctypes.byref(cnt)), self.ctx.handle)
        return out[:cnt.value]

    def diagnostics(self) -> dict:
        d = C.Diagnostics()
        _check(C.lib().bemgpu_solution_diagnostics(self.handle, ctypes.byref(d)))
        if self.method == "hmatrix":  # the reference's GMRES diagnostics (full.jl:160-176)
            st = self.hmatrix_stats()
            return _diag_dict(d, {"method": "gmres", "converged": bool(st["gmres_converged"]),
                                  "iterations": st["gmres_iterations"],
                                  "residual_history": self.residual_history(0),
                                  "compression": st, "meshsize": self.body.resolution,
                                  "illumination": "plane_wave", "mesh_hash": self.body.hash})
        if isinstance(self.body, (list, tuple)):  # coupled regions
            return _diag_dict(d, {"meshsize": max(s_.resolution for s_ in self.body),
                                  "illumination": "plane_wave", "interface_count": len(self.body),
                                  "mesh_hash": [s_.hash for s_ in self.body]})
        extra = {"meshsize": self.body.resolution, "illumination": "plane_wave",
                 "mesh_hash": self.body.hash, "discretization": self.discretization}
        if self.discretization == "nystrom":
            extra["correction"] = {"method": "dim", "basis": "plane_waves"}
        return _diag_dict(d, extra)

    def close(self):
        if getattr(self, "handle", None):
            C.lib().bemgpu_solution_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------------------------ compressed operators
_GMRES_KEYS = {"reltol", "abstol", "restart", "maxiter"}


def _hmatrix_options(compression, gmres_kwargs):
    """HmatrixOptions for compression=(method=:hmatrix, tol[, eta, leaf_size]) with
    gmres_kwargs, or None for the dense path (full.jl:52-58 defaults)."""
    comp = dict(compression or {"method": "none"})
    method = comp.pop("method", "none")
    gm = dict(gmres_kwargs or {})
    if set(gm) - _GMRES_KEYS:
        raise ArgumentError(f"unknown gmres option(s): {sorted(set(gm) - _GMRES_KEYS)}")
    if method == "none":
        if comp:
            raise ArgumentError("compression=(method=:none,) takes no other options")
        return None
    if method != "hmatrix":
        raise ArgumentError("compression method must be :none or :hmatrix")
    keys = {"tol", "eta", "leaf_size", "neighbours"}
    if set(comp) - keys:
        raise ArgumentError(f"unknown compression option(s): {sorted(set(comp) - keys)}")
    o = C.HmatrixOptions()
    C.lib().bemgpu_hmatrix_options_init(ctypes.byref(o))
    o.tol = float(comp.get("tol", o.tol))
    o.eta = float(comp.get("eta", o.eta))
    o.leaf_size = int(comp.get("leaf_size", o.leaf_size))
    o.neighbours = int(comp.get("neighbours", o.neighbours))
    o.reltol = float(gm.get("reltol", o.reltol))
    o.abstol = float(gm.get("abstol", o.abstol))
    o.restart = int(gm.get("restart", o.restart))
    o.maxiter = int(gm.get("maxiter", o.maxiter))
    return o


def _bem_hmatrix(surface, boundary, k, angles, azimuths, opts, *, formulation, precision, ctx,
                 discretization="collocation"):
    if isinstance(boundary, FluidFilled):
        raise ArgumentError(
            "hierarchical compression applies to Rigid and PressureRelease boundaries")
    ctx = ctx or context()
    p = _problem(boundary, k, formulation=formulation, precision=precision,
                 discretization=discretization)
    angles = np.atleast_1d(np.asarray(angles, dtype=np.float64))
    az = np.broadcast_to(np.asarray(azimuths, dtype=np.float64), angles.shape)
    inc = np.ascontiguousarray(np.stack([angles, az], axis=1).reshape(-1))
    h = ctypes.c_void_p()
    _check(C.lib().bemgpu_hmatrix_solve(ctx.handle, surface.handle(ctx), ctypes.byref(p),
                                        ctypes.byref(opts), len(angles), C.dptr(inc),
                                        ctypes.byref(h)), ctx.handle)
    sol = BEMSolution(ctx, h, surface, boundary, k, angles, az, discretization=discretization)
    sol.method = "hmatrix"
    st = sol.hmatrix_stats()
    if not st["gmres_converged"]:
        warnings.warn("solve_full_bem: GMRES did not converge to the requested tolerance, "
                      f"result may be inaccurate (boundary={boundary}, "
                      f"iters={st['gmres_iterations']})", RuntimeWarning, stacklevel=3)
    return sol


def hmatrix_apply(surface: Mesh, boundary, k, X, *, op=0, formulation=None, tol=1e-5,
                  eta=3.0, leaf_size=64, precision="double", ctx=None):
    """Products M X of the compressed rigid/soft operators (op 0: M1 = 1/2 I - D - a H,
    op 1: M2 = S + a (1/2 I + K')) and their statistics, for inspecting the compression.
    precision="mixed": complex64 operators with FP32 entries and products."""
    ctx = ctx or context()
    p = _problem(boundary, k, formulation=formulation, precision=precision)
    o = _hmatrix_options(dict(method="hmatrix", tol=tol, eta=eta, leaf_size=leaf_size), None)
    X = np.asarray(X, dtype=np.complex128)
    if X.ndim == 1:
        X = X[:, None]
    X = np.asfortranarray(X)
    Y = np.zeros_like(X, order="F")
    st = C.HmatrixStats()
    _check(C.lib().bemgpu_hmatrix_apply(ctx.handle, surface.handle(ctx), ctypes.byref(p),
                                        ctypes.byref(o), int(op), X.shape[1], C.dptr(X),
                                        C.dptr(Y), ctypes.byref(st)), ctx.handle)
    return Y, {f: getattr(st, f) for f, _ in C.HmatrixStats._fields_ if f != "pad"}


# ------------------------------------------------------------------ reference-named API
def bem(surface: Mesh, boundary, k, *, incidence_angle=math.pi / 2, incidence_azimuth=0.0,
        formulation=None, precision="double", equilibrate=True, refinement=None,
        assembly=None, ctx: Context | None = None, parents=None, compression=None,
        gmres_kwargs=None, discretization="collocation", condition_limit=512, norm_floor=0.0,
        **unsupported) -> BEMSolution:
    """Full-3D BEM on a supplied surface (solvers/bem/surface.jl:10-23), or, given lists of
    surfaces and FluidFilled materials, the coupled fluid regions of
    bem(surfaces, materials, k; parents) (solvers/bem/regions.jl:132-150).

    compression=dict(method="hmatrix", tol=1e-5) selects the reference's compressed
    operators with GMRES (solve_full_bem, full.jl:52-58; gmres_kwargs reltol, abstol,
    restart, maxiter as there) for Rigid and PressureRelease bodies; precision="mixed"
    then stores the operators as complex64 with FP32 entries and products (GMRES itself
    stays FP64), which limits the attainable relative residual to about 1e-6.  Without it
    (or with method="none") the system is factored densely; gmres_kwargs then have no
    effect, as the direct solve meets any GMRES tolerance.

    discretization="nystrom" (one surface, dense factor) puts the unknowns on the seven
    quadrature nodes of every panel with the density-interpolation correction of the
    reference's Nyström operators (full.jl:68-128 and 289-346, correction=(method=:dim,));
    traces then hold one value per node, and pressure() recovers the nearest element by
    the same correction (the reference's exclude_nearest evaluation).

    condition_limit and norm_floor are the reference's factor options (full.jl:364-409):
    systems of order at most condition_limit report SVD condition numbers in
    diagnostics(); norm_floor bounds the equilibration's scales from below (double
    precision only)."""
    if unsupported:
        raise ArgumentError(f"unsupported option(s): {sorted(unsupported)}")
    if discretization not in C.DISCRETIZATION:
        raise ArgumentError("discretization must be :collocation or :nystrom")
    hm = _hmatrix_options(compression, gmres_kwargs)
    if hm is not None:
        if isinstance(surface, (list, tuple)) or parents is not None:
            raise ArgumentError("hierarchical compression applies to a single surface")
        if not isinstance(surface, Mesh):
            raise ArgumentError("surface must be a Mesh from mesh(nodes, triangles)")
        if not (math.isfinite(incidence_angle) and math.isfinite(incidence_azimuth)):
            raise ArgumentError("incidence angles must be finite")
        return _bem_hmatrix(surface, boundary, k, [incidence_angle], [incidence_azimuth], hm,
                            formulation=formulation, precision=precision, ctx=ctx,
                            discretization=discretization)
    if isinstance(surface, (list, tuple)):
        return _bem_regions(list(surface), boundary, k, parents=parents,
                            incidence_angle=incidence_angle,
                            incidence_azimuth=incidence_azimuth, formulation=formulation,
                            precision=precision, equilibrate=equilibrate,
                            refinement=refinement, assembly=assembly, ctx=ctx,
                            discretization=discretization)
    if parents is not None:
        raise ArgumentError("parents applies to lists of surfaces and materials")
    if not isinstance(surface, Mesh):
        raise ArgumentError("surface must be a Mesh from mesh(nodes, triangles)")
    if not (math.isfinite(incidence_angle) and math.isfinite(incidence_azimuth)):
        raise ArgumentError("incidence angles must be finite")
    k = float(k)
    if not (math.isfinite(k) and k > 0):
        raise ArgumentError("k must be finite and positive")
    f = Factor(surface, boundary, k, ctx=ctx, formulation=formulation, precision=precision,
               equilibrate=equilibrate, refinement=refinement, assembly=assembly,
               discretization=discretization, condition_limit=condition_limit,
               norm_floor=norm_floor)
    try:
        return f.solve([incidence_angle], [incidence_azimuth])
    finally:
        f.close()


def _bem_regions(surfaces, materials, k, *, parents, incidence_angle, incidence_azimuth,
                 formulation, precision, equilibrate, refinement, assembly, ctx,
                 discretization="collocation"):
    ctx = ctx or context()
    count = len(surfaces)
    if count == 0:
        raise ArgumentError("at least one interface is required")
    materials = list(materials) if isinstance(materials, (list, tuple)) else None
    if materials is None or len(materials) != count:
        raise ArgumentError("supply one material and parent per interface")
    if not all(isinstance(s_, Mesh) for s_ in surfaces):
        raise ArgumentError("each interface must be a Mesh from mesh(nodes, triangles)")
    if not all(isinstance(m, FluidFilled) for m in materials):
        raise ArgumentError("materials must be FluidFilled")
    parents = list(range(count)) if parents is None else [int(p) for p in parents]
    if len(parents) != count:
        raise ArgumentError("supply one material and parent per interface")
    if not all(0 <= parents[i] <= i for i in range(count)):
        raise ArgumentError("each parent must be zero or an earlier region index")
    if formulation not in (None, "muller", "cbie"):
        raise ArgumentError("formulation must be :muller or :cbie")
    if not (math.isfinite(incidence_angle) and math.isfinite(incidence_azimuth)):
        raise ArgumentError("incidence angles must be finite")
    # the problem fields that apply (boundary and contrasts are per region)
    p = _problem(FluidFilled(1.0, 1.0), float(k), formulation=formulation,
                 precision=precision, equilibrate=equilibrate, refinement=refinement,
                 assembly=assembly, discretization=discretization)
    handles = (ctypes.c_void_p * count)(*[s_.handle(ctx) for s_ in surfaces])
    dens = np.array([m.density_contrast for m in materials], dtype=np.float64)
    speeds = np.array([m.soundspeed_contrast for m in materials], dtype=np.float64)
    par = (ctypes.c_int32 * count)(*parents)
    inc = np.array([incidence_angle, incidence_azimuth], dtype=np.float64)
    out = ctypes.c_void_p()
    _check(C.lib().bemgpu_region_solve(ctx.handle, count, handles, C.dptr(dens), C.dptr(speeds),
                                       par, ctypes.byref(p), 1, C.dptr(inc), ctypes.byref(out)),
           ctx.handle)
    return BEMSolution(ctx, out, list(surfaces), list(materials), float(k), [incidence_angle],
                       [incidence_azimuth], discretization=discretization)


def factor_batch(items, ctx: Context | None = None):
    """Assemble and factor many problems in fused batched launches.

    ``items``: sequence of (surface, boundary, k, options-dict).  Returns Factors in order.
    """
    ctx = ctx or context()
    items = list(items)
    if not items:
        raise ArgumentError("empty batch")
    probs = (C.Problem * len(items))()
    meshes = (ctypes.c_void_p * len(items))()
    for t, (surf, bc, k, opts) in enumerate(items):
        probs[t] = _problem(bc, k, **(opts or {}))
        meshes[t] = surf.handle(ctx)
    outs = (ctypes.c_void_p * len(items))()
    _check(C.lib().bemgpu_factor_create_batch(ctx.handle, len(items), meshes, probs, outs),
           ctx.handle)
    return [Factor._wrap(ctx, ctypes.c_void_p(outs[t]), items[t][0], items[t][1], items[t][2],
                         probs[t]) for t in range(len(items))]


def solve_batch(factors, angles, azimuths=None):
    """Solve every factor for its incidence set in one batched launch sequence.

    ``angles[i]`` (and ``azimuths[i]``) are the polar (azimuthal) angles of factor i."""
    factors = list(factors)
    ctx = factors[0].ctx
    n = len(factors)
    incs, keep = [], []
    nr = (ctypes.c_int32 * n)()
    ptrs = (ctypes.POINTER(ctypes.c_double) * n)()
    for t, f in enumerate(factors):
        a = np.atleast_1d(np.asarray(angles[t], dtype=np.float64))
        z = np.broadcast_to(np.asarray(0.0 if azimuths is None else azimuths[t],
                                       dtype=np.float64), a.shape)
        inc = np.ascontiguousarray(np.stack([a, z], axis=1).reshape(-1))
        keep.append((a, z, inc))
        nr[t] = len(a)
        ptrs[t] = C.dptr(inc)
    fh = (ctypes.c_void_p * n)(*[f.handle for f in factors])
    outs = (ctypes.c_void_p * n)()
    _check(C.lib().bemgpu_factor_solve_batch(ctx.handle, n, fh, nr, ptrs, outs), ctx.handle)
    return [BEMSolution(ctx, ctypes.c_void_p(outs[t]), factors[t].surface, factors[t].boundary,
                        factors[t].k, keep[t][0], keep[t][1]) for t in range(n)]


def scattering_amplitude(sol: BEMSolution, *, direction=None, rhs: int = 0) -> complex:
    """Far-field amplitude f(x_hat) [m]; default backscatter x_hat = -d
    (solvers/bem/postprocessing.jl:1-13)."""
    if direction is not None:
        d = np.asarray(direction, dtype=np.float64).reshape(-1)
        if d.size != 3 or not np.all(np.isfinite(d)) or abs(np.linalg.norm(d) - 1) > 1e-8:
            raise ArgumentError("direction must be a finite unit vector with three components")
        return complex(sol.far_field(d, rhs)[0])
    return complex(sol.far_field(None, rhs)[0])


def target_strength(x, *, direction=None, rhs: int = 0) -> float:
    """20 log10 |f| (postprocessing/target_strength.jl:8, 26)."""
    if isinstance(x, BEMSolution):
        x = scattering_amplitude(x, direction=direction, rhs=rhs)
    return 20.0 * math.log10(abs(x))


def diagnostics(sol) -> dict:
    return sol.diagnostics()


def pressure(sol: BEMSolution, points, *, field: str = "total", rhs: int = 0, region=None):
    """Pressure at points (fields/pressure.jl:42-53, full-BEM branch :404-471).

    ``points``: one point (3 numbers) -> complex; a sequence of points or a 3 x N / N x 3
    array -> complex array.  field: "total" (incident + scattered outside, interior field
    inside a fluid body), "scattered", "incident" or "interior".  region (coupled-region
    solutions, fields/regions.jl:1-65): None = each point's own region, else 0 (the
    unbounded region) or an interface index whose interior the point belongs to."""
    arr = np.asarray(points, dtype=np.float64)
    if arr.size == 0:
        return np.zeros(0, dtype=np.complex128)
    single = arr.ndim == 1
    if single and arr.size != 3:
        raise ArgumentError("a point has three coordinates")
    if arr.ndim == 2 and arr.shape[0] == 3 and arr.shape[1] != 3:
        arr = arr.T
    if not np.all(np.isfinite(arr)):
        raise ArgumentError("point coordinates must be finite")
    out = sol.pressure(arr.reshape(-1, 3), field=field, rhs=rhs, region=region)
    return complex(out[0]) if single else out


class Server:
    """Continuous-batching request loop of libbemgpu.

    submit() queues one surface / boundary problem at several wavenumbers and incidence
    directions and returns a ticket; wait() returns the backscatter amplitudes
    (nfreq x nangles) and the request's latency.  ``lanes`` batches run on the device at
    once, each on its own streams; a free lane takes waiting work of one size class, so
    short requests overtake long ones.  Factors are cached across requests (LRU,
    ``cache_bytes``; 0 = a quarter of the budget)."""

    def __init__(self, ctx: Context | None = None, max_batch: int = 64, queue_limit: int = 4096,
                 cache_bytes: int = 0, lanes: int = 2):
        self.ctx = ctx or context()
        o = C.ServerOptions()
        C.lib().bemgpu_server_options_init(ctypes.byref(o))
        o.max_batch, o.queue_limit, o.cache_bytes = max_batch, queue_limit, cache_bytes
        o.lanes = lanes
        h = ctypes.c_void_p()
        _check(C.lib().bemgpu_server_create(self.ctx.handle, ctypes.byref(o), ctypes.byref(h)),
               self.ctx.handle)
        self.handle = h
        self._shapes = {}

    def submit(self, surface: Mesh, boundary, ks, angles, azimuths=0.0, **options) -> int:
        ks = np.atleast_1d(np.asarray(ks, dtype=np.float64))
        a = np.atleast_1d(np.asarray(angles, dtype=np.float64))
        z = np.broadcast_to(np.asarray(azimuths, dtype=np.float64), a.shape)
        inc = np.ascontiguousarray(np.stack([a, z], axis=1).reshape(-1))
        p = _problem(boundary, float(ks[0]), **options)
        t = ctypes.c_int64()
        _check(C.lib().bemgpu_server_submit(self.handle, surface.handle(self.ctx), ctypes.byref(p),
                                            len(ks), C.dptr(np.ascontiguousarray(ks)), len(a),
                                            C.dptr(inc), ctypes.byref(t)), self.ctx.handle)
        self._shapes[t.value] = (len(ks), len(a))
        return t.value

    def wait(self, ticket: int, timeout_ms: int = -1):
        nf, na = self._shapes.pop(ticket)
        out = np.zeros((nf, na), dtype=np.complex128)
        lat = ctypes.c_double()
        st = C.lib().bemgpu_server_wait(self.handle, ticket, timeout_ms, C.dptr(out),
                                        ctypes.byref(lat))
        if st == C.ETIMEOUT:
            self._shapes[ticket] = (nf, na)
            raise TimeoutError("request not finished")
        _check(st, self.ctx.handle)
        return out, lat.value

    def stats(self) -> dict:
        s = C.ServerStats()
        _check(C.lib().bemgpu_server_stats_get(self.handle, ctypes.byref(s)))
        return {f: getattr(s, f) for f, _ in C.ServerStats._fields_}

    def close(self):
        if getattr(self, "handle", None):
            C.lib().bemgpu_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass
class SweepResult:
    angles: np.ndarray
    amplitudes: np.ndarray
    target_strength: np.ndarray
    diagnostics: dict = field(default_factory=dict)


def incidence_angle_sweep(surface: Mesh, boundary, k, angles, *, incidence_azimuth=0.0,
                          formulation=None, precision="double", equilibrate=True,
                          refinement=None, assembly=None, ctx=None, compression=None,
                          gmres_kwargs=None, discretization="collocation", condition_limit=512,
                          norm_floor=0.0) -> SweepResult:
    """Backscatter at many polar incidence angles from one factorisation
    (postprocessing/sweeps.jl:626-701): assembled and factored once, all angles
    solved as one multi-right-hand-side batch.  With compression=(method=:hmatrix, ...)
    the operators are compressed once and every angle runs its own GMRES (batched)."""
    angles = np.asarray(angles, dtype=np.float64)
    if angles.ndim != 1 or angles.size == 0 or not np.all(np.isfinite(angles)):
        raise ArgumentError("angles must be a nonempty vector of finite values")
    if not math.isfinite(incidence_azimuth):
        raise ArgumentError("incidence_azimuth must be finite")
    hm = _hmatrix_options(compression, gmres_kwargs)
    if hm is not None:
        sol = _bem_hmatrix(surface, boundary, k, angles, incidence_azimuth, hm,
                           formulation=formulation, precision=precision, ctx=ctx,
                           discretization=discretization)
        try:
            amps = np.array([scattering_amplitude(sol, rhs=r) for r in range(len(angles))])
            diag = sol.diagnostics()
        finally:
            sol.close()
        return SweepResult(angles, amps, 20 * np.log10(np.abs(amps)), diag)
    f = Factor(surface, boundary, k, ctx=ctx, formulation=formulation, precision=precision,
               equilibrate=equilibrate, refinement=refinement, assembly=assembly,
               discretization=discretization, condition_limit=condition_limit,
               norm_floor=norm_floor)
    try:
        sol = f.solve(angles, incidence_azimuth)
        amps = np.array([scattering_amplitude(sol, rhs=r) for r in range(len(angles))])
        diag = sol.diagnostics()
        sol.close()
    finally:
        f.close()
    return SweepResult(angles, amps, 20 * np.log10(np.abs(amps)), diag)


@dataclass
class FrequencySweep:
    frequencies: np.ndarray
    k: np.ndarray
    target_strength: np.ndarray
    amplitudes: np.ndarray


def frequency_sweep(solve, frequencies, sound_speed) -> FrequencySweep:
    """Call ``solve(k)`` for each frequency (postprocessing/sweeps.jl:103-110)."""
    if not (math.isfinite(sound_speed) and sound_speed > 0):
        raise ArgumentError("sound_speed must be finite and positive")
    freqs = np.asarray(frequencies, dtype=np.float64)
    if not np.all(freqs > 0):
        raise ArgumentError("frequencies must be positive")
    ks = 2 * math.pi * freqs / sound_speed
    amps = []
    for k in ks:
        s = solve(k)
        amps.append(scattering_amplitude(s) if isinstance(s, BEMSolution) else complex(s))
    amps = np.array(amps)
    return FrequencySweep(freqs, ks, 20 * np.log10(np.abs(amps)), amps)


def dense_solve(A, B, *, precision="double", equilibrate=True, refinement=None, ctx=None):
    """Solve A X = B with the BEM factor path (full.jl:364-440; fluid_system.jl:172-309)
    for a hand-built complex matrix; returns (X, diagnostics)."""
    ctx = ctx or context()
    A = np.asfortranarray(np.asarray(A, dtype=np.complex128))
    B = np.asarray(B, dtype=np.complex128)
    vec = B.ndim == 1
    X = np.asfortranarray(B.reshape(B.shape[0], -1).copy())
    n = A.shape[0]
    if A.ndim != 2 or A.shape[1] != n or n == 0:
        raise ArgumentError("expected a nonempty square matrix")
    if X.shape[0] != n:
        raise ArgumentError("right-hand side length")
    p = _problem(Rigid(), 1.0, precision=precision, equilibrate=equilibrate,
                 refinement=refinement)
    d = C.Diagnostics()
    _check(C.lib().bemgpu_dense_solve(ctx.handle, n, C.dptr(A), X.shape[1], C.dptr(X),
                                      p.precision, p.equilibrate, p.refine_tolerance,
                                      p.refine_maxiter, p.condition_guard, ctypes.byref(d)),
           ctx.handle)
    return (X[:, 0] if vec else X), _diag_dict(d)


def assemble(surface: Mesh, boundary, k, *, formulation=None, precision="double",
             assembly=None, ctx=None, discretization="collocation"):
    """The assembled operators (rigid/soft: M1 = 1/2 I - D - a H and
    M2 = S + a (1/2 I + K'); fluid: the 2n x 2n system) as complex128 arrays; Nyström:
    the node operators (7 n x 7 n) with the element corrections applied."""
    ctx = ctx or context()
    p = _problem(boundary, k, formulation=formulation, precision=precision, assembly=assembly,
                 discretization=discretization)
    n = surface.n_panels * C.NODES_PER_PANEL[discretization]
    if isinstance(boundary, FluidFilled):
        M1 = np.zeros((2 * n, 2 * n), dtype=np.complex128, order="F")
        _check(C.lib().bemgpu_assemble_dense(ctx.handle, surface.handle(ctx), ctypes.byref(p),
                                             C.dptr(M1), None), ctx.handle)
        return M1
    M1 = np.zeros((n, n), dtype=np.complex128, order="F")
    M2 = np.zeros((n, n), dtype=np.complex128, order="F")
    _check(C.lib().bemgpu_assemble_dense(ctx.handle, surface.handle(ctx), ctypes.byref(p),
                                         C.dptr(M1), C.dptr(M2)), ctx.handle)
    return M1, M2
