"""Host-side checks that need no GPU: surface generators, the C ABI's host functions
(topology validation, SHA-256, near pairs) against the oracle, the exported symbol
set, and argument validation of the Python mirror."""
import ctypes
import json
import math
import os
import re

import numpy as np
import pytest

import bemgpu
from bemgpu import _lib as C
from bemgpu import meshes
from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def test_workload_mesh_counts_and_hashes():
    want = json.load(open(os.path.join(GOLDEN, "mesh_hashes.json")))
    got = {"icosphere_0.01_3": meshes.icosphere(0.01, 3),
           "uv_spheroid_0.02_0.01_64x40_j0.02_s20261203":
               meshes.uv_spheroid(0.02, 0.01, 64, 40, jitter=0.02, seed=20261203),
           "uv_spheroid_0.05_0.0125_128x80": meshes.uv_spheroid(0.05, 0.0125, 128, 80)}
    for name, (nodes, tris) in got.items():
        assert nodes.shape[1] == want[name]["nodes"]
        assert tris.shape[1] == want[name]["triangles"]
        assert meshes.mesh_hash(nodes, tris) == want[name]["hash"]
    assert (642, 1280) == (got["icosphere_0.01_3"][0].shape[1],
                           got["icosphere_0.01_3"][1].shape[1])


def test_library_hash_matches_python():
    nodes, tris = meshes.uv_spheroid(0.02, 0.01, 16, 10, jitter=0.02, seed=3)
    s = bemgpu.mesh(nodes, tris)
    assert s.hash == meshes.mesh_hash(nodes, tris)


def test_library_near_pairs_match_oracle():
    for nodes, tris in (meshes.icosphere(1.0, 2),
                        meshes.uv_spheroid(0.02, 0.01, 24, 16, jitter=0.02, seed=9),
                        meshes.body_of_revolution(0.01, 4.0, [0.03, -0.02, 0.01, 0.04], 20, 30)):
        n = tris.shape[1]
        rp = np.zeros(n + 1, dtype=np.int64)
        cap = 200 * n
        cols = np.zeros(cap, dtype=np.int64)
        cnt = ctypes.c_int64()
        nf = np.asfortranarray(nodes)
        tf = np.asfortranarray(tris)
        st = C.lib().bemgpu_near_pairs(C.dptr(nf), nf.shape[1], C.i64ptr(tf), n, 2.0,
                                       C.i64ptr(rp), C.i64ptr(cols), cap, ctypes.byref(cnt))
        assert st == C.OK
        orp, ocols = O.Panels(nodes, tris).near_pairs(2.0)
        assert np.array_equal(rp, orp)
        assert np.array_equal(cols[:cnt.value], ocols)


def _tetra():
    nodes = np.array([[0.0, 1, 0, 0], [0, 0, 1, 0], [0, 0, 0, 1]])
    tris = np.array([[1, 1, 1, 2], [3, 2, 4, 3], [2, 4, 3, 4]])
    return nodes, tris


def test_validation_accepts_reference_tetrahedron():
    nodes, tris = _tetra()
    s = bemgpu.mesh(nodes, tris)
    assert s.n_panels == 4 and s.resolution == pytest.approx(math.sqrt(2))


@pytest.mark.parametrize("mutate,msg", [
    (lambda n, t: (n, t[:, :3]), "incident triangles"),
    (lambda n, t: (n, t[[0, 2, 1], :]), "positive volume"),
    (lambda n, t: (n, np.concatenate([t[:, :3], t[[0, 2, 1], 3:]], axis=1)), "orientation"),
    (lambda n, t: (n, np.where(t == 4, 5, t)), "invalid node index"),
    (lambda n, t: (np.where(np.isclose(n, 1.0), np.nan, n), t), "finite"),
    (lambda n, t: (n, np.concatenate([t[:, :1], [[1], [1], [2]], t[:, 1:]], axis=1)),
     "repeats a node"),
])
def test_validation_rejects(mutate, msg):
    nodes, tris = mutate(*_tetra())
    with pytest.raises(bemgpu.ArgumentError, match=msg):
        bemgpu.mesh(nodes, tris)


def test_validation_rejects_disconnected_and_nonmanifold():
    n1, t1 = _tetra()
    n2 = n1 + 5.0
    nodes = np.concatenate([n1, n2], axis=1)
    tris = np.concatenate([t1, t1 + 4], axis=1)
    with pytest.raises(bemgpu.ArgumentError, match="connected"):
        bemgpu.mesh(nodes, tris)
    # two tetrahedra sharing one vertex: every edge has two triangles, the shared
    # vertex has two separate fans
    n3 = np.concatenate([n1, (n1[:, 1:] * -1.0)], axis=1)
    t2 = np.where(t1 == 1, 1, t1 + 3)
    t2 = t2[[0, 2, 1], :]
    with pytest.raises(bemgpu.ArgumentError, match="nonmanifold|connected"):
        bemgpu.mesh(n3, np.concatenate([t1, t2], axis=1))


def test_library_exports_every_declared_symbol():
    header = open(os.path.join(ROOT, "include", "bemgpu.h")).read()
    declared = set(re.findall(r"^(?:int|void|const char \*)\s*(bemgpu_\w+)\(", header, re.M))
    assert len(declared) > 30
    L = C.lib()
    missing = [name for name in declared if not hasattr(L, name)]
    assert not missing, missing
    assert declared == set(C.SIGNATURES), declared ^ set(C.SIGNATURES)
    assert C.lib().bemgpu_version().decode().startswith("bemgpu")


def test_problem_defaults_follow_reference():
    p = C.Problem()
    C.lib().bemgpu_problem_init(ctypes.byref(p))
    assert p.refine_tolerance == 1e-13 and p.refine_maxiter == 8
    assert p.condition_guard == pytest.approx(10 * np.finfo(np.float32).eps)
    assert p.equilibrate == 1 and p.formulation == C.FORMULATION_DEFAULT
    # the reference's _factor_fluid_system defaults (full.jl:364-366)
    assert p.condition_limit == 512 and p.norm_floor == 0.0
    o = C.ServerOptions()
    C.lib().bemgpu_server_options_init(ctypes.byref(o))
    assert o.max_batch == 64 and o.lanes == 2


@pytest.mark.parametrize("kw,msg", [
    (dict(k=0.0), "k must be"), (dict(k=-1.0), "k must be"), (dict(k=math.inf), "k must be"),
    (dict(k=math.nan), "k must be"), (dict(formulation="unknown"), "formulation"),
    (dict(precision="invalid"), "precision"),
    (dict(precision="mixed", equilibrate=False), "equilibrate"),
    (dict(refinement={"maxiter": 2}), "require precision"),
    (dict(precision="mixed", refinement={"maxiter": -1}), "maxiter"),
    (dict(precision="mixed", refinement={"tolerance": math.nan}), "tolerance"),
    (dict(precision="mixed", refinement={"unknown": 1}), "unknown refinement"),
    (dict(incidence_angle=math.nan), "incidence"),
    (dict(condition_limit=-1), "condition_limit"),
    (dict(norm_floor=-1.0), "norm_floor"), (dict(norm_floor=math.nan), "norm_floor"),
    (dict(precision="mixed", norm_floor=1.0), "norm_floor"),
])
def test_bem_argument_errors_before_any_device_work(kw, msg):
    nodes, tris = _tetra()
    s = bemgpu.mesh(nodes, tris)
    k = kw.pop("k", 0.3)
    with pytest.raises(bemgpu.ArgumentError, match=msg):
        bemgpu.bem(s, bemgpu.Rigid(), k, **kw)


@pytest.mark.parametrize("g,h", [(0.0, 1.0), (1.0, -1.0), (math.inf, 1.0), (1.0, math.nan)])
def test_fluid_contrast_errors(g, h):
    nodes, tris = _tetra()
    with pytest.raises(bemgpu.ArgumentError, match="contrasts"):
        bemgpu.bem(bemgpu.mesh(nodes, tris), bemgpu.FluidFilled(g, h), 1.0)


def test_fluid_formulation_error():
    nodes, tris = _tetra()
    with pytest.raises(bemgpu.ArgumentError, match="fluid formulation"):
        bemgpu.bem(bemgpu.mesh(nodes, tris), bemgpu.FluidFilled(1.2, 1.1), 1.0,
                   formulation="burton_miller")


def test_context_without_gpu_reports_no_device():
    n = ctypes.c_int()
    try:
        import subprocess
        has_gpu = subprocess.run(["nvidia-smi", "-L"], capture_output=True).returncode == 0
    except OSError:
        has_gpu = False
    if has_gpu:
        pytest.skip("a GPU is present")
    with pytest.raises(bemgpu.BEMGPUError, match="no CUDA device"):
        bemgpu.Context(0)
