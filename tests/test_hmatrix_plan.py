"""Host logic of the compressed operators (no GPU): the block partition of the cluster tree
covers every matrix entry exactly once, keeps every near pair (singular-rule pair) in a
full leaf block, respects the leaf size and is deterministic."""
import ctypes

import numpy as np
import pytest

from bemgpu import _lib as C
from bemgpu import meshes


def _plan(nodes, tris, near_eta=2.0, **kw):
    L = C.lib()
    o = C.HmatrixOptions()
    L.bemgpu_hmatrix_options_init(ctypes.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    nodes = np.ascontiguousarray(np.asarray(nodes, dtype=np.float64).reshape(3, -1).T)
    tris = np.ascontiguousarray(np.asarray(tris, dtype=np.int64).reshape(3, -1).T)
    nn, nt = nodes.shape[0], tris.shape[0]
    counts = np.zeros(4, dtype=np.int64)
    rc = L.bemgpu_hmatrix_plan(C.dptr(nodes), nn, C.i64ptr(tris), nt, near_eta, ctypes.byref(o),
                               C.i64ptr(counts), None, 0, None)
    assert rc == 0
    cap = int(counts[0] + counts[1])
    blocks = np.zeros((cap, 5), dtype=np.int32)
    perm = np.zeros(nt, dtype=np.int32)
    i32 = ctypes.POINTER(ctypes.c_int32)
    rc = L.bemgpu_hmatrix_plan(C.dptr(nodes), nn, C.i64ptr(tris), nt, near_eta, ctypes.byref(o),
                               C.i64ptr(counts), blocks.ctypes.data_as(i32), cap,
                               perm.ctypes.data_as(i32))
    assert rc == 0
    # near pairs of the same surface
    rowptr = np.zeros(nt + 1, dtype=np.int64)
    cnt = ctypes.c_int64()
    L.bemgpu_near_pairs(C.dptr(nodes), nn, C.i64ptr(tris), nt, near_eta, C.i64ptr(rowptr), None,
                        0, ctypes.byref(cnt))
    cols = np.zeros(cnt.value, dtype=np.int64)
    assert L.bemgpu_near_pairs(C.dptr(nodes), nn, C.i64ptr(tris), nt, near_eta,
                               C.i64ptr(rowptr), C.i64ptr(cols), cnt.value,
                               ctypes.byref(cnt)) == 0
    return counts, blocks, perm, rowptr, cols


@pytest.mark.parametrize("mesh,leaf,eta", [
    (lambda: meshes.icosphere(0.01, 3), 64, 3.0),
    (lambda: meshes.uv_spheroid(0.02, 0.01, 64, 40, jitter=0.02, seed=7), 32, 2.0),
    (lambda: meshes.uv_spheroid(0.05, 0.0125, 48, 24), 16, 3.0),
])
def test_partition_covers_once_and_keeps_near_pairs_full(mesh, leaf, eta):
    nodes, tris = mesh()
    counts, blocks, perm, rowptr, cols = _plan(nodes, tris, leaf_size=leaf, eta=eta)
    n = perm.size
    assert np.array_equal(np.sort(perm), np.arange(n))
    assert counts[0] > 0 and counts[1] > 0  # something is compressed at these sizes
    cover = np.zeros((n, n), dtype=np.int16)
    owner = np.full((n, n), -1, dtype=np.int32)
    for b, (kind, r0, m, c0, w) in enumerate(blocks):
        cover[r0:r0 + m, c0:c0 + w] += 1
        owner[r0:r0 + m, c0:c0 + w] = b
        if kind == 0:
            assert m <= leaf and w <= leaf
    assert np.all(cover == 1)
    iperm = np.empty(n, dtype=np.int64)
    iperm[perm] = np.arange(n)
    rows = np.repeat(np.arange(n), np.diff(rowptr))
    kinds = blocks[owner[iperm[rows], iperm[cols]], 0]
    assert np.all(kinds == 0), "a near pair fell into a compressed block"
    # the diagonal is never compressed
    assert np.all(blocks[owner[np.arange(n), np.arange(n)], 0] == 0)


def test_partition_is_deterministic():
    nodes, tris = meshes.uv_spheroid(0.02, 0.01, 64, 40, jitter=0.02, seed=3)
    a = _plan(nodes, tris)
    b = _plan(nodes, tris)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_plan_rejects_bad_options():
    nodes, tris = meshes.icosphere(0.01, 2)
    L = C.lib()
    o = C.HmatrixOptions()
    L.bemgpu_hmatrix_options_init(ctypes.byref(o))
    # the reference's defaults (solvers/bem/full.jl:56-58); no Schwarz preconditioner
    assert (o.tol, o.eta, o.restart, o.reltol, o.maxiter, o.neighbours) == \
        (1e-5, 3.0, 150, 1e-4, 1200, 0)
    nodes = np.ascontiguousarray(np.asarray(nodes, dtype=np.float64).reshape(3, -1).T)
    tris = np.ascontiguousarray(np.asarray(tris, dtype=np.int64).reshape(3, -1).T)
    counts = np.zeros(4, dtype=np.int64)
    for field, bad in (("tol", 0.0), ("tol", 1.5), ("eta", -1.0), ("leaf_size", 4),
                       ("restart", 0), ("maxiter", -1), ("reltol", float("nan")),
                       ("neighbours", -1), ("neighbours", 129)):
        o2 = C.HmatrixOptions()
        ctypes.pointer(o2)[0] = o
        setattr(o2, field, bad)
        rc = L.bemgpu_hmatrix_plan(C.dptr(nodes), nodes.shape[0], C.i64ptr(tris), tris.shape[0],
                                   2.0, ctypes.byref(o2), C.i64ptr(counts), None, 0, None)
        assert rc == 1, (field, bad)
