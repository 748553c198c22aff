"""The allocation-free entry point bemgpu_cgemm_update_noalloc, checked through the C ABI.

It serves callers that cannot allocate device memory where they need the complex64
tensor-core update (hosts whose HBM belongs to their own pool allocator, codes that may
not allocate after start-up): its scratch is a fixed file-scope device array.  The test
compares it with the allocating entry point bemgpu_debug_cgemm on the same data, on two
calls in a row with different data (the shared array must not carry state between
calls), and checks that sizes beyond the array's limit are rejected.  The device
buffers of the test itself come from torch.
"""
import ctypes

import numpy as np
import pytest

import bemgpu
from bemgpu import _lib as C

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _cplx(rng, shape):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)


def _dev(a, ld=None, fill=0):
    """Column-major complex64 on the device with leading dimension ld >= rows: the
    transpose of a C-contiguous (cols, ld) buffer whose rows beyond the matrix hold
    `fill`."""
    rows, cols = a.shape
    ld = ld or rows
    host = np.full((cols, ld), fill, dtype=np.complex64)
    host[:, :rows] = a.T
    return torch.from_numpy(host).to("cuda")


def _noalloc(A, B, Cm, lda=None, ldb=None, ldc=None):
    m, k = A.shape
    n = B.shape[1]
    lda, ldb, ldc = lda or m, ldb or k, ldc or m
    dA, dB, dC = _dev(A, lda, 7 + 7j), _dev(B, ldb, -5 + 1j), _dev(Cm, ldc, 3 - 2j)
    stream = torch.cuda.current_stream().cuda_stream
    st = C.lib().bemgpu_cgemm_update_noalloc(ctypes.c_void_p(stream), m, n, k,
                                             ctypes.c_void_p(dA.data_ptr()), lda,
                                             ctypes.c_void_p(dB.data_ptr()), ldb,
                                             ctypes.c_void_p(dC.data_ptr()), ldc)
    full = dC.cpu().numpy()
    # the rows of C's buffer beyond the matrix must be untouched
    assert np.all(full[:, m:] == np.complex64(3 - 2j))
    return st, full[:, :m].T


def test_noalloc_matches_allocating_entry_point_twice(ctx):
    rng = np.random.default_rng(7)
    for (m, n, k) in ((300, 257, 96), (128, 640, 128)):
        A, B, Cm = _cplx(rng, (m, k)), _cplx(rng, (k, n)), _cplx(rng, (m, n))
        st, got = _noalloc(A, B, Cm)
        assert st == C.OK, bemgpu.api._last_error()
        want = ctx.debug_cgemm(A, B, Cm)
        scale = np.linalg.norm(A) * np.linalg.norm(B)
        assert np.linalg.norm(got - want) / scale < 1e-6
        ref = Cm.astype(np.complex128) - A.astype(np.complex128) @ B.astype(np.complex128)
        assert np.linalg.norm(got - ref) / scale < 5e-5


@pytest.mark.parametrize("m,n,k,pad", [(300, 200, 40, (5, 3, 9)), (2048, 2048, 128, (0, 0, 0)),
                                       (129, 2048, 33, (1, 2, 3))])
def test_noalloc_padded_partial_and_maximal_sizes(ctx, m, n, k, pad):
    """Leading dimensions larger than the matrices, a K that is no multiple of the
    32-wide chunk, and the largest accepted size (whose packed images fill the array)."""
    rng = np.random.default_rng(m + n + k)
    A, B, Cm = _cplx(rng, (m, k)), _cplx(rng, (k, n)), _cplx(rng, (m, n))
    st, got = _noalloc(A, B, Cm, m + pad[0], k + pad[1], m + pad[2])
    assert st == C.OK, bemgpu.api._last_error()
    ref = Cm.astype(np.complex128) - A.astype(np.complex128) @ B.astype(np.complex128)
    scale = np.linalg.norm(A) * np.linalg.norm(B)
    assert np.linalg.norm(got - ref) / scale < 5e-5
    want = ctx.debug_cgemm(A, B, Cm)
    assert np.linalg.norm(got - want) / scale < 1e-6


def test_noalloc_rejects_sizes_beyond_its_array():
    rng = np.random.default_rng(1)
    A, B, Cm = _cplx(rng, (8, 129)), _cplx(rng, (129, 8)), _cplx(rng, (8, 8))
    st, _ = _noalloc(A, B, Cm)
    assert st == C.EINVAL
    assert "maximum" in bemgpu.api._last_error()
