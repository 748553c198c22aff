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


def _dev(a):
    # column-major complex64 on the device: the transpose of a C-contiguous buffer
    t = torch.from_numpy(np.ascontiguousarray(a.T)).to("cuda")
    return t


def _noalloc(A, B, Cm):
    m, k = A.shape
    n = B.shape[1]
    dA, dB, dC = _dev(A), _dev(B), _dev(Cm)
    stream = torch.cuda.current_stream().cuda_stream
    st = C.lib().bemgpu_cgemm_update_noalloc(ctypes.c_void_p(stream), m, n, k,
                                             ctypes.c_void_p(dA.data_ptr()), m,
                                             ctypes.c_void_p(dB.data_ptr()), k,
                                             ctypes.c_void_p(dC.data_ptr()), m)
    return st, dC.cpu().numpy().T


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


def test_noalloc_rejects_sizes_beyond_its_array():
    rng = np.random.default_rng(1)
    A, B, Cm = _cplx(rng, (8, 129)), _cplx(rng, (129, 8)), _cplx(rng, (8, 8))
    st, _ = _noalloc(A, B, Cm)
    assert st == C.EINVAL
    assert "maximum" in bemgpu.api._last_error()
