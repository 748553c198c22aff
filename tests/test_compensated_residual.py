"""The FP64-accurate residual of the mixed path in FP32 arithmetic (refine.cu, gemv_a32_body),
emulated on the CPU operation by operation: a complex64 matrix times an FP64 vector split
as hi + lo in FP32, each product split exactly into p + e (its FMA error term), the
products summed as TwoSum pairs (s, t), the pairs folded into FP64 every 32 columns, eight
column chunks added in order.  The mixed refinement accepts a solution at a componentwise
backward error of 1e-13 (fluid_system.jl:241-262), so the residual's own rounding must
stay below 1e-13 of |b| + |A||x| in every row; plain FP32 sums are off by about 1e-7 of
it."""
import math

import numpy as np

from bemgpu import meshes
from oracle import oracle as O

F = np.float32


def _pair_add_prod(s, t, u, v):
    """pair_add_prod of refine.cu on float32 arrays (u * v is exact in float64, so the
    FMA error term is exact too)."""
    p = (u * v).astype(F)
    e = (u.astype(np.float64) * v.astype(np.float64) - p.astype(np.float64)).astype(F)
    s2 = (s + p).astype(F)
    bb = (s2 - s).astype(F)
    err = ((s - (s2 - bb).astype(F)).astype(F) + (p - bb).astype(F)).astype(F)
    t2 = (t + (err + e).astype(F)).astype(F)
    return s2, t2


def _fma(a, b, c):
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(F)


def _gpu_product(A32, x, chunks=8, fold=32):
    """y = A x as the compact residual kernel computes it (all rows at once)."""
    n = A32.shape[1]
    ar, ai = A32.real.astype(F), A32.imag.astype(F)
    hr, hi = x.real.astype(F), x.imag.astype(F)
    lr = (x.real - hr.astype(np.float64)).astype(F)
    li = (x.imag - hi.astype(np.float64)).astype(F)
    w = (n + chunks - 1) // chunks
    total = np.zeros(A32.shape[0], dtype=np.complex128)
    for c in range(chunks):
        j0, j1 = min(n, c * w), min(n, c * w + w)
        acc_r = np.zeros(A32.shape[0])
        acc_i = np.zeros(A32.shape[0])
        for jf in range(j0, j1, fold):
            rs = rt = is_ = it = np.zeros(A32.shape[0], dtype=F)
            for j in range(jf, min(j1, jf + fold)):
                a_x, a_y = ar[:, j], ai[:, j]
                xr, xi, xlr, xli = hr[j], hi[j], lr[j], li[j]
                rs, rt = _pair_add_prod(rs, rt, a_x, np.full_like(a_x, xr))
                rs, rt = _pair_add_prod(rs, rt, -a_y, np.full_like(a_x, xi))
                is_, it = _pair_add_prod(is_, it, a_x, np.full_like(a_x, xi))
                is_, it = _pair_add_prod(is_, it, a_y, np.full_like(a_x, xr))
                rt = _fma(a_x, np.full_like(a_x, xlr), _fma(-a_y, np.full_like(a_x, xli), rt))
                it = _fma(a_x, np.full_like(a_x, xli), _fma(a_y, np.full_like(a_x, xlr), it))
            acc_r += rs.astype(np.float64) + rt.astype(np.float64)
            acc_i += is_.astype(np.float64) + it.astype(np.float64)
        total += acc_r + 1j * acc_i
    return total


def _systems():
    k = 2 * math.pi * 38e3 / 1477.4
    M1, _ = O.assemble_bm(O.Panels(*meshes.icosphere(0.01, 2)), k, True)      # 320 x 320
    F2 = O.assemble_fluid(O.Panels(*meshes.icosphere(0.01, 1)), k, 1.05, 1.02, "muller")
    return [M1, F2]                                                          # 160 x 160


def test_compact_residual_is_accurate_enough_for_the_refinement():
    """For an exact solution x (b = A x), the residual the kernel computes is its rounding
    error alone, and max |r| / (|b| + |A||x|) is the componentwise backward error the
    refinement would report: it must stay below the 1e-13 at which the refinement accepts.
    Measured with this emulation: at most about 6e-14 on these small systems (median about
    3e-15), where one dominant diagonal block carries most of a row; plain FP32 sums give
    about 1e-7."""
    for A in _systems():
        A32 = A.astype(np.complex64)
        n = A.shape[0]
        for seed in range(3):
            rng = np.random.default_rng(seed)
            x = np.linalg.solve(A32.astype(np.complex128),
                                rng.standard_normal(n) + 1j * rng.standard_normal(n))
            b = A32.astype(np.clongdouble) @ x.astype(np.clongdouble)
            den = np.abs(A32).astype(np.float64) @ np.abs(x) + np.abs(b.astype(np.complex128))
            got = _gpu_product(A32, x)
            err = np.abs(got - b.astype(np.complex128)) / den
            assert err.max() < 1e-13 and np.median(err) < 1e-14, (n, seed, err.max())
            plain = (A32 @ x.astype(np.complex64)).astype(np.complex128)
            assert (np.abs(plain - b.astype(np.complex128)) / den).max() > 1e-9
