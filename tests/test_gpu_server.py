"""Continuous-batching server: every result is the same alone and in the mix, factors are
reused across requests, and the budget-driven admission completes everything."""
import math

import numpy as np
import pytest

import bemgpu
from bemgpu import meshes

pytestmark = pytest.mark.gpu


def _surfaces():
    a = bemgpu.mesh(*meshes.icosphere(0.01, 2))
    b = bemgpu.mesh(*meshes.uv_spheroid(0.02, 0.008, 24, 16, jitter=0.02, seed=5))
    c = bemgpu.mesh(*meshes.body_of_revolution(0.01, 2.5, [0.03, -0.02, 0.01, 0.04], 16, 20))
    return a, b, c


def test_same_alone_and_in_the_mix(ctx):
    a, b, c = _surfaces()
    req = (a, bemgpu.Rigid(), [300.0, 420.0], [0.3, 1.1, 2.0])
    srv = bemgpu.Server(ctx, max_batch=8)
    try:
        t = srv.submit(*req, precision="mixed")
        alone, lat = srv.wait(t)
        assert lat > 0 and np.all(np.isfinite(alone))
    finally:
        srv.close()
    # a fresh server (empty factor cache): the same request among others of different
    # sizes and kinds, submitted together, is assembled, factored and solved inside the
    # mixed batches, not served from the lone run's factors
    srv = bemgpu.Server(ctx, max_batch=8)
    try:
        tickets = [srv.submit(b, bemgpu.FluidFilled(1.0357, 1.0279), [500.0, 700.0], [0.5],
                              precision="mixed"),
                   srv.submit(*req, precision="mixed"),
                   srv.submit(c, bemgpu.PressureRelease(), [250.0], [0.2, 0.4],
                              precision="mixed"),
                   srv.submit(a, bemgpu.Rigid(), [300.0], [0.7], precision="double")]
        res = [srv.wait(tk)[0] for tk in tickets]
        st = srv.stats()
    finally:
        srv.close()
    assert st["cache_hits"] == 0 and st["factorizations"] == 6, st
    assert np.array_equal(res[1], alone)   # bit-identical: batching is not arithmetic
    assert st["completed"] == 4 and st["failed"] == 0


def test_batch_out_of_device_memory_runs_again_alone(ctx):
    """A batch whose device allocation fails (injected on the host: the allocator sees
    cudaErrorMemoryAllocation without calling the driver) goes back to the head of the
    queue once and runs again when no other batch is on the device, with the same bits as
    without the failure; when the re-run fails too, the request fails with the error."""
    a, _, _ = _surfaces()
    req = (a, bemgpu.Rigid(), [300.0, 420.0], [0.3, 1.1])
    srv = bemgpu.Server(ctx, max_batch=8)
    try:
        ref = srv.wait(srv.submit(*req, precision="mixed"))[0]   # the mesh is resident now
    finally:
        srv.close()
    for failures in (1, 2):
        srv = bemgpu.Server(ctx, max_batch=8)
        try:
            ctx.inject_alloc_failures(failures)
            t = srv.submit(*req, precision="mixed")
            if failures == 1:
                got = srv.wait(t)[0]
            else:
                with pytest.raises(bemgpu.BEMGPUError, match="out of memory"):
                    srv.wait(t)
            st = srv.stats()
        finally:
            ctx.inject_alloc_failures(0)
            srv.close()
        assert st["retries"] == 2, st          # both frequencies of the batch, once
        if failures == 1:
            assert np.array_equal(got, ref) and st["completed"] == 1 and st["failed"] == 0
        else:
            assert st["completed"] == 0 and st["failed"] == 1
    with pytest.raises(bemgpu.ArgumentError):
        ctx.inject_alloc_failures(-1)


def test_cached_factors_are_reused(ctx):
    a, _, _ = _surfaces()
    req = (a, bemgpu.Rigid(), [300.0, 420.0], [0.3, 1.1])
    srv = bemgpu.Server(ctx, max_batch=8)
    try:
        first = srv.wait(srv.submit(*req, precision="mixed"))[0]
        again = srv.wait(srv.submit(*req, precision="mixed"))[0]
        st = srv.stats()
    finally:
        srv.close()
    assert st["cache_hits"] == 2 and st["factorizations"] == 2, st
    assert np.array_equal(first, again)


def test_server_matches_direct_solve(ctx):
    a, _, _ = _surfaces()
    srv = bemgpu.Server(ctx)
    try:
        angles = [0.3, 1.2]
        t = srv.submit(a, bemgpu.Rigid(), [350.0], angles)
        got, _ = srv.wait(t)
    finally:
        srv.close()
    for r, ang in enumerate(angles):
        sol = bemgpu.bem(a, bemgpu.Rigid(), 350.0, incidence_angle=ang, ctx=ctx)
        want = bemgpu.scattering_amplitude(sol)
        assert abs(got[0, r] - want) <= 1e-12 * abs(want)


def test_server_many_requests_complete(ctx):
    a, b, c = _surfaces()
    srv = bemgpu.Server(ctx, max_batch=4, cache_bytes=1 << 20)
    rng = np.random.default_rng(3)
    try:
        tickets = []
        for i in range(12):
            s = (a, b, c)[i % 3]
            bc = bemgpu.Rigid() if i % 2 else bemgpu.PressureRelease()
            ks = rng.uniform(200, 600, size=1 + i % 3)
            tickets.append(srv.submit(s, bc, ks, rng.uniform(0, math.pi, size=1 + i % 2),
                                      precision="mixed"))
        for tk in tickets:
            out, lat = srv.wait(tk, timeout_ms=120000)
            assert np.all(np.isfinite(out)) and lat > 0
        st = srv.stats()
        assert st["completed"] == 12 and st["batches"] >= 2
    finally:
        srv.close()


def test_small_request_overtakes_a_large_one(ctx):
    """Two lanes: a small request submitted just after a large one is taken by the free
    lane, completes first, and gives the same bits as when it runs alone."""
    import time

    small = (bemgpu.mesh(*meshes.icosphere(0.01, 2)), bemgpu.Rigid(), [320.0], [0.4, 1.3])
    big_mesh = bemgpu.mesh(*meshes.uv_spheroid(0.05, 0.0125, 96, 40))   # 7680 panels
    big = (big_mesh, bemgpu.Rigid(), [200.0, 230.0, 260.0, 290.0], [0.2])
    srv = bemgpu.Server(ctx, lanes=2)
    try:
        alone = srv.wait(srv.submit(*small, precision="mixed"))[0]
    finally:
        srv.close()
    srv = bemgpu.Server(ctx, lanes=2)
    try:
        t0 = time.perf_counter()
        tb = srv.submit(*big, precision="mixed")
        tb_sub = time.perf_counter() - t0
        ts = srv.submit(*small, precision="mixed")
        ts_sub = time.perf_counter() - t0
        out_s, lat_s = srv.wait(ts)
        out_b, lat_b = srv.wait(tb)
        st = srv.stats()
    finally:
        srv.close()
    done_small = ts_sub * 1e3 + lat_s
    done_big = tb_sub * 1e3 + lat_b
    assert done_small < done_big, (done_small, done_big)
    assert np.array_equal(out_s, alone)
    assert np.all(np.isfinite(out_b))
    assert st["batches"] >= 2 and st["cache_hits"] == 0, st
