"""Host logic of bench.py that needs no GPU: the served-stream driver reports failed
requests in its line (and counts only completed ones) instead of aborting a long run, the
nvidia-smi sampler's clock, throttle-reason and memory parsing, the memory grouping of the
uneven batch, and the seeded request stream (a shorter run serves a prefix of a longer)."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


class _FakeServer:
    """Stands in for bemgpu.Server: request 3 fails the way an out-of-memory batch
    reported itself before the server re-ran such batches."""
    precision = "mixed"

    def __init__(self):
        self.n = 0

    def submit(self, surface, boundary, ks, angles, precision):
        self.n += 1
        return self.n - 1

    def wait(self, ticket, timeout_ms=-1):
        if ticket == 3:
            raise RuntimeError("CUDA error: request failed: cudaMalloc: out of memory")
        return np.full((1, 2), 1.0 + 0.5j), 10.0 * (ticket + 1)

    def stats(self):
        return {"completed": 4, "failed": 1}

    def close(self):
        pass


def test_served_stream_reports_failed_requests():
    bodies = [{"boundary": "rigid"}]
    reqs = [(0, np.array([100.0]), np.array([0.1, 0.2]))] * 5
    res, out = bench._serve(_FakeServer, [None], bodies, reqs, list(range(5)), 1e6, 7)
    assert res["failed_requests"] == 1 and "out of memory" in res["first_error"]
    assert sorted(out) == [0, 1, 2, 4]
    assert res["solves"] == 4 * 2 and res["requests"] == 5
    lats = [10.0, 20.0, 30.0, 50.0]
    assert res["p50_ms"] == np.percentile(lats, 50) and res["max_ms"] == 50.0


def test_clock_sampler_parses_reasons_and_memory():
    c = bench.Clocks(0)
    c.rows = [["0", "2070", "2070", "900.1", "0x0", "Not Active", "Not Active", "Not Active",
               "Active", "150000", "284208"],
              ["0", "1995", "2070", "1380.0", "0x4", "Not Active", "Not Active", "Not Active",
               "Active", "281487", "284208"],
              ["0", "[N/A]", "2070"]]
    out = c.stop()
    assert out["sm_max_mhz"] == 2070.0 and out["samples"] == 2
    assert out["sm_mhz"] == np.median([2070.0, 1995.0])
    assert out["reasons"] == ["sw_power_cap"]
    assert out["memory_used_mib_max"] == 281487.0 and out["memory_total_mib"] == 284208.0


def test_memory_groups_cover_every_instance_within_the_budget():
    sizes = [500, 12000, 800, 7000, 7000, 3000, 11000, 600]
    per = 24.0
    budget = 12000 ** 2 * per * 1.5
    groups = bench._memory_groups(sizes, budget, per)
    assert [i for g in groups for i in g] == list(range(len(sizes)))   # in order, once each
    for g in groups:
        assert len(g) == 1 or sum(sizes[i] ** 2 * per for i in g) <= budget


def test_request_stream_is_seeded_and_prefix_stable():
    """The served stream's first requests are the same whatever its length, so a shorter
    run measures a prefix of the longer one."""
    b1, r1 = bench._request_stream(20, 16)
    b2, r2 = bench._request_stream(50, 16)
    assert b1 == b2
    for (i1, k1, a1), (i2, k2, a2) in zip(r1, r2[:20]):
        assert i1 == i2 and np.array_equal(k1, k2) and np.array_equal(a1, a2)
    assert all(1 <= len(k) <= 32 and 1 <= len(a) <= 64 for _, k, a in r2)


def test_lu_update_flops_account_for_the_factorisation():
    """The roofline's algorithmic flops (the LU's tensor-core updates, 8 real flops per
    complex multiply-add) are most of a complex LU's 8/3 N^3, short of it by the panel
    and triangular-block work, which grows with the block width."""
    N = 10240
    f256 = bench.lu_update_flops(N, 256)
    f128 = bench.lu_update_flops(N, 128)
    total = 8.0 / 3.0 * N ** 3
    assert 0.95 < f256 / total < 1.0 and 0.95 < f128 / total < 1.0
    assert f128 > f256          # narrower steps leave less outside the updates
    # one K = 256 trailing update of an m x m block: 8 m^2 K flops, C read and written
    # once (16 B per complex64 entry) and the two operand images read once
    assert bench._upd(5504, 5504, 256) == (8.0 * 5504 ** 2 * 256,
                                           16.0 * 5504 ** 2 + 8.0 * 256 * 2 * 5504)
