#!/usr/bin/env python3
"""Headline benchmark: BEM solves/s (mixed vs FP64) on one GB300 at <= 0.01 dB TS error.

Workload (batched frequency sweep): fluid-filled prolate spheroid, semi-axes 0.02 m
(x, symmetry axis) and 0.01 m, UV mesh of 64 longitudes x 40 rings = 5120 flat
triangles with seeded vertex jitter of +-2 % of the mean edge, density contrast
g = 1.0357, sound-speed contrast h = 1.0279, exterior 1500 m/s, 64 frequencies evenly
spaced over 12-120 kHz, plane wave at the reference's default incidence (polar pi/2,
azimuth 0), backscatter.  Mueller formulation, 2n = 10240 complex unknowns per
frequency.  One step = all 64 frequencies assembled, factored and solved as one batch
(one solve = one (geometry, frequency, incidence) carried to a TS value).

value: mixed precision (FP32 regular-pair quadrature, complex64 LU, FP64 refinement of
the FP64-residual system), mesh resident on the device.  e2e: the same through the
host API with host buffers (mesh validated, hashed and uploaded every step, amplitudes
copied back).  FP64 (complex128 everywhere) is measured on a subset of the frequencies
and reported beside it, together with the max |TS_mixed - TS_fp64| over that subset.

--impl reference: the CPU restatement of the reference's path (oracle/, C assembly +
LAPACK LU + the reference's mixed refinement) on the host cores, one frequency per step.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "acousticscattering.jl_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "BEM solves/s & p99 latency, mixed vs FP64 on 1 GB300 at ≤0.01 dB TS error"
SEED = 20261203
W = dict(a=0.02, b=0.01, nlon=64, nrings=40, jitter=0.02, g=1.0357, h=1.0279, c=1500.0,
         f0=12e3, f1=120e3, nfreq=64, beta=math.pi / 2, alpha=0.0)


def workload_mesh(nlon, nrings):
    from bemgpu import meshes
    return meshes.uv_spheroid(W["a"], W["b"], nlon, nrings, jitter=W["jitter"], seed=SEED)


def wavenumbers(nfreq):
    f = np.linspace(W["f0"], W["f1"], nfreq)
    return f, 2 * math.pi * f / W["c"]


# ------------------------------------------------------------------ clocks
class Clocks:
    """nvidia-smi sampling during the timed region (every 200 ms)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.thread:
            self.thread.join(timeout=5)
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                mx = max(mx, float(r[2]))
            except ValueError:
                continue
            for name, v in zip(names, r[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": mx or None, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as fh:
            d = json.load(fh)
        return d.get("hbm_gbs", 6800.0), d.get("bf16_tflops", 1900.0), "measured"
    return 6800.0, 1900.0, "fallback"


def _upd(m, n, k):
    """C (m x n complex64) -= A (m x k) B (k x n): real flops (8 per complex MAC) and
    bytes (C read and written, packed split-bf16 images of A and B read, 8 B per complex)."""
    if m <= 0 or n <= 0 or k <= 0:
        return 0.0, 0.0
    return 8.0 * m * n * k, 16.0 * m * n + 8.0 * k * (m + n)


def lu_update_work(N, nb):
    """Algorithmic flops and bytes of the updates timed as the LU's tensor-core GEMM
    family: with 128-column halves of 256-column steps (nb = 256), the left half's
    update of the right half (K = 128) and the trailing update (K = 256); with nb = 128
    the trailing update of every 128-column step."""
    flops = byts = 0.0
    half = nb // 2 if nb == 256 else nb
    for k0 in range(0, N, nb):
        if nb == 256:
            kk1 = max(0, min(half, N - k0 - half))
            f, b = _upd(N - k0 - half, kk1, min(half, N - k0))
            flops, byts = flops + f, byts + b
        m = N - k0 - min(nb, N - k0)
        f, b = _upd(m, m, min(nb, N - k0))
        flops, byts = flops + f, byts + b
    return flops, byts


def lu_update_flops(N, nb):
    return lu_update_work(N, nb)[0]


# DRAM traffic of one k_tc_cgemm launch over its algorithmic bytes, from one ncu capture
# (--set full) of `bench.py --freqs 2 --nlon 48 --nrings 30`: 4th launch = trailing
# update of outer step 1 of 2 x 5760 unknowns (m = n = 5504, k = 128),
# dram__bytes_read.sum + dram__bytes_write.sum = 507.54 + 423.62 MB.
NCU_GEMM_TRAFFIC = (507.543808e6 + 423.618560e6) / (2 * (16.0 * 5504 ** 2 + 8.0 * 128 * 2 * 5504))


def aggregate_replicas(ms, units, world):
    """Replicas only: every rank solves its own copy of the workload; the step time is
    the max over ranks and the throughput counts the units of all ranks."""
    if world > 1:
        import torch.distributed as dist
        if not dist.is_initialized():
            dist.init_process_group("gloo")
        out = [None] * world
        dist.all_gather_object(out, float(ms))
        ms = max(out)
    return ms, world * units / (ms * 1e-3)


# ------------------------------------------------------------------ our arm
def run_ours(args):
    import bemgpu
    from bemgpu import FluidFilled

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    ctx = bemgpu.Context(local)
    nodes, tris = workload_mesh(args.nlon, args.nrings)
    surf = bemgpu.mesh(nodes, tris)
    surf.handle(ctx)
    freqs, ks = wavenumbers(args.freqs)
    fl = FluidFilled(W["g"], W["h"])
    n = surf.n_panels
    N = 2 * n

    def step(surface, precision, kk):
        items = [(surface, fl, float(k), dict(precision=precision)) for k in kk]
        fs = bemgpu.factor_batch(items, ctx)
        sols = bemgpu.solve_batch(fs, [[W["beta"]]] * len(fs), [[W["alpha"]]] * len(fs))
        amps = np.array([bemgpu.scattering_amplitude(s) for s in sols])
        diags = [s.diagnostics() for s in sols]
        for s in sols:
            s.close()
        for f in fs:
            f.close()
        return amps, diags

    # ---- warm-up
    for _ in range(args.warmup):
        step(surf, "mixed", ks)
    # ---- timed region: device events on the library stream, clocks sampled
    clocks = Clocks(local)
    clocks.start()
    ctx.profile(True)
    ctx.profile_reset()
    l0 = bemgpu.Context.launch_count()
    times = []
    amps_mixed = diags_mixed = None
    for _ in range(args.steps):
        ctx.timer_start()
        amps_mixed, diags_mixed = step(surf, "mixed", ks)
        times.append(ctx.timer_stop())
    launches = bemgpu.Context.launch_count() - l0
    prof = {fam: ctx.profile_read(fam) for fam in
            ("assemble", "near", "equilibrate", "scale_copy", "getf2", "laswp", "trsm",
             "gemm_panel", "gemm_c64", "tc_pack", "gemm_tc", "gecon", "incident", "forcing",
             "getrs", "residual")}
    ctx.profile(False)
    clk = clocks.stop()
    ms = float(np.mean(times))
    # ---- e2e: host buffers through the public API
    e2e_times = []
    h2d = nodes.nbytes + tris.nbytes
    for _ in range(max(1, min(args.steps, 3))):
        t0 = time.perf_counter()
        s2 = bemgpu.mesh(nodes, tris)
        a2, _ = step(s2, "mixed", ks)
        s2.release()
        e2e_times.append((time.perf_counter() - t0) * 1e3)
    e2e_ms = float(np.mean(e2e_times))
    # ---- FP64 on a subset + TS error of the mixed results against it
    sub = np.unique(np.linspace(0, args.freqs - 1, max(1, args.fp64_freqs)).round().astype(int))
    ctx.timer_start()
    amps64, diags64 = step(surf, "double", ks[sub])
    fp64_ms = ctx.timer_stop()
    ts_err = np.abs(20 * np.log10(np.abs(amps_mixed[sub])) - 20 * np.log10(np.abs(amps64)))
    # ---- roofline of the dominant kernel (trailing complex update of the LU)
    hbm, bf16, which = measured_peaks()
    fam = "gemm_tc" if prof["gemm_tc"][0] else "gemm_c64"
    nb = 256 if fam == "gemm_tc" else 32
    flops_one, bytes_one = lu_update_work(N, nb)
    flops_step, bytes_step = args.freqs * flops_one, args.freqs * bytes_one
    gl, gms = prof[fam]
    secs = gms * 1e-3 / args.steps if gms else 0.0
    achieved_gbs = bytes_step / secs / 1e9 if secs else 0.0
    achieved_tf = flops_step / secs / 1e12 if secs else 0.0
    launches_step = max(1, gl // args.steps)
    ms, value = aggregate_replicas(ms, args.freqs, world)
    if rank != 0:
        return None
    cpu = None if args.no_cpu else cpu_baseline(ks, args)
    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c64 factor (fp32 regular quadrature) + fp64 refinement",
        "data": "synthetic (seeded UV spheroid mesh, 64 frequencies)",
        "config": {"workload": "fluid prolate spheroid 0.02x0.01 m, 5120 panels, 64 freqs "
                               "12-120 kHz, g=1.0357 h=1.0279, Mueller",
                   "panels": n, "unknowns": N, "frequencies": args.freqs,
                   "precision": "mixed", "l2": "inputs larger than L2 (per-step matrices "
                   f"{args.freqs * N * N * 24 / 1e9:.0f} GB)", "seed": SEED},
        "latency_ms": {"p50": float(np.percentile(times, 50)),
                       "p99": float(np.percentile(times, 99)),
                       "per": "batch of 64 frequencies"},
        "fp64": {"solves_per_s": len(sub) / (fp64_ms * 1e-3), "frequencies": len(sub),
                 "ms": fp64_ms, "ts_error_db_max": float(np.max(ts_err)),
                 "ratio_mixed_over_fp64": value / (len(sub) / (fp64_ms * 1e-3))},
        "refinement": {"iterations_max": max(d["refinement_iterations"] for d in diags_mixed),
                       "normwise_backward_error_max": max(d["normwise_backward_error"]
                                                          for d in diags_mixed),
                       "factor_precision": sorted({d["factor_precision"] for d in diags_mixed})},
        "e2e": {"value": args.freqs / (e2e_ms * 1e-3), "unit": "solves/s",
                "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(16 * args.freqs)},
        # K = 256 complex update: 8 x 256 flops per 16 bytes of C = 128 flop/byte, above
        # the ridge of the split-bf16 tensor path (measured bf16 / 3 bf16 MMAs per real
        # product over measured HBM = 93 flop/byte), so the tensor pipe bounds it
        "roofline": {"bound": "tensor", "kernel": "k_tc_cgemm (LU tensor-core updates)",
                     "achieved": achieved_tf, "peak": bf16, "unit": "TFLOP/s",
                     "frac": achieved_tf / bf16 if bf16 else None,
                     "peak_source": f"{which} bf16 dense",
                     "traffic": NCU_GEMM_TRAFFIC * bytes_step / launches_step,
                     "algorithmic_bytes_per_launch": bytes_step / launches_step,
                     "traffic_note": "ncu dram bytes of a smaller capture, scaled by C size",
                     "launches": gl, "kernel_ms_per_step": gms / args.steps,
                     "split_bf16_view": {"executed_tflops": 3.0 * achieved_tf,
                                         "frac": 3.0 * achieved_tf / bf16 if bf16 else None,
                                         "note": "3 bf16 MMAs per real product (hi*hi, "
                                                 "hi*lo, lo*hi): executed = 3 x algorithmic"},
                     "hbm_view": {"achieved_gbs": achieved_gbs, "peak_gbs": hbm,
                                  "frac": achieved_gbs / hbm if hbm else None}},
        "phase_ms_per_step": {k: v[1] / args.steps for k, v in prof.items() if v[0]},
        "gpu_launches": int(launches // max(1, args.steps)),
        "clocks": clk,
        "cpu_baseline": cpu,
    }
    print(json.dumps(line))
    return line


# ------------------------------------------------------------------ CPU baseline
def _oracle_one(k, nodes, tris, precision):
    from oracle import oracle as O
    t0 = time.perf_counter()
    r = O.solve(nodes, tris, "fluid", float(k), incidence_angle=W["beta"],
                incidence_azimuth=W["alpha"], g=W["g"], h=W["h"], precision=precision)
    return time.perf_counter() - t0, r["amplitudes"][0]


def cpu_baseline(ks, args):
    """The oracle (CPU restatement of the reference's path) on all host cores, one
    frequency (the middle one) of the same workload: a bounded sample."""
    nodes, tris = workload_mesh(args.nlon, args.nrings)
    k = ks[len(ks) // 2]
    dt, _ = _oracle_one(k, nodes, tris, "mixed")
    return {"value": 1.0 / dt, "unit": "solves/s", "cores": os.cpu_count(), "kind": "port",
            "sample": f"1 of {len(ks)} frequencies (k={k:.2f}/m), mixed precision, "
                      f"oracle C assembly (OpenMP) + LAPACK cgetrf/zgetrf, {dt:.1f} s"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return None
    nodes, tris = workload_mesh(args.nlon, args.nrings)
    freqs, ks = wavenumbers(args.freqs)
    for w in range(args.warmup):
        _oracle_one(ks[w % len(ks)], nodes, tris, "mixed")
    times = []
    for s in range(args.steps):
        dt, _ = _oracle_one(ks[(args.warmup + s) % len(ks)], nodes, tris, "mixed")
        times.append(dt)
    ms = float(np.mean(times)) * 1e3
    v = 1.0 / (ms * 1e-3)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "solves/s",
            "n_gpus": int(os.environ.get("WORLD_SIZE", "1")), "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c64 factor + fp64 refinement",
            "data": "synthetic (seeded UV spheroid mesh)",
            "config": {"workload": "fluid prolate spheroid 0.02x0.01 m, 5120 panels, 64 freqs "
                                   "12-120 kHz, g=1.0357 h=1.0279, Mueller",
                       "panels": tris.shape[1], "unknowns": 2 * tris.shape[1],
                       "frequencies": args.freqs, "precision": "mixed", "seed": SEED},
            "cpu_baseline": {"value": v, "unit": "solves/s", "cores": os.cpu_count(),
                             "kind": "port",
                             "sample": "one frequency per step (the reference's Julia code "
                                       "cannot run here; CPU restatement in oracle/)"},
            "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return line


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--freqs", type=int, default=W["nfreq"])
    ap.add_argument("--fp64-freqs", type=int, default=2)
    ap.add_argument("--nlon", type=int, default=W["nlon"])
    ap.add_argument("--nrings", type=int, default=W["nrings"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
