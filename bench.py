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
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap,"
         "memory.used,memory.total")

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
        sm, mx, reasons, mem = [], 0.0, set(), []
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
            try:
                mem.append((float(r[9]), float(r[10])))
            except (IndexError, ValueError):
                pass
        out = {"sm_mhz": float(np.median(sm)) if sm else None,
               "sm_max_mhz": mx or None, "reasons": sorted(reasons),
               "samples": len(sm)}
        if mem:  # device memory in use (all processes) during the region, MiB
            out["memory_used_mib_max"] = max(u for u, _ in mem)
            out["memory_total_mib"] = mem[0][1]
        return out


def measured_peaks(sustained=False):
    """(HBM GB/s, bf16 TFLOP/s, source).  sustained=True gives the bf16 rate of a
    seconds-long GEMM loop under the power cap, the right peak for a kernel timed inside
    a long step; otherwise the burst rate of a kernel timed alone."""
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as fh:
            d = json.load(fh)
        if sustained and "bf16_tflops_sustained" in d:
            return d.get("hbm_gbs", 6800.0), d["bf16_tflops_sustained"], "measured (sustained)"
        return d.get("hbm_gbs", 6800.0), d.get("bf16_tflops", 1900.0), "measured"
    return 6800.0, (1700.0 if sustained else 1900.0), "fallback"


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
# (--set full) of `bench.py --freqs 8 --nlon 48 --nrings 30`: 6th launch = K = 256
# trailing update of the first step of 8 x 5760 unknowns (m = n = 5504),
# dram__bytes_read.sum + dram__bytes_write.sum = 2.119512 + 1.876776 GB.
NCU_GEMM_TRAFFIC = (2.119512e9 + 1.876776e9) / (8 * (16.0 * 5504 ** 2 + 8.0 * 256 * 2 * 5504))


def headline_config(n_panels, freqs):
    """The workload description shared by both arms (identical dicts)."""
    N = 2 * n_panels
    return {"workload": "fluid prolate spheroid 0.02x0.01 m, 5120 panels, 64 freqs "
                        "12-120 kHz, g=1.0357 h=1.0279, Mueller",
            "panels": n_panels, "unknowns": N, "frequencies": freqs, "precision": "mixed",
            "l2": "inputs larger than L2 (per-step matrices "
                  f"{freqs * N * N * 24 / 1e9:.0f} GB)", "seed": SEED}


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
             "getrs", "residual", "far_field")}
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
    # ---- roofline of the dominant kernel (trailing complex update of the LU), timed
    # inside a seconds-long step: against the sustained bf16 rate
    hbm, bf16, which = measured_peaks(sustained=True)
    fam = "gemm_tc" if prof["gemm_tc"][0] else "gemm_c64"
    nb = 256 if fam == "gemm_tc" else 32
    flops_one, bytes_one = lu_update_work(N, nb)
    flops_step, bytes_step = args.freqs * flops_one, args.freqs * bytes_one
    gl, gms = prof[fam]
    secs = gms * 1e-3 / args.steps if gms else 0.0
    achieved_gbs = bytes_step / secs / 1e9 if secs else 0.0
    achieved_tf = flops_step / secs / 1e12 if secs else 0.0
    launches_step = max(1, gl // args.steps)
    asm_bytes = args.freqs * 4.0 * n * n * 8.0
    ff_bytes = args.freqs * n * (7 * 7 * 8.0 + 8.0 + 2 * 16.0)
    ms, value = aggregate_replicas(ms, args.freqs, world)
    if rank != 0:
        return None
    cpu = oracle_err = None
    if not args.no_cpu:
        cpu, oracle_err = cpu_baseline(ks, args)
        # the GPU's own results at the oracle's frequency (the FP64 subset holds it)
        j = len(ks) // 2
        a_or, a_or_mixed = oracle_err.pop("_fp64"), oracle_err.pop("_mixed")
        oracle_err["mixed_ts_error_db"] = float(abs(20 * np.log10(abs(amps_mixed[j]))
                                                    - 20 * np.log10(abs(a_or))))
        oracle_err["mixed_amplitude_rel_error"] = float(abs(amps_mixed[j] - a_or) / abs(a_or))
        if j in set(sub.tolist()):
            a64 = amps64[list(sub).index(j)]
            oracle_err["fp64_amplitude_rel_error"] = float(abs(a64 - a_or) / abs(a_or))
        oracle_err["oracle_mixed_ts_error_db"] = float(abs(20 * np.log10(abs(a_or_mixed))
                                                           - 20 * np.log10(abs(a_or))))
    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c64 factor (fp32 regular quadrature) + fp64 refinement",
        "data": "synthetic (seeded UV spheroid mesh, 64 frequencies)",
        "config": headline_config(n, args.freqs),
        "latency_ms": {"p50": float(np.percentile(times, 50)),
                       "p99": float(np.percentile(times, 99)),
                       "per": "batch of 64 frequencies"},
        "fp64": {"solves_per_s": len(sub) / (fp64_ms * 1e-3), "frequencies": len(sub),
                 "ms": fp64_ms, "ts_error_db_max": float(np.max(ts_err)),
                 "ratio_mixed_over_fp64": value / (len(sub) / (fp64_ms * 1e-3))},
        "fp64_oracle_error": oracle_err,
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
                     "burst_frac": achieved_tf / measured_peaks()[1],
                     "traffic": NCU_GEMM_TRAFFIC * bytes_step / launches_step,
                     "algorithmic_bytes_per_launch_avg": bytes_step / launches_step,
                     "per_launch": "average over the step's launches of the family (the "
                                   "step's sum / its launch count), for achieved and traffic",
                     "traffic_note": "ncu dram bytes of a smaller capture, scaled by C size",
                     "launches": gl, "kernel_ms_per_step": gms / args.steps,
                     "split_bf16_view": {"executed_tflops": 3.0 * achieved_tf,
                                         "frac": 3.0 * achieved_tf / bf16 if bf16 else None,
                                         "note": "3 bf16 MMAs per real product (hi*hi, "
                                                 "hi*lo, lo*hi): executed = 3 x algorithmic"},
                     "hbm_view": {"achieved_gbs": achieved_gbs, "peak_gbs": hbm,
                                  "frac": achieved_gbs / hbm if hbm else None}},
        # assembly and far field: achieved HBM bandwidth of their algorithmic bytes (both
        # are FP32/SFU (assembly) or FP64 (far field) issue-bound, not bandwidth-bound)
        "assembly_hbm": {
            "bytes_per_step": asm_bytes,
            "achieved_gbs": asm_bytes / (prof["assemble"][1] * 1e-3 / args.steps) / 1e9
            if prof["assemble"][1] else None,
            "peak_gbs": hbm,
            "note": "complex64 entries written (4 blocks of n^2) / regular-assembly time"},
        "far_field_hbm": {
            "bytes_per_step": ff_bytes,
            "achieved_gbs": ff_bytes / (prof["far_field"][1] * 1e-3 / args.steps) / 1e9
            if prof["far_field"][1] else None,
            "peak_gbs": hbm,
            "note": "panel records (7 nodes x 7 doubles + area) and 2 complex traces per "
                    "panel per direction"},
        "phase_ms_per_step": {k: v[1] / args.steps for k, v in prof.items() if v[0]},
        "phase_note": "event time per family on the main stream; the triangular solves' "
                      "side-stream look-ahead overlaps other phases, so the sum exceeds "
                      "ms_per_step",
        "gpu_launches": int(launches // max(1, args.steps)),
        "clocks": clk,
        "cpu_baseline": cpu,
    }
    print(json.dumps(line))
    return line


# ------------------------------------------------------------------ other workloads
# The remaining named workloads, selected with --config; each prints its own JSON line
# (the default line above is the headline workload).
def _base_line(metric, value, unit, ms, args, config, **kw):
    line = {"metric": metric, "value": value, "unit": unit, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "data": "synthetic", "config": config}
    line.update(kw)
    return line


def run_config0(args):
    """Rigid sphere a = 0.01 m, icosphere 1280 panels, c = 1477.4 m/s, f = 38 kHz, plane
    wave along +z (polar pi/2, azimuth pi/2), Burton-Miller alpha = i/k: one solve per step
    (assembly + factor + solve + backscatter), mixed and FP64."""
    import bemgpu
    from bemgpu import meshes
    ctx = bemgpu.Context(0)
    nodes, tris = meshes.icosphere(0.01, 3)
    surf = bemgpu.mesh(nodes, tris)
    k = 2 * math.pi * 38e3 / 1477.4
    beta, alpha = math.pi / 2, math.pi / 2

    def one(precision):
        sol = bemgpu.bem(surf, bemgpu.Rigid(), k, incidence_angle=beta, incidence_azimuth=alpha,
                         precision=precision, ctx=ctx)
        f = bemgpu.scattering_amplitude(sol)
        sol.close()
        return f

    steps = max(args.steps, 20)
    out = {}
    for prec in ("mixed", "double"):
        for _ in range(max(args.warmup, 3)):
            one(prec)
        clocks = Clocks(0)
        clocks.start()
        l0 = bemgpu.Context.launch_count()
        ts = []
        for _ in range(steps):
            ctx.timer_start()
            f = one(prec)
            ts.append(ctx.timer_stop())
        out[prec] = (f, float(np.mean(ts)), float(np.percentile(ts, 50)),
                     float(np.percentile(ts, 99)), clocks.stop(),
                     (bemgpu.Context.launch_count() - l0) // steps)
    fm, fd = out["mixed"][0], out["double"][0]
    ms = out["mixed"][1]
    # the same body in the Nystrom discretisation (7 quadrature-node unknowns per panel,
    # density-interpolation correction): one solve per step, outside the headline timing
    ny = {"unknowns": 7 * tris.shape[1]}
    for prec, reps in (("mixed", 5), ("double", 1)):
        def one_ny():
            sol = bemgpu.bem(surf, bemgpu.Rigid(), k, incidence_angle=beta,
                             incidence_azimuth=alpha, precision=prec, ctx=ctx,
                             discretization="nystrom")
            f = bemgpu.scattering_amplitude(sol)
            d = sol.diagnostics()
            sol.close()
            return f, d
        one_ny()
        ts = []
        for _ in range(reps):
            ctx.timer_start()
            f, d = one_ny()
            ts.append(ctx.timer_stop())
        ny[prec] = {"solves_per_s": 1e3 / float(np.mean(ts)), "ms": float(np.mean(ts)),
                    "assemble_ms": d["assemble_ms"], "factor_ms": d["factor_ms"],
                    "solve_ms": d["solve_ms"], "ts_db": 20 * math.log10(abs(f))}
    ny["ts_db_minus_collocation_fp64"] = ny["double"]["ts_db"] - 20 * math.log10(abs(fd))
    cpu = None
    if not args.no_cpu:
        from oracle import oracle as O
        t0 = time.perf_counter()
        O.solve(nodes, tris, "rigid", k, incidence_angle=beta, incidence_azimuth=alpha)
        dt = time.perf_counter() - t0
        cpu = {"value": 1.0 / dt, "unit": "solves/s", "cores": os.cpu_count(), "kind": "port",
               "sample": f"one FP64 solve of the same sphere by the oracle, {dt:.2f} s"}
    line = _base_line(
        "BEM solves/s, rigid sphere 1280 panels (plain FP64 case)", 1e3 / ms, "solves/s", ms,
        args, {"workload": "rigid sphere a=0.01 m, icosphere 1280 panels, f=38 kHz, "
                           "c=1477.4 m/s, +z incidence, Burton-Miller", "panels": 1280},
        steps=steps, dtype="c64 factor + fp64 refinement",
        latency_ms={"p50": out["mixed"][2], "p99": out["mixed"][3]},
        fp64={"solves_per_s": 1e3 / out["double"][1], "p50_ms": out["double"][2],
              "p99_ms": out["double"][3], "ts_db": 20 * math.log10(abs(fd))},
        ts_db=20 * math.log10(abs(fm)),
        ts_error_db_vs_fp64=abs(20 * math.log10(abs(fm)) - 20 * math.log10(abs(fd))),
        amplitude_rel_error_vs_fp64=abs(fm - fd) / abs(fd), nystrom=ny,
        clocks=out["mixed"][4], gpu_launches=out["mixed"][5], cpu_baseline=cpu)
    print(json.dumps(line))
    return line


def run_config2(args):
    """Rigid prolate spheroid 0.05 x 0.0125 m, 128 x 80 UV mesh (20480 panels), f = 60 kHz,
    c = 1500 m/s: one factor, 181 incidence angles 0..180 deg (monostatic backscatter),
    refined to a relative backward error of 1e-10; FP64 on the same factor path for the
    per-angle error."""
    import bemgpu
    from bemgpu import meshes
    ctx = bemgpu.Context(0)
    nodes, tris = meshes.uv_spheroid(0.05, 0.0125, 128, 80)
    surf = bemgpu.mesh(nodes, tris)
    k = 2 * math.pi * 60e3 / 1500.0
    angles = np.linspace(0.0, math.pi, 181)

    def sweep(precision, **kw):
        return bemgpu.incidence_angle_sweep(surf, bemgpu.Rigid(), k, angles,
                                            precision=precision, ctx=ctx, **kw)

    ref = dict(refinement=dict(tolerance=1e-10))
    for _ in range(max(1, args.warmup)):
        sweep("mixed", **ref)
    clocks = Clocks(0)
    clocks.start()
    ctx.profile(True)
    ctx.profile_reset()
    l0 = bemgpu.Context.launch_count()
    ts = []
    for _ in range(args.steps):
        ctx.timer_start()
        sw = sweep("mixed", **ref)
        ts.append(ctx.timer_stop())
    launches = (bemgpu.Context.launch_count() - l0) // args.steps
    prof = {fam: ctx.profile_read(fam)[1] / args.steps for fam in
            ("assemble", "near", "getf2", "gemm_tc", "trsm", "gecon", "getrs", "residual",
             "forcing", "far_field")}
    ctx.profile(False)
    clk = clocks.stop()
    ctx.timer_start()
    sw64 = sweep("double")
    fp64_ms = ctx.timer_stop()
    err = np.abs(sw.target_strength - sw64.target_strength)
    ms = float(np.mean(ts))
    line = _base_line(
        "BEM solves/s, rigid spheroid 20480 panels x 181 angles (precision study)",
        181 * 1e3 / ms, "solves/s", ms, args,
        {"workload": "rigid prolate spheroid 0.05x0.0125 m, 20480 panels, f=60 kHz, "
                     "181 incidence angles, refinement tolerance 1e-10", "panels": 20480,
         "angles": 181},
        dtype="c64 factor + fp64 refinement", phase_ms_per_step=prof,
        fp64={"solves_per_s": 181 * 1e3 / fp64_ms, "ms": fp64_ms},
        ts_error_db={"max": float(err.max()), "median": float(np.median(err))},
        diagnostics={k2: (v if isinstance(v, (int, float, str)) else str(v))
                     for k2, v in sw.diagnostics.items()},
        target_strength_db=[round(float(v), 4) for v in sw.target_strength],
        fp64_error_db_per_angle=[float(v) for v in err],
        clocks=clk, gpu_launches=launches)
    print(json.dumps(line))
    return line


def _uneven_batch(master, count, panel_range):
    from bemgpu import meshes
    bodies = []
    for i in range(count):
        b = meshes.random_body(master, i, panel_range)
        nodes, tris = meshes.body_of_revolution(b["b"], b["aspect"], b["coeffs"], b["nlon"],
                                                b["nrings"])
        bodies.append((b, nodes, tris))
    return bodies


def _memory_groups(sizes, budget_bytes, per_unknown2):
    """Consecutive groups whose summed n^2 * per_unknown2 stays within the budget."""
    groups, cur, acc = [], [], 0.0
    for i, n in enumerate(sizes):
        b = n * n * per_unknown2
        if cur and acc + b > budget_bytes:
            groups.append(cur)
            cur, acc = [], 0.0
        cur.append(i)
        acc += b
    if cur:
        groups.append(cur)
    return groups


def run_config3(args):
    """256 seeded bodies of revolution (panels log-uniform 500..12000, f ~ U(10, 200) kHz,
    incidence uniform on the sphere, rigid / pressure release 50/50, Burton-Miller),
    assembled, factored and solved as uneven batches (grouped to a device-memory budget)."""
    import bemgpu
    ctx = bemgpu.Context(0)
    count = args.bodies
    bodies = _uneven_batch(SEED + 3, count, (500, 12000))
    surfs = [bemgpu.mesh(nodes, tris) for _, nodes, tris in bodies]
    for s_ in surfs:
        s_.handle(ctx)
    sizes = [s_.n_panels for s_ in surfs]
    groups = _memory_groups(sizes, 90e9, 24.0 + 40.0 / 1e3)

    def step(precision, idx):
        amps = {}
        for g in _memory_groups([sizes[i] for i in idx], 90e9, 24.0 if precision == "mixed"
                                else 48.0):
            ids = [idx[q] for q in g]
            items = []
            for i in ids:
                b = bodies[i][0]
                bc = bemgpu.Rigid() if b["boundary"] == "rigid" else bemgpu.PressureRelease()
                items.append((surfs[i], bc, 2 * math.pi * b["frequency"] / 1500.0,
                              dict(precision=precision)))
            fs = bemgpu.factor_batch(items, ctx)
            sols = bemgpu.solve_batch(fs, [[bodies[i][0]["incidence_angle"]] for i in ids],
                                      [[bodies[i][0]["incidence_azimuth"]] for i in ids])
            for i, s_ in zip(ids, sols):
                amps[i] = bemgpu.scattering_amplitude(s_)
                s_.close()
            for f in fs:
                f.close()
        return amps

    allidx = list(range(count))
    for _ in range(max(1, args.warmup)):
        step("mixed", allidx)
    clocks = Clocks(0)
    clocks.start()
    l0 = bemgpu.Context.launch_count()
    ts = []
    for _ in range(args.steps):
        ctx.timer_start()
        am = step("mixed", allidx)
        ts.append(ctx.timer_stop())
    launches = (bemgpu.Context.launch_count() - l0) // args.steps
    clk = clocks.stop()
    gstats = ctx.graph_stats()
    # the same steps with the launch-shape tuner and the captured LU graphs switched off
    ctx.set_autotune(False)
    ctx.set_graphs(False)
    step("mixed", allidx)
    ts_plain = []
    for _ in range(args.steps):
        ctx.timer_start()
        ap = step("mixed", allidx)
        ts_plain.append(ctx.timer_stop())
    ctx.set_autotune(True)
    ctx.set_graphs(True)
    same_bits = all(np.array_equal(am[i], ap[i]) for i in allidx)
    # FP64 on a subset spanning the sizes: the FP64 LU of all 256 bodies at the GB300's
    # FP64 rate would take about a quarter of an hour
    order = np.argsort(sizes)
    sub = [int(i) for i in order[:: max(1, count // args.fp64_bodies)]][: args.fp64_bodies]
    ctx.timer_start()
    a64 = step("double", sub)
    fp64_ms = ctx.timer_stop()
    err = [abs(20 * math.log10(abs(am[i])) - 20 * math.log10(abs(a64[i]))) for i in sub]
    ms = float(np.mean(ts))
    line = _base_line(
        "BEM solves/s, uneven batch of 256 bodies of revolution", count * 1e3 / ms, "solves/s",
        ms, args,
        {"workload": f"{count} seeded bodies of revolution, panels log-uniform 500-12000, "
                     "f 10-200 kHz, rigid/soft 50/50, Burton-Miller", "bodies": count,
         "panels_total": int(sum(sizes)), "panels_max": int(max(sizes)),
         "memory_groups": len(groups), "seed": SEED + 3},
        dtype="c64 factor + fp64 refinement",
        fp64={"solves_per_s": len(sub) * 1e3 / fp64_ms, "bodies": len(sub),
              "panels": [sizes[i] for i in sub]},
        ts_error_db={"max": float(max(err)), "per_body": [float(e) for e in err],
                     "vs": "GPU FP64 on the subset (the GPU FP64 path is pinned to the CPU "
                           "oracle on four of these bodies by the GPU tests)"},
        untuned={"solves_per_s": count * 1e3 / float(np.mean(ts_plain)),
                 "ms_per_step": float(np.mean(ts_plain)),
                 "note": "launch-shape tuner and captured LU graphs off",
                 "same_bits": same_bits},
        lu_graphs=gstats,
        clocks=clk, gpu_launches=launches)
    print(json.dumps(line))
    return line


def _request_stream(nreq, pool):
    """The served request stream: each request draws one body from a pool of `pool`
    seeded bodies of the uneven distribution (panels 500..16000), 1-32 frequencies
    (5 % apart from the body's frequency) and 1-64 polar incidence angles."""
    from bemgpu import meshes
    rng = np.random.default_rng(SEED + 4)
    bodies = [meshes.random_body(SEED + 4, i, (500, 16000)) for i in range(pool)]
    reqs = []
    for _ in range(nreq):
        bi = int(rng.integers(0, pool))
        nf = int(rng.integers(1, 33))
        na = int(rng.integers(1, 65))
        freqs = bodies[bi]["frequency"] * (1.0 + 0.05 * np.arange(nf))
        reqs.append((bi, 2 * math.pi * freqs / 1500.0, rng.uniform(0.0, math.pi, size=na)))
    return bodies, reqs


def _serve(srv_factory, surfs, bodies, reqs, subset, rate, seed):
    """Open-loop Poisson arrivals at `rate` requests/s into a fresh server; latency =
    completion - submission, measured by the library."""
    import queue
    import threading as th

    import bemgpu
    srv = srv_factory()
    arrivals = np.cumsum(np.random.default_rng(seed).exponential(1.0 / rate, size=len(subset)))
    tickets = queue.Queue()
    lat, errors = {}, []

    def waiter():
        while True:
            item = tickets.get()
            if item is None:
                return
            tk, i = item
            try:
                lat[i] = srv.wait(tk, timeout_ms=-1)
            except Exception as e:  # noqa: BLE001 - reported in the result line
                errors.append(f"request {i}: {e}")
    wt = th.Thread(target=waiter)
    t0 = time.perf_counter()
    wt.start()
    try:
        for j, i in enumerate(subset):
            now = time.perf_counter() - t0
            if arrivals[j] > now:
                time.sleep(arrivals[j] - now)
            bi, ks, ang = reqs[i]
            bc = bemgpu.Rigid() if bodies[bi]["boundary"] == "rigid" else bemgpu.PressureRelease()
            tickets.put((srv.submit(surfs[bi], bc, ks, ang, precision=srv.precision), i))
            if (j + 1) % 500 == 0:
                print(f"# submitted {j + 1} of {len(subset)} at "
                      f"{time.perf_counter() - t0:.0f} s, {len(lat)} done", file=sys.stderr,
                      flush=True)
    finally:
        tickets.put(None)
        wt.join()
    wall = time.perf_counter() - t0
    st = srv.stats()
    srv.close()
    done = [i for i in subset if i in lat]
    if not done:
        raise RuntimeError(f"every request failed; first: {errors[0]}")
    lats = np.array([lat[i][1] for i in done])
    solves = sum(len(reqs[i][1]) * len(reqs[i][2]) for i in done)
    res = dict(wall_s=wall, requests=len(subset), solves=solves, solves_per_s=solves / wall,
               rate_per_s=rate, p50_ms=float(np.percentile(lats, 50)),
               p99_ms=float(np.percentile(lats, 99)), max_ms=float(lats.max()),
               failed_requests=len(errors), stats=st)
    if errors:  # reported in the line (solves/s and latencies count completed requests)
        res["first_error"] = errors[0]
    return res, {i: lat[i][0] for i in done}


def run_config4(args):
    """Open-loop Poisson request stream into the continuous-batching server: 10^4
    requests (bodies of revolution, 500-16000 panels, 1-32 frequencies, 1-64 incidence
    angles), HBM budget 150 GB, offered at 70 % of the capacity measured closed-loop on
    the first 2 % of the requests.  The same stream's first --fp64-requests requests are
    then served in FP64 (at 70 % of the FP64 capacity measured closed-loop on them, which
    is far lower: the GB300's FP64 rate bounds its LU) and in mixed precision at that same
    rate, for the latency and the TS error of mixed against FP64 on identical requests."""
    import bemgpu
    ctx = bemgpu.Context(0, hbm_budget_bytes=int(150e9))
    bodies, reqs = _request_stream(args.requests, args.pool)
    surfs = []
    for b in bodies:
        nodes, tris = bemgpu.meshes.body_of_revolution(b["b"], b["aspect"], b["coeffs"],
                                                       b["nlon"], b["nrings"])
        s_ = bemgpu.mesh(nodes, tris)
        s_.handle(ctx)  # meshes resident before the stream starts
        surfs.append(s_)

    def factory(precision):
        def make():
            srv = bemgpu.Server(ctx, max_batch=64, cache_bytes=int(40e9), lanes=args.lanes)
            srv.precision = precision
            return srv
        return make

    def capacity(precision, subset):
        res, out = _serve(factory(precision), surfs, bodies, reqs, subset, 1e6, SEED + 40)
        return res["requests"] / res["wall_s"], out

    warm = list(range(min(len(reqs), max(32, args.requests // 50))))
    cap_m, _ = capacity("mixed", warm)
    rate = args.rate or 0.7 * cap_m
    clocks = Clocks(0)
    clocks.start()
    l0 = bemgpu.Context.launch_count()
    res_m, out_m = _serve(factory("mixed"), surfs, bodies, reqs, list(range(len(reqs))), rate,
                          SEED + 41)
    launches = bemgpu.Context.launch_count() - l0
    clk = clocks.stop()
    # FP64 and mixed on the same first requests, at 70 % of the FP64 capacity
    sub = list(range(min(len(reqs), args.fp64_requests)))
    cap_d, _ = capacity("double", sub)
    rate_d = 0.7 * cap_d
    res_d, out_d = _serve(factory("double"), surfs, bodies, reqs, sub, rate_d, SEED + 42)
    res_ms, out_ms = _serve(factory("mixed"), surfs, bodies, reqs, sub, rate_d, SEED + 42)
    both = [i for i in sub if i in out_ms and i in out_d]
    err = [float(np.max(np.abs(20 * np.log10(np.abs(out_ms[i])) -
                               20 * np.log10(np.abs(out_d[i]))))) for i in both]
    same = all(np.array_equal(out_ms[i], out_m[i]) for i in both if i in out_m)
    line = _base_line(
        "BEM solves/s & p99 latency, served Poisson stream", res_m["solves_per_s"], "solves/s",
        res_m["wall_s"] * 1e3, args,
        {"workload": f"{len(reqs)} Poisson requests over {args.pool} seeded bodies of "
                     "revolution (500-16000 panels), 1-32 frequencies, 1-64 angles, HBM "
                     "budget 150 GB, continuous batching on "
                     f"{args.lanes} lanes with a factor cache", "requests": len(reqs),
         "pool": args.pool, "seed": SEED + 4, "lanes": args.lanes},
        dtype="c64 factor + fp64 refinement",
        latency_ms={"p50": res_m["p50_ms"], "p99": res_m["p99_ms"], "max": res_m["max_ms"]},
        failed_requests=res_m["failed_requests"],
        **({"first_error": res_m["first_error"]} if "first_error" in res_m else {}),
        offered_rate_per_s=rate, closed_loop_capacity_per_s=cap_m,
        server=res_m["stats"],
        fp64_same_stream={"requests": len(sub), "rate_per_s": rate_d,
                          "fp64": {k2: v for k2, v in res_d.items() if k2 != "stats"},
                          "mixed": {k2: v for k2, v in res_ms.items() if k2 != "stats"},
                          "solves_per_s_ratio_mixed_over_fp64":
                              res_ms["solves_per_s"] / res_d["solves_per_s"],
                          "closed_loop_capacity_ratio": cap_m / cap_d},
        ts_error_db={"max": max(err) if err else None, "requests": len(both),
                     "vs": "the same requests served in FP64"},
        same_bits_in_two_different_streams=same,
        clocks=clk, gpu_launches=int(launches))
    print(json.dumps(line))
    return line


def run_config4_phases(args):
    """Where a served stream's device time goes: the items (request, frequency) of the
    stream's first --requests requests, grouped as the server groups them (one size class
    of at most 64 factorisations and about 100 GB per batch), factored and solved through
    the batch API with per-family CUDA-event times; once with every request's angles and
    once with one angle per item."""
    import bemgpu
    ctx = bemgpu.Context(0, hbm_budget_bytes=int(150e9))
    bodies, reqs = _request_stream(args.requests, args.pool)
    surfs = {}
    for bi in sorted({r[0] for r in reqs}):
        b = bodies[bi]
        nodes, tris = bemgpu.meshes.body_of_revolution(b["b"], b["aspect"], b["coeffs"],
                                                       b["nlon"], b["nrings"])
        surfs[bi] = bemgpu.mesh(nodes, tris)
        surfs[bi].handle(ctx)
    items = sorted(((bi, float(k), ang) for bi, ks, ang in reqs for k in ks),
                   key=lambda it: surfs[it[0]].n_panels)
    groups, cur = [], []
    for it in items:
        n = surfs[it[0]].n_panels
        if cur and (n > 2 * surfs[cur[0][0]].n_panels or len(cur) >= 64 or
                    24.0 * sum(surfs[c[0]].n_panels ** 2 for c in cur + [it]) > 100e9):
            groups.append(cur)
            cur = []
        cur.append(it)
    groups.append(cur)
    fams = ("assemble", "near", "equilibrate", "scale_copy", "getf2", "laswp", "trsm",
            "tc_pack", "gemm_tc", "gemm_panel", "getrs", "gecon", "residual", "forcing",
            "incident", "far_field")

    def run(one_angle):
        ctx.timer_start()
        for g in groups:
            its = [(surfs[bi], bemgpu.Rigid() if bodies[bi]["boundary"] == "rigid"
                    else bemgpu.PressureRelease(), k, dict(precision="mixed"))
                   for bi, k, _ in g]
            fs = bemgpu.factor_batch(its, ctx)
            angs = [list(a[:1]) if one_angle else list(a) for _, _, a in g]
            sols = bemgpu.solve_batch(fs, angs, [[0.0] * len(a) for a in angs])
            for s_ in sols:
                bemgpu.scattering_amplitude(s_)
                s_.close()
            for f in fs:
                f.close()
        return ctx.timer_stop()

    out = {}
    for one in (False, True):
        run(one)  # warm-up (tuner, first-time setup)
        ctx.profile(True)
        ctx.profile_reset()
        ms = run(one)
        prof = {f: round(ctx.profile_read(f)[1], 1) for f in fams}
        ctx.profile(False)
        out["one_angle" if one else "all_angles"] = {"ms": ms, "phase_ms": prof}
    line = {"metric": "device time by phase of served items (batched closed loop)",
            "requests": len(reqs), "items": len(items), "batches": len(groups),
            "panels_per_batch_head": [surfs[g[0][0]].n_panels for g in groups],
            "angles_per_item_mean": float(np.mean([len(a) for _, _, a in items])), **out,
            "note": "profiled runs: per-family CUDA events on the main stream"}
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
    frequency (the middle one) of the same workload: a bounded sample.  The same
    frequency is then solved by the oracle in FP64 (untimed) as the error reference of
    the GPU's results.  Returns (baseline, oracle-error record)."""
    nodes, tris = workload_mesh(args.nlon, args.nrings)
    k = ks[len(ks) // 2]
    dt, a_mixed = _oracle_one(k, nodes, tris, "mixed")
    dt64, a64 = _oracle_one(k, nodes, tris, "double")
    base = {"value": 1.0 / dt, "unit": "solves/s", "cores": os.cpu_count(), "kind": "port",
            "sample": f"1 of {len(ks)} frequencies (k={k:.2f}/m), mixed precision, "
                      f"oracle C assembly (OpenMP) + LAPACK cgetrf/zgetrf, {dt:.1f} s"}
    err = {"oracle": "CPU FP64 restatement (C assembly + LAPACK zgetrf), "
                     f"{dt64:.1f} s", "frequency_index": len(ks) // 2, "k": float(k),
           "_fp64": a64, "_mixed": a_mixed}
    return base, err


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
            "config": headline_config(int(tris.shape[1]), args.freqs),
            "cpu_baseline": {"value": v, "unit": "solves/s", "cores": os.cpu_count(),
                             "kind": "port",
                             "sample": "one frequency per step (the reference's Julia code "
                                       "cannot run here; CPU restatement in oracle/)"},
            "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return line


NCU_HM_TRAFFIC = 362.57e6 / 360.526e6


def run_config5(args):
    """The reference's default rigid path, compressed operators + GMRES
    (solve_full_bem(...; compression=(method=:hmatrix, tol=1e-5), gmres_kwargs=(reltol=1e-4,
    restart=150, maxiter=1200)), full.jl:52-184) on the 20480-panel rigid prolate spheroid
    0.05 x 0.0125 m at 60 kHz: one bem() call per step (cluster tree cached on the mesh;
    cross approximation, full blocks, GMRES and far field every step), complex64/FP32
    operators (precision=:mixed) and complex128 (precision=:double); TS against the dense
    refined solve of the same incidence; an 81920-panel body as the size the dense path
    cannot reach in comparable time, and a 327680-panel one whose dense system (860 GB)
    does not fit one GPU."""
    import bemgpu
    from bemgpu import meshes
    ctx = bemgpu.Context(0)
    nodes, tris = meshes.uv_spheroid(0.05, 0.0125, 128, 80)
    surf = bemgpu.mesh(nodes, tris)
    k = 2 * math.pi * 60e3 / 1500.0
    beta, alpha = 1.0, 0.3
    hm = dict(method="hmatrix", tol=1e-5)
    gk = dict(reltol=1e-4, restart=150, maxiter=1200)

    def one(prec):
        sol = bemgpu.bem(surf, bemgpu.Rigid(), k, incidence_angle=beta, incidence_azimuth=alpha,
                         compression=hm, gmres_kwargs=gk, precision=prec, ctx=ctx)
        f = bemgpu.scattering_amplitude(sol)
        st = sol.hmatrix_stats()
        sol.close()
        return f, st

    out = {}
    for prec in ("mixed", "double"):
        for _ in range(max(args.warmup, 3)):
            one(prec)
        steps = args.steps if prec == "mixed" else max(1, min(args.steps, 3))
        clocks = Clocks(0)
        clocks.start()
        ctx.profile(True)
        ctx.profile_reset()
        l0 = bemgpu.Context.launch_count()
        ts = []
        for _ in range(steps):
            ctx.timer_start()
            f, st = one(prec)
            ts.append(ctx.timer_stop())
        launches = (bemgpu.Context.launch_count() - l0) // steps
        prof = {fam: ctx.profile_read(fam)[1] / steps for fam in
                ("hm_aca", "hm_dense", "near", "hm_matvec", "gmres", "incident", "far_field")}
        ctx.profile(False)
        out[prec] = dict(f=f, ms=float(np.mean(ts)), clocks=clocks.stop(), launches=launches,
                         prof=prof, stats=st)
    # accurate reference: the dense refined solve of the same incidence
    ref = bemgpu.bem(surf, bemgpu.Rigid(), k, incidence_angle=beta, incidence_azimuth=alpha,
                     precision="mixed", refinement=dict(tolerance=1e-12), ctx=ctx)
    f_ref = bemgpu.scattering_amplitude(ref)
    ref.close()
    ctx.timer_start()
    ref = bemgpu.bem(surf, bemgpu.Rigid(), k, incidence_angle=beta, incidence_azimuth=alpha,
                     precision="mixed", ctx=ctx)
    dense_ms = ctx.timer_stop()
    ref.close()
    ts_ref = 20 * math.log10(abs(f_ref))
    # 81920 panels, mixed
    n2, t2 = meshes.uv_spheroid(0.1, 0.025, 256, 160)
    big = bemgpu.mesh(n2, t2)
    bemgpu.bem(big, bemgpu.Rigid(), k, compression=hm, gmres_kwargs=gk, precision="mixed",
               ctx=ctx).close()
    ctx.timer_start()
    sb = bemgpu.bem(big, bemgpu.Rigid(), k, compression=hm, gmres_kwargs=gk, precision="mixed",
                    ctx=ctx)
    big_ms = ctx.timer_stop()
    big_st = sb.hmatrix_stats()
    sb.close()
    # 327680 panels, the same body: beyond one GPU's memory as a dense system (860 GB)
    n3, t3 = meshes.uv_spheroid(0.1, 0.025, 512, 320)
    huge = bemgpu.mesh(n3, t3)
    bemgpu.bem(huge, bemgpu.Rigid(), k, compression=hm, gmres_kwargs=gk, precision="mixed",
               ctx=ctx).close()
    ctx.timer_start()
    sh = bemgpu.bem(huge, bemgpu.Rigid(), k, compression=hm, gmres_kwargs=gk, precision="mixed",
                    ctx=ctx)
    huge_ms = ctx.timer_stop()
    huge_st, huge_d = sh.hmatrix_stats(), sh.diagnostics()
    huge_ts = 20 * math.log10(abs(bemgpu.scattering_amplitude(sh)))
    sh.close()
    # the same body (64 x 40 UV panels) in the reference's own discretisation: 35840
    # quadrature-node unknowns, dense factor and compressed node operators + GMRES
    nn_, tn_ = meshes.uv_spheroid(0.05, 0.0125, 64, 40)
    sny = bemgpu.mesh(nn_, tn_)
    ny = {"panels": int(np.asarray(tn_).shape[1])}
    for label, extra in (("dense", {}), ("compressed", dict(compression=hm, gmres_kwargs=gk))):
        def one_ny():
            return bemgpu.bem(sny, bemgpu.Rigid(), k, incidence_angle=beta,
                              incidence_azimuth=alpha, precision="mixed", ctx=ctx,
                              discretization="nystrom", **extra)
        one_ny().close()  # node set and its cluster tree, built once per mesh
        ctx.timer_start()
        sn = one_ny()
        ms_ = ctx.timer_stop()
        d_ = sn.diagnostics()
        ny[label] = {"ms": ms_, "ts_db": 20 * math.log10(abs(bemgpu.scattering_amplitude(sn))),
                     "device_bytes": d_["device_bytes"]}
        if extra:
            st_ = sn.hmatrix_stats()
            ny[label].update(gmres_iterations=st_["gmres_iterations"],
                             gmres_converged=bool(st_["gmres_converged"]),
                             compression=st_["compression"], build_ms=st_["build_ms"],
                             gmres_ms=st_["gmres_ms"])
        sn.close()
    ny["unknowns"] = 7 * ny["panels"]
    ny["ts_db_compressed_minus_dense"] = ny["compressed"]["ts_db"] - ny["dense"]["ts_db"]
    m = out["mixed"]
    st = m["stats"]
    hbm, _, which = measured_peaks()
    n = int(np.asarray(tris).shape[1])
    # one product of the system operator: its stored entries (complex64) once, the vector in
    # and out (complex128)
    mv_bytes = (st["lowrank_entries"] + st["dense_entries"]) / 2 * 8 + 2 * 16 * n
    mv_ms = m["prof"]["hm_matvec"]
    achieved = mv_bytes / (mv_ms * 1e-3) / 1e9 if mv_ms else None
    cpu = None
    if not args.no_cpu:
        from oracle import oracle as O
        ns, tsm = meshes.uv_spheroid(0.05, 0.0125, 48, 30)
        t0 = time.perf_counter()
        rep = O.solve_gmres(ns, tsm, "rigid", k, incidence_angle=beta, incidence_azimuth=alpha,
                            reltol=1e-4, restart=150, maxiter=1200)
        dt = time.perf_counter() - t0
        cpu = {"value": 1.0 / dt, "unit": "solves/s", "cores": os.cpu_count(), "kind": "port",
               "sample": f"the oracle's GMRES path (dense operators, compression=:none) on the "
                         f"same spheroid meshed with {int(np.asarray(tsm).shape[1])} panels "
                         f"(a smaller body: the dense CPU path at 20480 panels takes minutes), "
                         f"{rep['iterations']} iterations, {dt:.2f} s"}
    line = _base_line(
        "BEM solves/s, rigid spheroid 20480 panels, compressed operators + GMRES",
        1e3 / m["ms"], "solves/s", m["ms"], args,
        {"workload": "rigid prolate spheroid 0.05x0.0125 m, 20480 panels, f=60 kHz, one "
                     "incidence per solve, compression=(hmatrix, tol 1e-5), GMRES reltol 1e-4 "
                     "restart 150", "panels": n, "leaf_size": 64, "eta": 3.0},
        dtype="c64 operators (FP32 entries and products) + fp64 GMRES",
        e2e={"value": 1e3 / m["ms"], "unit": "solves/s", "h2d_bytes_per_step": 16,
             "d2h_bytes_per_step": 16,
             "note": "each step is the public bem() call: angles in, amplitude out"},
        phase_ms_per_step=m["prof"],
        compression=st,
        fp64={"solves_per_s": 1e3 / out["double"]["ms"], "phase_ms_per_step": out["double"]["prof"],
              "ts_db": 20 * math.log10(abs(out["double"]["f"]))},
        ts_db=20 * math.log10(abs(m["f"])), ts_dense_refined_db=ts_ref,
        ts_error_db_vs_dense=abs(20 * math.log10(abs(m["f"])) - ts_ref),
        ts_error_db_fp64_vs_dense=abs(20 * math.log10(abs(out["double"]["f"])) - ts_ref),
        dense_mixed_ms=dense_ms,
        large={"panels": int(np.asarray(t2).shape[1]), "ms": big_ms,
               "compression": big_st["compression"], "gmres_iterations": big_st["gmres_iterations"],
               "dense_complex64_bytes": int(np.asarray(t2).shape[1]) ** 2 * 8},
        huge={"panels": int(np.asarray(t3).shape[1]), "ms": huge_ms,
              "device_bytes": huge_d["device_bytes"], "compression": huge_st["compression"],
              "gmres_iterations": huge_st["gmres_iterations"],
              "gmres_converged": bool(huge_st["gmres_converged"]), "ts_db": huge_ts,
              "dense_complex64_bytes": int(np.asarray(t3).shape[1]) ** 2 * 8},
        nystrom=ny,
        roofline={"bound": "hbm", "kernel": "hierarchical product (k_hm_vt, k_hm_lblk, "
                                            "k_hm_dblk, k_hm_gather)",
                  "achieved": achieved, "peak": hbm, "unit": "GB/s",
                  "frac": achieved / hbm if achieved else None, "peak_source": f"{which} HBM",
                  # ncu DRAM bytes of the four product kernels over the algorithmic bytes,
                  # one capture of the same workload (362.57 MB read+written, 360.53 MB)
                  "traffic": NCU_HM_TRAFFIC * mv_bytes, "algorithmic_bytes_per_launch": mv_bytes},
        clocks=m["clocks"], gpu_launches=m["launches"], cpu_baseline=cpu)
    print(json.dumps(line))
    return line


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--freqs", type=int, default=W["nfreq"])
    ap.add_argument("--fp64-freqs", type=int, default=3)
    ap.add_argument("--nlon", type=int, default=W["nlon"])
    ap.add_argument("--nrings", type=int, default=W["nrings"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--config", type=int, default=1, choices=[0, 1, 2, 3, 4, 5],
                    help="workload: 1 = headline batched frequency sweep (default); 0 rigid "
                         "sphere; 2 large single solve x 181 angles; 3 uneven batch; 4 serving; "
                         "5 compressed operators + GMRES (the reference's default rigid path)")
    ap.add_argument("--bodies", type=int, default=256, help="config 3: bodies")
    ap.add_argument("--fp64-bodies", type=int, default=16,
                    help="config 3: bodies also solved in FP64")
    ap.add_argument("--requests", type=int, default=10000, help="config 4: requests")
    ap.add_argument("--pool", type=int, default=512, help="config 4: distinct bodies")
    ap.add_argument("--lanes", type=int, default=2, help="config 4: server lanes")
    ap.add_argument("--fp64-requests", type=int, default=16,
                    help="config 4: requests of the stream also served in FP64")
    ap.add_argument("--rate", type=float, default=0.0, help="config 4: arrivals/s (0: 70%% load)")
    ap.add_argument("--phases", action="store_true",
                    help="config 4: device time by phase of the stream's first --requests "
                         "requests, batched closed loop, instead of serving them")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.config == 4 and args.phases:
        run_config4_phases(args)
    elif args.config == 1:
        run_ours(args)
    else:
        {0: run_config0, 2: run_config2, 3: run_config3, 4: run_config4,
         5: run_config5}[args.config](args)


if __name__ == "__main__":
    main()
