"""GPU results against the CPU FP64 oracle on the benchmark workloads themselves.

The smaller parity tests pin every kernel at 80-1280 panels; these pin the solves the
throughput figures are quoted on, at their full sizes:

* the batched frequency sweep: fluid-filled prolate spheroid 0.02 x 0.01 m, 5120 jittered
  UV panels (seed 20261203), g = 1.0357, h = 1.0279, c = 1500 m/s, at 12 kHz, 66.9 kHz and
  120 kHz (k = 50.3, 280.0 and 502.7 1/m: the first, middle and last of the 64 frequencies);
* the large single solve: rigid prolate spheroid 0.05 x 0.0125 m, 20480 UV panels, 60 kHz,
  seven of the 181 incidence angles on one factorisation;
* the uneven batch: four bodies of the seeded body-of-revolution distribution
  (master seed 20261206), two rigid and two pressure-release, solved as one batch.

Bounds (the reference's contracts, test/basic/bem/formulations.jl:411-449 for mixed vs
double): FP64 GPU amplitudes within 1e-9 relative of the oracle's complex128 LAPACK solve;
mixed-precision target strengths within 0.01 dB of it, with refined backward errors at
or below the 1e-13 acceptance (1e-10 where the workload asks for that tolerance).
"""
import math

import numpy as np
import pytest

import bemgpu
from bemgpu import meshes
from oracle import oracle as O

pytestmark = pytest.mark.gpu

FP64_REL = 1e-9
MIXED_DB = 0.01


def _db(a, b):
    return abs(20 * math.log10(abs(a)) - 20 * math.log10(abs(b)))


# ---------------------------------------------------------------- batched frequency sweep
SWEEP_SEED = 20261203
SWEEP_G, SWEEP_H, SWEEP_C = 1.0357, 1.0279, 1500.0
SWEEP_FREQS = np.linspace(12e3, 120e3, 64)[[0, 32, 63]]


@pytest.fixture(scope="module")
def sweep_case():
    nodes, tris = meshes.uv_spheroid(0.02, 0.01, 64, 40, jitter=0.02, seed=SWEEP_SEED)
    ks = 2 * math.pi * SWEEP_FREQS / SWEEP_C
    P = O.Panels(nodes, tris)
    ref = [O.solve(nodes, tris, "fluid", float(k), incidence_angle=math.pi / 2,
                   incidence_azimuth=0.0, g=SWEEP_G, h=SWEEP_H, panels=P)["amplitudes"][0]
           for k in ks]
    return nodes, tris, ks, np.array(ref)


def _sweep_gpu(ctx, nodes, tris, ks, precision):
    surf = bemgpu.mesh(nodes, tris)
    fl = bemgpu.FluidFilled(SWEEP_G, SWEEP_H)
    fs = bemgpu.factor_batch([(surf, fl, float(k), dict(precision=precision)) for k in ks], ctx)
    sols = bemgpu.solve_batch(fs, [[math.pi / 2]] * len(fs), [[0.0]] * len(fs))
    amps = np.array([bemgpu.scattering_amplitude(s) for s in sols])
    diags = [s.diagnostics() for s in sols]
    for s in sols:
        s.close()
    for f in fs:
        f.close()
    return amps, diags


def test_frequency_sweep_fp64_matches_oracle(ctx, sweep_case):
    nodes, tris, ks, ref = sweep_case
    amps, _ = _sweep_gpu(ctx, nodes, tris, ks, "double")
    rel = np.abs(amps - ref) / np.abs(ref)
    assert np.all(rel < FP64_REL), rel


def test_frequency_sweep_mixed_within_001_db_of_oracle(ctx, sweep_case):
    nodes, tris, ks, ref = sweep_case
    amps, diags = _sweep_gpu(ctx, nodes, tris, ks, "mixed")
    err = [_db(a, b) for a, b in zip(amps, ref)]
    assert max(err) < MIXED_DB, err
    for d in diags:
        assert d["normwise_backward_error"] <= 1e-13, d
        assert d["componentwise_backward_error"] <= 1e-13, d


# ---------------------------------------------------------------- large single solve
LARGE_ANGLES = np.deg2rad([0.0, 30.0, 60.0, 90.0, 120.0, 150.0, 180.0])


@pytest.fixture(scope="module")
def large_case():
    nodes, tris = meshes.uv_spheroid(0.05, 0.0125, 128, 80)
    k = 2 * math.pi * 60e3 / 1500.0
    P = O.Panels(nodes, tris)
    M1, M2 = O.assemble_bm(P, k, True)
    Q = np.empty((P.n, len(LARGE_ANGLES)), dtype=np.complex128)
    dirs = []
    for r, beta in enumerate(LARGE_ANGLES):
        d = O.incidence_direction(float(beta), 0.0)
        _, Q[:, r] = O.incident(P, k, d)
        dirs.append(d)
    B = M2 @ Q
    del M2
    X = O.DoubleFactor(M1).solve(B)
    del M1
    ref = np.array([O.far_field(P, k, -dirs[r], X[:, r], -Q[:, r])
                    for r in range(len(LARGE_ANGLES))])
    return nodes, tris, k, ref


def test_large_solve_fp64_matches_oracle(ctx, large_case):
    nodes, tris, k, ref = large_case
    sw = bemgpu.incidence_angle_sweep(bemgpu.mesh(nodes, tris), bemgpu.Rigid(), k, LARGE_ANGLES,
                                      precision="double", ctx=ctx)
    rel = np.abs(sw.amplitudes - ref) / np.abs(ref)
    assert np.all(rel < FP64_REL), rel


def test_large_solve_mixed_within_001_db_of_oracle(ctx, large_case):
    nodes, tris, k, ref = large_case
    sw = bemgpu.incidence_angle_sweep(bemgpu.mesh(nodes, tris), bemgpu.Rigid(), k, LARGE_ANGLES,
                                      precision="mixed", refinement=dict(tolerance=1e-10),
                                      ctx=ctx)
    err = [_db(a, b) for a, b in zip(sw.amplitudes, ref)]
    assert max(err) < MIXED_DB, err
    assert sw.diagnostics["normwise_backward_error"] <= 1e-10, sw.diagnostics


# ---------------------------------------------------------------- uneven batch
UNEVEN_SEED = 20261206
# indices into the seeded distribution: rigid 2440 and 8136 panels (83.7, 105.5 kHz),
# pressure release 2720 and 3920 panels (61.3, 135.9 kHz)
UNEVEN_PICK = (144, 204, 92, 179)


@pytest.fixture(scope="module")
def uneven_case():
    cases = []
    for i in UNEVEN_PICK:
        b = meshes.random_body(UNEVEN_SEED, i, (500, 12000))
        nodes, tris = meshes.body_of_revolution(b["b"], b["aspect"], b["coeffs"], b["nlon"],
                                                b["nrings"])
        k = 2 * math.pi * b["frequency"] / 1500.0
        ref = O.solve(nodes, tris, b["boundary"], k, incidence_angle=b["incidence_angle"],
                      incidence_azimuth=b["incidence_azimuth"])["amplitudes"][0]
        cases.append((b, nodes, tris, k, ref))
    kinds = sorted(c[0]["boundary"] for c in cases)
    assert kinds == ["pressure_release", "pressure_release", "rigid", "rigid"]
    return cases


def _uneven_gpu(ctx, cases, precision):
    items, angles, azis = [], [], []
    for b, nodes, tris, k, _ in cases:
        bc = bemgpu.Rigid() if b["boundary"] == "rigid" else bemgpu.PressureRelease()
        items.append((bemgpu.mesh(nodes, tris), bc, k, dict(precision=precision)))
        angles.append([b["incidence_angle"]])
        azis.append([b["incidence_azimuth"]])
    fs = bemgpu.factor_batch(items, ctx)
    sols = bemgpu.solve_batch(fs, angles, azis)
    amps = np.array([bemgpu.scattering_amplitude(s) for s in sols])
    diags = [s.diagnostics() for s in sols]
    for s in sols:
        s.close()
    for f in fs:
        f.close()
    return amps, diags


def test_uneven_batch_fp64_matches_oracle(ctx, uneven_case):
    amps, _ = _uneven_gpu(ctx, uneven_case, "double")
    ref = np.array([c[4] for c in uneven_case])
    rel = np.abs(amps - ref) / np.abs(ref)
    assert np.all(rel < FP64_REL), rel


def test_uneven_batch_mixed_within_001_db_of_oracle(ctx, uneven_case):
    amps, diags = _uneven_gpu(ctx, uneven_case, "mixed")
    err = [_db(a, c[4]) for a, c in zip(amps, uneven_case)]
    assert max(err) < MIXED_DB, err
    for d in diags:
        assert d["normwise_backward_error"] <= 1e-13, d
