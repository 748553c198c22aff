"""Regenerate the golden fixtures of tests/golden/ (run in the build container).

reference_amplitudes.json
    Independent far-field amplitudes hard-coded in the reference's own tests, read as
    text from the reference checkout whose path the REFERENCE environment variable
    gives (required; e.g. REFERENCE=/root/reference python tests/golden/make_golden.py):
      test/extended/bem/sphere/full3d.jl   "Independent transmission amplitudes"
      test/extended/bem/spheroid/full3d.jl "Full BEM against independent rigid-spheroid
                                            outputs"
    The reference compares its own BEM to these at 0.1 dB and 1 %.
oracle_golden.json
    Oracle outputs on small deterministic meshes (amplitudes, operator checksums),
    the regression pins of the CPU restatement and the parity targets of the GPU tests.
mesh_hashes.json
    SHA-256 fingerprints of the workload meshes (bit-exact connectivity and nodes).
"""
from __future__ import annotations

import json
import math
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "acousticscattering.jl_gb300")]
REFERENCE = os.environ.get("REFERENCE")

_CPLX = r"(-?[0-9.]+(?:e-?[0-9]+)?)\s*([+-])\s*([0-9.]+(?:e-?[0-9]+)?)im"


def _complex(m):
    re_, sign, im = m
    return [float(re_), (1.0 if sign == "+" else -1.0) * float(im)]


def reference_amplitudes():
    if not REFERENCE:
        raise SystemExit("set REFERENCE to the reference checkout (AcousticScattering.jl)")
    out = {"source": "reference tests (read as text)", "tolerance": {"db": 0.1, "rel": 0.01}}
    sph = open(os.path.join(REFERENCE, "test/extended/bem/sphere/full3d.jl")).read()
    block = sph[sph.index("Independent transmission amplitudes"):]
    block = block[:block.index("for (g, h, k, meshsize")]
    cases = []
    for m in re.finditer(r"\(([0-9.]+),\s*([0-9.]+),\s*([0-9.]+),\s*([0-9.]+),\s*(\d+),\s*(\d+),"
                         r"\s*\((.*?)\)\)", block, re.S):
        amps = [_complex(a) for a in re.findall(_CPLX, m.group(7))]
        cases.append({"g": float(m.group(1)), "h": float(m.group(2)), "k": float(m.group(3)),
                      "radius": 1.0, "incidence_angle": 0.0, "incidence_azimuth": 0.0,
                      "directions": [[-1.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0]],
                      "amplitudes": amps})
    out["fluid_sphere"] = cases
    spd = open(os.path.join(REFERENCE, "test/extended/bem/spheroid/full3d.jl")).read()
    block = spd[spd.index("independent rigid-spheroid outputs"):]
    block = block[:block.index("solution = bem(")]
    refs = []
    for m in re.finditer(r"\(\[([^\]]*)\],\s*" + _CPLX + r"\)", block):
        d = [eval(x.replace("sqrt", "math.sqrt"), {"math": math}) for x in m.group(1).split(",")]
        refs.append({"direction": d, "amplitude": _complex(m.groups()[1:4])})
    out["rigid_spheroid"] = {"a": 1.5, "b": 1.0, "k": 2.0, "incidence_angle": math.pi / 3,
                             "incidence_azimuth": 0.0, "references": refs}
    return out


def oracle_golden():
    import numpy as np

    from bemgpu import meshes
    from oracle import oracle as O

    nodes, tris = meshes.icosphere(1.0, 2)
    P = O.Panels(nodes, tris)
    out = {"mesh": "icosphere(1.0, 2): 320 panels", "cases": []}
    for boundary, form, k, g, h in (("rigid", "burton_miller", 1.7, 1, 1),
                                    ("rigid", "cbie", 1.7, 1, 1),
                                    ("pressure_release", "burton_miller", 1.7, 1, 1),
                                    ("pressure_release", "cbie", 1.7, 1, 1),
                                    ("fluid", "muller", 1.5, 1.04, 1.04),
                                    ("fluid", "cbie", 1.5, 1.04, 1.04),
                                    ("fluid", "muller", 1.0, 1000.0, 2.0)):
        r = O.solve(nodes, tris, boundary, k, incidence_angle=0.4, incidence_azimuth=0.3,
                    formulation=form, g=g, h=h, panels=P,
                    directions=[[-1.0, 0.0, 0.0], [0.0, 0.6, 0.8]])
        out["cases"].append({"boundary": boundary, "formulation": form, "k": k, "g": g, "h": h,
                             "incidence_angle": 0.4, "incidence_azimuth": 0.3,
                             "directions": [[-1.0, 0.0, 0.0], [0.0, 0.6, 0.8]],
                             "amplitudes": [[a.real, a.imag] for a in r["amplitudes"]],
                             "matrix_abs_sum": float(np.sum(np.abs(r["A"])))})
    return out


def mesh_hashes():
    from bemgpu import meshes

    out = {}
    for name, (nodes, tris) in {
            "icosphere_0.01_3": meshes.icosphere(0.01, 3),
            "uv_spheroid_0.02_0.01_64x40_j0.02_s20261203":
                meshes.uv_spheroid(0.02, 0.01, 64, 40, jitter=0.02, seed=20261203),
            "uv_spheroid_0.05_0.0125_128x80": meshes.uv_spheroid(0.05, 0.0125, 128, 80)}.items():
        out[name] = {"hash": meshes.mesh_hash(nodes, tris), "nodes": int(nodes.shape[1]),
                     "triangles": int(tris.shape[1])}
    return out


def main():
    with open(os.path.join(HERE, "reference_amplitudes.json"), "w") as fh:
        json.dump(reference_amplitudes(), fh, indent=1)
    with open(os.path.join(HERE, "oracle_golden.json"), "w") as fh:
        json.dump(oracle_golden(), fh, indent=1)
    with open(os.path.join(HERE, "mesh_hashes.json"), "w") as fh:
        json.dump(mesh_hashes(), fh, indent=1)


if __name__ == "__main__":
    main()
