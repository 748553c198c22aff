"""Analytic sphere modal series (test infrastructure only: the physics check).

Restates solvers/modal/sphere.jl of the reference: mode count (:1-3), coefficients for
rigid (:5-8), pressure release (:10-13) and fluid-filled spheres (:21-41), and the form
function f(theta) = -(i/k) sum (2m+1) P_m(cos theta) A_m (:279-288), with the spherical
Bessel/Hankel functions of numerics/special_functions.jl:8-39 taken from scipy.
"""
from __future__ import annotations

import math

import numpy as np
from scipy.special import eval_legendre, spherical_jn, spherical_yn


def mode_count(ka):
    return max(20, math.ceil(2.5 * ka + 4 * (ka + 1) ** (1.0 / 3.0) + 10))


def _js(m, x):
    return spherical_jn(m, x)


def _jsd(m, x):
    return spherical_jn(m, x, derivative=True)


def _hs(m, x):
    return spherical_jn(m, x) + 1j * spherical_yn(m, x)


def _hsd(m, x):
    return spherical_jn(m, x, derivative=True) + 1j * spherical_yn(m, x, derivative=True)


def coefficient(boundary, m, k, a, g=1.0, h=1.0):
    ka = k * a
    if boundary == "rigid":
        return -_jsd(m, ka) / _hsd(m, ka)
    if boundary == "pressure_release":
        return -_js(m, ka) / _hs(m, ka)
    if boundary == "fluid":
        kai = ka / h
        gh = g * h
        jd_int, jd_ext = _jsd(m, kai), _jsd(m, ka)
        j_int, j_ext = _js(m, kai), _js(m, ka)
        h_ext, hd_ext = _hs(m, ka), _hsd(m, ka)
        den = gh * j_int * hd_ext - h_ext * jd_int
        return (j_ext * jd_int - gh * j_int * jd_ext) / den
    raise ValueError(boundary)


def form_function(boundary, k, a, angle=math.pi, g=1.0, h=1.0, m_max=None):
    """Far-field amplitude of a sphere at scattering angle ``angle`` (pi = backscatter)."""
    m_max = mode_count(k * a) if m_max is None else m_max
    x = math.cos(angle)
    total = 0j
    for m in range(m_max + 1):
        total += (2 * m + 1) * eval_legendre(m, x) * coefficient(boundary, m, k, a, g, h)
    return -1j / k * total


def scattered_field(boundary, k, a, r, cos_theta, g=1.0, h=1.0, m_max=None):
    """Scattered pressure of a unit plane wave at distance r >= a from the sphere's centre,
    cos_theta = incidence direction . point direction: sum (2m+1) i^m A_m h_m(kr)
    P_m(cos theta), the near-field form of form_function (whose r -> infinity limit it is)."""
    m_max = mode_count(k * a) if m_max is None else m_max
    total = 0j
    for m in range(m_max + 1):
        total += ((2 * m + 1) * (1j ** m) * coefficient(boundary, m, k, a, g, h) *
                  _hs(m, k * r) * eval_legendre(m, cos_theta))
    return total
