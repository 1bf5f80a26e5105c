"""Analytic rigid-sphere scattering (Mie series) -- TEST INFRASTRUCTURE ONLY.

Restates ``ps`` of misc/analytic_sphere.py:13-26: the scattered pressure at distance r and
angle theta (from the propagation direction) of a unit plane wave on a rigid sphere of radius a,

    p_s = conj( - sum_n i^n (2n+1) j_n'(ka)/h_n'(ka) P_n(cos theta) h_n(kr) ),

with h_n = j_n + i y_n and N = 100 terms. The conjugate converts to the e^{+i w t} convention of
the BEM kernel e^{-ikr}/(4 pi r).
"""
from __future__ import annotations

import numpy as np
import scipy.special as sp


def scattered_pressure(r: float, theta, k: float, a: float, n_terms: int = 100) -> np.ndarray:
    theta = np.atleast_1d(np.asarray(theta, dtype=np.float64))
    ct = np.cos(theta)
    val = np.zeros(theta.shape, np.complex128)
    for n in range(n_terms):
        djn = sp.spherical_jn(n, k * a, True)
        dhn = sp.spherical_jn(n, k * a, True) + 1j * sp.spherical_yn(n, k * a, True)
        hn = sp.spherical_jn(n, k * r) + 1j * sp.spherical_yn(n, k * r)
        val -= (1j ** n) * (2 * n + 1) * (djn / dhn) * sp.eval_legendre(n, ct) * hn
    return np.conj(val)
