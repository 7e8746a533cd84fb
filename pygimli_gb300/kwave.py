"""Wavenumbers and weights of the 2.5-D inverse Fourier (cosine) transform.

Restates core/src/bert/bertMisc.cpp:36-129 (``initKWaveList``) and the
Gauss quadrature nodes of core/src/numericbase.cpp:51-155, which follow the
published Numerical Recipes routines ``gauleg`` (Newton iteration on the
Legendre recurrence, stop when |z - z1| <= 3e-6) and ``gaulag`` (alpha = 0,
stop when |z - z1| <= 3e-11, at most 20 iterations).  The reference's
tolerances are kept because they decide the last digits of k and w and so
the potentials at the 1e-7 level.

3-D meshes use the single wavenumber k = 0 with weight 1.
"""
from __future__ import annotations

import math

import numpy as np


def gauss_legendre(x1, x2, n):
    """n-point Gauss-Legendre nodes/weights on [x1, x2] (NR gauleg)."""
    x = np.zeros(n)
    w = np.zeros(n)
    eps = 3.0e-6
    m = (n + 1.0) / 2.0
    xm = 0.5 * (x2 + x1)
    xl = 0.5 * (x2 - x1)
    i = 1
    while i <= m:
        z = math.cos(math.pi * (i - 0.25) / (n + 0.5))
        z1 = z + 2.0 * eps
        pp = 0.0
        while abs(z - z1) > eps:
            p1, p2 = 1.0, 0.0
            for j in range(1, n + 1):
                p3 = p2
                p2 = p1
                p1 = ((2.0 * j - 1.0) * z * p2 - (j - 1.0) * p3) / float(j)
            pp = float(n) * (z * p1 - p2) / (z * z - 1.0)
            z1 = z
            z = z1 - p1 / pp
        x[i - 1] = xm - xl * z
        x[n - i] = xm + xl * z
        w[i - 1] = 2.0 * xl / ((1.0 - z * z) * pp * pp)
        w[n - i] = w[i - 1]
        i += 1
    return x, w


def gauss_laguerre(n):
    """n-point Gauss-Laguerre nodes/weights, alpha = 0 (NR gaulag)."""
    x = np.zeros(n)
    w = np.zeros(n)
    eps = 3.0e-11
    maxiter = 20
    z = 0.0
    pp = p2 = 0.0
    for i in range(1, n + 1):
        if i == 1:
            z = 3.0 / (1.0 + 2.4 * n)
        elif i == 2:
            z = z + 15.0 / (1.0 + 2.5 * n)
        else:
            ai = i - 2
            z = z + (1.0 + 2.55 * ai) / (1.9 * ai) * (z - x[ai - 1])
        for _ in range(maxiter):
            p1, p2 = 1.0, 0.0
            for j in range(1, n + 1):
                p3 = p2
                p2 = p1
                p1 = ((2.0 * j - 1 - z) * p2 - (j - 1) * p3) / j
            pp = n * (p1 - p2) / z
            z1 = z
            z = z1 - p1 / pp
            if abs(z - z1) <= eps:
                break
        x[i - 1] = z
        w[i - 1] = -1.0 / (pp * n * p2)
    return x, w


def kwave_list(r_min, r_max, n_legendre, n_laguerre):
    """k and w for half-distances r_min..r_max (bertMisc.cpp:88-103)."""
    k0 = 1.0 / (2.0 * r_min)
    x, w = gauss_legendre(0.0, 1.0, n_legendre)
    k_leg = k0 * x * x
    w_leg = 2.0 * k0 * x * w / math.pi
    x, w = gauss_laguerre(n_laguerre)
    k_lag = k0 * (x + 1.0)
    w_lag = k0 * np.exp(x) * w / math.pi
    return np.concatenate([k_leg, k_lag]), np.concatenate([w_leg, w_lag])


def init_kwave_list(dim, sensor_pos):
    """Default k/w for a mesh of dimension ``dim`` and the sensor positions
    (bertMisc.cpp:36-86)."""
    if dim == 3:
        return np.zeros(1), np.ones(1)
    p = np.asarray(sensor_pos, dtype=np.float64)
    if len(p) < 2:
        raise ValueError("at least two sensors are needed for the default wavenumbers")
    r_min, r_max = np.inf, -np.inf
    for i in range(len(p)):
        d = np.linalg.norm(p[i + 1:] - p[i], axis=1)
        if len(d):
            r_min = min(r_min, d.min())
            r_max = max(r_max, d.max())
    r_min /= 2.0
    r_max *= 2.0
    n_leg = max(int(math.floor(6.0 * math.log10(r_max / r_min))), 4)
    return kwave_list(r_min, r_max, n_leg, 4)
