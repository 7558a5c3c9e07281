"""Complex-energy contours for the strength function.

``circle`` follows pynfam's CIRCLE contour (pynfam/strength/contour.py:212-282):
a circle centred on the real axis between energy_min and energy_max,
Gauss-Legendre angles, and only the first (npts+1)//2 points computed (the
others follow from S(w*) = S(w)* on a closed contour).
"""
from __future__ import annotations

import numpy as np


def circle(energy_min: float, energy_max: float, npts: int, use_gauleg: bool = True,
           theta_init: float = 0.0, max_height: float = np.inf) -> np.ndarray:
    if use_gauleg:
        theta, _ = np.polynomial.legendre.leggauss(npts)
        t1 = theta_init + 2.0 * np.pi
        theta = theta * 0.5 * (t1 - theta_init) + 0.5 * (theta_init + t1)
    else:
        theta = np.linspace(theta_init, theta_init + 2.0 * np.pi, npts)
    r0 = 0.5 * (energy_max + energy_min)
    r = energy_max - r0
    if r > max_height:
        z = r0 + r * np.cos(theta) + max_height * np.sin(theta) * 1j
    else:
        z = r0 + r * np.exp(1j * theta)
    ncomp = (npts + 1) // 2
    if use_gauleg and abs(np.mod(theta_init, np.pi)) > 1e-10:
        ncomp = npts
    return z[:ncomp]
