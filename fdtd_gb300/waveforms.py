"""Source waveforms evaluated on the host once per time step.

Same definitions as fdtd/waveforms.py:8-53; the time-step kernels receive the
resulting scalar per step in a waveform table.
"""

from math import cos, exp, log, sin, sqrt

import numpy as np


def hanning(f, t, n):
    """Sine at angular rate f under a raised-cosine window of n cycles."""
    return (1 / 2) * (1 - cos(f * t / n)) * (sin(f * t))


fwhm_constant = 2.0 * sqrt(2.0 * log(2))


def normalized_gaussian_pulse(x, fwhm, center=0.0):
    """Gaussian of unit peak with full width at half maximum ``fwhm``."""
    sigma = fwhm / fwhm_constant
    return np.exp(-(((x - center) ** 2.0) / (2.0 * (sigma ** 2.0))))


def normalized_gaussian_derivative_pulse(x, fwhm, center=0.0):
    """Derivative-of-Gaussian pulse scaled to unit peak."""
    sigma = fwhm / fwhm_constant
    return (exp((1.0 / 2.0) - ((x - center) ** 2.0) / (2.0 * sigma ** 2.0)) * (x - center)) / sigma
