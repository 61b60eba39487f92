"""FrequencyRoutines (fdtd/fourier.py) against the reference's own outputs.

Fixture tests/golden/ref_saps_fourier.npz (tests/golden/make_golden.py): the
reference's FFT of a plain array, the impedance of the SoftArbitraryPointSource
of the 'saps' golden scene and the FFT of its CurrentDetector, after 60 steps.
"""

import os

import numpy as np
import pytest
import torch

import golden_scenes
from helpers import rel_l2

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_padding_matches_reference_rule(fd):
    """tests/test_fft.py:17-33: 1000 samples at 1 ns; the reference returns
    (1001, 1.0000000000000002e-06) (ceil of 2000 plus round-off)."""
    g = fd.Grid((4, 4, 4))
    fr = fd.FrequencyRoutines(g, None)
    pad, end_time = fr.compute_padding(torch.zeros(1000, dtype=torch.float64), dt=1e-9)
    assert (pad, end_time) == (1001, 1.0000000000000002e-06)


def test_fft_of_an_array_matches_reference(fd):
    ref = np.load(os.path.join(GOLDEN, "ref_saps_fourier.npz"))
    fd.set_backend("gb300.float64")
    grid, steps, _ = golden_scenes.SCENES["saps"](fd)
    grid.time_steps_passed = steps
    f, s = fd.FrequencyRoutines(grid, ref["arr"]).FFT()
    assert rel_l2(f, ref["arr_freqs"]) <= 1e-15
    assert rel_l2(s.real, ref["arr_fft"].real) <= 1e-12 and rel_l2(s.imag, ref["arr_fft"].imag) <= 1e-12
    assert fd.FrequencyRoutines(fd.Grid((4, 4, 4)), ref["arr"]).FFT() == ([], [])  # nothing run yet


@pytest.mark.gpu
@pytest.mark.parametrize("precision, tol", [("float64", 1e-10), ("float32", 1e-3)])
def test_impedance_and_current_fft_match_reference(fd, precision, tol):
    ref = np.load(os.path.join(GOLDEN, "ref_saps_fourier.npz"))
    fd.set_backend("gb300." + precision)
    grid, steps, drive = golden_scenes.SCENES["saps"](fd)
    drive(grid, steps)
    src = grid.sources[0]
    f, z = fd.FrequencyRoutines(grid, src).impedance()
    assert rel_l2(f, ref["imp_freqs"]) <= 1e-15
    assert rel_l2(torch.view_as_real(z), np.stack([ref["imp"].real, ref["imp"].imag], -1)) <= tol
    f, s = fd.FrequencyRoutines(grid, grid.current).FFT()
    assert rel_l2(f, ref["cur_freqs"]) <= 1e-15
    assert rel_l2(torch.view_as_real(s), np.stack([ref["cur_fft"].real, ref["cur_fft"].imag], -1)) <= tol
