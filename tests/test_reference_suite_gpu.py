"""The reference's own detector, source and FFT tests, run on the GB300 backend.

Mirrors tests/test_detectors.py:32-107, tests/test_sources.py:14-15 and
tests/test_fft.py:37-59 of the reference (its `grid` fixture: 10^3 cells,
100 nm, vacuum).  Where the reference test only checks shapes or that the call
works, the time histories are also compared with the CPU oracle run in the
same process (float64, bit for bit).
"""

import numpy as np
import pytest
import torch

from oracle import fdtd_oracle as fo

pytestmark = pytest.mark.gpu

X_, Y_, Z_ = 4, 4, 4


def _grid(mod):
    return mod.Grid(shape=(10, 10, 10), grid_spacing=100e-9, permittivity=1.0, permeability=1.0)


def _dc_absorbing(mod, n):
    """tests/test_detectors.py:32-88: absorbing block around a point driven by
    writing a Gaussian pulse into E_z between the half steps, with a
    CurrentDetector and a single-point BlockDetector on the point."""
    grid = _grid(mod)
    grid[0:2, :, :] = mod.PML(name="PML")
    grid[X_ - 1:X_ + 1, Y_ - 1:Y_ + 1, Z_ - 1:Z_ + 1] = mod.AbsorbingObject(permittivity=1.0, conductivity=1e9)
    grid[X_, Y_, Z_] = mod.CurrentDetector(name="Dave")
    grid[X_:X_, Y_:Y_, Z_:Z_] = mod.BlockDetector()
    for _ in range(n):
        grid.update_E()
        t = grid.time_steps_passed * grid.time_step
        sigma = ((n / 10.0) * grid.time_step) / (2.0 * np.sqrt(2.0 * np.log(2)))
        grid.E[X_, Y_, Z_, 2] = float(np.exp(-((t - (n / 2) * grid.time_step) ** 2.0) / (2.0 * sigma ** 2.0)))
        grid.update_H()
        grid.time_steps_passed += 1
    return grid


def test_dc_absorbing_current_detector(fd):
    fd.set_backend("gb300.float64")
    n = 200
    g, o = _dc_absorbing(fd, n), _dc_absorbing(fo, n)
    cur = np.asarray(g.detectors[0].I).reshape(n)
    ocur = np.array(o.detectors[0].I).reshape(n)
    e = np.asarray(g.detectors[1].E).reshape(n, 3)[:, 2]
    oe = np.array(o.detectors[1].E).reshape(n, 3)[:, 2]
    assert np.array_equal(cur, ocur) and np.array_equal(e, oe)
    assert np.abs(cur).max() > 0.0


def test_current_detector_shape(fd):
    """tests/test_detectors.py:91-100."""
    fd.set_backend("gb300.float64")
    grid = _grid(fd)
    edetector = fd.BlockDetector()
    cdetector = fd.CurrentDetector()
    grid[4, 4, 4] = cdetector
    grid[4, 4, 5] = edetector
    grid.run(10, progress_bar=False)
    assert np.asarray(cdetector.I).shape[0:2] == np.asarray(edetector.E).shape[0:2]
    assert np.asarray(cdetector.I).shape[0] == 10


def test_saps_registers_its_current_detector(fd):
    """tests/test_detectors.py:103-107 and tests/test_sources.py:14-15."""
    fd.set_backend("gb300.float64")
    grid = _grid(fd)
    source = fd.SoftArbitraryPointSource(torch.zeros(1), impedance=50.0)
    grid[4, 4, 4] = source
    grid.run(100, progress_bar=False)
    assert isinstance(grid.detectors[0], fd.CurrentDetector)
    assert len(source.source_voltage) == 100 and len(grid.detectors[0].I) == 100


def test_fft_of_a_block_detector(fd):
    """tests/test_fft.py:37-50."""
    fd.set_backend("gb300.float64")
    grid = _grid(fd)
    detector = fd.BlockDetector()
    grid[4, 4, 4] = detector
    assert fd.FrequencyRoutines(grid, detector).FFT() == ([], [])
    grid[4, 4, 4] = fd.PointSource(period=20, name="src")
    grid.run(100, progress_bar=False)
    freqs, spectrum = fd.FrequencyRoutines(grid, detector).FFT()
    # the reference transforms E[:][0][0][0]: the (z, component) array of the
    # first record, padded to 2 rows and transformed along its last axis
    assert tuple(spectrum.shape) == (1, 3) and tuple(freqs.shape) == (1,)
    rec = torch.as_tensor(np.asarray(detector.E)[0, 0, 0], dtype=torch.float64)
    want = np.fft.fft(np.pad(rec.numpy(), ((0, 1), (0, 0)), "edge"))[0:-1]
    assert np.allclose(spectrum.cpu().numpy(), want, rtol=1e-12, atol=0.0)


def test_saps_impedance_runs(fd):
    """tests/test_fft.py:53-57: a source with a zero waveform gives zero
    spectra, and the impedance is zero where the current spectrum is zero."""
    fd.set_backend("gb300.float64")
    grid = _grid(fd)
    source = fd.SoftArbitraryPointSource(np.zeros(1), impedance=50.0)
    grid[4, 4, 4] = source
    grid.run(100, progress_bar=False)
    freqs, z = fd.FrequencyRoutines(grid, source).impedance()
    assert z.shape == freqs.shape and torch.all(z == 0)
