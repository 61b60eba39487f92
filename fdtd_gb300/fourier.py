"""Frequency-domain post-processing of detector records (API of fdtd/fourier.py).

``FrequencyRoutines(grid, objs)`` takes the same inputs as the reference
(fdtd/fourier.py:17-50): a plain array, a LineDetector/BlockDetector, a
CurrentDetector, a SoftArbitraryPointSource, or a (detector,
current_detector) tuple for ``impedance``.  It selects the same record slices
as the reference, pads with the last value to the same length
(fdtd/fourier.py:51-120), and transforms with ``torch.fft`` on the device the
records live on, returning torch tensors (as the reference does on its torch
backends).  The reference's selections are kept as they are: ``FFT`` of a
line or block detector transforms ``E[:][0][0][0]`` (one index of the first
record, the reference's FIXME; for a block detector that is a (z, component)
array, padded along its first axis and transformed along its last one, as
numpy.pad and numpy.fft.fft do there), and ``impedance`` divides the spectra
where the current spectrum is non-zero, zero elsewhere.

One difference: with ``freq_window_tuple`` the reference's
``compute_frequencies`` reads undefined names and raises NameError
(fdtd/fourier.py:134-137); here it picks the bins closest to the window ends.
"""

from math import ceil

import numpy as np
import torch

from .detectors import BlockDetector, CurrentDetector, LineDetector
from .sources import SoftArbitraryPointSource


def _as_tensor(data, device):
    if torch.is_tensor(data):
        return data.to(device=device, dtype=torch.float64)
    if isinstance(data, (list, tuple)) and data and torch.is_tensor(data[0]):
        return torch.stack([d.to(torch.float64) for d in data]).to(device)
    return torch.as_tensor(np.asarray(data, dtype=np.float64), device=device)


def _pad_edge(x, n):
    """numpy.pad(x, (0, n), 'edge') along the first axis."""
    if n <= 0:
        if n < 0:
            raise ValueError("index can't contain negative values")
        return x
    return torch.cat([x, x[-1:].expand((n,) + tuple(x.shape[1:]))], 0)


class FrequencyRoutines:
    """FFT and impedance of detector records (fdtd/fourier.py:17-260)."""

    def __init__(self, grid, objs):
        self.grid = grid
        self.objs = objs

    def _device(self):
        return getattr(self.grid, "_device", "cpu")

    def compute_padding(self, input_data, dt, freq_window_tuple=None, fft_num_bins_in_window=None,
                        fft_bin_freq_resolution=None):
        """Padding that gives the requested bin resolution (fdtd/fourier.py:51-120);
        returns (required_padding, end_time)."""
        input_length = input_data.shape[0]
        if freq_window_tuple is None:
            begin_freq = 0
            end_freq = (input_length / 2.0) / (dt * input_length)
        else:
            begin_freq, end_freq = freq_window_tuple
        end_time = input_length * dt
        if fft_num_bins_in_window is None and fft_bin_freq_resolution is not None:
            fft_num_bins_in_window = (begin_freq - end_freq) / fft_bin_freq_resolution
        elif not (fft_num_bins_in_window or fft_bin_freq_resolution):
            fft_num_bins_in_window = input_data.shape[0]
        waveform_frequency_resolution = 1.0 / end_time
        fft_bin_resolution = (1.0 / dt) / fft_num_bins_in_window
        print("Waveform data has an intrinsic resolution of: {:.2E} Hz".format(waveform_frequency_resolution))
        print("FFT bin: {:.2E} Hz".format(fft_bin_resolution))
        required_padding = ceil(fft_num_bins_in_window / ((end_freq - begin_freq) * dt)) - input_length
        return required_padding, end_time

    def compute_frequencies(self, length_with_padding, dt, freq_window_tuple=None):
        """Bin frequencies and the index range of the window (fdtd/fourier.py:122-139)."""
        spectrum_freqs = torch.fft.fftfreq(length_with_padding, d=dt, dtype=torch.float64, device=self._device())
        if freq_window_tuple is None:
            begin_freq_idx = 0
            end_freq_idx = -1
        else:
            begin_freq, end_freq = freq_window_tuple
            begin_freq_idx = int(torch.abs(spectrum_freqs - begin_freq).argmin())
            end_freq_idx = int(torch.abs(spectrum_freqs - end_freq).argmin())
        return spectrum_freqs, begin_freq_idx, end_freq_idx

    def export_touchstone_s2p(self):
        raise NotImplementedError

    def S_parameters(self, waveform=None, node=None):
        raise NotImplementedError

    def FFT(self, freq_window_tuple=None, fft_num_bins_in_window=None, fft_bin_freq_resolution=None):
        """Spectrum of one record series (fdtd/fourier.py:172-212)."""
        if self.grid.time_steps_passed == 0:
            return [], []
        o = self.objs
        if isinstance(o, (np.ndarray, list)) or torch.is_tensor(o):
            input_data = o
        elif isinstance(o, (LineDetector, BlockDetector)):
            input_data = o.E[:][0][0][0]
        elif isinstance(o, SoftArbitraryPointSource):
            input_data = o.source_voltage[:][0][0][0]
        elif isinstance(o, CurrentDetector):
            input_data = o.I[:][0][0][0]
        else:
            raise ValueError("Sorry, FFT can't yet interpret the argument given.")
        input_data = _as_tensor(input_data, self._device())
        required_padding, _ = self.compute_padding(input_data, self.grid.time_step,
                                                   freq_window_tuple=freq_window_tuple,
                                                   fft_num_bins_in_window=fft_num_bins_in_window,
                                                   fft_bin_freq_resolution=fft_bin_freq_resolution)
        input_data = _pad_edge(input_data, required_padding)
        spectrum = torch.fft.fft(input_data)  # last axis, like numpy.fft.fft
        freqs, b, e = self.compute_frequencies(input_data.shape[0], self.grid.time_step,
                                               freq_window_tuple=freq_window_tuple)
        return freqs[b:e], spectrum[b:e]

    def impedance(self, freq_window_tuple=None, fft_num_bins_in_window=None, fft_bin_freq_resolution=None):
        """Voltage spectrum over current spectrum (fdtd/fourier.py:216-260)."""
        if self.grid.time_steps_passed == 0:
            return [], []
        o = self.objs
        dev = self._device()
        if isinstance(o, SoftArbitraryPointSource):
            voltage_array = _as_tensor(o.source_voltage, dev)
            current_array = o.current_detector.I.tensor().to(device=dev, dtype=torch.float64)
        elif (isinstance(o, tuple) and isinstance(o[0], (BlockDetector, LineDetector))
              and isinstance(o[1], CurrentDetector)):
            voltage_array = o[0].E.tensor().to(device=dev, dtype=torch.float64)[:][0, 0, 0]
            current_array = o[1].I.tensor().to(device=dev, dtype=torch.float64)
        else:
            raise ValueError("Sorry, FFT can't yet interpret the argument given.")
        required_padding, _ = self.compute_padding(voltage_array, self.grid.time_step,
                                                   freq_window_tuple=freq_window_tuple,
                                                   fft_num_bins_in_window=fft_num_bins_in_window,
                                                   fft_bin_freq_resolution=fft_bin_freq_resolution)
        voltage_array = voltage_array.reshape(self.grid.time_steps_passed)
        current_array = current_array.reshape(self.grid.time_steps_passed)
        voltage_array = _pad_edge(voltage_array, required_padding)
        current_array = _pad_edge(current_array, required_padding)
        voltage_spectrum = torch.fft.fft(voltage_array)
        current_spectrum = torch.fft.fft(current_array)
        nonzero = current_spectrum != 0
        impedance_spectrum = torch.where(nonzero, voltage_spectrum / torch.where(nonzero, current_spectrum, 1),
                                         torch.zeros_like(voltage_spectrum))
        freqs, b, e = self.compute_frequencies(voltage_array.shape[0], self.grid.time_step,
                                               freq_window_tuple=freq_window_tuple)
        return freqs[b:e], impedance_spectrum[b:e]
