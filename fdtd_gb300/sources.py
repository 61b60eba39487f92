"""Sources (API of fdtd/sources.py).

The waveform of every source is evaluated on the host once per time step with
the reference's own expressions (Python floats) and handed to the kernels in a
per-step table; the kernels apply ``weight * value`` per point:

    PointSource    soft, E_z += amplitude * sin(2 pi q / period + phase)   (or the
                   Hanning pulse), fdtd/sources.py:93-109
    LineSource     soft, E_z[p] += profile[p] * sin(...) per point, points
                   applied in order (a repeated point adds twice),
                   fdtd/sources.py:278-297
    PlaneSource    hard, E[pol] = amplitude * sin(...) and H[Hpol] = the same
                   value on the plane, fdtd/sources.py:476-486
    GaussianPlaneSource (not in the reference) hard like PlaneSource with a
                   Gaussian envelope, see its docstring.

``period`` is converted to whole time steps at registration (int(T/dt + 0.5)),
as in fdtd/grid.py:177-181.
"""

from math import pi, sin

import numpy as np

from .waveforms import hanning, normalized_gaussian_pulse


class _Source:
    _hard = False

    def _register_name(self, grid):
        if self.name is not None:
            if hasattr(grid, self.name):
                raise ValueError(f"The grid already has an attribute with name {self.name}")
            setattr(grid, self.name, self)

    def __repr__(self):
        return (f"{self.__class__.__name__}(period={self.period}, amplitude={self.amplitude}, "
                f"phase_shift={self.phase_shift}, name={repr(self.name)})")


class _PulsedWave(_Source):
    def _init_wave(self, period, amplitude, phase_shift, name, pulse, cycle, hanning_dt):
        self.grid = None
        self.period = period
        self.amplitude = amplitude
        self.phase_shift = phase_shift
        self.name = name
        self.pulse = pulse
        self.cycle = cycle
        self.frequency = 1.0 / period
        self.hanning_dt = hanning_dt if hanning_dt is not None else 0.5 / self.frequency

    def _shape(self, q):
        """Unscaled waveform value at step q (sin or Hanning pulse)."""
        if self.pulse:
            t1 = int(2 * pi / (self.frequency * self.hanning_dt / self.cycle))
            if q < t1:
                return hanning(self.frequency, q * self.hanning_dt, self.cycle)
            return 0.0
        return sin(2 * pi * q / self.period + self.phase_shift)


class PointSource(_PulsedWave):
    """Soft source on a single cell, adding to E_z."""

    def __init__(self, period=15, amplitude: float = 1.0, phase_shift: float = 0.0, name: str = None,
                 pulse: bool = False, cycle: int = 5, hanning_dt: float = 10.0):
        self._init_wave(period, amplitude, phase_shift, name, pulse, cycle, hanning_dt)

    def _register_grid(self, grid, x, y, z):
        try:
            (x,), (y,), (z,) = x, y, z
        except (TypeError, ValueError):
            raise ValueError("a point source should be placed on a single grid cell.")
        xs, ys, zs = grid._handle_tuple((x, y, z))
        for v, n in zip((xs, ys, zs), grid.shape):
            if not -n <= v < n:
                raise IndexError(f"point source index {v} outside the grid")
        self._register_name(grid)
        self.grid = grid
        self.x, self.y, self.z = xs, ys, zs
        self.period = grid._handle_time(self.period)
        self.frequency = 1.0 / self.period
        grid.sources.append(self)
        grid._invalidate()

    def _value(self, q):
        return self.amplitude * self._shape(q)

    def _items(self):
        """[(field, kind, comp, lo, hi, weight)] with one column per source."""
        p = tuple(v % n for v, n in zip((self.x, self.y, self.z), self.grid.shape))
        return [("E", "soft", 2, p, tuple(v + 1 for v in p), 1.0)]

    def __str__(self):
        return "    " + repr(self) + "\n" + f"        @ x={self.x}, y={self.y}, z={self.z}\n"


class LineSource(_PulsedWave):
    """Soft source along the diagonal of a box with a Gaussian profile."""

    def __init__(self, period=15, amplitude: float = 1.0, phase_shift: float = 0.0, name: str = None,
                 pulse: bool = False, cycle: int = 5, hanning_dt: float = 10.0):
        self._init_wave(period, amplitude, phase_shift, name, pulse, cycle, hanning_dt)

    def _handle_slices(self, grid, x, y, z):
        if isinstance(x, list) and isinstance(y, list) and isinstance(z, list):
            if len(x) != len(y) or len(y) != len(z) or len(z) != len(x):
                raise IndexError("sources require grid to be indexed with slices or equal length list-indices")
            return ([grid._handle_distance(v) for v in x], [grid._handle_distance(v) for v in y],
                    [grid._handle_distance(v) for v in z])
        conv = []
        for s in (x, y, z):
            if isinstance(s, list):
                s = slice(grid._handle_distance(s[0]), grid._handle_distance(s[-1]), None)
            conv.append(s)
        lo = [grid._handle_distance(s.start if s.start is not None else 0) for s in conv]
        hi = [grid._handle_distance(s.stop if s.stop is not None else n) for s, n in zip(conv, grid.shape)]
        m = max(abs(h - l) for l, h in zip(lo, hi))
        if m < 2:
            raise ValueError("a LineSource should consist of at least two gridpoints")
        return tuple([int(v) for v in np.array(np.linspace(l, h, m, endpoint=False), np.int64)]
                     for l, h in zip(lo, hi))

    def _register_grid(self, grid, x, y, z):
        xs, ys, zs = self._handle_slices(grid, x, y, z)
        for pts, n in zip((xs, ys, zs), grid.shape):
            if any(not -n <= v < n for v in pts):
                raise IndexError("line source point outside the grid")
        self._register_name(grid)
        self.grid = grid
        self.x, self.y, self.z = xs, ys, zs
        self.period = grid._handle_time(self.period)
        self.frequency = 1.0 / self.period
        L = len(self.x)
        # squared distance to the middle point, then the Gaussian of its square
        # (fdtd/sources.py:197-207), normalised to sum 1 and scaled
        vect = np.array((np.array(self.x) - self.x[L // 2]) ** 2 + (np.array(self.y) - self.y[L // 2]) ** 2
                        + (np.array(self.z) - self.z[L // 2]) ** 2, np.float64)
        profile = np.exp(-(vect ** 2) / (2 * (0.5 * vect.max()) ** 2))
        profile /= profile.sum()
        profile *= self.amplitude
        self.profile = profile
        grid.sources.append(self)
        grid._invalidate()

    def _value(self, q):
        return self._shape(q)

    def _items(self):
        out = []
        for x, y, z, w in zip(self.x, self.y, self.z, np.asarray(self.profile, dtype=np.float64)):
            p = tuple(v % n for v, n in zip((x, y, z), self.grid.shape))
            out.append(("E", "soft", 2, p, tuple(v + 1 for v in p), float(w)))
        return out

    def __str__(self):
        return ("    " + repr(self) + "\n" + f"        @ x=[{self.x[0]}, ... , {self.x[-1]}], "
                f"y=[{self.y[0]}, ... , {self.y[-1]}], z=[{self.z[0]}, ... , {self.z[-1]}]\n")


class PlaneSource(_Source):
    """Hard source on a plane: overwrites one E and one H component."""

    _hard = True

    def __init__(self, period=15, amplitude: float = 1.0, phase_shift: float = 0.0, name: str = None,
                 polarization: str = "z"):
        self.grid = None
        self.period = period
        self.amplitude = amplitude
        self.phase_shift = phase_shift
        self.name = name
        self.polarization = polarization

    def _handle_slices(self, grid, x, y, z):
        out = []
        for s, n in zip((x, y, z), grid.shape):
            if not isinstance(s, slice):
                if isinstance(s, list):
                    (s,) = s
                s = slice(grid._handle_distance(s), grid._handle_distance(s) + 1, None)
            a0 = grid._handle_distance(s.start if s.start is not None else 0)
            a1 = grid._handle_distance(s.stop if s.stop is not None else n)
            out.append(slice(a0, a1) if a0 < a1 else (slice(a1, a0) if a0 > a1 else slice(a0, a0 + 1)))
        lengths = [s.stop - s.start for s in out]
        if lengths.count(0) > 0:
            raise ValueError("Given location for PlaneSource results in slices of length 0!")
        if lengths.count(1) == 0:
            raise ValueError("Given location for PlaneSource is not a 2D plane!")
        if lengths.count(1) > 1:
            raise ValueError("Given location for PlaneSource should have no more than one dimension in which "
                             "it's flat.\nUse a LineSource for lower dimensional sources.")
        epol = "xyz".index(self.polarization)
        if lengths[epol] == 1:
            raise ValueError("PlaneSource cannot be polarized perpendicular to the orientation of the plane.")
        flat, first, second = [(2, 1, 2), (2, 0, 2), (1, 0, 1)][epol]
        hpol = first if lengths[flat] == 1 else second
        return out, epol, hpol

    def _register_grid(self, grid, x, y, z):
        (xs, ys, zs), epol, hpol = self._handle_slices(grid, x, y, z)
        self._register_name(grid)
        self.grid = grid
        self.x, self.y, self.z = xs, ys, zs
        self._Epol, self._Hpol = epol, hpol
        self._register_period(grid)
        shape = (xs.stop - xs.start, ys.stop - ys.start, zs.stop - zs.start)
        self.profile = self.amplitude * np.ones(shape)
        grid.sources.append(self)
        grid._invalidate()

    def _register_period(self, grid):
        self.period = grid._handle_time(self.period)
        self.frequency = 1.0 / self.period

    def _value(self, q):
        return sin(2 * pi * q / self.period + self.phase_shift)

    def _items(self):
        prof = np.asarray(self.profile, dtype=np.float64)
        w = float(prof.flat[0])
        if not np.all(prof == w):
            raise NotImplementedError("the gb300 backend needs a uniform PlaneSource profile")
        # the numpy meaning of the slices (negative indices wrap, an empty range sets nothing)
        rng = [s.indices(n)[:2] for s, n in zip((self.x, self.y, self.z), self.grid.shape)]
        if any(b <= a for a, b in rng):
            return []
        lo, hi = tuple(a for a, _ in rng), tuple(b for _, b in rng)
        return [("E", "hard", self._Epol, lo, hi, w), ("H", "hard", self._Hpol, lo, hi, w)]

    def __repr__(self):
        return (f"{self.__class__.__name__}(period={self.period}, amplitude={self.amplitude}, "
                f"phase_shift={self.phase_shift}, name={repr(self.name)}, "
                f"polarization={repr(self.polarization)})")

    def __str__(self):
        return ("    " + repr(self) + "\n" + f"        @ x=[{self.x.start}, ... , {self.x.stop}], "
                f"y=[{self.y.start}, ... , {self.y.stop}], z=[{self.z.start}, ... , {self.z.stop}]\n")


class GaussianPlaneSource(PlaneSource):
    """Hard plane source with a Gaussian envelope (not in the reference).

    value(q) = amplitude * g(q dt) * sin(2 pi q dt / period + phase_shift),
    g = normalized_gaussian_pulse(t, fwhm, center) (unit peak).  Unlike
    PlaneSource the carrier period is not rounded to whole time steps, so a
    broadband pulse keeps its centre frequency.  ``period``, ``fwhm`` and
    ``center`` are in seconds (an int period counts time steps); defaults:
    fwhm = 4 periods, center = 2 fwhm.  E[pol] and H[Hpol] on the plane are
    overwritten with that value each step, like PlaneSource.
    """

    def __init__(self, period=15, amplitude: float = 1.0, phase_shift: float = 0.0, name: str = None,
                 polarization: str = "z", fwhm: float = None, center: float = None):
        super().__init__(period, amplitude, phase_shift, name, polarization)
        self.fwhm, self.center = fwhm, center

    def _register_period(self, grid):
        period_s = self.period * grid.time_step if isinstance(self.period, int) else float(self.period)
        super()._register_period(grid)
        self.period_s = period_s
        self.fwhm_s = 4.0 * period_s if self.fwhm is None else float(self.fwhm)
        self.center_s = 2.0 * self.fwhm_s if self.center is None else float(self.center)

    def _value(self, q):
        t = q * self.grid.time_step
        env = float(normalized_gaussian_pulse(t, self.fwhm_s, self.center_s))
        return env * sin(2 * pi * t / self.period_s + self.phase_shift)


class SoftArbitraryPointSource:
    """Voltage-driven point source with a current feedback loop
    (fdtd/sources.py:504-643).

    At every E half step q the device adds ``output / grid_spacing`` to E_z at
    the point, output = input + impedance * I (the impedance term only when
    impedance > 0), input = waveform_array[q] (0 past its end) and I the
    current its own CurrentDetector measured after the previous H half step
    (0 at step 0).  The current is read on the device, so the feedback costs
    no host round trip.  ``input_voltage`` and ``source_voltage`` give the
    reference's per-step records ``[[[v]]]``, rebuilt from the waveform and
    the detector's current records with the same float64 expressions.

    Registration differs from the reference in two ways: a failing
    registration leaves nothing in ``grid.sources`` (the reference appends
    first), and a named source names its detector ``<name>_I`` (the reference
    raises UnboundLocalError for a named source, fdtd/sources.py:592-595)."""

    def __init__(self, waveform_array, name: str = None, impedance: float = 0.0):
        self.grid = None
        self.name = name
        self.current_detector = None
        self.waveform_array = waveform_array
        self.impedance = impedance
        # E halves run so far, as runs [q0, n, frozen, r0]: step q0 + k used the
        # current record frozen + r0 + k (none at step 0 or for r0 + k < 0);
        # contiguous calls extend the last run, so stepping adds no entries
        self._runs = []

    def _register_grid(self, grid, x, y, z):
        from .detectors import CurrentDetector

        try:
            (x,), (y,), (z,) = x, y, z
        except (TypeError, ValueError):
            raise ValueError("a point source should be placed on a single grid cell.")
        if self.name is not None and hasattr(grid, self.name):
            raise ValueError(f"The grid already has an attribute with name {self.name}")
        self.x, self.y, self.z = grid._handle_tuple((x, y, z))
        self.grid = grid
        grid.sources.append(self)
        if self.name is not None:
            setattr(grid, self.name, self)
        self.current_detector = CurrentDetector(name=None if self.name is None else self.name + "_I")
        grid[x, y, z] = self.current_detector
        grid._invalidate()

    def _value(self, q):
        """input_voltage at step q (fdtd/sources.py:605-609)."""
        w = self.waveform_array
        return float(w[q]) if q < np.shape(w)[0] else 0.0

    def _items(self):
        return [("E", "feedback", 2, (self.x, self.y, self.z), (self.x + 1, self.y + 1, self.z + 1),
                 float(self.impedance))]

    def _note_steps(self, q0, n, frozen, r0):
        """Record n E halves from step q0 whose first used current record r0."""
        if self._runs:
            last = self._runs[-1]
            if q0 == last[0] + last[1] and frozen == last[2] and r0 == last[3] + last[1]:
                last[1] += n
                return
        self._runs.append([q0, n, frozen, r0])

    def _steps(self):
        """(step index, index of the current record it used or -1) per E half."""
        for q0, n, frozen, r0 in self._runs:
            for k in range(n):
                r = r0 + k
                yield q0 + k, (frozen + r if (q0 + k > 0 and r >= 0) else -1)

    def _voltages(self):
        ins, outs = [], []
        I = self.current_detector.I
        for q, r in self._steps():
            vin = self._value(q)
            cur = float(I[r].reshape(-1)[0]) if r >= 0 else 0.0
            vout = vin + self.impedance * cur if self.impedance > 0 else vin
            ins.append([[[vin]]])
            outs.append([[[vout]]])
        return ins, outs

    @property
    def input_voltage(self):
        """Per-step waveform input, [[[v]]] records (fdtd/sources.py:628)."""
        return self._voltages()[0]

    @property
    def source_voltage(self):
        """Per-step output voltage incl. the impedance term, [[[v]]] records
        (fdtd/sources.py:629)."""
        return self._voltages()[1]

    def __repr__(self):
        return f"{self.__class__.__name__}()"

    def __str__(self):
        return f"    {repr(self)}\n        @ x={self.x}, y={self.y}, z={self.z}\n"
