"""Detectors (API of fdtd/detectors.py) plus plane and DFT detectors.

Detector samples are written by a gather kernel, after every half step, into a
device trace buffer owned by the grid's engine.  ``det.E`` / ``det.H`` keep the
reference's list semantics (one record per step, ``len``, indexing, iteration;
fdtd/detectors.py:114-124, 241-265) through ``TraceList``, a read-only
sequence of device tensors; ``.tensor()`` stacks them without a host copy and
``numpy.asarray(det.E)`` gives the host array.

Record shapes: LineDetector (points, 3); BlockDetector (nx+1, ny+1, nz+1, 3)
over INCLUSIVE index ranges as in fdtd/detectors.py:236-239 (the array form of
the reference's nested lists); PlaneDetector (nx, ny, nz, 3) over the
half-open box.  DFTPlaneDetector accumulates a running DFT instead.
"""

import collections.abc

import numpy as np
import torch

from . import constants as const


class TraceList(collections.abc.Sequence):
    """Per-step records of one detector field, read-only list semantics."""

    def __init__(self, det, field):
        self._det = det
        self._field = field

    def _chunks(self):
        det = self._det
        chunks = list(det._frozen[self._field])
        eng = det._engine
        if eng is not None:
            live = eng.detector_records(det, self._field)
            if live is not None and live.shape[0]:
                chunks.append(live)
        return chunks

    def __len__(self):
        return sum(c.shape[0] for c in self._chunks())

    def __getitem__(self, idx):
        if isinstance(idx, slice):
            return [self[i] for i in range(*idx.indices(len(self)))]
        n = len(self)
        if idx < 0:
            idx += n
        if not 0 <= idx < n:
            raise IndexError("detector record index out of range")
        for c in self._chunks():
            if idx < c.shape[0]:
                return c[idx]
            idx -= c.shape[0]
        raise IndexError(idx)

    def tensor(self):
        """All records stacked as one tensor of shape (steps, *record)."""
        chunks = self._chunks()
        if not chunks:
            return torch.zeros((0,) + self._det._rec_shape)
        return chunks[0].clone() if len(chunks) == 1 else torch.cat(chunks, 0)

    def tensor_tail(self, n):
        """The last n records as one tensor: a view of the device trace buffer
        when they were all written since the last plan rebuild."""
        chunks = self._chunks()
        if chunks and chunks[-1].shape[0] >= n:
            return chunks[-1][chunks[-1].shape[0] - n:]
        return self.tensor()[len(self) - n:]

    def numpy(self):
        return self.tensor().detach().cpu().numpy()

    def __array__(self, dtype=None, copy=None):
        a = self.numpy()
        return a if dtype is None else a.astype(dtype)

    def __repr__(self):
        return f"TraceList({self._det.__class__.__name__}.{self._field}, {len(self)} records)"


class _Detector:
    def __init__(self, name=None):
        self.grid = None
        self.name = name
        self._frozen = {"E": [], "H": []}
        self._engine = None
        self.E = TraceList(self, "E")
        self.H = TraceList(self, "H")

    def _register_name(self, grid):
        if self.name is not None:
            if hasattr(grid, self.name):
                raise ValueError(f"The grid already has an attribute with name {self.name}")
            setattr(grid, self.name, self)

    def _finish_register(self, grid):
        self._register_name(grid)
        self.grid = grid
        grid.detectors.append(self)
        grid._invalidate()

    def _probe_cells(self):
        """Linear cell indices (numpy int64) sampled by this detector."""
        xs, ys, zs = (np.asarray(v, dtype=np.int64).reshape(-1) for v in self._point_lists())
        n = self.grid.shape
        for v, m in zip((xs, ys, zs), n):
            if v.size and (v.min() < -m or v.max() >= m):
                raise IndexError(f"{self.__class__.__name__} index outside the grid of size {n}")
        xs, ys, zs = xs % n[0], ys % n[1], zs % n[2]
        return (xs * n[1] + ys) * n[2] + zs

    def detector_values(self):
        """Outputs of the detector, {'E': records, 'H': records}."""
        return {"E": self.E, "H": self.H}

    def __repr__(self):
        return f"{self.__class__.__name__}(name={repr(self.name)})"


class LineDetector(_Detector):
    """Samples E and H along the diagonal of a box (fdtd/detectors.py:20-140)."""

    @staticmethod
    def _all_lists(x, y, z):
        if isinstance(x, list) and isinstance(y, list) and isinstance(z, list):
            if len(x) != len(y) or len(y) != len(z) or len(z) != len(x):
                raise IndexError("sources require grid to be indexed with slices or equal length list-indices")
            return True
        return False

    @staticmethod
    def _ranges(grid, x, y, z):
        """Start and stop per axis; a list index [a, ..., b] counts as a:b
        (fdtd/detectors.py:89-105)."""
        conv = []
        for s in (x, y, z):
            if isinstance(s, list):
                s = slice(s[0], s[-1], None)
            conv.append(s)
        lo = [s.start if s.start is not None else 0 for s in conv]
        hi = [s.stop if s.stop is not None else n for s, n in zip(conv, grid.shape)]
        return lo, hi

    def _register_grid(self, grid, x, y, z):
        if self._all_lists(x, y, z):
            self.x, self.y, self.z = list(x), list(y), list(z)
        else:
            lo, hi = self._ranges(grid, x, y, z)
            m = max(abs(h - l) for l, h in zip(lo, hi))
            self.x, self.y, self.z = ([int(v) for v in np.array(np.linspace(l, h, m, endpoint=False), np.int64)]
                                      for l, h in zip(lo, hi))
        self._rec_shape = (len(self.x), 3)
        self._finish_register(grid)

    def _point_lists(self):
        return self.x, self.y, self.z

    def __str__(self):
        s = "    " + repr(self) + "\n"
        if self.x:
            s += (f"        @ x=[{self.x[0]}, ... , {self.x[-1]}], y=[{self.y[0]}, ... , {self.y[-1]}], "
                  f"z=[{self.z[0]}, ... , {self.z[-1]}]\n")
        return s


class BlockDetector(LineDetector):
    """Samples E and H on an inclusive index block (fdtd/detectors.py:146-281)."""

    def _register_grid(self, grid, x, y, z):
        if self._all_lists(x, y, z):
            self.x, self.y, self.z = list(x), list(y), list(z)
        else:
            lo, hi = self._ranges(grid, x, y, z)
            self.x, self.y, self.z = ([int(v) for v in np.arange(l, h + 1)] for l, h in zip(lo, hi))
        self._rec_shape = (len(self.x), len(self.y), len(self.z), 3)
        self._finish_register(grid)

    def _point_lists(self):
        X, Y, Z = np.meshgrid(np.asarray(self.x, np.int64), np.asarray(self.y, np.int64),
                              np.asarray(self.z, np.int64), indexing="ij")
        return X, Y, Z


def _half_open_box(grid, x, y, z):
    out = []
    for s, n in zip((x, y, z), grid.shape):
        if isinstance(s, list):
            if len(s) != 1:
                raise IndexError("use slices or single indices for a plane detector")
            i = s[0] + n if s[0] < 0 else s[0]
            if not 0 <= i < n:
                raise IndexError(f"plane detector index {s[0]} outside the grid")
            out.append(slice(i, i + 1))
        else:
            a0, a1, step = s.indices(n)
            if step != 1 or a1 <= a0:
                raise IndexError("a plane detector needs a non-empty unit-step range")
            out.append(slice(a0, a1))
    return tuple(out)


class PlaneDetector(_Detector):
    """Records E[box] after every E half step and H[box] after every H half step
    (not in the reference).  The box is half-open, usually one cell thick;
    each record has shape (nx, ny, nz, 3)."""

    def _register_grid(self, grid, x, y, z):
        self.x, self.y, self.z = _half_open_box(grid, x, y, z)
        self._rec_shape = (self.x.stop - self.x.start, self.y.stop - self.y.start,
                           self.z.stop - self.z.start, 3)
        self._finish_register(grid)

    def _point_lists(self):
        return np.meshgrid(np.arange(self.x.start, self.x.stop), np.arange(self.y.start, self.y.stop),
                           np.arange(self.z.start, self.z.stop), indexing="ij")


class DFTPlaneDetector(_Detector):
    """Running discrete Fourier transform of E on a half-open box (not in the
    reference).  After every E half step at step index q (time q*dt):

        dft[f] += E[box] * exp(-2j*pi*frequencies[f]*q*dt)

    accumulated in float64 (complex128) on the device whatever the field
    precision.  Give ``frequencies`` in Hz or ``wavelengths`` in metres."""

    def __init__(self, frequencies=None, wavelengths=None, name=None):
        super().__init__(name=name)
        if (frequencies is None) == (wavelengths is None):
            raise ValueError("give exactly one of frequencies or wavelengths")
        if wavelengths is not None:
            frequencies = [const.c / float(w) for w in np.atleast_1d(wavelengths)]
        self.frequencies = [float(f) for f in np.atleast_1d(frequencies)]

    def _register_grid(self, grid, x, y, z):
        self.x, self.y, self.z = _half_open_box(grid, x, y, z)
        self._rec_shape = (self.x.stop - self.x.start, self.y.stop - self.y.start,
                           self.z.stop - self.z.start, 3)
        self.dft = torch.zeros((len(self.frequencies),) + self._rec_shape, dtype=torch.complex128,
                               device=grid._device)
        self._finish_register(grid)

    def reset(self):
        """Clear the accumulated transform."""
        self.dft.zero_()

    def detector_values(self):
        """Outputs of the detector, {'dft': (frequencies, *box, 3) complex128}."""
        return {"dft": self.dft}


class CurrentDetector(_Detector):
    """Current around a point after every H half step (fdtd/detectors.py:284-496).

    For every point of the index block (inclusive ranges like BlockDetector)
    the device computes the reference's ``single_point_current``: the loop
    integral of H around the z edge in the planes z and z-1, averaged, with the
    reference's arithmetic order (including its running sum of the second
    y term) and Python's wrap-around of the index -1.  ``det.I`` holds one
    record per step of shape (nx, ny, nz) (the array form of the reference's
    nested lists)."""

    def __init__(self, name=None):
        super().__init__(name=name)
        del self.E, self.H
        self._frozen = {"I": []}
        self.orientation = None
        self.I = TraceList(self, "I")

    def _register_grid(self, grid, x, y, z):
        if LineDetector._all_lists(x, y, z):
            self.x, self.y, self.z = list(x), list(y), list(z)
        else:
            lo, hi = LineDetector._ranges(grid, x, y, z)
            self.x, self.y, self.z = ([int(v) for v in np.arange(l, h + 1)] for l, h in zip(lo, hi))
        self._rec_shape = (len(self.x), len(self.y), len(self.z))
        self._finish_register(grid)

    def _point_lists(self):
        return np.meshgrid(np.asarray(self.x, np.int64), np.asarray(self.y, np.int64),
                           np.asarray(self.z, np.int64), indexing="ij")

    def single_point_current(self, px, py, pz):
        """The current around the z edge at (px, py, pz) from the grid's
        present H (fdtd/detectors.py:404-464), with the reference's operation
        order, its running sum of the second y term and Python's wrap-around of
        index -1; a 0-d tensor.  The time step computes the same on the
        device for every point of the detector."""
        H, du = self.grid.H, self.grid.grid_spacing
        cv1 = (H[px, py - 1, pz, 0] - H[px, py, pz, 0]) * du
        cv2 = (H[px, py, pz, 1] - H[px - 1, py, pz, 1]) * du
        c1 = cv1 + cv2
        cv1 = (H[px, py - 1, pz - 1, 0] - H[px, py, pz - 1, 0]) * du
        cv2 = cv2 + (H[px, py, pz - 1, 1] - H[px - 1, py, pz - 1, 1]) * du
        c2 = cv1 + cv2
        return (c1 + c2) / 2.0

    def detector_values(self):
        """Outputs of the detector, {'I': records}."""
        return {"I": self.I}

    def __str__(self):
        return (f"    {repr(self)}\n        @ x=[{self.x[0]}, ... , {self.x[-1]}], y=[{self.y[0]}, ... , "
                f"{self.y[-1]}], z=[{self.z[0]}, ... , {self.z[-1]}]\n")
