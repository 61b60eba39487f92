"""The FDTD grid (API of fdtd/grid.py:80-514) driving the GB300 kernels.

Construction, unit handling and ``grid[x, y, z] = component`` registration
keep the reference's semantics (fdtd/grid.py:90-223, 358-375).  The time step
(``run``, ``step``, ``update_E``, ``update_H``; fdtd/grid.py:250-325) is
executed by ``fdtd_gb300.engine.Engine``, which compiles the registered
components into one device plan and calls the C ABI.  Field arrays live on the
GPU in the backend precision as ``(Nx, Ny, Nz, 3)`` tensors; writing into them
between half steps works as in the reference.  There is no CPU time step: on a
machine without CUDA a grid can be built and inspected but stepping raises.
"""

import os
from datetime import datetime

import numpy as np
import torch

from . import constants as const
from .backend import backend as bd

# the per-component hooks the reference's Grid calls every half step
# (fdtd/grid.py:275-325); the fused time step replaces them
_STEP_HOOKS = ("update_phi_E", "update_phi_H", "update_E", "update_H", "detect_E", "detect_H")


def _curl(name, F):
    """A stand-alone curl through the C ABI (fdtd_curl_E / fdtd_curl_H) on the
    current CUDA stream; float32 stays float32, anything else runs in float64."""
    from . import _native

    if not torch.cuda.is_available():
        raise RuntimeError("the gb300 backend needs a CUDA device; this machine has none")
    t = torch.as_tensor(F)
    if t.dtype != torch.float32:
        t = t.to(torch.float64)
    if t.dim() != 4 or t.shape[-1] != 3:
        raise ValueError("the field must have the shape (Nx, Ny, Nz, 3)")
    t = t.to("cuda").contiguous()
    out = torch.empty_like(t)
    precision = _native.FLOAT32 if t.dtype == torch.float32 else _native.FLOAT64
    stream = torch.cuda.current_stream(t.device).cuda_stream
    nx, ny, nz, _ = t.shape
    _native.check(getattr(_native.load(), name)(precision, t.data_ptr(), out.data_ptr(), nx, ny, nz, stream), name)
    return out


def curl_E(E):
    """Forward-difference curl of E with the reference's edge rule: the
    difference is dropped on the last plane of its axis (fdtd/grid.py:29-51).
    Returns a CUDA tensor."""
    return _curl("fdtd_curl_E", E)


def curl_H(H):
    """Backward-difference curl of H with the reference's edge rule: the
    difference is dropped on the first plane of its axis (fdtd/grid.py:54-76).
    Returns a CUDA tensor."""
    return _curl("fdtd_curl_H", H)


class Grid:
    """The FDTD grid: fields, materials and the registered components."""

    def __init__(self, shape, grid_spacing: float = 155e-9, permittivity=1.0, permeability=1.0,
                 courant_number: float = None):
        self.grid_spacing = float(grid_spacing)
        self.Nx, self.Ny, self.Nz = self._handle_tuple(shape)
        self.D = int(self.Nx > 1) + int(self.Ny > 1) + int(self.Nz > 1)
        max_courant_number = float(self.D) ** (-0.5)
        if courant_number is None:
            self.courant_number = 0.99 * max_courant_number
        elif courant_number > max_courant_number:
            raise ValueError(f"courant_number {courant_number} too high for a {self.D}D simulation")
        else:
            self.courant_number = float(courant_number)
        self.time_step = self.courant_number * self.grid_spacing / const.c

        self.precision = bd.precision
        self._dtype = bd.float
        self._device = bd.device
        self._engine = None
        self._engine_key = None
        self._dirty = True
        shp = (self.Nx, self.Ny, self.Nz, 3)
        self._E = torch.zeros(shp, dtype=self._dtype, device=self._device)
        self._H = torch.zeros(shp, dtype=self._dtype, device=self._device)
        if bd.compensated:
            self._E_lo = torch.zeros(shp, dtype=self._dtype, device=self._device)
            self._H_lo = torch.zeros(shp, dtype=self._dtype, device=self._device)
        else:
            self._E_lo = self._H_lo = None
        self._inverse_permittivity = self._inverse_material(permittivity)
        self._inverse_permeability = self._inverse_material(permeability)

        self.time_steps_passed = 0
        self.sources = []
        self.boundaries = []
        self.detectors = []
        self.objects = []
        self.folder = None

    # --- materials and fields --------------------------------------------------
    def _inverse_material(self, value):
        """ones / value as an (Nx, Ny, Nz, 3) tensor (fdtd/grid.py:141-151),
        divided in float64 then stored in the grid precision."""
        shp = (self.Nx, self.Ny, self.Nz, 3)
        if torch.is_tensor(value) or isinstance(value, np.ndarray):
            if torch.is_tensor(value):
                t = value.detach().to(device=self._device, dtype=torch.float64)
            else:
                t = torch.as_tensor(value, dtype=torch.float64).to(self._device)
            if t.ndim == 3:
                t = t[:, :, :, None]
            inv = torch.broadcast_to(1.0 / t, shp)
        else:
            inv = torch.full(shp, 1.0 / float(value), dtype=torch.float64, device=self._device)
        return inv.to(self._dtype).contiguous()

    def _assign(self, current, value, name):
        """In-place assignment that keeps the device buffer the plan points to."""
        if torch.is_tensor(value):
            v = value.detach().to(device=self._device, dtype=self._dtype)
        else:
            v = torch.as_tensor(np.asarray(value, dtype=np.float64), device=self._device).to(self._dtype)
        current.copy_(torch.broadcast_to(v, current.shape))
        return current

    @property
    def E(self):
        """Electric field, (Nx, Ny, Nz, 3) device tensor (for float32c: the leading float part)."""
        return self._E

    @E.setter
    def E(self, value):
        self._assign(self._E, value, "E")
        if self._E_lo is not None:
            self._E_lo.zero_()

    @property
    def H(self):
        """Magnetic field, (Nx, Ny, Nz, 3) device tensor (for float32c: the leading float part)."""
        return self._H

    @H.setter
    def H(self, value):
        self._assign(self._H, value, "H")
        if self._H_lo is not None:
            self._H_lo.zero_()

    @property
    def inverse_permittivity(self):
        return self._inverse_permittivity

    @inverse_permittivity.setter
    def inverse_permittivity(self, value):
        self._assign(self._inverse_permittivity, value, "inverse_permittivity")

    @property
    def inverse_permeability(self):
        return self._inverse_permeability

    @inverse_permeability.setter
    def inverse_permeability(self, value):
        self._assign(self._inverse_permeability, value, "inverse_permeability")

    def field(self, name):
        """E or H including the float32c compensation term, as a float64 tensor."""
        hi = self._E if name == "E" else self._H
        lo = self._E_lo if name == "E" else self._H_lo
        out = hi.to(torch.float64)
        return out + lo.to(torch.float64) if lo is not None else out

    # --- unit handling, fdtd/grid.py:171-223 ----------------------------------
    def _handle_distance(self, distance) -> int:
        """transform a distance to an integer number of gridpoints"""
        if not isinstance(distance, int):
            return int(float(distance) / self.grid_spacing + 0.5)
        return distance

    def _handle_time(self, time) -> int:
        """transform a time value to an integer number of timesteps"""
        if not isinstance(time, int):
            return int(float(time) / self.time_step + 0.5)
        return time

    def _handle_tuple(self, shape):
        if len(shape) != 3:
            raise ValueError(f"invalid grid shape {shape}\ngrid shape should be a 3D tuple containing floats or ints")
        x, y, z = shape
        return self._handle_distance(x), self._handle_distance(y), self._handle_distance(z)

    def _handle_slice(self, s: slice) -> slice:
        conv = lambda v: self._handle_distance(v) if isinstance(v, float) else v
        return slice(conv(s.start), conv(s.stop), conv(s.step))

    def _handle_single_key(self, key):
        try:
            len(key)
            return [self._handle_distance(k) for k in key]
        except TypeError:
            if isinstance(key, slice):
                return self._handle_slice(key)
            return [self._handle_distance(key)]

    @property
    def x(self):
        return self.Nx * self.grid_spacing

    @property
    def y(self):
        return self.Ny * self.grid_spacing

    @property
    def z(self):
        return self.Nz * self.grid_spacing

    @property
    def shape(self):
        return (self.Nx, self.Ny, self.Nz)

    @property
    def time_passed(self) -> float:
        return self.time_steps_passed * self.time_step

    def __setitem__(self, key, attr):
        if not isinstance(key, tuple):
            x, y, z = key, slice(None), slice(None)
        elif len(key) == 1:
            x, y, z = key[0], slice(None), slice(None)
        elif len(key) == 2:
            x, y, z = key[0], key[1], slice(None)
        elif len(key) == 3:
            x, y, z = key
        else:
            raise KeyError("maximum number of indices for the grid is 3")
        hooks = [h for h in _STEP_HOOKS if callable(getattr(attr, h, None))]
        if hooks:
            # a component (e.g. a user subclass) that brings its own per-step
            # hooks cannot run inside the fused time step
            raise NotImplementedError(f"{type(attr).__name__} defines the per-step hook(s) {', '.join(hooks)}; "
                                      "the gb300 backend fuses the time step and does not call component hooks")
        attr._register_grid(grid=self, x=self._handle_single_key(x), y=self._handle_single_key(y),
                            z=self._handle_single_key(z))

    def _invalidate(self):
        self._dirty = True

    # --- time stepping, fdtd/grid.py:250-331 ----------------------------------
    def _ensure_engine(self):
        from .engine import Engine

        if self._engine is None:
            self._engine = Engine(self)
        else:
            self._engine.refresh()
        return self._engine

    def run(self, total_time, progress_bar: bool = True):
        """Run ``total_time`` steps (int) or seconds (float)."""
        if isinstance(total_time, float):
            total_time /= self.time_step
        n = int(total_time)
        if n <= 0:
            return
        eng = self._ensure_engine()
        bar = None
        if progress_bar:
            try:
                from tqdm import tqdm

                bar = tqdm(total=n)
            except ImportError:
                bar = None
        if bar is None:
            eng.run(n)
            eng.check_status()
            return
        chunk = max(1, n // 100)
        done = 0
        while done < n:
            m = min(chunk, n - done)
            eng.run(m)
            done += m
            bar.update(m)
        bar.close()
        eng.check_status()

    def step(self):
        """One E half step, one H half step, then time_steps_passed += 1."""
        self._ensure_engine().run(1)

    def update_E(self):
        """The E half step at the current time_steps_passed (no increment)."""
        self._ensure_engine().half("E")

    def update_H(self):
        """The H half step at the current time_steps_passed (no increment)."""
        self._ensure_engine().half("H")

    def reset(self):
        """Zero E and H and the step counter (PML auxiliaries are kept, like
        fdtd/grid.py:327-331)."""
        self._H *= 0.0
        self._E *= 0.0
        if self._E_lo is not None:
            self._E_lo.zero_()
            self._H_lo.zero_()
        self.time_steps_passed *= 0

    def field_stats(self):
        """Health check of the fields: sum of squares, max |value| and the count
        of non-finite values, computed on the device."""
        return self._ensure_engine().stats()

    # --- representation ---------------------------------------------------------
    def __repr__(self):
        return (f"{self.__class__.__name__}(shape=({self.Nx},{self.Ny},{self.Nz}), "
                f"grid_spacing={self.grid_spacing:.2e}, courant_number={self.courant_number:.2f})")

    def __str__(self):
        s = repr(self) + "\n"
        if self.sources:
            s += "\nsources:\n" + "".join(str(src) for src in self.sources)
        if self.detectors:
            s += "\ndetectors:\n" + "".join(str(det) for det in self.detectors)
        if self.boundaries:
            s += "\nboundaries:\n" + "".join(str(bnd) for bnd in self.boundaries)
        if self.objects:
            s += "\nobjects:\n" + "".join(str(obj) for obj in self.objects)
        return s

    # --- detector export (fdtd/grid.py:407-439, 490-514) -----------------------
    # --- plotting and complex fields: not part of this backend ------------------
    def visualize(self, *args, **kwargs):
        """fdtd/visualization.py:28-336 plots with matplotlib; this backend has no
        plotting (copy grid.E / grid.H to the host and plot them there)."""
        raise NotImplementedError("visualize is not part of the gb300 backend (no plotting)")

    def generate_video(self, delete_frames=False):
        """fdtd/grid.py:441-488 calls ffmpeg on plotted frames; not part of this backend."""
        raise NotImplementedError("generate_video is not part of the gb300 backend (no plotting)")

    def promote_dtypes_to_complex(self):
        """fdtd/grid.py:353-356: complex fields are not supported (and broken in
        the reference's boundaries, fdtd/boundaries.py:106-116)."""
        raise NotImplementedError("complex fields are not supported by the gb300 backend")

    def save_simulation(self, sim_name=None):
        """Create ``fdtd_output/fdtd_output_<timestamp> (<sim_name>)`` and remember it."""
        os.makedirs("fdtd_output", exist_ok=True)
        now = datetime.now()
        full = f"{now.year}-{now.month}-{now.day}-{now.hour}-{now.minute}-{now.second}"
        if sim_name is not None:
            full = full + " (" + sim_name + ")"
        self.folder = os.path.abspath(os.path.join("fdtd_output", "fdtd_output_" + full))
        self.full_sim_name = full
        os.makedirs(self.folder, exist_ok=True)
        return self.folder

    def save_data(self):
        """Write the detector records to ``detector_readings.npz`` in the folder
        of ``save_simulation`` (fdtd/grid.py:490-514), read straight from the
        device traces: for every detector the keys '<name> (E)' and
        '<name> (H)', each an array of shape (steps, *record).  Detectors
        without E/H records (the reference raises KeyError there) store their
        own outputs instead: a CurrentDetector '<name> (I)', a DFTPlaneDetector
        '<name> (dft)'."""
        if self.folder is None:
            raise Exception("Save location not initialized. Please read about "
                            "'fdtd.Grid.saveSimulation()' or try running 'grid.saveSimulation()'.")
        dic = {}
        for det in self.detectors:
            vals = det.detector_values()
            keys = ("E", "H") if ("E" in vals or "H" in vals) else tuple(vals)
            for key in keys:
                v = vals[key]
                dic[f"{det.name} ({key})"] = v.detach().cpu().numpy() if hasattr(v, "detach") else np.asarray(v)
        np.savez(os.path.join(self.folder, "detector_readings"), **dic)
