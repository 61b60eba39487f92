"""Boundaries: PML slabs and periodic boundaries (API of fdtd/boundaries.py).

Registration (``grid[...] = PML()``) keeps the reference's placement rules and
errors (fdtd/boundaries.py:295-365): a PML must be indexed with slices that
touch a grid border and always spans the full cross-section of its side; a
periodic boundary is a single index 0 or -1.

Storage differs from the reference: a slab normal to axis ``n`` has only two
auxiliaries per half step that can be non-zero (the psi of the two tangential
field components along ``n``; every other psi has zero conductivity and
therefore a zero coefficient), so ``psi_E`` and ``psi_H`` are compact
``(*slab_shape, 2)`` device arrays and the coefficients are 1D profiles along
``n``.  The reference-shaped arrays (``psi_Ex``, ``bE``, ``phi_E``, ...) are
available as read-only properties built on demand.
"""

import numpy as np
import torch

from .backend import backend as bd

_AXES = "xyz"


class Boundary:
    """Base class of the grid boundaries."""

    def __init__(self, name: str = None):
        self.grid = None
        self.name = name

    def _register_name(self, grid):
        if self.name is not None:
            if hasattr(grid, self.name):
                raise ValueError(f"The grid already has an attribute with name {self.name}")
            setattr(grid, self.name, self)

    def _slice_text(self):
        def fmt(s):
            return str(s).replace("slice(", "").replace(")", "").replace(", ", ":").replace("None", "")

        s = f"        @ x={fmt(self.x)}, y={fmt(self.y)}, z={fmt(self.z)}".replace(":,", ",")
        return s[:-1] if s.endswith(":") else s

    def __repr__(self):
        return f"{self.__class__.__name__}(name={repr(self.name)})"

    def __str__(self):
        return "    " + repr(self) + "\n" + self._slice_text() + "\n"


class PeriodicBoundary(Boundary):
    """Periodic boundary: after every E half step E[0] = E[-1] along its axis,
    after every H half step H[-1] = H[0] (fdtd/boundaries.py:184-219)."""

    @staticmethod
    def _index(s):
        if isinstance(s, list):
            if len(s) > 1:
                raise ValueError("Use slices or single numbers to index the grid for a boundary")
            return s[0]
        if isinstance(s, slice):
            if s.start is not None and s.stop is not None and (s.start == s.stop or abs(s.start - s.stop) == 1):
                return s.start
            return s
        raise ValueError("Invalid grid indexing used for boundary")

    def _register_grid(self, grid, x, y, z):
        self.x, self.y, self.z = self._index(x), self._index(y), self._index(z)
        for axis, v in enumerate((self.x, self.y, self.z)):
            if not isinstance(v, slice) and (v == 0 or v == -1):
                break
        else:
            raise IndexError("A periodic boundary should be placed at the boundary of the "
                             "grid using a single index (either 0 or -1)")
        tag = _AXES[axis]
        if hasattr(grid, f"_{tag}low_boundary") or hasattr(grid, f"_{tag}high_boundary"):
            raise AttributeError(f"grid already has an {tag}low/{tag}high boundary!")
        self._register_name(grid)
        setattr(grid, f"_{tag}low_boundary", self)
        setattr(grid, f"_{tag}high_boundary", self)
        self.grid = grid
        self.axis = axis
        grid.boundaries.append(self)
        grid._invalidate()


def pml_profiles(thickness, high, a, courant, k=1.0):
    """1D coefficients (bE, cE, bH, cH) along the slab normal, float64 numpy.

    sigma(v) = 40 v^3 / (thickness + 1)^4 sampled at the half-integer (E) and
    integer (H) positions of fdtd/boundaries.py:502-625 -- low side
    th-1/2 ... 1/2 and th-1 ... 1, high side mirrored, last H plane 0 -- and
    b = exp(-(sigma/k + a) courant), c = (b - 1) sigma / (sigma k + a k^2)
    (fdtd/boundaries.py:395-407)."""
    th = thickness
    if high:
        vE = np.arange(0.5, th + 0.5, 1.0)
        vH = np.arange(1.0, th, 1.0)
    else:
        vE = np.arange(th - 0.5, -0.5, -1.0)
        vH = np.arange(th - 1.0, 0, -1.0)
    sigma_E = 40 * vE ** 3 / (th + 1) ** 4
    sigma_H = np.zeros(th)
    sigma_H[:-1] = 40 * vH ** 3 / (th + 1) ** 4
    bE = np.exp(-(sigma_E / k + a) * courant)
    cE = (bE - 1.0) * sigma_E / (sigma_E * k + a * k ** 2)
    bH = np.exp(-(sigma_H / k + a) * courant)
    cH = (bH - 1.0) * sigma_H / (sigma_H * k + a * k ** 2)
    return sigma_E, sigma_H, bE, cE, bH, cH


class PML(Boundary):
    """Convolutional perfectly matched layer on one side of the grid."""

    def __init__(self, a: float = 1e-8, name: str = None):
        super().__init__(name=name)
        self.k = 1.0
        self.thickness = 0
        self.a = a

    @staticmethod
    def _slice(s):
        if isinstance(s, list):
            raise ValueError("One can only use slices to index the grid for a PML")
        if isinstance(s, slice):
            return s
        raise ValueError("Invalid grid indexing used for boundary")

    def _register_grid(self, grid, x, y, z):
        self.x, self.y, self.z = self._slice(x), self._slice(y), self._slice(z)
        found = None
        for axis, s in enumerate((self.x, self.y, self.z)):
            if (s.start is None or s.start == 0) and s.stop is not None and s.stop > 0:
                found = (axis, 0, s.stop)
                break
            if s.start is not None and s.stop is None and s.start < 0:
                found = (axis, 1, -s.start)
                break
        if found is None:
            raise IndexError("not a valid slice for a PML. Make sure the slice is at the border of the PML")
        axis, high, th = found
        side = _AXES[axis] + ("high" if high else "low")
        if hasattr(grid, f"_{side}_boundary"):
            raise AttributeError(f"grid already has an {side} boundary!")
        n = grid.shape[axis]
        if th > n:
            raise IndexError(f"PML thickness {th} larger than the grid ({n} cells along {_AXES[axis]})")
        self._register_name(grid)
        setattr(grid, f"_{side}_boundary", self)
        self.grid = grid
        self.axis, self.high, self.thickness = axis, high, th
        self.start = n - th if high else 0
        shape = list(grid.shape)
        shape[axis] = th
        self.shape = tuple(shape)
        sE, sH, bE, cE, bH, cH = pml_profiles(th, high, self.a, grid.courant_number, self.k)
        self.sigma_E_profile, self.sigma_H_profile = sE, sH
        dev, dt = grid._device, grid._dtype
        self.b_E = torch.tensor(bE, dtype=dt, device=dev)
        self.c_E = torch.tensor(cE, dtype=dt, device=dev)
        self.b_H = torch.tensor(bH, dtype=dt, device=dev)
        self.c_H = torch.tensor(cH, dtype=dt, device=dev)
        # compact auxiliaries: [..., 0] drives field[(axis+1)%3], [..., 1] field[(axis+2)%3];
        # a z slab stores an even number of planes (16-byte rows for bulk copies)
        store = list(self.shape)
        if axis == 2:
            store[2] = th + (th % 2)
        self._psi_E = torch.zeros(tuple(store) + (2,), dtype=dt, device=dev)
        self._psi_H = torch.zeros(tuple(store) + (2,), dtype=dt, device=dev)
        grid.boundaries.append(self)
        grid._invalidate()

    @property
    def psi_E(self):
        """Compact E-side auxiliaries, shape (*slab_shape, 2)."""
        return self._psi_E[:, :, : self.thickness] if self.axis == 2 else self._psi_E

    @property
    def psi_H(self):
        """Compact H-side auxiliaries, shape (*slab_shape, 2)."""
        return self._psi_H[:, :, : self.thickness] if self.axis == 2 else self._psi_H

    # --- reference-shaped views (fdtd/boundaries.py:367-407) ------------------
    @property
    def loc(self):
        sl = [slice(None)] * 4
        sl[self.axis] = slice(self.start, self.start + self.thickness)
        return tuple(sl)

    def _per_component(self, profile, other):
        """(slab, 3) array that equals ``profile`` along the normal component
        and ``other`` in the two tangential ones (an expanded view)."""
        t = torch.full((self.thickness, 3), float(other), dtype=torch.float64)
        t[:, self.axis] = torch.as_tensor(profile, dtype=torch.float64)
        shp = [1, 1, 1, 3]
        shp[self.axis] = self.thickness
        view = t.reshape(shp).to(self.grid._device)
        return view.expand(self.shape + (3,))

    @property
    def sigmaE(self):
        return self._per_component(self.sigma_E_profile, 0.0)

    @property
    def sigmaH(self):
        return self._per_component(self.sigma_H_profile, 0.0)

    @property
    def bE(self):
        import math

        return self._per_component(self.b_E.double().cpu().numpy(), math.exp(-self.a * self.grid.courant_number))

    @property
    def bH(self):
        import math

        return self._per_component(self.b_H.double().cpu().numpy(), math.exp(-self.a * self.grid.courant_number))

    @property
    def cE(self):
        return self._per_component(self.c_E.double().cpu().numpy(), 0.0)

    @property
    def cH(self):
        return self._per_component(self.c_H.double().cpu().numpy(), 0.0)

    def _psi_full(self, field, comp):
        store = self.psi_E if field == "E" else self.psi_H
        out = torch.zeros(self.shape + (3,), dtype=store.dtype, device=store.device)
        t1, t2 = (self.axis + 1) % 3, (self.axis + 2) % 3
        if comp == t1:
            out[..., self.axis] = store[..., 0]
        elif comp == t2:
            out[..., self.axis] = store[..., 1]
        return out

    psi_Ex = property(lambda self: self._psi_full("E", 0))
    psi_Ey = property(lambda self: self._psi_full("E", 1))
    psi_Ez = property(lambda self: self._psi_full("E", 2))
    psi_Hx = property(lambda self: self._psi_full("H", 0))
    psi_Hy = property(lambda self: self._psi_full("H", 1))
    psi_Hz = property(lambda self: self._psi_full("H", 2))

    def _phi(self, field):
        store = self.psi_E if field == "E" else self.psi_H
        out = torch.zeros(self.shape + (3,), dtype=store.dtype, device=store.device)
        out[..., (self.axis + 1) % 3] = -store[..., 0]
        out[..., (self.axis + 2) % 3] = store[..., 1]
        return out

    phi_E = property(lambda self: self._phi("E"))
    phi_H = property(lambda self: self._phi("H"))

    def __repr__(self):
        return f"PML(name={repr(self.name)})"


def DomainBorderPML(grid, border_cells=5):
    """A PML of ``border_cells`` on all six faces (fdtd/boundaries.py:628-656).

    Each PML spans the full cross-section of its side whatever the slice's
    tangential extent, so the six slabs overlap at the edges and corners."""
    b = border_cells
    if grid.Nx < b * 2 or grid.Ny < b * 2 or grid.Nz < b * 2:
        raise IndexError("PML border_cells larger than domain!")
    grid[:, :, 0:b] = PML()
    grid[:, :, -b:] = PML()
    grid[0:b, :, b:-b] = PML()
    grid[-b:, :, b:-b] = PML()
    grid[b:-b, 0:b, b:-b] = PML()
    grid[b:-b, -b:, b:-b] = PML()
