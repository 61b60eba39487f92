"""Objects: boxes with their own E update (API of fdtd/objects.py).

Registration follows fdtd/objects.py:37-92 exactly, including its quirks:
the object's inverse permittivity on its last plane per component is copied
from the grid's LAST plane of the whole grid (fdtd/objects.py:79-90), and the
grid's inverse permittivity inside the box is set to zero, so the bulk update
adds nothing there and the PML correction inside an object uses zero too.

The time-step kernels read per-cell coefficient arrays derived from the
object's attributes (``inverse_permittivity``, ``conductivity``):

    Object             coef0 = courant * inverse_permittivity
    AbsorbingObject    coef0 = (1 - f) / (1 + f), coef1 = courant * inverse_permittivity,
                       coef2 = 1 + f, f = absorption_factor (float32 plans use
                       coef1 / coef2 premultiplied)
    AnisotropicObject  coef0 = inverse_permittivity (3x3 per cell)

They are rebuilt whenever an attribute is reassigned or modified in place.
"""

import torch

from . import constants as const
from .backend import backend as bd


def _as_f64(value, device):
    if torch.is_tensor(value):
        return value.detach().to(device=device, dtype=torch.float64)
    return torch.as_tensor(value, dtype=torch.float64, device=device)


class Object:
    """A dielectric box: E[box] += courant * inverse_permittivity * curl_H[box]."""

    _kind = 0

    def __init__(self, permittivity, name: str = None):
        self.grid = None
        self.name = name
        if bd.is_complex(permittivity):
            raise NotImplementedError("complex permittivity is not supported by the gb300 backend")
        self.permittivity = _as_f64(permittivity, "cpu")

    def _handle_slice(self, s, max_index=None):
        if isinstance(s, list):
            if len(s) == 1:
                return slice(s[0], s[0] + 1, None)
            raise IndexError("One can only use slices or single indices to index the grid for an Object")
        if isinstance(s, slice):
            start, stop, step = s.start, s.stop, s.step
            if step is not None and step != 1:
                raise IndexError("Can only use slices with unit step to index the grid for an Object")
            start = 0 if start is None else start
            start = max_index + start if start < 0 else start
            stop = max_index if stop is None else stop
            stop = max_index + stop if stop < 0 else stop
            return slice(start, stop, None)
        raise ValueError("Invalid grid indexing used for object")

    def _register_grid(self, grid, x, y, z):
        xs = self._handle_slice(x, max_index=grid.Nx)
        ys = self._handle_slice(y, max_index=grid.Ny)
        zs = self._handle_slice(z, max_index=grid.Nz)
        if self.name is not None and hasattr(grid, self.name):
            raise ValueError(f"The grid already has an attribute with name {self.name}")
        for s, n in zip((xs, ys, zs), grid.shape):
            if not (0 <= s.start < s.stop <= n):
                raise IndexError(f"object slice {s} outside the grid (size {n})")
        self.grid = grid
        self.x, self.y, self.z = xs, ys, zs
        self.Nx = abs(self.x.stop - self.x.start)
        self.Ny = abs(self.y.stop - self.y.start)
        self.Nz = abs(self.z.stop - self.z.start)
        dev = grid._device
        perm = self.permittivity.to(dev)
        if perm.ndim == 3:
            perm = perm[:, :, :, None]
        ie = torch.ones((self.Nx, self.Ny, self.Nz, 3), dtype=torch.float64, device=dev) / perm
        gie = grid.inverse_permittivity
        if self.Nx > 1:
            ie[-1, :, :, 0] = gie[-1, self.y, self.z, 0].to(torch.float64)
        if self.Ny > 1:
            ie[:, -1, :, 1] = gie[self.x, -1, self.z, 1].to(torch.float64)
        if self.Nz > 1:
            ie[:, :, -1, 2] = gie[self.x, self.y, -1, 2].to(torch.float64)
        gie[self.x, self.y, self.z] = 0
        self._inverse_permittivity = ie.contiguous()
        self._setup()
        if self.name is not None:
            setattr(grid, self.name, self)
        grid.objects.append(self)
        grid._invalidate()

    def _setup(self):
        pass

    # inverse_permittivity is the design variable of the adjoint; assignments
    # are converted to a float64 device tensor of the object's shape
    @property
    def inverse_permittivity(self):
        return self._inverse_permittivity

    @inverse_permittivity.setter
    def inverse_permittivity(self, value):
        t = _as_f64(value, self.grid._device if self.grid is not None else "cpu")
        if self.grid is not None:
            t = torch.broadcast_to(t, self._inverse_permittivity.shape).contiguous()
        self._inverse_permittivity = t
        if self.grid is not None:
            self._after_update()
            self.grid._invalidate()

    def _after_update(self):
        pass

    # --- coefficient arrays for the kernels ----------------------------------
    def _coef_key(self):
        ie = self._inverse_permittivity
        return (id(ie), ie._version)

    def _coefficients(self, dtype):
        """Per-cell coefficient tensors in the plan's dtype (cached)."""
        key = (self._coef_key(), dtype, self.grid.courant_number)
        cached = getattr(self, "_coef_cache", None)
        if cached is not None and cached[0] == key:
            return cached[1]
        coefs = self._make_coefficients(dtype)
        self._coef_cache = (key, coefs)
        return coefs

    def _make_coefficients(self, dtype):
        # host float64 arithmetic: elementwise IEEE results identical to numpy's
        ci = self.grid.courant_number * self._inverse_permittivity.cpu()
        return [ci.to(dtype).to(self.grid._device).contiguous()]

    def __repr__(self):
        return f"{self.__class__.__name__}(name={repr(self.name)})"

    def __str__(self):
        def fmt(s):
            return str(s).replace("slice(", "").replace(")", "").replace(", ", ":").replace("None", "")

        s = "    " + repr(self) + "\n"
        s += f"        @ x={fmt(self.x)}, y={fmt(self.y)}, z={fmt(self.z)}".replace(":,", ",")
        if s[-1] == ":":
            s = s[:-1]
        return s + "\n"


class AbsorbingObject(Object):
    """A conductive box: E *= (1-f)/(1+f); E += courant*eps^-1*curl_H/(1+f)
    with f = 0.5*courant*eps^-1*sigma*du*eta0 (fdtd/objects.py:163-221)."""

    _kind = 1

    def __init__(self, permittivity, conductivity, name: str = None):
        super().__init__(permittivity, name)
        self.conductivity = _as_f64(conductivity, "cpu")

    def _setup(self):
        cond = self.conductivity.to(self.grid._device)
        while cond.ndim < self._inverse_permittivity.ndim:
            cond = cond[..., None]
        self.conductivity = torch.broadcast_to(cond, self._inverse_permittivity.shape)
        self._after_update()

    def _after_update(self):
        g = self.grid
        f = (0.5 * g.courant_number * self._inverse_permittivity.cpu() * self.conductivity.cpu()
             * g.grid_spacing * const.eta0)
        self.absorption_factor = f.to(g._device)

    def _coef_key(self):
        ie, cond = self._inverse_permittivity, self.conductivity
        return (id(ie), ie._version, id(cond), cond._version)

    def _make_coefficients(self, dtype):
        self._after_update()
        # host float64 arithmetic: elementwise IEEE results identical to numpy's
        f = self.absorption_factor.cpu()
        r = (1 - f) / (1 + f)
        ci = self.grid.courant_number * self._inverse_permittivity.cpu()
        opf = 1 + f
        dev = self.grid._device
        if dtype == torch.float64:
            return [r.contiguous().to(dev), ci.contiguous().to(dev), opf.contiguous().to(dev)]
        return [r.to(dtype).contiguous().to(dev), (ci / opf).to(dtype).contiguous().to(dev)]


class AnisotropicObject(Object):
    """A box with a full 3x3 inverse permittivity per cell:
    E[box] += courant * (eps^-1 @ curl_H) (fdtd/objects.py:232-269)."""

    _kind = 2

    def _setup(self):
        ie = self._inverse_permittivity
        eye = torch.eye(3, dtype=torch.float64, device=ie.device)
        self._inverse_permittivity = (ie[..., None, :] * eye).contiguous()

    def _make_coefficients(self, dtype):
        return [self._inverse_permittivity.to(dtype).contiguous()]
