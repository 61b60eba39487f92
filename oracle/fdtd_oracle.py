"""CPU oracle for the fdtd time step: a numpy float64 restatement of the reference.

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` may import this module, and only as the checker
(or, in the bench, as the timed CPU baseline).  The product path in
``fdtd_gb300`` never imports it.

The module mirrors the public API of the reference package (``Grid``,
``grid[x, y, z] = component``, ``PML``, ``PeriodicBoundary``, ``Object``,
``AbsorbingObject``, ``AnisotropicObject``, ``PointSource``, ``LineSource``,
``PlaneSource``, ``LineDetector``, ``BlockDetector``) so that one scene builder
drives the reference, this oracle and the GPU backend alike.  The structure is
my own (a flat list of stages per half step, compact PML auxiliaries); the
arithmetic of every stage follows the reference operation for operation so
that float64 results agree bit for bit with the reference numpy backend.  The
golden fixtures under ``tests/golden`` were produced by running the reference
itself and pin this restatement (``tests/test_oracle_golden.py``).

Features the reference does not have (``GaussianPlaneSource``,
``PlaneDetector``, ``DFTPlaneDetector``) are defined here; the GPU backend is
checked against these definitions.

Citations are ``path:line`` inside the reference project (fdtd v0.3.6).
"""

import math

import numpy as np

# fdtd/constants.py:5-23
C0 = 299792458.0
MU0 = 4e-7 * math.pi
EPS0 = 1.0 / (MU0 * C0 ** 2)
ETA0 = MU0 * C0


# ---------------------------------------------------------------------------
# curls (fdtd/grid.py:29-76)
# ---------------------------------------------------------------------------
def _diff_fwd(a, axis):
    """a[n+1] - a[n] along ``axis``; the last plane of the axis is 0."""
    out = np.zeros_like(a)
    n = a.shape[axis]
    hi = [slice(None)] * a.ndim
    lo = [slice(None)] * a.ndim
    hi[axis] = slice(1, n)
    lo[axis] = slice(0, n - 1)
    out[tuple(lo)] = a[tuple(hi)] - a[tuple(lo)]
    return out


def _diff_bwd(a, axis):
    """a[n] - a[n-1] along ``axis``; the first plane of the axis is 0."""
    out = np.zeros_like(a)
    n = a.shape[axis]
    hi = [slice(None)] * a.ndim
    lo = [slice(None)] * a.ndim
    hi[axis] = slice(1, n)
    lo[axis] = slice(0, n - 1)
    out[tuple(hi)] = a[tuple(hi)] - a[tuple(lo)]
    return out


def curl_E(E):
    """Forward-difference curl of an E-type field, component-last layout.

    Follows fdtd/grid.py:29-51: each component is (first difference) minus
    (second difference) and the out-of-grid difference on the last plane of
    its axis is dropped (taken as 0), which is not a PEC wall.
    """
    ex, ey, ez = E[..., 0], E[..., 1], E[..., 2]
    out = np.empty_like(E)
    out[..., 0] = _diff_fwd(ez, 1) - _diff_fwd(ey, 2)
    out[..., 1] = _diff_fwd(ex, 2) - _diff_fwd(ez, 0)
    out[..., 2] = _diff_fwd(ey, 0) - _diff_fwd(ex, 1)
    return out


def curl_H(H):
    """Backward-difference curl of an H-type field (fdtd/grid.py:54-76).

    The difference is dropped on the first plane of its axis.
    """
    hx, hy, hz = H[..., 0], H[..., 1], H[..., 2]
    out = np.empty_like(H)
    out[..., 0] = _diff_bwd(hz, 1) - _diff_bwd(hy, 2)
    out[..., 1] = _diff_bwd(hx, 2) - _diff_bwd(hz, 0)
    out[..., 2] = _diff_bwd(hy, 0) - _diff_bwd(hx, 1)
    return out


# ---------------------------------------------------------------------------
# waveforms (fdtd/waveforms.py)
# ---------------------------------------------------------------------------
def hanning(f, t, n):
    """Hanning-windowed sine, fdtd/waveforms.py:8-9."""
    return (1 / 2) * (1 - math.cos(f * t / n)) * (math.sin(f * t))


FWHM_CONSTANT = 2.0 * math.sqrt(2.0 * math.log(2))  # fdtd/waveforms.py:31


def normalized_gaussian_pulse(x, fwhm, center=0.0):
    """Unit-peak Gaussian, fdtd/waveforms.py:34-46."""
    sigma = fwhm / FWHM_CONSTANT
    return np.exp(-(((x - center) ** 2.0) / (2.0 * (sigma ** 2.0))))


# ---------------------------------------------------------------------------
# grid
# ---------------------------------------------------------------------------
class Grid:
    """Oracle grid; constructor semantics of fdtd/grid.py:90-169."""

    def __init__(self, shape, grid_spacing=155e-9, permittivity=1.0,
                 permeability=1.0, courant_number=None):
        self.grid_spacing = float(grid_spacing)
        if len(shape) != 3:  # fdtd/grid.py:187-191
            raise ValueError(f"invalid grid shape {shape}")
        self.Nx, self.Ny, self.Nz = (self._handle_distance(s) for s in shape)
        self.D = int(self.Nx > 1) + int(self.Ny > 1) + int(self.Nz > 1)
        max_courant = float(self.D) ** (-0.5)  # fdtd/grid.py:119-129
        if courant_number is None:
            self.courant_number = 0.99 * max_courant
        elif courant_number > max_courant:
            raise ValueError(f"courant_number {courant_number} too high for a {self.D}D simulation")
        else:
            self.courant_number = float(courant_number)
        self.time_step = self.courant_number * self.grid_spacing / C0
        shp = (self.Nx, self.Ny, self.Nz, 3)
        self.E = np.zeros(shp)
        self.H = np.zeros(shp)
        # fdtd/grid.py:141-151
        self.inverse_permittivity = np.ones(shp) / _material(permittivity)
        self.inverse_permeability = np.ones(shp) / _material(permeability)
        self.time_steps_passed = 0
        self.sources, self.boundaries, self.detectors, self.objects = [], [], [], []

    # --- unit handling, fdtd/grid.py:171-223 --------------------------------
    def _handle_distance(self, d):
        if not isinstance(d, int):
            return int(float(d) / self.grid_spacing + 0.5)
        return d

    def _handle_time(self, t):
        if not isinstance(t, int):
            return int(float(t) / self.time_step + 0.5)
        return t

    def _handle_slice(self, s):
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

    def __setitem__(self, key, comp):  # fdtd/grid.py:358-375
        if not isinstance(key, tuple):
            key = (key,)
        if len(key) > 3 or len(key) == 0:
            raise KeyError("maximum number of indices for the grid is 3")
        key = tuple(key) + (slice(None),) * (3 - len(key))
        x, y, z = (self._handle_single_key(k) for k in key)
        comp._attach(self, x, y, z)

    @property
    def shape(self):
        return (self.Nx, self.Ny, self.Nz)

    @property
    def time_passed(self):
        return self.time_steps_passed * self.time_step

    # --- time stepping, fdtd/grid.py:250-331 --------------------------------
    def run(self, total_time, progress_bar=False):
        if isinstance(total_time, float):
            total_time /= self.time_step
        for _ in range(int(total_time)):
            self.step()

    def step(self):
        self.update_E()
        self.update_H()
        self.time_steps_passed += 1

    def update_E(self):
        """E half step in the order of fdtd/grid.py:275-299."""
        for b in self.boundaries:
            b.phi_E()
        curl = curl_H(self.H)
        self.E += self.courant_number * self.inverse_permittivity * curl
        for o in self.objects:
            o.apply_E(curl)
        for b in self.boundaries:
            b.correct_E()
        for s in self.sources:
            s.inject_E()
        for d in self.detectors:
            d.sample_E()

    def update_H(self):
        """H half step in the order of fdtd/grid.py:301-325 (objects have no H update)."""
        for b in self.boundaries:
            b.phi_H()
        curl = curl_E(self.E)
        self.H -= self.courant_number * self.inverse_permeability * curl
        for b in self.boundaries:
            b.correct_H()
        for s in self.sources:
            s.inject_H()
        for d in self.detectors:
            d.sample_H()

    def reset(self):  # fdtd/grid.py:327-331 (PML auxiliaries are not cleared)
        self.H *= 0.0
        self.E *= 0.0
        self.time_steps_passed *= 0


def _material(value):
    """Permittivity/permeability argument -> array broadcastable to (Nx,Ny,Nz,3)."""
    arr = np.asarray(value, dtype=np.float64)
    if arr.ndim == 3:
        arr = arr[:, :, :, None]
    return arr


def _named(grid, comp):
    name = getattr(comp, "name", None)
    if name is not None:
        if hasattr(grid, name):
            raise ValueError(f"The grid already has an attribute with name {name}")
        setattr(grid, name, comp)


# ---------------------------------------------------------------------------
# boundaries (fdtd/boundaries.py)
# ---------------------------------------------------------------------------
class PeriodicBoundary:
    """Plane copies after each half step, fdtd/boundaries.py:143-219."""

    def __init__(self, name=None):
        self.name = name

    @staticmethod
    def _index(s):  # fdtd/boundaries.py:62-77
        if isinstance(s, list):
            if len(s) > 1:
                raise ValueError("Use slices or single numbers to index the grid for a boundary")
            return s[0]
        if isinstance(s, slice):
            if s.start is not None and s.stop is not None and (
                    s.start == s.stop or abs(s.start - s.stop) == 1):
                return s.start
            return s
        raise ValueError("Invalid grid indexing used for boundary")

    def _attach(self, grid, x, y, z):
        idx = [self._index(s) for s in (x, y, z)]
        for axis, v in enumerate(idx):  # fdtd/boundaries.py:158-180
            if not isinstance(v, slice) and (v == 0 or v == -1):
                break
        else:
            raise IndexError("A periodic boundary should be placed at the boundary of the "
                             "grid using a single index (either 0 or -1)")
        tag = "xyz"[axis]
        if hasattr(grid, f"_{tag}low_boundary") or hasattr(grid, f"_{tag}high_boundary"):
            raise AttributeError(f"grid already has an {tag}low/{tag}high boundary!")
        setattr(grid, f"_{tag}low_boundary", self)
        setattr(grid, f"_{tag}high_boundary", self)
        self.grid, self.axis = grid, axis
        grid.boundaries.append(self)
        _named(grid, self)

    def _plane(self, i):
        sl = [slice(None)] * 4
        sl[self.axis] = i
        return tuple(sl)

    def phi_E(self):
        pass

    def phi_H(self):
        pass

    def correct_E(self):  # E[0] = E[-1]
        self.grid.E[self._plane(0)] = self.grid.E[self._plane(-1)]

    def correct_H(self):  # H[-1] = H[0]
        self.grid.H[self._plane(-1)] = self.grid.H[self._plane(0)]


def pml_sigma(v, thickness):
    """Cubic conductivity profile, fdtd/boundaries.py:291-293."""
    return 40 * v ** 3 / (thickness + 1) ** 4


def pml_profiles(thickness, high, a, courant):
    """1D PML coefficients along the normal axis of a slab.

    Returns (bE, cE, bH, cH), each of length ``thickness`` and indexed by the
    slab-local position.  Profiles follow fdtd/boundaries.py:502-625 (low side
    sigma_E at th-1/2 ... 1/2, sigma_H at th-1 ... 1 with the last plane 0; the
    high side mirrored) and the coefficients fdtd/boundaries.py:395-407 with
    k = 1.  The components tangential to the slab have sigma = 0, hence c = 0,
    so their auxiliaries stay identically zero and are not stored.
    """
    th = thickness
    if high:
        sE = pml_sigma(np.arange(0.5, th + 0.5, 1.0), th)
        sH_core = pml_sigma(np.arange(1.0, th, 1.0), th)
    else:
        sE = pml_sigma(np.arange(th - 0.5, -0.5, -1.0), th)
        sH_core = pml_sigma(np.arange(th - 1.0, 0, -1.0), th)
    sH = np.zeros(th)
    sH[:-1] = sH_core
    k = 1.0

    def coeffs(sigma):
        b = np.exp(-(sigma / k + a) * courant)
        c = (b - 1.0) * sigma / (sigma * k + a * k ** 2)
        return b, c

    bE, cE = coeffs(sE)
    bH, cH = coeffs(sH)
    return bE, cE, bH, cH


class PML:
    """Convolutional PML slab, fdtd/boundaries.py:225-487.

    Only the two auxiliaries per half step that the reference can make
    non-zero are kept: for a slab normal to axis ``n`` the E side tracks
    psi_E[(n+1)%3][n] and psi_E[(n+2)%3][n] (the ``psi_E<comp>[..., n]``
    arrays of the reference) and likewise for H.  phi is then
    phi[(n+1)%3] = -psi_a ... see ``correct_E``.
    """

    def __init__(self, a=1e-8, name=None):
        self.name = name
        self.a = a
        self.k = 1.0
        self.thickness = 0

    def _attach(self, grid, x, y, z):
        for s in (x, y, z):  # fdtd/boundaries.py:360-365
            if isinstance(s, list):
                raise ValueError("One can only use slices to index the grid for a PML")
        found = None
        for axis, s in enumerate((x, y, z)):  # fdtd/boundaries.py:301-358
            if (s.start is None or s.start == 0) and s.stop is not None and s.stop > 0:
                found = (axis, 0, s.stop)
                break
            if s.start is not None and s.stop is None and s.start < 0:
                found = (axis, 1, -s.start)
                break
        if found is None:
            raise IndexError("not a valid slice for a PML. Make sure the slice is at the border of the PML")
        axis, high, th = found
        tag = "xyz"[axis] + ("high" if high else "low")
        if hasattr(grid, f"_{tag}_boundary"):
            raise AttributeError(f"grid already has an {tag} boundary!")
        setattr(grid, f"_{tag}_boundary", self)
        self.grid, self.axis, self.high, self.thickness = grid, axis, high, th
        n = (grid.Nx, grid.Ny, grid.Nz)[axis]
        self.start = n - th if high else 0
        self.bE, self.cE, self.bH, self.cH = pml_profiles(th, high, self.a, grid.courant_number)
        shp = [grid.Nx, grid.Ny, grid.Nz]
        shp[axis] = th
        self.slab_shape = tuple(shp)
        # psiE[0] drives phi_E[(axis+1)%3], psiE[1] drives phi_E[(axis+2)%3]
        self.psiE = np.zeros((2,) + self.slab_shape)
        self.psiH = np.zeros((2,) + self.slab_shape)
        grid.boundaries.append(self)
        _named(grid, self)

    def _loc(self):
        sl = [slice(None)] * 3
        sl[self.axis] = slice(self.start, self.start + self.thickness)
        return tuple(sl)

    def _prof(self, p):
        shp = [1, 1, 1]
        shp[self.axis] = self.thickness
        return p.reshape(shp)

    # The normal-axis terms of fdtd/boundaries.py:448-455 (E) and 476-483 (H).
    # For normal axis n with tangential axes t1=(n+1)%3, t2=(n+2)%3:
    #   E side: psi_E[t1][n] += d_n H[t2] * c ; psi_E[t2][n] += d_n H[t1] * c
    #   phi_E[t1] = -psi_E[t1][n] ; phi_E[t2] = +psi_E[t2][n]
    # (e.g. x slab: psi_Ey[...,0] += dHz/dx, psi_Ez[...,0] += dHy/dx,
    #  phi_E = (0, -psi_Ey0, psi_Ez0)).
    def phi_E(self):
        n, t1, t2 = self.axis, (self.axis + 1) % 3, (self.axis + 2) % 3
        H = self.grid.H[self._loc()]
        b, c = self._prof(self.bE), self._prof(self.cE)
        self.psiE *= b
        inner = [slice(None)] * 3
        inner[n] = slice(1, None)  # slab-local index >= 1 (backward difference)
        inner = tuple(inner)
        self.psiE[(0,) + inner] += _diff_bwd(H[..., t2], n)[inner] * c[inner]
        self.psiE[(1,) + inner] += _diff_bwd(H[..., t1], n)[inner] * c[inner]

    def phi_H(self):
        n, t1, t2 = self.axis, (self.axis + 1) % 3, (self.axis + 2) % 3
        E = self.grid.E[self._loc()]
        b, c = self._prof(self.bH), self._prof(self.cH)
        self.psiH *= b
        inner = [slice(None)] * 3
        inner[n] = slice(None, -1)  # slab-local index <= th-2 (forward difference)
        inner = tuple(inner)
        self.psiH[(0,) + inner] += _diff_fwd(E[..., t2], n)[inner] * c[inner]
        self.psiH[(1,) + inner] += _diff_fwd(E[..., t1], n)[inner] * c[inner]

    def correct_E(self):  # fdtd/boundaries.py:409-419
        n, t1, t2 = self.axis, (self.axis + 1) % 3, (self.axis + 2) % 3
        loc = self._loc()
        g = self.grid
        ce = g.courant_number * g.inverse_permittivity[loc]
        g.E[loc + (t1,)] += ce[..., t1] * (-self.psiE[0])
        g.E[loc + (t2,)] += ce[..., t2] * self.psiE[1]

    def correct_H(self):  # fdtd/boundaries.py:421-431
        n, t1, t2 = self.axis, (self.axis + 1) % 3, (self.axis + 2) % 3
        loc = self._loc()
        g = self.grid
        cm = g.courant_number * g.inverse_permeability[loc]
        g.H[loc + (t1,)] -= cm[..., t1] * (-self.psiH[0])
        g.H[loc + (t2,)] -= cm[..., t2] * self.psiH[1]

    # reference-shaped views of the auxiliaries, e.g. psi_Ey[..., axis]
    def psi(self, field, comp):
        """Reference layout ``psi_<field><comp>`` of shape (slab, 3)."""
        out = np.zeros(self.slab_shape + (3,))
        n, t1, t2 = self.axis, (self.axis + 1) % 3, (self.axis + 2) % 3
        store = self.psiE if field == "E" else self.psiH
        if comp == t1:
            out[..., n] = store[0]
        elif comp == t2:
            out[..., n] = store[1]
        return out


def DomainBorderPML(grid, border_cells=5):
    """Six PML slabs around the domain, fdtd/boundaries.py:628-656."""
    b = border_cells
    if grid.Nx < b * 2 or grid.Ny < b * 2 or grid.Nz < b * 2:
        raise IndexError("PML border_cells larger than domain!")
    grid[:, :, 0:b] = PML()
    grid[:, :, -b:] = PML()
    grid[0:b, :, b:-b] = PML()
    grid[-b:, :, b:-b] = PML()
    grid[b:-b, 0:b, b:-b] = PML()
    grid[b:-b, -b:, b:-b] = PML()


# ---------------------------------------------------------------------------
# objects (fdtd/objects.py)
# ---------------------------------------------------------------------------
def _object_slice(s, n):  # fdtd/objects.py:94-116
    if isinstance(s, list):
        if len(s) == 1:
            return slice(s[0], s[0] + 1, None)
        raise IndexError("One can only use slices or single indices to index the grid for an Object")
    if isinstance(s, slice):
        start, stop, step = s.start, s.stop, s.step
        if step is not None and step != 1:
            raise IndexError("Can only use slices with unit step to index the grid for an Object")
        start = 0 if start is None else start
        start = n + start if start < 0 else start
        stop = n if stop is None else stop
        stop = n + stop if stop < 0 else stop
        return slice(start, stop, None)
    raise ValueError("Invalid grid indexing used for object")


class Object:
    """Dielectric box, fdtd/objects.py:24-137."""

    def __init__(self, permittivity, name=None):
        self.name = name
        perm = np.array(permittivity)
        if np.iscomplexobj(perm):
            raise NotImplementedError("complex permittivity")
        self.permittivity = np.asarray(perm, dtype=np.float64)

    def _attach(self, grid, x, y, z):
        self.grid = grid
        self.x = _object_slice(x, grid.Nx)
        self.y = _object_slice(y, grid.Ny)
        self.z = _object_slice(z, grid.Nz)
        self.Nx = abs(self.x.stop - self.x.start)
        self.Ny = abs(self.y.stop - self.y.start)
        self.Nz = abs(self.z.stop - self.z.start)
        perm = self.permittivity
        if perm.ndim == 3:
            perm = perm[:, :, :, None]
        ie = np.ones((self.Nx, self.Ny, self.Nz, 3)) / perm
        gie = grid.inverse_permittivity
        # border symmetrisation quirk, fdtd/objects.py:79-90: the object's last
        # plane per component takes the grid value at index -1 of the WHOLE grid
        if self.Nx > 1:
            ie[-1, :, :, 0] = gie[-1, self.y, self.z, 0]
        if self.Ny > 1:
            ie[:, -1, :, 1] = gie[self.x, -1, self.z, 1]
        if self.Nz > 1:
            ie[:, :, -1, 2] = gie[self.x, self.y, -1, 2]
        gie[self.x, self.y, self.z] = 0  # fdtd/objects.py:92
        self.inverse_permittivity = ie
        self._setup()
        grid.objects.append(self)
        _named(grid, self)

    def _setup(self):
        pass

    def _loc(self):
        return (self.x, self.y, self.z)

    def apply_E(self, curl):  # fdtd/objects.py:118-129
        loc = self._loc()
        g = self.grid
        g.E[loc] = g.E[loc] + (g.courant_number * self.inverse_permittivity * curl[loc])


class AbsorbingObject(Object):
    """Conductive box, fdtd/objects.py:163-229."""

    def __init__(self, permittivity, conductivity, name=None):
        super().__init__(permittivity, name)
        self.conductivity = np.asarray(np.array(conductivity), dtype=np.float64)

    def _setup(self):
        cond = self.conductivity
        while cond.ndim < self.inverse_permittivity.ndim:
            cond = cond[..., None]
        self.conductivity = np.broadcast_to(cond, self.inverse_permittivity.shape)
        g = self.grid
        # fdtd/objects.py:198-205
        self.absorption_factor = (0.5 * g.courant_number * self.inverse_permittivity
                                  * self.conductivity * g.grid_spacing * ETA0)

    def apply_E(self, curl):  # fdtd/objects.py:207-221
        loc = self._loc()
        g = self.grid
        f = self.absorption_factor
        g.E[loc] *= (1 - f) / (1 + f)
        g.E[loc] += g.courant_number * self.inverse_permittivity * curl[loc] / (1 + f)


class AnisotropicObject(Object):
    """Box with a 3x3 inverse permittivity per cell, fdtd/objects.py:232-277."""

    def _setup(self):
        n = self.Nx * self.Ny * self.Nz
        eye = np.zeros((n, 3, 3))
        eye[:, range(3), range(3)] = 1.0
        self.inverse_permittivity = np.reshape(
            np.reshape(self.inverse_permittivity, (-1, 1, 3)) * eye,
            (self.Nx, self.Ny, self.Nz, 3, 3))

    def apply_E(self, curl):  # fdtd/objects.py:254-269
        loc = self._loc()
        g = self.grid
        m = np.einsum("ijk,ikl->ijl", np.reshape(self.inverse_permittivity, (-1, 3, 3)),
                      np.reshape(curl[loc], (-1, 3, 1)))
        g.E[loc] += np.reshape(g.courant_number * m, (self.Nx, self.Ny, self.Nz, 3))


# ---------------------------------------------------------------------------
# sources (fdtd/sources.py)
# ---------------------------------------------------------------------------
def _linspace_points(a0, a1, m):
    return [int(v) for v in np.array(np.linspace(a0, a1, m, endpoint=False), np.int64)]


class _Waveform:
    """Shared sin / Hanning waveform of PointSource and LineSource
    (fdtd/sources.py:93-109 and 278-297)."""

    def _init_wave(self, period, amplitude, phase_shift, name, pulse, cycle, hanning_dt):
        self.period, self.amplitude, self.phase_shift = period, amplitude, phase_shift
        self.name, self.pulse, self.cycle = name, pulse, cycle
        self.frequency = 1.0 / period
        self.hanning_dt = hanning_dt if hanning_dt is not None else 0.5 / self.frequency

    def wave(self, q):
        if self.pulse:
            t1 = int(2 * math.pi / (self.frequency * self.hanning_dt / self.cycle))
            if q < t1:
                return hanning(self.frequency, q * self.hanning_dt, self.cycle)
            return 0.0
        return math.sin(2 * math.pi * q / self.period + self.phase_shift)


class PointSource(_Waveform):
    """Soft z-directed point source, fdtd/sources.py:25-127."""

    def __init__(self, period=15, amplitude=1.0, phase_shift=0.0, name=None, pulse=False,
                 cycle=5, hanning_dt=10.0):
        self._init_wave(period, amplitude, phase_shift, name, pulse, cycle, hanning_dt)

    def _attach(self, grid, x, y, z):
        try:
            (x,), (y,), (z,) = x, y, z
        except (TypeError, ValueError):
            raise ValueError("a point source should be placed on a single grid cell.")
        self.grid = grid
        self.x, self.y, self.z = (grid._handle_distance(v) for v in (x, y, z))
        self.period = grid._handle_time(self.period)
        self.frequency = 1.0 / self.period
        grid.sources.append(self)
        _named(grid, self)

    def inject_E(self):
        src = self.amplitude * self.wave(self.grid.time_steps_passed)
        self.grid.E[self.x, self.y, self.z, 2] += src

    def inject_H(self):
        pass


class LineSource(_Waveform):
    """Soft z-directed source with a Gaussian profile along a diagonal,
    fdtd/sources.py:131-315."""

    def __init__(self, period=15, amplitude=1.0, phase_shift=0.0, name=None, pulse=False,
                 cycle=5, hanning_dt=10.0):
        self._init_wave(period, amplitude, phase_shift, name, pulse, cycle, hanning_dt)

    def _points(self, grid, x, y, z):  # fdtd/sources.py:209-276
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
        x, y, z = conv
        lo = [grid._handle_distance(s.start if s.start is not None else 0) for s in (x, y, z)]
        hi = [grid._handle_distance(s.stop if s.stop is not None else n)
              for s, n in zip((x, y, z), grid.shape)]
        m = max(abs(h - l) for l, h in zip(lo, hi))
        if m < 2:
            raise ValueError("a LineSource should consist of at least two gridpoints")
        return tuple(_linspace_points(l, h, m) for l, h in zip(lo, hi))

    def _attach(self, grid, x, y, z):
        self.grid = grid
        self.x, self.y, self.z = self._points(grid, x, y, z)
        self.period = grid._handle_time(self.period)
        self.frequency = 1.0 / self.period
        L = len(self.x)
        # fdtd/sources.py:197-207 (squared distance, squared again)
        vect = np.array((np.array(self.x) - self.x[L // 2]) ** 2
                        + (np.array(self.y) - self.y[L // 2]) ** 2
                        + (np.array(self.z) - self.z[L // 2]) ** 2, np.float64)
        self.profile = np.exp(-(vect ** 2) / (2 * (0.5 * vect.max()) ** 2))
        self.profile /= self.profile.sum()
        self.profile *= self.amplitude
        grid.sources.append(self)
        _named(grid, self)

    def inject_E(self):
        vect = self.profile * self.wave(self.grid.time_steps_passed)
        for x, y, z, v in zip(self.x, self.y, self.z, vect):
            self.grid.E[x, y, z, 2] += v

    def inject_H(self):
        pass


class PlaneSource:
    """Hard plane source that overwrites one E and one H component,
    fdtd/sources.py:319-501."""

    def __init__(self, period=15, amplitude=1.0, phase_shift=0.0, name=None, polarization="z"):
        self.period, self.amplitude, self.phase_shift = period, amplitude, phase_shift
        self.name, self.polarization = name, polarization

    def _box(self, grid, x, y, z):  # fdtd/sources.py:390-474
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
            raise ValueError("Given location for PlaneSource should have no more than one "
                             "dimension in which it's flat.")
        epol = "xyz".index(self.polarization)
        if lengths[epol] == 1:
            raise ValueError("PlaneSource cannot be polarized perpendicular to the orientation of the plane.")
        hp = [(2, 1, 2), (2, 0, 2), (1, 0, 1)][epol]
        hpol = hp[1] if lengths[hp[0]] == 1 else hp[2]
        return out, epol, hpol

    def _attach(self, grid, x, y, z):
        self.grid = grid
        (self.x, self.y, self.z), self._Epol, self._Hpol = self._box(grid, x, y, z)
        self.period = grid._handle_time(self.period)
        self.frequency = 1.0 / self.period
        shp = (self.x.stop - self.x.start, self.y.stop - self.y.start, self.z.stop - self.z.start)
        self.profile = self.amplitude * np.ones(shp)
        grid.sources.append(self)
        _named(grid, self)

    def wave(self, q):
        return math.sin(2 * math.pi * q / self.period + self.phase_shift)

    def inject_E(self):
        vect = self.profile * self.wave(self.grid.time_steps_passed)
        self.grid.E[self.x, self.y, self.z, self._Epol] = vect

    def inject_H(self):
        vect = self.profile * self.wave(self.grid.time_steps_passed)
        self.grid.H[self.x, self.y, self.z, self._Hpol] = vect


class GaussianPlaneSource(PlaneSource):
    """Hard plane source with a Gaussian envelope (not in the reference).

    value(q) = amplitude * g(q dt) * sin(2 pi q dt / T + phase_shift), with
    g = normalized_gaussian_pulse(t, fwhm, center) of fdtd/waveforms.py:34-46.
    Unlike PlaneSource the carrier period T is NOT rounded to whole time steps
    (a broadband pulse must keep its centre frequency).  ``period``, ``fwhm``
    and ``center`` are in seconds; defaults: fwhm = 4 periods, center = 2 fwhm.
    """

    def __init__(self, period=15, amplitude=1.0, phase_shift=0.0, name=None, polarization="z",
                 fwhm=None, center=None):
        super().__init__(period, amplitude, phase_shift, name, polarization)
        self.fwhm, self.center = fwhm, center

    def _attach(self, grid, x, y, z):
        period_s = self.period * grid.time_step if isinstance(self.period, int) else float(self.period)
        super()._attach(grid, x, y, z)
        self.period_s = period_s
        self.fwhm_s = 4.0 * period_s if self.fwhm is None else float(self.fwhm)
        self.center_s = 2.0 * self.fwhm_s if self.center is None else float(self.center)

    def wave(self, q):
        t = q * self.grid.time_step
        env = float(normalized_gaussian_pulse(t, self.fwhm_s, self.center_s))
        return env * math.sin(2 * math.pi * t / self.period_s + self.phase_shift)


# ---------------------------------------------------------------------------
# detectors (fdtd/detectors.py)
# ---------------------------------------------------------------------------
def _detector_ranges(grid, x, y, z):
    """Common part of LineDetector/BlockDetector._handle_slices
    (fdtd/detectors.py:63-112 and 191-239); returns None for equal lists."""
    if isinstance(x, list) and isinstance(y, list) and isinstance(z, list):
        if len(x) != len(y) or len(y) != len(z) or len(z) != len(x):
            raise IndexError("sources require grid to be indexed with slices or equal length list-indices")
        return None
    conv = []
    for s in (x, y, z):
        if isinstance(s, list):
            s = slice(s[0], s[-1], None)
        conv.append(s)
    lo = [s.start if s.start is not None else 0 for s in conv]
    hi = [s.stop if s.stop is not None else n for s, n in zip(conv, grid.shape)]
    return lo, hi


class LineDetector:
    """Samples E/H along a diagonal after each half step, fdtd/detectors.py:20-140."""

    def __init__(self, name=None):
        self.name = name
        self.E, self.H = [], []

    def _attach(self, grid, x, y, z):
        r = _detector_ranges(grid, x, y, z)
        if r is None:
            self.x, self.y, self.z = x, y, z
        else:
            lo, hi = r
            m = max(abs(h - l) for l, h in zip(lo, hi))
            self.x, self.y, self.z = (_linspace_points(l, h, m) for l, h in zip(lo, hi))
        self.grid = grid
        grid.detectors.append(self)
        _named(grid, self)

    def sample_E(self):
        self.E.append(self.grid.E[self.x, self.y, self.z])

    def sample_H(self):
        self.H.append(self.grid.H[self.x, self.y, self.z])

    def detector_values(self):
        return {"E": self.E, "H": self.H}


class BlockDetector(LineDetector):
    """Samples an inclusive index block, fdtd/detectors.py:146-281.

    Each record has shape (len(x), len(y), len(z), 3) -- the array form of
    the reference's nested lists."""

    def _attach(self, grid, x, y, z):
        r = _detector_ranges(grid, x, y, z)
        if r is None:
            self.x, self.y, self.z = x, y, z
        else:
            lo, hi = r
            self.x, self.y, self.z = ([int(v) for v in np.arange(l, h + 1)] for l, h in zip(lo, hi))
        self.grid = grid
        grid.detectors.append(self)
        _named(grid, self)

    def sample_E(self):
        self.E.append(self.grid.E[np.ix_(self.x, self.y, self.z)])

    def sample_H(self):
        self.H.append(self.grid.H[np.ix_(self.x, self.y, self.z)])


class CurrentDetector:
    """Loop current around a point after each H half step,
    fdtd/detectors.py:284-496 (single_point_current :404-464).  Index ranges
    are inclusive like BlockDetector; each record is an (nx, ny, nz) array,
    the array form of the reference's nested lists."""

    def __init__(self, name=None):
        self.name = name
        self.I = []

    def _attach(self, grid, x, y, z):
        r = _detector_ranges(grid, x, y, z)
        if r is None:
            self.x, self.y, self.z = x, y, z
        else:
            lo, hi = r
            self.x, self.y, self.z = ([int(v) for v in np.arange(l, h + 1)] for l, h in zip(lo, hi))
        self.grid = grid
        grid.detectors.append(self)
        _named(grid, self)

    def _point(self, px, py, pz):
        # the reference's order, its running sum of the second y term, and
        # numpy's wrap-around of index -1
        H, du = self.grid.H, self.grid.grid_spacing
        cv1 = (H[px, py - 1, pz, 0] - H[px, py, pz, 0]) * du
        cv2 = (H[px, py, pz, 1] - H[px - 1, py, pz, 1]) * du
        c1 = cv1 + cv2
        cv1 = (H[px, py - 1, pz - 1, 0] - H[px, py, pz - 1, 0]) * du
        cv2 += (H[px, py, pz - 1, 1] - H[px - 1, py, pz - 1, 1]) * du
        c2 = cv1 + cv2
        return (c1 + c2) / 2.0

    def sample_E(self):
        pass

    def sample_H(self):
        self.I.append(np.array([[[self._point(px, py, pz) for pz in self.z] for py in self.y] for px in self.x]))

    def detector_values(self):
        return {"I": self.I}


class SoftArbitraryPointSource:
    """Voltage-driven point source with current feedback, fdtd/sources.py:504-643:
    E_z += (input + impedance * I_prev) / grid_spacing at the point, I_prev the
    last record of its own CurrentDetector (0 at step 0).  A named source names
    its detector <name>_I (the reference fails for named sources)."""

    def __init__(self, waveform_array, name=None, impedance=0.0):
        self.name = name
        self.waveform_array = waveform_array
        self.impedance = impedance
        self.input_voltage, self.source_voltage = [], []

    def _attach(self, grid, x, y, z):
        try:
            (x,), (y,), (z,) = x, y, z
        except (TypeError, ValueError):
            raise ValueError("a point source should be placed on a single grid cell.")
        self.grid = grid
        self.x, self.y, self.z = (grid._handle_distance(v) for v in (x, y, z))
        grid.sources.append(self)
        _named(grid, self)
        self.current_detector = CurrentDetector(name=None if self.name is None else self.name + "_I")
        grid[x, y, z] = self.current_detector

    def inject_E(self):  # fdtd/sources.py:600-629
        g = self.grid
        q = g.time_steps_passed
        vin = self.waveform_array[q] if q < self.waveform_array.shape[0] else 0.0
        cur = self.current_detector.I[-1][0][0][0] if q > 0 else 0.0
        vout = vin + self.impedance * cur if self.impedance > 0 else vin
        g.E[self.x, self.y, self.z, 2] += vout / g.grid_spacing
        self.input_voltage.append([[[vin]]])
        self.source_voltage.append([[[vout]]])

    def inject_H(self):
        pass


def _half_open_box(grid, x, y, z):
    out = []
    for s, n in zip((x, y, z), grid.shape):
        if isinstance(s, list):
            if len(s) != 1:
                raise IndexError("use slices or single indices for a plane detector")
            i = s[0] + n if s[0] < 0 else s[0]
            out.append(slice(i, i + 1))
        else:
            a0, a1, _ = s.indices(n)
            if a1 <= a0:
                raise IndexError("empty detector range")
            out.append(slice(a0, a1))
    return tuple(out)


class PlaneDetector:
    """Records the field on a half-open box (usually a plane) after every
    half step (not in the reference).  Each E record is E[box] of shape
    (nx, ny, nz, 3), taken after sources, like LineDetector.detect_E."""

    def __init__(self, name=None):
        self.name = name
        self.E, self.H = [], []

    def _attach(self, grid, x, y, z):
        self.grid = grid
        self.x, self.y, self.z = _half_open_box(grid, x, y, z)
        grid.detectors.append(self)
        _named(grid, self)

    def sample_E(self):
        self.E.append(self.grid.E[self.x, self.y, self.z].copy())

    def sample_H(self):
        self.H.append(self.grid.H[self.x, self.y, self.z].copy())

    def detector_values(self):
        return {"E": self.E, "H": self.H}


def dft_factor(frequency, q, dt):
    """exp(-i 2 pi f q dt) as (cos, -sin) pair, evaluated with Python math."""
    theta = 2.0 * math.pi * frequency * (q * dt)
    return math.cos(theta), -math.sin(theta)


class DFTPlaneDetector:
    """Running discrete Fourier transform of E on a half-open box (not in the
    reference).  After every E half step at step index q:

        dft[f] += E[box] * exp(-i 2 pi frequencies[f] q dt)   (complex128)

    ``frequencies`` in Hz (or give ``wavelengths`` in metres)."""

    def __init__(self, frequencies=None, wavelengths=None, name=None):
        if (frequencies is None) == (wavelengths is None):
            raise ValueError("give exactly one of frequencies or wavelengths")
        if wavelengths is not None:
            frequencies = [C0 / float(w) for w in np.atleast_1d(wavelengths)]
        self.frequencies = [float(f) for f in np.atleast_1d(frequencies)]
        self.name = name

    def _attach(self, grid, x, y, z):
        self.grid = grid
        self.x, self.y, self.z = _half_open_box(grid, x, y, z)
        shp = (self.x.stop - self.x.start, self.y.stop - self.y.start, self.z.stop - self.z.start, 3)
        self.dft = np.zeros((len(self.frequencies),) + shp, dtype=np.complex128)
        grid.detectors.append(self)
        _named(grid, self)

    def sample_E(self):
        e = self.grid.E[self.x, self.y, self.z]
        q = self.grid.time_steps_passed
        for f, fr in enumerate(self.frequencies):
            c, s = dft_factor(fr, q, self.grid.time_step)
            self.dft[f].real += e * c
            self.dft[f].imag += e * s

    def sample_H(self):
        pass
