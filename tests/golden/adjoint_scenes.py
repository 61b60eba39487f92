"""Small differentiable scenes whose reference gradients are committed as fixtures.

Each scene builds a grid with one design object on an fdtd-like module ``fd``
(the reference package with its torch.float64 backend, or fdtd_gb300) and
defines a scalar loss over field samples taken after every step:

* ``ref_loss(grid, torch)`` runs the scene's steps on the reference the way a
  reference user differentiates it (a manual ``grid.step()`` loop, loss
  terms built from cloned field slices) and returns the loss tensor;
* ``detectors(fd, grid)`` registers fdtd_gb300 detectors on the same samples
  and ``gb_loss(outs, torch)`` builds the same loss from the outputs of
  ``fdtd_gb300.adjoint.run``.

``make_golden_adjoint.py`` differentiates ``ref_loss`` with autograd through
the reference's time step (grad of the loss with respect to the design
tensor) and stores the gradient; the GPU tests compare the adjoint gradient
with it.
"""

import math

import numpy as np

C0 = 299792458.0
PERIOD = 1550e-9 / C0


def _pml_all(fd, grid, th):
    grid[0:th, :, :] = fd.PML(name="pml_xlow")
    grid[-th:, :, :] = fd.PML(name="pml_xhigh")
    grid[:, 0:th, :] = fd.PML(name="pml_ylow")
    grid[:, -th:, :] = fd.PML(name="pml_yhigh")
    grid[:, :, 0:th] = fd.PML(name="pml_zlow")
    grid[:, :, -th:] = fd.PML(name="pml_zhigh")


class PlaneScene:
    """Config-4 shape at 16x16x20: 4-cell PML on every face, hard plane source
    at z=3 (x polarised), 6^3 design Object, loss = sum of Ez^2 on the plane
    z=16 over the last 20 of 60 steps."""

    name = "adj_plane"
    steps = 60
    window = (40, 60)
    design_shape = (6, 6, 6)

    def build(self, fd):
        grid = fd.Grid((16, 16, 20), grid_spacing=155e-9)
        _pml_all(fd, grid, 4)
        obj = fd.Object(permittivity=2.0, name="design")
        grid[5:11, 5:11, 7:13] = obj
        grid[:, :, 3] = fd.PlaneSource(period=PERIOD, polarization="x", name="src")
        return grid, obj

    def design(self):
        return np.random.default_rng(4).uniform(1.0 / 12.0, 1.0, size=self.design_shape)

    def ref_loss(self, grid, torch):
        loss = torch.zeros((), dtype=torch.float64)
        for t in range(self.steps):
            grid.step()
            if self.window[0] <= t < self.window[1]:
                loss = loss + (grid.E[:, :, 16, 2].clone() ** 2).sum()
        return loss

    def detectors(self, fd, grid):
        grid[:, :, 16] = fd.PlaneDetector(name="plane")

    def gb_loss(self, outs, torch):
        e = outs["plane"]["E"][self.window[0]: self.window[1], :, :, 0, 2]
        return (e.to(torch.float64) ** 2).sum()


class PeriodicScene:
    """Periodic x boundary with 3-cell PML on y and z, a non-design absorbing
    object, soft point and line sources, a design Object overlapping the
    absorber's neighbourhood; loss mixes a weighted linear E term along a line
    and an H^2 term on a second line, over all 40 steps.  ``periodic_first``
    selects the boundary registration order."""

    steps = 40
    design_shape = (5, 5, 5)

    def __init__(self, periodic_first):
        self.periodic_first = periodic_first
        self.name = "adj_periodic_first" if periodic_first else "adj_periodic_last"

    def build(self, fd):
        rng = np.random.default_rng(8)
        eps = rng.uniform(1.0, 3.0, size=(14, 12, 16))
        grid = fd.Grid((14, 12, 16), grid_spacing=155e-9, permittivity=eps)
        if self.periodic_first:
            grid[0, :, :] = fd.PeriodicBoundary(name="periodic")
        grid[:, 0:3, :] = fd.PML(name="pml_ylow")
        grid[:, -3:, :] = fd.PML(name="pml_yhigh")
        grid[:, :, 0:3] = fd.PML(name="pml_zlow")
        grid[:, :, -3:] = fd.PML(name="pml_zhigh")
        if not self.periodic_first:
            grid[0, :, :] = fd.PeriodicBoundary(name="periodic")
        grid[1:5, 3:8, 4:9] = fd.AbsorbingObject(permittivity=2.5, conductivity=2e4, name="absorber")
        obj = fd.Object(permittivity=2.0, name="design")
        grid[6:11, 4:9, 6:11] = obj
        grid[3, 6, 4] = fd.PointSource(period=PERIOD, amplitude=1.0, name="point")
        grid[8, 2:10, 12] = fd.LineSource(period=PERIOD * 0.8, amplitude=0.5, name="line")
        return grid, obj

    def design(self):
        return np.random.default_rng(5).uniform(1.0 / 12.0, 1.0, size=self.design_shape)

    def weights(self):
        return np.random.default_rng(6).standard_normal((14, 3))

    def ref_loss(self, grid, torch):
        w = torch.as_tensor(self.weights())
        loss = torch.zeros((), dtype=torch.float64)
        for _ in range(self.steps):
            grid.step()
            loss = loss + (grid.E[:, 6, 13, :].clone() * w).sum()
            loss = loss + (grid.H[4, :, 10, :].clone() ** 2).sum()
        return loss

    def detectors(self, fd, grid):
        grid[:, 6, 13] = fd.LineDetector(name="lineE")
        grid[4, :, 10] = fd.LineDetector(name="lineH")

    def gb_loss(self, outs, torch):
        w = torch.as_tensor(self.weights(), device=outs["lineE"]["E"].device)
        a = (outs["lineE"]["E"].to(torch.float64) * w).sum()
        b = (outs["lineH"]["H"].to(torch.float64) ** 2).sum()
        return a + b


class AnisoDftScene:
    """6^3 AnisotropicObject design (SPD inverse permittivity tensors) in a
    16^3 grid with 4-cell PML, hard plane source at z=3 (y polarised); loss =
    sum over two frequencies and the plane z=12 of |F(Ex)|^2 + |F(Ey)|^2, F the
    running DFT exp(-i 2 pi f q dt) over all 50 steps."""

    name = "adj_aniso_dft"
    steps = 50
    design_shape = (6, 6, 6, 3, 3)
    wavelengths = (1400e-9, 1700e-9)

    def build(self, fd):
        grid = fd.Grid((16, 16, 16), grid_spacing=155e-9)
        _pml_all(fd, grid, 4)
        obj = fd.AnisotropicObject(permittivity=2.0, name="design")
        grid[5:11, 5:11, 5:11] = obj
        grid[:, :, 3] = fd.PlaneSource(period=PERIOD, polarization="y", name="src")
        return grid, obj

    def design(self):
        rng = np.random.default_rng(7)
        q, _ = np.linalg.qr(rng.standard_normal((216, 3, 3)))
        lam = rng.uniform(2.0, 6.0, size=(216, 3))
        m = np.einsum("nij,nj,nkj->nik", q, 1.0 / lam, q)
        return m.reshape(self.design_shape)

    def ref_loss(self, grid, torch):
        freqs = [C0 / w for w in self.wavelengths]
        F = [torch.zeros((16, 16, 2), dtype=torch.complex128) for _ in freqs]
        for _ in range(self.steps):
            grid.step()
            q = grid.time_steps_passed - 1
            e = grid.E[:, :, 12, 0:2].clone()
            for n, f in enumerate(freqs):
                theta = 2.0 * math.pi * f * (q * grid.time_step)
                F[n] = F[n] + e * complex(math.cos(theta), -math.sin(theta))
        return sum((f.abs() ** 2).sum() for f in F)

    def detectors(self, fd, grid):
        grid[:, :, 12] = fd.DFTPlaneDetector(wavelengths=list(self.wavelengths), name="dft")

    def gb_loss(self, outs, torch):
        F = outs["dft"]["dft"][:, :, :, 0, 0:2]
        return (F.abs() ** 2).sum()


class RandomScene:
    """A random forward scene of tests/test_fuzz_gpu.py (less its
    PlaneDetector, which the reference lacks) with a design Object or
    AnisotropicObject on a random box; loss = a random weighting of E^2 and H^2
    at every line and block detector cell over all steps (the detectors'
    samples taken from the fields after each step)."""

    steps = 24

    def __init__(self, seed):
        self.seed = seed
        self.name = f"adj_random_{seed}"

    def build(self, fd):
        import os
        import sys

        tests_dir = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
        if tests_dir not in sys.path:
            sys.path.insert(0, tests_dir)
        from test_fuzz_gpu import random_scene

        grid = random_scene(fd, self.seed, plane_detector=False)
        bd = getattr(fd, "backend", None)
        for o in grid.objects:  # the scene sets anisotropic tensors as numpy arrays
            if bd is not None and isinstance(o.inverse_permittivity, np.ndarray):
                o.inverse_permittivity = bd.array(o.inverse_permittivity)
        rng = np.random.default_rng(self.seed + 9000)
        n = (grid.Nx, grid.Ny, grid.Nz)
        lo = [int(rng.integers(0, max(1, m - 3))) if m > 1 else 0 for m in n]
        hi = [min(m, l + int(rng.integers(1, 4))) for l, m in zip(lo, n)]
        self.box_shape = tuple(h - l for l, h in zip(lo, hi))
        self.aniso = bool(rng.random() < 0.4)
        obj = fd.AnisotropicObject(permittivity=2.0, name="design") if self.aniso else fd.Object(
            permittivity=2.0, name="design")
        grid[tuple(slice(l, h) for l, h in zip(lo, hi))] = obj
        for i, d in enumerate(grid.detectors):
            d.name = f"d{i}"
        return grid, obj

    def design(self):
        rng = np.random.default_rng(self.seed + 9100)
        if self.aniso:
            t = rng.standard_normal(self.box_shape + (3, 3)) * 0.05
            return np.eye(3) * rng.uniform(0.3, 0.7, size=self.box_shape + (1, 1)) + (t + np.swapaxes(t, -1, -2))
        return rng.uniform(0.3, 0.9, size=self.box_shape)

    def weights(self, grid):
        rng = np.random.default_rng(self.seed + 9200)
        return {(d.name, f): rng.uniform(0.0, 1.0, size=3) for d in grid.detectors for f in ("E", "H")}

    @staticmethod
    def _cells(det):
        if type(det).__name__ == "BlockDetector":
            return np.ix_(np.asarray(det.x), np.asarray(det.y), np.asarray(det.z))
        return (np.asarray(det.x), np.asarray(det.y), np.asarray(det.z))

    def ref_loss(self, grid, torch):
        w = {k: torch.as_tensor(v) for k, v in self.weights(grid).items()}
        loss = torch.zeros((), dtype=torch.float64)
        for _ in range(self.steps):
            grid.step()
            for d in grid.detectors:
                cells = tuple(torch.as_tensor(c) for c in self._cells(d))
                loss = loss + ((grid.E[cells].clone() ** 2) * w[(d.name, "E")]).sum()
                loss = loss + ((grid.H[cells].clone() ** 2) * w[(d.name, "H")]).sum()
        return loss

    def detectors(self, fd, grid):
        # the random scene registers its own; the loss weights follow them
        self._weights = self.weights(grid)

    def gb_loss(self, outs, torch):
        total = torch.zeros((), dtype=torch.float64)
        for (name, field), w in self._weights.items():
            x = outs[name][field]
            total = total + ((x.to(torch.float64) ** 2) * torch.as_tensor(w, device=x.device)).sum()
        return total


SCENES = {s.name: s for s in (PlaneScene(), PeriodicScene(True), PeriodicScene(False), AnisoDftScene())}

# random scenes checked on the CPU oracle only (tests/test_adjoint_oracle.py)
RANDOM_SCENES = {s.name: s for s in (RandomScene(seed) for seed in (0, 1, 3, 4, 6, 8, 10, 11, 12))}
