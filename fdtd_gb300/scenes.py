"""Synthetic benchmark and parity scenes.

Every builder takes an ``fd`` module that exposes the fdtd API (``Grid``,
``PML``, ``PeriodicBoundary``, the objects, sources and detectors) and builds
the scene through that API only, so the same function drives this package,
the CPU oracle used by the tests and the reference package itself.  All random
inputs come from ``numpy.random.default_rng(seed)``; sizes scale with ``n`` so
that the full-size workloads and their small parity crops share one generator.

Scenes (full sizes):
  c1  64^3 vacuum, 10-cell PML on six faces, Object eps=2.25 at 24:40,
      PointSource at the centre, LineDetector along x.
  c2  256^3 uniaxial random medium eps ~ U[1,12] smoothed by a 3-cell box
      filter, 16-cell PML, AbsorbingObject 64^3 (sigma = 1e4 S/m) at the
      centre, PlaneSource at z=20 (x-polarised), 32^3 BlockDetector.
  c3  768^3, 400 random blocks eps in {1, 2.25, 12.1} rasterised into the
      grid permittivity (last writer wins), 20-cell PML on y and z, periodic x,
      PointSource at the centre.
  c4  128^3, 12-cell PML, 48^3 design Object with inverse permittivity
      ~ U[1/12, 1], PlaneSource at z=16, PlaneDetector at z=110.
  c5  384x384x192, 20-cell PML, 96x96x48 AnisotropicObject with random SPD
      permittivity (eigenvalues U[2,6]), Gaussian-modulated PlaneSource near
      z=24, DFT plane detector near z=168 at 1500/1550/1600 nm.
"""

import numpy as np

C0 = 299792458.0
WAVELENGTH = 1550e-9
SPACING = 155e-9


def _scale(v, n, full):
    return int(round(v * n / full))


def pml6(fd, grid, t):
    """Six PML slabs of thickness ``t`` (x, y, z low/high, in that order)."""
    grid[0:t, :, :] = fd.PML(name="pml_xlow")
    grid[-t:, :, :] = fd.PML(name="pml_xhigh")
    grid[:, 0:t, :] = fd.PML(name="pml_ylow")
    grid[:, -t:, :] = fd.PML(name="pml_yhigh")
    grid[:, :, 0:t] = fd.PML(name="pml_zlow")
    grid[:, :, -t:] = fd.PML(name="pml_zhigh")


def c1(fd, n=64, pml=10):
    grid = fd.Grid((n, n, n), grid_spacing=SPACING, permittivity=1.0, permeability=1.0)
    pml6(fd, grid, pml)
    a, b = _scale(24, n, 64), _scale(40, n, 64)
    grid[a:b, a:b, a:b] = fd.Object(permittivity=2.25, name="object")
    c = n // 2
    grid[c, c, c] = fd.PointSource(period=WAVELENGTH / C0, amplitude=1.0, name="source")
    grid[:, c, c] = fd.LineDetector(name="detector")
    return grid


def c2_permittivity(n, seed=2):
    from scipy.ndimage import uniform_filter

    rng = np.random.default_rng(seed)
    eps = rng.uniform(1.0, 12.0, size=(n, n, n, 3))
    return uniform_filter(eps, size=(3, 3, 3, 1), mode="nearest")


def c2(fd, n=256, pml=16, seed=2, conductivity=1e4, eps=None):
    if eps is None:
        eps = c2_permittivity(n, seed)
    grid = fd.Grid((n, n, n), grid_spacing=SPACING, permittivity=eps, permeability=1.0)
    pml6(fd, grid, pml)
    a, b = _scale(96, n, 256), _scale(160, n, 256)
    grid[a:b, a:b, a:b] = fd.AbsorbingObject(permittivity=eps[a:b, a:b, a:b],
                                             conductivity=conductivity, name="absorber")
    grid[:, :, _scale(20, n, 256)] = fd.PlaneSource(period=WAVELENGTH / C0, polarization="x",
                                                    name="source")
    lo, hi = _scale(112, n, 256), _scale(144, n, 256)
    zlo, zhi = _scale(200, n, 256), _scale(232, n, 256)
    grid[lo:hi, lo:hi, zlo:zhi] = fd.BlockDetector(name="detector")
    return grid


def c3_permittivity(n, seed=3, nblocks=400, device=None):
    """400 random axis-aligned blocks rasterised in seed order (last writer wins).

    With ``device`` the (n, n, n) float64 array is a torch tensor built on that
    device (same values; avoids a multi-GB host array at full size)."""
    rng = np.random.default_rng(seed)
    if device is not None:
        import torch

        eps = torch.ones((n, n, n), dtype=torch.float64, device=device)
    else:
        eps = np.ones((n, n, n), dtype=np.float64)
    values = np.array([1.0, 2.25, 12.1])
    for _ in range(nblocks):
        edges = rng.integers(8, 65, size=3)
        edges = np.maximum(2, np.rint(edges * n / 768.0)).astype(int)
        origin = [int(rng.integers(0, n - e + 1)) for e in edges]
        val = float(values[int(rng.integers(0, 3))])
        eps[origin[0]:origin[0] + edges[0], origin[1]:origin[1] + edges[1],
            origin[2]:origin[2] + edges[2]] = val
    return eps


def c3(fd, n=768, pml=20, seed=3, periodic_first=False, eps=None, detector=False):
    if eps is None:
        eps = c3_permittivity(n, seed)
    grid = fd.Grid((n, n, n), grid_spacing=SPACING, permittivity=eps, permeability=1.0)
    if periodic_first:
        grid[0, :, :] = fd.PeriodicBoundary(name="xbounds")
    if pml:
        grid[:, 0:pml, :] = fd.PML(name="pml_ylow")
        grid[:, -pml:, :] = fd.PML(name="pml_yhigh")
        grid[:, :, 0:pml] = fd.PML(name="pml_zlow")
        grid[:, :, -pml:] = fd.PML(name="pml_zhigh")
    if not periodic_first:
        grid[0, :, :] = fd.PeriodicBoundary(name="xbounds")
    c = n // 2
    grid[c, c, c] = fd.PointSource(period=WAVELENGTH / C0, name="source")
    if detector:
        grid[:, c, c] = fd.LineDetector(name="detector")
    return grid


def c4_design(d, seed=4):
    rng = np.random.default_rng(seed)
    return rng.uniform(1.0 / 12.0, 1.0, size=(d, d, d))


def c4(fd, n=128, pml=12, d=48, seed=4, plane_detector=True):
    grid = fd.Grid((n, n, n), grid_spacing=SPACING)
    pml6(fd, grid, pml)
    a = (n - d) // 2
    inv = c4_design(d, seed)
    grid[a:a + d, a:a + d, a:a + d] = fd.Object(permittivity=1.0 / inv, name="design")
    grid[:, :, _scale(16, n, 128)] = fd.PlaneSource(period=WAVELENGTH / C0, polarization="x",
                                                    name="source")
    if plane_detector:
        grid[:, :, _scale(110, n, 128)] = fd.PlaneDetector(name="detector")
    return grid


def c5_tensors(nx, ny, nz, seed=5):
    """Random SPD inverse permittivities Q diag(1/lambda) Q^T, lambda ~ U[2,6]."""
    rng = np.random.default_rng(seed)
    m = nx * ny * nz
    lam = rng.uniform(2.0, 6.0, size=(m, 3))
    g = rng.standard_normal(size=(m, 3, 3))
    q, _ = np.linalg.qr(g)
    inv = np.einsum("nij,nj,nkj->nik", q, 1.0 / lam, q)
    return inv.reshape(nx, ny, nz, 3, 3)


def c5(fd, nx=384, ny=384, nz=192, pml=20, seed=5, dft=True):
    grid = fd.Grid((nx, ny, nz), grid_spacing=SPACING)
    pml6(fd, grid, pml)
    ox, oy, oz = nx // 4, ny // 4, nz // 4
    dx, dy, dz = nx // 4, ny // 4, nz // 4
    obj = fd.AnisotropicObject(permittivity=3.0, name="design")
    grid[2 * ox - dx // 2:2 * ox + dx // 2, 2 * oy - dy // 2:2 * oy + dy // 2,
         2 * oz - dz // 2:2 * oz + dz // 2] = obj
    obj.inverse_permittivity = c5_tensors(obj.Nx, obj.Ny, obj.Nz, seed)
    grid[:, :, _scale(24, nz, 192)] = fd.GaussianPlaneSource(
        period=WAVELENGTH / C0, polarization="x", name="source")
    if dft:
        grid[:, :, _scale(168, nz, 192)] = fd.DFTPlaneDetector(
            wavelengths=[1500e-9, 1550e-9, 1600e-9], name="dft")
    return grid

