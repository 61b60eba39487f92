"""Small scenes whose reference outputs are committed as golden fixtures.

Each builder takes an fdtd-like module ``fd`` and returns ``(grid, steps, driver)``
where ``driver(grid, steps)`` advances the grid the way the scene is meant to
be run (``grid.run`` or a manual half-step loop).  The same builders run on the
reference package (``make_golden.py``), on the CPU oracle and on the GPU
backend, so parity is checked on identical inputs.
"""

import numpy as np

from fdtd_gb300 import scenes

C0 = 299792458.0


def run_steps(grid, steps):
    grid.run(steps, progress_bar=False)


def g_c1(fd):
    """Config 1 at 16^3 with 4-cell PML."""
    return scenes.c1(fd, n=16, pml=4), 40, run_steps


def g_c2(fd):
    """Config 2 geometry at 16^3: random uniaxial medium, absorber, plane source."""
    return scenes.c2(fd, n=16, pml=3), 30, run_steps


def g_c3_periodic_first(fd):
    """Config 3 generator at 16^3, periodic x registered before the PMLs."""
    return scenes.c3(fd, n=16, pml=3, periodic_first=True), 30, run_steps


def g_c3_periodic_last(fd):
    """Config 3 generator at 16^3, periodic x registered after the PMLs."""
    return scenes.c3(fd, n=16, pml=3, periodic_first=False), 30, run_steps


def g_mix(fd):
    """Non-cubic grid (Nz not a multiple of 4) with overlapping objects and
    every source kind: composition order, hard/soft source order, slab overlaps."""
    rng = np.random.default_rng(11)
    eps = rng.uniform(1.0, 4.0, size=(14, 12, 11))
    grid = fd.Grid((14, 12, 11), grid_spacing=100e-9, permittivity=eps,
                   permeability=rng.uniform(1.0, 1.5, size=(14, 12, 11, 3)))
    grid[0:4, :, :] = fd.PML(name="pml_xlow")
    grid[:, -3:, :] = fd.PML(name="pml_yhigh")
    grid[:, :, 0:3] = fd.PML(name="pml_zlow")
    grid[:, :, -2:] = fd.PML(name="pml_zhigh", a=1e-6)
    grid[2:9, 3:10, 2:8] = fd.Object(permittivity=rng.uniform(1.5, 3.0, size=(7, 7, 6, 3)), name="o1")
    grid[6:12, 1:6, 4:10] = fd.AbsorbingObject(permittivity=2.0,
                                               conductivity=rng.uniform(1e3, 5e4, size=(6, 5, 6)),
                                               name="o2")
    aniso = fd.AnisotropicObject(permittivity=2.5, name="o3")
    grid[7:11, 6:10, 3:7] = aniso
    t = rng.standard_normal((4, 4, 4, 3, 3)) * 0.05
    aniso.inverse_permittivity = _np(aniso.inverse_permittivity) + (t + np.swapaxes(t, -1, -2))
    grid[3:11, 2:9, 5] = fd.LineSource(period=12, pulse=True, cycle=3, hanning_dt=2.0, name="ls")
    grid[5, 5, 5] = fd.PointSource(period=9, amplitude=0.7, phase_shift=0.3, name="ps")
    grid[4, :, :] = fd.PlaneSource(period=15, amplitude=0.5, polarization="y", name="plane")
    grid[1:13, 2:10, 1:9] = fd.LineDetector(name="line")
    grid[9:11, 3:5, 6:8] = fd.BlockDetector(name="block")
    return grid, 30, run_steps


def g_2d(fd):
    """2D grid (Nz = 1): courant 0.99/sqrt(2), periodic z on a single plane."""
    grid = fd.Grid((30, 24, 1), grid_spacing=155e-9, permittivity=1.0)
    grid[0:5, :, :] = fd.PML(name="pml_xlow")
    grid[-5:, :, :] = fd.PML(name="pml_xhigh")
    grid[:, 0:4, :] = fd.PML(name="pml_ylow")
    grid[:, -4:, :] = fd.PML(name="pml_yhigh")
    grid[:, :, 0] = fd.PeriodicBoundary(name="zbounds")
    grid[12:20, 8:16, 0] = fd.Object(permittivity=1.7 ** 2, name="object")
    grid[20:26, 14:20, 0] = fd.AbsorbingObject(permittivity=2.5, conductivity=1e5, name="absorber")
    grid[7:9, 6:18, 0] = fd.LineSource(period=1550e-9 / C0, name="source")
    grid[22, :, 0] = fd.LineDetector(name="detector")
    grid[10:12, 10:13, 0:0] = fd.BlockDetector(name="block")
    return grid, 40, run_steps


def g_manual(fd):
    """Half-step API with a write into grid.E between the halves
    (the driving pattern of the reference's current-detector test)."""
    grid = fd.Grid((10, 10, 10), grid_spacing=100e-9)
    grid[0:2, :, :] = fd.PML(name="pml")
    grid[3:5, 3:5, 3:5] = fd.AbsorbingObject(permittivity=1.0, conductivity=1e7)
    grid[4:4, 4:4, 4:4] = fd.BlockDetector(name="block")

    def drive(g, steps):
        for q in range(steps):
            g.update_E()
            g.E[4, 4, 4, 2] = float(np.exp(-((q - 8.0) ** 2) / 8.0))
            g.update_H()
            g.time_steps_passed += 1

    return grid, 20, drive


def g_domain_pml(fd):
    """DomainBorderPML plus a pulsed point source."""
    grid = fd.Grid((14, 13, 12), grid_spacing=155e-9)
    fd.DomainBorderPML(grid, border_cells=3)
    grid[7, 6, 6] = fd.PointSource(period=10, pulse=True, cycle=4, hanning_dt=1.5, name="ps")
    grid[:, 6, 6] = fd.LineDetector(name="detector")
    return grid, 30, run_steps


def g_saps(fd):
    """SoftArbitraryPointSource with a source impedance (the current measured
    by its own CurrentDetector feeds back into the next E half step), a
    separate CurrentDetector block, a conducting plate and a line detector in
    a PML box with millimetre cells (the setting of the reference's impedance
    test, tests/test_antenna_impedance.py).  The impedance, 0.2, keeps the
    feedback loop stable: in the reference's field units the loop gain grows
    with the impedance and at 1 or more the fields grow without bound."""
    grid = fd.Grid((14, 12, 12), grid_spacing=1e-3)
    fd.DomainBorderPML(grid, border_cells=3)
    grid[4:10, 4:8, 5:6] = fd.AbsorbingObject(permittivity=1.0, conductivity=1e6, name="plate")
    t = np.arange(60) * grid.time_step
    wave = np.exp(-((t - 25 * grid.time_step) ** 2) / (2 * (6 * grid.time_step) ** 2))
    grid[7, 6, 7] = fd.SoftArbitraryPointSource(wave, impedance=0.2)
    grid[5:7, 3:5, 8] = fd.CurrentDetector(name="current")
    grid[:, 6, 7] = fd.LineDetector(name="line")
    return grid, 60, run_steps


SCENES = {
    "c1": g_c1,
    "c2": g_c2,
    "c3_periodic_first": g_c3_periodic_first,
    "c3_periodic_last": g_c3_periodic_last,
    "mix": g_mix,
    "2d": g_2d,
    "manual": g_manual,
    "domain_pml": g_domain_pml,
    "saps": g_saps,
}


def snapshot(grid):
    """Final fields and every detector trace as float64 numpy arrays."""
    out = {"E": _np(grid.E), "H": _np(grid.H), "q": np.array(grid.time_steps_passed)}
    for i, det in enumerate(grid.detectors):
        if hasattr(det, "I"):  # CurrentDetector
            out[f"det{i}_I"] = np.stack([_np(c) for c in det.I]) if len(det.I) else np.zeros((0,))
            continue
        out[f"det{i}_E"] = np.stack([_np(e) for e in det.E]) if len(det.E) else np.zeros((0,))
        out[f"det{i}_H"] = np.stack([_np(h) for h in det.H]) if len(det.H) else np.zeros((0,))
    for j, src in enumerate(grid.sources):
        if hasattr(src, "source_voltage"):  # SoftArbitraryPointSource
            out[f"src{j}_Vin"] = _np(src.input_voltage)
            out[f"src{j}_Vout"] = _np(src.source_voltage)
    return out


def _np(a):
    if hasattr(a, "detach"):
        return a.detach().cpu().numpy().astype(np.float64)
    return np.asarray(a, dtype=np.float64)
