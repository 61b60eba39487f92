"""Seeded random scenes: the CUDA time step against the CPU oracle.

Every scene draws a grid shape (odd and even nz, sometimes 2D), a random or a
few-valued permittivity (the latter read through compact material copies by
the staged passes), PML slabs and
periodic boundaries on random axes in a random registration order, up to
three overlapping objects of all kinds, point, line and plane sources,
line/block/plane detectors, and a plan choice (kernel variant, PML mode, tile
rows, x chunk, material copies).  float64 must match the oracle to 1e-12 relative L2, float32
and compensated float32 to 1e-4, on E, H and every detector trace.
"""

import os

import numpy as np
import pytest

from helpers import rel_l2
from oracle import fdtd_oracle as fo

pytestmark = pytest.mark.gpu


def random_scene(mod, seed, plane_detector=True):
    """The scene of a seed; without the PlaneDetector (not a reference
    component) it also builds on the reference package."""
    rng = np.random.default_rng(seed)
    side = np.random.default_rng(seed + 2000)  # draws added later, kept off the main stream
    nz = int(rng.choice([1, 7, 8, 12, 13, 16]))
    if nz == 16 and side.random() < 0.5:
        nz = 32
    nx, ny = int(rng.integers(8, 19)), int(rng.integers(8, 19))
    eps = rng.uniform(1.0, 3.0, size=(nx, ny, nz))
    if side.random() < 0.5:
        eps = np.round(eps * 2.0) / 2.0  # a few distinct values: compact material copies
    grid = mod.Grid((nx, ny, nz), grid_spacing=120e-9, permittivity=eps)
    n = (nx, ny, nz)
    # boundaries: per axis none / PML on one or both sides / periodic
    entries = []
    for a in range(3):
        kind = rng.choice(["none", "pml_lo", "pml_hi", "pml_both", "periodic"]) if n[a] > 6 else "none"
        if a == 2 and nz == 1:
            kind = rng.choice(["none", "periodic"])
        if kind.startswith("pml"):
            for side in (["lo", "hi"] if kind == "pml_both" else [kind[-2:]]):
                th = int(rng.integers(2, 4))
                sl = [slice(None)] * 3
                sl[a] = slice(0, th) if side == "lo" else slice(-th, None)
                entries.append((tuple(sl), "pml", float(rng.choice([1e-8, 1e-6]))))
        elif kind == "periodic":
            sl = [slice(None)] * 3
            sl[a] = 0
            entries.append((tuple(sl), "periodic", None))
    rng.shuffle(entries)
    for sl, kind, a in entries:
        grid[sl] = mod.PML(a=a) if kind == "pml" else mod.PeriodicBoundary()

    def box():
        lo = [int(rng.integers(0, m - 1)) if m > 1 else 0 for m in n]
        hi = [min(m, l + int(rng.integers(1, 5))) for l, m in zip(lo, n)]
        return tuple(slice(l, h) for l, h in zip(lo, hi)), tuple(h - l for l, h in zip(lo, hi))

    for _ in range(int(rng.integers(0, 4))):
        sl, shp = box()
        kind = rng.choice(["object", "absorbing", "anisotropic"])
        if kind == "object":
            grid[sl] = mod.Object(permittivity=rng.uniform(1.2, 3.0, size=shp + (3,)))
        elif kind == "absorbing":
            grid[sl] = mod.AbsorbingObject(permittivity=float(rng.uniform(1.0, 2.5)),
                                           conductivity=rng.uniform(1e3, 5e4, size=shp))
        else:
            obj = mod.AnisotropicObject(permittivity=float(rng.uniform(1.5, 2.5)))
            grid[sl] = obj
            t = rng.standard_normal(shp + (3, 3)) * 0.03
            ie = obj.inverse_permittivity
            ie = ie.detach().cpu().numpy() if hasattr(ie, "detach") else ie
            obj.inverse_permittivity = ie + (t + np.swapaxes(t, -1, -2))
    # sources
    p = [int(rng.integers(0, m)) for m in n]
    grid[p[0], p[1], p[2]] = mod.PointSource(period=int(rng.integers(8, 20)), amplitude=float(rng.uniform(0.5, 1.5)))
    if nx > 4 and rng.random() < 0.7:
        x0 = int(rng.integers(0, nx - 3))
        grid[x0:x0 + 3, p[1], p[2]] = mod.LineSource(period=int(rng.integers(8, 20)), pulse=bool(rng.random() < 0.5),
                                                    cycle=3, hanning_dt=1.5)
    if rng.random() < 0.6:
        a = int(rng.integers(0, 3)) if nz > 1 else 2  # in 2D only the z plane has one flat axis
        pol = "xyz"[int(rng.choice([q for q in range(3) if q != a]))]
        sl = [slice(None)] * 3
        sl[a] = int(rng.integers(0, n[a]))
        grid[tuple(sl)] = mod.PlaneSource(period=int(rng.integers(8, 20)), amplitude=0.7, polarization=pol)
    # detectors
    grid[:, p[1], p[2]] = mod.LineDetector()
    b0 = [int(rng.integers(0, max(1, m - 2))) for m in n]
    grid[b0[0]:b0[0] + 1, b0[1]:b0[1] + 1, b0[2]:b0[2] + (1 if nz > 1 else 0)] = mod.BlockDetector()
    if plane_detector:
        grid[:, :, int(rng.integers(0, nz))] = mod.PlaneDetector()
    return grid


def random_tuning(seed, nz, precision):
    rng = np.random.default_rng(seed + 1000)
    vmax = 2 if precision == "float64" else 4
    tune = {"pml_mode": int(rng.integers(0, 4)), "x_chunk": int(rng.choice([0, 3, 5])),
            "materials": int(np.random.default_rng(seed + 3000).integers(0, 2))}
    if nz % vmax == 0 and rng.random() < 0.5:
        tune.update(variant=2, tile_rows=int(rng.choice([4, 8, 16])), stages=int(rng.choice([2, 3])))
    else:
        tune.update(variant=1)
    return tune


# FDTD_FUZZ_SEEDS widens the sweep (e.g. 400 for a longer soak)
SEEDS = list(range(int(os.environ.get("FDTD_FUZZ_SEEDS", "40"))))


@pytest.mark.parametrize("precision", ["float64", "float32", "float32c"])
@pytest.mark.parametrize("seed", SEEDS)
def test_random_scene_matches_oracle(fd, seed, precision):
    fd.set_backend("gb300." + precision)
    g = random_scene(fd, seed)
    o = random_scene(fo, seed)
    tune = random_tuning(seed, g.Nz, precision)
    eng = g._ensure_engine()
    try:
        eng.set_tuning(**tune)
    except RuntimeError:
        # a staged tile that the slab count or shared memory does not allow
        tune = {"variant": 1, "pml_mode": tune["pml_mode"], "materials": tune["materials"]}
        eng.set_tuning(variant=1, tile_rows=0, stages=0)
    steps = 15
    g.run(steps, progress_bar=False)
    o.run(steps)
    tol = 1e-12 if precision == "float64" else 1e-4
    label = f"seed {seed} {precision} {tune}"
    assert rel_l2(g.E, o.E) <= tol, label
    assert rel_l2(g.H, o.H) <= tol, label
    for d, od in zip(g.detectors, o.detectors):
        if hasattr(d, "E"):
            assert rel_l2(np.asarray(d.E), np.stack(od.E)) <= tol, label + f" {d!r}"
            assert rel_l2(np.asarray(d.H), np.stack(od.H)) <= tol, label + f" {d!r}"
