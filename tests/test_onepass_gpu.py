"""One pass per time step (float32): the fused E+H pass against the two-pass
plans, bit for bit.

The one-pass kernel (fdtd_gb300/csrc/fdtd_onepass.cuh) reads the old fields
from one buffer and writes the new ones to another, recomputing the new E one
row, one cell and one plane past each tile.  Its per-cell arithmetic is the
two-pass kernels', so E, H, every detector record and every DFT accumulator
must be identical to the two-pass plan's after any number of steps (an odd
count ends with one two-pass step), for every tile height, ring depth and x
chunk -- chunks of one plane exercise the staged plane before a chunk and the
recomputed plane after it on every CTA, and the first chunk's periodic
prologue.  The two-pass plans are tested against the reference's fixtures and
the oracle elsewhere; the fixtures are checked here as well.
"""

import os

import numpy as np
import pytest

import golden_scenes
from fdtd_gb300 import scenes
from helpers import rel_l2, to_np

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _wide(fd):
    """Several tiles along y and z, periodic x after y/z PML slabs, objects of
    all three kinds crossing tile edges, soft point and line sources, hard
    plane source, line, block, plane and DFT detectors."""
    eps = scenes.c3_permittivity(40, seed=9)[:22, :37, :1] * np.ones((1, 1, 136))
    g = fd.Grid((22, 37, 136), grid_spacing=155e-9, permittivity=eps)
    g[:, 0:4, :] = fd.PML(name="pyl")
    g[:, -3:, :] = fd.PML(name="pyh")
    g[:, :, 0:5] = fd.PML(name="pzl")
    g[:, :, -6:] = fd.PML(name="pzh", a=1e-6)
    g[0, :, :] = fd.PeriodicBoundary(name="px")
    g[4:15, 6:30, 100:132] = fd.Object(permittivity=3.0, name="o1")
    g[3:12, 7:21, 120:130] = fd.AbsorbingObject(permittivity=2.0, conductivity=2e4, name="o2")
    a = fd.AnisotropicObject(permittivity=2.5, name="o3")
    g[9:14, 5:13, 124:132] = a
    t = np.random.default_rng(3).standard_normal((5, 8, 8, 3, 3)) * 0.05
    a.inverse_permittivity = np.asarray(a.inverse_permittivity.cpu()) + (t + np.swapaxes(t, -1, -2))
    g[10, 18, 68] = fd.PointSource(period=13, name="ps")
    g[3:17, 9, 60:74] = fd.LineSource(period=11, name="ls")
    g[5:18, 2:35, 90] = fd.PlaneSource(period=9, polarization="x", name="plane")
    g[:, 18, 60] = fd.LineDetector(name="line")
    g[2:5, 7:9, 126:129] = fd.BlockDetector(name="block")
    g[:, :, 100] = fd.PlaneDetector(name="pd")
    g[:, :, 70] = fd.DFTPlaneDetector(frequencies=[3e14, 4e14], name="dft")
    return g


SCENES = {
    "c3_64": lambda fd: scenes.c3(fd, n=64, pml=4, detector=True),  # y/z PML, periodic x last
    "c1_48": lambda fd: scenes.c1(fd, n=48, pml=6),                  # six faces (x slabs), Object
    "c2_32": lambda fd: scenes.c2(fd, n=32, pml=4),                  # random eps, absorber, plane source
    "c5_small": lambda fd: scenes.c5(fd, nx=40, ny=36, nz=32, pml=5),  # anisotropic, Gaussian source, DFT
    "wide": _wide,
}

PLANS = [dict(), dict(tile_rows=4), dict(tile_rows=8, stages=3), dict(tile_rows=4, stages=4, x_chunk=5),
         dict(tile_rows=8, x_chunk=1), dict(tile_rows=4, x_chunk=2), dict(tile_rows=4, x_chunk=1),
         dict(x_chunk=4096)]


def _outputs(g):
    out = {"E": to_np(g.E), "H": to_np(g.H)}
    for i, det in enumerate(g.detectors):
        if hasattr(det, "dft"):
            out[f"d{i}_dft"] = det.dft.detach().cpu().numpy()
        else:
            out[f"d{i}_E"] = to_np(det.E.tensor())
            out[f"d{i}_H"] = to_np(det.H.tensor())
    return out


@pytest.mark.parametrize("steps", [12, 7])
@pytest.mark.parametrize("name", sorted(SCENES))
def test_onepass_bitwise_equals_two_pass(fd, name, steps):
    fd.set_backend("gb300.float32")
    ref = SCENES[name](fd)
    ref._ensure_engine().set_tuning(step_fusion=1)
    ref.run(steps, progress_bar=False)
    want = _outputs(ref)
    ran = 0
    for plan in PLANS:
        g = SCENES[name](fd)
        eng = g._ensure_engine()
        try:
            eng.set_tuning(step_fusion=2, **plan)
        except RuntimeError as exc:
            # 8-row tiles or deep rings with slabs on every axis (or full
            # material tiles) need more shared memory than an SM has
            assert "shared memory" in str(exc) and (plan.get("tile_rows") == 8 or "stages" in plan), (plan, exc)
            continue
        assert eng.step_fusion() == (True, True), plan
        ran += 1
        info = eng.tiling()
        assert info["variant"] == 4 and (plan.get("tile_rows") in (None, info["rows_y"])), info
        g.run(steps, progress_bar=False)
        eng.check_status()
        got = _outputs(g)
        for key, val in want.items():
            assert np.array_equal(got[key], val), f"{name} {plan} {key}: max |diff| {np.abs(got[key] - val).max()}"
    assert ran >= 4


def test_onepass_runs_and_single_steps_mix(fd):
    """run() in pairs, single steps, half steps with writes between them and
    runs again: the same bits as the two-pass plan."""
    fd.set_backend("gb300.float32")
    grids = [SCENES["wide"](fd) for _ in range(2)]
    grids[0]._ensure_engine().set_tuning(step_fusion=1)
    grids[1]._ensure_engine().set_tuning(step_fusion=2, x_chunk=3)
    for g in grids:
        g.run(5, progress_bar=False)
        g.step()
        g.update_E()
        g.E[7, 20, 64, 2] += 0.25
        g.update_H()
        g.time_steps_passed += 1
        g.run(4, progress_bar=False)
    a, b = _outputs(grids[0]), _outputs(grids[1])
    for key in a:
        assert np.array_equal(a[key], b[key]), key


@pytest.mark.parametrize("name", ["c1", "c2", "c3_periodic_last", "2d", "manual"])
def test_onepass_against_reference_golden(fd, name):
    """Scenes of the reference's own fixtures that allow one pass per step."""
    fd.set_backend("gb300.float32")
    grid, steps, drive = golden_scenes.SCENES[name](fd)
    eng = grid._ensure_engine()
    allowed, _ = eng.step_fusion()
    if not allowed:
        pytest.skip(f"{name} does not allow one pass per step")
    eng.set_tuning(step_fusion=2)
    drive(grid, steps)
    eng.check_status()
    ref = np.load(os.path.join(GOLDEN, f"ref_{name}.npz"))
    snap = golden_scenes.snapshot(grid)
    for key in ref.files:
        if key in ("steps", "q"):
            continue
        assert rel_l2(snap[key], ref[key]) <= 1e-4, key


def test_onepass_not_allowed_cases(fd):
    """Grids the one-pass step does not take run on the two-pass plans;
    asking for it there raises."""
    fd.set_backend("gb300.float32")
    g = fd.Grid((16, 16, 16), grid_spacing=155e-9)
    g[0, :, :] = fd.PeriodicBoundary()
    g[:, 0:3, :] = fd.PML()  # a PML after the periodic boundary
    eng = g._ensure_engine()
    assert eng.step_fusion() == (False, False)
    with pytest.raises(RuntimeError):
        eng.set_tuning(step_fusion=2)
    fd.set_backend("gb300.float64")
    g = scenes.c3(fd, n=32, pml=3)
    assert g._ensure_engine().step_fusion() == (False, False)
