"""Parity of the CUDA time step (through the C ABI) with the reference.

* float64 plans against the golden fixtures made by the reference itself:
  relative L2 <= 1e-12 on E, H and every detector trace (the spec bar).
* float32 and compensated float32 plans against the same fixtures: <= 1e-4.
* larger seeded scenes against the CPU oracle run in-process, with the same
  tolerances, covering every config generator (c1..c5) at reduced size.
* edge behaviour: run/step/half-step equivalence, tiling invariance, plan
  rebuilds, stand-alone curls on the reference's known-answer inputs.
"""

import ctypes
import os

import numpy as np
import pytest
import torch

import golden_scenes
from helpers import rel_l2, to_np
from oracle import fdtd_oracle as fo

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
TOL64 = 1e-12   # float64: relative L2 against the reference numpy float64 backend
TOL32 = 1e-4    # float32 / float32c: relative L2 of detector traces and fields


@pytest.fixture(scope="module", autouse=True)
def native():
    from fdtd_gb300 import _native

    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    return _native.load()


def _compare(snap, ref, tol, label):
    worst = 0.0
    for key in ref.files:
        if key in ("steps",):
            continue
        a, b = snap[key], ref[key]
        assert a.shape == b.shape, f"{label}:{key} shape {a.shape} vs {b.shape}"
        if key == "q":
            assert int(a) == int(b)
            continue
        err = rel_l2(a, b)
        worst = max(worst, err)
        assert err <= tol, f"{label}:{key} relative L2 {err:.3e} > {tol:.0e}"
    return worst


@pytest.mark.parametrize("name", sorted(golden_scenes.SCENES))
def test_float64_matches_reference_golden(fd, name):
    fd.set_backend("gb300.float64")
    grid, steps, drive = golden_scenes.SCENES[name](fd)
    drive(grid, steps)
    ref = np.load(os.path.join(GOLDEN, f"ref_{name}.npz"))
    _compare(golden_scenes.snapshot(grid), ref, TOL64, name)


@pytest.mark.parametrize("name", sorted(set(golden_scenes.SCENES) - {"mix"}))
def test_float64_bit_identical_to_reference_arithmetic(fd, name):
    """Same operation order as the reference: identical bits to the oracle run
    on this host (the oracle is bit-identical to the reference, see
    test_oracle_golden.py) on every golden scene without an anisotropic object.
    Compared on the same host because numpy's exp, used at registration and by
    the "manual" scene's driver, can differ in the last bit between machines."""
    fd.set_backend("gb300.float64")
    grid, steps, drive = golden_scenes.SCENES[name](fd)
    drive(grid, steps)
    ogrid, _, odrive = golden_scenes.SCENES[name](fo)
    odrive(ogrid, steps)
    snap, ref = golden_scenes.snapshot(grid), golden_scenes.snapshot(ogrid)
    for key, val in ref.items():
        assert np.array_equal(snap[key], val), f"{name}:{key} max |diff| {np.abs(snap[key] - val).max()}"


@pytest.mark.parametrize("prec", ["float32", "float32c"])
@pytest.mark.parametrize("name", sorted(golden_scenes.SCENES))
def test_float32_close_to_reference_golden(fd, prec, name):
    fd.set_backend("gb300." + prec)
    grid, steps, drive = golden_scenes.SCENES[name](fd)
    drive(grid, steps)
    ref = np.load(os.path.join(GOLDEN, f"ref_{name}.npz"))
    _compare(golden_scenes.snapshot(grid), ref, TOL32, f"{name}/{prec}")


STAGED_PLANS = [dict(variant=2, pml_mode=1), dict(variant=2, pml_mode=2), dict(variant=2, pml_mode=3)]


@pytest.mark.parametrize("tune", STAGED_PLANS, ids=lambda t: f"pml{t['pml_mode']}")
@pytest.mark.parametrize("prec", ["float64", "float32"])
@pytest.mark.parametrize("name", ["c1", "c3_periodic_first", "c3_periodic_last"])
def test_staged_compact_plans_against_reference_golden(fd, prec, name, tune):
    """The TMA-staged passes reading compact material copies (one-byte
    indices; these scenes have a few permittivity values and nz = 16), with
    the PML slabs fused, split, or partly kept, against the fixtures the
    reference itself made."""
    fd.set_backend("gb300." + prec)
    grid, steps, drive = golden_scenes.SCENES[name](fd)
    eng = grid._ensure_engine()
    eng.set_tuning(**tune)
    assert eng.tiling()["variant"] == 2 and eng.compact_materials()[0] is not None
    drive(grid, steps)
    eng.check_status()
    ref = np.load(os.path.join(GOLDEN, f"ref_{name}.npz"))
    _compare(golden_scenes.snapshot(grid), ref, TOL64 if prec == "float64" else TOL32, f"{name}/{prec}/{tune}")


def _curl_via_abi(native, fn, arr, precision, dtype):
    t = torch.as_tensor(arr, dtype=dtype, device="cuda").contiguous()
    out = torch.empty_like(t)
    nx, ny, nz, _ = t.shape
    rc = fn(precision, t.data_ptr(), out.data_ptr(), nx, ny, nz, None)
    assert rc == 0
    torch.cuda.synchronize()
    return out.cpu().numpy()


def test_curl_functions_on_reference_known_answers(fd):
    """fdtd_gb300.grid.curl_E / curl_H, the counterparts of the reference's
    fdtd.grid.curl_E / curl_H, on the inputs of its known-answer tests."""
    d = np.load(os.path.join(GOLDEN, "ref_curls.npz"))
    assert np.array_equal(fd.grid.curl_E(d["E"]).cpu().numpy(), d["curl_E"])
    assert np.array_equal(fd.grid.curl_H(d["H"]).cpu().numpy(), d["curl_H"])
    c32 = fd.grid.curl_H(torch.as_tensor(d["H"], dtype=torch.float32)).cpu().numpy()
    assert c32.dtype == np.float32 and np.allclose(c32, d["curl_H"], rtol=1e-5, atol=1e-5)


def test_curls_on_reference_known_answers(native):
    d = np.load(os.path.join(GOLDEN, "ref_curls.npz"))
    assert np.array_equal(_curl_via_abi(native, native.fdtd_curl_E, d["E"], 2, torch.float64), d["curl_E"])
    assert np.array_equal(_curl_via_abi(native, native.fdtd_curl_H, d["H"], 2, torch.float64), d["curl_H"])
    c32 = _curl_via_abi(native, native.fdtd_curl_E, d["E"], 0, torch.float32)
    assert np.allclose(c32, d["curl_E"], rtol=1e-5, atol=1e-5)


def test_curls_random_against_oracle(native):
    rng = np.random.default_rng(7)
    for shape in [(5, 7, 9, 3), (16, 4, 32, 3), (1, 6, 1, 3)]:
        a = rng.standard_normal(shape)
        assert np.array_equal(_curl_via_abi(native, native.fdtd_curl_E, a, 2, torch.float64), fo.curl_E(a))
        assert np.array_equal(_curl_via_abi(native, native.fdtd_curl_H, a, 2, torch.float64), fo.curl_H(a))


SCENES = {
    "c1_n32": (lambda fd: fo_scene(fd, "c1", n=32, pml=6), 60),
    "c2_n24": (lambda fd: fo_scene(fd, "c2", n=24, pml=4), 50),
    "c3_n32_periodic_last": (lambda fd: fo_scene(fd, "c3", n=32, pml=5), 50),
    "c3_n32_periodic_first": (lambda fd: fo_scene(fd, "c3", n=32, pml=5, periodic_first=True), 50),
    "c4_n32": (lambda fd: fo_scene(fd, "c4", n=32, pml=4, d=12), 50),
    "c5_small": (lambda fd: fo_scene(fd, "c5", nx=32, ny=28, nz=24, pml=4), 60),
}


def fo_scene(fd, which, **kw):
    from fdtd_gb300 import scenes

    return getattr(scenes, which)(fd, **kw)


def _run_both(fd, prec, key):
    build, steps = SCENES[key]
    fd.set_backend("gb300." + prec)
    g = build(fd)
    g.run(steps, progress_bar=False)
    o = build(fo)
    o.run(steps)
    return g, o


def _dft_or_records(det):
    if hasattr(det, "dft"):
        return to_np(det.dft.real), to_np(det.dft.imag)
    return (np.asarray(det.E), np.asarray(det.H))


@pytest.mark.parametrize("key", sorted(SCENES))
@pytest.mark.parametrize("prec,tol", [("float64", TOL64), ("float32", TOL32), ("float32c", TOL32)])
def test_scenes_against_oracle(fd, key, prec, tol):
    g, o = _run_both(fd, prec, key)
    assert rel_l2(g.E, o.E) <= tol
    assert rel_l2(g.H, o.H) <= tol
    assert len(g.detectors) == len(o.detectors)
    for det, odet in zip(g.detectors, o.detectors):
        mine, theirs = _dft_or_records(det), _dft_or_records(odet)
        for a, b in zip(mine, theirs):
            assert a.shape == np.asarray(b).shape
            assert rel_l2(a, b) <= tol, f"{key}/{prec} {type(det).__name__}"


def test_run_step_and_halves_agree(fd):
    fd.set_backend("gb300.float64")
    build, _ = SCENES["c1_n32"]
    a, b, c = build(fd), build(fd), build(fd)
    a.run(12, progress_bar=False)
    for _ in range(12):
        b.step()
    for _ in range(12):
        c.update_E()
        c.update_H()
        c.time_steps_passed += 1
    for g in (b, c):
        assert torch.equal(a.E, g.E) and torch.equal(a.H, g.H)
        assert np.array_equal(np.asarray(a.detector.E), np.asarray(g.detector.E))


TILINGS = [dict(variant=1, x_chunk=1), dict(variant=1, x_chunk=7), dict(variant=2, tile_rows=8, stages=2),
           dict(variant=2, tile_rows=4, stages=3, x_chunk=5), dict(variant=2, tile_rows=8, stages=3, x_chunk=24),
           dict(variant=1, pml_mode=2), dict(variant=2, tile_rows=8, stages=2, pml_mode=2),
           dict(variant=2, tile_rows=4, stages=3, x_chunk=5, pml_mode=2),
           dict(variant=2, tile_rows=16, stages=2, pml_mode=2), dict(variant=2, tile_rows=16, stages=3, x_chunk=6,
                                                                 pml_mode=2),
           dict(variant=2, tile_rows=8, stages=3, pml_mode=3), dict(variant=1, pml_mode=3, x_chunk=5),
           dict(variant=2, tile_rows=16, stages=2, pml_mode=3),
           dict(variant=2, tile_rows=8, pml_mode=4), dict(variant=2, tile_rows=16, stages=3, x_chunk=5, pml_mode=4),
           dict(variant=2, tile_rows=4, stages=2, pml_mode=4), dict(variant=1, pml_mode=4, x_chunk=3)]

# tiling()["pml_split"] of each PML mode: 1 slab kernels of their own, 2 interior/shell partition
SPLIT_OF_MODE = {2: 1, 3: 1, 4: 2}


@pytest.mark.parametrize("prec", ["float64", "float32", "float32c"])
def test_kernel_variants_and_tiling_agree_bitwise(fd, prec):
    """Register-streaming and TMA-staged kernels, any tile shape and ring depth,
    PML slabs inside the fused pass, in kernels of their own, or in the
    register-streaming pass over the shell boxes around a slab-free interior,
    give identical bits (same per-cell arithmetic, only the data path
    differs).  Compensated float32 renormalises its two-float pair after
    every slab kernel, so there the separate-slab plans agree to round-off
    instead."""
    fd.set_backend("gb300." + prec)
    build, _ = SCENES["c2_n24"]
    ref = build(fd)
    ref._ensure_engine().set_tuning(variant=1, pml_mode=1)
    ref.run(20, progress_bar=False)
    for tune in TILINGS:
        g = build(fd)
        g._ensure_engine().set_tuning(**tune)
        info = g._engine.tiling()
        assert info["variant"] == tune["variant"]
        assert info["pml_split"] == SPLIT_OF_MODE.get(tune.get("pml_mode", 1), 0)
        g.run(20, progress_bar=False)
        if prec == "float32c" and tune.get("pml_mode", 1) in (2, 3):
            assert rel_l2(g.E, ref.E) <= 1e-6 and rel_l2(g.H, ref.H) <= 1e-6, tune
            continue
        assert torch.equal(g.E, ref.E) and torch.equal(g.H, ref.H), tune
        assert np.array_equal(np.asarray(g.detector.E), np.asarray(ref.detector.E)), tune


@pytest.mark.parametrize("tile_rows", [8, 16])
@pytest.mark.parametrize("pml_mode", [1, 2, 3, 4])
@pytest.mark.parametrize("prec", ["float64", "float32"])
def test_tma_variant_on_wide_grid_against_oracle(fd, prec, pml_mode, tile_rows):
    """A grid wider than one TMA tile along z and y (several CTAs, tile edges,
    periodic x, PML on y/z, objects crossing tile borders), PML slabs inside
    the fused pass, in kernels of their own, or in the shell boxes around a
    slab-free interior (objects crossing the interior's faces), 32x8 and
    16x16 tiles."""
    fd.set_backend("gb300." + prec)
    from fdtd_gb300 import scenes

    def build(mod):
        g = mod.Grid((20, 36, 136), grid_spacing=155e-9, permittivity=scenes.c3_permittivity(36, seed=9)[:20, :, :1]
                     * np.ones((1, 1, 136)))
        g[:, 0:4, :] = mod.PML()
        g[:, -3:, :] = mod.PML()
        g[:, :, 0:5] = mod.PML()
        g[:, :, -4:] = mod.PML()
        g[0, :, :] = mod.PeriodicBoundary()
        g[5:15, 2:30, 100:134] = mod.Object(permittivity=3.0)
        g[3:12, 10:20, 60:70] = mod.AbsorbingObject(permittivity=2.0, conductivity=2e4)
        g[10, 18, 68] = mod.PointSource(period=13)
        g[:, 18, 60] = mod.LineDetector()
        return g

    g, o = build(fd), build(fo)
    g._ensure_engine().set_tuning(variant=2, pml_mode=pml_mode, tile_rows=tile_rows)
    assert g._engine.tiling()["variant"] == 2 and g._engine.tiling()["rows_y"] == tile_rows
    assert g._engine.tiling()["pml_split"] == SPLIT_OF_MODE.get(pml_mode, 0)
    g.run(40, progress_bar=False)
    o.run(40)
    tol = TOL64 if prec == "float64" else TOL32
    assert rel_l2(g.E, o.E) <= tol and rel_l2(g.H, o.H) <= tol
    assert rel_l2(np.asarray(g.detectors[0].E), np.stack(o.detectors[0].E)) <= tol


def test_records_survive_plan_rebuild(fd):
    fd.set_backend("gb300.float64")
    build, _ = SCENES["c1_n32"]
    g, o = build(fd), build(fo)
    g.run(5, progress_bar=False)
    o.run(5)
    g[:, 3, 3] = fd.LineDetector(name="late")
    o[:, 3, 3] = fo.LineDetector(name="late")
    g.run(6, progress_bar=False)
    o.run(6)
    assert len(g.detector.E) == 11 and len(g.late.E) == 6
    assert rel_l2(np.asarray(g.detector.E), np.stack(o.detector.E)) <= TOL64
    assert rel_l2(np.asarray(g.late.H), np.stack(o.late.H)) <= TOL64


def test_object_change_between_runs(fd):
    """Assigning an object's inverse permittivity rebuilds its coefficients."""
    fd.set_backend("gb300.float64")
    build, _ = SCENES["c4_n32"]
    g, o = build(fd), build(fo)
    g.run(10, progress_bar=False)
    o.run(10)
    new = np.full(o.objects[0].inverse_permittivity.shape, 0.3)
    g.objects[0].inverse_permittivity = new
    o.objects[0].inverse_permittivity = new.copy()
    g.run(10, progress_bar=False)
    o.run(10)
    assert rel_l2(g.E, o.E) <= TOL64


def test_field_stats_detects_nonfinite(fd):
    fd.set_backend("gb300.float32")
    build, _ = SCENES["c1_n32"]
    g = build(fd)
    g.run(10, progress_bar=False)
    s = g.field_stats()
    e = g.E.double()
    assert s["nonfinite"] == 0
    assert s["sum_E2"] == pytest.approx(float((e * e).sum()), rel=1e-6)
    assert s["max_abs_E"] == pytest.approx(float(e.abs().max()), rel=1e-7)
    g.E[3, 4, 5, 1] = float("nan")
    g.H[1, 1, 1, 0] = float("inf")
    assert g.field_stats()["nonfinite"] == 2


def test_reset_keeps_plan(fd):
    fd.set_backend("gb300.float64")
    build, _ = SCENES["c1_n32"]
    g = build(fd)
    g.run(5, progress_bar=False)
    g.reset()
    assert g.time_steps_passed == 0 and float(g.E.abs().max()) == 0.0
    g.run(3, progress_bar=False)
    assert float(g.E.abs().max()) > 0.0


@pytest.mark.parametrize("name", ["c2", "saps"])
def test_save_data_matches_device_traces_and_reference(fd, name, tmp_path, monkeypatch):
    """Grid.save_data (fdtd/grid.py:490-514): '<name> (E)' and '<name> (H)'
    for every E/H detector, read from the device traces; the saved records
    match the traces and the reference's own records of the scene.  A
    CurrentDetector (on which the reference raises KeyError) stores
    '<name> (I)'."""
    monkeypatch.chdir(tmp_path)
    fd.set_backend("gb300.float64")
    grid, steps, drive = golden_scenes.SCENES[name](fd)
    drive(grid, steps)
    folder = grid.save_simulation("parity")
    grid.save_data()
    got = np.load(os.path.join(folder, "detector_readings.npz"))
    want = np.load(os.path.join(GOLDEN, f"ref_{name}.npz"))
    keys = set()
    for i, det in enumerate(grid.detectors):
        if hasattr(det, "I"):
            keys.add(f"{det.name} (I)")
            assert np.array_equal(got[f"{det.name} (I)"], np.asarray(det.I))
            assert rel_l2(got[f"{det.name} (I)"], want[f"det{i}_I"]) <= TOL64
            continue
        for f in ("E", "H"):
            key = f"{det.name} ({f})"
            keys.add(key)
            assert np.array_equal(got[key], np.asarray(getattr(det, f)))
            assert got[key].shape == want[f"det{i}_{f}"].shape
            assert rel_l2(got[key], want[f"det{i}_{f}"]) <= TOL64
    assert set(got.files) == keys
