"""Compact material copies on the GPU.

The staged passes can read a one-byte index per cell into a shared-memory
table of the distinct inverse-material triples, or nothing when the material
is uniform, instead of three values per cell.  The values and the arithmetic
are unchanged, so E, H and every detector trace must be bit-identical to the
same plan reading the full arrays, and match the oracle (float64 1e-12,
float32 1e-4 relative L2).  In-place changes of the materials between runs
must be followed.
"""

import ctypes

import numpy as np
import pytest
import torch

from helpers import rel_l2
from oracle import fdtd_oracle as fo

pytestmark = pytest.mark.gpu

TOL = {"float64": 1e-12, "float32": 1e-4, "float32c": 1e-4}


def scene(mod, nz=32, levels=True, objects=True, pml=True):
    nx, ny = 20, 18
    rng = np.random.default_rng(7)
    eps = rng.choice([1.0, 1.5, 2.25, 3.0], size=(nx, ny, nz)) if levels else 1.0
    grid = mod.Grid((nx, ny, nz), grid_spacing=100e-9, permittivity=eps, permeability=1.0)
    if pml:
        grid[0:3, :, :] = mod.PML(name="pxlo")
        grid[-3:, :, :] = mod.PML(name="pxhi")
        grid[:, :, -4:] = mod.PML(name="pzhi")
    grid[:, 0, :] = mod.PeriodicBoundary(name="py")
    if objects:
        grid[5:9, 4:10, 6:14] = mod.Object(permittivity=2.0, name="obj")
        grid[11:14, 9:13, 12:20] = mod.AbsorbingObject(permittivity=1.5, conductivity=2e4, name="absorber")
        grid[7:10, 12:16, 18:24] = mod.AnisotropicObject(permittivity=2.5, name="aniso")
    grid[10, 9, 16] = mod.PointSource(period=14, name="src")
    grid[:, :, 9] = mod.PlaneSource(period=18, amplitude=0.5, polarization="x", name="plane")
    grid[4:16, 9, 16] = mod.LineDetector(name="line")
    grid[8:10, 8:10, 20:22] = mod.BlockDetector(name="block")
    return grid


def _records(grid):
    out = [grid.E, grid.H]
    for d in grid.detectors:
        out += [torch.as_tensor(np.asarray(d.E)), torch.as_tensor(np.asarray(d.H))]
    return [torch.as_tensor(t).detach().cpu() for t in out]


def _bits(t):
    return t.view(torch.int32 if t.dtype == torch.float32 else torch.int64)


def _run(fd, precision, tune, materials, steps=20, **kw):
    fd.set_backend("gb300." + precision)
    g = scene(fd, **kw)
    eng = g._ensure_engine()
    eng.set_tuning(variant=2, materials=materials, **tune)
    g.run(steps, progress_bar=False)
    eng.check_status()
    return g, eng


TUNES = [dict(tile_rows=8, pml_mode=1), dict(tile_rows=4, pml_mode=2), dict(tile_rows=16, pml_mode=2),
         dict(tile_rows=8, pml_mode=2, stages=2)]


@pytest.mark.parametrize("tune", TUNES, ids=lambda t: "-".join(f"{k}{v}" for k, v in t.items()))
@pytest.mark.parametrize("precision", ["float64", "float32", "float32c"])
def test_index_materials_bit_identical_to_full(fd, precision, tune):
    g, eng = _run(fd, precision, tune, materials=0)
    modes = eng.compact_materials()
    assert modes[0][0] == "index" and modes[1] == ("uniform", 1), modes
    assert eng.tiling()["variant"] == 2
    f, feng = _run(fd, precision, tune, materials=1)
    assert feng.compact_materials() == [None, None]
    for a, b in zip(_records(g), _records(f)):
        assert torch.equal(_bits(a), _bits(b))
    o = scene(fo)
    o.run(20)
    assert rel_l2(g.E, o.E) <= TOL[precision] and rel_l2(g.H, o.H) <= TOL[precision]
    for d, od in zip(g.detectors, o.detectors):
        assert rel_l2(np.asarray(d.E), np.stack(od.E)) <= TOL[precision]


@pytest.mark.parametrize("precision", ["float64", "float32"])
def test_uniform_materials(fd, precision):
    kw = dict(levels=False, objects=False)
    g, eng = _run(fd, precision, dict(tile_rows=8), materials=0, **kw)
    assert eng.compact_materials() == [("uniform", 1), ("uniform", 1)]
    f, _ = _run(fd, precision, dict(tile_rows=8), materials=1, **kw)
    for a, b in zip(_records(g), _records(f)):
        assert torch.equal(_bits(a), _bits(b))


def test_random_medium_falls_back_to_full_arrays(fd):
    fd.set_backend("gb300.float32")
    g = fd.Grid((16, 16, 32), grid_spacing=100e-9,
                permittivity=np.random.default_rng(1).uniform(1.0, 3.0, size=(16, 16, 32)))
    g[8, 8, 16] = fd.PointSource(period=12)
    eng = g._ensure_engine()
    eng.set_tuning(variant=2)
    assert eng.compact_materials()[0] is None and eng.compact_materials()[1] == ("uniform", 1)
    g.run(5, progress_bar=False)
    eng.check_status()


def test_index_needs_nz_multiple_of_16(fd):
    fd.set_backend("gb300.float32")
    g = scene(fd, nz=24)
    eng = g._ensure_engine()
    eng.set_tuning(variant=2, tile_rows=8)
    assert eng.compact_materials() == [None, ("uniform", 1)]


@pytest.mark.parametrize("precision", ["float64", "float32"])
def test_in_place_material_changes_are_followed(fd, precision):
    fd.set_backend("gb300." + precision)
    g = scene(fd)
    o = scene(fo)
    eng = g._ensure_engine()
    eng.set_tuning(variant=2, tile_rows=8, pml_mode=2)
    g.run(8, progress_bar=False)
    o.run(8)
    n0 = eng.compact_materials()[0][1]
    # an existing value triple: same table size, updated in place
    g.inverse_permittivity[14:18, 2:6, 2:30] = 1.0 / 1.5
    o.inverse_permittivity[14:18, 2:6, 2:30] = 1.0 / 1.5
    g.run(8, progress_bar=False)
    o.run(8)
    assert eng.compact_materials()[0][1] == n0
    # a new value: larger table, plan rebuilt
    g.inverse_permittivity[2:5, 3:7, 1:5] = 0.3
    o.inverse_permittivity[2:5, 3:7, 1:5] = 0.3
    g.run(8, progress_bar=False)
    o.run(8)
    assert eng.compact_materials()[0][1] > n0
    # a uniform permeability that stops being uniform
    g.inverse_permeability[6:8, 6:8, 6:8] = 0.5
    o.inverse_permeability[6:8, 6:8, 6:8] = 0.5
    g.run(8, progress_bar=False)
    o.run(8)
    assert eng.compact_materials()[1][0] == "index"
    eng.check_status()
    assert rel_l2(g.E, o.E) <= TOL[precision] and rel_l2(g.H, o.H) <= TOL[precision]
    for d, od in zip(g.detectors, o.detectors):
        assert rel_l2(np.asarray(d.E), np.stack(od.E)) <= TOL[precision]


def _raw_run(lib, fields, ie, imu, steps, eps_compact=None, mu_compact=None):
    """Plan through the C ABI with the given material arrays (and compact
    copies), `steps` steps from the given fields; returns (E, H)."""
    from fdtd_gb300 import _native

    E, H = (f.clone() for f in fields)
    d = _native.GridDesc()
    d.abi_version = _native.ABI_VERSION
    d.precision = _native.FLOAT32
    d.nx, d.ny, d.nz = E.shape[:3]
    d.courant = 0.99 / 3 ** 0.5
    d.E, d.H, d.inv_eps, d.inv_mu = E.data_ptr(), H.data_ptr(), ie.data_ptr(), imu.data_ptr()
    d.variant = 2
    for enc, tab, n, idx in ((eps_compact, "eps_table", "n_eps_table", "eps_index"),
                             (mu_compact, "mu_table", "n_mu_table", "mu_index")):
        if enc is not None:
            setattr(d, tab, enc[0].data_ptr())
            setattr(d, n, enc[0].shape[0])
            setattr(d, idx, enc[1].data_ptr() if enc[1] is not None else None)
    plan = ctypes.c_void_p()
    assert lib.fdtd_plan_create(ctypes.byref(d), ctypes.byref(plan)) == 0
    try:
        a = _native.RunArgs()
        a.n_steps = steps
        stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        assert lib.fdtd_run(plan, ctypes.byref(a), stream) == 0
        st = ctypes.c_int32(-1)
        assert lib.fdtd_plan_status(plan, ctypes.byref(st), 0, stream) == 0 and st.value == 0
        torch.cuda.synchronize()
    finally:
        lib.fdtd_plan_destroy(plan)
    return E, H


def test_c_abi_compact_fields(fd):
    """A caller of the C ABI passing its own table and index gets the bits of
    the full-array plan; index bytes past the table read zeros."""
    from fdtd_gb300 import _native
    from fdtd_gb300.engine import compact_material

    lib = _native.load()
    gen = torch.Generator(device="cuda").manual_seed(11)
    shape = (24, 20, 32)
    E = torch.randn(shape + (3,), device="cuda", generator=gen)
    H = torch.randn(shape + (3,), device="cuda", generator=gen)
    levels = torch.tensor([1.0, 0.5, 1 / 3.0, 0.25], device="cuda")
    ie = levels[torch.randint(0, 4, shape, device="cuda", generator=gen)][..., None].expand(shape + (3,)).contiguous()
    imu = torch.ones(shape + (3,), device="cuda")
    full = _raw_run(lib, (E, H), ie, imu, 12)
    enc = compact_material(ie)
    assert enc is not None and enc[1] is not None
    mu_enc = compact_material(imu)
    comp = _raw_run(lib, (E, H), ie, imu, 12, enc, mu_enc)
    for a, b in zip(full, comp):
        assert torch.equal(a.view(torch.int32), b.view(torch.int32))
    # index bytes past the table: zeros, like a full array holding zeros there
    idx = enc[1].clone()
    idx[3:6, 4:9, 8:20] = 200
    ie0 = ie.clone()
    ie0[3:6, 4:9, 8:20] = 0.0
    want = _raw_run(lib, (E, H), ie0, imu, 12)
    got = _raw_run(lib, (E, H), ie, imu, 12, (enc[0], idx), mu_enc)
    for a, b in zip(want, got):
        assert torch.equal(a.view(torch.int32), b.view(torch.int32))


@pytest.mark.parametrize("precision", ["float32", "float64"])
def test_half_steps_with_writes_between(fd, precision):
    """Half-step API on a staged plan with compact materials and the y slabs
    kept in the fused pass: writes into E between the halves are seen by the
    H half (tests/test_detectors.py:62-70 of the reference does this)."""
    fd.set_backend("gb300." + precision)
    g, o = scene(fd), scene(fo)
    eng = g._ensure_engine()
    eng.set_tuning(variant=2, tile_rows=8, pml_mode=3)
    assert eng.compact_materials()[0][0] == "index"
    for q in range(6):
        for grid in (g, o):
            grid.update_E()
            grid.E[9, 8, 17, 2] = 0.25 * (q + 1)
            grid.update_H()
            grid.time_steps_passed += 1
    eng.check_status()
    assert rel_l2(g.E, o.E) <= TOL[precision] and rel_l2(g.H, o.H) <= TOL[precision]
