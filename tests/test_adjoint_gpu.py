"""Reverse-time adjoint on the GPU (fdtd_gb300.adjoint.run, fdtd_adjoint_run).

* against gradients from autograd through the reference (fixtures made by
  tests/golden/make_golden_adjoint.py): float64 relative L2 <= 1e-9, float32
  <= 1e-4;
* against the CPU adjoint oracle on a scene with every transposed stage
  (odd nz, periodic y, three PML axes, overlapping objects, hard and soft
  sources, block detector seeds on E and H);
* against central finite differences of the float64 forward on a
  config-4-shaped grid at reduced size (16 voxels, step 1e-3): relative
  <= 1e-3 for float32 and float64 adjoints;
* invariance under the checkpoint interval, and the forward side effects
  (final state, detector traces) equal to a plain grid.run.
"""

import os

import numpy as np
import pytest
import torch

import adjoint_scenes
from helpers import rel_l2
from oracle import fdtd_adjoint_oracle as fa
from oracle import fdtd_oracle as fo

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
TOL64 = 1e-9   # float64 adjoint gradient vs reference autograd, relative L2
TOL32 = 1e-4   # float32 adjoint gradient vs reference autograd, relative L2
TOL_FD = 1e-3  # adjoint vs central finite differences, relative L2 over the sampled voxels


@pytest.fixture(scope="module", autouse=True)
def native():
    from fdtd_gb300 import _native

    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    return _native.load()


def gb_loss_and_grad(fd, sc, design_values, precision, checkpoint_every, pml_mode=0, variant=0):
    fd.set_backend("gb300." + precision)
    grid, obj = sc.build(fd)
    sc.detectors(fd, grid)
    if pml_mode or variant:
        grid._ensure_engine().set_tuning(pml_mode=pml_mode, variant=variant)
    p = torch.tensor(np.asarray(design_values), dtype=torch.float64, device="cuda", requires_grad=True)
    outs = fd.adjoint.run(grid, sc.steps, design={obj: p}, checkpoint_every=checkpoint_every)
    loss = sc.gb_loss(outs, torch)
    loss.backward()
    return float(loss.detach()), p.grad.detach().cpu().numpy(), grid


@pytest.mark.parametrize("name", sorted(adjoint_scenes.SCENES))
@pytest.mark.parametrize("precision", ["float64", "float32"])
def test_adjoint_matches_reference_autograd(fd, name, precision):
    ref = np.load(os.path.join(GOLDEN, f"ref_{name}.npz"))
    sc = adjoint_scenes.SCENES[name]
    loss, grad, _ = gb_loss_and_grad(fd, sc, ref["design"], precision, checkpoint_every=7)
    tol = TOL64 if precision == "float64" else TOL32
    assert abs(loss - float(ref["loss"])) <= tol * abs(float(ref["loss"]))
    err = rel_l2(grad, ref["grad"])
    assert err <= tol, f"{name} {precision}: gradient relative L2 {err:.3e}"


@pytest.mark.parametrize("name", sorted(adjoint_scenes.SCENES))
def test_adjoint_with_pml_slab_kernels_matches_reference_autograd(fd, name):
    """Plans that run the PML slabs in kernels of their own (the choice on
    large grids) run the PML transposes in kernels of their own too."""
    ref = np.load(os.path.join(GOLDEN, f"ref_{name}.npz"))
    sc = adjoint_scenes.SCENES[name]
    loss, grad, grid = gb_loss_and_grad(fd, sc, ref["design"], "float64", checkpoint_every=9, pml_mode=2)
    assert grid._engine.tiling()["pml_split"] == 1
    assert abs(loss - float(ref["loss"])) <= TOL64 * abs(float(ref["loss"]))
    err = rel_l2(grad, ref["grad"])
    assert err <= TOL64, f"{name}: gradient relative L2 {err:.3e}"


class _TallPlaneScene(adjoint_scenes.PlaneScene):
    """The plane scene on 16x16x40: tall enough along z for an interior box
    (z 16..36) inside the 4-cell PML, with the design object crossing the
    interior's lower z face."""

    name = "adj_plane_tall"

    def build(self, fd):
        grid = fd.Grid((16, 16, 40), grid_spacing=155e-9)
        adjoint_scenes._pml_all(fd, grid, 4)
        obj = fd.Object(permittivity=2.0, name="design")
        grid[5:11, 5:11, 13:19] = obj
        grid[:, :, 3] = fd.PlaneSource(period=adjoint_scenes.PERIOD, polarization="x", name="src")
        return grid, obj

    def detectors(self, fd, grid):
        grid[:, :, 30] = fd.PlaneDetector(name="plane")


@pytest.mark.parametrize("variant", [1, 2])
@pytest.mark.parametrize("precision", ["float64", "float32"])
def test_adjoint_of_partition_plans_equals_fused_plans(fd, precision, variant):
    """Interior/shell partition plans (the choice on large grids with thick
    PML) run the forward bit for bit like the fused plans, and the transposed
    steps with the PML inside the register-streaming passes: the same loss
    and gradient bits as a fused plan."""
    sc = _TallPlaneScene()
    design = sc.design()
    loss_p, grad_p, grid_p = gb_loss_and_grad(fd, sc, design, precision, checkpoint_every=9, pml_mode=4,
                                              variant=variant)
    info = grid_p._engine.tiling()
    assert info["pml_split"] == 2 and info["variant"] == variant, info
    loss_f, grad_f, _ = gb_loss_and_grad(fd, sc, design, precision, checkpoint_every=9, pml_mode=1, variant=1)
    assert loss_p == loss_f
    assert np.array_equal(grad_p, grad_f)
    assert np.abs(grad_p).max() > 0


def test_checkpoint_interval_does_not_change_the_gradient(fd):
    sc = adjoint_scenes.SCENES["adj_periodic_first"]
    ref = np.load(os.path.join(GOLDEN, f"ref_{sc.name}.npz"))
    grads = [gb_loss_and_grad(fd, sc, ref["design"], "float64", k)[1] for k in (1, 6, sc.steps)]
    # segments are recomputed with the same kernels from bit-exact checkpoints
    assert np.array_equal(grads[0], grads[1]) and np.array_equal(grads[0], grads[2])


def test_forward_side_effects_match_plain_run(fd):
    sc = adjoint_scenes.SCENES["adj_plane"]
    design = np.load(os.path.join(GOLDEN, f"ref_{sc.name}.npz"))["design"]
    _, _, g1 = gb_loss_and_grad(fd, sc, design, "float64", checkpoint_every=9)
    grid, obj = sc.build(fd)
    sc.detectors(fd, grid)
    obj.inverse_permittivity = torch.tensor(design)[..., None].expand(*design.shape, 3)
    grid.run(sc.steps, progress_bar=False)
    assert g1.time_steps_passed == grid.time_steps_passed == sc.steps
    assert torch.equal(g1.E, grid.E) and torch.equal(g1.H, grid.H)
    assert torch.equal(g1.plane.E.tensor(), grid.plane.E.tensor())
    for a, b in zip((g1.pml_zlow, g1.pml_xhigh), (grid.pml_zlow, grid.pml_xhigh)):
        assert torch.equal(a.psi_E, b.psi_E) and torch.equal(a.psi_H, b.psi_H)


class MixedScene:
    """Every transposed stage on one grid: nz odd (one cell per thread), a
    periodic y boundary between PML slabs of three axes (one with a different
    a), a design Object overlapping an absorbing object, a non-design
    anisotropic object, hard plane and soft point sources, and a loss on
    block-detector E and H samples."""

    name = "mixed"
    steps = 24
    design_shape = (5, 4, 5)

    def build(self, fd):
        rng = np.random.default_rng(21)
        eps = rng.uniform(1.0, 3.0, size=(13, 11, 13))
        grid = fd.Grid((13, 11, 13), grid_spacing=120e-9, permittivity=eps,
                       permeability=rng.uniform(1.0, 1.3, size=(13, 11, 13, 3)))
        grid[0:3, :, :] = fd.PML(name="pml_xlow")
        grid[:, 0, :] = fd.PeriodicBoundary(name="periodic")
        grid[:, :, 0:3] = fd.PML(name="pml_zlow")
        grid[-2:, :, :] = fd.PML(name="pml_xhigh")
        grid[:, :, -3:] = fd.PML(name="pml_zhigh", a=1e-6)
        grid[5:9, 2:7, 3:8] = fd.AbsorbingObject(permittivity=2.0, conductivity=3e4, name="absorber")
        obj = fd.Object(permittivity=2.5, name="design")
        grid[4:9, 5:9, 5:10] = obj
        an = fd.AnisotropicObject(permittivity=1.5, name="aniso")
        grid[8:11, 1:4, 6:9] = an
        grid[:, :, 2] = fd.PlaneSource(period=12, polarization="y", name="plane_src")
        grid[6, 8, 4] = fd.PointSource(period=9, amplitude=0.7, name="point")
        return grid, obj

    def design(self):
        return np.random.default_rng(22).uniform(0.2, 0.9, size=self.design_shape)

    def detectors(self, fd, grid):
        grid[3:6, 2:5, 9:11] = fd.BlockDetector(name="block")

    def gb_loss(self, outs, torch):
        e = outs["block"]["E"].to(torch.float64)
        h = outs["block"]["H"].to(torch.float64)
        return (e ** 2).sum() + 0.5 * (h[..., 1] * h[..., 2]).sum()


@pytest.mark.parametrize("precision", ["float64", "float32"])
@pytest.mark.parametrize("name", sorted(adjoint_scenes.SCENES))
def test_staged_adjoint_matches_reference_autograd(fd, name, precision):
    """TMA-staged forward passes with the PML slabs in kernels of their own
    (the plan of large grids) run TMA-staged transposed passes: against the
    reference's autograd, and bit for bit against the register-streaming
    transposed passes of the same split plan."""
    ref = np.load(os.path.join(GOLDEN, f"ref_{name}.npz"))
    sc = adjoint_scenes.SCENES[name]
    loss, grad, grid = gb_loss_and_grad(fd, sc, ref["design"], precision, checkpoint_every=9, pml_mode=2,
                                        variant=2)
    info = grid._engine.tiling()
    assert info["variant"] == 2 and info["pml_split"] == 1, info
    grid._engine.check_status()
    tol = TOL64 if precision == "float64" else TOL32
    assert abs(loss - float(ref["loss"])) <= tol * abs(float(ref["loss"]))
    err = rel_l2(grad, ref["grad"])
    assert err <= tol, f"{name} {precision}: gradient relative L2 {err:.3e}"
    loss_r, grad_r, grid_r = gb_loss_and_grad(fd, sc, ref["design"], precision, checkpoint_every=9, pml_mode=2,
                                              variant=1)
    assert grid_r._engine.tiling()["variant"] == 1
    assert loss_r == loss and np.array_equal(grad_r, grad), f"max |diff| {np.abs(grad_r - grad).max():.3e}"


@pytest.mark.parametrize("pml_mode", [0, 2])
def test_adjoint_matches_oracle_on_every_stage(fd, pml_mode):
    sc = MixedScene()
    design = sc.design()
    grid, obj = sc.build(fo)
    sc.detectors(fo, grid)
    obj.inverse_permittivity = np.repeat(design[..., None], 3, axis=-1)
    recs, curls = fa.forward_records(grid, sc.steps, obj)
    outs = {n: {k: torch.tensor(v, requires_grad=True) for k, v in r.items()} for n, r in recs.items()}
    loss = sc.gb_loss(outs, torch)
    loss.backward()
    seeds = {n: {k: (None if t.grad is None else t.grad.numpy()) for k, t in r.items()} for n, r in outs.items()}
    want = fa.adjoint_gradient(grid, sc.steps, obj, 0, seeds, curls).sum(axis=-1)
    got_loss, got, _ = gb_loss_and_grad(fd, sc, design, "float64", checkpoint_every=5, pml_mode=pml_mode)
    assert abs(got_loss - float(loss.detach())) <= 1e-10 * abs(float(loss.detach()))
    err = rel_l2(got, want)
    assert err <= TOL64, err


def _c4_small(fd, design_values):
    """Config-4 shape at reduced size: 40^3 grid, 6-cell PML, 12^3 design
    Object at the centre, plane source at z=6, plane detector at z=33."""
    grid = fd.Grid((40, 40, 40), grid_spacing=155e-9)
    for sl in ((slice(0, 6), slice(None), slice(None)), (slice(-6, None), slice(None), slice(None)),
               (slice(None), slice(0, 6), slice(None)), (slice(None), slice(-6, None), slice(None)),
               (slice(None), slice(None), slice(0, 6)), (slice(None), slice(None), slice(-6, None))):
        grid[sl] = fd.PML()
    obj = fd.Object(permittivity=2.0, name="design")
    grid[14:26, 14:26, 14:26] = obj
    grid[:, :, 6] = fd.PlaneSource(period=adjoint_scenes.PERIOD, polarization="x", name="src")
    grid[:, :, 33] = fd.PlaneDetector(name="plane")
    obj.inverse_permittivity = torch.as_tensor(design_values)[..., None].expand(12, 12, 12, 3)
    return grid, obj


C4S_STEPS, C4S_WINDOW = 200, 40


def _c4_loss(E):
    return float((E[-C4S_WINDOW:, :, :, 0, 2].double() ** 2).sum())


@pytest.mark.parametrize("precision", ["float32", "float64"])
def test_adjoint_matches_finite_differences(fd, precision):
    rng = np.random.default_rng(4)
    design = rng.uniform(1.0 / 12.0, 1.0, size=(12, 12, 12))
    fd.set_backend("gb300." + precision)
    grid, obj = _c4_small(fd, design)
    p = torch.tensor(design, dtype=torch.float64, device="cuda", requires_grad=True)
    outs = fd.adjoint.run(grid, C4S_STEPS, design={obj: p}, checkpoint_every=50)
    loss = (outs["plane"]["E"][-C4S_WINDOW:, :, :, 0, 2].to(torch.float64) ** 2).sum()
    loss.backward()
    g = p.grad.cpu().numpy()
    # central differences of the float64 forward at 16 voxels
    fd.set_backend("gb300.float64")
    flat = rng.choice(design.size, size=16, replace=False)
    h = 1e-3
    fdg, adj = [], []
    for f in flat:
        idx = np.unravel_index(f, design.shape)
        vals = []
        for sgn in (1.0, -1.0):
            d = design.copy()
            d[idx] += sgn * h
            gr, _ = _c4_small(fd, d)
            gr.run(C4S_STEPS, progress_bar=False)
            vals.append(_c4_loss(gr.plane.E.tensor()))
        fdg.append((vals[0] - vals[1]) / (2 * h))
        adj.append(g[idx])
    err = rel_l2(np.array(adj), np.array(fdg))
    assert err <= TOL_FD, f"{precision}: adjoint vs finite differences relative L2 {err:.3e}"
