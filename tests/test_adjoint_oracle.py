"""The CPU adjoint oracle against gradients from autograd through the reference.

Fixtures: tests/golden/ref_adj_*.npz, made by tests/golden/make_golden_adjoint.py
(the reference's torch.float64 backend with autograd).  The oracle's explicit
transposes must give the same loss and gradient to round-off.
"""

import os

import numpy as np
import pytest
import torch

import adjoint_scenes
from oracle import fdtd_adjoint_oracle as fa
from oracle import fdtd_oracle as fo

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def oracle_loss_and_grad(sc, design_values):
    """Loss and d loss / d design of a scene on the CPU oracle."""
    grid, obj = sc.build(fo)
    sc.detectors(fo, grid)
    p = np.asarray(design_values, dtype=np.float64)
    obj.inverse_permittivity = p.copy() if p.ndim == 5 else np.repeat(p[..., None], 3, axis=-1)
    recs, curls = fa.forward_records(grid, sc.steps, obj)
    outs = {name: {k: torch.tensor(v, requires_grad=True) for k, v in r.items()} for name, r in recs.items()}
    loss = sc.gb_loss(outs, torch)
    loss.backward()
    seeds = {name: {k: (None if t.grad is None else t.grad.numpy()) for k, t in r.items()}
             for name, r in outs.items()}
    grad = fa.adjoint_gradient(grid, sc.steps, obj, 0, seeds, curls)
    if p.ndim == 3:
        grad = grad.sum(axis=-1)
    return float(loss.detach()), grad


@pytest.mark.parametrize("name", sorted(adjoint_scenes.SCENES) + sorted(adjoint_scenes.RANDOM_SCENES))
def test_adjoint_oracle_matches_reference_autograd(name):
    ref = np.load(os.path.join(GOLDEN, f"ref_{name}.npz"))
    sc = adjoint_scenes.SCENES.get(name) or adjoint_scenes.RANDOM_SCENES[name]
    loss, grad = oracle_loss_and_grad(sc, ref["design"])
    assert abs(loss - float(ref["loss"])) <= 1e-12 * abs(float(ref["loss"]))
    err = np.linalg.norm(grad - ref["grad"]) / np.linalg.norm(ref["grad"])
    assert err <= 1e-11, err


def _plane_periodic_scene(design):
    grid = fo.Grid((12, 10, 1), grid_spacing=100e-9)
    grid[:, 0, :] = fo.PeriodicBoundary()
    grid[:, :, 0] = fo.PeriodicBoundary()  # one plane: the copy is the identity
    grid[0:3, :, :] = fo.PML()
    obj = fo.Object(permittivity=2.0)
    grid[5:8, 3:7, 0:1] = obj
    obj.inverse_permittivity = np.repeat(design[..., None], 3, axis=-1)
    grid[9, 5, 0] = fo.PointSource(period=8)
    grid[:, 5, 0] = fo.LineDetector()
    return grid, obj


def test_periodic_one_plane_axis_transposes_to_identity():
    """A periodic boundary on an axis of one plane copies each value onto
    itself; its transpose must leave the adjoint alone (not move and zero it).
    Checked against central differences of the forward."""
    steps = 14
    rng = np.random.default_rng(3)
    design = rng.uniform(0.4, 0.9, size=(3, 4, 1))

    def loss_of(d):
        grid, obj = _plane_periodic_scene(d)
        recs, curls = fa.forward_records(grid, steps, obj)
        name = next(iter(recs))
        e = torch.tensor(recs[name]["E"], requires_grad=True)
        loss = (e ** 2).sum()
        return loss, e, grid, obj, curls, name

    loss, e, grid, obj, curls, name = loss_of(design)
    loss.backward()
    seeds = {name: {"E": e.grad.numpy(), "H": None}}
    grad = fa.adjoint_gradient(grid, steps, obj, 0, seeds, curls).sum(axis=-1)
    h = 1e-6
    for idx in [(0, 0, 0), (1, 2, 0), (2, 3, 0)]:
        dp, dm = design.copy(), design.copy()
        dp[idx] += h
        dm[idx] -= h
        fd = (float(loss_of(dp)[0].detach()) - float(loss_of(dm)[0].detach())) / (2 * h)
        assert abs(fd - grad[idx]) <= 1e-6 * max(1.0, abs(fd)), (idx, fd, grad[idx])


@pytest.mark.parametrize("seed", [0, 3, 10, 13, 35, 114])
def test_adjoint_oracle_matches_central_differences_on_random_scenes(seed):
    """The adjoint oracle on the random scenes of the GPU adjoint fuzz test
    (random boundaries, objects, sources, detectors, design kind) against
    central differences of the oracle's own forward loss at three design
    entries."""
    import test_adjoint_fuzz_gpu as fz

    steps = fz.STEPS

    def run(value):
        grid, design, _, weights, _, _ = fz.adjoint_scene(fo, seed)
        design.inverse_permittivity = value if value.ndim == 5 else np.repeat(value[..., None], 3, axis=-1)
        recs, curls = fa.forward_records(grid, steps, design)
        outs = {name: {f: torch.tensor(v, requires_grad=True) for f, v in r.items()} for name, r in recs.items()}
        return fz.loss_of(outs, weights), outs, grid, design, curls

    _, _, value, _, _, _ = fz.adjoint_scene(fo, seed)
    loss, outs, grid, design, curls = run(value)
    loss.backward()
    seeds = {name: {f: (None if t.grad is None else t.grad.numpy()) for f, t in r.items()}
             for name, r in outs.items()}
    grad = fa.adjoint_gradient(grid, steps, design, 0, seeds, curls)
    if value.ndim == 3:
        grad = grad.sum(axis=-1)
    rng = np.random.default_rng(seed + 77)
    h = 1e-6
    for _ in range(3):
        idx = tuple(int(rng.integers(0, m)) for m in value.shape)
        vp, vm = value.copy(), value.copy()
        vp[idx] += h
        vm[idx] -= h
        fd = (float(run(vp)[0].detach()) - float(run(vm)[0].detach())) / (2 * h)
        # central differences: truncation ~h^2, rounding ~eps*|loss|/h
        noise = 1e-9 * max(1.0, abs(float(loss.detach())))
        assert abs(fd - grad[idx]) <= 1e-5 * abs(fd) + noise, (seed, idx, fd, grad[idx])
