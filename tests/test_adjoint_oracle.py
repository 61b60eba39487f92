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


@pytest.mark.parametrize("name", sorted(adjoint_scenes.SCENES))
def test_adjoint_oracle_matches_reference_autograd(name):
    ref = np.load(os.path.join(GOLDEN, f"ref_{name}.npz"))
    sc = adjoint_scenes.SCENES[name]
    loss, grad = oracle_loss_and_grad(sc, ref["design"])
    assert abs(loss - float(ref["loss"])) <= 1e-12 * abs(float(ref["loss"]))
    err = np.linalg.norm(grad - ref["grad"]) / np.linalg.norm(ref["grad"])
    assert err <= 1e-11, err
