"""Seeded random scenes for the adjoint: fdtd_gb300.adjoint.run against the
CPU adjoint oracle (which is pinned to autograd through the reference).

Each scene is a random forward scene (tests/test_fuzz_gpu.py) plus a design
Object or AnisotropicObject and a DFT plane detector; the loss is a random
quadratic form of every detector output; the checkpoint interval and the PML
mode (slabs inside the fused pass or in kernels of their own) are random.
float64 gradients must match to 1e-9 relative L2.
"""

import os

import numpy as np
import pytest
import torch

from helpers import rel_l2
from oracle import fdtd_adjoint_oracle as fa
from oracle import fdtd_oracle as fo
from test_fuzz_gpu import random_scene

pytestmark = pytest.mark.gpu

STEPS = 18


def adjoint_scene(mod, seed):
    grid = random_scene(mod, seed)
    rng = np.random.default_rng(seed + 5000)
    n = grid.shape
    lo = [int(rng.integers(0, max(1, m - 3))) if m > 1 else 0 for m in n]
    hi = [min(m, l + int(rng.integers(1, 4))) for l, m in zip(lo, n)]
    box = tuple(slice(l, h) for l, h in zip(lo, hi))
    shp = tuple(h - l for l, h in zip(lo, hi))
    aniso = bool(rng.random() < 0.4)
    design = mod.AnisotropicObject(permittivity=2.0) if aniso else mod.Object(permittivity=2.0)
    grid[box] = design
    if aniso:
        t = rng.standard_normal(shp + (3, 3)) * 0.05
        value = np.eye(3) * rng.uniform(0.3, 0.7, size=shp + (1, 1)) + (t + np.swapaxes(t, -1, -2))
    else:
        value = rng.uniform(0.3, 0.9, size=shp)
    period = int(rng.integers(8, 16))
    grid[:, :, int(rng.integers(0, n[2]))] = mod.DFTPlaneDetector(
        frequencies=[1.0 / (period * grid.time_step), 1.0 / (1.5 * period * grid.time_step)])
    for i, d in enumerate(grid.detectors):
        d.name = f"d{i}"
    weights = {}
    for d in grid.detectors:
        for field in (("dft",) if hasattr(d, "frequencies") else ("E", "H")):
            weights[(d.name, field)] = rng.uniform(0.0, 1.0, size=3)
    k = int(rng.choice([1, 4, 7, STEPS]))
    pml_mode = int(rng.choice([0, 1, 2]))
    return grid, design, value, weights, k, pml_mode


def loss_of(outs, weights):
    total = torch.zeros((), dtype=torch.float64)
    for (name, field), w in weights.items():
        x = outs[name][field]
        w = torch.as_tensor(w, device=x.device)
        if field == "dft":
            total = total + ((x.abs() ** 2) * w).sum().cpu()
        else:
            total = total + ((x.to(torch.float64) ** 2) * w).sum().cpu()
    return total


@pytest.mark.parametrize("seed", list(range(int(os.environ.get("FDTD_ADJOINT_FUZZ_SEEDS", "16")))))
def test_random_scene_gradient_matches_adjoint_oracle(fd, seed):
    fd.set_backend("gb300.float64")
    g, gd, value, weights, k, pml_mode = adjoint_scene(fd, seed)
    o, od, _, _, _, _ = adjoint_scene(fo, seed)
    # oracle: forward records, seeds from the loss, transposed stages
    od.inverse_permittivity = value if value.ndim == 5 else np.repeat(value[..., None], 3, axis=-1)
    recs, curls = fa.forward_records(o, STEPS, od)
    outs = {name: {f: torch.tensor(v, requires_grad=True) for f, v in r.items()} for name, r in recs.items()}
    loss = loss_of(outs, weights)
    loss.backward()
    seeds = {name: {f: (None if t.grad is None else t.grad.numpy()) for f, t in r.items()}
             for name, r in outs.items()}
    want = fa.adjoint_gradient(o, STEPS, od, 0, seeds, curls)
    if value.ndim == 3:
        want = want.sum(axis=-1)
    # GPU
    # half of the split-slab scenes run the TMA-staged passes (and so the
    # staged transposed passes) where nz allows it
    variant = 2 if pml_mode == 2 and g.Nz % 2 == 0 and seed % 2 == 0 else 0
    g._ensure_engine().set_tuning(pml_mode=pml_mode, variant=variant)
    p = torch.tensor(value, dtype=torch.float64, device="cuda", requires_grad=True)
    gouts = fd.adjoint.run(g, STEPS, design={gd: p}, checkpoint_every=k)
    gloss = loss_of(gouts, weights)
    gloss.backward()
    label = f"seed {seed} K={k} pml_mode={pml_mode} variant={variant} aniso={value.ndim == 5}"
    assert abs(float(gloss.detach()) - float(loss.detach())) <= 1e-10 * abs(float(loss.detach())), label
    assert rel_l2(p.grad.cpu().numpy(), want) <= 1e-9, label
