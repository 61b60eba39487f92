"""Parity at the benchmark configurations' own sizes.

* Config 1 exactly as specified (64^3, 10-cell PML on six faces, Object 2.25
  at 24:40, point source at the centre, x line detector, 500 steps), for the
  automatic plan and the other kernel plans: float64 bit for bit against the
  CPU oracle run on this host and within 1e-12 (relative L2) of the fixture
  the reference itself made at full size (detector traces, three planes of
  the final fields, the fields' sums of squares; tests/golden/ref_c1_full.npz);
  float32 and compensated float32 within 1e-4.
* Crops of configs 2, 3 and 5 at the sizes the oracle can run (128^3,
  192^3 and 192x192x96, the same generators with the PML scaled), started
  from seeded random E and H so that every cell, PML slabs included, carries
  signal from the first step, and run with the kernel plan the full-size
  grid gets (TMA-staged passes, PML slabs in kernels of their own, compact
  material copies, the full-size tile shape): float64 bit for bit against
  the oracle (within 1e-12 where an anisotropic object's 3x3 products are
  summed in another order), float32 / float32c within 1e-4, DFT
  accumulators included.
"""

import os

import numpy as np
import pytest
import torch

from fdtd_gb300 import scenes
from helpers import rel_l2, to_np
from oracle import fdtd_oracle as fo

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
TOL64 = 1e-12
TOL32 = 1e-4

# kernel plans of the config-1 runs: the automatic one (register streaming with
# the PML inside the fused pass at this size) and the ones larger grids use
C1_PLANS = {
    "automatic": {},
    "staged_split_compact": dict(variant=2, pml_mode=2),
    "staged_fused_compact": dict(variant=2, pml_mode=1),
    "register_split": dict(variant=1, pml_mode=2),
}


@pytest.fixture(scope="module")
def c1_oracle():
    o = scenes.c1(fo)
    o.run(500)
    d = o.detectors[0]
    return {"E": np.array(o.E), "H": np.array(o.H), "trace_E": np.stack(d.E), "trace_H": np.stack(d.H)}


@pytest.fixture(scope="module")
def c1_fixture():
    return np.load(os.path.join(GOLDEN, "ref_c1_full.npz"))


def _run_c1(fd, prec, plan):
    fd.set_backend("gb300." + prec)
    g = scenes.c1(fd)
    eng = g._ensure_engine()
    eng.set_tuning(**C1_PLANS[plan])
    if plan != "automatic":
        assert eng.tiling()["variant"] == C1_PLANS[plan]["variant"]
    g.run(500, progress_bar=False)
    eng.check_status()
    d = g.detectors[0]
    return {"E": to_np(g.E), "H": to_np(g.H), "trace_E": to_np(d.E.tensor()), "trace_H": to_np(d.H.tensor())}


def _against_fixture(got, fix, tol, label):
    planes = list(fix["planes"])
    for f in ("E", "H"):
        err = rel_l2(got[f"trace_{f}"], fix[f"trace_{f}"])
        assert err <= tol, f"{label} trace {f}: {err:.3e}"
        err = rel_l2(got[f][planes], fix[f"{f}_planes"])
        assert err <= tol, f"{label} {f} planes: {err:.3e}"
        s = float((got[f] ** 2).sum())
        assert abs(s - float(fix[f"{f}_sumsq"])) <= tol * float(fix[f"{f}_sumsq"]), f"{label} {f} sum of squares"


@pytest.mark.parametrize("plan", sorted(C1_PLANS))
def test_config1_full_size_float64(fd, c1_oracle, c1_fixture, plan):
    got = _run_c1(fd, "float64", plan)
    assert got["trace_E"].shape == (500, 64, 3)
    for key, want in c1_oracle.items():
        assert np.array_equal(got[key], want), f"{plan} {key}: max |diff| {np.abs(got[key] - want).max():.3e}"
    _against_fixture(got, c1_fixture, TOL64, plan)


@pytest.mark.parametrize("plan", ["automatic", "staged_split_compact"])
@pytest.mark.parametrize("prec", ["float32", "float32c"])
def test_config1_full_size_float32(fd, c1_oracle, c1_fixture, prec, plan):
    got = _run_c1(fd, prec, plan)
    for key, want in c1_oracle.items():
        err = rel_l2(got[key], want)
        assert err <= TOL32, f"{prec}/{plan} {key}: {err:.3e}"
    _against_fixture(got, c1_fixture, TOL32, f"{prec}/{plan}")


# crops: builder, steps, full-size plan per precision, anisotropic (no bit identity)
# the plans the full-size grids get: configs 2 and 5 the interior/shell
# partition (register-streaming interior, or the staged one for float32 with
# compact materials), config 3 its slabs in kernels of their own (float64:
# the partition)
CROPS = {
    "c2_128": (lambda m: scenes.c2(m, n=128, pml=8), 8,
               {"float64": dict(variant=1, pml_mode=4), "float32": dict(variant=1, pml_mode=4),
                "float32c": dict(variant=1, pml_mode=4)}, False),
    "c3_192": (lambda m: scenes.c3(m, n=192, pml=5, detector=True), 8,
               {"float64": dict(variant=1, pml_mode=4),
                "float32": dict(variant=2, pml_mode=3, tile_rows=8),
                "float32c": dict(variant=2, pml_mode=2, tile_rows=8)}, False),
    "c5_192x192x96": (lambda m: scenes.c5(m, nx=192, ny=192, nz=96, pml=10), 8,
                      {"float64": dict(variant=1, pml_mode=4),
                       "float32": dict(variant=2, pml_mode=4, tile_rows=16),
                       "float32c": dict(variant=1, pml_mode=4)}, True),
}
SPLIT_OF_MODE = {2: 1, 3: 1, 4: 2}


def _random_start(shape, seed):
    rng = np.random.default_rng(seed)
    return rng.standard_normal(shape + (3,)), rng.standard_normal(shape + (3,))


def _outputs(g):
    out = {"E": to_np(g.E), "H": to_np(g.H)}
    for i, det in enumerate(g.detectors):
        if hasattr(det, "dft"):
            out[f"d{i}_dft_re"], out[f"d{i}_dft_im"] = to_np(det.dft.real), to_np(det.dft.imag)
        else:
            for f in ("E", "H"):
                out[f"d{i}_{f}"] = np.stack([to_np(r) for r in getattr(det, f)])
    return out


@pytest.fixture(scope="module")
def crop_oracle():
    cache = {}

    def get(name):
        if name not in cache:
            build, steps, _, _ = CROPS[name]
            o = build(fo)
            E0, H0 = _random_start(tuple(o.E.shape[:3]), seed=len(name))
            o.E[...] = E0
            o.H[...] = H0
            o.run(steps)
            cache[name] = (_outputs(o), E0, H0)
        return cache[name]

    return get


@pytest.mark.parametrize("prec", ["float64", "float32", "float32c"])
@pytest.mark.parametrize("name", sorted(CROPS))
def test_config_crops_with_full_size_plans(fd, crop_oracle, name, prec):
    build, steps, plans, aniso = CROPS[name]
    want, E0, H0 = crop_oracle(name)
    fd.set_backend("gb300." + prec)
    g = build(fd)
    eng = g._ensure_engine()
    eng.set_tuning(**plans[prec])
    info = eng.tiling()
    assert info["variant"] == plans[prec]["variant"], info
    assert info["pml_split"] == SPLIT_OF_MODE[plans[prec]["pml_mode"]], info
    g.E.copy_(torch.as_tensor(E0, dtype=g.E.dtype))
    g.H.copy_(torch.as_tensor(H0, dtype=g.H.dtype))
    g.run(steps, progress_bar=False)
    eng.check_status()
    got = _outputs(g)
    assert set(got) == set(want)
    for key, ref in want.items():
        if prec == "float64" and not aniso:
            assert np.array_equal(got[key], ref), f"{name} {key}: max |diff| {np.abs(got[key] - ref).max():.3e}"
        else:
            err = rel_l2(got[key], ref)
            assert err <= (TOL64 if prec == "float64" else TOL32), f"{name}/{prec} {key}: {err:.3e}"
