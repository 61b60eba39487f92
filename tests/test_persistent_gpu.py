"""The persistent time loop of small grids (fdtd_gb300/csrc/fdtd_persistent.cuh).

All full steps of a run() in one cooperative launch whose blocks meet at a
grid-wide barrier between half steps; detector gathers and DFT sums run
inside it.  Its per-cell arithmetic is the register-streaming passes', so E,
H, every detector record and every DFT accumulator must equal, bit for bit,
the plan that launches each half step on its own, after runs of any length
mixed with single steps and half steps, and in every precision.
"""

import numpy as np
import pytest

import golden_scenes
from fdtd_gb300 import scenes
from helpers import to_np

pytestmark = pytest.mark.gpu


def _dft_scene(fd):
    g = scenes.c4(fd, n=40, pml=6, d=12)
    g[:, :, 30] = fd.DFTPlaneDetector(frequencies=[2e14, 3e14], name="dft")
    g[:, 20, 20] = fd.LineDetector(name="line")
    return g


SCENES = {
    "c1_32": lambda fd: scenes.c1(fd, n=32, pml=6),
    "c4_40_dft": _dft_scene,
    "c2_24": lambda fd: scenes.c2(fd, n=24, pml=4),
    "mix": lambda fd: golden_scenes.g_mix(fd)[0],
    "c5_small": lambda fd: scenes.c5(fd, nx=40, ny=36, nz=24, pml=5),
}


def _outputs(g):
    out = {"E": to_np(g.E), "H": to_np(g.H)}
    for i, det in enumerate(g.detectors):
        if hasattr(det, "dft"):
            out[f"d{i}_dft"] = det.dft.detach().cpu().numpy()
        elif hasattr(det, "I"):
            out[f"d{i}_I"] = to_np(det.I.tensor())
        else:
            out[f"d{i}_E"] = to_np(det.E.tensor())
            out[f"d{i}_H"] = to_np(det.H.tensor())
    return out


def _drive(g):
    g.run(9, progress_bar=False)
    g.step()
    g.update_E()
    g.update_H()
    g.time_steps_passed += 1
    g.run(6, progress_bar=False)


@pytest.mark.parametrize("prec", ["float64", "float32", "float32c"])
@pytest.mark.parametrize("name", sorted(SCENES))
def test_persistent_loop_bitwise_equals_per_half_launches(fd, name, prec):
    fd.set_backend("gb300." + prec)
    ref = SCENES[name](fd)
    ref._ensure_engine().set_tuning(persistent=1)
    assert ref._engine.tiling()["persistent"] == 0
    _drive(ref)
    g = SCENES[name](fd)
    eng = g._ensure_engine()
    eng.set_tuning(persistent=2)
    info = eng.tiling()
    assert info["persistent"] == 1 and info["variant"] == 1, info
    _drive(g)
    eng.check_status()
    want, got = _outputs(ref), _outputs(g)
    assert set(want) == set(got)
    for key, val in want.items():
        assert np.array_equal(got[key], val), f"{name}/{prec} {key}: max |diff| {np.abs(got[key] - val).max()}"


def test_persistent_is_the_automatic_choice_on_small_grids(fd):
    fd.set_backend("gb300.float32")
    g = scenes.c1(fd, n=32, pml=6)
    assert g._ensure_engine().tiling()["persistent"] == 1
