"""The CPU oracle against golden vectors produced by the reference itself.

Fixtures: tests/golden/ref_*.npz, made by tests/golden/make_golden.py with the
reference's numpy float64 backend.  The oracle must reproduce them bit for bit.
"""

import os

import numpy as np
import pytest

import golden_scenes
from oracle import fdtd_oracle as fo

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_curl_known_answers():
    """Known-answer inputs of the reference's tests/test_grid.py:47-164."""
    d = np.load(os.path.join(GOLDEN, "ref_curls.npz"))
    assert np.array_equal(d["E"], np.random.RandomState(0).randn(3, 3, 3, 3))
    assert np.array_equal(d["H"], np.random.RandomState(1).randn(3, 3, 3, 3))
    assert np.array_equal(fo.curl_E(d["E"]), d["curl_E"])
    assert np.array_equal(fo.curl_H(d["H"]), d["curl_H"])
    # the edge semantics: curl_E drops the last planes, curl_H the first
    assert d["curl_E"][2, 2, 2, 0] == 0.0 and d["curl_H"][0, 0, 0, 0] == 0.0


@pytest.mark.parametrize("name", sorted(golden_scenes.SCENES))
def test_oracle_matches_reference(name):
    ref = np.load(os.path.join(GOLDEN, f"ref_{name}.npz"))
    grid, steps, drive = golden_scenes.SCENES[name](fo)
    assert steps == int(ref["steps"])
    drive(grid, steps)
    snap = golden_scenes.snapshot(grid)
    for key in ref.files:
        if key == "steps":
            continue
        assert key in snap, key
        assert snap[key].shape == ref[key].shape, key
        assert np.array_equal(snap[key], ref[key]), f"{name}:{key} differs from the reference"


def test_oracle_pml_profiles_match_reference_formula():
    """Low/high side sampling positions of the conductivity profile."""
    bE, cE, bH, cH = fo.pml_profiles(4, False, 1e-8, 0.5)
    assert cE[0] < cE[-1] < 0  # strongest at the outer edge (index 0) on the low side
    assert cH[-1] == 0.0
    bE2, cE2, bH2, cH2 = fo.pml_profiles(4, True, 1e-8, 0.5)
    assert np.array_equal(cE2, cE[::-1])
    assert cH2[-1] == 0.0 and np.array_equal(cH2[:-1], cH[:-1][::-1])


def test_oracle_dft_and_plane_detector_definitions():
    """The new detectors on a tiny grid: the DFT equals the explicit sum of
    the recorded planes times exp(-i w q dt)."""
    g = fo.Grid((8, 8, 8), grid_spacing=155e-9)
    g[4, 4, 2] = fo.PointSource(period=7)
    g[:, :, 5] = fo.PlaneDetector()
    g[:, :, 5] = fo.DFTPlaneDetector(frequencies=[1e14, 2e14])
    g.run(25)
    pd, dd = g.detectors
    rec = np.stack(pd.E)
    for f, fr in enumerate(dd.frequencies):
        w = np.array([complex(*fo.dft_factor(fr, q, g.time_step)) for q in range(25)])
        ref = np.tensordot(w, rec, axes=(0, 0))
        assert np.allclose(dd.dft[f], ref, rtol=1e-12, atol=1e-18)


def test_gaussian_plane_source_envelope():
    g = fo.Grid((6, 6, 12), grid_spacing=155e-9)
    src = fo.GaussianPlaneSource(period=1550e-9 / fo.C0, polarization="x")
    g[:, :, 3] = src
    vals = np.array([src.wave(q) for q in range(400)])
    peak = np.argmax(np.abs(vals))
    assert abs(peak * g.time_step - src.center_s) < 2 * src.period_s
    assert abs(vals[0]) < 1e-3


def _fuzz_fixture():
    return np.load(os.path.join(GOLDEN, "ref_fuzz.npz"))


@pytest.mark.parametrize("seed", list(range(12)))
def test_oracle_matches_reference_on_random_scenes(seed):
    """The random forward scenes of the GPU fuzz test (less their
    PlaneDetector), run by the reference itself (tests/golden/make_golden.py):
    the oracle the GPU fuzz compares against reproduces them bit for bit, or
    to 1e-14 where an anisotropic object's 3x3 product is summed in another
    order than numpy's einsum."""
    import test_fuzz_gpu

    ref = _fuzz_fixture()
    assert seed in ref["seeds"]
    grid = test_fuzz_gpu.random_scene(fo, seed, plane_detector=False)
    grid.run(int(ref["steps"]))
    aniso = any(isinstance(o, fo.AnisotropicObject) for o in grid.objects)
    got = {f"s{seed}_E": grid.E, f"s{seed}_H": grid.H}
    for i, d in enumerate(grid.detectors):
        got[f"s{seed}_d{i}_E"] = np.array(d.E)
        got[f"s{seed}_d{i}_H"] = np.array(d.H)
    keys = [k for k in ref.files if k.startswith(f"s{seed}_")]
    assert sorted(keys) == sorted(got)
    for k in keys:
        a, b = np.asarray(got[k], dtype=np.float64), ref[k]
        assert a.shape == b.shape, k
        if aniso:
            scale = max(np.linalg.norm(b), 1e-300)
            assert np.linalg.norm(a - b) <= 1e-14 * scale, k
        else:
            assert np.array_equal(a, b), k


def test_oracle_config1_full_size_bit_identical():
    """Config 1 at its full size and step count (64^3, 500 steps) against the
    reference's own run: identical traces and planes, and identical SHA-256
    digests of the whole final E and H (ref_c1_full.npz).  The digests pin
    every bit on an x86 host like the one that made the fixture; a host whose
    numpy exp rounds a PML coefficient differently still matches the planes
    and traces to 1e-12."""
    import hashlib
    import platform

    from fdtd_gb300 import scenes

    fix = np.load(os.path.join(GOLDEN, "ref_c1_full.npz"))
    g = scenes.c1(fo)
    g.run(int(fix["steps"]))
    E, H = np.ascontiguousarray(g.E, np.float64), np.ascontiguousarray(g.H, np.float64)
    planes = list(fix["planes"])
    d = g.detectors[0]
    got = {"trace_E": np.stack(d.E), "trace_H": np.stack(d.H), "E_planes": E[planes], "H_planes": H[planes]}
    if platform.machine() in ("x86_64", "AMD64"):
        for key, val in got.items():
            assert np.array_equal(val, fix[key]), key
        assert hashlib.sha256(E.tobytes()).hexdigest() == str(fix["E_sha256"])
        assert hashlib.sha256(H.tobytes()).hexdigest() == str(fix["H_sha256"])
    else:
        for key, val in got.items():
            assert np.linalg.norm(val - fix[key]) <= 1e-12 * np.linalg.norm(fix[key]), key
