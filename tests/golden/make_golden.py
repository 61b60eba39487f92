"""Generate the golden fixtures by running the reference fdtd package (numpy backend).

Usage (needs a checkout of the reference; nothing else in the repository reads it):

    python tests/golden/make_golden.py <path to the reference checkout> [scene ...]

The reference imports matplotlib for plotting only; a no-op stand-in from
``tests/golden/mplstub`` is put on ``sys.path`` first.  Outputs:

* ``ref_curls.npz`` -- curl_E / curl_H of the reference applied to the inputs of
  its own known-answer tests (tests/test_grid.py:47-164 use
  ``RandomState(0).randn(3,3,3,3)`` and ``RandomState(1).randn(3,3,3,3)``).
* ``ref_<scene>.npz`` -- final E, H and every detector trace for each scene of
  ``golden_scenes.SCENES`` after its stated number of steps.
* ``ref_fuzz.npz`` -- the same for the first random forward scenes of
  ``tests/test_fuzz_gpu.py`` (scene argument ``fuzz``).
* ``ref_c1_full.npz`` -- config 1 at its full size and step count (scene
  argument ``c1_full``, only when named): traces, three planes of the final
  fields and digests of the whole final fields.
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))


def load_reference(path):
    sys.path.insert(0, os.path.join(HERE, "mplstub"))
    sys.path.insert(0, path)
    import fdtd  # noqa: E402  (the reference package)
    import fdtd.boundaries

    fdtd.set_backend("numpy")
    fdtd.DomainBorderPML = fdtd.boundaries.DomainBorderPML
    fdtd.SoftArbitraryPointSource = fdtd.sources.SoftArbitraryPointSource
    return fdtd


def fourier_fixture(fdtd, grid):
    """FrequencyRoutines (fdtd/fourier.py) outputs on the 'saps' scene."""
    from fdtd.fourier import FrequencyRoutines

    src = next(s for s in grid.sources if isinstance(s, fdtd.SoftArbitraryPointSource))
    f_z, z = FrequencyRoutines(grid, src).impedance()
    f_i, s_i = FrequencyRoutines(grid, grid.current).FFT()
    arr = np.sin(np.arange(37) * 0.3)
    f_a, s_a = FrequencyRoutines(grid, arr).FFT()
    return dict(imp_freqs=np.asarray(f_z), imp=np.asarray(z), cur_freqs=np.asarray(f_i), cur_fft=np.asarray(s_i),
                arr=arr, arr_freqs=np.asarray(f_a), arr_fft=np.asarray(s_a))


FUZZ_SEEDS = list(range(12))
FUZZ_STEPS = 15


def fuzz_fixture(fdtd):
    """Final E, H and every detector trace of the random forward scenes of
    tests/test_fuzz_gpu.py (without their PlaneDetector) after FUZZ_STEPS."""
    sys.path.insert(0, os.path.join(REPO, "tests"))
    from test_fuzz_gpu import random_scene

    out = {"seeds": np.array(FUZZ_SEEDS), "steps": np.array(FUZZ_STEPS)}
    for seed in FUZZ_SEEDS:
        grid = random_scene(fdtd, seed, plane_detector=False)
        grid.run(FUZZ_STEPS, progress_bar=False)
        out[f"s{seed}_E"] = np.asarray(grid.E)
        out[f"s{seed}_H"] = np.asarray(grid.H)
        for i, d in enumerate(grid.detectors):
            out[f"s{seed}_d{i}_E"] = np.array(d.E)
            out[f"s{seed}_d{i}_H"] = np.array(d.H)
    return out


FULL_C1_PLANES = (5, 32, 58)  # x planes kept of the full fields: low PML, centre, high PML


def full_c1_fixture(fdtd):
    """Config 1 at its full size (64^3, 10-cell PML on six faces, Object
    2.25 at 24:40, point source, x line detector, 500 steps): the detector
    traces, three x planes of the final E and H, and SHA-256 digests and sums
    of squares of the whole final fields (full fields would be 12 MB)."""
    import hashlib

    from fdtd_gb300 import scenes

    grid = scenes.c1(fdtd)
    grid.run(500, progress_bar=False)
    E, H = np.ascontiguousarray(grid.E, np.float64), np.ascontiguousarray(grid.H, np.float64)
    det = grid.detectors[0]
    return dict(steps=np.array(500), trace_E=np.array(det.E), trace_H=np.array(det.H),
                planes=np.array(FULL_C1_PLANES), E_planes=E[list(FULL_C1_PLANES)],
                H_planes=H[list(FULL_C1_PLANES)], E_sha256=np.array(hashlib.sha256(E.tobytes()).hexdigest()),
                H_sha256=np.array(hashlib.sha256(H.tobytes()).hexdigest()),
                E_sumsq=np.array(float((E * E).sum())), H_sumsq=np.array(float((H * H).sum())))


def main(ref_path, only=None):
    fdtd = load_reference(ref_path)
    sys.path.insert(0, REPO)
    sys.path.insert(0, HERE)
    import golden_scenes
    from fdtd.grid import curl_E, curl_H

    E0 = np.random.RandomState(0).randn(3, 3, 3, 3)
    H1 = np.random.RandomState(1).randn(3, 3, 3, 3)
    np.savez(os.path.join(HERE, "ref_curls.npz"), E=E0, curl_E=curl_E(E0), H=H1, curl_H=curl_H(H1),
             reference_version=fdtd.__version__)
    if only and "c1_full" in only:
        np.savez_compressed(os.path.join(HERE, "ref_c1_full.npz"), **full_c1_fixture(fdtd))
        print("c1_full")
    if not only or "fuzz" in only:
        np.savez_compressed(os.path.join(HERE, "ref_fuzz.npz"), **fuzz_fixture(fdtd))
        print("fuzz", len(FUZZ_SEEDS), "seeds")
    for name, build in golden_scenes.SCENES.items():
        if only and name not in only:
            continue
        grid, steps, drive = build(fdtd)
        drive(grid, steps)
        snap = golden_scenes.snapshot(grid)
        snap["steps"] = np.array(steps)
        np.savez_compressed(os.path.join(HERE, f"ref_{name}.npz"), **snap)
        print(name, {k: v.shape for k, v in snap.items()})
        if name == "saps":
            np.savez_compressed(os.path.join(HERE, "ref_saps_fourier.npz"), **fourier_fixture(fdtd, grid))


if __name__ == "__main__":
    # optional further arguments: only these scenes
    if len(sys.argv) < 2:
        sys.exit(__doc__)
    main(sys.argv[1], sys.argv[2:] or None)
