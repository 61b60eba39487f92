"""The reference package selecting this backend: ``fdtd.set_backend("gb300.*")``.

The unmodified reference (installed into baseline/_ref by pip, with the
no-op matplotlib stand-in of tests/golden/mplstub because its plotting module
is imported at package import) gets its ``set_backend`` wrapped by
``fdtd_gb300.install``.  The CPU test checks the routing and its undoing; the
GPU test builds every golden scene through the reference module's own names
after ``fdtd.set_backend("gb300.<dtype>")`` and compares with the fixtures the
reference itself made (float64 <= 1e-12, float32 <= 1e-4 relative L2).
"""

import os
import sys

import numpy as np
import pytest

import golden_scenes
from helpers import rel_l2

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.path.join(ROOT, "baseline", "_ref")
GOLDEN = os.path.join(ROOT, "tests", "golden")


@pytest.fixture(scope="module")
def ref():
    if not os.path.isfile(os.path.join(REF, "fdtd", "__init__.py")):
        pytest.skip("the reference package is not installed in baseline/_ref")
    for p in (REF, os.path.join(GOLDEN, "mplstub")):
        if p not in sys.path:
            sys.path.insert(0, p)
    tqdm_stub = os.path.join(GOLDEN, "tqdmstub")  # used only where tqdm is not installed
    if tqdm_stub not in sys.path:
        sys.path.append(tqdm_stub)
    import fdtd
    import fdtd_gb300

    assert os.path.dirname(os.path.dirname(os.path.abspath(fdtd.__file__))) == REF
    fdtd_gb300.install(fdtd)
    yield fdtd
    fdtd_gb300.uninstall(fdtd)
    fdtd_gb300.set_backend("gb300.float64")


def test_install_routes_names_and_restores(ref):
    import fdtd_gb300

    own = {name: getattr(ref, name) for name in ("Grid", "PML", "PointSource", "LineDetector")}
    ref.set_backend("numpy")
    assert ref.Grid is own["Grid"]
    for name in ("gb300", "gb300.float32", "gb300.float32c", "gb300.float64", "gb300.cuda.float32"):
        ref.set_backend(name)
        assert ref.Grid is fdtd_gb300.Grid and ref.PML is fdtd_gb300.PML
        assert ref.backend is fdtd_gb300.backend
        assert ref.sources.SoftArbitraryPointSource is fdtd_gb300.SoftArbitraryPointSource
        assert ref.boundaries.DomainBorderPML is fdtd_gb300.DomainBorderPML
    assert fdtd_gb300.backend.precision == "float32"
    # a grid built through the reference's names is this package's grid
    g = ref.Grid((8, 8, 8), grid_spacing=155e-9)
    g[0:2, :, :] = ref.PML(name="pml")
    g[4, 4, 4] = ref.PointSource(period=10)
    assert isinstance(g, fdtd_gb300.Grid) and g.boundaries[0].__class__ is fdtd_gb300.PML
    # unknown gb300 names keep the reference's error type
    with pytest.raises(ValueError):
        ref.set_backend("gb300.float16")
    # the reference's own names and backends come back
    ref.set_backend("numpy.float32")
    for name, cls in own.items():
        assert getattr(ref, name) is cls
    assert not hasattr(ref, "PlaneDetector")
    assert type(ref.backend).__name__ == "NumpyBackend"
    with pytest.raises(ValueError):
        ref.set_backend("jax")
    ref.set_backend("numpy")


@pytest.mark.gpu
@pytest.mark.parametrize("prec,tol", [("float64", 1e-12), ("float32", 1e-4)])
@pytest.mark.parametrize("name", sorted(golden_scenes.SCENES))
def test_reference_set_backend_runs_golden_scenes(ref, name, prec, tol):
    ref.set_backend("gb300." + prec)
    try:
        grid, steps, drive = golden_scenes.SCENES[name](ref)
        assert type(grid).__module__ == "fdtd_gb300.grid"
        drive(grid, steps)
        snap = golden_scenes.snapshot(grid)
    finally:
        ref.set_backend("numpy")
    want = np.load(os.path.join(GOLDEN, f"ref_{name}.npz"))
    for key in want.files:
        if key in ("steps", "q"):
            continue
        assert snap[key].shape == want[key].shape, key
        err = rel_l2(snap[key], want[key])
        assert err <= tol, f"{name}/{prec}:{key} relative L2 {err:.3e} > {tol:.0e}"
