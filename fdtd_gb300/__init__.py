"""GB300-native time-step backend for the fdtd 3D FDTD simulator.

Drop-in for the time-stepping path of fdtd (fdtd/grid.py:250-325 and the
component hooks it calls): the same ``Grid``, boundaries, objects, sources and
detectors, with every E and H half step executed by one fused sm_103a CUDA
kernel pass through the C ABI in include/fdtd_gb300.h.

    import fdtd_gb300 as fdtd
    fdtd.set_backend("gb300.float32")      # or "gb300.float64", "gb300.float32c"
    grid = fdtd.Grid((64, 64, 64), grid_spacing=155e-9)
    grid[0:10, :, :] = fdtd.PML(name="pml_xlow")
    ...
    grid.run(500)

The reference package itself selects this backend once
``fdtd_gb300.install(fdtd)`` has wrapped its ``set_backend``:
``fdtd.set_backend("gb300.float32")`` then routes ``fdtd.Grid`` and the
component classes here (``fdtd_gb300.plugin``).

Gradients with respect to design objects' inverse permittivity come from a
reverse-time adjoint behind torch.autograd (``fdtd_gb300.adjoint.run``).
"""

__version__ = "0.1.0"

from .backend import backend, set_backend
from .boundaries import DomainBorderPML, PeriodicBoundary, PML
from .detectors import BlockDetector, CurrentDetector, DFTPlaneDetector, LineDetector, PlaneDetector
from .fourier import FrequencyRoutines
from .grid import Grid
from .objects import AbsorbingObject, AnisotropicObject, Object
from .sources import GaussianPlaneSource, LineSource, PlaneSource, PointSource, SoftArbitraryPointSource
from . import adjoint, constants, waveforms, conversions, visualization
from .plugin import install, uninstall
from .visualization import dB_map_2D, plot_detection

__all__ = [
    "Grid", "PML", "PeriodicBoundary", "DomainBorderPML", "Object", "AbsorbingObject",
    "AnisotropicObject", "PointSource", "LineSource", "PlaneSource", "GaussianPlaneSource",
    "SoftArbitraryPointSource", "LineDetector", "BlockDetector", "CurrentDetector", "PlaneDetector",
    "DFTPlaneDetector", "FrequencyRoutines", "backend", "set_backend", "adjoint", "constants", "waveforms",
    "conversions", "visualization", "dB_map_2D", "plot_detection", "install", "uninstall",
]
