"""Select this backend from the reference package: ``fdtd.set_backend("gb300...")``.

The reference chooses its array backend with ``fdtd.set_backend(name)``
(fdtd/backend.py:367-439), which knows only ``numpy`` and ``torch`` names and
raises ``ValueError`` for anything else.  ``install(fdtd)`` wraps that
function in place so that the same call also accepts this package's names:

    import fdtd, fdtd_gb300
    fdtd_gb300.install(fdtd)              # once per process
    fdtd.set_backend("gb300.float32")     # or gb300, gb300.float64, gb300.float32c
    grid = fdtd.Grid((64, 64, 64), grid_spacing=155e-9)
    grid[0:10, :, :] = fdtd.PML(name="pml_xlow")
    ...
    grid.run(500)
    fdtd.set_backend("numpy")             # back to the reference's own classes

A ``gb300`` name points the reference module's public names (``Grid``, the
boundaries, objects, sources, detectors, ``FrequencyRoutines``, the plotting
helpers, and ``backend``) and the two component classes the reference keeps
only in submodules (``fdtd.sources.SoftArbitraryPointSource``,
``fdtd.boundaries.DomainBorderPML``) at this package's classes; the names this
package adds (``PlaneDetector``, ``DFTPlaneDetector``, ``GaussianPlaneSource``,
``adjoint``) become module attributes too.  Any other name restores every
original attribute and then calls the reference's own ``set_backend``, with
its own errors for unknown names.

Code that looks names up on the module at call time (``fdtd.Grid(...)``)
follows the switch; a name bound earlier (``from fdtd import Grid``) keeps
the class it was bound to.  Grids built under one backend keep running on it.
"""

import sys

# public names of the reference package routed to this package's classes
ROUTED = ("Grid", "PointSource", "LineSource", "PlaneSource", "LineDetector", "BlockDetector", "CurrentDetector",
          "Object", "AbsorbingObject", "AnisotropicObject", "PeriodicBoundary", "PML", "FrequencyRoutines",
          "dB_map_2D", "plot_detection", "SoftArbitraryPointSource", "DomainBorderPML", "PlaneDetector",
          "DFTPlaneDetector", "GaussianPlaneSource", "adjoint")
# classes the reference defines only in a submodule: (submodule, name)
SUBMODULE_ROUTED = (("sources", "SoftArbitraryPointSource"), ("boundaries", "DomainBorderPML"))

_MISSING = object()


def _package():
    return sys.modules[__name__.rsplit(".", 1)[0]]


def install(fdtd=None):
    """Wrap ``fdtd.set_backend`` of the reference module ``fdtd`` (imported
    when not given) so that it accepts ``gb300`` names; returns the module.
    Installing twice is a no-op."""
    if fdtd is None:
        import fdtd  # the reference package
    if getattr(fdtd, "_gb300_original_set_backend", None) is not None:
        return fdtd
    pkg = _package()
    original_set_backend = fdtd.set_backend
    saved = {name: getattr(fdtd, name, _MISSING) for name in ROUTED}
    saved["backend"] = getattr(fdtd, "backend", _MISSING)
    saved_sub = {}
    for sub, name in SUBMODULE_ROUTED:
        mod = sys.modules.get(f"{fdtd.__name__}.{sub}")
        if mod is not None:
            saved_sub[(sub, name)] = (mod, getattr(mod, name, _MISSING))

    def _restore():
        for name, value in saved.items():
            if value is _MISSING:
                if hasattr(fdtd, name):
                    delattr(fdtd, name)
            else:
                setattr(fdtd, name, value)
        for (sub, name), (mod, value) in saved_sub.items():
            if value is _MISSING:
                if hasattr(mod, name):
                    delattr(mod, name)
            else:
                setattr(mod, name, value)

    def set_backend(name: str):
        """The reference's set_backend (fdtd/backend.py:367-439), plus the
        names of the GB300 backend: gb300, gb300.float32, gb300.float32c,
        gb300.float64 (and gb300.cuda[.dtype])."""
        if isinstance(name, str) and name.split(".")[0] == "gb300":
            selected = pkg.set_backend(name)  # validates the name first
            for attr in ROUTED:
                setattr(fdtd, attr, getattr(pkg, attr))
            fdtd.backend = selected
            for (sub, attr), (mod, _) in saved_sub.items():
                setattr(mod, attr, getattr(pkg, attr))
            fdtd._gb300_active = True
            return selected
        _restore()
        fdtd._gb300_active = False
        return original_set_backend(name)

    set_backend.__wrapped__ = original_set_backend
    fdtd.set_backend = set_backend
    fdtd._gb300_original_set_backend = original_set_backend
    fdtd._gb300_active = False
    return fdtd


def uninstall(fdtd):
    """Undo ``install``: the reference's own names and set_backend again."""
    original = getattr(fdtd, "_gb300_original_set_backend", None)
    if original is None:
        return fdtd
    if fdtd._gb300_active:
        fdtd.set_backend("numpy")  # restores every routed attribute
    fdtd.set_backend = original
    del fdtd._gb300_original_set_backend
    del fdtd._gb300_active
    return fdtd
