"""Names of the reference's plotting helpers (fdtd/visualization.py).

The reference plots with matplotlib; this backend has no plotting, so these
raise NotImplementedError.  Copy fields or detector records to the host
(``grid.E.cpu().numpy()``, ``numpy.asarray(det.E)``) and plot them there.
"""


def visualize(*args, **kwargs):
    """fdtd/visualization.py:28-336."""
    raise NotImplementedError("visualize is not part of the gb300 backend (no plotting)")


def dB_map_2D(*args, **kwargs):
    """fdtd/visualization.py:339-394."""
    raise NotImplementedError("dB_map_2D is not part of the gb300 backend (no plotting)")


def plot_detection(*args, **kwargs):
    """fdtd/visualization.py:397-492."""
    raise NotImplementedError("plot_detection is not part of the gb300 backend (no plotting)")
