"""Backend selection for the GB300 time-step library.

Mirrors ``fdtd.set_backend`` / ``fdtd.backend`` (fdtd/backend.py:345-439):
``set_backend(name)`` mutates the module-level singleton ``backend``, whose
array namespace (``zeros``, ``ones``, ``array``, ``numpy``, ``bmm``, ...) keeps
the semantics of the reference's ``TorchCudaBackend`` (fdtd/backend.py:322-355)
so user code written against ``fdtd.backend`` keeps working.

Accepted names (``lib[.device][.dtype]`` like the reference):

    gb300                 float64 fields (the reference's default precision)
    gb300.float64         float64, same operation order as the reference
    gb300.float32         float32 fields and arithmetic
    gb300.float32c        float32 fields plus a float32 compensation term per
                          E/H value (two-float accumulation for long runs)
    gb300.cuda.<dtype>    the same with the device spelled out

There is no CPU path: ``numpy`` and ``torch`` names raise ``ValueError``
(use the reference package for those).  Without a CUDA device, grids can still
be built and inspected (arrays live in host memory), but every time step
raises ``RuntimeError``.
"""

import numpy

import torch

PRECISIONS = ("float32", "float32c", "float64")


class GB300Backend:
    """Array namespace plus the precision of the time-step kernels."""

    pi = numpy.pi
    int = torch.int64

    def __init__(self, precision="float64"):
        self._set(precision)

    def _set(self, precision):
        if precision not in PRECISIONS:
            raise ValueError(f"Unknown dtype '{precision}'. Available: {', '.join(PRECISIONS)}")
        self.precision = precision
        self.float = torch.float64 if precision == "float64" else torch.float32
        self.complex = torch.complex128 if precision == "float64" else torch.complex64
        self.compensated = precision == "float32c"

    @property
    def device(self):
        return torch.device("cuda") if torch.cuda.is_available() else torch.device("cpu")

    def __repr__(self):
        return f"GB300Backend(precision={self.precision!r}, device={self.device.type!r})"

    # --- array namespace (TorchCudaBackend semantics) -------------------------
    def zeros(self, shape, dtype=None, **kw):
        return torch.zeros(shape, dtype=dtype or self.float, device=self.device, **kw)

    def ones(self, shape, dtype=None, **kw):
        return torch.ones(shape, dtype=dtype or self.float, device=self.device, **kw)

    def array(self, arr, dtype=None, **kw):
        dtype = dtype or self.float
        if torch.is_tensor(arr):
            return arr.clone().to(device=self.device, dtype=dtype, **kw)
        return torch.tensor(numpy.asarray(arr), device=self.device, dtype=dtype, **kw)

    def asarray(self, arr, dtype=None):
        if torch.is_tensor(arr):
            return arr.to(device=self.device, dtype=dtype or arr.dtype)
        return torch.as_tensor(numpy.asarray(arr), device=self.device, dtype=dtype)

    def numpy(self, arr):
        if torch.is_tensor(arr):
            return arr.detach().cpu().numpy()
        return numpy.asarray(arr)

    @staticmethod
    def is_array(arr):
        return isinstance(arr, numpy.ndarray) or torch.is_tensor(arr)

    @staticmethod
    def is_complex(x):
        return isinstance(x, complex) or (torch.is_tensor(x) and torch.is_complex(x)) or (
            isinstance(x, numpy.ndarray) and numpy.iscomplexobj(x))

    def arange(self, *args, **kw):
        kw.setdefault("device", self.device)
        return torch.arange(*args, **kw)

    def linspace(self, start, stop, num=50, endpoint=True):
        vals = numpy.linspace(start, stop, num, endpoint=endpoint)
        return torch.tensor(vals, device=self.device, dtype=self.float)

    exp = staticmethod(torch.exp)
    sin = staticmethod(torch.sin)
    cos = staticmethod(torch.cos)
    sum = staticmethod(torch.sum)
    max = staticmethod(torch.max)
    stack = staticmethod(torch.stack)
    reshape = staticmethod(torch.reshape)
    squeeze = staticmethod(torch.squeeze)
    broadcast_to = staticmethod(torch.broadcast_to)
    broadcast_arrays = staticmethod(torch.broadcast_tensors)
    bmm = staticmethod(torch.bmm)
    divide = staticmethod(torch.div)

    @staticmethod
    def transpose(arr, axes=None):
        if axes is None:
            axes = tuple(range(arr.ndim - 1, -1, -1))
        return arr.permute(*axes)


backend = GB300Backend()


def set_backend(name: str):
    """Select the precision of the GB300 kernels (see module docstring)."""
    if not isinstance(name, str):
        raise ValueError(f"Unknown backend '{name}'")
    parts = name.split(".")
    lib = parts[0]
    if lib in ("numpy", "torch"):
        raise ValueError(
            f"Backend '{name}' is a CPU/generic backend of the reference package; fdtd_gb300 only "
            "provides 'gb300', 'gb300.float32', 'gb300.float32c' and 'gb300.float64'.")
    if lib != "gb300":
        raise ValueError(f"Unknown backend '{lib}'. Available backends: 'gb300'")
    if len(parts) == 1:
        dtype = "float64"
    elif len(parts) == 2:
        dtype = "float64" if parts[1] == "cuda" else parts[1]
    elif len(parts) == 3:
        if parts[1] != "cuda":
            raise ValueError(f"Unknown device '{parts[1]}'. Available devices: 'cuda'")
        dtype = parts[2]
    else:
        raise ValueError(f"Unknown backend '{name}'")
    backend._set(dtype)
    return backend
