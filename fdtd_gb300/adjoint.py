"""Differentiable runs: gradients of detector outputs with respect to the
inverse permittivity of design objects, by a reverse-time adjoint.

The reference has no gradients of its own (it disables autograd at
fdtd/backend.py:57-60); the way to differentiate it is autograd through its
torch backend.  This module gives the same gradients without an autograd
graph of the time loop:

    outs = fdtd_gb300.adjoint.run(grid, 1000, design={grid.design: p}, checkpoint_every=50)
    loss = (outs["plane"]["E"][800:, ..., 2] ** 2).sum()
    loss.backward()                     # p.grad = dloss / d inverse_permittivity

``design`` maps registered ``Object``/``AnisotropicObject`` instances to
tensors of their inverse permittivity: ``(nx, ny, nz)`` (one value for the
three components), ``(nx, ny, nz, 3)``, or ``(nx, ny, nz, 3, 3)`` for an
anisotropic object.  The run starts from the grid's current state, which is
treated as a constant, and advances the grid by ``n_steps`` like
``grid.run``.  The outputs are, per detector name, ``{"E": ..., "H": ...}``
traces of this run (``(n_steps, *record_shape)``) for line, block and plane
detectors, and ``{"dft": ...}`` (the accumulator after the run, complex128)
for DFT plane detectors.

How: the forward pass runs in segments of ``checkpoint_every`` steps and keeps
a copy of the state (E, H, PML auxiliaries) at the start of every segment;
the curl of H on the design boxes is captured during the last segment.  The
backward pass walks the segments in reverse: it restores a segment's
checkpoint, recomputes the segment while capturing the design-box curls
(detectors off), then runs the transposed steps of that segment
(``fdtd_adjoint_run``), which add the detector gradients as sources and
accumulate the design gradient in float64.  At the end the grid gets back the
state it had after the forward pass.  Memory: one state copy per segment plus
``checkpoint_every`` design-box curls per design object.
"""

import ctypes

import torch

from . import _native
from .boundaries import PML
from .detectors import CurrentDetector, DFTPlaneDetector
from .objects import AnisotropicObject, Object, AbsorbingObject


def _det_name(det, i):
    return det.name if det.name is not None else f"detector{i}"


class _Runner:
    def __init__(self, grid, n_steps, objects, checkpoint_every):
        if grid.precision not in ("float32", "float64"):
            raise NotImplementedError("the adjoint supports the gb300.float32 and gb300.float64 backends")
        for o in objects:
            if o.grid is not grid:
                raise ValueError(f"{o!r} is not registered on this grid")
            if isinstance(o, AbsorbingObject) or not isinstance(o, Object):
                raise NotImplementedError("design objects must be Object or AnisotropicObject instances")
        for src in grid.sources:
            if hasattr(src, "current_detector"):
                raise NotImplementedError("the adjoint does not transpose the current feedback of a "
                                          "SoftArbitraryPointSource")
        self.grid = grid
        self.n = int(n_steps)
        if self.n < 1:
            raise ValueError("n_steps must be at least 1")
        self.K = int(checkpoint_every) if checkpoint_every else self.n
        self.K = max(1, min(self.K, self.n))
        self.objects = list(objects)

    # --- state checkpoints ------------------------------------------------------
    def _state_tensors(self):
        g = self.grid
        ts = [g._E, g._H]
        for b in g.boundaries:
            if isinstance(b, PML):
                ts += [b._psi_E, b._psi_H]
        return ts

    def _snapshot(self):
        return [t.clone() for t in self._state_tensors()]

    def _restore(self, snap):
        for t, s in zip(self._state_tensors(), snap):
            t.copy_(s)

    def _curl_buffers(self, rows):
        g = self.grid
        out = []
        for o in g.objects:
            if o in self.objects:
                cells = o.Nx * o.Ny * o.Nz
                out.append(torch.empty((rows, cells, 3), dtype=g._dtype, device=g._device))
            else:
                out.append(None)
        return out

    # --- forward ----------------------------------------------------------------
    def forward(self, params):
        g = self.grid
        with torch.no_grad():
            for o, p in zip(self.objects, params):
                o.inverse_permittivity = p.detach()
        eng = g._ensure_engine()
        self.engine = eng
        self.plan_id = eng.plan.value
        self.q0 = g.time_steps_passed
        self.rec_E0, self.rec_H0 = eng.rec_E, eng.rec_H
        self.segments = [(t0, min(t0 + self.K, self.n)) for t0 in range(0, self.n, self.K)]
        self.checkpoints = []
        self.curls = self._curl_buffers(self.K)
        for t0, t1 in self.segments:
            if t1 < self.n:
                self.checkpoints.append(self._snapshot())
                eng.run(t1 - t0)
            else:
                self.checkpoints.append(None)
                eng.run_capture(t1 - t0, self.curls, detectors=True)
        eng.check_status()
        self.trace_dets, self.dft_dets, outs = [], [], []
        for i, det in enumerate(g.detectors):
            if isinstance(det, CurrentDetector):
                continue  # records only, not differentiable outputs
            if isinstance(det, DFTPlaneDetector):
                self.dft_dets.append(det)
                outs.append(det.dft.clone())
            else:
                self.trace_dets.append(det)
                for field, r0 in (("E", self.rec_E0), ("H", self.rec_H0)):
                    rec = eng.detector_records(det, field)
                    outs.append(rec[r0: r0 + self.n].clone())
        return outs

    def pack(self, flat):
        out, k = {}, 0
        for i, det in enumerate(self.grid.detectors):
            name = _det_name(det, i)
            if isinstance(det, CurrentDetector):
                continue
            if isinstance(det, DFTPlaneDetector):
                out[name] = {"dft": flat[k]}
                k += 1
            else:
                out[name] = {"E": flat[k], "H": flat[k + 1]}
                k += 2
        return out

    # --- backward ---------------------------------------------------------------
    def backward(self, grads):
        g = self.grid
        eng = self.engine
        if g._engine is not eng or eng.plan is None or eng.plan.value != self.plan_id or g._dirty:
            raise RuntimeError("the grid changed between the forward and the backward pass of the adjoint run")
        lib = _native.load()
        dev, dt = g._device, g._dtype
        stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)

        # detector seeds in the probe layout of the plan: (n, n_probe, 3)
        seed = {"E": None, "H": None}
        k = 0
        gdft = []
        for det in g.detectors:
            if isinstance(det, CurrentDetector):
                continue
            if isinstance(det, DFTPlaneDetector):
                gg = grads[k]
                k += 1
                gdft.append(None if gg is None else torch.view_as_real(gg.to(torch.complex128).contiguous())
                            .contiguous())
                continue
            p0, p1 = eng.det_ranges[det]
            for field in ("E", "H"):
                gg = grads[k]
                k += 1
                if gg is None:
                    continue
                if seed[field] is None:
                    seed[field] = torch.zeros((self.n, eng.n_probe, 3), dtype=dt, device=dev)
                seed[field][:, p0:p1, :] = gg.reshape(self.n, p1 - p0, 3).to(dt)

        lam_E = torch.zeros_like(g._E)
        lam_H = torch.zeros_like(g._H)
        args = _native.AdjointArgs()
        args.lam_E, args.lam_H = lam_E.data_ptr(), lam_H.data_ptr()
        keep = [lam_E, lam_H]
        for bi, b in enumerate(g.boundaries):
            if isinstance(b, PML):
                for q in range(2):
                    aE, aH = torch.zeros_like(b._psi_E), torch.zeros_like(b._psi_H)
                    keep += [aE, aH]
                    args.aux_E[bi][q] = aE.data_ptr()
                    args.aux_H[bi][q] = aH.data_ptr()
        args.seed_E = _native.ptr(seed["E"])
        args.seed_H = _native.ptr(seed["H"])
        n_dft = len(eng.dfts)
        dft_arr = (ctypes.c_void_p * max(1, n_dft))(*[_native.ptr(t) for t in gdft])
        args.dft_grad = dft_arr
        gacc = []
        for o in g.objects:
            if o in self.objects:
                cells = o.Nx * o.Ny * o.Nz
                shape = (cells, 3, 3) if isinstance(o, AnisotropicObject) else (cells, 3)
                gacc.append(torch.zeros(shape, dtype=torch.float64, device=dev))
            else:
                gacc.append(None)
        grad_arr = (ctypes.c_void_p * max(1, len(gacc)))(*[_native.ptr(t) for t in gacc])
        curl_arr = (ctypes.c_void_p * max(1, len(self.curls)))(*[_native.ptr(t) for t in self.curls])
        args.grad = grad_arr
        args.curl = curl_arr
        args.n_objects = len(g.objects)

        final = self._snapshot()
        parity = 0
        any_dft = any(t is not None for t in gdft)
        for (t0, t1), ck in zip(reversed(self.segments), reversed(self.checkpoints)):
            m = t1 - t0
            if ck is not None:  # recompute the segment, capturing the design-box curls
                self._restore(ck)
                g.time_steps_passed = self.q0 + t0
                eng.run_capture(m, self.curls, detectors=False)
            phase = None
            if any_dft:
                phase = eng.upload_phase(eng.phase_table([self.q0 + t for t in range(t1 - 1, t0 - 1, -1)]))
            args.n_steps = m
            args.parity = parity
            args.seed_row = t1 - 1
            args.curl_row = m - 1
            args.phase = _native.ptr(phase)
            _native.check(lib.fdtd_adjoint_run(eng.plan, ctypes.byref(args), stream), "fdtd_adjoint_run")
            parity ^= m & 1
        self._restore(final)
        g.time_steps_passed = self.q0 + self.n
        eng.check_status()
        del keep

        out = []
        for o, p in zip(self.objects, self.params_shape):
            gi = gacc[g.objects.index(o)]
            out.append(gi.reshape(o._inverse_permittivity.shape).to(p[1]))
        return out


class _AdjointFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, runner, *params):
        ctx.set_materialize_grads(False)  # outputs the loss ignores seed nothing
        outs = runner.forward(params)
        ctx.runner = runner
        return tuple(outs)

    @staticmethod
    def backward(ctx, *grads):
        runner = ctx.runner
        ctx.runner = None
        return (None,) + tuple(runner.backward(grads))


def _full_param(obj, p):
    """The design tensor broadcast to the object's inverse permittivity shape."""
    target = tuple(obj._inverse_permittivity.shape)
    if not torch.is_tensor(p):
        p = torch.as_tensor(p, dtype=torch.float64)
    p = p.to(device=obj.grid._device)
    if isinstance(obj, AnisotropicObject):
        if tuple(p.shape) != target:
            raise ValueError(f"an anisotropic design tensor must have shape {target}")
        return p
    if tuple(p.shape) == target[:3]:
        p = p[..., None]
    return p.expand(target)


def run(grid, n_steps, design, checkpoint_every=50):
    """Differentiable ``grid.run(n_steps)``; see the module docstring."""
    objects = list(design.keys())
    runner = _Runner(grid, n_steps, objects, checkpoint_every)
    params = [_full_param(o, design[o]) for o in objects]
    runner.params_shape = [(tuple(p.shape), p.dtype) for p in params]
    flat = _AdjointFunction.apply(runner, *params)
    return runner.pack(flat)
