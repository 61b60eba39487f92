"""Plan compilation and time stepping through the C ABI.

``Engine`` turns a grid's registered components into an ``fdtd_grid_desc``
(include/fdtd_gb300.h), creates the native plan, and runs steps:

* waveform table -- for a call covering steps q0..q0+n-1 the host evaluates
  every source's waveform with the reference's Python expressions and copies
  the (n, n_sources) float64 table to the device through a pinned buffer;
* detector traces -- one device buffer (capacity, n_probe_cells, 3) in the
  grid precision, grown geometrically; detectors view their slice of it;
* DFT phases -- (n, n_freq_total, 2) float64 (cos, -sin) per step.

* compact material copies -- for the staged passes, a table of the distinct
  inverse-material value triples and a one-byte index per cell (or one triple
  for a uniform material), kept in step with in-place changes of the
  material arrays (``compact_material``).

The plan is rebuilt when components are registered, when an object's
coefficients change, when the compact copies change layout, or when the
tiling option changes; detector records taken before a rebuild are kept
(copied out of the old buffer).
"""

import ctypes
import math

import numpy as np
import torch

from . import _native
from .boundaries import PML, PeriodicBoundary
from .detectors import CurrentDetector, DFTPlaneDetector

_PRECISION = {"float32": _native.FLOAT32, "float32c": _native.FLOAT32C, "float64": _native.FLOAT64}


def _require_gpu(grid):
    if not torch.cuda.is_available():
        raise RuntimeError("the gb300 backend needs a CUDA device; this machine has none "
                           "(there is no CPU time step)")
    if grid._E.device.type != "cuda":
        raise RuntimeError("this grid was built without a CUDA device; rebuild it on a GPU machine")
    return _native.load()


_MAX_TABLE = 256  # distinct value triples a one-byte material index can address


def compact_material(x, chunk=1 << 25, index_ok=True):
    """Compact copy of a (nx, ny, nz, 3) inverse-material array for the staged
    passes: ``(table, index)`` with ``table`` an (n, 3) array of value triples
    and ``index`` the uint8 (nx, ny, nz) table row of every cell, or
    ``(table, None)`` when every cell holds the same triple; ``None`` when the
    cells hold more than 256 distinct triples, or more than one and
    ``index_ok`` is false.  Values are compared as bit patterns, so signed
    zeros and NaN payloads keep their own rows and ``table[index] == x`` holds
    bit for bit.

    One pass decides uniformity.  The distinct values of each component are
    taken from a strided sample and one more pass finds every cell's value by
    binary search, forming its key (the mixed-radix number of its three value
    positions); only if the sample missed a value are the components sorted
    in full.  When the product of the three value counts is at most 256 the
    key is the index (the table lists every combination); otherwise the keys
    present are ranked and a last pass maps every cell's key to its rank.
    Besides the index only per-chunk temporaries are allocated."""
    itype = torch.int32 if x.element_size() == 4 else torch.int64
    dev = x.device
    bits = x.contiguous().view(itype).reshape(-1, 3)
    ncell = bits.shape[0]
    if ncell == 0:
        return None
    starts = range(0, ncell, chunk)
    first = bits[:1]
    differs = torch.zeros((), dtype=torch.bool, device=dev)
    for a in starts:
        differs |= (bits[a:a + chunk] != first).any()
    if not bool(differs):
        return x.reshape(-1, 3)[:1].clone(), None
    if not index_ok:
        return None
    # quick rejection on a strided sample (random media, graded profiles)
    sample = bits[::max(1, ncell // 65536)]
    if torch.unique(sample, dim=0).shape[0] > _MAX_TABLE:
        return None
    comps = [torch.unique(sample[:, c]) for c in range(3)]

    def keys(a, check=None):
        k = None
        for c in range(3):
            col = bits[a:a + chunk, c].contiguous()
            pos = torch.searchsorted(comps[c], col).clamp_(max=comps[c].numel() - 1)
            if check is not None:
                check |= (comps[c][pos] != col).any()
            k = pos if k is None else k * comps[c].numel() + pos
        return k

    index = torch.empty(ncell, dtype=torch.uint8, device=dev)
    combos = comps[0].numel() * comps[1].numel() * comps[2].numel()
    missed = torch.zeros((), dtype=torch.bool, device=dev)
    present = None if combos <= _MAX_TABLE else torch.zeros(combos, dtype=torch.bool, device=dev)
    for a in starts:
        k = keys(a, missed)
        if present is None:
            index[a:a + chunk] = k.to(torch.uint8)
        else:
            present[k] = True
    if bool(missed):
        # the sample missed some values: every distinct value, by sorting
        comps = []
        for c in range(3):
            parts = [torch.unique(bits[a:a + chunk, c]) for a in starts]
            comps.append(torch.unique(torch.cat(parts)) if len(parts) > 1 else parts[0])
        if max(u.numel() for u in comps) > _MAX_TABLE:
            return None
        combos = comps[0].numel() * comps[1].numel() * comps[2].numel()
        present = None if combos <= _MAX_TABLE else torch.zeros(combos, dtype=torch.bool, device=dev)
        for a in starts:
            k = keys(a)
            if present is None:
                index[a:a + chunk] = k.to(torch.uint8)
            else:
                present[k] = True
    n0, n1, n2 = (u.numel() for u in comps)
    if present is None:
        rows = torch.arange(combos, device=dev)
    else:
        rows = torch.nonzero(present).reshape(-1)
        if rows.numel() > _MAX_TABLE:
            return None
        rank = torch.zeros(combos, dtype=torch.uint8, device=dev)
        rank[rows] = torch.arange(rows.numel(), device=dev).to(torch.uint8)
        for a in starts:
            index[a:a + chunk] = rank[keys(a)]
    i2 = rows % n2
    i1 = (rows // n2) % n1
    i0 = rows // (n1 * n2)
    table = torch.stack([comps[0][i0], comps[1][i1], comps[2][i2]], dim=1).view(x.dtype).contiguous()
    return table, index.reshape(x.shape[:-1])


_FUSION_REASONS = {
    1: "float32 plans only", 2: "nz must be a multiple of 4 (and the buffers 16-byte aligned)",
    3: "a SoftArbitraryPointSource", 4: "a PML registered after a periodic boundary",
    5: "a periodic boundary not along x (or fewer than 4 planes along x)",
    6: "an object or source on a periodic plane", 7: "the second buffers could not be allocated",
    8: "too little shared memory for the stages", 9: "the grid is too large for the launch",
    10: "a tensor map was refused",
}


class _PinnedStager:
    """Double-buffered pinned host staging for small per-call tables."""

    def __init__(self):
        self._bufs = [None, None]
        self._events = [None, None]
        self._dev = None
        self._turn = 0

    def upload(self, array, device):
        n = array.size
        k = self._turn
        self._turn ^= 1
        if self._events[k] is not None:
            self._events[k].synchronize()
        if self._bufs[k] is None or self._bufs[k].numel() < n:
            self._bufs[k] = torch.empty(max(n, 1024), dtype=torch.float64).pin_memory()
        host = self._bufs[k][:n]
        host.numpy()[:] = array.reshape(-1)
        dev = torch.empty(n, dtype=torch.float64, device=device)
        dev.copy_(host, non_blocking=True)
        # the copy runs on the current stream of the tensor's device; the event
        # that guards the pinned buffer's reuse must follow that stream
        ev = torch.cuda.Event()
        ev.record(torch.cuda.current_stream(dev.device))
        self._events[k] = ev
        return dev


class Engine:
    def __init__(self, grid, x_chunk=0):
        self.grid = grid
        self.x_chunk = x_chunk
        # fused-pass kernel choice: variant 0 auto / 1 register streaming / 2 TMA-staged
        # materials: 0 compact copies for the staged passes where possible, 1 full arrays only
        # step_fusion: 0 auto / 1 two passes per step / 2 one pass per step (where allowed)
        # persistent: 0 auto / 1 one launch per half step / 2 one persistent launch per run() (where allowed)
        self.tuning = {"variant": 0, "tile_rows": 0, "stages": 0, "pml_mode": 0, "materials": 0, "step_fusion": 0,
                       "persistent": 0}
        self._alt = None  # second buffers of E, H and the PML auxiliaries for one-pass steps
        self.plan = None
        self._key = None
        self._keep = []
        self._scaled = None
        self._scaled_keys = [None, None]
        self._compact = [None, None]  # per material: (table, index or None) or None
        self._compact_keys = [None, None]
        self.trace_E = self.trace_H = self.trace_I = None
        self.capacity = 0
        self.rec_E = self.rec_H = self.rec_I = 0
        self.n_probe = 0
        self.n_current = 0
        self.det_ranges = {}
        self.cur_ranges = {}
        self.dfts = []
        self.n_phase = 0
        self._wave_stage = _PinnedStager()
        self._phase_stage = _PinnedStager()
        self.launches_per_step = 0
        self.refresh()

    # --- plan -------------------------------------------------------------------
    def _state_key(self):
        g = self.grid
        return (tuple(o._coef_key() for o in g.objects), self.x_chunk, tuple(sorted(self.tuning.items())),
                g.courant_number, g._E.data_ptr(), g._H.data_ptr())

    def refresh(self):
        g = self.grid
        key = self._state_key()
        if self.plan is not None and not g._dirty and key == self._key:
            self._sync_scaled_materials()
            if not self._sync_compact_materials():
                return
        self._build()
        self._key = self._state_key()
        g._dirty = False

    # float64 plans read courant * inverse material (the products the
    # reference forms first, rounded the same way) from arrays kept here; they
    # follow in-place changes of the grid's materials before every launch
    def _sync_scaled_materials(self):
        g = self.grid
        if self._scaled is None:
            return
        for src, dst, ver in zip((g._inverse_permittivity, g._inverse_permeability), self._scaled,
                                 range(2)):
            key = (id(src), src._version, g.courant_number)
            if self._scaled_keys[ver] != key:
                torch.mul(src, g.courant_number, out=dst)
                self._scaled_keys[ver] = key

    def _material_arrays(self):
        g = self.grid
        if self._scaled is not None:
            return self._scaled
        return g._inverse_permittivity, g._inverse_permeability

    @staticmethod
    def _layout(enc):
        if enc is None:
            return None
        return (enc[0].shape[0], enc[1] is not None)

    # compact copies follow in-place changes of the material arrays; returns
    # True when their layout changed and the plan must be rebuilt
    def _sync_compact_materials(self):
        g = self.grid
        want = self.tuning["materials"] == 0
        rebuild = False
        for q, src in enumerate(self._material_arrays()):
            key = (src.data_ptr(), src._version, want)
            if self._compact_keys[q] == key:
                continue
            # index maps are read by TMA in rows of nz bytes: nz a multiple of 16;
            # without the memory for the copy the plan reads the full arrays
            enc = None
            if want:
                try:
                    enc = compact_material(src, index_ok=g.Nz % 16 == 0)
                except torch.cuda.OutOfMemoryError:
                    enc = None
            old = self._compact[q]
            if enc is not None and old is not None and self._layout(enc) == self._layout(old):
                old[0].copy_(enc[0])
                if enc[1] is not None:
                    old[1].copy_(enc[1])
            else:
                rebuild |= self._layout(enc) != self._layout(old)
                self._compact[q] = enc
            self._compact_keys[q] = key
        return rebuild

    def compact_materials(self):
        """How the plan's staged passes read each material (inverse permittivity,
        inverse permeability): None (full arrays; always for the register
        kernels), ("uniform", 1) or ("index", n distinct value triples)."""
        if self.plan is None or self.tiling()["variant"] not in (2, 4):
            return [None, None]
        return [None if e is None else (("index", e[0].shape[0]) if e[1] is not None else ("uniform", 1))
                for e in self._compact]

    def set_x_chunk(self, x_chunk):
        self.x_chunk = int(x_chunk)
        self.refresh()

    def set_tuning(self, variant=None, tile_rows=None, stages=None, x_chunk=None, pml_mode=None, materials=None,
                   step_fusion=None, persistent=None):
        """Choose the fused-pass kernels (0 auto, 1 register streaming, 2 TMA-staged),
        the TMA tile rows (4 or 8 with 32-thread-wide tiles, 16 with 16-wide) and
        ring stages, where the PML slabs run
        (0 auto, 1 inside the fused pass, 2 kernels of their own; 3 only the
        leading x/y slabs split off; 4 interior/shell partition: the fused
        pass over the box inside every slab, one kernel with every slab over
        the shell around it), how the staged passes read the
        materials (0 a one-byte index into a table of distinct value triples,
        or nothing for a uniform material, where the materials allow; 1 the
        full arrays), and whether full steps run as one pass each (0 auto:
        currently never, the two-pass plans measured faster; 1 never; 2
        where the grid allows it, else RuntimeError); 0 keeps the automatic
        choice.  The one-pass step uses tile_rows 4 or 8, stages >= 3 and
        x_chunk when given.  persistent: 0 auto (float32 grids below 3M
        cells, float64 below 8M, whose plan allows it), 1 one launch per half step, 2 where allowed: every
        full step of a run() in one cooperative launch."""
        for k, v in (("variant", variant), ("tile_rows", tile_rows), ("stages", stages), ("pml_mode", pml_mode),
                     ("materials", materials), ("step_fusion", step_fusion), ("persistent", persistent)):
            if v is not None:
                self.tuning[k] = int(v)
        if x_chunk is not None:
            self.x_chunk = int(x_chunk)
        self.refresh()

    def tiling(self):
        """dict of the launch shape the plan chose."""
        out = (ctypes.c_int64 * 8)()
        _native.check(_native.load().fdtd_plan_tiling(self.plan, out), "fdtd_plan_tiling")
        keys = ("cells_per_thread_z", "threads_z", "rows_y", "planes_x", "ctas", "launches_per_step",
                "variant", "stages")
        info = dict(zip(keys, (int(v) for v in out)))
        # pml_split: 0 slabs inside the fused pass, 1 slabs in kernels of
        # their own, 2 interior/shell partition (the interior's tiling reported)
        info["pml_split"] = info["variant"] // 10
        info["variant"] %= 10
        # 5: the persistent loop over register-streaming tiles
        info["persistent"] = int(info["variant"] == 5)
        if info["persistent"]:
            info["variant"] = 1
        return info

    def check_status(self):
        """Raise RuntimeError if a staged kernel reported a pipeline failure."""
        lib = _native.load()
        st = ctypes.c_int32(0)
        stream = torch.cuda.current_stream(self.grid._device).cuda_stream
        _native.check(lib.fdtd_plan_status(self.plan, ctypes.byref(st), 1, ctypes.c_void_p(stream)),
                      "fdtd_plan_status")
        if st.value != 0:
            raise RuntimeError(f"fdtd kernel reported failure status {st.value}; results of the last run are "
                               "invalid")

    def _freeze_traces(self):
        for ranges, fields in ((self.det_ranges, ("E", "H")), (self.cur_ranges, ("I",))):
            for det in ranges:
                for field in fields:
                    live = self.detector_records(det, field)
                    if live is not None and live.shape[0]:
                        det._frozen[field].append(live.clone())
                det._engine = None
        self.det_ranges = {}
        self.cur_ranges = {}
        self.trace_E = self.trace_H = self.trace_I = None
        self.capacity = self.rec_E = self.rec_H = self.rec_I = 0

    def _destroy(self):
        if self.plan is not None:
            lib = _native.load()
            torch.cuda.current_stream().synchronize()
            lib.fdtd_plan_destroy(self.plan)
            self.plan = None

    def __del__(self):
        try:
            self._destroy()
        except Exception:
            pass

    def _build(self):
        g = self.grid
        lib = _require_gpu(g)
        self._freeze_traces()
        self._destroy()
        keep = []
        dt = g._dtype
        d = _native.GridDesc()
        d.abi_version = _native.ABI_VERSION
        d.precision = _PRECISION[g.precision]
        d.nx, d.ny, d.nz = g.Nx, g.Ny, g.Nz
        d.x_chunk = self.x_chunk
        d.variant = self.tuning["variant"]
        d.tile_rows = self.tuning["tile_rows"]
        d.stages = self.tuning["stages"]
        d.pml_mode = self.tuning["pml_mode"]
        d.persistent = self.tuning["persistent"]
        d.courant = g.courant_number
        d.E, d.H = g._E.data_ptr(), g._H.data_ptr()
        d.E_lo = g._E_lo.data_ptr() if g._E_lo is not None else None
        d.H_lo = g._H_lo.data_ptr() if g._H_lo is not None else None
        if g.precision == "float64":
            if self._scaled is None or self._scaled[0].shape != g._inverse_permittivity.shape:
                self._scaled = (torch.empty_like(g._inverse_permittivity), torch.empty_like(g._inverse_permeability))
                self._compact_keys = [None, None]  # new arrays: fill and encode them afresh
                self._scaled_keys = [None, None]
            self._sync_scaled_materials()
            d.inv_eps, d.inv_mu = self._scaled[0].data_ptr(), self._scaled[1].data_ptr()
            d.materials_scaled = 1
        else:
            self._scaled = None
            d.inv_eps = g._inverse_permittivity.data_ptr()
            d.inv_mu = g._inverse_permeability.data_ptr()
        # compact copies: re-encoded only if the arrays changed since the last plan
        self._sync_compact_materials()
        for enc, tab, n, idx in ((self._compact[0], "eps_table", "n_eps_table", "eps_index"),
                                 (self._compact[1], "mu_table", "n_mu_table", "mu_index")):
            if enc is not None:
                setattr(d, tab, enc[0].data_ptr())
                setattr(d, n, enc[0].shape[0])
                setattr(d, idx, enc[1].data_ptr() if enc[1] is not None else None)

        if len(g.boundaries) > _native.MAX_BOUNDARIES:
            raise NotImplementedError("more boundaries than the gb300 backend supports")
        for i, b in enumerate(g.boundaries):
            bd_ = d.boundaries[i]
            if isinstance(b, PML):
                bd_.kind = _native.BOUNDARY_PML
                bd_.axis, bd_.high, bd_.thickness = b.axis, b.high, b.thickness
                for name in ("psi_E", "psi_H", "b_E", "c_E", "b_H", "c_H"):
                    t = getattr(b, "_" + name if name.startswith("psi") else name)
                    if t.dtype != dt or not t.is_contiguous() or t.device.type != "cuda":
                        raise RuntimeError(f"PML {name} must be a contiguous {dt} CUDA tensor")
                    setattr(bd_, name, t.data_ptr())
            elif isinstance(b, PeriodicBoundary):
                bd_.kind = _native.BOUNDARY_PERIODIC
                bd_.axis = b.axis
            else:
                raise NotImplementedError(f"boundary {type(b).__name__} is not supported by the gb300 backend")
        d.n_boundaries = len(g.boundaries)

        objs = (_native.ItemDesc * max(1, len(g.objects)))()
        for i, o in enumerate(g.objects):
            coefs = o._coefficients(dt)
            keep.extend(coefs)
            it = objs[i]
            it.kind = o._kind
            it.lo[:] = [o.x.start, o.y.start, o.z.start]
            it.hi[:] = [o.x.stop, o.y.stop, o.z.stop]
            for q, c in enumerate(coefs):
                it.coef[q] = c.data_ptr()
        d.n_objects = len(g.objects)
        d.objects = objs
        keep.append(objs)

        cells, ccells = [], []
        self.n_probe = self.n_current = 0
        self.det_ranges = {}
        self.cur_ranges = {}
        self.dfts = []
        dfts = []
        nph = 0
        for det in g.detectors:
            if isinstance(det, DFTPlaneDetector):
                dd = _native.DftDesc()
                dd.lo[:] = [det.x.start, det.y.start, det.z.start]
                dd.hi[:] = [det.x.stop, det.y.stop, det.z.stop]
                dd.n_freq = len(det.frequencies)
                dd.phase_offset = nph
                dd.acc = det.dft.data_ptr()
                nph += dd.n_freq
                dfts.append(dd)
                self.dfts.append(det)
            elif isinstance(det, CurrentDetector):
                c = det._probe_cells()
                self.cur_ranges[det] = (self.n_current, self.n_current + c.size)
                self.n_current += c.size
                ccells.append(c)
                det._engine = self
            elif hasattr(det, "_probe_cells"):
                c = det._probe_cells()
                self.det_ranges[det] = (self.n_probe, self.n_probe + c.size)
                self.n_probe += c.size
                cells.append(c)
                det._engine = self
            else:
                raise NotImplementedError(f"detector {type(det).__name__} is not supported by the gb300 backend")
        if self.n_probe:
            probe = torch.as_tensor(np.concatenate(cells), dtype=torch.int64, device=g._device)
            keep.append(probe)
            d.n_probe_cells, d.probe_cells = self.n_probe, probe.data_ptr()
        if self.n_current:
            cur = torch.as_tensor(np.concatenate(ccells), dtype=torch.int64, device=g._device)
            keep.append(cur)
            d.n_current_cells, d.current_cells = self.n_current, cur.data_ptr()
        d.grid_spacing = g.grid_spacing
        arrD = (_native.DftDesc * max(1, len(dfts)))(*dfts)
        d.n_dft, d.dft = len(dfts), arrD
        d.n_phase_columns = nph
        self.n_phase = nph
        keep.append(arrD)

        itemsE, itemsH = [], []
        self.sources = list(g.sources)
        for col, s in enumerate(self.sources):
            if not hasattr(s, "_items"):
                raise NotImplementedError(f"source {type(s).__name__} is not supported by the gb300 backend")
            for field, kind, comp, lo, hi, w in s._items():
                it = _native.ItemDesc()
                it.kind = {"soft": _native.ITEM_SOFT, "hard": _native.ITEM_HARD,
                           "feedback": _native.ITEM_FEEDBACK}[kind]
                if kind == "feedback":
                    det = s.current_detector
                    if det not in self.cur_ranges:
                        raise RuntimeError("a SoftArbitraryPointSource needs its current detector in grid.detectors")
                    it.aux = self.cur_ranges[det][0]
                it.comp, it.column, it.source = comp, col, col
                it.lo[:] = list(lo)
                it.hi[:] = list(hi)
                it.weight = w
                (itemsE if field == "E" else itemsH).append(it)
        arrE = (_native.ItemDesc * max(1, len(itemsE)))(*itemsE)
        arrH = (_native.ItemDesc * max(1, len(itemsH)))(*itemsH)
        d.n_sources_E, d.sources_E = len(itemsE), arrE
        d.n_sources_H, d.sources_H = len(itemsH), arrH
        d.n_columns = len(self.sources)
        keep.extend([arrE, arrH])


        # one pass per step: the library decides whether the grid allows it;
        # the second buffers it needs are allocated only when it will be used
        # (when asked: the automatic choice keeps the two-pass plans, which
        # measured faster on every benchmark grid)
        req = self.tuning["step_fusion"]
        if self._alt is not None and (req == 1 or not self._alt_fits()):
            self._alt = None
        if self._alt is not None:
            self._set_alt(d)
            d.step_fusion = req
        else:
            d.step_fusion = 1 if req == 2 else req  # without the buffers: only ask whether it is allowed
        plan = ctypes.c_void_p()
        _native.check(lib.fdtd_plan_create(ctypes.byref(d), ctypes.byref(plan)), "fdtd_plan_create")
        allowed, active, why = ctypes.c_int32(0), ctypes.c_int32(0), ctypes.c_int32(0)
        _native.check(lib.fdtd_plan_step_fusion(plan, ctypes.byref(allowed), ctypes.byref(active), ctypes.byref(why)),
                      "fdtd_plan_step_fusion")
        want = req == 2
        if allowed.value and want and not active.value and self._alt is None:
            try:
                self._alloc_alt()
            except torch.cuda.OutOfMemoryError:
                self._alt = None
            if self._alt is not None:
                lib.fdtd_plan_destroy(plan)
                self._set_alt(d)
                d.step_fusion = req
                plan = ctypes.c_void_p()
                _native.check(lib.fdtd_plan_create(ctypes.byref(d), ctypes.byref(plan)), "fdtd_plan_create")
                _native.check(lib.fdtd_plan_step_fusion(plan, ctypes.byref(allowed), ctypes.byref(active),
                                                        ctypes.byref(why)), "fdtd_plan_step_fusion")
        if req == 2 and not active.value:
            lib.fdtd_plan_destroy(plan)
            self._alt = None
            raise RuntimeError(f"one pass per time step (step_fusion=2) is not possible here: "
                               f"{_FUSION_REASONS.get(why.value, why.value)}")
        if not active.value:
            self._alt = None
        self.plan = plan
        self._keep = keep
        self.launches_per_step = self.tiling()["launches_per_step"]

    # --- one pass per step: second buffers -----------------------------------------
    def _alt_shapes(self):
        g = self.grid
        shapes = [tuple(g._E.shape), tuple(g._H.shape)]
        for b in g.boundaries:
            if isinstance(b, PML):
                shapes += [tuple(b._psi_E.shape), tuple(b._psi_H.shape)]
        return shapes

    def _alt_fits(self):
        return [tuple(t.shape) for t in self._alt] == self._alt_shapes() and self._alt[0].dtype == self.grid._dtype

    def _alloc_alt(self):
        g = self.grid
        alt = [torch.empty_like(g._E), torch.empty_like(g._H)]
        for b in g.boundaries:
            if isinstance(b, PML):
                alt += [torch.empty_like(b._psi_E), torch.empty_like(b._psi_H)]
        self._alt = alt

    def _set_alt(self, d):
        g = self.grid
        d.E_alt, d.H_alt = self._alt[0].data_ptr(), self._alt[1].data_ptr()
        q = 2
        for i, b in enumerate(g.boundaries):
            if isinstance(b, PML):
                d.psi_alt[i][0] = self._alt[q].data_ptr()
                d.psi_alt[i][1] = self._alt[q + 1].data_ptr()
                q += 2

    def step_fusion(self):
        """(allowed, active): whether this grid admits one pass per time step
        and whether its full steps run that way."""
        allowed, active = ctypes.c_int32(0), ctypes.c_int32(0)
        _native.check(_native.load().fdtd_plan_step_fusion(self.plan, ctypes.byref(allowed), ctypes.byref(active),
                                                            None), "fdtd_plan_step_fusion")
        return bool(allowed.value), bool(active.value)

    # --- traces ---------------------------------------------------------------
    def _ensure_capacity(self, need):
        if need <= self.capacity:
            return
        g = self.grid
        cap = max(need, 2 * self.capacity, 16)
        newE = torch.empty((cap, self.n_probe, 3), dtype=g._dtype, device=g._device)
        newH = torch.empty((cap, self.n_probe, 3), dtype=g._dtype, device=g._device)
        newI = torch.empty((cap, self.n_current), dtype=g._dtype, device=g._device)
        if self.trace_E is not None:
            newE[: self.rec_E].copy_(self.trace_E[: self.rec_E])
            newH[: self.rec_H].copy_(self.trace_H[: self.rec_H])
            newI[: self.rec_I].copy_(self.trace_I[: self.rec_I])
        self.trace_E, self.trace_H, self.trace_I, self.capacity = newE, newH, newI, cap

    def detector_records(self, det, field):
        if field == "I":
            rng = self.cur_ranges.get(det)
            if rng is None or self.trace_I is None:
                return None
            p0, p1 = rng
            return self.trace_I[: self.rec_I, p0:p1].reshape((self.rec_I,) + det._rec_shape)
        rng = self.det_ranges.get(det)
        buf = self.trace_E if field == "E" else self.trace_H
        if rng is None or buf is None:
            return None
        n = self.rec_E if field == "E" else self.rec_H
        p0, p1 = rng
        return buf[:n, p0:p1, :].reshape((n,) + det._rec_shape)

    # --- stepping --------------------------------------------------------------
    def phase_table(self, steps):
        """(len(steps), n_phase, 2) float64 numpy table of the DFT factors
        (cos, -sin) of 2 pi f q dt for the step indices q in ``steps``."""
        g = self.grid
        ph = np.empty((len(steps), self.n_phase, 2), dtype=np.float64)
        t = np.asarray(steps, dtype=np.float64) * g.time_step
        col = 0
        for det in self.dfts:
            for f in det.frequencies:
                theta = (2.0 * math.pi * f) * t
                ph[:, col, 0] = np.cos(theta)
                ph[:, col, 1] = -np.sin(theta)
                col += 1
        return ph

    def upload_phase(self, table):
        return self._phase_stage.upload(table, self.grid._device)

    def _tables(self, q0, n, dft=True):
        g = self.grid
        wave = phase = None
        if self.sources:
            tab = np.empty((n, len(self.sources)), dtype=np.float64)
            for c, s in enumerate(self.sources):
                # the reference's scalar expressions (math.sin), one per step
                tab[:, c] = [s._value(q) for q in range(q0, q0 + n)]
            wave = self._wave_stage.upload(tab, g._device)
        if self.n_phase and dft:
            phase = self.upload_phase(self.phase_table(range(q0, q0 + n)))
        return wave, phase

    def _launch(self, n, half, capture=None):
        """fdtd_run, or with ``capture = (detectors, curls)`` fdtd_run_capture
        (curls: per object a device tensor of n rows or None)."""
        g = self.grid
        lib = _native.load()
        q0 = g.time_steps_passed
        detect = capture is None or capture[0]
        wave, phase = self._tables(q0, n, dft=detect)
        a = _native.RunArgs()
        a.n_steps, a.half = n, half
        a.wave = wave.data_ptr() if wave is not None else None
        a.phase = phase.data_ptr() if phase is not None else None
        a.step0 = q0
        if (self.n_probe or self.n_current) and detect:
            need_E = self.rec_E + (n if half != 2 else 0)
            need_H = max(self.rec_H, self.rec_I) + (n if half != 1 else 0)
            self._ensure_capacity(max(need_E, need_H))
            a.trace_E, a.trace_H = self.trace_E.data_ptr(), self.trace_H.data_ptr()
            a.trace_I = self.trace_I.data_ptr()
            a.trace_capacity = self.capacity
            a.record_E, a.record_H, a.record_I = self.rec_E, self.rec_H, self.rec_I
            if half != 2:
                # feedback sources: the current record each E half step reads
                # (the record of the previous H half; none at step 0)
                for src in self.sources:
                    if hasattr(src, "current_detector") and src.current_detector in self.cur_ranges:
                        det = src.current_detector
                        frozen = sum(c.shape[0] for c in det._frozen["I"])
                        src._note_steps(q0, n, frozen, self.rec_I - 1)
        stream = ctypes.c_void_p(torch.cuda.current_stream(g._device).cuda_stream)
        if capture is None:
            _native.check(lib.fdtd_run(self.plan, ctypes.byref(a), stream), "fdtd_run")
        else:
            curls = capture[1]
            c = _native.CaptureArgs()
            c.detectors = 1 if detect else 0
            c.n_curl = len(curls)
            arr = (ctypes.c_void_p * max(1, len(curls)))(*[_native.ptr(t) for t in curls])
            c.curl = arr
            _native.check(lib.fdtd_run_capture(self.plan, ctypes.byref(a), ctypes.byref(c), stream),
                          "fdtd_run_capture")
        if (self.n_probe or self.n_current) and detect:
            if half != 2:
                self.rec_E += n
            if half != 1:
                self.rec_H += n
                self.rec_I += n

    def run_capture(self, n, curls, detectors):
        """n full steps from time_steps_passed capturing curl_H on object boxes
        (reverse-time adjoint); time_steps_passed += n."""
        if n <= 0:
            return
        self._launch(n, 0, capture=(detectors, curls))
        self.grid.time_steps_passed += n

    def run(self, n):
        """n full steps from time_steps_passed, then time_steps_passed += n."""
        self.refresh()
        if n <= 0:
            return
        self._launch(n, 0)
        self.grid.time_steps_passed += n

    def half(self, field):
        """One E (field='E') or H half step at the current step index."""
        self.refresh()
        self._launch(1, 1 if field == "E" else 2)

    def stats(self):
        lib = _native.load()
        g = self.grid
        nbytes = lib.fdtd_stats_scratch_bytes(self.plan)
        scratch = torch.empty(max(int(nbytes), 8), dtype=torch.uint8, device=g._device)
        out = torch.empty(5, dtype=torch.float64, device=g._device)
        stream = torch.cuda.current_stream(g._device).cuda_stream
        _native.check(lib.fdtd_field_stats(self.plan, out.data_ptr(), scratch.data_ptr(), ctypes.c_void_p(stream)),
                      "fdtd_field_stats")
        v = out.cpu().tolist()
        self.check_status()
        return {"sum_E2": v[0], "sum_H2": v[1], "max_abs_E": v[2], "max_abs_H": v[3], "nonfinite": int(v[4])}
