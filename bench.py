#!/usr/bin/env python
"""Throughput benchmark of the GB300 fdtd time step.

Workload: config 3 -- a 768^3 grid with 400 random dielectric blocks
(eps in {1, 2.25, 12.1}, seed 3) rasterised into the grid permittivity,
20-cell PML on y and z, periodic x, a point source at the centre and a line
detector along x through the centre.  A step is one full E + H time step of
the whole grid.  Fields and materials (about 22 GB in float32) are larger
than L2, so no flush is needed between steps.

Printed line (rank 0): value = float32 Gcell-updates/s of all ranks, with
the float64 and compensated float32 runs of the same grid, the float32 /
float64 detector-trace error (the timed records and the 1000-step run), the
roofline of the fused half-step kernels (HBM-bound), the end-to-end figure
through the public API with per-step host<->device copies, launch count and
SM clocks sampled during the timed region; configs 2 and 5 at full size
(throughput and HBM fraction per precision, long-run float32 / float32c
error against float64: config 2's block detector over 2000 steps, config
5's DFT accumulators); the cost of a differentiable run (adjoint) over a
forward run on configs 4 and 5, with the config-4 gradient checked against
central finite differences; and the reference's own CPU time step (its
numpy backend, and its torch.float64 backend on all host threads) on a
128^3 crop of the config-3 generator.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

``--impl reference`` times the reference's own numpy time step (the
unmodified package installed in baseline/_ref; the oracle port of it only if
that is absent) on the same 128^3 crop, one contract step per time step.
N > 1 runs one independent replica per rank (the path has no exchange step).
"""

import argparse
import gc
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time
from datetime import datetime

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Gcell-updates/s FP32 vs FP64 at stated error; %HBM peak; adjoint/forward time"
UNIT = "Gcell-updates/s"
# algorithmic bytes per cell and half step: read field, read neighbour field,
# read inverse material, write field (3 components each); compensated adds the
# read and write of the compensation term.  PML slab cells add the read and
# write of their two auxiliaries.
CELL_BYTES = {"float32": 48, "float32c": 72, "float64": 96}  # per cell and half step, full material arrays
SLAB_BYTES = {"float32": 16, "float32c": 16, "float64": 32}
MAT_BYTES = {"float32": 12, "float32c": 12, "float64": 24}  # the three material values of a cell


def half_bytes(prec, layout):
    """Algorithmic bytes per cell of one fused half step for a material layout
    (None: full arrays, ("index", n): one byte, ("uniform", 1): nothing)."""
    mat = MAT_BYTES[prec] if layout is None else (1 if layout[0] == "index" else 0)
    return CELL_BYTES[prec] - MAT_BYTES[prec] + mat


def parse():
    p = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=100)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", choices=["gb300", "reference", "reference-gpu"], default="gb300",
                   help="reference: the reference's own numpy time step on the host cores; "
                        "reference-gpu: the reference's own torch CUDA backend from baseline/_ref")
    p.add_argument("--ref-backend", default="torch.cuda.float64",
                   help="backend name of the reference for --impl reference-gpu")
    p.add_argument("--n", type=int, default=768, help="grid edge (config 3 is 768)")
    p.add_argument("--pml", type=int, default=-1, help="PML cells on y and z (default 20 scaled by n/768; 0 = none)")
    p.add_argument("--x-chunk", type=int, default=0, help="planes per CTA along x (0 = plan default)")
    p.add_argument("--variant", type=int, default=0, help="0 auto, 1 register streaming, 2 TMA-staged")
    p.add_argument("--tile-rows", type=int, default=0)
    p.add_argument("--stages", type=int, default=0)
    p.add_argument("--pml-mode", type=int, default=0,
                   help="0 auto, 1 PML inside the fused pass, 2 slab kernels, 3 leading x/y slabs fused and the "
                        "rest in slab kernels")
    p.add_argument("--materials", type=int, default=0,
                   help="0 compact material copies where possible (one-byte index or uniform), 1 full arrays")
    p.add_argument("--cpu-seconds", type=float, default=15.0, help="CPU baseline budget")
    p.add_argument("--skip-cpu", action="store_true")
    p.add_argument("--skip-adjoint", action="store_true", help="skip the adjoint/forward timing (configs 4, 5)")
    p.add_argument("--adjoint-only", choices=["c4", "c5", "both"], default=None,
                   help="only the adjoint/forward timing of the named configs (prints its own JSON line)")
    p.add_argument("--only", choices=["float32", "float32c", "float64"], default=None)
    p.add_argument("--error-steps", type=int, default=1000,
                   help="config 3: steps of the long-run float32 / float32c trace error against float64 (0 = off)")
    p.add_argument("--skip-configs", action="store_true",
                   help="skip configs 2 and 5 (forward throughput, roofline and long-run errors)")
    p.add_argument("--step-fusion", type=int, default=0,
                   help="0 auto, 1 two passes per step, 2 one pass per step (float32 grids that allow it)")
    p.add_argument("--forward-only", choices=["c1", "c2", "c4", "c5"], default=None,
                   help="only --warmup + --steps float32 forward steps of the named config (a profiling target; "
                        "prints its own JSON line)")
    p.add_argument("--configs-only", action="store_true",
                   help="only configs 2 and 5 (prints its own JSON line)")
    p.add_argument("--small", action="store_true",
                   help="with --forward-only: the same scene generator on a smaller grid that gets the same "
                        "automatic plan (config 2: 208^3 with a 13-cell PML; config 5: 256x256x192 with its 20-cell "
                        "PML), about 1 GB on the device, for detailed ncu captures")
    return p.parse_args()


# --------------------------------------------------------------------------
# distributed helpers (replicas only)
# --------------------------------------------------------------------------
class Dist:
    def __init__(self):
        import torch

        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist

            backend = "nccl" if torch.cuda.is_available() else "gloo"
            if torch.cuda.is_available():
                torch.cuda.set_device(self.local)
            dist.init_process_group(backend=backend)
            self.pg = dist

    def barrier(self):
        if self.pg is not None:
            self.pg.barrier()

    def max(self, v):
        if self.pg is None:
            return v
        import torch

        t = torch.tensor([v], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg is not None:
            self.pg.destroy_process_group()


# --------------------------------------------------------------------------
# clocks during the timed region
# --------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(prefix="clocks", suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None
        time.sleep(0.3)

    def stop(self, t0, t1):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        self.proc.wait()
        rows = []
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 10:
                continue
            try:
                ts = datetime.strptime(parts[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
            except ValueError:
                continue
            rows.append((ts, parts))
        os.unlink(self.path)
        inside = [p for ts, p in rows if t0 - 0.15 <= ts <= t1 + 0.15] or [p for _, p in rows]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        sm, smax, power = [], [], []
        for p in inside:
            try:
                sm.append(float(p[2]))
                smax.append(float(p[3]))
                power.append(float(p[4]))
            except ValueError:
                pass
            for k, name in enumerate(names):
                if p[6 + k].lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "power_w_max": max(power) if power else None, "samples": len(inside),
                "reasons": sorted(reasons)}


# --------------------------------------------------------------------------
# GPU arm
# --------------------------------------------------------------------------
def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def traffic_from_profile(precision, n, half, materials, automatic_plan):
    """DRAM bytes of one half step (fused pass and its slab kernels) from the
    committed ncu summary, if it covers this precision, material layout and
    (automatic) plan."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    if (not os.path.exists(path) or not automatic_plan or materials["E"] is None or materials["H"] is None
            or (materials["E"][0], materials["H"][0]) != ("index", "uniform")):
        return None
    with open(path) as f:
        d = json.load(f)
    ent = d.get(precision, {}).get(half)
    if not ent:
        return None
    # per-cell traffic measured on a smaller grid, scaled to this workload
    return ent["bytes_per_cell"] * n ** 3


def build_grid(fd, scenes, prec, n, eps, args):
    fd.set_backend("gb300." + prec)
    pml = max(2, int(round(20 * n / 768))) if args.pml < 0 else args.pml
    g = scenes.c3(fd, n=n, pml=pml, eps=eps, detector=True)
    eng = g._ensure_engine()
    eng.set_tuning(variant=args.variant, tile_rows=args.tile_rows, stages=args.stages, x_chunk=args.x_chunk,
                   pml_mode=args.pml_mode, materials=args.materials, step_fusion=args.step_fusion)
    return g, eng


def slab_cells(grid):
    from fdtd_gb300 import PML

    tot = 0
    for b in grid.boundaries:
        if isinstance(b, PML):
            tot += b.shape[0] * b.shape[1] * b.shape[2]
    return tot


def run_precision(prec, args, dist, fd, scenes, eps, want_halves, want_e2e, sampler=None):
    import torch

    n = args.n
    cells = n ** 3
    g, eng = build_grid(fd, scenes, prec, n, eps, args)
    tiling = eng.tiling()
    g.run(args.warmup, progress_bar=False)
    torch.cuda.synchronize()
    dist.barrier()
    stream = torch.cuda.current_stream()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if sampler is not None:
        sampler.start()
    t0 = time.time()
    ev0.record(stream)
    g.run(args.steps, progress_bar=False)
    ev1.record(stream)
    torch.cuda.synchronize()
    t1 = time.time()
    dist.barrier()
    ms = dist.max(ev0.elapsed_time(ev1))
    clocks = sampler.stop(t0, t1) if sampler is not None else None
    out = {
        "precision": prec,
        "ms_per_step": ms / args.steps,
        "gcells": cells * args.steps * dist.world / (ms * 1e-3) / 1e9,
        "launches_per_step": tiling["launches_per_step"],
        "tiling": tiling,
        "clocks": clocks,
        "trace": g.detector.E.tensor()[: args.warmup + args.steps].double().cpu(),
        "stats": g.field_stats(),
    }
    layout = eng.compact_materials()
    out["materials"] = {"E": layout[0], "H": layout[1]}
    slabs = slab_cells(g) * SLAB_BYTES[prec]
    out["algo_bytes"] = {"E": cells * half_bytes(prec, layout[0]) + slabs,
                         "H": cells * half_bytes(prec, layout[1]) + slabs}
    out["full_bytes_half"] = cells * CELL_BYTES[prec] + slabs
    if want_halves:
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True),
                torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        torch.cuda.synchronize()
        for a, b, c in evs:
            a.record(stream)
            g.update_E()
            b.record(stream)
            g.update_H()
            c.record(stream)
            g.time_steps_passed += 1
        torch.cuda.synchronize()
        tE = [a.elapsed_time(b) for a, b, c in evs]
        tH = [b.elapsed_time(c) for a, b, c in evs]
        out["half_ms"] = {"E": statistics.mean(tE), "H": statistics.mean(tH)}
    if want_e2e:
        m = g.detector._rec_shape
        host = torch.empty((args.steps,) + m, dtype=g.E.dtype).pin_memory()
        torch.cuda.synchronize()
        w0 = time.perf_counter()
        for s in range(args.steps):
            g.step()
            host[s].copy_(g.detector.E[-1], non_blocking=True)
        torch.cuda.synchronize()
        w1 = time.perf_counter()
        e2e_s = dist.max(w1 - w0)
        out["e2e"] = {"value": cells * args.steps * dist.world / e2e_s / 1e9, "unit": UNIT,
                      "h2d_bytes_per_step": 8 * len(g.sources),
                      "d2h_bytes_per_step": int(host[0].numel() * host.element_size()),
                      "how": "per step: grid.step() (host waveform -> pinned -> device, fused kernels via the "
                             "C ABI) then the step's detector record copied device -> pinned host"}
    if args.error_steps and g.time_steps_passed < args.error_steps:
        # same physical steps in every precision (runs, half steps, single
        # steps): continue to the long-run length and keep that trace
        g.run(args.error_steps - g.time_steps_passed, progress_bar=False)
        torch.cuda.synchronize()
        out["trace_long"] = g.detector.E.tensor()[: args.error_steps].double().cpu()
    del g, eng
    gc.collect()  # grids and their components reference each other
    torch.cuda.empty_cache()
    return out


CPU_CROP = 128  # edge of the config-3 crop every CPU figure runs on


def reference_module():
    """The unmodified reference package installed in baseline/_ref (pip
    install of the reference), imported with the no-op matplotlib stand-in
    its plotting module needs (and a tqdm stand-in where tqdm is absent);
    None when it is not installed."""
    ref_dir = os.path.join(ROOT, "baseline", "_ref")
    if not os.path.isfile(os.path.join(ref_dir, "fdtd", "__init__.py")):
        return None
    for p in (ref_dir, os.path.join(ROOT, "tests", "golden", "mplstub")):
        if p not in sys.path:
            sys.path.insert(0, p)
    stub = os.path.join(ROOT, "tests", "golden", "tqdmstub")
    if stub not in sys.path:
        sys.path.append(stub)
    import fdtd as ref

    return ref


def cpu_rate(backend="numpy", steps=None, budget_s=None, warmup=1, n=CPU_CROP):
    """Gcell-updates/s of the reference's own CPU time step (``backend``
    "numpy" or "torch.float64") on the config-3 generator cropped to n^3,
    either for ``steps`` timed steps or for about ``budget_s`` seconds.
    Falls back to the oracle port of the numpy time step when the reference
    is not installed."""
    import torch

    from fdtd_gb300 import scenes

    pml = max(2, int(round(20 * n / 768)))
    dtype0 = torch.get_default_dtype()  # importing the reference sets float64
    ref = reference_module()
    threads = 1
    if ref is not None:
        ref.set_backend(backend)
        mod, kind = ref, "reference"
        if backend.startswith("torch"):
            threads = torch.get_num_threads()
    else:
        if backend != "numpy":
            return None
        from oracle import fdtd_oracle as fo

        mod, kind = fo, "port"
    try:
        g = scenes.c3(mod, n=n, pml=pml, detector=True)
        run = (lambda k: g.run(k, progress_bar=False)) if kind == "reference" else g.run
        run(max(1, warmup))
        if steps is None:
            t0 = time.perf_counter()
            run(1)
            per = time.perf_counter() - t0
            steps = int(max(3, min(2000, budget_s / max(per, 1e-4))))
        t0 = time.perf_counter()
        run(steps)
        dt = time.perf_counter() - t0
    finally:
        if ref is not None:
            ref.set_backend("numpy")
        torch.set_default_dtype(dtype0)
    what = {"reference": f"the reference's own {backend} backend (baseline/_ref, unmodified)",
            "port": "the numpy oracle port of the reference's time step (reference not installed)"}[kind]
    return {"value": n ** 3 * steps / dt / 1e9, "unit": UNIT, "cores": threads, "host_cores": os.cpu_count(),
            "kind": kind, "steps": steps, "seconds": dt,
            "sample": f"{what}, float64, on the config-3 generator cropped to {n}^3 ({pml}-cell PML on y/z, "
                      f"periodic x, centre point source, x line detector), {steps} steps in {dt:.1f} s, "
                      + ("one host core (numpy elementwise is single-threaded)" if threads == 1 else
                         f"{threads} torch threads")}


def c4_finite_differences(fd, scenes, grad, loss_of, voxels=16, h=1e-3, seed=4):
    """Central differences of the config-4 loss at random design voxels with
    the float64 forward, against the adjoint gradient: relative L2 over the
    sampled voxels."""
    import numpy as np
    import torch

    fd.set_backend("gb300.float64")
    base = scenes.c4_design(48)
    rng = np.random.default_rng(seed)
    flat = rng.choice(base.size, size=voxels, replace=False)
    fdg, adj = [], []
    t = time.perf_counter()
    for f in flat:
        idx = np.unravel_index(f, base.shape)
        vals = []
        for sgn in (1.0, -1.0):
            d = base.copy()
            d[idx] += sgn * h
            g = scenes.c4(fd)
            g.design.inverse_permittivity = torch.as_tensor(d)[..., None].expand(48, 48, 48, 3)
            g.run(1000, progress_bar=False)
            vals.append(float(loss_of({"detector": {"E": g.detector.E.tensor()}})))
            del g
        fdg.append((vals[0] - vals[1]) / (2 * h))
        adj.append(float(grad[idx]))
    fdg, adj = np.array(fdg), np.array(adj)
    fd.set_backend("gb300.float32")
    return {"voxels": voxels, "step": h, "forward": "f64", "seconds": time.perf_counter() - t,
            "rel_l2": float(np.linalg.norm(adj - fdg) / np.linalg.norm(fdg)),
            "max_rel": float(np.max(np.abs(adj - fdg) / np.maximum(np.abs(fdg), 1e-300)))}


def adjoint_ratio(fd, scenes, which, fd_check=True):
    """Wall time of a differentiable run (fdtd_gb300.adjoint.run plus the
    backward pass) over the wall time of the same forward run (grid.run),
    configs 4 and 5 at full size, float32 fields and float64 gradients."""
    import torch

    def sync():
        torch.cuda.synchronize()

    out = {}
    for cfg in which:
        fd.set_backend("gb300.float32")
        if cfg == "c4":
            steps, K = 1000, 50
            make = lambda: scenes.c4(fd)
            design = lambda: torch.tensor(scenes.c4_design(48), device="cuda", requires_grad=True)
            # the last 200 records (steps 800-999 of the timed run); the warm-up run
            # uses the same operations on its own last records
            loss_of = lambda o: (o["detector"]["E"][-200:, :, :, 0, 2].double() ** 2).sum()
            desc = ("128^3, 12-cell PML, 48^3 design Object, plane source z=16, loss sum Ez^2 on the plane "
                    "z=110 over steps 800-999")
        else:
            steps, K = 2000, 100
            make = lambda: scenes.c5(fd)
            design = lambda: torch.tensor(scenes.c5_tensors(96, 96, 48), device="cuda", requires_grad=True)
            loss_of = lambda o: (o["dft"]["dft"][..., 0:2].abs() ** 2).sum()
            desc = ("384x384x192, 20-cell PML, 96x96x48 anisotropic design (3x3 per cell), Gaussian plane "
                    "source, loss sum over 1500/1550/1600 nm and the DFT plane of |F(Ex)|^2+|F(Ey)|^2")
        g = make()
        g.run(3, progress_bar=False)
        sync()
        t = time.perf_counter()
        g.run(steps, progress_bar=False)
        sync()
        t_fwd = time.perf_counter() - t
        del g
        # warm-up differentiable run (loads the adjoint kernels), then the timed one
        g = make()
        p = design()
        loss_of(fd.adjoint.run(g, 2 * K, {g.design: p}, checkpoint_every=K)).backward()
        del g, p
        gc.collect()
        torch.cuda.empty_cache()
        g = make()
        p = design()
        sync()
        t = time.perf_counter()
        outs = fd.adjoint.run(g, steps, {g.design: p}, checkpoint_every=K)
        loss = loss_of(outs)
        loss.backward()
        sync()
        t_adj = time.perf_counter() - t
        out[cfg] = {"workload": desc, "steps": steps, "checkpoint_every": K, "forward_ms": t_fwd * 1e3,
                    "adjoint_ms": t_adj * 1e3, "adjoint_over_forward": t_adj / t_fwd,
                    "precision": "f32 fields, f64 gradient accumulation",
                    "loss": float(loss.detach()), "grad_norm": float(p.grad.norm())}
        grad_ck = p.grad.detach().clone()
        del g, p, outs, loss
        gc.collect()
        torch.cuda.empty_cache()
        # the same run keeping the design-box curls of every step in device
        # memory (checkpoint_every=None: one segment, no recompute)
        g = make()
        p = design()
        sync()
        t = time.perf_counter()
        outs = fd.adjoint.run(g, steps, {g.design: p}, checkpoint_every=None)
        loss = loss_of(outs)
        loss.backward()
        sync()
        t_st = time.perf_counter() - t
        cells = g.design.Nx * g.design.Ny * g.design.Nz
        out[cfg]["all_curls_kept"] = {
            "adjoint_ms": t_st * 1e3, "adjoint_over_forward": t_st / t_fwd,
            "curl_store_gb": steps * cells * 3 * 4 / 1e9,
            "grad_rel_diff_vs_checkpointed": float((p.grad - grad_ck).norm() / grad_ck.norm())}
        del grad_ck
        if cfg == "c4" and fd_check:
            out[cfg]["fd_check"] = c4_finite_differences(fd, scenes, p.grad.detach().cpu().numpy(), loss_of)
        del g, p, outs, loss
        gc.collect()
        torch.cuda.empty_cache()
    return out


def config_runs(fd, scenes, which=("c2", "c5")):
    """Configs 2 and 5 at full size in float64, float32 and float32c from zero
    fields: forward Gcell-updates/s and the fraction of the measured HBM
    bandwidth by the algorithmic bytes of the step (CUDA events around the
    whole run), and the long-run error of float32 / float32c against float64
    on the same grid: config 2 the 33^3 BlockDetector E and H records over
    2000 steps, config 5 the float64 DFT accumulators after 2000 steps."""
    import torch

    peak, _ = peaks()
    out = {}
    for cfg in which:
        if cfg == "c2":
            steps = 2000
            eps = scenes.c2_permittivity(256)
            make = lambda: scenes.c2(fd, eps=eps)
            desc = ("256^3 uniaxial random eps ~ U[1,12] smoothed by a 3-cell box filter, 16-cell PML, "
                    "AbsorbingObject 64^3 sigma 1e4 S/m, x-polarised PlaneSource z=20, 33^3 BlockDetector")
        else:
            steps = 2000
            make = lambda: scenes.c5(fd)
            desc = ("384x384x192, 20-cell PML, 96x96x48 AnisotropicObject (random SPD), Gaussian PlaneSource "
                    "z=24, float64 DFT plane z=168 at 1500/1550/1600 nm")
        res, ref_out = {}, None
        for prec in ("float64", "float32", "float32c"):
            fd.set_backend("gb300." + prec)
            g = make()
            g.run(3, progress_bar=False)  # plan, material copies and kernels loaded
            del g
            gc.collect()
            g = make()
            eng = g._ensure_engine()
            eng.refresh()
            cells = g.Nx * g.Ny * g.Nz
            layout = eng.compact_materials()
            slabs = slab_cells(g) * SLAB_BYTES[prec]
            step_bytes = cells * (half_bytes(prec, layout[0]) + half_bytes(prec, layout[1])) + 2 * slabs
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            g.run(steps, progress_bar=False)
            e1.record()
            torch.cuda.synchronize()
            eng.check_status()
            ms = e0.elapsed_time(e1)
            det = g.detectors[0]
            if cfg == "c2":
                rec = (det.E.tensor().double(), det.H.tensor().double())
            else:
                rec = (det.dft.clone(),)
            res[prec] = {"value": cells * steps / (ms * 1e-3) / 1e9, "ms_per_step": ms / steps,
                         "hbm_frac": step_bytes * steps / (ms * 1e-3) / 1e9 / peak,
                         "algo_bytes_per_step": step_bytes, "tiling": eng.tiling(),
                         "materials": {"E": layout[0], "H": layout[1]}}
            if prec == "float64":
                ref_out = rec
            else:
                res[prec]["rel_l2_vs_fp64"] = [float((a - b).abs().norm() / b.abs().norm())
                                               for a, b in zip(rec, ref_out)]
            del g, eng, det, rec
            gc.collect()
            torch.cuda.empty_cache()
        out[cfg] = {"workload": desc, "steps": steps, "runs": res,
                    "error_of": "BlockDetector E and H records" if cfg == "c2" else "DFT accumulators",
                    "hbm_peak_gbs": peak}
        del ref_out
        gc.collect()
        torch.cuda.empty_cache()
    fd.set_backend("gb300.float32")
    return out


def gb300_arm(args):
    import torch

    import fdtd_gb300 as fd
    from fdtd_gb300 import scenes

    dist = Dist()
    if torch.cuda.is_available():
        torch.cuda.set_device(dist.local)
    n = args.n
    eps = scenes.c3_permittivity(n, device="cuda")
    precs = [args.only] if args.only else ["float32", "float64", "float32c"]
    res = {}
    for prec in precs:
        sampler = ClockSampler(dist.local) if prec == precs[0] else None
        res[prec] = run_precision(prec, args, dist, fd, scenes, eps, want_halves=prec != "float32c",
                                  want_e2e=prec == precs[0], sampler=sampler)
    del eps
    main = res[precs[0]]
    peak, peak_kind = peaks()
    kern = max(main["half_ms"], key=main["half_ms"].get) if "half_ms" in main else "E"
    t_kern = main["half_ms"][kern] if "half_ms" in main else main["ms_per_step"] / 2
    algo_kern = main["algo_bytes"][kern]
    achieved = algo_kern / (t_kern * 1e-3) / 1e9
    automatic = (args.variant, args.tile_rows, args.stages, args.pml_mode, args.materials, args.x_chunk) == (0,) * 6
    traffic = traffic_from_profile(precs[0], n, kern, json.loads(json.dumps(main["materials"])), automatic)
    line = {
        "metric": METRIC,
        "value": main["gcells"],
        "unit": UNIT,
        "n_gpus": dist.world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": main["ms_per_step"],
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": {"float32": "f32", "float32c": "f32 (compensated)", "float64": "f64"}[precs[0]],
        "data": "synthetic: config-3 generator (seed 3), zero initial fields",
        "config": {
            "workload": f"config3_{n}^3_{precs[0]}",
            "grid": [n, n, n],
            "geometry": "400 random blocks eps in {1,2.25,12.1}, PML y/z, periodic x, centre point source, "
                        "line detector",
            "pml": max(2, int(round(20 * n / 768))) if args.pml < 0 else args.pml,
            "l2": "inputs larger than L2 (fields + materials >= 22 GB at 768^3); no flush",
            "parallelism": "replicas" if dist.world > 1 else "single GPU",
        },
        "roofline": {
            "bound": "hbm",
            "kernel": f"k_update_{kern}{'_tma' if main['tiling']['variant'] == 2 else ''} ({precs[0]}, fused {kern} "
                      "half step incl. its small epilogue kernels)",
            "achieved": achieved,
            "peak": peak,
            "unit": "GB/s",
            "frac": achieved / peak,
            "peak_kind": f"{peak_kind} (STREAM-style copy, MEASURED_PEAKS.json hbm_gbs)",
            "algo_bytes_per_launch": algo_kern,
            "materials": main["materials"],
            "full_array_equivalent_gbs": main["full_bytes_half"] / (t_kern * 1e-3) / 1e9,
            "traffic": traffic,
        },
        "gpu_launches": main["launches_per_step"] * args.steps,
        "clocks": main["clocks"],
        "e2e": main.get("e2e"),
        "tiling": main["tiling"],
    }
    if "float64" in res:
        f64 = res["float64"]
        line["fp64"] = {"value": f64["gcells"], "ms_per_step": f64["ms_per_step"],
                        "hbm_frac": max(f64["algo_bytes"][h] / (f64["half_ms"][h] * 1e-3) / 1e9
                                        for h in ("E", "H")) / peak if "half_ms" in f64 else None,
                        "materials": f64["materials"]}
        if precs[0] == "float32":
            line["fp32_over_fp64"] = main["gcells"] / f64["gcells"]
        ref = f64["trace"]
        errs = {}
        for prec in ("float32", "float32c"):
            if prec in res:
                tr = res[prec]["trace"]
                errs[prec] = float((tr - ref).norm() / ref.norm())
        line["error"] = {"trace_rel_l2_vs_fp64": errs, "records": int(ref.shape[0]),
                         "detector": "line along x through the source"}
        if "trace_long" in f64:
            refl = f64["trace_long"]
            line["error"]["c3"] = {
                "records": int(refl.shape[0]), "detector": "line along x through the source",
                "trace_rel_l2_vs_fp64": {p: float((res[p]["trace_long"] - refl).norm() / refl.norm())
                                         for p in ("float32", "float32c") if "trace_long" in res[p]}}
    if "float32c" in res:
        line["fp32c"] = {"value": res["float32c"]["gcells"], "ms_per_step": res["float32c"]["ms_per_step"]}
    line["nonfinite"] = {p: r["stats"]["nonfinite"] for p, r in res.items()}
    if dist.rank == 0 and not args.skip_configs and args.n == 768:
        line["configs"] = config_runs(fd, scenes)
        if "error" in line:
            for cfg, r in line["configs"].items():
                line["error"][cfg] = {"steps": r["steps"], "of": r["error_of"],
                                      "rel_l2_vs_fp64": {p: r["runs"][p]["rel_l2_vs_fp64"]
                                                         for p in ("float32", "float32c")}}
    if dist.rank == 0 and not args.skip_adjoint:
        line["adjoint"] = adjoint_ratio(fd, scenes, ["c4", "c5"])
    if dist.rank == 0 and not args.skip_cpu:
        line["cpu_baseline"] = cpu_rate("numpy", budget_s=args.cpu_seconds)
        torch_cpu = cpu_rate("torch.float64", budget_s=args.cpu_seconds / 2)
        if torch_cpu is not None:
            line["cpu_baseline_torch"] = torch_cpu
    if dist.rank == 0:
        print(json.dumps(line), flush=True)
    dist.close()


# --------------------------------------------------------------------------
# reference arm: the CPU implementation of the algorithm (numpy oracle port)
# --------------------------------------------------------------------------
def reference_arm(args):
    """The reference's own CPU time step: its numpy backend (the unmodified
    package in baseline/_ref) on the host, one step per step of the contract,
    on the config-3 crop every CPU figure uses.  numpy elementwise runs on one
    core; the reference's torch.float64 CPU backend (all threads) is the
    second CPU figure of the GPU arm's line."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    r = cpu_rate("numpy", steps=args.steps, warmup=args.warmup)
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": r["value"],
        "unit": UNIT,
        "n_gpus": int(os.environ.get("WORLD_SIZE", "1")),
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": r["seconds"] / args.steps * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic: config-3 generator (seed 3), zero initial fields",
        "config": {"workload": f"config3_{args.n}^3_float32", "sample_grid": [CPU_CROP] * 3,
                   "parallelism": "single host process"},
        "cpu_baseline": r,
        "e2e": {"value": r["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def reference_gpu_arm(args):
    """The reference's own GPU path (its torch CUDA backend: one PyTorch
    elementwise kernel per operation, about 490 launches per step) on the same
    config-3 grid, from the unmodified package installed in baseline/_ref
    (with the no-op matplotlib stand-in of tests/golden/mplstub, and of
    tests/golden/tqdmstub where tqdm is not installed).  A comparison
    figure for the GPU arm, not the CPU baseline of the contract."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    ref = reference_module()
    if ref is None:
        print(json.dumps({"impl": "reference-gpu", "unavailable": "reference not installed in baseline/_ref"}))
        return
    import torch

    from fdtd_gb300 import scenes

    ref.set_backend(args.ref_backend)
    n = args.n
    pml = max(2, int(round(20 * n / 768))) if args.pml < 0 else args.pml
    g = scenes.c3(ref, n=n, pml=pml, eps=scenes.c3_permittivity(n), detector=True)
    g.run(args.warmup, progress_bar=False)
    on_gpu = "cuda" in args.ref_backend
    if on_gpu:
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record()
        g.run(args.steps, progress_bar=False)
        ev1.record()
        torch.cuda.synchronize()
        ms = ev0.elapsed_time(ev1)
    else:
        t0 = time.perf_counter()
        g.run(args.steps, progress_bar=False)
        ms = (time.perf_counter() - t0) * 1e3
    print(json.dumps({
        "impl": "reference-gpu", "metric": METRIC, "value": n ** 3 * args.steps / (ms * 1e-3) / 1e9, "unit": UNIT,
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "backend": args.ref_backend, "data": "synthetic: config-3 generator (seed 3)",
        "config": {"workload": f"config3_{n}^3", "grid": [n, n, n], "pml": pml},
        "threads": None if on_gpu else torch.get_num_threads(),
        "peak_memory_gb": torch.cuda.max_memory_allocated() / 1e9 if on_gpu else None}), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        reference_arm(args)
    elif args.impl == "reference-gpu":
        reference_gpu_arm(args)
    elif args.forward_only:
        import torch

        import fdtd_gb300 as fd
        from fdtd_gb300 import scenes

        fd.set_backend("gb300.float32")
        if args.forward_only == "c1":
            g = scenes.c1(fd)
        elif args.forward_only == "c4":
            g = scenes.c4(fd)
        elif args.forward_only == "c2":
            g = scenes.c2(fd, n=208, pml=13) if args.small else scenes.c2(fd)
        else:
            g = scenes.c5(fd, nx=256, ny=256) if args.small else scenes.c5(fd)
        g._ensure_engine().set_tuning(variant=args.variant, tile_rows=args.tile_rows, stages=args.stages,
                                      x_chunk=args.x_chunk, pml_mode=args.pml_mode, materials=args.materials,
                                      step_fusion=args.step_fusion)
        g.run(args.warmup, progress_bar=False)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        g.run(args.steps, progress_bar=False)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / max(1, args.steps)
        print(json.dumps({"forward": args.forward_only, "ms_per_step": ms,
                          "gcells": g.Nx * g.Ny * g.Nz / ms / 1e6, "tiling": g._engine.tiling()}), flush=True)
    elif args.configs_only:
        import fdtd_gb300 as fd
        from fdtd_gb300 import scenes

        print(json.dumps({"configs": config_runs(fd, scenes)}), flush=True)
    elif args.adjoint_only:
        import fdtd_gb300 as fd
        from fdtd_gb300 import scenes

        which = ["c4", "c5"] if args.adjoint_only == "both" else [args.adjoint_only]
        print(json.dumps({"adjoint": adjoint_ratio(fd, scenes, which)}), flush=True)
    else:
        gb300_arm(args)


if __name__ == "__main__":
    main()
