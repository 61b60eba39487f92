"""Multi-rank paths on CPU ranks (torch.distributed, gloo, 127.0.0.1).

* the replica helper of bench.py (barrier, max over ranks) at world size 2;
* the x-slab decomposition of the time step (oracle/fdtd_decomposition.py):
  a scene split over 2-4 ranks with one ghost plane per half step and the
  periodic wrap as a message gives the same bits as the single-process run.
"""

import os
import socket
import tempfile

import numpy as np
import pytest
import torch.multiprocessing as mp

import golden_scenes
from oracle import fdtd_decomposition as fdec
from oracle import fdtd_oracle as fo

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _dist_worker(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import sys

    sys.path.insert(0, ROOT)
    import bench

    d = bench.Dist()
    d.barrier()
    v = d.max(float(rank) + 1.5)
    with open(os.path.join(out_dir, f"rank{rank}.txt"), "w") as f:
        f.write(f"{d.world} {d.rank} {v}\n")
    d.close()


def test_replica_helper_two_ranks():
    with tempfile.TemporaryDirectory() as tmp:
        mp.spawn(_dist_worker, args=(2, _free_port(), tmp), nprocs=2, join=True)
        rows = [open(os.path.join(tmp, f"rank{r}.txt")).read().split() for r in range(2)]
    for r, (world, rank, v) in enumerate(rows):
        assert int(world) == 2 and int(rank) == r and float(v) == 2.5


@pytest.mark.parametrize("builder, world, steps", [
    ("g_c3_periodic_first", 2, 25),  # periodic x registered before the y/z PMLs
    ("g_c3_periodic_last", 3, 25),   # ... and after them, middle rank present
    ("g_mix", 4, 20),                # x PML slab spanning two ranks, objects, every source kind
])
def test_x_slab_decomposition_matches_single_process(builder, world, steps):
    grid, _, _ = getattr(golden_scenes, builder)(fo)
    for _ in range(steps):
        grid.step()
    with tempfile.TemporaryDirectory() as tmp:
        out = os.path.join(tmp, "split.npz")
        mp.spawn(fdec.split_worker, args=(world, _free_port(), builder, steps, out), nprocs=world, join=True)
        got = np.load(out)
        assert np.array_equal(got["E"], grid.E)
        assert np.array_equal(got["H"], grid.H)


def test_partition_covers_the_axis():
    for n, w in ((16, 2), (14, 4), (7, 3), (5, 5)):
        parts = fdec.partition(n, w)
        assert parts[0][0] == 0 and parts[-1][1] == n
        assert all(a < b for a, b in parts) and all(p[1] == q[0] for p, q in zip(parts, parts[1:]))
