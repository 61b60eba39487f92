"""x-slab decomposition of the fdtd time step over ranks, on the CPU oracle.

TEST INFRASTRUCTURE ONLY.  Only ``tests/`` may import this module.  The GPU
product runs one grid per GPU (replicas); this module checks on CPU ranks
(torch.distributed, gloo) the exchange schedule that splitting one grid over
several GPUs would need, using the oracle's stages as the per-rank step.

Each rank holds the whole grid (built by the same scene builder, so every
component exists on every rank) and owns the planes [x0, x1) of a contiguous
partition along x.  The stencils of fdtd/grid.py:29-76 and the PML
auxiliaries of fdtd/boundaries.py:433-487 reach one plane along x, so per half
step a rank needs one ghost plane from one neighbour:

* before the E half: H[x0-1] from the left neighbour (backward differences);
* before the H half: E[x1] from the right neighbour (forward differences);

and a periodic x boundary (fdtd/boundaries.py:184-219) becomes a message
between the first and the last rank at its place in the boundary order
(E[0] = E[N-1]: last -> first; H[N-1] = H[0]: first -> last).  After every
half step a rank overwrites the planes it does not own with NaN, so its owned
planes can only stay finite (and equal to the single-process run) if every
value they read came from its own planes or from a message.  Objects, sources
and detectors act cell by cell and need no exchange.
"""

import os

import numpy as np
import torch
import torch.distributed as dist

from oracle import fdtd_oracle as fo


def partition(n, world):
    """Contiguous x ranges [x0, x1) of the ranks."""
    return [(n * r // world, n * (r + 1) // world) for r in range(world)]


class SplitStepper:
    """Steps an oracle grid as rank ``rank`` of ``world`` (process group initialised)."""

    def __init__(self, grid, rank, world):
        self.g, self.rank, self.world = grid, rank, world
        self.x0, self.x1 = partition(grid.Nx, world)[rank]
        for b in grid.boundaries:
            if isinstance(b, fo.PeriodicBoundary) and b.axis == 0 and world > 1:
                b.correct_E = self._periodic_E
                b.correct_H = self._periodic_H

    @staticmethod
    def _send(arr, dst):
        dist.send(torch.from_numpy(np.ascontiguousarray(arr)), dst)

    @staticmethod
    def _recv(like, src):
        t = torch.empty(like.shape, dtype=torch.float64)
        dist.recv(t, src)
        return t.numpy()

    def _periodic_E(self):
        g, last = self.g, self.world - 1
        if self.rank == last:
            self._send(g.E[-1], 0)
        if self.rank == 0:
            g.E[0] = self._recv(g.E[0], last)

    def _periodic_H(self):
        g, last = self.g, self.world - 1
        if self.rank == 0:
            self._send(g.H[0], last)
        if self.rank == last:
            g.H[-1] = self._recv(g.H[-1], 0)

    def _halo_before_E(self):
        g = self.g
        if self.rank < self.world - 1:
            self._send(g.H[self.x1 - 1], self.rank + 1)
        if self.rank > 0:
            g.H[self.x0 - 1] = self._recv(g.H[0], self.rank - 1)

    def _halo_before_H(self):
        g = self.g
        if self.rank > 0:
            self._send(g.E[self.x0], self.rank - 1)
        if self.rank < self.world - 1:
            g.E[self.x1] = self._recv(g.E[0], self.rank + 1)

    def _poison(self, arr):
        arr[:self.x0] = np.nan
        arr[self.x1:] = np.nan

    def step(self):
        if self.world > 1:
            self._halo_before_E()
        self.g.update_E()
        if self.world > 1:
            self._poison(self.g.E)
            self._halo_before_H()
        self.g.update_H()
        if self.world > 1:
            self._poison(self.g.H)
        self.g.time_steps_passed += 1

    def gather(self, field):
        """The owned planes of every rank, assembled on rank 0 (None elsewhere)."""
        arr = self.g.E if field == "E" else self.g.H
        if self.rank != 0:
            self._send(arr[self.x0:self.x1], 0)
            return None
        out = arr.copy()
        for r, (a, b) in enumerate(partition(self.g.Nx, self.world)):
            if r:
                out[a:b] = self._recv(arr[a:b], r)
        return out


def split_worker(rank, world, port, builder_name, steps, out_path):
    """Entry point of one rank (torch.multiprocessing.spawn): run a scene of
    ``tests/golden/golden_scenes.py`` split over ``world`` ranks and save the
    gathered fields on rank 0."""
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import golden_scenes

        grid, _, _ = getattr(golden_scenes, builder_name)(fo)
        st = SplitStepper(grid, rank, world)
        st._poison(grid.E)
        st._poison(grid.H)
        for _ in range(steps):
            st.step()
        E, H = st.gather("E"), st.gather("H")
        if rank == 0:
            np.savez(out_path, E=E, H=H)
    finally:
        dist.destroy_process_group()
