// Persistent time loop for small grids: all steps of one fdtd_run call in a
// single cooperative launch.
//
// A grid of a few million cells takes tens of microseconds per half step, so
// a run of two launches per step (plus detector gathers) is bound by launch
// latency and by the partly filled last wave of each launch rather than by
// memory.  Here the blocks share out the register-streaming tiles of a
// half step (tile_update_E / tile_update_H, the same per-cell arithmetic as
// the one-launch-per-half-step plan, so the same bits), then all blocks meet
// at a grid-wide barrier before the other half step.  Detector gathers and
// DFT accumulation of a half step run after its barrier, interleaved with the
// next half step (which never writes the field they read).
//
// Fields the other half step wrote are read with L2-only loads (the
// read-only path may keep lines in L1 across the barrier).
//
// The launch is cooperative (all blocks resident at once, so the barrier
// cannot wait for a block that never runs).  Barrier waits are bounded: a
// block that gives up sets bit 2 of the plan's status word and returns, and
// so do the others when their own waits expire; the context stays usable.
#pragma once

#include "fdtd_kernels.cuh"

namespace fdtd {

constexpr int kPersistMaxDft = 4;

// Everything the persistent loop needs besides the GridK.
struct PersistArgs {
    long long n_steps;
    const double *wave;
    int n_columns;
    int gz, gy, gx;  // register-streaming tile grid
    int n_probe;
    const int64_t *probe_cells;
    void *trace_E, *trace_H;  // first rows of this call
    const double *phase;      // [n_steps][n_phase_columns][2]
    int n_phase_columns;
    int n_dft;
    fdtd_dft_desc dft[kPersistMaxDft];
    unsigned *barrier;                // arrival counter, zero at launch
    unsigned long long *tickets;      // tile tickets drawn, zero at launch
    const int *order;                 // tile of each ticket, heaviest first (null: grid order)
    unsigned limit;                   // polls before a barrier wait gives up
};

// Grid-wide barrier number `epoch` (1, 2, ...): the counter counts every
// arrival, and barrier k is complete once it reaches k * gridDim.x.  Returns
// false on expiry (after recording it in *status).
__device__ __forceinline__ bool grid_barrier(unsigned *counter, unsigned epoch, unsigned limit, int *status) {
    __shared__ int ok_s;
    __syncthreads();
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        __threadfence();  // this block's writes before the arrival
        atomicAdd(counter, 1u);
        const unsigned target = epoch * gridDim.x;
        int ok = 0;
        for (unsigned it = 0; it < limit; ++it) {
            unsigned v;
            asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(counter) : "memory");
            if ((int)(v - target) >= 0) {
                ok = 1;
                break;
            }
            __nanosleep(64);
        }
        if (!ok) atomicOr(status, 4);
        __threadfence();
        ok_s = ok;
    }
    __syncthreads();
    return ok_s != 0;
}

template <class T, bool COMP>
__device__ __forceinline__ void persist_dft(const GridK &g, const fdtd_dft_desc &d, const double *phase, long tid,
                                            long nthr) {
    const int b0 = d.hi[0] - d.lo[0], b1 = d.hi[1] - d.lo[1], b2 = d.hi[2] - d.lo[2];
    const long ncell = (long)b0 * b1 * b2;
    const T *E = (const T *)g.E;
    const T *Elo = (const T *)g.Elo;
    for (long t = tid; t < ncell * 3; t += nthr) {
        const long cell = t / 3;
        const int comp = (int)(t % 3);
        const int i = d.lo[0] + (int)(cell / ((long)b1 * b2)), j = d.lo[1] + (int)((cell / b2) % b1),
                  k = d.lo[2] + (int)(cell % b2);
        const size_t at = 3 * (((size_t)i * g.ny + j) * g.nz + k) + comp;
        double e = (double)E[at];
        if constexpr (COMP) e = e + (double)Elo[at];
        for (int f = 0; f < d.n_freq; ++f) {
            const double cs = phase[2 * (d.phase_offset + f)], sn = phase[2 * (d.phase_offset + f) + 1];
            double *acc = d.acc + 2 * ((size_t)f * ncell * 3 + t);
            acc[0] = __dadd_rn(acc[0], __dmul_rn(e, cs));
            acc[1] = __dadd_rn(acc[1], __dmul_rn(e, sn));
        }
    }
}

// The tiles of one half step: each block's first tile is its own (the
// heaviest tiles go to the first blocks), the rest are handed out by ticket:
// a block draws tickets from one counter until it draws one past the last
// tile, so a block that got light tiles takes more of them and the half step
// ends with no block left holding a queue of its own.  Each block draws
// exactly one ticket past the end, so half step h owns tickets [h ntiles,
// (h + 1) ntiles) and the counter never needs resetting.  A block draws its
// next ticket before its current tile runs, hiding the atomic's latency.
// With no more tiles than blocks nothing is drawn.
template <bool IS_E, class P, int V>
__device__ __forceinline__ void persist_half(const GridK &g, const PersistArgs &a, const double *wave, int ntiles,
                                             unsigned long long base) {
    __shared__ int ticket_s;
    const bool lead = threadIdx.x == 0 && threadIdx.y == 0;
    const int nblk = (int)gridDim.x;
    const bool draw = ntiles > nblk;
    int t = blockIdx.x;
    while (t < ntiles) {
        unsigned long long next = 0;
        if (lead && draw) next = atomicAdd(a.tickets, 1ull);
        const int tile = a.order ? a.order[t] : t;
        const int bx = tile % a.gz, by = (tile / a.gz) % a.gy, bz = tile / (a.gz * a.gy);
        if constexpr (IS_E) tile_update_E<P, V, true>(g, wave, bx, by, bz, tile);
        else tile_update_H<P, V, true>(g, wave, bx, by, bz, tile);
        if (!draw) break;
        __syncthreads();  // every thread has read ticket_s
        if (lead) ticket_s = nblk + (int)(next - base);
        __syncthreads();
        t = ticket_s;
    }
}

template <class P, int V>
__global__ void __launch_bounds__(kThreads) k_run_persistent(const GridK g, const PersistArgs a) {
    using T = typename P::T;
    const int ntiles = a.gz * a.gy * a.gx;
    const long nthr = (long)gridDim.x * kThreads;
    const long tid = (long)blockIdx.x * kThreads + threadIdx.y * blockDim.x + threadIdx.x;
    const unsigned long long per_half = ntiles > (int)gridDim.x ? (unsigned long long)ntiles : 0ull;
    unsigned long long base = 0;
    unsigned epoch = 0;
    for (long long s = 0; s < a.n_steps; ++s) {
        const double *wave = a.n_columns > 0 ? a.wave + s * a.n_columns : nullptr;
        persist_half<true, P, V>(g, a, wave, ntiles, base);
        base += per_half;
        if (!grid_barrier(a.barrier, ++epoch, a.limit, g.status)) return;
        // E is final for this step: gathers and DFT overlap the H half
        if (a.n_probe) {
            T *out = (T *)a.trace_E + s * 3 * a.n_probe;
            for (long q = tid; q < 3L * a.n_probe; q += nthr) out[q] = ((const T *)g.E)[3 * a.probe_cells[q / 3] + q % 3];
        }
        for (int d = 0; d < a.n_dft; ++d)
            persist_dft<T, P::COMP>(g, a.dft[d], a.phase + s * 2 * a.n_phase_columns, tid, nthr);
        persist_half<false, P, V>(g, a, wave, ntiles, base);
        base += per_half;
        if (!grid_barrier(a.barrier, ++epoch, a.limit, g.status)) return;
        if (a.n_probe) {
            T *out = (T *)a.trace_H + s * 3 * a.n_probe;
            for (long q = tid; q < 3L * a.n_probe; q += nthr) out[q] = ((const T *)g.H)[3 * a.probe_cells[q / 3] + q % 3];
        }
    }
}

}  // namespace fdtd
