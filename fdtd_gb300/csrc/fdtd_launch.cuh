// Launch sequence of one fdtd_run call, templated on the precision policy.
#pragma once

#include "fdtd_kernels.cuh"
#include "fdtd_plan.hpp"

namespace fdtd {

template <class P>
static int check_launch() {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_last_cuda_error((int)e);
        return FDTD_ERR_CUDA;
    }
    return FDTD_OK;
}

template <class P>
static void launch_fused(Plan &p, bool is_E, const double *wave, cudaStream_t st) {
    constexpr int VV = P::V;
    if (p.V == 1) {
        if (is_E) k_update_E<P, 1><<<p.grid, p.block, 0, st>>>(p.k, wave);
        else k_update_H<P, 1><<<p.grid, p.block, 0, st>>>(p.k, wave);
    } else {
        if (is_E) k_update_E<P, VV><<<p.grid, p.block, 0, st>>>(p.k, wave);
        else k_update_H<P, VV><<<p.grid, p.block, 0, st>>>(p.k, wave);
    }
}

template <class P>
static void launch_epilogue(Plan &p, bool is_E, const double *wave, cudaStream_t st) {
    using T = typename P::T;
    const std::vector<EpiOp> &ops = is_E ? p.epi_E : p.epi_H;
    const GridK &g = p.k;
    for (const EpiOp &op : ops) {
        switch (op.kind) {
            case EPI_COPY: {
                const int n = op.axis == 0 ? g.nx : (op.axis == 1 ? g.ny : g.nz);
                const int n1 = op.axis == 0 ? g.ny : g.nx, n2 = op.axis == 2 ? g.ny : g.nz;
                const int blocks = grid_stride_blocks((long)n1 * n2 * 3);
                T *F = (T *)(is_E ? g.E : g.H);
                T *Flo = (T *)(is_E ? g.Elo : g.Hlo);
                const int dst = is_E ? 0 : n - 1, src = is_E ? n - 1 : 0;
                k_plane_copy<T, P::COMP><<<blocks, kThreads, 0, st>>>(F, Flo, g.nx, g.ny, g.nz, op.axis, dst, src);
                break;
            }
            case EPI_SLAB: {
                const SlabK &S = g.slab[op.slab];
                const long cells = (long)(S.axis == 0 ? S.th : g.nx) * (S.axis == 1 ? S.th : g.ny) *
                                   (S.axis == 2 ? S.th : g.nz);
                if (is_E) k_slab_correct<P, true><<<grid_stride_blocks(cells), kThreads, 0, st>>>(g, op.slab);
                else k_slab_correct<P, false><<<grid_stride_blocks(cells), kThreads, 0, st>>>(g, op.slab);
                break;
            }
            case EPI_SOFT: {
                const int blocks = (op.run_count + kThreads - 1) / kThreads;
                k_soft_runs<P><<<blocks, kThreads, 0, st>>>(g, p.runs + op.run_begin, op.run_count, wave,
                                                             is_E ? 0 : 1);
                break;
            }
            case EPI_HARD: {
                k_hard_box<P><<<grid_stride_blocks(1L << 20), kThreads, 0, st>>>(g, op.item, wave, is_E ? 0 : 1);
                break;
            }
        }
    }
}

template <class P>
static int run_impl(Plan &p, const fdtd_run_args *a, cudaStream_t st) {
    using T = typename P::T;
    if (a->n_steps < 0 || (a->half != 0 && a->n_steps != 1) || a->half < 0 || a->half > 2)
        return FDTD_ERR_ARGUMENT;
    if (p.n_columns > 0 && a->wave == nullptr && a->n_steps > 0) return FDTD_ERR_ARGUMENT;
    if (!p.dft.empty() && a->phase == nullptr && a->n_steps > 0 && a->half != 2) return FDTD_ERR_ARGUMENT;
    const bool probe = p.n_probe > 0;
    if (probe) {
        if (a->half != 2 && (a->trace_E == nullptr || a->record_E < 0 ||
                             a->record_E + a->n_steps > a->trace_capacity))
            return FDTD_ERR_RANGE;
        if (a->half != 1 && (a->trace_H == nullptr || a->record_H < 0 ||
                             a->record_H + a->n_steps > a->trace_capacity))
            return FDTD_ERR_RANGE;
    }
    const GridK &g = p.k;
    const int pblocks = (3 * p.n_probe + kThreads - 1) / kThreads;
    for (int64_t s = 0; s < a->n_steps; ++s) {
        const double *wave = p.n_columns > 0 ? a->wave + s * p.n_columns : nullptr;
        if (a->half != 2) {
            launch_fused<P>(p, true, wave, st);
            launch_epilogue<P>(p, true, wave, st);
            if (probe)
                k_probe<T><<<pblocks, kThreads, 0, st>>>((const T *)g.E, p.probe_cells, p.n_probe,
                                                        (T *)a->trace_E + (a->record_E + s) * 3 * p.n_probe);
            for (const fdtd_dft_desc &d : p.dft) {
                const long cells = (long)(d.hi[0] - d.lo[0]) * (d.hi[1] - d.lo[1]) * (d.hi[2] - d.lo[2]);
                k_dft<T, P::COMP><<<grid_stride_blocks(cells * 3), kThreads, 0, st>>>(
                    (const T *)g.E, (const T *)g.Elo, g.ny, g.nz, d, a->phase + s * 2 * p.n_phase_columns);
            }
        }
        if (a->half != 1) {
            launch_fused<P>(p, false, wave, st);
            launch_epilogue<P>(p, false, wave, st);
            if (probe)
                k_probe<T><<<pblocks, kThreads, 0, st>>>((const T *)g.H, p.probe_cells, p.n_probe,
                                                        (T *)a->trace_H + (a->record_H + s) * 3 * p.n_probe);
        }
        const int rc = check_launch<P>();
        if (rc != FDTD_OK) return rc;
    }
    return FDTD_OK;
}

}  // namespace fdtd
