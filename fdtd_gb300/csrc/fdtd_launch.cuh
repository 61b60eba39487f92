// Launch sequence of one fdtd_run call, templated on the precision policy.
#pragma once

#include <cudaTypedefs.h>

#include <type_traits>

#include "fdtd_adjoint.cuh"
#include "fdtd_kernels.cuh"
#include "fdtd_persistent.cuh"
#include "fdtd_plan.hpp"
#include "fdtd_tma.cuh"

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

// One slab kernel: one thread per cell with 32-bit cell indices below 2^31
// cells, else a grid-stride loop with 64-bit indices.
template <class P, bool IS_E, int A>
static void launch_pml_slab_axis(const GridK &g, int slab, long cells, cudaStream_t st) {
    if (cells < (1L << 31)) {
        const unsigned blocks = (unsigned)((cells + kThreads - 1) / kThreads);
        k_pml_slab<P, IS_E, A, uint32_t><<<blocks > 0 ? blocks : 1, kThreads, 0, st>>>(g, slab);
    } else {
        k_pml_slab<P, IS_E, A, uint64_t><<<grid_stride_blocks(cells), kThreads, 0, st>>>(g, slab);
    }
}

template <class P, bool IS_E>
static void launch_pml_slab(const GridK &g, int slab, cudaStream_t st) {
    const SlabK &S = g.slab[slab];
    const long cells = (long)(S.axis == 0 ? S.th : g.nx) * (S.axis == 1 ? S.th : g.ny) * (S.axis == 2 ? S.th : g.nz);
    if (S.axis == 0) launch_pml_slab_axis<P, IS_E, 0>(g, slab, cells, st);
    else if (S.axis == 1) launch_pml_slab_axis<P, IS_E, 1>(g, slab, cells, st);
    else launch_pml_slab_axis<P, IS_E, 2>(g, slab, cells, st);
}

template <class P, int TZ, int TY, int MAT>
static void launch_tma_mat(Plan &p, bool is_E, const double *wave, cudaStream_t st) {
    const dim3 block(TZ, TY, 1);
    const CUtensorMap *m = p.maps;
    if (is_E)
        k_update_E_tma<P, TZ, TY, MAT><<<p.grid, block, p.smem_bytes, st>>>(
            p.kf, wave, m[MAP_H_NBR], m[MAP_E_OWN], m[MAP_IE], m[P::COMP ? MAP_ELO : MAP_E_OWN]);
    else
        k_update_H_tma<P, TZ, TY, MAT><<<p.grid, block, p.smem_bytes, st>>>(
            p.kfH, wave, m[MAP_E_NBR], m[MAP_H_OWN], m[MAP_MU], m[P::COMP ? MAP_HLO : MAP_H_OWN]);
}

template <class P, int TZ, int TY>
static void launch_tma(Plan &p, bool is_E, const double *wave, cudaStream_t st) {
    switch (is_E ? p.kf.mat_E : p.kf.mat_H) {
        case MAT_IDS:
            launch_tma_mat<P, TZ, TY, MAT_IDS>(p, is_E, wave, st);
            break;
        case MAT_UNIFORM:
            launch_tma_mat<P, TZ, TY, MAT_UNIFORM>(p, is_E, wave, st);
            break;
        default:
            launch_tma_mat<P, TZ, TY, MAT_FULL>(p, is_E, wave, st);
    }
}

// Staged-kernel tile shapes (threads along z x rows): 32x8, 32x4, 16x16.
// The fused pass of a half step: one launch over the tile box and, for a
// partitioned plan, one launch over the shell boxes, on the plan's second
// stream (joined before the half step's later stages) when the plan lets the
// two run at the same time (disjoint cells; a half step writes only its own
// field).
template <class P>
static void launch_fused(Plan &p, bool is_E, const double *wave, cudaStream_t st) {
    constexpr int VV = P::V;
    if (p.n_shell && p.shell_overlap) {
        cudaEventRecord(p.shell_fork, st);
        cudaStreamWaitEvent(p.shell_stream, p.shell_fork, 0);
    }
    if (p.variant == 2) {
        if (p.kf.TY == 16) launch_tma<P, 16, 16>(p, is_E, wave, st);
        else if (p.kf.TY == 8) launch_tma<P, 32, 8>(p, is_E, wave, st);
        else launch_tma<P, 32, 4>(p, is_E, wave, st);
    } else if (p.V == 1) {
        if (is_E) k_update_E<P, 1><<<p.grid, p.block, 0, st>>>(p.kf, wave);
        else k_update_H<P, 1><<<p.grid, p.block, 0, st>>>(p.kf, wave);
    } else {
        if (is_E) k_update_E<P, VV><<<p.grid, p.block, 0, st>>>(p.kf, wave);
        else k_update_H<P, VV><<<p.grid, p.block, 0, st>>>(p.kf, wave);
    }
    if (p.n_shell) {
        const unsigned blocks = p.shellk.first[p.shellk.nbox];
        cudaStream_t ss = p.shell_overlap ? p.shell_stream : st;
        constexpr int SV = shell_v<typename P::T>();
        if (is_E) k_shell_E<P, SV><<<blocks, kThreads, 0, ss>>>(p.kshell, p.shellk, wave);
        else k_shell_H<P, SV><<<blocks, kThreads, 0, ss>>>(p.kshell, p.shellk, wave);
        if (p.shell_overlap) {
            cudaEventRecord(p.shell_join, ss);
            cudaStreamWaitEvent(st, p.shell_join, 0);
        }
    }
}

template <class P>
static void launch_epilogue(Plan &p, bool is_E, const double *wave, cudaStream_t st,
                            const typename P::T *iprev = nullptr) {
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
            case EPI_PML: {
                if (is_E) launch_pml_slab<P, true>(g, op.slab, st);
                else launch_pml_slab<P, false>(g, op.slab, st);
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
            case EPI_FEEDBACK: {
                k_feedback<P><<<1, 32, 0, st>>>(g, op.item, wave, iprev, p.grid_spacing);
                break;
            }
        }
    }
}

// --- TMA-staged plan preparation ------------------------------------------
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (fn == nullptr) {
        void *ptr = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(ptr);
    }
    return fn;
}

// 2D view of the one-byte material indices: rows = nx*ny, row = nz bytes;
// box = box_w bytes by box_rows rows.
static bool encode_index_map(CUtensorMap *m, const void *base, const GridK &g, int box_w, int box_rows) {
    PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
    if (enc == nullptr || base == nullptr) return false;
    cuuint64_t dims[2] = {(cuuint64_t)g.nz, (cuuint64_t)g.nx * g.ny};
    cuuint64_t strides[1] = {(cuuint64_t)g.nz};
    cuuint32_t box[2] = {(cuuint32_t)box_w, (cuuint32_t)box_rows};
    cuuint32_t es[2] = {1, 1};
    CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, const_cast<void *>(base), dims, strides, box, es,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

// 2D view of an (nx, ny, nz, 3) field: rows = nx*ny, row = 3*nz values, as
// 8-byte elements; box = box_w elements by box_rows rows.
static bool encode_field_map(CUtensorMap *m, const void *base, const GridK &g, int esize, int box_w, int box_rows) {
    PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
    if (enc == nullptr || base == nullptr) return false;
    cuuint64_t dims[2] = {(cuuint64_t)g.nz * 3 * esize / 8, (cuuint64_t)g.nx * g.ny};
    cuuint64_t strides[1] = {(cuuint64_t)g.nz * 3 * esize};
    cuuint32_t box[2] = {(cuuint32_t)box_w, (cuuint32_t)box_rows};
    cuuint32_t es[2] = {1, 1};
    CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_UINT64, 2, const_cast<void *>(base), dims, strides, box, es,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

// Map of one pass's material tile: the full values, the indices, or none.
template <class P, int TZ, int TY>
static bool encode_material_map(CUtensorMap *m, int mat, const void *full, const void *index, const GridK &g) {
    using G = StageGeom<typename P::T, TZ, TY, P::COMP>;
    if (mat == MAT_FULL) return encode_field_map(m, full, g, (int)sizeof(typename P::T), G::boxO, TY);
    if (mat == MAT_IDS) return encode_index_map(m, index, g, G::boxI, TY);
    return true;
}

template <class P, int TZ, int TY, int MAT>
static cudaError_t allow_smem(bool is_E, size_t bytes) {
    if (is_E)
        return cudaFuncSetAttribute(k_update_E_tma<P, TZ, TY, MAT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)bytes);
    return cudaFuncSetAttribute(k_update_H_tma<P, TZ, TY, MAT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)bytes);
}

template <class P, int TZ, int TY>
static cudaError_t allow_smem_mode(int mat, bool is_E, size_t bytes) {
    if (mat == MAT_IDS) return allow_smem<P, TZ, TY, MAT_IDS>(is_E, bytes);
    if (mat == MAT_UNIFORM) return allow_smem<P, TZ, TY, MAT_UNIFORM>(is_E, bytes);
    return allow_smem<P, TZ, TY, MAT_FULL>(is_E, bytes);
}

template <class P, int TZ, int TY>
static int prepare_tma_rows(Plan &p) {
    using G = StageGeom<typename P::T, TZ, TY, P::COMP>;
    const GridK &g = p.k;
    const int es = (int)sizeof(typename P::T);
    bool ok = encode_field_map(&p.maps[MAP_H_NBR], g.H, g, es, G::boxN, TY + 1) &&
              encode_field_map(&p.maps[MAP_E_NBR], g.E, g, es, G::boxN, TY + 1) &&
              encode_field_map(&p.maps[MAP_E_OWN], g.E, g, es, G::boxO, TY) &&
              encode_field_map(&p.maps[MAP_H_OWN], g.H, g, es, G::boxO, TY) &&
              encode_material_map<P, TZ, TY>(&p.maps[MAP_IE], g.mat_E, g.ie, p.index_E, g) &&
              encode_material_map<P, TZ, TY>(&p.maps[MAP_MU], g.mat_H, g.imu, p.index_H, g);
    if (ok && P::COMP)
        ok = encode_field_map(&p.maps[MAP_ELO], g.Elo, g, es, G::boxO, TY) &&
             encode_field_map(&p.maps[MAP_HLO], g.Hlo, g, es, G::boxO, TY);
    if (!ok) return FDTD_ERR_UNSUPPORTED;
    p.smem_bytes = (size_t)g.stages * g.stage_bytes + (size_t)g.stages * 8 +
                   ((size_t)g.coef_values + 4 * (size_t)g.lut_rows) * sizeof(typename P::T) + 16 + 128;
    cudaError_t e = allow_smem_mode<P, TZ, TY>(g.mat_E, true, p.smem_bytes);
    if (e == cudaSuccess) e = allow_smem_mode<P, TZ, TY>(g.mat_H, false, p.smem_bytes);
    if (e != cudaSuccess) {
        set_last_cuda_error((int)e);
        return FDTD_ERR_CUDA;
    }
    return FDTD_OK;
}

template <class P>
static int prepare_tma_impl(Plan &p) {
    if (p.k.TY == 16) return prepare_tma_rows<P, 16, 16>(p);
    return p.k.TY == 8 ? prepare_tma_rows<P, 32, 8>(p) : prepare_tma_rows<P, 32, 4>(p);
}

template <class P, int TZ, int TY>
static size_t stage_bytes_mode(int mat) {
    using T = typename P::T;
    if (mat == MAT_IDS) return (size_t)StageGeom<T, TZ, TY, P::COMP, MAT_IDS>::stageBytes;
    if (mat == MAT_UNIFORM) return (size_t)StageGeom<T, TZ, TY, P::COMP, MAT_UNIFORM>::stageBytes;
    return (size_t)StageGeom<T, TZ, TY, P::COMP, MAT_FULL>::stageBytes;
}

template <class P>
static size_t stage_bytes_of(int tile_rows, int mat_E, int mat_H) {
    size_t a, b;
    if (tile_rows == 16) {
        a = stage_bytes_mode<P, 16, 16>(mat_E);
        b = stage_bytes_mode<P, 16, 16>(mat_H);
    } else if (tile_rows == 8) {
        a = stage_bytes_mode<P, 32, 8>(mat_E);
        b = stage_bytes_mode<P, 32, 8>(mat_H);
    } else {
        a = stage_bytes_mode<P, 32, 4>(mat_E);
        b = stage_bytes_mode<P, 32, 4>(mat_H);
    }
    return a > b ? a : b;
}

// All steps of a call in one cooperative launch (fdtd_persistent.cuh).
template <class P>
static int run_persistent(Plan &p, const fdtd_run_args *a, bool detect, cudaStream_t st) {
    PersistArgs pa{};
    pa.n_steps = a->n_steps;
    pa.wave = a->wave;
    pa.n_columns = p.n_columns;
    pa.gz = (int)p.grid.x;
    pa.gy = (int)p.grid.y;
    pa.gx = (int)p.grid.z;
    pa.n_probe = detect ? p.n_probe : 0;
    pa.probe_cells = p.probe_cells;
    if (pa.n_probe) {
        pa.trace_E = (typename P::T *)a->trace_E + a->record_E * 3 * p.n_probe;
        pa.trace_H = (typename P::T *)a->trace_H + a->record_H * 3 * p.n_probe;
    }
    pa.phase = a->phase;
    pa.n_phase_columns = p.n_phase_columns;
    pa.n_dft = detect ? (int)p.dft.size() : 0;
    for (int q = 0; q < pa.n_dft; ++q) pa.dft[q] = p.dft[q];
    pa.barrier = p.persist_bar;
    pa.tickets = p.persist_tickets;
    pa.order = p.persist_order;
    pa.limit = 1u << 23;
    const bool vec = p.V > 1;
    const void *fn = vec ? (const void *)k_run_persistent<P, P::V> : (const void *)k_run_persistent<P, 1>;
    if (p.persist_blocks == 0) {
        int per_sm = 0, dev = 0, n_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
        cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kThreads, 0);
        if (e != cudaSuccess || per_sm < 1) {
            set_last_cuda_error((int)e);
            return FDTD_ERR_CUDA;
        }
        p.persist_blocks = per_sm * n_sm;
    }
    const int tiles = (int)(p.grid.x * p.grid.y * p.grid.z);
    const int blocks = std::min(tiles, p.persist_blocks);
    // the barrier counter and, 8 bytes on, the ticket counter
    cudaError_t e = cudaMemsetAsync(p.persist_bar, 0, 16, st);
    if (e == cudaSuccess) {
        GridK gk = p.kf;
        void *args[] = {&gk, &pa};
        e = cudaLaunchCooperativeKernel(fn, dim3(blocks), p.block, args, 0, st);
    }
    if (e != cudaSuccess) {
        set_last_cuda_error((int)e);
        return FDTD_ERR_CUDA;
    }
    return FDTD_OK;
}

// n_steps full steps (or one half step).  With capture arguments: detectors
// and DFTs only when cap->detectors is set, and curl_H on every object box
// with a capture pointer before each E half (reverse-time adjoint).
template <class P>
static int run_impl(Plan &p, const fdtd_run_args *a, const fdtd_capture_args *cap, cudaStream_t st) {
    using T = typename P::T;
    if (a->n_steps < 0 || (a->half != 0 && a->n_steps != 1) || a->half < 0 || a->half > 2)
        return FDTD_ERR_ARGUMENT;
    if (cap != nullptr) {
        if (a->half != 0 || (cap->n_curl != 0 && cap->n_curl != p.n_objects) ||
            (cap->n_curl != 0 && cap->curl == nullptr))
            return FDTD_ERR_ARGUMENT;
    }
    const bool detect = cap == nullptr || cap->detectors != 0;
    if (p.n_columns > 0 && a->wave == nullptr && a->n_steps > 0) return FDTD_ERR_ARGUMENT;
    if (detect && !p.dft.empty() && a->phase == nullptr && a->n_steps > 0 && a->half != 2)
        return FDTD_ERR_ARGUMENT;
    const bool probe = detect && p.n_probe > 0;
    if (!detect && p.has_feedback) return FDTD_ERR_UNSUPPORTED;  // the currents drive the sources
    const bool current = detect && p.n_current > 0;
    if (current && (a->trace_I == nullptr || a->record_I < 0 ||
                    (a->half != 1 && a->record_I + a->n_steps > a->trace_capacity)))
        return FDTD_ERR_RANGE;
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
    // small plans: every full step of the call in one cooperative launch
    if (p.persistent && a->half == 0 && cap == nullptr && a->n_steps >= 2)
        return run_persistent<P>(p, a, detect, st);
    // one pass per full step (float32 plans that have it), in pairs: the first
    // pass of a pair writes the alternate buffers, the second the caller's; an
    // odd last step runs the two passes
    int64_t nfused = 0;
    if constexpr (std::is_same<P, PF32>::value) {
        if (p.onepass && a->half == 0 && cap == nullptr) nfused = a->n_steps & ~(int64_t)1;
    }
    for (int64_t s = 0; s < a->n_steps; ++s) {
        const double *wave = p.n_columns > 0 ? a->wave + s * p.n_columns : nullptr;
        if (s < nfused) {
            const int dir = (int)(s & 1);
            const GridK &ko = p.ko[dir];
            onepass_step_f32(p, dir, wave, st);
            if (probe) {
                k_probe<T><<<pblocks, kThreads, 0, st>>>((const T *)ko.E, p.probe_cells, p.n_probe,
                                                        (T *)a->trace_E + (a->record_E + s) * 3 * p.n_probe);
                k_probe<T><<<pblocks, kThreads, 0, st>>>((const T *)ko.H, p.probe_cells, p.n_probe,
                                                        (T *)a->trace_H + (a->record_H + s) * 3 * p.n_probe);
            }
            for (const fdtd_dft_desc &d : p.dft) {
                const long cells = (long)(d.hi[0] - d.lo[0]) * (d.hi[1] - d.lo[1]) * (d.hi[2] - d.lo[2]);
                k_dft<T, P::COMP><<<grid_stride_blocks(cells * 3), kThreads, 0, st>>>(
                    (const T *)ko.E, (const T *)g.Elo, g.ny, g.nz, d, a->phase + s * 2 * p.n_phase_columns);
            }
            if (current)
                k_current<T><<<(p.n_current + kThreads - 1) / kThreads, kThreads, 0, st>>>(
                    (const T *)ko.H, p.current_cells, p.n_current, g.nx, g.ny, g.nz, p.grid_spacing,
                    (T *)a->trace_I + (a->record_I + s) * p.n_current);
            const int rc = check_launch<P>();
            if (rc != FDTD_OK) return rc;
            continue;
        }
        if (cap != nullptr) {
            for (int q = 0; q < cap->n_curl; ++q) {
                if (cap->curl[q] == nullptr) continue;
                const ItemK &o = p.items_host[q];
                const long cells = (long)(o.hi[0] - o.lo[0]) * (o.hi[1] - o.lo[1]) * (o.hi[2] - o.lo[2]);
                k_capture_curl<T><<<grid_stride_blocks(cells), kThreads, 0, st>>>(g, q, (T *)cap->curl[q] +
                                                                                          s * 3 * cells);
            }
        }
        if (a->half != 2) {
            // the current of the previous H half, for feedback sources
            const T *iprev = nullptr;
            if (current && a->step0 + s > 0 && a->record_I + s - 1 >= 0)
                iprev = (const T *)a->trace_I + (a->record_I + s - 1) * p.n_current;
            launch_fused<P>(p, true, wave, st);
            launch_epilogue<P>(p, true, wave, st, iprev);
            if (probe)
                k_probe<T><<<pblocks, kThreads, 0, st>>>((const T *)g.E, p.probe_cells, p.n_probe,
                                                        (T *)a->trace_E + (a->record_E + s) * 3 * p.n_probe);
            if (detect) {
                for (const fdtd_dft_desc &d : p.dft) {
                    const long cells = (long)(d.hi[0] - d.lo[0]) * (d.hi[1] - d.lo[1]) * (d.hi[2] - d.lo[2]);
                    k_dft<T, P::COMP><<<grid_stride_blocks(cells * 3), kThreads, 0, st>>>(
                        (const T *)g.E, (const T *)g.Elo, g.ny, g.nz, d, a->phase + s * 2 * p.n_phase_columns);
                }
            }
        }
        if (a->half != 1) {
            launch_fused<P>(p, false, wave, st);
            launch_epilogue<P>(p, false, wave, st);
            if (probe)
                k_probe<T><<<pblocks, kThreads, 0, st>>>((const T *)g.H, p.probe_cells, p.n_probe,
                                                        (T *)a->trace_H + (a->record_H + s) * 3 * p.n_probe);
            if (current)
                k_current<T><<<(p.n_current + kThreads - 1) / kThreads, kThreads, 0, st>>>(
                    (const T *)g.H, p.current_cells, p.n_current, g.nx, g.ny, g.nz, p.grid_spacing,
                    (T *)a->trace_I + (a->record_I + s) * p.n_current);
        }
        const int rc = check_launch<P>();
        if (rc != FDTD_OK) return rc;
    }
    return FDTD_OK;
}

}  // namespace fdtd
