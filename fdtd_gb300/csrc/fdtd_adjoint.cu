// Launch sequence of the reverse-time adjoint (fdtd_adjoint_run), float32 and
// float64 instantiations.
#include "fdtd_adjoint.cuh"
#include "fdtd_adjoint_tma.cuh"
#include "fdtd_launch.cuh"
#include "fdtd_plan.hpp"

namespace fdtd {

// ---- TMA-staged transposed passes (fdtd_adjoint_tma.cuh) -------------------
// Used by plans whose forward passes are TMA-staged with the PML slabs in
// kernels of their own; they reuse the forward tiling, launch order and
// material copies.  Tensor maps of the adjoint fields are encoded per call
// (the caller's buffers), those of the materials' neighbour footprints too
// (a few host calls per fdtd_adjoint_run).

static int optin_smem() {
    static int v = 0;
    if (v == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    }
    return v;
}

template <class T, int TZ, int TY, int MAT>
static int adj_staged_launch(const Plan &p, const GridK &g0, bool is_H, cudaStream_t st) {
    using G = AdjGeom<T, TZ, TY, MAT>;
    const int esz = (int)sizeof(T);
    GridK g = g0;
    g.stage_bytes = G::stageBytes;
    // ring depth: two CTAs per SM with at least three stages where that fits
    const size_t extra = 16 + 4 * 256 * (size_t)esz + 128;
    auto smem_of = [&](int S) { return (size_t)S * (G::stageBytes + 8) + extra; };
    int S = 0;
    for (int q = 6; q >= 3 && S == 0; --q)
        if ((long)smem_of(q) + 1024 <= 114L * 1024 && smem_of(q) <= (size_t)optin_smem()) S = q;
    for (int q = 6; q >= 2 && S == 0; --q)
        if (smem_of(q) <= (size_t)optin_smem()) S = q;
    if (S == 0) return FDTD_ERR_UNSUPPORTED;
    g.stages = S;
    const size_t smem = smem_of(S);
    // neighbour tile of the field read, its material footprint, own tile of the field updated
    CUtensorMap mN, mM, mO;
    const void *read = is_H ? g.H : g.E, *upd = is_H ? g.E : g.H;
    bool ok = encode_field_map(&mN, read, g, esz, G::boxN, TY + 1) && encode_field_map(&mO, upd, g, esz, G::boxO, TY);
    const int mat = is_H ? g.mat_H : g.mat_E;
    if (mat == MAT_FULL) ok = ok && encode_field_map(&mM, is_H ? g.imu : g.ie, g, esz, G::boxN, TY + 1);
    else if (mat == MAT_IDS) ok = ok && encode_index_map(&mM, is_H ? p.index_H : p.index_E, g, G::idxN, TY + 1);
    else mM = mN;
    if (!ok) return FDTD_ERR_UNSUPPORTED;
    const dim3 block(TZ, TY, 1);
    cudaError_t e;
    if (is_H) {
        e = cudaFuncSetAttribute(k_adj_H_tma<T, TZ, TY, MAT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e == cudaSuccess) k_adj_H_tma<T, TZ, TY, MAT><<<p.grid, block, smem, st>>>(g, mN, mM, mO);
    } else {
        e = cudaFuncSetAttribute(k_adj_E_tma<T, TZ, TY, MAT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e == cudaSuccess) k_adj_E_tma<T, TZ, TY, MAT><<<p.grid, block, smem, st>>>(g, mN, mM, mO);
    }
    if (e != cudaSuccess) {
        set_last_cuda_error((int)e);
        return FDTD_ERR_CUDA;
    }
    return FDTD_OK;
}

template <class T, int TZ, int TY>
static int adj_staged_mat(const Plan &p, const GridK &g, bool is_H, cudaStream_t st) {
    switch (is_H ? g.mat_H : g.mat_E) {
        case MAT_IDS:
            return adj_staged_launch<T, TZ, TY, MAT_IDS>(p, g, is_H, st);
        case MAT_UNIFORM:
            return adj_staged_launch<T, TZ, TY, MAT_UNIFORM>(p, g, is_H, st);
        default:
            return adj_staged_launch<T, TZ, TY, MAT_FULL>(p, g, is_H, st);
    }
}

// One transposed bulk pass of a staged plan (the forward passes' tile shape).
template <class T>
static int adj_staged(const Plan &p, const GridK &g, bool is_H, cudaStream_t st) {
    if (p.k.TY == 16) return adj_staged_mat<T, 16, 16>(p, g, is_H, st);
    if (p.k.TY == 8) return adj_staged_mat<T, 32, 8>(p, g, is_H, st);
    return adj_staged_mat<T, 32, 4>(p, g, is_H, st);
}

static bool aligned16(const void *ptr) { return ((uintptr_t)ptr & 15u) == 0; }

static long box_cells(const ItemK &o) {
    return (long)(o.hi[0] - o.lo[0]) * (o.hi[1] - o.lo[1]) * (o.hi[2] - o.lo[2]);
}

static int validate(const Plan &p, const fdtd_adjoint_args *a) {
    if (a->n_steps < 0 || (a->parity != 0 && a->parity != 1)) return FDTD_ERR_ARGUMENT;
    if (p.has_feedback) return FDTD_ERR_UNSUPPORTED;  // no transpose of the current feedback
    if (!a->lam_E || !a->lam_H) return FDTD_ERR_ARGUMENT;
    if (p.adj_V > 1 && (!aligned16(a->lam_E) || !aligned16(a->lam_H))) return FDTD_ERR_ARGUMENT;
    if ((a->curl || a->grad) && a->n_objects != p.n_objects) return FDTD_ERR_ARGUMENT;
    for (int s = 0; s < p.k.nslab; ++s) {
        const int b = p.slab_boundary[s];
        for (int q = 0; q < 2; ++q)
            if (!a->aux_E[b][q] || !a->aux_H[b][q]) return FDTD_ERR_ARGUMENT;
    }
    if (a->n_steps == 0) return FDTD_OK;
    if ((a->seed_E || a->seed_H) && (p.n_probe == 0 || a->seed_row - (a->n_steps - 1) < 0))
        return FDTD_ERR_RANGE;
    bool any_dft = false;
    if (a->dft_grad)
        for (size_t q = 0; q < p.dft.size(); ++q) any_dft |= a->dft_grad[q] != nullptr;
    if (any_dft && !a->phase) return FDTD_ERR_ARGUMENT;
    if (a->grad) {
        for (int q = 0; q < p.n_objects; ++q) {
            if (!a->grad[q]) continue;
            const int kind = p.items_host[q].kind;
            if (kind != FDTD_ITEM_OBJECT && kind != FDTD_ITEM_ANISOTROPIC) return FDTD_ERR_UNSUPPORTED;
            if (!a->curl || !a->curl[q]) return FDTD_ERR_ARGUMENT;
            if (a->curl_row - (a->n_steps - 1) < 0) return FDTD_ERR_RANGE;
        }
    }
    return FDTD_OK;
}

// One transposed slab kernel: one thread per cell with 32-bit cell indices
// below 2^31 cells, else a grid-stride loop with 64-bit indices.
template <class T, bool IS_E, int A>
static void launch_adj_slab_axis(const GridK &g, const AdjAux &x, int slab, long cells, cudaStream_t st) {
    if (cells < (1L << 31)) {
        const unsigned blocks = (unsigned)((cells + kThreads - 1) / kThreads);
        k_adj_slab<T, IS_E, A, uint32_t><<<blocks > 0 ? blocks : 1, kThreads, 0, st>>>(g, x, slab);
    } else {
        k_adj_slab<T, IS_E, A, uint64_t><<<grid_stride_blocks(cells), kThreads, 0, st>>>(g, x, slab);
    }
}

template <class T, bool IS_E>
static void launch_adj_slab(const GridK &g, const AdjAux &x, int slab, long cells, cudaStream_t st) {
    const int a = g.slab[slab].axis;
    if (a == 0) launch_adj_slab_axis<T, IS_E, 0>(g, x, slab, cells, st);
    else if (a == 1) launch_adj_slab_axis<T, IS_E, 1>(g, x, slab, cells, st);
    else launch_adj_slab_axis<T, IS_E, 2>(g, x, slab, cells, st);
}

template <class T, int V>
static int adjoint_impl(Plan &p, const fdtd_adjoint_args *a, cudaStream_t st) {
    GridK g = p.k;
    g.E = a->lam_E;
    g.H = a->lam_H;
    g.Elo = g.Hlo = nullptr;
    g.TZ = p.adj_TZ;
    g.TY = p.adj_TY;
    g.XC = p.adj_XC;
    T *LE = (T *)a->lam_E;
    T *LH = (T *)a->lam_H;
    // plans that run the forward PML slabs in kernels of their own do the same
    // for the transposes: slab-free bulk passes, then one kernel per slab
    GridK gb = g;
    if (p.pml_split) gb.nslab = 0;
    // partition plans: slab-free transposed passes over the interior box and
    // the shell kernels with every slab around it
    GridK gi = g;
    if (p.n_shell) {
        gi.nslab = 0;
        gi.nslab_fused = 0;
        gi.TZ = p.adjin_TZ;
        gi.TY = p.adjin_TY;
        gi.XC = p.adjin_XC;
        gi.ox = p.kf.ox;
        gi.oy = p.kf.oy;
        gi.oz = p.kf.oz;
        gi.ex = p.kf.ex;
        gi.ey = p.kf.ey;
        gi.ez = p.kf.ez;
    }
    constexpr int SV = shell_v<T>();
    const unsigned shell_blocks = p.n_shell ? p.shellk.first[p.shellk.nbox] : 0u;
    // staged forward plans with the slabs on their own, or staged partition
    // interiors: staged transposed passes (over the interior box, then the
    // shell kernels)
    const bool staged = p.variant == 2 && (p.pml_split || p.n_shell) && p.adj_V == (sizeof(T) == 4 ? 4 : 2);
    GridK gs = p.k;  // the forward staged tiling, launch order and material copies
    gs.E = a->lam_E;
    gs.H = a->lam_H;
    gs.Elo = gs.Hlo = nullptr;
    gs.nslab = 0;
    gs.nslab_fused = 0;
    if (p.n_shell) {
        gs.ox = p.kf.ox;
        gs.oy = p.kf.oy;
        gs.oz = p.kf.oz;
        gs.ex = p.kf.ex;
        gs.ey = p.kf.ey;
        gs.ez = p.kf.ez;
    }
    auto slab_cells = [&](const SlabK &S) {
        return (long)(S.axis == 0 ? S.th : g.nx) * (S.axis == 1 ? S.th : g.ny) * (S.axis == 2 ? S.th : g.nz);
    };
    const int pblocks = (3 * p.n_probe + kThreads - 1) / kThreads;
    int par = a->parity;
    for (int64_t s = 0; s < a->n_steps; ++s) {
        AdjAux x{};
        for (int q = 0; q < g.nslab; ++q) {
            const int b = p.slab_boundary[q];
            x.Eo[q] = a->aux_E[b][par];
            x.En[q] = a->aux_E[b][par ^ 1];
            x.Ho[q] = a->aux_H[b][par];
            x.Hn[q] = a->aux_H[b][par ^ 1];
        }
        const int64_t srow = a->seed_row - s, crow = a->curl_row - s;

        // transposed H half: detectors, sources, boundaries after the first
        // periodic one (reverse order), then the fused pass
        if (a->seed_H && p.n_probe)
            k_adj_seed_probe<T><<<pblocks, kThreads, 0, st>>>(LH, p.probe_cells, p.n_probe,
                                                              (const T *)a->seed_H + srow * 3 * p.n_probe);
        for (int q = p.srcH0; q < p.srcH0 + p.n_srcH; ++q)
            if (p.items_host[q].kind == FDTD_ITEM_HARD)
                k_adj_zero_box<T><<<grid_stride_blocks(box_cells(p.items_host[q])), kThreads, 0, st>>>(g, q, LH);
        for (const EpiOp &op : p.adj_H) {
            if (op.kind == EPI_COPY) {
                const int n = op.axis == 0 ? g.nx : (op.axis == 1 ? g.ny : g.nz);
                const int n1 = op.axis == 0 ? g.ny : g.nx, n2 = op.axis == 2 ? g.ny : g.nz;
                k_adj_periodic<T><<<grid_stride_blocks((long)n1 * n2 * 3), kThreads, 0, st>>>(LH, g.nx, g.ny, g.nz,
                                                                                           op.axis, n - 1, 0);
            } else {
                const SlabK &S = g.slab[op.slab];
                const long cells = (long)(S.axis == 0 ? S.th : g.nx) * (S.axis == 1 ? S.th : g.ny) *
                                   (S.axis == 2 ? S.th : g.nz);
                k_adj_slab_inc<T, false><<<grid_stride_blocks(cells), kThreads, 0, st>>>(
                    g, op.slab, (T *)a->aux_H[p.slab_boundary[op.slab]][par]);
            }
        }
        if (staged) {
            const int rc = adj_staged<T>(p, gs, true, st);
            if (rc != FDTD_OK) return rc;
            if (p.n_shell) k_adj_shell_H<T, SV><<<shell_blocks, kThreads, 0, st>>>(g, p.shellk, x);
        } else if (p.n_shell) {
            k_adj_H<T, V><<<p.adjin_grid, p.adjin_block, 0, st>>>(gi, x);
            k_adj_shell_H<T, SV><<<shell_blocks, kThreads, 0, st>>>(g, p.shellk, x);
        } else {
            k_adj_H<T, V><<<p.adj_grid, p.adj_block, 0, st>>>(gb, x);
        }
        if (p.pml_split)
            for (int q = 0; q < g.nslab; ++q)
                launch_adj_slab<T, false>(g, x, q, slab_cells(g.slab[q]), st);

        // transposed E half
        if (a->seed_E && p.n_probe)
            k_adj_seed_probe<T><<<pblocks, kThreads, 0, st>>>(LE, p.probe_cells, p.n_probe,
                                                              (const T *)a->seed_E + srow * 3 * p.n_probe);
        if (a->dft_grad) {
            for (size_t q = 0; q < p.dft.size(); ++q) {
                if (!a->dft_grad[q]) continue;
                const fdtd_dft_desc &d = p.dft[q];
                const long cells = (long)(d.hi[0] - d.lo[0]) * (d.hi[1] - d.lo[1]) * (d.hi[2] - d.lo[2]);
                k_adj_seed_dft<T><<<grid_stride_blocks(cells * 3), kThreads, 0, st>>>(
                    LE, g.ny, g.nz, d, a->dft_grad[q], a->phase + s * 2 * p.n_phase_columns);
            }
        }
        for (int q = p.srcE0; q < p.srcE0 + p.n_srcE; ++q)
            if (p.items_host[q].kind == FDTD_ITEM_HARD)
                k_adj_zero_box<T><<<grid_stride_blocks(box_cells(p.items_host[q])), kThreads, 0, st>>>(g, q, LE);
        for (const EpiOp &op : p.adj_E) {
            if (op.kind == EPI_COPY) {
                const int n = op.axis == 0 ? g.nx : (op.axis == 1 ? g.ny : g.nz);
                const int n1 = op.axis == 0 ? g.ny : g.nx, n2 = op.axis == 2 ? g.ny : g.nz;
                k_adj_periodic<T><<<grid_stride_blocks((long)n1 * n2 * 3), kThreads, 0, st>>>(LE, g.nx, g.ny, g.nz,
                                                                                           op.axis, 0, n - 1);
            } else {
                const SlabK &S = g.slab[op.slab];
                const long cells = (long)(S.axis == 0 ? S.th : g.nx) * (S.axis == 1 ? S.th : g.ny) *
                                   (S.axis == 2 ? S.th : g.nz);
                k_adj_slab_inc<T, true><<<grid_stride_blocks(cells), kThreads, 0, st>>>(
                    g, op.slab, (T *)a->aux_E[p.slab_boundary[op.slab]][par]);
            }
        }
        if (staged) {
            const int rc = adj_staged<T>(p, gs, false, st);
            if (rc != FDTD_OK) return rc;
            if (p.n_shell) k_adj_shell_E<T, SV><<<shell_blocks, kThreads, 0, st>>>(g, p.shellk, x);
        } else if (p.n_shell) {
            k_adj_E<T, V><<<p.adjin_grid, p.adjin_block, 0, st>>>(gi, x);
            k_adj_shell_E<T, SV><<<shell_blocks, kThreads, 0, st>>>(g, p.shellk, x);
        } else {
            k_adj_E<T, V><<<p.adj_grid, p.adj_block, 0, st>>>(gb, x);
        }
        if (p.pml_split)
            for (int q = 0; q < g.nslab; ++q)
                launch_adj_slab<T, true>(g, x, q, slab_cells(g.slab[q]), st);
        for (int q = p.n_objects - 1; q >= 0; --q) {
            const ItemK &o = p.items_host[q];
            const long reach = (long)(o.hi[0] - std::max(0, o.lo[0] - 1)) * (o.hi[1] - std::max(0, o.lo[1] - 1)) *
                               (o.hi[2] - std::max(0, o.lo[2] - 1));
            double *gr = a->grad ? a->grad[q] : nullptr;
            const T *cu = gr ? (const T *)a->curl[q] + crow * 3 * box_cells(o) : nullptr;
            k_adj_object<T><<<grid_stride_blocks(reach), kThreads, 0, st>>>(g, q, cu, gr);
            if (o.kind == FDTD_ITEM_ABSORBING)
                k_adj_absorb_scale<T><<<grid_stride_blocks(3 * box_cells(o)), kThreads, 0, st>>>(g, q);
        }
        par ^= 1;
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) {
            set_last_cuda_error((int)e);
            return FDTD_ERR_CUDA;
        }
    }
    return FDTD_OK;
}

int adjoint_f32(Plan &p, const fdtd_adjoint_args *a, cudaStream_t st) {
    const int rc = validate(p, a);
    if (rc != FDTD_OK) return rc;
    return p.adj_V == 4 ? adjoint_impl<float, 4>(p, a, st) : adjoint_impl<float, 1>(p, a, st);
}

int adjoint_f64(Plan &p, const fdtd_adjoint_args *a, cudaStream_t st) {
    const int rc = validate(p, a);
    if (rc != FDTD_OK) return rc;
    return p.adj_V == 2 ? adjoint_impl<double, 2>(p, a, st) : adjoint_impl<double, 1>(p, a, st);
}

}  // namespace fdtd
