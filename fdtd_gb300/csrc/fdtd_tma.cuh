// TMA-staged fused half steps.
//
// A CTA of TZ x TY threads (32 x 8, 32 x 4 or 16 x 16) owns a tile of TY rows
// (y) by TZ*V cells (z) and marches along x over a chunk of planes.  Each
// field is viewed as a 2D tensor of (nx*ny) rows by 3*nz values (8-byte
// elements for the tensor map) and one TMA load per field and plane fills a
// shared-memory stage:
//
//   E half: H tile of TY+1 rows (row 0 = j0-1) with a 4-value prefix that
//           holds the cell k0-1, plus the E, inverse-permittivity (and
//           compensation) tiles of TY rows;
//   H half: E tile of TY+1 rows (row TY = j0+TY) with a 4-value suffix that
//           holds the cell k0+TZ*V, plus the H, inverse-permeability (and
//           compensation) tiles.  Plane i needs E(i) and E(i+1), so two
//           stages are read at once.
//
// The material tile is the three values per cell, a one-byte index per cell
// into a table staged in shared memory at kernel start (a uint8 tensor map
// of (nx*ny) rows by nz bytes), or absent for a uniform material (MAT).
//
// A ring of S stages keeps S-1 planes of loads in flight while the threads
// compute from shared memory; the E half keeps H(i-1) in registers.  The
// tiles reach past the grid edges where the differences are dropped; the
// TMA unit fills out-of-range rows and columns with zeros.  Every mbarrier
// wait is bounded: on expiry the CTA records bit 0 in the plan's status word,
// drains its outstanding copies (bounded again; bit 1 when a drain wait also
// expires) and returns.
#pragma once

#include <cuda.h>

#include "fdtd_cell.cuh"

namespace fdtd {

constexpr unsigned kWaitLimit = 1u << 22;

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity, unsigned limit = kWaitLimit) {
    for (unsigned it = 0; it < limit; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int x, int y, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
        : "memory");
}

__device__ __forceinline__ void bulk_copy_g2s(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(dst), "l"(reinterpret_cast<uint64_t>(src)), "r"(bytes), "r"(bar)
                 : "memory");
}

__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

// The tile a CTA works on: blocks are launched in the order of g.cta_order
// when the plan has one (the tiles that carry objects or PML slabs first, so
// that they do not finish last), else in grid order.
struct TileId {
    int bx, by, bz, cta;
};

__device__ __forceinline__ TileId tile_of(const GridK &g) {
    int lin = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
    if (g.cta_order) lin = g.cta_order[lin];
    TileId t;
    t.cta = lin;
    t.bx = lin % gridDim.x;
    t.by = (lin / gridDim.x) % gridDim.y;
    t.bz = lin / (gridDim.x * gridDim.y);
    return t;
}

// Byte layout of the field part of one stage: the neighbour tile (TY+1 rows
// of 3*Zc+4 values), the own field tile (TY rows of 3*Zc values), the own
// material tile (values, indices or nothing) and, compensated, the own
// compensation tile, each 128-byte aligned.  The PML auxiliary slots follow
// at g.psi_off[s].  A tile is TZ threads (V cells each) along z by TY rows.
template <class T, int TZ, int TY, bool COMP, int MAT = MAT_FULL>
struct StageGeom {
    static constexpr int V = sizeof(T) == 4 ? 4 : 2;
    static constexpr int Zc = TZ * V;  // cells per tile row
    static constexpr int pitchN = 3 * Zc + 4;  // values per neighbour row
    static constexpr int pitchO = 3 * Zc;
    static constexpr int nbrBytes = (TY + 1) * pitchN * (int)sizeof(T);
    static constexpr int ownBytes = TY * pitchO * (int)sizeof(T);
    static constexpr int matBytes = MAT == MAT_FULL ? ownBytes : (MAT == MAT_IDS ? TY * Zc : 0);
    static constexpr int al(int v) { return (v + 127) & ~127; }
    static constexpr int ownOff = al(nbrBytes);
    static constexpr int matOff = ownOff + al(ownBytes);
    static constexpr int loOff = matOff + al(matBytes);
    static constexpr int stageBytes = loOff + (COMP ? al(ownBytes) : 0);
    static constexpr uint32_t txBytes = (uint32_t)(nbrBytes + ownBytes + matBytes + (COMP ? ownBytes : 0));
    // tensor-map boxes in 8-byte elements (fields, full materials) and bytes (indices)
    static constexpr int boxN = pitchN * (int)sizeof(T) / 8;
    static constexpr int boxO = pitchO * (int)sizeof(T) / 8;
    static constexpr int boxI = Zc;
};

// Fill one stage for plane p (warp 0 of the CTA, all lanes).  The PML auxiliary rows of
// every staged slab crossing the tile at plane p are copied with 1D bulk copies (one
// row per lane), then lane 0 arms the stage barrier with the total byte count
// and issues the field tiles.
template <class T, int TY>
__device__ __forceinline__ void fill_stage(const GridK &g, unsigned char *st, uint32_t bar, int p, bool with_psi,
                                           bool is_E, int k0c, int j0, int Zc, const CUtensorMap *tmN, int xN,
                                           int yN, const CUtensorMap *tmF, const CUtensorMap *tmM,
                                           const CUtensorMap *tmL, bool comp, int xO, int xM, int mat,
                                           uint32_t field_tx, int ownOff, int matOff, int loOff) {
    const int lane = (threadIdx.y * blockDim.x + threadIdx.x) & 31;
    uint32_t bytes[2] = {0u, 0u};
    const void *srcp[2] = {nullptr, nullptr};
    uint32_t dst[2] = {0u, 0u};
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int q = lane + 32 * h;
        const int si = q / TY, rr = q % TY;
        const int j = j0 + rr;
        if (!with_psi || si >= g.n_staged || j >= g.ny) continue;
        const int s = g.staged_slab[si];
        const SlabK &S = g.slab[s];
        const T *psi = (const T *)(is_E ? S.psiE_rd : S.psiH_rd);
        const int cells = min(Zc, g.nz - k0c);
        size_t off;
        uint32_t nb;
        if (S.axis == 0) {
            const int l = p - S.start;
            if ((unsigned)l >= (unsigned)S.th) continue;
            off = (((size_t)l * g.ny + j) * g.nz + k0c) * 2;
            nb = (uint32_t)(2 * cells * sizeof(T));
        } else if (S.axis == 1) {
            const int l = j - S.start;
            if ((unsigned)l >= (unsigned)S.th) continue;
            off = (((size_t)p * S.th + l) * g.nz + k0c) * 2;
            nb = (uint32_t)(2 * cells * sizeof(T));
        } else {
            if (k0c >= S.start + S.th || k0c + Zc <= S.start) continue;
            off = ((size_t)p * g.ny + j) * S.thp * 2;
            nb = (uint32_t)(2 * S.thp * sizeof(T));
        }
        bytes[h] = nb;
        srcp[h] = psi + off;
        dst[h] = smem_u32(st + g.psi_off[s] + (size_t)rr * g.psi_pitch[s] * sizeof(T));
    }
    const uint32_t tot = __reduce_add_sync(0xffffffffu, bytes[0] + bytes[1]);
    if (lane == 0) mbar_expect_tx(bar, field_tx + tot);
    __syncwarp();
#pragma unroll
    for (int h = 0; h < 2; ++h)
        if (bytes[h]) bulk_copy_g2s(dst[h], srcp[h], bytes[h], bar);
    if (lane == 0) {
        const int yO = yN + (is_E ? 1 : 0);
        tma_load_2d(smem_u32(st), tmN, xN, yN, bar);
        tma_load_2d(smem_u32(st + ownOff), tmF, xO, yO, bar);
        if (mat == MAT_FULL) tma_load_2d(smem_u32(st + matOff), tmM, xO, yO, bar);
        else if (mat == MAT_IDS) tma_load_2d(smem_u32(st + matOff), tmM, xM, yO, bar);
        if (comp) tma_load_2d(smem_u32(st + loOff), tmL, xO, yO, bar);
    }
}

// Copy the PML b/c tables of the half step into shared memory (all threads).
template <class T>
__device__ __forceinline__ void stage_coef_tables(const GridK &g, T *tab, bool is_E) {
    const int nthr = blockDim.x * blockDim.y, tid = threadIdx.y * blockDim.x + threadIdx.x;
    for (int s = 0; s < g.nslab; ++s) {
        const SlabK &S = g.slab[s];
        const T *b = (const T *)(is_E ? S.bE : S.bH);
        const T *c = (const T *)(is_E ? S.cE : S.cH);
        for (int t = tid; t < 2 * S.th; t += nthr) tab[g.coef_off[s] + t] = t < S.th ? b[t] : c[t - S.th];
    }
}

// Copy the n material value triples of a half step into the padded 4-value
// rows of the shared-memory table; rows n .. rows-1 are zero (all threads).
template <class T>
__device__ __forceinline__ void stage_material_table(const void *lut, int n, int rows, T *dst) {
    const int nthr = blockDim.x * blockDim.y, tid = threadIdx.y * blockDim.x + threadIdx.x;
    const T *src = (const T *)lut;
    for (int t = tid; t < 4 * rows; t += nthr) {
        const int r = t >> 2, c = t & 3;
        dst[t] = (r < n && c < 3) ? src[3 * r + c] : T(0);
    }
}

// One padded table row (three values) from shared memory.
__device__ __forceinline__ void lut_row(float *m, const float *row) {
    const float4 q = *reinterpret_cast<const float4 *>(row);
    m[0] = q.x;
    m[1] = q.y;
    m[2] = q.z;
}
__device__ __forceinline__ void lut_row(double *m, const double *row) {
    const double2 q = *reinterpret_cast<const double2 *>(row);
    m[0] = q.x;
    m[1] = q.y;
    m[2] = row[2];
}

// The inverse material of a thread's V cells from the stage: the values
// (MAT_FULL, at value offset oo of the material tile), the table rows of
// their indices (MAT_IDS, at byte offset io), or the one table row.
template <class T, int V, int MAT>
__device__ __forceinline__ void stage_material(T (&m)[3 * V], const unsigned char *tile, int oo, int io,
                                               const T *lut) {
    if constexpr (MAT == MAT_FULL) {
        ld_vec(m, reinterpret_cast<const T *>(tile) + oo);
    } else if constexpr (MAT == MAT_IDS) {
        unsigned char id[V];
        if constexpr (V == 4) {
            const uchar4 q = *reinterpret_cast<const uchar4 *>(tile + io);
            id[0] = q.x;
            id[1] = q.y;
            id[2] = q.z;
            id[3] = q.w;
        } else {
            const uchar2 q = *reinterpret_cast<const uchar2 *>(tile + io);
            id[0] = q.x;
            id[1] = q.y;
        }
#pragma unroll
        for (int v = 0; v < V; ++v) lut_row(m + 3 * v, lut + 4 * (int)id[v]);
    } else {
#pragma unroll
        for (int v = 0; v < V; ++v) lut_row(m + 3 * v, lut);
    }
}

template <class P, int TZ, int TY, int MAT>
__global__ void __launch_bounds__(TZ *TY)
    k_update_E_tma(const GridK g, const double *__restrict__ wave, const __grid_constant__ CUtensorMap tmN,
                   const __grid_constant__ CUtensorMap tmF, const __grid_constant__ CUtensorMap tmM,
                   const __grid_constant__ CUtensorMap tmL) {
    using T = typename P::T;
    using G = StageGeom<T, TZ, TY, P::COMP, MAT>;
    constexpr int V = G::V;
    constexpr int N = 3 * V;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ int abort_flag;
    // TMA destinations must be 128-byte aligned; the launch adds 128 bytes of slack
    unsigned char *smem = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);
    const int S = g.stages;
    const int SB = g.stage_bytes;
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + (size_t)S * SB);
    T *ctab = reinterpret_cast<T *>(smem + (size_t)S * SB + 8 * (size_t)S);
    // material table (MAT_IDS, MAT_UNIFORM): padded rows, 16-byte aligned
    T *mlut = reinterpret_cast<T *>((reinterpret_cast<uintptr_t>(ctab + g.coef_values) + 15) & ~uintptr_t(15));
    const int tz = threadIdx.x, ty = threadIdx.y, tid = ty * TZ + tz;
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const TileId tile = tile_of(g);
    const int k0c = g.oz + tile.bx * G::Zc, j0 = g.oy + tile.by * TY;
    const int k0 = k0c + tz * V, j = j0 + ty;
    const int xa = g.ox + tile.bz * g.XC, xb = min(g.ex, xa + g.XC);
    const int np = xb - xa;
    const bool act = (j < g.ey) && (k0 < g.ez);
    const int cta = tile.cta;
    const T c = courant_of<T>(g);
    const T *__restrict__ H = (const T *)g.H;
    T *E = (T *)g.E;
    T *Elo = (T *)g.Elo;
    const int ob0 = g.obj_off[cta], ob1 = g.obj_off[cta + 1];
    int sb0 = 0, sb1 = 0;
    if (g.fuse_src_E) {
        sb0 = g.srcE_off[cta];
        sb1 = g.srcE_off[cta + 1];
    }
    const int xN = (3 * k0c - 4) * (int)sizeof(T) / 8;  // neighbour tile starts 4 values early
    const int xO = 3 * k0c * (int)sizeof(T) / 8;

    if (tid == 0) {
        abort_flag = 0;
        for (int s = 0; s < S; ++s) mbar_init(smem_u32(&bars[s]), 1);
        fence_mbar_init();
        fence_proxy_async();
    }
    if (g.coef_values) stage_coef_tables<T>(g, ctab, true);
    if constexpr (MAT != MAT_FULL) stage_material_table<T>(g.mlut_E, g.nlut_E, g.lut_rows, mlut);
    __syncthreads();

    auto issue = [&](int r) {
        const int p = xa + r;
        fill_stage<T, TY>(g, smem + (size_t)(r % S) * SB, smem_u32(&bars[r % S]), p, true, true, k0c, j0, G::Zc,
                          &tmN, xN, p * ny + j0 - 1, &tmF, &tmM, &tmL, P::COMP, xO, k0c, MAT, G::txBytes, G::ownOff,
                          G::matOff, G::loOff);
    };
    int issued = 0;
    for (; issued < min(S, np); ++issued)
        if (tid < 32) issue(issued);

    const unsigned mask_yz = slab_mask_yz(g, j, k0, V);
    alignas(16) T hp[N];  // H at plane i-1 (registers)
#pragma unroll
    for (int q = 0; q < N; ++q) hp[q] = T(0);
    if (act && xa > 0) ld_vec_ro(hp, H + 3 * (((size_t)(xa - 1) * ny + j) * nz + k0));

    int r = 0;
    for (; r < np; ++r) {
        const int i = xa + r;
        const unsigned char *st = smem + (size_t)(r % S) * SB;
        const bool ok = mbar_wait_bounded(smem_u32(&bars[r % S]), (uint32_t)((r / S) & 1));
        if (!ok) abort_flag = 1;
        if (act && ok) {
            const T *Hn = reinterpret_cast<const T *>(st);
            const T *Ef = reinterpret_cast<const T *>(st + G::ownOff);
            const int on = (ty + 1) * G::pitchN + 4 + 3 * tz * V;  // own row in the neighbour tile
            const int oo = ty * G::pitchO + 3 * tz * V;
            alignas(16) T hc[N], hj[N], e[N], el[N], m[N];
            ld_vec(hc, Hn + on);
            ld_vec(hj, Hn + on - G::pitchN);
            ld_vec(e, Ef + oo);
            stage_material<T, V, MAT>(m, st + G::matOff, oo, ty * G::Zc + tz * V, mlut);
            if constexpr (P::COMP) {
                ld_vec(el, reinterpret_cast<const T *>(st + G::loOff) + oo);
            } else {
#pragma unroll
                for (int q = 0; q < N; ++q) el[q] = T(0);
            }
            const T kx = Hn[on - 3], ky = Hn[on - 2];  // cell k0-1 (prefix when tz == 0)
            const PsiSrc<T> src{st, ty, k0c, g.coef_values ? ctab : nullptr};
            const unsigned slabs = mask_yz | slab_mask_x(g, i);
            thread_E<P, V>(g, wave, i, j, k0, c, hc, hp, hj, kx, ky, m, e, el, ob0, ob1, sb0, sb1, src, slabs);
            const size_t cell0 = ((size_t)i * ny + j) * nz + k0;
            st_vec(E + 3 * cell0, e);
            if constexpr (P::COMP) st_vec(Elo + 3 * cell0, el);
#pragma unroll
            for (int q = 0; q < N; ++q) hp[q] = hc[q];
        }
        __syncthreads();
        if (abort_flag) break;
        if (issued < np) {
            if (tid < 32) {
                fence_proxy_async();
                issue(issued);
            }
            ++issued;
        }
    }
    if (abort_flag && tid == 0) {
        atomicOr(g.status, 1);
        // a drain wait that also runs out leaves copies into shared memory in
        // flight after the CTA exits: bit 1 marks later results untrusted
        for (int q = r; q < issued; ++q)
            if (!mbar_wait_bounded(smem_u32(&bars[q % S]), (uint32_t)((q / S) & 1))) atomicOr(g.status, 2);
    }
}

template <class P, int TZ, int TY, int MAT>
__global__ void __launch_bounds__(TZ *TY)
    k_update_H_tma(const GridK g, const double *__restrict__ wave, const __grid_constant__ CUtensorMap tmN,
                   const __grid_constant__ CUtensorMap tmF, const __grid_constant__ CUtensorMap tmM,
                   const __grid_constant__ CUtensorMap tmL) {
    using T = typename P::T;
    using G = StageGeom<T, TZ, TY, P::COMP, MAT>;
    constexpr int V = G::V;
    constexpr int N = 3 * V;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ int abort_flag;
    unsigned char *smem = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);
    const int S = g.stages;
    const int SB = g.stage_bytes;
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + (size_t)S * SB);
    T *ctab = reinterpret_cast<T *>(smem + (size_t)S * SB + 8 * (size_t)S);
    // material table (MAT_IDS, MAT_UNIFORM): padded rows, 16-byte aligned
    T *mlut = reinterpret_cast<T *>((reinterpret_cast<uintptr_t>(ctab + g.coef_values) + 15) & ~uintptr_t(15));
    const int tz = threadIdx.x, ty = threadIdx.y, tid = ty * TZ + tz;
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const TileId tile = tile_of(g);
    const int k0c = g.oz + tile.bx * G::Zc, j0 = g.oy + tile.by * TY;
    const int k0 = k0c + tz * V, j = j0 + ty;
    const int xa = g.ox + tile.bz * g.XC, xb = min(g.ex, xa + g.XC);
    const int np = xb - xa;
    const int nfill = np + 1;  // E of plane xb is needed by the last plane
    const bool act = (j < g.ey) && (k0 < g.ez);
    const int cta = tile.cta;
    const T c = courant_of<T>(g);
    T *H = (T *)g.H;
    T *Hlo = (T *)g.Hlo;
    int sb0 = 0, sb1 = 0;
    if (g.fuse_src_H) {
        sb0 = g.srcH_off[cta];
        sb1 = g.srcH_off[cta + 1];
    }
    const int xO = 3 * k0c * (int)sizeof(T) / 8;

    if (tid == 0) {
        abort_flag = 0;
        for (int s = 0; s < S; ++s) mbar_init(smem_u32(&bars[s]), 1);
        fence_mbar_init();
        fence_proxy_async();
    }
    if (g.coef_values) stage_coef_tables<T>(g, ctab, false);
    if constexpr (MAT != MAT_FULL) stage_material_table<T>(g.mlut_H, g.nlut_H, g.lut_rows, mlut);
    __syncthreads();

    auto issue = [&](int r) {
        const int p = xa + r;
        fill_stage<T, TY>(g, smem + (size_t)(r % S) * SB, smem_u32(&bars[r % S]), p, p < xb, false, k0c, j0,
                          G::Zc, &tmN, xO, p * ny + j0, &tmF, &tmM, &tmL, P::COMP, xO, k0c, MAT, G::txBytes,
                          G::ownOff, G::matOff, G::loOff);
    };
    int issued = 0;
    for (; issued < min(S, nfill); ++issued)
        if (tid < 32) issue(issued);

    const unsigned mask_yz = slab_mask_yz(g, j, k0, V);
    int r = 0;
    for (; r < np; ++r) {
        const int i = xa + r;
        const unsigned char *st = smem + (size_t)(r % S) * SB;
        const unsigned char *sn = smem + (size_t)((r + 1) % S) * SB;
        bool ok = mbar_wait_bounded(smem_u32(&bars[r % S]), (uint32_t)((r / S) & 1));
        ok = ok && mbar_wait_bounded(smem_u32(&bars[(r + 1) % S]), (uint32_t)(((r + 1) / S) & 1));
        if (!ok) abort_flag = 1;
        if (act && ok) {
            const T *En = reinterpret_cast<const T *>(st);
            const T *Ex1 = reinterpret_cast<const T *>(sn);
            const T *Hf = reinterpret_cast<const T *>(st + G::ownOff);
            const int on = ty * G::pitchN + 3 * tz * V;
            const int oo = ty * G::pitchO + 3 * tz * V;
            alignas(16) T ec[N], en[N], ej[N], h[N], hl[N], m[N];
            ld_vec(ec, En + on);
            ld_vec(ej, En + on + G::pitchN);
            ld_vec(en, Ex1 + on);
            ld_vec(h, Hf + oo);
            stage_material<T, V, MAT>(m, st + G::matOff, oo, ty * G::Zc + tz * V, mlut);
            if constexpr (P::COMP) {
                ld_vec(hl, reinterpret_cast<const T *>(st + G::loOff) + oo);
            } else {
#pragma unroll
                for (int q = 0; q < N; ++q) hl[q] = T(0);
            }
            const T kx = En[on + N], ky = En[on + N + 1];  // cell k0+V (suffix for the last lane)
            const PsiSrc<T> src{st, ty, k0c, g.coef_values ? ctab : nullptr};
            const unsigned slabs = mask_yz | slab_mask_x(g, i);
            thread_H<P, V>(g, wave, i, j, k0, c, ec, en, ej, kx, ky, m, h, hl, sb0, sb1, src, slabs);
            const size_t cell0 = ((size_t)i * ny + j) * nz + k0;
            st_vec(H + 3 * cell0, h);
            if constexpr (P::COMP) st_vec(Hlo + 3 * cell0, hl);
        }
        __syncthreads();
        if (abort_flag) break;
        if (issued < nfill) {
            if (tid < 32) {
                fence_proxy_async();
                issue(issued);
            }
            ++issued;
        }
    }
    if (abort_flag && tid == 0) {
        atomicOr(g.status, 1);
        // a drain wait that also runs out leaves copies into shared memory in
        // flight after the CTA exits: bit 1 marks later results untrusted
        for (int q = r; q < issued; ++q)
            if (!mbar_wait_bounded(smem_u32(&bars[q % S]), (uint32_t)((q / S) & 1))) atomicOr(g.status, 2);
    }
}

}  // namespace fdtd
