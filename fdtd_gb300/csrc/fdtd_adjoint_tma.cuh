// TMA-staged transposed half steps of the reverse-time adjoint (plans whose
// forward pass is TMA-staged with the PML slabs in kernels of their own; the
// transposed slab terms then run in k_adj_slab, objects in k_adj_object).
//
// The transposed halves have the forward passes' shape with the roles of the
// fields swapped (fdtd_adjoint.cuh derives them):
//   k_adj_H_tma: lam_E -= curl_D1(w),  w = (c mu) lam_H, backward neighbours
//                (plane i-1 in registers, row j-1 and cell k-1 in the stage),
//                like the forward E pass;
//   k_adj_E_tma: lam_H += curl_D2(u),  u = (c eps) lam_E, forward neighbours
//                (planes i and i+1 staged, row j+TY and cell k0c+Zc as halo),
//                like the forward H pass.
// A scaled neighbour value needs the material of the neighbour cell, so the
// material tile has the neighbour tile's footprint: values with the same
// prefix / suffix, a one-byte index row starting 16 cells early (H) or
// reaching 16 cells past the tile (E) so that every TMA x coordinate stays
// on a 16-byte boundary, or nothing for a uniform material.  The arithmetic
// is the register-streaming kernels' ((c m) lam products, the same
// differences), so both give the same bits.  Waits are bounded: on expiry
// the CTA records bit 0 in the plan's status word, drains its copies (bit 1
// if a drain wait expires too) and returns.
#pragma once

#include "fdtd_adjoint.cuh"
#include "fdtd_tma.cuh"

namespace fdtd {

template <class T, int TZ, int TY, int MAT>
struct AdjGeom {
    static constexpr int V = sizeof(T) == 4 ? 4 : 2;
    static constexpr int Zc = TZ * V;
    static constexpr int pitchN = 3 * Zc + 4;  // values per neighbour row (4-value prefix or suffix)
    static constexpr int pitchO = 3 * Zc;
    static constexpr int idxN = Zc + 16;       // bytes per index row of the neighbour footprint
    static constexpr int al(int v) { return (v + 127) & ~127; }
    static constexpr int nbrBytes = (TY + 1) * pitchN * (int)sizeof(T);
    static constexpr int matBytes = MAT == MAT_FULL ? nbrBytes : (MAT == MAT_IDS ? (TY + 1) * idxN : 0);
    static constexpr int ownBytes = TY * pitchO * (int)sizeof(T);
    static constexpr int matOff = al(nbrBytes);
    static constexpr int ownOff = matOff + al(matBytes);
    static constexpr int stageBytes = ownOff + al(ownBytes);
    static constexpr uint32_t txBytes = (uint32_t)(nbrBytes + matBytes + ownBytes);
    static constexpr int boxN = pitchN * (int)sizeof(T) / 8;
    static constexpr int boxO = pitchO * (int)sizeof(T) / 8;
};

// (c m) lam for one cell's three values: the neighbour tile holds lam at value
// offset vo; the material is the matching values (FULL), the table row of the
// index byte at io (IDS) or the single row (UNIFORM).
template <class T, int MAT>
__device__ __forceinline__ void adj_scaled3(T *out, const T *lam, int vo, const unsigned char *mat, int io,
                                            const T *lut, T c) {
    if constexpr (MAT == MAT_FULL) {
        const T *m = reinterpret_cast<const T *>(mat) + vo;
#pragma unroll
        for (int q = 0; q < 3; ++q) out[q] = (c * m[q]) * lam[vo + q];
    } else if constexpr (MAT == MAT_IDS) {
        const T *m = lut + 4 * (int)mat[io];
#pragma unroll
        for (int q = 0; q < 3; ++q) out[q] = (c * m[q]) * lam[vo + q];
    } else {
#pragma unroll
        for (int q = 0; q < 3; ++q) out[q] = (c * lut[q]) * lam[vo + q];
    }
}

// Fill one stage of the transposed passes: neighbour tile (lam of the field
// read), its material footprint, and the own tile of the field updated.
// Lane 0 of warp 0 only.
__device__ __forceinline__ void adj_fill(unsigned char *st, uint32_t bar, uint32_t tx, const CUtensorMap *tmN, int xN,
                                         int yN, const CUtensorMap *tmM, int xM, bool mat, const CUtensorMap *tmO,
                                         int xO, int yO, int matOff, int ownOff, bool own) {
    mbar_expect_tx(bar, tx);
    tma_load_2d(smem_u32(st), tmN, xN, yN, bar);
    if (mat) tma_load_2d(smem_u32(st + matOff), tmM, xM, yN, bar);
    if (own) tma_load_2d(smem_u32(st + ownOff), tmO, xO, yO, bar);
}

// Transposed H half (slab-free): lam_E -= curl_D1((c mu) lam_H).
template <class T, int TZ, int TY, int MAT>
__global__ void __launch_bounds__(TZ *TY)
    k_adj_H_tma(const GridK g, const __grid_constant__ CUtensorMap tmN, const __grid_constant__ CUtensorMap tmM,
                const __grid_constant__ CUtensorMap tmO) {
    using G = AdjGeom<T, TZ, TY, MAT>;
    constexpr int V = G::V;
    constexpr int N = 3 * V;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ int abort_flag;
    unsigned char *smem = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);
    const int S = g.stages;
    const int SB = g.stage_bytes;
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + (size_t)S * SB);
    T *lut = reinterpret_cast<T *>((reinterpret_cast<uintptr_t>(bars + S) + 15) & ~uintptr_t(15));
    const int tz = threadIdx.x, ty = threadIdx.y, tid = ty * TZ + tz;
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const TileId tile = tile_of(g);
    const int k0c = g.oz + tile.bx * G::Zc, j0 = g.oy + tile.by * TY;
    const int k0 = k0c + tz * V, j = j0 + ty;
    const int xa = g.ox + tile.bz * g.XC, xb = min(g.ex, xa + g.XC);
    const int np = xb - xa;
    const bool act = (j < g.ey) && (k0 < g.ez);
    const T c = material_courant<T>(g);
    T *LE = (T *)g.E;
    const T *LH = (const T *)g.H;
    const T *__restrict__ MU = (const T *)g.imu;
    const int xN = (3 * k0c - 4) * (int)sizeof(T) / 8, xO = 3 * k0c * (int)sizeof(T) / 8;
    const int xM = MAT == MAT_IDS ? k0c - 16 : xN;

    if (tid == 0) {
        abort_flag = 0;
        for (int s = 0; s < S; ++s) mbar_init(smem_u32(&bars[s]), 1);
        fence_mbar_init();
        fence_proxy_async();
    }
    if constexpr (MAT != MAT_FULL) stage_material_table<T>(g.mlut_H, g.nlut_H, MAT == MAT_IDS ? 256 : 1, lut);
    __syncthreads();

    auto issue = [&](int r) {
        const int p = xa + r;
        adj_fill(smem + (size_t)(r % S) * SB, smem_u32(&bars[r % S]), G::txBytes, &tmN, xN, p * ny + j0 - 1, &tmM, xM,
                 MAT != MAT_UNIFORM, &tmO, xO, p * ny + j0, G::matOff, G::ownOff, true);
    };
    int issued = 0;
    for (; issued < min(S, np); ++issued)
        if (tid == 0) issue(issued);

    alignas(16) T wp[N];  // w at plane i-1
    zero(wp);
    if (act && xa > 0) load_scaled<T, V>(wp, LH, MU, ((size_t)(xa - 1) * ny + j) * nz + k0, c);

    int r = 0;
    for (; r < np; ++r) {
        const int i = xa + r;
        const unsigned char *st = smem + (size_t)(r % S) * SB;
        const bool ok = mbar_wait_bounded(smem_u32(&bars[r % S]), (uint32_t)((r / S) & 1));
        if (!ok) abort_flag = 1;
        if (act && ok) {
            const T *Ln = reinterpret_cast<const T *>(st);
            const unsigned char *Mt = st + G::matOff;
            const int on = (ty + 1) * G::pitchN + 4 + 3 * tz * V;  // own row in the neighbour tile
            const int io = (ty + 1) * G::idxN + 16 + tz * V;       // its index bytes
            alignas(16) T w[N], wj[N], e[N];
#pragma unroll
            for (int v = 0; v < V; ++v) {
                adj_scaled3<T, MAT>(w + 3 * v, Ln, on + 3 * v, Mt, io + v, lut, c);
                adj_scaled3<T, MAT>(wj + 3 * v, Ln, on - G::pitchN + 3 * v, Mt, io - G::idxN + v, lut, c);
            }
            T k3[3];  // w at cell k0-1 (the prefix when tz == 0)
            adj_scaled3<T, MAT>(k3, Ln, on - 3, Mt, io - 1, lut, c);
            const T kx = k3[0], ky = k3[1];
            ld_vec(e, reinterpret_cast<const T *>(st + G::ownOff) + ty * G::pitchO + 3 * tz * V);
            const bool xin = i < nx - 1, xbk = i > 0;
            const bool yin = j < ny - 1, ybk = j > 0;
#pragma unroll
            for (int v = 0; v < V; ++v) {
                const int k = k0 + v;
                const bool zin = k < nz - 1, zbk = k > 0;
                const T zx = v > 0 ? w[3 * (v - 1)] : kx;
                const T zy = v > 0 ? w[3 * (v - 1) + 1] : ky;
                const T wx = w[3 * v], wy = w[3 * v + 1], wz = w[3 * v + 2];
                const T dy_z = (yin ? wz : T(0)) - (ybk ? wj[3 * v + 2] : T(0));
                const T dz_y = (zin ? wy : T(0)) - (zbk ? zy : T(0));
                const T dz_x = (zin ? wx : T(0)) - (zbk ? zx : T(0));
                const T dx_z = (xin ? wz : T(0)) - (xbk ? wp[3 * v + 2] : T(0));
                const T dx_y = (xin ? wy : T(0)) - (xbk ? wp[3 * v + 1] : T(0));
                const T dy_x = (yin ? wx : T(0)) - (ybk ? wj[3 * v] : T(0));
                e[3 * v] -= dy_z - dz_y;
                e[3 * v + 1] -= dz_x - dx_z;
                e[3 * v + 2] -= dx_y - dy_x;
            }
            st_vec(LE + 3 * (((size_t)i * ny + j) * nz + k0), e);
#pragma unroll
            for (int q = 0; q < N; ++q) wp[q] = w[q];
        }
        __syncthreads();
        if (abort_flag) break;
        if (issued < np) {
            if (tid == 0) {
                fence_proxy_async();
                issue(issued);
            }
            ++issued;
        }
    }
    if (abort_flag && tid == 0) {
        atomicOr(g.status, 1);
        for (int q = r; q < issued; ++q)
            if (!mbar_wait_bounded(smem_u32(&bars[q % S]), (uint32_t)((q / S) & 1))) atomicOr(g.status, 2);
    }
}

// Transposed E half (slab-free): lam_H += curl_D2((c eps) lam_E).
template <class T, int TZ, int TY, int MAT>
__global__ void __launch_bounds__(TZ *TY)
    k_adj_E_tma(const GridK g, const __grid_constant__ CUtensorMap tmN, const __grid_constant__ CUtensorMap tmM,
                const __grid_constant__ CUtensorMap tmO) {
    using G = AdjGeom<T, TZ, TY, MAT>;
    constexpr int V = G::V;
    constexpr int N = 3 * V;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ int abort_flag;
    unsigned char *smem = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);
    const int S = g.stages;
    const int SB = g.stage_bytes;
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + (size_t)S * SB);
    T *lut = reinterpret_cast<T *>((reinterpret_cast<uintptr_t>(bars + S) + 15) & ~uintptr_t(15));
    const int tz = threadIdx.x, ty = threadIdx.y, tid = ty * TZ + tz;
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const TileId tile = tile_of(g);
    const int k0c = g.oz + tile.bx * G::Zc, j0 = g.oy + tile.by * TY;
    const int k0 = k0c + tz * V, j = j0 + ty;
    const int xa = g.ox + tile.bz * g.XC, xb = min(g.ex, xa + g.XC);
    const int np = xb - xa;
    const int nfill = np + 1;  // lam_E of plane xb is needed by the last plane
    const bool act = (j < g.ey) && (k0 < g.ez);
    const T c = material_courant<T>(g);
    T *LH = (T *)g.H;
    const int xN = 3 * k0c * (int)sizeof(T) / 8;
    const int xM = MAT == MAT_IDS ? k0c : xN;

    if (tid == 0) {
        abort_flag = 0;
        for (int s = 0; s < S; ++s) mbar_init(smem_u32(&bars[s]), 1);
        fence_mbar_init();
        fence_proxy_async();
    }
    if constexpr (MAT != MAT_FULL) stage_material_table<T>(g.mlut_E, g.nlut_E, MAT == MAT_IDS ? 256 : 1, lut);
    __syncthreads();

    auto issue = [&](int r) {
        const int p = xa + r;
        // the last fill (plane xb) only provides the x neighbour: no own tile
        adj_fill(smem + (size_t)(r % S) * SB, smem_u32(&bars[r % S]),
                 p < xb ? G::txBytes : (uint32_t)(G::nbrBytes + G::matBytes), &tmN, xN, p * ny + j0, &tmM, xM,
                 MAT != MAT_UNIFORM, &tmO, xN, p * ny + j0, G::matOff, G::ownOff, p < xb);
    };
    int issued = 0;
    for (; issued < min(S, nfill); ++issued)
        if (tid == 0) issue(issued);

    int r = 0;
    for (; r < np; ++r) {
        const int i = xa + r;
        const unsigned char *st = smem + (size_t)(r % S) * SB;
        const unsigned char *sn = smem + (size_t)((r + 1) % S) * SB;
        bool ok = mbar_wait_bounded(smem_u32(&bars[r % S]), (uint32_t)((r / S) & 1));
        ok = ok && mbar_wait_bounded(smem_u32(&bars[(r + 1) % S]), (uint32_t)(((r + 1) / S) & 1));
        if (!ok) abort_flag = 1;
        if (act && ok) {
            const T *Lc = reinterpret_cast<const T *>(st);
            const T *Ln = reinterpret_cast<const T *>(sn);
            const int on = ty * G::pitchN + 3 * tz * V;
            const int io = ty * G::idxN + tz * V;
            alignas(16) T u[N], un[N], uj[N], h[N];
#pragma unroll
            for (int v = 0; v < V; ++v) {
                adj_scaled3<T, MAT>(u + 3 * v, Lc, on + 3 * v, st + G::matOff, io + v, lut, c);
                adj_scaled3<T, MAT>(un + 3 * v, Ln, on + 3 * v, sn + G::matOff, io + v, lut, c);
                adj_scaled3<T, MAT>(uj + 3 * v, Lc, on + G::pitchN + 3 * v, st + G::matOff, io + G::idxN + v, lut,
                                    c);
            }
            T k3[3];  // u at cell k0+V (the suffix for the last lane)
            adj_scaled3<T, MAT>(k3, Lc, on + N, st + G::matOff, io + V, lut, c);
            const T kx = k3[0], ky = k3[1];
            ld_vec(h, reinterpret_cast<const T *>(st + G::ownOff) + ty * G::pitchO + 3 * tz * V);
            const bool xn = i < nx - 1, xo = i > 0;
            const bool yn = j < ny - 1, yo = j > 0;
#pragma unroll
            for (int v = 0; v < V; ++v) {
                const int k = k0 + v;
                const bool zn = k < nz - 1, zo = k > 0;
                const T nzx = v < V - 1 ? u[3 * (v + 1)] : kx;
                const T nzy = v < V - 1 ? u[3 * (v + 1) + 1] : ky;
                const T ux = u[3 * v], uy = u[3 * v + 1], uz = u[3 * v + 2];
                const T dy_z = (yn ? uj[3 * v + 2] : T(0)) - (yo ? uz : T(0));
                const T dz_y = (zn ? nzy : T(0)) - (zo ? uy : T(0));
                const T dz_x = (zn ? nzx : T(0)) - (zo ? ux : T(0));
                const T dx_z = (xn ? un[3 * v + 2] : T(0)) - (xo ? uz : T(0));
                const T dx_y = (xn ? un[3 * v + 1] : T(0)) - (xo ? uy : T(0));
                const T dy_x = (yn ? uj[3 * v] : T(0)) - (yo ? ux : T(0));
                h[3 * v] += dy_z - dz_y;
                h[3 * v + 1] += dz_x - dx_z;
                h[3 * v + 2] += dx_y - dy_x;
            }
            st_vec(LH + 3 * (((size_t)i * ny + j) * nz + k0), h);
        }
        __syncthreads();
        if (abort_flag) break;
        if (issued < nfill) {
            if (tid == 0) {
                fence_proxy_async();
                issue(issued);
            }
            ++issued;
        }
    }
    if (abort_flag && tid == 0) {
        atomicOr(g.status, 1);
        for (int q = r; q < issued; ++q)
            if (!mbar_wait_bounded(smem_u32(&bars[q % S]), (uint32_t)((q / S) & 1))) atomicOr(g.status, 2);
    }
}

}  // namespace fdtd
