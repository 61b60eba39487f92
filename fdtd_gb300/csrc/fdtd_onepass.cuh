// One pass per time step: the E half step and the H half step of a whole time
// step in one TMA-staged kernel.
//
// The two-pass plans read E, H and the materials twice per step (E pass: H,
// E, eps; H pass: E, H, mu).  Here a CTA marching along x computes, for each
// plane p, the new E of plane p and then the new H of plane p-1, which needs
// the new E of planes p-1 and p only; every field value is read once and
// written once per step.  Tiles of neighbouring CTAs are updated in the same
// pass, so the step reads the old fields from one buffer and writes the new
// ones to another (E, H and the PML auxiliaries are double buffered; plans
// alternate the direction so that an even number of steps ends in the
// caller's buffers), and every tile recomputes, without storing it, the new E
// of the cells its H update reads across its edges: one row past the tile
// along y (an extra warp), one cell past it along z (the same warp), and the
// first plane of the next x chunk.
//
// CTA: 32 threads along z (V cells each, Zc = 32*V cells) by TY own rows plus
// the halo warp.  Per plane one stage holds (all TMA, zero fill past the grid):
//   H tile   TY+2 rows (j0-1 .. j0+TY) x (cell k0c-1 (4-value prefix), Zc cells, cell k0c+Zc (suffix))
//   E tile   TY+1 rows (j0 .. j0+TY)  x (Zc cells, cell k0c+Zc)
//   E material (values, one-byte indices or none) over the E tile's cells
//   H material over the own cells
//   PML auxiliary rows: E side TY+1 rows (x/y slabs Zc+2 pairs), H side TY rows
// Stage r is used in iteration r (E of its plane) and iteration r+1 (its H
// tile as the x neighbour of the next plane, and the H update of its plane),
// then refilled: a ring of S >= 3 stages keeps S-2 planes of loads in flight.
// The new E of the current and the previous plane live in two shared-memory
// slots of (TY+1) rows x (Zc+1) cells; a thread's H update reads the new E of
// its own cells at plane p from its registers, so one barrier per plane
// suffices.
//
// The per-cell arithmetic is the two-pass kernels' (thread_E / thread_H), so
// every bit of the result is the same.  A periodic boundary along x
// registered after the PML slabs (E[0] = E[nx-1] after the E half,
// H[nx-1] = H[0] after the H half) is supported: the CTAs of the first chunk
// recompute the new E of plane nx-1 (prologue) and use it as plane 0, and the
// H copy runs as a small kernel after the pass.  Waits are bounded like the
// staged kernels' (status bit 0, bit 1 for an expired drain).
#pragma once

#include "fdtd_tma.cuh"

namespace fdtd {

constexpr int ONE_LOAD = 0;   // stage only provides the x neighbour of the next plane
constexpr int ONE_PRO = 1;    // periodic prologue: new E of plane nx-1, not stored
constexpr int ONE_FULL = 2;   // own plane: new E stored, new H of this plane in the next iteration
constexpr int ONE_EHALO = 3;  // first plane of the next chunk: new E of own cells, not stored

template <class T, int TY, int MATE, int MATH>
struct OneGeom {
    static constexpr int TZ = 32;
    static constexpr int V = sizeof(T) == 4 ? 4 : 2;
    static constexpr int Zc = TZ * V;
    static constexpr int pitchH = 3 * Zc + 8;  // values per H tile row
    static constexpr int pitchE = 3 * Zc + 4;  // values per E tile row
    static constexpr int pitchO = 3 * Zc;      // values per own-cell row
    static constexpr int idxE = Zc + 16;       // bytes per E index row
    static constexpr int al(int v) { return (v + 127) & ~127; }
    static constexpr int hBytes = (TY + 2) * pitchH * (int)sizeof(T);
    static constexpr int eBytes = (TY + 1) * pitchE * (int)sizeof(T);
    static constexpr int meBytes = MATE == MAT_FULL ? eBytes : (MATE == MAT_IDS ? (TY + 1) * idxE : 0);
    static constexpr int mhBytes = MATH == MAT_FULL ? TY * pitchO * (int)sizeof(T) : (MATH == MAT_IDS ? TY * Zc : 0);
    static constexpr int eOff = al(hBytes);
    static constexpr int meOff = eOff + al(eBytes);
    static constexpr int mhOff = meOff + al(meBytes);
    static constexpr int fieldBytes = mhOff + al(mhBytes);
    // new-E exchange slot: TY+1 rows x (Zc+1) cells, rows padded to 16 bytes
    static constexpr int xPitch = 3 * (Zc + 4);
    static constexpr int xBytes = al((TY + 1) * xPitch * (int)sizeof(T));
    __host__ __device__ static constexpr uint32_t tx(int role) {
        return (uint32_t)(hBytes + (role == ONE_LOAD ? 0 : eBytes + meBytes) + (role == ONE_FULL ? mhBytes : 0));
    }
};

// Sequence of planes a CTA stages: plane and role of sequence entry r.
struct OneSeq {
    int xa, xb, nx, first, n;
    bool pro;
    __device__ __forceinline__ OneSeq(int xa_, int xb_, int nx_, bool periodic) : xa(xa_), xb(xb_), nx(nx_) {
        pro = periodic && xa == 0;
        first = pro ? 2 : (xa > 0 ? 1 : 0);
        n = first + (xb - xa) + (xb < nx ? 1 : 0);
    }
    __device__ __forceinline__ int plane(int r) const {
        if (r < first) return pro ? nx - 2 + r : xa - 1;
        return xa + (r - first);
    }
    __device__ __forceinline__ int role(int r) const {
        if (r < first) return (pro && r == 1) ? ONE_PRO : ONE_LOAD;
        return xa + (r - first) < xb ? ONE_FULL : ONE_EHALO;
    }
};

// One PML auxiliary row copy of a stage: q enumerates (E side: slab, row of
// TY+1; then H side: slab, row of TY).  Returns the bytes (0: nothing to copy).
template <class T, int TY>
__device__ __forceinline__ uint32_t one_psi_row(const GridK &g, unsigned char *st, int q, int nE, int p, int k0c,
                                                int j0, int Zc, const T **src, uint32_t *dst) {
    const bool is_e = q < nE;
    const int rows = is_e ? TY + 1 : TY;
    const int qq = is_e ? q : q - nE;
    const int s = qq / rows, rr = qq - s * rows;
    const int j = j0 + rr;
    if (j >= g.ny) return 0;
    const SlabK &S = g.slab[s];
    const T *psi = (const T *)(is_e ? S.psiE_rd : S.psiH_rd);
    size_t off;
    uint32_t nb;
    if (S.axis != 2) {
        const int l = (S.axis == 0 ? p : j) - S.start;
        if ((unsigned)l >= (unsigned)S.th) return 0;
        // the E side also holds the pair of the z-halo cell (two pairs: 16 bytes)
        const int cells = min(is_e ? Zc + 2 : Zc, g.nz - k0c);
        off = S.axis == 0 ? (((size_t)l * g.ny + j) * g.nz + k0c) * 2 : (((size_t)p * S.th + l) * g.nz + k0c) * 2;
        nb = (uint32_t)(2 * cells * sizeof(T));
    } else {
        const int kend = k0c + (is_e ? Zc + 1 : Zc);
        if (k0c >= S.start + S.th || kend <= S.start) return 0;
        off = ((size_t)p * g.ny + j) * S.thp * 2;
        nb = (uint32_t)(2 * S.thp * sizeof(T));
    }
    *src = psi + off;
    *dst = smem_u32(st + (is_e ? g.psi_off[s] : g.psi_offH[s]) +
                    (size_t)rr * (is_e ? g.psi_pitch[s] : g.psi_pitchH[s]) * sizeof(T));
    return nb;
}

// Fill the stage of plane p for a role (one warp, all lanes).
template <class T, int TY, int MATE, int MATH>
__device__ __forceinline__ void one_fill(const GridK &g, unsigned char *st, uint32_t bar, int p, int role, int k0c,
                                         int j0, const CUtensorMap *tmH, const CUtensorMap *tmE,
                                         const CUtensorMap *tmME, const CUtensorMap *tmMH) {
    using G = OneGeom<T, TY, MATE, MATH>;
    const int lane = threadIdx.x;
    const int nE = role != ONE_LOAD ? g.nslab * (TY + 1) : 0;
    const int nH = role == ONE_FULL ? g.nslab * TY : 0;
    uint32_t bytes = 0;
    for (int q = lane; q < nE + nH; q += 32) {
        const T *src;
        uint32_t dst;
        bytes += one_psi_row<T, TY>(g, st, q, nE, p, k0c, j0, G::Zc, &src, &dst);
    }
    const uint32_t tot = __reduce_add_sync(0xffffffffu, bytes);
    if (lane == 0) mbar_expect_tx(bar, G::tx(role) + tot);
    __syncwarp();
    for (int q = lane; q < nE + nH; q += 32) {
        const T *src;
        uint32_t dst;
        const uint32_t nb = one_psi_row<T, TY>(g, st, q, nE, p, k0c, j0, G::Zc, &src, &dst);
        if (nb) bulk_copy_g2s(dst, src, nb, bar);
    }
    if (lane == 0) {
        const int row = p * g.ny + j0;
        const int xH = (3 * k0c - 4) * (int)sizeof(T) / 8, xE = 3 * k0c * (int)sizeof(T) / 8;
        tma_load_2d(smem_u32(st), tmH, xH, row - 1, bar);
        if (role != ONE_LOAD) {
            tma_load_2d(smem_u32(st + G::eOff), tmE, xE, row, bar);
            if (MATE == MAT_FULL) tma_load_2d(smem_u32(st + G::meOff), tmME, xE, row, bar);
            else if (MATE == MAT_IDS) tma_load_2d(smem_u32(st + G::meOff), tmME, k0c, row, bar);
        }
        if (role == ONE_FULL) {
            if (MATH == MAT_FULL) tma_load_2d(smem_u32(st + G::mhOff), tmMH, xE, row, bar);
            else if (MATH == MAT_IDS) tma_load_2d(smem_u32(st + G::mhOff), tmMH, k0c, row, bar);
        }
    }
}

// Inverse material of n cells from a stage tile: values at value offset vo,
// indices at byte offset io, or the uniform row.
template <class T, int N, int MAT>
__device__ __forceinline__ void one_material(T (&m)[3 * N], const unsigned char *tile, int vo, int io, const T *lut) {
    if constexpr (MAT == MAT_FULL) {
        if constexpr (N == 1) {
            const T *v = reinterpret_cast<const T *>(tile) + vo;
            m[0] = v[0];
            m[1] = v[1];
            m[2] = v[2];
        } else {
            ld_vec(m, reinterpret_cast<const T *>(tile) + vo);
        }
    } else if constexpr (MAT == MAT_IDS) {
#pragma unroll
        for (int v = 0; v < N; ++v) lut_row(m + 3 * v, lut + 4 * (int)tile[io + v]);
    } else {
#pragma unroll
        for (int v = 0; v < N; ++v) lut_row(m + 3 * v, lut);
    }
}

template <class T, int N>
__device__ __forceinline__ void ld_any(T (&d)[N], const T *p) {
    if constexpr ((N * sizeof(T)) % 16 == 0) {
        ld_vec(d, p);
    } else {
#pragma unroll
        for (int q = 0; q < N; ++q) d[q] = p[q];
    }
}

template <class T, int N>
__device__ __forceinline__ void st_any(T *p, const T (&s)[N]) {
    if constexpr ((N * sizeof(T)) % 16 == 0) {
        st_vec(p, s);
    } else {
#pragma unroll
        for (int q = 0; q < N; ++q) p[q] = s[q];
    }
}

// New E of N cells (i, j, k..k+N-1) whose values start at cell column c
// (0 .. Zc) of the tile row `row` (0 .. TY), from stage `st` (plane i) and
// `sp` (plane i-1).  store: write the updated PML auxiliaries.
template <class P, int N, int TY, int MATE, int MATH>
__device__ __forceinline__ void one_E_cells(const GridK &g, const double *__restrict__ wave,
                                            const unsigned char *st, const unsigned char *sp, int i, int j, int k,
                                            int row, int c, typename P::T cour, const typename P::T *lutE,
                                            const typename P::T *ctabE, int k0c, int ob0, int ob1, int sb0, int sb1,
                                            unsigned mask_yz, bool store, typename P::T (&e)[3 * N]) {
    using T = typename P::T;
    using G = OneGeom<T, TY, MATE, MATH>;
    const T *Hn = reinterpret_cast<const T *>(st);
    const T *Hp = reinterpret_cast<const T *>(sp);
    const int on = (row + 1) * G::pitchH + 4 + 3 * c;
    alignas(16) T hc[3 * N], hp[3 * N], hj[3 * N], m[3 * N], el[3 * N];
    ld_any(hc, Hn + on);
    ld_any(hp, Hp + on);
    ld_any(hj, Hn + on - G::pitchH);
    ld_any(e, reinterpret_cast<const T *>(st + G::eOff) + row * G::pitchE + 3 * c);
    if constexpr (MATE == MAT_IDS)
        one_material<T, N, MATE>(m, st + G::meOff, 0, row * G::idxE + c, lutE);
    else
        one_material<T, N, MATE>(m, st + G::meOff, row * G::pitchE + 3 * c, 0, lutE);
#pragma unroll
    for (int q = 0; q < 3 * N; ++q) el[q] = T(0);
    const T kx = Hn[on - 3], ky = Hn[on - 2];  // cell k-1 (the prefix at c = 0)
    const PsiSrc<T> src{st, row, k0c, ctabE};
    const unsigned slabs = mask_yz | slab_mask_x(g, i);
    thread_E<P, N>(g, wave, i, j, k, cour, hc, hp, hj, kx, ky, m, e, el, ob0, ob1, sb0, sb1, src, slabs, store);
}

template <class P, int TY, int MATE, int MATH>
__global__ void __launch_bounds__(32 * (TY + 1))
    k_step_onepass(const GridK g, const double *__restrict__ wave, const __grid_constant__ CUtensorMap tmH,
                   const __grid_constant__ CUtensorMap tmE, const __grid_constant__ CUtensorMap tmME,
                   const __grid_constant__ CUtensorMap tmMH) {
    using T = typename P::T;
    using G = OneGeom<T, TY, MATE, MATH>;
    constexpr int V = G::V;
    constexpr int N = 3 * V;
    constexpr int Zc = G::Zc;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ int abort_flag;
    unsigned char *smem = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);
    const int S = g.stages;
    const int SB = g.stage_bytes;
    T *X = reinterpret_cast<T *>(smem + (size_t)S * SB);  // two new-E slots
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + (size_t)S * SB + 2 * G::xBytes);
    T *ctabE = reinterpret_cast<T *>(smem + (size_t)S * SB + 2 * G::xBytes + 8 * (size_t)S);
    T *ctabH = ctabE + g.coef_values;
    T *lutE = reinterpret_cast<T *>((reinterpret_cast<uintptr_t>(ctabH + g.coef_values) + 15) & ~uintptr_t(15));
    T *lutH = lutE + 4 * (MATE == MAT_IDS ? 256 : (MATE == MAT_UNIFORM ? 1 : 0));
    const int tz = threadIdx.x, ty = threadIdx.y, tid = ty * 32 + tz;
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const int k0c = blockIdx.x * Zc, j0 = blockIdx.y * TY;
    const int k0 = k0c + tz * V, j = j0 + ty;
    const int xa = blockIdx.z * g.XC, xb = min(nx, xa + g.XC);
    const OneSeq seq(xa, xb, nx, g.periodic_x != 0);
    const int cta = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
    const T c = courant_of<T>(g);
    T *E = (T *)g.E;
    T *H = (T *)g.H;
    const int ob0 = g.obj_off[cta], ob1 = g.obj_off[cta + 1];
    const int sE0 = g.srcE_off[cta], sE1 = g.srcE_off[cta + 1];
    const int sH0 = g.srcH_off[cta], sH1 = g.srcH_off[cta + 1];
    const bool own = ty < TY;
    const bool act = (j < ny) && (k0 < nz);
    // the halo warp's lane l < TY also computes the z-halo cell of row l
    const int hz_row = tz, hz_j = j0 + tz, hz_k = k0c + Zc;
    const bool hz_act = !own && tz < TY && hz_j < ny && hz_k < nz;
    // slabs along y and z do not change along x: their masks once per thread
    const unsigned mask_yz = slab_mask_yz(g, j, k0, V);
    const unsigned hz_mask_yz = slab_mask_yz(g, hz_j, hz_k, 1);
    // the halo warp, which has no H update, fills the stages
    const bool filler = !own;

    if (tid == 0) {
        abort_flag = 0;
        for (int s = 0; s < S; ++s) mbar_init(smem_u32(&bars[s]), 1);
        fence_mbar_init();
        fence_proxy_async();
    }
    if (g.coef_values) {
        stage_coef_tables<T>(g, ctabE, true);
        stage_coef_tables<T>(g, ctabH, false);
    }
    // material tables: 256 padded rows for an index map (every byte reads
    // inside the table), one row for a uniform material
    if constexpr (MATE != MAT_FULL) stage_material_table<T>(g.mlut_E, g.nlut_E, MATE == MAT_IDS ? 256 : 1, lutE);
    if constexpr (MATH != MAT_FULL) stage_material_table<T>(g.mlut_H, g.nlut_H, MATH == MAT_IDS ? 256 : 1, lutH);
    __syncthreads();
    const T *ctE = g.coef_values ? ctabE : nullptr;
    const T *ctH = g.coef_values ? ctabH : nullptr;

    auto issue = [&](int r) {
        one_fill<T, TY, MATE, MATH>(g, smem + (size_t)(r % S) * SB, smem_u32(&bars[r % S]), seq.plane(r),
                                    seq.role(r), k0c, j0, &tmH, &tmE, &tmME, &tmMH);
    };
    int issued = 0;
    for (; issued < min(S, seq.n); ++issued)
        if (filler) issue(issued);

    alignas(16) T e[N];
#pragma unroll
    for (int q = 0; q < N; ++q) e[q] = T(0);
    int r = 0;
    for (; r <= seq.n; ++r) {
        // r == seq.n: only the H update of the last plane when the chunk ends the grid
        const bool tail = r == seq.n;
        if (tail && seq.role(r - 1) != ONE_FULL) break;
        bool ok = true;
        if (!tail) ok = mbar_wait_bounded(smem_u32(&bars[r % S]), (uint32_t)((r / S) & 1));
        if (!ok) abort_flag = 1;
        const unsigned char *st = smem + (size_t)(r % S) * SB;
        const unsigned char *sp = smem + (size_t)((r + S - 1) % S) * SB;  // stage r-1
        T *Xc = X + (size_t)(r & 1) * (G::xBytes / sizeof(T));
        const T *Xp = X + (size_t)((r + 1) & 1) * (G::xBytes / sizeof(T));
        if (ok && !tail) {
            const int role = seq.role(r), p = seq.plane(r);
            if (role != ONE_LOAD) {
                // ---- new E of plane p ----
                const bool replace = role == ONE_FULL && p == 0 && g.periodic_x;  // E[0] = E[nx-1]
                const bool row_needed = own || role != ONE_EHALO;
                if (act && row_needed && !(replace && !own)) {
                    one_E_cells<P, V, TY, MATE, MATH>(g, wave, st, r > 0 ? sp : st, p, j, k0, ty, tz * V, c, lutE,
                                                      ctE, k0c, ob0, ob1, sE0, sE1, mask_yz,
                                                      own && role == ONE_FULL, e);
                }
                if (replace && act) ld_vec(e, Xp + ty * G::xPitch + 3 * tz * V);
                if (act && row_needed) {
                    st_vec(Xc + ty * G::xPitch + 3 * tz * V, e);
                    if (own && role == ONE_FULL) st_vec(E + 3 * (((size_t)p * ny + j) * nz + k0), e);
                }
                if (hz_act && role != ONE_EHALO) {
                    T e1[3];
                    if (replace) {
                        ld_any(e1, Xp + hz_row * G::xPitch + 3 * Zc);
                    } else {
                        one_E_cells<P, 1, TY, MATE, MATH>(g, wave, st, r > 0 ? sp : st, p, hz_j, hz_k, hz_row, Zc,
                                                          c, lutE, ctE, k0c, ob0, ob1, sE0, sE1, hz_mask_yz, false,
                                                          e1);
                    }
                    st_any(Xc + hz_row * G::xPitch + 3 * Zc, e1);
                }
            }
        }
        // ---- new H of plane seq.plane(r-1) ----
        if (ok && r > 0 && seq.role(r - 1) == ONE_FULL && own && act) {
            const int i = seq.plane(r - 1);
            const T *Hf = reinterpret_cast<const T *>(sp);
            alignas(16) T ec[N], ej[N], h[N], hl[N], m[N];
            ld_vec(ec, Xp + ty * G::xPitch + 3 * tz * V);
            ld_vec(ej, Xp + (ty + 1) * G::xPitch + 3 * tz * V);
            ld_vec(h, Hf + (ty + 1) * G::pitchH + 4 + 3 * tz * V);
            if constexpr (MATH == MAT_IDS)
                one_material<T, V, MATH>(m, sp + G::mhOff, 0, ty * Zc + tz * V, lutH);
            else
                one_material<T, V, MATH>(m, sp + G::mhOff, ty * G::pitchO + 3 * tz * V, 0, lutH);
#pragma unroll
            for (int q = 0; q < N; ++q) hl[q] = T(0);
            const T kx = Xp[ty * G::xPitch + 3 * (tz * V + V)];  // cell k0+V (the z-halo for the last lane)
            const T ky = Xp[ty * G::xPitch + 3 * (tz * V + V) + 1];
            const PsiSrc<T> src{sp, ty, k0c, ctH};
            const unsigned slabs = mask_yz | slab_mask_x(g, i);
            thread_H<P, V, true>(g, wave, i, j, k0, c, ec, e, ej, kx, ky, m, h, hl, sH0, sH1, src, slabs, true);
            st_vec(H + 3 * (((size_t)i * ny + j) * nz + k0), h);
        }
        __syncthreads();
        if (abort_flag) break;
        if (r >= 1 && issued < seq.n) {
            if (filler) {
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
