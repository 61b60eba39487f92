// Kernels of the GB300 FDTD time step.
//
// k_update_E / k_update_H are the fused half steps.  One pass per half step
// does, per cell and in the reference's order (fdtd/grid.py:275-325):
//   PML auxiliary update (fdtd/boundaries.py:433-487, slab-local index rules)
//   Yee curl (fdtd/grid.py:29-76, out-of-grid differences dropped)
//   bulk update E += c*eps^-1*curlH / H -= c*mu^-1*curlE
//   objects in registration order (fdtd/objects.py:118-277)
//   PML corrections in boundary order (fdtd/boundaries.py:409-431)
//   sources in registration order (fdtd/sources.py:93-109,278-297,476-486)
// A CTA covers TZ*V cells along z, TY rows along y and XC planes along x; a
// thread streams along x holding the neighbour plane in registers.
#pragma once

#include "fdtd_cell.cuh"

namespace fdtd {

#define FULL_MASK 0xffffffffu

// Register-streaming kernels: neighbour values come from global memory
// (L1/L2) and from the lane to the left/right; used for shapes the staged
// kernels do not take (nz not a multiple of the vector width, unaligned data).
// One tile of the E half (bx, by, bz: tile coordinates; cta: its index in the
// per-CTA lists), for the one-tile-per-block kernel and the persistent one.
// CG: the other half's field is written by other blocks of the same launch
// (persistent loop), so it is loaded through L2 only, not the read-only path.
template <class P, int V, bool CG = false>
__device__ __forceinline__ void tile_update_E(const GridK &g, const double *__restrict__ wave, int bx, int by, int bz,
                                              int cta) {
    using T = typename P::T;
    constexpr int N = 3 * V;
    const int tz = threadIdx.x, ty = threadIdx.y;
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const int k0 = g.oz + (bx * g.TZ + tz) * V;
    const int j = g.oy + by * g.TY + ty;
    const int xa = g.ox + bz * g.XC;
    const int xb = min(g.ex, xa + g.XC);
    const bool act = (j < g.ey) && (k0 < g.ez);
    const T c = courant_of<T>(g);
    const T *__restrict__ H = (const T *)g.H;
    T *E = (T *)g.E;
    T *Elo = (T *)g.Elo;
    const T *__restrict__ IE = (const T *)g.ie;
    const int ob0 = g.obj_off[cta], ob1 = g.obj_off[cta + 1];
    int sb0 = 0, sb1 = 0;
    if (g.fuse_src_E) {
        sb0 = g.srcE_off[cta];
        sb1 = g.srcE_off[cta + 1];
    }

    const PsiSrc<T> nostage{nullptr, 0, 0, nullptr};
    const unsigned mask_yz = slab_mask_yz(g, j, k0, V);
    alignas(16) T hp[N];  // H at plane i-1
#pragma unroll
    for (int q = 0; q < N; ++q) hp[q] = T(0);
    if (act && xa > 0) ld_field<CG>(hp, H + 3 * (((size_t)(xa - 1) * ny + j) * nz + k0));

    for (int i = xa; i < xb; ++i) {
        const size_t cell0 = ((size_t)i * ny + j) * nz + k0;
        alignas(16) T hc[N], hj[N], e[N], el[N], m[N];
#pragma unroll
        for (int q = 0; q < N; ++q) {
            hc[q] = T(0);
            hj[q] = T(0);
            e[q] = T(0);
            el[q] = T(0);
            m[q] = T(0);
        }
        if (act) {
            ld_field<CG>(hc, H + 3 * cell0);
            if (j > 0) ld_field<CG>(hj, H + 3 * (cell0 - nz));
            ld_vec(e, E + 3 * cell0);
            if constexpr (P::COMP) ld_vec(el, Elo + 3 * cell0);
            ld_vec_ro(m, IE + 3 * cell0);
        }
        // (Hx, Hy) at k0-1: from the lane to the left, or from memory at a row start
        T kx = __shfl_up_sync(FULL_MASK, hc[N - 3], 1);
        T ky = __shfl_up_sync(FULL_MASK, hc[N - 2], 1);
        if (tz == 0 && act && k0 > 0) {
            kx = ld_field1<CG>(H + 3 * (cell0 - 1));
            ky = ld_field1<CG>(H + 3 * (cell0 - 1) + 1);
        }
        if (act) {
            const unsigned slabs = mask_yz | slab_mask_x(g, i);
            thread_E<P, V>(g, wave, i, j, k0, c, hc, hp, hj, kx, ky, m, e, el, ob0, ob1, sb0, sb1, nostage, slabs);
            st_vec(E + 3 * cell0, e);
            if constexpr (P::COMP) st_vec(Elo + 3 * cell0, el);
        }
#pragma unroll
        for (int q = 0; q < N; ++q) hp[q] = hc[q];
    }
}

template <class P, int V>
__global__ void __launch_bounds__(kThreads) k_update_E(const GridK g, const double *__restrict__ wave) {
    tile_update_E<P, V>(g, wave, blockIdx.x, blockIdx.y, blockIdx.z,
                        blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z));
}

template <class P, int V, bool CG = false>
__device__ __forceinline__ void tile_update_H(const GridK &g, const double *__restrict__ wave, int bx, int by, int bz,
                                              int cta) {
    using T = typename P::T;
    constexpr int N = 3 * V;
    const int tz = threadIdx.x, ty = threadIdx.y;
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const int k0 = g.oz + (bx * g.TZ + tz) * V;
    const int j = g.oy + by * g.TY + ty;
    const int xa = g.ox + bz * g.XC;
    const int xb = min(g.ex, xa + g.XC);
    const bool act = (j < g.ey) && (k0 < g.ez);
    const T c = courant_of<T>(g);
    const T *__restrict__ E = (const T *)g.E;
    T *H = (T *)g.H;
    T *Hlo = (T *)g.Hlo;
    const T *__restrict__ MU = (const T *)g.imu;
    int sb0 = 0, sb1 = 0;
    if (g.fuse_src_H) {
        sb0 = g.srcH_off[cta];
        sb1 = g.srcH_off[cta + 1];
    }

    const PsiSrc<T> nostage{nullptr, 0, 0, nullptr};
    const unsigned mask_yz = slab_mask_yz(g, j, k0, V);
    alignas(16) T ec[N];  // E at plane i
#pragma unroll
    for (int q = 0; q < N; ++q) ec[q] = T(0);
    if (act && xa < xb) ld_field<CG>(ec, E + 3 * (((size_t)xa * ny + j) * nz + k0));

    for (int i = xa; i < xb; ++i) {
        const size_t cell0 = ((size_t)i * ny + j) * nz + k0;
        alignas(16) T en[N], ej[N], h[N], hl[N], m[N];
#pragma unroll
        for (int q = 0; q < N; ++q) {
            en[q] = T(0);
            ej[q] = T(0);
            h[q] = T(0);
            hl[q] = T(0);
            m[q] = T(0);
        }
        if (act) {
            if (i + 1 < nx) ld_field<CG>(en, E + 3 * (cell0 + (size_t)ny * nz));
            if (j + 1 < ny) ld_field<CG>(ej, E + 3 * (cell0 + nz));
            ld_vec(h, H + 3 * cell0);
            if constexpr (P::COMP) ld_vec(hl, Hlo + 3 * cell0);
            ld_vec_ro(m, MU + 3 * cell0);
        }
        // (Ex, Ey) at k0+V: from the lane to the right, or from memory at a row end
        T kx = __shfl_down_sync(FULL_MASK, ec[0], 1);
        T ky = __shfl_down_sync(FULL_MASK, ec[1], 1);
        // (the last lane of the tile, or the last of the box when the box ends inside the tile)
        if ((tz == g.TZ - 1 || k0 + V >= g.ez) && act && k0 + V < nz) {
            kx = ld_field1<CG>(E + 3 * (cell0 + V));
            ky = ld_field1<CG>(E + 3 * (cell0 + V) + 1);
        }
        if (act) {
            const unsigned slabs = mask_yz | slab_mask_x(g, i);
            thread_H<P, V>(g, wave, i, j, k0, c, ec, en, ej, kx, ky, m, h, hl, sb0, sb1, nostage, slabs);
            st_vec(H + 3 * cell0, h);
            if constexpr (P::COMP) st_vec(Hlo + 3 * cell0, hl);
        }
#pragma unroll
        for (int q = 0; q < N; ++q) ec[q] = en[q];
    }
}

template <class P, int V>
__global__ void __launch_bounds__(kThreads) k_update_H(const GridK g, const double *__restrict__ wave) {
    tile_update_H<P, V>(g, wave, blockIdx.x, blockIdx.y, blockIdx.z,
                        blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z));
}

// ---------------------------------------------------------------------------
// Shell boxes of an interior/shell partition: one thread per cell, the whole
// per-cell half step (bulk, objects, every PML slab in order, sources) with
// the neighbour values read through L1/L2, and the compact material copy
// when the plan has one.  Each cell is read and written once; the slab-free
// staged pass covers the interior.
// ---------------------------------------------------------------------------

// Loads and stores of a thread's V cells: 16-byte accesses where the run's
// size allows, else 8-byte ones (float pairs: a run of 3V floats starting at
// an even cell is 8-byte aligned), else single values.
template <bool RO, class T, int N>
__device__ __forceinline__ void shell_ld(T (&dst)[N], const T *p) {
    if constexpr ((N * sizeof(T)) % 16 == 0) {
        if constexpr (RO) ld_vec_ro(dst, p);
        else ld_vec(dst, p);
    } else if constexpr ((N * sizeof(T)) % 8 == 0) {
        const uint2 *q = reinterpret_cast<const uint2 *>(p);
#pragma unroll
        for (int i = 0; i < (int)(N * sizeof(T) / 8); ++i) {
            const uint2 t = RO ? __ldg(q + i) : q[i];
            *reinterpret_cast<uint2 *>(&dst[i * 8 / sizeof(T)]) = t;
        }
    } else {
#pragma unroll
        for (int i = 0; i < N; ++i) dst[i] = RO ? __ldg(p + i) : p[i];
    }
}

template <class T, int N>
__device__ __forceinline__ void shell_st(T *p, const T (&src)[N]) {
    if constexpr ((N * sizeof(T)) % 16 == 0) {
        st_vec(p, src);
    } else if constexpr ((N * sizeof(T)) % 8 == 0) {
        uint2 *q = reinterpret_cast<uint2 *>(p);
#pragma unroll
        for (int i = 0; i < (int)(N * sizeof(T) / 8); ++i) q[i] = *reinterpret_cast<const uint2 *>(&src[i * 8 / sizeof(T)]);
    } else {
#pragma unroll
        for (int i = 0; i < N; ++i) p[i] = src[i];
    }
}

// The V cells (k0 .. k0+V-1 along z) of this thread: false past the end of
// its box (box z extents and origins are multiples of V).
template <int V>
__device__ __forceinline__ bool shell_cells(const ShellK &sh, int &i, int &j, int &k0, unsigned &slabs) {
    int b = 0;
    while (b + 1 < sh.nbox && blockIdx.x >= sh.first[b + 1]) ++b;
    const unsigned local = (blockIdx.x - sh.first[b]) * blockDim.x + threadIdx.x;
    const unsigned nzv = (unsigned)(sh.n[b][2] / V), ny = (unsigned)sh.n[b][1];
    if (local >= (unsigned)sh.n[b][0] * ny * nzv) return false;
    const unsigned r = div_magic(local, sh.mz[b], sh.sz[b]);
    const unsigned x = div_magic(r, sh.my[b], sh.sy[b]);
    k0 = sh.o[b][2] + V * (int)(local - r * nzv);
    j = sh.o[b][1] + (int)(r - x * ny);
    i = sh.o[b][0] + (int)x;
    slabs = sh.slabs[b];
    return true;
}

// The slabs among `cand` that contain cells of this thread (the slab mask of
// the other kernels, tested only against the slabs that reach the box).
template <int V>
__device__ __forceinline__ unsigned shell_mask(const GridK &g, unsigned cand, int i, int j, int k0) {
    unsigned m = 0;
    for (unsigned sm = cand; sm; sm &= sm - 1) {
        const int s = __ffs(sm) - 1;
        const SlabK &S = g.slab[s];
        const int c = S.axis == 0 ? i : (S.axis == 1 ? j : k0);
        const int w = S.axis == 2 ? V : 1;
        if (c < S.start + S.th && c + w > S.start) m |= 1u << s;
    }
    return m;
}

// Inverse material of V cells: the values, table rows by index, or the one row.
template <class T, int V>
__device__ __forceinline__ void shell_material(T (&m)[3 * V], int mat, const T *full, const unsigned char *mid,
                                               const T *lut, int nlut, size_t cell0) {
    if (mat == MAT_FULL) {
        shell_ld<true>(m, full + 3 * cell0);
    } else {
#pragma unroll
        for (int v = 0; v < V; ++v) {
            // an index past the table reads zeros, as in the staged passes
            const int id = mat == MAT_IDS ? (int)mid[cell0 + v] : 0;
#pragma unroll
            for (int q = 0; q < 3; ++q) m[3 * v + q] = id < nlut ? lut[3 * id + q] : T(0);
        }
    }
}

template <class P, int V>
__global__ void __launch_bounds__(kThreads) k_shell_E(const GridK g, const ShellK sh, const double *__restrict__ wave) {
    using T = typename P::T;
    constexpr int N = 3 * V;
    int i, j, k0;
    unsigned cand;
    if (!shell_cells<V>(sh, i, j, k0, cand)) return;
    const int ny = g.ny, nz = g.nz;
    const size_t cell0 = ((size_t)i * ny + j) * nz + k0;
    const T *__restrict__ H = (const T *)g.H;
    T *E = (T *)g.E;
    T *Elo = (T *)g.Elo;
    alignas(16) T hc[N], hp[N], hj[N], e[N], el[N], m[N];
#pragma unroll
    for (int q = 0; q < N; ++q) {
        hp[q] = T(0);
        hj[q] = T(0);
        el[q] = T(0);
    }
    shell_ld<true>(hc, H + 3 * cell0);
    if (i > 0) shell_ld<true>(hp, H + 3 * (cell0 - (size_t)ny * nz));
    if (j > 0) shell_ld<true>(hj, H + 3 * (cell0 - nz));
    shell_ld<false>(e, E + 3 * cell0);
    if constexpr (P::COMP) shell_ld<false>(el, Elo + 3 * cell0);
    const T kx = k0 > 0 ? H[3 * (cell0 - 1)] : T(0), ky = k0 > 0 ? H[3 * (cell0 - 1) + 1] : T(0);
    shell_material<T, V>(m, g.mat_E, (const T *)g.ie, g.mid_E, (const T *)g.mlut_E, g.nlut_E, cell0);
    const int cta = blockIdx.x;
    const int ob0 = g.obj_off[cta], ob1 = g.obj_off[cta + 1];
    int sb0 = 0, sb1 = 0;
    if (g.fuse_src_E) {
        sb0 = g.srcE_off[cta];
        sb1 = g.srcE_off[cta + 1];
    }
    const PsiSrc<T> nostage{nullptr, 0, 0, nullptr};
    const unsigned slabs = shell_mask<V>(g, cand, i, j, k0);
    thread_E<P, V>(g, wave, i, j, k0, courant_of<T>(g), hc, hp, hj, kx, ky, m, e, el, ob0, ob1, sb0, sb1, nostage,
                   slabs);
    shell_st(E + 3 * cell0, e);
    if constexpr (P::COMP) shell_st(Elo + 3 * cell0, el);
}

template <class P, int V>
__global__ void __launch_bounds__(kThreads) k_shell_H(const GridK g, const ShellK sh, const double *__restrict__ wave) {
    using T = typename P::T;
    constexpr int N = 3 * V;
    int i, j, k0;
    unsigned cand;
    if (!shell_cells<V>(sh, i, j, k0, cand)) return;
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const size_t cell0 = ((size_t)i * ny + j) * nz + k0;
    const T *__restrict__ E = (const T *)g.E;
    T *H = (T *)g.H;
    T *Hlo = (T *)g.Hlo;
    alignas(16) T ec[N], en[N], ej[N], h[N], hl[N], m[N];
#pragma unroll
    for (int q = 0; q < N; ++q) {
        en[q] = T(0);
        ej[q] = T(0);
        hl[q] = T(0);
    }
    shell_ld<true>(ec, E + 3 * cell0);
    if (i + 1 < nx) shell_ld<true>(en, E + 3 * (cell0 + (size_t)ny * nz));
    if (j + 1 < ny) shell_ld<true>(ej, E + 3 * (cell0 + nz));
    shell_ld<false>(h, H + 3 * cell0);
    if constexpr (P::COMP) shell_ld<false>(hl, Hlo + 3 * cell0);
    const bool kn = k0 + V < nz;
    const T kx = kn ? E[3 * (cell0 + V)] : T(0), ky = kn ? E[3 * (cell0 + V) + 1] : T(0);
    shell_material<T, V>(m, g.mat_H, (const T *)g.imu, g.mid_H, (const T *)g.mlut_H, g.nlut_H, cell0);
    const int cta = blockIdx.x;
    int sb0 = 0, sb1 = 0;
    if (g.fuse_src_H) {
        sb0 = g.srcH_off[cta];
        sb1 = g.srcH_off[cta + 1];
    }
    const PsiSrc<T> nostage{nullptr, 0, 0, nullptr};
    const unsigned slabs = shell_mask<V>(g, cand, i, j, k0);
    thread_H<P, V>(g, wave, i, j, k0, courant_of<T>(g), ec, en, ej, kx, ky, m, h, hl, sb0, sb1, nostage, slabs);
    shell_st(H + 3 * cell0, h);
    if constexpr (P::COMP) shell_st(Hlo + 3 * cell0, hl);
}

// ---------------------------------------------------------------------------
// Small kernels used when a periodic boundary fixes the order of the stages
// after the fused pass, plus detectors, DFT, stand-alone curls and stats.
// ---------------------------------------------------------------------------

// Periodic plane copy (fdtd/boundaries.py:184-219): F[plane dst] = F[plane src].
template <class T, bool COMP>
__global__ void k_plane_copy(T *F, T *Flo, int nx, int ny, int nz, int axis, int dst, int src) {
    const int n1 = axis == 0 ? ny : nx;
    const int n2 = axis == 2 ? ny : nz;
    const long total = (long)n1 * n2 * 3;
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
        const int comp = (int)(t % 3);
        const long pc = t / 3;
        const int a = (int)(pc / n2), b = (int)(pc % n2);
        size_t cd, cs;
        if (axis == 0) {
            cd = ((size_t)dst * ny + a) * nz + b;
            cs = ((size_t)src * ny + a) * nz + b;
        } else if (axis == 1) {
            cd = ((size_t)a * ny + dst) * nz + b;
            cs = ((size_t)a * ny + src) * nz + b;
        } else {
            cd = ((size_t)a * ny + b) * nz + dst;
            cs = ((size_t)a * ny + b) * nz + src;
        }
        F[3 * cd + comp] = F[3 * cs + comp];
        if constexpr (COMP) Flo[3 * cd + comp] = Flo[3 * cs + comp];
    }
}

// PML correction of one slab on its own (boundary after a periodic boundary).
template <class P, bool IS_E>
__global__ void k_slab_correct(const GridK g, int s) {
    using T = typename P::T;
    const SlabK &S = g.slab[s];
    const int a = S.axis;
    const int n0 = a == 0 ? S.th : g.nx, n1 = a == 1 ? S.th : g.ny, n2 = a == 2 ? S.th : g.nz;
    const int p2 = a == 2 ? S.thp : g.nz;  // stored extent of the last axis
    const long total = (long)n0 * n1 * n2;
    const T c = courant_of<T>(g);
    T *F = (T *)(IS_E ? g.E : g.H);
    T *Flo = (T *)(IS_E ? g.Elo : g.Hlo);
    const T *M = (const T *)(IS_E ? g.ie : g.imu);
    const T *psi = (const T *)(IS_E ? S.psiE : S.psiH);
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
        const int i0 = (int)(t / ((long)n1 * n2)), i1 = (int)((t / n2) % n1), i2 = (int)(t % n2);
        const int gi = a == 0 ? i0 + S.start : i0, gj = a == 1 ? i1 + S.start : i1, gk = a == 2 ? i2 + S.start : i2;
        const size_t cell = ((size_t)gi * g.ny + gj) * g.nz + gk;
        const size_t pt = ((size_t)i0 * n1 + i1) * p2 + i2;
        const T p0 = psi[2 * pt], p1 = psi[2 * pt + 1];
        const int t1 = (a + 1) % 3, t2 = (a + 2) % 3;
        T x1 = F[3 * cell + t1], x2 = F[3 * cell + t2];
        T l1 = T(0), l2 = T(0);
        if constexpr (P::COMP) {
            l1 = Flo[3 * cell + t1];
            l2 = Flo[3 * cell + t2];
        }
        const T c1 = P::cm(c, M[3 * cell + t1]), c2 = P::cm(c, M[3 * cell + t2]);
        if (IS_E) {
            P::add_prod(x1, l1, c1, -p0);
            P::add_prod(x2, l2, c2, p1);
        } else {
            P::sub_prod(x1, l1, c1, -p0);
            P::sub_prod(x2, l2, c2, p1);
        }
        P::finish(x1, l1);
        P::finish(x2, l2);
        F[3 * cell + t1] = x1;
        F[3 * cell + t2] = x2;
        if constexpr (P::COMP) {
            Flo[3 * cell + t1] = l1;
            Flo[3 * cell + t2] = l2;
        }
    }
}

// One PML slab on its own (slabs outside the fused pass): the auxiliary
// update of fdtd/boundaries.py:433-487 with the slab-local index rules, then
// the correction of fdtd/boundaries.py:409-431, per slab cell and with the
// same per-cell arithmetic as the fused pass.  The neighbour field is not
// written during the half step, so its differences can be read here.  The
// slab normal A is a template parameter and the cell index type I is 32-bit
// whenever the slab has fewer than 2^31 cells (no 64-bit divisions); all
// buffers are distinct, so every load of a cell can issue up front.
template <class P, bool IS_E, int A, class I>
__global__ void __launch_bounds__(kThreads) k_pml_slab(const GridK g, int s) {
    using T = typename P::T;
    const SlabK &S = g.slab[s];
    const int n1 = A == 1 ? S.th : g.ny, n2 = A == 2 ? S.th : g.nz;
    const int p2 = A == 2 ? S.thp : g.nz;
    const I total = (I)(A == 0 ? S.th : g.nx) * (I)n1 * (I)n2;
    const T c = courant_of<T>(g);
    T *__restrict__ F = (T *)(IS_E ? g.E : g.H);
    T *__restrict__ Flo = (T *)(IS_E ? g.Elo : g.Hlo);
    const T *__restrict__ N = (const T *)(IS_E ? g.H : g.E);  // neighbour field
    const T *__restrict__ M = (const T *)(IS_E ? g.ie : g.imu);
    T *__restrict__ psi = (T *)(IS_E ? S.psiE : S.psiH);
    const T *__restrict__ bt = (const T *)(IS_E ? S.bE : S.bH);
    const T *__restrict__ ct = (const T *)(IS_E ? S.cE : S.cH);
    // materials: through the staged passes' compact copy when the plan has one
    const int mat = IS_E ? g.mat_E : g.mat_H;
    const T *__restrict__ lut = (const T *)(IS_E ? g.mlut_E : g.mlut_H);
    const unsigned char *__restrict__ mid = IS_E ? g.mid_E : g.mid_H;
    const int nlut = IS_E ? g.nlut_E : g.nlut_H;
    constexpr int t1 = (A + 1) % 3, t2 = (A + 2) % 3;
    const size_t stride = A == 0 ? 3 * (size_t)g.ny * g.nz : (A == 1 ? 3 * (size_t)g.nz : 3);
    for (I t = (I)blockIdx.x * (I)blockDim.x + threadIdx.x; t < total; t += (I)gridDim.x * (I)blockDim.x) {
        const I r = t / (I)n2;
        const int i2 = (int)(t - r * (I)n2), i1 = (int)(r % (I)n1), i0 = (int)(r / (I)n1);
        const int l = A == 0 ? i0 : (A == 1 ? i1 : i2);
        const int gi = A == 0 ? i0 + S.start : i0, gj = A == 1 ? i1 + S.start : i1, gk = A == 2 ? i2 + S.start : i2;
        const size_t cell = ((size_t)gi * g.ny + gj) * g.nz + gk;
        const size_t at = 3 * cell;
        const size_t pt = 2 * (((size_t)i0 * n1 + i1) * p2 + i2);
        T p0 = psi[pt], p1 = psi[pt + 1];
        T x1 = F[at + t1], x2 = F[at + t2];
        T m1, m2;
        if (mat == MAT_FULL) {
            m1 = M[at + t1];
            m2 = M[at + t2];
        } else {
            // a table row; an index past the table reads zeros, as in the staged passes
            const int id = mat == MAT_IDS ? (int)mid[cell] : 0;
            m1 = id < nlut ? lut[3 * id + t1] : T(0);
            m2 = id < nlut ? lut[3 * id + t2] : T(0);
        }
        T l1 = T(0), l2 = T(0);
        if constexpr (P::COMP) {
            l1 = Flo[at + t1];
            l2 = Flo[at + t2];
        }
        const T b = bt[l], cc = ct[l];
        if (IS_E ? (l >= 1) : (l <= S.th - 2)) {
            // E: backward difference of H along the normal; H: forward difference of E
            const T d0 = IS_E ? N[at + t2] - N[at - stride + t2] : N[at + stride + t2] - N[at + t2];
            const T d1 = IS_E ? N[at + t1] - N[at - stride + t1] : N[at + stride + t1] - N[at + t1];
            p0 = P::psi(p0, b, d0, cc);
            p1 = P::psi(p1, b, d1, cc);
        } else {
            p0 = P::mul(p0, b);
            p1 = P::mul(p1, b);
        }
        psi[pt] = p0;
        psi[pt + 1] = p1;
        pml_correct<P, IS_E>(x1, l1, P::cm(c, m1), -p0);
        pml_correct<P, IS_E>(x2, l2, P::cm(c, m2), p1);
        P::finish(x1, l1);
        P::finish(x2, l2);
        F[at + t1] = x1;
        F[at + t2] = x2;
        if constexpr (P::COMP) {
            Flo[at + t1] = l1;
            Flo[at + t2] = l2;
        }
    }
}

// Soft source points applied on their own: one thread per run of items that
// share a cell, applied in order (a LineSource may list a cell twice).
template <class P>
__global__ void k_soft_runs(const GridK g, const int2 *runs, int nruns, const double *wave, int field) {
    using T = typename P::T;
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nruns) return;
    T *F = (T *)(field == 0 ? g.E : g.H);
    T *Flo = (T *)(field == 0 ? g.Elo : g.Hlo);
    const int2 run = runs[r];
    const ItemK &first = g.items[run.x];
    const size_t cell = ((size_t)first.lo[0] * g.ny + first.lo[1]) * g.nz + first.lo[2];
    const size_t at = 3 * cell + first.comp;
    T x = F[at];
    T lo = T(0);
    if constexpr (P::COMP) lo = Flo[at];
    for (int q = 0; q < run.y; ++q) {
        const ItemK &s = g.items[run.x + q];
        P::add_prod(x, lo, (T)s.weight, (T)wave[s.column]);
    }
    P::finish(x, lo);
    F[at] = x;
    if constexpr (P::COMP) Flo[at] = lo;
}

// Hard source box applied on its own (PlaneSource.update_E/H).
template <class P>
__global__ void k_hard_box(const GridK g, int item, const double *wave, int field) {
    using T = typename P::T;
    const ItemK &s = g.items[item];
    const int b0 = s.hi[0] - s.lo[0], b1 = s.hi[1] - s.lo[1], b2 = s.hi[2] - s.lo[2];
    const long total = (long)b0 * b1 * b2;
    T *F = (T *)(field == 0 ? g.E : g.H);
    T *Flo = (T *)(field == 0 ? g.Elo : g.Hlo);
    const T val = P::mul((T)s.weight, (T)wave[s.column]);
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
        const int i = s.lo[0] + (int)(t / ((long)b1 * b2)), j = s.lo[1] + (int)((t / b2) % b1),
                  k = s.lo[2] + (int)(t % b2);
        const size_t at = 3 * (((size_t)i * g.ny + j) * g.nz + k) + s.comp;
        F[at] = val;
        if constexpr (P::COMP) Flo[at] = T(0);
    }
}

// Feedback source (SoftArbitraryPointSource.update_E, fdtd/sources.py:600-629):
// output = input + impedance * I_prev (only for impedance > 0), then
// E[comp] += output / grid_spacing; I_prev is the source's current-probe point
// after the previous H half, 0 at step 0 (iprev = null).
template <class P>
__global__ void k_feedback(const GridK g, int item, const double *wave, const typename P::T *iprev, double du) {
    using T = typename P::T;
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    const ItemK &s = g.items[item];
    T *E = (T *)g.E;
    T *Elo = (T *)g.Elo;
    const size_t at = 3 * (((size_t)s.lo[0] * g.ny + s.lo[1]) * g.nz + s.lo[2]) + s.comp;
    const T in = (T)wave[s.column];
    const T cur = iprev ? iprev[s.aux] : T(0);
    T out = in;
    if (s.weight > 0.0) {
        if constexpr (sizeof(T) == 8) out = __dadd_rn(in, __dmul_rn((T)s.weight, cur));
        else out = in + (T)s.weight * cur;
    }
    T v;
    if constexpr (sizeof(T) == 8) v = __ddiv_rn(out, (T)du);
    else v = out / (T)du;
    T x = E[at], lo = T(0);
    if constexpr (P::COMP) lo = Elo[at];
    P::add_prod(x, lo, v, T(1));
    P::finish(x, lo);
    E[at] = x;
    if constexpr (P::COMP) Elo[at] = lo;
}

// Current probes (CurrentDetector.single_point_current, fdtd/detectors.py:404-464):
// out[p] = I at cells[p] from H, with the reference's arithmetic order, its
// running accumulation of the second y term, and negative neighbour indices
// wrapping to the far side of the grid as Python indexing does.
template <class T>
__global__ void k_current(const T *__restrict__ H, const int64_t *__restrict__ cells, int n, int nx, int ny, int nz,
                          double du_d, T *out) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const long c = cells[p];
    const int px = (int)(c / ((long)ny * nz)), py = (int)((c / nz) % ny), pz = (int)(c % nz);
    const int xm = px > 0 ? px - 1 : nx - 1, ym = py > 0 ? py - 1 : ny - 1, zm = pz > 0 ? pz - 1 : nz - 1;
    auto h = [&](int i, int j, int k, int comp) { return H[3 * (((size_t)i * ny + j) * nz + k) + comp]; };
    const T du = (T)du_d;
    T cur1, cur2;
    if constexpr (sizeof(T) == 8) {
        double cv1 = __dmul_rn(__dsub_rn(h(px, ym, pz, 0), h(px, py, pz, 0)), du);
        double cv2 = __dmul_rn(__dsub_rn(h(px, py, pz, 1), h(xm, py, pz, 1)), du);
        cur1 = __dadd_rn(cv1, cv2);
        cv1 = __dmul_rn(__dsub_rn(h(px, ym, zm, 0), h(px, py, zm, 0)), du);
        cv2 = __dadd_rn(cv2, __dmul_rn(__dsub_rn(h(px, py, zm, 1), h(xm, py, zm, 1)), du));
        cur2 = __dadd_rn(cv1, cv2);
        out[p] = __ddiv_rn(__dadd_rn(cur1, cur2), 2.0);
    } else {
        T cv1 = (h(px, ym, pz, 0) - h(px, py, pz, 0)) * du;
        T cv2 = (h(px, py, pz, 1) - h(xm, py, pz, 1)) * du;
        cur1 = cv1 + cv2;
        cv1 = (h(px, ym, zm, 0) - h(px, py, zm, 0)) * du;
        cv2 = cv2 + (h(px, py, zm, 1) - h(xm, py, zm, 1)) * du;
        cur2 = cv1 + cv2;
        out[p] = (cur1 + cur2) / T(2);
    }
}

// Detector sampling: out[p][c] = F[cells[p]][c].
template <class T>
__global__ void k_probe(const T *__restrict__ F, const int64_t *__restrict__ cells, int n, T *out) {
    const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (t >= 3L * n) return;
    const long p = t / 3;
    const int comp = (int)(t % 3);
    out[t] = F[3 * cells[p] + comp];
}

// Running DFT of E on a box, accumulated in double.
template <class T, bool COMP>
__global__ void k_dft(const T *__restrict__ E, const T *__restrict__ Elo, int ny, int nz, fdtd_dft_desc d,
                      const double *__restrict__ phase) {
    const int b0 = d.hi[0] - d.lo[0], b1 = d.hi[1] - d.lo[1], b2 = d.hi[2] - d.lo[2];
    const long ncell = (long)b0 * b1 * b2;
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < ncell * 3; t += (long)gridDim.x * blockDim.x) {
        const long cell = t / 3;
        const int comp = (int)(t % 3);
        const int i = d.lo[0] + (int)(cell / ((long)b1 * b2)), j = d.lo[1] + (int)((cell / b2) % b1),
                  k = d.lo[2] + (int)(cell % b2);
        const size_t at = 3 * (((size_t)i * ny + j) * nz + k) + comp;
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

// Stand-alone curls, one thread per cell (fdtd/grid.py:29-76).
template <class T>
__global__ void k_curl_E(const T *__restrict__ E, T *out, int nx, int ny, int nz) {
    const long n = (long)nx * ny * nz;
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
        const int i = (int)(t / ((long)ny * nz)), j = (int)((t / nz) % ny), k = (int)(t % nz);
        const T *e = E + 3 * t;
        const T dxEy = i < nx - 1 ? e[3L * ny * nz + 1] - e[1] : T(0);
        const T dxEz = i < nx - 1 ? e[3L * ny * nz + 2] - e[2] : T(0);
        const T dyEx = j < ny - 1 ? e[3L * nz] - e[0] : T(0);
        const T dyEz = j < ny - 1 ? e[3L * nz + 2] - e[2] : T(0);
        const T dzEx = k < nz - 1 ? e[3] - e[0] : T(0);
        const T dzEy = k < nz - 1 ? e[4] - e[1] : T(0);
        out[3 * t] = dyEz - dzEy;
        out[3 * t + 1] = dzEx - dxEz;
        out[3 * t + 2] = dxEy - dyEx;
    }
}

template <class T>
__global__ void k_curl_H(const T *__restrict__ H, T *out, int nx, int ny, int nz) {
    const long n = (long)nx * ny * nz;
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
        const int i = (int)(t / ((long)ny * nz)), j = (int)((t / nz) % ny), k = (int)(t % nz);
        const T *h = H + 3 * t;
        const T dxHy = i > 0 ? h[1] - h[1 - 3L * ny * nz] : T(0);
        const T dxHz = i > 0 ? h[2] - h[2 - 3L * ny * nz] : T(0);
        const T dyHx = j > 0 ? h[0] - h[-3L * nz] : T(0);
        const T dyHz = j > 0 ? h[2] - h[2 - 3L * nz] : T(0);
        const T dzHx = k > 0 ? h[0] - h[-3] : T(0);
        const T dzHy = k > 0 ? h[1] - h[-2] : T(0);
        out[3 * t] = dyHz - dzHy;
        out[3 * t + 1] = dzHx - dxHz;
        out[3 * t + 2] = dxHy - dyHx;
    }
}

// Field statistics, first pass: one partial row of 5 doubles per CTA.
template <class T, bool COMP>
__global__ void __launch_bounds__(kThreads) k_stats_partial(const T *__restrict__ E, const T *__restrict__ Elo,
                                                            const T *__restrict__ H, const T *__restrict__ Hlo,
                                                            long nvals, double *partial) {
    double se = 0.0, sh = 0.0, me = 0.0, mh = 0.0, bad = 0.0;
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < nvals; t += (long)gridDim.x * blockDim.x) {
        double e = (double)E[t], h = (double)H[t];
        if constexpr (COMP) {
            e += (double)Elo[t];
            h += (double)Hlo[t];
        }
        if (!isfinite(e)) bad += 1.0;
        else {
            se += e * e;
            me = fmax(me, fabs(e));
        }
        if (!isfinite(h)) bad += 1.0;
        else {
            sh += h * h;
            mh = fmax(mh, fabs(h));
        }
    }
    __shared__ double red[5][kThreads / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        se += __shfl_down_sync(FULL_MASK, se, off);
        sh += __shfl_down_sync(FULL_MASK, sh, off);
        me = fmax(me, __shfl_down_sync(FULL_MASK, me, off));
        mh = fmax(mh, __shfl_down_sync(FULL_MASK, mh, off));
        bad += __shfl_down_sync(FULL_MASK, bad, off);
    }
    if (lane == 0) {
        red[0][w] = se;
        red[1][w] = sh;
        red[2][w] = me;
        red[3][w] = mh;
        red[4][w] = bad;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a0 = 0, a1 = 0, a2 = 0, a3 = 0, a4 = 0;
        for (int q = 0; q < kThreads / 32; ++q) {
            a0 += red[0][q];
            a1 += red[1][q];
            a2 = fmax(a2, red[2][q]);
            a3 = fmax(a3, red[3][q]);
            a4 += red[4][q];
        }
        double *row = partial + 5 * blockIdx.x;
        row[0] = a0;
        row[1] = a1;
        row[2] = a2;
        row[3] = a3;
        row[4] = a4;
    }
}

// Float fields, first pass: 16-byte loads, squares of each 4-vector summed in
// float and added to a double per vector, maxima in float.
__device__ __forceinline__ void stats_vec4(float4 v, double &s, float &m, unsigned &bad) {
    float q = 0.0f;
    const float x[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        if (isfinite(x[c])) {
            q = fmaf(x[c], x[c], q);
            m = fmaxf(m, fabsf(x[c]));
        } else {
            bad++;
        }
    }
    s += (double)q;
}

template <bool COMP>
__global__ void __launch_bounds__(kThreads) k_stats_partial4(const float4 *__restrict__ E,
                                                             const float4 *__restrict__ Elo,
                                                             const float4 *__restrict__ H,
                                                             const float4 *__restrict__ Hlo, long nvec,
                                                             double *partial) {
    double se = 0.0, sh = 0.0;
    float fme = 0.0f, fmh = 0.0f;
    unsigned nbad = 0;
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < nvec; t += (long)gridDim.x * blockDim.x) {
        float4 e = E[t], h = H[t];
        if constexpr (COMP) {
            const float4 el = Elo[t], hl = Hlo[t];
            e.x += el.x;
            e.y += el.y;
            e.z += el.z;
            e.w += el.w;
            h.x += hl.x;
            h.y += hl.y;
            h.z += hl.z;
            h.w += hl.w;
        }
        stats_vec4(e, se, fme, nbad);
        stats_vec4(h, sh, fmh, nbad);
    }
    double me = fme, mh = fmh, bad = (double)nbad;
    __shared__ double red[5][kThreads / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        se += __shfl_down_sync(FULL_MASK, se, off);
        sh += __shfl_down_sync(FULL_MASK, sh, off);
        me = fmax(me, __shfl_down_sync(FULL_MASK, me, off));
        mh = fmax(mh, __shfl_down_sync(FULL_MASK, mh, off));
        bad += __shfl_down_sync(FULL_MASK, bad, off);
    }
    if (lane == 0) {
        red[0][w] = se;
        red[1][w] = sh;
        red[2][w] = me;
        red[3][w] = mh;
        red[4][w] = bad;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a0 = 0, a1 = 0, a2 = 0, a3 = 0, a4 = 0;
        for (int q = 0; q < kThreads / 32; ++q) {
            a0 += red[0][q];
            a1 += red[1][q];
            a2 = fmax(a2, red[2][q]);
            a3 = fmax(a3, red[3][q]);
            a4 += red[4][q];
        }
        double *row = partial + 5 * blockIdx.x;
        row[0] = a0;
        row[1] = a1;
        row[2] = a2;
        row[3] = a3;
        row[4] = a4;
    }
}

// Second pass: one thread folds the CTA rows in order (deterministic).
static __global__ void k_stats_final(const double *partial, int nrows, double *out) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    double a0 = 0, a1 = 0, a2 = 0, a3 = 0, a4 = 0;
    for (int r = 0; r < nrows; ++r) {
        a0 += partial[5 * r];
        a1 += partial[5 * r + 1];
        a2 = fmax(a2, partial[5 * r + 2]);
        a3 = fmax(a3, partial[5 * r + 3]);
        a4 += partial[5 * r + 4];
    }
    out[0] = a0;
    out[1] = a1;
    out[2] = a2;
    out[3] = a3;
    out[4] = a4;
}

}  // namespace fdtd
