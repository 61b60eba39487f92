// Shared device-side definitions of the GB300 FDTD time-step library.
//
// Layout: every field is component-last, element (i, j, k, c) at
// ((i*ny + j)*nz + k)*3 + c.  A thread owns V consecutive cells along z
// (3*V contiguous values = three 16-byte vectors when V = 4 floats or
// V = 2 doubles) and marches along x over a chunk of planes, keeping the
// previous plane of the neighbour field in registers.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/fdtd_gb300.h"

namespace fdtd {

constexpr int kMaxSlabs = 6;
constexpr int kThreads = 256;

// One PML slab as the kernels see it.  `start` is the global index of the
// slab-local plane 0 along `axis`.
struct SlabK {
    int axis, high, th, start;
    int thp;  // stored slab-local extent: th, padded to even for z slabs
    void *psiE, *psiH;
    const void *bE, *cE, *bH, *cH;
    // where the staged passes read the auxiliaries from: psiE / psiH, or the
    // other buffer of the pair in a one-pass step (which writes psiE / psiH)
    const void *psiE_rd, *psiH_rd;
};

// An object or source box on the device.  bny/bnz are the box extents used
// for box-local coefficient indexing.
struct ItemK {
    int kind, comp, column, source;
    int lo[3], hi[3];
    int bny, bnz;
    double weight;
    const void *coef[3];
    int aux;  // FDTD_ITEM_FEEDBACK: its point in the current-probe list
};

// Material modes of a staged pass: the inverse material read per cell as
// three values (MAT_FULL), as a one-byte index into a small table of value
// triples (MAT_IDS), or not at all when every cell has the same triple
// (MAT_UNIFORM).  The values and the arithmetic are the same in every mode.
constexpr int MAT_FULL = 0, MAT_IDS = 1, MAT_UNIFORM = 2;

// Everything a half-step kernel needs, passed by value.
struct GridK {
    int nx, ny, nz;
    double courant;
    float courant_f;  // courant rounded once on the host (float plans)
    void *E, *H, *Elo, *Hlo;
    const void *ie, *imu;
    int nslab;        // PML slabs in boundary order
    int nslab_fused;  // slabs [0, nslab_fused) are corrected inside the fused pass
    SlabK slab[kMaxSlabs];
    const ItemK *items;
    const int *obj_off, *obj_idx;    // per-CTA object lists (E half only)
    const int *srcE_off, *srcE_idx;  // per-CTA source lists
    const int *srcH_off, *srcH_idx;
    int fuse_src_E, fuse_src_H;      // sources applied inside the fused pass
    int TZ, TY, XC;                  // threads along z, rows along y, planes along x per CTA
    // the box of cells the tiles cover: [ox, ex) x [oy, ey) x [oz, ez) (the
    // whole grid, or one part of an interior/shell partition); oz is a
    // multiple of 16 cells for the staged passes
    int ox, oy, oz, ex, ey, ez;
    int stages;                      // shared-memory ring depth of the staged (TMA) kernels
    int *status;                     // device error word (bit 0: a pipeline wait timed out)
    // staged kernels: bytes of one stage, and per slab the byte offset (in a
    // stage) and row pitch (values) of its psi slot
    int stage_bytes;
    int psi_off[kMaxSlabs], psi_pitch[kMaxSlabs];
    int n_staged;                  // staged passes: slabs whose auxiliary rows a stage holds,
    int staged_slab[kMaxSlabs];    // and their indices
    // one-pass step: offset and row pitch of each slab's H-side auxiliary slot
    int psi_offH[kMaxSlabs], psi_pitchH[kMaxSlabs];
    int coef_off[kMaxSlabs];  // per slab: offset (values) of its b/c tables in shared memory
    int coef_values;          // values of all staged b/c tables (0: tables are read from global)
    int scaled;               // ie / imu hold courant * inverse material (float64 plans)
    // staged passes: material mode of the E and H pass (MAT_FULL, MAT_IDS,
    // MAT_UNIFORM) and the value-triple tables they index
    int mat_E, mat_H;
    const void *mlut_E, *mlut_H;
    int nlut_E, nlut_H;
    int lut_rows;  // padded 4-value rows reserved for the table in shared memory
    const unsigned char *mid_E, *mid_H;  // one-byte material indices (MAT_IDS)
    int periodic_x;  // one-pass step: a periodic boundary along x follows the PML slabs
    const int *cta_order;  // staged passes: tile of each launched block, heaviest first (null: grid order)
};

// Shell boxes of an interior/shell partition: box b covers blocks
// [first[b], first[b + 1]) of the launch, its cells in (x, y, z) order from
// origin o with extents n, and meets the PML slabs in slabs[b].  The GridK
// of the launch carries per-block object and source lists.
// Cells per thread along z of the shell kernels: two floats or one double,
// which keeps the registers low enough for four blocks of 256 threads per SM.
template <class T>
constexpr int shell_v() {
    return sizeof(T) == 4 ? 2 : 1;
}

struct ShellK {
    int nbox;
    int o[6][3], n[6][3];
    unsigned first[7];
    unsigned slabs[6];  // per box: the PML slabs that reach into it
    // per box: x / d as umulhi(x, m) >> sh for d = its thread slots per row
    // (z) and its rows (y); exact for x < 2^31 (magic_div)
    unsigned mz[6], my[6];
    int sz[6], sy[6];
};

// Multiplier and shift of x / d for x < 2^31: with l = ceil(log2 d) and
// m = ceil(2^(31+l) / d) < 2^32, floor(x m / 2^(31+l)) = floor(x / d), since
// the error x (m - 2^(31+l)/d) / 2^(31+l) < 2^-l <= 1/d.  d = 1: m = 0, the
// caller takes x itself.
inline void magic_div(unsigned d, unsigned &m, int &shift) {
    if (d <= 1) {
        m = 0;
        shift = 0;
        return;
    }
    int l = 0;
    while ((1ull << l) < d) ++l;
    m = (unsigned)(((1ull << (31 + l)) + d - 1) / d);
    shift = l - 1;
}

__device__ __forceinline__ unsigned div_magic(unsigned x, unsigned m, int shift) {
    return m == 0 ? x : (__umulhi(x, m) >> shift);
}

template <class T>
__device__ __forceinline__ T courant_of(const GridK &g);
template <>
__device__ __forceinline__ float courant_of<float>(const GridK &g) {
    return g.courant_f;
}
template <>
__device__ __forceinline__ double courant_of<double>(const GridK &g) {
    return g.courant;
}

// Multiplier of the inverse materials in a product courant * material:
// 1 when the plan's material arrays already hold that product.
template <class T>
__device__ __forceinline__ T material_courant(const GridK &g) {
    return g.scaled ? T(1) : courant_of<T>(g);
}

// ---------------------------------------------------------------------------
// Precision policies.  The float64 policy reproduces the reference's numpy
// operation order with explicitly rounded operations (no fused multiply-add),
// so a float64 plan matches the reference bit for bit wherever the reference
// order is a plain sequence of elementwise operations.
// ---------------------------------------------------------------------------
struct PF64 {
    using T = double;
    static constexpr bool COMP = false;
    static constexpr int V = 2;
    __device__ __forceinline__ static T mul(T a, T b) { return __dmul_rn(a, b); }
    // courant * inverse material of a cell (the reference forms this product first)
    __device__ __forceinline__ static T cm(T c, T m) { return __dmul_rn(c, m); }
    __device__ __forceinline__ static void add_prod(T &x, T &, T a, T b) {
        x = __dadd_rn(x, __dmul_rn(a, b));
    }
    __device__ __forceinline__ static void sub_prod(T &x, T &, T a, T b) {
        x = __dsub_rn(x, __dmul_rn(a, b));
    }
    __device__ __forceinline__ static void scale(T &x, T &, T r) { x = __dmul_rn(x, r); }
    __device__ __forceinline__ static void set(T &x, T &, T v) { x = v; }
    // x += (a*b)/d, the AbsorbingObject order
    __device__ __forceinline__ static void add_quot(T &x, T &, T a, T b, T d) {
        x = __dadd_rn(x, __ddiv_rn(__dmul_rn(a, b), d));
    }
    __device__ __forceinline__ static T psi(T p, T b, T d, T c) {
        return __dadd_rn(__dmul_rn(p, b), __dmul_rn(d, c));
    }
    __device__ __forceinline__ static T dot3(T a0, T a1, T a2, T b0, T b1, T b2) {
        return __dadd_rn(__dadd_rn(__dmul_rn(a0, b0), __dmul_rn(a1, b1)), __dmul_rn(a2, b2));
    }
    __device__ __forceinline__ static void finish(T &, T &) {}
};

// float64 with the inverse materials already multiplied by the courant number
// on the host (the same rounded products the reference forms), so the
// kernels skip that product; GB300's float64 rate bounds these kernels.
struct PF64S : PF64 {
    __device__ __forceinline__ static T cm(T, T m) { return m; }
};

struct PF32 {
    using T = float;
    static constexpr bool COMP = false;
    static constexpr int V = 4;
    __device__ __forceinline__ static T mul(T a, T b) { return a * b; }
    __device__ __forceinline__ static T cm(T c, T m) { return c * m; }
    __device__ __forceinline__ static void add_prod(T &x, T &, T a, T b) { x = fmaf(a, b, x); }
    __device__ __forceinline__ static void sub_prod(T &x, T &, T a, T b) { x = fmaf(-a, b, x); }
    __device__ __forceinline__ static void scale(T &x, T &, T r) { x = x * r; }
    __device__ __forceinline__ static void set(T &x, T &, T v) { x = v; }
    __device__ __forceinline__ static void add_quot(T &x, T &, T a, T b, T) { x = fmaf(a, b, x); }
    __device__ __forceinline__ static T psi(T p, T b, T d, T c) { return fmaf(d, c, p * b); }
    __device__ __forceinline__ static T dot3(T a0, T a1, T a2, T b0, T b1, T b2) {
        return fmaf(a2, b2, fmaf(a1, b1, a0 * b0));
    }
    __device__ __forceinline__ static void finish(T &, T &) {}
};

// Two-float accumulation: a field value is hi + lo.  Every update that adds
// to or scales the value keeps the rounding error of that operation in lo
// (TwoSum for additions, an FMA residual for products), so round-off does
// not accumulate over long runs.  Stencil differences read hi only.
struct PF32C {
    using T = float;
    static constexpr bool COMP = true;
    static constexpr int V = 4;
    __device__ __forceinline__ static void two_sum(T a, T b, T &s, T &e) {
        s = a + b;
        T bp = s - a;
        T ap = s - bp;
        e = (a - ap) + (b - bp);
    }
    __device__ __forceinline__ static T mul(T a, T b) { return a * b; }
    __device__ __forceinline__ static T cm(T c, T m) { return c * m; }
    __device__ __forceinline__ static void add_prod(T &x, T &lo, T a, T b) {
        T p = a * b;
        T pe = fmaf(a, b, -p);
        T s, e;
        two_sum(x, p, s, e);
        x = s;
        lo = lo + (e + pe);
    }
    __device__ __forceinline__ static void sub_prod(T &x, T &lo, T a, T b) { add_prod(x, lo, -a, b); }
    __device__ __forceinline__ static void scale(T &x, T &lo, T r) {
        T p = x * r;
        T pe = fmaf(x, r, -p);
        lo = fmaf(lo, r, pe);
        x = p;
    }
    __device__ __forceinline__ static void set(T &x, T &lo, T v) {
        x = v;
        lo = 0.0f;
    }
    __device__ __forceinline__ static void add_quot(T &x, T &lo, T a, T b, T) { add_prod(x, lo, a, b); }
    __device__ __forceinline__ static T psi(T p, T b, T d, T c) { return fmaf(d, c, p * b); }
    __device__ __forceinline__ static T dot3(T a0, T a1, T a2, T b0, T b1, T b2) {
        return fmaf(a2, b2, fmaf(a1, b1, a0 * b0));
    }
    __device__ __forceinline__ static void finish(T &x, T &lo) {
        T s, e;
        two_sum(x, lo, s, e);
        x = s;
        lo = e;
    }
};

// ---------------------------------------------------------------------------
// Loads and stores of N contiguous values; 16-byte vectors when N*sizeof(T)
// is a multiple of 16 (the caller guarantees 16-byte alignment then).
// ---------------------------------------------------------------------------
template <class T, int N>
__device__ __forceinline__ void ld_vec(T (&dst)[N], const T *p) {
    if constexpr ((N * sizeof(T)) % 16 == 0) {
        const uint4 *q = reinterpret_cast<const uint4 *>(p);
#pragma unroll
        for (int i = 0; i < (int)(N * sizeof(T) / 16); ++i) {
            uint4 t = q[i];
            *reinterpret_cast<uint4 *>(&dst[i * 16 / sizeof(T)]) = t;
        }
    } else {
#pragma unroll
        for (int i = 0; i < N; ++i) dst[i] = p[i];
    }
}

// Read-only (non-coherent path) variant, only for data the kernel never writes.
template <class T, int N>
__device__ __forceinline__ void ld_vec_ro(T (&dst)[N], const T *__restrict__ p) {
    if constexpr ((N * sizeof(T)) % 16 == 0) {
        const uint4 *q = reinterpret_cast<const uint4 *>(p);
#pragma unroll
        for (int i = 0; i < (int)(N * sizeof(T) / 16); ++i) {
            uint4 t = __ldg(q + i);
            *reinterpret_cast<uint4 *>(&dst[i * 16 / sizeof(T)]) = t;
        }
    } else {
#pragma unroll
        for (int i = 0; i < N; ++i) dst[i] = __ldg(p + i);
    }
}

// Load cached in L2 only: for data that other blocks of the same launch
// write (the persistent time loop), which L1 could hold stale copies of.
template <class T, int N>
__device__ __forceinline__ void ld_vec_cg(T (&dst)[N], const T *p) {
    if constexpr ((N * sizeof(T)) % 16 == 0) {
        const uint4 *q = reinterpret_cast<const uint4 *>(p);
#pragma unroll
        for (int i = 0; i < (int)(N * sizeof(T) / 16); ++i) {
            uint4 t = __ldcg(q + i);
            *reinterpret_cast<uint4 *>(&dst[i * 16 / sizeof(T)]) = t;
        }
    } else {
#pragma unroll
        for (int i = 0; i < N; ++i) dst[i] = __ldcg(p + i);
    }
}

// Field loads of the register-streaming tiles: the read-only path (CG =
// false, one launch per half step) or L2 only (CG = true, persistent loop).
template <bool CG, class T, int N>
__device__ __forceinline__ void ld_field(T (&dst)[N], const T *p) {
    if constexpr (CG) ld_vec_cg(dst, p);
    else ld_vec_ro(dst, p);
}

template <bool CG, class T>
__device__ __forceinline__ T ld_field1(const T *p) {
    if constexpr (CG) return __ldcg(p);
    else return *p;
}

template <class T, int N>
__device__ __forceinline__ void st_vec(T *p, const T (&src)[N]) {
    if constexpr ((N * sizeof(T)) % 16 == 0) {
        uint4 *q = reinterpret_cast<uint4 *>(p);
#pragma unroll
        for (int i = 0; i < (int)(N * sizeof(T) / 16); ++i)
            q[i] = *reinterpret_cast<const uint4 *>(&src[i * 16 / sizeof(T)]);
    } else {
#pragma unroll
        for (int i = 0; i < N; ++i) p[i] = src[i];
    }
}

__device__ __forceinline__ bool in_box(const ItemK &it, int i, int j, int k) {
    return i >= it.lo[0] && i < it.hi[0] && j >= it.lo[1] && j < it.hi[1] && k >= it.lo[2] &&
           k < it.hi[2];
}

__device__ __forceinline__ size_t box_index(const ItemK &it, int i, int j, int k) {
    return ((size_t)(i - it.lo[0]) * it.bny + (j - it.lo[1])) * it.bnz + (k - it.lo[2]);
}

}  // namespace fdtd
