// Per-cell body of the fused half steps, shared by the register-streaming and
// the TMA-staged kernels.  The caller supplies the six one-sided differences of
// the neighbour field (zero where the reference drops the out-of-grid
// difference), the inverse material of the cell and the running field value;
// the body then applies, in the reference's order (fdtd/grid.py:275-325):
//   curl and bulk update, objects (E only), PML auxiliaries and corrections,
//   sources.
#pragma once

#include "fdtd_common.cuh"

namespace fdtd {

// Where a cell's PML auxiliaries and coefficient tables are read from: the
// shared-memory stage of the staged kernels, or global memory (stage = null).
// Updated auxiliaries are always written to global memory.
template <class T>
struct PsiSrc {
    const unsigned char *stage;  // stage base, psi slots at g.psi_off[s]
    int row;                     // this thread's row in the tile
    int k0c;                     // first cell of the tile along z
    const T *ctab;               // b/c tables at g.coef_off[s] (null: global)
};

// Bit s set: PML slab s can contain cells of this thread.  The y and z parts
// do not change along x (computed once per thread), the x part per plane.
__device__ __forceinline__ unsigned slab_mask_yz(const GridK &g, int j, int k0, int V) {
    unsigned m = 0;
    for (int s = 0; s < g.nslab; ++s) {
        const SlabK &S = g.slab[s];
        if (S.axis == 1) {
            if ((unsigned)(j - S.start) < (unsigned)S.th) m |= 1u << s;
        } else if (S.axis == 2) {
            if (k0 < S.start + S.th && k0 + V > S.start) m |= 1u << s;
        }
    }
    return m;
}

__device__ __forceinline__ unsigned slab_mask_x(const GridK &g, int i) {
    unsigned m = 0;
    for (int s = 0; s < g.nslab; ++s) {
        const SlabK &S = g.slab[s];
        if (S.axis == 0 && (unsigned)(i - S.start) < (unsigned)S.th) m |= 1u << s;
    }
    return m;
}

// Objects of one cell (fdtd/objects.py:118-277), in registration order.
template <class P>
__device__ __forceinline__ void apply_object_cell(const ItemK &o, size_t li, typename P::T c, typename P::T cu0,
                                                  typename P::T cu1, typename P::T cu2, typename P::T &ex,
                                                  typename P::T &ey, typename P::T &ez, typename P::T &lx,
                                                  typename P::T &ly, typename P::T &lz) {
    using T = typename P::T;
    if (o.kind == FDTD_ITEM_OBJECT) {
        const T *cf = (const T *)o.coef[0] + 3 * li;
        P::add_prod(ex, lx, cf[0], cu0);
        P::add_prod(ey, ly, cf[1], cu1);
        P::add_prod(ez, lz, cf[2], cu2);
    } else if (o.kind == FDTD_ITEM_ABSORBING) {
        const T *r = (const T *)o.coef[0] + 3 * li;
        const T *ci = (const T *)o.coef[1] + 3 * li;
        P::scale(ex, lx, r[0]);
        P::scale(ey, ly, r[1]);
        P::scale(ez, lz, r[2]);
        if constexpr (sizeof(T) == 4) {
            P::add_prod(ex, lx, ci[0], cu0);
            P::add_prod(ey, ly, ci[1], cu1);
            P::add_prod(ez, lz, ci[2], cu2);
        } else {
            const T *opf = (const T *)o.coef[2] + 3 * li;
            P::add_quot(ex, lx, ci[0], cu0, opf[0]);
            P::add_quot(ey, ly, ci[1], cu1, opf[1]);
            P::add_quot(ez, lz, ci[2], cu2, opf[2]);
        }
    } else {
        const T *M = (const T *)o.coef[0] + 9 * li;
        P::add_prod(ex, lx, c, P::dot3(M[0], M[1], M[2], cu0, cu1, cu2));
        P::add_prod(ey, ly, c, P::dot3(M[3], M[4], M[5], cu0, cu1, cu2));
        P::add_prod(ez, lz, c, P::dot3(M[6], M[7], M[8], cu0, cu1, cu2));
    }
}

__device__ __forceinline__ bool aligned16_ptr(const void *p) { return ((uintptr_t)p & 15u) == 0; }

// Ask L2 for the `bytes` bytes at p (one request per 128-byte line): the
// object coefficients of the next plane, so that its loads hit L2 instead of
// waiting for DRAM inside the plane loop.
__device__ __forceinline__ void prefetch_l2(const void *p, int bytes) {
    const char *c = reinterpret_cast<const char *>(p);
    for (int o = 0; o < bytes; o += 128) asm volatile("prefetch.global.L2 [%0];" ::"l"(c + o));
}

// Objects of a thread's V cells (fdtd/objects.py:92-129, 198-221, 256-269),
// items in list order; each cell gets the same operations in the same order
// as one at a time.  In float32, where all V cells lie in a box and their
// coefficients start on a 16-byte boundary, they are read with 16-byte
// loads: one 4-byte load per value at a 3- or 9-value stride touches a sector
// per lane, and the CTAs holding a 1.6 % anisotropic box (config 5) took
// twice as long per plane as the others.
template <class P, int V>
__device__ __forceinline__ void apply_objects_v(const GridK &g, int i, int j, int k0, typename P::T c,
                                                const typename P::T (&cu)[3][V], typename P::T (&e)[3 * V],
                                                typename P::T (&el)[3 * V], int ob0, int ob1) {
    using T = typename P::T;
    for (int it = ob0; it < ob1; ++it) {
        const ItemK &o = g.items[g.obj_idx[it]];
        if (i < o.lo[0] || i >= o.hi[0] || j < o.lo[1] || j >= o.hi[1] || k0 >= o.hi[2] || k0 + V <= o.lo[2])
            continue;
        // float32 only: in float64 the values held for the wide loads pushed
        // the staged E pass past 128 registers (one CTA per SM instead of
        // two: config 3 float64 15.3 -> 14.0 Gcell/s)
        if constexpr (V > 1 && sizeof(T) == 4) {
            const size_t li = k0 >= o.lo[2] ? box_index(o, i, j, k0) : 0;
            const bool whole = k0 >= o.lo[2] && k0 + V <= o.hi[2];
            // the next plane of the box one plane ahead
            const size_t plane = (size_t)o.bny * o.bnz;
            const bool ahead = i + 1 < o.hi[0];
            if (whole && o.kind == FDTD_ITEM_ANISOTROPIC) {
                const T *src = (const T *)o.coef[0] + 9 * li;
                if (aligned16_ptr(src)) {
                    alignas(16) T M[9 * V];
                    ld_vec_ro(M, src);
                    if (ahead) prefetch_l2(src + 9 * plane, 9 * V * (int)sizeof(T));
#pragma unroll
                    for (int v = 0; v < V; ++v) {
                        const T *m = M + 9 * v;
                        P::add_prod(e[3 * v], el[3 * v], c, P::dot3(m[0], m[1], m[2], cu[0][v], cu[1][v], cu[2][v]));
                        P::add_prod(e[3 * v + 1], el[3 * v + 1], c,
                                    P::dot3(m[3], m[4], m[5], cu[0][v], cu[1][v], cu[2][v]));
                        P::add_prod(e[3 * v + 2], el[3 * v + 2], c,
                                    P::dot3(m[6], m[7], m[8], cu[0][v], cu[1][v], cu[2][v]));
                    }
                    continue;
                }
            } else if (whole && o.kind == FDTD_ITEM_OBJECT) {
                const T *src = (const T *)o.coef[0] + 3 * li;
                if (aligned16_ptr(src)) {
                    alignas(16) T cf[3 * V];
                    ld_vec_ro(cf, src);
                    if (ahead) prefetch_l2(src + 3 * plane, 3 * V * (int)sizeof(T));
#pragma unroll
                    for (int v = 0; v < V; ++v)
#pragma unroll
                        for (int q = 0; q < 3; ++q) P::add_prod(e[3 * v + q], el[3 * v + q], cf[3 * v + q], cu[q][v]);
                    continue;
                }
            } else if (whole && o.kind == FDTD_ITEM_ABSORBING) {
                const T *rs = (const T *)o.coef[0] + 3 * li, *cs = (const T *)o.coef[1] + 3 * li;
                const T *os = sizeof(T) == 8 ? (const T *)o.coef[2] + 3 * li : rs;
                if (aligned16_ptr(rs) && aligned16_ptr(cs) && aligned16_ptr(os)) {
                    alignas(16) T r[3 * V], ci[3 * V];
                    ld_vec_ro(r, rs);
                    ld_vec_ro(ci, cs);
                    if (ahead) {
                        prefetch_l2(rs + 3 * plane, 3 * V * (int)sizeof(T));
                        prefetch_l2(cs + 3 * plane, 3 * V * (int)sizeof(T));
                    }
                    if constexpr (sizeof(T) == 4) {
#pragma unroll
                        for (int q = 0; q < 3 * V; ++q) {
                            P::scale(e[q], el[q], r[q]);
                            P::add_prod(e[q], el[q], ci[q], cu[q % 3][q / 3]);
                        }
                    } else {
                        alignas(16) T opf[3 * V];
                        ld_vec_ro(opf, os);
#pragma unroll
                        for (int q = 0; q < 3 * V; ++q) {
                            P::scale(e[q], el[q], r[q]);
                            P::add_quot(e[q], el[q], ci[q], cu[q % 3][q / 3], opf[q]);
                        }
                    }
                    continue;
                }
            }
        }
#pragma unroll
        for (int v = 0; v < V; ++v) {
            const int k = k0 + v;
            if (k < o.lo[2] || k >= o.hi[2]) continue;
            apply_object_cell<P>(o, box_index(o, i, j, k), c, cu[0][v], cu[1][v], cu[2][v], e[3 * v], e[3 * v + 1],
                                 e[3 * v + 2], el[3 * v], el[3 * v + 1], el[3 * v + 2]);
        }
    }
}

// Sources of one cell (fdtd/sources.py:93-109, 278-297, 476-486), in order.
template <class P>
__device__ __forceinline__ void apply_sources(const GridK &g, const int *idx, const double *__restrict__ wave, int i,
                                              int j, int k, typename P::T &fx, typename P::T &fy, typename P::T &fz,
                                              typename P::T &lx, typename P::T &ly, typename P::T &lz, int sb0,
                                              int sb1) {
    using T = typename P::T;
    for (int it = sb0; it < sb1; ++it) {
        const ItemK &s = g.items[idx[it]];
        if (!in_box(s, i, j, k)) continue;
        const T w = (T)s.weight, wv = (T)wave[s.column];
        if (s.kind == FDTD_ITEM_SOFT) {
            if (s.comp == 0) P::add_prod(fx, lx, w, wv);
            else if (s.comp == 1) P::add_prod(fy, ly, w, wv);
            else P::add_prod(fz, lz, w, wv);
        } else {
            const T val = P::mul(w, wv);
            if (s.comp == 0) P::set(fx, lx, val);
            else if (s.comp == 1) P::set(fy, ly, val);
            else P::set(fz, lz, val);
        }
    }
}

// E += (c m) phi for the E half, H -= (c m) phi for the H half.
template <class P, bool IS_E>
__device__ __forceinline__ void pml_correct(typename P::T &f, typename P::T &fl, typename P::T cm, typename P::T phi) {
    if (IS_E) P::add_prod(f, fl, cm, phi);
    else P::sub_prod(f, fl, cm, phi);
}

// One PML slab (index s, normal to axis A) on a thread's V cells: the body
// of apply_pml below, compiled once per normal axis.
template <class P, int V, bool IS_E, bool HOFF, int A>
__device__ __forceinline__ void apply_pml_slab(const GridK &g, int s, int i, int j, int k0, typename P::T c,
                                               const typename P::T (&d)[6][V], const typename P::T (&m)[3 * V],
                                               typename P::T (&f)[3 * V], typename P::T (&fl)[3 * V],
                                               const PsiSrc<typename P::T> &src, bool store) {
    using T = typename P::T;
    const SlabK &S = g.slab[s];
    const int th = S.th;
    T *psi = (T *)(IS_E ? S.psiE : S.psiH);
    const T *bt = (const T *)(IS_E ? S.bE : S.bH);
    const T *ct = (const T *)(IS_E ? S.cE : S.cH);
    // slab-local index of cell k0 and the rows of its auxiliaries
    const int l0 = (A == 0 ? i : (A == 1 ? j : k0)) - S.start;
    long gofs;
    if constexpr (A == 0) gofs = ((long)l0 * g.ny + j) * g.nz + k0;
    else if constexpr (A == 1) gofs = ((long)i * th + l0) * g.nz + k0;
    else gofs = ((long)i * g.ny + j) * S.thp + l0;
    T *gp = psi + 2 * gofs;
    const T *sp = nullptr;
    if (src.stage)
        sp = reinterpret_cast<const T *>(src.stage + (HOFF ? g.psi_offH[s] : g.psi_off[s])) +
             src.row * (HOFF ? g.psi_pitchH[s] : g.psi_pitch[s]) + (A == 2 ? 2 * l0 : 2 * (k0 - src.k0c));
    const T *tb = src.ctab ? src.ctab + g.coef_off[s] : bt;  // b at [l], c at [th + l] (shared) or ct[l]
    const T *tc = src.ctab ? src.ctab + g.coef_off[s] + th : ct;
    const bool corr = s < g.nslab_fused;
    // phi[(A+1)%3] = -p0, phi[(A+2)%3] = +p1 (fdtd/boundaries.py:457-459, 485-487);
    // p0 is driven by the difference d0, p1 by d1
    constexpr int q0 = A == 0 ? 1 : (A == 1 ? 2 : 5);
    constexpr int q1 = A == 0 ? 0 : (A == 1 ? 3 : 4);
    constexpr int c0 = (A + 1) % 3, c1 = (A + 2) % 3;
    // all loads first (a store to the auxiliaries would otherwise order every
    // later load behind it), then the updates, then the stores
    T p0[V], p1[V];
    if constexpr (A != 2) {
        // x/y slab: the V cells share one slab-local index
        if constexpr (V > 1) {
            // one contiguous, 16-byte aligned run of pairs
            alignas(16) T pr[2 * V];
            if (sp) ld_vec(pr, sp);
            else ld_vec(pr, (const T *)gp);
#pragma unroll
            for (int v = 0; v < V; ++v) {
                p0[v] = pr[2 * v];
                p1[v] = pr[2 * v + 1];
            }
        } else {
            const T *q = sp ? sp : gp;
            p0[0] = q[0];
            p1[0] = q[1];
        }
        const T b = tb[l0], cc = tc[l0];
        if (IS_E ? (l0 >= 1) : (l0 <= th - 2)) {
#pragma unroll
            for (int v = 0; v < V; ++v) {
                p0[v] = P::psi(p0[v], b, d[q0][v], cc);
                p1[v] = P::psi(p1[v], b, d[q1][v], cc);
            }
        } else {
#pragma unroll
            for (int v = 0; v < V; ++v) {
                p0[v] = P::mul(p0[v], b);
                p1[v] = P::mul(p1[v], b);
            }
        }
        if (corr) {
#pragma unroll
            for (int v = 0; v < V; ++v) {
                pml_correct<P, IS_E>(f[3 * v + c0], fl[3 * v + c0], P::cm(c, m[3 * v + c0]), -p0[v]);
                pml_correct<P, IS_E>(f[3 * v + c1], fl[3 * v + c1], P::cm(c, m[3 * v + c1]), p1[v]);
            }
        }
        if (!store) {
        } else if constexpr (V > 1) {
            alignas(16) T pr[2 * V];
#pragma unroll
            for (int v = 0; v < V; ++v) {
                pr[2 * v] = p0[v];
                pr[2 * v + 1] = p1[v];
            }
            st_vec(gp, pr);
        } else {
            gp[0] = p0[0];
            gp[1] = p1[0];
        }
    } else {
        // z slab: the V cells have consecutive slab-local indices, some may lie outside
#pragma unroll
        for (int v = 0; v < V; ++v) {
            const int l = l0 + v;
            p0[v] = T(0);
            p1[v] = T(0);
            if ((unsigned)l >= (unsigned)th) continue;
            if (sp) {
                p0[v] = sp[2 * v];
                p1[v] = sp[2 * v + 1];
            } else {
                p0[v] = gp[2 * v];
                p1[v] = gp[2 * v + 1];
            }
        }
#pragma unroll
        for (int v = 0; v < V; ++v) {
            const int l = l0 + v;
            if ((unsigned)l >= (unsigned)th) continue;
            const T b = tb[l], cc = tc[l];
            if (IS_E ? (l >= 1) : (l <= th - 2)) {
                p0[v] = P::psi(p0[v], b, d[q0][v], cc);
                p1[v] = P::psi(p1[v], b, d[q1][v], cc);
            } else {
                p0[v] = P::mul(p0[v], b);
                p1[v] = P::mul(p1[v], b);
            }
            if (corr) {
                pml_correct<P, IS_E>(f[3 * v + c0], fl[3 * v + c0], P::cm(c, m[3 * v + c0]), -p0[v]);
                pml_correct<P, IS_E>(f[3 * v + c1], fl[3 * v + c1], P::cm(c, m[3 * v + c1]), p1[v]);
            }
        }
        if (store) {
#pragma unroll
            for (int v = 0; v < V; ++v) {
                const int l = l0 + v;
                if ((unsigned)l >= (unsigned)th) continue;
                gp[2 * v] = p0[v];
                gp[2 * v + 1] = p1[v];
            }
        }
    }
}

// PML auxiliaries and corrections of a thread's V cells, slab by slab in
// boundary order (the per-cell order of fdtd/grid.py:279-291 is kept: every
// slab touching a cell acts on it in ascending slab order).  d[q][v] are the
// six one-sided differences of the neighbour field F of cell v, in the order
// (dx F_y, dx F_z, dy F_x, dy F_z, dz F_x, dz F_y); a slab normal to axis a
// drives its pair with (dF_(a+2)%3, dF_(a+1)%3) along a.  IS_E selects the E
// rule (increment at slab-local index >= 1, E += c m phi) or the H rule
// (index <= th-2, H -= c m phi).  store = false computes without writing the
// updated auxiliaries (a neighbour's cell recomputed by the one-pass step);
// HOFF selects the stage's H-side auxiliary slots (g.psi_offH/psi_pitchH) of
// the one-pass step instead of g.psi_off/psi_pitch.  Each slab runs the code
// compiled for its normal axis.
template <class P, int V, bool IS_E, bool HOFF = false>
__device__ __forceinline__ void apply_pml(const GridK &g, int i, int j, int k0, typename P::T c,
                                          const typename P::T (&d)[6][V], const typename P::T (&m)[3 * V],
                                          typename P::T (&f)[3 * V], typename P::T (&fl)[3 * V],
                                          const PsiSrc<typename P::T> &src, unsigned slabs, bool store = true) {
    for (unsigned sm = slabs; sm; sm &= sm - 1) {
        const int s = __ffs(sm) - 1;
        const int a = g.slab[s].axis;
        if (a == 0) apply_pml_slab<P, V, IS_E, HOFF, 0>(g, s, i, j, k0, c, d, m, f, fl, src, store);
        else if (a == 1) apply_pml_slab<P, V, IS_E, HOFF, 1>(g, s, i, j, k0, c, d, m, f, fl, src, store);
        else apply_pml_slab<P, V, IS_E, HOFF, 2>(g, s, i, j, k0, c, d, m, f, fl, src, store);
    }
}

// E half step of a thread's V cells at (i, j, k0..k0+V-1).  hc: H of the cells,
// hp: H at plane i-1, hj: H at row j-1, (kx, ky): Hx, Hy at k0-1.  store and
// HOFF as for apply_pml.
template <class P, int V, bool HOFF = false>
__device__ __forceinline__ void thread_E(const GridK &g, const double *__restrict__ wave, int i, int j, int k0,
                                         typename P::T c, const typename P::T (&hc)[3 * V],
                                         const typename P::T (&hp)[3 * V], const typename P::T (&hj)[3 * V],
                                         typename P::T kx, typename P::T ky, const typename P::T (&m)[3 * V],
                                         typename P::T (&e)[3 * V], typename P::T (&el)[3 * V], int ob0, int ob1,
                                         int sb0, int sb1, const PsiSrc<typename P::T> &src, unsigned slabs,
                                         bool store = true) {
    using T = typename P::T;
    T d[6][V];  // dxHy, dxHz, dyHx, dyHz, dzHx, dzHy (backward, zero on the first plane)
    T cu[3][V];  // curl H
#pragma unroll
    for (int v = 0; v < V; ++v) {
        const int k = k0 + v;
        const T hx = hc[3 * v], hy = hc[3 * v + 1], hz = hc[3 * v + 2];
        const T pkx = (v > 0) ? hc[3 * (v - 1)] : kx;
        const T pky = (v > 0) ? hc[3 * (v - 1) + 1] : ky;
        d[0][v] = (i > 0) ? hy - hp[3 * v + 1] : T(0);
        d[1][v] = (i > 0) ? hz - hp[3 * v + 2] : T(0);
        d[2][v] = (j > 0) ? hx - hj[3 * v] : T(0);
        d[3][v] = (j > 0) ? hz - hj[3 * v + 2] : T(0);
        d[4][v] = (k > 0) ? hx - pkx : T(0);
        d[5][v] = (k > 0) ? hy - pky : T(0);
        cu[0][v] = d[3][v] - d[5][v];
        cu[1][v] = d[4][v] - d[1][v];
        cu[2][v] = d[0][v] - d[2][v];
        P::add_prod(e[3 * v], el[3 * v], P::cm(c, m[3 * v]), cu[0][v]);
        P::add_prod(e[3 * v + 1], el[3 * v + 1], P::cm(c, m[3 * v + 1]), cu[1][v]);
        P::add_prod(e[3 * v + 2], el[3 * v + 2], P::cm(c, m[3 * v + 2]), cu[2][v]);
    }
    if (ob0 < ob1) apply_objects_v<P, V>(g, i, j, k0, c, cu, e, el, ob0, ob1);
    if (slabs) apply_pml<P, V, true, HOFF>(g, i, j, k0, c, d, m, e, el, src, slabs, store);
#pragma unroll
    for (int v = 0; v < V; ++v) {
        if (sb0 < sb1)
            apply_sources<P>(g, g.srcE_idx, wave, i, j, k0 + v, e[3 * v], e[3 * v + 1], e[3 * v + 2], el[3 * v],
                             el[3 * v + 1], el[3 * v + 2], sb0, sb1);
        P::finish(e[3 * v], el[3 * v]);
        P::finish(e[3 * v + 1], el[3 * v + 1]);
        P::finish(e[3 * v + 2], el[3 * v + 2]);
    }
}

// H half step of a thread's V cells.  ec: E of the cells, en: E at plane i+1,
// ej: E at row j+1, (kx, ky): Ex, Ey at k0+V.  store and HOFF as for apply_pml.
template <class P, int V, bool HOFF = false>
__device__ __forceinline__ void thread_H(const GridK &g, const double *__restrict__ wave, int i, int j, int k0,
                                         typename P::T c, const typename P::T (&ec)[3 * V],
                                         const typename P::T (&en)[3 * V], const typename P::T (&ej)[3 * V],
                                         typename P::T kx, typename P::T ky, const typename P::T (&m)[3 * V],
                                         typename P::T (&h)[3 * V], typename P::T (&hl)[3 * V], int sb0, int sb1,
                                         const PsiSrc<typename P::T> &src, unsigned slabs, bool store = true) {
    using T = typename P::T;
    T d[6][V];  // dxEy, dxEz, dyEx, dyEz, dzEx, dzEy (forward, zero on the last plane)
#pragma unroll
    for (int v = 0; v < V; ++v) {
        const int k = k0 + v;
        const T ex_ = ec[3 * v], ey_ = ec[3 * v + 1], ez_ = ec[3 * v + 2];
        const T nkx = (v < V - 1) ? ec[3 * (v + 1)] : kx;
        const T nky = (v < V - 1) ? ec[3 * (v + 1) + 1] : ky;
        d[0][v] = (i < g.nx - 1) ? en[3 * v + 1] - ey_ : T(0);
        d[1][v] = (i < g.nx - 1) ? en[3 * v + 2] - ez_ : T(0);
        d[2][v] = (j < g.ny - 1) ? ej[3 * v] - ex_ : T(0);
        d[3][v] = (j < g.ny - 1) ? ej[3 * v + 2] - ez_ : T(0);
        d[4][v] = (k < g.nz - 1) ? nkx - ex_ : T(0);
        d[5][v] = (k < g.nz - 1) ? nky - ey_ : T(0);
        P::sub_prod(h[3 * v], hl[3 * v], P::cm(c, m[3 * v]), d[3][v] - d[5][v]);
        P::sub_prod(h[3 * v + 1], hl[3 * v + 1], P::cm(c, m[3 * v + 1]), d[4][v] - d[1][v]);
        P::sub_prod(h[3 * v + 2], hl[3 * v + 2], P::cm(c, m[3 * v + 2]), d[0][v] - d[2][v]);
    }
    if (slabs) apply_pml<P, V, false, HOFF>(g, i, j, k0, c, d, m, h, hl, src, slabs, store);
#pragma unroll
    for (int v = 0; v < V; ++v) {
        if (sb0 < sb1)
            apply_sources<P>(g, g.srcH_idx, wave, i, j, k0 + v, h[3 * v], h[3 * v + 1], h[3 * v + 2], hl[3 * v],
                             hl[3 * v + 1], hl[3 * v + 2], sb0, sb1);
        P::finish(h[3 * v], hl[3 * v]);
        P::finish(h[3 * v + 1], hl[3 * v + 1]);
        P::finish(h[3 * v + 2], hl[3 * v + 2]);
    }
}

}  // namespace fdtd
