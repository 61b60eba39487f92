// Kernels of the reverse-time adjoint (no reference counterpart; the
// reference offers gradients only through autograd of its torch backend).
//
// The forward half steps are affine in the state (E, H, PML auxiliaries
// psi), so the gradient of a loss that reads detector samples is carried
// backwards by the transposed half steps acting on the adjoint state:
// lam_E, lam_H (adjoints of E and H) and, per PML slab, the adjoints of the
// two stored auxiliaries.  With the forward curls written as one-sided
// differences whose out-of-grid term is dropped,
//   curl_H uses  B u[n] = u[n] - u[n-1] (n >= 1), 0 at n = 0
//   curl_E uses  F u[n] = u[n+1] - u[n] (n <= N-2), 0 at n = N-1
// their transposes are again differences with the edge rules moved:
//   F^T v = -D1 v,  D1 v[n] = [n <= N-2] v[n] - [n >= 1] v[n-1]
//   B^T v = -D2 v,  D2 v[n] = [n <= N-2] v[n+1] - [n >= 1] v[n]
// so the transposed H half (k_adj_H) updates lam_E with a curl_H-shaped
// stencil of w = courant*inv_mu*lam_H, and the transposed E half (k_adj_E)
// updates lam_H with a curl_E-shaped stencil of u = courant*inv_eps*lam_E:
//   lam_E -= curl_D1(w)        (transpose of H -= c mu^-1 curl_E(E))
//   lam_H += curl_D2(u)        (transpose of E += c eps^-1 curl_H(H))
// The PML terms transpose the same way with the slab-local index rules of
// the forward auxiliaries (E side: increment at l >= 1; H side: l <= th-2).
// Adjoint auxiliaries are double buffered (read the current buffer, write
// the other) because a cell's update reads its neighbour's auxiliary.
// Objects (grid inverse permittivity is zero inside them) are transposed by
// box kernels that also accumulate the design gradient.
#pragma once

#include "fdtd_kernels.cuh"

namespace fdtd {

// Current (read) and next (written) adjoint auxiliaries per PML slab.
struct AdjAux {
    const void *Eo[kMaxSlabs];
    void *En[kMaxSlabs];
    const void *Ho[kMaxSlabs];
    void *Hn[kMaxSlabs];
};

// Pair index of cell (i, j, k) in the compact auxiliary layout of slab S.
__device__ __forceinline__ long slab_pair(const GridK &g, const SlabK &S, int i, int j, int k) {
    if (S.axis == 0) return ((long)(i - S.start) * g.ny + j) * g.nz + k;
    if (S.axis == 1) return ((long)i * S.th + (j - S.start)) * g.nz + k;
    return ((long)i * g.ny + j) * S.thp + (k - S.start);
}

// dst[q] = (c * m[q]) * lam[q] for the 3V values at cell0.
template <class T, int V>
__device__ __forceinline__ void load_scaled(T (&dst)[3 * V], const T *lam, const T *__restrict__ m, size_t cell0,
                                            T c) {
    alignas(16) T l[3 * V], mm[3 * V];
    ld_vec(l, lam + 3 * cell0);
    ld_vec_ro(mm, m + 3 * cell0);
#pragma unroll
    for (int q = 0; q < 3 * V; ++q) dst[q] = (c * mm[q]) * l[q];
}

template <class T, int N>
__device__ __forceinline__ void zero(T (&a)[N]) {
#pragma unroll
    for (int q = 0; q < N; ++q) a[q] = T(0);
}

// PML part of the transposed H half for a thread's V cells (slabs in `slabs`).
// Forward, slab normal a with t1 = (a+1)%3, t2 = (a+2)%3:
//   psiH0 = bH psiH0 + cH F(E_t2), psiH1 = bH psiH1 + cH F(E_t1)  (l <= th-2)
//   H_t1 += c mu_t1 psiH0,  H_t2 -= c mu_t2 psiH1
// Transposed (nu = adjoint auxiliaries, w = c mu lam_H):
//   nu0 += w_t1, nu1 -= w_t2 (slabs corrected in the fused pass; the others
//   were incremented by k_adj_slab_inc), lam_E_t2 -= D1(cH nu0),
//   lam_E_t1 -= D1(cH nu1), nu <- bH nu.
template <class T, int V, int A>
__device__ __forceinline__ void adj_slab_H(const GridK &g, const AdjAux &x, int s, int i, int j, int k0,
                                           const T (&w)[3 * V], const T (&wp)[3 * V], const T (&wj)[3 * V], T kx,
                                           T ky, T (&e)[3 * V]) {
    constexpr int t1 = (A + 1) % 3, t2 = (A + 2) % 3;
    const SlabK &S = g.slab[s];
    const int th = S.th;
    const T *no = (const T *)x.Ho[s];
    T *nn = (T *)x.Hn[s];
    const T *bt = (const T *)S.bH;
    const T *ct = (const T *)S.cH;
    const T f = s < g.nslab_fused ? T(1) : T(0);
    const long back = A == 0 ? (long)g.ny * g.nz : (A == 1 ? (long)g.nz : 1L);
#pragma unroll
    for (int v = 0; v < V; ++v) {
        const int l = (A == 0 ? i : (A == 1 ? j : k0 + v)) - S.start;
        if ((unsigned)l >= (unsigned)th) continue;
        const long pt = slab_pair(g, S, i, j, k0 + v);
        const T n0 = no[2 * pt] + f * w[3 * v + t1];
        const T n1 = no[2 * pt + 1] - f * w[3 * v + t2];
        T d0 = T(0), d1 = T(0);
        if (l <= th - 2) {
            d0 = ct[l] * n0;
            d1 = ct[l] * n1;
        }
        if (l >= 1) {
            T pw1, pw2;
            if constexpr (A == 0) {
                pw1 = wp[3 * v + t1];
                pw2 = wp[3 * v + t2];
            } else if constexpr (A == 1) {
                pw1 = wj[3 * v + t1];
                pw2 = wj[3 * v + t2];
            } else {  // t1 = x, t2 = y
                pw1 = v > 0 ? w[3 * (v - 1)] : kx;
                pw2 = v > 0 ? w[3 * (v - 1) + 1] : ky;
            }
            const long pq = pt - back;
            const T p0 = no[2 * pq] + f * pw1;
            const T p1 = no[2 * pq + 1] - f * pw2;
            d0 -= ct[l - 1] * p0;
            d1 -= ct[l - 1] * p1;
        }
        e[3 * v + t2] -= d0;
        e[3 * v + t1] -= d1;
        nn[2 * pt] = bt[l] * n0;
        nn[2 * pt + 1] = bt[l] * n1;
    }
}

template <class T, int V>
__device__ __forceinline__ void adj_pml_H(const GridK &g, const AdjAux &x, int i, int j, int k0, const T (&w)[3 * V],
                                          const T (&wp)[3 * V], const T (&wj)[3 * V], T kx, T ky, T (&e)[3 * V],
                                          unsigned slabs) {
    for (unsigned sm = slabs; sm; sm &= sm - 1) {
        const int s = __ffs(sm) - 1;
        const int a = g.slab[s].axis;
        if (a == 0) adj_slab_H<T, V, 0>(g, x, s, i, j, k0, w, wp, wj, kx, ky, e);
        else if (a == 1) adj_slab_H<T, V, 1>(g, x, s, i, j, k0, w, wp, wj, kx, ky, e);
        else adj_slab_H<T, V, 2>(g, x, s, i, j, k0, w, wp, wj, kx, ky, e);
    }
}

// PML part of the transposed E half.  Forward:
//   psiE0 = bE psiE0 + cE B(H_t2), psiE1 = bE psiE1 + cE B(H_t1)  (l >= 1)
//   E_t1 -= c eps_t1 psiE0,  E_t2 += c eps_t2 psiE1
// Transposed (mu = adjoint auxiliaries, u = c eps lam_E):
//   mu0 -= u_t1, mu1 += u_t2, lam_H_t2 -= D2(cE mu0), lam_H_t1 -= D2(cE mu1),
//   mu <- bE mu.
template <class T, int V, int A>
__device__ __forceinline__ void adj_slab_E(const GridK &g, const AdjAux &x, int s, int i, int j, int k0,
                                           const T (&u)[3 * V], const T (&un)[3 * V], const T (&uj)[3 * V], T kx,
                                           T ky, T (&h)[3 * V]) {
    constexpr int t1 = (A + 1) % 3, t2 = (A + 2) % 3;
    const SlabK &S = g.slab[s];
    const int th = S.th;
    const T *mo = (const T *)x.Eo[s];
    T *mn = (T *)x.En[s];
    const T *bt = (const T *)S.bE;
    const T *ct = (const T *)S.cE;
    const T f = s < g.nslab_fused ? T(1) : T(0);
    const long fwd = A == 0 ? (long)g.ny * g.nz : (A == 1 ? (long)g.nz : 1L);
#pragma unroll
    for (int v = 0; v < V; ++v) {
        const int l = (A == 0 ? i : (A == 1 ? j : k0 + v)) - S.start;
        if ((unsigned)l >= (unsigned)th) continue;
        const long pt = slab_pair(g, S, i, j, k0 + v);
        const T m0 = mo[2 * pt] - f * u[3 * v + t1];
        const T m1 = mo[2 * pt + 1] + f * u[3 * v + t2];
        T d0 = T(0), d1 = T(0);
        if (l >= 1) {
            d0 = -(ct[l] * m0);
            d1 = -(ct[l] * m1);
        }
        if (l <= th - 2) {
            T nu1, nu2;
            if constexpr (A == 0) {
                nu1 = un[3 * v + t1];
                nu2 = un[3 * v + t2];
            } else if constexpr (A == 1) {
                nu1 = uj[3 * v + t1];
                nu2 = uj[3 * v + t2];
            } else {  // t1 = x, t2 = y
                nu1 = v < V - 1 ? u[3 * (v + 1)] : kx;
                nu2 = v < V - 1 ? u[3 * (v + 1) + 1] : ky;
            }
            const long pq = pt + fwd;
            const T q0 = mo[2 * pq] - f * nu1;
            const T q1 = mo[2 * pq + 1] + f * nu2;
            d0 += ct[l + 1] * q0;
            d1 += ct[l + 1] * q1;
        }
        h[3 * v + t2] -= d0;
        h[3 * v + t1] -= d1;
        mn[2 * pt] = bt[l] * m0;
        mn[2 * pt + 1] = bt[l] * m1;
    }
}

template <class T, int V>
__device__ __forceinline__ void adj_pml_E(const GridK &g, const AdjAux &x, int i, int j, int k0, const T (&u)[3 * V],
                                          const T (&un)[3 * V], const T (&uj)[3 * V], T kx, T ky, T (&h)[3 * V],
                                          unsigned slabs) {
    for (unsigned sm = slabs; sm; sm &= sm - 1) {
        const int s = __ffs(sm) - 1;
        const int a = g.slab[s].axis;
        if (a == 0) adj_slab_E<T, V, 0>(g, x, s, i, j, k0, u, un, uj, kx, ky, h);
        else if (a == 1) adj_slab_E<T, V, 1>(g, x, s, i, j, k0, u, un, uj, kx, ky, h);
        else adj_slab_E<T, V, 2>(g, x, s, i, j, k0, u, un, uj, kx, ky, h);
    }
}

// Bulk of the transposed H half on a thread's V cells: lam_E (e) -=
// curl_D1(w), w = c mu^-1 lam_H at the cells, wp / wj at plane i-1 / row
// j-1, (kx, ky) = (w_x, w_y) at k0-1.
template <class T, int V>
__device__ __forceinline__ void adj_bulk_H(const GridK &g, int i, int j, int k0, const T (&w)[3 * V],
                                           const T (&wp)[3 * V], const T (&wj)[3 * V], T kx, T ky, T (&e)[3 * V]) {
    const bool xin = i < g.nx - 1, xbk = i > 0;
    const bool yin = j < g.ny - 1, ybk = j > 0;
#pragma unroll
    for (int v = 0; v < V; ++v) {
        const int k = k0 + v;
        const bool zin = k < g.nz - 1, zbk = k > 0;
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
}

// Bulk of the transposed E half on a thread's V cells: lam_H (h) +=
// curl_D2(u), u = c eps^-1 lam_E at the cells, un / uj at plane i+1 / row
// j+1, (kx, ky) = (u_x, u_y) at k0+V.
template <class T, int V>
__device__ __forceinline__ void adj_bulk_E(const GridK &g, int i, int j, int k0, const T (&u)[3 * V],
                                           const T (&un)[3 * V], const T (&uj)[3 * V], T kx, T ky, T (&h)[3 * V]) {
    const bool xn = i < g.nx - 1, xo = i > 0;
    const bool yn = j < g.ny - 1, yo = j > 0;
#pragma unroll
    for (int v = 0; v < V; ++v) {
        const int k = k0 + v;
        const bool zn = k < g.nz - 1, zo = k > 0;
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
}

// Transposed H half: lam_E -= curl_D1(c mu^-1 lam_H) plus the H-side PML
// terms.  g.E / g.H are lam_E / lam_H.  Same tiling and x-march as
// k_update_E (the backward neighbours of w come from plane i-1, row j-1 and
// the lane to the left), over the GridK's tile box.
template <class T, int V>
__global__ void __launch_bounds__(kThreads) k_adj_H(const GridK g, const AdjAux x) {
    constexpr int N = 3 * V;
    const int tz = threadIdx.x, ty = threadIdx.y;
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const int k0 = g.oz + (blockIdx.x * g.TZ + tz) * V;
    const int j = g.oy + blockIdx.y * g.TY + ty;
    const int xa = g.ox + blockIdx.z * g.XC;
    const int xb = min(g.ex, xa + g.XC);
    const bool act = (j < g.ey) && (k0 < g.ez);
    const T c = material_courant<T>(g);  // courant * material factor
    const T *LH = (const T *)g.H;
    T *LE = (T *)g.E;
    const T *__restrict__ MU = (const T *)g.imu;
    const unsigned mask_yz = act ? slab_mask_yz(g, j, k0, V) : 0u;

    alignas(16) T wp[N];  // w at plane i-1
    zero(wp);
    if (act && xa > 0) load_scaled<T, V>(wp, LH, MU, ((size_t)(xa - 1) * ny + j) * nz + k0, c);

    for (int i = xa; i < xb; ++i) {
        const size_t cell0 = ((size_t)i * ny + j) * nz + k0;
        alignas(16) T w[N], wj[N], e[N];
        zero(w);
        zero(wj);
        zero(e);
        if (act) {
            load_scaled<T, V>(w, LH, MU, cell0, c);
            if (j > 0) load_scaled<T, V>(wj, LH, MU, cell0 - nz, c);
            ld_vec(e, LE + 3 * cell0);
        }
        // (w_x, w_y) at k0-1: from the lane to the left, or from memory at a row start
        T kx = __shfl_up_sync(FULL_MASK, w[N - 3], 1);
        T ky = __shfl_up_sync(FULL_MASK, w[N - 2], 1);
        if (tz == 0 && act && k0 > 0) {
            kx = (c * MU[3 * (cell0 - 1)]) * LH[3 * (cell0 - 1)];
            ky = (c * MU[3 * (cell0 - 1) + 1]) * LH[3 * (cell0 - 1) + 1];
        }
        if (act) {
            adj_bulk_H<T, V>(g, i, j, k0, w, wp, wj, kx, ky, e);
            const unsigned slabs = mask_yz | slab_mask_x(g, i);
            if (slabs) adj_pml_H<T, V>(g, x, i, j, k0, w, wp, wj, kx, ky, e, slabs);
            st_vec(LE + 3 * cell0, e);
        }
#pragma unroll
        for (int q = 0; q < N; ++q) wp[q] = w[q];
    }
}

// Transposed E half (bulk and PML part): lam_H += curl_D2(c eps^-1 lam_E)
// plus the E-side PML terms.  Same tiling as k_update_H (forward neighbours
// of u from plane i+1, row j+1 and the lane to the right).  Objects follow in
// k_adj_object.
template <class T, int V>
__global__ void __launch_bounds__(kThreads) k_adj_E(const GridK g, const AdjAux x) {
    constexpr int N = 3 * V;
    const int tz = threadIdx.x, ty = threadIdx.y;
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const int k0 = g.oz + (blockIdx.x * g.TZ + tz) * V;
    const int j = g.oy + blockIdx.y * g.TY + ty;
    const int xa = g.ox + blockIdx.z * g.XC;
    const int xb = min(g.ex, xa + g.XC);
    const bool act = (j < g.ey) && (k0 < g.ez);
    const T c = material_courant<T>(g);  // courant * material factor
    const T *LE = (const T *)g.E;
    T *LH = (T *)g.H;
    const T *__restrict__ IE = (const T *)g.ie;
    const unsigned mask_yz = act ? slab_mask_yz(g, j, k0, V) : 0u;

    alignas(16) T u[N];  // u at plane i
    zero(u);
    if (act && xa < xb) load_scaled<T, V>(u, LE, IE, ((size_t)xa * ny + j) * nz + k0, c);

    for (int i = xa; i < xb; ++i) {
        const size_t cell0 = ((size_t)i * ny + j) * nz + k0;
        alignas(16) T un[N], uj[N], h[N];
        zero(un);
        zero(uj);
        zero(h);
        if (act) {
            if (i + 1 < nx) load_scaled<T, V>(un, LE, IE, cell0 + (size_t)ny * nz, c);
            if (j + 1 < ny) load_scaled<T, V>(uj, LE, IE, cell0 + nz, c);
            ld_vec(h, LH + 3 * cell0);
        }
        // (u_x, u_y) at k0+V: from the lane to the right, or from memory at a row end
        T kx = __shfl_down_sync(FULL_MASK, u[0], 1);
        T ky = __shfl_down_sync(FULL_MASK, u[1], 1);
        if ((tz == g.TZ - 1 || k0 + V >= g.ez) && act && k0 + V < nz) {
            kx = (c * IE[3 * (cell0 + V)]) * LE[3 * (cell0 + V)];
            ky = (c * IE[3 * (cell0 + V) + 1]) * LE[3 * (cell0 + V) + 1];
        }
        if (act) {
            adj_bulk_E<T, V>(g, i, j, k0, u, un, uj, kx, ky, h);
            const unsigned slabs = mask_yz | slab_mask_x(g, i);
            if (slabs) adj_pml_E<T, V>(g, x, i, j, k0, u, un, uj, kx, ky, h, slabs);
            st_vec(LH + 3 * cell0, h);
        }
#pragma unroll
        for (int q = 0; q < N; ++q) u[q] = un[q];
    }
}

// Shell boxes of an interior/shell partition plan, transposed: one thread per
// V cells along z, the bulk and every PML slab's terms of the transposed half
// (the same per-cell arithmetic as k_adj_H / k_adj_E), neighbours read
// through L1/L2.  The slab-free k_adj_H / k_adj_E cover the interior box.

// dst[q] = (c * m[q]) * lam[q] for the 3V values at cell0 (8- or 16-byte loads).
template <class T, int V>
__device__ __forceinline__ void shell_scaled(T (&dst)[3 * V], const T *lam, const T *m, size_t cell0, T c) {
    alignas(16) T l[3 * V], mm[3 * V];
    shell_ld<false>(l, lam + 3 * cell0);
    shell_ld<true>(mm, m + 3 * cell0);
#pragma unroll
    for (int q = 0; q < 3 * V; ++q) dst[q] = (c * mm[q]) * l[q];
}

template <class T, int V>
__global__ void __launch_bounds__(kThreads) k_adj_shell_H(const GridK g, const ShellK sh, const AdjAux x) {
    constexpr int N = 3 * V;
    int i, j, k0;
    unsigned cand;
    if (!shell_cells<V>(sh, i, j, k0, cand)) return;
    const int ny = g.ny, nz = g.nz;
    const size_t cell0 = ((size_t)i * ny + j) * nz + k0;
    const T c = material_courant<T>(g);
    const T *LH = (const T *)g.H;
    T *LE = (T *)g.E;
    const T *MU = (const T *)g.imu;
    alignas(16) T w[N], wp[N], wj[N], e[N];
    zero(wp);
    zero(wj);
    shell_scaled<T, V>(w, LH, MU, cell0, c);
    if (i > 0) shell_scaled<T, V>(wp, LH, MU, cell0 - (size_t)ny * nz, c);
    if (j > 0) shell_scaled<T, V>(wj, LH, MU, cell0 - nz, c);
    shell_ld<false>(e, LE + 3 * cell0);
    T kx = T(0), ky = T(0);
    if (k0 > 0) {
        kx = (c * MU[3 * (cell0 - 1)]) * LH[3 * (cell0 - 1)];
        ky = (c * MU[3 * (cell0 - 1) + 1]) * LH[3 * (cell0 - 1) + 1];
    }
    adj_bulk_H<T, V>(g, i, j, k0, w, wp, wj, kx, ky, e);
    const unsigned slabs = shell_mask<V>(g, cand, i, j, k0);
    if (slabs) adj_pml_H<T, V>(g, x, i, j, k0, w, wp, wj, kx, ky, e, slabs);
    shell_st(LE + 3 * cell0, e);
}

template <class T, int V>
__global__ void __launch_bounds__(kThreads) k_adj_shell_E(const GridK g, const ShellK sh, const AdjAux x) {
    constexpr int N = 3 * V;
    int i, j, k0;
    unsigned cand;
    if (!shell_cells<V>(sh, i, j, k0, cand)) return;
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const size_t cell0 = ((size_t)i * ny + j) * nz + k0;
    const T c = material_courant<T>(g);
    const T *LE = (const T *)g.E;
    T *LH = (T *)g.H;
    const T *IE = (const T *)g.ie;
    alignas(16) T u[N], un[N], uj[N], h[N];
    zero(un);
    zero(uj);
    shell_scaled<T, V>(u, LE, IE, cell0, c);
    if (i + 1 < nx) shell_scaled<T, V>(un, LE, IE, cell0 + (size_t)ny * nz, c);
    if (j + 1 < ny) shell_scaled<T, V>(uj, LE, IE, cell0 + nz, c);
    shell_ld<false>(h, LH + 3 * cell0);
    T kx = T(0), ky = T(0);
    if (k0 + V < nz) {
        kx = (c * IE[3 * (cell0 + V)]) * LE[3 * (cell0 + V)];
        ky = (c * IE[3 * (cell0 + V) + 1]) * LE[3 * (cell0 + V) + 1];
    }
    adj_bulk_E<T, V>(g, i, j, k0, u, un, uj, kx, ky, h);
    const unsigned slabs = shell_mask<V>(g, cand, i, j, k0);
    if (slabs) adj_pml_E<T, V>(g, x, i, j, k0, u, un, uj, kx, ky, h, slabs);
    shell_st(LH + 3 * cell0, h);
}

// PML transposes of one slab on their own (plans whose forward pass runs the
// slabs in kernels of their own): the per-cell terms of adj_slab_E (IS_E,
// transposed E half: lam_H and the E-side adjoint auxiliaries, after k_adj_E)
// or adj_slab_H (lam_E and the H-side ones, after k_adj_H).  The kernel reads
// the adjoint field it does not write, and the current auxiliary buffer.
// The slab normal A is a template parameter and the cell index type I is
// 32-bit whenever the slab has fewer than 2^31 cells (no 64-bit divisions).
template <class T, bool IS_E, int A, class I>
__global__ void __launch_bounds__(kThreads) k_adj_slab(const GridK g, const AdjAux x, int s) {
    const SlabK &S = g.slab[s];
    constexpr int a = A;
    const int th = S.th;
    const int n1 = a == 1 ? th : g.ny, n2 = a == 2 ? th : g.nz;
    const I total = (I)(a == 0 ? th : g.nx) * (I)n1 * (I)n2;
    const T c = material_courant<T>(g);  // courant * material factor
    const T *L = (const T *)(IS_E ? g.E : g.H);  // lam_E (E half) or lam_H (H half), read
    T *O = (T *)(IS_E ? g.H : g.E);              // the adjoint field updated
    const T *__restrict__ M = (const T *)(IS_E ? g.ie : g.imu);
    const T *ao = (const T *)(IS_E ? x.Eo[s] : x.Ho[s]);
    T *an = (T *)(IS_E ? x.En[s] : x.Hn[s]);
    const T *__restrict__ bt = (const T *)(IS_E ? S.bE : S.bH);
    const T *__restrict__ ct = (const T *)(IS_E ? S.cE : S.cH);
    const T f = s < g.nslab_fused ? T(1) : T(0);
    constexpr int t1 = (a + 1) % 3, t2 = (a + 2) % 3;
    // one step along the normal, in cells and in auxiliary pairs (same count)
    const long cstride = a == 0 ? (long)g.ny * g.nz : (a == 1 ? (long)g.nz : 1L);
    const long pstride = cstride;
    for (I t = (I)blockIdx.x * (I)blockDim.x + threadIdx.x; t < total; t += (I)gridDim.x * (I)blockDim.x) {
        const I r = t / (I)n2;
        const int i2 = (int)(t - r * (I)n2), i1 = (int)(r % (I)n1), i0 = (int)(r / (I)n1);
        const int l = a == 0 ? i0 : (a == 1 ? i1 : i2);
        const int gi = a == 0 ? i0 + S.start : i0, gj = a == 1 ? i1 + S.start : i1, gk = a == 2 ? i2 + S.start : i2;
        const size_t cell = ((size_t)gi * g.ny + gj) * g.nz + gk;
        const long pt = slab_pair(g, S, gi, gj, gk);
        const T v1 = (c * M[3 * cell + t1]) * L[3 * cell + t1];
        const T v2 = (c * M[3 * cell + t2]) * L[3 * cell + t2];
        T d0 = T(0), d1 = T(0), a0, a1;
        if (IS_E) {
            a0 = ao[2 * pt] - f * v1;
            a1 = ao[2 * pt + 1] + f * v2;
            if (l >= 1) {
                d0 = -(ct[l] * a0);
                d1 = -(ct[l] * a1);
            }
            if (l <= th - 2) {
                const size_t nc = cell + cstride;
                const long pq = pt + pstride;
                const T q0 = ao[2 * pq] - f * ((c * M[3 * nc + t1]) * L[3 * nc + t1]);
                const T q1 = ao[2 * pq + 1] + f * ((c * M[3 * nc + t2]) * L[3 * nc + t2]);
                d0 += ct[l + 1] * q0;
                d1 += ct[l + 1] * q1;
            }
        } else {
            a0 = ao[2 * pt] + f * v1;
            a1 = ao[2 * pt + 1] - f * v2;
            if (l <= th - 2) {
                d0 = ct[l] * a0;
                d1 = ct[l] * a1;
            }
            if (l >= 1) {
                const size_t pc = cell - cstride;
                const long pq = pt - pstride;
                const T p0 = ao[2 * pq] + f * ((c * M[3 * pc + t1]) * L[3 * pc + t1]);
                const T p1 = ao[2 * pq + 1] - f * ((c * M[3 * pc + t2]) * L[3 * pc + t2]);
                d0 -= ct[l - 1] * p0;
                d1 -= ct[l - 1] * p1;
            }
        }
        O[3 * cell + t2] -= d0;
        O[3 * cell + t1] -= d1;
        an[2 * pt] = bt[l] * a0;
        an[2 * pt + 1] = bt[l] * a1;
    }
}

// u_obj = (d E_after / d curl_H)^T lam_E of one object at cell (i, j, k),
// zero outside its box.  Object: coef0 = courant*inverse_permittivity;
// absorbing: courant*inverse_permittivity/(1+f); anisotropic: courant*M^T.
template <class T>
__device__ __forceinline__ void object_u(const GridK &g, const ItemK &o, const T *LE, int i, int j, int k, T (&u)[3]) {
    u[0] = u[1] = u[2] = T(0);
    if (!in_box(o, i, j, k)) return;
    const size_t cell = ((size_t)i * g.ny + j) * g.nz + k;
    const T l0 = LE[3 * cell], l1 = LE[3 * cell + 1], l2 = LE[3 * cell + 2];
    const size_t li = box_index(o, i, j, k);
    if (o.kind == FDTD_ITEM_OBJECT) {
        const T *cf = (const T *)o.coef[0] + 3 * li;
        u[0] = cf[0] * l0;
        u[1] = cf[1] * l1;
        u[2] = cf[2] * l2;
    } else if (o.kind == FDTD_ITEM_ABSORBING) {
        const T *ci = (const T *)o.coef[1] + 3 * li;
        if constexpr (sizeof(T) == 4) {
            u[0] = ci[0] * l0;
            u[1] = ci[1] * l1;
            u[2] = ci[2] * l2;
        } else {
            const T *opf = (const T *)o.coef[2] + 3 * li;
            u[0] = (ci[0] / opf[0]) * l0;
            u[1] = (ci[1] / opf[1]) * l1;
            u[2] = (ci[2] / opf[2]) * l2;
        }
    } else {
        const T *M = (const T *)o.coef[0] + 9 * li;
        const T c = courant_of<T>(g);
        u[0] = c * (M[0] * l0 + M[3] * l1 + M[6] * l2);
        u[1] = c * (M[1] * l0 + M[4] * l1 + M[7] * l2);
        u[2] = c * (M[2] * l0 + M[5] * l1 + M[8] * l2);
    }
}

// Transpose of one object's E update: lam_H += curl_D2(u_obj) on the cells
// the object's box reaches ([lo-1, hi) per axis), and, with a gradient
// accumulator, grad += courant * curl_H * lam_E on the box
// (anisotropic: grad[a][b] += courant * lam_E[a] * curl_H[b]).
template <class T>
__global__ void k_adj_object(const GridK g, int item, const T *__restrict__ curl, double *grad) {
    const ItemK &o = g.items[item];
    const int a0 = max(0, o.lo[0] - 1), a1 = max(0, o.lo[1] - 1), a2 = max(0, o.lo[2] - 1);
    const int e0 = o.hi[0] - a0, e1 = o.hi[1] - a1, e2 = o.hi[2] - a2;
    const long total = (long)e0 * e1 * e2;
    const T *LE = (const T *)g.E;
    T *LH = (T *)g.H;
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
        const int i = a0 + (int)(t / ((long)e1 * e2)), j = a1 + (int)((t / e2) % e1), k = a2 + (int)(t % e2);
        T u0[3], ux[3], uy[3], uz[3];
        object_u<T>(g, o, LE, i, j, k, u0);
        object_u<T>(g, o, LE, i + 1, j, k, ux);
        object_u<T>(g, o, LE, i, j + 1, k, uy);
        object_u<T>(g, o, LE, i, j, k + 1, uz);
        const bool xn = i < g.nx - 1, xo = i > 0, yn = j < g.ny - 1, yo = j > 0, zn = k < g.nz - 1, zo = k > 0;
        auto D = [](bool nxt, bool own, T vn, T vo) { return (nxt ? vn : T(0)) - (own ? vo : T(0)); };
        const size_t cell = ((size_t)i * g.ny + j) * g.nz + k;
        LH[3 * cell] += D(yn, yo, uy[2], u0[2]) - D(zn, zo, uz[1], u0[1]);
        LH[3 * cell + 1] += D(zn, zo, uz[0], u0[0]) - D(xn, xo, ux[2], u0[2]);
        LH[3 * cell + 2] += D(xn, xo, ux[1], u0[1]) - D(yn, yo, uy[0], u0[0]);
        if (grad != nullptr && in_box(o, i, j, k)) {
            const size_t li = box_index(o, i, j, k);
            const double c = g.courant;
            const double l[3] = {(double)LE[3 * cell], (double)LE[3 * cell + 1], (double)LE[3 * cell + 2]};
            const double cu[3] = {(double)curl[3 * li], (double)curl[3 * li + 1], (double)curl[3 * li + 2]};
            if (o.kind == FDTD_ITEM_ANISOTROPIC) {
                double *gr = grad + 9 * li;
#pragma unroll
                for (int p = 0; p < 3; ++p)
#pragma unroll
                    for (int q = 0; q < 3; ++q) gr[3 * p + q] += c * l[p] * cu[q];
            } else {
                double *gr = grad + 3 * li;
#pragma unroll
                for (int q = 0; q < 3; ++q) gr[q] += c * cu[q] * l[q];
            }
        }
    }
}

// lam_E[box] *= (1-f)/(1+f): the transpose of AbsorbingObject's E scaling.
template <class T>
__global__ void k_adj_absorb_scale(const GridK g, int item) {
    const ItemK &o = g.items[item];
    const int b0 = o.hi[0] - o.lo[0], b1 = o.hi[1] - o.lo[1], b2 = o.hi[2] - o.lo[2];
    const long total = 3L * b0 * b1 * b2;
    T *LE = (T *)g.E;
    const T *r = (const T *)o.coef[0];
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
        const long li = t / 3;
        const int comp = (int)(t % 3);
        const int i = o.lo[0] + (int)(li / ((long)b1 * b2)), j = o.lo[1] + (int)((li / b2) % b1),
                  k = o.lo[2] + (int)(li % b2);
        const size_t at = 3 * (((size_t)i * g.ny + j) * g.nz + k) + comp;
        LE[at] = LE[at] * r[t];
    }
}

// Detector seeds: lam[cells[p]][c] += seed[p][c] (atomic: detectors may share cells).
template <class T>
__global__ void k_adj_seed_probe(T *lam, const int64_t *__restrict__ cells, int n, const T *__restrict__ seed) {
    const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (t >= 3L * n) return;
    atomicAdd(lam + 3 * cells[t / 3] + (t % 3), seed[t]);
}

// DFT seeds, the transpose of acc[f] += E * (phase_re, phase_im):
// lam_E[cell][c] += sum_f (g_re * phase_re + g_im * phase_im), g = dL/d acc.
template <class T>
__global__ void k_adj_seed_dft(T *lam, int ny, int nz, fdtd_dft_desc d, const double *__restrict__ gacc,
                               const double *__restrict__ phase) {
    const int b0 = d.hi[0] - d.lo[0], b1 = d.hi[1] - d.lo[1], b2 = d.hi[2] - d.lo[2];
    const long ncell = (long)b0 * b1 * b2;
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < ncell * 3; t += (long)gridDim.x * blockDim.x) {
        const long cell = t / 3;
        const int comp = (int)(t % 3);
        const int i = d.lo[0] + (int)(cell / ((long)b1 * b2)), j = d.lo[1] + (int)((cell / b2) % b1),
                  k = d.lo[2] + (int)(cell % b2);
        double s = 0.0;
        for (int f = 0; f < d.n_freq; ++f) {
            const double cs = phase[2 * (d.phase_offset + f)], sn = phase[2 * (d.phase_offset + f) + 1];
            const double *gg = gacc + 2 * ((size_t)f * ncell * 3 + t);
            s = fma(gg[0], cs, fma(gg[1], sn, s));
        }
        const size_t at = 3 * (((size_t)i * ny + j) * nz + k) + comp;
        lam[at] = lam[at] + (T)s;
    }
}

// Hard source cells: lam[box][comp] = 0 (the forward value was overwritten).
template <class T>
__global__ void k_adj_zero_box(const GridK g, int item, T *lam) {
    const ItemK &s = g.items[item];
    const int b0 = s.hi[0] - s.lo[0], b1 = s.hi[1] - s.lo[1], b2 = s.hi[2] - s.lo[2];
    const long total = (long)b0 * b1 * b2;
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
        const int i = s.lo[0] + (int)(t / ((long)b1 * b2)), j = s.lo[1] + (int)((t / b2) % b1),
                  k = s.lo[2] + (int)(t % b2);
        lam[3 * (((size_t)i * g.ny + j) * g.nz + k) + s.comp] = T(0);
    }
}

// Transpose of the periodic copy F[dst] = F[src]: lam[src] += lam[dst]; lam[dst] = 0.
template <class T>
__global__ void k_adj_periodic(T *lam, int nx, int ny, int nz, int axis, int dst, int src) {
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
        lam[3 * cs + comp] += lam[3 * cd + comp];
        lam[3 * cd + comp] = T(0);
    }
}

// Auxiliary increment of a slab corrected after a periodic copy, at its
// place in the transposed boundary order: E side mu0 -= u_t1, mu1 += u_t2;
// H side nu0 += w_t1, nu1 -= w_t2.
template <class T, bool IS_E>
__global__ void k_adj_slab_inc(const GridK g, int s, T *aux) {
    const SlabK &S = g.slab[s];
    const int a = S.axis;
    const int n0 = a == 0 ? S.th : g.nx, n1 = a == 1 ? S.th : g.ny, n2 = a == 2 ? S.th : g.nz;
    const int p2 = a == 2 ? S.thp : g.nz;
    const long total = (long)n0 * n1 * n2;
    const T c = material_courant<T>(g);  // courant * material factor
    const T *L = (const T *)(IS_E ? g.E : g.H);
    const T *M = (const T *)(IS_E ? g.ie : g.imu);
    const int t1 = (a + 1) % 3, t2 = (a + 2) % 3;
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
        const int i0 = (int)(t / ((long)n1 * n2)), i1 = (int)((t / n2) % n1), i2 = (int)(t % n2);
        const int gi = a == 0 ? i0 + S.start : i0, gj = a == 1 ? i1 + S.start : i1, gk = a == 2 ? i2 + S.start : i2;
        const size_t cell = ((size_t)gi * g.ny + gj) * g.nz + gk;
        const size_t pt = ((size_t)i0 * n1 + i1) * p2 + i2;
        const T q1 = (c * M[3 * cell + t1]) * L[3 * cell + t1];
        const T q2 = (c * M[3 * cell + t2]) * L[3 * cell + t2];
        if (IS_E) {
            aux[2 * pt] -= q1;
            aux[2 * pt + 1] += q2;
        } else {
            aux[2 * pt] += q1;
            aux[2 * pt + 1] -= q2;
        }
    }
}

// curl_H(H) on an object's box (fdtd/grid.py:54-76 differences), for the
// gradient of the reverse pass: out[box cell][c].
template <class T>
__global__ void k_capture_curl(const GridK g, int item, T *out) {
    const ItemK &o = g.items[item];
    const int b0 = o.hi[0] - o.lo[0], b1 = o.hi[1] - o.lo[1], b2 = o.hi[2] - o.lo[2];
    const long total = (long)b0 * b1 * b2;
    const T *H = (const T *)g.H;
    const long sx = 3L * g.ny * g.nz, sy = 3L * g.nz;
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
        const int i = o.lo[0] + (int)(t / ((long)b1 * b2)), j = o.lo[1] + (int)((t / b2) % b1),
                  k = o.lo[2] + (int)(t % b2);
        const T *h = H + 3 * (((size_t)i * g.ny + j) * g.nz + k);
        const T dxHy = i > 0 ? h[1] - h[1 - sx] : T(0);
        const T dxHz = i > 0 ? h[2] - h[2 - sx] : T(0);
        const T dyHx = j > 0 ? h[0] - h[-sy] : T(0);
        const T dyHz = j > 0 ? h[2] - h[2 - sy] : T(0);
        const T dzHx = k > 0 ? h[0] - h[-3] : T(0);
        const T dzHy = k > 0 ? h[1] - h[-2] : T(0);
        out[3 * t] = dyHz - dzHy;
        out[3 * t + 1] = dzHx - dxHz;
        out[3 * t + 2] = dxHy - dyHx;
    }
}

}  // namespace fdtd
