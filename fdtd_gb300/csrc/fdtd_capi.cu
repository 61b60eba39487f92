// C ABI of the GB300 FDTD library (declared in include/fdtd_gb300.h):
// descriptor validation, launch tiling, per-CTA object/source lists and
// dispatch to the per-precision launch sequences.
#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

#include "fdtd_kernels.cuh"
#include "fdtd_persistent.cuh"
#include "fdtd_plan.hpp"

struct fdtd_plan {
    fdtd::Plan p;
};

namespace fdtd {

static thread_local int g_last_cuda = 0;
void set_last_cuda_error(int e) { g_last_cuda = e; }

static int cuda_fail(cudaError_t e) {
    g_last_cuda = (int)e;
    return FDTD_ERR_CUDA;
}

static int next_pow2(int v) {
    int p = 1;
    while (p < v) p <<= 1;
    return p;
}

static bool aligned16(const void *ptr) { return ((uintptr_t)ptr & 15u) == 0; }

// Threads along z of a register-streaming tile for zt threads' worth of
// cells: the next power of two up to 32, or 16 where that pads less (config 5,
// 48 threads: 32-wide tiles leave a quarter of the threads idle).
static int tile_width(int zt) {
    if (zt <= 32) return next_pow2(zt);
    const int pad32 = (zt + 31) / 32 * 32 - zt, pad16 = (zt + 15) / 16 * 16 - zt;
    return pad16 < pad32 ? 16 : 32;
}

// Planes per CTA of the register-streaming kernels: at most 32, and fewer
// until the grid has eight waves of CTAs (a chunk re-reads one halo plane, a
// partly filled last wave idles SMs).  Measured: 2D 8192^2 float32, 2 waves of
// 432-plane chunks 39.5, 27 waves of 32-plane chunks 58.0 Gcell/s; config 4
// (128^3, 16 columns) one plane per chunk 20.9 vs 19.3 with four.
static int register_chunk(int nx, long cols, long wave) {
    long chunks = (8 * wave + cols - 1) / cols;
    chunks = std::max(chunks, ((long)nx + 31) / 32);
    chunks = std::max(1L, std::min(chunks, (long)nx));
    return (int)((nx + chunks - 1) / chunks);
}

// Padded 4-value rows of the shared-memory material table of a staged pass.
static int mat_lut_rows(int mat) { return mat == MAT_IDS ? 256 : (mat == MAT_UNIFORM ? 1 : 0); }

static bool box_ok(const int32_t lo[3], const int32_t hi[3], int nx, int ny, int nz) {
    const int n[3] = {nx, ny, nz};
    for (int a = 0; a < 3; ++a)
        if (lo[a] < 0 || hi[a] > n[a] || lo[a] >= hi[a]) return false;
    return true;
}

// Ranges of CTA coordinates that a box touches, for the per-CTA lists.
struct Tiling {
    int V, TZ, TY, XC, gz, gy, gx;
    int o[3], e[3];  // the box of cells the tiles cover, [o, e) along x, y, z
};

// With `halo`, a CTA also covers the cell past its tile along each axis (the
// one-pass step recomputes the new E there), so an item starting at a tile's
// first cell is listed for the tile before it as well.
// The tile ranges are inclusive, in tile coordinates of the tiling's box; an
// item outside the box gets an empty range.
static void cta_range(const Tiling &t, const int32_t lo[3], const int32_t hi[3], int r[6], bool halo = false) {
    const int zc = t.V * t.TZ, h = halo ? 1 : 0;
    const int unit[3] = {t.XC, t.TY, zc};
    for (int a = 0; a < 3; ++a) {
        const int l = std::max(lo[a] - h, t.o[a]) - t.o[a], u = std::min(hi[a], t.e[a]) - t.o[a];
        const int q = 2 * (2 - a);  // r: z range, y range, x range
        if (u <= l) {
            for (int k = 0; k < 6; k += 2) {
                r[k] = 0;
                r[k + 1] = -1;
            }
            return;
        }
        r[q] = l / unit[a];
        r[q + 1] = (u - 1) / unit[a];
    }
}

// CSR lists: for every CTA, the indices (into the device item array) of the
// items whose box intersects the CTA's cells (and its halo), in item order.
static void build_csr(const Tiling &t, const std::vector<ItemK> &items, int first, int count,
                      std::vector<int> &off, std::vector<int> &idx, bool halo = false) {
    const long ncta = (long)t.gz * t.gy * t.gx;
    off.assign(ncta + 1, 0);
    idx.clear();
    std::vector<int> cnt(ncta, 0);
    for (int q = first; q < first + count; ++q) {
        int r[6];
        cta_range(t, items[q].lo, items[q].hi, r, halo);
        for (int cx = r[4]; cx <= r[5]; ++cx)
            for (int cy = r[2]; cy <= r[3]; ++cy)
                for (int cz = r[0]; cz <= r[1]; ++cz) cnt[cz + t.gz * (cy + (long)t.gy * cx)]++;
    }
    for (long c = 0; c < ncta; ++c) off[c + 1] = off[c] + cnt[c];
    idx.assign(off[ncta], 0);
    std::vector<int> fill(off.begin(), off.end() - 1);
    for (int q = first; q < first + count; ++q) {
        int r[6];
        cta_range(t, items[q].lo, items[q].hi, r, halo);
        for (int cx = r[4]; cx <= r[5]; ++cx)
            for (int cy = r[2]; cy <= r[3]; ++cy)
                for (int cz = r[0]; cz <= r[1]; ++cz) idx[fill[cz + t.gz * (cy + (long)t.gy * cx)]++] = q;
    }
}

static ItemK to_item(const fdtd_item_desc &d) {
    ItemK it{};
    it.kind = d.kind;
    it.comp = d.comp;
    it.column = d.column;
    it.source = d.source;
    for (int a = 0; a < 3; ++a) {
        it.lo[a] = d.lo[a];
        it.hi[a] = d.hi[a];
    }
    it.bny = d.hi[1] - d.lo[1];
    it.bnz = d.hi[2] - d.lo[2];
    it.weight = d.weight;
    for (int q = 0; q < 3; ++q) it.coef[q] = d.coef[q];
    it.aux = d.aux;
    return it;
}

static bool touches_periodic_plane(const ItemK &it, const std::vector<int> &periodic_axes, const int n[3]) {
    for (int a : periodic_axes) {
        if (n[a] <= 1) continue;
        if (it.lo[a] == 0 || it.hi[a] == n[a]) return true;
    }
    return false;
}

static int create(const fdtd_grid_desc *d, Plan &p) {
    if (d->abi_version != FDTD_ABI_VERSION) return FDTD_ERR_ARGUMENT;
    if (d->precision < FDTD_FLOAT32 || d->precision > FDTD_FLOAT64) return FDTD_ERR_ARGUMENT;
    if (d->nx < 1 || d->ny < 1 || d->nz < 1) return FDTD_ERR_ARGUMENT;
    if (!d->E || !d->H || !d->inv_eps || !d->inv_mu) return FDTD_ERR_ARGUMENT;
    const bool comp = d->precision == FDTD_FLOAT32C;
    if (comp != (d->E_lo != nullptr) || comp != (d->H_lo != nullptr)) return FDTD_ERR_ARGUMENT;
    if (d->n_boundaries < 0 || d->n_boundaries > FDTD_MAX_BOUNDARIES) return FDTD_ERR_ARGUMENT;
    if (d->n_objects < 0 || d->n_sources_E < 0 || d->n_sources_H < 0 || d->n_columns < 0 ||
        d->n_probe_cells < 0 || d->n_dft < 0 || d->n_phase_columns < 0 || d->x_chunk < 0 ||
        d->n_current_cells < 0 || (d->n_current_cells && !d->current_cells))
        return FDTD_ERR_ARGUMENT;
    if ((d->n_objects && !d->objects) || (d->n_sources_E && !d->sources_E) || (d->n_sources_H && !d->sources_H) ||
        (d->n_probe_cells && !d->probe_cells) || (d->n_dft && !d->dft))
        return FDTD_ERR_ARGUMENT;
    const int n[3] = {d->nx, d->ny, d->nz};
    const size_t esize = d->precision == FDTD_FLOAT64 ? 8 : 4;

    GridK &g = p.k;
    memset(&g, 0, sizeof(g));
    p.precision = d->precision;
    p.has_feedback = 0;
    p.n_current = 0;
    g.nx = d->nx;
    g.ny = d->ny;
    g.nz = d->nz;
    g.ex = d->nx;  // tiles cover the whole grid unless the plan partitions it
    g.ey = d->ny;
    g.ez = d->nz;
    g.courant = d->courant;
    g.courant_f = (float)d->courant;
    g.E = d->E;
    g.H = d->H;
    g.Elo = d->E_lo;
    g.Hlo = d->H_lo;
    g.ie = d->inv_eps;
    g.imu = d->inv_mu;
    if (d->materials_scaled != 0 && d->materials_scaled != 1) return FDTD_ERR_ARGUMENT;
    if (d->materials_scaled && d->precision != FDTD_FLOAT64) return FDTD_ERR_UNSUPPORTED;
    g.scaled = d->materials_scaled;
    // compact material copies: validated here, used only by the staged passes
    int mat_want[2] = {MAT_FULL, MAT_FULL};
    {
        const void *tab[2] = {d->eps_table, d->mu_table};
        const int nt[2] = {d->n_eps_table, d->n_mu_table};
        const uint8_t *idx[2] = {d->eps_index, d->mu_index};
        for (int q = 0; q < 2; ++q) {
            if (nt[q] < 0 || nt[q] > 256) return FDTD_ERR_ARGUMENT;
            if (nt[q] == 0) continue;
            if (!tab[q] || (!idx[q] && nt[q] != 1)) return FDTD_ERR_ARGUMENT;
            if (idx[q] && (d->nz % 16 != 0 || !aligned16(idx[q]))) continue;  // no index map: full arrays
            mat_want[q] = idx[q] ? MAT_IDS : MAT_UNIFORM;
        }
    }

    // boundaries: PML slabs in order, periodic axes, the first periodic position
    int first_periodic = d->n_boundaries;
    std::vector<int> slab_pos, periodic_axes;
    for (int b = 0; b < d->n_boundaries; ++b) {
        const fdtd_boundary_desc &bd = d->boundaries[b];
        if (bd.axis < 0 || bd.axis > 2) return FDTD_ERR_ARGUMENT;
        if (bd.kind == FDTD_BOUNDARY_PML) {
            if (g.nslab >= kMaxSlabs) return FDTD_ERR_UNSUPPORTED;
            if (bd.thickness < 1 || bd.thickness > n[bd.axis]) return FDTD_ERR_ARGUMENT;
            if (!bd.psi_E || !bd.psi_H || !bd.b_E || !bd.c_E || !bd.b_H || !bd.c_H) return FDTD_ERR_ARGUMENT;
            SlabK &S = g.slab[g.nslab];
            S.axis = bd.axis;
            S.high = bd.high ? 1 : 0;
            S.th = bd.thickness;
            S.start = bd.high ? n[bd.axis] - bd.thickness : 0;
            S.thp = bd.axis == 2 ? bd.thickness + (bd.thickness & 1) : bd.thickness;
            S.psiE = bd.psi_E;
            S.psiH = bd.psi_H;
            S.psiE_rd = bd.psi_E;
            S.psiH_rd = bd.psi_H;
            S.bE = bd.b_E;
            S.cE = bd.c_E;
            S.bH = bd.b_H;
            S.cH = bd.c_H;
            slab_pos.push_back(b);
            g.nslab++;
        } else if (bd.kind == FDTD_BOUNDARY_PERIODIC) {
            if (first_periodic == d->n_boundaries) first_periodic = b;
            periodic_axes.push_back(bd.axis);
        } else {
            return FDTD_ERR_ARGUMENT;
        }
    }
    g.nslab_fused = 0;
    for (int s = 0; s < g.nslab; ++s)
        if (slab_pos[s] < first_periodic) g.nslab_fused = s + 1;
    bool slab_after_periodic = g.nslab_fused < g.nslab;
    for (int b = first_periodic, s = g.nslab_fused; b < d->n_boundaries; ++b) {
        const fdtd_boundary_desc &bd = d->boundaries[b];
        EpiOp op{};
        if (bd.kind == FDTD_BOUNDARY_PERIODIC) {
            if (n[bd.axis] <= 1) continue;  // copying a plane onto itself
            op.kind = EPI_COPY;
            op.axis = bd.axis;
        } else {
            op.kind = EPI_SLAB;
            op.slab = s++;
        }
        p.epi_E.push_back(op);
        p.epi_H.push_back(op);
    }
    // the adjoint undoes these boundary stages in reverse order
    p.adj_E.assign(p.epi_E.rbegin(), p.epi_E.rend());
    p.adj_H = p.adj_E;
    for (int s = 0; s < g.nslab; ++s) p.slab_boundary[s] = slab_pos[s];

    // tiling
    int dev = 0, n_sm = 152, optin = 0;
    cudaError_t ce = cudaGetDevice(&dev);
    if (ce != cudaSuccess) return cuda_fail(ce);
    cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    const int vmax = d->precision == FDTD_FLOAT64 ? PF64::V : PF32::V;
    bool vec = (d->nz % vmax) == 0 && aligned16(d->E) && aligned16(d->H) && aligned16(d->inv_eps) &&
               aligned16(d->inv_mu) && (!comp || (aligned16(d->E_lo) && aligned16(d->H_lo)));
    if (d->variant < 0 || d->variant > 2) return FDTD_ERR_ARGUMENT;
    if (d->variant == 2 && !vec) return FDTD_ERR_UNSUPPORTED;
    if (d->pml_mode < 0 || d->pml_mode > 4) return FDTD_ERR_ARGUMENT;
    const int pml_base = d->pml_mode;
    // Mode 4: interior/shell partition.  The box inside every PML slab (its
    // z faces on 16-cell boundaries, so that the staged passes' tensor-map
    // coordinates stay aligned) runs the slab-free fused pass; the rest of
    // the grid, cut into up to six boxes, runs one kernel with every slab
    // (one thread per one or two cells).  Every cell is then read and
    // written once per half step (the split slab kernels re-read each slab
    // cell the bulk pass has just written), and each cell still gets bulk,
    // objects, slabs in registration order and sources in that order, as in
    // every mode.  Automatic on grids of 8M cells or more whose shell holds
    // at least a fifth of the cells, a tenth in float64 (float32 ms per step, split slabs vs
    // partition: config 2 0.443 vs 0.375, config 5 0.618 vs 0.608; float64
    // config 2 1.74 vs 1.49; float32c config 5 1.10 vs 0.85; config 3, 12 %
    // of its cells in the shell, stays faster with its slabs split: 5.47 vs
    // 5.77 float32).
    int ibox[6] = {0, 0, 0, d->nx, d->ny, d->nz};  // tile box of the fused pass: [lo, hi) per axis
    p.n_shell = 0;
    p.shell_overlap = 0;
    const long ncell = (long)d->nx * d->ny * d->nz;
    if (pml_base == 4 || pml_base == 0) {
        int lo[3] = {0, 0, 0}, hi[3] = {d->nx, d->ny, d->nz};
        for (int s = 0; s < g.nslab; ++s) {
            const SlabK &S = g.slab[s];
            if (S.high) hi[S.axis] = std::min(hi[S.axis], S.start);
            else lo[S.axis] = std::max(lo[S.axis], S.start + S.th);
        }
        // z faces: on 16-cell boundaries where a staged interior reads a
        // one-byte material index map (its tensor-map x coordinate is in
        // bytes), and for float fields (a row start on a 32-byte sector
        // boundary: config 5 float32c 0.804 vs 0.832 ms per step with the
        // interior from z = 20); float64 on 4-cell boundaries (96 bytes; the
        // field maps' x coordinate, 3 k esize / 8, is then even; config 5
        // float64 2.42 vs 2.47 ms with 12 fewer shell cells per z face)
        const bool stg = d->variant == 2 || (d->variant == 0 && d->precision == FDTD_FLOAT32 &&
                                              mat_want[0] != MAT_FULL && mat_want[1] != MAT_FULL);
        const bool idx = stg && (mat_want[0] == MAT_IDS || mat_want[1] == MAT_IDS);
        const int za = idx || d->precision != FDTD_FLOAT64 ? 16 : 4;
        lo[2] = (lo[2] + za - 1) / za * za;
        hi[2] = hi[2] / vmax * vmax;
        const bool inner = lo[0] < hi[0] && lo[1] < hi[1] && lo[2] < hi[2];
        const bool ok = g.nslab > 0 && !slab_after_periodic && vec && inner;
        if (pml_base == 4 && !ok) return FDTD_ERR_UNSUPPORTED;
        bool want = ok && pml_base == 4;
        if (ok && pml_base == 0 && ncell >= (8L << 20)) {
            // a fifth of the cells in the shell; float64 (arithmetic bound,
            // register-streaming interior) from a tenth (config 3: 29.1 vs
            // 30.4 ms per step)
            const long inside = (long)(hi[0] - lo[0]) * (hi[1] - lo[1]) * (hi[2] - lo[2]);
            const long frac = d->precision == FDTD_FLOAT64 ? 10 : 5;
            want = frac * (ncell - inside) >= ncell;
        }
        if (want) {
            for (int a = 0; a < 3; ++a) {
                ibox[a] = lo[a];
                ibox[3 + a] = hi[a];
            }
            p.n_shell = -1;  // boxes cut below, once the interior tiling is known
        }
    }
    // PML slabs in kernels of their own let the fused pass run without slab
    // work (the staged kernels reach the HBM roofline there); the slab kernels
    // re-read only the slab cells.  The per-cell order of the reference is
    // kept: bulk and objects in the fused pass, then every boundary in
    // registration order, then the sources.  Automatic choice: on grids below
    // 8M cells a step takes tens of microseconds and the extra launches per
    // slab cost more than the divergence they remove.
    //
    // Mode 3 keeps the slabs normal to x or y that lead the boundary list
    // inside the fused pass (their extra work is the same for every warp of a
    // CTA) and splits off the rest.  With full material arrays and one CTA per
    // SM it measured slower than splitting every slab (config 3: 58.0 vs 63.2
    // Gcell/s).  With compact material copies and two CTAs per SM it is the
    // faster float32 plan on config 3 (80.8 vs 78.7 Gcell/s) but not the
    // faster float64 (15.1 vs 15.3) or float32c (47.0 vs 48.2) plan, whose
    // fused passes are arithmetic-bound, and keeping leading x slabs as well
    // slowed config 5 (x, y, z slab pairs) by 29%: whole slab planes make the
    // CTAs that hold them late, and their auxiliary rows enlarge every stage.
    // The automatic choice therefore keeps only leading y slabs, for float32
    // with compact materials.
    // 2D grids (nz = 1) of 8M cells and more split too (8192^2 float32: 63.1
    // vs 58.0 Gcell/s with 32-plane chunks)
    p.pml_split = g.nslab > 0 && p.n_shell == 0 &&
                  (pml_base >= 2 ||
                   (pml_base == 0 && ncell >= (8L << 20) &&
                    ((vec && (long)d->nz * 3 * (long)esize >= 768) || d->nz == 1)));
    int kfs = 0;  // leading slabs kept in the fused pass when split
    const bool auto_keep = pml_base == 0 && d->precision == FDTD_FLOAT32 && mat_want[0] != MAT_FULL &&
                           mat_want[1] != MAT_FULL;
    if (p.pml_split && (pml_base == 3 || auto_keep)) {
        while (kfs < d->n_boundaries && d->boundaries[kfs].kind == FDTD_BOUNDARY_PML &&
               (auto_keep ? d->boundaries[kfs].axis == 1 : d->boundaries[kfs].axis != 2))
            ++kfs;
        if (kfs == g.nslab) {  // nothing left to split off
            p.pml_split = 0;
            kfs = 0;
        }
    }
    p.fused_slabs = kfs;
    if (p.pml_split) {
        p.epi_E.clear();
        for (int b = kfs, s = kfs; b < d->n_boundaries; ++b) {
            const fdtd_boundary_desc &bd = d->boundaries[b];
            EpiOp op{};
            if (bd.kind == FDTD_BOUNDARY_PERIODIC) {
                if (n[bd.axis] <= 1) continue;
                op.kind = EPI_COPY;
                op.axis = bd.axis;
            } else {
                op.kind = EPI_PML;
                op.slab = s++;
            }
            p.epi_E.push_back(op);
        }
        p.epi_H = p.epi_E;
    }
    // extents of the fused pass's tile box
    const int bnx = ibox[3] - ibox[0], bny = ibox[4] - ibox[1];
    int bnz = ibox[5] - ibox[2];
    // slabs the fused pass handles (none in the interior of a partition)
    const int ks = p.n_shell ? 0 : (p.pml_split ? kfs : g.nslab);
    g.n_staged = 0;
    for (int s = 0; s < ks; ++s) g.staged_slab[g.n_staged++] = s;
    // automatic choice: the TMA-staged kernels reach the HBM roofline on grids
    // without PML; with PML slabs the warps holding slab cells do more work per
    // plane and the staged kernels' per-plane CTA barrier makes the whole tile
    // wait for them, so the register-streaming kernels are faster there
    bool fused_z = false;  // a z slab inside the fused pass (divergent warps)
    for (int s = 0; s < ks; ++s) fused_z |= g.slab[s].axis == 2;
    // a partition's interior: the staged pass for float32 with compact
    // materials on both passes, else the register-streaming one (measured:
    // config 2, full permittivity, 0.375 vs 0.494 ms per step; config 5
    // float64 2.49 vs 2.57, float32c 0.85 vs 0.95; float32 config 5 with
    // compact materials 0.608 vs 0.636)
    const bool shell_tma = d->precision == FDTD_FLOAT32 && mat_want[0] != MAT_FULL && mat_want[1] != MAT_FULL;
    const bool tma = d->variant == 2 || (d->variant == 0 && vec && !fused_z && (long)bnz * 3 * (long)esize >= 768 &&
                                         (p.n_shell == 0 || shell_tma));
    Tiling t{};
    for (int a = 0; a < 3; ++a) {
        t.o[a] = ibox[a];
        t.e[a] = ibox[3 + a];
    }
    int ctas_per_sm = 2;
    bool use_tma = tma;
    // staged passes: ring depth, stage bytes and auxiliary slot offsets of the E (0) and H (1) pass
    int pass_stages[2] = {0, 0}, pass_stage_bytes[2] = {0, 0};
    int pass_psi_off[2][kMaxSlabs] = {{0}};
    if (use_tma) {
        t.V = vmax;
        if (d->tile_rows != 0 && d->tile_rows != 4 && d->tile_rows != 8 && d->tile_rows != 16)
            return FDTD_ERR_ARGUMENT;
        // tile shapes: 32 threads along z x 8 (or 4) rows, or 16 x 16 (one
        // halo row per 16 rows).  Stage layout of a tile height: field tiles, then one PML auxiliary
        // slot per group of slabs of one axis that never meet in the same tile
        // (rows copied per stage); returns the stage bytes and fills the slot
        // offsets and pitches of the plan
        const int lut_rows = std::max(mat_lut_rows(mat_want[0]), mat_lut_rows(mat_want[1]));
        auto stage_layout = [&](int TY, int TZ, int m0 = -1, int *off_out = nullptr) -> size_t {
            const int Zc = TZ * t.V;
            // field part: the larger of the two passes', or one pass's (m0: its material mode)
            const size_t field = m0 < 0 ? tma_stage_bytes(d->precision, TY, mat_want[0], mat_want[1])
                                        : tma_stage_bytes(d->precision, TY, m0, m0);
            struct Slot {
                int axis;
                size_t bytes;
                std::vector<std::pair<int, int>> ranges;
                size_t off;
            };
            std::vector<Slot> slots;
            int slot_of[kMaxSlabs] = {0};
            for (int s = 0; s < ks; ++s) {
                const SlabK &S = g.slab[s];
                const int unit = S.axis == 0 ? 1 : (S.axis == 1 ? TY : Zc);
                const std::pair<int, int> rg(S.start / unit, (S.start + S.th - 1) / unit);
                const int pitch = S.axis == 2 ? 2 * S.thp : 2 * Zc;
                const size_t bytes = (size_t)TY * pitch * esize;
                g.psi_pitch[s] = pitch;
                int found = -1;
                for (int q = 0; q < (int)slots.size() && found < 0; ++q) {
                    if (slots[q].axis != S.axis) continue;
                    bool disjoint = true;
                    for (auto &o : slots[q].ranges)
                        if (!(rg.second < o.first || o.second < rg.first)) disjoint = false;
                    if (disjoint) found = q;
                }
                if (found < 0) {
                    slots.push_back(Slot{S.axis, 0, {}, 0});
                    found = (int)slots.size() - 1;
                }
                slots[found].ranges.push_back(rg);
                slots[found].bytes = std::max(slots[found].bytes, bytes);
                slot_of[s] = found;
            }
            size_t stage = field;
            for (auto &sl : slots) {
                sl.off = stage;
                stage += (sl.bytes + 127) & ~(size_t)127;
            }
            for (int s = 0; s < ks; ++s) (off_out ? off_out : g.psi_off)[s] = (int)slots[slot_of[s]].off;
            return stage;
        };
        int coef = 0;
        for (int s = 0; s < ks; ++s) {
            g.coef_off[s] = coef;
            coef += 2 * g.slab[s].th;
        }
        g.coef_values = (size_t)coef * esize <= 16384 ? coef : 0;
        // shared memory after the ring: barriers, b/c tables, then (16-byte
        // aligned) the material table of the pass: 256 padded rows for
        // indices, so that every index byte reads inside it
        const size_t extra = (size_t)g.coef_values * esize + (size_t)lut_rows * 4 * esize + 16 + 128;
        const long per_sm = 228L * 1024;  // shared memory of one SM
        auto smem_of = [&](size_t stage, int S) { return (size_t)S * stage + (size_t)S * 8 + extra; };
        auto resident = [&](size_t smem) { return std::max(1, (int)(per_sm / (long)(smem + 1024))); };
        // ring stages that let two CTAs share an SM (0 if fewer than 3 fit)
        auto stages_for_two = [&](size_t stage) {
            const long room = per_sm / 2 - 1024 - (long)extra;
            const long S2 = std::min<long>(6, room / (long)(stage + 8));
            return S2 >= 3 && smem_of(stage, (int)S2) <= (size_t)optin ? (int)S2 : 0;
        };
        // tile height.  Explicit: as asked (16 rows are 16 threads wide).
        // Automatic: 16 x 16 tiles where they waste less of the z extent
        // than 32-wide ones (config 5: nz = 192) and the stage holds their
        // slab rows (at most 4 slabs, 64 lanes' worth); else 8 rows, or 4
        // when only 4-row stages let two CTAs share an SM.  One CTA of 8 warps
        // leaves the staged passes latency-bound once the per-cell bytes
        // drop (one-byte material indices): two CTAs per SM measured 77 vs
        // 67 Gcell/s on config 3 (float32) and 15.2 vs 12.6 (float64), and
        // the same as one CTA with full material arrays
        const int staged_slabs = ks;  // slabs whose auxiliary rows the stage holds
        int rows = d->tile_rows;
        if (rows == 16 && staged_slabs > 4) {
            if (d->variant == 2) return FDTD_ERR_UNSUPPORTED;
            rows = 8;
        }
        if (rows == 0) {
            const long z32 = 32L * vmax, z16 = 16L * vmax;
            const long waste32 = (bnz + z32 - 1) / z32 * z32 - bnz;
            const long waste16 = (bnz + z16 - 1) / z16 * z16 - bnz;
            if (waste16 < waste32 && staged_slabs <= 4) {
                rows = 16;
            } else {
                rows = 8;
                if (!stages_for_two(stage_layout(8, 32)) && stages_for_two(stage_layout(4, 32))) rows = 4;
            }
        }
        t.TY = rows;
        t.TZ = rows == 16 ? 16 : 32;
        const size_t stage = stage_layout(t.TY, t.TZ);
        g.stage_bytes = (int)stage;
        int S = d->stages;
        if (S == 0) {
            S = stages_for_two(stage);
            if (S == 0) S = (int)std::max<long>(0, std::min<long>(6, ((long)optin - (long)extra) / (long)(stage + 8)));
        }
        const size_t smem = smem_of(stage, S);
        if (S < 2 || smem > (size_t)optin) {
            if (d->variant == 2) return FDTD_ERR_UNSUPPORTED;
            use_tma = false;  // automatic choice: too little shared memory, use the register kernels
        } else {
            g.stages = S;
            ctas_per_sm = resident(smem);
            p.variant = 2;
            // each pass lays out its own stages inside the same shared memory:
            // a pass whose stage is smaller than the larger one gets a deeper
            // ring (the H pass holds two planes at once, so its loads in flight
            // are one stage fewer; config 2 with full permittivity runs its H
            // pass on 4-row tiles sized for the E pass's material tile)
            for (int pass = 0; pass < 2; ++pass) {
                const size_t sb = stage_layout(t.TY, t.TZ, mat_want[pass], pass_psi_off[pass]);
                int sp = S;
                if (d->stages == 0)
                    for (int q = 8; q > S; --q)
                        if (smem_of(sb, q) <= smem) {
                            sp = q;
                            break;
                        }
                pass_stage_bytes[pass] = (int)sb;
                pass_stages[pass] = sp;
            }
            stage_layout(t.TY, t.TZ);  // g.psi_off of the shared layout again
            g.mat_E = mat_want[0];
            g.mat_H = mat_want[1];
            g.mlut_E = d->eps_table;
            g.mlut_H = d->mu_table;
            g.nlut_E = g.mat_E == MAT_FULL ? 0 : d->n_eps_table;
            g.nlut_H = g.mat_H == MAT_FULL ? 0 : d->n_mu_table;
            g.lut_rows = lut_rows;
            p.index_E = d->eps_index;
            p.index_H = d->mu_index;
            g.mid_E = g.mat_E == MAT_IDS ? d->eps_index : nullptr;
            g.mid_H = g.mat_H == MAT_IDS ? d->mu_index : nullptr;
        }
    }
    if (!use_tma) {
        t.V = vec ? vmax : 1;
        const int zthreads0 = (bnz + t.V - 1) / t.V;
        t.TZ = tile_width(zthreads0);
        t.TY = kThreads / t.TZ;
        g.stages = 0;
        p.variant = 1;
    }
    if (p.n_shell) {
        // the interior's last z tile: when less than half of it would be
        // active, its cells go to the shell (config 5 float32: z 32..172
        // would take three 64-cell tiles, the last 12 cells active; float32c:
        // 20..172, the last 24 of 64 active, 0.834 vs 0.804 ms per step)
        const int zc = t.V * t.TZ, rem = bnz % zc;
        if (rem != 0 && 2 * rem < zc && bnz > zc) {
            bnz -= rem;
            ibox[5] -= rem;
            t.e[2] = ibox[5];
        }
    }
    const int zthreads = (bnz + t.V - 1) / t.V;
    t.gz = (zthreads + t.TZ - 1) / t.TZ;
    t.gy = (bny + t.TY - 1) / t.TY;
    if (t.gy > 65535) return FDTD_ERR_UNSUPPORTED;
    if (d->x_chunk > 0) {
        t.XC = d->x_chunk;
    } else {
        // Staged kernels: about twenty waves of the resident CTAs, so the
        // partly filled last wave costs little (measured on 768^3 with one CTA
        // per SM: 3.8 waves 58.7, 7.6 waves 61.4, 22.7 waves 63.1 Gcell/s),
        // with at least 12 planes per chunk (a chunk refills the ring and
        // re-reads one halo plane; configs 2 and 5, which reach only three
        // waves with 32-plane chunks, measured best at 12).  Register
        // kernels: register_chunk.
        const long cols = (long)t.gz * t.gy;
        const long wave = (long)n_sm * ctas_per_sm;
        if (use_tma) {
            long chunks = cols >= 20L * wave ? 1 : (20L * wave + cols - 1) / cols;
            chunks = std::max(1L, std::min(chunks, std::max(1L, (long)bnx / 12)));
            t.XC = (int)((bnx + chunks - 1) / chunks);
        } else {
            t.XC = register_chunk(bnx, cols, wave);
        }
    }
    t.gx = (bnx + t.XC - 1) / t.XC;
    if (t.gx > 65535) return FDTD_ERR_UNSUPPORTED;
    // adjoint kernels: register streaming, tiled like the register kernels
    {
        const int V = vec ? vmax : 1;
        const int zt = (d->nz + V - 1) / V;
        const int TZ = tile_width(zt);
        const int TY = kThreads / TZ;
        const int gz = (zt + TZ - 1) / TZ, gy = (d->ny + TY - 1) / TY;
        // x chunks as for the register-streaming forward kernels
        const int XC = register_chunk(d->nx, (long)gz * gy, 2L * n_sm);
        p.adj_V = V;
        p.adj_TZ = TZ;
        p.adj_TY = TY;
        p.adj_XC = XC;
        p.adj_grid = dim3(gz, gy, (d->nx + XC - 1) / XC);
        p.adj_block = dim3(TZ, TY, 1);
        if (p.n_shell) {
            // the interior box of a partition (its z bounds are multiples of V)
            const int zti = bnz / V, TZi = tile_width(zti), TYi = kThreads / TZi;
            const int gzi = (zti + TZi - 1) / TZi, gyi = (bny + TYi - 1) / TYi;
            const int XCi = register_chunk(bnx, (long)gzi * gyi, 2L * n_sm);
            p.adjin_TZ = TZi;
            p.adjin_TY = TYi;
            p.adjin_XC = XCi;
            p.adjin_grid = dim3(gzi, gyi, (bnx + XCi - 1) / XCi);
            p.adjin_block = dim3(TZi, TYi, 1);
        }
    }
    p.V = t.V;
    g.TZ = t.TZ;
    g.TY = t.TY;
    g.XC = t.XC;
    p.grid = dim3(t.gz, t.gy, t.gx);
    p.block = dim3(t.TZ, t.TY, 1);

    // items: objects, E sources, H sources
    std::vector<ItemK> items;
    for (int q = 0; q < d->n_objects; ++q) {
        const fdtd_item_desc &o = d->objects[q];
        if (o.kind < FDTD_ITEM_OBJECT || o.kind > FDTD_ITEM_ANISOTROPIC) return FDTD_ERR_ARGUMENT;
        if (!box_ok(o.lo, o.hi, d->nx, d->ny, d->nz) || !o.coef[0]) return FDTD_ERR_ARGUMENT;
        if (o.kind == FDTD_ITEM_ABSORBING && (!o.coef[1] || (d->precision == FDTD_FLOAT64 && !o.coef[2])))
            return FDTD_ERR_ARGUMENT;
        items.push_back(to_item(o));
    }
    const int srcE0 = (int)items.size();
    for (int side = 0; side < 2; ++side) {
        const int cnt = side == 0 ? d->n_sources_E : d->n_sources_H;
        const fdtd_item_desc *src = side == 0 ? d->sources_E : d->sources_H;
        const int begin = (int)items.size();
        for (int q = 0; q < cnt; ++q) {
            const fdtd_item_desc &s = src[q];
            if (s.kind != FDTD_ITEM_SOFT && s.kind != FDTD_ITEM_HARD && s.kind != FDTD_ITEM_FEEDBACK)
                return FDTD_ERR_ARGUMENT;
            if (s.kind == FDTD_ITEM_FEEDBACK) {
                // E side only, one cell, a current-probe point, a grid spacing
                if (side != 0 || s.aux < 0 || s.aux >= d->n_current_cells || !(d->grid_spacing > 0.0))
                    return FDTD_ERR_ARGUMENT;
                if (s.hi[0] - s.lo[0] != 1 || s.hi[1] - s.lo[1] != 1 || s.hi[2] - s.lo[2] != 1)
                    return FDTD_ERR_ARGUMENT;
                p.has_feedback = 1;
            }
            if (!box_ok(s.lo, s.hi, d->nx, d->ny, d->nz) || s.comp < 0 || s.comp > 2) return FDTD_ERR_ARGUMENT;
            if (s.column < 0 || s.column >= d->n_columns) return FDTD_ERR_ARGUMENT;
            if (s.kind == FDTD_ITEM_SOFT && (s.hi[0] - s.lo[0] != 1 || s.hi[1] - s.lo[1] != 1 || s.hi[2] - s.lo[2] != 1))
                return FDTD_ERR_ARGUMENT;
            if (q > 0 && s.source < src[q - 1].source) return FDTD_ERR_ARGUMENT;  // grid.sources order
            items.push_back(to_item(s));
        }
        // within one soft source, order the points by cell (stable: repeated
        // points keep their order) so that a run of equal cells is contiguous
        int q = begin;
        while (q < (int)items.size()) {
            int e = q + 1;
            while (e < (int)items.size() && items[e].source == items[q].source) ++e;
            if (items[q].kind == FDTD_ITEM_SOFT) {
                std::stable_sort(items.begin() + q, items.begin() + e, [&](const ItemK &x, const ItemK &y) {
                    const long cx = ((long)x.lo[0] * d->ny + x.lo[1]) * d->nz + x.lo[2];
                    const long cy = ((long)y.lo[0] * d->ny + y.lo[1]) * d->nz + y.lo[2];
                    return cx < cy;
                });
            }
            q = e;
        }
    }
    const int srcH0 = srcE0 + d->n_sources_E;
    const int nitems = (int)items.size();
    p.items_host = items;
    p.n_objects = d->n_objects;
    p.srcE0 = srcE0;
    p.n_srcE = d->n_sources_E;
    p.srcH0 = srcH0;
    p.n_srcH = d->n_sources_H;

    // sources inside the fused pass unless a periodic copy must come first
    const std::vector<ItemK> &cit = items;
    auto touches_slab = [&](const ItemK &it) {  // a slab corrected after the fused pass
        for (int s = p.fused_slabs; s < g.nslab; ++s) {
            const SlabK &S = g.slab[s];
            if (it.lo[S.axis] < S.start + S.th && it.hi[S.axis] > S.start) return true;
        }
        return false;
    };
    auto can_fuse = [&](int first, int count) {
        if (p.epi_E.empty()) return true;
        if (p.pml_split) {
            for (int q = first; q < first + count; ++q)
                if (touches_periodic_plane(cit[q], periodic_axes, n) || touches_slab(cit[q])) return false;
            return true;
        }
        if (slab_after_periodic) return false;
        for (int q = first; q < first + count; ++q)
            if (touches_periodic_plane(cit[q], periodic_axes, n)) return false;
        return true;
    };
    // feedback sources read the current on the device: all E sources run as
    // epilogue kernels then, in order
    g.fuse_src_E = (!p.has_feedback && can_fuse(srcE0, d->n_sources_E)) ? 1 : 0;
    g.fuse_src_H = can_fuse(srcH0, d->n_sources_H) ? 1 : 0;

    // epilogue source launches and soft runs
    std::vector<int2> runs;
    for (int side = 0; side < 2; ++side) {
        const bool fused = side == 0 ? g.fuse_src_E : g.fuse_src_H;
        if (fused) continue;
        const int first = side == 0 ? srcE0 : srcH0;
        const int last = first + (side == 0 ? d->n_sources_E : d->n_sources_H);
        std::vector<EpiOp> &ops = side == 0 ? p.epi_E : p.epi_H;
        int q = first;
        while (q < last) {
            int e = q + 1;
            while (e < last && items[e].source == items[q].source) ++e;
            if (items[q].kind == FDTD_ITEM_HARD || items[q].kind == FDTD_ITEM_FEEDBACK) {
                for (int h = q; h < e; ++h) {
                    EpiOp op{};
                    op.kind = items[q].kind == FDTD_ITEM_HARD ? EPI_HARD : EPI_FEEDBACK;
                    op.item = h;
                    ops.push_back(op);
                }
            } else {
                EpiOp op{};
                op.kind = EPI_SOFT;
                op.run_begin = (int)runs.size();
                int r = q;
                while (r < e) {
                    int re = r + 1;
                    while (re < e && items[re].lo[0] == items[r].lo[0] && items[re].lo[1] == items[r].lo[1] &&
                           items[re].lo[2] == items[r].lo[2] && items[re].comp == items[r].comp)
                        ++re;
                    runs.push_back(make_int2(r, re - r));
                    r = re;
                }
                op.run_count = (int)runs.size() - op.run_begin;
                ops.push_back(op);
            }
            q = e;
        }
    }

    std::vector<int> obj_off, obj_idx, se_off, se_idx, sh_off, sh_idx;
    build_csr(t, items, 0, srcE0, obj_off, obj_idx);
    build_csr(t, items, srcE0, d->n_sources_E, se_off, se_idx);
    build_csr(t, items, srcH0, d->n_sources_H, sh_off, sh_idx);

    // interior/shell partition: the boxes around the interior (x faces whole,
    // y faces within the interior's x range, z faces within its x and y
    // ranges), one thread per sv cells along z, each block inside one box;
    // per-block object and source lists
    ShellK shk{};
    std::vector<int> shl[6];  // object, E source, H source lists (offsets, indices)
    if (p.n_shell) {
        const int *lo = ibox, *hi = ibox + 3;
        const int boxes[6][6] = {{0, 0, 0, lo[0], n[1], n[2]},         {hi[0], 0, 0, n[0], n[1], n[2]},
                                 {lo[0], 0, 0, hi[0], lo[1], n[2]},     {lo[0], hi[1], 0, hi[0], n[1], n[2]},
                                 {lo[0], lo[1], 0, hi[0], hi[1], lo[2]}, {lo[0], lo[1], hi[2], hi[0], hi[1], n[2]}};
        const int sv = d->precision == FDTD_FLOAT64 ? shell_v<double>() : shell_v<float>();
        long blocks = 0;
        for (const auto &b : boxes) {
            if (b[3] <= b[0] || b[4] <= b[1] || b[5] <= b[2]) continue;
            const int q = shk.nbox++;
            for (int a = 0; a < 3; ++a) {
                shk.o[q][a] = b[a];
                shk.n[q][a] = b[3 + a] - b[a];
            }
            for (int sl = 0; sl < g.nslab; ++sl) {
                const SlabK &S = g.slab[sl];
                if (S.start < b[3 + S.axis] && S.start + S.th > b[S.axis]) shk.slabs[q] |= 1u << sl;
            }
            shk.first[q] = (unsigned)blocks;
            magic_div((unsigned)(shk.n[q][2] / sv), shk.mz[q], shk.sz[q]);
            magic_div((unsigned)shk.n[q][1], shk.my[q], shk.sy[q]);
            blocks += ((long)shk.n[q][0] * shk.n[q][1] * (shk.n[q][2] / sv) + kThreads - 1) / kThreads;
            if (blocks * kThreads >= (1L << 31)) return FDTD_ERR_UNSUPPORTED;
        }
        shk.first[shk.nbox] = (unsigned)blocks;
        // the blocks an item's cells fall in, ascending (rows of a box are
        // consecutive runs of cells, boxes follow one another)
        auto lists = [&](int first, int count, std::vector<int> &off, std::vector<int> &idx) {
            off.assign(blocks + 1, 0);
            for (int pass = 0; pass < 2; ++pass) {
                std::vector<int> fill;
                if (pass == 1) {
                    for (long c = 0; c < blocks; ++c) off[c + 1] += off[c];
                    idx.assign(off[blocks], 0);
                    fill.assign(off.begin(), off.end() - 1);
                }
                for (int q = first; q < first + count; ++q) {
                    const ItemK &it = items[q];
                    long last = -1;
                    for (int b = 0; b < shk.nbox; ++b) {
                        int l[3], u[3];
                        bool empty = false;
                        for (int a = 0; a < 3; ++a) {
                            l[a] = std::max(it.lo[a], shk.o[b][a]);
                            u[a] = std::min(it.hi[a], shk.o[b][a] + shk.n[b][a]);
                            empty |= u[a] <= l[a];
                        }
                        if (empty) continue;
                        for (int x = l[0]; x < u[0]; ++x)
                            for (int y = l[1]; y < u[1]; ++y) {
                                // thread slots of the row: sv cells each
                                const long row = ((long)(x - shk.o[b][0]) * shk.n[b][1] + (y - shk.o[b][1])) *
                                                 (shk.n[b][2] / sv);
                                const long b0 = shk.first[b] + (row + (l[2] - shk.o[b][2]) / sv) / kThreads;
                                const long b1 = shk.first[b] + (row + (u[2] - 1 - shk.o[b][2]) / sv) / kThreads;
                                for (long blk = std::max(b0, last + 1); blk <= b1; ++blk) {
                                    if (pass == 0) off[blk + 1]++;
                                    else idx[fill[blk]++] = q;
                                }
                                last = std::max(last, b1);
                            }
                    }
                }
            }
        };
        lists(0, srcE0, shl[0], shl[1]);
        lists(srcE0, d->n_sources_E, shl[2], shl[3]);
        lists(srcH0, d->n_sources_H, shl[4], shl[5]);
        p.n_shell = shk.nbox;
    }
    size_t shell_ints = 0;
    for (const auto &v : shl) shell_ints += v.size() + 1;

    // Launch order of the staged passes (and tile order of the persistent
    // loop over register-streaming tiles): the tiles that carry more work per
    // plane (object cells, weighted by the coefficient values they read, and
    // cells of the PML slabs inside the fused pass) first, so that they run
    // in the first waves instead of finishing last; the rest in grid order.
    std::vector<int> cta_order;
    {
        const long ncta = (long)t.gz * t.gy * t.gx;
        const int zc = t.V * t.TZ;
        std::vector<double> extra(ncta, 0.0);
        auto add_box = [&](const int32_t lo[3], const int32_t hi[3], double w) {
            int r[6];
            cta_range(t, lo, hi, r);
            for (int cx = r[4]; cx <= r[5]; ++cx)
                for (int cy = r[2]; cy <= r[3]; ++cy)
                    for (int cz = r[0]; cz <= r[1]; ++cz) {
                        const int x0 = t.o[0] + cx * t.XC, y0 = t.o[1] + cy * t.TY, z0 = t.o[2] + cz * zc;
                        const long ox = std::min({hi[0], x0 + t.XC, t.e[0]}) - std::max(lo[0], x0);
                        const long oy = std::min({hi[1], y0 + t.TY, t.e[1]}) - std::max(lo[1], y0);
                        const long oz = std::min({hi[2], z0 + zc, t.e[2]}) - std::max(lo[2], z0);
                        if (ox > 0 && oy > 0 && oz > 0) extra[cz + t.gz * (cy + (long)t.gy * cx)] += w * ox * oy * oz;
                    }
        };
        for (int q = 0; q < srcE0; ++q) {
            const ItemK &o = items[q];
            add_box(o.lo, o.hi, o.kind == FDTD_ITEM_ANISOTROPIC ? 3.0 : (o.kind == FDTD_ITEM_ABSORBING ? 2.0 : 1.0));
        }
        const int fused = p.pml_split ? p.fused_slabs : g.nslab;
        for (int sl = 0; sl < fused; ++sl) {
            const SlabK &S = g.slab[sl];
            int32_t lo[3] = {0, 0, 0}, hi[3] = {d->nx, d->ny, d->nz};
            lo[S.axis] = S.start;
            hi[S.axis] = S.start + S.th;
            add_box(lo, hi, 1.0);
        }
        bool any = false;
        for (double w : extra) any |= w > 0.0;
        if (any) {
            cta_order.resize(ncta);
            for (long c = 0; c < ncta; ++c) cta_order[c] = (int)c;
            std::stable_sort(cta_order.begin(), cta_order.end(), [&](int a, int b) { return extra[a] > extra[b]; });
        }
    }

    // ---- one pass per time step (fdtd_onepass.cuh) ----
    // Allowed for float32 plans whose every PML slab precedes any periodic
    // boundary, with periodic boundaries only along x, no object or source on
    // a periodic plane and no feedback source; used when the caller gave the
    // second buffers and asked for it.
    if (d->step_fusion < 0 || d->step_fusion > 2) return FDTD_ERR_ARGUMENT;
    p.onepass = p.onepass_ok = p.onepass_hcopy = p.onepass_why = 0;
    GridK kl;  // tiling and stage layout of the one-pass kernel
    memset(&kl, 0, sizeof(kl));
    Tiling to{};
    for (int a = 0; a < 3; ++a) to.e[a] = n[a];
    std::vector<int> oo_off, oo_idx, ose_off, ose_idx, osh_off, osh_idx;
    {
        int why = 0;  // first reason the grid does not allow it (fdtd_plan_step_fusion)
        auto refuse = [&](int r) {
            if (why == 0) why = r;
        };
        if (d->precision != FDTD_FLOAT32) refuse(1);
        if (!vec) refuse(2);
        if (p.has_feedback) refuse(3);
        bool periodic_seen = false, per_x = false;
        for (int b = 0; b < d->n_boundaries; ++b) {
            const fdtd_boundary_desc &bd = d->boundaries[b];
            if (bd.kind == FDTD_BOUNDARY_PERIODIC) {
                if (n[bd.axis] <= 1) continue;  // a plane copied onto itself
                if (bd.axis != 0 || per_x) refuse(5);
                per_x = true;
                periodic_seen = true;
            } else if (periodic_seen) {
                refuse(4);  // a PML slab after a periodic boundary
            }
        }
        if (per_x && d->nx < 4) refuse(5);
        if (per_x)
            for (const ItemK &it : items)
                if (it.lo[0] == 0 || it.hi[0] == d->nx) refuse(6);
        const bool ok = why == 0;
        p.onepass_ok = ok ? 1 : 0;
        bool alt = d->E_alt != nullptr && d->H_alt != nullptr && aligned16(d->E_alt) && aligned16(d->H_alt);
        for (int b = 0; b < d->n_boundaries; ++b)
            if (d->boundaries[b].kind == FDTD_BOUNDARY_PML &&
                (!d->psi_alt[b][0] || !d->psi_alt[b][1] || !aligned16(d->psi_alt[b][0]) ||
                 !aligned16(d->psi_alt[b][1])))
                alt = false;
        // automatic choice: never -- the two-pass plans measured faster on every
        // configuration (the one-pass stage holds about twice the bytes per cell,
        // so fewer planes are in flight per SM and the pass is latency-bound)
        const bool want = d->step_fusion == 2;
        if (ok && !alt) refuse(7);
        p.onepass_why = why;
        if (want && ok && alt) {
            const int V = PF32::V, Zc = 32 * V;
            const int matE = mat_want[0], matH = mat_want[1] == MAT_IDS ? MAT_FULL : mat_want[1];
            const int lut_rows = std::max(mat_lut_rows(matE), mat_lut_rows(matH));
            int coef = 0;
            for (int s = 0; s < g.nslab; ++s) {
                kl.coef_off[s] = coef;
                coef += 2 * g.slab[s].th;
            }
            kl.coef_values = (size_t)coef * esize <= 16384 ? coef : 0;
            // stage layout of a tile height: field tiles, then per group of slabs of
            // one axis that never meet in one stage an E-side slot (TY+1 rows;
            // x/y slabs Zc+2 pairs) and an H-side slot (TY rows)
            auto layout = [&](int TY) -> size_t {
                size_t stage = onepass_bytes(d->precision, TY, matE, matH, 0);
                struct Slot {
                    int axis;
                    size_t bE, bH, offE, offH;
                    std::vector<std::pair<int, int>> ranges;
                };
                std::vector<Slot> slots;
                int slot_of[kMaxSlabs] = {0};
                for (int s = 0; s < g.nslab; ++s) {
                    const SlabK &S = g.slab[s];
                    const int unit = S.axis == 0 ? 1 : (S.axis == 1 ? TY : Zc);
                    const int lo = S.axis == 0 ? S.start : std::max(0, S.start - 1);  // tiles whose halo reaches it
                    const std::pair<int, int> rg(lo / unit, (S.start + S.th - 1) / unit);
                    const int pE = S.axis == 2 ? 2 * S.thp : 2 * (Zc + 2);
                    const int pH = S.axis == 2 ? 2 * S.thp : 2 * Zc;
                    kl.psi_pitch[s] = pE;
                    kl.psi_pitchH[s] = pH;
                    const size_t bE = (size_t)(TY + 1) * pE * esize, bH = (size_t)TY * pH * esize;
                    int found = -1;
                    for (int q = 0; q < (int)slots.size() && found < 0; ++q) {
                        if (slots[q].axis != S.axis) continue;
                        bool disjoint = true;
                        for (auto &o : slots[q].ranges)
                            if (!(rg.second < o.first || o.second < rg.first)) disjoint = false;
                        if (disjoint) found = q;
                    }
                    if (found < 0) {
                        slots.push_back(Slot{S.axis, 0, 0, 0, 0, {}});
                        found = (int)slots.size() - 1;
                    }
                    slots[found].ranges.push_back(rg);
                    slots[found].bE = std::max(slots[found].bE, bE);
                    slots[found].bH = std::max(slots[found].bH, bH);
                    slot_of[s] = found;
                }
                for (auto &sl : slots) {
                    sl.offE = stage;
                    stage += (sl.bE + 127) & ~(size_t)127;
                    sl.offH = stage;
                    stage += (sl.bH + 127) & ~(size_t)127;
                }
                for (int s = 0; s < g.nslab; ++s) {
                    kl.psi_off[s] = (int)slots[slot_of[s]].offE;
                    kl.psi_offH[s] = (int)slots[slot_of[s]].offH;
                }
                return stage;
            };
            // material tables: 256 padded rows for an index map, one for a uniform material
            const size_t extra = 2 * (size_t)kl.coef_values * esize + 4 * esize * (size_t)mat_lut_rows(matE) +
                                 4 * esize * (size_t)mat_lut_rows(matH) + 16 + 128;
            const long per_sm = 228L * 1024;
            auto smem_of = [&](int TY, size_t stage, int S) {
                return (size_t)S * stage + (size_t)S * 8 + 2 * onepass_bytes(d->precision, TY, matE, matH, 1) + extra;
            };
            // tile height and ring depth: two CTAs per SM with at least three
            // stages where that fits, else one CTA with up to six stages
            int TY = (d->tile_rows == 4 || d->tile_rows == 8) ? d->tile_rows : 0;
            int S = d->stages >= 3 ? d->stages : 0;
            auto fit_two = [&](int ty) {
                const size_t st = layout(ty);
                for (int q = 6; q >= 3; --q)
                    if ((long)smem_of(ty, st, q) + 1024 <= per_sm / 2 && smem_of(ty, st, q) <= (size_t)optin) return q;
                return 0;
            };
            if (TY == 0) TY = fit_two(8) ? 8 : 4;
            const size_t stage = layout(TY);
            if (S == 0) {
                S = fit_two(TY);
                if (S == 0)
                    for (int q = 6; q >= 3 && S == 0; --q)
                        if (smem_of(TY, stage, q) <= (size_t)optin) S = q;
            }
            const size_t smem = S >= 3 ? smem_of(TY, stage, S) : 0;
            if (S < 3 || smem > (size_t)optin) {
                p.onepass_why = 8;
            } else {
                const int ctas = std::max(1, (int)(per_sm / (long)(smem + 1024)));
                to.V = V;
                to.TZ = 32;
                to.TY = TY;
                to.gz = (d->nz + Zc - 1) / Zc;
                to.gy = (d->ny + TY - 1) / TY;
                if (d->x_chunk > 0) {
                    to.XC = d->x_chunk;
                } else {
                    // about forty waves of CTAs (a short last wave), at least 32
                    // planes per chunk (a chunk stages one plane before it and
                    // recomputes one after it)
                    const long cols = (long)to.gz * to.gy, wave = (long)n_sm * ctas;
                    long chunks = (40L * wave + cols - 1) / cols;
                    chunks = std::max(1L, std::min(chunks, std::max(1L, (long)d->nx / 32)));
                    to.XC = (int)((d->nx + chunks - 1) / chunks);
                }
                to.gx = (d->nx + to.XC - 1) / to.XC;
                if (to.gy <= 65535 && to.gx <= 65535) {
                    kl.TZ = 32;
                    kl.TY = TY;
                    kl.XC = to.XC;
                    kl.stages = S;
                    kl.stage_bytes = (int)stage;
                    kl.lut_rows = lut_rows;
                    kl.mat_E = matE;
                    kl.mat_H = matH;
                    kl.periodic_x = per_x ? 1 : 0;
                    p.osmem = smem;
                    p.ogrid = dim3(to.gz, to.gy, to.gx);
                    p.oblock = dim3(32, TY + 1, 1);
                    p.onepass = 1;
                    p.onepass_hcopy = per_x ? 1 : 0;
                    build_csr(to, items, 0, srcE0, oo_off, oo_idx, true);
                    build_csr(to, items, srcE0, d->n_sources_E, ose_off, ose_idx, true);
                    build_csr(to, items, srcH0, d->n_sources_H, osh_off, osh_idx, true);
                } else {
                    p.onepass_why = 9;
                }
            }
        }
    }

    // probes, current probes and DFT boxes
    p.n_probe = d->n_probe_cells;
    p.probe_cells = d->probe_cells;
    p.n_current = d->n_current_cells;
    p.current_cells = d->current_cells;
    p.grid_spacing = d->grid_spacing;
    for (int q = 0; q < d->n_dft; ++q) {
        const fdtd_dft_desc &dd = d->dft[q];
        if (!box_ok(dd.lo, dd.hi, d->nx, d->ny, d->nz) || dd.n_freq < 1 || !dd.acc || dd.phase_offset < 0 ||
            dd.phase_offset + dd.n_freq > d->n_phase_columns)
            return FDTD_ERR_ARGUMENT;
        p.dft.push_back(dd);
    }
    p.n_columns = d->n_columns;
    p.n_phase_columns = d->n_phase_columns;
    (void)esize;

    // one device allocation for the plan's tables
    auto align = [](size_t v) { return (v + 255) & ~(size_t)255; };
    const size_t b_items = align(sizeof(ItemK) * std::max(1, nitems));
    const size_t b_lists = align(sizeof(int) * (obj_off.size() + obj_idx.size() + se_off.size() + se_idx.size() +
                                                sh_off.size() + sh_idx.size() + oo_off.size() + oo_idx.size() +
                                                ose_off.size() + ose_idx.size() + osh_off.size() + osh_idx.size() +
                                                cta_order.size() + 13 + shell_ints));
    const size_t b_runs = align(sizeof(int2) * std::max<size_t>(1, runs.size()));
    const size_t b_status = 512;  // status word; at +256 the persistent loop's barrier and tile counters
    std::vector<char> host(b_items + b_lists + b_runs + b_status, 0);
    if (nitems) memcpy(host.data(), items.data(), sizeof(ItemK) * nitems);
    int *lists = (int *)(host.data() + b_items);
    size_t pos = 0;
    size_t at_obj_off, at_obj_idx, at_se_off, at_se_idx, at_sh_off, at_sh_idx;
    auto put = [&](const std::vector<int> &v, size_t &at) {
        at = pos;
        if (!v.empty()) memcpy(lists + pos, v.data(), sizeof(int) * v.size());
        pos += v.size() + 1;
    };
    put(obj_off, at_obj_off);
    put(obj_idx, at_obj_idx);
    put(se_off, at_se_off);
    put(se_idx, at_se_idx);
    put(sh_off, at_sh_off);
    put(sh_idx, at_sh_idx);
    size_t at_oo_off, at_oo_idx, at_ose_off, at_ose_idx, at_osh_off, at_osh_idx;
    put(oo_off, at_oo_off);
    put(oo_idx, at_oo_idx);
    put(ose_off, at_ose_off);
    put(ose_idx, at_ose_idx);
    put(osh_off, at_osh_off);
    put(osh_idx, at_osh_idx);
    size_t at_order;
    put(cta_order, at_order);
    size_t at_shell[6];
    for (int q = 0; q < 6; ++q) put(shl[q], at_shell[q]);
    if (!runs.empty()) memcpy(host.data() + b_items + b_lists, runs.data(), sizeof(int2) * runs.size());
    ce = cudaMalloc(&p.dev_mem, host.size());
    if (ce != cudaSuccess) return cuda_fail(ce);
    ce = cudaMemcpy(p.dev_mem, host.data(), host.size(), cudaMemcpyHostToDevice);
    if (ce != cudaSuccess) {
        cudaFree(p.dev_mem);
        p.dev_mem = nullptr;
        return cuda_fail(ce);
    }
    char *base = (char *)p.dev_mem;
    const int *dl = (const int *)(base + b_items);
    g.items = (const ItemK *)base;
    g.obj_off = dl + at_obj_off;
    g.obj_idx = dl + at_obj_idx;
    g.srcE_off = dl + at_se_off;
    g.srcE_idx = dl + at_se_idx;
    g.srcH_off = dl + at_sh_off;
    g.srcH_idx = dl + at_sh_idx;
    const int *order = cta_order.empty() ? nullptr : dl + at_order;
    g.cta_order = p.variant == 2 ? order : nullptr;
    p.persist_order = p.variant == 1 ? order : nullptr;
    p.runs = (const int2 *)(base + b_items + b_lists);
    g.status = (int *)(base + b_items + b_lists + b_runs);
    p.persist_bar = (unsigned *)(base + b_items + b_lists + b_runs + 256);
    p.persist_tickets = (unsigned long long *)(base + b_items + b_lists + b_runs + 264);
    if (p.variant == 2) {
        const int rc = d->precision == FDTD_FLOAT32    ? prepare_tma_f32(p)
                       : d->precision == FDTD_FLOAT32C ? prepare_tma_f32c(p)
                                                       : prepare_tma_f64(p);
        if (rc != FDTD_OK) return rc;
    }

    p.kf = p.k;
    if (p.pml_split) {
        p.kf.nslab = p.fused_slabs;
        p.kf.nslab_fused = p.fused_slabs;
    }
    if (p.n_shell) {
        // the shell launch: every slab, its own per-block lists
        GridK &k = p.kshell;
        k = p.k;
        k.obj_off = dl + at_shell[0];
        k.obj_idx = dl + at_shell[1];
        k.srcE_off = dl + at_shell[2];
        k.srcE_idx = dl + at_shell[3];
        k.srcH_off = dl + at_shell[4];
        k.srcH_idx = dl + at_shell[5];
        k.cta_order = nullptr;
        p.shellk = shk;
        // beside a register-streaming interior in float32 and float32c the
        // shell launch fills the interior's last wave (config 2 float32 0.375
        // vs 0.395 ms per step, config 5 float32c 0.853 vs 0.870); the staged
        // interior holds every register of its SMs and float64 is arithmetic
        // bound, and both measured faster one after the other (config 5
        // float32 0.578 vs 0.608, config 2 float64 1.39 vs 1.49)
        p.shell_overlap = p.variant == 1 && d->precision != FDTD_FLOAT64;
        if (p.shell_overlap) {
            ce = cudaStreamCreateWithFlags(&p.shell_stream, cudaStreamNonBlocking);
            if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&p.shell_fork, cudaEventDisableTiming);
            if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&p.shell_join, cudaEventDisableTiming);
            if (ce != cudaSuccess) return cuda_fail(ce);
        }
    }
    if (p.n_shell) {
        // the interior: no slab cells
        p.kf.nslab = 0;
        p.kf.nslab_fused = 0;
        p.kf.n_staged = 0;
        p.kf.ox = ibox[0];
        p.kf.oy = ibox[1];
        p.kf.oz = ibox[2];
        p.kf.ex = ibox[3];
        p.kf.ey = ibox[4];
        p.kf.ez = ibox[5];
    }
    p.kfH = p.kf;
    if (p.variant == 2) {
        GridK *pass_k[2] = {&p.kf, &p.kfH};
        for (int pass = 0; pass < 2; ++pass) {
            pass_k[pass]->stages = pass_stages[pass];
            pass_k[pass]->stage_bytes = pass_stage_bytes[pass];
            for (int s = 0; s < kMaxSlabs; ++s) pass_k[pass]->psi_off[s] = pass_psi_off[pass][s];
        }
    }

    if (p.onepass) {
        // direction 0 reads the caller's buffers and writes the alternates,
        // direction 1 the reverse; every slab is handled inside the pass
        for (int dir = 0; dir < 2; ++dir) {
            GridK &k = p.ko[dir];
            k = p.k;
            k.nslab_fused = k.nslab;
            k.TZ = kl.TZ;
            k.TY = kl.TY;
            k.XC = kl.XC;
            k.stages = kl.stages;
            k.stage_bytes = kl.stage_bytes;
            for (int s = 0; s < kMaxSlabs; ++s) {
                k.psi_off[s] = kl.psi_off[s];
                k.psi_pitch[s] = kl.psi_pitch[s];
                k.psi_offH[s] = kl.psi_offH[s];
                k.psi_pitchH[s] = kl.psi_pitchH[s];
                k.coef_off[s] = kl.coef_off[s];
            }
            k.coef_values = kl.coef_values;
            k.lut_rows = kl.lut_rows;
            k.mat_E = kl.mat_E;
            k.mat_H = kl.mat_H;
            k.mlut_E = d->eps_table;
            k.mlut_H = d->mu_table;
            k.nlut_E = kl.mat_E == MAT_FULL ? 0 : d->n_eps_table;
            k.nlut_H = kl.mat_H == MAT_FULL ? 0 : d->n_mu_table;
            k.mid_E = kl.mat_E == MAT_IDS ? d->eps_index : nullptr;
            k.mid_H = nullptr;
            k.periodic_x = kl.periodic_x;
            k.obj_off = dl + at_oo_off;
            k.obj_idx = dl + at_oo_idx;
            k.srcE_off = dl + at_ose_off;
            k.srcE_idx = dl + at_ose_idx;
            k.srcH_off = dl + at_osh_off;
            k.srcH_idx = dl + at_osh_idx;
            k.fuse_src_E = k.fuse_src_H = 1;
            k.cta_order = nullptr;  // the one-pass kernel launches in grid order
            void *Ea = d->E, *Ha = d->H, *Eb = d->E_alt, *Hb = d->H_alt;
            k.E = dir == 0 ? Eb : Ea;  // written
            k.H = dir == 0 ? Hb : Ha;
            for (int s = 0; s < k.nslab; ++s) {
                const int b = p.slab_boundary[s];
                void *pa_E = d->boundaries[b].psi_E, *pa_H = d->boundaries[b].psi_H;
                void *pb_E = d->psi_alt[b][0], *pb_H = d->psi_alt[b][1];
                k.slab[s].psiE = dir == 0 ? pb_E : pa_E;
                k.slab[s].psiH = dir == 0 ? pb_H : pa_H;
                k.slab[s].psiE_rd = dir == 0 ? pa_E : pb_E;
                k.slab[s].psiH_rd = dir == 0 ? pa_H : pb_H;
            }
        }
        const int rc = prepare_onepass_f32(p);
        if (rc == FDTD_ERR_UNSUPPORTED) {
            p.onepass = 0;  // a tensor map the one-pass kernel needs was refused
            p.onepass_why = 10;
        } else if (rc != FDTD_OK) {
            return rc;
        }
    }

    // persistent time loop (fdtd_persistent.cuh): small register-streaming
    // plans with nothing between the half steps but gathers and DFT sums
    if (d->persistent < 0 || d->persistent > 2) return FDTD_ERR_ARGUMENT;
    {
        int coop = 0;
        cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
        p.persist_ok = coop && p.variant == 1 && p.n_shell == 0 && p.epi_E.empty() && p.epi_H.empty() && !p.has_feedback &&
                       p.n_current == 0 && (int)p.dft.size() <= kPersistMaxDft;
        // automatic: float32 below 3M cells, float64 below 8M (measured
        // against one launch per half step, register tiles, 500 steps: 64^3
        // with a 10-cell PML 1.54x float32 / 1.25x float64; 128^3 with PML
        // and objects 1.03-1.12x; 192x192x96 with PML and an anisotropic box
        // 0.985x float32, 1.07x float64)
        const long auto_cells = d->precision == FDTD_FLOAT64 ? (8L << 20) : 3000000L;
        p.persistent = p.persist_ok && (d->persistent == 2 || (d->persistent == 0 && ncell < auto_cells));
        p.persist_blocks = 0;
    }
    p.stats_ctas = std::max(1, std::min(4 * n_sm, FDTD_STATS_STATIC_MAX_ROWS));
    p.device = dev;
    p.launches_per_step = 2 + (p.n_shell ? 2 : 0) + (int)p.epi_E.size() + (int)p.epi_H.size() + (p.n_probe > 0 ? 2 : 0) +
                          (p.n_current > 0 ? 1 : 0) + (int)p.dft.size();
    return FDTD_OK;
}

}  // namespace fdtd

using namespace fdtd;

// The shell stream and its events (created with the plan's shell launch).
static void release_shell(Plan &p) {
    if (p.shell_fork) cudaEventDestroy(p.shell_fork);
    if (p.shell_join) cudaEventDestroy(p.shell_join);
    if (p.shell_stream) cudaStreamDestroy(p.shell_stream);
    p.shell_fork = p.shell_join = nullptr;
    p.shell_stream = nullptr;
}

extern "C" {

int fdtd_plan_create(const fdtd_grid_desc *desc, fdtd_plan **out) {
    if (!desc || !out) return FDTD_ERR_ARGUMENT;
    *out = nullptr;
    fdtd_plan *h = new fdtd_plan();
    h->p.dev_mem = nullptr;
    h->p.shell_stream = nullptr;
    h->p.shell_fork = h->p.shell_join = nullptr;
    const int rc = create(desc, h->p);
    if (rc != FDTD_OK) {
        release_shell(h->p);
        if (h->p.dev_mem) cudaFree(h->p.dev_mem);
        delete h;
        return rc;
    }
    *out = h;
    return FDTD_OK;
}

int fdtd_plan_destroy(fdtd_plan *plan) {
    if (!plan) return FDTD_ERR_ARGUMENT;
    int rc = FDTD_OK;
    release_shell(plan->p);
    if (plan->p.dev_mem) {
        cudaError_t e = cudaFree(plan->p.dev_mem);
        if (e != cudaSuccess) rc = cuda_fail(e);
    }
    delete plan;
    return rc;
}

int fdtd_plan_status(fdtd_plan *plan, int32_t *out, int32_t reset, fdtd_stream_t stream) {
    if (!plan || !out) return FDTD_ERR_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    int v = 0;
    cudaError_t e = cudaMemcpyAsync(&v, plan->p.k.status, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e == cudaSuccess && reset) e = cudaMemsetAsync(plan->p.k.status, 0, sizeof(int), st);
    if (e != cudaSuccess) return cuda_fail(e);
    *out = v;
    return FDTD_OK;
}

int fdtd_selftest_bounded_wait(uint32_t polls, int32_t *status_out, fdtd_stream_t stream) {
    if (!status_out) return FDTD_ERR_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    int *d = nullptr;
    cudaError_t e = cudaMalloc(&d, sizeof(int));
    if (e != cudaSuccess) return cuda_fail(e);
    int v = 0;
    e = cudaMemsetAsync(d, 0, sizeof(int), st);
    if (e == cudaSuccess) {
        launch_wait_selftest(d, polls, st);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(&v, d, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(d);
    if (e != cudaSuccess) return cuda_fail(e);
    *status_out = v;
    return FDTD_OK;
}

int fdtd_run(fdtd_plan *plan, const fdtd_run_args *args, fdtd_stream_t stream) {
    if (!plan || !args) return FDTD_ERR_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    switch (plan->p.precision) {
        case FDTD_FLOAT32:
            return run_f32(plan->p, args, nullptr, st);
        case FDTD_FLOAT32C:
            return run_f32c(plan->p, args, nullptr, st);
        case FDTD_FLOAT64:
            return run_f64(plan->p, args, nullptr, st);
    }
    return FDTD_ERR_ARGUMENT;
}

int fdtd_run_capture(fdtd_plan *plan, const fdtd_run_args *args, const fdtd_capture_args *cap,
                     fdtd_stream_t stream) {
    if (!plan || !args || !cap) return FDTD_ERR_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    switch (plan->p.precision) {
        case FDTD_FLOAT32:
            return run_f32(plan->p, args, cap, st);
        case FDTD_FLOAT32C:
            return run_f32c(plan->p, args, cap, st);
        case FDTD_FLOAT64:
            return run_f64(plan->p, args, cap, st);
    }
    return FDTD_ERR_ARGUMENT;
}

int fdtd_adjoint_run(fdtd_plan *plan, const fdtd_adjoint_args *args, fdtd_stream_t stream) {
    if (!plan || !args) return FDTD_ERR_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    switch (plan->p.precision) {
        case FDTD_FLOAT32:
            return adjoint_f32(plan->p, args, st);
        case FDTD_FLOAT64:
            return adjoint_f64(plan->p, args, st);
    }
    return FDTD_ERR_UNSUPPORTED;
}

static int curl_common(int32_t precision, const void *in, void *out, int32_t nx, int32_t ny, int32_t nz,
                       fdtd_stream_t stream, bool is_E) {
    if (!in || !out || nx < 1 || ny < 1 || nz < 1) return FDTD_ERR_ARGUMENT;
    if (precision < FDTD_FLOAT32 || precision > FDTD_FLOAT64) return FDTD_ERR_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    const int blocks = grid_stride_blocks((long)nx * ny * nz);
    if (precision == FDTD_FLOAT64) {
        if (is_E) k_curl_E<double><<<blocks, kThreads, 0, st>>>((const double *)in, (double *)out, nx, ny, nz);
        else k_curl_H<double><<<blocks, kThreads, 0, st>>>((const double *)in, (double *)out, nx, ny, nz);
    } else {
        if (is_E) k_curl_E<float><<<blocks, kThreads, 0, st>>>((const float *)in, (float *)out, nx, ny, nz);
        else k_curl_H<float><<<blocks, kThreads, 0, st>>>((const float *)in, (float *)out, nx, ny, nz);
    }
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? FDTD_OK : cuda_fail(e);
}

int fdtd_curl_E(int32_t precision, const void *E, void *out, int32_t nx, int32_t ny, int32_t nz,
                fdtd_stream_t stream) {
    return curl_common(precision, E, out, nx, ny, nz, stream, true);
}

int fdtd_curl_H(int32_t precision, const void *H, void *out, int32_t nx, int32_t ny, int32_t nz,
                fdtd_stream_t stream) {
    return curl_common(precision, H, out, nx, ny, nz, stream, false);
}

}  // extern "C"

namespace fdtd {
// First pass of the field statistics into `rows` partial rows: 16-byte
// vector loads for float fields whose value count is a multiple of 4.
static void launch_stats_partial(const Plan &p, int rows, double *part, cudaStream_t st) {
    const GridK &g = p.k;
    const long nvals = 3L * g.nx * g.ny * g.nz;
    const bool comp = p.precision == FDTD_FLOAT32C;
    const bool vec = p.precision != FDTD_FLOAT64 && nvals % 4 == 0 && aligned16(g.E) && aligned16(g.H) &&
                     (!comp || (aligned16(g.Elo) && aligned16(g.Hlo)));
    if (vec) {
        if (comp)
            k_stats_partial4<true><<<rows, kThreads, 0, st>>>((const float4 *)g.E, (const float4 *)g.Elo,
                                                              (const float4 *)g.H, (const float4 *)g.Hlo, nvals / 4,
                                                              part);
        else
            k_stats_partial4<false><<<rows, kThreads, 0, st>>>((const float4 *)g.E, nullptr, (const float4 *)g.H,
                                                               nullptr, nvals / 4, part);
    } else if (p.precision == FDTD_FLOAT64) {
        k_stats_partial<double, false><<<rows, kThreads, 0, st>>>((const double *)g.E, nullptr,
                                                                 (const double *)g.H, nullptr, nvals, part);
    } else if (comp) {
        k_stats_partial<float, true><<<rows, kThreads, 0, st>>>((const float *)g.E, (const float *)g.Elo,
                                                               (const float *)g.H, (const float *)g.Hlo, nvals, part);
    } else {
        k_stats_partial<float, false><<<rows, kThreads, 0, st>>>((const float *)g.E, nullptr, (const float *)g.H,
                                                                nullptr, nvals, part);
    }
}
}  // namespace fdtd

extern "C" {

size_t fdtd_stats_scratch_bytes(const fdtd_plan *plan) {
    if (!plan) return 0;
    return sizeof(double) * 5 * (size_t)plan->p.stats_ctas;
}

int fdtd_field_stats(const fdtd_plan *plan, double *stats, void *scratch, fdtd_stream_t stream) {
    if (!plan || !stats || !scratch) return FDTD_ERR_ARGUMENT;
    const Plan &p = plan->p;
    cudaStream_t st = (cudaStream_t)stream;
    double *part = (double *)scratch;
    launch_stats_partial(p, p.stats_ctas, part, st);
    k_stats_final<<<1, 32, 0, st>>>(part, p.stats_ctas, stats);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? FDTD_OK : cuda_fail(e);
}

}  // extern "C"

// Partial sums of fdtd_field_stats_noalloc: a fixed array in device memory,
// one copy per GPU that loads the library.  Host code must not use the
// symbol itself as a device address (it is a host-side stand-in); its device
// address is looked up once per device with cudaGetSymbolAddress.
static __device__ __align__(256) double g_stats_rows[FDTD_STATS_STATIC_MAX_ROWS * 5];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_rows_mutex;
double *g_rows_addr[kMaxDevices] = {nullptr};
CUcontext g_rows_ctx[kMaxDevices] = {nullptr};

using CtxGetCurrentFn = CUresult (*)(CUcontext *);

// The driver's cuCtxGetCurrent, found through the runtime (the library links
// no driver import library).
CtxGetCurrentFn ctx_get_current() {
    static CtxGetCurrentFn fn = nullptr;
    if (fn == nullptr) {
        void *ptr = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &ptr, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<CtxGetCurrentFn>(ptr);
    }
    return fn;
}

// Device address of g_stats_rows on the current device, looked up once per
// device with that device current and kept.  The context it was looked up
// in is kept too: after a device reset (cudaDeviceReset, or a new primary
// context) the old address is stale, and the first call in the new context
// looks it up again.
int stats_rows_address(double **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e);
    if (dev < 0 || dev >= kMaxDevices) return FDTD_ERR_UNSUPPORTED;
    CtxGetCurrentFn get = ctx_get_current();
    auto current = [&]() {
        CUcontext c = nullptr;
        if (get == nullptr || get(&c) != CUDA_SUCCESS) c = nullptr;
        return c;
    };
    // a thread that has not used the runtime yet has no current context: the
    // lookup below binds the device's primary context to it
    CUcontext ctx = current();
    std::lock_guard<std::mutex> lock(g_rows_mutex);
    if (g_rows_addr[dev] == nullptr || ctx == nullptr || g_rows_ctx[dev] != ctx) {
        void *ptr = nullptr;
        e = cudaGetSymbolAddress(&ptr, g_stats_rows);
        if (e != cudaSuccess) return cuda_fail(e);
        g_rows_addr[dev] = static_cast<double *>(ptr);
        g_rows_ctx[dev] = current();
    }
    *out = g_rows_addr[dev];
    return FDTD_OK;
}
}  // namespace

extern "C" {

int fdtd_field_stats_noalloc(const fdtd_plan *plan, double *stats, int32_t n_rows, fdtd_stream_t stream) {
    if (!plan || !stats || n_rows < 0) return FDTD_ERR_ARGUMENT;
    const Plan &p = plan->p;
    const int rows = n_rows ? n_rows : p.stats_ctas;
    if (rows > FDTD_STATS_STATIC_MAX_ROWS) return FDTD_ERR_RANGE;
    // the array used is the current device's: it must be the plan's device
    int cur = 0;
    cudaError_t ce = cudaGetDevice(&cur);
    if (ce != cudaSuccess) return cuda_fail(ce);
    if (cur != p.device) return FDTD_ERR_ARGUMENT;
    double *part = nullptr;
    const int rc = stats_rows_address(&part);
    if (rc != FDTD_OK) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    launch_stats_partial(p, rows, part, st);
    k_stats_final<<<1, 32, 0, st>>>(part, rows, stats);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? FDTD_OK : cuda_fail(e);
}

int fdtd_plan_step_fusion(const fdtd_plan *plan, int32_t *allowed, int32_t *active, int32_t *reason) {
    if (!plan || !allowed || !active) return FDTD_ERR_ARGUMENT;
    *allowed = plan->p.onepass_ok;
    *active = plan->p.onepass;
    if (reason) *reason = plan->p.onepass ? 0 : plan->p.onepass_why;
    return FDTD_OK;
}

int fdtd_plan_tiling(const fdtd_plan *plan, int64_t *out8) {
    if (!plan || !out8) return FDTD_ERR_ARGUMENT;
    const Plan &p = plan->p;
    if (p.onepass) {  // full steps run as one pass each
        out8[0] = PF32::V;
        out8[1] = 32;
        out8[2] = p.ko[0].TY;
        out8[3] = p.ko[0].XC;
        out8[4] = (int64_t)p.ogrid.x * p.ogrid.y * p.ogrid.z;
        out8[5] = 1 + p.onepass_hcopy + (p.n_probe > 0 ? 2 : 0) + (p.n_current > 0 ? 1 : 0) + (int64_t)p.dft.size();
        out8[6] = 4;
        out8[7] = p.ko[0].stages;
        return FDTD_OK;
    }
    out8[0] = p.V;
    out8[1] = p.k.TZ;
    out8[2] = p.k.TY;
    out8[3] = p.k.XC;
    out8[4] = (int64_t)p.grid.x * p.grid.y * p.grid.z;
    out8[5] = p.persistent ? 1 : p.launches_per_step;  // persistent: one launch per fdtd_run call
    out8[6] = p.persistent ? 5 : p.variant + (p.pml_split ? 10 : 0) + (p.n_shell ? 20 : 0);
    out8[7] = p.k.stages;
    return FDTD_OK;
}

const char *fdtd_status_string(int32_t status) {
    switch (status) {
        case FDTD_OK:
            return "ok";
        case FDTD_ERR_ARGUMENT:
            return "invalid argument";
        case FDTD_ERR_UNSUPPORTED:
            return "unsupported configuration";
        case FDTD_ERR_CUDA:
            return "CUDA error";
        case FDTD_ERR_NONFINITE:
            return "non-finite field value";
        case FDTD_ERR_RANGE:
            return "out of range";
    }
    return "unknown status";
}

int32_t fdtd_last_cuda_error(void) { return g_last_cuda; }

size_t fdtd_abi_sizeof(int32_t which) {
    switch (which) {
        case 0:
            return sizeof(fdtd_grid_desc);
        case 1:
            return sizeof(fdtd_boundary_desc);
        case 2:
            return sizeof(fdtd_item_desc);
        case 3:
            return sizeof(fdtd_dft_desc);
        case 4:
            return sizeof(fdtd_run_args);
        case 5:
            return sizeof(fdtd_capture_args);
        case 6:
            return sizeof(fdtd_adjoint_args);
    }
    return 0;
}

}  // extern "C"
