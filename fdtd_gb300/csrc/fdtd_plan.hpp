// Host-side plan of the GB300 FDTD library: launch tiling, the fused-pass
// parameters and the ordered list of small kernels that follow the fused
// pass when a periodic boundary fixes the order of the later stages.
#pragma once

#include <cuda.h>

#include <vector>

#include "fdtd_common.cuh"

namespace fdtd {

enum EpiKind { EPI_COPY = 0, EPI_SLAB = 1, EPI_SOFT = 2, EPI_HARD = 3, EPI_PML = 4, EPI_FEEDBACK = 5 };

struct EpiOp {
    int kind;
    int axis;       // EPI_COPY
    int slab;       // EPI_SLAB (correction only), EPI_PML (auxiliary update and correction)
    int item;       // EPI_HARD, EPI_FEEDBACK
    int run_begin;  // EPI_SOFT
    int run_count;
};

// Tensor maps of the TMA-staged kernels (one 2D view per field and box shape).
enum MapId { MAP_H_NBR = 0, MAP_E_NBR, MAP_E_OWN, MAP_H_OWN, MAP_IE, MAP_MU, MAP_ELO, MAP_HLO, MAP_COUNT };

struct Plan {
    int precision;
    GridK k;           // the grid with every PML slab (epilogue and adjoint kernels)
    GridK kf;          // what the fused pass sees: k, or k without slabs when they run on their own
    GridK kfH;         // the same for the H pass of staged plans (its own ring depth and stage layout)
    int pml_split;     // 1: PML slabs from fused_slabs on run as EPI_PML kernels after the fused pass
    int fused_slabs;   // with pml_split: leading slabs (normal to x or y) kept in the fused pass
    int V;             // cells per thread along z
    dim3 grid, block;  // fused-pass launch shape
    int variant;       // 1 register streaming, 2 TMA-staged
    size_t smem_bytes; // dynamic shared memory of the TMA-staged kernels
    CUtensorMap maps[MAP_COUNT];
    const void *index_E, *index_H;  // one-byte material indices (MAT_IDS)
    std::vector<EpiOp> epi_E, epi_H;
    const int2 *runs;  // device, soft-source runs for EPI_SOFT
    int n_probe;
    const int64_t *probe_cells;
    int n_current;                  // current-probe points (CurrentDetector)
    int has_feedback;               // an FDTD_ITEM_FEEDBACK source exists
    const int64_t *current_cells;
    double grid_spacing;
    std::vector<fdtd_dft_desc> dft;
    int n_columns, n_phase_columns;
    void *dev_mem;     // the plan's own device tables
    int stats_ctas;    // partial rows of the field statistics: 4 per SM, at most FDTD_STATS_STATIC_MAX_ROWS
    int device;        // CUDA device the plan was created on
    int launches_per_step;
    // reverse-time adjoint: launch shape of k_adj_E / k_adj_H, host copies of
    // the items (objects, then E sources, then H sources), the grid.boundaries
    // index of every slab, and the periodic transposes / slab increments that
    // precede the transposed fused pass, in reverse boundary order
    int adj_V;
    dim3 adj_grid, adj_block;
    int adj_TZ, adj_TY, adj_XC;
    // partition plans: the transposed passes' tiling of the interior box
    dim3 adjin_grid, adjin_block;
    int adjin_TZ, adjin_TY, adjin_XC;
    std::vector<ItemK> items_host;
    int n_objects, srcE0, n_srcE, srcH0, n_srcH;
    int slab_boundary[kMaxSlabs];
    std::vector<EpiOp> adj_E, adj_H;
    // one pass per time step (fused E and H half steps on double-buffered
    // state): whether the grid allows it, whether full steps use it (and why
    // not), the periodic H copy it needs after each pass, the GridK of each
    // direction (0: caller buffers -> alternates, 1: back), their tensor maps
    // (H source, E source, E material, H material) and the launch shape
    int onepass_ok, onepass, onepass_hcopy, onepass_why;
    // persistent time loop of small register-streaming plans: allowed, used,
    // its grid-wide barrier and tile-ticket counters (device), the tile order
    // (heaviest first; null: grid order) and resident blocks (0: not yet
    // looked up)
    int persist_ok, persistent;
    unsigned *persist_bar;
    unsigned long long *persist_tickets;
    const int *persist_order;
    int persist_blocks;
    // interior/shell partition (pml_mode 4): the fused pass's tiles cover the
    // interior box; the n_shell boxes around it run one thread per cell with
    // every slab (kshell: the plan's GridK with per-block lists)
    int n_shell;
    GridK kshell;
    ShellK shellk;
    // shell_overlap: the shell launch runs on a second stream beside the
    // interior pass; the stream, fork and join events
    int shell_overlap;
    cudaStream_t shell_stream;
    cudaEvent_t shell_fork, shell_join;
    GridK ko[2];
    CUtensorMap omaps[2][4];
    dim3 ogrid, oblock;
    size_t osmem;
};

// Per-precision entry points (one translation unit per precision).  `cap`
// may be null (plain fdtd_run).
int run_f32(Plan &p, const fdtd_run_args *a, const fdtd_capture_args *cap, cudaStream_t st);
int run_f32c(Plan &p, const fdtd_run_args *a, const fdtd_capture_args *cap, cudaStream_t st);
int run_f64(Plan &p, const fdtd_run_args *a, const fdtd_capture_args *cap, cudaStream_t st);
int adjoint_f32(Plan &p, const fdtd_adjoint_args *a, cudaStream_t st);
int adjoint_f64(Plan &p, const fdtd_adjoint_args *a, cudaStream_t st);

// Stage size in bytes of the TMA-staged kernels for a precision, tile rows
// and the material modes of the E and H passes (the larger of the two).
size_t tma_stage_bytes(int precision, int tile_rows, int mat_E, int mat_H);

// One CTA waiting (bounded) on an mbarrier nothing arrives at; sets bit 0 of
// *status (device) on expiry.
void launch_wait_selftest(int *status, unsigned limit, cudaStream_t st);
// Tensor maps and the shared-memory attribute of the TMA-staged kernels.
int prepare_tma_f32(Plan &p);
int prepare_tma_f32c(Plan &p);
int prepare_tma_f64(Plan &p);

void set_last_cuda_error(int e);

// One-pass step (float32): tensor maps and shared-memory attribute; the pass
// of one direction; bytes of the field part of a stage (what = 0) or of one
// new-E exchange slot (what = 1) for a tile height and the material modes.
int prepare_onepass_f32(Plan &p);
int onepass_step_f32(Plan &p, int dir, const double *wave, cudaStream_t st);
size_t onepass_bytes(int precision, int tile_rows, int mat_E, int mat_H, int what);

inline int grid_stride_blocks(long total) {
    long b = (total + kThreads - 1) / kThreads;
    if (b < 1) b = 1;
    if (b > 152L * 16) b = 152L * 16;
    return (int)b;
}

}  // namespace fdtd
