/*
 * fdtd_gb300.h -- C ABI of the GB300 time-step library for the fdtd FDTD
 * simulator.
 *
 * The reference package (fdtd v0.3.6) is pure Python; its time step is
 * Grid.update_E / Grid.update_H (fdtd/grid.py:275-325), which call the Yee
 * curls (fdtd/grid.py:29-76) and the per-component hooks (PML
 * fdtd/boundaries.py:409-487, periodic copies fdtd/boundaries.py:184-219,
 * objects fdtd/objects.py:118-277, sources fdtd/sources.py:93-109,278-297,
 * 476-486, detectors fdtd/detectors.py:114-124,241-265).  This library
 * replaces that whole chain: one plan describes a registered grid, and each
 * E or H half step is one fused kernel pass over the grid, followed by small
 * kernels where the reference's order requires them (PML slabs run on their
 * own on large grids, periodic plane copies, sources on those planes or
 * slabs, detector gathers).  A reverse-time adjoint (fdtd_run_capture,
 * fdtd_adjoint_run) gives gradients with respect to object materials.
 *
 * Conventions
 *  - Every pointer inside a descriptor is a DEVICE pointer unless stated.
 *  - Fields are component-last: element (i, j, k, c) of an (nx, ny, nz, 3)
 *    array lives at ((i*ny + j)*nz + k)*3 + c.  The element type follows the
 *    plan precision: float for FDTD_FLOAT32 and FDTD_FLOAT32C, double for
 *    FDTD_FLOAT64.
 *  - Functions return an fdtd_status; FDTD_ERR_CUDA keeps the CUDA error code
 *    for fdtd_last_cuda_error().  Nothing traps or aborts.
 *  - Stream arguments are cudaStream_t values (0 = legacy default stream).
 *  - The caller owns every buffer it passes; a plan borrows the pointers in
 *    its descriptor until fdtd_plan_destroy.  A plan allocates only its own
 *    small index tables.  Calls on one plan must be serialised by the caller.
 */
#ifndef FDTD_GB300_H
#define FDTD_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FDTD_ABI_VERSION 5
#define FDTD_MAX_BOUNDARIES 9 /* six PML slabs and three periodic axes */

typedef void *fdtd_stream_t; /* a cudaStream_t */

typedef enum {
    FDTD_OK = 0,
    FDTD_ERR_ARGUMENT = 1,    /* bad descriptor, size or pointer */
    FDTD_ERR_UNSUPPORTED = 2, /* valid input this library does not handle */
    FDTD_ERR_CUDA = 3,        /* a CUDA call failed, see fdtd_last_cuda_error */
    FDTD_ERR_NONFINITE = 4,   /* a field holds NaN or Inf */
    FDTD_ERR_RANGE = 5        /* a record or size is out of range */
} fdtd_status;

typedef enum {
    FDTD_FLOAT32 = 0,  /* float fields and arithmetic */
    FDTD_FLOAT32C = 1, /* float fields plus a float compensation term per
                          E/H value (two-float accumulation) */
    FDTD_FLOAT64 = 2   /* double, same operation order as the reference */
} fdtd_precision;

typedef enum { FDTD_BOUNDARY_PML = 0, FDTD_BOUNDARY_PERIODIC = 1 } fdtd_boundary_kind;

/* One entry of grid.boundaries, in registration order.
 * PML slab: replaces PML.update_phi_E/H and PML.update_E/H
 * (fdtd/boundaries.py:409-487) for the slab subclasses of
 * fdtd/boundaries.py:490-625.  Only the two auxiliaries per half step that
 * can be non-zero are stored (compact layout): psi_E holds, for every slab
 * cell, the pair (psi driving E[(axis+1)%3], psi driving E[(axis+2)%3]); the
 * slab cells are ordered like the grid with the slab axis cut to `thickness`
 * (for a z slab the stored z extent is thickness rounded up to even, so that
 * every row of auxiliaries is a multiple of 16 bytes).
 * Periodic: replaces _PeriodicBoundary{X,Y,Z}.update_E/H
 * (fdtd/boundaries.py:184-219). */
typedef struct {
    int32_t kind;       /* fdtd_boundary_kind */
    int32_t axis;       /* 0 = x, 1 = y, 2 = z */
    int32_t high;       /* PML: 0 = low side, 1 = high side */
    int32_t thickness;  /* PML: cells along axis */
    void *psi_E;        /* PML: [slab cells][2] */
    void *psi_H;        /* PML: [slab cells][2] */
    const void *b_E;    /* PML: [thickness] exp(-(sigma_E/k + a) * courant) */
    const void *c_E;    /* PML: [thickness] */
    const void *b_H;    /* PML: [thickness] */
    const void *c_H;    /* PML: [thickness] */
} fdtd_boundary_desc;

typedef enum {
    FDTD_ITEM_OBJECT = 0,      /* E += coef0 * curlH; coef0 = courant * inverse_permittivity
                                  (fdtd/objects.py:118-129) */
    FDTD_ITEM_ABSORBING = 1,   /* E = E*coef0 + (coef1*curlH)/coef2 with coef0 = (1-f)/(1+f),
                                  coef1 = courant*inverse_permittivity, coef2 = 1+f
                                  (fdtd/objects.py:207-221); float plans use coef1/coef2
                                  premultiplied in coef1 and ignore coef2 */
    FDTD_ITEM_ANISOTROPIC = 2, /* E += courant * (coef0 @ curlH), coef0 [cell][3][3]
                                  (fdtd/objects.py:254-269) */
    FDTD_ITEM_SOFT = 3,        /* F[comp] += weight * wave[column] (PointSource, LineSource) */
    FDTD_ITEM_HARD = 4,        /* F[comp]  = weight * wave[column] (PlaneSource) */
    FDTD_ITEM_FEEDBACK = 5     /* E[comp] += (wave[column] + weight * I) / grid_spacing, I the
                                  current of current-probe point `aux` after the previous H
                                  half (0 at step 0); the weight term only when weight > 0
                                  (SoftArbitraryPointSource.update_E, fdtd/sources.py:600-629) */
} fdtd_item_kind;

/* An object box or a source box/point.  Object coefficient arrays are
 * box-local: cell (i, j, k) of the box is entry ((i*bny + j)*bnz + k). */
typedef struct {
    int32_t kind;     /* fdtd_item_kind */
    int32_t comp;     /* sources: field component 0..2 */
    int32_t column;   /* sources: column of the per-step waveform row */
    int32_t source;   /* sources: index in grid.sources (fixes the order) */
    int32_t lo[3];    /* first cell (x, y, z) */
    int32_t hi[3];    /* one past the last cell (x, y, z) */
    double weight;    /* sources: amplitude or profile weight; feedback: source impedance */
    const void *coef[3];
    int32_t aux;      /* FDTD_ITEM_FEEDBACK: index of its point in current_cells */
    int32_t reserved;
} fdtd_item_desc;

/* Running DFT of E on a box: acc[f][cell][c] += E[cell][c] * (phase_re + i*phase_im),
 * accumulated in double after every E half step (not in the reference). */
typedef struct {
    int32_t lo[3];
    int32_t hi[3];
    int32_t n_freq;
    int32_t phase_offset; /* first frequency column of the per-step phase row */
    double *acc;          /* [n_freq][box cells][3] interleaved (re, im) */
} fdtd_dft_desc;

typedef struct {
    int32_t abi_version;  /* FDTD_ABI_VERSION */
    int32_t precision;    /* fdtd_precision */
    int32_t nx, ny, nz;
    int32_t x_chunk;      /* planes per CTA along x; 0 = automatic */
    int32_t variant;      /* fused-pass kernels: 0 automatic, 1 register streaming,
                             2 TMA-staged (needs nz a multiple of 4 floats / 2 doubles) */
    int32_t tile_rows;    /* TMA-staged: rows per CTA, 4 or 8 (tiles 32 threads wide along z)
                             or 16 (16 threads wide); 0 = automatic */
    int32_t stages;       /* TMA-staged: shared-memory ring depth, >= 2; 0 = automatic */
    int32_t pml_mode;     /* PML slabs: 0 automatic, 1 inside the fused pass, 2 one kernel per
                             slab after the fused pass (auxiliary update and correction),
                             3 the slabs normal to x or y that lead the boundary list inside
                             the fused pass and the others in kernels of their own,
                             4 interior/shell partition: the fused pass (staged or register
                             streaming) over the box inside every slab, one kernel with every
                             slab over the boxes around it (needs nz a multiple of the vector
                             width, every PML before any periodic boundary and a non-empty
                             interior; else FDTD_ERR_UNSUPPORTED) */
    double courant;
    void *E;              /* [nx][ny][nz][3] */
    void *H;
    void *E_lo;           /* FDTD_FLOAT32C: compensation terms, else NULL */
    void *H_lo;
    const void *inv_eps;  /* [nx][ny][nz][3] grid.inverse_permittivity */
    const void *inv_mu;   /* [nx][ny][nz][3] grid.inverse_permeability */
    int32_t n_boundaries;
    fdtd_boundary_desc boundaries[FDTD_MAX_BOUNDARIES];
    int32_t n_objects;    /* grid.objects, registration order */
    const fdtd_item_desc *objects;    /* HOST array */
    int32_t n_sources_E;  /* source items acting in the E half step, grid.sources order */
    const fdtd_item_desc *sources_E;  /* HOST array */
    int32_t n_sources_H;
    const fdtd_item_desc *sources_H;  /* HOST array */
    int32_t n_columns;    /* width of one waveform row */
    int32_t n_probe_cells;            /* detector sample points, all detectors */
    const int64_t *probe_cells;       /* [n_probe_cells] linear cell index */
    int32_t n_dft;
    const fdtd_dft_desc *dft;         /* HOST array */
    int32_t n_phase_columns;          /* width of one DFT phase row (pairs) */
    int32_t n_current_cells;          /* current-probe points (CurrentDetector), all detectors */
    const int64_t *current_cells;     /* [n_current_cells] linear cell index */
    double grid_spacing;              /* metres (current probes, feedback sources) */
    int32_t materials_scaled;         /* FDTD_FLOAT64 only: 1 = inv_eps and inv_mu hold
                                         courant * inverse_permittivity / permeability (the
                                         products the reference forms first), so the kernels
                                         skip that multiply; 0 = plain inverse materials */
    /* Optional compact copies of inv_eps / inv_mu for the TMA-staged passes
     * (inv_eps and inv_mu stay required in full for the other kernels): a
     * table of n value triples (plan element type) and a one-byte index per
     * cell ([nx][ny][nz], nz a multiple of 16) with inv_eps[cell] ==
     * table[index[cell]] for every cell; or n = 1 and index = NULL when every
     * cell holds table[0].  The staged passes (and the PML slab kernels of
     * such plans) then read one byte per cell, or nothing, instead of three
     * values.  n = 0: not given.  The caller keeps the copies consistent with
     * the full arrays; an index byte >= n reads zeros.  An index whose
     * pointer is not 16-byte aligned, or nz not a multiple of 16, leaves the
     * plan on the full arrays. */
    const void *eps_table;
    int32_t n_eps_table;                /* 0 .. 256 */
    const uint8_t *eps_index;
    const void *mu_table;
    int32_t n_mu_table;
    const uint8_t *mu_index;
    /* One pass per time step (ABI 5).  The E and H half steps of a full step
     * run as one TMA-staged pass that reads E, H, the PML auxiliaries and the
     * materials once and writes E, H and the auxiliaries once; it reads the
     * old values from one copy and writes the new ones to another, so the
     * caller provides a second buffer of the same size for E, H and every PML
     * auxiliary array (contents ignored).  Steps run in pairs that end in the
     * caller's own buffers; an odd last step, single half steps and
     * fdtd_run_capture use the two-pass kernels.  Float32 plans whose PML
     * slabs all precede any periodic boundary, with periodic boundaries only
     * along x, no object or source on a periodic plane, and without a
     * feedback source.  step_fusion: 0 automatic (currently off: the
     * two-pass plans measured faster on every benchmark grid), 1 off, 2 on
     * where the grid allows it.  fdtd_plan_step_fusion reports whether a grid allows it (before any
     * buffer is allocated), whether the plan uses it, and why not. */
    int32_t step_fusion;
    /* Persistent time loop (ABI 5): on small grids whose plan runs the
     * register-streaming passes with nothing between them but detector
     * gathers and DFT sums, fdtd_run runs all full steps of a call in one
     * cooperative launch whose blocks meet at a grid-wide barrier between
     * half steps (bounded waits: bit 2 of the status word on expiry).  0
     * automatic (float32 grids below 3M cells, float64 below 8M), 1 off, 2 on
     * where the plan allows it. */
    int32_t persistent;
    void *E_alt;
    void *H_alt;
    void *psi_alt[FDTD_MAX_BOUNDARIES][2]; /* per PML boundary: second psi_E, psi_H; NULL for periodic */
} fdtd_grid_desc;

typedef struct fdtd_plan fdtd_plan;

/* Arguments of one fdtd_run call: n_steps full steps, or a single half step. */
typedef struct {
    int64_t n_steps;
    int32_t half;          /* 0: full steps; 1: only the E half; 2: only the H half (n_steps = 1) */
    int32_t reserved;
    const double *wave;    /* [n_steps][n_columns] waveform value per source column, step s */
    const double *phase;   /* [n_steps][n_phase_columns][2] DFT factors (cos, -sin) */
    void *trace_E;         /* [capacity][n_probe_cells][3] detector samples after E halves */
    void *trace_H;         /* [capacity][n_probe_cells][3] after H halves */
    int64_t trace_capacity;
    int64_t record_E;      /* row of trace_E written by the first E half */
    int64_t record_H;
    void *trace_I;         /* [capacity][n_current_cells] currents after H halves
                              (CurrentDetector.detect_H, fdtd/detectors.py:404-480) */
    int64_t record_I;      /* row of trace_I written by the first H half */
    int64_t step0;         /* time_steps_passed at the first step (feedback sources use the
                              previous current only after step 0) */
} fdtd_run_args;

/* Build a plan for a registered grid (replaces the per-step dispatch of
 * fdtd/grid.py:275-325).  Validates the descriptor, chooses the launch
 * tiling and builds the per-CTA object and source lists. */
int fdtd_plan_create(const fdtd_grid_desc *desc, fdtd_plan **out);

/* Release the plan's own tables (never the caller's buffers). */
int fdtd_plan_destroy(fdtd_plan *plan);

/* Device status word of the plan, copied to *out after synchronising the
 * stream: 0 = healthy; bit 0 = a staged kernel's pipeline wait expired (the
 * step's results are invalid); bit 1 = besides, a CTA gave up waiting for its
 * own copies in flight (results of later kernels on this context are
 * untrusted too); bit 2 = a persistent run's grid-wide barrier wait expired
 * (the run's results are invalid).  reset != 0 clears the word afterwards.  No
 * reference counterpart (the reference cannot fail this way). */
int fdtd_plan_status(fdtd_plan *plan, int32_t *out, int32_t reset, fdtd_stream_t stream);

/* Device check of the staged passes' failure path; no counterpart in the
 * reference.  One CTA waits on an mbarrier that nothing arrives at, giving up
 * after `polls` polls (the staged passes use the same bounded wait), and sets
 * bit 0 of a status word on expiry, which *status_out receives (1 expected).
 * Nothing faults; the context stays usable.  Synchronises `stream`. */
int fdtd_selftest_bounded_wait(uint32_t polls, int32_t *status_out, fdtd_stream_t stream);

/* Grid.run / Grid.step / Grid.update_E / Grid.update_H
 * (fdtd/grid.py:250-325): n_steps steps (or one half step) with detector
 * sampling and DFT accumulation after each half step. */
int fdtd_run(fdtd_plan *plan, const fdtd_run_args *args, fdtd_stream_t stream);

/* ---------------------------------------------------------------------------
 * Reverse-time adjoint (no counterpart in the reference, which has no
 * gradients; it stands in for autograd through the reference's torch
 * backend).  The time step is affine in the state (E, H, PML auxiliaries),
 * so the adjoint state (lam_E, lam_H and two adjoint auxiliaries per PML
 * slab) evolves backwards under the transposed step, independent of the
 * forward fields.  The gradient of a loss with respect to an object's
 * inverse permittivity needs the forward curl_H on the object's box at every
 * step; fdtd_run_capture stores it while running forward steps (the caller
 * recomputes segments from its own field checkpoints).
 * ------------------------------------------------------------------------- */
typedef struct {
    int32_t detectors;     /* 1: sample detectors and accumulate DFTs as fdtd_run does;
                              0: skip them (recomputing a segment) */
    int32_t n_curl;        /* entries of `curl`: 0 or the plan's object count */
    void *const *curl;     /* HOST array of DEVICE pointers: per object NULL, or
                              [n_steps][box cells][3] curl_H(H) on the object's box taken
                              before each E half step (plan element type) */
} fdtd_capture_args;

/* fdtd_run (full steps only) plus the captures above. */
int fdtd_run_capture(fdtd_plan *plan, const fdtd_run_args *args, const fdtd_capture_args *cap,
                     fdtd_stream_t stream);

typedef struct {
    int64_t n_steps;       /* reverse steps of this call: forward steps top-1 down to top-n_steps */
    int32_t parity;        /* which buffer of every aux pair holds the current adjoint auxiliaries;
                              the call leaves them in buffer parity ^ (n_steps & 1) */
    int32_t n_objects;     /* entries of `curl` and `grad`: the plan's object count */
    void *lam_E;           /* [nx][ny][nz][3] adjoint of E, plan element type */
    void *lam_H;
    void *aux_E[FDTD_MAX_BOUNDARIES][2]; /* per PML boundary (grid.boundaries index): two
                                            buffers of psi_E's layout; NULL for periodic */
    void *aux_H[FDTD_MAX_BOUNDARIES][2];
    const void *seed_E;    /* [rows][n_probe_cells][3] dL/d(trace_E), or NULL */
    const void *seed_H;    /* [rows][n_probe_cells][3] dL/d(trace_H), or NULL */
    int64_t seed_row;      /* seed row of the first reverse step; one less per step */
    const double *const *dft_grad; /* HOST array of n_dft DEVICE pointers (NULL entries allowed):
                                      dL/d(acc) as [n_freq][box cells][3][re, im] */
    const double *phase;   /* [n_steps][n_phase_columns][2] (cos, -sin) of the DFT at the
                              forward step of reverse step s, row s */
    const void *const *curl;   /* HOST array: per object NULL or the captures of
                                  fdtd_run_capture */
    int64_t curl_row;      /* capture row of the first reverse step; one less per step */
    double *const *grad;   /* HOST array: per object NULL or the gradient accumulator,
                              [box cells][3] (FDTD_ITEM_OBJECT: dL/d inverse_permittivity) or
                              [box cells][3][3] (FDTD_ITEM_ANISOTROPIC), added to */
} fdtd_adjoint_args;

/* n_steps reverse steps of the adjoint (float32 and float64 plans): per step
 * the transposed H half then the transposed E half, with detector seeds added
 * where the forward step sampled, hard-source cells zeroed, periodic copies
 * transposed (lam[src] += lam[dst]; lam[dst] = 0), and gradient accumulation
 * grad += courant * curl_H * lam_E on every object box with a grad pointer.
 * Objects with a grad pointer must be FDTD_ITEM_OBJECT or
 * FDTD_ITEM_ANISOTROPIC. */
int fdtd_adjoint_run(fdtd_plan *plan, const fdtd_adjoint_args *args, fdtd_stream_t stream);

/* curl_E (fdtd/grid.py:29-51) and curl_H (fdtd/grid.py:54-76) as
 * stand-alone kernels: out = curl(in), both [nx][ny][nz][3]. */
int fdtd_curl_E(int32_t precision, const void *E, void *out, int32_t nx, int32_t ny, int32_t nz,
                fdtd_stream_t stream);
int fdtd_curl_H(int32_t precision, const void *H, void *out, int32_t nx, int32_t ny, int32_t nz,
                fdtd_stream_t stream);

/* Field statistics for failure detection (no reference counterpart; the
 * reference has no health check): stats[0] = sum E^2, stats[1] = sum H^2,
 * stats[2] = max |E|, stats[3] = max |H|, stats[4] = number of non-finite
 * values, written to the DEVICE array `stats` (5 doubles).  Uses `scratch`,
 * a device buffer of fdtd_stats_scratch_bytes(plan) bytes.  Returns
 * FDTD_OK; the caller reads stats[4] to decide. */
size_t fdtd_stats_scratch_bytes(const fdtd_plan *plan);
int fdtd_field_stats(const fdtd_plan *plan, double *stats, void *scratch, fdtd_stream_t stream);

/* fdtd_field_stats without any device allocation, for callers that cannot
 * call cudaMalloc or hand out a scratch buffer: for example a host
 * application whose device memory is owned by another framework's allocator,
 * or a monitoring hook between time steps that must not touch an allocator
 * (cudaMalloc/cudaFree can synchronise the device and fragment a caching
 * allocator).  The per-CTA partial sums live in a fixed device array compiled
 * into this library: FDTD_STATS_STATIC_MAX_ROWS rows of 5 doubles (40 KiB),
 * held by every GPU that loads the library until the process exits.
 * n_rows = number of partial rows (CTAs) to use, 0 = the plan's default (the
 * same rows fdtd_field_stats uses, so both give identical results); a value
 * above FDTD_STATS_STATIC_MAX_ROWS returns FDTD_ERR_RANGE without launching.
 * The current device must be the plan's device (else FDTD_ERR_ARGUMENT).
 * The first call on a device looks up the array's device address (with that
 * device current) and keeps it with the context it belongs to; make that
 * first call before any stream capture.  After a device reset
 * (cudaDeviceReset, a new primary context) the kept address is stale: the
 * first call in the new context looks it up again, so make that call before
 * any capture too.  All calls share the array and it keeps the last call's contents
 * (every row used is rewritten before it is read, so nothing needs clearing);
 * calls that overlap on the GPU race with each other.  No counterpart in the
 * reference (the reference has no health check). */
#define FDTD_STATS_STATIC_MAX_ROWS 1024
int fdtd_field_stats_noalloc(const fdtd_plan *plan, double *stats, int32_t n_rows, fdtd_stream_t stream);

/* One pass per time step: *allowed = 1 when the grid admits it (whether or
 * not the second buffers were given), *active = 1 when full steps of this
 * plan run as one pass each; *reason (may be NULL) says why not: 0 active
 * or not asked, 1 not float32, 2 nz not a multiple of 4 or an unaligned
 * buffer, 3 a feedback source, 4 a PML slab after a periodic boundary,
 * 5 a periodic boundary not along x (or nx < 4), 6 an object or source on a
 * periodic plane, 7 no second buffers, 8 too little shared memory, 9 grid
 * too large for the launch, 10 a tensor map was refused.  No reference
 * counterpart. */
int fdtd_plan_step_fusion(const fdtd_plan *plan, int32_t *allowed, int32_t *active, int32_t *reason);

/* Launch tiling chosen by the plan: out[0..7] = cells per thread along z,
 * threads along z, rows along y, planes along x per CTA, CTAs, kernels per
 * full step, variant (1 register streaming, 2 TMA-staged; plus 10 when the
 * PML slabs run in kernels of their own, plus 20 for an interior/shell
 * partition, whose interior tiling is then reported; 4 one pass per full
 * step, whose tiling is then reported; 5 the persistent loop of
 * register-streaming tiles, one launch per fdtd_run call), ring stages. */
int fdtd_plan_tiling(const fdtd_plan *plan, int64_t *out8);

const char *fdtd_status_string(int32_t status);
int32_t fdtd_last_cuda_error(void);
/* sizeof of the ABI structs, for binding checks: 0 grid_desc, 1 boundary_desc,
 * 2 item_desc, 3 dft_desc, 4 run_args, 5 capture_args, 6 adjoint_args. */
size_t fdtd_abi_sizeof(int32_t which);

#ifdef __cplusplus
}
#endif
#endif /* FDTD_GB300_H */
