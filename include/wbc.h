/*
 * wbc.h — C-ABI of libwbc_gb300.so, the GB300 (sm_103a) implementation of WarpBioCell's
 * coupled cell step.
 *
 * Every entry point takes plain device pointers and sizes, launches asynchronously on the
 * given CUDA stream (`stream` is a cudaStream_t passed as void*; NULL = legacy default stream)
 * and returns WBC_OK or a negative WBC_ERR_* code. Nothing here allocates, frees or owns
 * memory: the caller owns every buffer (capacity-sized, as in the reference's CellPopulation)
 * and passes the scratch buffers whose sizes the *_workspace_bytes queries return.
 *
 * Layouts (all C order, little-endian):
 *   position, velocity     float[capacity][3]   (x, y, z) per slot
 *   per-cell scalars       float/int32/uint32[capacity]
 *   fields                 float[nx][ny][nz]    (k fastest, as the reference's array3d)
 *   deposit accumulator    int64[4][nx][ny][nz] (state layer, then node)
 *   network states         uint64[capacity][n_words], node i at word i/64, bit i%64
 *
 * Each declaration names the reference function it replaces (paths inside the
 * Gennappio/WarpBioCell project, src/warpbiocell/...).
 */
#ifndef WBC_H
#define WBC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------------------------ */
#define WBC_OK 0
#define WBC_ERR_INVALID (-1)       /* bad argument (null pointer, negative size, bad geometry) */
#define WBC_ERR_CAPACITY (-2)      /* more cells than the allocation holds */
#define WBC_ERR_CUDA (-4)          /* a CUDA launch or runtime call failed; see wbc_last_error */
#define WBC_ERR_TIMEOUT (-5)       /* a bounded device-side wait ran out */
#define WBC_ERR_WORKSPACE (-6)     /* scratch buffer smaller than the *_workspace_bytes query */

/* Cell states (cells/model.py:14-18) and network fate bits (kernels/network_kernels.py:29-32). */
#define WBC_STATE_PROLIFERATIVE 0
#define WBC_STATE_QUIESCENT 1
#define WBC_STATE_HYPOXIC 2
#define WBC_STATE_DEAD 3
#define WBC_FATE_PROLIFERATION 1
#define WBC_FATE_APOPTOSIS 2
#define WBC_FATE_GROWTH_ARREST 4
#define WBC_FATE_NECROSIS 8

/* Library version and the last CUDA error message seen by this thread (never NULL). */
int wbc_version(void);
const char* wbc_last_error(void);
/* Number of CUDA devices visible to the runtime (0 on a machine without a GPU). */
int wbc_device_count(void);
/* Kernels launched by this library in this process so far (all threads and devices). */
int64_t wbc_launch_count(void);

/* ---- per-cell random streams --------------------------------------------------------------- */
/* rng_state[i] = stream start of slot i for every slot in [0, capacity).
 * Replaces cells/state.py:25-28 (_init_rng) as launched at cells/state.py:110. */
int wbc_rng_init(int32_t seed, uint32_t* rng_state, int64_t capacity, void* stream);
/* Test hooks: draw `draws` uniform floats / unit-sphere directions from streams [0, n); the
 * streams advance in place (same functions the lifecycle and placement kernels use). */
int wbc_rng_uniform(int32_t n, int32_t draws, uint32_t* rng_state, float* out, void* stream);
int wbc_rng_sphere(int32_t n, uint32_t* rng_state, float* out_xyz, void* stream);
/* Test hook: the project's exp(x) on n floats (used for every death / division probability). */
int wbc_expf_batch(int32_t n, const float* x, float* out, void* stream);
/* Test hook: the solver's correctly rounded division a[i] / b[i] (bit-identical to IEEE). */
int wbc_div_batch(int32_t n, const float* a, const float* b, float* out, void* stream);
/* Self-check of that division on the device. mode 0: the refined reciprocal of every float with
 * exponent in [e_lo, e_hi] (both signs) against IEEE 1/b; mode 1: `pairs` seeded operand pairs
 * (raw bit patterns, wide exponents, exact products, near-midpoint quotients) against IEEE a/b.
 * Adds the number of differing results to *mismatches (device) and stores the first differing
 * operands (a, b bits) in first_bad[0..1] (device). */
int wbc_div_check(int32_t mode, int32_t e_lo, int32_t e_hi, uint32_t seed, int64_t pairs,
                  unsigned long long* mismatches, uint32_t* first_bad, void* stream);

/* ---- hash-grid binning + contact mechanics -------------------------------------------------- */
typedef struct wbc_neighbor_grid {
    int32_t dim;             /* buckets per axis; cells hash as (floor(x / bucket)) mod dim      */
    float cell_size;         /* query radius [um]; the bucket edge is cell_size * (1 + 2^-10)   */
    int32_t* bucket_count;   /* int32[dim^3]                                                     */
    int32_t* bucket_start;   /* int32[dim^3] exclusive prefix sum of bucket_count                */
    int32_t* cell_bucket;    /* int32[capacity] bucket of each slot                               */
    int32_t* cell_rank;      /* int32[capacity] arrival rank inside the bucket (unordered)         */
    int32_t* scatter;        /* int32[capacity] slots grouped by bucket, unordered inside one      */
    int32_t* sorted_id;      /* int32[capacity] slots grouped by bucket, ascending inside one      */
    float* sorted_xyzr;      /* float[capacity][4] (x, y, z, radius) in sorted_id order            */
    int32_t* scan_partials;  /* scratch, wbc_scan_workspace_bytes(dim^3) bytes                     */
    int64_t capacity;
} wbc_neighbor_grid;

size_t wbc_scan_workspace_bytes(int64_t n);
/* Bin the active prefix [0, n): counting sort of slots into hashed buckets, stable in slot
 * order, plus a coalesced float4 copy of (x, y, z, r). Replaces spatial/neighbors.py:33-37
 * (NeighborGrid.build -> warp HashGrid.build). */
int wbc_grid_build(const wbc_neighbor_grid* grid, int32_t n, const float* position, const float* radius,
                   void* stream);
/* One contact substep over a built grid: neighbour count (|x_i - x_j| < query_radius, j != i),
 * overlap-repulsion velocity, and x += v dt, fused. Replaces kernels/mechanics_kernels.py:26-57
 * (contact_velocities) + :60-67 (integrate_positions) as driven by cells/mechanics.py:75-109. */
int wbc_contact_substep(const wbc_neighbor_grid* grid, int32_t n, float query_radius, float rate, float dt,
                        float* position, float* velocity, int32_t* neighbor_count, void* stream);

/* ---- fields ------------------------------------------------------------------------------------ */
typedef struct wbc_grid_geometry {
    int32_t nx, ny, nz;
    float origin_x, origin_y, origin_z;
    float inv_dx;
} wbc_grid_geometry;

/* ---- tissue region ------------------------------------------------------------------------------
 * A signed-distance field on its own grid (negative inside) and its node gradient. */
typedef struct wbc_tissue_region {
    wbc_grid_geometry geom;
    const float* sdf;             /* float[nodes]                                                    */
    const float* gradient;        /* float[nodes][3] (x, y, z)                                       */
    float wall_rate;              /* ContactParams.wall_rate [1/h]                                   */
} wbc_tissue_region;

/* wbc_contact_substep plus the region's confinement push before the Euler step
 * (cells/mechanics.py:75-110 with kernels/geometry_kernels.py:59-79). */
int wbc_contact_substep_region(const wbc_neighbor_grid* grid, int32_t n, float query_radius, float rate, float dt,
                               const wbc_tissue_region* region, float* position, float* velocity,
                               int32_t* neighbor_count, void* stream);
/* Trilinear signed distance at each cell, positions clamped to the grid
 * (kernels/geometry_kernels.py:46-56, geometry/region.py sample_at). */
int wbc_sample_sdf(const wbc_tissue_region* region, int32_t n, const float* position, float* out, void* stream);

/* accumulator[state][node] += int64(w * 2^24 + 0.5) for the 8 trilinear corners of each living
 * or dead cell with 0 <= state < 4; cells outside the trilinear support are skipped.
 * Replaces kernels/field_kernels.py:78-116 (deposit_trilinear). The accumulator is not cleared. */
int wbc_deposit(const wbc_grid_geometry* geom, int32_t n, const float* position, const int32_t* cell_state,
                int64_t* accumulator, void* stream);
/* density[s][node] = float(acc[s][node]) / 2^24 * inv_voxel_volume (kernels/field_kernels.py:119-126)
 * and, when `combined` is non-NULL, combined[node] = sum_k weights[k] * density[k][node] in the
 * reference's order (kernels/field_kernels.py:129-142). `clear` != 0 zeroes the accumulator as it
 * is read. `density` may be NULL when only the combination is wanted. */
int wbc_density_convert(int64_t nodes, int64_t* accumulator, float inv_voxel_volume, float* density,
                        const float* weights4, float* combined, int32_t clear, void* stream);
/* The same deposit as wbc_deposit (kernels/field_kernels.py:78-116, the same integer sums) into a
 * 32-bit accumulator with an exact carry: `accumulator` holds uint32 low words L[4][nodes], uint32
 * wrap counts C[4][nodes] and a carry flag (wbc_deposit32_bytes(nodes) bytes, 16-byte aligned).
 * The low words are added to in aligned pairs (2m, 2m+1) by 64-bit atomics, so the sum of word w
 * is L[w] + 2^32 C[w] for even w and L[w] + 2^32 C[w] - C[w-1] for odd w (C is all zero, and the
 * sums are the low words, while the carry flag is 0). The call clears the low words first (and the
 * counts when the previous deposit wrapped), so the caller never clears it, and it keeps the sums
 * until the next deposit. `order` (NULL = 0 .. n - 1) is a permutation of the cells to visit, e.g.
 * the hash grid's sorted ids: the sums do not depend on it, but the atomics of neighbouring cells
 * then hit nearby lines. Replaces
 * fields/densities.py:26-43 (CellDensities.deposit's int64 accumulator). */
size_t wbc_deposit32_bytes(int64_t nodes);
int wbc_deposit32(const wbc_grid_geometry* geom, int32_t n, const float* position, const int32_t* cell_state,
                  const int32_t* order, void* accumulator, size_t accumulator_bytes, void* stream);
/* wbc_density_convert from the 32-bit accumulator, which it leaves as it is (the per-state densities
 * can be produced later from the same deposit): density[4][nodes] when non-NULL and combined =
 * sum_k weights4[k] density_k when non-NULL (kernels/field_kernels.py:119-142). */
int wbc_convert32(int64_t nodes, const void* accumulator, float inv_voxel_volume, float* density,
                  const float* weights4, float* combined, void* stream);
/* out = sum_k weights[k] * density[k] (kernels/field_kernels.py:129-142, fields/densities.py:45-50). */
int wbc_density_combine(int64_t nodes, const float* weights4, const float* density, float* out, void* stream);
/* Clamped trilinear interpolation at each cell (kernels/field_kernels.py:153-182). */
int wbc_sample(const wbc_grid_geometry* geom, const float* field, int32_t n, const float* position,
               float* out, void* stream);

typedef struct wbc_sor_params {
    int32_t nx, ny, nz;
    int32_t bc_x, bc_y, bc_z;    /* 0 = Dirichlet face (never written), 1 = Neumann (mirror)      */
    float omega;
    float dx2_over_D;            /* h = dx^2 / D                                                    */
    float uptake_max;
    float michaelis_k;
    float reference;             /* residual scale: boundary value, or 1 when it is 0               */
    int32_t has_source;
    float source_k;
} wbc_sor_params;

/* `sweeps` red-black SOR sweeps in place (kernels/field_kernels.py:185-212 launched as in
 * fields/diffusion.py:103-112), then, when residual_out is non-NULL, the max-norm residual of
 * the result (kernels/field_kernels.py:215-243) written to residual_out[0] (device float).
 * `fixed` int32[nodes] (non-zero = pinned) may be NULL when no node is pinned; `production` and
 * `source` may be NULL. */
int wbc_sor_sweeps(const wbc_sor_params* p, int32_t sweeps, const int32_t* fixed, const float* density,
                   const float* production, const float* source, float* field, float* residual_out,
                   void* stream);
typedef struct wbc_sor_report {
    int32_t sweeps;              /* sweeps performed (a multiple of check_every, or max_sweeps)     */
    float residual;              /* max-norm residual after the last check                          */
    int32_t converged;           /* residual < tolerance                                             */
    int32_t path;                /* 2 = shared-memory resident solver, 1 = streaming colour launches */
    int32_t tiles;               /* CTAs of the resident solver (0 for the streaming path)           */
    int32_t strips;              /* strips along j the tiles are cut from (resident path)             */
} wbc_sor_report;

/* Optional choices for the resident solver (NULL or zeros = automatic). The (i, j) plane of
 * columns is cut into `strips` strips along j, and each strip's columns, row by row, into equal
 * runs, one per tile: `tiles` tiles (CTAs, at most one per SM; 0 = every SM). Every choice gives
 * the same field bits. */
typedef struct wbc_sor_tuning {
    int32_t tiles;
    int32_t strips;
} wbc_sor_tuning;

/* Scratch bytes wbc_sor_solve needs for this grid (control block, halo exchange buffers, the
 * coefficient copy and the production-term copy); the workspace must be 16-byte aligned. */
size_t wbc_sor_solve_workspace_bytes(const wbc_sor_params* p);
/* Solve to the residual tolerance from the field's current values (warm start), checking the
 * residual every `check_every` sweeps and stopping at `max_sweeps`: the sweep count, residual and
 * stopping rule of fields/diffusion.py:79-123 (kernels/field_kernels.py:185-243). path 0 = auto:
 * one persistent cooperative launch with the field tile resident in shared memory when the grid
 * fits on chip, otherwise streaming colour launches with a host check per chunk; 1 = streaming;
 * 2 = resident only. Synchronises `stream` and fills the host-side `report`; when residual_out is
 * non-NULL the final residual is also written there (device float, the reference's
 * residual_buffer). The field after the solve is bit-identical on both paths and for every
 * `tuning` (may be NULL). Returns WBC_ERR_TIMEOUT if a device wait timed out. */
int wbc_sor_solve(const wbc_sor_params* p, int32_t check_every, int32_t max_sweeps, double tolerance,
                  const int32_t* fixed, const float* density, const float* production, const float* source,
                  float* field, float* residual_out, wbc_sor_report* report, void* workspace,
                  size_t workspace_bytes, int32_t path, const wbc_sor_tuning* tuning, void* stream);
/* wbc_sor_solve without waiting for its report: the resident solve copies its report into
 * `record` (host memory of wbc_sor_report_record_bytes() bytes, pinned so that the copy stays
 * asynchronous) in stream order and the call returns at once; wbc_sor_report_decode reads it once
 * the stream has passed the solve (after a synchronisation the caller makes anyway, e.g. reading
 * the division count). A grid that is solved on the streaming path is solved synchronously and
 * its record is final at once. The same solve, sweeps and bits as wbc_sor_solve. */
size_t wbc_sor_report_record_bytes(void);
int wbc_sor_solve_deferred(const wbc_sor_params* p, int32_t check_every, int32_t max_sweeps, double tolerance,
                           const int32_t* fixed, const float* density, const float* production, const float* source,
                           float* field, float* residual_out, void* record, void* workspace, size_t workspace_bytes,
                           int32_t path, const wbc_sor_tuning* tuning, void* stream);
/* The report of a deferred solve (WBC_ERR_TIMEOUT if one of its device waits timed out). */
int wbc_sor_report_decode(const void* record, wbc_sor_report* report);
/* The linear system d_a x_a - sum_nb x_nb = b_a (d_a > 0; nodes with d_a <= 0 and Dirichlet faces
 * keep their values in x) by red-black SOR with relaxation p->omega in the same resident
 * launch as wbc_sor_solve, from x's current values, checking every `check_every` sweeps whether
 * max_a |b_a + sum_nb x_nb - d_a x_a| < tolerance * max_a max(6 |x_a|, |b_a|). Only nx, ny, nz,
 * the boundary flags and omega of `p` are read. Used by the hand-written adjoint (the transposed
 * linearised field operator) and by its Newton correction of the forward steady state; no
 * counterpart in the reference. Synchronises `stream`; WBC_ERR_INVALID if the grid does not fit
 * the resident solver. */
int wbc_sor_linear_solve(const wbc_sor_params* p, int32_t check_every, int32_t max_sweeps, double tolerance,
                         const float* diag, const float* rhs, float* x, wbc_sor_report* report, void* workspace,
                         size_t workspace_bytes, void* stream);
/* Self-test of the solver's bounded device waits (no counterpart in the reference): runs the grid
 * barrier of the resident solver `rounds` times on `ctas` expected CTAs, of which `ctas - missing`
 * are launched (cooperatively, one small CTA each; ctas <= the SM count). With missing = 0 the
 * barriers complete and WBC_OK is returned; with missing > 0 the missing CTAs never arrive, every
 * launched CTA stops waiting after its time limit (2 s), and WBC_ERR_TIMEOUT is returned with
 * the device context intact. `workspace` (at least the control block and barrier flags of
 * wbc_sor_solve_workspace_bytes, 16-byte aligned) is cleared first. Synchronises `stream`. */
int wbc_sor_wait_selftest(int32_t ctas, int32_t missing, int32_t rounds, void* workspace, size_t workspace_bytes,
                          void* stream);
/* Times the resident solver on a copy of `field` (into `scratch_field`, nx*ny*nz floats) for
 * 2 * check_every sweeps under each candidate tuning (one tile per SM; the strip count whose
 * largest tile and bounding box are smallest, and the strip counts one and two either side of it)
 * and returns the fastest in
 * *best (zeros if the grid does not fit on chip) and its time per sweep in *best_us_per_sweep (may
 * be NULL). `field` is not modified; synchronises `stream`. The choice changes speed only: every
 * tuning gives the same field bits. */
int wbc_sor_autotune(const wbc_sor_params* p, int32_t check_every, const int32_t* fixed, const float* density,
                     const float* production, const float* source, const float* field, float* scratch_field,
                     void* workspace, size_t workspace_bytes, wbc_sor_tuning* best, float* best_us_per_sweep,
                     void* stream);
/* ---- batched solves: many grids in one persistent launch -------------------------------------------
 * Each item is one wbc_sor_solve (resident path, halo depth 1) with its own grid, coefficients,
 * field and workspace. The items' tiles form one work list; a CTA takes the next tile and runs it
 * until that item's solve ends, so small and large grids share the GPU in one launch, and each
 * item stops at its own sweep count, residual and stopping rule, with the same field bits as its
 * own wbc_sor_solve. No counterpart in the reference. */
typedef struct wbc_sor_batch_item {
    wbc_sor_params params;
    const int32_t* fixed;         /* may be NULL                                                    */
    const float* density;
    const float* production;      /* may be NULL                                                    */
    const float* source;          /* required when params.has_source                                */
    float* field;
    void* workspace;              /* wbc_sor_solve_workspace_bytes(&params) bytes, 16-byte aligned  */
} wbc_sor_batch_item;

typedef struct wbc_sor_batch {    /* filled by wbc_sor_batch_prepare                                */
    int32_t items, total_tiles, ctas, threads, zclamp, has_prod;
    int64_t smem_bytes;
    void* device_plan;
} wbc_sor_batch;

size_t wbc_sor_batch_plan_bytes(int32_t n);
/* Plans the work list from `weights` (host, one positive value per item: nodes x expected sweeps,
 * e.g. of recent solves; NULL = node counts, i.e. equal sweeps): items ordered by sweep count
 * (weight / nodes), cut into waves that run together by dynamic programming on a modelled
 * duration (per tile and sweep: owned nodes, halo nodes and a fixed cost), each item of a wave
 * given the compact tiling whose tile count makes the wave's items end together; copies the work
 * list into `plan` (device memory) and fills `out`. WBC_ERR_INVALID if a grid fits no tiling in
 * shared memory. Synchronises `stream`; not for use during stream capture. */
int wbc_sor_batch_prepare(int32_t n, const wbc_sor_batch_item* items, const float* weights, int32_t check_every,
                          int32_t max_sweeps, double tolerance, void* plan, size_t plan_bytes, wbc_sor_batch* out,
                          void* stream);
/* The plan wbc_sor_batch_prepare makes, computed on the host alone (no device needed): for `ctas`
 * CTAs with `smem_bytes` of dynamic shared memory each (152 and 231424 on the GB300), the work
 * list's order of the items (`order`, n item indices) and, per position in it, the item's tile
 * count, strip count, wave index (`wave`, may be NULL) and modelled sweep time in ns (`sweep_ns`,
 * may be NULL). For inspection and tests. */
int wbc_sor_batch_plan_host(int32_t n, const wbc_sor_params* params, const float* weights, int32_t ctas,
                            int64_t smem_bytes, int32_t* order, int32_t* tiles, int32_t* strips, int32_t* wave,
                            double* sweep_ns);
/* Solves every item from its field's current values; nothing is read back (capturable). */
int wbc_sor_batch_solve(const wbc_sor_batch* b, void* stream);
/* The items' reports (host array of b->items); synchronises. WBC_ERR_TIMEOUT if a solve timed out. */
int wbc_sor_batch_reports(const wbc_sor_batch* b, wbc_sor_report* reports, void* stream);

/* Explicit FTCS step field_out = field_in + dt (D lap - uptake + production) (validation only;
 * kernels/field_kernels.py:246-273). `p->dx2_over_D` carries D/dx^2 here. */
int wbc_ftcs_step(const wbc_sor_params* p, float dt, const int32_t* fixed, const float* density,
                  const float* production, const float* source, const float* field_in, float* field_out,
                  void* stream);

/* ---- lifecycle ----------------------------------------------------------------------------------- */
typedef struct wbc_lifecycle_params {
    float dt;
    float death_rate;
    float anoxic_death_rate;
    float division_rate;
    int32_t inhibition_threshold;
    float hypoxia_threshold;
    float death_threshold;
    float glucose_threshold;
    float glucose_death_threshold;
    int32_t necrosis_requires_glucose;
    int32_t phenotype_model;      /* 0 = rules, 1 = network                                        */
    float apoptosis_rate;
    float necrosis_rate;
} wbc_lifecycle_params;

/* Death / state / division intent per cell (kernels/cell_kernels.py:77-154, cells/lifecycle.py:96-132). */
int wbc_lifecycle_decide(const wbc_lifecycle_params* p, int32_t n, int32_t* cell_state, float* age,
                         const int32_t* neighbor_count, const float* oxygen_local, const float* glucose_local,
                         const int32_t* fate_flags, uint32_t* rng_state, int32_t* divide_flag, void* stream);
/* Inclusive prefix sum of divide_flag[0, n) into division_offset; total_out[0] (device int32)
 * receives the last value. Replaces warp.utils.array_scan at cells/lifecycle.py:146. */
int wbc_division_scan(int32_t n, const int32_t* divide_flag, int32_t* division_offset, int32_t* total_out,
                      void* workspace, size_t workspace_bytes, void* stream);
/* Allocation-free variant of wbc_division_scan, for callers that cannot allocate device memory
 * (a host framework that owns the whole device memory budget, or a loop that must not incur the
 * device-wide synchronisation cudaMalloc can cause). It takes no workspace: the tile partials live
 * in a 32,772-byte array inside the library, which every GPU that loads the library holds until
 * the process exits. It accepts at most WBC_NOALLOC_SCAN_MAX_CELLS cells and returns
 * WBC_ERR_INVALID (with wbc_last_error explaining) beyond that. The first call on a device looks
 * up that array's device address (once per device, with the device current); make that first
 * call before any stream capture. The cached address belongs to the device's current context:
 * after cudaDeviceReset it is stale, so a process that resets a device must not call this entry
 * point on that device again. Every call shares the array, which keeps the previous call's
 * partials (each call overwrites the entries it reads, so nothing needs clearing): calls that
 * overlap on the GPU, on any stream, race and must be serialised by the caller. Allocates nothing
 * and frees nothing. This entry point has no counterpart in the reference. */
#define WBC_NOALLOC_SCAN_MAX_CELLS 33554432
int wbc_division_scan_noalloc(int32_t n, const int32_t* divide_flag, int32_t* division_offset, int32_t* total_out,
                              void* stream);
/* Daughter of the k-th dividing cell into slot count + k (kernels/cell_kernels.py:157-200). */
int wbc_place_daughters(int32_t count, float placement_factor, const int32_t* divide_flag,
                        const int32_t* division_offset, float* position, float* radius, int32_t* cell_state,
                        int32_t* cell_type, float* age, float* oxygen_local, float* glucose_local,
                        uint32_t* rng_state, float* velocity, int32_t* neighbor_count, int32_t* fate_flags,
                        void* stream);
/* counts[state] += cells in that state (kernels/cell_kernels.py:203-208). counts is int32[4]. */
int wbc_count_states(int32_t n, const int32_t* cell_state, int32_t* counts, void* stream);

/* ---- Boolean networks --------------------------------------------------------------------------- */
typedef struct wbc_network_program {
    int32_t n_nodes;
    int32_t n_words;             /* ceil(n_nodes / 64), at most 4                                   */
    int32_t n_ops;
    int32_t n_updatable;
    const int32_t* ops;          /* postfix opcodes: 0 VAR, 1 NOT, 2 AND, 3 OR, 4 CONST             */
    const int32_t* args;
    const int32_t* start;        /* per node                                                         */
    const int32_t* length;       /* per node                                                         */
    const int32_t* updatable;    /* node ids of the non-input nodes                                  */
    /* Optional truth tables, all three null or all three set. For node i with table_arity[i] = a
     * in [0, 6], its logic value is bit  sum_j state(table_inputs[6 i + j]) << j  of
     * table_bits[i]; table_arity[i] = -1 evaluates node i's program instead. The tables must be
     * the programs' Boolean functions (network/model.py derives them by running each program's
     * postfix semantics over every input pattern), so both routes give the same bits. */
    const int32_t* table_arity;
    const int32_t* table_inputs; /* 6 per node                                                       */
    const uint64_t* table_bits;
} wbc_network_program;

/* Zero the words, then node i ON when randf < p_on[i] (kernels/network_kernels.py:81-95). */
int wbc_network_initialize(const wbc_network_program* prog, int32_t n, const float* p_on, uint32_t* rng_state,
                           uint64_t* states, void* stream);
/* Input clamps from sampled fields or constants (kernels/network_kernels.py:98-132). */
int wbc_network_clamp_inputs(int32_t n, int32_t n_words, int32_t n_clamps, const int32_t* clamp_node,
                             const int32_t* clamp_source, const float* clamp_threshold, const int32_t* clamp_above,
                             const float* oxygen_local, const float* glucose_local, const float* extra_a,
                             const float* extra_b, uint64_t* states, void* stream);
/* `sweeps` synchronous updates (kernels/network_kernels.py:157-175 launched as in
 * network/runtime.py:170-172); the state words stay in registers across sweeps. */
int wbc_network_update_sync(const wbc_network_program* prog, int32_t n, int32_t sweeps, uint64_t* states,
                            void* stream);
/* `n_updates` random single-node updates per cell (kernels/network_kernels.py:135-154). */
int wbc_network_update_async(const wbc_network_program* prog, int32_t n, int32_t n_updates, uint32_t* rng_state,
                             uint64_t* states, void* stream);
/* Gillespie simulation of the MaBoSS chain for `duration` (kernels/network_kernels.py:178-245). */
int wbc_network_update_maboss(const wbc_network_program* prog, int32_t n, float duration, int32_t max_events,
                              const float* rate_up_true, const float* rate_up_false, const float* rate_down_true,
                              const float* rate_down_false, uint32_t* rng_state, uint64_t* states, void* stream);
/* Pack the four fate nodes (-1 = absent) into fate_flags (kernels/network_kernels.py:248-268). */
int wbc_network_read_fates(int32_t n, int32_t n_words, int32_t node_proliferation, int32_t node_apoptosis,
                           int32_t node_growth_arrest, int32_t node_necrosis, const uint64_t* states,
                           int32_t* fate_flags, void* stream);
/* Daughters copy their parent's words (kernels/network_kernels.py:271-284). */
int wbc_network_inherit(int32_t count_before, int32_t n_words, const int32_t* divide_flag,
                        const int32_t* division_offset, uint64_t* states, void* stream);
/* counts[k] += (living) cells with node nodes[k] ON (kernels/network_kernels.py:287-302). */
int wbc_network_count_on(int32_t n, int32_t n_words, int32_t n_query, const int32_t* nodes, int32_t living_only,
                         const int32_t* cell_state, const uint64_t* states, int32_t* counts, void* stream);

/* ---- adjoint of the coupled steady state ------------------------------------------------------------
 * Forward: K contact steps (wbc_contact_substep), a deposit of per-cell uptake capacities, the
 * steady Michaelis-Menten field (wbc_sor_solve with uptake_max = 1 on the deposited capacities).
 * Reverse: the hand-written adjoint below. No counterpart in the reference. */
/* acc[node] += int64(w * weight_i * 2^24 + 0.5) for the trilinear corners of each cell inside the
 * deposit support (the rule of wbc_deposit); one layer, deterministic. */
int wbc_deposit_weighted(const wbc_grid_geometry* geom, int32_t n, const float* position, const float* weight,
                         int64_t* accumulator, void* stream);
/* out[node] = float(acc[node]) / 2^24 * factor; clear != 0 zeroes acc. */
int wbc_weighted_convert(int64_t nodes, int64_t* accumulator, float factor, float* out, int32_t clear,
                         void* stream);
/* One reverse contact step over the grid built at the step's start positions:
 * lambda_out = lambda_in + dt J^T lambda_in, vdot[i] = lambda_in_i . v_i / rate. */
int wbc_adjoint_contact(const wbc_neighbor_grid* grid, int32_t n, float query_radius, float rate, float dt,
                        const float* lambda_in, float* lambda_out, float* vdot, void* stream);
/* Field adjoint (Dirichlet faces): red-black SOR on (6 + h kappa) mu - sum_nb mu = grad_u from mu's
 * current values (start from zeros), kappa = U K / (K + u)^2, until max |residual| is below
 * tolerance x max(6 |mu|, |grad_u|) (checked every check_every sweeps, synchronising); then
 * phi = mu u / (K + u) and sums = {dL/dK, D dL/dD, dL/dO_b} (device doubles). kappa, phi:
 * float[nodes] scratch/outputs; residual_bits: two device uint32. */
int wbc_adjoint_field_solve(const wbc_sor_params* p, const float* u, const float* U, const float* grad_u, float* mu,
                            float* kappa, int32_t check_every, int32_t max_sweeps, float tolerance, float* phi,
                            double* sums, uint32_t* residual_bits, wbc_sor_report* report, void* stream);
/* `steps` contact steps (each wbc_grid_build + wbc_contact_substep, same bits) in one cooperative
 * launch whose phases are separated by bounded grid barriers; `grid` supplies dim, cell_size and
 * the per-cell scratch (cell_bucket, cell_rank, scatter), the workspace
 * (wbc_contact_steps_workspace_bytes(dim, capacity, slots), 256-byte aligned) holds the grids.
 * checkpoints (NULL or float[steps / every + 1][n][3]) receives x_t before step t for t % every
 * == 0. history = 1 builds step t's grid into workspace slot t (steps <= slots) for
 * wbc_adjoint_steps; last_build_only = 1 builds the last step's grid without moving the cells.
 * position_lo (NULL or float[n][3], with checkpoints_lo beside checkpoints) makes the positions
 * compensated, position + position_lo: pair differences include the low parts and the Euler step
 * is an exact two-sum, so the trajectory keeps about 48 bits (forces stay in float).
 * sync_status = 1 synchronises `stream` and returns WBC_ERR_TIMEOUT if a barrier timed out. The
 * adjoint model's forward steps and its checkpoint-segment recomputation; no counterpart in the
 * reference. */
size_t wbc_contact_steps_workspace_bytes(int32_t dim, int64_t capacity, int32_t slots);
int wbc_contact_steps(const wbc_neighbor_grid* grid, int32_t n, float query_radius, float rate, float dt,
                      int32_t steps, float* position, float* position_lo, const float* radius, float* velocity,
                      int32_t* neighbor_count, float* checkpoints, float* checkpoints_lo, int32_t checkpoint_every,
                      int32_t slots, int32_t history, int32_t last_build_only, void* workspace,
                      size_t workspace_bytes, int32_t sync_status, void* stream);
/* The reverse of `steps` contact steps whose grids wbc_contact_steps left in history slots
 * 0 .. steps - 1 of `workspace`, in one cooperative launch: lambda (dL/dx after the steps on
 * entry, dL/dx before them on return; lambda_tmp is scratch of the same size) goes through
 * lambda_t = lambda_{t+1} + dt J(x_t)^T lambda_{t+1}, and rate_dot[0] (device double, not cleared)
 * accumulates sum_t sum_i lambda_{t+1,i} . v_i(x_t) / rate. compensated = 1 when the grids were
 * built from compensated positions. */
int wbc_adjoint_steps(const wbc_neighbor_grid* grid, int32_t n, float query_radius, float rate, float dt,
                      int32_t steps, int32_t compensated, float* lambda, float* lambda_tmp, double* rate_dot,
                      int32_t slots, void* workspace, size_t workspace_bytes, int32_t sync_status, void* stream);
/* Mixed-precision refinement (the fp32 solves stop near a relative residual of 1e-6): the Newton
 * step of the steady field at u (FP64): diag = 6 + h U K / (K + u)^2 and rhs = sum_nb u -
 * (6 + h U / (K + u)) u in FP64 (diag = -1 at faces and at nodes held at the zero clamp), to be
 * solved by wbc_sor_linear_solve and added by wbc_adjoint_newton_apply (u += d, clamped at 0). */
int wbc_adjoint_newton_prepare(const wbc_sor_params* p, const double* u, const float* U, float* diag, float* rhs,
                               void* stream);
int wbc_adjoint_newton_apply(int64_t nodes, const float* delta, double* u, void* stream);
/* out[i] = (double) in[i]. */
int wbc_widen(int64_t n, const float* in, double* out, void* stream);
/* Small device helpers of the adjoint's host code, so that its passes launch only this library's
 * kernels: out[i] = (float) in[i]; out[i] = value; `bytes` zero bytes at ptr (a memset);
 * out[i] = in[i] / divisor; x64[i] = (double) hi[i] + lo[i] with pos[i] = (float) x64[i]; and
 * scratch[0] = the mean of x[0 .. n) in FP64 by a fixed-order reduction (0 for n = 0), scratch
 * holding WBC_MEAN_SCRATCH doubles. */
#define WBC_MEAN_SCRATCH 257
int wbc_narrow(int64_t n, const double* in, float* out, void* stream);
int wbc_fill(int64_t n, float value, float* out, void* stream);
int wbc_zero(void* ptr, size_t bytes, void* stream);
int wbc_divide(int64_t n, const float* in, float divisor, float* out, void* stream);
int wbc_compensated_sum(int64_t n, const float* hi, const float* lo, double* x64, float* pos, void* stream);
int wbc_mean(int64_t n, const float* x, double* scratch, void* stream);
/* r = b - (diag x - sum_nb x) in FP64 where diag > 0, 0 elsewhere (the adjoint's refinement step). */
int wbc_adjoint_linear_residual(const wbc_sor_params* p, const float* diag, const float* b, const float* x, float* r,
                                void* stream);
/* The field's gradient sums from the refined field u (FP64) and adjoint mu0 + dmu: sums = {dL/dK,
 * D dL/dD, dL/dO_b} (cleared first) and phi = mu u / (K + u) for wbc_adjoint_cells. */
int wbc_adjoint_field_grads(const wbc_sor_params* p, const double* u, const float* U, const float* mu0,
                            const float* dmu, const float* diag, const float* grad_u, float* phi, double* sums,
                            void* stream);
/* Per cell: grad_vmax = coef sum_a w_a phi_a, grad_x += coef vmax grad_x(sum_a w_a phi_a). */
int wbc_adjoint_cells(const wbc_grid_geometry* geom, int32_t n, const float* position, const float* vmax,
                      const float* phi, float coef, float* grad_vmax, float* grad_x, void* stream);

/* ---- batches: many independent spheroids advanced together ------------------------------------
 * One instance = one population with its hash grid and oxygen grid, described by device pointers
 * into arrays the caller owns (the same arrays the single-population calls take). Every batched
 * call launches one kernel per stage for all instances over a static work list and reads each
 * instance's cell count from counts[instance] in device memory; no call reads anything back to
 * the host, so a whole step can be captured in a CUDA graph. Each instance's results are
 * bit-identical to the single-population calls on it. No counterpart in the reference, whose
 * parameter sweep runs its experiments one after another (simulation/sweep.py:132-139). */
typedef struct wbc_batch_instance {
    int32_t capacity;
    float* position;              /* float[capacity][3]                                             */
    float* radius;
    int32_t* cell_state;
    int32_t* cell_type;
    float* age;
    float* oxygen_local;
    float* glucose_local;
    uint32_t* rng_state;
    float* velocity;              /* float[capacity][3]                                             */
    int32_t* neighbor_count;
    int32_t* divide_flag;
    int32_t* division_offset;
    int32_t* fate_flags;
    wbc_neighbor_grid grid;       /* this instance's hash grid (scan_partials unused)               */
    float query_radius;           /* contact: ContactParams.query_radius                            */
    float contact_rate;           /* stiffness / damping                                            */
    float contact_dt;             /* dt_mechanics                                                    */
    int32_t contact_substeps;
    wbc_grid_geometry geom;       /* the oxygen grid                                                 */
    void* accumulator;            /* the 32-bit accumulator of wbc_deposit32 (wbc_deposit32_bytes(   */
                                  /* nodes) bytes, 16-byte aligned), cleared by each batched deposit  */
    float* density;               /* unused: per-state densities are converted from the accumulator  */
                                  /* by wbc_convert32 when they are wanted                           */
    float* uptake_density;        /* the solver's combined uptake density, float[nodes]              */
    float uptake_weights[4];
    float inv_voxel_volume;
    float* field;                 /* oxygen values sampled into oxygen_local                         */
    wbc_lifecycle_params lifecycle;
    float placement_factor;
} wbc_batch_instance;

typedef struct wbc_batch {        /* filled by wbc_batch_prepare                                     */
    int32_t instances;
    void* device_plan;
    int32_t cell_chunks, node_chunks, bucket_tiles, slot_tiles;
    int32_t max_substeps;
} wbc_batch;

/* Device bytes of the plan for these instances (0 if the description is too large). */
size_t wbc_batch_plan_bytes(int32_t n, const wbc_batch_instance* insts);
/* Copies the descriptions and the work lists into `plan` (device memory) and fills `out`.
 * Synchronises `stream`; not for use during stream capture. */
int wbc_batch_prepare(int32_t n, const wbc_batch_instance* insts, void* plan, size_t plan_bytes, wbc_batch* out,
                      void* stream);
/* wbc_grid_build for every instance. */
int wbc_batch_grid_build(const wbc_batch* b, const int32_t* counts, void* stream);
/* wbc_contact_substep for every instance (one substep). */
int wbc_batch_contact(const wbc_batch* b, const int32_t* counts, void* stream);
/* wbc_deposit32 (cells in slot order) then wbc_convert32 of the combined uptake density only, for
 * every instance. */
int wbc_batch_deposit(const wbc_batch* b, const int32_t* counts, void* stream);
/* wbc_sample of `field` into oxygen_local for every instance. */
int wbc_batch_sample(const wbc_batch* b, const int32_t* counts, void* stream);
/* wbc_lifecycle_decide, wbc_division_scan and wbc_place_daughters for every instance, then
 * counts[i] += daughters. An instance whose daughters would exceed its capacity places none,
 * keeps its count and gets status[i] = WBC_ERR_CAPACITY (status may be NULL). */
int wbc_batch_lifecycle(const wbc_batch* b, int32_t* counts, int32_t* status, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* WBC_H */
