/* C ABI of the GB300 Z-grid engine (libtay_gb300.so).
 *
 * This is the layer that replaces the reference's OpenCL device layer for Z-grid
 * groups: program text generation and compilation (tay/ocl.c:100-177), buffer creation,
 * push and fetch (tay/ocl.c:59-98, 238-272), the grid sort launcher
 * (tay/ocl_grid.c:241-374) and the per-pass see/act launches (tay/ocl.c:208-236), plus
 * the CPU thread pool those passes ran on for CPU structures (tay/thread.c).  The
 * reference-compatible API in tay.h is implemented on top of it; hosts may also call it
 * directly (plain pointers and sizes, no C++ or torch types).
 *
 * A "batch" holds one or more groups that share a model and a pass sequence.  Each
 * group becomes one segment of concatenated device buffers; tgpu_batch_run advances all
 * of them with one launch per kernel per step.  Every function returns TGPU_OK or an
 * error code; tgpu_last_error() describes the last failure of the calling thread.
 */
#ifndef TAY_GPU_H
#define TAY_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct TgpuBatch TgpuBatch;

enum {
    TGPU_OK = 0,
    TGPU_ERR_ARG = 1,          /* bad argument, or groups that cannot share a batch */
    TGPU_ERR_UNKNOWN_FUNC = 2, /* a func_name no registered device model provides */
    TGPU_ERR_PROGRAM = 3,      /* pass sequence the model does not support */
    TGPU_ERR_CUDA = 4,         /* a CUDA call failed (message has the CUDA error) */
    TGPU_ERR_DEVICE = 5        /* a kernel reported an error through the device error word */
};

/* One registered pass, as stored by tay_add_see / tay_add_act
 * (tay/state.c:135-158): func_name selects the device function. */
typedef struct TgpuPass {
    const char *func_name;
    int is_see;
    float radii[4];
    int self_see;
    const void *context;      /* borrowed; copied at create and by tgpu_batch_set_contexts */
    unsigned context_size;
} TgpuPass;

/* One group (tay_add_group + tay_configure_space + tay_fix_space_box,
 * tay/state.c:73-125). */
typedef struct TgpuGroup {
    unsigned agent_size;      /* bytes per AoS record */
    unsigned count;           /* agents */
    float min_part_sizes[4];  /* minimum cell edge per axis */
    int shared_megabytes;     /* memory for the structure (bounds the dense cell table) */
    int box_fixed;
    float box_min[4];
    float box_max[4];
    int pass_count;
    const TgpuPass *passes;
    int dims;                 /* tay_configure_space dims: 1, 2 or 3 (0 means 3); the box test
                                 and the grid use the first `dims` axes (min over seer and
                                 seen group for a two-group pass), tay/space.c:62-68 */
} TgpuGroup;

/* Creates a batch of `group_count` groups; all must resolve to the same model and the
 * same pass sequence. */
int tgpu_batch_create(const TgpuGroup *groups, int group_count, TgpuBatch **out);
void tgpu_batch_destroy(TgpuBatch *batch);

/* One pass of a state whose groups are mixed by its passes (tay_add_see with
 * seer_group != seen_group, several see passes per group; tay/state_compile.c:109-120,
 * test/test_combo.c:114-119).  seer_group is the acting group of an act pass;
 * seen_group is used by see passes only.  Both index the `groups` array. */
typedef struct TgpuStatePass {
    TgpuPass pass;
    int seer_group;
    int seen_group;
} TgpuStatePass;

/* Creates a batch for one state of `group_count` groups of one device model, stepped by
 * the state-level pass list `passes` (registration order; groups[k].passes is not used).
 * Every pass runs as its own kernel over its seer (or acting) group, a see pass reading
 * the seen group's cell table and streams; seer == seen is skipped only inside one group
 * without self_see.  A group may have several see passes when the model's see function
 * accumulates onto the seer's stored fields (the test model); otherwise one.  Push,
 * fetch and run work per group as for tgpu_batch_create. */
int tgpu_state_create(const TgpuGroup *groups, int group_count, const TgpuStatePass *passes, int pass_count,
                      TgpuBatch **out);

/* Copies the contexts and radii of a state's passes again (same order as at create). */
int tgpu_state_set_contexts(TgpuBatch *batch, const TgpuStatePass *passes, int pass_count);

/* Failure-path self-test of the radix sort's bounded waits: runs one tile of a radix pass
 * whose predecessor never publishes its counts, so its look-back waits run out (each in
 * well under a second) and the kernel returns after recording the failure.  Stores the
 * device error word it read back (2 = look-back wait ran out) and returns TGPU_OK, or
 * TGPU_ERR_CUDA.  The context stays usable. */
int tgpu_selftest_sort_wait(unsigned *device_error);

/* 1 when the device model providing `func_name` holds non-point (box) agents, 0 when it
 * holds point agents, -1 when no model provides it. */
int tgpu_model_nonpoint(const char *func_name);

/* Copies the pass contexts of group `group` again (contexts are borrowed by the host
 * API and re-read at every tay_run, as tay/ocl.c:252-259 does). */
int tgpu_batch_set_contexts(TgpuBatch *batch, int group, const TgpuGroup *desc);

/* Uploads `count` AoS records (as given at create) of group `group`. */
int tgpu_batch_push(TgpuBatch *batch, int group, const void *host_records);

/* Runs `steps` steps (sort, passes, table clear) and waits for them. */
int tgpu_batch_run(TgpuBatch *batch, int steps);

/* Same as tgpu_batch_run but only enqueues; tgpu_batch_sync waits. */
int tgpu_batch_enqueue(TgpuBatch *batch, int steps);
int tgpu_batch_sync(TgpuBatch *batch);

/* Downloads the records of group `group` in the current (cell) order, as
 * tay_get_agent exposes them (tay/state.c:178-181). */
int tgpu_batch_fetch(TgpuBatch *batch, int group, void *host_records);

/* Write-through fetch of group `group` into page-locked `host_records` (from
 * tgpu_host_alloc or cudaHostAlloc; NULL turns it off; pageable memory is refused with
 * TGPU_ERR_ARG): the last step of every following run writes the group's records there
 * from its final see pass, each CTA storing its seers' records as it ends, so the host
 * link overlaps the rest of the pass (after the step when the last pass is an act or
 * covers one group of a state); a tgpu_batch_fetch into the same buffer after such a run
 * only waits.  Replaces the fetch after every run of the reference's OpenCL path
 * (tay/ocl.c:261-272) for hosts that read their agents after each run. */
int tgpu_batch_write_through(TgpuBatch *batch, int group, void *host_records);

/* Device time in ms of the last tgpu_batch_run / enqueue+sync, from CUDA events on the
 * batch's stream, and the number of pairs that passed the box test in it. */
double tgpu_batch_last_device_ms(const TgpuBatch *batch);
unsigned long long tgpu_batch_last_pairs(const TgpuBatch *batch);

/* Profiled run: enqueues `steps` steps without graphs, with CUDA events on the batch's
 * stream around each kernel class, waits, and adds the device ms of each class to
 * ms[0..n): 0 bounding box, 1 keys + radix sort, 2 cell table write + clear, 3 reorder,
 * 4.. the model's pass kernels in program order. Returns TGPU_OK or an error. */
int tgpu_batch_profile(TgpuBatch *batch, int steps, double *ms, int n);

/* Telemetry of the last run, summed over its steps and see passes (the GPU counterpart
 * of the reference's TAY_TELEMETRY counters, tay/space.c:50-60, tay/thread.c:137-242):
 * out[0] candidates box-tested (broad phase; out[0] vs pairs gives the neighbour-finding
 * efficiency), out[1] see CTAs that staged their halo in shared memory, out[2] see CTAs
 * that read it from global memory, out[3] warps that walked their union box, out[4]
 * warps whose lanes walked their own boxes, out[5] warps that replayed a pair list
 * (pair_list_cap) instead of walking. */
int tgpu_batch_telemetry(const TgpuBatch *batch, unsigned long long *out, int n);

/* Number of kernel classes tgpu_batch_profile reports (4 + pass kernels). */
int tgpu_batch_kernel_classes(const TgpuBatch *batch);

/* Evicts the L2 cache by writing a scratch buffer larger than it on the batch's stream
 * (for timing without warm-cache carry-over between steps). */
int tgpu_batch_flush_l2(TgpuBatch *batch);

/* Page-locked host memory for AoS storage (faster push/fetch); falls back to ordinary
 * zeroed memory when no CUDA device is usable.  Free with tgpu_host_free. */
void *tgpu_host_alloc(unsigned long long bytes);
void tgpu_host_free(void *ptr);

/* Number of kernel launches one step enqueues. */
int tgpu_batch_launches_per_step(const TgpuBatch *batch);

/* Name of the model the batch runs ("test_basic", "boids", "sph"), and the index of the
 * pass sequence within the model. */
const char *tgpu_batch_model(const TgpuBatch *batch);
int tgpu_batch_program(const TgpuBatch *batch);

/* Tuning of the see kernel and the grid; applies to batches created afterwards.
 *   stage          1: each see CTA stages its halo cells in shared memory; 0: candidates
 *                  are read through the L1 cache (more CTAs per SM)
 *   stage_cap      agents staged per CTA (0 = default)
 *   stage_cells    halo cells per CTA (0 = default)
 *   cell_multiple  grid cell edge = cell_multiple x min_part_sizes (0 = 1)
 *   union_factor   a warp walks the union of its seers' cell boxes (one read serves all
 *                  32 lanes) when that union is at most union_factor times the largest
 *                  single box; otherwise each lane walks its own box.  1 (the default; 0
 *                  means 1): each lane always walks its own box (cell order 1 then runs a
 *                  kernel without the warp walks, which holds fewer registers)
 *   use_graphs     capture each step in a CUDA graph and replay it
 *   cell_order     0: cells in 3-D Morton order, a {first, end} table entry per cell;
 *                  1: x-rows (x fastest inside (y, z) rows, rows in 2-D Morton order),
 *                  a seer's box is one candidate range per row (no staging)
 *   hit_masks      cell order 1: each lane box-tests up to 32 candidates into a mask
 *                  before the lanes run the see function over their hits together
 *   x_cell_factor  cell order 1: x cells are this fraction of the y / z cells (finer x
 *                  cells tighten each row's candidate range without adding rows)
 *   pair_list_cap  cell order 1, no staging or hit masks: entries per agent of the pair
 *                  list a see pass records for the next see pass over the same positions
 *                  when the model pairs them (SPH density -> force), rounded up to a
 *                  multiple of 4; agents with more pairs are walked again.  0: no pair
 *                  lists */
typedef struct TgpuTuning {
    int stage;
    unsigned stage_cap;
    unsigned stage_cells;
    float cell_multiple;
    unsigned union_factor;
    int use_graphs;
    unsigned cell_order;
    unsigned hit_masks;
    float x_cell_factor;
    unsigned pair_list_cap;
} TgpuTuning;

void tgpu_set_tuning(const TgpuTuning *tuning);  /* NULL restores the defaults */
void tgpu_get_tuning(TgpuTuning *tuning);

/* Adjoint of SPH rollouts (a hand-written reverse mode; no counterpart in the
 * reference).  For a batch running the full SPH sequence (sph_density, sph_pressure,
 * sph_force, sph_integrate):
 *   tgpu_adjoint_create   prepares a rollout of `steps` steps; checkpoint_every = k > 0
 *                         keeps the state of every k-th step and recomputes each k-step
 *                         segment during the backward sweep, except the last
 *                         keep_segments segments (>= 1), which the forward run records
 *                         (k steps of records each); 0 records every step in the forward
 *                         run (no recomputation, more memory);
 *   tgpu_adjoint_forward  runs the rollout from the batch's current state;
 *   tgpu_adjoint_backward given dL/d(final positions) and dL/d(final velocities) (host,
 *                         float4 per agent, agents of group g at rows begin(g) + id, id =
 *                         the record's id field), returns dL/d(initial positions),
 *                         dL/d(initial velocities) in the same layout and dL/d(alpha, c0)
 *                         per group (2 doubles per group).  Neighbour sets are held fixed
 *                         within each step.  Any output pointer may be NULL.  When it
 *                         recomputed a segment, the recomputation was recorded over the
 *                         forward run's records, and the next backward needs another
 *                         tgpu_adjoint_forward (it returns TGPU_ERR_ARG until then); with
 *                         every step recorded, or every segment kept, it may run again. */
typedef struct TgpuAdjoint TgpuAdjoint;
int tgpu_adjoint_create(TgpuBatch *batch, int steps, int checkpoint_every, int keep_segments, TgpuAdjoint **out);
int tgpu_adjoint_forward(TgpuAdjoint *adjoint);
int tgpu_adjoint_backward(TgpuAdjoint *adjoint, const float *dl_dpos, const float *dl_dvel, float *dpos0,
                          float *dvel0, double *dparams);
double tgpu_adjoint_forward_ms(const TgpuAdjoint *adjoint);
double tgpu_adjoint_backward_ms(const TgpuAdjoint *adjoint);
unsigned long long tgpu_adjoint_device_bytes(const TgpuAdjoint *adjoint);
void tgpu_adjoint_destroy(TgpuAdjoint *adjoint);

/* Device memory in bytes held by a batch (streams, tables, sort buffers). */
unsigned long long tgpu_batch_device_bytes(const TgpuBatch *batch);

/* Allocation-free neighbour pass.  No counterpart in the reference: it exists for callers
 * that cannot call cudaMalloc when they need the pass - hosts whose memory manager owns
 * the whole device heap (a framework's caching allocator, a fixed per-process budget),
 * plugins that may not allocate after initialisation, and latency-sensitive loops that
 * cannot afford cudaMalloc's implicit synchronisation.
 *
 * Runs the test model's see pass ("agent_see": per agent, the sum of b.p - a.p over the
 * other agents inside the per-axis radii, and their count) on `n` float4 positions that
 * are already in device memory, and writes one float4 per agent to the device buffer
 * `out`, in the input order: x, y, z = the sum, w = the count as int bits.  radii and
 * min_part_sizes are 4 host floats each.  All intermediate buffers live in one fixed
 * array (about 5 MB) of the library's own device memory, which every GPU that loads the
 * library holds until the process exits; no device memory is allocated.
 *   - n must not exceed tgpu_noalloc_max_agents() (65536); larger calls fail with
 *     TGPU_ERR_ARG and a message from tgpu_noalloc_last_error();
 *   - the array is shared by every call and keeps the last call's contents (each call
 *     clears what must start at zero); calls whose work overlaps on the GPU race;
 *   - every call looks up the array's device address in the current device's context
 *     (a host-side query), so it stays valid after that context is recreated;
 *   - work is enqueued on `stream` (a cudaStream_t, NULL for the default stream) and the
 *     call returns once it has finished: it synchronises and reads back a status word,
 *     so it may not be called while any stream is capturing;
 *   - a CUDA error pending from earlier work is left in place for its owner and the call
 *     returns TGPU_ERR_CUDA without starting. */
int tgpu_see_noalloc(const float *positions, unsigned n, const float *radii, const float *min_part_sizes,
                     float *out, void *stream);
unsigned tgpu_noalloc_max_agents(void);
const char *tgpu_noalloc_last_error(void);

/* Device models a host brings itself (the counterpart of the reference's ocl_add_source,
 * tay/ocl.c:274-282, and of its func_name-keyed kernels, tay/ocl.c:284-291 and
 * tay/ocl_grid.c:376-417).  A model is CUDA code compiled by the host against
 * include/tay_gpu_model.cuh: __device__ see / act policies, the record codec, the stream
 * layout and the supported pass programs, gathered in one descriptor.  After
 * registration its func names work in tay_add_see / tay_add_act on TAY_GPU_Z_GRID groups
 * like the library's own models.
 *   tgpu_register_model          registers a descriptor (a tgpu::ModelDesc) that stays
 *                                valid for the life of the process; `abi` is
 *                                TGPU_MODEL_ABI as the model was compiled.  Refused with
 *                                TGPU_ERR_ARG (and a message) when the ABI differs, a field
 *                                is missing or out of range, or a func name is already
 *                                provided by another model.
 *   tgpu_register_model_library  loads a shared library built from such a model (kept
 *                                loaded) and registers the descriptor its exported
 *                                `const void *tgpu_model_entry(unsigned *abi)` returns.
 * Registration is process-wide and may happen before or between runs. */
int tgpu_register_model(const void *desc, unsigned abi);
int tgpu_register_model_library(const char *path);

/* Resolves a func_name to its model; returns the model name or NULL. */
const char *tgpu_model_of(const char *func_name);

/* Number of CUDA devices visible to the process (0 when none or no driver). */
int tgpu_device_count(void);

const char *tgpu_last_error(void);

#ifdef __cplusplus
}
#endif

#endif
