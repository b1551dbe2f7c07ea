/* Tay public C API, GB300 edition (libtay_gb300.so).
 *
 * Source-compatible with the reference's public header (tay/tay.h:1-119): same types,
 * same enum values, same function names, arguments and 0/NULL-on-failure convention, so
 * a host written against the reference compiles against this header unchanged.
 * Additions, all marked NEW below:
 *   - TAY_GPU_Z_GRID: a space type whose groups run on the GPU Z-grid engine;
 *   - TAY_ERROR_CUDA and TAY_ERROR_DEVICE_MODEL;
 *   - tay_run_batch: many states advanced together, one launch per kernel per step;
 *   - tay_run_backward and friends: the adjoint of an SPH rollout (tay_adjoint.h).
 *
 * This library implements the GPU Z-grid path only.  Groups configured with a CPU
 * structure (TAY_CPU_SIMPLE ... TAY_CPU_Z_GRID) make tay_run fail with
 * TAY_ERROR_NOT_IMPLEMENTED; the reference library remains the implementation of those.
 * On the GPU path the see/act function pointers are not called: func_name selects the
 * device function, as it selects the generated kernel in the reference's OpenCL path
 * (tay/ocl.c:284-291).
 */
#ifndef tay_h
#define tay_h

#define float4_agent_position(__agent_tag__) (*(float4 *)((TayAgentTag *)(__agent_tag__) + 1))
#define float3_agent_position(__agent_tag__) (*(float3 *)((TayAgentTag *)(__agent_tag__) + 1))
#define float2_agent_position(__agent_tag__) (*(float2 *)((TayAgentTag *)(__agent_tag__) + 1))

#define float4_agent_min(__agent_tag__) (*(float4 *)((TayAgentTag *)(__agent_tag__) + 1))
#define float3_agent_min(__agent_tag__) (*(float3 *)((TayAgentTag *)(__agent_tag__) + 1))
#define float2_agent_min(__agent_tag__) (*(float2 *)((TayAgentTag *)(__agent_tag__) + 1))
#define float4_agent_max(__agent_tag__) (*(float4 *)((char *)(__agent_tag__) + sizeof(TayAgentTag) + sizeof(float4)))
#define float3_agent_max(__agent_tag__) (*(float3 *)((char *)(__agent_tag__) + sizeof(TayAgentTag) + sizeof(float4)))
#define float2_agent_max(__agent_tag__) (*(float2 *)((char *)(__agent_tag__) + sizeof(TayAgentTag) + sizeof(float4)))

#ifdef __cplusplus
extern "C" {
#endif

typedef enum TayBool {
    TAY_FALSE,
    TAY_TRUE,
} TayBool;

/* Same values as tay/tay.h:21-29 for the CPU types; TAY_GPU_Z_GRID is NEW. */
typedef enum TaySpaceType {
    TAY_SPACE_NONE,
    TAY_CPU_SIMPLE,
    TAY_CPU_KD_TREE,
    TAY_CPU_AABB_TREE,
    TAY_CPU_GRID,
    TAY_CPU_Z_GRID,
    TAY_GPU_Z_GRID,
    TAY_SPACE_COUNT,
} TaySpaceType;

/* Same values as tay/tay.h:31-39; the last three are NEW. */
typedef enum TayError {
    TAY_ERROR_NONE = 0,
    TAY_ERROR_POINT_NONPOINT_MISMATCH,
    TAY_ERROR_SPACE_INDEX_OUT_OF_RANGE,
    TAY_ERROR_GROUP_INDEX_OUT_OF_RANGE,
    TAY_ERROR_STATE_STATUS,
    TAY_ERROR_NOT_IMPLEMENTED,
    TAY_ERROR_OCL,
    TAY_ERROR_CUDA,          /* a CUDA call or a kernel failed */
    TAY_ERROR_DEVICE_MODEL,  /* func_name / pass sequence not provided by a device model */
    TAY_ERROR_BATCH,         /* states passed to tay_run_batch cannot run together */
} TayError;

#pragma pack(push, 1)

typedef struct float3 {
    union {
        struct {
            float x, y, z;
        };
        float arr[3];
    };
} float3;

typedef struct float4 {
    union {
        struct {
            float x, y, z, w;
        };
        float3 xyz;
        float arr[4];
    };
} float4;

typedef struct float2 {
    union {
        struct {
            float x, y;
        };
        float arr[2];
    };
} float2;

typedef struct {
    float4 min;
    float4 max;
} Box;

typedef struct TayAgentTag {
    unsigned part_i;
    unsigned cell_agent_i;
} TayAgentTag;

#pragma pack(pop)

typedef struct TayState TayState;
typedef struct TayGroup TayGroup;
typedef struct TayPass TayPass;

TayState *tay_create_state(void); /* tay/tay.h:87, tay/state.c:11 */
void tay_destroy_state(TayState *state); /* tay/tay.h:88, tay/state.c:35 */
int tay_switch_to_ocl(TayState *state); /* tay/tay.h:89, tay/state.c:42 */
int tay_switch_to_host(TayState *state); /* tay/tay.h:90, tay/state.c:50 */

TayError tay_get_error(TayState *state); /* tay/tay.h:92, tay/state.c:59 */

TayGroup *tay_add_group(TayState *state, unsigned agent_size, unsigned agent_capacity, int is_point); /* tay/tay.h:94, tay/state.c:73 */
void tay_configure_space(TayState *state, TayGroup *group, TaySpaceType space_type, int space_dims, float4 min_part_sizes, int shared_size_in_megabytes); /* tay/tay.h:95, tay/state.c:109 */
void tay_fix_space_box(TayState *state, TayGroup *group, float4 min, float4 max); /* tay/tay.h:96, tay/state.c:120 */

void tay_add_see(TayState *state, TayGroup *seer_group, TayGroup *seen_group, void (*func)(void *, void *, void *), char *func_name, float4 radii, int self_see, void *context, unsigned context_size); /* tay/tay.h:98, tay/state.c:135 */
void tay_add_act(TayState *state, TayGroup *act_group, void (*func)(void *, void *), char *func_name, void *context, unsigned context_size); /* tay/tay.h:99, tay/state.c:149 */

void tay_clear_all_agents(TayState *state, TayGroup *group); /* tay/tay.h:101, tay/state.c:160 */
void *tay_get_available_agent(TayState *state, TayGroup *group); /* tay/tay.h:102, tay/state.c:166 */
void tay_commit_available_agent(TayState *state, TayGroup *group); /* tay/tay.h:103, tay/state.c:172 */
void *tay_get_agent(TayState *state, TayGroup *group, int index); /* tay/tay.h:104, tay/state.c:178 */

void tay_simulation_start(TayState *state); /* tay/tay.h:106, tay/state.c:183 */
int tay_run(TayState *state, int steps); /* tay/tay.h:107, tay/state.c:194-323 */
void tay_simulation_end(TayState *state); /* tay/tay.h:108, tay/state.c:325 */

double tay_get_ms_per_step_for_last_run(TayState *state); /* tay/tay.h:110, tay/state.c:336 */
void tay_log(void *file, char *fmt, ...); /* tay/tay.h:111, tay/thread.c:206 */

void ocl_add_source(TayState *state, const char *source); /* tay/tay.h:113, tay/ocl.c:274 */

void tay_threads_start(unsigned threads_count, unsigned thread_storage_size); /* tay/tay.h:115, tay/thread.c:70 */
void tay_threads_stop(void); /* tay/tay.h:116, tay/thread.c:116 */
unsigned tay_get_number_of_threads(void); /* tay/tay.h:117, tay/thread.c:120 */

/* NEW: advances `count` states by `steps` steps together: every state must hold one
 * TAY_GPU_Z_GRID group running the same device model and pass sequence (agent counts,
 * radii, contexts and space sizes may differ).  Each state's group becomes one segment
 * of one device batch.  Returns steps run, or 0 with the error set on every state. */
int tay_run_batch(TayState **states, int count, int steps);

/* NEW: number of pairs that passed the box test during the last tay_run /
 * tay_run_batch of this state (the reference's narrow-phase counter,
 * tay/space.c:56-60), and the device time of its steps in ms. */
unsigned long long tay_get_pairs_for_last_run(TayState *state);
double tay_get_device_ms_for_last_run(TayState *state);

/* NEW: commits `count` agents at once, copied from `records` (count * agent_size
 * bytes); equivalent to `count` rounds of tay_get_available_agent + copy +
 * tay_commit_available_agent.  Returns the number committed (fewer when the group
 * fills up). */
unsigned tay_commit_agents(TayState *state, TayGroup *group, const void *records, unsigned count);

/* NEW: number of committed agents of a group. */
unsigned tay_get_agent_count(TayState *state, TayGroup *group);

/* NEW: agents stay on the device between tay_run calls; tay_get_agent fetches a group's
 * records (in cell order) only when the device holds newer ones, and tay_run pushes a
 * group only when its host records changed through tay_commit_available_agent,
 * tay_commit_agents, tay_clear_all_agents or tay_configure_space.  A host that writes
 * records through the pointer tay_get_agent returns calls this so that the next
 * tay_run pushes them. */
void tay_mark_agents_changed(TayState *state, TayGroup *group);

/* NEW: differentiable SPH rollouts (a hand-written adjoint; no
 * counterpart in the reference).  tay_run_recorded advances `count` states (each one
 * TAY_GPU_Z_GRID group running sph_density, sph_pressure, sph_force, sph_integrate) by
 * `steps` steps like tay_run_batch, recording what the adjoint needs: with
 * checkpoint_every = k > 0 the state of every k-th step (segments are recomputed during
 * the backward sweep), with 0 every step.  tay_run_backward then takes dL/d(final
 * positions) and dL/d(final velocities) and returns dL/d(initial positions), dL/d(initial
 * velocities) and dL/d(alpha, c0) of each state's SPH context.  Per-agent arrays hold 4
 * floats per agent, the agents of state s at rows offset(s) + id (offset(s) = the agent
 * counts of the states before s, id = the agent's id field); dloss_dparams holds 2
 * doubles per state.  Neighbour sets are held fixed within each step.  Returns 1 on
 * success, 0 with the error set. */
int tay_run_recorded(TayState **states, int count, int steps, int checkpoint_every);
int tay_run_backward(TayState **states, int count, const float *dloss_dp, const float *dloss_dv, float *dloss_dp0,
                     float *dloss_dv0, double *dloss_dparams);
/* NEW: device ms of the last recorded forward and of the last backward sweep, and the
 * device memory they held (bytes). */
double tay_get_recorded_forward_ms(void);
double tay_get_backward_ms(void);
unsigned long long tay_get_adjoint_device_bytes(void);

/* NEW: last error message (CUDA or device model) of this state. */
const char *tay_get_error_message(TayState *state);

#ifdef __cplusplus
}
#endif

#endif
