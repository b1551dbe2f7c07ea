/* Host side of the Tay C API for the GB300 Z-grid path.
 *
 * Keeps the reference's state model (tay/state.c, tay/state.h:217-271): a state owns up
 * to TAY_MAX_GROUPS groups with host AoS storage and up to TAY_MAX_PASSES passes in
 * registration order; errors are sticky and functions return 0/NULL on failure.
 * tay_run compiles the state on first use (tay/state_compile.c:5-175) and runs the steps
 * on the device.  The agents stay on the device between runs: a group's host records are
 * pushed only when they changed (commit, clear, configure, tay_mark_agents_changed; the
 * reference's OpenCL path pushes on configure/clear, tay/ocl.c:238-250) and fetched back
 * in cell order only when the host reads them (tay_get_agent, tay_simulation_end), where
 * the OpenCL path fetches after every run (tay/ocl.c:261-272).  States with several
 * groups, mixed by their see passes, run as one state batch (tgpu_state_create).
 * The device work is delegated to the C ABI in tay_gpu.h.
 */
#include "tay.h"
#include "tay_gpu.h"

#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#define TAY_MAX_GROUPS 8
#define TAY_MAX_PASSES 32
#define TAY_MAX_FUNC_NAME 512
#define TAY_MB (1 << 20)

struct TayGroup {
    char *storage;
    unsigned agent_size;
    unsigned capacity;
    unsigned count;
    int is_point;
    TaySpaceType type;
    int dims;
    float4 part;
    int shared_mb;
    int box_fixed;
    float4 box_min, box_max;
    unsigned id;
    int host_dirty; /* host records changed since the last push */
    int host_stale; /* the device holds newer records than the host */
    int slot;       /* segment of the compiled batch, or -1 */
    int read_since_run; /* tay_get_agent was called since the last run */
    int write_through;  /* the batch writes this group's records to storage at each run's end */
};

struct TayPass {
    int is_see;
    TayGroup *seer_group; /* act group for act passes */
    TayGroup *seen_group;
    char func_name[TAY_MAX_FUNC_NAME];
    float4 radii;
    int self_see;
    void *context;
    unsigned context_size;
};

struct TayState {
    TayGroup groups[TAY_MAX_GROUPS];
    TayPass passes[TAY_MAX_PASSES];
    unsigned passes_count;
    int is_running;
    int recompile;
    TayError error;
    char message[512];
    double ms_per_step;
    double device_ms;
    unsigned long long pairs;
    unsigned next_group_id;
    /* compiled form */
    TgpuBatch *batch;
    int gpu_group;                  /* single-group states: index of the group */
    int ngpu;                       /* groups of the compiled state */
    int gpu_slots[TAY_MAX_GROUPS];  /* group index of each segment */
    int state_batch;                /* the batch was made by tgpu_state_create */
    TgpuPass tpasses[TAY_MAX_PASSES];
    TgpuStatePass spasses[TAY_MAX_PASSES];
    TgpuGroup tgroup;               /* single-group form (tgpu_batch_create, tay_run_batch) */
    TgpuGroup tgroups[TAY_MAX_GROUPS];
    unsigned version;               /* bumped by every successful validation */
};

static unsigned g_threads = 0;

static void set_error(TayState *state, TayError error, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(state->message, sizeof(state->message), fmt, ap);
    va_end(ap);
    fprintf(stderr, "ERROR: %s\n", state->message);
    state->error = error;
}

static int group_active(const TayGroup *g) { return g->storage != 0; }

TayState *tay_create_state(void) {
    TayState *state = (TayState *)calloc(1, sizeof(TayState));
    if (!state) return 0;
    state->error = TAY_ERROR_NONE;
    state->gpu_group = -1;
    return state;
}

static int device_fail(TayState *state, int rc);

/* Brings a group's host records up to date with the device (a lazy fetch). */
static int fetch_group(TayState *state, TayGroup *g) {
    if (!g->host_stale) return 1;
    g->host_stale = 0;
    if (!state->batch || g->slot < 0) return 1;
    int rc = tgpu_batch_fetch(state->batch, g->slot, g->storage);
    return rc == TGPU_OK ? 1 : device_fail(state, rc);
}

static int sync_host(TayState *state) {
    int ok = 1;
    for (int i = 0; i < TAY_MAX_GROUPS; ++i)
        if (group_active(state->groups + i) && !fetch_group(state, state->groups + i)) ok = 0;
    return ok;
}

/* Drops the device batch after fetching what only the device holds. */
static void release_batch(TayState *state) {
    if (state->batch) {
        sync_host(state);
        tgpu_batch_destroy(state->batch);
    }
    state->batch = 0;
    for (int i = 0; i < TAY_MAX_GROUPS; ++i) {
        state->groups[i].slot = -1;
        state->groups[i].host_dirty = 1;
        state->groups[i].host_stale = 0;
        state->groups[i].write_through = 0;
    }
}

static void drop_batch_cache(void);
static int cache_refers_to(const TayState *state);

void tay_destroy_state(TayState *state) {
    if (!state) return;
    if (cache_refers_to(state)) drop_batch_cache();
    release_batch(state);
    for (int i = 0; i < TAY_MAX_GROUPS; ++i) tgpu_host_free(state->groups[i].storage);
    free(state);
}

/* There is no OpenCL device layer in this library: the GPU path is selected per group
 * with TAY_GPU_Z_GRID.  Both switches report "no OpenCL device". */
int tay_switch_to_ocl(TayState *state) {
    (void)state;
    return 0;
}

int tay_switch_to_host(TayState *state) {
    (void)state;
    return 0;
}

TayError tay_get_error(TayState *state) { return state->error; }

const char *tay_get_error_message(TayState *state) { return state->message; }

TayGroup *tay_add_group(TayState *state, unsigned agent_size, unsigned agent_capacity, int is_point) {
    int i = 0;
    for (; i < TAY_MAX_GROUPS; ++i)
        if (!group_active(state->groups + i)) break;
    if (i == TAY_MAX_GROUPS) {
        set_error(state, TAY_ERROR_GROUP_INDEX_OUT_OF_RANGE, "too many groups");
        return 0;
    }
    TayGroup *g = state->groups + i;
    memset(g, 0, sizeof(*g));
    g->storage = (char *)tgpu_host_alloc((unsigned long long)(agent_capacity ? agent_capacity : 1) * (agent_size ? agent_size : 1));
    if (!g->storage) {
        set_error(state, TAY_ERROR_GROUP_INDEX_OUT_OF_RANGE, "out of host memory");
        return 0;
    }
    g->agent_size = agent_size;
    g->capacity = agent_capacity;
    g->is_point = is_point;
    g->type = TAY_CPU_SIMPLE; /* the reference's default (tay/state.c:96) */
    g->dims = 3;
    g->part.x = g->part.y = g->part.z = g->part.w = 1.0f;
    g->id = state->next_group_id++;
    g->host_dirty = 1;
    g->slot = -1;
    state->recompile = 1;
    return g;
}

void tay_configure_space(TayState *state, TayGroup *group, TaySpaceType space_type, int space_dims, float4 min_part_sizes, int shared_size_in_megabytes) {
    fetch_group(state, group);
    group->host_dirty = 1;
    group->type = space_type;
    group->dims = space_dims;
    group->part = min_part_sizes;
    group->shared_mb = shared_size_in_megabytes;
    state->recompile = 1;
}

void tay_fix_space_box(TayState *state, TayGroup *group, float4 min, float4 max) {
    group->box_min = min;
    group->box_max = max;
    group->box_fixed = 1;
    state->recompile = 1;
}

void tay_add_see(TayState *state, TayGroup *seer_group, TayGroup *seen_group, void (*func)(void *, void *, void *), char *func_name, float4 radii, int self_see, void *context, unsigned context_size) {
    (void)func;
    if (state->passes_count >= TAY_MAX_PASSES) {
        set_error(state, TAY_ERROR_NOT_IMPLEMENTED, "too many passes");
        return;
    }
    TayPass *p = state->passes + state->passes_count++;
    memset(p, 0, sizeof(*p));
    p->is_see = 1;
    p->seer_group = seer_group;
    p->seen_group = seen_group;
    snprintf(p->func_name, TAY_MAX_FUNC_NAME, "%s", func_name ? func_name : "");
    p->radii = radii;
    p->self_see = self_see;
    p->context = context;
    p->context_size = context_size;
    state->recompile = 1;
}

void tay_add_act(TayState *state, TayGroup *act_group, void (*func)(void *, void *), char *func_name, void *context, unsigned context_size) {
    (void)func;
    if (state->passes_count >= TAY_MAX_PASSES) {
        set_error(state, TAY_ERROR_NOT_IMPLEMENTED, "too many passes");
        return;
    }
    TayPass *p = state->passes + state->passes_count++;
    memset(p, 0, sizeof(*p));
    p->is_see = 0;
    p->seer_group = act_group;
    p->seen_group = act_group;
    snprintf(p->func_name, TAY_MAX_FUNC_NAME, "%s", func_name ? func_name : "");
    p->context = context;
    p->context_size = context_size;
    state->recompile = 1;
}

void tay_clear_all_agents(TayState *state, TayGroup *group) {
    group->host_stale = 0;
    group->host_dirty = 1;
    group->count = 0;
    state->recompile = 1;
}

void *tay_get_available_agent(TayState *state, TayGroup *group) {
    if (group->count >= group->capacity) {
        set_error(state, TAY_ERROR_GROUP_INDEX_OUT_OF_RANGE, "group is full");
        return 0;
    }
    return group->storage + (size_t)group->agent_size * group->count;
}

void tay_commit_available_agent(TayState *state, TayGroup *group) {
    fetch_group(state, group);
    group->host_dirty = 1;
    if (group->count < group->capacity) ++group->count;
    state->recompile = 1;
}

unsigned tay_commit_agents(TayState *state, TayGroup *group, const void *records, unsigned count) {
    fetch_group(state, group);
    group->host_dirty = 1;
    unsigned room = group->capacity - group->count;
    unsigned n = count < room ? count : room;
    if (n < count) set_error(state, TAY_ERROR_GROUP_INDEX_OUT_OF_RANGE, "group is full");
    memcpy(group->storage + (size_t)group->agent_size * group->count, records, (size_t)group->agent_size * n);
    group->count += n;
    state->recompile = 1;
    return n;
}

unsigned tay_get_agent_count(TayState *state, TayGroup *group) {
    (void)state;
    return group->count;
}

void *tay_get_agent(TayState *state, TayGroup *group, int index) {
    group->read_since_run = 1;
    if (!fetch_group(state, group)) return 0;
    return group->storage + (size_t)group->agent_size * (size_t)index;
}

void tay_mark_agents_changed(TayState *state, TayGroup *group) {
    (void)state;
    group->host_stale = 0;
    group->host_dirty = 1;
}

void tay_simulation_start(TayState *state) {
    if (state->is_running) {
        set_error(state, TAY_ERROR_STATE_STATUS, "cannot start simulation if it's already running");
        return;
    }
    state->recompile = 1;
    state->is_running = 1;
}

void tay_simulation_end(TayState *state) {
    if (!state->is_running) {
        set_error(state, TAY_ERROR_STATE_STATUS, "cannot end simulation if it's not running");
        return;
    }
    state->is_running = 0;
    release_batch(state);
}

static int find_group(const TayState *state, const TayGroup *g) {
    for (int i = 0; i < TAY_MAX_GROUPS; ++i)
        if (g == state->groups + i) return group_active(g) ? i : -1;
    return -1;
}

/* Validation (the GPU counterpart of tay/state_compile.c:5-175): checks the groups and
 * passes and fills the device descriptors; the device batch is built lazily. */
static int validate(TayState *state) {
    if (!state->recompile) return 1;
    release_batch(state);
    state->gpu_group = -1;
    state->ngpu = 0;
    for (int i = 0; i < TAY_MAX_GROUPS; ++i) {
        TayGroup *g = state->groups + i;
        if (!group_active(g)) continue;
        if (g->type != TAY_GPU_Z_GRID) {
            set_error(state, TAY_ERROR_NOT_IMPLEMENTED,
                      "group %d uses a CPU structure; this library runs TAY_GPU_Z_GRID groups only", i);
            return 0;
        }

        if (g->dims < 1 || g->dims > 3) {
            set_error(state, TAY_ERROR_NOT_IMPLEMENTED, "the GPU Z-grid supports 1 to 3 dimensions");
            return 0;
        }
        g->slot = state->ngpu;
        state->gpu_slots[state->ngpu++] = i;
    }
    if (state->ngpu == 0) {
        set_error(state, TAY_ERROR_STATE_STATUS, "no active group");
        return 0;
    }
    if (state->passes_count == 0) {
        set_error(state, TAY_ERROR_STATE_STATUS, "no passes");
        return 0;
    }
    for (unsigned k = 0; k < state->passes_count; ++k) {
        TayPass *p = state->passes + k;
        int seer = find_group(state, p->seer_group), seen = find_group(state, p->seen_group);
        if (seer < 0 || (p->is_see && seen < 0)) {
            set_error(state, TAY_ERROR_GROUP_INDEX_OUT_OF_RANGE, "pass %u: group is not part of this state", k);
            return 0;
        }
        if (p->context && !p->context_size) {
            set_error(state, TAY_ERROR_DEVICE_MODEL, "pass context set but context size is 0");
            return 0;
        }
        if (!p->context && p->context_size) {
            set_error(state, TAY_ERROR_DEVICE_MODEL, "pass context not set but context size is not 0");
            return 0;
        }
        if (p->func_name[0] == '\0') {
            set_error(state, TAY_ERROR_DEVICE_MODEL, "pass with no func name set");
            return 0;
        }
        TgpuPass *t = state->tpasses + k;
        t->func_name = p->func_name;
        t->is_see = p->is_see;
        t->radii[0] = p->radii.x;
        t->radii[1] = p->radii.y;
        t->radii[2] = p->radii.z;
        t->radii[3] = p->radii.w;
        t->self_see = p->self_see;
        t->context = p->context;
        t->context_size = p->context_size;
        TgpuStatePass *sp = state->spasses + k;
        sp->pass = *t;
        sp->seer_group = state->groups[seer].slot;
        sp->seen_group = p->is_see ? state->groups[seen].slot : sp->seer_group;
    }
    /* a group's shape must be the one its device model holds: the reference's grids take
     * point agents only ("grid structure can only contain point agents"); here box
     * agents have their own device model and the Z-grid keys them by their min corner */
    for (unsigned k = 0; k < state->passes_count; ++k) {
        const TayPass *p = state->passes + k;
        int np = tgpu_model_nonpoint(p->func_name);
        if (np < 0) continue;
        if ((np == 1) == (p->seer_group->is_point != 0) ||
            (p->is_see && (np == 1) == (p->seen_group->is_point != 0))) {
            set_error(state, TAY_ERROR_POINT_NONPOINT_MISMATCH, "pass %u: '%s' takes %s agents", k, p->func_name,
                      np ? "non-point" : "point");
            return 0;
        }
    }
    for (int s = 0; s < state->ngpu; ++s) {
        const TayGroup *g = state->groups + state->gpu_slots[s];
        TgpuGroup *tg = state->tgroups + s;
        memset(tg, 0, sizeof(*tg));
        tg->agent_size = g->agent_size;
        tg->count = g->count;
        for (int a = 0; a < 4; ++a) {
            tg->min_part_sizes[a] = g->part.arr[a];
            tg->box_min[a] = g->box_min.arr[a];
            tg->box_max[a] = g->box_max.arr[a];
        }
        tg->shared_megabytes = g->shared_mb;
        tg->box_fixed = g->box_fixed;
        tg->dims = g->dims;
    }
    if (state->ngpu == 1) {
        state->gpu_group = state->gpu_slots[0];
        state->tgroup = state->tgroups[0];
        state->tgroup.pass_count = (int)state->passes_count;
        state->tgroup.passes = state->tpasses;
    }
    if (!tgpu_model_of(state->tpasses[0].func_name)) {
        set_error(state, TAY_ERROR_DEVICE_MODEL, "no device model provides '%s'", state->tpasses[0].func_name);
        return 0;
    }
    state->recompile = 0;
    ++state->version;
    return 1;
}

/* A single group whose pass list a device model runs as a program gets a program batch
 * (fused see + act kernels, and tay_run_batch); anything else a state batch. */
static int compile(TayState *state) {
    if (!validate(state)) return 0;
    if (state->batch) return 1;
    int rc = TGPU_ERR_PROGRAM;
    state->state_batch = 0;
    if (state->ngpu == 1) rc = tgpu_batch_create(&state->tgroup, 1, &state->batch);
    if (rc == TGPU_ERR_PROGRAM) {
        state->state_batch = 1;
        rc = tgpu_state_create(state->tgroups, state->ngpu, state->spasses, (int)state->passes_count, &state->batch);
    }
    if (rc != TGPU_OK) {
        set_error(state, rc == TGPU_ERR_CUDA ? TAY_ERROR_CUDA : TAY_ERROR_DEVICE_MODEL, "%s", tgpu_last_error());
        state->batch = 0;
        return 0;
    }
    for (int s = 0; s < state->ngpu; ++s) {
        state->groups[state->gpu_slots[s]].host_dirty = 1;
        state->groups[state->gpu_slots[s]].write_through = 0;
    }
    return 1;
}

static double now_s(void) {
    struct timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return (double)t.tv_sec + 1e-9 * (double)t.tv_nsec;
}

static int device_fail(TayState *state, int rc) {
    set_error(state, rc == TGPU_ERR_CUDA || rc == TGPU_ERR_DEVICE ? TAY_ERROR_CUDA : TAY_ERROR_DEVICE_MODEL, "%s",
              tgpu_last_error());
    return 0;
}

int tay_run(TayState *state, int steps) {
    if (!state->is_running) {
        set_error(state, TAY_ERROR_STATE_STATUS, "cannot run simulation steps if simulation is not started");
        return 0;
    }
    if (!compile(state)) return 0;
    double t0 = now_s();
    int rc = state->state_batch ? tgpu_state_set_contexts(state->batch, state->spasses, (int)state->passes_count)
                                : tgpu_batch_set_contexts(state->batch, 0, &state->tgroup);
    for (int s = 0; s < state->ngpu && rc == TGPU_OK; ++s) {
        TayGroup *g = state->groups + state->gpu_slots[s];
        if (!g->host_dirty) continue;
        rc = tgpu_batch_push(state->batch, s, g->storage);
        g->host_dirty = 0;
    }
    /* A group the host read after its previous run is written through to its storage at
     * the end of this one (the fetch overlaps the last pass); one it did not read stays on
     * the device until tay_get_agent asks for it. */
    for (int s = 0; s < state->ngpu && rc == TGPU_OK; ++s) {
        TayGroup *g = state->groups + state->gpu_slots[s];
        const int want = g->read_since_run && steps > 0;
        g->read_since_run = 0;
        if (want == g->write_through) continue;
        g->write_through = tgpu_batch_write_through(state->batch, s, want ? g->storage : 0) == TGPU_OK && want;
    }
    if (rc == TGPU_OK) rc = tgpu_batch_run(state->batch, steps);
    if (rc != TGPU_OK) return device_fail(state, rc);
    for (int s = 0; s < state->ngpu; ++s) {
        TayGroup *g = state->groups + state->gpu_slots[s];
        g->host_stale = !(g->write_through && steps > 0);
    }
    double t = now_s() - t0;
    state->ms_per_step = steps ? t / (double)steps * 1000.0 : 0.0;
    state->device_ms = tgpu_batch_last_device_ms(state->batch);
    state->pairs = tgpu_batch_last_pairs(state->batch);
    return steps;
}

/* Batched run: one device batch whose segments are the states' GPU groups.  The batch
 * is cached for the last list of states it was built for. */
static struct {
    TgpuBatch *batch;
    TgpuAdjoint *adjoint;
    TayState **states;
    unsigned *versions;
    int count;
} g_batch_cache;

static void drop_batch_cache(void) {
    if (g_batch_cache.adjoint) tgpu_adjoint_destroy(g_batch_cache.adjoint);
    if (g_batch_cache.batch) tgpu_batch_destroy(g_batch_cache.batch);
    free(g_batch_cache.states);
    free(g_batch_cache.versions);
    memset(&g_batch_cache, 0, sizeof(g_batch_cache));
}

static int cache_refers_to(const TayState *state) {
    for (int i = 0; i < g_batch_cache.count; ++i)
        if (g_batch_cache.states[i] == state) return 1;
    return 0;
}

static int cache_matches(TayState **states, int count) {
    if (!g_batch_cache.batch || g_batch_cache.count != count) return 0;
    for (int i = 0; i < count; ++i) {
        if (g_batch_cache.states[i] != states[i]) return 0;
        if (g_batch_cache.versions[i] != states[i]->version) return 0;
    }
    return 1;
}

/* Builds (or reuses) the cached batch of `states`; returns it or NULL with errors set. */
static TgpuBatch *batch_for(TayState **states, int count) {
    if (count <= 0) return 0;
    for (int i = 0; i < count; ++i) {
        if (!states[i]->is_running) {
            set_error(states[i], TAY_ERROR_STATE_STATUS, "cannot run simulation steps if simulation is not started");
            return 0;
        }
        if (!validate(states[i])) return 0;
        if (states[i]->ngpu != 1) {
            set_error(states[i], TAY_ERROR_BATCH, "tay_run_batch runs states of one group each");
            return 0;
        }
        if (!sync_host(states[i])) return 0;
    }
    if (!cache_matches(states, count)) {
        drop_batch_cache();
        TgpuGroup *groups = (TgpuGroup *)calloc((size_t)count, sizeof(TgpuGroup));
        for (int i = 0; i < count; ++i) groups[i] = states[i]->tgroup;
        TgpuBatch *b = 0;
        int rc = tgpu_batch_create(groups, count, &b);
        free(groups);
        if (rc != TGPU_OK) {
            for (int i = 0; i < count; ++i)
                set_error(states[i], rc == TGPU_ERR_CUDA ? TAY_ERROR_CUDA : TAY_ERROR_BATCH, "%s", tgpu_last_error());
            return 0;
        }
        g_batch_cache.batch = b;
        g_batch_cache.count = count;
        g_batch_cache.states = (TayState **)malloc(sizeof(TayState *) * (size_t)count);
        g_batch_cache.versions = (unsigned *)malloc(sizeof(unsigned) * (size_t)count);
        for (int i = 0; i < count; ++i) {
            g_batch_cache.states[i] = states[i];
            g_batch_cache.versions[i] = states[i]->version;
        }
    }
    return g_batch_cache.batch;
}

static int push_all(TgpuBatch *b, TayState **states, int count) {
    int rc = TGPU_OK;
    for (int i = 0; i < count && rc == TGPU_OK; ++i) {
        rc = tgpu_batch_set_contexts(b, i, &states[i]->tgroup);
        if (rc == TGPU_OK) rc = tgpu_batch_push(b, i, states[i]->groups[states[i]->gpu_group].storage);
    }
    return rc;
}

/* Batched runs keep the eager contract: every state's records are pushed before and
 * fetched after; each state's own device copy is then out of date. */
static int fetch_all(TgpuBatch *b, TayState **states, int count) {
    int rc = TGPU_OK;
    for (int i = 0; i < count && rc == TGPU_OK; ++i) {
        TayGroup *g = states[i]->groups + states[i]->gpu_group;
        rc = tgpu_batch_fetch(b, i, g->storage);
        g->host_dirty = 1;
        g->host_stale = 0;
    }
    return rc;
}

int tay_run_batch(TayState **states, int count, int steps) {
    if (!states || count <= 0) return 0;
    TgpuBatch *b = batch_for(states, count);
    if (!b) return 0;
    double t0 = now_s();
    int rc = push_all(b, states, count);
    /* every state is fetched after the run: write its records through where its storage
     * is page-locked (the fetch then only waits) */
    for (int i = 0; i < count && rc == TGPU_OK; ++i)
        tgpu_batch_write_through(b, i, states[i]->groups[states[i]->gpu_group].storage);
    if (rc == TGPU_OK) rc = tgpu_batch_run(b, steps);
    if (rc == TGPU_OK) rc = fetch_all(b, states, count);
    if (rc != TGPU_OK) {
        for (int i = 0; i < count; ++i) device_fail(states[i], rc);
        return 0;
    }
    double t = now_s() - t0;
    for (int i = 0; i < count; ++i) {
        states[i]->ms_per_step = steps ? t / (double)steps * 1000.0 : 0.0;
        states[i]->device_ms = tgpu_batch_last_device_ms(b);
        states[i]->pairs = tgpu_batch_last_pairs(b);
    }
    return steps;
}

int tay_run_recorded(TayState **states, int count, int steps, int checkpoint_every) {
    if (!states || count <= 0 || steps <= 0) return 0;
    TgpuBatch *b = batch_for(states, count);
    if (!b) return 0;
    if (g_batch_cache.adjoint) {
        tgpu_adjoint_destroy(g_batch_cache.adjoint);
        g_batch_cache.adjoint = 0;
    }
    double t0 = now_s();
    int rc = push_all(b, states, count);
    if (rc == TGPU_OK) rc = tgpu_adjoint_create(b, steps, checkpoint_every, 1, &g_batch_cache.adjoint);
    if (rc == TGPU_OK) rc = tgpu_adjoint_forward(g_batch_cache.adjoint);
    if (rc == TGPU_OK) rc = fetch_all(b, states, count);
    if (rc != TGPU_OK) {
        for (int i = 0; i < count; ++i) device_fail(states[i], rc);
        return 0;
    }
    double t = now_s() - t0;
    for (int i = 0; i < count; ++i) {
        states[i]->ms_per_step = t / (double)steps * 1000.0;
        states[i]->device_ms = tgpu_adjoint_forward_ms(g_batch_cache.adjoint);
    }
    return 1;
}

int tay_run_backward(TayState **states, int count, const float *dloss_dp, const float *dloss_dv, float *dloss_dp0,
                     float *dloss_dv0, double *dloss_dparams) {
    if (!states || count <= 0) return 0;
    if (!g_batch_cache.adjoint || !cache_matches(states, count)) {
        for (int i = 0; i < count; ++i)
            set_error(states[i], TAY_ERROR_STATE_STATUS, "tay_run_backward needs a tay_run_recorded of the same states");
        return 0;
    }
    int rc = tgpu_adjoint_backward(g_batch_cache.adjoint, dloss_dp, dloss_dv, dloss_dp0, dloss_dv0, dloss_dparams);
    if (rc != TGPU_OK) {
        for (int i = 0; i < count; ++i) device_fail(states[i], rc);
        return 0;
    }
    return 1;
}

double tay_get_recorded_forward_ms(void) {
    return g_batch_cache.adjoint ? tgpu_adjoint_forward_ms(g_batch_cache.adjoint) : 0.0;
}

double tay_get_backward_ms(void) {
    return g_batch_cache.adjoint ? tgpu_adjoint_backward_ms(g_batch_cache.adjoint) : 0.0;
}

unsigned long long tay_get_adjoint_device_bytes(void) {
    unsigned long long bytes = 0;
    if (g_batch_cache.batch) bytes += tgpu_batch_device_bytes(g_batch_cache.batch);
    if (g_batch_cache.adjoint) bytes += tgpu_adjoint_device_bytes(g_batch_cache.adjoint);
    return bytes;
}

double tay_get_ms_per_step_for_last_run(TayState *state) { return state->ms_per_step; }
double tay_get_device_ms_for_last_run(TayState *state) { return state->device_ms; }
unsigned long long tay_get_pairs_for_last_run(TayState *state) { return state->pairs; }

void tay_log(void *file, char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vfprintf(stdout, fmt, ap);
    va_end(ap);
    fflush(stdout);
    if (file) {
        va_start(ap, fmt);
        vfprintf((FILE *)file, fmt, ap);
        va_end(ap);
    }
}

/* Device models are compiled into the library; OpenCL sources have no use here. */
void ocl_add_source(TayState *state, const char *source) {
    (void)state;
    (void)source;
}

/* The CPU thread pool of the reference (tay/thread.c) is replaced by device launches;
 * the thread count is kept for hosts that query it. */
void tay_threads_start(unsigned threads_count, unsigned thread_storage_size) {
    (void)thread_storage_size;
    g_threads = threads_count ? threads_count : 1;
}

void tay_threads_stop(void) { g_threads = 0; }

unsigned tay_get_number_of_threads(void) { return g_threads; }
