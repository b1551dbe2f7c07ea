/* Driver that runs a workload through the reference Tay library's own public C API.
 *
 * TEST INFRASTRUCTURE ONLY.  Linked by oracle/ref/Makefile together with the reference
 * sources (compiled where they lie) into oracle/_ref/libtayref.so.  It does what the
 * reference's own harness does (test/test_basic.c:92-165): create a state, add one
 * group, configure its space, register the passes, commit agents, tay_run, then read the
 * agents back with tay_get_agent and order them by their id field (the reference's
 * result_index idiom, test/test.c:92-122).
 *
 * Models:
 *   REF_MODEL_TEST  - the reference's own test agent (test/agent.c agent_see/agent_act)
 *   REF_MODEL_BOIDS - oracle boids (oracle/oracle_models.h), run by the reference framework
 *   REF_MODEL_SPH   - oracle SPH, run by the reference framework
 *   REF_MODEL_BOX   - the reference's own box agent (test/agent.c box_agent_see/act), a
 *                     non-point group
 */
#include "tay.h"
#include "thread.h"
#include "agent_host.h"

#include <stdlib.h>
#include <string.h>

#define REAL float
#include "../oracle_models.h"

enum { REF_MODEL_TEST = 0, REF_MODEL_BOIDS = 1, REF_MODEL_SPH = 2, REF_MODEL_BOX = 3 };

/* pass mask bits, in registration order */
enum { REF_PASS_SEE0 = 1, REF_PASS_ACT0 = 2, REF_PASS_SEE1 = 4, REF_PASS_ACT1 = 8 };

static unsigned ref_threads = 0;

/* Space options of the following runs: tay_configure_space dims and tay_fix_space_box. */
static int ref_dims = 3;
static int ref_box_fixed = 0;
static float4 ref_box_min, ref_box_max;

void ref_set_space(int dims, int box_fixed, const float *box_min, const float *box_max) {
    ref_dims = dims;
    ref_box_fixed = box_fixed;
    for (int i = 0; i < 3; ++i) {
        ref_box_min.arr[i] = box_fixed ? box_min[i] : 0.0f;
        ref_box_max.arr[i] = box_fixed ? box_max[i] : 0.0f;
    }
    ref_box_min.arr[3] = ref_box_max.arr[3] = 0.0f;
}

static void configure(TayState *tay, TayGroup *group, int space_type, float part_size, int mb) {
    float4 part = {{{part_size, part_size, part_size, part_size}}};
    tay_configure_space(tay, group, (TaySpaceType)space_type, ref_dims, part, mb);
    if (ref_box_fixed)
        tay_fix_space_box(tay, group, ref_box_min, ref_box_max);
}

static void ensure_threads(int threads) {
    if (threads <= 0)
        threads = 1;
    if (ref_threads == (unsigned)threads)
        return;
    if (ref_threads)
        tay_threads_stop();
    tay_threads_start((unsigned)threads, 1u << 16);
    ref_threads = (unsigned)threads;
}

unsigned ref_agent_size(int model) {
    switch (model) {
        case REF_MODEL_TEST: return (unsigned)sizeof(Agent);
        case REF_MODEL_BOIDS: return (unsigned)sizeof(OBoid);
        case REF_MODEL_SPH: return (unsigned)sizeof(OSphParticle);
        case REF_MODEL_BOX: return (unsigned)sizeof(BoxAgent);
        default: return 0;
    }
}

static int agent_id(int model, const char *agent) {
    switch (model) {
        case REF_MODEL_TEST: return ((const Agent *)agent)->result_index;
        case REF_MODEL_BOIDS: return ((const OBoid *)agent)->id;
        case REF_MODEL_SPH: return ((const OSphParticle *)agent)->id;
        case REF_MODEL_BOX: return ((const BoxAgent *)agent)->result_index;
        default: return -1;
    }
}

/* Runs `steps` steps.  `agents` holds n AoS records in id order on entry and on return.
 * `see_ctx`/`act_ctx` are the model contexts (copied).  `radii` are the see radii,
 * `part_size` the structure's minimum part size (isotropic), `mb` its shared memory.
 * Returns the number of steps run (0 on error) and the reference's ms/step. */
int ref_run(int model, int space_type, int n, void *agents, const void *see_ctx, const void *act_ctx,
            float radius, float part_size, int mb, int steps, unsigned pass_mask, int threads,
            double *ms_per_step) {
    ensure_threads(threads);
    unsigned agent_size = ref_agent_size(model);
    if (!agent_size || n <= 0)
        return 0;

    static SeeContext test_see_ctx;
    static ActContext test_act_ctx;
    static OBoidsContext boids_ctx;
    static OSphContext sph_ctx;

    TayState *tay = tay_create_state();
    TayGroup *group = tay_add_group(tay, agent_size, (unsigned)n, model == REF_MODEL_BOX ? TAY_FALSE : TAY_TRUE);
    configure(tay, group, space_type, part_size, mb);

    float4 radii = {{{radius, radius, radius, radius}}};
    if (model == REF_MODEL_BOX) {
        memcpy(&test_see_ctx, see_ctx, sizeof(test_see_ctx));
        memcpy(&test_act_ctx, act_ctx, sizeof(test_act_ctx));
        radii.w = 0.0f;
        if (pass_mask & REF_PASS_SEE0)
            tay_add_see(tay, group, group, (void (*)(void *, void *, void *))box_agent_see, "box_agent_see", radii,
                        TAY_FALSE, &test_see_ctx, sizeof(test_see_ctx));
        if (pass_mask & REF_PASS_ACT0)
            tay_add_act(tay, group, (void (*)(void *, void *))box_agent_act, "box_agent_act", &test_act_ctx,
                        sizeof(test_act_ctx));
    }
    else if (model == REF_MODEL_TEST) {
        memcpy(&test_see_ctx, see_ctx, sizeof(test_see_ctx));
        memcpy(&test_act_ctx, act_ctx, sizeof(test_act_ctx));
        radii.w = 0.0f;
        if (pass_mask & REF_PASS_SEE0)
            tay_add_see(tay, group, group, (void (*)(void *, void *, void *))agent_see, "agent_see", radii, TAY_FALSE,
                        &test_see_ctx, sizeof(test_see_ctx));
        if (pass_mask & REF_PASS_ACT0)
            tay_add_act(tay, group, (void (*)(void *, void *))agent_act, "agent_act", &test_act_ctx, sizeof(test_act_ctx));
    }
    else if (model == REF_MODEL_BOIDS) {
        memcpy(&boids_ctx, see_ctx, sizeof(boids_ctx));
        if (pass_mask & REF_PASS_SEE0)
            tay_add_see(tay, group, group, o_boids_see, "boids_see", radii, TAY_FALSE, &boids_ctx, sizeof(boids_ctx));
        if (pass_mask & REF_PASS_ACT0)
            tay_add_act(tay, group, o_boids_act, "boids_act", &boids_ctx, sizeof(boids_ctx));
    }
    else {
        memcpy(&sph_ctx, see_ctx, sizeof(sph_ctx));
        if (pass_mask & REF_PASS_SEE0)
            tay_add_see(tay, group, group, o_sph_density, "sph_density", radii, TAY_TRUE, &sph_ctx, sizeof(sph_ctx));
        if (pass_mask & REF_PASS_ACT0)
            tay_add_act(tay, group, o_sph_pressure, "sph_pressure", &sph_ctx, sizeof(sph_ctx));
        if (pass_mask & REF_PASS_SEE1)
            tay_add_see(tay, group, group, o_sph_force, "sph_force", radii, TAY_FALSE, &sph_ctx, sizeof(sph_ctx));
        if (pass_mask & REF_PASS_ACT1)
            tay_add_act(tay, group, o_sph_integrate, "sph_integrate", &sph_ctx, sizeof(sph_ctx));
    }

    for (int i = 0; i < n; ++i) {
        void *slot = tay_get_available_agent(tay, group);
        memcpy(slot, (char *)agents + (size_t)agent_size * i, agent_size);
        tay_commit_available_agent(tay, group);
    }

    tay_simulation_start(tay);
    int run = tay_run(tay, steps);
    if (ms_per_step)
        *ms_per_step = tay_get_ms_per_step_for_last_run(tay);

    if (run == steps) {
        for (int i = 0; i < n; ++i) {
            char *a = (char *)tay_get_agent(tay, group, i);
            int id = agent_id(model, a);
            if (id < 0 || id >= n) {
                run = 0;
                break;
            }
            memcpy((char *)agents + (size_t)agent_size * id, a, agent_size);
        }
    }
    tay_simulation_end(tay);
    tay_destroy_state(tay);
    return run;
}

/* Several groups of one model in one reference state, with a pass list that mixes groups
 * (the shape of test/test_combo.c:114-119).  Same contract as oracle_run_groups: pass k
 * is tay_add_see(group pass_seer[k], group pass_seen[k]) or tay_add_act(group
 * pass_seer[k]); agents[g] holds counts[g] records in id order on entry and on return. */
int ref_run_groups(int model, int space_type, int ngroups, const int *counts, void **agents, const void *see_ctx,
                   const void *act_ctx, float radius, float part_size, int mb, int steps, int npasses,
                   const int *pass_is_see, const int *pass_seer, const int *pass_seen, const int *pass_self_see,
                   int threads, double *ms_per_step) {
    enum { kMaxGroups = 8 };
    ensure_threads(threads);
    unsigned agent_size = ref_agent_size(model);
    if (!agent_size || ngroups <= 0 || ngroups > kMaxGroups || (model != REF_MODEL_TEST && model != REF_MODEL_BOIDS))
        return 0;
    for (int k = 0; k < npasses; ++k)
        if (pass_seer[k] < 0 || pass_seer[k] >= ngroups || (pass_is_see[k] && (pass_seen[k] < 0 || pass_seen[k] >= ngroups)))
            return 0;

    static SeeContext test_see_ctx;
    static ActContext test_act_ctx;
    static OBoidsContext boids_ctx;

    TayState *tay = tay_create_state();
    TayGroup *groups[kMaxGroups];
    for (int g = 0; g < ngroups; ++g) {
        groups[g] = tay_add_group(tay, agent_size, (unsigned)counts[g], TAY_TRUE);
        configure(tay, groups[g], space_type, part_size, mb);
    }
    float4 radii = {{{radius, radius, radius, radius}}};
    if (model == REF_MODEL_TEST) {
        memcpy(&test_see_ctx, see_ctx, sizeof(test_see_ctx));
        memcpy(&test_act_ctx, act_ctx, sizeof(test_act_ctx));
        radii.w = 0.0f;
    }
    else {
        memcpy(&boids_ctx, see_ctx, sizeof(boids_ctx));
    }
    for (int k = 0; k < npasses; ++k) {
        TayGroup *seer = groups[pass_seer[k]];
        if (pass_is_see[k]) {
            TayGroup *seen = groups[pass_seen[k]];
            if (model == REF_MODEL_TEST)
                tay_add_see(tay, seer, seen, (void (*)(void *, void *, void *))agent_see, "agent_see", radii,
                            pass_self_see[k], &test_see_ctx, sizeof(test_see_ctx));
            else
                tay_add_see(tay, seer, seen, o_boids_see, "boids_see", radii, pass_self_see[k], &boids_ctx,
                            sizeof(boids_ctx));
        }
        else {
            if (model == REF_MODEL_TEST)
                tay_add_act(tay, seer, (void (*)(void *, void *))agent_act, "agent_act", &test_act_ctx,
                            sizeof(test_act_ctx));
            else
                tay_add_act(tay, seer, o_boids_act, "boids_act", &boids_ctx, sizeof(boids_ctx));
        }
    }
    for (int g = 0; g < ngroups; ++g)
        for (int i = 0; i < counts[g]; ++i) {
            void *slot = tay_get_available_agent(tay, groups[g]);
            memcpy(slot, (char *)agents[g] + (size_t)agent_size * i, agent_size);
            tay_commit_available_agent(tay, groups[g]);
        }

    tay_simulation_start(tay);
    int run = tay_run(tay, steps);
    if (ms_per_step)
        *ms_per_step = tay_get_ms_per_step_for_last_run(tay);
    for (int g = 0; g < ngroups && run == steps; ++g)
        for (int i = 0; i < counts[g]; ++i) {
            char *a = (char *)tay_get_agent(tay, groups[g], i);
            int id = agent_id(model, a);
            if (id < 0 || id >= counts[g]) {
                run = 0;
                break;
            }
            memcpy((char *)agents[g] + (size_t)agent_size * id, a, agent_size);
        }
    tay_simulation_end(tay);
    tay_destroy_state(tay);
    return run;
}

int ref_space_enum(const char *name) {
    if (!strcmp(name, "simple")) return TAY_CPU_SIMPLE;
    if (!strcmp(name, "kd_tree")) return TAY_CPU_KD_TREE;
    if (!strcmp(name, "grid")) return TAY_CPU_GRID;
    if (!strcmp(name, "z_grid")) return TAY_CPU_Z_GRID;
    return -1;
}
