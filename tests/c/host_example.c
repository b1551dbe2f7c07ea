/* A C host of the Tay API, written the way the reference's own harness drives it
 * (test/test_basic.c:92-165, test/test_combo.c:40-130): it includes include/tay.h, links
 * libtay_gb300.so and runs
 *   1. one group of the test agent, see + act, a few steps, agents read back with
 *      tay_get_agent (a lazy fetch) and checked for motion and neighbour counts;
 *   2. two groups mixed by their see passes (the combination test's pass list);
 *   3. two single-group states advanced by tay_run_batch.
 * It prints one line per part and exits 0 when every check holds.  The record layout is the
 * reference's test agent (test/agent.h:2-19). */
#include "tay.h"

#include <math.h>
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>

#pragma pack(push, 1)
typedef struct {
    TayAgentTag tag;
    float4 p;
    float4 v;
    float4 b_buffer;
    int b_buffer_count;
    float4 f_buffer;
    int result_index;
} Agent;
typedef struct {
    float4 radii;
} SeeContext;
typedef struct {
    float4 min;
    float4 max;
} ActContext;
#pragma pack(pop)

static unsigned long long rng_state = 0x9E3779B97F4A7C15ull;

static float rnd(float lo, float hi) {
    rng_state = rng_state * 6364136223846793005ull + 1442695040888963407ull;
    return lo + (hi - lo) * (float)((rng_state >> 40) & 0xFFFFFF) / 16777216.0f;
}

static void add_agents(TayState *tay, TayGroup *g, int n) {
    for (int i = 0; i < n; ++i) {
        Agent *a = (Agent *)tay_get_available_agent(tay, g);
        a->p.x = rnd(0.0f, 1000.0f);
        a->p.y = rnd(0.0f, 1000.0f);
        a->p.z = rnd(0.0f, 1000.0f);
        a->v.x = rnd(-1.0f, 1.0f);
        a->v.y = rnd(-1.0f, 1.0f);
        a->v.z = rnd(-1.0f, 1.0f);
        a->b_buffer_count = 0;
        a->result_index = i;
        tay_commit_available_agent(tay, g);
    }
}

static int fail(const char *what, TayState *tay) {
    fprintf(stderr, "FAIL %s: error %d %s\n", what, (int)tay_get_error(tay), tay_get_error_message(tay));
    return 1;
}

int main(void) {
    const int n = 20000;
    float4 part = {{{50.0f, 50.0f, 50.0f, 50.0f}}};
    float4 radii = {{{50.0f, 50.0f, 50.0f, 0.0f}}};
    static SeeContext see_ctx;
    static ActContext act_ctx;
    see_ctx.radii = radii;
    act_ctx.max.x = act_ctx.max.y = act_ctx.max.z = 1000.0f;

    /* 1. one group */
    TayState *tay = tay_create_state();
    TayGroup *g = tay_add_group(tay, sizeof(Agent), n, TAY_TRUE);
    tay_configure_space(tay, g, TAY_GPU_Z_GRID, 3, part, 250);
    tay_add_see(tay, g, g, 0, "agent_see", radii, TAY_FALSE, &see_ctx, sizeof(see_ctx));
    tay_add_act(tay, g, 0, "agent_act", &act_ctx, sizeof(act_ctx));
    add_agents(tay, g, n);
    tay_simulation_start(tay);
    if (tay_run(tay, 5) != 5) return fail("tay_run", tay);
    double moved = 0.0, fsum = 0.0;
    int ids_ok = 1;
    static int seen[20000];
    for (int i = 0; i < n; ++i) {
        Agent *a = (Agent *)tay_get_agent(tay, g, i);
        if (!a) return fail("tay_get_agent", tay);
        if (a->result_index < 0 || a->result_index >= n || seen[a->result_index]++) ids_ok = 0;
        moved += fabs(a->v.x) + fabs(a->v.y) + fabs(a->v.z);
        fsum += fabs(a->f_buffer.x) + fabs(a->f_buffer.y) + fabs(a->f_buffer.z);
    }
    unsigned long long pairs = tay_get_pairs_for_last_run(tay);
    printf("one group: %d agents, 5 steps, %.3f ms/step, %llu pairs, ids %s\n", n, tay_get_ms_per_step_for_last_run(tay),
           pairs, ids_ok ? "ok" : "BAD");
    if (!ids_ok || pairs == 0 || !(fsum > 0.0) || !(moved > 0.0)) return fail("one-group checks", tay);
    tay_simulation_end(tay);
    tay_destroy_state(tay);

    /* 2. two groups, the combination test's passes */
    tay = tay_create_state();
    TayGroup *ga = tay_add_group(tay, sizeof(Agent), n / 2, TAY_TRUE);
    TayGroup *gb = tay_add_group(tay, sizeof(Agent), n / 2, TAY_TRUE);
    tay_configure_space(tay, ga, TAY_GPU_Z_GRID, 3, part, 250);
    tay_configure_space(tay, gb, TAY_GPU_Z_GRID, 3, part, 250);
    tay_add_see(tay, ga, ga, 0, "agent_see", radii, TAY_FALSE, &see_ctx, sizeof(see_ctx));
    tay_add_see(tay, ga, gb, 0, "agent_see", radii, TAY_FALSE, &see_ctx, sizeof(see_ctx));
    tay_add_see(tay, gb, gb, 0, "agent_see", radii, TAY_FALSE, &see_ctx, sizeof(see_ctx));
    tay_add_see(tay, gb, ga, 0, "agent_see", radii, TAY_FALSE, &see_ctx, sizeof(see_ctx));
    add_agents(tay, ga, n / 2);
    add_agents(tay, gb, n / 2);
    tay_simulation_start(tay);
    if (tay_run(tay, 1) != 1) return fail("tay_run (two groups)", tay);
    long long counts = 0;
    for (int i = 0; i < n / 2; ++i) counts += ((Agent *)tay_get_agent(tay, ga, i))->b_buffer_count;
    printf("two groups: %llu pairs, group a counts %lld\n", tay_get_pairs_for_last_run(tay), counts);
    if (counts <= 0 || (unsigned long long)counts > tay_get_pairs_for_last_run(tay))
        return fail("two-group checks", tay);
    tay_simulation_end(tay);
    tay_destroy_state(tay);

    /* 3. two states in one batch */
    TayState *states[2];
    TayGroup *groups[2];
    for (int s = 0; s < 2; ++s) {
        states[s] = tay_create_state();
        groups[s] = tay_add_group(states[s], sizeof(Agent), n / 4, TAY_TRUE);
        tay_configure_space(states[s], groups[s], TAY_GPU_Z_GRID, 3, part, 64);
        tay_add_see(states[s], groups[s], groups[s], 0, "agent_see", radii, TAY_FALSE, &see_ctx, sizeof(see_ctx));
        tay_add_act(states[s], groups[s], 0, "agent_act", &act_ctx, sizeof(act_ctx));
        add_agents(states[s], groups[s], n / 4);
        tay_simulation_start(states[s]);
    }
    if (tay_run_batch(states, 2, 3) != 3) return fail("tay_run_batch", states[0]);
    printf("batch: 2 states, %llu pairs\n", tay_get_pairs_for_last_run(states[0]));
    for (int s = 0; s < 2; ++s) {
        tay_simulation_end(states[s]);
        tay_destroy_state(states[s]);
    }
    printf("ok\n");
    return 0;
}
