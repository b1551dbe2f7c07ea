/* ORACLE (test infrastructure, not the product).
 *
 * A plain-C restatement of the reference Tay CPU path for one group of point agents:
 * the step loop (tay/state.c:194-323), the CpuSimple, CpuGrid and CpuZGrid structures
 * (tay/cpu_simple.c, tay/cpu_grid.c, tay/cpu_z_grid.c), the point-point pairing kernels
 * (tay/space.c:62-68, 106-148), the act pass (tay/space.c:250-263) and the static thread
 * split (tay/thread.c:244-250), on a POSIX thread pool.
 *
 * It is compiled twice into oracle/_build/liboracle.so: REAL=float with
 * -ffp-contract=off (the FP32 oracle, pinned against the reference itself and against
 * the committed golden vectors) and REAL=double (the FP64 oracle that every FP32 float
 * result is also compared with).  Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg load it.
 */
#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <unistd.h>

#ifndef REAL
#define REAL float
#endif
#ifndef SUFFIX
#define SUFFIX _f32
#endif

#include "oracle_models.h"

#define O_CAT2(a, b) a##b
#define O_CAT(a, b) O_CAT2(a, b)
#define O_NAME(x) O_CAT(x, SUFFIX)

#if defined(ORACLE_DOUBLE)
#define O_FLOOR floor
#define O_CEIL ceil
#define O_POW pow
#define O_BIG DBL_MAX
#else
#define O_FLOOR floorf
#define O_CEIL ceilf
#define O_POW powf
#define O_BIG FLT_MAX
#endif

enum { O_SPACE_SIMPLE = 1, O_SPACE_GRID = 4, O_SPACE_Z_GRID = 5 };
enum { O_MODEL_TEST = 0, O_MODEL_BOIDS = 1, O_MODEL_SPH = 2, O_MODEL_BOX = 3 };
enum { O_PASS_SEE0 = 1, O_PASS_ACT0 = 2, O_PASS_SEE1 = 4, O_PASS_ACT1 = 8 };

typedef void (*OSeeFn)(void *, void *, void *);
typedef void (*OActFn)(void *, void *);

/* ------------------------------------------------------------------ thread pool */

typedef struct OTask OTask;
typedef void (*OTaskFn)(OTask *task, int thread_i, int threads);
struct OTask {
    OTaskFn fn;
    void *arg;
};

static struct {
    int count;
    pthread_t handles[64];
    pthread_mutex_t lock;
    pthread_cond_t go, done;
    unsigned long long generation;
    int remaining;
    int stop;
    OTask *task;
} O_NAME(pool) = {0, {0}, PTHREAD_MUTEX_INITIALIZER, PTHREAD_COND_INITIALIZER, PTHREAD_COND_INITIALIZER, 0, 0, 0, 0};
#define POOL O_NAME(pool)

typedef struct {
    int index;
    unsigned long long start_generation; /* generation current when the worker was created */
} OWorkerArg;
static OWorkerArg O_NAME(worker_args)[64];

static void *O_NAME(worker)(void *varg) {
    int index = ((OWorkerArg *)varg)->index;
    unsigned long long seen = ((OWorkerArg *)varg)->start_generation;
    for (;;) {
        pthread_mutex_lock(&POOL.lock);
        while (POOL.generation == seen)
            pthread_cond_wait(&POOL.go, &POOL.lock);
        seen = POOL.generation;
        int stop = POOL.stop;
        OTask *task = POOL.task;
        pthread_mutex_unlock(&POOL.lock);
        if (!stop)
            task->fn(task, index, POOL.count);
        pthread_mutex_lock(&POOL.lock);
        if (--POOL.remaining == 0)
            pthread_cond_signal(&POOL.done);
        pthread_mutex_unlock(&POOL.lock);
        if (stop)
            return 0;
    }
}

static void O_NAME(pool_run)(OTask *task) {
    pthread_mutex_lock(&POOL.lock);
    POOL.task = task;
    POOL.remaining = POOL.count;
    ++POOL.generation;
    pthread_cond_broadcast(&POOL.go);
    while (POOL.remaining > 0)
        pthread_cond_wait(&POOL.done, &POOL.lock);
    pthread_mutex_unlock(&POOL.lock);
}

static void O_NAME(pool_stop)(void) {
    if (!POOL.count)
        return;
    POOL.stop = 1;
    OTask none = {0, 0};
    O_NAME(pool_run)(&none);
    for (int i = 0; i < POOL.count; ++i)
        pthread_join(POOL.handles[i], 0);
    POOL.count = 0;
    POOL.stop = 0;
}

static void O_NAME(pool_start)(int threads) {
    if (threads <= 0) {
        long online = sysconf(_SC_NPROCESSORS_ONLN);
        threads = online > 0 ? (int)online : 1;
    }
    if (threads > 64)
        threads = 64;
    if (POOL.count == threads)
        return;
    O_NAME(pool_stop)();
    POOL.count = threads;
    for (int i = 0; i < threads; ++i) {
        O_NAME(worker_args)[i].index = i;
        O_NAME(worker_args)[i].start_generation = POOL.generation;
        pthread_create(&POOL.handles[i], 0, O_NAME(worker), &O_NAME(worker_args)[i]);
    }
}

/* tay/thread.c:244-250: equal shares, the last thread takes the remainder */
static inline void o_range(unsigned count, int thread_i, int threads, unsigned *beg, unsigned *end) {
    unsigned share = count / (unsigned)threads;
    *beg = share * (unsigned)thread_i;
    *end = (thread_i + 1 < threads) ? *beg + share : count;
}

/* ------------------------------------------------------------------ group and space */

typedef struct {
    unsigned count;
    unsigned first;
} OZCell;

typedef struct OGCell {
    struct OGCell *next;
    unsigned count;
    unsigned first;
    int idx[3];
} OGCell;

typedef struct {
    char *storage;
    char *sort_storage;
    unsigned agent_size;
    unsigned count;
    int space;
    int dims;                         /* tay_configure_space dims: 1..3 */
    int is_point;                     /* 0: box agents, min at the position's offset, max after it */
    int box_fixed;                    /* tay_fix_space_box */
    REAL fixed_min[3], fixed_max[3];
    REAL part[3];
    REAL box_min[3], box_max[3];
    /* grids */
    REAL origin[3];
    REAL cell_size[3];
    int cell_counts[3];
    unsigned cells_count;
    unsigned max_cells;
    OZCell *zcells;
    OGCell *gcells;
    OGCell *first_gcell;
} OGroup;

typedef struct {
    int is_see;
    OSeeFn see;
    OActFn act;
    REAL radii[3];
    int self_see;
    void *ctx;
} OPass;

static inline REAL *o_pos(const OGroup *g, unsigned i) {
    return (REAL *)(g->storage + (size_t)g->agent_size * i + sizeof(OTag));
}

/* a box agent's max corner follows its min (the position), tay/state.h float4_agent_max */
static inline REAL *o_max(const OGroup *g, unsigned i) {
    return o_pos(g, i) + 4;
}

static inline OTag *o_tag(const OGroup *g, unsigned i) {
    return (OTag *)(g->storage + (size_t)g->agent_size * i);
}

/* tay/space.c:9-48: the agents' box over the space's dims, unless the box is fixed */
static void o_update_box(OGroup *g) {
    if (g->box_fixed) {
        for (int i = 0; i < 3; ++i) {
            g->box_min[i] = g->fixed_min[i];
            g->box_max[i] = g->fixed_max[i];
        }
        return;
    }
    for (int i = 0; i < 3; ++i) {
        g->box_min[i] = O_BIG;
        g->box_max[i] = -O_BIG;
    }
    for (unsigned a = 0; a < g->count; ++a) {
        const REAL *p = o_pos(g, a);
        for (int i = 0; i < g->dims; ++i) {
            if (p[i] < g->box_min[i])
                g->box_min[i] = p[i];
            if (p[i] > g->box_max[i])
                g->box_max[i] = p[i];
        }
    }
}

/* 10 bits per axis, x at bit 0 (tay/cpu_z_grid.c:57-77) */
static inline unsigned o_spread10(unsigned v) {
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

static inline unsigned o_morton3(int x, int y, int z) {
    return o_spread10((unsigned)x) | (o_spread10((unsigned)y) << 1) | (o_spread10((unsigned)z) << 2);
}

static inline unsigned o_compact10(unsigned v) {
    v &= 0x09249249u;
    v = (v | (v >> 2)) & 0x030c30c3u;
    v = (v | (v >> 4)) & 0x0300f00fu;
    v = (v | (v >> 8)) & 0xff0000ffu;
    v = (v | (v >> 16)) & 0x000003ffu;
    return v;
}

/* tay/cpu_z_grid.c:12-35, tay/cpu_grid.c:18-40: the first `dims` indices; the others 0 */
static inline void o_cell_indices(const REAL *p, const REAL *o, const REAL *s, int *idx, int dims) {
    for (int i = 0; i < 3; ++i)
        idx[i] = i < dims ? (int)O_FLOOR((p[i] - o[i]) / s[i]) : 0;
}

/* tay/cpu_z_grid.c:156-221 */
static void o_z_grid_sort(OGroup *g) {
    o_update_box(g);
    unsigned n = 0;
    for (int i = 0; i < 3; ++i) {
        REAL cs = g->part[i];
        REAL size = g->box_max[i] - g->box_min[i] + cs * (REAL)0.001;
        unsigned cells = (unsigned)O_FLOOR(size / cs);
        unsigned side_n = 0;
        /* bounded at 30: the reference's loop never ends for extents of 2^31 cells or more */
        while (side_n < 30u && (1u << (side_n + 1u)) <= cells)
            ++side_n;
        if (side_n > n)
            n = side_n;
    }
    for (;;) {
        unsigned side = 1u << (n + 1u);
        if (side * side * side <= g->max_cells)
            break;
        --n;
    }
    for (int i = 0; i < 3; ++i) {
        REAL cs = g->part[i];
        REAL size = g->box_max[i] - g->box_min[i] + cs * (REAL)0.001;
        g->origin[i] = g->box_min[i];
        g->cell_counts[i] = 1 << n;
        g->cell_size[i] = size / (REAL)g->cell_counts[i];
    }
    g->cells_count = (1u << n) * (1u << n) * (1u << n);

    for (unsigned a = 0; a < g->count; ++a) {
        int idx[3];
        o_cell_indices(o_pos(g, a), g->origin, g->cell_size, idx, 3);
        unsigned cell_i = o_morton3(idx[0], idx[1], idx[2]);
        OTag *tag = o_tag(g, a);
        tag->part_i = cell_i;
        tag->cell_agent_i = g->zcells[cell_i].count++;
    }
    unsigned first = 0;
    for (unsigned c = 0; c < g->cells_count; ++c) {
        g->zcells[c].first = first;
        first += g->zcells[c].count;
    }
    for (unsigned a = 0; a < g->count; ++a) {
        OTag *tag = o_tag(g, a);
        unsigned dst = g->zcells[tag->part_i].first + tag->cell_agent_i;
        memcpy(g->sort_storage + (size_t)g->agent_size * dst, tag, g->agent_size);
    }
    char *t = g->storage;
    g->storage = g->sort_storage;
    g->sort_storage = t;
}

/* tay/cpu_grid.c:74-156.  Returns 0, without touching the cells, when the grid has more
 * cells than the structure's memory holds: the reference's shrink step rounds every axis
 * up (tay/cpu_grid.c:100-108), which can leave cells_count above max_cells, and the
 * reference then indexes past its cell array (the 1M-boid workload with 256 MB does this).
 * Every other grid is the reference's, unchanged. */
static int o_grid_sort(OGroup *g) {
    o_update_box(g);
    g->first_gcell = 0;
    unsigned long long cells_count = 1;
    for (int i = 0; i < 3; ++i) {
        g->origin[i] = g->box_min[i];
        g->cell_counts[i] = 1;
        g->cell_size[i] = 1;
    }
    for (int i = 0; i < g->dims; ++i) {
        REAL cs = g->part[i];
        REAL size = g->box_max[i] - g->box_min[i] + cs * (REAL)0.001;
        g->cell_counts[i] = (int)O_CEIL(size / cs);
        g->cell_size[i] = size / (REAL)g->cell_counts[i];
        cells_count *= (unsigned long long)g->cell_counts[i];
    }
    if (cells_count > g->max_cells) {
        REAL volume_ratio = (REAL)cells_count / (REAL)g->max_cells;
        REAL ratio = O_POW(volume_ratio, (REAL)1 / (REAL)g->dims);
        for (int i = 0; i < g->dims; ++i) {
            REAL cs = g->part[i];
            REAL size = g->box_max[i] - g->box_min[i] + cs * (REAL)0.001;
            g->cell_counts[i] = (int)O_CEIL(g->cell_counts[i] / ratio);
            g->cell_size[i] = size / (REAL)g->cell_counts[i];
        }
        unsigned long long shrunk = 1;
        for (int i = 0; i < g->dims; ++i)
            shrunk *= (unsigned long long)g->cell_counts[i];
        if (shrunk > g->max_cells)
            return 0;
    }
    for (unsigned a = 0; a < g->count; ++a) {
        int idx[3];
        o_cell_indices(o_pos(g, a), g->origin, g->cell_size, idx, g->dims);
        unsigned cell_i = (unsigned)(idx[2] * g->cell_counts[0] * g->cell_counts[1] + idx[1] * g->cell_counts[0] + idx[0]);
        OGCell *cell = g->gcells + cell_i;
        if (cell->count == 0) {
            cell->next = g->first_gcell;
            g->first_gcell = cell;
            cell->idx[0] = idx[0];
            cell->idx[1] = idx[1];
            cell->idx[2] = idx[2];
        }
        OTag *tag = o_tag(g, a);
        tag->part_i = cell_i;
        tag->cell_agent_i = cell->count++;
    }
    unsigned first = 0;
    for (OGCell *c = g->first_gcell; c; c = c->next) {
        c->first = first;
        first += c->count;
    }
    for (unsigned a = 0; a < g->count; ++a) {
        OTag *tag = o_tag(g, a);
        unsigned dst = g->gcells[tag->part_i].first + tag->cell_agent_i;
        memcpy(g->sort_storage + (size_t)g->agent_size * dst, tag, g->agent_size);
    }
    char *t = g->storage;
    g->storage = g->sort_storage;
    g->sort_storage = t;
    return 1;
}

static void o_unsort(OGroup *g) {
    if (g->space == O_SPACE_Z_GRID)
        memset(g->zcells, 0, sizeof(OZCell) * g->cells_count); /* tay/cpu_z_grid.c:223-225 */
    else if (g->space == O_SPACE_GRID)
        for (OGCell *c = g->first_gcell; c; c = c->next) /* tay/cpu_grid.c:153-156 */
            c->count = 0;
}

/* ------------------------------------------------------------------ pairing */

/* tay/space.c:106-148; `skip_self` selects space_see_point_point (same group, no
 * self-see) over space_see_point_point_self_see */
static unsigned long long O_NAME(pairs_by_thread)[64];

static unsigned long long o_pair(const OGroup *g, const OGroup *h, const OPass *pass, unsigned seer_beg, unsigned seer_end,
                                 unsigned seen_beg, unsigned seen_end, int skip_self, int dims) {
    unsigned long long pairs = 0;
    for (unsigned s = seer_beg; s < seer_end; ++s) {
        char *seer = g->storage + (size_t)g->agent_size * s;
        const REAL *sp = o_pos(g, s);
        for (unsigned b = seen_beg; b < seen_end; ++b) {
            if (skip_self && s == b)
                continue;
            const REAL *bp = o_pos(h, b);
            int skip = 0;
            if (g->is_point) {
                for (int i = 0; i < dims; ++i) {
                    REAL d = sp[i] - bp[i];
                    if (d < -pass->radii[i] || d > pass->radii[i]) {
                        skip = 1;
                        break;
                    }
                }
            }
            else {
                /* _NONPOINT_NONPOINT_NARROW_PHASE_TEST, tay/space.c:92-103 */
                const REAL *smax = o_max(g, s), *bmax = o_max(h, b);
                for (int i = 0; i < dims; ++i) {
                    if (sp[i] - bmax[i] > pass->radii[i] || bp[i] - smax[i] > pass->radii[i]) {
                        skip = 1;
                        break;
                    }
                }
            }
            if (skip)
                continue;
            ++pairs; /* the reference's narrow-phase counter, tay/space.c:56-60 */
            pass->see(seer, h->storage + (size_t)h->agent_size * b, pass->ctx);
        }
    }
    return pairs;
}

/* neighbour cell index box for a seer box (tay/cpu_z_grid.c:232-247, tay/cpu_grid.c:158-174) */
static void o_index_box(const OGroup *g, const REAL *bmin, const REAL *bmax, int *lo, int *hi, int dims) {
    o_cell_indices(bmin, g->origin, g->cell_size, lo, dims);
    o_cell_indices(bmax, g->origin, g->cell_size, hi, dims);
    for (int i = 0; i < dims; ++i) {
        if (lo[i] < 0) lo[i] = 0;
        if (hi[i] < 0) hi[i] = 0;
        if (lo[i] >= g->cell_counts[i]) lo[i] = g->cell_counts[i] - 1;
        if (hi[i] >= g->cell_counts[i]) hi[i] = g->cell_counts[i] - 1;
    }
}

/* g: the seer (or acting) group, h: the seen group (== g for a single-group pass) */
typedef struct {
    OGroup *g;
    OGroup *h;
    OPass *pass;
    int skip_self;
} OPassArg;

/* tay/cpu_z_grid.c:283-321 (_see_func: seers walked cell run by cell run, seer box = the
 * seer cell's box in the seer group's grid, widened by the radii) and :232-277
 * (cpu_z_grid_see_seen: that box mapped to the seen group's grid); tay/cpu_grid.c:244-281
 * the same on CpuGrid; tay/cpu_simple.c:6-38 against all seen agents. */
static void o_see_task(OTask *task, int thread_i, int threads) {
    OPassArg *arg = (OPassArg *)task->arg;
    OGroup *g = arg->g;
    OGroup *h = arg->h;
    OPass *pass = arg->pass;
    int skip_self = arg->skip_self;
    int dims = g->dims < h->dims ? g->dims : h->dims; /* min_dims, tay/cpu_z_grid.c:289-291 */
    unsigned beg, end;
    o_range(g->count, thread_i, threads, &beg, &end);

    unsigned long long pairs = 0;
    if (g->space == O_SPACE_SIMPLE || h->space == O_SPACE_SIMPLE) {
        O_NAME(pairs_by_thread)[thread_i] += o_pair(g, h, pass, beg, end, 0, h->count, skip_self, dims);
        return;
    }

    unsigned s = beg;
    while (s < end) {
        const OTag *tag = o_tag(g, s);
        int idx[3];
        unsigned run_end;
        if (g->space == O_SPACE_Z_GRID) {
            idx[0] = (int)o_compact10(tag->part_i);
            idx[1] = (int)o_compact10(tag->part_i >> 1);
            idx[2] = (int)o_compact10(tag->part_i >> 2);
            const OZCell *cell = g->zcells + tag->part_i;
            run_end = cell->first + cell->count;
        }
        else {
            const OGCell *cell = g->gcells + tag->part_i;
            idx[0] = cell->idx[0];
            idx[1] = cell->idx[1];
            idx[2] = cell->idx[2];
            run_end = cell->first + cell->count;
        }
        if (run_end > end)
            run_end = end;
        REAL bmin[3] = {0, 0, 0}, bmax[3] = {0, 0, 0};
        for (int i = 0; i < dims; ++i) {
            REAL m = g->origin[i] + idx[i] * g->cell_size[i];
            bmin[i] = m - pass->radii[i];
            bmax[i] = m + g->cell_size[i] + pass->radii[i];
        }
        int lo[3], hi[3];
        o_index_box(h, bmin, bmax, lo, hi, dims);
        for (int x = lo[0]; x <= hi[0]; ++x)
            for (int y = lo[1]; y <= hi[1]; ++y)
                for (int z = lo[2]; z <= hi[2]; ++z) {
                    unsigned first, count;
                    if (h->space == O_SPACE_Z_GRID) {
                        const OZCell *c = h->zcells + o_morton3(x, y, z);
                        first = c->first;
                        count = c->count;
                    }
                    else {
                        const OGCell *c = h->gcells + (z * h->cell_counts[0] * h->cell_counts[1] + y * h->cell_counts[0] + x);
                        first = c->first;
                        count = c->count;
                    }
                    pairs += o_pair(g, h, pass, s, run_end, first, first + count, skip_self, dims);
                }
        s = run_end;
    }
    O_NAME(pairs_by_thread)[thread_i] += pairs;
}

static void o_act_task(OTask *task, int thread_i, int threads) {
    OPassArg *arg = (OPassArg *)task->arg;
    unsigned beg, end;
    o_range(arg->g->count, thread_i, threads, &beg, &end);
    for (unsigned a = beg; a < end; ++a)
        arg->pass->act(arg->g->storage + (size_t)arg->g->agent_size * a, arg->pass->ctx);
}

/* ------------------------------------------------------------------ entry point */

static unsigned o_agent_size(int model) {
    switch (model) {
        case O_MODEL_TEST: return (unsigned)sizeof(OTestAgent);
        case O_MODEL_BOIDS: return (unsigned)sizeof(OBoid);
        case O_MODEL_SPH: return (unsigned)sizeof(OSphParticle);
        case O_MODEL_BOX: return (unsigned)sizeof(OBoxAgent);
        default: return 0;
    }
}

static int o_agent_id(int model, const char *a) {
    switch (model) {
        case O_MODEL_TEST: return ((const OTestAgent *)a)->result_index;
        case O_MODEL_BOIDS: return ((const OBoid *)a)->id;
        case O_MODEL_BOX: return ((const OBoxAgent *)a)->result_index;
        default: return ((const OSphParticle *)a)->id;
    }
}

/* Box-test passes summed over the passes and steps of the last oracle_run. */
unsigned long long O_NAME(oracle_last_pairs)(void) {
    unsigned long long s = 0;
    for (int i = 0; i < 64; ++i)
        s += O_NAME(pairs_by_thread)[i];
    return s;
}

unsigned O_NAME(oracle_agent_size)(int model) {
    return o_agent_size(model);
}

/* Space options of the groups of the following runs (tay_configure_space dims,
 * tay_fix_space_box): dims 3 and no fixed box unless set. */
static int o_opt_dims = 3;
static int o_opt_box_fixed = 0;
static REAL o_opt_min[3], o_opt_max[3];

void O_NAME(oracle_set_space)(int dims, int box_fixed, const REAL *box_min, const REAL *box_max) {
    o_opt_dims = dims;
    o_opt_box_fixed = box_fixed;
    for (int i = 0; i < 3; ++i) {
        o_opt_min[i] = box_fixed ? box_min[i] : 0;
        o_opt_max[i] = box_fixed ? box_max[i] : 0;
    }
}

static void o_group_init(OGroup *g, unsigned agent_size, int space, int n, const void *agents, REAL part_size, int mb) {
    memset(g, 0, sizeof(*g));
    g->dims = o_opt_dims;
    g->is_point = 1;
    g->box_fixed = o_opt_box_fixed;
    for (int i = 0; i < 3; ++i) {
        g->fixed_min[i] = o_opt_min[i];
        g->fixed_max[i] = o_opt_max[i];
    }
    g->agent_size = agent_size;
    g->count = (unsigned)n;
    g->space = space;
    g->part[0] = g->part[1] = g->part[2] = part_size;
    g->storage = (char *)malloc((size_t)agent_size * (n ? n : 1));
    g->sort_storage = (char *)malloc((size_t)agent_size * (n ? n : 1));
    memcpy(g->storage, agents, (size_t)agent_size * n);
    size_t shared = (size_t)mb << 20;
    if (space == O_SPACE_Z_GRID) {
        g->max_cells = (unsigned)(shared / 8u); /* sizeof(ZGridCell), tay/cpu_z_grid.c:7-10,152 */
        g->zcells = (OZCell *)calloc(g->max_cells, sizeof(OZCell));
    }
    else if (space == O_SPACE_GRID) {
        g->max_cells = (unsigned)(shared / 32u); /* sizeof(GridCell) on LP64, tay/cpu_grid.c:6-11,62 */
        g->gcells = (OGCell *)calloc(g->max_cells, sizeof(OGCell));
    }
}

/* Writes the group's records back to `agents` in id order; 0 if an id is out of range. */
static int o_group_finish(OGroup *g, int model, void *agents) {
    int ok = 1;
    for (unsigned a = 0; a < g->count; ++a) {
        const char *rec = g->storage + (size_t)g->agent_size * a;
        int id = o_agent_id(model, rec);
        if (id < 0 || id >= (int)g->count) {
            ok = 0;
            break;
        }
        memcpy((char *)agents + (size_t)g->agent_size * id, rec, g->agent_size);
    }
    free(g->storage);
    free(g->sort_storage);
    free(g->zcells);
    free(g->gcells);
    return ok;
}

/* 0 when the group's structure cannot hold its grid (o_grid_sort). */
static int o_sort(OGroup *g) {
    if (g->space == O_SPACE_Z_GRID)
        o_z_grid_sort(g);
    else if (g->space == O_SPACE_GRID)
        return o_grid_sort(g);
    return 1;
}

static double o_seconds(const struct timespec *t0, const struct timespec *t1) {
    return (double)(t1->tv_sec - t0->tv_sec) + 1e-9 * (double)(t1->tv_nsec - t0->tv_nsec);
}

/* Runs `steps` steps of one model on one group.  Same contract as the reference driver:
 * `agents` holds n AoS records in id order on entry and on return; the pass mask selects
 * which of the model's passes are registered, in the model's order; returns the number
 * of steps run (0 on error) and the wall-clock ms per step (tay/state.c:204-206,317-320). */
int O_NAME(oracle_run)(int model, int space, int n, void *agents, const void *see_ctx, const void *act_ctx,
                       REAL radius, REAL part_size, int mb, int steps, unsigned pass_mask, int threads,
                       double *ms_per_step) {
    unsigned agent_size = o_agent_size(model);
    if (!agent_size || n <= 0 || steps < 0)
        return 0;
    if (space != O_SPACE_SIMPLE && space != O_SPACE_GRID && space != O_SPACE_Z_GRID)
        return 0;
    /* the reference's Z-grid pairs nothing below 3 dims (tay/cpu_z_grid.c:254-260) */
    if (o_opt_dims < 1 || o_opt_dims > 3 || (space == O_SPACE_Z_GRID && o_opt_dims != 3))
        return 0;
    /* grids hold point agents only (tay/state_compile.c: "grid structure can only contain
     * point agents"); box agents run on CpuSimple */
    if (model == O_MODEL_BOX && space != O_SPACE_SIMPLE)
        return 0;
    O_NAME(pool_start)(threads);

    OGroup g;
    o_group_init(&g, agent_size, space, n, agents, part_size, mb);
    g.is_point = model != O_MODEL_BOX;

    /* contexts are copied, as the OpenCL path copies them per run (tay/ocl.c:252-259) */
    OTestActContext test_act;
    OBoidsContext boids;
    OSphContext sph;
    OPass passes[4];
    int passes_count = 0;
    REAL radii[3] = {radius, radius, radius};
    if (model == O_MODEL_TEST || model == O_MODEL_BOX) {
        memcpy(&test_act, act_ctx, sizeof(test_act));
        OSeeFn see = model == O_MODEL_TEST ? o_test_see : o_box_see;
        OActFn act = model == O_MODEL_TEST ? o_test_act : o_box_act;
        if (pass_mask & O_PASS_SEE0)
            passes[passes_count++] = (OPass){1, see, 0, {radii[0], radii[1], radii[2]}, 0, 0};
        if (pass_mask & O_PASS_ACT0)
            passes[passes_count++] = (OPass){0, 0, act, {0, 0, 0}, 0, &test_act};
    }
    else if (model == O_MODEL_BOIDS) {
        memcpy(&boids, see_ctx, sizeof(boids));
        if (pass_mask & O_PASS_SEE0)
            passes[passes_count++] = (OPass){1, o_boids_see, 0, {radii[0], radii[1], radii[2]}, 0, &boids};
        if (pass_mask & O_PASS_ACT0)
            passes[passes_count++] = (OPass){0, 0, o_boids_act, {0, 0, 0}, 0, &boids};
    }
    else {
        memcpy(&sph, see_ctx, sizeof(sph));
        if (pass_mask & O_PASS_SEE0)
            passes[passes_count++] = (OPass){1, o_sph_density, 0, {radii[0], radii[1], radii[2]}, 1, &sph};
        if (pass_mask & O_PASS_ACT0)
            passes[passes_count++] = (OPass){0, 0, o_sph_pressure, {0, 0, 0}, 0, &sph};
        if (pass_mask & O_PASS_SEE1)
            passes[passes_count++] = (OPass){1, o_sph_force, 0, {radii[0], radii[1], radii[2]}, 0, &sph};
        if (pass_mask & O_PASS_ACT1)
            passes[passes_count++] = (OPass){0, 0, o_sph_integrate, {0, 0, 0}, 0, &sph};
    }

    memset(O_NAME(pairs_by_thread), 0, sizeof(O_NAME(pairs_by_thread)));
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    int sorted = 1;
    for (int step = 0; step < steps && sorted; ++step) {
        sorted = o_sort(&g);
        if (!sorted)
            break;
        for (int p = 0; p < passes_count; ++p) {
            OPassArg arg = {&g, &g, passes + p, passes[p].is_see && !passes[p].self_see};
            OTask task = {passes[p].is_see ? o_see_task : o_act_task, &arg};
            O_NAME(pool_run)(&task);
        }
        o_unsort(&g);
    }
    clock_gettime(CLOCK_MONOTONIC, &t1);
    if (ms_per_step)
        *ms_per_step = steps ? o_seconds(&t0, &t1) / steps * 1000.0 : 0.0;
    return o_group_finish(&g, model, agents) && sorted ? steps : 0;
}

/* Runs `steps` steps of a state with several groups of one model (the test model's
 * agent_see / agent_act or the boids' see / act), each group on its own structure of
 * type `space`, with a pass list that mixes groups (tay/state.c:208-316; the combination
 * test's pass list is test/test_combo.c:114-119).  Pass k is a see of group
 * pass_seer[k] over group pass_seen[k] (is_see) or an act of group pass_seer[k]; a see
 * pass skips seer == seen only inside one group and without self_see
 * (tay/state_compile.c:109-120).  agents[g] holds counts[g] records in id order on entry
 * and on return. */
int O_NAME(oracle_run_groups)(int model, int space, int ngroups, const int *counts, void **agents, const void *see_ctx,
                              const void *act_ctx, REAL radius, REAL part_size, int mb, int steps, int npasses,
                              const int *pass_is_see, const int *pass_seer, const int *pass_seen,
                              const int *pass_self_see, int threads, double *ms_per_step) {
    enum { kMaxGroups = 8, kMaxPasses = 32 };
    unsigned agent_size = o_agent_size(model);
    if (!agent_size || ngroups <= 0 || ngroups > kMaxGroups || npasses < 0 || npasses > kMaxPasses || steps < 0)
        return 0;
    if (model != O_MODEL_TEST && model != O_MODEL_BOIDS && model != O_MODEL_BOX)
        return 0;
    if (model == O_MODEL_BOX && space != O_SPACE_SIMPLE)
        return 0;
    if (space != O_SPACE_SIMPLE && space != O_SPACE_GRID && space != O_SPACE_Z_GRID)
        return 0;
    if (o_opt_dims < 1 || o_opt_dims > 3 || (space == O_SPACE_Z_GRID && o_opt_dims != 3))
        return 0;
    for (int k = 0; k < ngroups; ++k)
        if (counts[k] <= 0)
            return 0;
    for (int k = 0; k < npasses; ++k)
        if (pass_seer[k] < 0 || pass_seer[k] >= ngroups || (pass_is_see[k] && (pass_seen[k] < 0 || pass_seen[k] >= ngroups)))
            return 0;
    O_NAME(pool_start)(threads);

    OGroup g[kMaxGroups];
    for (int k = 0; k < ngroups; ++k) {
        o_group_init(g + k, agent_size, space, counts[k], agents[k], part_size, mb);
        g[k].is_point = model != O_MODEL_BOX;
    }
    OTestActContext test_act;
    OBoidsContext boids;
    if (model == O_MODEL_TEST || model == O_MODEL_BOX)
        memcpy(&test_act, act_ctx, sizeof(test_act));
    else
        memcpy(&boids, see_ctx, sizeof(boids));
    OPass passes[kMaxPasses];
    for (int k = 0; k < npasses; ++k) {
        OPass p = {pass_is_see[k], 0, 0, {radius, radius, radius}, pass_self_see[k], 0};
        if (model == O_MODEL_TEST || model == O_MODEL_BOX) {
            p.see = model == O_MODEL_TEST ? o_test_see : o_box_see;
            p.act = model == O_MODEL_TEST ? o_test_act : o_box_act;
            p.ctx = pass_is_see[k] ? 0 : &test_act;
        }
        else {
            p.see = o_boids_see;
            p.act = o_boids_act;
            p.ctx = &boids;
        }
        passes[k] = p;
    }

    memset(O_NAME(pairs_by_thread), 0, sizeof(O_NAME(pairs_by_thread)));
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    int sorted = 1;
    for (int step = 0; step < steps && sorted; ++step) {
        for (int k = 0; k < ngroups; ++k)
            sorted &= o_sort(g + k);
        if (!sorted) {
            for (int k = 0; k < ngroups; ++k)
                o_unsort(g + k);
            break;
        }
        for (int p = 0; p < npasses; ++p) {
            OGroup *seer = g + pass_seer[p];
            OGroup *seen = passes[p].is_see ? g + pass_seen[p] : seer;
            OPassArg arg = {seer, seen, passes + p, passes[p].is_see && seer == seen && !passes[p].self_see};
            OTask task = {passes[p].is_see ? o_see_task : o_act_task, &arg};
            O_NAME(pool_run)(&task);
        }
        for (int k = 0; k < ngroups; ++k)
            o_unsort(g + k);
    }
    clock_gettime(CLOCK_MONOTONIC, &t1);
    if (ms_per_step)
        *ms_per_step = steps ? o_seconds(&t0, &t1) / steps * 1000.0 : 0.0;
    int ok = sorted ? steps : 0;
    for (int k = 0; k < ngroups; ++k)
        if (!o_group_finish(g + k, model, agents[k]))
            ok = 0;
    return ok;
}
