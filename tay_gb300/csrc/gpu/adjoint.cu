// Hand-written adjoint of the SPH step, for batches running the full SPH pass sequence
// (density, pressure, force, integrate).
//
// Forward (recorded): every step runs the normal sort and the density+pressure kernel,
// then a force+integrate kernel that also stores the acceleration; the step's sorted
// state (positions, velocities, {rho, P}, acceleration, global ids), its sorted keys and
// its bounding boxes are recorded.  With checkpoint_every = k > 0 only the state at every
// k-th step is kept and each k-step segment is recomputed, with recording, during the
// backward sweep; with k = 0 every step is recorded during the forward run.
//
// Backward, per step in reverse order, with the forward step's neighbour sets held fixed:
// the cell table is rebuilt from the recorded keys and boxes, then
//   integrate adjoint -> force adjoint (+ pressure adjoint) -> density adjoint
//   -> scatter of the step's input adjoints back to id order,
// and the per-particle parameter gradients are summed per segment in a fixed order
// (deterministic).  Outputs: dL/dx0, dL/dv0 in id order, dL/d(alpha, c0) per segment.
#include <algorithm>
#include <cstring>
#include <vector>

#include "runtime_internal.cuh"

namespace tgpu {
namespace {

enum { A_POS = 0, A_VEL = 1, A_RP = 2, A_ABAR = 3, A_XBAR = 4, A_VBAR = 5, A_RHOBAR = 6, A_THETA = 7 };
constexpr int SPH_POS = 0, SPH_VEL = 1, SPH_RP = 2, SPH_ACC = 3, SPH_ID = 0;

struct Record {
    float4 *pos, *vel, *rp, *acc;
    uint32_t *gid, *keys;
    BoxAcc *box;
};

struct Checkpoint {
    float4 *pos, *vel;
    uint32_t *id;
};

// The pair list of one step of a segment (the batch's list layout, PairList): recorded by
// the step's forward density pass, replayed by its forward force pass and, in the backward
// sweep, by the force and density adjoints.
struct StepList {
    uint4 *idx;
    uint2 *count;
};

// gid[i] = begin(segment of i) + id[i]
__global__ void __launch_bounds__(kSortThreads) gid_kernel(const SegmentSpec *__restrict__ specs,
                                                           const uint32_t *__restrict__ tile_seg,
                                                           const uint32_t *__restrict__ id, uint32_t *__restrict__ gid) {
    const SegmentSpec s = specs[tile_seg[blockIdx.x]];
    const uint32_t t = blockIdx.x - s.tile_begin;
    const uint32_t beg = s.begin + t * kSortTile;
    const uint32_t end = min(beg + (uint32_t)kSortTile, s.begin + s.count);
    for (uint32_t i = beg + threadIdx.x; i < end; i += kSortThreads) gid[i] = s.begin + id[i];
}

// Per-segment sum of the particles' parameter gradients, in a fixed order: one block per
// segment, each thread a strided partial sum, then a shared-memory tree.
__global__ void __launch_bounds__(256) theta_reduce_kernel(const SegmentSpec *__restrict__ specs,
                                                           const float4 *__restrict__ theta, double *__restrict__ acc) {
    __shared__ double sa[256], sc[256];
    const SegmentSpec s = specs[blockIdx.x];
    double a = 0.0, c = 0.0;
    for (uint32_t i = s.begin + threadIdx.x; i < s.begin + s.count; i += 256) {
        const float4 t = theta[i];
        a += (double)t.x;
        c += (double)t.y;
    }
    sa[threadIdx.x] = a;
    sc[threadIdx.x] = c;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) {
            sa[threadIdx.x] += sa[threadIdx.x + o];
            sc[threadIdx.x] += sc[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        acc[2 * blockIdx.x] += sa[0];
        acc[2 * blockIdx.x + 1] += sc[0];
    }
}

}  // namespace
}  // namespace tgpu

struct TgpuAdjoint {
    TgpuBatch *b = nullptr;
    int steps = 0, every = 0;
    int keep = 1;  // trailing segments recorded during the forward run (checkpoint mode)
    const tgpu::SphAdjointKernels *K = nullptr;
    std::vector<tgpu::Record> rec;
    std::vector<tgpu::Checkpoint> cp;  // cp[k] = state before step k*every; last = final state
    // checkpoint mode with pair lists: one list per step of a segment, filled by the forward
    // run for the last segment and by each recomputation for the others
    std::vector<tgpu::StepList> lists;
    float4 *xbar_id = nullptr, *vbar_id = nullptr, *xbar_s = nullptr, *vbar_s = nullptr;
    float4 *abar = nullptr, *rhobar = nullptr, *theta = nullptr;
    double *d_theta = nullptr;
    std::vector<void *> allocs;
    size_t bytes = 0;
    bool recorded = false;
    double fwd_ms = 0.0, bwd_ms = 0.0;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
};

namespace tgpu {
namespace {

template <class T>
int alloc(TgpuAdjoint *a, T **p, size_t count) {
    void *q = nullptr;
    cudaError_t e = cudaMalloc(&q, count * sizeof(T));
    if (e != cudaSuccess) return fail(TGPU_ERR_CUDA, "adjoint: cudaMalloc of %zu bytes failed: %s", count * sizeof(T),
                                      cudaGetErrorString(e));
    a->allocs.push_back(q);
    a->bytes += count * sizeof(T);
    *p = static_cast<T *>(q);
    return TGPU_OK;
}

int alloc_record(TgpuAdjoint *a, Record &r) {
    const size_t n = std::max<uint32_t>(a->b->total, 1);
    int rc = alloc(a, &r.pos, n);
    if (!rc) rc = alloc(a, &r.vel, n);
    if (!rc) rc = alloc(a, &r.rp, n);
    if (!rc) rc = alloc(a, &r.acc, n);
    if (!rc) rc = alloc(a, &r.gid, n);
    if (!rc) rc = alloc(a, &r.keys, n);
    if (!rc) rc = alloc(a, &r.box, (size_t)a->b->nseg);
    return rc;
}

int alloc_checkpoint(TgpuAdjoint *a, Checkpoint &c) {
    const size_t n = std::max<uint32_t>(a->b->total, 1);
    int rc = alloc(a, &c.pos, n);
    if (!rc) rc = alloc(a, &c.vel, n);
    if (!rc) rc = alloc(a, &c.id, n);
    return rc;
}

void save_checkpoint(TgpuBatch *b, const Checkpoint &c) {
    const size_t n = b->total;
    cudaMemcpyAsync(c.pos, b->f4[SPH_POS][b->cur_f4[SPH_POS]], n * sizeof(float4), cudaMemcpyDeviceToDevice, b->st);
    cudaMemcpyAsync(c.vel, b->f4[SPH_VEL][b->cur_f4[SPH_VEL]], n * sizeof(float4), cudaMemcpyDeviceToDevice, b->st);
    cudaMemcpyAsync(c.id, b->u32[SPH_ID][b->cur_u32[SPH_ID]], n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, b->st);
}

void restore_checkpoint(TgpuBatch *b, const Checkpoint &c) {
    const size_t n = b->total;
    cudaMemcpyAsync(b->f4[SPH_POS][b->cur_f4[SPH_POS]], c.pos, n * sizeof(float4), cudaMemcpyDeviceToDevice, b->st);
    cudaMemcpyAsync(b->f4[SPH_VEL][b->cur_f4[SPH_VEL]], c.vel, n * sizeof(float4), cudaMemcpyDeviceToDevice, b->st);
    cudaMemcpyAsync(b->u32[SPH_ID][b->cur_u32[SPH_ID]], c.id, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, b->st);
}

SeeLaunch see_launch(TgpuBatch *b, const KernelRun &r, const PassIO &io) {
    SeeLaunch S{};
    S.specs = b->d_specs;
    S.box = b->d_box;
    S.grids = b->d_grids;
    S.table = b->table;
    S.cta_table = b->d_cta;
    S.radii = r.d_radii;
    S.ctx = r.d_see_ctx;
    S.ctx_stride = (uint32_t)b->ctx_stride;
    S.act_ctx = r.d_act_ctx ? r.d_act_ctx : r.d_see_ctx;
    S.act_ctx_stride = (uint32_t)b->ctx_stride;
    S.ctas = b->ctas;
    S.skip_self = r.skip_self;
    S.stage_cap = 0;
    S.stage_cells = 0;
    S.union_factor = r.union_factor;
    S.rows = b->cell_order == kOrderRows ? 1u : 0u;
    S.hit_masks = b->hit_masks;
    S.err = b->d_err;
    S.pairs = b->d_pairs;
    S.telemetry = nullptr;
    S.io = io;
    return S;
}

// One forward step (the SPH program's kernels, with the acceleration stored), recording
// the step into `r` when given, and its pair list into `pl` when given (else into the
// batch's own list).
void recorded_step(TgpuAdjoint *a, Record *r, const StepList *pl = nullptr) {
    TgpuBatch *b = a->b;
    cudaStream_t st = b->st;
    SortLaunch L = sort_launch(b);
    launch_box(L, st);
    uint32_t *skeys = nullptr, *perm = nullptr;
    launch_sort(L, st, &skeys, &perm);
    GatherSet g{};
    for (int c = 0; c < b->m->nf4; ++c) {
        if (b->m->role_f4[c] != kState) continue;
        g.src_f4[g.nf4] = b->f4[c][b->cur_f4[c]];
        g.dst_f4[g.nf4] = b->f4[c][1 - b->cur_f4[c]];
        b->cur_f4[c] ^= 1;
        ++g.nf4;
    }
    for (int c = 0; c < b->m->nu32; ++c) {
        g.src_u32[g.nu32] = b->u32[c][b->cur_u32[c]];
        g.dst_u32[g.nu32] = b->u32[c][1 - b->cur_u32[c]];
        b->cur_u32[c] ^= 1;
        ++g.nu32;
    }
    launch_cell_table(L, skeys, 1, st, perm, &g);  // and the reorder into cell order
    // density + pressure (recording the batch's pair list, when it keeps one)
    const KernelRun &rd = b->runs[0];
    SeeLaunch SD = see_launch(b, rd, make_io(b, rd.k, true, 0));
    attach_pair_list(b, rd, SD);
    if (pl && SD.plist.mode) {
        SD.plist.idx = pl->idx;
        SD.plist.count = pl->count;
    }
    rd.k->launch_see(SD, 0, st);
    // force + integrate, acceleration stored (replaying the list)
    const KernelRun &rf = b->runs[1];
    PassIO io = make_io(b, rf.k, true, 0);
    const float4 *pos_in = io.in_f4[SPH_POS], *vel_in = io.in_f4[SPH_VEL];
    SeeLaunch SF = see_launch(b, rf, io);
    attach_pair_list(b, rf, SF);
    if (pl && SF.plist.mode) {
        SF.plist.idx = pl->idx;
        SF.plist.count = pl->count;
    }
    a->K->force_record(SF, 0, st);
    for (int c = 0; c < b->m->nf4; ++c)
        if (b->m->role_f4[c] == kState && (rf.k->writes_f4 >> c & 1u) && (rf.k->seen_f4 >> c & 1u)) b->cur_f4[c] ^= 1;
    if (r) {
        const size_t n = b->total;
        cudaMemcpyAsync(r->pos, pos_in, n * sizeof(float4), cudaMemcpyDeviceToDevice, st);
        cudaMemcpyAsync(r->vel, vel_in, n * sizeof(float4), cudaMemcpyDeviceToDevice, st);
        cudaMemcpyAsync(r->rp, b->f4[SPH_RP][0], n * sizeof(float4), cudaMemcpyDeviceToDevice, st);
        cudaMemcpyAsync(r->acc, b->f4[SPH_ACC][0], n * sizeof(float4), cudaMemcpyDeviceToDevice, st);
        cudaMemcpyAsync(r->keys, skeys, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st);
        cudaMemcpyAsync(r->box, b->d_box, (size_t)b->nseg * sizeof(BoxAcc), cudaMemcpyDeviceToDevice, st);
        gid_kernel<<<b->tiles, kSortThreads, 0, st>>>(b->d_specs, b->d_tile_seg, b->u32[SPH_ID][b->cur_u32[SPH_ID]],
                                                      r->gid);
    }
    launch_cell_table(L, skeys, 0, st);
}

// One backward step.  With `pl` (the step's stored pair list) the force adjoint and the
// density adjoint replay it; without, the force adjoint walks and records the batch's list
// for the density adjoint.
void backward_step(TgpuAdjoint *a, const Record &r, const StepList *pl = nullptr) {
    TgpuBatch *b = a->b;
    cudaStream_t st = b->st;
    cudaMemcpyAsync(b->d_box, r.box, (size_t)b->nseg * sizeof(BoxAcc), cudaMemcpyDeviceToDevice, st);
    SortLaunch L = sort_launch(b);
    launch_grids(L, st);  // the recorded step's grids from its restored boxes
    launch_cell_table(L, r.keys, 1, st);

    PassIO io{};
    io.in_f4[A_POS] = io.out_f4[A_POS] = r.pos;
    io.in_f4[A_VEL] = io.out_f4[A_VEL] = r.vel;
    io.in_f4[A_RP] = io.out_f4[A_RP] = r.rp;
    io.in_u32[0] = io.out_u32[0] = r.gid;

    // integrate adjoint: reads the recorded acceleration (slot 3 in) and the id-order
    // adjoints (slots 4, 5 in), writes abar and the sorted partial adjoints
    PassIO ia = io;
    ia.in_f4[A_ABAR] = r.acc;
    ia.out_f4[A_ABAR] = a->abar;
    ia.in_f4[A_XBAR] = a->xbar_id;
    ia.out_f4[A_XBAR] = a->xbar_s;
    ia.in_f4[A_VBAR] = a->vbar_id;
    ia.out_f4[A_VBAR] = a->vbar_s;
    const KernelRun &rd = b->runs[0];
    const KernelRun &rf = b->runs[1];
    ActLaunch A{};
    A.specs = b->d_specs;
    A.tile_seg = b->d_tile_seg;
    A.ctx = rf.d_act_ctx ? rf.d_act_ctx : rf.d_see_ctx;
    A.ctx_stride = (uint32_t)b->ctx_stride;
    A.tiles = b->tiles;
    A.io = ia;
    a->K->integrate_adj(A, st);

    PassIO fa = io;
    fa.in_f4[A_ABAR] = fa.out_f4[A_ABAR] = a->abar;
    fa.in_f4[A_XBAR] = fa.out_f4[A_XBAR] = a->xbar_s;
    fa.in_f4[A_VBAR] = fa.out_f4[A_VBAR] = a->vbar_s;
    fa.in_f4[A_RHOBAR] = fa.out_f4[A_RHOBAR] = a->rhobar;
    fa.in_f4[A_THETA] = fa.out_f4[A_THETA] = a->theta;
    // the force adjoint records the step's pairs for the density adjoint when the batch
    // keeps pair lists for its forward passes (the same cell order and walk conditions)
    SeeLaunch F = see_launch(b, rf, fa);
    SeeLaunch D = see_launch(b, rd, fa);
    D.skip_self = 1;  // the self pair contributes nothing to the density adjoint
    if (pl) {
        // the forward density pass's list: it holds every pair inside the support (and the
        // particle itself, which both adjoints skip)
        F.plist = PairList{pl->idx, pl->count, b->total, b->plist_cap, 2u, rd.d_radii, rd.d_see_ctx};
        D.plist = F.plist;
        a->K->force_adj_replay(F, 0, st);
    } else {
        if (b->plist_idx && rf.skip_self) {
            F.plist = PairList{b->plist_idx, b->plist_count, b->total, b->plist_cap, 1u, nullptr, nullptr};
            D.plist = PairList{b->plist_idx, b->plist_count, b->total, b->plist_cap, 2u, rf.d_radii, rf.d_see_ctx};
        }
        a->K->force_adj(F, 0, st);
    }
    a->K->density_adj(D, 0, st);

    PassIO sa = io;
    sa.in_f4[A_XBAR] = a->xbar_s;
    sa.out_f4[A_XBAR] = a->xbar_id;
    sa.in_f4[A_VBAR] = a->vbar_s;
    sa.out_f4[A_VBAR] = a->vbar_id;
    A.io = sa;
    a->K->scatter_adj(A, st);
    theta_reduce_kernel<<<b->nseg, 256, 0, st>>>(b->d_specs, a->theta, a->d_theta);
    launch_cell_table(L, r.keys, 0, st);
}

}  // namespace
}  // namespace tgpu

using namespace tgpu;

extern "C" {

void tgpu_adjoint_destroy(TgpuAdjoint *a) {
    if (!a) return;
    for (void *p : a->allocs) cudaFree(p);
    if (a->e0) cudaEventDestroy(a->e0);
    if (a->e1) cudaEventDestroy(a->e1);
    delete a;
}

int tgpu_adjoint_create(TgpuBatch *b, int steps, int checkpoint_every, int keep_segments, TgpuAdjoint **out) {
    if (!b || !out || steps <= 0 || checkpoint_every < 0) return fail(TGPU_ERR_ARG, "adjoint: bad arguments");
    *out = nullptr;
    if (b->m != model_sph() || b->program != 3)
        return fail(TGPU_ERR_PROGRAM, "adjoint: the batch must run the full SPH sequence "
                                      "(sph_density, sph_pressure, sph_force, sph_integrate)");
    int rc = prepare_specs(b);
    if (rc) return rc;
    TgpuAdjoint *a = new TgpuAdjoint();
    a->b = b;
    a->steps = steps;
    a->every = checkpoint_every;
    a->K = sph_adjoint_kernels();
    const int segs = checkpoint_every == 0 ? 1 : (steps + checkpoint_every - 1) / checkpoint_every;
    a->keep = checkpoint_every == 0 ? 0 : std::max(1, std::min(keep_segments, segs));
    const int nrec = checkpoint_every == 0 ? steps : std::min(steps, checkpoint_every * a->keep);
    const int ncp = checkpoint_every == 0 ? 1 : (steps + checkpoint_every - 1) / checkpoint_every + 1;
    a->rec.resize(nrec);
    a->cp.resize(ncp);
    const size_t n = std::max<uint32_t>(b->total, 1);
    for (auto &r : a->rec)
        if ((rc = alloc_record(a, r))) break;
    for (auto &c : a->cp)
        if (!rc && (rc = alloc_checkpoint(a, c))) break;
    if (!rc) rc = alloc(a, &a->xbar_id, n);
    if (!rc) rc = alloc(a, &a->vbar_id, n);
    if (!rc) rc = alloc(a, &a->xbar_s, n);
    if (!rc) rc = alloc(a, &a->vbar_s, n);
    if (!rc) rc = alloc(a, &a->abar, n);
    if (!rc) rc = alloc(a, &a->rhobar, n);
    if (!rc) rc = alloc(a, &a->theta, n);
    if (!rc) rc = alloc(a, &a->d_theta, 2 * (size_t)b->nseg);
    // per-step lists of one segment when the batch pairs its density and force passes
    // through a list (checkpoint mode only: a list per step of the whole rollout would not fit)
    if (!rc && checkpoint_every > 0 && b->plist_idx && b->runs.size() == 2 && b->runs[0].list_mode == 1u &&
        b->runs[1].list_mode == 2u) {
        a->lists.resize((size_t)checkpoint_every);
        for (auto &l : a->lists) {
            if ((rc = alloc(a, &l.idx, (size_t)(b->plist_cap / 4u) * n))) break;
            if ((rc = alloc(a, &l.count, n))) break;
        }
    }
    if (!rc && (cudaEventCreate(&a->e0) != cudaSuccess || cudaEventCreate(&a->e1) != cudaSuccess))
        rc = fail(TGPU_ERR_CUDA, "adjoint: cudaEventCreate failed");
    if (rc) {
        tgpu_adjoint_destroy(a);
        return rc;
    }
    *out = a;
    return TGPU_OK;
}

int tgpu_adjoint_forward(TgpuAdjoint *a) {
    if (!a) return fail(TGPU_ERR_ARG, "adjoint: null");
    TgpuBatch *b = a->b;
    int rc = prepare_specs(b);
    if (rc) return rc;
    cudaEventRecord(a->e0, b->st);
    const int segs = a->every == 0 ? 1 : (a->steps + a->every - 1) / a->every;
    const int first_kept = segs - a->keep;  // segments from here on are recorded now
    for (int s = 0; s < a->steps; ++s) {
        if (a->every == 0) {
            if (s == 0) save_checkpoint(b, a->cp[0]);
            recorded_step(a, &a->rec[s]);
        } else {
            const int seg = s / a->every;
            if (s % a->every == 0) save_checkpoint(b, a->cp[seg]);
            // the last segment's lists stay for the first segment of the backward sweep
            const StepList *pl = seg == segs - 1 && !a->lists.empty() ? &a->lists[s % a->every] : nullptr;
            recorded_step(a, seg >= first_kept ? &a->rec[(seg - first_kept) * a->every + s % a->every] : nullptr, pl);
        }
    }
    if (a->every > 0) save_checkpoint(b, a->cp.back());
    cudaEventRecord(a->e1, b->st);
    cudaError_t e = cudaStreamSynchronize(b->st);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) return fail(TGPU_ERR_CUDA, "adjoint forward: %s", cudaGetErrorString(e));
    if (int rc = check_device_error(b)) return rc;
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, a->e0, a->e1);
    a->fwd_ms = ms;
    a->recorded = true;
    return TGPU_OK;
}

int tgpu_adjoint_backward(TgpuAdjoint *a, const float *dl_dpos, const float *dl_dvel, float *dpos0, float *dvel0,
                          double *dparams) {
    if (!a || !a->recorded) return fail(TGPU_ERR_ARG, "adjoint: run tgpu_adjoint_forward first");
    TgpuBatch *b = a->b;
    const size_t n = b->total;
    cudaStream_t st = b->st;
    cudaMemsetAsync(a->xbar_id, 0, n * sizeof(float4), st);
    cudaMemsetAsync(a->vbar_id, 0, n * sizeof(float4), st);
    if (dl_dpos) cudaMemcpyAsync(a->xbar_id, dl_dpos, n * sizeof(float4), cudaMemcpyHostToDevice, st);
    if (dl_dvel) cudaMemcpyAsync(a->vbar_id, dl_dvel, n * sizeof(float4), cudaMemcpyHostToDevice, st);
    cudaMemsetAsync(a->d_theta, 0, 2 * (size_t)b->nseg * sizeof(double), st);
    cudaEventRecord(a->e0, st);
    if (a->every == 0) {
        for (int s = a->steps - 1; s >= 0; --s) backward_step(a, a->rec[s]);
    } else {
        const int segs = (a->steps + a->every - 1) / a->every;
        const int first_kept = segs - a->keep;
        for (int k = segs - 1; k >= 0; --k) {
            const int first = k * a->every;
            const int len = std::min(a->every, a->steps - first);
            int base = 0;
            // stored pair lists: the last segment's from the forward run, a recomputed
            // segment's from its recomputation; other kept segments walk
            const bool lists = !a->lists.empty() && (k == segs - 1 || k < first_kept);
            if (k >= first_kept) {
                base = (k - first_kept) * a->every;  // recorded by the forward run
            } else {
                restore_checkpoint(b, a->cp[k]);  // recompute the segment, recording it
                for (int s = 0; s < len; ++s) recorded_step(a, &a->rec[s], lists ? &a->lists[s] : nullptr);
            }
            for (int s = len - 1; s >= 0; --s) backward_step(a, a->rec[base + s], lists ? &a->lists[s] : nullptr);
        }
        restore_checkpoint(b, a->cp.back());  // the batch ends where the forward run ended
        // a recomputed segment was recorded over the first kept segment's records (and its
        // lists over the last segment's): another backward needs another forward run
        if (first_kept > 0) a->recorded = false;
    }
    cudaEventRecord(a->e1, st);
    if (dpos0) cudaMemcpyAsync(dpos0, a->xbar_id, n * sizeof(float4), cudaMemcpyDeviceToHost, st);
    if (dvel0) cudaMemcpyAsync(dvel0, a->vbar_id, n * sizeof(float4), cudaMemcpyDeviceToHost, st);
    if (dparams)
        cudaMemcpyAsync(dparams, a->d_theta, 2 * (size_t)b->nseg * sizeof(double), cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) return fail(TGPU_ERR_CUDA, "adjoint backward: %s", cudaGetErrorString(e));
    if (int rc = check_device_error(b)) return rc;
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, a->e0, a->e1);
    a->bwd_ms = ms;
    return TGPU_OK;
}

double tgpu_adjoint_forward_ms(const TgpuAdjoint *a) { return a ? a->fwd_ms : 0.0; }
double tgpu_adjoint_backward_ms(const TgpuAdjoint *a) { return a ? a->bwd_ms : 0.0; }
unsigned long long tgpu_adjoint_device_bytes(const TgpuAdjoint *a) { return a ? a->bytes : 0ull; }

}  // extern "C"
