// Batch runtime behind the C ABI in include/tay_gpu.h.
//
// Owns the device buffers of a batch of segments, resolves the registered passes to a
// device model and its fused kernels, and enqueues each step as:
//   bounding box + grid -> keys + radix passes -> cell table -> reorder of the state
//   streams -> the model's pass kernels -> cell table clear
// (the step of tay/state.c:221-311: sort every group, run the passes in order, unsort).
// Steps are captured once per buffer-parity pattern into CUDA graphs and replayed.
#include <dlfcn.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "runtime_internal.cuh"

namespace {
thread_local std::string g_err;
}  // namespace

namespace tgpu {

int fail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

}  // namespace tgpu

namespace {

#define CK(call)                                                                                          \
    do {                                                                                                  \
        cudaError_t e_ = (call);                                                                          \
        if (e_ != cudaSuccess)                                                                            \
            return fail(TGPU_ERR_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
    } while (0)

TgpuTuning default_tuning() {
    TgpuTuning t;
    t.stage = 0;
    t.stage_cap = 0;
    t.stage_cells = 0;
    t.cell_multiple = 1.0f;
    t.union_factor = 1;
    t.use_graphs = 1;
    // row order with x cells of half the y / z cell: the autotuner's choice for every
    // workload measured on GB300 (boids, SPH, batched states)
    t.cell_order = 1;
    t.hit_masks = 0;
    t.x_cell_factor = 0.5f;
    // 251 lattice neighbours lie inside the SPH benchmark's support (2h = 4 spacings),
    // with room for compression
    t.pair_list_cap = 320;
    return t;
}
TgpuTuning g_tuning = default_tuning();

// Models a host registered (tgpu_register_model): kept for the life of the process, looked
// up after the library's own.
std::mutex g_models_lock;
std::vector<const ModelDesc *> g_registered;

const ModelDesc *model_list(int i) {
    switch (i) {
        case 0: return model_test_basic();
        case 1: return model_boids();
        case 2: return model_sph();
        case 3: return model_box();
        default: {
            std::lock_guard<std::mutex> guard(g_models_lock);
            const size_t k = (size_t)(i - 4);
            return i >= 4 && k < g_registered.size() ? g_registered[k] : nullptr;
        }
    }
}

bool model_has_func(const ModelDesc *m, const char *name) {
    for (int k = 0; k < m->nkernels; ++k) {
        const KernelDesc &d = m->kernels[k];
        if ((d.see && !strcmp(d.see, name)) || (d.act && !strcmp(d.act, name))) return true;
    }
    return false;
}

const ModelDesc *find_model(const char *name) {
    for (int i = 0; const ModelDesc *m = model_list(i); ++i)
        if (model_has_func(m, name)) return m;
    return nullptr;
}

uint32_t next_pow2(uint32_t v) {
    uint32_t p = 1;
    while (p < v) p <<= 1;
    return p;
}

uint32_t log2u(uint32_t v) {
    uint32_t n = 0;
    while ((1u << n) < v) ++n;
    return n;
}

}  // namespace

namespace {

void free_batch(TgpuBatch *b) {
    if (!b) return;
    for (auto &kv : b->graphs) cudaGraphExecDestroy(kv.second);
    cudaFree(b->d_specs);
    cudaFree(b->d_extent);
    cudaFree(b->d_tile_seg);
    cudaFree(b->d_cta);
    cudaFree(b->d_box);
    cudaFree(b->d_grids);
    for (int c = 0; c < kMaxF4; ++c)
        for (int k = 0; k < 2; ++k) cudaFree(b->f4[c][k]);
    for (int c = 0; c < kMaxU32; ++c)
        for (int k = 0; k < 2; ++k) cudaFree(b->u32[c][k]);
    for (int k = 0; k < 2; ++k) {
        cudaFree(b->keys[k]);
        cudaFree(b->vals[k]);
    }
    cudaFree(b->sort_scratch);
    cudaFree(b->d_status);  // also the error word, the pair counter and the telemetry
    cudaFreeHost(b->h_status);
    cudaFreeHost(b->h_extent);
    cudaFree(b->table);
    cudaFree(b->d_aos);
    cudaFree(b->plist_idx);
    cudaFree(b->plist_count);
    for (auto &r : b->runs) {
        cudaFree(r.d_radii);
        cudaFree(r.d_see_ctx);
        cudaFree(r.d_act_ctx);
    }
    if (b->e0) cudaEventDestroy(b->e0);
    if (b->e1) cudaEventDestroy(b->e1);
    cudaFree(b->d_wt);
    if (b->st) cudaStreamDestroy(b->st);
    delete b;
}

// Matches a group's pass list against the model's supported sequences.
int match_program(const ModelDesc *m, const TgpuGroup &g) {
    for (int p = 0; p < m->nprograms; ++p) {
        const ProgramDesc &pd = m->programs[p];
        if (pd.passes != g.pass_count) continue;
        bool ok = true;
        for (int k = 0; k < pd.passes && ok; ++k) ok = !strcmp(pd.names[k], g.passes[k].func_name);
        if (ok) return p;
    }
    return -1;
}

int pass_index(const TgpuGroup &g, const char *name, int from) {
    for (int k = from; k < g.pass_count; ++k)
        if (!strcmp(g.passes[k].func_name, name)) return k;
    return -1;
}

// See radii of a pass as the kernels use them: the reference's box test skips the axes
// beyond the space's dims (tay/space.c:62-68), here those radii are +inf.
float4 pass_radii(const TgpuPass &tp, int dims) {
    const float inf = INFINITY;
    return make_float4(tp.radii[0], dims > 1 ? tp.radii[1] : inf, dims > 2 ? tp.radii[2] : inf, tp.radii[3]);
}

}  // namespace

// Reads and clears the device error word; kernels never trap, they record failures there.
int tgpu::check_device_error(TgpuBatch *b) {
    uint32_t err = 0;
    CK(cudaMemcpy(&err, b->d_err, sizeof(err), cudaMemcpyDeviceToHost));
    if (!err) return TGPU_OK;
    CK(cudaMemset(b->d_err, 0, sizeof(err)));
    return fail(TGPU_ERR_DEVICE, "device error 0x%x%s", err,
                (err & kErrSortLookback) ? " (radix sort look-back wait ran out)"
        : (err & kErrStageWait) ? " (a see CTA's wait for its bulk copies ran out)"
        : (err & kErrStageRange) ? " (a see lane's row range fell outside the staged run)" : "");
}

namespace {

// Device address of page-locked host memory (the kernels then read or write the records
// in place, one pass over the host link instead of a copy plus a pass), or nullptr for
// pageable memory, which goes through the device staging buffer.
void *pinned_device_ptr(const void *host) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, host) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

int upload_contexts(TgpuBatch *b, int seg) {
    std::vector<char> buf(b->ctx_stride);
    const HostSeg &h = b->hs[seg];
    if (b->ctx_shadow.size() != b->runs.size() * 3 * (size_t)b->nseg) b->ctx_shadow.assign(b->runs.size() * 3 * b->nseg, {});
    bool copied = false;
    // uploads `bytes` to `dst` unless they equal what the last upload to that slot sent
    auto upload = [&](size_t slot, void *dst, const void *src, size_t bytes) -> cudaError_t {
        std::string &shadow = b->ctx_shadow[slot * b->nseg + seg];
        if (shadow.size() == bytes && !memcmp(shadow.data(), src, bytes)) return cudaSuccess;
        shadow.assign(static_cast<const char *>(src), bytes);
        copied = true;
        return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, b->st);
    };
    for (size_t k = 0; k < b->runs.size(); ++k) {
        const KernelRun &r = b->runs[k];
        for (int which = 0; which < 2; ++which) {
            int p = which == 0 ? r.see_pass : r.act_pass;
            char *dst = which == 0 ? r.d_see_ctx : r.d_act_ctx;
            if (p < 0 || !dst) continue;
            std::fill(buf.begin(), buf.end(), 0);
            const TgpuPass &tp = h.passes[p];
            if (tp.context && tp.context_size)
                memcpy(buf.data(), tp.context, std::min((size_t)tp.context_size, b->ctx_stride));
            CK(upload(3 * k + (size_t)which, dst + (size_t)seg * b->ctx_stride, buf.data(), b->ctx_stride));
        }
        if (r.see_pass >= 0) {
            const TgpuPass &tp = h.passes[r.see_pass];
            float4 rr = pass_radii(tp, seg_dims(b->specs[seg]));
            CK(upload(3 * k + 2, r.d_radii + seg, &rr, sizeof(float4)));
        }
    }
    if (copied) CK(cudaStreamSynchronize(b->st));
    return TGPU_OK;
}

// Per-segment grid bounds from the pushed agents: each axis gets a power-of-two cell
// budget with 10% headroom over the pushed extent (bounded to 1024, the 10-bit Morton
// limit); the dense table gets at most shared_megabytes of uint2 entries.
}  // namespace

int tgpu::prepare_specs(TgpuBatch *b) {
    if (!b->specs_dirty) return TGPU_OK;
    b->specs_dirty = false;
    std::vector<SegmentSpec> next = b->specs;
    uint64_t table_total = 0;
    uint32_t max_key_bits = 3;
    for (int s = 0; s < b->nseg; ++s) {
        SegmentSpec &sp = next[s];
        const HostSeg &h = b->hs[s];
        uint32_t want[3] = {2, 2, 2};
        for (int a = 0; a < seg_dims(sp); ++a) {
            float lo = h.g.box_fixed ? h.g.box_min[a] : h.host_min[a];
            float hi = h.g.box_fixed ? h.g.box_max[a] : h.host_max[a];
            float ext = hi > lo ? hi - lo : 0.0f;
            double cells = floor((double)ext / (double)sp.part[a]) + 1.0;
            want[a] = std::min(1024u, next_pow2((uint32_t)std::min(1024.0, std::max(2.0, ceil(cells * 1.1)))));
        }
        // Morton order: one bound for all axes; row order: each axis its own bound, so
        // that the key takes the bits the three budgets need and no more
        const bool rows = b->cell_order == kOrderRows;
        const uint32_t axis = rows ? want[0] : std::max(want[0], std::max(want[1], want[2]));
        sp.axis_cells_max = axis;
        sp.axis_cells_y = rows ? want[1] : axis;
        sp.axis_cells_z = rows ? want[2] : axis;
        const uint32_t seg_key_bits = log2u(axis) + log2u(sp.axis_cells_y) + log2u(sp.axis_cells_z);
        uint64_t cap_mem = ((uint64_t)std::max(h.g.shared_megabytes, 1) << 20) / sizeof(uint2);
        uint64_t cap_axis = (uint64_t)axis * sp.axis_cells_y * sp.axis_cells_z;
        uint64_t cap = std::min(cap_mem, cap_axis);
        cap = std::max<uint64_t>(cap, 8);
        cap = std::min<uint64_t>(cap, 0x7FFFFFFEull);
        cap = (cap + 1) & ~1ull;  // even: every segment's table starts 16-byte aligned (row headers)
        // row order: headers for up to y x z bound rows, at most a quarter of the table
        sp.row_cap = rows ? (uint32_t)std::max<uint64_t>(
                                1, std::min<uint64_t>((uint64_t)sp.axis_cells_y * sp.axis_cells_z, cap / 4))
                          : 0u;
        sp.table_base = (uint32_t)table_total;
        sp.table_cap = (uint32_t)cap;
        table_total += cap;
        max_key_bits = std::max(max_key_bits, seg_key_bits);
    }
    if (table_total > 0xFFFFFFFFull)
        return fail(TGPU_ERR_ARG, "cell tables too large (%llu entries)", (unsigned long long)table_total);
    const uint32_t key_bits = max_key_bits;
    const bool same = b->table && key_bits == b->key_bits &&
                      !memcmp(next.data(), b->specs.data(), sizeof(SegmentSpec) * b->nseg);
    if (same) return TGPU_OK;  // the table is left clean by every completed step
    b->specs = next;
    b->key_bits = key_bits;
    if (table_total > b->table_entries) {
        cudaFree(b->table);
        b->table = nullptr;
        b->table_entries = 0;
        CK(cudaMalloc(&b->table, table_total * sizeof(uint2)));
        b->table_entries = table_total;
    }
    CK(cudaMemsetAsync(b->table, 0, b->table_entries * sizeof(uint2), b->st));
    CK(cudaMemcpyAsync(b->d_specs, b->specs.data(), sizeof(SegmentSpec) * b->nseg, cudaMemcpyHostToDevice, b->st));
    for (auto &kv : b->graphs) cudaGraphExecDestroy(kv.second);
    b->graphs.clear();
    // box reset, bounding box (+ grids), keys and histograms (+ digit offsets), one kernel
    // per radix pass, cell table (+ reorder), the passes, and the table clear when it is
    // a kernel (Morton order, or more segments than separate header memsets)
    const int passes = sort_passes(b->key_bits);
    const bool clear_kernel = b->cell_order != kOrderRows || b->nseg > kMemsetClearSegments;
    b->launches_per_step = 2 + 1 + passes + 1 + (int)b->runs.size() + (clear_kernel ? 1 : 0);
    return TGPU_OK;
}

PassIO tgpu::make_io(TgpuBatch *b, const KernelDesc *k, bool fused_see, uint32_t offset) {
    PassIO io{};
    for (int c = 0; c < b->m->nf4; ++c) {
        if (b->m->role_f4[c] == kState) {
            io.in_f4[c] = b->f4[c][b->cur_f4[c]] + offset;
            if (k && (k->writes_f4 >> c & 1u)) {
                bool alt = fused_see && (k->seen_f4 >> c & 1u);
                io.out_f4[c] = b->f4[c][alt ? 1 - b->cur_f4[c] : b->cur_f4[c]] + offset;
            } else {
                io.out_f4[c] = b->f4[c][b->cur_f4[c]] + offset;
            }
        } else {
            io.in_f4[c] = b->f4[c][0] + offset;
            io.out_f4[c] = b->f4[c][0] + offset;
        }
    }
    for (int c = 0; c < b->m->nu32; ++c) {
        io.in_u32[c] = b->u32[c][b->cur_u32[c]] + offset;
        io.out_u32[c] = b->u32[c][b->cur_u32[c]] + offset;
    }
    return io;
}

SortLaunch tgpu::sort_launch(TgpuBatch *b) {
    SortLaunch L{};
    L.specs = b->d_specs;
    L.tile_seg = b->d_tile_seg;
    L.box = b->d_box;
    L.pos = b->f4[0][b->cur_f4[0]];
    L.pos_max = b->m->nonpoint ? b->f4[1][b->cur_f4[1]] : nullptr;
    L.keys[0] = b->keys[0];
    L.keys[1] = b->keys[1];
    L.vals[0] = b->vals[0];
    L.vals[1] = b->vals[1];
    L.sort_scratch = b->sort_scratch;
    L.err = b->d_err;
    L.table = b->table;
    L.grids = b->d_grids;
    L.segments = (uint32_t)b->nseg;
    L.tiles = b->tiles;
    L.key_bits = b->key_bits;
    return L;
}

namespace {

void mark(const StepEvents *e, int k, cudaStream_t st) {
    if (e) cudaEventRecord(e->ev[k], st);
}

// The model's unpack program for fetched records: the batch's program, or for state
// batches 0 (accumulators visible) unless an act pass consumed them.
uint32_t unpack_program(const TgpuBatch *b) {
    uint32_t program = (uint32_t)b->program;
    if (!b->state_passes.empty()) {
        program = 0u;
        for (const auto &p : b->state_passes)
            if (!p.pass.is_see) program = 0xFFFFFFFFu;
    }
    return program;
}

// Records [lo, hi) of the batch (current buffers) into the write-through host copies of
// the segments they belong to.
void unpack_range(TgpuBatch *b, uint32_t lo, uint32_t hi, cudaStream_t st) {
    const uint32_t words = b->m->agent_bytes / 4;
    for (int s = 0; s < b->nseg; ++s) {
        if (!b->wt_dev[s]) continue;
        const SegmentSpec &sp = b->specs[s];
        const uint32_t a = max(lo, sp.begin), e = min(hi, sp.begin + sp.count);
        if (a >= e) continue;
        b->m->unpack(b->wt_dev[s] + (size_t)(a - sp.begin) * words, e - a, make_io(b, nullptr, false, a),
                     unpack_program(b), st);
    }
}

}  // namespace

void tgpu::attach_pair_list(const TgpuBatch *b, const KernelRun &r, SeeLaunch &S) {
    if (!r.list_mode) return;
    S.plist.idx = b->plist_idx;
    S.plist.count = b->plist_count;
    S.plist.stride = b->total;
    S.plist.cap = b->plist_cap;
    S.plist.mode = r.list_mode;
    if (r.list_mode == 2u) {
        S.plist.rec_radii = b->runs[r.list_src].d_radii;
        S.plist.rec_ctx = b->runs[r.list_src].d_see_ctx;
    }
}

void tgpu::enqueue_step(TgpuBatch *b, const StepEvents *E, bool write_through) {
    if (b->total == 0 || b->tiles == 0) return;
    cudaStream_t st = b->st;
    SortLaunch L = sort_launch(b);
    mark(E, 0, st);
    launch_box(L, st);
    mark(E, 1, st);
    uint32_t *skeys = nullptr, *perm = nullptr;
    mark(E, 2, st);
    launch_sort(L, st, &skeys, &perm);
    mark(E, 3, st);
    GatherSet g{};
    for (int c = 0; c < b->m->nf4; ++c) {
        if (b->m->role_f4[c] != kState) continue;
        g.src_f4[g.nf4] = b->f4[c][b->cur_f4[c]];
        g.dst_f4[g.nf4] = b->f4[c][1 - b->cur_f4[c]];
        b->cur_f4[c] ^= 1;
        ++g.nf4;
    }
    for (int c = 0; c < b->m->nu32; ++c) {
        if (b->m->role_u32[c] != kState) continue;
        g.src_u32[g.nu32] = b->u32[c][b->cur_u32[c]];
        g.dst_u32[g.nu32] = b->u32[c][1 - b->cur_u32[c]];
        b->cur_u32[c] ^= 1;
        ++g.nu32;
    }
    // the cell table and the reorder into cell order, one launch
    mark(E, 4, st);
    launch_cell_table(L, skeys, 1, st, perm, &g);
    mark(E, 5, st);
    mark(E, 6, st);
    mark(E, 7, st);

    int kidx = 0;
    bool written = false;
    for (auto &r : b->runs) {
        mark(E, 8 + 2 * kidx, st);
        const bool see = r.k->see != nullptr;
        const bool last = kidx + 1 == (int)b->runs.size();
        PassIO io = make_io(b, r.k, see, 0);
        if (see) {
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
            S.stage_cap = r.stage_cap;
            S.stage_cells = r.stage_cells;
            S.union_factor = r.union_factor;
            S.rows = b->cell_order == kOrderRows ? 1u : 0u;
            S.hit_masks = b->hit_masks;
            S.err = b->d_err;
            if (r.seer_seg >= 0) {
                // one seer segment; the seen agents are another segment's (or its own)
                S.cta_offset = b->cta_begin[r.seer_seg];
                S.ctas = b->cta_begin[r.seer_seg + 1] - b->cta_begin[r.seer_seg];
                S.cross = r.seen_seg != r.seer_seg ? 1u : 0u;
                S.seen_seg = (uint32_t)r.seen_seg;
            }
            S.pairs = b->d_pairs;
            S.telemetry = b->d_telemetry;
            S.io = io;
            attach_pair_list(b, r, S);
            // Write-through on the final pass over every segment: each CTA stores its seers'
            // finished records to the host as it ends, so the host link overlaps the pass.
            if (write_through && last && r.seer_seg < 0) {
                S.wt = b->d_wt;
                S.wt_program = unpack_program(b);
            }
            // a pass without a record codec does not write through; the records are then
            // unpacked after the step
            if (r.k->launch_see(S, r.smem, st) && S.wt) written = true;
            for (int c = 0; c < b->m->nf4; ++c)
                if (b->m->role_f4[c] == kState && (r.k->writes_f4 >> c & 1u) && (r.k->seen_f4 >> c & 1u))
                    b->cur_f4[c] ^= 1;
        } else {
            ActLaunch A{};
            A.specs = b->d_specs;
            A.tile_seg = b->d_tile_seg;
            A.ctx = r.d_act_ctx;
            A.ctx_stride = (uint32_t)b->ctx_stride;
            A.tiles = b->tiles;
            if (r.seer_seg >= 0) {
                A.tile_offset = b->specs[r.seer_seg].tile_begin;
                A.tiles = b->specs[r.seer_seg].tile_count;
            }
            A.io = io;
            r.k->launch_act(A, st);
        }
        mark(E, 9 + 2 * kidx, st);
        ++kidx;
    }
    // write-through when the last pass is not one see over every segment: after the step
    if (write_through && !written) unpack_range(b, 0, b->total, st);
    if (E) cudaEventRecord(E->ev2[0], st);
    if (b->cell_order == kOrderRows && b->nseg <= kMemsetClearSegments) {
        // row order: zeroing each segment's header region clears every row (entries are
        // read only inside a row's span), one short memset instead of a pass over the keys
        for (int s = 0; s < b->nseg; ++s)
            cudaMemsetAsync(b->table + b->specs[s].table_base, 0, (size_t)b->specs[s].row_cap * sizeof(uint4), st);
    } else {
        launch_cell_table(L, skeys, 0, st);
    }
    if (E) cudaEventRecord(E->ev2[1], st);
}

namespace {

// Graph-cache key bit of a step that writes its records through to the host.
constexpr uint64_t kWriteThroughGraph = 1ull << 62;

uint64_t parity_signature(const TgpuBatch *b) {
    uint64_t s = 0;
    for (int c = 0; c < kMaxF4; ++c) s |= (uint64_t)b->cur_f4[c] << c;
    for (int c = 0; c < kMaxU32; ++c) s |= (uint64_t)b->cur_u32[c] << (kMaxF4 + c);
    return s;
}

// Host-side buffer parity after one step, mirroring the flips enqueue_step makes (used
// when a captured step is replayed instead of re-enqueued).
void advance_parity(TgpuBatch *b) {
    for (int c = 0; c < b->m->nf4; ++c)
        if (b->m->role_f4[c] == kState) b->cur_f4[c] ^= 1;
    for (int c = 0; c < b->m->nu32; ++c)
        if (b->m->role_u32[c] == kState) b->cur_u32[c] ^= 1;
    for (auto &r : b->runs)
        if (r.k->see)
            for (int c = 0; c < b->m->nf4; ++c)
                if (b->m->role_f4[c] == kState && (r.k->writes_f4 >> c & 1u) && (r.k->seen_f4 >> c & 1u))
                    b->cur_f4[c] ^= 1;
}

}  // namespace

// ------------------------------------------------------------------ C ABI

extern "C" {

const char *tgpu_last_error(void) { return g_err.c_str(); }

int tgpu_batch_telemetry(const TgpuBatch *b, unsigned long long *out, int n) {
    if (!b || !out) return fail(TGPU_ERR_ARG, "bad telemetry");
    for (int k = 0; k < n && k < 8; ++k) out[k] = b->last_telemetry[k];
    return TGPU_OK;
}

unsigned long long tgpu_batch_device_bytes(const TgpuBatch *b) {
    if (!b) return 0ull;
    const unsigned long long n = b->total ? b->total : 1;
    unsigned long long bytes = 0;
    for (int c = 0; c < b->m->nf4; ++c) bytes += n * 16ull * (b->m->role_f4[c] == kState ? 2 : 1);
    bytes += n * 4ull * 2 * b->m->nu32;
    bytes += n * 4ull * 4;  // keys, permutation (ping-pong)
    bytes += 256ull * 4 * (b->tiles ? b->tiles : 1);
    bytes += b->table_entries * sizeof(uint2);
    bytes += n * b->m->agent_bytes;
    if (b->plist_idx) bytes += n * (4ull * b->plist_cap + sizeof(uint2));
    return bytes;
}

int tgpu_batch_kernel_classes(const TgpuBatch *b) { return b ? 4 + (int)b->runs.size() : 0; }

int tgpu_batch_profile(TgpuBatch *b, int steps, double *ms, int n) {
    if (!b || steps < 0 || !ms) return fail(TGPU_ERR_ARG, "bad profile");
    int rc = prepare_specs(b);
    if (rc) return rc;
    const int classes = 4 + (int)b->runs.size();
    std::vector<cudaEvent_t> ev(2 * classes), ev2(2);
    for (auto &e : ev) CK(cudaEventCreate(&e));
    for (auto &e : ev2) CK(cudaEventCreate(&e));
    StepEvents E{ev.data(), ev2.data()};
    for (int s = 0; s < steps; ++s) {
        enqueue_step(b, &E);
        CK(cudaStreamSynchronize(b->st));
        for (int k = 0; k < classes && k < n; ++k) {
            float t = 0.0f;
            CK(cudaEventElapsedTime(&t, ev[2 * k], ev[2 * k + 1]));
            ms[k] += t;
        }
        float t = 0.0f;
        CK(cudaEventElapsedTime(&t, ev2[0], ev2[1]));
        if (n > 2) ms[2] += t;
    }
    for (auto &e : ev) cudaEventDestroy(e);
    for (auto &e : ev2) cudaEventDestroy(e);
    CK(cudaGetLastError());
    return TGPU_OK;
}

int tgpu_batch_flush_l2(TgpuBatch *b) {
    if (!b) return fail(TGPU_ERR_ARG, "null batch");
    static void *scratch = nullptr;
    static size_t scratch_bytes = 0;
    int dev = 0, l2 = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev));
    const size_t want = std::max<size_t>(2 * (size_t)l2, 256u << 20);
    if (scratch_bytes < want) {
        cudaFree(scratch);
        scratch = nullptr;
        scratch_bytes = 0;
        CK(cudaMalloc(&scratch, want));
        scratch_bytes = want;
    }
    CK(cudaMemsetAsync(scratch, (int)(b->total & 0xFF), scratch_bytes, b->st));
    return TGPU_OK;
}

void *tgpu_host_alloc(unsigned long long bytes) {
    void *p = nullptr;
    if (bytes == 0) bytes = 1;
    if (cudaHostAlloc(&p, (size_t)bytes, cudaHostAllocDefault) == cudaSuccess) {
        memset(p, 0, (size_t)bytes);
        return p;
    }
    cudaGetLastError();
    // no usable device: ordinary memory, tagged so tgpu_host_free can tell them apart
    unsigned char *q = (unsigned char *)calloc(1, (size_t)bytes + 64);
    if (!q) return nullptr;
    q[0] = 0xA5;
    return q + 64;
}

void tgpu_host_free(void *ptr) {
    if (!ptr) return;
    cudaPointerAttributes attr;
    if (cudaPointerGetAttributes(&attr, ptr) == cudaSuccess && attr.type == cudaMemoryTypeHost) {
        cudaFreeHost(ptr);
        return;
    }
    cudaGetLastError();
    free((unsigned char *)ptr - 64);
}

int tgpu_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

void tgpu_set_tuning(const TgpuTuning *t) {
    g_tuning = t ? *t : default_tuning();
    if (!(g_tuning.cell_multiple > 0.0f)) g_tuning.cell_multiple = 1.0f;
    if (!(g_tuning.x_cell_factor > 0.0f)) g_tuning.x_cell_factor = 1.0f;
    if (!g_tuning.union_factor) g_tuning.union_factor = 1;
}

void tgpu_get_tuning(TgpuTuning *t) {
    if (t) *t = g_tuning;
}

// A host-built model: checked field by field before it joins the registry, so that a
// descriptor built against another layout or with missing launchers is refused here rather
// than failing inside a run.
int tgpu_register_model(const void *desc, unsigned abi) {
    if (!desc) return fail(TGPU_ERR_ARG, "tgpu_register_model: null descriptor");
    if (abi != kModelAbi)
        return fail(TGPU_ERR_ARG, "tgpu_register_model: descriptor built for model ABI 0x%08x, library has 0x%08x",
                    abi, kModelAbi);
    const ModelDesc *m = static_cast<const ModelDesc *>(desc);
    if (!m->name || !m->name[0]) return fail(TGPU_ERR_ARG, "tgpu_register_model: model without a name");
    if (m->agent_bytes < 24 || m->agent_bytes % 4)
        return fail(TGPU_ERR_ARG, "model '%s': records of %u bytes (a multiple of 4, at least the tag and the position)",
                    m->name, m->agent_bytes);
    if (m->nf4 < 1 || m->nf4 > kMaxF4 || m->nu32 < 0 || m->nu32 > kMaxU32)
        return fail(TGPU_ERR_ARG, "model '%s': %d float4 and %d u32 streams (1..%d and 0..%d)", m->name, m->nf4,
                    m->nu32, kMaxF4, kMaxU32);
    if (m->role_f4[0] != kState) return fail(TGPU_ERR_ARG, "model '%s': float4 stream 0 (the position) must be state", m->name);
    for (int c = 0; c < m->nf4; ++c)
        if (m->role_f4[c] != kState && m->role_f4[c] != kStep)
            return fail(TGPU_ERR_ARG, "model '%s': float4 stream %d has no role", m->name, c);
    for (int c = 0; c < m->nu32; ++c)
        if (m->role_u32[c] != kState && m->role_u32[c] != kStep)
            return fail(TGPU_ERR_ARG, "model '%s': u32 stream %d has no role", m->name, c);
    if (!m->pack || !m->unpack) return fail(TGPU_ERR_ARG, "model '%s': no record codec", m->name);
    if (m->see_ctx_bytes > 65536 || m->act_ctx_bytes > 65536)
        return fail(TGPU_ERR_ARG, "model '%s': contexts above 64 KB", m->name);
    if (!m->kernels || m->nkernels < 1 || !m->programs || m->nprograms < 1)
        return fail(TGPU_ERR_ARG, "model '%s': no kernels or programs", m->name);
    const uint32_t all_f4 = (1u << m->nf4) - 1u, all_u32 = (1u << m->nu32) - 1u;
    for (int k = 0; k < m->nkernels; ++k) {
        const KernelDesc &d = m->kernels[k];
        const bool ok = d.see ? (d.launch_see && d.prepare) : (d.act && d.launch_act);
        if (!ok || (d.writes_f4 & ~all_f4) || (d.seen_f4 & ~all_f4) || (d.writes_u32 & ~all_u32) ||
            d.staged_f4 < 0 || d.staged_f4 > kMaxF4 || d.pair_list < 0 || d.pair_list > 2)
            return fail(TGPU_ERR_ARG, "model '%s': kernel %d is incomplete or names streams it does not have", m->name, k);
    }
    for (int p = 0; p < m->nprograms; ++p) {
        const ProgramDesc &pr = m->programs[p];
        if (pr.passes < 1 || pr.passes > 4 || pr.kernels < 1 || pr.kernels > 4)
            return fail(TGPU_ERR_ARG, "model '%s': program %d has %d passes in %d kernels", m->name, p, pr.passes,
                        pr.kernels);
        for (int q = 0; q < pr.passes; ++q)
            if (!pr.names[q] || !model_has_func(m, pr.names[q]))
                return fail(TGPU_ERR_ARG, "model '%s': program %d names a func no kernel provides", m->name, p);
        for (int q = 0; q < pr.kernels; ++q)
            if (pr.kernel_index[q] < 0 || pr.kernel_index[q] >= m->nkernels)
                return fail(TGPU_ERR_ARG, "model '%s': program %d uses kernel %d of %d", m->name, p,
                            pr.kernel_index[q], m->nkernels);
    }
    // a func name selects exactly one model (checked and added under one lock, so two
    // registrations of the same name cannot both pass)
    std::lock_guard<std::mutex> guard(g_models_lock);
    for (int k = 0; k < m->nkernels; ++k)
        for (const char *fn : {m->kernels[k].see, m->kernels[k].act}) {
            if (!fn) continue;
            const ModelDesc *other = nullptr;
            for (int i = 0; i < 4 && !other; ++i)
                if (model_has_func(model_list(i), fn)) other = model_list(i);
            for (size_t i = 0; i < g_registered.size() && !other; ++i)
                if (model_has_func(g_registered[i], fn)) other = g_registered[i];
            if (other)
                return fail(TGPU_ERR_ARG, "model '%s': func '%s' is already provided by model '%s'", m->name, fn,
                            other->name);
        }
    g_registered.push_back(m);
    return TGPU_OK;
}

int tgpu_register_model_library(const char *path) {
    if (!path) return fail(TGPU_ERR_ARG, "tgpu_register_model_library: null path");
    // kept loaded for the life of the process once registered: the registry points into it
    void *h = dlopen(path, RTLD_NOW | RTLD_LOCAL);
    if (!h) return fail(TGPU_ERR_ARG, "tgpu_register_model_library: %s", dlerror());
    using Entry = const void *(*)(unsigned *);
    Entry entry = reinterpret_cast<Entry>(dlsym(h, "tgpu_model_entry"));
    if (!entry) {
        dlclose(h);
        return fail(TGPU_ERR_ARG, "tgpu_register_model_library: %s exports no tgpu_model_entry", path);
    }
    unsigned abi = 0;
    const void *desc = entry(&abi);
    const int rc = tgpu_register_model(desc, abi);
    if (rc != TGPU_OK) dlclose(h);  // nothing of it was kept
    return rc;
}

const char *tgpu_model_of(const char *func_name) {
    const ModelDesc *m = func_name ? find_model(func_name) : nullptr;
    return m ? m->name : nullptr;
}

int tgpu_selftest_sort_wait(unsigned *device_error) {
    if (!device_error) return fail(TGPU_ERR_ARG, "null output");
    uint32_t err = 0;
    cudaError_t e = selftest_sort_wait(&err);
    if (e != cudaSuccess) return fail(TGPU_ERR_CUDA, "sort wait self-test: %s", cudaGetErrorString(e));
    *device_error = err;
    return TGPU_OK;
}

int tgpu_model_nonpoint(const char *func_name) {
    const ModelDesc *m = func_name ? find_model(func_name) : nullptr;
    return m ? (m->nonpoint ? 1 : 0) : -1;
}

const char *tgpu_batch_model(const TgpuBatch *b) { return b && b->m ? b->m->name : nullptr; }
int tgpu_batch_program(const TgpuBatch *b) { return b ? b->program : -1; }
double tgpu_batch_last_device_ms(const TgpuBatch *b) { return b ? b->last_ms : 0.0; }
unsigned long long tgpu_batch_last_pairs(const TgpuBatch *b) { return b ? b->last_pairs : 0ull; }
int tgpu_batch_launches_per_step(const TgpuBatch *b) { return b ? b->launches_per_step : 0; }

void tgpu_batch_destroy(TgpuBatch *b) { free_batch(b); }

}  // extern "C"

namespace {

// Segments of a new batch, one per group: packed agent ranges, radix tiles and see CTAs.
// reach[g][a] is the largest see radius per axis of the passes whose seers are group g.
int add_segments(TgpuBatch *b, const TgpuGroup *groups, int group_count, const std::vector<std::array<float, 3>> &reach) {
    uint32_t total = 0;
    for (int s = 0; s < group_count; ++s) {
        const TgpuGroup &g = groups[s];
        if (g.agent_size != b->m->agent_bytes)
            return fail(TGPU_ERR_ARG, "group %d: agent size %u, device model '%s' expects %u", s, g.agent_size,
                        b->m->name, b->m->agent_bytes);
        HostSeg h;
        h.g = g;
        if (g.passes && g.pass_count > 0) h.passes.assign(g.passes, g.passes + g.pass_count);
        h.g.passes = nullptr;
        for (int a = 0; a < 3; ++a) {
            h.host_min[a] = 0.0f;
            h.host_max[a] = 0.0f;
        }
        b->hs.push_back(h);
        SegmentSpec sp{};
        sp.begin = total;
        sp.count = g.count;
        sp.fixed_box = g.box_fixed ? 1u : 0u;
        sp.order = b->cell_order;
        sp.dims = (g.dims >= 1 && g.dims <= 3) ? (uint32_t)g.dims : 3u;
        for (int a = 0; a < 3; ++a) {
            float part = g.min_part_sizes[a] > 0.0f ? g.min_part_sizes[a] : 1.0f;
            sp.part[a] = part * g_tuning.cell_multiple;
            // row order: x cells only tighten each row's range, so they may be finer
            if (a == 0 && b->cell_order == kOrderRows) sp.part[a] *= g_tuning.x_cell_factor;
            sp.box_min[a] = g.box_min[a];
            sp.box_max[a] = g.box_max[a];
            sp.reach[a] = reach[s][a];
        }
        sp.tile_begin = (uint32_t)b->tile_seg.size();
        sp.tile_count = (g.count + kSortTile - 1) / kSortTile;
        for (uint32_t t = 0; t < sp.tile_count; ++t) b->tile_seg.push_back((uint32_t)s);
        b->cta_begin.push_back((uint32_t)b->cta.size());
        for (uint32_t c = 0; c < g.count; c += kSeeThreads) b->cta.push_back(make_uint2((uint32_t)s, total + c));
        b->specs.push_back(sp);
        total += g.count;
    }
    b->cta_begin.push_back((uint32_t)b->cta.size());
    b->total = total;
    b->wt_dev.assign((size_t)group_count, nullptr);
    b->wt_done.assign((size_t)group_count, 0);
    b->tiles = (uint32_t)b->tile_seg.size();
    b->ctas = (uint32_t)b->cta.size();
    return TGPU_OK;
}

#define CKR(call)                                                                                    \
    do {                                                                                             \
        cudaError_t e_ = (call);                                                                     \
        if (e_ != cudaSuccess) return fail(TGPU_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

// Stream, events and every device buffer of a batch whose segments are set.
int alloc_batch(TgpuBatch *b) {
    const ModelDesc *m = b->m;
    CKR(cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking));
    CKR(cudaEventCreate(&b->e0));
    CKR(cudaEventCreate(&b->e1));
    const size_t n = std::max<uint32_t>(b->total, 1);
    CKR(cudaMalloc(&b->d_specs, sizeof(SegmentSpec) * b->nseg));
    CKR(cudaMalloc(&b->d_extent, sizeof(BoxAcc)));
    CKR(cudaMalloc(&b->d_tile_seg, sizeof(uint32_t) * std::max<uint32_t>(b->tiles, 1)));
    CKR(cudaMalloc(&b->d_cta, sizeof(uint2) * std::max<uint32_t>(b->ctas, 1)));
    CKR(cudaMalloc(&b->d_box, sizeof(BoxAcc) * b->nseg));
    CKR(cudaMalloc(&b->d_grids, sizeof(SegGrid) * b->nseg));
    if (b->tiles) CKR(cudaMemcpy(b->d_tile_seg, b->tile_seg.data(), sizeof(uint32_t) * b->tiles, cudaMemcpyHostToDevice));
    if (b->ctas) CKR(cudaMemcpy(b->d_cta, b->cta.data(), sizeof(uint2) * b->ctas, cudaMemcpyHostToDevice));
    for (int c = 0; c < m->nf4; ++c) {
        CKR(cudaMalloc(&b->f4[c][0], sizeof(float4) * n));
        CKR(cudaMemset(b->f4[c][0], 0, sizeof(float4) * n));
        if (m->role_f4[c] == kState) {
            CKR(cudaMalloc(&b->f4[c][1], sizeof(float4) * n));
            CKR(cudaMemset(b->f4[c][1], 0, sizeof(float4) * n));
        }
    }
    for (int c = 0; c < m->nu32; ++c) {
        CKR(cudaMalloc(&b->u32[c][0], sizeof(uint32_t) * n));
        CKR(cudaMalloc(&b->u32[c][1], sizeof(uint32_t) * n));
    }
    for (int k = 0; k < 2; ++k) {
        CKR(cudaMalloc(&b->keys[k], sizeof(uint32_t) * n));
        CKR(cudaMalloc(&b->vals[k], sizeof(uint32_t) * n));
    }
    CKR(cudaMalloc(&b->sort_scratch, sort_scratch_bytes((uint32_t)b->nseg, std::max<uint32_t>(b->tiles, 1))));
    // status block: [0] pair counter, [1..8] telemetry, [9] the device error word (low half)
    CKR(cudaMalloc(&b->d_status, sizeof(unsigned long long) * kStatusWords));
    CKR(cudaMemset(b->d_status, 0, sizeof(unsigned long long) * kStatusWords));
    CKR(cudaMallocHost(&b->h_status, sizeof(unsigned long long) * kStatusWords));
    CKR(cudaMallocHost(&b->h_extent, sizeof(BoxAcc) * (size_t)std::max(b->nseg, 1)));
    b->d_pairs = b->d_status;
    b->d_telemetry = b->d_status + 1;
    b->d_err = reinterpret_cast<uint32_t *>(b->d_status + 9);
    CKR(cudaMalloc(&b->d_aos, (size_t)m->agent_bytes * n));
    b->ctx_stride = (std::max(m->see_ctx_bytes, m->act_ctx_bytes) + 15u) & ~15u;
    return TGPU_OK;
}

// Per-kernel see configuration from the tuning: radii / context buffers, staging.
int setup_see_run(TgpuBatch *b, KernelRun &r, int self_see) {
    r.skip_self = self_see ? 0 : 1;
    CKR(cudaMalloc(&r.d_radii, sizeof(float4) * b->nseg));
    CKR(cudaMemset(r.d_radii, 0, sizeof(float4) * b->nseg));
    CKR(cudaMalloc(&r.d_see_ctx, b->ctx_stride * b->nseg));
    CKR(cudaMemset(r.d_see_ctx, 0, b->ctx_stride * b->nseg));
    const uint32_t cap_default = r.k->staged_f4 <= 1 ? 1024u : 768u;
    r.union_factor = g_tuning.union_factor;
    if (g_tuning.stage && g_tuning.cell_order == kOrderRows) {
        // row order: bulk-copied union rows; stage_cells bounds the rows per CTA
        r.stage_cap = g_tuning.stage_cap ? g_tuning.stage_cap : cap_default;
        r.stage_cells = g_tuning.stage_cells ? g_tuning.stage_cells : 64u;
        r.smem = (size_t)r.k->staged_f4 * r.stage_cap * sizeof(float4) + (2ull * r.stage_cells + 2) * sizeof(uint32_t) +
                 sizeof(uint64_t);
    } else if (g_tuning.stage) {
        r.stage_cap = g_tuning.stage_cap ? g_tuning.stage_cap : cap_default;
        r.stage_cells = g_tuning.stage_cells ? g_tuning.stage_cells : 512u;
        r.smem = (size_t)r.k->staged_f4 * r.stage_cap * sizeof(float4) + (2ull * r.stage_cells + 1) * sizeof(uint32_t);
    } else {
        r.stage_cap = 0;
        r.stage_cells = 0;
        r.smem = 0;
    }
    if (r.smem > 220 * 1024) return fail(TGPU_ERR_ARG, "staging buffer of %zu bytes exceeds shared memory", r.smem);
    CKR(r.k->prepare(r.smem));
    return TGPU_OK;
}

// Pair lists between consecutive see runs of a batch's program: the first declares it
// can record (pair_list 1), the next that it can replay (2), and the positions do not
// change in between.  Row order walks through L1 only (the walks that record), and a
// list that holds the seer itself unless the replaying pass skips it.  Whether the
// recorded set covers the replaying pass's pairs depends on the radii and contexts of
// each run, which can change between runs: the kernel checks that on the device and
// walks when it does not hold.
int setup_pair_lists(TgpuBatch *b) {
    const uint32_t cap = g_tuning.pair_list_cap > 0xFFFFFFF0u ? 0xFFFFFFF0u : (g_tuning.pair_list_cap + 3u) & ~3u;
    if (!cap || b->cell_order != kOrderRows || b->hit_masks || b->total == 0) return TGPU_OK;
    bool any = false;
    for (size_t k = 0; k + 1 < b->runs.size(); ++k) {
        KernelRun &a = b->runs[k], &c = b->runs[k + 1];
        if (a.k->pair_list != 1 || c.k->pair_list != 2 || a.list_mode || a.stage_cap || c.stage_cap) continue;
        if (a.seer_seg >= 0 || c.seer_seg >= 0 || b->m->nonpoint) continue;
        if (a.k->writes_f4 & 1u) continue;            // positions (stream 0) change in between
        if (a.skip_self && !c.skip_self) continue;    // the list lacks the seer itself
        a.list_mode = 1u;
        c.list_mode = 2u;
        c.list_src = (int)k;
        any = true;
    }
    if (!any) return TGPU_OK;
    if ((uint64_t)cap * b->total > (1ull << 38))  // 1 TB of entries: a capacity no device holds
        return fail(TGPU_ERR_ARG, "pair list of %u entries per agent for %u agents is too large", cap, b->total);
    b->plist_cap = cap;
    CKR(cudaMalloc(&b->plist_idx, (size_t)(cap / 4u) * b->total * sizeof(uint4)));
    CKR(cudaMalloc(&b->plist_count, (size_t)b->total * sizeof(uint2)));
    return TGPU_OK;
}

#undef CKR

const KernelDesc *find_kernel(const ModelDesc *m, const char *see, const char *act) {
    for (int k = 0; k < m->nkernels; ++k) {
        const KernelDesc &d = m->kernels[k];
        const bool see_ok = see ? (d.see && !strcmp(d.see, see)) : !d.see;
        const bool act_ok = act ? (d.act && !strcmp(d.act, act)) : !d.act;
        if (see_ok && act_ok) return &d;
    }
    return nullptr;
}

// Contexts and radii of a state-level pass list (tgpu_state_create), one per seer segment.
int upload_state_contexts(TgpuBatch *b) {
    std::vector<char> buf(b->ctx_stride);
    for (size_t k = 0; k < b->runs.size(); ++k) {
        const KernelRun &r = b->runs[k];
        const TgpuPass &tp = b->state_passes[k].pass;
        std::fill(buf.begin(), buf.end(), 0);
        if (tp.context && tp.context_size) memcpy(buf.data(), tp.context, std::min((size_t)tp.context_size, b->ctx_stride));
        char *dst = r.k->see ? r.d_see_ctx : r.d_act_ctx;
        CK(cudaMemcpyAsync(dst + (size_t)r.seer_seg * b->ctx_stride, buf.data(), b->ctx_stride, cudaMemcpyHostToDevice,
                           b->st));
        if (r.k->see) {
            // the box test over min(seer dims, seen dims) axes (tay/cpu_z_grid.c:289-291)
            const int dims = std::min(seg_dims(b->specs[r.seer_seg]), seg_dims(b->specs[r.seen_seg]));
            float4 rr = pass_radii(tp, dims);
            CK(cudaMemcpyAsync(r.d_radii + r.seer_seg, &rr, sizeof(float4), cudaMemcpyHostToDevice, b->st));
        }
    }
    CK(cudaStreamSynchronize(b->st));
    return TGPU_OK;
}

}  // namespace

namespace {

// The extents of the pushes that completed (the stream was synchronized since): each
// pending one becomes its group's host extent, and a changed extent re-sizes the grid
// budgets at the next run.
void apply_extents(TgpuBatch *b) {
    for (int s = 0; s < b->nseg; ++s) {
        HostSeg &h = b->hs[s];
        if (!h.extent_pending) continue;
        h.extent_pending = false;
        const BoxAcc &ext = b->h_extent[s];
        for (int a = 0; a < 3; ++a) {
            const float lo = ordered_to_float(ext.lo[a]), hi = ordered_to_float(ext.hi[a]);
            if (lo != h.host_min[a] || hi != h.host_max[a]) b->specs_dirty = true;
            h.host_min[a] = lo;
            h.host_max[a] = hi;
        }
    }
}

}  // namespace

extern "C" {

int tgpu_batch_create(const TgpuGroup *groups, int group_count, TgpuBatch **out) {
    if (!out || !groups || group_count <= 0) return fail(TGPU_ERR_ARG, "no groups");
    *out = nullptr;
    const TgpuGroup &g0 = groups[0];
    if (g0.pass_count <= 0 || !g0.passes) return fail(TGPU_ERR_ARG, "group has no passes");
    const ModelDesc *m = find_model(g0.passes[0].func_name ? g0.passes[0].func_name : "");
    if (!m) return fail(TGPU_ERR_UNKNOWN_FUNC, "no device model provides '%s'", g0.passes[0].func_name);
    for (int k = 0; k < g0.pass_count; ++k)
        if (!g0.passes[k].func_name || !model_has_func(m, g0.passes[k].func_name))
            return fail(TGPU_ERR_UNKNOWN_FUNC, "func '%s' is not part of device model '%s'",
                        g0.passes[k].func_name ? g0.passes[k].func_name : "(null)", m->name);
    const int program = match_program(m, g0);
    if (program < 0) return fail(TGPU_ERR_PROGRAM, "pass sequence not supported by device model '%s'", m->name);
    std::vector<std::array<float, 3>> reach(group_count);
    for (int s = 0; s < group_count; ++s) {
        const TgpuGroup &g = groups[s];
        if (!g.passes || match_program(m, g) != program) return fail(TGPU_ERR_ARG, "group %d: pass sequence differs from group 0", s);
        for (int a = 0; a < 3; ++a) {
            reach[s][a] = 0.0f;
            for (int k = 0; k < g.pass_count; ++k)
                if (g.passes[k].is_see) reach[s][a] = std::max(reach[s][a], g.passes[k].radii[a]);
        }
    }

    TgpuBatch *b = new TgpuBatch();
    b->m = m;
    b->program = program;
    b->nseg = group_count;
    b->use_graphs = g_tuning.use_graphs != 0;
    b->cell_order = g_tuning.cell_order == kOrderRows ? kOrderRows : kOrderMorton;
    b->hit_masks = g_tuning.hit_masks ? 1u : 0u;
    int rc = add_segments(b, groups, group_count, reach);
    if (!rc) rc = alloc_batch(b);
    const ProgramDesc &pd = m->programs[program];
    int cursor = 0;
    for (int k = 0; k < pd.kernels && !rc; ++k) {
        KernelRun r{};
        r.k = &m->kernels[pd.kernel_index[k]];
        r.see_pass = r.k->see ? pass_index(g0, r.k->see, cursor) : -1;
        r.act_pass = r.k->act ? pass_index(g0, r.k->act, r.see_pass >= 0 ? r.see_pass + 1 : cursor) : -1;
        cursor = std::max(r.see_pass, r.act_pass) + 1;
        if (r.see_pass >= 0) rc = setup_see_run(b, r, g0.passes[r.see_pass].self_see);
        if (!rc && r.act_pass >= 0) {
            if (cudaMalloc(&r.d_act_ctx, b->ctx_stride * b->nseg) != cudaSuccess)
                rc = fail(TGPU_ERR_CUDA, "cudaMalloc of the act contexts failed");
        }
        b->runs.push_back(r);
    }
    if (!rc) rc = setup_pair_lists(b);
    for (int s = 0; s < b->nseg && !rc; ++s) rc = upload_contexts(b, s);
    if (rc) {
        free_batch(b);
        return rc;
    }
    *out = b;
    return TGPU_OK;
}

int tgpu_state_create(const TgpuGroup *groups, int group_count, const TgpuStatePass *passes, int pass_count,
                      TgpuBatch **out) {
    if (!out || !groups || group_count <= 0 || !passes || pass_count <= 0) return fail(TGPU_ERR_ARG, "no groups or passes");
    *out = nullptr;
    const ModelDesc *m = find_model(passes[0].pass.func_name ? passes[0].pass.func_name : "");
    if (!m) return fail(TGPU_ERR_UNKNOWN_FUNC, "no device model provides '%s'", passes[0].pass.func_name);
    std::vector<std::array<float, 3>> reach(group_count);
    for (auto &r : reach) r = {0.0f, 0.0f, 0.0f};
    std::vector<int> see_passes(group_count, 0);
    std::vector<const KernelDesc *> kernels(pass_count);
    for (int k = 0; k < pass_count; ++k) {
        const TgpuStatePass &sp = passes[k];
        const char *fn = sp.pass.func_name;
        if (!fn || !model_has_func(m, fn))
            return fail(TGPU_ERR_UNKNOWN_FUNC, "func '%s' is not part of device model '%s'", fn ? fn : "(null)", m->name);
        if (sp.seer_group < 0 || sp.seer_group >= group_count || (sp.pass.is_see && (sp.seen_group < 0 || sp.seen_group >= group_count)))
            return fail(TGPU_ERR_ARG, "pass %d: group index out of range", k);
        kernels[k] = sp.pass.is_see ? find_kernel(m, fn, nullptr) : find_kernel(m, nullptr, fn);
        if (!kernels[k])
            return fail(TGPU_ERR_PROGRAM, "pass %d: device model '%s' has no standalone %s kernel for '%s'", k, m->name,
                        sp.pass.is_see ? "see" : "act", fn);
        const KernelDesc &d = *kernels[k];
        for (int c = 0; c < m->nf4; ++c)
            if (m->role_f4[c] == kState && (d.writes_f4 >> c & 1u) && (d.seen_f4 >> c & 1u))
                return fail(TGPU_ERR_PROGRAM, "pass %d: '%s' writes a stream other agents see", k, fn);
        if (sp.pass.is_see) {
            if (++see_passes[sp.seer_group] > 1 && !d.accumulates)
                return fail(TGPU_ERR_PROGRAM, "group %d: several '%s' see passes, and the see function of model '%s' does not accumulate",
                            sp.seer_group, fn, m->name);
            for (int a = 0; a < 3; ++a) reach[sp.seer_group][a] = std::max(reach[sp.seer_group][a], sp.pass.radii[a]);
        }
    }

    TgpuBatch *b = new TgpuBatch();
    b->m = m;
    b->program = -1;
    b->nseg = group_count;
    b->use_graphs = g_tuning.use_graphs != 0;
    b->cell_order = g_tuning.cell_order == kOrderRows ? kOrderRows : kOrderMorton;
    b->hit_masks = g_tuning.hit_masks ? 1u : 0u;
    b->state_passes.assign(passes, passes + pass_count);
    int rc = add_segments(b, groups, group_count, reach);
    if (!rc) rc = alloc_batch(b);
    for (int k = 0; k < pass_count && !rc; ++k) {
        const TgpuStatePass &sp = passes[k];
        KernelRun r{};
        r.k = kernels[k];
        r.see_pass = sp.pass.is_see ? k : -1;
        r.act_pass = sp.pass.is_see ? -1 : k;
        r.seer_seg = sp.seer_group;
        r.seen_seg = sp.pass.is_see ? sp.seen_group : sp.seer_group;
        if (sp.pass.is_see) {
            rc = setup_see_run(b, r, sp.pass.self_see || sp.seen_group != sp.seer_group);
        } else if (cudaMalloc(&r.d_act_ctx, b->ctx_stride * b->nseg) != cudaSuccess) {
            rc = fail(TGPU_ERR_CUDA, "cudaMalloc of the act contexts failed");
        }
        b->runs.push_back(r);
    }
    if (!rc) rc = upload_state_contexts(b);
    if (rc) {
        free_batch(b);
        return rc;
    }
    *out = b;
    return TGPU_OK;
}

int tgpu_state_set_contexts(TgpuBatch *b, const TgpuStatePass *passes, int pass_count) {
    if (!b || !passes || b->state_passes.empty()) return fail(TGPU_ERR_ARG, "not a state batch");
    if (pass_count != (int)b->state_passes.size()) return fail(TGPU_ERR_ARG, "pass count changed");
    for (int k = 0; k < pass_count; ++k) {
        b->state_passes[k].pass.context = passes[k].pass.context;
        b->state_passes[k].pass.context_size = passes[k].pass.context_size;
        for (int a = 0; a < 4; ++a) b->state_passes[k].pass.radii[a] = passes[k].pass.radii[a];
    }
    return upload_state_contexts(b);
}

int tgpu_batch_set_contexts(TgpuBatch *b, int group, const TgpuGroup *desc) {
    if (!b || !desc || group < 0 || group >= b->nseg) return fail(TGPU_ERR_ARG, "bad group");
    if (!b->state_passes.empty()) return fail(TGPU_ERR_ARG, "state batch: use tgpu_state_set_contexts");
    if (desc->pass_count != (int)b->hs[group].passes.size()) return fail(TGPU_ERR_ARG, "pass count changed");
    for (int k = 0; k < desc->pass_count; ++k) {
        b->hs[group].passes[k].context = desc->passes[k].context;
        b->hs[group].passes[k].context_size = desc->passes[k].context_size;
        for (int a = 0; a < 4; ++a) b->hs[group].passes[k].radii[a] = desc->passes[k].radii[a];
    }
    return upload_contexts(b, group);
}

int tgpu_batch_push(TgpuBatch *b, int group, const void *host) {
    if (!b || group < 0 || group >= b->nseg || !host) return fail(TGPU_ERR_ARG, "bad push");
    HostSeg &h = b->hs[group];
    const SegmentSpec &sp = b->specs[group];
    const uint32_t n = sp.count;
    // A group whose grid budget was already sized by a push gets this push's extent at the
    // next sync, without waiting here: every step derives its grid from the device's box,
    // so a budget one run behind only bounds the cells differently (the pairs are the
    // same), and the host does not stall between the push and the run.
    const bool sized = h.pushed && b->table != nullptr;
    h.pushed = true;
    b->wt_done[group] = 0;
    if (!n) {
        for (int a = 0; a < 3; ++a) h.host_min[a] = h.host_max[a] = 0.0f;
        h.extent_pending = false;
        b->specs_dirty = true;
        return TGPU_OK;
    }
    uint32_t *aos = static_cast<uint32_t *>(pinned_device_ptr(host));
    if (!aos) {
        aos = b->d_aos + (size_t)sp.begin * (b->m->agent_bytes / 4);
        CK(cudaMemcpyAsync(aos, host, (size_t)n * b->m->agent_bytes, cudaMemcpyHostToDevice, b->st));
    }
    // pack into the current buffers of every stream
    PassIO io{};
    for (int c = 0; c < b->m->nf4; ++c) {
        int k = b->m->role_f4[c] == kState ? b->cur_f4[c] : 0;
        io.out_f4[c] = b->f4[c][k] + sp.begin;
        io.in_f4[c] = io.out_f4[c];
    }
    for (int c = 0; c < b->m->nu32; ++c) {
        io.out_u32[c] = b->u32[c][b->cur_u32[c]] + sp.begin;
        io.in_u32[c] = io.out_u32[c];
    }
    // the pack also reduces the extent of the pushed positions (it sizes the segment's
    // grid budget) on the device
    reset_extent(b->d_extent, b->st);
    b->m->pack(aos, n, io, b->d_extent, b->st);
    CK(cudaMemcpyAsync(b->h_extent + group, b->d_extent, sizeof(BoxAcc), cudaMemcpyDeviceToHost, b->st));
    CK(cudaGetLastError());
    if (sized) {
        h.extent_pending = true;
        return TGPU_OK;
    }
    CK(cudaStreamSynchronize(b->st));
    h.extent_pending = true;
    apply_extents(b);
    return TGPU_OK;
}

int tgpu_batch_enqueue(TgpuBatch *b, int steps) {
    if (!b || steps < 0) return fail(TGPU_ERR_ARG, "bad run");
    int rc = prepare_specs(b);
    if (rc) return rc;
    CK(cudaMemsetAsync(b->d_status, 0, sizeof(unsigned long long) * 9, b->st));  // pairs, telemetry
    bool any_wt = false;
    for (int s = 0; s < b->nseg; ++s) {
        b->wt_done[s] = 0;
        any_wt = any_wt || b->wt_dev[s] != nullptr;
    }
    CK(cudaEventRecord(b->e0, b->st));
    for (int i = 0; i < steps; ++i) {
        const bool wt = any_wt && i + 1 == steps;  // the run's last step writes through
        if (!b->use_graphs) {
            enqueue_step(b, nullptr, wt);
            continue;
        }
        const uint64_t sig = parity_signature(b) | (wt ? kWriteThroughGraph : 0ull);
        auto it = b->graphs.find(sig);
        if (it != b->graphs.end()) {
            CK(cudaGraphLaunch(it->second, b->st));
            advance_parity(b);
            continue;
        }
        cudaGraph_t graph = nullptr;
        CK(cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal));
        enqueue_step(b, nullptr, wt);
        CK(cudaStreamEndCapture(b->st, &graph));
        cudaGraphExec_t exec = nullptr;
        cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) return fail(TGPU_ERR_CUDA, "cudaGraphInstantiate failed: %s", cudaGetErrorString(e));
        b->graphs.emplace(sig, exec);
        CK(cudaGraphLaunch(exec, b->st));
    }
    CK(cudaEventRecord(b->e1, b->st));
    // the run's status (pairs, telemetry, error word) comes back with the run
    CK(cudaMemcpyAsync(b->h_status, b->d_status, sizeof(unsigned long long) * kStatusWords, cudaMemcpyDeviceToHost,
                       b->st));
    CK(cudaGetLastError());
    if (any_wt && steps > 0)
        for (int s = 0; s < b->nseg; ++s) b->wt_done[s] = b->wt_dev[s] != nullptr;
    return TGPU_OK;
}

int tgpu_batch_write_through(TgpuBatch *b, int group, void *host) {
    if (!b || group < 0 || group >= b->nseg) return fail(TGPU_ERR_ARG, "bad write-through");
    uint32_t *dev = nullptr;
    if (host) {
        dev = static_cast<uint32_t *>(pinned_device_ptr(host));
        if (!dev) return fail(TGPU_ERR_ARG, "write-through needs page-locked host records");
        if (!b->d_wt) CK(cudaMalloc(&b->d_wt, sizeof(uint32_t *) * (size_t)b->nseg));
    }
    if (dev == b->wt_dev[group]) return TGPU_OK;
    b->wt_dev[group] = dev;
    b->wt_done[group] = 0;
    // the kernels read the addresses from the device array when they run (captured steps
    // stay valid); stream-ordered before the next step
    if (b->d_wt)
        CK(cudaMemcpyAsync(b->d_wt, b->wt_dev.data(), sizeof(uint32_t *) * (size_t)b->nseg, cudaMemcpyHostToDevice,
                           b->st));
    return TGPU_OK;
}

int tgpu_batch_sync(TgpuBatch *b) {
    if (!b) return fail(TGPU_ERR_ARG, "null batch");
    CK(cudaStreamSynchronize(b->st));
    apply_extents(b);
    float ms = 0.0f;
    CK(cudaEventElapsedTime(&ms, b->e0, b->e1));
    b->last_ms = ms;
    b->last_pairs = b->h_status[0];
    for (int k = 0; k < 8; ++k) b->last_telemetry[k] = b->h_status[1 + k];
    if (!(uint32_t)b->h_status[9]) return TGPU_OK;
    return check_device_error(b);  // reads and clears the word, and reports it
}

int tgpu_batch_run(TgpuBatch *b, int steps) {
    int rc = tgpu_batch_enqueue(b, steps);
    if (rc) return rc;
    return tgpu_batch_sync(b);
}

int tgpu_batch_fetch(TgpuBatch *b, int group, void *host) {
    if (!b || group < 0 || group >= b->nseg || !host) return fail(TGPU_ERR_ARG, "bad fetch");
    const SegmentSpec &sp = b->specs[group];
    if (!sp.count) return TGPU_OK;
    uint32_t *pinned = static_cast<uint32_t *>(pinned_device_ptr(host));
    if (b->wt_done[group] && pinned == b->wt_dev[group]) {
        // the last run wrote these records through already
        CK(cudaStreamSynchronize(b->st));
        return TGPU_OK;
    }
    uint32_t *aos = pinned ? pinned : b->d_aos + (size_t)sp.begin * (b->m->agent_bytes / 4);
    PassIO io = make_io(b, nullptr, false, sp.begin);
    b->m->unpack(aos, sp.count, io, unpack_program(b), b->st);
    CK(cudaGetLastError());
    if (!pinned)
        CK(cudaMemcpyAsync(host, aos, (size_t)sp.count * b->m->agent_bytes, cudaMemcpyDeviceToHost, b->st));
    CK(cudaStreamSynchronize(b->st));
    return TGPU_OK;
}

}  // extern "C"
