// Internal view of a batch, shared by the runtime and the adjoint module.
#pragma once

#include <map>
#include <string>
#include <vector>

#include "model.cuh"
#include "tay_gpu.h"

namespace tgpu {

// 64-bit words of a batch's status block: the pair counter, 8 telemetry counters, the
// device error word.
constexpr int kStatusWords = 10;

// Segments up to which a row-order step clears its table with one memset per segment.
constexpr int kMemsetClearSegments = 4;

struct KernelRun {
    const KernelDesc *k;
    int see_pass;  // index into the group's pass list, or -1
    int act_pass;
    float4 *d_radii = nullptr;  // [segments]
    char *d_see_ctx = nullptr;  // [segments * ctx_stride]
    char *d_act_ctx = nullptr;
    size_t smem = 0;
    uint32_t stage_cap = 0, stage_cells = 0, union_factor = 2;
    int skip_self = 0;
    int seer_seg = -1;  // state batches: the pass's seer (acting) segment; -1: every segment
    int seen_seg = -1;  // state batches: the segment whose agents a see pass reads
    uint32_t list_mode = 0;  // pair list (PairList): 0 none, 1 record, 2 replay
    int list_src = -1;       // replay: the run that records the list
};

struct HostSeg {
    TgpuGroup g;
    std::vector<TgpuPass> passes;
    float host_min[3], host_max[3];
    bool pushed = false;
    bool extent_pending = false;  // a push's extent is on its way to h_extent (read at the next sync)
};

// Optional per-class timing of one enqueued step: an event is recorded before and after
// each kernel class (ev[2k], ev[2k+1] for classes 0..3, then one pair per pass kernel);
// the table clear at the end is timed by ev2[0..1].
struct StepEvents {
    cudaEvent_t *ev;
    cudaEvent_t *ev2;
};

int check_device_error(TgpuBatch *b);

}  // namespace tgpu

using namespace tgpu;

struct TgpuBatch {
    const tgpu::ModelDesc *m = nullptr;
    int program = -1;
    int nseg = 0;
    uint32_t total = 0;
    std::vector<HostSeg> hs;
    std::vector<SegmentSpec> specs;
    std::vector<uint32_t> tile_seg;
    std::vector<uint2> cta;
    std::vector<uint32_t> cta_begin;           // first CTA of each segment, + total
    std::vector<TgpuStatePass> state_passes;   // tgpu_state_create: the state's pass list
    uint32_t tiles = 0, ctas = 0, key_bits = 0;
    bool specs_dirty = true;

    SegmentSpec *d_specs = nullptr;
    uint32_t *d_tile_seg = nullptr;
    uint2 *d_cta = nullptr;
    BoxAcc *d_box = nullptr;
    SegGrid *d_grids = nullptr;  // per segment: this step's grid (from the box)
    float4 *f4[kMaxF4][2] = {};
    uint32_t *u32[kMaxU32][2] = {};
    int cur_f4[kMaxF4] = {};
    int cur_u32[kMaxU32] = {};
    uint32_t *keys[2] = {}, *vals[2] = {}, *sort_scratch = nullptr;
    uint32_t *d_err = nullptr;  // device error word (DeviceError bits), read at every sync
    uint2 *table = nullptr;
    size_t table_entries = 0;
    uint32_t *d_aos = nullptr;
    // one device block for the run's status (pair counter, telemetry, error word), read back
    // by one copy into page-locked h_status at the end of every run
    unsigned long long *d_status = nullptr, *h_status = nullptr;
    unsigned long long *d_pairs = nullptr;      // d_status[0]
    unsigned long long *d_telemetry = nullptr;  // d_status[1..8]: kTelemetry counters, summed over a run
    // the context and radii bytes last uploaded per (run, see context / act context / radii,
    // segment): a run uploads only what the host changed
    std::vector<std::string> ctx_shadow;
    unsigned long long last_telemetry[8] = {};
    size_t ctx_stride = 0;
    std::vector<KernelRun> runs;
    int launches_per_step = 0;
    // pair list of a recording see pass for the next one (PairList): [cap / 4][total]
    // groups of four entries and per agent {entries, box-test passes with other agents}
    uint4 *plist_idx = nullptr;
    uint2 *plist_count = nullptr;
    uint32_t plist_cap = 0;

    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    double last_ms = 0.0;
    unsigned long long last_pairs = 0;
    bool use_graphs = true;
    uint32_t cell_order = kOrderMorton;  // key order and table layout of every segment
    BoxAcc *d_extent = nullptr;          // pushed extent of one group
    BoxAcc *h_extent = nullptr;          // page-locked, per segment: the extent of its last push
    uint32_t hit_masks = 0;              // see walk: hit masks (row order)
    std::map<uint64_t, cudaGraphExec_t> graphs;

    // Write-through fetch: per segment, the device address of page-locked host records
    // that the last step of a run fills as its final pass finishes (or null), the same
    // array on the device, and the segments whose host copy the last run made current.
    std::vector<uint32_t *> wt_dev;
    uint32_t **d_wt = nullptr;
    std::vector<char> wt_done;
};


namespace tgpu {

// Runtime functions the adjoint module reuses.
int prepare_specs(TgpuBatch *b);
void enqueue_step(TgpuBatch *b, const StepEvents *E = nullptr, bool write_through = false);
// The batch's pair list on a see launch of run r, when r records or replays one.
void attach_pair_list(const TgpuBatch *b, const KernelRun &r, SeeLaunch &S);
PassIO make_io(TgpuBatch *b, const KernelDesc *k, bool fused_see, uint32_t offset);
SortLaunch sort_launch(TgpuBatch *b);
int fail(int code, const char *fmt, ...);

}  // namespace tgpu
