// Launch descriptions shared between the sort, see/act kernels and the runtime.
#pragma once

#include "tgpu_internal.cuh"

namespace tgpu {

// Everything the sort needs for one batch of segments.
struct SortLaunch {
    const SegmentSpec *specs;  // [segments]
    const uint32_t *tile_seg;  // [tiles] segment of each radix tile
    BoxAcc *box;               // [segments]
    const float4 *pos;         // positions, current order
    const float4 *pos_max;     // non-point agents: max corners, current order (else null)
    uint32_t *keys[2];         // [n] ping-pong key buffers
    uint32_t *vals[2];         // [n] ping-pong permutation buffers
    uint32_t *sort_scratch;    // sort_scratch_bytes(segments, tiles): digit histograms, tile
                               // counters and look-back words, zeroed by every sort
    uint32_t *err;             // device error word (DeviceError bits)
    uint2 *table;              // dense cell tables of all segments
    SegGrid *grids;            // [segments] this step's grids, written by launch_box / launch_grids
    uint32_t segments;
    uint32_t tiles;
    uint32_t key_bits;
};

struct GatherSet {
    const float4 *src_f4[kMaxF4];
    float4 *dst_f4[kMaxF4];
    const uint32_t *src_u32[kMaxU32];
    uint32_t *dst_u32[kMaxU32];
    int nf4;
    int nu32;
};

// Streams seen by a pass kernel.  Index meaning is model-specific; float4 stream 0 is
// always the position.
struct PassIO {
    const float4 *in_f4[kMaxF4];
    float4 *out_f4[kMaxF4];
    const uint32_t *in_u32[kMaxU32];
    uint32_t *out_u32[kMaxU32];
};

// Pair list shared by two consecutive see passes over unchanged positions (row order):
// the recording pass stores, per seer, the candidates that passed the box test and the
// model's keep test, in walk order; the replaying pass runs its see function over them
// instead of walking the rows again.  Entries come in groups of four: entries 4g..4g+3 of
// seer i are the 16 bytes idx[g * stride + i], so a lane stores one group per four
// entries and the lanes of a warp read their g-th groups from 512 consecutive bytes.
struct PairList {
    uint4 *idx;
    uint2 *count;             // per seer {entries (may exceed cap: overflow), box-test passes
                              // with agents other than itself}
    uint32_t stride;          // agents of the batch
    uint32_t cap;             // entries per seer (a multiple of 4)
    uint32_t mode;            // 0: none, 1: record, 2: replay
    const float4 *rec_radii;  // replay: the recording pass's radii, per segment
    const char *rec_ctx;      // replay: the recording pass's see contexts (stride ctx_stride)
};

struct SeeLaunch {
    const SegmentSpec *specs;
    const BoxAcc *box;
    const SegGrid *grids;     // per segment this step's grid and rounding pad
    const uint2 *table;
    const uint2 *cta_table;   // per CTA {segment, first seer}
    const float4 *radii;      // per segment see radii of this pass
    const char *ctx;          // per segment see context, stride ctx_stride
    uint32_t ctx_stride;
    const char *act_ctx;      // per segment context of a fused act pass (or = ctx)
    uint32_t act_ctx_stride;
    uint32_t ctas;
    int skip_self;            // same group and !self_see: a seer never sees itself
    uint32_t stage_cap;       // staged agents per CTA (0: no staging, read through L1)
    uint32_t stage_cells;     // halo cells per CTA
    uint32_t union_factor;    // a warp walks its union box when union <= factor x lane box
    uint32_t rows;            // 1: the table is in row order (see_rows_kernel)
    uint32_t hit_masks;       // row order: lanes collect box-test hits in 32-bit masks first
    uint32_t *err;            // device error word (DeviceError bits)
    uint32_t cta_offset;      // first entry of cta_table this launch covers
    uint32_t cross;           // 1: the seen agents are segment seen_seg (a two-group pass)
    uint32_t seen_seg;
    unsigned long long *pairs;  // box-test passes, summed over the launch
    // telemetry (the reference's TAY_TELEMETRY counters, tay/space.c:50-60, plus the
    // kernel's own paths): [0] candidates box-tested (broad phase), [1] staged CTAs,
    // [2] CTAs that read the halo from global memory, [3] warps that walked the union
    // box, [4] warps whose lanes walked their own boxes, [5] warps that replayed a pair
    // list
    unsigned long long *telemetry;
    PassIO io;
    // write-through (the last pass of a run): per segment the device address of the
    // page-locked host records its seers' finished records go to (null: none), and the
    // model's unpack program
    uint32_t *const *wt;
    uint32_t wt_program;
    PairList plist;
};

struct ActLaunch {
    const SegmentSpec *specs;
    const uint32_t *tile_seg;
    const char *ctx;
    uint32_t ctx_stride;
    uint32_t tiles;
    uint32_t tile_offset;     // first entry of tile_seg this launch covers
    PassIO io;
};

// Bounding boxes of every segment and, from them, their grids (the last block of each
// segment derives its grid).
void launch_box(const SortLaunch &L, cudaStream_t st);
// Grids of every segment from the boxes in L.box (after they were set or restored).
void launch_grids(const SortLaunch &L, cudaStream_t st);
constexpr int kMaxSortPasses = 4;  // 32-bit keys in 8-bit digits
constexpr uint32_t kMaxRadix = 512;  // bins of the widest digit (9 bits)

// Digit width of a radix sort of `key_bits`-bit keys: 9 bits where that takes one pass
// fewer than 8-bit digits (17-18 and 25-27-bit keys), else 8.
constexpr int sort_digit_bits(uint32_t key_bits) { return (key_bits + 8u) / 9u < (key_bits + 7u) / 8u ? 9 : 8; }
constexpr int sort_passes(uint32_t key_bits) {
    return (int)((key_bits + (uint32_t)sort_digit_bits(key_bits) - 1u) / (uint32_t)sort_digit_bits(key_bits));
}

// Bytes of the sort's scratch: per-segment histograms of every digit, one tile counter per
// pass, two per-segment block counters (keys/histogram and bounding box), and the
// look-back words of every (pass, tile, digit).
constexpr size_t sort_scratch_bytes(uint32_t segments, uint32_t tiles) {
    return sizeof(uint32_t) * ((size_t)segments * kMaxSortPasses * kMaxRadix + kMaxSortPasses + 2u * (size_t)segments +
                               (size_t)kMaxSortPasses * tiles * kMaxRadix);
}

// Bounding box of n positions into *out (reset first), for the pushed extent.
// Resets an extent accumulator (the pack kernel reduces the pushed positions into it).
void reset_extent(BoxAcc *out, cudaStream_t st);
void launch_sort(const SortLaunch &L, cudaStream_t st, uint32_t **sorted_keys, uint32_t **perm);
// Writes (write_runs = 1) or clears (0) the cell table of the sorted keys.  With `set`, the
// same launch reorders its streams into cell order: dst[i] = src[perm[i]] for every agent.
void launch_cell_table(const SortLaunch &L, const uint32_t *sorted_keys, int write_runs, cudaStream_t st,
                       const uint32_t *perm = nullptr, const GatherSet *set = nullptr);
// Runs one radix tile whose predecessor never publishes; returns the device error word.
cudaError_t selftest_sort_wait(uint32_t *err_host);

}  // namespace tgpu
