// Z-grid sort for a batch of segments: bounding box and grid, cell keys (3-D Morton or
// x-rows), a stable LSD radix sort of the keys (8- or 9-bit digits), the cell table, and the
// reorder of the structure-of-arrays streams into cell order.
//
// Replaces, for the GPU Z-grid, the reference's serial counting sort
// (tay/cpu_z_grid.c:156-221: count per cell, exclusive scan over every cell, memcpy of
// each AoS agent) and its OpenCL twin (tay/ocl_grid.c:43-209, whose order within a cell
// is not deterministic).  Here the order is deterministic and stable: agents in the
// same cell keep their previous relative order, as the reference's CPU sort does.
#include "tgpu_internal.cuh"
#include "tgpu_kernels.cuh"

namespace tgpu {

namespace {

TGPU_D uint32_t lane_id() { return threadIdx.x & 31u; }

template <typename T>
TGPU_D T warp_min(T v) {
    for (int o = 16; o > 0; o >>= 1) {
        T w = __shfl_xor_sync(0xffffffffu, v, o);
        v = w < v ? w : v;
    }
    return v;
}
template <typename T>
TGPU_D T warp_max(T v) {
    for (int o = 16; o > 0; o >>= 1) {
        T w = __shfl_xor_sync(0xffffffffu, v, o);
        v = w > v ? w : v;
    }
    return v;
}

// Mask of pass `pass`'s digit of D-bit digits (the last pass may have fewer bits).
template <int D>
TGPU_D uint32_t digit_mask(uint32_t key_bits, int pass) {
    const int bits = min(D, (int)key_bits - D * pass);
    return bits >= D ? (1u << D) - 1u : ((1u << bits) - 1u);
}

TGPU_D uint32_t warp_incl_scan(uint32_t v) {
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t w = __shfl_up_sync(0xffffffffu, v, o);
        if ((int)lane_id() >= o) v += w;
    }
    return v;
}

}  // namespace

// ------------------------------------------------------------------ bounding box

// Each segment's grid for this step from its box (or fixed box), with its rounding pad.
TGPU_D void write_grid(const SegmentSpec &sp, const BoxAcc &b, SegGrid *grids, uint32_t seg) {
    SegGrid out;
    out.g = segment_grid(sp, b);
    out.pad = grid_pad(out.g, sp, b);
    grids[seg] = out;
}

// Bounding box of the positions (the min corners of non-point agents) per segment, and
// for non-point agents (pos_max != nullptr) the largest box edge per axis, which widens
// every seer's search over the seen agents' min corners.  The segment's last block to
// finish (a counter in `done`, zeroed by box_reset_kernel) then derives its grid.
__global__ void __launch_bounds__(kSortThreads) bbox_kernel(const SegmentSpec *__restrict__ specs,
                                                            const uint32_t *__restrict__ tile_seg,
                                                            const float4 *__restrict__ pos,
                                                            const float4 *__restrict__ pos_max, BoxAcc *box,
                                                            SegGrid *__restrict__ grids, uint32_t *done) {
    const uint32_t seg = tile_seg[blockIdx.x];
    const SegmentSpec s = specs[seg];
    const uint32_t t = blockIdx.x - s.tile_begin;
    const uint32_t beg = s.begin + t * kSortTile;
    const uint32_t end = min(beg + (uint32_t)kSortTile, s.begin + s.count);
    __shared__ uint32_t red[6][kSortThreads / 32];
    __shared__ bool s_last;
    if (!s.fixed_box || pos_max) {
        uint32_t lo[3] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu};
        uint32_t hi[3] = {0u, 0u, 0u};
        uint32_t sz[3] = {0u, 0u, 0u};
#pragma unroll
        for (uint32_t k = 0; k < kSortTile / kSortThreads; ++k) {  // every load of the thread in flight
            const uint32_t i = beg + k * kSortThreads + threadIdx.x;
            if (i >= end) continue;
            float4 p = pos[i];
            float c[3] = {p.x, p.y, p.z};
            for (int a = 0; a < 3; ++a) {
                uint32_t o = float_to_ordered(c[a]);
                lo[a] = min(lo[a], o);
                hi[a] = max(hi[a], o);
            }
            if (pos_max) {
                const float4 q = pos_max[i];
                const float d[3] = {q.x - p.x, q.y - p.y, q.z - p.z};
                for (int a = 0; a < 3; ++a) sz[a] = max(sz[a], float_to_ordered(fmaxf(d[a], 0.0f)));
            }
        }
        if (pos_max) {
            for (int a = 0; a < 3; ++a) {
                const uint32_t v = warp_max(sz[a]);
                if (lane_id() == 0 && v) atomicMax(&box[seg].size[a], v);
            }
        }
        if (!s.fixed_box) {
            for (int a = 0; a < 3; ++a) {
                uint32_t l = warp_min(lo[a]);
                uint32_t h = warp_max(hi[a]);
                if (lane_id() == 0) {
                    red[a][threadIdx.x >> 5] = l;
                    red[3 + a][threadIdx.x >> 5] = h;
                }
            }
            __syncthreads();
            if (threadIdx.x < 32) {
                for (int a = 0; a < 3; ++a) {
                    uint32_t l = threadIdx.x < kSortThreads / 32 ? red[a][threadIdx.x] : 0xFFFFFFFFu;
                    uint32_t h = threadIdx.x < kSortThreads / 32 ? red[3 + a][threadIdx.x] : 0u;
                    l = warp_min(l);
                    h = warp_max(h);
                    if (threadIdx.x == 0) {
                        atomicMin(&box[seg].lo[a], l);
                        atomicMax(&box[seg].hi[a], h);
                    }
                }
            }
        }
    }
    // every thread's box updates ordered before the block counts itself done
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = atomicAdd(done + seg, 1u) == s.tile_count - 1u;
    __syncthreads();
    if (s_last && threadIdx.x == 0) {
        __threadfence();
        BoxAcc b;
        for (int a = 0; a < 3; ++a) {
            b.lo[a] = __ldcg(&box[seg].lo[a]);
            b.hi[a] = __ldcg(&box[seg].hi[a]);
            b.size[a] = __ldcg(&box[seg].size[a]);
        }
        write_grid(s, b, grids, seg);
    }
}

// Resets the box accumulators (and, with `done`, the bbox kernel's block counters); a
// segment without agents gets its grid here, from the reset box, since no bbox block
// runs for it.
__global__ void box_reset_kernel(BoxAcc *box, uint32_t segments, const SegmentSpec *__restrict__ specs,
                                 SegGrid *__restrict__ grids, uint32_t *done) {
    uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= segments) return;
    BoxAcc b;
    for (int a = 0; a < 3; ++a) {
        b.lo[a] = 0xFFFFFFFFu;
        b.hi[a] = 0u;
        b.size[a] = float_to_ordered(0.0f);
    }
    box[s] = b;
    if (done) {
        done[s] = 0u;
        const SegmentSpec sp = specs[s];
        if (sp.tile_count == 0) write_grid(sp, b, grids, s);
    }
}

// Each segment's grid from its box as it stands (restored boxes of recorded steps): one
// thread per segment.
__global__ void grid_kernel(const SegmentSpec *__restrict__ specs, const BoxAcc *__restrict__ box,
                            SegGrid *__restrict__ grids, uint32_t segments) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= segments) return;
    write_grid(specs[s], box[s], grids, s);
}

// ------------------------------------------------------------------ keys + histograms

// One segment's histograms become each digit's first output slot (the segment's begin
// plus the exclusive prefix over digits), pass by pass; run by one block of kSortThreads
// threads, each owning R / kSortThreads consecutive digits.  The counts are read from L2
// (other blocks added them).
template <uint32_t R>
TGPU_D void segment_digit_offsets(const SegmentSpec &s, uint32_t *seg_hist, int passes, uint32_t *warp_sums) {
    constexpr uint32_t kPer = R / kSortThreads;
    const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
    for (int p = 0; p < passes; ++p) {
        uint32_t *h = seg_hist + (size_t)p * kMaxRadix + threadIdx.x * kPer;
        uint32_t v[kPer], sum = 0;
#pragma unroll
        for (uint32_t k = 0; k < kPer; ++k) {
            v[k] = __ldcg(h + k);
            sum += v[k];
        }
        const uint32_t incl = warp_incl_scan(sum);
        if (lane == 31) warp_sums[warp] = incl;
        __syncthreads();
        if (warp == 0) {
            const uint32_t w = lane < kSortThreads / 32 ? warp_sums[lane] : 0u;
            const uint32_t wi = warp_incl_scan(w);
            if (lane < kSortThreads / 32) warp_sums[lane] = wi - w;
        }
        __syncthreads();
        uint32_t run = s.begin + warp_sums[warp] + incl - sum;
#pragma unroll
        for (uint32_t k = 0; k < kPer; ++k) {
            h[k] = run;
            run += v[k];
        }
        __syncthreads();
    }
}

// One pass over the positions: the cell key of every agent, and per-segment histograms of
// every D-bit digit of the keys (order-independent, so all passes' digit offsets are known
// before the first scatter).  The segment's last block to finish (a counter in `done`,
// zeroed with the histograms) turns its histograms into digit offsets.  hist layout:
// [segment][pass][kMaxRadix].
template <int D>
__global__ void __launch_bounds__(kSortThreads) keys_hist_kernel(const SegmentSpec *__restrict__ specs,
                                                                 const uint32_t *__restrict__ tile_seg,
                                                                 const SegGrid *__restrict__ grids,
                                                                 const float4 *__restrict__ pos,
                                                                 uint32_t *__restrict__ keys,
                                                                 uint32_t *__restrict__ hist, uint32_t *done,
                                                                 int passes, uint32_t key_bits) {
    constexpr uint32_t R = 1u << D;
    __shared__ uint32_t h[kMaxSortPasses][R];
    __shared__ uint32_t warp_sums[kSortThreads / 32];
    __shared__ bool s_last;
    const uint32_t seg = tile_seg[blockIdx.x];
    const SegmentSpec s = specs[seg];
    const Grid g = grids[seg].g;
    const uint32_t t = blockIdx.x - s.tile_begin;
    const uint32_t beg = s.begin + t * kSortTile;
    const uint32_t end = min(beg + (uint32_t)kSortTile, s.begin + s.count);
    for (int p = 0; p < passes; ++p)
        for (uint32_t d = threadIdx.x; d < R; d += kSortThreads) h[p][d] = 0;
    __syncthreads();
    const uint32_t lane = lane_id();
#pragma unroll
    for (uint32_t r = 0; r < kSortTile / kSortThreads; ++r) {  // every load of the thread in flight
        const uint32_t i = beg + r * kSortThreads + threadIdx.x;
        const bool live = i < end;
        const uint32_t m = __ballot_sync(0xffffffffu, live);  // warp-uniform: i grows with the lane
        if (!live) continue;
        float4 q = pos[i];
        uint32_t cx = (uint32_t)cell_coord(q.x, g.origin[0], g.inv_cs[0], g.dims[0]);
        uint32_t cy = (uint32_t)cell_coord(q.y, g.origin[1], g.inv_cs[1], g.dims[1]);
        uint32_t cz = (uint32_t)cell_coord(q.z, g.origin[2], g.inv_cs[2], g.dims[2]);
        uint32_t k = cell_key(s, cx, cy, cz);
        keys[i] = k;
        // A tile's agents are neighbours in space (last step's order), so most share their
        // upper digits: one shared atomic per distinct digit of the warp, not per agent.
        for (int p = 0; p < passes; ++p) {
            const uint32_t d = (k >> (D * p)) & digit_mask<D>(key_bits, p);
            const uint32_t peers = __match_any_sync(m, d);
            if (lane == (uint32_t)(__ffs(peers) - 1)) atomicAdd(&h[p][d], (uint32_t)__popc(peers));
        }
    }
    __syncthreads();
    uint32_t *seg_hist = hist + (size_t)seg * kMaxSortPasses * kMaxRadix;
    for (int p = 0; p < passes; ++p)
        for (uint32_t d = threadIdx.x; d < R; d += kSortThreads) {
            const uint32_t c = h[p][d];
            if (c) atomicAdd(&seg_hist[(size_t)p * kMaxRadix + d], c);
        }
    // every thread's counts ordered before the block counts itself done
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = atomicAdd(done + seg, 1u) == s.tile_count - 1u;
    __syncthreads();
    if (s_last) {
        __threadfence();
        segment_digit_offsets<R>(s, seg_hist, passes, warp_sums);
    }
}

// Decoupled look-back words: a count for one digit (kLookAgg) or an inclusive prefix
// (kLookPrefix), with the flag in the top two bits.
constexpr uint32_t kLookAgg = 1u << 30;
constexpr uint32_t kLookPrefix = 2u << 30;
constexpr uint32_t kLookValue = (1u << 30) - 1u;
constexpr uint32_t kLookSpinLimit = 1u << 20;  // polls of one predecessor word before giving up
// Tiles per look-back group: the last tile of each group of a segment publishes the
// group's count and then its inclusive prefix in its own slot, so that a later tile adds at
// most kLookGroup - 1 tile words of its own group and then one word per earlier group.
constexpr uint32_t kLookGroup = 16;

// Adds to excl[] the look-back words of `count` tiles: from, from - stride, ... (windows of
// up to 8 loaded together for every digit still open), stopping per digit at the first
// inclusive prefix (done[]).  A word not yet published is polled, bounded: a wait that
// runs out reports kErrSortLookback and counts as a prefix.
template <uint32_t kPer, uint32_t R>
TGPU_D void look_back(const uint32_t *tile_look, uint32_t from, uint32_t count, uint32_t stride, uint32_t d0,
                      uint32_t *excl, bool *done, uint32_t *err) {
    bool open = false;
#pragma unroll
    for (uint32_t k = 0; k < kPer; ++k) open = open || !done[k];
    for (uint32_t i = 0; i < count && open;) {
        const uint32_t n = min(8u, count - i);
        uint32_t v[kPer][8];
#pragma unroll
        for (uint32_t k = 0; k < kPer; ++k)
#pragma unroll
            for (uint32_t q = 0; q < 8; ++q)
                v[k][q] = (!done[k] && q < n)
                              ? *(const volatile uint32_t *)(tile_look + (size_t)(from - (i + q) * stride) * R + d0 + k)
                              : 0u;
        open = false;
#pragma unroll
        for (uint32_t k = 0; k < kPer; ++k) {
            for (uint32_t q = 0; q < n && !done[k]; ++q) {
                const volatile uint32_t *w = tile_look + (size_t)(from - (i + q) * stride) * R + d0 + k;
                uint32_t x = v[k][q];
                for (uint32_t spin = 0; (x >> 30) == 0u; ++spin) {
                    if (spin == kLookSpinLimit) {
                        atomicOr(err, kErrSortLookback);
                        break;
                    }
                    __nanosleep(32);
                    x = *w;
                }
                excl[k] += x & kLookValue;
                if ((x >> 30) != 1u) done[k] = true;  // an inclusive prefix (or a wait that ran out)
            }
            open = open || !done[k];
        }
        i += n;
    }
}

// One radix pass as a single kernel (the "onesweep" scheme): a block takes the next tile in
// input order from an atomic counter, counts its 2048 keys per digit, publishes the counts,
// ranks its keys stably (8 warps, each owning 256 consecutive items in 8 rounds of 32:
// __match_any_sync ranks and per-warp running digit counts), and finds its per-digit output
// offsets by looking back over the earlier tiles of its segment (the segment's first tile
// starts from the segment's digit offsets).  The look-back is two-level: a tile adds the
// words of the earlier tiles of its group of kLookGroup, then one word per earlier group
// (its last tile's slot: the group's count, then its inclusive prefix), so the chain a tile
// may wait along grows with the number of groups, not of tiles.  Tiles take ids in order
// and wait only on lower ids, so every tile a block waits for is already running; each wait
// is bounded and reports kErrSortLookback through *err when it runs out.  D-bit digits
// (R = 2^D bins); each thread owns R / 256 consecutive digits for the per-digit work, and
// looks back for all of them together.
template <int D>
__global__ void __launch_bounds__(kSortThreads, 4) onesweep_kernel(const SegmentSpec *__restrict__ specs,
                                                                const uint32_t *__restrict__ tile_seg,
                                                                const uint32_t *__restrict__ keys_in,
                                                                const uint32_t *__restrict__ vals_in,
                                                                uint32_t *__restrict__ keys_out,
                                                                uint32_t *__restrict__ vals_out,
                                                                const uint32_t *__restrict__ hist,
                                                                uint32_t *__restrict__ look, uint32_t *tile_ctr,
                                                                uint32_t *err, int pass, uint32_t mask) {
    constexpr uint32_t R = 1u << D;
    constexpr uint32_t kPer = R / kSortThreads;  // digits per thread
    constexpr int kWarps = kSortThreads / 32;
    constexpr int kRounds = kSortTile / kSortThreads;
    __shared__ uint32_t warp_hist[kWarps][R];
    __shared__ uint32_t digit_base[R];
    __shared__ uint32_t local_start[R];
    __shared__ uint32_t warp_sums[kWarps];
    __shared__ uint32_t keys_s[kSortTile], vals_s[kSortTile];
    __shared__ uint32_t tile_hist[R];
    __shared__ uint32_t s_tile;
    if (threadIdx.x == 0) s_tile = atomicAdd(tile_ctr + pass, 1u);
    for (uint32_t i = threadIdx.x; i < kWarps * R; i += kSortThreads) (&warp_hist[0][0])[i] = 0;
    for (uint32_t d = threadIdx.x; d < R; d += kSortThreads) tile_hist[d] = 0;
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint32_t seg = tile_seg[tile];
    const SegmentSpec s = specs[seg];
    const uint32_t t = tile - s.tile_begin;
    const uint32_t beg = s.begin + t * kSortTile;
    const uint32_t end = min(beg + (uint32_t)kSortTile, s.begin + s.count);
    const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
    const int shift = D * pass;
    const uint32_t *seg_hist = hist + ((size_t)seg * kMaxSortPasses + pass) * kMaxRadix;
    uint32_t *tile_look = look + ((size_t)pass * gridDim.x) * R;  // [tile][R] of this pass
    const uint32_t d0 = threadIdx.x * kPer;                         // this thread's first digit
    const uint32_t g0 = tile - t % kLookGroup;                      // first tile of this tile's group
    const bool group_last = t % kLookGroup == kLookGroup - 1u || t + 1u == s.tile_count;

    uint32_t key[kRounds], val[kRounds], rank[kRounds], dig[kRounds], peer[kRounds];
    // the tile's digit counts first, published before the ranking so that later tiles
    // find them when they look back
#pragma unroll
    for (int r = 0; r < kRounds; ++r) {
        const uint32_t i = beg + warp * (kSortTile / kWarps) + r * 32 + lane;
        key[r] = i < end ? keys_in[i] : 0u;
        dig[r] = i < end ? ((key[r] >> shift) & mask) : R;
    }
#pragma unroll
    for (int r = 0; r < kRounds; ++r) {
        // one shared atomic per distinct digit of the warp (a tile's keys share their upper
        // digits, which per-key atomics would serialize on one address); the lanes with
        // the same digit are kept for the ranking
        peer[r] = __match_any_sync(0xffffffffu, dig[r]);
        if (dig[r] < R && lane == (uint32_t)(__ffs(peer[r]) - 1)) atomicAdd(&tile_hist[dig[r]], (uint32_t)__popc(peer[r]));
    }
    __syncthreads();
    uint32_t cnt[kPer], excl[kPer];
#pragma unroll
    for (uint32_t k = 0; k < kPer; ++k) {
        cnt[k] = tile_hist[d0 + k];
        excl[k] = t == 0 ? seg_hist[d0 + k] : 0u;
        volatile uint32_t *mine = tile_look + (size_t)tile * R + d0 + k;
        if (t == 0)
            *mine = kLookPrefix | ((excl[k] + cnt[k]) & kLookValue);
        else if (!group_last)
            *mine = kLookAgg | cnt[k];  // (a group's last tile publishes the group's count below)
    }
#pragma unroll
    for (int r = 0; r < kRounds; ++r) {
        const uint32_t i = beg + warp * (kSortTile / kWarps) + r * 32 + lane;
        const bool valid = i < end;
        const uint32_t k = key[r];
        const uint32_t d = dig[r];
        const uint32_t peers = peer[r];
        const uint32_t below = __popc(peers & ((1u << lane) - 1u));
        const uint32_t before = valid ? warp_hist[warp][d] : 0u;
        __syncwarp();
        if (valid && below == 0) warp_hist[warp][d] = before + __popc(peers);
        __syncwarp();
        key[r] = k;
        val[r] = valid ? (vals_in ? vals_in[i] : i) : 0u;
        rank[r] = before + below;
        dig[r] = d;
    }
    __syncthreads();
    // the look-back, after the ranking: by then the earlier tiles have published their
    // counts, and most their prefixes
    if (t != 0) {
        bool done[kPer];
#pragma unroll
        for (uint32_t k = 0; k < kPer; ++k) done[k] = false;
        // the earlier tiles of this group (tile words)
        look_back<kPer, R>(tile_look, tile - 1u, tile - g0, 1u, d0, excl, done, err);
        if (group_last) {
#pragma unroll
            for (uint32_t k = 0; k < kPer; ++k)
                if (!done[k]) *(volatile uint32_t *)(tile_look + (size_t)tile * R + d0 + k) = kLookAgg | (excl[k] + cnt[k]);
        }
        // the earlier groups (their last tiles' slots)
        look_back<kPer, R>(tile_look, g0 - 1u, (g0 - s.tile_begin) / kLookGroup, kLookGroup, d0, excl, done, err);
#pragma unroll
        for (uint32_t k = 0; k < kPer; ++k) {
            // counts only, down to the segment's first tile: start from its digit offsets
            if (!done[k]) excl[k] += seg_hist[d0 + k];
            *(volatile uint32_t *)(tile_look + (size_t)tile * R + d0 + k) = kLookPrefix | ((excl[k] + cnt[k]) & kLookValue);
        }
    }
    {
        // per digit (kPer consecutive ones per thread): prefix over warps, then the tile's
        // own digit-sorted layout (exclusive scan of its digit counts)
        uint32_t sum = 0;
#pragma unroll
        for (uint32_t k = 0; k < kPer; ++k) {
            uint32_t acc = 0;
            for (int w = 0; w < kWarps; ++w) {
                const uint32_t c = warp_hist[w][d0 + k];
                warp_hist[w][d0 + k] = acc;
                acc += c;
            }
            digit_base[d0 + k] = excl[k];
            sum += cnt[k];
        }
        const uint32_t incl = warp_incl_scan(sum);
        if (lane == 31) warp_sums[warp] = incl;
        __syncthreads();
        uint32_t before = 0;
        for (uint32_t w = 0; w < warp; ++w) before += warp_sums[w];
        uint32_t start = before + incl - sum;
#pragma unroll
        for (uint32_t k = 0; k < kPer; ++k) {
            local_start[d0 + k] = start;
            start += cnt[k];
        }
    }
    __syncthreads();
    // stage the tile in digit order, then write runs of equal digits to consecutive
    // global slots (coalesced), not one sector per key
#pragma unroll
    for (int r = 0; r < kRounds; ++r) {
        if (dig[r] < R) {
            const uint32_t j = local_start[dig[r]] + warp_hist[warp][dig[r]] + rank[r];
            keys_s[j] = key[r];
            vals_s[j] = val[r];
        }
    }
    __syncthreads();
    const uint32_t count = end - beg;
#pragma unroll
    for (int r = 0; r < kRounds; ++r) {
        const uint32_t j = (uint32_t)r * kSortThreads + threadIdx.x;
        if (j < count) {
            const uint32_t k = keys_s[j];
            const uint32_t dd = (k >> shift) & mask;
            const uint32_t p = digit_base[dd] + (j - local_start[dd]);
            keys_out[p] = k;
            vals_out[p] = vals_s[j];
        }
    }
}

// ------------------------------------------------------------------ cell table

constexpr uint32_t kTableBlocks = kSortTile / kSortThreads;

// Records {first, end} of every run of equal keys at the run's cell (write_runs = 1), or
// clears those entries again (write_runs = 0) before the next sort.  Row order: the first
// agent of each cell writes its index into the start entries of the empty cells before
// it in its row and its own; the last agent of a row writes the row's end into the
// entries after its cell; a row's first agent clears the whole row.
// With perm, the launch also reorders the streams of `set` into cell order (the reorder
// of the reference's sort, which copies each agent to its slot).
__global__ void __launch_bounds__(kSortThreads) cell_table_kernel(const SegmentSpec *__restrict__ specs,
                                                                  const uint32_t *__restrict__ tile_seg,
                                                                  const SegGrid *__restrict__ grids,
                                                                  const uint32_t *__restrict__ keys,
                                                                  uint2 *__restrict__ table, int write_runs,
                                                                  const uint32_t *__restrict__ perm, GatherSet set) {
    // kTableBlocks blocks per radix tile, one key per thread
    const uint32_t tile = blockIdx.x / kTableBlocks, part = blockIdx.x % kTableBlocks;
    const uint32_t seg = tile_seg[tile];
    const SegmentSpec s = specs[seg];
    const uint32_t dx = (uint32_t)grids[seg].g.dims[0], dy = (uint32_t)grids[seg].g.dims[1];
    const uint32_t beg = s.begin + (tile - s.tile_begin) * kSortTile + part * kSortThreads;
    const uint32_t seg_end = s.begin + s.count;
    const uint32_t end = min(beg + (uint32_t)kSortThreads, seg_end);
    const uint32_t i = beg + threadIdx.x;
    if (perm && i < end) {
        const uint32_t src = perm[i];
#pragma unroll
        for (int c = 0; c < kMaxF4; ++c)
            if (c < set.nf4) set.dst_f4[c][i] = __ldg(set.src_f4[c] + src);
#pragma unroll
        for (int c = 0; c < kMaxU32; ++c)
            if (c < set.nu32) set.dst_u32[c][i] = __ldg(set.src_u32[c] + src);
    }
    if (s.order == kOrderRows) {
        // The first agent of a row writes its header's x_first / first, the last agent
        // x_last / end, and the first agent of every other cell the start entries of the
        // cells after the previous occupied one up to its own; the clear zeroes headers
        // (entries are read only inside a row's occupied span, where every step writes them).
        // A gap of up to kLaneGap entries is written by its own lane; longer ones by the
        // warp together, 32 consecutive entries per store.
        constexpr uint32_t kLaneGap = 32;
        uint4 *hdr = reinterpret_cast<uint4 *>(table + s.table_base);
        uint32_t *words = reinterpret_cast<uint32_t *>(table + s.table_base) + row_entry_word(s);
        const uint32_t b = axis_bits(s);
        const uint32_t xmask = (1u << b) - 1u;
        const uint32_t lane = threadIdx.x & 31u;
        uint32_t off = 0u, len = 0u;
        if (i < end) {
            const uint32_t k = keys[i];
            const uint32_t row = k >> b, x = k & xmask;
            const uint32_t kp = i == s.begin ? ~k : keys[i - 1];
            const bool row_first = (kp >> b) != row;
            const bool row_last = (i + 1 == seg_end) || (keys[i + 1] >> b) != row;
            uint32_t ry, rz;
            row_of_code(s, row, ry, rz);
            const uint32_t r = rz * dy + ry;
            if (!write_runs) {
                if (row_first) hdr[r] = make_uint4(0u, 0u, 0u, 0u);
            } else {
                uint32_t *h = reinterpret_cast<uint32_t *>(hdr + r);
                if (row_first) {
                    h[0] = x;
                    h[2] = i;
                } else if (kp != k) {
                    const uint32_t x0 = (kp & xmask) + 1u;
                    off = r * dx + x0;
                    len = x + 1u - x0;
                    if (len <= kLaneGap) {
                        for (uint32_t c = 0; c < len; ++c) words[off + c] = i;
                        len = 0u;
                    }
                }
                if (row_last) {
                    h[1] = x;
                    h[3] = i + 1u;
                }
            }
        }
        uint32_t m = __ballot_sync(0xffffffffu, len > 0u);
        while (m) {
            const int l = __ffs(m) - 1;
            m &= m - 1u;
            const uint32_t o = __shfl_sync(0xffffffffu, off, l);
            const uint32_t n = __shfl_sync(0xffffffffu, len, l);
            const uint32_t v = __shfl_sync(0xffffffffu, i, l);
            for (uint32_t c = lane; c < n; c += 32u) words[o + c] = v;
        }
        return;
    }
    if (i < end) {
        const uint32_t k = keys[i];
        const bool first = (i == s.begin) || keys[i - 1] != k;
        const bool last = (i + 1 == seg_end) || keys[i + 1] != k;
        if (!first && !last) return;
        uint2 *e = table + s.table_base + ((compact10(k >> 2) * dy + compact10(k >> 1)) * dx + compact10(k));
        if (write_runs) {
            if (first) e->x = i;
            if (last) e->y = i + 1;
        } else if (first) {
            *e = make_uint2(0u, 0u);
        }
    }
}

// ------------------------------------------------------------------ host-side launchers

void reset_extent(BoxAcc *out, cudaStream_t st) {
    box_reset_kernel<<<1, 32, 0, st>>>(out, 1, nullptr, nullptr, nullptr);
}

namespace {

// The sort scratch (sort_scratch_bytes): digit histograms [segments][kMaxSortPasses]
// [kMaxRadix], tile counters [kMaxSortPasses], the keys/histogram kernel's block counters
// [segments], the bbox kernel's block counters [segments], then the look-back words
// [pass][tile][radix].
struct Scratch {
    uint32_t *hist, *tile_ctr, *hist_done, *box_done, *look;
};
Scratch scratch_of(const SortLaunch &L) {
    Scratch c;
    c.hist = L.sort_scratch;
    c.tile_ctr = c.hist + (size_t)L.segments * kMaxSortPasses * kMaxRadix;
    c.hist_done = c.tile_ctr + kMaxSortPasses;
    c.box_done = c.hist_done + L.segments;
    c.look = c.box_done + L.segments;
    return c;
}

}  // namespace

void launch_box(const SortLaunch &L, cudaStream_t st) {
    const Scratch c = scratch_of(L);
    box_reset_kernel<<<(L.segments + 127) / 128, 128, 0, st>>>(L.box, L.segments, L.specs, L.grids, c.box_done);
    bbox_kernel<<<L.tiles, kSortThreads, 0, st>>>(L.specs, L.tile_seg, L.pos, L.pos_max, L.box, L.grids,
                                                  c.box_done);
}

void launch_grids(const SortLaunch &L, cudaStream_t st) {
    grid_kernel<<<(L.segments + 127) / 128, 128, 0, st>>>(L.specs, L.box, L.grids, L.segments);
}

// Sorts the keys of every segment; on return *sorted_keys / *perm point at the buffers
// holding the sorted keys and the permutation (sorted slot -> previous slot).
template <int D>
void launch_sort_digits(const SortLaunch &L, cudaStream_t st, uint32_t **sorted_keys, uint32_t **perm) {
    constexpr uint32_t R = 1u << D;
    uint32_t *kin = L.keys[0], *kout = L.keys[1];
    uint32_t *vin = nullptr, *vout = L.vals[1];
    const int passes = sort_passes(L.key_bits);
    const Scratch c = scratch_of(L);
    uint32_t *hist = c.hist, *tile_ctr = c.tile_ctr, *look = c.look;
    // zero the histograms, the counters and the look-back words of the passes used
    cudaMemsetAsync(L.sort_scratch, 0, sizeof(uint32_t) * ((size_t)(look - L.sort_scratch) + (size_t)passes * L.tiles * R),
                    st);
    keys_hist_kernel<D><<<L.tiles, kSortThreads, 0, st>>>(L.specs, L.tile_seg, L.grids, L.pos, kin, hist,
                                                          c.hist_done, passes, L.key_bits);
    for (int p = 0; p < passes; ++p) {
        const int bits = std::min(D, (int)L.key_bits - D * p);
        onesweep_kernel<D><<<L.tiles, kSortThreads, 0, st>>>(L.specs, L.tile_seg, kin, vin, kout, vout, hist, look,
                                                             tile_ctr, L.err, p, (1u << bits) - 1u);
        // ping-pong: the next pass reads what this one wrote
        uint32_t *tk = kin;
        kin = kout;
        kout = tk;
        if (p == 0) {
            vin = vout;
            vout = L.vals[0];
        } else {
            uint32_t *tv = vin;
            vin = vout;
            vout = tv;
        }
    }
    *sorted_keys = kin;
    *perm = vin;
}

void launch_sort(const SortLaunch &L, cudaStream_t st, uint32_t **sorted_keys, uint32_t **perm) {
    if (sort_digit_bits(L.key_bits) == 9)
        launch_sort_digits<9>(L, st, sorted_keys, perm);
    else
        launch_sort_digits<8>(L, st, sorted_keys, perm);
}

// Self-test of the look-back's bounded wait: one block takes tile 1 of a two-tile segment
// whose tile 0 never publishes, so every digit's wait runs out (each after kLookSpinLimit
// polls, well under a second) and the kernel reports kErrSortLookback in *err and returns.
// All accesses stay inside the buffers given (2 tiles of keys, values and look-back words).
cudaError_t selftest_sort_wait(uint32_t *err_host) {
    SegmentSpec spec{};
    spec.begin = 0;
    spec.count = 2u * kSortTile;
    spec.tile_begin = 0;
    spec.tile_count = 2;
    const uint32_t tile_seg[2] = {0u, 0u};
    const size_t hist_words = (size_t)kMaxSortPasses * kMaxRadix;
    SegmentSpec *d_spec = nullptr;
    uint32_t *d_tile_seg = nullptr, *d_keys = nullptr, *d_out = nullptr, *d_hist = nullptr, *d_look = nullptr,
             *d_ctr = nullptr, *d_err = nullptr;
    cudaError_t e = cudaMalloc(&d_spec, sizeof(spec));
    if (e == cudaSuccess) e = cudaMalloc(&d_tile_seg, sizeof(tile_seg));
    if (e == cudaSuccess) e = cudaMalloc(&d_keys, sizeof(uint32_t) * 2 * kSortTile);
    if (e == cudaSuccess) e = cudaMalloc(&d_out, sizeof(uint32_t) * 4 * kSortTile);
    if (e == cudaSuccess) e = cudaMalloc(&d_hist, sizeof(uint32_t) * hist_words);
    if (e == cudaSuccess) e = cudaMalloc(&d_look, sizeof(uint32_t) * 2 * 256u);
    if (e == cudaSuccess) e = cudaMalloc(&d_ctr, sizeof(uint32_t) * kMaxSortPasses);
    if (e == cudaSuccess) e = cudaMalloc(&d_err, sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemcpy(d_spec, &spec, sizeof(spec), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d_tile_seg, tile_seg, sizeof(tile_seg), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(d_keys, 0, sizeof(uint32_t) * 2 * kSortTile);
    if (e == cudaSuccess) e = cudaMemset(d_hist, 0, sizeof(uint32_t) * hist_words);
    if (e == cudaSuccess) e = cudaMemset(d_look, 0, sizeof(uint32_t) * 2 * 256u);
    if (e == cudaSuccess) e = cudaMemset(d_err, 0, sizeof(uint32_t));
    // the tile counter starts at 1: the single block is tile 1 and waits for tile 0
    const uint32_t ctr[kMaxSortPasses] = {1u, 0u, 0u, 0u};
    if (e == cudaSuccess) e = cudaMemcpy(d_ctr, ctr, sizeof(ctr), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        // gridDim.x = 1 but tile = 1: the look-back words of tile t sit at t * 256 (two
        // tiles' worth allocated), keys and values out of tile 1 land in [0, 2 * kSortTile)
        onesweep_kernel<8><<<1, kSortThreads>>>(d_spec, d_tile_seg, d_keys, nullptr, d_out, d_out + 2 * kSortTile,
                                                d_hist, d_look, d_ctr, d_err, 0, 0xFFu);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(err_host, d_err, sizeof(uint32_t), cudaMemcpyDeviceToHost);
    cudaFree(d_spec);
    cudaFree(d_tile_seg);
    cudaFree(d_keys);
    cudaFree(d_out);
    cudaFree(d_hist);
    cudaFree(d_look);
    cudaFree(d_ctr);
    cudaFree(d_err);
    return e;
}

void launch_cell_table(const SortLaunch &L, const uint32_t *sorted_keys, int write_runs, cudaStream_t st,
                       const uint32_t *perm, const GatherSet *set) {
    const GatherSet none{};
    cell_table_kernel<<<L.tiles * kTableBlocks, kSortThreads, 0, st>>>(
        L.specs, L.tile_seg, L.grids, sorted_keys, L.table, write_runs, set ? perm : nullptr, set ? *set : none);
}

}  // namespace tgpu
