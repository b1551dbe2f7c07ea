// See-pass and act-pass kernel templates.
//
// See pass (replaces tay/cpu_z_grid.c:232-321 + tay/space.c:106-148, and the generated
// OpenCL see kernel, tay/ocl_grid.c:376-417 + tay/ocl_generics.c:13-114):
//   * one CTA = 128 consecutive seers in cell order (never crossing a segment), one seer
//     per thread;
//   * each seer's neighbour cells are the cells overlapping its box p +- r (padded by a
//     fraction of a cell against rounding), clamped to the grid;
//   * row order (see_rows_kernel, the default): each lane walks its own rows of cells,
//     one contiguous candidate range per (y, z) row found from the row table, reading the
//     candidates through L1; Morton order (see_kernel): cell by cell;
//   * every candidate gets the reference's inclusive per-axis box test (space.c:62-68:
//     skip when d < -r || d > r, d = seer - seen) and, when it passes, the model's see
//     function on registers: no atomics on agent state, the seer writes only its own
//     accumulators; a fused act runs in the epilogue;
//   * tunings: a warp walks the union of its lanes' boxes with hit masks (union_factor,
//     hit_masks), or the CTA first copies its union rows (row order, TMA bulk copies) or
//     cells (Morton) into shared memory (stage); and a write-through instance stores the
//     finished records to page-locked host memory from the epilogue;
//   * pair lists: a pass can record each seer's kept candidates for the next pass over the
//     same positions, which runs its see function over them instead of walking the rows
//     (SPH density -> force); every walk and the replay visit a seer's neighbours in the
//     same order, so they give the same bits.
// Act pass (replaces tay/space.c:250-263): one thread per agent.
#pragma once

#include <climits>
#include <type_traits>

#include "tgpu_internal.cuh"
#include "tgpu_kernels.cuh"

namespace tgpu {

namespace see_detail {

TGPU_D int warp_min_i(int v) {
    for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
TGPU_D int warp_max_i(int v) {
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
TGPU_D uint32_t warp_sum_u(uint32_t v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Cell range along one axis for the interval [p - r, p + r], widened by `pad` cells on
// each side so that rounding in the key computation can never put a neighbour that
// passes the box test outside the range.
TGPU_D void axis_range(float p, float r, float origin, float inv_cs, int dim, float pad, int &lo, int &hi) {
    float a = ((p - r) - origin) * inv_cs - pad;
    float b = ((p + r) - origin) * inv_cs + pad;
    int l = (int)floorf(a), h = (int)floorf(b);
    lo = l < 0 ? 0 : (l >= dim ? dim - 1 : l);
    hi = h < 0 ? 0 : (h >= dim ? dim - 1 : h);
}

// Cell range along one axis for the interval [lo_v, hi_v] (a seer's search interval over
// the seen agents' positions), widened by `pad` cells as in axis_range.
TGPU_D void axis_span(float lo_v, float hi_v, float origin, float inv_cs, int dim, float pad, int &lo, int &hi) {
    float a = (lo_v - origin) * inv_cs - pad;
    float b = (hi_v - origin) * inv_cs + pad;
    int l = (int)floorf(a), h = (int)floorf(b);
    lo = l < 0 ? 0 : (l >= dim ? dim - 1 : l);
    hi = h < 0 ? 0 : (h >= dim ? dim - 1 : h);
}

// Non-point seer over non-point seen agents (tay/space.c:92-103): skipped when on any
// axis seer_min - seen_max > r or seen_min - seer_max > r.
TGPU_D bool boxes_hit(const float4 &amin, const float4 &amax, const float4 &bmin, const float4 &bmax, const float4 &r) {
    return !(amin.x - bmax.x > r.x) && !(bmin.x - amax.x > r.x) && !(amin.y - bmax.y > r.y) &&
           !(bmin.y - amax.y > r.y) && !(amin.z - bmax.z > r.z) && !(bmin.z - amax.z > r.z);
}

// Whether pass P runs over non-point (box) agents: P::kBox when it declares one.
template <class P, class = void>
struct BoxOf {
    static constexpr bool value = false;
};
template <class P>
struct BoxOf<P, decltype((void)P::kBox)> {
    static constexpr bool value = P::kBox;
};

// Inclusive per-axis box test of the reference: a pair is skipped when any
// d = seer - seen satisfies d < -r || d > r, i.e. |d| > r (NaN compares false both ways).
TGPU_D bool box_hit(const float4 &a, const float4 &b, const float4 &r) {
    return !(fabsf(a.x - b.x) > r.x) && !(fabsf(a.y - b.y) > r.y) && !(fabsf(a.z - b.z) > r.z);
}

struct SmemSeen {
    static constexpr bool kGlobal = false;
    const float4 *base;
    uint32_t cap;
    TGPU_D float4 f4(int k, uint32_t j) const { return base[(uint32_t)k * cap + j]; }
};

template <int N>
struct GlobalSeen {
    static constexpr bool kGlobal = true;
    const float4 *s[N];
    TGPU_D float4 f4(int k, uint32_t j) const { return __ldg(s[k] + j); }
};

// Loads a candidate position from shared memory (staged) or through the read-only cache.
TGPU_D float4 load_pos(const float4 *src, uint32_t j, bool global) {
    return global ? __ldg(src + j) : src[j];
}

// A pass's role in a pair list (PairList): P::kPairList when it declares one, else 0.
template <class P, class = void>
struct ListOf {
    static constexpr int value = 0;
};
template <class P>
struct ListOf<P, decltype((void)P::kPairList)> {
    static constexpr int value = P::kPairList;
};

// The walk of a pass that records no pair list.
struct NoRec {};

// One seer's pair-list recorder: box-test passes with agents other than itself, and the
// candidates the model keeps (P::keep), appended in walk order up to the capacity (the
// count keeps growing past it, which marks the list incomplete).  Each entry goes straight
// to its word of its group of four (measured faster than staging the group in shared
// memory and storing it whole); a partial last group's other words are never read.
struct ListRec {
    uint4 *idx;
    uint32_t stride, cap, seer, n, other;
};

template <class P>
TGPU_D void record_pair(ListRec &r, const float4 &a, const float4 &b, uint32_t j, const typename P::SeeCtx &c) {
    r.other += j != r.seer ? 1u : 0u;
    if (P::keep(a, b, c)) {
        if (r.n < r.cap)
            reinterpret_cast<uint32_t *>(r.idx)[((size_t)(r.n >> 2) * r.stride + r.seer) * 4u + (r.n & 3u)] = j;
        ++r.n;
    }
}

// Union walk over candidates [j0, j1) of `src`: batches of up to 32, a box-test phase
// into per-lane hit masks (all lanes read the same candidate), then a see phase in which
// every lane with hits runs the see function on its next hit (each lane's hits in the
// order of its own walk).
template <class P, class Acc>
TGPU_D void union_batches(typename P::Seer &s, const float4 &sp, const float4 &r4, bool active, uint32_t j0,
                          uint32_t j1, uint32_t self, const float4 *src, const Acc &acc,
                          const typename P::SeeCtx &sctx, uint32_t &pairs, uint32_t &tested) {
    constexpr bool kGlobal = Acc::kGlobal;
    for (uint32_t jb = j0; jb < j1; jb += 32) {
        const uint32_t nb = min(32u, j1 - jb);
        if (active) tested += nb;
        uint32_t hits = 0;
#pragma unroll 8
        for (uint32_t k = 0; k < nb; ++k) {
            const float4 bp = load_pos(src, jb + k, kGlobal);
            hits |= (uint32_t)(box_hit(sp, bp, r4) && jb + k != self) << k;
        }
        if (!active) hits = 0;
        pairs += __popc(hits);
        while (__any_sync(0xffffffffu, hits != 0)) {
            if (hits) {
                const uint32_t j = jb + (uint32_t)(__ffs(hits) - 1);
                hits &= hits - 1u;
                P::see(s, sp, load_pos(src, j, kGlobal), acc, j, sctx);
            }
        }
    }
}

// Candidates a lane loads per iteration of its walk: P::kLaneUnroll when the pass
// declares one (light see bodies gain from more loads in flight), else 2.
template <class P, class = void>
struct UnrollOf {
    static constexpr int value = 2;
};
template <class P>
struct UnrollOf<P, decltype((void)P::kLaneUnroll)> {
    static constexpr int value = P::kLaneUnroll;
};

// Whether pass P gates its see body on its keep test (P::kKeepGate): the see function
// does nothing for a pair that passed the box test but not P::keep, so the walk counts the
// box-test pass without a branch and enters the body (and the recorder) only for kept
// pairs.  The gated walk tests the seer like any other candidate (it lies in its own range
// and is met exactly once) and takes its box-test pass off the counter at the end when the
// pass skips self.  When keep(a, a) is false (P::kKeepRejectsSelf: a distance test with
// d2 > 0) no index is compared with the seer's; otherwise only kept candidates are.
template <class P, class = void>
struct GateOf {
    static constexpr bool value = false;
};
template <class P>
struct GateOf<P, decltype((void)P::kKeepGate)> {
    static constexpr bool value = P::kKeepGate;
};
template <class P, class = void>
struct SelfSafeOf {
    static constexpr bool value = false;
};
template <class P>
struct SelfSafeOf<P, decltype((void)P::kKeepRejectsSelf)> {
    static constexpr bool value = P::kKeepRejectsSelf;
};

// The direction of the difference a gated pass's keep and see functions compute: seen -
// seer when P::kSeenMinusSeer (boids), else seer - seen (the reference's d); the gated box
// test computes the same one (|d| is the same float either way), so the compiler shares it.
template <class P, class = void>
struct SeenMinusSeerOf {
    static constexpr bool value = false;
};
template <class P>
struct SeenMinusSeerOf<P, decltype((void)P::kSeenMinusSeer)> {
    static constexpr bool value = P::kSeenMinusSeer;
};

// A kept candidate into the recorder's list (the gated walk counts box-test passes itself).
TGPU_D void record_kept(ListRec &r, uint32_t j) {
    if (r.n < r.cap) reinterpret_cast<uint32_t *>(r.idx)[((size_t)(r.n >> 2) * r.stride + r.seer) * 4u + (r.n & 3u)] = j;
    ++r.n;
}

// One candidate of a lane's walk: the reference's box test and self skip, the pair
// counter, the recorder, and the see function (behind P::keep when the pass gates on it).
template <class P, bool kGate, class Acc, class Rec>
TGPU_D void lane_one(typename P::Seer &s, const float4 &sp, const float4 &b, const float4 &r4, uint32_t j,
                     uint32_t self, const Acc &acc, const typename P::SeeCtx &sctx, uint32_t &pairs, Rec *rec) {
    constexpr bool kRec = std::is_same_v<Rec, ListRec>;
    if constexpr (kGate) {
        // the reference's test on d = seer - seen, computed in the direction the model's keep
        // and see use (|seen - seer| is the same float), so the compiler shares it
        bool hit;
        if constexpr (SeenMinusSeerOf<P>::value)
            hit = !(fabsf(b.x - sp.x) > r4.x) && !(fabsf(b.y - sp.y) > r4.y) && !(fabsf(b.z - sp.z) > r4.z);
        else
            hit = !(fabsf(sp.x - b.x) > r4.x) && !(fabsf(sp.y - b.y) > r4.y) && !(fabsf(sp.z - b.z) > r4.z);
        pairs += hit ? 1u : 0u;
        if (hit && (SelfSafeOf<P>::value || j != self) && P::keep(sp, b, sctx)) {
            if constexpr (kRec) record_kept(*rec, j);
            P::see(s, sp, b, acc, j, sctx);
        }
    } else {
        if (j != self && box_hit(sp, b, r4)) {
            ++pairs;
            if constexpr (kRec) record_pair<P>(*rec, sp, b, j, sctx);
            P::see(s, sp, b, acc, j, sctx);
        }
    }
}

// Per-lane walk over candidates [j0, j1): UnrollOf<P> candidates per iteration for
// independent loads in flight; a recording pass passes its recorder as `rec`; kGate: the
// keep-gated candidate step (GateOf).
template <class P, class Acc, class Rec = NoRec, bool kGate = false>
TGPU_D void lane_run(typename P::Seer &s, const float4 &sp, const float4 &r4, uint32_t j0, uint32_t j1, uint32_t self,
                     const float4 *src, const Acc &acc, const typename P::SeeCtx &sctx, uint32_t &pairs,
                     uint32_t &tested, Rec *rec = nullptr) {
    constexpr bool kGlobal = Acc::kGlobal;
    constexpr int U = UnrollOf<P>::value;
    if (j1 <= j0) return;
    tested += j1 - j0;
    uint32_t j = j0;
    // counted on the remaining length, not on j + U - 1, which can wrap for indices
    // near 2^32 (ranges translated into staged slots)
    for (; j1 - j >= (uint32_t)U; j += U) {
        float4 b[U];
#pragma unroll
        for (int u = 0; u < U; ++u) b[u] = load_pos(src, j + u, kGlobal);
#pragma unroll
        for (int u = 0; u < U; ++u) lane_one<P, kGate>(s, sp, b[u], r4, j + u, self, acc, sctx, pairs, rec);
    }
    // the last j1 - j < U candidates: their loads issued together (indices clamped into the
    // range, so every load is in bounds), then tested in order
    const uint32_t rem = j1 - j;
    if (rem) {
        float4 b[U];
#pragma unroll
        for (int u = 0; u < U; ++u) b[u] = load_pos(src, j + min((uint32_t)u, rem - 1u), kGlobal);
#pragma unroll
        for (int u = 0; u < U - 1; ++u)
            if ((uint32_t)u < rem) lane_one<P, kGate>(s, sp, b[u], r4, j + u, self, acc, sctx, pairs, rec);
    }
}

// Replay of a recorded pair list: the see function over the seer's n entries in their
// recorded order, one group of four per load, two positions loaded ahead; words past the
// n-th are never used; the seer itself is skipped when the pass skips self.
template <class P, class Acc>
TGPU_D void list_run(typename P::Seer &s, const float4 &sp, const PairList &pl, uint32_t i, uint32_t n, uint32_t self,
                     const float4 *pos, const Acc &acc, const typename P::SeeCtx &sctx) {
    const uint4 *e = pl.idx + i;
    const size_t stride = pl.stride;
    for (uint32_t t = 0; t < n; t += 4) {
        const uint4 g = __ldg(e + (size_t)(t >> 2) * stride);
        const uint32_t m = n - t;  // entries of this group: min(m, 4)
        {
            const float4 b0 = __ldg(pos + g.x);
            const float4 b1 = m > 1u ? __ldg(pos + g.y) : b0;
            if (g.x != self) P::see(s, sp, b0, acc, g.x, sctx);
            if (m > 1u && g.y != self) P::see(s, sp, b1, acc, g.y, sctx);
        }
        if (m > 2u) {
            const float4 b2 = __ldg(pos + g.z);
            const float4 b3 = m > 3u ? __ldg(pos + g.w) : b2;
            if (g.z != self) P::see(s, sp, b2, acc, g.z, sctx);
            if (m > 3u && g.w != self) P::see(s, sp, b3, acc, g.w, sctx);
        }
    }
}

// Candidate range of cells [x0, x1] of one row of a row-order table: the header and the
// two start entries are loaded together; an entry is used only inside the row's occupied
// span (x_first, x_last], where it is valid for this step.
TGPU_D uint2 row_range(const uint32_t *words, const uint4 *hdr, uint32_t row, uint32_t dx, int x0, int x1) {
    const uint4 h = __ldg(hdr + row);
    const uint32_t e0 = __ldg(words + row * dx + (uint32_t)x0);
    const uint32_t e1 = __ldg(words + row * dx + min((uint32_t)x1 + 1u, dx - 1u));
    if ((uint32_t)x0 > h.y || (uint32_t)x1 < h.x) return make_uint2(0u, 0u);
    return make_uint2((uint32_t)x0 <= h.x ? h.z : e0, (uint32_t)x1 >= h.y ? h.w : e1);
}

// ---- bulk copies (TMA, non-tensor) into shared memory, completed on an mbarrier ----
TGPU_D uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
TGPU_D void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
TGPU_D void fence_mbar_init() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
TGPU_D void mbar_inval(uint64_t *bar) {
    asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_addr(bar)) : "memory");
}
TGPU_D void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
// one contiguous run of bytes (16-byte aligned, a multiple of 16) global -> shared
TGPU_D void bulk_copy_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}
TGPU_D bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait for phase 0 of a one-shot barrier; false when the bound ran out.
constexpr uint32_t kStageSpinLimit = 1u << 22;
TGPU_D bool mbar_wait_bounded(uint64_t *bar) {
    for (uint32_t it = 0; it < kStageSpinLimit; ++it)
        if (mbar_try_wait(bar, 0)) return true;
    return false;
}

// Per-lane candidates [j0, j1) in batches of 32, the see function run over hit masks:
// every lane box-tests its own next (up to) 32 candidates into a mask, then the lanes
// with hits run the see function together, one hit each per round, so the see body runs
// for all lanes that have hits instead of for the few whose current candidate passed.
// All 32 lanes of the warp must call it (lanes with an empty range pass j0 = j1).
template <class P, class Acc>
TGPU_D void lane_run_masked(typename P::Seer &s, const float4 &sp, const float4 &r4, uint32_t j0, uint32_t j1,
                            uint32_t self, const float4 *pos, const Acc &acc, const typename P::SeeCtx &sctx,
                            uint32_t &pairs, uint32_t &tested) {
    tested += j1 - j0;
    for (uint32_t jb = j0; __any_sync(0xffffffffu, jb < j1); jb += 32u) {
        const uint32_t nb = jb < j1 ? min(32u, j1 - jb) : 0u;
        uint32_t hits = 0;
        uint32_t k = 0;
        for (; k + 1 < nb; k += 2) {
            const float4 b0 = __ldg(pos + jb + k);
            const float4 b1 = __ldg(pos + jb + k + 1);
            hits |= (uint32_t)(box_hit(sp, b0, r4) && jb + k != self) << k;
            hits |= (uint32_t)(box_hit(sp, b1, r4) && jb + k + 1 != self) << (k + 1);
        }
        if (k < nb) {
            const float4 b0 = __ldg(pos + jb + k);
            hits |= (uint32_t)(box_hit(sp, b0, r4) && jb + k != self) << k;
        }
        pairs += __popc(hits);
        while (__any_sync(0xffffffffu, hits != 0u)) {
            if (hits) {
                const uint32_t j = jb + (uint32_t)(__ffs(hits) - 1);
                hits &= hits - 1u;
                P::see(s, sp, __ldg(pos + j), acc, j, sctx);
            }
        }
    }
}

// Per-lane walk of box agents over candidates [j0, j1): min corners from `pos`, max
// corners from `pos_max`.
template <class P, class Acc>
TGPU_D void lane_run_boxes(typename P::Seer &s, const float4 &amin, const float4 &amax, const float4 &r4, uint32_t j0,
                           uint32_t j1, uint32_t self, const float4 *pos, const float4 *pos_max, const Acc &acc,
                           const typename P::SeeCtx &sctx, uint32_t &pairs, uint32_t &tested) {
    tested += j1 - j0;
    for (uint32_t j = j0; j < j1; ++j) {
        const float4 bmin = __ldg(pos + j);
        const float4 bmax = __ldg(pos_max + j);
        if (j != self && boxes_hit(amin, amax, bmin, bmax, r4)) {
            ++pairs;
            P::see(s, amin, bmin, acc, j, sctx);
        }
    }
}

// The seer's cell box in the seen grid: its search interval p +- r per axis, for box
// agents [min - r - S, max + r] with S the seen agents' largest edge on that axis.
template <bool kBox>
TGPU_D void seer_cells(const float4 &sp, const float4 &smax, const float4 &r4, const BoxAcc &B, const Grid &g, float pad,
                       int *lo, int *hi) {
    if (!kBox) {
        axis_range(sp.x, r4.x, g.origin[0], g.inv_cs[0], g.dims[0], pad, lo[0], hi[0]);
        axis_range(sp.y, r4.y, g.origin[1], g.inv_cs[1], g.dims[1], pad, lo[1], hi[1]);
        axis_range(sp.z, r4.z, g.origin[2], g.inv_cs[2], g.dims[2], pad, lo[2], hi[2]);
        return;
    }
    const float sx = ordered_to_float(B.size[0]), sy = ordered_to_float(B.size[1]), sz = ordered_to_float(B.size[2]);
    axis_span((sp.x - r4.x) - sx, smax.x + r4.x, g.origin[0], g.inv_cs[0], g.dims[0], pad, lo[0], hi[0]);
    axis_span((sp.y - r4.y) - sy, smax.y + r4.y, g.origin[1], g.inv_cs[1], g.dims[1], pad, lo[1], hi[1]);
    axis_span((sp.z - r4.z) - sz, smax.z + r4.z, g.origin[2], g.inv_cs[2], g.dims[2], pad, lo[2], hi[2]);
}

// The record codec of pass P's model (P::Codec), or void when the pass declares none.
template <class P, class = void>
struct CodecOf {
    using type = void;
};
template <class P>
struct CodecOf<P, std::void_t<typename P::Codec>> {
    using type = typename P::Codec;
};

// Write-through epilogue of a see CTA: its seers' finished records (the streams this
// launch wrote, the others as they are) in the model's AoS layout, staged in shared
// memory and stored to the segment's page-locked host records with 16-byte stores, so
// the host link works while the rest of the pass runs.  Every thread of the CTA calls it.
template <class C>
TGPU_D void write_through_cta(const SeeLaunch &L, uint32_t *wt, uint32_t first, uint32_t seg_begin,
                              uint32_t seg_end, uint32_t *sm) {
    constexpr uint32_t W = C::kAgentBytes / 4;
    PassIO wio = L.io;
#pragma unroll
    for (int c = 0; c < kMaxF4; ++c) wio.in_f4[c] = wio.out_f4[c];
    const uint32_t cnt = min((uint32_t)kSeeThreads, seg_end - first);
    if (threadIdx.x < cnt) C::unpack(sm + threadIdx.x * W, wio, first + threadIdx.x, L.wt_program);
    __syncthreads();
    uint32_t *dst = wt + (size_t)(first - seg_begin) * W;
    const uint32_t words = cnt * W;
    uint32_t w0 = 0;
    if ((reinterpret_cast<uintptr_t>(dst) & 15u) == 0) {
        const uint4 *s4 = reinterpret_cast<const uint4 *>(sm);
        uint4 *d4 = reinterpret_cast<uint4 *>(dst);
        for (uint32_t v = threadIdx.x; v < words / 4u; v += kSeeThreads) d4[v] = s4[v];
        w0 = words & ~3u;
    }
    for (uint32_t w = w0 + threadIdx.x; w < words; w += kSeeThreads) dst[w] = sm[w];
}

}  // namespace see_detail

template <class P, bool kWrite = false>
__global__ void __launch_bounds__(kSeeThreads) see_kernel(SeeLaunch L) {
    using namespace see_detail;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float4 *stage = reinterpret_cast<float4 *>(smem_raw);
    uint32_t *cell_off = reinterpret_cast<uint32_t *>(stage + (size_t)P::kSeenF4 * L.stage_cap);
    uint32_t *cell_first = cell_off + L.stage_cells + 1;
    __shared__ int hbox[6];
    __shared__ uint32_t warp_sums[kSeeThreads / 32];
    __shared__ uint32_t s_total;

    const uint2 cta = L.cta_table[L.cta_offset + blockIdx.x];
    const uint32_t seg = cta.x;
    const SegmentSpec S = L.specs[seg];                       // seers
    const SegmentSpec T = L.specs[L.cross ? L.seen_seg : seg];  // seen agents: grid and table
    const BoxAcc B = L.box[L.cross ? L.seen_seg : seg];
    const SegGrid &G = L.grids[L.cross ? L.seen_seg : seg];
    const Grid g = G.g;
    const float pad = G.pad;
    const float4 r4 = L.radii[seg];
    const typename P::SeeCtx &sctx = *reinterpret_cast<const typename P::SeeCtx *>(L.ctx + (size_t)seg * L.ctx_stride);
    const typename P::ActCtx &actx =
        *reinterpret_cast<const typename P::ActCtx *>(L.act_ctx + (size_t)seg * L.act_ctx_stride);
    const uint32_t seg_end = S.begin + S.count;
    const uint32_t i = cta.y + threadIdx.x;
    const bool active = i < seg_end;
    const uint32_t lane = threadIdx.x & 31u;

    constexpr bool kBox = BoxOf<P>::value;
    float4 sp = make_float4(0.f, 0.f, 0.f, 0.f), smax = sp;
    typename P::Seer s;
    int lo[3] = {INT_MAX, INT_MAX, INT_MAX}, hi[3] = {INT_MIN, INT_MIN, INT_MIN};
    if (active) {
        sp = L.io.in_f4[0][i];
        if (kBox) smax = L.io.in_f4[1][i];
        P::load(s, L.io, i, sctx, actx);
        seer_cells<kBox>(sp, smax, r4, B, g, pad, lo, hi);
    }

    // CTA halo box = union of the seers' cell boxes
    if (threadIdx.x < 6) hbox[threadIdx.x] = threadIdx.x < 3 ? INT_MAX : INT_MIN;
    __syncthreads();
    {
        int l0 = warp_min_i(lo[0]), l1 = warp_min_i(lo[1]), l2 = warp_min_i(lo[2]);
        int h0 = warp_max_i(hi[0]), h1 = warp_max_i(hi[1]), h2 = warp_max_i(hi[2]);
        if (lane == 0 && l0 <= h0) {
            atomicMin(&hbox[0], l0);
            atomicMin(&hbox[1], l1);
            atomicMin(&hbox[2], l2);
            atomicMax(&hbox[3], h0);
            atomicMax(&hbox[4], h1);
            atomicMax(&hbox[5], h2);
        }
    }
    __syncthreads();
    const int H0x = hbox[0], H0y = hbox[1], H0z = hbox[2];
    const int hx = hbox[3] - H0x + 1, hy = hbox[4] - H0y + 1, hz = hbox[5] - H0z + 1;
    const long long V = (hx > 0 && hy > 0 && hz > 0) ? (long long)hx * hy * hz : 0;
    bool staged = !kBox && L.stage_cap > 0 && V > 0 && V <= (long long)L.stage_cells;
    const uint2 *table = L.table + T.table_base;
    const uint32_t dx0 = (uint32_t)g.dims[0], dy0 = (uint32_t)g.dims[1];

    uint32_t total = 0;
    if (staged) {
        const uint32_t nv = (uint32_t)V;
        for (uint32_t c = threadIdx.x; c < nv; c += kSeeThreads) {
            uint32_t x = c % (uint32_t)hx, yz = c / (uint32_t)hx;
            uint32_t y = yz % (uint32_t)hy, z = yz / (uint32_t)hy;
            uint2 e = table[((uint32_t)(H0z + (int)z) * dy0 + (uint32_t)(H0y + (int)y)) * dx0 + (uint32_t)(H0x + (int)x)];
            cell_first[c] = e.x;
            cell_off[c] = e.y - e.x;
        }
        __syncthreads();
        // exclusive scan of the cell counts: each thread scans a contiguous chunk
        const uint32_t per = (nv + kSeeThreads - 1) / kSeeThreads;
        const uint32_t c0 = threadIdx.x * per;
        const uint32_t c1 = min(c0 + per, nv);
        uint32_t sum = 0;
        for (uint32_t c = c0; c < c1; ++c) sum += cell_off[c];
        uint32_t incl = sum;
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t w = __shfl_up_sync(0xffffffffu, incl, o);
            if ((int)lane >= o) incl += w;
        }
        if (lane == 31) warp_sums[threadIdx.x >> 5] = incl;
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t run = 0;
            for (int w = 0; w < kSeeThreads / 32; ++w) {
                uint32_t t = warp_sums[w];
                warp_sums[w] = run;
                run += t;
            }
            s_total = run;
        }
        __syncthreads();
        uint32_t run = warp_sums[threadIdx.x >> 5] + incl - sum;
        for (uint32_t c = c0; c < c1; ++c) {
            uint32_t t = cell_off[c];
            cell_off[c] = run;
            run += t;
        }
        if (threadIdx.x == 0) cell_off[nv] = s_total;
        total = s_total;
        staged = total <= L.stage_cap;
        __syncthreads();
        if (staged) {
            for (uint32_t j = threadIdx.x; j < total; j += kSeeThreads) {
                // last cell whose offset is <= j
                uint32_t a = 0, b = nv;
                while (b - a > 1) {
                    uint32_t m = (a + b) >> 1;
                    if (cell_off[m] <= j) a = m; else b = m;
                }
                const uint32_t src = cell_first[a] + (j - cell_off[a]);
#pragma unroll
                for (int k = 0; k < P::kSeenF4; ++k) stage[(uint32_t)k * L.stage_cap + j] = __ldg(L.io.in_f4[P::seen_stream(k)] + src);
            }
            __syncthreads();
        }
    }

    // per-warp union of the seers' cell boxes
    const int wl0 = warp_min_i(lo[0]), wl1 = warp_min_i(lo[1]), wl2 = warp_min_i(lo[2]);
    const int wh0 = warp_max_i(hi[0]), wh1 = warp_max_i(hi[1]), wh2 = warp_max_i(hi[2]);
    uint32_t pairs = 0;
    uint32_t tested = 0;
    if (L.telemetry && threadIdx.x == 0) atomicAdd(L.telemetry + (staged ? 1 : 2), 1ull);
    if (wl0 <= wh0) {
        // A warp walks the union of its lanes' cell boxes (one broadcast read serves all
        // 32 lanes) when the union is compact; when its seers are spread out, as in sparse
        // regions, each lane walks its own box instead.
        const int lane_vol = active ? max(0, hi[0] - lo[0] + 1) * max(0, hi[1] - lo[1] + 1) * max(0, hi[2] - lo[2] + 1) : 0;
        const long long union_vol = (long long)(wh0 - wl0 + 1) * (wh1 - wl1 + 1) * (wh2 - wl2 + 1);
        const bool union_mode = !kBox && union_vol <= (long long)L.union_factor * warp_max_i(lane_vol);
        if (L.telemetry && lane == 0) atomicAdd(L.telemetry + (union_mode ? 3 : 4), 1ull);
        if (staged) {
            uint32_t self_slot = 0xFFFFFFFFu;
            if (active && L.skip_self) {
                int cx = cell_coord(sp.x, g.origin[0], g.inv_cs[0], g.dims[0]) - H0x;
                int cy = cell_coord(sp.y, g.origin[1], g.inv_cs[1], g.dims[1]) - H0y;
                int cz = cell_coord(sp.z, g.origin[2], g.inv_cs[2], g.dims[2]) - H0z;
                if (cx >= 0 && cx < hx && cy >= 0 && cy < hy && cz >= 0 && cz < hz) {
                    uint32_t c = ((uint32_t)cz * (uint32_t)hy + (uint32_t)cy) * (uint32_t)hx + (uint32_t)cx;
                    self_slot = cell_off[c] + (i - cell_first[c]);
                }
            }
            const SmemSeen acc{stage, L.stage_cap};
            if (union_mode) {
                // Two phases per batch of up to 32 staged agents: every lane box-tests
                // its seer against the batch (broadcast reads) into a hit mask, then the
                // lanes run the see function over their own hits together.
                for (int z = wl2; z <= wh2; ++z)
                    for (int y = wl1; y <= wh1; ++y) {
                        const uint32_t row = ((uint32_t)(z - H0z) * (uint32_t)hy + (uint32_t)(y - H0y)) * (uint32_t)hx;
                        const uint32_t j0 = cell_off[row + (uint32_t)(wl0 - H0x)];
                        const uint32_t j1 = cell_off[row + (uint32_t)(wh0 - H0x) + 1];
                        union_batches<P>(s, sp, r4, active, j0, j1, self_slot, stage, acc, sctx, pairs, tested);
                    }
            } else if (active) {
                for (int z = lo[2]; z <= hi[2]; ++z)
                    for (int y = lo[1]; y <= hi[1]; ++y) {
                        const uint32_t row = ((uint32_t)(z - H0z) * (uint32_t)hy + (uint32_t)(y - H0y)) * (uint32_t)hx;
                        const uint32_t j0 = cell_off[row + (uint32_t)(lo[0] - H0x)];
                        const uint32_t j1 = cell_off[row + (uint32_t)(hi[0] - H0x) + 1];
                        lane_run<P>(s, sp, r4, j0, j1, self_slot, stage, acc, sctx, pairs, tested);
                    }
            }
        } else {
            GlobalSeen<P::kSeenF4> acc;
#pragma unroll
            for (int k = 0; k < P::kSeenF4; ++k) acc.s[k] = L.io.in_f4[P::seen_stream(k)];
            const float4 *pos = L.io.in_f4[0];
            const uint32_t self = (active && L.skip_self) ? i : 0xFFFFFFFFu;
            if (union_mode) {
                // same two-phase walk over the union box, cell by cell from the table:
                // every lane reads the same address, which L1 serves once for the warp
                for (int z = wl2; z <= wh2; ++z)
                    for (int y = wl1; y <= wh1; ++y)
                        for (int x = wl0; x <= wh0; ++x) {
                            const uint2 e = table[((uint32_t)z * dy0 + (uint32_t)y) * dx0 + (uint32_t)x];
                            union_batches<P>(s, sp, r4, active, e.x, e.y, self, pos, acc, sctx, pairs, tested);
                        }
            } else if (active) {
                for (int z = lo[2]; z <= hi[2]; ++z)
                    for (int y = lo[1]; y <= hi[1]; ++y)
                        for (int x = lo[0]; x <= hi[0]; ++x) {
                            const uint2 e = table[((uint32_t)z * dy0 + (uint32_t)y) * dx0 + (uint32_t)x];
                            if (kBox)
                                lane_run_boxes<P>(s, sp, smax, r4, e.x, e.y, self, pos, L.io.in_f4[1], acc, sctx,
                                                  pairs, tested);
                            else
                                lane_run<P>(s, sp, r4, e.x, e.y, self, pos, acc, sctx, pairs, tested);
                        }
            }
        }
    }
    if (active) P::finish(s, sp, L.io, i, sctx, actx);
    if (L.pairs) {
        uint32_t w = warp_sum_u(pairs);
        if (lane == 0 && w) atomicAdd(L.pairs, (unsigned long long)w);
    }
    if (L.telemetry) {
        uint32_t w = warp_sum_u(tested);
        if (lane == 0 && w) atomicAdd(L.telemetry, (unsigned long long)w);
    }
    if constexpr (kWrite) {
        using C = typename CodecOf<P>::type;
        __shared__ __align__(16) uint32_t wt_sm[kSeeThreads * (C::kAgentBytes / 4)];
        uint32_t *wt = L.wt[seg];
        if (wt) write_through_cta<C>(L, wt, cta.y, S.begin, seg_end, wt_sm);
    }
}

// See pass over a row-order table (kOrderRows): the agents of x-adjacent cells are
// contiguous, so a seer's cell box is one candidate range per (y, z) row, read from two
// start entries of the row.  Lanes of a warp are consecutive seers along a row: their
// ranges are nearly the same length and their candidate loads fall on neighbouring
// addresses.  No staging; a warp whose union box is compact walks the union's row
// ranges with the two-phase batches instead.
// At most 64 registers (8 CTAs of 128 threads per SM) except for the staged walk: a few
// spills cost less than the occupancy step above 64 (measured on the boids and SPH passes).
// kWarpWalks: the instance also holds the warp-union and hit-mask walks (tunings union_factor
// > 1 or hit_masks).  Without them (the default tunings) lanes always walk their own boxes,
// which gives the same bits, and the kernel holds no spills at 64 registers: measured with
// them compiled in, their register needs spilled into the lane walk (SPH step 1.509 ->
// 1.458 ms and the 1M-boid see pass 395.7 -> 391.3 us without).
template <class P, bool kStage = false, bool kWrite = false, bool kWarpWalks = true>
__global__ void __launch_bounds__(kSeeThreads, kStage ? 1 : 8) see_rows_kernel(SeeLaunch L) {
    using namespace see_detail;
    const uint2 cta = L.cta_table[L.cta_offset + blockIdx.x];
    const uint32_t seg = cta.x;
    const SegmentSpec S = L.specs[seg];                       // seers
    const SegmentSpec T = L.specs[L.cross ? L.seen_seg : seg];  // seen agents: grid and table
    const BoxAcc B = L.box[L.cross ? L.seen_seg : seg];
    const SegGrid &G = L.grids[L.cross ? L.seen_seg : seg];
    const Grid g = G.g;
    const float pad = G.pad;
    const float4 r4 = L.radii[seg];
    const typename P::SeeCtx &sctx = *reinterpret_cast<const typename P::SeeCtx *>(L.ctx + (size_t)seg * L.ctx_stride);
    const typename P::ActCtx &actx =
        *reinterpret_cast<const typename P::ActCtx *>(L.act_ctx + (size_t)seg * L.act_ctx_stride);
    const uint32_t seg_end = S.begin + S.count;
    const uint32_t i = cta.y + threadIdx.x;
    const bool active = i < seg_end;
    const uint32_t lane = threadIdx.x & 31u;

    constexpr bool kBox = BoxOf<P>::value;
    float4 sp = make_float4(0.f, 0.f, 0.f, 0.f), smax = sp;
    typename P::Seer s;
    int lo[3] = {INT_MAX, INT_MAX, INT_MAX}, hi[3] = {INT_MIN, INT_MIN, INT_MIN};
    if (active) {
        sp = L.io.in_f4[0][i];
        if (kBox) smax = L.io.in_f4[1][i];
        P::load(s, L.io, i, sctx, actx);
        seer_cells<kBox>(sp, smax, r4, B, g, pad, lo, hi);
    }
    const uint4 *hdr = reinterpret_cast<const uint4 *>(L.table + T.table_base);
    const uint32_t *words = reinterpret_cast<const uint32_t *>(L.table + T.table_base) + row_entry_word(T);
    const uint32_t dx0 = (uint32_t)g.dims[0], dy0 = (uint32_t)g.dims[1];
    GlobalSeen<P::kSeenF4> acc;
#pragma unroll
    for (int k = 0; k < P::kSeenF4; ++k) acc.s[k] = L.io.in_f4[P::seen_stream(k)];
    const float4 *pos = L.io.in_f4[0];
    const uint32_t self = (active && L.skip_self) ? i : 0xFFFFFFFFu;
    uint32_t pairs = 0;
    uint32_t tested = 0;
    constexpr int kList = ListOf<P>::value;

    // Replay of the previous pass's pair list (same positions, same table): a warp whose
    // lanes all hold complete lists runs the see function over them in the recorded order,
    // which is the order the row walk would visit them in; otherwise the warp walks.
    bool replayed = false;
    if constexpr (kList == 2 && !kBox) {
        if (L.plist.mode == 2u) {
            const float4 rr = L.plist.rec_radii[seg];
            const auto &rctx =
                *reinterpret_cast<const typename P::SeeCtx *>(L.plist.rec_ctx + (size_t)seg * L.ctx_stride);
            // the recorded set covers this pass's pairs: the same box, and a keep test at
            // least as wide as what this pass's see function acts on
            const bool covers = rr.x == r4.x && rr.y == r4.y && rr.z == r4.z && P::replay_ok(sctx, rctx);
            const uint2 c = active ? L.plist.count[i] : make_uint2(0u, 0u);
            replayed = __all_sync(0xffffffffu, covers && c.x <= L.plist.cap);
            if (replayed && L.telemetry && lane == 0) atomicAdd(L.telemetry + 5, 1ull);
            if (replayed && active) {
                list_run<P>(s, sp, L.plist, i, c.x, self, pos, acc, sctx);
                // the walk's count: box-test passes with every other agent, and the seer
                // itself unless the pass skips it
                pairs += c.y + ((!L.skip_self && box_hit(sp, sp, r4)) ? 1u : 0u);
            }
        }
    }

    // Optional staging (stage_cap > 0, point agents): the rows of the union of the CTA's
    // seer boxes are contiguous runs of agents, each copied into shared memory by one bulk
    // copy (TMA) per seen stream, completed on an mbarrier; the lanes then walk their rows
    // there.  CTAs whose halo does not fit fall back to the walk through L1.
    bool staged = false;
    if constexpr (kStage && !kBox) {
        extern __shared__ __align__(16) unsigned char smem_raw[];
        float4 *stage = reinterpret_cast<float4 *>(smem_raw);
        uint32_t *row_off = reinterpret_cast<uint32_t *>(stage + (size_t)P::kSeenF4 * L.stage_cap);
        uint32_t *row_j0 = row_off + L.stage_cells;
        // row_off starts 16-byte aligned and the two tables hold 2 * stage_cells words,
        // so the barrier after them is 8-byte aligned
        uint64_t *bar = reinterpret_cast<uint64_t *>(row_off + 2u * L.stage_cells);
        __shared__ int hb[6];
        __shared__ uint32_t s_total;
        if (threadIdx.x < 6) hb[threadIdx.x] = threadIdx.x < 3 ? INT_MAX : INT_MIN;
        __syncthreads();
        {
            const int l0 = warp_min_i(lo[0]), l1 = warp_min_i(lo[1]), l2 = warp_min_i(lo[2]);
            const int h0 = warp_max_i(hi[0]), h1 = warp_max_i(hi[1]), h2 = warp_max_i(hi[2]);
            if (lane == 0 && l0 <= h0) {
                atomicMin(&hb[0], l0);
                atomicMin(&hb[1], l1);
                atomicMin(&hb[2], l2);
                atomicMax(&hb[3], h0);
                atomicMax(&hb[4], h1);
                atomicMax(&hb[5], h2);
            }
        }
        __syncthreads();
        const int X0 = hb[0], Y0 = hb[1], Z0 = hb[2];
        const int ny = hb[4] - Y0 + 1, nz = hb[5] - Z0 + 1;
        // (never for a pass that records or replays a pair list)
        const long long nrows =
            (L.plist.mode == 0u && hb[3] >= X0 && ny > 0 && nz > 0) ? (long long)ny * nz : 0;
        if (nrows > 0 && nrows <= (long long)L.stage_cells) {
            // each union row's candidate range over the union's x cells
            for (uint32_t t = threadIdx.x; t < (uint32_t)nrows; t += kSeeThreads) {
                const uint32_t z = (uint32_t)Z0 + t / (uint32_t)ny, y = (uint32_t)Y0 + t % (uint32_t)ny;
                const uint2 jr = row_range(words, hdr, z * dy0 + y, dx0, X0, hb[3]);
                row_j0[t] = jr.x;
                row_off[t] = jr.y - jr.x;
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                uint32_t run = 0;
                for (uint32_t t = 0; t < (uint32_t)nrows; ++t) {
                    const uint32_t c = row_off[t];
                    row_off[t] = run;
                    run += c;
                }
                s_total = run;
                if (run > 0 && run <= L.stage_cap) {
                    mbar_init(bar, 1);
                    fence_mbar_init();
                }
            }
            __syncthreads();
            const uint32_t total = s_total;
            if (total > 0 && total <= L.stage_cap) {
                if (threadIdx.x == 0) {
                    mbar_arrive_expect_tx(bar, total * (uint32_t)sizeof(float4) * (uint32_t)P::kSeenF4);
                    for (uint32_t t = 0; t < (uint32_t)nrows; ++t) {
                        const uint32_t c = (t + 1 < (uint32_t)nrows ? row_off[t + 1] : total) - row_off[t];
                        if (!c) continue;
#pragma unroll
                        for (int k = 0; k < P::kSeenF4; ++k)
                            bulk_copy_g2s(stage + (size_t)k * L.stage_cap + row_off[t],
                                          L.io.in_f4[P::seen_stream(k)] + row_j0[t], c * (uint32_t)sizeof(float4),
                                          bar);
                    }
                }
                staged = mbar_wait_bounded(bar);
                if (!staged) {
                    // a wait that ran out: report it, and let the copies in flight land
                    // before this CTA's shared memory can be given to another CTA
                    if (threadIdx.x == 0 && L.err) atomicOr(L.err, kErrStageWait);
                    mbar_wait_bounded(bar);
                }
                staged = __syncthreads_and(staged);
                // every thread has left the wait; a barrier whose copies may still be pending
                // (the waits ran out) is not invalidated
                if (staged && threadIdx.x == 0) mbar_inval(bar);
                if (staged) {
                    const SmemSeen sacc{stage, L.stage_cap};
                    if (active) {
                        for (int z = lo[2]; z <= hi[2]; ++z)
                            for (int y = lo[1]; y <= hi[1]; ++y) {
                                const uint32_t t = (uint32_t)(z - Z0) * (uint32_t)ny + (uint32_t)(y - Y0);
                                const uint2 jr = row_range(words, hdr, (uint32_t)z * dy0 + (uint32_t)y, dx0, lo[0], hi[0]);
                                if (jr.y <= jr.x) continue;  // an empty row is never translated
                                const uint32_t shift = row_off[t] - row_j0[t];  // global index -> staged slot
                                const uint32_t cnt = (t + 1 < (uint32_t)nrows ? row_off[t + 1] : total) - row_off[t];
                                // the lane's x range lies inside the union's, so its run lies
                                // inside the staged one; checked, reported and skipped if not
                                if (jr.x < row_j0[t] || jr.y - row_j0[t] > cnt) {
                                    if (L.err) atomicOr(L.err, kErrStageRange);
                                    continue;
                                }
                                // the seer's own slot, only when it sits in this row's staged run
                                const uint32_t self_s =
                                    (self >= row_j0[t] && self - row_j0[t] < cnt) ? self + shift : 0xFFFFFFFFu;
                                lane_run<P>(s, sp, r4, jr.x + shift, jr.y + shift, self_s, stage, sacc, sctx, pairs,
                                            tested);
                            }
                    }
                }
            }
        }
    }
    if (L.telemetry && threadIdx.x == 0) atomicAdd(L.telemetry + (staged ? 1 : 2), 1ull);

    // the warp's union box (only the warp walks use it; without them a vote says whether any
    // lane has cells)
    int wl0 = 0, wl1 = 0, wl2 = 0, wh0 = -1, wh1 = -1, wh2 = -1;
    bool warp_cells;
    if constexpr (kWarpWalks) {
        wl0 = warp_min_i(lo[0]);
        wl1 = warp_min_i(lo[1]);
        wl2 = warp_min_i(lo[2]);
        wh0 = warp_max_i(hi[0]);
        wh1 = warp_max_i(hi[1]);
        wh2 = warp_max_i(hi[2]);
        warp_cells = wl0 <= wh0;
    } else {
        warp_cells = __any_sync(0xffffffffu, lo[0] <= hi[0]);
    }
    // a recording pass (launch-uniform) takes the per-lane walk, which records (every walk
    // visits a lane's hits in the same order; recording along the union walk measured slower)
    const bool recording = kList == 1 && !kBox && L.plist.mode == 1u;
    if (!staged && !replayed && warp_cells) {
        bool union_mode = false;
        if constexpr (kWarpWalks) {
            const int lane_vol = active ? (hi[1] - lo[1] + 1) * (hi[2] - lo[2] + 1) * (hi[0] - lo[0] + 1) : 0;
            const long long union_vol = (long long)(wh0 - wl0 + 1) * (wh1 - wl1 + 1) * (wh2 - wl2 + 1);
            union_mode = !kBox && !recording && union_vol <= (long long)L.union_factor * warp_max_i(lane_vol);
        }
        if (L.telemetry && lane == 0) atomicAdd(L.telemetry + (union_mode ? 3 : 4), 1ull);
        bool walked = false;
        if constexpr (kList == 1 && !kBox) {
            if (recording) {
                // the per-lane walk with the recorder (a block of its own: folded into the
                // plain walks it costs the non-recording kernels registers)
                if (active) {
                    ListRec rec{L.plist.idx, L.plist.stride, L.plist.cap, i, 0u, 0u};
                    const uint32_t before = pairs;
                    for (int z = lo[2]; z <= hi[2]; ++z)
                        for (int y = lo[1]; y <= hi[1]; ++y) {
                            const uint2 jr =
                                row_range(words, hdr, (uint32_t)z * dy0 + (uint32_t)y, dx0, lo[0], hi[0]);
                            lane_run<P, decltype(acc), ListRec, GateOf<P>::value>(s, sp, r4, jr.x, jr.y, self, pos,
                                                                                   acc, sctx, pairs, tested, &rec);
                        }
                    if constexpr (GateOf<P>::value) {
                        // the gated walk counted the seer's own box-test pass (met once)
                        const uint32_t own = box_hit(sp, sp, r4) ? 1u : 0u;
                        rec.other = pairs - before - own;
                        if (L.skip_self) pairs -= own;
                    }
                    L.plist.count[i] = make_uint2(rec.n, rec.other);
                }
                walked = true;
            }
        }
        if (walked) {
        } else if (union_mode) {
            for (int z = wl2; z <= wh2; ++z)
                for (int y = wl1; y <= wh1; ++y) {
                    const uint2 jr = row_range(words, hdr, (uint32_t)z * dy0 + (uint32_t)y, dx0, wl0, wh0);
                    union_batches<P>(s, sp, r4, active, jr.x, jr.y, self, pos, acc, sctx, pairs, tested);
                }
        } else if (kWarpWalks && !kBox && L.hit_masks) {
            // rows of the warp's union box (a warp-uniform loop), each lane's own x range
            for (int z = wl2; z <= wh2; ++z)
                for (int y = wl1; y <= wh1; ++y) {
                    uint2 jr = make_uint2(0u, 0u);
                    if (active && z >= lo[2] && z <= hi[2] && y >= lo[1] && y <= hi[1])
                        jr = row_range(words, hdr, (uint32_t)z * dy0 + (uint32_t)y, dx0, lo[0], hi[0]);
                    lane_run_masked<P>(s, sp, r4, jr.x, jr.y, self, pos, acc, sctx, pairs, tested);
                }
        } else if (active) {
            for (int z = lo[2]; z <= hi[2]; ++z)
                for (int y = lo[1]; y <= hi[1]; ++y) {
                    const uint2 jr = row_range(words, hdr, (uint32_t)z * dy0 + (uint32_t)y, dx0, lo[0], hi[0]);
                    if (kBox)
                        lane_run_boxes<P>(s, sp, smax, r4, jr.x, jr.y, self, pos, L.io.in_f4[1], acc, sctx, pairs,
                                          tested);
                    else
                        lane_run<P, decltype(acc), NoRec, GateOf<P>::value>(s, sp, r4, jr.x, jr.y, self, pos, acc,
                                                                             sctx, pairs, tested);
                }
            // the gated walk tested the seer too (it lies in its own range): its box-test
            // pass comes off the counter when the pass skips self
            if constexpr (GateOf<P>::value && !kBox)
                if (L.skip_self && box_hit(sp, sp, r4)) --pairs;
        }
    } else if (recording && active) {
        L.plist.count[i] = make_uint2(0u, 0u);  // no cell to walk: an empty, complete list
    }
    if (active) P::finish(s, sp, L.io, i, sctx, actx);
    if (L.pairs) {
        uint32_t w = warp_sum_u(pairs);
        if (lane == 0 && w) atomicAdd(L.pairs, (unsigned long long)w);
    }
    if (L.telemetry) {
        uint32_t w = warp_sum_u(tested);
        if (lane == 0 && w) atomicAdd(L.telemetry, (unsigned long long)w);
    }
    if constexpr (kWrite) {
        using C = typename CodecOf<P>::type;
        __shared__ __align__(16) uint32_t wt_sm[kSeeThreads * (C::kAgentBytes / 4)];
        uint32_t *wt = L.wt[seg];
        if (wt) write_through_cta<C>(L, wt, cta.y, S.begin, seg_end, wt_sm);
    }
}

template <class A>
__global__ void __launch_bounds__(kSortThreads) act_kernel(ActLaunch L) {
    const uint32_t tile = L.tile_offset + blockIdx.x;
    const uint32_t seg = L.tile_seg[tile];
    const SegmentSpec S = L.specs[seg];
    const typename A::ActCtx &actx = *reinterpret_cast<const typename A::ActCtx *>(L.ctx + (size_t)seg * L.ctx_stride);
    const uint32_t t = tile - S.tile_begin;
    const uint32_t beg = S.begin + t * kSortTile;
    const uint32_t end = min(beg + (uint32_t)kSortTile, S.begin + S.count);
    for (uint32_t i = beg + threadIdx.x; i < end; i += kSortThreads) A::act(L.io, i, actx);
}

// AoS <-> SoA conversion for push and fetch (replaces the OpenCL path's whole-buffer
// copies, tay/ocl.c:238-272).  `aos` is the record array in device memory.
template <class M>
// AoS records <-> SoA streams, 256 records per block staged in shared memory, so the
// records are read (pack) or written (unpack) as one contiguous run of words per block:
// coalesced in device memory, and large requests when `aos` is page-locked host memory
// the kernel reads or writes in place (no separate copy).
__global__ void __launch_bounds__(256) pack_kernel(const uint32_t *__restrict__ aos, uint32_t n, PassIO io,
                                                   BoxAcc *extent) {
    constexpr uint32_t W = M::kAgentBytes / 4;
    __shared__ __align__(16) uint32_t sm[256 * W];
    const uint32_t first = blockIdx.x * 256u;
    const uint32_t cnt = min(256u, n - first);
    const uint32_t *src = aos + (size_t)first * W;
    const uint32_t words = cnt * W;
    uint32_t w0 = 0;
    if ((reinterpret_cast<uintptr_t>(src) & 15u) == 0) {
        // 16-byte loads for the aligned bulk, words for the tail
        const uint4 *s4 = reinterpret_cast<const uint4 *>(src);
        uint4 *d4 = reinterpret_cast<uint4 *>(sm);
        for (uint32_t v = threadIdx.x; v < words / 4u; v += 256u) d4[v] = s4[v];
        w0 = words & ~3u;
    }
    for (uint32_t w = w0 + threadIdx.x; w < words; w += 256u) sm[w] = src[w];
    __syncthreads();
    const bool live = threadIdx.x < cnt;
    if (live) M::pack(sm + threadIdx.x * W, io, first + threadIdx.x);
    if (!extent) return;
    // the extent of the packed positions (the grid budget's input), one atomic per warp
    // and axis; the thread reads back the position it just wrote
    float4 p = make_float4(0.f, 0.f, 0.f, 0.f);
    if (live) p = io.out_f4[0][first + threadIdx.x];
    const float c[3] = {p.x, p.y, p.z};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        uint32_t l = live ? float_to_ordered(c[a]) : 0xFFFFFFFFu, h = live ? float_to_ordered(c[a]) : 0u;
        for (int o = 16; o > 0; o >>= 1) {
            l = min(l, __shfl_xor_sync(0xffffffffu, l, o));
            h = max(h, __shfl_xor_sync(0xffffffffu, h, o));
        }
        if ((threadIdx.x & 31u) == 0 && l <= h) {
            atomicMin(&extent->lo[a], l);
            atomicMax(&extent->hi[a], h);
        }
    }
}

template <class M>
__global__ void __launch_bounds__(256) unpack_kernel(uint32_t *__restrict__ aos, uint32_t n, PassIO io,
                                                     uint32_t program) {
    constexpr uint32_t W = M::kAgentBytes / 4;
    __shared__ __align__(16) uint32_t sm[256 * W];
    const uint32_t first = blockIdx.x * 256u;
    const uint32_t cnt = min(256u, n - first);
    if (threadIdx.x < cnt) M::unpack(sm + threadIdx.x * W, io, first + threadIdx.x, program);
    __syncthreads();
    uint32_t *dst = aos + (size_t)first * W;
    const uint32_t words = cnt * W;
    uint32_t w0 = 0;
    if ((reinterpret_cast<uintptr_t>(dst) & 15u) == 0) {
        const uint4 *s4 = reinterpret_cast<const uint4 *>(sm);
        uint4 *d4 = reinterpret_cast<uint4 *>(dst);
        for (uint32_t v = threadIdx.x; v < words / 4u; v += 256u) d4[v] = s4[v];
        w0 = words & ~3u;
    }
    for (uint32_t w = w0 + threadIdx.x; w < words; w += 256u) dst[w] = sm[w];
}

}  // namespace tgpu
