// The reference's box agent (a non-point test agent) on the GPU: test/agent.h:21-29
// (BoxAgent) and test/agent.c:57-118 (box_agent_see, box_agent_act), registered under
// the same func names "box_agent_see" / "box_agent_act".
//
// Non-point agents are kept in the Z-grid by their min corner; a seer's search over the
// seen agents' min corners is widened by the seen group's largest box edge, and pairs
// pass the reference's non-point test (tay/space.c:92-103) on min and max corners.
//
// AoS record (96 bytes, packed): tag u32[2] @0, min float4 @8, max float4 @24, v float4 @40,
// b_buffer float4 @56, b_buffer_count int @72, f_buffer float4 @76, result_index int @92.
// Streams (all persistent state):
//   f4[0] MIN  = min (the agent's position)   f4[1] MAX = max   f4[2] VEL = v
//   f4[3] BBUF = b_buffer.xyz, w = b_buffer_count (int bits)
//   f4[4] FBUF = f_buffer.xyz, w = result_index (int bits)
// As for the point test agent, the w components the reference leaves undefined are
// fetched as 0.
#include "model.cuh"

namespace tgpu {
namespace box {

enum { MIN = 0, MAX = 1, VEL = 2, BBUF = 3, FBUF = 4 };

struct SeeCtx {
    float4 radii;
};
struct ActCtx {
    float4 min;
    float4 max;
};

struct Seer {
    float bx, by, bz;
    int count;
    float4 mx, v, f;
};

// test/agent.c:57-63: b_buffer += b.min - a.min; b_buffer_count++
template <class Acc>
TGPU_D void see_fn(Seer &s, const float4 &a, const float4 &b, const Acc &, uint32_t, const SeeCtx &) {
    s.bx = s.bx + (b.x - a.x);
    s.by = s.by + (b.y - a.y);
    s.bz = s.bz + (b.z - a.z);
    s.count += 1;
}

// test/agent.c:65-118 on registers: fold, move both corners, then the walls in the order
// min x, y, z, max x, y, z.
TGPU_D void act_fn(float4 &mn, float4 &mx, float4 &v, float &bx, float &by, float &bz, int &count, float4 &f,
                   const ActCtx &c) {
    if (count != 0) {
        const float n = (float)count;
        f.x = f.x + bx / n;
        f.y = f.y + by / n;
        f.z = f.z + bz / n;
        bx = 0.0f;
        by = 0.0f;
        bz = 0.0f;
        count = 0;
    }
    const float sx = mx.x - mn.x, sy = mx.y - mn.y, sz = mx.z - mn.z;
    mn.x = mn.x + v.x;
    mn.y = mn.y + v.y;
    mn.z = mn.z + v.z;
    mx.x = mx.x + v.x;
    mx.y = mx.y + v.y;
    mx.z = mx.z + v.z;
    if (mn.x < c.min.x) { mn.x = c.min.x; mx.x = c.min.x + sx; v.x = -v.x; }
    if (mn.y < c.min.y) { mn.y = c.min.y; mx.y = c.min.y + sy; v.y = -v.y; }
    if (mn.z < c.min.z) { mn.z = c.min.z; mx.z = c.min.z + sz; v.z = -v.z; }
    if (mx.x > c.max.x) { mx.x = c.max.x; mn.x = c.max.x - sx; v.x = -v.x; }
    if (mx.y > c.max.y) { mx.y = c.max.y; mn.y = c.max.y - sy; v.y = -v.y; }
    if (mx.z > c.max.z) { mx.z = c.max.z; mn.z = c.max.z - sz; v.z = -v.z; }
}

struct Codec;  // the record codec, defined below

struct SeeOnly {
    using SeeCtx = box::SeeCtx;
    using Codec = box::Codec;
    using ActCtx = box::SeeCtx;
    using Seer = box::Seer;
    static constexpr bool kBox = true;
    static constexpr int kSeenF4 = 1;
    TGPU_D static int seen_stream(int) { return MIN; }
    TGPU_D static void load(Seer &s, const PassIO &io, uint32_t i, const SeeCtx &, const ActCtx &) {
        const float4 b = io.in_f4[BBUF][i];
        s.bx = b.x;
        s.by = b.y;
        s.bz = b.z;
        s.count = __float_as_int(b.w);
    }
    template <class Acc>
    TGPU_D static void see(Seer &s, const float4 &a, const float4 &b, const Acc &acc, uint32_t j, const SeeCtx &c) {
        see_fn(s, a, b, acc, j, c);
    }
    TGPU_D static void finish(Seer &s, const float4 &, const PassIO &io, uint32_t i, const SeeCtx &, const ActCtx &) {
        io.out_f4[BBUF][i] = make_float4(s.bx, s.by, s.bz, __int_as_float(s.count));
    }
};

struct SeeAct {
    using SeeCtx = box::SeeCtx;
    using Codec = box::Codec;
    using ActCtx = box::ActCtx;
    using Seer = box::Seer;
    static constexpr bool kBox = true;
    static constexpr int kSeenF4 = 1;
    TGPU_D static int seen_stream(int) { return MIN; }
    TGPU_D static void load(Seer &s, const PassIO &io, uint32_t i, const SeeCtx &, const ActCtx &) {
        const float4 b = io.in_f4[BBUF][i];
        s.bx = b.x;
        s.by = b.y;
        s.bz = b.z;
        s.count = __float_as_int(b.w);
        s.mx = io.in_f4[MAX][i];
        s.v = io.in_f4[VEL][i];
        s.f = io.in_f4[FBUF][i];
    }
    template <class Acc>
    TGPU_D static void see(Seer &s, const float4 &a, const float4 &b, const Acc &acc, uint32_t j, const SeeCtx &c) {
        see_fn(s, a, b, acc, j, c);
    }
    TGPU_D static void finish(Seer &s, const float4 &a, const PassIO &io, uint32_t i, const SeeCtx &,
                              const ActCtx &c) {
        float4 mn = a;
        act_fn(mn, s.mx, s.v, s.bx, s.by, s.bz, s.count, s.f, c);
        io.out_f4[MIN][i] = mn;
        io.out_f4[MAX][i] = s.mx;
        io.out_f4[VEL][i] = s.v;
        io.out_f4[BBUF][i] = make_float4(s.bx, s.by, s.bz, __int_as_float(s.count));
        io.out_f4[FBUF][i] = s.f;
    }
};

struct Act {
    using ActCtx = box::ActCtx;
    TGPU_D static void act(const PassIO &io, uint32_t i, const ActCtx &c) {
        float4 mn = io.in_f4[MIN][i], mx = io.in_f4[MAX][i], v = io.in_f4[VEL][i], b = io.in_f4[BBUF][i],
               f = io.in_f4[FBUF][i];
        int count = __float_as_int(b.w);
        act_fn(mn, mx, v, b.x, b.y, b.z, count, f, c);
        b.w = __int_as_float(count);
        io.out_f4[MIN][i] = mn;
        io.out_f4[MAX][i] = mx;
        io.out_f4[VEL][i] = v;
        io.out_f4[BBUF][i] = b;
        io.out_f4[FBUF][i] = f;
    }
};

struct Codec {
    static constexpr uint32_t kAgentBytes = 96;
    TGPU_D static void pack(const uint32_t *w, const PassIO &io, uint32_t i) {
        io.out_f4[MIN][i] = ld_words4(w + 2);
        io.out_f4[MAX][i] = ld_words4(w + 6);
        io.out_f4[VEL][i] = ld_words4(w + 10);
        io.out_f4[BBUF][i] = make_float4(__uint_as_float(w[14]), __uint_as_float(w[15]), __uint_as_float(w[16]),
                                         __uint_as_float(w[18]));
        io.out_f4[FBUF][i] = make_float4(__uint_as_float(w[19]), __uint_as_float(w[20]), __uint_as_float(w[21]),
                                         __uint_as_float(w[23]));
    }
    TGPU_D static void unpack(uint32_t *w, const PassIO &io, uint32_t i, uint32_t) {
        const float4 mn = io.in_f4[MIN][i], mx = io.in_f4[MAX][i], b = io.in_f4[BBUF][i], f = io.in_f4[FBUF][i];
        w[0] = 0u;
        w[1] = 0u;
        st_words4(w + 2, mn);
        st_words4(w + 6, mx);
        st_words4(w + 10, io.in_f4[VEL][i]);
        w[14] = __float_as_uint(b.x);
        w[15] = __float_as_uint(b.y);
        w[16] = __float_as_uint(b.z);
        w[17] = 0u;
        w[18] = __float_as_uint(b.w);
        w[19] = __float_as_uint(f.x);
        w[20] = __float_as_uint(f.y);
        w[21] = __float_as_uint(f.z);
        w[22] = 0u;
        w[23] = __float_as_uint(f.w);
    }
};

constexpr uint32_t bit(int k) { return 1u << k; }

const KernelDesc kKernels[] = {
    {"box_agent_see", nullptr, bit(BBUF), 0, bit(MIN) | bit(MAX), 1, launch_see_t<SeeOnly>, nullptr,
     prepare_see_t<SeeOnly>, 1, 0},
    {"box_agent_see", "box_agent_act", bit(MIN) | bit(MAX) | bit(VEL) | bit(BBUF) | bit(FBUF), 0, bit(MIN) | bit(MAX), 1,
     launch_see_t<SeeAct>, nullptr, prepare_see_t<SeeAct>, 0, 0},
    {nullptr, "box_agent_act", bit(MIN) | bit(MAX) | bit(VEL) | bit(BBUF) | bit(FBUF), 0, 0, 0, nullptr,
     launch_act_t<Act>, nullptr, 0, 0},
};

const ProgramDesc kPrograms[] = {
    {1, {"box_agent_see"}, 1, {0}},
    {1, {"box_agent_act"}, 1, {2}},
    {2, {"box_agent_see", "box_agent_act"}, 1, {1}},
};

const ModelDesc kModel = {
    "box",     96, 5, 0, {kState, kState, kState, kState, kState}, {}, (uint32_t)sizeof(SeeCtx),
    (uint32_t)sizeof(ActCtx), kKernels, 3, kPrograms, 3, pack_t<Codec>, unpack_t<Codec>, 1,
};

}  // namespace box

const ModelDesc *model_box() { return &box::kModel; }

}  // namespace tgpu
