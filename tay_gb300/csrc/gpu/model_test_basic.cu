// The reference's test model on the GPU: test/agent.h:2-19 (Agent, ActContext,
// SeeContext) and test/agent.c:2-55 (agent_see, agent_act), registered under the same
// func names "agent_see" / "agent_act".
//
// AoS record (80 bytes, packed): tag u32[2] @0, p float4 @8, v float4 @24,
// b_buffer float4 @40, b_buffer_count int @56, f_buffer float4 @60, result_index int @76.
// Streams (all persistent state):
//   f4[0] POS  = p (w kept)          f4[1] VEL  = v (w kept)
//   f4[2] BBUF = b_buffer.xyz, w = b_buffer_count (int bits)
//   f4[3] FBUF = f_buffer.xyz, w = result_index (int bits)
// The reference's float4 helpers touch x, y, z only (test/taystd.c:94-135), so the w
// components of b_buffer and f_buffer are never defined by the model; fetch writes 0
// there, and 0 into the framework-owned tag.
#include "model.cuh"

namespace tgpu {
namespace test_basic {

enum { POS = 0, VEL = 1, BBUF = 2, FBUF = 3 };

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
    float4 v, f;
};

// test/agent.c:2-8: b_buffer += b.p - a.p; b_buffer_count++
template <class Acc>
TGPU_D void see_fn(Seer &s, const float4 &a, const float4 &b, const Acc &, uint32_t, const SeeCtx &) {
    s.bx = s.bx + (b.x - a.x);
    s.by = s.by + (b.y - a.y);
    s.bz = s.bz + (b.z - a.z);
    s.count += 1;
}

// test/agent.c:10-55 on registers
TGPU_D void act_fn(float4 &p, float4 &v, float &bx, float &by, float &bz, int &count, float4 &f, const ActCtx &c) {
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
    p.x = p.x + v.x;
    p.y = p.y + v.y;
    p.z = p.z + v.z;
    if (p.x < c.min.x) { p.x = c.min.x; v.x = -v.x; }
    if (p.y < c.min.y) { p.y = c.min.y; v.y = -v.y; }
    if (p.z < c.min.z) { p.z = c.min.z; v.z = -v.z; }
    if (p.x > c.max.x) { p.x = c.max.x; v.x = -v.x; }
    if (p.y > c.max.y) { p.y = c.max.y; v.y = -v.y; }
    if (p.z > c.max.z) { p.z = c.max.z; v.z = -v.z; }
}

struct Codec;  // the record codec, defined below

struct SeeOnly {
    using SeeCtx = test_basic::SeeCtx;
    using Codec = test_basic::Codec;
    using ActCtx = test_basic::SeeCtx;
    using Seer = test_basic::Seer;
    static constexpr int kSeenF4 = 1;
    TGPU_D static int seen_stream(int) { return POS; }
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
    using SeeCtx = test_basic::SeeCtx;
    using Codec = test_basic::Codec;
    using ActCtx = test_basic::ActCtx;
    using Seer = test_basic::Seer;
    static constexpr int kSeenF4 = 1;
    TGPU_D static int seen_stream(int) { return POS; }
    TGPU_D static void load(Seer &s, const PassIO &io, uint32_t i, const SeeCtx &, const ActCtx &) {
        const float4 b = io.in_f4[BBUF][i];
        s.bx = b.x;
        s.by = b.y;
        s.bz = b.z;
        s.count = __float_as_int(b.w);
        s.v = io.in_f4[VEL][i];
        s.f = io.in_f4[FBUF][i];
    }
    template <class Acc>
    TGPU_D static void see(Seer &s, const float4 &a, const float4 &b, const Acc &acc, uint32_t j, const SeeCtx &c) {
        see_fn(s, a, b, acc, j, c);
    }
    TGPU_D static void finish(Seer &s, const float4 &a, const PassIO &io, uint32_t i, const SeeCtx &,
                              const ActCtx &c) {
        float4 p = a;
        act_fn(p, s.v, s.bx, s.by, s.bz, s.count, s.f, c);
        io.out_f4[POS][i] = p;
        io.out_f4[VEL][i] = s.v;
        io.out_f4[BBUF][i] = make_float4(s.bx, s.by, s.bz, __int_as_float(s.count));
        io.out_f4[FBUF][i] = s.f;
    }
};

struct Act {
    using ActCtx = test_basic::ActCtx;
    TGPU_D static void act(const PassIO &io, uint32_t i, const ActCtx &c) {
        float4 p = io.in_f4[POS][i], v = io.in_f4[VEL][i], b = io.in_f4[BBUF][i], f = io.in_f4[FBUF][i];
        int count = __float_as_int(b.w);
        act_fn(p, v, b.x, b.y, b.z, count, f, c);
        b.w = __int_as_float(count);
        io.out_f4[POS][i] = p;
        io.out_f4[VEL][i] = v;
        io.out_f4[BBUF][i] = b;
        io.out_f4[FBUF][i] = f;
    }
};

struct Codec {
    static constexpr uint32_t kAgentBytes = 80;
    TGPU_D static void pack(const uint32_t *w, const PassIO &io, uint32_t i) {
        io.out_f4[POS][i] = ld_words4(w + 2);
        io.out_f4[VEL][i] = ld_words4(w + 6);
        io.out_f4[BBUF][i] = make_float4(__uint_as_float(w[10]), __uint_as_float(w[11]), __uint_as_float(w[12]),
                                         __uint_as_float(w[14]));
        io.out_f4[FBUF][i] = make_float4(__uint_as_float(w[15]), __uint_as_float(w[16]), __uint_as_float(w[17]),
                                         __uint_as_float(w[19]));
    }
    TGPU_D static void unpack(uint32_t *w, const PassIO &io, uint32_t i, uint32_t) {
        const float4 b = io.in_f4[BBUF][i], f = io.in_f4[FBUF][i];
        w[0] = 0u;
        w[1] = 0u;
        st_words4(w + 2, io.in_f4[POS][i]);
        st_words4(w + 6, io.in_f4[VEL][i]);
        w[10] = __float_as_uint(b.x);
        w[11] = __float_as_uint(b.y);
        w[12] = __float_as_uint(b.z);
        w[13] = 0u;
        w[14] = __float_as_uint(b.w);
        w[15] = __float_as_uint(f.x);
        w[16] = __float_as_uint(f.y);
        w[17] = __float_as_uint(f.z);
        w[18] = 0u;
        w[19] = __float_as_uint(f.w);
    }
};

constexpr uint32_t bit(int k) { return 1u << k; }

const KernelDesc kKernels[] = {
    {"agent_see", nullptr, bit(BBUF), 0, bit(POS), 1, launch_see_t<SeeOnly>, nullptr, prepare_see_t<SeeOnly>, 1, 0},
    {"agent_see", "agent_act", bit(POS) | bit(VEL) | bit(BBUF) | bit(FBUF), 0, bit(POS), 1, launch_see_t<SeeAct>,
     nullptr, prepare_see_t<SeeAct>, 0, 0},
    {nullptr, "agent_act", bit(POS) | bit(VEL) | bit(BBUF) | bit(FBUF), 0, 0, 0, nullptr, launch_act_t<Act>, nullptr, 0, 0},
};

const ProgramDesc kPrograms[] = {
    {1, {"agent_see"}, 1, {0}},
    {1, {"agent_act"}, 1, {2}},
    {2, {"agent_see", "agent_act"}, 1, {1}},
};

const ModelDesc kModel = {
    "test_basic", 80, 4, 0, {kState, kState, kState, kState}, {}, (uint32_t)sizeof(SeeCtx), (uint32_t)sizeof(ActCtx),
    kKernels, 3, kPrograms, 3, pack_t<Codec>, unpack_t<Codec>, 0,
};

}  // namespace test_basic

const ModelDesc *model_test_basic() { return &test_basic::kModel; }

}  // namespace tgpu
