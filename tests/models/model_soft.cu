// A device model the library does not ship, built by the tests as its own shared library
// and registered through tgpu_register_model_library: soft-sphere repulsion with
// damping, func names "soft_see" / "soft_act".
//
//   see(a, b):  d = a.p - b.p, d2 = (dx*dx + dy*dy) + dz*dz (each product and sum rounded
//               separately); if 0 < d2 < r2:  dist = sqrt(d2) (correctly rounded),
//               f += k (r - dist) / dist * d, count++
//   act(a):     v = damping v + dt f;  p += dt v;  a component outside [lo, hi] is clamped
//               and its velocity reversed;  f = 0, count = 0
// AoS record (64 bytes): tag u32[2] @0, p float4 @8, v float4 @24, f float4 @40 (w: the
// count as int bits), id int @56, pad @60.
// Streams: f4[0] POS, f4[1] VEL, u32[0] ID (state); f4[2] FRC = f.xyz + count (per step).
#include "tay_gpu_model.cuh"

namespace soft {

using namespace tgpu;

enum { POS = 0, VEL = 1, FRC = 2 };
enum { ID = 0 };

struct Ctx {
    float r, r2, k, dt, damping, lo[3], hi[3], pad;
};

struct Seer {
    float fx, fy, fz;
    int count;
    float4 v;
};

template <class Acc>
TGPU_D void see_fn(Seer &s, const float4 &a, const float4 &b, const Acc &, uint32_t, const Ctx &c) {
    const float dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
    float d2 = __fmul_rn(dx, dx);
    d2 = __fadd_rn(d2, __fmul_rn(dy, dy));
    d2 = __fadd_rn(d2, __fmul_rn(dz, dz));
    if (d2 < c.r2 && d2 > 0.0f) {
        const float dist = __fsqrt_rn(d2);
        const float w = __fdiv_rn(__fmul_rn(c.k, __fsub_rn(c.r, dist)), dist);
        s.fx = __fadd_rn(s.fx, __fmul_rn(w, dx));
        s.fy = __fadd_rn(s.fy, __fmul_rn(w, dy));
        s.fz = __fadd_rn(s.fz, __fmul_rn(w, dz));
        s.count += 1;
    }
}

TGPU_D void act_fn(float4 &p, float4 &v, float fx, float fy, float fz, const Ctx &c) {
    float pv[3] = {p.x, p.y, p.z}, vv[3] = {v.x, v.y, v.z};
    const float f[3] = {fx, fy, fz};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        vv[k] = __fadd_rn(__fmul_rn(c.damping, vv[k]), __fmul_rn(c.dt, f[k]));
        pv[k] = __fadd_rn(pv[k], __fmul_rn(c.dt, vv[k]));
        if (pv[k] < c.lo[k]) {
            pv[k] = c.lo[k];
            vv[k] = -vv[k];
        }
        if (pv[k] > c.hi[k]) {
            pv[k] = c.hi[k];
            vv[k] = -vv[k];
        }
    }
    p = make_float4(pv[0], pv[1], pv[2], p.w);
    v = make_float4(vv[0], vv[1], vv[2], v.w);
}

struct Codec {
    static constexpr uint32_t kAgentBytes = 64;
    TGPU_D static void pack(const uint32_t *w, const PassIO &io, uint32_t i) {
        io.out_f4[POS][i] = ld_words4(w + 2);
        io.out_f4[VEL][i] = ld_words4(w + 6);
        io.out_u32[ID][i] = w[14];
    }
    // program 0: see only (forces and counts visible); 1: see + act and 2: act (consumed)
    TGPU_D static void unpack(uint32_t *w, const PassIO &io, uint32_t i, uint32_t program) {
        w[0] = 0u;
        w[1] = 0u;
        st_words4(w + 2, io.in_f4[POS][i]);
        st_words4(w + 6, io.in_f4[VEL][i]);
        st_words4(w + 10, program == 0 ? io.in_f4[FRC][i] : make_float4(0.f, 0.f, 0.f, 0.f));
        w[14] = io.in_u32[ID][i];
        w[15] = 0u;
    }
};

struct SeeOnly {
    using SeeCtx = Ctx;
    using ActCtx = Ctx;
    using Codec = soft::Codec;
    using Seer = soft::Seer;
    static constexpr int kSeenF4 = 1;
    TGPU_D static int seen_stream(int) { return POS; }
    TGPU_D static void load(Seer &s, const PassIO &, uint32_t, const Ctx &, const Ctx &) {
        s.fx = s.fy = s.fz = 0.0f;
        s.count = 0;
    }
    template <class Acc>
    TGPU_D static void see(Seer &s, const float4 &a, const float4 &b, const Acc &acc, uint32_t j, const Ctx &c) {
        see_fn(s, a, b, acc, j, c);
    }
    TGPU_D static void finish(Seer &s, const float4 &, const PassIO &io, uint32_t i, const Ctx &, const Ctx &) {
        io.out_f4[FRC][i] = make_float4(s.fx, s.fy, s.fz, __int_as_float(s.count));
    }
};

struct SeeAct {
    using SeeCtx = Ctx;
    using ActCtx = Ctx;
    using Codec = soft::Codec;
    using Seer = soft::Seer;
    static constexpr int kSeenF4 = 1;
    TGPU_D static int seen_stream(int) { return POS; }
    TGPU_D static void load(Seer &s, const PassIO &io, uint32_t i, const Ctx &, const Ctx &) {
        s.fx = s.fy = s.fz = 0.0f;
        s.count = 0;
        s.v = io.in_f4[VEL][i];
    }
    template <class Acc>
    TGPU_D static void see(Seer &s, const float4 &a, const float4 &b, const Acc &acc, uint32_t j, const Ctx &c) {
        see_fn(s, a, b, acc, j, c);
    }
    TGPU_D static void finish(Seer &s, const float4 &a, const PassIO &io, uint32_t i, const Ctx &, const Ctx &c) {
        float4 p = a, v = s.v;
        act_fn(p, v, s.fx, s.fy, s.fz, c);
        io.out_f4[POS][i] = p;
        io.out_f4[VEL][i] = v;
    }
};

struct Act {
    using ActCtx = Ctx;
    TGPU_D static void act(const PassIO &io, uint32_t i, const Ctx &c) {
        float4 p = io.in_f4[POS][i], v = io.in_f4[VEL][i];
        const float4 f = io.in_f4[FRC][i];
        act_fn(p, v, f.x, f.y, f.z, c);
        io.out_f4[POS][i] = p;
        io.out_f4[VEL][i] = v;
    }
};

constexpr uint32_t bit(int k) { return 1u << k; }

// Built with -DSOFT_SEE_NAME='"boids_see"' the model claims a func name the library's boids
// model owns, which registration must refuse.
#ifndef SOFT_SEE_NAME
#define SOFT_SEE_NAME "soft_see"
#endif

const KernelDesc kKernels[] = {
    {SOFT_SEE_NAME, nullptr, bit(FRC), 0, bit(POS), 1, launch_see_t<SeeOnly>, nullptr, prepare_see_t<SeeOnly>, 0, 0},
    {SOFT_SEE_NAME, "soft_act", bit(POS) | bit(VEL), 0, bit(POS), 1, launch_see_t<SeeAct>, nullptr,
     prepare_see_t<SeeAct>, 0, 0},
    {nullptr, "soft_act", bit(POS) | bit(VEL), 0, 0, 0, nullptr, launch_act_t<Act>, nullptr, 0, 0},
};

const ProgramDesc kPrograms[] = {
    {1, {SOFT_SEE_NAME}, 1, {0}},
    {2, {SOFT_SEE_NAME, "soft_act"}, 1, {1}},
    {1, {"soft_act"}, 1, {2}},
};

const ModelDesc kModel = {
    "soft_spheres", Codec::kAgentBytes, 3, 1, {kState, kState, kStep}, {kState}, (uint32_t)sizeof(Ctx),
    (uint32_t)sizeof(Ctx), kKernels, 3, kPrograms, 3, pack_t<Codec>, unpack_t<Codec>, 0,
};

}  // namespace soft

extern "C" const void *tgpu_model_entry(unsigned *abi) {
    if (abi) *abi = TGPU_MODEL_ABI;
    return &soft::kModel;
}
