// Boids on the GPU, registered as "boids_see" / "boids_act".
//
// Model: Reynolds' rules in the steering form of Shiffman's "Nature of Code" flocking
// (weights 1.5 / 1.0 / 1.0, max speed 2, max force 0.03): neighbours inside radius r,
// separation from neighbours inside sep_r.
//   see(a, b):  d = b.p - a.p, d2 = (dx*dx + dy*dy) + dz*dz, each product and sum rounded
//               separately (no FMA), so the neighbour decisions are bit-identical to an
//               IEEE evaluation of the same expression on the CPU (the separation term's
//               products too: a product the compiler may fuse into the sum in one inlined
//               copy of the see body and not in another would make results depend on the
//               walk);
//               if 0 < d2 < r2:   count++, coh += d, ali += b.v
//                  if d2 < sep_r2: sep_count++, sep -= d * (1 / d2)
//   act(a):     for (vec, n, w) in (sep, sep_count, w_sep), (ali, count, w_ali),
//               (coh, count, w_coh): if n > 0 and |vec| > 0:
//                  s = vec * (max_speed / |vec|) - v, limited to |s| <= max_force;
//                  acc += w * s
//               v += dt*acc; clamp |v| to max_speed; p += dt*v
// Accumulators are per-step outputs: every see pass starts them from zero and the act
// pass consumes them, so after a see+act step they read back as zero.
//
// AoS record (104 bytes): tag u32[2] @0, p float4 @8, v float4 @24, coh float4 @40,
// ali float4 @56, sep float4 @72, count int @88, sep_count int @92, id int @96, pad @100.
// Streams: f4[0] POS, f4[1] VEL, u32[0] ID (state); f4[2] ACC0 = coh.xyz + count,
// f4[3] ACC1 = ali.xyz + sep_count, f4[4] ACC2 = sep.xyz (per-step).
#include "model.cuh"

namespace tgpu {
namespace boids {

enum { POS = 0, VEL = 1, ACC0 = 2, ACC1 = 3, ACC2 = 4 };
enum { ID = 0 };

struct Ctx {
    float r, r2, sep_r2, w_sep, w_ali, w_coh, max_speed, max_force, dt, pad[3];
};

struct Seer {
    float cx, cy, cz, ax, ay, az, sx, sy, sz;
    int count, sep_count;
    float4 v;
};

TGPU_D void zero(Seer &s) {
    s.cx = s.cy = s.cz = 0.0f;
    s.ax = s.ay = s.az = 0.0f;
    s.sx = s.sy = s.sz = 0.0f;
    s.count = 0;
    s.sep_count = 0;
}

template <class Acc>
TGPU_D void see_fn(Seer &s, const float4 &a, const float4 &b, const Acc &acc, uint32_t j, const Ctx &c) {
    const float dx = b.x - a.x, dy = b.y - a.y, dz = b.z - a.z;
    float d2 = __fmul_rn(dx, dx);
    d2 = __fadd_rn(d2, __fmul_rn(dy, dy));
    d2 = __fadd_rn(d2, __fmul_rn(dz, dz));
    if (d2 < c.r2 && d2 > 0.0f) {
        const float4 bv = acc.f4(1, j);
        s.count += 1;
        s.cx += dx;
        s.cy += dy;
        s.cz += dz;
        s.ax += bv.x;
        s.ay += bv.y;
        s.az += bv.z;
        if (d2 < c.sep_r2) {
            const float inv = __frcp_rn(d2);
            s.sep_count += 1;
            s.sx -= __fmul_rn(dx, inv);
            s.sy -= __fmul_rn(dy, inv);
            s.sz -= __fmul_rn(dz, inv);
        }
    }
}

// The pairs see_fn acts on: 0 < d2 < r2, d2 rounded exactly as see_fn rounds it (the walk
// enters the see body only for these).
TGPU_D bool keep_fn(const float4 &a, const float4 &b, const Ctx &c) {
    const float dx = b.x - a.x, dy = b.y - a.y, dz = b.z - a.z;
    float d2 = __fmul_rn(dx, dx);
    d2 = __fadd_rn(d2, __fmul_rn(dy, dy));
    d2 = __fadd_rn(d2, __fmul_rn(dz, dz));
    return d2 < c.r2 && d2 > 0.0f;
}

TGPU_D float len3(float x, float y, float z) {
    float s = x * x;
    s = s + y * y;
    s = s + z * z;
    return sqrtf(s);
}

TGPU_D void steer(float vx, float vy, float vz, int n, float w, const float4 &v, const Ctx &c, float &ax, float &ay,
                  float &az) {
    if (n <= 0) return;
    const float len = len3(vx, vy, vz);
    if (!(len > 0.0f)) return;
    const float k = c.max_speed / len;
    float sx = vx * k - v.x, sy = vy * k - v.y, sz = vz * k - v.z;
    const float sl = len3(sx, sy, sz);
    if (sl > c.max_force) {
        const float f = c.max_force / sl;
        sx *= f;
        sy *= f;
        sz *= f;
    }
    ax += w * sx;
    ay += w * sy;
    az += w * sz;
}

TGPU_D void act_fn(float4 &p, float4 &v, const Seer &s, const Ctx &c) {
    float ax = 0.0f, ay = 0.0f, az = 0.0f;
    steer(s.sx, s.sy, s.sz, s.sep_count, c.w_sep, v, c, ax, ay, az);
    steer(s.ax, s.ay, s.az, s.count, c.w_ali, v, c, ax, ay, az);
    steer(s.cx, s.cy, s.cz, s.count, c.w_coh, v, c, ax, ay, az);
    v.x = v.x + c.dt * ax;
    v.y = v.y + c.dt * ay;
    v.z = v.z + c.dt * az;
    const float speed = len3(v.x, v.y, v.z);
    if (speed > c.max_speed) {
        const float k = c.max_speed / speed;
        v.x *= k;
        v.y *= k;
        v.z *= k;
    }
    p.x = p.x + c.dt * v.x;
    p.y = p.y + c.dt * v.y;
    p.z = p.z + c.dt * v.z;
}

struct Codec;  // the record codec, defined below

struct SeeOnly {
    using SeeCtx = Ctx;
    using Codec = boids::Codec;
    using ActCtx = Ctx;
    using Seer = boids::Seer;
    static constexpr int kSeenF4 = 2;
    static constexpr int kLaneUnroll = 4;
    static constexpr bool kKeepGate = true;
    static constexpr bool kKeepRejectsSelf = true;  // 0 < d2
    static constexpr bool kSeenMinusSeer = true;    // d = b - a
    TGPU_D static bool keep(const float4 &a, const float4 &b, const Ctx &c) { return keep_fn(a, b, c); }
    TGPU_D static int seen_stream(int k) { return k == 0 ? POS : VEL; }
    TGPU_D static void load(Seer &s, const PassIO &, uint32_t, const Ctx &, const Ctx &) { zero(s); }
    template <class Acc>
    TGPU_D static void see(Seer &s, const float4 &a, const float4 &b, const Acc &acc, uint32_t j, const Ctx &c) {
        see_fn(s, a, b, acc, j, c);
    }
    TGPU_D static void finish(Seer &s, const float4 &, const PassIO &io, uint32_t i, const Ctx &, const Ctx &) {
        io.out_f4[ACC0][i] = make_float4(s.cx, s.cy, s.cz, __int_as_float(s.count));
        io.out_f4[ACC1][i] = make_float4(s.ax, s.ay, s.az, __int_as_float(s.sep_count));
        io.out_f4[ACC2][i] = make_float4(s.sx, s.sy, s.sz, 0.0f);
    }
};

struct SeeAct {
    using SeeCtx = Ctx;
    using Codec = boids::Codec;
    using ActCtx = Ctx;
    using Seer = boids::Seer;
    static constexpr int kSeenF4 = 2;
    static constexpr int kLaneUnroll = 4;
    static constexpr bool kKeepGate = true;
    static constexpr bool kKeepRejectsSelf = true;  // 0 < d2
    static constexpr bool kSeenMinusSeer = true;    // d = b - a
    TGPU_D static bool keep(const float4 &a, const float4 &b, const Ctx &c) { return keep_fn(a, b, c); }
    TGPU_D static int seen_stream(int k) { return k == 0 ? POS : VEL; }
    TGPU_D static void load(Seer &s, const PassIO &io, uint32_t i, const Ctx &, const Ctx &) {
        zero(s);
        s.v = io.in_f4[VEL][i];
    }
    template <class Acc>
    TGPU_D static void see(Seer &s, const float4 &a, const float4 &b, const Acc &acc, uint32_t j, const Ctx &c) {
        see_fn(s, a, b, acc, j, c);
    }
    TGPU_D static void finish(Seer &s, const float4 &a, const PassIO &io, uint32_t i, const Ctx &, const Ctx &c) {
        float4 p = a, v = s.v;
        act_fn(p, v, s, c);
        io.out_f4[POS][i] = p;
        io.out_f4[VEL][i] = v;
    }
};

// boids_act as its own pass (after a boids_see of the same group, e.g. over another
// group): folds the accumulators the see pass left in ACC0..2.
struct Act {
    using ActCtx = Ctx;
    TGPU_D static void act(const PassIO &io, uint32_t i, const Ctx &c) {
        float4 p = io.in_f4[POS][i], v = io.in_f4[VEL][i];
        const float4 a0 = io.in_f4[ACC0][i], a1 = io.in_f4[ACC1][i], a2 = io.in_f4[ACC2][i];
        Seer s;
        s.cx = a0.x;
        s.cy = a0.y;
        s.cz = a0.z;
        s.count = __float_as_int(a0.w);
        s.ax = a1.x;
        s.ay = a1.y;
        s.az = a1.z;
        s.sep_count = __float_as_int(a1.w);
        s.sx = a2.x;
        s.sy = a2.y;
        s.sz = a2.z;
        act_fn(p, v, s, c);
        io.out_f4[POS][i] = p;
        io.out_f4[VEL][i] = v;
    }
};

struct Codec {
    static constexpr uint32_t kAgentBytes = 104;
    TGPU_D static void pack(const uint32_t *w, const PassIO &io, uint32_t i) {
        io.out_f4[POS][i] = ld_words4(w + 2);
        io.out_f4[VEL][i] = ld_words4(w + 6);
        io.out_u32[ID][i] = w[24];
    }
    // program 0: see only (accumulators visible); program 1: see + act (consumed)
    TGPU_D static void unpack(uint32_t *w, const PassIO &io, uint32_t i, uint32_t program) {
        w[0] = 0u;
        w[1] = 0u;
        st_words4(w + 2, io.in_f4[POS][i]);
        st_words4(w + 6, io.in_f4[VEL][i]);
        float4 a0 = make_float4(0.f, 0.f, 0.f, 0.f), a1 = a0, a2 = a0;
        if (program == 0) {
            a0 = io.in_f4[ACC0][i];
            a1 = io.in_f4[ACC1][i];
            a2 = io.in_f4[ACC2][i];
        }
        st_words4(w + 10, make_float4(a0.x, a0.y, a0.z, 0.f));
        st_words4(w + 14, make_float4(a1.x, a1.y, a1.z, 0.f));
        st_words4(w + 18, make_float4(a2.x, a2.y, a2.z, 0.f));
        w[22] = __float_as_uint(a0.w);
        w[23] = __float_as_uint(a1.w);
        w[24] = io.in_u32[ID][i];
        w[25] = 0u;
    }
};

constexpr uint32_t bit(int k) { return 1u << k; }

const KernelDesc kKernels[] = {
    {"boids_see", nullptr, bit(ACC0) | bit(ACC1) | bit(ACC2), 0, bit(POS) | bit(VEL), 2, launch_see_t<SeeOnly>, nullptr,
     prepare_see_t<SeeOnly>, 0, 0},
    {"boids_see", "boids_act", bit(POS) | bit(VEL), 0, bit(POS) | bit(VEL), 2, launch_see_t<SeeAct>, nullptr,
     prepare_see_t<SeeAct>, 0, 0},
    {nullptr, "boids_act", bit(POS) | bit(VEL), 0, 0, 0, nullptr, launch_act_t<Act>, nullptr, 0, 0},
};

const ProgramDesc kPrograms[] = {
    {1, {"boids_see"}, 1, {0}},
    {2, {"boids_see", "boids_act"}, 1, {1}},
    {1, {"boids_act"}, 1, {2}},
};

const ModelDesc kModel = {
    "boids", 104, 5, 1, {kState, kState, kStep, kStep, kStep}, {kState}, (uint32_t)sizeof(Ctx), (uint32_t)sizeof(Ctx),
    kKernels, 3, kPrograms, 3, pack_t<Codec>, unpack_t<Codec>, 0,
};

}  // namespace boids

const ModelDesc *model_boids() { return &boids::kModel; }

}  // namespace tgpu
