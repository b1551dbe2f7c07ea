// Weakly compressible SPH on the GPU, registered as "sph_density", "sph_pressure",
// "sph_force", "sph_integrate" (pass order of the reference SPH, m_sph/main.c:72-75).
//
// Cubic-spline kernel (Monaghan 1992), support 2h, sigma = 1 / (pi h^3):
//   W(q)  = sigma (1 - 1.5 q^2 + 0.75 q^3), q < 1;  sigma 0.25 (2 - q)^3, 1 <= q < 2
//   dW/dr = sigma/h (-3 q + 2.25 q^2),      q < 1; -sigma/h 0.75 (2 - q)^2, 1 <= q < 2
// density (self included):  rho_i = sum_j m W(|x_i - x_j| / h)
// pressure (Tait, gamma 7):  P_i = B ((rho_i / rho0)^7 - 1), B = c0^2 rho0 / 7
// force (j != i):            a_i += -m (P_i/rho_i^2 + P_j/rho_j^2 + Pi_ij) dW/dr x_ij / r,
//                            Pi_ij = -alpha c0 mu_ij / rho_bar when v_ij.x_ij < 0,
//                            mu_ij = h v_ij.x_ij / (r^2 + 0.01 h^2)
// integrate:                 v += dt (a + g); x += dt v; walls: clamp, v *= -0.5
// The neighbour decision r2 < (2h)^2 uses separately rounded products and sums.
//
// AoS record (72 bytes): tag u32[2] @0, p float4 @8, v float4 @24, a float4 @40,
// rho @56, P @60, id @64, pad @68.
// Streams: f4[0] POS, f4[1] VEL, u32[0] ID (state); f4[2] RP = {rho, P} and
// f4[3] ACC = a.xyz (per-step: density and acceleration start from zero every step,
// pressure is recomputed every step; integrate leaves rho = a = 0).
#include "model.cuh"

namespace tgpu {
namespace sph {

enum { POS = 0, VEL = 1, RP = 2, ACC = 3 };
enum { ID = 0 };

struct Ctx {
    float h, inv_h, support2, sigma, m, rho0, B, c0, alpha, eta2, dt;
    float g[3];
    float mn[3];
    float mx[3];
};

TGPU_D float kernel_w(float q, float sigma) {
    if (q < 1.0f) {
        const float q2 = q * q;
        return sigma * ((1.0f - 1.5f * q2) + 0.75f * (q2 * q));
    }
    if (q < 2.0f) {
        const float t = 2.0f - q;
        return sigma * (0.25f * ((t * t) * t));
    }
    return 0.0f;
}

TGPU_D float kernel_dw(float q, float sigma, float inv_h) {
    if (q < 1.0f) return (sigma * inv_h) * (-3.0f * q + 2.25f * (q * q));
    if (q < 2.0f) {
        const float t = 2.0f - q;
        return -(sigma * inv_h) * (0.75f * (t * t));
    }
    return 0.0f;
}

TGPU_D float dist2(float dx, float dy, float dz) {
    float r2 = __fmul_rn(dx, dx);
    r2 = __fadd_rn(r2, __fmul_rn(dy, dy));
    return __fadd_rn(r2, __fmul_rn(dz, dz));
}

TGPU_D float pressure(float rho, const Ctx &c) {
    const float x = rho / c.rho0;
    const float x2 = x * x;
    const float x4 = x2 * x2;
    const float x7 = (x4 * x2) * x;
    return c.B * (x7 - 1.0f);
}

// ---------------------------------------------------------------- density (+ pressure)

struct DensitySeer {
    float rho;
};

template <bool kPressure>
struct Density {
    using SeeCtx = Ctx;
    using ActCtx = Ctx;
    using Seer = DensitySeer;
    static constexpr int kSeenF4 = 1;
    TGPU_D static int seen_stream(int) { return POS; }
    TGPU_D static void load(Seer &s, const PassIO &, uint32_t, const Ctx &, const Ctx &) { s.rho = 0.0f; }
    template <class Acc>
    TGPU_D static void see(Seer &s, const float4 &a, const float4 &b, const Acc &, uint32_t, const Ctx &c) {
        const float r2 = dist2(a.x - b.x, a.y - b.y, a.z - b.z);
        if (r2 < c.support2) {
            const float q = __fsqrt_rn(r2) * c.inv_h;
            s.rho += c.m * kernel_w(q, c.sigma);
        }
    }
    TGPU_D static void finish(Seer &s, const float4 &, const PassIO &io, uint32_t i, const Ctx &c, const Ctx &) {
        io.out_f4[RP][i] = make_float4(s.rho, kPressure ? pressure(s.rho, c) : 0.0f, 0.0f, 0.0f);
    }
};

// ---------------------------------------------------------------- force (+ integrate)

struct ForceSeer {
    float ax, ay, az;
    float rho, P;
    float4 v;
};

template <bool kIntegrate>
struct Force {
    using SeeCtx = Ctx;
    using ActCtx = Ctx;
    using Seer = ForceSeer;
    static constexpr int kSeenF4 = 3;
    TGPU_D static int seen_stream(int k) { return k == 0 ? POS : (k == 1 ? VEL : RP); }
    TGPU_D static void load(Seer &s, const PassIO &io, uint32_t i, const Ctx &, const Ctx &) {
        s.ax = s.ay = s.az = 0.0f;
        const float4 rp = io.in_f4[RP][i];
        s.rho = rp.x;
        s.P = rp.y;
        s.v = io.in_f4[VEL][i];
    }
    template <class Acc>
    TGPU_D static void see(Seer &s, const float4 &a, const float4 &b, const Acc &acc, uint32_t j, const Ctx &c) {
        const float dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
        const float r2 = dist2(dx, dy, dz);
        if (r2 < c.support2 && r2 > 0.0f) {
            const float4 bv = acc.f4(1, j);
            const float4 brp = acc.f4(2, j);
            const float r = __fsqrt_rn(r2);
            const float q = r * c.inv_h;
            const float dw = kernel_dw(q, c.sigma, c.inv_h);
            const float vx = s.v.x - bv.x, vy = s.v.y - bv.y, vz = s.v.z - bv.z;
            const float vr = (vx * dx + vy * dy) + vz * dz;
            float visc = 0.0f;
            if (vr < 0.0f) {
                const float mu = (c.h * vr) / (r2 + c.eta2);
                const float rho_bar = 0.5f * (s.rho + brp.x);
                visc = -(c.alpha * c.c0 * mu) / rho_bar;
            }
            const float pa = s.P / (s.rho * s.rho);
            const float pb = brp.y / (brp.x * brp.x);
            const float coef = -c.m * ((pa + pb) + visc) * (dw / r);
            s.ax += coef * dx;
            s.ay += coef * dy;
            s.az += coef * dz;
        }
    }
    TGPU_D static void finish(Seer &s, const float4 &a, const PassIO &io, uint32_t i, const Ctx &, const Ctx &c) {
        if (!kIntegrate) {
            io.out_f4[ACC][i] = make_float4(s.ax, s.ay, s.az, 0.0f);
            return;
        }
        float p[3] = {a.x, a.y, a.z};
        float v[3] = {s.v.x, s.v.y, s.v.z};
        const float acc[3] = {s.ax, s.ay, s.az};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            v[k] = v[k] + c.dt * (acc[k] + c.g[k]);
            p[k] = p[k] + c.dt * v[k];
        }
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            if (p[k] < c.mn[k]) {
                p[k] = c.mn[k];
                v[k] = -0.5f * v[k];
            }
            if (p[k] > c.mx[k]) {
                p[k] = c.mx[k];
                v[k] = -0.5f * v[k];
            }
        }
        io.out_f4[POS][i] = make_float4(p[0], p[1], p[2], a.w);
        io.out_f4[VEL][i] = make_float4(v[0], v[1], v[2], s.v.w);
    }
};

struct Codec {
    static constexpr uint32_t kAgentBytes = 72;
    TGPU_D static void pack(const uint32_t *w, const PassIO &io, uint32_t i) {
        io.out_f4[POS][i] = ld_words4(w + 2);
        io.out_f4[VEL][i] = ld_words4(w + 6);
        io.out_u32[ID][i] = w[16];
    }
    // program 0: density; 1: density + pressure; 2: ... + force; 3: full step
    TGPU_D static void unpack(uint32_t *w, const PassIO &io, uint32_t i, uint32_t program) {
        w[0] = 0u;
        w[1] = 0u;
        st_words4(w + 2, io.in_f4[POS][i]);
        st_words4(w + 6, io.in_f4[VEL][i]);
        const float4 rp = io.in_f4[RP][i];
        float4 a = make_float4(0.f, 0.f, 0.f, 0.f);
        if (program == 2) a = io.in_f4[ACC][i];
        st_words4(w + 10, a);
        w[14] = __float_as_uint(program == 3 ? 0.0f : rp.x);
        w[15] = __float_as_uint(program == 0 ? 0.0f : rp.y);
        w[16] = io.in_u32[ID][i];
        w[17] = 0u;
    }
};

constexpr uint32_t bit(int k) { return 1u << k; }

const KernelDesc kKernels[] = {
    {"sph_density", nullptr, bit(RP), 0, bit(POS), 1, launch_see_t<Density<false>>, nullptr,
     prepare_see_t<Density<false>>},
    {"sph_density", "sph_pressure", bit(RP), 0, bit(POS), 1, launch_see_t<Density<true>>, nullptr,
     prepare_see_t<Density<true>>},
    {"sph_force", nullptr, bit(ACC), 0, bit(POS) | bit(VEL) | bit(RP), 3, launch_see_t<Force<false>>, nullptr,
     prepare_see_t<Force<false>>},
    {"sph_force", "sph_integrate", bit(POS) | bit(VEL), 0, bit(POS) | bit(VEL) | bit(RP), 3,
     launch_see_t<Force<true>>, nullptr, prepare_see_t<Force<true>>},
};

const ProgramDesc kPrograms[] = {
    {1, {"sph_density"}, 1, {0}},
    {2, {"sph_density", "sph_pressure"}, 1, {1}},
    {3, {"sph_density", "sph_pressure", "sph_force"}, 2, {1, 2}},
    {4, {"sph_density", "sph_pressure", "sph_force", "sph_integrate"}, 2, {1, 3}},
};

const ModelDesc kModel = {
    "sph", 72, 4, 1, {kState, kState, kStep, kStep}, {kState}, (uint32_t)sizeof(Ctx), (uint32_t)sizeof(Ctx),
    kKernels, 4, kPrograms, 4, pack_t<Codec>, unpack_t<Codec>,
};

}  // namespace sph

const ModelDesc *model_sph() { return &sph::kModel; }

}  // namespace tgpu
