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
// The neighbour decision r2 < (2h)^2 uses separately rounded products and sums.  Every
// multiply-add of the see functions is an explicit fused one, and 2 - q after q = r / h is
// an explicitly rounded subtraction (a plain one may be fused with the product in one
// inlined copy and not in another): each copy of a see body (row walk, union walk,
// recording walk, list replay) and of the integrate epilogue rounds the same way.
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
        return sigma * __fmaf_rn(0.75f, q2 * q, __fmaf_rn(-1.5f, q2, 1.0f));
    }
    if (q < 2.0f) {
        const float t = __fsub_rn(2.0f, q);
        return sigma * (0.25f * ((t * t) * t));
    }
    return 0.0f;
}

TGPU_D float kernel_dw(float q, float sigma, float inv_h) {
    if (q < 1.0f) return (sigma * inv_h) * __fmaf_rn(2.25f, q * q, -3.0f * q);
    if (q < 2.0f) {
        const float t = __fsub_rn(2.0f, q);
        return -(sigma * inv_h) * (0.75f * (t * t));
    }
    return 0.0f;
}

TGPU_D float dist2(float dx, float dy, float dz) {
    float r2 = __fmul_rn(dx, dx);
    r2 = __fadd_rn(r2, __fmul_rn(dy, dy));
    return __fadd_rn(r2, __fmul_rn(dz, dz));
}

TGPU_D float kernel_d2w(float q, float sigma, float inv_h) {
    const float s2 = sigma * inv_h * inv_h;
    if (q < 1.0f) return s2 * __fmaf_rn(4.5f, q, -3.0f);
    if (q < 2.0f) return s2 * (1.5f * (2.0f - q));
    return 0.0f;
}

TGPU_D float pressure(float rho, const Ctx &c) {
    const float x = rho / c.rho0;
    const float x2 = x * x;
    const float x4 = x2 * x2;
    const float x7 = (x4 * x2) * x;
    return c.B * (x7 - 1.0f);
}

// ---------------------------------------------------------------- density (+ pressure)

struct Codec;  // the record codec, defined below

struct DensitySeer {
    float rho;
};

template <bool kPressure>
struct Density {
    using SeeCtx = Ctx;
    using Codec = sph::Codec;
    using ActCtx = Ctx;
    using Seer = DensitySeer;
    static constexpr int kSeenF4 = 1;
    // records the pairs inside the support for the force pass that follows (positions do
    // not change between the two)
    static constexpr int kPairList = 1;
    // the see body runs only for pairs inside the support (keep), the particle itself included
    static constexpr bool kKeepGate = true;
    TGPU_D static int seen_stream(int) { return POS; }
    TGPU_D static bool keep(const float4 &a, const float4 &b, const Ctx &c) {
        return dist2(a.x - b.x, a.y - b.y, a.z - b.z) < c.support2;
    }
    TGPU_D static void load(Seer &s, const PassIO &, uint32_t, const Ctx &, const Ctx &) { s.rho = 0.0f; }
    template <class Acc>
    TGPU_D static void see(Seer &s, const float4 &a, const float4 &b, const Acc &, uint32_t, const Ctx &c) {
        const float r2 = dist2(a.x - b.x, a.y - b.y, a.z - b.z);
        if (r2 < c.support2) {
            const float q = __fsqrt_rn(r2) * c.inv_h;
            s.rho = __fmaf_rn(c.m, kernel_w(q, c.sigma), s.rho);
        }
    }
    TGPU_D static void finish(Seer &s, const float4 &, const PassIO &io, uint32_t i, const Ctx &c, const Ctx &) {
        const float P = kPressure ? pressure(s.rho, c) : 0.0f;
        // A = P / rho^2, the pressure term every pair of the force pass needs
        io.out_f4[RP][i] = make_float4(s.rho, P, P / (s.rho * s.rho), 0.0f);
    }
};

// ---------------------------------------------------------------- force (+ integrate)

struct ForceSeer {
    float ax, ay, az;
    float rho, A;
    float4 v;
};

template <bool kIntegrate, bool kStoreAcc = false>
struct Force {
    using SeeCtx = Ctx;
    using Codec = std::conditional_t<kStoreAcc, void, sph::Codec>;  // not the adjoint's recording pass
    using ActCtx = Ctx;
    using Seer = ForceSeer;
    static constexpr int kSeenF4 = 3;
    // replays the density pass's list: its keep test (r2 < that pass's support2) admits
    // every pair this see function acts on (r2 < support2, r2 > 0) when the support is not
    // wider here; for the other candidates the see function does nothing
    static constexpr int kPairList = 2;
    TGPU_D static bool replay_ok(const Ctx &mine, const Ctx &rec) { return mine.support2 <= rec.support2; }
    // when it walks: the see body runs only for 0 < r2 < support2
    static constexpr bool kKeepGate = true;
    static constexpr bool kKeepRejectsSelf = true;
    TGPU_D static bool keep(const float4 &a, const float4 &b, const Ctx &c) {
        const float r2 = dist2(a.x - b.x, a.y - b.y, a.z - b.z);
        return r2 < c.support2 && r2 > 0.0f;
    }
    TGPU_D static int seen_stream(int k) { return k == 0 ? POS : (k == 1 ? VEL : RP); }
    TGPU_D static void load(Seer &s, const PassIO &io, uint32_t i, const Ctx &, const Ctx &) {
        s.ax = s.ay = s.az = 0.0f;
        const float4 rp = io.in_f4[RP][i];
        s.rho = rp.x;
        s.A = rp.z;
        s.v = io.in_f4[VEL][i];
    }
    template <class Acc>
    TGPU_D static void see(Seer &s, const float4 &a, const float4 &b, const Acc &acc, uint32_t j, const Ctx &c) {
        const float dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
        const float r2 = dist2(dx, dy, dz);
        if (r2 < c.support2 && r2 > 0.0f) {
            const float4 bv = acc.f4(1, j);
            const float4 brp = acc.f4(2, j);
            // 1/r from one correctly rounded reciprocal square root, r = r2 * (1/r), dw / r
            // as a product, and the viscosity term's two divisions as one
            const float inv_r = __frsqrt_rn(r2);
            const float r = r2 * inv_r;
            const float q = r * c.inv_h;
            const float dw = kernel_dw(q, c.sigma, c.inv_h);
            const float vx = s.v.x - bv.x, vy = s.v.y - bv.y, vz = s.v.z - bv.z;
            const float vr = __fmaf_rn(vz, dz, __fmaf_rn(vy, dy, vx * dx));
            float visc = 0.0f;
            if (vr < 0.0f) {
                const float rho_bar = 0.5f * (s.rho + brp.x);
                visc = -(c.alpha * c.c0 * (c.h * vr)) / ((r2 + c.eta2) * rho_bar);
            }
            const float coef = -c.m * ((s.A + brp.z) + visc) * (dw * inv_r);
            s.ax = __fmaf_rn(coef, dx, s.ax);
            s.ay = __fmaf_rn(coef, dy, s.ay);
            s.az = __fmaf_rn(coef, dz, s.az);
        }
    }
    TGPU_D static void finish(Seer &s, const float4 &a, const PassIO &io, uint32_t i, const Ctx &, const Ctx &c) {
        if (!kIntegrate || kStoreAcc) io.out_f4[ACC][i] = make_float4(s.ax, s.ay, s.az, 0.0f);
        if (!kIntegrate) return;
        float p[3] = {a.x, a.y, a.z};
        float v[3] = {s.v.x, s.v.y, s.v.z};
        const float acc[3] = {s.ax, s.ay, s.az};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            v[k] = __fmaf_rn(c.dt, acc[k] + c.g[k], v[k]);
            p[k] = __fmaf_rn(c.dt, v[k], p[k]);
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
     prepare_see_t<Density<false>>, 0, 0},
    {"sph_density", "sph_pressure", bit(RP), 0, bit(POS), 1, launch_see_t<Density<true>>, nullptr,
     prepare_see_t<Density<true>>, 0, 1},
    {"sph_force", nullptr, bit(ACC), 0, bit(POS) | bit(VEL) | bit(RP), 3, launch_see_t<Force<false>>, nullptr,
     prepare_see_t<Force<false>>, 0, 2},
    {"sph_force", "sph_integrate", bit(POS) | bit(VEL), 0, bit(POS) | bit(VEL) | bit(RP), 3,
     launch_see_t<Force<true>>, nullptr, prepare_see_t<Force<true>>, 0, 2},
};

const ProgramDesc kPrograms[] = {
    {1, {"sph_density"}, 1, {0}},
    {2, {"sph_density", "sph_pressure"}, 1, {1}},
    {3, {"sph_density", "sph_pressure", "sph_force"}, 2, {1, 2}},
    {4, {"sph_density", "sph_pressure", "sph_force", "sph_integrate"}, 2, {1, 3}},
};


// ---------------------------------------------------------------- adjoint passes
//
// Reverse mode of one SPH step, with the neighbour sets of the forward step held fixed.
// Streams of the adjoint (a separate PassIO, sorted order of the step being reversed):
//   f4 [0] POS, [1] VEL, [2] RP = {rho, P}, [3] ABAR (adjoint of the acceleration),
//   [4] XBAR, [5] VBAR (adjoints of the step's initial position and velocity),
//   [6] RHOBAR, [7] THETA = {d/dalpha, d/dc0} per particle; u32 [0] GID (global id).
// The force is antisymmetric, f_jk = -f_kj (same |x|, s = v.x and rho_bar for both
// orders), so every term a particle receives from its neighbours' accelerations is a
// gather with weight (abar_k - abar_j): the adjoint passes are see passes over the same
// neighbours as the forward ones.
enum { A_POS = 0, A_VEL = 1, A_RP = 2, A_ABAR = 3, A_XBAR = 4, A_VBAR = 5, A_RHOBAR = 6, A_THETA = 7 };
enum { A_GID = 0 };

// integrate (v' = v + dt (a + g), x' = x + dt v', walls) reversed; the wall test is
// re-evaluated from the recorded state, so clamped components pass no gradient through
// the position and -0.5 through the velocity.
struct IntegrateAdj {
    using ActCtx = Ctx;
    TGPU_D static void act(const PassIO &io, uint32_t i, const Ctx &c) {
        const uint32_t gid = io.in_u32[A_GID][i];
        const float4 x = io.in_f4[A_POS][i], v = io.in_f4[A_VEL][i], a = io.in_f4[ACC][i];
        const float4 xb = io.in_f4[A_XBAR][gid], vb = io.in_f4[A_VBAR][gid];  // id order
        const float xs[3] = {x.x, x.y, x.z}, vs[3] = {v.x, v.y, v.z}, as[3] = {a.x, a.y, a.z};
        const float xbs[3] = {xb.x, xb.y, xb.z}, vbs[3] = {vb.x, vb.y, vb.z};
        float ybar[3], ubar[3], abar[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float u = vs[k] + c.dt * (as[k] + c.g[k]);
            const float y = xs[k] + c.dt * u;
            const bool clamped = (y < c.mn[k]) || (y > c.mx[k]);
            ybar[k] = clamped ? 0.0f : xbs[k];
            ubar[k] = clamped ? -0.5f * vbs[k] : vbs[k];
            ubar[k] += c.dt * ybar[k];
            abar[k] = c.dt * ubar[k];
        }
        io.out_f4[A_XBAR][i] = make_float4(ybar[0], ybar[1], ybar[2], 0.0f);
        io.out_f4[A_VBAR][i] = make_float4(ubar[0], ubar[1], ubar[2], 0.0f);
        io.out_f4[A_ABAR][i] = make_float4(abar[0], abar[1], abar[2], 0.0f);
    }
};

struct ForceAdjSeer {
    float4 v, ab;
    float rho, P, A;
    float inv_rho2, drho_A;  // 1 / rho^2 and dA/drho at fixed P = -2 P / rho^3
    float xb[3], vb[3];
    float rhob, Pb, ta, tc;
};

// force adjoint: for each neighbour j, with d = x_k - x_j, w = abar_k - abar_j and
// f_kj = c d, c = -m (A_k + A_j + Pi) D(r), D = W'(r)/r:
//   xbar_k += c w + (w.d) dc/dx_k,  vbar_k += (w.d) dc/dv_k,
//   rhobar_k += (w.d) dc/drho_k,    Pbar_k += (w.d) dc/dP_k,
//   theta += (abar_k.d) dc/d(alpha, c0)
// then the pressure adjoint: rhobar_k += Pbar_k dP/drho, dL/dc0 += Pbar_k 2 P_k / c0.
// The adjoint decides nothing, so it uses the fast reciprocal square root and divisions.
// Every product and sum is an explicit rounded operation (or an explicit fused one), so
// the walk that records the pair list and the replay of a stored list (ForceAdjReplay)
// give the same bits.
struct ForceAdj {
    using SeeCtx = Ctx;
    using ActCtx = Ctx;
    using Seer = ForceAdjSeer;
    static constexpr int kSeenF4 = 4;
    // records the step's pairs inside the support for the density adjoint that follows
    static constexpr int kPairList = 1;
    static constexpr bool kKeepGate = true;
    TGPU_D static bool keep(const float4 &a, const float4 &b, const Ctx &c) {
        return dist2(a.x - b.x, a.y - b.y, a.z - b.z) < c.support2;
    }
    TGPU_D static int seen_stream(int k) { return k == 0 ? A_POS : (k == 1 ? A_VEL : (k == 2 ? A_RP : A_ABAR)); }
    TGPU_D static void load(Seer &s, const PassIO &io, uint32_t i, const Ctx &, const Ctx &) {
        s.v = io.in_f4[A_VEL][i];
        s.ab = io.in_f4[A_ABAR][i];
        const float4 rp = io.in_f4[A_RP][i];
        s.rho = rp.x;
        s.P = rp.y;
        s.A = rp.z;
        s.inv_rho2 = __fdividef(1.0f, rp.x * rp.x);
        s.drho_A = -2.0f * s.A / rp.x;
        s.xb[0] = s.xb[1] = s.xb[2] = 0.0f;
        s.vb[0] = s.vb[1] = s.vb[2] = 0.0f;
        s.rhob = s.Pb = s.ta = s.tc = 0.0f;
    }
    template <class Acc>
    TGPU_D static void see(Seer &s, const float4 &a, const float4 &b, const Acc &acc, uint32_t j, const Ctx &c) {
        const float dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
        const float r2 = dist2(dx, dy, dz);
        if (!(r2 < c.support2 && r2 > 0.0f)) return;
        const float4 bv = acc.f4(1, j), brp = acc.f4(2, j), bab = acc.f4(3, j);
        const float rinv = rsqrtf(r2);
        const float r = __fmul_rn(r2, rinv);
        const float q = __fmul_rn(r, c.inv_h);
        const float dw = kernel_dw(q, c.sigma, c.inv_h);
        const float d2w = kernel_d2w(q, c.sigma, c.inv_h);
        const float D = __fmul_rn(dw, rinv);
        const float Dp_r = __fmul_rn(__fmul_rn(__fsub_rn(d2w, D), rinv), rinv);  // (dD/dr) / r
        const float vx = s.v.x - bv.x, vy = s.v.y - bv.y, vz = s.v.z - bv.z;
        const float sv = __fmaf_rn(vz, dz, __fmaf_rn(vy, dy, __fmul_rn(vx, dx)));
        float Pi = 0.0f, Pi_s = 0.0f, Pi_r2 = 0.0f, Pi_rb = 0.0f, Pi_al = 0.0f, Pi_c0 = 0.0f;
        if (sv < 0.0f) {
            const float inv_rb = __fdividef(2.0f, __fadd_rn(s.rho, brp.x));
            const float inv_den = __fdividef(1.0f, __fadd_rn(r2, c.eta2));
            const float k0 = __fmul_rn(__fmul_rn(c.h, inv_den), inv_rb);
            Pi_al = __fmul_rn(__fmul_rn(-c.c0, k0), sv);
            Pi_c0 = __fmul_rn(__fmul_rn(-c.alpha, k0), sv);
            Pi = __fmul_rn(c.alpha, Pi_al);
            Pi_s = __fmul_rn(__fmul_rn(-c.alpha, c.c0), k0);
            Pi_r2 = __fmul_rn(-Pi, inv_den);
            Pi_rb = __fmul_rn(-Pi, inv_rb);
        }
        const float T = __fadd_rn(__fadd_rn(s.A, brp.z), Pi);
        const float mD = __fmul_rn(-c.m, D);
        const float cc = __fmul_rn(mD, T);
        const float wx = s.ab.x - bab.x, wy = s.ab.y - bab.y, wz = s.ab.z - bab.z;
        const float xw = __fmaf_rn(dz, wz, __fmaf_rn(dy, wy, __fmul_rn(dx, wx)));
        const float coef_d = __fmul_rn(-c.m, __fmaf_rn(T, Dp_r, __fmul_rn(__fmul_rn(2.0f, Pi_r2), D)));
        const float coef_v = __fmul_rn(mD, Pi_s);
        const float dd[3] = {dx, dy, dz}, ww[3] = {wx, wy, wz}, vv[3] = {vx, vy, vz};
        const float xwv = __fmul_rn(xw, coef_v);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float inner = __fmaf_rn(coef_d, dd[k], __fmul_rn(coef_v, vv[k]));
            s.xb[k] = __fadd_rn(s.xb[k], __fmaf_rn(xw, inner, __fmul_rn(cc, ww[k])));
            s.vb[k] = __fmaf_rn(xwv, dd[k], s.vb[k]);
        }
        const float xmD = __fmul_rn(xw, mD);
        s.rhob = __fmaf_rn(xmD, __fmaf_rn(0.5f, Pi_rb, s.drho_A), s.rhob);
        s.Pb = __fadd_rn(s.Pb, xmD);
        const float ad = __fmul_rn(__fmaf_rn(s.ab.z, dz, __fmaf_rn(s.ab.y, dy, __fmul_rn(s.ab.x, dx))), mD);
        s.ta = __fmaf_rn(ad, Pi_al, s.ta);
        s.tc = __fmaf_rn(ad, Pi_c0, s.tc);
    }
    TGPU_D static void finish(Seer &s, const float4 &, const PassIO &io, uint32_t i, const Ctx &c, const Ctx &) {
        s.Pb *= s.inv_rho2;  // dc/dP_k = -m D / rho_k^2
        const float x = s.rho / c.rho0;
        const float x2 = x * x;
        const float x6 = (x2 * x2) * x2;
        s.rhob += s.Pb * (c.B * 7.0f * x6 / c.rho0);
        s.tc += s.Pb * (2.0f * s.P / c.c0);
        io.out_f4[A_RHOBAR][i] = make_float4(s.rhob, 0.0f, 0.0f, 0.0f);
        const float4 xb = io.in_f4[A_XBAR][i], vb = io.in_f4[A_VBAR][i];
        io.out_f4[A_XBAR][i] = make_float4(xb.x + s.xb[0], xb.y + s.xb[1], xb.z + s.xb[2], 0.0f);
        io.out_f4[A_VBAR][i] = make_float4(vb.x + s.vb[0], vb.y + s.vb[1], vb.z + s.vb[2], 0.0f);
        io.out_f4[A_THETA][i] = make_float4(s.ta, s.tc, 0.0f, 0.0f);
    }
};

// The force adjoint over a stored pair list of the step (the list its forward density pass
// recorded): the same see function, no walk and no recording; DensityAdj then replays the
// same list.
struct ForceAdjReplay : ForceAdj {
    static constexpr int kPairList = 2;
    TGPU_D static bool replay_ok(const Ctx &mine, const Ctx &rec) { return mine.support2 <= rec.support2; }
};

struct DensityAdjSeer {
    float rhob;
    float xb[3];
};

// density adjoint: xbar_k += sum_j (rhobar_k + rhobar_j) m W'(r) d / r
struct DensityAdj {
    using SeeCtx = Ctx;
    using ActCtx = Ctx;
    using Seer = DensityAdjSeer;
    static constexpr int kSeenF4 = 2;
    // replays the force adjoint's list (same pairs: r2 < support2, r2 > 0)
    static constexpr int kPairList = 2;
    TGPU_D static bool replay_ok(const Ctx &mine, const Ctx &rec) { return mine.support2 <= rec.support2; }
    // when it walks: the see body runs only for 0 < r2 < support2
    static constexpr bool kKeepGate = true;
    static constexpr bool kKeepRejectsSelf = true;
    TGPU_D static bool keep(const float4 &a, const float4 &b, const Ctx &c) {
        const float r2 = dist2(a.x - b.x, a.y - b.y, a.z - b.z);
        return r2 < c.support2 && r2 > 0.0f;
    }
    TGPU_D static int seen_stream(int k) { return k == 0 ? A_POS : A_RHOBAR; }
    TGPU_D static void load(Seer &s, const PassIO &io, uint32_t i, const Ctx &, const Ctx &) {
        s.rhob = io.in_f4[A_RHOBAR][i].x;
        s.xb[0] = s.xb[1] = s.xb[2] = 0.0f;
    }
    template <class Acc>
    TGPU_D static void see(Seer &s, const float4 &a, const float4 &b, const Acc &acc, uint32_t j, const Ctx &c) {
        const float dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
        const float r2 = dist2(dx, dy, dz);
        if (!(r2 < c.support2 && r2 > 0.0f)) return;
        const float rinv = rsqrtf(r2);
        const float g = (s.rhob + acc.f4(1, j).x) * c.m * kernel_dw(r2 * rinv * c.inv_h, c.sigma, c.inv_h) * rinv;
        s.xb[0] = __fmaf_rn(g, dx, s.xb[0]);
        s.xb[1] = __fmaf_rn(g, dy, s.xb[1]);
        s.xb[2] = __fmaf_rn(g, dz, s.xb[2]);
    }
    TGPU_D static void finish(Seer &s, const float4 &, const PassIO &io, uint32_t i, const Ctx &, const Ctx &) {
        const float4 xb = io.in_f4[A_XBAR][i];
        io.out_f4[A_XBAR][i] = make_float4(xb.x + s.xb[0], xb.y + s.xb[1], xb.z + s.xb[2], 0.0f);
    }
};

// adjoints of the step's initial state back to id order (the order of the step before)
struct ScatterAdj {
    using ActCtx = Ctx;
    TGPU_D static void act(const PassIO &io, uint32_t i, const Ctx &) {
        const uint32_t gid = io.in_u32[A_GID][i];
        io.out_f4[A_XBAR][gid] = io.in_f4[A_XBAR][i];
        io.out_f4[A_VBAR][gid] = io.in_f4[A_VBAR][i];
    }
};

const SphAdjointKernels kAdjoint = {
    launch_see_t<Force<true, true>>, prepare_see_t<Force<true, true>>,
    launch_act_t<IntegrateAdj>,
    launch_see_t<ForceAdj>, prepare_see_t<ForceAdj>,
    launch_see_t<ForceAdjReplay>, prepare_see_t<ForceAdjReplay>,
    launch_see_t<DensityAdj>, prepare_see_t<DensityAdj>,
    launch_act_t<ScatterAdj>,
    (uint32_t)sizeof(Ctx),
};

const ModelDesc kModel = {
    "sph", 72, 4, 1, {kState, kState, kStep, kStep}, {kState}, (uint32_t)sizeof(Ctx), (uint32_t)sizeof(Ctx),
    kKernels, 4, kPrograms, 4, pack_t<Codec>, unpack_t<Codec>, 0,
};

}  // namespace sph

const ModelDesc *model_sph() { return &sph::kModel; }
const SphAdjointKernels *sph_adjoint_kernels() { return &sph::kAdjoint; }

}  // namespace tgpu
