/* Oracle model definitions: agent structs and see/act functions in plain C.
 *
 * TEST INFRASTRUCTURE ONLY.  Included by the oracle restatement (oracle/tay_oracle.c,
 * compiled once with REAL=float and once with REAL=double) and by the reference driver
 * (oracle/ref/ref_driver.c, REAL=float) which runs the same functions through the
 * reference's own CPU framework.  Nothing in the shipped library includes this file; the
 * CUDA models are written separately so that the two implementations check each other.
 *
 * Agent layout follows the reference's contract (tay/tay.h:4-13, 76-79): an 8-byte
 * TayAgentTag first, the position as four REALs right after it.  With REAL=float every
 * struct below is layout-compatible with a reference agent.
 *
 * All arithmetic is written out operation by operation in a fixed order, and the oracle
 * is compiled with -ffp-contract=off, so the FP32 build evaluates exactly the IEEE
 * operations listed here (the GPU models use __fadd_rn/__fmul_rn where a decision such
 * as a neighbour count depends on the result).
 */
#ifndef ORACLE_MODELS_H
#define ORACLE_MODELS_H

#include <math.h>

#ifndef REAL
#define REAL float
#pragma pack(pop)

#endif

#define O_SQRT(x) ((REAL)sqrt((double)(x)))

/* Records are packed, like the reference's agents (test/agent.h:2, __attribute__((packed))),
 * so the FP64 build has no alignment padding either and Python can describe every record
 * with a packed dtype. */
#pragma pack(push, 1)

typedef struct {
    unsigned part_i;
    unsigned cell_agent_i;
} OTag;

/* ---------------------------------------------------------------------------------
 * Test model: restates the reference's test agent (test/agent.h:2-10, test/agent.c:2-55).
 *   see: b_buffer += b.p - a.p (x, y, z), b_buffer_count += 1
 *   act: fold the mean displacement into f_buffer, move by v, reflect at the box walls.
 * float4 helpers in the reference touch x, y, z only (test/taystd.c:94-135).
 * --------------------------------------------------------------------------------- */
typedef struct {
    OTag tag;
    REAL p[4];
    REAL v[4];
    REAL b_buffer[4];
    int b_buffer_count;
    REAL f_buffer[4];
    int result_index;
} OTestAgent;

typedef struct {
    REAL min[4];
    REAL max[4];
} OTestActContext;

static inline void o_test_see(void *va, void *vb, void *vc) {
    OTestAgent *a = (OTestAgent *)va;
    OTestAgent *b = (OTestAgent *)vb;
    (void)vc;
    for (int i = 0; i < 3; ++i)
        a->b_buffer[i] = a->b_buffer[i] + (b->p[i] - a->p[i]);
    a->b_buffer_count++;
}

static inline void o_test_act(void *va, void *vc) {
    OTestAgent *a = (OTestAgent *)va;
    const OTestActContext *c = (const OTestActContext *)vc;
    if (a->b_buffer_count != 0) {
        REAL n = (REAL)a->b_buffer_count;
        for (int i = 0; i < 3; ++i) {
            a->f_buffer[i] = a->f_buffer[i] + a->b_buffer[i] / n;
            a->b_buffer[i] = 0;
        }
        a->b_buffer_count = 0;
    }
    for (int i = 0; i < 3; ++i)
        a->p[i] = a->p[i] + a->v[i];
    /* test/agent.c:26-54: all three min walls first, then all three max walls */
    for (int i = 0; i < 3; ++i)
        if (a->p[i] < c->min[i]) {
            a->p[i] = c->min[i];
            a->v[i] = -a->v[i];
        }
    for (int i = 0; i < 3; ++i)
        if (a->p[i] > c->max[i]) {
            a->p[i] = c->max[i];
            a->v[i] = -a->v[i];
        }
}

/* ---------------------------------------------------------------------------------
 * Box test model (non-point agents): restates the reference's box agent
 * (test/agent.h:21-29, test/agent.c:57-118).
 *   see: b_buffer += b.min - a.min (x, y, z), b_buffer_count += 1
 *   act: fold the mean into f_buffer, move min and max by v, then at each wall in the
 *        order min x, y, z, max x, y, z: clamp that corner to the wall, put the other
 *        corner at the size's distance, reverse that velocity component.
 * The reference's float4 helpers leave the w components of min, max, b_buffer and
 * f_buffer undefined once written.
 * --------------------------------------------------------------------------------- */
typedef struct {
    OTag tag;
    REAL min[4];
    REAL max[4];
    REAL v[4];
    REAL b_buffer[4];
    int b_buffer_count;
    REAL f_buffer[4];
    int result_index;
} OBoxAgent;

static inline void o_box_see(void *va, void *vb, void *vc) {
    OBoxAgent *a = (OBoxAgent *)va;
    OBoxAgent *b = (OBoxAgent *)vb;
    (void)vc;
    for (int i = 0; i < 3; ++i)
        a->b_buffer[i] = a->b_buffer[i] + (b->min[i] - a->min[i]);
    a->b_buffer_count++;
}

static inline void o_box_act(void *va, void *vc) {
    OBoxAgent *a = (OBoxAgent *)va;
    const OTestActContext *c = (const OTestActContext *)vc;
    if (a->b_buffer_count != 0) {
        REAL n = (REAL)a->b_buffer_count;
        for (int i = 0; i < 3; ++i) {
            a->f_buffer[i] = a->f_buffer[i] + a->b_buffer[i] / n;
            a->b_buffer[i] = 0;
        }
        a->b_buffer_count = 0;
    }
    REAL size[3];
    for (int i = 0; i < 3; ++i) {
        size[i] = a->max[i] - a->min[i];
        a->min[i] = a->min[i] + a->v[i];
        a->max[i] = a->max[i] + a->v[i];
    }
    for (int i = 0; i < 3; ++i)
        if (a->min[i] < c->min[i]) {
            a->min[i] = c->min[i];
            a->max[i] = c->min[i] + size[i];
            a->v[i] = -a->v[i];
        }
    for (int i = 0; i < 3; ++i)
        if (a->max[i] > c->max[i]) {
            a->max[i] = c->max[i];
            a->min[i] = c->max[i] - size[i];
            a->v[i] = -a->v[i];
        }
}

/* ---------------------------------------------------------------------------------
 * Boids (Reynolds' rules in the steering form of Shiffman's "Nature of Code" flocking,
 * with its weights 1.5 / 1.0 / 1.0 and max speed 2): neighbours within radius r,
 * separation from neighbours within sep_r.
 *   see(a, b): d = b.p - a.p, d2 = (dx*dx + dy*dy) + dz*dz
 *              if 0 < d2 < r2:   count++, coh += d, ali += b.v
 *                 if d2 < sep_r2: sep_count++, sep -= d * (1 / d2)
 *   act(a):    for (vec, n, w) in (sep, sep_count, w_sep), (ali, count, w_ali), (coh, count, w_coh):
 *                 if n > 0 and |vec| > 0:
 *                    s = vec * (max_speed / |vec|) - v;  if |s| > max_force: s *= max_force / |s|
 *                    acc += w * s
 *              v += dt * acc; if |v| > max_speed: v *= max_speed / |v|; p += dt * v
 *              accumulators reset
 * --------------------------------------------------------------------------------- */
typedef struct {
    OTag tag;
    REAL p[4];
    REAL v[4];
    REAL coh[4];
    REAL ali[4];
    REAL sep[4];
    int count;
    int sep_count;
    int id;
    int pad;
} OBoid;

typedef struct {
    REAL r;
    REAL r2;
    REAL sep_r2;
    REAL w_sep;
    REAL w_ali;
    REAL w_coh;
    REAL max_speed;
    REAL max_force;
    REAL dt;
    REAL pad[3];
} OBoidsContext;

static inline void o_boids_see(void *va, void *vb, void *vc) {
    OBoid *a = (OBoid *)va;
    const OBoid *b = (const OBoid *)vb;
    const OBoidsContext *c = (const OBoidsContext *)vc;
    REAL dx = b->p[0] - a->p[0];
    REAL dy = b->p[1] - a->p[1];
    REAL dz = b->p[2] - a->p[2];
    REAL d2 = dx * dx;
    d2 = d2 + dy * dy;
    d2 = d2 + dz * dz;
    if (d2 < c->r2 && d2 > (REAL)0) {
        a->count++;
        a->coh[0] = a->coh[0] + dx;
        a->coh[1] = a->coh[1] + dy;
        a->coh[2] = a->coh[2] + dz;
        a->ali[0] = a->ali[0] + b->v[0];
        a->ali[1] = a->ali[1] + b->v[1];
        a->ali[2] = a->ali[2] + b->v[2];
        if (d2 < c->sep_r2) {
            REAL inv = (REAL)1 / d2;
            a->sep_count++;
            a->sep[0] = a->sep[0] - dx * inv;
            a->sep[1] = a->sep[1] - dy * inv;
            a->sep[2] = a->sep[2] - dz * inv;
        }
    }
}

static inline REAL o_len3(const REAL *x) {
    REAL s = x[0] * x[0];
    s = s + x[1] * x[1];
    s = s + x[2] * x[2];
    return O_SQRT(s);
}

static inline void o_boids_steer(const REAL *vec, int n, REAL w, const REAL *v, const OBoidsContext *c, REAL *acc) {
    if (n <= 0)
        return;
    REAL len = o_len3(vec);
    if (!(len > (REAL)0))
        return;
    REAL k = c->max_speed / len;
    REAL s[3];
    for (int i = 0; i < 3; ++i)
        s[i] = vec[i] * k - v[i];
    REAL sl = o_len3(s);
    if (sl > c->max_force) {
        REAL f = c->max_force / sl;
        for (int i = 0; i < 3; ++i)
            s[i] = s[i] * f;
    }
    for (int i = 0; i < 3; ++i)
        acc[i] = acc[i] + w * s[i];
}

static inline void o_boids_act(void *va, void *vc) {
    OBoid *a = (OBoid *)va;
    const OBoidsContext *c = (const OBoidsContext *)vc;
    REAL acc[3] = {0, 0, 0};
    o_boids_steer(a->sep, a->sep_count, c->w_sep, a->v, c, acc);
    o_boids_steer(a->ali, a->count, c->w_ali, a->v, c, acc);
    o_boids_steer(a->coh, a->count, c->w_coh, a->v, c, acc);
    for (int i = 0; i < 3; ++i)
        a->v[i] = a->v[i] + c->dt * acc[i];
    REAL speed = o_len3(a->v);
    if (speed > c->max_speed) {
        REAL k = c->max_speed / speed;
        for (int i = 0; i < 3; ++i)
            a->v[i] = a->v[i] * k;
    }
    for (int i = 0; i < 3; ++i) {
        a->p[i] = a->p[i] + c->dt * a->v[i];
        a->coh[i] = 0;
        a->ali[i] = 0;
        a->sep[i] = 0;
    }
    a->count = 0;
    a->sep_count = 0;
}

/* ---------------------------------------------------------------------------------
 * Weakly compressible SPH (dam break).  Cubic-spline kernel with support 2h
 * (Monaghan 1992), sigma = 1 / (pi h^3):
 *     W(q)   = sigma * (1 - 1.5 q^2 + 0.75 q^3)   0 <= q < 1
 *            = sigma * 0.25 * (2 - q)^3           1 <= q < 2
 *     dW/dr  = sigma / h * (-3 q + 2.25 q^2)      0 <= q < 1
 *            = -sigma / h * 0.75 * (2 - q)^2      1 <= q < 2
 * Passes, in order (the reference SPH's order, m_sph/main.c:72-75):
 *   density see (self included):  rho_i = sum_j m W(|x_i - x_j|)
 *   pressure act:                  P_i = B ((rho_i / rho0)^7 - 1), B = c0^2 rho0 / 7
 *   force see (j != i):            a_i += -m (P_i/rho_i^2 + P_j/rho_j^2 + Pi_ij) dW/dr x_ij / r
 *                                  Pi_ij = -alpha c0 mu_ij / rho_bar, mu = h v_ij.x_ij / (r^2 + 0.01 h^2)
 *                                  when v_ij.x_ij < 0, else 0 (Monaghan artificial viscosity)
 *   integrate act:                 v += dt (a + g); x += dt v; walls clamp with v *= -0.5
 * --------------------------------------------------------------------------------- */
typedef struct {
    OTag tag;
    REAL p[4];
    REAL v[4];
    REAL a[4];
    REAL rho;
    REAL P;
    int id;
    int pad;
} OSphParticle;

typedef struct {
    REAL h;
    REAL inv_h;
    REAL support2; /* (2h)^2 */
    REAL sigma;    /* 1 / (pi h^3) */
    REAL m;
    REAL rho0;
    REAL B;        /* c0^2 rho0 / 7 */
    REAL c0;
    REAL alpha;
    REAL eta2;     /* 0.01 h^2 */
    REAL dt;
    REAL g[3];
    REAL min[3];
    REAL max[3];
} OSphContext;

static inline REAL o_sph_w(REAL q, REAL sigma) {
    if (q < (REAL)1) {
        REAL q2 = q * q;
        REAL q3 = q2 * q;
        return sigma * (((REAL)1 - (REAL)1.5 * q2) + (REAL)0.75 * q3);
    }
    if (q < (REAL)2) {
        REAL t = (REAL)2 - q;
        return sigma * ((REAL)0.25 * ((t * t) * t));
    }
    return (REAL)0;
}

static inline REAL o_sph_dw(REAL q, REAL sigma, REAL inv_h) {
    if (q < (REAL)1)
        return (sigma * inv_h) * ((REAL)-3 * q + (REAL)2.25 * (q * q));
    if (q < (REAL)2) {
        REAL t = (REAL)2 - q;
        return -(sigma * inv_h) * ((REAL)0.75 * (t * t));
    }
    return (REAL)0;
}

static inline void o_sph_density(void *va, void *vb, void *vc) {
    OSphParticle *a = (OSphParticle *)va;
    const OSphParticle *b = (const OSphParticle *)vb;
    const OSphContext *c = (const OSphContext *)vc;
    REAL dx = a->p[0] - b->p[0];
    REAL dy = a->p[1] - b->p[1];
    REAL dz = a->p[2] - b->p[2];
    REAL r2 = dx * dx;
    r2 = r2 + dy * dy;
    r2 = r2 + dz * dz;
    if (r2 < c->support2) {
        REAL q = O_SQRT(r2) * c->inv_h;
        a->rho = a->rho + c->m * o_sph_w(q, c->sigma);
    }
}

static inline void o_sph_pressure(void *va, void *vc) {
    OSphParticle *a = (OSphParticle *)va;
    const OSphContext *c = (const OSphContext *)vc;
    REAL x = a->rho / c->rho0;
    REAL x2 = x * x;
    REAL x4 = x2 * x2;
    REAL x7 = (x4 * x2) * x;
    a->P = c->B * (x7 - (REAL)1);
}

static inline void o_sph_force(void *va, void *vb, void *vc) {
    OSphParticle *a = (OSphParticle *)va;
    const OSphParticle *b = (const OSphParticle *)vb;
    const OSphContext *c = (const OSphContext *)vc;
    REAL dx = a->p[0] - b->p[0];
    REAL dy = a->p[1] - b->p[1];
    REAL dz = a->p[2] - b->p[2];
    REAL r2 = dx * dx;
    r2 = r2 + dy * dy;
    r2 = r2 + dz * dz;
    if (r2 < c->support2 && r2 > (REAL)0) {
        REAL r = O_SQRT(r2);
        REAL q = r * c->inv_h;
        REAL dw = o_sph_dw(q, c->sigma, c->inv_h);
        REAL vx = a->v[0] - b->v[0];
        REAL vy = a->v[1] - b->v[1];
        REAL vz = a->v[2] - b->v[2];
        REAL vr = vx * dx;
        vr = vr + vy * dy;
        vr = vr + vz * dz;
        REAL visc = 0;
        if (vr < (REAL)0) {
            REAL mu = (c->h * vr) / (r2 + c->eta2);
            REAL rho_bar = (REAL)0.5 * (a->rho + b->rho);
            visc = -(c->alpha * c->c0 * mu) / rho_bar;
        }
        REAL pa = a->P / (a->rho * a->rho);
        REAL pb = b->P / (b->rho * b->rho);
        REAL coef = -c->m * ((pa + pb) + visc) * (dw / r);
        a->a[0] = a->a[0] + coef * dx;
        a->a[1] = a->a[1] + coef * dy;
        a->a[2] = a->a[2] + coef * dz;
    }
}

static inline void o_sph_integrate(void *va, void *vc) {
    OSphParticle *a = (OSphParticle *)va;
    const OSphContext *c = (const OSphContext *)vc;
    for (int i = 0; i < 3; ++i) {
        a->v[i] = a->v[i] + c->dt * (a->a[i] + c->g[i]);
        a->p[i] = a->p[i] + c->dt * a->v[i];
    }
    for (int i = 0; i < 3; ++i) {
        if (a->p[i] < c->min[i]) {
            a->p[i] = c->min[i];
            a->v[i] = (REAL)-0.5 * a->v[i];
        }
        if (a->p[i] > c->max[i]) {
            a->p[i] = c->max[i];
            a->v[i] = (REAL)-0.5 * a->v[i];
        }
    }
    a->rho = 0;
    a->a[0] = 0;
    a->a[1] = 0;
    a->a[2] = 0;
}

#pragma pack(pop)

#endif
