/* ORACLE (test infrastructure, not the product): FP64 CPU adjoint of the SPH rollout.
 *
 * The forward step is the oracle SPH model (oracle/oracle_models.h: o_sph_density,
 * o_sph_pressure, o_sph_force, o_sph_integrate, compiled here with REAL=double), over every
 * pair within the support.  The pairs come from a uniform grid of cells no smaller than the
 * support (only the 27 cells around a particle's cell can hold its neighbours), and each
 * particle's neighbours are visited in ascending index order, so every per-particle sum is
 * the one an all-pairs loop over j = 0 .. n-1 gives, bit for bit.  Particles are split
 * over the host's cores (each thread owns a range of particles and writes only their
 * entries; the two parameter gradients are summed per particle, then over particles in
 * index order).  The backward sweep is the reverse mode of that step with the neighbour
 * sets held fixed, written independently of the CUDA adjoint:
 *   integrate: clamped components pass no gradient through the position and -0.5 through
 *              the velocity; ubar = vbar' (+ dt xbar'), abar = dt ubar;
 *   force:     f_kj = c d, c = -m (A_k + A_j + Pi) W'(r)/r, d = x_k - x_j; the gradient a
 *              particle receives is a sum over neighbours with weight (abar_k - abar_j)
 *              because f_jk = -f_kj;
 *   pressure:  rhobar += Pbar dP/drho, d/dc0 += Pbar 2P/c0;
 *   density:   xbar_k += sum_j (rhobar_k + rhobar_j) m W'(r) d / r.
 * Only tests/ load it.
 */
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#define REAL double
#include "oracle_models.h"

typedef struct {
    double x[3], v[3];
} OState;

/* ---- a parallel loop over particle ranges: one thread per core, each a contiguous range */

typedef void (*ORangeFn)(void *arg, int lo, int hi, int thread);

typedef struct {
    ORangeFn fn;
    void *arg;
    int lo, hi, thread;
} OJob;

static void *o_job_main(void *p) {
    OJob *j = (OJob *)p;
    j->fn(j->arg, j->lo, j->hi, j->thread);
    return NULL;
}

enum { O_MAX_THREADS = 64 };

static int o_threads(int n) {
    long t = sysconf(_SC_NPROCESSORS_ONLN);
    if (t < 1) t = 1;
    if (t > O_MAX_THREADS) t = O_MAX_THREADS;
    if (t > n / 256 + 1) t = n / 256 + 1;
    return (int)t;
}

/* Runs fn over [0, n) split into `threads` ranges; a range whose thread cannot be started
 * runs on the calling thread. */
static void o_parallel(int n, int threads, ORangeFn fn, void *arg) {
    pthread_t th[O_MAX_THREADS];
    int started[O_MAX_THREADS];
    OJob jobs[O_MAX_THREADS];
    for (int t = 0; t < threads; ++t) {
        jobs[t].fn = fn;
        jobs[t].arg = arg;
        jobs[t].lo = (int)((long long)n * t / threads);
        jobs[t].hi = (int)((long long)n * (t + 1) / threads);
        jobs[t].thread = t;
        started[t] = t > 0 && pthread_create(&th[t], NULL, o_job_main, &jobs[t]) == 0;
    }
    for (int t = 0; t < threads; ++t)
        if (!started[t]) o_job_main(&jobs[t]);
    for (int t = 1; t < threads; ++t)
        if (started[t]) pthread_join(th[t], NULL);
}

/* ---- neighbour lists (compressed rows): the neighbours of particle i, itself included, are
 * idx[off[i] .. off[i+1]), ascending; a neighbour is every j with r2 < support2, r2
 * computed as the forward and backward loops compute it. */
typedef struct {
    int *off;
    int *idx;
} ONbr;

static double o_r2(const OState *a, const OState *b) {
    const double dx = a->x[0] - b->x[0], dy = a->x[1] - b->x[1], dz = a->x[2] - b->x[2];
    return dx * dx + dy * dy + dz * dz;
}

static void nbr_free(ONbr *nb) {
    free(nb->off);
    free(nb->idx);
    nb->off = nb->idx = NULL;
}

typedef struct {
    int n;
    const OState *in;
    double support2;
    int dim[3];
    double lo[3], inv[3];
    const int *cell_of, *start, *order;
    int *count;                      /* [n] neighbours of each particle */
    int *part_idx[O_MAX_THREADS];    /* each thread's lists, its particles in order */
    size_t part_len[O_MAX_THREADS];
    int failed;
} ONbrBuild;

/* One thread's particles: scans the 3 x 3 x 3 cells around each particle's own, marks its
 * neighbours in a bitmap over particle indices and reads the bitmap back in ascending
 * order. */
static void nbr_range(void *varg, int lo, int hi, int thread) {
    ONbrBuild *B = (ONbrBuild *)varg;
    const int n = B->n;
    const size_t words = ((size_t)n + 63) / 64;
    unsigned long long *bits = (unsigned long long *)calloc(words, sizeof(unsigned long long));
    size_t cap = (size_t)(hi - lo) * 64 + 64, len = 0;
    int *out = (int *)malloc(sizeof(int) * cap);
    B->part_idx[thread] = NULL;
    B->part_len[thread] = 0;
    if (!bits || !out) {
        free(bits);
        free(out);
        B->failed = 1;
        return;
    }
    for (int i = lo; i < hi; ++i) {
        const int c = B->cell_of[i];
        const int cx = c % B->dim[0], cy = (c / B->dim[0]) % B->dim[1], cz = c / (B->dim[0] * B->dim[1]);
        int jlo = n, jhi = -1;
        for (int z = cz - 1; z <= cz + 1; ++z)
            for (int y = cy - 1; y <= cy + 1; ++y)
                for (int x = cx - 1; x <= cx + 1; ++x) {
                    if (x < 0 || y < 0 || z < 0 || x >= B->dim[0] || y >= B->dim[1] || z >= B->dim[2]) continue;
                    const int cc = (z * B->dim[1] + y) * B->dim[0] + x;
                    for (int t = B->start[cc]; t < B->start[cc + 1]; ++t) {
                        const int j = B->order[t];
                        if (o_r2(&B->in[i], &B->in[j]) < B->support2) {
                            bits[j >> 6] |= 1ull << (j & 63);
                            if (j < jlo) jlo = j;
                            if (j > jhi) jhi = j;
                        }
                    }
                }
        const size_t first = len;
        for (int w = jlo >> 6; jhi >= 0 && w <= (jhi >> 6); ++w) {
            unsigned long long m = bits[w];
            bits[w] = 0;
            while (m) {
                const int b = __builtin_ctzll(m);
                m &= m - 1;
                if (len == cap) {
                    int *grown = (int *)realloc(out, sizeof(int) * cap * 2);
                    if (!grown) {
                        free(bits);
                        free(out);
                        B->failed = 1;
                        return;
                    }
                    out = grown;
                    cap *= 2;
                }
                out[len++] = (w << 6) + b;
            }
        }
        B->count[i] = (int)(len - first);
    }
    free(bits);
    B->part_idx[thread] = out;
    B->part_len[thread] = len;
}

/* Builds the lists with a grid of cells of edge >= sqrt(support2). */
static int nbr_build(int n, const OState *in, double support2, int threads, ONbr *nb) {
    ONbrBuild B;
    memset(&B, 0, sizeof(B));
    B.n = n;
    B.in = in;
    B.support2 = support2;
    const double cs = sqrt(support2);
    double hi[3];
    long long cells = 1;
    for (int k = 0; k < 3; ++k) {
        B.lo[k] = hi[k] = in[0].x[k];
        for (int i = 1; i < n; ++i) {
            if (in[i].x[k] < B.lo[k]) B.lo[k] = in[i].x[k];
            if (in[i].x[k] > hi[k]) hi[k] = in[i].x[k];
        }
        const double e = (hi[k] - B.lo[k]) / cs;
        B.dim[k] = e < 1.0 ? 1 : (e > 1024.0 ? 1024 : (int)e + 1);
        cells *= B.dim[k];
        /* cells of edge max((hi - lo) / dim, cs): never smaller than the support */
        double edge = (hi[k] - B.lo[k]) / B.dim[k];
        if (edge < cs) edge = cs;
        B.inv[k] = 1.0 / edge;
    }
    int *cell_of = (int *)malloc(sizeof(int) * (size_t)n);
    int *start = (int *)calloc((size_t)cells + 1, sizeof(int));
    int *order = (int *)malloc(sizeof(int) * (size_t)n);
    int *fill = (int *)malloc(sizeof(int) * (size_t)cells);
    nb->off = (int *)malloc(sizeof(int) * ((size_t)n + 1));
    nb->idx = NULL;
    B.count = (int *)malloc(sizeof(int) * (size_t)n);
    int ok = cell_of && start && order && fill && nb->off && B.count;
    if (ok) {
        for (int i = 0; i < n; ++i) {
            int c[3];
            for (int k = 0; k < 3; ++k) {
                int v = (int)((in[i].x[k] - B.lo[k]) * B.inv[k]);
                c[k] = v < 0 ? 0 : (v >= B.dim[k] ? B.dim[k] - 1 : v);
            }
            cell_of[i] = (c[2] * B.dim[1] + c[1]) * B.dim[0] + c[0];
            start[cell_of[i] + 1]++;
        }
        for (long long c = 0; c < cells; ++c) start[c + 1] += start[c];
        memcpy(fill, start, sizeof(int) * (size_t)cells);
        for (int i = 0; i < n; ++i) order[fill[cell_of[i]]++] = i;
        B.cell_of = cell_of;
        B.start = start;
        B.order = order;
        o_parallel(n, threads, nbr_range, &B);
        ok = !B.failed;
    }
    if (ok) {
        size_t total = 0;
        for (int t = 0; t < threads; ++t) total += B.part_len[t];
        nb->idx = (int *)malloc(sizeof(int) * (total > 0 ? total : 1));
        ok = nb->idx != NULL;
        if (ok) {
            size_t at = 0;
            for (int t = 0; t < threads; ++t) {
                if (B.part_len[t]) memcpy(nb->idx + at, B.part_idx[t], sizeof(int) * B.part_len[t]);
                at += B.part_len[t];
            }
            int o = 0;
            for (int i = 0; i < n; ++i) {
                nb->off[i] = o;
                o += B.count[i];
            }
            nb->off[n] = o;
        }
    }
    for (int t = 0; t < threads; ++t) free(B.part_idx[t]);
    free(B.count);
    free(cell_of);
    free(start);
    free(order);
    free(fill);
    if (!ok) nbr_free(nb);
    return ok;
}

static double o_d2w(double q, double sigma, double inv_h) {
    double s2 = sigma * inv_h * inv_h;
    if (q < 1.0) return s2 * (-3.0 + 4.5 * q);
    if (q < 2.0) return s2 * (1.5 * (2.0 - q));
    return 0.0;
}

/* ---- forward step */

typedef struct {
    const OState *in;
    OState *out;
    double *rho, *P, *a;
    const OSphContext *c;
    const ONbr *nb;
} OFwd;

static void fwd_density(void *varg, int lo, int hi, int thread) {
    const OFwd *F = (const OFwd *)varg;
    const OState *in = F->in;
    const OSphContext *c = F->c;
    (void)thread;
    for (int i = lo; i < hi; ++i) {
        double r = 0.0;
        for (int t = F->nb->off[i]; t < F->nb->off[i + 1]; ++t) {
            const int j = F->nb->idx[t];
            double dx = in[i].x[0] - in[j].x[0], dy = in[i].x[1] - in[j].x[1], dz = in[i].x[2] - in[j].x[2];
            double r2 = dx * dx + dy * dy + dz * dz;
            if (r2 < c->support2) r += c->m * o_sph_w(sqrt(r2) * c->inv_h, c->sigma);
        }
        F->rho[i] = r;
        double xr = r / c->rho0;
        F->P[i] = c->B * (pow(xr, 7.0) - 1.0);
    }
}

static void fwd_force(void *varg, int lo, int hi, int thread) {
    const OFwd *F = (const OFwd *)varg;
    const OState *in = F->in;
    const OSphContext *c = F->c;
    const double *rho = F->rho, *P = F->P;
    (void)thread;
    for (int i = lo; i < hi; ++i) {
        double acc[3] = {0, 0, 0};
        for (int t = F->nb->off[i]; t < F->nb->off[i + 1]; ++t) {
            const int j = F->nb->idx[t];
            if (j == i) continue;
            double d[3] = {in[i].x[0] - in[j].x[0], in[i].x[1] - in[j].x[1], in[i].x[2] - in[j].x[2]};
            double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
            if (!(r2 < c->support2 && r2 > 0.0)) continue;
            double r = sqrt(r2);
            double dw = o_sph_dw(r * c->inv_h, c->sigma, c->inv_h);
            double vr = 0.0;
            for (int k = 0; k < 3; ++k) vr += (in[i].v[k] - in[j].v[k]) * d[k];
            double visc = 0.0;
            if (vr < 0.0) visc = -(c->alpha * c->c0 * (c->h * vr / (r2 + c->eta2))) / (0.5 * (rho[i] + rho[j]));
            double coef = -c->m * (P[i] / (rho[i] * rho[i]) + P[j] / (rho[j] * rho[j]) + visc) * (dw / r);
            for (int k = 0; k < 3; ++k) acc[k] += coef * d[k];
        }
        for (int k = 0; k < 3; ++k) {
            F->a[3 * i + k] = acc[k];
            double u = in[i].v[k] + c->dt * (acc[k] + c->g[k]);
            double y = in[i].x[k] + c->dt * u;
            if (y < c->min[k]) {
                y = c->min[k];
                u = -0.5 * u;
            }
            else if (y > c->max[k]) {
                y = c->max[k];
                u = -0.5 * u;
            }
            F->out[i].x[k] = y;
            F->out[i].v[k] = u;
        }
    }
}

/* One forward step from (x, v); fills rho, P, a of the step and the new state. */
static void forward_step(int n, int threads, const OState *in, OState *out, double *rho, double *P, double *a,
                         const OSphContext *c, const ONbr *nb) {
    OFwd F = {in, out, rho, P, a, c, nb};
    o_parallel(n, threads, fwd_density, &F);
    o_parallel(n, threads, fwd_force, &F);
}

/* ---- backward step */

typedef struct {
    const OState *in;
    const double *rho, *P, *a;
    const OSphContext *c;
    const ONbr *nb;
    const double *xb, *vb;
    double *abar, *rhob, *Pb, *nx, *nv, *th; /* th: per particle, its share of the 2 theta sums */
} OBwd;

static void bwd_integrate(void *varg, int lo, int hi, int thread) {
    const OBwd *W = (const OBwd *)varg;
    const OSphContext *c = W->c;
    (void)thread;
    for (int i = lo; i < hi; ++i)
        for (int k = 0; k < 3; ++k) {
            double u = W->in[i].v[k] + c->dt * (W->a[3 * i + k] + c->g[k]);
            double y = W->in[i].x[k] + c->dt * u;
            int clamped = (y < c->min[k]) || (y > c->max[k]);
            double ybar = clamped ? 0.0 : W->xb[3 * i + k];
            double ubar = clamped ? -0.5 * W->vb[3 * i + k] : W->vb[3 * i + k];
            ubar += c->dt * ybar;
            W->nx[3 * i + k] = ybar;
            W->nv[3 * i + k] = ubar;
            W->abar[3 * i + k] = c->dt * ubar;
        }
}

static void bwd_force(void *varg, int lo, int hi, int thread) {
    const OBwd *W = (const OBwd *)varg;
    const OState *in = W->in;
    const OSphContext *c = W->c;
    const double *rho = W->rho, *P = W->P, *abar = W->abar;
    (void)thread;
    for (int k = lo; k < hi; ++k) {
        double th0 = 0.0, th1 = 0.0;
        for (int t = W->nb->off[k]; t < W->nb->off[k + 1]; ++t) {
            const int j = W->nb->idx[t];
            if (j == k) continue;
            double d[3], vkj[3], w[3];
            for (int q = 0; q < 3; ++q) {
                d[q] = in[k].x[q] - in[j].x[q];
                vkj[q] = in[k].v[q] - in[j].v[q];
                w[q] = abar[3 * k + q] - abar[3 * j + q];
            }
            double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
            if (!(r2 < c->support2 && r2 > 0.0)) continue;
            double r = sqrt(r2), q = r * c->inv_h;
            double dw = o_sph_dw(q, c->sigma, c->inv_h), d2w = o_d2w(q, c->sigma, c->inv_h);
            double D = dw / r, Dp = (d2w * r - dw) / r2;
            double s = vkj[0] * d[0] + vkj[1] * d[1] + vkj[2] * d[2];
            double rb = 0.5 * (rho[k] + rho[j]), den = r2 + c->eta2;
            double Pi = 0, Pi_s = 0, Pi_r2 = 0, Pi_rb = 0, Pi_al = 0, Pi_c0 = 0;
            if (s < 0.0) {
                double k0 = c->h / (den * rb);
                Pi_al = -c->c0 * k0 * s;
                Pi_c0 = -c->alpha * k0 * s;
                Pi = c->alpha * Pi_al;
                Pi_s = -c->alpha * c->c0 * k0;
                Pi_r2 = -Pi / den;
                Pi_rb = -Pi / rb;
            }
            double T = P[k] / (rho[k] * rho[k]) + P[j] / (rho[j] * rho[j]) + Pi;
            double cc = -c->m * T * D;
            double xw = d[0] * w[0] + d[1] * w[1] + d[2] * w[2];
            double coef_d = -c->m * (2.0 * Pi_r2 * D + T * Dp / r), coef_v = -c->m * D * Pi_s;
            for (int u = 0; u < 3; ++u) {
                W->nx[3 * k + u] += cc * w[u] + xw * (coef_v * vkj[u] + coef_d * d[u]);
                W->nv[3 * k + u] += xw * coef_v * d[u];
            }
            W->rhob[k] += xw * (-c->m * D) * (-2.0 * P[k] / (rho[k] * rho[k] * rho[k]) + 0.5 * Pi_rb);
            W->Pb[k] += xw * (-c->m * D / (rho[k] * rho[k]));
            double ad = abar[3 * k] * d[0] + abar[3 * k + 1] * d[1] + abar[3 * k + 2] * d[2];
            th0 += ad * (-c->m * D * Pi_al);
            th1 += ad * (-c->m * D * Pi_c0);
        }
        double xr = rho[k] / c->rho0;
        W->rhob[k] += W->Pb[k] * c->B * 7.0 * pow(xr, 6.0) / c->rho0;
        th1 += W->Pb[k] * 2.0 * P[k] / c->c0;
        W->th[2 * k] = th0;
        W->th[2 * k + 1] = th1;
    }
}

static void bwd_density(void *varg, int lo, int hi, int thread) {
    const OBwd *W = (const OBwd *)varg;
    const OState *in = W->in;
    const OSphContext *c = W->c;
    (void)thread;
    for (int k = lo; k < hi; ++k)
        for (int t = W->nb->off[k]; t < W->nb->off[k + 1]; ++t) {
            const int j = W->nb->idx[t];
            if (j == k) continue;
            double d[3] = {in[k].x[0] - in[j].x[0], in[k].x[1] - in[j].x[1], in[k].x[2] - in[j].x[2]};
            double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
            if (!(r2 < c->support2 && r2 > 0.0)) continue;
            double r = sqrt(r2);
            double g = (W->rhob[k] + W->rhob[j]) * c->m * o_sph_dw(r * c->inv_h, c->sigma, c->inv_h) / r;
            for (int u = 0; u < 3; ++u) W->nx[3 * k + u] += g * d[u];
        }
}

static int backward_step(int n, int threads, const OState *in, const double *rho, const double *P, const double *a,
                         const OSphContext *c, const ONbr *nb, double *xb, double *vb, double *theta) {
    OBwd W;
    W.in = in;
    W.rho = rho;
    W.P = P;
    W.a = a;
    W.c = c;
    W.nb = nb;
    W.xb = xb;
    W.vb = vb;
    W.abar = (double *)calloc((size_t)n * 3, sizeof(double));
    W.rhob = (double *)calloc((size_t)n, sizeof(double));
    W.Pb = (double *)calloc((size_t)n, sizeof(double));
    W.nx = (double *)calloc((size_t)n * 3, sizeof(double));
    W.nv = (double *)calloc((size_t)n * 3, sizeof(double));
    W.th = (double *)calloc((size_t)n * 2, sizeof(double));
    int ok = W.abar && W.rhob && W.Pb && W.nx && W.nv && W.th;
    if (ok) {
        o_parallel(n, threads, bwd_integrate, &W);
        o_parallel(n, threads, bwd_force, &W);
        o_parallel(n, threads, bwd_density, &W);
        for (int k = 0; k < n; ++k) {
            theta[0] += W.th[2 * k];
            theta[1] += W.th[2 * k + 1];
        }
        memcpy(xb, W.nx, sizeof(double) * 3 * (size_t)n);
        memcpy(vb, W.nv, sizeof(double) * 3 * (size_t)n);
    }
    free(W.abar);
    free(W.rhob);
    free(W.Pb);
    free(W.nx);
    free(W.nv);
    free(W.th);
    return ok;
}

/* x0, v0, dl_dx, dl_dv, dx0, dv0, x_final, v_final: n * 3 doubles (by particle);
 * ctx: an OSphContext of doubles; theta: 2 doubles (dL/dalpha, dL/dc0).  With dx0 NULL
 * only the forward rollout runs (x_final, v_final).  Returns steps, or 0 on failure. */
int oracle_sph_adjoint_f64(int n, const double *x0, const double *v0, const void *vctx, int steps,
                           const double *dl_dx, const double *dl_dv, double *dx0, double *dv0, double *theta,
                           double *x_final, double *v_final) {
    const OSphContext *c = (const OSphContext *)vctx;
    if (n <= 0 || steps <= 0) return 0;
    const int threads = o_threads(n);
    OState *states = (OState *)calloc((size_t)n * (size_t)(steps + 1), sizeof(OState));
    double *rho = (double *)calloc((size_t)n * (size_t)steps, sizeof(double));
    double *P = (double *)calloc((size_t)n * (size_t)steps, sizeof(double));
    double *a = (double *)calloc((size_t)n * 3 * (size_t)steps, sizeof(double));
    double *xb = (double *)calloc((size_t)n * 3, sizeof(double));
    double *vb = (double *)calloc((size_t)n * 3, sizeof(double));
    int ok = states && rho && P && a && xb && vb;
    for (int i = 0; i < n && ok; ++i)
        for (int k = 0; k < 3; ++k) {
            states[i].x[k] = x0[3 * i + k];
            states[i].v[k] = v0[3 * i + k];
        }
    for (int s = 0; s < steps && ok; ++s) {
        ONbr nb = {NULL, NULL};
        ok = nbr_build(n, states + (size_t)s * n, c->support2, threads, &nb);
        if (ok)
            forward_step(n, threads, states + (size_t)s * n, states + (size_t)(s + 1) * n, rho + (size_t)s * n,
                         P + (size_t)s * n, a + (size_t)s * n * 3, c, &nb);
        nbr_free(&nb);
    }
    const OState *fin = ok ? states + (size_t)steps * n : NULL;
    for (int i = 0; i < n && ok; ++i)
        for (int k = 0; k < 3; ++k) {
            if (x_final) x_final[3 * i + k] = fin[i].x[k];
            if (v_final) v_final[3 * i + k] = fin[i].v[k];
        }
    if (ok && dx0) {
        for (int i = 0; i < 3 * n; ++i) {
            xb[i] = dl_dx ? dl_dx[i] : 0.0;
            vb[i] = dl_dv ? dl_dv[i] : 0.0;
        }
        theta[0] = theta[1] = 0.0;
        for (int s = steps - 1; s >= 0 && ok; --s) {
            ONbr nb = {NULL, NULL};
            ok = nbr_build(n, states + (size_t)s * n, c->support2, threads, &nb);
            if (ok)
                ok = backward_step(n, threads, states + (size_t)s * n, rho + (size_t)s * n, P + (size_t)s * n,
                                   a + (size_t)s * n * 3, c, &nb, xb, vb, theta);
            nbr_free(&nb);
        }
        if (ok) {
            memcpy(dx0, xb, sizeof(double) * 3 * (size_t)n);
            memcpy(dv0, vb, sizeof(double) * 3 * (size_t)n);
        }
    }
    free(states);
    free(rho);
    free(P);
    free(a);
    free(xb);
    free(vb);
    return ok ? steps : 0;
}
