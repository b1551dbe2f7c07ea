/* ORACLE (test infrastructure, not the product): FP64 CPU adjoint of the SPH rollout.
 *
 * The forward step is the oracle SPH model (oracle/oracle_models.h: o_sph_density,
 * o_sph_pressure, o_sph_force, o_sph_integrate, compiled here with REAL=double), over all
 * pairs within the support instead of a grid (the pair set is the same).  The backward
 * sweep is the reverse mode of that step with the neighbour sets held fixed, written
 * independently of the CUDA adjoint:
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
#include <stdlib.h>
#include <string.h>

#define REAL double
#include "oracle_models.h"

typedef struct {
    double x[3], v[3];
} OState;

static double o_d2w(double q, double sigma, double inv_h) {
    double s2 = sigma * inv_h * inv_h;
    if (q < 1.0) return s2 * (-3.0 + 4.5 * q);
    if (q < 2.0) return s2 * (1.5 * (2.0 - q));
    return 0.0;
}

/* One forward step from (x, v); fills rho, P, a of the step and the new state. */
static void forward_step(int n, const OState *in, OState *out, double *rho, double *P, double *a, const OSphContext *c) {
    for (int i = 0; i < n; ++i) {
        double r = 0.0;
        for (int j = 0; j < n; ++j) {
            double dx = in[i].x[0] - in[j].x[0], dy = in[i].x[1] - in[j].x[1], dz = in[i].x[2] - in[j].x[2];
            double r2 = dx * dx + dy * dy + dz * dz;
            if (r2 < c->support2) r += c->m * o_sph_w(sqrt(r2) * c->inv_h, c->sigma);
        }
        rho[i] = r;
        double xr = r / c->rho0;
        P[i] = c->B * (pow(xr, 7.0) - 1.0);
    }
    for (int i = 0; i < n; ++i) {
        double acc[3] = {0, 0, 0};
        for (int j = 0; j < n; ++j) {
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
            a[3 * i + k] = acc[k];
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
            out[i].x[k] = y;
            out[i].v[k] = u;
        }
    }
}

static void backward_step(int n, const OState *in, const double *rho, const double *P, const double *a,
                          const OSphContext *c, double *xb, double *vb, double *theta) {
    double *abar = (double *)calloc((size_t)n * 3, sizeof(double));
    double *rhob = (double *)calloc((size_t)n, sizeof(double));
    double *Pb = (double *)calloc((size_t)n, sizeof(double));
    double *nx = (double *)calloc((size_t)n * 3, sizeof(double));
    double *nv = (double *)calloc((size_t)n * 3, sizeof(double));
    /* integrate */
    for (int i = 0; i < n; ++i)
        for (int k = 0; k < 3; ++k) {
            double u = in[i].v[k] + c->dt * (a[3 * i + k] + c->g[k]);
            double y = in[i].x[k] + c->dt * u;
            int clamped = (y < c->min[k]) || (y > c->max[k]);
            double ybar = clamped ? 0.0 : xb[3 * i + k];
            double ubar = clamped ? -0.5 * vb[3 * i + k] : vb[3 * i + k];
            ubar += c->dt * ybar;
            nx[3 * i + k] = ybar;
            nv[3 * i + k] = ubar;
            abar[3 * i + k] = c->dt * ubar;
        }
    /* force + pressure */
    for (int k = 0; k < n; ++k) {
        for (int j = 0; j < n; ++j) {
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
            for (int t = 0; t < 3; ++t) {
                nx[3 * k + t] += cc * w[t] + xw * (coef_v * vkj[t] + coef_d * d[t]);
                nv[3 * k + t] += xw * coef_v * d[t];
            }
            rhob[k] += xw * (-c->m * D) * (-2.0 * P[k] / (rho[k] * rho[k] * rho[k]) + 0.5 * Pi_rb);
            Pb[k] += xw * (-c->m * D / (rho[k] * rho[k]));
            double ad = abar[3 * k] * d[0] + abar[3 * k + 1] * d[1] + abar[3 * k + 2] * d[2];
            theta[0] += ad * (-c->m * D * Pi_al);
            theta[1] += ad * (-c->m * D * Pi_c0);
        }
        double xr = rho[k] / c->rho0;
        rhob[k] += Pb[k] * c->B * 7.0 * pow(xr, 6.0) / c->rho0;
        theta[1] += Pb[k] * 2.0 * P[k] / c->c0;
    }
    /* density */
    for (int k = 0; k < n; ++k)
        for (int j = 0; j < n; ++j) {
            if (j == k) continue;
            double d[3] = {in[k].x[0] - in[j].x[0], in[k].x[1] - in[j].x[1], in[k].x[2] - in[j].x[2]};
            double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
            if (!(r2 < c->support2 && r2 > 0.0)) continue;
            double r = sqrt(r2);
            double g = (rhob[k] + rhob[j]) * c->m * o_sph_dw(r * c->inv_h, c->sigma, c->inv_h) / r;
            for (int t = 0; t < 3; ++t) nx[3 * k + t] += g * d[t];
        }
    memcpy(xb, nx, sizeof(double) * 3 * (size_t)n);
    memcpy(vb, nv, sizeof(double) * 3 * (size_t)n);
    free(abar);
    free(rhob);
    free(Pb);
    free(nx);
    free(nv);
}

/* x0, v0, dl_dx, dl_dv, dx0, dv0, x_final, v_final: n * 3 doubles (by particle);
 * ctx: an OSphContext of doubles; theta: 2 doubles (dL/dalpha, dL/dc0). */
int oracle_sph_adjoint_f64(int n, const double *x0, const double *v0, const void *vctx, int steps,
                           const double *dl_dx, const double *dl_dv, double *dx0, double *dv0, double *theta,
                           double *x_final, double *v_final) {
    const OSphContext *c = (const OSphContext *)vctx;
    if (n <= 0 || steps <= 0) return 0;
    OState *states = (OState *)calloc((size_t)n * (size_t)(steps + 1), sizeof(OState));
    double *rho = (double *)calloc((size_t)n * (size_t)steps, sizeof(double));
    double *P = (double *)calloc((size_t)n * (size_t)steps, sizeof(double));
    double *a = (double *)calloc((size_t)n * 3 * (size_t)steps, sizeof(double));
    for (int i = 0; i < n; ++i)
        for (int k = 0; k < 3; ++k) {
            states[i].x[k] = x0[3 * i + k];
            states[i].v[k] = v0[3 * i + k];
        }
    for (int s = 0; s < steps; ++s)
        forward_step(n, states + (size_t)s * n, states + (size_t)(s + 1) * n, rho + (size_t)s * n, P + (size_t)s * n,
                     a + (size_t)s * n * 3, c);
    const OState *fin = states + (size_t)steps * n;
    for (int i = 0; i < n; ++i)
        for (int k = 0; k < 3; ++k) {
            if (x_final) x_final[3 * i + k] = fin[i].x[k];
            if (v_final) v_final[3 * i + k] = fin[i].v[k];
        }
    double *xb = (double *)calloc((size_t)n * 3, sizeof(double));
    double *vb = (double *)calloc((size_t)n * 3, sizeof(double));
    for (int i = 0; i < 3 * n; ++i) {
        xb[i] = dl_dx ? dl_dx[i] : 0.0;
        vb[i] = dl_dv ? dl_dv[i] : 0.0;
    }
    theta[0] = theta[1] = 0.0;
    for (int s = steps - 1; s >= 0; --s)
        backward_step(n, states + (size_t)s * n, rho + (size_t)s * n, P + (size_t)s * n, a + (size_t)s * n * 3, c, xb,
                      vb, theta);
    memcpy(dx0, xb, sizeof(double) * 3 * (size_t)n);
    memcpy(dv0, vb, sizeof(double) * 3 * (size_t)n);
    free(states);
    free(rho);
    free(P);
    free(a);
    free(xb);
    free(vb);
    return steps;
}
