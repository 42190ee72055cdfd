/*
 * psim_tangent.c -- FP64 forward-mode tangent of the differentiable
 * trajectory's loss.
 *
 * TEST INFRASTRUCTURE ONLY: the checker of the GPU adjoint (psim_adjoint_*),
 * from the other direction.  The trajectory is the positions form of the
 * vGB steps (brownianIntegrator.cpp:191-296, as firstStep then normal
 * steps) with the given noise, under the pair force of the AO plugin
 * (AOPotential.cpp:50-130), the LennardJones plugin's Yukawa term with
 * ljNum = 0 and its LJ(n) term (LJPotential.cpp:96-109), each inside its own
 * cutoff.  The loss is the squared distance between the time-averaged,
 * Gaussian-smoothed g(r) and a target.  Six tangents -- one per parameter
 * (the AO coefficients c1 and c2, the Yukawa amplitude and length, the LJ
 * energy and contact diameter) -- are carried through every step:
 *
 *   x'_1     = c_f F'(x_0)
 *   x'_{t+1} = c0 x'_t - a0 x'_{t-1} + b1 F'_t - b2 F'_{t-1},
 *   F'_t     = J(x_t) x'_t + dF/dth (x_t),
 *
 * and dL/dth follows from the tangents of the sampled pair distances.  The
 * pair sums are brute force over all pairs (minimum image), in FP64.
 */
#include "psim_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define NTH 6

typedef struct {
    double c1, c2, ao_rc2;
    double Y, lam, y_rc2;
    double eps, sig, lj_rc2;
    int ljn;
} tpair;

/* s(r) = fNet / r along x_j - x_i, ds/dr and ds/dth (th = c1, c2, Y, lambda,
 * eps, sigma) */
static void pair_s(const tpair* q, double r2, double* s, double* ds, double dth[NTH]) {
    const double r = sqrt(r2), ri = 1.0 / r, ri2 = ri * ri, ri3 = ri2 * ri;
    *s = 0.0;
    *ds = 0.0;
    for (int k = 0; k < NTH; k++) dth[k] = 0.0;
    if (r2 < q->ao_rc2) {   /* fNet = -(36 r^-38 + c1 / r + c2 r) */
        const double ri39 = pow(ri, 39.0);
        *s += -(36.0 * ri39 + q->c1 * ri2 + q->c2);
        *ds += 36.0 * 39.0 * ri39 * ri + 2.0 * q->c1 * ri3;
        dth[0] = -ri2;
        dth[1] = -1.0;
    }
    if (r2 < q->y_rc2) {    /* fNet = -Y e^{-r/lambda} (lambda + r) / r^2 */
        const double e = exp(-r / q->lam), lr = q->lam + r;
        *s += -q->Y * e * lr * ri3;
        *ds += q->Y * e * ri3 * (r / q->lam + 3.0 * lr * ri);
        dth[2] = -e * lr * ri3;
        dth[3] = -q->Y * e * ri3 * (r * lr / (q->lam * q->lam) + 1.0);
    }
    if (r2 < q->lj_rc2) {   /* fNet = -eps (2L - 1) 4n L / r, L = (sigma / r)^n */
        const double n = (double)q->ljn, L = pow(q->sig * ri, n);
        const double base = -4.0 * n * (2.0 * L - 1.0) * L * ri2;
        *s += q->eps * base;
        *ds += 4.0 * n * q->eps * L * (n * (4.0 * L - 1.0) + 2.0 * (2.0 * L - 1.0)) * ri3;
        dth[4] = base;
        dth[5] = -4.0 * n * n * q->eps * (4.0 * L - 1.0) * L * ri2 / q->sig;
    }
}

static double wrap_box(double x, double L) { return x - L * floor(x / L); }

static double min_image(double d, double L) {
    const double h = 0.5 * L;
    return d > h ? d - L : (d < -h ? d + L : d);
}

/* forces F (3n, AoS) at x and the tangents dF[k] of the forces for the
 * position tangents dx[k] */
static void forces(int n, double L, const tpair* q, double rc2, const double* x,
                   double* const dx[NTH], double* F, double* const dF[NTH]) {
    memset(F, 0, sizeof(double) * 3 * (size_t)n);
    for (int k = 0; k < NTH; k++) memset(dF[k], 0, sizeof(double) * 3 * (size_t)n);
    for (int i = 0; i < n; i++) {
        const double xi[3] = {wrap_box(x[3 * i], L), wrap_box(x[3 * i + 1], L),
                              wrap_box(x[3 * i + 2], L)};
        for (int j = i + 1; j < n; j++) {
            double d[3];
            for (int a = 0; a < 3; a++) d[a] = min_image(wrap_box(x[3 * j + a], L) - xi[a], L);
            const double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
            if (!(r2 < rc2)) continue;
            double s, ds, dth[NTH];
            pair_s(q, r2, &s, &ds, dth);
            const double c = ds / sqrt(r2);
            for (int a = 0; a < 3; a++) {
                F[3 * i + a] += s * d[a];
                F[3 * j + a] -= s * d[a];
            }
            for (int k = 0; k < NTH; k++) {
                double dd[3], ddd = 0.0;
                for (int a = 0; a < 3; a++) {
                    dd[a] = dx[k][3 * j + a] - dx[k][3 * i + a];
                    ddd += d[a] * dd[a];
                }
                for (int a = 0; a < 3; a++) {
                    const double t = s * dd[a] + c * d[a] * ddd + dth[k] * d[a];
                    dF[k][3 * i + a] += t;
                    dF[k][3 * j + a] -= t;
                }
            }
        }
    }
}

/* the smoothed pair counts h (n_bins) of x and their tangents dh[k] */
static void hist(int n, double L, const double* x, double* const dx[NTH], double r_min,
                 double dr, int n_bins, double sigma, double* h, double* dh) {
    const double reach_r = (r_min + dr * n_bins) + 4.0 * sigma, rw2 = reach_r * reach_r;
    const int reach = (int)ceil(4.0 * sigma / dr) + 1;
    const double norm = 1.0 / (sqrt(2.0 * M_PI) * sigma);
    for (int i = 0; i < n; i++)
        for (int j = i + 1; j < n; j++) {
            double d[3];
            for (int a = 0; a < 3; a++)
                d[a] = min_image(wrap_box(x[3 * j + a], L) - wrap_box(x[3 * i + a], L), L);
            const double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
            if (!(r2 < rw2)) continue;
            const double r = sqrt(r2);
            double rdot[NTH];
            for (int k = 0; k < NTH; k++) {
                double t = 0.0;
                for (int a = 0; a < 3; a++) t += d[a] * (dx[k][3 * j + a] - dx[k][3 * i + a]);
                rdot[k] = t / r;
            }
            const int b0 = (int)floor((r - r_min) / dr);
            const int lo = b0 - reach < 0 ? 0 : b0 - reach;
            const int hi = b0 + reach > n_bins - 1 ? n_bins - 1 : b0 + reach;
            for (int b = lo; b <= hi; b++) {
                const double z = (r - (r_min + (b + 0.5) * dr)) / sigma;
                const double G = norm * exp(-0.5 * z * z);
                h[b] += 2.0 * dr * G;   /* the ordered pairs (i, j) and (j, i) */
                for (int k = 0; k < NTH; k++)
                    dh[(size_t)k * n_bins + b] += 2.0 * dr * G * (-z / sigma) * rdot[k];
            }
        }
}

/* AO coefficients (AOPotential.cpp:50-55) and their derivatives in wellDepth
 * and the range rc */
static void ao_d(double kT, double wd, double rc, double c[2], double dwd[2], double drc[2]) {
    const double q = rc / (rc - 1.0);
    const double a1 = -kT * wd * q * q * q, a2 = -3.0 / (2.0 * rc), a3 = 1.0 / (2.0 * rc * rc * rc);
    c[0] = -a1 * a2;
    c[1] = -3.0 * a1 * a3;
    const double a1_wd = -kT * q * q * q;
    const double a1_rc = 3.0 * kT * wd * rc * rc / pow(rc - 1.0, 4.0);
    const double a2_rc = 3.0 / (2.0 * rc * rc), a3_rc = -3.0 / (2.0 * rc * rc * rc * rc);
    dwd[0] = -a1_wd * a2;
    dwd[1] = -3.0 * a1_wd * a3;
    drc[0] = -(a1_rc * a2 + a1 * a2_rc);
    drc[1] = -3.0 * (a1_rc * a3 + a1 * a3_rc);
}

int oracle_adjoint_tangent(int n, double box, const oracle_adj_params* p, const oracle_vgb* c,
                           double dt, double mass, int n_steps, int sample_every, double r_min,
                           double r_max, int n_bins, double sigma, const double* pos0,
                           const double* vel0, const double* noise, const double* g_target,
                           double* loss, double* g_mean, double* grad) {
    tpair q;
    memset(&q, 0, sizeof q);
    double cc[2] = {0.0, 0.0}, dwd[2] = {0.0, 0.0}, drc[2] = {0.0, 0.0};
    if (p->ao_cutoff > 0.0) {
        ao_d(p->kT, p->ao_well_depth, p->ao_range > 0.0 ? p->ao_range : p->ao_cutoff, cc, dwd, drc);
        q.c1 = cc[0];
        q.c2 = cc[1];
        q.ao_rc2 = p->ao_cutoff * p->ao_cutoff;
    }
    if (p->yuk_cutoff > 0.0) {
        q.Y = p->yuk_amplitude;
        q.lam = p->yuk_length;
        q.y_rc2 = p->yuk_cutoff * p->yuk_cutoff;
    }
    if (p->lj_cutoff > 0.0) {
        q.eps = p->lj_epsilon;
        q.sig = p->lj_sigma;
        q.ljn = p->lj_n;
        q.lj_rc2 = p->lj_cutoff * p->lj_cutoff;
    }
    double rc2 = q.ao_rc2;
    if (q.y_rc2 > rc2) rc2 = q.y_rc2;
    if (q.lj_rc2 > rc2) rc2 = q.lj_rc2;
    /* the vGB positions update (the GPU adjoint's own coefficients) */
    const double m = 1.0 / mass, dt2 = dt * dt;
    const double c0 = 1.0 + c->coeff0, a0 = c->coeff0;
    const double b1 = m * dt2 * (c->coeff1 + c->coeff2), b2 = m * dt2 * c->coeff2;
    const double cv = c->coeff1 * dt, cf = c->coeff3 * dt2 * m;
    const size_t N3 = 3 * (size_t)n;
    const double dr = (r_max - r_min) / n_bins;
    /* buffers: x_{t-1}, x_t, F_{t-1}, F_t and their NTH tangents, noise memory */
    double* buf = (double*)calloc(N3 * 4 * (NTH + 1) + N3, sizeof(double));
    double* h = (double*)calloc((size_t)n_bins * (NTH + 1), sizeof(double));
    if (!buf || !h) {
        free(buf);
        free(h);
        return 7706;
    }
    double *xp = buf, *x = buf + N3, *Fp = buf + 2 * N3, *F = buf + 3 * N3;
    double *dxp[NTH], *dx[NTH], *dFp[NTH], *dF[NTH];
    for (int k = 0; k < NTH; k++) {
        double* b = buf + 4 * N3 * (size_t)(k + 1);
        dxp[k] = b;
        dx[k] = b + N3;
        dFp[k] = b + 2 * N3;
        dF[k] = b + 3 * N3;
    }
    double* mem = buf + 4 * N3 * (NTH + 1);
    double* dh = h + n_bins;
    memcpy(x, pos0, sizeof(double) * N3);
    int samples = 0;
    for (int t = 0; t <= n_steps; t++) {
        if (t > 0 && t % sample_every == 0) {
            hist(n, box, x, dx, r_min, dr, n_bins, sigma, h, dh);
            samples++;
        }
        if (t == n_steps) break;
        forces(n, box, &q, rc2, x, dx, F, dF);
        const double* xi = noise + (size_t)t * (size_t)n * 6;
        for (int i = 0; i < n; i++)
            for (int a = 0; a < 3; a++) {
                const size_t o = 3 * (size_t)i + a;
                double xn;
                if (t == 0) {   /* firstStep */
                    mem[o] = xi[6 * (size_t)i + a];
                    xn = x[o] + cv * (vel0 ? vel0[o] : 0.0) + cf * F[o] + c->sig1 * xi[6 * (size_t)i + a];
                    for (int k = 0; k < NTH; k++) dxp[k][o] = cf * dF[k][o];   /* x'_1 */
                } else {
                    const double mc = c->sig2 * (c->corr * mem[o] + c->dev * xi[6 * (size_t)i + a]);
                    mem[o] = xi[6 * (size_t)i + 3 + a];
                    xn = c0 * x[o] - a0 * xp[o] + b1 * F[o] - b2 * Fp[o] +
                         c->sig1 * xi[6 * (size_t)i + 3 + a] + c->coeff0 * mc;
                    for (int k = 0; k < NTH; k++)
                        dxp[k][o] = c0 * dx[k][o] - a0 * dxp[k][o] + b1 * dF[k][o] - b2 * dFp[k][o];
                }
                xp[o] = x[o];
                x[o] = xn;
            }
        /* dxp now holds x'_{t+1}: it becomes the current tangent, x'_t the previous */
        for (int k = 0; k < NTH; k++) {
            double* tmp = dx[k];
            dx[k] = dxp[k];
            dxp[k] = tmp;
            tmp = dF[k];
            dF[k] = dFp[k];
            dFp[k] = tmp;
        }
        {
            double* tmp = F;
            F = Fp;
            Fp = tmp;
        }
    }
    /* g(r), the loss and its derivatives */
    const double rho = n / (box * box * box);
    double th[NTH] = {0, 0, 0, 0, 0, 0}, L2 = 0.0;
    for (int b = 0; b < n_bins; b++) {
        const double rb = r_min + (b + 0.5) * dr;
        const double Cb = n * rho * 4.0 * M_PI * rb * rb * dr;
        const double g = h[b] / (samples * Cb);
        if (g_mean) g_mean[b] = g;
        const double diff = g - g_target[b];
        L2 += diff * diff;
        for (int k = 0; k < NTH; k++) th[k] += 2.0 * diff * dh[(size_t)k * n_bins + b] / (samples * Cb);
    }
    *loss = L2;
    grad[0] = th[0] * dwd[0] + th[1] * dwd[1];
    grad[1] = th[0] * drc[0] + th[1] * drc[1];
    grad[2] = th[2];
    grad[3] = th[3];
    grad[4] = th[4];
    grad[5] = th[5];
    free(buf);
    free(h);
    return 0;
}
