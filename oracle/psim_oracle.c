/*
 * psim_oracle.c -- CPU restatement of ProteinSim2015's Langevin step.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the GB300 kernels and the "port"
 * CPU baseline.  Nothing in the product library links or calls this file.
 *
 * Every function restates one reference routine (cited file:line, paths
 * relative to the reference project).  Floating-point expressions keep the
 * reference's operand order so that, built with -ffp-contract=off, results
 * are bit-identical to the reference's own x86-64 build (checked by
 * tests/test_oracle_golden.py against the fixtures tests/golden/make_golden.py
 * wrote from the reference rebuilt in oracle/_ref).  The one deliberate change:
 * the reference's unstable __gnu_parallel::sort is replaced by a stable
 * counting sort, i.e. the order inside a cell is by original index.  The
 * reference leaves that order unspecified; cell membership is unchanged.
 */
#include "psim_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define SENTINEL 0xffffffffu

void oracle_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

int oracle_get_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* AOPotential.cpp:50-55 */
void oracle_ao_coeffs(double kT, double wd, double rc, double* c1, double* c2) {
    double q = rc / (rc - 1.0);
    double a1 = -kT * wd * q * q * q;
    double a2 = -3.0 / (2.0 * rc);
    double a3 = 1.0 / (2.0 * rc * rc * rc);
    *c1 = -a1 * a2;
    *c2 = -3.0 * a1 * a3;
}

/* ---------------------------------------------------------------- cells */

static inline int cell_of(double x, double cs) { return (int)floor(x / cs); }

/* systemHandling.cpp:33-48 */
void oracle_hash(const oracle_geom* g, const double* pos, int* hi) {
    const int s = g->scale, s2 = s * s;
    const double cs = g->cell_size;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < g->n; i++) {
        int cx = cell_of(pos[3 * i + 0], cs);
        int cy = cell_of(pos[3 * i + 1], cs);
        int cz = cell_of(pos[3 * i + 2], cs);
        hi[2 * i + 0] = cx + s * cy + s2 * cz;
        hi[2 * i + 1] = i;
    }
}

/* systemHandling.cpp:50-52, as a stable counting sort on the hash. */
void oracle_sort(const oracle_geom* g, int* hi) {
    const int n = g->n;
    const long ncell = (long)g->scale * g->scale * g->scale;
    int* cnt = (int*)calloc((size_t)ncell + 1, sizeof(int));
    int* tmp = (int*)malloc(sizeof(int) * 2 * (size_t)(n > 0 ? n : 1));
    for (int i = 0; i < n; i++) {
        int h = hi[2 * i];
        if (h < 0 || h >= ncell) h = (int)ncell; /* out-of-grid keys sort last */
        cnt[h]++;
    }
    long run = 0;
    for (long c = 0; c <= ncell; c++) { int k = cnt[c]; cnt[c] = (int)run; run += k; }
    for (int i = 0; i < n; i++) {
        int h = hi[2 * i];
        int b = (h < 0 || h >= ncell) ? (int)ncell : h;
        int d = cnt[b]++;
        tmp[2 * d] = h;
        tmp[2 * d + 1] = hi[2 * i + 1];
    }
    memcpy(hi, tmp, sizeof(int) * 2 * (size_t)n);
    free(tmp);
    free(cnt);
}

/* system.h:166 (clearCells) + systemHandling.cpp:54-85 (reorderParticles) */
void oracle_reorder(const oracle_geom* g, const double* pos, const double* radius,
                    const int* hi, uint32_t* cse, double* sorted) {
    const int n = g->n;
    const long ncell = (long)g->scale * g->scale * g->scale;
    for (long c = 0; c < 2 * ncell; c++) cse[c] = SENTINEL;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; i++) {
        int h = hi[2 * i];
        if (i == 0) cse[2 * h] = 0;
        if (i > 0) {
            int hp = hi[2 * (i - 1)];
            if (hp != h) {
                cse[2 * h] = (uint32_t)i;
                cse[2 * hp + 1] = (uint32_t)i;
            }
        }
        if (i == n - 1) cse[2 * h + 1] = (uint32_t)n;
        int idx = hi[2 * i + 1];
        sorted[4 * i + 0] = pos[3 * idx + 0];
        sorted[4 * i + 1] = pos[3 * idx + 1];
        sorted[4 * i + 2] = pos[3 * idx + 2];
        sorted[4 * i + 3] = radius[idx];
    }
}

void oracle_build_cells(const oracle_geom* g, const double* pos, const double* radius,
                        int* hi, uint32_t* cse, double* sorted) {
    oracle_hash(g, pos, hi);
    oracle_sort(g, hi);
    oracle_reorder(g, pos, radius, hi, cse, sorted);
}

/* --------------------------------------------------------------- forces */

/* utilities.cpp:79-104 (pbcDist) */
static inline double pbc_dist2(const double* a, const double* b, double L) {
    double dx = fabs(a[0] - b[0]);
    double dy = fabs(a[1] - b[1]);
    double dz = fabs(a[2] - b[2]);
    double half = L / 2.0;
    if (dx > half) dx -= L;
    if (dy > half) dy -= L;
    if (dz > half) dz -= L;
    return (dx * dx) + (dy * dy) + (dz * dz);
}

/* utilities.cpp:114-142 (unitVectorAdv).  The reference passes L as int, so
 * the image threshold is the integer L/2; for a real-valued box the natural
 * threshold L/2 is used.  Both are inert for in-range pairs (r < L/3). */
static inline void unit_vec(const double* a, const double* b, double r, double L,
                            double half_uv, double u[3]) {
    double d[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
    double one_over = 1.0 / r;
    for (int k = 0; k < 3; k++) {
        if (fabs(d[k]) > half_uv) { if (d[k] < 0) d[k] += L; else d[k] -= L; }
        u[k] = d[k] * one_over;
    }
}

/* utilities.cpp:144-154 (powBinaryDecomp) */
static inline double pow_binary(double base, int e) {
    double ans = 1;
    while (e) {
        if (e & 1) ans *= base;
        e >>= 1;
        base *= base;
    }
    return ans;
}

static inline double uv_half(double L) {
    double fl = floor(L);
    if (fl == L && L < 2147483647.0) return (double)(((int)L) / 2);
    return L / 2.0;
}

enum { PASS_AO = 1, PASS_LJ = 2, PASS_CAL = 3 };

/* Pair magnitude fNet for one in-range pair; the plugin bodies
 * AOPotential.cpp:90-110, LJPotential.cpp:96-109, Calibration.cpp:75-81. */
static inline double pair_fnet(int pass, const oracle_force* f, double r2, double r,
                               double size, int* err, double* terms) {
    if (pass == PASS_AO) {
        double r_inv = 1.0 / r;
        double r_36 = pow(r_inv, 36);
        double r_38 = r_36 / r2;
        double fnet = 36.0 * r_38 + f->ao_c1 * r_inv + f->ao_c2 * r;
        fnet = -fnet;
        if (isnan(fnet) && *err == 0) *err = ORACLE_ERR_NAN;
        *terms = fabs(36.0 * r_38) + fabs(f->ao_c1 * r_inv) + fabs(f->ao_c2 * r);
        return fnet;
    } else if (pass == PASS_LJ) {
        double r_inv = (1.0 / r);
        double yuk_exp = exp(-1.0 * (r * (1.0 / f->debye_length)));
        double lj = pow_binary((size / r), f->lj_num);
        double attract = ((2.0 * lj) - 1.0);
        attract *= (4.0 * f->lj_num * r_inv * lj);
        double repel = yuk_exp;
        repel *= (r_inv * r_inv * (f->debye_length + r) * f->yuk_str);
        *terms = fabs(f->kT * f->well_depth) *
                 (fabs(2.0 * lj * 4.0 * f->lj_num * r_inv * lj) +
                  fabs(4.0 * f->lj_num * r_inv * lj) + fabs(repel));
        return -f->kT * f->well_depth * (attract + repel);
    } else {
        double r_inv = 1.0 / r;
        double r_37 = 36.0 * pow(r_inv, 37);
        *terms = fabs(r_37);
        return -r_37;
    }
}

/* One plugin pass over all particles: defaultForceManager.cpp:55-65 calling
 * <plugin>::getAcceleration (e.g. AOPotential.cpp:132-175), which visits the
 * 27 cells x-outer / y / z-inner and sums per-cell partials (iterCells,
 * AOPotential.cpp:61-130). */
static int force_pass(int pass, const oracle_geom* g, const oracle_force* f, double rc,
                      const double* sorted, const int* hi, const uint32_t* cse,
                      double* out, int accumulate, double* scale_out) {
    const int n = g->n, s = g->scale, s2 = s * s;
    const double L = g->box, cs = g->cell_size, hu = uv_half(L);
    const double rc2 = rc * rc;
    int err_all = 0;
#pragma omp parallel
    {
        int err = 0;
#pragma omp for schedule(dynamic, 256)
        for (int index = 0; index < n; index++) {
            const double* pi = &sorted[4 * index];
            int cx = cell_of(pi[0], cs), cy = cell_of(pi[1], cs), cz = cell_of(pi[2], cs);
            double net[3] = {0.0, 0.0, 0.0};
            double mag = 0.0;
            for (int x = -1; x <= 1; x++)
                for (int y = -1; y <= 1; y++)
                    for (int z = -1; z <= 1; z++) {
                        int rx = (cx + x) % s, ry = (cy + y) % s, rz = (cz + z) % s;
                        rx = rx < 0 ? rx + s : rx;
                        ry = ry < 0 ? ry + s : ry;
                        rz = rz < 0 ? rz + s : rz;
                        int h = rx + s * ry + s2 * rz;
                        double cf[3] = {0.0, 0.0, 0.0};
                        uint32_t start = cse[2 * h];
                        if (start != SENTINEL) {
                            uint32_t end = cse[2 * h + 1];
                            for (uint32_t i = start; i < end; i++) {
                                if ((int)i == index) continue;
                                const double* pj = &sorted[4 * i];
                                double r2 = pbc_dist2(pi, pj, L);
                                if (r2 < rc2) {
                                    double r = sqrt(r2);
                                    double size = pi[3] + pj[3];
                                    if (r < 0.8 * size && err == 0) err = ORACLE_ERR_OVERLAP;
                                    double terms;
                                    double fnet = pair_fnet(pass, f, r2, r, size, &err, &terms);
                                    double u[3];
                                    unit_vec(pi, pj, r, L, hu, u);
                                    cf[0] += fnet * u[0];
                                    cf[1] += fnet * u[1];
                                    cf[2] += fnet * u[2];
                                    mag += terms;
                                }
                            }
                        }
                        net[0] += cf[0];
                        net[1] += cf[1];
                        net[2] += cf[2];
                    }
            int real = 3 * hi[2 * index + 1];
            if (accumulate) {
                out[real] += net[0];
                out[real + 1] += net[1];
                out[real + 2] += net[2];
            } else {
                out[real] = net[0];
                out[real + 1] = net[1];
                out[real + 2] = net[2];
            }
            if (scale_out) scale_out[hi[2 * index + 1]] += mag;
        }
#pragma omp critical
        {
            if (err != 0 && (err_all == 0 || err < err_all)) err_all = err;
        }
    }
    return err_all;
}

int oracle_forces(const oracle_geom* g, const oracle_force* f, const double* sorted,
                  const int* hi, const uint32_t* cse, double* force) {
    switch (f->kind) {
    case ORACLE_AO:
        return force_pass(PASS_AO, g, f, f->cutoff, sorted, hi, cse, force, 0, NULL);
    case ORACLE_LJ:
        return force_pass(PASS_LJ, g, f, f->cutoff, sorted, hi, cse, force, 0, NULL);
    case ORACLE_CAL:
        return force_pass(PASS_CAL, g, f, f->cutoff, sorted, hi, cse, force, 0, NULL);
    case ORACLE_AO_YUK: {
        /* The reference evaluates only flist[0] (defaultForceManager.cpp:56);
         * the composite is the sum of an AO pass and an LJ(n) pass. */
        int e1 = force_pass(PASS_AO, g, f, f->cutoff, sorted, hi, cse, force, 0, NULL);
        int e2 = force_pass(PASS_LJ, g, f, f->cutoff2, sorted, hi, cse, force, 1, NULL);
        return e1 ? e1 : e2;
    }
    }
    return 7706;
}

void oracle_force_scale(const oracle_geom* g, const oracle_force* f, const double* sorted,
                        const int* hi, const uint32_t* cse, double* scale_out) {
    double* tmp = (double*)malloc(sizeof(double) * 3 * (size_t)(g->n > 0 ? g->n : 1));
    memset(scale_out, 0, sizeof(double) * (size_t)g->n);
    switch (f->kind) {
    case ORACLE_AO: force_pass(PASS_AO, g, f, f->cutoff, sorted, hi, cse, tmp, 0, scale_out); break;
    case ORACLE_LJ: force_pass(PASS_LJ, g, f, f->cutoff, sorted, hi, cse, tmp, 0, scale_out); break;
    case ORACLE_CAL: force_pass(PASS_CAL, g, f, f->cutoff, sorted, hi, cse, tmp, 0, scale_out); break;
    case ORACLE_AO_YUK:
        force_pass(PASS_AO, g, f, f->cutoff, sorted, hi, cse, tmp, 0, scale_out);
        force_pass(PASS_LJ, g, f, f->cutoff2, sorted, hi, cse, tmp, 0, scale_out);
        break;
    }
    free(tmp);
}

/* ----------------------------------------------------------- integrator */

/* brownianIntegrator.cpp:27-99 with setupHigh :111-133, setupLow :135-166,
 * setupZero :168-175.  setupLow leaves coEff0 at the setupHigh value. */
void oracle_vgb_coeffs(double gamma, double dt, double kT, oracle_vgb* c) {
    double y = gamma * dt;
    c->y = y;
    {   /* setupHigh */
        double ty = 2.0 * y;
        c->coeff0 = exp(-y);
        double aa1 = 1.0 - c->coeff0;
        double aa2 = 0.5 * y * (1.0 + c->coeff0) - aa1;
        double aa3 = y - aa1;
        c->coeff1 = aa1 / y;
        c->coeff2 = aa2 / (y * y);
        c->coeff3 = aa3 / (y * y);
        c->sig1 = 2.0 * y - 3.0 + 4.0 * exp(-y) - exp(-ty);
        c->sig2 = -2.0 * y - 3.0 + 4.0 * exp(y) - exp(ty);
        c->gn = exp(y) - ty - exp(-y);
        c->goy2 = c->gn / (y * y);
        c->goy3 = c->gn / (y * y * y);
        c->hn = y / (exp(y) - exp(-y));
    }
    if (gamma < 0.05) {   /* setupLow */
        double y1 = y, y2 = y1 * y1, y3 = y2 * y1, y4 = y3 * y1, y5 = y4 * y1;
        double y6 = y5 * y1, y7 = y6 * y1, y8 = y7 * y1, y9 = y8 * y1;
        c->coeff1 = 1.0 - 0.5 * y1 + (1.0 / 6.0) * y2 - (1.0 / 24.0) * y3 + (1.0 / 120.0) * y4;
        c->coeff2 = (1.0 / 12.0) * y1 - (1.0 / 24.0) * y2 + (1.0 / 80.0) * y3 - (1.0 / 360.0) * y4;
        c->coeff3 = 0.5 - (1.0 / 6.0) * y1 + (1.0 / 24.0) * y2 - (1.0 / 120.0) * y3;
        c->sig1 = +(2.0 / 3.0) * y3 - 0.5 * y4 + (7.0 / 30.0) * y5 - (1.0 / 12.0) * y6
                  + (31.0 / 1260.0) * y7 - (1.0 / 160.0) * y8 + (127.0 / 90720.0) * y9;
        c->sig2 = -(2.0 / 3.0) * y3 - 0.5 * y4 - (7.0 / 30.) * y5 - (1.0 / 12.0) * y6
                  - (31.0 / 1260.0) * y7 - (1.0 / 160.0) * y8 - (127.0 / 90720.0) * y9;
        c->goy2 = (1.0 / 3.0) * y1 + (1.0 / 60.0) * y3;
        c->goy3 = 1.0 / 3.0 + (1.0 / 60.0) * y2;
        c->hn = 0.5 - (1.00 / 12.0) * y2 + (7.0 / 720.0) * y4;
        c->gn = (1.0 / 3.0) * y3 + (1.0 / 60.0) * y5;
    }
    if (gamma == 0) {     /* setupZero */
        c->coeff0 = 1.0;
        c->coeff1 = 1.0;
        c->coeff2 = 0.0;
        c->coeff3 = 0.5;
    }
    double gamma2 = gamma * gamma;
    c->sig1 = sqrt(+kT * c->sig1 / gamma2);
    c->sig2 = sqrt(-kT * c->sig2 / gamma2);
    c->corr = (kT / (gamma2)) * (c->gn / (c->sig1 * c->sig2));
    c->dev = sqrt(1.0 - (c->corr * c->corr));
}

/* systemHandling.cpp:87-92 + particle.cpp:115-131 */
void oracle_push_force(int n, const double* force, double* frc, double* frc0) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < 3 * n; i++) {
        frc0[i] = frc[i];
        frc[i] = force[i];
    }
}

/* utilities.cpp:26-50 */
static inline double safe_mod(double v, double base) {
    if (v < 0) return v + base;
    if (v >= base) return v - base;
    return v;
}
static inline double safe_mod0(double v0, double v, double base) {
    double dx = v - v0;
    return (fabs(dx) > (base / 2)) ? ((dx < 0) ? v0 - base : v0 + base) : v0;
}

/* particle.cpp:61-99 (setX/setY/setZ via setPos) */
static inline int set_pos(double* pos, double* pos0, const double nw[3], double L) {
    int bad = 0;
    for (int k = 0; k < 3; k++) {
        double old = pos[k];
        pos[k] = safe_mod(nw[k], L);
        pos0[k] = safe_mod0(old, pos[k], L);
        if ((pos[k] < 0.0) || (pos[k] >= L)) bad = 1;
    }
    return bad;
}

int oracle_vgb_step(const oracle_geom* g, const oracle_vgb* c, double dt, int first,
                    int vel_step, const double* noise, double* pos, double* pos0,
                    double* vel, const double* frc, const double* frc0,
                    const double* mass, double* mem, double* mem_corr) {
    const int n = g->n;
    const double L = g->box;
    int bad_all = 0;
    if (first) {
        /* brownianIntegrator.cpp:191-223 (G&B 1981 eq. 2.26) */
#pragma omp parallel for schedule(static) reduction(| : bad_all)
        for (int i = 0; i < n; i++) {
            double* p = &pos[3 * i];
            mem_corr[3 * i] = 0.0; mem_corr[3 * i + 1] = 0.0; mem_corr[3 * i + 2] = 0.0;
            mem[3 * i + 0] = noise[6 * (size_t)i + 0];
            mem[3 * i + 1] = noise[6 * (size_t)i + 1];
            mem[3 * i + 2] = noise[6 * (size_t)i + 2];
            double m = 1.0 / mass[i];
            double nw[3];
            for (int k = 0; k < 3; k++)
                nw[k] = p[k] + (vel[3 * i + k] * c->coeff1 * dt)
                        + (frc[3 * i + k] * c->coeff3 * dt * dt * m) + (c->sig1 * mem[3 * i + k]);
            bad_all |= set_pos(p, &pos0[3 * i], nw, L);
        }
    } else {
        /* brownianIntegrator.cpp:225-296, velocityStep :298-356 */
        const double dt2 = dt * dt;
        const double c0 = 1.0 + c->coeff0;
        const double dt_inv = 1.0 / dt;
#pragma omp parallel for schedule(static) reduction(| : bad_all)
        for (int i = 0; i < n; i++) {
            double* p = &pos[3 * i];
            double* p0 = &pos0[3 * i];
            double* mx = &mem[3 * i];
            double* mc = &mem_corr[3 * i];
            const double* F = &frc[3 * i];
            const double* F0 = &frc0[3 * i];
            const double* xi = &noise[6 * (size_t)i];
            for (int k = 0; k < 3; k++) mc[k] = xi[k];
            for (int k = 0; k < 3; k++) mc[k] = c->sig2 * ((c->corr * mx[k]) + (c->dev * mc[k]));
            for (int k = 0; k < 3; k++) mx[k] = xi[3 + k];
            double m = 1.0 / mass[i];
            double c1 = m * dt2 * c->coeff1;
            double c2 = m * dt2 * c->coeff2;
            double nw[3];
            for (int k = 0; k < 3; k++) {
                nw[k] = (c0 * p[k]);
                nw[k] -= (c->coeff0 * p0[k]);
                nw[k] += (c1 * F[k]);
                nw[k] += (c2 * (F[k] - F0[k]));
                nw[k] += (c->sig1 * mx[k]) + (c->coeff0 * mc[k]);
            }
            if (vel_step) {
                double dt3 = dt * dt2;
                double g2 = m * dt2 * c->goy2;
                double g3 = m * dt3 * c->goy3;
                double g4 = c->hn * dt_inv;
                for (int k = 0; k < 3; k++) {
                    double d0 = p[k] - p0[k];
                    double xn = safe_mod(nw[k], L);
                    double x0 = safe_mod0(p[k], xn, L);
                    double d = xn - x0;
                    double v = d + d0;
                    v += (g2 * F[k]);
                    v -= (g3 * (F[k] - F0[k]));
                    v += (mc[k] - c->sig1 * mx[k]);
                    v *= g4;
                    vel[3 * i + k] = v;
                }
            }
            bad_all |= set_pos(p, p0, nw, L);
        }
    }
    return bad_all ? ORACLE_ERR_BOUNDS : 0;
}

/* Six standard normal deviates for (step, particle) from a counter-based
 * generator (SplitMix64 finaliser, Steele et al. 2014, + Box-Muller); used
 * when no injected noise is given, e.g. for timing the CPU path. */
static inline uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static void counter_noise(int step, int n, double* out) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; i++) {
        uint64_t key = ((uint64_t)(uint32_t)step << 32) ^ (uint64_t)(uint32_t)i;
        for (int k = 0; k < 3; k++) {
            uint64_t a = mix64(key * 6 + 2 * k), b = mix64(key * 6 + 2 * k + 1);
            double u1 = ((double)(a >> 11) + 1.0) * (1.0 / 9007199254740992.0);
            double u2 = (double)(b >> 11) * (1.0 / 9007199254740992.0);
            double r = sqrt(-2.0 * log(u1));
            out[6 * (size_t)i + 2 * k] = r * cos(6.283185307179586 * u2);
            out[6 * (size_t)i + 2 * k + 1] = r * sin(6.283185307179586 * u2);
        }
    }
}

/* system.cpp:170-212, the hot loop without the analysis-only sweep. */
int oracle_run(const oracle_geom* g, const oracle_force* f, const oracle_vgb* c,
               double dt, int step0, int n_steps, int vel_freq, int* vel_counter,
               const double* noise, int noise_steps, double* pos, double* pos0, double* vel,
               double* frc, double* frc0, const double* radius, const double* mass,
               double* mem, double* mem_corr, int* hi, uint32_t* cse, double* sorted,
               double* force) {
    const int n = g->n;
    double* own = noise ? NULL : (double*)malloc(sizeof(double) * 6 * (size_t)(n > 0 ? n : 1));
    for (int t = 0; t < n_steps; t++) {
        int step = step0 + t;
        int e = oracle_forces(g, f, sorted, hi, cse, force);
        if (e) { free(own); return e; }
        oracle_push_force(n, force, frc, frc0);
        const double* nz;
        if (own) {
            counter_noise(step, n, own);
            nz = own;
        } else {
            const int nt = noise_steps > 0 ? t % noise_steps : t;
            nz = noise + (size_t)nt * (size_t)n * 6;
        }
        if (step == 0) {
            e = oracle_vgb_step(g, c, dt, 1, 0, nz, pos, pos0, vel, frc, frc0, mass, mem, mem_corr);
        } else {
            int vs = (vel_freq == 0 || *vel_counter == vel_freq);
            e = oracle_vgb_step(g, c, dt, 0, vs, nz, pos, pos0, vel, frc, frc0, mass, mem, mem_corr);
            *vel_counter = (*vel_counter == vel_freq) ? 0 : *vel_counter + 1;
        }
        if (e) { free(own); return e; }
        oracle_build_cells(g, pos, radius, hi, cse, sorted);
    }
    free(own);
    return 0;
}

/* ------------------------------------------------------ reference RNG */

/* fastRandom.cpp:27-33 */
void oracle_fastrandom_init(oracle_fastrandom* r) {
    memset(r, 0, sizeof(*r));
}

/* fastRandom.cpp:40-89 (psdrand) */
static double fr_psdrand(oracle_fastrandom* r, int iseed) {
    const int ndim = 55, m10 = 1000000000, is = 21, ir = 30;
    int32_t* st = r->istack;
    if ((!r->init) || (iseed < 0)) {
        iseed = abs(iseed);
        st[ndim] = iseed;
        int j = iseed, k = 1;
        for (int i = 1; i <= ndim - 1; ++i) {
            int inx = i * is - (int)((double)(i * is) / (double)ndim) * ndim;
            st[inx] = k;
            k = j - k;
            if (k < 0) k += m10;
            j = st[inx];
        }
        for (int jj = 1; jj <= 3; ++jj)
            for (int i = 1; i <= ndim; ++i) {
                int inx = i + ir - (int)((double)(i + ir) / (double)ndim) * ndim;
                st[i] = (int32_t)((uint32_t)st[i] - (uint32_t)st[inx + 1]);
                if (st[i] < 0) st[i] += m10;
            }
        r->jrand = 0;
        r->init = 1;
    }
    r->jrand += 1;
    if (r->jrand > ndim) {
        for (int i = 1; i <= ndim; ++i) {
            int inx = i + ir - ((int)((double)(i + ir) / (double)ndim)) * ndim;
            st[i] = (int32_t)((uint32_t)st[i] - (uint32_t)st[inx + 1]);
            if (st[i] < 0) st[i] += m10;
        }
        r->jrand = 1;
    }
    return ((double)st[r->jrand]) / 1.0E9;
}

/* fastRandom.cpp:92-124 (g250, mu = 0, sigma = 1) */
double oracle_fastrandom_g250(oracle_fastrandom* r, int seed) {
    if (!r->deviate_available) {
        double v1, v2, rsq;
        do {
            v1 = 2.0 * fr_psdrand(r, seed) - 1.0;
            v2 = 2.0 * fr_psdrand(r, seed) - 1.0;
            rsq = v1 * v1 + v2 * v2;
        } while (rsq >= 1.0 || rsq == 0.0);
        double polar = sqrt(-2.0 * log(rsq) / rsq);
        r->stored_deviate = (float)(v1 * polar);
        r->deviate_available = 1;
        return v2 * polar * 1.0 + 0.0;
    }
    r->deviate_available = 0;
    return r->stored_deviate * 1.0 + 0.0;
}

/* The reference's own noise stream in the injected-noise layout
 * out[(t*n + i)*6 + k].  Particle i draws from its own generator gens[i]
 * with threadSeed = seed*(i+1) (brownianIntegrator.cpp:204, :236; int
 * arithmetic, so valid only while that product fits an int).  The first
 * step draws memX, memY, memZ (:206-208) into k = 0..2; a normal step draws
 * the three memCorr deviates then memX, memY, memZ (:238-249) into
 * k = 0..5.  first != 0: local step 0 is the first step. */
void oracle_fastrandom_fill(oracle_fastrandom* gens, int n, int seed, int first,
                            int n_steps, double* out) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; i++) {
        const int ts = (int)(int32_t)((uint32_t)seed * (uint32_t)(i + 1));
        for (int t = 0; t < n_steps; t++) {
            double* o = out + ((size_t)t * (size_t)n + (size_t)i) * 6;
            const int draws = (first && t == 0) ? 3 : 6;
            for (int k = 0; k < draws; k++) o[k] = oracle_fastrandom_g250(&gens[i], ts);
            for (int k = draws; k < 6; k++) o[k] = 0.0;
        }
    }
}
