/*
 * psim_oracle.h -- CPU restatement of ProteinSim2015's Langevin step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker that the GB300 kernels are
 * compared against, and the "port" CPU baseline that bench.py times.  Only
 * tests/, __graft_entry__.smoke() and bench.py's CPU legs may load it; the
 * product library (proteinsim2015_gb300) never links or calls it.
 *
 * Parity pin: this restatement is checked against the reference itself,
 * rebuilt from its own sources by oracle/build_ref.sh into oracle/_ref/, and
 * against the golden fixtures in tests/golden/ that the reference produced
 * (tests/golden/make_golden.py).
 *
 * Layout follows the reference's own host arrays:
 *   particles        original order; pos/pos0/vel/frc/frc0 are AoS xyz (3n)
 *   hash_index       2n ints, pairs (hash, original index)   -- particleHashIndex
 *   cell_start_end   2*s^3 uint32, pairs (start, end), empty = 0xffffffff
 *                                                              -- cellStartEnd
 *   sorted           4n doubles {x, y, z, radius} in sorted order
 *                                                              -- sortedParticles
 *   force            3n doubles in ORIGINAL order            -- particleForce
 */
#ifndef PSIM_ORACLE_H
#define PSIM_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Mirrors PSim::systemState (ClusteredCore/include/structs/systemState.h:7-19)
 * with the box and cell edge widened to double.  For an integer box the
 * results are those of the reference's int fields. */
typedef struct {
    int n;             /* nParticles */
    double box;        /* boxSize L */
    double cell_size;  /* cellSize */
    int scale;         /* cellScale s; s^3 cells */
} oracle_geom;

enum { ORACLE_AO = 1, ORACLE_LJ = 2, ORACLE_CAL = 3, ORACLE_AO_YUK = 4 };

/* Pair-force parameters, filled from the same settings.cfg keys as the
 * reference plugins (AOPotential.cpp:33-59, LJPotential.cpp:29-62,
 * Calibration.cpp:30-39). */
typedef struct {
    int kind;
    double cutoff;       /* cutOff */
    /* AO */
    double ao_c1, ao_c2; /* coEff1, coEff2 */
    /* LJ / Yukawa */
    double kT, well_depth, yuk_str, debye_length;
    int lj_num;
    /* composite AO + LJ(n) : the LJ part has its own cutoff */
    double cutoff2;
} oracle_force;

/* vGB coefficients (brownianIntegrator.cpp:27-99, :111-175). */
typedef struct {
    double y, coeff0, coeff1, coeff2, coeff3;
    double sig1, sig2, corr, dev;
    double goy2, goy3, hn, gn;
} oracle_vgb;

/* error codes: the reference's exit codes (ClusteredCore/src/utilities/error.cpp) */
enum { ORACLE_OK = 0, ORACLE_ERR_BOUNDS = 7703, ORACLE_ERR_OVERLAP = 7704,
       ORACLE_ERR_NAN = 7705 };

void oracle_set_threads(int n);
int  oracle_get_threads(void);

/* AO coefficient setup (AOPotential.cpp:50-55). */
void oracle_ao_coeffs(double kT, double well_depth, double cutoff,
                      double* c1, double* c2);

/* a1: system::hashParticles (systemHandling.cpp:33-48). */
void oracle_hash(const oracle_geom* g, const double* pos, int* hash_index);
/* a2: sortParticles, made stable on (hash, index) (systemHandling.cpp:50-52). */
void oracle_sort(const oracle_geom* g, int* hash_index);
/* a3: clearCells + reorderParticles (system.h:166, systemHandling.cpp:54-85). */
void oracle_reorder(const oracle_geom* g, const double* pos, const double* radius,
                    const int* hash_index, uint32_t* cell_start_end,
                    double* sorted);
/* a1..a3 in one call. */
void oracle_build_cells(const oracle_geom* g, const double* pos,
                        const double* radius, int* hash_index,
                        uint32_t* cell_start_end, double* sorted);

/* a4..a8: defaultForceManager::getAcceleration + plugin iterCells.
 * Returns 0 or the first error code the reference would have exited with. */
int oracle_forces(const oracle_geom* g, const oracle_force* f,
                  const double* sorted, const int* hash_index,
                  const uint32_t* cell_start_end, double* force);

/* Per-particle sum over in-range pairs of the absolute values of the terms
 * of the pair force (the condition scale of the force sum: relative errors
 * are measured against it, since the terms of AO and LJ cancel near the
 * zero of the pair force). */
void oracle_force_scale(const oracle_geom* g, const oracle_force* f,
                        const double* sorted, const int* hash_index,
                        const uint32_t* cell_start_end, double* scale_out);

/* a10 */
void oracle_vgb_coeffs(double gamma, double dt, double kT, oracle_vgb* c);

/* a9: pushParticleForce / particle::setForce (systemHandling.cpp:87-92,
 * particle.cpp:115-131). */
void oracle_push_force(int n, const double* force, double* frc, double* frc0);

/* a11/a12/a14: one nextSystem call (brownianIntegrator.cpp:181-356).
 * first != 0 selects firstStep.  noise holds 6 Gaussians per particle in the
 * reference's draw order (first step uses the first 3).  vel_step != 0 runs
 * velocityStep for every particle.  mem/mem_corr: 3n each, particle order. */
int oracle_vgb_step(const oracle_geom* g, const oracle_vgb* c, double dt,
                    int first, int vel_step, const double* noise,
                    double* pos, double* pos0, double* vel,
                    const double* frc, const double* frc0,
                    const double* mass, double* mem, double* mem_corr);

/* a15: system::run loop (system.cpp:170-212) for n_steps from step0, with
 * injected noise noise[((t % noise_steps)*n + i)*6 + k] for local step t,
 * or (noise == NULL) Gaussians from a counter-based generator keyed by
 * (step, particle).  vel_freq as the integrator's
 * velFreq; *vel_counter carries the integrator's velCounter across calls.
 * Returns 0 or an error code. */
int oracle_run(const oracle_geom* g, const oracle_force* f, const oracle_vgb* c,
               double dt, int step0, int n_steps, int vel_freq, int* vel_counter,
               const double* noise, int noise_steps,
               double* pos, double* pos0, double* vel, double* frc, double* frc0,
               const double* radius, const double* mass,
               double* mem, double* mem_corr,
               int* hash_index, uint32_t* cell_start_end, double* sorted,
               double* force);

/* The reference's per-particle generator (fastRandom.cpp:40-124): a
 * subtractive lagged generator plus polar Box-Muller whose stored deviate is
 * a float.  state: 60 ints per generator (55+3 lag words, jrand, flags). */
typedef struct {
    int32_t istack[58];
    int32_t jrand;
    int32_t init;
    int32_t deviate_available;
    float stored_deviate;
} oracle_fastrandom;
void   oracle_fastrandom_init(oracle_fastrandom* r);
double oracle_fastrandom_g250(oracle_fastrandom* r, int seed);
/* n_steps of the reference's own per-particle noise (generators gens[0..n),
 * threadSeed = seed*(i+1)), in the layout oracle_run takes as injected noise:
 * out[(t*n + i)*6 + k]; with first != 0 local step 0 is firstStep's three
 * draws (k = 3..5 zero). */
void   oracle_fastrandom_fill(oracle_fastrandom* gens, int n, int seed, int first,
                              int n_steps, double* out);

/* The differentiable trajectory's parameters, as psim_adjoint_params. */
typedef struct {
    double kT;
    double ao_well_depth, ao_cutoff;
    double yuk_amplitude, yuk_length, yuk_cutoff;
    double ao_range;
    double lj_epsilon, lj_sigma, lj_cutoff;
    int32_t lj_n;
} oracle_adj_params;

/* psim_tangent.c: the loss of the differentiable trajectory (n_steps vGB
 * steps from pos0/vel0, 3n AoS each, vel0 may be NULL, with the injected
 * noise noise[(t n + i) 6 + k]; time-averaged smoothed g(r) against
 * g_target) and its gradient grad[6] = dL/d(ao_well_depth, ao_range,
 * yuk_amplitude, yuk_length, lj_epsilon, lj_sigma) by FP64 forward-mode
 * tangents.  g_mean (n_bins) may be NULL.  Returns 0. */
int oracle_adjoint_tangent(int n, double box, const oracle_adj_params* p, const oracle_vgb* c,
                           double dt, double mass, int n_steps, int sample_every, double r_min,
                           double r_max, int n_bins, double sigma, const double* pos0,
                           const double* vel0, const double* noise, const double* g_target,
                           double* loss, double* g_mean, double* grad);

#ifdef __cplusplus
}
#endif
#endif
