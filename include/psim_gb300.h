/*
 * psim_gb300.h -- C ABI of the GB300-native ProteinSim2015 Langevin step.
 *
 * One library, libpsim_gb300.so, runs the reference's hot path on one GPU
 * (sm_103a): the hashed cell-list rebuild, pair forces from the IForce
 * plugins (AOPotential, LennardJones, Calibration) and the van Gunsteren-
 * Berendsen stochastic-dynamics integrator.  Plain pointers and sizes only.
 *
 * Three layers of entry points:
 *   1. Drop-ins that take the reference's own host arrays (psim_cells_build,
 *      psim_force_evaluate, psim_integrator_*): each replaces one reference
 *      routine, cited beside it, with the same array layouts.  Host buffers in,
 *      host buffers out; the copies to and from the GPU are inside the call.
 *   2. A device-resident system (psim_system_*): the whole step loop of
 *      system::run on the GPU with no per-step host traffic.
 *   3. Plugin parameters (psim_force_params_*): the settings.cfg keys each
 *      plugin reads, so a plugin's getForce(config*) factory maps onto a
 *      device pair functor.
 *
 * Status codes are the reference's exit codes (ClusteredCore/src/utilities/
 * error.cpp:27-68; the loader's 100 from ClusteredUI/src/runSim.cpp:41-58),
 * returned instead of terminating the process.
 *
 * Array layouts (the reference's, ClusteredCore/include/system.h:33-38):
 *   pos, pos0, vel, frc, frc0   3n doubles, xyz per particle, original order
 *   particle_hash_index         2n int32 (cell hash, original index), sorted
 *   cell_start_end              2*s^3 uint32 (start, end); empty = 0xffffffff
 *   sorted_particles            4n doubles {x, y, z, radius}, sorted order
 *   particle_force              3n doubles, original order
 */
#ifndef PSIM_GB300_H
#define PSIM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    PSIM_OK = 0,
    PSIM_ERR_LOAD = 100,             /* plugin not loadable (runSim.cpp:41-58) */
    PSIM_ERR_INIT = 7701,            /* error.cpp:27-32 */
    PSIM_ERR_CELL_BOUNDS = 7702,     /* error.cpp:34-38: a particle hashed outside the grid */
    PSIM_ERR_PARTICLE_BOUNDS = 7703, /* error.cpp:40-45: particle.cpp:67-69 */
    PSIM_ERR_OVERLAP = 7704,         /* error.cpp:47-55: AOPotential.cpp:85-88 */
    PSIM_ERR_NAN_FORCE = 7705,       /* error.cpp:57-62: AOPotential.cpp:105-109 */
    PSIM_ERR_INPUT = 7706,           /* error.cpp:64-68: invalid arguments */
    PSIM_ERR_CUDA = 7790,            /* CUDA runtime failure, see psim_last_error_string */
    PSIM_ERR_NO_DEVICE = 7791        /* no CUDA device */
};

typedef enum {
    PSIM_FORCE_AO = 1,          /* AOPotential/src/AOPotential.cpp */
    PSIM_FORCE_LJ = 2,          /* LennardJones/src/LJPotential.cpp */
    PSIM_FORCE_CALIBRATION = 3, /* Calibration/src/Calibration.cpp */
    PSIM_FORCE_AO_YUKAWA = 4,   /* AO + LJ(n) summed (the reference evaluates one plugin only) */
    PSIM_FORCE_PLUGIN = 5       /* a plugin's own device functor, run through its
                                   psim_force_launch entry (see psim_force_args) */
} psim_force_kind;

typedef enum {
    PSIM_PRECISION_FP64 = 0,  /* plain form: FP64 throughout, reference operation order */
    PSIM_PRECISION_MIXED = 1  /* FP32 pair math + Kahan-compensated FP32 sums, FP64 update */
} psim_precision;

typedef enum {
    PSIM_NOISE_PHILOX = 0,   /* counter-based Philox4x32-10 Gaussians keyed by (seed, particle) */
    PSIM_NOISE_INJECTED = 1  /* caller-supplied Gaussians in the reference draw order */
} psim_noise_mode;

/* Pair-force parameters under the reference's settings.cfg keys.
 * AOPotential.cpp:33-59: kT, wellDepth (0.261), cutOff (1.1).
 * LJPotential.cpp:29-62: kT, wellDepth (10), yukawaStrength (8), ljNum (18),
 *                        cutOff (2.5), debyeLength (0.5).
 * Calibration.cpp:30-39: cutOff (1.1).
 * PSIM_FORCE_AO_YUKAWA: the AO part uses kT/well_depth/cutoff, the LJ(n)
 * part kT/well_depth2/yukawa_strength/debye_length/lj_num/cutoff2.
 * PSIM_FORCE_PLUGIN: the library reads only `cutoff` (the cell-size check,
 * the candidate test and the pair list's radius); `user` carries whatever
 * the plugin's functor needs, filled by the plugin itself. */
typedef struct {
    int32_t kind;
    int32_t lj_num;
    double kT;
    double cutoff;
    double well_depth;
    double yukawa_strength;
    double debye_length;
    double cutoff2;
    double well_depth2;
    double user[8];
} psim_force_params;

/* Cell-grid geometry: mirrors systemState's boxSize/cellSize/cellScale
 * (ClusteredCore/include/structs/systemState.h:7-19), widened to double so a
 * box need not be an integer.  Requires scale >= 3, cell_size * scale == box
 * and cell_size >= the largest cutoff (checked; the reference does not). */
typedef struct {
    int32_t n_particles;
    int32_t cell_scale;
    double box_size;
    double cell_size;
} psim_geometry;

/* vGB coefficients (brownianIntegrator.cpp:27-99, :111-175). */
typedef struct {
    double y, coeff0, coeff1, coeff2, coeff3;
    double sig1, sig2, corr, dev;
    double goy2, goy3, hn, gn;
} psim_vgb_coeffs;

/* Integrator settings: the brownianIntegrator keys of settings.cfg
 * (brownianIntegrator.cpp:33-83): gamma (0.5), timeStep (0.001), kT (1),
 * velFreq (1000), seed (90210). */
typedef struct {
    double gamma;
    double dt;
    double kT;
    int32_t vel_freq;
    int32_t seed;
} psim_integrator_config;

/* ------------------------------------------------ plugin device entry */

/* What a force plugin's device entry receives: one force pass over the
 * system's current cell list or pair list, queued on the caller's stream.
 * The pointers are device memory owned by the library; the plugin owns only
 * its parameters.  Each force plugin (a shared object that exports the
 * reference factory getForce(config*), e.g. AOPotential.h:77-80) also
 * exports
 *     int psim_force_launch(const psim_force_args* args, void* stream);
 * built from the library's header-only force templates instantiated with the
 * plugin's own __device__ pair functor (csrc/psim_plugin.cuh), so a new
 * potential needs no rebuild of the library.  It returns 0 or a PSIM_ERR_*
 * code (PSIM_ERR_CUDA for a failed launch); physical errors (overlap,
 * non-finite force) are latched in *err as the library's own passes do. */
#define PSIM_FORCE_ABI 2
typedef enum {
    PSIM_PASS_FP64 = 0,   /* plain FP64 form, 27-cell walk over pos_fp64 */
    PSIM_PASS_MIXED = 1,  /* FP32 pairs + Kahan sums, 27-cell walk over pos_hi/pos_lo */
    PSIM_PASS_LIST = 2    /* FP32 pairs + Kahan sums over the Verlet pair list */
} psim_force_pass;
typedef struct {
    int32_t abi;                      /* PSIM_FORCE_ABI */
    int32_t pass;                     /* psim_force_pass */
    const psim_force_params* params;  /* the plugin's parameters */
    /* the cell grid (systemState's nParticles, cellScale, boxSize, cellSize) */
    int32_t n_particles;
    int32_t cell_scale;
    double box_size;
    double cell_size;
    /* the cell list in sorted order (PSIM_PASS_FP64 / PSIM_PASS_MIXED) */
    const void* pos_fp64;             /* n x {x, y, z, R} doubles, 32-byte aligned */
    const void* pos_hi;               /* n x {x, y, z, R} floats (rounded) */
    const void* pos_lo;               /* n x float4 low parts (x - x_hi, ...) */
    const int32_t* cell_id;           /* cell of each sorted slot */
    const int32_t* cell_start;        /* first sorted slot of each cell */
    const int32_t* cell_count;        /* particles of each cell */
    float prefilter_r2;               /* FP32 candidate bound on r^2 (>= cutoff^2) */
    int32_t tile;                     /* 0: a warp per 32 sorted particles; 1: a block per cell */
    /* the Verlet pair list (PSIM_PASS_LIST) */
    const void* list_pos;             /* records, list order (compact: 16 B; full: 32 B) */
    const int32_t* list_count;        /* entries of each list slot */
    const uint32_t* list;             /* entries, groups of 8 per slot */
    int32_t list_stride;
    int32_t list_compact;
    float list_radius;                /* the one radius of compact records */
    float list_unit;                  /* unit 2^-k of compact records' fixed-point coordinates */
    /* output, in the pass's order (sorted or list order) */
    double* fx;
    double* fy;
    double* fz;
    uint32_t* err;                    /* error bits, OR-ed */
    const int32_t* gate;              /* NULL, or: the pass runs only when *gate != 0 */
} psim_force_args;
typedef int (*psim_force_launch_fn)(const psim_force_args* args, void* stream);

/* ------------------------------------------------------------ general */

/* Version of this ABI (bumped on any layout change). */
int psim_abi_version(void);
/* Text of the last error on the calling thread ("" if none). */
const char* psim_last_error_string(void);
/* Number of usable CUDA devices (0 on a machine without a GPU). */
int psim_device_count(void);

/* ---------------------------------------------------- plugin parameters */

/* Fill params from settings.cfg text (key = value lines; '#' at column 0
 * starts a comment, as config.cpp:27-56) with the plugin's defaults for
 * missing keys.  plugin is the reference plugin name: "AOPotential",
 * "LennardJones", "Calibration", or "AOYukawa" for the composite, whose LJ
 * part reads the keys prefixed "yukawa." (e.g. "yukawa.cutOff").
 * Replaces the plugin constructors AOPotential.cpp:33-59,
 * LJPotential.cpp:29-62, Calibration.cpp:30-39.  Returns PSIM_ERR_LOAD for
 * an unknown plugin name. */
int psim_force_params_from_settings(const char* plugin, const char* settings_text,
                                    psim_force_params* out);

/* The AO coefficients coEff1/coEff2 (AOPotential.cpp:50-55). */
int psim_ao_coefficients(double kT, double well_depth, double cutoff, double* coeff1,
                         double* coeff2);

/* ------------------------------------ drop-ins on the reference layout */

/* Host arrays of the drop-ins.  On a device that can access pageable host
 * memory (a Grace host's coherent link, cudaDevAttrPageableMemoryAccess) the
 * GPU reads the caller's input arrays and writes its output arrays in place,
 * pinned or not; elsewhere, or with PSIM_DROPIN_COPIES=1 in the environment,
 * the calls copy them in and out.  Either way the arrays must stay valid and
 * untouched by other threads for the call, and the results are identical. */

/* system::hashParticles + sortParticles + clearCells + reorderParticles
 * (ClusteredCore/src/system/systemHandling.cpp:33-85, system.h:166).
 * pos: 3n original order; radius: n.  Outputs particle_hash_index (2n),
 * cell_start_end (2*s^3) and sorted_particles (4n).  Within a cell particles
 * are ordered by original index (the reference's sort is unstable; cell
 * membership and hashes are identical). */
int psim_cells_build(const psim_geometry* geom, const double* pos, const double* radius,
                     int32_t* particle_hash_index, uint32_t* cell_start_end,
                     double* sorted_particles);

/* The cell-list build of psim_cells_build for callers that cannot allocate
 * device memory (hosts that own all device memory through their own pool and
 * forbid cudaMalloc/cudaFree in their step loop, or that cannot afford an
 * allocation's latency).  No counterpart in the reference, which has no
 * device code.  All buffers are the caller's device buffers, in the same
 * layouts as psim_cells_build: d_pos (3n), d_radius (n) in; d_hash_index
 * (2n), d_cell_start_end (2*s^3), d_sorted (4n, 32-byte aligned) out.  Work
 * is queued on `stream` (a cudaStream_t; NULL = default stream) and the call
 * blocks until it is done, so it cannot be called while a stream is being
 * captured.  The scratch is one static 32 MiB device array held by every GPU
 * that loads the library until exit; each call looks its address up with the
 * caller's device current (so calls after a device reset are fine); calls
 * that overlap on the GPU share and race on it.  Problems needing more
 * scratch than the array (about 76 bytes per particle plus 8 per cell) return
 * PSIM_ERR_INPUT.  Allocates no device memory. */
int psim_cells_build_noalloc(const psim_geometry* geom, const double* d_pos,
                             const double* d_radius, int32_t* d_hash_index,
                             uint32_t* d_cell_start_end, double* d_sorted, void* stream);

/* defaultForceManager::getAcceleration (defaultForceManager.cpp:55-65) with
 * the plugin's getAcceleration/iterCells (e.g. AOPotential.cpp:61-175) on
 * a cell list in the reference layout.  Writes particle_force (3n, original
 * order).  Returns PSIM_ERR_OVERLAP / PSIM_ERR_NAN_FORCE where the
 * reference would have exited with those codes. */
int psim_force_evaluate(const psim_force_params* params, const psim_geometry* geom,
                        int32_t precision, const double* sorted_particles,
                        const int32_t* particle_hash_index, const uint32_t* cell_start_end,
                        double* particle_force);

/* psim_force_evaluate through a force plugin's device entry (its
 * psim_force_launch, with its parameters): defaultForceManager::
 * getAcceleration for a plugin whose pair functor is not built into this
 * library.  Same arrays, precisions and errors as psim_force_evaluate. */
int psim_force_evaluate_plugin(psim_force_launch_fn launch, const psim_force_params* params,
                               const psim_geometry* geom, int32_t precision,
                               const double* sorted_particles,
                               const int32_t* particle_hash_index,
                               const uint32_t* cell_start_end, double* particle_force);

/* The pair list of psim_force_evaluate's mixed precision.  The call walks the
 * pairs within cutOff + skin of a list it built on an earlier call, found
 * from that call's cell list, and keeps doing so while no particle (by its
 * original index) has moved skin/2 since that build; it builds a new list
 * otherwise, and whenever n, the grid or the cutoff changed.  The forces are
 * those of this call's positions either way (every pair within cutOff is in
 * the list); only the FP32 summation order follows the list.  skin 0
 * (default): a list of each call's own pairs, built every call, so that a
 * call depends on its arguments alone, as the reference's does; skin < 0:
 * the smaller of 0.4 and cellSize - cutOff, if at least 0.1, else none;
 * skin > 0: that skin, at most cellSize - cutOff.  A caller that steps one
 * system through the drop-ins opts in to the kept list.  No counterpart in
 * the reference. */
int psim_force_set_list_skin(double skin);
/* Mixed-precision psim_force_evaluate calls so far, and the pair lists they
 * built. */
int psim_force_list_stats(int64_t* calls, int64_t* builds);

/* The brownianIntegrator constructor's coefficient set-up
 * (brownianIntegrator.cpp:27-99).  gamma == 0 reproduces the reference's
 * non-finite noise widths; such coefficients are refused by the steppers. */
int psim_vgb_coefficients(double gamma, double dt, double kT, psim_vgb_coeffs* out);

/* brownianIntegrator: the object holding the per-particle noise memory
 * (memX/Y/Z, memCorrX/Y/Z) and the velocity counter
 * (ClusteredCore/include/integrator.h:20-158).  Device-resident. */
typedef struct psim_integrator psim_integrator;
psim_integrator* psim_integrator_create(const psim_integrator_config* cfg, int32_t n_particles);
void psim_integrator_destroy(psim_integrator* integ);

/* system::pushParticleForce (systemHandling.cpp:87-92) when particle_force is
 * not NULL, then brownianIntegrator::nextSystem (brownianIntegrator.cpp:
 * 181-356) on host arrays in original order.  current_time == 0 selects
 * firstStep as the reference does.  noise: n*6 Gaussians in the reference
 * draw order (firstStep uses the first 3 per particle) for
 * PSIM_NOISE_INJECTED, ignored for PSIM_NOISE_PHILOX.  pos/pos0/vel/frc/frc0
 * are updated in place.  box_size: the box edge L.  Host arrays as for the
 * other drop-ins (PSIM_DROPIN_COPIES is read when the integrator is created). */
int psim_integrator_next_system(psim_integrator* integ, double current_time, double box_size,
                                int32_t noise_mode, const double* noise,
                                const double* particle_force, double* pos, double* pos0,
                                double* vel, double* frc, double* frc0, const double* mass);

/* --------------------------------------------- device-resident system */

typedef struct psim_system psim_system;

typedef struct {
    psim_geometry geom;
    psim_integrator_config integ;
    psim_force_params force;
    int32_t precision;   /* psim_precision */
    int32_t noise_mode;  /* psim_noise_mode */
    int32_t device;      /* CUDA device ordinal */
    /* Verlet pair-list skin (mixed form only; 0: the force pass walks the
     * 27 cells every step).  With skin > 0 the pairs within cutOff + skin are
     * listed from the cell walk and reused until a particle has moved skin/2;
     * each step's force is the same set of pair terms.  Needs
     * cellSize >= cutOff + skin. */
    double skin;
    /* NULL: the library's own functor for force.kind.  Otherwise a force
     * plugin's psim_force_launch entry: every force pass of the system runs
     * through it (force.kind may then be PSIM_FORCE_PLUGIN). */
    psim_force_launch_fn force_launch;
} psim_system_config;

/* ---------------------------------------------- initial states (host) */

/* Random sequential addition: n points uniform in the periodic cube of edge
 * box, each at least min_sep from all earlier ones (pos: 3n, original order).
 * Stands in for the reference's initialiser (systemInit.cpp:31-160), whose
 * O(N^2) overlap sweep cannot build large or dense systems.  max_trials > 0
 * bounds the attempts (7701 when exceeded, near the RSA jamming limit). */
int psim_init_rsa(int32_t n, double box, double min_sep, uint64_t seed, int64_t max_trials,
                  double* pos);

/* The same construction on a GPU: the same trials in the same order (a trial
 * is kept when no earlier kept trial lies within min_sep), evaluated in
 * chunks of trials in parallel; the result is psim_init_rsa's for the same
 * arithmetic.  Falls back to psim_init_rsa for boxes of fewer than 3 cells of
 * min_sep a side. */
int psim_init_rsa_device(int32_t n, double box, double min_sep, uint64_t seed,
                         int64_t max_trials, double* pos, int32_t device);

/* ------------------------------------------- differentiable trajectory */

/* Gradients of a trajectory loss with the noise held fixed (no reference
 * counterpart: the reference has no derivatives).  The trajectory is the vGB
 * positions update of the plain FP64 form (brownianIntegrator.cpp:191-296:
 * firstStep, then normal steps, Philox noise keyed by particle and step as
 * the system's, uniform mass) under the AO plugin plus the Yukawa term of the
 * LennardJones plugin with ljNum = 0; the loss is the squared distance
 * between the trajectory's time-averaged, Gaussian-smoothed g(r) (samples
 * every sample_every steps; n_bins bins of [r_min, r_max), kernel width
 * sigma) and a target.  The reverse pass recomputes checkpoint_every-step
 * segments from checkpoints of the forward pass. */
typedef struct psim_adjoint psim_adjoint;

typedef struct {
    psim_geometry geom;             /* cellSize >= every cutoff and r_max + 4 sigma */
    psim_integrator_config integ;   /* gamma, dt, kT, seed (velFreq unused) */
    double mass;
    int32_t n_steps, checkpoint_every, sample_every;
    double r_min, r_max;
    int32_t n_bins;
    double sigma;
} psim_adjoint_config;

typedef struct {
    double kT;
    double ao_well_depth, ao_cutoff;   /* AOPotential wellDepth, cutOff (0: no AO term) */
    double yuk_amplitude;              /* kT wellDepth yukawaStrength of the LJ plugin */
    double yuk_length;                 /* debyeLength */
    double yuk_cutoff;                 /* its cutOff (0: no Yukawa term) */
    /* the AO coefficients' range 1 + q (0: ao_cutoff); differentiating with
     * respect to it holds the cutoff distance ao_cutoff fixed */
    double ao_range;
    /* the LennardJones plugin's LJ(n) term: fNet = -eps (2L - 1) 4n L / r,
     * L = (sigma / r)^n (eps = kT wellDepth, sigma the contact diameter) */
    double lj_epsilon, lj_sigma;
    double lj_cutoff;                  /* 0: no LJ(n) term */
    int32_t lj_n;
} psim_adjoint_params;

psim_adjoint* psim_adjoint_create(const psim_adjoint_config* cfg, int32_t device);
/* The Philox Gaussians the systems and the adjoint draw (PSIM_NOISE_PHILOX):
 * n_steps steps from first_step for particles 0..n-1 with `seed`, in the
 * injected-noise layout out[((step - first_step) n + i) 6 + k] (host memory,
 * n_steps n 6 doubles), computed on `device`.  With them a CPU checker can
 * replay a Philox run exactly. */
int psim_philox_noise(uint32_t seed, int32_t n, int64_t first_step, int32_t n_steps,
                      double* out, int32_t device);
void psim_adjoint_destroy(psim_adjoint* adj);
/* The trajectory from pos0/vel0 (3n, original order; vel0 may be NULL):
 * g_mean (n_bins) and, if not NULL, the final positions (3n, unwrapped). */
int psim_adjoint_forward(psim_adjoint* adj, const psim_adjoint_params* p, const double* pos0,
                         const double* vel0, double* g_mean, double* pos_final);
/* Loss against g_target, its g_mean (may be NULL), and the gradient
 * grad[6] = dL/d(ao_well_depth, ao_range, yuk_amplitude, yuk_length,
 * lj_epsilon, lj_sigma) -- the AO range through the AO coefficients only,
 * the cutoff distance held fixed -- and, if not NULL, dL/d(pos0) (3n). */
int psim_adjoint_gradient(psim_adjoint* adj, const psim_adjoint_params* p, const double* pos0,
                          const double* vel0, const double* g_target, double* loss,
                          double* g_mean, double* grad, double* grad_pos0);

/* ---------------------------------------------- batches of replicas */

/* One replica of a batch: its own box and cell grid, plugin parameters and
 * Philox seed.  All replicas of a batch use the same plugin (and ljNum); the
 * AO + Yukawa composite is not batched. */
typedef struct {
    psim_geometry geom;
    psim_force_params force;
    int32_t seed;
} psim_replica;

/* Independent systems stepped together: every step is one launch per phase
 * over all replicas (the force pass runs a warp task per 32 particles of one
 * replica, with that replica's grid and plugin parameters).  No reference
 * counterpart (the reference runs one system per process); each replica is
 * exactly the system psim_system_create would build from its settings, with
 * integ.seed replaced by the replica's seed, and steps bit for bit like it.
 * The returned handle takes every psim_system_* call; its arrays are the
 * replicas' arrays concatenated in replica order (original order within
 * each).  No pair-list skin (see psim_batch_create_list). */
psim_system* psim_batch_create(const psim_replica* reps, int32_t n_reps,
                               const psim_integrator_config* integ, int32_t precision,
                               int32_t noise_mode, int32_t device);

/* A batch whose force pass reads a Verlet pair list (mixed precision form):
 * every replica's cellSize must be >= its cutOff + skin.  The list is built
 * for all replicas together, on the step after a particle of any replica has
 * moved skin / 2; each replica keeps its own box, grid, pair parameters and
 * noise.  skin 0 is psim_batch_create. */
psim_system* psim_batch_create_list(const psim_replica* reps, int32_t n_reps,
                                    const psim_integrator_config* integ, int32_t precision,
                                    int32_t noise_mode, int32_t device, double skin);

/* Creates the system and its device buffers (the role of system::system,
 * system.cpp:69-103, without the random initialisation: states are uploaded). */
psim_system* psim_system_create(const psim_system_config* cfg);
void psim_system_destroy(psim_system* sys);

/* Loads a particle state (original order, reference layout) and builds the
 * first cell list (system.cpp:101-103).  pos0/vel/frc/frc0/mass may be NULL
 * (zeros; mass 1).  The step counter restarts at 0, so the next step is the
 * reference's firstStep, as after RecoverySystem (systemRecovery.cpp:43-81). */
int psim_system_upload(psim_system* sys, const double* pos, const double* pos0,
                       const double* vel, const double* frc, const double* frc0,
                       const double* radius, const double* mass);

/* Injected noise for PSIM_NOISE_INJECTED: n_steps*n*6 doubles, step-major,
 * then particle (original index), then the 6 draws of one normal step
 * (xi_x, xi_y, xi_z, mem_x, mem_y, mem_z; firstStep uses the first 3).
 * Covers steps [first_step, first_step + n_steps) of the step counter. */
int psim_system_set_noise(psim_system* sys, const double* noise, int32_t n_steps,
                          int32_t first_step);

/* Runs n_steps iterations of system::run's hot loop (system.cpp:187-206):
 * forces, push, nextSystem, cell-list rebuild.  Asynchronous launches; the
 * call waits for the GPU at the end and returns the first error any step
 * raised (the state is then that of the failing step). */
int psim_system_step(psim_system* sys, int32_t n_steps);

/* Enqueues n_steps without waiting (timing loops); errors are latched and
 * returned by the next psim_system_step / psim_system_sync. */
int psim_system_step_async(psim_system* sys, int32_t n_steps);
int psim_system_sync(psim_system* sys);

/* Current state in original order.  Any pointer may be NULL. */
int psim_system_download(psim_system* sys, double* pos, double* pos0, double* vel,
                         double* frc, double* frc0);
/* Current cell list in the reference layout.  Any pointer may be NULL.  With
 * a pair list the system re-sorts its particles only when the list is
 * rebuilt, so the cell list of the current positions is computed here. */
int psim_system_download_cells(psim_system* sys, int32_t* particle_hash_index,
                               uint32_t* cell_start_end, double* sorted_particles);

/* Snapshot on a side stream: positions (3n, original order) are copied into
 * host memory without stalling the step stream; psim_system_snapshot_wait
 * blocks until that copy is complete.  host_pos should be pinned
 * (cudaHostAlloc) for the copy to be asynchronous. */
int psim_system_snapshot_async(psim_system* sys, double* host_pos);
int psim_system_snapshot_wait(psim_system* sys);

/* Step counter (0 = next step is firstStep) and velocity counter. */
int psim_system_get_step(psim_system* sys, int64_t* step, int32_t* vel_counter);

/* The plugin force on every particle at the current state (reference
 * particle_force layout: 3n doubles, original order), from the same force
 * pass the next step will run (the pair list with a skin).  It does not step. */
int psim_system_forces(psim_system* sys, double* force);

/* ------------------------------------------- observables of the state */

/* analysisManager::getTemperature (analysisGeneral.cpp:26-43): sum of v^2 over
 * 3N, from the velocities of the last velocity step. */
int psim_system_temperature(psim_system* sys, double* kT);
/* analysisManager::meanDisplacement (analysisGeneral.cpp:45-55): mean
 * |x - x0|^2 over the particles (x0: the previous position, re-imaged). */
int psim_system_mean_displacement(psim_system* sys, double* msd);
/* <EAP> of analysisOutput.cpp:117-123: particle::calculatePotential
 * (particle.cpp:133-149, FP32 as there) averaged over the particles. */
int psim_system_potential(psim_system* sys, double* eap);
/* initDisplacementTracker (analysisTracker.cpp:26-37): from here on every
 * crossing of the box is counted by the integrator. */
int psim_system_track_start(psim_system* sys);
/* trackedDisplacement (analysisTracker.cpp:66-85): mean squared unwrapped
 * displacement since psim_system_track_start. */
int psim_system_tracked_displacement(psim_system* sys, double* msd);
/* system::updateInteractions (systemHandling.cpp:94-161): per particle, the
 * neighbours of its 27 cells closer than r_contact (the reference uses 1.2);
 * coor: n ints in original order (may be NULL), total: their sum (may be NULL).
 * r_contact <= cellSize.  Single systems only.  Counted inside one force pass
 * on the current state (the FP64 form with the reference's own test; the
 * mixed form in FP32, through its pair list when r_contact <= cutOff), else
 * by a separate 27-cell walk. */
int psim_system_interactions(psim_system* sys, double r_contact, int32_t* coor, int64_t* total);
/* analysisManager::findClusters / writeClusters (analysisCluster.cpp:26-78):
 * the connected components of the contact graph (pairs closer than r_contact,
 * the reference uses 1.2).  root: n ints in original order (may be NULL), the
 * smallest original index of each particle's cluster; n_clusters: clusters of
 * more than min_size particles (the reference keeps > 4); avg_size: their
 * members over their number, in integers as writeClusters returns it.
 * r_contact <= cellSize.  Single systems only. */
int psim_system_clusters(psim_system* sys, double r_contact, int32_t min_size, int32_t* root,
                         int32_t* n_clusters, int32_t* avg_size);

/* The radial distribution function: ordered pairs per particle with r in each
 * of n_bins equal bins of [r_min, r_max), over the ideal-gas count
 * N rho 4/3 pi (r1^3 - r0^3).  r_max <= cellSize.  Single systems only. */
int psim_system_rdf(psim_system* sys, double r_min, double r_max, int32_t n_bins, double* g);

/* Potential energy and virial of the current state, in FP64 whatever the
 * system's precision (no reference counterpart: the reference reports only
 * its work estimate <EAP>).  The pair energy u(r) is the integral of the
 * plugin's force law fNet (AOPotential.cpp:90-99, LJPotential.cpp:96-109,
 * Calibration.cpp:75-81: u' = fNet) shifted to zero at the cutoff;
 * potential = sum over pairs of u(r_ij) / N, virial = sum over pairs of
 * r_ij . f_ij / N (pressure = rho (kT + virial / 3)).  Single systems with a
 * library functor only (a plugin's energy is not known here). */
int psim_system_energy(psim_system* sys, double* potential, double* virial);

/* Threads per particle of the pair-list force pass (mixed form with a skin,
 * compact records): 1 (default), 2 or 4.  Each lane of a particle takes its
 * 8 / lanes entries of every group of 8 list entries, and the lanes' sums are
 * added in lane order, so the forces do not depend on the timing of the run;
 * an autotuner picks the fastest (no reference counterpart). */
int psim_system_set_list_lanes(psim_system* sys, int32_t lanes);

/* Pair-list rebuilds since the upload (0 without a skin; the list the upload
 * builds is not counted). */
int psim_system_list_builds(psim_system* sys, int32_t* builds);

/* The CUDA stream all step kernels are launched on (cudaStream_t). */
void* psim_system_stream(psim_system* sys);

/* Per-phase device time of the last n_steps, measured with CUDA events on
 * the step stream: out_ms[0] forces, [1] integrator, [2] cell-list rebuild,
 * [3] total.  Runs n_steps steps. */
int psim_system_profile(psim_system* sys, int32_t n_steps, double* out_ms);

/* Number of kernel launches one step issues (for launch accounting). */
int psim_system_launches_per_step(psim_system* sys);
/* Kernel launches of a step's pair-list rebuild (0 without a pair list): with
 * a pair list a step launches psim_system_launches_per_step kernels, and the
 * steps that rebuild the list this many more. */
int psim_system_launches_per_rebuild(psim_system* sys);

/* Occupancy of the current cell list: max and mean particles per cell. */
int psim_system_cell_occupancy(psim_system* sys, int32_t* max_occ, double* mean_occ);

/* Enqueues n_steps and returns their device time in milliseconds, measured
 * with CUDA events recorded on the step stream around the launches. */
int psim_system_time_steps(psim_system* sys, int32_t n_steps, double* ms);

/* Mean number of ordered pairs (i, j != i) closer than `cutoff` per
 * particle in the current cell list (diagnostic for the pair-work count). */
int psim_system_pair_count(psim_system* sys, double cutoff, double* mean_pairs);

/* ----------------------------------------------------------- measurement */

/* Sustained FP32 FMA throughput of `device` in TFLOP/s (an FMA = 2 flops),
 * measured with a register-resident FMA-chain kernel over all SMs; the
 * denominator of the force pass's FP32 roofline. */
int psim_measure_fp32_peak(int32_t device, double* tflops);

/* Host-link bandwidth of `device` in GB/s, measured with SM loads and stores
 * on pinned host memory (128 MiB): reading host memory, writing it, and both
 * at once (host to host through the SMs, each byte counted once per
 * crossing); the denominators of the drop-ins' end-to-end roofline. */
int psim_measure_host_link(int32_t device, double* read_gbs, double* write_gbs,
                           double* both_gbs);

#ifdef __cplusplus
}
#endif
#endif /* PSIM_GB300_H */
