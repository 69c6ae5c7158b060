/*
 * fs_gpu.h -- C ABI of the GB300 FLIP substep (libfsgpu.so).
 *
 * Drop-in boundary for FlipSolver2d's per-substep hot path.  The reference
 * has no plugin system; its seams are the FlipSolver class
 * (FlipSolver2dLib/flipsolver2d.h:183-432) and LinearSolver::solve
 * (FlipSolver2dLib/linearsolver.h:15-20).  Every entry point below names the
 * reference member it replaces.  Plain C types only; all pointers are host
 * pointers unless the name says _device.  A handle owns its device memory and
 * one CUDA stream; a handle is not re-entrant (neither is the reference:
 * ThreadPool::i() and the static RNG distribution, flipsolver2d.cpp:1015).
 *
 * Errors: every call returns fs_status; FS_OK is 0.  fs_last_error() gives a
 * message for the calling thread's last failure.  There is no CPU fallback:
 * without a CUDA device fs_create fails with FS_ERR_CUDA.
 */
#ifndef FS_GPU_H
#define FS_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum fs_status {
    FS_OK = 0,
    FS_ERR_BAD_ARG = 1,     /* invalid argument or size mismatch */
    FS_ERR_CUDA = 2,        /* a CUDA runtime call failed / no device */
    FS_ERR_OOM = 3,         /* device allocation failed */
    FS_ERR_TIMEOUT = 4,     /* a bounded device-side wait gave up */
    FS_ERR_UNSUPPORTED = 5, /* feature outside the supported path */
    FS_ERR_STATE = 6,       /* call not valid in the handle's current state */
    FS_ERR_NONFINITE = 7    /* a substep produced a NaN or infinite particle velocity
                               (checked on every particle in G2P); the handle's
                               state is left as the substep made it */
} fs_status;

/* Field-for-field FlipSolverParameters (flipsolver2d.h:33-56); units and
 * meaning as in the reference (dx in metres, gravity in m/s^2, fps, ...). */
typedef struct fs_params {
    double fluidDensity;
    unsigned int seed;
    double dx;
    int particlesPerCell;
    float globalAccelerationI;
    float globalAccelerationJ;
    float resolution;
    int fps;
    int maxSubsteps;
    float picRatio;
    float cflNumber;
    float particleScale;
    int pcgIterLimit;
    float domainSizeI;
    float domainSizeJ;
    int gridSizeI;
    int gridSizeJ;
    float sceneScale;
    int viscosityEnabled;        /* each substep applies the viscosity model after
                                    the friction update and projects again, and
                                    the density correction is skipped (:425-454);
                                    the projection's tolerance becomes 1e-6 (:73) */
    int useHeavyViscosity;       /* the heavy (coupled U+V) model instead of the
                                    light one (:77-84, viscositymodel.cpp) */
    int simulationMethod;        /* must be 0 = SIMULATION_LIQUID */
    int parameterHandlingMethod; /* 0 PARTICLE, 1 HYBRID, 2 GRID */
} fs_params;

/* Pressure and density solves of a solver handle:
 *   FS_PCG_FP32  the reference's PCG and stopping rule with FP32 vectors
 *   FS_PCG_FP64  the same in FP64, bit for bit the reference's
 *   FS_PCG_SPEC  every solve to a true relative residual of 1e-6: FP32 inner
 *                PCG with the textbook incomplete-Poisson preconditioner and
 *                FP64 refinement (fs_pcg_solve_spec's method); FP64
 *                right-hand sides and pressures.  Up to the on-chip limit
 *                of fs_pcg_solve_batch a solve runs on one thread-block
 *                cluster, above it as the whole-GPU cooperative solve with
 *                its outer loop on the device.  The density push is skipped
 *                when its solve hits 20000 inner iterations, the counterpart
 *                of the reference's limit test. */
enum { FS_PCG_FP32 = 0, FS_PCG_FP64 = 1, FS_PCG_SPEC = 2 };

/* Execution knobs with no counterpart in FlipSolverParameters. */
typedef struct fs_exec_params {
    int pcg_precision; /* FS_PCG_FP32 (default), FS_PCG_FP64 or FS_PCG_SPEC */
    int pool_threads;  /* chunk count of the reference's max-abs residual test
                          (ThreadPool size, threadpool.cpp:12); 0 = this host's
                          std::thread::hardware_concurrency() like the reference */
    int device;        /* CUDA device ordinal */
    int wait_polls;    /* every bounded device-side wait of the PCG kernels (grid
                          barriers, neighbour hand-offs, TMA completions) gives
                          up after this many polls and the call returns
                          FS_ERR_TIMEOUT; 0 = the default, seconds of polling */
    int reserved[4];
} fs_exec_params;

/* Stage ids: the calls FlipSolver::step() makes, in order
 * (flipsolver2d.cpp:412-462).  Used by fs_run_stage for stage-level checks. */
enum {
    FS_STAGE_ADVECT = 0,         /* advect()                          :414 */
    FS_STAGE_DECOMPOSITION = 1,  /* matrix + IPP coefficients         :417-418 */
    FS_STAGE_REBIN = 2,          /* pruneParticles + rebinParticles   :421-422 */
    FS_STAGE_DENSITY = 3,        /* densityCorrection()               :428 */
    FS_STAGE_P2G = 4,            /* particleToGrid(); on the GPU fused with
                                    updateSdf() and updateMaterials() */
    FS_STAGE_SDF = 5,            /* no-op here: fused into FS_STAGE_P2G */
    FS_STAGE_MATERIALS = 6,      /* no-op here: fused into FS_STAGE_P2G */
    FS_STAGE_AFTER_TRANSFER = 7, /* afterTransfer(): sources only, no-op */
    FS_STAGE_LEVELSET = 8,       /* extrapolateLevelsetInside         :436 */
    FS_STAGE_VEL_EXTRAP = 9,     /* m_fluidVelocityGrid.extrapolate   :437,:455 */
    FS_STAGE_SAVE_GRID = 10,     /* saved grid copy                   :439 */
    FS_STAGE_BODY_FORCES = 11,   /* applyBodyForces()                 :440 */
    FS_STAGE_PROJECT = 12,       /* project()                         :444 */
    FS_STAGE_FRICTION = 13,      /* updateVelocityFromSolids()        :447 */
    FS_STAGE_G2P = 14,           /* particleUpdate()                  :456 */
    FS_STAGE_COUNT = 15,         /* countParticles()                  :459 */
    FS_STAGE_RESEED = 16,        /* reseedParticles(): sources only, no-op */
    FS_STAGE_DENSITY_GRID = 17,  /* updateDensityGrid() alone (plus its RHS) */
    FS_STAGE_LEVELSET_OUTSIDE = 18, /* extrapolateLevelsetOutside      :1496-1558 */
    FS_STAGE_VISCOSITY = 19      /* applyViscosity(): the light or heavy model of
                                    viscositymodel.cpp on U and V      :128-136;
                                    fs_step runs it (then FS_STAGE_PROJECT again)
                                    after the friction update when viscosity is on */
};

/* An NB-FLIP handle (fs_create_nbflip) runs the same stage ids, four of them
 * as NBFlipSolver's overrides (nbflipsolver.cpp):
 *   FS_STAGE_ADVECT          advect(): FlipSolver::advect, pruneNarrowBand, and
 *                            the semi-Lagrangian u, v, SDF and viscosity :66-109
 *   FS_STAGE_P2G             particleToGrid() with its centredParamsToGrid
 *                            (:445-504), fused with updateSdf(); no materials
 *   FS_STAGE_MATERIALS       updateMaterials(), which NB-FLIP runs after the
 *                            combination
 *   FS_STAGE_AFTER_TRANSFER  afterTransfer(): updateGridFromSources and
 *                            combineAdvectedGrids                       :111-116
 *   FS_STAGE_RESEED          reseedParticles(): band reseeding         :118-201
 * Its step (:26-64) is ADVECT, REBIN, P2G, VEL_EXTRAP, SAVE_GRID,
 * LEVELSET_OUTSIDE, AFTER_TRANSFER, LEVELSET, MATERIALS, BODY_FORCES,
 * DECOMPOSITION, PROJECT (+ FRICTION), VEL_EXTRAP, G2P, COUNT, RESEED. */

/* Grid ids for fs_get_grid / fs_set_grid.  c = NI*NJ, u = (NI+1)*NJ,
 * v = NI*(NJ+1) elements, row-major. */
enum {
    FS_GRID_MATERIAL = 0,         /* int8   c  MaterialGrid codes (materialgrid.h:6-13) */
    FS_GRID_SOLID_SDF = 1,        /* float  c  m_solidSdf */
    FS_GRID_FLUID_SDF = 2,        /* float  c  m_fluidSdf */
    FS_GRID_U = 3,                /* float  u  velocityGridU */
    FS_GRID_V = 4,                /* float  v  velocityGridV */
    FS_GRID_U_VALID = 5,          /* uint8  u  */
    FS_GRID_V_VALID = 6,          /* uint8  v  */
    FS_GRID_SAVED_U = 7,          /* float  u  m_savedFluidVelocityGrid */
    FS_GRID_SAVED_V = 8,          /* float  v  */
    FS_GRID_VISCOSITY = 9,        /* float  c  m_viscosityGrid */
    FS_GRID_KNOWN_CENTERED = 10,  /* uint8  c  m_knownCenteredParams */
    FS_GRID_DENSITY = 11,         /* float  c  m_densityGrid */
    FS_GRID_PARTICLE_COUNTS = 12, /* int32  c  m_fluidParticleCounts */
    FS_GRID_SOLID_ID = 13,        /* int32  c  m_solidId */
    FS_GRID_DIV_CONTROL = 14,     /* float  c  m_divergenceControl */
    FS_GRID_DENSITY_RHS = 15,     /* double c  m_pressureRhs */
    FS_GRID_DENSITY_PRESSURE = 16,/* double c  m_pressureSolverResult */
    FS_GRID_PRESSURE = 17,        /* double c  projection pressure */
    FS_GRID_PRESSURE_RHS = 18,    /* double c  projection right-hand side */
    FS_GRID_EMITTER_ID = 19,      /* int32  c  m_emitterId */
    FS_GRID_ADVECTED_U = 20,      /* float  u  NB-FLIP m_advectedVelocity (nbflipsolver.h:64) */
    FS_GRID_ADVECTED_V = 21,      /* float  v  */
    FS_GRID_ADVECTED_SDF = 22,    /* float  c  NB-FLIP m_advectedSdf (:65) */
    FS_GRID_ADVECTED_VISCOSITY = 23 /* float c NB-FLIP m_advectedViscosity (:63) */
};

enum {
    FS_STAT_DENSITY_ITERS = 0,  /* SolverStats::densityIterations()  */
    FS_STAT_PRESSURE_ITERS = 1, /* SolverStats::pressureIterations() */
    FS_STAT_SUBSTEPS = 2,       /* SolverStats::substepCount()       */
    FS_STAT_FRAME = 3,          /* FlipSolver::frameNumber()         */
    FS_STAT_POOL_THREADS = 4,   /* chunk count of the residual test  */
    FS_STAT_SUBSTEPS_TOTAL = 5, /* substeps since fs_create (no reference counterpart) */
    FS_STAT_VISCOSITY_ITERS = 6 /* SolverStats::viscosityIterations(): the model's return
                                   value of the last substep (-1: its solve failed) */
};

typedef struct fs_solver fs_solver;

const char *fs_status_string(fs_status s);
const char *fs_last_error(void);

/* FlipSolver::FlipSolver(const FlipSolverParameters*) (flipsolver2d.cpp:27-86)
 * followed by initAdditionalParameters() (:1613-1616).  exec may be NULL. */
fs_status fs_create(const fs_params *p, const fs_exec_params *exec, fs_solver **out);
/* NBFlipSolver::NBFlipSolver(const NBFlipParameters*) (nbflipsolver.cpp:9-24)
 * followed by initAdditionalParameters(); NBFlipParameters adds nothing to
 * FlipSolverParameters.  The handle takes every other call below; its
 * particle capacity is 2 particlesPerCell per cell.  fs_batch_add refuses it. */
fs_status fs_create_nbflip(const fs_params *p, const fs_exec_params *exec, fs_solver **out);
/* The solver's std::mt19937 (m_randEngine, flipsolver2d.h:371): 625 words,
 * the 624 state words then the index of the next one (0..624). */
fs_status fs_get_rng_state(fs_solver *s, uint32_t *state);
fs_status fs_set_rng_state(fs_solver *s, const uint32_t *state);
/* FlipSolver::~FlipSolver */
fs_status fs_destroy(fs_solver *s);

/* FlipSolver::addGeometry / addInitialFluid / addSink (flipsolver2d.cpp:602-620);
 * xy holds n (x, y) vertex pairs in scene units. */
fs_status fs_add_geometry(fs_solver *s, float friction, const float *xy, int n);
fs_status fs_add_initial_fluid(fs_solver *s, float viscosity, const float *xy, int n);
fs_status fs_add_sink(fs_solver *s, float divergence, const float *xy, int n);
/* FlipSolver::addSource (flipsolver2d.cpp:607-610) with an Emitter
 * (emitter.h): polygon in scene units, viscosity, divergence, velocity
 * (vx, vy) in scene units per second and whether it transfers velocity
 * (velocityTransfer).  Source cells reseed every substep
 * (reseedParticles, flipsolver2d.cpp:627-680; nbflipsolver.cpp:118-201).
 * Before fs_first_frame_init only; fs_batch_add refuses such a handle. */
fs_status fs_add_source(fs_solver *s, const float *xy, int n, float viscosity, float divergence,
                        float vx, float vy, int velocity_transfer);

/* FlipSolver::firstFrameInit (flipsolver2d.cpp:788-795) */
fs_status fs_first_frame_init(fs_solver *s);
/* FlipSolver::stepFrame (flipsolver2d.cpp:464-500) */
fs_status fs_step_frame(fs_solver *s);
/* FlipSolver::step (flipsolver2d.cpp:412-462) with the current step dt */
fs_status fs_step(fs_solver *s);
/* m_stepDt, set by stepFrame's CFL loop in the reference (:490) */
fs_status fs_set_step_dt(fs_solver *s, float dt);
fs_status fs_get_step_dt(fs_solver *s, float *dt);
/* one protected stage of step(), FS_STAGE_* */
fs_status fs_run_stage(fs_solver *s, int stage);
/* FlipSolver::maxParticleVelocity (flipsolver2d.cpp:1560-1574) */
fs_status fs_max_particle_velocity(fs_solver *s, float *out);

/* FlipSolver::particleCount / MarkerParticleSystem bins */
fs_status fs_particle_count(fs_solver *s, size_t *n);
fs_status fs_bin_count(fs_solver *s, size_t *n);
/* particles bin by bin in the reference's storage order; dead is set for
 * particles marked for death between FS_STAGE_ADVECT and FS_STAGE_REBIN */
fs_status fs_get_particles(fs_solver *s, int32_t *bin_counts, float *pos_xy, float *vel_xy,
                           float *visc, uint8_t *dead);
fs_status fs_set_particles(fs_solver *s, const int32_t *bin_counts, const float *pos_xy,
                           const float *vel_xy, const float *visc, const uint8_t *dead);

fs_status fs_grid_bytes(fs_solver *s, int which, size_t *bytes);
fs_status fs_get_grid(fs_solver *s, int which, void *out, size_t bytes);
fs_status fs_set_grid(fs_solver *s, int which, const void *in, size_t bytes);
fs_status fs_get_stat(fs_solver *s, int which, int *out);
/* Device memory the handle holds now, in bytes (no reference counterpart;
 * for admission by footprint). */
fs_status fs_device_bytes(fs_solver *s, size_t *bytes);

/* Device timing of the last fs_step / fs_step_frame calls, accumulated since
 * fs_reset_timers: which = 0 whole substeps, 1 PCG kernels, 2 launches
 * counted (as a float).  Times in milliseconds from CUDA events recorded on
 * the handle's stream. */
fs_status fs_enable_timers(fs_solver *s, int enable);
/* With timers on, fs_step / fs_step_frame also time the stage groups that
 * FlipSolver::step ends (flipsolver2d.cpp:412-462) with CUDA events; this
 * returns the accumulated milliseconds of one SolverStage
 * (flipsolver2d.h:58-72: 0 advection, 1 decomposition, 2 density,
 * 3 particle rebin, 4 particle to grid (fused into 5 here), 5 grid update,
 * 6 after transfer, 7 pressure, 8 viscosity and 9 repressure (always 0),
 * 10 particle update, 11 particle reseed).  The level set joins the main
 * stream while timed, so it counts in after transfer. */
fs_status fs_get_stage_time(fs_solver *s, int stage, double *ms);
fs_status fs_reset_timers(fs_solver *s);
fs_status fs_get_timer(fs_solver *s, int which, double *value);
/* the handle's cudaStream_t, as an opaque pointer */
fs_status fs_get_stream(fs_solver *s, void **stream);
fs_status fs_synchronize(fs_solver *s);

/* LinearSolver::solve (linearsolver.cpp:25-73) on the operator and IPP
 * coefficients that getPressureProjectionMatrix and getIPPCoefficients
 * (flipsolver2d.cpp:797-945) build from `material` (MaterialGrid codes,
 * ni*nj, row-major) with scale = dt / (density * dx * dx).  result is
 * overwritten (the reference assigns zeros first); *iterations receives the
 * reference's return value: the loop index at convergence, iter_limit on
 * failure, 0 for a zero right-hand side.  exec may be NULL. */
fs_status fs_pcg_solve(int ni, int nj, const int8_t *material, float dt, double density,
                       double dx, const double *rhs, double *result, int iter_limit,
                       double tol, const fs_exec_params *exec, int *iterations);

/* Same solve with every array already in device memory: material (int8),
 * rhs and result in FP32 (precision FS_PCG_FP32) or FP64 (FS_PCG_FP64).
 * Scratch comes from a per-device cache that grows on demand.  Runs on the
 * legacy default stream and returns after the solve completed. */
fs_status fs_pcg_solve_device(int ni, int nj, const int8_t *material_device, float dt,
                              double density, double dx, const void *rhs_device,
                              void *result_device, int iter_limit, double tol,
                              const fs_exec_params *exec, int *iterations);

/* LinearSolver::solve (linearsolver.cpp:25-73) on an operator given as its
 * rows rather than as a material grid: what IndexedPressureParameters and
 * IndexedIPPCoefficients hold (pressuredata.h:97-151,
 * PressureIPPCoeficients.h:11-47), one byte per cell:
 *   bit 7     the cell is a unit row (IndexedPressureParameterUnit)
 *   bits 4-6  its nonsolidNeighborCount (0..4); needed for every cell that
 *             neighbours a unit row, because the IPP coefficients are
 *             1 / (count(neighbour) * scale) (flipsolver2d.cpp:924-927)
 *   bits 0-3  fluidNeighborMask (NeighborMask: i-1, i+1, j-1, j+1); unit rows only
 * scale is IndexedPressureParameters' m_scale, dt / (density dx^2).  Host
 * arrays; precision, iterations and return convention as fs_pcg_solve. */
fs_status fs_pcg_solve_operator(int ni, int nj, const uint8_t *cell_info, double scale,
                                const double *rhs, double *result, int iter_limit, double tol,
                                const fs_exec_params *exec, int *iterations);

/* Spec mode: solve the same pressure system to a true relative residual,
 * ||rhs - A result|| <= rel_tol ||rhs|| (2-norms).  The reference's hot-path
 * PCG cannot do this (its IPP is not symmetric and the iteration stalls);
 * this uses the textbook incomplete-Poisson preconditioner the reference
 * ships but does not use (inversepoissonpreconditioner.h:45-79),
 * M = (I - L D^-1)(I - L D^-1)^T, in FP32 inner PCG iterations, with the
 * residual recomputed and the solution accumulated in FP64 between them
 * (iterative refinement).  max_iter caps the inner iterations in total;
 * *iterations receives their count and *rel_residual the final FP64
 * relative residual.  Host arrays as fs_pcg_solve; exec may be NULL. */
fs_status fs_pcg_solve_spec(int ni, int nj, const int8_t *material, float dt, double density,
                            double dx, const double *rhs, double *result, double rel_tol,
                            int max_iter, const fs_exec_params *exec, int *iterations,
                            double *rel_residual);

/* One system of fs_pcg_solve_batch: the problem of fs_pcg_solve_spec
 * (host arrays; result and the two outputs are written). */
typedef struct fs_poisson_system {
    int ni, nj;
    const int8_t *material; /* ni * nj material codes */
    float dt;
    double density, dx;
    const double *rhs;      /* ni * nj */
    double *result;         /* ni * nj, written */
    int iterations;         /* out: inner PCG iterations */
    double rel_residual;    /* out: ||rhs - A result|| / ||rhs|| (FP64) */
} fs_poisson_system;

/* Batched spec-mode solve, with no reference counterpart as a batch: every
 * system is the solve of fs_pcg_solve_spec (the reference's pressure
 * operator, LinearSolver::solve's problem, linearsolver.h:15-20, to a true
 * relative residual), and all of them run at once -- one thread-block cluster
 * per system, systems of one cluster size in one launch, every vector of the
 * iteration held on chip.  A system's result does not depend on the other
 * systems of the call.  A system larger than the on-chip limit (512 x 512
 * cells on GB300) is rejected with FS_ERR_BAD_ARG before any device work; a
 * system that does not reach rel_tol within max_iter inner iterations
 * returns its best result with its residual.  exec may be NULL. */
fs_status fs_pcg_solve_batch(fs_poisson_system *systems, int n, double rel_tol, int max_iter,
                             const fs_exec_params *exec);

/* A batch of solver handles stepped together; no reference counterpart as a
 * batch (each handle is a FlipSolver, flipsolver2d.h:183-432).  Members
 * advance by whole frames exactly as fs_step_frame would (FlipSolver::
 * stepFrame's CFL loop, flipsolver2d.cpp:464-500) and give the same results
 * bit for bit.  The members' substeps run in rounds: a round advances every
 * member that is inside a frame by one substep, each substep as captured
 * CUDA graphs, and the density and pressure solves of all of them -- plus
 * any standalone systems submitted -- share one cluster launch per plan.
 * Members must use FS_PCG_SPEC, sit on the batch's device and have timers
 * off.  The graphs hold each member's device buffers; they are captured
 * again when a frame starts on buffers that moved (first-frame seeding,
 * fs_set_particles).  Between frames a member may be read or stepped on its
 * own.  After an error the members' state is undefined.
 *
 * fs_batch_create   a batch of n members (n may be 0: the current device)
 * fs_batch_add / fs_batch_remove   membership (not while inside a frame)
 * fs_batch_begin_frame   start a frame of one member
 * fs_batch_round    one round; *busy = members still inside a frame
 * fs_batch_in_frame whether a member's frame is still running
 * fs_batch_step_frame   one whole frame of every member
 * fs_batch_run_frames   several frames of every member, pipelined
 * fs_batch_submit_solve   copy a standalone system (fs_pcg_solve_spec's
 *                   problem, host arrays, any size) to the device; the next
 *                   round solves it (in the merged launch up to the on-chip
 *                   limit of fs_pcg_solve_batch, as a chained cooperative
 *                   solve above it)
 * fs_batch_solve_done / fs_batch_take_solve   its completion; take copies
 *                   result, iterations and rel_residual out and frees it
 * fs_batch_destroy  frees the batch; the members stay alive */
typedef struct fs_batch fs_batch;
fs_status fs_batch_create(fs_solver *const *solvers, int n, fs_batch **out);
fs_status fs_batch_add(fs_batch *batch, fs_solver *solver);
fs_status fs_batch_remove(fs_batch *batch, fs_solver *solver);
fs_status fs_batch_begin_frame(fs_batch *batch, fs_solver *solver);
fs_status fs_batch_round(fs_batch *batch, int *busy);
fs_status fs_batch_in_frame(fs_batch *batch, fs_solver *solver, int *in_frame);
fs_status fs_batch_step_frame(fs_batch *batch);
/* `frames` whole frames of every member, pipelined: a member whose frame ends
 * starts its next one in the next round instead of waiting for the others
 * (each member's results are those of `frames` calls of fs_step_frame). */
fs_status fs_batch_run_frames(fs_batch *batch, int frames);
fs_status fs_batch_submit_solve(fs_batch *batch, const fs_poisson_system *system,
                                unsigned long long *ticket);
fs_status fs_batch_solve_done(fs_batch *batch, unsigned long long ticket, int *done);
fs_status fs_batch_take_solve(fs_batch *batch, unsigned long long ticket, fs_poisson_system *system);
fs_status fs_batch_destroy(fs_batch *batch);
/* Batch timing since creation or the last reset: which = 0 device time of
 * the merged solves (ms, CUDA events on the batch's solve stream), 1 host
 * wall time of the rounds (ms), 2 rounds run; 3 resets all three (and
 * writes 0). */
fs_status fs_batch_timer(fs_batch *batch, int which, double *value);

/* Autotuner of the FP32 solve's resident tile shape (no reference
 * counterpart): times every shape of one tile per SM for an ni x nj grid
 * (200 iterations of a synthetic fluid-in-a-box system, the best of three
 * host-timed solves) and records the fastest for this grid shape in the
 * process; handles created and FP32 solves run afterwards use it.  Results
 * depend on the tile shape in the last bits (the order of the sums), so a
 * process that needs reproducible FP32 bits tunes once, before its first
 * handle, or not at all.  Without a call the shape is the one with the
 * fewest cells per block including its ring.  Any output may be NULL. */
fs_status fs_resident_autotune(int ni, int nj, int device, int *tile_rows, int *tile_cols,
                               float *us_per_iteration);

/* A device-resident request loop for spec-mode solves (no reference
 * counterpart; each request is the problem of fs_pcg_solve_spec, solved by the
 * cluster solve of fs_pcg_solve_batch).  One persistent launch keeps running
 * while requests arrive: its thread-block clusters take requests from a ring
 * the host fills in mapped pinned memory and flag each result there, so a
 * request needs no launch and no host synchronisation with the device.  The
 * launch leaves after about 50 ms without requests; the next submit or poll
 * starts another.  While it runs it holds the SMs its clusters fit on, so
 * other work on the device waits for it to leave.
 *   fs_server_create: systems up to max_ni x max_nj (within the on-chip limit
 *     of fs_pcg_solve_batch, else FS_ERR_BAD_ARG), `slots` requests in flight,
 *     every solve to rel_tol within max_iter inner iterations.
 *   fs_server_submit: copies the system's material, rhs and dt to a free slot
 *     and queues it; FS_ERR_STATE when every slot holds a request not yet
 *     taken.  system->result is not used; the call returns a ticket.
 *   fs_server_poll: *done = 1 once the ticket's result is in device memory.
 *   fs_server_take: copies the result, the inner iterations and the final
 *     relative residual (any may be NULL but result) and frees the slot;
 *     FS_ERR_STATE before the request is done.
 *   fs_server_clusters: clusters of the last launch (requests solved at once).
 *   fs_server_destroy: stops the loop after the requests being solved; requests
 *     not yet taken by a cluster are dropped.
 * Calls on one server are serialised by a lock; results do not depend on the
 * other requests or on the order of arrival. */
typedef struct fs_server fs_server;
fs_status fs_server_create(int device, int max_ni, int max_nj, int slots, double rel_tol, int max_iter,
                           fs_server **server);
fs_status fs_server_submit(fs_server *server, const fs_poisson_system *system, unsigned long long *ticket);
fs_status fs_server_poll(fs_server *server, unsigned long long ticket, int *done);
fs_status fs_server_take(fs_server *server, unsigned long long ticket, double *result, int *iterations,
                         double *rel_residual);
fs_status fs_server_clusters(fs_server *server, int *clusters);
fs_status fs_server_destroy(fs_server *server);

/* Autotuner of the cluster solve (no reference counterpart): times every
 * cluster size that fits an ni x nj system (64 inner iterations on a
 * synthetic fluid-in-a-box system, CUDA events) and records the best for
 * this shape in the process.  objective 0 minimises SM time per iteration
 * (throughput: batches), 1 the time per iteration (latency: one system
 * alone).  Every later plan of that shape uses the choice: FS_PCG_SPEC
 * handles created afterwards, fs_pcg_solve_batch and batch solves -- so tune
 * before creating the handles that should share a plan.  *clusters receives
 * the chosen CTAs per cluster, *us_per_iteration its time per iteration
 * (either may be NULL). */
fs_status fs_cluster_autotune(int ni, int nj, int objective, int device, int *clusters,
                              float *us_per_iteration);

/* fs_pcg_solve_device without any device allocation.  This entry point has
 * no counterpart in the reference.  It is for callers that cannot allocate
 * device memory while they run: a loop that reserved its whole device budget
 * at start-up, or one that cannot take the device synchronisation that
 * cudaMalloc / cudaFree may cause while its other streams are busy.  The
 * solve (FP32 only; rhs and result are float arrays) uses one fixed scratch
 * array compiled into the library instead of the growing cache.
 * Limits: ni * nj <= 262144 cells (512 x 512) and at most 4096 pool threads;
 * larger requests fail with FS_ERR_BAD_ARG before any device work, and
 * pcg_precision FS_PCG_FP64 fails with FS_ERR_UNSUPPORTED.
 * The first call on a device looks up the scratch array's address on that
 * device; make that first call before any stream capture begins.  The address
 * is kept for the life of the process: calls after a reset of that device
 * (cudaDeviceReset) are not supported.  All calls
 * share the array and it keeps what the last call left in it (each call
 * clears what must start at zero).  Calls that overlapped on the GPU would
 * race on it: the function holds a process-wide lock, runs on the legacy
 * default stream and returns after its solve finished, so its own calls do
 * not overlap. */
fs_status fs_pcg_solve_device_noalloc(int ni, int nj, const int8_t *material_device, float dt,
                                      double density, double dx, const float *rhs_device,
                                      float *result_device, int iter_limit, double tol,
                                      const fs_exec_params *exec, int *iterations);

#ifdef __cplusplus
}
#endif

#endif /* FS_GPU_H */
