/*
 * fsoracle.h -- C interface shared by the two CPU oracles of the FLIP substep.
 *
 * TEST INFRASTRUCTURE.  Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline / reference arm may load these libraries, and only as the
 * checker or the timed CPU baseline; the product (flipsolver2d_gb300) never
 * links or calls them.
 *
 * Two libraries export exactly this interface:
 *   - oracle/_ref/libfsref.so    : the reference FlipSolver2d compiled from its
 *                                  own sources (FlipSolver2dLib, .cpp files) plus
 *                                  ref_harness.cpp, which drives it through its
 *                                  C++ API.  Buildable only where the reference
 *                                  sources are present.
 *   - oracle/_build/libfsoracle.so : fsoracle.c, a plain-C restatement of the
 *                                  same algorithm, built everywhere.  It is
 *                                  pinned bit-for-bit against libfsref.so and
 *                                  against the committed golden fixtures.
 *
 * Units follow the reference: positions in cell units (i + U(0,1),
 * flipsolver2d.cpp:1013-1019), velocities in cells/s, linear index
 * i*gridSizeJ + j (linearindexable2d.h:30-37).
 */
#ifndef FSORACLE_H
#define FSORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Field-for-field mirror of FlipSolverParameters (flipsolver2d.h:33-56). */
typedef struct fso_params {
    double fluidDensity;
    unsigned int seed;
    double dx;
    int particlesPerCell;
    float globalAccelerationI; /* Vec3::x() of globalAcceleration */
    float globalAccelerationJ; /* Vec3::y() */
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
    int viscosityEnabled;
    int useHeavyViscosity;
    int simulationMethod;        /* 0 = SIMULATION_LIQUID */
    int parameterHandlingMethod; /* 0 = PARTICLE, 1 = HYBRID, 2 = GRID */
} fso_params;

/* Stages of FlipSolver::step() (flipsolver2d.cpp:412-462), in call order. */
enum fso_stage {
    FSO_ADVECT = 0,        /* advect()                                   :414 */
    FSO_DECOMPOSITION = 1, /* getPressureProjectionMatrix + IPP          :417-418 */
    FSO_REBIN = 2,         /* pruneParticles + rebinParticles            :421-422 */
    FSO_DENSITY = 3,       /* densityCorrection()                        :428 */
    FSO_P2G = 4,           /* particleToGrid()                           :1207 */
    FSO_SDF = 5,           /* updateSdf()                                :1209 */
    FSO_MATERIALS = 6,     /* updateMaterials()                          :1210 */
    FSO_AFTER_TRANSFER = 7,/* afterTransfer()                            :435 */
    FSO_LEVELSET = 8,      /* extrapolateLevelsetInside(m_fluidSdf)      :436 */
    FSO_VEL_EXTRAP = 9,    /* m_fluidVelocityGrid.extrapolate(10)        :437, :455 */
    FSO_SAVE_GRID = 10,    /* m_savedFluidVelocityGrid = m_fluidVelocityGrid :439 */
    FSO_BODY_FORCES = 11,  /* applyBodyForces()                          :440 */
    FSO_PROJECT = 12,      /* project()                                  :444 */
    FSO_FRICTION = 13,     /* updateVelocityFromSolids()                 :447 */
    FSO_G2P = 14,          /* particleUpdate()                           :456 */
    FSO_COUNT = 15,        /* countParticles()                           :459 */
    FSO_RESEED = 16,       /* reseedParticles()                          :460 */
    FSO_DENSITY_GRID = 17, /* updateDensityGrid() alone                  :166 */
    FSO_LEVELSET_OUTSIDE = 18, /* extrapolateLevelsetOutside(m_fluidSdf)  :1496-1558 */
    FSO_VISCOSITY = 19,    /* applyViscosity(): the light or heavy model :128-136 */
    FSO_STAGE_COUNT = 20
};

/* NB-FLIP (NBFlipSolver, nbflipsolver.cpp) runs the same stage ids; four of
 * them are its overrides:
 *   FSO_ADVECT          NBFlipSolver::advect: FlipSolver::advect, then
 *                       pruneNarrowBand and the semi-Lagrangian advection of
 *                       u, v, the fluid SDF and the viscosity     :66-109, 227-253
 *   FSO_P2G             particleToGrid with NBFlipSolver::centeredParamsToGrid
 *                                                                  :445-504
 *   FSO_AFTER_TRANSFER  FlipSolver::afterTransfer, updateGridFromSources,
 *                       combineAdvectedGrids                       :111-116, 332-427
 *   FSO_RESEED          NBFlipSolver::reseedParticles              :118-201
 * and its step (:26-64) is advect, rebin, P2G, extrapolation, saved grid,
 * SDF, outside level set, after transfer, inside level set, materials, body
 * forces, decomposition, projection, friction, extrapolation, G2P, count,
 * reseed. */

/* Grids that can be read and written. */
enum fso_grid {
    FSO_G_MATERIAL = 0,        /* int8   NI*NJ     MaterialGrid          */
    FSO_G_SOLID_SDF = 1,       /* float  NI*NJ     m_solidSdf            */
    FSO_G_FLUID_SDF = 2,       /* float  NI*NJ     m_fluidSdf            */
    FSO_G_U = 3,               /* float  (NI+1)*NJ velocityGridU         */
    FSO_G_V = 4,               /* float  NI*(NJ+1) velocityGridV         */
    FSO_G_U_VALID = 5,         /* uint8  (NI+1)*NJ uSampleValidity       */
    FSO_G_V_VALID = 6,         /* uint8  NI*(NJ+1) vSampleValidity       */
    FSO_G_SAVED_U = 7,         /* float  (NI+1)*NJ saved grid U          */
    FSO_G_SAVED_V = 8,         /* float  NI*(NJ+1) saved grid V          */
    FSO_G_VISCOSITY = 9,       /* float  NI*NJ     m_viscosityGrid       */
    FSO_G_KNOWN_CENTERED = 10, /* uint8  NI*NJ     m_knownCenteredParams */
    FSO_G_DENSITY = 11,        /* float  NI*NJ     m_densityGrid         */
    FSO_G_PARTICLE_COUNTS = 12,/* int32  NI*NJ     m_fluidParticleCounts */
    FSO_G_SOLID_ID = 13,       /* int32  NI*NJ     m_solidId             */
    FSO_G_DIV_CONTROL = 14,    /* float  NI*NJ     m_divergenceControl   */
    FSO_G_DENSITY_RHS = 15,    /* double NI*NJ     m_pressureRhs         */
    FSO_G_DENSITY_PRESSURE = 16,/* double NI*NJ    m_pressureSolverResult*/
    FSO_G_PRESSURE = 17,       /* double NI*NJ     projection pressure   */
    FSO_G_PRESSURE_RHS = 18,   /* double NI*NJ     projection RHS        */
    FSO_G_EMITTER_ID = 19,     /* int32  NI*NJ     m_emitterId           */
    FSO_G_ADVECTED_U = 20,     /* float  (NI+1)*NJ NB-FLIP m_advectedVelocity U */
    FSO_G_ADVECTED_V = 21,     /* float  NI*(NJ+1) NB-FLIP m_advectedVelocity V */
    FSO_G_ADVECTED_SDF = 22,   /* float  NI*NJ     NB-FLIP m_advectedSdf       */
    FSO_G_ADVECTED_VISCOSITY = 23, /* float NI*NJ  NB-FLIP m_advectedViscosity */
    FSO_G_COUNT = 24
};

enum fso_stat {
    FSO_S_DENSITY_ITERS = 0,   /* iterations of the last density solve    */
    FSO_S_PRESSURE_ITERS = 1,  /* iterations of the last pressure solve   */
    FSO_S_SUBSTEPS = 2,        /* substeps of the last stepFrame          */
    FSO_S_FRAME = 3,           /* frame number                            */
    FSO_S_POOL_THREADS = 4,    /* chunk count used by the vector kernels  */
    FSO_S_VISCOSITY_ITERS = 5  /* the viscosity model's return value      */
};

typedef struct fso_solver fso_solver;

fso_solver *fso_create(const fso_params *p);
/* NBFlipSolver(const NBFlipParameters *) (nbflipsolver.cpp:9-23);
 * NBFlipParameters adds nothing to FlipSolverParameters. */
fso_solver *fso_create_nbflip(const fso_params *p);
void fso_destroy(fso_solver *s);

/* The solver's std::mt19937 (m_randEngine, flipsolver2d.h:371): the 624
 * state words and the position of the next word, in this order. */
int fso_get_rng(fso_solver *s, uint32_t state[625]);
int fso_set_rng(fso_solver *s, const uint32_t state[625]);

/* Scene objects; vertices are (x, y) pairs in scene units (metres). */
int fso_add_geometry(fso_solver *s, float friction, const float *xy, int n);
int fso_add_initial_fluid(fso_solver *s, float viscosity, const float *xy, int n);
int fso_add_sink(fso_solver *s, float divergence, const float *xy, int n);
/* FlipSolver::addSource (flipsolver2d.cpp:607-610) with an Emitter
 * (emitter.h) of these parameters; velocity in scene units per second. */
int fso_add_source(fso_solver *s, const float *xy, int n, float viscosity, float divergence,
                   float vx, float vy, int velocity_transfer);

void fso_first_frame_init(fso_solver *s);
void fso_step_frame(fso_solver *s);
void fso_set_step_dt(fso_solver *s, float dt);
float fso_step_dt(fso_solver *s);
void fso_step(fso_solver *s);
int fso_run_stage(fso_solver *s, int stage);
float fso_max_particle_velocity(fso_solver *s);

size_t fso_bin_count(fso_solver *s);
size_t fso_particle_count(fso_solver *s);
/* Particles bin by bin, in each bin's storage order. */
void fso_get_particles(fso_solver *s, int32_t *bin_counts, float *pos_xy,
                       float *vel_xy, float *visc, uint8_t *dead);
void fso_set_particles(fso_solver *s, const int32_t *bin_counts,
                       const float *pos_xy, const float *vel_xy,
                       const float *visc, const uint8_t *dead);

size_t fso_grid_bytes(fso_solver *s, int which);
int fso_get_grid(fso_solver *s, int which, void *out);
int fso_set_grid(fso_solver *s, int which, const void *in);
int fso_stat(fso_solver *s, int which);

/* LinearSolver::solve (linearsolver.cpp:25-73) on the operator and IPP
 * coefficients that getPressureProjectionMatrix / getIPPCoefficients
 * (flipsolver2d.cpp:797-945) build from `material` with
 * scale = dt / (density * dx * dx).  Returns the solver's iteration count. */
int fso_pcg_solve(int ni, int nj, const int8_t *material, float dt,
                  double density, double dx, const double *rhs, double *result,
                  int iter_limit, double tol);

/* Spec-mode oracle: full-FP64 PCG with the reference's textbook incomplete-
 * Poisson preconditioner (inversepoissonpreconditioner.h:45-79) on the same
 * operator, stopped at ||b - A x|| <= rel_tol ||b||.  Returns the iteration
 * count; *rel_residual receives the final true relative residual. */
int fso_spec_solve(int ni, int nj, const int8_t *material, float dt, double density, double dx,
                   const double *rhs, double *result, double rel_tol, int max_iter,
                   double *rel_residual);

/* std::thread::hardware_concurrency() of this host (glibc get_nprocs) */
int fso_hardware_concurrency(void);

#ifdef __cplusplus
}
#endif

#endif
