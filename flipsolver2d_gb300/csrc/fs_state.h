// fs_state.h -- device-resident state of one FLIP scene and the launch
// interface between the host driver (fs_api.cu) and the kernel files.
//
// HBM layout (all arrays row-major, linear index i*NJ + j as in
// linearindexable2d.h:30-37):
//   particles  bin-CSR: bin b owns slots [bin_start[b], bin_start[b] + bin_count[b]);
//              slots past bin_count[b] up to bin_start[b+1] are gaps left by
//              countParticles erasures.  pos/vel are float2 (the reference's
//              Vec3 z component is always 0), visc float.  Within a bin the
//              slots are in the reference's ParticleBin storage order.
//   cell grids NI*NJ: material (int8), solid/fluid SDF, viscosity, density
//              (float), known-centred / counts / solid id, cell_info (u8 packed
//              pressure-operator row, see fs_grid.cu).
//   face grids U (NI+1)*NJ and V NI*(NJ+1) float + u8 validity, current and
//              saved copies.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "fs_common.cuh"

namespace fsg {

struct SceneParams {
    double fluidDensity;
    double dx;
    int particlesPerCell;
    float gI, gJ;
    float picRatio;
    float particleScale;
    int pcgIterLimit;
    int parameterHandlingMethod;
    int viscosityEnabled;
    double projectTolerance; // flipsolver2d.cpp:73
};

struct Particles {
    float2 *pos = nullptr, *vel = nullptr;
    float *visc = nullptr;
    int *slot_bin = nullptr;
    float2 *pos2 = nullptr, *vel2 = nullptr;
    float *visc2 = nullptr;
    int *slot_bin2 = nullptr;
    uint8_t *flag = nullptr;   // P_STAY / P_MOVE / P_KILL / P_GAP after advection
    int *dest = nullptr;       // destination bin of a moved particle
    int *prune_slot = nullptr; // slot inside its bin after the swap-erase prune
    int *bin_start = nullptr;  // nbins + 1
    int *bin_count = nullptr;  // nbins
    int *bin_start2 = nullptr, *bin_count2 = nullptr;
    int *survivors = nullptr, *incoming = nullptr, *inc_off = nullptr; // nbins (+1)
    int *mkey = nullptr, *mval = nullptr, *mkey2 = nullptr, *mval2 = nullptr; // moved list
    int *nmoved = nullptr;     // device scalar
    int cap = 0;               // slot capacity
    int bound = 0;             // launch bound for per-slot kernels: >= the occupied slots
                               // (the capacity, or NB-FLIP's count read at each substep)
    int nbins = 0;
};

struct Grids {
    int8_t *material = nullptr;
    float *solid_sdf = nullptr;
    int *solid_id = nullptr;
    float *fluid_sdf = nullptr;
    float *u = nullptr, *v = nullptr;
    uint8_t *uvalid = nullptr, *vvalid = nullptr;
    float *u2 = nullptr, *v2 = nullptr; // extrapolation output buffers
    uint8_t *uvalid2 = nullptr, *vvalid2 = nullptr;
    float *su = nullptr, *sv = nullptr; // saved grid (flipsolver2d.cpp:439)
    uint8_t *suvalid = nullptr, *svvalid = nullptr;
    float *visc = nullptr;
    uint8_t *known = nullptr;
    float *divc = nullptr;
    float *density = nullptr;
    int *counts = nullptr;
    uint8_t *cell_info = nullptr; // pressure-operator rows frozen at DECOMPOSITION
    float *ufric = nullptr, *vfric = nullptr; // 1 - mean friction, or NaN when not affected
    int *emitter_id = nullptr;
    unsigned long long *levelset_cells = nullptr; // packed (marker, value) per cell
    uint8_t *levelset_act = nullptr;  // 3 x tiles activity flags (pass ring)
    int *levelset_active = nullptr;   // per pass: any cell assigned
};

// scratch scalars living in device memory
struct Scalars {
    float dt;              // m_stepDt of the running substep
    unsigned int maxv2;    // float bits of max |v|^2 (atomicMax on bits)
    int density_iters;     // LinearSolver::solve return values
    int pressure_iters;
    int pcg_status;        // 0 ok, 1 a grid-barrier wait timed out
    int wrap_units;        // a unit row lies on the j = 0 or j = NJ-1 edge
    int nb_overflow;       // NB-FLIP reseeding: more bin-crossing candidates than kept
    int nonfinite;         // a particle velocity of a substep was NaN or infinite
};

// NB-FLIP (nbflipsolver.h:63-66): the grids advected semi-Lagrangian each
// substep, same shapes as U, V and the cell grids
struct NbGrids {
    float *adv_u = nullptr, *adv_v = nullptr, *adv_sdf = nullptr, *adv_visc = nullptr;
};

// an Emitter's parameters (emitter.h) as the liquid solvers read them;
// velocity in scene units per second
struct SourceParams {
    float visc, div, vx, vy;
    int transfer, pad[3];
};
struct Sources {
    const SourceParams *p = nullptr; // device, n entries
    int n = 0;
    const float *xy = nullptr;       // device polygon vertices (the scene's)
    const int *off = nullptr;        // vertex offsets per source polygon (n + 1)
};

// reseeding scratch (NB-FLIP's band, or FLIP's source cells); candidates are
// numbered in the reference's order (row-major cell, then draw)
constexpr int kNbCrossMax = 1 << 16; // candidates whose position left their cell's bin
struct NbReseed {
    uint32_t *rng = nullptr;   // std::mt19937 state: 624 words, next index
    int *cand_n = nullptr;     // ncell: candidates per cell
    int *cand_off = nullptr;   // ncell + 1: first candidate per cell, total at [ncell]
    float *draws = nullptr;    // 2 per candidate
    float2 *cand_pos = nullptr;
    float2 *cand_vel = nullptr;
    float *cand_visc = nullptr;
    int *cand_bin = nullptr;   // bin of the position, -1 when not kept
    int *cand_cb = nullptr;    // bin of the cell
    int *pos_of = nullptr;     // rank in the sorted list of kept candidates
    int *cross = nullptr;      // kNbCrossMax
    int *cross_n = nullptr;
    int *status = nullptr;     // 1 when more than kNbCrossMax crossed bins
    int ncell = 0;
};

// launch helpers implemented in the kernel files
void launch_advect(const GridDims &d, const Particles &P, const Grids &G, const Scalars *sc,
                   cudaStream_t st);
void launch_rebin(const GridDims &d, Particles &P, void *scratch, size_t scratch_bytes,
                  cudaStream_t st);
size_t rebin_scratch_bytes(const Particles &P);
// fs_get_particles: pack the particles in bin order into pos2 / vel2 / visc2,
// offsets in bin_start2 (scratch: the rebin scratch); fs_set_particles: the
// bin of every occupied slot from bin_start / bin_count
void launch_gather_bins(const Particles &P, void *scratch, cudaStream_t st);
void launch_slot_bin(const Particles &P, cudaStream_t st);
void launch_adjust(const GridDims &d, const SceneParams &sp, const Particles &P, const Grids &G,
                   const void *pressure, int pressure_is_double, const Scalars *sc,
                   cudaStream_t st);
void launch_g2p(const GridDims &d, const SceneParams &sp, const Particles &P, const Grids &G,
                Scalars *sc,
                cudaStream_t st);
void launch_count_erase(const GridDims &d, const SceneParams &sp, Particles &P, const Grids &G,
                        cudaStream_t st);
void launch_max_velocity(const Particles &P, Scalars *sc, cudaStream_t st);

// the pressure-operator rows plus, per splitRange chunk of the reference's
// max-abs test (ps cells per chunk, the first `rem` chunks one more), the
// last unit row of the chunk
void launch_decomposition(const GridDims &d, const Grids &G, int *chunk_last, int nchunks,
                          long long ps, long long rem, Scalars *sc, cudaStream_t st);
void launch_density_grid(const GridDims &d, const SceneParams &sp, const Particles &P,
                         const Grids &G, void *rhs, int rhs_is_double, const Scalars *sc,
                         cudaStream_t st);
// nb: NB-FLIP's centred weights, and no material update (it follows the
// grid combination there)
void launch_p2g_sdf_materials(const GridDims &d, const SceneParams &sp, const Particles &P,
                              const Grids &G, bool nb, cudaStream_t st);
// extrapolateLevelsetInside, or with `outside` extrapolateLevelsetOutside
// status (may be null): with it, and when every tile fits on the device at
// once, all passes run in one cooperative launch whose grid-barrier timeouts
// set *status; spin_limit: polls before a barrier wait gives up (0: default)
void launch_levelset(const GridDims &d, Grids &G, bool outside, cudaStream_t st, int *status = nullptr,
                     long long spin_limit = 0);
int levelset_launches(const GridDims &d, bool with_status); // kernels one launch_levelset enqueues
void launch_vel_extrapolate(const GridDims &d, Grids &G, const SceneParams &sp,
                            const Scalars *sc, bool save_and_gravity, cudaStream_t st);
void launch_pressure_rhs(const GridDims &d, const Grids &G, void *rhs, int rhs_is_double,
                         const SceneParams &sp, cudaStream_t st);
void launch_apply_pressure(const GridDims &d, const SceneParams &sp, const Grids &G,
                           const void *pressure, int pressure_is_double, const Scalars *sc,
                           bool with_friction, cudaStream_t st);
void launch_friction(const GridDims &d, const Grids &G, cudaStream_t st);
void launch_save_grid(const GridDims &d, const Grids &G, cudaStream_t st);
void launch_body_forces(const GridDims &d, const SceneParams &sp, const Grids &G,
                        const Scalars *sc, cudaStream_t st);
int levelset_max_passes(const GridDims &d);
// sinks, solids and the initial fluid; with `nb` the initial fluid sets the
// fluid SDF as NBFlipSolver::fluidSdfFromInitialFluid does and clears counts
// (poly_kind 0 solid, 1 initial fluid, 2 sink, 3 source; poly_val the
// friction, viscosity, divergence or divergence)
void launch_scene_classify(const GridDims &d, const Grids &G, float dx, const float *poly_xy,
                           const int *poly_off, const int *poly_kind, const float *poly_val,
                           int npoly, bool nb, cudaStream_t st);
void launch_friction_factors(const GridDims &d, const Grids &G, const float *obst_friction,
                             cudaStream_t st);
void launch_fill_u8(uint8_t *p, uint8_t v, size_t n, cudaStream_t st);

// NB-FLIP (fs_nbflip.cu, fs_particles.cu)
void mt_seed_host(uint32_t *state, uint32_t seed);
void mt_discard_host(uint32_t *state, unsigned long long n);
void launch_mt_draws(uint32_t *state, float *out, const int *count, int per, cudaStream_t st);
// narrow-band pruning after advection, then the four semi-Lagrangian grids
void launch_nb_advect_extra(const GridDims &d, const SceneParams &sp, const Particles &P,
                            const Grids &G, const NbGrids &N, const Scalars *sc, cudaStream_t st);
// FlipSolver::afterTransfer's source cells; with NB-FLIP also
// updateGridFromSources and combineAdvectedGrids
void launch_sources_after_transfer(const GridDims &d, const Grids &G, const Sources &S, double dx,
                                   cudaStream_t st);
void launch_nb_combine(const GridDims &d, const Grids &G, const NbGrids &N, const Sources &S,
                       double dx, cudaStream_t st);
void launch_nb_materials(const GridDims &d, const Grids &G, cudaStream_t st);
// nb: NB-FLIP's band and source cells, else FlipSolver::reseedParticles'
// source cells
void launch_nb_candidates(const GridDims &d, const SceneParams &sp, const Grids &G,
                          const NbReseed &R, const Sources &S, bool nb, void *scan_scratch,
                          cudaStream_t st);
// ncand: the candidate total of launch_nb_candidates, read back by the host
void launch_nb_append(Particles &P, const NbReseed &R, int ncand, void *scratch,
                      cudaStream_t st);

// exclusive scan of n ints (out may alias nothing); writes the total to out[n]
size_t scan_scratch_bytes(int n);
void scan_exclusive(const int *in, int *out, int n, void *scratch, cudaStream_t st);

} // namespace fsg
