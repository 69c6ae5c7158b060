// fs_api.cu -- host driver of the GB300 FLIP substep and the C ABI of
// include/fs_gpu.h.
//
// One handle = one scene resident in HBM (fs_state.h) plus one CUDA stream.
// FlipSolver::step() (flipsolver2d.cpp:412-462) becomes a fixed sequence of
// kernel launches on that stream; the level-set extrapolation, whose result no
// later stage of the substep reads, runs on a second stream and overlaps the
// rest.  FlipSolver::stepFrame() keeps the reference's host-side CFL loop
// (:464-500): one 32-byte device-to-host read per substep brings back the
// maximum particle speed and the two solvers' iteration counts.
//
// Scene setup (frame 0) classifies cells on the GPU and seeds particles on the
// host with std::mt19937 + std::uniform_real_distribution<float>, the same
// generator and distribution the reference draws from
// (flipsolver2d.cpp:71, 1013-1019), so initial particles are bit-identical.
#include <algorithm>
#include <atomic>
#include <cfloat>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <random>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "../../include/fs_gpu.h"
#include "fs_cluster.h"
#include "fs_pcg.h"
#include "fs_pcg_tma.h"
#include "fs_spec.h"
#include "fs_state.h"
#include "fs_viscosity.h"

using namespace fsg;

namespace fsg {
std::atomic<long long> g_kernel_launches{0};
}

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------
// FS_PCG_SPEC: the relative residual every pressure and density solve
// reaches, and its inner-iteration cap (a solve that hits it counts as
// failed, like the reference's iteration limit)
constexpr double kSpecRelTol = 1e-6;
constexpr int kSpecMaxIter = 20000;
constexpr int kSpecMaxOuter = 12; // refinements of a chained solve (2 or 3 are typical)

static thread_local std::string t_last_error;

static fs_status fail(fs_status st, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    t_last_error = buf;
    return st;
}

#define CK(call)                                                                                   \
    do {                                                                                           \
        cudaError_t _e = (call);                                                                   \
        if (_e != cudaSuccess) {                                                                   \
            if (_e == cudaErrorMemoryAllocation)                                                   \
                return fail(FS_ERR_OOM, "%s: %s (%s:%d)", #call, cudaGetErrorString(_e), __FILE__, \
                            __LINE__);                                                             \
            return fail(FS_ERR_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(_e), __FILE__,    \
                        __LINE__);                                                                 \
        }                                                                                          \
    } while (0)

#define TRY(expr)                                                                                  \
    do {                                                                                           \
        fs_status _s = (expr);                                                                     \
        if (_s != FS_OK) return _s;                                                                \
    } while (0)

extern "C" const char *fs_status_string(fs_status s)
{
    switch (s) {
    case FS_OK: return "ok";
    case FS_ERR_BAD_ARG: return "bad argument";
    case FS_ERR_CUDA: return "CUDA error";
    case FS_ERR_OOM: return "out of device memory";
    case FS_ERR_TIMEOUT: return "device wait timed out";
    case FS_ERR_UNSUPPORTED: return "unsupported";
    case FS_ERR_STATE: return "invalid state";
    case FS_ERR_NONFINITE: return "non-finite value";
    }
    return "unknown";
}

extern "C" const char *fs_last_error(void) { return t_last_error.c_str(); }

// ---------------------------------------------------------------------------
// ThreadPool::splitRange (threadpool.cpp:41-76): the chunk ends of the
// reference's max-abs residual test
// ---------------------------------------------------------------------------
static std::vector<int> split_range_ends(long long length, long long parts)
{
    std::vector<int> ends;
    if (length == 0) return ends;
    long long numParts = parts < 1 ? 1 : parts;
    if (length < numParts) numParts = length;
    long long partSize = length / numParts;
    if (partSize < 1) partSize = 1;
    long long remainder = 0;
    if (partSize * numParts < length) remainder = length - partSize * numParts;
    long long cs = 0, ce = std::min(partSize, length);
    for (long long i = 0; i < numParts; i++) {
        if (i < remainder) ce++;
        ends.push_back((int)ce);
        cs = ce;
        ce = std::min(cs + partSize, length);
        if (ce == cs) break;
    }
    return ends;
}

static void split_range_params(long long length, long long parts, long long *ps, long long *rem)
{
    long long numParts = parts < 1 ? 1 : parts;
    if (length < numParts) numParts = length;
    if (numParts < 1) numParts = 1;
    long long partSize = length / numParts;
    if (partSize < 1) partSize = 1;
    *ps = partSize;
    *rem = partSize * numParts < length ? length - partSize * numParts : 0;
}

static int default_pool_threads()
{
    unsigned n = std::thread::hardware_concurrency();
    return n ? (int)n : 1;
}

// ---------------------------------------------------------------------------
// handle
// ---------------------------------------------------------------------------
struct Poly {
    int kind; // 0 solid, 1 initial fluid, 2 sink
    float value;
    std::vector<float> xy;
};

__global__ void k_set_dt(Scalars *sc, float dt) { sc->dt = dt; }
// a batch round: the scene's dt from the batch's table
__global__ void k_set_dt_from(Scalars *sc, const float *dt) { sc->dt = *dt; }
__global__ void k_fill_i32(int *p, int v, size_t n)
{
    size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) p[k] = v;
}

struct fs_solver {
    fs_params p{};
    fs_exec_params ex{};
    GridDims d{};
    SceneParams sp{};
    Particles P;
    Grids G;
    Scalars *sc = nullptr;      // device
    Scalars *sc_host = nullptr; // pinned mirror
    int prec = FS_PCG_FP32;
    size_t esz = 4;
    size_t ncell = 0, nu = 0, nv = 0;
    void *dens_rhs = nullptr, *dens_x = nullptr, *pres_rhs = nullptr, *pres_x = nullptr;
    void *r0 = nullptr, *r1 = nullptr, *s0 = nullptr, *s1 = nullptr;
    double *partials = nullptr;
    int pcg_grid = 0;
    int *chunk_end = nullptr, *chunk_last = nullptr;
    double *chunk_val = nullptr;
    int nchunks = 0;
    long long chunk_ps = 1, chunk_rem = 0; // splitRange part size and remainder
    GridBarrier *bar = nullptr;
    bool tma = false;          // TMA-staged FP32 PCG available for this grid
    int tma_ti = 0, tma_tj = 0;
    bool resident = false;     // FP32 PCG with every tile resident in shared memory
    LlBuffers ll;              // the resident PCG's exchange words
    ClusterPlan spec_plan{};   // FS_PCG_SPEC: how the cluster solve runs this grid
    ClusterSystem *spec_sys = nullptr; // FS_PCG_SPEC: the density and pressure systems
    double *spec_rel = nullptr;        // their final relative residuals
    bool spec_large = false;           // FS_PCG_SPEC above the on-chip limit: chained
    SpecSolve spec_chain[2] = {};      // cooperative solves (density, pressure)
    int res_ti = 0, res_tj = 0;
    TmaMaps maps_dens{}, maps_pres{};
    void *rebin_scratch = nullptr;
    size_t rebin_scratch_size = 0;
    cudaStream_t st = nullptr, side = nullptr;
    cudaEvent_t ev_p2g = nullptr, ev_levelset = nullptr;
    bool levelset_pending = false;
    std::vector<Poly> polys;
    std::vector<float> obst_friction;
    float *d_obst_friction = nullptr;
    bool friction_dirty = true;
    std::mt19937 rng; // m_randEngine (flipsolver2d.cpp:71), persists across calls
    bool nb = false;  // NBFlipSolver (nbflipsolver.cpp); its engine state lives in R.rng
    std::vector<SourceParams> src_params; // addSource order
    Sources S;               // device copy from first-frame init on
    bool grows = false;      // particles are added every substep (NB-FLIP or sources)
    bool rng_dev = false;    // the engine state is R.rng (else the host's rng)
    NbGrids N;
    NbReseed R;
    int nb_max_cand = 0;     // particlesPerCell candidates per cell at most
    void *nb_scan = nullptr; // scan scratch for the candidate counts
    int frame = 0;
    float step_dt = 0.f, frame_dt = 0.f;
    bool initialized = false;
    bool after_advect = false;
    int density_iters_max = 0, pressure_iters_max = 0, substeps = 0;
    long long substeps_total = 0; // every substep since creation
    bool timers = false;
    double t_step_ms = 0.0, t_pcg_ms = 0.0, launches = 0.0;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    // per-stage timing (timers on): events after each group of stages, and
    // the accumulated milliseconds per SolverStage (flipsolver2d.h:58-72)
    cudaEvent_t stage_ev[10] = {};
    int stage_of[10] = {};   // the SolverStage each recorded event ends
    double t_stage_ms[12] = {};
    // viscosity (FlipSolverParameters::viscosityEnabled): the model's system
    // and solver buffers, and its return value of the last substep
    ViscBuffers visc;
    int visc_iters = 0;
    // PCG timing events per solve of a substep (0 density, 1 pressure); read
    // after the substep so that timing adds no host wait inside it
    cudaEvent_t p0[2] = {nullptr, nullptr}, p1[2] = {nullptr, nullptr};
    bool pcg_timed[2] = {false, false};
    std::vector<void *> allocs;
    std::vector<size_t> alloc_bytes; // beside allocs
    size_t device_bytes = 0;
};

template <typename T> static fs_status dalloc(fs_solver *s, T **p, size_t count)
{
    void *q = nullptr;
    size_t bytes = count * sizeof(T);
    if (bytes == 0) bytes = 16;
    CK(cudaMalloc(&q, bytes));
    s->allocs.push_back(q);
    s->alloc_bytes.push_back(bytes);
    s->device_bytes += bytes;
    *p = (T *)q;
    return FS_OK;
}

static void dfree(fs_solver *s, void *p)
{
    if (!p) return;
    auto it = std::find(s->allocs.begin(), s->allocs.end(), p);
    if (it != s->allocs.end()) {
        const size_t k = (size_t)(it - s->allocs.begin());
        s->device_bytes -= s->alloc_bytes[k];
        s->alloc_bytes.erase(s->alloc_bytes.begin() + (long)k);
        s->allocs.erase(it);
    }
    cudaFree(p);
}

static fs_status set_device(const fs_solver *s)
{
    CK(cudaSetDevice(s->ex.device));
    return FS_OK;
}

static fs_status alloc_particles(fs_solver *s, int cap)
{
    Particles &P = s->P;
    void *old[] = {P.pos, P.vel, P.visc, P.slot_bin, P.pos2, P.vel2, P.visc2, P.slot_bin2,
                   P.flag, P.dest, P.prune_slot, P.mkey, P.mval, P.mkey2, P.mval2};
    for (void *q : old) dfree(s, q);
    dfree(s, s->rebin_scratch);
    P.cap = cap;
    P.bound = cap;
    const size_t n = (size_t)std::max(cap, 1);
    TRY(dalloc(s, &P.pos, n));
    TRY(dalloc(s, &P.vel, n));
    TRY(dalloc(s, &P.visc, n));
    TRY(dalloc(s, &P.slot_bin, n));
    TRY(dalloc(s, &P.pos2, n));
    TRY(dalloc(s, &P.vel2, n));
    TRY(dalloc(s, &P.visc2, n));
    TRY(dalloc(s, &P.slot_bin2, n));
    TRY(dalloc(s, &P.flag, n));
    TRY(dalloc(s, &P.dest, n));
    TRY(dalloc(s, &P.prune_slot, n));
    TRY(dalloc(s, &P.mkey, n));
    TRY(dalloc(s, &P.mval, n));
    TRY(dalloc(s, &P.mkey2, n));
    TRY(dalloc(s, &P.mval2, n));
    s->rebin_scratch_size = rebin_scratch_bytes(P);
    void *q = nullptr;
    CK(cudaMalloc(&q, s->rebin_scratch_size));
    s->allocs.push_back(q);
    s->alloc_bytes.push_back(s->rebin_scratch_size);
    s->device_bytes += s->rebin_scratch_size;
    s->rebin_scratch = q;
    return FS_OK;
}

static fs_status upload_particles(fs_solver *s, const std::vector<int> &counts,
                                  const std::vector<float2> &pos, const std::vector<float2> &vel,
                                  const std::vector<float> &visc)
{
    const int nb = s->P.nbins;
    const int total = (int)pos.size();
    if (total > s->P.cap || s->P.pos == nullptr) {
        // NB-FLIP keeps room for 2 particlesPerCell per cell (reseeding)
        const long long keep = s->grows ? 2LL * s->p.particlesPerCell * (long long)s->ncell : 0;
        TRY(alloc_particles(s, (int)std::max<long long>(total, keep)));
    }
    std::vector<int> start(nb + 1, 0), slot_bin(total);
    for (int b = 0; b < nb; b++) start[b + 1] = start[b] + counts[b];
    for (int b = 0; b < nb; b++)
        for (int k = start[b]; k < start[b + 1]; k++) slot_bin[k] = b;
    Particles &P = s->P;
    CK(cudaMemcpyAsync(P.bin_start, start.data(), (nb + 1) * sizeof(int), cudaMemcpyHostToDevice, s->st));
    CK(cudaMemcpyAsync(P.bin_count, counts.data(), nb * sizeof(int), cudaMemcpyHostToDevice, s->st));
    if (total) {
        CK(cudaMemcpyAsync(P.pos, pos.data(), total * sizeof(float2), cudaMemcpyHostToDevice, s->st));
        CK(cudaMemcpyAsync(P.vel, vel.data(), total * sizeof(float2), cudaMemcpyHostToDevice, s->st));
        CK(cudaMemcpyAsync(P.visc, visc.data(), total * sizeof(float), cudaMemcpyHostToDevice, s->st));
        CK(cudaMemcpyAsync(P.slot_bin, slot_bin.data(), total * sizeof(int), cudaMemcpyHostToDevice, s->st));
    }
    CK(cudaStreamSynchronize(s->st));
    s->after_advect = false;
    if (s->grows) P.bound = std::max(total, 1);
    return FS_OK;
}

// updateVelocityFromSolids factors depend on solid cells, solid ids and the
// obstacles' friction; recompute them whenever one of those was replaced
static fs_status ensure_friction(fs_solver *s)
{
    if (!s->friction_dirty) return FS_OK;
    if (!s->d_obst_friction) TRY(dalloc(s, &s->d_obst_friction, s->obst_friction.size() + 1));
    if (!s->obst_friction.empty())
        CK(cudaMemcpyAsync(s->d_obst_friction, s->obst_friction.data(), s->obst_friction.size() * 4,
                           cudaMemcpyHostToDevice, s->st));
    launch_friction_factors(s->d, s->G, s->d_obst_friction, s->st);
    g_kernel_launches += 1;
    CK(cudaStreamSynchronize(s->st));
    s->friction_dirty = false;
    return FS_OK;
}

static fs_status wait_side(fs_solver *s)
{
    if (s->levelset_pending) {
        CK(cudaStreamWaitEvent(s->st, s->ev_levelset, 0));
        s->levelset_pending = false;
    }
    return FS_OK;
}

static fs_status sync_all(fs_solver *s)
{
    TRY(wait_side(s));
    CK(cudaStreamSynchronize(s->st));
    CK(cudaGetLastError());
    return FS_OK;
}

static fs_status create_impl(const fs_params *p, const fs_exec_params *exec, bool nb, fs_solver **out)
{
    if (!p || !out) return fail(FS_ERR_BAD_ARG, "fs_create: null argument");
    *out = nullptr;
    if (p->gridSizeI < 1 || p->gridSizeJ < 1 || p->dx <= 0 || p->fps <= 0 ||
        p->particlesPerCell < 1 || p->pcgIterLimit < 0)
        return fail(FS_ERR_BAD_ARG, "fs_create: invalid parameters");
    if ((long long)p->gridSizeI * p->gridSizeJ > (1LL << 30))
        return fail(FS_ERR_BAD_ARG, "fs_create: grid too large");
    // SIMULATION_LIQUID, or SIMULATION_NBFLIP for the narrow-band solver
    if (p->simulationMethod != 0 && !(nb && p->simulationMethod == 3))
        return fail(FS_ERR_UNSUPPORTED, "fs_create: only the liquid solvers are supported");
    if (nb && (long long)p->gridSizeI * p->gridSizeJ * p->particlesPerCell * 2 > INT_MAX)
        return fail(FS_ERR_BAD_ARG, "fs_create_nbflip: particle capacity above 2^31");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return fail(FS_ERR_CUDA, "fs_create: no CUDA device");
    fs_solver *s = new fs_solver();
    s->p = *p;
    if (exec) s->ex = *exec;
    if (s->ex.pool_threads <= 0) s->ex.pool_threads = default_pool_threads();
    if (s->ex.pool_threads > 4096) s->ex.pool_threads = 4096;
    if (s->ex.device < 0 || s->ex.device >= ndev) {
        delete s;
        return fail(FS_ERR_BAD_ARG, "fs_create: bad device ordinal");
    }
    s->prec = s->ex.pcg_precision == FS_PCG_FP64 ? FS_PCG_FP64
            : s->ex.pcg_precision == FS_PCG_SPEC ? FS_PCG_SPEC
                                                 : FS_PCG_FP32;
    s->esz = s->prec == FS_PCG_FP32 ? 4 : 8;
    auto cleanup = [&](fs_status st) {
        fs_destroy(s);
        return st;
    };
    if (set_device(s) != FS_OK) return cleanup(FS_ERR_CUDA);
    GridDims &d = s->d;
    d.ni = p->gridSizeI;
    d.nj = p->gridSizeJ;
    d.bni = d.ni / 3 + (d.ni % 3 != 0);
    d.bnj = d.nj / 3 + (d.nj % 3 != 0);
    s->ncell = (size_t)d.ni * d.nj;
    s->nu = (size_t)(d.ni + 1) * d.nj;
    s->nv = (size_t)d.ni * (d.nj + 1);
    SceneParams &sp = s->sp;
    sp.fluidDensity = p->fluidDensity;
    sp.dx = p->dx;
    sp.particlesPerCell = p->particlesPerCell;
    sp.gI = p->globalAccelerationI;
    sp.gJ = p->globalAccelerationJ;
    sp.picRatio = p->picRatio;
    sp.particleScale = p->particleScale;
    sp.pcgIterLimit = p->pcgIterLimit;
    sp.parameterHandlingMethod = p->parameterHandlingMethod;
    sp.viscosityEnabled = p->viscosityEnabled;
    sp.projectTolerance = p->viscosityEnabled ? 1e-6 : 1e-2; // flipsolver2d.cpp:73
    if (nb) sp.projectTolerance = 1e-6;                       // nbflipsolver.cpp:22
    s->step_dt = 1.f / p->fps; // flipsolver2d.cpp:46-47
    s->frame_dt = 1.f / p->fps;
    s->rng = std::mt19937(p->seed);

    fs_status st = FS_OK;
#define A(expr)                                                                                    \
    do {                                                                                           \
        st = (expr);                                                                               \
        if (st != FS_OK) return cleanup(st);                                                       \
    } while (0)
    if (cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&s->side, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&s->ev_p2g, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&s->ev_levelset, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreate(&s->e0) != cudaSuccess || cudaEventCreate(&s->e1) != cudaSuccess ||
        cudaEventCreate(&s->p0[0]) != cudaSuccess || cudaEventCreate(&s->p1[0]) != cudaSuccess ||
        cudaEventCreate(&s->p0[1]) != cudaSuccess || cudaEventCreate(&s->p1[1]) != cudaSuccess)
        return cleanup(fail(FS_ERR_CUDA, "fs_create: stream/event creation failed"));
    const size_t n = s->ncell;
    Grids &G = s->G;
    A(dalloc(s, &G.material, n));
    A(dalloc(s, &G.solid_sdf, n));
    A(dalloc(s, &G.solid_id, n));
    A(dalloc(s, &G.fluid_sdf, n));
    A(dalloc(s, &G.u, s->nu));
    A(dalloc(s, &G.v, s->nv));
    A(dalloc(s, &G.uvalid, s->nu));
    A(dalloc(s, &G.vvalid, s->nv));
    A(dalloc(s, &G.u2, s->nu));
    A(dalloc(s, &G.v2, s->nv));
    A(dalloc(s, &G.uvalid2, s->nu));
    A(dalloc(s, &G.vvalid2, s->nv));
    A(dalloc(s, &G.su, s->nu));
    A(dalloc(s, &G.sv, s->nv));
    A(dalloc(s, &G.suvalid, s->nu));
    A(dalloc(s, &G.svvalid, s->nv));
    A(dalloc(s, &G.visc, n));
    A(dalloc(s, &G.known, n));
    A(dalloc(s, &G.divc, n));
    A(dalloc(s, &G.density, n));
    A(dalloc(s, &G.counts, n));
    A(dalloc(s, &G.cell_info, n));
    A(dalloc(s, &G.ufric, n));
    A(dalloc(s, &G.vfric, n));
    A(dalloc(s, &G.emitter_id, n));
    A(dalloc(s, &G.levelset_cells, n));
    A(dalloc(s, &G.levelset_act, 3 * ((size_t)(d.ni + 31) / 32) * ((d.nj + 31) / 32) + 8));
    A(dalloc(s, &G.levelset_active, (size_t)levelset_max_passes(d) + 1));
    Particles &P = s->P;
    P.nbins = d.bni * d.bnj;
    A(dalloc(s, &P.bin_start, (size_t)P.nbins + 1));
    A(dalloc(s, &P.bin_count, (size_t)P.nbins));
    A(dalloc(s, &P.bin_start2, (size_t)P.nbins + 1));
    A(dalloc(s, &P.bin_count2, (size_t)P.nbins));
    A(dalloc(s, &P.survivors, (size_t)P.nbins));
    A(dalloc(s, &P.incoming, (size_t)P.nbins + 1));
    A(dalloc(s, &P.inc_off, (size_t)P.nbins + 1));
    A(dalloc(s, &P.nmoved, 1));
    A(dalloc(s, &s->sc, 1));
    if (cudaMallocHost(&s->sc_host, sizeof(Scalars)) != cudaSuccess)
        return cleanup(fail(FS_ERR_OOM, "fs_create: pinned allocation failed"));
    if (p->viscosityEnabled) { // the light or heavy model's system (viscositymodel.cpp)
        ViscBuffers &V = s->visc;
        const bool heavy = p->useHeavyViscosity != 0;
        V.n = visc_unknowns(d, heavy);
        V.ncoef = visc_coef_count(d, heavy);
        double **vv[] = {&V.b, &V.x, &V.r, &V.p, &V.t, &V.invdiag};
        for (double **q : vv) A(dalloc(s, q, (size_t)V.n));
        A(dalloc(s, &V.coef, (size_t)V.ncoef));
        A(dalloc(s, &V.part, (size_t)3 * kViscBlocksMax));
        A(dalloc(s, &V.ctl, 1));
        if (cudaMallocHost(&V.ctl_host, sizeof(ViscCtl)) != cudaSuccess)
            return cleanup(fail(FS_ERR_OOM, "fs_create: pinned allocation failed"));
    }
    // PCG vectors
    const size_t vb = n * s->esz;
    void **vecs[] = {&s->dens_rhs, &s->dens_x, &s->pres_rhs, &s->pres_x, &s->r0, &s->r1, &s->s0, &s->s1};
    for (void **v : vecs) {
        char *q = nullptr;
        A(dalloc(s, &q, vb));
        *v = q;
    }
    s->pcg_grid = s->prec == FS_PCG_FP32 ? pcg_grid_size<float>((long long)n)
                                         : pcg_grid_size<double>((long long)n);
    A(dalloc(s, &s->partials, (size_t)8 * s->pcg_grid + 16));
    A(dalloc(s, &s->bar, 1));
    if (s->prec == FS_PCG_FP32)
        s->resident = resident_tile_shape(d.ni, d.nj, &s->res_ti, &s->res_tj);
    if (s->resident) {
        s->ll.words = n;
        A(dalloc(s, &s->ll.r, n));
        A(dalloc(s, &s->ll.s, n));
        A(dalloc(s, &s->ll.rec, kLlRecWords));
    }
    if (s->prec == FS_PCG_FP32 && tma_tile_shape(d.ni, d.nj, &s->tma_ti, &s->tma_tj)) {
        s->tma = tma_maps(&s->maps_dens, d.ni, d.nj, s->tma_ti, s->tma_tj, G.cell_info,
                          (const float *)s->dens_rhs, (const float *)s->dens_x,
                          (const float *)s->r0, (const float *)s->r1, (const float *)s->s0,
                          (const float *)s->s1) &&
                 tma_store_maps(&s->maps_dens, d.ni, d.nj, s->tma_ti, s->tma_tj,
                                (const float *)s->r0, (const float *)s->r1, (const float *)s->s0,
                                (const float *)s->s1) &&
                 tma_maps(&s->maps_pres, d.ni, d.nj, s->tma_ti, s->tma_tj, G.cell_info,
                          (const float *)s->pres_rhs, (const float *)s->pres_x,
                          (const float *)s->r0, (const float *)s->r1, (const float *)s->s0,
                          (const float *)s->s1) &&
                 tma_store_maps(&s->maps_pres, d.ni, d.nj, s->tma_ti, s->tma_tj,
                                (const float *)s->r0, (const float *)s->r1, (const float *)s->s0,
                                (const float *)s->s1);
    }
    if (s->prec == FS_PCG_SPEC && !cluster_plan(d.ni, d.nj, &s->spec_plan)) {
        // above the on-chip limit: the cooperative solve, chained on the
        // device (launch_spec_chain)
        s->spec_large = true;
        A(dalloc(s, &s->spec_rel, 2));
        float *r = nullptr, *dd = nullptr, *sv = nullptr, *q = nullptr, *z = nullptr;
        float2 *parts = nullptr;
        double *rpart = nullptr;
        unsigned *count = nullptr;
        SpecCtl *ctl = nullptr;
        A(dalloc(s, &r, n));
        A(dalloc(s, &dd, n));
        A(dalloc(s, &sv, n));
        A(dalloc(s, &q, n));
        A(dalloc(s, &z, n));
        A(dalloc(s, &parts, (size_t)spec_partials_needed()));
        A(dalloc(s, &rpart, (size_t)kSpecResBlocks));
        A(dalloc(s, &count, 1));
        A(dalloc(s, &ctl, 1));
        // inner solves on the resident kernel where the grid fits it (the
        // handle's exchange words, unused by the FP32 path in this mode)
        int rti = 0, rtj = 0;
        const bool res = spec_resident_shape(d.ni, d.nj, &rti, &rtj);
        if (res) {
            s->ll.words = n;
            A(dalloc(s, &s->ll.r, n));
            A(dalloc(s, &s->ll.s, n));
            A(dalloc(s, &s->ll.rec, kLlRecWords));
        }
        for (int k = 0; k < 2; k++) {
            SpecSolve &c = s->spec_chain[k];
            c.ni = d.ni;
            c.nj = d.nj;
            c.info = G.cell_info;
            c.b = (const double *)(k == 0 ? s->dens_rhs : s->pres_rhs);
            c.x = (double *)(k == 0 ? s->dens_x : s->pres_x);
            c.dt = &s->sc->dt;
            c.density = p->fluidDensity;
            c.dx = p->dx;
            c.r = r;
            c.d = dd;
            c.s = sv;
            c.q = q;
            c.z = z;
            c.partials = parts;
            c.rpart = rpart;
            c.count = count;
            c.status = &s->sc->pcg_status;
            c.ctl = ctl;
            c.iters_out = k == 0 ? &s->sc->density_iters : &s->sc->pressure_iters;
            c.rel_out = s->spec_rel + k;
            c.tol = kSpecRelTol;
            c.max_iter = kSpecMaxIter;
            c.max_outer = kSpecMaxOuter;
            if (res) {
                c.res_ti = rti;
                c.res_tj = rtj;
                c.ll = &s->ll;
                c.wrap_flag = &s->sc->wrap_units;
            }
        }
    } else if (s->prec == FS_PCG_SPEC) {
        A(dalloc(s, &s->spec_sys, 2));
        A(dalloc(s, &s->spec_rel, 2));
        ClusterSystem hs[2];
        for (int k = 0; k < 2; k++) {
            hs[k].ni = d.ni;
            hs[k].nj = d.nj;
            hs[k].info = G.cell_info;
            hs[k].b = (const double *)(k == 0 ? s->dens_rhs : s->pres_rhs);
            hs[k].x = (double *)(k == 0 ? s->dens_x : s->pres_x);
            hs[k].dt = &s->sc->dt;
            hs[k].density = p->fluidDensity;
            hs[k].dx = p->dx;
            hs[k].iters = k == 0 ? &s->sc->density_iters : &s->sc->pressure_iters;
            hs[k].rel_res = s->spec_rel + k;
        }
        if (cudaMemcpy(s->spec_sys, hs, sizeof(hs), cudaMemcpyHostToDevice) != cudaSuccess)
            return cleanup(fail(FS_ERR_CUDA, "fs_create: upload failed"));
    }
    std::vector<int> ends = split_range_ends((long long)n, s->ex.pool_threads);
    s->nchunks = (int)ends.size();
    split_range_params((long long)n, s->ex.pool_threads, &s->chunk_ps, &s->chunk_rem);
    A(dalloc(s, &s->chunk_end, ends.size() + 1));
    A(dalloc(s, &s->chunk_last, ends.size() + 1));
    A(dalloc(s, &s->chunk_val, ends.size() + 1));
    if (!ends.empty() &&
        cudaMemcpy(s->chunk_end, ends.data(), ends.size() * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess)
        return cleanup(fail(FS_ERR_CUDA, "fs_create: upload failed"));

    // initial grid state (FlipSolver ctor, flipsolver2d.cpp:27-45)
    cudaStream_t q = s->st;
    bool ok = cudaMemsetAsync(G.material, 0x10, n, q) == cudaSuccess; // EMPTY
    k_fill_i32<<<(unsigned)((n + 255) / 256), 256, 0, q>>>(G.solid_id, -1, n);
    k_fill_i32<<<(unsigned)((n + 255) / 256), 256, 0, q>>>(G.emitter_id, -1, n);
    // no unit row anywhere until the first decomposition: a solve run before
    // it (fs_run_stage) sees an operator of identity rows
    k_fill_i32<<<(unsigned)((ends.size() + 256) / 256), 256, 0, q>>>(s->chunk_last, -1, ends.size() + 1);
    void *zero[] = {G.solid_sdf, G.fluid_sdf, G.visc, G.known, G.divc, G.density, G.counts,
                    G.cell_info};
    size_t zsz[] = {n * 4, n * 4, n * 4, n, n * 4, n * 4, n * 4, n};
    for (int k = 0; k < 8; k++) ok = ok && cudaMemsetAsync(zero[k], 0, zsz[k], q) == cudaSuccess;
    void *zu[] = {G.u, G.u2, G.su};
    void *zv[] = {G.v, G.v2, G.sv};
    for (int k = 0; k < 3; k++) {
        ok = ok && cudaMemsetAsync(zu[k], 0, s->nu * 4, q) == cudaSuccess;
        ok = ok && cudaMemsetAsync(zv[k], 0, s->nv * 4, q) == cudaSuccess;
    }
    void *zf[] = {G.uvalid, G.uvalid2, G.suvalid};
    void *zg[] = {G.vvalid, G.vvalid2, G.svvalid};
    for (int k = 0; k < 3; k++) {
        ok = ok && cudaMemsetAsync(zf[k], 0, s->nu, q) == cudaSuccess;
        ok = ok && cudaMemsetAsync(zg[k], 0, s->nv, q) == cudaSuccess;
    }
    for (void *v : {s->dens_rhs, s->dens_x, s->pres_rhs, s->pres_x})
        ok = ok && cudaMemsetAsync(v, 0, vb, q) == cudaSuccess;
    ok = ok && cudaMemsetAsync(P.bin_start, 0, (P.nbins + 1) * sizeof(int), q) == cudaSuccess;
    ok = ok && cudaMemsetAsync(P.bin_count, 0, P.nbins * sizeof(int), q) == cudaSuccess;
    ok = ok && cudaMemsetAsync(s->sc, 0, sizeof(Scalars), q) == cudaSuccess;
    ok = ok && cudaStreamSynchronize(q) == cudaSuccess;
    if (!ok) return cleanup(fail(FS_ERR_CUDA, "fs_create: initialisation failed"));
    if (nb) {
        // NB-FLIP: after countParticles every cell holds at most
        // 2 particlesPerCell, and reseeding tops band cells up to
        // particlesPerCell, so 2 particlesPerCell per cell bounds the count
        s->nb = true;
        const int ppc = p->particlesPerCell;
        A(alloc_particles(s, (int)(2LL * ppc * (long long)n)));
        NbGrids &N = s->N;
        A(dalloc(s, &N.adv_u, s->nu));
        A(dalloc(s, &N.adv_v, s->nv));
        A(dalloc(s, &N.adv_sdf, n));
        A(dalloc(s, &N.adv_visc, n));
        s->nb_max_cand = (int)((long long)ppc * (long long)n);
        const size_t mc = (size_t)s->nb_max_cand;
        NbReseed &R = s->R;
        R.ncell = (int)n;
        A(dalloc(s, &R.rng, 625));
        A(dalloc(s, &R.cand_n, n));
        A(dalloc(s, &R.cand_off, n + 1));
        A(dalloc(s, &R.draws, 2 * mc));
        A(dalloc(s, &R.cand_pos, mc));
        A(dalloc(s, &R.cand_vel, mc));
        A(dalloc(s, &R.cand_visc, mc));
        A(dalloc(s, &R.cand_bin, mc));
        A(dalloc(s, &R.cand_cb, mc));
        A(dalloc(s, &R.pos_of, mc));
        A(dalloc(s, &R.cross, (size_t)kNbCrossMax));
        A(dalloc(s, &R.cross_n, 1));
        R.status = &s->sc->nb_overflow;
        char *scan = nullptr;
        A(dalloc(s, &scan, scan_scratch_bytes((int)n)));
        s->nb_scan = scan;
        ok = true;
        for (float *g : {N.adv_u, N.adv_v}) ok = ok && cudaMemsetAsync(g, 0, (g == N.adv_u ? s->nu : s->nv) * 4, q) == cudaSuccess;
        for (float *g : {N.adv_sdf, N.adv_visc}) ok = ok && cudaMemsetAsync(g, 0, n * 4, q) == cudaSuccess;
        uint32_t st0[625];
        mt_seed_host(st0, p->seed); // m_randEngine = std::mt19937(p->seed), flipsolver2d.cpp:71
        ok = ok && cudaMemcpyAsync(R.rng, st0, sizeof(st0), cudaMemcpyHostToDevice, q) == cudaSuccess;
        ok = ok && cudaStreamSynchronize(q) == cudaSuccess;
        if (!ok) return cleanup(fail(FS_ERR_CUDA, "fs_create_nbflip: initialisation failed"));
        s->grows = true;
        s->rng_dev = true;
    } else {
        A(alloc_particles(s, 0));
    }
    *out = s;
    return FS_OK;
#undef A
}

extern "C" fs_status fs_create(const fs_params *p, const fs_exec_params *exec, fs_solver **out)
{
    return create_impl(p, exec, false, out);
}

extern "C" fs_status fs_create_nbflip(const fs_params *p, const fs_exec_params *exec, fs_solver **out)
{
    return create_impl(p, exec, true, out);
}

extern "C" fs_status fs_get_rng_state(fs_solver *s, uint32_t *state)
{
    if (!s || !state) return fail(FS_ERR_BAD_ARG, "null argument");
    TRY(set_device(s));
    if (s->rng_dev) {
        TRY(sync_all(s));
        CK(cudaMemcpy(state, s->R.rng, 625 * sizeof(uint32_t), cudaMemcpyDeviceToHost));
        return FS_OK;
    }
    // libstdc++ writes the 624 state words, then the index of the next one
    std::ostringstream os;
    os << s->rng;
    std::istringstream is(os.str());
    for (int k = 0; k < 625; k++) {
        unsigned long v = 0;
        if (!(is >> v)) return fail(FS_ERR_CUDA, "fs_get_rng_state: unexpected engine format");
        state[k] = (uint32_t)v;
    }
    return FS_OK;
}

extern "C" fs_status fs_set_rng_state(fs_solver *s, const uint32_t *state)
{
    if (!s || !state) return fail(FS_ERR_BAD_ARG, "null argument");
    if (state[624] > 624) return fail(FS_ERR_BAD_ARG, "fs_set_rng_state: index above 624");
    TRY(set_device(s));
    if (s->rng_dev) {
        TRY(sync_all(s));
        CK(cudaMemcpy(s->R.rng, state, 625 * sizeof(uint32_t), cudaMemcpyHostToDevice));
        return FS_OK;
    }
    std::ostringstream os;
    for (int k = 0; k < 625; k++) os << state[k] << (k < 624 ? " " : "");
    std::istringstream is(os.str());
    is >> s->rng;
    if (is.fail()) return fail(FS_ERR_BAD_ARG, "fs_set_rng_state: rejected state");
    return FS_OK;
}

extern "C" fs_status fs_destroy(fs_solver *s)
{
    if (!s) return FS_OK;
    cudaSetDevice(s->ex.device);
    if (s->st) cudaStreamSynchronize(s->st);
    if (s->side) cudaStreamSynchronize(s->side);
    for (void *q : s->allocs) cudaFree(q);
    if (s->sc_host) cudaFreeHost(s->sc_host);
    if (s->visc.ctl_host) cudaFreeHost(s->visc.ctl_host);
    cudaEvent_t evs[] = {s->ev_p2g, s->ev_levelset, s->e0, s->e1, s->p0[0], s->p1[0], s->p0[1], s->p1[1]};
    for (cudaEvent_t e : evs)
        if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : s->stage_ev)
        if (e) cudaEventDestroy(e);
    if (s->st) cudaStreamDestroy(s->st);
    if (s->side) cudaStreamDestroy(s->side);
    delete s;
    return FS_OK;
}

static fs_status add_poly(fs_solver *s, int kind, float value, const float *xy, int n)
{
    if (!s || !xy || n < 1) return fail(FS_ERR_BAD_ARG, "polygon needs at least one vertex");
    Poly g;
    g.kind = kind;
    g.value = value;
    g.xy.assign(xy, xy + 2 * n);
    s->polys.push_back(g);
    if (kind == 0) s->obst_friction.push_back(value);
    return FS_OK;
}

extern "C" fs_status fs_add_geometry(fs_solver *s, float friction, const float *xy, int n)
{
    return add_poly(s, 0, friction, xy, n);
}
extern "C" fs_status fs_add_initial_fluid(fs_solver *s, float viscosity, const float *xy, int n)
{
    return add_poly(s, 1, viscosity, xy, n);
}
extern "C" fs_status fs_add_sink(fs_solver *s, float divergence, const float *xy, int n)
{
    return add_poly(s, 2, divergence, xy, n);
}

extern "C" fs_status fs_add_source(fs_solver *s, const float *xy, int n, float viscosity,
                                   float divergence, float vx, float vy, int velocity_transfer)
{
    if (s && s->initialized) return fail(FS_ERR_STATE, "fs_add_source: the scene is initialised");
    TRY(add_poly(s, 3, divergence, xy, n));
    SourceParams e{};
    e.visc = viscosity;
    e.div = divergence;
    e.vx = vx;
    e.vy = vy;
    e.transfer = velocity_transfer != 0;
    s->src_params.push_back(e);
    return FS_OK;
}

static fs_status download_bins(fs_solver *s, std::vector<int> &start, std::vector<int> &count);

// ---- host restatement of the sampler used for seeding (grid2d.h:187-216) --
static inline float h_frac(float v) { return v - (float)(long long)v; }
static inline float h_lerp(float a, float b, float f) { return (a * (1.0f - f)) + (b * f); }
static inline float h_get(const std::vector<float> &g, int si, int sj, long long i, long long j)
{
    i = std::clamp<long long>(i, 0, si - 1);
    j = std::clamp<long long>(j, 0, sj - 1);
    return g[(size_t)i * sj + j];
}
static float h_grid_lerp(const std::vector<float> &g, int si, int sj, float ox, float oy, float i,
                         float j)
{
    i += ox;
    j += oy;
    i = std::clamp(i, 0.f, (float)(si - 1));
    j = std::clamp(j, 0.f, (float)(sj - 1));
    long long ci = (long long)std::floor(i), cj = (long long)std::floor(j);
    float fi = h_frac(i), fj = h_frac(j);
    long long c2j = fj >= 0.5f ? cj + 1 : cj - 1;
    long long c3i = fi >= 0.5f ? ci + 1 : ci - 1;
    float il = fi < 0.5f ? 0.5f - fi : fi - 0.5f;
    float jl = fj < 0.5f ? 0.5f - fj : fj - 0.5f;
    float v1 = h_lerp(h_get(g, si, sj, ci, cj), h_get(g, si, sj, c3i, cj), il);
    float v2 = h_lerp(h_get(g, si, sj, ci, c2j), h_get(g, si, sj, c3i, c2j), il);
    return h_lerp(v1, v2, jl);
}

// the source table and polygons on the device for the substeps (frame-0
// setup copies every polygon only for the classification)
static fs_status upload_sources(fs_solver *s)
{
    if (s->src_params.empty() || s->S.n) return FS_OK;
    std::vector<float> xy;
    std::vector<int> off(1, 0);
    for (const Poly &g : s->polys)
        if (g.kind == 3) {
            xy.insert(xy.end(), g.xy.begin(), g.xy.end());
            off.push_back(off.back() + (int)(g.xy.size() / 2));
        }
    SourceParams *p = nullptr;
    float *dxy = nullptr;
    int *doff = nullptr;
    TRY(dalloc(s, &p, s->src_params.size()));
    TRY(dalloc(s, &dxy, xy.size()));
    TRY(dalloc(s, &doff, off.size()));
    CK(cudaMemcpy(p, s->src_params.data(), s->src_params.size() * sizeof(SourceParams),
                  cudaMemcpyHostToDevice));
    CK(cudaMemcpy(dxy, xy.data(), xy.size() * 4, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(doff, off.data(), off.size() * 4, cudaMemcpyHostToDevice));
    s->S.p = p;
    s->S.xy = dxy;
    s->S.off = doff;
    s->S.n = (int)s->src_params.size();
    return FS_OK;
}

// FLIP with sources reseeds every substep (reseedParticles): the same
// candidate scratch as NB-FLIP, sized for particlesPerCell / 2 per cell
static fs_status alloc_flip_reseed(fs_solver *s)
{
    if (s->R.rng) return FS_OK;
    const size_t n = s->ncell;
    const int per = std::max(1, s->p.particlesPerCell / 2);
    s->nb_max_cand = (int)std::min<long long>((long long)per * (long long)n, INT_MAX / 2);
    const size_t mc = (size_t)s->nb_max_cand;
    NbReseed &R = s->R;
    R.ncell = (int)n;
    TRY(dalloc(s, &R.rng, 625));
    TRY(dalloc(s, &R.cand_n, n));
    TRY(dalloc(s, &R.cand_off, n + 1));
    TRY(dalloc(s, &R.draws, 2 * mc));
    TRY(dalloc(s, &R.cand_pos, mc));
    TRY(dalloc(s, &R.cand_vel, mc));
    TRY(dalloc(s, &R.cand_visc, mc));
    TRY(dalloc(s, &R.cand_bin, mc));
    TRY(dalloc(s, &R.cand_cb, mc));
    TRY(dalloc(s, &R.pos_of, mc));
    TRY(dalloc(s, &R.cross, (size_t)kNbCrossMax));
    TRY(dalloc(s, &R.cross_n, 1));
    R.status = &s->sc->nb_overflow;
    char *scan = nullptr;
    TRY(dalloc(s, &scan, scan_scratch_bytes((int)n)));
    s->nb_scan = scan;
    return FS_OK;
}

// the host engine state (std::mt19937, after the frame-0 seeding) to the
// device, where the substeps' reseeding draws from it
static fs_status rng_to_device(fs_solver *s)
{
    std::ostringstream os;
    os << s->rng; // libstdc++: the 624 state words, then the index of the next
    std::istringstream is(os.str());
    uint32_t st[625];
    for (int k = 0; k < 625; k++) {
        unsigned long v = 0;
        if (!(is >> v)) return fail(FS_ERR_CUDA, "unexpected engine format");
        st[k] = (uint32_t)v;
    }
    CK(cudaMemcpy(s->R.rng, st, sizeof(st), cudaMemcpyHostToDevice));
    s->rng_dev = true;
    return FS_OK;
}

extern "C" fs_status fs_first_frame_init(fs_solver *s)
{
    if (!s) return fail(FS_ERR_BAD_ARG, "null handle");
    TRY(set_device(s));
    TRY(sync_all(s));
    const GridDims &d = s->d;
    // polygons -> device
    std::vector<float> xy;
    std::vector<int> off(1, 0), kind;
    std::vector<float> val;
    for (const Poly &g : s->polys) {
        xy.insert(xy.end(), g.xy.begin(), g.xy.end());
        off.push_back(off.back() + (int)(g.xy.size() / 2));
        kind.push_back(g.kind);
        val.push_back(g.value);
    }
    float *dxy = nullptr, *dval = nullptr;
    int *doff = nullptr, *dkind = nullptr;
    TRY(dalloc(s, &dxy, xy.size() + 2));
    TRY(dalloc(s, &doff, off.size()));
    TRY(dalloc(s, &dkind, kind.size() + 1));
    TRY(dalloc(s, &dval, val.size() + 1));
    if (!xy.empty()) CK(cudaMemcpy(dxy, xy.data(), xy.size() * 4, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(doff, off.data(), off.size() * 4, cudaMemcpyHostToDevice));
    if (!kind.empty()) {
        CK(cudaMemcpy(dkind, kind.data(), kind.size() * 4, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(dval, val.data(), val.size() * 4, cudaMemcpyHostToDevice));
    }
    // updateSinks, updateSources (none), updateSolids, updateInitialFluid
    launch_scene_classify(d, s->G, (float)s->p.dx, dxy, doff, dkind, dval, (int)s->polys.size(),
                          s->nb, s->st);
    g_kernel_launches += 1;
    CK(cudaGetLastError());
    s->friction_dirty = true;
    TRY(ensure_friction(s));
    TRY(upload_sources(s));
    if (s->S.n && !s->nb) {
        s->grows = true; // the seeding upload below keeps room for the sources' particles
        TRY(alloc_flip_reseed(s));
    }
    if (s->nb) {
        // NBFlipSolver::initialFluidSeed (nbflipsolver.cpp:255-297) adds no
        // particle but draws two numbers for each of particlesPerCell
        // candidates in every cell with a negative SDF
        std::vector<float> sdf(s->ncell);
        CK(cudaMemcpyAsync(sdf.data(), s->G.fluid_sdf, s->ncell * 4, cudaMemcpyDeviceToHost, s->st));
        std::vector<uint32_t> rs(625);
        CK(cudaMemcpyAsync(rs.data(), s->R.rng, 625 * 4, cudaMemcpyDeviceToHost, s->st));
        CK(cudaStreamSynchronize(s->st));
        unsigned long long neg = 0;
        for (float v : sdf) neg += v < 0.f;
        mt_discard_host(rs.data(), neg * 2ULL * (unsigned long long)s->p.particlesPerCell);
        CK(cudaMemcpyAsync(s->R.rng, rs.data(), 625 * 4, cudaMemcpyHostToDevice, s->st));
        CK(cudaStreamSynchronize(s->st));
        dfree(s, dxy);
        dfree(s, doff);
        dfree(s, dkind);
        dfree(s, dval);
        s->initialized = true;
        return FS_OK;
    }
    // seedInitialFluid (flipsolver2d.cpp:682-707) on the host
    std::vector<int8_t> mat(s->ncell);
    std::vector<float> visc(s->ncell), u(s->nu), v(s->nv);
    CK(cudaMemcpyAsync(mat.data(), s->G.material, s->ncell, cudaMemcpyDeviceToHost, s->st));
    CK(cudaMemcpyAsync(visc.data(), s->G.visc, s->ncell * 4, cudaMemcpyDeviceToHost, s->st));
    CK(cudaMemcpyAsync(u.data(), s->G.u, s->nu * 4, cudaMemcpyDeviceToHost, s->st));
    CK(cudaMemcpyAsync(v.data(), s->G.v, s->nv * 4, cudaMemcpyDeviceToHost, s->st));
    CK(cudaStreamSynchronize(s->st));
    std::mt19937 &rng = s->rng;
    std::uniform_real_distribution<float> dist(0.f, 1.f);
    const int nb = s->P.nbins;
    std::vector<std::vector<float2>> bpos(nb), bvel(nb);
    std::vector<std::vector<float>> bvisc(nb);
    {
        // particles already present stay first in their bins; the seeds are
        // appended (ParticleBin::addMarkerParticle pushes back)
        std::vector<int> st, ct;
        TRY(download_bins(s, st, ct));
        const int nslots = st[nb];
        if (nslots > 0) {
            std::vector<float2> p(nslots), v(nslots);
            std::vector<float> vi(nslots);
            CK(cudaMemcpy(p.data(), s->P.pos, nslots * sizeof(float2), cudaMemcpyDeviceToHost));
            CK(cudaMemcpy(v.data(), s->P.vel, nslots * sizeof(float2), cudaMemcpyDeviceToHost));
            CK(cudaMemcpy(vi.data(), s->P.visc, nslots * sizeof(float), cudaMemcpyDeviceToHost));
            for (int b = 0; b < nb; b++)
                for (int q = st[b]; q < st[b] + ct[b]; q++) {
                    bpos[b].push_back(p[q]);
                    bvel[b].push_back(v[q]);
                    bvisc[b].push_back(vi[q]);
                }
        }
    }
    auto bin_of = [&](long long i, long long j) -> long long {
        long long bi = i / 3, bj = j / 3;
        if (bi < 0 || bi >= d.bni || bj < 0 || bj >= d.bnj) return -1;
        return bi * d.bnj + bj;
    };
    for (long long i = 0; i < d.ni; i++)
        for (long long j = 0; j < d.nj; j++) {
            if (mat[(size_t)i * d.nj + j] != M_FLUID) continue;
            const long long cellbin = bin_of(i, j);
            for (int k = 0; k < s->p.particlesPerCell; k++) {
                float x = (float)i + dist(rng);
                float y = (float)j + dist(rng);
                float vx = h_grid_lerp(u, d.ni + 1, d.nj, 0.5f, 0.f, x, y);
                float vy = h_grid_lerp(v, d.ni, d.nj + 1, 0.f, 0.5f, x, y);
                float vis = h_grid_lerp(visc, d.ni, d.nj, 0.5f, 0.5f, x, y);
                const long long pb = bin_of((long long)x, (long long)y);
                if (pb < 0) continue;
                const size_t idx = bpos[pb].size();
                bpos[pb].push_back(make_float2(x, y));
                bvel[pb].push_back(make_float2(vx, vy));
                bvisc[pb].push_back(0.f);
                // the reference writes the viscosity through the cell's bin at
                // the index returned by the position's bin (:692-702)
                if (idx < bvisc[cellbin].size()) bvisc[cellbin][idx] = vis;
            }
        }
    std::vector<int> counts(nb);
    std::vector<float2> pos, vel;
    std::vector<float> pv;
    for (int b = 0; b < nb; b++) {
        counts[b] = (int)bpos[b].size();
        pos.insert(pos.end(), bpos[b].begin(), bpos[b].end());
        vel.insert(vel.end(), bvel[b].begin(), bvel[b].end());
        pv.insert(pv.end(), bvisc[b].begin(), bvisc[b].end());
    }
    TRY(upload_particles(s, counts, pos, vel, pv));
    if (s->S.n) TRY(rng_to_device(s));
    dfree(s, dxy);
    dfree(s, doff);
    dfree(s, dkind);
    dfree(s, dval);
    s->initialized = true;
    return FS_OK;
}

// ---------------------------------------------------------------------------
// the substep
// ---------------------------------------------------------------------------
template <typename T> static PcgArgs<T> pcg_args(fs_solver *s, const void *b, void *x, int *iters)
{
    PcgArgs<T> a{};
    a.ni = s->d.ni;
    a.nj = s->d.nj;
    a.N = (long long)s->ncell;
    a.info = s->G.cell_info;
    a.b = (const T *)b;
    a.x = (T *)x;
    a.r0 = (T *)s->r0;
    a.r1 = (T *)s->r1;
    a.s0 = (T *)s->s0;
    a.s1 = (T *)s->s1;
    a.ll_r = s->ll.r;
    a.ll_s = s->ll.s;
    a.partials = s->partials;
    a.chunk_end = s->chunk_end;
    a.chunk_last_unit = s->chunk_last;
    a.chunk_val = s->chunk_val;
    a.nchunks = s->nchunks;
    a.sc = s->sc;
    a.density = s->sp.fluidDensity;
    a.dx = s->sp.dx;
    a.iter_limit = s->sp.pcgIterLimit;
    a.tol = s->sp.projectTolerance;
    a.iters_out = iters;
    a.status = &s->sc->pcg_status;
    a.spin_limit = s->ex.wait_polls;
    a.bar = s->bar;
    a.wrap_flag = &s->sc->wrap_units;
    a.mode = 0;
    return a;
}

static ClusterParams spec_params()
{
    ClusterParams cp;
    cp.tol = kSpecRelTol;
    cp.eps_in = 1e-4f;
    cp.max_iter = kSpecMaxIter;
    cp.max_outer = 32;
    return cp;
}

static fs_status run_pcg(fs_solver *s, const void *b, void *x, int *iters)
{
    const int slot = b == s->dens_rhs ? 0 : 1;
    if (s->timers) CK(cudaEventRecord(s->p0[slot], s->st));
    cudaError_t e;
    int launched = 0;
    if (s->prec == FS_PCG_FP64) {
        e = launch_pcg<double>(pcg_args<double>(s, b, x, iters), s->st, &launched);
    } else if (s->prec == FS_PCG_SPEC && s->spec_large) {
        e = launch_spec_chain(s->spec_chain[slot], s->st);
        launched = spec_chain_kernels(s->spec_chain[slot]);
    } else if (s->prec == FS_PCG_SPEC) {
        e = launch_pcg_cluster(s->spec_sys + slot, 1, s->spec_plan, spec_params(), s->st);
        launched = 1;
    } else if (s->resident) {
        PcgArgs<float> pa = pcg_args<float>(s, b, x, iters);
        pa.mode = 2; // unless a unit row sits on a j edge
        e = launch_pcg_resident(pa, s->res_ti, s->res_tj, s->st, &s->ll);
        if (e == cudaSuccess) e = launch_pcg_linear_if_wrap(pa, s->st);
        launched = 2;
    } else if (s->tma) {
        PcgArgs<float> pa = pcg_args<float>(s, b, x, iters);
        pa.mode = 2; // unless a unit row sits on a j edge
        e = launch_pcg_tma(pa, b == s->dens_rhs ? s->maps_dens : s->maps_pres, s->tma_ti,
                           s->tma_tj, s->st);
        if (e == cudaSuccess) e = launch_pcg_linear_if_wrap(pa, s->st);
        launched = 2;
    } else {
        e = launch_pcg<float>(pcg_args<float>(s, b, x, iters), s->st, &launched);
    }
    g_kernel_launches += launched;
    if (e != cudaSuccess) return fail(FS_ERR_CUDA, "PCG launch: %s", cudaGetErrorString(e));
    if (s->timers) {
        CK(cudaEventRecord(s->p1[slot], s->st));
        s->pcg_timed[slot] = true;
    }
    return FS_OK;
}

// adds the PCG times recorded since the last call (waits for them)
static fs_status collect_pcg_timers(fs_solver *s)
{
    for (int k = 0; k < 2; k++) {
        if (!s->pcg_timed[k]) continue;
        CK(cudaEventSynchronize(s->p1[k]));
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, s->p0[k], s->p1[k]));
        s->t_pcg_ms += ms;
        s->pcg_timed[k] = false;
    }
    return FS_OK;
}

static fs_status stage(fs_solver *s, int which, bool in_step)
{
    const GridDims &d = s->d;
    const int dbl = s->prec != FS_PCG_FP32;
    cudaStream_t q = s->st;
    switch (which) {
    case FS_STAGE_ADVECT:
        launch_advect(d, s->P, s->G, s->sc, q);
        g_kernel_launches += 1;
        if (s->nb) { // NBFlipSolver::advect: narrow band, then the grids (:66-109)
            launch_nb_advect_extra(d, s->sp, s->P, s->G, s->N, s->sc, q);
            g_kernel_launches += 2;
        }
        s->after_advect = true;
        break;
    case FS_STAGE_DECOMPOSITION:
        launch_decomposition(d, s->G, s->chunk_last, s->nchunks, s->chunk_ps, s->chunk_rem, s->sc, q);
        g_kernel_launches += 1;
        break;
    case FS_STAGE_REBIN: {
        long long before = g_kernel_launches;
        launch_rebin(d, s->P, s->rebin_scratch, s->rebin_scratch_size, q);
        int bits = 0;
        while ((1 << bits) < s->P.nbins) bits++;
        g_kernel_launches = before + 15 + 5 * ((bits + 7) / 8);
        s->after_advect = false;
        break;
    }
    case FS_STAGE_DENSITY:
        if (s->sp.viscosityEnabled) break;
        launch_density_grid(d, s->sp, s->P, s->G, s->dens_rhs, dbl, s->sc, q);
        g_kernel_launches += 1;
        TRY(run_pcg(s, s->dens_rhs, s->dens_x, &s->sc->density_iters));
        if (s->prec == FS_PCG_SPEC) {
            // the push is skipped only when the solve ran out of iterations
            SceneParams sp = s->sp;
            sp.pcgIterLimit = kSpecMaxIter;
            launch_adjust(d, sp, s->P, s->G, s->dens_x, dbl, s->sc, q);
        } else {
            launch_adjust(d, s->sp, s->P, s->G, s->dens_x, dbl, s->sc, q);
        }
        g_kernel_launches += 1;
        break;
    case FS_STAGE_DENSITY_GRID:
        launch_density_grid(d, s->sp, s->P, s->G, s->dens_rhs, dbl, s->sc, q);
        g_kernel_launches += 1;
        break;
    case FS_STAGE_P2G:
        TRY(wait_side(s)); // the previous level-set pass writes the fluid SDF
        launch_p2g_sdf_materials(d, s->sp, s->P, s->G, s->nb, q);
        g_kernel_launches += 1;
        break;
    case FS_STAGE_SDF: // fused into FS_STAGE_P2G
        break;
    case FS_STAGE_MATERIALS: // fused into FS_STAGE_P2G, except for NB-FLIP
        if (s->nb) {
            launch_nb_materials(d, s->G, q);
            g_kernel_launches += 1;
        }
        break;
    case FS_STAGE_AFTER_TRANSFER: // sources, plus NB-FLIP's combination
        if (s->nb) {
            launch_nb_combine(d, s->G, s->N, s->S, s->p.dx, q);
            g_kernel_launches += 3 + (s->S.n ? 1 : 0);
        } else if (s->S.n) {
            launch_sources_after_transfer(d, s->G, s->S, s->p.dx, q);
            g_kernel_launches += 1;
        }
        break;
    case FS_STAGE_RESEED: // sources, or NB-FLIP's band reseeding
        if (s->nb || (s->S.n && s->R.rng)) {
            launch_nb_candidates(d, s->sp, s->G, s->R, s->S, s->nb, s->nb_scan, q);
            // the candidate total sizes the append's launches (one small read)
            int ncand = 0;
            CK(cudaMemcpyAsync(&ncand, s->R.cand_off + s->ncell, sizeof(int), cudaMemcpyDeviceToHost, q));
            CK(cudaStreamSynchronize(q));
            launch_nb_append(s->P, s->R, ncand, s->rebin_scratch, q);
            int bits = 0;
            while ((1 << bits) < s->P.nbins) bits++;
            g_kernel_launches += 6 + 16 + 5 * ((bits + 7) / 8);
        }
        break;
    case FS_STAGE_LEVELSET_OUTSIDE:
        launch_levelset(d, s->G, true, q, &s->sc->pcg_status, s->ex.wait_polls);
        g_kernel_launches += levelset_launches(d, true);
        break;
    case FS_STAGE_LEVELSET:
        if (in_step && !s->nb) {
            CK(cudaEventRecord(s->ev_p2g, q));
            CK(cudaStreamWaitEvent(s->side, s->ev_p2g, 0));
            launch_levelset(d, s->G, false, s->side, &s->sc->pcg_status, s->ex.wait_polls);
            CK(cudaEventRecord(s->ev_levelset, s->side));
            s->levelset_pending = true;
        } else {
            launch_levelset(d, s->G, false, q, &s->sc->pcg_status, s->ex.wait_polls);
        }
        g_kernel_launches += levelset_launches(d, true);
        break;
    case FS_STAGE_VEL_EXTRAP:
        launch_vel_extrapolate(d, s->G, s->sp, s->sc, false, q);
        g_kernel_launches += 1;
        break;
    case FS_STAGE_SAVE_GRID:
        launch_save_grid(d, s->G, q);
        g_kernel_launches += 1;
        break;
    case FS_STAGE_BODY_FORCES:
        launch_body_forces(d, s->sp, s->G, s->sc, q);
        g_kernel_launches += 1;
        break;
    case FS_STAGE_PROJECT:
        launch_pressure_rhs(d, s->G, s->pres_rhs, dbl, s->sp, q);
        g_kernel_launches += 1;
        TRY(run_pcg(s, s->pres_rhs, s->pres_x, &s->sc->pressure_iters));
        launch_apply_pressure(d, s->sp, s->G, s->pres_x, dbl, s->sc, in_step, q);
        g_kernel_launches += 1;
        break;
    case FS_STAGE_FRICTION:
        if (!in_step) {
            launch_friction(d, s->G, q);
            g_kernel_launches += 1;
        }
        break;
    case FS_STAGE_G2P:
        launch_g2p(d, s->sp, s->P, s->G, s->sc, q);
        g_kernel_launches += 1;
        break;
    case FS_STAGE_COUNT:
        launch_count_erase(d, s->sp, s->P, s->G, q);
        g_kernel_launches += 1;
        break;
    case FS_STAGE_VISCOSITY: { // FlipSolver::applyViscosity (flipsolver2d.cpp:128-136)
        if (!s->sp.viscosityEnabled)
            return fail(FS_ERR_STATE, "FS_STAGE_VISCOSITY: the handle was created without viscosity");
        long long launched = 0;
        const cudaError_t e =
            s->p.useHeavyViscosity
                ? visc_heavy(d, s->G, s->step_dt, (float)s->p.dx, (float)s->sp.fluidDensity, s->visc, q,
                             &s->visc_iters, &launched)
                : visc_light(d, s->G, s->step_dt, (float)s->sp.fluidDensity, s->visc, q, &s->visc_iters,
                             &launched);
        g_kernel_launches += launched;
        if (e != cudaSuccess) return fail(FS_ERR_CUDA, "viscosity: %s", cudaGetErrorString(e));
        break;
    }
    default:
        return fail(FS_ERR_BAD_ARG, "unknown stage %d", which);
    }
    CK(cudaGetLastError());
    return FS_OK;
}

// Timed stage groups end with mark(SolverStage index, flipsolver2d.h:58-72)
// in the order step() ends them (flipsolver2d.cpp:412-462): advect;
// decomposition; prune + rebin; density correction; grid update (P2G, SDF
// and materials, fused here); after transfer (level set, extrapolation,
// saved grid, body forces); pressure; with viscosity, the viscosity model and
// the second projection; particle update (friction is in the pressure apply
// here, then extrapolation and G2P); the last group, count and reseed, ends
// the substep.

// FlipSolver::step (flipsolver2d.cpp:412-462)
template <class Mark> static fs_status step_flip(fs_solver *s, bool timed, Mark &mark)
{
    TRY(stage(s, FS_STAGE_ADVECT, true));
    TRY(mark(0));
    TRY(stage(s, FS_STAGE_DECOMPOSITION, true));
    TRY(mark(1));
    TRY(stage(s, FS_STAGE_REBIN, true));
    TRY(mark(3));
    if (!s->sp.viscosityEnabled) { // densityCorrection and its endStage (:425-430)
        TRY(stage(s, FS_STAGE_DENSITY, true));
        TRY(mark(2));
    }
    TRY(stage(s, FS_STAGE_P2G, true)); // + updateSdf + updateMaterials
    TRY(mark(5));
    if (s->S.n) TRY(stage(s, FS_STAGE_AFTER_TRANSFER, true)); // sources (:435)
    TRY(stage(s, FS_STAGE_LEVELSET, true));
    // extrapolate(10), saved copy and body forces in one pass (:437-440)
    launch_vel_extrapolate(s->d, s->G, s->sp, s->sc, true, s->st);
    g_kernel_launches += 1;
    if (timed) TRY(wait_side(s)); // the level set counts in its own stage
    TRY(mark(6));
    TRY(stage(s, FS_STAGE_PROJECT, true)); // + updateVelocityFromSolids
    TRY(mark(7));
    if (s->sp.viscosityEnabled) { // applyViscosity, then project() again (:448-454)
        TRY(stage(s, FS_STAGE_VISCOSITY, true));
        TRY(mark(8));
        TRY(stage(s, FS_STAGE_PROJECT, false));
        TRY(mark(9));
    }
    TRY(stage(s, FS_STAGE_VEL_EXTRAP, true));
    TRY(stage(s, FS_STAGE_G2P, true));
    TRY(mark(10));
    TRY(stage(s, FS_STAGE_COUNT, true));
    if (s->S.n) TRY(stage(s, FS_STAGE_RESEED, true)); // sources (:460)
    return FS_OK;
}

// NB-FLIP's particle count changes every substep (reseeding): per-slot
// launches are sized by the occupied slots, read here (the stream is idle at
// a substep's start in the frame loop, so the read costs one round trip)
static fs_status nb_refresh_bound(fs_solver *s)
{
    int n = 0;
    CK(cudaMemcpyAsync(&n, s->P.bin_start + s->P.nbins, sizeof(int), cudaMemcpyDeviceToHost, s->st));
    CK(cudaStreamSynchronize(s->st));
    s->P.bound = std::max(1, std::min(n, s->P.cap));
    return FS_OK;
}

// NBFlipSolver::step (nbflipsolver.cpp:26-64) ends its stages as: advection;
// rebin; particle to grid (P2G, extrapolation, saved grid); after transfer
// (inside gridUpdate, :213-225: SDF, outside level set, combination, inside
// level set); grid update (materials, body forces); decomposition; pressure;
// with viscosity, the viscosity model and the second projection (:49-56);
// particle update; reseed
static const int kNbStageOfGroup[9] = {0, 3, 4, 6, 5, 1, 7, 10, 11};

static fs_status step_impl(fs_solver *s)
{
    TRY(ensure_friction(s));
    const bool timed = s->timers && s->stage_ev[0];
    int group = 0;
    auto mark = [&](int solver_stage) -> fs_status {
        if (timed) {
            s->stage_of[group] = solver_stage;
            CK(cudaEventRecord(s->stage_ev[group++], s->st));
        }
        return FS_OK;
    };
    if (s->timers) CK(cudaEventRecord(s->e0, s->st));
    k_set_dt<<<1, 1, 0, s->st>>>(s->sc, s->step_dt);
    g_kernel_launches += 1;
    if (s->nb) {
        TRY(nb_refresh_bound(s));
        static const int groups[9][4] = {
            {FS_STAGE_ADVECT, -1},
            {FS_STAGE_REBIN, -1},
            {FS_STAGE_P2G, FS_STAGE_VEL_EXTRAP, FS_STAGE_SAVE_GRID, -1},
            {FS_STAGE_LEVELSET_OUTSIDE, FS_STAGE_AFTER_TRANSFER, FS_STAGE_LEVELSET, -1},
            {FS_STAGE_MATERIALS, FS_STAGE_BODY_FORCES, -1},
            {FS_STAGE_DECOMPOSITION, -1},
            {FS_STAGE_PROJECT, -1}, // + updateVelocityFromSolids
            {FS_STAGE_VEL_EXTRAP, FS_STAGE_G2P, -1},
            {FS_STAGE_COUNT, FS_STAGE_RESEED, -1}};
        for (int g = 0; g < 9; g++) {
            for (int k = 0; k < 4 && groups[g][k] >= 0; k++) TRY(stage(s, groups[g][k], true));
            if (g < 8) TRY(mark(kNbStageOfGroup[g]));
            if (groups[g][0] == FS_STAGE_PROJECT && s->sp.viscosityEnabled) {
                TRY(stage(s, FS_STAGE_VISCOSITY, true));
                TRY(mark(8));
                TRY(stage(s, FS_STAGE_PROJECT, false));
                TRY(mark(9));
            }
        }
    } else {
        if (s->grows) TRY(nb_refresh_bound(s));
        TRY(step_flip(s, timed, mark));
    }
    if (s->timers) {
        TRY(wait_side(s));
        CK(cudaEventRecord(s->e1, s->st));
        CK(cudaEventSynchronize(s->e1));
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, s->e0, s->e1));
        s->t_step_ms += ms;
        if (timed) {
            cudaEvent_t prev = s->e0;
            for (int g = 0; g <= group; g++) {
                cudaEvent_t cur = g < group ? s->stage_ev[g] : s->e1;
                CK(cudaEventElapsedTime(&ms, prev, cur));
                s->t_stage_ms[g < group ? s->stage_of[g] : 11] += ms; // the last: PARTICLE_RESEED
                prev = cur;
            }
        }
        TRY(collect_pcg_timers(s));
    }
    return FS_OK;
}

// read back the device scalars (one small copy) and fold the iteration counts
// into the frame statistics the way SolverStats does (max over the frame)
static fs_status read_scalars(fs_solver *s)
{
    CK(cudaMemcpyAsync(s->sc_host, s->sc, sizeof(Scalars), cudaMemcpyDeviceToHost, s->st));
    CK(cudaStreamSynchronize(s->st));
    if (s->sc_host->pcg_status != 0)
        return fail(FS_ERR_TIMEOUT, "a PCG grid barrier wait timed out");
    if (s->sc_host->nonfinite != 0) {
        // reported once; the state that produced it stays as it is
        CK(cudaMemsetAsync(&s->sc->nonfinite, 0, sizeof(int), s->st));
        return fail(FS_ERR_NONFINITE, "a substep left a NaN or infinite particle velocity");
    }
    if (s->sc_host->nb_overflow != 0)
        return fail(FS_ERR_UNSUPPORTED,
                    "NB-FLIP reseeding: more than %d candidates left their cell's bin, or the "
                    "particles exceeded the capacity (more than 2 particlesPerCell in a cell)",
                    kNbCrossMax);
    return FS_OK;
}

static fs_status max_velocity(fs_solver *s, float *out)
{
    launch_max_velocity(s->P, s->sc, s->st);
    g_kernel_launches += 2;
    CK(cudaGetLastError());
    TRY(read_scalars(s));
    unsigned bits = s->sc_host->maxv2;
    float v2;
    memcpy(&v2, &bits, 4);
    *out = std::sqrt(v2);
    return FS_OK;
}

extern "C" fs_status fs_step(fs_solver *s)
{
    if (!s) return fail(FS_ERR_BAD_ARG, "null handle");
    TRY(set_device(s));
    CK(cudaMemsetAsync(&s->sc->density_iters, 0, 2 * sizeof(int), s->st));
    s->substeps = 0;
    TRY(step_impl(s));
    s->substeps_total++;
    TRY(read_scalars(s));
    s->density_iters_max = s->sc_host->density_iters;
    s->pressure_iters_max = s->sc_host->pressure_iters;
    return FS_OK;
}

extern "C" fs_status fs_step_frame(fs_solver *s)
{
    if (!s) return fail(FS_ERR_BAD_ARG, "null handle");
    TRY(set_device(s));
    if (s->frame == 0) TRY(fs_first_frame_init(s)); // flipsolver2d.cpp:466-469
    float substepTime = 0.f;
    bool finished = false;
    int substepCount = 0;
    s->density_iters_max = s->pressure_iters_max = s->substeps = 0;
    while (!finished) {
        float vel;
        TRY(max_velocity(s, &vel));
        if (substepCount > 0) {
            s->density_iters_max = std::max(s->density_iters_max, s->sc_host->density_iters);
            s->pressure_iters_max = std::max(s->pressure_iters_max, s->sc_host->pressure_iters);
        }
        float maxSubstepSize = s->p.cflNumber / (vel + 1e-15f);
        if (substepTime + maxSubstepSize >= s->frame_dt || substepCount == (s->p.maxSubsteps - 1)) {
            maxSubstepSize = s->frame_dt - substepTime;
            finished = true;
        } else if (substepTime + 2.f * maxSubstepSize >= s->frame_dt) {
            maxSubstepSize = 0.5f * (s->frame_dt - substepTime);
        }
        s->step_dt = maxSubstepSize;
        CK(cudaMemsetAsync(&s->sc->density_iters, 0, 2 * sizeof(int), s->st));
        TRY(step_impl(s));
        s->substeps++;
        s->substeps_total++;
        substepTime += maxSubstepSize;
        substepCount++;
        if (substepCount > 50) break;
    }
    TRY(read_scalars(s));
    s->density_iters_max = std::max(s->density_iters_max, s->sc_host->density_iters);
    s->pressure_iters_max = std::max(s->pressure_iters_max, s->sc_host->pressure_iters);
    s->frame++;
    return FS_OK;
}

extern "C" fs_status fs_set_step_dt(fs_solver *s, float dt)
{
    if (!s) return fail(FS_ERR_BAD_ARG, "null handle");
    s->step_dt = dt;
    TRY(set_device(s));
    k_set_dt<<<1, 1, 0, s->st>>>(s->sc, dt);
    CK(cudaGetLastError());
    return FS_OK;
}

extern "C" fs_status fs_get_step_dt(fs_solver *s, float *dt)
{
    if (!s || !dt) return fail(FS_ERR_BAD_ARG, "null argument");
    *dt = s->step_dt;
    return FS_OK;
}

extern "C" fs_status fs_run_stage(fs_solver *s, int which)
{
    if (!s) return fail(FS_ERR_BAD_ARG, "null handle");
    TRY(set_device(s));
    TRY(ensure_friction(s));
    // a frame's last level set may still run on the side stream: a stage on
    // its own comes after it (two level sets on one set of buffers race)
    TRY(wait_side(s));
    k_set_dt<<<1, 1, 0, s->st>>>(s->sc, s->step_dt);
    if (s->grows && !s->after_advect) TRY(nb_refresh_bound(s));
    if (which == FS_STAGE_DENSITY) CK(cudaMemsetAsync(&s->sc->density_iters, 0, sizeof(int), s->st));
    if (which == FS_STAGE_PROJECT) CK(cudaMemsetAsync(&s->sc->pressure_iters, 0, sizeof(int), s->st));
    TRY(stage(s, which, false));
    TRY(sync_all(s));
    TRY(collect_pcg_timers(s));
    TRY(read_scalars(s));
    if (which == FS_STAGE_DENSITY) s->density_iters_max = s->sc_host->density_iters;
    if (which == FS_STAGE_PROJECT) s->pressure_iters_max = s->sc_host->pressure_iters;
    return FS_OK;
}

extern "C" fs_status fs_max_particle_velocity(fs_solver *s, float *out)
{
    if (!s || !out) return fail(FS_ERR_BAD_ARG, "null argument");
    TRY(set_device(s));
    return max_velocity(s, out);
}

// ---------------------------------------------------------------------------
// state access
// ---------------------------------------------------------------------------
extern "C" fs_status fs_bin_count(fs_solver *s, size_t *n)
{
    if (!s || !n) return fail(FS_ERR_BAD_ARG, "null argument");
    *n = (size_t)s->P.nbins;
    return FS_OK;
}

static fs_status download_bins(fs_solver *s, std::vector<int> &start, std::vector<int> &count)
{
    start.resize(s->P.nbins + 1);
    count.resize(s->P.nbins);
    CK(cudaMemcpyAsync(start.data(), s->P.bin_start, start.size() * 4, cudaMemcpyDeviceToHost, s->st));
    CK(cudaMemcpyAsync(count.data(), s->P.bin_count, count.size() * 4, cudaMemcpyDeviceToHost, s->st));
    CK(cudaStreamSynchronize(s->st));
    return FS_OK;
}

extern "C" fs_status fs_particle_count(fs_solver *s, size_t *n)
{
    if (!s || !n) return fail(FS_ERR_BAD_ARG, "null argument");
    TRY(set_device(s));
    TRY(sync_all(s));
    std::vector<int> st, ct;
    TRY(download_bins(s, st, ct));
    size_t t = 0;
    for (int c : ct) t += (size_t)c;
    *n = t;
    return FS_OK;
}

extern "C" fs_status fs_get_particles(fs_solver *s, int32_t *bin_counts, float *pos_xy,
                                      float *vel_xy, float *visc, uint8_t *dead)
{
    if (!s) return fail(FS_ERR_BAD_ARG, "null handle");
    TRY(set_device(s));
    TRY(sync_all(s));
    if (!s->after_advect && s->P.cap > 0) {
        // outside a substep no particle is marked: pack the bins on the
        // device and copy each array straight into the caller's memory
        // (pinned caller memory makes these full-bandwidth copies)
        const Particles &P = s->P;
        launch_gather_bins(P, s->rebin_scratch, s->st);
        g_kernel_launches += 4;
        int total = 0;
        CK(cudaMemcpyAsync(&total, P.bin_start2 + P.nbins, sizeof(int), cudaMemcpyDeviceToHost, s->st));
        CK(cudaStreamSynchronize(s->st));
        if (bin_counts)
            CK(cudaMemcpyAsync(bin_counts, P.bin_count, (size_t)P.nbins * 4, cudaMemcpyDeviceToHost, s->st));
        if (total > 0) {
            if (pos_xy)
                CK(cudaMemcpyAsync(pos_xy, P.pos2, (size_t)total * sizeof(float2), cudaMemcpyDeviceToHost, s->st));
            if (vel_xy)
                CK(cudaMemcpyAsync(vel_xy, P.vel2, (size_t)total * sizeof(float2), cudaMemcpyDeviceToHost, s->st));
            if (visc) CK(cudaMemcpyAsync(visc, P.visc2, (size_t)total * sizeof(float), cudaMemcpyDeviceToHost, s->st));
        }
        CK(cudaStreamSynchronize(s->st));
        if (dead) memset(dead, 0, (size_t)total);
        return FS_OK;
    }
    std::vector<int> st, ct;
    TRY(download_bins(s, st, ct));
    const int nslots = st[s->P.nbins];
    std::vector<float2> p(nslots), v(nslots);
    std::vector<float> vi(nslots);
    std::vector<uint8_t> fl(nslots, 0);
    if (nslots) {
        CK(cudaMemcpy(p.data(), s->P.pos, nslots * sizeof(float2), cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(v.data(), s->P.vel, nslots * sizeof(float2), cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(vi.data(), s->P.visc, nslots * sizeof(float), cudaMemcpyDeviceToHost));
        if (s->after_advect) CK(cudaMemcpy(fl.data(), s->P.flag, nslots, cudaMemcpyDeviceToHost));
    }
    size_t k = 0;
    for (int b = 0; b < s->P.nbins; b++) {
        if (bin_counts) bin_counts[b] = ct[b];
        for (int q = st[b]; q < st[b] + ct[b]; q++, k++) {
            if (pos_xy) {
                pos_xy[2 * k] = p[q].x;
                pos_xy[2 * k + 1] = p[q].y;
            }
            if (vel_xy) {
                vel_xy[2 * k] = v[q].x;
                vel_xy[2 * k + 1] = v[q].y;
            }
            if (visc) visc[k] = vi[q];
            if (dead) dead[k] = (s->after_advect && fl[q] != P_STAY) ? 1 : 0;
        }
    }
    return FS_OK;
}

// whether any of n bytes is nonzero: an OR over 8-byte words, no early exit,
// so the loop vectorises
static bool any_nonzero(const uint8_t *p, size_t n)
{
    uint64_t acc = 0;
    size_t k = 0;
    for (; k + 8 <= n; k += 8) {
        uint64_t w;
        memcpy(&w, p + k, 8);
        acc |= w;
    }
    for (; k < n; k++) acc |= p[k];
    return acc != 0;
}

extern "C" fs_status fs_set_particles(fs_solver *s, const int32_t *bin_counts, const float *pos_xy,
                                      const float *vel_xy, const float *visc, const uint8_t *dead)
{
    if (!s || !bin_counts || !pos_xy || !vel_xy || !visc)
        return fail(FS_ERR_BAD_ARG, "null argument");
    TRY(set_device(s));
    TRY(sync_all(s));
    const int nb = s->P.nbins;
    size_t total = 0;
    bool negative = false;
    for (int b = 0; b < nb; b++) {
        negative |= bin_counts[b] < 0;
        total += (size_t)(unsigned)bin_counts[b];
    }
    if (negative) return fail(FS_ERR_BAD_ARG, "negative bin count");
    if (total > (size_t)INT32_MAX / 2) return fail(FS_ERR_BAD_ARG, "too many particles");
    if (dead && any_nonzero(dead, total))
        return fail(FS_ERR_UNSUPPORTED, "particles marked for death can only exist inside a substep");
    // the positions and velocities are float pairs already: copy them
    // straight from the caller's memory; the slot-to-bin map is built on the
    // device
    if ((int)total > s->P.cap || s->P.pos == nullptr) {
        // NB-FLIP keeps room for 2 particlesPerCell per cell (reseeding)
        const long long keep = s->grows ? 2LL * s->p.particlesPerCell * (long long)s->ncell : 0;
        TRY(alloc_particles(s, (int)std::max<long long>((long long)total, keep)));
    }
    Particles &P = s->P;
    // the counts straight from the caller's memory; the bin starts by a device
    // scan of them (pinned caller memory then needs no staging copy)
    CK(cudaMemcpyAsync(P.bin_count, bin_counts, nb * sizeof(int), cudaMemcpyHostToDevice, s->st));
    if (s->rebin_scratch && scan_scratch_bytes(nb) <= s->rebin_scratch_size) {
        scan_exclusive(P.bin_count, P.bin_start, nb, s->rebin_scratch, s->st);
        g_kernel_launches += 3;
    } else {
        std::vector<int> start(nb + 1, 0);
        for (int b = 0; b < nb; b++) start[b + 1] = start[b] + bin_counts[b];
        CK(cudaMemcpyAsync(P.bin_start, start.data(), (nb + 1) * sizeof(int), cudaMemcpyHostToDevice,
                           s->st));
    }
    if (total) {
        CK(cudaMemcpyAsync(P.pos, pos_xy, total * sizeof(float2), cudaMemcpyHostToDevice, s->st));
        CK(cudaMemcpyAsync(P.vel, vel_xy, total * sizeof(float2), cudaMemcpyHostToDevice, s->st));
        CK(cudaMemcpyAsync(P.visc, visc, total * sizeof(float), cudaMemcpyHostToDevice, s->st));
        launch_slot_bin(P, s->st);
        g_kernel_launches += 1;
    }
    CK(cudaStreamSynchronize(s->st));
    CK(cudaGetLastError());
    s->after_advect = false;
    s->initialized = true;
    if (s->grows) P.bound = std::max((int)total, 1);
    return FS_OK;
}

struct GridRef {
    void *ptr;
    size_t elems;
    int elem_size;   // bytes on the device
    int host_size;   // bytes in the API (double for the solver vectors)
    bool solver_vec; // device element is the PCG precision
};

static bool grid_ref(fs_solver *s, int which, GridRef &g)
{
    const size_t n = s->ncell;
    const int e = (int)s->esz;
    switch (which) {
    case FS_GRID_MATERIAL: g = {s->G.material, n, 1, 1, false}; return true;
    case FS_GRID_SOLID_SDF: g = {s->G.solid_sdf, n, 4, 4, false}; return true;
    case FS_GRID_FLUID_SDF: g = {s->G.fluid_sdf, n, 4, 4, false}; return true;
    case FS_GRID_U: g = {s->G.u, s->nu, 4, 4, false}; return true;
    case FS_GRID_V: g = {s->G.v, s->nv, 4, 4, false}; return true;
    case FS_GRID_U_VALID: g = {s->G.uvalid, s->nu, 1, 1, false}; return true;
    case FS_GRID_V_VALID: g = {s->G.vvalid, s->nv, 1, 1, false}; return true;
    case FS_GRID_SAVED_U: g = {s->G.su, s->nu, 4, 4, false}; return true;
    case FS_GRID_SAVED_V: g = {s->G.sv, s->nv, 4, 4, false}; return true;
    case FS_GRID_VISCOSITY: g = {s->G.visc, n, 4, 4, false}; return true;
    case FS_GRID_KNOWN_CENTERED: g = {s->G.known, n, 1, 1, false}; return true;
    case FS_GRID_DENSITY: g = {s->G.density, n, 4, 4, false}; return true;
    case FS_GRID_PARTICLE_COUNTS: g = {s->G.counts, n, 4, 4, false}; return true;
    case FS_GRID_SOLID_ID: g = {s->G.solid_id, n, 4, 4, false}; return true;
    case FS_GRID_DIV_CONTROL: g = {s->G.divc, n, 4, 4, false}; return true;
    case FS_GRID_DENSITY_RHS: g = {s->dens_rhs, n, e, 8, true}; return true;
    case FS_GRID_DENSITY_PRESSURE: g = {s->dens_x, n, e, 8, true}; return true;
    case FS_GRID_PRESSURE: g = {s->pres_x, n, e, 8, true}; return true;
    case FS_GRID_PRESSURE_RHS: g = {s->pres_rhs, n, e, 8, true}; return true;
    case FS_GRID_EMITTER_ID: g = {s->G.emitter_id, n, 4, 4, false}; return true;
    case FS_GRID_ADVECTED_U: g = {s->N.adv_u, s->nu, 4, 4, false}; return s->nb;
    case FS_GRID_ADVECTED_V: g = {s->N.adv_v, s->nv, 4, 4, false}; return s->nb;
    case FS_GRID_ADVECTED_SDF: g = {s->N.adv_sdf, n, 4, 4, false}; return s->nb;
    case FS_GRID_ADVECTED_VISCOSITY: g = {s->N.adv_visc, n, 4, 4, false}; return s->nb;
    default: return false;
    }
}

extern "C" fs_status fs_grid_bytes(fs_solver *s, int which, size_t *bytes)
{
    GridRef g;
    if (!s || !bytes || !grid_ref(s, which, g)) return fail(FS_ERR_BAD_ARG, "bad grid id");
    *bytes = g.elems * g.host_size;
    return FS_OK;
}

extern "C" fs_status fs_get_grid(fs_solver *s, int which, void *out, size_t bytes)
{
    GridRef g;
    if (!s || !out || !grid_ref(s, which, g)) return fail(FS_ERR_BAD_ARG, "bad grid id");
    if (bytes != g.elems * g.host_size) return fail(FS_ERR_BAD_ARG, "grid size mismatch");
    TRY(set_device(s));
    TRY(sync_all(s));
    if (g.solver_vec && g.elem_size == 4) {
        std::vector<float> tmp(g.elems);
        CK(cudaMemcpy(tmp.data(), g.ptr, g.elems * 4, cudaMemcpyDeviceToHost));
        double *o = (double *)out;
        for (size_t k = 0; k < g.elems; k++) o[k] = tmp[k];
    } else {
        CK(cudaMemcpy(out, g.ptr, bytes, cudaMemcpyDeviceToHost));
    }
    return FS_OK;
}

extern "C" fs_status fs_set_grid(fs_solver *s, int which, const void *in, size_t bytes)
{
    GridRef g;
    if (!s || !in || !grid_ref(s, which, g)) return fail(FS_ERR_BAD_ARG, "bad grid id");
    if (bytes != g.elems * g.host_size) return fail(FS_ERR_BAD_ARG, "grid size mismatch");
    TRY(set_device(s));
    TRY(sync_all(s));
    if (g.solver_vec && g.elem_size == 4) {
        std::vector<float> tmp(g.elems);
        const double *src = (const double *)in;
        for (size_t k = 0; k < g.elems; k++) tmp[k] = (float)src[k];
        CK(cudaMemcpy(g.ptr, tmp.data(), g.elems * 4, cudaMemcpyHostToDevice));
    } else {
        CK(cudaMemcpy(g.ptr, in, bytes, cudaMemcpyHostToDevice));
    }
    if (which == FS_GRID_MATERIAL || which == FS_GRID_SOLID_ID) s->friction_dirty = true;
    return FS_OK;
}

extern "C" fs_status fs_get_stat(fs_solver *s, int which, int *out)
{
    if (!s || !out) return fail(FS_ERR_BAD_ARG, "null argument");
    switch (which) {
    case FS_STAT_DENSITY_ITERS: *out = s->density_iters_max; return FS_OK;
    case FS_STAT_PRESSURE_ITERS: *out = s->pressure_iters_max; return FS_OK;
    case FS_STAT_SUBSTEPS: *out = s->substeps; return FS_OK;
    case FS_STAT_FRAME: *out = s->frame; return FS_OK;
    case FS_STAT_POOL_THREADS: *out = s->ex.pool_threads; return FS_OK;
    case FS_STAT_SUBSTEPS_TOTAL: *out = (int)s->substeps_total; return FS_OK;
    case FS_STAT_VISCOSITY_ITERS: *out = s->visc_iters; return FS_OK;
    default: return fail(FS_ERR_BAD_ARG, "bad stat id");
    }
}

extern "C" fs_status fs_enable_timers(fs_solver *s, int enable)
{
    if (!s) return fail(FS_ERR_BAD_ARG, "null handle");
    if (enable && !s->stage_ev[0]) {
        TRY(set_device(s));
        for (cudaEvent_t &e : s->stage_ev) CK(cudaEventCreate(&e));
    }
    s->timers = enable != 0;
    return FS_OK;
}

extern "C" fs_status fs_reset_timers(fs_solver *s)
{
    if (!s) return fail(FS_ERR_BAD_ARG, "null handle");
    s->t_step_ms = s->t_pcg_ms = 0.0;
    for (double &t : s->t_stage_ms) t = 0.0;
    g_kernel_launches = 0;
    return FS_OK;
}

extern "C" fs_status fs_get_timer(fs_solver *s, int which, double *value)
{
    if (!s || !value) return fail(FS_ERR_BAD_ARG, "null argument");
    switch (which) {
    case 0: *value = s->t_step_ms; return FS_OK;
    case 1: *value = s->t_pcg_ms; return FS_OK;
    case 2: *value = (double)g_kernel_launches.load(); return FS_OK;
    default: return fail(FS_ERR_BAD_ARG, "bad timer id");
    }
}

extern "C" fs_status fs_get_stage_time(fs_solver *s, int stage, double *ms)
{
    if (!s || !ms || stage < 0 || stage >= 12) return fail(FS_ERR_BAD_ARG, "fs_get_stage_time: invalid argument");
    *ms = s->t_stage_ms[stage];
    return FS_OK;
}

extern "C" fs_status fs_get_stream(fs_solver *s, void **stream)
{
    if (!s || !stream) return fail(FS_ERR_BAD_ARG, "null argument");
    *stream = (void *)s->st;
    return FS_OK;
}

extern "C" fs_status fs_device_bytes(fs_solver *s, size_t *bytes)
{
    if (!s || !bytes) return fail(FS_ERR_BAD_ARG, "null argument");
    *bytes = s->device_bytes;
    return FS_OK;
}

extern "C" fs_status fs_synchronize(fs_solver *s)
{
    if (!s) return fail(FS_ERR_BAD_ARG, "null handle");
    TRY(set_device(s));
    return sync_all(s);
}

// ---------------------------------------------------------------------------
// fs_batch: solver handles stepped together (no reference counterpart)
//
// Every handle advances by whole frames with the CFL loop of fs_step_frame
// (FlipSolver::stepFrame, flipsolver2d.cpp:464-500), substep by substep.  The
// handles' substeps run in rounds: in a round every handle still inside its
// frame runs one substep.  A substep is three captured CUDA graphs per handle
// (everything before the density solve; between the solves; after the
// pressure solve, ending with the max-velocity reduction the next round's dt
// needs), and the density and pressure solves of all those handles are one
// cluster launch per plan (fs_cluster.cu) in between.  The host waits once
// per round, for the max velocities.
//
// A substep swaps the particle buffers once (the rebin) and the velocity
// grids twice, so the device pointers a substep uses repeat with period two:
// two versions of each graph are captured, for even and odd substeps, and
// the handle's host-side pointer state follows the parity.
// ---------------------------------------------------------------------------
static bool valid_material(const int8_t *m, size_t n);

struct BatchScene {
    fs_solver *s = nullptr;
    int slot = 0; // its entry in the batch's dt table (fixed while it is a member)
    cudaGraphExec_t g[2][3] = {{nullptr, nullptr, nullptr}, {nullptr, nullptr, nullptr}};
    long long launches[3] = {0, 0, 0};
    Particles P[2];
    Grids G[2];
    int parity = 0;
    cudaEvent_t ev = nullptr;
    // the frame in progress (fs_step_frame's locals)
    bool in_frame = false;
    bool last = false; // the substep of this round ends the frame
    float substep_time = 0.f;
    int substep_count = 0;
};

// a standalone system submitted to the batch: device copies of its arrays
struct BatchSolve {
    unsigned long long ticket = 0;
    int ni = 0, nj = 0;
    void *mem = nullptr; // one allocation: material, info, b, x, dt, iters, rel
    ClusterSystem sys{};
    ClusterPlan plan{};
    bool done = false;
    bool large = false; // above the on-chip limit: a chained solve
    SpecSolve chain{};
    void *chain_mem = nullptr;
    LlBuffers ll; // its resident inner solves' exchange words (in chain_mem)
};

struct fs_batch {
    std::vector<BatchScene> sc;
    std::vector<BatchSolve> solves;
    unsigned long long next_ticket = 1;
    int device = 0;
    static constexpr int kSlots = 4096;
    std::vector<int> free_slots;
    cudaStream_t bst = nullptr; // merged solves
    cudaEvent_t ev_solve = nullptr;
    float *d_dt = nullptr, *h_dt = nullptr;              // kSlots
    ClusterSystem *d_list = nullptr, *h_list = nullptr; // two lists of list_cap
    size_t list_cap = 0;
    int *chunk_last = nullptr; // decomposition scratch of submitted systems
    Scalars *dsc = nullptr;
    cudaEvent_t ev_t[4] = {nullptr, nullptr, nullptr, nullptr}; // merged solves, timed
    // one stream per plan group, so that clusters of different sizes share
    // the SMs (a GPC left over by 16-CTA clusters takes smaller ones)
    static constexpr int kGroups = 6;
    cudaStream_t gst[kGroups] = {};
    cudaEvent_t gev[kGroups] = {};
    cudaEvent_t ev_fork = nullptr;
    double solve_ms = 0.0, frame_ms = 0.0;
    long long rounds = 0;
};

static fs_status batch_capture(fs_batch *b, BatchScene &bs, int parity)
{
    fs_solver *s = bs.s;
    const GridDims &d = s->d;
    const int dbl = 1;
    cudaStream_t q = s->st;
    for (int seg = 0; seg < 3; seg++) {
        const long long before = g_kernel_launches;
        CK(cudaStreamBeginCapture(q, cudaStreamCaptureModeRelaxed));
        fs_status st = FS_OK;
        if (seg == 0) {
            k_set_dt_from<<<1, 1, 0, q>>>(s->sc, b->d_dt + bs.slot);
            g_kernel_launches += 1;
            cudaMemsetAsync(&s->sc->density_iters, 0, 2 * sizeof(int), q);
            st = stage(s, FS_STAGE_ADVECT, true);
            if (st == FS_OK) st = stage(s, FS_STAGE_DECOMPOSITION, true);
            if (st == FS_OK) st = stage(s, FS_STAGE_REBIN, true);
            if (st == FS_OK) {
                launch_density_grid(d, s->sp, s->P, s->G, s->dens_rhs, dbl, s->sc, q);
                g_kernel_launches += 1;
                if (s->spec_large) { // its own chained solve, not a merged one
                    if (launch_spec_chain(s->spec_chain[0], q) != cudaSuccess)
                        st = fail(FS_ERR_CUDA, "fs_batch: capture of a chained solve");
                    g_kernel_launches += spec_chain_kernels(s->spec_chain[0]);
                }
            }
        } else if (seg == 1) {
            SceneParams sp = s->sp;
            sp.pcgIterLimit = kSpecMaxIter;
            launch_adjust(d, sp, s->P, s->G, s->dens_x, dbl, s->sc, q);
            g_kernel_launches += 1;
            st = stage(s, FS_STAGE_P2G, true);
            if (st == FS_OK) st = stage(s, FS_STAGE_LEVELSET, true);
            if (st == FS_OK) {
                launch_vel_extrapolate(d, s->G, s->sp, s->sc, true, q);
                launch_pressure_rhs(d, s->G, s->pres_rhs, dbl, s->sp, q);
                g_kernel_launches += 2;
                st = wait_side(s); // the level set joins before the graph ends
                if (st == FS_OK && s->spec_large) {
                    if (launch_spec_chain(s->spec_chain[1], q) != cudaSuccess)
                        st = fail(FS_ERR_CUDA, "fs_batch: capture of a chained solve");
                    g_kernel_launches += spec_chain_kernels(s->spec_chain[1]);
                }
            }
        } else {
            launch_apply_pressure(d, s->sp, s->G, s->pres_x, dbl, s->sc, true, q);
            g_kernel_launches += 1;
            st = stage(s, FS_STAGE_VEL_EXTRAP, true);
            if (st == FS_OK) st = stage(s, FS_STAGE_G2P, true);
            if (st == FS_OK) st = stage(s, FS_STAGE_COUNT, true);
            if (st == FS_OK) {
                launch_max_velocity(s->P, s->sc, q);
                g_kernel_launches += 2;
                cudaMemcpyAsync(s->sc_host, s->sc, sizeof(Scalars), cudaMemcpyDeviceToHost, q);
            }
        }
        cudaGraph_t graph = nullptr;
        const cudaError_t ec = cudaStreamEndCapture(q, &graph);
        if (st != FS_OK) {
            if (graph) cudaGraphDestroy(graph);
            return st;
        }
        if (ec != cudaSuccess) return fail(FS_ERR_CUDA, "fs_batch: capture: %s", cudaGetErrorString(ec));
        const cudaError_t ei = cudaGraphInstantiate(&bs.g[parity][seg], graph, 0);
        cudaGraphDestroy(graph);
        if (ei != cudaSuccess) return fail(FS_ERR_CUDA, "fs_batch: instantiate: %s", cudaGetErrorString(ei));
        bs.launches[seg] = g_kernel_launches - before;
    }
    return FS_OK;
}

static void batch_release_graphs(BatchScene &bs)
{
    for (auto &row : bs.g)
        for (cudaGraphExec_t &e : row) {
            if (e) cudaGraphExecDestroy(e);
            e = nullptr;
        }
}

// captures both substep parities from the handle's current buffers; the
// handle's host-side pointer state is left as it was
static fs_status batch_prepare(fs_batch *b, BatchScene &bs)
{
    fs_solver *s = bs.s;
    batch_release_graphs(bs);
    TRY(ensure_friction(s));
    TRY(sync_all(s));
    bs.P[0] = s->P;
    bs.G[0] = s->G;
    fs_status st = batch_capture(b, bs, 0);
    if (st == FS_OK) {
        bs.P[1] = s->P;
        bs.G[1] = s->G;
        st = batch_capture(b, bs, 1);
    }
    const bool back = memcmp(&s->P, &bs.P[0], sizeof(Particles)) == 0 &&
                      memcmp(&s->G, &bs.G[0], sizeof(Grids)) == 0;
    s->P = bs.P[0];
    s->G = bs.G[0];
    bs.parity = 0;
    if (st == FS_OK && !back) st = fail(FS_ERR_CUDA, "fs_batch: substep buffers do not repeat");
    if (st != FS_OK) batch_release_graphs(bs);
    return st;
}

static BatchScene *batch_find(fs_batch *b, fs_solver *s)
{
    for (BatchScene &bs : b->sc)
        if (bs.s == s) return &bs;
    return nullptr;
}

static fs_status batch_check_handle(fs_batch *b, fs_solver *s, const char *where)
{
    if (!s) return fail(FS_ERR_BAD_ARG, "%s: null handle", where);
    if (s->prec != FS_PCG_SPEC) return fail(FS_ERR_UNSUPPORTED, "%s: the handle is not in FS_PCG_SPEC mode", where);
    if (s->ex.device != b->device) return fail(FS_ERR_BAD_ARG, "%s: the handle is on another device", where);
    if (s->timers) return fail(FS_ERR_UNSUPPORTED, "%s: the handle has timers on", where);
    return FS_OK;
}

extern "C" fs_status fs_batch_destroy(fs_batch *b)
{
    if (!b) return FS_OK;
    cudaSetDevice(b->device);
    cudaDeviceSynchronize();
    for (BatchScene &bs : b->sc) {
        batch_release_graphs(bs);
        if (bs.ev) cudaEventDestroy(bs.ev);
    }
    for (BatchSolve &q : b->solves) {
        if (q.mem) cudaFree(q.mem);
        if (q.chain_mem) cudaFree(q.chain_mem);
    }
    if (b->ev_solve) cudaEventDestroy(b->ev_solve);
    for (cudaEvent_t e : b->ev_t)
        if (e) cudaEventDestroy(e);
    for (int g = 0; g < fs_batch::kGroups; g++) {
        if (b->gst[g]) cudaStreamDestroy(b->gst[g]);
        if (b->gev[g]) cudaEventDestroy(b->gev[g]);
    }
    if (b->ev_fork) cudaEventDestroy(b->ev_fork);
    if (b->bst) cudaStreamDestroy(b->bst);
    if (b->d_dt) cudaFree(b->d_dt);
    if (b->d_list) cudaFree(b->d_list);
    if (b->chunk_last) cudaFree(b->chunk_last);
    if (b->dsc) cudaFree(b->dsc);
    if (b->h_dt) cudaFreeHost(b->h_dt);
    if (b->h_list) cudaFreeHost(b->h_list);
    delete b;
    return FS_OK;
}

extern "C" fs_status fs_batch_add(fs_batch *b, fs_solver *s)
{
    if (!b) return fail(FS_ERR_BAD_ARG, "null batch");
    TRY(batch_check_handle(b, s, "fs_batch_add"));
    if (batch_find(b, s)) return fail(FS_ERR_BAD_ARG, "fs_batch_add: the handle is already a member");
    if (b->free_slots.empty()) return fail(FS_ERR_BAD_ARG, "fs_batch_add: the batch is full (%d)", fs_batch::kSlots);
    if (s->nb) return fail(FS_ERR_UNSUPPORTED, "fs_batch_add: NB-FLIP scenes step on their own");
    if (!s->src_params.empty())
        return fail(FS_ERR_UNSUPPORTED, "fs_batch_add: scenes with sources step on their own");
    // the viscosity solve reads its stopping flag on the host between
    // iteration batches, which a captured substep graph cannot
    if (s->sp.viscosityEnabled)
        return fail(FS_ERR_UNSUPPORTED, "fs_batch_add: scenes with viscosity step on their own");
    CK(cudaSetDevice(b->device));
    BatchScene bs;
    bs.s = s;
    if (cudaEventCreateWithFlags(&bs.ev, cudaEventDisableTiming) != cudaSuccess)
        return fail(FS_ERR_CUDA, "fs_batch_add: event");
    bs.slot = b->free_slots.back();
    // a handle that has not stepped yet is captured at its first frame,
    // once its particles exist
    if (s->frame > 0) {
        const fs_status st = batch_prepare(b, bs);
        if (st != FS_OK) {
            cudaEventDestroy(bs.ev);
            return st;
        }
    }
    b->free_slots.pop_back();
    b->sc.push_back(bs);
    return FS_OK;
}

extern "C" fs_status fs_batch_remove(fs_batch *b, fs_solver *s)
{
    if (!b || !s) return fail(FS_ERR_BAD_ARG, "null argument");
    for (size_t k = 0; k < b->sc.size(); k++) {
        BatchScene &bs = b->sc[k];
        if (bs.s != s) continue;
        if (bs.in_frame) return fail(FS_ERR_BAD_ARG, "fs_batch_remove: the handle is inside a frame");
        CK(cudaSetDevice(b->device));
        TRY(sync_all(s));
        batch_release_graphs(bs);
        if (bs.ev) cudaEventDestroy(bs.ev);
        b->free_slots.push_back(bs.slot);
        b->sc.erase(b->sc.begin() + (long)k);
        return FS_OK;
    }
    return fail(FS_ERR_BAD_ARG, "fs_batch_remove: not a member");
}

extern "C" fs_status fs_batch_create(fs_solver *const *solvers, int n, fs_batch **out)
{
    if (!out || n < 0 || (n > 0 && !solvers)) return fail(FS_ERR_BAD_ARG, "fs_batch_create: invalid argument");
    *out = nullptr;
    int dev = 0;
    if (n > 0) {
        if (!solvers[0]) return fail(FS_ERR_BAD_ARG, "fs_batch_create: null handle 0");
        dev = solvers[0]->ex.device;
    } else {
        CK(cudaGetDevice(&dev));
    }
    fs_batch *b = new fs_batch();
    b->device = dev;
    auto cleanup = [&](fs_status st) {
        fs_batch_destroy(b);
        return st;
    };
    if (cudaSetDevice(b->device) != cudaSuccess) return cleanup(fail(FS_ERR_CUDA, "fs_batch_create: device"));
    if (cudaStreamCreateWithFlags(&b->bst, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->ev_solve, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreate(&b->ev_t[0]) != cudaSuccess || cudaEventCreate(&b->ev_t[1]) != cudaSuccess ||
        cudaEventCreate(&b->ev_t[2]) != cudaSuccess || cudaEventCreate(&b->ev_t[3]) != cudaSuccess ||
        cudaMalloc(&b->d_dt, (size_t)fs_batch::kSlots * sizeof(float)) != cudaSuccess ||
        cudaMallocHost(&b->h_dt, (size_t)fs_batch::kSlots * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&b->chunk_last, 2 * sizeof(int)) != cudaSuccess ||
        cudaMalloc(&b->dsc, sizeof(Scalars)) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming) != cudaSuccess)
        return cleanup(fail(FS_ERR_OOM, "fs_batch_create: allocation failed"));
    for (int g = 0; g < fs_batch::kGroups; g++)
        if (cudaStreamCreateWithFlags(&b->gst[g], cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&b->gev[g], cudaEventDisableTiming) != cudaSuccess)
            return cleanup(fail(FS_ERR_CUDA, "fs_batch_create: stream"));
    if (cudaMemset(b->dsc, 0, sizeof(Scalars)) != cudaSuccess)
        return cleanup(fail(FS_ERR_CUDA, "fs_batch_create: memset"));
    for (int k = fs_batch::kSlots - 1; k >= 0; k--) b->free_slots.push_back(k);
    for (int k = 0; k < n; k++) {
        const fs_status st = fs_batch_add(b, solvers[k]);
        if (st != FS_OK) return cleanup(st);
    }
    *out = b;
    return FS_OK;
}

// starts a frame of a member (fs_step_frame's set-up): first-frame seeding at
// frame 0, a new capture if the handle's buffers moved since the last one
// (seeding, fs_set_particles, ...), and the max velocity the first substep's
// dt needs (into the pinned scalars; waited for before the round reads it)
static fs_status batch_begin(fs_batch *b, BatchScene &bs)
{
    fs_solver *s = bs.s;
    if (s->frame == 0) TRY(fs_first_frame_init(s));
    TRY(sync_all(s));
    if (!bs.g[0][0] || memcmp(&s->P, &bs.P[bs.parity], sizeof(Particles)) != 0 ||
        memcmp(&s->G, &bs.G[bs.parity], sizeof(Grids)) != 0)
        TRY(batch_prepare(b, bs));
    launch_max_velocity(s->P, s->sc, s->st);
    g_kernel_launches += 2;
    CK(cudaMemcpyAsync(s->sc_host, s->sc, sizeof(Scalars), cudaMemcpyDeviceToHost, s->st));
    bs.substep_time = 0.f;
    bs.substep_count = 0;
    bs.in_frame = true;
    s->density_iters_max = s->pressure_iters_max = s->substeps = 0;
    return FS_OK;
}

extern "C" fs_status fs_batch_begin_frame(fs_batch *b, fs_solver *s)
{
    if (!b) return fail(FS_ERR_BAD_ARG, "null batch");
    BatchScene *bs = batch_find(b, s);
    if (!bs) return fail(FS_ERR_BAD_ARG, "fs_batch_begin_frame: not a member");
    if (bs->in_frame) return fail(FS_ERR_BAD_ARG, "fs_batch_begin_frame: the handle is inside a frame");
    CK(cudaSetDevice(b->device));
    TRY(batch_begin(b, *bs));
    CK(cudaStreamSynchronize(s->st));
    return FS_OK;
}

extern "C" fs_status fs_batch_in_frame(fs_batch *b, fs_solver *s, int *in_frame)
{
    if (!b || !in_frame) return fail(FS_ERR_BAD_ARG, "null argument");
    BatchScene *bs = batch_find(b, s);
    if (!bs) return fail(FS_ERR_BAD_ARG, "fs_batch_in_frame: not a member");
    *in_frame = bs->in_frame ? 1 : 0;
    return FS_OK;
}

extern "C" fs_status fs_batch_submit_solve(fs_batch *b, const fs_poisson_system *q, unsigned long long *ticket)
{
    if (!b || !q || !ticket || q->ni < 1 || q->nj < 1 || !q->material || !q->rhs)
        return fail(FS_ERR_BAD_ARG, "fs_batch_submit_solve: invalid argument");
    const size_t N = (size_t)q->ni * q->nj;
    if (!valid_material(q->material, N)) return fail(FS_ERR_BAD_ARG, "fs_batch_submit_solve: unknown material code");
    BatchSolve v;
    v.large = !cluster_plan(q->ni, q->nj, &v.plan);
    CK(cudaSetDevice(b->device));
    if (v.large) {
        // the chained cooperative solve's vectors and control block
        const size_t fb = ((N * 4 + 255) & ~(size_t)255);
        const size_t pb = (((size_t)spec_partials_needed() * sizeof(float2) + 255) & ~(size_t)255);
        int rti = 0, rtj = 0;
        const bool res = spec_resident_shape(q->ni, q->nj, &rti, &rtj);
        const size_t lb = res ? 2 * N * 8 + kLlRecWords * 8 : 0; // exchange words
        const size_t cbytes = 5 * fb + pb + (size_t)kSpecResBlocks * 8 + 256 + lb;
        cudaError_t ec = cudaMalloc(&v.chain_mem, cbytes);
        if (ec != cudaSuccess)
            return fail(ec == cudaErrorMemoryAllocation ? FS_ERR_OOM : FS_ERR_CUDA,
                        "fs_batch_submit_solve: cudaMalloc: %s", cudaGetErrorString(ec));
        char *c = static_cast<char *>(v.chain_mem);
        v.chain.r = reinterpret_cast<float *>(c);
        v.chain.d = reinterpret_cast<float *>(c + fb);
        v.chain.s = reinterpret_cast<float *>(c + 2 * fb);
        v.chain.q = reinterpret_cast<float *>(c + 3 * fb);
        v.chain.z = reinterpret_cast<float *>(c + 4 * fb);
        v.chain.partials = reinterpret_cast<float2 *>(c + 5 * fb);
        v.chain.rpart = reinterpret_cast<double *>(c + 5 * fb + pb);
        char *t = c + 5 * fb + pb + (size_t)kSpecResBlocks * 8;
        v.chain.ctl = reinterpret_cast<SpecCtl *>(t);
        v.chain.count = reinterpret_cast<unsigned *>(t + 64);
        v.chain.status = reinterpret_cast<int *>(t + 128);
        if (res) {
            // its own copy of the decomposition's j-edge flag (the batch's
            // scalars serve every submission)
            v.chain.wrap_flag = reinterpret_cast<const int *>(t + 192);
            v.chain.res_ti = rti;
            v.chain.res_tj = rtj;
            unsigned long long *w = reinterpret_cast<unsigned long long *>(t + 256);
            v.ll.r = w;
            v.ll.s = w + N;
            v.ll.rec = w + 2 * N;
            v.ll.words = N;
        }
        if ((ec = cudaMemset(t + 128, 0, sizeof(int))) != cudaSuccess) {
            cudaFree(v.chain_mem);
            return fail(FS_ERR_CUDA, "fs_batch_submit_solve: %s", cudaGetErrorString(ec));
        }
    }
    const size_t a = (N + 255) & ~(size_t)255;
    const size_t bytes = 2 * a + 16 * N + 256;
    cudaError_t e = cudaMalloc(&v.mem, bytes);
    if (e != cudaSuccess)
        return fail(e == cudaErrorMemoryAllocation ? FS_ERR_OOM : FS_ERR_CUDA, "fs_batch_submit_solve: cudaMalloc: %s",
                    cudaGetErrorString(e));
    char *p = static_cast<char *>(v.mem);
    int8_t *mat = reinterpret_cast<int8_t *>(p);
    uint8_t *info = reinterpret_cast<uint8_t *>(p + a);
    double *bv = reinterpret_cast<double *>(p + 2 * a);
    double *xv = bv + N;
    char *tail = reinterpret_cast<char *>(xv + N);
    float *dt = reinterpret_cast<float *>(tail);
    int *iters = reinterpret_cast<int *>(tail + 16);
    double *rel = reinterpret_cast<double *>(tail + 32);
    cudaStream_t st = b->bst;
    auto bail = [&](cudaError_t err) {
        cudaFree(v.mem);
        if (v.chain_mem) cudaFree(v.chain_mem);
        return fail(FS_ERR_CUDA, "fs_batch_submit_solve: %s", cudaGetErrorString(err));
    };
    if ((e = cudaMemcpyAsync(mat, q->material, N, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
        (e = cudaMemcpyAsync(bv, q->rhs, N * 8, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
        (e = cudaMemcpyAsync(dt, &q->dt, sizeof(float), cudaMemcpyHostToDevice, st)) != cudaSuccess)
        return bail(e);
    GridDims gd{q->ni, q->nj, q->ni / 3 + (q->ni % 3 != 0), q->nj / 3 + (q->nj % 3 != 0)};
    Grids G;
    G.material = mat;
    G.cell_info = info;
    launch_decomposition(gd, G, b->chunk_last, 1, (long long)N, 0, b->dsc, st);
    g_kernel_launches += 1;
    if ((e = cudaGetLastError()) != cudaSuccess) return bail(e);
    if (v.chain.wrap_flag &&
        (e = cudaMemcpyAsync(const_cast<int *>(v.chain.wrap_flag), &b->dsc->wrap_units, sizeof(int),
                             cudaMemcpyDeviceToDevice, st)) != cudaSuccess)
        return bail(e);
    // the host arrays may be reused once this returns
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return bail(e);
    v.ticket = b->next_ticket++;
    v.ni = q->ni;
    v.nj = q->nj;
    ClusterSystem &c = v.sys;
    c.ni = q->ni;
    c.nj = q->nj;
    c.info = info;
    c.b = bv;
    c.x = xv;
    c.dt = dt;
    c.density = q->density;
    c.dx = q->dx;
    c.iters = iters;
    c.rel_res = rel;
    if (v.large) {
        SpecSolve &ch = v.chain;
        ch.ni = q->ni;
        ch.nj = q->nj;
        ch.info = info;
        ch.b = bv;
        ch.x = xv;
        ch.dt = dt;
        ch.density = q->density;
        ch.dx = q->dx;
        ch.iters_out = iters;
        ch.rel_out = rel;
        ch.tol = kSpecRelTol;
        ch.max_iter = kSpecMaxIter;
        ch.max_outer = kSpecMaxOuter;
    }
    b->solves.push_back(v);
    *ticket = v.ticket;
    return FS_OK;
}

static BatchSolve *batch_find_solve(fs_batch *b, unsigned long long ticket, size_t *index)
{
    for (size_t k = 0; k < b->solves.size(); k++)
        if (b->solves[k].ticket == ticket) {
            if (index) *index = k;
            return &b->solves[k];
        }
    return nullptr;
}

extern "C" fs_status fs_batch_solve_done(fs_batch *b, unsigned long long ticket, int *done)
{
    if (!b || !done) return fail(FS_ERR_BAD_ARG, "null argument");
    BatchSolve *v = batch_find_solve(b, ticket, nullptr);
    if (!v) return fail(FS_ERR_BAD_ARG, "fs_batch_solve_done: unknown ticket");
    *done = v->done ? 1 : 0;
    return FS_OK;
}

extern "C" fs_status fs_batch_take_solve(fs_batch *b, unsigned long long ticket, fs_poisson_system *q)
{
    if (!b || !q || !q->result) return fail(FS_ERR_BAD_ARG, "null argument");
    size_t k = 0;
    BatchSolve *v = batch_find_solve(b, ticket, &k);
    if (!v) return fail(FS_ERR_BAD_ARG, "fs_batch_take_solve: unknown ticket");
    if (!v->done) return fail(FS_ERR_BAD_ARG, "fs_batch_take_solve: not solved yet");
    if (q->ni != v->ni || q->nj != v->nj) return fail(FS_ERR_BAD_ARG, "fs_batch_take_solve: shape mismatch");
    CK(cudaSetDevice(b->device));
    const size_t N = (size_t)v->ni * v->nj;
    int it = 0;
    double rel = 0.0;
    CK(cudaMemcpy(q->result, v->sys.x, N * 8, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(&it, v->sys.iters, sizeof(int), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(&rel, v->sys.rel_res, sizeof(double), cudaMemcpyDeviceToHost));
    int chain_status = 0;
    if (v->large) CK(cudaMemcpy(&chain_status, v->chain.status, sizeof(int), cudaMemcpyDeviceToHost));
    q->iterations = it;
    q->rel_residual = rel;
    cudaFree(v->mem);
    if (v->chain_mem) cudaFree(v->chain_mem);
    b->solves.erase(b->solves.begin() + (long)k);
    if (chain_status != 0) return fail(FS_ERR_TIMEOUT, "fs_batch_take_solve: a grid barrier wait timed out");
    return FS_OK;
}

extern "C" fs_status fs_batch_timer(fs_batch *b, int which, double *value)
{
    if (!b || !value) return fail(FS_ERR_BAD_ARG, "null argument");
    switch (which) {
    case 0: *value = b->solve_ms; return FS_OK;
    case 1: *value = b->frame_ms; return FS_OK;
    case 2: *value = (double)b->rounds; return FS_OK;
    case 3: b->solve_ms = b->frame_ms = 0.0; b->rounds = 0; *value = 0.0; return FS_OK;
    default: return fail(FS_ERR_BAD_ARG, "bad timer id");
    }
}

// one merged solve (0 density, 1 pressure) over the scenes of `act` plus,
// for the pressure solve, the submitted standalone systems `extra`
static fs_status batch_solve(fs_batch *b, const std::vector<int> &act, const std::vector<int> &extra,
                             int which)
{
    const size_t total = act.size() + (which == 1 ? extra.size() : 0);
    if (total > b->list_cap) {
        CK(cudaDeviceSynchronize());
        if (b->d_list) cudaFree(b->d_list);
        if (b->h_list) cudaFreeHost(b->h_list);
        b->d_list = nullptr;
        b->h_list = nullptr;
        b->list_cap = 0;
        const size_t cap = std::max<size_t>(2 * total, 64);
        CK(cudaMalloc(&b->d_list, 2 * cap * sizeof(ClusterSystem)));
        CK(cudaMallocHost(&b->h_list, 2 * cap * sizeof(ClusterSystem)));
        b->list_cap = cap;
    }
    ClusterSystem *hl = b->h_list + (size_t)which * b->list_cap;
    ClusterSystem *dl = b->d_list + (size_t)which * b->list_cap;
    // entries: scenes then standalone systems, each with its plan
    std::vector<std::pair<ClusterPlan, ClusterSystem>> ent;
    ent.reserve(total);
    for (int k : act) {
        fs_solver *s = b->sc[k].s;
        if (s->spec_large) continue; // solved inside its own graphs
        ClusterSystem c;
        c.ni = s->d.ni;
        c.nj = s->d.nj;
        c.info = s->G.cell_info;
        c.b = (const double *)(which == 0 ? s->dens_rhs : s->pres_rhs);
        c.x = (double *)(which == 0 ? s->dens_x : s->pres_x);
        c.dt = &s->sc->dt;
        c.density = s->sp.fluidDensity;
        c.dx = s->sp.dx;
        c.iters = which == 0 ? &s->sc->density_iters : &s->sc->pressure_iters;
        c.rel_res = s->spec_rel + which;
        ent.push_back({s->spec_plan, c});
    }
    if (which == 1)
        for (int k : extra)
            if (!b->solves[k].large) ent.push_back({b->solves[k].plan, b->solves[k].sys});
    if (which == 1) {
        // standalone systems above the on-chip limit: their chained solves
        for (int k : act) CK(cudaStreamWaitEvent(b->bst, b->sc[k].ev, 0));
        for (int k : extra)
            if (b->solves[k].large) {
                BatchSolve &v = b->solves[k];
                v.chain.ll = v.chain.res_ti > 0 ? &v.ll : nullptr; // the vector may have moved it
                CK(launch_spec_chain(v.chain, b->bst));
                g_kernel_launches += spec_chain_kernels(v.chain);
            }
    }
    if (ent.empty()) {
        CK(cudaEventRecord(b->ev_t[2 * which], b->bst));
        CK(cudaEventRecord(b->ev_t[2 * which + 1], b->bst));
        CK(cudaEventRecord(b->ev_solve, b->bst));
        return FS_OK;
    }
    auto key = [](const ClusterPlan &q) { return q.C * 64 + q.K; };
    // the largest clusters first: they wait longest for whole GPCs
    std::stable_sort(ent.begin(), ent.end(), [&](const auto &x, const auto &y) { return key(x.first) > key(y.first); });
    for (size_t t = 0; t < ent.size(); t++) hl[t] = ent[t].second;
    for (int k : act) CK(cudaStreamWaitEvent(b->bst, b->sc[k].ev, 0));
    CK(cudaMemcpyAsync(dl, hl, ent.size() * sizeof(ClusterSystem), cudaMemcpyHostToDevice, b->bst));
    CK(cudaEventRecord(b->ev_t[2 * which], b->bst));
    CK(cudaEventRecord(b->ev_fork, b->bst));
    const ClusterParams cp = spec_params();
    int ng = 0;
    for (size_t t0 = 0; t0 < ent.size();) {
        size_t t1 = t0;
        ClusterPlan g = ent[t0].first;
        while (t1 < ent.size() && key(ent[t1].first) == key(ent[t0].first)) g.smem = std::max(g.smem, ent[t1++].first.smem);
        const int gi = ng % fs_batch::kGroups;
        cudaStream_t gs = b->gst[gi];
        CK(cudaStreamWaitEvent(gs, b->ev_fork, 0));
        CK(launch_pcg_cluster(dl + t0, (int)(t1 - t0), g, cp, gs));
        CK(cudaEventRecord(b->gev[gi], gs));
        ng++;
        g_kernel_launches += 1;
        t0 = t1;
    }
    for (int gi = 0; gi < std::min(ng, (int)fs_batch::kGroups); gi++) CK(cudaStreamWaitEvent(b->bst, b->gev[gi], 0));
    CK(cudaEventRecord(b->ev_t[2 * which + 1], b->bst));
    CK(cudaEventRecord(b->ev_solve, b->bst));
    return FS_OK;
}

// one round: a substep of every member inside a frame, the standalone
// systems submitted so far solved with the round's pressure solves
static fs_status batch_round(fs_batch *b, int *busy)
{
    const auto t0 = std::chrono::steady_clock::now();
    std::vector<int> act, extra;
    // the CFL step of every member inside its frame (fs_step_frame's loop)
    for (int k = 0; k < (int)b->sc.size(); k++) {
        BatchScene &bs = b->sc[k];
        fs_solver *s = bs.s;
        if (!bs.in_frame) continue;
        if (s->sc_host->pcg_status != 0) return fail(FS_ERR_TIMEOUT, "batch member %d: solver status", k);
        if (s->sc_host->nonfinite != 0)
            return fail(FS_ERR_NONFINITE, "batch member %d: a substep left a NaN or infinite particle velocity", k);
        if (bs.substep_count > 0) {
            s->density_iters_max = std::max(s->density_iters_max, s->sc_host->density_iters);
            s->pressure_iters_max = std::max(s->pressure_iters_max, s->sc_host->pressure_iters);
        }
        unsigned bits = s->sc_host->maxv2;
        float v2;
        memcpy(&v2, &bits, 4);
        const float vel = std::sqrt(v2);
        float maxSubstepSize = s->p.cflNumber / (vel + 1e-15f);
        bool last = false;
        if (bs.substep_time + maxSubstepSize >= s->frame_dt || bs.substep_count == (s->p.maxSubsteps - 1)) {
            maxSubstepSize = s->frame_dt - bs.substep_time;
            last = true;
        } else if (bs.substep_time + 2.f * maxSubstepSize >= s->frame_dt) {
            maxSubstepSize = 0.5f * (s->frame_dt - bs.substep_time);
        }
        s->step_dt = maxSubstepSize;
        b->h_dt[bs.slot] = maxSubstepSize;
        bs.substep_time += maxSubstepSize;
        bs.substep_count++;
        bs.last = last || bs.substep_count > 50;
        act.push_back(k);
    }
    for (int k = 0; k < (int)b->solves.size(); k++)
        if (!b->solves[k].done) extra.push_back(k);
    if (act.empty() && extra.empty()) {
        *busy = 0;
        return FS_OK;
    }
    CK(cudaMemcpyAsync(b->d_dt, b->h_dt, (size_t)fs_batch::kSlots * sizeof(float), cudaMemcpyHostToDevice, b->bst));
    CK(cudaEventRecord(b->ev_solve, b->bst));
    for (int k : act) {
        BatchScene &bs = b->sc[k];
        CK(cudaStreamWaitEvent(bs.s->st, b->ev_solve, 0));
        CK(cudaGraphLaunch(bs.g[bs.parity][0], bs.s->st));
        CK(cudaEventRecord(bs.ev, bs.s->st));
        g_kernel_launches += bs.launches[0];
    }
    if (!act.empty()) TRY(batch_solve(b, act, extra, 0));
    for (int k : act) {
        BatchScene &bs = b->sc[k];
        CK(cudaStreamWaitEvent(bs.s->st, b->ev_solve, 0));
        CK(cudaGraphLaunch(bs.g[bs.parity][1], bs.s->st));
        CK(cudaEventRecord(bs.ev, bs.s->st));
        g_kernel_launches += bs.launches[1];
    }
    TRY(batch_solve(b, act, extra, 1));
    for (int k : act) {
        BatchScene &bs = b->sc[k];
        CK(cudaStreamWaitEvent(bs.s->st, b->ev_solve, 0));
        CK(cudaGraphLaunch(bs.g[bs.parity][2], bs.s->st));
        CK(cudaEventRecord(bs.ev, bs.s->st));
        g_kernel_launches += bs.launches[2];
        bs.parity ^= 1;
        bs.s->substeps++;
        bs.s->substeps_total++;
    }
    // the round's own work only: each member's last graph (it ends with the
    // scalars the next CFL step reads) and the merged solves; unrelated work
    // on the device does not hold the round
    for (int k : act) CK(cudaEventSynchronize(b->sc[k].ev));
    CK(cudaEventSynchronize(b->ev_solve));
    for (int w = act.empty() ? 1 : 0; w < 2; w++) {
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, b->ev_t[2 * w], b->ev_t[2 * w + 1]));
        b->solve_ms += ms;
    }
    b->rounds++;
    for (int k : extra) b->solves[k].done = true;
    int still = 0;
    for (int k : act) {
        BatchScene &bs = b->sc[k];
        if (!bs.last) {
            still++;
            continue;
        }
        // the frame ends (fs_step_frame after its loop)
        fs_solver *s = bs.s;
        s->density_iters_max = std::max(s->density_iters_max, s->sc_host->density_iters);
        s->pressure_iters_max = std::max(s->pressure_iters_max, s->sc_host->pressure_iters);
        s->P = bs.P[bs.parity];
        s->G = bs.G[bs.parity];
        s->frame++;
        bs.in_frame = false;
    }
    b->frame_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    *busy = still;
    return FS_OK;
}

extern "C" fs_status fs_batch_round(fs_batch *b, int *busy)
{
    if (!b || !busy) return fail(FS_ERR_BAD_ARG, "null argument");
    CK(cudaSetDevice(b->device));
    return batch_round(b, busy);
}

extern "C" fs_status fs_batch_run_frames(fs_batch *b, int frames)
{
    if (!b || frames < 0) return fail(FS_ERR_BAD_ARG, "fs_batch_run_frames: invalid argument");
    CK(cudaSetDevice(b->device));
    for (BatchScene &bs : b->sc)
        if (bs.in_frame) return fail(FS_ERR_BAD_ARG, "fs_batch_run_frames: a member is inside a frame");
    if (frames == 0) return FS_OK;
    std::vector<int> left(b->sc.size(), frames);
    for (size_t k = 0; k < b->sc.size(); k++) {
        TRY(batch_begin(b, b->sc[k]));
        left[k]--;
    }
    CK(cudaDeviceSynchronize());
    for (;;) {
        int busy = 0;
        TRY(batch_round(b, &busy));
        // a member whose frame ended starts its next one in the next round
        bool began = false;
        for (size_t k = 0; k < b->sc.size(); k++)
            if (!b->sc[k].in_frame && left[k] > 0) {
                TRY(batch_begin(b, b->sc[k]));
                left[k]--;
                began = true;
            }
        if (began) CK(cudaDeviceSynchronize());
        if (!began && busy == 0) break;
    }
    return FS_OK;
}

extern "C" fs_status fs_batch_step_frame(fs_batch *b)
{
    if (!b) return fail(FS_ERR_BAD_ARG, "null batch");
    CK(cudaSetDevice(b->device));
    for (BatchScene &bs : b->sc)
        if (bs.in_frame) return fail(FS_ERR_BAD_ARG, "fs_batch_step_frame: a member is inside a frame");
    for (BatchScene &bs : b->sc) TRY(batch_begin(b, bs));
    CK(cudaDeviceSynchronize());
    for (int busy = 1; busy;) TRY(batch_round(b, &busy));
    return FS_OK;
}

// ---------------------------------------------------------------------------
// standalone LinearSolver::solve drop-in
// ---------------------------------------------------------------------------
namespace {
struct PcgCache {
    int device = -1;
    size_t cap_cells = 0;
    size_t esz = 0;
    int grid = 0;
    int8_t *material = nullptr;
    uint8_t *info = nullptr;
    void *b = nullptr, *x = nullptr, *r0 = nullptr, *r1 = nullptr, *s0 = nullptr, *s1 = nullptr;
    double *partials = nullptr;
    int *chunk_end = nullptr, *chunk_last = nullptr;
    double *chunk_val = nullptr;
    int chunk_cap = 0;
    GridBarrier *bar = nullptr;
    Scalars *sc = nullptr;
    Scalars *sc_host = nullptr;
    LlBuffers ll; // the resident FP32 kernel's exchange words
    void release()
    {
        void *ps[] = {material, info, b, x, r0, r1, s0, s1, partials, chunk_end, chunk_last, chunk_val, bar, sc,
                      ll.r, ll.s, ll.rec};
        for (void *p : ps)
            if (p) cudaFree(p);
        if (sc_host) cudaFreeHost(sc_host);
        *this = PcgCache();
    }
};
std::mutex g_pcg_mu;
PcgCache g_pcg[64];
} // namespace

static fs_status pcg_cache_get(int dev, size_t cells, size_t esz, int nchunks, PcgCache **out)
{
    if (dev < 0 || dev >= 64) return fail(FS_ERR_BAD_ARG, "bad device");
    PcgCache &c = g_pcg[dev];
    if (c.device == dev && c.cap_cells >= cells && c.esz == esz && c.chunk_cap >= nchunks) {
        *out = &c;
        return FS_OK;
    }
    c.release();
    c.device = dev;
    c.cap_cells = cells;
    c.esz = esz;
    c.chunk_cap = nchunks + 1;
    c.grid = esz == 8 ? pcg_grid_size<double>((long long)cells) : pcg_grid_size<float>((long long)cells);
    CK(cudaMalloc(&c.material, cells));
    CK(cudaMalloc(&c.info, cells));
    void **vs[] = {&c.b, &c.x, &c.r0, &c.r1, &c.s0, &c.s1};
    for (void **v : vs) CK(cudaMalloc(v, cells * esz));
    if (esz == 4) {
        c.ll.words = cells;
        CK(cudaMalloc(&c.ll.r, cells * sizeof(unsigned long long)));
        CK(cudaMalloc(&c.ll.s, cells * sizeof(unsigned long long)));
        CK(cudaMalloc(&c.ll.rec, kLlRecWords * sizeof(unsigned long long)));
    }
    int maxgrid = std::max(pcg_grid_size<double>(1LL << 40), pcg_grid_size<float>(1LL << 40));
    CK(cudaMalloc(&c.partials, (size_t)(8 * maxgrid + 16) * sizeof(double)));
    CK(cudaMalloc(&c.chunk_end, (size_t)c.chunk_cap * sizeof(int)));
    CK(cudaMalloc(&c.chunk_last, (size_t)c.chunk_cap * sizeof(int)));
    CK(cudaMalloc(&c.chunk_val, (size_t)c.chunk_cap * sizeof(double)));
    CK(cudaMalloc(&c.bar, sizeof(GridBarrier)));
    CK(cudaMalloc(&c.sc, sizeof(Scalars)));
    CK(cudaMallocHost(&c.sc_host, sizeof(Scalars)));
    *out = &c;
    return FS_OK;
}

static bool valid_material(const int8_t *m, size_t n)
{
    for (size_t k = 0; k < n; k++) {
        const int8_t v = m[k];
        if (v != M_FLUID && v != M_SOURCE && v != M_SOLID && v != M_SINK && v != M_EMPTY) return false;
    }
    return true;
}

static fs_status pcg_solve_common(int ni, int nj, const int8_t *mat_dev, float dt, double density,
                                  double dx, const void *rhs_dev, void *res_dev, int iter_limit,
                                  double tol, const fs_exec_params *exec, int *iterations,
                                  PcgCache *c, int prec, const uint8_t *info_host = nullptr,
                                  double scale = 0.0)
{
    const size_t N = (size_t)ni * nj;
    const int T = (exec && exec->pool_threads > 0) ? exec->pool_threads : default_pool_threads();
    std::vector<int> ends = split_range_ends((long long)N, T);
    cudaStream_t st = 0;
    CK(cudaMemcpyAsync(c->chunk_end, ends.data(), ends.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    if (info_host) {
        // the operator comes packed from the caller: what the decomposition
        // derives from it -- the last unit row of each chunk and whether a
        // unit row sits on a j edge -- is found here
        std::vector<int> last(ends.size(), -1);
        int wrap = 0;
        size_t k = 0;
        for (size_t cidx = 0; cidx < N; cidx++) {
            while (k + 1 < ends.size() && (long long)cidx >= ends[k]) k++;
            if (info_host[cidx] & 0x80) {
                last[k] = (int)cidx;
                const size_t j = cidx % (size_t)nj;
                if (j == 0 || j == (size_t)nj - 1) wrap = 1;
            }
        }
        CK(cudaMemcpyAsync(c->info, info_host, N, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(c->chunk_last, last.data(), last.size() * sizeof(int), cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(&c->sc->wrap_units, &wrap, sizeof(int), cudaMemcpyHostToDevice, st));
        CK(cudaStreamSynchronize(st)); // the host vectors above go out of scope
    } else {
        GridDims d{ni, nj, ni / 3 + (ni % 3 != 0), nj / 3 + (nj % 3 != 0)};
        Grids G;
        G.material = const_cast<int8_t *>(mat_dev);
        G.cell_info = c->info;
        long long ps = 1, rem = 0;
        split_range_params((long long)N, T, &ps, &rem);
        launch_decomposition(d, G, c->chunk_last, (int)ends.size(), ps, rem, c->sc, st);
        g_kernel_launches += 1;
    }
    k_set_dt<<<1, 1, 0, st>>>(c->sc, dt);
    CK(cudaMemsetAsync(&c->sc->pcg_status, 0, sizeof(int), st));
    g_kernel_launches += 1;
    cudaError_t e;
    int launched = 0;
    if (prec == FS_PCG_FP64) {
        PcgArgs<double> a{};
        a.ni = ni; a.nj = nj; a.N = (long long)N; a.info = c->info;
        a.b = (const double *)rhs_dev; a.x = (double *)res_dev;
        a.r0 = (double *)c->r0; a.r1 = (double *)c->r1; a.s0 = (double *)c->s0; a.s1 = (double *)c->s1;
        a.partials = c->partials; a.chunk_end = c->chunk_end; a.chunk_last_unit = c->chunk_last;
        a.chunk_val = c->chunk_val;
        a.nchunks = (int)ends.size(); a.sc = c->sc; a.density = density; a.dx = dx; a.scale = scale;
        a.iter_limit = iter_limit; a.tol = tol; a.iters_out = &c->sc->density_iters;
        a.status = &c->sc->pcg_status; a.bar = c->bar;
        a.spin_limit = exec ? exec->wait_polls : 0;
        a.wrap_flag = &c->sc->wrap_units; a.mode = 0;
        e = launch_pcg<double>(a, st, &launched);
    } else {
        PcgArgs<float> a{};
        a.ni = ni; a.nj = nj; a.N = (long long)N; a.info = c->info;
        a.b = (const float *)rhs_dev; a.x = (float *)res_dev;
        a.r0 = (float *)c->r0; a.r1 = (float *)c->r1; a.s0 = (float *)c->s0; a.s1 = (float *)c->s1;
        a.ll_r = c->ll.r; a.ll_s = c->ll.s;
        a.partials = c->partials; a.chunk_end = c->chunk_end; a.chunk_last_unit = c->chunk_last;
        a.chunk_val = c->chunk_val;
        a.nchunks = (int)ends.size(); a.sc = c->sc; a.density = density; a.dx = dx; a.scale = scale;
        a.iter_limit = iter_limit; a.tol = tol; a.iters_out = &c->sc->density_iters;
        a.status = &c->sc->pcg_status; a.bar = c->bar;
        a.spin_limit = exec ? exec->wait_polls : 0;
        a.wrap_flag = &c->sc->wrap_units; a.mode = 0;
        int ti = 0, tj = 0;
        TmaMaps maps;
        if (resident_tile_shape(ni, nj, &ti, &tj)) {
            a.mode = 2;
            e = launch_pcg_resident(a, ti, tj, st, &c->ll);
            if (e == cudaSuccess) e = launch_pcg_linear_if_wrap(a, st);
            launched = 2;
        } else if (tma_tile_shape(ni, nj, &ti, &tj) &&
            tma_maps(&maps, ni, nj, ti, tj, c->info, (const float *)rhs_dev, (const float *)res_dev,
                     (const float *)c->r0, (const float *)c->r1, (const float *)c->s0,
                     (const float *)c->s1) &&
            tma_store_maps(&maps, ni, nj, ti, tj, (const float *)c->r0, (const float *)c->r1,
                           (const float *)c->s0, (const float *)c->s1)) {
            a.mode = 2;
            e = launch_pcg_tma(a, maps, ti, tj, st);
            if (e == cudaSuccess) e = launch_pcg_linear_if_wrap(a, st);
            launched = 2;
        } else {
            e = launch_pcg<float>(a, st, &launched);
        }
    }
    g_kernel_launches += launched;
    if (e != cudaSuccess) return fail(FS_ERR_CUDA, "PCG launch: %s", cudaGetErrorString(e));
    CK(cudaMemcpyAsync(c->sc_host, c->sc, sizeof(Scalars), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (c->sc_host->pcg_status != 0) return fail(FS_ERR_TIMEOUT, "a PCG grid barrier wait timed out");
    if (iterations) *iterations = c->sc_host->density_iters;
    return FS_OK;
}

extern "C" fs_status fs_pcg_solve(int ni, int nj, const int8_t *material, float dt, double density,
                                  double dx, const double *rhs, double *result, int iter_limit,
                                  double tol, const fs_exec_params *exec, int *iterations)
{
    if (ni < 1 || nj < 1 || !material || !rhs || !result || iter_limit < 0)
        return fail(FS_ERR_BAD_ARG, "fs_pcg_solve: invalid argument");
    const size_t N = (size_t)ni * nj;
    if (!valid_material(material, N)) return fail(FS_ERR_BAD_ARG, "fs_pcg_solve: unknown material code");
    const int dev = exec ? exec->device : 0;
    const int prec = (exec && exec->pcg_precision == FS_PCG_FP64) ? FS_PCG_FP64 : FS_PCG_FP32;
    const size_t esz = prec == FS_PCG_FP64 ? 8 : 4;
    std::lock_guard<std::mutex> lk(g_pcg_mu);
    CK(cudaSetDevice(dev));
    const int T = (exec && exec->pool_threads > 0) ? exec->pool_threads : default_pool_threads();
    PcgCache *c = nullptr;
    TRY(pcg_cache_get(dev, N, esz, std::min<long long>(T, (long long)N), &c));
    CK(cudaMemcpy(c->material, material, N, cudaMemcpyHostToDevice));
    if (prec == FS_PCG_FP64) {
        CK(cudaMemcpy(c->b, rhs, N * 8, cudaMemcpyHostToDevice));
    } else {
        std::vector<float> tmp(N);
        for (size_t k = 0; k < N; k++) tmp[k] = (float)rhs[k];
        CK(cudaMemcpy(c->b, tmp.data(), N * 4, cudaMemcpyHostToDevice));
    }
    TRY(pcg_solve_common(ni, nj, c->material, dt, density, dx, c->b, c->x, iter_limit, tol, exec,
                         iterations, c, prec));
    if (prec == FS_PCG_FP64) {
        CK(cudaMemcpy(result, c->x, N * 8, cudaMemcpyDeviceToHost));
    } else {
        std::vector<float> tmp(N);
        CK(cudaMemcpy(tmp.data(), c->x, N * 4, cudaMemcpyDeviceToHost));
        for (size_t k = 0; k < N; k++) result[k] = tmp[k];
    }
    return FS_OK;
}

extern "C" fs_status fs_pcg_solve_device(int ni, int nj, const int8_t *material_device, float dt,
                                         double density, double dx, const void *rhs_device,
                                         void *result_device, int iter_limit, double tol,
                                         const fs_exec_params *exec, int *iterations)
{
    if (ni < 1 || nj < 1 || !material_device || !rhs_device || !result_device || iter_limit < 0)
        return fail(FS_ERR_BAD_ARG, "fs_pcg_solve_device: invalid argument");
    const size_t N = (size_t)ni * nj;
    const int dev = exec ? exec->device : 0;
    const int prec = (exec && exec->pcg_precision == FS_PCG_FP64) ? FS_PCG_FP64 : FS_PCG_FP32;
    const size_t esz = prec == FS_PCG_FP64 ? 8 : 4;
    std::lock_guard<std::mutex> lk(g_pcg_mu);
    CK(cudaSetDevice(dev));
    const int T = (exec && exec->pool_threads > 0) ? exec->pool_threads : default_pool_threads();
    PcgCache *c = nullptr;
    TRY(pcg_cache_get(dev, N, esz, std::min<long long>(T, (long long)N), &c));
    return pcg_solve_common(ni, nj, material_device, dt, density, dx, rhs_device, result_device,
                            iter_limit, tol, exec, iterations, c, prec);
}

extern "C" fs_status fs_pcg_solve_operator(int ni, int nj, const uint8_t *cell_info, double scale,
                                           const double *rhs, double *result, int iter_limit,
                                           double tol, const fs_exec_params *exec, int *iterations)
{
    if (ni < 1 || nj < 1 || !cell_info || !rhs || !result || iter_limit < 0 || !(scale > 0.0))
        return fail(FS_ERR_BAD_ARG, "fs_pcg_solve_operator: invalid argument");
    const size_t N = (size_t)ni * nj;
    // a neighbour whose linear index falls outside [0, N) reads as 0 in the
    // reference's multiply (pressuredata.h:132-146): its mask bit is dropped
    std::vector<uint8_t> info(cell_info, cell_info + N);
    for (size_t k = 0; k < N; k++) {
        uint8_t b = info[k];
        if (((b >> 4) & 7) > 4 || (!(b & 0x80) && (b & 0x0f)))
            return fail(FS_ERR_BAD_ARG, "fs_pcg_solve_operator: cell %zu: bad operator byte 0x%02x", k, b);
        if (k < (size_t)nj) b &= (uint8_t)~1u;
        if (k + (size_t)nj >= N) b &= (uint8_t)~2u;
        if (k == 0) b &= (uint8_t)~4u;
        if (k + 1 >= N) b &= (uint8_t)~8u;
        info[k] = b;
    }
    const int dev = exec ? exec->device : 0;
    const int prec = (exec && exec->pcg_precision == FS_PCG_FP64) ? FS_PCG_FP64 : FS_PCG_FP32;
    const size_t esz = prec == FS_PCG_FP64 ? 8 : 4;
    std::lock_guard<std::mutex> lk(g_pcg_mu);
    CK(cudaSetDevice(dev));
    const int T = (exec && exec->pool_threads > 0) ? exec->pool_threads : default_pool_threads();
    PcgCache *c = nullptr;
    TRY(pcg_cache_get(dev, N, esz, std::min<long long>(T, (long long)N), &c));
    if (prec == FS_PCG_FP64) {
        CK(cudaMemcpy(c->b, rhs, N * 8, cudaMemcpyHostToDevice));
    } else {
        std::vector<float> tmp(N);
        for (size_t k = 0; k < N; k++) tmp[k] = (float)rhs[k];
        CK(cudaMemcpy(c->b, tmp.data(), N * 4, cudaMemcpyHostToDevice));
    }
    TRY(pcg_solve_common(ni, nj, nullptr, 0.f, 1.0, 1.0, c->b, c->x, iter_limit, tol, exec, iterations,
                         c, prec, info.data(), scale));
    if (prec == FS_PCG_FP64) {
        CK(cudaMemcpy(result, c->x, N * 8, cudaMemcpyDeviceToHost));
    } else {
        std::vector<float> tmp(N);
        CK(cudaMemcpy(tmp.data(), c->x, N * 4, cudaMemcpyDeviceToHost));
        for (size_t k = 0; k < N; k++) result[k] = tmp[k];
    }
    return FS_OK;
}

// ---------------------------------------------------------------------------
// fs_pcg_solve_spec: the pressure solve to a true relative residual with FP32
// inner PCG iterations (textbook incomplete-Poisson preconditioner) and FP64
// outer refinement (fs_spec.cu).
// ---------------------------------------------------------------------------
extern "C" fs_status fs_pcg_solve_spec(int ni, int nj, const int8_t *material, float dt, double density,
                                       double dx, const double *rhs, double *result, double rel_tol,
                                       int max_iter, const fs_exec_params *exec, int *iterations,
                                       double *rel_residual)
{
    if (ni < 1 || nj < 1 || !material || !rhs || !result || max_iter < 0 || !(rel_tol > 0.0))
        return fail(FS_ERR_BAD_ARG, "fs_pcg_solve_spec: invalid argument");
    if (!valid_material(material, (size_t)ni * nj))
        return fail(FS_ERR_BAD_ARG, "fs_pcg_solve_spec: unknown material code");
    const long long N = (long long)ni * nj;
    const int dev = exec ? exec->device : 0;
    CK(cudaSetDevice(dev));
    cudaStream_t st = 0;
    // device buffers for this call
    std::vector<void *> bufs;
    auto release = [&]() {
        for (void *q : bufs) cudaFree(q);
        bufs.clear();
    };
    auto dalloc_tmp = [&](void **p, size_t bytes) -> fs_status {
        cudaError_t e = cudaMalloc(p, bytes);
        if (e != cudaSuccess) {
            release();
            return fail(e == cudaErrorMemoryAllocation ? FS_ERR_OOM : FS_ERR_CUDA,
                        "fs_pcg_solve_spec: cudaMalloc: %s", cudaGetErrorString(e));
        }
        bufs.push_back(*p);
        return FS_OK;
    };
    auto check = [&](cudaError_t e, const char *what) -> fs_status {
        if (e == cudaSuccess) return FS_OK;
        release();
        return fail(FS_ERR_CUDA, "fs_pcg_solve_spec: %s: %s", what, cudaGetErrorString(e));
    };
    int8_t *mat = nullptr;
    uint8_t *info = nullptr;
    double *b = nullptr, *x = nullptr, *rpart = nullptr, *rel_dev = nullptr;
    float *r = nullptr, *d = nullptr, *s = nullptr, *q = nullptr, *z = nullptr, *dt_dev = nullptr;
    float2 *partials = nullptr;
    int *chunk_last = nullptr, *iters_dev = nullptr;
    Scalars *sc = nullptr;
    unsigned *count = nullptr;
    SpecCtl *ctl = nullptr;
    TRY(dalloc_tmp((void **)&mat, N));
    TRY(dalloc_tmp((void **)&info, N));
    TRY(dalloc_tmp((void **)&b, N * 8));
    TRY(dalloc_tmp((void **)&x, N * 8));
    float **fv[] = {&r, &d, &s, &q, &z};
    for (float **v : fv) TRY(dalloc_tmp((void **)v, N * 4));
    TRY(dalloc_tmp((void **)&partials, (size_t)spec_partials_needed() * sizeof(float2)));
    TRY(dalloc_tmp((void **)&rpart, (size_t)kSpecResBlocks * 8));
    TRY(dalloc_tmp((void **)&chunk_last, 2 * sizeof(int)));
    TRY(dalloc_tmp((void **)&sc, sizeof(Scalars)));
    TRY(dalloc_tmp((void **)&count, sizeof(unsigned)));
    TRY(dalloc_tmp((void **)&ctl, sizeof(SpecCtl)));
    TRY(dalloc_tmp((void **)&dt_dev, sizeof(float)));
    TRY(dalloc_tmp((void **)&iters_dev, sizeof(int)));
    TRY(dalloc_tmp((void **)&rel_dev, sizeof(double)));
    TRY(check(cudaMemcpyAsync(mat, material, N, cudaMemcpyHostToDevice, st), "upload"));
    TRY(check(cudaMemcpyAsync(b, rhs, N * 8, cudaMemcpyHostToDevice, st), "upload"));
    TRY(check(cudaMemcpyAsync(dt_dev, &dt, sizeof(float), cudaMemcpyHostToDevice, st), "upload"));
    TRY(check(cudaMemsetAsync(sc, 0, sizeof(Scalars), st), "memset"));
    GridDims gd{ni, nj, ni / 3 + (ni % 3 != 0), nj / 3 + (nj % 3 != 0)};
    Grids G;
    G.material = mat;
    G.cell_info = info;
    launch_decomposition(gd, G, chunk_last, 1, N, 0, sc, st);
    g_kernel_launches += 1;
    // the whole solve -- outer loop included -- enqueued at once
    SpecSolve p{};
    p.ni = ni;
    p.nj = nj;
    p.info = info;
    p.b = b;
    p.x = x;
    p.dt = dt_dev;
    p.density = density;
    p.dx = dx;
    p.r = r;
    p.d = d;
    p.s = s;
    p.q = q;
    p.z = z;
    p.partials = partials;
    p.rpart = rpart;
    p.count = count;
    p.status = &sc->pcg_status;
    p.ctl = ctl;
    p.iters_out = iters_dev;
    p.rel_out = rel_dev;
    p.tol = rel_tol;
    p.max_iter = max_iter;
    p.max_outer = kSpecMaxOuter;
    // inner solves on the resident kernel where the grid fits it
    LlBuffers ll;
    int rti = 0, rtj = 0;
    if (spec_resident_shape(ni, nj, &rti, &rtj)) {
        TRY(dalloc_tmp((void **)&ll.r, N * 8));
        TRY(dalloc_tmp((void **)&ll.s, N * 8));
        TRY(dalloc_tmp((void **)&ll.rec, kLlRecWords * 8));
        ll.words = N;
        p.res_ti = rti;
        p.res_tj = rtj;
        p.ll = &ll;
        p.wrap_flag = &sc->wrap_units;
    }
    TRY(check(launch_spec_chain(p, st), "solve"));
    g_kernel_launches += spec_chain_kernels(p);
    int h_status = 0, it = 0;
    double rel = 0.0;
    TRY(check(cudaMemcpyAsync(&h_status, &sc->pcg_status, sizeof(int), cudaMemcpyDeviceToHost, st), "readback"));
    TRY(check(cudaMemcpyAsync(&it, iters_dev, sizeof(int), cudaMemcpyDeviceToHost, st), "readback"));
    TRY(check(cudaMemcpyAsync(&rel, rel_dev, sizeof(double), cudaMemcpyDeviceToHost, st), "readback"));
    TRY(check(cudaStreamSynchronize(st), "sync"));
    if (h_status != 0) {
        release();
        return fail(FS_ERR_TIMEOUT, "fs_pcg_solve_spec: a grid barrier wait timed out");
    }
    TRY(check(cudaMemcpy(result, x, N * 8, cudaMemcpyDeviceToHost), "download"));
    release();
    if (iterations) *iterations = it;
    if (rel_residual) *rel_residual = rel;
    return FS_OK;
}

// ---------------------------------------------------------------------------
// fs_pcg_solve_batch: many spec-mode solves in one launch per cluster size,
// one thread-block cluster per system (fs_cluster.cu).
// ---------------------------------------------------------------------------
extern "C" fs_status fs_pcg_solve_batch(fs_poisson_system *systems, int n, double rel_tol,
                                        int max_iter, const fs_exec_params *exec)
{
    if (n < 0 || (n > 0 && !systems) || max_iter < 0 || !(rel_tol > 0.0))
        return fail(FS_ERR_BAD_ARG, "fs_pcg_solve_batch: invalid argument");
    if (n == 0) return FS_OK;
    const int dev = exec ? exec->device : 0;
    CK(cudaSetDevice(dev));
    std::vector<ClusterPlan> plan(n);
    std::vector<size_t> off(n + 1, 0);
    for (int k = 0; k < n; k++) {
        const fs_poisson_system &q = systems[k];
        if (q.ni < 1 || q.nj < 1 || !q.material || !q.rhs || !q.result)
            return fail(FS_ERR_BAD_ARG, "fs_pcg_solve_batch: system %d: invalid argument", k);
        if (!valid_material(q.material, (size_t)q.ni * q.nj))
            return fail(FS_ERR_BAD_ARG, "fs_pcg_solve_batch: system %d: unknown material code", k);
        if (!cluster_plan(q.ni, q.nj, &plan[k]))
            return fail(FS_ERR_BAD_ARG,
                        "fs_pcg_solve_batch: system %d (%d x %d) exceeds the on-chip limit of %lld cells",
                        k, q.ni, q.nj, cluster_max_cells());
        off[k + 1] = off[k] + (size_t)q.ni * q.nj;
    }
    const size_t N = off[n];
    std::vector<void *> bufs;
    auto release = [&]() {
        for (void *p : bufs) cudaFree(p);
        bufs.clear();
    };
    auto dalloc_tmp = [&](void **p, size_t bytes) -> fs_status {
        cudaError_t e = cudaMalloc(p, bytes);
        if (e != cudaSuccess) {
            release();
            return fail(e == cudaErrorMemoryAllocation ? FS_ERR_OOM : FS_ERR_CUDA,
                        "fs_pcg_solve_batch: cudaMalloc: %s", cudaGetErrorString(e));
        }
        bufs.push_back(*p);
        return FS_OK;
    };
    auto check = [&](cudaError_t e, const char *what) -> fs_status {
        if (e == cudaSuccess) return FS_OK;
        release();
        return fail(FS_ERR_CUDA, "fs_pcg_solve_batch: %s: %s", what, cudaGetErrorString(e));
    };
    int8_t *mat = nullptr;
    uint8_t *info = nullptr;
    double *b = nullptr, *x = nullptr, *rel = nullptr;
    float *dts = nullptr;
    int *iters = nullptr, *chunk_last = nullptr;
    Scalars *sc = nullptr;
    ClusterSystem *sys = nullptr;
    TRY(dalloc_tmp((void **)&mat, N));
    TRY(dalloc_tmp((void **)&info, N));
    TRY(dalloc_tmp((void **)&b, N * 8));
    TRY(dalloc_tmp((void **)&x, N * 8));
    TRY(dalloc_tmp((void **)&rel, (size_t)n * 8));
    TRY(dalloc_tmp((void **)&dts, (size_t)n * 4));
    TRY(dalloc_tmp((void **)&iters, (size_t)n * 4));
    TRY(dalloc_tmp((void **)&chunk_last, 2 * sizeof(int)));
    TRY(dalloc_tmp((void **)&sc, sizeof(Scalars)));
    TRY(dalloc_tmp((void **)&sys, (size_t)n * sizeof(ClusterSystem)));
    cudaStream_t st = 0;
    std::vector<float> hdt(n);
    for (int k = 0; k < n; k++) hdt[k] = systems[k].dt;
    TRY(check(cudaMemcpyAsync(dts, hdt.data(), (size_t)n * 4, cudaMemcpyHostToDevice, st), "upload"));
    TRY(check(cudaMemsetAsync(sc, 0, sizeof(Scalars), st), "memset"));
    // the systems ordered by cluster size: one launch per size
    std::vector<int> order(n);
    for (int k = 0; k < n; k++) order[k] = k;
    auto key = [&](int k) { return plan[k].C * 64 + plan[k].K; };
    std::stable_sort(order.begin(), order.end(), [&](int a, int c) { return key(a) < key(c); });
    std::vector<ClusterSystem> hsys(n);
    for (int t = 0; t < n; t++) {
        const int k = order[t];
        const fs_poisson_system &q = systems[k];
        const size_t nk = (size_t)q.ni * q.nj;
        TRY(check(cudaMemcpyAsync(mat + off[k], q.material, nk, cudaMemcpyHostToDevice, st), "upload"));
        TRY(check(cudaMemcpyAsync(b + off[k], q.rhs, nk * 8, cudaMemcpyHostToDevice, st), "upload"));
        GridDims gd{q.ni, q.nj, q.ni / 3 + (q.ni % 3 != 0), q.nj / 3 + (q.nj % 3 != 0)};
        Grids G;
        G.material = mat + off[k];
        G.cell_info = info + off[k];
        launch_decomposition(gd, G, chunk_last, 1, (long long)nk, 0, sc, st);
        g_kernel_launches += 1;
        ClusterSystem &c = hsys[t];
        c.ni = q.ni;
        c.nj = q.nj;
        c.info = info + off[k];
        c.b = b + off[k];
        c.x = x + off[k];
        c.dt = dts + k;
        c.density = q.density;
        c.dx = q.dx;
        c.iters = iters + k;
        c.rel_res = rel + k;
    }
    TRY(check(cudaMemcpyAsync(sys, hsys.data(), (size_t)n * sizeof(ClusterSystem), cudaMemcpyHostToDevice, st),
              "upload"));
    ClusterParams cp;
    cp.tol = rel_tol;
    cp.eps_in = 1e-4f;
    cp.max_iter = max_iter;
    cp.max_outer = 32;
    for (int t0 = 0; t0 < n;) {
        int t1 = t0;
        ClusterPlan g = plan[order[t0]];
        while (t1 < n && key(order[t1]) == key(order[t0])) g.smem = std::max(g.smem, plan[order[t1++]].smem);
        TRY(check(launch_pcg_cluster(sys + t0, t1 - t0, g, cp, st), "cluster PCG"));
        g_kernel_launches += 1;
        t0 = t1;
    }
    std::vector<int> hit(n);
    std::vector<double> hrel(n);
    TRY(check(cudaMemcpyAsync(hit.data(), iters, (size_t)n * 4, cudaMemcpyDeviceToHost, st), "readback"));
    TRY(check(cudaMemcpyAsync(hrel.data(), rel, (size_t)n * 8, cudaMemcpyDeviceToHost, st), "readback"));
    for (int k = 0; k < n; k++) {
        const size_t nk = (size_t)systems[k].ni * systems[k].nj;
        TRY(check(cudaMemcpyAsync(systems[k].result, x + off[k], nk * 8, cudaMemcpyDeviceToHost, st),
                  "download"));
    }
    TRY(check(cudaStreamSynchronize(st), "sync"));
    release();
    for (int k = 0; k < n; k++) {
        systems[k].iterations = hit[k];
        systems[k].rel_residual = hrel[k];
    }
    return FS_OK;
}

// ---------------------------------------------------------------------------
// fs_cluster_autotune: picks the cluster size of the cluster solve for one
// grid shape by timing every size that fits (no reference counterpart)
// ---------------------------------------------------------------------------
extern "C" fs_status fs_cluster_autotune(int ni, int nj, int objective, int device, int *clusters,
                                         float *us_per_iteration)
{
    if (ni < 1 || nj < 1 || (objective != 0 && objective != 1))
        return fail(FS_ERR_BAD_ARG, "fs_cluster_autotune: invalid argument");
    CK(cudaSetDevice(device));
    std::vector<ClusterPlan> cand;
    cluster_candidates(ni, nj, &cand);
    if (cand.empty())
        return fail(FS_ERR_BAD_ARG, "fs_cluster_autotune: %d x %d exceeds the on-chip limit of %lld cells", ni,
                    nj, cluster_max_cells());
    // a synthetic system of this shape: fluid inside a one-cell solid wall,
    // a seeded right-hand side on the fluid cells
    const size_t N = (size_t)ni * nj;
    std::vector<int8_t> mat(N, (int8_t)M_FLUID);
    std::vector<double> rhs(N, 0.0);
    unsigned long long rng = 0x9E3779B97F4A7C15ull;
    for (int i = 0; i < ni; i++)
        for (int j = 0; j < nj; j++) {
            const size_t c = (size_t)i * nj + j;
            if (i == 0 || j == 0 || i == ni - 1 || j == nj - 1) {
                mat[c] = (int8_t)M_SOLID;
            } else {
                rng = rng * 6364136223846793005ull + 1442695040888963407ull;
                rhs[c] = (double)((rng >> 11) * (1.0 / 9007199254740992.0)) - 0.5;
            }
        }
    std::vector<void *> bufs;
    auto release = [&]() {
        for (void *p : bufs) cudaFree(p);
        bufs.clear();
    };
    auto dev = [&](size_t bytes) -> void * {
        void *p = nullptr;
        if (cudaMalloc(&p, bytes) != cudaSuccess) return nullptr;
        bufs.push_back(p);
        return p;
    };
    int8_t *dmat = (int8_t *)dev(N);
    uint8_t *info = (uint8_t *)dev(N);
    double *b = (double *)dev(N * 8), *x = (double *)dev(N * 8), *rel = (double *)dev(8);
    float *dt = (float *)dev(4);
    int *iters = (int *)dev(4), *chunk_last = (int *)dev(8);
    Scalars *sc = (Scalars *)dev(sizeof(Scalars));
    ClusterSystem *sys = (ClusterSystem *)dev(sizeof(ClusterSystem));
    if (!dmat || !info || !b || !x || !rel || !dt || !iters || !chunk_last || !sc || !sys) {
        release();
        return fail(FS_ERR_OOM, "fs_cluster_autotune: cudaMalloc failed");
    }
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    auto check = [&](cudaError_t e, const char *what) -> fs_status {
        if (e == cudaSuccess) return FS_OK;
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        release();
        return fail(FS_ERR_CUDA, "fs_cluster_autotune: %s: %s", what, cudaGetErrorString(e));
    };
    const float hdt = 1.f / 30.f;
    TRY(check(cudaMemcpy(dmat, mat.data(), N, cudaMemcpyHostToDevice), "upload"));
    TRY(check(cudaMemcpy(b, rhs.data(), N * 8, cudaMemcpyHostToDevice), "upload"));
    TRY(check(cudaMemcpy(dt, &hdt, 4, cudaMemcpyHostToDevice), "upload"));
    TRY(check(cudaMemset(sc, 0, sizeof(Scalars)), "memset"));
    GridDims gd{ni, nj, ni / 3 + (ni % 3 != 0), nj / 3 + (nj % 3 != 0)};
    Grids G;
    G.material = dmat;
    G.cell_info = info;
    launch_decomposition(gd, G, chunk_last, 1, (long long)N, 0, sc, 0);
    ClusterSystem hs;
    hs.ni = ni;
    hs.nj = nj;
    hs.info = info;
    hs.b = b;
    hs.x = x;
    hs.dt = dt;
    hs.density = 1000.0;
    hs.dx = 1.0 / std::max(ni, nj);
    hs.iters = iters;
    hs.rel_res = rel;
    TRY(check(cudaMemcpy(sys, &hs, sizeof(hs), cudaMemcpyHostToDevice), "upload"));
    TRY(check(cudaEventCreate(&e0), "event"));
    TRY(check(cudaEventCreate(&e1), "event"));
    // a fixed number of inner iterations (no stopping on the residual)
    const int kIters = 64;
    ClusterParams cp;
    cp.tol = 1e-300;
    cp.eps_in = 0.f;
    cp.max_iter = kIters;
    cp.max_outer = 1;
    int best = -1;
    float best_cost = 0.f, best_us = 0.f;
    for (size_t k = 0; k < cand.size(); k++) {
        float ms = 0.f;
        for (int rep = 0; rep < 2; rep++) { // the first run warms up
            TRY(check(cudaEventRecord(e0, 0), "event"));
            TRY(check(launch_pcg_cluster(sys, 1, cand[k], cp, 0), "launch"));
            TRY(check(cudaEventRecord(e1, 0), "event"));
            TRY(check(cudaEventSynchronize(e1), "sync"));
            TRY(check(cudaEventElapsedTime(&ms, e0, e1), "event"));
        }
        int it = 0;
        TRY(check(cudaMemcpy(&it, iters, 4, cudaMemcpyDeviceToHost), "readback"));
        const float us = 1e3f * ms / (float)std::max(it, 1);
        // throughput: SM time per iteration; latency: time per iteration
        const float cost = objective == 0 ? us * (float)cand[k].C : us;
        if (best < 0 || cost < best_cost) {
            best = (int)k;
            best_cost = cost;
            best_us = us;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    release();
    cluster_set_tuned(ni, nj, cand[best]);
    if (clusters) *clusters = cand[best].C;
    if (us_per_iteration) *us_per_iteration = best_us;
    return FS_OK;
}

// ---------------------------------------------------------------------------
// fs_resident_autotune: times every resident tile shape of the FP32 solve for
// a grid shape (200 iterations of a synthetic system through
// fs_pcg_solve_device, the best of three per shape) and records the fastest
// for later handles and solves of that shape in this process.
// ---------------------------------------------------------------------------
extern "C" fs_status fs_resident_autotune(int ni, int nj, int device, int *tile_rows, int *tile_cols,
                                          float *us_per_iteration)
{
    if (ni < 1 || nj < 1) return fail(FS_ERR_BAD_ARG, "fs_resident_autotune: invalid argument");
    CK(cudaSetDevice(device));
    std::vector<std::pair<int, int>> cand;
    resident_candidates(ni, nj, &cand);
    if (cand.empty())
        return fail(FS_ERR_BAD_ARG, "fs_resident_autotune: %d x %d needs more tiles than SMs", ni, nj);
    // fluid inside a one-cell solid wall, a seeded right-hand side on the fluid
    const size_t N = (size_t)ni * nj;
    std::vector<int8_t> mat(N, (int8_t)M_FLUID);
    std::vector<float> rhs(N, 0.f);
    unsigned long long rng = 0x9E3779B97F4A7C15ull;
    for (int i = 0; i < ni; i++)
        for (int j = 0; j < nj; j++) {
            const size_t c = (size_t)i * nj + j;
            if (i == 0 || j == 0 || i == ni - 1 || j == nj - 1) {
                mat[c] = (int8_t)M_SOLID;
            } else {
                rng = rng * 6364136223846793005ull + 1442695040888963407ull;
                rhs[c] = (float)((rng >> 11) * (1.0 / 9007199254740992.0)) - 0.5f;
            }
        }
    int8_t *dm = nullptr;
    float *db = nullptr, *dres = nullptr;
    auto release = [&]() {
        if (dm) cudaFree(dm);
        if (db) cudaFree(db);
        if (dres) cudaFree(dres);
    };
    cudaError_t e = cudaMalloc(&dm, N);
    if (e == cudaSuccess) e = cudaMalloc(&db, N * 4);
    if (e == cudaSuccess) e = cudaMalloc(&dres, N * 4);
    if (e == cudaSuccess) e = cudaMemcpy(dm, mat.data(), N, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(db, rhs.data(), N * 4, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        release();
        return fail(e == cudaErrorMemoryAllocation ? FS_ERR_OOM : FS_ERR_CUDA, "fs_resident_autotune: %s",
                    cudaGetErrorString(e));
    }
    fs_exec_params ex{FS_PCG_FP32, 1, device, 0, {0, 0, 0, 0}};
    double best_us = -1.0;
    size_t best = 0;
    for (size_t k = 0; k < cand.size(); k++) {
        resident_set_tuned(ni, nj, cand[k].first, cand[k].second);
        double t_min = -1.0;
        for (int rep = 0; rep < 4; rep++) {
            int its = 0;
            const auto t0 = std::chrono::steady_clock::now();
            // tolerance 0: every solve runs its 200 iterations
            const fs_status st = fs_pcg_solve_device(ni, nj, dm, 1.0f / 60.0f, 1000.0, 1.0 / ni, db, dres, 200, 0.0,
                                                     &ex, &its);
            const double us = std::chrono::duration<double, std::micro>(std::chrono::steady_clock::now() - t0).count();
            if (st != FS_OK) {
                resident_set_tuned(ni, nj, 0, 0);
                release();
                return st;
            }
            if (rep > 0 && (t_min < 0.0 || us < t_min)) t_min = us; // the first is a warm-up
        }
        if (best_us < 0.0 || t_min < best_us) {
            best_us = t_min;
            best = k;
        }
    }
    release();
    resident_set_tuned(ni, nj, cand[best].first, cand[best].second);
    if (tile_rows) *tile_rows = cand[best].first;
    if (tile_cols) *tile_cols = cand[best].second;
    if (us_per_iteration) *us_per_iteration = (float)(best_us / 200.0);
    return FS_OK;
}

// ---------------------------------------------------------------------------
// fs_server_*: the device-resident request loop (no reference counterpart).
// One persistent launch of the cluster solve (launch_serve, fs_cluster.cu)
// whose clusters take requests from a ring in mapped pinned memory: the host
// copies a request's material, right-hand side and dt into a free slot,
// writes the slot into the ring and advances the tail; a cluster claims it,
// builds the operator, solves, and flags the slot done in mapped memory.  The
// host never waits for the device to accept a request.  The launch leaves
// when the ring stays empty for about 50 ms (or on destroy); a submit or a
// poll that finds unclaimed requests and no launch running starts another.
// ---------------------------------------------------------------------------
namespace {
constexpr unsigned kServeRing = 1u << 16; // ring entries; requests in flight never exceed the slots
constexpr long long kServeIdlePolls = 25000;
constexpr size_t kServeHead = 64; // tail, stop
} // namespace

struct fs_server {
    int device = 0;
    int max_ni = 0, max_nj = 0, slots = 0;
    ClusterPlan plan{};
    ClusterParams params{};
    cudaStream_t kst = nullptr, cst = nullptr; // the server launch; copies
    cudaEvent_t ev = nullptr;                  // recorded after each server launch
    bool launched = false;
    int clusters = 0;
    unsigned char *host = nullptr, *mapped = nullptr; // control block: host / device address
    ServeSlot *d_slots = nullptr;
    unsigned *d_claimed = nullptr;
    void *slot_mem = nullptr;
    size_t slot_bytes = 0, cells = 0;
    std::vector<int> free_slots;
    struct Req {
        unsigned k;
        int slot, ni, nj;
    };
    std::vector<std::pair<unsigned long long, Req>> reqs;
    unsigned next_k = 0;
    unsigned long long next_ticket = 1;
    std::mutex mu;

    volatile unsigned *tail() { return reinterpret_cast<volatile unsigned *>(host); }
    volatile int *stop() { return reinterpret_cast<volatile int *>(host + 4); }
    volatile unsigned *ring() { return reinterpret_cast<volatile unsigned *>(host + kServeHead); }
    volatile unsigned *started() { return ring() + kServeRing; }
    volatile unsigned *done() { return started() + slots; }
    // a slot's buffers: material, operator bytes, b, x, then dt, iterations, residual
    unsigned char *slot_base(int k) { return static_cast<unsigned char *>(slot_mem) + (size_t)k * slot_bytes; }
    size_t a256(size_t x) const { return (x + 255) & ~(size_t)255; }
    int8_t *mat(int k) { return reinterpret_cast<int8_t *>(slot_base(k)); }
    uint8_t *info(int k) { return slot_base(k) + a256(cells); }
    double *b(int k) { return reinterpret_cast<double *>(slot_base(k) + 2 * a256(cells)); }
    double *x(int k) { return b(k) + cells; }
    unsigned char *tailb(int k) { return reinterpret_cast<unsigned char *>(x(k) + cells); }
    float *dt(int k) { return reinterpret_cast<float *>(tailb(k)); }
    int *iters(int k) { return reinterpret_cast<int *>(tailb(k) + 16); }
    double *rel(int k) { return reinterpret_cast<double *>(tailb(k) + 32); }
};

static void server_free(fs_server *s)
{
    if (s->kst) cudaStreamDestroy(s->kst);
    if (s->cst) cudaStreamDestroy(s->cst);
    if (s->ev) cudaEventDestroy(s->ev);
    if (s->host) cudaFreeHost(s->host);
    if (s->d_slots) cudaFree(s->d_slots);
    if (s->d_claimed) cudaFree(s->d_claimed);
    if (s->slot_mem) cudaFree(s->slot_mem);
    delete s;
}

// a server launch is running, or one is started; FS_ERR_CUDA if the last
// launch failed
static fs_status server_running(fs_server *s)
{
    if (s->launched) {
        const cudaError_t q = cudaEventQuery(s->ev);
        if (q == cudaErrorNotReady) return FS_OK;
        if (q != cudaSuccess) return fail(FS_ERR_CUDA, "fs_server: the server launch failed: %s", cudaGetErrorString(q));
    }
    ServeQueue q{};
    q.slots = s->d_slots;
    q.tail = reinterpret_cast<const unsigned *>(s->mapped);
    q.stop = reinterpret_cast<const int *>(s->mapped + 4);
    q.ring = reinterpret_cast<const unsigned *>(s->mapped + kServeHead);
    q.ring_size = kServeRing;
    q.claimed = s->d_claimed;
    q.started = reinterpret_cast<unsigned *>(s->mapped + kServeHead) + kServeRing;
    q.done = q.started + s->slots;
    q.idle_polls = kServeIdlePolls;
    cudaError_t e = launch_serve(q, s->plan, s->params, s->kst, &s->clusters);
    if (e == cudaSuccess) e = cudaEventRecord(s->ev, s->kst);
    if (e != cudaSuccess) return fail(FS_ERR_CUDA, "fs_server: launch: %s", cudaGetErrorString(e));
    s->launched = true;
    g_kernel_launches += 1;
    return FS_OK;
}

extern "C" fs_status fs_server_create(int device, int max_ni, int max_nj, int slots, double rel_tol,
                                      int max_iter, fs_server **out)
{
    if (!out || max_ni < 1 || max_nj < 1 || slots < 1 || slots > 4096 || !(rel_tol > 0.0) || max_iter < 1)
        return fail(FS_ERR_BAD_ARG, "fs_server_create: invalid argument");
    *out = nullptr;
    if (cudaSetDevice(device) != cudaSuccess) return fail(FS_ERR_CUDA, "fs_server_create: no device %d", device);
    fs_server *s = new fs_server();
    s->device = device;
    s->max_ni = max_ni;
    s->max_nj = max_nj;
    s->slots = slots;
    if (!cluster_plan(max_ni, max_nj, &s->plan)) {
        delete s;
        return fail(FS_ERR_BAD_ARG, "fs_server_create: %d x %d exceeds the on-chip limit of the cluster solve",
                    max_ni, max_nj);
    }
    s->params = spec_params();
    s->params.tol = rel_tol;
    s->params.max_iter = max_iter;
    s->cells = (size_t)max_ni * max_nj;
    s->slot_bytes = s->a256(2 * s->a256(s->cells) + 16 * s->cells + 64);
    const size_t hbytes = kServeHead + 4 * ((size_t)kServeRing + 2 * (size_t)slots);
    cudaError_t e = cudaStreamCreateWithFlags(&s->kst, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->cst, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->ev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaHostAlloc((void **)&s->host, hbytes, cudaHostAllocMapped);
    if (e == cudaSuccess) e = cudaHostGetDevicePointer((void **)&s->mapped, s->host, 0);
    if (e == cudaSuccess) e = cudaMalloc(&s->d_slots, (size_t)slots * sizeof(ServeSlot));
    if (e == cudaSuccess) e = cudaMalloc(&s->d_claimed, sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMalloc(&s->slot_mem, (size_t)slots * s->slot_bytes);
    if (e == cudaSuccess) e = cudaMemset(s->d_claimed, 0, sizeof(unsigned));
    if (e != cudaSuccess) {
        server_free(s);
        return fail(e == cudaErrorMemoryAllocation ? FS_ERR_OOM : FS_ERR_CUDA, "fs_server_create: %s",
                    cudaGetErrorString(e));
    }
    memset(s->host, 0, hbytes);
    for (int k = slots - 1; k >= 0; k--) s->free_slots.push_back(k);
    *out = s;
    return FS_OK;
}

extern "C" fs_status fs_server_submit(fs_server *s, const fs_poisson_system *q, unsigned long long *ticket)
{
    if (!s || !q || !ticket || q->ni < 1 || q->nj < 1 || !q->material || !q->rhs)
        return fail(FS_ERR_BAD_ARG, "fs_server_submit: invalid argument");
    if (q->ni > s->max_ni || q->nj > s->max_nj)
        return fail(FS_ERR_BAD_ARG, "fs_server_submit: %d x %d exceeds the server's %d x %d", q->ni, q->nj, s->max_ni,
                    s->max_nj);
    const size_t N = (size_t)q->ni * q->nj;
    if (!valid_material(q->material, N)) return fail(FS_ERR_BAD_ARG, "fs_server_submit: unknown material code");
    std::lock_guard<std::mutex> lock(s->mu);
    if (s->free_slots.empty()) return fail(FS_ERR_STATE, "fs_server_submit: every slot holds a request not yet taken");
    CK(cudaSetDevice(s->device));
    const int k = s->free_slots.back();
    ServeSlot h{};
    h.sys.ni = q->ni;
    h.sys.nj = q->nj;
    h.sys.info = s->info(k);
    h.sys.b = s->b(k);
    h.sys.x = s->x(k);
    h.sys.dt = s->dt(k);
    h.sys.density = q->density;
    h.sys.dx = q->dx;
    h.sys.iters = s->iters(k);
    h.sys.rel_res = s->rel(k);
    h.material = s->mat(k);
    h.info = s->info(k);
    cudaError_t e = cudaMemcpyAsync(s->mat(k), q->material, N, cudaMemcpyHostToDevice, s->cst);
    if (e == cudaSuccess) e = cudaMemcpyAsync(s->b(k), q->rhs, N * 8, cudaMemcpyHostToDevice, s->cst);
    if (e == cudaSuccess) e = cudaMemcpyAsync(s->dt(k), &q->dt, sizeof(float), cudaMemcpyHostToDevice, s->cst);
    if (e == cudaSuccess) e = cudaMemcpyAsync(s->d_slots + k, &h, sizeof(h), cudaMemcpyHostToDevice, s->cst);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->cst); // in device memory before the ring names it
    if (e != cudaSuccess) return fail(FS_ERR_CUDA, "fs_server_submit: %s", cudaGetErrorString(e));
    s->free_slots.pop_back();
    const unsigned rk = s->next_k++;
    s->started()[k] = 0u;
    s->done()[k] = 0u;
    s->ring()[rk % kServeRing] = (unsigned)k;
    std::atomic_thread_fence(std::memory_order_seq_cst);
    *s->tail() = rk + 1;
    std::atomic_thread_fence(std::memory_order_seq_cst);
    *ticket = s->next_ticket++;
    s->reqs.push_back({*ticket, fs_server::Req{rk, k, q->ni, q->nj}});
    return server_running(s);
}

static fs_server::Req *server_find(fs_server *s, unsigned long long ticket, size_t *at)
{
    for (size_t i = 0; i < s->reqs.size(); i++)
        if (s->reqs[i].first == ticket) {
            if (at) *at = i;
            return &s->reqs[i].second;
        }
    return nullptr;
}

extern "C" fs_status fs_server_poll(fs_server *s, unsigned long long ticket, int *done)
{
    if (!s || !done) return fail(FS_ERR_BAD_ARG, "fs_server_poll: invalid argument");
    std::lock_guard<std::mutex> lock(s->mu);
    fs_server::Req *r = server_find(s, ticket, nullptr);
    if (!r) return fail(FS_ERR_BAD_ARG, "fs_server_poll: unknown ticket");
    *done = s->done()[r->slot] == r->k + 1 ? 1 : 0;
    std::atomic_thread_fence(std::memory_order_seq_cst);
    if (*done) return FS_OK;
    CK(cudaSetDevice(s->device));
    // a request not yet claimed needs a launch to claim it (one that left
    // for lack of work is started again); a claimed one is being solved
    return server_running(s);
}

extern "C" fs_status fs_server_take(fs_server *s, unsigned long long ticket, double *result, int *iterations,
                                    double *rel_residual)
{
    if (!s || !result) return fail(FS_ERR_BAD_ARG, "fs_server_take: invalid argument");
    std::lock_guard<std::mutex> lock(s->mu);
    size_t at = 0;
    fs_server::Req *r = server_find(s, ticket, &at);
    if (!r) return fail(FS_ERR_BAD_ARG, "fs_server_take: unknown ticket");
    if (s->done()[r->slot] != r->k + 1) return fail(FS_ERR_STATE, "fs_server_take: the request is not done");
    std::atomic_thread_fence(std::memory_order_seq_cst);
    CK(cudaSetDevice(s->device));
    const int k = r->slot;
    const size_t N = (size_t)r->ni * r->nj;
    int it = 0;
    double rel = 0.0;
    cudaError_t e = cudaMemcpyAsync(result, s->x(k), N * 8, cudaMemcpyDeviceToHost, s->cst);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&it, s->iters(k), sizeof(int), cudaMemcpyDeviceToHost, s->cst);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&rel, s->rel(k), sizeof(double), cudaMemcpyDeviceToHost, s->cst);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->cst);
    if (e != cudaSuccess) return fail(FS_ERR_CUDA, "fs_server_take: %s", cudaGetErrorString(e));
    if (iterations) *iterations = it;
    if (rel_residual) *rel_residual = rel;
    s->free_slots.push_back(k);
    s->reqs.erase(s->reqs.begin() + (long)at);
    return FS_OK;
}

extern "C" fs_status fs_server_clusters(fs_server *s, int *clusters)
{
    if (!s || !clusters) return fail(FS_ERR_BAD_ARG, "fs_server_clusters: invalid argument");
    std::lock_guard<std::mutex> lock(s->mu);
    *clusters = s->clusters;
    return FS_OK;
}

extern "C" fs_status fs_server_destroy(fs_server *s)
{
    if (!s) return FS_OK;
    fs_status st = FS_OK;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        cudaSetDevice(s->device);
        *s->stop() = 1;
        std::atomic_thread_fence(std::memory_order_seq_cst);
        // the launch leaves after the requests its clusters hold (each bounded
        // by the inner iteration limit); requests not yet claimed are dropped
        if (s->launched && cudaEventSynchronize(s->ev) != cudaSuccess)
            st = fail(FS_ERR_CUDA, "fs_server_destroy: the server launch failed");
    }
    server_free(s);
    return st;
}

// ---------------------------------------------------------------------------
// fs_pcg_solve_device_noalloc: the FP32 device-pointer solve with all of its
// scratch in one fixed device array (no counterpart in the reference).
//
// Some callers cannot allocate device memory once they are running: a
// simulation or serving loop that reserved its whole device budget when it
// started (a cudaMalloc there can fail), or one that cannot afford the device
// synchronisation cudaMalloc and cudaFree may imply while its other streams
// are busy.  This path calls neither, nor any other allocating routine; it
// uses only the array below, which is part of the library's device image and
// so exists, on every device the library is loaded on, before the first call.
// Its cost for everyone is kNaBytes (about 9 MB) of device memory.
//
// Limit: ni * nj <= kNoAllocMaxCells (512 x 512 = 262144 cells), FP32 only,
// at most kNoAllocMaxParts pool threads.  Larger requests are rejected before
// any device work.
//
// The first call on a device looks up the array's address there
// (cudaGetSymbolAddress, with that device current); make that first call
// before any stream capture begins.  The address is kept for the life of the
// process, so calls after a reset of that device (cudaDeviceReset) are not
// supported.  All calls use the same array and it keeps
// whatever the last call left in it, so each call clears the words that must
// start at zero (scalars, barrier counter, epoch flags) itself.  Two calls that
// overlapped on the GPU would race on the array; this function holds a
// process-wide lock and returns only after its solve has finished, so its own
// calls never overlap.
// ---------------------------------------------------------------------------
namespace {
constexpr size_t kNoAllocMaxCells = 512 * 512;
constexpr int kNoAllocMaxGrid = 4096;  // cooperative blocks the solve may use
constexpr int kNoAllocMaxParts = 4096; // splitRange parts (pool threads)
constexpr size_t na_up(size_t x) { return (x + 255) & ~(size_t)255; }
constexpr size_t kNaInfo = 0;
constexpr size_t kNaR0 = na_up(kNaInfo + kNoAllocMaxCells);
constexpr size_t kNaR1 = na_up(kNaR0 + 4 * kNoAllocMaxCells);
constexpr size_t kNaS0 = na_up(kNaR1 + 4 * kNoAllocMaxCells);
constexpr size_t kNaS1 = na_up(kNaS0 + 4 * kNoAllocMaxCells);
constexpr size_t kNaPartials = na_up(kNaS1 + 4 * kNoAllocMaxCells);
constexpr size_t kNaChunkEnd = na_up(kNaPartials + 8 * (8 * (size_t)kNoAllocMaxGrid + 16));
constexpr size_t kNaChunkLast = na_up(kNaChunkEnd + 4 * ((size_t)kNoAllocMaxParts + 1));
constexpr size_t kNaChunkVal = na_up(kNaChunkLast + 4 * ((size_t)kNoAllocMaxParts + 1));
constexpr size_t kNaLlR = na_up(kNaChunkVal + 8 * ((size_t)kNoAllocMaxParts + 1));
constexpr size_t kNaLlS = na_up(kNaLlR + 8 * kNoAllocMaxCells);
constexpr size_t kNaLlRec = na_up(kNaLlS + 8 * kNoAllocMaxCells);
constexpr size_t kNaBar = na_up(kNaLlRec + 8 * kLlRecWords);
constexpr size_t kNaScalars = na_up(kNaBar + sizeof(GridBarrier));
constexpr size_t kNaBytes = na_up(kNaScalars + sizeof(Scalars));
} // namespace

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNaBytes];

static std::mutex g_noalloc_mu;
static unsigned char *g_noalloc_base[64]; // the array's address per device
static LlBuffers g_noalloc_ll[64];        // its exchange-word regions per device

// splitRange chunk ends (the reference's partition of [0, N) into parts)
__global__ void k_na_chunk_ends(int *ends, int parts, long long ps, long long rem)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < parts) ends[i] = (int)((long long)(i + 1) * ps + min((long long)(i + 1), rem));
}

extern "C" fs_status fs_pcg_solve_device_noalloc(int ni, int nj, const int8_t *material_device,
                                                 float dt, double density, double dx,
                                                 const float *rhs_device, float *result_device,
                                                 int iter_limit, double tol,
                                                 const fs_exec_params *exec, int *iterations)
{
    if (ni < 1 || nj < 1 || !material_device || !rhs_device || !result_device || iter_limit < 0)
        return fail(FS_ERR_BAD_ARG, "fs_pcg_solve_device_noalloc: invalid argument");
    const long long N = (long long)ni * nj;
    if (N > (long long)kNoAllocMaxCells)
        return fail(FS_ERR_BAD_ARG,
                    "fs_pcg_solve_device_noalloc: %d x %d = %lld cells exceeds the fixed scratch "
                    "maximum of %zu cells",
                    ni, nj, N, kNoAllocMaxCells);
    if (exec && exec->pcg_precision == FS_PCG_FP64)
        return fail(FS_ERR_UNSUPPORTED, "fs_pcg_solve_device_noalloc: FP32 only");
    const int dev = exec ? exec->device : 0;
    if (dev < 0 || dev >= 64) return fail(FS_ERR_BAD_ARG, "fs_pcg_solve_device_noalloc: bad device");
    const int T = (exec && exec->pool_threads > 0) ? exec->pool_threads : default_pool_threads();
    const long long parts = std::max<long long>(1, std::min<long long>(T, N));
    if (parts > kNoAllocMaxParts)
        return fail(FS_ERR_BAD_ARG, "fs_pcg_solve_device_noalloc: %lld pool threads exceed %d", parts,
                    kNoAllocMaxParts);

    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    CK(cudaSetDevice(dev));
    if (!g_noalloc_base[dev]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return fail(FS_ERR_CUDA, "fs_pcg_solve_device_noalloc: cudaGetSymbolAddress: %s",
                        cudaGetErrorString(e));
        g_noalloc_base[dev] = static_cast<unsigned char *>(p);
    }
    if (pcg_grid_size<float>(N) > kNoAllocMaxGrid)
        return fail(FS_ERR_UNSUPPORTED, "fs_pcg_solve_device_noalloc: device needs more than %d blocks",
                    kNoAllocMaxGrid);
    unsigned char *base = g_noalloc_base[dev];
    uint8_t *info = base + kNaInfo;
    int *chunk_end = reinterpret_cast<int *>(base + kNaChunkEnd);
    int *chunk_last = reinterpret_cast<int *>(base + kNaChunkLast);
    Scalars *sc = reinterpret_cast<Scalars *>(base + kNaScalars);
    cudaStream_t st = 0;

    long long ps = 1, rem = 0;
    split_range_params(N, T, &ps, &rem);
    // status, iteration count and wrap flag start at zero; the barrier words
    // and epoch flags are zeroed by the PCG launchers
    CK(cudaMemsetAsync(sc, 0, sizeof(Scalars), st));
    k_na_chunk_ends<<<(unsigned)((parts + 255) / 256), 256, 0, st>>>(chunk_end, (int)parts, ps, rem);
    k_set_dt<<<1, 1, 0, st>>>(sc, dt);
    GridDims d{ni, nj, ni / 3 + (ni % 3 != 0), nj / 3 + (nj % 3 != 0)};
    Grids G;
    G.material = const_cast<int8_t *>(material_device);
    G.cell_info = info;
    launch_decomposition(d, G, chunk_last, (int)parts, ps, rem, sc, st);
    g_kernel_launches += 3;

    PcgArgs<float> a{};
    a.ni = ni;
    a.nj = nj;
    a.N = N;
    a.info = info;
    a.b = rhs_device;
    a.x = result_device;
    a.r0 = reinterpret_cast<float *>(base + kNaR0);
    a.r1 = reinterpret_cast<float *>(base + kNaR1);
    a.s0 = reinterpret_cast<float *>(base + kNaS0);
    a.s1 = reinterpret_cast<float *>(base + kNaS1);
    LlBuffers &ll = g_noalloc_ll[dev];
    ll.r = reinterpret_cast<unsigned long long *>(base + kNaLlR);
    ll.s = reinterpret_cast<unsigned long long *>(base + kNaLlS);
    ll.rec = reinterpret_cast<unsigned long long *>(base + kNaLlRec);
    ll.words = kNoAllocMaxCells;
    a.ll_r = ll.r;
    a.ll_s = ll.s;
    a.partials = reinterpret_cast<double *>(base + kNaPartials);
    a.chunk_end = chunk_end;
    a.chunk_last_unit = chunk_last;
    a.chunk_val = reinterpret_cast<double *>(base + kNaChunkVal);
    a.nchunks = (int)parts;
    a.sc = sc;
    a.density = density;
    a.dx = dx;
    a.iter_limit = iter_limit;
    a.tol = tol;
    a.iters_out = &sc->density_iters;
    a.status = &sc->pcg_status;
    a.spin_limit = exec ? exec->wait_polls : 0;
    a.bar = reinterpret_cast<GridBarrier *>(base + kNaBar);
    a.wrap_flag = &sc->wrap_units;
    a.mode = 0;
    cudaError_t e;
    int launched = 0, ti = 0, tj = 0;
    // the kernel choice of fs_pcg_solve_device: resident tiles, else TMA
    // tiles (their tensor maps are host structures that point into the fixed
    // array and the caller's buffers), else the tiled / linear-index pair
    TmaMaps maps;
    if (resident_tile_shape(ni, nj, &ti, &tj)) {
        a.mode = 2; // the linear-index kernel takes over when a unit row wraps
        e = launch_pcg_resident(a, ti, tj, st, &ll);
        if (e == cudaSuccess) e = launch_pcg_linear_if_wrap(a, st);
        launched = 2;
    } else if (tma_tile_shape(ni, nj, &ti, &tj) &&
               tma_maps(&maps, ni, nj, ti, tj, info, rhs_device, result_device, a.r0, a.r1, a.s0,
                        a.s1) &&
               tma_store_maps(&maps, ni, nj, ti, tj, a.r0, a.r1, a.s0, a.s1)) {
        a.mode = 2;
        e = launch_pcg_tma(a, maps, ti, tj, st);
        if (e == cudaSuccess) e = launch_pcg_linear_if_wrap(a, st);
        launched = 2;
    } else {
        e = launch_pcg<float>(a, st, &launched);
    }
    g_kernel_launches += launched;
    if (e != cudaSuccess)
        return fail(FS_ERR_CUDA, "fs_pcg_solve_device_noalloc: PCG launch: %s", cudaGetErrorString(e));
    Scalars h{};
    CK(cudaMemcpyAsync(&h, sc, sizeof(Scalars), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (h.pcg_status != 0)
        return fail(FS_ERR_TIMEOUT, "fs_pcg_solve_device_noalloc: a PCG grid barrier wait timed out");
    if (iterations) *iterations = h.density_iters;
    return FS_OK;
}
