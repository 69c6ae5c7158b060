// ref_harness.cpp -- drives the reference FlipSolver2d through its own C++ API
// and exports the oracle interface of fsoracle.h.
//
// TEST INFRASTRUCTURE: compiled (by oracle/Makefile.ref) together with the
// reference sources, in place, into oracle/_ref/libfsref.so.  It runs the
// reference's own code paths unmodified: FlipSolver::step()
// (flipsolver2d.cpp:412-462), FlipSolver::stepFrame() (:464-500) and the
// protected stage methods that step() calls, reached through a subclass.  The
// harness adds only state import/export (particles bin by bin, grids) and a
// capture of the projection's right-hand side and pressure, which the
// reference keeps in locals (flipsolver2d.cpp:96-105).
#include "fsoracle.h"

#include <cstring>
#include <sstream>
#include <type_traits>
#include <vector>

#include "flipsolver2d.h"
#include "nbflipsolver.h"

namespace {

// what the C interface calls, for either solver class
struct RefApi {
    virtual ~RefApi() = default;
    virtual void runStage(int stage) = 0;
    virtual void stepOnce() = 0;
    virtual void frame() = 0;
    virtual void setStepDt(float dt) = 0;
    virtual float getStepDt() = 0;
    virtual void firstInit() = 0;
    virtual float maxVel() = 0;
    virtual size_t gridBytes(int which) = 0;
    virtual int getGrid(int which, void *out) = 0;
    virtual int setGrid(int which, const void *in) = 0;
    virtual size_t binCount() = 0;
    virtual size_t nParticles() = 0;
    virtual void getParticles(int32_t *counts, float *pos, float *vel, float *visc, uint8_t *dead) = 0;
    virtual void setParticles(const int32_t *counts, const float *pos, const float *vel,
                              const float *visc, const uint8_t *dead) = 0;
    virtual int stat(int which) = 0;
    virtual int getRng(uint32_t *state) = 0;
    virtual int setRng(const uint32_t *state) = 0;
    virtual void addGeom(Obstacle &o) = 0;
    virtual void addFluid(Emitter &e) = 0;
    virtual void addSinkObj(Sink &k) = 0;
    virtual void addSrc(Emitter &e) = 0;
};

// Base: FlipSolver or NBFlipSolver.  The stages reach the protected methods
// step() calls; virtual dispatch selects NB-FLIP's overrides of advect,
// afterTransfer, centeredParamsToGrid, reseedParticles, firstFrameInit and
// step.
template <class Base> class RefSolverT : public Base, public RefApi {
public:
    using Base::m_stats; using Base::m_stepDt; using Base::m_viscosityPropertyIndex;
    using Base::m_sizeI; using Base::m_sizeJ; using Base::m_materialGrid; using Base::m_solidSdf;
    using Base::m_fluidSdf; using Base::m_fluidVelocityGrid; using Base::m_savedFluidVelocityGrid;
    using Base::m_viscosityGrid; using Base::m_knownCenteredParams; using Base::m_densityGrid;
    using Base::m_fluidParticleCounts; using Base::m_solidId; using Base::m_divergenceControl;
    using Base::m_pressureRhs; using Base::m_pressureSolverResult; using Base::m_emitterId;
    using Base::m_markerParticles; using Base::m_pressureMatrix; using Base::m_pressurePrecond;
    using Base::m_pressureSolver; using Base::m_pcgIterLimit; using Base::m_projectTolerance;
    using Base::m_viscosityEnabled; using Base::m_randEngine;
    using Base::getPressureProjectionMatrix; using Base::getIPPCoefficients; using Base::cellCount;
    using Base::calcPressureRhs;

    template <class P> explicit RefSolverT(const P *p) : Base(p) {}

    bool capturePressure = true;
    std::vector<double> capRhs;
    std::vector<double> capPressure;

    // The projection keeps its pressure in a local vector; capture it by
    // running the same two calls the reference's project() makes
    // (calcPressureRhs, LinearSolver::solve; flipsolver2d.cpp:99-105) before
    // delegating to the reference's project().  The solve is deterministic, so
    // the captured vector equals the one project() applies.
    void project() override
    {
        if (capturePressure) {
            capRhs.assign(cellCount(), 0.0);
            capPressure.assign(cellCount(), 0.0);
            calcPressureRhs(capRhs);
            m_pressureSolver.solve(m_pressureMatrix, m_pressurePrecond, capPressure,
                                   capRhs, m_pcgIterLimit, m_projectTolerance);
        }
        FlipSolver::project();
    }

    void runStage(int stage) override
    {
        switch (stage) {
        case FSO_ADVECT: this->advect(); break;
        case FSO_DECOMPOSITION:
            m_pressureMatrix = getPressureProjectionMatrix();
            m_pressurePrecond = getIPPCoefficients(m_pressureMatrix);
            break;
        case FSO_REBIN:
            this->pruneParticles();
            m_markerParticles.rebinParticles();
            break;
        case FSO_DENSITY:
            m_stats.reset(); // report this stage's solve
            if (!m_viscosityEnabled) this->densityCorrection();
            break;
        case FSO_P2G: this->particleToGrid(); break;
        case FSO_SDF: this->updateSdf(); break;
        case FSO_MATERIALS: this->updateMaterials(); break;
        case FSO_AFTER_TRANSFER: this->afterTransfer(); break;
        case FSO_LEVELSET: this->extrapolateLevelsetInside(m_fluidSdf); break;
        case FSO_LEVELSET_OUTSIDE: this->extrapolateLevelsetOutside(m_fluidSdf); break;
        case FSO_VEL_EXTRAP: m_fluidVelocityGrid.extrapolate(10); break;
        case FSO_SAVE_GRID: m_savedFluidVelocityGrid = m_fluidVelocityGrid; break;
        case FSO_BODY_FORCES: this->applyBodyForces(); break;
        case FSO_PROJECT:
            m_stats.reset();
            project();
            break;
        case FSO_FRICTION: this->updateVelocityFromSolids(); break;
        case FSO_G2P: this->particleUpdate(); break;
        case FSO_COUNT: this->countParticles(); break;
        case FSO_RESEED: this->reseedParticles(); break;
        case FSO_DENSITY_GRID: this->updateDensityGrid(); break;
        case FSO_VISCOSITY: this->applyViscosity(); break;
        default: break;
        }
    }

    void stepOnce() override
    {
        m_stats.reset();
        this->step();
    }
    void frame() override { this->stepFrame(); }

    void setStepDt(float dt) override { m_stepDt = dt; }
    float getStepDt() override { return this->stepDt(); }
    void firstInit() override { this->firstFrameInit(); }
    float maxVel() override { return this->maxParticleVelocity(); }
    size_t nParticles() override { return this->particleCount(); }
    void addGeom(Obstacle &o) override { this->addGeometry(o); }
    void addFluid(Emitter &e) override { this->addInitialFluid(e); }
    void addSinkObj(Sink &k) override { this->addSink(k); }
    void addSrc(Emitter &e) override { this->addSource(e); }

    // libstdc++ writes the 624 state words, then the position of the next one
    int getRng(uint32_t *state) override
    {
        std::ostringstream os;
        os << m_randEngine;
        std::istringstream is(os.str());
        for (int k = 0; k < 625; k++) {
            unsigned long v = 0;
            if (!(is >> v)) return -1;
            state[k] = static_cast<uint32_t>(v);
        }
        return 0;
    }
    int setRng(const uint32_t *state) override
    {
        std::ostringstream os;
        for (int k = 0; k < 625; k++) os << state[k] << (k < 624 ? " " : "");
        std::istringstream is(os.str());
        is >> m_randEngine;
        return is.fail() ? -1 : 0;
    }
    int stat(int which) override
    {
        switch (which) {
        case FSO_S_DENSITY_ITERS: return m_stats.densityIterations();
        case FSO_S_PRESSURE_ITERS: return m_stats.pressureIterations();
        case FSO_S_SUBSTEPS: return m_stats.substepCount();
        case FSO_S_FRAME: return this->frameNumber();
        case FSO_S_POOL_THREADS: return static_cast<int>(ThreadPool::i()->threadCount());
        case FSO_S_VISCOSITY_ITERS: return m_stats.viscosityIterations();
        default: return -1;
        }
    }
    static constexpr bool kNb = std::is_same_v<Base, NBFlipSolver>;

    size_t viscIndex() const { return m_viscosityPropertyIndex; }
    const SolverStats &stats() const { return m_stats; }

    size_t gridBytes(int which) override
    {
        const size_t n = static_cast<size_t>(m_sizeI) * m_sizeJ;
        const size_t nu = static_cast<size_t>(m_sizeI + 1) * m_sizeJ;
        const size_t nv = static_cast<size_t>(m_sizeI) * (m_sizeJ + 1);
        switch (which) {
        case FSO_G_MATERIAL: return n;
        case FSO_G_SOLID_SDF: case FSO_G_FLUID_SDF: case FSO_G_VISCOSITY:
        case FSO_G_DENSITY: case FSO_G_DIV_CONTROL: return n * 4;
        case FSO_G_U: case FSO_G_SAVED_U: return nu * 4;
        case FSO_G_V: case FSO_G_SAVED_V: return nv * 4;
        case FSO_G_U_VALID: return nu;
        case FSO_G_V_VALID: return nv;
        case FSO_G_KNOWN_CENTERED: return n;
        case FSO_G_PARTICLE_COUNTS: case FSO_G_SOLID_ID: case FSO_G_EMITTER_ID: return n * 4;
        case FSO_G_DENSITY_RHS: case FSO_G_DENSITY_PRESSURE: case FSO_G_PRESSURE:
        case FSO_G_PRESSURE_RHS: return n * 8;
        case FSO_G_ADVECTED_U: return kNb ? nu * 4 : 0;
        case FSO_G_ADVECTED_V: return kNb ? nv * 4 : 0;
        case FSO_G_ADVECTED_SDF: case FSO_G_ADVECTED_VISCOSITY: return kNb ? n * 4 : 0;
        default: return 0;
        }
    }

    template <class T> static void getVec(const std::vector<T> &v, void *out, size_t bytes)
    {
        if (v.size() * sizeof(T) == bytes) std::memcpy(out, v.data(), bytes);
        else std::memset(out, 0, bytes);
    }
    template <class T> static void setVec(std::vector<T> &v, const void *in, size_t bytes)
    {
        v.resize(bytes / sizeof(T));
        std::memcpy(v.data(), in, bytes);
    }
    static void getBool(const std::vector<bool> &v, void *out)
    {
        uint8_t *o = static_cast<uint8_t *>(out);
        for (size_t i = 0; i < v.size(); i++) o[i] = v[i] ? 1 : 0;
    }
    static void setBool(std::vector<bool> &v, const void *in)
    {
        const uint8_t *p = static_cast<const uint8_t *>(in);
        for (size_t i = 0; i < v.size(); i++) v[i] = p[i] != 0;
    }

    int getGrid(int which, void *out) override
    {
        const size_t bytes = gridBytes(which);
        switch (which) {
        case FSO_G_MATERIAL: getVec(m_materialGrid.data(), out, bytes); break;
        case FSO_G_SOLID_SDF: getVec(m_solidSdf.data(), out, bytes); break;
        case FSO_G_FLUID_SDF: getVec(m_fluidSdf.data(), out, bytes); break;
        case FSO_G_U: getVec(m_fluidVelocityGrid.velocityGridU().data(), out, bytes); break;
        case FSO_G_V: getVec(m_fluidVelocityGrid.velocityGridV().data(), out, bytes); break;
        case FSO_G_U_VALID: getBool(m_fluidVelocityGrid.uSampleValidityGrid().data(), out); break;
        case FSO_G_V_VALID: getBool(m_fluidVelocityGrid.vSampleValidityGrid().data(), out); break;
        case FSO_G_SAVED_U: getVec(m_savedFluidVelocityGrid.velocityGridU().data(), out, bytes); break;
        case FSO_G_SAVED_V: getVec(m_savedFluidVelocityGrid.velocityGridV().data(), out, bytes); break;
        case FSO_G_VISCOSITY: getVec(m_viscosityGrid.data(), out, bytes); break;
        case FSO_G_KNOWN_CENTERED: getBool(m_knownCenteredParams.data(), out); break;
        case FSO_G_DENSITY: getVec(m_densityGrid.data(), out, bytes); break;
        case FSO_G_PARTICLE_COUNTS: getVec(m_fluidParticleCounts.data(), out, bytes); break;
        case FSO_G_SOLID_ID: getVec(m_solidId.data(), out, bytes); break;
        case FSO_G_DIV_CONTROL: getVec(m_divergenceControl.data(), out, bytes); break;
        case FSO_G_DENSITY_RHS: getVec(m_pressureRhs, out, bytes); break;
        case FSO_G_DENSITY_PRESSURE: getVec(m_pressureSolverResult, out, bytes); break;
        case FSO_G_PRESSURE: getVec(capPressure, out, bytes); break;
        case FSO_G_PRESSURE_RHS: getVec(capRhs, out, bytes); break;
        case FSO_G_EMITTER_ID: getVec(m_emitterId.data(), out, bytes); break;
        case FSO_G_ADVECTED_U: case FSO_G_ADVECTED_V: case FSO_G_ADVECTED_SDF:
        case FSO_G_ADVECTED_VISCOSITY:
            if constexpr (kNb) {
                getVec(nbGrid(which), out, bytes);
                break;
            }
            return -1;
        default: return -1;
        }
        return 0;
    }

    int setGrid(int which, const void *in) override
    {
        const size_t bytes = gridBytes(which);
        switch (which) {
        case FSO_G_MATERIAL: std::memcpy(m_materialGrid.data().data(), in, bytes); break;
        case FSO_G_SOLID_SDF: std::memcpy(m_solidSdf.data().data(), in, bytes); break;
        case FSO_G_FLUID_SDF: std::memcpy(m_fluidSdf.data().data(), in, bytes); break;
        case FSO_G_U: std::memcpy(m_fluidVelocityGrid.velocityGridU().data().data(), in, bytes); break;
        case FSO_G_V: std::memcpy(m_fluidVelocityGrid.velocityGridV().data().data(), in, bytes); break;
        case FSO_G_U_VALID: setBool(m_fluidVelocityGrid.uSampleValidityGrid().data(), in); break;
        case FSO_G_V_VALID: setBool(m_fluidVelocityGrid.vSampleValidityGrid().data(), in); break;
        case FSO_G_SAVED_U: std::memcpy(m_savedFluidVelocityGrid.velocityGridU().data().data(), in, bytes); break;
        case FSO_G_SAVED_V: std::memcpy(m_savedFluidVelocityGrid.velocityGridV().data().data(), in, bytes); break;
        case FSO_G_VISCOSITY: std::memcpy(m_viscosityGrid.data().data(), in, bytes); break;
        case FSO_G_KNOWN_CENTERED: setBool(m_knownCenteredParams.data(), in); break;
        case FSO_G_DENSITY: std::memcpy(m_densityGrid.data().data(), in, bytes); break;
        case FSO_G_PARTICLE_COUNTS: std::memcpy(m_fluidParticleCounts.data().data(), in, bytes); break;
        case FSO_G_SOLID_ID: std::memcpy(m_solidId.data().data(), in, bytes); break;
        case FSO_G_DIV_CONTROL: std::memcpy(m_divergenceControl.data().data(), in, bytes); break;
        case FSO_G_DENSITY_RHS: setVec(m_pressureRhs, in, bytes); break;
        case FSO_G_DENSITY_PRESSURE: setVec(m_pressureSolverResult, in, bytes); break;
        case FSO_G_PRESSURE: setVec(capPressure, in, bytes); break;
        case FSO_G_PRESSURE_RHS: setVec(capRhs, in, bytes); break;
        case FSO_G_EMITTER_ID: std::memcpy(m_emitterId.data().data(), in, bytes); break;
        case FSO_G_ADVECTED_U: case FSO_G_ADVECTED_V: case FSO_G_ADVECTED_SDF:
        case FSO_G_ADVECTED_VISCOSITY:
            if constexpr (kNb) {
                std::memcpy(nbGrid(which).data(), in, bytes);
                break;
            }
            return -1;
        default: return -1;
        }
        return 0;
    }

    size_t binCount() override { return m_markerParticles.bins().linearSize(); }

    void getParticles(int32_t *counts, float *pos, float *vel, float *visc, uint8_t *dead) override
    {
        auto &bins = m_markerParticles.bins().data();
        size_t k = 0;
        for (size_t b = 0; b < bins.size(); b++) {
            ParticleBin &bin = bins[b];
            counts[b] = static_cast<int32_t>(bin.size());
            auto &vv = bin.particleProperties<float>(m_viscosityPropertyIndex);
            for (size_t p = 0; p < bin.size(); p++, k++) {
                pos[2 * k] = bin.particlePosition(p).x();
                pos[2 * k + 1] = bin.particlePosition(p).y();
                vel[2 * k] = bin.particleVelocity(p).x();
                vel[2 * k + 1] = bin.particleVelocity(p).y();
                visc[k] = vv[p];
                dead[k] = bin.markedForDeath(p) ? 1 : 0;
            }
        }
    }

    void setParticles(const int32_t *counts, const float *pos, const float *vel,
                      const float *visc, const uint8_t *dead) override
    {
        auto &bins = m_markerParticles.bins().data();
        size_t k = 0;
        for (size_t b = 0; b < bins.size(); b++) {
            ParticleBin &bin = bins[b];
            bin.clear();
            for (int32_t p = 0; p < counts[b]; p++, k++) {
                size_t idx = bin.addMarkerParticle(Vec3(pos[2 * k], pos[2 * k + 1]),
                                                   Vec3(vel[2 * k], vel[2 * k + 1]));
                bin.particleProperties<float>(m_viscosityPropertyIndex)[idx] = visc[k];
                if (dead[k]) bin.markForDeath(idx);
            }
        }
    }

    // the advected grids of NB-FLIP (nbflipsolver.h:63-66)
    std::vector<float> &nbGrid(int which)
    {
        if constexpr (kNb) {
            switch (which) {
            case FSO_G_ADVECTED_U: return this->m_advectedVelocity.velocityGridU().data();
            case FSO_G_ADVECTED_V: return this->m_advectedVelocity.velocityGridV().data();
            case FSO_G_ADVECTED_SDF: return this->m_advectedSdf.data();
            default: return this->m_advectedViscosity.data();
            }
        }
        static std::vector<float> none;
        return none;
    }

    // LinearSolver::solve on the system built from the current material grid.
    int pcgSolve(const double *rhs, double *result, int iterLimit, double tol)
    {
        m_pressureMatrix = getPressureProjectionMatrix();
        m_pressurePrecond = getIPPCoefficients(m_pressureMatrix);
        std::vector<double> b(rhs, rhs + cellCount());
        std::vector<double> x(cellCount(), 0.0);
        int iters = m_pressureSolver.solve(m_pressureMatrix, m_pressurePrecond, x, b,
                                           iterLimit, tol);
        std::memcpy(result, x.data(), x.size() * sizeof(double));
        return iters;
    }
};

FlipSolverParameters toRef(const fso_params *p)
{
    FlipSolverParameters r{};
    r.fluidDensity = p->fluidDensity;
    r.seed = p->seed;
    r.dx = p->dx;
    r.particlesPerCell = p->particlesPerCell;
    r.globalAcceleration = Vec3(p->globalAccelerationI, p->globalAccelerationJ);
    r.resolution = p->resolution;
    r.fps = p->fps;
    r.maxSubsteps = p->maxSubsteps;
    r.picRatio = p->picRatio;
    r.cflNumber = p->cflNumber;
    r.particleScale = p->particleScale;
    r.pcgIterLimit = p->pcgIterLimit;
    r.domainSizeI = p->domainSizeI;
    r.domainSizeJ = p->domainSizeJ;
    r.gridSizeI = p->gridSizeI;
    r.gridSizeJ = p->gridSizeJ;
    r.sceneScale = p->sceneScale;
    r.viscosityEnabled = p->viscosityEnabled != 0;
    r.useHeavyViscosity = p->useHeavyViscosity != 0;
    r.simulationMethod = static_cast<SimulationMethod>(p->simulationMethod);
    r.parameterHandlingMethod = static_cast<ParameterHandlingMethod>(p->parameterHandlingMethod);
    return r;
}

Geometry2d polygon(const float *xy, int n)
{
    Geometry2d g;
    for (int i = 0; i < n; i++) g.addVertex(Vec3(xy[2 * i], xy[2 * i + 1]));
    return g;
}

using RefSolver = RefSolverT<FlipSolver>;
using RefNBSolver = RefSolverT<NBFlipSolver>;

RefApi *S(fso_solver *s) { return reinterpret_cast<RefApi *>(s); }

} // namespace

extern "C" {

fso_solver *fso_create(const fso_params *p)
{
    FlipSolverParameters r = toRef(p);
    RefSolver *s = new RefSolver(&r);
    // JsonSceneReader::loadJson calls this right after construction
    // (jsonscenereader.cpp:64); it registers the viscosity particle property.
    s->initAdditionalParameters();
    return reinterpret_cast<fso_solver *>(static_cast<RefApi *>(s));
}

fso_solver *fso_create_nbflip(const fso_params *p)
{
    FlipSolverParameters r = toRef(p);
    NBFlipParameters nr;
    static_cast<FlipSolverParameters &>(nr) = r;
    RefNBSolver *s = new RefNBSolver(&nr);
    s->initAdditionalParameters();
    return reinterpret_cast<fso_solver *>(static_cast<RefApi *>(s));
}

void fso_destroy(fso_solver *s) { delete S(s); }

int fso_get_rng(fso_solver *s, uint32_t state[625]) { return S(s)->getRng(state); }
int fso_set_rng(fso_solver *s, const uint32_t state[625]) { return S(s)->setRng(state); }

int fso_add_geometry(fso_solver *s, float friction, const float *xy, int n)
{
    Geometry2d g = polygon(xy, n);
    Obstacle o(friction, g);
    S(s)->addGeom(o);
    return 0;
}

int fso_add_initial_fluid(fso_solver *s, float viscosity, const float *xy, int n)
{
    Geometry2d g = polygon(xy, n);
    Emitter e(g);
    e.setViscosity(viscosity);
    e.setTemperature(273.f);
    e.setConcentrartion(1.f);
    e.setFuel(1.f);
    e.setDivergence(0.f);
    e.setVelocity(Vec3());
    e.setVelocityTransfer(false);
    S(s)->addFluid(e);
    return 0;
}

int fso_add_source(fso_solver *s, const float *xy, int n, float viscosity, float divergence,
                   float vx, float vy, int velocity_transfer)
{
    // JsonSceneReader::emitterFromJson (jsonscenereader.cpp:200-225) with its
    // defaults for the parameters the liquid solvers do not read
    Geometry2d g = polygon(xy, n);
    Emitter e(g);
    e.setTemperature(273.f);
    e.setConcentrartion(1.f);
    e.setViscosity(viscosity);
    e.setFuel(1.f);
    e.setDivergence(divergence);
    e.setVelocity(Vec3(vx, vy));
    e.setVelocityTransfer(velocity_transfer != 0);
    S(s)->addSrc(e);
    return 0;
}

int fso_add_sink(fso_solver *s, float divergence, const float *xy, int n)
{
    Geometry2d g = polygon(xy, n);
    Sink k(divergence, g);
    S(s)->addSinkObj(k);
    return 0;
}

void fso_first_frame_init(fso_solver *s) { S(s)->firstInit(); }
void fso_step_frame(fso_solver *s) { S(s)->frame(); }
void fso_set_step_dt(fso_solver *s, float dt) { S(s)->setStepDt(dt); }
float fso_step_dt(fso_solver *s) { return S(s)->getStepDt(); }
void fso_step(fso_solver *s) { S(s)->stepOnce(); }
float fso_max_particle_velocity(fso_solver *s) { return S(s)->maxVel(); }

int fso_run_stage(fso_solver *s, int stage)
{
    if (stage < 0 || stage >= FSO_STAGE_COUNT) return -1;
    S(s)->runStage(stage);
    return 0;
}

size_t fso_bin_count(fso_solver *s) { return S(s)->binCount(); }
size_t fso_particle_count(fso_solver *s) { return S(s)->nParticles(); }

void fso_get_particles(fso_solver *s, int32_t *counts, float *pos, float *vel, float *visc,
                       uint8_t *dead)
{
    S(s)->getParticles(counts, pos, vel, visc, dead);
}

void fso_set_particles(fso_solver *s, const int32_t *counts, const float *pos,
                       const float *vel, const float *visc, const uint8_t *dead)
{
    S(s)->setParticles(counts, pos, vel, visc, dead);
}

size_t fso_grid_bytes(fso_solver *s, int which) { return S(s)->gridBytes(which); }
int fso_get_grid(fso_solver *s, int which, void *out) { return S(s)->getGrid(which, out); }
int fso_set_grid(fso_solver *s, int which, const void *in) { return S(s)->setGrid(which, in); }

int fso_stat(fso_solver *s, int which) { return S(s)->stat(which); }

int fso_pcg_solve(int ni, int nj, const int8_t *material, float dt, double density,
                  double dx, const double *rhs, double *result, int iter_limit, double tol)
{
    fso_params p{};
    p.fluidDensity = density;
    p.dx = dx;
    p.particlesPerCell = 4;
    p.fps = 30;
    p.maxSubsteps = 1;
    p.pcgIterLimit = iter_limit;
    p.gridSizeI = ni;
    p.gridSizeJ = nj;
    FlipSolverParameters r = toRef(&p);
    RefSolver solver(&r);
    solver.setGrid(FSO_G_MATERIAL, material);
    solver.setStepDt(dt);
    return solver.pcgSolve(rhs, result, iter_limit, tol);
}

} // extern "C"
