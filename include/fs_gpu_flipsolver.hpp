/*
 * fs_gpu_flipsolver.hpp -- C++ drop-ins for FlipSolver2d's hot path, built on
 * the C ABI of fs_gpu.h (libfsgpu.so).  Header-only; it is compiled inside the
 * reference project against its own headers (FlipSolver2dLib/), so it names
 * the reference's types directly.
 *
 *   fsgpu::GpuLinearSolver   LinearSolver (linearsolver.h:10-23): the same
 *                            solve() signature, arguments and return value,
 *                            run by fs_pcg_solve_operator on the GPU.
 *   fsgpu::GpuStepSolver     a FlipSolver (flipsolver2d.h:183-432) whose
 *                            protected virtual step() (flipsolver2d.cpp:412-462)
 *                            runs on the GPU through fs_step.  Everything else
 *                            -- construction, addGeometry/addInitialFluid/...,
 *                            stepFrame's CFL loop, the accessors -- is the
 *                            reference's own code, and the solver's state is
 *                            the reference's own members, copied to the
 *                            device before each substep and back after it.
 *
 * Errors: the reference's hot path has no error channel besides the solve's
 * return value; a failing GPU call here throws fsgpu::Error with the
 * library's message.  There is no CPU fallback.
 */
#ifndef FS_GPU_FLIPSOLVER_HPP
#define FS_GPU_FLIPSOLVER_HPP

#include <cmath>
#include <cstdint>
#include <cstring>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "flipsolver2d.h"
#include "linearsolver.h"

#include "fs_gpu.h"

namespace fsgpu {

class Error : public std::runtime_error {
public:
    Error(fs_status s, const std::string &where)
        : std::runtime_error(where + ": " + fs_status_string(s) + ": " + fs_last_error()), status(s)
    {
    }
    fs_status status;
};

inline void check(fs_status s, const char *where)
{
    if (s != FS_OK) throw Error(s, where);
}

namespace detail {

// The operator's grid indexer and scale are protected members of
// IndexedPressureParameters (pressuredata.h:239-242), the IPP units a
// protected member of IndexedIPPCoefficients (PressureIPPCoeficients.h:
// 136-138).  A pointer to a protected member, formed inside a derived class,
// reads them from any object of the base class.
struct PressureParametersView : IndexedPressureParameters {
    static const LinearIndexable2d &indexer(const IndexedPressureParameters &p)
    {
        return p.*(&PressureParametersView::m_indexer);
    }
    static double scale(const IndexedPressureParameters &p) { return p.*(&PressureParametersView::m_scale); }
};
struct IppCoefficientsView : IndexedIPPCoefficients {
    static const std::vector<IndexedIPPCoefficientUnit> &units(const IndexedIPPCoefficients &c)
    {
        return c.*(&IppCoefficientsView::m_data);
    }
};

} // namespace detail

/* The operator byte of fs_pcg_solve_operator for every cell, from the
 * reference's operator rows and IPP coefficients:
 *  - a unit row (IndexedPressureParameterUnit) sets bit 7, its
 *    nonsolidNeighborCount in bits 4-6 and its fluidNeighborMask in bits 0-3;
 *  - the IPP coefficient toward a neighbour n is 1 / (count(n) * scale)
 *    (getIPPCoefficients, flipsolver2d.cpp:924-927), so each coefficient also
 *    gives that neighbour's count: round(1 / (coefficient * scale)), and 0
 *    where the coefficient is infinite (a count of zero).
 * Neighbours are the reference's linear-index offsets (linearIdxOfOffset,
 * linearindexable2d.h:103-106); those outside [0, N) carry no byte. */
inline std::vector<uint8_t> operator_bytes(const IndexedPressureParameters &matrix,
                                           const IndexedIPPCoefficients &precond, double scale,
                                           ssize_t ni, ssize_t nj)
{
    const ssize_t n = ni * nj;
    std::vector<uint8_t> info((size_t)n, 0);
    for (const IndexedPressureParameterUnit &u : matrix.data()) {
        if ((ssize_t)u.unitIndex >= n) continue;
        info[u.unitIndex] = (uint8_t)(0x80 | ((u.nonsolidNeighborCount & 7) << 4) | (u.fluidNeighborMask & 0x0f));
    }
    for (const IndexedIPPCoefficientUnit &u : detail::IppCoefficientsView::units(precond)) {
        const ssize_t c = (ssize_t)u.unitIndex;
        const ssize_t nb[4] = {c - nj, c + nj, c - 1, c + 1};
        const double coef[4] = {u.iNeg, u.iPos, u.jNeg, u.jPos};
        for (int d = 0; d < 4; d++) {
            if (nb[d] < 0 || nb[d] >= n) continue;
            long cnt = 0;
            if (std::isfinite(coef[d]) && coef[d] > 0.0) cnt = std::lround(1.0 / (coef[d] * scale));
            if (cnt < 0) cnt = 0;
            if (cnt > 4) cnt = 4;
            uint8_t &b = info[(size_t)nb[d]];
            b = (uint8_t)((b & 0x8f) | (cnt << 4));
        }
    }
    return info;
}

/* LinearSolver on the GPU.  solve() keeps LinearSolver::solve's signature
 * (linearsolver.h:15-20) and meaning: result is resized to rhs and
 * overwritten, the return value is the loop index at convergence, iterLimit
 * on failure, 0 for a zero right-hand side.  precision FS_PCG_FP64 (the
 * default) is the reference's arithmetic with the dot products summed in
 * another order; FS_PCG_FP32 is the production mode.  pool_threads sets the
 * chunk count of the reference's max-abs stopping test (0: this host's
 * std::thread::hardware_concurrency(), as the reference's ThreadPool). */
class GpuLinearSolver {
public:
    explicit GpuLinearSolver(int precision = FS_PCG_FP64, int pool_threads = 0, int device = 0)
    {
        std::memset(&m_exec, 0, sizeof(m_exec));
        m_exec.pcg_precision = precision;
        m_exec.pool_threads = pool_threads;
        m_exec.device = device;
    }

    int solve(const IndexedPressureParameters &matrixIn, const IndexedIPPCoefficients &precond,
              std::vector<double> &result, const std::vector<double> &vec, int iterLimit = 20,
              double tol = 1e-6)
    {
        const LinearIndexable2d &ix = detail::PressureParametersView::indexer(matrixIn);
        const double scale = detail::PressureParametersView::scale(matrixIn);
        const ssize_t ni = ix.sizeI(), nj = ix.sizeJ();
        if ((ssize_t)vec.size() != ni * nj)
            throw Error(FS_ERR_BAD_ARG, "GpuLinearSolver::solve: right-hand side size");
        const std::vector<uint8_t> info = operator_bytes(matrixIn, precond, scale, ni, nj);
        result.assign(vec.size(), 0.0);
        int iterations = 0;
        check(fs_pcg_solve_operator((int)ni, (int)nj, info.data(), scale, vec.data(), result.data(),
                                    iterLimit, tol, &m_exec, &iterations),
              "fs_pcg_solve_operator");
        return iterations;
    }

private:
    fs_exec_params m_exec;
};

/* A FlipSolver whose substep runs on the GPU.  Construct it like the
 * reference's FlipSolver (FlipSolver(const FlipSolverParameters*)), add
 * geometry, sources, sinks and initial fluid with the reference's own calls,
 * and drive it with stepFrame().  The GPU handle is created at the first
 * substep, from the solver's parameters and objects; each substep then
 * uploads the particles and the state grids, runs fs_step with m_stepDt and
 * writes the results back into the reference's members, so every accessor
 * (markerParticles(), materialGrid(), fluidVelocityGrid(), ...) reads the
 * GPU's results.  With viscosityEnabled the substep applies the light or
 * heavy viscosity model on the GPU and projects again, like FlipSolver::step
 * (flipsolver2d.cpp:448-454). */
class GpuStepSolver : public FlipSolver {
public:
    explicit GpuStepSolver(const FlipSolverParameters *p, int precision = FS_PCG_FP32,
                           int pool_threads = 0, int device = 0)
        : FlipSolver(p), m_heavyViscosity(p->useHeavyViscosity)
    {
        std::memset(&m_exec, 0, sizeof(m_exec));
        m_exec.pcg_precision = precision;
        m_exec.pool_threads = pool_threads;
        m_exec.device = device;
    }

    ~GpuStepSolver() override
    {
        if (m_handle) fs_destroy(m_handle);
    }

    GpuStepSolver(const GpuStepSolver &) = delete;
    GpuStepSolver &operator=(const GpuStepSolver &) = delete;

    fs_solver *handle() const { return m_handle; }

protected:
    void step() override
    {
        ensureHandle();
        upload();
        check(fs_set_step_dt(m_handle, m_stepDt), "fs_set_step_dt");
        check(fs_step(m_handle), "fs_step");
        download();
    }

private:
    // FlipSolverParameters as the solver holds them (flipsolver2d.cpp:27-86)
    fs_params params()
    {
        fs_params q;
        std::memset(&q, 0, sizeof(q));
        q.fluidDensity = m_fluidDensity;
        q.seed = m_seed;
        q.dx = m_dx;
        q.particlesPerCell = m_particlesPerCell;
        q.globalAccelerationI = m_globalAcceleration.x();
        q.globalAccelerationJ = m_globalAcceleration.y();
        q.resolution = m_resolution;
        q.fps = m_fps;
        q.maxSubsteps = m_maxSubsteps;
        q.picRatio = m_picRatio;
        q.cflNumber = m_cflNumber;
        q.particleScale = m_particleScale;
        q.pcgIterLimit = m_pcgIterLimit;
        q.domainSizeI = m_domainSizeI;
        q.domainSizeJ = m_domainSizeJ;
        q.gridSizeI = (int)m_sizeI;
        q.gridSizeJ = (int)m_sizeJ;
        q.sceneScale = m_sceneScale;
        q.viscosityEnabled = m_viscosityEnabled ? 1 : 0;
        // FlipSolver keeps only the model it built from this flag (:77-84)
        q.useHeavyViscosity = m_heavyViscosity ? 1 : 0;
        q.simulationMethod = (int)m_simulationMethod;
        q.parameterHandlingMethod = (int)m_parameterHandlingMethod;
        return q;
    }

    static std::vector<float> flat(Geometry2d &g)
    {
        std::vector<float> xy;
        for (const Vec3 &v : g.verts()) {
            xy.push_back(v.x());
            xy.push_back(v.y());
        }
        return xy;
    }

    // the handle mirrors the solver's objects; its first-frame set-up gives
    // it the solid data (distance field, ids, friction factors), and the
    // fluid state is replaced by the solver's own before every substep
    void ensureHandle()
    {
        if (m_handle) return;
        const fs_params q = params();
        check(fs_create(&q, &m_exec, &m_handle), "fs_create");
        for (Obstacle &o : m_obstacles) {
            std::vector<float> xy = flat(o.geometry());
            check(fs_add_geometry(m_handle, o.friction(), xy.data(), (int)(xy.size() / 2)), "fs_add_geometry");
        }
        for (Sink &k : m_sinks) {
            std::vector<float> xy = flat(k.geo());
            check(fs_add_sink(m_handle, k.divergence(), xy.data(), (int)(xy.size() / 2)), "fs_add_sink");
        }
        for (Emitter &e : m_sources) {
            std::vector<float> xy = flat(e.geometry());
            const Vec3 v = e.velocity();
            check(fs_add_source(m_handle, xy.data(), (int)(xy.size() / 2), e.viscosity(), e.divergence(),
                                v.x(), v.y(), e.velocityTransfer() ? 1 : 0),
                  "fs_add_source");
        }
        for (Emitter &e : m_initialFluid) {
            std::vector<float> xy = flat(e.geometry());
            check(fs_add_initial_fluid(m_handle, e.viscosity(), xy.data(), (int)(xy.size() / 2)),
                  "fs_add_initial_fluid");
        }
        check(fs_first_frame_init(m_handle), "fs_first_frame_init");
    }

    template <typename T> void putGrid(int which, const std::vector<T> &v)
    {
        check(fs_set_grid(m_handle, which, v.data(), v.size() * sizeof(T)), "fs_set_grid");
    }
    template <typename T> void getGrid(int which, std::vector<T> &v)
    {
        check(fs_get_grid(m_handle, which, v.data(), v.size() * sizeof(T)), "fs_get_grid");
    }
    // Grid2d<bool> is a std::vector<bool>: one byte per cell on the wire
    void putBools(int which, const std::vector<bool> &v)
    {
        std::vector<uint8_t> b(v.size());
        for (size_t k = 0; k < v.size(); k++) b[k] = v[k] ? 1 : 0;
        putGrid(which, b);
    }
    void getBools(int which, std::vector<bool> &v)
    {
        std::vector<uint8_t> b(v.size());
        getGrid(which, b);
        for (size_t k = 0; k < v.size(); k++) v[k] = b[k] != 0;
    }
    // libstdc++ writes a std::mt19937 as its 624 state words, then the index
    // of the next one: the layout of fs_set_rng_state
    void putRng()
    {
        std::stringstream ss;
        ss << m_randEngine;
        uint32_t st[625];
        for (int k = 0; k < 625; k++) ss >> st[k];
        check(fs_set_rng_state(m_handle, st), "fs_set_rng_state");
    }
    void getRng()
    {
        uint32_t st[625];
        check(fs_get_rng_state(m_handle, st), "fs_get_rng_state");
        std::stringstream ss;
        for (int k = 0; k < 625; k++) ss << st[k] << ' ';
        ss >> m_randEngine;
    }

    void upload()
    {
        // particles bin by bin in storage order, as ParticleBin keeps them
        auto &bins = m_markerParticles.bins().data();
        std::vector<int32_t> counts(bins.size());
        std::vector<float> pos, vel, visc;
        std::vector<uint8_t> dead;
        for (size_t b = 0; b < bins.size(); b++) {
            ParticleBin &bin = bins[b];
            counts[b] = (int32_t)bin.size();
            const std::vector<float> &vv = bin.particleProperties<float>(m_viscosityPropertyIndex);
            for (size_t k = 0; k < bin.size(); k++) {
                pos.push_back(bin.particlePosition(k).x());
                pos.push_back(bin.particlePosition(k).y());
                vel.push_back(bin.particleVelocity(k).x());
                vel.push_back(bin.particleVelocity(k).y());
                visc.push_back(vv[k]);
                dead.push_back(bin.markedForDeath(k) ? 1 : 0);
            }
        }
        check(fs_set_particles(m_handle, counts.data(), pos.data(), vel.data(), visc.data(), dead.data()),
              "fs_set_particles");
        putGrid(FS_GRID_MATERIAL, m_materialGrid.data());
        putGrid(FS_GRID_FLUID_SDF, m_fluidSdf.data());
        putGrid(FS_GRID_U, m_fluidVelocityGrid.velocityGridU().data());
        putGrid(FS_GRID_V, m_fluidVelocityGrid.velocityGridV().data());
        putBools(FS_GRID_U_VALID, m_fluidVelocityGrid.uSampleValidityGrid().data());
        putBools(FS_GRID_V_VALID, m_fluidVelocityGrid.vSampleValidityGrid().data());
        putGrid(FS_GRID_SAVED_U, m_savedFluidVelocityGrid.velocityGridU().data());
        putGrid(FS_GRID_SAVED_V, m_savedFluidVelocityGrid.velocityGridV().data());
        putGrid(FS_GRID_VISCOSITY, m_viscosityGrid.data());
        putBools(FS_GRID_KNOWN_CENTERED, m_knownCenteredParams.data());
        putGrid(FS_GRID_DENSITY, m_densityGrid.data());
        putGrid(FS_GRID_PARTICLE_COUNTS, m_fluidParticleCounts.data());
        putGrid(FS_GRID_DIV_CONTROL, m_divergenceControl.data());
        putGrid(FS_GRID_EMITTER_ID, m_emitterId.data());
        putRng();
    }

    void download()
    {
        size_t nbins = 0, n = 0;
        check(fs_bin_count(m_handle, &nbins), "fs_bin_count");
        check(fs_particle_count(m_handle, &n), "fs_particle_count");
        std::vector<int32_t> counts(nbins);
        std::vector<float> pos(2 * n), vel(2 * n), visc(n);
        std::vector<uint8_t> dead(n);
        check(fs_get_particles(m_handle, counts.data(), pos.data(), vel.data(), visc.data(), dead.data()),
              "fs_get_particles");
        auto &bins = m_markerParticles.bins().data();
        size_t k = 0;
        for (size_t b = 0; b < bins.size() && b < nbins; b++) {
            ParticleBin &bin = bins[b];
            bin.clear();
            for (int32_t p = 0; p < counts[b]; p++, k++) {
                const size_t idx = bin.addMarkerParticle(Vec3(pos[2 * k], pos[2 * k + 1]),
                                                         Vec3(vel[2 * k], vel[2 * k + 1]));
                bin.particleProperties<float>(m_viscosityPropertyIndex)[idx] = visc[k];
                if (dead[k]) bin.markForDeath(idx);
            }
        }
        getGrid(FS_GRID_MATERIAL, m_materialGrid.data());
        getGrid(FS_GRID_FLUID_SDF, m_fluidSdf.data());
        getGrid(FS_GRID_U, m_fluidVelocityGrid.velocityGridU().data());
        getGrid(FS_GRID_V, m_fluidVelocityGrid.velocityGridV().data());
        getBools(FS_GRID_U_VALID, m_fluidVelocityGrid.uSampleValidityGrid().data());
        getBools(FS_GRID_V_VALID, m_fluidVelocityGrid.vSampleValidityGrid().data());
        getGrid(FS_GRID_SAVED_U, m_savedFluidVelocityGrid.velocityGridU().data());
        getGrid(FS_GRID_SAVED_V, m_savedFluidVelocityGrid.velocityGridV().data());
        getGrid(FS_GRID_VISCOSITY, m_viscosityGrid.data());
        getBools(FS_GRID_KNOWN_CENTERED, m_knownCenteredParams.data());
        getGrid(FS_GRID_DENSITY, m_densityGrid.data());
        getGrid(FS_GRID_PARTICLE_COUNTS, m_fluidParticleCounts.data());
        getGrid(FS_GRID_DIV_CONTROL, m_divergenceControl.data());
        getGrid(FS_GRID_EMITTER_ID, m_emitterId.data());
        m_pressureRhs.resize(cellCount());
        m_pressureSolverResult.resize(cellCount());
        getGrid(FS_GRID_DENSITY_RHS, m_pressureRhs);
        getGrid(FS_GRID_DENSITY_PRESSURE, m_pressureSolverResult);
        getRng();
        int it = 0;
        check(fs_get_stat(m_handle, FS_STAT_DENSITY_ITERS, &it), "fs_get_stat");
        m_stats.setDensityIters(it);
        check(fs_get_stat(m_handle, FS_STAT_PRESSURE_ITERS, &it), "fs_get_stat");
        m_stats.setPressureIterations(it);
        if (m_viscosityEnabled) {
            check(fs_get_stat(m_handle, FS_STAT_VISCOSITY_ITERS, &it), "fs_get_stat");
            m_stats.setViscosityIterations(it);
        }
    }

    fs_exec_params m_exec;
    fs_solver *m_handle = nullptr;
    bool m_heavyViscosity;
};

} // namespace fsgpu

#endif // FS_GPU_FLIPSOLVER_HPP
