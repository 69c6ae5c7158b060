// Compile-and-link check of include/fs_gpu_flipsolver.hpp against the
// reference's own headers and objects (test infrastructure; built and run by
// tests/test_dropin_cpp.py).  It
//  1. builds a small dam break through the reference's API, freezes its
//     pressure operator and IPP coefficients as FlipSolver::step does
//     (getPressureProjectionMatrix / getIPPCoefficients), and prints the
//     material grid and fsgpu::operator_bytes of them, one line each;
//  2. constructs an fsgpu::GpuStepSolver and an fsgpu::GpuLinearSolver and
//     calls each once: on a machine without a CUDA device both must throw
//     fsgpu::Error (no CPU fallback), which it reports; with a device it
//     reports the solve's iteration count.
#include <cstdio>
#include <vector>

#include "fs_gpu_flipsolver.hpp"

namespace {

FlipSolverParameters dam_parameters(int n)
{
    FlipSolverParameters p{};
    p.fluidDensity = 1000.0;
    p.seed = 42;
    p.dx = 1.0 / n;
    p.particlesPerCell = 4;
    p.globalAcceleration = Vec3(9.81f, 0.f);
    p.resolution = (float)n;
    p.fps = 30;
    p.maxSubsteps = 10;
    p.picRatio = 0.03f;
    p.cflNumber = 5.f;
    p.particleScale = 0.8f;
    p.pcgIterLimit = 200;
    p.domainSizeI = 1.f;
    p.domainSizeJ = 1.f;
    p.gridSizeI = n;
    p.gridSizeJ = n;
    p.sceneScale = 1.f;
    p.viscosityEnabled = false;
    p.useHeavyViscosity = false;
    p.simulationMethod = static_cast<SimulationMethod>(0);
    p.parameterHandlingMethod = static_cast<ParameterHandlingMethod>(0);
    return p;
}

Geometry2d box(float i0, float j0, float i1, float j1)
{
    Geometry2d g;
    g.addVertex(Vec3(i0, j0));
    g.addVertex(Vec3(i1, j0));
    g.addVertex(Vec3(i1, j1));
    g.addVertex(Vec3(i0, j1));
    return g;
}

template <class S> void add_dam(S &s, int n)
{
    const float dx = 1.f / n;
    Geometry2d walls[4] = {box(0, 0, dx, 1), box(1 - dx, 0, 1, 1), box(0, 0, 1, dx), box(0, 1 - dx, 1, 1)};
    for (Geometry2d &g : walls) {
        Obstacle o(0.f, g);
        s.addGeometry(o);
    }
    Geometry2d fluid = box(0.4f, dx, 1 - dx, 0.4f);
    Emitter e(fluid);
    s.addInitialFluid(e);
}

// the reference solver with its operator frozen as step() freezes it
class Probe : public FlipSolver {
public:
    using FlipSolver::FlipSolver;
    void freeze(float dt)
    {
        firstFrameInit();
        m_stepDt = dt;
        IndexedPressureParameters m = getPressureProjectionMatrix();
        IndexedIPPCoefficients ipp = getIPPCoefficients(m);
        const double scale = m_stepDt / (m_fluidDensity * m_dx * m_dx);
        bytes = fsgpu::operator_bytes(m, ipp, scale, m_sizeI, m_sizeJ);
        material.assign(m_materialGrid.data().begin(), m_materialGrid.data().end());
    }
    std::vector<uint8_t> bytes;
    std::vector<int8_t> material;
};

} // namespace

int main()
{
    const int n = 24;
    FlipSolverParameters p = dam_parameters(n);
    Probe probe(&p);
    probe.initAdditionalParameters();
    add_dam(probe, n);
    probe.freeze(1.f / 60);
    std::printf("material");
    for (int8_t m : probe.material) std::printf(" %d", (int)m);
    std::printf("\noperator");
    for (uint8_t b : probe.bytes) std::printf(" %u", (unsigned)b);
    std::printf("\n");

    fsgpu::GpuStepSolver gpu(&p, FS_PCG_FP64, 8);
    gpu.initAdditionalParameters();
    add_dam(gpu, n);
    try {
        gpu.stepFrame();
        std::printf("step ok %zu\n", gpu.particleCount());
    } catch (const fsgpu::Error &e) {
        std::printf("step error %d %s\n", (int)e.status, e.what());
    }
    return 0;
}
