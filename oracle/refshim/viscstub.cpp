// Stand-in for the reference's viscositymodel.cpp, which needs the real Eigen
// sparse solvers (absent here).  Viscosity is disabled in every scene the
// oracle runs (FlipSolverParameters::viscosityEnabled = false), so
// FlipSolver::applyViscosity (flipsolver2d.cpp:128-136) is never reached; the
// two virtual overrides only have to exist for the vtables to link.
// Test infrastructure: compiled only into the reference oracle.
#include "viscositymodel.h"

int LightViscosityModel::apply(StaggeredVelocityGrid &, const Grid2d<float> &,
                               const MaterialGrid &, float, float, float)
{
    return 0;
}

int HeavyViscosityModel::apply(StaggeredVelocityGrid &, const Grid2d<float> &,
                               const MaterialGrid &, float, float, float)
{
    return 0;
}
