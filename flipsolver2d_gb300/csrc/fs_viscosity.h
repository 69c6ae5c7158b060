// fs_viscosity.h -- the viscosity models of FlipSolver::applyViscosity
// (flipsolver2d.cpp:128-136, viscositymodel.cpp) on the GPU.
//
// Both models assemble a sparse system with coeffRef and solve it with
// Eigen::ConjugateGradient<SparseMatrix<double>, Upper> and Eigen's diagonal
// preconditioner (viscositymodel.h:21, tolerance 1e-4, at most 2n
// iterations): the matrix acts as the self-adjoint matrix of its upper
// triangle.  On a structured grid that self-adjoint matrix is a fixed
// stencil, so it is stored here as per-unknown coefficients (structure of
// arrays), each the exact double the reference's assembly leaves in that
// upper-triangle entry, and applied in gather form:
//
//  light (N = NI NJ cells, one matrix solved for U and then for V):
//    coef[0] diagonal, coef[1] entry (k, k+1), coef[2] entry (k, k+NJ)
//  heavy (NU = (NI+1) NJ U faces, then NV = NI (NJ+1) V faces):
//    U face: diagonal, u(i+1,j), u(i,j+1), v(i,j), v(i-1,j), v(i,j+1),
//            v(i-1,j+1)  (7 arrays of NU)
//    V face: diagonal, v(i,j+1), v(i+1,j)  (3 arrays of NV, after the U ones)
//
// The conjugate gradient is Eigen's (x0 = 0, stop when ||r||^2 <
// max(tol^2 ||b||^2, DBL_MIN) or after 2n iterations, Success when
// sqrt(||r||^2 / ||b||^2) <= tol) with every dot product summed over a fixed
// block partition in a fixed order: run to run the solve gives the same bits.
#pragma once

#include <cuda_runtime.h>

#include "fs_state.h"

namespace fsg {

constexpr int kViscThreads = 256;
constexpr int kViscBlocksMax = 1216; // block partials of one dot product at most
constexpr int kViscBatch = 32;       // iterations enqueued between convergence reads
constexpr double kViscTol = 1e-4;    // viscositymodel.cpp: setTolerance(1e-4)

// the solve's state on the device; abs_new is indexed by iteration parity so
// that the kernel writing the next value never overwrites the one its other
// blocks still read
struct ViscCtl {
    double rhs_norm2;  // ||b||^2
    double threshold;  // max(tol^2 ||b||^2, DBL_MIN)
    double abs_new[2]; // r.z of iterations it (it & 1) and it + 1
    double res_norm2;  // ||r||^2 where the solve stopped
    int iters;         // completed iterations where it stopped
    int done;          // 1 once stopped
};

struct ViscBuffers {
    long long n = 0;     // unknowns
    long long ncoef = 0; // coefficient doubles
    double *b = nullptr, *x = nullptr, *r = nullptr, *p = nullptr, *t = nullptr;
    double *invdiag = nullptr; // 1 / diagonal, 1 where the diagonal is 0
    double *coef = nullptr;
    double *part = nullptr;    // 2 * kViscBlocksMax block partials
    ViscCtl *ctl = nullptr;    // device
    ViscCtl *ctl_host = nullptr; // pinned mirror
};

// sizes of the buffers for a model on a grid
long long visc_unknowns(const GridDims &d, bool heavy);
long long visc_coef_count(const GridDims &d, bool heavy);

// LightViscosityModel::apply (viscositymodel.cpp:4-63): *iters is the V
// solve's iteration count, or -1 when a solve failed (that solve is not
// applied, and the V solve is not run after a failed U solve)
cudaError_t visc_light(const GridDims &d, const Grids &G, float dt, float density, ViscBuffers &vb,
                       cudaStream_t st, int *iters, long long *launches);
// HeavyViscosityModel::apply (viscositymodel.cpp:164-200): *iters is the
// coupled solve's iteration count, or -1 when it failed (nothing applied)
cudaError_t visc_heavy(const GridDims &d, const Grids &G, float dt, float dx, float density,
                       ViscBuffers &vb, cudaStream_t st, int *iters, long long *launches);

} // namespace fsg
