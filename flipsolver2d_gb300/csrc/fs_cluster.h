// fs_cluster.h -- launch interface of the cluster pressure solve
// (fs_cluster.cu): many independent systems in one launch, one thread-block
// cluster per system, every vector of the inner iteration on chip.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>
#include <vector>

namespace fsg {

// one pressure system A x = b of the reference's operator
// (getPressureProjectionMatrix) on an ni x nj material grid
struct ClusterSystem {
    int ni, nj;
    const uint8_t *info;  // packed operator byte per cell (k_decomposition)
    const double *b;      // right-hand side, ni * nj
    double *x;            // solution, ni * nj (overwritten; starts from 0)
    const float *dt;      // the step's dt on the device: scale = dt / (density dx^2)
    double density, dx;
    int *iters;           // out: inner PCG iterations, summed over refinements
    double *rel_res;      // out: ||b - A x|| / ||b|| of the returned x (0 for b = 0)
};

struct ClusterParams {
    double tol;     // stop when ||b - A x|| <= tol ||b|| (FP64)
    float eps_in;   // relative reduction of one inner FP32 solve
    int max_iter;   // inner iterations over all refinements
    int max_outer;  // refinements
};

// how one system runs: C CTAs per cluster, K own cells per thread at most,
// smem bytes of dynamic shared memory per CTA
struct ClusterPlan {
    int C, K;
    size_t smem;
};
// false: the system does not fit on chip (or there is no device).  The plan
// the autotuner chose for this shape if there is one, else the smallest C
// whose CTAs fit.
bool cluster_plan(int ni, int nj, ClusterPlan *plan);
// every C that fits, with its plan (the autotuner's candidates)
void cluster_candidates(int ni, int nj, std::vector<ClusterPlan> *out);
// records the autotuner's choice for a shape (later cluster_plan calls use it)
void cluster_set_tuned(int ni, int nj, const ClusterPlan &plan);
// the most cells a system may have
long long cluster_max_cells();

// solves systems[0 .. n) (device array), all with the same C and K; smem =
// the largest of their needs
cudaError_t launch_pcg_cluster(const ClusterSystem *systems_dev, int n, const ClusterPlan &plan,
                               const ClusterParams &p, cudaStream_t st);

} // namespace fsg
