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

// One request slot of the device-resident server: the request's material
// (copied in by the host), its operator bytes (written by the server before
// the solve) and the system it solves (sys.info == info).
struct ServeSlot {
    ClusterSystem sys;
    const int8_t *material;
    uint8_t *info;
};
// The request ring of the device-resident server.  The host writes the slot
// of request k at ring[k % ring_size] and then advances *tail (both in mapped
// pinned memory); the clusters of the server launch claim requests in order
// through *claimed (device memory), set started[slot] = k + 1 when they take
// request k and done[slot] = k + 1 when its result is in device memory.
struct ServeQueue {
    const ServeSlot *slots;    // device, one per slot
    const unsigned *tail;      // mapped: requests published
    const unsigned *ring;      // mapped
    unsigned ring_size;
    unsigned *claimed;         // device: requests taken
    unsigned *started, *done;  // mapped, one per slot
    const int *stop;           // mapped: 1 = leave after the current request
    long long idle_polls;      // polls of an empty ring (about 2 us each) before leaving
};
// Launches the server (as many clusters of `plan` as fit at once, each
// looping over requests); *clusters receives that number.
cudaError_t launch_serve(const ServeQueue &q, const ClusterPlan &plan, const ClusterParams &p, cudaStream_t st,
                         int *clusters);

// solves systems[0 .. n) (device array), all with the same C and K; smem =
// the largest of their needs
cudaError_t launch_pcg_cluster(const ClusterSystem *systems_dev, int n, const ClusterPlan &plan,
                               const ClusterParams &p, cudaStream_t st);

} // namespace fsg
