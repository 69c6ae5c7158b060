// fs_spec.h -- launch interface of the spec-mode solve (fs_spec.cu).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "fs_pcg.h"

namespace fsg {

// the state of one chained solve on the device (launch_spec_chain): the
// outer loop's decisions live here, so the whole solve is enqueued at once
struct SpecCtl {
    double bb;    // ||b||^2 (the first check)
    double rr;    // ||b - A x||^2 of the last check
    float eps_in; // relative reduction asked of the next inner solve
    int done;     // 1: stop (converged, out of iterations, or no progress)
    int outer;    // checks run
    int total;    // inner iterations so far
    int last_it;  // inner iterations of the last inner solve
    int pad;
};

struct SpecArgs {
    int ni, nj;
    long long N;
    const uint8_t *info; // packed operator byte per cell (k_decomposition)
    double scale;        // dt / (density dx^2)
    float *r;            // in: outer residual (FP32); out: inner residual
    float *d;            // out: correction
    float *s, *q, *y, *z; // y unused: the kernel forms K K^T r in one pass
    float2 *partials;    // 3 * grid + 8
    unsigned *count;     // grid barrier counter
    int *status;         // 1 when a barrier wait gave up
    int *iters;          // out: inner iterations
    float eps_in;        // relative reduction of the inner residual norm
    int max_iter;
    SpecCtl *ctl;        // chained solves: skip when done, eps_in and the
                         // remaining iterations from here, totals back here
    const float *dt;     // when set: scale = *dt / (density dx^2) on the device
    double density, dx;
    const int *wrap_flag; // with mode 1: run only when a unit row touches a j edge
    int mode;             // 0 always, 1 only if *wrap_flag
};

// one whole spec-mode solve of A x = b enqueued on a stream with no host
// synchronisation: x = 0, then max_outer rounds of FP64 residual, check,
// inner FP32 PCG and FP64 update, then a last residual and check.  Each
// kernel reads the control block and does nothing once the solve is done.
constexpr int kSpecResBlocks = 1024;
struct SpecSolve {
    int ni, nj;
    const uint8_t *info;
    const double *b;
    double *x;
    const float *dt; // device: scale = dt / (density dx^2)
    double density, dx;
    float *r, *d, *s, *q, *z;  // N floats each
    float2 *partials;          // spec_partials_needed()
    double *rpart;             // kSpecResBlocks
    unsigned *count;
    int *status;
    SpecCtl *ctl;
    int *iters_out;   // optional: total inner iterations
    double *rel_out;  // optional: final relative residual
    double tol;
    int max_iter, max_outer;
    // Inner solves on the shared-memory-resident kernel when the grid fits
    // one tile per SM (res_ti > 0, tile res_ti x res_tj, exchange words in
    // *ll).  Its tiles treat cells outside the grid as absent, the linear
    // index wraps j edges into the next row, so on a grid whose unit rows
    // touch a j edge (*wrap_flag, set by the decomposition) the streaming
    // kernel runs instead; the choice is made on the device.
    int res_ti, res_tj;
    LlBuffers *ll;
    const int *wrap_flag;
};
cudaError_t launch_spec_chain(const SpecSolve &p, cudaStream_t st);
// kernels one launch_spec_chain enqueues
int spec_chain_kernels(const SpecSolve &p);

int spec_partials_needed();
cudaError_t launch_spec_residual(const uint8_t *info, const double *b, const double *x, float *r32,
                                 long long N, int NJ, double scale, double *partial, int nblocks,
                                 cudaStream_t st);
cudaError_t launch_spec_update(double *x, const float *d, long long N, cudaStream_t st);
cudaError_t launch_spec_pcg(const SpecArgs &a, cudaStream_t st);

} // namespace fsg
