// fs_spec.h -- launch interface of the spec-mode solve (fs_spec.cu).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace fsg {

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
};

int spec_partials_needed();
cudaError_t launch_spec_residual(const uint8_t *info, const double *b, const double *x, float *r32,
                                 long long N, int NJ, double scale, double *partial, int nblocks,
                                 cudaStream_t st);
cudaError_t launch_spec_update(double *x, const float *d, long long N, cudaStream_t st);
cudaError_t launch_spec_pcg(const SpecArgs &a, cudaStream_t st);

} // namespace fsg
