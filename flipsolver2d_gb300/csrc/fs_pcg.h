// fs_pcg.h -- launch interface of the cooperative PCG kernel (fs_pcg.cu).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "fs_state.h"

namespace fsg {

struct GridBarrier {
    unsigned int count;
    unsigned int gen;
};

template <typename T> struct PcgArgs {
    int ni, nj;
    long long N;
    const uint8_t *info;       // packed operator rows (fs_grid.cu k_decomposition)
    const T *b;                // right-hand side
    T *x;                      // solution
    T *r0, *r1, *s0, *s1;      // ping-pong work vectors
    double *partials;          // 3 * grid doubles
    const int *chunk_end;      // splitRange chunk ends (exclusive)
    const int *chunk_last_unit;// last unit row per chunk or -1
    int nchunks;
    const Scalars *sc;         // dt of the substep
    double density, dx;
    int iter_limit;
    double tol;
    int *iters_out;
    int *status;               // set to 1 when a barrier wait times out
    GridBarrier *bar;
};

template <typename T> int pcg_grid_size(long long N);
template <typename T> cudaError_t launch_pcg(const PcgArgs<T> &a, int grid, cudaStream_t st);
void launch_chunk_last_unit(const uint8_t *info, const int *chunk_end, int nchunks, int *last,
                            cudaStream_t st);

} // namespace fsg
