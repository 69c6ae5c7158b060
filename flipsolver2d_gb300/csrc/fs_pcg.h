// fs_pcg.h -- launch interface of the cooperative PCG kernel (fs_pcg.cu).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "fs_state.h"

namespace fsg {

struct GridBarrier {
    unsigned int count;
    unsigned int gen;
    double result[4]; // scalars published by the last block to arrive
};

template <typename T> struct PcgArgs {
    int ni, nj;
    long long N;
    const uint8_t *info;       // packed operator rows (fs_grid.cu k_decomposition)
    const T *b;                // right-hand side
    T *x;                      // solution
    T *r0, *r1, *s0, *s1;      // ping-pong work vectors
    // The resident kernel's exchange words (fs_pcg_tma.cu): N 8-byte words
    // each for r and s, a float and the epoch that published it, and the
    // first epoch of this launch (set by launch_pcg_resident)
    unsigned long long *ll_r, *ll_s;
    unsigned long long *ll_rec; // per-block partial records of its reductions
    unsigned ll_base;
    double *partials;          // 8 * grid + 16 doubles (per-block partial records)
    const int *chunk_end;      // splitRange chunk ends (exclusive)
    const int *chunk_last_unit;// last unit row per chunk or -1
    double *chunk_val;         // per chunk |r| at its last unit row (scratch)
    int nchunks;
    const Scalars *sc;         // dt of the substep
    double density, dx;
    double scale;              // > 0: the operator's scale dt / (density dx^2) as
                               // given (fs_pcg_solve_operator); else from dt
    int iter_limit;
    double tol;
    int *iters_out;
    int *status;               // set to 1 when a barrier wait times out
    long long spin_limit;      // polls after which a device wait gives up (0: the
                               // kernel's default, seconds)
    GridBarrier *bar;
    const int *wrap_flag;      // set by the decomposition when a unit row sits on
                               // the j = 0 or j = NJ-1 edge (linear-index wrap)
    int mode;                  // 0 run, 1 run only if *wrap_flag, 2 only if !*wrap_flag
    // spec-mode inner solves (the resident kernel with the K K^T
    // preconditioner): the chained solve's control block (skip when done,
    // inner tolerance and iterations left from it, totals back to it) and
    // the device dt the operator's scale comes from
    struct SpecCtl *spec_ctl;
    const float *spec_dt;
};

// Owner of a set of exchange-word buffers (a solver handle, the per-device
// cache of the standalone solves, the fixed scratch of the no-allocation
// solve).  Epochs grow across the launches that share the buffers, so words
// left by an earlier launch never match; the buffers are cleared on first use
// and when the epochs would wrap.
struct LlBuffers {
    unsigned long long *r = nullptr, *s = nullptr; // `words` words each
    unsigned long long *rec = nullptr;             // kLlRecWords words
    size_t words = 0;
    unsigned next = 0; // first epoch of the next launch; 0: clear first
};
// The resident kernel's small exchange-word regions, one allocation: the
// partial records (two sets of at most 256 blocks, its tile limit, of one
// 128-byte line each), then per chunk of the max-abs test the index of its
// last live unit row (at most kLlMaxChunks chunks)
constexpr size_t kLlRecSets = 2 * 256 * 16;
constexpr size_t kLlEffOff = kLlRecSets;
constexpr size_t kLlMaxChunks = 4096;
constexpr size_t kLlRecWords = kLlEffOff + kLlMaxChunks;

// scale = dt / (density dx^2) of the pressure operator (flipsolver2d.cpp:797-887)
template <typename T> __device__ __forceinline__ double pcg_scale(const PcgArgs<T> &a)
{
    return a.scale > 0.0 ? a.scale : (double)a.sc->dt / (a.density * a.dx * a.dx);
}

template <typename T> int pcg_grid_size(long long N);
// Runs the solve: FP32 uses the shared-memory tiled kernel, falling back to
// the linear-index kernel when a unit row touches the j edges; FP64 always
// uses the linear-index kernel.  Returns the number of kernels launched.
template <typename T> cudaError_t launch_pcg(const PcgArgs<T> &a, cudaStream_t st, int *launched);
cudaError_t launch_pcg_linear_if_wrap(const PcgArgs<float> &a, cudaStream_t st);


// The index of the last nonzero entry in [lo, hi], or lo - 1 if there is
// none: the backward search of VOps::maxAbs (vmath.cpp:100-136) for a chunk
// whose last unit row holds a zero.  Warp-cooperative: all 32 lanes of a
// warp call it with the same arguments and get the same result; each step
// reads 256 entries with eight loads in flight per lane.  (A residual that
// is still zero over most of the grid -- a scene at rest -- otherwise means
// a serial walk over tens of thousands of entries per chunk per iteration.)
template <typename Load>
__device__ __forceinline__ long long warp_last_nonzero(long long lo, long long hi, Load load)
{
    const int lane = threadIdx.x & 31;
    for (; hi >= lo; hi -= 256) {
        bool nz[8];
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const long long e = hi - (j * 32 + lane);
            nz[j] = e >= lo && load(e) != 0;
        }
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const unsigned b = __ballot_sync(0xffffffffu, nz[j]);
            if (b) return hi - (j * 32 + (__ffs((int)b) - 1));
        }
    }
    return lo - 1;
}

} // namespace fsg
