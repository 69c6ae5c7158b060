// fs_pcg_tma.h -- launch interface of the TMA-staged FP32 PCG (fs_pcg_tma.cu).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <utility>
#include <vector>

#include "fs_pcg.h"

namespace fsg {

// Tensor maps of one solve: load maps (boxes with a 2-row / 4-column halo;
// 16 columns for the u8 operator rows) and store maps (boxes of one tile).
struct TmaMaps {
    CUtensorMap info, b, x, r0, r1, s0, s1;
    CUtensorMap r0_st, r1_st, s0_st, s1_st;
};

// tile shape for an ni x nj grid; false when TMA cannot be used (row pitch
// not a multiple of 16 bytes for the u8 rows)
bool tma_tile_shape(int ni, int nj, int *ti, int *tj);
bool tma_maps(TmaMaps *m, int ni, int nj, int ti, int tj, const uint8_t *info, const float *b,
              const float *x, const float *r0, const float *r1, const float *s0, const float *s1);
bool tma_store_maps(TmaMaps *m, int ni, int nj, int ti, int tj, const float *r0, const float *r1,
                    const float *s0, const float *s1);
cudaError_t launch_pcg_tma(const PcgArgs<float> &a, const TmaMaps &maps, int ti, int tj,
                           cudaStream_t st);
// one tile per block resident in shared memory for the whole solve; false
// when the grid needs more tiles than there are SMs
bool resident_tile_shape(int ni, int nj, int *ti, int *tj);
// every feasible resident tile shape (rows, columns) of a grid, and the
// autotuner's record of the one to use for a grid shape (ti <= 0 clears it)
void resident_candidates(int ni, int nj, std::vector<std::pair<int, int>> *out);
void resident_set_tuned(int ni, int nj, int ti, int tj);
// The shared-memory-resident FP32 solve; `ll` owns the exchange-word buffers
// (a.ll_r / a.ll_s are taken from it) and their epoch counter.
cudaError_t launch_pcg_resident(const PcgArgs<float> &a, int ti, int tj, cudaStream_t st,
                                LlBuffers *ll);
// Spec mode: the resident kernel as the inner FP32 solve of a chained
// spec-mode solve (K K^T preconditioner, r.r stopping rule, a.spec_ctl).
// The caller assigns the launch its exchange-word epochs: a.ll_base and the
// spec_resident_epochs(a.iter_limit) that follow.  False from the shape
// query when the grid does not fit register strips one tile per SM.
bool spec_resident_shape(int ni, int nj, int *ti, int *tj);
unsigned long long spec_resident_epochs(int max_iter);
cudaError_t launch_spec_resident(const PcgArgs<float> &a, int ti, int tj, cudaStream_t st);

} // namespace fsg
