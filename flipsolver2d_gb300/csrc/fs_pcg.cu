// fs_pcg.cu -- the pressure / density-correction solve: LinearSolver::solve
// (linearsolver.cpp:25-73) on the matrix-free 5-point operator
// (IndexedPressureParameterUnit::multiply, pressuredata.h:132-146) with the
// IPP preconditioner the reference builds (IndexedIPPCoefficientUnit::multiply,
// PressureIPPCoeficients.h:23-40; coefficients flipsolver2d.cpp:889-945).
//
// One cooperative persistent kernel runs the whole solve.  Each iteration is
// two fused sweeps over the grid, separated by grid-wide barriers:
//   sweep 1: s_i = M r_i + beta s_{i-1} (M r recomputed from r's halo),
//            q_i = A s_i (s_i recomputed on the halo), partial q.s
//   sweep 2: x += alpha s_i, r_{i+1} = r_i - alpha q_i (q recomputed),
//            partial (M r_{i+1}).r_{i+1}
// so the vectors x, r, s (plus the packed u8 operator row) are the only
// traffic: 13 + 21 bytes per cell-iteration in FP32.
//
// The reference's semantics are kept: no preconditioner on iteration 0,
// alpha = sigma / (q.s + 1e-8), convergence when VOps::maxAbs(r) <= tol where
// maxAbs is the reference's (vmath.cpp:100-136): the vector is cut into the
// thread pool's splitRange chunks and each chunk reports |its last non-zero
// element|; the solver returns the loop index on convergence.  Since r is
// exactly zero outside the operator's unit rows, a chunk's last non-zero is
// found from the chunk's last unit row, walking back only if r is zero there.
//
// Precision: T = float keeps vectors and stencil arithmetic in FP32 with FMA;
// every cross-thread reduction (dot products, residual max) is FP64.  T =
// double reproduces the reference's FP64 element arithmetic exactly (explicit
// round-to-nearest intrinsics, no contraction); only the summation order of
// the dot products differs.
#include <cfloat>
#include <cstdio>
#include <cuda/atomic>

#include "fs_device.h"
#include "fs_pcg.h"

namespace fsg {

constexpr int kPcgThreads = 512;
constexpr long long kBarrierSpinLimit = 1LL << 24; // ~2 s with 64 ns sleeps

// Bounded-spin grid barrier.  Co-residency is guaranteed by the cooperative
// launch; if a wait still exceeds the limit the kernel records status 1 and
// every block returns, leaving the context usable.
__device__ __forceinline__ bool grid_barrier(GridBarrier *gb, unsigned nblocks, int *status,
                                             long long lim)
{
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        cuda::atomic_ref<unsigned, cuda::thread_scope_device> gen(gb->gen);
        cuda::atomic_ref<unsigned, cuda::thread_scope_device> cnt(gb->count);
        const unsigned g = gen.load(cuda::memory_order_acquire);
        __threadfence();
        const unsigned arrived = cnt.fetch_add(1u, cuda::memory_order_acq_rel);
        ok = 1;
        if (arrived == nblocks - 1) {
            cnt.store(0u, cuda::memory_order_relaxed);
            gen.fetch_add(1u, cuda::memory_order_release);
        } else {
            long long spins = 0;
            while (gen.load(cuda::memory_order_acquire) == g) {
                if (++spins > lim) {
                    atomicExch(status, 1);
                    ok = 0;
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
        // one verdict for the whole block (status can change between reads)
        if (*((volatile int *)status) != 0) ok = 0;
    }
    __syncthreads();
    return ok != 0;
}

// block-wide FP64 sum; result valid in every thread
__device__ __forceinline__ double block_sum(double v, double *sm)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) sm[w] = v;
    __syncthreads();
    if (w == 0) {
        double x = lane < (int)(blockDim.x >> 5) ? sm[lane] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (lane == 0) sm[32] = x;
    }
    __syncthreads();
    const double r = sm[32];
    __syncthreads();
    return r;
}

// sum of one double per block, in a fixed order (same result in every block)
__device__ __forceinline__ double grid_sum(const double *partials, int nblocks, double *sm)
{
    if (threadIdx.x < 32) {
        double a = 0.0;
        for (int k = threadIdx.x; k < nblocks; k += 32) a += partials[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
        if (threadIdx.x == 0) sm[33] = a;
    }
    __syncthreads();
    const double r = sm[33];
    __syncthreads();
    return r;
}

// Barrier that also reduces one or two FP64 values per block.  Every block
// publishes its partials and arrives; the last block to arrive sums all
// partials with its whole thread block in a fixed order (so every run and
// every block sees the same totals), optionally evaluates the reference's
// chunked max-abs residual test, publishes the results in the barrier
// record and releases the others.  Waits are bounded like grid_barrier.
template <typename R>
__device__ __forceinline__ bool grid_reduce(GridBarrier *gb, double *partials, unsigned nblocks,
                                            double v0, double v1, int nvals, int *status,
                                            double *sm, double out[3], R last_block_extra)
{
    __shared__ int s_last;
    __shared__ unsigned s_gen;
    __syncthreads();
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = v0;
        if (nvals > 1) partials[nblocks + blockIdx.x] = v1;
        cuda::atomic_ref<unsigned, cuda::thread_scope_device> gen(gb->gen);
        cuda::atomic_ref<unsigned, cuda::thread_scope_device> cnt(gb->count);
        s_gen = gen.load(cuda::memory_order_acquire);
        __threadfence();
        const unsigned arrived = cnt.fetch_add(1u, cuda::memory_order_acq_rel);
        s_last = arrived == nblocks - 1;
    }
    __syncthreads();
    if (s_last) {
        __threadfence();
        double a = 0.0, b = 0.0;
        for (unsigned k = threadIdx.x; k < nblocks; k += blockDim.x) {
            a += ((volatile double *)partials)[k];
            if (nvals > 1) b += ((volatile double *)partials)[nblocks + k];
        }
        a = block_sum(a, sm);
        if (nvals > 1) b = block_sum(b, sm);
        const double extra = last_block_extra();
        if (threadIdx.x == 0) {
            gb->result[0] = a;
            gb->result[1] = b;
            gb->result[2] = extra;
            __threadfence();
            cuda::atomic_ref<unsigned, cuda::thread_scope_device> gen(gb->gen);
            cuda::atomic_ref<unsigned, cuda::thread_scope_device> cnt(gb->count);
            cnt.store(0u, cuda::memory_order_relaxed);
            gen.fetch_add(1u, cuda::memory_order_release);
        }
    } else if (threadIdx.x == 0) {
        cuda::atomic_ref<unsigned, cuda::thread_scope_device> gen(gb->gen);
        long long spins = 0;
        while (gen.load(cuda::memory_order_acquire) == s_gen) {
            if (++spins > kBarrierSpinLimit) {
                atomicExch(status, 1);
                break;
            }
            __nanosleep(32);
        }
    }
    __syncthreads();
    if (*((volatile int *)status) != 0) return false;
    out[0] = ((volatile double *)gb->result)[0];
    out[1] = ((volatile double *)gb->result)[1];
    out[2] = ((volatile double *)gb->result)[2];
    return true;
}

// ---- element arithmetic --------------------------------------------------
template <typename T> struct Ops;

template <> struct Ops<float> {
    static __device__ __forceinline__ float mul(float a, float b) { return a * b; }
    static __device__ __forceinline__ float add(float a, float b) { return a + b; }
    static __device__ __forceinline__ float fma(float a, float b, float c) { return fmaf(a, b, c); }
};
template <> struct Ops<double> {
    static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
    static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
    // no contraction in the FP64 mode: round the product, then the sum
    static __device__ __forceinline__ double fma(double a, double b, double c)
    {
        return __dadd_rn(__dmul_rn(a, b), c);
    }
};

template <typename T> struct Coef {
    T ascale;   // scale
    T inv[5];   // 1 / (n * scale), n = nonsolid neighbour count of a neighbour
};

template <typename T>
__device__ __forceinline__ T ld(const T *__restrict__ v, long long k, long long N)
{
    return (k >= 0 && k < N) ? v[k] : (T)0;
}

// IPP row (PressureIPPCoeficients.h:23-40); identity on non-unit rows
template <typename T>
__device__ __forceinline__ T ipp_apply(const uint8_t *__restrict__ info, const T *__restrict__ r,
                                       long long c, int nj, long long N, const Coef<T> &cf)
{
    const uint8_t ic = info[c];
    const T rc = r[c];
    if (!(ic & 0x80)) return rc;
    const long long im = c - nj, ip = c + nj, jm = c - 1, jp = c + 1;
    const T iNeg = im >= 0 ? cf.inv[(info[im] >> 4) & 7] : (T)0;
    const T iPos = ip < N ? cf.inv[(info[ip] >> 4) & 7] : (T)0;
    const T jNeg = jm >= 0 ? cf.inv[(info[jm] >> 4) & 7] : (T)0;
    const T jPos = jp < N ? cf.inv[(info[jp] >> 4) & 7] : (T)0;
    typedef Ops<T> O;
    const T diag = O::add(O::add((T)1, O::mul(iNeg, iNeg)), O::mul(jNeg, jNeg));
    T acc = O::mul(diag, rc);
    acc = O::fma(jNeg, ld(r, jm, N), acc);
    acc = O::fma(jPos, ld(r, jp, N), acc);
    acc = O::fma(iNeg, ld(r, im, N), acc);
    acc = O::fma(iPos, ld(r, ip, N), acc);
    return acc;
}

// A row (pressuredata.h:132-146); identity on non-unit rows
template <typename T>
__device__ __forceinline__ T a_apply_vals(uint8_t ic, T sc_, T sim, T sip, T sjm, T sjp,
                                          const Coef<T> &cf)
{
    if (!(ic & 0x80)) return sc_;
    typedef Ops<T> O;
    const T count = (T)((ic >> 4) & 7);
    const T ns = -cf.ascale;
    T acc = O::mul(O::mul(cf.ascale, count), sc_);
    acc = O::fma(O::mul(ns, (T)(ic & 1)), sim, acc);
    acc = O::fma(O::mul(ns, (T)((ic >> 1) & 1)), sip, acc);
    acc = O::fma(O::mul(ns, (T)((ic >> 2) & 1)), sjm, acc);
    acc = O::fma(O::mul(ns, (T)((ic >> 3) & 1)), sjp, acc);
    return acc;
}

// s_i at cell c: first iteration s_0 = b (stored); later M r_i + beta s_{i-1}
template <typename T>
__device__ __forceinline__ T s_new_at(const uint8_t *__restrict__ info, const T *__restrict__ r,
                                      const T *__restrict__ sold, long long c, int nj, long long N,
                                      const Coef<T> &cf, T beta, bool first)
{
    if (c < 0 || c >= N) return (T)0;
    if (first) return sold[c];
    const T z = ipp_apply(info, r, c, nj, N, cf);
    return Ops<T>::fma(sold[c], beta, z);
}

template <typename T>
__device__ __forceinline__ T q_at(const uint8_t *__restrict__ info, const T *__restrict__ s,
                                  long long c, int nj, long long N, const Coef<T> &cf)
{
    if (c < 0 || c >= N) return (T)0;
    return a_apply_vals(info[c], s[c], ld(s, c - nj, N), ld(s, c + nj, N), ld(s, c - 1, N),
                        ld(s, c + 1, N), cf);
}

template <typename T>
__global__ void __launch_bounds__(kPcgThreads) k_pcg(PcgArgs<T> a)
{
    const long long lim = a.spin_limit > 0 ? a.spin_limit : kBarrierSpinLimit;
    __shared__ double sm[40];
    __shared__ double bcast[4];
    if (a.mode == 1 && *a.wrap_flag == 0) return;
    if (a.mode == 2 && *a.wrap_flag != 0) return;
    const long long N = a.N;
    const int nj = a.nj;
    const int G = gridDim.x;
    const long long per = ((N + G - 1) / G + blockDim.x - 1) / blockDim.x * blockDim.x;
    const long long lo = (long long)blockIdx.x * per;
    const long long hi = lo + per < N ? lo + per : N;
    double *pA = a.partials, *pB = a.partials + 2 * G;

    // operator coefficients (flipsolver2d.cpp:799, 891, 924-927)
    const double scale_d = pcg_scale(a);
    Coef<T> cf;
    cf.ascale = (T)scale_d;
#pragma unroll
    for (int n = 0; n < 5; n++) cf.inv[n] = (T)(1.0 / (n * scale_d));

    // phase 0: x = 0, r = s = b, sigma = b.b, zero test (VOps::isZero, 1e-15)
    float bb_f = 0.f;
    double bb_d = 0.0;
    int nz = 0;
    for (long long c = lo + threadIdx.x; c < hi; c += blockDim.x) {
        const T bv = a.b[c];
        a.x[c] = (T)0;
        a.r0[c] = bv;
        a.s0[c] = bv;
        if (sizeof(T) == 4) bb_f = fmaf((float)bv, (float)bv, bb_f);
        else bb_d = __dadd_rn(bb_d, __dmul_rn((double)bv, (double)bv));
        nz |= fabs((double)bv) > 1.0e-15;
    }
    double part = block_sum(sizeof(T) == 4 ? (double)bb_f : bb_d, sm);
    int anynz = __syncthreads_or(nz);
    if (threadIdx.x == 0) {
        pA[blockIdx.x] = part;
        pA[G + blockIdx.x] = anynz ? 1.0 : 0.0;
    }
    if (!grid_barrier(a.bar, G, a.status, lim)) return;
    double sigma = grid_sum(pA, G, sm);
    const double nzsum = grid_sum(pA + G, G, sm);
    if (nzsum == 0.0) {
        if (blockIdx.x == 0 && threadIdx.x == 0) *a.iters_out = 0;
        return;
    }

    double beta = 0.0;
    int result = a.iter_limit;
    for (int it = 0; it < a.iter_limit; it++) {
        T *rc = (it & 1) ? a.r1 : a.r0;         // r_it
        T *rn = (it & 1) ? a.r0 : a.r1;         // r_{it+1}
        T *sc_ = (it & 1) ? a.s1 : a.s0;        // s_it
        const T *sp = (it & 1) ? a.s0 : a.s1;   // s_{it-1}
        const bool first = it == 0;
        const T tb = (T)beta;

        // ---- sweep 1 -------------------------------------------------
        float qs_f = 0.f;
        double qs_d = 0.0;
        for (long long c = lo + threadIdx.x; c < hi; c += blockDim.x) {
            const T s_c = first ? sc_[c] : s_new_at(a.info, rc, sp, c, nj, N, cf, tb, false);
            const T s_im = first ? ld(sc_, c - nj, N) : s_new_at(a.info, rc, sp, c - nj, nj, N, cf, tb, false);
            const T s_ip = first ? ld(sc_, c + nj, N) : s_new_at(a.info, rc, sp, c + nj, nj, N, cf, tb, false);
            const T s_jm = first ? ld(sc_, c - 1, N) : s_new_at(a.info, rc, sp, c - 1, nj, N, cf, tb, false);
            const T s_jp = first ? ld(sc_, c + 1, N) : s_new_at(a.info, rc, sp, c + 1, nj, N, cf, tb, false);
            const T q = a_apply_vals(a.info[c], s_c, s_im, s_ip, s_jm, s_jp, cf);
            if (!first) sc_[c] = s_c;
            if (sizeof(T) == 4) qs_f = fmaf((float)q, (float)s_c, qs_f);
            else qs_d = __dadd_rn(qs_d, __dmul_rn((double)q, (double)s_c));
        }
        part = block_sum(sizeof(T) == 4 ? (double)qs_f : qs_d, sm);
        if (threadIdx.x == 0) pA[blockIdx.x] = part;
        if (!grid_barrier(a.bar, G, a.status, lim)) return;
        const double qs = grid_sum(pA, G, sm);
        const double alpha = sigma / (qs + 1e-8);
        const T ta = (T)alpha;

        // ---- sweep 2 -------------------------------------------------
        float zr_f = 0.f;
        double zr_d = 0.0;
        for (long long c = lo + threadIdx.x; c < hi; c += blockDim.x) {
            typedef Ops<T> O;
            const T q_c = q_at(a.info, sc_, c, nj, N, cf);
            const T r_c = O::add(rc[c], -O::mul(q_c, ta));
            a.x[c] = O::fma(sc_[c], ta, a.x[c]);
            rn[c] = r_c;
            T z;
            const uint8_t ic = a.info[c];
            if (!(ic & 0x80)) {
                z = r_c;
            } else {
                const long long im = c - nj, ip = c + nj, jm = c - 1, jp = c + 1;
                auto rnew = [&](long long k) -> T {
                    if (k < 0 || k >= N) return (T)0;
                    return O::add(rc[k], -O::mul(q_at(a.info, sc_, k, nj, N, cf), ta));
                };
                const T iNeg = im >= 0 ? cf.inv[(a.info[im] >> 4) & 7] : (T)0;
                const T iPos = ip < N ? cf.inv[(a.info[ip] >> 4) & 7] : (T)0;
                const T jNeg = jm >= 0 ? cf.inv[(a.info[jm] >> 4) & 7] : (T)0;
                const T jPos = jp < N ? cf.inv[(a.info[jp] >> 4) & 7] : (T)0;
                const T diag = O::add(O::add((T)1, O::mul(iNeg, iNeg)), O::mul(jNeg, jNeg));
                T acc = O::mul(diag, r_c);
                acc = O::fma(jNeg, rnew(jm), acc);
                acc = O::fma(jPos, rnew(jp), acc);
                acc = O::fma(iNeg, rnew(im), acc);
                acc = O::fma(iPos, rnew(ip), acc);
                z = acc;
            }
            if (sizeof(T) == 4) zr_f = fmaf((float)z, (float)r_c, zr_f);
            else zr_d = __dadd_rn(zr_d, __dmul_rn((double)z, (double)r_c));
        }
        part = block_sum(sizeof(T) == 4 ? (double)zr_f : zr_d, sm);
        if (threadIdx.x == 0) pB[blockIdx.x] = part;
        if (!grid_barrier(a.bar, G, a.status, lim)) return;

        // VOps::maxAbs with the reference's chunking (vmath.cpp:100-136):
        // one warp per chunk, the max over warps (order-independent)
        {
            const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
            double m = 0.0;
            for (int k = warp; k < a.nchunks; k += nw) {
                const long long start = k == 0 ? 0 : a.chunk_end[k - 1];
                const long long last = a.chunk_last_unit[k];
                const long long idx =
                    last < 0 ? -1 : warp_last_nonzero(start, last, [&](long long e) { return rn[e]; });
                const double v = idx >= start ? fabs((double)rn[idx]) : DBL_MIN;
                if (v > m) m = v;
            }
            if (lane == 0) sm[warp] = m;
            __syncthreads();
            if (threadIdx.x == 0) {
                for (int w = 1; w < nw; w++)
                    if (sm[w] > m) m = sm[w];
                bcast[0] = m;
            }
        }
        __syncthreads();
        const double err = bcast[0];
        const double newSigma = grid_sum(pB, G, sm);
        if (err <= a.tol) {
            result = it;
            break;
        }
        beta = newSigma / sigma;
        sigma = newSigma;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *a.iters_out = result;
}

// ---------------------------------------------------------------------------
// Shared-memory tiled FP32 kernel.  The grid is cut into tiles of TI x TJ
// cells sized at launch so that each block owns about one tile per sweep
// (large tiles keep many loads in flight and amortise the halo).  A sweep
// stages its inputs with a halo of two cells, computes the recomputed
// intermediate (M r, then s; or A s, then r) once per halo-1 cell in shared
// memory and the final stencil on the tile.  Neighbours are the 2-D
// neighbours, equal to the reference's linear-index neighbours except across
// the j = 0 / j = NJ-1 edges; a decomposition flag routes grids with unit rows
// on those edges to the linear kernel above.
// ---------------------------------------------------------------------------
constexpr int kTiledThreads = 1024;
constexpr int kMaxTileCells = 12288;

struct TileShape {
    int ti, tj; // tile rows / columns
};

__device__ __forceinline__ float ipp_tile(const float *__restrict__ R, const uint8_t *__restrict__ I,
                                          int c2, int w2, const float inv[5])
{
    const uint8_t ic = I[c2];
    const float rc = R[c2];
    if (!(ic & 0x80)) return rc;
    const float iNeg = inv[(I[c2 - w2] >> 4) & 7];
    const float iPos = inv[(I[c2 + w2] >> 4) & 7];
    const float jNeg = inv[(I[c2 - 1] >> 4) & 7];
    const float jPos = inv[(I[c2 + 1] >> 4) & 7];
    const float diag = (1.f + iNeg * iNeg) + jNeg * jNeg;
    float acc = diag * rc;
    acc = fmaf(jNeg, R[c2 - 1], acc);
    acc = fmaf(jPos, R[c2 + 1], acc);
    acc = fmaf(iNeg, R[c2 - w2], acc);
    acc = fmaf(iPos, R[c2 + w2], acc);
    return acc;
}

// A row from array S (row stride `stride`) at index c
__device__ __forceinline__ float a_tile(const float *__restrict__ S, uint8_t ic, int c, int stride,
                                        float scale)
{
    const float sc_ = S[c];
    if (!(ic & 0x80)) return sc_;
    float nb = 0.f;
    if (ic & 1) nb += S[c - stride];
    if (ic & 2) nb += S[c + stride];
    if (ic & 4) nb += S[c - 1];
    if (ic & 8) nb += S[c + 1];
    return scale * ((float)((ic >> 4) & 7) * sc_ - nb);
}

// ---- reductions that keep FP64 arithmetic off the 1024-thread paths --------
// GB300's FP64 pipe runs at a small fraction of FP32, so a block-wide FP64
// shuffle tree costs microseconds.  Inside a warp the partial sums travel as
// compensated FP32 pairs (Knuth's two-sum keeps the rounding error of every
// addition in the low word, ~48 significant bits); FP64 arithmetic starts at
// the 32 per-warp pairs (one warp) and at the per-block partials (one warp).
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e)
{
    s = a + b;
    const float bv = s - a;
    e = (a - (s - bv)) + (b - bv);
}

// block-wide sum of per-thread FP32 partials; FP64 result in every thread
__device__ __forceinline__ double block_sum_ff(float v, double *sm)
{
    float hi = v, lo = 0.f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float h2 = __shfl_down_sync(0xffffffffu, hi, o);
        const float l2 = __shfl_down_sync(0xffffffffu, lo, o);
        float s, e;
        two_sum(hi, h2, s, e);
        hi = s;
        lo = lo + l2 + e;
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) sm[w] = (double)hi + (double)lo;
    __syncthreads();
    if (w == 0) {
        double x = lane < (int)(blockDim.x >> 5) ? sm[lane] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (lane == 0) sm[32] = x;
    }
    __syncthreads();
    const double r = sm[32];
    __syncthreads();
    return r;
}

// sum of the per-block partials after a barrier, by one warp in a fixed order
__device__ __forceinline__ double sum_partials_w(const double *partials, int nblocks, double *sm)
{
    if (threadIdx.x < 32) {
        double a = 0.0;
        for (int k = threadIdx.x; k < nblocks; k += 32) a += ((volatile const double *)partials)[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
        if (threadIdx.x == 0) sm[34] = a;
    }
    __syncthreads();
    const double r = sm[34];
    __syncthreads();
    return r;
}

// Tight-spin grid barrier (bounded like grid_barrier; spins without sleeping
// first, since a barrier here normally completes within microseconds).
__device__ __forceinline__ bool grid_sync_fast(GridBarrier *gb, unsigned nblocks, int *status,
                                               long long lim)
{
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned *vgen = &gb->gen;
        const unsigned g = *vgen;
        __threadfence();
        const unsigned arrived = atomicAdd(&gb->count, 1u);
        if (arrived == nblocks - 1) {
            gb->count = 0;
            __threadfence();
            atomicAdd(&gb->gen, 1u);
        } else {
            long long spins = 0;
            while (*vgen == g) {
                if (++spins > lim) {
                    atomicExch(status, 1);
                    break;
                }
                if (spins > 4096) __nanosleep(64);
            }
        }
        __threadfence();
        // one verdict for the whole block (status can change between reads)
        s_ok = *((volatile int *)status) == 0;
    }
    __syncthreads();
    return s_ok != 0;
}

// sum of the per-block partials after a barrier: one load per thread, then a
// fixed-order block reduction (identical in every block)
__device__ __forceinline__ double sum_partials(const double *partials, int nblocks, double *sm)
{
    double v = 0.0;
    for (int k = threadIdx.x; k < nblocks; k += blockDim.x) v += ((volatile const double *)partials)[k];
    return block_sum(v, sm);
}

// Batched halo load: every thread issues all of its global loads before any
// shared-memory store, so up to kLoadBatch loads are in flight per thread.
constexpr int kLoadBatch = 16;

template <typename V>
__device__ __forceinline__ void load_region(V *__restrict__ dst, const V *__restrict__ src, int ti0,
                                            int tj0, int halo, int h, int w, int NI, int NJ)
{
    const int n = h * w;
    for (int base = 0; base < n; base += kLoadBatch * (int)blockDim.x) {
        V v[kLoadBatch];
#pragma unroll
        for (int k = 0; k < kLoadBatch; k++) {
            const int e = base + k * (int)blockDim.x + (int)threadIdx.x;
            v[k] = (V)0;
            if (e < n) {
                const int gi = ti0 - halo + e / w, gj = tj0 - halo + e % w;
                if (gi >= 0 && gi < NI && gj >= 0 && gj < NJ) v[k] = src[(size_t)gi * NJ + gj];
            }
        }
#pragma unroll
        for (int k = 0; k < kLoadBatch; k++) {
            const int e = base + k * (int)blockDim.x + (int)threadIdx.x;
            if (e < n) dst[e] = v[k];
        }
    }
}

__global__ void __launch_bounds__(kTiledThreads) k_pcg_tiled(PcgArgs<float> a, TileShape ts)
{
    // tight spins first, so the default allows more polls than grid_barrier's
    const long long lim_fast = a.spin_limit > 0 ? a.spin_limit : (kBarrierSpinLimit << 4);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ double sm[40];
    __shared__ double s_err;
    if (a.mode == 1 && *a.wrap_flag == 0) return;
    if (a.mode == 2 && *a.wrap_flag != 0) return;
    const int NI = a.ni, NJ = a.nj;
    const long long N = a.N;
    const int G = gridDim.x;
    const int TI = ts.ti, TJ = ts.tj;
    const int W2 = TJ + 4, H2 = TI + 4, W1 = TJ + 2, H1 = TI + 2;
    float *A2 = reinterpret_cast<float *>(smem_raw);
    float *B1 = A2 + H2 * W2;
    uint8_t *I2 = reinterpret_cast<uint8_t *>(B1 + H1 * W1);
    const int tiles_j = (NJ + TJ - 1) / TJ, tiles_i = (NI + TI - 1) / TI;
    const int ntiles = tiles_i * tiles_j;
    double *pA = a.partials, *pB = a.partials + G, *pC = a.partials + 2 * G;
    double *chunk_val = a.chunk_val;

    const double scale_d = pcg_scale(a);
    const float scale = (float)scale_d;
    float inv[5];
    inv[0] = 0.f; // only outside the grid
#pragma unroll
    for (int n = 1; n < 5; n++) inv[n] = (float)(1.0 / (n * scale_d));

    // phase 0 (contiguous ranges): x = 0, r = s = b, sigma = b.b, zero test
    const long long per = ((N + G - 1) / G + blockDim.x - 1) / blockDim.x * blockDim.x;
    const long long lo = (long long)blockIdx.x * per;
    const long long hi = lo + per < N ? lo + per : N;
    float bb = 0.f;
    int nz = 0;
    for (long long c = lo + threadIdx.x; c < hi; c += blockDim.x) {
        const float bv = a.b[c];
        a.x[c] = 0.f;
        a.r0[c] = bv;
        a.s0[c] = bv;
        bb = fmaf(bv, bv, bb);
        nz |= fabsf(bv) > 1.0e-15f;
    }
    {
        const double part = block_sum_ff(bb, sm);
        const int anynz = __syncthreads_or(nz);
        if (threadIdx.x == 0) {
            pA[blockIdx.x] = part;
            pC[blockIdx.x] = anynz ? 1.0 : 0.0;
        }
    }
    if (!grid_sync_fast(a.bar, G, a.status, lim_fast)) return;
    double sigma = sum_partials_w(pA, G, sm);
    if (sum_partials_w(pC, G, sm) == 0.0) {
        if (blockIdx.x == 0 && threadIdx.x == 0) *a.iters_out = 0;
        return;
    }

    double beta = 0.0;
    int result = a.iter_limit;
    for (int it = 0; it < a.iter_limit; it++) {
        float *rc = (it & 1) ? a.r1 : a.r0;
        float *rn = (it & 1) ? a.r0 : a.r1;
        float *scur = (it & 1) ? a.s1 : a.s0;
        const float *sprev = (it & 1) ? a.s0 : a.s1;
        const bool first = it == 0;
        const float fb = (float)beta;

        // ---- sweep 1: s = M r + beta s_prev on the halo, q = A s, q.s ----
        float qs = 0.f;
        for (int t = blockIdx.x; t < ntiles; t += G) {
            const int ti0 = (t / tiles_j) * TI, tj0 = (t % tiles_j) * TJ;
            load_region<uint8_t>(I2, a.info, ti0, tj0, 2, H2, W2, NI, NJ);
            if (!first) load_region<float>(A2, rc, ti0, tj0, 2, H2, W2, NI, NJ);
            load_region<float>(B1, first ? scur : sprev, ti0, tj0, 1, H1, W1, NI, NJ);
            __syncthreads();
            if (!first) {
                for (int e = threadIdx.x; e < H1 * W1; e += blockDim.x) {
                    const int r = e / W1, q = e - r * W1;
                    const int c2 = (r + 1) * W2 + (q + 1);
                    B1[e] = fmaf(B1[e], fb, ipp_tile(A2, I2, c2, W2, inv));
                }
                __syncthreads();
            }
            for (int e = threadIdx.x; e < TI * TJ; e += blockDim.x) {
                const int r = e / TJ, q = e - r * TJ;
                const int gi = ti0 + r, gj = tj0 + q;
                if (gi >= NI || gj >= NJ) continue;
                const int c1 = (r + 1) * W1 + (q + 1);
                const uint8_t ic = I2[(r + 2) * W2 + (q + 2)];
                const float s_c = B1[c1];
                const float qv = a_tile(B1, ic, c1, W1, scale);
                qs = fmaf(qv, s_c, qs);
                if (!first) scur[(size_t)gi * NJ + gj] = s_c;
            }
            __syncthreads();
        }
        {
            const double part = block_sum_ff(qs, sm);
            if (threadIdx.x == 0) pA[blockIdx.x] = part;
        }
        if (!grid_sync_fast(a.bar, G, a.status, lim_fast)) return;
        const double alpha = sigma / (sum_partials_w(pA, G, sm) + 1e-8);
        const float fa = (float)alpha;

        // ---- sweep 2: r' = r - alpha A s on the halo, z = M r', x += alpha s
        float zr = 0.f;
        for (int t = blockIdx.x; t < ntiles; t += G) {
            const int ti0 = (t / tiles_j) * TI, tj0 = (t % tiles_j) * TJ;
            load_region<uint8_t>(I2, a.info, ti0, tj0, 2, H2, W2, NI, NJ);
            load_region<float>(A2, scur, ti0, tj0, 2, H2, W2, NI, NJ);
            load_region<float>(B1, rc, ti0, tj0, 1, H1, W1, NI, NJ);
            __syncthreads();
            for (int e = threadIdx.x; e < H1 * W1; e += blockDim.x) {
                const int r = e / W1, q = e - r * W1;
                const int c2 = (r + 1) * W2 + (q + 1);
                B1[e] = fmaf(-a_tile(A2, I2[c2], c2, W2, scale), fa, B1[e]);
            }
            __syncthreads();
            for (int e = threadIdx.x; e < TI * TJ; e += blockDim.x) {
                const int r = e / TJ, q = e - r * TJ;
                const int gi = ti0 + r, gj = tj0 + q;
                if (gi >= NI || gj >= NJ) continue;
                const int c1 = (r + 1) * W1 + (q + 1);
                const int c2 = (r + 2) * W2 + (q + 2);
                const uint8_t ic = I2[c2];
                const float r_c = B1[c1];
                float z = r_c;
                if (ic & 0x80) {
                    const float iNeg = inv[(I2[c2 - W2] >> 4) & 7];
                    const float iPos = inv[(I2[c2 + W2] >> 4) & 7];
                    const float jNeg = inv[(I2[c2 - 1] >> 4) & 7];
                    const float jPos = inv[(I2[c2 + 1] >> 4) & 7];
                    const float diag = (1.f + iNeg * iNeg) + jNeg * jNeg;
                    z = diag * r_c;
                    z = fmaf(jNeg, B1[c1 - 1], z);
                    z = fmaf(jPos, B1[c1 + 1], z);
                    z = fmaf(iNeg, B1[c1 - W1], z);
                    z = fmaf(iPos, B1[c1 + W1], z);
                }
                zr = fmaf(z, r_c, zr);
                const size_t g = (size_t)gi * NJ + gj;
                a.x[g] = fmaf(A2[c2], fa, a.x[g]);
                rn[g] = r_c;
            }
            __syncthreads();
        }
        // VOps::maxAbs (vmath.cpp:100-136): each chunk's value is |r| at the
        // chunk's last unit row, read here by the block that wrote it; -1
        // marks the rare case r == 0 there, resolved after the barrier.
        for (int k = threadIdx.x; k < a.nchunks; k += blockDim.x) {
            const int idx = a.chunk_last_unit[k];
            if (idx < 0) continue;
            const int gi = idx / NJ, gj = idx - gi * NJ;
            const int owner = ((gi / TI) * tiles_j + gj / TJ) % G;
            if (owner != (int)blockIdx.x) continue;
            const float v = rn[idx];
            chunk_val[k] = v != 0.f ? fabs((double)v) : -1.0;
        }
        {
            const double part = block_sum_ff(zr, sm);
            if (threadIdx.x == 0) pB[blockIdx.x] = part;
        }
        if (!grid_sync_fast(a.bar, G, a.status, lim_fast)) return;
        {
            // one warp per chunk, the max over warps (order-independent)
            const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
            double m = 0.0;
            for (int k = warp; k < a.nchunks; k += nw) {
                const long long start = k == 0 ? 0 : a.chunk_end[k - 1];
                const int last = a.chunk_last_unit[k];
                double v;
                if (last < 0) {
                    v = DBL_MIN;
                } else {
                    v = ((volatile double *)chunk_val)[k];
                    if (v < 0.0) {
                        const long long idx = warp_last_nonzero(
                            start, (long long)last - 1, [&](long long e) { return ((volatile float *)rn)[e]; });
                        v = idx >= start ? fabs((double)((volatile float *)rn)[idx]) : DBL_MIN;
                    }
                }
                if (v > m) m = v;
            }
            if (lane == 0) sm[warp] = m;
            __syncthreads();
            if (threadIdx.x == 0) {
                for (int w = 1; w < nw; w++)
                    if (sm[w] > m) m = sm[w];
                s_err = m;
            }
        }
        __syncthreads();
        const double err = s_err;
        const double newSigma = sum_partials_w(pB, G, sm);
        if (err <= a.tol) {
            result = it;
            break;
        }
        beta = newSigma / sigma;
        sigma = newSigma;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *a.iters_out = result;
}

static size_t tiled_smem(TileShape ts)
{
    return (size_t)(ts.ti + 4) * (ts.tj + 4) * 4 + (size_t)(ts.ti + 2) * (ts.tj + 2) * 4 +
           (size_t)(ts.ti + 4) * (ts.tj + 4) + 16;
}

// Tiles of up to 128 columns; rows chosen so that the tile count is at most
// `blocks` x k for the smallest k whose tiles fit in shared memory, i.e. every
// block owns k tiles per sweep (k = 1 whenever the grid allows).
static TileShape tile_shape(int ni, int nj, int blocks)
{
    TileShape ts;
    ts.tj = nj < 128 ? ((nj + 31) / 32) * 32 : 128;
    const long long tiles_j = (nj + ts.tj - 1) / ts.tj;
    const long long cap = kMaxTileCells / ts.tj;
    for (long long k = 1;; k++) {
        long long max_ti = (long long)blocks * k / tiles_j;
        if (max_ti < 1) continue;
        long long ti = (ni + max_ti - 1) / max_ti;
        // at least 8 rows: thinner tiles would mostly load halo
        if (ti < 8) ti = ni < 8 ? ni : 8;
        if (ti <= cap || k > 4096) {
            ts.ti = (int)(ti < cap ? ti : cap);
            return ts;
        }
    }
}

// resident blocks of the linear-index kernel on the current device
template <typename T> static int linear_grid()
{
    static std::atomic<int> slots[kMaxDevices];
    return device_cached(slots, [] { return occupancy_grid((const void *)k_pcg<T>, kPcgThreads, 64); });
}

// largest grid any PCG launch may use (sizes the partial-sum buffer)
template <typename T> int pcg_grid_size(long long N)
{
    (void)N;
    const int lin = linear_grid<T>(), sms = device_sm_count();
    return lin > sms ? lin : sms;
}

template <typename T>
static cudaError_t coop(const void *fn, PcgArgs<T> args, int grid, int threads, cudaStream_t st)
{
    void *kargs[] = {&args};
    cudaError_t e = cudaMemsetAsync(args.bar, 0, sizeof(GridBarrier), st);
    if (e != cudaSuccess) return e;
    return cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(threads), kargs, 0, st);
}

template <typename T> cudaError_t launch_pcg(const PcgArgs<T> &a, cudaStream_t st, int *launched)
{
    const int lin = linear_grid<T>();
    long long want = (a.N + kPcgThreads * 4 - 1) / (kPcgThreads * 4);
    int glin = (int)(want < 1 ? 1 : (want < lin ? want : lin));
    if (sizeof(T) == 8) {
        PcgArgs<T> b = a;
        b.mode = 0;
        *launched = 1;
        return coop((const void *)k_pcg<T>, b, glin, kPcgThreads, st);
    }
    const int sms = device_sm_count();
    {
        // a function attribute belongs to the current device's context
        const TileShape big{kMaxTileCells / 128, 128};
        cudaError_t e = cudaFuncSetAttribute((const void *)k_pcg_tiled,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)tiled_smem(big));
        if (e != cudaSuccess) return e;
    }
    const TileShape ts = tile_shape(a.ni, a.nj, sms);
    const long long ntiles = (long long)((a.ni + ts.ti - 1) / ts.ti) * ((a.nj + ts.tj - 1) / ts.tj);
    // equal tile counts per block
    const long long tpb = (ntiles + sms - 1) / sms;
    const int gtil = (int)((ntiles + tpb - 1) / tpb);
    PcgArgs<T> b = a;
    b.mode = 2; // tiled unless a unit row touches the j edges
    {
        PcgArgs<float> fa = *reinterpret_cast<PcgArgs<float> *>(&b);
        TileShape tsv = ts;
        void *kargs[] = {&fa, &tsv};
        cudaError_t e = cudaMemsetAsync(fa.bar, 0, sizeof(GridBarrier), st);
        if (e != cudaSuccess) return e;
        e = cudaLaunchCooperativeKernel((const void *)k_pcg_tiled, dim3(gtil), dim3(kTiledThreads),
                                        kargs, tiled_smem(ts), st);
        if (e != cudaSuccess) return e;
    }
    b.mode = 1;
    *launched = 2;
    return coop((const void *)k_pcg<T>, b, glin, kPcgThreads, st);
}

// the linear-index FP32 kernel, run only when the decomposition flagged unit
// rows on the j edges (the TMA kernel runs otherwise)
cudaError_t launch_pcg_linear_if_wrap(const PcgArgs<float> &a, cudaStream_t st)
{
    const int lin = linear_grid<float>();
    long long want = (a.N + kPcgThreads * 4 - 1) / (kPcgThreads * 4);
    int glin = (int)(want < 1 ? 1 : (want < lin ? want : lin));
    PcgArgs<float> b = a;
    b.mode = 1;
    return coop((const void *)k_pcg<float>, b, glin, kPcgThreads, st);
}

template int pcg_grid_size<float>(long long);
template int pcg_grid_size<double>(long long);
template cudaError_t launch_pcg<float>(const PcgArgs<float> &, cudaStream_t, int *);
template cudaError_t launch_pcg<double>(const PcgArgs<double> &, cudaStream_t, int *);

} // namespace fsg
