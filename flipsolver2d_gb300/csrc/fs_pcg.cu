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

#include "fs_pcg.h"

namespace fsg {

constexpr int kPcgThreads = 512;
constexpr long long kBarrierSpinLimit = 1LL << 24; // ~2 s with 64 ns sleeps

// Bounded-spin grid barrier.  Co-residency is guaranteed by the cooperative
// launch; if a wait still exceeds the limit the kernel records status 1 and
// every block returns, leaving the context usable.
__device__ __forceinline__ bool grid_barrier(GridBarrier *gb, unsigned nblocks, int *status)
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
                if (++spins > kBarrierSpinLimit) {
                    atomicExch(status, 1);
                    ok = 0;
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return ok != 0 && *((volatile int *)status) == 0;
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
    __shared__ double sm[40];
    __shared__ double bcast[4];
    const long long N = a.N;
    const int nj = a.nj;
    const int G = gridDim.x;
    const long long per = ((N + G - 1) / G + blockDim.x - 1) / blockDim.x * blockDim.x;
    const long long lo = (long long)blockIdx.x * per;
    const long long hi = lo + per < N ? lo + per : N;
    double *pA = a.partials, *pB = a.partials + 2 * G;

    // operator coefficients (flipsolver2d.cpp:799, 891, 924-927)
    const double scale_d = (double)a.sc->dt / (a.density * a.dx * a.dx);
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
    if (!grid_barrier(a.bar, G, a.status)) return;
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
        if (!grid_barrier(a.bar, G, a.status)) return;
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
        if (!grid_barrier(a.bar, G, a.status)) return;

        // VOps::maxAbs with the reference's chunking (vmath.cpp:100-136)
        if (threadIdx.x < 32) {
            double m = 0.0;
            for (int k = threadIdx.x; k < a.nchunks; k += 32) {
                const long long start = k == 0 ? 0 : a.chunk_end[k - 1];
                long long idx = a.chunk_last_unit[k];
                while (idx >= start && rn[idx] == (T)0) idx--;
                const double v = idx >= start ? fabs((double)rn[idx]) : DBL_MIN;
                if (v > m) m = v;
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const double t = __shfl_down_sync(0xffffffffu, m, o);
                if (t > m) m = t;
            }
            if (threadIdx.x == 0) bcast[0] = m;
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

// last unit row of each splitRange chunk (or -1); one warp per chunk
__global__ void k_chunk_last_unit(const uint8_t *__restrict__ info, const int *__restrict__ chunk_end,
                                  int nchunks, int *__restrict__ last)
{
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= nchunks) return;
    const long long start = w == 0 ? 0 : chunk_end[w - 1];
    long long hiIdx = chunk_end[w] - 1;
    long long found = -1;
    while (hiIdx >= start) {
        const long long k = hiIdx - lane;
        const bool u = k >= start && (info[k] & 0x80);
        const unsigned bal = __ballot_sync(0xffffffffu, u);
        if (bal) {
            found = hiIdx - (__ffs(bal) - 1);
            break;
        }
        hiIdx -= 32;
    }
    if (lane == 0) last[w] = (int)found;
}

void launch_chunk_last_unit(const uint8_t *info, const int *chunk_end, int nchunks, int *last,
                            cudaStream_t st)
{
    const int threads = 256;
    const int blocks = (nchunks * 32 + threads - 1) / threads;
    k_chunk_last_unit<<<blocks, threads, 0, st>>>(info, chunk_end, nchunks, last);
}

template <typename T> int pcg_grid_size(long long N)
{
    static int cached = 0;
    if (!cached) {
        int dev = 0, sms = 0, per = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_pcg<T>, kPcgThreads, 0);
        cached = sms * (per > 0 ? per : 1);
    }
    long long want = (N + kPcgThreads * 4 - 1) / (kPcgThreads * 4);
    if (want < 1) want = 1;
    return (int)(want < cached ? want : cached);
}

template <typename T> cudaError_t launch_pcg(const PcgArgs<T> &a, int grid, cudaStream_t st)
{
    PcgArgs<T> args = a;
    void *kargs[] = {&args};
    cudaMemsetAsync(a.bar, 0, sizeof(GridBarrier), st);
    return cudaLaunchCooperativeKernel((const void *)k_pcg<T>, dim3(grid), dim3(kPcgThreads),
                                       kargs, 0, st);
}

template int pcg_grid_size<float>(long long);
template int pcg_grid_size<double>(long long);
template cudaError_t launch_pcg<float>(const PcgArgs<float> &, int, cudaStream_t);
template cudaError_t launch_pcg<double>(const PcgArgs<double> &, int, cudaStream_t);

int pcg_partials_per_block() { return 4; }

} // namespace fsg
