// fs_spec.cu -- the spec-mode pressure solve: mixed precision to a true
// relative residual.
//
// The reference's hot-path PCG (linearsolver.cpp:25-73 with the asymmetric
// IPP of getIPPCoefficients) cannot reach a 1e-6 relative residual: its
// preconditioner is not symmetric and the iteration stalls.  The reference
// also ships a textbook incomplete-Poisson preconditioner it never uses on
// the hot path (inversepoissonpreconditioner.h:45-79): M = K K^T with
// K = I - L D^-1, L the strictly lower part of the pressure matrix A (linear
// index order) and D its diagonal.  This file solves A x = b with it:
//
//   outer (FP64):  r = b - A x;  stop when ||r|| <= tol ||b||
//   inner (FP32):  PCG on A d = r with M, to a relative reduction eps_in
//   outer (FP64):  x += d
//
// A is the operator of getPressureProjectionMatrix exactly as the reference
// builds it (unit rows with their fluid-neighbour mask and non-solid count,
// linear-index neighbours, identity rows elsewhere), read from the packed
// operator byte of k_decomposition.  K(c, n) for a lower neighbour n of unit
// row c is scale / A(n, n) (Eigen's zero-diagonal rule: 1), i.e. 1 / count(n)
// for a unit n.
//
// The inner PCG is one cooperative kernel over the linear index with FP32
// vectors and float-pair reductions.  It forms q = A s as A z + beta q and
// z = K K^T r in one pass (each saves a grid barrier), so an iteration takes
// three barriers.
#include <cfloat>
#include <cstdint>
#include <cuda_runtime.h>

#include "fs_device.h"
#include "fs_pcg.h"
#include "fs_pcg_tma.h"
#include "fs_spec.h"

namespace fsg {

constexpr int kSpecThreads = 512;
constexpr long long kSpecSpin = 1LL << 25;

// ---------------------------------------------------------------------------
// the operator and the preconditioner, from the packed operator byte
// (bit 7 unit row, bits 4-6 non-solid count, bits 0-3 fluid-neighbour mask)
// ---------------------------------------------------------------------------
__device__ __forceinline__ float spec_k(uint8_t info_n, float scale)
{
    const int cnt = (info_n >> 4) & 7;
    return ((info_n & 0x80) && cnt > 0) ? 1.f / (float)cnt : scale;
}

template <typename T>
__device__ __forceinline__ T spec_a(const uint8_t *__restrict__ info, const T *__restrict__ v, long long c,
                                    long long N, int NJ, T scale)
{
    const uint8_t p = info[c];
    const T vc = v[c];
    if (!(p & 0x80)) return vc;
    T nb = 0;
    if ((p & 1) && c - NJ >= 0) nb += v[c - NJ];
    if ((p & 2) && c + NJ < N) nb += v[c + NJ];
    if ((p & 4) && c - 1 >= 0) nb += v[c - 1];
    if ((p & 8) && c + 1 < N) nb += v[c + 1];
    return scale * ((T)((p >> 4) & 7) * vc - nb);
}

// ---------------------------------------------------------------------------
// FP64 outer residual r = b - A x, its FP32 copy and the block sums of r.r
// ---------------------------------------------------------------------------
__global__ void k_spec_residual(const uint8_t *__restrict__ info, const double *__restrict__ b,
                                const double *__restrict__ x, float *__restrict__ r32, long long N,
                                int NJ, double scale, double *__restrict__ partial,
                                const SpecCtl *ctl, const float *dt, double density, double dx)
{
    __shared__ double sm[32];
    if (ctl) {
        if (*((volatile const int *)&ctl->done)) return;
        scale = (double)*dt / (density * dx * dx);
    }
    double acc = 0.0;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < N;
         c += (long long)gridDim.x * blockDim.x) {
        const double r = b[c] - spec_a<double>(info, x, c, N, NJ, scale);
        r32[c] = (float)r;
        acc += r * r;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        double v = threadIdx.x < (blockDim.x >> 5) ? sm[threadIdx.x] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (threadIdx.x == 0) partial[blockIdx.x] = v;
    }
}

__global__ void k_spec_update(double *__restrict__ x, const float *__restrict__ d, long long N,
                              const SpecCtl *ctl)
{
    if (ctl && *((volatile const int *)&ctl->done)) return;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < N;
         c += (long long)gridDim.x * blockDim.x)
        x[c] += (double)d[c];
}

// the outer loop's decision: ||r||^2 from the residual partials (summed in a
// fixed order), ||b||^2 the first time, stop or the next inner tolerance
__global__ void k_spec_check(const double *__restrict__ partial, int nparts, SpecCtl *ctl, double tol,
                             int max_iter, int max_outer, int *iters_out, double *rel_out)
{
    __shared__ double sm[32];
    if (*((volatile const int *)&ctl->done)) return;
    double v = 0.0;
    for (int k = threadIdx.x; k < nparts; k += blockDim.x) v += partial[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double rr = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) rr += sm[w];
        if (ctl->outer == 0) ctl->bb = rr;
        const double bb = ctl->bb;
        ctl->rr = rr;
        const bool stop = bb == 0.0 || rr <= tol * tol * bb || ctl->total >= max_iter ||
                          ctl->outer >= max_outer || (ctl->outer > 0 && ctl->last_it == 0);
        // the inner solve needs to bring the residual just below the target
        // (never below what FP32 iterations reach)
        const double want = rr > 0.0 ? 0.3 * tol * sqrt(bb / rr) : 0.5;
        ctl->eps_in = (float)fmin(fmax(want, 1e-4), 0.5);
        ctl->outer++;
        if (stop) ctl->done = 1;
        if (iters_out) *iters_out = ctl->total;
        if (rel_out) *rel_out = bb > 0.0 ? sqrt(rr / bb) : 0.0;
    }
}

// ---------------------------------------------------------------------------
// inner FP32 PCG
// ---------------------------------------------------------------------------
__device__ __forceinline__ void spec_two_sum(float a, float b, float &s, float &e)
{
    s = a + b;
    const float bv = s - a;
    e = (a - (s - bv)) + (b - bv);
}
__device__ __forceinline__ float2 spec_ff_add(float2 a, float2 b)
{
    float s, e;
    spec_two_sum(a.x, b.x, s, e);
    e += a.y + b.y;
    const float h = s + e;
    return make_float2(h, e - (h - s));
}
__device__ __forceinline__ float2 spec_shfl(float2 v, int o)
{
    return make_float2(__shfl_down_sync(0xffffffffu, v.x, o), __shfl_down_sync(0xffffffffu, v.y, o));
}
__device__ __forceinline__ float spec_ff_div(float2 a, float2 b)
{
    const float q = __fdiv_rn(a.x, b.x);
    const float r = (fmaf(-q, b.x, a.x) + a.y) - q * b.y;
    return q + __fdiv_rn(r, b.x);
}

// block sums of two per-thread values as float pairs; results in thread 0
__device__ __forceinline__ void spec_bsum2(float v0, float v1, float2 *sm, float2 &o0, float2 &o1)
{
    float2 a = make_float2(v0, 0.f), b = make_float2(v1, 0.f);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a = spec_ff_add(a, spec_shfl(a, o));
        b = spec_ff_add(b, spec_shfl(b, o));
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) {
        sm[w] = a;
        sm[32 + w] = b;
    }
    __syncthreads();
    if (w == 0) {
        const bool in = lane < (int)(blockDim.x >> 5);
        a = in ? sm[lane] : make_float2(0.f, 0.f);
        b = in ? sm[32 + lane] : make_float2(0.f, 0.f);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            a = spec_ff_add(a, spec_shfl(a, o));
            b = spec_ff_add(b, spec_shfl(b, o));
        }
    }
    o0 = a;
    o1 = b;
    __syncthreads();
}

__device__ __forceinline__ unsigned spec_ld_acquire(const unsigned *p)
{
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

struct SpecGrid {
    unsigned *count; // monotonic arrival counter (zeroed at launch)
    int *status;
    unsigned n;      // barriers passed
};

// grid barrier: fence + relaxed add, then one thread polls the counter
__device__ __forceinline__ bool spec_sync(SpecGrid &g)
{
    __syncthreads();
    g.n++;
    if (threadIdx.x == 0) {
        asm volatile("fence.acq_rel.gpu;" ::: "memory");
        asm volatile("red.relaxed.gpu.global.add.u32 [%0], 1;" ::"l"(g.count) : "memory");
        const unsigned target = g.n * gridDim.x;
        long long spins = 0;
        while ((int)(spec_ld_acquire(g.count) - target) < 0) {
            if (++spins > kSpecSpin || ((spins & 1023) == 0 && *((volatile int *)g.status) != 0)) {
                atomicExch(g.status, 1);
                break;
            }
        }
    }
    __syncthreads();
    return *((volatile int *)g.status) == 0;
}

// every block sums the per-block float pairs in the same order
__device__ __forceinline__ float2 spec_psum(const float2 *p, int G, float2 *bc, int which)
{
    if (threadIdx.x < 32) {
        float2 a = make_float2(0.f, 0.f);
        for (int k = threadIdx.x; k < G; k += 32) a = spec_ff_add(a, __ldcg(p + k));
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) a = spec_ff_add(a, spec_shfl(a, o));
        if (threadIdx.x == 0) bc[which] = a;
    }
    __syncthreads();
    return bc[which];
}

// two blocks per SM (64 registers a thread) and four cells in flight per
// thread in every sweep: the sweeps stream vectors through L2 and HBM and are
// bound by how many loads are outstanding
__global__ void __launch_bounds__(kSpecThreads, 2) k_pcg_spec(SpecArgs a)
{
    __shared__ float2 sm[64];
    __shared__ float2 bc[4];
    const long long N = a.N;
    const int NJ = a.nj;
    const int G = gridDim.x;
    const long long stride = (long long)G * blockDim.x;
    const long long c0 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const float scale = a.dt ? (float)((double)*a.dt / (a.density * a.dx * a.dx)) : (float)a.scale;
    const uint8_t *__restrict__ info = a.info;
    float *__restrict__ r = a.r, *__restrict__ s = a.s, *__restrict__ q = a.q;
    float *__restrict__ z = a.z, *__restrict__ d = a.d;
    float2 *pA = a.partials, *pB = a.partials + G, *pC = a.partials + 2 * G;
    SpecGrid g{a.count, a.status, 0u};
    if (a.mode == 1 && *a.wrap_flag == 0) return; // the resident kernel solved it
    float eps_in = a.eps_in;
    int max_iter = a.max_iter;
    if (a.ctl) {
        // every block reads the same values before the first grid barrier;
        // block 0 writes the totals back only after the last one
        if (*((volatile const int *)&a.ctl->done)) return;
        eps_in = *((volatile const float *)&a.ctl->eps_in);
        max_iter = a.max_iter - *((volatile const int *)&a.ctl->total);
    }

    // y = K^T r
    auto kt = [&](long long n) {
        float v = r[n];
        const float k = spec_k(info[n], scale);
        if (n + NJ < N && (info[n + NJ] & 0x81) == 0x81) v = fmaf(k, r[n + NJ], v);
        if (n + 1 < N && (info[n + 1] & 0x84) == 0x84) v = fmaf(k, r[n + 1], v);
        return v;
    };
    // z = K K^T r in one pass: K^T r at c and at its upper and left
    // neighbours, combined in the order of z = K y (y = K^T r is not stored,
    // which saves a sweep and a grid barrier per iteration)
    auto kkt = [&](long long c) {
        const uint8_t p = info[c];
        float v = kt(c);
        if (p & 0x80) {
            if ((p & 1) && c - NJ >= 0) v = fmaf(spec_k(info[c - NJ], scale), kt(c - NJ), v);
            if ((p & 4) && c - 1 >= 0) v = fmaf(spec_k(info[c - 1], scale), kt(c - 1), v);
        }
        return v;
    };

    // f(c) for this thread's cells, four at a time (independent iterations
    // the compiler interleaves)
    auto sweep = [&](auto &&f) {
        for (long long cb = c0; cb < N; cb += 4 * stride) {
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const long long c = cb + u * stride;
                if (c < N) f(c);
            }
        }
    };

    // r_0 = the outer residual (already in r), d = 0, z = M r, s = z
    float rz = 0.f, rr = 0.f;
    sweep([&](long long c) {
        const float zc = kkt(c);
        d[c] = 0.f;
        z[c] = zc;
        s[c] = zc;
        rz = fmaf(r[c], zc, rz);
        rr = fmaf(r[c], r[c], rr);
    });
    {
        float2 b0, b1;
        spec_bsum2(rz, rr, sm, b0, b1);
        if (threadIdx.x == 0) {
            pA[blockIdx.x] = b0;
            pB[blockIdx.x] = b1;
        }
    }
    if (!spec_sync(g)) return;
    float2 sigma = spec_psum(pA, G, bc, 0);
    const float2 rr0 = spec_psum(pB, G, bc, 1);
    const float stop = eps_in * eps_in * rr0.x;
    int it = 0;
    bool first = true;
    float fb = 0.f;
    while (rr0.x > 0.f && it < max_iter) {
        // s = z + beta s, q = A s = A z + beta q, and s.q
        float sq = 0.f;
        sweep([&](long long c) {
            const float az = spec_a<float>(info, z, c, N, NJ, scale);
            const float sc = first ? z[c] : fmaf(fb, s[c], z[c]);
            const float qc = first ? az : fmaf(fb, q[c], az);
            s[c] = sc;
            q[c] = qc;
            sq = fmaf(sc, qc, sq);
        });
        {
            float2 b0, b1;
            spec_bsum2(sq, 0.f, sm, b0, b1);
            if (threadIdx.x == 0) pC[blockIdx.x] = b0;
        }
        if (!spec_sync(g)) return;
        const float fa = spec_ff_div(sigma, spec_psum(pC, G, bc, 2));
        sweep([&](long long c) {
            d[c] = fmaf(fa, s[c], d[c]);
            r[c] = fmaf(-fa, q[c], r[c]);
        });
        if (!spec_sync(g)) return;
        rz = 0.f;
        rr = 0.f;
        sweep([&](long long c) {
            const float zc = kkt(c);
            z[c] = zc;
            rz = fmaf(r[c], zc, rz);
            rr = fmaf(r[c], r[c], rr);
        });
        {
            float2 b0, b1;
            spec_bsum2(rz, rr, sm, b0, b1);
            if (threadIdx.x == 0) {
                pA[blockIdx.x] = b0;
                pB[blockIdx.x] = b1;
            }
        }
        if (!spec_sync(g)) return;
        it++;
        const float2 nsig = spec_psum(pA, G, bc, 0);
        const float2 nrr = spec_psum(pB, G, bc, 1);
        if (nrr.x <= stop) break;
        fb = spec_ff_div(nsig, sigma);
        sigma = nsig;
        first = false;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        if (a.iters) *a.iters = it;
        if (a.ctl) {
            a.ctl->total += it;
            a.ctl->last_it = it;
        }
    }
}

static int spec_grid()
{
    static std::atomic<int> slots[kMaxDevices];
    return device_cached(slots, [] { return occupancy_grid((const void *)k_pcg_spec, kSpecThreads, 1 << 30); });
}

int spec_partials_needed() { return 3 * spec_grid() + 8; }

int spec_chain_kernels(const SpecSolve &p)
{
    const bool res = p.res_ti > 0 && p.ll && p.wrap_flag;
    return (res ? 5 : 4) * p.max_outer + 2;
}

cudaError_t launch_spec_residual(const uint8_t *info, const double *b, const double *x, float *r32,
                                 long long N, int NJ, double scale, double *partial, int nblocks,
                                 cudaStream_t st)
{
    k_spec_residual<<<nblocks, 256, 0, st>>>(info, b, x, r32, N, NJ, scale, partial, nullptr, nullptr, 0.0,
                                             0.0);
    return cudaGetLastError();
}

cudaError_t launch_spec_update(double *x, const float *d, long long N, cudaStream_t st)
{
    const int blocks = (int)((N + 255) / 256 < 4096 ? (N + 255) / 256 : 4096);
    k_spec_update<<<blocks > 0 ? blocks : 1, 256, 0, st>>>(x, d, N, nullptr);
    return cudaGetLastError();
}

cudaError_t launch_spec_pcg(const SpecArgs &args, cudaStream_t st)
{
    SpecArgs a = args;
    const long long want = (a.N + kSpecThreads - 1) / kSpecThreads;
    int grid = spec_grid();
    if (want < grid) grid = (int)(want < 1 ? 1 : want);
    cudaError_t e = cudaMemsetAsync(a.count, 0, sizeof(unsigned), st);
    if (e != cudaSuccess) return e;
    void *kargs[] = {&a};
    return cudaLaunchCooperativeKernel((const void *)k_pcg_spec, dim3(grid), dim3(kSpecThreads), kargs,
                                       0, st);
}

cudaError_t launch_spec_chain(const SpecSolve &p, cudaStream_t st)
{
    const long long N = (long long)p.ni * p.nj;
    cudaError_t e = cudaMemsetAsync(p.ctl, 0, sizeof(SpecCtl), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(p.x, 0, (size_t)N * 8, st);
    if (e != cudaSuccess) return e;
    // the resident inner solves: one range of exchange-word epochs per
    // round, all taken now (a captured chain replays with the same epochs,
    // so it clears the words inside the capture and leaves them to be
    // cleared again before the next launch outside it)
    const bool res = p.res_ti > 0 && p.ll && p.wrap_flag;
    PcgArgs<float> ra{};
    const unsigned long long span = spec_resident_epochs(p.max_iter);
    if (res) {
        LlBuffers *ll = p.ll;
        if (!ll->r || !ll->s || !ll->rec || ll->words < (size_t)N) return cudaErrorInvalidValue;
        const unsigned long long need = span * (unsigned long long)(p.max_outer + 1);
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if ((e = cudaStreamIsCapturing(st, &cs)) != cudaSuccess) return e;
        const bool capturing = cs != cudaStreamCaptureStatusNone;
        if (capturing || ll->next == 0 || (unsigned long long)ll->next + need > 0xfffffff0ull) {
            e = cudaMemsetAsync(ll->r, 0, ll->words * sizeof(unsigned long long), st);
            if (e == cudaSuccess) e = cudaMemsetAsync(ll->s, 0, ll->words * sizeof(unsigned long long), st);
            if (e == cudaSuccess) e = cudaMemsetAsync(ll->rec, 0, kLlRecWords * sizeof(unsigned long long), st);
            if (e != cudaSuccess) return e;
            ll->next = 1;
        }
        ra.ni = p.ni;
        ra.nj = p.nj;
        ra.N = N;
        ra.info = p.info;
        ra.b = p.r;
        ra.x = p.d;
        ra.ll_r = ll->r;
        ra.ll_s = ll->s;
        ra.ll_rec = ll->rec;
        ra.ll_base = ll->next;
        ra.density = p.density;
        ra.dx = p.dx;
        ra.iter_limit = p.max_iter;
        ra.status = p.status;
        ra.wrap_flag = p.wrap_flag;
        ra.mode = 2; // unless a unit row touches a j edge
        ra.spec_ctl = p.ctl;
        ra.spec_dt = p.dt;
        ll->next = capturing ? 0u : (unsigned)(ll->next + need);
    }
    const int ublocks = (int)((N + 255) / 256 < 4096 ? (N + 255) / 256 : 4096);
    SpecArgs a{};
    a.ni = p.ni;
    a.nj = p.nj;
    a.N = N;
    a.info = p.info;
    a.r = p.r;
    a.d = p.d;
    a.s = p.s;
    a.q = p.q;
    a.y = nullptr;
    a.z = p.z;
    a.partials = p.partials;
    a.count = p.count;
    a.status = p.status;
    a.iters = nullptr;
    a.eps_in = 1e-4f;
    a.max_iter = p.max_iter;
    a.ctl = p.ctl;
    a.wrap_flag = p.wrap_flag;
    a.mode = res ? 1 : 0;
    for (int round = 0;; round++) {
        k_spec_residual<<<kSpecResBlocks, 256, 0, st>>>(p.info, p.b, p.x, p.r, N, p.nj, 0.0, p.rpart, p.ctl,
                                                        p.dt, p.density, p.dx);
        k_spec_check<<<1, 1024, 0, st>>>(p.rpart, kSpecResBlocks, p.ctl, p.tol, p.max_iter, p.max_outer,
                                         p.iters_out, p.rel_out);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        if (round == p.max_outer) break;
        a.dt = p.dt; // the scale from the device dt, like the residual
        a.density = p.density;
        a.dx = p.dx;
        if (res) {
            e = launch_spec_resident(ra, p.res_ti, p.res_tj, st);
            ra.ll_base += (unsigned)span;
        }
        if (e == cudaSuccess) e = launch_spec_pcg(a, st);
        if (e != cudaSuccess) return e;
        k_spec_update<<<ublocks > 0 ? ublocks : 1, 256, 0, st>>>(p.x, p.d, N, p.ctl);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

} // namespace fsg
