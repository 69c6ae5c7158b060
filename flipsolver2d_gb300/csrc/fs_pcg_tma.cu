// fs_pcg_tma.cu -- the FP32 pressure / density solve with TMA-staged tiles.
//
// Same algorithm and semantics as fs_pcg.cu (LinearSolver::solve,
// linearsolver.cpp:25-73, with the reference's operator and IPP rows), but
// every tile moves through the Tensor Memory Accelerator: one thread issues
// 2-D box copies global -> shared (cp.async.bulk.tensor, completion on an
// mbarrier), the boxes start two rows / four columns before the tile and
// the hardware fills cells outside the grid with zeros -- exactly the
// reference's treatment of indices outside the vector.  Tile results (s, r,
// x) are staged in shared memory and written back with TMA stores.  The
// threads only compute, mapped warp-per-row and lane-per-column.
//
// TMA rules respected here: boxes start at a column that is a multiple of
// 16 bytes (columns tj0 - 4 for floats, tj0 - 16 for the u8 operator rows,
// tj0 a multiple of 32), stores start inside the grid, row pitches are
// multiples of 16 bytes (NJ % 16 == 0, checked by the host, else the
// non-TMA kernel runs), shared destinations are 128-byte aligned.
//
// Cross-block visibility: a block's TMA stores are complete
// (cp.async.bulk.wait_group 0) and ordered for the generic and async proxies
// (fence.proxy.async) before it arrives at the grid barrier; after the barrier
// the loading thread fences again before issuing the next TMA loads.
#include <cfloat>
#include <initializer_list>
#include <map>
#include <mutex>
#include <utility>
#include <vector>
#include <cstdio>
#include <cuda.h>
#include <cudaTypedefs.h>

#include "fs_device.h"
#include "fs_pcg.h"
#include "fs_pcg_tma.h"
#include "fs_spec.h"

namespace fsg {

constexpr int kThreads = 1024;
constexpr int kStripThreads = 512;
constexpr int kMaxOwnedChunks = 64; // chunk ends a resident tile lists in shared memory
constexpr int kPartRounds = 8;      // per-lane partial loads: up to 256 resident blocks // resident kernel with register strips: 128 registers a thread
constexpr long long kSpinLimit = 1LL << 25; // default polls of a device wait: seconds

__device__ __forceinline__ unsigned smem_u32(const void *p)
{
    return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, unsigned parity)
{
    unsigned ok;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(smem_u32(bar)), "r"(parity)
                 : "memory");
    return ok != 0;
}
__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y,
                                            unsigned long long *bar)
{
    asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
                 " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
                 "l"(map), "r"(x), "r"(y), "r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ void tma_store_2d(const CUtensorMap *map, int x, int y, const void *src)
{
    asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%1, %2}], [%3];" ::"l"(map),
                 "r"(x), "r"(y), "r"(smem_u32(src))
                 : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void fence_async_shared() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fence_async_all() { asm volatile("fence.proxy.async;" ::: "memory"); }

__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e)
{
    s = a + b;
    const float bv = s - a;
    e = (a - (s - bv)) + (b - bv);
}

// Scalars of the iteration (dot products, alpha, beta) are carried as
// unevaluated float pairs (hi + lo, about 48 significant bits).  Double
// arithmetic would be simpler, but on this part every FP64 operation has a
// latency of a few hundred cycles, and the reductions and two divisions of
// an iteration sit on the critical path between grid barriers.
__device__ __forceinline__ float2 ff_add(float2 a, float2 b)
{
    float s, e;
    two_sum(a.x, b.x, s, e);
    e += a.y + b.y;
    const float h = s + e;
    return make_float2(h, e - (h - s));
}

__device__ __forceinline__ float2 ff_shfl_down(float2 v, int o)
{
    return make_float2(__shfl_down_sync(0xffffffffu, v.x, o), __shfl_down_sync(0xffffffffu, v.y, o));
}

// a / b rounded to float (error within about one float ulp)
__device__ __forceinline__ float ff_div(float2 a, float2 b)
{
    const float q = __fdiv_rn(a.x, b.x);
    const float r = (fmaf(-q, b.x, a.x) + a.y) - q * b.y;
    return q + __fdiv_rn(r, b.x);
}

// block sum of per-thread FP32 partials as a float pair; same value in every
// thread.  sm holds at least 36 float2.
__device__ __forceinline__ float2 bsum(float v, float2 *sm)
{
    float2 a = make_float2(v, 0.f);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) a = ff_add(a, ff_shfl_down(a, o));
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) sm[w] = a;
    __syncthreads();
    if (w == 0) {
        float2 x = lane < (int)(blockDim.x >> 5) ? sm[lane] : make_float2(0.f, 0.f);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x = ff_add(x, ff_shfl_down(x, o));
        if (lane == 0) sm[32] = x;
    }
    __syncthreads();
    const float2 r = sm[32];
    __syncthreads();
    return r;
}

// sum of the blocks' partials in a fixed order, so every block obtains the
// same value; read through L2 (other blocks wrote them)
__device__ __forceinline__ float2 psum(const float2 *partials, int nblocks, float2 *sm)
{
    if (threadIdx.x < 32) {
        float2 a = make_float2(0.f, 0.f);
        if (nblocks <= 32 * kPartRounds) {
            // issue every load before consuming any: one L2 round trip
            float2 v[kPartRounds];
#pragma unroll
            for (int i = 0; i < kPartRounds; i++) {
                const int k = (int)threadIdx.x + 32 * i;
                v[i] = k < nblocks ? __ldcg(partials + k) : make_float2(0.f, 0.f);
            }
#pragma unroll
            for (int i = 0; i < kPartRounds; i++) a = ff_add(a, v[i]);
        } else {
            for (int k = threadIdx.x; k < nblocks; k += 32) a = ff_add(a, __ldcg(partials + k));
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) a = ff_add(a, ff_shfl_down(a, o));
        if (threadIdx.x == 0) sm[34] = a;
    }
    __syncthreads();
    const float2 r = sm[34];
    __syncthreads();
    return r;
}

// The stopping test err <= tol of the reference (double) evaluated on float
// magnitudes: err is either the largest |r| found (a float) or, when no
// chunk holds a nonzero, DBL_MIN (VOps::maxAbs) or 0 (no chunks).
struct TolTest {
    float tf;     // largest float f with (double)f <= tol
    int min_ok;   // DBL_MIN <= tol
    int zero_ok;  // 0 <= tol
};

__device__ __forceinline__ TolTest tol_test(double tol)
{
    TolTest t;
    float f = (float)tol;
    if ((double)f > tol) f = nextafterf(f, -INFINITY);
    t.tf = f;
    t.min_ok = DBL_MIN <= tol;
    t.zero_ok = 0.0 <= tol;
    return t;
}

__device__ __forceinline__ bool tol_met(const TolTest &t, float mx, int has_min)
{
    if (mx > 0.f) return mx <= t.tf;
    return has_min ? t.min_ok : t.zero_ok;
}

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p)
{
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned atom_add_acq_rel(unsigned *p, unsigned v)
{
    unsigned old;
    asm volatile("atom.add.acq_rel.gpu.global.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}
__device__ __forceinline__ void st_release_u32(unsigned *p, unsigned v)
{
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Grid barrier with bounded spins.  Arrival is an acquire-release add on the
// counter (it publishes the block's writes, ordered before it by the block
// barrier); the last block resets the counter and releases the next
// generation, which the others acquire.  With async_proxy the block's TMA
// stores are complete and fenced for the generic proxy before it arrives.
__device__ __forceinline__ bool gsync(GridBarrier *gb, unsigned nblocks, int *status, long long lim,
                                      bool async_proxy = true)
{
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        if (async_proxy) {
            bulk_wait_all();
            fence_async_all();
        }
        const unsigned g = ld_acquire_u32(&gb->gen);
        const unsigned arrived = atom_add_acq_rel(&gb->count, 1u);
        if (arrived == nblocks - 1) {
            gb->count = 0;
            st_release_u32(&gb->gen, g + 1);
        } else {
            long long spins = 0;
            while (ld_acquire_u32(&gb->gen) == g) {
                ++spins;
                if (spins > lim ||
                    ((spins & 1023) == 0 && *((volatile int *)status) != 0)) {
                    atomicExch(status, 1);
                    break;
                }
            }
        }
        if (async_proxy) fence_async_all();
        // one verdict for the whole block (status can change between reads)
        s_ok = *((volatile int *)status) == 0;
    }
    __syncthreads();
    return s_ok != 0;
}

// VOps::maxAbs (vmath.cpp:100-136) with the reference's chunking, then the
// stopping test: the value of a chunk is |r| at its last nonzero entry.  The
// owner tile of each chunk's last unit row stored |r| there in chunk_val (or
// -1 when it is zero, then the chunk is scanned backwards here).  lastl(k):
// the last unit row of chunk k that r can reach (-1: none).
template <typename Load, typename LastLoad>
__device__ __forceinline__ bool chunk_converged(const PcgArgs<float> &a, Load rn, LastLoad lastl,
                                                const TolTest &tt, int *s_flag)
{
    __shared__ float s_mx[32];
    __shared__ int s_min[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const float *cv = reinterpret_cast<const float *>(a.chunk_val);
    // one warp per chunk; the max is order-independent
    float mx = 0.f;
    int has_min = 0;
    for (int k = warp; k < a.nchunks; k += nw) {
        const long long start = k == 0 ? 0 : a.chunk_end[k - 1];
        const int last = lastl(k);
        if (last < 0) {
            has_min = 1;
            continue;
        }
        float v = __ldcg(cv + k);
        if (v < 0.f) {
            const long long idx = warp_last_nonzero(start, (long long)last - 1, rn);
            if (idx >= start) {
                v = fabsf(rn(idx));
            } else {
                has_min = 1;
                v = 0.f;
            }
        }
        mx = fmaxf(mx, v);
    }
    if (lane == 0) {
        s_mx[warp] = mx;
        s_min[warp] = has_min;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < nw; w++) {
            mx = fmaxf(mx, s_mx[w]);
            has_min |= s_min[w];
        }
        *s_flag = tol_met(tt, mx, has_min) ? 1 : 0;
    }
    __syncthreads();
    const int f = *s_flag;
    __syncthreads();
    return f != 0;
}

// wait for the current TMA load batch.  After `lim` polls (or once another
// block reported a timeout) the solve is given up, but the block still waits
// -- bounded again -- for its own copies to land in its shared memory before
// it may leave.  Block-uniform result (a block barrier).
__device__ __forceinline__ bool load_wait(unsigned long long *bar, unsigned &phase, int *status,
                                          long long lim)
{
    long long spins = 0;
    bool failed = false;
    while (!mbar_try_wait(bar, phase & 1)) {
        ++spins;
        if (!failed && (spins > lim || *((volatile int *)status) != 0)) {
            atomicExch(status, 1);
            failed = true;
            spins = 0;
        }
        if (failed && spins > kSpinLimit) break; // a copy that never lands
    }
    phase++;
    return __syncthreads_or(failed) == 0;
}

struct SmemLayout {
    int ti, tj;
    int wr;  // columns of a float box: tj + 8
    int wi;  // columns of the u8 box: tj + 32
    int h2;  // rows of a box: ti + 4
    int w1, h1;
    size_t off_ib, off_rb, off_sb, off_b1, off_st, off_xb, bytes;
};

__host__ __device__ inline size_t a128(size_t x) { return (x + 127) & ~(size_t)127; }

__host__ __device__ inline SmemLayout smem_layout(int ti, int tj)
{
    SmemLayout L;
    L.ti = ti;
    L.tj = tj;
    L.wr = tj + 8;
    L.wi = tj + 32;
    L.h2 = ti + 4;
    L.w1 = tj + 2;
    L.h1 = ti + 2;
    size_t o = 0;
    L.off_ib = o;
    o = a128(o + (size_t)L.h2 * L.wi);
    L.off_rb = o;
    o = a128(o + (size_t)L.h2 * L.wr * 4);
    L.off_sb = o;
    o = a128(o + (size_t)L.h2 * L.wr * 4);
    L.off_b1 = o;
    o = a128(o + (size_t)L.h1 * L.w1 * 4);
    L.off_st = o;
    o = a128(o + (size_t)ti * tj * 4);
    L.off_xb = o;
    o = a128(o + (size_t)ti * tj * 4);
    L.bytes = o + 128; // + alignment slack
    return L;
}

// indices: a float box element (row r, col q) of the tile's halo coordinates
// (r in [-2, ti+2), q in [-4, tj+4)) lives at (r + 2) * wr + (q + 4); the u8
// box uses (r + 2) * wi + (q + 16)

__global__ void __launch_bounds__(kThreads, 1)
k_pcg_tma(PcgArgs<float> a, const __grid_constant__ TmaMaps m, int ti, int tj)
{
    const long long lim = a.spin_limit > 0 ? a.spin_limit : kSpinLimit;
    extern __shared__ unsigned char smem_dyn[];
    __shared__ float2 sm[40];
    __shared__ int s_flag;
    __shared__ __align__(8) unsigned long long bar;
    if (a.mode == 1 && *a.wrap_flag == 0) return;
    if (a.mode == 2 && *a.wrap_flag != 0) return;
    unsigned char *base = reinterpret_cast<unsigned char *>(
        ((size_t)smem_dyn + 127) & ~(size_t)127);
    const SmemLayout L = smem_layout(ti, tj);
    uint8_t *IB = base + L.off_ib;
    float *RB = reinterpret_cast<float *>(base + L.off_rb);
    float *SB = reinterpret_cast<float *>(base + L.off_sb);
    float *B1 = reinterpret_cast<float *>(base + L.off_b1);
    float *ST = reinterpret_cast<float *>(base + L.off_st);
    float *XB = reinterpret_cast<float *>(base + L.off_xb);
    const int NI = a.ni, NJ = a.nj;
    const int G = gridDim.x;
    const int tiles_j = (NJ + tj - 1) / tj, tiles_i = (NI + ti - 1) / ti;
    const int ntiles = tiles_i * tiles_j;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    float2 *pA = reinterpret_cast<float2 *>(a.partials), *pB = pA + G, *pC = pA + 2 * G;
    const TolTest tt = tol_test(a.tol);
    // 1e-8 added to the denominator of alpha, as a float pair
    const float2 eps8 = make_float2((float)1e-8, (float)(1e-8 - (double)(float)1e-8));
    const unsigned box_f = (unsigned)(L.h2 * L.wr * 4), box_i = (unsigned)(L.h2 * L.wi);
    const unsigned box_x = (unsigned)(ti * tj * 4);

    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    unsigned phase = 0;

    const double scale_d = pcg_scale(a);
    const float scale = (float)scale_d;
    __shared__ float inv[8];
    if (threadIdx.x < 8) inv[threadIdx.x] = (threadIdx.x >= 1 && threadIdx.x <= 4)
                                                ? (float)(1.0 / (threadIdx.x * scale_d)) : 0.f;

    // phase 0: sigma = b.b and the zero test (VOps::isZero, 1e-15)
    {
        const long long N = a.N;
        const long long per = ((N + G - 1) / G + blockDim.x - 1) / blockDim.x * blockDim.x;
        const long long lo = (long long)blockIdx.x * per;
        const long long hi = lo + per < N ? lo + per : N;
        float bb = 0.f;
        int nz = 0;
        for (long long c = lo + threadIdx.x; c < hi; c += blockDim.x) {
            const float bv = a.b[c];
            bb = fmaf(bv, bv, bb);
            nz |= fabsf(bv) > 1.0e-15f;
        }
        const float2 part = bsum(bb, sm);
        const int anynz = __syncthreads_or(nz);
        if (threadIdx.x == 0) {
            pA[blockIdx.x] = part;
            pC[blockIdx.x] = make_float2(anynz ? 1.f : 0.f, 0.f);
        }
    }
    if (!gsync(a.bar, G, a.status, lim)) return;
    float2 sigma = psum(pA, G, sm);
    if (psum(pC, G, sm).x == 0.f) {
        // the reference leaves result at zero
        for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < a.N;
             c += (long long)G * blockDim.x)
            a.x[c] = 0.f;
        if (blockIdx.x == 0 && threadIdx.x == 0) *a.iters_out = 0;
        return;
    }

    float fb = 0.f;
    int result = a.iter_limit;
    for (int it = 0; it < a.iter_limit; it++) {
        const bool first = it == 0;
        // r_it: b on the first iteration, then the ping-pong buffers
        const CUtensorMap *mr_cur = first ? &m.b : ((it & 1) ? &m.r1 : &m.r0);
        const CUtensorMap *ms_cur = first ? &m.b : ((it & 1) ? &m.s1 : &m.s0);
        // s_0 = b is never stored, so iteration 1 reads it from b
        const CUtensorMap *ms_prev = it == 1 ? &m.b : ((it & 1) ? &m.s0 : &m.s1);
        const CUtensorMap *ms_cur_st = (it & 1) ? &m.s1_st : &m.s0_st;
        const CUtensorMap *mr_next_st = (it & 1) ? &m.r0_st : &m.r1_st;

        // ---- sweep 1: s = M r + beta s_prev on the halo, q = A s, q.s ----
        float qs = 0.f;
        for (int t = blockIdx.x; t < ntiles; t += G) {
            const int ti0 = (t / tiles_j) * ti, tj0 = (t % tiles_j) * tj;
            if (threadIdx.x == 0) {
                bulk_wait_read(); // staging of an earlier store may still be read
                mbar_expect_tx(&bar, box_i + (first ? 0u : box_f) + box_f);
                tma_load_2d(IB, &m.info, tj0 - 16, ti0 - 2, &bar);
                if (!first) tma_load_2d(RB, mr_cur, tj0 - 4, ti0 - 2, &bar);
                tma_load_2d(SB, first ? ms_cur : ms_prev, tj0 - 4, ti0 - 2, &bar);
            }
            if (!load_wait(&bar, phase, a.status, lim)) return;
            // s on the tile and its 1-halo
            for (int r = warp; r < L.h1; r += nw) {
                const int rr = r - 1;
                for (int q = lane; q < L.w1; q += 32) {
                    const int qq = q - 1;
                    const int cf = (rr + 2) * L.wr + (qq + 4);
                    float s = SB[cf];
                    if (!first) {
                        const int ci = (rr + 2) * L.wi + (qq + 16);
                        const uint8_t ic = IB[ci];
                        float z = RB[cf];
                        if (ic & 0x80) {
                            const float iNeg = inv[(IB[ci - L.wi] >> 4) & 7];
                            const float iPos = inv[(IB[ci + L.wi] >> 4) & 7];
                            const float jNeg = inv[(IB[ci - 1] >> 4) & 7];
                            const float jPos = inv[(IB[ci + 1] >> 4) & 7];
                            const float diag = (1.f + iNeg * iNeg) + jNeg * jNeg;
                            float acc = diag * z;
                            acc = fmaf(jNeg, RB[cf - 1], acc);
                            acc = fmaf(jPos, RB[cf + 1], acc);
                            acc = fmaf(iNeg, RB[cf - L.wr], acc);
                            acc = fmaf(iPos, RB[cf + L.wr], acc);
                            z = acc;
                        }
                        s = fmaf(s, fb, z);
                    }
                    B1[r * L.w1 + q] = s;
                }
            }
            __syncthreads();
            // q = A s on the tile
            for (int r = warp; r < ti; r += nw) {
                for (int q = lane; q < tj; q += 32) {
                    const int c1 = (r + 1) * L.w1 + (q + 1);
                    const uint8_t ic = IB[(r + 2) * L.wi + (q + 16)];
                    const float s_c = B1[c1];
                    float qv = s_c;
                    if (ic & 0x80) {
                        float nb = 0.f;
                        if (ic & 1) nb += B1[c1 - L.w1];
                        if (ic & 2) nb += B1[c1 + L.w1];
                        if (ic & 4) nb += B1[c1 - 1];
                        if (ic & 8) nb += B1[c1 + 1];
                        qv = scale * ((float)((ic >> 4) & 7) * s_c - nb);
                    }
                    if (ti0 + r < NI && tj0 + q < NJ) qs = fmaf(qv, s_c, qs);
                    ST[r * tj + q] = s_c;
                }
            }
            if (!first) {
                fence_async_shared();
                __syncthreads();
                if (threadIdx.x == 0) {
                    tma_store_2d(ms_cur_st, tj0, ti0, ST);
                    bulk_commit();
                }
            }
            __syncthreads();
        }
        {
            const float2 part = bsum(qs, sm);
            if (threadIdx.x == 0) pA[blockIdx.x] = part;
        }
        if (!gsync(a.bar, G, a.status, lim)) return;
        const float fa = ff_div(sigma, ff_add(psum(pA, G, sm), eps8));

        // ---- sweep 2: r' = r - alpha A s on the halo, z = M r', x += alpha s
        float zr = 0.f;
        for (int t = blockIdx.x; t < ntiles; t += G) {
            const int ti0 = (t / tiles_j) * ti, tj0 = (t % tiles_j) * tj;
            if (threadIdx.x == 0) {
                bulk_wait_read();
                mbar_expect_tx(&bar, box_i + 2 * box_f + (first ? 0u : box_x));
                tma_load_2d(IB, &m.info, tj0 - 16, ti0 - 2, &bar);
                tma_load_2d(SB, ms_cur, tj0 - 4, ti0 - 2, &bar);
                tma_load_2d(RB, mr_cur, tj0 - 4, ti0 - 2, &bar);
                if (!first) tma_load_2d(XB, &m.x, tj0, ti0, &bar);
            }
            if (!load_wait(&bar, phase, a.status, lim)) return;
            // r' on the tile and its 1-halo
            for (int r = warp; r < L.h1; r += nw) {
                const int rr = r - 1;
                for (int q = lane; q < L.w1; q += 32) {
                    const int qq = q - 1;
                    const int cf = (rr + 2) * L.wr + (qq + 4);
                    const uint8_t ic = IB[(rr + 2) * L.wi + (qq + 16)];
                    const float s_c = SB[cf];
                    float qv = s_c;
                    if (ic & 0x80) {
                        float nb = 0.f;
                        if (ic & 1) nb += SB[cf - L.wr];
                        if (ic & 2) nb += SB[cf + L.wr];
                        if (ic & 4) nb += SB[cf - 1];
                        if (ic & 8) nb += SB[cf + 1];
                        qv = scale * ((float)((ic >> 4) & 7) * s_c - nb);
                    }
                    B1[r * L.w1 + q] = fmaf(-qv, fa, RB[cf]);
                }
            }
            __syncthreads();
            // z = M r', x += alpha s on the tile
            for (int r = warp; r < ti; r += nw) {
                for (int q = lane; q < tj; q += 32) {
                    const int c1 = (r + 1) * L.w1 + (q + 1);
                    const int ci = (r + 2) * L.wi + (q + 16);
                    const uint8_t ic = IB[ci];
                    const float r_c = B1[c1];
                    float z = r_c;
                    if (ic & 0x80) {
                        const float iNeg = inv[(IB[ci - L.wi] >> 4) & 7];
                        const float iPos = inv[(IB[ci + L.wi] >> 4) & 7];
                        const float jNeg = inv[(IB[ci - 1] >> 4) & 7];
                        const float jPos = inv[(IB[ci + 1] >> 4) & 7];
                        const float diag = (1.f + iNeg * iNeg) + jNeg * jNeg;
                        z = diag * r_c;
                        z = fmaf(jNeg, B1[c1 - 1], z);
                        z = fmaf(jPos, B1[c1 + 1], z);
                        z = fmaf(iNeg, B1[c1 - L.w1], z);
                        z = fmaf(iPos, B1[c1 + L.w1], z);
                    }
                    if (ti0 + r < NI && tj0 + q < NJ) zr = fmaf(z, r_c, zr);
                    const float s_c = SB[(r + 2) * L.wr + (q + 4)];
                    const float x_old = first ? 0.f : XB[r * tj + q];
                    XB[r * tj + q] = fmaf(s_c, fa, x_old);
                    ST[r * tj + q] = r_c;
                }
            }
            fence_async_shared();
            __syncthreads();
            if (threadIdx.x == 0) {
                tma_store_2d(&m.x, tj0, ti0, XB);
                tma_store_2d(mr_next_st, tj0, ti0, ST);
                bulk_commit();
            }
            // VOps::maxAbs (vmath.cpp:100-136): |r'| at each chunk's last unit
            // row, taken from the tile that computed it; -1 marks r' == 0
            for (int k = threadIdx.x; k < a.nchunks; k += blockDim.x) {
                const int idx = a.chunk_last_unit[k];
                if (idx < 0) continue;
                const int gi = idx / NJ, gj = idx - gi * NJ;
                if (gi < ti0 || gi >= ti0 + ti || gj < tj0 || gj >= tj0 + tj) continue;
                const float v = ST[(gi - ti0) * tj + (gj - tj0)];
                reinterpret_cast<float *>(a.chunk_val)[k] = v != 0.f ? fabsf(v) : -1.f;
            }
            __syncthreads();
        }
        {
            const float2 part = bsum(zr, sm);
            if (threadIdx.x == 0) pB[blockIdx.x] = part;
        }
        if (!gsync(a.bar, G, a.status, lim)) return;
        const float *rn = (it & 1) ? a.r0 : a.r1;
        const float2 newSigma = psum(pB, G, sm);
        if (chunk_converged(
                a, [&](long long e) { return __ldcg(rn + e); }, [&](int k) { return a.chunk_last_unit[k]; }, tt,
                &s_flag)) {
            result = it;
            break;
        }
        fb = ff_div(newSigma, sigma);
        sigma = newSigma;
    }
    if (threadIdx.x == 0) bulk_wait_all();
    if (blockIdx.x == 0 && threadIdx.x == 0) *a.iters_out = result;
}

// ---------------------------------------------------------------------------
// Shared-memory-resident variant: one tile per block for the whole solve.
// r, s (with a 2-cell halo), x and the operator rows live in shared memory;
// per sweep a block publishes its tile of the vector it just updated (plain
// stores, ping-pong buffers by iteration parity so a neighbour still reading
// the previous value is never overwritten) and, after the grid barrier,
// reads back only the 2-deep ring of neighbour cells around its tile.  Used
// when every tile fits one block and the tile count does not exceed the SMs.
// ---------------------------------------------------------------------------
struct ResLayout {
    int ti, tj, w2, h2, w1, h1, hp;
    size_t off_rb, off_sb, off_b1, off_xt, off_op, bytes;
};

// r and s with a 2-cell halo (h2 x w2), the sweep results on the tile and a
// 1-cell halo (h1 x w1), x on the tile, and a packed operator word per
// tile-plus-1-halo cell.  hp >= h1 pads the tile-plus-1-halo rows to whole
// register strips: rows h1 .. hp - 1 exist in Rb, Sb and the operator words
// so that strip loads need no bounds test.
__host__ __device__ inline ResLayout res_layout(int ti, int tj, int hp = 0)
{
    ResLayout L;
    L.ti = ti;
    L.tj = tj;
    L.w2 = tj + 4;
    L.w1 = tj + 2;
    L.h1 = ti + 2;
    L.hp = hp > L.h1 ? hp : L.h1;
    L.h2 = L.hp + 2;
    size_t o = 0;
    L.off_rb = o;
    o = a128(o + (size_t)L.h2 * L.w2 * 4);
    L.off_sb = o;
    o = a128(o + (size_t)L.h2 * L.w2 * 4);
    L.off_b1 = o; // also holds the operator bytes (h2 x w2) during set-up
    const size_t b1 = (size_t)L.h1 * L.w1 * 4, ib = (size_t)L.h2 * L.w2;
    o = a128(o + (b1 > ib ? b1 : ib));
    L.off_xt = o;
    o = a128(o + (size_t)ti * tj * 4);
    L.off_op = o;
    o = a128(o + (size_t)L.hp * L.w1 * 4);
    L.bytes = o + 128;
    return L;
}

// the k-th cell of the 2-deep ring around a tile, in halo coordinates
__device__ __forceinline__ void ring_cell(int k, int ti, int tj, int &r, int &q)
{
    const int w2 = tj + 4;
    if (k < 2 * w2) { // two rows above
        r = k / w2 - 2;
        q = k % w2 - 2;
        return;
    }
    k -= 2 * w2;
    if (k < 2 * w2) { // two rows below
        r = ti + k / w2;
        q = k % w2 - 2;
        return;
    }
    k -= 2 * w2;
    r = k >> 2; // ti rows x 4 side cells
    const int s = k & 3;
    q = s < 2 ? s - 2 : tj + (s - 2);
}

__device__ __forceinline__ void load_ring(float *dst, const float *__restrict__ src, int ti0,
                                          int tj0, int ti, int tj, int NI, int NJ)
{
    const int w2 = tj + 4;
    const int n = 4 * w2 + 4 * ti;
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        int r, q;
        ring_cell(k, ti, tj, r, q);
        const int gi = ti0 + r, gj = tj0 + q;
        float v = 0.f;
        if (gi >= 0 && gi < NI && gj >= 0 && gj < NJ) v = __ldcg(src + (size_t)gi * NJ + gj);
        dst[(r + 2) * w2 + (q + 2)] = v;
    }
}

// ---------------------------------------------------------------------------
// Exchange words.  The resident kernel moves everything another block reads
// -- the per-block partials of the two grid reductions and the 2-cell bands
// along tile borders -- as 8-byte words that hold a 32-bit payload and the
// epoch that published it.  An aligned 8-byte access is single-copy atomic,
// so a reader that sees the epoch it expects also sees that epoch's payload:
// no fence, no separate flag and no counter round trip is needed.  Epochs
// only grow across the launches that share a buffer (the host hands each
// launch a fresh range), so a word left by an earlier launch never matches.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long ll_pack(unsigned payload, unsigned epoch)
{
    return ((unsigned long long)epoch << 32) | payload;
}
__device__ __forceinline__ unsigned ll_epoch(unsigned long long w) { return (unsigned)(w >> 32); }
__device__ __forceinline__ void st_ll(unsigned long long *p, unsigned long long w)
{
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(w) : "memory");
}
__device__ __forceinline__ void st_ll2(unsigned long long *p, unsigned long long a, unsigned long long b)
{
    asm volatile("st.relaxed.gpu.global.v2.u64 [%0], {%1, %2};" ::"l"(p), "l"(a), "l"(b) : "memory");
}
__device__ __forceinline__ unsigned long long ld_ll(const unsigned long long *p)
{
    unsigned long long w;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(w) : "l"(p) : "memory");
    return w;
}
__device__ __forceinline__ void ld_ll2(const unsigned long long *p, unsigned long long &a,
                                       unsigned long long &b)
{
    asm volatile("ld.relaxed.gpu.global.v2.u64 {%0, %1}, [%2];" : "=l"(a), "=l"(b) : "l"(p) : "memory");
}

// words of one block's partial record: hi, lo of a float-pair sum, then a
// word whose low 31 bits are a non-negative float (a max) and whose top bit
// is a flag (an OR), then one unused word (spec mode: a second pair).  Each
// record has a 128-byte line to itself: every block polls every record, and
// with four records a line (32 bytes each) the polls of a line's four
// readers-by-152 slowed the publishes into it -- measured on GB300, the
// padded layout took the 1024^2 solves from 4.95 to 4.51 ms per substep and
// the 256^2 ones from 3.43 to 2.5 ms, bit-identical
constexpr int kRecWords = 16;

// reduction k of a launch uses set k & 1 of two sets of G records
static_assert(kRecWords * 2 * 256 == (int)kLlRecSets, "record buffer");

// float-pair accumulation without renormalising: hi carries the running
// sum, lo the rounding errors of the additions and the low parts
__device__ __forceinline__ float2 ff_acc(float2 a, float2 b)
{
    float s, e;
    two_sum(a.x, b.x, s, e);
    return make_float2(s, (a.y + b.y) + e);
}
__device__ __forceinline__ float2 ff_norm(float2 a)
{
    const float h = a.x + a.y;
    return make_float2(h, a.y - (h - a.x));
}

// Block sum of per-thread FP32 partials as a float pair, valid in thread 0
// only.  The caller orders the next use of sm (64 floats) with a block
// barrier.  (Plain float sums inside the warps were measured to let the
// unconverged 200-iteration solves drift visibly further from FP64.)
__device__ __forceinline__ float2 bsum0(float v, float *sm)
{
    float2 a0 = make_float2(v, 0.f);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) a0 = ff_acc(a0, ff_shfl_down(a0, o));
    a0 = ff_norm(a0);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) {
        sm[2 * w] = a0.x;
        sm[2 * w + 1] = a0.y;
    }
    __syncthreads();
    float2 x = make_float2(0.f, 0.f);
    if (w == 0) {
        x = lane < (int)(blockDim.x >> 5) ? make_float2(sm[2 * lane], sm[2 * lane + 1])
                                          : make_float2(0.f, 0.f);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x = ff_acc(x, ff_shfl_down(x, o));
        x = ff_norm(x);
    }
    return x;
}

// bsum0 of two values at once (sm: 4 floats a warp, at most 16 warps)
__device__ __forceinline__ void bsum0_2(float v0, float v1, float *sm, float2 &o0, float2 &o1)
{
    float2 a0 = make_float2(v0, 0.f), a1 = make_float2(v1, 0.f);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a0 = ff_acc(a0, ff_shfl_down(a0, o));
        a1 = ff_acc(a1, ff_shfl_down(a1, o));
    }
    a0 = ff_norm(a0);
    a1 = ff_norm(a1);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) {
        sm[4 * w] = a0.x;
        sm[4 * w + 1] = a0.y;
        sm[4 * w + 2] = a1.x;
        sm[4 * w + 3] = a1.y;
    }
    __syncthreads();
    o0 = o1 = make_float2(0.f, 0.f);
    if (w == 0) {
        const bool in = lane < (int)(blockDim.x >> 5);
        float2 x0 = in ? make_float2(sm[4 * lane], sm[4 * lane + 1]) : make_float2(0.f, 0.f);
        float2 x1 = in ? make_float2(sm[4 * lane + 2], sm[4 * lane + 3]) : make_float2(0.f, 0.f);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            x0 = ff_acc(x0, ff_shfl_down(x0, o));
            x1 = ff_acc(x1, ff_shfl_down(x1, o));
        }
        o0 = ff_norm(x0);
        o1 = ff_norm(x1);
    }
}

__device__ __forceinline__ unsigned ld_relaxed_u32(const unsigned *p)
{
    unsigned v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed_u32(unsigned *p, unsigned v)
{
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void red_relaxed_add(unsigned *p, unsigned v)
{
    asm volatile("red.relaxed.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void fence_acq_rel_gpu() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }

// Bounded spin of one thread until *p >= target (acquire); false on timeout
// or when another block reported one.
__device__ __forceinline__ bool spin_until(const unsigned *p, unsigned target, int *status,
                                           long long lim)
{
    long long spins = 0;
    while ((int)(ld_acquire_u32(p) - target) < 0) {
        ++spins;
        if (spins > lim || ((spins & 1023) == 0 && *((volatile int *)status) != 0)) {
            atomicExch(status, 1);
            return false;
        }
    }
    return true;
}

// Runs f(r, q) over the h1 x w1 tile-plus-1-halo region: warps take rows and
// lanes the interior columns, then the two halo columns of every row go out
// to all threads in one pass (instead of a nearly idle extra pass per row).
template <typename F>
__device__ __forceinline__ void for_halo1(int h1, int w1, F f)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int r = warp; r < h1; r += nw)
        for (int q = lane + 1; q < w1 - 1; q += 32) f(r, q);
    for (int k = threadIdx.x; k < 2 * h1; k += blockDim.x) f(k >> 1, (k & 1) ? w1 - 1 : 0);
}

// z = M v at one cell from its value and its four neighbours' values, for
// operator word p (IncompletePoissonPreconditioner with the reference's
// asymmetric rows); branch-free so that every tile costs the same whatever
// its fluid fraction.  inv[n] = 1 / (n scale) for n = 1..4, else 0.
__device__ __forceinline__ float ipp_apply(unsigned p, const float *inv, float vc, float up, float dn,
                                           float lf, float rt)
{
    const float iNeg = inv[(p >> 8) & 7];
    const float iPos = inv[(p >> 11) & 7];
    const float jNeg = inv[(p >> 14) & 7];
    const float jPos = inv[(p >> 17) & 7];
    const float diag = (1.f + iNeg * iNeg) + jNeg * jNeg;
    float acc = diag * vc;
    acc = fmaf(jNeg, lf, acc);
    acc = fmaf(jPos, rt, acc);
    acc = fmaf(iNeg, up, acc);
    acc = fmaf(iPos, dn, acc);
    return (p & 0x80) ? acc : vc;
}

// z = K K^T v at one cell, the textbook incomplete-Poisson preconditioner of
// the spec-mode solve (inversepoissonpreconditioner.h:45-79: K = I - L D^-1,
// L the strictly lower part of the pressure matrix, D its diagonal), from
// the cell's value and six neighbours' (down, right, up, up-right, left,
// down-left).  y = K^T v at the cell and at its upper and left neighbours,
// then z = K y, each combined in the order the linear-index form evaluates
// it.  Operator word p (the spec packing):
//   bits 0-7   the cell's own operator byte
//   bit 8      the cell below is a unit row whose upper neighbour is fluid
//   bit 9      the cell to the right is a unit row whose left neighbour is fluid
//   bits 10-12 K code of the upper neighbour, bit 13 its bit 9
//   bits 14-16 K code of the left neighbour, bit 17 its bit 8
// K code: the non-solid count of a unit row with one, else 0; kk[code] is
// 1 / count, or the operator's scale for code 0 (Eigen's zero-diagonal rule
// on an identity row).
__device__ __forceinline__ float kkt_apply(unsigned p, const float *kk, float vc, float dn, float rt,
                                           float up, float ur, float lf, float dl)
{
    const float kc = kk[(p & 0x80) ? ((p >> 4) & 7) : 0];
    const float ku = kk[(p >> 10) & 7], kl = kk[(p >> 14) & 7];
    const bool up_in = (p & 0x81) == 0x81; // unit row, upper neighbour fluid
    const bool lf_in = (p & 0x84) == 0x84; // unit row, left neighbour fluid
    float yc = vc;
    yc = (p & 0x100) ? fmaf(kc, dn, yc) : yc;
    yc = (p & 0x200) ? fmaf(kc, rt, yc) : yc;
    float yu = up;
    yu = up_in ? fmaf(ku, vc, yu) : yu;
    yu = (p & 0x2000) ? fmaf(ku, ur, yu) : yu;
    float yl = lf;
    yl = (p & 0x20000) ? fmaf(kl, dl, yl) : yl;
    yl = lf_in ? fmaf(kl, vc, yl) : yl;
    float z = yc;
    z = up_in ? fmaf(ku, yu, z) : z;
    z = lf_in ? fmaf(kl, yl, z) : z;
    return z;
}

// (A v) at one cell (the pressure matrix row; identity on non-unit rows)
__device__ __forceinline__ float op_apply(unsigned p, float scale, float vc, float up, float dn,
                                          float lf, float rt)
{
    float nb = (p & 1) ? up : 0.f;
    nb += (p & 2) ? dn : 0.f;
    nb += (p & 4) ? lf : 0.f;
    nb += (p & 8) ? rt : 0.f;
    const float av = scale * ((float)((p >> 4) & 7) * vc - nb);
    return (p & 0x80) ? av : vc;
}

// ---------------------------------------------------------------------------
// The resident kernel.  Synchronisation, all by thread 0 of a block after a
// block barrier:
//  * a grid barrier is a monotonic arrival counter: fence.acq_rel, then a
//    relaxed reduction-add (fire and forget); barrier k is complete when the
//    counter reads G k (acquire).  The counter is zeroed at launch.
//  * a block publishes each vector it stores with an epoch flag (relaxed
//    store after the same fence); neighbours whose halo ring reads that
//    vector wait for the flag instead of the grid barrier.
// Iteration it publishes s_it as epoch 2 it + 1 and r_{it+1} as 2 it + 2.
//
// RPS = 0: every sweep reads and writes the shared-memory arrays.
// RPS > 0 (register strips): warp w owns columns 32 (w % G) .. +31 of the
// tile (G = tj / 32 column groups) and a strip of at most RPS consecutive rows
// of the tile-plus-1-halo region; each thread keeps r, s and the operator
// words of its strip in registers, so only horizontal neighbours and the rows
// just outside its strip come from shared memory.  The two halo columns are
// computed from shared memory by a few threads per warp.  Every cell, strip
// or halo, goes through the same ipp_apply / op_apply, so values that two
// tiles both compute agree bit for bit.
// ---------------------------------------------------------------------------
template <int RPS, bool SPEC>
__global__ void __launch_bounds__(RPS > 0 ? kStripThreads : kThreads, 1)
k_pcg_resident(PcgArgs<float> a, int ti, int tj)
{
    static_assert(!SPEC || RPS > 0, "spec-mode solves run on register strips");
    const long long lim = a.spin_limit > 0 ? a.spin_limit : kSpinLimit;
    extern __shared__ unsigned char smem_dyn[];
    __shared__ float smf[64];
    __shared__ float4 s_gw[8]; // per-warp sums of a reduction's records
    __shared__ int s_gwf[8];   // and whether that warp's wait gave up
    __shared__ int s_flag;
    __shared__ float inv[8];
    __shared__ int s_cmax, s_cscan;
    __shared__ int s_nown;           // chunks whose last unit row is in this tile
    __shared__ int2 s_own[kMaxOwnedChunks]; // (chunk, Rb index)
    if (a.mode == 1 && *a.wrap_flag == 0) return;
    if (a.mode == 2 && *a.wrap_flag != 0) return;
    // spec mode: the chained solve's state, read by every block before any
    // block publishes (block 0 writes the totals back only after the last
    // reduction, which every block has joined)
    int iter_limit = a.iter_limit;
    float eps_in = 0.f;
    if constexpr (SPEC) {
        if (*((volatile const int *)&a.spec_ctl->done)) return;
        eps_in = *((volatile const float *)&a.spec_ctl->eps_in);
        iter_limit = a.iter_limit - *((volatile const int *)&a.spec_ctl->total);
    }
    if (threadIdx.x == 0) s_nown = 0; // ordered before its use by the set-up barriers
    // no TMA here, so the 16-byte alignment of dynamic shared memory is
    // enough; indexing smem_dyn directly keeps the accesses in the shared
    // window (32-bit addresses, LDS/STS)
    unsigned char *base = smem_dyn;
    // register strips: warp w owns column group w % ngrp and strip w / ngrp
    constexpr int kR = RPS > 0 ? RPS : 1;
    const int ngrp = tj >> 5;
    const int nstrips = (int)(blockDim.x >> 5) / ngrp;
    const ResLayout L = res_layout(ti, tj, RPS > 0 ? nstrips * RPS : 0);
    float *Rb = reinterpret_cast<float *>(base + L.off_rb);
    float *Sb = reinterpret_cast<float *>(base + L.off_sb);
    float *B1 = reinterpret_cast<float *>(base + L.off_b1);
    float *Xt = reinterpret_cast<float *>(base + L.off_xt);
    unsigned *Op = reinterpret_cast<unsigned *>(base + L.off_op);
    const int NI = a.ni, NJ = a.nj;
    const int G = gridDim.x;
    const int tiles_j = (NJ + tj - 1) / tj;
    const int ti0 = ((int)blockIdx.x / tiles_j) * ti, tj0 = ((int)blockIdx.x % tiles_j) * tj;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int w2 = L.w2, w1 = L.w1, h1 = L.h1;
    // partial records of the grid reductions (exchange words, two sets of G
    // records); reduction k of this launch has epoch ep0 + 1 + k
    unsigned long long *recs = a.ll_rec;
    const unsigned ep0 = a.ll_base;
    unsigned nred = 0;                // reductions published so far
    unsigned *count = SPEC ? nullptr : &a.bar->count; // arrivals at the rare fenced barrier
    unsigned nfenced = 0;
    // chunks without a unit row report DBL_MIN (VOps::maxAbs) on every iteration
    int has_min_static = 0;
    for (int k = 0; k < a.nchunks; k++) has_min_static |= a.chunk_last_unit[k] < 0;
    // Live chunk ends: a unit row whose b is zero, in a fluid component of
    // at most four cells that all have b = 0 and whose non-fluid neighbours
    // have b = 0 (a small droplet), keeps r exactly zero through every
    // iteration (A s, z = M r and s there only combine zeros).  The max-abs value of a chunk -- |r| at its last nonzero
    // entry -- therefore never comes from such a row, and its last live unit
    // row serves as the chunk's end: a flying droplet at the end of a chunk
    // no longer sends every iteration to the backward search.  Per launch,
    // the largest live index per chunk as (epoch << 32 | index + 1).
    unsigned long long *effw = a.ll_rec + kLlEffOff;
    const bool eff = !SPEC && a.nchunks > 0 && a.nchunks <= (int)kLlMaxChunks;
    auto last_unit = [&](int k) -> int {
        if (!eff) return a.chunk_last_unit[k];
        const unsigned long long w = __ldcg(effw + k);
        return (unsigned)(w >> 32) == ep0 ? (int)(unsigned)w - 1 : -1;
    };
    const TolTest tt = tol_test(a.tol);
    const float2 eps8 = make_float2((float)1e-8, (float)(1e-8 - (double)(float)1e-8));

    const double scale_d = SPEC ? (double)*a.spec_dt / (a.density * a.dx * a.dx) : pcg_scale(a);
    const float scale = (float)scale_d;
    // the preconditioner's coefficients by neighbour count: IPP 1 / (n
    // scale); spec mode the K table (1 / n, the scale for code 0)
    if (threadIdx.x < 8) {
        const int n = (int)threadIdx.x;
        if constexpr (SPEC)
            inv[n] = n == 0 ? scale : (n <= 4 ? 1.f / (float)n : 0.f);
        else
            inv[n] = (n >= 1 && n <= 4) ? (float)(1.0 / (n * scale_d)) : 0.f;
    }

    // thread 0, holding the block's partial (hi, lo) and the extra word:
    // publish them as this block's record of the next reduction.  Every
    // thread counts the reduction.
    // (Spec mode: a second pair, r.r, in the last two words.)
    auto publish = [&](float2 part, unsigned extra, float2 part2 = make_float2(0.f, 0.f)) {
        if (threadIdx.x == 0) {
            const unsigned ep = ep0 + 1 + nred;
            unsigned long long *r = recs + ((size_t)(nred & 1) * G + blockIdx.x) * kRecWords;
            st_ll2(r, ll_pack(__float_as_uint(part.x), ep), ll_pack(__float_as_uint(part.y), ep));
            if constexpr (SPEC)
                st_ll2(r + 2, ll_pack(__float_as_uint(part2.x), ep), ll_pack(__float_as_uint(part2.y), ep));
            else
                st_ll(r + 2, ll_pack(extra, ep));
        }
        nred++;
    };
    bool gfail = false; // the last wait_sum gave up (the same in every thread)
    // completes the last reduction published: warp w gathers records
    // 32 w .. 32 w + 31 (one per lane; the G <= 256 records take at most 8
    // warps, whose loads are all in flight at once), sums them in a fixed
    // order (a shuffle tree per warp, then the warps in order), so every
    // block obtains the same scalars: (pair hi, lo, max, flag) in every
    // thread.  gfail, read after it, is block-uniform: true after a timeout.
    // (One warp polling all G records, several per lane, took 4-5 us from
    // the last block's publish to completion at 1024^2; a lane per record
    // and a warp per 32 records take under 1 us.)
    float fa_prev = 0.f; // alpha of the last iteration
    auto wait_sum = [&](bool with_x) -> float4 {
        const unsigned k = nred - 1, ep = ep0 + nred;
        const int ngw = (G + 31) >> 5;
        if (warp >= ngw && with_x) {
            if constexpr (RPS > 0) {
                // x += alpha s of the last iteration (s is still in Sb): the
                // warps that gather no records do it while the others poll
                const int nx = nw - ngw;
                for (int r = warp - ngw; r < ti; r += nx)
                    for (int q = lane; q < tj; q += 32)
                        Xt[r * tj + q] = fmaf(Sb[(r + 2) * w2 + (q + 2)], fa_prev, Xt[r * tj + q]);
            }
        }
        if (warp < ngw) {
            const unsigned long long *base = recs + (size_t)(k & 1) * G * kRecWords;
            const int b = warp * 32 + lane;
            unsigned long long w0 = 0ull, w1 = 0ull, w2 = 0ull, w3 = 0ull;
            bool failed = false;
            if (b < G) {
                const unsigned long long *rp = base + (size_t)b * kRecWords;
                auto load = [&]() {
                    ld_ll2(rp, w0, w1);
                    if constexpr (SPEC) ld_ll2(rp + 2, w2, w3);
                    else w2 = ld_ll(rp + 2);
                };
                load();
                long long spins = 0;
                while (ll_epoch(w0) != ep || ll_epoch(w1) != ep || ll_epoch(w2) != ep ||
                       (SPEC && ll_epoch(w3) != ep)) {
                    if (++spins > lim || ((spins & 255) == 0 && *((volatile int *)a.status) != 0)) {
                        atomicExch(a.status, 1);
                        failed = true;
                        break;
                    }
                    load();
                }
            }
            // records past G are zeros: adding them changes nothing
            float2 acc = make_float2(__uint_as_float((unsigned)w0), __uint_as_float((unsigned)w1));
            float4 gw;
            if constexpr (SPEC) {
                float2 acc2 = make_float2(__uint_as_float((unsigned)w2), __uint_as_float((unsigned)w3));
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    acc = ff_acc(acc, ff_shfl_down(acc, o));
                    acc2 = ff_acc(acc2, ff_shfl_down(acc2, o));
                }
                gw = make_float4(acc.x, acc.y, acc2.x, acc2.y);
            } else {
                float mx = __uint_as_float((unsigned)w2 & 0x7fffffffu);
                unsigned flag = (unsigned)w2 >> 31;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    acc = ff_acc(acc, ff_shfl_down(acc, o));
                    mx = fmaxf(mx, __shfl_down_sync(0xffffffffu, mx, o));
                    flag |= __shfl_down_sync(0xffffffffu, flag, o);
                }
                gw = make_float4(acc.x, acc.y, mx, flag ? 1.f : 0.f);
            }
            failed = __any_sync(0xffffffffu, failed);
            if (lane == 0) {
                s_gw[warp] = gw;
                s_gwf[warp] = (failed || *((volatile int *)a.status) != 0) ? 1 : 0;
            }
        }
        __syncthreads();
        // every thread adds the warps' sums in the same fixed order: the same
        // bits everywhere, with no second barrier.  (The next writes of s_gw
        // come after at least one more block barrier.)
        float2 acc = make_float2(0.f, 0.f), acc2 = make_float2(0.f, 0.f);
        float mx = 0.f, flag = 0.f;
        int failed = 0;
        for (int w = 0; w < ngw; w++) {
            const float4 g = s_gw[w];
            acc = ff_acc(acc, make_float2(g.x, g.y));
            if constexpr (SPEC) {
                acc2 = ff_acc(acc2, make_float2(g.z, g.w));
            } else {
                mx = fmaxf(mx, g.z);
                flag = fmaxf(flag, g.w);
            }
            failed |= s_gwf[w];
        }
        gfail = failed != 0;
        acc = ff_norm(acc);
        if constexpr (SPEC) {
            acc2 = ff_norm(acc2);
            return make_float4(acc.x, acc.y, acc2.x, acc2.y); // the two pairs
        }
        return make_float4(acc.x, acc.y, mx, flag);
    };
    // block-uniform: no wait of this launch has timed out (a block barrier)
    auto ok = [&]() { return __syncthreads_or(*((volatile int *)a.status) != 0) == 0; };
    // the rare full barrier with release / acquire semantics (the backward
    // max-abs scan reads r anywhere and the chunk-end values of all tiles)
    auto fenced_barrier = [&]() -> bool {
        __syncthreads();
        nfenced++;
        if (threadIdx.x == 0) {
            fence_acq_rel_gpu();
            red_relaxed_add(count, 1u);
            spin_until(count, nfenced * (unsigned)G, a.status, lim);
        }
        return ok();
    };

    // load the operator rows (bytes, into B1 for now) and r_0 = s_0 = b with
    // their halo; x = 0
    uint8_t *Ib = reinterpret_cast<uint8_t *>(B1); // h2*w2 bytes fit in h1*w1 floats
    float bb = 0.f;
    int nz = 0;
    for (int r = warp; r < L.h2; r += nw) {
        const int gi = ti0 - 2 + r;
        for (int q = lane; q < w2; q += 32) {
            const int gj = tj0 - 2 + q;
            const bool inb = gi >= 0 && gi < NI && gj >= 0 && gj < NJ;
            const size_t g = (size_t)gi * NJ + gj;
            const float bv = inb ? a.b[g] : 0.f;
            Rb[r * w2 + q] = bv;
            Sb[r * w2 + q] = bv;
            Ib[r * w2 + q] = inb ? a.info[g] : (uint8_t)0;
            const bool own = r >= 2 && r < ti + 2 && q >= 2 && q < tj + 2 && inb;
            if (own) {
                bb = fmaf(bv, bv, bb);
                nz |= fabsf(bv) > 1.0e-15f;
            }
        }
    }
    for (int e = threadIdx.x; e < ti * tj; e += blockDim.x) Xt[e] = 0.f;
    __syncthreads();
    // the chunk ends this tile owns, listed once (more than kMaxOwnedChunks,
    // possible only with tiny chunks, falls back to a scan of all chunks)
    auto list_owned = [&]() {
        for (int k = threadIdx.x; k < a.nchunks; k += blockDim.x) {
            const int idx = last_unit(k);
            if (idx < 0) continue;
            const int gi = idx / NJ, gj = idx - gi * NJ;
            if (gi < ti0 || gi >= ti0 + ti || gj < tj0 || gj >= tj0 + tj) continue;
            const int slot = atomicAdd(&s_nown, 1);
            if (slot < kMaxOwnedChunks) s_own[slot] = make_int2(k, (gi - ti0 + 2) * w2 + (gj - tj0 + 2));
        }
    };
    if (!eff) {
        list_owned();
    } else {
        // this tile's live unit rows: per row segment, the highest live
        // lane of each chunk; a warp keeps its running maximum per chunk and
        // folds it into the chunk's word when the chunk changes
        auto chunk_index = [&](long long e) { // the first chunk whose end exceeds e
            int lo = 0, hi = a.nchunks - 1;
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (a.chunk_end[mid] > e) hi = mid;
                else lo = mid + 1;
            }
            return lo;
        };
        // A unit row with b = 0 whose fluid component has at most kDeadCells
        // cells, all with b = 0, and whose non-fluid neighbours hold b = 0 as
        // well: r, s and z stay exactly zero there (the operator couples it
        // only to the component; M also reads the non-fluid neighbours, whose
        // identity rows keep r = b = 0).  A small flood over the operator
        // bytes and b in global memory (set-up only).
        constexpr int kDeadCells = 4;
        auto dead_unit = [&](int e0) -> bool {
            int comp[kDeadCells];
            int n = 0;
            comp[n++] = e0;
            for (int k = 0; k < n; k++) {
                const int e = comp[k];
                const int ei = e / NJ, ej = e - ei * NJ;
                const unsigned p = __ldg(a.info + e);
                const int nbr[4] = {e - NJ, e + NJ, e - 1, e + 1};
                const bool in[4] = {ei > 0, ei < NI - 1, ej > 0, ej < NJ - 1};
#pragma unroll
                for (int t = 0; t < 4; t++) {
                    if (!in[t]) continue;
                    const int f = nbr[t];
                    if (p & (1u << t)) { // a fluid neighbour: part of the component
                        bool seen = false;
                        for (int u = 0; u < n; u++) seen |= comp[u] == f;
                        if (seen) continue;
                        if (n == kDeadCells || __ldg(a.b + f) != 0.f) return false;
                        comp[n++] = f;
                    } else if (__ldg(a.b + f) != 0.f) {
                        return false;
                    }
                }
            }
            return true;
        };
        const unsigned long long tag = (unsigned long long)ep0 << 32;
        unsigned long long wbest = 0ull;
        int wk = -1;
        for (int r = warp; r < ti; r += nw) {
            const int gi = ti0 + r;
            if (gi >= NI) break;
            for (int q0 = 0; q0 < tj && tj0 + q0 < NJ; q0 += 32) {
                const int q = q0 + lane, gj = tj0 + q;
                bool live = false;
                if (q < tj && gj < NJ) {
                    const int c = (r + 2) * w2 + (q + 2);
                    if (Ib[c] & 0x80u) live = Rb[c] != 0.f || !dead_unit(gi * NJ + gj);
                }
                unsigned lv = __ballot_sync(0xffffffffu, live);
                if (!lv) continue;
                // the chunk of each lane's cell: one search for the segment,
                // one a lane only where a chunk boundary falls inside it
                const long long e0 = (long long)gi * NJ + tj0 + q0, e = e0 + lane;
                const int seg_last = min(31, min(tj, NJ - tj0) - 1 - q0);
                int k0 = 0;
                if (lane == 0) k0 = chunk_index(e0);
                k0 = __shfl_sync(0xffffffffu, k0, 0);
                const bool one = e0 + seg_last < a.chunk_end[k0];
                const int kl = one ? k0 : (lane <= seg_last ? chunk_index(e) : k0);
                while (lv) {
                    const int h = 31 - __clz((int)lv);
                    const int kh = __shfl_sync(0xffffffffu, kl, h);
                    const unsigned long long ph = tag | (unsigned long long)(e0 + h + 1);
                    lv &= ~__ballot_sync(0xffffffffu, kl == kh);
                    if (kh != wk) {
                        if (wk >= 0 && lane == 0) atomicMax(effw + wk, wbest);
                        wk = kh;
                        wbest = ph;
                    } else if (ph > wbest) {
                        wbest = ph;
                    }
                }
            }
        }
        if (wk >= 0 && lane == 0) atomicMax(effw + wk, wbest);
    }
    // packed operator word of each tile-plus-1-halo cell: its own row byte
    // (bits 0-7) and the cell counts of its four neighbours (3 bits each:
    // i-1 at 8, i+1 at 11, j-1 at 14, j+1 at 17), which select the IPP
    // coefficients
    // (spec mode: the K K^T packing of kkt_apply instead)
    for (int e = threadIdx.x; e < L.hp * w1; e += blockDim.x) {
        const int r = e / w1, q = e - r * w1;
        const int c2 = (r + 1) * w2 + (q + 1);
        if constexpr (SPEC) {
            auto kcode = [](unsigned b) { return (b & 0x80) ? ((b >> 4) & 7u) : 0u; };
            auto dn_in = [](unsigned b) { return (b & 0x81) == 0x81 ? 1u : 0u; }; // its upper neighbour
            auto rt_in = [](unsigned b) { return (b & 0x84) == 0x84 ? 1u : 0u; }; // its left neighbour
            Op[e] = (unsigned)Ib[c2] | (dn_in(Ib[c2 + w2]) << 8) | (rt_in(Ib[c2 + 1]) << 9) |
                    (kcode(Ib[c2 - w2]) << 10) | (rt_in(Ib[c2 - w2 + 1]) << 13) | (kcode(Ib[c2 - 1]) << 14) |
                    (dn_in(Ib[c2 + w2 - 1]) << 17);
        } else {
            Op[e] = (unsigned)Ib[c2] | ((unsigned)((Ib[c2 - w2] >> 4) & 7) << 8) |
                    ((unsigned)((Ib[c2 + w2] >> 4) & 7) << 11) |
                    ((unsigned)((Ib[c2 - 1] >> 4) & 7) << 14) | ((unsigned)((Ib[c2 + 1] >> 4) & 7) << 17);
        }
    }
    float2 sigma;
    bool zero;
    float stop = 0.f; // spec mode: r.r at which the inner solve stops
    if constexpr (SPEC) {
        // z_0 = K K^T r_0 on the tile and its 1-halo (r_0 = b is known on the
        // 2-halo) becomes s_0 there; sigma = r.z and r.r over the tile
        __syncthreads();
        float rz = 0.f;
        for (int e = threadIdx.x; e < h1 * w1; e += blockDim.x) {
            const int r = e / w1, q = e - r * w1;
            const int c = (r + 1) * w2 + (q + 1);
            const float z = kkt_apply(Op[e], inv, Rb[c], Rb[c + w2], Rb[c + 1], Rb[c - w2], Rb[c - w2 + 1],
                                      Rb[c - 1], Rb[c + w2 - 1]);
            Sb[c] = z;
            if (r >= 1 && r <= ti && q >= 1 && q <= tj) rz = fmaf(Rb[c], z, rz);
        }
        float2 prz, prr;
        bsum0_2(rz, bb, smf, prz, prr);
        publish(prz, 0u, prr);
        const float4 s0 = wait_sum(false);
        if (gfail) return;
        sigma = make_float2(s0.x, s0.y);
        zero = !(s0.z > 0.f);
        stop = eps_in * eps_in * s0.z;
    } else {
        const float2 part = bsum0(bb, smf); // its block barrier also retires Ib
        const int anynz = __syncthreads_or(nz);
        // the live-end maxima of every thread of the block are ordered before
        // the record (release); the gathering lanes acquire after it
        if (eff && threadIdx.x == 0) fence_acq_rel_gpu();
        publish(part, anynz ? 0x80000000u : 0u); // the flag: b has a nonzero
        const float4 s0 = wait_sum(false);
        if (gfail) return;
        sigma = make_float2(s0.x, s0.y);
        zero = s0.w == 0.f;
        if (eff) {
            if (warp < ((G + 31) >> 5)) fence_acq_rel_gpu();
            __syncthreads();
            list_owned();
            int hm = 0;
            for (int k = threadIdx.x; k < a.nchunks; k += blockDim.x) hm |= last_unit(k) < 0;
            has_min_static = __syncthreads_or(hm);
        }
    }

    // the neighbours' values on the 2-deep ring around the tile, from their
    // exchange words of epoch ep (bounded polls); a block barrier, then a
    // block-uniform false on timeout
    auto load_ring_ll = [&](float *dst, const unsigned long long *src, unsigned ep) -> bool {
        // two cells per thread per round, both loads issued before either is
        // polled, so a thread with two ring cells waits one round trip
        const int n = 4 * w2 + 4 * ti;
        const int nt = (int)blockDim.x;
        for (int k0 = threadIdx.x; k0 < n; k0 += 2 * nt) {
            const unsigned long long *p[2] = {nullptr, nullptr};
            int cell[2] = {-1, -1};
            unsigned long long w[2] = {0ull, 0ull};
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int k = k0 + h * nt;
                if (k >= n) continue;
                int r, q;
                ring_cell(k, ti, tj, r, q);
                cell[h] = (r + 2) * w2 + (q + 2);
                const int gi = ti0 + r, gj = tj0 + q;
                if (gi >= 0 && gi < NI && gj >= 0 && gj < NJ) {
                    p[h] = src + (size_t)gi * NJ + gj;
                    w[h] = ld_ll(p[h]);
                }
            }
#pragma unroll
            for (int h = 0; h < 2; h++) {
                if (cell[h] < 0) continue;
                float v = 0.f;
                if (p[h]) {
                    long long spins = 0;
                    while (ll_epoch(w[h]) != ep) {
                        if (++spins > lim || ((spins & 255) == 0 && *((volatile int *)a.status) != 0)) {
                            atomicExch(a.status, 1);
                            break;
                        }
                        w[h] = ld_ll(p[h]);
                    }
                    v = __uint_as_float((unsigned)w[h]);
                }
                dst[cell[h]] = v;
            }
        }
        return ok();
    };

    // strips: the neighbours' values on the 1-deep ring around the tile (the
    // tile's 1-halo), from their exchange words of epoch ep, into dst (the
    // tile-plus-1-halo layout, pitch w1); two cells per thread per round,
    // both loads issued before either is polled.  A block barrier, then a
    // block-uniform false on timeout.
    auto load_ring1 = [&](float *dst, const unsigned long long *src, unsigned ep) -> bool {
        // strips of one or two rows (small grids): a quarter of the threads
        // poll, four cells each -- fewer pollers at once (256^2: 2.27
        // against 2.6 ms of PCG per substep on GB300; at 1024^2 the same
        // cost 6 %, so taller strips keep two cells a thread on every thread)
        constexpr int kC = RPS <= 2 ? 4 : 2;
        const int n = 2 * w1 + 2 * ti;
        const int nt = kC == 4 ? (int)blockDim.x / 4 : (int)blockDim.x;
        for (int k0 = threadIdx.x; k0 < n && (int)threadIdx.x < nt; k0 += kC * nt) {
            int g[kC], cell[kC];
            unsigned long long w[kC];
#pragma unroll
            for (int h = 0; h < kC; h++) {
                g[h] = -1;
                cell[h] = -1;
                w[h] = 0ull;
            }
#pragma unroll
            for (int h = 0; h < kC; h++) {
                const int k = k0 + h * nt;
                if (k >= n) continue;
                int hr, hq;
                if (k < 2 * w1) {
                    hr = k < w1 ? 0 : h1 - 1;
                    hq = k < w1 ? k : k - w1;
                } else {
                    hr = 1 + ((k - 2 * w1) >> 1);
                    hq = ((k - 2 * w1) & 1) ? w1 - 1 : 0;
                }
                cell[h] = hr * w1 + hq;
                const int gi = ti0 + hr - 1, gj = tj0 + hq - 1;
                if (gi >= 0 && gi < NI && gj >= 0 && gj < NJ) {
                    g[h] = gi * NJ + gj;
                    w[h] = ld_ll(src + g[h]);
                }
            }
#pragma unroll
            for (int h = 0; h < kC; h++) {
                if (cell[h] < 0) continue;
                float v = 0.f;
                if (g[h] >= 0) {
                    long long spins = 0;
                    while (ll_epoch(w[h]) != ep) {
                        if (++spins > lim || ((spins & 255) == 0 && *((volatile int *)a.status) != 0)) {
                            atomicExch(a.status, 1);
                            break;
                        }
                        w[h] = ld_ll(src + g[h]);
                    }
                    v = __uint_as_float((unsigned)w[h]);
                }
                dst[cell[h]] = v;
            }
        }
        return ok();
    };

    // the stencils on a row-major shared array of pitch w, centred at c
    auto precond = [&](unsigned p, const float *v, int c, int w) -> float {
        return ipp_apply(p, inv, v[c], v[c - w], v[c + w], v[c - 1], v[c + 1]);
    };
    auto apply_a = [&](unsigned p, const float *v, int c, int w) -> float {
        return op_apply(p, scale, v[c], v[c - w], v[c + w], v[c - 1], v[c + 1]);
    };

    // register strips (RPS > 0): this thread's strip is rows row0 ..
    // row0 + RPS - 1 of the (padded) tile-plus-1-halo region in column qb.
    // Rows >= h1 are padding: computed, never stored.  Row h1 itself is the
    // outer ring row below the tile; its registers are refreshed from the
    // ring so that row h1 - 1 can take its lower neighbour from a register.
    const int row0 = (warp / ngrp) * kR;
    const int qb = 1 + 32 * (warp % ngrp) + lane; // column in the 1-halo region
    const int cbase = (row0 + 1) * w2 + (qb + 1); // its first cell in Rb / Sb
    // Rr: r; Sr: s, or between a sweep's two halves the value that does not
    // need the new scalar yet (z = M r, then A s) -- s itself is in Sb then
    float Rr[kR], Sr[kR];
    const unsigned *Ost = Op + row0 * w1 + qb; // operator words of the strip, pitch w1
    if constexpr (RPS > 0) {
#pragma unroll
        for (int rr = 0; rr < kR; rr++) {
            Rr[rr] = Rb[cbase + rr * w2];
            Sr[rr] = SPEC ? Sb[cbase + rr * w2] : Rr[rr]; // s_0: z_0 in spec mode, else b
        }
    }
    auto live = [&](int rr) { return row0 + rr < h1; };                     // stored rows
    auto on_tile = [&](int rr) { return row0 + rr >= 1 && row0 + rr <= ti; }; // tile rows
    // lower neighbour of strip row rr: a register inside the strip, shared
    // memory below its last row
    auto dn_of = [&](const float *reg, const float *arr, int rr, int c) -> float {
        return rr + 1 < kR ? reg[rr + 1 < kR ? rr + 1 : 0] : arr[c + w2];
    };
    auto up_of = [&](const float *reg, const float *arr, int rr, int c) -> float {
        return rr > 0 ? reg[rr > 0 ? rr - 1 : 0] : arr[c - w2];
    };
    // tile cells within two of the tile border (what a neighbour's ring reads)
    // tile cells on the tile's border: neighbours read them as their 1-halo
    // ring (z after the z sweep, A s after the A s sweep)
    const int tcol = qb - 1;
    const bool col_band = tcol == 0 || tcol == tj - 1;
    auto in_band = [&](int rr) {
        const int tr = row0 + rr - 1;
        return col_band || tr == 0 || tr == ti - 1;
    };
    // all of the tile's r (in Rb) into r0 (plain stores; the fenced barrier
    // that follows orders them before any block reads them)
    auto publish_tile_r = [&]() {
        for (int r = warp; r < ti; r += nw) {
            const int gi = ti0 + r;
            if (gi >= NI) break;
            for (int q = lane; q < tj; q += 32) {
                const int gj = tj0 + q;
                if (gj < NJ) a.r0[(size_t)gi * NJ + gj] = Rb[(r + 2) * w2 + (q + 2)];
            }
        }
    };
    // halo-column cells (1-halo columns 0 and w1 - 1; their z and A s land in
    // B1 with the rings): with strips of 4 rows
    // or more, one a thread on the warps whose strips hold no 1-halo row
    // (strips 1 .. smax, which have no halo row of their own to compute) when
    // they are enough; else four a warp, spread over the warps.  (Measured
    // on GB300: the first takes 0.11 ms off a 200-iteration solve at 1024^2
    // and 0.08 ms at 512^2, but adds 0.14 ms at 256^2, where strips are one
    // row high.)
    int edge0 = (threadIdx.x & 7) == 0 ? (int)(threadIdx.x >> 3) : 1 << 30;
    int edge_step = (int)(blockDim.x >> 3);
    if constexpr (RPS >= 4) {
        const int smax = (h1 - 1 - kR) / kR;
        const int nmid = (smax >= 1 ? smax : 0) * ngrp * 32;
        if (nmid >= 2 * h1) {
            const int t = (int)threadIdx.x - ngrp * 32;
            edge0 = (t >= 0 && t < nmid) ? t : 1 << 30;
            edge_step = nmid;
        }
    }
    auto edge_cell = [&](int e) { return ((e >> 1) + 1) * w2 + ((e & 1) ? w1 : 1); };
    // the same halo-column cell in the tile-plus-1-halo layout of B1
    auto edge_b1 = [&](int e) { return (e >> 1) * w1 + ((e & 1) ? w1 - 1 : 0); };
    auto edge_op = [&](int e) { return Op[(e >> 1) * w1 + ((e & 1) ? w1 - 1 : 0)]; };

    // |r_{it+1}| at each chunk's last (live) unit row, from the tile holding it (Rb
    // holds r_{it+1} on the tile); the block barrier of the z.r sum orders
    // s_cmax / s_cscan before thread 0 publishes them
    auto chunk_ends = [&]() {
        auto chunk_end_value = [&](int k, float v) {
            reinterpret_cast<float *>(a.chunk_val)[k] = v != 0.f ? fabsf(v) : -1.f;
            if (v != 0.f) atomicMax(&s_cmax, __float_as_int(fabsf(v))); // order of non-negative floats
            else s_cscan = 1;
        };
        if (s_nown <= kMaxOwnedChunks) {
            for (int j = threadIdx.x; j < s_nown; j += blockDim.x)
                chunk_end_value(s_own[j].x, Rb[s_own[j].y]);
        } else {
            for (int k = threadIdx.x; k < a.nchunks; k += blockDim.x) {
                const int idx = last_unit(k);
                if (idx < 0) continue;
                const int gi = idx / NJ, gj = idx - gi * NJ;
                if (gi < ti0 || gi >= ti0 + ti || gj < tj0 || gj >= tj0 + tj) continue;
                chunk_end_value(k, Rb[(gi - ti0 + 2) * w2 + (gj - tj0 + 2)]);
            }
        }
    };

    float fb = 0.f;
    int result = zero || iter_limit <= 0 ? 0 : iter_limit;
    for (int it = 0; !zero && iter_limit > 0; it++) {
        const bool first = it == 0;
        const unsigned ep_s = ep0 + 2u * it + 1u; // epoch of s_it's exchange words
        const unsigned ep_r = ep0 + 2u * it + 2u; // epoch of r_{it+1}'s

        // ---- sweep 1 -------------------------------------------------------
        if (!first) {
            const bool more = it < iter_limit;
            if (more) {
                if constexpr (RPS > 0) {
                    // z_it on the tile's 1-halo as the neighbours computed it on
                    // their border (their z sweep published it); z on the tile
                    // rows came with the last sweep's z.r.  Halo columns read it
                    // from B1 in the s update.
                    if (!load_ring1(B1, a.ll_r, ep0 + 2u * it)) return;
#pragma unroll
                    for (int rr = 0; rr < kR; rr++)
                        if (live(rr) && !on_tile(rr)) Sr[rr] = B1[(row0 + rr) * w1 + qb];
                } else {
                    // z_it = M r_it on the tile and its 1-halo while the grid
                    // barrier of the last sweep completes
                    if (!load_ring_ll(Rb, a.ll_r, ep0 + 2u * it)) return;
                    for_halo1(h1, w1, [&](int r, int q) {
                        B1[r * w1 + q] = precond(Op[r * w1 + q], Rb, (r + 1) * w2 + (q + 1), w2);
                    });
                }
            }
            // end of iteration it - 1: beta and the stopping test
            const float4 rec = wait_sum(true); // and x += alpha s_{it-1}
            if (gfail) return;
            const float2 newSigma = make_float2(rec.x, rec.y);
            if constexpr (SPEC) {
                // spec mode: r.r against the inner tolerance (k_pcg_spec's rule)
                if (rec.z <= stop || !more) {
                    result = it;
                    break;
                }
            } else {
                // a zero at a chunk-end unit row needs the backward scan;
                // otherwise the largest |r| over the blocks decides
                if (rec.w != 0.f) {
                    // the scan reads r anywhere in a chunk: every tile
                    // publishes all of r_it (still intact in Rb) and the grid
                    // meets at a fenced barrier
                    publish_tile_r();
                    if (!fenced_barrier()) return;
                }
                const bool done =
                    rec.w != 0.f
                        ? chunk_converged(a, [&](long long e) { return __ldcg(a.r0 + e); }, last_unit, tt, &s_flag)
                        : tol_met(tt, rec.z, has_min_static);
                if (done) {
                    result = it - 1;
                    break;
                }
                if (!more) break;
            }
            fb = ff_div(newSigma, sigma);
            sigma = newSigma;
            // s_it = z_it + beta s_{it-1}
            if constexpr (RPS > 0) {
#pragma unroll
                for (int rr = 0; rr < kR; rr++) {
                    const int c = cbase + rr * w2;
                    Sr[rr] = fmaf(Sb[c], fb, Sr[rr]);
                }
#pragma unroll
                for (int rr = 0; rr < kR; rr++)
                    if (live(rr)) Sb[cbase + rr * w2] = Sr[rr];
                for (int ed = edge0; ed < 2 * h1; ed += edge_step) {
                    const int c = edge_cell(ed);
                    Sb[c] = fmaf(Sb[c], fb, B1[edge_b1(ed)]); // z from the ring
                }
            } else {
                for_halo1(h1, w1, [&](int r, int q) {
                    B1[r * w1 + q] = fmaf(Sb[(r + 1) * w2 + (q + 1)], fb, B1[r * w1 + q]);
                });
            }
        } else if constexpr (RPS == 0) {
            for_halo1(h1, w1, [&](int r, int q) { B1[r * w1 + q] = Sb[(r + 1) * w2 + (q + 1)]; });
        }
        __syncthreads();
        float qs = 0.f;
        if constexpr (RPS > 0) {
            const int gj = tj0 + qb - 1;
            float prev = 0.f; // s of the row above, before it was overwritten
#pragma unroll
            for (int rr = 0; rr < kR; rr++) {
                const int c = cbase + rr * w2;
                const float cur = Sr[rr];
                const float up = rr > 0 ? prev : Sb[c - w2];
                const float q = op_apply(Ost[rr * w1], scale, cur, up, dn_of(Sr, Sb, rr, c),
                                         Sb[c - 1], Sb[c + 1]);
                // padding rows may hold anything, even inf: select, do not scale
                qs = on_tile(rr) ? fmaf(q, cur, qs) : qs;
                // A s on the tile rows is the next sweep's A s there too; s
                // itself stays in Sb
                Sr[rr] = on_tile(rr) ? q : cur;
                prev = cur;
            }
            // A s on the tile's border: the neighbours' 1-halo ring in their
            // sweep 2 (iteration 0 computes it from s_0 = b instead, except in
            // spec mode, where s_0 = z_0 is known on the 1-halo only)
            if ((SPEC || !first) && gj < NJ) {
#pragma unroll
                for (int rr = 0; rr < kR; rr++) {
                    const int gi = ti0 + row0 + rr - 1;
                    if (on_tile(rr) && in_band(rr) && gi < NI)
                        st_ll(a.ll_s + (size_t)gi * NJ + gj, ll_pack(__float_as_uint(Sr[rr]), ep_s));
                }
            }
        } else {
            for (int r = warp; r < ti; r += nw) {
                const int gi = ti0 + r;
                for (int q = lane; q < tj; q += 32) {
                    const int gj = tj0 + q;
                    const int c1 = (r + 1) * w1 + (q + 1);
                    const float s_c = B1[c1];
                    qs = fmaf(apply_a(Op[c1], B1, c1, w1), s_c, qs);
                    if (!first) {
                        Sb[(r + 2) * w2 + (q + 2)] = s_c;
                        if (gi < NI && gj < NJ)
                            st_ll(a.ll_s + (size_t)gi * NJ + gj, ll_pack(__float_as_uint(s_c), ep_s));
                    }
                }
            }
        }
        {
            const float2 part = bsum0(qs, smf);
            if (threadIdx.x == 0) {
                s_cmax = 0;
                s_cscan = 0;
            }
            publish(part, 0u);
        }

        // ---- sweep 2 -------------------------------------------------------
        // A s_it on the tile's 1-halo while the grid barrier completes; the
        // tile rows' A s came with s.As
        if constexpr (RPS > 0) {
            if (first && !SPEC) {
                // s_0 = b is known on the 2-halo since the set-up: A s_0 on the
                // 1-halo from Sb (its 1-halo rows into registers, its halo
                // columns into B1 where later iterations' rings land)
#pragma unroll
                for (int rr = 0; rr < kR; rr++)
                    if (!on_tile(rr)) Sr[rr] = apply_a(Ost[rr * w1], Sb, cbase + rr * w2, w2);
                for (int ed = edge0; ed < 2 * h1; ed += edge_step)
                    B1[edge_b1(ed)] = apply_a(edge_op(ed), Sb, edge_cell(ed), w2);
            } else {
                // as the neighbours computed it on their border
                if (!load_ring1(B1, a.ll_s, ep_s)) return;
#pragma unroll
                for (int rr = 0; rr < kR; rr++)
                    if (live(rr) && !on_tile(rr)) Sr[rr] = B1[(row0 + rr) * w1 + qb];
            }
        } else {
            if (!first && !load_ring_ll(Sb, a.ll_s, ep_s)) return; // neighbours' s_it
            for_halo1(h1, w1, [&](int r, int q) {
                B1[r * w1 + q] = apply_a(Op[r * w1 + q], Sb, (r + 1) * w2 + (q + 1), w2);
            });
        }
        const float4 qsum = wait_sum(false);
        if (gfail) return;
        // (the reference adds 1e-8 to s.As; the spec-mode solve does not)
        const float fa = SPEC ? ff_div(sigma, make_float2(qsum.x, qsum.y))
                              : ff_div(sigma, ff_add(make_float2(qsum.x, qsum.y), eps8));
        fa_prev = fa;
        // r_{it+1} = r_it - alpha A s_it (x += alpha s_it on the tile comes
        // during the next iteration's beta reduction)
        if constexpr (RPS > 0) {
#pragma unroll
            for (int rr = 0; rr < kR; rr++) Rr[rr] = fmaf(-Sr[rr], fa, Rr[rr]);
#pragma unroll
            for (int rr = 0; rr < kR; rr++)
                if (live(rr)) Rb[cbase + rr * w2] = Rr[rr];
            for (int ed = edge0; ed < 2 * h1; ed += edge_step) {
                const int c = edge_cell(ed);
                Rb[c] = fmaf(-B1[edge_b1(ed)], fa, Rb[c]); // A s on the halo column
            }
        } else {
            for_halo1(h1, w1, [&](int r, int q) {
                B1[r * w1 + q] = fmaf(-B1[r * w1 + q], fa, Rb[(r + 1) * w2 + (q + 1)]);
            });
        }
        __syncthreads();
        float zr = 0.f, rr2 = 0.f;
        if constexpr (RPS > 0) {
            // r_{it+1} is in Rb since the barrier above: no barrier of its own
            if constexpr (!SPEC) chunk_ends();
            const int gj = tj0 + qb - 1;
#pragma unroll
            for (int rr = 0; rr < kR; rr++) {
                const int c = cbase + rr * w2;
                float z;
                if constexpr (SPEC) {
                    z = kkt_apply(Ost[rr * w1], inv, Rr[rr], dn_of(Rr, Rb, rr, c), Rb[c + 1], up_of(Rr, Rb, rr, c),
                                  Rb[c - w2 + 1], Rb[c - 1], Rb[c + w2 - 1]);
                    rr2 = on_tile(rr) ? fmaf(Rr[rr], Rr[rr], rr2) : rr2;
                } else {
                    z = ipp_apply(Ost[rr * w1], inv, Rr[rr], up_of(Rr, Rb, rr, c), dn_of(Rr, Rb, rr, c),
                                  Rb[c - 1], Rb[c + 1]);
                }
                zr = on_tile(rr) ? fmaf(z, Rr[rr], zr) : zr;
                // z on the tile rows is the next sweep's z there too
                Sr[rr] = on_tile(rr) ? z : Sr[rr];
            }
            // z on the tile's border: the neighbours' 1-halo ring in their next
            // sweep 1; the rare backward max-abs scan gets the tile's whole r
            // on demand (publish_tile_r)
            if (gj < NJ) {
#pragma unroll
                for (int rr = 0; rr < kR; rr++) {
                    const int gi = ti0 + row0 + rr - 1;
                    if (on_tile(rr) && in_band(rr) && gi < NI)
                        st_ll(a.ll_r + (size_t)gi * NJ + gj, ll_pack(__float_as_uint(Sr[rr]), ep_r));
                }
            }
        } else {
            for (int r = warp; r < ti; r += nw) {
                const int gi = ti0 + r;
                for (int q = lane; q < tj; q += 32) {
                    const int gj = tj0 + q;
                    const int c1 = (r + 1) * w1 + (q + 1);
                    const int c2 = (r + 2) * w2 + (q + 2);
                    const float r_c = B1[c1];
                    zr = fmaf(precond(Op[c1], B1, c1, w1), r_c, zr);
                    Xt[r * tj + q] = fmaf(Sb[c2], fa, Xt[r * tj + q]);
                    Rb[c2] = r_c;
                    if (gi < NI && gj < NJ)
                        st_ll(a.ll_r + (size_t)gi * NJ + gj, ll_pack(__float_as_uint(r_c), ep_r));
                }
            }
        }
        if constexpr (RPS == 0) {
            __syncthreads(); // the sweep above stored r_{it+1} in Rb
            chunk_ends();
        }
        if constexpr (SPEC) {
            float2 pzr, prr;
            bsum0_2(zr, rr2, smf, pzr, prr);
            publish(pzr, 0u, prr);
        } else {
            const float2 part = bsum0(zr, smf); // its barrier also orders s_cmax / s_cscan
            publish(part, (unsigned)s_cmax | (s_cscan ? 0x80000000u : 0u));
        }
    }
    // the solution leaves shared memory once
    for (int r = warp; r < ti; r += nw) {
        const int gi = ti0 + r;
        if (gi >= NI) break;
        for (int q = lane; q < tj; q += 32) {
            const int gj = tj0 + q;
            if (gj < NJ) a.x[(size_t)gi * NJ + gj] = Xt[r * tj + q];
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        if (a.iters_out) *a.iters_out = result;
        if constexpr (SPEC) {
            a.spec_ctl->total += result;
            a.spec_ctl->last_it = result;
        }
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
// the driver's tensor-map encoder (one process-wide entry point; the
// initialisation of a function-local static is thread-safe)
static PFN_cuTensorMapEncodeTiled_v12000 encode_fn()
{
    static const PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                             &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
        cudaGetLastError();
        return (PFN_cuTensorMapEncodeTiled_v12000) nullptr;
    }();
    return fn;
}

static bool encode(CUtensorMap *map, const void *ptr, CUtensorMapDataType dt, int esz, int ni,
                   int nj, int box_w, int box_h)
{
    auto fn = encode_fn();
    if (!fn || ((size_t)ptr & 15)) return false;
    cuuint64_t dims[2] = {(cuuint64_t)nj, (cuuint64_t)ni};
    cuuint64_t strides[1] = {(cuuint64_t)nj * esz};
    cuuint32_t box[2] = {(cuuint32_t)box_w, (cuuint32_t)box_h};
    cuuint32_t es[2] = {1, 1};
    return fn(map, dt, 2, const_cast<void *>(ptr), dims, strides, box, es,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
              CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) ==
           CUDA_SUCCESS;
}

static int sm_count() { return device_sm_count(); }

constexpr int kMaxTmaCells = 54 * 128;

bool tma_tile_shape(int ni, int nj, int *ti, int *tj)
{
    if (nj % 16 != 0) return false;
    const int blocks = sm_count();
    int w = nj < 128 ? nj : 128;
    if (w % 32 != 0) w = ((w + 31) / 32) * 32;
    const long long tiles_j = (nj + w - 1) / w;
    const long long cap = kMaxTmaCells / w;
    for (long long k = 1; k <= 4096; k++) {
        long long max_ti = (long long)blocks * k / tiles_j;
        if (max_ti < 1) continue;
        long long h = (ni + max_ti - 1) / max_ti;
        if (h < 8) h = ni < 8 ? ni : 8;
        if (h <= cap) {
            *ti = (int)h;
            *tj = w;
            return h + 4 <= 256;
        }
    }
    return false;
}

bool tma_maps(TmaMaps *m, int ni, int nj, int ti, int tj, const uint8_t *info, const float *b,
              const float *x, const float *r0, const float *r1, const float *s0, const float *s1)
{
    const CUtensorMapDataType F = CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
    const CUtensorMapDataType U = CU_TENSOR_MAP_DATA_TYPE_UINT8;
    return encode(&m->info, info, U, 1, ni, nj, tj + 32, ti + 4) &&
           encode(&m->b, b, F, 4, ni, nj, tj + 8, ti + 4) &&
           encode(&m->x, x, F, 4, ni, nj, tj, ti) &&
           encode(&m->r0, r0, F, 4, ni, nj, tj + 8, ti + 4) &&
           encode(&m->r1, r1, F, 4, ni, nj, tj + 8, ti + 4) &&
           encode(&m->s0, s0, F, 4, ni, nj, tj + 8, ti + 4) &&
           encode(&m->s1, s1, F, 4, ni, nj, tj + 8, ti + 4);
}

// r and s are loaded with halo boxes and stored with tile boxes, so each has
// a second map encoded with the tile box for the stores
bool tma_store_maps(TmaMaps *m, int ni, int nj, int ti, int tj, const float *r0, const float *r1,
                    const float *s0, const float *s1)
{
    const CUtensorMapDataType F = CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
    return encode(&m->r0_st, r0, F, 4, ni, nj, tj, ti) &&
           encode(&m->r1_st, r1, F, 4, ni, nj, tj, ti) &&
           encode(&m->s0_st, s0, F, 4, ni, nj, tj, ti) &&
           encode(&m->s1_st, s1, F, 4, ni, nj, tj, ti);
}

constexpr size_t kMaxResidentSmem = 220 * 1024;

// rows per register strip for a tile shape (0: strips do not apply)
static int strip_rows(int ti, int tj)
{
    const int warps = kStripThreads / 32;
    if (tj % 32 != 0 || tj / 32 > warps || warps % (tj / 32) != 0) return 0;
    const int nstrips = warps / (tj / 32);
    const int rps = (ti + 2 + nstrips - 1) / nstrips;
    // the instantiated strip heights; the smallest that covers the rows, so
    // that few padding rows are computed (56 rows in 4 strips: 14, not 16)
    for (int h : {1, 2, 4, 6, 8, 10, 12, 14, 16})
        if (rps <= h) return h;
    return 0;
}

// shared memory of the resident kernel for a tile shape (strips pad rows)
static size_t resident_smem(int ti, int tj)
{
    const int rps = strip_rows(ti, tj);
    const int nstrips = rps > 0 ? kStripThreads / 32 / (tj / 32) : 0;
    return res_layout(ti, tj, nstrips * rps).bytes;
}

// every tile shape of width 32 .. 256 with at most one tile per SM (and no
// more tiles than the grid reduction reads partials for) whose shared memory
// fits: the rows per tile are the fewest that cover the grid in that many
void resident_candidates(int ni, int nj, std::vector<std::pair<int, int>> *out)
{
    out->clear();
    const int blocks = min(sm_count(), 32 * kPartRounds);
    for (int w = 32; w <= 256; w *= 2) {
        const long long tiles_j = (nj + w - 1) / w;
        if (tiles_j > blocks) continue;
        const long long max_ti = blocks / tiles_j;
        long long h = (ni + max_ti - 1) / max_ti;
        if (h < 1) h = 1;
        const long long ntiles = ((ni + h - 1) / h) * tiles_j;
        if (ntiles > blocks) continue;
        if (resident_smem((int)h, w) > kMaxResidentSmem) continue;
        out->push_back({(int)h, w});
        if (w >= nj) break; // wider tiles only add empty columns
    }
}

// shapes chosen by the autotuner, by grid shape (this process)
static std::mutex g_res_mu;
static std::map<std::pair<int, int>, std::pair<int, int>> g_res_tuned;

void resident_set_tuned(int ni, int nj, int ti, int tj)
{
    std::lock_guard<std::mutex> lock(g_res_mu);
    if (ti > 0) g_res_tuned[{ni, nj}] = {ti, tj};
    else g_res_tuned.erase({ni, nj});
}

bool resident_tile_shape(int ni, int nj, int *ti, int *tj)
{
    {
        std::lock_guard<std::mutex> lock(g_res_mu);
        auto it = g_res_tuned.find({ni, nj});
        if (it != g_res_tuned.end()) {
            *ti = it->second.first;
            *tj = it->second.second;
            return true;
        }
    }
    // the default: the candidate with the fewest cells per block including
    // the 1-halo around its tile
    std::vector<std::pair<int, int>> cand;
    resident_candidates(ni, nj, &cand);
    long long best = -1;
    for (const auto &c : cand) {
        const long long cost = (long long)(c.first + 2) * (c.second + 2);
        if (best < 0 || cost < best) {
            best = cost;
            *ti = c.first;
            *tj = c.second;
        }
    }
    return best >= 0;
}

template <int RPS, bool SPEC = false>
static cudaError_t launch_resident_rps(const PcgArgs<float> &a, int ti, int tj, int grid,
                                       cudaStream_t st)
{
    const int nstrips = (RPS > 0 ? kStripThreads : kThreads) / 32 / (tj / 32);
    const size_t smem = res_layout(ti, tj, RPS > 0 ? nstrips * RPS : 0).bytes;
    const void *fn = (const void *)k_pcg_resident<RPS, SPEC>;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    PcgArgs<float> args = a;
    int vti = ti, vtj = tj;
    void *kargs[] = {&args, &vti, &vtj};
    return cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(RPS > 0 ? kStripThreads : kThreads), kargs, smem,
                                       st);
}

cudaError_t launch_pcg_resident(const PcgArgs<float> &a0, int ti, int tj, cudaStream_t st,
                                LlBuffers *ll)
{
    const int grid = ((a0.ni + ti - 1) / ti) * ((a0.nj + tj - 1) / tj);
    if (!ll || !ll->r || !ll->s || !ll->rec || ll->words < (size_t)a0.N || grid > 256)
        return cudaErrorInvalidValue;
    // epochs one launch may use: 1 + 2 per iteration for the reductions and
    // 2 per iteration for the ring words, with slack
    const unsigned long long span = 2ull * (unsigned long long)(a0.iter_limit > 0 ? a0.iter_limit : 0) + 8ull;
    if (span > (1ull << 30)) return cudaErrorInvalidValue;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaError_t e = cudaStreamIsCapturing(st, &cs);
    if (e != cudaSuccess) return e;
    // a captured launch replays with the same epochs, so it clears the
    // buffers inside the capture every time and leaves them to be cleared
    // again before the next launch outside it
    const bool capturing = cs != cudaStreamCaptureStatusNone;
    if (capturing || ll->next == 0 || (unsigned long long)ll->next + span > 0xfffffff0ull) {
        e = cudaMemsetAsync(ll->r, 0, ll->words * sizeof(unsigned long long), st);
        if (e == cudaSuccess) e = cudaMemsetAsync(ll->s, 0, ll->words * sizeof(unsigned long long), st);
        if (e == cudaSuccess) e = cudaMemsetAsync(ll->rec, 0, kLlRecWords * sizeof(unsigned long long), st);
        if (e != cudaSuccess) return e;
        ll->next = 1;
    }
    PcgArgs<float> a = a0;
    a.ll_r = ll->r;
    a.ll_s = ll->s;
    a.ll_rec = ll->rec;
    a.ll_base = ll->next;
    ll->next = capturing ? 0u : (unsigned)(ll->next + span);
    e = cudaMemsetAsync(a.bar, 0, sizeof(GridBarrier), st);
    if (e != cudaSuccess) return e;
    switch (strip_rows(ti, tj)) {
    case 1: return launch_resident_rps<1>(a, ti, tj, grid, st);
    case 2: return launch_resident_rps<2>(a, ti, tj, grid, st);
    case 4: return launch_resident_rps<4>(a, ti, tj, grid, st);
    case 6: return launch_resident_rps<6>(a, ti, tj, grid, st);
    case 8: return launch_resident_rps<8>(a, ti, tj, grid, st);
    case 10: return launch_resident_rps<10>(a, ti, tj, grid, st);
    case 12: return launch_resident_rps<12>(a, ti, tj, grid, st);
    case 14: return launch_resident_rps<14>(a, ti, tj, grid, st);
    case 16: return launch_resident_rps<16>(a, ti, tj, grid, st);
    default: return launch_resident_rps<0>(a, ti, tj, grid, st);
    }
}

bool spec_resident_shape(int ni, int nj, int *ti, int *tj)
{
    int a = 0, b = 0;
    if (!resident_tile_shape(ni, nj, &a, &b) || strip_rows(a, b) == 0) return false;
    *ti = a;
    *tj = b;
    return true;
}

unsigned long long spec_resident_epochs(int max_iter)
{
    return 2ull * (unsigned long long)(max_iter > 0 ? max_iter : 0) + 8ull;
}

cudaError_t launch_spec_resident(const PcgArgs<float> &a, int ti, int tj, cudaStream_t st)
{
    const int grid = ((a.ni + ti - 1) / ti) * ((a.nj + tj - 1) / tj);
    if (!a.ll_r || !a.ll_s || !a.ll_rec || !a.spec_ctl || !a.spec_dt || grid > 256) return cudaErrorInvalidValue;
    switch (strip_rows(ti, tj)) {
    case 1: return launch_resident_rps<1, true>(a, ti, tj, grid, st);
    case 2: return launch_resident_rps<2, true>(a, ti, tj, grid, st);
    case 4: return launch_resident_rps<4, true>(a, ti, tj, grid, st);
    case 6: return launch_resident_rps<6, true>(a, ti, tj, grid, st);
    case 8: return launch_resident_rps<8, true>(a, ti, tj, grid, st);
    case 10: return launch_resident_rps<10, true>(a, ti, tj, grid, st);
    case 12: return launch_resident_rps<12, true>(a, ti, tj, grid, st);
    case 14: return launch_resident_rps<14, true>(a, ti, tj, grid, st);
    case 16: return launch_resident_rps<16, true>(a, ti, tj, grid, st);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_pcg_tma(const PcgArgs<float> &a, const TmaMaps &maps, int ti, int tj,
                           cudaStream_t st)
{
    const SmemLayout L = smem_layout(ti, tj);
    cudaError_t e = cudaFuncSetAttribute((const void *)k_pcg_tma,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)L.bytes);
    if (e != cudaSuccess) return e;
    const long long ntiles = (long long)((a.ni + ti - 1) / ti) * ((a.nj + tj - 1) / tj);
    const long long tpb = (ntiles + sm_count() - 1) / sm_count();
    const int grid = (int)((ntiles + tpb - 1) / tpb);
    PcgArgs<float> args = a;
    TmaMaps mm = maps;
    int vti = ti, vtj = tj;
    void *kargs[] = {&args, &mm, &vti, &vtj};
    e = cudaMemsetAsync(args.bar, 0, sizeof(GridBarrier), st);
    if (e != cudaSuccess) return e;
    return cudaLaunchCooperativeKernel((const void *)k_pcg_tma, dim3(grid), dim3(kThreads), kargs,
                                       L.bytes, st);
}

} // namespace fsg
