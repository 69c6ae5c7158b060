// fs_cluster.cu -- many independent pressure systems in one launch, one
// thread-block cluster per system.
//
// Each system is the reference's operator (getPressureProjectionMatrix,
// flipsolver2d.cpp:797-887) solved to a true relative residual the way the
// spec-mode solve does it (fs_spec.cu): FP32 inner PCG with the textbook
// incomplete-Poisson preconditioner M = K K^T, K = I - L D^-1
// (inversepoissonpreconditioner.h:45-79), and FP64 outer refinement
// r = b - A x, x += d.  Here the whole solve -- outer loop included -- is one
// cluster of C CTAs (C = 1 .. 16), so a launch carries any number of systems
// of different sizes and none of them needs global scratch:
//
// - CTA k of the cluster owns the grid rows [k ni / C, (k+1) ni / C).  Its
//   r, s and y live in shared memory with one halo row above and below;
//   the correction d and the per-cell q or z live in registers.
// - Neighbour data moves through distributed shared memory at the two
//   hardware cluster barriers of an iteration: after the s.q barrier a CTA
//   reads its neighbours' boundary rows of q and updates its halo copies of
//   r with them; after the r.z barrier it reads their boundary rows of z and
//   updates its halo copies of s.  The halo copies are computed with the
//   same operands as the owners' rows, so they are bitwise the same values.
//   y = K^T r is formed for the row above the CTA as well, which is all
//   z = K y needs.
// - Dot products: FP32 per thread, then float pairs (about 44 significant
//   bits) across threads, warps and the cluster's CTAs, in a fixed order --
//   every CTA adds the same partials in the same order and takes the same
//   decisions.  GB300's FP64 rate is a small fraction of its FP32 rate; FP64
//   is kept for the outer residual r = b - A x and its norm, which decide
//   convergence.
//
// The barriers are hardware cluster barriers: no spin loop, nothing to time
// out.  Every CTA of a cluster runs the same number of them because every
// branch depends only on values all CTAs computed identically.
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <map>
#include <mutex>
#include <utility>
#include <vector>

#include "fs_cluster.h"
#include "fs_common.cuh"
#include "fs_device.h"

namespace cg = cooperative_groups;

namespace fsg {

constexpr int kClThreads = 512;
constexpr int kClWarps = kClThreads / 32;
constexpr int kClMaxCells = 32;                     // own cells per thread at most
constexpr int kClMaxOwn = kClThreads * kClMaxCells; // own cells per CTA at most
constexpr size_t kClTail = 1024;                    // reduction scratch after the vectors

// r and s with a halo row above and below, the operator words of the same
// cells, then the boundary rows of q and z
__host__ __device__ inline size_t cl_vec_bytes(int rows_max, int nj)
{
    const size_t W = (size_t)(rows_max + 2) * nj;
    const size_t words = (8 * W + 2 * W + 15) & ~(size_t)15;
    return words + 16 * (size_t)nj;
}

__device__ __forceinline__ void cl_two_sum(float a, float b, float &s, float &e)
{
    s = a + b;
    const float bv = s - a;
    e = (a - (s - bv)) + (b - bv);
}
__device__ __forceinline__ float2 cl_add(float2 a, float2 b)
{
    float s, e;
    cl_two_sum(a.x, b.x, s, e);
    e += a.y + b.y;
    const float h = s + e;
    return make_float2(h, e - (h - s));
}
__device__ __forceinline__ float2 cl_shfl(float2 v, int o)
{
    return make_float2(__shfl_down_sync(0xffffffffu, v.x, o), __shfl_down_sync(0xffffffffu, v.y, o));
}
// a / b for float pairs, to about float precision
__device__ __forceinline__ float cl_div(float2 a, float2 b)
{
    const float q = __fdiv_rn(a.x, b.x);
    const float r = (fmaf(-q, b.x, a.x) + a.y) - q * b.y;
    return q + __fdiv_rn(r, b.x);
}

// The operator word of a cell, built once per solve from the packed operator
// byte of k_decomposition (bit 7 unit row, bits 4-6 non-solid count, bits 0-3
// fluid-neighbour mask up/down/left/right):
//   bits 0-3   the fluid-neighbour mask, kept only for neighbours inside the
//              grid (the linear index range [0, ni nj))
//   bits 4-7   count and unit bit as in the byte
//   bit 8      (K^T r)(c) takes r(c + nj): c + nj is a unit row whose mask
//              has its upper neighbour c
//   bit 9      (K^T r)(c) takes r(c + 1): the same for the left neighbour
//   bits 10-12 k(c) = scale / A(c, c): the count of a unit row (k = 1 / count),
//              0 otherwise (Eigen's zero-diagonal rule, k = scale)
// Inputs are read through the read-only cache (__ldg) when they stay fixed
// for the whole launch; a server launch (FRESH) serves many requests from the
// same buffers, which the host rewrites between them, so it reads past L1.
template <bool FRESH, typename T> __device__ __forceinline__ T cl_ro(const T *p)
{
    if constexpr (FRESH) return __ldcg(p);
    else return __ldg(p);
}

template <bool FRESH = false>
__device__ __forceinline__ unsigned cl_word(const uint8_t *__restrict__ info, int c, int N, int nj)
{
    if (c < 0 || c >= N) return 0u;
    const unsigned p = cl_ro<FRESH>(info + c);
    unsigned m = p & 0xFu;
    if (c - nj < 0) m &= ~1u;
    if (c + nj >= N) m &= ~2u;
    if (c - 1 < 0) m &= ~4u;
    if (c + 1 >= N) m &= ~8u;
    unsigned w = (p & 0xF0u) | m;
    if (c + nj < N && (cl_ro<FRESH>(info + c + nj) & 0x81) == 0x81) w |= 0x100u;
    if (c + 1 < N && (cl_ro<FRESH>(info + c + 1) & 0x84) == 0x84) w |= 0x200u;
    const unsigned cnt = (p >> 4) & 7u;
    if ((p & 0x80u) && cnt > 0) w |= cnt << 10;
    return w;
}

// One system's whole solve by the calling thread-block cluster.
// K = template cells per thread: the own cells of a CTA are
// tid + k * kClThreads, k < K; d and the per-cell q or z stay in registers
template <int K, bool FRESH = false>
__device__ __forceinline__ void cluster_solve(const ClusterSystem S, const ClusterParams &P)
{
    cg::cluster_group cl = cg::this_cluster();
    const int C = (int)cl.num_blocks();
    const int rank = (int)cl.block_rank();
    const int ni = S.ni, nj = S.nj;
    const int N = ni * nj; // at most the on-chip limit, far below 2^31
    const int i0 = (int)((long long)rank * ni / C);
    const int i1 = (int)((long long)(rank + 1) * ni / C);
    const int R = i1 - i0;
    const int Rmax = (ni + C - 1) / C;
    const int nown = R * nj;
    const int cb = i0 * nj; // linear index of own cell 0
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const bool has_up = rank > 0, has_dn = rank < C - 1;

    extern __shared__ __align__(16) unsigned char cl_smem[];
    const size_t W = (size_t)(Rmax + 2) * nj;
    float *r = reinterpret_cast<float *>(cl_smem);
    float *s = r + W;
    uint16_t *wd = reinterpret_cast<uint16_t *>(s + W);
    float *qb = reinterpret_cast<float *>(cl_smem + ((10 * W + 15) & ~(size_t)15)); // q of the first and the last own row
    float *zb = qb + 2 * nj; // z of the first and the last own row
    unsigned char *tail = cl_smem + cl_vec_bytes(Rmax, nj);
    float4 *part = reinterpret_cast<float4 *>(tail); // [2] published pair sums
    float4 *bc = part + 2;                           // [2] cluster sums
    double *dpart = reinterpret_cast<double *>(bc + 2); // [2]
    double *dbc = dpart + 2;                             // [2]
    float2 *wsum = reinterpret_cast<float2 *>(dbc + 2);  // [64]
    double *dwsum = reinterpret_cast<double *>(wsum + 64); // [32]
    float *ktab = reinterpret_cast<float *>(dwsum + 32);   // [8] k by word code

    const double scale_d = (double)cl_ro<FRESH>(S.dt) / (S.density * S.dx * S.dx);
    const float scale = (float)scale_d;
    if (tid < 8) ktab[tid] = (tid >= 1 && tid <= 4) ? 1.f / (float)tid : scale;

    // own cell l (0 <= l < nown) sits at index l + nj of r, s and wd and has
    // linear index cb + l
    auto own = [&](auto &&f) {
#pragma unroll
        for (int k = 0; k < K; k++) {
            const int l = tid + k * kClThreads;
            if (l < nown) f(k, l);
        }
    };
    // the sum over the cluster of two per-thread floats, as float pairs;
    // publishes this CTA's sums in slot `slot` (consecutive calls alternate)
    auto cluster_sum = [&](float v0, float v1, int slot) -> float4 {
        float2 a = make_float2(v0, 0.f), b = make_float2(v1, 0.f);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            a = cl_add(a, cl_shfl(a, o));
            b = cl_add(b, cl_shfl(b, o));
        }
        if (lane == 0) {
            wsum[warp] = a;
            wsum[32 + warp] = b;
        }
        __syncthreads();
        if (warp == 0) {
            a = lane < kClWarps ? wsum[lane] : make_float2(0.f, 0.f);
            b = lane < kClWarps ? wsum[32 + lane] : make_float2(0.f, 0.f);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                a = cl_add(a, cl_shfl(a, o));
                b = cl_add(b, cl_shfl(b, o));
            }
            if (lane == 0) part[slot] = make_float4(a.x, a.y, b.x, b.y);
        }
        cl.sync();
        if (warp == 0) {
            float2 ca = make_float2(0.f, 0.f), cbv = make_float2(0.f, 0.f);
            if (lane < C) {
                const float4 v = *cl.map_shared_rank(part + slot, lane);
                ca = make_float2(v.x, v.y);
                cbv = make_float2(v.z, v.w);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                ca = cl_add(ca, cl_shfl(ca, o));
                cbv = cl_add(cbv, cl_shfl(cbv, o));
            }
            if (lane == 0) bc[slot] = make_float4(ca.x, ca.y, cbv.x, cbv.y);
        }
        __syncthreads();
        return bc[slot];
    };
    // the FP64 sum over the cluster of one per-thread double
    auto cluster_dsum = [&](double v, int slot) -> double {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) dwsum[warp] = v;
        __syncthreads();
        if (warp == 0) {
            v = lane < kClWarps ? dwsum[lane] : 0.0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
            if (lane == 0) dpart[slot] = v;
        }
        cl.sync();
        if (warp == 0) {
            double t = lane < C ? *cl.map_shared_rank(dpart + slot, lane) : 0.0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
            if (lane == 0) dbc[slot] = t;
        }
        __syncthreads();
        return dbc[slot];
    };

    // (b - A x)(c) in FP64 from the global x (written by other CTAs of the
    // cluster before the last cluster barrier: read past L1)
    auto res64 = [&](int m, int c) -> double {
        const unsigned w = wd[m];
        const double xc = __ldcg(S.x + c);
        double ax = xc;
        if (w & 0x80u) {
            double nb = 0.0;
            if (w & 1u) nb += __ldcg(S.x + c - nj);
            if (w & 2u) nb += __ldcg(S.x + c + nj);
            if (w & 4u) nb += __ldcg(S.x + c - 1);
            if (w & 8u) nb += __ldcg(S.x + c + 1);
            ax = scale_d * ((double)((w >> 4) & 7u) * xc - nb);
        }
        return cl_ro<FRESH>(S.b + c) - ax;
    };
    // (A s) at own index m
    auto a32 = [&](int m) -> float {
        const unsigned w = wd[m];
        const float vc = s[m];
        if (!(w & 0x80u)) return vc;
        float nb = 0.f;
        if (w & 1u) nb += s[m - nj];
        if (w & 2u) nb += s[m + nj];
        if (w & 4u) nb += s[m - 1];
        if (w & 8u) nb += s[m + 1];
        return scale * ((float)((w >> 4) & 7u) * vc - nb);
    };
    // (K^T r) at index mn
    auto yv = [&](int mn, unsigned w) -> float {
        float v = r[mn];
        const float k = ktab[(w >> 10) & 7u];
        if (w & 0x100u) v = fmaf(k, r[mn + nj], v);
        if (w & 0x200u) v = fmaf(k, r[mn + 1], v);
        return v;
    };
    // (K K^T r) at own index m: K^T r at m and at its upper and left
    // neighbours, in the order of the two-pass form (y = K^T r, z = K y)
    auto zv = [&](int m) -> float {
        const unsigned w = wd[m];
        float v = yv(m, w);
        if (w & 0x80u) {
            if (w & 1u) {
                const unsigned wu = wd[m - nj];
                v = fmaf(ktab[(wu >> 10) & 7u], yv(m - nj, wu), v);
            }
            if (w & 4u) {
                const unsigned wl = wd[m - 1];
                v = fmaf(ktab[(wl >> 10) & 7u], yv(m - 1, wl), v);
            }
        }
        return v;
    };
    // keeps the first and the last own row of a per-cell value for the neighbours
    auto boundary = [&](float *dst, int l, float v) {
        if (l < nj) dst[l] = v;
        if (l >= nown - nj) dst[l - nown + 2 * nj] = v;
    };
    // r on the own rows and both halo rows = (float)(b - A x); FP64 r.r over own rows
    const int lo = has_up ? -nj : 0, hi = nown + (has_dn ? nj : 0);
    auto residual = [&]() -> double {
        double acc = 0.0;
        for (int l = lo + tid; l < hi; l += kClThreads) {
            const double rv = res64(l + nj, cb + l);
            r[l + nj] = (float)rv;
            if (l >= 0 && l < nown) acc = fma(rv, rv, acc);
        }
        return cluster_dsum(acc, 1);
    };

    // neighbours' boundary rows (valid once a cluster barrier has passed)
    const float *up_q = has_up ? cl.map_shared_rank(qb, rank - 1) + nj : nullptr; // their last row
    const float *dn_q = has_dn ? cl.map_shared_rank(qb, rank + 1) : nullptr;      // their first row
    const float *up_z = has_up ? cl.map_shared_rank(zb, rank - 1) + nj : nullptr;
    const float *dn_z = has_dn ? cl.map_shared_rank(zb, rank + 1) : nullptr;
    float *r_up = r, *r_dn = r + (size_t)(R + 1) * nj; // halo rows
    float *s_up = s, *s_dn = s + (size_t)(R + 1) * nj;

    // operator words of the own and halo rows (zero outside the grid); halo
    // rows outside the grid are never read, clear them anyway
    for (int l = -nj + tid; l < nown + nj; l += kClThreads)
        wd[l + nj] = (uint16_t)cl_word<FRESH>(S.info, cb + l, N, nj);
    for (int j = tid; j < nj; j += kClThreads) r_up[j] = r_dn[j] = s_up[j] = s_dn[j] = 0.f;
    // x = 0 (the reference clears the result) and ||b||^2
    double bsq = 0.0;
    for (int l = tid; l < nown; l += kClThreads) {
        S.x[cb + l] = 0.0;
        const double bv = cl_ro<FRESH>(S.b + cb + l);
        bsq = fma(bv, bv, bsq);
    }
    const double bb = cluster_dsum(bsq, 0);
    double rrt = residual();
    int total = 0, outer = 0;
    const double tol2 = P.tol * P.tol;
    while (!(bb == 0.0 || rrt <= tol2 * bb || total >= P.max_iter || outer >= P.max_outer)) {
        float d[K], t[K];
        // the inner solve needs to bring the residual just below the target:
        // its relative reduction, never below what FP32 iterations reach
        const double want = 0.3 * P.tol * sqrt(bb / rrt);
        const float eps = (float)fmin(fmax(want, (double)P.eps_in), 0.5);
        // r_0 = the outer residual, d = 0, z = M r, s = z
        float rz = 0.f, rr = 0.f;
        own([&](int k, int l) {
            const int m = l + nj;
            const float z = zv(m);
            const float rv = r[m];
            d[k] = 0.f;
            t[k] = z;
            rz = fmaf(rv, z, rz);
            rr = fmaf(rv, rv, rr);
            boundary(zb, l, z);
        });
        own([&](int k, int l) { s[l + nj] = t[k]; });
        const float4 s0 = cluster_sum(rz, rr, 1);
        float2 sigma = make_float2(s0.x, s0.y);
        const float rr0 = s0.z;
        for (int j = tid; j < nj; j += kClThreads) {
            if (has_up) s_up[j] = up_z[j];
            if (has_dn) s_dn[j] = dn_z[j];
        }
        __syncthreads();
        const float stop = eps * eps * rr0;
        const int limit = P.max_iter - total;
        int it = 0;
        while (rr0 > 0.f && it < limit) {
            // q = A s and s.q
            float sq = 0.f;
            own([&](int k, int l) {
                const int m = l + nj;
                const float q = a32(m);
                t[k] = q;
                sq = fmaf(s[m], q, sq);
                boundary(qb, l, q);
            });
            const float4 sa = cluster_sum(sq, 0.f, 0);
            const float alpha = cl_div(sigma, make_float2(sa.x, sa.y));
            // d += alpha s, r -= alpha q (own rows and the halo copies)
            own([&](int k, int l) {
                const int m = l + nj;
                d[k] = fmaf(alpha, s[m], d[k]);
                r[m] = fmaf(-alpha, t[k], r[m]);
            });
            for (int j = tid; j < nj; j += kClThreads) {
                if (has_up) r_up[j] = fmaf(-alpha, up_q[j], r_up[j]);
                if (has_dn) r_dn[j] = fmaf(-alpha, dn_q[j], r_dn[j]);
            }
            __syncthreads();
            // z = M r, r.z and r.r
            rz = 0.f;
            rr = 0.f;
            own([&](int k, int l) {
                const int m = l + nj;
                const float z = zv(m);
                const float rv = r[m];
                t[k] = z;
                rz = fmaf(rv, z, rz);
                rr = fmaf(rv, rv, rr);
                boundary(zb, l, z);
            });
            const float4 sb = cluster_sum(rz, rr, 1);
            it++;
            if (sb.z <= stop) break;
            const float beta = cl_div(make_float2(sb.x, sb.y), sigma);
            sigma = make_float2(sb.x, sb.y);
            // s = z + beta s (own rows and the halo copies)
            own([&](int k, int l) {
                const int m = l + nj;
                s[m] = fmaf(beta, s[m], t[k]);
            });
            for (int j = tid; j < nj; j += kClThreads) {
                if (has_up) s_up[j] = fmaf(beta, s_up[j], up_z[j]);
                if (has_dn) s_dn[j] = fmaf(beta, s_dn[j], dn_z[j]);
            }
            __syncthreads();
        }
        total += it;
        outer++;
        own([&](int k, int l) { S.x[cb + l] += (double)d[k]; });
        cl.sync(); // x complete before any CTA reads its neighbours' rows
        if (it == 0) break; // no progress possible; x and rrt unchanged
        rrt = residual();
    }
    if (rank == 0 && tid == 0) {
        *S.iters = total;
        *S.rel_res = bb > 0.0 ? sqrt(rrt / bb) : 0.0;
    }
    cl.sync(); // no CTA leaves while another may still read its shared memory
}

template <int K>
__global__ void __launch_bounds__(kClThreads, K >= 16 ? 1 : 2)
k_pcg_cluster(const ClusterSystem *__restrict__ systems, ClusterParams P)
{
    cluster_solve<K>(systems[blockIdx.x / cg::this_cluster().num_blocks()], P);
}

// ---------------------------------------------------------------------------
// The device-resident server (fs_server_*): a persistent launch whose
// clusters take requests from a ring the host fills in mapped pinned memory.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned sv_ld_acquire_sys(const unsigned *p)
{
    unsigned v;
    asm volatile("ld.acquire.sys.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void sv_st_release_sys(unsigned *p, unsigned v)
{
    asm volatile("st.release.sys.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// The packed operator byte of k_decomposition (fs_grid.cu) for one cell:
// non-solid neighbour count at bits 4-6, and for a fluid cell the unit bit
// and the fluid-neighbour mask with the linear-index bounds of
// getPressureProjectionMatrix (flipsolver2d.cpp:797-887); neighbours outside
// the grid read as the cell's nearest edge cell (OOB_EXTEND).
__device__ __forceinline__ uint8_t sv_operator_byte(const int8_t *__restrict__ m, int ni, int nj, int c)
{
    const int i = c / nj, j = c - i * nj;
    auto at = [&](int a, int b) { return __ldcg(m + (size_t)clampi(a, 0, ni - 1) * nj + clampi(b, 0, nj - 1)); };
    const int8_t mim = at(i - 1, j), mip = at(i + 1, j);
    const int8_t mjm = at(i, j - 1), mjp = at(i, j + 1);
    const int nsc = !t_solid(mim) + !t_solid(mip) + !t_solid(mjm) + !t_solid(mjp);
    uint8_t b = (uint8_t)(nsc << 4);
    const int N = ni * nj;
    if (t_fluid(__ldcg(m + c))) {
        b |= 0x80;
        if (t_fluid(mim) && c - nj >= 0) b |= 1;
        if (t_fluid(mip) && c + nj < N) b |= 2;
        if (t_fluid(mjm) && c - 1 >= 0) b |= 4;
        if (t_fluid(mjp) && c + 1 < N) b |= 8;
    }
    return b;
}

// rank 0 thread 0 of a cluster: the slot of the next request, or -1 when the
// host asked the server to stop or nothing arrived for q.idle_polls polls
__device__ int sv_claim(const ServeQueue &q)
{
    long long idle = 0;
    for (;;) {
        if (*((volatile const int *)q.stop)) return -1;
        const unsigned tail = sv_ld_acquire_sys(q.tail);
        const unsigned c = *((volatile unsigned *)q.claimed);
        if ((int)(tail - c) > 0) {
            if (atomicCAS(q.claimed, c, c + 1) == c) {
                const int slot = (int)*((volatile const unsigned *)(q.ring + (c % q.ring_size)));
                sv_st_release_sys(q.started + slot, c + 1);
                return slot;
            }
            continue; // another cluster took request c
        }
        if (++idle > q.idle_polls) return -1;
        __nanosleep(2000);
    }
}

template <int K>
__global__ void __launch_bounds__(kClThreads, K >= 16 ? 1 : 2) k_serve(ServeQueue q, ClusterParams P)
{
    cg::cluster_group cl = cg::this_cluster();
    const int C = (int)cl.num_blocks(), rank = (int)cl.block_rank();
    __shared__ int s_slot;
    for (;;) {
        if (rank == 0 && threadIdx.x == 0) s_slot = sv_claim(q);
        cl.sync();
        const int slot = *cl.map_shared_rank(&s_slot, 0);
        cl.sync(); // every CTA has its copy before rank 0 claims again
        if (slot < 0) break;
        // the slot as the host last wrote it (read past L1: the same slot
        // served other requests earlier in this launch)
        ServeSlot sl;
        {
            const unsigned long long *src = reinterpret_cast<const unsigned long long *>(q.slots + slot);
            unsigned long long *dst = reinterpret_cast<unsigned long long *>(&sl);
#pragma unroll
            for (int w = 0; w < (int)(sizeof(ServeSlot) / 8); w++) dst[w] = __ldcg(src + w);
        }
        const ClusterSystem S = sl.sys;
        // the operator bytes of the request's material, split over the CTAs
        const int N = S.ni * S.nj;
        const int c0 = (int)((long long)rank * N / C), c1 = (int)((long long)(rank + 1) * N / C);
        for (int c = c0 + (int)threadIdx.x; c < c1; c += blockDim.x)
            sl.info[c] = sv_operator_byte(sl.material, S.ni, S.nj, c);
        cl.sync(); // the whole operator before any CTA reads its halo rows
        cluster_solve<K, true>(S, P);
        if (rank == 0 && threadIdx.x == 0) {
            // x, the iterations and the residual are written (the solve's
            // last cluster barrier); make them visible to the host's copies
            __threadfence_system();
            sv_st_release_sys(q.done + slot, *((volatile unsigned *)(q.started + slot)));
        }
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
// per device: the largest cluster it co-schedules with full-size CTAs and
// the opt-in shared memory per CTA (-1: not yet probed).  Function
// attributes belong to a device's context, so they are set once per device.
struct ClDevice {
    int max_cluster = -1;
    size_t smem_limit = 0;
};
static std::mutex g_cl_mu;
static ClDevice g_cl[kMaxDevices];

template <int K> static void cl_set_attributes(int optin)
{
    const void *fn = (const void *)k_pcg_cluster<K>;
    cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
    cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
}

static ClDevice cl_probe(int dev)
{
    ClDevice d;
    int optin = 0;
    if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) {
        cudaGetLastError();
        d.max_cluster = 0;
        return d;
    }
    d.smem_limit = (size_t)optin;
    cl_set_attributes<8>(optin);
    cl_set_attributes<16>(optin);
    cl_set_attributes<32>(optin);
    d.max_cluster = 1;
    for (int C = 16; C >= 2; C /= 2) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(C);
        cfg.blockDim = dim3(kClThreads);
        cfg.dynamicSmemBytes = (size_t)optin;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = C;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        int nc = 0;
        if (cudaOccupancyMaxActiveClusters(&nc, (const void *)k_pcg_cluster<32>, &cfg) == cudaSuccess &&
            nc > 0) {
            d.max_cluster = C;
            break;
        }
        cudaGetLastError();
    }
    return d;
}

// the current device's cluster facts, probed on first use there
static ClDevice cl_init()
{
    const int dev = current_device();
    if (dev < 0) {
        cudaGetLastError();
        return ClDevice{0, 0};
    }
    if (dev >= kMaxDevices) return cl_probe(dev);
    std::lock_guard<std::mutex> lock(g_cl_mu);
    if (g_cl[dev].max_cluster < 0) g_cl[dev] = cl_probe(dev);
    return g_cl[dev];
}

// Rows split over C CTAs at floor(k ni / C), so every CTA has at most
// ceil(ni / C) rows and, for C <= ni, at least one.  The plan for one C, if
// its CTAs fit: the fewest cells per thread that hold the rows.
static bool cl_plan_c(int ni, int nj, int C, size_t smem_limit, ClusterPlan *out)
{
    if (C > ni) return false;
    const long long rows = (ni + C - 1) / C;
    const long long cells = rows * nj;
    if (cells > kClMaxOwn) return false;
    const size_t need = cl_vec_bytes((int)rows, nj) + kClTail;
    if (need > smem_limit) return false;
    out->C = C;
    out->K = cells <= 8 * kClThreads ? 8 : (cells <= 16 * kClThreads ? 16 : 32);
    out->smem = need;
    return true;
}

// the default: the smallest C whose CTAs fit (fewest CTAs for the work)
static bool cl_plan(int ni, int nj, int max_c, size_t smem_limit, ClusterPlan *out)
{
    for (int C = 1; C <= max_c; C *= 2)
        if (cl_plan_c(ni, nj, C, smem_limit, out)) return true;
    return false;
}

// plans chosen by the autotuner, by grid shape (this process)
static std::mutex g_tuned_mu;
static std::map<std::pair<int, int>, ClusterPlan> g_tuned;

bool cluster_plan(int ni, int nj, ClusterPlan *plan)
{
    const ClDevice D = cl_init();
    if (D.max_cluster <= 0 || ni < 1 || nj < 1) return false;
    {
        std::lock_guard<std::mutex> lock(g_tuned_mu);
        auto it = g_tuned.find({ni, nj});
        if (it != g_tuned.end()) {
            *plan = it->second;
            return true;
        }
    }
    return cl_plan(ni, nj, D.max_cluster, D.smem_limit, plan);
}

void cluster_candidates(int ni, int nj, std::vector<ClusterPlan> *out)
{
    const ClDevice D = cl_init();
    out->clear();
    for (int C = 1; C <= D.max_cluster; C *= 2) {
        ClusterPlan p;
        if (cl_plan_c(ni, nj, C, D.smem_limit, &p)) out->push_back(p);
    }
}

void cluster_set_tuned(int ni, int nj, const ClusterPlan &plan)
{
    std::lock_guard<std::mutex> lock(g_tuned_mu);
    g_tuned[{ni, nj}] = plan;
}

long long cluster_max_cells()
{
    const ClDevice D = cl_init();
    return D.max_cluster > 0 ? (long long)D.max_cluster * kClMaxOwn : 0;
}

template <int K>
static cudaError_t launch_k(const ClusterSystem *systems_dev, int n, int C, size_t smem,
                           const ClusterParams &p, cudaStream_t st)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)n * (unsigned)C);
    cfg.blockDim = dim3(kClThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = (unsigned)C;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    ClusterParams pp = p;
    return cudaLaunchKernelEx(&cfg, k_pcg_cluster<K>, systems_dev, pp);
}

template <int K> static cudaError_t launch_serve_k(const ServeQueue &q, const ClusterPlan &plan,
                                                  const ClusterParams &p, cudaStream_t st, int *clusters)
{
    const void *fn = (const void *)k_serve<K>;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)plan.smem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.blockDim = dim3(kClThreads);
    cfg.dynamicSmemBytes = plan.smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = (unsigned)plan.C;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    // as many clusters as fit at once: each loops over requests
    cfg.gridDim = dim3((unsigned)plan.C);
    int nc = 0;
    if ((e = cudaOccupancyMaxActiveClusters(&nc, fn, &cfg)) != cudaSuccess) return e;
    if (nc < 1) return cudaErrorInvalidConfiguration;
    cfg.gridDim = dim3((unsigned)(nc * plan.C));
    *clusters = nc;
    ServeQueue qq = q;
    ClusterParams pp = p;
    return cudaLaunchKernelEx(&cfg, k_serve<K>, qq, pp);
}

cudaError_t launch_serve(const ServeQueue &q, const ClusterPlan &plan, const ClusterParams &p, cudaStream_t st,
                         int *clusters)
{
    const ClDevice D = cl_init();
    if (plan.C < 1 || plan.C > D.max_cluster || plan.smem > D.smem_limit) return cudaErrorInvalidValue;
    switch (plan.K) {
    case 8: return launch_serve_k<8>(q, plan, p, st, clusters);
    case 16: return launch_serve_k<16>(q, plan, p, st, clusters);
    case 32: return launch_serve_k<32>(q, plan, p, st, clusters);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_pcg_cluster(const ClusterSystem *systems_dev, int n, const ClusterPlan &plan,
                               const ClusterParams &p, cudaStream_t st)
{
    const ClDevice D = cl_init();
    if (n <= 0) return cudaSuccess;
    if (plan.C < 1 || plan.C > D.max_cluster || plan.smem > D.smem_limit) return cudaErrorInvalidValue;
    switch (plan.K) {
    case 8: return launch_k<8>(systems_dev, n, plan.C, plan.smem, p, st);
    case 16: return launch_k<16>(systems_dev, n, plan.C, plan.smem, p, st);
    case 32: return launch_k<32>(systems_dev, n, plan.C, plan.smem, p, st);
    default: return cudaErrorInvalidValue;
    }
}

} // namespace fsg
