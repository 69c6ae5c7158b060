// fs_particles.cu -- per-particle and per-bin kernels of the FLIP substep:
// RK4 advection with solid push-out, the rebin (swap-erase prune + stable key
// sort of moved particles), the density push, G2P, countParticles erasure
// and the CFL velocity reduction.  Also the integer scan used by the rebin.
//
// Compiled with -fmad=false: every float expression is evaluated as the
// reference writes it (see fs_common.cuh), so positions, bins and the storage
// order match the reference bit for bit.
#include <cfloat>
#include <climits>
#include <cstdio>

#include "fs_state.h"

namespace fsg {

constexpr int kThreads = 256;

static inline int nblk(long long n, int t) { return (int)((n + t - 1) / t); }

// ---------------------------------------------------------------------------
// block scan helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ int warp_incl_scan(int v)
{
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

// exclusive scan across the block; returns the exclusive prefix, sets total
template <int BLOCK>
__device__ __forceinline__ int block_excl_scan(int v, int *sm_warp, int &total)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int inc = warp_incl_scan(v);
    if (lane == 31) sm_warp[w] = inc;
    __syncthreads();
    if (w == 0) {
        int x = lane < BLOCK / 32 ? sm_warp[lane] : 0;
        int xi = warp_incl_scan(x);
        if (lane < BLOCK / 32) sm_warp[lane] = xi - x;
        if (lane == BLOCK / 32 - 1) sm_warp[32] = xi;
    }
    __syncthreads();
    int res = inc - v + sm_warp[w];
    total = sm_warp[32];
    __syncthreads();
    return res;
}

// ---------------------------------------------------------------------------
// exclusive scan of n ints: tile sums -> scan of tile sums -> tile scans
// ---------------------------------------------------------------------------
constexpr int kScanBlock = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanBlock * kScanItems;

__global__ void k_scan_tile_sums(const int *__restrict__ in, int n, int *__restrict__ sums)
{
    __shared__ int sw[33];
    const int base = blockIdx.x * kScanTile;
    int s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        int idx = base + k * kScanBlock + threadIdx.x;
        if (idx < n) s += in[idx];
    }
    int total;
    block_excl_scan<kScanBlock>(s, sw, total);
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void k_scan_sums(int *sums, int ntiles)
{
    __shared__ int sw[33];
    int carry = 0;
    for (int base = 0; base < ntiles; base += kScanBlock) {
        int idx = base + threadIdx.x;
        int v = idx < ntiles ? sums[idx] : 0;
        int total;
        int ex = block_excl_scan<kScanBlock>(v, sw, total);
        if (idx < ntiles) sums[idx] = ex + carry;
        carry += total;
    }
    if (threadIdx.x == 0) sums[ntiles] = carry;
}

__global__ void k_scan_tiles(const int *__restrict__ in, int *__restrict__ out, int n,
                             const int *__restrict__ sums, int ntiles)
{
    __shared__ int sw[33];
    const int base = blockIdx.x * kScanTile;
    // each thread owns kScanItems consecutive items
    int vals[kScanItems];
    int s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        int idx = base + threadIdx.x * kScanItems + k;
        vals[k] = idx < n ? in[idx] : 0;
        s += vals[k];
    }
    int total;
    int ex = block_excl_scan<kScanBlock>(s, sw, total) + sums[blockIdx.x];
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        int idx = base + threadIdx.x * kScanItems + k;
        if (idx < n) out[idx] = ex;
        ex += vals[k];
    }
    if (blockIdx.x == ntiles - 1 && threadIdx.x == 0) out[n] = sums[ntiles];
}

size_t scan_scratch_bytes(int n) { return (size_t)(nblk(n, kScanTile) + 1) * sizeof(int); }

void scan_exclusive(const int *in, int *out, int n, void *scratch, cudaStream_t st)
{
    int ntiles = nblk(n > 0 ? n : 1, kScanTile);
    int *sums = (int *)scratch;
    k_scan_tile_sums<<<ntiles, kScanBlock, 0, st>>>(in, n, sums);
    k_scan_sums<<<1, kScanBlock, 0, st>>>(sums, ntiles);
    k_scan_tiles<<<ntiles, kScanBlock, 0, st>>>(in, out, n, sums, ntiles);
}

// ---------------------------------------------------------------------------
// advection: FlipSolver::advectThread (flipsolver2d.cpp:305-338)
// ---------------------------------------------------------------------------
// SdfGrid::closestSurfacePoint (sdfgrid.cpp:15-46) with
// simmath::gradCenteredGrid (mathfuncs.cpp:87-98): float coordinates are
// truncated toward zero when passed as the gradient's integer cell.
__device__ __forceinline__ float2 grad_centered(const float *__restrict__ g, int si, int sj,
                                               long long i, long long j)
{
    return make_float2((gget(g, si, sj, i + 1, j) - gget(g, si, sj, i - 1, j)) / 2.f,
                       (gget(g, si, sj, i, j + 1) - gget(g, si, sj, i, j - 1)) / 2.f);
}

__device__ float2 closest_surface_point(const float *__restrict__ g, const GridDims &d, float2 p)
{
    const int si = d.ni, sj = d.nj;
    float cx = p.x, cy = p.y;
    float value = grid_lerp(g, si, sj, 0.f, 0.f, cx, cy);
    float2 gr = grad_centered(g, si, sj, (long long)cx, (long long)cy);
    for (int it = 0; it < 100; it++) {
        float alpha = 1;
        for (int jt = 0; jt < 10; jt++) {
            float av = alpha * value;
            float qx = cx - gr.x * av, qy = cy - gr.y * av;
            float vq = grid_lerp(g, si, sj, 0.f, 0.f, qx, qy);
            if (fabsf(vq) < fabsf(value)) {
                cx = qx;
                cy = qy;
                value = vq;
                gr = grad_centered(g, si, sj, (long long)qx, (long long)qy);
                if (fabsf(value) < 1e-5f) return make_float2(cx, cy);
            } else {
                alpha *= 0.7f;
            }
        }
    }
    return make_float2(cx, cy);
}

__global__ void k_advect(GridDims d, Particles P, const float *__restrict__ u,
                         const float *__restrict__ v, const float *__restrict__ solid_sdf,
                         const int8_t *__restrict__ material, const Scalars *__restrict__ sc)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    const int nslots = P.bin_start[P.nbins];
    if (s >= nslots) return;
    const int b = P.slot_bin[s];
    if (s - P.bin_start[b] >= P.bin_count[b]) {
        P.flag[s] = P_GAP;
        return;
    }
    const float dt = sc->dt;
    float2 p = P.pos[s];
    const int oldBin = bin_of_pos(d, p.x, p.y);
    // FlipSolver::rk4Integrate (flipsolver2d.cpp:1195-1203)
    float2 k = velocity_at(u, v, d, p.x, p.y);
    float k1x = k.x * dt, k1y = k.y * dt;
    k = velocity_at(u, v, d, p.x + k1x * 0.5f, p.y + k1y * 0.5f);
    float k2x = k.x * dt, k2y = k.y * dt;
    k = velocity_at(u, v, d, p.x + k2x * 0.5f, p.y + k2y * 0.5f);
    float k3x = k.x * dt, k3y = k.y * dt;
    k = velocity_at(u, v, d, p.x + k3x, p.y + k3y);
    float k4x = k.x * dt, k4y = k.y * dt;
    float sx = ((k1x + k2x * 2.f) + k3x * 2.f) + k4x;
    float sy = ((k1y + k2y * 2.f) + k3y * 2.f) + k4y;
    p.x = p.x + sx * (1.0f / 6.0f);
    p.y = p.y + sy * (1.0f / 6.0f);
    if (grid_lerp(solid_sdf, d.ni, d.nj, 0.f, 0.f, p.x, p.y) < 0.f)
        p = closest_surface_point(solid_sdf, d, p);
    P.pos[s] = p;
    const int pI = sm_integr(p.x), pJ = sm_integr(p.y);
    const int newBin = bin_of_pos(d, p.x, p.y);
    const bool inb = pI >= 0 && pI < d.ni && pJ >= 0 && pJ < d.nj;
    if (!inb || t_sink(mat_at(material, d, pI, pJ))) {
        P.flag[s] = P_KILL;
    } else if (newBin != oldBin) {
        P.flag[s] = P_MOVE;
        P.dest[s] = newBin;
    } else {
        P.flag[s] = P_STAY;
    }
}

void launch_advect(const GridDims &d, const Particles &P, const Grids &G, const Scalars *sc,
                   cudaStream_t st)
{
    if (P.cap == 0) return;
    k_advect<<<nblk(P.bound, kThreads), kThreads, 0, st>>>(d, P, G.u, G.v, G.solid_sdf,
                                                         G.material, sc);
}

// ---------------------------------------------------------------------------
// rebin = FlipSolver::pruneParticles + MarkerParticleSystem::rebinParticles
// (flipsolver2d.cpp:353-359, markerparticlesystem.cpp:47-58, 248-269)
// ---------------------------------------------------------------------------
// Per bin: ParticleBin::pruneParticles swap-erases every marked particle
// (killed or moved).  Its result is: survivors in [0, k) keep their slot;
// the holes in [0, k) are filled, in ascending order, by the survivors found
// in [k, n) taken from the back.  k = number of survivors.
__global__ void k_prune(Particles P)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= P.nbins) return;
    const int st = P.bin_start[b], n = P.bin_count[b];
    const uint8_t *f = P.flag + st;
    int k = 0;
    for (int i = 0; i < n; i++) k += (f[i] == P_STAY);
    int hi = n - 1;
    for (int i = 0; i < k; i++) {
        if (f[i] == P_STAY) {
            P.prune_slot[st + i] = i;
        } else {
            // a survivor exists in [k, n) for every hole in [0, k); the bound
            // only guards against inconsistent flags
            while (hi >= k && f[hi] != P_STAY) hi--;
            if (hi < k) break;
            P.prune_slot[st + hi] = i;
            hi--;
        }
    }
    P.survivors[b] = k;
    P.incoming[b] = 0;
}

// stable compaction of moved particles in slot order: count per tile
__global__ void k_moved_tile_counts(const Particles P, int *__restrict__ tile_counts)
{
    __shared__ int sw[33];
    const int nslots = P.bin_start[P.nbins];
    const int base = blockIdx.x * kScanTile;
    int c = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        int s = base + threadIdx.x * kScanItems + k;
        if (s < nslots && P.flag[s] == P_MOVE) c++;
    }
    int total;
    block_excl_scan<kScanBlock>(c, sw, total);
    if (threadIdx.x == 0) tile_counts[blockIdx.x] = total;
}

__global__ void k_moved_write(Particles P, const int *__restrict__ tile_off)
{
    __shared__ int sw[33];
    const int nslots = P.bin_start[P.nbins];
    const int base = blockIdx.x * kScanTile;
    int c = 0;
    uint8_t fl[kScanItems];
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        int s = base + threadIdx.x * kScanItems + k;
        fl[k] = (s < nslots) ? P.flag[s] : (uint8_t)P_GAP;
        c += (fl[k] == P_MOVE);
    }
    int total;
    int off = block_excl_scan<kScanBlock>(c, sw, total) + tile_off[blockIdx.x];
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        int s = base + threadIdx.x * kScanItems + k;
        if (fl[k] == P_MOVE) {
            int dst = P.dest[s];
            P.mkey[off] = dst;
            P.mval[off] = s;
            atomicAdd(&P.incoming[dst], 1); // order-independent count
            off++;
        }
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) *P.nmoved = tile_off[gridDim.x];
}

// --- stable LSD radix sort of (dest bin, slot) pairs, 8-bit digits --------
constexpr int kRadixBlock = 1024;
constexpr int kRadixItems = 4;
constexpr int kRadixTile = kRadixBlock * kRadixItems;

__global__ void k_radix_hist(const int *__restrict__ keys, const int *__restrict__ nptr, int shift,
                             int *__restrict__ hist, int ntiles)
{
    __shared__ int h[256];
    const int n = *nptr;
    for (int i = threadIdx.x; i < 256; i += blockDim.x) h[i] = 0;
    __syncthreads();
    const int base = blockIdx.x * kRadixTile;
    for (int k = 0; k < kRadixItems; k++) {
        int idx = base + k * kRadixBlock + threadIdx.x;
        if (idx < n) atomicAdd(&h[(keys[idx] >> shift) & 255], 1);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 256; i += blockDim.x) hist[i * ntiles + blockIdx.x] = h[i];
}

__global__ void k_radix_scatter(const int *__restrict__ kin, const int *__restrict__ vin,
                                int *__restrict__ kout, int *__restrict__ vout,
                                const int *__restrict__ nptr, int shift,
                                const int *__restrict__ hist_off, int ntiles)
{
    __shared__ int running[256];
    __shared__ int rtot[256];
    __shared__ int wcount[kRadixBlock / 32][256];
    const int n = *nptr;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < 256; i += blockDim.x) running[i] = hist_off[i * ntiles + blockIdx.x];
    const int base = blockIdx.x * kRadixTile;
    // items are ranked in index order: round by round, warp by warp, lane by lane
    for (int r = 0; r < kRadixItems; r++) {
        for (int i = threadIdx.x; i < (kRadixBlock / 32) * 256; i += blockDim.x)
            (&wcount[0][0])[i] = 0;
        __syncthreads();
        const int idx = base + r * kRadixBlock + threadIdx.x;
        const bool valid = idx < n;
        const int key = valid ? kin[idx] : 0;
        const int digit = valid ? ((key >> shift) & 255) : 256 + lane; // invalid lanes stay alone
        const unsigned peers = __match_any_sync(0xffffffffu, digit);
        const int rank = __popc(peers & ((1u << lane) - 1u));
        if (valid && rank == 0) wcount[w][digit] = __popc(peers);
        __syncthreads();
        if (threadIdx.x < 256) {
            int acc = 0;
            for (int ww = 0; ww < kRadixBlock / 32; ww++) {
                int c = wcount[ww][threadIdx.x];
                wcount[ww][threadIdx.x] = acc;
                acc += c;
            }
            rtot[threadIdx.x] = acc;
        }
        __syncthreads();
        if (valid) {
            const int pos = running[digit] + wcount[w][digit] + rank;
            kout[pos] = key;
            vout[pos] = vin[idx];
        }
        __syncthreads();
        if (threadIdx.x < 256) running[threadIdx.x] += rtot[threadIdx.x];
        __syncthreads();
    }
}

struct RebinScratch {
    int *tile_counts; // moved compaction tile offsets (ntiles + 1)
    int *hist;        // 256 * rtiles (+1)
    void *scan_tmp;
};

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

size_t rebin_scratch_bytes(const Particles &P)
{
    int ntiles = nblk(P.cap > 0 ? P.cap : 1, kScanTile);
    int rtiles = nblk(P.cap > 0 ? P.cap : 1, kRadixTile);
    size_t b = align256((size_t)(ntiles + 1) * sizeof(int));
    b += align256((size_t)(256 * rtiles + 1) * sizeof(int));
    int nscan = 256 * rtiles;
    if (P.nbins + 1 > nscan) nscan = P.nbins + 1;
    if (ntiles + 1 > nscan) nscan = ntiles + 1;
    b += align256(scan_scratch_bytes(nscan));
    return b;
}

__global__ void k_new_counts(Particles P)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= P.nbins) return;
    P.bin_count2[b] = P.survivors[b] + P.incoming[b];
}

__global__ void k_scatter_survivors(Particles P)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    const int nslots = P.bin_start[P.nbins];
    if (s >= nslots || P.flag[s] != P_STAY) return;
    const int b = P.slot_bin[s];
    const int dst = P.bin_start2[b] + P.prune_slot[s];
    P.pos2[dst] = P.pos[s];
    P.vel2[dst] = P.vel[s];
    P.visc2[dst] = P.visc[s];
    P.slot_bin2[dst] = b;
}

__global__ void k_scatter_incoming(Particles P)
{
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= *P.nmoved) return;
    const int d = P.mkey[m], s = P.mval[m];
    // rank among particles moving to d = m - first sorted position of d
    const int dst = P.bin_start2[d] + P.survivors[d] + (m - P.inc_off[d]);
    P.pos2[dst] = P.pos[s];
    P.vel2[dst] = P.vel[s];
    P.visc2[dst] = P.visc[s];
    P.slot_bin2[dst] = d;
}

void launch_rebin(const GridDims &d, Particles &P, void *scratch, size_t, cudaStream_t st)
{
    if (P.cap == 0) return;
    // scratch laid out for the capacity, launches sized for the bound
    char *p = (char *)scratch;
    int *tile_counts = (int *)p;
    p += align256((size_t)(nblk(P.cap, kScanTile) + 1) * sizeof(int));
    int *hist = (int *)p;
    p += align256((size_t)(256 * nblk(P.cap, kRadixTile) + 1) * sizeof(int));
    void *scan_tmp = p;
    const int ntiles = nblk(P.bound, kScanTile);
    const int rtiles = nblk(P.bound, kRadixTile);

    k_prune<<<nblk(P.nbins, kThreads), kThreads, 0, st>>>(P);
    k_moved_tile_counts<<<ntiles, kScanBlock, 0, st>>>(P, tile_counts);
    scan_exclusive(tile_counts, tile_counts, ntiles, scan_tmp, st);
    k_moved_write<<<ntiles, kScanBlock, 0, st>>>(P, tile_counts);

    // LSD passes over the bits needed for bin indices
    int bits = 0;
    while ((1 << bits) < P.nbins) bits++;
    int *kin = P.mkey, *vin = P.mval, *kout = P.mkey2, *vout = P.mval2;
    for (int shift = 0; shift < bits; shift += 8) {
        k_radix_hist<<<rtiles, kRadixBlock, 0, st>>>(kin, P.nmoved, shift, hist, rtiles);
        scan_exclusive(hist, hist, 256 * rtiles, scan_tmp, st);
        k_radix_scatter<<<rtiles, kRadixBlock, 0, st>>>(kin, vin, kout, vout, P.nmoved, shift,
                                                        hist, rtiles);
        int *t = kin; kin = kout; kout = t;
        t = vin; vin = vout; vout = t;
    }
    if (kin != P.mkey) { // keep the sorted list in mkey/mval
        int *t = P.mkey; P.mkey = P.mkey2; P.mkey2 = t;
        t = P.mval; P.mval = P.mval2; P.mval2 = t;
    }
    // first sorted position of each destination bin
    scan_exclusive(P.incoming, P.inc_off, P.nbins, scan_tmp, st);
    k_new_counts<<<nblk(P.nbins, kThreads), kThreads, 0, st>>>(P);
    scan_exclusive(P.bin_count2, P.bin_start2, P.nbins, scan_tmp, st);
    k_scatter_survivors<<<nblk(P.bound, kThreads), kThreads, 0, st>>>(P);
    k_scatter_incoming<<<nblk(P.bound, kThreads), kThreads, 0, st>>>(P);
    // swap buffers
    float2 *tp;
    tp = P.pos; P.pos = P.pos2; P.pos2 = tp;
    tp = P.vel; P.vel = P.vel2; P.vel2 = tp;
    float *tf = P.visc; P.visc = P.visc2; P.visc2 = tf;
    int *ti = P.slot_bin; P.slot_bin = P.slot_bin2; P.slot_bin2 = ti;
    ti = P.bin_start; P.bin_start = P.bin_start2; P.bin_start2 = ti;
    ti = P.bin_count; P.bin_count = P.bin_count2; P.bin_count2 = ti;
}

// ---------------------------------------------------------------------------
// NB-FLIP reseeding, append side (nbflipsolver.cpp:118-201): kept candidates
// are appended to their bins in candidate (row-major cell, then draw) order,
// as ParticleBin::addMarkerParticle pushes them back one by one.  Existing
// particles keep their order; the layout is rebuilt without gaps.
// ---------------------------------------------------------------------------
__global__ void k_nb_bins_init(Particles P)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= P.nbins) return;
    P.survivors[b] = P.bin_count[b];
    P.incoming[b] = 0;
}

// stable compaction of kept candidates in candidate order: count per tile
__global__ void k_nb_keep_tile_counts(const int *__restrict__ cand_bin, const int *__restrict__ nptr,
                                      int *__restrict__ tile_counts)
{
    __shared__ int sw[33];
    const int n = *nptr;
    const int base = blockIdx.x * kScanTile;
    int c = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        const int e = base + threadIdx.x * kScanItems + k;
        if (e < n && cand_bin[e] >= 0) c++;
    }
    int total;
    block_excl_scan<kScanBlock>(c, sw, total);
    if (threadIdx.x == 0) tile_counts[blockIdx.x] = total;
}

__global__ void k_nb_keep_write(Particles P, const int *__restrict__ cand_bin,
                                const int *__restrict__ nptr, const int *__restrict__ tile_off)
{
    __shared__ int sw[33];
    const int n = *nptr;
    const int base = blockIdx.x * kScanTile;
    int c = 0;
    int bk[kScanItems];
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        const int e = base + threadIdx.x * kScanItems + k;
        bk[k] = e < n ? cand_bin[e] : -1;
        c += bk[k] >= 0;
    }
    int total;
    int off = block_excl_scan<kScanBlock>(c, sw, total) + tile_off[blockIdx.x];
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        if (bk[k] >= 0) {
            P.mkey[off] = bk[k];
            P.mval[off] = base + threadIdx.x * kScanItems + k;
            atomicAdd(&P.incoming[bk[k]], 1); // order-independent count
            off++;
        }
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) *P.nmoved = tile_off[gridDim.x];
}

// every live particle to the same place in its bin of the new layout (a
// layout beyond the capacity -- possible only for a state loaded with more
// than 2 particlesPerCell in a cell and reseeded without counting -- is not
// written and raises the status)
__global__ void k_nb_scatter_live(Particles P, int *status)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= P.bin_start[P.nbins]) return;
    if (P.bin_start2[P.nbins] > P.cap) {
        if (s == 0) atomicExch(status, 1);
        return;
    }
    const int b = P.slot_bin[s];
    const int r = s - P.bin_start[b];
    if (r >= P.bin_count[b]) return;
    const int dst = P.bin_start2[b] + r;
    P.pos2[dst] = P.pos[s];
    P.vel2[dst] = P.vel[s];
    P.visc2[dst] = P.visc[s];
    P.slot_bin2[dst] = b;
}

// the kept candidates after them (velocity and viscosity as placed); the
// viscosity goes through the cell's bin,
// so a particle whose position lies in another bin keeps 0 (the fix-up
// below stores its viscosity where the reference does)
__global__ void k_nb_scatter_new(Particles P, NbReseed R)
{
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= *P.nmoved || P.bin_start2[P.nbins] > P.cap) return;
    const int d = P.mkey[m], k = P.mval[m];
    const int dst = P.bin_start2[d] + P.survivors[d] + (m - P.inc_off[d]);
    P.pos2[dst] = R.cand_pos[k];
    P.vel2[dst] = R.cand_vel[k];
    P.visc2[dst] = R.cand_cb[k] == d ? R.cand_visc[k] : 0.f;
    P.slot_bin2[dst] = d;
    R.pos_of[k] = m;
}

// The reference stores a reseeded particle's viscosity in the property
// vector of the cell's bin at the index the position's bin returned
// (nbflipsolver.cpp:190-194); where the two bins differ (i + U(0,1) rounded
// into the next bin) that overwrites an earlier particle of the cell's bin,
// if the index exists there at that moment.  These cases are rare; one
// thread replays them in candidate order.
__global__ void k_nb_cross_fix(Particles P, NbReseed R)
{
    if (P.bin_start2[P.nbins] > P.cap) return;
    const int n = min(*R.cross_n, kNbCrossMax);
    if (*R.cross_n > kNbCrossMax) atomicExch(R.status, 1);
    for (int a = 1; a < n; a++) { // insertion sort: the list is short
        const int v = R.cross[a];
        int b = a - 1;
        while (b >= 0 && R.cross[b] > v) {
            R.cross[b + 1] = R.cross[b];
            b--;
        }
        R.cross[b + 1] = v;
    }
    for (int a = 0; a < n; a++) {
        const int k = R.cross[a];
        const int pb = R.cand_bin[k], cb = R.cand_cb[k];
        const int pidx = P.survivors[pb] + (R.pos_of[k] - P.inc_off[pb]);
        // the cell's bin at that moment: its old particles and its kept
        // candidates that come before k (sorted by candidate index)
        int lo = P.inc_off[cb], hi = P.inc_off[cb] + P.incoming[cb];
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (P.mval[mid] < k) lo = mid + 1;
            else hi = mid;
        }
        const int size = P.survivors[cb] + (lo - P.inc_off[cb]);
        if (pidx < size) P.visc2[P.bin_start2[cb] + pidx] = R.cand_visc[k];
    }
}

void launch_nb_append(Particles &P, const NbReseed &R, int ncand, void *scratch,
                      cudaStream_t st)
{
    if (P.cap == 0 || ncand <= 0) return;
    char *p = (char *)scratch;
    int *tile_counts = (int *)p;
    p += align256((size_t)(nblk(P.cap, kScanTile) + 1) * sizeof(int));
    int *hist = (int *)p;
    p += align256((size_t)(256 * nblk(P.cap, kRadixTile) + 1) * sizeof(int));
    void *scan_tmp = p;
    // the candidates and the occupied slots are known bounds here
    const int ntiles = nblk(ncand, kScanTile);
    const int rtiles = nblk(ncand, kRadixTile);
    const int *ncand_dev = R.cand_off + R.ncell;

    k_nb_bins_init<<<nblk(P.nbins, kThreads), kThreads, 0, st>>>(P);
    k_nb_keep_tile_counts<<<ntiles, kScanBlock, 0, st>>>(R.cand_bin, ncand_dev, tile_counts);
    scan_exclusive(tile_counts, tile_counts, ntiles, scan_tmp, st);
    k_nb_keep_write<<<ntiles, kScanBlock, 0, st>>>(P, R.cand_bin, ncand_dev, tile_counts);
    int bits = 0;
    while ((1 << bits) < P.nbins) bits++;
    int *kin = P.mkey, *vin = P.mval, *kout = P.mkey2, *vout = P.mval2;
    for (int shift = 0; shift < bits; shift += 8) {
        k_radix_hist<<<rtiles, kRadixBlock, 0, st>>>(kin, P.nmoved, shift, hist, rtiles);
        scan_exclusive(hist, hist, 256 * rtiles, scan_tmp, st);
        k_radix_scatter<<<rtiles, kRadixBlock, 0, st>>>(kin, vin, kout, vout, P.nmoved, shift,
                                                        hist, rtiles);
        int *t = kin; kin = kout; kout = t;
        t = vin; vin = vout; vout = t;
    }
    if (kin != P.mkey) {
        int *t = P.mkey; P.mkey = P.mkey2; P.mkey2 = t;
        t = P.mval; P.mval = P.mval2; P.mval2 = t;
    }
    scan_exclusive(P.incoming, P.inc_off, P.nbins, scan_tmp, st);
    k_new_counts<<<nblk(P.nbins, kThreads), kThreads, 0, st>>>(P);
    scan_exclusive(P.bin_count2, P.bin_start2, P.nbins, scan_tmp, st);
    k_nb_scatter_live<<<nblk(P.bound, kThreads), kThreads, 0, st>>>(P, R.status);
    k_nb_scatter_new<<<nblk(ncand, kThreads), kThreads, 0, st>>>(P, R);
    k_nb_cross_fix<<<1, 1, 0, st>>>(P, R);
    float2 *tp;
    tp = P.pos; P.pos = P.pos2; P.pos2 = tp;
    tp = P.vel; P.vel = P.vel2; P.vel2 = tp;
    float *tf = P.visc; P.visc = P.visc2; P.visc2 = tf;
    int *ti = P.slot_bin; P.slot_bin = P.slot_bin2; P.slot_bin2 = ti;
    ti = P.bin_start; P.bin_start = P.bin_start2; P.bin_start2 = ti;
    ti = P.bin_count; P.bin_count = P.bin_count2; P.bin_count2 = ti;
    const long long nb = (long long)P.bound + ncand;
    P.bound = nb < (long long)P.cap ? (int)nb : P.cap;
}

// ---------------------------------------------------------------------------
// particle state to and from the host in bin order (fs_get/set_particles)
// ---------------------------------------------------------------------------
// the live particles of every bin, packed in bin order at off[b]
__global__ void k_gather_bins(Particles P, const int *__restrict__ off, float2 *__restrict__ pos_out,
                              float2 *__restrict__ vel_out, float *__restrict__ visc_out)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= P.nbins) return;
    const int s0 = P.bin_start[b], n = P.bin_count[b], o = off[b];
    for (int k = 0; k < n; k++) {
        pos_out[o + k] = P.pos[s0 + k];
        vel_out[o + k] = P.vel[s0 + k];
        visc_out[o + k] = P.visc[s0 + k];
    }
}

// the bin of every occupied slot
__global__ void k_slot_bin(Particles P)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= P.nbins) return;
    const int s0 = P.bin_start[b], n = P.bin_count[b];
    for (int k = 0; k < n; k++) P.slot_bin[s0 + k] = b;
}

// packs the particles into pos2 / vel2 / visc2 (free outside a substep) with
// the bin offsets in bin_start2; off[nbins] is the total
void launch_gather_bins(const Particles &P, void *scratch, cudaStream_t st)
{
    const int ntiles = nblk(P.cap > 0 ? P.cap : 1, kScanTile);
    const int rtiles = nblk(P.cap > 0 ? P.cap : 1, kRadixTile);
    char *p = (char *)scratch;
    p += align256((size_t)(ntiles + 1) * sizeof(int));
    p += align256((size_t)(256 * rtiles + 1) * sizeof(int));
    scan_exclusive(P.bin_count, P.bin_start2, P.nbins, p, st);
    k_gather_bins<<<nblk(P.nbins, kThreads), kThreads, 0, st>>>(P, P.bin_start2, P.pos2, P.vel2, P.visc2);
}

void launch_slot_bin(const Particles &P, cudaStream_t st)
{
    k_slot_bin<<<nblk(P.nbins, kThreads), kThreads, 0, st>>>(P);
}

// ---------------------------------------------------------------------------
// density push: FlipSolver::adjustParticlesByDensityThread (:261-303)
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_adjust(GridDims d, Particles P, const T *__restrict__ p,
                         const int8_t *__restrict__ material, double density, double dx,
                         const Scalars *__restrict__ sc, int iter_limit)
{
    if (sc->density_iters >= iter_limit) return; // the reference skips the push (:179-182)
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    const int nslots = P.bin_start[P.nbins];
    if (s >= nslots) return;
    const int b = P.slot_bin[s];
    if (s - P.bin_start[b] >= P.bin_count[b]) return;
    const float dt = sc->dt;
    const float scale = (float)((double)(dt * dt) / (density * dx * dx));
    float2 q = P.pos[s];
    const int iCorr = clampi((int)(q.x - 0.5f), 0, d.ni);
    const int jCorr = clampi((int)(q.y - 0.5f), 0, d.nj);
    const int i = clampi((int)q.x, 0, d.ni);
    const int j = clampi((int)q.y, 0, d.nj);
    auto P_at = [&](int a, int c) -> float {
        // linearIndex is -1 outside the grid, where the reference reads before
        // its vector; such reads are taken as 0 here
        if (a < 0 || a >= d.ni || c < 0 || c >= d.nj) return 0.f;
        return (float)p[(size_t)a * d.nj + c];
    };
    float pCurrentI = P_at(iCorr, j);
    float pCurrentJ = P_at(i, jCorr);
    float pI = P_at(iCorr + 1, j);
    float pJ = P_at(i, jCorr + 1);
    if (t_solid(mat_at(material, d, iCorr + 1, j)) || t_solid(mat_at(material, d, iCorr, j)))
        pI = pCurrentI;
    if (t_solid(mat_at(material, d, i, jCorr + 1)) || t_solid(mat_at(material, d, i, jCorr)))
        pJ = pCurrentJ;
    float gu = pI - pCurrentI, gv = pJ - pCurrentJ;
    q.x = q.x + gu * scale;
    q.y = q.y + gv * scale;
    P.pos[s] = q;
}

void launch_adjust(const GridDims &d, const SceneParams &sp, const Particles &P, const Grids &G,
                   const void *pressure, int is_double, const Scalars *sc, cudaStream_t st)
{
    if (P.cap == 0) return;
    if (is_double)
        k_adjust<double><<<nblk(P.bound, kThreads), kThreads, 0, st>>>(
            d, P, (const double *)pressure, G.material, sp.fluidDensity, sp.dx, sc,
            sp.pcgIterLimit);
    else
        k_adjust<float><<<nblk(P.bound, kThreads), kThreads, 0, st>>>(
            d, P, (const float *)pressure, G.material, sp.fluidDensity, sp.dx, sc,
            sp.pcgIterLimit);
}

// ---------------------------------------------------------------------------
// G2P: FlipSolver::particleUpdate (flipsolver2d.cpp:361-388)
// ---------------------------------------------------------------------------
__global__ void k_g2p(GridDims d, Particles P, const float *__restrict__ u,
                      const float *__restrict__ v, const float *__restrict__ su,
                      const float *__restrict__ sv, float pic, Scalars *__restrict__ sc)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    const int nslots = P.bin_start[P.nbins];
    if (s >= nslots) return;
    const int b = P.slot_bin[s];
    if (s - P.bin_start[b] >= P.bin_count[b]) return;
    const float2 q = P.pos[s];
    const float ox = grid_lerp(su, d.ni + 1, d.nj, 0.5f, 0.f, q.x, q.y);
    const float oy = grid_lerp(sv, d.ni, d.nj + 1, 0.f, 0.5f, q.x, q.y);
    const float2 nv = velocity_at(u, v, d, q.x, q.y);
    float2 vel = P.vel[s];
    const float ax = nv.x * pic, ay = nv.y * pic;
    const float tx = (vel.x + nv.x) - ox, ty = (vel.y + nv.y) - oy;
    const float flip = 1.f - pic;
    vel.x = ax + tx * flip;
    vel.y = ay + ty * flip;
    P.vel[s] = vel;
    // the substep's sentinel: every particle velocity it leaves is finite
    // (isfinite of NaN and of +-inf is false); one flag word, set rarely
    if (!(isfinite(vel.x) && isfinite(vel.y))) atomicOr(&sc->nonfinite, 1);
}

void launch_g2p(const GridDims &d, const SceneParams &sp, const Particles &P, const Grids &G,
                Scalars *sc, cudaStream_t st)
{
    if (P.cap == 0) return;
    k_g2p<<<nblk(P.bound, kThreads), kThreads, 0, st>>>(d, P, G.u, G.v, G.su, G.sv, sp.picRatio, sc);
}

// ---------------------------------------------------------------------------
// FlipSolver::countParticles (flipsolver2d.cpp:1021-1051), one thread per bin
// ---------------------------------------------------------------------------
__device__ __forceinline__ void swap_erase(Particles &P, int st, int k, int last)
{
    float2 tp = P.pos[st + k]; P.pos[st + k] = P.pos[st + last]; P.pos[st + last] = tp;
    float2 tv = P.vel[st + k]; P.vel[st + k] = P.vel[st + last]; P.vel[st + last] = tv;
    float tf = P.visc[st + k]; P.visc[st + k] = P.visc[st + last]; P.visc[st + last] = tf;
}

__global__ void k_count_erase(GridDims d, Particles P, int *__restrict__ counts, int cap_per_cell)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= P.nbins) return;
    const int bi = b / d.bnj, bj = b - bi * d.bnj;
    const int i0 = bi * 3, j0 = bj * 3;
    const int st = P.bin_start[b];
    int n = P.bin_count[b];
    int c9[9];
#pragma unroll
    for (int q = 0; q < 9; q++) c9[q] = 0;
    bool over = false;
    for (int k = 0; k < n; k++) {
        float2 p = P.pos[st + k];
        long long i = (long long)floorf(p.x), j = (long long)floorf(p.y);
        long long di = i - i0, dj = j - j0;
        if (di >= 0 && di < 3 && dj >= 0 && dj < 3 && i < d.ni && j < d.nj) {
            int q = (int)(di * 3 + dj);
            c9[q]++;
            if (c9[q] > cap_per_cell) over = true;
        }
    }
    if (over) {
        // exact replay: cells of this bin in linear (i-major) order, each
        // scanning the bin and swap-erasing particles beyond the cap
        for (int q = 0; q < 9; q++) {
            const int ci = i0 + q / 3, cj = j0 + q % 3;
            if (ci >= d.ni || cj >= d.nj) continue;
            int cnt = 0;
            for (int k = 0; k < n; k++) {
                float2 p = P.pos[st + k];
                if ((long long)floorf(p.x) == ci && (long long)floorf(p.y) == cj) {
                    if (cnt >= cap_per_cell) {
                        swap_erase(P, st, k, n - 1);
                        n--;
                        k--;
                        continue;
                    }
                    cnt++;
                }
            }
            c9[q] = cnt;
        }
        P.bin_count[b] = n;
    }
    for (int q = 0; q < 9; q++) {
        const int ci = i0 + q / 3, cj = j0 + q % 3;
        if (ci < d.ni && cj < d.nj) counts[(size_t)ci * d.nj + cj] = c9[q];
    }
}

void launch_count_erase(const GridDims &d, const SceneParams &sp, Particles &P, const Grids &G,
                        cudaStream_t st)
{
    k_count_erase<<<nblk(P.nbins, kThreads), kThreads, 0, st>>>(d, P, G.counts,
                                                               2 * sp.particlesPerCell);
}

// ---------------------------------------------------------------------------
// FlipSolver::maxParticleVelocity (flipsolver2d.cpp:1560-1574): max |v|^2 over
// stored particles, as float bits (non-negative floats order like integers)
// ---------------------------------------------------------------------------
__global__ void k_max_v2(Particles P, Scalars *sc)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    const int nslots = P.bin_start[P.nbins];
    float m = FLT_MIN;
    if (s < nslots) {
        const int b = P.slot_bin[s];
        if (s - P.bin_start[b] < P.bin_count[b]) {
            float2 v = P.vel[s];
            float v2 = v.x * v.x + v.y * v.y;
            if (v2 > m) m = v2;
        }
    }
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(&sc->maxv2, __float_as_uint(m));
}

__global__ void k_reset_maxv2(Scalars *sc) { sc->maxv2 = __float_as_uint(FLT_MIN); }

void launch_max_velocity(const Particles &P, Scalars *sc, cudaStream_t st)
{
    k_reset_maxv2<<<1, 1, 0, st>>>(sc);
    if (P.cap == 0) return;
    k_max_v2<<<nblk(P.bound, kThreads), kThreads, 0, st>>>(P, sc);
}

} // namespace fsg
