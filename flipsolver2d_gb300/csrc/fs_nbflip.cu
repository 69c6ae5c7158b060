// fs_nbflip.cu -- the kernels NB-FLIP (NBFlipSolver, nbflipsolver.cpp) adds to
// the FLIP substep: narrow-band pruning, semi-Lagrangian advection of the
// grids, the combination of advected and transferred grids, the material
// update after it, band reseeding with the solver's std::mt19937 stream, and
// the engine itself.
//
// Built with -fmad=false like the other FLIP kernels: every float expression
// rounds as the reference's CPU build does.
//
// Sources (emitters) enter through the material (SOURCE cells), the
// emitter id grid and the source table: FlipSolver::afterTransfer, NB-FLIP's
// pruneNarrowBand, updateGridFromSources and reseedParticles, and FLIP's
// reseedParticles read them.
#include <cfloat>
#include <cstdint>

#include "fs_state.h"

namespace fsg {

namespace {
constexpr int kThreads = 256;
inline int nblk(long long n, int t) { return (int)((n + t - 1) / t); }

constexpr float kNarrowBand = -3.f;      // m_narrowBand,      nbflipsolver.cpp:20
constexpr float kCombinationBand = -2.f; // m_combinationBand, :21
constexpr float kResamplingBand = -1.f;  // m_resamplingBand,  :22
} // namespace

// ---------------------------------------------------------------------------
// the Mersenne Twister MT19937 (Matsumoto and Nishimura 1998), the engine of
// std::mt19937: 624 state words, regenerated 624 at a time, tempered on
// output.  State layout: words 0..623, then the index of the next word.
// ---------------------------------------------------------------------------
constexpr int kMtN = 624, kMtM = 397;
constexpr uint32_t kMtMatrix = 0x9908b0dfu, kMtUpper = 0x80000000u, kMtLower = 0x7fffffffu;

__host__ __device__ inline uint32_t mt_temper(uint32_t y)
{
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    return y;
}

__host__ __device__ inline uint32_t mt_mix(uint32_t a, uint32_t b, uint32_t c)
{
    const uint32_t y = (a & kMtUpper) | (b & kMtLower);
    return c ^ (y >> 1) ^ ((y & 1u) ? kMtMatrix : 0u);
}

void mt_seed_host(uint32_t *st, uint32_t seed)
{
    st[0] = seed;
    for (int i = 1; i < kMtN; i++) st[i] = 1812433253u * (st[i - 1] ^ (st[i - 1] >> 30)) + (uint32_t)i;
    st[kMtN] = kMtN;
}

static void mt_twist_host(uint32_t *x)
{
    for (int k = 0; k < kMtN; k++) x[k] = mt_mix(x[k], x[(k + 1) % kMtN], x[(k + kMtM) % kMtN]);
}

void mt_discard_host(uint32_t *st, unsigned long long n)
{
    while (n > 0) {
        if (st[kMtN] >= (uint32_t)kMtN) {
            mt_twist_host(st);
            st[kMtN] = 0;
        }
        const unsigned long long take = n < (unsigned long long)(kMtN - st[kMtN])
                                            ? n
                                            : (unsigned long long)(kMtN - st[kMtN]);
        st[kMtN] += (uint32_t)take;
        n -= take;
    }
}

// std::uniform_real_distribution<float>(0, 1) over a 32-bit engine: one word,
// converted to float (round to nearest), scaled by 2^-32 (exact), a result
// that rounded up to 1 replaced by the largest float below 1, then
// (b - a) * r + a = r
__device__ __forceinline__ float mt_canonical(uint32_t w)
{
    float r = __uint2float_rn(w) * 0x1p-32f;
    if (r >= 1.f) r = 0x1.fffffep-1f;
    return r;
}

// The next per * count[0] draws of the engine, in order, as floats in [0, 1).
// One block: a regeneration runs as four dependent phases (words 0..226 read
// old words only; 227..453 read words 0..226; 454..622 read 227..395; 623
// reads word 0 and 396), each read into registers before any is written.
__global__ void __launch_bounds__(1024) k_mt_draws(uint32_t *__restrict__ st, float *__restrict__ out,
                                                   const int *__restrict__ count, int per)
{
    __shared__ uint32_t x[kMtN];
    const int t = threadIdx.x;
    for (int i = t; i < kMtN; i += blockDim.x) x[i] = st[i];
    int idx = (int)st[kMtN];
    const long long n = (long long)count[0] * per;
    __syncthreads();
    long long done = 0;
    auto phase = [&](int lo, int hi) {
        uint32_t v = 0;
        const int k = lo + t;
        if (k < hi) v = mt_mix(x[k], x[(k + 1) % kMtN], x[(k + kMtM) % kMtN]);
        __syncthreads();
        if (k < hi) x[k] = v;
        __syncthreads();
    };
    while (done < n) {
        if (idx >= kMtN) {
            phase(0, kMtN - kMtM);
            phase(kMtN - kMtM, 2 * (kMtN - kMtM));
            phase(2 * (kMtN - kMtM), kMtN - 1);
            phase(kMtN - 1, kMtN);
            idx = 0;
        }
        const long long left = n - done;
        const int take = left < (long long)(kMtN - idx) ? (int)left : kMtN - idx;
        for (int k = t; k < take; k += blockDim.x) out[done + k] = mt_canonical(mt_temper(x[idx + k]));
        idx += take;
        done += take;
        __syncthreads(); // the next regeneration overwrites what was read
    }
    for (int i = t; i < kMtN; i += blockDim.x) st[i] = x[i];
    if (t == 0) st[kMtN] = (uint32_t)idx;
}

void launch_mt_draws(uint32_t *state, float *out, const int *count, int per, cudaStream_t st)
{
    k_mt_draws<<<1, 1024, 0, st>>>(state, out, count, per);
}

// ---------------------------------------------------------------------------
// NBFlipSolver::pruneNarrowBand (:227-253).  Killed particles and the
// originals of moved ones are already marked (a moved particle's copy in the
// rebin set keeps its unmarked flag); marking them again changes nothing, so
// only particles that stay in their bin are tested.
// ---------------------------------------------------------------------------
__global__ void k_nb_prune_band(GridDims d, Particles P, const float *__restrict__ sdf,
                                const int *__restrict__ counts, const int8_t *__restrict__ material,
                                int cap2)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= P.bin_start[P.nbins] || P.flag[s] != P_STAY) return;
    const float2 p = P.pos[s];
    const long long i = (long long)p.x, j = (long long)p.y; // ssize_t i = position.x()
    const float v = grid_lerp(sdf, d.ni, d.nj, 0.f, 0.f, p.x, p.y);
    const bool src = material[i * d.nj + j] == M_SOURCE;
    if ((!src && v < kNarrowBand) || ((src || v < kResamplingBand) && counts[i * d.nj + j] > cap2))
        P.flag[s] = P_KILL;
}

// FlipSolver::rk4Integrate (flipsolver2d.cpp:1195-1203) through the velocity grid
__device__ __forceinline__ float2 rk4_integrate(const float *__restrict__ u, const float *__restrict__ v,
                                                const GridDims &d, float2 p, float dt)
{
    float2 k = velocity_at(u, v, d, p.x, p.y);
    const float k1x = k.x * dt, k1y = k.y * dt;
    k = velocity_at(u, v, d, p.x + k1x * 0.5f, p.y + k1y * 0.5f);
    const float k2x = k.x * dt, k2y = k.y * dt;
    k = velocity_at(u, v, d, p.x + k2x * 0.5f, p.y + k2y * 0.5f);
    const float k3x = k.x * dt, k3y = k.y * dt;
    k = velocity_at(u, v, d, p.x + k3x, p.y + k3y);
    const float k4x = k.x * dt, k4y = k.y * dt;
    const float sx = ((k1x + k2x * 2.f) + k3x * 2.f) + k4x;
    const float sy = ((k1y + k2y * 2.f) + k3y * 2.f) + k4y;
    return make_float2(p.x + sx * (1.0f / 6.0f), p.y + sy * (1.0f / 6.0f));
}

// FlipSolver::eulerAdvectionThread (flipsolver2d.cpp:340-351) for the four
// grids of NBFlipSolver::advect (:66-109) in one launch.  Every sample (i, j)
// of U, V, the fluid SDF and the viscosity starts its rk4Integrate(-dt) trace
// at Vec3(i, j) through the same velocity grid, so the trace is computed once
// per lattice point (i, j), 0 <= i <= NI, 0 <= j <= NJ, and every grid that
// has a sample (i, j) is sampled there (with its own offset).
__global__ void k_nb_euler(GridDims d, const float *__restrict__ u, const float *__restrict__ v,
                           const float *__restrict__ sdf, const float *__restrict__ visc,
                           float *__restrict__ au, float *__restrict__ av, float *__restrict__ asdf,
                           float *__restrict__ avisc, const Scalars *__restrict__ sc)
{
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long cols = d.nj + 1;
    if (e >= (long long)(d.ni + 1) * cols) return;
    const int i = (int)(e / cols), j = (int)(e - (long long)i * cols);
    const float2 p = rk4_integrate(u, v, d, make_float2((float)i, (float)j), -sc->dt);
    if (j < d.nj) au[(size_t)i * d.nj + j] = grid_lerp(u, d.ni + 1, d.nj, 0.5f, 0.f, p.x, p.y);
    if (i < d.ni) {
        av[(size_t)i * (d.nj + 1) + j] = grid_lerp(v, d.ni, d.nj + 1, 0.f, 0.5f, p.x, p.y);
        if (j < d.nj) {
            const size_t c = (size_t)i * d.nj + j;
            asdf[c] = grid_lerp(sdf, d.ni, d.nj, 0.f, 0.f, p.x, p.y);
            avisc[c] = grid_lerp(visc, d.ni, d.nj, 0.5f, 0.5f, p.x, p.y);
        }
    }
}

void launch_nb_advect_extra(const GridDims &d, const SceneParams &sp, const Particles &P,
                            const Grids &G, const NbGrids &N, const Scalars *sc, cudaStream_t st)
{
    if (P.cap > 0)
        k_nb_prune_band<<<nblk(P.bound, kThreads), kThreads, 0, st>>>(d, P, G.fluid_sdf, G.counts,
                                                                    G.material, 2 * sp.particlesPerCell);
    const long long n = (long long)(d.ni + 1) * (d.nj + 1);
    k_nb_euler<<<nblk(n, kThreads), kThreads, 0, st>>>(d, G.u, G.v, G.fluid_sdf, G.visc, N.adv_u,
                                                       N.adv_v, N.adv_sdf, N.adv_visc, sc);
}

// ---------------------------------------------------------------------------
// NBFlipSolver::afterTransfer (:111-116) without sources: updateGridFromSources
// (:332-364) leaves the SDF at std::min(FLT_MAX, sdf); combineLevelset
// (:373-384) takes std::min(advected + 1, sdf); combineVelocityGrid and
// combineCenteredGrids (:386-427) keep the transferred value where the SDF
// sampled at the face or cell centre exceeds the combination band, else the
// advected one.  std::min(a, b) is (b < a) ? b : a.
// ---------------------------------------------------------------------------
// FlipSolver::afterTransfer (flipsolver2d.cpp:390-410): source cells take the
// emitter's viscosity and, when it transfers velocity, faces (i, j) of U and
// V take its velocity / dx (float / double) and become valid
__global__ void k_sources_after_transfer(GridDims d, Grids G, Sources S, double dx)
{
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= (long long)d.ni * d.nj || G.material[c] != M_SOURCE) return;
    const long long i = c / d.nj, j = c - i * d.nj;
    const SourceParams e = S.p[G.emitter_id[c]];
    G.visc[c] = e.visc;
    if (e.transfer) {
        G.u[i * d.nj + j] = (float)((double)e.vx / dx);
        G.v[i * (d.nj + 1) + j] = (float)((double)e.vy / dx);
        G.uvalid[i * d.nj + j] = 1;
        G.vvalid[i * (d.nj + 1) + j] = 1;
    }
}

// updateGridFromSources (:332-364): the nearest source's signed distance at
// the cell corner (i dx, j dx) in cells; sdf = std::min(dist, sdf) (FLT_MAX
// with no source); inside a source the viscosity grids take its viscosity
__global__ void k_nb_sources_grid(GridDims d, Grids G, NbGrids N, Sources S, float dx)
{
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= (long long)d.ni * d.nj) return;
    const long long i = c / d.nj, j = c - i * d.nj;
    float dist = FLT_MAX;
    int id = -1;
    for (int k = 0; k < S.n; k++) {
        const float v = polygon_sdf(S.xy + 2 * S.off[k], S.off[k + 1] - S.off[k], (float)i * dx,
                                    (float)j * dx) / dx;
        if (v < dist) {
            dist = v;
            id = k;
        }
    }
    const float f = G.fluid_sdf[c];
    G.fluid_sdf[c] = f < dist ? f : dist;
    if (dist < 0 && id != -1) {
        G.visc[c] = S.p[id].visc;
        N.adv_visc[c] = S.p[id].visc;
    }
}

__global__ void k_nb_combine_sdf(long long n, float *__restrict__ sdf, const float *__restrict__ asdf)
{
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const float b = sdf[c];
    const float a = asdf[c] + 1.f;
    sdf[c] = b < a ? b : a;
}

__global__ void k_nb_combine_grids(GridDims d, Grids G, NbGrids N)
{
    const long long nu = (long long)(d.ni + 1) * d.nj, nv = (long long)d.ni * (d.nj + 1);
    const long long nc = (long long)d.ni * d.nj;
    long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < nu) {
        const long long i = e / d.nj, j = e - i * d.nj;
        const float s = grid_lerp(G.fluid_sdf, d.ni, d.nj, 0.f, 0.f, (float)i, 0.5f + (float)j);
        if (!(s > kCombinationBand)) G.u[e] = N.adv_u[e];
    } else if ((e -= nu) < nv) {
        const long long i = e / (d.nj + 1), j = e - i * (d.nj + 1);
        const float s = grid_lerp(G.fluid_sdf, d.ni, d.nj, 0.f, 0.f, 0.5f + (float)i, (float)j);
        if (!(s > kCombinationBand)) G.v[e] = N.adv_v[e];
    } else if ((e -= nv) < nc) {
        const long long i = e / d.nj, j = e - i * d.nj;
        // Vec3(0.5f + i, j + 0.5): the second coordinate is a double sum
        const float s = grid_lerp(G.fluid_sdf, d.ni, d.nj, 0.f, 0.f, 0.5f + (float)i,
                                  (float)((double)j + 0.5));
        if (!(s > kCombinationBand)) G.visc[e] = N.adv_visc[e];
    }
}

// FlipSolver::updateMaterials (flipsolver2d.cpp:1053-1075), which NB-FLIP
// runs after the combination and the inside level set
__global__ void k_nb_materials(long long n, const float *__restrict__ sdf, int8_t *__restrict__ mat)
{
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const int8_t m = mat[c];
    if (sdf[c] < 0.f) {
        if (t_empty(m)) mat[c] = M_FLUID;
    } else if (t_strict_fluid(m)) {
        mat[c] = M_EMPTY;
    }
}

void launch_sources_after_transfer(const GridDims &d, const Grids &G, const Sources &S, double dx,
                                   cudaStream_t st)
{
    if (S.n == 0) return;
    const long long nc = (long long)d.ni * d.nj;
    k_sources_after_transfer<<<nblk(nc, kThreads), kThreads, 0, st>>>(d, G, S, dx);
}

void launch_nb_combine(const GridDims &d, const Grids &G, const NbGrids &N, const Sources &S,
                       double dx, cudaStream_t st)
{
    const long long nc = (long long)d.ni * d.nj;
    launch_sources_after_transfer(d, G, S, dx, st);
    k_nb_sources_grid<<<nblk(nc, kThreads), kThreads, 0, st>>>(d, G, N, S, (float)dx);
    k_nb_combine_sdf<<<nblk(nc, kThreads), kThreads, 0, st>>>(nc, G.fluid_sdf, N.adv_sdf);
    const long long n = (long long)(d.ni + 1) * d.nj + (long long)d.ni * (d.nj + 1) + nc;
    k_nb_combine_grids<<<nblk(n, kThreads), kThreads, 0, st>>>(d, G, N);
}

void launch_nb_materials(const GridDims &d, const Grids &G, cudaStream_t st)
{
    const long long nc = (long long)d.ni * d.nj;
    k_nb_materials<<<nblk(nc, kThreads), kThreads, 0, st>>>(nc, G.fluid_sdf, G.material);
}

// ---------------------------------------------------------------------------
// NBFlipSolver::reseedParticles (:118-201), candidate side.  Cells inside
// the resampling band with fewer than particlesPerCell particles get
// particlesPerCell - count candidates, in row-major cell order; each takes
// two draws (jitteredPosInCell, flipsolver2d.cpp:1013-1019) and is kept
// unless its interpolated SDF is below the narrow band.  A kept candidate
// goes to the bin of its position with zero velocity and the viscosity
// interpolated there.  A position rounded out of the grid has no bin (the
// reference indexes past its bin array) and is dropped.
// ---------------------------------------------------------------------------
// NB-FLIP: band and source cells top up to particlesPerCell; FLIP
// (reseedParticles, flipsolver2d.cpp:627-680): source cells to
// particlesPerCell / 2
__global__ void k_nb_cand_count(long long n, const float *__restrict__ sdf,
                                const int *__restrict__ counts, const int8_t *__restrict__ material,
                                int ppc, int nb, int *__restrict__ cand_n)
{
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const bool src = material[c] == M_SOURCE;
    int add = 0;
    if (nb) {
        const float s = sdf[c];
        if (src || (s < kResamplingBand && s > kNarrowBand)) add = ppc - counts[c];
    } else if (src) {
        add = ppc / 2 - counts[c];
    }
    cand_n[c] = add > 0 ? add : 0;
}

// a candidate's position, test, velocity and viscosity:
//  NB-FLIP  dropped when the cell is a source with sdf above the resampling
//           band or the position's sdf is below the narrow band; velocity
//           from the grid when the cell's emitter transfers velocity;
//           the emitter's viscosity, else the grid's at the position
//  FLIP     source cells only: always kept, velocity as above, the
//           emitter's viscosity
__global__ void k_nb_place(GridDims d, NbReseed R, const float *__restrict__ sdf,
                           const float *__restrict__ visc, const int8_t *__restrict__ material,
                           const int *__restrict__ emitter_id, const float *__restrict__ u,
                           const float *__restrict__ v, Sources S, int nb)
{
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= (long long)d.ni * d.nj) return;
    const int k0 = R.cand_off[c], k1 = R.cand_off[c + 1];
    if (k0 == k1) return;
    const long long i = c / d.nj, j = c - i * d.nj;
    const int cb = bin_of_cell(d, i, j);
    const bool src = material[c] == M_SOURCE;
    const float sc = sdf[c];
    const int eid = emitter_id[c];
    const bool has_e = eid != -1 && eid < S.n;
    const bool transfer = has_e && S.p[eid].transfer;
    for (int k = k0; k < k1; k++) {
        const float x = (float)i + R.draws[2 * (size_t)k];
        const float y = (float)j + R.draws[2 * (size_t)k + 1];
        const int pb = bin_of_pos(d, x, y);
        bool keep = pb >= 0;
        if (nb) {
            const float ns = grid_lerp(sdf, d.ni, d.nj, 0.f, 0.f, x, y);
            keep = keep && !((src && sc > kResamplingBand) || ns < kNarrowBand);
        }
        R.cand_pos[k] = make_float2(x, y);
        R.cand_vel[k] = transfer ? velocity_at(u, v, d, x, y) : make_float2(0.f, 0.f);
        R.cand_visc[k] = has_e ? S.p[eid].visc : grid_lerp(visc, d.ni, d.nj, 0.5f, 0.5f, x, y);
        R.cand_bin[k] = keep ? pb : -1;
        R.cand_cb[k] = cb;
        if (keep && pb != cb) {
            const int q = atomicAdd(R.cross_n, 1);
            if (q < kNbCrossMax) R.cross[q] = k;
        }
    }
}

void launch_nb_candidates(const GridDims &d, const SceneParams &sp, const Grids &G,
                          const NbReseed &R, const Sources &S, bool nb, void *scan_scratch,
                          cudaStream_t st)
{
    const long long nc = (long long)d.ni * d.nj;
    k_nb_cand_count<<<nblk(nc, kThreads), kThreads, 0, st>>>(nc, G.fluid_sdf, G.counts, G.material,
                                                            sp.particlesPerCell, nb ? 1 : 0, R.cand_n);
    scan_exclusive(R.cand_n, R.cand_off, (int)nc, scan_scratch, st);
    launch_mt_draws(R.rng, R.draws, R.cand_off + nc, 2, st);
    cudaMemsetAsync(R.cross_n, 0, sizeof(int), st);
    k_nb_place<<<nblk(nc, kThreads), kThreads, 0, st>>>(d, R, G.fluid_sdf, G.visc, G.material,
                                                        G.emitter_id, G.u, G.v, S, nb ? 1 : 0);
}

} // namespace fsg
