// fs_grid.cu -- per-cell and per-face kernels of the FLIP substep.
//
//   scene classification   updateSinks / updateSolids / updateInitialFluid
//   friction factors       updateVelocityFromSolids precomputation
//   decomposition          getPressureProjectionMatrix + getIPPCoefficients,
//                          matrix-free: one packed byte per cell
//   density grid + RHS     updateDensityGrid + calcDensityCorrectionRhs
//   P2G + SDF + materials  particleVelocityToGrid, centeredParamsToGrid,
//                          updateSdf, updateMaterials fused into one gather
//   level set / velocity   extrapolateLevelsetInside, breadthFirstExtrapolate:
//   extrapolation          layer-synchronous, temporally blocked in shared memory
//   pressure RHS / apply   calcPressureRhs, applyPressureThreadU/V fused with
//                          the solid friction
//
// Compiled with -fmad=false so each float expression rounds exactly as the
// reference's (-ffp-contract=off) build does.
#include <cfloat>
#include <climits>

#include "fs_device.h"
#include "fs_state.h"

namespace fsg {

constexpr int kThreads = 256;
static inline int nblk(long long n, int t) { return (int)((n + t - 1) / t); }

// ---------------------------------------------------------------------------
// scene classification (flipsolver2d.cpp:502-590), frame 0 only
// ---------------------------------------------------------------------------
// kind: 0 solid (value = friction), 1 initial fluid (value = viscosity),
// 2 sink (value = divergence), 3 source (value = divergence)
__global__ void k_scene_classify(GridDims d, Grids G, float dx, const float *__restrict__ xy,
                                 const int *__restrict__ off, const int *__restrict__ kind,
                                 const float *__restrict__ val, int npoly, int nb)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= d.ni * d.nj) return;
    const int i = c / d.nj, j = c - i * d.nj;
    int8_t m = G.material[c];
    // updateSinks (:554-571)
    for (int k = 0; k < npoly; k++) {
        if (kind[k] != 2) continue;
        if (polygon_sdf(xy + 2 * off[k], off[k + 1] - off[k], ((float)i + 0.5f) * dx,
                        ((float)j + 0.5f) * dx) <= 0.f) {
            m = M_SINK;
            G.divc[c] = val[k];
        }
    }
    // updateSources (:532-552): the last source containing the cell centre
    // (i dx + dx / 2, in float) makes it a source
    {
        const float hdx = (float)((double)dx / 2.0);
        int src = 0;
        for (int k = 0; k < npoly; k++) {
            if (kind[k] != 3) continue;
            if (polygon_sdf(xy + 2 * off[k], off[k + 1] - off[k], (float)i * dx + hdx,
                            (float)j * dx + hdx) <= 0.f) {
                m = M_SOURCE;
                G.emitter_id[c] = src;
                G.divc[c] = val[k];
            }
            src++;
        }
    }
    // updateSolids (:502-530); (float(i)+0.5)*dx is evaluated in double
    float dist = FLT_MAX;
    int minIdx = 0, solidIdx = 0;
    const float x = (float)(((double)(float)i + 0.5) * (double)dx);
    const float y = (float)(((double)(float)j + 0.5) * (double)dx);
    for (int k = 0; k < npoly; k++) {
        if (kind[k] != 0) continue;
        float sdf = polygon_sdf(xy + 2 * off[k], off[k + 1] - off[k], x, y) / dx;
        if (sdf < dist) {
            minIdx = solidIdx;
            dist = sdf;
        }
        solidIdx++;
    }
    G.solid_sdf[c] = dist;
    if (dist < 0) {
        m = M_SOLID;
        G.solid_id[c] = minIdx;
    }
    if (nb) {
        // NBFlipSolver::fluidSdfFromInitialFluid (nbflipsolver.cpp:299-330):
        // the nearest initial fluid's signed distance at the cell centre
        float fd = FLT_MAX;
        int fid = -1;
        for (int k = 0; k < npoly; k++) {
            if (kind[k] != 1) continue;
            const float sdf = polygon_sdf(xy + 2 * off[k], off[k + 1] - off[k], x, y) / dx;
            if (sdf < fd) {
                fd = sdf;
                fid = k;
            }
        }
        G.fluid_sdf[c] = fd;
        if (fd < 0) {
            m = M_FLUID;
            if (fid != -1) G.visc[c] = val[fid];
        }
        G.counts[c] = 0;
    } else {
        // updateInitialFluid (:573-590)
        for (int k = 0; k < npoly; k++) {
            if (kind[k] != 1) continue;
            if (polygon_sdf(xy + 2 * off[k], off[k + 1] - off[k], ((float)i + 0.5f) * dx,
                            ((float)j + 0.5f) * dx) <= 0.f) {
                m = M_FLUID;
                G.visc[c] = val[k];
            }
        }
    }
    G.material[c] = m;
}

void launch_scene_classify(const GridDims &d, const Grids &G, float dx, const float *poly_xy,
                           const int *poly_off, const int *poly_kind, const float *poly_val,
                           int npoly, bool nb, cudaStream_t st)
{
    k_scene_classify<<<nblk((long long)d.ni * d.nj, kThreads), kThreads, 0, st>>>(
        d, G, dx, poly_xy, poly_off, poly_kind, poly_val, npoly, nb ? 1 : 0);
}

// updateVelocityFromSolids (flipsolver2d.cpp:1077-1104) depends only on solid
// cells and solid ids, which never change after frame 0: precompute per face
// the factor (1 - mean friction) or NaN where the face is not affected.
__global__ void k_friction_factors(GridDims d, Grids G, const float *__restrict__ fric)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= d.ni * d.nj) return;
    const int i = c / d.nj, j = c - i * d.nj;
    float sum = 0;
    int cnt = 0;
    for (int io = -1; io < 2; io++)
        for (int jo = -1; jo < 2; jo++) {
            int a = i + io, b = j + jo;
            if (a < 0 || a >= d.ni || b < 0 || b >= d.nj) continue;
            int id = G.solid_id[(size_t)a * d.nj + b];
            if (id != -1) {
                sum += fric[id];
                cnt++;
            }
        }
    float fu = __int_as_float(0x7fc00000), fv = fu;
    if (cnt > 0) {
        float avg = sum / (float)cnt;
        const int8_t *m = G.material;
        bool uA = t_solid(mat_at(m, d, i, j + 1)) || t_solid(mat_at(m, d, i - 1, j + 1)) ||
                  t_solid(mat_at(m, d, i, j)) || t_solid(mat_at(m, d, i - 1, j)) ||
                  t_solid(mat_at(m, d, i, j - 1)) || t_solid(mat_at(m, d, i - 1, j - 1));
        bool vA = t_solid(mat_at(m, d, i + 1, j)) || t_solid(mat_at(m, d, i + 1, j - 1)) ||
                  t_solid(mat_at(m, d, i, j)) || t_solid(mat_at(m, d, i, j - 1)) ||
                  t_solid(mat_at(m, d, i - 1, j)) || t_solid(mat_at(m, d, i - 1, j - 1));
        if (uA) fu = 1 - avg;
        if (vA) fv = 1 - avg;
    }
    G.ufric[c] = fu;
    G.vfric[c] = fv;
}

void launch_friction_factors(const GridDims &d, const Grids &G, const float *obst_friction,
                             cudaStream_t st)
{
    k_friction_factors<<<nblk((long long)d.ni * d.nj, kThreads), kThreads, 0, st>>>(
        d, G, obst_friction);
}

__global__ void k_fill_u8(uint8_t *p, uint8_t v, size_t n)
{
    size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) p[k] = v;
}
void launch_fill_u8(uint8_t *p, uint8_t v, size_t n, cudaStream_t st)
{
    if (n) k_fill_u8<<<nblk((long long)n, kThreads), kThreads, 0, st>>>(p, v, n);
}

// ---------------------------------------------------------------------------
// decomposition: one byte per cell, frozen for both solves of the substep.
//   bit 7      the cell is a unit (fluid at this stage)
//   bits 4..6  nonsolidNeighborCount of the cell (materialgrid.cpp:137-140);
//              for a unit this equals its fluid-or-empty neighbour count
//              (getPressureProjectionMatrix, flipsolver2d.cpp:832-869)
//   bits 0..3  NeighborMask (pressuredata.h:87-95): fluid neighbour whose
//              linear index lies inside the grid
// IPP off-diagonals are 1/(nsc(neighbour) * scale) (flipsolver2d.cpp:924-927).
// ---------------------------------------------------------------------------
__device__ __forceinline__ int chunk_of(long long c, long long ps, long long rem)
{
    // ThreadPool::splitRange: the first `rem` chunks hold ps + 1 cells
    const long long big = rem * (ps + 1);
    return (int)(c < big ? c / (ps + 1) : rem + (c - big) / ps);
}

__global__ void k_decomposition(GridDims d, const int8_t *__restrict__ m, uint8_t *__restrict__ info,
                                int *__restrict__ chunk_last, int nchunks, long long ps,
                                long long rem, int *__restrict__ wrap)
{
    __shared__ int last_sm[8];
    __shared__ int k0_sm;
    const long long N = (long long)d.ni * d.nj;
    const long long blo = (long long)blockIdx.x * blockDim.x;
    const long long bhi = (blo + blockDim.x < N ? blo + blockDim.x : N) - 1;
    if (threadIdx.x == 0) k0_sm = chunk_of(blo, ps, rem);
    if (threadIdx.x < 8) last_sm[threadIdx.x] = -1;
    __syncthreads();
    const int k0 = k0_sm;
    const bool few = chunk_of(bhi, ps, rem) - k0 < 8;
    const long long c = blo + threadIdx.x;
    if (c < N) {
        const int i = (int)(c / d.nj), j = (int)(c - (long long)i * d.nj);
        const int8_t mim = mat_at(m, d, i - 1, j), mip = mat_at(m, d, i + 1, j);
        const int8_t mjm = mat_at(m, d, i, j - 1), mjp = mat_at(m, d, i, j + 1);
        const int nsc = !t_solid(mim) + !t_solid(mip) + !t_solid(mjm) + !t_solid(mjp);
        uint8_t b = (uint8_t)(nsc << 4);
        if (t_fluid(m[c])) {
            b |= 0x80;
            if (t_fluid(mim) && c - d.nj >= 0) b |= 1;
            if (t_fluid(mip) && c + d.nj < N) b |= 2;
            if (t_fluid(mjm) && c - 1 >= 0) b |= 4;
            if (t_fluid(mjp) && c + 1 < N) b |= 8;
            if (j == 0 || j == d.nj - 1) atomicOr(wrap, 1);
            const int k = chunk_of(c, ps, rem);
            if (few) atomicMax(&last_sm[k - k0], (int)c);
            else atomicMax(&chunk_last[k], (int)c);
        }
        info[c] = b;
    }
    __syncthreads();
    if (few && threadIdx.x < 8 && last_sm[threadIdx.x] >= 0 && k0 + (int)threadIdx.x < nchunks)
        atomicMax(&chunk_last[k0 + threadIdx.x], last_sm[threadIdx.x]);
}

void launch_decomposition(const GridDims &d, const Grids &G, int *chunk_last, int nchunks,
                          long long ps, long long rem, Scalars *sc, cudaStream_t st)
{
    cudaMemsetAsync(chunk_last, 0xff, (size_t)nchunks * sizeof(int), st);
    cudaMemsetAsync(&sc->wrap_units, 0, sizeof(int), st);
    k_decomposition<<<nblk((long long)d.ni * d.nj, kThreads), kThreads, 0, st>>>(
        d, G.material, G.cell_info, chunk_last, nchunks, ps, rem, &sc->wrap_units);
}

// ---------------------------------------------------------------------------
// density grid + RHS: updateDensityGridThread (flipsolver2d.cpp:201-249) and
// calcDensityCorrectionRhs (:993-1011)
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_density_grid(GridDims d, Particles P, const int8_t *__restrict__ m,
                               float *__restrict__ dens, T *__restrict__ rhs, double density,
                               double dx, int ppc, const Scalars *__restrict__ sc)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= d.ni * d.nj) return;
    const int ci = c / d.nj, cj = c - ci * d.nj;
    const float cellVolume = (float)(dx * dx * dx);
    const float particleMass = (float)((density * cellVolume) / ((float)ppc));
    const int cbi = ci / 3, cbj = cj / 3;
    float acc = 0.f;
    for (int io = -1; io <= 1; io++) {
        const int bi = cbi + io;
        if (bi < 0 || bi >= d.bni) continue;
        for (int jo = -1; jo <= 1; jo++) {
            const int bj = cbj + jo;
            if (bj < 0 || bj >= d.bnj) continue;
            const int b = bi * d.bnj + bj;
            const int st = P.bin_start[b], n = P.bin_count[b];
            for (int k = 0; k < n; k++) {
                const float2 p = P.pos[st + k];
                const float w = sm_bilinear_hat(p.x - (float)ci - 0.5f, p.y - (float)cj - 0.5f);
                if (fabsf(w) > 1e-6f) acc += w * particleMass;
            }
        }
    }
    acc /= cellVolume;
    const int8_t mc = m[c];
    if (t_fluid(mc) && (t_empty(mat_at(m, d, ci + 1, cj)) || t_empty(mat_at(m, d, ci - 1, cj)) ||
                        t_empty(mat_at(m, d, ci, cj + 1)) || t_empty(mat_at(m, d, ci, cj - 1))))
        acc = clampf(acc, (float)density, FLT_MAX);
    dens[c] = acc;
    const double scale = 1.0 / (double)sc->dt;
    rhs[c] = t_fluid(mc) ? (T)(scale * (1.0 - clampd((double)acc / density, 0.5, 1.5))) : (T)0;
}

void launch_density_grid(const GridDims &d, const SceneParams &sp, const Particles &P,
                         const Grids &G, void *rhs, int is_double, const Scalars *sc,
                         cudaStream_t st)
{
    const int nb = nblk((long long)d.ni * d.nj, kThreads);
    if (is_double)
        k_density_grid<double><<<nb, kThreads, 0, st>>>(d, P, G.material, G.density,
                                                        (double *)rhs, sp.fluidDensity, sp.dx,
                                                        sp.particlesPerCell, sc);
    else
        k_density_grid<float><<<nb, kThreads, 0, st>>>(d, P, G.material, G.density, (float *)rhs,
                                                       sp.fluidDensity, sp.dx,
                                                       sp.particlesPerCell, sc);
}

// ---------------------------------------------------------------------------
// P2G + centred parameters + fluid SDF + materials, one gather per cell:
//   particleVelocityToGridThread (flipsolver2d.cpp:1329-1377)
//   centeredParamsToGridThread   (:1394-1431)
//   updateSdfThread              (:1276-1311)
//   updateMaterials              (:1053-1075)
// The U row i = NI and the V column j = NJ are never written by the
// reference's loop over NI*NJ cells and stay at their fill values 0 / false.
// ---------------------------------------------------------------------------
// NB: NB-FLIP's centredParamsToGrid (nbflipsolver.cpp:463-504) keeps
// centred weights with |w| > 1e-6 (the same sums otherwise, and 0 where none
// is kept, which 0 / 1e-10 also gives), and its materials are classified
// only after the grid combination (k_nb_materials)
template <bool NB>
__global__ void k_p2g_sdf_materials(GridDims d, Particles P, Grids G, float particleScale,
                                    int handling)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= d.ni * d.nj) return;
    const int ci = c / d.nj, cj = c - ci * d.nj;
    const int cbi = ci / 3, cbj = cj / 3;
    const float threshold = 1e-9f;
    const float c_threshold = NB ? 1e-6f : threshold;
    float uW = 1e-10f, vW = 1e-10f, uVel = 0.0f, vVel = 0.0f;
    bool uValid = false, vValid = false;
    float wT = (float)1e-10, vis = 0.0f;
    bool visValid = false;
    float d2 = FLT_MAX;
    const float fi = (float)ci, fj = (float)cj;
    const float cx = fi + 0.5f, cy = fj + 0.5f;
    for (int io = -1; io <= 1; io++) {
        const int bi = cbi + io;
        if (bi < 0 || bi >= d.bni) continue;
        for (int jo = -1; jo <= 1; jo++) {
            const int bj = cbj + jo;
            if (bj < 0 || bj >= d.bnj) continue;
            const int b = bi * d.bnj + bj;
            const int st = P.bin_start[b], n = P.bin_count[b];
            for (int k = 0; k < n; k++) {
                const float2 p = P.pos[st + k];
                // SDF: min squared distance to the cell centre
                const float ddx = p.x - cx, ddy = p.y - cy;
                const float nd = ddx * ddx + ddy * ddy;
                if (nd < d2) d2 = nd;
                // every B-spline below is zero unless the particle is within
                // 2 cells of (i, j) in both axes: skip the rest of the far ones
                if (!(fabsf(p.x - fi) < 2.f && fabsf(p.y - fj) < 2.f)) continue;
                // velocity: weights at (i, j+0.5) for U and (i+0.5, j) for V
                const float wU = sm_qbspline(p.x - fi, p.y - (fj + 0.5f));
                const float wV = sm_qbspline(p.x - (fi + 0.5f), p.y - fj);
                if (wU > threshold && wV > threshold) {
                    const float2 v = P.vel[st + k];
                    uW += wU;
                    uVel += wU * v.x;
                    uValid = true;
                    vW += wV;
                    vVel += wV * v.y;
                    vValid = true;
                }
                if (handling != 2) {
                    const float wc = sm_qbspline(p.x - fi, p.y - fj);
                    if ((NB ? fabsf(wc) : wc) > c_threshold) {
                        wT += wc;
                        vis += wc * P.visc[st + k];
                        visValid = true;
                    }
                }
            }
        }
    }
    const int NV = d.nj + 1;
    G.u[(size_t)ci * d.nj + cj] = uVel / uW;
    G.uvalid[(size_t)ci * d.nj + cj] = uValid;
    G.v[(size_t)ci * NV + cj] = vVel / vW;
    G.vvalid[(size_t)ci * NV + cj] = vValid;
    if (ci == d.ni - 1) { // U row NI stays at the fill value
        G.u[(size_t)d.ni * d.nj + cj] = 0.f;
        G.uvalid[(size_t)d.ni * d.nj + cj] = 0;
    }
    if (cj == d.nj - 1) { // V column NJ stays at the fill value
        G.v[(size_t)ci * NV + d.nj] = 0.f;
        G.vvalid[(size_t)ci * NV + d.nj] = 0;
    }
    if (handling != 2) {
        G.visc[c] = vis / wT;
        G.known[c] = visValid;
        G.divc[c] = 0.f;
    }
    const float sdf = sqrtf(d2) - particleScale;
    G.fluid_sdf[c] = sdf;
    if (NB) return;
    const int8_t mc = G.material[c];
    if (sdf < 0.f) {
        if (t_empty(mc)) G.material[c] = M_FLUID;
    } else {
        if (t_strict_fluid(mc)) G.material[c] = M_EMPTY;
    }
}

void launch_p2g_sdf_materials(const GridDims &d, const SceneParams &sp, const Particles &P,
                              const Grids &G, bool nb, cudaStream_t st)
{
    if (nb)
        k_p2g_sdf_materials<true><<<nblk((long long)d.ni * d.nj, kThreads), kThreads, 0, st>>>(
            d, P, G, sp.particleScale, sp.parameterHandlingMethod);
    else
        k_p2g_sdf_materials<false><<<nblk((long long)d.ni * d.nj, kThreads), kThreads, 0, st>>>(
            d, P, G, sp.particleScale, sp.parameterHandlingMethod);
}

// ---------------------------------------------------------------------------
// Breadth-first extrapolation, layer-synchronous.
// In the reference's FIFO BFS (mathfuncs.cpp:152-215, flipsolver2d.cpp:
// 1433-1494) a cell's marker is its 8-neighbour graph distance to the seed
// cells, every cell of layer k is finished before any cell of layer k+1, and
// a layer-k cell reads only neighbours of layers < k.  Processing whole layers
// at once therefore gives the same values.  A tile of TILE x TILE cells is
// loaded with a halo of H cells; H layers are advanced in shared memory, after
// which every interior cell is exact (each layer consumes one halo ring).
// ---------------------------------------------------------------------------
constexpr int kTile = 32;
constexpr int kMarkInf = INT_MAX;
constexpr int kMarkOut = INT_MIN; // outside the grid: not a neighbour

template <int H>
struct BfsTile {
    static constexpr int W = kTile + 2 * H;
    int mark[W * W];
    float val[W * W];
};

// average over the 8-neighbourhood in the reference's order, neighbours with
// a smaller marker only, summed in double
// the markers of the eight neighbours of (r, q) in the reference's order,
// kMarkOut outside the window
template <int W>
__device__ __forceinline__ void bfs_marks(const int *mark, int r, int q, int nm[8])
{
    int k = 0;
#pragma unroll
    for (int io = -1; io <= 1; io++)
#pragma unroll
        for (int jo = -1; jo <= 1; jo++) {
            if (io == 0 && jo == 0) continue;
            const int rr = r + io, qq = q + jo;
            nm[k++] = (rr < 0 || rr >= W || qq < 0 || qq >= W) ? kMarkOut : mark[rr * W + qq];
        }
}

template <int W>
__device__ __forceinline__ double bfs_avg(const int *nm, const float *val, int r, int q, int k,
                                          int &count)
{
    double avg = 0;
    count = 0;
    int t = 0;
#pragma unroll
    for (int io = -1; io <= 1; io++)
#pragma unroll
        for (int jo = -1; jo <= 1; jo++) {
            if (io == 0 && jo == 0) continue;
            const int rr = r + io, qq = q + jo;
            const int mk = nm[t++];
            if (mk == kMarkOut) continue;
            if (mk < k) {
                avg += (double)val[rr * W + qq];
                count++;
            }
        }
    return avg;
}

__device__ __forceinline__ void ls_two_sum(float a, float b, float &s, float &e)
{
    s = a + b;
    const float bv = s - a;
    e = (a - (s - bv)) + (b - bv);
}

// The value of a BFS cell: avg / count (velocity extrapolation,
// mathfuncs.cpp:152-215) or avg / count - 1 (level set, flipsolver2d.cpp:
// 1433-1494), with avg the double sum of the smaller-marker neighbours in the
// reference's order, rounded to float at the end.  FP64 operations have a
// latency of hundreds of cycles here and every BFS layer waits for its
// slowest cell, so the value is first formed in float-pair arithmetic: the
// sum and its rounding errors are carried exactly enough (s + eh + el), the
// quotient keeps its remainder.  Its distance from the reference's double
// result is below 2^-44 (sum |v| + 1); when that bound cannot place the value
// strictly inside one float's rounding interval, the cell is recomputed in
// double exactly like the reference.  Either way the result is the
// reference's float.
template <int W>
__device__ __forceinline__ float bfs_layer_value(const int *nm, const float *val, int r, int q, int k,
                                                 int add)
{
    float s = 0.f, eh = 0.f, el = 0.f, m = 0.f;
    int count = 0, mine = INT_MAX;
    bool el_exact = true;
    int t = 0;
#pragma unroll
    for (int io = -1; io <= 1; io++)
#pragma unroll
        for (int jo = -1; jo <= 1; jo++) {
            if (io == 0 && jo == 0) continue;
            const int rr = r + io, qq = q + jo;
            const int mk = nm[t++];
            if (mk == kMarkOut || mk >= k) continue;
            const float x = val[rr * W + qq];
            float t2, er, t3, er2;
            ls_two_sum(s, x, t2, er);
            s = t2;
            ls_two_sum(eh, er, t3, er2);
            eh = t3;
            el_exact &= er2 == 0.f;
            el += er2;
            m += fabsf(x);
            if (x != 0.f) {
                // ilogbf from the exponent field for normal numbers
                const int ex = (__float_as_int(x) >> 23) & 255;
                mine = min(mine, (ex != 0 && ex != 255) ? ex - 127 : ilogbf(x));
            }
            count++;
        }
    const float cf = (float)count;
    const float qh = __fdiv_rn(s, cf);
    const float rem = fmaf(-qh, cf, s); // exact
    float t1, t2, v, ev, u, eu;
    ls_two_sum(rem, eh, t1, t2);
    ls_two_sum(t2, el, v, ev);
    ls_two_sum(t1, v, u, eu);
    const float ql = __fdiv_rn(u, cf);
    // the quotient qh + ql is exact when the remainder terms added exactly
    // and ql times the count gives them back
    const bool q_exact = ev == 0.f && eu == 0.f && fmaf(ql, cf, -u) == 0.f;
    float h, l, err3 = 0.f;
    if (add != 0) {
        ls_two_sum(qh, (float)add, h, l);
        float l2;
        ls_two_sum(l, ql, l2, err3);
        l = l2;
    } else {
        h = qh;
        l = ql;
    }
    const float f = h + l;
    // Exact case, which covers the frequent exact ties (a value exactly half
    // way between two floats): when every error term above was captured
    // exactly (el_exact, q_exact, err3 == 0), h + l is the exact value.  When
    // the inputs also span few enough binades (27 for the sum; 52 bits for the
    // quotient minus one) every double operation of the reference is exact as
    // well, and both round the same exact value to float, ties to even.
    if (count > 0 && el_exact && q_exact && err3 == 0.f && mine >= -100 && m < 0x1p100f) {
        const int em = m > 0.f ? ilogbf(m) : -1000;
        const bool sum_exact = m == 0.f || em - mine <= 27;
        const int ea = qh != 0.f ? ilogbf(qh) : -1000;
        const int lsb = min(qh != 0.f ? ilogbf(qh) - 23 : INT_MAX, ql != 0.f ? ilogbf(ql) - 23 : INT_MAX);
        // qh + ql (the quotient) must fit a double, and so must it minus one
        // (a zero quotient, qh = ql = 0, is exact; lsb is INT_MAX then)
        const bool sub_exact = (qh == 0.f && ql == 0.f) ||
                               (add != 0 ? (max(ea, 0) + 1 - min(lsb, 0) <= 52) : (ea - lsb <= 51));
        if (sum_exact && sub_exact) {
            if (f != 0.f && isfinite(f)) return f;
            // an exact zero sum: the reference's double sum is +0 as well
            if (add == 0 && s == 0.f && eh == 0.f && el == 0.f) return 0.f;
        }
    }
    // f is the reference's float when the double result D lies strictly
    // inside f's rounding interval (half the smaller spacing either side):
    // |D - f| <= |h + l - f| + bound, and h + l - f = d within one rounding
    // of d (h - f is exact).  The factor 1.0001 covers the float roundings of
    // this test itself; a cell whose value sits closer to a rounding
    // boundary than that (about 1 in 10^4) takes the double path below.
    const float d = (h - f) + l;
    const float bound = (m + 1.f) * 0x1p-44f;
    const float gap = 0.5f * fminf(nextafterf(f, INFINITY) - f, f - nextafterf(f, -INFINITY));
    if (count > 0 && isfinite(f) && isfinite(m) && fabsf(f) >= 0x1p-100f &&
        (fabsf(d) + bound) * 1.0001f < gap)
        return f;
    const double avg = bfs_avg<W>(nm, val, r, q, k, count);
    // dividing by 1, 2, 4 or 8 is an exact scaling, the same as multiplying
    // by the reciprocal -- and a multiply has a fraction of the latency
    const double inv2 = count == 1 ? 1.0 : count == 2 ? 0.5 : count == 4 ? 0.25 : 0.125;
    const double a = (count & (count - 1)) == 0 ? avg * inv2 : avg / count;
    return add != 0 ? (float)(a + (double)add) : (float)a;
}

// Advance layers k0+1 .. k0+H of the breadth-first extrapolation inside a
// loaded tile.  The frontier of each layer is kept as a list in shared memory:
// cells of layer k are the unmarked neighbours of layer k-1 cells (claimed
// with a compare-and-swap, so each is listed once); their values are then
// computed from neighbours of smaller layers, in the reference's neighbour
// order.  The set of cells per layer, hence every value, is deterministic.
// `add` selects the form: 0 the velocity average, -1 the inside level set
// (average - 1), +1 the outside level set (average + 1).
// Appends `cnt_mine` entries per thread to a shared list with one atomic per
// warp; returns this thread's first slot.  All threads of the warp call it.
__device__ __forceinline__ int warp_append(int *counter, int cnt_mine)
{
    const int lane = threadIdx.x & 31;
    int incl = cnt_mine;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    int base = 0;
    if (lane == 31 && incl > 0) base = atomicAdd(counter, incl);
    base = __shfl_sync(0xffffffffu, base, 31);
    return base + incl - cnt_mine;
}

template <int W, int H>
__device__ __forceinline__ void bfs_layers(int *mark, float *val, short *fa, short *fb, int *cnt,
                                           int k0, int add)
{
    // cnt[0..2]: rotating list lengths (the list of layer k is counted in
    // cnt[k % 3]; cnt[(k + 2) % 3] is free while layer k is processed)
    if (threadIdx.x < 3) cnt[threadIdx.x] = 0;
    __syncthreads();
    // claims the unmarked neighbours of cell e for layer k + 1 and lists them
    // (all threads of a warp call it; `live` says whether e is a real cell)
    // nm: the neighbours' markers read before (a claim by another thread
    // since then only makes the compare-and-swap fail)
    auto expand = [&](bool live, int e, const int *nm, int k, short *out, int *counter) {
        int r = 0, q = 0;
        unsigned got = 0; // bit (io+1)*3+(jo+1) for each neighbour claimed
        if (live) {
            r = e / W;
            q = e - r * W;
            int t = 0;
#pragma unroll
            for (int io = -1; io <= 1; io++)
#pragma unroll
                for (int jo = -1; jo <= 1; jo++) {
                    if (io == 0 && jo == 0) continue;
                    const int mk = nm[t++];
                    if (mk != kMarkInf) continue; // also outside the window (kMarkOut)
                    const int n = (r + io) * W + (q + jo);
                    if (atomicCAS(&mark[n], kMarkInf, k + 1) == kMarkInf)
                        got |= 1u << ((io + 1) * 3 + (jo + 1));
                }
        }
        int slot = warp_append(counter, __popc(got));
#pragma unroll
        for (int b = 0; b < 9; b++)
            if (got & (1u << b)) out[slot++] = (short)((r + b / 3 - 1) * W + (q + b % 3 - 1));
    };
    // layer k0 (final from earlier passes) discovers layer k0 + 1; a warp
    // with no layer-k0 cell in this round skips the expansion (its append
    // would add nothing)
    for (int e0 = 0; e0 < W * W; e0 += blockDim.x) {
        const int e = e0 + (int)threadIdx.x;
        const bool live = e < W * W && mark[e] == k0;
        if (!__any_sync(0xffffffffu, live)) continue;
        int nm[8];
        if (live) bfs_marks<W>(mark, e / W, e - (e / W) * W, nm);
        expand(live, e, nm, k0, fa, &cnt[(k0 + 1) % 3]);
    }
    __syncthreads();
    short *cur = fa, *nxt = fb;
    // One phase per layer k: the values of layer-k cells (they read only
    // layers < k, all final) and the discovery of layer k + 1 from them
    // (claiming cells that are unmarked; a value never counts a neighbour of
    // layer k or above, so the two do not interfere).
    for (int k = k0 + 1; k <= k0 + H; k++) {
        const int ncur = cnt[k % 3];
        if (ncur == 0) break;
        if (threadIdx.x == 0) cnt[(k + 2) % 3] = 0;
        const bool more = k < k0 + H;
        for (int f0 = 0; f0 < ncur; f0 += blockDim.x) {
            const int f = f0 + (int)threadIdx.x;
            const bool live = f < ncur;
            if (f0 + (int)(threadIdx.x & ~31u) >= ncur) continue; // a warp past the list
            int e = 0;
            int nm[8];
            if (live) {
                e = cur[f];
                const int r = e / W, q = e - r * W;
                bfs_marks<W>(mark, r, q, nm);
                val[e] = bfs_layer_value<W>(nm, val, r, q, k, add);
            }
            if (more) expand(live, e, nm, k, nxt, &cnt[(k + 1) % 3]);
        }
        __syncthreads();
        short *tmp = cur;
        cur = nxt;
        nxt = tmp;
    }
}

// Velocity extrapolation, breadthFirstExtrapolate(grid, flags, 10, ...):
// layers 1..11 (a layer-k cell discovers layer k+1 while k <= 10).
// With `save_gravity` the output also performs the two steps that follow the
// first extrapolation in FlipSolver::step (:439-440): the saved copy receives
// the extrapolated grid and the live grid gets + dt/dx * g.
constexpr int kVelH = 11;

__global__ void __launch_bounds__(1024) k_vel_extrap(GridDims d, Grids G, float gI, float gJ,
                                                    double dx, const Scalars *__restrict__ sc,
                                                    int save_gravity)
{
    __shared__ BfsTile<kVelH> t;
    __shared__ short fa[BfsTile<kVelH>::W * BfsTile<kVelH>::W];
    __shared__ short fb[BfsTile<kVelH>::W * BfsTile<kVelH>::W];
    __shared__ int cnt[3];
    constexpr int W = BfsTile<kVelH>::W;
    const bool isV = blockIdx.z == 1;
    const int si = isV ? d.ni : d.ni + 1, sj = isV ? d.nj + 1 : d.nj;
    const float *__restrict__ g = isV ? G.v : G.u;
    const uint8_t *__restrict__ fl = isV ? G.vvalid : G.uvalid;
    float *__restrict__ go = isV ? G.v2 : G.u2;
    uint8_t *__restrict__ flo = isV ? G.vvalid2 : G.uvalid2;
    const int ti0 = blockIdx.y * kTile, tj0 = blockIdx.x * kTile;
    if (ti0 >= si || tj0 >= sj) return;
    for (int e = threadIdx.x; e < W * W; e += blockDim.x) {
        const int r = e / W, q = e - r * W;
        const int gi = ti0 - kVelH + r, gj = tj0 - kVelH + q;
        if (gi < 0 || gi >= si || gj < 0 || gj >= sj) {
            t.mark[e] = kMarkOut;
            t.val[e] = 0.f;
        } else {
            const size_t idx = (size_t)gi * sj + gj;
            t.mark[e] = fl[idx] ? 0 : kMarkInf;
            t.val[e] = g[idx];
        }
    }
    bool has_seed = false, has_inf = false;
    for (int e = threadIdx.x; e < W * W; e += blockDim.x) {
        has_seed |= t.mark[e] == 0;
        has_inf |= t.mark[e] == kMarkInf;
    }
    // a tile whose loaded region lacks either seeds or unknown cells assigns
    // nothing and only copies its interior through
    const bool work = __syncthreads_or(has_seed) && __syncthreads_or(has_inf);
    if (work) bfs_layers<W, kVelH>(t.mark, t.val, fa, fb, cnt, 0, 0);
    const float factor = (float)((double)sc->dt / dx);
    const float add = factor * (isV ? gJ : gI);
    for (int e = threadIdx.x; e < kTile * kTile; e += blockDim.x) {
        const int r = e / kTile + kVelH, q = e % kTile + kVelH;
        const int gi = ti0 - kVelH + r, gj = tj0 - kVelH + q;
        if (gi >= si || gj >= sj) continue;
        const size_t idx = (size_t)gi * sj + gj;
        const int mk = t.mark[r * W + q];
        const float vv = t.val[r * W + q];
        const uint8_t valid = (mk != kMarkInf) ? 1 : 0;
        if (save_gravity) {
            (isV ? G.sv : G.su)[idx] = vv;
            (isV ? G.svvalid : G.suvalid)[idx] = valid;
            go[idx] = vv + add;
        } else {
            go[idx] = vv;
        }
        flo[idx] = valid;
    }
}

void launch_vel_extrapolate(const GridDims &d, Grids &G, const SceneParams &sp,
                            const Scalars *sc, bool save_and_gravity, cudaStream_t st)
{
    dim3 grid(nblk(d.nj + 1, kTile), nblk(d.ni + 1, kTile), 2);
    k_vel_extrap<<<grid, 1024, 0, st>>>(d, G, sp.gI, sp.gJ, sp.dx, sc, save_and_gravity ? 1 : 0);
    float *t = G.u; G.u = G.u2; G.u2 = t;
    t = G.v; G.v = G.v2; G.v2 = t;
    uint8_t *b = G.uvalid; G.uvalid = G.uvalid2; G.uvalid2 = b;
    b = G.vvalid; G.vvalid = G.vvalid2; G.vvalid2 = b;
}

// Level set inside extrapolation (flipsolver2d.cpp:1433-1494): seeds are
// cells with sdf > 0, depth unbounded, value = average - 1.  The outside
// form (:1496-1558, NB-FLIP) seeds every cell below NI * NJ and assigns
// average + 1; both run the same passes.  Pass p advances
// layers p*H+1 .. (p+1)*H.  Each cell's (marker, value) pair lives in one
// 64-bit word that is read and written whole.  A tile only trusts halo cells
// of earlier passes (markers <= p*H, final since the previous launch); cells
// a concurrently running neighbour tile assigned in this pass are reset and
// recomputed, giving the same values.  Only newly assigned interior cells are
// written (and copied to the fluid SDF).  A tile
// works in pass p only if a tile within one tile of it assigned cells in pass
// p-1: the frontier of layer p*H is otherwise out of its reach.  Once a pass
// assigns nothing, the remaining passes return immediately.
// Two tile shapes (T x T tiles with an H-cell halo, 1024 threads a tile):
// - 64 x 64 with H = 32: (64 + 64)^2 cells of (marker, value) plus two
//   frontier lists, 192 KiB of dynamic shared memory, 32 layers a pass;
// - 86 x 86 with H = 24: 210 KiB, 24 layers a pass.  At 1024^2 this is 144
//   tiles, one wave on 152 SMs, where 64 x 64 tiles need two waves a pass.
// launch_levelset picks the shape with the fewer waves per layer.  Larger
// tiles than the velocity extrapolation's cut the halo cells a tile reloads
// per interior cell and the number of passes.
template <int T, int H> struct LsShape {
    static constexpr int kTile = T, kHalo = H, kW = T + 2 * H;
    static constexpr size_t kSmem = (size_t)kW * kW * (4 + 4 + 2 + 2) + 16;
};
using LsNarrow = LsShape<64, 32>;
using LsWide = LsShape<86, 24>;
static_assert(LsWide::kW * LsWide::kW < 32768, "frontier indices are shorts");

__device__ __forceinline__ unsigned long long ls_pack(int mark, float v)
{
    return ((unsigned long long)(unsigned)mark << 32) | (unsigned long long)__float_as_uint(v);
}

// seeds: sdf > 0 inside; sdf < NI * NJ outside (extrapolateLevelsetOutside,
// flipsolver2d.cpp:1496-1512: everything else is unknown)
__global__ void k_levelset_init(GridDims d, const float *__restrict__ sdf,
                                unsigned long long *__restrict__ cells, uint8_t *__restrict__ act,
                                int ntiles, int *__restrict__ active, int passes, int outside)
{
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long N = (long long)d.ni * d.nj;
    if (c < N) {
        const float v = sdf[c];
        const bool seed = outside ? v < (float)((size_t)d.ni * (size_t)d.nj) : v > 0.f;
        cells[c] = ls_pack(seed ? 0 : kMarkInf, v);
    }
    if (c < 3LL * ntiles) act[c] = 0;
    if (c <= passes) active[c] = 0; // active[passes]: the one-launch form's barrier counter
}

// one BFS pass of a tile (the block); every thread of the block takes the
// same exits
template <class S>
__device__ __forceinline__ void ls_pass(GridDims d, float *__restrict__ sdf, unsigned long long *__restrict__ cells,
                                        uint8_t *__restrict__ act, int *__restrict__ active, int pass, int add)
{
    extern __shared__ int ls_smem[];
    constexpr int W = S::kW;
    constexpr int kLsTile = S::kTile, kLsH = S::kHalo;
    struct {
        int *mark;
        float *val;
    } t{ls_smem, reinterpret_cast<float *>(ls_smem + W * W)};
    short *fa = reinterpret_cast<short *>(ls_smem + 2 * W * W);
    short *fb = fa + W * W;
    int *cnt = reinterpret_cast<int *>(fb + W * W);
    const int si = d.ni, sj = d.nj;
    const int tiles_i = gridDim.y, tiles_j = gridDim.x;
    const int ntiles = tiles_i * tiles_j;
    const int tile = blockIdx.y * tiles_j + blockIdx.x;
    uint8_t *act_prev = act + (size_t)((pass + 2) % 3) * ntiles;
    uint8_t *act_cur = act + (size_t)(pass % 3) * ntiles;
    uint8_t *act_next = act + (size_t)((pass + 1) % 3) * ntiles;
    // whether this tile works in this pass is decided once, by thread 0, and
    // shared through the barrier: every thread of the block takes the same
    // exit, so the warp-wide shuffles of the BFS always see full warps
    bool work = true;
    if (threadIdx.x == 0) {
        if (pass > 0 && ((volatile int *)active)[pass - 1] == 0) {
            work = false;
        } else {
            act_next[tile] = 0;
            if (pass > 0) {
                bool near = false;
                for (int a = -1; a <= 1; a++)
                    for (int b = -1; b <= 1; b++) {
                        const int ti = (int)blockIdx.y + a, tj = (int)blockIdx.x + b;
                        if (ti >= 0 && ti < tiles_i && tj >= 0 && tj < tiles_j)
                            near |= ((volatile uint8_t *)act_prev)[ti * tiles_j + tj] != 0;
                    }
                work = near;
            }
        }
    }
    if (!__syncthreads_or(threadIdx.x == 0 && work)) return;
    const int ti0 = blockIdx.y * kLsTile, tj0 = blockIdx.x * kLsTile;
    const int k0 = pass * kLsH;
    int open = 0;
    for (int e = threadIdx.x; e < W * W; e += blockDim.x) {
        const int r = e / W, q = e - r * W;
        const int gi = ti0 - kLsH + r, gj = tj0 - kLsH + q;
        if (gi < 0 || gi >= si || gj < 0 || gj >= sj) {
            t.mark[e] = kMarkOut;
            t.val[e] = 0.f;
        } else {
            const unsigned long long w = ((volatile unsigned long long *)cells)[(size_t)gi * sj + gj];
            int mk = (int)(w >> 32);
            // a halo cell a neighbour tile already assigned in this same pass
            // is recomputed here: the frontier of every layer must come from
            // this tile's own BFS, or cells next to it could be missed
            if (mk > k0 && mk != kMarkInf) mk = kMarkInf;
            t.mark[e] = mk;
            t.val[e] = __uint_as_float((unsigned)(w & 0xffffffffu));
            open |= mk == kMarkInf;
        }
    }
    // a tile whose cells are all assigned already has nothing to do
    if (!__syncthreads_or(open)) return;
    bfs_layers<W, kLsH>(t.mark, t.val, fa, fb, cnt, k0, add);
    bool assigned = false;
    for (int e = threadIdx.x; e < kLsTile * kLsTile; e += blockDim.x) {
        const int r = e / kLsTile + kLsH, q = e % kLsTile + kLsH;
        const int gi = ti0 - kLsH + r, gj = tj0 - kLsH + q;
        if (gi >= si || gj >= sj) continue;
        const int mk = t.mark[r * W + q];
        if (mk > k0 && mk != kMarkInf) {
            const size_t idx = (size_t)gi * sj + gj;
            const float v = t.val[r * W + q];
            cells[idx] = ls_pack(mk, v);
            sdf[idx] = v;
            assigned = true;
        }
    }
    if (__syncthreads_or(assigned) && threadIdx.x == 0) {
        act_cur[tile] = 1;
        atomicExch(&active[pass], 1);
    }
}

template <class S>
__global__ void __launch_bounds__(1024, 1) k_levelset_pass(GridDims d, float *__restrict__ sdf,
                                                       unsigned long long *__restrict__ cells,
                                                       uint8_t *__restrict__ act,
                                                       int *__restrict__ active, int pass, int add)
{
    ls_pass<S>(d, sdf, cells, act, active, pass, add);
}

// All passes in one cooperative launch when every tile is resident at once
// (one tile per SM): a grid barrier between passes instead of a kernel
// boundary, and the launch ends after the first pass that assigns nothing,
// instead of the remaining launches each returning at once.  The barrier is
// an arrival counter (active[passes], zeroed by k_levelset_init): release
// fence and relaxed add, then bounded acquire polls by thread 0 of a block;
// a timeout sets *status (reported like a PCG wait) and the blocks leave.
template <class S>
__global__ void __launch_bounds__(1024, 1) k_levelset_all(GridDims d, float *__restrict__ sdf,
                                                      unsigned long long *__restrict__ cells,
                                                      uint8_t *__restrict__ act, int *__restrict__ active,
                                                      int passes, int add, int *__restrict__ status,
                                                      long long lim)
{
    unsigned *count = reinterpret_cast<unsigned *>(active + passes);
    const unsigned nb = gridDim.x * gridDim.y;
    for (int pass = 0; pass < passes; pass++) {
        if (pass > 0 && ((volatile int *)active)[pass - 1] == 0) break; // the same in every block
        ls_pass<S>(d, sdf, cells, act, active, pass, add);
        __syncthreads();
        int gave_up = 0;
        if (threadIdx.x == 0) {
            asm volatile("fence.acq_rel.gpu;" ::: "memory");
            asm volatile("red.relaxed.gpu.global.add.u32 [%0], 1;" ::"l"(count) : "memory");
            const unsigned target = (unsigned)(pass + 1) * nb;
            long long spins = 0;
            for (;;) {
                unsigned v;
                asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(count) : "memory");
                if ((int)(v - target) >= 0) break;
                if (++spins > lim || ((spins & 1023) == 0 && *((volatile int *)status) != 0)) {
                    atomicExch(status, 1);
                    gave_up = 1;
                    break;
                }
            }
        }
        if (__syncthreads_or(gave_up)) return;
    }
}

// waves per BFS layer: a pass of H layers plus the tile load (about five
// layers' time) runs its tiles in ceil(tiles / SMs) waves
static bool ls_wide(const GridDims &d)
{
    const int sms = device_sm_count();
    auto cost = [&](int T, int H) {
        const long long tiles = (long long)nblk(d.ni, T) * nblk(d.nj, T);
        return (double)((tiles + sms - 1) / sms) * (H + 5) / H;
    };
    return cost(LsWide::kTile, LsWide::kHalo) < cost(LsNarrow::kTile, LsNarrow::kHalo);
}

int levelset_max_passes(const GridDims &d)
{
    int m = d.ni > d.nj ? d.ni : d.nj;
    return m / (ls_wide(d) ? LsWide::kHalo : LsNarrow::kHalo) + 2;
}

// whether every tile of shape S fits on the device at once (one launch)
template <class S> static bool ls_one_launch(const GridDims &d)
{
    const long long tiles = (long long)nblk(d.nj, S::kTile) * nblk(d.ni, S::kTile);
    static std::atomic<int> slots[kMaxDevices];
    const int per_sm = device_cached(slots, [] {
        cudaFuncSetAttribute((const void *)k_levelset_all<S>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)S::kSmem);
        int nb = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, (const void *)k_levelset_all<S>, 1024, S::kSmem) !=
            cudaSuccess) {
            cudaGetLastError();
            return 0;
        }
        return nb;
    });
    return per_sm > 0 && tiles <= (long long)per_sm * device_sm_count();
}

template <class S>
static void launch_levelset_shape(const GridDims &d, Grids &G, bool outside, cudaStream_t st, int *status,
                                  long long spin_limit)
{
    constexpr int kLsTile = S::kTile;
    const int passes = levelset_max_passes(d);
    dim3 grid(nblk(d.nj, kLsTile), nblk(d.ni, kLsTile));
    const int ntiles = grid.x * grid.y;
    const long long n = (long long)d.ni * d.nj;
    long long init_n = n > 3LL * ntiles ? n : 3LL * ntiles;
    if (init_n < passes + 1) init_n = passes + 1;
    unsigned long long *cells = reinterpret_cast<unsigned long long *>(G.levelset_cells);
    k_levelset_init<<<nblk(init_n, kThreads), kThreads, 0, st>>>(d, G.fluid_sdf, cells,
                                                               G.levelset_act, ntiles,
                                                               G.levelset_active, passes,
                                                               outside ? 1 : 0);
    if (status && ls_one_launch<S>(d)) {
        cudaFuncSetAttribute((const void *)k_levelset_all<S>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)S::kSmem);
        GridDims dd = d;
        float *sdf = G.fluid_sdf;
        uint8_t *act = G.levelset_act;
        int *active = G.levelset_active;
        int np = passes, add = outside ? 1 : -1;
        int *stp = status;
        long long lim = spin_limit > 0 ? spin_limit : (1LL << 25);
        void *args[] = {&dd, &sdf, &cells, &act, &active, &np, &add, &stp, &lim};
        if (cudaLaunchCooperativeKernel((const void *)k_levelset_all<S>, grid, dim3(1024), args, S::kSmem, st) ==
            cudaSuccess)
            return;
        cudaGetLastError(); // not launched: the passes one launch each
    }
    cudaFuncSetAttribute((const void *)k_levelset_pass<S>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)S::kSmem);
    for (int p = 0; p < passes; p++)
        k_levelset_pass<S><<<grid, 1024, S::kSmem, st>>>(d, G.fluid_sdf, cells, G.levelset_act,
                                                          G.levelset_active, p, outside ? 1 : -1);
}

void launch_levelset(const GridDims &d, Grids &G, bool outside, cudaStream_t st, int *status, long long spin_limit)
{
    if (ls_wide(d)) launch_levelset_shape<LsWide>(d, G, outside, st, status, spin_limit);
    else launch_levelset_shape<LsNarrow>(d, G, outside, st, status, spin_limit);
}

int levelset_launches(const GridDims &d, bool with_status)
{
    const bool one = with_status && (ls_wide(d) ? ls_one_launch<LsWide>(d) : ls_one_launch<LsNarrow>(d));
    return one ? 2 : 1 + levelset_max_passes(d);
}

// ---------------------------------------------------------------------------
// pressure RHS: calcPressureRhs (flipsolver2d.cpp:962-991) with divergenceAt
// (:759-764), evaluated in double like the reference
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_pressure_rhs(GridDims d, const float *__restrict__ u, const float *__restrict__ v,
                               const float *__restrict__ divc, const int8_t *__restrict__ m,
                               T *__restrict__ rhs, double scale)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= d.ni * d.nj) return;
    const int i = c / d.nj, j = c - i * d.nj;
    if (!t_fluid(m[c])) {
        rhs[c] = (T)0;
        return;
    }
    const int NV = d.nj + 1;
    const float u0 = u[(size_t)i * d.nj + j], u1 = u[(size_t)(i + 1) * d.nj + j];
    const float v0 = v[(size_t)i * NV + j], v1 = v[(size_t)i * NV + j + 1];
    const double div = (double)(u1 - u0 + v1 - v0 + divc[c]);
    double val = -scale * div;
    val -= (double)t_solid(mat_at(m, d, i - 1, j)) * scale * (double)(u0 - 0);
    val += (double)t_solid(mat_at(m, d, i + 1, j)) * scale * (double)(u1 - 0);
    val -= (double)t_solid(mat_at(m, d, i, j - 1)) * scale * (double)(v0 - 0);
    val += (double)t_solid(mat_at(m, d, i, j + 1)) * scale * (double)(v1 - 0);
    rhs[c] = (T)val;
}

void launch_pressure_rhs(const GridDims &d, const Grids &G, void *rhs, int is_double,
                         const SceneParams &sp, cudaStream_t st)
{
    const double scale = 1.f / sp.dx;
    const int nb = nblk((long long)d.ni * d.nj, kThreads);
    if (is_double)
        k_pressure_rhs<double><<<nb, kThreads, 0, st>>>(d, G.u, G.v, G.divc, G.material,
                                                        (double *)rhs, scale);
    else
        k_pressure_rhs<float><<<nb, kThreads, 0, st>>>(d, G.u, G.v, G.divc, G.material,
                                                       (float *)rhs, scale);
}

// ---------------------------------------------------------------------------
// applyPressureThreadU/V (flipsolver2d.cpp:1133-1193) followed, per face, by
// updateVelocityFromSolids (:1077-1104) through the precomputed factors
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_apply_pressure(GridDims d, Grids G, const T *__restrict__ p, double density,
                                 double dx, const Scalars *__restrict__ sc, int with_friction)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= d.ni * d.nj) return;
    const int i = c / d.nj, j = c - i * d.nj;
    const double scale = (double)sc->dt / (density * dx);
    const int8_t *m = G.material;
    const double pc = (double)p[c];
    // U face (i, j) between cells (i-1, j) and (i, j)
    {
        const double pim1 = i - 1 < 0 ? 0.0 : (double)p[c - d.nj];
        const int8_t ma = mat_at(m, d, i - 1, j), mb = m[c];
        const size_t f = (size_t)i * d.nj + j;
        if (t_fluid(ma) || t_fluid(mb)) {
            if (t_solid(ma) || t_solid(mb)) G.u[f] = 0.f;
            else G.u[f] = (float)((double)G.u[f] - scale * (pc - pim1));
        } else {
            G.uvalid[f] = 0;
        }
        if (with_friction) {
            const float fr = G.ufric[c];
            if (fr == fr) G.u[f] = G.u[f] * fr;
        }
    }
    // V face (i, j) between cells (i, j-1) and (i, j)
    {
        const double pjm1 = j - 1 < 0 ? 0.0 : (double)p[c - 1];
        const int8_t ma = mat_at(m, d, i, j - 1), mb = m[c];
        const size_t f = (size_t)i * (d.nj + 1) + j;
        if (t_fluid(ma) || t_fluid(mb)) {
            if (t_solid(ma) || t_solid(mb)) G.v[f] = 0.f;
            else G.v[f] = (float)((double)G.v[f] - scale * (pc - pjm1));
        } else {
            G.vvalid[f] = 0;
        }
        if (with_friction) {
            const float fr = G.vfric[c];
            if (fr == fr) G.v[f] = G.v[f] * fr;
        }
    }
}

void launch_apply_pressure(const GridDims &d, const SceneParams &sp, const Grids &G,
                           const void *pressure, int is_double, const Scalars *sc,
                           bool with_friction, cudaStream_t st)
{
    const int nb = nblk((long long)d.ni * d.nj, kThreads);
    if (is_double)
        k_apply_pressure<double><<<nb, kThreads, 0, st>>>(d, G, (const double *)pressure,
                                                          sp.fluidDensity, sp.dx, sc,
                                                          with_friction ? 1 : 0);
    else
        k_apply_pressure<float><<<nb, kThreads, 0, st>>>(d, G, (const float *)pressure,
                                                         sp.fluidDensity, sp.dx, sc,
                                                         with_friction ? 1 : 0);
}

// updateVelocityFromSolids on its own (stage-level API)
__global__ void k_friction(GridDims d, Grids G)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= d.ni * d.nj) return;
    const int i = c / d.nj, j = c - i * d.nj;
    const float fu = G.ufric[c], fv = G.vfric[c];
    if (fu == fu) G.u[(size_t)i * d.nj + j] = G.u[(size_t)i * d.nj + j] * fu;
    if (fv == fv) G.v[(size_t)i * (d.nj + 1) + j] = G.v[(size_t)i * (d.nj + 1) + j] * fv;
}

void launch_friction(const GridDims &d, const Grids &G, cudaStream_t st)
{
    k_friction<<<nblk((long long)d.ni * d.nj, kThreads), kThreads, 0, st>>>(d, G);
}

// m_savedFluidVelocityGrid = m_fluidVelocityGrid (flipsolver2d.cpp:439)
__global__ void k_save_grid(Grids G, size_t nu, size_t nv)
{
    const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nu) {
        G.su[k] = G.u[k];
        G.suvalid[k] = G.uvalid[k];
    }
    if (k < nv) {
        G.sv[k] = G.v[k];
        G.svvalid[k] = G.vvalid[k];
    }
}

void launch_save_grid(const GridDims &d, const Grids &G, cudaStream_t st)
{
    const size_t nu = (size_t)(d.ni + 1) * d.nj, nv = (size_t)d.ni * (d.nj + 1);
    const size_t n = nu > nv ? nu : nv;
    k_save_grid<<<nblk((long long)n, kThreads), kThreads, 0, st>>>(G, nu, nv);
}

// applyBodyForces (flipsolver2d.cpp:1222-1241): factor = dt / dx in float
__global__ void k_body_forces(Grids G, size_t nu, size_t nv, float gI, float gJ, double dx,
                              const Scalars *__restrict__ sc)
{
    const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const float factor = (float)((double)sc->dt / dx);
    if (k < nu) G.u[k] += factor * gI;
    if (k < nv) G.v[k] += factor * gJ;
}

void launch_body_forces(const GridDims &d, const SceneParams &sp, const Grids &G,
                        const Scalars *sc, cudaStream_t st)
{
    const size_t nu = (size_t)(d.ni + 1) * d.nj, nv = (size_t)d.ni * (d.nj + 1);
    const size_t n = nu > nv ? nu : nv;
    k_body_forces<<<nblk((long long)n, kThreads), kThreads, 0, st>>>(G, nu, nv, sp.gI, sp.gJ,
                                                                    sp.dx, sc);
}

} // namespace fsg
