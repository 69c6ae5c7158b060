// fs_viscosity.cu -- LightViscosityModel and HeavyViscosityModel
// (viscositymodel.cpp) on the GPU: assembly of the upper-triangle entries the
// reference's coeffRef calls leave, then Eigen's diagonally preconditioned
// conjugate gradient over the self-adjoint matrix they define.
//
// Compiled with -fmad=false: every assembled entry is the reference's float
// product, converted to double and summed in the reference's order, bit for
// bit.  The solve's dot products are summed over a fixed block partition in a
// fixed order (not left to right as on the CPU), so its iterates agree with
// the reference's to rounding, and are the same bits run to run.
#include "fs_viscosity.h"

#include <algorithm>
#include <cfloat>
#include <cmath>

namespace fsg {

long long visc_unknowns(const GridDims &d, bool heavy)
{
    const long long ni = d.ni, nj = d.nj;
    return heavy ? (ni + 1) * nj + ni * (nj + 1) : ni * nj;
}

long long visc_coef_count(const GridDims &d, bool heavy)
{
    const long long ni = d.ni, nj = d.nj;
    return heavy ? 7 * (ni + 1) * nj + 3 * ni * (nj + 1) : 3 * ni * nj;
}

// ---------------------------------------------------------------------------
// assembly
// ---------------------------------------------------------------------------

// LightViscosityModel::getMatrix (viscositymodel.cpp:65-135).  Cell (i, j)
// writes (assigns, coeffRef = value) its diagonal and, unless solid, the
// entries towards its four neighbours in both of their rows; cells are
// visited row-major, so an upper-triangle entry (k, k+1) keeps the value the
// later cell k+1 wrote (its jm1) when k+1 is not solid, else cell k's jp1,
// else it is absent.  The same for (k, k+NJ) with im1 of cell k+NJ and ip1
// of cell k.  Each factor is 1.0 * (double)(viscosity) * dt.
__global__ void __launch_bounds__(kViscThreads)
k_visc_light_coef(GridDims d, const int8_t *__restrict__ mat, const float *__restrict__ visc,
                  double scale, double *__restrict__ coef, double *__restrict__ invdiag)
{
    const long long n = (long long)d.ni * d.nj;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(k / d.nj), j = (int)(k - (long long)i * d.nj);
        const bool solid = t_solid(mat[k]);
        const float vc = visc[k];
        double diag = 1.0;
        if (!solid) {
            diag = 4.0;
            diag *= (double)vc * scale;
            diag += 1.0;
        }
        double er = 0.0, ed = 0.0;
        if (j + 1 < d.nj) {
            if (!t_solid(mat[k + 1])) er = 1.0 * ((double)(solid ? visc[k + 1] : vc) * scale);
            else if (!solid) er = 1.0 * ((double)vc * scale);
        }
        if (i + 1 < d.ni) {
            const long long kd = k + d.nj;
            if (!t_solid(mat[kd])) ed = 1.0 * ((double)(solid ? visc[kd] : vc) * scale);
            else if (!solid) ed = 1.0 * ((double)vc * scale);
        }
        coef[k] = diag;
        coef[n + k] = er;
        coef[2 * n + k] = ed;
        invdiag[k] = diag != 0.0 ? 1.0 / diag : 1.0;
    }
}

// viscosity at a face corner: Grid2d::interpolateAt with the grid's
// (0.5, 0.5) offset
__device__ __forceinline__ float visc_corner(const float *__restrict__ visc, const GridDims &d,
                                             float i, float j)
{
    return grid_lerp(visc, d.ni, d.nj, 0.5f, 0.5f, i, j);
}

// HeavyViscosityModel::getMatrix (viscositymodel.cpp:202-402).  Every entry
// of a face's row is written while the loop visits that face's own (i, j), as
// coeffRef += (float product), so each row is assembled here by its own
// thread in the reference's order: density, the i-1 / i+1 (U) or j-1 / j+1
// (V) second differences, then the two cross-derivative blocks.  Entries
// left of the diagonal are not stored (the solve reads the upper triangle);
// in particular the V rows' U columns, including the one the reference
// indexes with a V-grid linear index (uIpOneJmOneLinearIdx, :383, :395), all
// lie left of the diagonal.
__global__ void __launch_bounds__(kViscThreads)
k_visc_heavy_coef(GridDims d, const float *__restrict__ visc, float scaleTwoDt, float scaleTwoDx,
                  float density, double *__restrict__ coef, double *__restrict__ invdiag)
{
    const int NI = d.ni, NJ = d.nj;
    const long long NU = (long long)(NI + 1) * NJ, NV = (long long)NI * (NJ + 1);
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < NU + NV;
         k += (long long)gridDim.x * blockDim.x) {
        double dg = 0.0;
        dg += density;
        if (k < NU) {
            const int i = (int)(k / NJ), j = (int)(k - (long long)i * NJ);
            const float fi = (float)i, fj = (float)j;
            double eip = 0.0, ejp = 0.0, v00 = 0.0, vm0 = 0.0, v0p = 0.0, vmp = 0.0;
            if (i - 1 >= 0) dg += scaleTwoDt * gget(visc, NI, NJ, i - 1, j);
            if (i + 1 <= NI) {
                const float vs = gget(visc, NI, NJ, i, j);
                eip += -scaleTwoDt * vs;
                dg += scaleTwoDt * vs;
            }
            if (j - 1 >= 0 && i < NI && i - 1 >= 0) {
                const float lv = visc_corner(visc, d, fi - 0.5f, fj - 0.5f);
                v00 += scaleTwoDx * lv;
                vm0 += -scaleTwoDx * lv;
                dg += scaleTwoDx * lv;
            }
            if (j + 1 < NJ && i < NI && i - 1 >= 0) {
                const float lv = visc_corner(visc, d, fi - 0.5f, fj + 0.5f);
                ejp += -scaleTwoDx * lv;
                v0p += -scaleTwoDx * lv;
                vmp += scaleTwoDx * lv;
                dg += scaleTwoDx * lv;
            }
            coef[k] = dg;
            coef[NU + k] = eip;
            coef[2 * NU + k] = ejp;
            coef[3 * NU + k] = v00;
            coef[4 * NU + k] = vm0;
            coef[5 * NU + k] = v0p;
            coef[6 * NU + k] = vmp;
        } else {
            const long long kv = k - NU;
            const int i = (int)(kv / (NJ + 1)), j = (int)(kv - (long long)i * (NJ + 1));
            const float fi = (float)i, fj = (float)j;
            double ejp = 0.0, eip = 0.0;
            if (j - 1 >= 0) dg += scaleTwoDt * gget(visc, NI, NJ, i, j - 1);
            if (j + 1 <= NJ) {
                const float vs = gget(visc, NI, NJ, i, j);
                ejp += -scaleTwoDt * vs;
                dg += scaleTwoDt * vs;
            }
            if (j < NJ && j - 1 >= 0 && i - 1 >= 0) {
                const float lv = visc_corner(visc, d, fi - 0.5f, fj - 0.5f);
                dg += scaleTwoDx * lv;
            }
            if (j < NJ && i + 1 < NI && j - 1 >= 0) {
                const float lv = visc_corner(visc, d, fi + 0.5f, fj - 0.5f);
                eip += -scaleTwoDx * lv;
                dg += scaleTwoDx * lv;
            }
            double *cv = coef + 7 * NU;
            cv[kv] = dg;
            cv[NV + kv] = ejp;
            cv[2 * NV + kv] = eip;
        }
        invdiag[k] = dg != 0.0 ? 1.0 / dg : 1.0;
    }
}

// right-hand sides and results
// light: b = (double)(density * w) over the NI x NJ cells of U (row stride
// NJ) or V (row stride NJ + 1), fillRhs (:137-148); applyResult (:150-161)
// writes (float)(x / density) back
__global__ void k_visc_light_rhs(GridDims d, const float *__restrict__ w, int stride, float density,
                                 double *__restrict__ b)
{
    const long long n = (long long)d.ni * d.nj;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x) {
        const long long i = k / d.nj, j = k - i * d.nj;
        b[k] = (double)(density * w[i * stride + j]);
    }
}

__global__ void k_visc_light_apply(GridDims d, const double *__restrict__ x, int stride, double density,
                                   float *__restrict__ w)
{
    const long long n = (long long)d.ni * d.nj;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x) {
        const long long i = k / d.nj, j = k - i * d.nj;
        w[i * stride + j] = (float)(x[k] / density);
    }
}

// heavy: getRhs (:404-434) b = (double)(density * u), then V; applyResult
// (:436-469) writes (float)x back
__global__ void k_visc_heavy_rhs(long long nu, long long nv, const float *__restrict__ u,
                                 const float *__restrict__ v, float density, double *__restrict__ b)
{
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < nu + nv;
         k += (long long)gridDim.x * blockDim.x)
        b[k] = (double)(density * (k < nu ? u[k] : v[k - nu]));
}

__global__ void k_visc_heavy_apply(long long nu, long long nv, const double *__restrict__ x,
                                   float *__restrict__ u, float *__restrict__ v)
{
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < nu + nv;
         k += (long long)gridDim.x * blockDim.x) {
        if (k < nu) u[k] = (float)x[k];
        else v[k - nu] = (float)x[k];
    }
}

// ---------------------------------------------------------------------------
// the conjugate gradient
// ---------------------------------------------------------------------------

struct ViscSys {
    int ni, nj;
    long long n, nu, nv; // unknowns; the heavy model's U and V counts
    const double *coef;
    const double *invdiag;
};

// (S p)[k], S the self-adjoint matrix of the stored upper triangle: the
// row's own entries plus the entries of earlier rows that name column k
template <bool HEAVY>
__device__ __forceinline__ double sym_apply(const ViscSys &s, const double *__restrict__ p, long long k)
{
    const double *__restrict__ c = s.coef;
    if (!HEAVY) {
        const long long n = s.n, nj = s.nj;
        const long long i = k / nj, j = k - i * nj;
        double acc = c[k] * p[k];
        if (j + 1 < nj) acc += c[n + k] * p[k + 1];
        if (i + 1 < s.ni) acc += c[2 * n + k] * p[k + nj];
        if (j >= 1) acc += c[n + k - 1] * p[k - 1];
        if (i >= 1) acc += c[2 * n + k - nj] * p[k - nj];
        return acc;
    }
    const long long NU = s.nu, NV = s.nv, NJ = s.nj, NI = s.ni, W = NJ + 1;
    if (k < NU) { // U face (i, j)
        const long long i = k / NJ, j = k - i * NJ;
        const long long v0 = NU + i * W + j; // v(i, j)
        double acc = c[k] * p[k];
        if (i + 1 <= NI) acc += c[NU + k] * p[k + NJ];
        if (j + 1 < NJ) acc += c[2 * NU + k] * p[k + 1];
        if (i < NI) {
            acc += c[3 * NU + k] * p[v0];
            acc += c[5 * NU + k] * p[v0 + 1];
        }
        if (i >= 1) {
            acc += c[4 * NU + k] * p[v0 - W];
            acc += c[6 * NU + k] * p[v0 - W + 1];
            acc += c[NU + k - NJ] * p[k - NJ];
        }
        if (j >= 1) acc += c[2 * NU + k - 1] * p[k - 1];
        return acc;
    }
    // V face (i, j)
    const double *__restrict__ cv = c + 7 * NU;
    const long long kv = k - NU, i = kv / W, j = kv - i * W;
    double acc = cv[kv] * p[k];
    if (j + 1 <= NJ) acc += cv[NV + kv] * p[k + 1];
    if (i + 1 < NI) acc += cv[2 * NV + kv] * p[k + W];
    if (j >= 1) acc += cv[NV + kv - 1] * p[k - 1];
    if (i >= 1) acc += cv[2 * NV + kv - W] * p[k - W];
    // the U rows whose V columns name this face: u(i, j) (v00), u(i+1, j)
    // (vm0), u(i, j-1) (v0p), u(i+1, j-1) (vmp)
    const long long u0 = i * NJ + j;
    if (j < NJ) {
        acc += c[3 * NU + u0] * p[u0];
        acc += c[4 * NU + u0 + NJ] * p[u0 + NJ];
    }
    if (j >= 1) {
        acc += c[5 * NU + u0 - 1] * p[u0 - 1];
        acc += c[6 * NU + u0 + NJ - 1] * p[u0 + NJ - 1];
    }
    return acc;
}

// a block's sum of per-thread values, in a fixed order (valid in thread 0)
__device__ __forceinline__ double block_sum(double v, double *sh)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += sh[w];
    __syncthreads();
    return s;
}

// the total of nb block partials part[stride * b + off], summed the same way
// by every block (so every block holds the same bits)
__device__ __forceinline__ double sum_partials(const double *part, int nb, int stride, int off, double *sh)
{
    double v = 0.0;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) v += part[(long long)stride * b + off];
    v = block_sum(v, sh);
    if (threadIdx.x == 0) sh[32] = v;
    __syncthreads();
    const double s = sh[32];
    __syncthreads();
    return s;
}

// the solve's stop flag, read once per block so that every thread of a block
// takes the same branch
__device__ __forceinline__ bool stopped(const ViscCtl *ctl, int *flag)
{
    if (threadIdx.x == 0) *flag = *(volatile const int *)&ctl->done;
    __syncthreads();
    const bool s = *flag != 0;
    __syncthreads();
    return s;
}

// r = b, x = 0, p = M^-1 r; partials of b.b and r.p
__global__ void __launch_bounds__(kViscThreads)
k_vcg_start(long long n, const double *__restrict__ b, const double *__restrict__ invdiag,
            double *__restrict__ x, double *__restrict__ r, double *__restrict__ p, double *__restrict__ part)
{
    __shared__ double sh[34];
    double bb = 0.0, rp = 0.0;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x) {
        const double bk = b[k];
        const double pk = invdiag[k] * bk;
        x[k] = 0.0;
        r[k] = bk;
        p[k] = pk;
        bb += bk * bk;
        rp += bk * pk;
    }
    bb = block_sum(bb, sh);
    rp = block_sum(rp, sh);
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = bb;
        part[2 * blockIdx.x + 1] = rp;
    }
}

// one block: ||b||^2, the threshold, the first r.z; the stops before the
// loop (b = 0, or a residual already below the threshold)
__global__ void __launch_bounds__(kViscThreads)
k_vcg_start2(int nb, const double *__restrict__ part, ViscCtl *ctl)
{
    __shared__ double sh[34];
    const double bb = sum_partials(part, nb, 2, 0, sh);
    const double rp = sum_partials(part, nb, 2, 1, sh);
    if (threadIdx.x != 0) return;
    ctl->rhs_norm2 = bb;
    ctl->abs_new[0] = rp;
    ctl->abs_new[1] = rp;
    ctl->iters = 0;
    ctl->res_norm2 = bb; // r = b: ||r||^2 is the same sum
    if (bb == 0.0) {
        ctl->threshold = 0.0;
        ctl->res_norm2 = 0.0;
        ctl->done = 1;
        return;
    }
    const double threshold = fmax(kViscTol * kViscTol * bb, DBL_MIN);
    ctl->threshold = threshold;
    ctl->done = bb < threshold ? 1 : 0;
}

// t = S p; partials of p.t
template <bool HEAVY>
__global__ void __launch_bounds__(kViscThreads)
k_vcg_spmv(ViscSys s, const double *__restrict__ p, double *__restrict__ t, double *__restrict__ part,
           const ViscCtl *ctl)
{
    __shared__ double sh[34];
    __shared__ int flag;
    if (stopped(ctl, &flag)) return;
    double pt = 0.0;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < s.n;
         k += (long long)gridDim.x * blockDim.x) {
        const double q = sym_apply<HEAVY>(s, p, k);
        t[k] = q;
        pt += p[k] * q;
    }
    pt = block_sum(pt, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = pt;
}

// alpha = r.z / p.t; x += alpha p; r -= alpha t; partials of r.r and r.z
__global__ void __launch_bounds__(kViscThreads)
k_vcg_update(long long n, int nb, int it, const double *__restrict__ invdiag, double *__restrict__ x,
             double *__restrict__ r, const double *__restrict__ p, const double *__restrict__ t,
             const double *__restrict__ part_pt, double *__restrict__ part, const ViscCtl *ctl)
{
    __shared__ double sh[34];
    __shared__ int flag;
    if (stopped(ctl, &flag)) return;
    const double pt = sum_partials(part_pt, nb, 1, 0, sh);
    const double alpha = ctl->abs_new[it & 1] / pt;
    double rr = 0.0, rz = 0.0;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x) {
        x[k] += alpha * p[k];
        const double rk = r[k] - alpha * t[k];
        r[k] = rk;
        rr += rk * rk;
        rz += rk * (invdiag[k] * rk);
    }
    rr = block_sum(rr, sh);
    rz = block_sum(rz, sh);
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = rr;
        part[2 * blockIdx.x + 1] = rz;
    }
}

// the stopping test, beta = r.z / r.z_old, p = M^-1 r + beta p
__global__ void __launch_bounds__(kViscThreads)
k_vcg_dir(long long n, int nb, int it, int max_it, const double *__restrict__ invdiag,
          const double *__restrict__ r, double *__restrict__ p, const double *__restrict__ part, ViscCtl *ctl)
{
    __shared__ double sh[34];
    __shared__ int flag;
    if (stopped(ctl, &flag)) return;
    const double rr = sum_partials(part, nb, 2, 0, sh);
    const double rz = sum_partials(part, nb, 2, 1, sh);
    const bool lead = blockIdx.x == 0 && threadIdx.x == 0;
    if (rr < ctl->threshold) {
        if (lead) {
            ctl->res_norm2 = rr;
            ctl->iters = it;
            ctl->done = 1;
        }
        return;
    }
    const double beta = rz / ctl->abs_new[it & 1];
    if (lead) {
        ctl->abs_new[(it + 1) & 1] = rz;
        if (it + 1 >= max_it) {
            ctl->res_norm2 = rr;
            ctl->iters = it + 1;
            ctl->done = 1;
        }
    }
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x)
        p[k] = invdiag[k] * r[k] + beta * p[k];
}

static int vector_blocks(long long n)
{
    const long long b = (n + kViscThreads - 1) / kViscThreads;
    return (int)std::max(1LL, std::min<long long>(b, kViscBlocksMax));
}

// Eigen's conjugate_gradient over b (vb.b) into vb.x: the iterations run in
// batches of kViscBatch enqueued at once; the kernels of a batch after the
// stop return at once, and the host reads the stop flag between batches
static cudaError_t vcg_solve(const ViscSys &s, bool heavy, ViscBuffers &vb, cudaStream_t st, int *iters,
                             bool *ok, long long *launches)
{
    const long long n = s.n;
    const int nb = vector_blocks(n);
    double *part_pt = vb.part, *part2 = vb.part + kViscBlocksMax;
    k_vcg_start<<<nb, kViscThreads, 0, st>>>(n, vb.b, vb.invdiag, vb.x, vb.r, vb.p, part2);
    k_vcg_start2<<<1, kViscThreads, 0, st>>>(nb, part2, vb.ctl);
    *launches += 2;
    const long long max_it = 2 * n; // ConjugateGradient's default maxIterations
    long long it = 0;
    for (;;) {
        cudaError_t e = cudaMemcpyAsync(vb.ctl_host, vb.ctl, sizeof(ViscCtl), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return e;
        if (vb.ctl_host->done || it >= max_it) break;
        const long long end = std::min(max_it, it + kViscBatch);
        for (; it < end; it++) {
            if (heavy) k_vcg_spmv<true><<<nb, kViscThreads, 0, st>>>(s, vb.p, vb.t, part_pt, vb.ctl);
            else k_vcg_spmv<false><<<nb, kViscThreads, 0, st>>>(s, vb.p, vb.t, part_pt, vb.ctl);
            k_vcg_update<<<nb, kViscThreads, 0, st>>>(n, nb, (int)it, vb.invdiag, vb.x, vb.r, vb.p, vb.t,
                                                      part_pt, part2, vb.ctl);
            k_vcg_dir<<<nb, kViscThreads, 0, st>>>(n, nb, (int)it, (int)max_it, vb.invdiag, vb.r, vb.p,
                                                   part2, vb.ctl);
            *launches += 3;
        }
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    const ViscCtl &c = *vb.ctl_host;
    *iters = c.iters;
    *ok = c.rhs_norm2 == 0.0 || std::sqrt(c.res_norm2 / c.rhs_norm2) <= kViscTol;
    return cudaSuccess;
}

static int grid_blocks(long long n)
{
    const long long b = (n + kViscThreads - 1) / kViscThreads;
    return (int)std::max(1LL, std::min<long long>(b, 4096));
}

cudaError_t visc_light(const GridDims &d, const Grids &G, float dt, float density, ViscBuffers &vb,
                       cudaStream_t st, int *iters, long long *launches)
{
    const long long n = (long long)d.ni * d.nj;
    const int gb = grid_blocks(n);
    ViscSys s{d.ni, d.nj, n, 0, 0, vb.coef, vb.invdiag};
    k_visc_light_coef<<<gb, kViscThreads, 0, st>>>(d, G.material, G.visc, (double)dt, vb.coef, vb.invdiag);
    k_visc_light_rhs<<<gb, kViscThreads, 0, st>>>(d, G.u, d.nj, density, vb.b);
    *launches += 2;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    int it = 0;
    bool ok = false;
    e = vcg_solve(s, false, vb, st, &it, &ok, launches);
    if (e != cudaSuccess) return e;
    *iters = -1;
    if (!ok) return cudaSuccess;
    k_visc_light_apply<<<gb, kViscThreads, 0, st>>>(d, vb.x, d.nj, (double)density, G.u);
    k_visc_light_rhs<<<gb, kViscThreads, 0, st>>>(d, G.v, d.nj + 1, density, vb.b);
    *launches += 2;
    e = vcg_solve(s, false, vb, st, &it, &ok, launches);
    if (e != cudaSuccess) return e;
    if (!ok) return cudaSuccess;
    k_visc_light_apply<<<gb, kViscThreads, 0, st>>>(d, vb.x, d.nj + 1, (double)density, G.v);
    *launches += 1;
    *iters = it;
    return cudaGetLastError();
}

cudaError_t visc_heavy(const GridDims &d, const Grids &G, float dt, float dx, float density,
                       ViscBuffers &vb, cudaStream_t st, int *iters, long long *launches)
{
    const long long nu = (long long)(d.ni + 1) * d.nj, nv = (long long)d.ni * (d.nj + 1);
    const int gb = grid_blocks(nu + nv);
    // viscositymodel.cpp:210-211, float arithmetic
    const float scaleTwoDt = 2 * dt / (dx * dx);
    const float scaleTwoDx = dt / (2 * dx * dx);
    ViscSys s{d.ni, d.nj, nu + nv, nu, nv, vb.coef, vb.invdiag};
    k_visc_heavy_coef<<<gb, kViscThreads, 0, st>>>(d, G.visc, scaleTwoDt, scaleTwoDx, density, vb.coef,
                                                    vb.invdiag);
    k_visc_heavy_rhs<<<gb, kViscThreads, 0, st>>>(nu, nv, G.u, G.v, density, vb.b);
    *launches += 2;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    int it = 0;
    bool ok = false;
    e = vcg_solve(s, true, vb, st, &it, &ok, launches);
    if (e != cudaSuccess) return e;
    *iters = -1;
    if (!ok) return cudaSuccess;
    k_visc_heavy_apply<<<gb, kViscThreads, 0, st>>>(nu, nv, vb.x, G.u, G.v);
    *launches += 1;
    *iters = it;
    return cudaGetLastError();
}

} // namespace fsg
