// fs_common.cuh -- device-side building blocks shared by the FLIP substep
// kernels: material encoding, the reference's clamped "centered" bilinear
// sampler, B-spline / hat weights and the bin geometry.
//
// Every helper restates the reference's float expression in the same order
// (cited file:line).  The translation units that include this header are
// compiled with -fmad=false, so no multiply-add is contracted and each result
// matches the reference CPU build (-ffp-contract=off) bit for bit.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace fsg {

// FluidMaterial codes, materialgrid.h:6-13
enum : int8_t { M_FLUID = 0x40, M_SOURCE = 0x41, M_SOLID = 0x20, M_SINK = 0x12, M_EMPTY = 0x10 };

// per-particle advection outcome
enum : uint8_t { P_STAY = 0, P_MOVE = 1, P_KILL = 2, P_GAP = 3 };

struct GridDims {
    int ni, nj;   // cells
    int bni, bnj; // bins of 3x3 cells (markerparticlesystem.cpp:12-13)
};

__host__ __device__ inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (hi < v ? hi : v); }
__host__ __device__ inline long long clampll(long long v, long long lo, long long hi)
{
    return v < lo ? lo : (hi < v ? hi : v);
}
__host__ __device__ inline float clampf(float v, float lo, float hi)
{
    return (v < lo) ? lo : ((hi < v) ? hi : v); // std::clamp
}
__host__ __device__ inline double clampd(double v, double lo, double hi)
{
    return (v < lo) ? lo : ((hi < v) ? hi : v);
}

// MaterialGrid getAt with OOB_EXTEND (materialgrid.cpp:5-8, grid2d.h:124-143)
__device__ __forceinline__ int8_t mat_at(const int8_t *__restrict__ m, const GridDims &d, int i, int j)
{
    i = clampi(i, 0, d.ni - 1);
    j = clampi(j, 0, d.nj - 1);
    return m[(size_t)i * d.nj + j];
}
__device__ __forceinline__ bool t_fluid(int8_t m) { return (m & M_FLUID) != 0; }
__device__ __forceinline__ bool t_strict_fluid(int8_t m) { return m == M_FLUID; }
__device__ __forceinline__ bool t_empty(int8_t m) { return (m & M_EMPTY) != 0; }
__device__ __forceinline__ bool t_solid(int8_t m) { return (m & M_SOLID) != 0; }
__device__ __forceinline__ bool t_sink(int8_t m) { return m == M_SINK; }

// simmath::frac / integr / lerp (mathfuncs.cpp:17-30)
__device__ __forceinline__ float sm_frac(float v) { return v - (float)(long long)v; }
__device__ __forceinline__ int sm_integr(float v) { return (int)floorf(v); }
__device__ __forceinline__ float sm_lerp(float a, float b, float f) { return (a * (1.0f - f)) + (b * f); }

// simmath::bSpline / quadraticBSpline (mathfuncs.cpp:32-43)
__device__ __forceinline__ float sm_bspline(float value)
{
    value = fabsf(value);
    float a = (0.75f - value * value) * (float)(value < 0.5f);
    float b = (0.5f * (1.5f - value) * (1.5f - value)) * (float)(value >= 0.5f && value < 1.5f);
    return a + b;
}
__device__ __forceinline__ float sm_qbspline(float x, float y)
{
    return sm_bspline(x) * sm_bspline(y) * 0.75f; // bSpline(0) == 0.75f exactly
}

// simmath::linearHat / bilinearHat (mathfuncs.cpp:100-116)
__device__ __forceinline__ float sm_linear_hat(float v)
{
    if (v >= 0 && v <= 1) return 1 - v;
    else if (v < 0 && v >= -1) return 1 + v;
    return 0;
}
__device__ __forceinline__ float sm_bilinear_hat(float x, float y)
{
    return sm_linear_hat(x) * sm_linear_hat(y) * 1.0f; // linearHat(0) == 1
}

// OOB_EXTEND read of a float grid
__device__ __forceinline__ float gget(const float *__restrict__ g, int si, int sj, long long i,
                                      long long j)
{
    i = clampll(i, 0, si - 1);
    j = clampll(j, 0, sj - 1);
    return __ldg(&g[(size_t)i * sj + j]);
}

// Grid2d::lerp (grid2d.h:187-216) == simmath::lerpCenteredGrid with an offset
__device__ __forceinline__ float grid_lerp(const float *__restrict__ g, int si, int sj, float ox,
                                           float oy, float i, float j)
{
    i += ox;
    j += oy;
    i = clampf(i, 0.f, (float)(si - 1));
    j = clampf(j, 0.f, (float)(sj - 1));
    int ci = sm_integr(i), cj = sm_integr(j);
    float fi = sm_frac(i), fj = sm_frac(j);
    int c2j = fj >= 0.5f ? cj + 1 : cj - 1;
    int c3i = fi >= 0.5f ? ci + 1 : ci - 1;
    float il = fi < 0.5f ? 0.5f - fi : fi - 0.5f;
    float jl = fj < 0.5f ? 0.5f - fj : fj - 0.5f;
    float v1 = sm_lerp(gget(g, si, sj, ci, cj), gget(g, si, sj, c3i, cj), il);
    float v2 = sm_lerp(gget(g, si, sj, ci, c2j), gget(g, si, sj, c3i, c2j), il);
    return sm_lerp(v1, v2, jl);
}

// StaggeredVelocityGrid::velocityAt (staggeredvelocitygrid.cpp:158-162):
// U is (NI+1) x NJ with offset (0.5, 0), V is NI x (NJ+1) with (0, 0.5).
__device__ __forceinline__ float2 velocity_at(const float *__restrict__ u, const float *__restrict__ v,
                                              const GridDims &d, float x, float y)
{
    return make_float2(grid_lerp(u, d.ni + 1, d.nj, 0.5f, 0.f, x, y),
                       grid_lerp(v, d.ni, d.nj + 1, 0.f, 0.5f, x, y));
}

// Geometry2d::signedDistance (geometry2d.cpp:54-73)
__device__ __forceinline__ float polygon_sdf(const float *__restrict__ xy, int n, float px, float py)
{
    float dx0 = px - xy[0], dy0 = py - xy[1];
    float sq = dx0 * dx0 + dy0 * dy0 + 0.f * 0.f;
    float sgn = 1.0f;
    for (int i = 0, j = n - 1; i < n; j = i, i++) {
        float ex = xy[2 * j] - xy[2 * i], ey = xy[2 * j + 1] - xy[2 * i + 1];
        float wx = px - xy[2 * i], wy = py - xy[2 * i + 1];
        float wde = wx * ex + wy * ey + 0.f * 0.f;
        float ede = ex * ex + ey * ey + 0.f * 0.f;
        float h = clampf(wde / ede, 0.0f, 1.0f);
        float bx = wx - ex * h, by = wy - ey * h;
        float bb = bx * bx + by * by + 0.f * 0.f;
        sq = (bb < sq) ? bb : sq;
        bool xf = py >= xy[2 * i + 1];
        bool yf = py < xy[2 * j + 1];
        bool zf = ex * wy > ey * wx;
        if ((xf && yf && zf) || (!xf && !yf && !zf)) sgn = -sgn;
    }
    return (float)((double)sgn * sqrt((double)sq));
}

// MarkerParticleSystem::gridToBinIdx (markerparticlesystem.cpp:97-102, 156-159)
__device__ __forceinline__ int bin_of_cell(const GridDims &d, long long i, long long j)
{
    long long bi = i / 3, bj = j / 3; // integer division toward zero
    if (bi < 0 || bi >= d.bni || bj < 0 || bj >= d.bnj) return -1;
    return (int)(bi * d.bnj + bj);
}
__device__ __forceinline__ int bin_of_pos(const GridDims &d, float x, float y)
{
    return bin_of_cell(d, (long long)x, (long long)y); // float -> ssize_t truncation
}

} // namespace fsg
