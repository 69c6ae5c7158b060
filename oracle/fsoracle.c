/*
 * fsoracle.c -- plain-C restatement of FlipSolver2d's FLIP substep.
 *
 * TEST INFRASTRUCTURE (see fsoracle.h).  This file restates, function by
 * function, the reference's liquid FLIP path (FlipSolver2dLib/, cited as
 * file:line) with the same floating-point operations in the same order, so
 * that compiled with -ffp-contract=off it reproduces the reference build
 * (oracle/Makefile.ref) bit for bit.  It is the checker for the CUDA path and,
 * where the reference sources are not available, the timed CPU baseline.
 *
 * Parallelism: the reference dispatches independent loops (per bin, per cell,
 * per vector chunk) to a thread pool (threading/threadpool.cpp).  Here those
 * loops run on `host_threads` pthreads; the results do not depend on the
 * thread count.  The two reductions whose results DO depend on the pool size
 * (VOps::dot and VOps::maxAbs, vmath.cpp:25-45,100-136) are split into
 * `ref_threads` chunks exactly as ThreadPool::splitRange does
 * (threadpool.cpp:41-76), independent of the host thread count.
 *
 * Restated: the FLIP step (FlipSolver, flipsolver2d.cpp) and the narrow-band
 * step (NBFlipSolver, nbflipsolver.cpp) with its std::mt19937 draws, the
 * sources/emitters of both (addSource, updateSources, reseedParticles,
 * updateGridFromSources), and the FP64 spec-mode solve fso_spec_solve (a plain
 * double-precision PCG with the textbook incomplete-Poisson preconditioner,
 * inversepoissonpreconditioner.h:45-79).
 * Not restated: viscosity (viscositymodel.cpp, whose solves are Eigen's
 * conjugate gradient) and the smoke and fire solvers.
 */
#define _GNU_SOURCE
#include "fsoracle.h"

#include <float.h>
#include <limits.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <sys/sysinfo.h>

/* material codes, materialgrid.h:6-13 */
enum { M_FLUID = 0x40, M_SOURCE = 0x41, M_SOLID = 0x20, M_SINK = 0x12, M_EMPTY = 0x10 };

/* ------------------------------------------------------------------------ */
/* small thread pool                                                        */
/* ------------------------------------------------------------------------ */
typedef void (*range_fn)(void *ctx, size_t begin, size_t end);

typedef struct pool {
    int n;
    pthread_t *th;
    pthread_mutex_t mu;
    pthread_cond_t cv_job, cv_done;
    unsigned long gen;
    int pending;
    int quit;
    struct worker_arg *args;
    range_fn fn;
    void *ctx;
    size_t total;
} pool;

typedef struct worker_arg {
    pool *p;
    int idx;
} worker_arg;

static void pool_chunk(size_t total, int parts, int k, size_t *b, size_t *e)
{
    size_t base = total / (size_t)parts, rem = total % (size_t)parts;
    *b = (size_t)k * base + ((size_t)k < rem ? (size_t)k : rem);
    *e = *b + base + ((size_t)k < rem ? 1 : 0);
}

static void *pool_worker(void *arg)
{
    worker_arg *wa = (worker_arg *)arg;
    pool *p = wa->p;
    unsigned long seen = 0;
    for (;;) {
        pthread_mutex_lock(&p->mu);
        while (p->gen == seen && !p->quit) pthread_cond_wait(&p->cv_job, &p->mu);
        if (p->quit) {
            pthread_mutex_unlock(&p->mu);
            break;
        }
        seen = p->gen;
        range_fn fn = p->fn;
        void *ctx = p->ctx;
        size_t total = p->total;
        pthread_mutex_unlock(&p->mu);
        size_t b, e;
        pool_chunk(total, p->n, wa->idx, &b, &e);
        if (b < e) fn(ctx, b, e);
        pthread_mutex_lock(&p->mu);
        if (--p->pending == 0) pthread_cond_signal(&p->cv_done);
        pthread_mutex_unlock(&p->mu);
    }
    return NULL;
}

static pool *pool_create(int n)
{
    pool *p = (pool *)calloc(1, sizeof(pool));
    p->n = n < 1 ? 1 : n;
    pthread_mutex_init(&p->mu, NULL);
    pthread_cond_init(&p->cv_job, NULL);
    pthread_cond_init(&p->cv_done, NULL);
    if (p->n > 1) {
        p->th = (pthread_t *)calloc((size_t)p->n, sizeof(pthread_t));
        worker_arg *args = (worker_arg *)calloc((size_t)p->n, sizeof(worker_arg));
        for (int i = 0; i < p->n; i++) {
            args[i].p = p;
            args[i].idx = i;
            pthread_create(&p->th[i], NULL, pool_worker, &args[i]);
        }
        p->args = args;
    }
    return p;
}

static void pool_destroy(pool *p)
{
    if (!p) return;
    if (p->n > 1) {
        pthread_mutex_lock(&p->mu);
        p->quit = 1;
        pthread_cond_broadcast(&p->cv_job);
        pthread_mutex_unlock(&p->mu);
        for (int i = 0; i < p->n; i++) pthread_join(p->th[i], NULL);
        free(p->th);
        free(p->args);
    }
    free(p);
}

static void par_for(pool *p, size_t total, range_fn fn, void *ctx)
{
    if (total == 0) return;
    if (!p || p->n <= 1 || total < 2) {
        fn(ctx, 0, total);
        return;
    }
    pthread_mutex_lock(&p->mu);
    p->fn = fn;
    p->ctx = ctx;
    p->total = total;
    p->pending = p->n;
    p->gen++;
    pthread_cond_broadcast(&p->cv_job);
    while (p->pending > 0) pthread_cond_wait(&p->cv_done, &p->mu);
    pthread_mutex_unlock(&p->mu);
}

/* ------------------------------------------------------------------------ */
/* ThreadPool::splitRange (threadpool.cpp:41-76)                             */
/* ------------------------------------------------------------------------ */
typedef struct range {
    size_t start, end;
} range;

/* Writes at most `parts` ranges into out; returns how many. */
static size_t split_range(size_t length, size_t parts, range *out)
{
    if (length == 0) return 0;
    size_t numParts = parts;
    if (length < numParts) numParts = length;
    size_t partSize = length / numParts;
    if (partSize < 1) partSize = 1;
    size_t remainder = 0;
    if (partSize * numParts < length) remainder = length - partSize * numParts;
    size_t cs = 0, ce = partSize < length ? partSize : length;
    size_t k = 0;
    for (size_t i = 0; i < numParts; i++) {
        if (i < remainder) ce++;
        out[k].start = cs;
        out[k].end = ce;
        k++;
        cs = ce;
        ce = cs + partSize < length ? cs + partSize : length;
        if (ce == cs) break;
    }
    return k;
}

/* ------------------------------------------------------------------------ */
/* mt19937 (Matsumoto & Nishimura 1998) and the float draw of                */
/* std::uniform_real_distribution<float>(0,1) over it                        */
/* ------------------------------------------------------------------------ */
typedef struct mt19937 {
    uint32_t mt[624];
    int idx;
} mt19937;

static void mt_seed(mt19937 *g, uint32_t seed)
{
    g->mt[0] = seed;
    for (int i = 1; i < 624; i++)
        g->mt[i] = 1812433253u * (g->mt[i - 1] ^ (g->mt[i - 1] >> 30)) + (uint32_t)i;
    g->idx = 624;
}

static uint32_t mt_next(mt19937 *g)
{
    if (g->idx >= 624) {
        for (int i = 0; i < 624; i++) {
            uint32_t y = (g->mt[i] & 0x80000000u) | (g->mt[(i + 1) % 624] & 0x7fffffffu);
            uint32_t v = g->mt[(i + 397) % 624] ^ (y >> 1);
            if (y & 1u) v ^= 0x9908b0dfu;
            g->mt[i] = v;
        }
        g->idx = 0;
    }
    uint32_t y = g->mt[g->idx++];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    return y;
}

/* A 32-bit engine draw scaled into [0,1) in float: one draw, converted to
 * float with round-to-nearest, divided by 2^32, values that round up to 1
 * replaced by the largest float below 1. */
static float mt_uniform01f(mt19937 *g)
{
    float sum = 0.0f + (float)mt_next(g) * 1.0f;
    float r = sum / 4294967296.0f;
    if (r >= 1.0f) r = nextafterf(1.0f, 0.0f);
    return r * (1.0f - 0.0f) + 0.0f;
}

/* ------------------------------------------------------------------------ */
/* particle bins (markerparticlesystem.h:59-149)                             */
/* ------------------------------------------------------------------------ */
typedef struct pbin {
    size_t n, cap;
    float *pos;
    float *vel;
    float *visc;
    uint8_t *dead;
} pbin;

static void bin_reserve(pbin *b, size_t cap)
{
    if (cap <= b->cap) return;
    size_t c = b->cap ? b->cap : 8;
    while (c < cap) c *= 2;
    b->pos = (float *)realloc(b->pos, c * 2 * sizeof(float));
    b->vel = (float *)realloc(b->vel, c * 2 * sizeof(float));
    b->visc = (float *)realloc(b->visc, c * sizeof(float));
    b->dead = (uint8_t *)realloc(b->dead, c);
    b->cap = c;
}

static void bin_free(pbin *b)
{
    free(b->pos);
    free(b->vel);
    free(b->visc);
    free(b->dead);
    memset(b, 0, sizeof(*b));
}

/* ParticleBin::addMarkerParticle (markerparticlesystem.cpp:175-196) */
static size_t bin_push(pbin *b, float px, float py, float vx, float vy, float visc, uint8_t dead)
{
    bin_reserve(b, b->n + 1);
    size_t k = b->n++;
    b->pos[2 * k] = px;
    b->pos[2 * k + 1] = py;
    b->vel[2 * k] = vx;
    b->vel[2 * k + 1] = vy;
    b->visc[k] = visc;
    b->dead[k] = dead;
    return k;
}

/* ParticleBin::eraseMarkerParticle (markerparticlesystem.cpp:198-216):
 * swap with the last particle, then pop. */
static void bin_swap_erase(pbin *b, size_t k)
{
    size_t l = b->n - 1;
    float t;
    t = b->pos[2 * k]; b->pos[2 * k] = b->pos[2 * l]; b->pos[2 * l] = t;
    t = b->pos[2 * k + 1]; b->pos[2 * k + 1] = b->pos[2 * l + 1]; b->pos[2 * l + 1] = t;
    t = b->vel[2 * k]; b->vel[2 * k] = b->vel[2 * l]; b->vel[2 * l] = t;
    t = b->vel[2 * k + 1]; b->vel[2 * k + 1] = b->vel[2 * l + 1]; b->vel[2 * l + 1] = t;
    t = b->visc[k]; b->visc[k] = b->visc[l]; b->visc[l] = t;
    uint8_t d = b->dead[k]; b->dead[k] = b->dead[l]; b->dead[l] = d;
    b->n--;
}

/* ------------------------------------------------------------------------ */
/* solver state                                                             */
/* ------------------------------------------------------------------------ */
typedef struct poly {
    int n;
    float *xy;
    float a; /* friction / viscosity / divergence */
} poly;

/* Emitter (emitter.h): a polygon with the parameters the liquid solvers read */
typedef struct source {
    poly g;
    float visc, div, vx, vy;
    int transfer; /* velocityTransfer() */
} source;

typedef struct rebin_rec {
    size_t particle;
    size_t dest;
} rebin_rec;

typedef struct rec_list {
    size_t n, cap;
    rebin_rec *r;
} rec_list;

struct fso_solver {
    fso_params p;
    int ni, nj, bni, bnj;
    size_t ncell, nu, nv, nbins;
    double dx, density;
    float step_dt, frame_dt;
    int frame;

    pbin *bins;
    pbin rebin;
    size_t *rebin_dest;
    size_t rebin_dest_cap;
    rec_list *recs; /* per-bin advect rebin records */

    int8_t *material;
    float *solid_sdf, *fluid_sdf;
    int32_t *solid_id, *emitter_id, *counts;
    float *u, *v, *su, *sv;
    uint8_t *uvalid, *vvalid, *suvalid, *svvalid;
    float *visc_grid;
    uint8_t *known;
    float *divc;
    float *dens;
    double *dens_rhs, *dens_p;
    int dens_sized;
    double *pres, *pres_rhs;

    /* matrix frozen at the DECOMPOSITION stage */
    uint8_t *unit;    /* cell is a unit (fluid at build time) */
    uint8_t *mask;    /* NeighborMask bits */
    uint8_t *ucount;  /* nonsolidNeighborCount of the unit */
    double *ipp;      /* 4 per cell: iNeg, iPos, jNeg, jPos */
    double mscale;
    int have_units;

    /* PCG scratch */
    double *w_r, *w_aux, *w_s;

    poly *obst;
    int nobst;
    poly *fluids;
    int nfluids;
    poly *sinks;
    int nsinks;
    source *sources;
    int nsources;

    mt19937 rng;
    /* NB-FLIP (nbflipsolver.h:63-75): the advected grids */
    int nb;
    float *adv_u, *adv_v, *adv_sdf, *adv_visc;
    int density_iters, pressure_iters, substeps;
    int viscosity_iters; /* SolverStats::viscosityIterations */
    int ref_threads, host_threads;
    pool *pool;
};

/* ---- grid access with the reference's out-of-bounds strategies ---------- */
static inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (hi < v ? hi : v); }
static inline float clampf(float v, float lo, float hi) { return (v < lo) ? lo : ((hi < v) ? hi : v); }
static inline double clampd(double v, double lo, double hi) { return (v < lo) ? lo : ((hi < v) ? hi : v); }

/* MaterialGrid uses OOB_EXTEND (materialgrid.cpp:5-8, grid2d.h:124-143) */
static inline int8_t mat_at(const fso_solver *s, long i, long j)
{
    i = i < 0 ? 0 : (i > s->ni - 1 ? s->ni - 1 : i);
    j = j < 0 ? 0 : (j > s->nj - 1 ? s->nj - 1 : j);
    return s->material[i * s->nj + j];
}
static inline int is_fluid(const fso_solver *s, long i, long j) { return (mat_at(s, i, j) & M_FLUID) != 0; }
static inline int is_strict_fluid(const fso_solver *s, long i, long j) { return mat_at(s, i, j) == M_FLUID; }
static inline int is_empty(const fso_solver *s, long i, long j) { return (mat_at(s, i, j) & M_EMPTY) != 0; }
static inline int is_solid(const fso_solver *s, long i, long j) { return (mat_at(s, i, j) & M_SOLID) != 0; }
static inline int is_sink(const fso_solver *s, long i, long j) { return mat_at(s, i, j) == M_SINK; }
static inline int is_source(const fso_solver *s, long i, long j) { return mat_at(s, i, j) == M_SOURCE; }

/* LinearIndexable2d::linearIndex (linearindexable2d.h:30-37) */
static inline long lin_index(const fso_solver *s, long i, long j)
{
    if (i < 0 || i >= s->ni || j < 0 || j >= s->nj) return -1;
    return i * s->nj + j;
}
static inline int in_bounds(const fso_solver *s, long i, long j)
{
    return i >= 0 && i < s->ni && j >= 0 && j < s->nj;
}

/* OOB_EXTEND fetch of a float grid of size si x sj */
static inline float gget(const float *g, int si, int sj, long i, long j)
{
    i = i < 0 ? 0 : (i > si - 1 ? si - 1 : i);
    j = j < 0 ? 0 : (j > sj - 1 ? sj - 1 : j);
    return g[i * sj + j];
}

/* ---- simmath (mathfuncs.cpp) ------------------------------------------- */
static inline float sm_frac(float v) { return v - (float)(long)v; }             /* :17-20 */
static inline int sm_integr(float v) { return (int)floorf(v); }                 /* :22-25 */
static inline float sm_lerp(float a, float b, float f) { return (a * (1.0f - f)) + (b * f); } /* :27-30 */

static inline float sm_bspline(float value) /* :32-37 */
{
    value = fabsf(value);
    float a = (0.75f - value * value) * (float)(value < 0.5f);
    float b = (0.5f * (1.5f - value) * (1.5f - value)) * (float)(value >= 0.5f && value < 1.5f);
    return a + b;
}

static inline float sm_qbspline(float x, float y) /* :39-43 */
{
    return sm_bspline(x) * sm_bspline(y) * sm_bspline(0.f);
}

static inline float sm_linear_hat(float value) /* :100-111 */
{
    if (value >= 0 && value <= 1) return 1 - value;
    else if (value < 0 && value >= -1) return 1 + value;
    return 0;
}

static inline float sm_bilinear_hat(float x, float y) /* :113-116 */
{
    return sm_linear_hat(x) * sm_linear_hat(y) * sm_linear_hat(0.f);
}

/* Grid2d::lerp (grid2d.h:187-216) and simmath::lerpCenteredGrid
 * (mathfuncs.cpp:128-150): clamped "centered" bilinear sample. */
static float grid_lerp(const float *g, int si, int sj, float ox, float oy, float i, float j)
{
    i += ox;
    j += oy;
    i = clampf(i, 0.f, (float)(si - 1));
    j = clampf(j, 0.f, (float)(sj - 1));
    long ci = sm_integr(i), cj = sm_integr(j);
    float fi = sm_frac(i), fj = sm_frac(j);
    long c2i = ci, c2j = fj >= 0.5f ? cj + 1 : cj - 1;
    long c3i = fi >= 0.5f ? ci + 1 : ci - 1, c3j = fj >= 0.5f ? cj + 1 : cj - 1;
    long c4i = fi >= 0.5f ? ci + 1 : ci - 1, c4j = cj;
    float il = fi < 0.5f ? 0.5f - fi : fi - 0.5f;
    float jl = fj < 0.5f ? 0.5f - fj : fj - 0.5f;
    float v1 = sm_lerp(gget(g, si, sj, ci, cj), gget(g, si, sj, c4i, c4j), il);
    float v2 = sm_lerp(gget(g, si, sj, c2i, c2j), gget(g, si, sj, c3i, c3j), il);
    return sm_lerp(v1, v2, jl);
}

/* simmath::gradCenteredGrid (mathfuncs.cpp:87-98); the reference passes
 * float coordinates to ssize_t parameters, i.e. truncates toward zero. */
static void grad_centered(const float *g, int si, int sj, long i, long j, float *gi, float *gj)
{
    float ip1 = gget(g, si, sj, i + 1, j);
    float im1 = gget(g, si, sj, i - 1, j);
    float jp1 = gget(g, si, sj, i, j + 1);
    float jm1 = gget(g, si, sj, i, j - 1);
    *gi = (ip1 - im1) / 2.f;
    *gj = (jp1 - jm1) / 2.f;
}

/* StaggeredVelocityGrid::velocityAt (staggeredvelocitygrid.cpp:158-162):
 * U grid (NI+1) x NJ with offset (0.5, 0), V grid NI x (NJ+1) with (0, 0.5)
 * (staggeredvelocitygrid.cpp:6-14). */
static inline void velocity_at(const fso_solver *s, const float *u, const float *v, float x,
                               float y, float *ox, float *oy)
{
    *ox = grid_lerp(u, s->ni + 1, s->nj, 0.5f, 0.f, x, y);
    *oy = grid_lerp(v, s->ni, s->nj + 1, 0.f, 0.5f, x, y);
}

/* FlipSolver::rk4Integrate (flipsolver2d.cpp:1195-1203) */
static void rk4(const fso_solver *s, float *px, float *py, float dt)
{
    float x = *px, y = *py, vx, vy;
    velocity_at(s, s->u, s->v, x, y, &vx, &vy);
    float k1x = vx * dt, k1y = vy * dt;
    velocity_at(s, s->u, s->v, x + k1x * 0.5f, y + k1y * 0.5f, &vx, &vy);
    float k2x = vx * dt, k2y = vy * dt;
    velocity_at(s, s->u, s->v, x + k2x * 0.5f, y + k2y * 0.5f, &vx, &vy);
    float k3x = vx * dt, k3y = vy * dt;
    velocity_at(s, s->u, s->v, x + k3x, y + k3y, &vx, &vy);
    float k4x = vx * dt, k4y = vy * dt;
    float sx = ((k1x + k2x * 2.f) + k3x * 2.f) + k4x;
    float sy = ((k1y + k2y * 2.f) + k3y * 2.f) + k4y;
    *px = x + sx * (1.0f / 6.0f);
    *py = y + sy * (1.0f / 6.0f);
}

/* SdfGrid::closestSurfacePoint (sdfgrid.cpp:15-46) */
static void closest_surface_point(const fso_solver *s, float *px, float *py)
{
    const float *g = s->solid_sdf;
    int si = s->ni, sj = s->nj;
    float cx = *px, cy = *py;
    float value = grid_lerp(g, si, sj, 0.f, 0.f, cx, cy);
    float gx, gy;
    grad_centered(g, si, sj, (long)cx, (long)cy, &gx, &gy);
    for (int it = 0; it < 100; it++) {
        float alpha = 1;
        for (int jt = 0; jt < 10; jt++) {
            float av = alpha * value;
            float qx = cx - gx * av, qy = cy - gy * av;
            if (fabsf(grid_lerp(g, si, sj, 0.f, 0.f, qx, qy)) < fabsf(value)) {
                cx = qx;
                cy = qy;
                value = grid_lerp(g, si, sj, 0.f, 0.f, qx, qy);
                grad_centered(g, si, sj, (long)qx, (long)qy, &gx, &gy);
                if (fabsf(value) < 1e-5f) {
                    *px = cx;
                    *py = cy;
                    return;
                }
            } else {
                alpha *= 0.7f;
            }
        }
    }
    *px = cx;
    *py = cy;
}

/* MarkerParticleSystem::gridToBinIdx (markerparticlesystem.cpp:97-102,156-159):
 * cell -> bin by integer division (toward zero), -1 outside the bin grid. */
static inline long bin_of_cell(const fso_solver *s, long i, long j)
{
    long bi = i / 3, bj = j / 3;
    if (bi < 0 || bi >= s->bni || bj < 0 || bj >= s->bnj) return -1;
    return bi * s->bnj + bj;
}
static inline long bin_of_pos(const fso_solver *s, float x, float y)
{
    return bin_of_cell(s, (long)x, (long)y);
}

/* MarkerParticleSystem::binsForGridCell (markerparticlesystem.cpp:109-128) */
static void bins_for_cell(const fso_solver *s, long i, long j, long out[9])
{
    long ci = i / 3, cj = j / 3;
    int k = 0;
    for (long io = -1; io <= 1; io++)
        for (long jo = -1; jo <= 1; jo++) {
            long bi = ci + io, bj = cj + jo;
            out[k++] = (bi >= 0 && bi < s->bni && bj >= 0 && bj < s->bnj) ? bi * s->bnj + bj : -1;
        }
}

/* Geometry2d::signedDistance (geometry2d.cpp:54-73) */
static float polygon_sdf(const poly *g, float px, float py)
{
    float dx0 = px - g->xy[0], dy0 = py - g->xy[1];
    float sq = dx0 * dx0 + dy0 * dy0 + 0.f * 0.f;
    float sgn = 1.0f;
    int N = g->n;
    for (int i = 0, j = N - 1; i < N; j = i, i++) {
        float ex = g->xy[2 * j] - g->xy[2 * i], ey = g->xy[2 * j + 1] - g->xy[2 * i + 1];
        float wx = px - g->xy[2 * i], wy = py - g->xy[2 * i + 1];
        float wde = wx * ex + wy * ey + 0.f * 0.f;
        float ede = ex * ex + ey * ey + 0.f * 0.f;
        float h = clampf(wde / ede, 0.0f, 1.0f);
        float bx = wx - ex * h, by = wy - ey * h;
        float bb = bx * bx + by * by + 0.f * 0.f;
        sq = (bb < sq) ? bb : sq;
        int xf = py >= g->xy[2 * i + 1];
        int yf = py < g->xy[2 * j + 1];
        int zf = ex * wy > ey * wx;
        int allC = xf && yf && zf;
        int allNC = !xf && !yf && !zf;
        if (allC || allNC) sgn *= -1.0f;
    }
    return (float)((double)sgn * sqrt((double)sq));
}

/* ------------------------------------------------------------------------ */
/* creation / destruction                                                   */
/* ------------------------------------------------------------------------ */
static int env_int(const char *name, int dflt)
{
    const char *v = getenv(name);
    if (!v || !*v) return dflt;
    int x = atoi(v);
    return x > 0 ? x : dflt;
}

fso_solver *fso_create(const fso_params *p)
{
    fso_solver *s = (fso_solver *)calloc(1, sizeof(fso_solver));
    s->p = *p;
    s->ni = p->gridSizeI;
    s->nj = p->gridSizeJ;
    s->bni = s->ni / 3 + (s->ni % 3 != 0); /* markerparticlesystem.cpp:12-13 */
    s->bnj = s->nj / 3 + (s->nj % 3 != 0);
    s->ncell = (size_t)s->ni * s->nj;
    s->nu = (size_t)(s->ni + 1) * s->nj;
    s->nv = (size_t)s->ni * (s->nj + 1);
    s->nbins = (size_t)s->bni * s->bnj;
    s->dx = p->dx;
    s->density = p->fluidDensity;
    s->step_dt = 1.f / p->fps; /* flipsolver2d.cpp:46-47 */
    s->frame_dt = 1.f / p->fps;
    s->bins = (pbin *)calloc(s->nbins, sizeof(pbin));
    s->recs = (rec_list *)calloc(s->nbins, sizeof(rec_list));
    size_t n = s->ncell;
    s->material = (int8_t *)malloc(n);
    memset(s->material, M_EMPTY, n); /* MaterialGrid init EMPTY, materialgrid.cpp:6 */
    s->solid_sdf = (float *)calloc(n, sizeof(float));
    s->fluid_sdf = (float *)calloc(n, sizeof(float));
    s->solid_id = (int32_t *)malloc(n * sizeof(int32_t));
    s->emitter_id = (int32_t *)malloc(n * sizeof(int32_t));
    for (size_t k = 0; k < n; k++) s->solid_id[k] = s->emitter_id[k] = -1;
    s->counts = (int32_t *)calloc(n, sizeof(int32_t));
    s->u = (float *)calloc(s->nu, sizeof(float));
    s->v = (float *)calloc(s->nv, sizeof(float));
    s->su = (float *)calloc(s->nu, sizeof(float));
    s->sv = (float *)calloc(s->nv, sizeof(float));
    s->uvalid = (uint8_t *)calloc(s->nu, 1);
    s->vvalid = (uint8_t *)calloc(s->nv, 1);
    s->suvalid = (uint8_t *)calloc(s->nu, 1);
    s->svvalid = (uint8_t *)calloc(s->nv, 1);
    s->visc_grid = (float *)calloc(n, sizeof(float));
    s->known = (uint8_t *)calloc(n, 1);
    s->divc = (float *)calloc(n, sizeof(float));
    s->dens = (float *)calloc(n, sizeof(float));
    s->dens_rhs = (double *)calloc(n, sizeof(double));
    s->dens_p = (double *)calloc(n, sizeof(double));
    s->pres = (double *)calloc(n, sizeof(double));
    s->pres_rhs = (double *)calloc(n, sizeof(double));
    s->unit = (uint8_t *)calloc(n, 1);
    s->mask = (uint8_t *)calloc(n, 1);
    s->ucount = (uint8_t *)calloc(n, 1);
    s->ipp = (double *)calloc(4 * n, sizeof(double));
    s->w_r = (double *)calloc(n, sizeof(double));
    s->w_aux = (double *)calloc(n, sizeof(double));
    s->w_s = (double *)calloc(n, sizeof(double));
    mt_seed(&s->rng, p->seed); /* flipsolver2d.cpp:71 */
    s->ref_threads = env_int("FSO_REF_THREADS", 8);
    s->host_threads = env_int("FSO_HOST_THREADS", 1);
    s->pool = pool_create(s->host_threads);
    return s;
}

fso_solver *fso_create_nbflip(const fso_params *p) /* nbflipsolver.cpp:9-23 */
{
    fso_solver *s = fso_create(p);
    s->nb = 1;
    s->adv_u = (float *)calloc(s->nu, sizeof(float));
    s->adv_v = (float *)calloc(s->nv, sizeof(float));
    s->adv_sdf = (float *)calloc(s->ncell, sizeof(float));
    s->adv_visc = (float *)calloc(s->ncell, sizeof(float));
    return s;
}

int fso_get_rng(fso_solver *s, uint32_t state[625])
{
    memcpy(state, s->rng.mt, sizeof(s->rng.mt));
    state[624] = (uint32_t)s->rng.idx;
    return 0;
}

int fso_set_rng(fso_solver *s, const uint32_t state[625])
{
    if (state[624] > 624) return -1;
    memcpy(s->rng.mt, state, sizeof(s->rng.mt));
    s->rng.idx = (int)state[624];
    return 0;
}

static void free_polys(poly *p, int n)
{
    for (int i = 0; i < n; i++) free(p[i].xy);
    free(p);
}

void fso_destroy(fso_solver *s)
{
    if (!s) return;
    pool_destroy(s->pool);
    for (size_t b = 0; b < s->nbins; b++) {
        bin_free(&s->bins[b]);
        free(s->recs[b].r);
    }
    free(s->bins);
    free(s->recs);
    bin_free(&s->rebin);
    free(s->rebin_dest);
    void *ptrs[] = {s->material, s->solid_sdf, s->fluid_sdf, s->solid_id, s->emitter_id,
                    s->counts, s->u, s->v, s->su, s->sv, s->uvalid, s->vvalid, s->suvalid,
                    s->svvalid, s->visc_grid, s->known, s->divc, s->dens, s->dens_rhs, s->dens_p,
                    s->pres, s->pres_rhs, s->unit, s->mask, s->ucount, s->ipp, s->w_r,
                    s->w_aux, s->w_s, s->adv_u, s->adv_v, s->adv_sdf, s->adv_visc};
    for (size_t k = 0; k < sizeof(ptrs) / sizeof(ptrs[0]); k++) free(ptrs[k]);
    free_polys(s->obst, s->nobst);
    free_polys(s->fluids, s->nfluids);
    free_polys(s->sinks, s->nsinks);
    for (int k = 0; k < s->nsources; k++) free(s->sources[k].g.xy);
    free(s->sources);
    free(s);
}

static void add_poly(poly **arr, int *n, float a, const float *xy, int nv)
{
    *arr = (poly *)realloc(*arr, (size_t)(*n + 1) * sizeof(poly));
    poly *g = &(*arr)[*n];
    g->n = nv;
    g->a = a;
    g->xy = (float *)malloc((size_t)nv * 2 * sizeof(float));
    memcpy(g->xy, xy, (size_t)nv * 2 * sizeof(float));
    (*n)++;
}

int fso_add_source(fso_solver *s, const float *xy, int n, float viscosity, float divergence,
                   float vx, float vy, int transfer) /* FlipSolver::addSource, :602-605 */
{
    s->sources = (source *)realloc(s->sources, (size_t)(s->nsources + 1) * sizeof(source));
    source *e = &s->sources[s->nsources];
    e->g.n = n;
    e->g.a = 0.f;
    e->g.xy = (float *)malloc((size_t)n * 2 * sizeof(float));
    memcpy(e->g.xy, xy, (size_t)n * 2 * sizeof(float));
    e->visc = viscosity;
    e->div = divergence;
    e->vx = vx;
    e->vy = vy;
    e->transfer = transfer != 0;
    s->nsources++;
    return 0;
}

int fso_add_geometry(fso_solver *s, float friction, const float *xy, int n)
{
    add_poly(&s->obst, &s->nobst, friction, xy, n);
    return 0;
}
int fso_add_initial_fluid(fso_solver *s, float viscosity, const float *xy, int n)
{
    add_poly(&s->fluids, &s->nfluids, viscosity, xy, n);
    return 0;
}
int fso_add_sink(fso_solver *s, float divergence, const float *xy, int n)
{
    add_poly(&s->sinks, &s->nsinks, divergence, xy, n);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* frame-0 scene setup (flipsolver2d.cpp:502-590, 682-707, 788-795)          */
/* ------------------------------------------------------------------------ */
static void update_sinks(fso_solver *s) /* :554-571 */
{
    float dx = (float)s->dx;
    for (long i = 0; i < s->ni; i++)
        for (long j = 0; j < s->nj; j++)
            for (int k = 0; k < s->nsinks; k++)
                if (polygon_sdf(&s->sinks[k], ((float)i + 0.5f) * dx, ((float)j + 0.5f) * dx) <= 0.f) {
                    s->material[i * s->nj + j] = M_SINK;
                    s->divc[i * s->nj + j] = s->sinks[k].a;
                }
}

static void update_sources(fso_solver *s) /* :532-552 */
{
    const float dx = (float)s->dx;
    const float hdx = (float)(dx / 2.0);
    for (long i = 0; i < s->ni; i++)
        for (long j = 0; j < s->nj; j++)
            for (int k = 0; k < s->nsources; k++)
                if (polygon_sdf(&s->sources[k].g, (float)i * dx + hdx, (float)j * dx + hdx) <= 0.f) {
                    s->material[i * s->nj + j] = M_SOURCE;
                    s->emitter_id[i * s->nj + j] = k;
                    s->divc[i * s->nj + j] = s->sources[k].div;
                }
}

static void update_solids(fso_solver *s) /* :502-530 */
{
    float dx = (float)s->dx;
    for (long i = 0; i < s->ni; i++)
        for (long j = 0; j < s->nj; j++) {
            float dist = FLT_MAX;
            int minIdx = 0;
            for (int k = 0; k < s->nobst; k++) {
                /* (static_cast<float>(i)+0.5)*dx is evaluated in double */
                float x = (float)(((double)(float)i + 0.5) * (double)dx);
                float y = (float)(((double)(float)j + 0.5) * (double)dx);
                float sdf = polygon_sdf(&s->obst[k], x, y) / dx;
                if (sdf < dist) {
                    minIdx = k;
                    dist = sdf;
                }
            }
            s->solid_sdf[i * s->nj + j] = dist;
            if (dist < 0) {
                s->material[i * s->nj + j] = M_SOLID;
                s->solid_id[i * s->nj + j] = minIdx;
            }
        }
}

static void update_initial_fluid(fso_solver *s) /* :573-590 */
{
    float dx = (float)s->dx;
    for (long i = 0; i < s->ni; i++)
        for (long j = 0; j < s->nj; j++)
            for (int k = 0; k < s->nfluids; k++)
                if (polygon_sdf(&s->fluids[k], ((float)i + 0.5f) * dx, ((float)j + 0.5f) * dx) <= 0.f) {
                    s->material[i * s->nj + j] = M_FLUID;
                    s->visc_grid[i * s->nj + j] = s->fluids[k].a;
                }
}

static void seed_initial_fluid(fso_solver *s) /* :682-707 */
{
    for (long i = 0; i < s->ni; i++)
        for (long j = 0; j < s->nj; j++) {
            if (!is_strict_fluid(s, i, j)) continue;
            pbin *cellbin = &s->bins[bin_of_cell(s, i, j)];
            for (int k = 0; k < s->p.particlesPerCell; k++) {
                /* jitteredPosInCell, :1013-1019 */
                float x = (float)i + mt_uniform01f(&s->rng);
                float y = (float)j + mt_uniform01f(&s->rng);
                float vx, vy;
                velocity_at(s, s->u, s->v, x, y, &vx, &vy);
                float visc = grid_lerp(s->visc_grid, s->ni, s->nj, 0.5f, 0.5f, x, y);
                pbin *dst = &s->bins[bin_of_pos(s, x, y)];
                size_t idx = bin_push(dst, x, y, vx, vy, 0.f, 0);
                /* the reference stores the viscosity through the property
                 * vector of the cell's bin at the index returned by the
                 * position's bin; both are the same bin unless i + U(0,1)
                 * rounded up into the next bin */
                if (idx < cellbin->n) cellbin->visc[idx] = visc;
            }
        }
}

static void nb_first_frame_init(fso_solver *s);

void fso_first_frame_init(fso_solver *s)
{
    if (s->nb) {
        nb_first_frame_init(s);
        return;
    }
    update_sinks(s);
    update_sources(s);
    update_solids(s);
    update_initial_fluid(s);
    seed_initial_fluid(s);
}

/* ------------------------------------------------------------------------ */
/* advection (flipsolver2d.cpp:138-162, 305-338)                             */
/* ------------------------------------------------------------------------ */
static void advect_range(void *ctx, size_t b0, size_t b1)
{
    fso_solver *s = (fso_solver *)ctx;
    for (size_t b = b0; b < b1; b++) {
        pbin *bin = &s->bins[b];
        rec_list *rl = &s->recs[b];
        rl->n = 0;
        for (size_t k = 0; k < bin->n; k++) {
            float x = bin->pos[2 * k], y = bin->pos[2 * k + 1];
            long oldBin = bin_of_pos(s, x, y);
            rk4(s, &x, &y, s->step_dt);
            if (grid_lerp(s->solid_sdf, s->ni, s->nj, 0.f, 0.f, x, y) < 0.f)
                closest_surface_point(s, &x, &y);
            bin->pos[2 * k] = x;
            bin->pos[2 * k + 1] = y;
            long pI = sm_integr(x), pJ = sm_integr(y);
            long newBin = bin_of_pos(s, x, y);
            if (!in_bounds(s, pI, pJ) || is_sink(s, pI, pJ)) {
                bin->dead[k] = 1;
            } else if (newBin != oldBin) {
                if (rl->n == rl->cap) {
                    rl->cap = rl->cap ? 2 * rl->cap : 8;
                    rl->r = (rebin_rec *)realloc(rl->r, rl->cap * sizeof(rebin_rec));
                }
                rl->r[rl->n].particle = k;
                rl->r[rl->n].dest = (size_t)newBin;
                rl->n++;
            }
        }
    }
}

static void advect(fso_solver *s)
{
    par_for(s->pool, s->nbins, advect_range, s);
    /* MarkerParticleSystem::scheduleRebin / ParticleBin::scheduleRebin
     * (markerparticlesystem.cpp:60-63, 317-342): in bin order, copy each moved
     * particle into the rebin set and mark the original for death. */
    for (size_t b = 0; b < s->nbins; b++) {
        pbin *bin = &s->bins[b];
        rec_list *rl = &s->recs[b];
        for (size_t r = 0; r < rl->n; r++) {
            size_t k = rl->r[r].particle;
            size_t slot = bin_push(&s->rebin, bin->pos[2 * k], bin->pos[2 * k + 1],
                                   bin->vel[2 * k], bin->vel[2 * k + 1], bin->visc[k],
                                   bin->dead[k]);
            if (slot >= s->rebin_dest_cap) {
                s->rebin_dest_cap = s->rebin_dest_cap ? 2 * s->rebin_dest_cap : 64;
                while (s->rebin_dest_cap <= slot) s->rebin_dest_cap *= 2;
                s->rebin_dest = (size_t *)realloc(s->rebin_dest, s->rebin_dest_cap * sizeof(size_t));
            }
            s->rebin_dest[slot] = rl->r[r].dest;
            bin->dead[k] = 1;
        }
        rl->n = 0;
    }
}

/* ------------------------------------------------------------------------ */
/* pruning and rebinning                                                     */
/* ------------------------------------------------------------------------ */
static void prune(fso_solver *s) /* flipsolver2d.cpp:353-359; markerparticlesystem.cpp:248-258 */
{
    for (size_t b = 0; b < s->nbins; b++) {
        pbin *bin = &s->bins[b];
        for (size_t k = 0; k < bin->n; k++) {
            if (bin->dead[k]) {
                bin_swap_erase(bin, k);
                k--;
            }
        }
    }
}

static void rebin_range(void *ctx, size_t b0, size_t b1)
{
    fso_solver *s = (fso_solver *)ctx;
    pbin *rs = &s->rebin;
    for (size_t b = b0; b < b1; b++) {
        pbin *bin = &s->bins[b];
        /* ParticleBin::rebinParticles (markerparticlesystem.cpp:260-269):
         * every bin scans the whole rebin set */
        for (size_t r = 0; r < rs->n; r++)
            if (s->rebin_dest[r] == b)
                bin_push(bin, rs->pos[2 * r], rs->pos[2 * r + 1], rs->vel[2 * r],
                         rs->vel[2 * r + 1], rs->visc[r], rs->dead[r]);
    }
}

static void rebin(fso_solver *s) /* markerparticlesystem.cpp:47-58 */
{
    par_for(s->pool, s->nbins, rebin_range, s);
    s->rebin.n = 0;
}

/* ------------------------------------------------------------------------ */
/* pressure operator and IPP coefficients (flipsolver2d.cpp:797-945)         */
/* ------------------------------------------------------------------------ */
static int nonsolid_count_lin(const fso_solver *s, long lin) /* materialgrid.cpp:130-140 */
{
    long i = lin / s->nj;
    long j = lin - i * s->nj;
    return !is_solid(s, i - 1, j) + !is_solid(s, i + 1, j) + !is_solid(s, i, j - 1) +
           !is_solid(s, i, j + 1);
}

static void build_matrix(fso_solver *s)
{
    const double scale = s->step_dt / (s->density * s->dx * s->dx);
    const long N = (long)s->ncell;
    s->mscale = scale;
    s->have_units = 0;
    for (long i = 0; i < s->ni; i++)
        for (long j = 0; j < s->nj; j++) {
            long lin = i * s->nj + j;
            s->unit[lin] = 0;
            s->mask[lin] = 0;
            s->ucount[lin] = 0;
            if (!is_fluid(s, i, j)) continue;
            s->unit[lin] = 1;
            s->have_units = 1;
            uint8_t m = 0, c = 0;
            long nx = lin - s->nj, px = lin + s->nj, ny = lin - 1, py = lin + 1;
            if (is_fluid(s, i - 1, j)) {
                c++;
                if (nx >= 0 && nx < N) m |= 1;
            } else if (is_empty(s, i - 1, j)) c++;
            if (is_fluid(s, i + 1, j)) {
                c++;
                if (px >= 0 && px < N) m |= 2;
            } else if (is_empty(s, i + 1, j)) c++;
            if (is_fluid(s, i, j - 1)) {
                c++;
                if (ny >= 0 && ny < N) m |= 4;
            } else if (is_empty(s, i, j - 1)) c++;
            if (is_fluid(s, i, j + 1)) {
                c++;
                if (py >= 0 && py < N) m |= 8;
            } else if (is_empty(s, i, j + 1)) c++;
            s->mask[lin] = m;
            s->ucount[lin] = c;
            double *q = &s->ipp[4 * lin];
            q[0] = 1.0 / (nonsolid_count_lin(s, lin - s->nj) * scale); /* iNeg */
            q[1] = 1.0 / (nonsolid_count_lin(s, lin + s->nj) * scale); /* iPos */
            q[2] = 1.0 / (nonsolid_count_lin(s, lin - 1) * scale);     /* jNeg */
            q[3] = 1.0 / (nonsolid_count_lin(s, lin + 1) * scale);     /* jPos */
        }
}

static inline double vat(const double *x, long k, long N) { return (k >= 0 && k < N) ? x[k] : 0.0; }

typedef struct mv_ctx {
    fso_solver *s;
    const double *in;
    double *out;
} mv_ctx;

/* IndexedPressureParameterUnit::multiply (pressuredata.h:132-146); rows that
 * are not units copy the input (pressuredata.h:215-238). */
static void amul_range(void *ctx, size_t a, size_t b)
{
    mv_ctx *c = (mv_ctx *)ctx;
    fso_solver *s = c->s;
    const long N = (long)s->ncell, NJ = s->nj;
    const double scale = s->mscale;
    for (size_t k = a; k < b; k++) {
        long idx = (long)k;
        if (!s->unit[idx]) {
            c->out[idx] = c->in[idx];
            continue;
        }
        uint8_t m = s->mask[idx];
        c->out[idx] = (scale * s->ucount[idx]) * vat(c->in, idx, N) +
                      (-scale * (m & 1)) * vat(c->in, idx - NJ, N) +
                      (-scale * ((m & 2) >> 1)) * vat(c->in, idx + NJ, N) +
                      (-scale * ((m & 4) >> 2)) * vat(c->in, idx - 1, N) +
                      (-scale * ((m & 8) >> 3)) * vat(c->in, idx + 1, N);
    }
}

/* IndexedIPPCoefficientUnit::multiply (PressureIPPCoeficients.h:23-40) */
static void pmul_range(void *ctx, size_t a, size_t b)
{
    mv_ctx *c = (mv_ctx *)ctx;
    fso_solver *s = c->s;
    const long N = (long)s->ncell, NJ = s->nj;
    for (size_t k = a; k < b; k++) {
        long idx = (long)k;
        if (!s->unit[idx]) {
            c->out[idx] = c->in[idx];
            continue;
        }
        const double *q = &s->ipp[4 * idx];
        const double iNeg = q[0], iPos = q[1], jNeg = q[2], jPos = q[3];
        const double diag = 1.0 + iNeg * iNeg + jNeg * jNeg;
        c->out[idx] = diag * vat(c->in, idx, N) + jNeg * vat(c->in, idx - 1, N) +
                      jPos * vat(c->in, idx + 1, N) + iNeg * vat(c->in, idx - NJ, N) +
                      iPos * vat(c->in, idx + NJ, N);
    }
}

static void apply_a(fso_solver *s, const double *in, double *out)
{
    mv_ctx c = {s, in, out};
    if (!s->have_units) {
        memcpy(out, in, s->ncell * sizeof(double));
        return;
    }
    par_for(s->pool, s->ncell, amul_range, &c);
}

static void apply_ipp(fso_solver *s, const double *in, double *out)
{
    mv_ctx c = {s, in, out};
    if (!s->have_units) {
        memcpy(out, in, s->ncell * sizeof(double));
        return;
    }
    par_for(s->pool, s->ncell, pmul_range, &c);
}

/* ---- VOps (vmath.cpp) --------------------------------------------------- */
typedef struct red_ctx {
    const double *a, *b;
    const range *rg;
    double *partial;
} red_ctx;

static void dot_chunks(void *ctx, size_t c0, size_t c1) /* VOps::dotThread, :8-17 */
{
    red_ctx *c = (red_ctx *)ctx;
    for (size_t k = c0; k < c1; k++) {
        double r = 0.0;
        for (size_t i = c->rg[k].start; i < c->rg[k].end; i++) r += c->a[i] * c->b[i];
        c->partial[k] = r;
    }
}

static double vdot(fso_solver *s, const double *a, const double *b) /* VOps::dot, :25-45 */
{
    range rg[1024];
    double partial[1024];
    size_t nr = split_range(s->ncell, (size_t)s->ref_threads, rg);
    red_ctx c = {a, b, rg, partial};
    par_for(s->pool, nr, dot_chunks, &c);
    double result = 0;
    for (size_t k = 0; k < nr; k++) result += partial[k];
    return result;
}

static void maxabs_chunks(void *ctx, size_t c0, size_t c1) /* VOps::maxAbsThread, :100-111 */
{
    red_ctx *c = (red_ctx *)ctx;
    for (size_t k = c0; k < c1; k++) {
        /* the comparison is against the output slot (still 0), so the chunk
         * reports |last non-zero element| or DBL_MIN */
        double m = DBL_MIN;
        for (size_t i = c->rg[k].start; i < c->rg[k].end; i++)
            if (fabs(c->a[i]) > 0.0) m = fabs(c->a[i]);
        c->partial[k] = m;
    }
}

static double vmaxabs(fso_solver *s, const double *a) /* VOps::maxAbs, :113-136 */
{
    range rg[1024];
    double partial[1024];
    size_t nr = split_range(s->ncell, (size_t)s->ref_threads, rg);
    red_ctx c = {a, NULL, rg, partial};
    par_for(s->pool, nr, maxabs_chunks, &c);
    double mx = 0;
    for (size_t k = 0; k < nr; k++)
        if (partial[k] > mx) mx = fabs(partial[k]);
    return mx;
}

typedef struct axpy_ctx {
    double *out;
    const double *a, *b;
    double alpha;
    int sub;
} axpy_ctx;

static void axpy_range(void *ctx, size_t a, size_t b) /* VOps::addMul/subMul, :60-98 */
{
    axpy_ctx *c = (axpy_ctx *)ctx;
    if (c->sub)
        for (size_t i = a; i < b; i++) c->out[i] = c->a[i] - c->b[i] * c->alpha;
    else
        for (size_t i = a; i < b; i++) c->out[i] = c->a[i] + c->b[i] * c->alpha;
}

static void vaxpy(fso_solver *s, double *out, const double *a, const double *b, double alpha, int sub)
{
    axpy_ctx c = {out, a, b, alpha, sub};
    par_for(s->pool, s->ncell, axpy_range, &c);
}

/* LinearSolver::solve (linearsolver.cpp:25-73) */
static int linear_solve(fso_solver *s, double *result, const double *vec, int iterLimit, double tol)
{
    const size_t n = s->ncell;
    memset(result, 0, n * sizeof(double));
    int zero = 1; /* VOps::isZero(vec, 1e-15), vmath.cpp:47-58 */
    for (size_t i = 0; i < n; i++)
        if (fabs(vec[i]) > 1.0e-15) {
            zero = 0;
            break;
        }
    if (zero) return 0;
    double *residual = s->w_r, *aux = s->w_aux, *search = s->w_s;
    memcpy(residual, vec, n * sizeof(double));
    memcpy(aux, residual, n * sizeof(double));
    memcpy(search, aux, n * sizeof(double));
    double sigma = vdot(s, aux, residual);
    for (int i = 0; i < iterLimit; i++) {
        apply_a(s, search, aux);
        double alpha = sigma / (vdot(s, aux, search) + 1e-8);
        vaxpy(s, result, result, search, alpha, 0);
        vaxpy(s, residual, residual, aux, alpha, 1);
        double err = vmaxabs(s, residual);
        if (err <= tol) return i;
        apply_ipp(s, residual, aux);
        double newSigma = vdot(s, aux, residual);
        double beta = newSigma / (sigma);
        vaxpy(s, search, aux, search, beta, 0);
        sigma = newSigma;
    }
    return iterLimit;
}

static double project_tolerance(const fso_solver *s) /* flipsolver2d.cpp:73; nbflipsolver.cpp:22 */
{
    if (s->nb) return 1e-6;
    return s->p.viscosityEnabled ? 1e-6 : 1e-2;
}

/* ------------------------------------------------------------------------ */
/* density correction (flipsolver2d.cpp:164-303, 993-1011)                   */
/* ------------------------------------------------------------------------ */
static void density_grid_range(void *ctx, size_t a, size_t b) /* :201-249 */
{
    fso_solver *s = (fso_solver *)ctx;
    const float cellVolume = (float)(s->dx * s->dx * s->dx);
    const float particleMass = (float)((s->density * cellVolume) / ((float)s->p.particlesPerCell));
    for (size_t idx = a; idx < b; idx++) {
        long ci = (long)idx / s->nj, cj = (long)idx - ci * s->nj;
        long bl[9];
        bins_for_cell(s, ci, cj, bl);
        float d = 0.f;
        for (int q = 0; q < 9; q++) {
            if (bl[q] == -1) continue;
            const pbin *bin = &s->bins[bl[q]];
            for (size_t k = 0; k < bin->n; k++) {
                if (bin->dead[k]) continue;
                float w = sm_bilinear_hat(bin->pos[2 * k] - (float)ci - 0.5f,
                                          bin->pos[2 * k + 1] - (float)cj - 0.5f);
                if (fabsf(w) > 1e-6f) d += w * particleMass;
            }
        }
        d /= cellVolume;
        if (is_fluid(s, ci, cj) && (is_empty(s, ci + 1, cj) || is_empty(s, ci - 1, cj) ||
                                    is_empty(s, ci, cj + 1) || is_empty(s, ci, cj - 1)))
            d = clampf(d, (float)s->density, FLT_MAX);
        s->dens[idx] = d;
    }
}

static void update_density_grid(fso_solver *s) /* :188-199 */
{
    par_for(s->pool, s->ncell, density_grid_range, s);
}

static void adjust_range(void *ctx, size_t b0, size_t b1) /* :261-303 */
{
    fso_solver *s = (fso_solver *)ctx;
    const float scale = (float)((s->step_dt * s->step_dt) / (s->density * s->dx * s->dx));
    const double *p = s->dens_p;
    for (size_t b = b0; b < b1; b++) {
        pbin *bin = &s->bins[b];
        for (size_t k = 0; k < bin->n; k++) {
            if (bin->dead[k]) continue;
            float x = bin->pos[2 * k], y = bin->pos[2 * k + 1];
            long iCorr = clampi((int)(x - 0.5f), 0, s->ni);
            long jCorr = clampi((int)(y - 0.5f), 0, s->nj);
            long i = clampi((int)x, 0, s->ni);
            long j = clampi((int)y, 0, s->nj);
            /* an index outside the grid (linearIndex == -1) would read before
             * the vector in the reference; it is taken as 0 here */
            long l0 = lin_index(s, iCorr, j), l1 = lin_index(s, i, jCorr);
            long l2 = lin_index(s, iCorr + 1, j), l3 = lin_index(s, i, jCorr + 1);
            float pCurrentI = l0 < 0 ? 0.f : (float)p[l0];
            float pCurrentJ = l1 < 0 ? 0.f : (float)p[l1];
            float pI = l2 < 0 ? 0.f : (float)p[l2];
            float pJ = l3 < 0 ? 0.f : (float)p[l3];
            if (is_solid(s, iCorr + 1, j) || is_solid(s, iCorr, j)) pI = pCurrentI;
            if (is_solid(s, i, jCorr + 1) || is_solid(s, i, jCorr)) pJ = pCurrentJ;
            float gu = pI - pCurrentI, gv = pJ - pCurrentJ;
            bin->pos[2 * k] = x + gu * scale;
            bin->pos[2 * k + 1] = y + gv * scale;
        }
    }
}

static void density_correction(fso_solver *s) /* :164-186 */
{
    update_density_grid(s);
    s->dens_sized = 1;
    const double scale = 1.0 / s->step_dt;
    for (long i = 0; i < s->ni; i++)
        for (long j = 0; j < s->nj; j++) {
            long l = i * s->nj + j;
            s->dens_rhs[l] = is_fluid(s, i, j)
                                 ? scale * (1.0 - clampd(s->dens[l] / s->density, 0.5, 1.5))
                                 : 0.0;
        }
    int iters = linear_solve(s, s->dens_p, s->dens_rhs, s->p.pcgIterLimit, project_tolerance(s));
    if (iters > s->density_iters) s->density_iters = iters;
    if (iters >= s->p.pcgIterLimit) return;
    par_for(s->pool, s->nbins, adjust_range, s);
}

/* ------------------------------------------------------------------------ */
/* particle -> grid (flipsolver2d.cpp:1313-1431)                             */
/* ------------------------------------------------------------------------ */
static void p2g_range(void *ctx, size_t a, size_t b) /* :1329-1377 */
{
    fso_solver *s = (fso_solver *)ctx;
    const float threshold = 1e-9f;
    for (size_t idx = a; idx < b; idx++) {
        long ci = (long)idx / s->nj, cj = (long)idx - ci * s->nj;
        long bl[9];
        bins_for_cell(s, ci, cj, bl);
        float uW = 1e-10f, vW = 1e-10f, uVel = 0.0f, vVel = 0.0f;
        int uValid = 0, vValid = 0;
        for (int q = 0; q < 9; q++) {
            if (bl[q] < 0) continue;
            const pbin *bin = &s->bins[bl[q]];
            for (size_t k = 0; k < bin->n; k++) {
                float x = bin->pos[2 * k], y = bin->pos[2 * k + 1];
                float wU = sm_qbspline(x - (float)ci, y - ((float)cj + 0.5f));
                float wV = sm_qbspline(x - ((float)ci + 0.5f), y - (float)cj);
                if (wU > threshold && wV > threshold) {
                    uW += wU;
                    uVel += wU * bin->vel[2 * k];
                    uValid = 1;
                    vW += wV;
                    vVel += wV * bin->vel[2 * k + 1];
                    vValid = 1;
                }
            }
        }
        s->u[ci * s->nj + cj] = uVel / uW;
        s->uvalid[ci * s->nj + cj] = (uint8_t)uValid;
        s->v[ci * (s->nj + 1) + cj] = vVel / vW;
        s->vvalid[ci * (s->nj + 1) + cj] = (uint8_t)vValid;
    }
}

/* FlipSolver::centeredParamsToGridThread (:1394-1431); NB-FLIP's override
 * (nbflipsolver.cpp:463-504) accumulates the same sums in the same order
 * into the cleared grid and a weight grid starting at 1e-10, keeps weights
 * with |w| > 1e-6 and divides only where a weight was kept, which is 0 / w
 * otherwise: the result differs only in the threshold. */
static void centered_range(void *ctx, size_t a, size_t b)
{
    fso_solver *s = (fso_solver *)ctx;
    const float threshold = s->nb ? 1e-6f : 1e-9f;
    for (size_t idx = a; idx < b; idx++) {
        long ci = (long)idx / s->nj, cj = (long)idx - ci * s->nj;
        long bl[9];
        bins_for_cell(s, ci, cj, bl);
        float wT = (float)1e-10, val = 0.0f;
        int valid = 0;
        for (int q = 0; q < 9; q++) {
            if (bl[q] < 0) continue;
            const pbin *bin = &s->bins[bl[q]];
            for (size_t k = 0; k < bin->n; k++) {
                float w = sm_qbspline(bin->pos[2 * k] - (float)ci, bin->pos[2 * k + 1] - (float)cj);
                if ((s->nb ? fabsf(w) : w) > threshold) {
                    wT += w;
                    val += w * bin->visc[k];
                    valid = 1;
                }
            }
        }
        s->visc_grid[idx] = val / wT;
        s->known[idx] = (uint8_t)valid;
    }
}

static void particle_to_grid(fso_solver *s) /* :1213-1220, 1313-1327, 1379-1392 */
{
    memset(s->u, 0, s->nu * sizeof(float));
    memset(s->v, 0, s->nv * sizeof(float));
    memset(s->uvalid, 0, s->nu);
    memset(s->vvalid, 0, s->nv);
    par_for(s->pool, s->ncell, p2g_range, s);
    if (s->p.parameterHandlingMethod != 2) {
        memset(s->visc_grid, 0, s->ncell * sizeof(float));
        memset(s->divc, 0, s->ncell * sizeof(float));
        memset(s->known, 0, s->ncell);
        par_for(s->pool, s->ncell, centered_range, s);
    }
}

/* ------------------------------------------------------------------------ */
/* fluid SDF and materials (flipsolver2d.cpp:1243-1311, 1053-1075)           */
/* ------------------------------------------------------------------------ */
static void sdf_range(void *ctx, size_t a, size_t b)
{
    fso_solver *s = (fso_solver *)ctx;
    const float r = s->p.particleScale;
    for (size_t idx = a; idx < b; idx++) {
        long ci = (long)idx / s->nj, cj = (long)idx - ci * s->nj;
        long bl[9];
        bins_for_cell(s, ci, cj, bl);
        float d2 = FLT_MAX;
        float cx = (float)ci + 0.5f, cy = (float)cj + 0.5f;
        for (int q = 0; q < 9; q++) {
            if (bl[q] < 0) continue;
            const pbin *bin = &s->bins[bl[q]];
            for (size_t k = 0; k < bin->n; k++) {
                float dx = bin->pos[2 * k] - cx, dy = bin->pos[2 * k + 1] - cy;
                float nd = dx * dx + dy * dy;
                if (nd < d2) d2 = nd;
            }
        }
        s->fluid_sdf[idx] = sqrtf(d2) - r;
    }
}

static void update_sdf(fso_solver *s) { par_for(s->pool, s->ncell, sdf_range, s); }

static void update_materials(fso_solver *s)
{
    for (long i = 0; i < s->ni; i++)
        for (long j = 0; j < s->nj; j++) {
            long l = i * s->nj + j;
            if (s->fluid_sdf[l] < 0.f) {
                if (is_empty(s, i, j)) s->material[l] = M_FLUID;
            } else {
                if (is_strict_fluid(s, i, j)) s->material[l] = M_EMPTY;
            }
        }
}

/* ------------------------------------------------------------------------ */
/* breadth-first extrapolations                                              */
/* ------------------------------------------------------------------------ */
/* LinearIndexable2d::getNeighborhood (linearindexable2d.h:65-81) */
static void neighborhood(long si, long sj, long i, long j, long out[8])
{
    int k = 0;
    for (long io = -1; io <= 1; io++)
        for (long jo = -1; jo <= 1; jo++) {
            if (io == 0 && jo == 0) continue;
            long a = i + io, b = j + jo;
            out[k++] = (a < 0 || a >= si || b < 0 || b >= sj) ? -1 : a * sj + b;
        }
}

/* shared FIFO BFS of extrapolateLevelsetInside (flipsolver2d.cpp:1433-1494),
 * extrapolateLevelsetOutside (:1496-1558) and simmath::breadthFirstExtrapolate
 * (mathfuncs.cpp:152-215).
 * mode 0: level set inside (seed: value > 0, no depth limit, value - 1);
 * mode 1: velocity (seed: flag set, depth limit `radius`, sets flags);
 * mode 2: level set outside (seed: value < si * sj, no depth limit, value + 1). */
static void bfs_extrapolate(float *grid, uint8_t *flag, long si, long sj, int mode, int radius)
{
    size_t n = (size_t)si * sj;
    int *markers = (int *)malloc(n * sizeof(int));
    size_t *queue = (size_t *)malloc(n * sizeof(size_t));
    size_t head = 0, tail = 0;
    const float maxSdf = (float)n; /* :1500 */
    for (size_t k = 0; k < n; k++) {
        int seed = mode == 0 ? (grid[k] > 0.f) : mode == 2 ? (grid[k] < maxSdf) : (flag[k] != 0);
        markers[k] = seed ? 0 : INT_MAX;
    }
    long nb[8];
    for (long i = 0; i < si; i++)
        for (long j = 0; j < sj; j++) {
            if (markers[i * sj + j] == 0) continue;
            neighborhood(si, sj, i, j, nb);
            for (int q = 0; q < 8; q++) {
                if (nb[q] == -1) continue;
                if (markers[nb[q]] == 0) {
                    markers[i * sj + j] = 1;
                    queue[tail++] = (size_t)(i * sj + j);
                    break;
                }
            }
        }
    while (head < tail) {
        size_t index = queue[head];
        long i = (long)index / sj, j = (long)index - ((long)index / sj) * sj;
        neighborhood(si, sj, i, j, nb);
        double avg = 0;
        int count = 0;
        for (int q = 0; q < 8; q++) {
            if (nb[q] == -1) continue;
            if (markers[nb[q]] < markers[index]) {
                avg += grid[nb[q]];
                count++;
            }
            int lim_ok = mode != 1 ? (markers[index] <= 1e6) : (markers[index] <= radius);
            if (markers[nb[q]] == INT_MAX && lim_ok) {
                markers[nb[q]] = markers[index] + 1;
                queue[tail++] = (size_t)nb[q];
            }
        }
        if (mode == 0) {
            grid[index] = (float)(avg / count - 1.f);
        } else if (mode == 2) {
            grid[index] = (float)(avg / count + 1.f);
        } else {
            grid[index] = (float)(avg / count);
            flag[index] = 1;
        }
        head++;
    }
    free(markers);
    free(queue);
}

static void extrapolate_velocity(fso_solver *s) /* staggeredvelocitygrid.cpp:146-156 */
{
    bfs_extrapolate(s->u, s->uvalid, s->ni + 1, s->nj, 1, 10);
    bfs_extrapolate(s->v, s->vvalid, s->ni, s->nj + 1, 1, 10);
}

/* ------------------------------------------------------------------------ */
/* grid forces, projection, friction                                         */
/* ------------------------------------------------------------------------ */
static void body_forces(fso_solver *s) /* flipsolver2d.cpp:1222-1241 */
{
    const float factor = (float)(s->step_dt / s->dx);
    for (long i = 0; i < s->ni + 1; i++)
        for (long j = 0; j < s->nj + 1; j++) {
            if (i < s->ni + 1 && j < s->nj)
                s->u[i * s->nj + j] += factor * s->p.globalAccelerationI;
            if (i < s->ni && j < s->nj + 1)
                s->v[i * (s->nj + 1) + j] += factor * s->p.globalAccelerationJ;
        }
}

static void pressure_rhs(fso_solver *s, double *rhs) /* :962-991, divergenceAt :759-764 */
{
    const double scale = 1.f / s->dx;
    const long NJ = s->nj, NV = s->nj + 1;
    for (long i = 0; i < s->ni; i++)
        for (long j = 0; j < s->nj; j++) {
            long l = i * NJ + j;
            if (!is_fluid(s, i, j)) {
                rhs[l] = 0.0;
                continue;
            }
            float u0 = s->u[i * NJ + j], u1 = s->u[(i + 1) * NJ + j];
            float v0 = s->v[i * NV + j], v1 = s->v[i * NV + j + 1];
            double div = (double)(u1 - u0 + v1 - v0 + s->divc[l]);
            double val = -scale * div;
            val -= (double)is_solid(s, i - 1, j) * scale * (double)(u0 - 0);
            val += (double)is_solid(s, i + 1, j) * scale * (double)(u1 - 0);
            val -= (double)is_solid(s, i, j - 1) * scale * (double)(v0 - 0);
            val += (double)is_solid(s, i, j + 1) * scale * (double)(v1 - 0);
            rhs[l] = val;
        }
}

static void apply_pressure(fso_solver *s, const double *p) /* :1106-1193 */
{
    const double scale = s->step_dt / (s->density * s->dx);
    const long NJ = s->nj, NV = s->nj + 1;
    for (long i = 0; i < s->ni; i++)
        for (long j = 0; j < s->nj; j++) {
            long l = i * NJ + j;
            double pc = p[l];
            /* U face (i, j) between cells (i-1, j) and (i, j) */
            long lim1 = lin_index(s, i - 1, j);
            double pim1 = lim1 == -1 ? 0.0 : p[lim1];
            if (is_fluid(s, i - 1, j) || is_fluid(s, i, j)) {
                if (is_solid(s, i - 1, j) || is_solid(s, i, j)) s->u[i * NJ + j] = 0.f;
                else s->u[i * NJ + j] = (float)(s->u[i * NJ + j] - scale * (pc - pim1));
            } else {
                s->uvalid[i * NJ + j] = 0;
            }
            /* V face (i, j) between cells (i, j-1) and (i, j) */
            long ljm1 = lin_index(s, i, j - 1);
            double pjm1 = ljm1 == -1 ? 0.0 : p[ljm1];
            if (is_fluid(s, i, j - 1) || is_fluid(s, i, j)) {
                if (is_solid(s, i, j - 1) || is_solid(s, i, j)) s->v[i * NV + j] = 0.f;
                else s->v[i * NV + j] = (float)(s->v[i * NV + j] - scale * (pc - pjm1));
            } else {
                s->vvalid[i * NV + j] = 0;
            }
        }
}

static void project(fso_solver *s) /* :93-126 */
{
    pressure_rhs(s, s->pres_rhs);
    int iters = linear_solve(s, s->pres, s->pres_rhs, s->p.pcgIterLimit, project_tolerance(s));
    if (iters > s->pressure_iters) s->pressure_iters = iters;
    apply_pressure(s, s->pres);
}

/* ---- viscosity (viscositymodel.cpp) ---------------------------------- */
/* The reference assembles its viscosity systems with Eigen::SparseMatrix::
 * coeffRef and solves them with Eigen::ConjugateGradient<..., Eigen::Upper>
 * and Eigen's default diagonal preconditioner (viscositymodel.h:21).  Eigen
 * (3.4.0, a pinned dependency) is absent here: the reference build compiles
 * against oracle/refshim/Eigen, whose matrix stores entries per row in column
 * order and whose conjugate gradient restates Eigen's published algorithm.
 * This is the same assembly and the same solver, operation for operation. */
typedef struct vrow {
    long *col;
    double *val;
    int n, cap;
} vrow;

/* coeffRef(r, c): the entry, created as 0 in column order when absent */
static double *vrow_ref(vrow *row, long c)
{
    int k = 0;
    while (k < row->n && row->col[k] < c) k++;
    if (k < row->n && row->col[k] == c) return &row->val[k];
    if (row->n == row->cap) {
        row->cap = row->cap ? 2 * row->cap : 8;
        row->col = (long *)realloc(row->col, (size_t)row->cap * sizeof(long));
        row->val = (double *)realloc(row->val, (size_t)row->cap * sizeof(double));
    }
    memmove(row->col + k + 1, row->col + k, (size_t)(row->n - k) * sizeof(long));
    memmove(row->val + k + 1, row->val + k, (size_t)(row->n - k) * sizeof(double));
    row->col[k] = c;
    row->val[k] = 0.0;
    row->n++;
    return &row->val[k];
}

static void vrows_free(vrow *rows, long n)
{
    for (long r = 0; r < n; r++) {
        free(rows[r].col);
        free(rows[r].val);
    }
    free(rows);
}

/* ConjugateGradient<SparseMatrix<double>, Upper>::compute then solve: the
 * matrix acts as the self-adjoint matrix of its upper triangle; Jacobi
 * preconditioner (1 / diagonal, 1 where the diagonal is zero or absent);
 * x0 = 0; stop when ||r||^2 < max(tol^2 ||b||^2, DBL_MIN) or after 2n
 * iterations.  Returns the iteration count; *ok is Eigen's Success test
 * sqrt(||r||^2 / ||b||^2) <= tol. */
static double visc_dot(const double *a, const double *b, long n)
{
    double s = 0.0;
    for (long k = 0; k < n; k++) s += a[k] * b[k];
    return s;
}

static void vapply(const vrow *rows, long n, const double *x, double *y)
{
    for (long k = 0; k < n; k++) y[k] = 0.0;
    for (long r = 0; r < n; r++) {
        double acc = 0.0;
        for (int e = 0; e < rows[r].n; e++) {
            const long c = rows[r].col[e];
            if (c < r) continue; /* the lower triangle is not read */
            acc += rows[r].val[e] * x[c];
            if (c != r) y[c] += rows[r].val[e] * x[r];
        }
        y[r] += acc;
    }
}

static long vcg_solve(const vrow *rows, long n, double tol, const double *b, double *x, int *ok)
{
    double *invdiag = (double *)malloc((size_t)n * sizeof(double));
    double *r = (double *)malloc((size_t)n * sizeof(double)), *p = (double *)malloc((size_t)n * sizeof(double));
    double *z = (double *)malloc((size_t)n * sizeof(double)), *t = (double *)malloc((size_t)n * sizeof(double));
    for (long k = 0; k < n; k++) {
        invdiag[k] = 1.0;
        for (int e = 0; e < rows[k].n; e++)
            if (rows[k].col[e] == k && rows[k].val[e] != 0.0) invdiag[k] = 1.0 / rows[k].val[e];
        x[k] = 0.0;
        r[k] = b[k];
    }
    long iters = 0;
    double err = 0.0;
    const double rhsNorm2 = visc_dot(b, b, n);
    if (rhsNorm2 == 0.0) {
        *ok = 1;
        goto done;
    }
    {
        const double threshold = fmax(tol * tol * rhsNorm2, DBL_MIN);
        double residualNorm2 = visc_dot(r, r, n);
        if (residualNorm2 < threshold) {
            err = sqrt(residualNorm2 / rhsNorm2);
            *ok = err <= tol;
            goto done;
        }
        for (long k = 0; k < n; k++) p[k] = invdiag[k] * r[k];
        double absNew = visc_dot(r, p, n);
        long i = 0;
        while (i < 2 * n) {
            vapply(rows, n, p, t);
            const double alpha = absNew / visc_dot(p, t, n);
            for (long k = 0; k < n; k++) x[k] += alpha * p[k];
            for (long k = 0; k < n; k++) r[k] -= alpha * t[k];
            residualNorm2 = visc_dot(r, r, n);
            if (residualNorm2 < threshold) break;
            for (long k = 0; k < n; k++) z[k] = invdiag[k] * r[k];
            const double absOld = absNew;
            absNew = visc_dot(r, z, n);
            const double beta = absNew / absOld;
            for (long k = 0; k < n; k++) p[k] = z[k] + beta * p[k];
            i++;
        }
        err = sqrt(residualNorm2 / rhsNorm2);
        iters = i;
        *ok = err <= tol;
    }
done:
    free(invdiag);
    free(r);
    free(p);
    free(z);
    free(t);
    return iters;
}

/* Grid2d::at of the viscosity grid: an unchecked read in the reference; the
 * out-of-grid reads it makes are never stored, so any value serves */
static inline float visc_at(const fso_solver *s, long i, long j)
{
    i = i < 0 ? 0 : (i >= s->ni ? s->ni - 1 : i);
    j = j < 0 ? 0 : (j >= s->nj ? s->nj - 1 : j);
    return s->visc_grid[i * s->nj + j];
}

/* LightViscosityModel::apply (viscositymodel.cpp:4-63) with getMatrix
 * (:65-135), fillRhs (:137-148) and applyResult (:150-161): one system on
 * the NI x NJ cells, solved for U (rows 0..NI-1 of the U grid) and then for V
 * (columns 0..NJ-1 of the V grid).  The tolerance is 1e-4.  Returns the V
 * solve's iteration count, or -1 when a solve fails (the reference returns
 * without applying that solve). */
static int viscosity_light(fso_solver *s)
{
    const long NI = s->ni, NJ = s->nj, N = NI * NJ;
    const float dt = s->step_dt;
    const float density = (float)s->p.fluidDensity;
    const double scale = dt;
    vrow *rows = (vrow *)calloc((size_t)N, sizeof(vrow));
    for (long i = 0; i < NI; i++) {
        for (long j = 0; j < NJ; j++) {
            const long idx = i * NJ + j;
            double diag = 4.0, ip1 = 1.0, jp1 = 1.0, im1 = 1.0, jm1 = 1.0;
            if (is_solid(s, i, j)) {
                *vrow_ref(&rows[idx], idx) = 1.0;
                continue;
            }
            ip1 *= (double)(is_solid(s, i + 1, j) ? visc_at(s, i, j) : visc_at(s, i + 1, j)) * scale;
            jp1 *= (double)(is_solid(s, i, j + 1) ? visc_at(s, i, j) : visc_at(s, i, j + 1)) * scale;
            im1 *= (double)(is_solid(s, i - 1, j) ? visc_at(s, i, j) : visc_at(s, i - 1, j)) * scale;
            jm1 *= (double)(is_solid(s, i, j - 1) ? visc_at(s, i, j) : visc_at(s, i, j - 1)) * scale;
            diag *= (double)visc_at(s, i, j) * scale;
            diag += 1.;
            *vrow_ref(&rows[idx], idx) = diag;
            if (i + 1 < NI) {
                *vrow_ref(&rows[idx], idx + NJ) = ip1;
                *vrow_ref(&rows[idx + NJ], idx) = ip1;
            }
            if (j + 1 < NJ) {
                *vrow_ref(&rows[idx], idx + 1) = jp1;
                *vrow_ref(&rows[idx + 1], idx) = jp1;
            }
            if (i - 1 >= 0) {
                *vrow_ref(&rows[idx], idx - NJ) = im1;
                *vrow_ref(&rows[idx - NJ], idx) = im1;
            }
            if (j - 1 >= 0) {
                *vrow_ref(&rows[idx], idx - 1) = jm1;
                *vrow_ref(&rows[idx - 1], idx) = jm1;
            }
        }
    }
    double *b = (double *)calloc((size_t)N, sizeof(double)), *x = (double *)calloc((size_t)N, sizeof(double));
    int ok = 0;
    long iters = -1;
    for (long k = 0; k < N; k++) b[k] = (double)(density * s->u[(k / NJ) * NJ + k % NJ]);
    vcg_solve(rows, N, 1e-4, b, x, &ok);
    if (ok) {
        for (long k = 0; k < N; k++) s->u[(k / NJ) * NJ + k % NJ] = (float)(x[k] / (double)density);
        for (long k = 0; k < N; k++) b[k] = (double)(density * s->v[(k / NJ) * (NJ + 1) + k % NJ]);
        iters = vcg_solve(rows, N, 1e-4, b, x, &ok);
        if (ok) {
            for (long k = 0; k < N; k++) s->v[(k / NJ) * (NJ + 1) + k % NJ] = (float)(x[k] / (double)density);
        } else {
            iters = -1;
        }
    }
    free(b);
    free(x);
    vrows_free(rows, N);
    return (int)iters;
}

/* HeavyViscosityModel::apply (viscositymodel.cpp:164-200) with getMatrix
 * (:202-402), getRhs (:404-434) and applyResult (:436-469): one coupled
 * system over every U face then every V face.  Each entry accumulates
 * (coeffRef +=) the terms of its own row in the reference's order; float
 * products, double sums.  The viscosity at a face corner is
 * Grid2d::interpolateAt with the grid's (0.5, 0.5) offset.  The column
 * uIpOneJmOneLinearIdx is a V-grid linear index used in the U range, as in
 * the reference (:383, :395).  Tolerance 1e-4; returns the iteration count or
 * -1 when the solve fails (nothing applied). */
static inline long u_index(const fso_solver *s, long i, long j) /* U: (NI+1) x NJ */
{
    return (i < 0 || i > s->ni || j < 0 || j >= s->nj) ? -1 : i * s->nj + j;
}
static inline long v_index(const fso_solver *s, long i, long j) /* V: NI x (NJ+1) */
{
    return (i < 0 || i >= s->ni || j < 0 || j > s->nj) ? -1 : i * (s->nj + 1) + j;
}
static inline float visc_get(const fso_solver *s, long i, long j) /* getAt, OOB_EXTEND */
{
    return visc_at(s, i, j);
}
static inline float visc_interp(const fso_solver *s, float i, float j)
{
    return grid_lerp(s->visc_grid, (int)s->ni, (int)s->nj, 0.5f, 0.5f, i, j);
}

static int viscosity_heavy(fso_solver *s)
{
    const long NI = s->ni, NJ = s->nj;
    const long NU = (NI + 1) * NJ, NV = NI * (NJ + 1), N = NU + NV;
    const float dt = s->step_dt, dx = (float)s->p.dx;
    const float density = (float)s->p.fluidDensity;
    const float scaleTwoDt = 2 * dt / (dx * dx);
    const float scaleTwoDx = dt / (2 * dx * dx);
    const long vb = NU;
    vrow *rows = (vrow *)calloc((size_t)N, sizeof(vrow));
#define A(r, c) (*vrow_ref(&rows[(r)], (c)))
    for (long i = 0; i < NI + 1; i++) {
        for (long j = 0; j < NJ + 1; j++) {
            const long idxU = u_index(s, i, j), idxV = v_index(s, i, j);
            const float fi = (float)i, fj = (float)j;
            if (idxU != -1) {
                A(idxU, idxU) += density;
                const long uim1 = u_index(s, i - 1, j);
                if (uim1 != -1) {
                    A(idxU, uim1) += -scaleTwoDt * visc_get(s, i - 1, j);
                    A(idxU, idxU) += scaleTwoDt * visc_get(s, i - 1, j);
                }
                const long uip1 = u_index(s, i + 1, j);
                if (uip1 != -1) {
                    A(idxU, uip1) += -scaleTwoDt * visc_get(s, i, j);
                    A(idxU, idxU) += scaleTwoDt * visc_get(s, i, j);
                }
                const long ujm1 = u_index(s, i, j - 1), vim1 = v_index(s, i - 1, j);
                if (ujm1 != -1 && idxV != -1 && vim1 != -1) {
                    const float lv = visc_interp(s, fi - 0.5f, fj - 0.5f);
                    A(idxU, ujm1) += -scaleTwoDx * lv;
                    A(idxU, vb + idxV) += scaleTwoDx * lv;
                    A(idxU, vb + vim1) += -scaleTwoDx * lv;
                    A(idxU, idxU) += scaleTwoDx * lv;
                }
                const long ujp1 = u_index(s, i, j + 1), vjp1 = v_index(s, i, j + 1);
                const long vim1jp1 = v_index(s, i - 1, j + 1);
                if (ujp1 != -1 && vjp1 != -1 && vim1jp1 != -1) {
                    const float lv = visc_interp(s, fi - 0.5f, fj + 0.5f);
                    A(idxU, ujp1) += -scaleTwoDx * lv;
                    A(idxU, vb + vjp1) += -scaleTwoDx * lv;
                    A(idxU, vb + vim1jp1) += scaleTwoDx * lv;
                    A(idxU, idxU) += scaleTwoDx * lv;
                }
            }
            if (idxV != -1) {
                const long r = vb + idxV;
                A(r, r) += density;
                const long vjm1 = v_index(s, i, j - 1);
                if (vjm1 != -1) {
                    A(r, vb + vjm1) += -scaleTwoDt * visc_get(s, i, j - 1);
                    A(r, r) += scaleTwoDt * visc_get(s, i, j - 1);
                }
                const long vjp1 = v_index(s, i, j + 1);
                if (vjp1 != -1) {
                    A(r, vb + vjp1) += -scaleTwoDt * visc_get(s, i, j);
                    A(r, r) += scaleTwoDt * visc_get(s, i, j);
                }
                const long ujm1 = u_index(s, i, j - 1), vim1 = v_index(s, i - 1, j);
                if (idxU != -1 && ujm1 != -1 && vim1 != -1) {
                    const float lv = visc_interp(s, fi - 0.5f, fj - 0.5f);
                    A(r, idxU) += scaleTwoDx * lv;
                    A(r, ujm1) += -scaleTwoDx * lv;
                    A(r, vb + vim1) += -scaleTwoDx * lv;
                    A(r, r) += scaleTwoDx * lv;
                }
                const long uip1 = u_index(s, i + 1, j), uip1jm1 = v_index(s, i + 1, j - 1);
                const long vip1 = v_index(s, i + 1, j);
                if (uip1 != -1 && uip1jm1 != -1 && vip1 != -1) {
                    const float lv = visc_interp(s, fi + 0.5f, fj - 0.5f);
                    A(r, uip1) += -scaleTwoDx * lv;
                    A(r, uip1jm1) += scaleTwoDx * lv;
                    A(r, vb + vip1) += -scaleTwoDx * lv;
                    A(r, r) += scaleTwoDx * lv;
                }
            }
        }
    }
#undef A
    double *b = (double *)calloc((size_t)N, sizeof(double)), *x = (double *)calloc((size_t)N, sizeof(double));
    for (long k = 0; k < NU; k++) b[k] = (double)(density * s->u[k]);
    for (long k = 0; k < NV; k++) b[vb + k] = (double)(density * s->v[k]);
    int ok = 0;
    long iters = vcg_solve(rows, N, 1e-4, b, x, &ok);
    if (ok) {
        for (long k = 0; k < NU; k++) s->u[k] = (float)x[k];
        for (long k = 0; k < NV; k++) s->v[k] = (float)x[vb + k];
    } else {
        iters = -1;
    }
    free(b);
    free(x);
    vrows_free(rows, N);
    return (int)iters;
}

static void friction(fso_solver *s) /* :1077-1104, validSolidNeighborIds :766-786 */
{
    const long NJ = s->nj, NV = s->nj + 1;
    for (long i = 0; i < s->ni; i++)
        for (long j = 0; j < s->nj; j++) {
            float sum = 0;
            int cnt = 0;
            for (long io = -1; io < 2; io++)
                for (long jo = -1; jo < 2; jo++) {
                    if (!in_bounds(s, i + io, j + jo)) continue;
                    int id = s->solid_id[(i + io) * NJ + (j + jo)];
                    if (id != -1) {
                        sum += s->obst[id].a;
                        cnt++;
                    }
                }
            if (cnt == 0) continue;
            float avg = sum / (float)cnt;
            int uAff = is_solid(s, i, j + 1) || is_solid(s, i - 1, j + 1) || is_solid(s, i, j) ||
                       is_solid(s, i - 1, j) || is_solid(s, i, j - 1) || is_solid(s, i - 1, j - 1);
            int vAff = is_solid(s, i + 1, j) || is_solid(s, i + 1, j - 1) || is_solid(s, i, j) ||
                       is_solid(s, i, j - 1) || is_solid(s, i - 1, j) || is_solid(s, i - 1, j - 1);
            if (uAff) s->u[i * NJ + j] = s->u[i * NJ + j] * (1 - avg);
            if (vAff) s->v[i * NV + j] = s->v[i * NV + j] * (1 - avg);
        }
}

/* ------------------------------------------------------------------------ */
/* grid -> particle, counting (flipsolver2d.cpp:361-388, 1021-1051)          */
/* ------------------------------------------------------------------------ */
static void g2p(fso_solver *s)
{
    const float pic = s->p.picRatio;
    for (size_t b = 0; b < s->nbins; b++) {
        pbin *bin = &s->bins[b];
        for (size_t k = 0; k < bin->n; k++) {
            float x = bin->pos[2 * k], y = bin->pos[2 * k + 1];
            float ox = grid_lerp(s->su, s->ni + 1, s->nj, 0.5f, 0.f, x, y);
            float oy = grid_lerp(s->sv, s->ni, s->nj + 1, 0.f, 0.5f, x, y);
            float nx, ny;
            velocity_at(s, s->u, s->v, x, y, &nx, &ny);
            float vx = bin->vel[2 * k], vy = bin->vel[2 * k + 1];
            float ax = nx * pic, ay = ny * pic;
            float tx = (vx + nx) - ox, ty = (vy + ny) - oy;
            float flip = 1.f - pic;
            bin->vel[2 * k] = ax + tx * flip;
            bin->vel[2 * k + 1] = ay + ty * flip;
        }
    }
}

static void count_particles(fso_solver *s)
{
    const int cap = 2 * s->p.particlesPerCell;
    for (long idx = 0; idx < (long)s->ncell; idx++) {
        long ci = idx / s->nj, cj = idx - ci * s->nj;
        pbin *bin = &s->bins[bin_of_cell(s, ci, cj)];
        s->counts[idx] = 0;
        for (size_t k = 0; k < bin->n; k++) {
            long i = (long)floorf(bin->pos[2 * k]);
            long j = (long)floorf(bin->pos[2 * k + 1]);
            if (ci == i && cj == j) {
                if (s->counts[idx] >= cap) {
                    bin_swap_erase(bin, k);
                    k--;
                    continue;
                }
                s->counts[idx] += 1;
            }
        }
    }
}

/* ------------------------------------------------------------------------ */
/* sources (emitters)                                                       */
/* ------------------------------------------------------------------------ */
/* FlipSolver::afterTransfer (flipsolver2d.cpp:390-410): source cells take
 * the emitter's viscosity and, when it transfers velocity, the faces (i, j)
 * of U and V take its velocity / dx (float / double) and become valid. */
static void sources_after_transfer(fso_solver *s)
{
    for (long i = 0; i < s->ni; i++)
        for (long j = 0; j < s->nj; j++) {
            if (!is_source(s, i, j)) continue;
            const source *e = &s->sources[s->emitter_id[i * s->nj + j]];
            s->visc_grid[i * s->nj + j] = e->visc;
            if (e->transfer) {
                s->u[i * s->nj + j] = (float)((double)e->vx / s->dx);
                s->v[i * (s->nj + 1) + j] = (float)((double)e->vy / s->dx);
                s->uvalid[i * s->nj + j] = 1;
                s->vvalid[i * (s->nj + 1) + j] = 1;
            }
        }
}

/* FlipSolver::reseedParticles (flipsolver2d.cpp:627-680): source cells with
 * fewer than particlesPerCell / 2 particles get the difference, jittered,
 * with the grid velocity there when the emitter transfers velocity (else
 * zero) and the emitter's viscosity, stored through the cell's bin as in
 * seedInitialFluid. */
static void flip_reseed(fso_solver *s)
{
    for (long i = 0; i < s->ni; i++)
        for (long j = 0; j < s->nj; j++) {
            const long l = i * s->nj + j;
            const int additional = (s->p.particlesPerCell / 2) - s->counts[l];
            if (additional <= 0 || !is_source(s, i, j)) continue;
            const source *e = &s->sources[s->emitter_id[l]];
            pbin *cellbin = &s->bins[bin_of_cell(s, i, j)];
            for (int q = 0; q < additional; q++) {
                float x = (float)i + mt_uniform01f(&s->rng);
                float y = (float)j + mt_uniform01f(&s->rng);
                float vx = 0.f, vy = 0.f;
                if (e->transfer) velocity_at(s, s->u, s->v, x, y, &vx, &vy);
                long pb = bin_of_pos(s, x, y);
                if (pb < 0) continue;
                size_t idx = bin_push(&s->bins[pb], x, y, vx, vy, 0.f, 0);
                if (idx < cellbin->n) cellbin->visc[idx] = e->visc;
            }
        }
}

/* ------------------------------------------------------------------------ */
/* NB-FLIP (nbflipsolver.cpp)                                               */
/* ------------------------------------------------------------------------ */
#define NB_NARROW_BAND (-3.f)      /* m_narrowBand,      nbflipsolver.cpp:20 */
#define NB_COMBINATION_BAND (-2.f) /* m_combinationBand, :21 */
#define NB_RESAMPLING_BAND (-1.f)  /* m_resamplingBand,  :22 */

/* NBFlipSolver::pruneNarrowBand (:227-253).  Particles already marked (killed
 * in advect, or moved: scheduleRebin marked the original and the copy in the
 * rebin set keeps its unmarked flag) are skipped: marking them again changes
 * nothing. */
static void nb_prune_band(fso_solver *s)
{
    const int cap = 2 * s->p.particlesPerCell;
    for (size_t b = 0; b < s->nbins; b++) {
        pbin *bin = &s->bins[b];
        for (size_t k = 0; k < bin->n; k++) {
            if (bin->dead[k]) continue;
            float x = bin->pos[2 * k], y = bin->pos[2 * k + 1];
            long i = (long)x, j = (long)y; /* ssize_t i = position.x() */
            float sdf = grid_lerp(s->fluid_sdf, s->ni, s->nj, 0.f, 0.f, x, y);
            const int src = is_source(s, i, j);
            if (!src && sdf < NB_NARROW_BAND) {
                bin->dead[k] = 1;
                continue;
            }
            if ((src || sdf < NB_RESAMPLING_BAND) && s->counts[i * s->nj + j] > cap) bin->dead[k] = 1;
        }
    }
}

/* FlipSolver::eulerAdvectionThread (flipsolver2d.cpp:340-351): every sample
 * (i, j) of the output grid traced back with rk4Integrate(-dt) through the
 * velocity grid, then the input grid (offset ox, oy) sampled there. */
static void nb_euler(fso_solver *s, const float *in, int si, int sj, float ox, float oy, float *out)
{
    for (long i = 0; i < si; i++)
        for (long j = 0; j < sj; j++) {
            float x = (float)i, y = (float)j;
            rk4(s, &x, &y, -s->step_dt);
            out[i * sj + j] = grid_lerp(in, si, sj, ox, oy, x, y);
        }
}

/* NBFlipSolver::advect (:66-109) */
static void nb_advect(fso_solver *s)
{
    advect(s);
    nb_prune_band(s);
    nb_euler(s, s->u, s->ni + 1, s->nj, 0.5f, 0.f, s->adv_u);
    nb_euler(s, s->v, s->ni, s->nj + 1, 0.f, 0.5f, s->adv_v);
    nb_euler(s, s->fluid_sdf, s->ni, s->nj, 0.f, 0.f, s->adv_sdf);
    nb_euler(s, s->visc_grid, s->ni, s->nj, 0.5f, 0.5f, s->adv_visc);
}

/* NBFlipSolver::afterTransfer (:111-116): FlipSolver::afterTransfer (sources
 * only), updateGridFromSources (:332-364: with no source the distance stays
 * FLT_MAX and the SDF becomes std::min(FLT_MAX, sdf)), combineAdvectedGrids
 * (:366-427). */
static void nb_after_transfer(fso_solver *s)
{
    const long ni = s->ni, nj = s->nj;
    sources_after_transfer(s);
    /* updateGridFromSources (:332-364): the nearest source's distance at the
     * cell corner (i dx, j dx) */
    const float dxf = (float)s->dx;
    for (long i = 0; i < ni; i++)
        for (long j = 0; j < nj; j++) {
            float dist = FLT_MAX;
            int id = -1;
            for (int k = 0; k < s->nsources; k++) {
                float sdf = polygon_sdf(&s->sources[k].g, (float)i * dxf, (float)j * dxf) / dxf;
                if (sdf < dist) {
                    dist = sdf;
                    id = k;
                }
            }
            const long l = i * nj + j;
            const float f = s->fluid_sdf[l];
            s->fluid_sdf[l] = f < dist ? f : dist; /* std::min(dist, sdf) */
            if (dist < 0 && id != -1) {
                s->visc_grid[l] = s->sources[id].visc;
                s->adv_visc[l] = s->sources[id].visc;
            }
        }
    /* combineLevelset: std::min(advected + h, sdf), h = 1 */
    for (size_t k = 0; k < s->ncell; k++) {
        float a = s->adv_sdf[k] + 1.f, b = s->fluid_sdf[k];
        s->fluid_sdf[k] = b < a ? b : a;
    }
    /* combineVelocityGrid: nbCombine(advected, particle, sdf) keeps the
     * particle (transferred) value where sdf > m_combinationBand */
    for (long i = 0; i < ni + 1; i++)
        for (long j = 0; j < nj; j++) {
            float sdf = grid_lerp(s->fluid_sdf, (int)ni, (int)nj, 0.f, 0.f, (float)i, 0.5f + (float)j);
            long l = i * nj + j;
            s->u[l] = sdf > NB_COMBINATION_BAND ? s->u[l] : s->adv_u[l];
        }
    for (long i = 0; i < ni; i++)
        for (long j = 0; j < nj + 1; j++) {
            float sdf = grid_lerp(s->fluid_sdf, (int)ni, (int)nj, 0.f, 0.f, 0.5f + (float)i, (float)j);
            long l = i * (nj + 1) + j;
            s->v[l] = sdf > NB_COMBINATION_BAND ? s->v[l] : s->adv_v[l];
        }
    /* combineCenteredGrids */
    for (long i = 0; i < ni; i++)
        for (long j = 0; j < nj; j++) {
            float sdf = grid_lerp(s->fluid_sdf, (int)ni, (int)nj, 0.f, 0.f, 0.5f + (float)i,
                                  (float)((double)j + 0.5));
            long l = i * nj + j;
            s->visc_grid[l] = sdf > NB_COMBINATION_BAND ? s->visc_grid[l] : s->adv_visc[l];
        }
}

/* NBFlipSolver::reseedParticles (:118-201): cells inside the resampling band
 * with fewer than particlesPerCell particles get jittered candidates; each
 * candidate draws two numbers, and is kept unless its interpolated SDF is
 * below the narrow band.  Kept particles are appended to the bin of their
 * position with zero velocity; the viscosity is stored through the cell's
 * bin at the index the position's bin returned (both are the same bin unless
 * i + U(0,1) rounded up into the next bin).  A candidate whose position
 * rounded out of the grid has no bin (the reference indexes past its bin
 * array there) and is dropped. */
static void nb_reseed(fso_solver *s)
{
    const int ppc = s->p.particlesPerCell;
    for (long i = 0; i < s->ni; i++)
        for (long j = 0; j < s->nj; j++) {
            long l = i * s->nj + j;
            float sc = s->fluid_sdf[l];
            const int src = is_source(s, i, j);
            if (!(src || (sc < NB_RESAMPLING_BAND && sc > NB_NARROW_BAND))) continue;
            int additional = ppc - s->counts[l];
            if (additional <= 0) continue;
            const int eid = s->emitter_id[l];
            pbin *cellbin = &s->bins[bin_of_cell(s, i, j)];
            for (int q = 0; q < additional; q++) {
                float x = (float)i + mt_uniform01f(&s->rng);
                float y = (float)j + mt_uniform01f(&s->rng);
                float nsdf = grid_lerp(s->fluid_sdf, s->ni, s->nj, 0.f, 0.f, x, y);
                if ((src && sc > NB_RESAMPLING_BAND) || nsdf < NB_NARROW_BAND) continue;
                float vx = 0.f, vy = 0.f;
                if (eid != -1 && s->sources[eid].transfer) velocity_at(s, s->u, s->v, x, y, &vx, &vy);
                float visc = eid != -1 ? s->sources[eid].visc
                                       : grid_lerp(s->visc_grid, s->ni, s->nj, 0.5f, 0.5f, x, y);
                long pb = bin_of_pos(s, x, y);
                if (pb < 0) continue;
                size_t idx = bin_push(&s->bins[pb], x, y, vx, vy, 0.f, 0);
                if (idx < cellbin->n) cellbin->visc[idx] = visc;
            }
        }
}

/* NBFlipSolver::firstFrameInit (:203-211): updateSinks, updateSources (no
 * sources), updateSolids, fluidSdfFromInitialFluid (:299-330), counts = 0,
 * initialFluidSeed (:255-297), which adds no particle (its add is commented
 * out in the reference) but draws two numbers per candidate: particlesPerCell
 * candidates in every cell with a negative SDF. */
static void nb_first_frame_init(fso_solver *s)
{
    update_sinks(s);
    update_sources(s);
    update_solids(s);
    float dx = (float)s->dx;
    for (long i = 0; i < s->ni; i++)
        for (long j = 0; j < s->nj; j++) {
            float dist = FLT_MAX;
            int fluidId = -1;
            for (int k = 0; k < s->nfluids; k++) {
                /* (static_cast<float>(i)+0.5)*dx is evaluated in double */
                float x = (float)(((double)(float)i + 0.5) * (double)dx);
                float y = (float)(((double)(float)j + 0.5) * (double)dx);
                float sdf = polygon_sdf(&s->fluids[k], x, y) / dx;
                if (sdf < dist) {
                    dist = sdf;
                    fluidId = k;
                }
            }
            long l = i * s->nj + j;
            s->fluid_sdf[l] = dist;
            if (dist < 0) {
                s->material[l] = M_FLUID;
                if (fluidId != -1) s->visc_grid[l] = s->fluids[fluidId].a;
            }
        }
    memset(s->counts, 0, s->ncell * sizeof(int32_t));
    for (size_t l = 0; l < s->ncell; l++)
        if (s->fluid_sdf[l] < 0.f)
            for (int q = 0; q < 2 * s->p.particlesPerCell; q++) (void)mt_next(&s->rng);
}

/* ------------------------------------------------------------------------ */
/* driver                                                                   */
/* ------------------------------------------------------------------------ */
static int run_stage(fso_solver *s, int stage);

/* Stage entry point: like SolverStats::reset before the stage, so the solve
 * statistics report this stage's solve. */
int fso_run_stage(fso_solver *s, int stage)
{
    if (stage == FSO_DENSITY) s->density_iters = 0;
    if (stage == FSO_PROJECT) s->pressure_iters = 0;
    return run_stage(s, stage);
}

static int run_stage(fso_solver *s, int stage)
{
    switch (stage) {
    case FSO_ADVECT:
        if (s->nb) nb_advect(s);
        else advect(s);
        break;
    case FSO_DECOMPOSITION: build_matrix(s); break;
    case FSO_REBIN: prune(s); rebin(s); break;
    case FSO_DENSITY:
        if (!s->p.viscosityEnabled) density_correction(s);
        break;
    case FSO_P2G: particle_to_grid(s); break;
    case FSO_SDF: update_sdf(s); break;
    case FSO_MATERIALS: update_materials(s); break;
    case FSO_AFTER_TRANSFER: /* sources, plus NB-FLIP's grid combination */
        if (s->nb) nb_after_transfer(s);
        else sources_after_transfer(s);
        break;
    case FSO_LEVELSET: bfs_extrapolate(s->fluid_sdf, NULL, s->ni, s->nj, 0, 0); break;
    case FSO_VEL_EXTRAP: extrapolate_velocity(s); break;
    case FSO_SAVE_GRID:
        memcpy(s->su, s->u, s->nu * sizeof(float));
        memcpy(s->sv, s->v, s->nv * sizeof(float));
        memcpy(s->suvalid, s->uvalid, s->nu);
        memcpy(s->svvalid, s->vvalid, s->nv);
        break;
    case FSO_BODY_FORCES: body_forces(s); break;
    case FSO_PROJECT: project(s); break;
    case FSO_FRICTION: friction(s); break;
    case FSO_G2P: g2p(s); break;
    case FSO_COUNT: count_particles(s); break;
    case FSO_RESEED: /* sources, or NB-FLIP's band reseeding */
        if (s->nb) nb_reseed(s);
        else flip_reseed(s);
        break;
    case FSO_DENSITY_GRID: update_density_grid(s); break;
    case FSO_LEVELSET_OUTSIDE: bfs_extrapolate(s->fluid_sdf, NULL, s->ni, s->nj, 2, 0); break;
    case FSO_VISCOSITY: /* FlipSolver::applyViscosity, flipsolver2d.cpp:128-136 */
        s->viscosity_iters = s->p.useHeavyViscosity ? viscosity_heavy(s) : viscosity_light(s);
        break;
    default: return -1;
    }
    return 0;
}

static void step(fso_solver *s) /* FlipSolver::step, flipsolver2d.cpp:412-462 */
{
    static const int order[] = {FSO_ADVECT, FSO_DECOMPOSITION, FSO_REBIN, FSO_DENSITY, FSO_P2G,
                                FSO_SDF, FSO_MATERIALS, FSO_AFTER_TRANSFER, FSO_LEVELSET,
                                FSO_VEL_EXTRAP, FSO_SAVE_GRID, FSO_BODY_FORCES, FSO_PROJECT,
                                FSO_FRICTION, FSO_VEL_EXTRAP, FSO_G2P, FSO_COUNT, FSO_RESEED};
    /* NBFlipSolver::step (nbflipsolver.cpp:26-64), gridUpdate (:213-225) */
    static const int nb_order[] = {FSO_ADVECT, FSO_REBIN, FSO_P2G, FSO_VEL_EXTRAP, FSO_SAVE_GRID,
                                   FSO_SDF, FSO_LEVELSET_OUTSIDE, FSO_AFTER_TRANSFER, FSO_LEVELSET,
                                   FSO_MATERIALS, FSO_BODY_FORCES, FSO_DECOMPOSITION, FSO_PROJECT,
                                   FSO_FRICTION, FSO_VEL_EXTRAP, FSO_G2P, FSO_COUNT, FSO_RESEED};
    const int *ord = s->nb ? nb_order : order;
    const size_t n = s->nb ? sizeof(nb_order) / sizeof(nb_order[0]) : sizeof(order) / sizeof(order[0]);
    for (size_t k = 0; k < n; k++) {
        run_stage(s, ord[k]);
        /* with viscosity on, both steps apply it after the friction update
         * and project again (flipsolver2d.cpp:448-454, nbflipsolver.cpp:50-56) */
        if (ord[k] == FSO_FRICTION && s->p.viscosityEnabled) {
            run_stage(s, FSO_VISCOSITY);
            run_stage(s, FSO_PROJECT);
        }
    }
}

void fso_step(fso_solver *s)
{
    s->density_iters = 0;
    s->pressure_iters = 0;
    s->substeps = 0;
    step(s);
}

float fso_max_particle_velocity(fso_solver *s) /* :1560-1574 */
{
    float m = FLT_MIN;
    for (size_t b = 0; b < s->nbins; b++) {
        const pbin *bin = &s->bins[b];
        for (size_t k = 0; k < bin->n; k++) {
            float vx = bin->vel[2 * k], vy = bin->vel[2 * k + 1];
            float v2 = vx * vx + vy * vy;
            if (v2 > m) m = v2;
        }
    }
    return sqrtf(m);
}

void fso_step_frame(fso_solver *s) /* FlipSolver::stepFrame, :464-500 */
{
    if (s->frame == 0) fso_first_frame_init(s);
    float substepTime = 0.f;
    int finished = 0, substepCount = 0;
    s->density_iters = s->pressure_iters = s->substeps = 0;
    while (!finished) {
        float vel = fso_max_particle_velocity(s);
        float maxSubstepSize = s->p.cflNumber / (vel + 1e-15f);
        if (substepTime + maxSubstepSize >= s->frame_dt || substepCount == (s->p.maxSubsteps - 1)) {
            maxSubstepSize = s->frame_dt - substepTime;
            finished = 1;
        } else if (substepTime + 2.f * maxSubstepSize >= s->frame_dt) {
            maxSubstepSize = 0.5f * (s->frame_dt - substepTime);
        }
        s->step_dt = maxSubstepSize;
        step(s);
        s->substeps++;
        substepTime += maxSubstepSize;
        substepCount++;
        if (substepCount > 50) break;
    }
    s->frame++;
}

void fso_set_step_dt(fso_solver *s, float dt) { s->step_dt = dt; }
float fso_step_dt(fso_solver *s) { return s->step_dt; }

size_t fso_bin_count(fso_solver *s) { return s->nbins; }

size_t fso_particle_count(fso_solver *s)
{
    size_t n = 0;
    for (size_t b = 0; b < s->nbins; b++) n += s->bins[b].n;
    return n;
}

void fso_get_particles(fso_solver *s, int32_t *counts, float *pos, float *vel, float *visc,
                       uint8_t *dead)
{
    size_t k = 0;
    for (size_t b = 0; b < s->nbins; b++) {
        const pbin *bin = &s->bins[b];
        counts[b] = (int32_t)bin->n;
        memcpy(pos + 2 * k, bin->pos, bin->n * 2 * sizeof(float));
        memcpy(vel + 2 * k, bin->vel, bin->n * 2 * sizeof(float));
        memcpy(visc + k, bin->visc, bin->n * sizeof(float));
        memcpy(dead + k, bin->dead, bin->n);
        k += bin->n;
    }
}

void fso_set_particles(fso_solver *s, const int32_t *counts, const float *pos, const float *vel,
                       const float *visc, const uint8_t *dead)
{
    size_t k = 0;
    for (size_t b = 0; b < s->nbins; b++) {
        pbin *bin = &s->bins[b];
        size_t n = (size_t)counts[b];
        bin_reserve(bin, n);
        bin->n = n;
        memcpy(bin->pos, pos + 2 * k, n * 2 * sizeof(float));
        memcpy(bin->vel, vel + 2 * k, n * 2 * sizeof(float));
        memcpy(bin->visc, visc + k, n * sizeof(float));
        memcpy(bin->dead, dead + k, n);
        k += n;
    }
}

size_t fso_grid_bytes(fso_solver *s, int which)
{
    size_t n = s->ncell;
    switch (which) {
    case FSO_G_MATERIAL: case FSO_G_KNOWN_CENTERED: return n;
    case FSO_G_SOLID_SDF: case FSO_G_FLUID_SDF: case FSO_G_VISCOSITY: case FSO_G_DENSITY:
    case FSO_G_DIV_CONTROL: case FSO_G_PARTICLE_COUNTS: case FSO_G_SOLID_ID:
    case FSO_G_EMITTER_ID: return n * 4;
    case FSO_G_U: case FSO_G_SAVED_U: return s->nu * 4;
    case FSO_G_V: case FSO_G_SAVED_V: return s->nv * 4;
    case FSO_G_U_VALID: return s->nu;
    case FSO_G_V_VALID: return s->nv;
    case FSO_G_DENSITY_RHS: case FSO_G_DENSITY_PRESSURE: case FSO_G_PRESSURE:
    case FSO_G_PRESSURE_RHS: return n * 8;
    case FSO_G_ADVECTED_U: return s->nb ? s->nu * 4 : 0;
    case FSO_G_ADVECTED_V: return s->nb ? s->nv * 4 : 0;
    case FSO_G_ADVECTED_SDF: case FSO_G_ADVECTED_VISCOSITY: return s->nb ? n * 4 : 0;
    default: return 0;
    }
}

static void *grid_ptr(fso_solver *s, int which)
{
    switch (which) {
    case FSO_G_MATERIAL: return s->material;
    case FSO_G_SOLID_SDF: return s->solid_sdf;
    case FSO_G_FLUID_SDF: return s->fluid_sdf;
    case FSO_G_U: return s->u;
    case FSO_G_V: return s->v;
    case FSO_G_U_VALID: return s->uvalid;
    case FSO_G_V_VALID: return s->vvalid;
    case FSO_G_SAVED_U: return s->su;
    case FSO_G_SAVED_V: return s->sv;
    case FSO_G_VISCOSITY: return s->visc_grid;
    case FSO_G_KNOWN_CENTERED: return s->known;
    case FSO_G_DENSITY: return s->dens;
    case FSO_G_PARTICLE_COUNTS: return s->counts;
    case FSO_G_SOLID_ID: return s->solid_id;
    case FSO_G_DIV_CONTROL: return s->divc;
    case FSO_G_DENSITY_RHS: return s->dens_rhs;
    case FSO_G_DENSITY_PRESSURE: return s->dens_p;
    case FSO_G_PRESSURE: return s->pres;
    case FSO_G_PRESSURE_RHS: return s->pres_rhs;
    case FSO_G_EMITTER_ID: return s->emitter_id;
    case FSO_G_ADVECTED_U: return s->adv_u;
    case FSO_G_ADVECTED_V: return s->adv_v;
    case FSO_G_ADVECTED_SDF: return s->adv_sdf;
    case FSO_G_ADVECTED_VISCOSITY: return s->adv_visc;
    default: return NULL;
    }
}

int fso_get_grid(fso_solver *s, int which, void *out)
{
    void *p = grid_ptr(s, which);
    if (!p) return -1;
    memcpy(out, p, fso_grid_bytes(s, which));
    return 0;
}

int fso_set_grid(fso_solver *s, int which, const void *in)
{
    void *p = grid_ptr(s, which);
    if (!p) return -1;
    memcpy(p, in, fso_grid_bytes(s, which));
    return 0;
}

int fso_stat(fso_solver *s, int which)
{
    switch (which) {
    case FSO_S_DENSITY_ITERS: return s->density_iters;
    case FSO_S_PRESSURE_ITERS: return s->pressure_iters;
    case FSO_S_SUBSTEPS: return s->substeps;
    case FSO_S_FRAME: return s->frame;
    case FSO_S_POOL_THREADS: return s->ref_threads;
    case FSO_S_VISCOSITY_ITERS: return s->viscosity_iters;
    default: return -1;
    }
}

int fso_pcg_solve(int ni, int nj, const int8_t *material, float dt, double density, double dx,
                  const double *rhs, double *result, int iter_limit, double tol)
{
    fso_params p;
    memset(&p, 0, sizeof(p));
    p.fluidDensity = density;
    p.dx = dx;
    p.particlesPerCell = 4;
    p.fps = 30;
    p.maxSubsteps = 1;
    p.pcgIterLimit = iter_limit;
    p.gridSizeI = ni;
    p.gridSizeJ = nj;
    fso_solver *s = fso_create(&p);
    memcpy(s->material, material, s->ncell);
    s->step_dt = dt;
    build_matrix(s);
    int it = linear_solve(s, result, rhs, iter_limit, tol);
    fso_destroy(s);
    return it;
}


/* ---- spec mode: full-FP64 PCG with the textbook IPP ---------------------- *
 * The reference ships a second incomplete-Poisson preconditioner that it
 * never uses on the hot path (inversepoissonpreconditioner.h:45-79):
 * M = K K^T with K = I - L D^-1, L the strictly lower part of the pressure
 * matrix A (linear index order) and D its diagonal.  With A built as in
 * getPressureProjectionMatrix (unit rows only), K has 1 / count(n) at
 * (c, n) for the lower fluid neighbours n = c - NJ (mask bit 1) and
 * n = c - 1 (mask bit 4) of a unit row c.  This plain double-precision PCG
 * with M and a true relative-residual stopping test is the FP64 oracle of
 * the GPU's mixed-precision spec solve.  Deterministic for any thread count. */
/* K(c, n) for a strictly lower neighbour n of unit row c:
 * -A(c, n) / A(n, n) = scale / A(n, n), with Eigen's rule that a zero
 * diagonal counts as 1; a non-unit row of A is an identity row. */
static double spec_k(const fso_solver *s, long n)
{
    if (s->unit[n] && s->ucount[n] > 0) return 1.0 / s->ucount[n];
    return s->mscale;
}

/* The loops below run on the solver's pool (FSO_HOST_THREADS threads).  Every
 * cell is written by one thread, and the dot products sum SPEC_CHUNKS fixed
 * chunks in chunk order, so the results do not depend on the thread count. */
#define SPEC_CHUNKS 64

typedef struct spec_ctx {
    const fso_solver *s;
    const double *in, *in2;
    double *out, *out2;
    double alpha;
    long n;
    double part[SPEC_CHUNKS];
} spec_ctx;

/* y = K^T r: row n of K^T collects K(c, n) over the unit rows c whose lower
 * neighbour is n */
static void spec_kt_range(void *ctx, size_t a, size_t b)
{
    spec_ctx *c = (spec_ctx *)ctx;
    const fso_solver *s = c->s;
    const long N = (long)s->ncell, NJ = s->nj;
    const double *r = c->in;
    for (long n = (long)a; n < (long)b; n++) {
        double v = r[n];
        const double k = spec_k(s, n);
        if (n + NJ < N && s->unit[n + NJ] && (s->mask[n + NJ] & 1)) v += k * r[n + NJ];
        if (n + 1 < N && s->unit[n + 1] && (s->mask[n + 1] & 4)) v += k * r[n + 1];
        c->out[n] = v;
    }
}

/* z = K y */
static void spec_k_range(void *ctx, size_t a, size_t b)
{
    spec_ctx *c = (spec_ctx *)ctx;
    const fso_solver *s = c->s;
    const long NJ = s->nj;
    const double *y = c->in;
    for (long k = (long)a; k < (long)b; k++) {
        double v = y[k];
        if (s->unit[k]) {
            if ((s->mask[k] & 1) && k - NJ >= 0) v += spec_k(s, k - NJ) * y[k - NJ];
            if ((s->mask[k] & 4) && k - 1 >= 0) v += spec_k(s, k - 1) * y[k - 1];
        }
        c->out[k] = v;
    }
}

static void spec_apply_m(const fso_solver *s, const double *r, double *y, double *z)
{
    spec_ctx c;
    c.s = s;
    c.in = r;
    c.out = y;
    par_for(s->pool, s->ncell, spec_kt_range, &c);
    c.in = y;
    c.out = z;
    par_for(s->pool, s->ncell, spec_k_range, &c);
}

static void spec_apply_a(const fso_solver *s, const double *in, double *out)
{
    mv_ctx c = {(fso_solver *)s, in, out};
    par_for(s->pool, s->ncell, amul_range, &c);
}

static void spec_dot_range(void *ctx, size_t a, size_t b)
{
    spec_ctx *c = (spec_ctx *)ctx;
    for (size_t k = a; k < b; k++) {
        size_t lo, hi;
        pool_chunk((size_t)c->n, SPEC_CHUNKS, (int)k, &lo, &hi);
        double acc = 0.0;
        for (size_t e = lo; e < hi; e++) acc += c->in[e] * c->in2[e];
        c->part[k] = acc;
    }
}

static double spec_dot(const fso_solver *s, const double *a, const double *b, long n)
{
    spec_ctx c;
    c.in = a;
    c.in2 = b;
    c.n = n;
    par_for(s->pool, SPEC_CHUNKS, spec_dot_range, &c);
    double acc = 0.0;
    for (int k = 0; k < SPEC_CHUNKS; k++) acc += c.part[k];
    return acc;
}

/* x += alpha d and r -= alpha q */
static void spec_update_range(void *ctx, size_t a, size_t b)
{
    spec_ctx *c = (spec_ctx *)ctx;
    for (size_t k = a; k < b; k++) {
        c->out[k] += c->alpha * c->in[k];
        c->out2[k] -= c->alpha * c->in2[k];
    }
}

/* d = z + beta d */
static void spec_dir_range(void *ctx, size_t a, size_t b)
{
    spec_ctx *c = (spec_ctx *)ctx;
    for (size_t k = a; k < b; k++) c->out[k] = c->in[k] + c->alpha * c->out[k];
}

int fso_spec_solve(int ni, int nj, const int8_t *material, float dt, double density, double dx,
                   const double *rhs, double *result, double rel_tol, int max_iter,
                   double *rel_residual)
{
    fso_params p;
    memset(&p, 0, sizeof(p));
    p.fluidDensity = density;
    p.dx = dx;
    p.particlesPerCell = 4;
    p.fps = 30;
    p.maxSubsteps = 1;
    p.pcgIterLimit = max_iter;
    p.gridSizeI = ni;
    p.gridSizeJ = nj;
    fso_solver *s = fso_create(&p);
    memcpy(s->material, material, s->ncell);
    s->step_dt = dt;
    build_matrix(s);
    const long N = (long)s->ncell;
    double *r = (double *)calloc(N, sizeof(double)), *z = (double *)calloc(N, sizeof(double));
    double *y = (double *)calloc(N, sizeof(double)), *d = (double *)calloc(N, sizeof(double));
    double *q = (double *)calloc(N, sizeof(double));
    for (long k = 0; k < N; k++) {
        result[k] = 0.0;
        r[k] = rhs[k];
    }
    const double bnorm = sqrt(spec_dot(s, rhs, rhs, N));
    int it = 0;
    double rnorm = bnorm;
    spec_ctx c;
    if (bnorm > 0.0) {
        spec_apply_m(s, r, y, z);
        memcpy(d, z, N * sizeof(double));
        double rz = spec_dot(s, r, z, N);
        for (it = 0; it < max_iter; it++) {
            rnorm = sqrt(spec_dot(s, r, r, N));
            if (rnorm <= rel_tol * bnorm) break;
            spec_apply_a(s, d, q);
            c.alpha = rz / spec_dot(s, d, q, N);
            c.in = d;
            c.in2 = q;
            c.out = result;
            c.out2 = r;
            par_for(s->pool, (size_t)N, spec_update_range, &c);
            spec_apply_m(s, r, y, z);
            const double rz2 = spec_dot(s, r, z, N);
            c.alpha = rz2 / rz; /* beta */
            rz = rz2;
            c.in = z;
            c.out = d;
            par_for(s->pool, (size_t)N, spec_dir_range, &c);
        }
        /* true residual of the returned solution */
        spec_apply_a(s, result, q);
        for (long k = 0; k < N; k++) q[k] = rhs[k] - q[k];
        rnorm = sqrt(spec_dot(s, q, q, N));
    }
    if (rel_residual) *rel_residual = bnorm > 0.0 ? rnorm / bnorm : 0.0;
    free(r);
    free(z);
    free(y);
    free(d);
    free(q);
    fso_destroy(s);
    return it;
}

/* The processor count std::thread::hardware_concurrency() reports on this
 * host (libstdc++ asks glibc's get_nprocs), which sizes the reference's
 * thread pool (threadpool.cpp:12); recorded beside the CPU baseline. */
int fso_hardware_concurrency(void)
{
    return get_nprocs();
}
