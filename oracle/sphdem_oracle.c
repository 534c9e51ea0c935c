/*
 * sphdem_oracle.c -- CPU restatement of the reference WCSPH-DEM step.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle the GPU results are
 * compared with: the tests, the smoke test and the CPU-baseline leg of
 * bench.py load it; the product path never does.  It restates, kernel by kernel and in the reference's own expression
 * order, the Warp kernels of hojin9908/Warp_SPH_GPT (the kernel/ directory) and the step
 * ordering of source/Simulation.py.  Each function cites the lines it follows.
 *
 * Two builds come from this one source:
 *   liboracle_f32.so  (ORACLE_REAL=float)  "reference semantics": every value
 *       rounded in FP32 exactly where the reference rounds, compiled with
 *       -ffp-contract=off so no multiply-add is fused.  Judge of neighbour
 *       sets, contact CSR and integer work (bit-exact), and of fields.
 *   liboracle_f64.so  (ORACLE_REAL=double)  the same step with the physics in
 *       FP64; state stays float32 between kernels (the reference layout).
 *       Judge of the 1e-5 field tolerance.
 * In both builds every membership predicate (distance tests that decide a
 * neighbour or a contact) is evaluated in FP32, as the reference does, so both
 * oracles see the same neighbour and contact sets.
 *
 * Neighbour enumeration: the reference queries wp.HashGrid and then filters
 * every candidate with an explicit predicate; warp-lang 1.17's hash-grid query
 * returns every point of the cells overlapping the query box, so the member
 * sets are defined by the predicates alone.  Here a uniform cell list with a
 * slightly padded query box enumerates a superset of candidates and the same
 * predicates filter them.  Contact rows are written in ascending neighbour id
 * (the reference writes them in grid-traversal order; its own tests compare
 * rows as sets, tests/test_dem.py:75-83,216).
 *
 * Parallelism: subjects are independent in every reference kernel, so the
 * subject loop runs on a small pthread pool (oracle_set_threads).
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "sphdem.h"

#ifndef ORACLE_REAL
#define ORACLE_REAL float
#endif
typedef ORACLE_REAL real;
#define R(x) ((real)(x))

static const real PI_R = (real)3.14159265358979323846;
static const float R2_MIN = 1.0e-12f; /* kernel/Kernel_KNL.py:5 */

/* ------------------------------------------------------------------------ */
/* thread pool                                                               */
/* ------------------------------------------------------------------------ */
static int g_threads = 1;

int oracle_set_threads(int n) {
    g_threads = n < 1 ? 1 : (n > 256 ? 256 : n);
    return g_threads;
}

typedef void (*body_fn)(void* ctx, int i);
typedef struct {
    body_fn fn;
    void* ctx;
    int n;
    int chunk;
    int next;
} par_job;

static void* par_worker(void* arg) {
    par_job* job = (par_job*)arg;
    for (;;) {
        int start = __atomic_fetch_add(&job->next, job->chunk, __ATOMIC_RELAXED);
        if (start >= job->n) break;
        int end = start + job->chunk < job->n ? start + job->chunk : job->n;
        for (int i = start; i < end; ++i) job->fn(job->ctx, i);
    }
    return NULL;
}

/* Timing samples only: subjects i with i % g_stride != 0 are skipped, so a
   step costs ~1/g_stride of the full work (results are then incomplete).  The
   sampled subjects stay close to each other, so their neighbourhoods share
   caches as in a full pass; callers pick a stride coprime to the particle
   lattice's dimensions so the sample does not alias with its layers. */
static int g_stride = 1;

int oracle_set_subject_stride(int s) {
    g_stride = s < 1 ? 1 : s;
    return g_stride;
}

typedef struct {
    body_fn fn;
    void* ctx;
} strided_ctx;

static void strided_body(void* c, int i) {
    strided_ctx* s = (strided_ctx*)c;
    s->fn(s->ctx, i * g_stride);
}

static void par_for_all(int n, body_fn fn, void* ctx);

static void par_for(int n, body_fn fn, void* ctx) {
    if (g_stride > 1) {
        strided_ctx s = {fn, ctx};
        par_for_all((n + g_stride - 1) / g_stride, strided_body, &s);
        return;
    }
    par_for_all(n, fn, ctx);
}

static void par_for_all(int n, body_fn fn, void* ctx) {
    if (n <= 0) return;
    par_job job = {fn, ctx, n, 16, 0};
    int t = g_threads;
    if (t <= 1 || n < 64) {
        par_worker(&job);
        return;
    }
    pthread_t tid[256];
    int started = 0;
    for (int k = 1; k < t; ++k)
        if (pthread_create(&tid[started], NULL, par_worker, &job) == 0) ++started;
    par_worker(&job);
    for (int k = 0; k < started; ++k) pthread_join(tid[k], NULL);
}

/* ------------------------------------------------------------------------ */
/* uniform cell list (candidate enumeration only)                            */
/* ------------------------------------------------------------------------ */
typedef struct {
    double lo[3];
    double inv;
    int dim[3];
    int* start; /* [ncell+1] */
    int* idx;   /* [n] */
    int n;
} ogrid;

static int ocoord(double x, double lo, double inv, int dim) {
    double f = floor((x - lo) * inv);
    if (!(f == f) || f < 0.0) return 0;
    if (f >= (double)dim) return dim - 1;
    return (int)f;
}

static void ogrid_build(ogrid* g, const float* pos, int n, double cell) {
    double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    for (int i = 0; i < n; ++i)
        for (int d = 0; d < 3; ++d) {
            double x = pos[3 * i + d];
            if (!(x == x)) continue;
            if (i == 0 || x < lo[d]) lo[d] = x;
            if (i == 0 || x > hi[d]) hi[d] = x;
        }
    if (!(cell > 0.0)) cell = 1.0;
    long total;
    for (;;) { /* wider cells only add candidates; keep the table small */
        g->inv = 1.0 / cell;
        total = 1;
        for (int d = 0; d < 3; ++d) {
            g->lo[d] = lo[d];
            long dim = (long)floor((hi[d] - lo[d]) * g->inv) + 1;
            if (dim < 1) dim = 1;
            if (dim > 4096) dim = 4096; /* clamped bins stay complete */
            g->dim[d] = (int)dim;
            total *= dim;
        }
        if (total <= (1L << 24)) break;
        cell *= 1.5;
    }
    g->n = n;
    g->start = (int*)calloc((size_t)total + 1, sizeof(int));
    g->idx = (int*)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    int* key = (int*)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    for (int i = 0; i < n; ++i) {
        int c[3];
        for (int d = 0; d < 3; ++d) c[d] = ocoord(pos[3 * i + d], g->lo[d], g->inv, g->dim[d]);
        key[i] = (c[0] * g->dim[1] + c[1]) * g->dim[2] + c[2];
        g->start[key[i] + 1]++;
    }
    for (long k = 0; k < total; ++k) g->start[k + 1] += g->start[k];
    int* fill = (int*)malloc(sizeof(int) * (size_t)total);
    memcpy(fill, g->start, sizeof(int) * (size_t)total);
    for (int i = 0; i < n; ++i) g->idx[fill[key[i]]++] = i; /* stable by index */
    free(fill);
    free(key);
}

static void ogrid_free(ogrid* g) {
    free(g->start);
    free(g->idx);
}

/* Cell window of the query box centred at p with half width r (padded). */
typedef struct {
    int c0[3], c1[3];
} owin;

static owin ogrid_window(const ogrid* g, const float* p, double r) {
    owin w;
    double rq = r * 1.001 + 1.0e-6;
    for (int d = 0; d < 3; ++d) {
        w.c0[d] = ocoord((double)p[d] - rq, g->lo[d], g->inv, g->dim[d]);
        w.c1[d] = ocoord((double)p[d] + rq, g->lo[d], g->inv, g->dim[d]);
    }
    return w;
}

/* Iterate candidate point indices J of grid G around P within R. */
#define OGRID_FOR(G, P, RAD, J, ...)                                                     \
    do {                                                                                  \
        owin w_ = ogrid_window((G), (P), (RAD));                                          \
        for (int cx_ = w_.c0[0]; cx_ <= w_.c1[0]; ++cx_)                                  \
            for (int cy_ = w_.c0[1]; cy_ <= w_.c1[1]; ++cy_) {                            \
                int base_ = (cx_ * (G)->dim[1] + cy_) * (G)->dim[2];                      \
                int s_ = (G)->start[base_ + w_.c0[2]], e_ = (G)->start[base_ + w_.c1[2] + 1]; \
                for (int k_ = s_; k_ < e_; ++k_) {                                        \
                    int J = (G)->idx[k_];                                                 \
                    __VA_ARGS__                                                           \
                }                                                                         \
            }                                                                             \
    } while (0)

/* ------------------------------------------------------------------------ */
/* FP32 predicates (identical in both builds)                                */
/* ------------------------------------------------------------------------ */
/* dot(a-b, a-b) as Warp evaluates it: ((dx*dx + dy*dy) + dz*dz) in FP32. */
static inline float f_d2(const float* a, const float* b) {
    float dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
    float s = dx * dx;
    s = s + dy * dy;
    s = s + dz * dz;
    return s;
}
static inline float f_len(const float* a, const float* b) { return sqrtf(f_d2(a, b)); }

/* ------------------------------------------------------------------------ */
/* small vector helpers in `real`                                            */
/* ------------------------------------------------------------------------ */
typedef struct {
    real x, y, z;
} v3;
static inline v3 V(real x, real y, real z) { v3 r = {x, y, z}; return r; }
static inline v3 ld3(const float* a, int i) { return V((real)a[3 * i], (real)a[3 * i + 1], (real)a[3 * i + 2]); }
static inline void st3(float* a, int i, v3 v) {
    a[3 * i] = (float)v.x;
    a[3 * i + 1] = (float)v.y;
    a[3 * i + 2] = (float)v.z;
}
static inline v3 vadd(v3 a, v3 b) { return V(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 vsub(v3 a, v3 b) { return V(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 vmul(real s, v3 a) { return V(s * a.x, s * a.y, s * a.z); }
static inline v3 vdiv(v3 a, real s) { return V(a.x / s, a.y / s, a.z / s); }
static inline v3 vneg(v3 a) { return V(-a.x, -a.y, -a.z); }
static inline real vdot(v3 a, v3 b) {
    real s = a.x * b.x;
    s = s + a.y * b.y;
    s = s + a.z * b.z;
    return s;
}
static inline real vlen(v3 a) { return (real)sqrt((double)vdot(a, a)); }
static inline v3 vcross(v3 a, v3 b) {
    return V(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline real rsqrt_(real x) { return (real)sqrt((double)x); }
static inline real rpow(real a, real b) {
    if (sizeof(real) == sizeof(float)) return (real)powf((float)a, (float)b);
    return (real)pow((double)a, (double)b);
}
static inline real rmax(real a, real b) { return a > b ? a : b; }
static inline real rmin(real a, real b) { return a < b ? a : b; }
static inline real rclamp(real x, real a, real b) { return rmin(rmax(x, a), b); }
static inline real rabs(real x) { return x < 0 ? -x : x; }
/* wp.sign: -1 if x < 0 else 1 */
static inline real rsign(real x) { return x < R(0) ? R(-1) : R(1); }

/* ------------------------------------------------------------------------ */
/* Wendland C2, kernel/Kernel_KNL.py:7-41                                    */
/* ------------------------------------------------------------------------ */
static inline real wendland_w(real r, real h) {
    real q = r / h;
    real w = R(0);
    real u = R(1) - R(0.5) * q;
    if (q < R(2)) w = R(21) * u * u * u * u * (R(1) + R(2) * q) / (R(16) * PI_R * h * h * h);
    return w;
}
static inline real wendland_dw(real r, real h) {
    real q = r / h;
    real dw = R(0);
    if (q < R(2)) {
        real u = R(1) - R(0.5) * q;
        dw = R(21) * (R(-5) * q * u * u * u) / (R(16) * PI_R * h * h * h * h);
    }
    return dw;
}

void oracle_wendland(const float* r, int n, float h, double* w, double* dw) {
    for (int i = 0; i < n; ++i) {
        w[i] = (double)wendland_w((real)r[i], (real)h);
        dw[i] = (double)wendland_dw((real)r[i], (real)h);
    }
}

/* DEM_drag_beta, kernel/KERNEL_SPHDEM_interaction.py:11-40 */
static real drag_beta(real eps, real rho, real mu, real diameter, real speed) {
    real beta = R(0);
    real reynolds = rho * diameter * speed / (mu + R(1.0e-20));
    /* branch tests in FP32 as the reference evaluates them (both builds) */
    if ((float)eps <= 0.8f) {
        beta = R(150) * (R(1) - eps) / eps * mu / (diameter * diameter) + R(1.75) * rho * speed / diameter;
    } else {
        real cd_speed = R(0.44) * speed;
        if ((float)reynolds <= 1000.0f)
            cd_speed = R(24) * mu / (rho * diameter) * (R(1) + R(0.15) * rpow(reynolds, R(0.687)));
        beta = R(0.75) * cd_speed * rho / diameter * rpow(eps, R(-1.65));
    }
    return beta;
}

void oracle_drag_beta(const float* eps, const float* rho, const float* mu, const float* d,
                      const float* speed, int n, double* out) {
    for (int i = 0; i < n; ++i)
        out[i] = (double)drag_beta((real)eps[i], (real)rho[i], (real)mu[i], (real)d[i], (real)speed[i]);
}

/* ------------------------------------------------------------------------ */
/* SPH kernels                                                               */
/* ------------------------------------------------------------------------ */
typedef struct {
    sphdem_sph_t* P;
    const sphdem_bnd_t* B;
    const sphdem_dem_t* D;
    ogrid gs, gb, gd, gs2;
    float support, h, mu, g, sph_support, sph_h, eps_min, eps_max, rho0, c0, gamma;
    real* out; /* scratch (flt values, etc.) */
} sph_job;

/* Kernel_shepard_sph, kernel/KERNEL_rho.py:6-40 */
static void shepard_body(void* c, int i) {
    sph_job* J = (sph_job*)c;
    const float* ri = J->P->pos + 3 * i;
    float s2 = J->support * J->support;
    real h = (real)J->h, flt = R(0);
    OGRID_FOR(&J->gs, ri, J->support, j, {
        float tdist = f_d2(ri, J->P->pos + 3 * j);
        if (tdist < s2) {
            real wij = wendland_w(rsqrt_((real)tdist), h);
            flt = flt + ((real)J->P->m[j] / (real)J->P->rho[j]) * wij;
        }
    });
    OGRID_FOR(&J->gb, ri, J->support, bj, {
        float tdist = f_d2(ri, J->B->pos + 3 * bj);
        if (tdist < s2) {
            real wibj = wendland_w(rsqrt_((real)tdist), h);
            flt = flt + ((real)J->B->m[bj] / (real)J->B->rho[bj]) * wibj;
        }
    });
    J->out[i] = flt;
}

/* Kernel_density_sph, kernel/KERNEL_rho.py:45-82 */
static void density_sph_body(void* c, int i) {
    sph_job* J = (sph_job*)c;
    const float* ri = J->P->pos + 3 * i;
    float s2 = J->support * J->support;
    real h = (real)J->h, rhoi = R(0);
    OGRID_FOR(&J->gs, ri, J->support, j, {
        float tdist = f_d2(ri, J->P->pos + 3 * j);
        if (tdist < s2) rhoi = rhoi + (real)J->P->m[j] * wendland_w(rsqrt_((real)tdist), h);
    });
    OGRID_FOR(&J->gb, ri, J->support, bj, {
        float tdist = f_d2(ri, J->B->pos + 3 * bj);
        if (tdist < s2) rhoi = rhoi + (real)J->B->m[bj] * wendland_w(rsqrt_((real)tdist), h);
    });
    J->out[i] = rhoi / (real)J->P->flt[i];
}

/* Kernel_density_bnd, kernel/KERNEL_rho.py:87-126 (subject is a wall particle) */
static void density_bnd_body(void* c, int bi) {
    sph_job* J = (sph_job*)c;
    const float* rbi = J->B->pos + 3 * bi;
    float s2 = J->support * J->support;
    real h = (real)J->h, rhobi = R(0);
    OGRID_FOR(&J->gs, rbi, J->support, j, {
        float tdist = f_d2(rbi, J->P->pos + 3 * j);
        if (tdist < s2) rhobi = rhobi + (real)J->P->m[j] * wendland_w(rsqrt_((real)tdist), h);
    });
    OGRID_FOR(&J->gb, rbi, J->support, bj, {
        float tdist = f_d2(rbi, J->B->pos + 3 * bj);
        if (tdist < s2) rhobi = rhobi + (real)J->B->m[bj] * wendland_w(rsqrt_((real)tdist), h);
    });
    J->out[bi] = rhobi;
}

static void job_init(sph_job* J, sphdem_sph_t* P, const sphdem_bnd_t* B, float support) {
    memset(J, 0, sizeof(*J));
    J->P = P;
    J->B = B;
    ogrid_build(&J->gs, P->pos, P->n, support);
    ogrid_build(&J->gb, B->pos, B->n, support);
}
static void job_free(sph_job* J) {
    ogrid_free(&J->gs);
    ogrid_free(&J->gb);
    free(J->out);
}

void oracle_shepard_sph(sphdem_sph_t* P, const sphdem_bnd_t* B, float support, float h) {
    sph_job J;
    job_init(&J, P, B, support);
    J.support = support;
    J.h = h;
    J.out = (real*)malloc(sizeof(real) * (size_t)(P->n + 1));
    par_for(P->n, shepard_body, &J);
    for (int i = 0; i < P->n; ++i) P->flt[i] = (float)J.out[i];
    job_free(&J);
}

void oracle_density_sph(sphdem_sph_t* P, const sphdem_bnd_t* B, float support, float h) {
    sph_job J;
    job_init(&J, P, B, support);
    J.support = support;
    J.h = h;
    J.out = (real*)malloc(sizeof(real) * (size_t)(P->n + 1));
    par_for(P->n, density_sph_body, &J);
    for (int i = 0; i < P->n; ++i) P->rho[i] = (float)J.out[i];
    job_free(&J);
}

void oracle_density_bnd(sphdem_sph_t* P, sphdem_bnd_t* B, float support, float h) {
    sph_job J;
    job_init(&J, P, B, support);
    J.support = support;
    J.h = h;
    J.out = (real*)malloc(sizeof(real) * (size_t)(B->n + 1));
    par_for(B->n, density_bnd_body, &J);
    for (int i = 0; i < B->n; ++i) B->rho[i] = (float)J.out[i];
    job_free(&J);
}

/* Tait EOS, kernel/KERNEL_pres.py:6-45 */
static real tait(real rho, real rho0, real c0, real gamma) {
    real B = rho0 * c0 * c0 / gamma;
    real q = rpow(rho / rho0, gamma) - R(1);
    return B * rmax(q, R(0));
}
void oracle_pres_sph(sphdem_sph_t* P, float rho0, float c0, float gamma) {
    for (int i = 0; i < P->n; ++i) P->pres[i] = (float)tait((real)P->rho[i], (real)rho0, (real)c0, (real)gamma);
}
void oracle_pres_bnd(sphdem_bnd_t* B, float rho0, float c0, float gamma) {
    for (int i = 0; i < B->n; ++i) B->pres[i] = (float)tait((real)B->rho[i], (real)rho0, (real)c0, (real)gamma);
}

/* Kernel_force_sph, kernel/KERNEL_force.py:7-71 */
static void force_body(void* c, int i) {
    sph_job* J = (sph_job*)c;
    const sphdem_sph_t* P = J->P;
    const sphdem_bnd_t* B = J->B;
    const float* rif = P->pos + 3 * i;
    float s2 = J->support * J->support;
    real h = (real)J->h, mu = (real)J->mu;
    v3 ri = ld3(P->pos, i), vi = ld3(P->vel, i);
    real rhoi = (real)P->rho[i], presi = (real)P->pres[i];
    v3 acci = V(0, 0, 0);
    OGRID_FOR(&J->gs, rif, J->support, j, {
        float tdist = f_d2(rif, P->pos + 3 * j);
        if (tdist > R2_MIN && tdist < s2) {
            v3 rij = vsub(ri, ld3(P->pos, j));
            real td = vdot(rij, rij);
            real r = rsqrt_(td);
            v3 dwij = vmul(wendland_dw(r, h), vdiv(rij, r));
            real rhoj = (real)P->rho[j], presj = (real)P->pres[j], mj = (real)P->m[j];
            acci = vsub(acci, vmul(mj * (presi / (rhoi * rhoi) + presj / (rhoj * rhoj)), dwij));
            real visc = R(2) * mu * vdot(rij, dwij) / (rhoi * rhoj * (td + R(0.01) * h * h));
            acci = vadd(acci, vmul(mj * visc, vsub(vi, ld3(P->vel, j))));
        }
    });
    OGRID_FOR(&J->gb, rif, J->support, bj, {
        float tdist = f_d2(rif, B->pos + 3 * bj);
        if (tdist > R2_MIN && tdist < s2) {
            v3 ribj = vsub(ri, ld3(B->pos, bj));
            real td = vdot(ribj, ribj);
            real r = rsqrt_(td);
            v3 dwibj = vmul(wendland_dw(r, h), vdiv(ribj, r));
            real rhobj = (real)B->rho[bj], presbj = (real)B->pres[bj], mbj = (real)B->m[bj];
            acci = vsub(acci, vmul(mbj * (presi / (rhoi * rhoi) + presbj / (rhobj * rhobj)), dwibj));
            real visc = R(2) * mu * vdot(ribj, dwibj) / (rhoi * rhobj * (td + R(0.01) * h * h));
            acci = vadd(acci, vmul(mbj * visc, vsub(vi, ld3(B->vel, bj))));
        }
    });
    acci = vadd(acci, V(0, 0, -(real)J->g));
    J->out[3 * i] = acci.x;
    J->out[3 * i + 1] = acci.y;
    J->out[3 * i + 2] = acci.z;
}

void oracle_force_sph(sphdem_sph_t* P, const sphdem_bnd_t* B, float support, float h, float mu, float g) {
    sph_job J;
    job_init(&J, P, B, support);
    J.support = support;
    J.h = h;
    J.mu = mu;
    J.g = g;
    J.out = (real*)malloc(sizeof(real) * 3 * (size_t)(P->n + 1));
    par_for(P->n, force_body, &J);
    for (int i = 0; i < 3 * P->n; ++i) P->acc[i] = (float)J.out[i];
    job_free(&J);
}

/* Kernel_step_sph, kernel/KERNEL_step.py:6-22 */
void oracle_step_sph(sphdem_sph_t* P, float dt) {
    for (int i = 0; i < P->n; ++i) {
        v3 vel = vadd(ld3(P->vel, i), vmul((real)dt, ld3(P->acc, i)));
        st3(P->vel, i, vel);
        v3 vf = ld3(P->vel, i); /* the stored (float) velocity advances pos */
        st3(P->pos, i, vadd(ld3(P->pos, i), vmul((real)dt, vf)));
    }
}

/* ------------------------------------------------------------------------ */
/* DEM contacts                                                              */
/* ------------------------------------------------------------------------ */
/* DEM_contact, kernel/KERNEL_DEM_force.py:25-74 */
static void dem_contact(v3 normal, real overlap, real radius_a, real radius_b, v3 vel_a, v3 vel_b,
                        v3 omega_a, v3 omega_b, v3 tangent, real K, real eta, real mu, real dt,
                        v3* force, v3* displacement, v3* torque) {
    v3 rc_a = vmul(radius_a - R(0.5) * overlap, normal);
    v3 rc_b = vmul(-(radius_b - R(0.5) * overlap), normal);
    v3 urel = vsub(vsub(vadd(vel_b, vcross(omega_b, rc_b)), vel_a), vcross(omega_a, rc_a));
    v3 un = vmul(vdot(urel, normal), normal);
    v3 us = vsub(urel, un);
    v3 disp = vadd(tangent, vmul(dt, us));
    v3 direction = vdiv(us, vlen(us) + R(1.0e-20));
    v3 fn = vadd(vmul(-K * overlap, normal), vmul(eta, un));
    v3 fss = vadd(vmul(K, disp), vmul(eta, us));
    v3 fsf = vmul(mu * K * overlap, direction);
    v3 fs = fss;
    if (vlen(fss) >= vlen(fsf))
        fs = V(rsign(fss.x) * rabs(fsf.x), rsign(fss.y) * rabs(fsf.y), rsign(fss.z) * rabs(fsf.z));
    *force = vadd(fn, fs);
    *displacement = disp;
    *torque = vcross(rc_a, fs);
}

static int cmp_int(const void* a, const void* b) {
    int x = *(const int*)a, y = *(const int*)b;
    return (x > y) - (x < y);
}

typedef struct {
    sphdem_dem_t* D;
    const sphdem_dembnd_t* W;
    ogrid gd;
    int old_side;
    float radius_max, g, dt;
    int32_t* count;
    real* out; /* force/torque per subject (6) */
} dem_job;

/* Kernel_count_dem_contacts, kernel/KERNEL_DEM_force.py:9-22 */
static void count_dem_body(void* c, int a) {
    dem_job* J = (dem_job*)c;
    const sphdem_dem_t* D = J->D;
    const float* ra = D->pos + 3 * a;
    int count = 0;
    OGRID_FOR(&J->gd, ra, (double)(D->radius[a] + J->radius_max), b, {
        if (b != a) {
            float distance = f_len(D->pos + 3 * b, ra);
            if (D->radius[a] + D->radius[b] - distance > 0.0f) count = count + 1;
        }
    });
    J->count[a] = count;
}

/* Old-row history lookup by stable id (KERNEL_DEM_force.py:111-117). */
static v3 history_lookup(const sphdem_csr_t* old, int a, int b) {
    v3 t = V(0, 0, 0);
    for (int k = old->offset[a]; k < old->offset[a + 1]; ++k)
        if (old->id[k] == b) t = ld3(old->tang, k);
    return t;
}

/* Kernel_force_dem, kernel/KERNEL_DEM_force.py:77-135 */
static void force_dem_body(void* c, int a) {
    dem_job* J = (dem_job*)c;
    sphdem_dem_t* D = J->D;
    const sphdem_csr_t* old = &D->csr_dem[J->old_side];
    sphdem_csr_t* nw = &D->csr_dem[1 - J->old_side];
    const float* raf = D->pos + 3 * a;
    v3 ra = ld3(D->pos, a);
    v3 force = V(0, 0, -(real)D->m[a] * (real)J->g);
    v3 torque = V(0, 0, 0);
    int output_index = nw->offset[a];
    int cap = nw->offset[a + 1] - nw->offset[a];
    int* ids = (int*)malloc(sizeof(int) * (size_t)(cap > 0 ? cap : 1));
    int m = 0;
    OGRID_FOR(&J->gd, raf, (double)(D->radius[a] + J->radius_max), b, {
        if (b != a) {
            float dist = f_len(D->pos + 3 * b, raf);
            if (D->radius[a] + D->radius[b] - dist > 0.0f && m < cap) ids[m++] = b;
        }
    });
    qsort(ids, (size_t)m, sizeof(int), cmp_int);
    for (int k = 0; k < m; ++k) {
        int b = ids[k];
        v3 rab = vsub(ld3(D->pos, b), ra);
        real dist = vlen(rab);
        real overlap = (real)D->radius[a] + (real)D->radius[b] - dist;
        v3 tangent = history_lookup(old, a, b);
        v3 normal = V(1, 0, 0);
        if (a > b) normal = vneg(normal);
        if (dist > R(1.0e-12)) normal = vdiv(rab, dist);
        v3 fab, disp, tq;
        dem_contact(normal, overlap, (real)D->radius[a], (real)D->radius[b], ld3(D->vel, a), ld3(D->vel, b),
                    ld3(D->omega, a), ld3(D->omega, b), tangent, (real)D->K[a], (real)D->eta[a],
                    (real)D->mu[a], (real)J->dt, &fab, &disp, &tq);
        force = vadd(force, fab);
        torque = vadd(torque, tq);
        nw->id[output_index] = b;
        st3(nw->tang, output_index, disp);
        output_index = output_index + 1;
    }
    free(ids);
    J->out[6 * a + 0] = force.x;
    J->out[6 * a + 1] = force.y;
    J->out[6 * a + 2] = force.z;
    J->out[6 * a + 3] = torque.x;
    J->out[6 * a + 4] = torque.y;
    J->out[6 * a + 5] = torque.z;
}

/* Count + exclusive scan + fill of the DEM-DEM CSR (source/Simulation.py:142-165).
 * Writes side 1-old_side; the caller swaps.  Returns E, or -1 if E exceeds the
 * new side's capacity (nothing is filled then). */
int64_t oracle_force_dem(sphdem_dem_t* D, int old_side, float radius_max, float g, float dt) {
    dem_job J;
    memset(&J, 0, sizeof(J));
    J.D = D;
    J.old_side = old_side;
    J.radius_max = radius_max;
    J.g = g;
    J.dt = dt;
    int n = D->n;
    ogrid_build(&J.gd, D->pos, n, radius_max > 0 ? 2.0 * radius_max : 1.0);
    J.count = (int32_t*)calloc((size_t)n + 1, sizeof(int32_t));
    par_for(n, count_dem_body, &J);
    sphdem_csr_t* nw = &D->csr_dem[1 - old_side];
    int64_t total = 0;
    for (int a = 0; a < n; ++a) {
        nw->offset[a] = (int32_t)total;
        total += J.count[a];
    }
    nw->offset[n] = (int32_t)total;
    if (total > nw->capacity) {
        ogrid_free(&J.gd);
        free(J.count);
        return -1;
    }
    J.out = (real*)malloc(sizeof(real) * 6 * (size_t)(n + 1));
    par_for(n, force_dem_body, &J);
    for (int a = 0; a < n; ++a) {
        st3(D->force, a, V(J.out[6 * a], J.out[6 * a + 1], J.out[6 * a + 2]));
        st3(D->torque, a, V(J.out[6 * a + 3], J.out[6 * a + 4], J.out[6 * a + 5]));
    }
    ogrid_free(&J.gd);
    free(J.count);
    free(J.out);
    return total;
}

typedef struct {
    sphdem_dem_t* D;
    const sphdem_dembnd_t* W;
    ogrid gw;
    int old_side;
    float radius_max, dt;
    int32_t* count;
    real* out;
} bc_job;

/* Kernel_count_bnd_contacts, kernel/KERNEL_DEM_BC.py:10-24 */
static void count_bnd_body(void* c, int a) {
    bc_job* J = (bc_job*)c;
    const float* ra = J->D->pos + 3 * a;
    int count = 0;
    OGRID_FOR(&J->gw, ra, (double)(J->D->radius[a] + J->radius_max), dbj, {
        float distance = f_len(J->W->pos + 3 * dbj, ra);
        if (J->D->radius[a] + J->W->radius[dbj] - distance > 0.0f) count = count + 1;
    });
    J->count[a] = count;
}

/* Kernel_bc_dem, kernel/KERNEL_DEM_BC.py:27-84 */
static void bc_body(void* c, int a) {
    bc_job* J = (bc_job*)c;
    sphdem_dem_t* D = J->D;
    const sphdem_dembnd_t* W = J->W;
    const sphdem_csr_t* old = &D->csr_bnd[J->old_side];
    sphdem_csr_t* nw = &D->csr_bnd[1 - J->old_side];
    const float* raf = D->pos + 3 * a;
    v3 ra = ld3(D->pos, a);
    v3 force = V(0, 0, 0), torque = V(0, 0, 0);
    int output_index = nw->offset[a];
    int cap = nw->offset[a + 1] - nw->offset[a];
    int* ids = (int*)malloc(sizeof(int) * (size_t)(cap > 0 ? cap : 1));
    int m = 0;
    OGRID_FOR(&J->gw, raf, (double)(D->radius[a] + J->radius_max), dbj, {
        float dist = f_len(W->pos + 3 * dbj, raf);
        if (D->radius[a] + W->radius[dbj] - dist > 0.0f && m < cap) ids[m++] = dbj;
    });
    qsort(ids, (size_t)m, sizeof(int), cmp_int);
    for (int k = 0; k < m; ++k) {
        int dbj = ids[k];
        v3 radb = vsub(ld3(W->pos, dbj), ra);
        real dist = vlen(radb);
        real overlap = (real)D->radius[a] + (real)W->radius[dbj] - dist;
        v3 tangent = history_lookup(old, a, dbj);
        v3 normal = V(0, 0, -1);
        if (dist > R(1.0e-12)) normal = vdiv(radb, dist);
        v3 f, disp, tq;
        dem_contact(normal, overlap, (real)D->radius[a], (real)W->radius[dbj], ld3(D->vel, a),
                    ld3(W->vel, dbj), ld3(D->omega, a), ld3(W->omega, dbj), tangent, (real)D->K[a],
                    (real)D->eta[a], (real)D->mu[a], (real)J->dt, &f, &disp, &tq);
        force = vadd(force, f);
        torque = vadd(torque, tq);
        nw->id[output_index] = dbj;
        st3(nw->tang, output_index, disp);
        output_index = output_index + 1;
    }
    free(ids);
    v3 F = vadd(ld3(D->force, a), force), T = vadd(ld3(D->torque, a), torque);
    J->out[6 * a + 0] = F.x;
    J->out[6 * a + 1] = F.y;
    J->out[6 * a + 2] = F.z;
    J->out[6 * a + 3] = T.x;
    J->out[6 * a + 4] = T.y;
    J->out[6 * a + 5] = T.z;
}

/* Count + scan + fill of the DEM-wall CSR (source/Simulation.py:175-197). */
int64_t oracle_bc_dem(sphdem_dem_t* D, const sphdem_dembnd_t* W, int old_side, float radius_max, float dt) {
    bc_job J;
    memset(&J, 0, sizeof(J));
    J.D = D;
    J.W = W;
    J.old_side = old_side;
    J.radius_max = radius_max;
    J.dt = dt;
    int n = D->n;
    double cell = 2.0 * (double)radius_max;
    if (!(cell > 0)) cell = 1.0;
    ogrid_build(&J.gw, W->pos, W->n, cell);
    J.count = (int32_t*)calloc((size_t)n + 1, sizeof(int32_t));
    par_for(n, count_bnd_body, &J);
    sphdem_csr_t* nw = &D->csr_bnd[1 - old_side];
    int64_t total = 0;
    for (int a = 0; a < n; ++a) {
        nw->offset[a] = (int32_t)total;
        total += J.count[a];
    }
    nw->offset[n] = (int32_t)total;
    if (total > nw->capacity) {
        ogrid_free(&J.gw);
        free(J.count);
        return -1;
    }
    J.out = (real*)malloc(sizeof(real) * 6 * (size_t)(n + 1));
    par_for(n, bc_body, &J);
    for (int a = 0; a < n; ++a) {
        st3(D->force, a, V(J.out[6 * a], J.out[6 * a + 1], J.out[6 * a + 2]));
        st3(D->torque, a, V(J.out[6 * a + 3], J.out[6 * a + 4], J.out[6 * a + 5]));
    }
    ogrid_free(&J.gw);
    free(J.count);
    free(J.out);
    return total;
}

/* Kernel_step_dem, kernel/KERNEL_DEM_step.py:6-30 */
void oracle_step_dem(sphdem_dem_t* D, float dt) {
    for (int a = 0; a < D->n; ++a) {
        v3 acc = vdiv(ld3(D->force, a), (real)D->m[a]);
        v3 vel = vadd(ld3(D->vel, a), vmul((real)dt, acc));
        st3(D->acc, a, acc);
        st3(D->vel, a, vel);
        v3 vf = ld3(D->vel, a);
        st3(D->pos, a, vadd(ld3(D->pos, a), vmul((real)dt, vf)));
        v3 w = vadd(ld3(D->omega, a), vmul((real)dt, vdiv(ld3(D->torque, a), (real)D->inertia[a])));
        st3(D->omega, a, w);
    }
}

/* ------------------------------------------------------------------------ */
/* SPH-DEM coupling                                                          */
/* ------------------------------------------------------------------------ */
typedef struct {
    sphdem_sph_t* P;
    const sphdem_bnd_t* B;
    sphdem_dem_t* D;
    ogrid gs_sup, gs_sph, gb_sph, gd, gs_big;
    float support, h, sph_support, sph_h, eps_min, eps_max, mu, dt;
    real* out;
} cpl_job;

/* Kernel_prep_sphdem, kernel/KERNEL_SPHDEM_interaction.py:43-115 */
static void prep_body(void* c, int i) {
    cpl_job* J = (cpl_job*)c;
    const sphdem_sph_t* P = J->P;
    const sphdem_bnd_t* B = J->B;
    const sphdem_dem_t* D = J->D;
    const float* rif = P->pos + 3 * i;
    v3 ri = ld3(P->pos, i);
    real h = (real)J->h;
    real flt = R(0), solid = R(0);
    v3 pgf = V(0, 0, 0);
    if (J->h > 0.0f) {
        OGRID_FOR(&J->gs_sup, rif, J->support, j, {
            float distf = f_len(rif, P->pos + 3 * j);
            if (distf < J->support) {
                real dist = vlen(vsub(ri, ld3(P->pos, j)));
                flt = flt + (real)P->m[j] / (real)P->rho[j] * wendland_w(dist, h);
            }
        });
    }
    OGRID_FOR(&J->gd, rif, J->support, b, {
        float hbf = D->h[b];
        float distf = f_len(rif, D->pos + 3 * b);
        if (distf < 2.0f * hbf) {
            real hb = (real)hbf;
            real dist = vlen(vsub(ri, ld3(D->pos, b)));
            real local_flt = flt;
            if (J->h <= 0.0f) {
                local_flt = R(0);
                OGRID_FOR(&J->gs_big, rif, 2.0f * hbf, j, {
                    float fdf = f_len(rif, P->pos + 3 * j);
                    if (fdf < 2.0f * hbf) {
                        real fd = vlen(vsub(ri, ld3(P->pos, j)));
                        local_flt = local_flt + (real)P->m[j] / (real)P->rho[j] * wendland_w(fd, hb);
                    }
                });
            }
            solid = solid + (real)D->volume[b] * wendland_w(dist, hb) / (local_flt + R(1.0e-20));
        }
    });
    float ss2 = J->sph_support * J->sph_support;
    real sh = (real)J->sph_h, presi = (real)P->pres[i];
    OGRID_FOR(&J->gs_sph, rif, J->sph_support, j, {
        float r2 = f_d2(rif, P->pos + 3 * j);
        if (r2 > R2_MIN && r2 < ss2) {
            v3 rij = vsub(ri, ld3(P->pos, j));
            real dist = rsqrt_(vdot(rij, rij));
            v3 dwij = vdiv(vmul(wendland_dw(dist, sh), rij), dist);
            pgf = vsub(pgf, vmul((real)P->m[j] / (real)P->rho[j] * ((real)P->pres[j] - presi), dwij));
        }
    });
    OGRID_FOR(&J->gb_sph, rif, J->sph_support, bj, {
        float r2 = f_d2(rif, B->pos + 3 * bj);
        if (r2 > R2_MIN && r2 < ss2) {
            v3 ribj = vsub(ri, ld3(B->pos, bj));
            real dist = rsqrt_(vdot(ribj, ribj));
            v3 dwibj = vdiv(vmul(wendland_dw(dist, sh), ribj), dist);
            pgf = vsub(pgf, vmul((real)B->m[bj] / (real)B->rho[bj] * ((real)B->pres[bj] - presi), dwibj));
        }
    });
    J->out[4 * i] = rclamp(R(1) - solid, (real)J->eps_min, (real)J->eps_max);
    J->out[4 * i + 1] = pgf.x;
    J->out[4 * i + 2] = pgf.y;
    J->out[4 * i + 3] = pgf.z;
}

static float max_h(const sphdem_dem_t* D) {
    float m = 0.0f;
    for (int b = 0; b < D->n; ++b)
        if (D->h[b] > m) m = D->h[b];
    return m;
}

void oracle_prep_sphdem(sphdem_sph_t* P, const sphdem_bnd_t* B, sphdem_dem_t* D, float support, float h,
                        float sph_support, float sph_h, float eps_min, float eps_max) {
    cpl_job J;
    memset(&J, 0, sizeof(J));
    J.P = P;
    J.B = B;
    J.D = D;
    J.support = support;
    J.h = h;
    J.sph_support = sph_support;
    J.sph_h = sph_h;
    J.eps_min = eps_min;
    J.eps_max = eps_max;
    /* the fluid grid has the SPH support as cell width, as the reference's
       grid_sph (main.py:85); wider queries just visit more cells */
    ogrid_build(&J.gs_sup, P->pos, P->n, sph_support);
    ogrid_build(&J.gs_sph, P->pos, P->n, sph_support);
    ogrid_build(&J.gb_sph, B->pos, B->n, sph_support);
    ogrid_build(&J.gd, D->pos, D->n, support > 0 ? support : 1.0);
    ogrid_build(&J.gs_big, P->pos, P->n, sph_support);
    J.out = (real*)malloc(sizeof(real) * 4 * (size_t)(P->n + 1));
    par_for(P->n, prep_body, &J);
    for (int i = 0; i < P->n; ++i) {
        P->porosity[i] = (float)J.out[4 * i];
        st3(P->pgf, i, V(J.out[4 * i + 1], J.out[4 * i + 2], J.out[4 * i + 3]));
    }
    ogrid_free(&J.gs_sup);
    ogrid_free(&J.gs_sph);
    ogrid_free(&J.gb_sph);
    ogrid_free(&J.gd);
    ogrid_free(&J.gs_big);
    free(J.out);
}

/* Kernel_interaction_dem, kernel/KERNEL_SPHDEM_interaction.py:118-187 */
static void interaction_dem_body(void* c, int a) {
    cpl_job* J = (cpl_job*)c;
    const sphdem_sph_t* P = J->P;
    const sphdem_dem_t* D = J->D;
    const float* raf = D->pos + 3 * a;
    v3 ra = ld3(D->pos, a);
    real h = (real)D->h[a];
    float supportf = 2.0f * D->h[a];
    real flt = R(0), solid = R(0), rho_f = R(0);
    v3 vel_f = V(0, 0, 0), pgf = V(0, 0, 0);
    OGRID_FOR(&J->gs_big, raf, supportf, j, {
        float distf = f_len(raf, P->pos + 3 * j);
        if (distf < supportf) {
            real dist = vlen(vsub(ra, ld3(P->pos, j)));
            real Vw = (real)P->m[j] / (real)P->rho[j] * wendland_w(dist, h);
            flt = flt + Vw;
            rho_f = rho_f + (real)P->rho[j] * Vw;
            vel_f = vadd(vel_f, vmul(Vw, ld3(P->vel, j)));
            pgf = vadd(pgf, vmul(Vw, ld3(P->pgf, j)));
        }
    });
    OGRID_FOR(&J->gd, raf, supportf, b, {
        float distf = f_len(raf, D->pos + 3 * b);
        if (distf < supportf) {
            real dist = vlen(vsub(ra, ld3(D->pos, b)));
            solid = solid + (real)D->volume[b] * wendland_w(dist, h);
        }
    });
    real* o = J->out + 12 * a;
    /* o: flt_s, porosity, drag xyz, pressure_force xyz, force xyz, wet flag */
    o[0] = flt;
    o[1] = (real)J->eps_max;
    for (int k = 2; k < 8; ++k) o[k] = R(0);
    v3 F = ld3(D->force, a);
    if ((float)flt > 1.0e-12f) { /* FP32 test as the reference */
        real eps = rclamp(R(1) - solid / flt, (real)J->eps_min, (real)J->eps_max);
        v3 urel = vsub(vdiv(vel_f, flt), ld3(D->vel, a));
        real beta = drag_beta(eps, rho_f / flt, (real)J->mu, R(2) * (real)D->radius[a], vlen(urel));
        real coef = beta * (real)D->volume[a] / (real)D->m[a];
        v3 drag = vmul((real)D->m[a] * coef / (R(1) + (real)J->dt * coef), urel);
        v3 pressure_force = vdiv(vmul((real)D->m[a] / (real)D->rho[a], pgf), flt);
        o[1] = eps;
        o[2] = drag.x;
        o[3] = drag.y;
        o[4] = drag.z;
        o[5] = pressure_force.x;
        o[6] = pressure_force.y;
        o[7] = pressure_force.z;
        F = vadd(F, vadd(drag, pressure_force));
    }
    o[8] = F.x;
    o[9] = F.y;
    o[10] = F.z;
}

void oracle_interaction_dem(sphdem_sph_t* P, sphdem_dem_t* D, float mu, float eps_min, float eps_max, float dt) {
    cpl_job J;
    memset(&J, 0, sizeof(J));
    J.P = P;
    J.D = D;
    J.mu = mu;
    J.eps_min = eps_min;
    J.eps_max = eps_max;
    J.dt = dt;
    float hm = max_h(D);
    ogrid_build(&J.gs_big, P->pos, P->n, hm > 0 ? 2.0 * hm : 1.0);
    ogrid_build(&J.gd, D->pos, D->n, hm > 0 ? 2.0 * hm : 1.0);
    J.out = (real*)malloc(sizeof(real) * 12 * (size_t)(D->n + 1));
    par_for(D->n, interaction_dem_body, &J);
    for (int a = 0; a < D->n; ++a) {
        real* o = J.out + 12 * a;
        D->flt_s[a] = (float)o[0];
        D->porosity[a] = (float)o[1];
        st3(D->drag, a, V(o[2], o[3], o[4]));
        st3(D->pressure_force, a, V(o[5], o[6], o[7]));
        st3(D->force, a, V(o[8], o[9], o[10]));
    }
    ogrid_free(&J.gs_big);
    ogrid_free(&J.gd);
    free(J.out);
}

/* Kernel_interaction_sph, kernel/KERNEL_SPHDEM_interaction.py:190-226 */
static void interaction_sph_body(void* c, int i) {
    cpl_job* J = (cpl_job*)c;
    const sphdem_sph_t* P = J->P;
    const sphdem_dem_t* D = J->D;
    const float* rif = P->pos + 3 * i;
    v3 ri = ld3(P->pos, i);
    v3 force_density = V(0, 0, 0);
    OGRID_FOR(&J->gd, rif, J->support, b, {
        float distf = f_len(rif, D->pos + 3 * b);
        if (distf < 2.0f * D->h[b] && D->flt_s[b] > 1.0e-12f) {
            real dist = vlen(vsub(ri, ld3(D->pos, b)));
            force_density = vsub(force_density,
                                 vdiv(vmul(wendland_w(dist, (real)D->h[b]), ld3(D->drag, b)), (real)D->flt_s[b]));
        }
    });
    v3 acc = vdiv(force_density, (real)P->rho[i] * (real)P->porosity[i]);
    J->out[6 * i + 0] = acc.x;
    J->out[6 * i + 1] = acc.y;
    J->out[6 * i + 2] = acc.z;
    v3 tot = vadd(ld3(P->acc, i), acc);
    J->out[6 * i + 3] = tot.x;
    J->out[6 * i + 4] = tot.y;
    J->out[6 * i + 5] = tot.z;
}

void oracle_interaction_sph(sphdem_sph_t* P, sphdem_dem_t* D, float support) {
    cpl_job J;
    memset(&J, 0, sizeof(J));
    J.P = P;
    J.D = D;
    J.support = support;
    ogrid_build(&J.gd, D->pos, D->n, support > 0 ? support : 1.0);
    J.out = (real*)malloc(sizeof(real) * 6 * (size_t)(P->n + 1));
    par_for(P->n, interaction_sph_body, &J);
    for (int i = 0; i < P->n; ++i) {
        st3(P->acc_dem, i, V(J.out[6 * i], J.out[6 * i + 1], J.out[6 * i + 2]));
        st3(P->acc, i, V(J.out[6 * i + 3], J.out[6 * i + 4], J.out[6 * i + 5]));
    }
    ogrid_free(&J.gd);
    free(J.out);
}

/* ------------------------------------------------------------------------ */
/* whole steps, source/Simulation.py                                          */
/* ------------------------------------------------------------------------ */
/* SPH_OneStep, source/Simulation.py:17-99 */
void oracle_sph_onestep(sphdem_sph_t* P, sphdem_bnd_t* B, const sphdem_params_t* s, int step, int integrate) {
    int use_shepard = step == 0 || (s->shepard_step > 0 && step % s->shepard_step == 0);
    if (use_shepard) oracle_shepard_sph(P, B, s->support, s->h);
    oracle_density_sph(P, B, s->support, s->h);
    oracle_density_bnd(P, B, s->support, s->h);
    oracle_pres_sph(P, s->rho0, s->c0, s->gamma);
    oracle_pres_bnd(B, s->rho0, s->c0, s->gamma);
    oracle_force_sph(P, B, s->support, s->h, s->mu, s->g);
    if (integrate) oracle_step_sph(P, s->dt);
}

/* SPHDEM_OneStep, source/Simulation.py:102-221.  *old_dem / *old_bnd hold the
 * readable CSR sides and are swapped here.  Returns 0, or a positive code if a
 * contact CSR would overflow its capacity. */
int oracle_sphdem_onestep(sphdem_sph_t* P, sphdem_bnd_t* B, sphdem_dem_t* D, const sphdem_dembnd_t* W,
                          const sphdem_params_t* s, int step, int* old_dem, int* old_bnd) {
    oracle_sph_onestep(P, B, s, step, 0);
    if (oracle_force_dem(D, *old_dem, s->radius_max, s->g, s->dt) < 0) return SPHDEM_ERR_CSR_CAPACITY;
    *old_dem = 1 - *old_dem;
    if (oracle_bc_dem(D, W, *old_bnd, s->boundary_radius_max, s->dt) < 0) return SPHDEM_ERR_CSR_CAPACITY;
    *old_bnd = 1 - *old_bnd;
    oracle_prep_sphdem(P, B, D, 2.0f * s->h_max, s->h_uniform, s->support, s->h, s->porosity_min,
                       s->porosity_max);
    oracle_interaction_dem(P, D, s->mu, s->porosity_min, s->porosity_max, s->dt);
    oracle_interaction_sph(P, D, 2.0f * s->h_max);
    oracle_step_sph(P, s->dt);
    oracle_step_dem(D, s->dt);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* neighbour digests (SPHDEM_REL_* in sphdem.h)                              */
/* ------------------------------------------------------------------------ */
static inline uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

typedef struct {
    const sphdem_sph_t* P;
    const sphdem_bnd_t* B;
    const sphdem_dem_t* D;
    ogrid g;
    int rel;
    float radius;
    int32_t* count;
    uint64_t* hash;
} dig_job;

static void digest_body(void* c, int i) {
    dig_job* J = (dig_job*)c;
    const sphdem_sph_t* P = J->P;
    const sphdem_bnd_t* B = J->B;
    const sphdem_dem_t* D = J->D;
    const float* subj;
    const float* npos;
    switch (J->rel) {
        case SPHDEM_REL_BND_SPH_SUPPORT:
        case SPHDEM_REL_BND_BND_SUPPORT: subj = B->pos + 3 * i; break;
        case SPHDEM_REL_DEM_SPH_2H:
        case SPHDEM_REL_DEM_DEM_2H: subj = D->pos + 3 * i; break;
        default: subj = P->pos + 3 * i;
    }
    switch (J->rel) {
        case SPHDEM_REL_SPH_BND_SUPPORT:
        case SPHDEM_REL_BND_BND_SUPPORT:
        case SPHDEM_REL_SPH_BND_FORCE: npos = B->pos; break;
        case SPHDEM_REL_SPH_DEM_2H:
        case SPHDEM_REL_DEM_DEM_2H:
        case SPHDEM_REL_SPH_DEM_REACT: npos = D->pos; break;
        default: npos = P->pos;
    }
    float s = J->radius;
    if (J->rel == SPHDEM_REL_DEM_SPH_2H || J->rel == SPHDEM_REL_DEM_DEM_2H) s = 2.0f * D->h[i];
    float s2 = s * s;
    int32_t cnt = 0;
    uint64_t hs = 0;
    OGRID_FOR(&J->g, subj, s, j, {
        const float* pj = npos + 3 * j;
        int in = 0;
        switch (J->rel) {
            case SPHDEM_REL_SPH_SPH_SUPPORT:
            case SPHDEM_REL_SPH_BND_SUPPORT:
            case SPHDEM_REL_BND_SPH_SUPPORT:
            case SPHDEM_REL_BND_BND_SUPPORT: in = f_d2(subj, pj) < s2; break;
            case SPHDEM_REL_SPH_SPH_FORCE:
            case SPHDEM_REL_SPH_BND_FORCE: {
                float d2 = f_d2(subj, pj);
                in = d2 > R2_MIN && d2 < s2;
                break;
            }
            case SPHDEM_REL_SPH_SPH_LEN:
            case SPHDEM_REL_DEM_SPH_2H:
            case SPHDEM_REL_DEM_DEM_2H: in = f_len(subj, pj) < s; break;
            case SPHDEM_REL_SPH_DEM_2H: in = f_len(subj, pj) < 2.0f * D->h[j]; break;
            case SPHDEM_REL_SPH_DEM_REACT: in = f_len(subj, pj) < 2.0f * D->h[j] && D->flt_s[j] > 1.0e-12f; break;
        }
        if (in) {
            cnt++;
            hs += mix64((uint64_t)j);
        }
    });
    J->count[i] = cnt;
    J->hash[i] = hs;
}

int oracle_neighbour_digest(const sphdem_sph_t* P, const sphdem_bnd_t* B, const sphdem_dem_t* D, int rel,
                            float radius, int32_t* count, uint64_t* hash) {
    dig_job J;
    memset(&J, 0, sizeof(J));
    J.P = P;
    J.B = B;
    J.D = D;
    J.rel = rel;
    J.radius = radius;
    J.count = count;
    J.hash = hash;
    int nsub;
    const float* npos;
    int nn;
    double cell = radius > 0 ? radius : 1.0;
    switch (rel) {
        case SPHDEM_REL_BND_SPH_SUPPORT:
        case SPHDEM_REL_BND_BND_SUPPORT: nsub = B->n; break;
        case SPHDEM_REL_DEM_SPH_2H:
        case SPHDEM_REL_DEM_DEM_2H: nsub = D->n; break;
        default: nsub = P->n;
    }
    switch (rel) {
        case SPHDEM_REL_SPH_BND_SUPPORT:
        case SPHDEM_REL_BND_BND_SUPPORT:
        case SPHDEM_REL_SPH_BND_FORCE: npos = B->pos; nn = B->n; break;
        case SPHDEM_REL_SPH_DEM_2H:
        case SPHDEM_REL_DEM_DEM_2H:
        case SPHDEM_REL_SPH_DEM_REACT: npos = D->pos; nn = D->n; break;
        default: npos = P->pos; nn = P->n;
    }
    if (rel == SPHDEM_REL_DEM_SPH_2H || rel == SPHDEM_REL_DEM_DEM_2H) {
        float hm = max_h(D);
        cell = hm > 0 ? 2.0 * hm : 1.0;
    }
    if (rel < 0 || rel >= SPHDEM_REL_COUNT) return SPHDEM_ERR_INVALID;
    ogrid_build(&J.g, npos, nn, cell);
    par_for(nsub, digest_body, &J);
    ogrid_free(&J.g);
    return 0;
}

/* FP64 diagnostics (no reference counterpart): same definitions as the GPU's
 * sphdem_diagnostics, summed in double in index order. */
void oracle_diagnostics(const sphdem_sph_t* P, const sphdem_dem_t* D, float g, double* out) {
    for (int k = 0; k < 8; ++k) out[k] = 0.0;
    for (int i = 0; i < P->n; ++i) {
        double m = P->m[i], vx = P->vel[3 * i], vy = P->vel[3 * i + 1], vz = P->vel[3 * i + 2];
        out[0] += m;
        out[2] += m * vx;
        out[3] += m * vy;
        out[4] += m * vz;
        out[5] += 0.5 * m * (vx * vx + vy * vy + vz * vz);
        out[7] += m * (double)g * (double)P->pos[3 * i + 2];
    }
    if (D)
        for (int a = 0; a < D->n; ++a) {
            double m = D->m[a], vx = D->vel[3 * a], vy = D->vel[3 * a + 1], vz = D->vel[3 * a + 2];
            double wx = D->omega[3 * a], wy = D->omega[3 * a + 1], wz = D->omega[3 * a + 2];
            out[1] += m;
            out[2] += m * vx;
            out[3] += m * vy;
            out[4] += m * vz;
            out[5] += 0.5 * m * (vx * vx + vy * vy + vz * vz);
            out[6] += 0.5 * (double)D->inertia[a] * (wx * wx + wy * wy + wz * wz);
            out[7] += m * (double)g * (double)D->pos[3 * a + 2];
        }
}

int oracle_real_bytes(void) { return (int)sizeof(real); }
