// coupling.cu -- SPH-DEM exchange (kernel/KERNEL_SPHDEM_interaction.py).
//
//   k_near            porosity, first pass of Kernel_prep_sphdem (:43-115): each
//                     fluid particle looks for a DEM within 2 h_b.  With none,
//                     solid = 0 and porosity = clamp(1, min, max) whatever the
//                     fluid normaliser is, so that normaliser (a sum over the
//                     whole coupling support, ~2k-137k neighbours) is skipped;
//                     the result is identical.  Others are listed.
//   k_porosity_near   one warp per listed particle: the fluid normaliser as a
//                     warp-strided sum over the coupling support, then the solid
//                     fraction over the DEM neighbours.
//   k_interaction_dem one CTA per DEM (Kernel_interaction_dem, :118-187): block-
//                     wide volume-weighted sums of rho, u and -grad p, solid
//                     fraction, semi-implicit Ergun / Wen-Yu drag, buoyancy.
//   k_react           Kernel_interaction_sph (:190-226) fused with
//                     Kernel_step_sph (kernel/KERNEL_step.py:6-22).
// Sums use fixed lane/warp orders, so every result is deterministic.
#include "common.cuh"

namespace sd {

namespace {

// DEM_drag_beta (kernel/KERNEL_SPHDEM_interaction.py:11-40).
__device__ float drag_beta(float eps, float rho, float mu, float diameter, float speed) {
    float beta = 0.0f;
    const float reynolds = rho * diameter * speed / (mu + 1.0e-20f);
    if (eps <= 0.8f) {
        beta = 150.0f * (1.0f - eps) / eps * mu / (diameter * diameter) + 1.75f * rho * speed / diameter;
    } else {
        float cd_speed = 0.44f * speed;
        if (reynolds <= 1000.0f) cd_speed = 24.0f * mu / (rho * diameter) * (1.0f + 0.15f * powf(reynolds, 0.687f));
        beta = 0.75f * cd_speed * rho / diameter * powf(eps, -1.65f);
    }
    return beta;
}

__global__ void k_drag_beta(const float* eps, const float* rho, const float* mu, const float* d, const float* speed,
                            int n, float* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = drag_beta(eps[i], rho[i], mu[i], d[i], speed[i]);
}

struct CplArgs {
    Geo gs, gd;
    const float4* __restrict__ f_posv;  // x, y, z, m/rho
    const float4* __restrict__ f_vel;
    const float4* __restrict__ f_pgf;   // pgf, rho
    const float4* __restrict__ aux;     // per DEM: 1/h, cw, sqrt bound of 2h, 2h
    sphdem_sph_t P;
    sphdem_dem_t D;
    int* near_list;
    sphdem_ctl_t* ctl;
    float support, rq, t_support;  // coupling query radius (2 h_max), its padded and sqrt bounds
    float h;                       // uniform DEM h, or <= 0
    Kern kern;                     // Wendland of the uniform h
    float eps_min, eps_max, mu, dt;
};

__device__ __forceinline__ float w_aux(const float4& aux, float dist) {
    const float q = dist * aux.x;
    const float u = 1.0f - 0.5f * q;
    const float u2 = u * u;
    return q < 2.0f ? aux.y * u2 * u2 * (1.0f + 2.0f * q) : 0.0f;
}

// Porosity pass 1: dry particles get clamp(1); the rest are listed.
__global__ void k_near(CplArgs a) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= a.P.n) return;
    const int o = a.gs.order[k];
    const float4 p = a.f_posv[k];
    const int inst = inst_of(a.gs, o);
    bool near = false;
    if (a.D.n > 0) {
        const Win w = window(a.gd, p.x, p.y, p.z, a.rq);
        for_each_range(a.gd, w, inst, [&](int s, int e) {
            for (int j = s; j < e && !near; ++j) {
                const int b = a.gd.order[j];
                const float3 pb = ld3(a.D.pos, b);
                const D2 r = d2_exact(p.x, p.y, p.z, pb.x, pb.y, pb.z);
                if (r.d2 < a.aux[b].z) near = true;  // len < 2 h_b, :87-88
            }
        });
    }
    if (near)
        a.near_list[atomicAdd(&a.ctl->n_near, 1)] = k;
    else
        a.P.porosity[o] = fminf(fmaxf(1.0f, a.eps_min), a.eps_max);
}

// Warp-strided fluid sum sum_j V_j W(r_ij) over len(r_ij) < 2h (bound t2).
__device__ __forceinline__ float warp_fluid_sum(const CplArgs& a, int inst, float px, float py, float pz, float rq,
                                                float t2, const float4& kaux) {
    const int lane = threadIdx.x & 31;
    float acc = 0.0f;
    const Win w = window(a.gs, px, py, pz, rq);
    for_each_range(a.gs, w, inst, [&](int s, int e) {
        for (int j = s + lane; j < e; j += 32) {
            const float4 q = a.f_posv[j];
            const D2 r = d2_exact(px, py, pz, q.x, q.y, q.z);
            if (r.d2 < t2) acc += q.w * w_aux(kaux, fast_sqrt(r.d2));
        }
    });
    return warp_sum(acc);
}

// Porosity pass 2: one warp per listed particle.
__global__ void __launch_bounds__(256) k_porosity_near(CplArgs a) {
    const int lane = threadIdx.x & 31;
    const int warps = gridDim.x * (blockDim.x >> 5);
    const int n_near = a.ctl->n_near;
    const float4 kuni = make_float4(a.kern.inv_h, a.kern.cw, a.t_support, a.support);
    for (int idx = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); idx < n_near; idx += warps) {
        const int k = a.near_list[idx];
        const int o = a.gs.order[k];
        const float4 p = a.f_posv[k];
        const int inst = inst_of(a.gs, o);
        float flt = 0.0f;
        if (a.h > 0.0f) flt = warp_fluid_sum(a, inst, p.x, p.y, p.z, a.rq, a.t_support, kuni);
        float solid = 0.0f;
        const Win w = window(a.gd, p.x, p.y, p.z, a.rq);
        for_each_range(a.gd, w, inst, [&](int s, int e) {
            for (int j = s; j < e; ++j) {  // warp-uniform loop over DEM candidates
                const int b = a.gd.order[j];
                const float3 pb = ld3(a.D.pos, b);
                const D2 r = d2_exact(p.x, p.y, p.z, pb.x, pb.y, pb.z);
                const float4 ab = a.aux[b];
                if (r.d2 < ab.z) {
                    float local_flt = flt;
                    if (a.h <= 0.0f)
                        local_flt = warp_fluid_sum(a, inst, p.x, p.y, p.z, pad_radius(ab.w), ab.z, ab);
                    solid += a.D.volume[b] * w_aux(ab, fast_sqrt(r.d2)) / (local_flt + 1.0e-20f);
                }
            }
        });
        if (lane == 0) a.P.porosity[o] = fminf(fmaxf(1.0f - solid, a.eps_min), a.eps_max);
    }
}

constexpr int kIdThreads = 256;

// Kernel_interaction_dem: one CTA per DEM a.
__global__ void __launch_bounds__(kIdThreads) k_interaction_dem(CplArgs a) {
    __shared__ float red[kIdThreads / 32][8];
    const int am = blockIdx.x;
    const float3 pa = ld3(a.D.pos, am);
    const float4 aux = a.aux[am];  // 1/h, cw, bound(2h), 2h
    const int inst = inst_of(a.gd, am);
    float s[8] = {0, 0, 0, 0, 0, 0, 0, 0};  // flt, rho_f, vel_f xyz, pgf xyz
    if (a.P.n > 0) {
        const Win w = window(a.gs, pa.x, pa.y, pa.z, pad_radius(aux.w));
        for_each_range(a.gs, w, inst, [&](int rs, int re) {
            for (int j = rs + threadIdx.x; j < re; j += blockDim.x) {
                const float4 q = a.f_posv[j];
                const D2 r = d2_exact(pa.x, pa.y, pa.z, q.x, q.y, q.z);
                if (r.d2 < aux.z) {  // len < 2 h_a, :157-158
                    const float Vw = q.w * w_aux(aux, fast_sqrt(r.d2));
                    const float4 v = a.f_vel[j];
                    const float4 g = a.f_pgf[j];
                    s[0] += Vw;
                    s[1] += g.w * Vw;
                    s[2] += v.x * Vw;
                    s[3] += v.y * Vw;
                    s[4] += v.z * Vw;
                    s[5] += g.x * Vw;
                    s[6] += g.y * Vw;
                    s[7] += g.z * Vw;
                }
            }
        });
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        const float v = warp_sum(s[c]);
        if (lane == 0) red[wid][c] = v;
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    for (int c = 0; c < 8; ++c) {
        float t = 0.0f;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += red[k][c];
        s[c] = t;
    }
    // solid sum over DEM neighbours, a itself included (:165-168)
    float solid = 0.0f;
    const Win wd = window(a.gd, pa.x, pa.y, pa.z, pad_radius(aux.w));
    for_each_range(a.gd, wd, inst, [&](int rs, int re) {
        for (int j = rs; j < re; ++j) {
            const int b = a.gd.order[j];
            const float3 pb = ld3(a.D.pos, b);
            const D2 r = d2_exact(pa.x, pa.y, pa.z, pb.x, pb.y, pb.z);
            if (r.d2 < aux.z) solid += a.D.volume[b] * w_aux(aux, fast_sqrt(r.d2));
        }
    });
    const float flt = s[0];
    a.D.flt_s[am] = flt;
    float3 drag = make_float3(0.f, 0.f, 0.f), pf = make_float3(0.f, 0.f, 0.f);
    float por = a.eps_max;
    if (flt > 1.0e-12f) {
        const float iflt = 1.0f / flt;
        const float eps = fminf(fmaxf(1.0f - solid * iflt, a.eps_min), a.eps_max);
        const float3 va = ld3(a.D.vel, am);
        const float3 urel = make_float3(s[2] * iflt - va.x, s[3] * iflt - va.y, s[4] * iflt - va.z);
        const float speed = sqrtf(urel.x * urel.x + urel.y * urel.y + urel.z * urel.z);
        const float m = a.D.m[am];
        const float beta = drag_beta(eps, s[1] * iflt, a.mu, 2.0f * a.D.radius[am], speed);
        const float coef = beta * a.D.volume[am] / m;
        const float dc = m * coef / (1.0f + a.dt * coef);
        drag = make_float3(dc * urel.x, dc * urel.y, dc * urel.z);
        const float pc = m / a.D.rho[am] * iflt;
        pf = make_float3(pc * s[5], pc * s[6], pc * s[7]);
        por = eps;
        float3 F = ld3(a.D.force, am);
        st3(a.D.force, am, make_float3(F.x + (drag.x + pf.x), F.y + (drag.y + pf.y), F.z + (drag.z + pf.z)));
    }
    a.D.porosity[am] = por;
    st3(a.D.drag, am, drag);
    st3(a.D.pressure_force, am, pf);
}

// Kernel_interaction_sph (+ Kernel_step_sph when INTEGRATE), point order.
template <bool INTEGRATE>
__global__ void k_react(CplArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.P.n) return;
    const float3 pi = ld3(a.P.pos, i);
    float3 fd = make_float3(0.f, 0.f, 0.f);
    if (a.D.n > 0) {
        const int inst = inst_of(a.gs, i);
        const Win w = window(a.gd, pi.x, pi.y, pi.z, a.rq);
        for_each_range(a.gd, w, inst, [&](int s, int e) {
            for (int j = s; j < e; ++j) {
                const int b = a.gd.order[j];
                const float3 pb = ld3(a.D.pos, b);
                const D2 r = d2_exact(pi.x, pi.y, pi.z, pb.x, pb.y, pb.z);
                const float4 ab = a.aux[b];
                const float flt_s = a.D.flt_s[b];
                if (r.d2 < ab.z && flt_s > 1.0e-12f) {  // :220-221
                    const float c = w_aux(ab, fast_sqrt(r.d2)) / flt_s;
                    const float3 dr = ld3(a.D.drag, b);
                    fd.x -= dr.x * c;
                    fd.y -= dr.y * c;
                    fd.z -= dr.z * c;
                }
            }
        });
    }
    const float den = a.P.rho[i] * a.P.porosity[i];
    const float3 acc_dem = make_float3(fd.x / den, fd.y / den, fd.z / den);
    st3(a.P.acc_dem, i, acc_dem);
    float3 acc = ld3(a.P.acc, i);
    acc = make_float3(__fadd_rn(acc.x, acc_dem.x), __fadd_rn(acc.y, acc_dem.y), __fadd_rn(acc.z, acc_dem.z));
    st3(a.P.acc, i, acc);
    if (INTEGRATE) euler_store(a.P.pos, a.P.vel, i, acc, a.dt);
}

CplArgs make_args(const sphdem_ctx_t* c, float support, float h) {
    CplArgs a;
    a.gs = make_geo(c->grid_sph);
    a.gd = make_geo(c->grid_dem);
    a.f_posv = (const float4*)c->work.f_posv;
    a.f_vel = (const float4*)c->work.f_vel;
    a.f_pgf = (const float4*)c->work.f_pgf;
    a.aux = (const float4*)c->work.dem_aux;
    a.P = c->sph;
    a.D = c->dem;
    a.near_list = c->work.near_list;
    a.ctl = c->ctl;
    a.support = support;
    a.rq = pad_radius(support);
    a.t_support = sqrt_lt_bound(support);
    a.h = h;
    a.kern = make_kern(h > 0.0f ? h : 1.0f);
    a.eps_min = a.eps_max = 1.0f;
    a.mu = a.dt = 0.0f;
    return a;
}

}  // namespace

int run_porosity(const sphdem_ctx_t* c, float support, float h, float eps_min, float eps_max, cudaStream_t st) {
    const int n = c->sph.n;
    if (n <= 0) return SPHDEM_OK;
    CplArgs a = make_args(c, support, h);
    a.eps_min = eps_min;
    a.eps_max = eps_max;
    cudaError_t e = cudaMemsetAsync(&c->ctl->n_near, 0, sizeof(int), st);
    if (e != cudaSuccess) {
        set_error("porosity memset", e);
        return SPHDEM_ERR_CUDA;
    }
    k_near<<<blocks_for(n, 256), 256, 0, st>>>(a);
    if (c->dem.n > 0) {
        int dev = 0, sms = 148;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        int blocks = sms * 8;
        const int need = blocks_for(n, 8);
        if (need < blocks) blocks = need;
        k_porosity_near<<<blocks, 256, 0, st>>>(a);
    }
    return launch_status("porosity");
}

int run_interaction_dem(const sphdem_ctx_t* c, float mu, float eps_min, float eps_max, float dt, cudaStream_t st) {
    if (c->dem.n <= 0) return SPHDEM_OK;
    CplArgs a = make_args(c, 0.0f, 0.0f);
    a.mu = mu;
    a.eps_min = eps_min;
    a.eps_max = eps_max;
    a.dt = dt;
    k_interaction_dem<<<c->dem.n, kIdThreads, 0, st>>>(a);
    return launch_status("interaction_dem");
}

int run_react(const sphdem_ctx_t* c, float support, float dt, bool integrate, cudaStream_t st) {
    const int n = c->sph.n;
    if (n <= 0) return SPHDEM_OK;
    CplArgs a = make_args(c, support, 0.0f);
    a.dt = dt;
    if (integrate)
        k_react<true><<<blocks_for(n, 256), 256, 0, st>>>(a);
    else
        k_react<false><<<blocks_for(n, 256), 256, 0, st>>>(a);
    return launch_status("react");
}

int run_drag_beta(const float* eps, const float* rho, const float* mu, const float* d, const float* speed, int n,
                  float* out, cudaStream_t st) {
    if (n <= 0) return SPHDEM_OK;
    k_drag_beta<<<blocks_for(n, 256), 256, 0, st>>>(eps, rho, mu, d, speed, n, out);
    return launch_status("drag_beta");
}

}  // namespace sd
