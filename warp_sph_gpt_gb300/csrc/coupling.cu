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
//   k_interaction_dem one CTA per DEM (Kernel_interaction_dem, :118-187): its
//                     warps share the ball's columns; volume-weighted sums of
//                     rho, u and -grad p reduced over the CTA in fixed order,
//                     solid fraction, semi-implicit Ergun / Wen-Yu drag,
//                     buoyancy.
//   k_react           Kernel_interaction_sph (:190-226) fused with
//                     Kernel_step_sph (kernel/KERNEL_step.py:6-22).
// Sums use fixed lane/warp orders, so every result is deterministic.
#include "common.cuh"
#include "tma.cuh"

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
    pdl_wait();
    pdl_launch();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = drag_beta(eps[i], rho[i], mu[i], d[i], speed[i]);
}

struct CplArgs {
    Geo gs, gd;
    const float4* __restrict__ f_posv;  // x, y, z, m/rho
    const float4* __restrict__ f_vel;
    const float4* __restrict__ f_pgf;   // pgf, rho
    float4* f_posq;                     // x/h, y/h, z/h, m/rho (uniform h: written by k_near)
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

__device__ __forceinline__ float sqrt_approx(float x) {
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// V_j u^4 (1 + 2q) of one candidate (u = 1 - q/2), evaluated as the
// expanded polynomial  1 + s (-5/2 + q (5/2 + q (-15/16 + q/8))),  s = q^2,
// with s clamped to 4: one multiply fewer per candidate than the factored
// form, and the weight vanishes at q = 2 (every Horner step is exact there),
// so candidates beyond the ball add ~0 (|W| <= a few ulps of 1) and no
// membership branch or select is needed (warps walk 32 different candidates;
// a branch would diverge).  A pair whose membership the reference decides by
// its rounded length(r) < 2h lies, if near that boundary, within a few ulps
// of q = 2, where the weight is below 1e-6: the normaliser's value is the
// same to FP32 rounding (the neighbour sets themselves are checked with the
// exact predicate elsewhere).  The factor 21/(16 pi h^3) is applied by the
// caller once per sum.
__device__ __forceinline__ float wendland_poly(float s) {
    s = fminf(s, 4.0f);
    const float q = sqrt_approx(s);
    const float c = fmaf(fmaf(fmaf(0.125f, q, -0.9375f), q, 2.5f), q, -2.5f);
    return fmaf(c, s, 1.0f);
}

__device__ __forceinline__ float ball_weight(float px, float py, float pz, const float4& q, float ih2) {
    const float dx = px - q.x, dy = py - q.y, dz = pz - q.z;
    return q.w * wendland_poly(fmaf(dz, dz, fmaf(dy, dy, dx * dx)) * ih2);
}

// The same for coordinates already in units of h (p and q scaled by 1/h).
__device__ __forceinline__ float ball_weight_h(float px, float py, float pz, const float4& q) {
    const float dx = px - q.x, dy = py - q.y, dz = pz - q.z;
    return q.w * wendland_poly(fmaf(dz, dz, fmaf(dy, dy, dx * dx)));
}

// Porosity pass 1: dry particles get clamp(1); the rest are listed.  The list
// keeps slot order inside each block of 256 slots (ordered block compaction),
// so consecutive entries are neighbours in space.
__global__ void __launch_bounds__(256) k_near(CplArgs a) {
    pdl_wait();
    pdl_launch();
    __shared__ int warp_tot[8];
    __shared__ int base;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    bool near = false;
    int o = 0;
    if (k < a.P.n) {
        o = a.gs.order[k];
        const float4 p = a.f_posv[k];
        if (a.h > 0.0f && a.f_posq) {  // positions in units of the uniform coupling h
            const float ih = a.kern.inv_h;
            a.f_posq[k] = make_float4(p.x * ih, p.y * ih, p.z * ih, p.w);
        }
        const int inst = inst_of(a.gs, o);
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
    }
    int total;
    const int ex = block_exclusive_scan(near ? 1 : 0, warp_tot, total);
    if (threadIdx.x == 0) base = total ? atomicAdd(&a.ctl->n_near, total) : 0;
    __syncthreads();
    if (near)
        a.near_list[base + ex] = k;
    else if (k < a.P.n)
        a.P.porosity[o] = fminf(fmaxf(1.0f, a.eps_min), a.eps_max);
}

// Warp-strided fluid sum  sum_j V_j W(r_ij, h)  over len(r_ij) < 2h, where
// t2 is the exact sqrt bound of 2h and kaux = (1/h, 21/(16 pi h^3), ., .).
// Membership is exact (d2_below); for members r < 2h, so the Wendland
// cut-off test is not needed and 21/(16 pi h^3) is applied once at the end.
__device__ __forceinline__ float warp_fluid_sum(const CplArgs& a, int inst, float px, float py, float pz, float rq,
                                                float t2, const float4& kaux) {
    const int lane = threadIdx.x & 31;
    const float ih2 = kaux.x * kaux.x;
    float acc = 0.0f;
    warp_ranges_ball(a.gs, px, py, pz, rq, inst, [&](int s, int e) {
#pragma unroll 4
        for (int j = s + lane; j < e; j += 32) acc += ball_weight(px, py, pz, a.f_posv[j], ih2);
    });
    return warp_sum(acc) * kaux.y;
}

// Solid fraction of a listed particle: the DEM neighbours within 2 h_b, each
// V_b W(r, h_b) / normaliser (Kernel_prep_sphdem :89-108).  flt is the uniform
// normaliser: the lanes then take the DEM candidates of each range in turn
// (lane = offset in the range mod 32) and the terms are summed across the
// warp.  Without a uniform h each DEM in reach has its own (warp-wide) sum,
// so the warp walks the candidates together.
template <bool UNIFORM>
__device__ __forceinline__ float porosity_solid(const CplArgs& a, const float4& p, int inst, float flt) {
    float solid = 0.0f;
    const Win w = window(a.gd, p.x, p.y, p.z, a.rq);
    if (UNIFORM) {
        const int lane = threadIdx.x & 31;
        for_each_range(a.gd, w, inst, [&](int s, int e) {
            for (int j = s + lane; j < e; j += 32) {
                const int b = a.gd.order[j];
                const float3 pb = ld3(a.D.pos, b);
                const D2 r = d2_exact(p.x, p.y, p.z, pb.x, pb.y, pb.z);
                const float4 ab = a.aux[b];
                if (r.d2 < ab.z) solid += a.D.volume[b] * w_aux(ab, fast_sqrt(r.d2)) / (flt + 1.0e-20f);
            }
        });
        return warp_sum(solid);
    }
    for_each_range(a.gd, w, inst, [&](int s, int e) {
        for (int j = s; j < e; ++j) {  // warp-uniform loop over DEM candidates
            const int b = a.gd.order[j];
            const float3 pb = ld3(a.D.pos, b);
            const D2 r = d2_exact(p.x, p.y, p.z, pb.x, pb.y, pb.z);
            const float4 ab = a.aux[b];
            if (r.d2 < ab.z) {
                float local_flt = flt;
                if (!UNIFORM) local_flt = warp_fluid_sum(a, inst, p.x, p.y, p.z, pad_radius(ab.w), ab.z, ab);
                solid += a.D.volume[b] * w_aux(ab, fast_sqrt(r.d2)) / (local_flt + 1.0e-20f);
            }
        }
    });
    return solid;
}

// Porosity pass 2: one warp per listed particle.  UNIFORM: one DEM h for all
// spheres (the normaliser is one sum per particle); otherwise each DEM in
// reach has its own normaliser sum.  Warps take list entries from a shared
// counter (the work per entry varies with the fluid around it; a static
// split leaves SMs idle at the end), so the warps resident together work on
// consecutive entries (neighbours in space): they walk nearly the same
// candidates in the same column order and share them through L1.  Which warp
// takes an entry does not change its result.
template <bool UNIFORM>
__global__ void __launch_bounds__(256) k_porosity_near(CplArgs a) {
    pdl_wait();
    pdl_launch();
    const int lane = threadIdx.x & 31;
    const int n_near = a.ctl->n_near;
    for (;;) {
        int idx = 0;
        if (lane == 0) idx = atomicAdd(&a.ctl->near_next, 1);
        idx = __shfl_sync(0xffffffffu, idx, 0);
        if (idx >= n_near) break;
        const int k = a.near_list[idx];
        const int o = a.gs.order[k];
        const float4 p = a.f_posv[k];
        const int inst = inst_of(a.gs, o);
        float flt = 0.0f;
        if (UNIFORM) {
            // candidates from the scaled copy: the column walk uses world coordinates
            const float ih = a.kern.inv_h;
            const float sx = p.x * ih, sy = p.y * ih, sz = p.z * ih;
            float acc = 0.0f;
            warp_ranges_ball(a.gs, p.x, p.y, p.z, a.rq, inst, [&](int s, int e) {
#pragma unroll 4
                for (int j = s + lane; j < e; j += 32) acc += ball_weight_h(sx, sy, sz, a.f_posq[j]);
            });
            flt = warp_sum(acc) * a.kern.cw;
        }
        const float solid = porosity_solid<UNIFORM>(a, p, inst, flt);
        if (lane == 0) a.P.porosity[o] = fminf(fmaxf(1.0f - solid, a.eps_min), a.eps_max);
    }
}

// ---------------------------------------------------------------------------
// Porosity pass 2 for a uniform DEM h: shared-memory staged.  A CTA of 8 warps
// takes kGroup consecutive listed particles (kSubjPerWarp per warp; neighbours
// in space), trims the columns of their common query window to the ball
// around their bounding box, and streams the candidate ranges through two
// shared buffers: each buffer is packed with as many ranges (or range pieces)
// as fit, each piece one 1D TMA bulk copy (cp.async.bulk), all completing on
// the buffer's mbarrier; the next buffer fills while the current one is
// consumed.  Every staged candidate is tested against the warp's particles.
// The candidate in slot j is always handled by lane j % 32, in slot order, so
// each particle's sum does not depend on how particles were grouped or buffers
// packed.  (Measured slower than k_porosity_near on GB300 for the dam-break
// cases -- the sum is bound by FP32 issue, not by load latency -- so it is
// the second choice of the launch tuning.)
// ---------------------------------------------------------------------------
constexpr int kTileWarps = 8;
constexpr int kTileThreads = kTileWarps * 32;
constexpr int kSubjPerWarp = 1;
constexpr int kGroup = kTileWarps * kSubjPerWarp;
constexpr int kBuf = 1280;          // float4 per staging buffer (20 KB)
constexpr int kMaxPieces = 96;      // copies per buffer
constexpr int kMaxCols = 512;       // trimmed columns per batch
constexpr int kWaitPolls = 1 << 20;

struct TileShared {
    float4 buf[2][kBuf];
    uint64_t bar[2];
    int4 piece[2][kMaxPieces];  // slot, count, buffer offset
    int npiece[2];
    int rs[kMaxCols], re[kMaxCols];
    float4 subj[kGroup];
    int wtot[kTileWarps];
};

// Packs staging buffer b with the candidate ranges from cursor (r, o) on:
// every thread walks the same packing (so all agree on the cursor), thread 0
// records the pieces and issues one bulk copy per piece, all completing on
// the buffer's barrier.  Returns the number of staged candidates (0: done).
__device__ __forceinline__ int tile_fill(TileShared& sh, int b, int m, int& r, int& o, const float4* src, int tid) {
    int used = 0, np = 0, rr = r, oo = o;
    while (rr < m && used < kBuf && np < kMaxPieces) {
        const int take = min(sh.re[rr] - oo, kBuf - used);
        used += take;
        oo += take;
        if (oo >= sh.re[rr] && ++rr < m) oo = sh.rs[rr];
        ++np;
    }
    if (used == 0) return 0;
    if (tid == 0) {
        fence_proxy_async_smem();
        mbar_arrive_expect_tx(&sh.bar[b], (uint32_t)used * 16u);
        int u2 = 0, r2 = r, o2 = o;
        for (int q = 0; q < np; ++q) {
            const int take = min(sh.re[r2] - o2, kBuf - u2);
            sh.piece[b][q] = make_int4(o2, take, u2, 0);
            tma_load_1d(&sh.buf[b][u2], src + o2, (uint32_t)take * 16u, &sh.bar[b]);
            u2 += take;
            o2 += take;
            if (o2 >= sh.re[r2] && ++r2 < m) o2 = sh.rs[r2];
        }
        sh.npiece[b] = np;
    }
    r = rr;
    o = oo;
    return used;
}

__global__ void __launch_bounds__(kTileThreads, 3) k_porosity_tiles(CplArgs a) {
    pdl_wait();
    pdl_launch();
    __shared__ TileShared sh;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid == 0) {
        mbar_init(&sh.bar[0], 1);
        mbar_init(&sh.bar[1], 1);
        fence_mbar_init();
    }
    __syncthreads();
    uint32_t ph0 = 0u, ph1 = 0u;  // phase parity of each buffer's barrier
    const int n_near = a.ctl->n_near;
    const float rq = a.rq, t2 = a.t_support;
    const float ih2 = a.kern.inv_h * a.kern.inv_h;
    const Geo& G = a.gs;
    const float margin = 0.01f * G.cell;
    for (int g = blockIdx.x; g * kGroup < n_near; g += gridDim.x) {
        // this warp's particles (a missing one repeats the group's first)
        float3 p[kSubjPerWarp];
        int kk[kSubjPerWarp];
        bool ok[kSubjPerWarp];
#pragma unroll
        for (int s = 0; s < kSubjPerWarp; ++s) {
            const int idx = g * kGroup + warp * kSubjPerWarp + s;
            ok[s] = idx < n_near;
            kk[s] = a.near_list[ok[s] ? idx : g * kGroup];
            const float4 ps = a.f_posv[kk[s]];
            p[s] = make_float3(ps.x, ps.y, ps.z);
        }
        if (lane < kSubjPerWarp) sh.subj[warp * kSubjPerWarp + lane] = a.f_posv[kk[lane]];
        __syncthreads();
        float bx0 = INFINITY, bx1 = -INFINITY, by0 = INFINITY, by1 = -INFINITY, bz0 = INFINITY, bz1 = -INFINITY;
        for (int w = 0; w < kGroup; ++w) {
            const float4 q = sh.subj[w];
            bx0 = fminf(bx0, q.x); bx1 = fmaxf(bx1, q.x);
            by0 = fminf(by0, q.y); by1 = fmaxf(by1, q.y);
            bz0 = fminf(bz0, q.z); bz1 = fmaxf(bz1, q.z);
        }
        const int inst = 0;  // single-instance grids only (see run_porosity)
        const int x0 = coord(bx0 - rq, G.inv, G.lo[0], G.dim[0]), x1 = coord(bx1 + rq, G.inv, G.lo[0], G.dim[0]);
        const int y0 = coord(by0 - rq, G.inv, G.lo[1], G.dim[1]), y1 = coord(by1 + rq, G.inv, G.lo[1], G.dim[1]);
        const int ny = y1 - y0 + 1, ncols = (x1 - x0 + 1) * ny;
        float acc[kSubjPerWarp];
#pragma unroll
        for (int s = 0; s < kSubjPerWarp; ++s) acc[s] = 0.0f;
        for (int c0 = 0; c0 < ncols; c0 += kMaxCols) {
            // trim kMaxCols columns (contiguous per thread), compact the
            // non-empty ranges in column order
            constexpr int per = kMaxCols / kTileThreads;
            int ls[per], le[per], cnt = 0;
#pragma unroll
            for (int u = 0; u < per; ++u) {
                const int c = c0 + tid * per + u;
                ls[u] = le[u] = 0;
                if (c >= ncols) continue;
                const int cx = x0 + c / ny, cy = y0 + c % ny;
                const float xa = cx == 0 ? -INFINITY : (float)(G.lo[0] + cx) * G.cell;
                const float xb = cx == G.dim[0] - 1 ? INFINITY : (float)(G.lo[0] + cx + 1) * G.cell;
                const float ya = cy == 0 ? -INFINITY : (float)(G.lo[1] + cy) * G.cell;
                const float yb = cy == G.dim[1] - 1 ? INFINITY : (float)(G.lo[1] + cy + 1) * G.cell;
                const float gx = fmaxf(0.0f, fmaxf(xa - bx1, bx0 - xb) - margin);
                const float gy = fmaxf(0.0f, fmaxf(ya - by1, by0 - yb) - margin);
                const float rem = rq * rq - gx * gx - gy * gy;
                if (rem < 0.0f) continue;
                const float zr = sqrtf(rem) + margin;
                const int z0 = coord(bz0 - zr, G.inv, G.lo[2], G.dim[2]);
                const int z1 = coord(bz1 + zr, G.inv, G.lo[2], G.dim[2]);
                const int base = inst * G.ncl + (cx * G.dim[1] + cy) * G.dim[2];
                ls[u] = __ldg(G.start + base + z0);
                le[u] = __ldg(G.start + base + z1 + 1);
                if (le[u] > ls[u]) ++cnt;
            }
            int m;
            int off = block_exclusive_scan(cnt, sh.wtot, m);
#pragma unroll
            for (int u = 0; u < per; ++u)
                if (le[u] > ls[u]) {
                    sh.rs[off] = ls[u];
                    sh.re[off] = le[u];
                    ++off;
                }
            __syncthreads();
            if (m == 0) continue;
            // Pack buffers from the cursor (r, o) of the compacted ranges.
            int r = 0, o = sh.rs[0];
            int b = 0;
            int cur = tile_fill(sh, 0, m, r, o, a.f_posv, tid);
            while (cur > 0) {
                const int nxt = tile_fill(sh, b ^ 1, m, r, o, a.f_posv, tid);
                const uint32_t ph = b ? ph1 : ph0;
                const bool landed = mbar_wait(&sh.bar[b], ph, kWaitPolls);
                if (b) ph1 ^= 1u; else ph0 ^= 1u;
                if (__syncthreads_or(!landed)) {
                    // a copy did not land: report, let the copies in flight
                    // finish (bounded) and leave with the whole CTA
                    if (tid == 0) flag(a.ctl, SPHDEM_FLAG_TIMEOUT);
                    mbar_wait(&sh.bar[b], ph, kWaitPolls);
                    if (nxt > 0) mbar_wait(&sh.bar[b ^ 1], b ? ph0 : ph1, kWaitPolls);
                    return;
                }
                const int np = sh.npiece[b];
                for (int pc = 0; pc < np; ++pc) {
                    const int4 pe = sh.piece[b][pc];
                    const float4* B = &sh.buf[b][pe.z];
#pragma unroll 4
                    for (int i = (lane - pe.x) & 31; i < pe.y; i += 32) {
                        const float4 q = B[i];
#pragma unroll
                        for (int s = 0; s < kSubjPerWarp; ++s) acc[s] += ball_weight(p[s].x, p[s].y, p[s].z, q, ih2);
                    }
                }
                __syncthreads();  // buffer b is free again
                b ^= 1;
                cur = nxt;
            }
        }
#pragma unroll
        for (int s = 0; s < kSubjPerWarp; ++s) {
            const float flt = warp_sum(acc[s]) * a.kern.cw;
            if (!ok[s]) continue;
            float solid = 0.0f;
            const float3 ps = p[s];  // a scalar copy: capturing the array would force it to memory
            const Win w = window(a.gd, ps.x, ps.y, ps.z, rq);
            for_each_range(a.gd, w, inst, [&](int s0, int e0) {
                for (int j = s0; j < e0; ++j) {
                    const int bb = a.gd.order[j];
                    const float3 pb = ld3(a.D.pos, bb);
                    const D2 rr = d2_exact(ps.x, ps.y, ps.z, pb.x, pb.y, pb.z);
                    const float4 ab = a.aux[bb];
                    if (rr.d2 < ab.z) solid += a.D.volume[bb] * w_aux(ab, fast_sqrt(rr.d2)) / (flt + 1.0e-20f);
                }
            });
            if (lane == 0) a.P.porosity[a.gs.order[kk[s]]] = fminf(fmaxf(1.0f - solid, a.eps_min), a.eps_max);
        }
        __syncthreads();
    }
}

constexpr int kIdThreads = 256;

// Kernel_interaction_dem: one CTA per DEM a.
__global__ void __launch_bounds__(kIdThreads) k_interaction_dem(CplArgs a) {
    pdl_wait();
    pdl_launch();
    __shared__ float red[kIdThreads / 32][8];
    const int am = blockIdx.x;
    const float3 pa = ld3(a.D.pos, am);
    const float4 aux = a.aux[am];  // 1/h, cw, bound(2h), 2h
    const int inst = inst_of(a.gd, am);
    float s[8] = {0, 0, 0, 0, 0, 0, 0, 0};  // flt, rho_f, vel_f xyz, pgf xyz
    if (a.P.n > 0) {
        // the warps take turns at 32-column batches of the ball and their
        // lanes stride through each range (ranges are ~10x longer than a warp
        // and mostly shorter than the CTA)
        const float t_lo = band_lo(aux.z), t_hi = band_hi(aux.z);
        const int lane = threadIdx.x & 31;
        warp_ranges_ball(a.gs, pa.x, pa.y, pa.z, pad_radius(aux.w), inst, [&](int rs, int re) {
            for (int j = rs + lane; j < re; j += 32) {
                const float4 q = a.f_posv[j];
                float d2;
                if (d2_below(pa.x - q.x, pa.y - q.y, pa.z - q.z, t_lo, t_hi, aux.z, d2)) {  // len < 2 h_a, :157-158
                    const float Vw = q.w * w_aux(aux, fast_sqrt(d2));
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
        }, threadIdx.x >> 5, kIdThreads / 32);
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
    pdl_wait();
    pdl_launch();
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
    a.f_posq = (float4*)c->work.f_posq;
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

int run_porosity_mma(const sphdem_ctx_t* c, float support, float h, float eps_min, float eps_max, cudaStream_t st,
                     int part);

// part 0: the whole pass; 1: what depends on positions only (the tensor-core
// pass's near flags and tiles; nothing for the other variants); 2: the rest.
int run_porosity(const sphdem_ctx_t* c, float support, float h, float eps_min, float eps_max, cudaStream_t st,
                 int variant, int part) {
    const int n = c->sph.n;
    if (n <= 0) return SPHDEM_OK;
    // the tensor-core normaliser serves a uniform DEM h (variant 2)
    if (variant == 2 && h > 0.0f && c->dem.n > 0) return run_porosity_mma(c, support, h, eps_min, eps_max, st, part);
    if (part == 1) return SPHDEM_OK;
    CplArgs a = make_args(c, support, h);
    a.eps_min = eps_min;
    a.eps_max = eps_max;
    cudaError_t e = zero_words(&c->ctl->n_near, 2, st);  // n_near, near_next
    if (e != cudaSuccess) {
        set_error("porosity memset", e);
        return SPHDEM_ERR_CUDA;
    }
    launch_pdl(k_near, blocks_for(n, 256), 256, 0, st, a);
    if (c->dem.n > 0) {
        int dev = 0, sms = 148;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        // Two implementations of the uniform-h sum (same results, see the
        // kernels); variant 1 selects the shared-memory staged one, which
        // needs one instance per group of particles.
        const bool staged = variant == 1;
        if (staged && h > 0.0f && c->grid_sph.ninst <= 1) {
            const int need = blocks_for(n, kGroup);
            int blocks = sms * 4;  // resident CTAs of k_porosity_tiles per SM
            if (need < blocks) blocks = need;
            launch_pdl(k_porosity_tiles, blocks, kTileThreads, 0, st, a);
        } else {
            const int need = blocks_for(n, 8);
            int blocks = sms * 8;
            if (need < blocks) blocks = need;
            if (a.h > 0.0f)
                launch_pdl(k_porosity_near<true>, blocks, 256, 0, st, a);
            else
                launch_pdl(k_porosity_near<false>, blocks, 256, 0, st, a);
        }
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
    launch_pdl(k_interaction_dem, c->dem.n, kIdThreads, 0, st, a);
    return launch_status("interaction_dem");
}

int run_react(const sphdem_ctx_t* c, float support, float dt, bool integrate, cudaStream_t st) {
    const int n = c->sph.n;
    if (n <= 0) return SPHDEM_OK;
    CplArgs a = make_args(c, support, 0.0f);
    a.dt = dt;
    if (integrate)
        launch_pdl(k_react<true>, blocks_for(n, 256), 256, 0, st, a);
    else
        launch_pdl(k_react<false>, blocks_for(n, 256), 256, 0, st, a);
    return launch_status("react");
}

int run_drag_beta(const float* eps, const float* rho, const float* mu, const float* d, const float* speed, int n,
                  float* out, cudaStream_t st) {
    if (n <= 0) return SPHDEM_OK;
    launch_pdl(k_drag_beta, blocks_for(n, 256), 256, 0, st, eps, rho, mu, d, speed, n, out);
    return launch_status("drag_beta");
}

}  // namespace sd
