// common.cuh -- shared device code of libsphdem: grid geometry, candidate
// enumeration, the exact FP32 membership predicates and the Wendland kernel.
//
// Membership predicates decide neighbour and contact sets, which must equal
// the reference's bit for bit.  They are written with __f*_rn intrinsics so
// nvcc cannot fuse a multiply into an add: dot(r, r) is ((dx*dx + dy*dy) +
// dz*dz) rounded after every operation, as Warp evaluates it
// (kernel/KERNEL_rho.py:29, kernel/KERNEL_force.py:39).  Physics values that
// only enter sums use ordinary (FMA-contracted) arithmetic.
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include "sphdem.h"

namespace sd {

constexpr float kR2Min = 1.0e-12f;  // kernel/Kernel_KNL.py:5
constexpr double kPi = 3.14159265358979323846;
constexpr int kWarp = 32;

// ---------------------------------------------------------------------------
// Canonical cell lattice.  World cell index = floor(x * inv); a grid stores the
// world index `lo` of its local cell 0 and clamps at its faces.  Binning does
// not depend on the box, so two grids of the same cell width traverse the same
// world cells in the same order, and a point outside the box falls into a
// face cell (never missed: clamping is monotone).
// ---------------------------------------------------------------------------
struct Geo {
    int lo[3];
    int dim[3];
    float inv;
    float cell;  // cell width (1/inv)
    int ncl;    // cells per instance
    int ninst;  // instances sharing the geometry
    const int* __restrict__ start;
    const int* __restrict__ order;
    const int* __restrict__ key;
};

inline Geo make_geo(const sphdem_grid_t& g) {
    Geo G;
    for (int d = 0; d < 3; ++d) {
        G.lo[d] = g.lo[d];
        G.dim[d] = g.dim[d];
    }
    G.inv = g.inv_cell;
    G.cell = g.cell;
    G.ncl = g.ncell_local;
    G.ninst = g.ninst;
    G.start = g.cell_start;
    G.order = g.order;
    G.key = g.key;
    return G;
}

__device__ __forceinline__ int coord(float x, float inv, int lo, int dim) {
    float f = floorf(__fmul_rn(x, inv));
    f = fminf(fmaxf(f, -1.0e9f), 1.0e9f);  // NaN -> -1e9 (fmaxf drops NaN)
    int c = (int)f - lo;
    return c < 0 ? 0 : (c >= dim ? dim - 1 : c);
}

struct Win {
    int x0, x1, y0, y1, z0, z1;
};

// Cells overlapping [p - rq, p + rq]; rq is the padded query radius.
__device__ __forceinline__ Win window(const Geo& g, float px, float py, float pz, float rq) {
    Win w;
    w.x0 = coord(px - rq, g.inv, g.lo[0], g.dim[0]);
    w.x1 = coord(px + rq, g.inv, g.lo[0], g.dim[0]);
    w.y0 = coord(py - rq, g.inv, g.lo[1], g.dim[1]);
    w.y1 = coord(py + rq, g.inv, g.lo[1], g.dim[1]);
    w.z0 = coord(pz - rq, g.inv, g.lo[2], g.dim[2]);
    w.z1 = coord(pz + rq, g.inv, g.lo[2], g.dim[2]);
    return w;
}

// Query radius padded far beyond any FP32 rounding of the coordinates, so the
// window is a superset of every pair the exact predicate can accept.
__host__ __device__ __forceinline__ float pad_radius(float r) { return r * 1.001f + 1.0e-6f; }

// Calls f(s, e) for each contiguous sorted range [s, e) of candidate slots
// (one range per (x, y) column of the window, z-cells are adjacent).
template <class F>
__device__ __forceinline__ void for_each_range(const Geo& g, const Win& w, int inst, F&& f) {
    const int base_i = inst * g.ncl;
    for (int cx = w.x0; cx <= w.x1; ++cx)
        for (int cy = w.y0; cy <= w.y1; ++cy) {
            const int base = base_i + (cx * g.dim[1] + cy) * g.dim[2];
            const int s = __ldg(g.start + base + w.z0);
            const int e = __ldg(g.start + base + w.z1 + 1);
            if (s < e) f(s, e);
        }
}

// Ball-trimmed enumeration: like for_each_range, but each (x, y) column only
// contributes the z cells that a ball of radius rq around p can reach over
// that column's square, and columns beyond rq are skipped.  A point binned in
// column (cx, cy) lies within `margin` of that column's square (binning is
// floor(x * inv)), so its horizontal distance to p is at least the square's
// gap; if it is within rq of p its z lies within sqrt(rq^2 - gap^2) of p.z
// and its z cell is enumerated.  Face columns extend to infinity (clamping).
//
// column_range_ball gives the slot range [s, e) of column (cx, cy) trimmed to
// the ball (empty if the column lies beyond rq); for_each_range_ball visits
// the window's columns x-major.  Every operation is rounded on its own (no
// contraction), so each kernel that trims a column gets the same range: the
// density pass's walk masks are decoded against the force pass's own ranges.
__device__ __forceinline__ void column_range_ball(const Geo& g, int cx, int cy, float px, float py, float pz,
                                                  float rq, int inst, int& s, int& e) {
    const float margin = __fmul_rn(0.01f, g.cell);
    const float x0 = cx == 0 ? -INFINITY : __fmul_rn((float)(g.lo[0] + cx), g.cell);
    const float x1 = cx == g.dim[0] - 1 ? INFINITY : __fmul_rn((float)(g.lo[0] + cx + 1), g.cell);
    const float y0 = cy == 0 ? -INFINITY : __fmul_rn((float)(g.lo[1] + cy), g.cell);
    const float y1 = cy == g.dim[1] - 1 ? INFINITY : __fmul_rn((float)(g.lo[1] + cy + 1), g.cell);
    const float gx = fmaxf(0.0f, __fsub_rn(fmaxf(__fsub_rn(x0, px), __fsub_rn(px, x1)), margin));
    const float gy = fmaxf(0.0f, __fsub_rn(fmaxf(__fsub_rn(y0, py), __fsub_rn(py, y1)), margin));
    const float rem = __fsub_rn(__fsub_rn(__fmul_rn(rq, rq), __fmul_rn(gx, gx)), __fmul_rn(gy, gy));
    s = e = 0;
    if (rem < 0.0f) return;
    // MUFU root (its error is far inside the margin); capped at rq, so the
    // trimmed cells lie within the window's z cells (a member has |dz| < rq)
    const float zr = fminf(__fadd_rn(__fmul_rn(rem, rsqrtf(fmaxf(rem, 1.0e-30f))), margin), rq);
    const int z0 = coord(__fsub_rn(pz, zr), g.inv, g.lo[2], g.dim[2]);
    const int z1 = coord(__fadd_rn(pz, zr), g.inv, g.lo[2], g.dim[2]);
    const int base = inst * g.ncl + (cx * g.dim[1] + cy) * g.dim[2];
    s = __ldg(g.start + base + z0);
    e = __ldg(g.start + base + z1 + 1);
}

template <class F>
__device__ __forceinline__ void for_each_range_ball(const Geo& g, float px, float py, float pz, float rq, int inst,
                                                    F&& f) {
    const Win w = window(g, px, py, pz, rq);
    for (int cx = w.x0; cx <= w.x1; ++cx)
        for (int cy = w.y0; cy <= w.y1; ++cy) {
            int s, e;
            column_range_ball(g, cx, cy, px, py, pz, rq, inst, s, e);
            if (s < e) f(s, e);
        }
}

// ---------------------------------------------------------------------------
// Walk masks.  A pass that walks a subject's ball-trimmed ranges (in the order
// of for_each_range_ball, each range in slot order) records one bit per slot
// it walks, set for the members it accepted; word w of a subject's stream sits
// in row w of a rows x n array (subjects contiguous within a row, so a warp's
// stores and loads coalesce).  A later pass re-trims the same columns and
// decodes the bits back into the same member slots in the same order.
// ---------------------------------------------------------------------------
// Member slots of a recorded walk, one per next() call, -1 at the end.  Walk
// positions are consumed in order, so the word holding position b is loaded
// exactly when b is the first position of a word.
struct MaskIter {
    int x1, y0, y1, cx, cy;  // window columns still to trim
    int cur, end, b;         // unread part of the current range; walk position of cur
    uint32_t word, m;        // loaded word; unreported members of the current segment
    int mbase;               // slot of bit 0 of m
    __device__ __forceinline__ void init(const Geo& g, float px, float py, float pz, float rq) {
        const Win w = window(g, px, py, pz, rq);
        x1 = w.x1;
        y0 = w.y0;
        y1 = w.y1;
        cx = w.x0;
        cy = w.y0 - 1;
        cur = end = b = 0;
        word = m = 0u;
        mbase = 0;
    }
    // rows: the stream's cap words per subject (a walk longer than 32 cap ends
    // early instead of reading past them; the caller only decodes walks that fit)
    __device__ __forceinline__ int next(const Geo& g, float px, float py, float pz, float rq, int inst,
                                        const int32_t* __restrict__ rows, size_t n, int k, int cap) {
        for (;;) {
            if (m) {
                const int t = __ffs(m) - 1;
                m &= m - 1u;
                return mbase + t;
            }
            if (cur < end) {
                const int sh = b & 31;
                if (sh == 0) {
                    if ((b >> 5) >= cap) return -1;
                    word = (uint32_t)__ldg(rows + (size_t)(b >> 5) * n + k);
                }
                const int take = min(32 - sh, end - cur);
                m = word >> sh;
                if (take < 32) m &= (1u << take) - 1u;
                mbase = cur;
                cur += take;
                b += take;
                continue;
            }
            for (;;) {
                if (++cy > y1) {
                    cy = y0;
                    if (++cx > x1) {
                        cx = x1 + 1;
                        return -1;
                    }
                }
                column_range_ball(g, cx, cy, px, py, pz, rq, inst, cur, end);
                if (end > cur) break;
            }
        }
    }
};

// Warp-cooperative ball enumeration: the 32 lanes trim 32 columns at a time
// (instead of every lane trimming every column), then f(s, e) is called
// warp-uniformly for each non-empty range, in column order.
// With part / parts, the warp takes only every parts-th batch of 32 columns
// from batch `part` on (the warps of a CTA sharing one ball).
template <class F>
__device__ __forceinline__ void warp_ranges_ball(const Geo& g, float px, float py, float pz, float rq, int inst,
                                                 F&& f, int part = 0, int parts = 1) {
    const int lane = threadIdx.x & 31;
    const Win w = window(g, px, py, pz, rq);
    const int ny = w.y1 - w.y0 + 1;
    const int ncols = (w.x1 - w.x0 + 1) * ny;
    for (int c0 = 32 * part; c0 < ncols; c0 += 32 * parts) {
        int s = 0, e = 0;
        const int c = c0 + lane;
        if (c < ncols) column_range_ball(g, w.x0 + c / ny, w.y0 + c % ny, px, py, pz, rq, inst, s, e);
        unsigned mask = __ballot_sync(0xffffffffu, e > s);
        while (mask) {
            const int src = __ffs(mask) - 1;
            mask &= mask - 1;
            f(__shfl_sync(0xffffffffu, s, src), __shfl_sync(0xffffffffu, e, src));
        }
    }
}

// Membership d2 < t for a candidate, exactly as the FP32 predicate with every
// operation rounded, but decided from the cheaper contracted dot product
// whenever it is clear of the bound: fma-contracted and fully rounded dot
// products differ by a few ulps, far inside the 2^-20 relative band, so only
// candidates inside the band pay for the exact re-evaluation.
__device__ __forceinline__ bool d2_below(float dx, float dy, float dz, float t_lo, float t_hi, float t, float& d2) {
    d2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
    if (d2 < t_lo) return true;
    if (d2 >= t_hi) return false;
    const float ex = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
    return ex < t;
}
__host__ __device__ __forceinline__ float band_lo(float t) { return t * (1.0f - 9.5367431640625e-7f); }
__host__ __device__ __forceinline__ float band_hi(float t) { return t * (1.0f + 9.5367431640625e-7f); }

__device__ __forceinline__ int inst_of(const Geo& g, int point) {
    return (g.ninst > 1 && g.ncl > 0) ? __ldg(g.key + point) / g.ncl : 0;
}

// ---------------------------------------------------------------------------
// Exact FP32 predicates
// ---------------------------------------------------------------------------
struct D2 {
    float dx, dy, dz, d2;
};
// r = a - b and dot(r, r), each operation rounded (no contraction).
__device__ __forceinline__ D2 d2_exact(float ax, float ay, float az, float bx, float by, float bz) {
    D2 r;
    r.dx = __fsub_rn(ax, bx);
    r.dy = __fsub_rn(ay, by);
    r.dz = __fsub_rn(az, bz);
    r.d2 = __fadd_rn(__fadd_rn(__fmul_rn(r.dx, r.dx), __fmul_rn(r.dy, r.dy)), __fmul_rn(r.dz, r.dz));
    return r;
}

// Smallest float t >= 0 with fl(sqrt(t)) >= s.  Because correctly rounded
// sqrt is monotone, "fl(sqrt(d2)) < s" (wp.length(r) < s) holds exactly when
// d2 < t, so loops over many candidates test d2 < t without a square root.
__host__ __device__ inline float sqrt_lt_bound(float s) {
    if (!(s > 0.0f)) return 0.0f;
    if (s == INFINITY) return INFINITY;
    uint32_t lo = 0u, hi = 0x7f800000u;  // [0, +inf]
    while (lo < hi) {
        uint32_t mid = lo + ((hi - lo) >> 1);
#ifdef __CUDA_ARCH__
        float r = __fsqrt_rn(__uint_as_float(mid));
#else
        float x;
        memcpy(&x, &mid, 4);
        float r = sqrtf(x);
#endif
        if (r >= s)
            hi = mid;
        else
            lo = mid + 1;
    }
#ifdef __CUDA_ARCH__
    return __uint_as_float(lo);
#else
    float t;
    memcpy(&t, &lo, 4);
    return t;
#endif
}

// Distance for physics values only (never for membership): MUFU rsqrt, 0 at 0.
__device__ __forceinline__ float fast_sqrt(float x) {
    float r = x * rsqrtf(x);
    return x > 0.0f ? r : 0.0f;
}

// ---------------------------------------------------------------------------
// Wendland C2 in 3D, support 2h (kernel/Kernel_KNL.py:7-41)
//   W     = 21/(16 pi h^3) u^4 (1 + 2q),  u = 1 - q/2, q = r/h < 2
//   dW/dr = 21/(16 pi h^4) (-5 q u^3)
// ---------------------------------------------------------------------------
struct Kern {
    float inv_h, cw, cdw;
};
inline Kern make_kern(float h) {
    Kern k;
    double hd = (double)h;
    k.inv_h = (float)(1.0 / hd);
    k.cw = (float)(21.0 / (16.0 * kPi * hd * hd * hd));
    k.cdw = (float)(-105.0 / (16.0 * kPi * hd * hd * hd * hd));
    return k;
}
__device__ __forceinline__ Kern make_kern_dev(float h) {
    Kern k;
    double hd = (double)h;
    k.inv_h = (float)(1.0 / hd);
    k.cw = (float)(21.0 / (16.0 * kPi * hd * hd * hd));
    k.cdw = (float)(-105.0 / (16.0 * kPi * hd * hd * hd * hd));
    return k;
}
__device__ __forceinline__ float kern_w(const Kern& k, float r) {
    float q = r * k.inv_h;
    float u = 1.0f - 0.5f * q;
    float u2 = u * u;
    return q < 2.0f ? k.cw * u2 * u2 * (1.0f + 2.0f * q) : 0.0f;
}
__device__ __forceinline__ float kern_dw(const Kern& k, float r) {
    float q = r * k.inv_h;
    float u = 1.0f - 0.5f * q;
    return q < 2.0f ? k.cdw * q * u * u * u : 0.0f;
}

// Tait EOS with the negative-pressure clamp (kernel/KERNEL_pres.py:6-23),
// p = B max((rho/rho0)^gamma - 1, 0), evaluated as
// B expm1(gamma log1p((rho - rho0)/rho0)): rho - rho0 is exact near rest, so
// p keeps its relative accuracy where (rho/rho0)^gamma - 1 would cancel.
__device__ __forceinline__ float tait(float rho, float rho0, float B, float gamma) {
    float q = expm1f(gamma * log1pf((rho - rho0) / rho0));
    return B * fmaxf(q, 0.0f);
}

__device__ __forceinline__ void flag(sphdem_ctl_t* ctl, int bits) {
    if (ctl) atomicOr(&ctl->status, bits);
}

__device__ __forceinline__ float3 ld3(const float* p, int i) {
    return make_float3(p[3 * i], p[3 * i + 1], p[3 * i + 2]);
}
__device__ __forceinline__ void st3(float* p, int i, float3 v) {
    p[3 * i] = v.x;
    p[3 * i + 1] = v.y;
    p[3 * i + 2] = v.z;
}

// Warp-sum (fixed shuffle tree: deterministic).
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// v = v + a dt; x = x + v dt with every operation rounded (no FMA), shared by
// the SPH-only and coupled integrators so both give identical bits
// (kernel/KERNEL_step.py:18-22).
__device__ __forceinline__ void euler_store(float* pos, float* vel, int i, float3 a, float dt) {
    float3 v = ld3(vel, i), x = ld3(pos, i);
    v.x = __fadd_rn(v.x, __fmul_rn(a.x, dt));
    v.y = __fadd_rn(v.y, __fmul_rn(a.y, dt));
    v.z = __fadd_rn(v.z, __fmul_rn(a.z, dt));
    st3(vel, i, v);
    x.x = __fadd_rn(x.x, __fmul_rn(v.x, dt));
    x.y = __fadd_rn(x.y, __fmul_rn(v.y, dt));
    x.z = __fadd_rn(x.z, __fmul_rn(v.z, dt));
    st3(pos, i, x);
}

// Block-wide exclusive scan of one int per thread (blockDim a multiple of 32,
// warp_tot holds blockDim/32 ints); total receives the block sum.
__device__ __forceinline__ int block_exclusive_scan(int v, int* warp_tot, int& total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int nw = blockDim.x >> 5;
        int t = lane < nw ? warp_tot[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        if (lane < nw) warp_tot[lane] = t;
    }
    __syncthreads();
    int before = wid > 0 ? warp_tot[wid - 1] : 0;
    total = warp_tot[(blockDim.x >> 5) - 1];
    __syncthreads();
    return before + x - v;
}

}  // namespace sd

// ---------------------------------------------------------------------------
// host-side error plumbing shared by the translation units
// ---------------------------------------------------------------------------
namespace sd {
void set_error(const char* where, cudaError_t e);
void set_error_msg(const char* msg);
int launch_status(const char* where);
inline cudaStream_t as_stream(sphdem_stream_t s) { return (cudaStream_t)s; }
inline int blocks_for(long n, int threads) { return (int)((n + threads - 1) / threads); }

// Programmatic dependent launch: a step kernel is launched with programmatic
// stream serialization, so the GPU may schedule it while the previous kernel
// on the stream is still finishing; every such kernel calls pdl_wait() first
// (griddepcontrol.wait: blocks until the preceding grids have completed and
// their writes are visible -- the ordinary stream order, minus the launch gap)
// and pdl_launch() to let its own successor be scheduled.  Both are no-ops
// for an ordinary launch.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_launch() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <typename... P, typename... A>
inline void launch_pdl(void (*kernel)(P...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, A&&... args) {
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kernel, static_cast<P>(args)...);  // errors surface through launch_status
}
namespace {
// Zero fill as a kernel (not a memset node), so it stays in a chain of
// programmatic dependent launches.
__global__ void k_zero_words(int* __restrict__ p, long n) {
    pdl_wait();
    pdl_launch();
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) p[i] = 0;
}
}  // namespace

// Zero `words` 32-bit words at p on st (launch errors surface through the
// caller's launch_status / cudaGetLastError).
inline cudaError_t zero_words(void* p, long words, cudaStream_t st) {
    if (words <= 0) return cudaSuccess;
    const int grid = blocks_for(words, 256) < 1024 ? blocks_for(words, 256) : 1024;
    launch_pdl(k_zero_words, grid, 256, 0, st, static_cast<int*>(p), words);
    return cudaGetLastError();
}

}  // namespace sd
