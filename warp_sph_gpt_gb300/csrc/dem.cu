// dem.cu -- DEM contacts with a compact contact-history CSR, and the DEM
// integrator.
//
// The reference rebuilds each contact CSR per step with four launches, a
// host read-back of the edge count and two exact-size allocations
// (source/Simulation.py:142-203).  Here one cooperative CTA does the whole
// rebuild on the device -- count, segmented (exclusive) scan, fill, swap --
// into fixed-capacity buffers, so the step needs no host synchronisation and
// can be captured in a CUDA graph.  The logical edge count E = offset[n] is
// exact; E > capacity raises a status bit instead of writing past the end.
//
// Contact law: DEM_contact (kernel/KERNEL_DEM_force.py:25-74), evaluated in
// FP32 except the tangential spring displacement, which accumulates in FP64
// (tang64) behind the FP32 field tang.  A tang value edited by the caller
// (its float no longer equals the rounded FP64 value) is taken as given.
#include "common.cuh"

namespace sd {

namespace {

constexpr int kDemThreads = 1024;

struct DemArgs {
    sphdem_dem_t D;
    sphdem_dembnd_t W;
    Geo gd, gw;
    int* count;  // [2*(n+1)]
    sphdem_ctl_t* ctl;
    float radius_max, bnd_radius_max, g, dt;
    int which;  // bit 1: DEM-DEM, bit 2: DEM-wall
};

// (R_a + R_b) - |x_b - x_a| > 0 evaluated exactly as the reference
// (kernel/KERNEL_DEM_force.py:19-20, kernel/KERNEL_DEM_BC.py:156-157).
__device__ __forceinline__ bool overlapping(float ra, float rb, const D2& r) {
    return __fsub_rn(__fadd_rn(ra, rb), __fsqrt_rn(r.d2)) > 0.0f;
}

__device__ __forceinline__ float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
__device__ __forceinline__ float3 add(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 sub(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 mul(float s, float3 a) { return f3(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float len(float3 a) { return sqrtf(dot(a, a)); }
__device__ __forceinline__ float3 cross(float3 a, float3 b) {
    return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float sgn(float x) { return x < 0.0f ? -1.0f : 1.0f; }  // wp.sign

// One contact: returns force on a, writes displacement, adds torque.
__device__ float3 dem_contact(float3 normal, float overlap, float radius_a, float radius_b, float3 vel_a, float3 vel_b,
                              float3 omega_a, float3 omega_b, const double* t64, float K, float eta, float mu,
                              float dt, double* disp64, float3& torque) {
    const float3 rc_a = mul(radius_a - 0.5f * overlap, normal);
    const float3 rc_b = mul(-(radius_b - 0.5f * overlap), normal);
    const float3 urel = sub(sub(add(vel_b, cross(omega_b, rc_b)), vel_a), cross(omega_a, rc_a));
    const float3 un = mul(dot(urel, normal), normal);
    const float3 us = sub(urel, un);
    disp64[0] = t64[0] + (double)us.x * (double)dt;
    disp64[1] = t64[1] + (double)us.y * (double)dt;
    disp64[2] = t64[2] + (double)us.z * (double)dt;
    const float3 disp = f3((float)disp64[0], (float)disp64[1], (float)disp64[2]);
    const float3 direction = mul(1.0f / (len(us) + 1.0e-20f), us);
    const float3 fn = add(mul(-K * overlap, normal), mul(eta, un));
    const float3 fss = add(mul(K, disp), mul(eta, us));
    const float3 fsf = mul(mu * K * overlap, direction);
    float3 fs = fss;
    if (len(fss) >= len(fsf)) fs = f3(sgn(fss.x) * fabsf(fsf.x), sgn(fss.y) * fabsf(fsf.y), sgn(fss.z) * fabsf(fsf.z));
    torque = add(torque, cross(rc_a, fs));
    return add(fn, fs);
}

// Tangential history of (a, b) from the readable side: last match in the row,
// as the reference's linear search (kernel/KERNEL_DEM_force.py:114-117).
__device__ void history(const sphdem_csr_t& old, int a, int b, double* t64) {
    t64[0] = t64[1] = t64[2] = 0.0;
    const int s = old.offset[a], e = old.offset[a + 1];
    for (int k = s; k < e && k < old.capacity; ++k)
        if (old.id[k] == b) {
            const float tx = old.tang[3 * k], ty = old.tang[3 * k + 1], tz = old.tang[3 * k + 2];
            if (old.tang64 && (float)old.tang64[3 * k] == tx && (float)old.tang64[3 * k + 1] == ty &&
                (float)old.tang64[3 * k + 2] == tz) {
                t64[0] = old.tang64[3 * k];
                t64[1] = old.tang64[3 * k + 1];
                t64[2] = old.tang64[3 * k + 2];
            } else {
                t64[0] = tx;
                t64[1] = ty;
                t64[2] = tz;
            }
        }
}

__device__ int count_dem(const DemArgs& A, int a) {
    const float3 pa = ld3(A.D.pos, a);
    const float Ra = A.D.radius[a];
    const int inst = inst_of(A.gd, a);
    const Win w = window(A.gd, pa.x, pa.y, pa.z, pad_radius(Ra + A.radius_max));
    int c = 0;
    for_each_range(A.gd, w, inst, [&](int s, int e) {
        for (int k = s; k < e; ++k) {
            const int b = A.gd.order[k];
            if (b == a) continue;
            const float3 pb = ld3(A.D.pos, b);
            if (overlapping(Ra, A.D.radius[b], d2_exact(pb.x, pb.y, pb.z, pa.x, pa.y, pa.z))) ++c;
        }
    });
    return c;
}

__device__ int count_wall(const DemArgs& A, int a) {
    const float3 pa = ld3(A.D.pos, a);
    const float Ra = A.D.radius[a];
    const int inst = inst_of(A.gd, a);
    const Win w = window(A.gw, pa.x, pa.y, pa.z, pad_radius(Ra + A.bnd_radius_max));
    int c = 0;
    for_each_range(A.gw, w, inst, [&](int s, int e) {
        for (int k = s; k < e; ++k) {
            const int b = A.gw.order[k];
            const float3 pb = ld3(A.W.pos, b);
            if (overlapping(Ra, A.W.radius[b], d2_exact(pb.x, pb.y, pb.z, pa.x, pa.y, pa.z))) ++c;
        }
    });
    return c;
}

// Sort one CSR row of ids ascending in place (rows are short).
__device__ void sort_row(int* id, int s, int e) {
    for (int x = s + 1; x < e; ++x) {
        int v = id[x], y = x - 1;
        while (y >= s && id[y] > v) {
            id[y + 1] = id[y];
            --y;
        }
        id[y + 1] = v;
    }
}

// Fill the row of a for one contact kind: ids (enumeration order, then sorted),
// history, contact law; accumulates force and torque.
template <bool WALL>
__device__ void fill_row(const DemArgs& A, int a, const sphdem_csr_t& old, const sphdem_csr_t& nw, float3& force,
                         float3& torque) {
    const int s = nw.offset[a], e = nw.offset[a + 1];
    if (e > nw.capacity) return;  // overflow was flagged by the scan
    const float3 pa = ld3(A.D.pos, a);
    const float Ra = A.D.radius[a];
    const int inst = inst_of(A.gd, a);
    const Geo& G = WALL ? A.gw : A.gd;
    const float* npos = WALL ? A.W.pos : A.D.pos;
    const float* nrad = WALL ? A.W.radius : A.D.radius;
    const Win w = window(G, pa.x, pa.y, pa.z, pad_radius(Ra + (WALL ? A.bnd_radius_max : A.radius_max)));
    int out = s;
    for_each_range(G, w, inst, [&](int rs, int re) {
        for (int k = rs; k < re; ++k) {
            const int b = G.order[k];
            if (!WALL && b == a) continue;
            const float3 pb = ld3(npos, b);
            if (overlapping(Ra, nrad[b], d2_exact(pb.x, pb.y, pb.z, pa.x, pa.y, pa.z)) && out < e) nw.id[out++] = b;
        }
    });
    sort_row(nw.id, s, e);
    const float3 va = ld3(A.D.vel, a), wa = ld3(A.D.omega, a);
    const float K = A.D.K[a], eta = A.D.eta[a], mu = A.D.mu[a];
    for (int k = s; k < e; ++k) {
        const int b = nw.id[k];
        const float3 pb = ld3(npos, b);
        const float3 rab = sub(pb, pa);
        const float dist = len(rab);
        const float overlap = Ra + nrad[b] - dist;
        double t64[3], d64[3];
        history(old, a, b, t64);
        float3 normal = WALL ? f3(0.f, 0.f, -1.f) : f3(a > b ? -1.f : 1.f, 0.f, 0.f);
        if (dist > 1.0e-12f) normal = mul(1.0f / dist, rab);
        const float3 vb = WALL ? ld3(A.W.vel, b) : ld3(A.D.vel, b);
        const float3 wb = WALL ? ld3(A.W.omega, b) : ld3(A.D.omega, b);
        force = add(force, dem_contact(normal, overlap, Ra, nrad[b], va, vb, wa, wb, t64, K, eta, mu, A.dt, d64, torque));
        nw.tang[3 * k] = (float)d64[0];
        nw.tang[3 * k + 1] = (float)d64[1];
        nw.tang[3 * k + 2] = (float)d64[2];
        if (nw.tang64) {
            nw.tang64[3 * k] = d64[0];
            nw.tang64[3 * k + 1] = d64[1];
            nw.tang64[3 * k + 2] = d64[2];
        }
    }
}

// Single-CTA rebuild of the selected contact CSR kinds.
__global__ void __launch_bounds__(kDemThreads) k_contacts(DemArgs A) {
    pdl_wait();
    pdl_launch();
    __shared__ int warp_tot[kDemThreads / 32];
    const int n = A.D.n;
    const int old_d = A.ctl->old_dem, old_b = A.ctl->old_bnd;
    const bool do_d = A.which & 1, do_w = A.which & 2;
    int* cnt_d = A.count;
    int* cnt_w = A.count + (n + 1);
    for (int a = threadIdx.x; a < n; a += blockDim.x) {
        if (do_d) cnt_d[a] = count_dem(A, a);
        if (do_w) cnt_w[a] = count_wall(A, a);
    }
    __syncthreads();
    // exclusive scans -> new-side offsets
    for (int kind = 0; kind < 2; ++kind) {
        if (kind == 0 ? !do_d : !do_w) continue;
        const int* cnt = kind == 0 ? cnt_d : cnt_w;
        const sphdem_csr_t& nw = kind == 0 ? A.D.csr_dem[1 - old_d] : A.D.csr_bnd[1 - old_b];
        long long carry = 0;
        for (int base = 0; base < n; base += blockDim.x) {
            const int a = base + threadIdx.x;
            const int v = a < n ? cnt[a] : 0;
            int total;
            const int ex = block_exclusive_scan(v, warp_tot, total);
            if (a < n) nw.offset[a] = (int)(carry + ex);
            carry += total;
        }
        if (threadIdx.x == 0) {
            nw.offset[n] = (int)carry;
            if (kind == 0) A.ctl->e_dem = (int)carry;
            else A.ctl->e_bnd = (int)carry;
            if (carry > nw.capacity)
                atomicOr(&A.ctl->status, kind == 0 ? SPHDEM_FLAG_CSR_DEM_OVERFLOW : SPHDEM_FLAG_CSR_BND_OVERFLOW);
        }
        __syncthreads();
    }
    // fill rows, accumulate loads
    for (int a = threadIdx.x; a < n; a += blockDim.x) {
        float3 fd = f3(0.f, 0.f, 0.f), td = f3(0.f, 0.f, 0.f);
        if (do_d) {
            fd = f3(0.f, 0.f, -A.D.m[a] * A.g);  // gravity once, kernel/KERNEL_DEM_force.py:100
            fill_row<false>(A, a, A.D.csr_dem[old_d], A.D.csr_dem[1 - old_d], fd, td);
        } else {
            fd = ld3(A.D.force, a);
            td = ld3(A.D.torque, a);
        }
        if (do_w) {
            float3 fw = f3(0.f, 0.f, 0.f), tw = f3(0.f, 0.f, 0.f);
            fill_row<true>(A, a, A.D.csr_bnd[old_b], A.D.csr_bnd[1 - old_b], fw, tw);
            fd = add(fd, fw);  // kernel/KERNEL_DEM_BC.py:218-219
            td = add(td, tw);
        }
        st3(A.D.force, a, fd);
        st3(A.D.torque, a, td);
    }
    __syncthreads();
    // publish: the written side becomes readable (source/Simulation.py:166-171)
    if (threadIdx.x == 0) {
        if (do_d) A.ctl->old_dem = 1 - old_d;
        if (do_w) A.ctl->old_bnd = 1 - old_b;
    }
}

// Per-DEM coupling constants: 1/h, 21/(16 pi h^3), sqrt bound of 2h, 2h.
__global__ void k_dem_aux(const float* __restrict__ h, int n, float4* __restrict__ aux) {
    pdl_wait();
    pdl_launch();
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= n) return;
    const float hb = h[a];
    const Kern k = make_kern_dev(hb);
    aux[a] = make_float4(k.inv_h, k.cw, sqrt_lt_bound(2.0f * hb), 2.0f * hb);
}

// Kernel_step_dem (kernel/KERNEL_DEM_step.py:6-30), every operation rounded.
__global__ void k_step_dem(sphdem_dem_t D, float dt) {
    pdl_wait();
    pdl_launch();
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= D.n) return;
    const float m = D.m[a], I = D.inertia[a];
    const float3 F = ld3(D.force, a), T = ld3(D.torque, a);
    const float3 acc = make_float3(__fdiv_rn(F.x, m), __fdiv_rn(F.y, m), __fdiv_rn(F.z, m));
    st3(D.acc, a, acc);
    euler_store(D.pos, D.vel, a, acc, dt);
    float3 w = ld3(D.omega, a);
    w.x = __fadd_rn(w.x, __fmul_rn(__fdiv_rn(T.x, I), dt));
    w.y = __fadd_rn(w.y, __fmul_rn(__fdiv_rn(T.y, I), dt));
    w.z = __fadd_rn(w.z, __fmul_rn(__fdiv_rn(T.z, I), dt));
    st3(D.omega, a, w);
}

}  // namespace

int run_contacts(const sphdem_ctx_t* c, float radius_max, float bnd_radius_max, float g, float dt, int which,
                 cudaStream_t st) {
    if (c->dem.n <= 0) return SPHDEM_OK;
    DemArgs A;
    A.D = c->dem;
    A.W = c->dembnd;
    A.gd = make_geo(c->grid_dem);
    A.gw = make_geo(c->grid_dembnd);
    A.count = c->work.dem_count;
    A.ctl = c->ctl;
    A.radius_max = radius_max;
    A.bnd_radius_max = bnd_radius_max;
    A.g = g;
    A.dt = dt;
    A.which = which;
    launch_pdl(k_contacts, 1, kDemThreads, 0, st, A);
    return launch_status("contacts");
}

int run_dem_aux(const sphdem_ctx_t* c, cudaStream_t st) {
    if (c->dem.n <= 0) return SPHDEM_OK;
    launch_pdl(k_dem_aux, blocks_for(c->dem.n, 128), 128, 0, st, c->dem.h, c->dem.n, (float4*)c->work.dem_aux);
    return launch_status("dem_aux");
}

int run_step_dem(const sphdem_ctx_t* c, float dt, cudaStream_t st) {
    if (c->dem.n <= 0) return SPHDEM_OK;
    launch_pdl(k_step_dem, blocks_for(c->dem.n, 128), 128, 0, st, c->dem, dt);
    return launch_status("step_dem");
}

}  // namespace sd

// ===========================================================================
// Contact rebuild without caller-provided scratch.
//
// Some callers cannot allocate device memory: a host code whose GPU memory
// belongs to another framework's pool and that can only lend this library the
// particle and contact buffers it already owns, or a time loop that must not
// allocate once it runs.  For them the per-row contact counts, the only
// scratch the contact rebuild needs, live in the fixed array below instead of
// a caller buffer.  Every GPU that loads this library holds the array (512 KB)
// until the process exits.
// ===========================================================================
#include <mutex>

namespace {
static __device__ __align__(256) int g_contact_count_scratch[2 * (SPHDEM_NOALLOC_MAX_DEM + 1)];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
int* g_scratch_ptr[kMaxDevices] = {};

// Device address of the array on the current device, looked up once per
// device.  In host code the array's name stands for a host-side shadow, not a
// device address, so it must never be passed to a kernel directly.  The
// cached address belongs to the device's primary context as it was at the
// lookup: it does not survive cudaDeviceReset (or any other teardown of that
// context) in the same process, after which this entry point must not be
// called on that device again.
//
// The array is per device, so the call is refused when the current device is
// not the one that holds the caller's sphere buffers (the kernel would read
// one GPU's buffers while counting into another GPU's array).
int scratch_for_current_device(const void* probe, int** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        sd::set_error("contacts (no-alloc): cudaGetDevice", e);
        return SPHDEM_ERR_CUDA;
    }
    if (dev < 0 || dev >= kMaxDevices) {
        sd::set_error_msg("contacts (no-alloc): device index beyond the supported range");
        return SPHDEM_ERR_INVALID;
    }
    if (probe) {
        cudaPointerAttributes attr;
        e = cudaPointerGetAttributes(&attr, probe);
        if (e != cudaSuccess) {
            sd::set_error("contacts (no-alloc): cudaPointerGetAttributes", e);
            return SPHDEM_ERR_CUDA;
        }
        if (attr.type == cudaMemoryTypeDevice && attr.device != dev) {
            sd::set_error_msg("contacts (no-alloc): the sphere buffers live on another GPU than the current "
                              "device; make their GPU current first");
            return SPHDEM_ERR_INVALID;
        }
    }
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_ptr[dev]) {
        int* p = nullptr;
        e = cudaGetSymbolAddress((void**)&p, g_contact_count_scratch);
        if (e != cudaSuccess || !p) {
            sd::set_error("contacts (no-alloc): cudaGetSymbolAddress", e);
            return SPHDEM_ERR_CUDA;
        }
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return SPHDEM_OK;
}
}  // namespace

extern "C" int sphdem_contacts_noalloc(sphdem_ctx_t* c, float radius_max, float bnd_radius_max, float g, float dt,
                                       int which, sphdem_stream_t s) {
    if (!c || !c->ctl) {
        sd::set_error_msg("contacts (no-alloc): null context or control block");
        return SPHDEM_ERR_INVALID;
    }
    if (which < 1 || which > 3) {
        sd::set_error_msg("contacts (no-alloc): which must be 1 (DEM-DEM), 2 (DEM-wall) or 3 (both)");
        return SPHDEM_ERR_INVALID;
    }
    if (c->dem.n > SPHDEM_NOALLOC_MAX_DEM) {
        sd::set_error_msg("contacts (no-alloc): more moving DEM spheres than SPHDEM_NOALLOC_MAX_DEM (65536); "
                          "use sphdem_force_dem / sphdem_bc_dem with caller scratch");
        return SPHDEM_ERR_INVALID;
    }
    int* scratch = nullptr;
    int rc = scratch_for_current_device(c->dem.n > 0 ? c->dem.pos : nullptr, &scratch);
    if (rc) return rc;
    // Every count entry the rebuild reads is written by its own count pass
    // first, so nothing left in the array by an earlier call is ever used.
    sphdem_ctx_t cc = *c;
    cc.work.dem_count = scratch;
    return sd::run_contacts(&cc, radius_max, bnd_radius_max, g, dt, which, sd::as_stream(s));
}
