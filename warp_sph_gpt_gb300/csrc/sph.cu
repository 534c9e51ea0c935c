// sph.cu -- WCSPH neighbour loops on the sorted fluid / wall copies.
//
// One thread per subject (or, for small systems, one warp per subject: the
// launch option lanes = 32), subjects taken in cell order (grid order), so the
// threads of a warp query the same few cell columns and their float4
// neighbour loads hit the same L1 lines.  Neighbour membership uses the exact
// FP32 predicates of the reference; the physics sums use contracted FP32.
//
//   k_density        Kernel_shepard_sph + Kernel_density_sph + Kernel_pres_sph
//                    (kernel/KERNEL_rho.py:6-82, kernel/KERNEL_pres.py:6-23) in
//                    one pass: the Shepard sum, when due, shares the loop.
//   k_density_wall   Kernel_density_bnd + Kernel_pres_bnd (KERNEL_rho.py:87-126,
//                    KERNEL_pres.py:26-45) with the constant wall-wall part cached.
//   k_force          Kernel_force_sph (kernel/KERNEL_force.py:7-71) and the
//                    pressure-gradient half of Kernel_prep_sphdem
//                    (kernel/KERNEL_SPHDEM_interaction.py:97-112): same
//                    neighbours, same support, one loop.
//   k_step_sph       Kernel_step_sph (kernel/KERNEL_step.py:6-22).
//
// Neighbour records (one thread per subject): the density pass already
// decides every fluid-fluid and fluid-wall membership of the step (same
// support, same exact predicate as the force pass), so it records them and the
// force pass loops over exactly those members instead of testing every
// candidate.  A thread walking cells evaluates the force body for ~1 in 5
// candidates, and the warp pays for the body on every candidate some lane
// accepts; from the record every iteration is a member.  Same members, same
// order, same arithmetic: the forces are bit-identical.  Two forms
// (params.nbr_format): int32 member slots (SPHDEM_NBR_SLOTS, 4 bytes per
// member), or walk masks (SPHDEM_NBR_MASKS, one bit per walked slot, ~5 per
// member: a sixth of the bytes, but the force pass re-trims the ranges and
// decodes the bits).
#include "common.cuh"

namespace sd {

namespace {

// Subject of this thread (LANES = 1) or of this warp (LANES = 32), and the
// neighbour visitor: a thread walks every slot of the ball-trimmed ranges; a
// warp takes the ranges together and its lanes stride through each one.  The
// warp form has 32x the parallelism for small systems; its sums are reduced
// across lanes at the end (a different, equally valid FP32 summation order).
template <int LANES>
__device__ __forceinline__ int subject_index(int& lane) {
    const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
    lane = LANES == 1 ? 0 : (int)(threadIdx.x & 31);
    return (int)(LANES == 1 ? t : t >> 5);
}

template <int LANES, class F>
__device__ __forceinline__ void visit_ball(const Geo& g, float px, float py, float pz, float rq, int inst, int lane,
                                           F&& body) {
    if (LANES == 1) {
        for_each_range_ball(g, px, py, pz, rq, inst, [&](int s, int e) {
            for (int j = s; j < e; ++j) body(j);
        });
    } else {
        warp_ranges_ball(g, px, py, pz, rq, inst, [&](int s, int e) {
            for (int j = s + lane; j < e; j += 32) body(j);
        });
    }
}

template <int LANES>
__device__ __forceinline__ float lanes_sum(float v) {
    return LANES == 1 ? v : warp_sum(v);
}

// Thread-per-subject walk of the ball-trimmed ranges, candidate by candidate
// (the lanes of a warp, consecutive particles of one or two cells, mostly test
// the same candidate together, so its load is one broadcast), body(j, q, r)
// for the members.  With rows, the walk mask is recorded: each range is taken
// in segments that end where a 32-bit mask word ends, the segment's member
// bits gathered in a register and stored with the word.  Returns the slots
// walked.
template <class Body>
__device__ __forceinline__ int walk_record(const Geo& g, const float4* __restrict__ posm, const float4& p, float rq,
                                           int inst, float s2, int32_t* __restrict__ rows, size_t n, int k, int cap,
                                           Body&& body) {
    int pos = 0;
    uint32_t word = 0u;
    for_each_range_ball(g, p.x, p.y, p.z, rq, inst, [&](int s, int e) {
        for (int j0 = s; j0 < e;) {
            const int b = pos + (j0 - s);
            const int sh = b & 31;
            const int j1 = min(j0 + 32 - sh, e);
            uint32_t m = 0u, bit = 1u << sh;
            for (int j = j0; j < j1; ++j, bit <<= 1) {
                const float4 q = posm[j];
                const D2 r = d2_exact(p.x, p.y, p.z, q.x, q.y, q.z);
                if (r.d2 < s2) {
                    body(j, q, r);
                    m |= bit;
                }
            }
            if (rows) {
                word |= m;
                if (sh + (j1 - j0) == 32) {
                    if ((b >> 5) < cap) rows[(size_t)(b >> 5) * n + k] = (int32_t)word;
                    word = 0u;
                }
            }
            j0 = j1;
        }
        pos += e - s;
    });
    if (rows && (pos & 31) && (pos >> 5) < cap) rows[(size_t)(pos >> 5) * n + k] = (int32_t)word;
    return pos;
}

struct DensArgs {
    Geo gs, gb;
    const float4* __restrict__ f_posm;
    const float* __restrict__ f_vprev;  // m/rho before this pass (Shepard input)
    const float4* __restrict__ b_posm;
    const float* __restrict__ b_vprev;
    float* flt;
    float* rho;
    float* pres;
    float4* f_rp;    // out: rho, pres, pres/rho^2, 1/rho  (sorted)
    float4* f_posv;  // out: x, y, z, m/rho                 (sorted)
    int* nbr;        // out: neighbour records (sphdem_work_t.nbr), or null
    int cap;         // per subject and kind: slots or mask words
    int fmt;         // SPHDEM_NBR_SLOTS or SPHDEM_NBR_MASKS
    int n;
    float s2, rq;
    Kern kern;
    float rho0, B, gamma;
};

template <int LANES, bool FLT, bool RHO, bool PRES>
__global__ void __launch_bounds__(256) k_density(DensArgs a) {
    pdl_wait();
    pdl_launch();
    int lane;
    const int k = subject_index<LANES>(lane);
    if (k >= a.n) return;
    const int o = a.gs.order[k];
    const float4 p = a.f_posm[k];
    const int inst = inst_of(a.gs, o);
    float rho_sum = 0.0f, flt_sum = 0.0f;
    if (LANES == 1 && a.nbr != nullptr && a.fmt == SPHDEM_NBR_MASKS) {
        // the walks, recording their walk masks
        const size_t n = (size_t)a.n;
        int32_t* rows = a.nbr;
        const int wf = walk_record(a.gs, a.f_posm, p, a.rq, inst, a.s2, rows, n, k, a.cap,
                                   [&](int j, const float4& q, const D2& r) {
                                       const float w = kern_w(a.kern, fast_sqrt(r.d2));
                                       if (RHO) rho_sum += q.w * w;
                                       if (FLT) flt_sum += a.f_vprev[j] * w;
                                   });
        int wb = 0;
        if (a.gb.ncl > 0)
            wb = walk_record(a.gb, a.b_posm, p, a.rq, inst, a.s2, rows + (size_t)a.cap * n, n, k, a.cap,
                             [&](int j, const float4& q, const D2& r) {
                                 const float w = kern_w(a.kern, fast_sqrt(r.d2));
                                 if (RHO) rho_sum += q.w * w;
                                 if (FLT) flt_sum += a.b_vprev[j] * w;
                             });
        rows[(size_t)(2 * a.cap) * n + k] = wf;
        rows[(size_t)(2 * a.cap + 1) * n + k] = wb;
    } else {
        // the walks, recording the member slots when the step keeps them
        const bool list = LANES == 1 && a.nbr != nullptr;
        const size_t n = (size_t)a.n;
        int cf = 0, cb = 0;
        visit_ball<LANES>(a.gs, p.x, p.y, p.z, a.rq, inst, lane, [&](int j) {
            const float4 q = a.f_posm[j];
            const D2 r = d2_exact(p.x, p.y, p.z, q.x, q.y, q.z);
            if (r.d2 < a.s2) {
                const float w = kern_w(a.kern, fast_sqrt(r.d2));
                if (RHO) rho_sum += q.w * w;
                if (FLT) flt_sum += a.f_vprev[j] * w;
                if (list) {
                    if (cf < a.cap) a.nbr[(size_t)cf * n + k] = j;
                    ++cf;
                }
            }
        });
        if (a.gb.ncl > 0) {
            visit_ball<LANES>(a.gb, p.x, p.y, p.z, a.rq, inst, lane, [&](int j) {
                const float4 q = a.b_posm[j];
                const D2 r = d2_exact(p.x, p.y, p.z, q.x, q.y, q.z);
                if (r.d2 < a.s2) {
                    const float w = kern_w(a.kern, fast_sqrt(r.d2));
                    if (RHO) rho_sum += q.w * w;
                    if (FLT) flt_sum += a.b_vprev[j] * w;
                    if (list) {
                        if (cb < a.cap) a.nbr[(size_t)(a.cap + cb) * n + k] = j;
                        ++cb;
                    }
                }
            });
        }
        if (list) {
            a.nbr[(size_t)(2 * a.cap) * n + k] = cf;
            a.nbr[(size_t)(2 * a.cap + 1) * n + k] = cb;
        }
    }
    if (RHO) rho_sum = lanes_sum<LANES>(rho_sum);
    if (FLT) flt_sum = lanes_sum<LANES>(flt_sum);
    if (lane != 0) return;
    if (FLT) a.flt[o] = flt_sum;
    if (RHO) {
        const float flt = FLT ? flt_sum : a.flt[o];
        const float rho = rho_sum / flt;
        a.rho[o] = rho;
        if (PRES) {
            const float pr = tait(rho, a.rho0, a.B, a.gamma);
            a.pres[o] = pr;
            const float irho = 1.0f / rho;
            a.f_rp[k] = make_float4(rho, pr, pr * irho * irho, irho);
            a.f_posv[k] = make_float4(p.x, p.y, p.z, p.w * irho);
        }
    }
}

struct WallArgs {
    Geo gs, gb;
    const float4* __restrict__ f_posm;
    const float4* __restrict__ b_posm;
    const float* __restrict__ b_self;
    float* rho;
    float* pres;
    float4* b_rp;
    int n;
    float s2, rq;
    Kern kern;
    float rho0, B, gamma;
};

template <int LANES, bool PRES>
__global__ void __launch_bounds__(256) k_density_wall(WallArgs a) {
    pdl_wait();
    pdl_launch();
    int lane;
    const int k = subject_index<LANES>(lane);
    if (k >= a.n) return;
    const int o = a.gb.order[k];
    const float4 p = a.b_posm[k];
    const int inst = inst_of(a.gb, o);
    float rho_sum = 0.0f;
    if (a.gs.ncl > 0) {
        visit_ball<LANES>(a.gs, p.x, p.y, p.z, a.rq, inst, lane, [&](int j) {
            const float4 q = a.f_posm[j];
            const D2 r = d2_exact(p.x, p.y, p.z, q.x, q.y, q.z);
            if (r.d2 < a.s2) rho_sum += q.w * kern_w(a.kern, fast_sqrt(r.d2));
        });
    }
    rho_sum = lanes_sum<LANES>(rho_sum);
    if (lane != 0) return;
    const float rho = rho_sum + a.b_self[k];
    a.rho[o] = rho;
    if (PRES) {
        const float pr = tait(rho, a.rho0, a.B, a.gamma);
        a.pres[o] = pr;
        const float irho = 1.0f / rho;
        a.b_rp[k] = make_float4(rho, pr, pr * irho * irho, irho);
    }
}

struct ForceArgs {
    Geo gs, gb;
    const float4* __restrict__ f_posm;
    const float4* __restrict__ f_vel;
    const float4* __restrict__ f_rp;
    const float4* __restrict__ b_posm;
    const float4* __restrict__ b_vel;
    const float4* __restrict__ b_rp;
    float* acc;
    float* pgf;
    float4* f_pgf;     // out (sorted): pgf x, y, z, rho
    const int* nbr;    // neighbour records of this step's density pass, or null
    int cap;           // per subject and kind: slots or mask words
    int fmt;           // SPHDEM_NBR_SLOTS or SPHDEM_NBR_MASKS
    int n;
    float s2, rq;
    Kern kern;
    float two_mu, eps_h2, g;
};

// Pair term shared by the fluid and wall loops.  MODE bit 1: acceleration,
// bit 2: negative pressure gradient.
template <int MODE>
__device__ __forceinline__ void force_pair(const ForceArgs& a, const D2& r, const float4& vi, float pr_i,
                                           float p_i, float irho_i, const float4& q, const float4& rpj,
                                           const float4* __restrict__ velp, int j, float3& acc, float3& pgf) {
    const float rinv = rsqrtf(r.d2);
    const float dist = r.d2 * rinv;
    const float dwr = kern_dw(a.kern, dist) * rinv;  // (dW/dr) / r
    const float gx = dwr * r.dx, gy = dwr * r.dy, gz = dwr * r.dz;  // grad_i W
    if (MODE & 1) {
        const float sc = q.w * (pr_i + rpj.z);
        const float4 vj = velp[j];
        const float visc =
            __fdividef(a.two_mu * (r.dx * gx + r.dy * gy + r.dz * gz) * irho_i * rpj.w, r.d2 + a.eps_h2);
        const float mv = q.w * visc;
        acc.x += mv * (vi.x - vj.x) - sc * gx;
        acc.y += mv * (vi.y - vj.y) - sc * gy;
        acc.z += mv * (vi.z - vj.z) - sc * gz;
    }
    if (MODE & 2) {
        const float c = q.w * rpj.w * (rpj.y - p_i);
        pgf.x -= c * gx;
        pgf.y -= c * gy;
        pgf.z -= c * gz;
    }
}

// The c member slots rows[t * n + k] recorded for subject k, in walk order,
// four per round: their slots, then their positions, are loaded together so
// the gathers overlap (the loop is latency bound).
template <int MODE>
__device__ __forceinline__ void force_slots(const ForceArgs& a, const float4* __restrict__ posm,
                                            const float4* __restrict__ rp, const float4* __restrict__ vel,
                                            const int32_t* __restrict__ rows, int c, const float4& p,
                                            const float4& vi, const float4& rpi, int k, float3& acc, float3& pgf) {
    const size_t n = (size_t)a.n;
    for (int t = 0; t < c; t += 4) {
        int js[4];
        float4 qs[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) js[u] = t + u < c ? rows[(size_t)(t + u) * n + k] : rows[(size_t)t * n + k];
#pragma unroll
        for (int u = 0; u < 4; ++u) qs[u] = posm[js[u]];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const D2 r = d2_exact(p.x, p.y, p.z, qs[u].x, qs[u].y, qs[u].z);
            if (t + u < c && r.d2 > kR2Min)
                force_pair<MODE>(a, r, vi, rpi.z, rpi.y, rpi.w, qs[u], rp[js[u]], vel, js[u], acc, pgf);
        }
    }
}

// Ball-trimmed ranges a subject's walk-mask decode keeps in shared memory.
constexpr int kForceRanges = 16;

// The members a walk mask records for subject k over geometry g, in walk
// order, summed four per round (their slots, then their positions, are loaded
// together so the gathers overlap: the loop is latency bound).  The subject's
// non-empty ball-trimmed ranges are trimmed once into a table in shared memory
// -- per range, slot - walk position and the walk position where it ends -- so
// a member costs a find-first-set on its mask word and one table step.
// Returns false, having summed nothing, when the walk it re-trims is not the
// one recorded (more ranges than the table holds, or another length): the
// caller then walks the cells.
template <int MODE>
__device__ __forceinline__ bool force_members(const ForceArgs& a, const Geo& g, const float4* __restrict__ posm,
                                              const float4* __restrict__ rp, const float4* __restrict__ vel,
                                              const int32_t* __restrict__ rows, int walked, const float4& p,
                                              const float4& vi, const float4& rpi, int inst, int k, int32_t* tab,
                                              int ts, float3& acc, float3& pgf) {
    int nr = 0, pos = 0;
    for_each_range_ball(g, p.x, p.y, p.z, a.rq, inst, [&](int s, int e) {
        if (nr < kForceRanges) {
            tab[(2 * nr) * ts] = s - pos;  // slot of walk position q in this range: q + (s - pos)
            tab[(2 * nr + 1) * ts] = pos + (e - s);
        }
        ++nr;
        pos += e - s;
    });
    if (nr > kForceRanges || pos != walked) return false;
    const size_t n = (size_t)a.n;
    const int nwords = (pos + 31) >> 5;
    int wi = 0, base = 0, ri = 0;
    uint32_t word = nwords > 0 ? (uint32_t)__ldg(rows + k) : 0u;
    int off = nr > 0 ? tab[0] : 0, end = nr > 0 ? tab[ts] : 0;
    for (bool more = nwords > 0; more;) {
        int js[4] = {-1, -1, -1, -1};
#pragma unroll 1
        for (int u = 0; u < 4;) {
            if (word == 0u) {
                if (++wi >= nwords) {
                    more = false;
                    break;
                }
                word = (uint32_t)__ldg(rows + (size_t)wi * n + k);
                base = wi << 5;
                continue;
            }
            const int q = base + __ffs(word) - 1;
            word &= word - 1u;
            while (q >= end) {
                ++ri;
                off = tab[(2 * ri) * ts];
                end = tab[(2 * ri + 1) * ts];
            }
            js[0] = js[1];
            js[1] = js[2];
            js[2] = js[3];
            js[3] = q + off;
            ++u;
        }
        if (js[3] < 0) break;
        float4 qv[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) qv[u] = posm[js[u] < 0 ? js[3] : js[u]];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const D2 r = d2_exact(p.x, p.y, p.z, qv[u].x, qv[u].y, qv[u].z);
            if (js[u] >= 0 && r.d2 > kR2Min)
                force_pair<MODE>(a, r, vi, rpi.z, rpi.y, rpi.w, qv[u], rp[js[u]], vel, js[u], acc, pgf);
        }
    }
    return true;
}

template <int LANES, int MODE>
__global__ void __launch_bounds__(256, 4) k_force(ForceArgs a) {
    pdl_wait();
    pdl_launch();
    int lane;
    const int k = subject_index<LANES>(lane);
    if (k >= a.n) return;
    const int o = a.gs.order[k];
    const float4 p = a.f_posm[k];
    const float4 vi = a.f_vel[k];
    const float4 rpi = a.f_rp[k];
    const int inst = inst_of(a.gs, o);
    float3 acc = make_float3(0.f, 0.f, 0.f), pgf = make_float3(0.f, 0.f, 0.f);
    bool walk = true;
    if (LANES == 1 && a.nbr != nullptr && a.fmt == SPHDEM_NBR_MASKS) {
        // the members recorded by the density pass (all with d2 < s2), in walk order
        extern __shared__ int32_t force_tab[];
        const size_t n = (size_t)a.n;
        const int wf = a.nbr[(size_t)(2 * a.cap) * n + k], wb = a.nbr[(size_t)(2 * a.cap + 1) * n + k];
        if (wf <= 32 * a.cap && wb <= 32 * a.cap) {
            float3 af = acc, pf = pgf;
            bool ok = force_members<MODE>(a, a.gs, a.f_posm, a.f_rp, a.f_vel, a.nbr, wf, p, vi, rpi, inst, k,
                                          force_tab + threadIdx.x, blockDim.x, af, pf);
            if (ok && a.gb.ncl > 0 && wb > 0)
                ok = force_members<MODE>(a, a.gb, a.b_posm, a.b_rp, a.b_vel, a.nbr + (size_t)a.cap * n, wb, p, vi,
                                         rpi, inst, k, force_tab + threadIdx.x, blockDim.x, af, pf);
            if (ok) {
                walk = false;
                acc = af;
                pgf = pf;
            }
        }
    } else if (LANES == 1 && a.nbr != nullptr) {
        // the member slots recorded by the density pass (all with d2 < s2), in walk order
        const size_t n = (size_t)a.n;
        const int cf = a.nbr[(size_t)(2 * a.cap) * n + k], cb = a.nbr[(size_t)(2 * a.cap + 1) * n + k];
        if (cf <= a.cap && cb <= a.cap) {
            walk = false;
            force_slots<MODE>(a, a.f_posm, a.f_rp, a.f_vel, a.nbr, cf, p, vi, rpi, k, acc, pgf);
            force_slots<MODE>(a, a.b_posm, a.b_rp, a.b_vel, a.nbr + (size_t)a.cap * n, cb, p, vi, rpi, k, acc, pgf);
        }
    }
    if (walk) {
        visit_ball<LANES>(a.gs, p.x, p.y, p.z, a.rq, inst, lane, [&](int j) {
            const float4 q = a.f_posm[j];
            const D2 r = d2_exact(p.x, p.y, p.z, q.x, q.y, q.z);
            if (r.d2 > kR2Min && r.d2 < a.s2)
                force_pair<MODE>(a, r, vi, rpi.z, rpi.y, rpi.w, q, a.f_rp[j], a.f_vel, j, acc, pgf);
        });
        if (a.gb.ncl > 0) {
            visit_ball<LANES>(a.gb, p.x, p.y, p.z, a.rq, inst, lane, [&](int j) {
                const float4 q = a.b_posm[j];
                const D2 r = d2_exact(p.x, p.y, p.z, q.x, q.y, q.z);
                if (r.d2 > kR2Min && r.d2 < a.s2)
                    force_pair<MODE>(a, r, vi, rpi.z, rpi.y, rpi.w, q, a.b_rp[j], a.b_vel, j, acc, pgf);
            });
        }
    }
    if (MODE & 1) {
        acc.x = lanes_sum<LANES>(acc.x);
        acc.y = lanes_sum<LANES>(acc.y);
        acc.z = lanes_sum<LANES>(acc.z);
    }
    if (MODE & 2) {
        pgf.x = lanes_sum<LANES>(pgf.x);
        pgf.y = lanes_sum<LANES>(pgf.y);
        pgf.z = lanes_sum<LANES>(pgf.z);
    }
    if (lane != 0) return;
    if (MODE & 1) st3(a.acc, o, make_float3(acc.x, acc.y, acc.z - a.g));
    if (MODE & 2) {
        if (a.pgf) st3(a.pgf, o, pgf);
        a.f_pgf[k] = make_float4(pgf.x, pgf.y, pgf.z, rpi.x);
    }
}

__global__ void k_pres(const float* __restrict__ rho, float* __restrict__ pres, int n, float rho0, float B,
                       float gamma) {
    pdl_wait();
    pdl_launch();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) pres[i] = tait(rho[i], rho0, B, gamma);
}

}  // namespace

namespace {
__global__ void k_step_sph(float* pos, float* vel, const float* __restrict__ acc, int n, float dt) {
    pdl_wait();
    pdl_launch();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) euler_store(pos, vel, i, ld3(acc, i), dt);
}
}  // namespace

static float tait_B(float rho0, float c0, float gamma) { return rho0 * c0 * c0 / gamma; }

// Threads per block of the neighbour loops: 64, 128 or 256 (default 128).
static int launch_block(int b) { return (b == 64 || b == 256) ? b : 128; }

int run_density(const sphdem_ctx_t* c, float support, float h, bool flt, bool rho, bool pres, float rho0, float c0,
                float gamma, cudaStream_t st, int block, int lanes, int nbr_cap, int nbr_format) {
    const int n = c->sph.n;
    if (n <= 0) return SPHDEM_OK;
    DensArgs a;
    a.gs = make_geo(c->grid_sph);
    a.gb = make_geo(c->grid_bnd);
    if (c->bnd.n <= 0) a.gb.ncl = 0;
    a.f_posm = (const float4*)c->work.f_posm;
    a.f_vprev = c->work.f_vprev;
    a.b_posm = (const float4*)c->work.b_posm;
    a.b_vprev = c->work.b_vprev;
    a.flt = c->sph.flt;
    a.rho = c->sph.rho;
    a.pres = c->sph.pres;
    a.f_rp = (float4*)c->work.f_rp;
    a.f_posv = (float4*)c->work.f_posv;
    a.nbr = (nbr_cap > 0 && lanes != 32) ? c->work.nbr : nullptr;
    a.cap = nbr_cap;
    a.fmt = nbr_format;
    a.n = n;
    a.s2 = support * support;
    a.rq = pad_radius(support);
    a.kern = make_kern(h);
    a.rho0 = rho0;
    a.B = tait_B(rho0, c0, gamma);
    a.gamma = gamma;
    const int bs = launch_block(block);
    if (lanes == 32) {
        const int nb = blocks_for((long)n * 32, bs);
        if (flt && rho && pres)
            launch_pdl(k_density<32, true, true, true>, nb, bs, 0, st, a);
        else if (!flt && rho && pres)
            launch_pdl(k_density<32, false, true, true>, nb, bs, 0, st, a);
        else if (flt && !rho)
            launch_pdl(k_density<32, true, false, false>, nb, bs, 0, st, a);
        else if (!flt && rho && !pres)
            launch_pdl(k_density<32, false, true, false>, nb, bs, 0, st, a);
        else
            launch_pdl(k_density<32, true, true, false>, nb, bs, 0, st, a);
    } else {
        const int nb = blocks_for(n, bs);
        if (flt && rho && pres)
            launch_pdl(k_density<1, true, true, true>, nb, bs, 0, st, a);
        else if (!flt && rho && pres)
            launch_pdl(k_density<1, false, true, true>, nb, bs, 0, st, a);
        else if (flt && !rho)
            launch_pdl(k_density<1, true, false, false>, nb, bs, 0, st, a);
        else if (!flt && rho && !pres)
            launch_pdl(k_density<1, false, true, false>, nb, bs, 0, st, a);
        else
            launch_pdl(k_density<1, true, true, false>, nb, bs, 0, st, a);
    }
    return launch_status("density");
}

int run_density_wall(const sphdem_ctx_t* c, float support, float h, bool pres, float rho0, float c0, float gamma,
                     cudaStream_t st, int block, int lanes) {
    const int n = c->bnd.n;
    if (n <= 0) return SPHDEM_OK;
    WallArgs a;
    a.gs = make_geo(c->grid_sph);
    if (c->sph.n <= 0) a.gs.ncl = 0;
    a.gb = make_geo(c->grid_bnd);
    a.f_posm = (const float4*)c->work.f_posm;
    a.b_posm = (const float4*)c->work.b_posm;
    a.b_self = c->work.b_self;
    a.rho = c->bnd.rho;
    a.pres = c->bnd.pres;
    a.b_rp = (float4*)c->work.b_rp;
    a.n = n;
    a.s2 = support * support;
    a.rq = pad_radius(support);
    a.kern = make_kern(h);
    a.rho0 = rho0;
    a.B = tait_B(rho0, c0, gamma);
    a.gamma = gamma;
    const int bs = launch_block(block);
    if (lanes == 32) {
        const int nb = blocks_for((long)n * 32, bs);
        if (pres)
            launch_pdl(k_density_wall<32, true>, nb, bs, 0, st, a);
        else
            launch_pdl(k_density_wall<32, false>, nb, bs, 0, st, a);
    } else {
        if (pres)
            launch_pdl(k_density_wall<1, true>, blocks_for(n, bs), bs, 0, st, a);
        else
            launch_pdl(k_density_wall<1, false>, blocks_for(n, bs), bs, 0, st, a);
    }
    return launch_status("density_wall");
}

int run_force(const sphdem_ctx_t* c, float support, float h, float mu, float g, int mode, cudaStream_t st, int block,
              int lanes, int nbr_cap, int nbr_format) {
    const int n = c->sph.n;
    if (n <= 0) return SPHDEM_OK;
    ForceArgs a;
    a.gs = make_geo(c->grid_sph);
    a.gb = make_geo(c->grid_bnd);
    if (c->bnd.n <= 0) a.gb.ncl = 0;
    a.f_posm = (const float4*)c->work.f_posm;
    a.f_vel = (const float4*)c->work.f_vel;
    a.f_rp = (const float4*)c->work.f_rp;
    a.b_posm = (const float4*)c->work.b_posm;
    a.b_vel = (const float4*)c->work.b_vel;
    a.b_rp = (const float4*)c->work.b_rp;
    a.acc = c->sph.acc;
    a.pgf = c->sph.pgf;
    a.f_pgf = (float4*)c->work.f_pgf;
    a.nbr = (nbr_cap > 0 && lanes != 32) ? c->work.nbr : nullptr;
    a.cap = nbr_cap;
    a.fmt = nbr_format;
    a.n = n;
    a.s2 = support * support;
    a.rq = pad_radius(support);
    a.kern = make_kern(h);
    a.two_mu = 2.0f * mu;
    a.eps_h2 = 0.01f * h * h;
    a.g = g;
    const int bs = launch_block(block);
    if (lanes == 32) {
        const int nb = blocks_for((long)n * 32, bs);
        if (mode == 3)
            launch_pdl(k_force<32, 3>, nb, bs, 0, st, a);
        else if (mode == 2)
            launch_pdl(k_force<32, 2>, nb, bs, 0, st, a);
        else
            launch_pdl(k_force<32, 1>, nb, bs, 0, st, a);
    } else {
        const int nb = blocks_for(n, bs);
        const size_t smem =
            a.nbr && a.fmt == SPHDEM_NBR_MASKS ? (size_t)2 * kForceRanges * bs * sizeof(int32_t) : 0;  // 32 KB at 256
        if (mode == 3)
            launch_pdl(k_force<1, 3>, nb, bs, smem, st, a);
        else if (mode == 2)
            launch_pdl(k_force<1, 2>, nb, bs, smem, st, a);
        else
            launch_pdl(k_force<1, 1>, nb, bs, smem, st, a);
    }
    return launch_status("force");
}

int run_pres(const float* rho, float* pres, int n, float rho0, float c0, float gamma, cudaStream_t st) {
    if (n <= 0) return SPHDEM_OK;
    launch_pdl(k_pres, blocks_for(n, 256), 256, 0, st, rho, pres, n, rho0, tait_B(rho0, c0, gamma), gamma);
    return launch_status("pres");
}

int run_step_sph(const sphdem_ctx_t* c, float dt, cudaStream_t st) {
    const int n = c->sph.n;
    if (n <= 0) return SPHDEM_OK;
    launch_pdl(k_step_sph, blocks_for(n, 256), 256, 0, st, c->sph.pos, c->sph.vel, c->sph.acc, n, dt);
    return launch_status("step_sph");
}

}  // namespace sd
