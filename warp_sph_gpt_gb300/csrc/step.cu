// step.cu -- the C ABI: step orchestration, CUDA-graph replay, single-kernel
// entry points, verification digests and FP64 diagnostics.
//
// Step order follows source/Simulation.py:17-221:
//   SPH:     [Shepard +] density + Tait (fluid) ; density + Tait (walls) ;
//            force (+ -grad p when coupled)
//   coupled: DEM-DEM and DEM-wall CSR rebuild with loads ; porosity ;
//            fluid -> DEM exchange ; DEM -> fluid reaction + SPH integration ;
//            DEM integration
// The -grad p half of Kernel_prep_sphdem moves into the force loop: it reads
// the same pressures, positions and neighbours, none of which the DEM contact
// stage in between can change.
#include <stdio.h>
#include <string.h>

#include <map>
#include <mutex>

#include "common.cuh"
#include "sphdem_mpnn.h"
#include "tma.cuh"

namespace sd {

int build_grid(sphdem_grid_t* g, const float* pos, sphdem_ctl_t* ctl, cudaStream_t st);
int gather_fluid(const sphdem_ctx_t* c, cudaStream_t st);
int gather_wall(const sphdem_ctx_t* c, float support, float h, cudaStream_t st);
int gather_wall_rho(const sphdem_ctx_t* c, cudaStream_t st);
int run_density(const sphdem_ctx_t* c, float support, float h, bool flt, bool rho, bool pres, float rho0, float c0,
                float gamma, cudaStream_t st, int block = 0, int lanes = 1, int nbr_cap = 0, int nbr_format = 0);
int run_density_wall(const sphdem_ctx_t* c, float support, float h, bool pres, float rho0, float c0, float gamma,
                     cudaStream_t st, int block = 0, int lanes = 1);
int run_force(const sphdem_ctx_t* c, float support, float h, float mu, float g, int mode, cudaStream_t st,
              int block = 0, int lanes = 1, int nbr_cap = 0, int nbr_format = 0);
int run_pres(const float* rho, float* pres, int n, float rho0, float c0, float gamma, cudaStream_t st);
int run_step_sph(const sphdem_ctx_t* c, float dt, cudaStream_t st);
int run_contacts(const sphdem_ctx_t* c, float radius_max, float bnd_radius_max, float g, float dt, int which,
                 cudaStream_t st);
int run_dem_aux(const sphdem_ctx_t* c, cudaStream_t st);
int run_step_dem(const sphdem_ctx_t* c, float dt, cudaStream_t st);
int run_porosity(const sphdem_ctx_t* c, float support, float h, float eps_min, float eps_max, cudaStream_t st,
                 int variant = 0, int part = 0);
int run_interaction_dem(const sphdem_ctx_t* c, float mu, float eps_min, float eps_max, float dt, cudaStream_t st);
int porosity_setup();
int run_corrmax(const float* out, int nf, int nd, const float* scale4, float mdt, float* dst, cudaStream_t st);
int porosity_frame_edge(int frame);
int64_t porosity_frames(const sphdem_grid_t& g, int F);
int run_react(const sphdem_ctx_t* c, float support, float dt, bool integrate, cudaStream_t st);
int run_drag_beta(const float* eps, const float* rho, const float* mu, const float* d, const float* speed, int n,
                  float* out, cudaStream_t st);

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------
static thread_local char g_err[512] = "";

void set_error(const char* where, cudaError_t e) {
    snprintf(g_err, sizeof(g_err), "%s: %s (%d)", where, cudaGetErrorString(e), (int)e);
}
void set_error_msg(const char* msg) { snprintf(g_err, sizeof(g_err), "%s", msg); }
int launch_status(const char* where) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error(where, e);
        return SPHDEM_ERR_CUDA;
    }
    return SPHDEM_OK;
}

#define TRY(x)                   \
    do {                         \
        int rc_ = (x);           \
        if (rc_) return rc_;     \
    } while (0)

namespace {

// Neighbour lists between the density and force passes of a step, when the
// context provides their buffer.
int nbr_cap(const sphdem_ctx_t* c, const sphdem_params_t* p) {
    const bool known = p->nbr_format == SPHDEM_NBR_SLOTS || p->nbr_format == SPHDEM_NBR_MASKS;
    return (c->work.nbr != nullptr && p->nbr_cap > 0 && known) ? p->nbr_cap : 0;
}

bool shepard_due(const sphdem_params_t* p, int step) {
    return step == 0 || (p->shepard_step > 0 && step % p->shepard_step == 0);  // source/Simulation.py:45
}

// SPH densities, pressures and forces (source/Simulation.py:53-91); mode 3
// also forms -grad p for the coupling.  The pgf field is written only when
// write_pgf; the acceleration arithmetic is the same either way.
int sph_part(sphdem_ctx_t* c, const sphdem_params_t* p, bool shep, bool write_pgf, cudaStream_t st) {
    if (shep) TRY(gather_wall_rho(c, st));
    const int cap = nbr_cap(c, p);
    TRY(run_density(c, p->support, p->h, shep, true, true, p->rho0, p->c0, p->gamma, st, p->block_sph, p->lanes_sph,
                    cap, p->nbr_format));
    TRY(run_density_wall(c, p->support, p->h, true, p->rho0, p->c0, p->gamma, st, p->block_sph, p->lanes_sph));
    sphdem_ctx_t cc = *c;
    if (!write_pgf) cc.sph.pgf = nullptr;
    return run_force(&cc, p->support, p->h, p->mu, p->g, 3, st, p->block_sph, p->lanes_sph, cap, p->nbr_format);
}

int sph_onestep(sphdem_ctx_t* c, const sphdem_params_t* p, bool shep, bool integrate, cudaStream_t st) {
    TRY(sph_part(c, p, shep, false, st));
    if (integrate) TRY(run_step_sph(c, p->dt, st));
    return SPHDEM_OK;
}

// Two side streams and their fork/join events per device: the DEM contact
// branch and the porosity branch.
struct Fork {
    cudaStream_t side = nullptr, side2 = nullptr, side3 = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr, fork2 = nullptr, join2 = nullptr, ready = nullptr, wall = nullptr,
                dens = nullptr;
};
std::mutex g_fork_mu;
Fork g_fork[64];

int fork_for_current_device(Fork** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return launch_status("fork device");
    std::lock_guard<std::mutex> lock(g_fork_mu);
    Fork& f = g_fork[dev];
    if (!f.side) {
        cudaError_t e = cudaStreamCreateWithFlags(&f.side, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&f.side2, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&f.side3, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&f.fork, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&f.join, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&f.fork2, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&f.join2, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&f.ready, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&f.wall, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&f.dens, cudaEventDisableTiming);
        if (e != cudaSuccess) {
            set_error("fork stream", e);
            return SPHDEM_ERR_CUDA;
        }
    }
    *out = &f;
    return SPHDEM_OK;
}

// Three branches per step, forked and joined by events (inside a graph
// capture they become parallel branches of the graph):
//   contact branch: [DEM grid re-bin] -> DEM-DEM / DEM-wall contacts; it reads
//                   only DEM and wall-sphere state.
//   main:           [fluid grid re-bin + gather] -> DEM constants -> [wall
//                   m/rho for the Shepard filter] -> fluid density -> force
//                   (after the wall density) -> fluid -> DEM exchange (after
//                   the contacts: it adds to their forces; it reads -grad p,
//                   not the fluid porosity) -> reaction on the fluid and
//                   integrators (after the porosity branch).
//   wall branch:    wall density (it reads only positions and masses).
//   porosity branch: porosity, once the fluid density (m/rho) and the DEM
//                   grid are ready.
// build: the step first re-bins its moving grids (the loop body) -- the
// fluid grid only if !fluid_fresh; the single-call API has built them already.
// density_fresh (no Shepard step): the sorted copies, densities, pressures and
// neighbour records of the current positions are in place already (a learned
// jump's judge computed them), so the gather and the density pass are skipped.
int coupled_onestep(sphdem_ctx_t* c, const sphdem_params_t* p, bool shep, cudaStream_t st, bool build = false,
                    bool fluid_fresh = false, bool density_fresh = false) {
    Fork* f = nullptr;
    TRY(fork_for_current_device(&f));
    auto rec = [&](cudaEvent_t ev, cudaStream_t s) {
        const cudaError_t e = cudaEventRecord(ev, s);
        if (e != cudaSuccess) set_error("event record", e);
        return e == cudaSuccess ? SPHDEM_OK : SPHDEM_ERR_CUDA;
    };
    auto wait = [&](cudaStream_t s, cudaEvent_t ev) {
        const cudaError_t e = cudaStreamWaitEvent(s, ev, 0);
        if (e != cudaSuccess) set_error("event wait", e);
        return e == cudaSuccess ? SPHDEM_OK : SPHDEM_ERR_CUDA;
    };
    // contact branch
    TRY(rec(f->fork, st));
    TRY(wait(f->side, f->fork));
    if (build) TRY(build_grid(&c->grid_dem, c->dem.pos, c->ctl, f->side));
    TRY(rec(f->ready, f->side));
    TRY(run_contacts(c, p->radius_max, p->boundary_radius_max, p->g, p->dt, 3, f->side));
    TRY(rec(f->join, f->side));
    // main, up to the fork of the porosity branch
    if (build) {
        if (!fluid_fresh) TRY(build_grid(&c->grid_sph, c->sph.pos, c->ctl, st));
        if (!density_fresh) TRY(gather_fluid(c, st));
    }
    TRY(run_dem_aux(c, st));
    if (shep) TRY(gather_wall_rho(c, st));
    TRY(rec(f->fork2, st));
    TRY(wait(f->side3, f->fork2));
    TRY(run_density_wall(c, p->support, p->h, true, p->rho0, p->c0, p->gamma, f->side3, p->block_sph, p->lanes_sph));
    TRY(rec(f->wall, f->side3));
    const int cap = nbr_cap(c, p);
    if (!density_fresh)
        TRY(run_density(c, p->support, p->h, shep, true, true, p->rho0, p->c0, p->gamma, st, p->block_sph,
                        p->lanes_sph, cap, p->nbr_format));
    TRY(rec(f->dens, st));
    // porosity branch.  One state: what needs positions only (the sorted
    // copies and the DEM grid) runs beside the density pass, the normaliser
    // after it -- there the porosity pass is the long branch.  A batched
    // state: all of it after the density pass, which is then the long one and
    // would lose SMs to the early kernels (measured: 64 dam breaks 1.25 ms
    // per step as one block, 1.30 split; one 800k dam break 4.04 vs 3.80)
    const float support = 2.0f * p->h_max;  // source/Simulation.py:208
    if (c->grid_sph.ninst <= 1) {
        TRY(wait(f->side2, f->fork2));
        TRY(wait(f->side2, f->ready));
        TRY(run_porosity(c, support, p->h_uniform, p->porosity_min, p->porosity_max, f->side2, p->porosity_variant,
                         1));
        TRY(wait(f->side2, f->dens));
        TRY(run_porosity(c, support, p->h_uniform, p->porosity_min, p->porosity_max, f->side2, p->porosity_variant,
                         2));
    } else {
        TRY(wait(f->side2, f->dens));
        TRY(wait(f->side2, f->ready));
        TRY(run_porosity(c, support, p->h_uniform, p->porosity_min, p->porosity_max, f->side2, p->porosity_variant,
                         0));
    }
    TRY(rec(f->join2, f->side2));
    // main, continued
    TRY(wait(st, f->wall));
    TRY(run_force(c, p->support, p->h, p->mu, p->g, 3, st, p->block_sph, p->lanes_sph, cap, p->nbr_format));
    TRY(wait(st, f->join));
    TRY(run_interaction_dem(c, p->mu, p->porosity_min, p->porosity_max, p->dt, st));
    TRY(wait(st, f->join2));
    TRY(run_react(c, support, p->dt, true, st));
    return run_step_dem(c, p->dt, st);
}

// ---------------------------------------------------------------------------
// sorted-copy refresh for the single-kernel entry points
// ---------------------------------------------------------------------------
__global__ void k_refresh_fluid(sphdem_sph_t P, const int* __restrict__ order, float4* posm, float4* vel,
                                float* vprev, float4* rp, float4* posv, float4* pgf) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= P.n) return;
    const int o = order[k];
    const float m = P.m[o], rho = P.rho[o], pr = P.pres[o];
    const float3 x = ld3(P.pos, o), v = ld3(P.vel, o), g = ld3(P.pgf, o);
    posm[k] = make_float4(x.x, x.y, x.z, m);
    vel[k] = make_float4(v.x, v.y, v.z, 0.f);
    vprev[k] = m / rho;
    rp[k] = make_float4(rho, pr, pr / (rho * rho), 1.0f / rho);
    posv[k] = make_float4(x.x, x.y, x.z, m / rho);
    pgf[k] = make_float4(g.x, g.y, g.z, rho);
}

__global__ void k_refresh_wall(sphdem_bnd_t B, const int* __restrict__ order, float4* posm, float4* vel, float* vprev,
                               float4* rp) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= B.n) return;
    const int o = order[k];
    const float m = B.m[o], rho = B.rho[o], pr = B.pres[o];
    const float3 x = ld3(B.pos, o), v = ld3(B.vel, o);
    posm[k] = make_float4(x.x, x.y, x.z, m);
    vel[k] = make_float4(v.x, v.y, v.z, 0.f);
    vprev[k] = m / rho;
    rp[k] = make_float4(rho, pr, pr / (rho * rho), 1.0f / rho);
}

// ---------------------------------------------------------------------------
// CUDA-graph replay of run_forward's loop body
// ---------------------------------------------------------------------------
struct GraphEntry {
    sphdem_ctx_t snap;
    sphdem_params_t params;
    int coupled = -1;
    cudaStream_t cap = nullptr;
    cudaGraphExec_t exec[2] = {nullptr, nullptr};
    int kernels[2] = {0, 0};
};
std::mutex g_graph_mu;
std::map<const sphdem_ctx_t*, GraphEntry> g_graphs;

void drop_entry(GraphEntry& e) {
    for (auto& x : e.exec)
        if (x) {
            cudaGraphExecDestroy(x);
            x = nullptr;
        }
}

int loop_body(sphdem_ctx_t* c, const sphdem_params_t* p, bool shep, int coupled, cudaStream_t st) {
    if (coupled) return coupled_onestep(c, p, shep, st, true);
    TRY(build_grid(&c->grid_sph, c->sph.pos, c->ctl, st));
    TRY(gather_fluid(c, st));
    return sph_onestep(c, p, shep, true, st);
}

int count_kernel_nodes(cudaGraph_t graph) {
    size_t n_nodes = 0;
    cudaGraphGetNodes(graph, nullptr, &n_nodes);
    int n_kernels = 0;
    if (n_nodes) {
        cudaGraphNode_t* nodes = new cudaGraphNode_t[n_nodes];
        cudaGraphGetNodes(graph, nodes, &n_nodes);
        for (size_t i = 0; i < n_nodes; ++i) {
            cudaGraphNodeType t;
            if (cudaGraphNodeGetType(nodes[i], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++n_kernels;
        }
        delete[] nodes;
    }
    return n_kernels;
}

int capture(sphdem_ctx_t* c, const sphdem_params_t* p, bool shep, int coupled, GraphEntry& e) {
    cudaError_t err = cudaStreamBeginCapture(e.cap, cudaStreamCaptureModeThreadLocal);
    if (err != cudaSuccess) {
        set_error("graph capture begin", err);
        return SPHDEM_ERR_CUDA;
    }
    int rc = loop_body(c, p, shep, coupled, e.cap);
    cudaGraph_t graph = nullptr;
    err = cudaStreamEndCapture(e.cap, &graph);
    if (rc) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
    }
    if (err != cudaSuccess) {
        set_error("graph capture end", err);
        return SPHDEM_ERR_CUDA;
    }
    e.kernels[shep ? 1 : 0] = count_kernel_nodes(graph);
    err = cudaGraphInstantiate(&e.exec[shep ? 1 : 0], graph, 0);
    cudaGraphDestroy(graph);
    if (err != cudaSuccess) {
        set_error("graph instantiate", err);
        return SPHDEM_ERR_CUDA;
    }
    return SPHDEM_OK;
}

// ---------------------------------------------------------------------------
// verification digests
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

struct DigArgs {
    Geo gsub, gnb;  // subject grid (instance lookup) and neighbour grid
    const float* spos;
    const float* npos;
    int nsub;
    int rel;
    float s, s2, rq, t;  // radius, s*s, padded radius, sqrt bound of s
    const float4* aux;  // per DEM (neighbour or subject)
    const float* flt_s;
    int32_t* count;
    uint64_t* hash;
};

__global__ void k_digest(DigArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.nsub) return;
    const float3 p = ld3(a.spos, i);
    const int inst = inst_of(a.gsub, i);
    float rq = a.rq, t = a.t;
    if (a.rel == SPHDEM_REL_DEM_SPH_2H || a.rel == SPHDEM_REL_DEM_DEM_2H) {
        rq = pad_radius(a.aux[i].w);
        t = a.aux[i].z;
    }
    int cnt = 0;
    uint64_t hs = 0;
    for_each_range_ball(a.gnb, p.x, p.y, p.z, rq, inst, [&](int s, int e) {
        for (int k = s; k < e; ++k) {
            const int j = a.gnb.order[k];
            const float3 q = ld3(a.npos, j);
            const D2 r = d2_exact(p.x, p.y, p.z, q.x, q.y, q.z);
            bool in = false;
            switch (a.rel) {
                case SPHDEM_REL_SPH_SPH_SUPPORT:
                case SPHDEM_REL_SPH_BND_SUPPORT:
                case SPHDEM_REL_BND_SPH_SUPPORT:
                case SPHDEM_REL_BND_BND_SUPPORT: in = r.d2 < a.s2; break;
                case SPHDEM_REL_SPH_SPH_FORCE:
                case SPHDEM_REL_SPH_BND_FORCE: in = r.d2 > kR2Min && r.d2 < a.s2; break;
                case SPHDEM_REL_SPH_SPH_LEN:
                case SPHDEM_REL_DEM_SPH_2H:
                case SPHDEM_REL_DEM_DEM_2H: in = r.d2 < t; break;
                case SPHDEM_REL_SPH_DEM_2H: in = r.d2 < a.aux[j].z; break;
                case SPHDEM_REL_SPH_DEM_REACT: in = r.d2 < a.aux[j].z && a.flt_s[j] > 1.0e-12f; break;
            }
            if (in) {
                ++cnt;
                hs += mix64((uint64_t)j);
            }
        }
    });
    a.count[i] = cnt;
    a.hash[i] = hs;
}

// Member digests of the hot-path kernels' own decisions (not a re-evaluation
// of the predicate): the density pass's recorded members (slots or walk
// masks), the members the force pass takes from them (or, for a particle whose
// record overflowed, from
// its own cell walk -- exactly the branch k_force takes), and the porosity
// pass's near list.  One thread per fluid slot; outputs by point index.
struct MemArgs {
    Geo gs, gb;
    const float4* __restrict__ f_posm;
    const float4* __restrict__ b_posm;
    const int* __restrict__ nbr;
    int cap, fmt, n, which;
    float s2, rq;
    int32_t* count;
    uint64_t* hash;
};

__global__ void k_member_digest(MemArgs a) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= a.n) return;
    const int o = a.gs.order[k];
    const float4 p = a.f_posm[k];
    const bool wall = a.which == SPHDEM_MEMBERS_DENSITY_WALL || a.which == SPHDEM_MEMBERS_FORCE_WALL;
    const bool force = a.which == SPHDEM_MEMBERS_FORCE_FLUID || a.which == SPHDEM_MEMBERS_FORCE_WALL;
    const size_t n = (size_t)a.n;
    bool listed = false;
    const bool masks = a.fmt == SPHDEM_NBR_MASKS;
    if (a.nbr && a.cap > 0) {
        const int cf = a.nbr[(size_t)(2 * a.cap) * n + k];
        const int cb = a.nbr[(size_t)(2 * a.cap + 1) * n + k];
        // the force pass reads both records only when neither overflowed; the
        // density pass's record of one kind is complete when it fits
        const int lim = masks ? 32 * a.cap : a.cap;
        listed = force ? (cf <= lim && cb <= lim) : (wall ? cb <= lim : cf <= lim);
    }
    int cnt = 0;
    uint64_t hs = 0;
    const Geo& G = wall ? a.gb : a.gs;
    const float4* q4 = wall ? a.b_posm : a.f_posm;
    auto take = [&](int j) {
        if (force) {
            const float4 q = q4[j];
            const D2 r = d2_exact(p.x, p.y, p.z, q.x, q.y, q.z);
            if (!(r.d2 > kR2Min)) return;
        }
        ++cnt;
        hs += mix64((uint64_t)G.order[j]);
    };
    const int inst = inst_of(a.gs, o);
    const int32_t* rows = a.nbr ? a.nbr + (wall ? (size_t)a.cap * n : 0) : nullptr;
    if (G.ncl <= 0) {
    } else if (listed && masks) {
        MaskIter it;
        it.init(G, p.x, p.y, p.z, a.rq);
        for (int j; (j = it.next(G, p.x, p.y, p.z, a.rq, inst, rows, n, k, a.cap)) >= 0;) take(j);
    } else if (listed) {
        const int c = a.nbr[(size_t)(2 * a.cap + (wall ? 1 : 0)) * n + k];
        for (int t = 0; t < c; ++t) take(rows[(size_t)t * n + k]);
    } else {
        for_each_range_ball(G, p.x, p.y, p.z, a.rq, inst, [&](int s, int e) {
            for (int j = s; j < e; ++j) {
                const float4 q = q4[j];
                const D2 r = d2_exact(p.x, p.y, p.z, q.x, q.y, q.z);
                if (r.d2 < a.s2) take(j);
            }
        });
    }
    a.count[o] = cnt;
    a.hash[o] = hs;
}

// Near-list membership: count[point] = 1 for every listed fluid slot.
__global__ void k_near_digest(const int* __restrict__ order, const int* __restrict__ near_list,
                              const sphdem_ctl_t* __restrict__ ctl, int n, int32_t* count, uint64_t* hash) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int nn = ctl->n_near;
    if (i >= nn || i >= n) return;
    const int o = order[near_list[i]];
    count[o] = 1;
    hash[o] = 0;
}

// ---------------------------------------------------------------------------
// FP64 diagnostics (no reference counterpart): one block, fixed order.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(1024) k_diag(sphdem_sph_t P, sphdem_dem_t D, float g, double* out) {
    __shared__ double red[32][8];
    double s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int i = threadIdx.x; i < P.n; i += blockDim.x) {
        const double m = P.m[i], vx = P.vel[3 * i], vy = P.vel[3 * i + 1], vz = P.vel[3 * i + 2];
        s[0] += m;
        s[2] += m * vx;
        s[3] += m * vy;
        s[4] += m * vz;
        s[5] += 0.5 * m * (vx * vx + vy * vy + vz * vz);
        s[7] += m * (double)g * (double)P.pos[3 * i + 2];
    }
    for (int a = threadIdx.x; a < D.n; a += blockDim.x) {
        const double m = D.m[a], vx = D.vel[3 * a], vy = D.vel[3 * a + 1], vz = D.vel[3 * a + 2];
        const double wx = D.omega[3 * a], wy = D.omega[3 * a + 1], wz = D.omega[3 * a + 2];
        s[1] += m;
        s[2] += m * vx;
        s[3] += m * vy;
        s[4] += m * vz;
        s[5] += 0.5 * m * (vx * vx + vy * vy + vz * vz);
        s[6] += 0.5 * (double)D.inertia[a] * (wx * wx + wy * wy + wz * wz);
        s[7] += m * (double)g * (double)D.pos[3 * a + 2];
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int c = 0; c < 8; ++c) {
        const double v = warp_sum(s[c]);
        if (lane == 0) red[wid][c] = v;
    }
    __syncthreads();
    if (threadIdx.x < 8) {
        double t = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += red[k][threadIdx.x];
        out[threadIdx.x] = t;
    }
}

// Self-test of the bounded shared-memory barrier wait every staged kernel
// uses: a barrier that expects one arrival which never comes (no bulk copy
// or MMA is issued, so nothing asynchronous can be left in flight), polled
// `polls` times; on giving up the kernel raises SPHDEM_FLAG_TIMEOUT, as the
// production kernels do, and returns.
__global__ void k_wait_selftest(sphdem_ctl_t* ctl, int polls) {
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    const bool landed = mbar_wait(&bar, 0u, polls);
    if (__syncthreads_or(!landed) && threadIdx.x == 0) flag(ctl, SPHDEM_FLAG_TIMEOUT);
}

__global__ void k_wendland(const float* r, int n, Kern k, float* w, float* dw) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    w[i] = kern_w(k, r[i]);
    dw[i] = kern_dw(k, r[i]);
}

bool valid_ctx(const sphdem_ctx_t* c) {
    if (!c || !c->ctl) {
        set_error_msg("null context or control block");
        return false;
    }
    return true;
}

}  // namespace
namespace {

// The jump's backup (or its restore) in one launch: five contiguous segments.
struct KeepArgs {
    float* dst[5];
    const float* src[5];
    long len[5];
};
__global__ void k_keep(KeepArgs a) {
    pdl_wait();
    pdl_launch();
    const long stride = (long)gridDim.x * blockDim.x;
#pragma unroll 1
    for (int s = 0; s < 5; ++s)
        for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < a.len[s]; i += stride) a.dst[s][i] = a.src[s][i];
}

// stats: [0] jumps, [1] fallbacks, [2] largest accepted density judge value
// (float bits; values are >= 0), [3] 1 if the last jump fell back, [4]
// largest accepted position term (float bits).  One thread.
__global__ void k_decide(const float* __restrict__ dev, const sphdem_ctl_t* __restrict__ gctl, float tol,
                         float pos_tol, cudaGraphConditionalHandle cond, int32_t* __restrict__ stats) {
    const float d = dev[0], dx = dev[1];
    // NaN, a density change above tol, a correction beyond pos_tol, or a graph/kernel flag: fall back
    const bool fall = !(d <= tol) || (pos_tol > 0.0f && !(dx <= pos_tol)) || gctl->status != 0;
    stats[0] += 1;
    if (fall) {
        stats[1] += 1;
    } else {
        stats[2] = max(stats[2], __float_as_int(d));
        stats[4] = max(stats[4], __float_as_int(dx));
    }
    stats[3] = fall ? 1 : 0;
    cudaGraphSetConditional(cond, fall ? 1u : 0u);
}

}  // namespace

}  // namespace sd

using namespace sd;

// ===========================================================================
// extern "C"
// ===========================================================================
extern "C" {

int sphdem_abi_version(void) { return SPHDEM_ABI_VERSION; }
const char* sphdem_last_error(void) { return g_err; }

// sizeof of the ABI structs, so a binding can check its mirror of them.
int sphdem_struct_sizes(int64_t* out, int n) {
    const int64_t s[] = {(int64_t)sizeof(sphdem_sph_t),   (int64_t)sizeof(sphdem_bnd_t),
                         (int64_t)sizeof(sphdem_csr_t),   (int64_t)sizeof(sphdem_dem_t),
                         (int64_t)sizeof(sphdem_dembnd_t), (int64_t)sizeof(sphdem_grid_t),
                         (int64_t)sizeof(sphdem_ctl_t),   (int64_t)sizeof(sphdem_work_t),
                         (int64_t)sizeof(sphdem_params_t), (int64_t)sizeof(sphdem_ctx_t),
                         (int64_t)sizeof(sphdem_mpnn_nodes_t), (int64_t)sizeof(sphdem_mpnn_net_t),
                         (int64_t)sizeof(sphdem_mpnn_grad_t), (int64_t)sizeof(sphdem_jump_t)};
    const int m = (int)(sizeof(s) / sizeof(s[0]));
    for (int i = 0; i < n && i < m; ++i) out[i] = s[i];
    return m;
}

int sphdem_porosity_scratch(const sphdem_ctx_t* c, int frame, int64_t* out) {
    if (!c || !out || frame < 0) {
        set_error_msg("porosity scratch: null context/output or negative frame edge");
        return SPHDEM_ERR_INVALID;
    }
    const int64_t nfb = porosity_frames(c->grid_sph, porosity_frame_edge(frame));
    const int64_t n = c->sph.n > 0 ? c->sph.n : 0;
    out[0] = 2 * (nfb + 1);
    out[1] = 4 * (n + 1);
    out[2] = n * SPHDEM_POROSITY_SLABS;
    out[3] = n;
    return SPHDEM_OK;
}

int sphdem_grid_build(sphdem_ctx_t* c, int kind, const sphdem_params_t* p, sphdem_stream_t stream) {
    if (!valid_ctx(c)) return SPHDEM_ERR_INVALID;
    cudaStream_t st = as_stream(stream);
    switch (kind) {
        case 0:
            // kernel attributes of the tensor-core porosity pass, set here --
            // eagerly, before any graph captures a step that launches it
            if (c->work.pfb) TRY(porosity_setup());
            TRY(build_grid(&c->grid_sph, c->sph.pos, c->ctl, st));
            return gather_fluid(c, st);
        case 1:
            TRY(build_grid(&c->grid_bnd, c->bnd.pos, c->ctl, st));
            if (!p) {
                set_error_msg("wall grid build needs params (support, h)");
                return SPHDEM_ERR_INVALID;
            }
            return gather_wall(c, p->support, p->h, st);
        case 2: return build_grid(&c->grid_dem, c->dem.pos, c->ctl, st);
        case 3: return build_grid(&c->grid_dembnd, c->dembnd.pos, c->ctl, st);
        default: set_error_msg("grid kind must be 0..3"); return SPHDEM_ERR_INVALID;
    }
}

int sphdem_refresh_sorted(sphdem_ctx_t* c, sphdem_stream_t stream) {
    if (!valid_ctx(c)) return SPHDEM_ERR_INVALID;
    cudaStream_t st = as_stream(stream);
    const sphdem_work_t& w = c->work;
    if (c->sph.n > 0)
        k_refresh_fluid<<<blocks_for(c->sph.n, 256), 256, 0, st>>>(
            c->sph, c->grid_sph.order, (float4*)w.f_posm, (float4*)w.f_vel, w.f_vprev, (float4*)w.f_rp,
            (float4*)w.f_posv, (float4*)w.f_pgf);
    if (c->bnd.n > 0)
        k_refresh_wall<<<blocks_for(c->bnd.n, 256), 256, 0, st>>>(c->bnd, c->grid_bnd.order, (float4*)w.b_posm,
                                                                  (float4*)w.b_vel, w.b_vprev, (float4*)w.b_rp);
    TRY(launch_status("refresh_sorted"));
    return run_dem_aux(c, st);
}

int sphdem_sph_onestep(sphdem_ctx_t* c, const sphdem_params_t* p, int step, int integrate, sphdem_stream_t s) {
    if (!valid_ctx(c) || !p) return SPHDEM_ERR_INVALID;
    return sph_onestep(c, p, shepard_due(p, step), integrate != 0, as_stream(s));
}

int sphdem_sphdem_onestep(sphdem_ctx_t* c, const sphdem_params_t* p, int step, sphdem_stream_t s) {
    if (!valid_ctx(c) || !p) return SPHDEM_ERR_INVALID;
    return coupled_onestep(c, p, shepard_due(p, step), as_stream(s));
}

int sphdem_run(sphdem_ctx_t* c, const sphdem_params_t* p, int first_step, int n_steps, int coupled,
               sphdem_stream_t stream) {
    if (!valid_ctx(c) || !p || n_steps < 0) return SPHDEM_ERR_INVALID;
    cudaStream_t st = as_stream(stream);
    std::lock_guard<std::mutex> lock(g_graph_mu);
    GraphEntry& e = g_graphs[c];
    if (e.coupled != coupled || memcmp(&e.snap, c, sizeof(*c)) != 0 || memcmp(&e.params, p, sizeof(*p)) != 0) {
        drop_entry(e);
        e.snap = *c;
        e.params = *p;
        e.coupled = coupled;
    }
    if (!e.cap) {
        cudaError_t err = cudaStreamCreateWithFlags(&e.cap, cudaStreamNonBlocking);
        if (err != cudaSuccess) {
            set_error("capture stream", err);
            return SPHDEM_ERR_CUDA;
        }
    }
    for (int k = 0; k < n_steps; ++k) {
        const bool shep = shepard_due(p, first_step + k);
        cudaGraphExec_t& x = e.exec[shep ? 1 : 0];
        if (!x) TRY(capture(c, p, shep, coupled, e));
        cudaError_t err = cudaGraphLaunch(x, st);
        if (err != cudaSuccess) {
            set_error("graph launch", err);
            return SPHDEM_ERR_CUDA;
        }
    }
    return SPHDEM_OK;
}

// ---------------------------------------------------------------------------
// learned jump (include/sphdem_mpnn.h)
// ---------------------------------------------------------------------------
namespace {

int jump_keep(sphdem_ctx_t* c, const sphdem_jump_t* j, bool restore, cudaStream_t st) {
    const long nf = c->sph.n, nd = c->dem.n;
    float* k = j->keep;
    float* live[5] = {c->sph.pos, c->sph.vel, c->dem.pos, c->dem.vel, c->sph.rho};
    const long len[5] = {3 * nf, 3 * nf, 3 * nd, 3 * nd, nf};
    KeepArgs a;
    long total = 0;
    for (int i = 0; i < 5; ++i) {
        a.dst[i] = restore ? live[i] : k;
        a.src[i] = restore ? k : live[i];
        a.len[i] = len[i];
        k += len[i];
        total += len[i];
    }
    if (total == 0) return SPHDEM_OK;
    const int grid = blocks_for(total / 5 + 1, 256) < 1024 ? blocks_for(total / 5 + 1, 256) : 1024;
    launch_pdl(k_keep, grid, 256, 0, st, a);
    return launch_status("jump keep");
}

// dens_fresh: the previous jump's judge (or fallback body) left this state's
// density pass done (device-judged rollouts).
int jump_body(sphdem_ctx_t* c, const sphdem_params_t* p, const sphdem_jump_t* j, bool shep, bool fresh,
              cudaStream_t st, bool dens_fresh = false) {
    TRY(coupled_onestep(c, p, shep, st, true, fresh, dens_fresh && fresh && !shep));
    TRY(jump_keep(c, j, false, st));
    TRY(sphdem_mpnn_nodes(&j->nodes, st));
    sphdem_grid_t g = j->node_grid;
    TRY(sphdem_mpnn_graph(&g, j->nodes.node_pos3, j->nodes.node_pos4, j->net.n_recv, j->radius, j->net.offset,
                          j->net.sender, j->net.receiver, j->net.edge_capacity, j->scan_scratch, j->graph_ctl, st));
    TRY(sphdem_mpnn_forward(&j->net, 0, st));
    TRY(sphdem_mpnn_apply(c->sph.pos, c->sph.vel, c->sph.acc, c->sph.n, c->dem.pos, c->dem.vel, c->dem.acc,
                          c->dem.n, j->net.out, j->substeps, p->dt, j->scale, nullptr, nullptr, nullptr, st));
    cudaError_t e = zero_words(j->dev, 2, st);
    if (e != cudaSuccess) {
        set_error("jump", e);
        return SPHDEM_ERR_CUDA;
    }
    TRY(run_corrmax(j->net.out, c->sph.n, c->dem.n, j->scale, (float)j->substeps * p->dt, j->dev + 1, st));
    TRY(build_grid(&c->grid_sph, c->sph.pos, c->ctl, st));
    TRY(gather_fluid(c, st));
    // the judge's density is the full density pass of the next plain step
    // (pressures, sorted copies, neighbour records), so that step can skip it
    TRY(run_density(c, p->support, p->h, false, true, true, p->rho0, p->c0, p->gamma, st, p->block_sph, p->lanes_sph,
                    nbr_cap(c, p), p->nbr_format));
    const float* rho_old = j->keep + 6 * (size_t)c->sph.n + 6 * (size_t)c->dem.n;
    return sphdem_mpnn_maxdev(c->sph.rho, j->judge == 1 ? nullptr : rho_old, p->rho0, c->sph.n, 1.0f / p->rho0,
                              j->dev, st);
}

struct JumpEntry {
    sphdem_ctx_t snap;
    sphdem_params_t params;
    sphdem_jump_t jump;
    cudaStream_t cap = nullptr;
    cudaGraphExec_t exec[4] = {nullptr, nullptr, nullptr, nullptr};  // [Shepard + 2 fresh]
    bool warm[4] = {false, false, false, false};
    int kernels[4] = {0, 0, 0, 0};
};
std::map<const sphdem_ctx_t*, JumpEntry> g_jumps;

}  // namespace

int sphdem_jump(sphdem_ctx_t* c, const sphdem_params_t* p, const sphdem_jump_t* j, int step, int32_t flags,
                sphdem_stream_t stream) {
    if (!valid_ctx(c) || !p || !j || !j->keep || !j->dev || !j->graph_ctl || !j->scan_scratch || j->substeps < 1 ||
        c->dem.n < 0) {
        set_error_msg("jump: invalid arguments");
        return SPHDEM_ERR_INVALID;
    }
    cudaStream_t st = as_stream(stream);
    const bool shep = shepard_due(p, step);
    std::lock_guard<std::mutex> lock(g_graph_mu);
    JumpEntry& e = g_jumps[c];
    if (memcmp(&e.snap, c, sizeof(*c)) != 0 || memcmp(&e.params, p, sizeof(*p)) != 0 ||
        memcmp(&e.jump, j, sizeof(*j)) != 0) {
        for (auto& x : e.exec)
            if (x) {
                cudaGraphExecDestroy(x);
                x = nullptr;
            }
        for (auto& w : e.warm) w = false;
        e.snap = *c;
        e.params = *p;
        e.jump = *j;
    }
    const bool fresh = (flags & SPHDEM_JUMP_GRID_FRESH) != 0;
    const int v = (shep ? 1 : 0) + (fresh ? 2 : 0);
    if (!e.warm[v]) {  // first use runs eagerly (one-time kernel attribute set-up), later ones replay
        e.warm[v] = true;
        return jump_body(c, p, j, shep, fresh, st);
    }
    if (!e.cap) {
        cudaError_t err = cudaStreamCreateWithFlags(&e.cap, cudaStreamNonBlocking);
        if (err != cudaSuccess) {
            set_error("jump capture stream", err);
            return SPHDEM_ERR_CUDA;
        }
    }
    if (!e.exec[v]) {
        cudaError_t err = cudaStreamBeginCapture(e.cap, cudaStreamCaptureModeThreadLocal);
        if (err != cudaSuccess) {
            set_error("jump capture begin", err);
            return SPHDEM_ERR_CUDA;
        }
        int rc = jump_body(c, p, j, shep, fresh, e.cap);
        cudaGraph_t graph = nullptr;
        err = cudaStreamEndCapture(e.cap, &graph);
        if (rc) {
            if (graph) cudaGraphDestroy(graph);
            return rc;
        }
        if (err != cudaSuccess) {
            set_error("jump capture end", err);
            return SPHDEM_ERR_CUDA;
        }
        e.kernels[v] = count_kernel_nodes(graph);
        err = cudaGraphInstantiate(&e.exec[v], graph, 0);
        cudaGraphDestroy(graph);
        if (err != cudaSuccess) {
            set_error("jump graph instantiate", err);
            return SPHDEM_ERR_CUDA;
        }
    }
    cudaError_t err = cudaGraphLaunch(e.exec[v], st);
    if (err != cudaSuccess) {
        set_error("jump graph launch", err);
        return SPHDEM_ERR_CUDA;
    }
    return SPHDEM_OK;
}

int sphdem_jump_kernels(sphdem_ctx_t* c, int variant) {
    std::lock_guard<std::mutex> lock(g_graph_mu);
    auto it = g_jumps.find(c);
    if (it == g_jumps.end() || variant < 0 || variant > 3 || !it->second.exec[variant]) return -1;
    return it->second.kernels[variant];
}

int sphdem_jump_undo(sphdem_ctx_t* c, const sphdem_jump_t* j, sphdem_stream_t stream) {
    if (!valid_ctx(c) || !j || !j->keep) {
        set_error_msg("jump_undo: invalid arguments");
        return SPHDEM_ERR_INVALID;
    }
    return jump_keep(c, j, true, as_stream(stream));
}

// ---------------------------------------------------------------------------
// device-judged rollout: the jumps are replayed back to back with no host
// round trip.  Each rollout graph is the jump's graph plus a judge kernel
// that sets a conditional node: non-zero runs the fallback body (undo the
// substeps, m plain steps, then the fluid re-bin and density pass the next
// jump relies on: after any jump of a rollout, the next one's plain step
// skips both unless its step refreshes the Shepard normaliser).
// ---------------------------------------------------------------------------
namespace {

struct RolloutEntry {
    sphdem_ctx_t snap;
    sphdem_params_t params;
    sphdem_jump_t jump;
    float tol = 0.0f;
    int32_t* stats = nullptr;
    cudaStream_t cap = nullptr;
    // key: Shepard pattern of the K steps and of the next jump's first step, * 2 + fresh
    std::map<int64_t, cudaGraphExec_t> exec;
    std::map<int64_t, std::pair<int, int>> kernels;  // key -> (jump graph, fallback body) kernel nodes
};
std::map<const sphdem_ctx_t*, RolloutEntry> g_rollouts;

void drop_rollout(RolloutEntry& e) {
    for (auto& kv : e.exec)
        if (kv.second) cudaGraphExecDestroy(kv.second);
    e.exec.clear();
    e.kernels.clear();
}

int capture_err(const char* what, cudaError_t e) {
    set_error(what, e);
    return SPHDEM_ERR_CUDA;
}

// Capture the rollout graph of a jump starting at `step`.
int capture_rollout(sphdem_ctx_t* c, const sphdem_params_t* p, const sphdem_jump_t* j, int step, bool fresh,
                    float tol, int32_t* stats, cudaStream_t cap, cudaGraphExec_t* out, std::pair<int, int>* nk) {
    const bool shep = shepard_due(p, step);
    cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return capture_err("rollout capture begin", e);
    cudaStreamCaptureStatus cs;
    cudaGraph_t graph = nullptr;
    cudaGraphConditionalHandle cond = 0;
    e = cudaStreamGetCaptureInfo(cap, &cs, nullptr, &graph);
    if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&cond, graph, 0, cudaGraphCondAssignDefault);
    int rc = e == cudaSuccess ? jump_body(c, p, j, shep, fresh, cap, fresh) : SPHDEM_ERR_CUDA;
    cudaGraph_t body = nullptr;
    if (!rc) {
        k_decide<<<1, 1, 0, cap>>>(j->dev, j->graph_ctl, tol, j->pos_tol, cond, stats);
        const cudaGraphNode_t* deps = nullptr;
        size_t nd = 0;
        e = cudaStreamGetCaptureInfo(cap, &cs, nullptr, nullptr, &deps, nullptr, &nd);
        cudaGraphNodeParams np = {};
        np.type = cudaGraphNodeTypeConditional;
        np.conditional.handle = cond;
        np.conditional.type = cudaGraphCondTypeIf;
        np.conditional.size = 1;
        cudaGraphNode_t node = nullptr;
        if (e == cudaSuccess) e = cudaGraphAddNode(&node, graph, deps, nullptr, nd, &np);
        if (e == cudaSuccess) e = cudaStreamUpdateCaptureDependencies(cap, &node, nullptr, 1,
                                                                       cudaStreamSetCaptureDependencies);
        if (e == cudaSuccess) body = np.conditional.phGraph_out[0];
        if (e != cudaSuccess) rc = capture_err("rollout conditional", e);
    }
    cudaGraph_t done = nullptr;
    e = cudaStreamEndCapture(cap, &done);
    if (rc || e != cudaSuccess) {
        if (done) cudaGraphDestroy(done);
        return rc ? rc : capture_err("rollout capture end", e);
    }
    // the fallback body
    e = cudaStreamBeginCaptureToGraph(cap, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
        cudaGraphDestroy(done);
        return capture_err("rollout body capture", e);
    }
    rc = jump_keep(c, j, true, cap);
    for (int s = 1; !rc && s <= j->substeps; ++s) rc = loop_body(c, p, shepard_due(p, step + s), 1, cap);
    if (!rc) rc = build_grid(&c->grid_sph, c->sph.pos, c->ctl, cap);
    // and the density pass of the next jump's plain step, as a judge leaves it
    // -- unless that step refreshes the Shepard normaliser: it then runs its
    // own, from m / rho of this step's density (which must stay in place)
    if (!rc && !shepard_due(p, step + j->substeps + 1)) {
        rc = gather_fluid(c, cap);
        if (!rc)
            rc = run_density(c, p->support, p->h, false, true, true, p->rho0, p->c0, p->gamma, cap, p->block_sph,
                             p->lanes_sph, nbr_cap(c, p), p->nbr_format);
    }
    cudaGraph_t body_done = nullptr;
    e = cudaStreamEndCapture(cap, &body_done);
    if (rc || e != cudaSuccess) {
        cudaGraphDestroy(done);
        return rc ? rc : capture_err("rollout body capture end", e);
    }
    nk->first = count_kernel_nodes(done) ;
    nk->second = count_kernel_nodes(body);
    e = cudaGraphInstantiate(out, done, 0);
    cudaGraphDestroy(done);
    if (e != cudaSuccess) return capture_err("rollout graph instantiate", e);
    return SPHDEM_OK;
}

}  // namespace

int sphdem_rollout(sphdem_ctx_t* c, const sphdem_params_t* p, const sphdem_jump_t* j, int first_step, int n_jumps,
                   float tol, int32_t flags, int32_t* stats, sphdem_stream_t stream) {
    if (!valid_ctx(c) || !p || !j || !j->keep || !j->dev || !j->graph_ctl || !j->scan_scratch || j->substeps < 1 ||
        j->substeps > 29 || !stats || n_jumps < 0) {  // graphs keyed by the Shepard pattern of the K steps
        set_error_msg("rollout: invalid arguments (1 <= substeps <= 29)");
        return SPHDEM_ERR_INVALID;
    }
    cudaStream_t st = as_stream(stream);
    const int K = j->substeps + 1;
    std::lock_guard<std::mutex> lock(g_graph_mu);
    RolloutEntry& e = g_rollouts[c];
    if (memcmp(&e.snap, c, sizeof(*c)) != 0 || memcmp(&e.params, p, sizeof(*p)) != 0 ||
        memcmp(&e.jump, j, sizeof(*j)) != 0 || e.tol != tol || e.stats != stats) {
        drop_rollout(e);
        e.snap = *c;
        e.params = *p;
        e.jump = *j;
        e.tol = tol;
        e.stats = stats;
    }
    if (!e.cap) {
        cudaError_t err = cudaStreamCreateWithFlags(&e.cap, cudaStreamNonBlocking);
        if (err != cudaSuccess) return capture_err("rollout capture stream", err);
    }
    bool fresh = (flags & SPHDEM_JUMP_GRID_FRESH) != 0;
    for (int i = 0; i < n_jumps; ++i) {
        const int step = first_step + i * K;
        int64_t pattern = 0;
        for (int s = 0; s <= K; ++s) pattern |= shepard_due(p, step + s) ? (int64_t(1) << s) : 0;
        const int64_t key = pattern * 2 + (fresh ? 1 : 0);
        auto it = e.exec.find(key);
        if (it == e.exec.end()) {
            cudaGraphExec_t x = nullptr;
            std::pair<int, int> nk(0, 0);
            int rc = capture_rollout(c, p, j, step, fresh, tol, stats, e.cap, &x, &nk);
            if (rc) return rc;
            it = e.exec.emplace(key, x).first;
            e.kernels[key] = nk;
        }
        cudaError_t err = cudaGraphLaunch(it->second, st);
        if (err != cudaSuccess) return capture_err("rollout graph launch", err);
        fresh = true;  // an accepted jump's judge, or the fallback body, re-binned the fluid
    }
    return SPHDEM_OK;
}

// Kernel nodes per rollout jump: accepted (body = 0) or fallback body (body = 1),
// summed over the graphs captured for this context; -1 if none.
int64_t sphdem_rollout_kernels(sphdem_ctx_t* c, int first_step, int n_jumps, int32_t flags, int body) {
    std::lock_guard<std::mutex> lock(g_graph_mu);
    auto it = g_rollouts.find(c);
    if (it == g_rollouts.end()) return -1;
    const RolloutEntry& e = it->second;
    const int K = e.jump.substeps + 1;
    bool fresh = (flags & SPHDEM_JUMP_GRID_FRESH) != 0;
    int64_t total = 0;
    for (int i = 0; i < n_jumps; ++i) {
        int64_t pattern = 0;
        for (int s = 0; s <= K; ++s)
            pattern |= shepard_due(&e.params, first_step + i * K + s) ? (int64_t(1) << s) : 0;
        auto k = e.kernels.find(pattern * 2 + (fresh ? 1 : 0));
        if (k == e.kernels.end()) return -1;
        total += body ? k->second.second : k->second.first;
        fresh = true;
    }
    return total;
}

// Blocking helper: one loop body of run_forward (moving-grid rebuild + one
// step) with a CUDA event between phases on the launch stream; fills ms[k]
// with the duration of phase k (SPHDEM_PHASE_* order) and synchronises.
int sphdem_profile_step(sphdem_ctx_t* c, const sphdem_params_t* p, int step, int coupled, float* ms,
                        sphdem_stream_t stream) {
    if (!valid_ctx(c) || !p || !ms) return SPHDEM_ERR_INVALID;
    cudaStream_t st = as_stream(stream);
    cudaEvent_t ev[SPHDEM_PHASE_COUNT + 1];
    for (auto& e : ev)
        if (cudaEventCreate(&e) != cudaSuccess) return launch_status("profile events");
    const bool shep = shepard_due(p, step);
    int k = 0;
    auto mark = [&]() { cudaEventRecord(ev[k++], st); };
    int rc = SPHDEM_OK;
    do {
        mark();
        if ((rc = build_grid(&c->grid_sph, c->sph.pos, c->ctl, st)) || (rc = gather_fluid(c, st))) break;
        mark();
        if (coupled && (rc = build_grid(&c->grid_dem, c->dem.pos, c->ctl, st))) break;
        mark();
        if (shep && (rc = gather_wall_rho(c, st))) break;
        if ((rc = run_density(c, p->support, p->h, shep, true, true, p->rho0, p->c0, p->gamma, st, p->block_sph,
                              p->lanes_sph, nbr_cap(c, p), p->nbr_format)))
            break;
        mark();
        if ((rc = run_density_wall(c, p->support, p->h, true, p->rho0, p->c0, p->gamma, st, p->block_sph, p->lanes_sph))) break;
        mark();
        sphdem_ctx_t cc = *c;
        if (!coupled) cc.sph.pgf = nullptr;
        if ((rc = run_force(&cc, p->support, p->h, p->mu, p->g, 3, st, p->block_sph, p->lanes_sph, nbr_cap(c, p),
                            p->nbr_format)))
            break;
        mark();
        if (coupled && (rc = run_contacts(c, p->radius_max, p->boundary_radius_max, p->g, p->dt, 3, st))) break;
        mark();
        const float support = 2.0f * p->h_max;
        if (coupled && ((rc = run_dem_aux(c, st)) ||
                        (rc = run_porosity(c, support, p->h_uniform, p->porosity_min, p->porosity_max, st,
                                           p->porosity_variant))))
            break;
        mark();
        if (coupled && (rc = run_interaction_dem(c, p->mu, p->porosity_min, p->porosity_max, p->dt, st))) break;
        mark();
        if (coupled ? (rc = run_react(c, support, p->dt, true, st)) : (rc = run_step_sph(c, p->dt, st))) break;
        mark();
        if (coupled && (rc = run_step_dem(c, p->dt, st))) break;
        mark();
    } while (0);
    if (!rc) {
        cudaError_t e = cudaEventSynchronize(ev[SPHDEM_PHASE_COUNT]);
        if (e != cudaSuccess) {
            set_error("profile sync", e);
            rc = SPHDEM_ERR_CUDA;
        }
    }
    for (int i = 0; !rc && i < SPHDEM_PHASE_COUNT; ++i) cudaEventElapsedTime(&ms[i], ev[i], ev[i + 1]);
    for (auto& e : ev) cudaEventDestroy(e);
    return rc;
}

// Kernel nodes in the captured loop-body graph of ctx (variant 1: Shepard
// step, 0: other steps); -1 if that graph has not been captured.
int sphdem_graph_kernels(sphdem_ctx_t* c, int variant) {
    std::lock_guard<std::mutex> lock(g_graph_mu);
    auto it = g_graphs.find(c);
    if (it == g_graphs.end() || !it->second.exec[variant ? 1 : 0]) return -1;
    return it->second.kernels[variant ? 1 : 0];
}

int sphdem_release(sphdem_ctx_t* c) {
    std::lock_guard<std::mutex> lock(g_graph_mu);
    auto jt = g_jumps.find(c);
    if (jt != g_jumps.end()) {
        for (auto& x : jt->second.exec)
            if (x) cudaGraphExecDestroy(x);
        if (jt->second.cap) cudaStreamDestroy(jt->second.cap);
        g_jumps.erase(jt);
    }
    auto rt = g_rollouts.find(c);
    if (rt != g_rollouts.end()) {
        drop_rollout(rt->second);
        if (rt->second.cap) cudaStreamDestroy(rt->second.cap);
        g_rollouts.erase(rt);
    }
    auto it = g_graphs.find(c);
    if (it == g_graphs.end()) return SPHDEM_OK;
    drop_entry(it->second);
    if (it->second.cap) cudaStreamDestroy(it->second.cap);
    g_graphs.erase(it);
    return SPHDEM_OK;
}

int sphdem_shepard_sph(sphdem_ctx_t* c, float support, float h, sphdem_stream_t s) {
    if (!valid_ctx(c)) return SPHDEM_ERR_INVALID;
    return run_density(c, support, h, true, false, false, 1.f, 1.f, 1.f, as_stream(s));
}
int sphdem_density_sph(sphdem_ctx_t* c, float support, float h, sphdem_stream_t s) {
    if (!valid_ctx(c)) return SPHDEM_ERR_INVALID;
    return run_density(c, support, h, false, true, false, 1.f, 1.f, 1.f, as_stream(s));
}
int sphdem_density_bnd(sphdem_ctx_t* c, float support, float h, sphdem_stream_t s) {
    if (!valid_ctx(c)) return SPHDEM_ERR_INVALID;
    return run_density_wall(c, support, h, false, 1.f, 1.f, 1.f, as_stream(s));
}
int sphdem_pres_sph(sphdem_ctx_t* c, float rho0, float c0, float gamma, sphdem_stream_t s) {
    if (!valid_ctx(c)) return SPHDEM_ERR_INVALID;
    return run_pres(c->sph.rho, c->sph.pres, c->sph.n, rho0, c0, gamma, as_stream(s));
}
int sphdem_pres_bnd(sphdem_ctx_t* c, float rho0, float c0, float gamma, sphdem_stream_t s) {
    if (!valid_ctx(c)) return SPHDEM_ERR_INVALID;
    return run_pres(c->bnd.rho, c->bnd.pres, c->bnd.n, rho0, c0, gamma, as_stream(s));
}
int sphdem_force_sph(sphdem_ctx_t* c, float support, float h, float mu, float g, sphdem_stream_t s) {
    if (!valid_ctx(c)) return SPHDEM_ERR_INVALID;
    return run_force(c, support, h, mu, g, 1, as_stream(s));
}
int sphdem_step_sph(sphdem_ctx_t* c, float dt, sphdem_stream_t s) {
    if (!valid_ctx(c)) return SPHDEM_ERR_INVALID;
    return run_step_sph(c, dt, as_stream(s));
}
int sphdem_force_dem(sphdem_ctx_t* c, float radius_max, float g, float dt, sphdem_stream_t s) {
    if (!valid_ctx(c)) return SPHDEM_ERR_INVALID;
    return run_contacts(c, radius_max, 0.0f, g, dt, 1, as_stream(s));
}
int sphdem_bc_dem(sphdem_ctx_t* c, float radius_max, float dt, sphdem_stream_t s) {
    if (!valid_ctx(c)) return SPHDEM_ERR_INVALID;
    return run_contacts(c, 0.0f, radius_max, 0.0f, dt, 2, as_stream(s));
}
int sphdem_step_dem(sphdem_ctx_t* c, float dt, sphdem_stream_t s) {
    if (!valid_ctx(c)) return SPHDEM_ERR_INVALID;
    return run_step_dem(c, dt, as_stream(s));
}
int sphdem_prep_sphdem(sphdem_ctx_t* c, float support, float h, float sph_support, float sph_h, float eps_min,
                       float eps_max, sphdem_stream_t s) {
    if (!valid_ctx(c)) return SPHDEM_ERR_INVALID;
    cudaStream_t st = as_stream(s);
    TRY(run_dem_aux(c, st));
    // the tensor-core normaliser when the context carries its scratch
    TRY(run_porosity(c, support, h, eps_min, eps_max, st, c->work.pfb ? 2 : 0));
    sphdem_ctx_t cc = *c;  // -grad p only (mode 2)
    return run_force(&cc, sph_support, sph_h, 0.0f, 0.0f, 2, st);
}
int sphdem_interaction_dem(sphdem_ctx_t* c, float mu, float eps_min, float eps_max, float dt, sphdem_stream_t s) {
    if (!valid_ctx(c)) return SPHDEM_ERR_INVALID;
    cudaStream_t st = as_stream(s);
    TRY(run_dem_aux(c, st));
    return run_interaction_dem(c, mu, eps_min, eps_max, dt, st);
}
int sphdem_interaction_sph(sphdem_ctx_t* c, float support, sphdem_stream_t s) {
    if (!valid_ctx(c)) return SPHDEM_ERR_INVALID;
    cudaStream_t st = as_stream(s);
    TRY(run_dem_aux(c, st));
    return run_react(c, support, 0.0f, false, st);
}

int sphdem_wendland(const float* r, int32_t n, float h, float* w, float* dw, sphdem_stream_t s) {
    if (n <= 0) return SPHDEM_OK;
    k_wendland<<<blocks_for(n, 256), 256, 0, as_stream(s)>>>(r, n, make_kern(h), w, dw);
    return launch_status("wendland");
}

int sphdem_drag_beta(const float* eps, const float* rho, const float* mu, const float* d, const float* speed,
                     int32_t n, float* out, sphdem_stream_t s) {
    return run_drag_beta(eps, rho, mu, d, speed, n, out, as_stream(s));
}

int sphdem_wait_selftest(sphdem_ctl_t* ctl, int polls, sphdem_stream_t s) {
    if (!ctl || polls < 0 || polls > (1 << 20)) {
        set_error_msg("wait self-test: control block and 0 <= polls <= 2^20 required");
        return SPHDEM_ERR_INVALID;
    }
    k_wait_selftest<<<1, 64, 0, as_stream(s)>>>(ctl, polls);
    return launch_status("wait self-test");
}

int sphdem_member_digest(sphdem_ctx_t* c, const sphdem_params_t* p, int which, int32_t* count, uint64_t* hash,
                         sphdem_stream_t s) {
    if (!valid_ctx(c) || !p || !count || !hash) return SPHDEM_ERR_INVALID;
    if (which < 0 || which >= SPHDEM_MEMBERS_COUNT) {
        set_error_msg("unknown member set");
        return SPHDEM_ERR_INVALID;
    }
    cudaStream_t st = as_stream(s);
    const int n = c->sph.n;
    if (n <= 0) return SPHDEM_OK;
    if (which == SPHDEM_MEMBERS_POROSITY_NEAR) {
        TRY(zero_words(count, n, st));
        TRY(zero_words(hash, 2L * n, st));
        k_near_digest<<<blocks_for(n, 256), 256, 0, st>>>(c->grid_sph.order, c->work.near_list, c->ctl, n, count,
                                                          hash);
        return launch_status("near digest");
    }
    MemArgs a;
    a.gs = make_geo(c->grid_sph);
    a.gb = make_geo(c->grid_bnd);
    if (c->bnd.n <= 0) a.gb.ncl = 0;
    a.f_posm = (const float4*)c->work.f_posm;
    a.b_posm = (const float4*)c->work.b_posm;
    a.nbr = c->work.nbr;
    a.cap = nbr_cap(c, p);
    a.fmt = p->nbr_format;
    a.n = n;
    a.which = which;
    a.s2 = p->support * p->support;
    a.rq = pad_radius(p->support);
    a.count = count;
    a.hash = hash;
    k_member_digest<<<blocks_for(n, 128), 128, 0, st>>>(a);
    return launch_status("member digest");
}

int sphdem_neighbour_digest(sphdem_ctx_t* c, int rel, float radius, int32_t* count, uint64_t* hash,
                            sphdem_stream_t s) {
    if (!valid_ctx(c)) return SPHDEM_ERR_INVALID;
    if (rel < 0 || rel >= SPHDEM_REL_COUNT) {
        set_error_msg("unknown neighbour relation");
        return SPHDEM_ERR_INVALID;
    }
    cudaStream_t st = as_stream(s);
    TRY(run_dem_aux(c, st));
    DigArgs a;
    a.rel = rel;
    a.s = radius;
    a.s2 = radius * radius;
    a.rq = pad_radius(radius);
    a.t = sqrt_lt_bound(radius);
    a.aux = (const float4*)c->work.dem_aux;
    a.flt_s = c->dem.flt_s;
    a.count = count;
    a.hash = hash;
    switch (rel) {
        case SPHDEM_REL_BND_SPH_SUPPORT:
        case SPHDEM_REL_BND_BND_SUPPORT:
            a.gsub = make_geo(c->grid_bnd);
            a.spos = c->bnd.pos;
            a.nsub = c->bnd.n;
            break;
        case SPHDEM_REL_DEM_SPH_2H:
        case SPHDEM_REL_DEM_DEM_2H:
            a.gsub = make_geo(c->grid_dem);
            a.spos = c->dem.pos;
            a.nsub = c->dem.n;
            break;
        default:
            a.gsub = make_geo(c->grid_sph);
            a.spos = c->sph.pos;
            a.nsub = c->sph.n;
    }
    switch (rel) {
        case SPHDEM_REL_SPH_BND_SUPPORT:
        case SPHDEM_REL_BND_BND_SUPPORT:
        case SPHDEM_REL_SPH_BND_FORCE:
            a.gnb = make_geo(c->grid_bnd);
            a.npos = c->bnd.pos;
            break;
        case SPHDEM_REL_SPH_DEM_2H:
        case SPHDEM_REL_DEM_DEM_2H:
        case SPHDEM_REL_SPH_DEM_REACT:
            a.gnb = make_geo(c->grid_dem);
            a.npos = c->dem.pos;
            break;
        default:
            a.gnb = make_geo(c->grid_sph);
            a.npos = c->sph.pos;
    }
    if (a.nsub <= 0) return SPHDEM_OK;
    k_digest<<<blocks_for(a.nsub, 128), 128, 0, st>>>(a);
    return launch_status("digest");
}

int sphdem_diagnostics(sphdem_ctx_t* c, float g, double* out, sphdem_stream_t s) {
    if (!valid_ctx(c)) return SPHDEM_ERR_INVALID;
    k_diag<<<1, 1024, 0, as_stream(s)>>>(c->sph, c->dem, g, out);
    return launch_status("diagnostics");
}

}  // extern "C"
