// grid.cu -- neighbour grid build: counting sort of points by cell.
//
// Replaces wp.HashGrid.build (main.py:66,73,85,87).  Steps, all on one stream
// (small grids: all in one CTA, k_build_one):
//   1. bin      key[i] = cell of point i, count[key]++            (atomics)
//   2. scan     exclusive prefix sum of the counts -> cell_start   (tiled scan)
//   3. scatter  order[cell_start[key] + rank] = i                 (atomics)
//   4. sort     each cell's slots by point index, so the order is stable and
//               every later sum is deterministic run to run
//   5. gather   sorted copies of the fields that neighbour loops read
// Memory: cell_start [ncell+1], order/key [n], cursor [ncell] and scan scratch
// are caller-owned tensors; nothing is allocated here.
#include <limits.h>
#include <stdio.h>
#include <string.h>

#include "common.cuh"

namespace sd {

namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;  // 1024 cells per tile

__global__ void k_bin(const float* __restrict__ pos, int n, const int* __restrict__ inst, int lo0, int lo1,
                      int lo2, int d0, int d1, int d2, float inv, int ncl, int* __restrict__ key,
                      int* __restrict__ count, sphdem_ctl_t* ctl) {
    pdl_wait();
    pdl_launch();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float x = pos[3 * i], y = pos[3 * i + 1], z = pos[3 * i + 2];
    if (!isfinite(x) || !isfinite(y) || !isfinite(z)) flag(ctl, SPHDEM_FLAG_NONFINITE);
    int cx = coord(x, inv, lo0, d0), cy = coord(y, inv, lo1, d1), cz = coord(z, inv, lo2, d2);
    int k = (inst ? inst[i] : 0) * ncl + (cx * d1 + cy) * d2 + cz;
    key[i] = k;
    atomicAdd(count + k, 1);
}

// Each block scans one tile in place (exclusive) and records its total.
__global__ void __launch_bounds__(kScanThreads) k_scan_tiles(int* __restrict__ data, int n, int* __restrict__ sums) {
    pdl_wait();
    pdl_launch();
    __shared__ int warp_tot[kScanThreads / 32];
    const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    int v[kScanItems];
    int s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        v[k] = base + k < n ? data[base + k] : 0;
        s += v[k];
    }
    int total;
    int run = block_exclusive_scan(s, warp_tot, total);
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        if (base + k < n) data[base + k] = run;
        run += v[k];
    }
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// One block: exclusive scan of nb tile totals in place; sums[nb] = grand total.
__global__ void __launch_bounds__(1024) k_scan_sums(int* __restrict__ sums, int nb) {
    pdl_wait();
    pdl_launch();
    __shared__ int warp_tot[32];
    int carry = 0;
    for (int base = 0; base < nb; base += blockDim.x) {
        int i = base + threadIdx.x;
        int v = i < nb ? sums[i] : 0;
        int total;
        int ex = block_exclusive_scan(v, warp_tot, total);
        if (i < nb) sums[i] = carry + ex;
        carry += total;
    }
    if (threadIdx.x == 0) sums[nb] = carry;
}

__global__ void k_scan_add(int* __restrict__ data, int n, const int* __restrict__ sums, int total_points) {
    pdl_wait();
    pdl_launch();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) data[i] += sums[i / kScanTile];
    if (i == 0) data[n] = total_points;
}

// As k_scan_add, with data[n] = the grand total left by k_scan_sums.
__global__ void k_scan_add_total(int* __restrict__ data, int n, const int* __restrict__ sums, int nb) {
    pdl_wait();
    pdl_launch();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) data[i] += sums[i / kScanTile];
    if (i == 0) data[n] = sums[nb];
}

__global__ void k_scatter(const int* __restrict__ key, int n, const int* __restrict__ start, int* __restrict__ cursor,
                          int* __restrict__ order) {
    pdl_wait();
    pdl_launch();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int k = key[i];
    order[start[k] + atomicAdd(cursor + k, 1)] = i;
}

// Stable order inside each cell: the slots of a cell sorted by point index.
// One thread checks each cell; the warp then sorts its lanes' cells that hold
// 2..32 points one after another, each in registers by a bitonic network of
// shuffles.  Longer cells (rare) fall back to an insertion sort by their lane.
__device__ __forceinline__ int warp_bitonic_sort(int v, int lane) {
#pragma unroll
    for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1) {
            const int o = __shfl_xor_sync(0xffffffffu, v, j);
            const bool up = (lane & k) == 0;
            const bool lower = (lane & j) == 0;
            v = (lower == up) ? min(v, o) : max(v, o);
        }
    }
    return v;
}

// The 32 cells c0 .. c0 + 31 (this lane: c0 + lane), warp-wide.
__device__ __forceinline__ void sort_cells_warp(const int* __restrict__ start, int ncell, int* __restrict__ order,
                                                int c0) {
    const int lane = threadIdx.x & 31;
    const int c = c0 + lane;
    int s = 0, n = 0;
    if (c < ncell) {
        s = start[c];
        n = start[c + 1] - s;
    }
    unsigned todo = __ballot_sync(0xffffffffu, n >= 2 && n <= 32);
    while (todo) {
        const int src = __ffs(todo) - 1;
        todo &= todo - 1;
        const int cs = __shfl_sync(0xffffffffu, s, src), cn = __shfl_sync(0xffffffffu, n, src);
        int v = lane < cn ? order[cs + lane] : INT_MAX;
        v = warp_bitonic_sort(v, lane);
        if (lane < cn) order[cs + lane] = v;
    }
    if (n > 32) {
        for (int a = s + 1; a < s + n; ++a) {
            int v = order[a];
            int b = a - 1;
            while (b >= s && order[b] > v) {
                order[b + 1] = order[b];
                --b;
            }
            order[b + 1] = v;
        }
    }
}

__global__ void k_sort_cells(const int* __restrict__ start, int ncell, int* __restrict__ order) {
    pdl_wait();
    pdl_launch();
    sort_cells_warp(start, ncell, order, (blockIdx.x * blockDim.x + threadIdx.x) & ~31);
}

// The whole build in one CTA, for small grids (at most kOneMaxPoints points
// and kOneMaxCells cells): the same bin, exclusive scan, scatter and per-cell
// sort as the multi-kernel path, phase after phase behind __syncthreads, so
// the cell starts and the order are the same; one launch instead of eight
// (small systems are bound by launch latency, not by these loops).
constexpr int kOneThreads = 1024;
constexpr int kOneMaxPoints = 4096;
constexpr int kOneMaxCells = 65536;

__global__ void __launch_bounds__(kOneThreads) k_build_one(const float* __restrict__ pos, int n,
                                                          const int* __restrict__ inst, int lo0, int lo1, int lo2,
                                                          int d0, int d1, int d2, float inv, int ncl, int ncell,
                                                          int* __restrict__ key, int* __restrict__ start,
                                                          int* __restrict__ cursor, int* __restrict__ order,
                                                          sphdem_ctl_t* ctl) {
    pdl_wait();
    pdl_launch();
    __shared__ int warp_tot[kOneThreads / 32];
    const int tid = threadIdx.x;
    for (int c = tid; c <= ncell; c += kOneThreads) start[c] = 0;
    for (int c = tid; c < ncell; c += kOneThreads) cursor[c] = 0;
    __syncthreads();
    for (int i = tid; i < n; i += kOneThreads) {
        const float x = pos[3 * i], y = pos[3 * i + 1], z = pos[3 * i + 2];
        if (!isfinite(x) || !isfinite(y) || !isfinite(z)) flag(ctl, SPHDEM_FLAG_NONFINITE);
        const int cx = coord(x, inv, lo0, d0), cy = coord(y, inv, lo1, d1), cz = coord(z, inv, lo2, d2);
        const int k = (inst ? inst[i] : 0) * ncl + (cx * d1 + cy) * d2 + cz;
        key[i] = k;
        atomicAdd(start + k, 1);
    }
    __syncthreads();
    // exclusive scan: each thread a contiguous chunk of cells
    const int per = (ncell + kOneThreads - 1) / kOneThreads;
    const int c0 = tid * per, c1 = min(c0 + per, ncell);
    int sum = 0;
    for (int c = c0; c < c1; ++c) sum += start[c];
    int total;
    int run = block_exclusive_scan(sum, warp_tot, total);
    for (int c = c0; c < c1; ++c) {
        const int v = start[c];
        start[c] = run;
        run += v;
    }
    if (tid == 0) start[ncell] = n;
    __syncthreads();
    for (int i = tid; i < n; i += kOneThreads) {
        const int k = key[i];
        order[start[k] + atomicAdd(cursor + k, 1)] = i;
    }
    __syncthreads();
    for (int c = tid & ~31; c < ncell; c += kOneThreads) sort_cells_warp(start, ncell, order, c);
}

__global__ void k_gather_fluid(const int* __restrict__ order, int n, const float* __restrict__ pos,
                               const float* __restrict__ m, const float* __restrict__ vel,
                               const float* __restrict__ rho, float4* __restrict__ posm, float4* __restrict__ velo,
                               float* __restrict__ vprev) {
    pdl_wait();
    pdl_launch();
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int o = order[k];
    posm[k] = make_float4(pos[3 * o], pos[3 * o + 1], pos[3 * o + 2], m[o]);
    velo[k] = make_float4(vel[3 * o], vel[3 * o + 1], vel[3 * o + 2], 0.0f);
    vprev[k] = m[o] / rho[o];
}

__global__ void k_gather_vol(const int* __restrict__ order, int n, const float* __restrict__ m,
                             const float* __restrict__ rho, float* __restrict__ out) {
    pdl_wait();
    pdl_launch();
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) {
        int o = order[k];
        out[k] = m[o] / rho[o];
    }
}

// Wall-only part of the wall density, sum_{wall j, d2 < s^2} m_j W(r, h)
// (the second loop of Kernel_density_bnd, kernel/KERNEL_rho.py:119-125).  Walls
// never move, so this sum is a constant of the wall grid and is cached here.
__global__ void k_wall_self(Geo gb, const float4* __restrict__ posm, int n, float s2, float rq, Kern kern,
                            float* __restrict__ self) {
    pdl_wait();
    pdl_launch();
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    float4 p = posm[k];
    int inst = inst_of(gb, gb.order[k]);
    float acc = 0.0f;
    for_each_range_ball(gb, p.x, p.y, p.z, rq, inst, [&](int s, int e) {
        for (int j = s; j < e; ++j) {
            float4 q = posm[j];
            D2 r = d2_exact(p.x, p.y, p.z, q.x, q.y, q.z);
            if (r.d2 < s2) acc += q.w * kern_w(kern, fast_sqrt(r.d2));
        }
    });
    self[k] = acc;
}

int scan_cells(int* data, int ncell, int total_points, int* sums, cudaStream_t st) {
    int nb = (ncell + kScanTile - 1) / kScanTile;
    if (nb < 1) nb = 1;
    launch_pdl(k_scan_tiles, nb, kScanThreads, 0, st, data, ncell, sums);
    launch_pdl(k_scan_sums, 1, 1024, 0, st, sums, nb);
    launch_pdl(k_scan_add, blocks_for(ncell > 0 ? ncell : 1, 256), 256, 0, st, data, ncell, sums, total_points);
    return launch_status("scan_cells");
}

}  // namespace

// Exclusive scan of n counts in place, data[n] = their total (device side).
int scan_counts(int* data, int n, int* sums, cudaStream_t st) {
    int nb = (n + kScanTile - 1) / kScanTile;
    if (nb < 1) nb = 1;
    launch_pdl(k_scan_tiles, nb, kScanThreads, 0, st, data, n, sums);
    launch_pdl(k_scan_sums, 1, 1024, 0, st, sums, nb);
    launch_pdl(k_scan_add_total, blocks_for(n > 0 ? n : 1, 256), 256, 0, st, data, n, sums, nb);
    return launch_status("scan_counts");
}

// Bin + scan + scatter + stable per-cell sort of the points of one grid.
int build_grid(sphdem_grid_t* g, const float* pos, sphdem_ctl_t* ctl, cudaStream_t st) {
    const int ncell = g->ninst * g->ncell_local;
    if (ncell <= 0 || g->n < 0) {
        set_error_msg("grid: empty cell box");
        return SPHDEM_ERR_INVALID;
    }
    const int n = g->n;
    if (n <= kOneMaxPoints && ncell <= kOneMaxCells) {
        launch_pdl(k_build_one, 1, kOneThreads, 0, st, pos, n, g->inst, g->lo[0], g->lo[1], g->lo[2], g->dim[0], g->dim[1],
                                               g->dim[2], g->inv_cell, g->ncell_local, ncell, g->key, g->cell_start,
                                               g->cursor, g->order, ctl);
        return launch_status("build_grid");
    }
    cudaError_t e1 = zero_words(g->cell_start, (long)ncell + 1, st);
    cudaError_t e2 = zero_words(g->cursor, (long)ncell, st);
    if (e1 != cudaSuccess || e2 != cudaSuccess) {
        set_error("grid memset", e1 != cudaSuccess ? e1 : e2);
        return SPHDEM_ERR_CUDA;
    }
    if (n > 0)
        launch_pdl(k_bin, blocks_for(n, 256), 256, 0, st, pos, n, g->inst, g->lo[0], g->lo[1], g->lo[2], g->dim[0],
                                                  g->dim[1], g->dim[2], g->inv_cell, g->ncell_local, g->key,
                                                  g->cell_start, ctl);
    int rc = scan_cells(g->cell_start, ncell, n, g->block_sums, st);
    if (rc) return rc;
    if (n > 0) {
        launch_pdl(k_scatter, blocks_for(n, 256), 256, 0, st, g->key, n, g->cell_start, g->cursor, g->order);
        launch_pdl(k_sort_cells, blocks_for(ncell, 256), 256, 0, st, g->cell_start, ncell, g->order);
    }
    return launch_status("build_grid");
}

int gather_fluid(const sphdem_ctx_t* c, cudaStream_t st) {
    const int n = c->sph.n;
    if (n <= 0) return SPHDEM_OK;
    launch_pdl(k_gather_fluid, blocks_for(n, 256), 256, 0, st, c->grid_sph.order, n, c->sph.pos, c->sph.m, c->sph.vel,
                                                      c->sph.rho, (float4*)c->work.f_posm,
                                                      (float4*)c->work.f_vel, c->work.f_vprev);
    return launch_status("gather_fluid");
}

int gather_wall(const sphdem_ctx_t* c, float support, float h, cudaStream_t st) {
    const int n = c->bnd.n;
    if (n <= 0) return SPHDEM_OK;
    // Same gather as the fluid (x, y, z, m), then the wall self density.
    launch_pdl(k_gather_fluid, blocks_for(n, 256), 256, 0, st, c->grid_bnd.order, n, c->bnd.pos, c->bnd.m, c->bnd.vel,
                                                      c->bnd.rho, (float4*)c->work.b_posm,
                                                      (float4*)c->work.b_vel, c->work.b_vprev);
    Geo gb = make_geo(c->grid_bnd);
    launch_pdl(k_wall_self, blocks_for(n, 128), 128, 0, st, gb, (const float4*)c->work.b_posm, n, support * support,
                                                    pad_radius(support), make_kern(h), c->work.b_self);
    return launch_status("gather_wall");
}

int gather_wall_rho(const sphdem_ctx_t* c, cudaStream_t st) {
    const int n = c->bnd.n;
    if (n <= 0) return SPHDEM_OK;
    launch_pdl(k_gather_vol, blocks_for(n, 256), 256, 0, st, c->grid_bnd.order, n, c->bnd.m, c->bnd.rho, c->work.b_vprev);
    return launch_status("gather_wall_rho");
}

int64_t scan_scratch_words(int64_t ncell) { return (ncell + kScanTile - 1) / kScanTile + 2; }

}  // namespace sd

extern "C" int64_t sphdem_scan_scratch(int64_t ncell) { return sd::scan_scratch_words(ncell); }
