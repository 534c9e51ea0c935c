// mpnn.cu -- learned K-step surrogate: a message-passing network over the
// radius graph of all particles, trained and evaluated by tensor-core
// (tcgen05, BF16 operands, FP32 accumulation in tensor memory) kernels.
//
// Kernels (all persistent, 128 threads = 4 warps = the 128 TMEM lanes):
//   k_rows     node MLP layers: Y = X W^T (+ bias, SiLU), one 128-row tile per
//              MMA group; the weight image is bulk-copied (TMA) into shared
//              memory once per CTA.
//   k_edges    the fused edge pass: edge features -> layer 1 (edges x 128,
//              TMEM lane = edge) -> ReLU -> layer 2 computed transposed
//              (TMEM lane = feature, columns = edges) -> per-feature segmented
//              sums over the receiver-sorted edges: aggregation (forward) or
//              the scatter to senders (backward of the second round).
//   k_edges_bwd  backward of the first round and of the edge MLP: recomputes
//              both layers, forms dF, scatters dh0, and accumulates dW2 and
//              dW1 across all of the CTA's tiles in TMEM.
//   k_wgrad    weight gradients of the node layers, reduction over rows in
//              TMEM, per-CTA partials reduced in a fixed order.
// Every wait on an MMA or a bulk copy is bounded; on timeout the CTA raises
// SPHDEM_FLAG_TIMEOUT, waits once more (bounded), frees its tensor memory and
// returns.
#include <cuda_bf16.h>
#include <stdio.h>

#include <map>
#include <mutex>
#include <utility>

#include "common.cuh"
#include "sphdem_mpnn.h"
#include "umma.cuh"

namespace sd {

int build_grid(sphdem_grid_t* g, const float* pos, sphdem_ctl_t* ctl, cudaStream_t st);
int scan_counts(int* data, int n, int* sums, cudaStream_t st);

namespace {

using umma::tile_off;

constexpr int kH = SPHDEM_MPNN_HIDDEN;
constexpr int kT = 128;  // threads per CTA = rows per tile
constexpr int kRT = 4;   // node layers: threads per row (kRT x kT threads per CTA)
constexpr int kPolls = 1 << 20;
constexpr int kMaxCtas = 512;
constexpr int kBwdStride = 128 * 128 + 128 * 16 + 256;  // per-CTA partials of k_edges_bwd

// BF16 image offsets (halves) inside `packed`.
constexpr int P_E1 = 0, P_E2 = 2048, P_E2T = 18432, P_N1 = 34816, P_N2 = 36864, P_N2T = 53248, P_N3 = 69632,
              P_N3T = 71680;
static_assert(P_N3T + 2048 == SPHDEM_MPNN_PACKED, "packed layout");

enum { EPI_F32 = 0, EPI_SILU = 1 };
// Edge-input column 7 is the constant 1 and the layer-1 image holds the bias
// there, so the first edge MMA adds the bias itself.
constexpr int kBiasCol = 7;
enum { MODE_AGG = 0, MODE_SCATTER = 1 };

// SiLU z * sigmoid(z) with the fast exponential and reciprocal (relative
// error far below the BF16 rounding of the activations it feeds).
__device__ __forceinline__ float sigmoid(float z) { return __frcp_rn(1.0f + __expf(-z)); }
__device__ __forceinline__ float silu(float z) { return z * sigmoid(z); }
__device__ __forceinline__ float silu_grad(float z) {
    const float s = sigmoid(z);
    return s * (1.0f + z * (1.0f - s));
}
__device__ __forceinline__ uint32_t pack2(float a, float b) {
    __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<uint32_t*>(&h);
}
// max(a, 0), max(b, 0) rounded to BF16 and packed (a in the low half), one
// instruction.
__device__ __forceinline__ uint32_t pack2_relu(float a, float b) {
    uint32_t r;
    asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(b), "f"(a));
    return r;
}
__device__ __forceinline__ uint16_t bf16_bits(float a) {
    __nv_bfloat16 h = __float2bfloat16_rn(a);
    return *reinterpret_cast<uint16_t*>(&h);
}
__device__ __forceinline__ float bf(uint16_t u) { return __uint_as_float((uint32_t)u << 16); }
__device__ __forceinline__ void st_bf16(uint8_t* base, uint32_t off, float v) {
    *reinterpret_cast<uint16_t*>(base + off) = bf16_bits(v);
}

__device__ __forceinline__ void raise_flag(int32_t* status, int bits) {
    if (status) atomicOr(status, bits);
}

// CTA prologue: mbarriers ([0] MMA completion, [1] bulk copies) and tensor memory.
__device__ __forceinline__ uint32_t cta_begin(uint64_t* bars, uint32_t* slot, uint32_t ncols) {
    if (threadIdx.x == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        fence_mbar_init();
    }
    if ((threadIdx.x >> 5) == 0) umma::tmem_alloc(slot, ncols);
    umma::fence_before();
    __syncthreads();
    umma::fence_after();
    return *slot;
}

// The same prologue when thread 0 has already initialised the barriers.
__device__ __forceinline__ uint32_t cta_tmem(uint32_t* slot, uint32_t ncols) {
    if ((threadIdx.x >> 5) == 0) umma::tmem_alloc(slot, ncols);
    umma::fence_before();
    __syncthreads();
    umma::fence_after();
    return *slot;
}

// Issue (thread 0) after the operand tiles were written and fenced by all.
__device__ __forceinline__ void operands_ready() {
    fence_proxy_async_smem();
    umma::fence_before();
    __syncthreads();
}

// Wait for the MMA group with `phase`; returns false on a CTA-wide timeout.
__device__ __forceinline__ bool mma_done(uint64_t* bars, uint32_t& phase, bool& mine) {
    mine = mbar_wait(&bars[0], phase, kPolls);
    const bool bad = __syncthreads_or(!mine);
    if (!bad) phase ^= 1u;
    umma::fence_after();
    return !bad;
}

__device__ __forceinline__ void cta_end(uint64_t* bars, uint32_t phase, bool pending, uint32_t tmem, uint32_t ncols,
                                        int32_t* status, bool failed) {
    if (failed) {
        if (threadIdx.x == 0) raise_flag(status, SPHDEM_FLAG_TIMEOUT);
    }
    if (pending) mbar_wait(&bars[0], phase, kPolls);
    umma::fence_before();
    __syncthreads();
    if ((threadIdx.x >> 5) == 0) {
        umma::fence_after();
        umma::tmem_dealloc(tmem, ncols);
    }
}

// ---------------------------------------------------------------------------
// weight images
// ---------------------------------------------------------------------------
struct Img {
    int dst, src, R, K, trans;
};
__constant__ Img kImgs[8] = {
    {P_E1, SPHDEM_MPNN_E1_W, 128, 16, 0},   {P_E2, SPHDEM_MPNN_E2_W, 128, 128, 0},
    {P_E2T, SPHDEM_MPNN_E2_W, 128, 128, 1}, {P_N1, SPHDEM_MPNN_N1_W, 128, 16, 0},
    {P_N2, SPHDEM_MPNN_N2_W, 128, 128, 0},  {P_N2T, SPHDEM_MPNN_N2_W, 128, 128, 1},
    {P_N3, SPHDEM_MPNN_N3_W, 16, 128, 0},   {P_N3T, SPHDEM_MPNN_N3_W, 128, 16, 1},
};

// Image element (r, k) = W[r][k], or W[k][r] for a transposed image; W is
// row-major with (trans ? R : K) columns.
__global__ void k_pack(const float* __restrict__ theta, uint16_t* __restrict__ packed) {
    const Img im = kImgs[blockIdx.y];
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= im.R * im.K) return;
    const int r = idx / im.K, k = idx % im.K;
    float w = im.trans ? theta[im.src + k * im.R + r] : theta[im.src + r * im.K + k];
    if (im.dst == P_E1 && k == kBiasCol) w = theta[SPHDEM_MPNN_E1_B + r];  // layer-1 bias rides in the MMA
    packed[im.dst + tile_off(r, k, im.K) / 2] = bf16_bits(w);
}

// ---------------------------------------------------------------------------
// node MLP layers: out = epi(A[M,K] * B[N,K]^T + bias)
// ---------------------------------------------------------------------------
// add (optional, K = 128): rows r < n_add of the A operand are A[r] + add[r]
// (the residual h + s * sum_j f_ij (.) h_j, formed while staging the tile).
// list (optional): the layer runs on rows 0 .. n_direct - 1 and on the list[0]
// rows list[1 ..] (in any order: rows are independent); M bounds both.
template <int K, int N, int EPI, bool IMG>
__global__ void __launch_bounds__(kRT * kT) k_rows(const uint16_t* __restrict__ A, int M, const float* __restrict__ add,
                                             int n_add, const uint16_t* __restrict__ B,
                                             const float* __restrict__ bias, float* __restrict__ out_f32,
                                             uint16_t* __restrict__ out_bf, float* __restrict__ z_out,
                                             int32_t* status, const int* __restrict__ list, int n_direct,
                                             int early) {
    constexpr uint32_t kB = N * K * 2, kA = kT * K * 2;
    constexpr uint32_t kCols = N < 32 ? 32 : N;
    extern __shared__ __align__(1024) uint8_t sm[];
    uint8_t* sB = sm;
    uint8_t* sA = sm + kB;
    float* sbias = reinterpret_cast<float*>(sA + kA);
    uint64_t* bars = reinterpret_cast<uint64_t*>(sbias + (N < 2 ? 2 : N));
    uint32_t* slot = reinterpret_cast<uint32_t*>(bars + 2);
    // kRT threads per row: threads rt + i kT stage a share of row rt's
    // 16-byte chunks, and warps w, w + 4, ... (same TMEM lanes) split the
    // output columns
    const int tid = threadIdx.x, warp = tid >> 5, rt = tid & (kT - 1), hh = tid / kT;

    // early (inference): the weight image is fixed, so its copy starts before
    // the previous kernel is done (no kernel of the inference chain writes it)
    const bool pre = IMG && early;
    if (pre && tid == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        fence_mbar_init();
        mbar_arrive_expect_tx(&bars[1], kB);
        tma_load_1d(sB, B, kB, &bars[1]);
    }
    pdl_wait();
    pdl_launch();
    const uint32_t tmem = pre ? cta_tmem(slot, kCols) : cta_begin(bars, slot, kCols);
    for (int i = tid; i < N; i += kRT * kT) sbias[i] = bias ? bias[i] : 0.0f;
    bool mine = true, failed = false, pending = false;
    uint32_t phase = 0;
    if (IMG) {
        if (tid == 0 && !pre) {
            mbar_arrive_expect_tx(&bars[1], kB);
            tma_load_1d(sB, B, kB, &bars[1]);
        }
        failed = __syncthreads_or(!mbar_wait(&bars[1], 0, kPolls));
    } else {
        for (int idx = tid; idx < N * (K / 8); idx += kRT * kT) {
            const int r = idx / (K / 8), q = idx % (K / 8);
            *reinterpret_cast<uint4*>(sB + tile_off(r, 8 * q, K)) =
                __ldg(reinterpret_cast<const uint4*>(B + (size_t)r * K) + q);
        }
    }
    __syncthreads();
    constexpr uint32_t idesc = umma::idesc_bf16(128, N);
    const int Mv = list ? min(M, n_direct + __ldg(list)) : M;  // rows of this launch
    for (int tile = blockIdx.x; !failed && tile * kT < Mv; tile += gridDim.x) {
        int row = tile * kT + rt;
        if (list && row >= n_direct) row = row < Mv ? __ldg(list + 1 + (row - n_direct)) : M;  // M: no row
        const bool plus = add != nullptr && row < n_add;
        constexpr int CPT = K / 8 < kRT ? 1 : K / 8 / kRT;  // chunks per thread
#pragma unroll
        for (int q = hh * CPT; q < hh * CPT + CPT && q < K / 8; ++q) {
            uint4 v = make_uint4(0, 0, 0, 0);
            if (row < M) v = __ldg(reinterpret_cast<const uint4*>(A + (size_t)row * K) + q);
            if (plus) {
                const float4 a0 = __ldg(reinterpret_cast<const float4*>(add + (size_t)row * K + 8 * q));
                const float4 a1 = __ldg(reinterpret_cast<const float4*>(add + (size_t)row * K + 8 * q + 4));
                v = make_uint4(pack2(bf((uint16_t)v.x) + a0.x, bf((uint16_t)(v.x >> 16)) + a0.y),
                               pack2(bf((uint16_t)v.y) + a0.z, bf((uint16_t)(v.y >> 16)) + a0.w),
                               pack2(bf((uint16_t)v.z) + a1.x, bf((uint16_t)(v.z >> 16)) + a1.y),
                               pack2(bf((uint16_t)v.w) + a1.z, bf((uint16_t)(v.w >> 16)) + a1.w));
            }
            *reinterpret_cast<uint4*>(sA + tile_off(rt, 8 * q, K)) = v;
        }
        operands_ready();
        if (tid == 0) {
            umma::fence_after();
            umma::mma_tile(tmem, sA, sB, K, idesc, false);
            umma::commit(&bars[0]);
        }
        pending = true;
        if (!mma_done(bars, phase, mine)) {
            failed = true;
            break;
        }
        pending = false;
        // columns of this thread: [hh NH, hh NH + NH), or all 16 (thread rt) when N = 16
        constexpr int W = N < 32 ? 16 : 32, NH = N < 32 ? N : N / kRT;
        static_assert(N < 32 || NH % 32 == 0, "k_rows column split");
#pragma unroll
        for (int c0 = hh * NH; c0 < hh * NH + NH && c0 < N; c0 += W) {
            float v[32];
            if (N < 32)
                umma::tmem_ld16(umma::taddr(tmem, 32 * (warp & 3), c0), v);
            else
                umma::tmem_ld32(umma::taddr(tmem, 32 * (warp & 3), c0), v);
            if (row < M) {
                if (EPI == EPI_F32) {
                    float4* o = reinterpret_cast<float4*>(out_f32 + (size_t)row * N + c0);
#pragma unroll
                    for (int i = 0; i < W / 4; ++i)
                        o[i] = make_float4(v[4 * i] + sbias[c0 + 4 * i], v[4 * i + 1] + sbias[c0 + 4 * i + 1],
                                           v[4 * i + 2] + sbias[c0 + 4 * i + 2], v[4 * i + 3] + sbias[c0 + 4 * i + 3]);
                } else {
#pragma unroll
                    for (int i = 0; i < W; ++i) v[i] += sbias[c0 + i];
                    if (z_out) {
                        float4* o = reinterpret_cast<float4*>(z_out + (size_t)row * N + c0);
#pragma unroll
                        for (int i = 0; i < W / 4; ++i) o[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
                    }
                    uint4* o = reinterpret_cast<uint4*>(out_bf + (size_t)row * N + c0);
#pragma unroll
                    for (int i = 0; i < W / 8; ++i)
                        o[i] = make_uint4(pack2(silu(v[8 * i]), silu(v[8 * i + 1])),
                                          pack2(silu(v[8 * i + 2]), silu(v[8 * i + 3])),
                                          pack2(silu(v[8 * i + 4]), silu(v[8 * i + 5])),
                                          pack2(silu(v[8 * i + 6]), silu(v[8 * i + 7])));
                }
            }
        }
        umma::fence_before();
        __syncthreads();
    }
    cta_end(bars, phase, pending && !mine, tmem, kCols, status, failed);
}

// ---------------------------------------------------------------------------
// fused edge pass
// ---------------------------------------------------------------------------
struct EdgeArgs {
    const float4* pos;
    const float4* vel;
    const int* offset;
    const int* sender;
    const int* receiver;
    int n_recv, cap;
    float inv_r, inv_vs, inv_norm;
    const uint16_t* img_e1;
    const uint16_t* img_e2;
    const uint16_t* img_e2t;
    const float* b1;
    const float* b2;
    // forward: agg[r] += s * sum f (.) h[j]
    const uint16_t* h;
    float* agg;
    // backward (second round): dh[j] += s * f (.) g[r]
    const float* g;
    float* dh;
    // backward (first round + edge MLP)
    const float* g1;       // [n_recv,128]
    const float* g2;       // [n_recv,128]
    const uint16_t* h0;    // [n,128]
    const uint16_t* h2;    // [n,128]
    float* dh0;            // [n,128]
    float* partial;        // [grid][kBwdStride]
    int32_t* status;
    int early;             // inference: the weight images are copied before the previous kernel is done
};

// Edge features of edge e (zeros past the end): ((x_j-x_i)/R, |x_j-x_i|/R,
// (v_j-v_i)/v_s, 0...), as 16 BF16 values in two 16-byte words.
__device__ __forceinline__ void edge_features(const EdgeArgs& a, int e, int E, int& r, int& j, uint4& q0) {
    r = -1;
    j = -1;
    q0 = make_uint4(0, 0, 0, 0);
    if (e >= E) return;
    r = __ldg(a.receiver + e);
    j = __ldg(a.sender + e);
    const float4 pr = __ldg(a.pos + r), pj = __ldg(a.pos + j);
    const float4 vr = __ldg(a.vel + r), vj = __ldg(a.vel + j);
    const float dx = pj.x - pr.x, dy = pj.y - pr.y, dz = pj.z - pr.z;
    const float dist = sqrtf(dx * dx + dy * dy + dz * dz);
    q0.x = pack2(dx * a.inv_r, dy * a.inv_r);
    q0.y = pack2(dz * a.inv_r, dist * a.inv_r);
    q0.z = pack2((vj.x - vr.x) * a.inv_vs, (vj.y - vr.y) * a.inv_vs);
    q0.w = pack2((vj.z - vr.z) * a.inv_vs, 1.0f);
}

constexpr uint32_t kImg16 = 128 * 16 * 2;   // 4 KB
constexpr uint32_t kImg128 = 128 * 128 * 2;  // 32 KB
// k_edges shared memory: the weight images once, then per pipeline an edge
// feature tile, the hidden-activation tile, receiver/sender ids and an mbarrier.
// The forward pass also stages the senders' latent rows (128 x 256 B) by
// bulk copies issued when the tile is loaded, so they land during the MMAs.
constexpr uint32_t EF_IMG1 = 0, EF_IMG2 = EF_IMG1 + kImg16, EF_B1 = EF_IMG2 + kImg128, EF_B2 = EF_B1 + 512,
                   EF_BARS = EF_B2 + 512, EF_SLOT = EF_BARS + 48, EF_PIPE = (EF_SLOT + 16 + 1023) / 1024 * 1024,
                   EF_P_XS = 0, EF_P_ZR = EF_P_XS + kImg16, EF_P_SR = EF_P_ZR + kImg128, EF_P_SJ = EF_P_SR + 512,
                   EF_P_END = EF_P_SJ + 512, EF_P_H = EF_P_END + 16, EF_P_BYTES = EF_P_H + kImg128,
                   EF_BYTES = EF_PIPE + 2 * EF_P_BYTES;
static_assert(EF_PIPE % 1024 == 0 && EF_P_BYTES % 16 == 0 && EF_P_H % 16 == 0, "k_edges shared memory alignment");
static_assert(EF_BYTES <= 227 * 1024, "k_edges shared memory");

struct EdgeLoad {
    int r, j;
    float4 pr, pj, vr, vj;
};

// Edge ids of edge e (-1 past the end); positions and velocities follow in
// edge_load_state, so the two dependent loads can be issued at different points.
__device__ __forceinline__ void edge_load_ids(const EdgeArgs& a, int e, int E, EdgeLoad& L) {
    L.r = -1;
    L.j = -1;
    if (e < E) {
        L.r = __ldg(a.receiver + e);
        L.j = __ldg(a.sender + e);
    }
}

__device__ __forceinline__ void edge_load_state(const EdgeArgs& a, EdgeLoad& L) {
    if (L.r >= 0) {
        L.pr = __ldg(a.pos + L.r);
        L.pj = __ldg(a.pos + L.j);
        L.vr = __ldg(a.vel + L.r);
        L.vj = __ldg(a.vel + L.j);
    }
}

__device__ __forceinline__ uint4 edge_pack(const EdgeArgs& a, const EdgeLoad& L) {
    if (L.r < 0) return make_uint4(0, 0, 0, 0);
    const float dx = L.pj.x - L.pr.x, dy = L.pj.y - L.pr.y, dz = L.pj.z - L.pr.z;
    const float dist = sqrtf(dx * dx + dy * dy + dz * dz);
    return make_uint4(pack2(dx * a.inv_r, dy * a.inv_r), pack2(dz * a.inv_r, dist * a.inv_r),
                      pack2((L.vj.x - L.vr.x) * a.inv_vs, (L.vj.y - L.vr.y) * a.inv_vs),
                      pack2((L.vj.z - L.vr.z) * a.inv_vs, 1.0f));
}

// Two independent pipelines of 8 warps per CTA (warps 0-7, 8-15), each owning
// TMEM columns [128 p, 128 p + 128): layer 1 lands there (lane = edge), is
// consumed by its epilogue, and layer 2 (lane = feature) overwrites it.  In
// both epilogues warps w and w + 4 of a pipeline read the same 32 TMEM lanes
// and split the 128 columns.  The next tile's edge data are loaded while the
// current tile's epilogue runs; the senders' latent rows are bulk-copied into
// shared memory as soon as a tile's edges are known.
constexpr int kPT = 256;  // threads per pipeline

// Barrier of one 256-thread pipeline (named barrier 1 or 2, immediate ids).
__device__ __forceinline__ void pipe_sync256(int id) {
    if (id == 1)
        asm volatile("bar.sync 1, 256;" ::: "memory");
    else
        asm volatile("bar.sync 2, 256;" ::: "memory");
}
__device__ __forceinline__ bool pipe_or256(bool v, int id) {
    uint32_t r;
    if (id == 1)
        asm volatile(
            "{\n\t.reg .pred p, q;\n\t"
            "setp.ne.u32 p, %1, 0;\n\t"
            "bar.red.or.pred q, 1, 256, p;\n\t"
            "selp.u32 %0, 1, 0, q;\n\t}"
            : "=r"(r)
            : "r"((uint32_t)v)
            : "memory");
    else
        asm volatile(
            "{\n\t.reg .pred p, q;\n\t"
            "setp.ne.u32 p, %1, 0;\n\t"
            "bar.red.or.pred q, 2, 256, p;\n\t"
            "selp.u32 %0, 1, 0, q;\n\t}"
            : "=r"(r)
            : "r"((uint32_t)v)
            : "memory");
    return r != 0;
}

template <int MODE>
__global__ void __launch_bounds__(2 * kPT, 1) k_edges(EdgeArgs a) {
    extern __shared__ __align__(1024) uint8_t sm[];
    uint8_t* img1 = sm + EF_IMG1;
    uint8_t* img2 = sm + EF_IMG2;
    float* b2 = reinterpret_cast<float*>(sm + EF_B2);
    uint64_t* bars = reinterpret_cast<uint64_t*>(sm + EF_BARS);  // [0],[1] MMAs, [2] weights, [3],[4] sender rows
    uint32_t* slot = reinterpret_cast<uint32_t*>(sm + EF_SLOT);
    const int tid = threadIdx.x, warp = tid >> 5, p = warp >> 3, plt = tid & (kPT - 1);
    const int wq = warp & 7, lanes = 32 * (wq & 3), half = wq >> 2;
    const int lt = plt & (kT - 1);  // TMEM lane of this thread
    const bool loader = plt < kT;
    uint8_t* pb = sm + EF_PIPE + p * EF_P_BYTES;
    uint8_t* xs = pb + EF_P_XS;
    uint8_t* zr = pb + EF_P_ZR;
    int* sr = reinterpret_cast<int*>(pb + EF_P_SR);
    int* sj = reinterpret_cast<int*>(pb + EF_P_SJ);
    uint8_t* hs = pb + EF_P_H;  // [128 edges][128] BF16 sender rows
    uint64_t* bar = &bars[p];
    uint64_t* hbar = &bars[3 + p];
    const int bid = 1 + p;
    if (tid == 0) {
        for (int b = 0; b < 5; ++b) mbar_init(&bars[b], 1);
        fence_mbar_init();
        if (a.early) {  // the weight images are fixed: copy them while the previous kernel drains
            mbar_arrive_expect_tx(&bars[2], kImg16 + kImg128);
            tma_load_1d(img1, a.img_e1, kImg16, &bars[2]);
            tma_load_1d(img2, a.img_e2, kImg128, &bars[2]);
        }
    }
    pdl_wait();
    pdl_launch();
    const int E = min(__ldg(a.offset + a.n_recv), a.cap);
    if (warp == 0) umma::tmem_alloc(slot, 256);
    if (tid < 128) b2[tid] = a.b2[tid];
    umma::fence_before();
    __syncthreads();
    umma::fence_after();
    const uint32_t tmem = *slot + 128u * p;
    if (tid == 0 && !a.early) {
        mbar_arrive_expect_tx(&bars[2], kImg16 + kImg128);
        tma_load_1d(img1, a.img_e1, kImg16, &bars[2]);
        tma_load_1d(img2, a.img_e2, kImg128, &bars[2]);
    }
    bool failed = __syncthreads_or(!mbar_wait(&bars[2], 0, kPolls));
    bool mine = true, hmine = true, pending = false, hpending = false;
    uint32_t phase = 0, hphase = 0;
    constexpr uint32_t idesc = umma::idesc_bf16(128, 128);
    const int stride = 2 * gridDim.x;
    int tile = 2 * blockIdx.x + p;
    EdgeLoad nxt;
    nxt.r = nxt.j = -1;
    if (loader) {
        edge_load_ids(a, tile * kT + lt, E, nxt);
        edge_load_state(a, nxt);
    }
    for (; !failed && tile * kT < E; tile += stride) {
        if (loader) {
            const EdgeLoad cur_e = nxt;
            sr[lt] = cur_e.r;
            sj[lt] = cur_e.j;
            *reinterpret_cast<uint4*>(xs + tile_off(lt, 0, 16)) = edge_pack(a, cur_e);
            *reinterpret_cast<uint4*>(xs + tile_off(lt, 8, 16)) = make_uint4(0, 0, 0, 0);
            if (MODE == MODE_AGG && lt == 0) {
                const int valid = min(kT, E - tile * kT);
                mbar_arrive_expect_tx(hbar, (uint32_t)valid * 256u);
            }
        }
        fence_proxy_async_smem();
        umma::fence_before();
        pipe_sync256(bid);
        if (plt == 0) {
            umma::fence_after();
            umma::mma_tile(tmem, xs, img1, 16, idesc, false);  // D[e][k], layer-1 bias included
            umma::commit(bar);
        }
        if (loader) {
            if (MODE == MODE_AGG) {
                if (sj[lt] >= 0) tma_load_1d(hs + lt * 256, a.h + (size_t)sj[lt] * kH, 256, hbar);
                // edges after which the running sum is flushed: the last edge of a
                // receiver's run, and the last valid edge of each half-tile
                const int r = sr[lt];
                const bool flush = r >= 0 && (lt == kT - 1 || lt == kT / 2 - 1 || sr[lt + 1] != r);
                const unsigned m = __ballot_sync(0xffffffffu, flush);
                if ((lt & 31) == 0) reinterpret_cast<uint32_t*>(pb + EF_P_END)[lt >> 5] = m;
            }
            edge_load_ids(a, (tile + stride) * kT + lt, E, nxt);  // prefetch the next tile's ids
        }
        if (MODE == MODE_AGG) hpending = true;
        pending = true;
        // A wait that gives up is reported at the pipeline's next barrier,
        // which then reduces the outcome (what is read meanwhile is discarded).
        mine = mbar_wait(bar, phase, kPolls);
        if (mine) {
            phase ^= 1u;
            pending = false;
        }
        umma::fence_after();
        // layer-1 epilogue: lane = edge, this half's 64 hidden units
#pragma unroll
        for (int c0 = 64 * half; c0 < 64 * half + 64; c0 += 32) {
            float v[32];
            umma::tmem_ld32(umma::taddr(tmem, lanes, c0), v);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int k = c0 + 8 * q;
                uint4 w;
                w.x = pack2_relu(v[8 * q], v[8 * q + 1]);
                w.y = pack2_relu(v[8 * q + 2], v[8 * q + 3]);
                w.z = pack2_relu(v[8 * q + 4], v[8 * q + 5]);
                w.w = pack2_relu(v[8 * q + 6], v[8 * q + 7]);
                *reinterpret_cast<uint4*>(zr + tile_off(lt, k, 128)) = w;
            }
        }
        fence_proxy_async_smem();
        umma::fence_before();
        if (pipe_or256(!mine, bid)) { failed = true; break; }
        if (plt == 0) {
            umma::fence_after();
            umma::mma_tile(tmem, img2, zr, 128, idesc, false);  // D[c][e], over layer 1's columns
            umma::commit(bar);
        }
        if (loader) edge_load_state(a, nxt);  // the next tile's particle state
        pending = true;
        mine = mbar_wait(bar, phase, kPolls);
        if (mine) {
            phase ^= 1u;
            pending = false;
        }
        umma::fence_after();
        // layer-2 epilogue: lane = feature c, this half's 64 edges of the tile
        const int c = lt;
        const float bc = b2[c];
        int cur = -1;
        float gval = 0.0f;
        if (MODE == MODE_AGG) {
            hmine = mbar_wait(hbar, hphase, kPolls);
            if (hmine) {
                hphase ^= 1u;
                hpending = false;
            }
            const uint16_t* h16 = reinterpret_cast<const uint16_t*>(hs) + c;
            const uint32_t* ends = reinterpret_cast<const uint32_t*>(pb + EF_P_END);
            // Segmented sums over the receiver-sorted edges; a group of 8
            // edges that ends no run (most of them: ~30 edges per receiver)
            // runs without the per-edge flush tests.
            float acc = 0.0f;
#pragma unroll 1
            for (int c0 = 64 * half; c0 < 64 * half + 64; c0 += 32) {
                float v[32];
                umma::tmem_ld32(umma::taddr(tmem, lanes, c0), v);
                const uint32_t em = ends[c0 >> 5];  // warp-uniform: the same edges end a run for every feature
#pragma unroll
                for (int g = 0; g < 32; g += 8) {
                    if (((em >> g) & 0xffu) == 0u) {
#pragma unroll
                        for (int i = g; i < g + 8; ++i) acc = fmaf(v[i] + bc, bf(h16[(c0 + i) * kH]), acc);
                    } else {
#pragma unroll
                        for (int i = g; i < g + 8; ++i) {
                            const float t = fmaf(v[i] + bc, bf(h16[(c0 + i) * kH]), acc);
                            if (em & (1u << i)) {
                                atomicAdd(a.agg + (size_t)sr[c0 + i] * kH + c, t * a.inv_norm);
                                acc = 0.0f;
                            } else {
                                acc = t;
                            }
                        }
                    }
                }
            }
        } else {
#pragma unroll 1
            for (int c0 = 64 * half; c0 < 64 * half + 64; c0 += 32) {
                float v[32];
                umma::tmem_ld32(umma::taddr(tmem, lanes, c0), v);
#pragma unroll 4
                for (int i = 0; i < 32; ++i) {
                    const int rr = sr[c0 + i];
                    if (rr < 0) continue;
                    if (rr != cur) {
                        cur = rr;
                        gval = __ldg(a.g + (size_t)rr * kH + c) * a.inv_norm;
                    }
                    atomicAdd(a.dh + (size_t)sj[c0 + i] * kH + c, (v[i] + bc) * gval);
                }
            }
        }
        umma::fence_before();
        if (pipe_or256(!mine || !hmine, bid)) { failed = true; break; }
    }
    if (failed && plt == 0) raise_flag(a.status, SPHDEM_FLAG_TIMEOUT);
    if (pending && !mine) mbar_wait(bar, phase, kPolls);
    if (MODE == MODE_AGG && hpending) mbar_wait(hbar, hphase, kPolls);  // copies still landing
    umma::fence_before();
    __syncthreads();
    if (warp == 0) {
        umma::fence_after();
        umma::tmem_dealloc(*slot, 256);
    }
}

// k_edges_bwd shared memory
constexpr uint32_t EB_IMG1 = 0, EB_IMG2 = EB_IMG1 + kImg16, EB_IMG2T = EB_IMG2 + kImg128, EB_XS = EB_IMG2T + kImg128,
                   EB_XT = EB_XS + kImg16, EB_ZR = EB_XT + kImg16, EB_ZT = EB_ZR + kImg128, EB_DFT = EB_ZT + kImg128,
                   EB_DF = EB_DFT + kImg128, EB_B1 = EB_DF + kImg128, EB_B2 = EB_B1 + 512, EB_SR = EB_B2 + 512,
                   EB_SJ = EB_SR + 512, EB_BARS = EB_SJ + 512, EB_SLOT = EB_BARS + 16, EB_BYTES = EB_SLOT + 16;
static_assert(EB_BYTES <= 227 * 1024, "k_edges_bwd shared memory");

// TMEM columns: [0,128) layer 1 then dZ; [128,256) layer 2; [256,384) dW2; [384,400) dW1.
__global__ void __launch_bounds__(kT, 1) k_edges_bwd(EdgeArgs a) {
    extern __shared__ __align__(1024) uint8_t sm[];
    uint8_t* img1 = sm + EB_IMG1;
    uint8_t* img2 = sm + EB_IMG2;
    uint8_t* img2t = sm + EB_IMG2T;
    uint8_t* xs = sm + EB_XS;
    uint8_t* xt = sm + EB_XT;
    uint8_t* zr = sm + EB_ZR;  // Z rows (layer-2 B operand), then dP^T (dW1 A operand)
    uint8_t* zt = sm + EB_ZT;
    uint8_t* dft = sm + EB_DFT;
    uint8_t* dfr = sm + EB_DF;
    float* b1 = reinterpret_cast<float*>(sm + EB_B1);
    float* b2 = reinterpret_cast<float*>(sm + EB_B2);
    int* sr = reinterpret_cast<int*>(sm + EB_SR);
    int* sj = reinterpret_cast<int*>(sm + EB_SJ);
    uint64_t* bars = reinterpret_cast<uint64_t*>(sm + EB_BARS);
    uint32_t* slot = reinterpret_cast<uint32_t*>(sm + EB_SLOT);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int E = min(__ldg(a.offset + a.n_recv), a.cap);

    const uint32_t tmem = cta_begin(bars, slot, 512);
    b1[tid] = a.b1[tid];
    b2[tid] = a.b2[tid];
    if (tid == 0) {
        mbar_arrive_expect_tx(&bars[1], kImg16 + 2 * kImg128);
        tma_load_1d(img1, a.img_e1, kImg16, &bars[1]);
        tma_load_1d(img2, a.img_e2, kImg128, &bars[1]);
        tma_load_1d(img2t, a.img_e2t, kImg128, &bars[1]);
    }
    bool failed = __syncthreads_or(!mbar_wait(&bars[1], 0, kPolls));
    bool mine = true, pending = false, first = true;
    uint32_t phase = 0;
    constexpr uint32_t id128 = umma::idesc_bf16(128, 128), id16 = umma::idesc_bf16(128, 16);
    float db1 = 0.0f, db2 = 0.0f;
    const int c = tid;
    for (int tile = blockIdx.x; !failed && tile * kT < E; tile += gridDim.x) {
        if (pending) {  // dW1 of the previous tile still reads xt and the dP^T tile
            if (!mma_done(bars, phase, mine)) { failed = true; break; }
            pending = false;
        }
        int r, j;
        uint4 q0;
        edge_features(a, tile * kT + tid, E, r, j, q0);
        sr[tid] = r;
        sj[tid] = j;
        *reinterpret_cast<uint4*>(xs + tile_off(tid, 0, 16)) = q0;
        *reinterpret_cast<uint4*>(xs + tile_off(tid, 8, 16)) = make_uint4(0, 0, 0, 0);
        {
            const uint32_t w[4] = {q0.x, q0.y, q0.z, q0.w};
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                const uint16_t hv = i < kBiasCol ? (uint16_t)(w[i >> 1] >> (16 * (i & 1))) : (uint16_t)0;
                *reinterpret_cast<uint16_t*>(xt + tile_off(i, tid, 128)) = hv;
            }
        }
        operands_ready();
        if (tid == 0) {
            umma::fence_after();
            umma::mma_tile(tmem, xs, img1, 16, id128, false);
            umma::commit(&bars[0]);
        }
        pending = true;
        if (!mma_done(bars, phase, mine)) { failed = true; break; }
        pending = false;
        // layer-1 epilogue (row = edge): Z rows and Z^T
#pragma unroll 1
        for (int c0 = 0; c0 < 128; c0 += 32) {
            float v[32];
            umma::tmem_ld32(umma::taddr(tmem, 32 * warp, c0), v);
#pragma unroll
            for (int i = 0; i < 32; ++i) v[i] = fmaxf(v[i], 0.0f);
#pragma unroll
            for (int q = 0; q < 4; ++q)
                *reinterpret_cast<uint4*>(zr + tile_off(tid, c0 + 8 * q, 128)) =
                    make_uint4(pack2(v[8 * q], v[8 * q + 1]), pack2(v[8 * q + 2], v[8 * q + 3]),
                               pack2(v[8 * q + 4], v[8 * q + 5]), pack2(v[8 * q + 6], v[8 * q + 7]));
#pragma unroll
            for (int i = 0; i < 32; ++i) st_bf16(zt, tile_off(c0 + i, tid, 128), v[i]);
        }
        operands_ready();
        if (tid == 0) {
            umma::fence_after();
            umma::mma_tile(tmem + 128, img2, zr, 128, id128, false);
            umma::commit(&bars[0]);
        }
        pending = true;
        if (!mma_done(bars, phase, mine)) { failed = true; break; }
        pending = false;
        // layer-2 epilogue (lane = feature c): dF, scatter of dh0, db2
        {
            const float bc = b2[c];
            int cur = -1;
            float g1v = 0.0f, g2v = 0.0f;
#pragma unroll 1
            for (int c0 = 0; c0 < 128; c0 += 32) {
                float v[32], df[32];
                umma::tmem_ld32(umma::taddr(tmem + 128, 32 * warp, c0), v);
#pragma unroll 4
                for (int i = 0; i < 32; ++i) {
                    const int rr = sr[c0 + i], jj = sj[c0 + i];
                    df[i] = 0.0f;
                    if (rr < 0) continue;
                    if (rr != cur) {
                        cur = rr;
                        g1v = __ldg(a.g1 + (size_t)rr * kH + c) * a.inv_norm;
                        g2v = __ldg(a.g2 + (size_t)rr * kH + c) * a.inv_norm;
                    }
                    const float h0v = bf(__ldg(a.h0 + (size_t)jj * kH + c));
                    const float h2v = bf(__ldg(a.h2 + (size_t)jj * kH + c));
                    df[i] = g1v * h0v + g2v * h2v;
                    atomicAdd(a.dh0 + (size_t)jj * kH + c, (v[i] + bc) * g1v);
                }
#pragma unroll
                for (int i = 0; i < 32; ++i) db2 += df[i];
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    *reinterpret_cast<uint4*>(dft + tile_off(c, c0 + 8 * q, 128)) =
                        make_uint4(pack2(df[8 * q], df[8 * q + 1]), pack2(df[8 * q + 2], df[8 * q + 3]),
                                   pack2(df[8 * q + 4], df[8 * q + 5]), pack2(df[8 * q + 6], df[8 * q + 7]));
#pragma unroll
                for (int i = 0; i < 32; ++i) st_bf16(dfr, tile_off(c0 + i, c, 128), df[i]);
            }
        }
        operands_ready();
        if (tid == 0) {
            umma::fence_after();
            umma::mma_tile(tmem + 256, dft, zt, 128, id128, !first);  // dW2[c][k] += dF^T Z
            umma::mma_tile(tmem, img2t, dfr, 128, id128, false);      // dZ[k][e] = W2^T dF^T
            umma::commit(&bars[0]);
        }
        pending = true;
        if (!mma_done(bars, phase, mine)) { failed = true; break; }
        pending = false;
        // dZ epilogue (lane = hidden unit k): dP = dZ * relu'(P), db1, dP^T tile
        {
            const int k = tid;
#pragma unroll 1
            for (int c0 = 0; c0 < 128; c0 += 32) {
                float v[32];
                umma::tmem_ld32(umma::taddr(tmem, 32 * warp, c0), v);
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const uint4 zq = *reinterpret_cast<const uint4*>(zt + tile_off(k, c0 + 8 * q, 128));
                    const uint32_t zw[4] = {zq.x, zq.y, zq.z, zq.w};
#pragma unroll
                    for (int i = 0; i < 8; ++i) {
                        const uint16_t zb = (uint16_t)(zw[i >> 1] >> (16 * (i & 1)));
                        if (!(bf(zb) > 0.0f)) v[8 * q + i] = 0.0f;
                    }
                }
#pragma unroll
                for (int i = 0; i < 32; ++i) db1 += v[i];
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    *reinterpret_cast<uint4*>(zr + tile_off(k, c0 + 8 * q, 128)) =
                        make_uint4(pack2(v[8 * q], v[8 * q + 1]), pack2(v[8 * q + 2], v[8 * q + 3]),
                                   pack2(v[8 * q + 4], v[8 * q + 5]), pack2(v[8 * q + 6], v[8 * q + 7]));
            }
        }
        operands_ready();
        if (tid == 0) {
            umma::fence_after();
            umma::mma_tile(tmem + 384, zr, xt, 128, id16, !first);  // dW1[k][in] += dP^T X
            umma::commit(&bars[0]);
        }
        pending = true;
        first = false;
    }
    if (!failed && pending) {
        failed = !mma_done(bars, phase, mine);
        if (!failed) pending = false;
    }
    float* part = a.partial + (size_t)blockIdx.x * kBwdStride;
    if (!failed) {
#pragma unroll 1
        for (int c0 = 0; c0 < 128; c0 += 32) {
            float v[32];
            umma::tmem_ld32(umma::taddr(tmem + 256, 32 * warp, c0), v);
#pragma unroll
            for (int i = 0; i < 32; ++i) part[tid * 128 + c0 + i] = first ? 0.0f : v[i];
        }
        {
            float v[16];
            umma::tmem_ld16(umma::taddr(tmem + 384, 32 * warp, 0), v);
#pragma unroll
            for (int i = 0; i < 16; ++i) part[128 * 128 + tid * 16 + i] = first ? 0.0f : v[i];
        }
        part[128 * 128 + 128 * 16 + tid] = db1;
        part[128 * 128 + 128 * 16 + 128 + tid] = db2;
    }
    cta_end(bars, phase, pending && !mine, tmem, 512, a.status, failed);
}

// ---------------------------------------------------------------------------
// weight gradients of the node layers: C[128][N] = sum_r P[r][:]^T Q[r][:]
// ---------------------------------------------------------------------------
template <int N>
__global__ void __launch_bounds__(kT) k_wgrad(const uint16_t* __restrict__ P, const uint16_t* __restrict__ Q, int rows,
                                              float* __restrict__ partial, int32_t* status) {
    constexpr uint32_t kA = 128 * 128 * 2, kB = N * 128 * 2;
    constexpr uint32_t kCols = N < 32 ? 32 : N;
    extern __shared__ __align__(1024) uint8_t sm[];
    uint8_t* sA = sm;
    uint8_t* sB = sm + kA;
    uint64_t* bars = reinterpret_cast<uint64_t*>(sB + kB);
    uint32_t* slot = reinterpret_cast<uint32_t*>(bars + 2);
    const int tid = threadIdx.x, warp = tid >> 5;
    const uint32_t tmem = cta_begin(bars, slot, kCols);
    bool mine = true, failed = false, pending = false, first = true;
    uint32_t phase = 0;
    constexpr uint32_t idesc = umma::idesc_bf16(128, N);
    for (int chunk = blockIdx.x; chunk * kT < rows; chunk += gridDim.x) {
        const int row = chunk * kT + tid;
#pragma unroll 1
        for (int q = 0; q < 16; ++q) {
            uint4 v = make_uint4(0, 0, 0, 0);
            if (row < rows) v = __ldg(reinterpret_cast<const uint4*>(P + (size_t)row * 128) + q);
            const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
            for (int i = 0; i < 8; ++i)
                *reinterpret_cast<uint16_t*>(sA + tile_off(8 * q + i, tid, 128)) =
                    (uint16_t)(w[i >> 1] >> (16 * (i & 1)));
        }
#pragma unroll 1
        for (int q = 0; q < N / 8; ++q) {
            uint4 v = make_uint4(0, 0, 0, 0);
            if (row < rows) v = __ldg(reinterpret_cast<const uint4*>(Q + (size_t)row * N) + q);
            const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
            for (int i = 0; i < 8; ++i)
                *reinterpret_cast<uint16_t*>(sB + tile_off(8 * q + i, tid, 128)) =
                    (uint16_t)(w[i >> 1] >> (16 * (i & 1)));
        }
        operands_ready();
        if (tid == 0) {
            umma::fence_after();
            umma::mma_tile(tmem, sA, sB, 128, idesc, !first);
            umma::commit(&bars[0]);
        }
        pending = true;
        if (!mma_done(bars, phase, mine)) { failed = true; break; }
        pending = false;
        first = false;
    }
    if (!failed) {
        float* part = partial + (size_t)blockIdx.x * 128 * N;
#pragma unroll
        for (int c0 = 0; c0 < N; c0 += (N < 32 ? 16 : 32)) {
            float v[32];
            if (N < 32)
                umma::tmem_ld16(umma::taddr(tmem, 32 * warp, c0), v);
            else
                umma::tmem_ld32(umma::taddr(tmem, 32 * warp, c0), v);
#pragma unroll
            for (int i = 0; i < (N < 32 ? 16 : 32); ++i) part[tid * N + c0 + i] = first ? 0.0f : v[i];
        }
    }
    cta_end(bars, phase, pending && !mine, tmem, kCols, status, failed);
}

// dst[i] (or dst transposed) = sum over ctas of partial[cta * stride + off + i], fixed order.
__global__ void k_reduce(const float* __restrict__ partial, int ncta, int stride, int off, int count, int rows_t,
                         int cols_t, float* __restrict__ dst) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    float s = 0.0f;
    for (int b = 0; b < ncta; ++b) s += partial[(size_t)b * stride + off + i];
    if (rows_t > 0) {  // source [rows_t][cols_t] -> destination [cols_t][rows_t]
        const int a = i / cols_t, b = i % cols_t;
        dst[b * rows_t + a] = s;
    } else {
        dst[i] = s;
    }
}

// Column sums of a row-major [rows][cols] FP32 matrix, deterministic.
__global__ void k_colsum_part(const float* __restrict__ m, int rows, int cols, int chunk, float* __restrict__ part) {
    const int c = threadIdx.x;
    if (c >= cols) return;
    const int r0 = blockIdx.x * chunk, r1 = min(rows, r0 + chunk);
    float s = 0.0f;
    for (int r = r0; r < r1; ++r) s += m[(size_t)r * cols + c];
    part[blockIdx.x * cols + c] = s;
}

// ---------------------------------------------------------------------------
// elementwise pieces
// ---------------------------------------------------------------------------
// out[r] = h[r] + agg[r] for r < n_recv, h[r] otherwise (BF16 rows of 128).
__global__ void k_residual(const uint16_t* __restrict__ h, const float* __restrict__ agg, int n_recv, int rows,
                           uint16_t* __restrict__ out) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;  // pair index
    if (i >= (long)rows * 64) return;
    const long r = i / 64;
    const uint32_t hw = reinterpret_cast<const uint32_t*>(h)[i];
    float a = bf((uint16_t)hw), b = bf((uint16_t)(hw >> 16));
    if (r < n_recv) {
        const float2 g = reinterpret_cast<const float2*>(agg)[i];
        a += g.x;
        b += g.y;
    }
    reinterpret_cast<uint32_t*>(out)[i] = pack2(a, b);
}

// d <- d * silu'(z) (in place), BF16 copy.
__global__ void k_act_grad(float* __restrict__ d, const float* __restrict__ z, long n, uint16_t* __restrict__ out) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float v = d[i] * silu_grad(z[i]);
    d[i] = v;
    out[i] = bf16_bits(v);
}

__global__ void k_to_bf16(const float* __restrict__ s, long n, uint16_t* __restrict__ out) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = bf16_bits(s[i]);
}

// d_h2 = g2 on receiver rows, 0 elsewhere.
__global__ void k_init_rows(const float* __restrict__ g, int n_recv, int rows, float* __restrict__ d) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long)rows * kH) return;
    d[i] = i < (long)n_recv * kH ? g[i] : 0.0f;
}

__global__ void __launch_bounds__(1024) k_loss(const float* __restrict__ out, const float* __restrict__ target, int n,
                                               float* __restrict__ loss, float* __restrict__ d_out) {
    __shared__ float red[32];
    const float inv = n > 0 ? 1.0f / (6.0f * (float)n) : 0.0f;
    float s = 0.0f;
    for (long i = threadIdx.x; i < (long)n * 16; i += blockDim.x) {
        const int col = (int)(i & 15);
        float g = 0.0f;
        if (col < 6) {
            const float d = out[i] - target[i];
            s += d * d;
            g = 2.0f * d * inv;
        }
        d_out[i] = g;
    }
    s = warp_sum(s);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        float t = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0f;
        t = warp_sum(t);
        if (threadIdx.x == 0) *loss = t * inv;
    }
}

// Edge term of the loss: lambda / E * sum over edges (i <- j) of
// |dx_i - dx_j|^2, dx = out[:, 0:3] - target[:, 0:3] (senders that are not
// receivers do not move: dx_j = 0).  Adds its gradient to d_out and its value
// to *loss (atomics: the order of the FP32 additions is not fixed).
__global__ void k_edge_loss(const int* __restrict__ offset, const int* __restrict__ sender,
                            const int* __restrict__ receiver, int n_recv, int cap, const float* __restrict__ out,
                            const float* __restrict__ target, float lambda, float* __restrict__ d_out,
                            float* __restrict__ loss) {
    const int E = min(offset[n_recv], cap);
    const float w = E > 0 ? lambda / (float)E : 0.0f;
    float part = 0.0f;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < E; e += gridDim.x * blockDim.x) {
        const int i = receiver[e], j = sender[e];
        const bool jr = j < n_recv;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const float di = out[16 * i + d] - target[16 * i + d];
            const float dj = jr ? out[16 * j + d] - target[16 * j + d] : 0.0f;
            const float g = di - dj;
            part += g * g;
            atomicAdd(d_out + 16 * i + d, 2.0f * w * g);
            if (jr) atomicAdd(d_out + 16 * j + d, -2.0f * w * g);
        }
    }
    part = warp_sum(part * w);
    if ((threadIdx.x & 31) == 0 && part != 0.0f) atomicAdd(loss, part);
}

__global__ void k_adam(float* __restrict__ th, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, int n, float lr, float b1, float b2, float eps, float c1, float c2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    th[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
}

struct ApplyArgs {
    float* pos[2];
    float* vel[2];
    const float* acc[2];
    int n[2];
    const float* out;
    int m;
    float dt;
    float sx[2], sv[2];
    const float* x_t;
    const float* v_t;
    float* target;
};

__global__ void k_apply(ApplyArgs a) {
    pdl_wait();
    pdl_launch();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n[0] + a.n[1]) return;
    const int s = i < a.n[0] ? 0 : 1;
    const int k = s ? i - a.n[0] : i;
    const float m = (float)a.m, dt = a.dt;
    const float cx = 0.5f * dt * dt * m * (m + 1.0f), cv = m * dt;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const float x = a.pos[s][3 * k + d], v = a.vel[s][3 * k + d], acc = a.acc[s][3 * k + d];
        const float px = x + cv * v + cx * acc;  // prior: m substeps at constant acceleration
        const float pv = v + cv * acc;
        if (a.target) {
            a.target[16 * i + d] = (a.x_t[3 * i + d] - px) / a.sx[s];
            a.target[16 * i + 3 + d] = (a.v_t[3 * i + d] - pv) / a.sv[s];
        } else {
            a.pos[s][3 * k + d] = px + a.sx[s] * a.out[16 * i + d];
            a.vel[s][3 * k + d] = pv + a.sv[s] * a.out[16 * i + 3 + d];
        }
    }
    if (a.target) {
#pragma unroll
        for (int d = 6; d < 16; ++d) a.target[16 * i + d] = 0.0f;
    }
}

__global__ void k_maxdev(const float* __restrict__ a, const float* __restrict__ b, float ref, int n, float inv,
                         float* __restrict__ out) {
    pdl_wait();
    pdl_launch();
    float m = 0.0f;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        m = fmaxf(m, fabsf(a[i] - (b ? b[i] : ref)) * inv);
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && m > 0.0f) atomicMax(reinterpret_cast<int*>(out), __float_as_int(m));
}

// ---------------------------------------------------------------------------
// node inputs and the radius graph
// ---------------------------------------------------------------------------
__global__ void k_nodes(sphdem_mpnn_nodes_t a) {
    pdl_wait();
    pdl_launch();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int nf = a.n_fluid, nd = a.n_dem, nb = a.n_wall, nw = a.n_dem_wall;
    if (i >= nf + nd + nb + nw) return;
    float p[3], v[3] = {0, 0, 0}, ac[3] = {0, 0, 0};
    float rho = 0.0f, por = 0.0f, rad = 0.0f;
    int type;
    if (i < nf) {
        type = 0;
        for (int d = 0; d < 3; ++d) {
            p[d] = a.f_pos[3 * i + d];
            v[d] = a.f_vel[3 * i + d];
            ac[d] = a.f_acc[3 * i + d];
        }
        rho = (a.f_rho[i] / a.rho0 - 1.0f) * 100.0f;
        por = a.f_por[i] - 1.0f;
    } else if (i < nf + nd) {
        type = 1;
        const int k = i - nf;
        for (int d = 0; d < 3; ++d) {
            p[d] = a.d_pos[3 * k + d];
            v[d] = a.d_vel[3 * k + d];
            ac[d] = a.d_acc[3 * k + d];
        }
        rad = a.d_rad[k] * a.inv_radius;
    } else if (i < nf + nd + nb) {
        type = 2;
        const int k = i - nf - nd;
        for (int d = 0; d < 3; ++d) p[d] = a.b_pos[3 * k + d];
        rho = (a.b_rho[k] / a.rho0 - 1.0f) * 100.0f;
    } else {
        type = 3;
        const int k = i - nf - nd - nb;
        for (int d = 0; d < 3; ++d) p[d] = a.w_pos[3 * k + d];
        rad = a.w_rad[k] * a.inv_radius;
    }
    for (int d = 0; d < 3; ++d) a.node_pos3[3 * i + d] = p[d];
    reinterpret_cast<float4*>(a.node_pos4)[i] = make_float4(p[0], p[1], p[2], 0.0f);
    reinterpret_cast<float4*>(a.node_vel4)[i] = make_float4(v[0], v[1], v[2], 0.0f);
    float f[16] = {v[0] * a.inv_vscale, v[1] * a.inv_vscale, v[2] * a.inv_vscale, ac[0] * a.inv_ascale,
                   ac[1] * a.inv_ascale, ac[2] * a.inv_ascale, rho, por, 0, 0, 0, 0, rad, 0, 0, 0};
    f[8 + type] = 1.0f;
    uint4* o = reinterpret_cast<uint4*>(a.x + (size_t)i * 16);
    o[0] = make_uint4(pack2(f[0], f[1]), pack2(f[2], f[3]), pack2(f[4], f[5]), pack2(f[6], f[7]));
    o[1] = make_uint4(pack2(f[8], f[9]), pack2(f[10], f[11]), pack2(f[12], f[13]), pack2(f[14], f[15]));
}

// One warp per receiver: the lanes test 32 candidate slots at a time (ranges
// of the ball-trimmed cell columns, in column order); accepted senders are
// compacted in slot order by ballot, so the list is deterministic.
template <bool FILL>
__global__ void k_graph(Geo g, const float4* __restrict__ pos, int n_recv, float r2, float rq, int* __restrict__ offset,
                        int* __restrict__ sender, int* __restrict__ receiver, int cap, sphdem_ctl_t* ctl) {
    pdl_wait();
    pdl_launch();
    const int i = (int)((blockIdx.x * (long)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (i >= n_recv) return;  // warp-uniform
    const float4 p = __ldg(pos + i);
    const int inst = inst_of(g, i);
    const int base = FILL ? offset[i] : 0;
    const unsigned below = (1u << lane) - 1u;
    int cnt = 0;
    warp_ranges_ball(g, p.x, p.y, p.z, rq, inst, [&](int s, int e) {
        for (int k0 = s; k0 < e; k0 += 32) {
            const int k = k0 + lane;
            bool in = false;
            int j = -1;
            if (k < e) {
                j = __ldg(g.order + k);
                if (j != i) {
                    const float4 q = __ldg(pos + j);
                    in = d2_exact(p.x, p.y, p.z, q.x, q.y, q.z).d2 < r2;
                }
            }
            const unsigned m = __ballot_sync(0xffffffffu, in);
            if (FILL && in) {
                const int slot = base + cnt + __popc(m & below);
                if (slot < cap) {
                    sender[slot] = j;
                    receiver[slot] = i;
                }
            }
            cnt += __popc(m);
        }
    });
    if (lane == 0) {
        if (!FILL) offset[i] = cnt;
        else if (i == n_recv - 1 && base + cnt > cap) flag(ctl, SPHDEM_FLAG_ROW_OVERFLOW);
    }
}

// ---------------------------------------------------------------------------
// host helpers
// ---------------------------------------------------------------------------
int sm_count() {
    static int n[64] = {0};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) dev = 0;
    if (n[dev] == 0) {
        int v = 0;
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        n[dev] = v > 0 ? v : 1;
    }
    return n[dev];
}

// Opt a kernel into `bytes` of dynamic shared memory (once per kernel and device).
template <class Kern>
int smem_opt_in(Kern k, uint32_t bytes) {
    static std::mutex mu;
    static std::map<std::pair<const void*, int>, uint32_t> done;
    int dev = 0;
    cudaGetDevice(&dev);
    const auto key = std::make_pair(reinterpret_cast<const void*>(k), dev);
    std::lock_guard<std::mutex> lock(mu);
    auto it = done.find(key);
    if (it != done.end() && it->second >= bytes) return SPHDEM_OK;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e != cudaSuccess) {
        set_error("mpnn: shared memory opt-in", e);
        return SPHDEM_ERR_CUDA;
    }
    done[key] = bytes;
    return SPHDEM_OK;
}

template <int K, int N, int EPI, bool IMG>
int rows(const uint16_t* A, int M, const uint16_t* B, const float* bias, float* out_f32, uint16_t* out_bf,
         float* z_out, int32_t* status, cudaStream_t st, const float* add = nullptr, int n_add = 0,
         const int* list = nullptr, int n_direct = 0, int early = 0) {
    if (M <= 0) return SPHDEM_OK;
    constexpr uint32_t bytes = N * K * 2 + kT * K * 2 + 4 * (N < 2 ? 2 : N) + 16 + 16;
    int rc = smem_opt_in(k_rows<K, N, EPI, IMG>, bytes);
    if (rc) return rc;
    const int tiles = (M + kT - 1) / kT;
    const int grid = tiles < 2 * sm_count() ? tiles : 2 * sm_count();
    launch_pdl(k_rows<K, N, EPI, IMG>, grid, kRT * kT, bytes, st, A, M, add, n_add, B, bias, out_f32, out_bf, z_out, status,
               list, n_direct, early);
    return launch_status("mpnn rows");
}

template <int N>
int wgrad(const uint16_t* P, const uint16_t* Q, int n_rows, float* partial, int& ncta, int32_t* status,
          cudaStream_t st) {
    constexpr uint32_t bytes = 128 * 128 * 2 + N * 128 * 2 + 16 + 16;
    int rc = smem_opt_in(k_wgrad<N>, bytes);
    if (rc) return rc;
    const int chunks = (n_rows + kT - 1) / kT;
    ncta = chunks < 1 ? 1 : chunks;
    if (ncta > sm_count()) ncta = sm_count();
    if (ncta > kMaxCtas) ncta = kMaxCtas;
    k_wgrad<N><<<ncta, kT, bytes, st>>>(P, Q, n_rows, partial, status);
    return launch_status("mpnn wgrad");
}

int reduce(const float* partial, int ncta, int stride, int off, int count, int rows_t, int cols_t, float* dst,
           cudaStream_t st) {
    k_reduce<<<blocks_for(count, 256), 256, 0, st>>>(partial, ncta, stride, off, count, rows_t, cols_t, dst);
    return launch_status("mpnn reduce");
}

int colsum(const float* m, int n_rows, int cols, float* part, float* dst, cudaStream_t st) {
    int nb = 2 * sm_count();
    int chunk = (n_rows + nb - 1) / nb;
    if (chunk < 1) chunk = 1;
    nb = (n_rows + chunk - 1) / chunk;
    if (nb < 1) nb = 1;
    k_colsum_part<<<nb, 128, 0, st>>>(m, n_rows, cols, chunk, part);
    k_reduce<<<1, 128, 0, st>>>(part, nb, cols, 0, cols, 0, 0, dst);
    return launch_status("mpnn colsum");
}

EdgeArgs edge_args(const sphdem_mpnn_net_t* n) {
    EdgeArgs a;
    memset(&a, 0, sizeof(a));
    a.pos = reinterpret_cast<const float4*>(n->node_pos4);
    a.vel = reinterpret_cast<const float4*>(n->node_vel4);
    a.offset = n->offset;
    a.sender = n->sender;
    a.receiver = n->receiver;
    a.n_recv = n->n_recv;
    a.cap = n->edge_capacity;
    a.inv_r = n->inv_radius;
    a.inv_vs = n->inv_vscale;
    a.inv_norm = n->inv_norm;
    a.img_e1 = n->packed + P_E1;
    a.img_e2 = n->packed + P_E2;
    a.img_e2t = n->packed + P_E2T;
    a.b1 = n->theta + SPHDEM_MPNN_E1_B;
    a.b2 = n->theta + SPHDEM_MPNN_E2_B;
    a.status = n->status;
    return a;
}

int edge_grid(const sphdem_mpnn_net_t* n, int per_sm) {
    const long tiles = ((long)n->edge_capacity + kT - 1) / kT;
    long g = (long)per_sm * sm_count();
    if (g > tiles) g = tiles;
    if (g > kMaxCtas) g = kMaxCtas;
    return g < 1 ? 1 : (int)g;
}

template <int MODE>
int edges(const EdgeArgs& a, int grid, cudaStream_t st) {
    int rc = smem_opt_in(k_edges<MODE>, EF_BYTES);
    if (rc) return rc;
    launch_pdl(k_edges<MODE>, grid, 2 * kPT, EF_BYTES, st, a);
    return launch_status("mpnn edges");
}

bool net_ok(const sphdem_mpnn_net_t* n) {
    return n && n->n_nodes >= n->n_recv && n->n_recv >= 0 && n->edge_capacity > 0 && n->node_pos4 &&
           n->node_vel4 && n->x && n->offset && n->sender && n->receiver && n->theta && n->packed && n->h0 &&
           n->agg && n->h1 && n->h2 && n->h3 && n->out;
}

}  // namespace
}  // namespace sd

using namespace sd;

extern "C" int64_t sphdem_mpnn_partial_floats(void) { return (int64_t)kMaxCtas * kBwdStride; }

extern "C" int sphdem_mpnn_pack(const float* theta, uint16_t* packed, sphdem_stream_t stream) {
    if (!theta || !packed) {
        set_error_msg("mpnn_pack: NULL pointer");
        return SPHDEM_ERR_INVALID;
    }
    k_pack<<<dim3(128, 8), 128, 0, as_stream(stream)>>>(theta, packed);
    return launch_status("mpnn_pack");
}

extern "C" int sphdem_mpnn_nodes(const sphdem_mpnn_nodes_t* in, sphdem_stream_t stream) {
    if (!in || !in->node_pos3 || !in->node_pos4 || !in->node_vel4 || !in->x) {
        set_error_msg("mpnn_nodes: NULL pointer");
        return SPHDEM_ERR_INVALID;
    }
    const long n = (long)in->n_fluid + in->n_dem + in->n_wall + in->n_dem_wall;
    if (n <= 0) return SPHDEM_OK;
    launch_pdl(k_nodes, blocks_for(n, 256), 256, 0, as_stream(stream), *in);
    return launch_status("mpnn_nodes");
}

extern "C" int sphdem_mpnn_graph(sphdem_grid_t* grid, const float* node_pos3, const float* node_pos4, int32_t n_recv,
                                 float radius, int32_t* offset, int32_t* sender, int32_t* receiver,
                                 int32_t edge_capacity, int32_t* scan_scratch, sphdem_ctl_t* ctl,
                                 sphdem_stream_t stream) {
    if (!grid || !node_pos3 || !node_pos4 || !offset || !sender || !receiver || !scan_scratch || n_recv < 0 ||
        n_recv > grid->n || !(radius > 0.0f) || edge_capacity <= 0 || grid->cell < radius) {
        set_error_msg("mpnn_graph: invalid arguments (cell must be >= radius, n_recv <= nodes)");
        return SPHDEM_ERR_INVALID;
    }
    cudaStream_t st = as_stream(stream);
    int rc = build_grid(grid, node_pos3, ctl, st);
    if (rc) return rc;
    if (n_recv == 0) {
        cudaError_t e = cudaMemsetAsync(offset, 0, sizeof(int32_t), st);
        if (e != cudaSuccess) {
            set_error("mpnn_graph", e);
            return SPHDEM_ERR_CUDA;
        }
        return SPHDEM_OK;
    }
    const Geo g = make_geo(*grid);
    const float r2 = radius * radius;
    const float rq = pad_radius(radius);
    const float4* p4 = reinterpret_cast<const float4*>(node_pos4);
    const int nb = blocks_for((long)n_recv * 32, 256);
    launch_pdl(k_graph<false>, nb, 256, 0, st, g, p4, n_recv, r2, rq, offset, sender, receiver, edge_capacity, ctl);
    rc = scan_counts(offset, n_recv, scan_scratch, st);
    if (rc) return rc;
    launch_pdl(k_graph<true>, nb, 256, 0, st, g, p4, n_recv, r2, rq, offset, sender, receiver, edge_capacity, ctl);
    return launch_status("mpnn_graph");
}

namespace sd {
namespace {
// Non-receiver senders of the current graph, each listed once: list[0] is
// their count, list[1 ..] the nodes (order immaterial: node rows are
// independent).  Edge count from the CSR offsets, bounded by the edge buffer
// (an overflowing graph keeps its full count there but only `cap` edges).
__global__ void k_mark_senders(const int* __restrict__ offset, const int* __restrict__ sender, int n_recv,
                               int n_nodes, int cap, int* __restrict__ active, int* __restrict__ list) {
    pdl_wait();
    pdl_launch();
    const int E = min(__ldg(offset + n_recv), cap);
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < E; e += gridDim.x * blockDim.x) {
        const int s = __ldg(sender + e);
        if (s >= n_recv && s < n_nodes && atomicExch(active + s, 1) == 0) list[1 + atomicAdd(list, 1)] = s;
    }
}
}  // namespace
}  // namespace sd

extern "C" int sphdem_mpnn_forward(const sphdem_mpnn_net_t* n, int store_pre, sphdem_stream_t stream) {
    if (!net_ok(n) || (store_pre && (!n->z0 || !n->z2))) {
        set_error_msg("mpnn_forward: invalid network state");
        return SPHDEM_ERR_INVALID;
    }
    cudaStream_t st = as_stream(stream);
    const int nn = n->n_nodes, nr = n->n_recv;
    // inference: node layers on the receivers and the other nodes that send
    const int* list = nullptr;
    if (!store_pre && n->active && n->active_list && nn > nr) {
        cudaError_t e = zero_words(n->active, nn, st);
        if (e == cudaSuccess) e = zero_words(n->active_list, 1, st);
        if (e != cudaSuccess) {
            set_error("mpnn_forward", e);
            return SPHDEM_ERR_CUDA;
        }
        launch_pdl(k_mark_senders, 2 * sm_count(), 256, 0, st, n->offset, n->sender, nr, nn, n->edge_capacity,
                   n->active, n->active_list);
        list = n->active_list;
    }
    int rc = rows<16, 128, EPI_SILU, true>(n->x, nn, n->packed + P_N1, n->theta + SPHDEM_MPNN_N1_B, nullptr, n->h0,
                                           store_pre ? n->z0 : nullptr, n->status, st, nullptr, 0, list, nr,
                                           list != nullptr);
    if (rc) return rc;
    // Inference copies the weight images early: every kernel of the chain
    // runs behind kernels that do not write them (the first node layer only
    // behind the sender marking, which itself waits on whatever packed them).
    EdgeArgs a = edge_args(n);
    a.early = !store_pre;
    const int eg = edge_grid(n, 1);
    for (int round = 0; round < 2; ++round) {
        cudaError_t e = zero_words(n->agg, (long)nr * kH, st);
        if (e != cudaSuccess) {
            set_error("mpnn_forward", e);
            return SPHDEM_ERR_CUDA;
        }
        a.h = round == 0 ? n->h0 : n->h2;
        a.agg = n->agg;
        if (nr > 0 && (rc = edges<MODE_AGG>(a, eg, st))) return rc;
        if (round == 0) {
            if (store_pre) {  // the backward pass needs h1 itself
                k_residual<<<blocks_for((long)nn * 64, 256), 256, 0, st>>>(n->h0, n->agg, nr, nn, n->h1);
                rc = rows<128, 128, EPI_SILU, true>(n->h1, nn, n->packed + P_N2, n->theta + SPHDEM_MPNN_N2_B,
                                                    nullptr, n->h2, n->z2, n->status, st);
            } else {  // h1 = h0 + agg formed while staging
                rc = rows<128, 128, EPI_SILU, true>(n->h0, nn, n->packed + P_N2, n->theta + SPHDEM_MPNN_N2_B,
                                                    nullptr, n->h2, nullptr, n->status, st, n->agg, nr, list, nr, 1);
            }
            if (rc) return rc;
        } else if (store_pre) {
            k_residual<<<blocks_for((long)nr * 64, 256), 256, 0, st>>>(n->h2, n->agg, nr, nr, n->h3);
        }
    }
    if (store_pre)
        rc = rows<128, 16, EPI_F32, true>(n->h3, nr, n->packed + P_N3, n->theta + SPHDEM_MPNN_N3_B, n->out, nullptr,
                                          nullptr, n->status, st);
    else
        rc = rows<128, 16, EPI_F32, true>(n->h2, nr, n->packed + P_N3, n->theta + SPHDEM_MPNN_N3_B, n->out, nullptr,
                                          nullptr, n->status, st, n->agg, nr, nullptr, 0, 1);
    if (rc) return rc;
    return launch_status("mpnn_forward");
}

extern "C" int sphdem_mpnn_backward(const sphdem_mpnn_net_t* n, const sphdem_mpnn_grad_t* g,
                                    sphdem_stream_t stream) {
    if (!net_ok(n) || !n->z0 || !n->z2 || !g || !g->d_out || !g->g2 || !g->d_h2 || !g->d_h1 || !g->d_h0 ||
        !g->bf_a || !g->bf_b || !g->partial || !g->grad) {
        set_error_msg("mpnn_backward: invalid arguments");
        return SPHDEM_ERR_INVALID;
    }
    cudaStream_t st = as_stream(stream);
    const int nn = n->n_nodes, nr = n->n_recv;
    const long nh = (long)nn * kH;
    float* grad = g->grad;
    int ncta = 0, rc;
    // output layer
    k_to_bf16<<<blocks_for((long)nr * 16, 256), 256, 0, st>>>(g->d_out, (long)nr * 16, g->bf_b);
    if ((rc = wgrad<16>(n->h3, g->bf_b, nr, g->partial, ncta, n->status, st))) return rc;
    if ((rc = reduce(g->partial, ncta, 128 * 16, 0, 128 * 16, 128, 16, grad + SPHDEM_MPNN_N3_W, st))) return rc;
    if ((rc = colsum(g->d_out, nr, 16, g->partial, grad + SPHDEM_MPNN_N3_B, st))) return rc;
    if ((rc = rows<16, 128, EPI_F32, true>(g->bf_b, nr, n->packed + P_N3T, nullptr, g->g2, nullptr, nullptr,
                                           n->status, st)))
        return rc;
    // second message round
    k_init_rows<<<blocks_for(nh, 256), 256, 0, st>>>(g->g2, nr, nn, g->d_h2);
    EdgeArgs a = edge_args(n);
    a.g = g->g2;
    a.dh = g->d_h2;
    if (nr > 0 && (rc = edges<MODE_SCATTER>(a, edge_grid(n, 1), st))) return rc;
    // second node layer
    k_act_grad<<<blocks_for(nh, 256), 256, 0, st>>>(g->d_h2, n->z2, nh, g->bf_a);
    if ((rc = wgrad<128>(g->bf_a, n->h1, nn, g->partial, ncta, n->status, st))) return rc;
    if ((rc = reduce(g->partial, ncta, 128 * 128, 0, 128 * 128, 0, 0, grad + SPHDEM_MPNN_N2_W, st))) return rc;
    if ((rc = colsum(g->d_h2, nn, 128, g->partial, grad + SPHDEM_MPNN_N2_B, st))) return rc;
    if ((rc = rows<128, 128, EPI_F32, true>(g->bf_a, nn, n->packed + P_N2T, nullptr, g->d_h1, nullptr, nullptr,
                                            n->status, st)))
        return rc;
    // first message round and the edge MLP
    cudaError_t e = cudaMemcpyAsync(g->d_h0, g->d_h1, sizeof(float) * (size_t)nh, cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) {
        set_error("mpnn_backward", e);
        return SPHDEM_ERR_CUDA;
    }
    a.g1 = g->d_h1;
    a.g2 = g->g2;
    a.h0 = n->h0;
    a.h2 = n->h2;
    a.dh0 = g->d_h0;
    a.partial = g->partial;
    const int bg = edge_grid(n, 1);
    if ((rc = smem_opt_in(k_edges_bwd, EB_BYTES))) return rc;
    if (nr > 0) {
        k_edges_bwd<<<bg, kT, EB_BYTES, st>>>(a);
        if ((rc = launch_status("mpnn edges_bwd"))) return rc;
        if ((rc = reduce(g->partial, bg, kBwdStride, 0, 128 * 128, 0, 0, grad + SPHDEM_MPNN_E2_W, st))) return rc;
        if ((rc = reduce(g->partial, bg, kBwdStride, 128 * 128, 128 * 16, 0, 0, grad + SPHDEM_MPNN_E1_W, st)))
            return rc;
        if ((rc = reduce(g->partial, bg, kBwdStride, 128 * 128 + 128 * 16, 128, 0, 0, grad + SPHDEM_MPNN_E1_B, st)))
            return rc;
        if ((rc = reduce(g->partial, bg, kBwdStride, 128 * 128 + 128 * 16 + 128, 128, 0, 0, grad + SPHDEM_MPNN_E2_B,
                         st)))
            return rc;
    } else {
        e = cudaMemsetAsync(grad, 0, sizeof(float) * SPHDEM_MPNN_N1_W, st);
        if (e != cudaSuccess) {
            set_error("mpnn_backward", e);
            return SPHDEM_ERR_CUDA;
        }
    }
    // first node layer
    k_act_grad<<<blocks_for(nh, 256), 256, 0, st>>>(g->d_h0, n->z0, nh, g->bf_a);
    if ((rc = wgrad<16>(g->bf_a, n->x, nn, g->partial, ncta, n->status, st))) return rc;
    if ((rc = reduce(g->partial, ncta, 128 * 16, 0, 128 * 16, 0, 0, grad + SPHDEM_MPNN_N1_W, st))) return rc;
    if ((rc = colsum(g->d_h0, nn, 128, g->partial, grad + SPHDEM_MPNN_N1_B, st))) return rc;
    return launch_status("mpnn_backward");
}

extern "C" int sphdem_mpnn_loss(const float* out, const float* target, int32_t n, float* loss, float* d_out,
                                sphdem_stream_t stream) {
    if (!out || !target || !loss || !d_out || n < 0) {
        set_error_msg("mpnn_loss: invalid arguments");
        return SPHDEM_ERR_INVALID;
    }
    k_loss<<<1, 1024, 0, as_stream(stream)>>>(out, target, n, loss, d_out);
    return launch_status("mpnn_loss");
}

extern "C" int sphdem_mpnn_edge_loss(const int32_t* offset, const int32_t* sender, const int32_t* receiver,
                                     int32_t n_recv, int32_t edge_capacity, const float* out, const float* target,
                                     float lambda, float* loss, float* d_out, sphdem_stream_t stream) {
    if (!offset || !sender || !receiver || !out || !target || !loss || !d_out || n_recv < 0 || edge_capacity < 0) {
        set_error_msg("mpnn_edge_loss: invalid arguments");
        return SPHDEM_ERR_INVALID;
    }
    if (n_recv == 0 || edge_capacity == 0) return SPHDEM_OK;
    int grid = blocks_for(edge_capacity, 256);
    if (grid > 8 * sm_count()) grid = 8 * sm_count();
    k_edge_loss<<<grid, 256, 0, as_stream(stream)>>>(offset, sender, receiver, n_recv, edge_capacity, out, target,
                                                    lambda, d_out, loss);
    return launch_status("mpnn_edge_loss");
}

extern "C" int sphdem_mpnn_adam(float* theta, const float* grad, float* m, float* v, int32_t n, float lr, float beta1,
                                float beta2, float eps, int32_t step, sphdem_stream_t stream) {
    if (!theta || !grad || !m || !v || n < 0 || step < 1) {
        set_error_msg("mpnn_adam: invalid arguments");
        return SPHDEM_ERR_INVALID;
    }
    const float c1 = (float)(1.0 / (1.0 - pow((double)beta1, step)));
    const float c2 = (float)(1.0 / (1.0 - pow((double)beta2, step)));
    k_adam<<<blocks_for(n > 0 ? n : 1, 256), 256, 0, as_stream(stream)>>>(theta, grad, m, v, n, lr, beta1, beta2, eps,
                                                                          c1, c2);
    return launch_status("mpnn_adam");
}

extern "C" int sphdem_mpnn_apply(float* f_pos, float* f_vel, const float* f_acc, int32_t n_fluid, float* d_pos,
                                 float* d_vel, const float* d_acc, int32_t n_dem, const float* out, int32_t m,
                                 float dt, const float* scale4, const float* x_t, const float* v_t, float* target,
                                 sphdem_stream_t stream) {
    if (!scale4 || n_fluid < 0 || n_dem < 0 || (n_fluid > 0 && (!f_pos || !f_vel || !f_acc)) ||
        (n_dem > 0 && (!d_pos || !d_vel || !d_acc)) || (!target && !out) || (target && (!x_t || !v_t))) {
        set_error_msg("mpnn_apply: invalid arguments");
        return SPHDEM_ERR_INVALID;
    }
    ApplyArgs a;
    a.pos[0] = f_pos;
    a.pos[1] = d_pos;
    a.vel[0] = f_vel;
    a.vel[1] = d_vel;
    a.acc[0] = f_acc;
    a.acc[1] = d_acc;
    a.n[0] = n_fluid;
    a.n[1] = n_dem;
    a.out = out;
    a.m = m;
    a.dt = dt;
    a.sx[0] = scale4[0];
    a.sv[0] = scale4[1];
    a.sx[1] = scale4[2];
    a.sv[1] = scale4[3];
    a.x_t = x_t;
    a.v_t = v_t;
    a.target = target;
    const int n = n_fluid + n_dem;
    if (n == 0) return SPHDEM_OK;
    launch_pdl(k_apply, blocks_for(n, 256), 256, 0, as_stream(stream), a);
    return launch_status("mpnn_apply");
}

namespace sd {

// Largest correction displacement of a jump: max over the receivers (fluid
// rows first, then DEM) of |s_x out[0:3]| + mdt |s_v out[3:6]| into *dst
// (float bits, atomicMax; values >= 0; *dst starts at 0).
__global__ void k_corrmax(const float* __restrict__ out, int nf, int nd, float4 sc, float mdt, float* dst) {
    pdl_wait();
    pdl_launch();
    float m = 0.0f;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nf + nd; i += gridDim.x * blockDim.x) {
        const float sx = i < nf ? sc.x : sc.z, sv = i < nf ? sc.y : sc.w;
        const float* o = out + 16 * (size_t)i;
        const float dx = sx * sqrtf(o[0] * o[0] + o[1] * o[1] + o[2] * o[2]);
        const float dv = sv * sqrtf(o[3] * o[3] + o[4] * o[4] + o[5] * o[5]);
        m = fmaxf(m, dx + mdt * dv);
    }
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && m > 0.0f) atomicMax(reinterpret_cast<int*>(dst), __float_as_int(m));
}

int run_corrmax(const float* out, int nf, int nd, const float* scale4, float mdt, float* dst, cudaStream_t st) {
    if (nf + nd <= 0) return SPHDEM_OK;
    int grid = blocks_for(nf + nd, 256);
    if (grid > 4 * sm_count()) grid = 4 * sm_count();
    launch_pdl(k_corrmax, grid, 256, 0, st, out, nf, nd, make_float4(scale4[0], scale4[1], scale4[2], scale4[3]),
               mdt, dst);
    return launch_status("jump correction");
}

}  // namespace sd

extern "C" int sphdem_mpnn_maxdev(const float* a, const float* b, float ref, int32_t n, float inv, float* out,
                                  sphdem_stream_t stream) {
    if (!a || !out || n < 0) {
        set_error_msg("mpnn_maxdev: invalid arguments");
        return SPHDEM_ERR_INVALID;
    }
    if (n == 0) return SPHDEM_OK;
    int grid = blocks_for(n, 256);
    if (grid > 4 * sm_count()) grid = 4 * sm_count();
    launch_pdl(k_maxdev, grid, 256, 0, as_stream(stream), a, b, ref, n, inv, out);
    return launch_status("mpnn_maxdev");
}

extern "C" int sphdem_mpnn_gemm(const uint16_t* a, const uint16_t* b, float* c, int32_t m, int32_t n, int32_t k,
                                int32_t* status, sphdem_stream_t stream) {
    if (!a || !b || !c || m < 0 || (n != 16 && n != 128) || (k != 16 && k != 128)) {
        set_error_msg("mpnn_gemm: N and K must be 16 or 128");
        return SPHDEM_ERR_INVALID;
    }
    cudaStream_t st = as_stream(stream);
    if (k == 16 && n == 16) return rows<16, 16, EPI_F32, false>(a, m, b, nullptr, c, nullptr, nullptr, status, st);
    if (k == 16 && n == 128) return rows<16, 128, EPI_F32, false>(a, m, b, nullptr, c, nullptr, nullptr, status, st);
    if (k == 128 && n == 16) return rows<128, 16, EPI_F32, false>(a, m, b, nullptr, c, nullptr, nullptr, status, st);
    return rows<128, 128, EPI_F32, false>(a, m, b, nullptr, c, nullptr, nullptr, status, st);
}

extern "C" int sphdem_mpnn_wgrad(const uint16_t* p, const uint16_t* q, float* c, int32_t n_rows, int32_t n,
                                 float* partial, int32_t* status, sphdem_stream_t stream) {
    if (!p || !q || !c || !partial || n_rows < 0 || (n != 16 && n != 128)) {
        set_error_msg("mpnn_wgrad: N must be 16 or 128");
        return SPHDEM_ERR_INVALID;
    }
    cudaStream_t st = as_stream(stream);
    int ncta = 0, rc;
    if (n == 16)
        rc = wgrad<16>(p, q, n_rows, partial, ncta, status, st);
    else
        rc = wgrad<128>(p, q, n_rows, partial, ncta, status, st);
    if (rc) return rc;
    return reduce(partial, ncta, 128 * n, 0, 128 * n, 0, 0, c, st);
}
