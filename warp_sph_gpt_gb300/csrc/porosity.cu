// porosity.cu -- the porosity pass of Kernel_prep_sphdem
// (kernel/KERNEL_SPHDEM_interaction.py:43-95) for a uniform DEM coupling
// length h, with the fluid normaliser's pair distances on the tensor cores.
//
// The normaliser of a fluid particle i near a sphere is
//     flt_i = 21/(16 pi h^3) sum_j V_j w(|x_i - x_j|^2 / h^2),
//     w(s) = (1 - q/2)^4 (1 + 2q),  q = sqrt(s), s clamped to 4,
// over every fluid j (w vanishes from q = 2 on, so candidates beyond the
// coupling support add exact zeros and no membership test is needed).  At
// the large dam break a listed particle has ~54k neighbours, so the pass is
// ~4.5e9 pair evaluations per step.  Here the squared distances of a tile of
// 128 subjects against a chunk of 128 candidates come from one tcgen05 MMA:
//     s_ij = |p_i|^2 + |q_j|^2 - 2 p_i . q_j
// with p, q in units of h relative to a common centre, every FP32 operand
// split exactly into three BF16 pieces (a = a0 + a1 + a2) and the six
// significant products of p . q, plus the pieces of |p|^2 and |q|^2 times
// ones, laid along K = 32: the FP32 accumulation of exact BF16 products gives
// s to ~1e-6 of the ball radius squared.  The CUDA cores then evaluate only
// w(s) (one MUFU square root, the polynomial on packed FP32 pairs) and the
// V_j-weighted sums.
//
// Every subject's sum is canonical -- the same bits whatever the tiling, the
// launch shape or the other members of a batched state:
//   * the centre of a tile is the centre of a world-anchored frame block of
//     F x F x F fluid-grid cells, and a tile holds listed particles of one
//     frame block only, so p_i and q_j depend only on (i, j);
//   * candidate ranges are padded to slot offsets aligned to 8 within their
//     instance (padding carries V = 0), so candidate j always lands in
//     accumulator (slot - instance start) mod 8 of the eight per subject: the
//     two epilogue warps of a TMEM lane quarter own classes 0-3 and 4-7
//     (staging puts them in chunk columns 0-63 and 64-127);
//   * the window is cut into world-anchored column slabs of Wx columns; each
//     (tile, slab) work unit writes a partial sum per subject, and the finish
//     kernel adds a subject's slab partials in slab order.
// Candidates outside a subject's own ball add +0 exactly, so the extra
// candidates of a tile's wider window change nothing.
//
// Kernels (one porosity pass):
//   k_pnear      one thread per fluid slot: a DEM within 2 h_b?  Dry particles
//                get clamp(1); listed ones are counted per frame block, and a
//                frame block's first listed particle puts it on a list.
//   k_plist      one warp per listed frame block: reserves its segment of the
//                near list and of the tile table (atomics: segment placement
//                varies, results do not), writes its listed slots by 2 x 2 x 2
//                cell sub-blocks (so a tile of 128 is compact) and its tiles.
//   k_porosity_mma  persistent, 2 CTAs per SM: work units (tile, slab);
//                warps 0-7 epilogue (TMEM lane = subject; warp w reads lane
//                quarter w mod 4, chunk half w / 4), warp 8 issues the MMAs
//                and owns tensor memory, warps 9-10 stage candidate rows
//                (each thread loads its next chunk's candidates while it
//                builds the current chunk's rows).
//   k_pfinish    one thread per listed particle: slab partials -> flt, solid
//                fraction over the DEM neighbours, porosity.
// Every wait is bounded; a timeout raises SPHDEM_FLAG_TIMEOUT, the CTA drains
// its MMAs (bounded) and frees its tensor memory.
#include <cuda_bf16.h>

#include <map>
#include <mutex>
#include <utility>

#include "common.cuh"
#include "umma.cuh"

namespace sd {

namespace {

constexpr int kPM = 128;            // subjects per tile (MMA M, TMEM lanes)
constexpr int kPN = 128;            // candidates per chunk (MMA N, TMEM columns)
constexpr int kPK = 32;             // BF16 K of the distance MMA (24 used)
constexpr int kPStages = 6;         // candidate-row stages in shared memory
constexpr int kPSlabs = SPHDEM_POROSITY_SLABS;
constexpr int kPMaxRanges = 512;    // candidate ranges per column batch
constexpr int kPMaxChunks = 2048;   // chunks per column batch with a precomputed first range
constexpr int kPEpiWarps = 8;       // two per TMEM lane quarter, one per half of each chunk
constexpr int kPMmaWarp = 8;
constexpr int kPStageWarps = 2;
constexpr int kPThreads = 32 * (kPEpiWarps + 1 + kPStageWarps);  // 352
constexpr int kPStageThreads = 32 * kPStageWarps;
constexpr int kPAlign = 8;          // candidate class = slot offset in the instance mod 8
constexpr uint32_t kPRowBytes = kPK * 2;
constexpr uint32_t kPTileBytes = kPM * kPRowBytes;  // = kPN * kPRowBytes
constexpr uint32_t kPTmemCols = 2 * kPN;            // two accumulator buffers
constexpr int kPPolls = 1 << 20;

struct PorSmem {
    uint8_t A[kPTileBytes];               // subjects (1024-aligned)
    uint8_t B[kPStages][kPTileBytes];     // candidate rows
    float V[kPStages][kPN];               // candidate volumes (0: padding)
    int rs[kPMaxRanges];                  // aligned first slot of each range
    int info[kPMaxRanges];                // leading pad | (true length << 3)
    int pre[kPMaxRanges + 1];             // exclusive prefix of aligned lengths
    int cr[kPMaxChunks + 1];              // range holding each chunk's first candidate
    uint64_t full[kPStages], empty[kPStages], afull[2], aempty[2], drain;
    float red[6][4];
    float hsum[kPM];                      // second-half sums of each subject
    int wtot[kPThreads / 32];
    int unit, abort_flag;
    int tstart, tcount, slab;             // the current work unit's tile and slab
    uint32_t tmem;
};
// Dynamic shared memory per CTA: the struct, its 1024-byte alignment, and a
// floor that keeps at most two CTAs (2 x 256 TMEM columns) on an SM.
constexpr uint32_t kPSmemBytes = (sizeof(PorSmem) + 1024 > 80u * 1024u) ? (uint32_t)sizeof(PorSmem) + 1024u
                                                                         : 80u * 1024u;

struct PorArgs {
    Geo gs, gd;
    const float4* __restrict__ f_posm;  // x, y, z, m (fluid, grid order; the near flags read these)
    const float4* __restrict__ f_posv;  // x, y, z, m/rho (fluid, grid order)
    const float4* __restrict__ aux;     // per DEM: 1/h, cw, sqrt bound of 2h, 2h
    sphdem_sph_t P;
    sphdem_dem_t D;
    int* near_list;
    int* flag;      // [n_sph] near flag per slot
    int* cnt;       // [nfb] listed particles per frame block
    int* fbl;       // [nfb] frame blocks with listed particles
    int4* tiles;    // (near start, count, frame block, 0)
    float* part;    // [n_sph * kPSlabs]
    sphdem_ctl_t* ctl;
    float rq;       // padded coupling support (2 h, world units)
    float inv_h, cw, eps_min, eps_max;
    int F;          // frame-block edge in cells
    int f0[3], nf[3], nfb_local, nfb;
    int Wx;         // slab width in columns
};

__device__ __forceinline__ int floor_div(int a, int b) { return a >= 0 ? a / b : -((-a + b - 1) / b); }

__device__ __forceinline__ float sqrt_apx(float x) {
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// Exact three-piece BF16 split of an FP32 value: a = a0 + a1 + a2.
__device__ __forceinline__ void split3(float a, float& a0, float& a1, float& a2) {
    a0 = __bfloat162float(__float2bfloat16_rn(a));
    const float r1 = a - a0;
    a1 = __bfloat162float(__float2bfloat16_rn(r1));
    a2 = __bfloat162float(__float2bfloat16_rn(r1 - a1));
}

__device__ __forceinline__ uint32_t pk(float a, float b) {
    __nv_bfloat162 h = __floats2bfloat162_rn(a, b);  // exact: both already BF16 values
    return *reinterpret_cast<uint32_t*>(&h);
}

// One 64-byte operand row (32 BF16 along K) at row r of a K-major tile:
// v[0..23] the used columns, 24..31 zero.
__device__ __forceinline__ void store_row(uint8_t* tile, int r, const float* v) {
    uint4 w0 = make_uint4(pk(v[0], v[1]), pk(v[2], v[3]), pk(v[4], v[5]), pk(v[6], v[7]));
    uint4 w1 = make_uint4(pk(v[8], v[9]), pk(v[10], v[11]), pk(v[12], v[13]), pk(v[14], v[15]));
    uint4 w2 = make_uint4(pk(v[16], v[17]), pk(v[18], v[19]), pk(v[20], v[21]), pk(v[22], v[23]));
    *reinterpret_cast<uint4*>(tile + umma::tile_off(r, 0, kPK)) = w0;
    *reinterpret_cast<uint4*>(tile + umma::tile_off(r, 8, kPK)) = w1;
    *reinterpret_cast<uint4*>(tile + umma::tile_off(r, 16, kPK)) = w2;
    *reinterpret_cast<uint4*>(tile + umma::tile_off(r, 24, kPK)) = make_uint4(0, 0, 0, 0);
}

// Subject row: p pieces against -2 q pieces (p0q0, p0q1, p1q0, p0q2, p1q1,
// p2q0 per coordinate), |p|^2 pieces against ones, ones against |q|^2 pieces.
__device__ __forceinline__ void subject_row(float px, float py, float pz, float* v) {
    float x[3][3];
    split3(px, x[0][0], x[0][1], x[0][2]);
    split3(py, x[1][0], x[1][1], x[1][2]);
    split3(pz, x[2][0], x[2][1], x[2][2]);
    const float pp = fmaf(pz, pz, fmaf(py, py, px * px));
    const int pa[6] = {0, 0, 1, 0, 1, 2};
#pragma unroll
    for (int g = 0; g < 6; ++g)
#pragma unroll
        for (int d = 0; d < 3; ++d) v[3 * g + d] = x[d][pa[g]];
    split3(pp, v[18], v[19], v[20]);
    v[21] = v[22] = v[23] = 1.0f;
}

__device__ __forceinline__ void candidate_row(float qx, float qy, float qz, float* v) {
    float x[3][3];
    split3(-2.0f * qx, x[0][0], x[0][1], x[0][2]);
    split3(-2.0f * qy, x[1][0], x[1][1], x[1][2]);
    split3(-2.0f * qz, x[2][0], x[2][1], x[2][2]);
    const float qq = fmaf(qz, qz, fmaf(qy, qy, qx * qx));
    const int pb[6] = {0, 1, 0, 2, 1, 0};
#pragma unroll
    for (int g = 0; g < 6; ++g)
#pragma unroll
        for (int d = 0; d < 3; ++d) v[3 * g + d] = x[d][pb[g]];
    v[18] = v[19] = v[20] = 1.0f;
    split3(qq, v[21], v[22], v[23]);
}

// Frame block of local cell (cx, cy, cz) of instance inst.
__device__ __forceinline__ int frame_of(const PorArgs& a, int inst, int cx, int cy, int cz) {
    const int fx = floor_div(a.gs.lo[0] + cx, a.F) - a.f0[0];
    const int fy = floor_div(a.gs.lo[1] + cy, a.F) - a.f0[1];
    const int fz = floor_div(a.gs.lo[2] + cz, a.F) - a.f0[2];
    return inst * a.nfb_local + (fx * a.nf[1] + fy) * a.nf[2] + fz;
}

// Local cell range [c0, c1] of frame block coordinate f along axis d.
__device__ __forceinline__ void frame_cells(const PorArgs& a, int d, int f, int& c0, int& c1) {
    const int w0 = (a.f0[d] + f) * a.F;
    c0 = max(w0 - a.gs.lo[d], 0);
    c1 = min(w0 + a.F - 1 - a.gs.lo[d], a.gs.dim[d] - 1);
}

// ---------------------------------------------------------------------------
// near flags, dry particles, per-frame-block counts
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_pnear(PorArgs a) {
    pdl_wait();
    pdl_launch();
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= a.P.n) return;
    const int o = a.gs.order[k];
    const float4 p = a.f_posm[k];  // positions only: runs before the density pass is done
    const int key = a.gs.key[o];
    const int inst = a.gs.ncl > 0 ? key / a.gs.ncl : 0;
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
    a.flag[k] = near ? 1 : 0;
    if (near) {
        const int local = key - inst * a.gs.ncl;
        const int cz = local % a.gs.dim[2], cy = (local / a.gs.dim[2]) % a.gs.dim[1];
        const int cx = local / (a.gs.dim[2] * a.gs.dim[1]);
        const int fb = frame_of(a, inst, cx, cy, cz);
        if (atomicAdd(&a.cnt[fb], 1) == 0) a.fbl[atomicAdd(&a.ctl->n_pfb, 1)] = fb;
    } else {
        a.P.porosity[o] = fminf(fmaxf(1.0f, a.eps_min), a.eps_max);
    }
}

// ---------------------------------------------------------------------------
// listed slots of each frame block by sub-blocks of 2 x 2 x 2 cells, and its tiles
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_plist(PorArgs a) {
    pdl_wait();
    pdl_launch();
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    const int n_pfb = a.ctl->n_pfb;
    for (int i = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); i < n_pfb; i += nw) {
        const int fb = a.fbl[i];
        const int c = a.cnt[fb];
        const int nt = (c + kPM - 1) / kPM;
        int n0 = 0, t0 = 0;
        if (lane == 0) {
            n0 = atomicAdd(&a.ctl->n_near, c);
            t0 = atomicAdd(&a.ctl->n_ptiles, nt);
        }
        n0 = __shfl_sync(0xffffffffu, n0, 0);
        t0 = __shfl_sync(0xffffffffu, t0, 0);
        const int inst = fb / a.nfb_local;
        const int l = fb - inst * a.nfb_local;
        const int fz = l % a.nf[2], fy = (l / a.nf[2]) % a.nf[1], fx = l / (a.nf[2] * a.nf[1]);
        int x0, x1, y0, y1, z0, z1;
        frame_cells(a, 0, fx, x0, x1);
        frame_cells(a, 1, fy, y0, y1);
        frame_cells(a, 2, fz, z0, z1);
        int pos = n0;
        // 2 x 2 x 2-cell sub-blocks in turn, so that consecutive tiles are compact
        for (int bx = x0; bx <= x1; bx += 2)
            for (int by = y0; by <= y1; by += 2)
                for (int bz = z0; bz <= z1; bz += 2)
                    for (int cx = bx; cx <= min(bx + 1, x1); ++cx)
                        for (int cy = by; cy <= min(by + 1, y1); ++cy) {
                            const int base = inst * a.gs.ncl + (cx * a.gs.dim[1] + cy) * a.gs.dim[2];
                            const int s = a.gs.start[base + bz], e = a.gs.start[base + min(bz + 1, z1) + 1];
                            for (int k0 = s; k0 < e; k0 += 32) {
                                const int k = k0 + lane;
                                const bool near = k < e && a.flag[k] != 0;
                                const unsigned m = __ballot_sync(0xffffffffu, near);
                                if (near) a.near_list[pos + __popc(m & ((1u << lane) - 1u))] = k;
                                pos += __popc(m);
                            }
                        }
        for (int t = lane; t < nt; t += 32) a.tiles[t0 + t] = make_int4(n0 + kPM * t, min(kPM, c - kPM * t), fb, 0);
    }
}

// ---------------------------------------------------------------------------
// the normaliser on the tensor cores
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool bwait(uint64_t* bar, uint32_t parity, PorSmem& sh, sphdem_ctl_t* ctl) {
    if (mbar_wait(bar, parity, kPPolls)) return true;
    sh.abort_flag = 1;
    flag(ctl, SPHDEM_FLAG_TIMEOUT);
    return false;
}

// 16 columns of this thread's TMEM lane, loaded and waited for in one statement.
__device__ __forceinline__ void ld16(uint32_t taddr, uint32_t* r) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
}

// The polynomial's packed constants as 64-bit register pairs.
struct Kpk {
    unsigned long long k0, k1, k2, k3, one;
};
__device__ __forceinline__ unsigned long long pk2(float a) {
    return ((unsigned long long)__float_as_uint(a) << 32) | __float_as_uint(a);
}

// The weighted sums of 16 chunk columns r (s_ij bits of this thread's
// subject): column 4i + c holds a candidate of class c (or c + 4 in the second
// half of the chunk) and goes to accumulator c (a01 holds classes 0-1, a23
// classes 2-3, as FP32 pairs).  u^4 (1 + 2q), u = 1 - q/2, is evaluated as the
// expanded polynomial 1 + s (-5/2 + q (5/2 + q (-15/16 + q/8))) with s = q^2
// clamped to [0, 4] (|s| first: the MMA's rounding can leave a coincident pair
// slightly negative): every Horner step is exact at q = 2, so the weight there
// is exactly 0.  The polynomial and the sums run on packed FP32 pairs
// (fma.rn.ftz.f32x2: two independent round-to-nearest FMAs); V (candidate
// volumes, 0 for padding) is read from shared memory at vaddr.
//
// sums16_next is one statement that first issues the load of the lane's next
// 16 columns into s and ends with the wait for it: the arithmetic reads only
// registers that are not the load's destination, and nothing outside the
// statement sees s before the data has landed, so the load's latency hides
// behind the arithmetic without a register of a load in flight ever being
// read, moved or spilled.
// PTX of four columns: operands R0..R3 hold their s bits, V the shared-memory
// address of the chunk's volumes, OFF the byte offset of these four, A01/A23
// the accumulators, K0..K3/ONE the packed polynomial constants.
#define POR_SUMS4(R0, R1, R2, R3, V, OFF, A01, A23, K0, K1, K2, K3, ONE)                              \
    "mov.b32 s0, %" #R0 ";\n\tmov.b32 s1, %" #R1 ";\n\tmov.b32 s2, %" #R2 ";\n\tmov.b32 s3, %" #R3 ";\n\t" \
    "abs.ftz.f32 s0, s0;\n\tabs.ftz.f32 s1, s1;\n\tabs.ftz.f32 s2, s2;\n\tabs.ftz.f32 s3, s3;\n\t"        \
    "min.ftz.f32 s0, s0, 0f40800000;\n\tmin.ftz.f32 s1, s1, 0f40800000;\n\t"                           \
    "min.ftz.f32 s2, s2, 0f40800000;\n\tmin.ftz.f32 s3, s3, 0f40800000;\n\t"                           \
    "sqrt.approx.ftz.f32 q0, s0;\n\tsqrt.approx.ftz.f32 q1, s1;\n\t"                                    \
    "sqrt.approx.ftz.f32 q2, s2;\n\tsqrt.approx.ftz.f32 q3, s3;\n\t"                                    \
    "mov.b64 sa, {s0, s1};\n\tmov.b64 sb, {s2, s3};\n\tmov.b64 qa, {q0, q1};\n\tmov.b64 qb, {q2, q3};\n\t" \
    "fma.rn.ftz.f32x2 ca, %" #K0 ", qa, %" #K1 ";\n\tfma.rn.ftz.f32x2 cb, %" #K0 ", qb, %" #K1 ";\n\t"   \
    "fma.rn.ftz.f32x2 ca, ca, qa, %" #K2 ";\n\tfma.rn.ftz.f32x2 cb, cb, qb, %" #K2 ";\n\t"               \
    "fma.rn.ftz.f32x2 ca, ca, qa, %" #K3 ";\n\tfma.rn.ftz.f32x2 cb, cb, qb, %" #K3 ";\n\t"               \
    "fma.rn.ftz.f32x2 wa, ca, sa, %" #ONE ";\n\tfma.rn.ftz.f32x2 wb, cb, sb, %" #ONE ";\n\t"             \
    "ld.shared.v4.f32 {v0, v1, v2, v3}, [%" #V "+" #OFF "];\n\t"                                         \
    "mov.b64 va, {v0, v1};\n\tmov.b64 vb, {v2, v3};\n\t"                                                \
    "fma.rn.ftz.f32x2 %" #A01 ", va, wa, %" #A01 ";\n\tfma.rn.ftz.f32x2 %" #A23 ", vb, wb, %" #A23 ";\n\t"
#define POR_REGS                          \
    ".reg .f32 s<4>, q<4>, v<4>;\n\t"     \
    ".reg .b64 sa, sb, qa, qb, ca, cb, va, vb, wa, wb;\n\t"

// Operands: %0-%15 s (next columns), %16/%17 a01/a23, %18-%33 r, %34 vaddr,
// %35 the next columns' TMEM address, %36-%40 the constants.
__device__ __forceinline__ void sums16_next(const uint32_t* r, uint32_t vaddr, uint32_t tnext, uint32_t* s,
                                            unsigned long long& a01, unsigned long long& a23, const Kpk& K) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%35];\n\t"
        "{\n\t" POR_REGS
        POR_SUMS4(18, 19, 20, 21, 34, 0, 16, 17, 36, 37, 38, 39, 40)
        POR_SUMS4(22, 23, 24, 25, 34, 16, 16, 17, 36, 37, 38, 39, 40)
        POR_SUMS4(26, 27, 28, 29, 34, 32, 16, 17, 36, 37, 38, 39, 40)
        POR_SUMS4(30, 31, 32, 33, 34, 48, 16, 17, 36, 37, 38, 39, 40)
        "}\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(s[0]), "=r"(s[1]), "=r"(s[2]), "=r"(s[3]), "=r"(s[4]), "=r"(s[5]), "=r"(s[6]), "=r"(s[7]),
          "=r"(s[8]), "=r"(s[9]), "=r"(s[10]), "=r"(s[11]), "=r"(s[12]), "=r"(s[13]), "=r"(s[14]), "=r"(s[15]),
          "+l"(a01), "+l"(a23)
        : "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]), "r"(r[8]),
          "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15]), "r"(vaddr),
          "r"(tnext), "l"(K.k0), "l"(K.k1), "l"(K.k2), "l"(K.k3), "l"(K.one)
        : "memory");
}

// The same arithmetic on the last 16 columns of a chunk half (no load behind
// it).  Operands: %0/%1 a01/a23, %2-%17 r, %18 vaddr, %19-%23 the constants.
__device__ __forceinline__ void sums16(const uint32_t* r, uint32_t vaddr, unsigned long long& a01,
                                       unsigned long long& a23, const Kpk& K) {
    asm volatile(
        "{\n\t" POR_REGS
        POR_SUMS4(2, 3, 4, 5, 18, 0, 0, 1, 19, 20, 21, 22, 23)
        POR_SUMS4(6, 7, 8, 9, 18, 16, 0, 1, 19, 20, 21, 22, 23)
        POR_SUMS4(10, 11, 12, 13, 18, 32, 0, 1, 19, 20, 21, 22, 23)
        POR_SUMS4(14, 15, 16, 17, 18, 48, 0, 1, 19, 20, 21, 22, 23)
        "}"
        : "+l"(a01), "+l"(a23)
        : "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]), "r"(r[8]),
          "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15]), "r"(vaddr),
          "l"(K.k0), "l"(K.k1), "l"(K.k2), "l"(K.k3), "l"(K.one)
        : "memory");
}
#undef POR_SUMS4
#undef POR_REGS

__global__ void __launch_bounds__(kPThreads, 2) k_porosity_mma(PorArgs a) {
    pdl_wait();
    pdl_launch();
    extern __shared__ uint8_t raw[];
    PorSmem& sh = *reinterpret_cast<PorSmem*>((reinterpret_cast<uintptr_t>(raw) + 1023) & ~uintptr_t(1023));
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid == 0) {
        for (int s = 0; s < kPStages; ++s) {
            mbar_init(&sh.full[s], kPStageWarps);
            mbar_init(&sh.empty[s], 1 + kPEpiWarps);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&sh.afull[b], 1);
            mbar_init(&sh.aempty[b], kPEpiWarps);
        }
        mbar_init(&sh.drain, 1);
        fence_mbar_init();
        sh.abort_flag = 0;
    }
    if (warp == kPMmaWarp) umma::tmem_alloc(&sh.tmem, kPTmemCols);
    umma::fence_before();
    __syncthreads();
    umma::fence_after();
    const uint32_t tmem = sh.tmem;
    const Geo& G = a.gs;
    const int n_units = a.ctl->n_ptiles * kPSlabs;
    constexpr uint32_t idesc = umma::idesc_bf16(kPM, kPN);
    uint32_t g = 0;          // chunks run so far by this CTA (same count in every role)
    bool issued = false;     // this CTA issued MMAs (drained before freeing TMEM)

    for (;;) {
        __syncthreads();
        if (tid == 0) {
            const int u0 = sh.abort_flag ? n_units : atomicAdd(&a.ctl->near_next, 1);
            sh.unit = u0;
            if (u0 < n_units) {
                const int4 T0 = a.tiles[u0 / kPSlabs];
                sh.tstart = T0.x;
                sh.tcount = T0.y;
                sh.slab = u0 % kPSlabs;
            }
        }
        __syncthreads();
        const int u = sh.unit;
        if (u >= n_units) break;
        const int tile = u / kPSlabs, slab = u - tile * kPSlabs;
        const int4 T = a.tiles[tile];
        const int fb = T.z;
        const int inst = fb / a.nfb_local;
        const int l = fb - inst * a.nfb_local;
        const int fzl = l % a.nf[2], fyl = (l / a.nf[2]) % a.nf[1], fxl = l / (a.nf[2] * a.nf[1]);
        // canonical centre: the frame block's centre (world units)
        const float half = 0.5f * (float)a.F * G.cell;
        const float cxw = (float)((a.f0[0] + fxl) * a.F) * G.cell + half;
        const float cyw = (float)((a.f0[1] + fyl) * a.F) * G.cell + half;
        const float czw = (float)((a.f0[2] + fzl) * a.F) * G.cell + half;
        // subjects: A rows and the tile's world box (warps 0-3; row = tid)
        float2 acc01 = make_float2(0.f, 0.f), acc23 = make_float2(0.f, 0.f);
        if (warp < 4) {
            float px = 0.f, py = 0.f, pz = 0.f;
            float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
            if (tid < T.y) {
                const float4 x = a.f_posv[a.near_list[T.x + tid]];
                px = (x.x - cxw) * a.inv_h;
                py = (x.y - cyw) * a.inv_h;
                pz = (x.z - czw) * a.inv_h;
                lo[0] = hi[0] = x.x;
                lo[1] = hi[1] = x.y;
                lo[2] = hi[2] = x.z;
            }
            float v[24];
            subject_row(px, py, pz, v);
            store_row(sh.A, tid, v);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    lo[d] = fminf(lo[d], __shfl_xor_sync(0xffffffffu, lo[d], o));
                    hi[d] = fmaxf(hi[d], __shfl_xor_sync(0xffffffffu, hi[d], o));
                }
            if (lane == 0)
                for (int d = 0; d < 3; ++d) {
                    sh.red[d][warp] = lo[d];
                    sh.red[3 + d][warp] = hi[d];
                }
            fence_proxy_async_smem();  // A is read by the MMA (async proxy)
        }
        __syncthreads();
        float bb[6];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            bb[d] = fminf(fminf(sh.red[d][0], sh.red[d][1]), fminf(sh.red[d][2], sh.red[d][3]));
            bb[3 + d] = fmaxf(fmaxf(sh.red[3 + d][0], sh.red[3 + d][1]), fmaxf(sh.red[3 + d][2], sh.red[3 + d][3]));
        }
        // window columns of the tile, cut to this unit's world-anchored slab
        const float rq = a.rq;
        const int wx0 = coord(bb[0] - rq, G.inv, G.lo[0], G.dim[0]), wx1 = coord(bb[3] + rq, G.inv, G.lo[0], G.dim[0]);
        const int wy0 = coord(bb[1] - rq, G.inv, G.lo[1], G.dim[1]), wy1 = coord(bb[4] + rq, G.inv, G.lo[1], G.dim[1]);
        const int sw = floor_div(G.lo[0] + wx0, a.Wx) + slab;
        const int sx0 = max(wx0, sw * a.Wx - G.lo[0]), sx1 = min(wx1, sw * a.Wx + a.Wx - 1 - G.lo[0]);
        const int ny = wy1 - wy0 + 1;
        const int ncols = sx1 >= sx0 ? (sx1 - sx0 + 1) * ny : 0;
        const int S_m = G.start[inst * G.ncl];  // first slot of the instance (slot alignment origin)
        const float margin = 0.01f * G.cell;
        for (int c0 = 0; c0 < ncols; c0 += kPMaxRanges) {
            // trim each column of the batch to the ball around the bounding box,
            // pad to 8-aligned instance slot offsets, compact in column order
            constexpr int kPer = (kPMaxRanges + kPThreads - 1) / kPThreads;
            int ls[kPer], li[kPer], ln[kPer], cnt = 0, len_sum = 0;
#pragma unroll
            for (int q = 0; q < kPer; ++q) {
                const int c = c0 + tid * kPer + q;
                ln[q] = 0;
                if (c >= ncols || tid * kPer + q >= kPMaxRanges) continue;
                const int cx = sx0 + c / ny, cy = wy0 + c % ny;
                const float xa = cx == 0 ? -INFINITY : (float)(G.lo[0] + cx) * G.cell;
                const float xb = cx == G.dim[0] - 1 ? INFINITY : (float)(G.lo[0] + cx + 1) * G.cell;
                const float ya = cy == 0 ? -INFINITY : (float)(G.lo[1] + cy) * G.cell;
                const float yb = cy == G.dim[1] - 1 ? INFINITY : (float)(G.lo[1] + cy + 1) * G.cell;
                const float gx = fmaxf(0.0f, fmaxf(xa - bb[3], bb[0] - xb) - margin);
                const float gy = fmaxf(0.0f, fmaxf(ya - bb[4], bb[1] - yb) - margin);
                const float rem = rq * rq - gx * gx - gy * gy;
                if (rem < 0.0f) continue;
                const float zr = sqrtf(rem) + margin;
                const int z0 = coord(bb[2] - zr, G.inv, G.lo[2], G.dim[2]);
                const int z1 = coord(bb[5] + zr, G.inv, G.lo[2], G.dim[2]);
                const int base = inst * G.ncl + (cx * G.dim[1] + cy) * G.dim[2];
                const int s = __ldg(G.start + base + z0), e = __ldg(G.start + base + z1 + 1);
                if (e <= s) continue;
                const int al = s - ((s - S_m) & (kPAlign - 1));
                const int ae = e + ((kPAlign - ((e - S_m) & (kPAlign - 1))) & (kPAlign - 1));
                ls[q] = al;
                li[q] = (s - al) | ((e - s) << 3);
                ln[q] = ae - al;
                ++cnt;
                len_sum += ae - al;
            }
            int m, tot;
            int off = block_exclusive_scan(cnt, sh.wtot, m);
            int loff = block_exclusive_scan(len_sum, sh.wtot, tot);
#pragma unroll
            for (int q = 0; q < kPer; ++q)
                if (ln[q] > 0) {
                    sh.rs[off] = ls[q];
                    sh.info[off] = li[q];
                    sh.pre[off] = loff;
                    loff += ln[q];
                    ++off;
                }
            if (tid == 0) sh.pre[m] = tot;
            __syncthreads();
            const int nchunks = (tot + kPN - 1) / kPN;
            if (tid == 0 && nchunks > 0) atomicAdd(&a.ctl->n_pchunks, nchunks);
            const bool crs = nchunks <= kPMaxChunks;  // else each candidate searches all ranges
            if (crs) {
                for (int c = tid; c < nchunks; c += kPThreads) {
                    const int u0 = c * kPN;
                    int lo = 0, hi = m - 1;
                    while (lo < hi) {
                        const int mid = (lo + hi + 1) >> 1;
                        if (sh.pre[mid] <= u0) lo = mid;
                        else hi = mid - 1;
                    }
                    sh.cr[c] = lo;
                }
                if (tid == 0) sh.cr[nchunks] = m - 1;
                __syncthreads();
            }
            if (warp >= kPMmaWarp + 1) {
                // ---- staging: candidate rows and volumes ----
                // thread st builds chunk positions st, st + 32 kPStageWarps, ...;
                // the candidates of chunk c + 1 are loaded while chunk c's
                // rows are built
                const int st = tid - 32 * (kPMmaWarp + 1);
                auto fetch = [&](int c, int t, float4& x) {
                    const int uu = c * kPN + t;
                    x = make_float4(0.f, 0.f, 0.f, 0.f);  // V = 0: padding and past the end
                    if (uu >= tot) return;
                    int lo = crs ? sh.cr[c] : 0, hi = crs ? sh.cr[c + 1] : m - 1;
                    while (lo < hi) {
                        const int mid = (lo + hi + 1) >> 1;
                        if (sh.pre[mid] <= uu) lo = mid;
                        else hi = mid - 1;
                    }
                    const int off2 = uu - sh.pre[lo];
                    const int inf = sh.info[lo];
                    const int pf = inf & (kPAlign - 1), len = inf >> 3;
                    if (off2 >= pf && off2 < pf + len) x = __ldg(a.f_posv + sh.rs[lo] + off2);
                };
                auto put = [&](int s, int t, const float4& x) {
                    // chunk position t (= slot offset mod 8 in its low bits) -> column:
                    // classes 0-3 fill columns 0-63, classes 4-7 columns 64-127
                    const int col = (t & 4) * 16 + (t >> 3) * 4 + (t & 3);
                    float v[24];
                    candidate_row((x.x - cxw) * a.inv_h, (x.y - cyw) * a.inv_h, (x.z - czw) * a.inv_h, v);
                    store_row(sh.B[s], col, v);
                    sh.V[s][col] = x.w;
                };
                constexpr int kPerT = kPN / kPStageThreads;  // candidates per staging thread and chunk
                float4 x[kPerT];
                if (nchunks > 0)
#pragma unroll
                    for (int q = 0; q < kPerT; ++q) fetch(0, st + q * kPStageThreads, x[q]);
                for (int c = 0; c < nchunks && !sh.abort_flag; ++c) {
                    const uint32_t gi = g + c, s = gi % kPStages, k = gi / kPStages;
                    if (k > 0 && !bwait(&sh.empty[s], (k - 1) & 1u, sh, a.ctl)) break;
                    float4 y[kPerT];
#pragma unroll
                    for (int q = 0; q < kPerT; ++q) y[q] = x[q];
                    if (c + 1 < nchunks)
#pragma unroll
                        for (int q = 0; q < kPerT; ++q) fetch(c + 1, st + q * kPStageThreads, x[q]);
#pragma unroll
                    for (int q = 0; q < kPerT; ++q) put(s, st + q * kPStageThreads, y[q]);
                    fence_proxy_async_smem();
                    __syncwarp();
                    if (lane == 0) mbar_arrive(&sh.full[s]);  // one arrival per staging warp
                }
            } else if (warp == kPMmaWarp) {
                // ---- MMA issue ----
                if (lane == 0)
                    for (int c = 0; c < nchunks && !sh.abort_flag; ++c) {
                        const uint32_t gi = g + c, s = gi % kPStages, k = gi / kPStages;
                        const uint32_t b = gi & 1u, kb = gi >> 1;
                        if (!bwait(&sh.full[s], k & 1u, sh, a.ctl)) break;
                        if (kb > 0 && !bwait(&sh.aempty[b], (kb - 1) & 1u, sh, a.ctl)) break;
                        umma::fence_after();
                        umma::mma_tile(tmem + b * kPN, sh.A, sh.B[s], kPK, idesc, false);
                        umma::commit(&sh.afull[b]);
                        umma::commit(&sh.empty[s]);
                        issued = true;
                    }
                __syncwarp();
            } else {
                // ---- epilogue: w(s) and the volume-weighted sums ----
                for (int c = 0; c < nchunks && !sh.abort_flag; ++c) {
                    const uint32_t gi = g + c, s = gi % kPStages, b = gi & 1u, kb = gi >> 1;
                    const bool ok = mbar_wait(&sh.afull[b], kb & 1u, kPPolls);
                    if (__any_sync(0xffffffffu, !ok)) {
                        if (lane == 0) {
                            sh.abort_flag = 1;
                            flag(a.ctl, SPHDEM_FLAG_TIMEOUT);
                        }
                        break;
                    }
                    umma::fence_after();
                    // this warp's half of the chunk, 32 columns per load; the
                    // other epilogue warps of the sub-partition hide each load
                    const int h0 = (warp >> 2) * (kPN / 2);
                    const uint32_t tcol = tmem + ((uint32_t)(32 * (warp & 3)) << 16) + b * kPN + h0;
                    {
                        // 16 columns per step, the load of the next 16 behind the arithmetic
                        const Kpk K{pk2(0.125f), pk2(-0.9375f), pk2(2.5f), pk2(-2.5f), pk2(1.0f)};
                        const uint32_t va = (uint32_t)__cvta_generic_to_shared(&sh.V[s][h0]);
                        unsigned long long u01, u23;
                        memcpy(&u01, &acc01, 8);
                        memcpy(&u23, &acc23, 8);
                        uint32_t r0[16], r1[16];
                        ld16(tcol, r0);
                        sums16_next(r0, va, tcol + 16, r1, u01, u23, K);
                        sums16_next(r1, va + 64, tcol + 32, r0, u01, u23, K);
                        sums16_next(r0, va + 128, tcol + 48, r1, u01, u23, K);
                        sums16(r1, va + 192, u01, u23, K);
                        memcpy(&acc01, &u01, 8);
                        memcpy(&acc23, &u23, 8);
                    }
                    umma::fence_before();
                    __syncwarp();
                    if (lane == 0) {
                        mbar_arrive(&sh.aempty[b]);
                        mbar_arrive(&sh.empty[s]);
                    }
                }
            }
            g += nchunks;
            __syncthreads();
        }
        // classes 4-7 (warps 4-7) are added to classes 0-3 (warps 0-3) of the same subject
        if (warp >= 4 && warp < kPEpiWarps) sh.hsum[tid - 128] = (acc01.x + acc01.y) + (acc23.x + acc23.y);
        __syncthreads();
        if (warp < 4 && tid < sh.tcount)
            a.part[(size_t)(sh.tstart + tid) * kPSlabs + sh.slab] =
                ((acc01.x + acc01.y) + (acc23.x + acc23.y)) + sh.hsum[tid];
    }
    // drain this CTA's MMAs, then free tensor memory
    __syncthreads();
    if (warp == kPMmaWarp) {
        if (lane == 0 && issued) {
            umma::commit(&sh.drain);
            if (!mbar_wait(&sh.drain, 0, kPPolls)) flag(a.ctl, SPHDEM_FLAG_TIMEOUT);
        }
        __syncwarp();
    }
    umma::fence_before();
    __syncthreads();
    if (warp == kPMmaWarp) {
        umma::fence_after();
        umma::tmem_dealloc(tmem, kPTmemCols);
    }
}

// ---------------------------------------------------------------------------
// slab partials -> normaliser -> solid fraction -> porosity
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_pfinish(PorArgs a) {
    pdl_wait();
    pdl_launch();
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= a.ctl->n_near) return;
    const int k = a.near_list[idx];
    const int o = a.gs.order[k];
    float f = 0.0f;
#pragma unroll
    for (int s = 0; s < kPSlabs; ++s) f += a.part[(size_t)idx * kPSlabs + s];
    const float flt = f * a.cw;
    const float4 p = a.f_posv[k];
    const int inst = a.gs.ncl > 0 ? a.gs.key[o] / a.gs.ncl : 0;
    float solid = 0.0f;
    const Win w = window(a.gd, p.x, p.y, p.z, a.rq);
    for_each_range(a.gd, w, inst, [&](int s, int e) {
        for (int j = s; j < e; ++j) {
            const int b = a.gd.order[j];
            const float3 pb = ld3(a.D.pos, b);
            const D2 r = d2_exact(p.x, p.y, p.z, pb.x, pb.y, pb.z);
            const float4 ab = a.aux[b];
            if (r.d2 < ab.z) {  // len < 2 h_b, :87-88
                const float q = fast_sqrt(r.d2) * ab.x;
                const float uu = 1.0f - 0.5f * q;
                const float u2 = uu * uu;
                const float wb = q < 2.0f ? ab.y * u2 * u2 * (1.0f + 2.0f * q) : 0.0f;
                solid += a.D.volume[b] * wb / (flt + 1.0e-20f);
            }
        }
    });
    a.P.porosity[o] = fminf(fmaxf(1.0f - solid, a.eps_min), a.eps_max);
}

// Frame-block lattice of the fluid grid (world-anchored), per axis.
void frame_lattice(const sphdem_grid_t& g, int F, int* f0, int* nf) {
    for (int d = 0; d < 3; ++d) {
        auto fdiv = [&](int x) { return x >= 0 ? x / F : -((-x + F - 1) / F); };
        f0[d] = fdiv(g.lo[d]);
        nf[d] = fdiv(g.lo[d] + g.dim[d] - 1) - f0[d] + 1;
    }
}

int smem_opt_in_porosity() {
    static std::mutex mu;
    static std::map<int, bool> done;
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lock(mu);
    if (done[dev]) return SPHDEM_OK;
    cudaError_t e = cudaFuncSetAttribute(k_porosity_mma, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kPSmemBytes);
    if (e != cudaSuccess) {
        set_error("porosity: shared memory opt-in", e);
        return SPHDEM_ERR_CUDA;
    }
    done[dev] = true;
    return SPHDEM_OK;
}

}  // namespace

int porosity_frame_edge(int frame) { return frame > 0 ? frame : 4; }

int64_t porosity_frames(const sphdem_grid_t& g, int F) {
    if (F <= 0 || g.ncell_local <= 0) return 0;
    int f0[3], nf[3];
    frame_lattice(g, F, f0, nf);
    return (int64_t)nf[0] * nf[1] * nf[2] * (g.ninst > 0 ? g.ninst : 1);
}

// Kernel attributes of the tensor-core porosity pass; called eagerly (outside
// any stream capture) before its first launch on a device.
int porosity_setup() { return smem_opt_in_porosity(); }

// The tensor-core porosity pass (uniform DEM h > 0) with the frame-block
// edge its scratch was sized for.  Returns SPHDEM_ERR_INVALID when the
// context lacks those buffers.
// part 0: the whole pass; 1: the near flags and tiles (k_pnear, k_plist: they
// read positions only, so they may run while the density pass runs); 2: the
// normaliser and the finish (after the density pass and part 1).
int run_porosity_mma(const sphdem_ctx_t* c, float support, float h, float eps_min, float eps_max, cudaStream_t st,
                     int part) {
    const int n = c->sph.n;
    if (n <= 0) return SPHDEM_OK;
    const sphdem_work_t& w = c->work;
    const int F = porosity_frame_edge(w.pframe);
    const int64_t nfb = porosity_frames(c->grid_sph, F);
    if (!w.pfb || !w.ptiles || !w.ppart || !w.pflag || nfb <= 0 || 2 * (nfb + 1) > w.pfb_words ||
        nfb > (1 << 30)) {
        set_error_msg("porosity (tensor cores): frame-block scratch missing or too small for the fluid grid");
        return SPHDEM_ERR_INVALID;
    }
    const int rc = porosity_setup();
    if (rc) return rc;
    PorArgs a;
    a.gs = make_geo(c->grid_sph);
    a.gd = make_geo(c->grid_dem);
    a.f_posm = (const float4*)w.f_posm;
    a.f_posv = (const float4*)w.f_posv;
    a.aux = (const float4*)w.dem_aux;
    a.P = c->sph;
    a.D = c->dem;
    a.near_list = w.near_list;
    a.flag = w.pflag;
    a.nfb = (int)nfb;
    a.cnt = w.pfb;
    a.fbl = w.pfb + (nfb + 1);
    a.tiles = (int4*)w.ptiles;
    a.part = w.ppart;
    a.ctl = c->ctl;
    a.rq = pad_radius(support);
    const Kern k = make_kern(h);
    a.inv_h = k.inv_h;
    a.cw = k.cw;
    a.eps_min = eps_min;
    a.eps_max = eps_max;
    a.F = F;
    frame_lattice(c->grid_sph, F, a.f0, a.nf);
    a.nfb_local = a.nf[0] * a.nf[1] * a.nf[2];
    // slab width: kPSlabs slabs cover any tile window (frame block + 2 rq + clamping slack)
    const float cell = c->grid_sph.cell > 0.0f ? c->grid_sph.cell : 1.0f;
    const int span = (int)ceilf(2.0f * a.rq / cell) + F + 3;
    a.Wx = (span + kPSlabs - 2) / (kPSlabs - 1);
    if (a.Wx < 1) a.Wx = 1;
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (part != 2) {
        // counters: listed particles, work units, tiles, listed frame blocks,
        // evaluated chunks (control words 6..10)
        cudaError_t e = zero_words(&c->ctl->n_near, 5, st);
        if (e == cudaSuccess) e = zero_words(a.cnt, nfb, st);
        if (e != cudaSuccess) {
            set_error("porosity memset", e);
            return SPHDEM_ERR_CUDA;
        }
        launch_pdl(k_pnear, blocks_for(n, 256), 256, 0, st, a);
        launch_pdl(k_plist, 8 * sms, 256, 0, st, a);
    }
    if (part != 1) {
        launch_pdl(k_porosity_mma, 2 * sms, kPThreads, kPSmemBytes, st, a);
        launch_pdl(k_pfinish, blocks_for(n, 256), 256, 0, st, a);
    }
    return launch_status("porosity (tensor cores)");
}

}  // namespace sd
