/* sphdem_mpnn.h -- learned K-step surrogate of the WCSPH-DEM step: a small
 * message-passing network over the radius graph of all particles, with BF16
 * tensor-core (tcgen05) forward and backward kernels and FP32 accumulation.
 *
 * No counterpart in the reference (hojin9908/Warp_SPH_GPT has no learned
 * component): these entry points sit beside the plain step of sphdem.h, which
 * stays the surrogate's fallback and the judge of its density error.
 *
 * Network (per particle node i, edges j -> i for |x_j - x_i| < R, j != i):
 *   edge filter  f_ij = E2 relu(E1 e_ij + b_E1) + b_E2          (7 -> 128 -> 128)
 *   h0  = silu(N1 x_i + b_N1)                                   (16 -> 128)
 *   h1  = h0 + s * sum_j f_ij (.) h0_j   (receivers; others h1 = h0)
 *   h2  = silu(N2 h1 + b_N2)                                    (128 -> 128)
 *   h3  = h2 + s * sum_j f_ij (.) h2_j   (receivers)
 *   out = N3 h3 + b_N3                                          (128 -> 6)
 * e_ij = ((x_j - x_i)/R, |x_j - x_i|/R, (v_j - v_i)/v_s), zero-padded to 16;
 * s = 1 / aggregation normaliser.  Weights are stored [out][in] (row-major,
 * FP32 master copy `theta`); the kernels read BF16 images of them.
 *
 * Nodes are ordered fluid, DEM, wall, DEM wall; receivers (moving particles)
 * are nodes [0, n_recv).  All buffers are caller-owned device memory; every
 * call is asynchronous on `stream` and returns 0, SPHDEM_ERR_INVALID or
 * SPHDEM_ERR_CUDA (message: sphdem_last_error()).  Device conditions set
 * SPHDEM_FLAG_* bits in *status (edge capacity: SPHDEM_FLAG_ROW_OVERFLOW; a
 * bounded tensor-core wait giving up: SPHDEM_FLAG_TIMEOUT).
 */
#ifndef SPHDEM_MPNN_H
#define SPHDEM_MPNN_H

#include <stdint.h>

#include "sphdem.h"

#ifdef __cplusplus
extern "C" {
#endif

#define SPHDEM_MPNN_HIDDEN  128
#define SPHDEM_MPNN_NODE_IN 16
#define SPHDEM_MPNN_EDGE_IN 16 /* 7 used */
#define SPHDEM_MPNN_OUT     16 /* 6 used: dx, dy, dz, dvx, dvy, dvz */

/* FP32 parameter vector theta: offsets (floats) of each block. */
#define SPHDEM_MPNN_E1_W   0     /* [128][16]  */
#define SPHDEM_MPNN_E1_B   2048  /* [128]      */
#define SPHDEM_MPNN_E2_W   2176  /* [128][128] */
#define SPHDEM_MPNN_E2_B   18560 /* [128]      */
#define SPHDEM_MPNN_N1_W   18688 /* [128][16]  */
#define SPHDEM_MPNN_N1_B   20736 /* [128]      */
#define SPHDEM_MPNN_N2_W   20864 /* [128][128] */
#define SPHDEM_MPNN_N2_B   37248 /* [128]      */
#define SPHDEM_MPNN_N3_W   37376 /* [16][128]  rows 6..15 stay zero */
#define SPHDEM_MPNN_N3_B   39424 /* [16]       */
#define SPHDEM_MPNN_NPARAM 39440

/* BF16 operand images (uint16 halves): shared-memory tile layout, loaded by
 * bulk copy.  Written by sphdem_mpnn_pack. */
#define SPHDEM_MPNN_PACKED 73728

/* Node inputs from the four particle sets (reference field layout). */
typedef struct sphdem_mpnn_nodes {
    const float* f_pos; const float* f_vel; const float* f_acc; const float* f_rho; const float* f_por;
    int32_t n_fluid;
    const float* d_pos; const float* d_vel; const float* d_acc; const float* d_rad;
    int32_t n_dem;
    const float* b_pos; const float* b_rho;
    int32_t n_wall;
    const float* w_pos; const float* w_rad;
    int32_t n_dem_wall;
    float rho0, inv_vscale, inv_ascale, inv_radius;
    float* node_pos3;  /* [n,3] out: positions (grid build)            */
    float* node_pos4;  /* [n,4] out: x, y, z, 0                          */
    float* node_vel4;  /* [n,4] out: vx, vy, vz, 0                       */
    uint16_t* x;       /* [n,16] out: BF16 node inputs                   */
} sphdem_mpnn_nodes_t;

/* Radius graph and network state of one forward pass. */
typedef struct sphdem_mpnn_net {
    int32_t n_nodes, n_recv, edge_capacity, pad0;
    float inv_radius, inv_vscale, inv_norm, pad1;
    const float* node_pos4;   /* [n_nodes,4]                                  */
    const float* node_vel4;   /* [n_nodes,4]                                  */
    const uint16_t* x;        /* [n_nodes,16] BF16                            */
    int32_t* offset;          /* [n_recv+1] edges by receiver (CSR)           */
    int32_t* sender;          /* [edge_capacity]                              */
    int32_t* receiver;        /* [edge_capacity]                              */
    const float* theta;       /* [SPHDEM_MPNN_NPARAM] FP32 (biases)           */
    const uint16_t* packed;   /* [SPHDEM_MPNN_PACKED] BF16 weight images      */
    float* z0;  uint16_t* h0; /* [n_nodes,128] pre-activation FP32, BF16      */
    float* agg;               /* [n_recv,128] FP32 aggregation scratch        */
    uint16_t* h1;             /* [n_nodes,128]                                */
    float* z2;  uint16_t* h2; /* [n_nodes,128]                                */
    uint16_t* h3;             /* [n_recv,128]                                 */
    float* out;               /* [n_recv,16] FP32                             */
    int32_t* status;          /* device word, OR of SPHDEM_FLAG_* bits        */
    /* optional (inference): the node layers then run on the receivers and on
     * the non-receiver nodes that send an edge of the current graph only --
     * the others' latent rows are never read (NULL: every node) */
    int32_t* active;          /* [n_nodes] scratch flags                      */
    int32_t* active_list;     /* [1 + n_nodes - n_recv]: count, then nodes    */
} sphdem_mpnn_net_t;

/* Backward workspace. */
typedef struct sphdem_mpnn_grad {
    const float* d_out;       /* [n_recv,16] dL/d out                         */
    float* g2;                /* [n_recv,128]                                 */
    float* d_h2;              /* [n_nodes,128]                                */
    float* d_h1;              /* [n_nodes,128]                                */
    float* d_h0;              /* [n_nodes,128]                                */
    uint16_t* bf_a;           /* [n_nodes,128] BF16 scratch                   */
    uint16_t* bf_b;           /* [n_recv,16]   BF16 scratch                   */
    float* partial;           /* [sphdem_mpnn_partial_floats()] per-CTA sums  */
    float* grad;              /* [SPHDEM_MPNN_NPARAM] out (overwritten)       */
} sphdem_mpnn_grad_t;

/* Floats of per-CTA partial-sum scratch the backward pass needs. */
int64_t sphdem_mpnn_partial_floats(void);

/* theta (FP32) -> BF16 operand images. */
int sphdem_mpnn_pack(const float* theta, uint16_t* packed, sphdem_stream_t stream);

/* Node positions, velocities and BF16 inputs from the particle sets. */
int sphdem_mpnn_nodes(const sphdem_mpnn_nodes_t* in, sphdem_stream_t stream);

/* Radius graph over the nodes: bins node_pos3 in `grid` (cell >= radius, n =
 * n_nodes, caller-owned buffers as for sphdem_grid_build), then lists for
 * every receiver its senders j != i with |x_j - x_i|^2 < radius^2 in
 * cell-traversal order.  scan_scratch: sphdem_scan_scratch(n_recv) words.  offset[n_recv] = edges found; if that exceeds
 * edge_capacity, SPHDEM_FLAG_ROW_OVERFLOW is set and the list is cut. */
int sphdem_mpnn_graph(sphdem_grid_t* grid, const float* node_pos3, const float* node_pos4, int32_t n_recv,
                      float radius, int32_t* offset, int32_t* sender, int32_t* receiver, int32_t edge_capacity,
                      int32_t* scan_scratch, sphdem_ctl_t* ctl, sphdem_stream_t stream);

/* Forward pass: out = network(graph).  store_pre != 0 keeps z0, z2 for the
 * backward pass. */
int sphdem_mpnn_forward(const sphdem_mpnn_net_t* net, int store_pre, sphdem_stream_t stream);

/* Backward pass after a forward with store_pre: grad = dL/dtheta. */
int sphdem_mpnn_backward(const sphdem_mpnn_net_t* net, const sphdem_mpnn_grad_t* g, sphdem_stream_t stream);

/* Mean squared error over the 6 outputs of n rows: *loss (device), d_out. */
int sphdem_mpnn_loss(const float* out, const float* target, int32_t n, float* loss, float* d_out,
                     sphdem_stream_t stream);

/* Adds lambda / E * sum over the graph's edges (i <- j) of |dx_i - dx_j|^2,
 * dx = out[:, 0:3] - target[:, 0:3] (dx_j = 0 for senders that are not
 * receivers), to *loss and its gradient to d_out: relative displacement
 * errors between neighbours are what changes their SPH density. */
int sphdem_mpnn_edge_loss(const int32_t* offset, const int32_t* sender, const int32_t* receiver, int32_t n_recv,
                          int32_t edge_capacity, const float* out, const float* target, float lambda, float* loss,
                          float* d_out, sphdem_stream_t stream);

/* One Adam step (bias-corrected, step >= 1) on n parameters. */
int sphdem_mpnn_adam(float* theta, const float* grad, float* m, float* v, int32_t n, float lr, float beta1,
                     float beta2, float eps, int32_t step, sphdem_stream_t stream);

/* Jump of m substeps for fluid and DEM (node order), prior plus scaled output:
 *   x += m dt v + dt^2 a m(m+1)/2 + s_x out[0:3];  v += m dt a + s_v out[3:6]
 * (the prior is m symplectic-Euler substeps at constant acceleration a).
 * scale4 (HOST array) = {s_x fluid, s_v fluid, s_x DEM, s_v DEM}.  With target != NULL the
 * state is left alone and target = (x_T, v_T) written as normalised residual
 * rows instead (x_T, v_T: [n_fluid + n_dem, 3] positions/velocities m
 * substeps later). */
int sphdem_mpnn_apply(float* f_pos, float* f_vel, const float* f_acc, int32_t n_fluid, float* d_pos, float* d_vel,
                      const float* d_acc, int32_t n_dem, const float* out, int32_t m, float dt,
                      const float* scale4, const float* x_t, const float* v_t, float* target,
                      sphdem_stream_t stream);

/* max_i |a_i - b_i| * inv over n floats (b == NULL: b_i = ref) into *out
 * (device, FP32, >= 0; must start at 0). */
int sphdem_mpnn_maxdev(const float* a, const float* b, float ref, int32_t n, float inv, float* out,
                       sphdem_stream_t stream);

/* One learned jump, replayed from a CUDA graph per Shepard variant:
 *   1. the loop body of sphdem_run for `step` (moving grids + coupled step);
 *   2. backup of fluid/DEM positions and velocities and the fluid density
 *      into `keep`;
 *   3. node inputs, radius graph, forward pass, prior + correction of
 *      `substeps` steps applied in place (sphdem_mpnn_apply);
 *   4. the judge: fluid grid rebuilt and the filtered fluid density
 *      evaluated at the new positions (the density pass of the plain step),
 *      dev[0] = max_i |rho_new - rho_old| / rho0 (judge 0) or
 *      max_i |rho_new - rho0| / rho0 (judge 1); and the position term
 *      dev[1] = max_i |s_x out_x,i| + m dt |s_v out_v,i|, how far the
 *      network's correction moves a particle beyond the constant-acceleration
 *      prior, or will have moved it one jump later through its velocity [m].
 * The caller reads dev (and net.status) and, above its tolerances, calls
 * sphdem_jump_undo and runs the substeps with sphdem_run.  The plain step of
 * 1. flips the DEM contact CSR parity once. */
typedef struct sphdem_jump {
    sphdem_mpnn_nodes_t nodes;  /* node inputs; the fluid/DEM/wall pointers are the context's */
    sphdem_mpnn_net_t net;      /* network state; net.status points into graph_ctl */
    sphdem_grid_t node_grid;    /* grid over nodes.node_pos3, cell >= radius */
    int32_t* scan_scratch;      /* sphdem_scan_scratch(n_recv) words */
    sphdem_ctl_t* graph_ctl;    /* device control block of the node grid and kernels */
    float radius;
    int32_t substeps;
    float scale[4];             /* output scales, as sphdem_mpnn_apply's scale4 */
    float* keep;                /* [6 n_fluid + 6 n_dem + n_fluid] backup */
    float* dev;                 /* [2] judge values (device): [0] the density term below,
                                   [1] the largest correction displacement: max over
                                   particles of |s_x out_x| + m dt |s_v out_v| [m] */
    int32_t judge;              /* 0: max |rho_new - rho_old| / rho0 (change over the jump);
                                   1: max |rho_new - rho0| / rho0 (density deviation) */
    float pos_tol;              /* > 0: a jump whose dev[1] exceeds it [m] falls back too */
} sphdem_jump_t;

/* flags bit 0 (SPHDEM_JUMP_GRID_FRESH): the fluid grid is current -- the last
 * call on this context was a jump the caller accepted and nothing has moved
 * the fluid since (its judge re-binned the fluid at these positions) -- so
 * the plain step skips that re-bin (same grid, same results). */
#define SPHDEM_JUMP_GRID_FRESH 1
int sphdem_jump(sphdem_ctx_t* ctx, const sphdem_params_t* p, const sphdem_jump_t* j, int step, int32_t flags,
                sphdem_stream_t stream);

/* Kernel nodes of the jump's captured graph (variant bit 0: Shepard step, bit
 * 1: SPHDEM_JUMP_GRID_FRESH), or -1 if that variant has not been captured. */
int sphdem_jump_kernels(sphdem_ctx_t* ctx, int variant);

/* Restore positions, velocities and fluid density saved by the last jump. */
int sphdem_jump_undo(sphdem_ctx_t* ctx, const sphdem_jump_t* j, sphdem_stream_t stream);

/* n_jumps jumps from first_step, judged on the device: each is the jump's
 * graph plus a judge that, when j->dev[0] > tol, or j->pos_tol > 0 and
 * j->dev[1] > j->pos_tol (or a graph/kernel flag is
 * set), runs the fallback in a conditional graph node -- undo, the m
 * substeps as plain steps, a fluid re-bin -- so the host launches the jumps
 * back to back and reads the outcome once.  stats (device int32[6], the
 * caller zeroes it): jumps, fallbacks, largest accepted density judge value
 * (float bits), 1 if the last jump fell back, largest accepted position term
 * (float bits), unused.  Every jump runs 1 plain step (plus m
 * for a fallback): the DEM CSR parity flips that many times.  flags as for
 * sphdem_jump.  Needs one eager sphdem_jump on the context first (kernel
 * attributes are set there); 1 <= substeps <= 29. */
int sphdem_rollout(sphdem_ctx_t* ctx, const sphdem_params_t* p, const sphdem_jump_t* j, int first_step,
                   int n_jumps, float tol, int32_t flags, int32_t* stats, sphdem_stream_t stream);

/* Kernel nodes the rollout graphs of those jumps hold: of the jumps
 * themselves (body = 0) or of their fallback bodies (body = 1); -1 if a graph
 * has not been captured. */
int64_t sphdem_rollout_kernels(sphdem_ctx_t* ctx, int first_step, int n_jumps, int32_t flags, int body);

/* Tensor-core GEMM check: C[M,N] (FP32) = A[M,K] B[N,K]^T for BF16 row-major
 * A, B; K, N in {16, 128}. */
int sphdem_mpnn_gemm(const uint16_t* a, const uint16_t* b, float* c, int32_t m, int32_t n, int32_t k,
                     int32_t* status, sphdem_stream_t stream);

/* Weight-gradient GEMM check: C[128,N] = sum_r P[r,:]^T Q[r,:] for BF16
 * row-major P [rows,128], Q [rows,N]; N in {16, 128}. */
int sphdem_mpnn_wgrad(const uint16_t* p, const uint16_t* q, float* c, int32_t rows, int32_t n, float* partial,
                      int32_t* status, sphdem_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* SPHDEM_MPNN_H */
