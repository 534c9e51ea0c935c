/*
 * sphdem.h -- C ABI of libsphdem.so, the GB300 (sm_103a) implementation of the
 * 3D WCSPH-DEM time step of hojin9908/Warp_SPH_GPT.
 *
 * Ownership: every pointer in these structs is a DEVICE pointer owned by the
 * caller (the Python layer allocates and frees all tensors, including scratch,
 * CSR capacity and the control block).  The library never allocates device
 * memory, never frees it and never synchronises the host, except inside the
 * explicitly blocking helpers documented as such.
 *
 * Threading: every entry point enqueues work on the given stream and returns
 * at once.  Calls on one context are not re-entrant; different contexts on
 * different streams are independent.
 *
 * Layout: the four particle structs restate the reference's Warp structs
 * field by field (input/struct.py:3-104).  Scalar fields are float[n]; vec3
 * fields are float[n*3] packed x,y,z (byte-identical to a Warp vec3 array and
 * to a contiguous torch [n,3] float32 tensor).  CSR index fields are int32.
 *
 * Status: functions return SPHDEM_OK (0), a positive recoverable code, or a
 * negative code for a CUDA launch/configuration error.  Device-side
 * conditions (CSR capacity overflow, non-finite positions) are OR-ed into
 * sphdem_ctl_t.status as SPHDEM_FLAG_* bits and read by the host when it
 * chooses to synchronise.
 *
 * Every struct here is plain data: the same header is compiled by nvcc (the
 * library), by gcc (the CPU oracle used by the tests) and mirrored by ctypes.
 */
#ifndef SPHDEM_H
#define SPHDEM_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SPHDEM_ABI_VERSION 11

/* work.nbr forms (params.nbr_format): int32 member slots, or walk masks. */
#define SPHDEM_NBR_SLOTS 0
#define SPHDEM_NBR_MASKS 1

/* ---- return codes ---------------------------------------------------- */
#define SPHDEM_OK                0
#define SPHDEM_ERR_INVALID       2   /* bad size, NULL pointer or geometry        */
#define SPHDEM_ERR_CSR_CAPACITY  3   /* contact capacity would overflow (host check) */
#define SPHDEM_ERR_CUDA         -1   /* a CUDA call failed; see sphdem_last_error */

/* ---- device status bits (sphdem_ctl_t.status) ------------------------- */
#define SPHDEM_FLAG_CSR_DEM_OVERFLOW  0x1  /* DEM-DEM directed contacts > capacity  */
#define SPHDEM_FLAG_CSR_BND_OVERFLOW  0x2  /* DEM-wall directed contacts > capacity */
#define SPHDEM_FLAG_NONFINITE         0x4  /* a binned position was NaN/Inf         */
#define SPHDEM_FLAG_ROW_OVERFLOW      0x8  /* one contact row exceeded the per-row
                                              sort buffer (rows still complete)     */
#define SPHDEM_FLAG_TIMEOUT          0x10  /* a bounded wait on a shared-memory copy
                                              gave up; that kernel's results are void */

/* Opaque CUDA stream handle (cudaStream_t); 0 is the legacy default stream. */
typedef void* sphdem_stream_t;

/* Fluid particles.  Reference: SPHptl, input/struct.py:3-21. */
typedef struct sphdem_sph {
    float* pos;       /* [n,3] position [m]                                  */
    float* vel;       /* [n,3] velocity [m/s]                                */
    float* rho_raw;   /* [n]   initial density (never updated by the step)   */
    float* rho;       /* [n]   Shepard-filtered density [kg/m^3]             */
    float* pres;      /* [n]   pressure [Pa]                                 */
    float* acc;       /* [n,3] acceleration [m/s^2]                          */
    float* m;         /* [n]   mass [kg]                                     */
    float* flt;       /* [n]   Shepard filter                                */
    float* porosity;  /* [n]   fluid fraction                                */
    float* pgf;       /* [n,3] negative pressure gradient [Pa/m]             */
    float* acc_dem;   /* [n,3] DEM drag reaction acceleration [m/s^2]        */
    int32_t n;
} sphdem_sph_t;

/* Dummy wall particles.  Reference: BNDptl, input/struct.py:23-36. */
typedef struct sphdem_bnd {
    float* pos;
    float* vel;
    float* rho_raw;
    float* rho;
    float* pres;
    float* acc;
    float* m;
    int32_t n;
} sphdem_bnd_t;

/* One side of a compact contact-history CSR.  Reference: the *_old / *_new
 * field triples of DEMptl (input/struct.py:65-78).  The reference reallocates
 * id/tang to the exact edge count E every step (source/Simulation.py:157-160);
 * here they are fixed-capacity buffers and the logical length is offset[n]. */
typedef struct sphdem_csr {
    int32_t* offset;  /* [n_dem+1] row offsets; offset[n_dem] = E             */
    int32_t* id;      /* [capacity] stable neighbour index, ascending per row */
    float*   tang;    /* [capacity,3] tangential spring displacement [m]      */
    double*  tang64;  /* [capacity,3] FP64 accumulator behind tang, or NULL   */
    int64_t  capacity;
} sphdem_csr_t;

/* Moving DEM spheres.  Reference: DEMptl, input/struct.py:39-82.  The two
 * CSR sides of each contact kind are addressed by index; the index of the
 * readable ("old") side lives in the device control block. */
typedef struct sphdem_dem {
    float* pos;
    float* vel;
    float* acc;
    float* force;
    float* omega;
    float* torque;
    float* radius;
    float* rho;
    float* m;
    float* volume;
    float* inertia;
    float* K;
    float* eta;
    float* mu;
    float* h;
    sphdem_csr_t csr_dem[2];   /* DEM-DEM history, sides 0/1            */
    sphdem_csr_t csr_bnd[2];   /* DEM-wall-sphere history, sides 0/1    */
    float* flt_s;
    float* porosity;
    float* drag;
    float* pressure_force;
    int32_t n;
} sphdem_dem_t;

/* Fixed DEM wall spheres.  Reference: DEMBNDptl, input/struct.py:85-104. */
typedef struct sphdem_dembnd {
    float* pos;
    float* vel;
    float* omega;
    float* radius;
    float* rho;
    float* m;
    float* volume;
    float* inertia;
    float* K;
    float* eta;
    float* mu;
    int32_t n;
} sphdem_dembnd_t;

/* Dense cell grid that replaces wp.HashGrid (main.py:117-122).  The lattice is
 * anchored at the world origin (a point's world cell is floor(x*inv_cell)), so
 * grids of equal cell width agree on cells whatever their extent; the box is
 * [lo, lo+dim) in world cells and clamped at its faces, so points outside it
 * land in the face cells and no neighbour is ever missed.  Several
 * independent instances (batched dam breaks) share one geometry: a point's
 * cell key is inst*ncell_local + (cx*dim_y + cy)*dim_z + cz. */
typedef struct sphdem_grid {
    int32_t lo[3];         /* world cell index floor(x*inv_cell) of local cell 0 */
    float   cell;          /* cell width [m]                                 */
    float   inv_cell;      /* 1/cell (FP32); binning is floor(x*inv_cell)    */
    int32_t dim[3];        /* cells per axis                                 */
    int32_t ncell_local;   /* dim[0]*dim[1]*dim[2]                           */
    int32_t ninst;         /* number of instances (1 for one dam break)      */
    int32_t n;             /* number of binned points                        */
    int32_t* cell_start;   /* [ninst*ncell_local+1] exclusive offsets        */
    int32_t* order;        /* [n] sorted slot -> point index                 */
    int32_t* key;          /* [n] cell key of each point (by point index)    */
    int32_t* cursor;       /* [ninst*ncell_local] scatter scratch            */
    int32_t* block_sums;   /* [sphdem_scan_scratch(ncell)] scan scratch      */
    const int32_t* inst;   /* [n] instance of each point, or NULL (all 0)    */
} sphdem_grid_t;

/* Device control block: 16 int32 words in device memory. */
typedef struct sphdem_ctl {
    int32_t step;       /* step counter used by graph replay                    */
    int32_t old_dem;    /* index (0/1) of the readable DEM-DEM CSR side          */
    int32_t old_bnd;    /* index (0/1) of the readable DEM-wall CSR side         */
    int32_t status;     /* OR of SPHDEM_FLAG_* bits                              */
    int32_t e_dem;      /* directed DEM-DEM contacts of the last rebuild        */
    int32_t e_bnd;      /* directed DEM-wall contacts of the last rebuild       */
    int32_t n_near;     /* fluid particles with a DEM inside its coupling reach */
    int32_t near_next;  /* next near-list entry (or porosity work unit) to hand out */
    int32_t n_ptiles;   /* subject tiles of the tensor-core porosity pass        */
    int32_t n_pfb;      /* frame blocks with listed particles (same pass)        */
    int32_t n_pchunks;  /* 128 x 128 pair chunks the same pass evaluated          */
    int32_t pad[5];
} sphdem_ctl_t;

/* Sorted working copies (all device, all [n] in the order of their grid).
 * Neighbour loops read these instead of the reference-layout fields. */
typedef struct sphdem_work {
    /* fluid, in grid_sph order */
    float* f_posm;      /* [n_sph,4] x, y, z, m                                */
    float* f_vel;       /* [n_sph,4] vx, vy, vz, 0                             */
    float* f_rp;        /* [n_sph,4] rho, pres, pres/rho^2, 1/rho (this step)  */
    float* f_vprev;     /* [n_sph]   m/rho before this step's density pass     */
    float* f_posv;      /* [n_sph,4] x, y, z, m/rho (this step)                */
    float* f_pgf;       /* [n_sph,4] pgf x, y, z, rho (this step)              */
    int32_t* near_list; /* [n_sph]   fluid slots with a DEM within reach       */
    /* dummy wall, in grid_bnd order */
    float* b_posm;      /* [n_bnd,4] x, y, z, m                                */
    float* b_vel;       /* [n_bnd,4]                                           */
    float* b_rp;        /* [n_bnd,4] rho, pres, pres/rho^2, 1/rho              */
    float* b_vprev;     /* [n_bnd]   m/rho before this step's density pass     */
    float* b_self;      /* [n_bnd]   wall-only density sum (cached at build)   */
    /* DEM scratch, point order */
    int32_t* dem_count; /* [2*(n_dem+1)] per-row contact counts               */
    float* dem_aux;     /* [n_dem,4] 1/h, 21/(16 pi h^3), sqrt bound of 2h, 2h  */
    /* fluid, in grid_sph order, uniform DEM h only */
    float* f_posq;      /* [n_sph,4] x/h, y/h, z/h, m/rho (porosity sums)     */
    /* fluid neighbour records written by the density pass and read by the
     * force pass of the same step, particles in grid_sph order, rows of n_sph
     * words (particles contiguous within a row, so a warp's accesses
     * coalesce); rows [0, cap) fluid, rows [cap, 2 cap) wall, rows 2 cap and
     * 2 cap + 1 the fluid and wall counts.  params.nbr_format chooses the form:
     *   SPHDEM_NBR_SLOTS: row t holds member t's slot (d2 < support^2, walk
     *     order); counts = members (above cap: that particle's force pass walks
     *     its cells);
     *   SPHDEM_NBR_MASKS: one bit per slot the density pass walks (its
     *     ball-trimmed cell ranges in walk order), set for a member, 32-bit
     *     word w in row w; counts = slots walked (above 32 cap: walks).
     * cap = params.nbr_cap; NULL or cap 0: none, both passes walk. */
    int32_t* nbr;       /* [(2*cap+2), n_sph]                                  */
    /* scratch of the tensor-core porosity pass (porosity_variant 2); sizes from
     * sphdem_porosity_scratch.  NULL: that variant is unavailable. */
    int32_t* pfb;       /* [pfb_words] per frame block listed count, then the list of
                           frame blocks that have listed particles        */
    int32_t* ptiles;    /* [4*(n_sph+1)] subject tiles (near start, count, frame block) */
    float*   ppart;     /* [n_sph*SPHDEM_POROSITY_SLABS] per-slab partial normalisers */
    int32_t* pflag;     /* [n_sph] listed flag per fluid slot                  */
    int64_t  pfb_words; /* capacity of pfb in int32 words                      */
    int32_t  pframe;    /* frame-block edge in fluid cells the scratch is sized for */
    int32_t  pad_work;
} sphdem_work_t;

/* Solver controls.  Reference: Solv (input/Config.py:11-49 with the SPH-DEM
 * overrides of input/Config_SPH_DEM.py:6-15) plus the search scales of
 * dem_search_scales (input/input_reader.py:163-168). */
typedef struct sphdem_params {
    float h;                 /* SPH smoothing length [m]                      */
    float support;           /* 2*h                                           */
    float rho0;
    float c0;
    float gamma;
    float mu;                /* dynamic viscosity [Pa s]                      */
    float g;                 /* gravity magnitude along -z [m/s^2]            */
    float dt;
    int32_t shepard_step;
    float porosity_min;
    float porosity_max;
    float radius_max;        /* largest moving DEM radius                     */
    float boundary_radius_max;
    float h_max;             /* largest DEM coupling h                        */
    float h_uniform;         /* common DEM h, or 0 if heterogeneous           */
    /* launch tuning (neighbour sets unchanged; sums may change only by FP32
     * summation order): threads per block of the fluid and wall neighbour
     * loops (64, 128 or 256; 0 = 128), the porosity normaliser implementation
     * (0 = direct loads, one warp per particle; 1 = shared-memory staged with
     * TMA bulk copies, single-instance grids; 2 = pair distances on the tensor
     * cores, uniform DEM h, needs the work.p* scratch), and the lanes per subject of
     * the density, wall-density and force loops (0/1 = one thread per
     * particle; 32 = one warp per particle, for small systems). */
    int32_t block_sph;
    int32_t porosity_variant;
    int32_t lanes_sph;
    int32_t nbr_cap;         /* per particle and kind: slots (SPHDEM_NBR_SLOTS) or
                                mask words (SPHDEM_NBR_MASKS) of work.nbr       */
    int32_t nbr_format;      /* SPHDEM_NBR_SLOTS or SPHDEM_NBR_MASKS               */
} sphdem_params_t;

/* Everything one step touches. */
typedef struct sphdem_ctx {
    sphdem_sph_t    sph;
    sphdem_bnd_t    bnd;
    sphdem_dem_t    dem;
    sphdem_dembnd_t dembnd;
    sphdem_grid_t   grid_sph;
    sphdem_grid_t   grid_bnd;
    sphdem_grid_t   grid_dem;
    sphdem_grid_t   grid_dembnd;
    sphdem_work_t   work;
    sphdem_ctl_t*   ctl;     /* device control block                      */
} sphdem_ctx_t;

/* ---- library ---------------------------------------------------------- */
int         sphdem_abi_version(void);
const char* sphdem_last_error(void);
/* int32 words of scan scratch a grid with ncell cells needs. */
int64_t     sphdem_scan_scratch(int64_t ncell);
/* sizeof of the ABI structs, in declaration order (sph, bnd, csr, dem,
 * dembnd, grid, ctl, work, params, ctx), for bindings to check their mirrors;
 * writes min(n, count) values and returns the count. */
int         sphdem_struct_sizes(int64_t* out, int n);

/* Work units of the tensor-core porosity pass per subject tile: world-anchored
 * column slabs, whose partial normalisers are summed in slab order. */
#define SPHDEM_POROSITY_SLABS 8
/* Scratch sizes of the tensor-core porosity pass for ctx's fluid grid
 * geometry (grid_sph set) and a frame-block edge of `frame` cells (the tiles'
 * centres are the centres of world-anchored blocks of frame^3 cells):
 * out[0] int32 words of pfb, out[1] int32 words of ptiles, out[2] floats of
 * ppart, out[3] int32 words of pflag.  Returns 0, or SPHDEM_ERR_INVALID. */
int sphdem_porosity_scratch(const sphdem_ctx_t* ctx, int frame, int64_t* out);

/* ---- neighbour grid ---------------------------------------------------
 * Replaces wp.HashGrid.build(points, radius) (called at main.py:66,73,85,87).
 * Bins n points (float[n*3]) of one particle kind into g (stable: points of a
 * cell are ordered by index), then refreshes the sorted copies that kind's
 * neighbour loops read.  kind: 0 fluid, 1 dummy wall, 2 moving DEM, 3 DEM wall.
 * For kind 1 the cached wall-only density sum is recomputed as well. */
int sphdem_grid_build(sphdem_ctx_t* ctx, int kind, const sphdem_params_t* p,
                      sphdem_stream_t stream);

/* Re-gathers the sorted fluid and wall copies from the reference-layout
 * fields (after the caller edited a field outside a step). */
int sphdem_refresh_sorted(sphdem_ctx_t* ctx, sphdem_stream_t stream);

/* ---- whole steps -------------------------------------------------------- */
/* SPH_OneStep (source/Simulation.py:17-99).  step < 0 reads ctl->step. */
int sphdem_sph_onestep(sphdem_ctx_t* ctx, const sphdem_params_t* p, int step,
                       int integrate, sphdem_stream_t stream);
/* SPHDEM_OneStep (source/Simulation.py:102-221), grids already built.
 * step < 0 reads ctl->step (graph replay). */
int sphdem_sphdem_onestep(sphdem_ctx_t* ctx, const sphdem_params_t* p, int step,
                          sphdem_stream_t stream);
/* run_forward's inner loop (main.py:84-91) for n_steps steps starting at
 * first_step: rebuild the moving grids, then one step, captured once into a
 * CUDA graph per context and replayed.  coupled=0 runs SPH_OneStep. */
int sphdem_run(sphdem_ctx_t* ctx, const sphdem_params_t* p, int first_step,
               int n_steps, int coupled, sphdem_stream_t stream);
/* Releases the CUDA graph held for ctx (host-side object only). */
int sphdem_release(sphdem_ctx_t* ctx);
/* Kernel nodes of the captured loop-body graph of ctx (variant 1: a Shepard
 * step, 0: any other step), or -1 if sphdem_run has not captured it. */
int sphdem_graph_kernels(sphdem_ctx_t* ctx, int variant);
/* Phases of one loop body, in launch order (for sphdem_profile_step). */
#define SPHDEM_PHASE_GRID_SPH   0   /* fluid grid build + sorted gather          */
#define SPHDEM_PHASE_GRID_DEM   1   /* DEM grid build                            */
#define SPHDEM_PHASE_DENSITY    2   /* [Shepard +] fluid density + Tait          */
#define SPHDEM_PHASE_WALL       3   /* wall density + Tait                       */
#define SPHDEM_PHASE_FORCE      4   /* fluid force (+ -grad p)                   */
#define SPHDEM_PHASE_CONTACTS   5   /* DEM-DEM and DEM-wall CSR rebuild + loads  */
#define SPHDEM_PHASE_POROSITY   6   /* porosity                                  */
#define SPHDEM_PHASE_EXCHANGE   7   /* fluid -> DEM pressure force and drag      */
#define SPHDEM_PHASE_REACT      8   /* drag reaction + fluid integration         */
#define SPHDEM_PHASE_DEM_STEP   9   /* DEM integration                           */
#define SPHDEM_PHASE_COUNT     10
/* BLOCKING: one loop body (moving grids rebuilt, one step) with a CUDA event
 * between phases on the stream; ms[SPHDEM_PHASE_COUNT] receives the phase
 * durations in milliseconds.  Synchronises the stream before returning. */
int sphdem_profile_step(sphdem_ctx_t* ctx, const sphdem_params_t* p, int step, int coupled,
                        float* ms, sphdem_stream_t stream);

/* ---- single kernels (reference kernel entry points) -------------------- */
int sphdem_shepard_sph(sphdem_ctx_t* c, float support, float h, sphdem_stream_t s);   /* kernel/KERNEL_rho.py:6-40    */
int sphdem_density_sph(sphdem_ctx_t* c, float support, float h, sphdem_stream_t s);   /* kernel/KERNEL_rho.py:45-82   */
int sphdem_density_bnd(sphdem_ctx_t* c, float support, float h, sphdem_stream_t s);   /* kernel/KERNEL_rho.py:87-126  */
int sphdem_pres_sph(sphdem_ctx_t* c, float rho0, float c0, float gamma, sphdem_stream_t s); /* kernel/KERNEL_pres.py:6-23 */
int sphdem_pres_bnd(sphdem_ctx_t* c, float rho0, float c0, float gamma, sphdem_stream_t s); /* kernel/KERNEL_pres.py:26-45 */
int sphdem_force_sph(sphdem_ctx_t* c, float support, float h, float mu, float g,
                     sphdem_stream_t s);                                                 /* kernel/KERNEL_force.py:7-71  */
int sphdem_step_sph(sphdem_ctx_t* c, float dt, sphdem_stream_t s);                      /* kernel/KERNEL_step.py:6-22   */
/* Count, scan and fill the DEM-DEM CSR, then flip its old/new sides
 * (Kernel_count_dem_contacts + array_scan + Kernel_force_dem + swap,
 * kernel/KERNEL_DEM_force.py:9-135, source/Simulation.py:142-171). */
int sphdem_force_dem(sphdem_ctx_t* c, float radius_max, float g, float dt, sphdem_stream_t s);
/* Same for the DEM-wall CSR (kernel/KERNEL_DEM_BC.py:10-84, source/Simulation.py:175-203). */
int sphdem_bc_dem(sphdem_ctx_t* c, float radius_max, float dt, sphdem_stream_t s);
int sphdem_step_dem(sphdem_ctx_t* c, float dt, sphdem_stream_t s);                      /* kernel/KERNEL_DEM_step.py:6-30 */

/* Contact rebuild for callers that cannot allocate device memory (no
 * counterpart in the reference): the same count -> scan -> fill -> swap as
 * sphdem_force_dem (which & 1) and sphdem_bc_dem (which & 2), but the per-row
 * count scratch (work.dem_count) is a fixed array inside the library instead
 * of a caller buffer; the caller still passes every input and output through
 * ctx.  Limit: at most SPHDEM_NOALLOC_MAX_DEM moving spheres, larger inputs
 * return SPHDEM_ERR_INVALID.  Allocates nothing.  The first call on a device
 * looks up the array's device address, so make that first call before any
 * stream capture.  All calls share the one array per device: calls whose GPU
 * work overlaps (different streams) race on it.  The current device must be
 * the GPU that holds ctx's sphere buffers (else SPHDEM_ERR_INVALID).  The
 * looked-up address does not survive cudaDeviceReset in the same process:
 * after a reset, do not call this entry point on that device again. */
#define SPHDEM_NOALLOC_MAX_DEM 65536
int sphdem_contacts_noalloc(sphdem_ctx_t* c, float radius_max, float bnd_radius_max, float g,
                            float dt, int which, sphdem_stream_t s);
int sphdem_prep_sphdem(sphdem_ctx_t* c, float support, float h, float sph_support,
                       float sph_h, float eps_min, float eps_max, sphdem_stream_t s);   /* kernel/KERNEL_SPHDEM_interaction.py:43-115 */
int sphdem_interaction_dem(sphdem_ctx_t* c, float mu, float eps_min, float eps_max,
                           float dt, sphdem_stream_t s);                                 /* kernel/KERNEL_SPHDEM_interaction.py:118-187 */
int sphdem_interaction_sph(sphdem_ctx_t* c, float support, sphdem_stream_t s);         /* kernel/KERNEL_SPHDEM_interaction.py:190-226 */

/* ---- point evaluations for known-answer tests -------------------------- */
/* W and dW/dr of the 3D Wendland C2 kernel at n radii (kernel/Kernel_KNL.py:7-41). */
int sphdem_wendland(const float* r, int32_t n, float h, float* w, float* dw, sphdem_stream_t s);
/* beta/(1-eps) of DEM_drag_beta (kernel/KERNEL_SPHDEM_interaction.py:11-40). */
int sphdem_drag_beta(const float* eps, const float* rho, const float* mu,
                     const float* diameter, const float* speed, int32_t n, float* out,
                     sphdem_stream_t s);

/* ---- verification and diagnostics -------------------------------------- */
/* Neighbour relations of the step, each with the exact FP32 predicate of the
 * reference kernel it belongs to (s = radius argument, d2 = dot(r,r) and
 * len = sqrt(d2), both rounded in FP32 exactly as written):              */
#define SPHDEM_REL_SPH_SPH_SUPPORT 0  /* fluid-fluid  d2 < s*s       KERNEL_rho.py:30,72        */
#define SPHDEM_REL_SPH_BND_SUPPORT 1  /* fluid-wall   d2 < s*s       KERNEL_rho.py:37,79        */
#define SPHDEM_REL_BND_SPH_SUPPORT 2  /* wall-fluid   d2 < s*s       KERNEL_rho.py:116          */
#define SPHDEM_REL_BND_BND_SUPPORT 3  /* wall-wall    d2 < s*s       KERNEL_rho.py:123          */
#define SPHDEM_REL_SPH_SPH_FORCE   4  /* fluid-fluid  1e-12 < d2 < s*s  KERNEL_force.py:40-41    */
#define SPHDEM_REL_SPH_BND_FORCE   5  /* fluid-wall   1e-12 < d2 < s*s  KERNEL_force.py:57-58    */
#define SPHDEM_REL_SPH_SPH_LEN     6  /* fluid-fluid  len < s        KERNEL_SPHDEM_interaction.py:80-81 */
#define SPHDEM_REL_SPH_DEM_2H      7  /* fluid-DEM b  len < 2*h_b    KERNEL_SPHDEM_interaction.py:87-88 */
#define SPHDEM_REL_DEM_SPH_2H      8  /* DEM a-fluid  len < 2*h_a    KERNEL_SPHDEM_interaction.py:157-158 */
#define SPHDEM_REL_DEM_DEM_2H      9  /* DEM a-DEM b  len < 2*h_a (a included)  :166-167        */
#define SPHDEM_REL_SPH_DEM_REACT  10  /* fluid-DEM b  len < 2*h_b and flt_s[b] > 1e-12  :220-221 */
#define SPHDEM_REL_COUNT          11
/* Order-independent digest of one relation, per subject in point order:
 * count[i] = members, hash[i] = sum over members j of mix64(j) (mod 2^64),
 * mix64 = the SplitMix64 finaliser.  Device outputs. */
int sphdem_neighbour_digest(sphdem_ctx_t* c, int relation, float radius,
                            int32_t* count, uint64_t* hash, sphdem_stream_t s);
/* Member sets the hot-path kernels themselves decided in the last step, per
 * fluid particle in point order, in the digest form above (count, sum of
 * mix64(neighbour point index)):
 *   DENSITY_FLUID / DENSITY_WALL: the members the density pass recorded in
 *     work.nbr (its d2 < s*s decisions; relations SPH_SPH_SUPPORT and
 *     SPH_BND_SUPPORT); a particle whose record overflowed is digested by the
 *     same cell walk the force pass then takes;
 *   FORCE_FLUID / FORCE_WALL: the members the force pass sums over (the
 *     recorded members with 1e-12 < d2, or its own walk when a record overflowed;
 *     relations SPH_SPH_FORCE and SPH_BND_FORCE);
 *   POROSITY_NEAR: count = 1 for the particles the porosity pass listed as
 *     having a DEM within 2 h_b (relation SPH_DEM_2H non-empty), else 0.
 * Positions are the sorted copies of the step's start (work.f_posm, b_posm);
 * p supplies the support and the list capacity of the step. */
#define SPHDEM_MEMBERS_DENSITY_FLUID 0
#define SPHDEM_MEMBERS_DENSITY_WALL  1
#define SPHDEM_MEMBERS_FORCE_FLUID   2
#define SPHDEM_MEMBERS_FORCE_WALL    3
#define SPHDEM_MEMBERS_POROSITY_NEAR 4
#define SPHDEM_MEMBERS_COUNT         5
int sphdem_member_digest(sphdem_ctx_t* c, const sphdem_params_t* p, int which, int32_t* count, uint64_t* hash,
                         sphdem_stream_t s);
/* Self-test of the bounded device-side wait (no reference counterpart): one
 * CTA waits `polls` times (0..2^20) on a shared-memory barrier that nothing
 * arrives at -- no copy or MMA is issued -- then ORs SPHDEM_FLAG_TIMEOUT into
 * ctl->status and exits, exactly as a staged kernel whose copy never lands. */
int sphdem_wait_selftest(sphdem_ctl_t* ctl, int polls, sphdem_stream_t s);
/* FP64 global diagnostics of fluid + moving DEM: out[0] fluid mass, out[1] DEM
 * mass, out[2..4] momentum, out[5] translational kinetic energy, out[6]
 * rotational kinetic energy, out[7] potential energy m*g*z.  out is a device
 * double[8]. */
int sphdem_diagnostics(sphdem_ctx_t* c, float g, double* out, sphdem_stream_t s);

/* ---- frame output (host) -------------------------------------------------
 * ASCII formatting of VTK XML PolyData arrays as output/output.py:16-25
 * (_fmt_float / _fmt_int) writes them: "%.6g" of each float as a double, or
 * "%d", one space between values, per_line values per line, lines joined by
 * '\n', no trailing newline.  Split over `threads` host threads (0 = all) by
 * whole lines; the text does not depend on the thread count.  out == NULL
 * returns the byte count; otherwise the bytes written, -1 if cap is too small,
 * -2 for invalid arguments. */
int64_t sphdem_format_f32(const float* v, int64_t n, int32_t per_line, char* out, int64_t cap, int32_t threads);
int64_t sphdem_format_i32(const int32_t* v, int64_t n, int32_t per_line, char* out, int64_t cap,
                          int32_t threads);

#ifdef __cplusplus
}
#endif
#endif /* SPHDEM_H */
