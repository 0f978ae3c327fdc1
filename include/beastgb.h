/*
 * beastgb.h -- C ABI of libbeastgb, a GB300 (sm_103a) BEM Galerkin matrix-assembly engine.
 *
 * The library is the drop-in for the assembly path of BEASTGPU / BEAST:
 *   assemble_gpu(op, X, Y, config, writeBackStrategy; quadstrat)  (assamble_gpu.jl:8,25)
 *   BEAST.assemble(op, X, Y; quadstrat)                            (data/BEAST__multi.jl:15)
 * A Julia `ccall` shim marshals BEAST's assembly data into the structs below (the same
 * packing load_parameters.jl:25-54 does for the reference's kernels) and calls
 * bgb_assemble.  All pointers are plain host pointers unless a field says "device".
 *
 * Errors: every entry point returns 0 on success or a negative bgb_status; the message of
 * the last failure on the calling thread is bgb_last_error().  Nothing aborts the process
 * and no kernel traps.  No kernel of the library waits on another CTA, stream or device, so
 * there is no device-side wait to bound: BGB_ERR_TIMEOUT is reserved and never returned.
 *
 * Threading: one handle per host thread (or per CUDA stream); calls on different handles
 * may run concurrently.  A handle owns its device scratch and pinned staging buffers.
 */
#ifndef BEASTGB_H
#define BEASTGB_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BGB_ABI_VERSION 3

/* bgb_config.flags: copy pageable host outputs through the pinned ring even when the device
 * reaches pageable memory through the host page tables (by default such outputs are written
 * by DMA after their pages are faulted in). */
#define BGB_CFG_PAGEABLE_VIA_RING 1

typedef enum {
  BGB_OK = 0,
  BGB_ERR_INVALID = -1,       /* bad argument, inconsistent tables, degenerate geometry */
  BGB_ERR_OOM = -2,           /* device or pinned host allocation failed */
  BGB_ERR_CUDA = -3,          /* CUDA runtime error */
  BGB_ERR_TIMEOUT = -4,       /* reserved (no entry point returns it: no kernel waits) */
  BGB_ERR_ABORTED = -5,       /* bgb_abort() was called while the call ran */
  BGB_ERR_CAPACITY = -6,      /* a fixed capacity was exceeded */
  BGB_ERR_NOT_SUPPORTED = -7  /* operator / space / rule combination not implemented */
} bgb_status;

/* Operators (BEAST: Helmholtz3D.singlelayer, Maxwell3D.singlelayer, Maxwell3D.doublelayer). */
typedef enum {
  BGB_OP_HELMHOLTZ3D_SL = 0, /* alpha int int G f g */
  BGB_OP_MAXWELL3D_SL = 1,   /* int int G [alpha f.g + beta div f div g] */
  BGB_OP_MAXWELL3D_DL = 2,   /* alpha int int f(x) . (grad_x G(x,y) x g(y)) */
  BGB_OP_HELMHOLTZ3D_DL = 3,  /* alpha int int f(x) dG/dn_y g(y), dG/dn_y = n_y . grad_y G (Lagrange) */
  BGB_OP_HELMHOLTZ3D_DLT = 4, /* alpha int int f(x) dG/dn_x g(y), the transposed double layer (Lagrange) */
  BGB_OP_HELMHOLTZ3D_HS = 5   /* int int G [alpha (n_x.n_y) f g + beta curl f . curl g] (hypersingular,
                                 Maue's form; BEAST: alpha = gamma^2, beta = 1) */
} bgb_op_kind;

/* Local shape-function families (BEAST reference spaces). */
typedef enum {
  BGB_REFSPACE_LAGRANGE_C0D1 = 0, /* barycentric hats (u, v, 1-u-v) */
  BGB_REFSPACE_RT = 1             /* Raviart-Thomas / RWG: (x - v_i) / (2A), div 1/A */
} bgb_refspace;

typedef enum { BGB_PREC_FP64 = 0, BGB_PREC_MIXED = 1 } bgb_precision;

typedef enum {
  BGB_OUT_HOST_C64 = 0,   /* host complex double, (re, im) pairs */
  BGB_OUT_HOST_C32 = 1,   /* host complex float */
  BGB_OUT_DEVICE_C64 = 2, /* device complex double */
  BGB_OUT_DEVICE_C32 = 3  /* device complex float */
} bgb_out_kind;

/* Pair classes (quadrule_determine.jl:76). */
typedef enum { BGB_CLASS_FAR = 0, BGB_CLASS_CV = 1, BGB_CLASS_CE = 2, BGB_CLASS_CF = 3, BGB_CLASS_NEAR = 4 } bgb_pair_class;

/* Operator: G(R) = exp(-gamma R) / (4 pi R), gamma = i k.  Complex numbers are (re, im). */
typedef struct {
  int32_t kind;    /* bgb_op_kind */
  double alpha[2];
  double beta[2];  /* Maxwell single layer only */
  double gamma[2];
} bgb_operator;

/* Function space as per-triangle assembly tables (BEAST assemblydata, one function per
 * local shape as in load_parameters.jl:50-54).  Triangles are in chart order (v1, v2, v3);
 * local shape i belongs to vertex i (Lagrange) or to the edge opposite vertex i (RT). */
typedef struct {
  int32_t refspace;          /* bgb_refspace */
  int32_t nv, nt, nfun;
  const double* vertices;    /* [nv][3] */
  const int32_t* triangles;  /* [nt][3], 0-based vertex indices */
  const int32_t* fn_index;   /* [nt][3], global function of local shape i, -1 if none */
  const double* fn_coef;     /* [nt][3] */
} bgb_space;

/* Quadrature strategy (BEAST DoubleNumWiltonSauterQStrat fields used by the path).
 * Triangle rules: 1, 3, 4, 6, 7, 12 or 13 points (symmetric Dunavant rules).
 * Sauter-Schwab: Gauss-Legendre points per dimension, 1..16. */
typedef struct {
  int32_t far_test, far_trial;   /* reference: 3 and 4 (GPU_scheduler.jl:94-95) */
  int32_t near_test, near_trial;
  int32_t ss_cf, ss_ce, ss_cv;   /* reference: 4 (SauterSchwab.jl:331,433) */
} bgb_quadstrat;

/* Handle configuration (GPUConfiguration, utils/configuration.jl:11-26, reduced to what a
 * GB300 needs).  Zero-initialised fields take defaults. */
typedef struct {
  int32_t device;              /* CUDA device ordinal */
  int64_t hbm_budget_bytes;    /* 0 = 90% of free device memory; bounds row blocks */
  int64_t pinned_ring_bytes;   /* each half of the pinned ring that pageable host outputs are
                                  copied through (at least one column of the output); 0 = 512 MiB */
  int32_t tile_config;         /* -1 = first tile shape that fits shared memory, else a tile id (bgb_tile_info) */
  int32_t flags;               /* BGB_CFG_* bits */
} bgb_config;

typedef struct {
  int64_t pairs_total;          /* nt_test * nt_trial over the assembled rows */
  int64_t pairs_class[5];       /* far, CV, CE, CF, near */
  int64_t pairs_computed;       /* triangle pairs evaluated by the far kernel (incl. halo) */
  double ms_classify, ms_singular; /* device time of the classification / singular stages (a host
                                      output in several blocks integrates its singular entries in
                                      groups beside the far kernels: ms_singular spans them) */
  double ms_far;                /* device time of the far kernels (sum over output blocks; blocks on
                                   the two compute streams may overlap) */
  double ms_copy;               /* device-to-host copy time (sum over output blocks) */
  double ms_total;              /* wall time of the call */
  double ms_pipeline;           /* wall time of the far kernels and copies (overlapped) */
  double ms_plan;               /* host tile planning (runs beside the classification) */
  int32_t out_blocks;           /* output blocks: column ranges of a host output */
  int32_t tile_config;
  int32_t kernel_launches;      /* kernels this call launched */
  int32_t schedule;             /* batches: work-queue schedule (0 problem-major, 1 largest first) */
} bgb_stats;

typedef struct bgb_handle bgb_handle;

/* Create / destroy a handle on cfg->device (cfg may be NULL).
 * Replaces: the GPUConfiguration() constructor plus CUDA backend set-up
 * (utils/configuration.jl:29-50, assamble_gpu.jl:25-65). */
int bgb_create(bgb_handle** out, const bgb_config* cfg);
int bgb_destroy(bgb_handle* h);

/* Assemble rows [row0, row0 + nrows) of Z (test functions) against all trial functions.
 * nrows < 0 means all rows.  Output is column-major (Julia layout): element (m, n) at
 * out[(m - row0) + n * ld], ld >= nrows; `out` must hold ld * (trial->nfun - 1) + nrows entries of
 * the out_kind's type (complex double or complex float; the library cannot check).  Device outputs are written on `stream`
 * (a cudaStream_t, NULL = the handle's stream); host outputs are complete on return.
 * BGB_PREC_MIXED reduces the phase k R exactly for k times the diameter of the two meshes up to
 * 3e5 and returns BGB_ERR_NOT_SUPPORTED beyond (use BGB_PREC_FP64 there).
 * Replaces: assemble_gpu(op, X, Y, config, GpuWriteBackTrueInstance(); quadstrat)
 * (assamble_gpu.jl:25-137) and BEAST.assemble for the same operator (data/BEAST__multi.jl:15). */
int bgb_assemble(bgb_handle* h, const bgb_operator* op, const bgb_space* test,
                 const bgb_space* trial, const bgb_quadstrat* qs, int32_t precision,
                 void* out, int32_t out_kind, int64_t ld, int64_t row0, int64_t nrows,
                 void* stream, bgb_stats* stats);

/* One problem of a batch. */
typedef struct {
  bgb_operator op;
  bgb_space test, trial;
  bgb_quadstrat qs;
  void* out;        /* device or host per out_kind of the batch call */
  int64_t ld;
} bgb_problem;

/* Assemble n independent problems (uneven sizes and wave numbers) in one go: one launch
 * classifies all pairs, one integrates all singular / near pairs, and ONE persistent
 * far-pair launch pulls (problem, row block, column block) tiles from a work queue.  All
 * problems share the operator kind, the spaces' kind and the quadrature strategy; each has
 * its own operator parameters, mesh and output (ld >= rows).  Results are bit-identical to
 * assembling each problem with bgb_assemble.  No reference counterpart: the reference
 * assembles one operator per call (assamble_gpu.jl:25). */
int bgb_assemble_batch(bgb_handle* h, int32_t n, const bgb_problem* problems, int32_t precision,
                       int32_t out_kind, void* stream, bgb_stats* stats);

/* Plan / execute form of the batch: bgb_batch_create does the planning, runs every stage
 * once (the batch is assembled on return), optionally autotunes the tile shape and the
 * work-queue schedule (flags & 1: every fitting candidate is timed on this batch), and
 * captures the whole device sequence in a CUDA graph; bgb_batch_run replays that graph
 * (re-assembling the same problems into the same outputs) and copies host outputs.
 * stats->tile_config / schedule report the chosen tile shape / work-queue schedule (0 problem-major,
 * 1 largest tiles first); stats->ms_total of bgb_batch_run is the graph's device time. */
typedef struct bgb_batch bgb_batch;
int bgb_batch_create(bgb_handle* h, int32_t n, const bgb_problem* problems, int32_t precision,
                     int32_t out_kind, int32_t flags, bgb_batch** out, bgb_stats* stats);
int bgb_batch_run(bgb_batch* batch, void* stream, bgb_stats* stats);
int bgb_batch_destroy(bgb_batch* batch);

/* Pair classes of a block of triangle pairs on the device, out[(t - t0) * (s1 - s0) + (s - s0)]
 * (host int8 buffer).  Replaces: determine_quadrule_types / quadrule_determine_type
 * (quadrule_determine.jl:5-47,54-77). */
int bgb_classify_block(bgb_handle* h, const bgb_space* test, const bgb_space* trial, double k2,
                       int32_t t0, int32_t t1, int32_t s0, int32_t s1, int8_t* out);

/* Local 3x3 complex matrices of a list of triangle pairs (out: double[npairs][9][2], host),
 * with the rule chosen by classification or forced (force_class >= 0), computed by the
 * kernels bgb_assemble uses for `precision`: singular and near pairs by the FP64 kernel
 * (BGB_PREC_FP64) or the double-float kernel (BGB_PREC_MIXED), far pairs by the far
 * kernel's pair code.
 * Replaces the per-pair integrals of sauterschwab_parameterized_gpu_outside_loop_kernel!
 * (SauterSchwab.jl:212-262) and doubleQuadRuleMainCaseKernel! (doubleQuadRuleMainCase.jl:60-105)
 * before their scatter. */
int bgb_local_matrices(bgb_handle* h, const bgb_operator* op, const bgb_space* test,
                       const bgb_space* trial, const bgb_quadstrat* qs, int32_t precision, int64_t npairs,
                       const int32_t* tau, const int32_t* sigma, int32_t force_class,
                       double* out, int8_t* cls_out);

/* Pair classification into a CSR for callers that cannot allocate device memory (for
 * example a Julia or PyTorch process whose memory pool already holds the device, or an
 * embedding that forbids allocations outside its own allocator).  No reference counterpart:
 * it is an addition of this library.
 * Inputs are device arrays (vertices double[nv][3], triangles int32[nt][3]); outputs are
 * device arrays: d_offsets int64[nt_test + 1] (CSR over test triangles) and, per non-far
 * pair, d_tau / d_sigma int32 and d_class int8 (1 CV, 2 CE, 3 CF, 4 near), sorted by trial
 * triangle within each test triangle -- the same classes as bgb_classify_block.  *total
 * (host) receives the number of non-far pairs; if it exceeds `capacity` the call returns
 * BGB_ERR_CAPACITY after filling d_offsets and *total, so the caller can retry.
 * It calls no cudaMalloc / cudaFree: its scratch is a fixed 16 MiB device array of the
 * library, 156 bytes per test triangle plus 152 bytes per trial triangle (about 54,000
 * triangles per side when test and trial are the same mesh; larger inputs are rejected
 * with BGB_ERR_CAPACITY before any work).  Every device holds that array until the
 * process exits.  Each call looks up the array's address on the current device (so a reset
 * context is no problem); the first call on a device may also load the library's device
 * code there (make that first call before any stream capture).  nt > 0 with nv == 0 is
 * BGB_ERR_INVALID; a vertex index outside [0, nv) is reported as BGB_ERR_INVALID without
 * being read.  All calls on a device share the array: calls whose GPU
 * work overlaps race and must be serialised by the caller.  Work is queued on `stream`
 * (a cudaStream_t, NULL = default stream); the call waits for the pair count only. */
int bgb_classify_csr_noalloc(const double* d_vertices_test, const int32_t* d_triangles_test,
                             int32_t nv_test, int32_t nt_test, const double* d_vertices_trial,
                             const int32_t* d_triangles_trial, int32_t nv_trial, int32_t nt_trial,
                             double k2, int64_t* d_offsets, int32_t* d_tau, int32_t* d_sigma,
                             int8_t* d_class, int64_t capacity, int64_t* total, void* stream);

/* ---- Curves: BEAST Helmholtz2D on polygonal curves ----------------------------------------
 * The 2-D family of the reference's hypersingular prototype (old_code/doubleQuadRule_2d_gpu.jl:
 * kernel at :72-78, integrand at :88-97, double quadrature at :129-210 and :265-465), widened to
 * the four Helmholtz2D operators and to whole matrices.
 * Kernel: G(R) = -(i/4) H0^(2)(kR) for k > 0, -(1/2 pi) ln R for k = 0; grad_x G = (x - y) g1(R).
 * Cells are straight segments (v0, v1), chart x(s) = (1 - s) v0 + s v1 (s in [0, 1]), length l,
 * normal n = (d_y, -d_x) / l with d = v1 - v0 (outward on a counter-clockwise closed curve). */
typedef enum {
  BGB_OP2D_SL = 0,  /* alpha int int G f g */
  BGB_OP2D_DL = 1,  /* alpha int int f (n_y . grad_y G) g */
  BGB_OP2D_DLT = 2, /* alpha int int f (n_x . grad_x G) g */
  BGB_OP2D_HS = 3   /* int int G [alpha (n_x . n_y) f g + beta f' g'], f' the arc-length derivative
                       (BEAST and the prototype: alpha = -k^2, beta = 1) */
} bgb_op2d_kind;
typedef struct {
  int32_t kind;       /* bgb_op2d_kind */
  double wavenumber;  /* real k >= 0 */
  double alpha[2];
  double beta[2];     /* hypersingular only */
} bgb_operator2d;
typedef enum {
  BGB_REFSPACE2D_LAGRANGE_C0D1 = 0, /* hats 1 - s (vertex v0) and s (v1); derivatives -1/l, +1/l */
  BGB_REFSPACE2D_LAGRANGE_CXD0 = 1  /* one constant per segment (column 1 of the tables unused) */
} bgb_refspace2d;
typedef struct {
  int32_t refspace;          /* bgb_refspace2d */
  int32_t nv, ns, nfun;
  const double* vertices;    /* [nv][2] */
  const int32_t* segments;   /* [ns][2], 0-based vertex indices (v0, v1) */
  const int32_t* fn_index;   /* [ns][2], global function of local shape i, -1 if none */
  const double* fn_coef;     /* [ns][2] */
} bgb_curve_space;
/* Rules of the curve path.  Pair classes: the predicate of bgb_classify_block over the two
 * vertices of each segment, with the trial segment's length as its chart volume: 3 coincident
 * (two shared vertices), 1 common vertex, 4 near, 0 far.
 *   far pairs:   Gauss-Legendre far_test x far_trial points (1..32);
 *   near pairs:  near x near Gauss-Legendre points (1..32) on the leaves of a bisection of the
 *                chart square (the longer piece is halved until each piece pair is at least as
 *                far apart as its longer piece is long, at most 16 times);
 *   coincident / common vertex: order `singular` (1..16) graded rules after a split of the
 *                chart square along its diagonal: (3n + 1) n graded points (n Gauss points on
 *                3n + 1 intervals of ratio 0.35 towards the singularity) times n Gauss points.
 * Double layers vanish on coincident segments. */
typedef struct {
  int32_t far_test, far_trial;
  int32_t near;
  int32_t singular;
} bgb_quadstrat2d;
/* Assemble rows [row0, row0 + nrows) of the curve operator's matrix; arguments, output layout,
 * streams and errors as bgb_assemble.  precision: BGB_PREC_FP64 (all FP64, CUDA's Bessel
 * functions) or BGB_PREC_MIXED (far pairs in FP32 with polynomial Hankel approximations and the
 * phase k R carried in double-float per pair, for k times the curves' diameter up to 3e5, else
 * BGB_ERR_NOT_SUPPORTED; coincident and common-vertex pairs in double-float (single layer,
 * hypersingular) or FP64, near pairs in FP64).  stats:
 * pairs over all test segments of the rows and all trial segments, classes 0 far, 1 common
 * vertex, 3 coincident, 4 near.
 * Replaces: momintegrals_gpu_doubleQuad! of the 2-D prototype (doubleQuadRule_2d_gpu.jl:265-465),
 * one segment pair per call there, all pairs and the assembly here. */
int bgb_assemble_curve(bgb_handle* h, const bgb_operator2d* op, const bgb_curve_space* test,
                       const bgb_curve_space* trial, const bgb_quadstrat2d* qs, int32_t precision, void* out,
                       int32_t out_kind, int64_t ld, int64_t row0, int64_t nrows, void* stream, bgb_stats* stats);
/* Local 2x2 complex matrices of a list of segment pairs (out: double[npairs][2][2][2], host;
 * entries of absent shapes are zero) with the rule chosen by classification or forced
 * (force_class 0 far or 4 near for any pair; 1 / 3 only for pairs of that class), computed by
 * the kernels bgb_assemble_curve uses for `precision`.  cls_out (optional): int8[npairs]. */
int bgb_local_matrices_curve(bgb_handle* h, const bgb_operator2d* op, const bgb_curve_space* test,
                             const bgb_curve_space* trial, const bgb_quadstrat2d* qs, int32_t precision,
                             int64_t npairs, const int32_t* tau, const int32_t* sigma, int32_t force_class,
                             double* out, int8_t* cls_out);
/* Ask a running call on this handle to stop at its next check point (BGB_ERR_ABORTED). */
int bgb_abort(bgb_handle* h);

/* Tile shapes compiled into the far-pair kernel: fills up to `cap` ids, returns the count. */
int bgb_tile_info(int32_t* ids, int32_t cap);

/* Far-kernel tiling of one side, on the host (no device needed): the order in which tiles of
 * `width` functions take the functions [f_begin, f_end) of `s` (order[f_end - f_begin]; each run
 * of `width` is one tile, a compact patch of a recursive coordinate bisection of the functions'
 * centres) and, in *slots, the number of (tile, support triangle) entries those tiles stage, i.e.
 * the triangles per side the far kernel evaluates, halo included.  The tiling replaces the square
 * tiles of the reference's scheduler (GPU_scheduler.jl:108-129); it does not change any value. */
int bgb_plan_order(const bgb_space* s, int32_t f_begin, int32_t f_end, int32_t width, int32_t* order,
                   int64_t* slots);

/* FP32 / FP64 FMA issue peaks and MUFU throughput measured on the handle's device
 * (TFLOP/s, TFLOP/s, Tops/s), for roofline denominators. */
int bgb_measure_issue_peaks(bgb_handle* h, double* fp32_tflops, double* fp64_tflops, double* mufu_tops);

/* Message of the last failure on the calling thread ("" if none). */
const char* bgb_last_error(void);

int bgb_abi_version(void);

#ifdef __cplusplus
}
#endif

#endif
