/*
 * bemgpu — C ABI of the GB300 (sm_103a) implementation of bem's per-frequency
 * hot path: PMCHWT RWG impedance fill, dense complex LU, heat-transfer trace.
 *
 * Every entry point takes plain pointers and sizes and returns an int status
 * (BEMGPU_OK or a negative BEMGPU_ERR_*).  Device buffers are owned by the
 * handles; a host-side caller never needs a CUDA type.  Streams are passed as
 * opaque void* (cudaStream_t), NULL meaning the context's own stream.
 *
 * Reference interfaces replaced (claytonotey/bem):
 *   bemgpu_green_init   -> GreensFunction::init            src/GreensFunction.cpp:17-30
 *   bemgpu_zts[_host]   -> Zts(RWGTree*,RWGTree*,GreensFunction*,Options&)
 *                                                          src/Impedance.h:21, src/Impedance.cpp:388-413
 *   bemgpu_heat_transfer-> CalcHeatTransfer(a,eV,T1,T2,top,s,t,Options&)
 *                                                          src/HeatTransfer.h:33, src/HeatTransfer.cpp:8-59
 *   bemgpu_theta        -> Theta(omega,T)                  src/HeatTransfer.cpp:3-6
 *   bemgpu_geom_create / bemgpu_tree_create
 *                       -> the RWGTree a caller builds (src/RWGTree.cpp:602-722),
 *                          flattened: the RWG order of the table is the matrix order.
 */
#ifndef BEMGPU_H
#define BEMGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define BEMGPU_OK 0
#define BEMGPU_ERR_ARG (-1)          /* invalid argument (sizes, indices, null pointers) */
#define BEMGPU_ERR_OOM (-2)          /* device allocation failed / over the admission budget */
#define BEMGPU_ERR_CUDA (-3)         /* a CUDA runtime call failed */
#define BEMGPU_ERR_SINGULAR (-4)     /* zero pivot in the LU */
#define BEMGPU_ERR_NO_CONVERGE (-5)  /* iterative refinement did not reach its tolerance */
#define BEMGPU_ERR_TIMEOUT (-6)      /* a bounded device wait ran out */
#define BEMGPU_ERR_MESH (-7)         /* mesh/RWG table is not a valid closed RWG table */
#define BEMGPU_ERR_CANCELLED (-8)    /* a farm request was cancelled before it started */
#define BEMGPU_PENDING 1             /* a farm request has not finished (not an error) */

/* ---- precision modes ---- */
#define BEMGPU_PREC_FP64 0    /* plain path: every stage in FP64 / complex128 */
#define BEMGPU_PREC_MIXED 1   /* FP32 far pairs (centroid distance > 3 edge lengths), FP64
                                 near/singular; complex64 tensor-core LU + FP64 refinement */
#define BEMGPU_PREC_MIXED_LA 2 /* FP64-class fill in double-float arithmetic (pairs of FP32,
                                  ~48 bits, on the FP32 pipes; ~1e-13 of the FP64 fill's row
                                  scale), mixed-precision solve as in BEMGPU_PREC_MIXED */

typedef struct bemgpu_ctx_s *bemgpu_ctx_t;
typedef struct bemgpu_geom_s *bemgpu_geom_t;
typedef struct bemgpu_tree_s *bemgpu_tree_t;
typedef struct bemgpu_farm_s *bemgpu_farm_t;

/* GreensFunction fields (src/GreensFunction.h:7-28), complex values as {re, im}. */
typedef struct {
  double eps[2], mu[2], omega[2];
  double ksquared[2], k[2], ik[2], k2[2], Zeps[2], Zmu[2];
  int external;
} bemgpu_green_t;

/* The Options fields on the fill path (src/Options.h; defaults src/Options.cpp:23-26). */
typedef struct {
  double farThresh6, farThresh10, farThresh15, farThresh21;
} bemgpu_options_t;

/* One frequency point of CalcHeatTransfer. */
typedef struct {
  double a;          /* length scale of the mesh coordinates, metres */
  double eV;         /* photon energy */
  double T1, T2;     /* body temperatures, K */
  double eps1[2], mu1[2], eps2[2], mu2[2]; /* body material constants at eV */
} bemgpu_solve_req_t;

/* Per-solve diagnostics (any pointer argument may be NULL). */
typedef struct {
  double ms_fill, ms_lu, ms_solve, ms_trace, ms_refine; /* stage times, device clock */
  double S_re, S_im;        /* 0.25 * Tr(B2^H B1) before the Theta factor */
  double err_est;           /* estimated relative error of Re S (0 on the FP64 path) */
  int refine_iters;
  int64_t pairs_near, pairs_far_fp64, pairs_far_fp32;
  double ms_queued, ms_latency; /* farm requests: submit -> start and submit -> done, host clock */
  int solver;                   /* mixed path: 1 complex64 LU, 2 FP64-class tensor-core LU, 3 the plain
                                   FP64 LU after the FP64-class refinement stalled (err_est then 0) */
} bemgpu_solve_info_t;

/* ---- context ---- */
/* Creates a context on a CUDA device (its own stream and workspace). */
int bemgpu_ctx_create(int device, bemgpu_ctx_t *out);
int bemgpu_ctx_destroy(bemgpu_ctx_t ctx);
/* Last error message of this context (static storage, never NULL). */
const char *bemgpu_ctx_last_error(bemgpu_ctx_t ctx);
/* Library version string. */
const char *bemgpu_version(void);
/* The context's CUDA stream (cudaStream_t) on which all its work is launched. */
int bemgpu_ctx_stream(bemgpu_ctx_t ctx, void **stream);
/* Number of kernels the context launched since it was created. */
int64_t bemgpu_ctx_launches(bemgpu_ctx_t ctx);
/* Bytes of device workspace the context holds (it grows to the largest solve
 * seen and is kept for the next one), and giving all of it back. */
int64_t bemgpu_ctx_workspace_bytes(bemgpu_ctx_t ctx);
int bemgpu_ctx_trim(bemgpu_ctx_t ctx);
/* Device bytes one CalcHeatTransfer solve needs at most (fill scratch plus
 * solve buffers) for bodies of nrwg_s and nrwg_t RWGs, with the default
 * mixed-path solver (complex64 LU that may escalate to the FP64-class LU).
 * No reference counterpart. */
int64_t bemgpu_solve_footprint(int nrwg_s, int nrwg_t, int precision);
/* The same for a solve on this context, under its solver mode
 * (bemgpu_ctx_set_solver; FP64-class only needs no complex64 factors): the
 * admission figure of the request farm's lanes. */
int64_t bemgpu_ctx_solve_footprint(bemgpu_ctx_t ctx, int nrwg_s, int nrwg_t, int precision);
/* Engines of the complex64 products: gemm = LU and correction solves,
 * acc64 = refinement residual and trace (FP64 output); 0 = the library's
 * choice (tensor cores where the shape allows), 1 = tensor cores where the
 * shape allows, 2 = FMA pipes only.  No reference counterpart (tuning). */
int bemgpu_ctx_set_engines(bemgpu_ctx_t ctx, int gemm, int acc64);
/* Factorization of the mixed path: 0 = complex64 LU, escalating to the
 * FP64-class tensor-core LU when its refinement does not converge (default);
 * 1 = complex64 only; 2 = FP64-class only.  No reference counterpart. */
int bemgpu_ctx_set_solver(bemgpu_ctx_t ctx, int mode);
/* Error estimate of the complex64 refinement above which mode 0 escalates to
 * the FP64-class factorization (default 1e-6, the mixed path's bound). */
int bemgpu_ctx_set_escalation_tol(bemgpu_ctx_t ctx, double tol);
/* Error estimate of the FP64-class refinement above which mode 0 solves the
 * same W again on the plain FP64 path (default 1e-6): the refinement's
 * residual is exact to ~2^-40, so for W conditioned worse than ~1e6 its
 * estimate stalls above the bound while the FP64 LU still meets it. */
int bemgpu_ctx_set_fp64_fallback_tol(bemgpu_ctx_t ctx, double tol);
/* Launch-shape knobs of this context (no reference counterpart), set by the
 * project's autotuner (bem_gb300/tuning.py: it times each candidate on the
 * caller's workload and caches the best per GPU and size class).
 *   BEMGPU_TUNE_NEAR_MINB  CTAs per SM that the double-float near-pair kernel's
 *                          register budget allows: 2 (default), 3 (168
 *                          registers) or 4 (128, some spilled);
 *   BEMGPU_TUNE_FAR_ROWS   warps per CTA of the far-pair kernel: 1, 2, 4 (default), 8;
 *   BEMGPU_TUNE_RASTER     M-tiles per rasterization band of the tensor-core
 *                          products: 1..64 (default 8);
 *   BEMGPU_TUNE_PANEL_CTAS CTAs of a cooperative LU panel at most (fewer,
 *                          fuller CTAs leave SMs to other lanes' work while a
 *                          latency-bound panel runs): 0 (one per SM, default)
 *                          or a cap, raised where shared memory requires;
 *   BEMGPU_TUNE_NEAR_SYNC  1 (default): the double-float near-pair kernel's
 *                          CTAs barrier after each pair couple, keeping their
 *                          warps in the same code region; 0: no barrier;
 *   BEMGPU_TUNE_NEAR_GRID  CTAs per SM of the near-pair launch's grid at most:
 *                          1..64 (default 16);
 *   BEMGPU_TUNE_EX_WIDE    1 (default): the exact products with level-3/4
 *                          slice products (5 x 2, 5 x 3, 4 x 4) on 128 x 128
 *                          tiles when that grid has at least 4 waves; 2:
 *                          on 128 x 128 tiles at any size; 0: all on
 *                          128 x 64 tiles.  The two differ in the last bits
 *                          of an FP32 sum (levels 3 and 4 in one buffer or
 *                          two), well inside the products' 2^-40 accuracy;
 *   BEMGPU_TUNE_LU_SUPER   1 (default): the complex64 LU factors its 128-wide
 *                          panels in pairs and updates the trailing matrix
 *                          once per pair (K = 256); 0: after every panel.
 *                          The same updates, rounded in another order.
 * BEMGPU_ERR_ARG for an unknown knob or value.  Results do not depend on
 * them, except as BEMGPU_TUNE_EX_WIDE and BEMGPU_TUNE_LU_SUPER say. */
#define BEMGPU_TUNE_NEAR_MINB 0
#define BEMGPU_TUNE_FAR_ROWS 1
#define BEMGPU_TUNE_RASTER 2
#define BEMGPU_TUNE_PANEL_CTAS 3
#define BEMGPU_TUNE_NEAR_SYNC 4
#define BEMGPU_TUNE_NEAR_GRID 5
#define BEMGPU_TUNE_EX_WIDE 6
#define BEMGPU_TUNE_LU_SUPER 7
int bemgpu_ctx_set_tuning(bemgpu_ctx_t ctx, int knob, int value);
int bemgpu_ctx_get_tuning(bemgpu_ctx_t ctx, int knob, int *value);
/* Tracing: with BEMGPU_TRACE set (not "0") in the environment, the library
 * prints one line per refinement step and escalation decision to stderr. */
/* Failure-path self-test: one kernel polls a flag that nothing sets, gives up
 * after `spins` polls (or about a second), and records a timeout exactly as the
 * library's bounded waits do; returns BEMGPU_ERR_TIMEOUT and leaves the context
 * usable.  No reference counterpart. */
int bemgpu_ctx_wait_selftest(bemgpu_ctx_t ctx, int64_t spins);

/* ---- live kernel statistics (measurement hooks; no counterpart in the reference) ---- */
/* Kernel classes timed with CUDA events on the context stream while enabled. */
#define BEMGPU_K_FILL_FAR 0     /* far triangle pairs */
#define BEMGPU_K_FILL_NEAR 1    /* same / vertex-sharing triangle pairs */
#define BEMGPU_K_GATHER 2       /* half-pair blocks -> matrix entries */
#define BEMGPU_K_LU_PANEL 3     /* LU panel columns, row interchanges */
#define BEMGPU_K_LU_GEMM 4      /* LU trailing-matrix update */
#define BEMGPU_K_TRSM 5         /* triangular blocks (LU and solve) */
#define BEMGPU_K_SOLVE_GEMM 6   /* off-diagonal updates of the triangular solves */
#define BEMGPU_K_TRACE 7        /* sym, the two trace products, the trace reduction */
#define BEMGPU_K_REFINE_GEMM 8  /* refinement residual: far-part product */
#define BEMGPU_K_NEAR_SPMM 9    /* FP64 near-part products (residual and trace) */
#define BEMGPU_K_SLICE 10       /* tensor-core operand slicing */
#define BEMGPU_K_COUNT 11
/* Enables (1) or disables (0) event timing of every launch; resets the totals. */
int bemgpu_prof_enable(bemgpu_ctx_t ctx, int enable);
/* Totals of one kernel class since the last enable: launches, device ms,
 * algorithmic flops and algorithmic DRAM bytes (synchronizes the context stream). */
int bemgpu_prof_query(bemgpu_ctx_t ctx, int kind, int64_t *launches, double *ms, double *flops, double *bytes);
/* bf16 tensor-core flops the same launches executed: for each product of
 * sliced operands, its slice products x 8 m n k (0 for kinds off the tensor pipe). */
int bemgpu_prof_query_tensor(bemgpu_ctx_t ctx, int kind, double *tensor_flops);

/* ---- resident geometry and RWG trees ---- */
/* Uploads vertices (xyz[3*nv]) and triangles (tri[3*nt], vertex ids, each
 * triangle's own vertex order kept).  Vertex identity is the id: two bodies
 * never share vertex ids (sharedpoints, src/Triangle.h:23-30). */
int bemgpu_geom_create(bemgpu_ctx_t ctx, const double *xyz, int nv, const int *tri, int nt,
                       bemgpu_geom_t *out);
int bemgpu_geom_destroy(bemgpu_geom_t g);
/* An RWG table over a geometry: rwg[4*i] = {pos triangle, neg triangle, edge
 * vertex 1, edge vertex 2}; row i is matrix unknown pair (2i: J, 2i+1: M).
 * Precomputes the half-RWG frames (HalfRWG::HalfRWG, src/RWG.cpp:7-39). */
int bemgpu_tree_create(bemgpu_geom_t g, const int *rwg, int nrwg, bemgpu_tree_t *out);
/* Destroying a tree or geometry does not wait for the device: its device
 * memory (triangle records, near-pair lists) joins a process-wide list that
 * is freed in one batch, after one device synchronisation, once it holds 96
 * blocks or 512 MB, on bemgpu_ctx_trim, when a context is torn down, and
 * before a failed allocation is retried.  (cudaFree waits for the whole
 * device: freeing each request's geometry at once would drain every farm
 * lane's work per request.)  A tree must not be destroyed while a call that
 * uses it is running. */
int bemgpu_tree_destroy(bemgpu_tree_t t);
/* Bytes of destroyed trees' and geometries' device memory awaiting the next
 * batch free. */
int64_t bemgpu_pending_free_bytes(void);
int bemgpu_tree_size(bemgpu_tree_t t);
/* RWG table of one closed body, in the reference's edge-creation order
 * (ShapeMesh::ShapeMesh, src/ShapeMesh.cpp:857-928): triangles in order, each
 * edge (v0,v1), (v1,v2), (v2,v0) whose other triangle comes later becomes row
 * {this triangle, the other, the edge's vertices in this triangle's order}.
 * Writes min(cap, count) rows to rwg[4*cap] and the count (3 nt / 2) to
 * *nrwg; BEMGPU_ERR_ARG when cap is below the count, BEMGPU_ERR_MESH when an
 * edge does not have exactly two triangles.  Host only (no context). */
int bemgpu_mesh_rwgs(const int *tri, int nt, int nv, int *rwg, int cap, int *nrwg);

/* The same RWG table built on the device, with the tree's half-RWG frames:
 * the closed body formed by the geometry's triangles [tri0, tri0 + ntri),
 * its RWGs in the reference's edge-creation order (ShapeMesh::ShapeMesh,
 * src/ShapeMesh.cpp:857-928; rows as bemgpu_mesh_rwgs writes them, with
 * geometry triangle ids) and the records of HalfRWG::HalfRWG
 * (src/RWG.cpp:7-39), computed by kernels from the resident geometry
 * (mesh set-up for new geometries without the host builder).  BEMGPU_ERR_MESH
 * when the body is not a closed 2-manifold.  Synchronous. */
int bemgpu_tree_create_body_device(bemgpu_geom_t g, int tri0, int ntri, bemgpu_tree_t *out);
/* The two-body tree (RWGTree over both bodies, src/RWGTree.cpp:602-722 with
 * the bodies' RWGs one after the other): a's RWGs, then b's; the trees share
 * one geometry and no triangle.  The records are concatenated on the device. */
int bemgpu_tree_concat(bemgpu_tree_t a, bemgpu_tree_t b, bemgpu_tree_t *out);
/* A tree's RWG table (4 ints per RWG, as bemgpu_tree_create takes it): writes
 * min(cap, size) rows; returns the size. */
int bemgpu_tree_rwgs(bemgpu_tree_t t, int *rwg, int cap);

/* ---- Green's function / constants ---- */
/* GreensFunction::init(eps, mu, omega) (src/GreensFunction.cpp:17-30). */
int bemgpu_green_init(const double eps[2], const double mu[2], const double omega[2], int external,
                      bemgpu_green_t *out);
/* Default Options far-rule thresholds (src/Options.cpp:23-26). */
void bemgpu_options_default(bemgpu_options_t *opt);
/* Theta(omega, T) = hbar*omega/(exp(hbar*omega/(kb*T))-1) (src/HeatTransfer.cpp:3-6). */
double bemgpu_theta(double omega, double T);
/* Dimensionless frequency omega_SI*a/c used by CalcHeatTransfer (src/HeatTransfer.cpp:10-11). */
double bemgpu_dimensionless_omega(double a, double eV);

/* ---- impedance fill ---- */
/* Zts(t, s, g): fills dZ (device, column-major complex128 or complex64 per
 * precision, leading dimension ldz >= 2*size(t)) with the (2Nt x 2Ns) PMCHWT
 * block.  t and s must share one geometry.  Asynchronous on `stream`. */
int bemgpu_zts(bemgpu_ctx_t ctx, bemgpu_tree_t t, bemgpu_tree_t s, const bemgpu_green_t *g,
               const bemgpu_options_t *opt, int precision, void *dZ, int64_t ldz, void *stream);
/* Same, writing a host column-major complex128 matrix (synchronous). */
int bemgpu_zts_host(bemgpu_ctx_t ctx, bemgpu_tree_t t, bemgpu_tree_t s, const bemgpu_green_t *g,
                    const bemgpu_options_t *opt, int precision, double *Z, int64_t ldz);

/* Zts(t, s, g) in FP64 into the caller's device buffer dZ without allocating
 * device memory (no counterpart in the reference).  For callers that must not
 * allocate while they run: a solver loop with a latency budget that cannot
 * stall in cudaMalloc, or a host application whose own memory pool has
 * claimed the device memory.  The scratch is one file-scope device array of
 * 32 MiB that every GPU loading the library holds until the process exits; it
 * bounds size(t) * size(s) to 245760 RWG pairs (and the near-pair list to
 * 131072 pairs), larger requests return BEMGPU_ERR_ARG.  The first call on a
 * device does that device's set-up (the array's device address, and the
 * quadrature tables if no fill ran there yet): make it before any stream
 * capture.  Each call builds the near-pair list in host memory, copies it to
 * the scratch on `stream` and synchronises `stream` before it returns (dZ is
 * then written).  All calls share the array: calls from one process take
 * turns, but calls that overlap on the GPU (other processes' are separate)
 * would race, so serialise them. */
int bemgpu_zts_noalloc(bemgpu_ctx_t ctx, bemgpu_tree_t t, bemgpu_tree_t s, const bemgpu_green_t *g,
                       const bemgpu_options_t *opt, void *dZ, int64_t ldz, void *stream);

/* ---- dense complex algebra ---- */
/* C (m x n) = A (m x k) B (k x n) [+ C when accumulate], complex64 device
 * matrices, column-major with interleaved (re, im).  The product of the
 * mixed-precision LU and trace (addproduct -> zgemm, src/util/MatrixOperations.cpp:70-74):
 * engine 1 = tensor cores (bf16x3 split, six products, FP32 accumulate),
 * 2 = FP32 FMA pipes, 0 = the library's choice.  Synchronous. */
int bemgpu_cgemm(bemgpu_ctx_t ctx, int m, int n, int k, const float *dA, int64_t lda, const float *dB, int64_t ldb,
                 float *dC, int64_t ldc, int accumulate, int engine);
/* The refinement residual's product: C (complex128) = A B [+ C] with
 * complex64 A and B; products summed in short FP32 runs, the runs in
 * two-float sums.  engine 1 = tensor cores, 2 = FMA pipes, 0 = choice. */
int bemgpu_cgemm_acc64(bemgpu_ctx_t ctx, int m, int n, int k, const float *dA, int64_t lda, const float *dB,
                       int64_t ldb, double *dC, int64_t ldc, int accumulate, int engine);

/* C (complex128) = A B [+ C] with FP64-class accuracy on the tensor cores:
 * A, B complex128, cut into `slices` (4 or 5) block fixed-point bf16 slices
 * whose products the tensor cores sum exactly per K step; error ~2^(-8 slices)
 * of the K-blocks' largest magnitudes.  The product of the refinement
 * residual and the trace (src/HeatTransfer.cpp:40-58).  Synchronous. */
int bemgpu_zgemm_exact(bemgpu_ctx_t ctx, int m, int n, int k, const double *dA, int64_t lda, const double *dB,
                       int64_t ldb, double *dC, int64_t ldc, int accumulate, int slices);
/* The same with B quantized in place to the 3-slice block fixed point (B is
 * overwritten with the value its slices represent exactly) and A in 5 slices:
 * every slice product up to level 4 is kept (12 products), so C = A B to
 * ~2^-40 of |A||B| for the quantized B.  The refinement uses this form for
 * the residual of its first, complex64-accurate iterate. */
int bemgpu_zgemm_exact_quantized(bemgpu_ctx_t ctx, int m, int n, int k, const double *dA, int64_t lda, double *dB,
                                 int64_t ldb, double *dC, int64_t ldc, int accumulate);

/* ---- per-frequency solve ---- */
/* CalcHeatTransfer: top is the two-body tree (s's RWGs first, then t's),
 * s and t the one-body trees, all over one geometry.  Writes the spectral
 * power Re(S)*(Theta(omega,T1)-Theta(omega,T2)) to *P_out (synchronous). */
int bemgpu_heat_transfer(bemgpu_ctx_t ctx, bemgpu_tree_t top, bemgpu_tree_t s, bemgpu_tree_t t,
                         const bemgpu_solve_req_t *req, const bemgpu_options_t *opt, int precision,
                         double *P_out, bemgpu_solve_info_t *info);

/* Several CalcHeatTransfer requests solved together (no counterpart in the
 * reference, whose task farm solves one per process): request i is
 * (tops[i], ss[i], ts[i], reqs[i]).  The three fills of every request run in
 * one far-pair and one near-pair launch; the complex64 LU panels of requests
 * of equal size (a frequency sweep of one geometry) run in one cooperative
 * launch per block column; the rest is per request.  P_out[i] and infos[i]
 * (infos may be NULL; its ms_fill is the batch's fill time / nreq) equal
 * bemgpu_heat_transfer's for the same request bit for bit, and status[i] is
 * its status.  Returns the first non-zero status (BEMGPU_OK when all
 * succeeded).  At most 64 requests; the device memory it needs is
 * bemgpu_batch_footprint's.  Synchronous. */
int bemgpu_heat_transfer_batch(bemgpu_ctx_t ctx, int nreq, const bemgpu_tree_t *tops, const bemgpu_tree_t *ss,
                               const bemgpu_tree_t *ts, const bemgpu_solve_req_t *reqs, const bemgpu_options_t *opt,
                               int precision, double *P_out, bemgpu_solve_info_t *infos, int *status);
/* Device bytes a batch of nreq equal-size requests needs at most. */
int64_t bemgpu_batch_footprint(int nreq, int nrwg_s, int nrwg_t, int precision);

/* ---- request farm ----
 * Replaces the reference's MPI task farm (src/transfer-mpi.cpp:25-190: a Master
 * queue of (a, gap, f, T1, T2) jobs, Servants that run CalcHeatTransfer and
 * return one double) inside one process: `lanes` contexts on one device, each
 * driven by its own host thread, take requests from a FIFO, so several solves
 * overlap on the GPU.  Trees are used read-only and must outlive every request
 * that names them; they may belong to any context on the same device.  */
int bemgpu_farm_create(int device, int lanes, bemgpu_farm_t *out);
/* Drops the queued requests (their tickets become BEMGPU_ERR_CANCELLED),
 * waits for the running ones, and frees the lanes. */
int bemgpu_farm_destroy(bemgpu_farm_t farm);
int bemgpu_farm_lanes(bemgpu_farm_t farm);
/* Continuous batching: a lane that takes a request also takes up to
 * max_requests - 1 more queued requests of the same sizes, precision and
 * options (in queue order) and solves them together with
 * bemgpu_heat_transfer_batch, admitted by bemgpu_batch_footprint (a batch
 * over the budget runs its first request alone).  Results are those of the
 * requests solved one by one.  Default 1 (no batching); at most 64. */
int bemgpu_farm_set_batch(bemgpu_farm_t farm, int max_requests);
/* Device bytes the lanes may hold together (admission by footprint); the
 * default is 90 % of the memory free when the farm was created. */
int bemgpu_farm_set_budget(bemgpu_farm_t farm, int64_t bytes);
int64_t bemgpu_farm_budget(bemgpu_farm_t farm);
/* The context of one lane (for bemgpu_prof_* and bemgpu_ctx_launches). */
int bemgpu_farm_lane_ctx(bemgpu_farm_t farm, int lane, bemgpu_ctx_t *ctx);
/* Queues one CalcHeatTransfer request (the arguments of bemgpu_heat_transfer;
 * *req and *opt are copied) and returns its ticket. */
int bemgpu_farm_submit(bemgpu_farm_t farm, bemgpu_tree_t top, bemgpu_tree_t s, bemgpu_tree_t t,
                       const bemgpu_solve_req_t *req, const bemgpu_options_t *opt, int precision,
                       int64_t *ticket);
/* Waits up to timeout_ms (< 0: without limit, 0: not at all) for a request.
 * Returns BEMGPU_PENDING if it has not finished, else its status, exactly as
 * bemgpu_heat_transfer would have returned it, with *P_out and *info written;
 * a finished ticket is collected once.  */
int bemgpu_farm_poll(bemgpu_farm_t farm, int64_t ticket, double timeout_ms, double *P_out,
                     bemgpu_solve_info_t *info);
/* Removes a queued request: BEMGPU_OK (its poll returns BEMGPU_ERR_CANCELLED),
 * BEMGPU_PENDING if it has already started or finished (poll it as usual). */
int bemgpu_farm_cancel(bemgpu_farm_t farm, int64_t ticket);
/* Message of the farm's last failed call or collected failed request. */
const char *bemgpu_farm_last_error(bemgpu_farm_t farm);

#ifdef __cplusplus
}
#endif
#endif /* BEMGPU_H */
