// Internal declarations shared by the bemgpu translation units.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>
#include <map>
#include <mutex>
#include <initializer_list>

#include "../../include/bemgpu.h"

// src/util/MathUtils.h:16,33 (values as the reference defines them)
#define BEM_ONETHIRD 0.33333333333333333333333333333333
#define BEM_ONEOVER4PI 0.079577471545947667884441881686257

// Devices a process may use with this library: per-device state (quadrature
// tables loaded, the allocation-free fill's scratch address) lives in arrays
// of this size, and bemgpu_ctx_create rejects a higher device index.
#define BEM_MAX_DEVICES 64
// Requests of one bemgpu_heat_transfer_batch call at most.
#define BEM_MAX_BATCH 64

// Device-resident per-triangle record of one RWG tree (FP64).  The frame
// (p0, p1, p2 and derived vectors) is that of the triangle's first half-RWG in
// the tree's RWG order: Zts integrates the outer rule over t[0] and the inner
// rule over s[0] (src/Impedance.cpp:283, 156, 196), and the analytic terms use
// s[0] / t[0] (src/Impedance.cpp:196-204, 264-265, 308).
struct TriRec {
  double p0[3], p1[3], p2[3];
  double v01[3], v12[3], v20[3], v02[3];
  double n[3], m01[3], m12[3], m20[3];
  double nv01i, nv12i, nv20i, Ai, elen0;
  double c[3];        // centroid, ((p1+p2)+p3)*ONETHIRD in the triangle's own vertex order
  double emax;        // longest of the triangle's three edges
  double hp0[3][3];   // free vertex p0 of each half-RWG
  double helen[3];    // RWG edge length of each half
  int vid[3];         // vertex ids (vertex-sharing test)
  int gid;            // triangle id in the geometry
  int nh;             // number of half-RWGs on this triangle in this tree (1..3)
  int hrwg[3];        // RWG index (row/column pair of the matrix)
  int hneg[3];        // 0 for the positive half, 1 for the negative half
  int pad;
};

// A (test, source) near pair: shares at least one vertex, or is the same triangle.
struct NearPair {
  int t, s;      // local triangle indices in the two trees
  int same;      // 1 if the same triangle
  int pad;
};

struct bemgpu_geom_s;

struct bemgpu_tree_s {
  bemgpu_ctx_s *ctx = nullptr;
  bemgpu_geom_s *geom = nullptr;   // kept alive by the tree (reference count)
  int nrwg = 0;
  int ntri = 0;                 // triangles touched by the tree
  std::vector<int> rwg;         // host copy of the table (4*nrwg)
  std::vector<int> tri_gid;     // local triangle -> geometry triangle id
  std::vector<TriRec> host_rec;
  TriRec *d_rec = nullptr;
};

struct NearList {
  NearPair *d = nullptr;
  int64_t n = 0;
};

struct bemgpu_geom_s {
  bemgpu_ctx_s *ctx = nullptr;
  int refs = 1;  // the caller's handle + one per tree; freed at zero
  int nv = 0, nt = 0;
  std::vector<double> xyz;
  std::vector<int> tri;
  std::vector<std::vector<int>> tris_at_vertex;
  // per (t, s) tree pair over this geometry: the near-pair list (device) and
  // the far-pair counts per rule; shared by every context that solves the
  // trees (request-farm lanes), guarded by cache_mu
  std::mutex cache_mu;
  std::map<std::pair<const bemgpu_tree_s *, const bemgpu_tree_s *>, NearList> near_cache;
  std::map<std::pair<const bemgpu_tree_s *, const bemgpu_tree_s *>, std::vector<int64_t>> far_rule_cache;
};

struct bemgpu_ctx_s {
  int refs = 1;  // the caller's handle + one per geometry; torn down at zero
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  std::string last_error;
  std::mutex mu;
  // workspace: one growable device buffer per purpose
  std::map<std::string, std::pair<void *, size_t>> ws;
  cudaEvent_t ev[8];
  int64_t launches = 0;  // kernels launched by this context
  bool tc_ready = false;      // gemm_tc.cu kernels: shared-memory attribute set
  bool ex_ready = false;      // gemm_exact.cu kernels: shared-memory attribute set
  bool perm_ready = false;    // dense.cu perm_from_ipiv_kernel: shared-memory attribute set
  bool tc_err_ready = false;  // tensor-core pipeline error flag zeroed
  bool coop_panel = true;  // LU panels in one cooperative launch (else one launch per column)
  int gemm_engine = 0;   // complex64 LU/solve GEMMs: 0 tensor cores where possible, 2 FMA pipes only
  int acc_engine = 0;    // residual/trace GEMMs with FP64 output: same choices
  int solver = 0;        // mixed path: 0 complex64 with FP64-class escalation, 1 complex64, 2 FP64-class
  // launch shapes chosen by the autotuner (bemgpu_ctx_set_tuning); the
  // defaults are the measured best on the N = 7680 icosphere workload
  struct Tuning {
    int near_minb = 2;   // CTAs per SM of the double-float near-pair kernel's register budget (2, 3, 4)
    int far_rows = 4;    // warps per CTA of the far-pair kernel (1, 2, 4, 8)
    int raster = 8;      // M-tiles per rasterization band of the tensor-core products (1..64)
    int panel_ctas = 0;  // CTAs of a cooperative LU panel at most (0: one per SM)
    int near_sync = 1;   // double-float near-pair CTAs barrier after each pair couple (0, 1)
    int near_grid = 16;  // CTAs per SM in the near-pair launch's grid at most (1..64)
    int ex_wide = 1;     // exact products with level-3/4 work on 128 x 128 tiles: 0 never, 1 large grids, 2 always
    int lu_super = 1;    // complex64 LU panels in pairs, trailing updates of K = 256 (0, 1)
  } tune;
  double escalate_tol = 1e-6;  // complex64 refinement error estimate above which the solve escalates
  double fallback_tol = 1e-6;  // FP64-class error estimate above which mode 0 re-solves on the FP64 path
  // live kernel statistics
  bool prof = false;
  struct ProfRec {
    int kind;
    cudaEvent_t a, b;
    double flops, bytes;
    double tensor;  // bf16 tensor-core flops executed (slice products x 8 m n k), 0 off the tensor pipe
  };
  std::vector<ProfRec> prof_recs;
  std::vector<cudaEvent_t> ev_pool;
  size_t ev_used = 0;
};

// Records CUDA events around the launches in its scope when profiling is on.
struct ProfScope {
  bemgpu_ctx_s *ctx;
  int kind;
  cudaStream_t st;
  double flops, bytes;
  double tensor = 0.0;  // set by tensor-core products: bf16 flops executed
  cudaEvent_t a = nullptr;
  ProfScope(bemgpu_ctx_s *c, int k, cudaStream_t s, double f, double b);
  ~ProfScope();
};

// Device bytes of an exact-product operand (bem_exact_prep) and of the bf16x3
// slice planes of a complex64 tensor-core product (bem_cgemm_tc).
size_t bem_exact_operand_bytes(bool is_a, int rows, int k, int slices);
void bem_cgemm_tc_bytes(int m, int n, int k, size_t &a_bytes, size_t &b_bytes);
// Frees one named workspace buffer (after synchronising the context stream).
void bem_workspace_release(bemgpu_ctx_s *ctx, const std::string &name);
// Bytes of workspace the context holds.
size_t bem_workspace_bytes(const bemgpu_ctx_s *ctx);

// Sets ctx->last_error and returns code.
int bem_fail(bemgpu_ctx_s *ctx, int code, const char *fmt, ...);
// One line to stderr when the environment variable BEMGPU_TRACE is set to a
// non-empty value other than "0" (the solver's decisions: refinement steps,
// escalations); nothing otherwise.
void bem_trace(const char *fmt, ...);
// Returns a device buffer of at least `bytes` for `name` (grown on demand).
// Device memory of destroyed trees and geometries, freed in batches after a
// device synchronisation (context.cu).
void bem_defer_free(int device, void *p, size_t bytes);
void bem_flush_deferred_frees();
size_t bem_deferred_free_count();
void *bem_workspace(bemgpu_ctx_s *ctx, const std::string &name, size_t bytes);
// Near pairs of (t, s) built on the host (no device memory touched).
void bem_build_near_pairs(const bemgpu_tree_s *t, const bemgpu_tree_s *s, std::vector<NearPair> &pairs);
// Near-pair list of (t, s), built on the host once and cached on the device.
const NearList *bem_near_list(bemgpu_ctx_s *ctx, const bemgpu_tree_s *t, const bemgpu_tree_s *s);
// Far-pair counts per rule (6, 10, 15, 21, 36 points) of (t, s), classified on
// the host with the kernel's test; cached.  Used for algorithmic flop counts.
const int64_t *bem_far_rule_counts(bemgpu_ctx_s *ctx, const bemgpu_tree_s *t, const bemgpu_tree_s *s,
                                   const bemgpu_options_t *opt);

// Algorithmic work per unit (frozen counting convention: real +,-,*,/ = 1 flop,
// complex*complex = 6, complex+complex = 2, real*complex = 2; sqrt/exp/sincos/
// log/atan2 counted apart and not included).
inline double bem_far_pair_flops(int P) { return P * (148.0 * P + 324.0) + 9.0 * 26.0; }
inline double bem_near_pair_flops(bool neighbour) { return 105.0 * (91.0 * 158.0 + 200.0 + 324.0) + (neighbour ? 45.0 * 80.0 : 0.0); }
constexpr double BEM_HALFPAIR_BYTES_FP64 = 32.0;   // (cL, cK) complex128 per half-RWG pair

#define BEM_CUDA_TRY(ctx, call)                                                               \
  do {                                                                                        \
    cudaError_t e_ = (call);                                                                  \
    if (e_ != cudaSuccess)                                                                    \
      return bem_fail((ctx), BEMGPU_ERR_CUDA, "%s:%d %s: %s", __FILE__, __LINE__, #call,       \
                      cudaGetErrorString(e_));                                                \
  } while (0)

// ---- fill (fill.cu) ----
// Half-pair accumulator block for one RWG pair (i, j): four (cL, cK) complex
// values, one per (test half a, source half b), a,b in {pos, neg}.
struct HalfPairBlock {
  double v[16];  // [a*2+b] -> {cL.re, cL.im, cK.re, cK.im}
};

// Computes every triangle pair of (t, s) with one Green's function and writes
// the per-half-pair products into H (ntr x nsr blocks, index j*ntr+i).
// precision BEMGPU_PREC_MIXED integrates pairs farther apart than 3 edge lengths in FP32.
// One Zts fill of a group (bem_fill_group): tree pair, Green's function,
// half-pair blocks out; near/far pair counts written back.
struct FillJob {
  const bemgpu_tree_s *t, *s;
  bemgpu_green_t g;
  HalfPairBlock *H;
  int64_t near, far;
};
// Several fills in one far-pair and one near-pair launch (the three Zts of a
// solve, or of a batch of solves).
int bem_fill_group(bemgpu_ctx_s *ctx, FillJob *jobs, int njobs, const bemgpu_options_t *opt, int precision,
                   cudaStream_t stream);
int bem_fill_pairs(bemgpu_ctx_s *ctx, const bemgpu_tree_s *t, const bemgpu_tree_s *s,
                   const bemgpu_green_t *g, const bemgpu_options_t *opt, int precision, HalfPairBlock *H,
                   cudaStream_t stream, int64_t *n_near, int64_t *n_far);
// Z (complex128, column-major, ld) = gather of one H with g's Zeps/Zmu.
int bem_gather_z(bemgpu_ctx_s *ctx, const HalfPairBlock *H, int ntr, int nsr, const bemgpu_green_t *g,
                 double *Z, int64_t ld, cudaStream_t stream, bool df = false);
// W = gather(Hext, gext) (+ gather(Hint1, g1) on the s block, + gather(Hint2, g2) on the t block),
// G1 = gather(Hint1, g1), G2 = gather(Hint2, g2).
int bem_gather_w(bemgpu_ctx_s *ctx, const HalfPairBlock *Hext, const HalfPairBlock *H1,
                 const HalfPairBlock *H2, int ns, int nt, const bemgpu_green_t *gext,
                 const bemgpu_green_t *g1, const bemgpu_green_t *g2, double *W, int64_t ldw, double *G1,
                 int64_t ld1, double *G2, int64_t ld2, cudaStream_t stream, bool df = false);

// ---- dense complex linear algebra (dense.cu) ----
// In-place LU with partial pivoting of the n x n complex128 column-major A.
int bem_zgetrf(bemgpu_ctx_s *ctx, double *A, int64_t lda, int n, int *d_ipiv, int *d_info,
               cudaStream_t stream);
// B (n x nrhs) <- A^{-1} B using the LU factors and pivots of bem_zgetrf.
int bem_zgetrs(bemgpu_ctx_s *ctx, const double *A, int64_t lda, int n, const int *d_ipiv, double *B,
               int64_t ldb, int nrhs, cudaStream_t stream);
// FP64-class LU and solve on the tensor cores: FP64 panels and diagonal
// blocks, every trailing / off-diagonal update a 5-slice exact product.
int bem_zgetrf_exact(bemgpu_ctx_s *ctx, double *A, int64_t lda, int n, int *d_ipiv, int *d_info,
                     cudaStream_t stream);
int bem_zgetrs_exact(bemgpu_ctx_s *ctx, const double *A, int64_t lda, int n, const int *d_ipiv, double *B,
                     int64_t ldb, int nrhs, cudaStream_t stream);
// complex64 versions (mixed path).
int bem_cgetrf(bemgpu_ctx_s *ctx, float *A, int64_t lda, int n, int *d_ipiv, int *d_info, cudaStream_t stream);
// The same for nb matrices A + i strideA (pivots d_ipiv + i n, info d_info + i),
// their panels factored together in one cooperative launch.
int bem_cgetrf_batch(bemgpu_ctx_s *ctx, float *A, int64_t strideA, int nb, int64_t lda, int n, int *d_ipiv,
                     int *d_info, cudaStream_t stream);
int bem_cgetrs(bemgpu_ctx_s *ctx, const float *A, int64_t lda, int n, const int *d_ipiv, float *B, int64_t ldb,
               int nrhs, cudaStream_t stream);
// L^{-1} (unit lower) and U^{-1} (upper) of a packed complex64 LU (n x n,
// leading dimension ld), each stored dense (n x n, zeros in the other triangle).
int bem_ctri_inverses(bemgpu_ctx_s *ctx, const float *LU, int64_t ld, int n, float *Linv, float *Uinv,
                      cudaStream_t st);
// B <- U^{-1} L^{-1} P B with the explicit inverses (tmp: n x nrhs complex64).
int bem_capply_inverse_identity(bemgpu_ctx_s *ctx, const float *Linv, const float *Uinv, int n, const int *d_ipiv,
                                int row0, float *B, int64_t ldb, int nrhs, float *tmp, cudaStream_t st);
int bem_capply_inverse(bemgpu_ctx_s *ctx, const float *Linv, const float *Uinv, int n, const int *d_ipiv, float *B,
                       int64_t ldb, int nrhs, float *tmp, cudaStream_t st);
// complex64 GEMM: tensor cores where the shape allows (gemm_tc.cu), else FMA pipes.
int bem_cgemm(bemgpu_ctx_s *ctx, int kind, char opA, int m, int n, int k, const float alpha[2], const float *A,
              int64_t lda, const float *B, int64_t ldb, const float beta[2], float *C, int64_t ldc,
              cudaStream_t stream);
// Tensor-core complex64 GEMM: C (+)= sign * A B (A m x k, B k x n, column-major).
enum { TC_OUT_F32 = 0, TC_OUT_F64 = 1, TC_OUT_F64_COMP = 2 };
// tri: 0 general A, 1 lower-triangular A, 2 upper-triangular A (complex, square
// m = k; the zero triangle is skipped, F32 and F64 outputs only).
int bem_cgemm_tc(bemgpu_ctx_s *ctx, int kind, int m, int n, int k, float sign, const float *A, int64_t lda,
                 const float *B, int64_t ldb, void *C, int64_t ldc, int out, int accumulate, cudaStream_t st,
                 int tri = 0);
// The same product on the FP32 FMA pipes (any alpha, beta).
int bem_cgemm_comp64_fma(bemgpu_ctx_s *ctx, int kind, int m, int n, int k, const float alpha[2], const float *A,
                         int64_t lda, const float *B, int64_t ldb, const double beta[2], double *C, int64_t ldc,
                         cudaStream_t stream);
// Operand of the exact complex128 tensor-core GEMM (gemm_exact.cu): block
// fixed-point bf16 slices of A (m x k, role A) or of B (k x n, role B, `rows`
// = n), kept on the device so one slicing serves several products.
struct ExactOperand {
  void *S = nullptr;    // slices * rows_p * kp bf16
  int *aux = nullptr;   // [0] scaling exponent, [8..9] largest magnitude (bits)
  int rows = 0, k = 0, slices = 0;
  int64_t rows_p = 0, kp = 0;
  bool is_a = true;
  bool exact = false;   // B operand replaced by its quantized value (its slices are exact)
};
bool bem_exact_available();
// Slices sign * M (complex128, column-major, leading dimension ld): role A:
// M is rows x k; role B: M is k x rows.  Workspace named by `name`.
// quantize: M itself (role B, sign 1) is overwritten with the value its
// slices represent, so that products with it keep every level of A's slices.
int bem_exact_prep(bemgpu_ctx_s *ctx, const char *name, bool is_a, const double *M, int64_t ld, int rows, int k,
                   double sign, int slices, ExactOperand &op, cudaStream_t st, double *quantize = nullptr);
// C (+)= A B from prepared operands (complex128 C, column-major, ldc).
int bem_exact_gemm(bemgpu_ctx_s *ctx, int kind, const ExactOperand &a, const ExactOperand &b, double *C, int64_t ldc,
                   int accumulate, cudaStream_t st);
// Non-zero when a tensor-core pipeline wait ran out since the last reset (synchronizes).
int bem_tc_error(bemgpu_ctx_s *ctx, bool reset);
// C (complex128) = alpha A B + beta C, complex64 A and B, products summed
// in short FP32 runs and across runs as two-float sums (tensor cores where
// alpha = +-1 and beta = 0 or 1, else FMA pipes).
int bem_cgemm_comp64(bemgpu_ctx_s *ctx, int kind, int m, int n, int k, const float alpha[2], const float *A,
                     int64_t lda, const float *B, int64_t ldb, const double beta[2], double *C, int64_t ldc,
                     cudaStream_t stream);
int bem_cgemm_fma(bemgpu_ctx_s *ctx, int kind, char opA, int m, int n, int k, const float alpha[2], const float *A,
                  int64_t lda, const float *B, int64_t ldb, const float beta[2], float *C, int64_t ldc,
                  cudaStream_t stream);
// C = alpha * op(A) * op(B) + beta * C for complex128 column-major matrices.
// op: 'N' or 'C' (conjugate transpose) for A; 'N' for B.
int bem_zgemm(bemgpu_ctx_s *ctx, int kind, char opA, int m, int n, int k, const double alpha[2], const double *A,
              int64_t lda, const double *B, int64_t ldb, const double beta[2], double *C, int64_t ldc,
              cudaStream_t stream);

// ---- mixed-precision solve (mixed.cu) ----
// W (FP64, n x n, ld n), G1 (ns2 x ns2), G2 ((n-ns2) x (n-ns2)) as filled; writes S = 1/4 Tr(B2^H B1).
// Returns BEM_SOLVE_ON_FP64_PATH, with W, G1 and G2 untouched, when mode 0's
// FP64-class solve stays above ctx->fallback_tol: the caller then solves W
// on the plain FP64 path.
constexpr int BEM_SOLVE_ON_FP64_PATH = 100;
void bem_release_if_short(bemgpu_ctx_s *ctx, size_t need, std::initializer_list<const char *> names);
// The complex64 LU of W already done (a batch's bem_cgetrf_batch): the factors
// in place of fl32(W), the pivots and the zero-pivot info.
struct MixedLU {
  float *W32;
  int *ipiv, *info;
};
int bem_mixed_solve(bemgpu_ctx_s *ctx, double *W, int n, int ns2, const double *G1, const double *G2,
                    cudaStream_t st, double S_out[2], bemgpu_solve_info_t *info, const MixedLU *pre = nullptr);
void bem_c128_to_c64(bemgpu_ctx_s *ctx, const double *W, int n, float *W32, cudaStream_t st);
