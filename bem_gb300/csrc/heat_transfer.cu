// Per-frequency driver: CalcHeatTransfer (src/HeatTransfer.cpp:8-59) on the GPU.
//
//   W = Zext(top,top) + blockdiag(G1, G2)          (fill + gather, one pass)
//   X = W^{-1}[s rows, t cols]                      (LU, then solve with the t
//                                                   columns of the identity; the
//                                                   reference forms the whole inverse)
//   B1 = sym(G1) X,  B2 = X sym(G2)                 (the [s,t] blocks the reference
//                                                   keeps after its two full products)
//   S  = 1/4 sum conj(B2) o B1  = 1/4 Tr(B2^H B1)   (multiply_Adagger_B + trace)
//   P  = Re(S) (Theta(omega,T1) - Theta(omega,T2))
#include "bemgpu_internal.h"

#include <cmath>
#include <cstring>
#include <algorithm>

namespace {

__global__ void sym_kernel(double *G, int64_t ld, int m) {
  // symm, src/util/DenseMatrix.cpp:477-486: G <- G + G^H
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (i >= m || i < j) return;
  double2 *g = reinterpret_cast<double2 *>(G);
  if (i == j) {
    double2 d = g[i + ld * (int64_t)i];
    g[i + ld * (int64_t)i] = make_double2(d.x + d.x, 0.0);
    return;
  }
  const double2 a = g[i + ld * (int64_t)j], b = g[j + ld * (int64_t)i];
  const double2 nij = make_double2(a.x + b.x, a.y - b.y);
  g[i + ld * (int64_t)j] = nij;
  g[j + ld * (int64_t)i] = make_double2(nij.x, -nij.y);
}

__global__ void identity_cols_kernel(double *Y, int64_t ld, int n, int row0, int ncols) {
  // Y (n x ncols) = columns row0..row0+ncols of the n x n identity
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  const int c = blockIdx.y;
  if (r >= n) return;
  reinterpret_cast<double2 *>(Y)[r + ld * (int64_t)c] = make_double2(r == row0 + c ? 1.0 : 0.0, 0.0);
}

constexpr int TR_THREADS = 256;

// Partial sums of conj(B2) o B1 over a column-major (m x n) pair, fixed order.
__global__ void trace_partial_kernel(const double *B1, const double *B2, int64_t ld, int m, int n, double *partial) {
  __shared__ double sr[TR_THREADS], si[TR_THREADS];
  const int64_t total = (int64_t)m * n;
  double ar = 0, ai = 0;
  for (int64_t idx = (int64_t)blockIdx.x * TR_THREADS + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * TR_THREADS) {
    const int64_t r = idx % m, c = idx / m;
    const double2 b1 = reinterpret_cast<const double2 *>(B1)[r + ld * c];
    const double2 b2 = reinterpret_cast<const double2 *>(B2)[r + ld * c];
    ar += b2.x * b1.x + b2.y * b1.y;
    ai += b2.x * b1.y - b2.y * b1.x;
  }
  sr[threadIdx.x] = ar;
  si[threadIdx.x] = ai;
  __syncthreads();
  for (int s = TR_THREADS / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      sr[threadIdx.x] += sr[threadIdx.x + s];
      si[threadIdx.x] += si[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    partial[2 * blockIdx.x] = sr[0];
    partial[2 * blockIdx.x + 1] = si[0];
  }
}

__global__ void trace_final_kernel(const double *partial, int np, double *out) {
  if (threadIdx.x != 0) return;
  double r = 0, i = 0;
  for (int k = 0; k < np; k++) {
    r += partial[2 * k];
    i += partial[2 * k + 1];
  }
  out[0] = 0.25 * r;
  out[1] = 0.25 * i;
}

float elapsed(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0;
  cudaEventElapsedTime(&ms, a, b);
  return ms;
}

}  // namespace

namespace {

// Device bytes of the solve-phase buffers (everything allocated after the
// fill and gather), mirroring the allocation sites in mixed.cu, dense.cu,
// gemm_tc.cu and gemm_exact.cu (mixed path) or below (FP64 path).
// `solver` is the context's mixed-path mode (bemgpu_ctx_set_solver): with 1
// only the complex64 factors, inverses and their bf16x3 slice planes; with 2
// only the FP64-class LU's blocks and operands; with 0 the larger of the two
// stages, because an escalating solve gives the complex64 buffers back before
// it allocates the FP64-class ones (a copy of W, the FP64 fallback's Y, B1,
// B2) when free memory is short (bem_mixed_solve, heat_transfer below).
size_t solve_phase_bytes(int Ns, int Nt, int precision, int solver) {
  const size_t N = (size_t)Ns + Nt, n = 2 * N, ns2 = 2 * (size_t)Ns, nt2 = 2 * (size_t)Nt;
  const size_t nn = n * n, nm = n * nt2, st2 = ns2 * nt2;
  const size_t scratch = 8u << 20;  // LU panel candidates and rows (coop_*), flags, trace partials
  if (precision == BEMGPU_PREC_FP64)
    return 16 * nm + 2 * 16 * st2 + 4 * n + scratch;
  size_t b = 16 * (ns2 * ns2 + nt2 * nt2) + 3 * 16 * nm + 3 * 16 * st2;
  b += 4 * n + 16 * (((ns2 + 31) / 32) * ((nt2 + 31) / 32)) + 1024;
  // exact operands: -W, H1, H2 (5 slices), the iterate Y, the trace's X and X^H
  b += bem_exact_operand_bytes(true, (int)n, (int)n, 5) + bem_exact_operand_bytes(true, (int)ns2, (int)ns2, 5) +
       bem_exact_operand_bytes(true, (int)nt2, (int)nt2, 5) + bem_exact_operand_bytes(false, (int)nt2, (int)n, 5) +
       bem_exact_operand_bytes(false, (int)nt2, (int)ns2, 5) + bem_exact_operand_bytes(false, (int)ns2, (int)nt2, 5);
  // complex64 stage: W, L^-1, U^-1, two n x nt2 right-hand sides, and the
  // bf16x3 slice planes (the largest product is the application of L^-1 /
  // U^-1 to the n x nt2 right-hand sides; the triangular inverses' halves are
  // smaller) with the triangular-inverse scratch
  size_t c64 = 3 * 8 * nn + 2 * 8 * nm;
  {
    size_t a1, b1, a2, b2;
    bem_cgemm_tc_bytes((int)n, (int)nt2, (int)n, a1, b1);
    bem_cgemm_tc_bytes((int)(n / 2 + 64), (int)(n / 2 + 64), (int)(n / 2 + 64), a2, b2);
    c64 += std::max(a1, a2) + std::max(b1, b2) + 8 * (n / 2 + 64) * (n / 2 + 64);
  }
  // FP64-class stage: the inverted 512 x 512 diagonal blocks of L and U and
  // the sliced operands of its K = 512 exact updates (an n x 512 panel, a
  // 512 x n row block); escalating from complex64 it also factors a copy of
  // W and keeps room for the FP64 fallback's Y, B1, B2
  size_t f64 = 2 * 16 * n * 512 + bem_exact_operand_bytes(true, (int)n, 512, 5) +
               bem_exact_operand_bytes(false, (int)n, 512, 5);
  if (solver == 0) f64 += 16 * nn + 16 * nm + 2 * 16 * st2;
  b += solver == 1 ? c64 : solver == 2 ? f64 : std::max(c64, f64);
  b += scratch;
  return b;
}

size_t fill_phase_bytes(int Ns, int Nt) {
  const size_t N = (size_t)Ns + Nt, n = 2 * N, ns2 = 2 * (size_t)Ns, nt2 = 2 * (size_t)Nt;
  return sizeof(HalfPairBlock) * (N * N + (size_t)Ns * Ns + (size_t)Nt * Nt) + 16 * (n * n + ns2 * ns2 + nt2 * nt2);
}

}  // namespace

// The plain FP64 path after the fill: W = P L U by the FP64 LU, Y = W^-1 E_t,
// symm of G1, G2 in place, the two products and the trace.  Records ev[2..4]
// (after the LU, the solve, the trace).
static int fp64_path_solve(bemgpu_ctx_s *ctx, double *W, int n, int ns2, double *G1, double *G2, cudaStream_t st,
                           double S[2], cudaEvent_t *ev) {
  const int nt2 = n - ns2;
  const double one_c[2] = {1.0, 0.0};
  double *Y = (double *)bem_workspace(ctx, "Y", sizeof(double) * 2 * (size_t)n * nt2);
  double *B1 = (double *)bem_workspace(ctx, "B1", sizeof(double) * 2 * (size_t)ns2 * nt2);
  double *B2 = (double *)bem_workspace(ctx, "B2", sizeof(double) * 2 * (size_t)ns2 * nt2);
  int *ipiv = (int *)bem_workspace(ctx, "ipiv", sizeof(int) * (size_t)n);
  int *dinfo = (int *)bem_workspace(ctx, "info", sizeof(int));
  const int TRB = 1024;
  double *partial = (double *)bem_workspace(ctx, "trace_partial", sizeof(double) * 2 * TRB + 16);
  if (!Y || !B1 || !B2 || !ipiv || !dinfo || !partial)
    return bem_fail(ctx, BEMGPU_ERR_OOM, "heat_transfer: workspace allocation failed (n=%d)", n);
  double *dS = partial + 2 * TRB;
  int rc = bem_zgetrf(ctx, W, n, n, ipiv, dinfo, st);
  if (rc) return rc;
  cudaEventRecord(ev[2], st);
  {
    ProfScope ps(ctx, BEMGPU_K_SOLVE_GEMM, st, 0.0, 16.0 * n * nt2);
    identity_cols_kernel<<<dim3((n + 255) / 256, nt2), 256, 0, st>>>(Y, n, n, ns2, nt2);
    ctx->launches++;
  }
  rc = bem_zgetrs(ctx, W, n, n, ipiv, Y, n, nt2, st);
  if (rc) return rc;
  cudaEventRecord(ev[3], st);
  {
    ProfScope ps(ctx, BEMGPU_K_TRACE, st, 2.0 * ((double)ns2 * ns2 + (double)nt2 * nt2),
                 32.0 * ((double)ns2 * ns2 + (double)nt2 * nt2));
    sym_kernel<<<dim3((ns2 + 255) / 256, ns2), 256, 0, st>>>(G1, ns2, ns2);
    ctx->launches++;
    sym_kernel<<<dim3((nt2 + 255) / 256, nt2), 256, 0, st>>>(G2, nt2, nt2);
    ctx->launches++;
  }
  const double zero_c[2] = {0.0, 0.0};
  rc = bem_zgemm(ctx, BEMGPU_K_TRACE, 'N', ns2, nt2, ns2, one_c, G1, ns2, Y, n, zero_c, B1, ns2, st);
  if (!rc) rc = bem_zgemm(ctx, BEMGPU_K_TRACE, 'N', ns2, nt2, nt2, one_c, Y, n, G2, nt2, zero_c, B2, ns2, st);
  if (rc) return rc;
  {
    ProfScope ps(ctx, BEMGPU_K_TRACE, st, 8.0 * ns2 * nt2, 32.0 * ns2 * nt2);
    trace_partial_kernel<<<TRB, TR_THREADS, 0, st>>>(B1, B2, ns2, ns2, nt2, partial);
    ctx->launches++;
    trace_final_kernel<<<1, 32, 0, st>>>(partial, TRB, dS);
    ctx->launches++;
  }
  cudaEventRecord(ev[4], st);
  int hinfo = 0;
  BEM_CUDA_TRY(ctx, cudaMemcpyAsync(S, dS, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
  BEM_CUDA_TRY(ctx, cudaMemcpyAsync(&hinfo, dinfo, sizeof(int), cudaMemcpyDeviceToHost, st));
  BEM_CUDA_TRY(ctx, cudaStreamSynchronize(st));
  if (bem_tc_error(ctx, true))
    return bem_fail(ctx, BEMGPU_ERR_TIMEOUT, "heat_transfer: a grid-barrier or pipeline wait ran out");
  if (hinfo != 0) return bem_fail(ctx, BEMGPU_ERR_SINGULAR, "heat_transfer: zero pivot at column %d", hinfo);
  return BEMGPU_OK;
}

extern "C" int64_t bemgpu_solve_footprint(int nrwg_s, int nrwg_t, int precision) {
  if (nrwg_s < 1 || nrwg_t < 1) return BEMGPU_ERR_ARG;
  return (int64_t)(fill_phase_bytes(nrwg_s, nrwg_t) + solve_phase_bytes(nrwg_s, nrwg_t, precision, 0));
}

extern "C" int64_t bemgpu_ctx_solve_footprint(bemgpu_ctx_t ctx, int nrwg_s, int nrwg_t, int precision) {
  if (!ctx || nrwg_s < 1 || nrwg_t < 1) return BEMGPU_ERR_ARG;
  return (int64_t)(fill_phase_bytes(nrwg_s, nrwg_t) + solve_phase_bytes(nrwg_s, nrwg_t, precision, ctx->solver));
}

namespace {

// One request's sizes and Green's functions (GreensFunction::init of the
// exterior and the two bodies, src/HeatTransfer.cpp:10-24).
struct ReqSetup {
  int Ns, Nt, N, n, ns2, nt2;
  double omega;
  bemgpu_green_t gext, g1, g2;
};

int setup_request(bemgpu_ctx_s *ctx, const bemgpu_tree_s *top, const bemgpu_tree_s *s, const bemgpu_tree_s *t,
                  const bemgpu_solve_req_t *req, int precision, ReqSetup &r) {
  if (!top || !s || !t || !req) return bem_fail(ctx, BEMGPU_ERR_ARG, "heat_transfer: null argument");
  if (top->geom != s->geom || top->geom != t->geom)
    return bem_fail(ctx, BEMGPU_ERR_ARG, "heat_transfer: trees must share one geometry");
  if (top->geom->ctx->device != ctx->device)
    return bem_fail(ctx, BEMGPU_ERR_ARG, "heat_transfer: the trees live on device %d, the context on %d",
                    top->geom->ctx->device, ctx->device);
  if (top->nrwg != s->nrwg + t->nrwg)
    return bem_fail(ctx, BEMGPU_ERR_ARG, "heat_transfer: size(top) != size(s) + size(t)");
  if (precision != BEMGPU_PREC_FP64 && precision != BEMGPU_PREC_MIXED && precision != BEMGPU_PREC_MIXED_LA)
    return bem_fail(ctx, BEMGPU_ERR_ARG, "heat_transfer: unknown precision %d", precision);
  r.Ns = s->nrwg;
  r.Nt = t->nrwg;
  r.N = r.Ns + r.Nt;
  r.n = 2 * r.N;
  r.ns2 = 2 * r.Ns;
  r.nt2 = 2 * r.Nt;
  r.omega = bemgpu_dimensionless_omega(req->a, req->eV);
  const double om[2] = {r.omega, 0.0}, one_c[2] = {1.0, 0.0};
  bemgpu_green_init(one_c, one_c, om, 1, &r.gext);
  bemgpu_green_init(req->eps1, req->mu1, om, 0, &r.g1);
  bemgpu_green_init(req->eps2, req->mu2, om, 0, &r.g2);
  return BEMGPU_OK;
}

// The solve after W, G1, G2 are gathered: the mixed path (pre: its complex64
// LU done by a batch) or the plain FP64 path, then P.  ev[1..5] are used.
int finish_request(bemgpu_ctx_s *ctx, const ReqSetup &r, const bemgpu_solve_req_t *req, double *W, double *G1,
                   double *G2, int precision, cudaStream_t st, const MixedLU *pre, double *P_out,
                   bemgpu_solve_info_t *info) {
  cudaEvent_t *ev = ctx->ev;
  const int n = r.n, ns2 = r.ns2, nt2 = r.nt2;
  if (precision != BEMGPU_PREC_FP64) {
    bemgpu_solve_info_t mi;
    memset(&mi, 0, sizeof mi);
    double S[2] = {0, 0};
    int rc = bem_mixed_solve(ctx, W, n, ns2, G1, G2, st, S, &mi, pre);
    if (rc == BEM_SOLVE_ON_FP64_PATH) {
      // the FP64-class refinement stalled above the fallback tolerance: W is
      // as filled, solve it on the plain FP64 path (FP64 LU, no refinement);
      // the mixed stages' buffers go back first if its Y, B1, B2 would not fit
      bem_release_if_short(ctx, 16 * (size_t)n * nt2 + 2 * 16 * (size_t)ns2 * nt2,
                           {"m_Wlu", "m_W32", "m_R32", "m_Linv", "m_Uinv", "m_T32", "tc_A", "tc_B", "tri_tmp",
                            "ex_W", "ex_Y", "ex_X", "ex_XH", "ex_xm_A", "ex_xm_B"});
      cudaEventRecord(ev[1], st);
      rc = fp64_path_solve(ctx, W, n, ns2, G1, G2, st, S, ev);
      if (rc) return rc;
      mi.solver = 3;
      mi.err_est = 0.0;
      mi.ms_lu = elapsed(ev[1], ev[2]);
      mi.ms_solve = elapsed(ev[2], ev[3]);
      mi.ms_trace = elapsed(ev[3], ev[4]);
    }
    if (rc && rc != BEMGPU_ERR_NO_CONVERGE) return rc;
    *P_out = S[0] * (bemgpu_theta(r.omega, req->T1) - bemgpu_theta(r.omega, req->T2));
    if (info) {
      const double ms_fill = info->ms_fill;
      const int64_t pn = info->pairs_near, pf = info->pairs_far_fp64;
      *info = mi;
      info->ms_fill = ms_fill;
      info->pairs_near = pn;
      info->pairs_far_fp64 = pf;
      info->S_re = S[0];
      info->S_im = S[1];
    }
    return rc;
  }
  double S[2];
  cudaEventRecord(ev[1], st);
  int rc = fp64_path_solve(ctx, W, n, ns2, G1, G2, st, S, ev);
  if (rc) return rc;
  *P_out = S[0] * (bemgpu_theta(r.omega, req->T1) - bemgpu_theta(r.omega, req->T2));
  if (info) {
    info->ms_lu = elapsed(ev[1], ev[2]);
    info->ms_solve = elapsed(ev[2], ev[3]);
    info->ms_trace = elapsed(ev[3], ev[4]);
    info->S_re = S[0];
    info->S_im = S[1];
  }
  return BEMGPU_OK;
}

// Gives back the named half-pair blocks when the solve phase (`need` bytes)
// would not fit beside what the context holds (large solves).
void release_fill_if_short(bemgpu_ctx_s *ctx, size_t need, size_t fill, std::initializer_list<const char *> names) {
  size_t fr = 0, tot = 0;
  cudaMemGetInfo(&fr, &tot);
  const size_t held = bem_workspace_bytes(ctx);
  // solve-phase bytes not yet held (what the context holds beyond the fill
  // buffers is solve-phase workspace of an earlier request)
  const size_t missing = need - std::min(need, held > fill ? held - fill : (size_t)0);
  if ((double)fr < 1.05 * (double)missing + (double)(1u << 30))
    for (const char *nm : names) bem_workspace_release(ctx, nm);
}

}  // namespace

extern "C" int bemgpu_heat_transfer(bemgpu_ctx_t ctx, bemgpu_tree_t top, bemgpu_tree_t s, bemgpu_tree_t t,
                                    const bemgpu_solve_req_t *req, const bemgpu_options_t *opt, int precision,
                                    double *P_out, bemgpu_solve_info_t *info) {
  if (!ctx || !P_out) return bem_fail(ctx, BEMGPU_ERR_ARG, "heat_transfer: null argument");
  ReqSetup r;
  int rc = setup_request(ctx, top, s, t, req, precision, r);
  if (rc) return rc;
  bemgpu_options_t o;
  if (opt) o = *opt; else bemgpu_options_default(&o);
  std::lock_guard<std::mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  cudaStream_t st = ctx->stream;
  const int N = r.N, Ns = r.Ns, Nt = r.Nt, n = r.n, ns2 = r.ns2, nt2 = r.nt2;
  HalfPairBlock *He = (HalfPairBlock *)bem_workspace(ctx, "Hext", sizeof(HalfPairBlock) * (size_t)N * N);
  HalfPairBlock *H1 = (HalfPairBlock *)bem_workspace(ctx, "Hint1", sizeof(HalfPairBlock) * (size_t)Ns * Ns);
  HalfPairBlock *H2 = (HalfPairBlock *)bem_workspace(ctx, "Hint2", sizeof(HalfPairBlock) * (size_t)Nt * Nt);
  double *W = (double *)bem_workspace(ctx, "W", sizeof(double) * 2 * (size_t)n * n);
  double *G1 = (double *)bem_workspace(ctx, "G1", sizeof(double) * 2 * (size_t)ns2 * ns2);
  double *G2 = (double *)bem_workspace(ctx, "G2", sizeof(double) * 2 * (size_t)nt2 * nt2);
  if (!He || !H1 || !H2 || !W || !G1 || !G2)
    return bem_fail(ctx, BEMGPU_ERR_OOM, "heat_transfer: workspace allocation failed (n=%d)", n);
  cudaEvent_t *ev = ctx->ev;
  cudaEventRecord(ev[0], st);
  // the three Zts of CalcHeatTransfer (src/HeatTransfer.cpp:26-29) in one
  // far-pair and one near-pair launch
  FillJob jobs[3] = {{top, top, r.gext, He, 0, 0}, {s, s, r.g1, H1, 0, 0}, {t, t, r.g2, H2, 0, 0}};
  rc = bem_fill_group(ctx, jobs, 3, &o, precision, st);
  if (!rc)
    rc = bem_gather_w(ctx, He, H1, H2, Ns, Nt, &r.gext, &r.g1, &r.g2, W, n, G1, ns2, G2, nt2, st,
                      precision == BEMGPU_PREC_MIXED_LA);
  if (rc) return rc;
  cudaEventRecord(ev[7], st);
  // The half-pair blocks are dead once W, G1, G2 are gathered.  When the
  // solve phase would not fit beside them, give them back first (large
  // solves); otherwise keep them for the next request of this size.
  release_fill_if_short(ctx, solve_phase_bytes(Ns, Nt, precision, ctx->solver), fill_phase_bytes(Ns, Nt),
                        {"Hext", "Hint1", "Hint2"});
  bemgpu_solve_info_t mine;
  bemgpu_solve_info_t *pi = info ? info : &mine;
  memset(pi, 0, sizeof *pi);
  pi->pairs_near = jobs[0].near + jobs[1].near + jobs[2].near;
  pi->pairs_far_fp64 = jobs[0].far + jobs[1].far + jobs[2].far;
  rc = finish_request(ctx, r, req, W, G1, G2, precision, st, nullptr, P_out, pi);
  pi->ms_fill = elapsed(ev[0], ev[7]);  // the solve has synchronised the stream
  return rc;
}

extern "C" int64_t bemgpu_batch_footprint(int nreq, int nrwg_s, int nrwg_t, int precision) {
  if (nreq < 1 || nrwg_s < 1 || nrwg_t < 1) return BEMGPU_ERR_ARG;
  const size_t n = 2 * ((size_t)nrwg_s + nrwg_t);
  // every request's fill blocks and matrices, one solve phase, and the
  // complex64 factors of the batched LU beyond the one the solve holds
  size_t b = (size_t)nreq * fill_phase_bytes(nrwg_s, nrwg_t) + solve_phase_bytes(nrwg_s, nrwg_t, precision, 0);
  if (precision != BEMGPU_PREC_FP64) b += (size_t)nreq * (8 * n * n + 4 * n + 16);
  return (int64_t)b;
}

extern "C" int bemgpu_heat_transfer_batch(bemgpu_ctx_t ctx, int nreq, const bemgpu_tree_t *tops,
                                          const bemgpu_tree_t *ss, const bemgpu_tree_t *ts,
                                          const bemgpu_solve_req_t *reqs, const bemgpu_options_t *opt, int precision,
                                          double *P_out, bemgpu_solve_info_t *infos, int *status) {
  if (!ctx || nreq < 1 || !tops || !ss || !ts || !reqs || !P_out || !status)
    return bem_fail(ctx, BEMGPU_ERR_ARG, "heat_transfer_batch: null argument or empty batch");
  // until a request has its own outcome, every status is the batch's
  auto fail_all = [&](int rc) {
    for (int i = 0; i < nreq; i++) status[i] = rc;
    return rc;
  };
  if (nreq > BEM_MAX_BATCH)
    return fail_all(bem_fail(ctx, BEMGPU_ERR_ARG, "heat_transfer_batch: %d requests, at most %d", nreq, BEM_MAX_BATCH));
  std::vector<ReqSetup> r(nreq);
  for (int i = 0; i < nreq; i++) {
    const int rc = setup_request(ctx, tops[i], ss[i], ts[i], &reqs[i], precision, r[i]);
    if (rc) return fail_all(rc);
  }
  bemgpu_options_t o;
  if (opt) o = *opt; else bemgpu_options_default(&o);
  std::lock_guard<std::mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  cudaStream_t st = ctx->stream;
  // every request's half-pair blocks and matrices, side by side
  std::vector<size_t> hoff(nreq + 1, 0), moff(nreq + 1, 0);
  bool same = true;
  for (int i = 0; i < nreq; i++) {
    const size_t N = r[i].N, Ns = r[i].Ns, Nt = r[i].Nt;
    hoff[i + 1] = hoff[i] + N * N + Ns * Ns + Nt * Nt;
    moff[i + 1] = moff[i] + 2 * ((size_t)r[i].n * r[i].n + (size_t)r[i].ns2 * r[i].ns2 + (size_t)r[i].nt2 * r[i].nt2);
    same = same && r[i].Ns == r[0].Ns && r[i].Nt == r[0].Nt;
  }
  HalfPairBlock *H = (HalfPairBlock *)bem_workspace(ctx, "bH", sizeof(HalfPairBlock) * hoff[nreq]);
  double *M = (double *)bem_workspace(ctx, "bM", sizeof(double) * moff[nreq]);
  if (!H || !M) return fail_all(bem_fail(ctx, BEMGPU_ERR_OOM, "heat_transfer_batch: workspace allocation failed"));
  std::vector<FillJob> jobs(3 * (size_t)nreq);
  std::vector<double *> W(nreq), G1(nreq), G2(nreq);
  for (int i = 0; i < nreq; i++) {
    const size_t N = r[i].N, Ns = r[i].Ns;
    HalfPairBlock *He = H + hoff[i], *H1 = He + N * N, *H2 = H1 + Ns * Ns;
    jobs[3 * i] = {tops[i], tops[i], r[i].gext, He, 0, 0};
    jobs[3 * i + 1] = {ss[i], ss[i], r[i].g1, H1, 0, 0};
    jobs[3 * i + 2] = {ts[i], ts[i], r[i].g2, H2, 0, 0};
    W[i] = M + moff[i];
    G1[i] = W[i] + 2 * (size_t)r[i].n * r[i].n;
    G2[i] = G1[i] + 2 * (size_t)r[i].ns2 * r[i].ns2;
  }
  cudaEvent_t *ev = ctx->ev;
  cudaEventRecord(ev[0], st);
  // every request's three Zts in one far-pair and one near-pair launch
  int rc = bem_fill_group(ctx, jobs.data(), 3 * nreq, &o, precision, st);
  for (int i = 0; i < nreq && !rc; i++) {
    const HalfPairBlock *He = jobs[3 * i].H, *H1 = jobs[3 * i + 1].H, *H2 = jobs[3 * i + 2].H;
    rc = bem_gather_w(ctx, He, H1, H2, r[i].Ns, r[i].Nt, &r[i].gext, &r[i].g1, &r[i].g2, W[i], r[i].n, G1[i],
                      r[i].ns2, G2[i], r[i].nt2, st, precision == BEMGPU_PREC_MIXED_LA);
  }
  if (rc) return fail_all(rc);
  cudaEventRecord(ev[7], st);
  BEM_CUDA_TRY(ctx, cudaEventSynchronize(ev[7]));
  const float fill_ms = elapsed(ev[0], ev[7]);
  {
    size_t need = 0, fill = 0;
    for (int i = 0; i < nreq; i++) {
      need = std::max(need, solve_phase_bytes(r[i].Ns, r[i].Nt, precision, ctx->solver));
      fill += fill_phase_bytes(r[i].Ns, r[i].Nt);
    }
    release_fill_if_short(ctx, need, fill, {"bH"});
  }
  // the complex64 LU of equal-size requests together: their panels in one
  // cooperative launch per block column
  std::vector<MixedLU> pre;
  if (precision != BEMGPU_PREC_FP64 && ctx->solver != 2 && same && nreq > 1) {
    const int n = r[0].n;
    const size_t nn = (size_t)n * n;
    float *W32 = (float *)bem_workspace(ctx, "bW32", 8 * nn * nreq);
    int *piv = (int *)bem_workspace(ctx, "bipiv", 4 * (size_t)n * nreq);
    int *inf = (int *)bem_workspace(ctx, "binfo", 4 * (size_t)nreq);
    if (!W32 || !piv || !inf) return fail_all(bem_fail(ctx, BEMGPU_ERR_OOM, "heat_transfer_batch: LU workspace"));
    for (int i = 0; i < nreq; i++) bem_c128_to_c64(ctx, W[i], n, W32 + 2 * nn * i, st);
    rc = bem_cgetrf_batch(ctx, W32, (int64_t)(2 * nn), nreq, n, n, piv, inf, st);
    if (rc) return fail_all(rc);
    for (int i = 0; i < nreq; i++) pre.push_back({W32 + 2 * nn * i, piv + (size_t)n * i, inf + i});
  }
  int first = BEMGPU_OK;
  for (int i = 0; i < nreq; i++) {
    bemgpu_solve_info_t mine;
    bemgpu_solve_info_t *pi = infos ? &infos[i] : &mine;
    memset(pi, 0, sizeof *pi);
    pi->ms_fill = fill_ms / nreq;  // the batch's fill, shared
    pi->pairs_near = jobs[3 * i].near + jobs[3 * i + 1].near + jobs[3 * i + 2].near;
    pi->pairs_far_fp64 = jobs[3 * i].far + jobs[3 * i + 1].far + jobs[3 * i + 2].far;
    status[i] = finish_request(ctx, r[i], &reqs[i], W[i], G1[i], G2[i], precision, st,
                               pre.empty() ? nullptr : &pre[i], &P_out[i], pi);
    if (status[i] != BEMGPU_OK && first == BEMGPU_OK) first = status[i];
    if (status[i] == BEMGPU_ERR_TIMEOUT) {
      // a wait ran out: the device state of the batch is not to be trusted
      for (int j = i + 1; j < nreq; j++) status[j] = BEMGPU_ERR_TIMEOUT;
      return first;
    }
  }
  return first;
}
