// Mixed-precision per-frequency solve (BEMGPU_PREC_MIXED_LA, BEMGPU_PREC_MIXED).
//
// Input: W (FP64 complex, n x n) = Zext + blockdiag(G1, G2) as filled, G1, G2
// (FP64).  The reference inverts W in FP64 (src/util/DenseMatrix.cpp:65-77) and
// forms S = 1/4 tr(B2^H B1) (src/HeatTransfer.cpp:36-58).  Here:
//
//   1. W32 = fl32(W); LU of W32 in complex64, then L^{-1} and U^{-1} explicitly
//      (recursive blocked inversion: large tensor-core GEMMs), so that every
//      solve below is two GEMMs: W32^{-1} B = U^{-1} (L^{-1} (P B)).
//   2. Y0 = W32^{-1} E_t (E_t: the t columns of the identity), widened to FP64.
//   3. Iterative refinement: R = E_t - W Y with W and Y in FP64 on the tensor
//      cores (gemm_exact.cu: 5-slice block fixed point, exact slice sums, error
//      ~2^-41 of each K-block's largest term); Y += fl64(W32^{-1} fl32(R)).
//      The refinement's fixed point depends only on this residual; the
//      complex64 inverse sets how fast it is reached.
//      W is sliced once per solve, Y once per step.  A residual accurate only to
//      FP32 (2^-24 of |W||Y|) leaves the spectral power off by up to ~1e-6 at
//      low loss; the 41-bit product brings that to ~1e-9.
//   4. S = 1/4 sum conj(B2) o B1 with B1 = H1 X, B2 = X H2, X = Y[s rows],
//      H = G + G^H (FP64), both products exact on the tensor cores as in 3.
//      B2 is formed as C = H2 X^H = B2^H (H2 is Hermitian), so both products
//      are left multiplications; S = 1/4 sum_{k,j} C_jk B1_kj.
//   Refinement stops when S moves by less than 3e-7 relative, or stalls (at
//   most 4 steps).  err_est = |S_k - S_{k-1}| / |S_k| for the last step (an
//   upper estimate of the error of S_{k-1}; S_k is more accurate).
#include "bemgpu_internal.h"

#include <cmath>
#include <algorithm>
#include <initializer_list>

namespace {

constexpr int MIXED_SLICES = 5;  // block fixed-point slices of the refinement and trace products
constexpr int DELTA_SLICES = 3;  // slices of a correction: each correction is quantized to them in
                                 // place before it is added to the iterate, so the residual's
                                 // incremental products stay exact (to 2^-40 of |W||Y|)
constexpr int FIRST_SLICES = 2;  // slices of the complex64 path's first iterate, quantized to them in
                                 // place: 2^-17 of its block maxima, below the complex64 LU's own
                                 // error, so refinement corrects both in the same steps
constexpr int TRACE_SLICES = 4;  // slices of X in the full trace products H1 X, H2 X^H (10 products):
                                 // ~2^-33 of |H||X| per entry; the trace of a product of two
                                 // absorption (semi-definite) operators does not cancel, so S keeps
                                 // ~1e-9 (measured 4e-10 against 5 slices at N = 7680)

__global__ void c128_to_c64_kernel(const double *__restrict__ S, int64_t lds, float *__restrict__ D, int64_t ldd, int m,
                                   int n) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  const int c = blockIdx.y;
  if (r >= m || c >= n) return;
  const double2 v = reinterpret_cast<const double2 *>(S)[r + lds * (int64_t)c];
  reinterpret_cast<float2 *>(D)[r + ldd * (int64_t)c] = make_float2((float)v.x, (float)v.y);
}

// XH (FP64, m x k) = X^H for X (k x m, ld ldx).
__global__ void conj_transpose_kernel(const double *__restrict__ X, int64_t ldx, int k, int m,
                                      double *__restrict__ XH) {
  __shared__ double2 tile[32][33];
  const int bx = blockIdx.x * 32, by = blockIdx.y * 32;  // bx over X rows (k), by over X cols (m)
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int r = bx + threadIdx.x, c = by + j;
    if (r < k && c < m) tile[j][threadIdx.x] = reinterpret_cast<const double2 *>(X)[r + ldx * (int64_t)c];
  }
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int r = by + threadIdx.x, c = bx + j;  // XH(r, c) = conj(X(c, r))
    if (r < m && c < k) {
      const double2 v = tile[threadIdx.x][j];
      reinterpret_cast<double2 *>(XH)[r + (int64_t)m * c] = make_double2(v.x, -v.y);
    }
  }
}

// Partial sums of C(j, k) B1(k, j) (C: nt2 x ns2, B1: ns2 x nt2), tiled transpose.
__global__ void trace_tiles_kernel(const double *__restrict__ B1, const double *__restrict__ C, int ns2, int nt2,
                                   double *__restrict__ partial) {
  __shared__ double2 tile[32][33];
  __shared__ double red_r[256], red_i[256];
  const int kb = blockIdx.x * 32, jb = blockIdx.y * 32;
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {  // C(jb + tx, kb + j)
    const int r = jb + threadIdx.x, c = kb + j;
    tile[j][threadIdx.x] = (r < nt2 && c < ns2) ? reinterpret_cast<const double2 *>(C)[r + (int64_t)nt2 * c]
                                                : make_double2(0, 0);
  }
  __syncthreads();
  double ar = 0, ai = 0;
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {  // B1(kb + tx, jb + j) * C(jb + j, kb + tx)
    const int r = kb + threadIdx.x, c = jb + j;
    if (r < ns2 && c < nt2) {
      const double2 b = reinterpret_cast<const double2 *>(B1)[r + (int64_t)ns2 * c];
      const double2 cc = tile[threadIdx.x][j];
      ar += b.x * cc.x - b.y * cc.y;
      ai += b.x * cc.y + b.y * cc.x;
    }
  }
  const int t = threadIdx.y * 32 + threadIdx.x;
  red_r[t] = ar;
  red_i[t] = ai;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (t < s) {
      red_r[t] += red_r[t + s];
      red_i[t] += red_i[t + s];
    }
    __syncthreads();
  }
  if (t == 0) {
    const int b = blockIdx.y * gridDim.x + blockIdx.x;
    partial[2 * b] = red_r[0];
    partial[2 * b + 1] = red_i[0];
  }
}

// H = G + G^H in FP64 (symm, src/util/DenseMatrix.cpp:477-486), out of place.
__global__ void sym64_kernel(const double *__restrict__ G, int64_t ld, int m, double *__restrict__ H) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (i >= m) return;
  const double2 a = reinterpret_cast<const double2 *>(G)[i + ld * (int64_t)j];
  const double2 b = reinterpret_cast<const double2 *>(G)[j + ld * (int64_t)i];
  reinterpret_cast<double2 *>(H)[i + (int64_t)m * j] = make_double2(a.x + b.x, a.y - b.y);
}

// Y64 (+)= widen(D32); dY64 = widen(D32) when dY is given.
__global__ void update_kernel(double *__restrict__ Y, const float *__restrict__ D, int64_t ld, int n, int accumulate,
                              double *__restrict__ dY) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  const int c = blockIdx.y;
  if (r >= n) return;
  const int64_t idx = r + ld * (int64_t)c;
  const float2 d = reinterpret_cast<const float2 *>(D)[idx];
  double2 y = accumulate ? reinterpret_cast<double2 *>(Y)[idx] : make_double2(0, 0);
  y.x += (double)d.x;
  y.y += (double)d.y;
  reinterpret_cast<double2 *>(Y)[idx] = y;
  if (dY) reinterpret_cast<double2 *>(dY)[idx] = make_double2((double)d.x, (double)d.y);
}

// R32 = fl32(E_t + R64), E_t(r, c) = [r == row0 + c].
__global__ void residual_finish_kernel(const double *__restrict__ R64, float *__restrict__ R32, int64_t ld, int n,
                                       int row0) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  const int c = blockIdx.y;
  if (r >= n) return;
  const int64_t idx = r + ld * (int64_t)c;
  double2 v = reinterpret_cast<const double2 *>(R64)[idx];
  if (r == row0 + c) v.x += 1.0;
  reinterpret_cast<float2 *>(R32)[idx] = make_float2((float)v.x, (float)v.y);
}

// D = E_t + R64 in FP64 (the residual the FP64-class solve corrects with).
__global__ void residual_fp64_kernel(const double *__restrict__ R64, double *__restrict__ D, int64_t ld, int n,
                                     int row0) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  const int c = blockIdx.y;
  if (r >= n) return;
  const int64_t idx = r + ld * (int64_t)c;
  double2 v = reinterpret_cast<const double2 *>(R64)[idx];
  if (r == row0 + c) v.x += 1.0;
  reinterpret_cast<double2 *>(D)[idx] = v;
}

// Y += D (FP64).
__global__ void add_fp64_kernel(double *__restrict__ Y, const double *__restrict__ D, int64_t ld, int n) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  const int c = blockIdx.y;
  if (r >= n) return;
  const int64_t idx = r + ld * (int64_t)c;
  double2 y = reinterpret_cast<double2 *>(Y)[idx];
  const double2 d = reinterpret_cast<const double2 *>(D)[idx];
  y.x += d.x;
  y.y += d.y;
  reinterpret_cast<double2 *>(Y)[idx] = y;
}

__global__ void identity_cols_c128_kernel(double *Y, int64_t ld, int n, int row0) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  const int c = blockIdx.y;
  if (r >= n) return;
  reinterpret_cast<double2 *>(Y)[r + ld * (int64_t)c] = make_double2(r == row0 + c ? 1.0 : 0.0, 0.0);
}

// out = 1/4 sum of the np partial (re, im) pairs; one CTA of 256 threads, fixed
// summation order (deterministic).
__global__ void __launch_bounds__(256) trace_final_kernel(const double *partial, int np, double *out) {
  __shared__ double sr[256], si[256];
  double r = 0, i = 0;
  for (int k = threadIdx.x; k < np; k += 256) {
    r += partial[2 * k];
    i += partial[2 * k + 1];
  }
  sr[threadIdx.x] = r;
  si[threadIdx.x] = i;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      sr[threadIdx.x] += sr[threadIdx.x + s];
      si[threadIdx.x] += si[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = 0.25 * sr[0];
    out[1] = 0.25 * si[0];
  }
}

}  // namespace


namespace {

struct MixedBufs {
  float *W32 = nullptr, *R32 = nullptr, *Linv = nullptr, *Uinv = nullptr, *T32 = nullptr;
  double *H1, *H2, *Y, *dY, *R64, *XH, *B1, *C, *partial;
  int *ipiv, *info;
  int ntiles;
  ExactOperand opW, opH1, opH2;
};

float ev_ms(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0;
  cudaEventElapsedTime(&ms, a, b);
  return ms;
}

// S from B1 = H1 X and C = H2 X^H.  incremental: X moved by the correction
// dY of the last step, so B1 += H1 dX and C += H2 dX^H (3-slice products of
// the small correction) instead of the full 5-slice products.
int spectral_trace(bemgpu_ctx_s *ctx, MixedBufs &b, int n, int ns2, int nt2, cudaStream_t st, double S[2],
                   bool incremental) {
  const double *X = incremental ? b.dY : b.Y;  // rows [0, ns2), leading dimension n
  const int sl = incremental ? DELTA_SLICES : TRACE_SLICES;
  const int acc = incremental ? 1 : 0;
  ExactOperand opX, opXH;
  int rc = bem_exact_prep(ctx, "X", false, X, n, nt2, ns2, 1.0, sl, opX, st);
  if (!rc) rc = bem_exact_gemm(ctx, BEMGPU_K_TRACE, b.opH1, opX, b.B1, ns2, acc, st);
  if (rc) return rc;
  {
    ProfScope ps(ctx, BEMGPU_K_TRACE, st, 0.0, 32.0 * ns2 * (double)nt2);
    conj_transpose_kernel<<<dim3((ns2 + 31) / 32, (nt2 + 31) / 32), dim3(32, 8), 0, st>>>(X, n, ns2, nt2, b.XH);
    ctx->launches++;
  }
  rc = bem_exact_prep(ctx, "XH", false, b.XH, nt2, ns2, nt2, 1.0, sl, opXH, st);
  if (!rc) rc = bem_exact_gemm(ctx, BEMGPU_K_TRACE, b.opH2, opXH, b.C, nt2, acc, st);
  if (rc) return rc;
  const dim3 tg((ns2 + 31) / 32, (nt2 + 31) / 32);
  {
    ProfScope ps(ctx, BEMGPU_K_TRACE, st, 8.0 * ns2 * nt2, 32.0 * ns2 * nt2);
    trace_tiles_kernel<<<tg, dim3(32, 8), 0, st>>>(b.B1, b.C, ns2, nt2, b.partial);
    ctx->launches++;
    trace_final_kernel<<<1, 256, 0, st>>>(b.partial, b.ntiles, b.partial + 2 * b.ntiles);
    ctx->launches++;
  }
  BEM_CUDA_TRY(ctx, cudaMemcpyAsync(S, b.partial + 2 * b.ntiles, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
  BEM_CUDA_TRY(ctx, cudaStreamSynchronize(st));
  return BEMGPU_OK;
}

}  // namespace

namespace {

// Sizes a refinement correction dY (just quantized to DELTA_SLICES slices,
// op = its operand) against the iterate (eb_y: exponent field of Y's largest
// entry) and sets how the next products use it.  A small correction (|dY| <=
// 2^-12 |Y|): the residual update -W dY takes levels 0..2 of the slice
// products (error 2^-24 |W||dY| <= 2^-36 |W||Y|) and the trace is updated by
// H1 dX and H2 dX^H.  A large one (a slowly contracting refinement): the
// residual update takes every product of W's 5 slices and dY's 3 exact ones
// (2^-40 |W||dY|), and the trace is formed again from the whole iterate,
// since an incremental update carries 2^-24 of |dX| into S and S may be a
// small difference of its terms.  Synchronizes the stream (reads dY's exponent).
bool correction_is_small(bemgpu_ctx_s *ctx, ExactOperand &op, unsigned eb_y, cudaStream_t st) {
  unsigned eb_dy = 0;
  if (cudaMemcpyAsync(&eb_dy, op.aux + 8, sizeof(unsigned), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess) {
    cudaGetLastError();
    op.exact = true;
    return false;
  }
  (void)ctx;
  const bool small = (int)eb_dy - (int)eb_y <= -12;
  op.exact = !small;
  return small;
}

// The FP64-class solve: W (already sliced into b.opW) is factored in place by
// the tensor-core LU of FP64 accuracy (bem_zgetrf_exact), Y0 = W^-1 E_t by its
// blocked solve, then the same refinement and trace as the complex64 path with
// FP64 corrections.  Used when the complex64 factorization is not accurate
// enough for the refinement to converge (ill-conditioned W), or on request.
// W is factored in place; its residuals use b.opW, sliced before.
int fp64lu_solve(bemgpu_ctx_s *ctx, double *W, int n, int ns2, MixedBufs &b, cudaStream_t st, double S[2],
                 int &iters, double &err) {
  const int nt2 = n - ns2;
  const dim3 gm((n + 255) / 256, nt2);
  int rc = bem_zgetrf_exact(ctx, W, n, n, b.ipiv, b.info, st);
  if (rc) return rc;
  int hinfo = 0;
  BEM_CUDA_TRY(ctx, cudaMemcpyAsync(&hinfo, b.info, sizeof(int), cudaMemcpyDeviceToHost, st));
  BEM_CUDA_TRY(ctx, cudaStreamSynchronize(st));
  if (hinfo != 0) return bem_fail(ctx, BEMGPU_ERR_SINGULAR, "FP64-class LU: zero pivot at column %d", hinfo);
  identity_cols_c128_kernel<<<gm, 256, 0, st>>>(b.Y, n, n, ns2);
  ctx->launches++;
  rc = bem_zgetrs_exact(ctx, W, n, n, b.ipiv, b.Y, n, nt2, st);
  if (rc) return rc;
  double Sprev[2] = {0, 0};
  rc = spectral_trace(ctx, b, n, ns2, nt2, st, S, false);
  if (rc) return rc;
  err = 1.0;
  double err_prev = 1.0;
  // up to 6 steps: near its floor (cond(W) x ~1e-12) this refinement can
  // contract by only ~0.5 per step, and a step costs a fraction of the FP64
  // path it would otherwise fall back to; it stops when a step gains less
  // than 20 %
  ExactOperand opDY;  // the last correction, quantized: R64 and Y move by the same values
  unsigned eb_y = 0;   // FP64 exponent fields of the largest |Y| and |dY| entries
  for (iters = 1; iters <= 6; iters++) {
    if (iters == 1) {
      ExactOperand opY;
      rc = bem_exact_prep(ctx, "Y", false, b.Y, n, nt2, n, 1.0, MIXED_SLICES, opY, st);
      if (!rc) rc = bem_exact_gemm(ctx, BEMGPU_K_REFINE_GEMM, b.opW, opY, b.R64, n, 0, st);
      if (!rc) BEM_CUDA_TRY(ctx, cudaMemcpyAsync(&eb_y, opY.aux + 8, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    } else {
      // as in the complex64 refinement (exact products for a large correction)
      rc = bem_exact_gemm(ctx, BEMGPU_K_REFINE_GEMM, b.opW, opDY, b.R64, n, 1, st);
    }
    if (rc) return rc;
    residual_fp64_kernel<<<gm, 256, 0, st>>>(b.R64, b.dY, n, n, ns2);
    ctx->launches++;
    rc = bem_zgetrs_exact(ctx, W, n, n, b.ipiv, b.dY, n, nt2, st);
    if (!rc) rc = bem_exact_prep(ctx, "Y", false, b.dY, n, nt2, n, 1.0, DELTA_SLICES, opDY, st, b.dY);
    if (rc) return rc;
    add_fp64_kernel<<<gm, 256, 0, st>>>(b.Y, b.dY, n, n);
    ctx->launches++;
    const bool small = correction_is_small(ctx, opDY, eb_y, st);
    Sprev[0] = S[0];
    Sprev[1] = S[1];
    rc = spectral_trace(ctx, b, n, ns2, nt2, st, S, small);
    if (rc) return rc;
    if (bem_tc_error(ctx, true))
      return bem_fail(ctx, BEMGPU_ERR_TIMEOUT, "FP64-class solve: a tensor-core pipeline wait ran out");
    err_prev = err;
    err = fabs(S[0] - Sprev[0]) / fmax(fabs(S[0]), 1e-300);
    bem_trace("n=%d FP64-class refinement step %d: err_est %.3e", n, iters, err);
    if (err < 3e-7 || err > 0.8 * err_prev) break;
  }
  return BEMGPU_OK;
}

}  // namespace

// Gives back named workspace buffers that a later stage no longer needs
// when free device memory would not hold `need` more bytes beside them (the
// largest solves); otherwise keeps them for the next request.
void bem_release_if_short(bemgpu_ctx_s *ctx, size_t need, std::initializer_list<const char *> names) {
  size_t fr = 0, tot = 0;
  cudaMemGetInfo(&fr, &tot);
  if ((double)fr >= 1.05 * (double)need + (double)(1u << 30)) return;
  for (const char *nm : names) bem_workspace_release(ctx, nm);
}

// W32 = fl32(W) for the batch driver (heat_transfer.cu): the conversion the
// mixed solve does before its LU.
void bem_c128_to_c64(bemgpu_ctx_s *ctx, const double *W, int n, float *W32, cudaStream_t st) {
  const dim3 gn((n + 255) / 256, n);
  c128_to_c64_kernel<<<gn, 256, 0, st>>>(W, n, W32, n, n, n);
  ctx->launches++;
}

int bem_mixed_solve(bemgpu_ctx_s *ctx, double *W, int n, int ns2, const double *G1, const double *G2,
                    cudaStream_t st, double S_out[2], bemgpu_solve_info_t *info, const MixedLU *pre) {
  if (!bem_exact_available())
    return bem_fail(ctx, BEMGPU_ERR_CUDA, "mixed solve: tensor-map encoding (driver entry point) unavailable");
  const int nt2 = n - ns2;
  const size_t nn = (size_t)n * n, nm = (size_t)n * nt2, st2 = (size_t)ns2 * nt2;
  MixedBufs b;
  b.ntiles = ((ns2 + 31) / 32) * ((nt2 + 31) / 32);
  // the complex64 factors are not allocated when the context solves FP64-class only
  const bool c64 = ctx->solver != 2;
  if (pre && !c64) return bem_fail(ctx, BEMGPU_ERR_ARG, "mixed solve: complex64 factors given to an FP64-class solve");
  if (c64) {
    // a batch's complex64 LU (bem_cgetrf_batch) arrives factored
    b.W32 = pre ? pre->W32 : (float *)bem_workspace(ctx, "m_W32", 8 * nn);
    b.R32 = (float *)bem_workspace(ctx, "m_R32", 8 * nm);
    b.Linv = (float *)bem_workspace(ctx, "m_Linv", 8 * nn);
    b.Uinv = (float *)bem_workspace(ctx, "m_Uinv", 8 * nn);
    b.T32 = (float *)bem_workspace(ctx, "m_T32", 8 * nm);
  }
  b.H1 = (double *)bem_workspace(ctx, "m_H1", 16 * (size_t)ns2 * ns2);
  b.H2 = (double *)bem_workspace(ctx, "m_H2", 16 * (size_t)nt2 * nt2);
  b.Y = (double *)bem_workspace(ctx, "m_Y", 16 * nm);
  b.dY = (double *)bem_workspace(ctx, "m_dY", 16 * nm);
  b.R64 = (double *)bem_workspace(ctx, "m_R64", 16 * nm);
  b.XH = (double *)bem_workspace(ctx, "m_XH", 16 * st2);
  b.B1 = (double *)bem_workspace(ctx, "m_B1", 16 * st2);
  b.C = (double *)bem_workspace(ctx, "m_C", 16 * st2);
  b.partial = (double *)bem_workspace(ctx, "m_partial", 16 * (size_t)b.ntiles + 64);
  b.ipiv = pre ? pre->ipiv : (int *)bem_workspace(ctx, "m_ipiv", 4 * (size_t)n);
  b.info = pre ? pre->info : (int *)bem_workspace(ctx, "m_info", 16);
  const bool ok = (!c64 || (b.W32 && b.R32 && b.Linv && b.Uinv && b.T32)) && b.H1 && b.H2 && b.Y && b.dY && b.R64 &&
                  b.XH && b.B1 && b.C && b.partial && b.ipiv && b.info;
  if (!ok) return bem_fail(ctx, BEMGPU_ERR_OOM, "mixed solve: workspace allocation failed (n=%d)", n);
  cudaEvent_t *ev = ctx->ev;
  const dim3 gn((n + 255) / 256, n), gm((n + 255) / 256, nt2);
  {
    ProfScope ps(ctx, BEMGPU_K_LU_PANEL, st, 0.0, (c64 ? 24.0 * nn : 0.0) + 48.0 * ((double)ns2 * ns2 + (double)nt2 * nt2));
    if (c64 && !pre) {
      c128_to_c64_kernel<<<gn, 256, 0, st>>>(W, n, b.W32, n, n, n);
      ctx->launches++;
    }
    sym64_kernel<<<dim3((ns2 + 255) / 256, ns2), 256, 0, st>>>(G1, ns2, ns2, b.H1);
    ctx->launches++;
    sym64_kernel<<<dim3((nt2 + 255) / 256, nt2), 256, 0, st>>>(G2, nt2, nt2, b.H2);
    ctx->launches++;
  }
  BEM_CUDA_TRY(ctx, cudaGetLastError());
  // operands fixed for the whole solve: -W (residual), H1, H2 (trace)
  int rc = bem_exact_prep(ctx, "W", true, W, n, n, n, -1.0, MIXED_SLICES, b.opW, st);
  if (!rc) rc = bem_exact_prep(ctx, "H1", true, b.H1, ns2, ns2, ns2, 1.0, MIXED_SLICES, b.opH1, st);
  if (!rc) rc = bem_exact_prep(ctx, "H2", true, b.H2, nt2, nt2, nt2, 1.0, MIXED_SLICES, b.opH2, st);
  if (rc) return rc;
  cudaEventRecord(ev[1], st);
  if (ctx->solver == 2) {
    double S[2] = {0, 0}, err = 1.0;
    int iters = 0;
    rc = fp64lu_solve(ctx, W, n, ns2, b, st, S, iters, err);
    if (rc) return rc;
    cudaEventRecord(ev[5], st);
    BEM_CUDA_TRY(ctx, cudaStreamSynchronize(st));
    S_out[0] = S[0];
    S_out[1] = S[1];
    if (info) {
      info->ms_lu = ev_ms(ev[1], ev[5]);
      info->err_est = err;
      info->refine_iters = iters;
      info->solver = 2;
    }
    if (err > 1e-6) return bem_fail(ctx, BEMGPU_ERR_NO_CONVERGE, "FP64-class solve: refinement stalled at %.2e", err);
    return BEMGPU_OK;
  }
  if (!pre) rc = bem_cgetrf(ctx, b.W32, n, n, b.ipiv, b.info, st);
  if (!rc) rc = bem_ctri_inverses(ctx, b.W32, n, n, b.Linv, b.Uinv, st);
  if (rc) return rc;
  cudaEventRecord(ev[2], st);
  rc = bem_capply_inverse_identity(ctx, b.Linv, b.Uinv, n, b.ipiv, ns2, b.R32, n, nt2, b.T32, st);
  if (rc) return rc;
  update_kernel<<<gm, 256, 0, st>>>(b.Y, b.R32, n, n, 0, nullptr);
  ctx->launches++;
  cudaEventRecord(ev[3], st);
  int hinfo = 0;
  BEM_CUDA_TRY(ctx, cudaMemcpyAsync(&hinfo, b.info, sizeof(int), cudaMemcpyDeviceToHost, st));
  BEM_CUDA_TRY(ctx, cudaStreamSynchronize(st));
  if (hinfo != 0 && ctx->solver != 0)
    return bem_fail(ctx, BEMGPU_ERR_SINGULAR, "mixed solve: zero pivot at column %d", hinfo);
  cudaEventRecord(ev[4], st);
  double Sprev[2] = {0, 0}, S[2] = {0, 0};
  int iters = 0;
  double err = hinfo ? 1e300 : 1.0, err_prev = 1.0;
  // up to 6 steps while each gains at least a factor 2 (slowly contracting
  // refinements still finish well before an escalation would)
  const int max_iters = hinfo ? 0 : 6;
  ExactOperand opDY;  // the last correction, quantized: R64 and Y move by the same values
  unsigned eb_y = 0;   // FP64 exponent fields of the largest |Y| and |dY| entries
  while (iters < max_iters) {
    // R = E_t - W Y: R64 holds -W Y; the first step forms it from Y, later
    // steps add -W dY of the last correction (3-slice product)
    if (iters == 0) {
      // the first iterate (complex64 accuracy) is quantized to 2 slices in
      // place; W's 5 slices times those 2 then need 9 slice products, not 15,
      // for the same 2^-40 residual of the quantized iterate
      ExactOperand opY;
      rc = bem_exact_prep(ctx, "Y", false, b.Y, n, nt2, n, 1.0, FIRST_SLICES, opY, st, b.Y);
      if (!rc) rc = bem_exact_gemm(ctx, BEMGPU_K_REFINE_GEMM, b.opW, opY, b.R64, n, 0, st);
      if (!rc) BEM_CUDA_TRY(ctx, cudaMemcpyAsync(&eb_y, opY.aux + 8, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    } else {
      // -W dY of the last correction (its products chosen by its size,
      // correction_is_small)
      rc = bem_exact_gemm(ctx, BEMGPU_K_REFINE_GEMM, b.opW, opDY, b.R64, n, 1, st);
    }
    if (rc) return rc;
    residual_finish_kernel<<<gm, 256, 0, st>>>(b.R64, b.R32, n, n, ns2);
    ctx->launches++;
    rc = bem_capply_inverse(ctx, b.Linv, b.Uinv, n, b.ipiv, b.R32, n, nt2, b.T32, st);
    if (rc) return rc;
    // dY = widen(correction), quantized in place to the 3 slices the next
    // residual multiplies, then Y += dY: -W Y in R64 stays exact to the
    // product's 2^-40 however large the correction is (a slowly contracting
    // refinement's corrections are not small)
    update_kernel<<<gm, 256, 0, st>>>(b.dY, b.R32, n, n, 0, nullptr);
    ctx->launches++;
    rc = bem_exact_prep(ctx, "Y", false, b.dY, n, nt2, n, 1.0, DELTA_SLICES, opDY, st, b.dY);
    if (rc) return rc;
    add_fp64_kernel<<<gm, 256, 0, st>>>(b.Y, b.dY, n, n);
    ctx->launches++;
    const bool small = correction_is_small(ctx, opDY, eb_y, st);
    iters++;
    Sprev[0] = S[0];
    Sprev[1] = S[1];
    rc = spectral_trace(ctx, b, n, ns2, nt2, st, S, iters > 1 && small);
    if (rc) return rc;
    if (bem_tc_error(ctx, true))
      return bem_fail(ctx, BEMGPU_ERR_TIMEOUT, "mixed solve: a tensor-core pipeline wait ran out");
    if (iters == 1) continue;  // the spectral power of the unrefined solve is not needed
    err_prev = err;
    err = fabs(S[0] - Sprev[0]) / fmax(fabs(S[0]), 1e-300);
    bem_trace("n=%d complex64 refinement step %d: err_est %.3e", n, iters, err);
    // converged, or stalled at the accuracy floor of the residual
    if (err < 3e-7 || err > 0.5 * err_prev) break;
  }
  int solver = 1;
  if (ctx->solver == 0 && !(err <= ctx->escalate_tol)) {
    // the complex64 factors are not accurate enough for this W (refinement
    // diverged or stalled above the tolerance, or a zero pivot): factor a
    // copy of W in FP64-class arithmetic on the tensor cores and refine with
    // that.  W stays as filled for the last step: when even this refinement
    // stalls above the fallback tolerance (its residual's ~2^-40 accuracy
    // times the condition of W), the caller solves W on the FP64 path.
    bem_trace("n=%d escalating to the FP64-class LU (complex64 err_est %.3e, pivot info %d)", n, err, hinfo);
    // the complex64 stage is done: its buffers go back first if the copy of W
    // and the FP64-class blocks would not fit beside them
    bem_release_if_short(ctx, 16 * nn + 2 * 16 * (size_t)n * 512 + bem_exact_operand_bytes(true, n, 512, 5) +
                                  bem_exact_operand_bytes(false, n, 512, 5),
                         {"m_W32", "m_R32", "m_Linv", "m_Uinv", "m_T32", "tc_A", "tc_B", "tri_tmp"});
    double *Wlu = (double *)bem_workspace(ctx, "m_Wlu", 16 * nn);
    const bool keep_w = Wlu != nullptr;
    if (keep_w) {
      BEM_CUDA_TRY(ctx, cudaMemcpyAsync(Wlu, W, 16 * nn, cudaMemcpyDeviceToDevice, st));
    } else {
      // no room for the copy: factor W itself (no FP64 fallback afterwards)
      bem_trace("n=%d no memory for a copy of W: factoring it in place", n);
      Wlu = W;
    }
    rc = fp64lu_solve(ctx, Wlu, n, ns2, b, st, S, iters, err);
    if (rc) return rc;
    solver = 2;
    if (keep_w && !(err <= ctx->fallback_tol)) {
      bem_trace("n=%d FP64-class err_est %.3e above %.1e: solving on the FP64 path", n, err, ctx->fallback_tol);
      BEM_CUDA_TRY(ctx, cudaStreamSynchronize(st));
      if (info) {
        info->err_est = err;
        info->refine_iters = iters;
        info->solver = 2;
      }
      return BEM_SOLVE_ON_FP64_PATH;
    }
  }
  cudaEventRecord(ev[5], st);
  BEM_CUDA_TRY(ctx, cudaStreamSynchronize(st));
  S_out[0] = S[0];
  S_out[1] = S[1];
  if (info) {
    info->ms_lu = ev_ms(ev[1], ev[2]);
    info->ms_solve = ev_ms(ev[2], ev[3]);
    info->ms_trace = ev_ms(ev[3], ev[4]);
    info->ms_refine = ev_ms(ev[4], ev[5]);
    info->err_est = err;
    info->refine_iters = iters;
    info->solver = solver;
  }
  if (err > 1e-6) return bem_fail(ctx, BEMGPU_ERR_NO_CONVERGE, "mixed solve: refinement stalled at %.2e", err);
  return BEMGPU_OK;
}
