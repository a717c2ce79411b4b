// Mixed-precision per-frequency solve (BEMGPU_PREC_MIXED).
//
// Input: W (FP64 complex, n x n) = Zext + blockdiag(G1, G2) as filled (far pairs
// integrated in FP32, near pairs in FP64), G1, G2 (FP64).
//
//   1. W32 = fl32(W); LU of W32 in complex64.
//   2. Y0 = W32^{-1} E_t (E_t: the t columns of the identity), complex64.
//   3. Iterative refinement, residual R = E_t - W Y split by magnitude:
//        W = W_near + W_far, W_near = the entries above tau * row max (at most
//        NEAR_CAP per row, stored as an FP64 ELL matrix), W_far = the rest.
//        R = E_t - W_near Y (FP64) - W_far Y (complex64 GEMM).
//      The near-field entries are up to ~1e4 times larger than the typical entry
//      of a row; computing their product in FP64 and only the small dense
//      remainder in FP32 gives the residual the accuracy refinement needs (a
//      residual accumulated wholly in FP32 does not reduce the error at all).
//      Y (FP64) += W32^{-1} fl32(R); repeated until the spectral power moves by
//      less than 1e-7 relative (at most 4 steps).
//      The far product runs on the FP32 pipes with compensated accumulation
//      (FP32 within 8-deep K tiles, a two-float sum across them): plain FP32
//      accumulation over the whole K leaves a floor near 1e-6 in S.
//   4. S = 1/4 sum conj(B2) o B1 with B1 = H1 X, B2 = X H2, X = Y[s rows],
//      H = G + G^H (FP64); both products split like the residual (near part in
//      FP64 from an ELL copy, the rest in complex64 with FP64 output).  B2 is
//      formed as C = H2 X^H = B2^H (H2 is Hermitian), so both products are
//      left multiplications by a row-split matrix; S = 1/4 sum_{k,j} C_jk B1_kj.
//   err_est = |S_k - S_{k-1}| / |S_k| for the last step (an upper estimate of
//   the error of S_{k-1}; S_k is more accurate).
#include "bemgpu_internal.h"

#include <cmath>
#include <algorithm>

namespace {

// Near/far split thresholds (fraction of the row maximum) and the ELL capacity.
// The residual needs the finer split: at N = 7680, tau = 1e-2 leaves a far part
// whose FP32 accumulation error floors the spectral power near 1e-5 at low loss.
constexpr int NEAR_CAP = 1024;
constexpr double TAU_RESIDUAL = 1e-3;
constexpr double TAU_TRACE = 1e-2;

__global__ void c128_to_c64_kernel(const double *__restrict__ S, int64_t lds, float *__restrict__ D, int64_t ldd, int m,
                                   int n) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  const int c = blockIdx.y;
  if (r >= m || c >= n) return;
  const double2 v = reinterpret_cast<const double2 *>(S)[r + lds * (int64_t)c];
  reinterpret_cast<float2 *>(D)[r + ldd * (int64_t)c] = make_float2((float)v.x, (float)v.y);
}

// Row maxima of |W| (thread per row; consecutive threads read consecutive rows).
__global__ void rowmax_kernel(const double *__restrict__ W, int64_t ld, int n, double *__restrict__ rmax) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  double m = 0;
  for (int j = 0; j < n; j++) {
    const double2 v = reinterpret_cast<const double2 *>(W)[r + ld * (int64_t)j];
    m = fmax(m, v.x * v.x + v.y * v.y);
  }
  rmax[r] = sqrt(m);
}

// Splits W into the FP64 ELL near part and the complex64 far part.
__global__ void near_split_kernel(const double *__restrict__ W, int64_t ld, int n, const double *__restrict__ rmax,
                                  double tau, int *__restrict__ ecol, double2 *__restrict__ eval,
                                  int *__restrict__ ecount, float *__restrict__ Wf, int64_t ldf) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const double th = tau * rmax[r];
  const double th2 = th * th;
  int cnt = 0;
  for (int j = 0; j < n; j++) {
    const double2 v = reinterpret_cast<const double2 *>(W)[r + ld * (int64_t)j];
    float2 f = make_float2((float)v.x, (float)v.y);
    if (cnt < NEAR_CAP && v.x * v.x + v.y * v.y > th2) {
      ecol[(int64_t)cnt * n + r] = j;
      eval[(int64_t)cnt * n + r] = v;
      cnt++;
      f = make_float2(0.f, 0.f);
    }
    reinterpret_cast<float2 *>(Wf)[r + ldf * (int64_t)j] = f;
  }
  ecount[r] = cnt;
}

// OUT(r, c) = ACC(r, c) + sign * sum_k ELL(r, k) Y(col(r, k), c)  [+ E_t(r, c)];
// ACC and Y in FP64.  With R32 non-null the result is also written as complex64.
__global__ void ell_left_kernel(const int *__restrict__ ecol, const double2 *__restrict__ eval,
                                const int *__restrict__ ecount, int m, const double *__restrict__ Y, int64_t ldy,
                                double *__restrict__ ACC, int64_t ldacc, double sign, int add_identity_row0,
                                float *__restrict__ R32, int64_t ldr32) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  const int c = blockIdx.y;
  if (r >= m) return;
  double2 acc = reinterpret_cast<double2 *>(ACC)[r + ldacc * (int64_t)c];
  if (add_identity_row0 >= 0 && r == add_identity_row0 + c) acc.x += 1.0;
  const int cnt = ecount[r];
  const double2 *Yc = reinterpret_cast<const double2 *>(Y) + ldy * (int64_t)c;
  double sr = 0, si = 0;
  for (int k = 0; k < cnt; k++) {
    const double2 a = eval[(int64_t)k * m + r];
    const double2 y = Yc[ecol[(int64_t)k * m + r]];
    sr += a.x * y.x - a.y * y.y;
    si += a.x * y.y + a.y * y.x;
  }
  acc.x += sign * sr;
  acc.y += sign * si;
  reinterpret_cast<double2 *>(ACC)[r + ldacc * (int64_t)c] = acc;
  if (R32) reinterpret_cast<float2 *>(R32)[r + ldr32 * (int64_t)c] = make_float2((float)acc.x, (float)acc.y);
}

// XH (FP64, m x k) = X^H for X (k x m, ld ldx), and its complex64 rounding.
__global__ void conj_transpose_kernel(const double *__restrict__ X, int64_t ldx, int k, int m,
                                      double *__restrict__ XH, float *__restrict__ XH32) {
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
      reinterpret_cast<float2 *>(XH32)[r + (int64_t)m * c] = make_float2((float)v.x, (float)-v.y);
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

// Y64 (+)= widen(D32); Y32 = fl32(Y64); also accumulates |D|^2 and |Y|^2 per block.
__global__ void update_kernel(double *__restrict__ Y, const float *__restrict__ D, float *__restrict__ Y32, int64_t ld,
                              int n, int accumulate) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  const int c = blockIdx.y;
  if (r >= n) return;
  const int64_t idx = r + ld * (int64_t)c;
  const float2 d = reinterpret_cast<const float2 *>(D)[idx];
  double2 y = accumulate ? reinterpret_cast<double2 *>(Y)[idx] : make_double2(0, 0);
  y.x += (double)d.x;
  y.y += (double)d.y;
  reinterpret_cast<double2 *>(Y)[idx] = y;
  reinterpret_cast<float2 *>(Y32)[idx] = make_float2((float)y.x, (float)y.y);
}

__global__ void identity_cols_c64_kernel(float *Y, int64_t ld, int n, int row0, int ncols) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  const int c = blockIdx.y;
  if (r >= n) return;
  reinterpret_cast<float2 *>(Y)[r + ld * (int64_t)c] = make_float2(r == row0 + c ? 1.f : 0.f, 0.f);
}

__global__ void zero64_kernel(double *p, int64_t n2) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n2; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = 0.0;
}

constexpr int TR_THREADS = 256;

__global__ void trace32_partial_kernel(const float *B1, const float *B2, int64_t ld, int m, int n, double *partial) {
  __shared__ double sr[TR_THREADS], si[TR_THREADS];
  const int64_t total = (int64_t)m * n;
  double ar = 0, ai = 0;
  for (int64_t idx = (int64_t)blockIdx.x * TR_THREADS + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * TR_THREADS) {
    const int64_t r = idx % m, c = idx / m;
    const float2 b1 = reinterpret_cast<const float2 *>(B1)[r + ld * c];
    const float2 b2 = reinterpret_cast<const float2 *>(B2)[r + ld * c];
    ar += (double)b2.x * b1.x + (double)b2.y * b1.y;
    ai += (double)b2.x * b1.y - (double)b2.y * b1.x;
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

}  // namespace


namespace {

struct Ell {
  int *col = nullptr;
  double2 *val = nullptr;
  int *cnt = nullptr;
};

struct MixedBufs {
  float *W32, *Wf, *H1f, *H2f, *Y32, *R32, *XH32;
  double *H1, *H2, *Y, *R64, *XH, *B1, *C, *rmax, *partial;
  Ell eW, eH1, eH2;
  int *ipiv, *info;
  int ntiles;
};

float ev_ms(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0;
  cudaEventElapsedTime(&ms, a, b);
  return ms;
}

bool alloc_ell(bemgpu_ctx_s *ctx, const char *name, int m, Ell &e) {
  const std::string s(name);
  e.col = (int *)bem_workspace(ctx, s + "_col", 4 * (size_t)m * NEAR_CAP);
  e.val = (double2 *)bem_workspace(ctx, s + "_val", 16 * (size_t)m * NEAR_CAP);
  e.cnt = (int *)bem_workspace(ctx, s + "_cnt", 4 * (size_t)m);
  return e.col && e.val && e.cnt;
}

// Splits the FP64 square matrix M (m x m, ld m) into its row-ELL near part and
// the complex64 remainder F.
void split_near(bemgpu_ctx_s *ctx, const double *M, int m, double tau, double *rmax, Ell &e, float *F,
                cudaStream_t st) {
  rowmax_kernel<<<(m + 127) / 128, 128, 0, st>>>(M, m, m, rmax);
  ctx->launches++;
  near_split_kernel<<<(m + 127) / 128, 128, 0, st>>>(M, m, m, rmax, tau, e.col, e.val, e.cnt, F, m);
  ctx->launches++;
}

int spectral_trace(bemgpu_ctx_s *ctx, const MixedBufs &b, int n, int ns2, int nt2, cudaStream_t st, double S[2]) {
  const float one[2] = {1.f, 0.f};
  const double one64[2] = {1.0, 0.0};
  const double *X = b.Y;  // rows [0, ns2) of Y, leading dimension n
  {
    ProfScope ps(ctx, BEMGPU_K_NEAR_SPMM, st, 8.0 * ns2 * (double)nt2 * NEAR_CAP, 48.0 * ns2 * (double)nt2);
    zero64_kernel<<<1024, 256, 0, st>>>(b.B1, 2 * (int64_t)ns2 * nt2);
    ctx->launches++;
    ell_left_kernel<<<dim3((ns2 + 255) / 256, nt2), 256, 0, st>>>(b.eH1.col, b.eH1.val, b.eH1.cnt, ns2, X, n, b.B1,
                                                                   ns2, 1.0, -1, nullptr, 0);
    ctx->launches++;
  }
  int rc = bem_cgemm_comp64(ctx, BEMGPU_K_TRACE, ns2, nt2, ns2, one, b.H1f, ns2, b.Y32, n, one64, b.B1, ns2, st);
  if (rc) return rc;
  {
    ProfScope ps(ctx, BEMGPU_K_NEAR_SPMM, st, 8.0 * ns2 * (double)nt2 * NEAR_CAP, 64.0 * ns2 * (double)nt2);
    conj_transpose_kernel<<<dim3((ns2 + 31) / 32, (nt2 + 31) / 32), dim3(32, 8), 0, st>>>(X, n, ns2, nt2, b.XH,
                                                                                           b.XH32);
    ctx->launches++;
    zero64_kernel<<<1024, 256, 0, st>>>(b.C, 2 * (int64_t)ns2 * nt2);
    ctx->launches++;
    ell_left_kernel<<<dim3((nt2 + 255) / 256, ns2), 256, 0, st>>>(b.eH2.col, b.eH2.val, b.eH2.cnt, nt2, b.XH, nt2,
                                                                   b.C, nt2, 1.0, -1, nullptr, 0);
    ctx->launches++;
  }
  rc = bem_cgemm_comp64(ctx, BEMGPU_K_TRACE, nt2, ns2, nt2, one, b.H2f, nt2, b.XH32, nt2, one64, b.C, nt2, st);
  if (rc) return rc;
  const dim3 tg((ns2 + 31) / 32, (nt2 + 31) / 32);
  {
    ProfScope ps(ctx, BEMGPU_K_TRACE, st, 8.0 * ns2 * nt2, 32.0 * ns2 * nt2);
    trace_tiles_kernel<<<tg, dim3(32, 8), 0, st>>>(b.B1, b.C, ns2, nt2, b.partial);
    ctx->launches++;
    trace_final_kernel<<<1, 32, 0, st>>>(b.partial, b.ntiles, b.partial + 2 * b.ntiles);
    ctx->launches++;
  }
  BEM_CUDA_TRY(ctx, cudaMemcpyAsync(S, b.partial + 2 * b.ntiles, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
  BEM_CUDA_TRY(ctx, cudaStreamSynchronize(st));
  return BEMGPU_OK;
}

}  // namespace

int bem_mixed_solve(bemgpu_ctx_s *ctx, const double *W, int n, int ns2, const double *G1, const double *G2,
                    cudaStream_t st, double S_out[2], bemgpu_solve_info_t *info) {
  const int nt2 = n - ns2;
  const size_t nn = (size_t)n * n, nm = (size_t)n * nt2, st2 = (size_t)ns2 * nt2;
  MixedBufs b;
  b.ntiles = ((ns2 + 31) / 32) * ((nt2 + 31) / 32);
  b.W32 = (float *)bem_workspace(ctx, "m_W32", 8 * nn);
  b.Wf = (float *)bem_workspace(ctx, "m_Wf", 8 * nn);
  b.H1f = (float *)bem_workspace(ctx, "m_H1f", 8 * (size_t)ns2 * ns2);
  b.H2f = (float *)bem_workspace(ctx, "m_H2f", 8 * (size_t)nt2 * nt2);
  b.Y32 = (float *)bem_workspace(ctx, "m_Y32", 8 * nm);
  b.R32 = (float *)bem_workspace(ctx, "m_R32", 8 * nm);
  b.XH32 = (float *)bem_workspace(ctx, "m_XH32", 8 * st2);
  b.H1 = (double *)bem_workspace(ctx, "m_H1", 16 * (size_t)ns2 * ns2);
  b.H2 = (double *)bem_workspace(ctx, "m_H2", 16 * (size_t)nt2 * nt2);
  b.Y = (double *)bem_workspace(ctx, "m_Y", 16 * nm);
  b.R64 = (double *)bem_workspace(ctx, "m_R64", 16 * nm);
  b.XH = (double *)bem_workspace(ctx, "m_XH", 16 * st2);
  b.B1 = (double *)bem_workspace(ctx, "m_B1", 16 * st2);
  b.C = (double *)bem_workspace(ctx, "m_C", 16 * st2);
  b.rmax = (double *)bem_workspace(ctx, "m_rmax", 8 * (size_t)n);
  b.partial = (double *)bem_workspace(ctx, "m_partial", 16 * (size_t)b.ntiles + 64);
  b.ipiv = (int *)bem_workspace(ctx, "m_ipiv", 4 * (size_t)n);
  b.info = (int *)bem_workspace(ctx, "m_info", 16);
  bool ok = b.W32 && b.Wf && b.H1f && b.H2f && b.Y32 && b.R32 && b.XH32 && b.H1 && b.H2 && b.Y && b.R64 && b.XH &&
            b.B1 && b.C && b.rmax && b.partial && b.ipiv && b.info;
  ok = ok && alloc_ell(ctx, "m_eW", n, b.eW) && alloc_ell(ctx, "m_eH1", ns2, b.eH1) && alloc_ell(ctx, "m_eH2", nt2, b.eH2);
  if (!ok) return bem_fail(ctx, BEMGPU_ERR_OOM, "mixed solve: workspace allocation failed (n=%d)", n);
  cudaEvent_t *ev = ctx->ev;
  const dim3 gn((n + 255) / 256, n), gm((n + 255) / 256, nt2);
  {
    ProfScope ps(ctx, BEMGPU_K_LU_PANEL, st, 0.0, 56.0 * nn + 40.0 * ((double)ns2 * ns2 + (double)nt2 * nt2));
    c128_to_c64_kernel<<<gn, 256, 0, st>>>(W, n, b.W32, n, n, n);
    ctx->launches++;
    split_near(ctx, W, n, TAU_RESIDUAL, b.rmax, b.eW, b.Wf, st);
    sym64_kernel<<<dim3((ns2 + 255) / 256, ns2), 256, 0, st>>>(G1, ns2, ns2, b.H1);
    ctx->launches++;
    sym64_kernel<<<dim3((nt2 + 255) / 256, nt2), 256, 0, st>>>(G2, nt2, nt2, b.H2);
    ctx->launches++;
    split_near(ctx, b.H1, ns2, TAU_TRACE, b.rmax, b.eH1, b.H1f, st);
    split_near(ctx, b.H2, nt2, TAU_TRACE, b.rmax, b.eH2, b.H2f, st);
  }
  BEM_CUDA_TRY(ctx, cudaGetLastError());
  cudaEventRecord(ev[1], st);
  int rc = bem_cgetrf(ctx, b.W32, n, n, b.ipiv, b.info, st);  // NOLINT
  if (rc) return rc;
  cudaEventRecord(ev[2], st);
  identity_cols_c64_kernel<<<gm, 256, 0, st>>>(b.R32, n, n, ns2, nt2);
  ctx->launches++;
  rc = bem_cgetrs(ctx, b.W32, n, n, b.ipiv, b.R32, n, nt2, st);
  if (rc) return rc;
  update_kernel<<<gm, 256, 0, st>>>(b.Y, b.R32, b.Y32, n, n, 0);
  ctx->launches++;
  cudaEventRecord(ev[3], st);
  int hinfo = 0;
  BEM_CUDA_TRY(ctx, cudaMemcpyAsync(&hinfo, b.info, sizeof(int), cudaMemcpyDeviceToHost, st));
  BEM_CUDA_TRY(ctx, cudaStreamSynchronize(st));
  if (hinfo != 0) return bem_fail(ctx, BEMGPU_ERR_SINGULAR, "mixed solve: zero pivot at column %d", hinfo);
  cudaEventRecord(ev[4], st);
  const float mone[2] = {-1.f, 0.f};
  const double zero64[2] = {0.0, 0.0};
  double Sprev[2] = {0, 0}, S[2] = {0, 0};
  int iters = 0;
  double err = 1.0, err_prev = 1.0;
  const int max_iters = 4;
  while (iters < max_iters) {
    // R = E_t - W_far Y - W_near Y
    rc = bem_cgemm_comp64(ctx, BEMGPU_K_REFINE_GEMM, n, nt2, n, mone, b.Wf, n, b.Y32, n, zero64, b.R64, n, st);
    if (rc) return rc;
    {
      ProfScope ps(ctx, BEMGPU_K_NEAR_SPMM, st, 8.0 * n * (double)nt2 * 300, 40.0 * n * (double)nt2);
      ell_left_kernel<<<gm, 256, 0, st>>>(b.eW.col, b.eW.val, b.eW.cnt, n, b.Y, n, b.R64, n, -1.0, ns2, b.R32, n);
      ctx->launches++;
    }
    rc = bem_cgetrs(ctx, b.W32, n, n, b.ipiv, b.R32, n, nt2, st);
    if (rc) return rc;
    update_kernel<<<gm, 256, 0, st>>>(b.Y, b.R32, b.Y32, n, n, 1);
    ctx->launches++;
    iters++;
    Sprev[0] = S[0];
    Sprev[1] = S[1];
    rc = spectral_trace(ctx, b, n, ns2, nt2, st, S);
    if (rc) return rc;
    if (iters == 1) continue;  // the spectral power of the unrefined solve is not needed
    err_prev = err;
    err = fabs(S[0] - Sprev[0]) / fmax(fabs(S[0]), 1e-300);
    // converged, or stalled at the accuracy floor of the residual
    if (err < 3e-7 || err > 0.5 * err_prev) break;
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
  }
  if (err > 1e-6) return bem_fail(ctx, BEMGPU_ERR_NO_CONVERGE, "mixed solve: refinement stalled at %.2e", err);
  return BEMGPU_OK;
}
