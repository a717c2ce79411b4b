// Dense complex128 linear algebra for the plain (FP64) path:
//   LU with partial pivoting (the zgetrf of inverse(), src/util/DenseMatrix.cpp:65-77),
//   the corresponding solve, and a complex GEMM (src/util/MatrixOperations.cpp:70-74).
//
// All matrices are column-major with interleaved (re, im) doubles, as the
// reference's ComplexDenseMatrix stores them (src/util/DenseMatrix.h:195-198).
//
// LU: right-looking, panel width NB.  The panel is factored one column per
// launch (scale + rank-1 update of the panel + pivot search across CTAs, the
// last CTA to finish reduces the pivot and swaps the rows inside the panel),
// then the row interchanges are applied outside the panel, the U12 block is
// solved with the unit-lower L11 (warp per right-hand side, L11 in shared
// memory) and the trailing matrix is updated by the complex GEMM.
// Pivot choice is LAPACK's: the first row of largest |re|+|im| (izamax).
#include "bemgpu_internal.h"

#include <algorithm>

namespace {

constexpr int NB = 64;  // panel width

struct cd {
  double r, i;
};
__device__ __forceinline__ cd cmul(cd a, cd b) { return {a.r * b.r - a.i * b.i, a.r * b.i + a.i * b.r}; }
__device__ __forceinline__ cd cld(const double *A, int64_t idx) {
  double2 v = reinterpret_cast<const double2 *>(A)[idx];
  return {v.x, v.y};
}
__device__ __forceinline__ void cst(double *A, int64_t idx, cd v) {
  reinterpret_cast<double2 *>(A)[idx] = make_double2(v.r, v.i);
}
__device__ __forceinline__ cd crecip(cd a) {
  double d = a.r * a.r + a.i * a.i;
  return {a.r / d, -a.i / d};
}

// ---------------- panel factorization ----------------
struct PivCand {
  double val;
  int idx;
  int pad;
};

constexpr int PANEL_THREADS = 256;

// Step jj of the panel [k0, k0+w): applies the pending scale + rank-1 update
// of column jj-1 to rows >= k0+jj, then selects and swaps the pivot of column jj.
// With jj == w it only applies the final scale of column w-1.
__global__ void __launch_bounds__(PANEL_THREADS) panel_step_kernel(double *A, int64_t lda, int n, int k0, int w, int jj,
                                                                   int *ipiv, int *info, PivCand *cand,
                                                                   unsigned int *counter) {
  const int r0 = k0 + jj;  // first active row
  const int nrows = n - r0;
  double bestv = -1.0;
  int besti = 0x7fffffff;
  if (jj > 0) {
    const int pr = k0 + jj - 1;  // pivot row/column of the previous step
    const cd piv = cld(A, pr + lda * (int64_t)pr);
    const bool zero = (piv.r == 0.0 && piv.i == 0.0);
    const cd rp = zero ? cd{0, 0} : crecip(piv);
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nrows; t += gridDim.x * blockDim.x) {
      const int r = r0 + t;
      cd l = cld(A, r + lda * (int64_t)pr);
      if (!zero) {
        l = cmul(l, rp);
        cst(A, r + lda * (int64_t)pr, l);
      }
      for (int c = jj; c < w; c++) {
        const int64_t col = (int64_t)(k0 + c) * lda;
        const cd u = cld(A, pr + col);
        cd a = cld(A, r + col);
        a.r -= l.r * u.r - l.i * u.i;
        a.i -= l.r * u.i + l.i * u.r;
        cst(A, r + col, a);
        if (c == jj) {
          const double v = fabs(a.r) + fabs(a.i);
          if (v > bestv || (v == bestv && r < besti)) { bestv = v; besti = r; }
        }
      }
    }
  } else {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nrows; t += gridDim.x * blockDim.x) {
      const int r = r0 + t;
      const cd a = cld(A, r + lda * (int64_t)(k0));
      const double v = fabs(a.r) + fabs(a.i);
      if (v > bestv || (v == bestv && r < besti)) { bestv = v; besti = r; }
    }
  }
  if (jj == w) return;  // final scale only
  // block argmax
  __shared__ double sv[PANEL_THREADS];
  __shared__ int si[PANEL_THREADS];
  __shared__ bool last;
  sv[threadIdx.x] = bestv;
  si[threadIdx.x] = besti;
  __syncthreads();
  for (int s = PANEL_THREADS / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      const double v2 = sv[threadIdx.x + s];
      const int i2 = si[threadIdx.x + s];
      if (v2 > sv[threadIdx.x] || (v2 == sv[threadIdx.x] && i2 < si[threadIdx.x])) {
        sv[threadIdx.x] = v2;
        si[threadIdx.x] = i2;
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    cand[blockIdx.x] = {sv[0], si[0], 0};
    __threadfence();
    const unsigned int prev = atomicAdd(counter, 1u);
    last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  // last CTA: global argmax, record the pivot, swap rows inside the panel
  __shared__ int piv_row;
  if (threadIdx.x == 0) {
    double bv = -1.0;
    int bi = r0;
    for (int b = 0; b < gridDim.x; b++) {
      const volatile PivCand *vc = (const volatile PivCand *)cand + b;
      const double cv = vc->val;
      const int ci = vc->idx;
      if (ci == 0x7fffffff) continue;
      if (cv > bv || (cv == bv && ci < bi)) { bv = cv; bi = ci; }
    }
    if (bv == 0.0) {
      bi = r0;
      if (*info == 0) *info = r0 + 1;
    }
    ipiv[r0] = bi;
    piv_row = bi;
    *counter = 0u;
  }
  __syncthreads();
  const int p = piv_row;
  if (p != r0) {
    for (int c = threadIdx.x; c < w; c += blockDim.x) {
      const int64_t col = (int64_t)(k0 + c) * lda;
      const cd a = cld(A, r0 + col), b = cld(A, p + col);
      cst(A, r0 + col, b);
      cst(A, p + col, a);
    }
  }
}

// Applies the interchanges ipiv[k1..k2) to columns [c0, c1) (zlaswp).
__global__ void laswp_kernel(double *A, int64_t lda, int c0, int c1, int k1, int k2, const int *ipiv) {
  const int c = c0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= c1) return;
  const int64_t col = (int64_t)c * lda;
  for (int k = k1; k < k2; k++) {
    const int p = ipiv[k];
    if (p != k) {
      const cd a = cld(A, k + col), b = cld(A, p + col);
      cst(A, k + col, b);
      cst(A, p + col, a);
    }
  }
}

// B[0:w, :] <- L11^{-1} B (unit lower) or U11^{-1} B (upper) with the w x w
// diagonal block in shared memory; one warp per right-hand-side column, lane
// holds rows lane and lane+32.
template <bool UPPER>
__global__ void __launch_bounds__(256) trsm_block_kernel(const double *Ad, int64_t lda, int w, double *B, int64_t ldb,
                                                         int ncols) {
  extern __shared__ double2 Ls[];  // NB * NB
  for (int idx = threadIdx.x; idx < w * w; idx += blockDim.x) {
    const int r = idx % w, c = idx / w;
    Ls[r + NB * c] = reinterpret_cast<const double2 *>(Ad)[r + lda * (int64_t)c];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int nwarps = blockDim.x >> 5;
  for (int col = blockIdx.x * nwarps + warp; col < ncols; col += gridDim.x * nwarps) {
    double2 *b = reinterpret_cast<double2 *>(B) + ldb * (int64_t)col;
    cd x0 = {0, 0}, x1 = {0, 0};
    if (lane < w) x0 = {b[lane].x, b[lane].y};
    if (lane + 32 < w) x1 = {b[lane + 32].x, b[lane + 32].y};
    if (!UPPER) {
      for (int i = 0; i < w; i++) {
        const cd xi = {__shfl_sync(0xffffffffu, i < 32 ? x0.r : x1.r, i & 31),
                       __shfl_sync(0xffffffffu, i < 32 ? x0.i : x1.i, i & 31)};
        if (lane > i && lane < w) {
          const double2 l = Ls[lane + NB * i];
          x0.r -= l.x * xi.r - l.y * xi.i;
          x0.i -= l.x * xi.i + l.y * xi.r;
        }
        if (lane + 32 > i && lane + 32 < w) {
          const double2 l = Ls[lane + 32 + NB * i];
          x1.r -= l.x * xi.r - l.y * xi.i;
          x1.i -= l.x * xi.i + l.y * xi.r;
        }
      }
    } else {
      for (int i = w - 1; i >= 0; i--) {
        // x_i /= U_ii on the owning lane, then broadcast
        if (i < 32 && lane == i) {
          const double2 d = Ls[i + NB * i];
          x0 = cmul(x0, crecip({d.x, d.y}));
        }
        if (i >= 32 && lane == i - 32) {
          const double2 d = Ls[i + NB * i];
          x1 = cmul(x1, crecip({d.x, d.y}));
        }
        const cd xi = {__shfl_sync(0xffffffffu, i < 32 ? x0.r : x1.r, i & 31),
                       __shfl_sync(0xffffffffu, i < 32 ? x0.i : x1.i, i & 31)};
        if (lane < i) {
          const double2 u = Ls[lane + NB * i];
          x0.r -= u.x * xi.r - u.y * xi.i;
          x0.i -= u.x * xi.i + u.y * xi.r;
        }
        if (lane + 32 < i) {
          const double2 u = Ls[lane + 32 + NB * i];
          x1.r -= u.x * xi.r - u.y * xi.i;
          x1.i -= u.x * xi.i + u.y * xi.r;
        }
      }
    }
    if (lane < w) b[lane] = make_double2(x0.r, x0.i);
    if (lane + 32 < w) b[lane + 32] = make_double2(x1.r, x1.i);
  }
}

// ---------------- complex GEMM (FP64 FMA pipe) ----------------
// C = alpha op(A) B + beta C, 64x64 complex tile per CTA, 4x4 per thread.
constexpr int GBM = 64, GBN = 64, GBK = 8;

template <bool CONJ_A>
__global__ void __launch_bounds__(256) zgemm_kernel(int m, int n, int k, cd alpha, const double *__restrict__ A,
                                                    int64_t lda, const double *__restrict__ B, int64_t ldb, cd beta,
                                                    double *__restrict__ C, int64_t ldc) {
  __shared__ double2 As[GBK][GBM];
  __shared__ double2 Bs[GBK][GBN];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int m0 = blockIdx.x * GBM, n0 = blockIdx.y * GBN;
  const double2 *A2 = reinterpret_cast<const double2 *>(A);
  const double2 *B2 = reinterpret_cast<const double2 *>(B);
  cd acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int b = 0; b < 4; b++) acc[a][b] = {0, 0};
  for (int kk0 = 0; kk0 < k; kk0 += GBK) {
    // A tile: GBM x GBK
#pragma unroll
    for (int e = 0; e < 2; e++) {
      const int idx = threadIdx.x + 256 * e;
      int r, kk;
      if (!CONJ_A) { r = idx % GBM; kk = idx / GBM; }
      else { kk = idx % GBK; r = idx / GBK; }
      const int gr = m0 + r, gk = kk0 + kk;
      double2 v = make_double2(0, 0);
      if (gr < m && gk < k) {
        if (!CONJ_A) v = A2[gr + lda * (int64_t)gk];
        else { v = A2[gk + lda * (int64_t)gr]; v.y = -v.y; }
      }
      As[kk][r] = v;
    }
#pragma unroll
    for (int e = 0; e < 2; e++) {
      const int idx = threadIdx.x + 256 * e;
      const int kk = idx % GBK, c = idx / GBK;
      const int gk = kk0 + kk, gc = n0 + c;
      double2 v = make_double2(0, 0);
      if (gk < k && gc < n) v = B2[gk + ldb * (int64_t)gc];
      Bs[kk][c] = v;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < GBK; kk++) {
      double2 a[4], b[4];
#pragma unroll
      for (int q = 0; q < 4; q++) { a[q] = As[kk][ty + 16 * q]; b[q] = Bs[kk][tx + 16 * q]; }
#pragma unroll
      for (int p = 0; p < 4; p++)
#pragma unroll
        for (int q = 0; q < 4; q++) {
          acc[p][q].r = fma(a[p].x, b[q].x, acc[p][q].r);
          acc[p][q].r = fma(-a[p].y, b[q].y, acc[p][q].r);
          acc[p][q].i = fma(a[p].x, b[q].y, acc[p][q].i);
          acc[p][q].i = fma(a[p].y, b[q].x, acc[p][q].i);
        }
    }
    __syncthreads();
  }
  double2 *C2 = reinterpret_cast<double2 *>(C);
  const bool beta0 = (beta.r == 0.0 && beta.i == 0.0);
#pragma unroll
  for (int p = 0; p < 4; p++)
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int r = m0 + ty + 16 * p, c = n0 + tx + 16 * q;
      if (r < m && c < n) {
        cd v = cmul(alpha, acc[p][q]);
        if (!beta0) {
          const double2 o = C2[r + ldc * (int64_t)c];
          const cd ob = cmul(beta, {o.x, o.y});
          v.r += ob.r;
          v.i += ob.i;
        }
        C2[r + ldc * (int64_t)c] = make_double2(v.r, v.i);
      }
    }
}

constexpr int TRSM_SMEM = NB * NB * (int)sizeof(double2);

int set_trsm_attrs(bemgpu_ctx_s *ctx) {
  static bool done[64] = {false};
  if (done[ctx->device]) return BEMGPU_OK;
  BEM_CUDA_TRY(ctx, cudaFuncSetAttribute(trsm_block_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, TRSM_SMEM));
  BEM_CUDA_TRY(ctx, cudaFuncSetAttribute(trsm_block_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, TRSM_SMEM));
  done[ctx->device] = true;
  return BEMGPU_OK;
}

}  // namespace

int bem_zgemm(bemgpu_ctx_s *ctx, int kind, char opA, int m, int n, int k, const double alpha[2], const double *A, int64_t lda,
              const double *B, int64_t ldb, const double beta[2], double *C, int64_t ldc, cudaStream_t stream) {
  if (m <= 0 || n <= 0) return BEMGPU_OK;
  dim3 grd((m + GBM - 1) / GBM, (n + GBN - 1) / GBN);
  cd al = {alpha[0], alpha[1]}, be = {beta[0], beta[1]};
  ProfScope ps(ctx, kind, stream, 8.0 * m * n * k, 16.0 * ((double)m * k + (double)k * n + 2.0 * m * n));
  if (opA == 'C') {
    zgemm_kernel<true><<<grd, 256, 0, stream>>>(m, n, k, al, A, lda, B, ldb, be, C, ldc);
    ctx->launches++;
  } else {
    zgemm_kernel<false><<<grd, 256, 0, stream>>>(m, n, k, al, A, lda, B, ldb, be, C, ldc);
    ctx->launches++;
  }
  BEM_CUDA_TRY(ctx, cudaGetLastError());
  return BEMGPU_OK;
}

int bem_zgetrf(bemgpu_ctx_s *ctx, double *A, int64_t lda, int n, int *d_ipiv, int *d_info, cudaStream_t stream) {
  if (int rc0 = set_trsm_attrs(ctx)) return rc0;
  PivCand *cand = (PivCand *)bem_workspace(ctx, "lu_cand", sizeof(PivCand) * 1024);
  unsigned int *counter = (unsigned int *)bem_workspace(ctx, "lu_counter", sizeof(unsigned int));
  if (!cand || !counter) return bem_fail(ctx, BEMGPU_ERR_OOM, "zgetrf: workspace");
  BEM_CUDA_TRY(ctx, cudaMemsetAsync(counter, 0, sizeof(unsigned int), stream));
  BEM_CUDA_TRY(ctx, cudaMemsetAsync(d_info, 0, sizeof(int), stream));
  const double mone[2] = {-1.0, 0.0}, one[2] = {1.0, 0.0};
  for (int k0 = 0; k0 < n; k0 += NB) {
    const int w = std::min(NB, n - k0);
    const int rows = n - k0;
    const int blocks = std::max(1, std::min(ctx->num_sms * 2, (rows + PANEL_THREADS - 1) / PANEL_THREADS));
    for (int jj = 0; jj <= w; jj++) {
      ProfScope ps(ctx, BEMGPU_K_LU_PANEL, stream, 8.0 * (rows - jj) * (w - jj), 16.0 * 2 * (rows - jj) * (w - jj));
      panel_step_kernel<<<blocks, PANEL_THREADS, 0, stream>>>(A, lda, n, k0, w, jj, d_ipiv, d_info, cand, counter);
      ctx->launches++;
    }
    BEM_CUDA_TRY(ctx, cudaGetLastError());
    // interchanges to the left and right of the panel
    if (k0 > 0) {
      ProfScope ps(ctx, BEMGPU_K_LU_PANEL, stream, 0.0, 64.0 * w * k0);
      laswp_kernel<<<(k0 + 127) / 128, 128, 0, stream>>>(A, lda, 0, k0, k0, k0 + w, d_ipiv);
      ctx->launches++;
    }
    if (k0 + w < n) {
      const int nr = n - k0 - w;
      double *A11 = A + 2 * (k0 + lda * (int64_t)k0);
      double *A12 = A + 2 * (k0 + lda * (int64_t)(k0 + w));
      const int tb = std::min((nr + 7) / 8, ctx->num_sms * 4);
      {
        ProfScope ps(ctx, BEMGPU_K_LU_PANEL, stream, 0.0, 64.0 * w * nr);
        laswp_kernel<<<(nr + 127) / 128, 128, 0, stream>>>(A, lda, k0 + w, n, k0, k0 + w, d_ipiv);
        ctx->launches++;
      }
      {
        ProfScope ps(ctx, BEMGPU_K_TRSM, stream, 4.0 * w * w * nr, 32.0 * w * nr);
        trsm_block_kernel<false><<<tb, 256, TRSM_SMEM, stream>>>(A11, lda, w, A12, lda, nr);
        ctx->launches++;
      }
      double *A21 = A + 2 * (k0 + w + lda * (int64_t)k0);
      double *A22 = A + 2 * (k0 + w + lda * (int64_t)(k0 + w));
      int rc = bem_zgemm(ctx, BEMGPU_K_LU_GEMM, 'N', nr, nr, w, mone, A21, lda, A12, lda, one, A22, lda, stream);
      if (rc) return rc;
    }
    BEM_CUDA_TRY(ctx, cudaGetLastError());
  }
  return BEMGPU_OK;
}

int bem_zgetrs(bemgpu_ctx_s *ctx, const double *A, int64_t lda, int n, const int *d_ipiv, double *B, int64_t ldb,
               int nrhs, cudaStream_t stream) {
  if (int rc0 = set_trsm_attrs(ctx)) return rc0;
  const double mone[2] = {-1.0, 0.0}, one[2] = {1.0, 0.0};
  {
    ProfScope ps(ctx, BEMGPU_K_LU_PANEL, stream, 0.0, 64.0 * n * nrhs);
    laswp_kernel<<<(nrhs + 127) / 128, 128, 0, stream>>>(B, ldb, 0, nrhs, 0, n, d_ipiv);
    ctx->launches++;
  }
  const int tb = std::min((nrhs + 7) / 8, ctx->num_sms * 4);
  // forward: L Y = P B
  for (int k0 = 0; k0 < n; k0 += NB) {
    const int w = std::min(NB, n - k0);
    const double *L11 = A + 2 * (k0 + lda * (int64_t)k0);
    double *Bk = B + 2 * (int64_t)k0;
    {
      ProfScope ps(ctx, BEMGPU_K_TRSM, stream, 4.0 * w * w * nrhs, 32.0 * w * nrhs);
      trsm_block_kernel<false><<<tb, 256, TRSM_SMEM, stream>>>(L11, lda, w, Bk, ldb, nrhs);
      ctx->launches++;
    }
    if (k0 + w < n) {
      const double *L21 = A + 2 * (k0 + w + lda * (int64_t)k0);
      int rc = bem_zgemm(ctx, BEMGPU_K_SOLVE_GEMM, 'N', n - k0 - w, nrhs, w, mone, L21, lda, Bk, ldb, one, B + 2 * (int64_t)(k0 + w), ldb,
                         stream);
      if (rc) return rc;
    }
  }
  // backward: U X = Y
  const int nblk = (n + NB - 1) / NB;
  for (int bi = nblk - 1; bi >= 0; bi--) {
    const int k0 = bi * NB;
    const int w = std::min(NB, n - k0);
    const double *U11 = A + 2 * (k0 + lda * (int64_t)k0);
    double *Bk = B + 2 * (int64_t)k0;
    {
      ProfScope ps(ctx, BEMGPU_K_TRSM, stream, 4.0 * w * w * nrhs, 32.0 * w * nrhs);
      trsm_block_kernel<true><<<tb, 256, TRSM_SMEM, stream>>>(U11, lda, w, Bk, ldb, nrhs);
      ctx->launches++;
    }
    if (k0 > 0) {
      const double *U01 = A + 2 * (lda * (int64_t)k0);
      int rc = bem_zgemm(ctx, BEMGPU_K_SOLVE_GEMM, 'N', k0, nrhs, w, mone, U01, lda, Bk, ldb, one, B, ldb, stream);
      if (rc) return rc;
    }
  }
  BEM_CUDA_TRY(ctx, cudaGetLastError());
  return BEMGPU_OK;
}
