// Dense complex linear algebra, complex128 (plain path) and complex64 (mixed path):
//   LU with partial pivoting (the zgetrf of inverse(), src/util/DenseMatrix.cpp:65-77),
//   the corresponding solve, and a complex GEMM (src/util/MatrixOperations.cpp:70-74).
//
// All matrices are column-major with interleaved (re, im) values, as the
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

constexpr int NB = 64;  // panel width of the FP64 LU and of the blocked solves
constexpr int NB_MAX = 128;  // widest LU panel (complex64: LuCfg<float>)
// LU panel width per type: complex64 uses 128-wide panels so that the trailing
// updates are K = 128 tensor-core products (half the passes over the trailing
// matrix of 64-wide panels); complex128 keeps 64 (its diagonal block must fit
// the triangular-solve kernel's shared memory).
template <typename T>
struct LuCfg {
  static constexpr int NBL = 64;
};
template <>
struct LuCfg<float> {
  static constexpr int NBL = 128;
};

template <typename T>
struct V2;
template <>
struct V2<double> {
  typedef double2 type;
  __device__ __forceinline__ static double2 make(double a, double b) { return make_double2(a, b); }
};
template <>
struct V2<float> {
  typedef float2 type;
  __device__ __forceinline__ static float2 make(float a, float b) { return make_float2(a, b); }
};

template <typename T>
struct cx {
  T r, i;
};
template <typename T>
__device__ __forceinline__ cx<T> cmul(cx<T> a, cx<T> b) {
  return {a.r * b.r - a.i * b.i, a.r * b.i + a.i * b.r};
}
template <typename T>
__device__ __forceinline__ cx<T> cld(const T *A, int64_t idx) {
  typename V2<T>::type v = reinterpret_cast<const typename V2<T>::type *>(A)[idx];
  return {v.x, v.y};
}
template <typename T>
__device__ __forceinline__ void cst(T *A, int64_t idx, cx<T> v) {
  reinterpret_cast<typename V2<T>::type *>(A)[idx] = V2<T>::make(v.r, v.i);
}
template <typename T>
__device__ __forceinline__ cx<T> crecip(cx<T> a) {
  T d = a.r * a.r + a.i * a.i;
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
template <typename T>
__global__ void __launch_bounds__(PANEL_THREADS) panel_step_kernel(T *A, int64_t lda, int n, int k0, int w, int jj,
                                                                   int *ipiv, int *info, PivCand *cand,
                                                                   unsigned int *counter) {
  const int r0 = k0 + jj;  // first active row
  const int nrows = n - r0;
  double bestv = -1.0;
  int besti = 0x7fffffff;
  if (jj > 0) {
    const int pr = k0 + jj - 1;  // pivot row/column of the previous step
    const cx<T> piv = cld(A, pr + lda * (int64_t)pr);
    const bool zero = (piv.r == T(0) && piv.i == T(0));
    const cx<T> rp = zero ? cx<T>{0, 0} : crecip(piv);
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nrows; t += gridDim.x * blockDim.x) {
      const int r = r0 + t;
      cx<T> l = cld(A, r + lda * (int64_t)pr);
      if (!zero) {
        l = cmul(l, rp);
        cst(A, r + lda * (int64_t)pr, l);
      }
      for (int c = jj; c < w; c++) {
        const int64_t col = (int64_t)(k0 + c) * lda;
        const cx<T> u = cld(A, pr + col);
        cx<T> a = cld(A, r + col);
        a.r -= l.r * u.r - l.i * u.i;
        a.i -= l.r * u.i + l.i * u.r;
        cst(A, r + col, a);
        if (c == jj) {
          const double v = fabs((double)a.r) + fabs((double)a.i);
          if (v > bestv || (v == bestv && r < besti)) { bestv = v; besti = r; }
        }
      }
    }
  } else {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nrows; t += gridDim.x * blockDim.x) {
      const int r = r0 + t;
      const cx<T> a = cld(A, r + lda * (int64_t)(k0));
      const double v = fabs((double)a.r) + fabs((double)a.i);
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
      const cx<T> a = cld(A, r0 + col), b = cld(A, p + col);
      cst(A, r0 + col, b);
      cst(A, p + col, a);
    }
  }
}

// Applies the interchanges ipiv[k1..k2) to columns [c0, c1) (zlaswp).
template <typename T>
__global__ void laswp_kernel(T *A, int64_t lda, int c0, int c1, int k1, int k2, const int *ipiv) {
  const int c = c0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= c1) return;
  const int64_t col = (int64_t)c * lda;
  for (int k = k1; k < k2; k++) {
    const int p = ipiv[k];
    if (p != k) {
      const cx<T> a = cld(A, k + col), b = cld(A, p + col);
      cst(A, k + col, b);
      cst(A, p + col, a);
    }
  }
}

// The row interchanges ipiv[0..n) (applied in order, as laswp does) as one
// permutation: perm[i] = the row whose content ends in row i.  One CTA: ipiv
// and the row labels in shared memory, one thread replays the swaps.
constexpr int PERM_MAX_N = 24576;  // 2 x 96 KB of shared memory

__global__ void perm_from_ipiv_kernel(const int *__restrict__ ipiv, int n, int *__restrict__ perm) {
  extern __shared__ int perm_smem[];
  int *pr = perm_smem, *pv = perm_smem + n;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    pr[i] = i;
    pv[i] = ipiv[i];
  }
  __syncthreads();
  if (threadIdx.x == 0)
    for (int k = 0; k < n; k++) {
      const int p = pv[k];
      if (p != k) {
        const int t = pr[k];
        pr[k] = pr[p];
        pr[p] = t;
      }
    }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) perm[i] = pr[i];
}

// out[i, c] = B[perm[i], c] for complex64 column-major B (n x ncols).
__global__ void gather_rows_c64_kernel(const float *__restrict__ B, int64_t ldb, const int *__restrict__ perm, int n,
                                       float *__restrict__ out, int64_t ldo) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t c = blockIdx.y;
  if (i >= n) return;
  reinterpret_cast<float2 *>(out)[i + ldo * c] = reinterpret_cast<const float2 *>(B)[perm[i] + ldb * c];
}

// The same interchanges for a panel of at most LASWP_MAXW rows, as one
// permutation: warp 0 of each CTA replays the swaps on row labels in shared
// memory (the panel's rows and the pivot rows below it), which gives for
// every touched row the row its final content comes from; then one warp per
// column gathers those entries into registers and writes them back (all
// loads of a column before its stores).  Same result as the swaps in order;
// each entry moves once instead of once per swap that touches it.
constexpr int LASWP_MAXW = 128;
constexpr int LASWP_WARPS = 8;

template <typename T>
__global__ void __launch_bounds__(32 * LASWP_WARPS)
    laswp_perm_kernel(T *A, int64_t lda, int c0, int c1, int k1, int k2, const int *ipiv) {
  __shared__ int row[2 * LASWP_MAXW], from[2 * LASWP_MAXW];
  __shared__ int nslot, nmove;
  __shared__ int mdst[2 * LASWP_MAXW], msrc[2 * LASWP_MAXW];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, m = k2 - k1;
  if (warp == 0) {
    for (int s = lane; s < m; s += 32) {
      row[s] = k1 + s;
      from[s] = k1 + s;
    }
    if (lane == 0) nslot = m;
    __syncwarp();
    for (int k = k1; k < k2; k++) {
      const int p = ipiv[k];
      if (p == k) continue;
      int sp;
      if (p < k2) {
        sp = p - k1;
      } else {
        // the slot of pivot row p among the rows below the panel (appended
        // on first use)
        const int ns = nslot;
        int found = -1;
        for (int s0 = m; s0 < ns; s0 += 32) {
          const int s = s0 + lane;
          const unsigned hit = __ballot_sync(0xffffffffu, s < ns && row[s] == p);
          if (hit) {
            found = s0 + __ffs(hit) - 1;
            break;
          }
        }
        if (found < 0) {
          found = ns;
          if (lane == 0) {
            row[ns] = p;
            from[ns] = p;
            nslot = ns + 1;
          }
        }
        __syncwarp();
        sp = found;
      }
      if (lane == 0) {
        const int t = from[k - k1];
        from[k - k1] = from[sp];
        from[sp] = t;
      }
      __syncwarp();
    }
    if (lane == 0) {
      int c = 0;
      for (int s = 0; s < nslot; s++)
        if (from[s] != row[s]) {
          mdst[c] = row[s];
          msrc[c] = from[s];
          c++;
        }
      nmove = c;
    }
  }
  __syncthreads();
  const int nm = nmove;
  constexpr int PER = 2 * LASWP_MAXW / 32;
  for (int c = c0 + blockIdx.x * LASWP_WARPS + warp; c < c1; c += gridDim.x * LASWP_WARPS) {
    const int64_t col = (int64_t)c * lda;
    cx<T> v[PER];
#pragma unroll
    for (int j = 0; j < PER; j++) {
      const int i = lane + 32 * j;
      if (i < nm) v[j] = cld(A, msrc[i] + col);
    }
    __syncwarp();
#pragma unroll
    for (int j = 0; j < PER; j++) {
      const int i = lane + 32 * j;
      if (i < nm) cst(A, mdst[i] + col, v[j]);
    }
  }
}

// ---------------- cooperative panel factorization ----------------
// The whole panel [k0, k0 + w) in one cooperative launch: CTA g keeps rows
// [k0 + g chunk, k0 + (g+1) chunk) of the panel in shared memory (row-major),
// and per column j: (1) each CTA publishes its local pivot candidate (value,
// row, the row's w entries) and, if it owns the diagonal row, that row;
// (2) one grid barrier; (3) every CTA reduces the G candidates to the same
// pivot, the owners of the diagonal and pivot rows exchange them, and each
// CTA scales column j and applies the rank-1 update to its own rows.  One
// barrier per column (candidate slots double-buffered by column parity); the
// barrier's spin is bounded and sets *err when it runs out.  Same pivots and
// arithmetic as the one-launch-per-column kernel above.
constexpr int COOP_THREADS = 256;
constexpr unsigned COOP_SPIN_LIMIT = 1u << 24;

__device__ __forceinline__ void arrive_release_u32(unsigned *p) {
  asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(p) : "memory");
}

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

template <typename T>
__global__ void __launch_bounds__(COOP_THREADS)
    panel_coop_kernel(T *A, int64_t lda, int n, int k0, int w, int chunk, int *ipiv, int *info, T *cval,
                      int *crow, T *cdata_raw, T *drow_raw, unsigned *counter, int *err,
                      unsigned long long *best, int64_t strideA) {
  typedef typename V2<T>::type T2;
  extern __shared__ __align__(16) unsigned char coop_smem[];
  {
    // a batch of equal-size matrices (blockIdx.y): its own matrix, pivots,
    // candidate slots and barrier; the CTAs of different matrices never wait
    // on one another
    const int64_t bb = blockIdx.y;
    A += bb * strideA;
    ipiv += bb * n;
    info += bb;
    cval += bb * 2 * gridDim.x;
    crow += bb * 2 * gridDim.x;
    cdata_raw += bb * 2 * 2 * (int64_t)gridDim.x * w;
    drow_raw += bb * 2 * 2 * (int64_t)w;
    counter += bb;
    best += 4 * bb;
  }
  T2 *P = reinterpret_cast<T2 *>(coop_smem);  // chunk x w, P[i * w + c]
  T2 *prow = P + (int64_t)chunk * w;           // the pivot (U) row of the current column
  T2 *A2 = reinterpret_cast<T2 *>(A);
  T2 *cdata = reinterpret_cast<T2 *>(cdata_raw);
  T2 *drow = reinterpret_cast<T2 *>(drow_raw);
  __shared__ T red_v[COOP_THREADS / 32];
  __shared__ int red_i[COOP_THREADS / 32], red_w[COOP_THREADS / 32];
  __shared__ int s_row, s_win;
  __shared__ bool s_abort, s_zero;
  const int G = gridDim.x, g = blockIdx.x, tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int rbeg = k0 + g * chunk, rend = min(n, rbeg + chunk);
  const int nloc = max(0, rend - rbeg);
  for (int idx = tid; idx < nloc * w; idx += COOP_THREADS) {
    const int i = idx % nloc, c = idx / nloc;
    P[i * w + c] = A2[(rbeg + i) + lda * (int64_t)(k0 + c)];
  }
  if (tid == 0) s_abort = false;
  __syncthreads();
  for (int j = 0; j < w; j++) {
    const int dr = k0 + j, par = j & 1;
    // (1) local candidate: first row of largest |re| + |im| in column j, rows >= dr
    T bv = T(-1);
    int bi = 0x7fffffff;
    for (int i = tid; i < nloc; i += COOP_THREADS) {
      const int r = rbeg + i;
      if (r < dr) continue;
      const T2 a = P[i * w + j];
      const T v = fabs(a.x) + fabs(a.y);
      if (v > bv || (v == bv && r < bi)) {
        bv = v;
        bi = r;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const T v2 = __shfl_xor_sync(0xffffffffu, bv, o);
      const int i2 = __shfl_xor_sync(0xffffffffu, bi, o);
      if (v2 > bv || (v2 == bv && i2 < bi)) {
        bv = v2;
        bi = i2;
      }
    }
    if (lane == 0) {
      red_v[wid] = bv;
      red_i[wid] = bi;
    }
    __syncthreads();
    // warp 0 publishes the CTA's candidate (value, row, row data) and the
    // diagonal row, then its lane 0 takes the grid barrier; the other warps
    // wait at the CTA barrier that follows
    if (wid == 0) {
      if (lane == 0) {
        for (int q = 1; q < COOP_THREADS / 32; q++)
          if (red_v[q] > bv || (red_v[q] == bv && red_i[q] < bi)) {
            bv = red_v[q];
            bi = red_i[q];
          }
        if constexpr (sizeof(T) == 4) {
          // complex64: the candidate goes into one packed key per column (slot
          // j % 3), magnitude bits over the complemented row, so the largest
          // key is the largest |re| + |im| and, among equal ones, the first row
          if (bi != 0x7fffffff)
            atomicMax(best + j % 3, ((unsigned long long)__float_as_uint((float)bv) << 32) |
                                        (unsigned long long)(0xffffffffu - (unsigned)bi));
        } else {
          cval[par * G + g] = bv;
          crow[par * G + g] = bi;
        }
      }
      bi = __shfl_sync(0xffffffffu, bi, 0);
      if (bi != 0x7fffffff)
        for (int c = lane; c < w; c += 32) cdata[(int64_t)(par * G + g) * w + c] = P[(bi - rbeg) * w + c];
      if (dr >= rbeg && dr < rend)
        for (int c = lane; c < w; c += 32) drow[par * w + c] = P[(dr - rbeg) * w + c];
      __syncwarp();
      // (2) grid barrier
      if (lane == 0) {
        // the warp's publishing writes (ordered before by the warp barrier and
        // the fence) are released with the arrival; the acquire load orders
        // the reads after the CTA barrier below
        __threadfence();
        arrive_release_u32(counter);
        const unsigned target = (unsigned)G * (unsigned)(j + 1);
        unsigned it = 0;
        while (ld_acquire_u32(counter) < target) {
          if (++it > COOP_SPIN_LIMIT) {
            atomicExch(err, 1);
            s_abort = true;
            break;
          }
        }
      }
    }
    __syncthreads();
    if (s_abort) return;
    // (3) the pivot, the pivot (U) row into shared memory, and the interchange
    if constexpr (sizeof(T) == 4) {
      if (wid == 0) {
        int row = 0, win = -1, zi = 0;
        if (lane == 0) {
          const unsigned long long key = __ldcg(best + j % 3);
          // slot (j - 1) % 3 was read by every CTA before it arrived here; it
          // is next used at column j + 2, after the barrier this CTA passes later
          if (g == 0 && j >= 1) atomicExch(best + (j - 1) % 3, 0ull);
          zi = (key >> 32) == 0ull;
          row = zi ? dr : (int)(0xffffffffu - (unsigned)(key & 0xffffffffull));
          win = zi ? -1 : (row - k0) / chunk;
          if (g == 0) {
            ipiv[dr] = row;
            if (zi && *info == 0) *info = dr + 1;
          }
          s_zero = zi != 0;
          s_row = row;
        }
        row = __shfl_sync(0xffffffffu, row, 0);
        win = __shfl_sync(0xffffffffu, win, 0);
        for (int c = lane; c < w; c += 32)
          prow[c] = (row == dr || win < 0) ? __ldcg(drow + par * w + c)
                                           : __ldcg(cdata + (int64_t)(par * G + win) * w + c);
        __syncwarp();
        if (row != dr) {
          if (dr >= rbeg && dr < rend)
            for (int c = lane; c < w; c += 32) P[(dr - rbeg) * w + c] = prow[c];
          if (row >= rbeg && row < rend)
            for (int c = lane; c < w; c += 32) P[(row - rbeg) * w + c] = __ldcg(drow + par * w + c);
        }
      }
      __syncthreads();
    } else {
    bv = T(-1);
    bi = 0x7fffffff;
    int bw = 0;
    if constexpr (sizeof(T) == 8) {
    for (int q = tid; q < G; q += COOP_THREADS) {
      const T v = __ldcg(cval + par * G + q);
      const int r = __ldcg(crow + par * G + q);
      if (r == 0x7fffffff) continue;
      if (v > bv || (v == bv && r < bi)) {
        bv = v;
        bi = r;
        bw = q;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const T v2 = __shfl_xor_sync(0xffffffffu, bv, o);
      const int i2 = __shfl_xor_sync(0xffffffffu, bi, o);
      const int w2 = __shfl_xor_sync(0xffffffffu, bw, o);
      if (v2 > bv || (v2 == bv && i2 < bi)) {
        bv = v2;
        bi = i2;
        bw = w2;
      }
    }
    if (lane == 0) {
      red_v[wid] = bv;
      red_i[wid] = bi;
      red_w[wid] = bw;
    }
    __syncthreads();
    if (tid == 0) {
      int win = bw;
      for (int q = 1; q < COOP_THREADS / 32; q++)
        if (red_v[q] > bv || (red_v[q] == bv && red_i[q] < bi)) {
          bv = red_v[q];
          bi = red_i[q];
          win = red_w[q];
        }
      if (bi == 0x7fffffff) win = -1;
      const bool zero = !(bv > T(0));
      if (zero) bi = dr;
      s_zero = zero;
      s_row = bi;
      s_win = win;
      if (g == 0) {
        ipiv[dr] = bi;
        if (zero && *info == 0) *info = dr + 1;
      }
    }
    __syncthreads();
    }
      const int p = s_row;
      for (int c = tid; c < w; c += COOP_THREADS) {
        T2 v;
        if (p == dr || s_win < 0) {
          const T2 *src = drow + par * w + c;
          v = __ldcg(src);
        } else {
          v = __ldcg(cdata + (int64_t)(par * G + s_win) * w + c);
        }
        prow[c] = v;
      }
      __syncthreads();
      if (p != dr) {
        if (dr >= rbeg && dr < rend)
          for (int c = tid; c < w; c += COOP_THREADS) P[(dr - rbeg) * w + c] = prow[c];
        if (p >= rbeg && p < rend)
          for (int c = tid; c < w; c += COOP_THREADS) P[(p - rbeg) * w + c] = __ldcg(drow + par * w + c);
      }
      __syncthreads();
    }
    // scale column j below the diagonal and the rank-1 update of columns > j,
    // one warp per row (the row's multiplier is read before it is overwritten)
    const bool zero = s_zero;
    const T2 pv = prow[j];
    const cx<T> rp = zero ? cx<T>{0, 0} : crecip(cx<T>{pv.x, pv.y});
    for (int i = wid; i < nloc; i += COOP_THREADS / 32) {
      if (rbeg + i <= dr) continue;
      const T2 a0 = P[i * w + j];
      T2 l = a0;
      if (!zero) {
        const cx<T> ls = cmul(cx<T>{a0.x, a0.y}, rp);
        l = V2<T>::make(ls.r, ls.i);
      }
      __syncwarp();
      if (lane == 0) P[i * w + j] = l;
      for (int c = j + 1 + lane; c < w; c += 32) {
        const T2 u = prow[c];
        T2 a = P[i * w + c];
        a.x -= l.x * u.x - l.y * u.y;
        a.y -= l.x * u.y + l.y * u.x;
        P[i * w + c] = a;
      }
    }
    __syncthreads();
  }
  for (int idx = tid; idx < nloc * w; idx += COOP_THREADS) {
    const int i = idx % nloc, c = idx / nloc;
    A2[(rbeg + i) + lda * (int64_t)(k0 + c)] = P[i * w + c];
  }
}

// B[0:w, :] <- L11^{-1} B (unit lower) or U11^{-1} B (upper) with the w x w
// diagonal block (w <= 32 R) in shared memory; one warp per right-hand-side
// column, lane holds rows lane + 32 r, r < R.
template <typename T, bool UPPER, int R>
__global__ void __launch_bounds__(256) trsm_block_kernel(const T *Ad, int64_t lda, int w, T *B, int64_t ldb,
                                                         int ncols) {
  typedef typename V2<T>::type T2;
  constexpr int LDS = 32 * R;
  extern __shared__ __align__(16) unsigned char trsm_smem[];
  T2 *Ls = reinterpret_cast<T2 *>(trsm_smem);  // LDS * LDS
  for (int idx = threadIdx.x; idx < w * w; idx += blockDim.x) {
    const int r = idx % w, c = idx / w;
    Ls[r + LDS * c] = reinterpret_cast<const T2 *>(Ad)[r + lda * (int64_t)c];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int nwarps = blockDim.x >> 5;
  for (int col = blockIdx.x * nwarps + warp; col < ncols; col += gridDim.x * nwarps) {
    T2 *b = reinterpret_cast<T2 *>(B) + ldb * (int64_t)col;
    cx<T> x[R];
#pragma unroll
    for (int r = 0; r < R; r++) {
      x[r] = {0, 0};
      if (lane + 32 * r < w) x[r] = {b[lane + 32 * r].x, b[lane + 32 * r].y};
    }
    if (!UPPER) {
      for (int i = 0; i < w; i++) {
        cx<T> own = {0, 0};
#pragma unroll
        for (int r = 0; r < R; r++)
          if ((i >> 5) == r) own = x[r];
        const cx<T> xi = {__shfl_sync(0xffffffffu, own.r, i & 31), __shfl_sync(0xffffffffu, own.i, i & 31)};
#pragma unroll
        for (int r = 0; r < R; r++) {
          const int row = lane + 32 * r;
          if (row > i && row < w) {
            const T2 l = Ls[row + LDS * i];
            x[r].r -= l.x * xi.r - l.y * xi.i;
            x[r].i -= l.x * xi.i + l.y * xi.r;
          }
        }
      }
    } else {
      for (int i = w - 1; i >= 0; i--) {
        // x_i /= U_ii on the owning lane, then broadcast
        const T2 d = Ls[i + LDS * i];
        cx<T> own = {0, 0};
#pragma unroll
        for (int r = 0; r < R; r++)
          if ((i >> 5) == r) {
            if (lane == (i & 31)) x[r] = cmul(x[r], crecip(cx<T>{d.x, d.y}));
            own = x[r];
          }
        const cx<T> xi = {__shfl_sync(0xffffffffu, own.r, i & 31), __shfl_sync(0xffffffffu, own.i, i & 31)};
#pragma unroll
        for (int r = 0; r < R; r++) {
          const int row = lane + 32 * r;
          if (row < i) {
            const T2 u = Ls[row + LDS * i];
            x[r].r -= u.x * xi.r - u.y * xi.i;
            x[r].i -= u.x * xi.i + u.y * xi.r;
          }
        }
      }
    }
#pragma unroll
    for (int r = 0; r < R; r++)
      if (lane + 32 * r < w) b[lane + 32 * r] = V2<T>::make(x[r].r, x[r].i);
  }
}

// ---------------- complex GEMM (FMA pipes) ----------------
// C = alpha op(A) B + beta C, BM x BN complex tile per CTA, TM x TN per thread,
// 256 threads.  FP64: 64x64 tiles; FP32: 128x64 tiles.
// COMP: the FP32 sums of each BK-deep K tile are added into a two-float
// (hi + lo) running sum (TwoSum), so accumulation error does not grow with K;
// TC is the output type (double to accumulate FP32 products into an FP64 C).
template <typename T, int BM, int BN, int TM, int TN, int BK, bool CONJ_A, typename TC = T, bool COMP = false>
__global__ void __launch_bounds__(256) cgemm_fma_kernel(int m, int n, int k, cx<T> alpha, const T *__restrict__ A,
                                                        int64_t lda, const T *__restrict__ B, int64_t ldb, cx<TC> beta,
                                                        TC *__restrict__ C, int64_t ldc, int64_t sA, int64_t sB,
                                                        int64_t sC) {
  typedef typename V2<T>::type T2;
  // strided batch: problem blockIdx.z (strides in elements of T / TC)
  A += sA * blockIdx.z;
  B += sB * blockIdx.z;
  C += sC * blockIdx.z;
  constexpr int TX = BN / TN, TY = BM / TM;
  static_assert(TX * TY == 256, "256 threads");
  __shared__ T2 As[BK][BM];
  __shared__ T2 Bs[BK][BN];
  const int tx = threadIdx.x % TX, ty = threadIdx.x / TX;
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
  const T2 *A2 = reinterpret_cast<const T2 *>(A);
  const T2 *B2 = reinterpret_cast<const T2 *>(B);
  cx<T> acc[TM][TN];
  cx<T> lo[COMP ? TM : 1][COMP ? TN : 1];
  cx<T> part[COMP ? TM : 1][COMP ? TN : 1];
#pragma unroll
  for (int a = 0; a < TM; a++)
#pragma unroll
    for (int b = 0; b < TN; b++) acc[a][b] = {0, 0};
  if (COMP) {
#pragma unroll
    for (int a = 0; a < (COMP ? TM : 1); a++)
#pragma unroll
      for (int b = 0; b < (COMP ? TN : 1); b++) { lo[a][b] = {0, 0}; part[a][b] = {0, 0}; }
  }
  for (int kk0 = 0; kk0 < k; kk0 += BK) {
#pragma unroll
    for (int e = 0; e < (BM * BK) / 256; e++) {
      const int idx = threadIdx.x + 256 * e;
      int r, kk;
      if (!CONJ_A) { r = idx % BM; kk = idx / BM; }
      else { kk = idx % BK; r = idx / BK; }
      const int gr = m0 + r, gk = kk0 + kk;
      T2 v = V2<T>::make(0, 0);
      if (gr < m && gk < k) {
        if (!CONJ_A) v = A2[gr + lda * (int64_t)gk];
        else { v = A2[gk + lda * (int64_t)gr]; v.y = -v.y; }
      }
      As[kk][r] = v;
    }
#pragma unroll
    for (int e = 0; e < (BN * BK) / 256; e++) {
      const int idx = threadIdx.x + 256 * e;
      const int kk = idx % BK, c = idx / BK;
      const int gk = kk0 + kk, gc = n0 + c;
      T2 v = V2<T>::make(0, 0);
      if (gk < k && gc < n) v = B2[gk + ldb * (int64_t)gc];
      Bs[kk][c] = v;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; kk++) {
      T2 a[TM], b[TN];
#pragma unroll
      for (int q = 0; q < TM; q++) a[q] = As[kk][ty + TY * q];
#pragma unroll
      for (int q = 0; q < TN; q++) b[q] = Bs[kk][tx + TX * q];
#pragma unroll
      for (int p = 0; p < TM; p++)
#pragma unroll
        for (int q = 0; q < TN; q++) {
          cx<T> &d = COMP ? part[COMP ? p : 0][COMP ? q : 0] : acc[p][q];
          d.r = fma(a[p].x, b[q].x, d.r);
          d.r = fma(-a[p].y, b[q].y, d.r);
          d.i = fma(a[p].x, b[q].y, d.i);
          d.i = fma(a[p].y, b[q].x, d.i);
        }
    }
    if (COMP) {
#pragma unroll
      for (int p = 0; p < TM; p++)
#pragma unroll
        for (int q = 0; q < TN; q++) {
          cx<T> &h = acc[p][q];
          cx<T> &l = lo[COMP ? p : 0][COMP ? q : 0];
          cx<T> &x = part[COMP ? p : 0][COMP ? q : 0];
          // TwoSum (Knuth): h + x = s + e exactly
          T s_ = h.r + x.r, bp = s_ - h.r;
          l.r += (h.r - (s_ - bp)) + (x.r - bp);
          h.r = s_;
          s_ = h.i + x.i; bp = s_ - h.i;
          l.i += (h.i - (s_ - bp)) + (x.i - bp);
          h.i = s_;
          x = {0, 0};
        }
    }
    __syncthreads();
  }
  typedef typename V2<TC>::type C2t;
  C2t *C2 = reinterpret_cast<C2t *>(C);
  const bool beta0 = (beta.r == TC(0) && beta.i == TC(0));
#pragma unroll
  for (int p = 0; p < TM; p++)
#pragma unroll
    for (int q = 0; q < TN; q++) {
      const int r = m0 + ty + TY * p, c = n0 + tx + TX * q;
      if (r < m && c < n) {
        cx<TC> av = {(TC)acc[p][q].r, (TC)acc[p][q].i};
        if (COMP) {
          av.r += (TC)lo[COMP ? p : 0][COMP ? q : 0].r;
          av.i += (TC)lo[COMP ? p : 0][COMP ? q : 0].i;
        }
        cx<TC> v = cmul(cx<TC>{(TC)alpha.r, (TC)alpha.i}, av);
        if (!beta0) {
          const C2t o = C2[r + ldc * (int64_t)c];
          const cx<TC> ob = cmul(beta, cx<TC>{o.x, o.y});
          v.r += ob.r;
          v.i += ob.i;
        }
        C2[r + ldc * (int64_t)c] = V2<TC>::make(v.r, v.i);
      }
    }
}

template <typename T>
struct GemmCfg;
template <>
struct GemmCfg<double> {
  static constexpr int BM = 64, BN = 64, TM = 4, TN = 4, BK = 8;
};
template <>
struct GemmCfg<float> {
  static constexpr int BM = 128, BN = 64, TM = 8, TN = 4, BK = 8;
};

template <typename T, int R = NB / 32>
constexpr int trsm_smem_bytes() { return 32 * R * 32 * R * (int)sizeof(typename V2<T>::type); }

template <typename T>
int set_trsm_attrs(bemgpu_ctx_s *ctx) {
  static bool done[64] = {false};
  if (done[ctx->device]) return BEMGPU_OK;
  constexpr int RL = LuCfg<T>::NBL / 32;
  BEM_CUDA_TRY(ctx, cudaFuncSetAttribute(trsm_block_kernel<T, false, NB / 32>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, trsm_smem_bytes<T>()));
  BEM_CUDA_TRY(ctx, cudaFuncSetAttribute(trsm_block_kernel<T, true, NB / 32>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, trsm_smem_bytes<T>()));
  BEM_CUDA_TRY(ctx, cudaFuncSetAttribute(trsm_block_kernel<T, false, RL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         trsm_smem_bytes<T, RL>()));
  done[ctx->device] = true;
  return BEMGPU_OK;
}

template <typename T>
int gemm_fma(bemgpu_ctx_s *ctx, int kind, char opA, int m, int n, int k, const T alpha[2], const T *A, int64_t lda,
             const T *B, int64_t ldb, const T beta[2], T *C, int64_t ldc, cudaStream_t stream) {
  if (m <= 0 || n <= 0) return BEMGPU_OK;
  typedef GemmCfg<T> G;
  dim3 grd((m + G::BM - 1) / G::BM, (n + G::BN - 1) / G::BN);
  cx<T> al = {alpha[0], alpha[1]}, be = {beta[0], beta[1]};
  ProfScope ps(ctx, kind, stream, 8.0 * m * n * k,
               2.0 * sizeof(T) * ((double)m * k + (double)k * n + 2.0 * m * n));
  if (opA == 'C') {
    cgemm_fma_kernel<T, G::BM, G::BN, G::TM, G::TN, G::BK, true>
        <<<grd, 256, 0, stream>>>(m, n, k, al, A, lda, B, ldb, be, C, ldc, 0, 0, 0);
  } else {
    cgemm_fma_kernel<T, G::BM, G::BN, G::TM, G::TN, G::BK, false>
        <<<grd, 256, 0, stream>>>(m, n, k, al, A, lda, B, ldb, be, C, ldc, 0, 0, 0);
  }
  ctx->launches++;
  BEM_CUDA_TRY(ctx, cudaGetLastError());
  return BEMGPU_OK;
}

}  // namespace

// Trailing / off-diagonal updates of the complex64 path go through bem_cgemm,
// which uses the tensor-core kernel where one is available (gemm_tc.cu).
int bem_zgemm(bemgpu_ctx_s *ctx, int kind, char opA, int m, int n, int k, const double alpha[2], const double *A,
              int64_t lda, const double *B, int64_t ldb, const double beta[2], double *C, int64_t ldc,
              cudaStream_t stream) {
  return gemm_fma<double>(ctx, kind, opA, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, stream);
}

// C (complex128) = alpha A B + beta C with complex64 A, B: FP32 products,
// compensated accumulation (per 8-deep K tile in FP32, across tiles as a
// two-float sum), FP64 output.
int bem_cgemm_comp64_fma(bemgpu_ctx_s *ctx, int kind, int m, int n, int k, const float alpha[2], const float *A,
                         int64_t lda, const float *B, int64_t ldb, const double beta[2], double *C, int64_t ldc,
                         cudaStream_t stream) {
  if (m <= 0 || n <= 0) return BEMGPU_OK;
  dim3 grd((m + 63) / 64, (n + 63) / 64);
  cx<float> al = {alpha[0], alpha[1]};
  cx<double> be = {beta[0], beta[1]};
  ProfScope ps(ctx, kind, stream, 8.0 * m * n * k, 8.0 * ((double)m * k + (double)k * n) + 32.0 * m * n);
  cgemm_fma_kernel<float, 64, 64, 4, 4, 8, false, double, true>
      <<<grd, 256, 0, stream>>>(m, n, k, al, A, lda, B, ldb, be, C, ldc, 0, 0, 0);
  ctx->launches++;
  BEM_CUDA_TRY(ctx, cudaGetLastError());
  return BEMGPU_OK;
}

int bem_cgemm_fma(bemgpu_ctx_s *ctx, int kind, char opA, int m, int n, int k, const float alpha[2], const float *A,
                  int64_t lda, const float *B, int64_t ldb, const float beta[2], float *C, int64_t ldc,
                  cudaStream_t stream) {
  return gemm_fma<float>(ctx, kind, opA, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, stream);
}

namespace {

template <typename T>
int gemm_any(bemgpu_ctx_s *ctx, int kind, char opA, int m, int n, int k, const T alpha[2], const T *A, int64_t lda,
             const T *B, int64_t ldb, const T beta[2], T *C, int64_t ldc, cudaStream_t stream);
template <>
int gemm_any<double>(bemgpu_ctx_s *ctx, int kind, char opA, int m, int n, int k, const double alpha[2],
                     const double *A, int64_t lda, const double *B, int64_t ldb, const double beta[2], double *C,
                     int64_t ldc, cudaStream_t stream) {
  return bem_zgemm(ctx, kind, opA, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, stream);
}
template <>
int gemm_any<float>(bemgpu_ctx_s *ctx, int kind, char opA, int m, int n, int k, const float alpha[2],
                    const float *A, int64_t lda, const float *B, int64_t ldb, const float beta[2], float *C,
                    int64_t ldc, cudaStream_t stream) {
  return bem_cgemm(ctx, kind, opA, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, stream);
}

constexpr int COOP_MAX_SMEM = 226 * 1024;  // below the 227 KB per-CTA limit, with room for the static part

// Factors the panel [k0, k0 + w) with one cooperative launch; returns false
// (nothing launched) when the panel does not fit the cooperative kernel.
template <typename T>
bool panel_coop(bemgpu_ctx_s *ctx, T *A, int64_t lda, int n, int k0, int w, int *d_ipiv, int *d_info,
                cudaStream_t stream, int &rc, int nb = 1, int64_t strideA = 0) {
  typedef typename V2<T>::type T2;
  rc = BEMGPU_OK;
  const int rows = n - k0;
  int G = std::max(1, std::min(ctx->num_sms, (rows + 15) / 16));
  {
    // fewer, fuller CTAs leave SMs to the other lanes' products while this
    // latency-bound panel runs (BEMGPU_TUNE_PANEL_CTAS), as far as shared
    // memory holds their rows
    const int cap = ctx->tune.panel_ctas;
    const int max_chunk = (int)(COOP_MAX_SMEM / (sizeof(T2) * (size_t)w)) - 1;
    if (cap > 0) G = std::max(std::min(G, cap), (rows + max_chunk - 1) / max_chunk);
  }
  if (nb > 1) {
    // a batch shares about the CTAs one panel would take (more rows per CTA,
    // up to what shared memory holds), so that its cooperative launch does
    // not need more of the GPU than a single panel's
    const int max_chunk = (int)(COOP_MAX_SMEM / (sizeof(T2) * (size_t)w)) - 1;
    G = std::max((rows + max_chunk - 1) / max_chunk, (G + nb - 1) / nb);
  }
  const int chunk = (rows + G - 1) / G;
  const size_t smem = sizeof(T2) * (size_t)(chunk + 1) * w;
  if (smem > (size_t)COOP_MAX_SMEM) return false;
  static bool attr[64][2] = {};
  const int ti = sizeof(T) == 8 ? 1 : 0;
  if (!attr[ctx->device][ti]) {
    if (cudaFuncSetAttribute(panel_coop_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, COOP_MAX_SMEM) !=
        cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    attr[ctx->device][ti] = true;
  }
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, panel_coop_kernel<T>, COOP_THREADS, smem) !=
          cudaSuccess ||
      per_sm * ctx->num_sms < G * nb) {
    cudaGetLastError();
    return false;
  }
  // candidate slots and barriers per matrix of the batch (the kernel offsets
  // them by blockIdx.y: 2 G values, rows and rows of w entries, 2 w for the
  // diagonal row, one counter, four pivot keys)
  T *cval = (T *)bem_workspace(ctx, "coop_cval", sizeof(T) * 2 * (size_t)G * nb);
  int *crow = (int *)bem_workspace(ctx, "coop_crow", sizeof(int) * 2 * (size_t)G * nb);
  T *cdata = (T *)bem_workspace(ctx, "coop_cdata", sizeof(T2) * 2 * (size_t)G * w * nb);
  T *drow = (T *)bem_workspace(ctx, "coop_drow", sizeof(T2) * 2 * (size_t)w * nb);
  unsigned *counter = (unsigned *)bem_workspace(ctx, "coop_counter", sizeof(unsigned) * (size_t)nb);
  unsigned long long *best =
      (unsigned long long *)bem_workspace(ctx, "coop_best", 4 * sizeof(unsigned long long) * (size_t)nb);
  int *err = (int *)bem_workspace(ctx, "tc_err", sizeof(int));
  if (!cval || !crow || !cdata || !drow || !counter || !best || !err || G > 1024 || w > NB_MAX) {
    rc = bem_fail(ctx, BEMGPU_ERR_OOM, "getrf: panel workspace");
    return true;
  }
  if (!ctx->tc_err_ready) {
    cudaMemsetAsync(err, 0, sizeof(int), stream);
    ctx->tc_err_ready = true;
  }
  cudaMemsetAsync(counter, 0, sizeof(unsigned) * (size_t)nb, stream);
  cudaMemsetAsync(best, 0, 4 * sizeof(unsigned long long) * (size_t)nb, stream);
  int n_ = n, k0_ = k0, w_ = w, chunk_ = chunk;
  void *args[] = {&A,    &lda,  &n_,    &k0_,  &w_,      &chunk_, &d_ipiv, &d_info,
                  &cval, &crow, &cdata, &drow, &counter, &err,    &best,   &strideA};
  const double cb = 2.0 * sizeof(T);
  ProfScope ps(ctx, BEMGPU_K_LU_PANEL, stream, 4.0 * (double)rows * w * w * nb, cb * 2.0 * rows * w * nb);
  const cudaError_t e = cudaLaunchCooperativeKernel((const void *)panel_coop_kernel<T>, dim3(G, nb),
                                                    dim3(COOP_THREADS), args, smem, stream);
  ctx->launches++;
  if (e != cudaSuccess) {
    cudaGetLastError();
    rc = bem_fail(ctx, BEMGPU_ERR_CUDA, "getrf: cooperative panel launch: %s", cudaGetErrorString(e));
  }
  return true;
}

// LU with partial pivoting of nb equal-size matrices A + i strideA (pivots
// d_ipiv + i n, info d_info + i): every panel of the batch in one cooperative
// launch (each matrix with its own CTAs and barrier), the interchanges,
// triangular blocks and trailing updates per matrix.  Each matrix gets the
// arithmetic of a batch of one.
template <typename T>
int getrf_impl(bemgpu_ctx_s *ctx, T *A0, int64_t lda, int n, int *d_ipiv0, int *d_info0, cudaStream_t stream,
               int nb = 1, int64_t strideA = 0) {
  if (int rc0 = set_trsm_attrs<T>(ctx)) return rc0;
  PivCand *cand = (PivCand *)bem_workspace(ctx, "lu_cand", sizeof(PivCand) * 1024);
  unsigned int *counter = (unsigned int *)bem_workspace(ctx, "lu_counter", sizeof(unsigned int));
  if (!cand || !counter) return bem_fail(ctx, BEMGPU_ERR_OOM, "getrf: workspace");
  BEM_CUDA_TRY(ctx, cudaMemsetAsync(counter, 0, sizeof(unsigned int), stream));
  BEM_CUDA_TRY(ctx, cudaMemsetAsync(d_info0, 0, sizeof(int) * (size_t)nb, stream));
  const T mone[2] = {T(-1), T(0)}, one[2] = {T(1), T(0)};
  const double cb = 2.0 * sizeof(T);  // bytes per complex element
  constexpr int NBL = LuCfg<T>::NBL;
  // complex64 super-blocks (BEMGPU_TUNE_LU_SUPER): panels in pairs A, B.
  // After A only B's columns take A's update; after B the rows of B and then
  // the trailing matrix beyond the pair take both at once, the latter as one
  // K = 2 NBL product (half the passes over the trailing matrix).  The same
  // updates as one panel at a time, associated differently.
  const bool super = sizeof(T) == 4 && ctx->tune.lu_super != 0;
  for (int k0 = 0; k0 < n; k0 += NBL) {
    const int w = std::min(NBL, n - k0);
    const int rows = n - k0;
    const bool first_half = super && (k0 / NBL) % 2 == 0;   // panel A (its B follows when k0 + w < n)
    const bool second_half = super && (k0 / NBL) % 2 == 1;  // panel B
    const int K0 = second_half ? k0 - NBL : k0;              // the pair's first column
    const int blocks = std::max(1, std::min(ctx->num_sms * 2, (rows + PANEL_THREADS - 1) / PANEL_THREADS));
    int prc = BEMGPU_OK;
    bool coop = ctx->coop_panel && panel_coop<T>(ctx, A0, lda, n, k0, w, d_ipiv0, d_info0, stream, prc, nb, strideA);
    if (prc) return prc;
    if (!coop && nb > 1 && ctx->coop_panel) {
      // the batch's panels do not fit at once: one cooperative panel per matrix
      coop = true;
      for (int i = 0; i < nb && coop; i++) {
        coop = panel_coop<T>(ctx, A0 + i * strideA, lda, n, k0, w, d_ipiv0 + (int64_t)i * n, d_info0 + i, stream,
                             prc);
        if (prc) return prc;
      }
      if (!coop && nb > 1) return bem_fail(ctx, BEMGPU_ERR_ARG, "getrf: batched panel does not fit");
    }
    for (int i = 0; i < nb; i++) {
      T *A = A0 + i * strideA;
      int *d_ipiv = d_ipiv0 + (int64_t)i * n;
      int *d_info = d_info0 + i;
      for (int jj = 0; !coop && jj <= w; jj++) {
        ProfScope ps(ctx, BEMGPU_K_LU_PANEL, stream, 8.0 * (rows - jj) * (w - jj), cb * 2 * (rows - jj) * (w - jj));
        panel_step_kernel<T><<<blocks, PANEL_THREADS, 0, stream>>>(A, lda, n, k0, w, jj, d_ipiv, d_info, cand,
                                                                   counter);
        ctx->launches++;
      }
      BEM_CUDA_TRY(ctx, cudaGetLastError());
      // interchanges to the left and right of the panel
      static_assert(NBL <= LASWP_MAXW, "panel wider than the interchange kernel's permutation");
      if (k0 > 0) {
        ProfScope ps(ctx, BEMGPU_K_LU_PANEL, stream, 0.0, 4.0 * cb * w * k0);
        const int g = std::min((k0 + LASWP_WARPS - 1) / LASWP_WARPS, 2 * ctx->num_sms);
        laswp_perm_kernel<T><<<g, 32 * LASWP_WARPS, 0, stream>>>(A, lda, 0, k0, k0, k0 + w, d_ipiv);
        ctx->launches++;
      }
      if (k0 + w < n) {
        const int nr = n - k0 - w;
        T *A11 = A + 2 * (k0 + lda * (int64_t)k0);
        T *A12 = A + 2 * (k0 + lda * (int64_t)(k0 + w));
        // one CTA per SM at most: each CTA stages the w x w diagonal block in
        // shared memory once and walks its share of the columns
        const int tb = std::min((nr + 7) / 8, NBL > 64 ? ctx->num_sms : ctx->num_sms * 4);
        {
          ProfScope ps(ctx, BEMGPU_K_LU_PANEL, stream, 0.0, 4.0 * cb * w * nr);
          const int g = std::min((nr + LASWP_WARPS - 1) / LASWP_WARPS, 2 * ctx->num_sms);
          laswp_perm_kernel<T><<<g, 32 * LASWP_WARPS, 0, stream>>>(A, lda, k0 + w, n, k0, k0 + w, d_ipiv);
          ctx->launches++;
        }
        if (second_half) {
          // panel A's update of B's rows beyond the pair:
          // A[k0:k0+w, k0+w:n] -= L[k0:k0+w, K0:k0] U[K0:k0, k0+w:n]
          int rc = gemm_any<T>(ctx, BEMGPU_K_LU_GEMM, 'N', w, nr, k0 - K0, mone, A + 2 * (k0 + lda * (int64_t)K0),
                               lda, A + 2 * (K0 + lda * (int64_t)(k0 + w)), lda, one, A12, lda, stream);
          if (rc) return rc;
        }
        {
          ProfScope ps(ctx, BEMGPU_K_TRSM, stream, 4.0 * w * w * nr, 2.0 * cb * w * nr);
          trsm_block_kernel<T, false, NBL / 32>
              <<<tb, 256, trsm_smem_bytes<T, NBL / 32>(), stream>>>(A11, lda, w, A12, lda, nr);
          ctx->launches++;
        }
        T *A22 = A + 2 * (k0 + w + lda * (int64_t)(k0 + w));
        int rc;
        if (first_half) {
          // panel B's columns only; the rest waits for B
          T *A21 = A + 2 * (k0 + w + lda * (int64_t)k0);
          rc = gemm_any<T>(ctx, BEMGPU_K_LU_GEMM, 'N', nr, std::min(NBL, nr), w, mone, A21, lda, A12, lda, one, A22,
                           lda, stream);
        } else {
          // the trailing matrix from the pair's panels at once (K = k0 + w - K0)
          T *L21 = A + 2 * (k0 + w + lda * (int64_t)K0);
          T *U12 = A + 2 * (K0 + lda * (int64_t)(k0 + w));
          rc = gemm_any<T>(ctx, BEMGPU_K_LU_GEMM, 'N', nr, nr, k0 + w - K0, mone, L21, lda, U12, lda, one, A22, lda,
                           stream);
        }
        if (rc) return rc;
      }
      BEM_CUDA_TRY(ctx, cudaGetLastError());
    }
  }
  return BEMGPU_OK;
}

template <typename T>
int getrs_impl(bemgpu_ctx_s *ctx, const T *A, int64_t lda, int n, const int *d_ipiv, T *B, int64_t ldb, int nrhs,
               cudaStream_t stream) {
  if (int rc0 = set_trsm_attrs<T>(ctx)) return rc0;
  const T mone[2] = {T(-1), T(0)}, one[2] = {T(1), T(0)};
  const double cb = 2.0 * sizeof(T);
  {
    ProfScope ps(ctx, BEMGPU_K_LU_PANEL, stream, 0.0, 4.0 * cb * n * nrhs);
    laswp_kernel<T><<<(nrhs + 127) / 128, 128, 0, stream>>>(B, ldb, 0, nrhs, 0, n, d_ipiv);
    ctx->launches++;
  }
  const int tb = std::min((nrhs + 7) / 8, ctx->num_sms * 4);
  // forward: L Y = P B
  for (int k0 = 0; k0 < n; k0 += NB) {
    const int w = std::min(NB, n - k0);
    const T *L11 = A + 2 * (k0 + lda * (int64_t)k0);
    T *Bk = B + 2 * (int64_t)k0;
    {
      ProfScope ps(ctx, BEMGPU_K_TRSM, stream, 4.0 * w * w * nrhs, 2.0 * cb * w * nrhs);
      trsm_block_kernel<T, false, NB / 32><<<tb, 256, trsm_smem_bytes<T>(), stream>>>(L11, lda, w, Bk, ldb, nrhs);
      ctx->launches++;
    }
    if (k0 + w < n) {
      const T *L21 = A + 2 * (k0 + w + lda * (int64_t)k0);
      int rc = gemm_any<T>(ctx, BEMGPU_K_SOLVE_GEMM, 'N', n - k0 - w, nrhs, w, mone, L21, lda, Bk, ldb, one,
                           B + 2 * (int64_t)(k0 + w), ldb, stream);
      if (rc) return rc;
    }
  }
  // backward: U X = Y
  const int nblk = (n + NB - 1) / NB;
  for (int bi = nblk - 1; bi >= 0; bi--) {
    const int k0 = bi * NB;
    const int w = std::min(NB, n - k0);
    const T *U11 = A + 2 * (k0 + lda * (int64_t)k0);
    T *Bk = B + 2 * (int64_t)k0;
    {
      ProfScope ps(ctx, BEMGPU_K_TRSM, stream, 4.0 * w * w * nrhs, 2.0 * cb * w * nrhs);
      trsm_block_kernel<T, true, NB / 32><<<tb, 256, trsm_smem_bytes<T>(), stream>>>(U11, lda, w, Bk, ldb, nrhs);
      ctx->launches++;
    }
    if (k0 > 0) {
      const T *U01 = A + 2 * (lda * (int64_t)k0);
      int rc = gemm_any<T>(ctx, BEMGPU_K_SOLVE_GEMM, 'N', k0, nrhs, w, mone, U01, lda, Bk, ldb, one, B, ldb, stream);
      if (rc) return rc;
    }
  }
  BEM_CUDA_TRY(ctx, cudaGetLastError());
  return BEMGPU_OK;
}

}  // namespace

int bem_zgetrf(bemgpu_ctx_s *ctx, double *A, int64_t lda, int n, int *d_ipiv, int *d_info, cudaStream_t stream) {
  return getrf_impl<double>(ctx, A, lda, n, d_ipiv, d_info, stream);
}
int bem_zgetrs(bemgpu_ctx_s *ctx, const double *A, int64_t lda, int n, const int *d_ipiv, double *B, int64_t ldb,
               int nrhs, cudaStream_t stream) {
  return getrs_impl<double>(ctx, A, lda, n, d_ipiv, B, ldb, nrhs, stream);
}
namespace {

constexpr int NBO = 512;  // super-block of the FP64-class LU and solve

__global__ void identity_block_kernel(double *X, int64_t ld, int w) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  const int c = blockIdx.y;
  if (r >= w) return;
  reinterpret_cast<double2 *>(X)[r + ld * (int64_t)c] = make_double2(r == c ? 1.0 : 0.0, 0.0);
}

// X (w x ncols, ld ldx) <- T^{-1} X for the w x w triangle T at (A, lda):
// unit lower (UPPER false) or upper; 64-row diagonal blocks in FP64
// (trsm_block_kernel), off-diagonal updates as 5-slice exact products.
int tri_solve_exact(bemgpu_ctx_s *ctx, const double *A, int64_t lda, int w, bool upper, double *X, int64_t ldx,
                    int ncols, cudaStream_t st) {
  const int tb = std::min((ncols + 7) / 8, ctx->num_sms * 4);
  const int nblk = (w + NB - 1) / NB;
  int rc = BEMGPU_OK;
  for (int q = 0; q < nblk && !rc; q++) {
    const int bi = upper ? nblk - 1 - q : q;
    const int j0 = bi * NB, jw = std::min(NB, w - j0);
    double *Xj = X + 2 * (int64_t)j0;
    {
      ProfScope ps(ctx, BEMGPU_K_TRSM, st, 4.0 * jw * jw * ncols, 32.0 * jw * ncols);
      if (upper)
        trsm_block_kernel<double, true, NB / 32><<<tb, 256, trsm_smem_bytes<double>(), st>>>(
            A + 2 * (j0 + lda * (int64_t)j0), lda, jw, Xj, ldx, ncols);
      else
        trsm_block_kernel<double, false, NB / 32><<<tb, 256, trsm_smem_bytes<double>(), st>>>(
            A + 2 * (j0 + lda * (int64_t)j0), lda, jw, Xj, ldx, ncols);
      ctx->launches++;
    }
    const int m = upper ? j0 : w - j0 - jw;  // rows still to update
    if (m > 0) {
      ExactOperand oa, ob;
      const double *Ablk = upper ? A + 2 * (lda * (int64_t)j0) : A + 2 * (j0 + jw + lda * (int64_t)j0);
      rc = bem_exact_prep(ctx, "ts_A", true, Ablk, lda, m, jw, -1.0, 5, oa, st);
      if (!rc) rc = bem_exact_prep(ctx, "ts_B", false, Xj, ldx, ncols, jw, 1.0, 5, ob, st);
      if (!rc) rc = bem_exact_gemm(ctx, BEMGPU_K_TRSM, oa, ob, upper ? X : Xj + 2 * (int64_t)jw, ldx, 1, st);
    }
  }
  return rc;
}

// Dst (m x ncols) (+)= sign * Ablk (m x k) * Bblk (k x ncols) as a 5-slice exact
// product; Bblk may be Dst itself when accumulate is 0 (it is sliced first).
int exact_mul(bemgpu_ctx_s *ctx, int kind, const double *Ablk, int64_t lda, int m, int k, double sign,
              const double *Bblk, int64_t ldb, int ncols, double *Dst, int64_t ldd, int accumulate, cudaStream_t st) {
  ExactOperand oa, ob;
  int rc = bem_exact_prep(ctx, "xm_A", true, Ablk, lda, m, k, sign, 5, oa, st);
  if (!rc) rc = bem_exact_prep(ctx, "xm_B", false, Bblk, ldb, ncols, k, 1.0, 5, ob, st);
  if (!rc) rc = bem_exact_gemm(ctx, kind, oa, ob, Dst, ldd, accumulate, st);
  return rc;
}

}  // namespace

// FP64-class LU on the tensor cores, blocked twice: 512-column super-panels
// are factored by 64-column cooperative panels whose updates stay inside the
// super-panel; then the super-panel's pivots are applied to the other
// columns, U12 = L11^{-1} A12 with the inverse of the 512 x 512 unit-lower
// diagonal block, and A22 -= A21 U12 as one K = 512 exact product.  The
// inverses of the diagonal super-blocks (L and U) are kept for
// bem_zgetrs_exact ("lu_Lb", "lu_Ub": n x 512, block K at rows [K0, K0+512)).
int bem_zgetrf_exact(bemgpu_ctx_s *ctx, double *A, int64_t lda, int n, int *d_ipiv, int *d_info, cudaStream_t stream) {
  if (int rc0 = set_trsm_attrs<double>(ctx)) return rc0;
  double *Lb = (double *)bem_workspace(ctx, "lu_Lb", 16 * (size_t)n * NBO);
  double *Ub = (double *)bem_workspace(ctx, "lu_Ub", 16 * (size_t)n * NBO);
  if (!Lb || !Ub) return bem_fail(ctx, BEMGPU_ERR_OOM, "getrf_exact: workspace");
  BEM_CUDA_TRY(ctx, cudaMemsetAsync(d_info, 0, sizeof(int), stream));
  const double cb = 16.0;
  int rc = BEMGPU_OK;
  for (int K0 = 0; K0 < n && !rc; K0 += NBO) {
    const int WO = std::min(NBO, n - K0);
    for (int k0 = K0; k0 < K0 + WO && !rc; k0 += NB) {
      const int w = std::min(NB, K0 + WO - k0);
      int prc = BEMGPU_OK;
      const bool coop = ctx->coop_panel && panel_coop<double>(ctx, A, lda, n, k0, w, d_ipiv, d_info, stream, prc);
      if (prc) return prc;
      if (!coop) {  // one launch per column when the panel does not fit the cooperative kernel
        PivCand *cand = (PivCand *)bem_workspace(ctx, "lu_cand", sizeof(PivCand) * 1024);
        unsigned int *counter = (unsigned int *)bem_workspace(ctx, "lu_counter", sizeof(unsigned int));
        if (!cand || !counter) return bem_fail(ctx, BEMGPU_ERR_OOM, "getrf_exact: workspace");
        BEM_CUDA_TRY(ctx, cudaMemsetAsync(counter, 0, sizeof(unsigned int), stream));
        const int rows = n - k0;
        const int blocks = std::max(1, std::min(ctx->num_sms * 2, (rows + PANEL_THREADS - 1) / PANEL_THREADS));
        for (int jj = 0; jj <= w; jj++) {
          ProfScope ps(ctx, BEMGPU_K_LU_PANEL, stream, 8.0 * (rows - jj) * (w - jj), 32.0 * (rows - jj) * (w - jj));
          panel_step_kernel<double><<<blocks, PANEL_THREADS, 0, stream>>>(A, lda, n, k0, w, jj, d_ipiv, d_info, cand,
                                                                           counter);
          ctx->launches++;
        }
      }
      {
        ProfScope ps(ctx, BEMGPU_K_LU_PANEL, stream, 0.0, 4.0 * cb * w * WO);
        if (k0 > K0) {
          laswp_kernel<double><<<(k0 - K0 + 127) / 128, 128, 0, stream>>>(A, lda, K0, k0, k0, k0 + w, d_ipiv);
          ctx->launches++;
        }
        if (k0 + w < K0 + WO) {
          laswp_kernel<double><<<(K0 + WO - k0 - w + 127) / 128, 128, 0, stream>>>(A, lda, k0 + w, K0 + WO, k0, k0 + w,
                                                                                 d_ipiv);
          ctx->launches++;
        }
      }
      const int nc = K0 + WO - k0 - w;  // super-panel columns right of this panel
      if (nc > 0) {
        const int tb = std::min((nc + 7) / 8, ctx->num_sms * 4);
        {
          ProfScope ps(ctx, BEMGPU_K_TRSM, stream, 4.0 * w * w * nc, 2.0 * cb * w * nc);
          trsm_block_kernel<double, false, NB / 32><<<tb, 256, trsm_smem_bytes<double>(), stream>>>(
              A + 2 * (k0 + lda * (int64_t)k0), lda, w, A + 2 * (k0 + lda * (int64_t)(k0 + w)), lda, nc);
          ctx->launches++;
        }
        if (k0 + w < n)
          rc = exact_mul(ctx, BEMGPU_K_LU_GEMM, A + 2 * (k0 + w + lda * (int64_t)k0), lda, n - k0 - w, w, -1.0,
                         A + 2 * (k0 + lda * (int64_t)(k0 + w)), lda, nc, A + 2 * (k0 + w + lda * (int64_t)(k0 + w)),
                         lda, 1, stream);
      }
    }
    if (rc) break;
    {
      ProfScope ps(ctx, BEMGPU_K_LU_PANEL, stream, 0.0, 4.0 * cb * WO * (n - WO));
      if (K0 > 0) {
        laswp_kernel<double><<<(K0 + 127) / 128, 128, 0, stream>>>(A, lda, 0, K0, K0, K0 + WO, d_ipiv);
        ctx->launches++;
      }
      if (K0 + WO < n) {
        laswp_kernel<double><<<(n - K0 - WO + 127) / 128, 128, 0, stream>>>(A, lda, K0 + WO, n, K0, K0 + WO, d_ipiv);
        ctx->launches++;
      }
    }
    // inverses of the diagonal super-block's triangles
    const double *AKK = A + 2 * (K0 + lda * (int64_t)K0);
    double *LbK = Lb + 2 * (int64_t)K0, *UbK = Ub + 2 * (int64_t)K0;
    identity_block_kernel<<<dim3((WO + 255) / 256, WO), 256, 0, stream>>>(LbK, n, WO);
    identity_block_kernel<<<dim3((WO + 255) / 256, WO), 256, 0, stream>>>(UbK, n, WO);
    ctx->launches += 2;
    rc = tri_solve_exact(ctx, AKK, lda, WO, false, LbK, n, WO, stream);
    if (!rc) rc = tri_solve_exact(ctx, AKK, lda, WO, true, UbK, n, WO, stream);
    if (rc || K0 + WO >= n) continue;
    const int nr = n - K0 - WO;
    double *A12 = A + 2 * (K0 + lda * (int64_t)(K0 + WO));
    rc = exact_mul(ctx, BEMGPU_K_TRSM, LbK, n, WO, WO, 1.0, A12, lda, nr, A12, lda, 0, stream);
    if (!rc)
      rc = exact_mul(ctx, BEMGPU_K_LU_GEMM, A + 2 * (K0 + WO + lda * (int64_t)K0), lda, nr, WO, -1.0, A12, lda, nr,
                     A + 2 * (K0 + WO + lda * (int64_t)(K0 + WO)), lda, 1, stream);
  }
  if (!rc) BEM_CUDA_TRY(ctx, cudaGetLastError());
  return rc;
}

// B <- A^{-1} B with the factors and diagonal-block inverses of
// bem_zgetrf_exact: row interchanges, then per 512-row super-block one exact
// product with the block's inverse and one K = 512 exact update of the rest.
int bem_zgetrs_exact(bemgpu_ctx_s *ctx, const double *A, int64_t lda, int n, const int *d_ipiv, double *B, int64_t ldb,
                     int nrhs, cudaStream_t stream) {
  const double *Lb = (const double *)bem_workspace(ctx, "lu_Lb", 16 * (size_t)n * NBO);
  const double *Ub = (const double *)bem_workspace(ctx, "lu_Ub", 16 * (size_t)n * NBO);
  if (!Lb || !Ub) return bem_fail(ctx, BEMGPU_ERR_OOM, "getrs_exact: workspace");
  {
    ProfScope ps(ctx, BEMGPU_K_LU_PANEL, stream, 0.0, 64.0 * n * (double)nrhs);
    laswp_kernel<double><<<(nrhs + 127) / 128, 128, 0, stream>>>(B, ldb, 0, nrhs, 0, n, d_ipiv);
    ctx->launches++;
  }
  int rc = BEMGPU_OK;
  for (int K0 = 0; K0 < n && !rc; K0 += NBO) {  // forward: L Y = P B
    const int WO = std::min(NBO, n - K0);
    double *BK = B + 2 * (int64_t)K0;
    rc = exact_mul(ctx, BEMGPU_K_SOLVE_GEMM, Lb + 2 * (int64_t)K0, n, WO, WO, 1.0, BK, ldb, nrhs, BK, ldb, 0, stream);
    if (!rc && K0 + WO < n)
      rc = exact_mul(ctx, BEMGPU_K_SOLVE_GEMM, A + 2 * (K0 + WO + lda * (int64_t)K0), lda, n - K0 - WO, WO, -1.0, BK,
                     ldb, nrhs, B + 2 * (int64_t)(K0 + WO), ldb, 1, stream);
  }
  const int nblk = (n + NBO - 1) / NBO;
  for (int bi = nblk - 1; bi >= 0 && !rc; bi--) {  // backward: U X = Y
    const int K0 = bi * NBO, WO = std::min(NBO, n - K0);
    double *BK = B + 2 * (int64_t)K0;
    rc = exact_mul(ctx, BEMGPU_K_SOLVE_GEMM, Ub + 2 * (int64_t)K0, n, WO, WO, 1.0, BK, ldb, nrhs, BK, ldb, 0, stream);
    if (!rc && K0 > 0)
      rc = exact_mul(ctx, BEMGPU_K_SOLVE_GEMM, A + 2 * (lda * (int64_t)K0), lda, K0, WO, -1.0, BK, ldb, nrhs, B, ldb, 1,
                     stream);
  }
  if (!rc) BEM_CUDA_TRY(ctx, cudaGetLastError());
  return rc;
}

int bem_cgetrf_batch(bemgpu_ctx_s *ctx, float *A, int64_t strideA, int nb, int64_t lda, int n, int *d_ipiv,
                     int *d_info, cudaStream_t stream) {
  if (nb < 1) return BEMGPU_OK;
  return getrf_impl<float>(ctx, A, lda, n, d_ipiv, d_info, stream, nb, strideA);
}

int bem_cgetrf(bemgpu_ctx_s *ctx, float *A, int64_t lda, int n, int *d_ipiv, int *d_info, cudaStream_t stream) {
  return getrf_impl<float>(ctx, A, lda, n, d_ipiv, d_info, stream);
}
int bem_cgetrs(bemgpu_ctx_s *ctx, const float *A, int64_t lda, int n, const int *d_ipiv, float *B, int64_t ldb,
               int nrhs, cudaStream_t stream) {
  return getrs_impl<float>(ctx, A, lda, n, d_ipiv, B, ldb, nrhs, stream);
}

// ---------------- explicit triangular inverses (complex64 mixed path) ----------------
// The correction solves of the refinement apply W32^{-1} = U^{-1} L^{-1} P to
// n_t right-hand sides several times per frequency.  Forming L^{-1} and U^{-1}
// once (recursive blocked inversion, ztrtri-style, whose work is large GEMMs)
// turns every solve into two large tensor-core GEMMs instead of 2 n / 64
// dependent rank-64 steps.
namespace {

// In-place inverses of the 64 x 64 diagonal blocks of X (n x n, ld ldx; the
// last block may be smaller): unit lower (UPPER = false) or upper.  CTA b
// inverts block b; thread j computes column j.
constexpr int TRI_INV_SMEM = 2 * 64 * 65 * 8;

template <bool UPPER>
__global__ void __launch_bounds__(64) tri_inv_block_kernel(float *X0, int64_t ldx, int n) {
  extern __shared__ float2 tri_smem[];
  float2(*T)[65] = reinterpret_cast<float2(*)[65]>(tri_smem);            // T[col][row]
  float2(*R)[65] = reinterpret_cast<float2(*)[65]>(tri_smem + 64 * 65);  // R[col][row]
  const int o = blockIdx.x * 64, w = min(64, n - o);
  float *X = X0 + 2 * ((int64_t)o + ldx * o);
  const int j = threadIdx.x;
  for (int c = 0; c < w; c++)
    if (j < w) T[c][j] = reinterpret_cast<const float2 *>(X)[j + ldx * (int64_t)c];
  __syncthreads();
  if (j < w) {
    if (!UPPER) {
      for (int i = 0; i < w; i++) R[j][i] = make_float2(i == j ? 1.f : 0.f, 0.f);
      for (int i = j + 1; i < w; i++) {  // x_i = -sum_{j <= k < i} L_ik x_k
        float sr = 0.f, si = 0.f;
        for (int k = j; k < i; k++) {
          const float2 l = T[k][i], x = R[j][k];
          sr += l.x * x.x - l.y * x.y;
          si += l.x * x.y + l.y * x.x;
        }
        R[j][i] = make_float2(-sr, -si);
      }
    } else {
      for (int i = 0; i < w; i++) R[j][i] = make_float2(0.f, 0.f);
      {
        const float2 d = T[j][j];
        const float dd = d.x * d.x + d.y * d.y;
        R[j][j] = make_float2(d.x / dd, -d.y / dd);
      }
      for (int i = j - 1; i >= 0; i--) {  // x_i = -(sum_{i < k <= j} U_ik x_k) / U_ii
        float sr = 0.f, si = 0.f;
        for (int k = i + 1; k <= j; k++) {
          const float2 u = T[k][i], x = R[j][k];
          sr += u.x * x.x - u.y * x.y;
          si += u.x * x.y + u.y * x.x;
        }
        const float2 d = T[i][i];
        const float dd = d.x * d.x + d.y * d.y;
        // -(s / d) = -(s conj(d)) / |d|^2
        R[j][i] = make_float2(-(sr * d.x + si * d.y) / dd, -(si * d.x - sr * d.y) / dd);
      }
    }
  }
  __syncthreads();
  for (int c = 0; c < w; c++)
    if (j < w) reinterpret_cast<float2 *>(X)[j + ldx * (int64_t)c] = R[c][j];
}

// Copies the unit-lower factor (UPPER = false: ones on the diagonal, zeros
// above) or the upper factor (zeros below) of the packed LU into D.
template <bool UPPER>
__global__ void tri_extract_kernel(const float *__restrict__ LU, int64_t ld, int n, float *__restrict__ D) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  const int c = blockIdx.y;
  if (r >= n) return;
  float2 v = reinterpret_cast<const float2 *>(LU)[r + ld * (int64_t)c];
  if (!UPPER) {
    if (r < c) v = make_float2(0.f, 0.f);
    if (r == c) v = make_float2(1.f, 0.f);
  } else if (r > c) {
    v = make_float2(0.f, 0.f);
  }
  reinterpret_cast<float2 *>(D)[r + (int64_t)n * c] = v;
}

// In-place inversion of a triangle X (n x n, ld n) whose 64 x 64 diagonal
// blocks are already inverted (tri_inv_block_kernel), bottom up: at block size
// b the pairs of adjacent inverted b-blocks at offsets o = 0, 2b, 4b, ... are
// joined, lower: X21 = -X22 (L21 X11), upper: X12 = -X11 (U12 X22).  Below
// 512 all full pairs of a level are two strided-batch launches on the FMA
// pipes (hundreds of tiny products become six launches); from 512 up each
// pair is two tensor-core products.
int tri_inv_bottom_up(bemgpu_ctx_s *ctx, bool upper, float *X, int n, float *tmp, cudaStream_t st) {
  const float one[2] = {1.f, 0.f}, mone[2] = {-1.f, 0.f}, zero[2] = {0.f, 0.f};
  int rc = BEMGPU_OK;
  for (int b = NB; b < n && !rc; b *= 2) {
    const int full = n / (2 * b);  // pairs with both blocks b wide
    const int o_last = full * 2 * b;
    const int b2_last = std::min(b, n - o_last - b);  // ragged pair at o_last, if any
    auto at = [&](int r, int c) { return X + 2 * ((int64_t)r + (int64_t)n * c); };
    if (b < 512 && full > 0) {
      typedef GemmCfg<float> G;
      const dim3 grd((b + G::BM - 1) / G::BM, (b + G::BN - 1) / G::BN, full);
      const int64_t sx = 2 * ((int64_t)2 * b + (int64_t)n * 2 * b), st_ = 2 * (int64_t)b * b;
      const cx<float> c1 = {1.f, 0.f}, cm1 = {-1.f, 0.f}, c0 = {0.f, 0.f};
      ProfScope ps(ctx, BEMGPU_K_TRSM, st, 16.0 * full * (double)b * b * b, 48.0 * full * (double)b * b);
      if (!upper) {
        cgemm_fma_kernel<float, G::BM, G::BN, G::TM, G::TN, G::BK, false><<<grd, 256, 0, st>>>(
            b, b, b, c1, at(b, 0), n, at(0, 0), n, c0, tmp, b, sx, sx, st_);
        cgemm_fma_kernel<float, G::BM, G::BN, G::TM, G::TN, G::BK, false><<<grd, 256, 0, st>>>(
            b, b, b, cm1, at(b, b), n, tmp, b, c0, at(b, 0), n, sx, st_, sx);
      } else {
        cgemm_fma_kernel<float, G::BM, G::BN, G::TM, G::TN, G::BK, false><<<grd, 256, 0, st>>>(
            b, b, b, c1, at(0, b), n, at(b, b), n, c0, tmp, b, sx, sx, st_);
        cgemm_fma_kernel<float, G::BM, G::BN, G::TM, G::TN, G::BK, false><<<grd, 256, 0, st>>>(
            b, b, b, cm1, at(0, 0), n, tmp, b, c0, at(0, b), n, sx, st_, sx);
      }
      ctx->launches += 2;
      BEM_CUDA_TRY(ctx, cudaGetLastError());
    }
    for (int pi = (b < 512 ? full : 0); pi <= full && !rc; pi++) {
      const int o = pi * 2 * b, bb = pi < full ? b : b2_last;
      if (bb <= 0) continue;
      if (!upper) {
        rc = bem_cgemm(ctx, BEMGPU_K_TRSM, 'N', bb, b, b, one, at(o + b, o), n, at(o, o), n, zero, tmp, bb, st);
        if (!rc)
          rc = bem_cgemm(ctx, BEMGPU_K_TRSM, 'N', bb, b, bb, mone, at(o + b, o + b), n, tmp, bb, zero, at(o + b, o), n,
                         st);
      } else {
        rc = bem_cgemm(ctx, BEMGPU_K_TRSM, 'N', b, bb, bb, one, at(o, o + b), n, at(o + b, o + b), n, zero, tmp, b, st);
        if (!rc)
          rc = bem_cgemm(ctx, BEMGPU_K_TRSM, 'N', b, bb, b, mone, at(o, o), n, tmp, b, zero, at(o, o + b), n, st);
      }
    }
  }
  return rc;
}

}  // namespace

int bem_ctri_inverses(bemgpu_ctx_s *ctx, const float *LU, int64_t ld, int n, float *Linv, float *Uinv,
                      cudaStream_t st) {
  float *tmp = (float *)bem_workspace(ctx, "tri_tmp", 8 * (size_t)(n / 2 + NB) * (size_t)(n / 2 + NB));
  if (!tmp) return bem_fail(ctx, BEMGPU_ERR_OOM, "tri_inverses: workspace");
  {
    ProfScope ps(ctx, BEMGPU_K_TRSM, st, 0.0, 32.0 * (double)n * n);
    const dim3 g((n + 255) / 256, n);
    tri_extract_kernel<false><<<g, 256, 0, st>>>(LU, ld, n, Linv);
    tri_extract_kernel<true><<<g, 256, 0, st>>>(LU, ld, n, Uinv);
    ctx->launches += 2;
  }
  {
    static bool attr[64] = {false};
    if (!attr[ctx->device]) {
      BEM_CUDA_TRY(ctx, cudaFuncSetAttribute(tri_inv_block_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             TRI_INV_SMEM));
      BEM_CUDA_TRY(ctx, cudaFuncSetAttribute(tri_inv_block_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             TRI_INV_SMEM));
      attr[ctx->device] = true;
    }
    const int nb = (n + NB - 1) / NB;
    ProfScope ps(ctx, BEMGPU_K_TRSM, st, 2.0 * nb * 4.0 * NB * NB * NB / 3.0, 2.0 * 16.0 * NB * (double)n);
    tri_inv_block_kernel<false><<<nb, 64, TRI_INV_SMEM, st>>>(Linv, n, n);
    tri_inv_block_kernel<true><<<nb, 64, TRI_INV_SMEM, st>>>(Uinv, n, n);
    ctx->launches += 2;
  }
  int rc = tri_inv_bottom_up(ctx, false, Linv, n, tmp, st);
  if (!rc) rc = tri_inv_bottom_up(ctx, true, Uinv, n, tmp, st);
  if (rc) return rc;
  BEM_CUDA_TRY(ctx, cudaGetLastError());
  return BEMGPU_OK;
}

namespace {

// T(:, c) = Linv(:, pos(row0 + c)): L^-1 applied to the interchanged identity
// column row0 + c, where pos follows that column's 1 through the row
// interchanges ipiv[0..n) (laswp order).
__global__ void gather_linv_cols_kernel(const float *__restrict__ Linv, int n, const int *__restrict__ ipiv, int row0,
                                        int ncols, float *__restrict__ T) {
  __shared__ int s_pos;
  const int c = blockIdx.x;
  if (c >= ncols) return;
  if (threadIdx.x == 0) {
    int pos = row0 + c;
    for (int k = 0; k < n; k++) {
      const int p = ipiv[k];
      if (pos == k) pos = p;
      else if (pos == p) pos = k;
    }
    s_pos = pos;
  }
  __syncthreads();
  const float2 *src = reinterpret_cast<const float2 *>(Linv) + (int64_t)n * s_pos;
  float2 *dst = reinterpret_cast<float2 *>(T) + (int64_t)n * c;
  for (int r = threadIdx.x; r < n; r += blockDim.x) dst[r] = src[r];
}

}  // namespace

// B = W32^-1 E_t for the identity columns row0 .. row0 + nrhs: the interchanges
// and L^-1 reduce to gathering columns of L^-1, then one product with U^-1.
int bem_capply_inverse_identity(bemgpu_ctx_s *ctx, const float *Linv, const float *Uinv, int n, const int *d_ipiv,
                                int row0, float *B, int64_t ldb, int nrhs, float *tmp, cudaStream_t st) {
  {
    ProfScope ps(ctx, BEMGPU_K_SOLVE_GEMM, st, 0.0, 16.0 * (double)n * nrhs);
    gather_linv_cols_kernel<<<nrhs, 256, 0, st>>>(Linv, n, d_ipiv, row0, nrhs, tmp);
    ctx->launches++;
  }
  if (ctx->gemm_engine != 2 && n >= 64 && nrhs >= 64)
    return bem_cgemm_tc(ctx, BEMGPU_K_SOLVE_GEMM, n, nrhs, n, 1.f, Uinv, n, tmp, n, B, ldb, TC_OUT_F32, 0, st, 2);
  const float one[2] = {1.f, 0.f}, zero[2] = {0.f, 0.f};
  return bem_cgemm(ctx, BEMGPU_K_SOLVE_GEMM, 'N', n, nrhs, n, one, Uinv, n, tmp, n, zero, B, ldb, st);
}

int bem_capply_inverse(bemgpu_ctx_s *ctx, const float *Linv, const float *Uinv, int n, const int *d_ipiv, float *B,
                       int64_t ldb, int nrhs, float *tmp, cudaStream_t st) {
  const bool gather = n <= PERM_MAX_N && ctx->gemm_engine != 2 && n >= 64 && nrhs >= 64;
  if (gather) {
    // the interchanges as one row permutation, gathered into tmp; the two
    // products then alternate between tmp and B, and tmp goes back to B
    int *perm = (int *)bem_workspace(ctx, "lu_perm", sizeof(int) * (size_t)n);
    if (!perm) return bem_fail(ctx, BEMGPU_ERR_OOM, "apply inverse: permutation");
    if (!ctx->perm_ready) {
      BEM_CUDA_TRY(ctx, cudaFuncSetAttribute(perm_from_ipiv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)(2 * sizeof(int) * PERM_MAX_N)));
      ctx->perm_ready = true;
    }
    {
      ProfScope ps(ctx, BEMGPU_K_LU_PANEL, st, 0.0, 8.0 * n + 24.0 * (double)n * nrhs);
      perm_from_ipiv_kernel<<<1, 256, 2 * sizeof(int) * (size_t)n, st>>>(d_ipiv, n, perm);
      gather_rows_c64_kernel<<<dim3((unsigned)((n + 255) / 256), (unsigned)nrhs), 256, 0, st>>>(B, ldb, perm, n,
                                                                                                tmp, n);
      ctx->launches += 2;
    }
    BEM_CUDA_TRY(ctx, cudaGetLastError());
    int rc = bem_cgemm_tc(ctx, BEMGPU_K_SOLVE_GEMM, n, nrhs, n, 1.f, Linv, n, tmp, n, B, ldb, TC_OUT_F32, 0, st, 1);
    if (!rc) rc = bem_cgemm_tc(ctx, BEMGPU_K_SOLVE_GEMM, n, nrhs, n, 1.f, Uinv, n, B, ldb, tmp, n, TC_OUT_F32, 0, st, 2);
    if (rc) return rc;
    {
      ProfScope ps(ctx, BEMGPU_K_LU_PANEL, st, 0.0, 16.0 * (double)n * nrhs);
      BEM_CUDA_TRY(ctx, cudaMemcpy2DAsync(B, sizeof(float) * 2 * ldb, tmp, sizeof(float) * 2 * (size_t)n,
                                          sizeof(float) * 2 * (size_t)n, nrhs, cudaMemcpyDeviceToDevice, st));
    }
    return BEMGPU_OK;
  }
  {
    ProfScope ps(ctx, BEMGPU_K_LU_PANEL, st, 0.0, 32.0 * (double)n * nrhs);
    laswp_kernel<float><<<(nrhs + 127) / 128, 128, 0, st>>>(B, ldb, 0, nrhs, 0, n, d_ipiv);
    ctx->launches++;
  }
  if (ctx->gemm_engine != 2 && n >= 64 && nrhs >= 64) {  // tensor cores, zero triangles skipped
    int rc = bem_cgemm_tc(ctx, BEMGPU_K_SOLVE_GEMM, n, nrhs, n, 1.f, Linv, n, B, ldb, tmp, n, TC_OUT_F32, 0, st, 1);
    if (!rc) rc = bem_cgemm_tc(ctx, BEMGPU_K_SOLVE_GEMM, n, nrhs, n, 1.f, Uinv, n, tmp, n, B, ldb, TC_OUT_F32, 0, st, 2);
    return rc;
  }
  const float one[2] = {1.f, 0.f}, zero[2] = {0.f, 0.f};
  int rc = bem_cgemm(ctx, BEMGPU_K_SOLVE_GEMM, 'N', n, nrhs, n, one, Linv, n, B, ldb, zero, tmp, n, st);
  if (!rc) rc = bem_cgemm(ctx, BEMGPU_K_SOLVE_GEMM, 'N', n, nrhs, n, one, Uinv, n, tmp, n, zero, B, ldb, st);
  return rc;
}
