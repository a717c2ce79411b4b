// complex64 GEMM on the 5th-generation tensor cores (tcgen05, sm_103a).
//
// C (complex, column-major) = op(A) B [+ C]  with FP32-class accuracy:
//   * realified: D' = A' B'^T with A' (2m x 2k) built from A as
//       A'(2r, 2q) = Ar, A'(2r, 2q+1) = -Ai, A'(2r+1, 2q) = Ai, A'(2r+1, 2q+1) = Ar
//     and B' (n x 2k) the float view of B's columns, so D'(rho, c) is exactly
//     the float at offset rho + 2 ldc c of the complex column-major C: the
//     epilogue writes lanes straight to memory, coalesced.
//   * every FP32 operand value is split into three bf16 slices of natural
//     magnitude (x = s1 + s2 + s3 exactly); the six products with
//     slice indices (0-based) summing to <= 2 are accumulated into one FP32 TMEM accumulator,
//     which reproduces an FP32 product to ~2^-24.
//   * one CTA computes a 128 x 128 tile of D': warp 0 streams the three A and
//     three B slice tiles of each 64-deep K step with TMA (128-byte swizzle)
//     into a 2-stage mbarrier pipeline, warp 1 issues tcgen05.mma (one elected
//     thread, M=128 N=128 K=16, bf16 in, FP32 accumulate in TMEM), warps 2..5
//     read the accumulator back with tcgen05.ld and write C.
//   * every wait is bounded; a wait that runs out sets an error flag, the CTA
//     finishes, frees its TMEM and the host returns BEMGPU_ERR_TIMEOUT.
#include "bemgpu_internal.h"

#include <algorithm>

#include "tc_common.cuh"

namespace {

constexpr int TC_BM = 128, TC_BN = 128, TC_BK = 64;   // tile of D'; K step (bf16 elements, 128 bytes)
constexpr int TC_STAGES = 2;
constexpr int TC_SLICES = 3;
constexpr int TC_TILE_BYTES = TC_BM * TC_BK * 2;      // 16 KB per slice tile (A and B alike)
constexpr int TC_STAGE_BYTES = 2 * TC_SLICES * TC_TILE_BYTES;  // 96 KB
constexpr int TC_SMEM_BYTES = TC_STAGES * TC_STAGE_BYTES + 1024 + 256;
constexpr int TC_THREADS = 192;

// products (a, b) with a + b <= 2 (0-based slice indices), level-major:
// (0,0) (0,1) (1,0) (0,2) (1,1) (2,0)
__host__ __device__ constexpr int tc_level(int p) { return p < 1 ? 0 : p < 3 ? 1 : 2; }
__host__ __device__ constexpr int tc_prod_a(int p) { return p - tc_level(p) * (tc_level(p) + 1) / 2; }
__host__ __device__ constexpr int tc_prod_b(int p) { return tc_level(p) - tc_prod_a(p); }

__device__ __forceinline__ void drain_copies(uint64_t *full, int issued, int *err) {
  for (int kt = issued > TC_STAGES ? issued - TC_STAGES : 0; kt < issued; kt++)
    if (!mbar_wait(&full[kt % TC_STAGES], (kt / TC_STAGES) & 1, err)) return;
}

struct TcMaps {
  CUtensorMap a[TC_SLICES];
  CUtensorMap b[TC_SLICES];
};

}  // namespace

namespace {

// One 128 x 128 tile of D' = sum_{(a,b)} A'_a B'_b^T over ktiles 64-deep K steps.
// C is written as TOUT at C[rho + ldcf * c] for rho < mvalid, c < nvalid
// (accumulate: C += D'; otherwise C = D').
template <typename TOUT>
__global__ void __launch_bounds__(TC_THREADS, 1)
    tc_gemm_kernel(const __grid_constant__ TcMaps maps, int ktiles, TOUT *__restrict__ C, int64_t ldcf, int mvalid,
                   int nvalid, int accumulate, int tri, int raster, int *err) {
  extern __shared__ unsigned char tc_smem_raw[];
  unsigned char *smem = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(tc_smem_raw) + 1023) &
                                                          ~(uintptr_t)1023);
  uint64_t *full = reinterpret_cast<uint64_t *>(smem + TC_STAGES * TC_STAGE_BYTES);
  uint64_t *empty = full + TC_STAGES;
  uint64_t *accum_bar = empty + TC_STAGES;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(accum_bar + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int mt, nt;
  grouped_tile(raster, mt, nt);
  const int m0 = mt * TC_BM, n0 = nt * TC_BN;

  if (threadIdx.x == 0) {
    for (int s = 0; s < TC_STAGES; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(accum_bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(TC_BN));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    asm volatile("tcgen05.fence::before_thread_sync;");
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = *tmem_slot;

  // K range: all of it, or for a triangular complex A only the K steps that
  // meet nonzero entries of this tile's rows (lower: columns <= row, upper:
  // columns >= row; realified row rho and column kappa belong to complex
  // row rho / 2 and column kappa / 2).
  const int kb = tri == 2 ? m0 / TC_BK : 0;
  const int ke = tri == 1 ? min(ktiles, (m0 + TC_BM + TC_BK - 1) / TC_BK) : ktiles;
  const int nk = max(0, ke - kb);
  if (warp == 0) {
    if (lane == 0) {
      int issued = 0;
      for (int j = 0; j < nk; j++) {
        const int kt = kb + j, s = j % TC_STAGES, round = j / TC_STAGES;
        if (j >= TC_STAGES && !mbar_wait(&empty[s], (round - 1) & 1, err)) break;
        mbar_expect_tx(&full[s], TC_STAGE_BYTES);
        unsigned char *st = smem + s * TC_STAGE_BYTES;
#pragma unroll
        for (int a = 0; a < TC_SLICES; a++) tma_load_2d(st + a * TC_TILE_BYTES, &maps.a[a], kt * TC_BK, m0, &full[s]);
#pragma unroll
        for (int b = 0; b < TC_SLICES; b++)
          tma_load_2d(st + (TC_SLICES + b) * TC_TILE_BYTES, &maps.b[b], kt * TC_BK, n0, &full[s]);
        issued = j + 1;
      }
      drain_copies(full, issued, err);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      constexpr uint32_t idesc = tc_idesc(TC_BM, TC_BN);
      bool ok = true;
      for (int j = 0; j < nk && ok; j++) {
        const int s = j % TC_STAGES, round = j / TC_STAGES;
        ok = mbar_wait(&full[s], round & 1, err);
        if (!ok) break;
        asm volatile("tcgen05.fence::after_thread_sync;");
        const uint64_t dbase = smem_desc_sw128(smem_u32(smem + s * TC_STAGE_BYTES));
#pragma unroll
        for (int ks = 0; ks < TC_BK / 16; ks++) {
#pragma unroll
          for (int p = 0; p < 6; p++) {
            const uint64_t da = dbase + (uint64_t)((tc_prod_a(p) * TC_TILE_BYTES + ks * 32) >> 4);
            const uint64_t db = dbase + (uint64_t)(((TC_SLICES + tc_prod_b(p)) * TC_TILE_BYTES + ks * 32) >> 4);
            tc_mma(tmem, da, db, idesc, (j | ks | p) != 0 ? 1u : 0u);
          }
        }
        tc_commit(&empty[s]);
      }
      tc_commit(accum_bar);
    }
  } else {
    // epilogue: warps 2..5; warp w reads TMEM lanes 32*(w % 4) .. +31
    const int sub = warp & 3;
    const bool ok = mbar_wait(accum_bar, 0, err);
    __syncwarp();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const int rho = m0 + sub * 32 + lane;
#pragma unroll 1
    for (int c0 = 0; c0 < TC_BN; c0 += 32) {
      // the chunk's old C values first, all loads in flight together
      TOUT old[32];
#pragma unroll
      for (int j = 0; j < 32; j++) {
        const int c = n0 + c0 + j;
        old[j] = (accumulate && ok && rho < mvalid && c < nvalid) ? C[rho + ldcf * (int64_t)c] : (TOUT)0;
      }
      float v[32];
      tc_ld32(tmem + ((uint32_t)(sub * 32) << 16) + (uint32_t)c0, v);
      if (nk == 0) {
#pragma unroll
        for (int j = 0; j < 32; j++) v[j] = 0.f;
      }
      if (ok && rho < mvalid) {
#pragma unroll
        for (int j = 0; j < 32; j++) {
          const int c = n0 + c0 + j;
          if (c < nvalid) C[rho + ldcf * (int64_t)c] = old[j] + (TOUT)v[j];
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_BN));
  }
}


constexpr int TCC_BN = 64;                     // tile of D': 128 x 64
constexpr int TCC_STAGES = 3;
constexpr int TCC_B_TILE_BYTES = TCC_BN * TC_BK * 2;  // 8 KB per B slice tile
constexpr int TCC_STAGE_BYTES = TC_SLICES * (TC_TILE_BYTES + TCC_B_TILE_BYTES);  // 72 KB
constexpr int TCC_SMEM_BYTES = TCC_STAGES * TCC_STAGE_BYTES + 1024 + 256;
constexpr int TCC_EPI_WARPS = 8;
constexpr int TCC_TMEM_COLS = 512;  // 2 x (X, Y1, Y2) x 64 columns, rounded to a power of two
constexpr int TCC_THREADS = 64 + 32 * TCC_EPI_WARPS;


// One 128 x 64 tile of D' summed exactly enough for a refinement residual.
// The operands arrive as block fixed-point slices (one exponent per row and
// 32-column block, split3_fixed), so per 64-deep K step the slice products of
// one level share one unit and the tensor cores sum them EXACTLY in FP32
// (64 products of |q| <= 2^16 stay below 2^24): level 0 (q1 q1) into X,
// level 1 (q1 q2, q2 q1) into Y1, level 2 (q1 q3, q2 q2, q3 q1) into Y2.  No
// rounding, hence no truncation bias, enters on the tensor cores; the only
// roundings are the slicing's (to nearest) and the FP32 adds of the drain.
// Buffers (TMEM columns, b = K step parity): X at 192 b, Y1 at 192 b + 64,
// Y2 at 192 b + 128.  Eight epilogue warps drain a step while the next runs:
// hi + lo += X by TwoSum, lo += Y1 + Y2.  Warp 2 + e holds TMEM lanes
// 32 (warp % 4) and tile columns 32 (e / 4) .. + 31.
// C (FP64) = hi + lo [+ C] at C[rho + ldcf c].
__global__ void __launch_bounds__(TCC_THREADS, 1)
    tc_gemm_comp_kernel(const __grid_constant__ TcMaps maps, int ktiles, double *__restrict__ C, int64_t ldcf,
                        int mvalid, int nvalid, int accumulate, int raster, int *err) {
  extern __shared__ unsigned char tc_smem_raw[];
  unsigned char *smem = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(tc_smem_raw) + 1023) &
                                                          ~(uintptr_t)1023);
  uint64_t *full = reinterpret_cast<uint64_t *>(smem + TCC_STAGES * TCC_STAGE_BYTES);
  uint64_t *empty = full + TCC_STAGES;
  uint64_t *accf = empty + TCC_STAGES;  // accumulator buffer b written (MMA -> epilogue)
  uint64_t *acce = accf + 2;            // accumulator buffer b drained (epilogue -> MMA)
  uint64_t *fin = acce + 2;             // all MMAs of this CTA complete
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(fin + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int mt, nt;
  grouped_tile(raster, mt, nt);
  const int m0 = mt * TC_BM, n0 = nt * TCC_BN;

  if (threadIdx.x == 0) {
    for (int s = 0; s < TCC_STAGES; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; b++) {
      mbar_init(&accf[b], 1);
      mbar_init(&acce[b], TCC_EPI_WARPS);
    }
    mbar_init(fin, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(TCC_TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    asm volatile("tcgen05.fence::before_thread_sync;");
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      int issued = 0;
      for (int kt = 0; kt < ktiles; kt++) {
        const int s = kt % TCC_STAGES, round = kt / TCC_STAGES;
        if (kt >= TCC_STAGES && !mbar_wait(&empty[s], (round - 1) & 1, err)) break;
        mbar_expect_tx(&full[s], TCC_STAGE_BYTES);
        unsigned char *st = smem + s * TCC_STAGE_BYTES;
#pragma unroll
        for (int a = 0; a < TC_SLICES; a++) tma_load_2d(st + a * TC_TILE_BYTES, &maps.a[a], kt * TC_BK, m0, &full[s]);
#pragma unroll
        for (int b = 0; b < TC_SLICES; b++)
          tma_load_2d(st + TC_SLICES * TC_TILE_BYTES + b * TCC_B_TILE_BYTES, &maps.b[b], kt * TC_BK, n0, &full[s]);
        issued = kt + 1;
      }
      for (int kt = issued > TCC_STAGES ? issued - TCC_STAGES : 0; kt < issued; kt++)
        if (!mbar_wait(&full[kt % TCC_STAGES], (kt / TCC_STAGES) & 1, err)) break;
    }
  } else if (warp == 1) {
    if (lane == 0) {
      constexpr uint32_t idesc = tc_idesc(TC_BM, TCC_BN);
      for (int kt = 0; kt < ktiles; kt++) {
        const int s = kt % TCC_STAGES, round = kt / TCC_STAGES, b = kt & 1, use = kt >> 1;
        if (kt >= 2 && !mbar_wait(&acce[b], (use - 1) & 1, err)) break;
        if (!mbar_wait(&full[s], round & 1, err)) break;
        asm volatile("tcgen05.fence::after_thread_sync;");
        const uint32_t st = smem_u32(smem + s * TCC_STAGE_BYTES);
        const uint32_t tx = tmem + (uint32_t)(3 * b * TCC_BN);
#pragma unroll
        for (int ks = 0; ks < TC_BK / 16; ks++) {
#pragma unroll
          for (int p = 0; p < 6; p++) {
            const uint64_t da = smem_desc_sw128(st + tc_prod_a(p) * TC_TILE_BYTES + ks * 32);
            const uint64_t db =
                smem_desc_sw128(st + TC_SLICES * TC_TILE_BYTES + tc_prod_b(p) * TCC_B_TILE_BYTES + ks * 32);
            const int level = p == 0 ? 0 : (p < 3 ? 1 : 2);
            const int first = p == 0 ? 0 : (p < 3 ? 1 : 3);  // first product of its level
            tc_mma(tx + (uint32_t)(level * TCC_BN), da, db, idesc, (ks != 0 || p != first) ? 1u : 0u);
          }
        }
        tc_commit(&empty[s]);
        tc_commit(&accf[b]);
      }
      tc_commit(fin);
      mbar_wait(fin, 0, err);
    }
  } else {
    const int quarter = warp & 3, group = (warp - 2) >> 2;
    float hi[32], lo[32];
#pragma unroll
    for (int j = 0; j < 32; j++) hi[j] = lo[j] = 0.f;
    bool ok = true;
#pragma unroll 1
    for (int kt = 0; kt < ktiles; kt++) {
      const int b = kt & 1, use = kt >> 1;
      int got = 1;
      if (lane == 0) got = mbar_wait(&accf[b], use & 1, err) ? 1 : 0;
      got = __shfl_sync(0xffffffffu, got, 0);
      if (!got) {
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;");
      const uint32_t tx = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(3 * b * TCC_BN + group * 32);
#pragma unroll
      for (int q = 0; q < 4; q++) {
        float x[8], y1[8], y2[8];
        tc_ld8(tx + 8 * q, x);
        tc_ld8(tx + TCC_BN + 8 * q, y1);
        tc_ld8(tx + 2 * TCC_BN + 8 * q, y2);
#pragma unroll
        for (int j = 0; j < 8; j++) {
          two_sum_acc(hi[8 * q + j], lo[8 * q + j], x[j]);
          lo[8 * q + j] += y1[j] + y2[j];
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;");
      __syncwarp();
      if (lane == 0) mbar_arrive(&acce[b]);
    }
    const int rho = m0 + quarter * 32 + lane;
    if (ok && rho < mvalid) {
#pragma unroll
      for (int j = 0; j < 32; j++) {
        const int c = n0 + group * 32 + j;
        if (c < nvalid) {
          double *p = C + rho + ldcf * (int64_t)c;
          const double v = (double)hi[j] + (double)lo[j];
          *p = accumulate ? *p + v : v;
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TCC_TMEM_COLS));
  }
}

__device__ __forceinline__ void split3(float x, __nv_bfloat16 &s1, __nv_bfloat16 &s2, __nv_bfloat16 &s3) {
  s1 = __float2bfloat16_rn(x);
  const float r1 = x - __bfloat162float(s1);
  s2 = __float2bfloat16_rn(r1);
  const float r2 = r1 - __bfloat162float(s2);
  s3 = __float2bfloat16_rn(r2);
}

// Block fixed point: with |x| < 2^E (E from the block's largest magnitude),
// x = (q1 2^-8 + q2 2^-16 + q3 2^-24) 2^E + r, integers |q1| <= 256,
// |q2|, |q3| <= 128, |r| <= 2^(E-25), each step rounded to nearest.  Every
// slice of the block is a multiple of one unit per level, so the tensor cores
// sum a block's slice products exactly.  E = FIXED_ZERO flushes the block.
constexpr int FIXED_ZERO = -1000;

__device__ __forceinline__ float pow2f(int e) { return __int_as_float((127 + e) << 23); }  // e in [-126, 127]

__device__ __forceinline__ void split3_fixed(float x, int E, __nv_bfloat16 &s1, __nv_bfloat16 &s2, __nv_bfloat16 &s3) {
  if (E == FIXED_ZERO) {
    s1 = s2 = s3 = __float2bfloat16_rn(0.f);
    return;
  }
  const float v1 = rintf(x * pow2f(8 - E)) * pow2f(E - 8);
  const float r1 = x - v1;  // exact
  const float v2 = rintf(r1 * pow2f(16 - E)) * pow2f(E - 16);
  const float r2 = r1 - v2;  // exact
  const float v3 = rintf(r2 * pow2f(24 - E)) * pow2f(E - 24);
  s1 = __float2bfloat16_rn(v1);  // exact: at most 9 significant bits
  s2 = __float2bfloat16_rn(v2);
  s3 = __float2bfloat16_rn(v3);
}

// E with mx < 2^E for a block whose largest magnitude is mx; FIXED_ZERO when
// the block is zero or below 2^-100.
__device__ __forceinline__ int block_exponent(float mx) {
  const int eb = (__float_as_int(mx) >> 23) & 0xff;  // mx in [2^(eb-127), 2^(eb-126))
  const int E = eb - 126;
  return (eb == 0 || E < -100) ? FIXED_ZERO : E;
}

__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// A' slices (Mp x Kp, K contiguous) from complex column-major A (m x k):
// rows 2r: (Ar, -Ai), rows 2r+1: (Ai, Ar) at columns (2q, 2q+1); times sign.
// fixed: block fixed point over each row's 32-column (one K step) blocks,
// else natural bf16 slices.  A warp covers one block (q aligned to 32).
__global__ void tc_prep_a_kernel(const float *__restrict__ A, int64_t lda, int m, int k, float sign,
                                 __nv_bfloat16 *__restrict__ S, int64_t Mp, int64_t Kp, int fixed) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;  // complex column (fast: coalesced writes)
  const int r = blockIdx.y;                              // complex row
  if (2 * q >= Kp) return;                              // whole warps: Kp / 2 is a multiple of 32
  float ar = 0.f, ai = 0.f;
  if (r < m && q < k) {
    const float2 v = reinterpret_cast<const float2 *>(A)[r + lda * (int64_t)q];
    ar = sign * v.x;
    ai = sign * v.y;
  }
  const int E = fixed ? block_exponent(warp_max(fmaxf(fabsf(ar), fabsf(ai)))) : 0;
  const float row0[2] = {ar, -ai}, row1[2] = {ai, ar};
  const int64_t plane = Mp * Kp;
  for (int h = 0; h < 2; h++) {
    const float *rv = h ? row1 : row0;
    __nv_bfloat16 a1, a2, a3, b1, b2, b3;
    if (fixed) {
      split3_fixed(rv[0], E, a1, a2, a3);
      split3_fixed(rv[1], E, b1, b2, b3);
    } else {
      split3(rv[0], a1, a2, a3);
      split3(rv[1], b1, b2, b3);
    }
    const int64_t idx = (int64_t)(2 * r + h) * Kp + 2 * q;
    reinterpret_cast<__nv_bfloat162 *>(S + idx)[0] = __halves2bfloat162(a1, b1);
    reinterpret_cast<__nv_bfloat162 *>(S + plane + idx)[0] = __halves2bfloat162(a2, b2);
    reinterpret_cast<__nv_bfloat162 *>(S + 2 * plane + idx)[0] = __halves2bfloat162(a3, b3);
  }
}

// B' slices (Np x Kp): row c = the float view of column c of complex B (k x n).
__global__ void tc_prep_b_kernel(const float *__restrict__ B, int64_t ldb, int k, int n, __nv_bfloat16 *__restrict__ S,
                                 int64_t Np, int64_t Kp, int fixed) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;  // complex row of B
  const int c = blockIdx.y;
  if (2 * q >= Kp) return;
  float br = 0.f, bi = 0.f;
  if (c < n && q < k) {
    const float2 v = reinterpret_cast<const float2 *>(B)[q + ldb * (int64_t)c];
    br = v.x;
    bi = v.y;
  }
  __nv_bfloat16 a1, a2, a3, b1, b2, b3;
  if (fixed) {
    const int E = block_exponent(warp_max(fmaxf(fabsf(br), fabsf(bi))));
    split3_fixed(br, E, a1, a2, a3);
    split3_fixed(bi, E, b1, b2, b3);
  } else {
    split3(br, a1, a2, a3);
    split3(bi, b1, b2, b3);
  }
  const int64_t plane = Np * Kp, idx = (int64_t)c * Kp + 2 * q;
  reinterpret_cast<__nv_bfloat162 *>(S + idx)[0] = __halves2bfloat162(a1, b1);
  reinterpret_cast<__nv_bfloat162 *>(S + plane + idx)[0] = __halves2bfloat162(a2, b2);
  reinterpret_cast<__nv_bfloat162 *>(S + 2 * plane + idx)[0] = __halves2bfloat162(a3, b3);
}

bool make_map(CUtensorMap *map, const void *base, int64_t rows, int64_t kp, int box_rows = TC_BM) {
  return make_map_bf16(map, base, rows, kp, TC_BK, box_rows, CU_TENSOR_MAP_SWIZZLE_128B);
}

}  // namespace

int bem_tc_error(bemgpu_ctx_s *ctx, bool reset) {
  int *err = (int *)bem_workspace(ctx, "tc_err", sizeof(int));
  if (!err) return 0;
  int h = 0;
  cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
  cudaStreamSynchronize(ctx->stream);
  if (reset && h) cudaMemsetAsync(err, 0, sizeof(int), ctx->stream);
  return h;
}

// C (+)= sign * A B on the tensor cores.  out: TC_OUT_F32 (complex64 C),
// TC_OUT_F64 (complex128 C, FP32 accumulation), TC_OUT_F64_COMP (complex128
// C, per-K-step FP32 sums accumulated as two-float sums).  Column-major, ldc.
void bem_cgemm_tc_bytes(int m, int n, int k, size_t &a_bytes, size_t &b_bytes) {
  const int64_t Mp = ((2 * (int64_t)m + TC_BM - 1) / TC_BM) * TC_BM;
  const int64_t Np = (((int64_t)n + TC_BN - 1) / TC_BN) * TC_BN;
  const int64_t Kp = ((2 * (int64_t)k + TC_BK - 1) / TC_BK) * TC_BK;
  a_bytes = sizeof(__nv_bfloat16) * TC_SLICES * (size_t)(Mp * Kp);
  b_bytes = sizeof(__nv_bfloat16) * TC_SLICES * (size_t)(Np * Kp);
}

int bem_cgemm_tc(bemgpu_ctx_s *ctx, int kind, int m, int n, int k, float sign, const float *A, int64_t lda,
                 const float *B, int64_t ldb, void *C, int64_t ldc, int out, int accumulate, cudaStream_t st,
                 int tri) {
  if (m <= 0 || n <= 0) return BEMGPU_OK;
  if (k <= 0) return bem_fail(ctx, BEMGPU_ERR_ARG, "cgemm_tc: k = %d", k);
  const int64_t Mp = ((2 * (int64_t)m + TC_BM - 1) / TC_BM) * TC_BM;
  const int bn = out == TC_OUT_F64_COMP ? TCC_BN : TC_BN;
  const int64_t Np = (((int64_t)n + bn - 1) / bn) * bn;
  const int64_t Kp = ((2 * (int64_t)k + TC_BK - 1) / TC_BK) * TC_BK;
  if (Mp / 2 > 65535 || Np > 65535) return bem_fail(ctx, BEMGPU_ERR_ARG, "cgemm_tc: %d x %d too large", m, n);
  if (!ctx->tc_ready) {
    BEM_CUDA_TRY(ctx, cudaFuncSetAttribute(tc_gemm_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           TC_SMEM_BYTES));
    BEM_CUDA_TRY(ctx, cudaFuncSetAttribute(tc_gemm_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           TC_SMEM_BYTES));
    BEM_CUDA_TRY(ctx, cudaFuncSetAttribute(tc_gemm_comp_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           TCC_SMEM_BYTES));
    ctx->tc_ready = true;
  }
  __nv_bfloat16 *SA = (__nv_bfloat16 *)bem_workspace(ctx, "tc_A", sizeof(__nv_bfloat16) * TC_SLICES * Mp * Kp);
  __nv_bfloat16 *SB = (__nv_bfloat16 *)bem_workspace(ctx, "tc_B", sizeof(__nv_bfloat16) * TC_SLICES * Np * Kp);
  int *err = (int *)bem_workspace(ctx, "tc_err", sizeof(int));
  if (!SA || !SB || !err) return bem_fail(ctx, BEMGPU_ERR_OOM, "cgemm_tc: workspace");
  if (!ctx->tc_err_ready) {
    BEM_CUDA_TRY(ctx, cudaMemsetAsync(err, 0, sizeof(int), st));
    ctx->tc_err_ready = true;
  }
  TcMaps maps;
  for (int i = 0; i < TC_SLICES; i++) {
    if (!make_map(&maps.a[i], SA + i * Mp * Kp, Mp, Kp) || !make_map(&maps.b[i], SB + i * Np * Kp, Np, Kp, bn))
      return bem_fail(ctx, BEMGPU_ERR_CUDA, "cgemm_tc: tensor map encoding failed");
  }
  {
    ProfScope ps(ctx, BEMGPU_K_SLICE, st, 0.0,
                 8.0 * ((double)m * k + (double)k * n) + 12.0 * ((double)Mp * Kp + (double)Np * Kp));
    const int fixed = out == TC_OUT_F64_COMP ? 1 : 0;
    tc_prep_a_kernel<<<dim3((unsigned)((Kp / 2 + 127) / 128), (unsigned)(Mp / 2)), 128, 0, st>>>(A, lda, m, k, sign, SA,
                                                                                                 Mp, Kp, fixed);
    ctx->launches++;
    tc_prep_b_kernel<<<dim3((unsigned)((Kp / 2 + 127) / 128), (unsigned)Np), 128, 0, st>>>(B, ldb, k, n, SB, Np, Kp,
                                                                                            fixed);
    ctx->launches++;
  }
  {
    const double cbytes = (out == TC_OUT_F32 ? 4.0 : 8.0) * 2.0 * m * n * (accumulate ? 2.0 : 1.0);
    // a triangular A: only the K steps the kernel runs for each M tile (the
    // bounds of tc_gemm_kernel) count as work
    double run = 1.0;
    if (tri) {
      const int64_t mtiles = Mp / TC_BM, ktiles = Kp / TC_BK;
      int64_t steps = 0;
      for (int64_t mt = 0; mt < mtiles; mt++) {
        const int64_t m0 = mt * TC_BM;
        const int64_t kb = tri == 2 ? m0 / TC_BK : 0;
        const int64_t ke = tri == 1 ? std::min(ktiles, (m0 + TC_BM + TC_BK - 1) / TC_BK) : ktiles;
        steps += std::max<int64_t>(0, ke - kb);
      }
      run = (double)steps / ((double)mtiles * (double)ktiles);
    }
    ProfScope ps(ctx, kind, st, 8.0 * m * n * (double)k * run,
                 12.0 * ((double)Mp * Kp * run + (double)Np * Kp) + cbytes);
    ps.tensor = 6.0 * ps.flops;  // slice products (a, b) with a + b <= 2 of 3 slices
    const dim3 grid((unsigned)(Mp / TC_BM), (unsigned)(Np / bn));
    const int kt = (int)(Kp / TC_BK);
    if (out == TC_OUT_F64_COMP)
      tc_gemm_comp_kernel<<<grid, TCC_THREADS, TCC_SMEM_BYTES, st>>>(maps, kt, (double *)C, 2 * ldc, 2 * m, n,
                                                                    accumulate, ctx->tune.raster, err);
    else if (out == TC_OUT_F64)
      tc_gemm_kernel<double><<<grid, TC_THREADS, TC_SMEM_BYTES, st>>>(maps, kt, (double *)C, 2 * ldc, 2 * m, n,
                                                                      accumulate, tri, ctx->tune.raster, err);
    else
      tc_gemm_kernel<float><<<grid, TC_THREADS, TC_SMEM_BYTES, st>>>(maps, kt, (float *)C, 2 * ldc, 2 * m, n,
                                                                     accumulate, tri, ctx->tune.raster, err);
    ctx->launches++;
  }
  BEM_CUDA_TRY(ctx, cudaGetLastError());
  return BEMGPU_OK;
}

// Below 64 (complex) K the FMA pipes win; from rank-64 updates on (the LU
// trailing matrix: 66 TF/s vs 28 at 7680^2 x 64) the tensor cores do.
constexpr int TC_MIN_K = 64;

static bool tc_usable(int engine, int m, int n, int k) {
  return engine != 2 && (engine == 1 || k >= TC_MIN_K) && m >= 64 && n >= 64 && k >= 16 && 2 * (int64_t)m <= 2 * 65535 &&
         (int64_t)n <= 65535 - TC_BN && encode_fn() != nullptr;
}

int bem_cgemm(bemgpu_ctx_s *ctx, int kind, char opA, int m, int n, int k, const float alpha[2], const float *A,
              int64_t lda, const float *B, int64_t ldb, const float beta[2], float *C, int64_t ldc,
              cudaStream_t stream) {
  const bool real_unit_alpha = alpha[1] == 0.f && (alpha[0] == 1.f || alpha[0] == -1.f);
  const bool beta01 = beta[1] == 0.f && (beta[0] == 0.f || beta[0] == 1.f);
  if (opA == 'N' && real_unit_alpha && beta01 && tc_usable(ctx->gemm_engine, m, n, k))
    return bem_cgemm_tc(ctx, kind, m, n, k, alpha[0], A, lda, B, ldb, C, ldc, TC_OUT_F32, beta[0] == 1.f ? 1 : 0,
                        stream);
  return bem_cgemm_fma(ctx, kind, opA, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, stream);
}

int bem_cgemm_comp64(bemgpu_ctx_s *ctx, int kind, int m, int n, int k, const float alpha[2], const float *A,
                     int64_t lda, const float *B, int64_t ldb, const double beta[2], double *C, int64_t ldc,
                     cudaStream_t stream) {
  const bool real_unit_alpha = alpha[1] == 0.f && (alpha[0] == 1.f || alpha[0] == -1.f);
  const bool beta01 = beta[1] == 0.0 && (beta[0] == 0.0 || beta[0] == 1.0);
  if (real_unit_alpha && beta01 && tc_usable(ctx->acc_engine, m, n, k))
    return bem_cgemm_tc(ctx, kind, m, n, k, alpha[0], A, lda, B, ldb, C, ldc, TC_OUT_F64_COMP,
                        beta[0] == 1.0 ? 1 : 0, stream);
  return bem_cgemm_comp64_fma(ctx, kind, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, stream);
}

extern "C" int bemgpu_cgemm(bemgpu_ctx_t ctx, int m, int n, int k, const float *dA, int64_t lda, const float *dB,
                            int64_t ldb, float *dC, int64_t ldc, int accumulate, int engine) {
  if (!ctx || !dA || !dB || !dC || m < 0 || n < 0 || k < 1 || lda < m || ldb < k || ldc < m)
    return bem_fail(ctx, BEMGPU_ERR_ARG, "cgemm: bad arguments");
  std::lock_guard<std::mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  const float one[2] = {1.f, 0.f}, zero[2] = {0.f, 0.f};
  int rc;
  if (engine == 1) {
    if (!encode_fn()) return bem_fail(ctx, BEMGPU_ERR_CUDA, "cgemm: tensor maps unavailable");
    rc = bem_cgemm_tc(ctx, BEMGPU_K_TRACE, m, n, k, 1.f, dA, lda, dB, ldb, dC, ldc, TC_OUT_F32, accumulate,
                      ctx->stream);
  } else if (engine == 2) {
    rc = bem_cgemm_fma(ctx, BEMGPU_K_TRACE, 'N', m, n, k, one, dA, lda, dB, ldb, accumulate ? one : zero, dC, ldc,
                       ctx->stream);
  } else {
    rc = bem_cgemm(ctx, BEMGPU_K_TRACE, 'N', m, n, k, one, dA, lda, dB, ldb, accumulate ? one : zero, dC, ldc,
                   ctx->stream);
  }
  if (rc) return rc;
  BEM_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  if (bem_tc_error(ctx, true)) return bem_fail(ctx, BEMGPU_ERR_TIMEOUT, "cgemm: a tensor-core pipeline wait ran out");
  return BEMGPU_OK;
}

extern "C" int bemgpu_cgemm_acc64(bemgpu_ctx_t ctx, int m, int n, int k, const float *dA, int64_t lda,
                                  const float *dB, int64_t ldb, double *dC, int64_t ldc, int accumulate,
                                  int engine) {
  if (!ctx || !dA || !dB || !dC || m < 0 || n < 0 || k < 1 || lda < m || ldb < k || ldc < m)
    return bem_fail(ctx, BEMGPU_ERR_ARG, "cgemm_acc64: bad arguments");
  std::lock_guard<std::mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  const float one[2] = {1.f, 0.f};
  const double one64[2] = {1.0, 0.0}, zero64[2] = {0.0, 0.0};
  int rc;
  if (engine == 1) {
    if (!encode_fn()) return bem_fail(ctx, BEMGPU_ERR_CUDA, "cgemm_acc64: tensor maps unavailable");
    rc = bem_cgemm_tc(ctx, BEMGPU_K_TRACE, m, n, k, 1.f, dA, lda, dB, ldb, dC, ldc, TC_OUT_F64_COMP, accumulate,
                      ctx->stream);
  } else if (engine == 2) {
    rc = bem_cgemm_comp64_fma(ctx, BEMGPU_K_TRACE, m, n, k, one, dA, lda, dB, ldb, accumulate ? one64 : zero64, dC,
                              ldc, ctx->stream);
  } else {
    rc = bem_cgemm_comp64(ctx, BEMGPU_K_TRACE, m, n, k, one, dA, lda, dB, ldb, accumulate ? one64 : zero64, dC, ldc,
                          ctx->stream);
  }
  if (rc) return rc;
  BEM_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  if (bem_tc_error(ctx, true))
    return bem_fail(ctx, BEMGPU_ERR_TIMEOUT, "cgemm_acc64: a tensor-core pipeline wait ran out");
  return BEMGPU_OK;
}

namespace {

// Polls a word that nothing sets, at most `spins` times and about a second of
// clock, then records a timeout in the context's error flag: the same exit
// every bounded wait of the library takes (TMA / MMA pipelines, grid barriers).
__global__ void wait_selftest_kernel(const unsigned *flag, long long spins, long long max_cycles, int *err) {
  if (threadIdx.x != 0) return;
  const long long t0 = clock64();
  for (long long it = 0; it < spins; it++) {
    if (*(volatile const unsigned *)flag != 0u) return;
    if (clock64() - t0 > max_cycles) break;
  }
  atomicExch(err, 1);
}

}  // namespace

extern "C" int bemgpu_ctx_wait_selftest(bemgpu_ctx_t ctx, int64_t spins) {
  if (!ctx || spins < 1 || spins > 100000000) return bem_fail(ctx, BEMGPU_ERR_ARG, "wait_selftest: spins in [1, 1e8]");
  std::lock_guard<std::mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  unsigned *flag = (unsigned *)bem_workspace(ctx, "selftest_flag", sizeof(unsigned));
  int *err = (int *)bem_workspace(ctx, "tc_err", sizeof(int));
  if (!flag || !err) return bem_fail(ctx, BEMGPU_ERR_OOM, "wait_selftest: workspace");
  if (!ctx->tc_err_ready) {
    BEM_CUDA_TRY(ctx, cudaMemsetAsync(err, 0, sizeof(int), ctx->stream));
    ctx->tc_err_ready = true;
  }
  BEM_CUDA_TRY(ctx, cudaMemsetAsync(flag, 0, sizeof(unsigned), ctx->stream));
  wait_selftest_kernel<<<1, 32, 0, ctx->stream>>>(flag, (long long)spins, 2000000000ll, err);
  ctx->launches++;
  BEM_CUDA_TRY(ctx, cudaGetLastError());
  if (bem_tc_error(ctx, true))
    return bem_fail(ctx, BEMGPU_ERR_TIMEOUT, "wait_selftest: the bounded wait ran out after %lld polls", (long long)spins);
  return BEMGPU_OK;
}

extern "C" int bemgpu_ctx_set_solver(bemgpu_ctx_t ctx, int mode) {
  if (!ctx || mode < 0 || mode > 2)
    return bem_fail(ctx, BEMGPU_ERR_ARG, "set_solver: modes are 0 (complex64, escalating), 1 (complex64), 2 (FP64-class)");
  std::lock_guard<std::mutex> lk(ctx->mu);
  ctx->solver = mode;
  return BEMGPU_OK;
}

extern "C" int bemgpu_ctx_set_escalation_tol(bemgpu_ctx_t ctx, double tol) {
  if (!ctx || !(tol >= 0.0)) return bem_fail(ctx, BEMGPU_ERR_ARG, "set_escalation_tol: tol >= 0");
  std::lock_guard<std::mutex> lk(ctx->mu);
  ctx->escalate_tol = tol;
  return BEMGPU_OK;
}

extern "C" int bemgpu_ctx_set_fp64_fallback_tol(bemgpu_ctx_t ctx, double tol) {
  if (!ctx || !(tol >= 0.0)) return bem_fail(ctx, BEMGPU_ERR_ARG, "set_fp64_fallback_tol: tol >= 0");
  std::lock_guard<std::mutex> lk(ctx->mu);
  ctx->fallback_tol = tol;
  return BEMGPU_OK;
}

extern "C" int bemgpu_ctx_set_engines(bemgpu_ctx_t ctx, int gemm, int acc64) {
  if (!ctx || gemm < 0 || gemm > 2 || acc64 < 0 || acc64 > 2)
    return bem_fail(ctx, BEMGPU_ERR_ARG, "set_engines: engines are 0 (choice), 1 (tensor cores), 2 (FMA pipes)");
  std::lock_guard<std::mutex> lk(ctx->mu);
  ctx->gemm_engine = gemm;
  ctx->acc_engine = acc64;
  return BEMGPU_OK;
}
