// Complex128 GEMM on the tensor cores with FP64-class results, for the
// refinement residual R = E - W Y and the trace products H X of the
// mixed-precision solve.
//
//   * realified like gemm_tc.cu: D' = A' B'^T, A' (2m x 2k) rows (Ar, -Ai) /
//     (Ai, Ar), B' (n x 2k) the float view of B's columns; D'(rho, c) is the
//     double at offset rho + 2 ldc c of the complex column-major C.
//   * block fixed point: after one exact power-of-two scaling per matrix
//     (largest magnitude -> below 1), every entry x of a 64-complex block along
//     K (one drain step = four 32-deep TMA stages; the same block for a row of
//     A and a column of B)
//     is written with the block's exponent E (block max < 2^E) as
//       x = sum_{l<SL} q_l 2^(E - 8(l+1)) + r,  |q_0| <= 256, |q_l| <= 128,
//     each q rounded to nearest, |r| <= 2^(E - 8 SL - 1); slice l holds
//     q_l 2^(E - 8(l+1)) as bf16 (exact: at most 9 significant bits).
//   * slice products of level L = a + b share one unit per drain step, and a
//     step's level sum stays below 2^24 units (128 products of |q q| <= 2^16
//     for level 0, 128 x (2^15 + 2^14 + 2^15) for level 2), so
//     the tensor cores sum levels 0..2 EXACTLY into FP32 TMEM buffers
//     (double-buffered by step parity); levels 3..SL-1 (below 2^-24 of level 0)
//     run in FP32 TMEM sums over the whole K.  Products of level >= SL are
//     dropped (below 2^(-8 SL) of the block maxima's product).
//   * eight epilogue warps drain each step while the next runs (three TMEM
//     loads behind one wait per 8 columns): hi + lo += X0
//     and += X1 (TwoSum each: exact), lo += X2 (rounding ~2^-40 of the sum);
//     at the end C = 2^-(sa+sb) (hi + lo + levels
//     3..) [+ C] in FP64.
//   * pipeline: warp 0 TMA (64-byte swizzle, 32-deep K steps, 3 stages),
//     warp 1 tcgen05.mma (M=128, N=64, K=16, bf16 -> FP32) and TMEM
//     allocation, warps 2..9 epilogue.  Every wait is bounded; a wait that
//     runs out sets the error flag and the CTA finishes.
#include "bemgpu_internal.h"

#include "tc_common.cuh"

namespace {

constexpr int EX_BM = 128, EX_BN = 64;  // tile of D'
constexpr int EX_SMEM_MAX = 232448;      // dynamic shared memory of one CTA (227 KB)
constexpr int EX_EPI_WARPS = 8;
constexpr int EX_THREADS = 64 + 32 * EX_EPI_WARPS;
constexpr int EX_TMEM_COLS = 512;  // 2 x levels 0..2 x 64 + levels 3, 4 x 64
constexpr int EX_SCALE_TARGET = 0;  // largest magnitude of a matrix is scaled to below 2^0: slice products
                                    // and their sums stay inside FP32's range
constexpr int EX_FLUSH_E = -80;     // blocks whose maximum (scaled) is below 2^-80 are zero (slices >= 2^-120)

// K step of one TMA stage: 64 bf16 (128-byte rows, 128-byte swizzle) where two
// stages fit in shared memory, else 32 (64-byte rows) in three stages (5 x 5
// slices).  Wider rows move twice the bytes per TMA row request.  A drain
// step is one exponent block: 128 realified K (64 complex).
template <int SA, int SB>
struct ExCfg {
  static constexpr int BK = 2 * (SA * EX_BM + SB * EX_BN) * 64 * 2 + 1280 <= EX_SMEM_MAX ? 64 : 32;
  static constexpr int A_TILE = EX_BM * BK * 2;
  static constexpr int B_TILE = EX_BN * BK * 2;
  static constexpr int STAGE = SA * A_TILE + SB * B_TILE;
  static constexpr int STAGES = (EX_SMEM_MAX - 1280) / STAGE < 3 ? (EX_SMEM_MAX - 1280) / STAGE : 3;
  static constexpr int DRAIN = 128 / BK;
  static constexpr int SMEM = STAGES * STAGE + 1024 + 256;
  static_assert(STAGES >= 2 && SMEM <= EX_SMEM_MAX, "exact gemm: shared memory");
};
template <int SA, int SB>
__host__ __device__ constexpr int ex_smem_bytes() { return ExCfg<SA, SB>::SMEM; }
// K step of the built (SA, SB) kernels, on the host
inline int ex_bk(int SA, int SB) {
  return SA == 5 && SB == 2   ? ExCfg<5, 2>::BK
         : SA == 5 && SB == 3 ? ExCfg<5, 3>::BK
         : SA == 5            ? ExCfg<5, 5>::BK
         : SA == 4            ? ExCfg<4, 4>::BK
                              : ExCfg<3, 3>::BK;
}

// The slice products of an (SA, SB) product: (a, b) with a < SA, b < SB and
// level a + b < SA, in level-major order (a ascending within a level).  SA =
// SB is the truncated square of a plain product; SB < SA multiplies A by an
// operand that its SB slices represent exactly (quantized), so every product
// up to level SA - 1 is kept.
template <int SA, int SB>
struct ExProducts {
  __host__ __device__ static constexpr int count() {
    int c = 0;
    for (int L = 0; L < SA; L++)
      for (int a = 0; a <= L && a < SA; a++)
        if (L - a < SB) c++;
    return c;
  }
  // level of product p (fst: a of product p)
  __host__ __device__ static constexpr int level(int p) {
    int c = 0;
    for (int L = 0; L < SA; L++)
      for (int a = 0; a <= L && a < SA; a++)
        if (L - a < SB) {
          if (c == p) return L;
          c++;
        }
    return 0;
  }
  __host__ __device__ static constexpr int a_of(int p) {
    int c = 0;
    for (int L = 0; L < SA; L++)
      for (int a = 0; a <= L && a < SA; a++)
        if (L - a < SB) {
          if (c == p) return a;
          c++;
        }
    return 0;
  }
  __host__ __device__ static constexpr bool first(int p) { return p == 0 || level(p - 1) != level(p); }
};

struct ExMaps {
  CUtensorMap a[5];
  CUtensorMap b[5];
};

template <int SA, int SB>
__global__ void __launch_bounds__(EX_THREADS, 1)
    ex_gemm_kernel(const __grid_constant__ ExMaps maps, int ktiles, double *__restrict__ C, int64_t ldcf, int mvalid,
                   int nvalid, int accumulate, const int *__restrict__ shifts, int raster, int *err) {
  typedef ExProducts<SA, SB> PR;
  typedef ExCfg<SA, SB> CF;
  constexpr int NP = PR::count();
  constexpr int STAGE = CF::STAGE, EX_STAGES = CF::STAGES, EX_BK = CF::BK, EX_DRAIN = CF::DRAIN;
  constexpr int EX_A_TILE = CF::A_TILE, EX_B_TILE = CF::B_TILE;
  extern __shared__ unsigned char ex_smem_raw[];
  unsigned char *smem = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(ex_smem_raw) + 1023) &
                                                          ~(uintptr_t)1023);
  uint64_t *full = reinterpret_cast<uint64_t *>(smem + EX_STAGES * STAGE);
  uint64_t *empty = full + EX_STAGES;
  uint64_t *accf = empty + EX_STAGES;  // step buffer b written (MMA -> epilogue)
  uint64_t *acce = accf + 2;           // step buffer b drained (epilogue -> MMA)
  uint64_t *fin = acce + 2;            // all MMAs of this CTA complete
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(fin + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int mt, nt;
  grouped_tile(raster, mt, nt);
  const int m0 = mt * EX_BM, n0 = nt * EX_BN;

  if (threadIdx.x == 0) {
    for (int s = 0; s < EX_STAGES; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; b++) {
      mbar_init(&accf[b], 1);
      mbar_init(&acce[b], EX_EPI_WARPS);
    }
    mbar_init(fin, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(EX_TMEM_COLS));
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
        const int s = kt % EX_STAGES, round = kt / EX_STAGES;
        if (kt >= EX_STAGES && !mbar_wait(&empty[s], (round - 1) & 1, err)) break;
        mbar_expect_tx(&full[s], STAGE);
        unsigned char *st = smem + s * STAGE;
#pragma unroll
        for (int a = 0; a < SA; a++) tma_load_2d(st + a * EX_A_TILE, &maps.a[a], kt * EX_BK, m0, &full[s]);
#pragma unroll
        for (int b = 0; b < SB; b++)
          tma_load_2d(st + SA * EX_A_TILE + b * EX_B_TILE, &maps.b[b], kt * EX_BK, n0, &full[s]);
        issued = kt + 1;
      }
      // copies still in flight after an early stop land before the CTA exits
      for (int kt = issued > EX_STAGES ? issued - EX_STAGES : 0; kt < issued; kt++)
        if (!mbar_wait(&full[kt % EX_STAGES], (kt / EX_STAGES) & 1, err)) break;
    }
  } else if (warp == 1) {
    if (lane == 0) {
      constexpr uint32_t idesc = tc_idesc(EX_BM, EX_BN);
      for (int kt = 0; kt < ktiles; kt++) {
        // drain step dt = kt / EX_DRAIN covers EX_DRAIN stages (one exponent block)
        const int s = kt % EX_STAGES, round = kt / EX_STAGES, dt = kt / EX_DRAIN, b = dt & 1, use = dt >> 1;
        const bool opening = kt % EX_DRAIN == 0, closing = kt % EX_DRAIN == EX_DRAIN - 1;
        if (opening && dt >= 2 && !mbar_wait(&acce[b], (use - 1) & 1, err)) break;
        if (!mbar_wait(&full[s], round & 1, err)) break;
        asm volatile("tcgen05.fence::after_thread_sync;");
        // descriptors: one per stage, the tiles and K steps as compile-time
        // offsets added to its address field (which never carries: smem < 256 KB)
        const uint64_t dbase =
            EX_BK == 64 ? smem_desc_sw128(smem_u32(smem + s * STAGE)) : smem_desc_sw64(smem_u32(smem + s * STAGE));
#pragma unroll
        for (int ks = 0; ks < EX_BK / 16; ks++) {
#pragma unroll
          for (int p = 0; p < NP; p++) {
            const int level = PR::level(p), a = PR::a_of(p), bb = level - a;
            const uint64_t da = dbase + (uint64_t)((a * EX_A_TILE + ks * 32) >> 4);
            const uint64_t db = dbase + (uint64_t)((SA * EX_A_TILE + bb * EX_B_TILE + ks * 32) >> 4);
            const bool first = opening && ks == 0 && PR::first(p);
            if (level <= 2)
              tc_mma(tmem + (uint32_t)((3 * b + level) * EX_BN), da, db, idesc, first ? 0u : 1u);
            else
              tc_mma(tmem + (uint32_t)((3 + level) * EX_BN), da, db, idesc, (first && kt == 0) ? 0u : 1u);
          }
        }
        tc_commit(&empty[s]);
        if (closing) tc_commit(&accf[b]);
      }
      tc_commit(fin);
      mbar_wait(fin, 0, err);
    }
  } else {
    const int quarter = warp & 3, group = (warp - 2) >> 2;
    const uint32_t lane_base = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(group * 32);
    float hi[32], lo[32];
#pragma unroll
    for (int j = 0; j < 32; j++) hi[j] = lo[j] = 0.f;
    bool ok = true;
#pragma unroll 1
    for (int dt = 0; dt < ktiles / EX_DRAIN; dt++) {
      const int b = dt & 1, use = dt >> 1;
      int got = 1;
      if (lane == 0) got = mbar_wait(&accf[b], use & 1, err) ? 1 : 0;
      got = __shfl_sync(0xffffffffu, got, 0);
      if (!got) {
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;");
      const uint32_t tx = lane_base + (uint32_t)(3 * b * EX_BN);
#pragma unroll
      for (int h = 0; h < 2; h++) {  // two halves of 16 columns, six loads behind one wait each
        uint32_t x[16], y1[16], y2[16];
#pragma unroll
        for (int q = 0; q < 2; q++) {
          tc_ld8_nowait(tx + 16 * h + 8 * q, x + 8 * q);
          tc_ld8_nowait(tx + EX_BN + 16 * h + 8 * q, y1 + 8 * q);
          tc_ld8_nowait(tx + 2 * EX_BN + 16 * h + 8 * q, y2 + 8 * q);
        }
        tc_wait_ld();
#pragma unroll
        for (int j = 0; j < 16; j++) {
          two_sum_acc(hi[16 * h + j], lo[16 * h + j], __uint_as_float(x[j]));
          two_sum_acc(hi[16 * h + j], lo[16 * h + j], __uint_as_float(y1[j]));
          lo[16 * h + j] += __uint_as_float(y2[j]);
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;");
      __syncwarp();
      if (lane == 0) mbar_arrive(&acce[b]);
    }
    if (ok && SA > 3) {
      int got = 1;
      if (lane == 0) got = mbar_wait(fin, 0, err) ? 1 : 0;
      ok = __shfl_sync(0xffffffffu, got, 0) != 0;
    }
    const int rho = m0 + quarter * 32 + lane;
    const double scale = ldexp(1.0, -(shifts[0] + shifts[1]));
#pragma unroll
    for (int q = 0; q < 4; q++) {
      float z3[8], z4[8];
#pragma unroll
      for (int j = 0; j < 8; j++) z3[j] = z4[j] = 0.f;
      if (ok && SA > 3) {
        asm volatile("tcgen05.fence::after_thread_sync;");
        tc_ld8(lane_base + (uint32_t)(6 * EX_BN) + 8 * q, z3);
        if (SA > 4) tc_ld8(lane_base + (uint32_t)(7 * EX_BN) + 8 * q, z4);
      }
      if (ok && rho < mvalid) {
#pragma unroll
        for (int j = 0; j < 8; j++) {
          const int c = n0 + group * 32 + 8 * q + j;
          if (c < nvalid) {
            double *p = C + rho + ldcf * (int64_t)c;
            const double v =
                scale * (((double)hi[8 * q + j] + (double)lo[8 * q + j]) + ((double)z3[j] + (double)z4[j]));
            *p = accumulate ? *p + v : v;
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(EX_TMEM_COLS));
  }
}

// ---------------- wide tiles: 128 x 128 of D' ----------------
//
// The same exact product with N = 128 MMAs (the tensor rate of M = 128, N =
// 128 against two thirds of it for N = 64).  TMEM holds 4 x 128 columns: the
// exact levels below ZLEV once each (not double-buffered: 768 columns would
// not fit) and one FP32 buffer summing the levels from ZLEV up over the whole
// K.  ZLEV = 3 keeps levels 0..2 exact as ex_gemm_kernel does (the quantized
// 5 x 2 and 5 x 3 products, whose truncation is 2^-40); ZLEV = 2 for the
// plain 4 x 4 and 3 x 3 products, whose truncation (2^-32, 2^-24 of the
// block maxima products) is far above the 2^-40 an FP32 level 2 adds.  Per
// 128-deep exponent block (4 TMA stages of 32-deep K steps, 64-byte rows)
// the MMA thread issues each stage's FP32-summed products (levels ZLEV and up)
// first; at a block's first stage it then waits, level by level, until the
// epilogue has drained that exact level of the previous block (one mbarrier
// per level), so the drain runs under the FP32-summed products and the MMAs
// into levels already drained.  The host takes these tiles for grids of 4
// waves or more (a smaller grid loses more in its last wave than it gains).
// Sixteen epilogue warps (a TMEM lane quarter and 32 columns each) drain the
// exact levels one after the other into their two-float (hi, lo) sums in the
// same order per entry as ex_gemm_kernel (TwoSum X0, TwoSum X1, lo += X2).
// Every wait is bounded.
constexpr int EXW_BN = 128;
constexpr int EXW_BK = 32;
constexpr int EXW_DRAIN = 128 / EXW_BK;  // TMA stages per exponent block
constexpr int EXW_EPI_WARPS = 16;
constexpr int EXW_THREADS = 64 + 32 * EXW_EPI_WARPS;
constexpr int EXW_TMEM_COLS = 512;  // three exact-level buffers and the FP32 sum, 128 columns each
constexpr int EXW_ZCOL = 3 * EXW_BN;

template <int SA, int SB>
struct ExWCfg {
  static constexpr int TILE = EX_BM * EXW_BK * 2;  // one slice tile, A or B (128 rows)
  static constexpr int STAGE = (SA + SB) * TILE;
  static constexpr int STAGES = (EX_SMEM_MAX - 1280) / STAGE < 4 ? (EX_SMEM_MAX - 1280) / STAGE : 4;
  static constexpr int SMEM = STAGES * STAGE + 1024 + 256;
  static_assert(STAGES >= 3 && SMEM <= EX_SMEM_MAX, "exact gemm (wide tiles): shared memory");
};
template <int SA, int SB>
__host__ __device__ constexpr int exw_smem_bytes() { return ExWCfg<SA, SB>::SMEM; }

template <int SA, int SB, int ZLEV>
__global__ void __launch_bounds__(EXW_THREADS, 1)
    ex_gemm_wide_kernel(const __grid_constant__ ExMaps maps, int ktiles, double *__restrict__ C, int64_t ldcf,
                        int mvalid, int nvalid, int accumulate, const int *__restrict__ shifts, int raster, int *err) {
  typedef ExWCfg<SA, SB> CF;
  constexpr int STAGE = CF::STAGE, NST = CF::STAGES, TILE = CF::TILE;
  static_assert(ZLEV >= 2 && ZLEV <= 3 && SA > ZLEV, "wide tiles need FP32-summed levels to hide the drain under");
  extern __shared__ unsigned char ex_smem_raw[];
  unsigned char *smem = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(ex_smem_raw) + 1023) &
                                                          ~(uintptr_t)1023);
  uint64_t *full = reinterpret_cast<uint64_t *>(smem + NST * STAGE);
  uint64_t *empty = full + NST;
  uint64_t *accf = empty + NST;  // a block's levels 0..2 written (MMA -> epilogue)
  uint64_t *accx = accf + 1;     // level L of the last block drained (epilogue -> MMA), L = 0, 1, 2
  uint64_t *fin = accx + 3;      // all MMAs of this CTA complete
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(fin + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int mt, nt;
  grouped_tile(raster, mt, nt);
  const int m0 = mt * EX_BM, n0 = nt * EXW_BN;

  if (threadIdx.x == 0) {
    for (int s = 0; s < NST; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(accf, 1);
    for (int l = 0; l < 3; l++) mbar_init(&accx[l], EXW_EPI_WARPS);
    mbar_init(fin, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(EXW_TMEM_COLS));
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
        const int s = kt % NST, round = kt / NST;
        if (kt >= NST && !mbar_wait(&empty[s], (round - 1) & 1, err)) break;
        mbar_expect_tx(&full[s], STAGE);
        unsigned char *st = smem + s * STAGE;
#pragma unroll
        for (int a = 0; a < SA; a++) tma_load_2d(st + a * TILE, &maps.a[a], kt * EXW_BK, m0, &full[s]);
#pragma unroll
        for (int b = 0; b < SB; b++) tma_load_2d(st + (SA + b) * TILE, &maps.b[b], kt * EXW_BK, n0, &full[s]);
        issued = kt + 1;
      }
      // copies still in flight after an early stop land before the CTA exits
      for (int kt = issued > NST ? issued - NST : 0; kt < issued; kt++)
        if (!mbar_wait(&full[kt % NST], (kt / NST) & 1, err)) break;
    }
  } else if (warp == 1) {
    if (lane == 0) {
      constexpr uint32_t idesc = tc_idesc(EX_BM, EXW_BN);
      bool ok = true, zfirst = true;
      for (int kt = 0; kt < ktiles && ok; kt++) {
        const int s = kt % NST, round = kt / NST, dt = kt / EXW_DRAIN, q = kt % EXW_DRAIN;
        if (!mbar_wait(&full[s], round & 1, err)) break;
        asm volatile("tcgen05.fence::after_thread_sync;");
        const uint64_t dbase = smem_desc_sw64(smem_u32(smem + s * STAGE));
        // levels >= 3: one FP32 sum over the whole K
#pragma unroll
        for (int ks = 0; ks < EXW_BK / 16; ks++)
#pragma unroll
          for (int a = 0; a < SA; a++)
#pragma unroll
            for (int b = 0; b < SB; b++) {
              if (a + b < ZLEV || a + b >= SA) continue;
              const uint64_t da = dbase + (uint64_t)((a * TILE + ks * 32) >> 4);
              const uint64_t db = dbase + (uint64_t)(((SA + b) * TILE + ks * 32) >> 4);
              tc_mma(tmem + (uint32_t)EXW_ZCOL, da, db, idesc, zfirst ? 0u : 1u);
              zfirst = false;
            }
        // levels 0..2: exact per block; at its first stage a level waits until
        // the epilogue has drained it
#pragma unroll
        for (int l = 0; l < ZLEV; l++) {
          if (q == 0 && dt >= 1) {
            if (!mbar_wait(&accx[l], (dt - 1) & 1, err)) {
              ok = false;
              break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;");
          }
          const int amin = l - (SB - 1) > 0 ? l - (SB - 1) : 0;
#pragma unroll
          for (int ks = 0; ks < EXW_BK / 16; ks++)
#pragma unroll
            for (int a = 0; a < SA; a++) {
              const int b = l - a;
              if (a > l || b >= SB) continue;
              const uint64_t da = dbase + (uint64_t)((a * TILE + ks * 32) >> 4);
              const uint64_t db = dbase + (uint64_t)(((SA + b) * TILE + ks * 32) >> 4);
              const bool first = q == 0 && ks == 0 && a == amin;
              tc_mma(tmem + (uint32_t)(l * EXW_BN), da, db, idesc, first ? 0u : 1u);
            }
        }
        if (!ok) break;
        tc_commit(&empty[s]);
        if (q == EXW_DRAIN - 1) tc_commit(accf);
      }
      tc_commit(fin);
      mbar_wait(fin, 0, err);
    }
  } else {
    const int quarter = warp & 3, group = (warp - 2) >> 2;  // TMEM lanes 32 quarter.., columns 32 group..
    const uint32_t lane_base = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(group * 32);
    float hi[32], lo[32];
#pragma unroll
    for (int j = 0; j < 32; j++) hi[j] = lo[j] = 0.f;
    bool ok = true;
#pragma unroll 1
    for (int dt = 0; dt < ktiles / EXW_DRAIN; dt++) {
      int got = 1;
      if (lane == 0) got = mbar_wait(accf, dt & 1, err) ? 1 : 0;
      got = __shfl_sync(0xffffffffu, got, 0);
      if (!got) {
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;");
#pragma unroll
      for (int l = 0; l < ZLEV; l++) {
#pragma unroll
        for (int c = 0; c < 4; c++) {  // 8 columns per load batch
          uint32_t v[8];
          tc_ld8_nowait(lane_base + (uint32_t)(l * EXW_BN + 8 * c), v);
          tc_wait_ld();
#pragma unroll
          for (int j = 0; j < 8; j++) {
            if (l < 2)
              two_sum_acc(hi[8 * c + j], lo[8 * c + j], __uint_as_float(v[j]));
            else
              lo[8 * c + j] += __uint_as_float(v[j]);
          }
        }
        asm volatile("tcgen05.fence::before_thread_sync;");
        __syncwarp();
        if (lane == 0) mbar_arrive(&accx[l]);
      }
    }
    if (ok) {
      int got = 1;
      if (lane == 0) got = mbar_wait(fin, 0, err) ? 1 : 0;
      ok = __shfl_sync(0xffffffffu, got, 0) != 0;
    }
    const int rho = m0 + quarter * 32 + lane;
    const double scale = ldexp(1.0, -(shifts[0] + shifts[1]));
    if (ok) asm volatile("tcgen05.fence::after_thread_sync;");
#pragma unroll
    for (int c = 0; c < 4; c++) {
      float z[8];
#pragma unroll
      for (int j = 0; j < 8; j++) z[j] = 0.f;
      if (ok) tc_ld8(lane_base + (uint32_t)(EXW_ZCOL + 8 * c), z);
      if (ok && rho < mvalid) {
#pragma unroll
        for (int j = 0; j < 8; j++) {
          const int col = n0 + group * 32 + 8 * c + j;
          if (col < nvalid) {
            double *p = C + rho + ldcf * (int64_t)col;
            const double v = scale * (((double)hi[8 * c + j] + (double)lo[8 * c + j]) + (double)z[j]);
            *p = accumulate ? *p + v : v;
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(EXW_TMEM_COLS));
  }
}

}  // namespace

namespace {

// Largest FP64 exponent field of max(|re|, |im|) over a complex128 matrix
// (m x k, column-major) -> *out (atomicMax).
__global__ void ex_absmax_kernel(const double *__restrict__ A, int64_t lda, int m, int k, unsigned *out) {
  unsigned mx = 0;
  const int64_t total = (int64_t)m * k;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = i / m, r = i - c * m;
    const longlong2 v = reinterpret_cast<const longlong2 *>(A)[r + lda * c];
    mx = max(mx, (unsigned)max((v.x >> 52) & 0x7ff, (v.y >> 52) & 0x7ff));
  }
  mx = __reduce_max_sync(0xffffffffu, mx);
  if ((threadIdx.x & 31) == 0 && mx > 0) atomicMax(out, mx);
}

// Scaling exponent g of the matrix whose largest exponent field is *amax:
// values times 2^g stay below 2^EX_SCALE_TARGET (0 for a zero matrix).
__device__ __forceinline__ int ex_matrix_shift(const unsigned *amax) {
  const int eb = (int)*amax;  // largest magnitude in [2^(eb-1023), 2^(eb-1022))
  return eb == 0 ? 0 : EX_SCALE_TARGET - (eb - 1022);
}

constexpr int EX_ZERO = -100000;

__device__ __forceinline__ int fp64_expfield(double x) { return (int)((__double_as_longlong(x) >> 52) & 0x7ff); }
__device__ __forceinline__ float pow2f(int e) { return __int_as_float((127 + e) << 23); }  // e in [-126, 127]

// Block fixed point by integer arithmetic on the FP64 fields: with x 2^g = M
// 2^(eb + g - 1075) and the block exponent E, N = round(x 2^(g + 8 SL - E))
// (|N| <= 2^(8 SL)), written in balanced base-256 digits q_0..q_{SL-1}
// (|q_0| <= 256, |q_l| <= 128); slice l holds q_l 2^(E - 8(l+1)) as bf16
// (exact: at most 8 significant bits).  FP64 subnormals count as zero.
template <int SL>
__device__ __forceinline__ void ex_split(double x, int g, int E, __nv_bfloat16 *s) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
  const int eb = (int)((bits >> 52) & 0x7ff);
  long long N = 0;
  if (E != EX_ZERO && eb != 0) {
    const long long mant = (long long)((bits & ((1ull << 52) - 1)) | (1ull << 52));
    const int rs = -(eb + g - 1075 + 8 * SL - E);  // >= 13 since |x 2^g| < 2^E
    if (rs < 55) N = (mant + (1ll << (rs - 1))) >> rs;
    if (bits >> 63) N = -N;
  }
  int q[SL];
#pragma unroll
  for (int l = SL - 1; l >= 1; l--) {
    int d = (int)(N & 255);
    if (d >= 128) d -= 256;
    q[l] = d;
    N = (N - d) >> 8;
  }
  q[0] = (int)N;
#pragma unroll
  for (int l = 0; l < SL; l++)
    s[l] = __float2bfloat16_rn(E == EX_ZERO ? 0.f : (float)q[l] * pow2f(E - 8 * (l + 1)));
}

// Maximum over the 64 consecutive threads (two warps) holding one exponent
// block; the CTA is 128 threads and every thread calls it.
__device__ __forceinline__ unsigned block64_max(unsigned v) {
  __shared__ unsigned wm[4];
  v = __reduce_max_sync(0xffffffffu, v);
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) wm[w] = v;
  __syncthreads();
  return max(wm[w & ~1], wm[w | 1]);
}

// Block exponent E (block max of x 2^g below 2^E) from the block's largest
// exponent field; flush marker for zero blocks and blocks below 2^EX_FLUSH_E.
__device__ __forceinline__ int ex_block_exponent(unsigned ebmax, int g) {
  const int E = (int)ebmax + g - 1022;
  return (ebmax == 0 || E < EX_FLUSH_E) ? EX_ZERO : E;
}

// A' slices (Mp x Kp) of sign * A (complex128, m x k, column-major), block
// fixed point over 64-complex blocks of each row (two warps, one drain step).  Thread
// (r, q): complex row r, complex column q (q fast).  Also records the
// matrix's scaling exponent in *shift.
template <int SL>
__global__ void ex_prep_a_kernel(const double *__restrict__ A, int64_t lda, int m, int k, double sign,
                                 const unsigned *amax, int *shift, __nv_bfloat16 *__restrict__ S, int64_t Mp,
                                 int64_t Kp) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  const int r = blockIdx.y;
  const bool active = 2 * q < Kp;
  const int g = ex_matrix_shift(amax);
  if (q == 0 && r == 0) *shift = g;
  double ar = 0.0, ai = 0.0;
  if (active && r < m && q < k) {
    const double2 v = reinterpret_cast<const double2 *>(A)[r + lda * (int64_t)q];
    ar = sign * v.x;
    ai = sign * v.y;
  }
  const int E = ex_block_exponent(block64_max((unsigned)max(fp64_expfield(ar), fp64_expfield(ai))), g);
  if (!active) return;
  __nv_bfloat16 sr[SL], si[SL], sn[SL];
  ex_split<SL>(ar, g, E, sr);
  ex_split<SL>(ai, g, E, si);
#pragma unroll
  for (int l = 0; l < SL; l++) sn[l] = __hneg(si[l]);
  const int64_t plane = Mp * Kp;
  const int64_t i0 = (int64_t)(2 * r) * Kp + 2 * q, i1 = i0 + Kp;
#pragma unroll
  for (int l = 0; l < SL; l++) {
    reinterpret_cast<__nv_bfloat162 *>(S + l * plane + i0)[0] = __halves2bfloat162(sr[l], sn[l]);  // (Ar, -Ai)
    reinterpret_cast<__nv_bfloat162 *>(S + l * plane + i1)[0] = __halves2bfloat162(si[l], sr[l]);  // (Ai, Ar)
  }
}

// B' slices (Np x Kp): row c = column c of complex128 B (k x n); blocks of 64
// complex rows (two warps).
// Bq: when given, B itself is replaced by the value its slices represent
// exactly (quantized to the block fixed point), so that a product with it can
// keep every slice level of the other operand.
template <int SL>
__global__ void ex_prep_b_kernel(const double *__restrict__ B, int64_t ldb, int k, int n,
                                 const unsigned *amax, int *shift, __nv_bfloat16 *__restrict__ S, int64_t Np,
                                 int64_t Kp, double *Bq) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  const int c = blockIdx.y;
  const bool active = 2 * q < Kp;
  const int g = ex_matrix_shift(amax);
  if (q == 0 && c == 0) *shift = g;
  double br = 0.0, bi = 0.0;
  if (active && c < n && q < k) {
    const double2 v = reinterpret_cast<const double2 *>(B)[q + ldb * (int64_t)c];
    br = v.x;
    bi = v.y;
  }
  const int E = ex_block_exponent(block64_max((unsigned)max(fp64_expfield(br), fp64_expfield(bi))), g);
  if (!active) return;
  __nv_bfloat16 sr[SL], si[SL];
  ex_split<SL>(br, g, E, sr);
  ex_split<SL>(bi, g, E, si);
  const int64_t plane = Np * Kp, i0 = (int64_t)c * Kp + 2 * q;
#pragma unroll
  for (int l = 0; l < SL; l++)
    reinterpret_cast<__nv_bfloat162 *>(S + l * plane + i0)[0] = __halves2bfloat162(sr[l], si[l]);
  if (Bq && c < n && q < k) {
    double qr = 0.0, qi = 0.0;  // exact: at most 8 SL + 1 significant bits
#pragma unroll
    for (int l = 0; l < SL; l++) {
      qr += (double)__bfloat162float(sr[l]);
      qi += (double)__bfloat162float(si[l]);
    }
    reinterpret_cast<double2 *>(Bq)[q + ldb * (int64_t)c] = make_double2(ldexp(qr, -g), ldexp(qi, -g));
  }
}

bool ex_maps(CUtensorMap *maps, const __nv_bfloat16 *S, int slices, int64_t rows, int64_t kp, int box_rows,
             int bk) {
  for (int l = 0; l < slices; l++)
    if (!make_map_bf16(&maps[l], S + l * rows * kp, rows, kp, bk, box_rows,
                       bk == 64 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B))
      return false;
  return true;
}

}  // namespace

// ---------------------------------------------------------------- host side

bool bem_exact_available() { return encode_fn() != nullptr; }

size_t bem_exact_operand_bytes(bool is_a, int rows, int k, int slices) {
  const int64_t rp = is_a ? ((2 * (int64_t)rows + EX_BM - 1) / EX_BM) * EX_BM
                          : (((int64_t)rows + EXW_BN - 1) / EXW_BN) * EXW_BN;
  const int64_t kp = ((2 * (int64_t)k + 127) / 128) * 128;
  return sizeof(__nv_bfloat16) * (size_t)slices * rp * kp + 64;
}

int bem_exact_prep(bemgpu_ctx_s *ctx, const char *name, bool is_a, const double *M, int64_t ld, int rows, int k,
                   double sign, int slices, ExactOperand &op, cudaStream_t st, double *quantize) {
  // 2 slices only for a quantized B operand (the 5 x 2 product)
  if (slices < (quantize ? 2 : 3) || slices > 5) return bem_fail(ctx, BEMGPU_ERR_ARG, "exact gemm: %d slices", slices);
  if (rows <= 0 || k <= 0) return bem_fail(ctx, BEMGPU_ERR_ARG, "exact gemm: empty operand");
  // B rows padded to the wide tile (a multiple of the narrow one)
  const int64_t rp = is_a ? ((2 * (int64_t)rows + EX_BM - 1) / EX_BM) * EX_BM
                          : (((int64_t)rows + EXW_BN - 1) / EXW_BN) * EXW_BN;
  const int64_t kp = ((2 * (int64_t)k + 127) / 128) * 128;  // whole exponent blocks (drain steps)
  if ((is_a ? rp / 2 : rp) > 65535) return bem_fail(ctx, BEMGPU_ERR_ARG, "exact gemm: %d rows too many", rows);
  const std::string base = std::string("ex_") + name;
  op.S = bem_workspace(ctx, base, sizeof(__nv_bfloat16) * (size_t)slices * rp * kp);
  op.aux = (int *)bem_workspace(ctx, base + "_aux", 64);
  if (!op.S || !op.aux) return bem_fail(ctx, BEMGPU_ERR_OOM, "exact gemm: workspace");
  op.rows = rows;
  op.k = k;
  op.rows_p = rp;
  op.kp = kp;
  op.slices = slices;
  op.is_a = is_a;
  op.exact = quantize != nullptr;
  if (quantize && (is_a || quantize != M || sign != 1.0))
    return bem_fail(ctx, BEMGPU_ERR_ARG, "exact gemm: only a B operand is quantized, in place, unscaled");
  unsigned *amax = reinterpret_cast<unsigned *>(op.aux + 8);
  {
    ProfScope ps(ctx, BEMGPU_K_SLICE, st, 0.0, 16.0 * (double)rows * k * 2 + 4.0 * slices * (double)rp * kp);
    BEM_CUDA_TRY(ctx, cudaMemsetAsync(amax, 0, sizeof(unsigned), st));
    ex_absmax_kernel<<<2 * 152, 256, 0, st>>>(M, ld, is_a ? rows : k, is_a ? k : rows, amax);
    ctx->launches++;
    const dim3 grid((unsigned)((kp / 2 + 127) / 128), (unsigned)(is_a ? rp / 2 : rp));
    __nv_bfloat16 *S = (__nv_bfloat16 *)op.S;
    if (is_a) {
      if (slices == 5)
        ex_prep_a_kernel<5><<<grid, 128, 0, st>>>(M, ld, rows, k, sign, amax, op.aux, S, rp, kp);
      else if (slices == 4)
        ex_prep_a_kernel<4><<<grid, 128, 0, st>>>(M, ld, rows, k, sign, amax, op.aux, S, rp, kp);
      else
        ex_prep_a_kernel<3><<<grid, 128, 0, st>>>(M, ld, rows, k, sign, amax, op.aux, S, rp, kp);
    } else {
      if (slices == 5)
        ex_prep_b_kernel<5><<<grid, 128, 0, st>>>(M, ld, k, rows, amax, op.aux, S, rp, kp, quantize);
      else if (slices == 4)
        ex_prep_b_kernel<4><<<grid, 128, 0, st>>>(M, ld, k, rows, amax, op.aux, S, rp, kp, quantize);
      else if (slices == 3)
        ex_prep_b_kernel<3><<<grid, 128, 0, st>>>(M, ld, k, rows, amax, op.aux, S, rp, kp, quantize);
      else
        ex_prep_b_kernel<2><<<grid, 128, 0, st>>>(M, ld, k, rows, amax, op.aux, S, rp, kp, quantize);
    }
    ctx->launches++;
  }
  BEM_CUDA_TRY(ctx, cudaGetLastError());
  return BEMGPU_OK;
}

int bem_exact_gemm(bemgpu_ctx_s *ctx, int kind, const ExactOperand &a, const ExactOperand &b, double *C, int64_t ldc,
                   int accumulate, cudaStream_t st) {
  // A plain B: SB = SA = the slices of B (A may carry more; its leading ones
  // are used), products of levels < SB, error ~2^(-8 SB) of the blocks'
  // maxima.  A quantized B (exactly its SB slices): SA = the slices of A,
  // every product of level < SA kept.
  if (!a.is_a || b.is_a || a.k != b.k || a.kp != b.kp || a.slices < b.slices)
    return bem_fail(ctx, BEMGPU_ERR_ARG, "exact gemm: operands do not match");
  const int m = a.rows, n = b.rows, SB = b.slices, SA = b.exact ? a.slices : b.slices;
  if (!((SA == SB && SA >= 3 && SA <= 5) || (SA == 5 && (SB == 3 || SB == 2))))
    return bem_fail(ctx, BEMGPU_ERR_ARG, "exact gemm: slices (%d, %d) not built", SA, SB);
  const int SL = SB;
  // 128 x 128 tiles where level-3/4 products hide the single-buffered drain,
  // for grids of at least 4 waves (a smaller grid leaves more of its last
  // wave's SMs idle with half as many tiles; ex_gemm_wide_kernel<5, 2> at
  // 240 tiles took 342 us against 312 for 450 narrow ones); BEMGPU_TUNE_EX_WIDE
  // 2 takes them whatever the grid
  const int64_t wtiles = (a.rows_p / EX_BM) * ((b.rows_p + EXW_BN - 1) / EXW_BN);
  const bool wide = ((SA == 5 && (SB == 2 || SB == 3)) || (SA == SB && (SA == 4 || SA == 3))) &&
                    (ctx->tune.ex_wide == 2 || (ctx->tune.ex_wide == 1 && wtiles >= 4 * (int64_t)ctx->num_sms));
  const int bn = wide ? EXW_BN : EX_BN;
  ExMaps maps;
  const int bk = wide ? EXW_BK : ex_bk(SA, SB);
  if (!ex_maps(maps.a, (const __nv_bfloat16 *)a.S, SA, a.rows_p, a.kp, EX_BM, bk) ||
      !ex_maps(maps.b, (const __nv_bfloat16 *)b.S, SB, b.rows_p, b.kp, bn, bk))
    return bem_fail(ctx, BEMGPU_ERR_CUDA, "exact gemm: tensor map encoding failed");
  int *err = (int *)bem_workspace(ctx, "tc_err", sizeof(int));
  if (!err) return bem_fail(ctx, BEMGPU_ERR_OOM, "exact gemm: workspace");
  if (!ctx->ex_ready) {
    BEM_CUDA_TRY(ctx, cudaFuncSetAttribute(ex_gemm_kernel<5, 5>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           ex_smem_bytes<5, 5>()));
    BEM_CUDA_TRY(ctx, cudaFuncSetAttribute(ex_gemm_kernel<4, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           ex_smem_bytes<4, 4>()));
    BEM_CUDA_TRY(ctx, cudaFuncSetAttribute(ex_gemm_kernel<3, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           ex_smem_bytes<3, 3>()));
    BEM_CUDA_TRY(ctx, cudaFuncSetAttribute(ex_gemm_kernel<5, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           ex_smem_bytes<5, 3>()));
    BEM_CUDA_TRY(ctx, cudaFuncSetAttribute(ex_gemm_kernel<5, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           ex_smem_bytes<5, 2>()));
    BEM_CUDA_TRY(ctx, cudaFuncSetAttribute(ex_gemm_wide_kernel<5, 2, 3>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, exw_smem_bytes<5, 2>()));
    BEM_CUDA_TRY(ctx, cudaFuncSetAttribute(ex_gemm_wide_kernel<5, 3, 3>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, exw_smem_bytes<5, 3>()));
    BEM_CUDA_TRY(ctx, cudaFuncSetAttribute(ex_gemm_wide_kernel<4, 4, 2>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, exw_smem_bytes<4, 4>()));
    BEM_CUDA_TRY(ctx, cudaFuncSetAttribute(ex_gemm_wide_kernel<3, 3, 2>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, exw_smem_bytes<3, 3>()));
    ctx->ex_ready = true;
  }
  if (!ctx->tc_err_ready) {
    BEM_CUDA_TRY(ctx, cudaMemsetAsync(err, 0, sizeof(int), st));
    ctx->tc_err_ready = true;
  }
  // shifts of A and B side by side for the kernel
  int *shifts = (int *)bem_workspace(ctx, "ex_shifts", 2 * sizeof(int));
  if (!shifts) return bem_fail(ctx, BEMGPU_ERR_OOM, "exact gemm: workspace");
  BEM_CUDA_TRY(ctx, cudaMemcpyAsync(shifts, a.aux, sizeof(int), cudaMemcpyDeviceToDevice, st));
  BEM_CUDA_TRY(ctx, cudaMemcpyAsync(shifts + 1, b.aux, sizeof(int), cudaMemcpyDeviceToDevice, st));
  ProfScope ps(ctx, kind, st, 8.0 * m * (double)n * a.k,
               2.0 * SA * ((double)a.rows_p * a.kp * ((b.rows_p + bn - 1) / bn) / 8.0) +
                   2.0 * SB * (double)b.rows_p * b.kp + 16.0 * m * (double)n * (accumulate ? 2 : 1));
  (void)SL;
  {
    // slice products (a, b) with a < SA, b < SB, a + b < SA
    int products = 0;
    for (int i = 0; i < SA; i++)
      for (int j = 0; j < SB; j++) products += (i + j < SA);
    ps.tensor = products * ps.flops;
  }
  const dim3 grid((unsigned)(a.rows_p / EX_BM), (unsigned)(b.rows_p / bn));
  const int ktiles = (int)(a.kp / bk);
  if (wide && SA == 5 && SB == 2)
    ex_gemm_wide_kernel<5, 2, 3><<<grid, EXW_THREADS, exw_smem_bytes<5, 2>(), st>>>(
        maps, ktiles, C, 2 * ldc, 2 * m, n, accumulate, shifts, ctx->tune.raster, err);
  else if (wide && SA == 5 && SB == 3)
    ex_gemm_wide_kernel<5, 3, 3><<<grid, EXW_THREADS, exw_smem_bytes<5, 3>(), st>>>(
        maps, ktiles, C, 2 * ldc, 2 * m, n, accumulate, shifts, ctx->tune.raster, err);
  else if (wide && SA == 4)
    ex_gemm_wide_kernel<4, 4, 2><<<grid, EXW_THREADS, exw_smem_bytes<4, 4>(), st>>>(
        maps, ktiles, C, 2 * ldc, 2 * m, n, accumulate, shifts, ctx->tune.raster, err);
  else if (wide)
    ex_gemm_wide_kernel<3, 3, 2><<<grid, EXW_THREADS, exw_smem_bytes<3, 3>(), st>>>(
        maps, ktiles, C, 2 * ldc, 2 * m, n, accumulate, shifts, ctx->tune.raster, err);
  else if (SA == 5 && SB == 2)
    ex_gemm_kernel<5, 2><<<grid, EX_THREADS, ex_smem_bytes<5, 2>(), st>>>(maps, ktiles, C, 2 * ldc, 2 * m, n,
                                                                          accumulate, shifts, ctx->tune.raster, err);
  else if (SA == 5 && SB == 3)
    ex_gemm_kernel<5, 3><<<grid, EX_THREADS, ex_smem_bytes<5, 3>(), st>>>(maps, ktiles, C, 2 * ldc, 2 * m, n,
                                                                          accumulate, shifts, ctx->tune.raster, err);
  else if (SA == 5)
    ex_gemm_kernel<5, 5><<<grid, EX_THREADS, ex_smem_bytes<5, 5>(), st>>>(maps, ktiles, C, 2 * ldc, 2 * m, n,
                                                                          accumulate, shifts, ctx->tune.raster, err);
  else if (SA == 4)
    ex_gemm_kernel<4, 4><<<grid, EX_THREADS, ex_smem_bytes<4, 4>(), st>>>(maps, ktiles, C, 2 * ldc, 2 * m, n,
                                                                          accumulate, shifts, ctx->tune.raster, err);
  else
    ex_gemm_kernel<3, 3><<<grid, EX_THREADS, ex_smem_bytes<3, 3>(), st>>>(maps, ktiles, C, 2 * ldc, 2 * m, n,
                                                                          accumulate, shifts, ctx->tune.raster, err);
  ctx->launches++;
  BEM_CUDA_TRY(ctx, cudaGetLastError());
  return BEMGPU_OK;
}

extern "C" int bemgpu_zgemm_exact(bemgpu_ctx_t ctx, int m, int n, int k, const double *dA, int64_t lda,
                                  const double *dB, int64_t ldb, double *dC, int64_t ldc, int accumulate, int slices) {
  if (!ctx || !dA || !dB || !dC || m < 1 || n < 1 || k < 1 || lda < m || ldb < k || ldc < m)
    return bem_fail(ctx, BEMGPU_ERR_ARG, "zgemm_exact: bad arguments");
  std::lock_guard<std::mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  if (!bem_exact_available()) return bem_fail(ctx, BEMGPU_ERR_CUDA, "zgemm_exact: tensor maps unavailable");
  ExactOperand a, b;
  int rc = bem_exact_prep(ctx, "cabi_a", true, dA, lda, m, k, 1.0, slices, a, ctx->stream);
  if (!rc) rc = bem_exact_prep(ctx, "cabi_b", false, dB, ldb, n, k, 1.0, slices, b, ctx->stream);
  if (!rc) rc = bem_exact_gemm(ctx, BEMGPU_K_TRACE, a, b, dC, ldc, accumulate, ctx->stream);
  if (rc) return rc;
  BEM_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  if (bem_tc_error(ctx, true)) return bem_fail(ctx, BEMGPU_ERR_TIMEOUT, "zgemm_exact: a pipeline wait ran out");
  return BEMGPU_OK;
}

extern "C" int bemgpu_zgemm_exact_quantized(bemgpu_ctx_t ctx, int m, int n, int k, const double *dA, int64_t lda,
                                            double *dB, int64_t ldb, double *dC, int64_t ldc, int accumulate) {
  if (!ctx || !dA || !dB || !dC || m < 1 || n < 1 || k < 1 || lda < m || ldb < k || ldc < m)
    return bem_fail(ctx, BEMGPU_ERR_ARG, "zgemm_exact_quantized: bad arguments");
  std::lock_guard<std::mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  if (!bem_exact_available()) return bem_fail(ctx, BEMGPU_ERR_CUDA, "zgemm_exact_quantized: tensor maps unavailable");
  ExactOperand a, b;
  int rc = bem_exact_prep(ctx, "cabi_a", true, dA, lda, m, k, 1.0, 5, a, ctx->stream);
  if (!rc) rc = bem_exact_prep(ctx, "cabi_b", false, dB, ldb, n, k, 1.0, 3, b, ctx->stream, dB);
  if (!rc) rc = bem_exact_gemm(ctx, BEMGPU_K_TRACE, a, b, dC, ldc, accumulate, ctx->stream);
  if (rc) return rc;
  BEM_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  if (bem_tc_error(ctx, true))
    return bem_fail(ctx, BEMGPU_ERR_TIMEOUT, "zgemm_exact_quantized: a pipeline wait ran out");
  return BEMGPU_OK;
}
