// PMCHWT RWG impedance fill on the GPU: Zts (src/Impedance.cpp:276-413).
//
// Work decomposition
//   * far pairs (no shared vertex): one thread per (test, source) triangle
//     pair over a 2-D grid, FP64 (plain path).  The reference contracts the
//     inner integrals per half-RWG (Gphi[j], DGxphi[j], src/Impedance.cpp:126-167);
//     here the inner loop accumulates four j-independent moments
//        I0 = sum w g,  A = sum w g (r_s - P_s),  Q0 = sum w q,  Q1 = sum w q (r_s - P_s)
//     (g, q of GreensFunction::scalar_gradient, gradient = q (r_t - r_s)), and the
//     outer loop eight moments U0..U3, V0..V3, from which all nine (i, j)
//     products L_ij, K_ij follow in closed form (derivation beside far_pair()).
//   * near pairs (same triangle or a shared vertex): one warp per pair, lanes over
//     the 105 outer nodes, each lane runs the 91-node smooth inner rule, the
//     analytic singular terms (EHNonSmoothIntegral, src/Source.cpp:16-86) and the
//     close-pair contraction of src/Impedance.cpp:194-250 in FP64; the
//     neighbour-edge K correction (src/Impedance.cpp:301-324) runs on the same warp.
//   * every pair writes its nine (c L_ij, c K_ij) half-pair products into a
//     half-pair block array H (one 128-byte block per RWG pair (i, j), four
//     slots for (pos/neg test half) x (pos/neg source half)); each slot has
//     exactly one writer, so no atomics are needed.  A gather kernel then
//     reduces each block into the 2x2 (J, M) entries of Z in RWG-pair order with
//     coalesced stores (src/Impedance.cpp:365-384).
#include "bemgpu_internal.h"
#include "quadrature_tables.h"
#include "df64.cuh"

#include <cmath>
#include <vector>

namespace {

struct GreenDev {
  double ikr, iki;      // ik
  double k2r, k2i;      // k2 = -ksquared/2
  double ksqr, ksqi;    // ksquared
  // the same as double-float pairs (hi, lo), split on the host
  float ikr_f[2], iki_f[2], k2r_f[2], k2i_f[2], ksqr_f[2], ksqi_f[2];
};

struct FarOpts {
  double th6, th10, th15, th21;
};

// Fill arithmetic: FP64 (parity path), FP32 far pairs beyond 3 edge lengths,
// or double-float for every quadrature node pair.
enum { FILL_FP64 = 0, FILL_FP32_FAR = 1, FILL_DF = 2 };

__constant__ double c_rule6[6][3];
__constant__ double c_rule10[10][3];
__constant__ double c_rule15[15][3];
__constant__ double c_rule21[21][3];
__constant__ double c_rule36[36][3];
__constant__ double c_rule91[91][3];
__constant__ double c_rule105[105][3];
__constant__ double c_line15[15][2];
// The triangle rules as double-float (xi1, xi2, w) -> (hi, lo) x 3, for the df fill.
__constant__ float c_rdf6[6][6];
__constant__ float c_rdf10[10][6];
__constant__ float c_rdf15[15][6];
__constant__ float c_rdf21[21][6];
__constant__ float c_rdf36[36][6];
__constant__ float c_rdf91[91][6];

// ---------------- small FP64 vector / complex helpers ----------------
struct d3 {
  double x, y, z;
};
struct z1 {
  double r, i;
};
struct z3 {
  z1 x, y, z;
};

__device__ __forceinline__ d3 ld3(const double *p) { return {p[0], p[1], p[2]}; }
__device__ __forceinline__ d3 operator+(d3 a, d3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ d3 operator-(d3 a, d3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ d3 operator*(double c, d3 a) { return {c * a.x, c * a.y, c * a.z}; }
__device__ __forceinline__ double dot(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ d3 cross(d3 a, d3 b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ z1 zmul(z1 a, z1 b) { return {a.r * b.r - a.i * b.i, a.r * b.i + a.i * b.r}; }
__device__ __forceinline__ z1 zadd(z1 a, z1 b) { return {a.r + b.r, a.i + b.i}; }
__device__ __forceinline__ z1 zsub(z1 a, z1 b) { return {a.r - b.r, a.i - b.i}; }
__device__ __forceinline__ z1 zscale(double c, z1 a) { return {c * a.r, c * a.i}; }
__device__ __forceinline__ z3 z3zero() { return {{0, 0}, {0, 0}, {0, 0}}; }
// complex scalar times real vector
__device__ __forceinline__ z3 zs_v(z1 c, d3 v) { return {{c.r * v.x, c.i * v.x}, {c.r * v.y, c.i * v.y}, {c.r * v.z, c.i * v.z}}; }
__device__ __forceinline__ z3 z3add(z3 a, z3 b) { return {zadd(a.x, b.x), zadd(a.y, b.y), zadd(a.z, b.z)}; }
__device__ __forceinline__ z3 z3sub(z3 a, z3 b) { return {zsub(a.x, b.x), zsub(a.y, b.y), zsub(a.z, b.z)}; }
__device__ __forceinline__ z3 z3add_r(z3 a, d3 b) { return {{a.x.r + b.x, a.x.i}, {a.y.r + b.y, a.y.i}, {a.z.r + b.z, a.z.i}}; }
__device__ __forceinline__ z3 z3scale(double c, z3 a) { return {zscale(c, a.x), zscale(c, a.y), zscale(c, a.z)}; }
// dot(real, complex) — no conjugation (ComplexVector3.h:124-126)
__device__ __forceinline__ z1 rdot(d3 a, z3 b) {
  return {a.x * b.x.r + a.y * b.y.r + a.z * b.z.r, a.x * b.x.i + a.y * b.y.i + a.z * b.z.i};
}
// complex x real cross product
__device__ __forceinline__ z3 zcross(z3 a, d3 b) {
  return {{a.y.r * b.z - a.z.r * b.y, a.y.i * b.z - a.z.i * b.y},
          {a.z.r * b.x - a.x.r * b.z, a.z.i * b.x - a.x.i * b.z},
          {a.x.r * b.y - a.y.r * b.x, a.x.i * b.y - a.y.i * b.x}};
}
// real x complex cross product
__device__ __forceinline__ z3 rcross(d3 a, z3 b) {
  return {{a.y * b.z.r - a.z * b.y.r, a.y * b.z.i - a.z * b.y.i},
          {a.z * b.x.r - a.x * b.z.r, a.z * b.x.i - a.x * b.z.i},
          {a.x * b.y.r - a.y * b.x.r, a.x * b.y.i - a.y * b.x.i}};
}
__device__ __forceinline__ void zacc(z1 &a, z1 b) { a.r += b.r; a.i += b.i; }

// exp(ikR) for real R: exp(Re(ik) R) * (cos(Im(ik) R), sin(Im(ik) R)).  A
// lossless medium (real k: the exterior fill) skips the exp, whose value is 1.
__device__ __forceinline__ z1 zexp_ikR(const GreenDev &g, double R) {
  double s, c;
  sincos(g.iki * R, &s, &c);
  if (g.ikr == 0.0) return {c, s};
  const double m = exp(g.ikr * R);
  return {m * c, m * s};
}

__device__ __forceinline__ int shares_vertex(const int *a, const int *b) {
  int c = 0;
#pragma unroll
  for (int i = 0; i < 3; i++) c += (a[i] == b[0]) | (a[i] == b[1]) | (a[i] == b[2]);
  return c;
}

// IEEE-exact squared distance without contraction (the far-rule test compares
// it with emax^2, src/Impedance.cpp:329-336).
__device__ __forceinline__ double dist2_rn(const double *a, const double *b) {
  double x = __dsub_rn(a[0], b[0]), y = __dsub_rn(a[1], b[1]), z = __dsub_rn(a[2], b[2]);
  return __dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z));
}

__device__ __forceinline__ void store_block(HalfPairBlock *H, int ntr, int i, int a, int j, int b, z1 cL, z1 cK) {
  double2 *p = reinterpret_cast<double2 *>(&H[(size_t)j * ntr + i].v[(a * 2 + b) * 4]);
  p[0] = make_double2(cL.r, cL.i);
  p[1] = make_double2(cK.r, cK.i);
}

// Double-float fill: the block holds each value as a float pair (hi, lo) in
// its 8-byte slot; the gather widens hi + lo (exact in FP64).
__device__ __forceinline__ void store_block_df(HalfPairBlock *H, int ntr, int i, int a, int j, int b, df Lr, df Li,
                                               df Kr, df Ki) {
  float4 *p = reinterpret_cast<float4 *>(&H[(size_t)j * ntr + i].v[(a * 2 + b) * 4]);
  p[0] = make_float4(Lr.hi, Lr.lo, Li.hi, Li.lo);
  p[1] = make_float4(Kr.hi, Kr.lo, Ki.hi, Ki.lo);
}

// Scatter coefficient of src/Impedance.cpp:372-375.
__device__ __forceinline__ double scatter_coef(const TriRec &T, int i, const TriRec &S, int j) {
  double c = BEM_ONEOVER4PI * T.helen[i] * S.helen[j];
  return (T.hneg[i] != S.hneg[j]) ? -c : c;
}

// The nine (c L_ij, c K_ij) of a far pair from its outer moments (closed form
// beside far_pair()).
__device__ __forceinline__ void far_contract(const TriRec &T, const TriRec &S, const GreenDev &g, z1 U0, z1 U1, z3 U2,
                                             z3 U3, z1 V0, z3 V1, z3 V2, z3 V3, HalfPairBlock *H, int ntr) {
  const d3 Pt = ld3(T.p0), Ps = ld3(S.p0);
  const z1 ksq = {g.ksqr, g.ksqi};
  for (int i = 0; i < T.nh; i++) {
    const d3 p0i = ld3(T.hp0[i]);
    const d3 ei = p0i - Pt;
    for (int j = 0; j < S.nh; j++) {
      const d3 p0j = ld3(S.hp0[j]);
      const d3 dj = p0j - Ps;
      const d3 D = p0i - p0j;
      // L_ij
      z1 bracket = zsub(zsub(U1, rdot(dj, U2)), rdot(ei, U3));
      zacc(bracket, zscale(dot(ei, dj), U0));
      const z1 L = zsub(zscale(0.25, zmul(ksq, bracket)), U0);
      // K_ij
      z3 X = z3sub(z3sub(V1, zcross(V2, ei)), rcross(dj, V3));
      X = z3add(X, zs_v(V0, cross(dj, ei)));
      const z1 K = zscale(-0.25, rdot(D, X));
      const double c = scatter_coef(T, i, S, j);
      store_block(H, ntr, T.hrwg[i], T.hneg[i], S.hrwg[j], S.hneg[j], zscale(c, L), zscale(c, K));
    }
  }
}

// ---------------- far pairs ----------------
//
// Closed form of the nine products.  With P_t, P_s the frame origins (p0 of
// t[0], s[0]), rho = r_t - P_t, l = r_s - P_s, e_i = p0_i - P_t, d_j = p0_j - P_s,
// D_ij = p0_i - p0_j (test half i, source half j):
//   Gphi_j(r_t)   = 1/2 (A - d_j I0)
//   DGxphi_j(r_t) = 1/2 (r_t - p0_j) x (Q1 - d_j Q0)     [(r_t-r_s)x(r_s-p0_j) = (r_t-p0_j)x(r_s-p0_j)]
//   phi_i . DGxphi_j = 1/4 D_ij . ((Q1 - d_j Q0) x (rho - e_i))   [a.(a x X) = 0]
// and, with the outer moments U0 = sum w I0, U1 = sum w rho.A, U2 = sum w I0 rho,
// U3 = sum w A, V0 = sum w Q0, V1 = sum w Q1 x rho, V2 = sum w Q1, V3 = sum w Q0 rho:
//   L_ij = k^2/4 [U1 - d_j.U2 - e_i.U3 + (e_i.d_j) U0] - U0
//   K_ij = -1/4 D_ij . [V1 - V2 x e_i - d_j x V3 + V0 (d_j x e_i)]
// which is LKFarOuterIntegrand (src/Impedance.cpp:154-168) summed over the outer rule.
__device__ __noinline__ void far_pair(const TriRec &T, const TriRec &S, const GreenDev &g,
                                      const double (*rule)[3], int nr, HalfPairBlock *H, int ntr) {
  const d3 Pt = ld3(T.p0), Ps = ld3(S.p0);
  const d3 v01t = ld3(T.v01), v02t = ld3(T.v02), v01s = ld3(S.v01), v02s = ld3(S.v02);
  z1 U0 = {0, 0}, U1 = {0, 0}, V0 = {0, 0};
  z3 U2 = z3zero(), U3 = z3zero(), V1 = z3zero(), V2 = z3zero(), V3 = z3zero();
  for (int q = 0; q < nr; q++) {
    const double a = rule[q][0], b = rule[q][1], w = rule[q][2];
    const d3 rho = a * v01t + b * v02t;
    const d3 rt = Pt + rho;
    z1 I0 = {0, 0}, Q0 = {0, 0};
    z3 A = z3zero(), Q1 = z3zero();
    for (int u = 0; u < nr; u++) {
      const double as = rule[u][0], bs = rule[u][1], ws = rule[u][2];
      const d3 l = as * v01s + bs * v02s;
      const d3 x = rt - (Ps + l);
      const double R2 = dot(x, x);
      const double Ri = rsqrt(R2);
      const double R = R2 * Ri;
      const z1 e = zexp_ikR(g, R);
      // scalar_gradient, src/GreensFunction.cpp:41-52
      const z1 gs = zscale(Ri, e);
      const z1 one_m_ikR = {1.0 - g.ikr * R, -g.iki * R};
      const z1 qq = zscale(Ri * Ri, zmul(gs, one_m_ikR));
      const z1 gw = zscale(ws, gs), qw = zscale(ws, qq);
      zacc(I0, gw);
      A = z3add(A, zs_v(gw, l));
      zacc(Q0, qw);
      Q1 = z3add(Q1, zs_v(qw, l));
    }
    zacc(U0, zscale(w, I0));
    zacc(U1, zscale(w, rdot(rho, A)));
    U2 = z3add(U2, zs_v(zscale(w, I0), rho));
    U3 = z3add(U3, z3scale(w, A));
    zacc(V0, zscale(w, Q0));
    V1 = z3add(V1, z3scale(w, zcross(Q1, rho)));
    V2 = z3add(V2, z3scale(w, Q1));
    V3 = z3add(V3, zs_v(zscale(w, Q0), rho));
  }
  far_contract(T, S, g, U0, U1, U2, U3, V0, V1, V2, V3, H, ntr);
}

// ---------------- far pairs in double-float (FP64-class on the FP32 pipes) ----------------
//
// far_pair() with the inner rule (the nr x nr node pairs, where the time goes)
// in double-float: pair-centred coordinates x = (D0 + rho) - l with D0 = P_t -
// P_s, e^{ikR} from df sincos / exp (quadrant and ln2 reductions in FP64), the
// four inner moments summed in df and widened to FP64 for the outer moments
// and the closed-form contraction, which stay as in far_pair().
struct df3 {
  df x, y, z;
};
__device__ __forceinline__ df3 df3_make(d3 a) { return {df_make(a.x), df_make(a.y), df_make(a.z)}; }

// e^{ikR} for the df distance R: (cos, sin)(Im(ik) R) e^{Re(ik) R}, all in df on
// the FP32 pipes (FP64 reductions for phases of 200 rad and more).
__device__ __forceinline__ void df_exp_ikR(const GreenDev &g, df ikr, df iki, df R, df &er, df &ei) {
  df sn, cs;
  const df th = df_mul(iki, R);
  if (fabsf(th.hi) < 200.f)
    df_sincos_df(th, sn, cs);
  else
    df_sincos(df_to_double(th), sn, cs);
  if (ikr.hi == 0.f) {  // real k (df_make keeps zero exactly): no FP64 compare per node
    er = cs;
    ei = sn;
    return;
  }
  const df a = df_mul(ikr, R);
  if (a.hi < -85.f) {  // below FP32's range: e^-85 of the neighbouring nodes' size
    er = {0.f, 0.f};
    ei = {0.f, 0.f};
    return;
  }
  const df m = df_exp_df(a);
  er = df_mul(m, cs);
  ei = df_mul(m, sn);
}

// ---------------- far pairs entirely in double-float ----------------
//
// Per triangle a double-float record (edge vectors, half-RWG free vertices
// relative to p0, scaled edge lengths) is built once per fill; the far pair
// then runs both rules, the outer moments and the closed-form contraction in
// df, and only widens the nine (c L, c K) products to FP64 for the store.
struct TriDF {
  float p0[3][2];              // df frame origin (first half-RWG's free vertex)
  float v01[3][2], v02[3][2];  // df edge vectors of the first half-RWG's frame
  float e[3][3][2];            // df hp0[i] - p0
  float hs[3][2];              // df helen[i] / sqrt(4 pi)
};

__global__ void tri_df_kernel(const TriRec *__restrict__ R, int n, TriDF *__restrict__ D) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const TriRec &T = R[i];
  TriDF o;
  const double sc = sqrt(BEM_ONEOVER4PI);
  for (int c = 0; c < 3; c++) {
    const df a = df_make(T.v01[c]), b = df_make(T.v02[c]), p = df_make(T.p0[c]);
    o.p0[c][0] = p.hi; o.p0[c][1] = p.lo;
    o.v01[c][0] = a.hi; o.v01[c][1] = a.lo;
    o.v02[c][0] = b.hi; o.v02[c][1] = b.lo;
  }
  for (int h = 0; h < 3; h++) {
    for (int c = 0; c < 3; c++) {
      const df e = df_make(h < T.nh ? T.hp0[h][c] - T.p0[c] : 0.0);
      o.e[h][c][0] = e.hi; o.e[h][c][1] = e.lo;
    }
    const df l = df_make(h < T.nh ? T.helen[h] * sc : 0.0);
    o.hs[h][0] = l.hi; o.hs[h][1] = l.lo;
  }
  D[i] = o;
}

struct cdf {
  df r, i;
};
struct cdf3 {
  cdf x, y, z;
};
__device__ __forceinline__ df3 ld_df3(const float (*v)[2]) { return {{v[0][0], v[0][1]}, {v[1][0], v[1][1]}, {v[2][0], v[2][1]}}; }
__device__ __forceinline__ df3 df3_add(df3 a, df3 b) { return {df_add(a.x, b.x), df_add(a.y, b.y), df_add(a.z, b.z)}; }
__device__ __forceinline__ df3 df3_sub(df3 a, df3 b) { return {df_sub(a.x, b.x), df_sub(a.y, b.y), df_sub(a.z, b.z)}; }
__device__ __forceinline__ df3 df3_scale(df s, df3 a) { return {df_mul(s, a.x), df_mul(s, a.y), df_mul(s, a.z)}; }
__device__ __forceinline__ df df3_dot(df3 a, df3 b) {
  return df_add(df_add(df_mul(a.x, b.x), df_mul(a.y, b.y)), df_mul(a.z, b.z));
}
__device__ __forceinline__ df3 df3_cross(df3 a, df3 b) {
  return {df_sub(df_mul(a.y, b.z), df_mul(a.z, b.y)), df_sub(df_mul(a.z, b.x), df_mul(a.x, b.z)),
          df_sub(df_mul(a.x, b.y), df_mul(a.y, b.x))};
}
__device__ __forceinline__ cdf cdf_add(cdf a, cdf b) { return {df_add(a.r, b.r), df_add(a.i, b.i)}; }
__device__ __forceinline__ cdf cdf_sub(cdf a, cdf b) { return {df_sub(a.r, b.r), df_sub(a.i, b.i)}; }
__device__ __forceinline__ cdf cdf_scale(df s, cdf a) { return {df_mul(s, a.r), df_mul(s, a.i)}; }
__device__ __forceinline__ cdf cdf_mul(cdf a, cdf b) {
  return {df_sub(df_mul(a.r, b.r), df_mul(a.i, b.i)), df_add(df_mul(a.r, b.i), df_mul(a.i, b.r))};
}
__device__ __forceinline__ cdf3 cdf3_add(cdf3 a, cdf3 b) { return {cdf_add(a.x, b.x), cdf_add(a.y, b.y), cdf_add(a.z, b.z)}; }
__device__ __forceinline__ cdf3 cdf3_sub(cdf3 a, cdf3 b) { return {cdf_sub(a.x, b.x), cdf_sub(a.y, b.y), cdf_sub(a.z, b.z)}; }
__device__ __forceinline__ cdf3 cdf_v(cdf c, df3 v) { return {cdf_scale(v.x, c), cdf_scale(v.y, c), cdf_scale(v.z, c)}; }
__device__ __forceinline__ cdf3 cdf3_scale(df s, cdf3 a) { return {cdf_scale(s, a.x), cdf_scale(s, a.y), cdf_scale(s, a.z)}; }
__device__ __forceinline__ cdf cdf_rdot(df3 a, cdf3 b) {
  return cdf_add(cdf_add(cdf_scale(a.x, b.x), cdf_scale(a.y, b.y)), cdf_scale(a.z, b.z));
}
// (complex vector) x (real vector)
__device__ __forceinline__ cdf3 cdf_zcross(cdf3 a, df3 b) {
  return {cdf_sub(cdf_scale(b.z, a.y), cdf_scale(b.y, a.z)), cdf_sub(cdf_scale(b.x, a.z), cdf_scale(b.z, a.x)),
          cdf_sub(cdf_scale(b.y, a.x), cdf_scale(b.x, a.y))};
}
// (real vector) x (complex vector)
__device__ __forceinline__ cdf3 cdf_rcross(df3 a, cdf3 b) {
  return {cdf_sub(cdf_scale(a.y, b.z), cdf_scale(a.z, b.y)), cdf_sub(cdf_scale(a.z, b.x), cdf_scale(a.x, b.z)),
          cdf_sub(cdf_scale(a.x, b.y), cdf_scale(a.y, b.x))};
}
__device__ __forceinline__ cdf3 cdf3_zero() {
  const df z = {0.f, 0.f};
  return {{z, z}, {z, z}, {z, z}};
}

__device__ __noinline__ void far_pair_df2(const TriRec &T, const TriRec &S, const TriDF &TD, const TriDF &SD,
                                          const GreenDev &g, const float (*rdf)[6], int nr, HalfPairBlock *H,
                                          int ntr) {
  const df3 D0 = df3_sub(ld_df3(TD.p0), ld_df3(SD.p0));  // P_t - P_s
  const df3 v01t = ld_df3(TD.v01), v02t = ld_df3(TD.v02), v01s = ld_df3(SD.v01), v02s = ld_df3(SD.v02);
  const df ikr = {g.ikr_f[0], g.ikr_f[1]}, iki = {g.iki_f[0], g.iki_f[1]};
  const df z0 = {0.f, 0.f};
  cdf U0 = {z0, z0}, U1 = {z0, z0}, V0 = {z0, z0};
  cdf3 U2 = cdf3_zero(), U3 = cdf3_zero(), V1 = cdf3_zero(), V2 = cdf3_zero(), V3 = cdf3_zero();
  for (int q = 0; q < nr; q++) {
    const df a = {rdf[q][0], rdf[q][1]}, b = {rdf[q][2], rdf[q][3]}, w = {rdf[q][4], rdf[q][5]};
    const df3 rho = df3_add(df3_scale(a, v01t), df3_scale(b, v02t));
    const df3 rts = df3_add(D0, rho);  // r_t - P_s
    df I0r = z0, I0i = z0, Q0r = z0, Q0i = z0;
    df Ar[3] = {z0, z0, z0}, Ai[3] = {z0, z0, z0}, Qr[3] = {z0, z0, z0}, Qi[3] = {z0, z0, z0};
    for (int u = 0; u < nr; u++) {
      const df as = {rdf[u][0], rdf[u][1]}, bs = {rdf[u][2], rdf[u][3]}, ws = {rdf[u][4], rdf[u][5]};
      const df l[3] = {df_add(df_mul(as, v01s.x), df_mul(bs, v02s.x)), df_add(df_mul(as, v01s.y), df_mul(bs, v02s.y)),
                       df_add(df_mul(as, v01s.z), df_mul(bs, v02s.z))};
      const df xx = df_sub(rts.x, l[0]), xy = df_sub(rts.y, l[1]), xz = df_sub(rts.z, l[2]);
      const df R2 = df_add(df_add(df_sqr(xx), df_sqr(xy)), df_sqr(xz));
      const df R = df_sqrt(R2);
      const df Ri = df_rcp(R);
      df er, ei;
      df_exp_ikR(g, ikr, iki, R, er, ei);
      const df gr = df_mul(er, Ri), gi = df_mul(ei, Ri);
      const df zr = df_mul(ikr, R), zi = df_mul(iki, R);
      const df mr = df_add_f(df_neg(zr), 1.f), mi = df_neg(zi);
      const df Ri2 = df_sqr(Ri);
      const df qr = df_mul(df_sub(df_mul(gr, mr), df_mul(gi, mi)), Ri2);
      const df qi = df_mul(df_add(df_mul(gr, mi), df_mul(gi, mr)), Ri2);
      const df gwr = df_mul(ws, gr), gwi = df_mul(ws, gi), qwr = df_mul(ws, qr), qwi = df_mul(ws, qi);
      I0r = df_add(I0r, gwr);
      I0i = df_add(I0i, gwi);
      Q0r = df_add(Q0r, qwr);
      Q0i = df_add(Q0i, qwi);
#pragma unroll
      for (int c = 0; c < 3; c++) {
        Ar[c] = df_add(Ar[c], df_mul(gwr, l[c]));
        Ai[c] = df_add(Ai[c], df_mul(gwi, l[c]));
        Qr[c] = df_add(Qr[c], df_mul(qwr, l[c]));
        Qi[c] = df_add(Qi[c], df_mul(qwi, l[c]));
      }
    }
    const cdf I0 = {I0r, I0i}, Q0 = {Q0r, Q0i};
    const cdf3 A = {{Ar[0], Ai[0]}, {Ar[1], Ai[1]}, {Ar[2], Ai[2]}};
    const cdf3 Q1 = {{Qr[0], Qi[0]}, {Qr[1], Qi[1]}, {Qr[2], Qi[2]}};
    const cdf wI0 = cdf_scale(w, I0), wQ0 = cdf_scale(w, Q0);
    U0 = cdf_add(U0, wI0);
    U1 = cdf_add(U1, cdf_scale(w, cdf_rdot(rho, A)));
    U2 = cdf3_add(U2, cdf_v(wI0, rho));
    U3 = cdf3_add(U3, cdf3_scale(w, A));
    V0 = cdf_add(V0, wQ0);
    V1 = cdf3_add(V1, cdf3_scale(w, cdf_zcross(Q1, rho)));
    V2 = cdf3_add(V2, cdf3_scale(w, Q1));
    V3 = cdf3_add(V3, cdf_v(wQ0, rho));
  }
  // the closed form of far_pair(), in df
  const cdf ksq = {{g.ksqr_f[0], g.ksqr_f[1]}, {g.ksqi_f[0], g.ksqi_f[1]}};
  const df quarter = {0.25f, 0.f};
  for (int i = 0; i < T.nh; i++) {
    const df3 ei = ld_df3(TD.e[i]);
    for (int j = 0; j < S.nh; j++) {
      const df3 dj = ld_df3(SD.e[j]);
      const df3 D = df3_sub(df3_add(D0, ei), dj);  // p0_i - p0_j
      cdf br = cdf_sub(cdf_sub(U1, cdf_rdot(dj, U2)), cdf_rdot(ei, U3));
      br = cdf_add(br, cdf_scale(df3_dot(ei, dj), U0));
      const cdf L = cdf_sub(cdf_scale(quarter, cdf_mul(ksq, br)), U0);
      cdf3 X = cdf3_sub(cdf3_sub(V1, cdf_zcross(V2, ei)), cdf_rcross(dj, V3));
      X = cdf3_add(X, cdf_v(V0, df3_cross(dj, ei)));
      const cdf K = cdf_scale(df_neg(quarter), cdf_rdot(D, X));
      df c = df_mul({TD.hs[i][0], TD.hs[i][1]}, {SD.hs[j][0], SD.hs[j][1]});
      if (T.hneg[i] != S.hneg[j]) c = df_neg(c);
      const cdf cL = cdf_scale(c, L), cK = cdf_scale(c, K);
      store_block_df(H, ntr, T.hrwg[i], T.hneg[i], S.hrwg[j], S.hneg[j], cL.r, cL.i, cK.r, cK.i);
    }
  }
}

// ---------------- far pairs in FP32 (mixed precision) ----------------
//
// Same closed form as far_pair(), evaluated in FP32 with a pair-centred
// distance: r_t - r_s = D0 + u, D0 = P_t - P_s (FP64 once per pair), u = rho - l
// (small, FP32).  R = R0 + dR with R0 = |D0| in FP64 and
// dR = (2 D0.u + u.u) / (R0 + R) in FP32, so the phase k R is k R0 reduced
// modulo 2 pi in FP64 once per pair plus k dR in FP32; the relative error of
// every node's e^{ikR}/R stays near FP32 rounding at any distance.
struct f3 {
  float x, y, z;
};
struct c1 {
  float r, i;
};
struct c3 {
  c1 x, y, z;
};
__device__ __forceinline__ f3 f3of(d3 a) { return {(float)a.x, (float)a.y, (float)a.z}; }
__device__ __forceinline__ f3 operator+(f3 a, f3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ f3 operator-(f3 a, f3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ f3 operator*(float c, f3 a) { return {c * a.x, c * a.y, c * a.z}; }
__device__ __forceinline__ float fdot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ f3 fcross(f3 a, f3 b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ c1 cmulf(c1 a, c1 b) { return {a.r * b.r - a.i * b.i, a.r * b.i + a.i * b.r}; }
__device__ __forceinline__ c1 csubf(c1 a, c1 b) { return {a.r - b.r, a.i - b.i}; }
__device__ __forceinline__ c1 cscalef(float c, c1 a) { return {c * a.r, c * a.i}; }
__device__ __forceinline__ void caccf(c1 &a, c1 b) { a.r += b.r; a.i += b.i; }
__device__ __forceinline__ c3 c3zerof() { return {{0, 0}, {0, 0}, {0, 0}}; }
__device__ __forceinline__ c3 cs_vf(c1 c, f3 v) { return {{c.r * v.x, c.i * v.x}, {c.r * v.y, c.i * v.y}, {c.r * v.z, c.i * v.z}}; }
__device__ __forceinline__ void c3accf(c3 &a, c3 b) {
  caccf(a.x, b.x); caccf(a.y, b.y); caccf(a.z, b.z);
}
__device__ __forceinline__ c3 c3scalef(float c, c3 a) { return {cscalef(c, a.x), cscalef(c, a.y), cscalef(c, a.z)}; }
__device__ __forceinline__ c3 c3subf(c3 a, c3 b) { return {csubf(a.x, b.x), csubf(a.y, b.y), csubf(a.z, b.z)}; }
__device__ __forceinline__ c1 rdotf(f3 a, c3 b) {
  return {a.x * b.x.r + a.y * b.y.r + a.z * b.z.r, a.x * b.x.i + a.y * b.y.i + a.z * b.z.i};
}
__device__ __forceinline__ c3 zcrossf(c3 a, f3 b) {
  return {{a.y.r * b.z - a.z.r * b.y, a.y.i * b.z - a.z.i * b.y},
          {a.z.r * b.x - a.x.r * b.z, a.z.i * b.x - a.x.i * b.z},
          {a.x.r * b.y - a.y.r * b.x, a.x.i * b.y - a.y.i * b.x}};
}
__device__ __forceinline__ c3 rcrossf(f3 a, c3 b) {
  return {{a.y * b.z.r - a.z * b.y.r, a.y * b.z.i - a.z * b.y.i},
          {a.z * b.x.r - a.x * b.z.r, a.z * b.x.i - a.x * b.z.i},
          {a.x * b.y.r - a.y * b.x.r, a.x * b.y.i - a.y * b.x.i}};
}

__device__ __noinline__ void far_pair_fp32(const TriRec &T, const TriRec &S, const GreenDev &g,
                                           const double (*rule)[3], int nr, HalfPairBlock *H, int ntr) {
  const d3 Pt = ld3(T.p0), Ps = ld3(S.p0);
  const d3 D0d = Pt - Ps;
  const double R0d = sqrt(dot(D0d, D0d));
  // per-pair FP64: magnitude and phase of e^{ik R0}
  const double ph0d = g.iki * R0d;
  const double ph0r = ph0d - 6.283185307179586476925286766559 * rint(ph0d * 0.15915494309189533576888376337251);
  const float ph0 = (float)ph0r;
  const float m0 = (float)exp(g.ikr * R0d);
  const float R0 = (float)R0d, R0sq = (float)(R0d * R0d);
  const f3 D0 = f3of(D0d);
  const float ikr = (float)g.ikr, iki = (float)g.iki;
  const f3 v01t = f3of(ld3(T.v01)), v02t = f3of(ld3(T.v02)), v01s = f3of(ld3(S.v01)), v02s = f3of(ld3(S.v02));
  c1 U0 = {0, 0}, U1 = {0, 0}, V0 = {0, 0};
  c3 U2 = c3zerof(), U3 = c3zerof(), V1 = c3zerof(), V2 = c3zerof(), V3 = c3zerof();
  for (int q = 0; q < nr; q++) {
    const float a = (float)rule[q][0], b = (float)rule[q][1], w = (float)rule[q][2];
    const f3 rho = a * v01t + b * v02t;
    c1 I0 = {0, 0}, Q0 = {0, 0};
    c3 A = c3zerof(), Q1 = c3zerof();
    for (int uix = 0; uix < nr; uix++) {
      const float as = (float)rule[uix][0], bs = (float)rule[uix][1], ws = (float)rule[uix][2];
      const f3 l = as * v01s + bs * v02s;
      const f3 u = rho - l;
      const float sdel = 2.0f * fdot(D0, u) + fdot(u, u);
      const float Rf = sqrtf(R0sq + sdel);
      const float dR = sdel / (R0 + Rf);
      const float R = R0 + dR;
      float sn, cs;
      sincosf(ph0 + iki * dR, &sn, &cs);
      const float mag = m0 * expf(ikr * dR);
      const float Ri = 1.0f / R;
      const c1 gs = {mag * cs * Ri, mag * sn * Ri};
      const c1 one_m_ikR = {1.0f - ikr * R, -iki * R};
      const c1 qq = cscalef(Ri * Ri, cmulf(gs, one_m_ikR));
      const c1 gw = cscalef(ws, gs), qw = cscalef(ws, qq);
      caccf(I0, gw);
      c3accf(A, cs_vf(gw, l));
      caccf(Q0, qw);
      c3accf(Q1, cs_vf(qw, l));
    }
    caccf(U0, cscalef(w, I0));
    caccf(U1, cscalef(w, rdotf(rho, A)));
    c3accf(U2, cs_vf(cscalef(w, I0), rho));
    c3accf(U3, c3scalef(w, A));
    caccf(V0, cscalef(w, Q0));
    c3accf(V1, c3scalef(w, zcrossf(Q1, rho)));
    c3accf(V2, c3scalef(w, Q1));
    c3accf(V3, cs_vf(cscalef(w, Q0), rho));
  }
  const c1 ksq = {(float)g.ksqr, (float)g.ksqi};
  for (int i = 0; i < T.nh; i++) {
    const f3 ei = f3of(ld3(T.hp0[i]) - Pt);
    for (int j = 0; j < S.nh; j++) {
      const f3 dj = f3of(ld3(S.hp0[j]) - Ps);
      const f3 D = (D0 + ei) - dj;
      c1 bracket = csubf(csubf(U1, rdotf(dj, U2)), rdotf(ei, U3));
      caccf(bracket, cscalef(fdot(ei, dj), U0));
      const c1 L = csubf(cscalef(0.25f, cmulf(ksq, bracket)), U0);
      c3 X = c3subf(c3subf(V1, zcrossf(V2, ei)), rcrossf(dj, V3));
      c3accf(X, cs_vf(V0, fcross(dj, ei)));
      const c1 K = cscalef(-0.25f, rdotf(D, X));
      const double c = scatter_coef(T, i, S, j);
      store_block(H, ntr, T.hrwg[i], T.hneg[i], S.hrwg[j], S.hneg[j], z1{c * L.r, c * L.i}, z1{c * K.r, c * K.i});
    }
  }
}

// One fill of a group launch: Zts(t, s, g) into the half-pair blocks H, with
// its share of the group's far tiles and near work units (prefix offsets).
struct FillTask {
  const TriRec *T, *S;       // test and source trees' records
  const TriDF *TD, *SD;      // their double-float records (double-float mode), else null
  const NearPair *near;      // the near-pair list of (t, s)
  HalfPairBlock *H;          // this fill's half-pair blocks
  int64_t nnear;             // near pairs
  int64_t near0;             // first near work unit of the group that is this task's
  int64_t far0;              // first far tile of the group that is this task's
  int ntT, ntS, ntr, far_tx; // triangles of t and s, RWGs of t, far tiles along s
  GreenDev g;
};

__device__ __forceinline__ int task_of_far(const FillTask *tk, int n, int64_t u) {
  int i = n - 1;
  while (i > 0 && u < tk[i].far0) i--;
  return i;
}

__device__ __forceinline__ int task_of_near(const FillTask *tk, int n, int64_t u) {
  int i = n - 1;
  while (i > 0 && u < tk[i].near0) i--;
  return i;
}

// mixed != 0: pairs whose centroid distance exceeds 3 edge lengths (the longer
// of the two triangles' longest edges) are integrated in FP32.
__device__ __forceinline__ void far_pair_at(const TriRec *__restrict__ Tr, int ntT, const TriRec *__restrict__ Sr,
                                            int ntS, const GreenDev &g, const FarOpts &o,
                                            HalfPairBlock *__restrict__ H, int ntr, int mode,
                                            const TriDF *__restrict__ TDr, const TriDF *__restrict__ SDr, int sb,
                                            int ta) {
  if (sb >= ntS || ta >= ntT) return;
  const TriRec &T = Tr[ta];
  const TriRec &S = Sr[sb];
  if (T.gid == S.gid || shares_vertex(T.vid, S.vid)) return;  // near kernel
  // far-rule choice, src/Impedance.cpp:329-360
  const double d = dist2_rn(T.c, S.c);
  const double e = fmax(T.emax, S.emax);
  const double emax2 = __dmul_rn(e, e);
  if (mode == FILL_DF) {
    const TriDF &TD = TDr[ta], &SD = SDr[sb];
    if (__dmul_rn(d, o.th6) > emax2) far_pair_df2(T, S, TD, SD, g, c_rdf6, 6, H, ntr);
    else if (__dmul_rn(d, o.th10) > emax2) far_pair_df2(T, S, TD, SD, g, c_rdf10, 10, H, ntr);
    else if (__dmul_rn(d, o.th15) > emax2) far_pair_df2(T, S, TD, SD, g, c_rdf15, 15, H, ntr);
    else if (__dmul_rn(d, o.th21) > emax2) far_pair_df2(T, S, TD, SD, g, c_rdf21, 21, H, ntr);
    else far_pair_df2(T, S, TD, SD, g, c_rdf36, 36, H, ntr);
    return;
  }
  if (mode == FILL_FP32_FAR && d > 9.0 * emax2) {
    // beyond 3 edge lengths every default threshold selects the 6-point rule;
    // the cascade is kept for non-default Options
    if (__dmul_rn(d, o.th6) > emax2) far_pair_fp32(T, S, g, c_rule6, 6, H, ntr);
    else if (__dmul_rn(d, o.th10) > emax2) far_pair_fp32(T, S, g, c_rule10, 10, H, ntr);
    else if (__dmul_rn(d, o.th15) > emax2) far_pair_fp32(T, S, g, c_rule15, 15, H, ntr);
    else if (__dmul_rn(d, o.th21) > emax2) far_pair_fp32(T, S, g, c_rule21, 21, H, ntr);
    else far_pair_fp32(T, S, g, c_rule36, 36, H, ntr);
    return;
  }
  if (__dmul_rn(d, o.th6) > emax2) far_pair(T, S, g, c_rule6, 6, H, ntr);
  else if (__dmul_rn(d, o.th10) > emax2) far_pair(T, S, g, c_rule10, 10, H, ntr);
  else if (__dmul_rn(d, o.th15) > emax2) far_pair(T, S, g, c_rule15, 15, H, ntr);
  else if (__dmul_rn(d, o.th21) > emax2) far_pair(T, S, g, c_rule21, 21, H, ntr);
  else far_pair(T, S, g, c_rule36, 36, H, ntr);
}

// One fill (t, s, g) -> H: thread (x, y) of the 2-D grid takes the source
// triangle blockIdx.x * 32 + x and the test triangle blockIdx.y * blockDim.y + y.
__global__ void __launch_bounds__(256) far_pairs_kernel(const TriRec *__restrict__ Tr, int ntT,
                                                        const TriRec *__restrict__ Sr, int ntS, GreenDev g,
                                                        FarOpts o, HalfPairBlock *__restrict__ H, int ntr, int mode,
                                                        const TriDF *__restrict__ TDr, const TriDF *__restrict__ SDr) {
  far_pair_at(Tr, ntT, Sr, ntS, g, o, H, ntr, mode, TDr, SDr, blockIdx.x * blockDim.x + threadIdx.x,
              blockIdx.y * blockDim.y + threadIdx.y);
}

// A group of fills in one launch (the three Zts of a solve, or of several
// requests): CTA b takes far tile b of the task whose range holds it, a tile
// being 32 source x blockDim.y test triangles.  The task's Green's function
// is staged in shared memory (one task per CTA).
__global__ void __launch_bounds__(256) far_pairs_group_kernel(const FillTask *__restrict__ tasks, int ntask,
                                                              FarOpts o, int mode) {
  __shared__ GreenDev s_g;
  const int i = task_of_far(tasks, ntask, blockIdx.x);
  const FillTask &tk = tasks[i];
  if (threadIdx.x == 0 && threadIdx.y == 0) s_g = tk.g;
  __syncthreads();
  const int64_t local = (int64_t)blockIdx.x - tk.far0;
  const int bx = (int)(local % tk.far_tx), by = (int)(local / tk.far_tx);
  far_pair_at(tk.T, tk.ntT, tk.S, tk.ntS, s_g, o, tk.H, tk.ntr, mode, tk.TD, tk.SD, bx * 32 + threadIdx.x,
              by * blockDim.y + threadIdx.y);
}

// ---------------- near pairs ----------------

// EHNonSmoothIntegral, src/Source.cpp:16-86 (frame of the source triangle's s[0]).
__device__ void eh_nonsmooth(const TriRec &S, d3 rt, double &ISn3h, double &ISn1, double &IS1, d3 &IL1,
                             d3 &IL3) {
  const double tol = 1e-6 * S.elen0;
  const d3 p0 = rt - ld3(S.p0), p1 = rt - ld3(S.p1), p2 = rt - ld3(S.p2);
  const double R02 = dot(p0, p0), R0 = sqrt(R02);
  const double R12 = dot(p1, p1), R1 = sqrt(R12);
  const double R22 = dot(p2, p2), R2 = sqrt(R22);
  const d3 a0 = (1. / R0) * p0, a1 = (1. / R1) * p1, a2 = (1. / R2) * p2;
  const d3 n = ld3(S.n);
  const double x = 1.0 + dot(a0, a1 + a2) + dot(a1, a2);
  const double y = fabs(dot(a0, cross(a1, a2)));
  const double h = dot(p0, n);
  ISn3h = (h < 0. ? -2. : 2.) * atan2(y, x);
  const d3 v01 = ld3(S.v01), v12 = ld3(S.v12), v20 = ld3(S.v20);
  double num, den;
  const double s010 = S.nv01i * dot(v01, p0), s011 = S.nv01i * dot(v01, p1);
  num = R1 - s011; den = R0 - s010;
  const double ILn1_01 = (fabs(num) < tol || fabs(den) < tol) ? 0. : log(num / den);
  const double s121 = S.nv12i * dot(v12, p1), s122 = S.nv12i * dot(v12, p2);
  num = R2 - s122; den = R1 - s121;
  const double ILn1_12 = (fabs(num) < tol || fabs(den) < tol) ? 0. : log(num / den);
  const double s202 = S.nv20i * dot(v20, p2), s200 = S.nv20i * dot(v20, p0);
  num = R0 - s200; den = R2 - s202;
  const double ILn1_20 = (fabs(num) < tol || fabs(den) < tol) ? 0. : log(num / den);
  const d3 m01 = ld3(S.m01), m12 = ld3(S.m12), m20 = ld3(S.m20);
  const double t01 = dot(m01, p0), t12 = dot(m12, p1), t20 = dot(m20, p2);
  ISn1 = -h * ISn3h - (t01 * ILn1_01 + t12 * ILn1_12 + t20 * ILn1_20);
  const double R02_01 = R02 - s010 * s010;
  const double IL1_01 = 0.5 * (R02_01 * ILn1_01 - (R1 * s011 - R0 * s010));
  const double R02_12 = R12 - s121 * s121;
  const double IL1_12 = 0.5 * (R02_12 * ILn1_12 - (R2 * s122 - R1 * s121));
  const double R02_20 = R22 - s202 * s202;
  const double IL1_20 = 0.5 * (R02_20 * ILn1_20 - (R0 * s200 - R2 * s202));
  const double IL3_01 = 0.75 * R02_01 * IL1_01 - 0.25 * (R12 * R1 * s011 - R02 * R0 * s010);
  const double IL3_12 = 0.75 * R02_12 * IL1_12 - 0.25 * (R22 * R2 * s122 - R12 * R1 * s121);
  const double IL3_20 = 0.75 * R02_20 * IL1_20 - 0.25 * (R02 * R0 * s200 - R22 * R2 * s202);
  IS1 = BEM_ONETHIRD * (h * h * ISn1 - (t01 * IL1_01 + t12 * IL1_12 + t20 * IL1_20));
  IL1 = IL1_01 * m01 + IL1_12 * m12 + IL1_20 * m20;
  IL3 = IL3_01 * m01 + IL3_12 * m12 + IL3_20 * m20;
}

// LKEdgeIntegral, src/Impedance.cpp:13-73 (frame of the test triangle's t[0]).
__device__ void lk_edge_integral(const TriRec &T, d3 rs, double &ISn1, d3 &IL1) {
  const d3 p0 = rs - ld3(T.p0), p1 = rs - ld3(T.p1), p2 = rs - ld3(T.p2);
  const double R02 = dot(p0, p0), R0 = sqrt(R02);
  const double R12 = dot(p1, p1), R1 = sqrt(R12);
  const double R22 = dot(p2, p2), R2 = sqrt(R22);
  const double tol = 1e-8 * T.elen0;
  const d3 a0 = (1. / R0) * p0, a1 = (1. / R1) * p1, a2 = (1. / R2) * p2;
  const double h = dot(p0, ld3(T.n));
  const double x = 1.0 + dot(a0, a1 + a2) + dot(a1, a2);
  const double y = fabs(dot(a0, cross(a1, a2)));
  const double ISn3h = (h < 0 ? -2. : 2.) * atan2(y, x);
  const d3 m01 = ld3(T.m01), m12 = ld3(T.m12), m20 = ld3(T.m20);
  const double t01 = dot(m01, p0), t12 = dot(m12, p1), t20 = dot(m20, p2);
  const d3 v01 = ld3(T.v01), v12 = ld3(T.v12), v20 = ld3(T.v20);
  double num, den;
  const double s010 = T.nv01i * dot(v01, p0), s011 = T.nv01i * dot(v01, p1);
  num = R1 - s011; den = R0 - s010;
  const double ILn1_01 = (fabs(num) < tol || fabs(den) < tol) ? 0. : log(num / den);
  const double s121 = T.nv12i * dot(v12, p1), s122 = T.nv12i * dot(v12, p2);
  num = R2 - s122; den = R1 - s121;
  const double ILn1_12 = (fabs(num) < tol || fabs(den) < tol) ? 0. : log(num / den);
  const double s202 = T.nv20i * dot(v20, p2), s200 = T.nv20i * dot(v20, p0);
  num = R0 - s200; den = R2 - s202;
  const double ILn1_20 = (fabs(num) < tol || fabs(den) < tol) ? 0. : log(num / den);
  ISn1 = -h * ISn3h - (t01 * ILn1_01 + t12 * ILn1_12 + t20 * ILn1_20);
  const double IL1_01 = 0.5 * ((R02 - s010 * s010) * ILn1_01 - (R1 * s011 - R0 * s010));
  const double IL1_12 = 0.5 * ((R12 - s121 * s121) * ILn1_12 - (R2 * s122 - R1 * s121));
  const double IL1_20 = 0.5 * ((R22 - s202 * s202) * ILn1_20 - (R0 * s200 - R2 * s202));
  IL1 = IL1_01 * m01 + IL1_12 * m12 + IL1_20 * m20;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

constexpr int NEAR_WARPS = 4;

// Moments of the smooth inner rule at one outer node (complex df):
// I0 = sum w g~, A = sum w g~ l, Q0 = sum w q~, Q1 = sum w q~ l.
struct InnerMomDF {
  cdf I0, Q0;
  cdf3 A, Q1;
};

// Smooth inner rule of a near pair at NP outer nodes at once, double-float
// version: the same moments as the FP64 loop in near_pairs_kernel
// (LKSmoothInnerIntegrand, src/Impedance.cpp:93-105, with
// scalar_gradient_smooth, src/GreensFunction.cpp:54-69), summed in df from df
// nodes (l, w).  The NP points are independent dependency chains over the same
// inner nodes, which the scheduler interleaves.
template <int NP>
__device__ __noinline__ void near_inner_df(const float (*nd)[8], const df3 *rp, const GreenDev &g, InnerMomDF *out) {
  const df ikr = {g.ikr_f[0], g.ikr_f[1]}, iki = {g.iki_f[0], g.iki_f[1]};
  const df k2r = {g.k2r_f[0], g.k2r_f[1]}, k2i = {g.k2i_f[0], g.k2i_f[1]};
  df3 r[NP];
  df I0r[NP], I0i[NP], Q0r[NP], Q0i[NP], Ar[NP][3], Ai[NP][3], Qr[NP][3], Qi[NP][3];
  const df z = {0.f, 0.f};
#pragma unroll
  for (int p = 0; p < NP; p++) {
    r[p] = rp[p];
    I0r[p] = z; I0i[p] = z; Q0r[p] = z; Q0i[p] = z;
#pragma unroll
    for (int c = 0; c < 3; c++) { Ar[p][c] = z; Ai[p][c] = z; Qr[p][c] = z; Qi[p][c] = z; }
  }
  for (int u = 0; u < BEMGPU_TRI_RULE91_N; u++) {
    const float4 n0 = *reinterpret_cast<const float4 *>(&nd[u][0]);
    const float4 n1 = *reinterpret_cast<const float4 *>(&nd[u][4]);
    const df l[3] = {{n0.x, n0.y}, {n0.z, n0.w}, {n1.x, n1.y}};
    const df ws = {n1.z, n1.w};
#pragma unroll
    for (int p = 0; p < NP; p++) {
      const df xx = df_sub(r[p].x, l[0]), xy = df_sub(r[p].y, l[1]), xz = df_sub(r[p].z, l[2]);
      const df R2 = df_add(df_add(df_sqr(xx), df_sqr(xy)), df_sqr(xz));
      const df R = df_sqrt(R2);
      const df Ri = df_rcp(R);
      df er, ei;
      df_exp_ikR(g, ikr, iki, R, er, ei);
      // g~ = (e - 1)/R - k2 R
      const df gr = df_sub(df_mul(df_add_f(er, -1.f), Ri), df_mul(k2r, R));
      const df gi = df_sub(df_mul(ei, Ri), df_mul(k2i, R));
      // q~ = (e (1 - ikR) + R^2 k2 - 1) / R^3
      const df zr = df_mul(ikr, R), zi = df_mul(iki, R);
      const df mr = df_add_f(df_neg(zr), 1.f), mi = df_neg(zi);
      df nr = df_sub(df_mul(er, mr), df_mul(ei, mi));
      df ni = df_add(df_mul(er, mi), df_mul(ei, mr));
      nr = df_add_f(df_add(nr, df_mul(R2, k2r)), -1.f);
      ni = df_add(ni, df_mul(R2, k2i));
      const df Ri3 = df_mul(df_sqr(Ri), Ri);
      const df qr = df_mul(Ri3, nr), qi = df_mul(Ri3, ni);
      const df gwr = df_mul(ws, gr), gwi = df_mul(ws, gi), qwr = df_mul(ws, qr), qwi = df_mul(ws, qi);
      I0r[p] = df_add(I0r[p], gwr);
      I0i[p] = df_add(I0i[p], gwi);
      Q0r[p] = df_add(Q0r[p], qwr);
      Q0i[p] = df_add(Q0i[p], qwi);
#pragma unroll
      for (int c = 0; c < 3; c++) {
        Ar[p][c] = df_add(Ar[p][c], df_mul(gwr, l[c]));
        Ai[p][c] = df_add(Ai[p][c], df_mul(gwi, l[c]));
        Qr[p][c] = df_add(Qr[p][c], df_mul(qwr, l[c]));
        Qi[p][c] = df_add(Qi[p][c], df_mul(qwi, l[c]));
      }
    }
  }
#pragma unroll
  for (int p = 0; p < NP; p++) {
    out[p].I0 = {I0r[p], I0i[p]};
    out[p].Q0 = {Q0r[p], Q0i[p]};
    out[p].A = {{Ar[p][0], Ai[p][0]}, {Ar[p][1], Ai[p][1]}, {Ar[p][2], Ai[p][2]}};
    out[p].Q1 = {{Qr[p][0], Qi[p][0]}, {Qr[p][1], Qi[p][1]}, {Qr[p][2], Qi[p][2]}};
  }
}

// A triangle in double-float, vertices relative to a chosen origin O (the
// test triangle's p0): what the closed-form integrals below read.
struct TriFrameDF {
  df3 p0, p1, p2, n, v01, v12, v20, m01, m12, m20;
  df nv01i, nv12i, nv20i;
};

__device__ void tri_frame_df(const TriRec &T, d3 O, TriFrameDF &F) {
  F.p0 = df3_make(ld3(T.p0) - O);
  F.p1 = df3_make(ld3(T.p1) - O);
  F.p2 = df3_make(ld3(T.p2) - O);
  F.n = df3_make(ld3(T.n));
  F.v01 = df3_make(ld3(T.v01));
  F.v12 = df3_make(ld3(T.v12));
  F.v20 = df3_make(ld3(T.v20));
  F.m01 = df3_make(ld3(T.m01));
  F.m12 = df3_make(ld3(T.m12));
  F.m20 = df3_make(ld3(T.m20));
  F.nv01i = df_make(T.nv01i);
  F.nv12i = df_make(T.nv12i);
  F.nv20i = df_make(T.nv20i);
}

__device__ __forceinline__ df log_ratio_df(df num, df den, float tol) {
  if (fabsf(num.hi) < tol || fabsf(den.hi) < tol) return {0.f, 0.f};
  return df_log(df_mul(num, df_rcp(den)));
}

// The closed-form potential integrals of a triangle F seen from the point r
// (both relative to the same origin), in double-float: the analytic part of
// EHNonSmoothIntegral (src/Source.cpp:16-86, with full = true: ISn3h, ISn1,
// IS1, IL1, IL3) and LKEdgeIntegral (src/Impedance.cpp:13-73, full = false:
// ISn3h, ISn1, IL1), step for step as eh_nonsmooth / lk_edge_integral do them
// in FP64; h = (r - p0) . n.  tol is the edge-line cut-off of the logarithms.
__device__ __noinline__ void tri_potentials_df(const TriFrameDF &F, df3 r, float tol, bool full, df &ISn3h,
                                               df &ISn1, df &IS1, df3 &IL1, df3 &IL3, df &h) {
  const df3 p0 = df3_sub(r, F.p0), p1 = df3_sub(r, F.p1), p2 = df3_sub(r, F.p2);
  const df R02 = df3_dot(p0, p0), R12 = df3_dot(p1, p1), R22 = df3_dot(p2, p2);
  const df R0 = df_sqrt(R02), R1 = df_sqrt(R12), R2 = df_sqrt(R22);
  const df3 a0 = df3_scale(df_rcp(R0), p0), a1 = df3_scale(df_rcp(R1), p1), a2 = df3_scale(df_rcp(R2), p2);
  const df x = df_add_f(df_add(df3_dot(a0, df3_add(a1, a2)), df3_dot(a1, a2)), 1.f);
  const df y = df_abs(df3_dot(a0, df3_cross(a1, a2)));
  h = df3_dot(p0, F.n);
  const df at = df_atan2(y, x);
  ISn3h = df_scale2(at, h.hi < 0.f ? -2.f : 2.f);
  const df s010 = df_mul(F.nv01i, df3_dot(F.v01, p0)), s011 = df_mul(F.nv01i, df3_dot(F.v01, p1));
  const df s121 = df_mul(F.nv12i, df3_dot(F.v12, p1)), s122 = df_mul(F.nv12i, df3_dot(F.v12, p2));
  const df s202 = df_mul(F.nv20i, df3_dot(F.v20, p2)), s200 = df_mul(F.nv20i, df3_dot(F.v20, p0));
  const df ILn1_01 = log_ratio_df(df_sub(R1, s011), df_sub(R0, s010), tol);
  const df ILn1_12 = log_ratio_df(df_sub(R2, s122), df_sub(R1, s121), tol);
  const df ILn1_20 = log_ratio_df(df_sub(R0, s200), df_sub(R2, s202), tol);
  const df t01 = df3_dot(F.m01, p0), t12 = df3_dot(F.m12, p1), t20 = df3_dot(F.m20, p2);
  const df tl = df_add(df_add(df_mul(t01, ILn1_01), df_mul(t12, ILn1_12)), df_mul(t20, ILn1_20));
  ISn1 = df_neg(df_add(df_mul(h, ISn3h), tl));
  const df R02_01 = df_sub(R02, df_sqr(s010));
  const df R02_12 = df_sub(R12, df_sqr(s121));
  const df R02_20 = df_sub(R22, df_sqr(s202));
  const df half = {0.5f, 0.f};
  const df IL1_01 = df_mul(half, df_sub(df_mul(R02_01, ILn1_01), df_sub(df_mul(R1, s011), df_mul(R0, s010))));
  const df IL1_12 = df_mul(half, df_sub(df_mul(R02_12, ILn1_12), df_sub(df_mul(R2, s122), df_mul(R1, s121))));
  const df IL1_20 = df_mul(half, df_sub(df_mul(R02_20, ILn1_20), df_sub(df_mul(R0, s200), df_mul(R2, s202))));
  IL1 = df3_add(df3_add(df3_scale(IL1_01, F.m01), df3_scale(IL1_12, F.m12)), df3_scale(IL1_20, F.m20));
  if (!full) return;
  const df q3 = {0.75f, 0.f}, q1 = {0.25f, 0.f};
  const df IL3_01 = df_sub(df_mul(q3, df_mul(R02_01, IL1_01)),
                           df_mul(q1, df_sub(df_mul(df_mul(R12, R1), s011), df_mul(df_mul(R02, R0), s010))));
  const df IL3_12 = df_sub(df_mul(q3, df_mul(R02_12, IL1_12)),
                           df_mul(q1, df_sub(df_mul(df_mul(R22, R2), s122), df_mul(df_mul(R12, R1), s121))));
  const df IL3_20 = df_sub(df_mul(q3, df_mul(R02_20, IL1_20)),
                           df_mul(q1, df_sub(df_mul(df_mul(R02, R0), s200), df_mul(df_mul(R22, R2), s202))));
  const df third = {0x1.555556p-2f, -0x1.555556p-27f};
  const df tI = df_add(df_add(df_mul(t01, IL1_01), df_mul(t12, IL1_12)), df_mul(t20, IL1_20));
  IS1 = df_mul(third, df_sub(df_mul(df_sqr(h), ISn1), tI));
  IL3 = df3_add(df3_add(df3_scale(IL3_01, F.m01), df3_scale(IL3_12, F.m12)), df3_scale(IL3_20, F.m20));
}

// Per-pair double-float constants of the close-pair contraction, relative to
// the test triangle's frame origin P_t: e_i = p0_i - P_t, f_j = p0_j - P_t,
// d_j = p0_j - P_s.  One per warp, in shared memory (every lane reads the same
// words).
struct NearPairDF {
  TriFrameDF Sf, Tf;        // source and test triangles
  df3 e[3], f[3], d[3];
  df3 sPs, v01t, v02t;      // P_s - P_t and the test triangle's edge vectors
  df Ai2;
  cdf ksq, k2, k2_3;
  float tol_eh, tol_plane, tol_edge;
};
// The nine L and K sums of a near pair (complex df).
struct NearAccDF {
  cdf L[9], K[9];
};

__device__ void near_pair_df_setup(const TriRec &T, const TriRec &S, const GreenDev &g, NearPairDF &pc) {
  const d3 Pt = ld3(T.p0), Ps = ld3(S.p0);
  tri_frame_df(S, Pt, pc.Sf);
  tri_frame_df(T, Pt, pc.Tf);
  for (int i = 0; i < 3; i++) {
    pc.e[i] = df3_make(i < T.nh ? ld3(T.hp0[i]) - Pt : d3{0, 0, 0});
    pc.f[i] = df3_make(i < S.nh ? ld3(S.hp0[i]) - Pt : d3{0, 0, 0});
    pc.d[i] = df3_make(i < S.nh ? ld3(S.hp0[i]) - Ps : d3{0, 0, 0});
  }
  pc.sPs = df3_make(Ps - Pt);
  pc.v01t = df3_make(ld3(T.v01));
  pc.v02t = df3_make(ld3(T.v02));
  pc.Ai2 = df_make(0.5 * S.Ai);
  pc.ksq = {{g.ksqr_f[0], g.ksqr_f[1]}, {g.ksqi_f[0], g.ksqi_f[1]}};
  pc.k2 = {{g.k2r_f[0], g.k2r_f[1]}, {g.k2i_f[0], g.k2i_f[1]}};
  pc.k2_3 = {df_make(BEM_ONETHIRD * g.k2r), df_make(BEM_ONETHIRD * g.k2i)};
  pc.tol_eh = (float)(1e-6 * S.elen0);
  pc.tol_plane = (float)(1e-8 * S.elen0);
  pc.tol_edge = (float)(1e-8 * T.elen0);
}

// One outer node of a near pair in double-float: given the node's smooth
// inner moments (near_inner_df), the analytic singular terms
// (tri_potentials_df) and the close-pair contraction of
// src/Impedance.cpp:194-250, added to acc.  rt1 is the node relative to P_t.
__device__ __noinline__ void near_outer_df(const InnerMomDF &m, const NearPairDF &pc, int nht, int nhs, df3 rt1,
                                           df wd, NearAccDF &acc) {
  const cdf I0 = m.I0, Q0 = m.Q0;
  const cdf3 A = m.A, Q1 = m.Q1;
  df ISn3h, ISn1, IS1, h;
  df3 IL1, IL3;
  tri_potentials_df(pc.Sf, rt1, pc.tol_eh, true, ISn3h, ISn1, IS1, IL1, IL3, h);
  // IL13 = Ai2 (k2/3 IL3 + IL1), ISn11 = Ai2 (ISn1 + k2 IS1), L2 = 2 ISn11 + I0
  cdf3 IL13 = cdf_v(pc.k2_3, IL3);
  IL13.x.r = df_add(IL13.x.r, IL1.x);
  IL13.y.r = df_add(IL13.y.r, IL1.y);
  IL13.z.r = df_add(IL13.z.r, IL1.z);
  IL13 = cdf3_scale(pc.Ai2, IL13);
  const cdf ISn11 = cdf_scale(pc.Ai2, cdf{df_add(ISn1, df_mul(pc.k2.r, IS1)), df_mul(pc.k2.i, IS1)});
  const cdf L2 = cdf_add(cdf_add(ISn11, ISn11), I0);
  const df half = {0.5f, 0.f};
  if (fabsf(h.hi) < pc.tol_plane) {
    for (int j = 0; j < nhs; j++) {
      const cdf3 Gphij = cdf3_scale(half, cdf3_sub(A, cdf_v(I0, pc.d[j])));
      const cdf3 K21 = cdf3_add(IL13, cdf_v(ISn11, df3_sub(rt1, pc.f[j])));
      const cdf3 GK = cdf3_add(Gphij, K21);
      for (int i = 0; i < nht; i++) {
        const df3 phi = df3_scale(half, df3_sub(rt1, pc.e[i]));
        const cdf t = cdf_sub(cdf_mul(pc.ksq, cdf_rdot(phi, GK)), L2);
        acc.L[i * 3 + j] = cdf_add(acc.L[i * 3 + j], cdf_scale(wd, t));
      }
    }
  } else {
    const df3 nS = pc.Sf.n;
    const df3 ISn3hn = df3_scale(df_mul(pc.Ai2, ISn3h), nS);
    const df3 rho1 = df3_sub(rt1, df3_scale(h, nS));
    const cdf Ai2k2 = cdf_scale(pc.Ai2, pc.k2);
    const cdf3 K31 = cdf_v(Ai2k2, df3_sub(IL1, df3_scale(df_mul(h, ISn1), nS)));
    for (int j = 0; j < nhs; j++) {
      const df3 rf = df3_sub(rt1, pc.f[j]);  // r_t - p0_j
      const cdf3 Gphij = cdf3_scale(half, cdf3_sub(A, cdf_v(I0, pc.d[j])));
      const cdf3 DGxphij = cdf3_scale(half, cdf_rcross(rf, cdf3_sub(Q1, cdf_v(Q0, pc.d[j]))));
      const cdf3 K21 = cdf3_add(IL13, cdf_v(ISn11, df3_sub(rho1, pc.f[j])));
      const cdf3 K41 = cdf_zcross(K31, rf);
      const cdf3 GK = cdf3_add(Gphij, K21);
      for (int i = 0; i < nht; i++) {
        const df3 phi = df3_scale(half, df3_sub(rt1, pc.e[i]));
        const cdf t = cdf_sub(cdf_mul(pc.ksq, cdf_rdot(phi, GK)), L2);
        acc.L[i * 3 + j] = cdf_add(acc.L[i * 3 + j], cdf_scale(wd, t));
        const df3 vx = df3_cross(df3_sub(pc.f[j], pc.e[i]), ISn3hn);  // (p0_j - p0_i) x ISn3hn
        cdf3 KK = cdf3_add(DGxphij, K41);
        KK.x.r = df_add(KK.x.r, vx.x);
        KK.y.r = df_add(KK.y.r, vx.y);
        KK.z.r = df_add(KK.z.r, vx.z);
        const cdf kk = cdf_rdot(phi, KK);
        acc.K[i * 3 + j] = cdf_sub(acc.K[i * 3 + j], cdf_scale(wd, kk));
      }
    }
  }
}

// The neighbour-edge K correction of src/Impedance.cpp:301-324 at one source
// edge node v (relative to P_t) in double-float: LKEdgeIntegral over the test
// triangle, then Ke[i] += w (IL1 + ISn1 (rho - p0_i)).
__device__ __noinline__ void near_edge_df(const NearPairDF &pc, int nht, df3 v, df w, df3 *Ke) {
  df ISn3h, ISn1, IS1, h;
  df3 IL1, IL3;
  tri_potentials_df(pc.Tf, v, pc.tol_edge, false, ISn3h, ISn1, IS1, IL1, IL3, h);
  const df3 rho = df3_sub(v, df3_scale(h, pc.Tf.n));
  for (int i = 0; i < nht; i++) {
    const df3 c = df3_add(IL1, df3_scale(ISn1, df3_sub(rho, pc.e[i])));
    Ke[i] = df3_add(Ke[i], df3_scale(w, c));
  }
}

__device__ __forceinline__ df warp_sum_df(df v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const df u = {__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)};
    v = df_add(v, u);
  }
  return v;
}

// DF: the smooth inner rule in double-float (near_inner_df), else FP64.
// The rest of one near pair in double-float once its nine L and K sums are in
// acc (spread over the warp's lanes): the warp sums, the neighbour-edge K
// correction of src/Impedance.cpp:301-324 (near_edge_df), and the scatter of
// the nine (c L, c K) into the half-pair blocks as float pairs.
__device__ __noinline__ void near_finish_df(const TriRec &T, const TriRec &S, int same, const NearPairDF &pc,
                                            const NearAccDF &acc, HalfPairBlock *H, int ntr) {
  const int lane = threadIdx.x & 31;
  const int nht = T.nh, nhs = S.nh;
  z1 L[9], K[9];
#pragma unroll
  for (int k = 0; k < 9; k++) {
    L[k] = {df_to_double(warp_sum_df(acc.L[k].r)), df_to_double(warp_sum_df(acc.L[k].i))};
    K[k] = {df_to_double(warp_sum_df(acc.K[k].r)), df_to_double(warp_sum_df(acc.K[k].i))};
  }
  if (!same) {
    df3 Kd[3][3];
    const df z = {0.f, 0.f};
#pragma unroll
    for (int e = 0; e < 3; e++)
#pragma unroll
      for (int i = 0; i < 3; i++) Kd[e][i] = {z, z, z};
    for (int idx = lane; idx < 45; idx += 32) {
      const int e = idx / 15, q = idx - e * 15;
      const df3 v0 = e == 0 ? pc.Sf.p0 : (e == 1 ? pc.Sf.p1 : pc.Sf.p2);
      const df3 v1 = e == 0 ? pc.Sf.v01 : (e == 1 ? pc.Sf.v12 : pc.Sf.v20);
      const df3 v = df3_add(v0, df3_scale(df_make(c_line15[q][0]), v1));
      near_edge_df(pc, nht, v, df_make(c_line15[q][1]), Kd[e]);
    }
    d3 Ke[3][3];
#pragma unroll
    for (int e = 0; e < 3; e++)
#pragma unroll
      for (int i = 0; i < 3; i++)
        Ke[e][i] = {df_to_double(warp_sum_df(Kd[e][i].x)), df_to_double(warp_sum_df(Kd[e][i].y)),
                    df_to_double(warp_sum_df(Kd[e][i].z))};
    const double c = 0.125 * T.Ai * S.Ai;
    const d3 m01 = ld3(S.m01), m12 = ld3(S.m12), m20 = ld3(S.m20);
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) {
        if (i >= nht || j >= nhs) continue;
        const d3 v = ld3(T.hp0[i]) - ld3(S.hp0[j]);
        K[i * 3 + j].r += c * (dot(cross(v, m01), Ke[0][i]) / S.nv01i + dot(cross(v, m12), Ke[1][i]) / S.nv12i +
                               dot(cross(v, m20), Ke[2][i]) / S.nv20i);
      }
  }
  if (lane < nht * nhs) {
    const int i = lane / nhs, j = lane - (lane / nhs) * nhs;
    z1 Lv = {0, 0}, Kv = {0, 0};
#pragma unroll
    for (int k = 0; k < 9; k++)
      if (k == i * 3 + j) { Lv = L[k]; Kv = K[k]; }
    const double c = scatter_coef(T, i, S, j);
    const z1 cL = zscale(c, Lv), cK = zscale(c, Kv);
    store_block_df(H, ntr, T.hrwg[i], T.hneg[i], S.hrwg[j], S.hneg[j], df_make(cL.r), df_make(cL.i), df_make(cK.r),
                   df_make(cK.i));
  }
}

// Near pairs in double-float, two pairs per warp: the 2 x 105 outer nodes of
// the pair couple are spread over the lanes in 7 rounds of 32 (94 % of the
// lanes busy, against 82 % for 105 nodes in 4 rounds); each lane adds to the
// sums of the pair its node belongs to, and the warp finishes the pairs one
// after the other.
// The pair couple (p0, p0 + 1) of `list` (one pair when p0 + 1 == npairs),
// worked by one warp in two parts: near_couple_df_sums runs the 2 x 105 outer
// nodes (inner rule, closed forms, contraction) into acc, near_couple_df_finish
// the warp sums, the neighbour-edge correction and the scatter.  nodes, pc:
// the warp's shared staging, outer: the outer rule in double-float.
struct NearCouple {
  NearPair npr[2];
  int np2;
  NearAccDF acc[2];
};

__device__ __forceinline__ void near_couple_df_sums(const TriRec *__restrict__ Tr, const TriRec *__restrict__ Sr,
                                                    const NearPair *__restrict__ list, int64_t npairs, int64_t p0,
                                                    const GreenDev &g, float (*nodes)[BEMGPU_TRI_RULE91_N][8],
                                                    const float (*outer)[6], NearPairDF *pcs, int lane,
                                                    NearCouple &cp) {
  const int np2 = p0 + 1 < npairs ? 2 : 1;
  cp.np2 = np2;
  NearPair *npr = cp.npr;
  npr[0] = list[p0];
  npr[1] = list[np2 == 2 ? p0 + 1 : p0];
  // inner nodes l = r_s - P_s and weights of both pairs, then their records
  for (int it = lane; it < np2 * BEMGPU_TRI_RULE91_N; it += 32) {
    const int k = it >= BEMGPU_TRI_RULE91_N ? 1 : 0, u = it - k * BEMGPU_TRI_RULE91_N;
    const TriRec &S = Sr[npr[k].s];
    const d3 l = c_rule91[u][0] * ld3(S.v01) + c_rule91[u][1] * ld3(S.v02);
    const double vals[4] = {l.x, l.y, l.z, c_rule91[u][2]};
#pragma unroll
    for (int c = 0; c < 4; c++) {
      const df v = df_make(vals[c]);
      nodes[k][u][2 * c] = v.hi;
      nodes[k][u][2 * c + 1] = v.lo;
    }
  }
  if (lane < np2) near_pair_df_setup(Tr[npr[lane].t], Sr[npr[lane].s], g, pcs[lane]);
  __syncwarp();
  NearAccDF *acc = cp.acc;
  const df z = {0.f, 0.f};
#pragma unroll
  for (int k = 0; k < 9; k++) {
    acc[0].L[k] = {z, z}; acc[0].K[k] = {z, z};
    acc[1].L[k] = {z, z}; acc[1].K[k] = {z, z};
  }
  for (int it = lane; it < np2 * BEMGPU_TRI_RULE105_N; it += 32) {
    const int k = it >= BEMGPU_TRI_RULE105_N ? 1 : 0, q = it - k * BEMGPU_TRI_RULE105_N;
    const NearPairDF &pc = pcs[k];
    const float *o = outer[q];
    const df xi1 = {o[0], o[1]}, xi2 = {o[2], o[3]}, wq = {o[4], o[5]};
    const df3 rt1 = df3_add(df3_scale(xi1, pc.v01t), df3_scale(xi2, pc.v02t));
    const df3 rs = df3_sub(rt1, pc.sPs);
    InnerMomDF mom;
    near_inner_df<1>(nodes[k], &rs, g, &mom);
    near_outer_df(mom, pc, Tr[npr[k].t].nh, Sr[npr[k].s].nh, rt1, wq, acc[k]);
  }
}

__device__ __forceinline__ void near_couple_df_finish(const TriRec *__restrict__ Tr, const TriRec *__restrict__ Sr,
                                                      HalfPairBlock *__restrict__ H, int ntr, const NearPairDF *pcs,
                                                      const NearCouple &cp) {
  for (int k = 0; k < cp.np2; k++)
    near_finish_df(Tr[cp.npr[k].t], Sr[cp.npr[k].s], cp.npr[k].same, pcs[k], cp.acc[k], H, ntr);
  __syncwarp();
}

__device__ __forceinline__ void stage_outer_df(float (*outer)[6]) {
  for (int u = threadIdx.x; u < BEMGPU_TRI_RULE105_N; u += blockDim.x)
    for (int c = 0; c < 3; c++) {
      const df v = df_make(c_rule105[u][c]);
      outer[u][2 * c] = v.hi;
      outer[u][2 * c + 1] = v.lo;
    }
  __syncthreads();
}

// A group of fills: the warps walk the group's pair couples (a task's couples
// are units [near0, near0 + ceil(nnear / 2)) of the group), each staging its
// task's Green's function in shared memory.  MINB: CTAs per SM that the
// register allocation must allow (2: ~250 registers; 3: 168; 4: 128 with
// spills), chosen by the context's tuning.
// Warp w of CTA b takes units b * NEAR_WARPS + w + k * (grid warps), k = 0, 1, ...
// SYNC: the CTA's warps meet at a barrier after the outer nodes of each unit
// and after its finish.  A pair couple runs several large code regions (the
// inner rule, the closed-form potentials, the edge correction); with two warps
// per scheduler, warps that have drifted into different regions stall on
// instruction fetch, which the barriers prevent.
// The units and their order per warp are the same either way.
template <int MINB, bool SYNC>
__global__ void __launch_bounds__(32 * NEAR_WARPS, MINB) near_pairs_df_group_kernel(const FillTask *__restrict__ tasks,
                                                                                    int ntask, int64_t units) {
  __shared__ __align__(16) float s_nodes[NEAR_WARPS][2][BEMGPU_TRI_RULE91_N][8];
  __shared__ float s_outer[BEMGPU_TRI_RULE105_N][6];
  __shared__ NearPairDF s_pc[NEAR_WARPS][2];
  __shared__ GreenDev s_g[NEAR_WARPS];
  const int lane = threadIdx.x & 31;
  const int wid = threadIdx.x >> 5;
  stage_outer_df(s_outer);
  const int64_t nw = (int64_t)gridDim.x * NEAR_WARPS;
  int cur = -1;
  for (int64_t base = (int64_t)blockIdx.x * NEAR_WARPS; base < units; base += nw) {
    const int64_t u = base + wid;
    const bool active = u < units;
    NearCouple cp;
    const FillTask *tk = nullptr;
    if (active) {
      const int i = task_of_near(tasks, ntask, u);
      tk = &tasks[i];
      if (i != cur) {
        if (lane == 0) s_g[wid] = tk->g;
        __syncwarp();
        cur = i;
      }
      near_couple_df_sums(tk->T, tk->S, tk->near, tk->nnear, 2 * (u - tk->near0), s_g[wid], s_nodes[wid], s_outer,
                          s_pc[wid], lane, cp);
    }
    // base is the same for the whole CTA: every warp meets both barriers
    if (SYNC) __syncthreads();
    if (active) near_couple_df_finish(tk->T, tk->S, tk->H, tk->ntr, s_pc[wid], cp);
    if (SYNC) __syncthreads();
  }
}

template <int MINB>
void launch_near_df(bool sync, int nb, cudaStream_t stream, const FillTask *tasks, int ntask, int64_t units) {
  if (sync)
    near_pairs_df_group_kernel<MINB, true><<<nb, 32 * NEAR_WARPS, 0, stream>>>(tasks, ntask, units);
  else
    near_pairs_df_group_kernel<MINB, false><<<nb, 32 * NEAR_WARPS, 0, stream>>>(tasks, ntask, units);
}

// Near pairs in FP64 (the plain path), one pair per warp: lanes take the
// outer nodes, each runs the 91-node smooth inner rule, the analytic singular
// terms and the close-pair contraction; the warp sums, adds the neighbour-edge
// K correction and scatters.
// Near pair p of `list` in FP64, worked by one warp (nodes: the warp's
// shared staging of the inner rule).
__device__ __forceinline__ void near_pair_fp64(const TriRec *__restrict__ Tr, const TriRec *__restrict__ Sr,
                                               const NearPair *__restrict__ list, int64_t p, const GreenDev &g,
                                               HalfPairBlock *__restrict__ H, int ntr, double (*nodes)[4], int lane) {
  const z1 ksq = {g.ksqr, g.ksqi};
  const z1 k2 = {g.k2r, g.k2i};
  const NearPair np = list[p];
  const TriRec &T = Tr[np.t];
  const TriRec &S = Sr[np.s];
  const d3 Pt = ld3(T.p0), Ps = ld3(S.p0);
  const d3 v01t = ld3(T.v01), v02t = ld3(T.v02);
  {
    const d3 v01s = ld3(S.v01), v02s = ld3(S.v02);
    for (int u = lane; u < BEMGPU_TRI_RULE91_N; u += 32) {
      const d3 l = c_rule91[u][0] * v01s + c_rule91[u][1] * v02s;
      nodes[u][0] = l.x; nodes[u][1] = l.y; nodes[u][2] = l.z;
      nodes[u][3] = c_rule91[u][2];
    }
  }
  __syncwarp();
  const int nht = T.nh, nhs = S.nh;
  d3 dj[3];
  for (int j = 0; j < 3; j++) dj[j] = (j < nhs) ? ld3(S.hp0[j]) - Ps : d3{0, 0, 0};
  z1 L[9], K[9];
#pragma unroll
  for (int k = 0; k < 9; k++) { L[k] = {0, 0}; K[k] = {0, 0}; }
  const d3 nS = ld3(S.n);
  const double Ai2 = 0.5 * S.Ai;
  for (int q = lane; q < BEMGPU_TRI_RULE105_N; q += 32) {
    const double w = c_rule105[q][2];
    const d3 rt = (Pt + c_rule105[q][0] * v01t) + c_rule105[q][1] * v02t;
    const d3 rts = rt - Ps;
    // LKSmoothInnerIntegrand over s[0] (src/Impedance.cpp:93-105) as moments
    z1 I0 = {0, 0}, Q0 = {0, 0};
    z3 A = z3zero(), Q1 = z3zero();
    for (int u = 0; u < BEMGPU_TRI_RULE91_N; u++) {
      const d3 l = {nodes[u][0], nodes[u][1], nodes[u][2]};
      const double ws = nodes[u][3];
      const d3 x = rts - l;
      const double R2 = dot(x, x);
      const double R = sqrt(R2);
      const z1 e = zexp_ikR(g, R);
      // scalar_gradient_smooth, src/GreensFunction.cpp:54-69
      const double Ri = 1.0 / R;
      const z1 gs = zsub(zscale(Ri, z1{e.r - 1.0, e.i}), zscale(R, k2));
      const z1 ikR = {g.ikr * R, g.iki * R};
      z1 num = zmul(e, z1{1.0 - ikR.r, -ikR.i});
      num = zadd(num, zscale(R2, k2));
      num.r -= 1.0;
      const z1 qq = zscale(Ri * Ri * Ri, num);
      const z1 gw = zscale(ws, gs), qw = zscale(ws, qq);
      zacc(I0, gw);
      A = z3add(A, zs_v(gw, l));
      zacc(Q0, qw);
      Q1 = z3add(Q1, zs_v(qw, l));
    }
    // LKCloseOuterIntegrand::weighPoint, src/Impedance.cpp:194-250
    double ISn3h, ISn1, IS1;
    d3 IL1, IL3;
    eh_nonsmooth(S, rt, ISn3h, ISn1, IS1, IL1, IL3);
    const z3 IL13 = z3scale(Ai2, z3add_r(zs_v(zscale(BEM_ONETHIRD, k2), IL3), IL1));
    z1 ISn11 = zscale(Ai2, z1{ISn1 + k2.r * IS1, k2.i * IS1});
    const double h = dot(rt - Ps, nS);
    const z1 L2 = zadd(zscale(2.0, ISn11), I0);
    if (fabs(h) < 1e-8 * S.elen0) {
#pragma unroll
      for (int j = 0; j < 3; j++) {
        if (j >= nhs) break;
        const z3 Gphij = z3scale(0.5, z3sub(A, zs_v(I0, dj[j])));
        const z3 K21 = z3add(IL13, zs_v(ISn11, rt - ld3(S.hp0[j])));
        const z3 GK = z3add(Gphij, K21);
#pragma unroll
        for (int i = 0; i < 3; i++) {
          if (i >= nht) break;
          const d3 phi = 0.5 * (rt - ld3(T.hp0[i]));
          const z1 t = zsub(zmul(ksq, rdot(phi, GK)), L2);
          zacc(L[i * 3 + j], zscale(w, t));
        }
      }
    } else {
      const d3 ISn3hn = (Ai2 * ISn3h) * nS;
      const d3 rho = rt - h * nS;
      const z1 Ai2k2 = zscale(Ai2, k2);
      const z3 K31 = zs_v(Ai2k2, IL1 - (h * ISn1) * nS);
#pragma unroll
      for (int j = 0; j < 3; j++) {
        if (j >= nhs) break;
        const d3 p0j = ld3(S.hp0[j]);
        const z3 Gphij = z3scale(0.5, z3sub(A, zs_v(I0, dj[j])));
        const z3 DGxphij = z3scale(0.5, rcross(rt - p0j, z3sub(Q1, zs_v(Q0, dj[j]))));
        const z3 K21 = z3add(IL13, zs_v(ISn11, rho - p0j));
        const z3 K41 = zcross(K31, rt - p0j);
        const z3 GK = z3add(Gphij, K21);
#pragma unroll
        for (int i = 0; i < 3; i++) {
          if (i >= nht) break;
          const d3 p0i = ld3(T.hp0[i]);
          const d3 phi = 0.5 * (rt - p0i);
          const z1 t = zsub(zmul(ksq, rdot(phi, GK)), L2);
          zacc(L[i * 3 + j], zscale(w, t));
          const d3 vts = p0j - p0i;
          const z3 KK = z3add(z3add_r(DGxphij, cross(vts, ISn3hn)), K41);
          const z1 kk = rdot(phi, KK);
          K[i * 3 + j].r -= w * kk.r;
          K[i * 3 + j].i -= w * kk.i;
        }
      }
    }
  }
#pragma unroll
  for (int k = 0; k < 9; k++) {
    L[k].r = warp_sum(L[k].r); L[k].i = warp_sum(L[k].i);
    K[k].r = warp_sum(K[k].r); K[k].i = warp_sum(K[k].i);
  }
  if (!np.same) {
    // neighbour-edge K correction, src/Impedance.cpp:301-324: three source
    // edges x QuadratureGauss15, LKNeighborEdgeIntegrand over t[0].
    d3 Ke[3][3];
#pragma unroll
    for (int e = 0; e < 3; e++)
#pragma unroll
      for (int i = 0; i < 3; i++) Ke[e][i] = {0, 0, 0};
    const d3 nT = ld3(T.n);
    for (int idx = lane; idx < 45; idx += 32) {
      const int e = idx / 15, q = idx - e * 15;
      const d3 v0 = e == 0 ? ld3(S.p0) : (e == 1 ? ld3(S.p1) : ld3(S.p2));
      const d3 v1 = e == 0 ? ld3(S.v01) : (e == 1 ? ld3(S.v12) : ld3(S.v20));
      const d3 v = v0 + c_line15[q][0] * v1;
      const double w = c_line15[q][1];
      double ISn1;
      d3 IL1;
      lk_edge_integral(T, v, ISn1, IL1);
      const double h = dot(v - Pt, nT);
      const d3 rho = v - h * nT;
#pragma unroll
      for (int i = 0; i < 3; i++) {
        if (i >= nht) break;
        const d3 c = IL1 + ISn1 * (rho - ld3(T.hp0[i]));
        if (e == 0) Ke[0][i] = Ke[0][i] + w * c;
        else if (e == 1) Ke[1][i] = Ke[1][i] + w * c;
        else Ke[2][i] = Ke[2][i] + w * c;
      }
    }
#pragma unroll
    for (int e = 0; e < 3; e++)
#pragma unroll
      for (int i = 0; i < 3; i++) {
        Ke[e][i].x = warp_sum(Ke[e][i].x);
        Ke[e][i].y = warp_sum(Ke[e][i].y);
        Ke[e][i].z = warp_sum(Ke[e][i].z);
      }
    const double c = 0.125 * T.Ai * S.Ai;
    const d3 m01 = ld3(S.m01), m12 = ld3(S.m12), m20 = ld3(S.m20);
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) {
        if (i >= nht || j >= nhs) continue;
        const d3 v = ld3(T.hp0[i]) - ld3(S.hp0[j]);
        K[i * 3 + j].r += c * (dot(cross(v, m01), Ke[0][i]) / S.nv01i + dot(cross(v, m12), Ke[1][i]) / S.nv12i +
                               dot(cross(v, m20), Ke[2][i]) / S.nv20i);
      }
  }
  if (lane < nht * nhs) {
    const int i = lane / nhs, j = lane - (lane / nhs) * nhs;
    z1 Lv = {0, 0}, Kv = {0, 0};
#pragma unroll
    for (int k = 0; k < 9; k++)
      if (k == i * 3 + j) { Lv = L[k]; Kv = K[k]; }
    const double c = scatter_coef(T, i, S, j);
    store_block(H, ntr, T.hrwg[i], T.hneg[i], S.hrwg[j], S.hneg[j], zscale(c, Lv), zscale(c, Kv));
  }
  __syncwarp();
}

__global__ void __launch_bounds__(32 * NEAR_WARPS) near_pairs_kernel(
    const TriRec *__restrict__ Tr, const TriRec *__restrict__ Sr, const NearPair *__restrict__ list, int64_t npairs,
    GreenDev g, HalfPairBlock *__restrict__ H, int ntr) {
  __shared__ double s_nodes[NEAR_WARPS][BEMGPU_TRI_RULE91_N][4];  // l = r_s - P_s (xyz), weight
  const int lane = threadIdx.x & 31;
  const int wid = threadIdx.x >> 5;
  for (int64_t p = (int64_t)blockIdx.x * NEAR_WARPS + wid; p < npairs; p += (int64_t)gridDim.x * NEAR_WARPS)
    near_pair_fp64(Tr, Sr, list, p, g, H, ntr, s_nodes[wid], lane);
}

// A group of fills in FP64: the warps walk the group's near pairs (a task's
// pairs are units [near0, near0 + nnear) of the group).
__global__ void __launch_bounds__(32 * NEAR_WARPS) near_pairs_group_kernel(const FillTask *__restrict__ tasks,
                                                                           int ntask, int64_t units) {
  __shared__ double s_nodes[NEAR_WARPS][BEMGPU_TRI_RULE91_N][4];
  __shared__ GreenDev s_g[NEAR_WARPS];
  const int lane = threadIdx.x & 31;
  const int wid = threadIdx.x >> 5;
  int cur = -1;
  for (int64_t u = (int64_t)blockIdx.x * NEAR_WARPS + wid; u < units; u += (int64_t)gridDim.x * NEAR_WARPS) {
    const int i = task_of_near(tasks, ntask, u);
    const FillTask &tk = tasks[i];
    if (i != cur) {
      if (lane == 0) s_g[wid] = tk.g;
      __syncwarp();
      cur = i;
    }
    near_pair_fp64(tk.T, tk.S, tk.near, u - tk.near0, s_g[wid], tk.H, tk.ntr, s_nodes[wid], lane);
  }
}

// ---------------- gather: half-pair blocks -> Z ----------------
struct ZDev {
  double zer, zei, zmr, zmi;  // Zeps, Zmu
};

template <bool DFH>
__device__ __forceinline__ void block_sum(const HalfPairBlock &b, z1 &sL, z1 &sK) {
  sL = {0, 0};
  sK = {0, 0};
  if (DFH) {
    // the four half-pair terms summed in double-float, widened once
    const float4 *p = reinterpret_cast<const float4 *>(b.v);
    df Lr = {0.f, 0.f}, Li = Lr, Kr = Lr, Ki = Lr;
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const float4 l = p[2 * k], kk = p[2 * k + 1];
      Lr = df_add(Lr, {l.x, l.y});
      Li = df_add(Li, {l.z, l.w});
      Kr = df_add(Kr, {kk.x, kk.y});
      Ki = df_add(Ki, {kk.z, kk.w});
    }
    sL = {df_to_double(Lr), df_to_double(Li)};
    sK = {df_to_double(Kr), df_to_double(Ki)};
    return;
  }
  const double2 *p = reinterpret_cast<const double2 *>(b.v);
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const double2 l = p[2 * k], kk = p[2 * k + 1];
    sL.r += l.x; sL.i += l.y;
    sK.r += kk.x; sK.i += kk.y;
  }
}

__device__ __forceinline__ void write_2x2(double *Z, int64_t ld, int i, int j, z1 Ze, z1 Zm, z1 sL, z1 sK) {
  // src/Impedance.cpp:378-381
  const z1 a = zmul(Ze, sL), d = zmul(Zm, sL);
  double2 *c0 = reinterpret_cast<double2 *>(Z + 2 * ((int64_t)2 * i + ld * (2 * (int64_t)j)));
  double2 *c1 = reinterpret_cast<double2 *>(Z + 2 * ((int64_t)2 * i + ld * (2 * (int64_t)j + 1)));
  c0[0] = make_double2(a.r, a.i);
  c0[1] = make_double2(-sK.r, -sK.i);
  c1[0] = make_double2(sK.r, sK.i);
  c1[1] = make_double2(d.r, d.i);
}

template <bool DFH>
__global__ void gather_z_kernel(const HalfPairBlock *__restrict__ H, int ntr, int nsr, ZDev z, double *Z, int64_t ld) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (i >= ntr) return;
  z1 sL, sK;
  block_sum<DFH>(H[(size_t)j * ntr + i], sL, sK);
  write_2x2(Z, ld, i, j, {z.zer, z.zei}, {z.zmr, z.zmi}, sL, sK);
}

// W = Z_ext + blockdiag(G1, G2) and the G blocks themselves (src/HeatTransfer.cpp:26-35).
template <bool DFH>
__global__ void gather_w_kernel(const HalfPairBlock *__restrict__ He, const HalfPairBlock *__restrict__ H1,
                                const HalfPairBlock *__restrict__ H2, int ns, int nt, ZDev ze, ZDev z1d, ZDev z2d,
                                double *W, int64_t ldw, double *G1, int64_t ld1, double *G2, int64_t ld2) {
  const int n = ns + nt;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (i >= n) return;
  z1 sL, sK;
  block_sum<DFH>(He[(size_t)j * n + i], sL, sK);
  z1 a = zmul({ze.zer, ze.zei}, sL), d = zmul({ze.zmr, ze.zmi}, sL), k = sK;
  const bool in1 = i < ns && j < ns, in2 = i >= ns && j >= ns;
  if (in1 || in2) {
    z1 gL, gK;
    const ZDev &zz = in1 ? z1d : z2d;
    const int li = in1 ? i : i - ns, lj = in1 ? j : j - ns, nn = in1 ? ns : nt;
    block_sum<DFH>((in1 ? H1 : H2)[(size_t)lj * nn + li], gL, gK);
    write_2x2(in1 ? G1 : G2, in1 ? ld1 : ld2, li, lj, {zz.zer, zz.zei}, {zz.zmr, zz.zmi}, gL, gK);
    const z1 ga = zmul({zz.zer, zz.zei}, gL), gd = zmul({zz.zmr, zz.zmi}, gL);
    a = zadd(a, ga);
    d = zadd(d, gd);
    k = zadd(k, gK);
  }
  double2 *c0 = reinterpret_cast<double2 *>(W + 2 * ((int64_t)2 * i + ldw * (2 * (int64_t)j)));
  double2 *c1 = reinterpret_cast<double2 *>(W + 2 * ((int64_t)2 * i + ldw * (2 * (int64_t)j + 1)));
  c0[0] = make_double2(a.r, a.i);
  c0[1] = make_double2(-k.r, -k.i);
  c1[0] = make_double2(k.r, k.i);
  c1[1] = make_double2(d.r, d.i);
}

void split_df(double x, float out[2]) {
  out[0] = (float)x;
  out[1] = (float)(x - (double)out[0]);
}

GreenDev to_dev(const bemgpu_green_t *g) {
  GreenDev d;
  d.ikr = g->ik[0]; d.iki = g->ik[1];
  d.k2r = g->k2[0]; d.k2i = g->k2[1];
  d.ksqr = g->ksquared[0]; d.ksqi = g->ksquared[1];
  split_df(d.ikr, d.ikr_f); split_df(d.iki, d.iki_f);
  split_df(d.k2r, d.k2r_f); split_df(d.k2i, d.k2i_f);
  split_df(d.ksqr, d.ksqr_f); split_df(d.ksqi, d.ksqi_f);
  return d;
}

ZDev to_zdev(const bemgpu_green_t *g) { return {g->Zeps[0], g->Zeps[1], g->Zmu[0], g->Zmu[1]}; }

bool g_tables_loaded[BEM_MAX_DEVICES] = {false};

std::mutex g_tables_mu;

int load_tables(bemgpu_ctx_s *ctx) {
  // once per device; contexts on several host threads (farm lanes) may race here
  if (ctx->device < 0 || ctx->device >= BEM_MAX_DEVICES)
    return bem_fail(ctx, BEMGPU_ERR_ARG, "device %d outside 0..%d", ctx->device, BEM_MAX_DEVICES - 1);
  std::lock_guard<std::mutex> lk(g_tables_mu);
  if (g_tables_loaded[ctx->device]) return BEMGPU_OK;
  BEM_CUDA_TRY(ctx, cudaMemcpyToSymbol(c_rule6, bemgpu_tri_rule6, sizeof(bemgpu_tri_rule6)));
  BEM_CUDA_TRY(ctx, cudaMemcpyToSymbol(c_rule10, bemgpu_tri_rule10, sizeof(bemgpu_tri_rule10)));
  BEM_CUDA_TRY(ctx, cudaMemcpyToSymbol(c_rule15, bemgpu_tri_rule15, sizeof(bemgpu_tri_rule15)));
  BEM_CUDA_TRY(ctx, cudaMemcpyToSymbol(c_rule21, bemgpu_tri_rule21, sizeof(bemgpu_tri_rule21)));
  BEM_CUDA_TRY(ctx, cudaMemcpyToSymbol(c_rule36, bemgpu_tri_rule36, sizeof(bemgpu_tri_rule36)));
  BEM_CUDA_TRY(ctx, cudaMemcpyToSymbol(c_rule91, bemgpu_tri_rule91, sizeof(bemgpu_tri_rule91)));
  BEM_CUDA_TRY(ctx, cudaMemcpyToSymbol(c_rule105, bemgpu_tri_rule105, sizeof(bemgpu_tri_rule105)));
  BEM_CUDA_TRY(ctx, cudaMemcpyToSymbol(c_line15, bemgpu_line_rule15, sizeof(bemgpu_line_rule15)));
  {
    auto split = [](const double (*rule)[3], int n, std::vector<float> &out) {
      out.resize(6 * (size_t)n);
      for (int i = 0; i < n; i++)
        for (int c = 0; c < 3; c++) {
          const float h = (float)rule[i][c];
          out[6 * i + 2 * c] = h;
          out[6 * i + 2 * c + 1] = (float)(rule[i][c] - (double)h);
        }
    };
    std::vector<float> v;
    split(bemgpu_tri_rule6, 6, v);
    BEM_CUDA_TRY(ctx, cudaMemcpyToSymbol(c_rdf6, v.data(), sizeof(float) * v.size()));
    split(bemgpu_tri_rule10, 10, v);
    BEM_CUDA_TRY(ctx, cudaMemcpyToSymbol(c_rdf10, v.data(), sizeof(float) * v.size()));
    split(bemgpu_tri_rule15, 15, v);
    BEM_CUDA_TRY(ctx, cudaMemcpyToSymbol(c_rdf15, v.data(), sizeof(float) * v.size()));
    split(bemgpu_tri_rule21, 21, v);
    BEM_CUDA_TRY(ctx, cudaMemcpyToSymbol(c_rdf21, v.data(), sizeof(float) * v.size()));
    split(bemgpu_tri_rule36, 36, v);
    BEM_CUDA_TRY(ctx, cudaMemcpyToSymbol(c_rdf36, v.data(), sizeof(float) * v.size()));
    split(bemgpu_tri_rule91, 91, v);
    BEM_CUDA_TRY(ctx, cudaMemcpyToSymbol(c_rdf91, v.data(), sizeof(float) * v.size()));
  }
  // the copies from host memory may return before they land: every stream
  // of the device reads the tables from now on
  BEM_CUDA_TRY(ctx, cudaDeviceSynchronize());
  g_tables_loaded[ctx->device] = true;
  return BEMGPU_OK;
}

}  // namespace

int bem_fill_group(bemgpu_ctx_s *ctx, FillJob *jobs, int njobs, const bemgpu_options_t *opt, int precision,
                   cudaStream_t stream) {
  if (njobs < 1) return BEMGPU_OK;
  int rc = load_tables(ctx);
  if (rc) return rc;
  const int mode = precision == BEMGPU_PREC_MIXED ? FILL_FP32_FAR : precision == BEMGPU_PREC_MIXED_LA ? FILL_DF : FILL_FP64;
  const FarOpts fo = {opt->farThresh6, opt->farThresh10, opt->farThresh15, opt->farThresh21};
  const int fr = ctx->tune.far_rows;
  std::vector<FillTask> tasks(njobs);
  std::vector<const NearList *> lists(njobs);
  size_t ndf = 0;
  for (int i = 0; i < njobs; i++) {
    lists[i] = bem_near_list(ctx, jobs[i].t, jobs[i].s);
    if (!lists[i]) return bem_fail(ctx, BEMGPU_ERR_OOM, "near list allocation failed");
    ndf += (size_t)jobs[i].t->ntri + jobs[i].s->ntri;
  }
  TriDF *df = nullptr;
  if (mode == FILL_DF) {
    df = (TriDF *)bem_workspace(ctx, "fill_tdf", sizeof(TriDF) * ndf);
    if (!df) return bem_fail(ctx, BEMGPU_ERR_OOM, "fill: double-float records");
  }
  FillTask *dtasks = (FillTask *)bem_workspace(ctx, "fill_tasks", sizeof(FillTask) * (size_t)njobs);
  if (!dtasks) return bem_fail(ctx, BEMGPU_ERR_OOM, "fill: task table");
  double far_flops = 0, far_bytes = 0, near_flops = 0, near_bytes = 0;
  int64_t far_tiles = 0, near_units = 0;
  size_t dfo = 0;
  for (int i = 0; i < njobs; i++) {
    const bemgpu_tree_s *t = jobs[i].t, *s = jobs[i].s;
    FillTask &tk = tasks[i];
    tk.T = t->d_rec;
    tk.S = s->d_rec;
    tk.TD = tk.SD = nullptr;
    if (df) {
      tk.TD = df + dfo;
      tk.SD = df + dfo + t->ntri;
      tri_df_kernel<<<(t->ntri + 127) / 128, 128, 0, stream>>>(t->d_rec, t->ntri, df + dfo);
      tri_df_kernel<<<(s->ntri + 127) / 128, 128, 0, stream>>>(s->d_rec, s->ntri, df + dfo + t->ntri);
      ctx->launches += 2;
      dfo += (size_t)t->ntri + s->ntri;
    }
    tk.near = lists[i]->d;
    tk.nnear = lists[i]->n;
    tk.H = jobs[i].H;
    tk.ntT = t->ntri;
    tk.ntS = s->ntri;
    tk.ntr = t->nrwg;
    tk.far_tx = (s->ntri + 31) / 32;
    tk.far0 = far_tiles;
    far_tiles += (int64_t)tk.far_tx * ((t->ntri + fr - 1) / fr);
    tk.near0 = near_units;
    near_units += mode == FILL_DF ? (tk.nnear + 1) / 2 : tk.nnear;  // the df kernel works pair couples
    tk.g = to_dev(&jobs[i].g);
    jobs[i].near = tk.nnear;
    jobs[i].far = (int64_t)t->ntri * s->ntri - tk.nnear;
    if (ctx->prof) {
      const int64_t *fc = bem_far_rule_counts(ctx, t, s, opt);
      const int P[5] = {6, 10, 15, 21, 36};
      int64_t nfar = 0;
      for (int k = 0; k < 5; k++) { far_flops += fc[k] * bem_far_pair_flops(P[k]); nfar += fc[k]; }
      // half-pair products written: 9 per pair on average (nh_t * nh_s)
      far_bytes += (double)nfar * 9.0 * BEM_HALFPAIR_BYTES_FP64;
      near_flops += (double)tk.nnear * bem_near_pair_flops(true);
      near_bytes += (double)tk.nnear * 9.0 * BEM_HALFPAIR_BYTES_FP64;
    }
  }
  // the table is copied from this call's host vector before the call returns
  BEM_CUDA_TRY(ctx, cudaMemcpyAsync(dtasks, tasks.data(), sizeof(FillTask) * (size_t)njobs, cudaMemcpyHostToDevice,
                                    stream));
  if (far_tiles > 0) {
    if (far_tiles > 0x7fffffffll) return bem_fail(ctx, BEMGPU_ERR_ARG, "fill: %lld far tiles", (long long)far_tiles);
    ProfScope ps(ctx, BEMGPU_K_FILL_FAR, stream, far_flops, far_bytes);
    far_pairs_group_kernel<<<(unsigned)far_tiles, dim3(32, fr), 0, stream>>>(dtasks, njobs, fo, mode);
    ctx->launches++;
  }
  BEM_CUDA_TRY(ctx, cudaGetLastError());
  if (near_units > 0) {
    const int nb = (int)std::min<int64_t>((near_units + NEAR_WARPS - 1) / NEAR_WARPS,
                                          (int64_t)ctx->num_sms * ctx->tune.near_grid);
    ProfScope ps(ctx, BEMGPU_K_FILL_NEAR, stream, near_flops, near_bytes);
    const bool sync = ctx->tune.near_sync != 0;
    if (mode == FILL_DF && ctx->tune.near_minb == 3)
      launch_near_df<3>(sync, nb, stream, dtasks, njobs, near_units);
    else if (mode == FILL_DF && ctx->tune.near_minb == 4)
      launch_near_df<4>(sync, nb, stream, dtasks, njobs, near_units);
    else if (mode == FILL_DF)
      launch_near_df<2>(sync, nb, stream, dtasks, njobs, near_units);
    else
      near_pairs_group_kernel<<<nb, 32 * NEAR_WARPS, 0, stream>>>(dtasks, njobs, near_units);
    ctx->launches++;
  }
  BEM_CUDA_TRY(ctx, cudaGetLastError());
  return BEMGPU_OK;
}

int bem_fill_pairs(bemgpu_ctx_s *ctx, const bemgpu_tree_s *t, const bemgpu_tree_s *s, const bemgpu_green_t *g,
                   const bemgpu_options_t *opt, int precision, HalfPairBlock *H, cudaStream_t stream,
                   int64_t *n_near, int64_t *n_far) {
  FillJob job = {t, s, *g, H, 0, 0};
  const int rc = bem_fill_group(ctx, &job, 1, opt, precision, stream);
  if (n_near) *n_near = job.near;
  if (n_far) *n_far = job.far;
  return rc;
}

int bem_gather_z(bemgpu_ctx_s *ctx, const HalfPairBlock *H, int ntr, int nsr, const bemgpu_green_t *g, double *Z,
                 int64_t ld, cudaStream_t stream, bool df) {
  dim3 blk(128);
  dim3 grd((ntr + 127) / 128, nsr);
  ProfScope ps(ctx, BEMGPU_K_GATHER, stream, (double)ntr * nsr * (6 * 8 + 2 * 6), (double)ntr * nsr * (128 + 64));
  if (df)
    gather_z_kernel<true><<<grd, blk, 0, stream>>>(H, ntr, nsr, to_zdev(g), Z, ld);
  else
    gather_z_kernel<false><<<grd, blk, 0, stream>>>(H, ntr, nsr, to_zdev(g), Z, ld);
  ctx->launches++;
  BEM_CUDA_TRY(ctx, cudaGetLastError());
  return BEMGPU_OK;
}

int bem_gather_w(bemgpu_ctx_s *ctx, const HalfPairBlock *Hext, const HalfPairBlock *H1, const HalfPairBlock *H2,
                 int ns, int nt, const bemgpu_green_t *gext, const bemgpu_green_t *g1, const bemgpu_green_t *g2,
                 double *W, int64_t ldw, double *G1, int64_t ld1, double *G2, int64_t ld2, cudaStream_t stream,
                 bool df) {
  dim3 blk(128);
  dim3 grd((ns + nt + 127) / 128, ns + nt);
  const double nn = (double)(ns + nt) * (ns + nt), nd = (double)ns * ns + (double)nt * nt;
  ProfScope ps(ctx, BEMGPU_K_GATHER, stream, nn * 60 + nd * 80, nn * 192 + nd * 192);
  if (df)
    gather_w_kernel<true><<<grd, blk, 0, stream>>>(Hext, H1, H2, ns, nt, to_zdev(gext), to_zdev(g1), to_zdev(g2), W,
                                                   ldw, G1, ld1, G2, ld2);
  else
    gather_w_kernel<false><<<grd, blk, 0, stream>>>(Hext, H1, H2, ns, nt, to_zdev(gext), to_zdev(g1), to_zdev(g2), W,
                                                    ldw, G1, ld1, G2, ld2);
  ctx->launches++;
  BEM_CUDA_TRY(ctx, cudaGetLastError());
  return BEMGPU_OK;
}

// ---------------- public Zts ----------------
extern "C" int bemgpu_zts(bemgpu_ctx_t ctx, bemgpu_tree_t t, bemgpu_tree_t s, const bemgpu_green_t *g,
                          const bemgpu_options_t *opt, int precision, void *dZ, int64_t ldz, void *stream) {
  if (!ctx || !t || !s || !g || !dZ) return bem_fail(ctx, BEMGPU_ERR_ARG, "zts: null argument");
  if (t->geom != s->geom) return bem_fail(ctx, BEMGPU_ERR_ARG, "zts: t and s must share one geometry");
  if (ldz < 2 * (int64_t)t->nrwg) return bem_fail(ctx, BEMGPU_ERR_ARG, "zts: ldz < 2*size(t)");
  if (precision != BEMGPU_PREC_FP64 && precision != BEMGPU_PREC_MIXED && precision != BEMGPU_PREC_MIXED_LA)
    return bem_fail(ctx, BEMGPU_ERR_ARG, "zts: unknown precision %d", precision);
  bemgpu_options_t o;
  if (opt) o = *opt; else bemgpu_options_default(&o);
  std::lock_guard<std::mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
  HalfPairBlock *H = (HalfPairBlock *)bem_workspace(ctx, "H0", sizeof(HalfPairBlock) * (size_t)t->nrwg * s->nrwg);
  if (!H) return bem_fail(ctx, BEMGPU_ERR_OOM, "zts: workspace allocation failed");
  int rc = bem_fill_pairs(ctx, t, s, g, &o, precision, H, st, nullptr, nullptr);
  if (rc) return rc;
  return bem_gather_z(ctx, H, t->nrwg, s->nrwg, g, (double *)dZ, ldz, st, precision == BEMGPU_PREC_MIXED_LA);
}

extern "C" int bemgpu_zts_host(bemgpu_ctx_t ctx, bemgpu_tree_t t, bemgpu_tree_t s, const bemgpu_green_t *g,
                               const bemgpu_options_t *opt, int precision, double *Z, int64_t ldz) {
  if (!ctx || !t || !s || !Z) return bem_fail(ctx, BEMGPU_ERR_ARG, "zts_host: null argument");
  const int64_t m = 2 * (int64_t)t->nrwg, n = 2 * (int64_t)s->nrwg;
  if (ldz < m) return bem_fail(ctx, BEMGPU_ERR_ARG, "zts_host: ldz < 2*size(t)");
  double *dZ = nullptr;
  {
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    dZ = (double *)bem_workspace(ctx, "Zhost", sizeof(double) * 2 * m * n);
    if (!dZ) return bem_fail(ctx, BEMGPU_ERR_OOM, "zts_host: workspace allocation failed");
  }
  int rc = bemgpu_zts(ctx, t, s, g, opt, precision, dZ, m, nullptr);
  if (rc) return rc;
  std::lock_guard<std::mutex> lk(ctx->mu);
  BEM_CUDA_TRY(ctx, cudaMemcpy2DAsync(Z, sizeof(double) * 2 * ldz, dZ, sizeof(double) * 2 * m, sizeof(double) * 2 * m,
                                      n, cudaMemcpyDeviceToHost, ctx->stream));
  BEM_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return BEMGPU_OK;
}

// ---------------- Zts without device allocation ----------------
//
// For callers that must not allocate device memory while they run: a solver
// loop with a latency budget that cannot stall in cudaMalloc (which may
// synchronise the device), or a host application whose own memory pool has
// claimed the device memory, so that a library allocation would fail or
// break its accounting.  bemgpu_zts_noalloc does the same FP64 fill as
// bemgpu_zts into the caller's buffer, but keeps its scratch (the half-pair
// blocks and the near-pair list) in one file-scope device array of fixed
// size, created when the library's module is loaded on a GPU and held until
// the process exits.
//
// What each call still does on the host: it builds the near-pair list of
// (t, s) in host memory (a std::vector), copies it into the scratch with
// cudaMemcpyAsync on the caller's stream and synchronises that stream before
// returning, since the host copy belongs to the call.  The first call on a
// device also does that device's set-up: cudaGetSymbolAddress of the scratch
// and, if no other fill ran there yet, the upload of the quadrature tables
// (cudaMemcpyToSymbol); make that first call before any stream capture.
namespace {

constexpr size_t NOALLOC_SCRATCH_BYTES = 32u << 20;   // 32 MiB
constexpr size_t NOALLOC_NEAR_BYTES = 2u << 20;       // first 2 MiB: the near-pair list
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

std::mutex g_noalloc_mu;
std::mutex g_noalloc_run_mu;  // one call at a time uses the shared scratch
void *g_noalloc_addr[BEM_MAX_DEVICES] = {nullptr};

}  // namespace

extern "C" int bemgpu_zts_noalloc(bemgpu_ctx_t ctx, bemgpu_tree_t t, bemgpu_tree_t s, const bemgpu_green_t *g,
                                  const bemgpu_options_t *opt, void *dZ, int64_t ldz, void *stream) {
  if (!ctx || !t || !s || !g || !dZ) return bem_fail(ctx, BEMGPU_ERR_ARG, "zts_noalloc: null argument");
  if (t->geom != s->geom) return bem_fail(ctx, BEMGPU_ERR_ARG, "zts_noalloc: t and s must share one geometry");
  if (ldz < 2 * (int64_t)t->nrwg) return bem_fail(ctx, BEMGPU_ERR_ARG, "zts_noalloc: ldz < 2*size(t)");
  if (ctx->device < 0 || ctx->device >= BEM_MAX_DEVICES)
    return bem_fail(ctx, BEMGPU_ERR_ARG, "zts_noalloc: device %d outside 0..%d", ctx->device, BEM_MAX_DEVICES - 1);
  const size_t hbytes = sizeof(HalfPairBlock) * (size_t)t->nrwg * (size_t)s->nrwg;
  if (hbytes > NOALLOC_SCRATCH_BYTES - NOALLOC_NEAR_BYTES)
    return bem_fail(ctx, BEMGPU_ERR_ARG,
                    "zts_noalloc: %d x %d RWGs need %zu bytes of scratch, the fixed scratch holds %zu "
                    "(at most size(t) * size(s) = %zu)",
                    t->nrwg, s->nrwg, hbytes, NOALLOC_SCRATCH_BYTES - NOALLOC_NEAR_BYTES,
                    (NOALLOC_SCRATCH_BYTES - NOALLOC_NEAR_BYTES) / sizeof(HalfPairBlock));
  std::vector<NearPair> pairs;
  bem_build_near_pairs(t, s, pairs);
  if (pairs.size() * sizeof(NearPair) > NOALLOC_NEAR_BYTES)
    return bem_fail(ctx, BEMGPU_ERR_ARG, "zts_noalloc: %zu near pairs exceed the fixed scratch (%zu)", pairs.size(),
                    NOALLOC_NEAR_BYTES / sizeof(NearPair));
  bemgpu_options_t o;
  if (opt) o = *opt; else bemgpu_options_default(&o);
  std::lock_guard<std::mutex> lk(ctx->mu);
  // the scratch is one array per process: calls from several contexts take
  // turns (each call ends with its stream synchronised)
  std::lock_guard<std::mutex> lkrun(g_noalloc_run_mu);
  cudaSetDevice(ctx->device);
  // Set-up, once per device with that device current: the host-side name of
  // the array is not a device address; ask the runtime for the address.
  unsigned char *base = nullptr;
  {
    std::lock_guard<std::mutex> lk2(g_noalloc_mu);
    if (!g_noalloc_addr[ctx->device]) {
      void *p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess || !p)
        return bem_fail(ctx, BEMGPU_ERR_CUDA, "zts_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
      g_noalloc_addr[ctx->device] = p;
    }
    base = (unsigned char *)g_noalloc_addr[ctx->device];
  }
  int rc = load_tables(ctx);
  if (rc) return rc;
  cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
  NearPair *dnear = reinterpret_cast<NearPair *>(base);
  HalfPairBlock *H = reinterpret_cast<HalfPairBlock *>(base + NOALLOC_NEAR_BYTES);
  if (!pairs.empty())
    BEM_CUDA_TRY(ctx, cudaMemcpyAsync(dnear, pairs.data(), pairs.size() * sizeof(NearPair), cudaMemcpyHostToDevice, st));
  // Every half-pair slot of H has exactly one writer (the pair kernels below),
  // so nothing left by an earlier call needs clearing.
  const GreenDev gd = to_dev(g);
  const FarOpts fo = {o.farThresh6, o.farThresh10, o.farThresh15, o.farThresh21};
  dim3 blk(32, 4);
  dim3 grd((s->ntri + 31) / 32, (t->ntri + 3) / 4);
  far_pairs_kernel<<<grd, blk, 0, st>>>(t->d_rec, t->ntri, s->d_rec, s->ntri, gd, fo, H, t->nrwg, FILL_FP64, nullptr,
                                        nullptr);
  ctx->launches++;
  if (!pairs.empty()) {
    const int64_t np = (int64_t)pairs.size();
    const int nb = (int)std::min<int64_t>((np + NEAR_WARPS - 1) / NEAR_WARPS, (int64_t)ctx->num_sms * 16);
    near_pairs_kernel<<<nb, 32 * NEAR_WARPS, 0, st>>>(t->d_rec, s->d_rec, dnear, np, gd, H, t->nrwg);
    ctx->launches++;
  }
  dim3 gblk(128);
  dim3 ggrd((t->nrwg + 127) / 128, s->nrwg);
  gather_z_kernel<false><<<ggrd, gblk, 0, st>>>(H, t->nrwg, s->nrwg, to_zdev(g), (double *)dZ, ldz);
  ctx->launches++;
  BEM_CUDA_TRY(ctx, cudaGetLastError());
  // The near-pair list was copied from host memory owned by this call.
  BEM_CUDA_TRY(ctx, cudaStreamSynchronize(st));
  return BEMGPU_OK;
}
