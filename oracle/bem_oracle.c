/*
 * ORACLE — test infrastructure only.  A plain-C restatement of the reference's
 * (claytonotey/bem) PMCHWT impedance fill, used by tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg as the checker.  Nothing in the product links,
 * imports or calls this file.
 *
 * It follows the reference step by step, in the reference's own loop structure
 * (per half-RWG pair contractions, the same quadrature rules, the same rule
 * selection), so that it checks the GPU kernels' restructured arithmetic rather
 * than sharing it.  Pinned against the reference binary built by
 * oracle/Makefile.ref (tests/test_oracle_pin.py, tests/golden/).
 *
 * Geometry is one shared index space (vertices + triangles); a "tree" is an RWG
 * table {pos triangle, neg triangle, edge vertex 1, edge vertex 2} whose row
 * order is the matrix order.  Zts(t, s) fills rows from t's RWGs and columns
 * from s's RWGs (src/Impedance.cpp:388-413).
 */
#include <complex.h>
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../bem_gb300/csrc/quadrature_tables.h"

typedef double complex cplx;
typedef struct { double x, y, z; } vec3;
typedef struct { cplx x, y, z; } cvec3;

/* src/util/MathUtils.h:16,33 */
#define ONETHIRD 0.33333333333333333333333333333333
#define ONEOVER4PI 0.079577471545947667884441881686257

/* ---- value-type semantics of src/util/Vector3.h and ComplexVector3.h ---- */
static inline vec3 v3(double x, double y, double z) { vec3 r = {x, y, z}; return r; }
static inline vec3 vadd(vec3 a, vec3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline vec3 vsub(vec3 a, vec3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline vec3 vscale(double c, vec3 a) { return v3(c * a.x, c * a.y, c * a.z); }
/* operator* on two Vector3 is the cross product (Vector3.h:86-89) */
static inline vec3 vcross(vec3 a, vec3 b) {
  return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
/* norm() is the squared length (Vector3.h:91-93) */
static inline double vnorm(vec3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
static inline double vdot(vec3 a, vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline vec3 vnormalized(vec3 a) {
  double ni = 1. / sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
  return v3(a.x * ni, a.y * ni, a.z * ni);
}
static inline cvec3 cv3(cplx x, cplx y, cplx z) { cvec3 r = {x, y, z}; return r; }
static inline cvec3 cvzero(void) { return cv3(0, 0, 0); }
static inline cvec3 cvadd(cvec3 a, cvec3 b) { return cv3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline cvec3 cvadd_r(cvec3 a, vec3 b) { return cv3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline cvec3 cvscale(cplx c, vec3 a) { return cv3(c * a.x, c * a.y, c * a.z); }
static inline cvec3 cvscalec(cplx c, cvec3 a) { return cv3(c * a.x, c * a.y, c * a.z); }
/* ComplexVector3 x Vector3 cross product (ComplexVector3.h:106-109) */
static inline cvec3 cvcross(cvec3 a, vec3 b) {
  return cv3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
/* dot(Vector3, ComplexVector3) does not conjugate (ComplexVector3.h:124-126) */
static inline cplx cvdot(vec3 a, cvec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

/* ---- GreensFunction (src/GreensFunction.cpp:17-69) ---- */
typedef struct {
  cplx eps, mu, omega, ksquared, k, ik, k2, Zeps, Zmu;
} green_t;

/* GreensFunction::init, src/GreensFunction.cpp:17-30 */
static void green_init(green_t *g, cplx eps, cplx mu, cplx omega) {
  g->eps = eps;
  g->mu = mu;
  g->omega = omega;
  g->ksquared = eps * mu * omega * omega;
  g->k = csqrt(g->ksquared);
  g->ik = I * g->k;
  g->k2 = -0.5 * g->ksquared;
  g->Zeps = 1. / (I * omega * eps);
  g->Zmu = 1. / (I * omega * mu);
}

/* GreensFunction::scalar_gradient, src/GreensFunction.cpp:41-52 */
static inline void scalar_gradient(const green_t *g, vec3 rt, vec3 rs, cplx *gs, cvec3 *gg) {
  double x = rt.x - rs.x, y = rt.y - rs.y, z = rt.z - rs.z;
  double R2 = x * x + y * y + z * z;
  double R = sqrt(R2);
  cplx ikR = g->ik * R;
  *gs = cexp(ikR) / R;
  cplx q = *gs * (1. - ikR) / R2;
  *gg = cv3(q * x, q * y, q * z);
}

/* GreensFunction::scalar_gradient_smooth, src/GreensFunction.cpp:54-69 */
static inline void scalar_gradient_smooth(const green_t *g, vec3 rt, vec3 rs, cplx *gs, cvec3 *gg) {
  double x = rt.x - rs.x, y = rt.y - rs.y, z = rt.z - rs.z;
  double R2 = x * x + y * y + z * z;
  double R = sqrt(R2);
  cplx ikR = g->ik * R;
  cplx expikR = cexp(ikR);
  *gs = (expikR - 1.0) / R - g->k2 * R;
  double R3 = R2 * R;
  cplx q = (expikR * (1.0 - ikR) + g->k2 * R2 - 1.0) / R3;
  *gg = cv3(q * x, q * y, q * z);
}

/* ---- HalfRWG, src/RWG.h:9-23, src/RWG.cpp:7-39 ---- */
typedef struct {
  vec3 p0, p1, p2, v01, v12, v20, v02, n, m01, m12, m20;
  double normv01i, normv12i, normv20i, Ai, elen;
  int rwg, positive;
} half_t;

typedef struct {
  int nh;
  half_t h[3]; /* in the order Zts pushes them: by RWG index, pos before neg */
} tri_halves_t;

typedef struct {
  const double *xyz;
  const int *tri;
  int nv, nt;
} geom_t;

static inline vec3 vtx(const geom_t *G, int i) { return v3(G->xyz[3 * i], G->xyz[3 * i + 1], G->xyz[3 * i + 2]); }

/* HalfRWG::HalfRWG: p0 is the triangle vertex off the edge, p1/p2 follow the
 * triangle's own vertex cycle (src/RWG.cpp:9-21 with the edge wiring of
 * src/ShapeMesh.cpp:867-928). */
static void half_init(half_t *h, const geom_t *G, int t, int ev1, int ev2, int positive, int rwg) {
  const int *tv = G->tri + 3 * t;
  int r;
  if (tv[0] != ev1 && tv[0] != ev2) r = 0;
  else if (tv[1] != ev1 && tv[1] != ev2) r = 1;
  else r = 2;
  h->p0 = vtx(G, tv[r]);
  h->p1 = vtx(G, tv[(r + 1) % 3]);
  h->p2 = vtx(G, tv[(r + 2) % 3]);
  h->v01 = vsub(h->p1, h->p0);
  h->v12 = vsub(h->p2, h->p1);
  h->v20 = vsub(h->p0, h->p2);
  h->v02 = vsub(h->p2, h->p0);
  h->normv01i = 1. / sqrt(vnorm(h->v01));
  h->normv12i = 1. / sqrt(vnorm(h->v12));
  h->normv20i = 1. / sqrt(vnorm(h->v20));
  vec3 n = vcross(h->v01, h->v02);
  double A2 = sqrt(vnorm(n));
  h->n = vscale(1. / A2, n);
  h->Ai = 2.0 / A2;
  h->m01 = vnormalized(vcross(h->v01, h->n));
  h->m12 = vnormalized(vcross(h->v12, h->n));
  h->m20 = vnormalized(vcross(h->v20, h->n));
  /* Edge::length, src/ShapeMesh.cpp:938-943 */
  h->elen = sqrt(vnorm(vsub(vtx(G, ev2), vtx(G, ev1))));
  h->rwg = rwg;
  h->positive = positive;
}

/* ---- analytic potential integrals ---- */

/* EHNonSmoothIntegral, src/Source.cpp:16-86 */
static void eh_nonsmooth(const half_t *sh, vec3 rt, double *ISn3h, double *ISn1, double *IS1,
                         vec3 *ILn1, vec3 *IL1, vec3 *IL3) {
  double tol = 1e-6 * sh->elen;
  vec3 p0 = vsub(rt, sh->p0), p1 = vsub(rt, sh->p1), p2 = vsub(rt, sh->p2);
  double R02 = vnorm(p0), R0 = sqrt(R02);
  double R12 = vnorm(p1), R1 = sqrt(R12);
  double R22 = vnorm(p2), R2 = sqrt(R22);
  vec3 a0 = vscale(1. / R0, p0), a1 = vscale(1. / R1, p1), a2 = vscale(1. / R2, p2);
  vec3 n = sh->n;
  double x = 1.0 + vdot(a0, vadd(a1, a2)) + vdot(a1, a2);
  double tp = vdot(a0, vcross(a1, a2));
  double y = sqrt(tp * tp);
  double h = vdot(p0, n);
  *ISn3h = (h < 0. ? -2. : 2.) * atan2(y, x);
  double num, den;
  double s010 = sh->normv01i * vdot(sh->v01, p0);
  double s011 = sh->normv01i * vdot(sh->v01, p1);
  num = (R1 - s011); den = (R0 - s010);
  double ILn1_01 = fabs(num) < tol || fabs(den) < tol ? 0. : log(num / den);
  double s121 = sh->normv12i * vdot(sh->v12, p1);
  double s122 = sh->normv12i * vdot(sh->v12, p2);
  num = (R2 - s122); den = (R1 - s121);
  double ILn1_12 = fabs(num) < tol || fabs(den) < tol ? 0. : log(num / den);
  double s202 = sh->normv20i * vdot(sh->v20, p2);
  double s200 = sh->normv20i * vdot(sh->v20, p0);
  num = (R0 - s200); den = (R2 - s202);
  double ILn1_20 = fabs(num) < tol || fabs(den) < tol ? 0. : log(num / den);
  double t01 = vdot(sh->m01, p0), t12 = vdot(sh->m12, p1), t20 = vdot(sh->m20, p2);
  *ISn1 = -h * *ISn3h - (t01 * ILn1_01 + t12 * ILn1_12 + t20 * ILn1_20);
  double R02_01 = (R02 - s010 * s010);
  double IL1_01 = 0.5 * (R02_01 * ILn1_01 - (R1 * s011 - R0 * s010));
  double R02_12 = (R12 - s121 * s121);
  double IL1_12 = 0.5 * (R02_12 * ILn1_12 - (R2 * s122 - R1 * s121));
  double R02_20 = (R22 - s202 * s202);
  double IL1_20 = 0.5 * (R02_20 * ILn1_20 - (R0 * s200 - R2 * s202));
  double IL3_01 = 0.75 * R02_01 * IL1_01 - 0.25 * (R12 * R1 * s011 - R02 * R0 * s010);
  double IL3_12 = 0.75 * R02_12 * IL1_12 - 0.25 * (R22 * R2 * s122 - R12 * R1 * s121);
  double IL3_20 = 0.75 * R02_20 * IL1_20 - 0.25 * (R02 * R0 * s200 - R22 * R2 * s202);
  *IS1 = ONETHIRD * (h * h * *ISn1 - (t01 * IL1_01 + t12 * IL1_12 + t20 * IL1_20));
  *ILn1 = vadd(vadd(vscale(ILn1_01, sh->m01), vscale(ILn1_12, sh->m12)), vscale(ILn1_20, sh->m20));
  *IL1 = vadd(vadd(vscale(IL1_01, sh->m01), vscale(IL1_12, sh->m12)), vscale(IL1_20, sh->m20));
  *IL3 = vadd(vadd(vscale(IL3_01, sh->m01), vscale(IL3_12, sh->m12)), vscale(IL3_20, sh->m20));
}

/* LKEdgeIntegral, src/Impedance.cpp:13-73 (note tol = 1e-8 * length here) */
static void lk_edge_integral(const half_t *th, vec3 rs, double *ISn1, vec3 *IL1) {
  vec3 p0 = vsub(rs, th->p0), p1 = vsub(rs, th->p1), p2 = vsub(rs, th->p2);
  double R02 = vnorm(p0), R0 = sqrt(R02);
  double R12 = vnorm(p1), R1 = sqrt(R12);
  double R22 = vnorm(p2), R2 = sqrt(R22);
  double tol = 1e-8 * th->elen;
  vec3 a0 = vscale(1. / R0, p0), a1 = vscale(1. / R1, p1), a2 = vscale(1. / R2, p2);
  double h = vdot(p0, th->n);
  double x = 1.0 + vdot(a0, vadd(a1, a2)) + vdot(a1, a2);
  double tp = vdot(a0, vcross(a1, a2));
  double y = sqrt(tp * tp);
  double ISn3h = (h < 0 ? -2. : 2.) * atan2(y, x);
  double t01 = vdot(th->m01, p0), t12 = vdot(th->m12, p1), t20 = vdot(th->m20, p2);
  double s010 = th->normv01i * vdot(th->v01, p0);
  double s011 = th->normv01i * vdot(th->v01, p1);
  double num, den;
  num = (R1 - s011); den = (R0 - s010);
  double ILn1_01 = fabs(num) < tol || fabs(den) < tol ? 0. : log(num / den);
  double s121 = th->normv12i * vdot(th->v12, p1);
  double s122 = th->normv12i * vdot(th->v12, p2);
  num = (R2 - s122); den = (R1 - s121);
  double ILn1_12 = fabs(num) < tol || fabs(den) < tol ? 0. : log(num / den);
  double s202 = th->normv20i * vdot(th->v20, p2);
  double s200 = th->normv20i * vdot(th->v20, p0);
  num = (R0 - s200); den = (R2 - s202);
  double ILn1_20 = fabs(num) < tol || fabs(den) < tol ? 0. : log(num / den);
  *ISn1 = -h * ISn3h - (t01 * ILn1_01 + t12 * ILn1_12 + t20 * ILn1_20);
  double R02_01 = (R02 - s010 * s010);
  double IL1_01 = 0.5 * (R02_01 * ILn1_01 - (R1 * s011 - R0 * s010));
  double R02_12 = (R12 - s121 * s121);
  double IL1_12 = 0.5 * (R02_12 * ILn1_12 - (R2 * s122 - R1 * s121));
  double R02_20 = (R22 - s202 * s202);
  double IL1_20 = 0.5 * (R02_20 * ILn1_20 - (R0 * s200 - R2 * s202));
  *IL1 = vadd(vadd(vscale(IL1_01, th->m01), vscale(IL1_12, th->m12)), vscale(IL1_20, th->m20));
}

/* ---- integrands (src/Impedance.cpp:75-274) ---- */

/* LKInnerIntegrand / LKSmoothInnerIntegrand state (src/Impedance.cpp:75-139) */
typedef struct {
  cplx G;
  cvec3 Gphi[3], DGxphi[3];
} inner_acc_t;

/* TriangleQuadrature::integrate of an inner integrand over the source
 * triangle s[0] for a fixed test point (src/Impedance.cpp:93-105, 126-138). */
static void inner_integrate(const green_t *g, int smooth, const double (*rule)[3], int nr,
                            const tri_halves_t *s, vec3 rt, inner_acc_t *acc) {
  const half_t *sh = &s->h[0];
  acc->G = 0.0;
  for (int i = 0; i < 3; i++) { acc->Gphi[i] = cvzero(); acc->DGxphi[i] = cvzero(); }
  for (int q = 0; q < nr; q++) {
    vec3 v = vadd(vadd(sh->p0, vscale(rule[q][0], sh->v01)), vscale(rule[q][1], sh->v02));
    double w = rule[q][2];
    cplx gs;
    cvec3 gg;
    if (smooth) scalar_gradient_smooth(g, rt, v, &gs, &gg);
    else scalar_gradient(g, rt, v, &gs, &gg);
    gs *= w;
    gg = cvscalec(w, gg);
    acc->G += gs;
    for (int i = 0; i < s->nh; i++) {
      vec3 phi = vscale(0.5, vsub(v, s->h[i].p0));
      acc->Gphi[i] = cvadd(acc->Gphi[i], cvscale(gs, phi));
      acc->DGxphi[i] = cvadd(acc->DGxphi[i], cvcross(gg, phi));
    }
  }
}

/* LKFarOuterIntegrand::weighPoint, src/Impedance.cpp:154-168 */
static void far_outer_point(const green_t *g, const double (*rule)[3], int nr, const tri_halves_t *t,
                            const tri_halves_t *s, double w, vec3 v, cplx *L, cplx *K) {
  inner_acc_t in;
  inner_integrate(g, 0, rule, nr, s, v, &in);
  int ij = 0;
  for (int i = 0; i < t->nh; i++) {
    vec3 phi = vscale(0.5, vsub(v, t->h[i].p0));
    for (int j = 0; j < s->nh; j++) {
      L[ij] += w * (g->ksquared * cvdot(phi, in.Gphi[j]) - in.G);
      K[ij] -= w * cvdot(phi, in.DGxphi[j]);
      ij++;
    }
  }
}

/* LKCloseOuterIntegrand::weighPoint, src/Impedance.cpp:194-250 */
static void close_outer_point(const green_t *g, const tri_halves_t *t, const tri_halves_t *s,
                              const vec3 *vts, double w, vec3 v, cplx *L, cplx *K) {
  inner_acc_t in;
  inner_integrate(g, 1, bemgpu_tri_rule91, BEMGPU_TRI_RULE91_N, s, v, &in);
  const half_t *sh = &s->h[0];
  double ISn3h, ISn1, IS1;
  vec3 ILn1, IL1, IL3;
  eh_nonsmooth(sh, v, &ISn3h, &ISn1, &IS1, &ILn1, &IL1, &IL3);
  cplx k2 = g->k2;
  double Ai = sh->Ai;
  double Ai2 = 0.5 * Ai;
  cvec3 IL13 = cvscalec(Ai2, cvadd_r(cvscale(ONETHIRD * k2, IL3), IL1));
  cplx ISn11 = Ai2 * (ISn1 + k2 * IS1);
  vec3 n = sh->n;
  double h = vdot(vsub(v, sh->p0), n);
  if (fabs(h) < 1e-8 * sh->elen) {
    cvec3 K21[3];
    for (int j = 0; j < s->nh; j++) K21[j] = cvadd(IL13, cvscale(ISn11, vsub(v, s->h[j].p0)));
    cplx L2 = 2.0 * ISn11 + in.G;
    int ij = 0;
    for (int i = 0; i < t->nh; i++) {
      vec3 phi = vscale(0.5, vsub(v, t->h[i].p0));
      for (int j = 0; j < s->nh; j++) {
        L[ij] += w * (g->ksquared * cvdot(phi, cvadd(in.Gphi[j], K21[j])) - L2);
        ij++;
      }
    }
  } else {
    vec3 ISn3hn = vscale(Ai2 * ISn3h, n);
    cvec3 K21[3], K41[3];
    vec3 rho = vsub(v, vscale(h, n));
    cvec3 K31 = cvscale(Ai2 * k2, vsub(IL1, vscale(h * ISn1, n)));
    for (int j = 0; j < s->nh; j++) {
      K21[j] = cvadd(IL13, cvscale(ISn11, vsub(rho, s->h[j].p0)));
      K41[j] = cvcross(K31, vsub(v, s->h[j].p0));
    }
    cplx L2 = 2.0 * ISn11 + in.G;
    int ij = 0;
    for (int i = 0; i < t->nh; i++) {
      vec3 phi = vscale(0.5, vsub(v, t->h[i].p0));
      for (int j = 0; j < s->nh; j++) {
        L[ij] += w * (g->ksquared * cvdot(phi, cvadd(in.Gphi[j], K21[j])) - L2);
        K[ij] -= w * cvdot(phi, cvadd(cvadd_r(in.DGxphi[j], vcross(vts[ij], ISn3hn)), K41[j]));
        ij++;
      }
    }
  }
}

/* LKNeighborEdgeIntegrand::weighPoint, src/Impedance.cpp:261-273 */
static void neighbor_edge_point(const tri_halves_t *t, double w, vec3 v, vec3 *K) {
  double ISn1;
  vec3 IL1;
  const half_t *th = &t->h[0];
  lk_edge_integral(th, v, &ISn1, &IL1);
  vec3 n = th->n;
  double h = vdot(vsub(v, th->p0), n);
  vec3 rho = vsub(v, vscale(h, n));
  for (int i = 0; i < t->nh; i++) {
    vec3 rho_p0 = vsub(rho, t->h[i].p0);
    K[i] = vadd(K[i], vscale(w, vadd(IL1, vscale(ISn1, rho_p0))));
  }
}

static void neighbor_edge_integrate(const tri_halves_t *t, vec3 v0, vec3 v1, vec3 *K) {
  for (int q = 0; q < BEMGPU_LINE_RULE15_N; q++) {
    vec3 v = vadd(v0, vscale(bemgpu_line_rule15[q][0], v1));
    neighbor_edge_point(t, bemgpu_line_rule15[q][1], v, K);
  }
}

static inline int shared_points(const int *a, const int *b) {
  /* sharedpoints, src/Triangle.h:23-30 (vertex identity = vertex id) */
  int c = 0;
  for (int i = 0; i < 3; i++)
    if (a[i] == b[0] || a[i] == b[1] || a[i] == b[2]) c++;
  return c;
}

static inline vec3 tri_center(const geom_t *G, int t) {
  /* center, src/Triangle.cpp:30-34 */
  const int *tv = G->tri + 3 * t;
  vec3 p = vadd(vadd(vtx(G, tv[0]), vtx(G, tv[1])), vtx(G, tv[2]));
  return vscale(ONETHIRD, p);
}

static inline double tri_emax(const geom_t *G, int t) {
  const int *tv = G->tri + 3 * t;
  double l12 = sqrt(vnorm(vsub(vtx(G, tv[1]), vtx(G, tv[0]))));
  double l23 = sqrt(vnorm(vsub(vtx(G, tv[2]), vtx(G, tv[1]))));
  double l31 = sqrt(vnorm(vsub(vtx(G, tv[0]), vtx(G, tv[2]))));
  return fmax(fmax(l12, l23), l31);
}

/* LKTriangle, src/Impedance.cpp:276-363: integrates L[9], K[9] for one
 * (test triangle, source triangle) pair.  Returns the rule used
 * (0 = same, 1 = neighbour, 6/10/15/21/36 = far rule). */
static int lk_triangle(const geom_t *G, const green_t *g, const double farThresh[4], int trit, int tris,
                       const tri_halves_t *t, const tri_halves_t *s, cplx *L, cplx *K) {
  for (int i = 0; i < 9; i++) { L[i] = 0; K[i] = 0; }
  const half_t *th = &t->h[0];
  int kind;
  if (trit == tris || shared_points(G->tri + 3 * trit, G->tri + 3 * tris) > 0) {
    vec3 vts[9];
    int ij = 0;
    for (int i = 0; i < t->nh; i++)
      for (int j = 0; j < s->nh; j++) vts[ij++] = vsub(s->h[j].p0, t->h[i].p0);
    for (int q = 0; q < BEMGPU_TRI_RULE105_N; q++) {
      const double *r = bemgpu_tri_rule105[q];
      vec3 v = vadd(vadd(th->p0, vscale(r[0], th->v01)), vscale(r[1], th->v02));
      close_outer_point(g, t, s, vts, r[2], v, L, K);
    }
    kind = 0;
    if (trit != tris) {
      kind = 1;
      /* neighbour K correction, src/Impedance.cpp:301-324 */
      const half_t *sh = &s->h[0];
      vec3 K01[3], K12[3], K20[3];
      memset(K01, 0, sizeof K01); memset(K12, 0, sizeof K12); memset(K20, 0, sizeof K20);
      neighbor_edge_integrate(t, sh->p0, sh->v01, K01);
      neighbor_edge_integrate(t, sh->p1, sh->v12, K12);
      neighbor_edge_integrate(t, sh->p2, sh->v20, K20);
      double c = 0.125 * t->h[0].Ai * s->h[0].Ai;
      ij = 0;
      for (int i = 0; i < t->nh; i++) {
        for (int j = 0; j < s->nh; j++) {
          vec3 v = vsub(t->h[i].p0, s->h[j].p0);
          K[ij] += c * (vdot(vcross(v, sh->m01), K01[i]) / sh->normv01i +
                        vdot(vcross(v, sh->m12), K12[i]) / sh->normv12i +
                        vdot(vcross(v, sh->m20), K20[i]) / sh->normv20i);
          ij++;
        }
      }
    }
  } else {
    vec3 pt = tri_center(G, trit), ps = tri_center(G, tris);
    double d = vnorm(vsub(pt, ps));
    double e = fmax(tri_emax(G, trit), tri_emax(G, tris));
    double emax2 = e * e;
    const double (*rule)[3];
    int nr;
    if (d * farThresh[0] > emax2) { rule = bemgpu_tri_rule6; nr = 6; }
    else if (d * farThresh[1] > emax2) { rule = bemgpu_tri_rule10; nr = 10; }
    else if (d * farThresh[2] > emax2) { rule = bemgpu_tri_rule15; nr = 15; }
    else if (d * farThresh[3] > emax2) { rule = bemgpu_tri_rule21; nr = 21; }
    else { rule = bemgpu_tri_rule36; nr = 36; }
    for (int q = 0; q < nr; q++) {
      vec3 v = vadd(vadd(th->p0, vscale(rule[q][0], th->v01)), vscale(rule[q][1], th->v02));
      far_outer_point(g, rule, nr, t, s, rule[q][2], v, L, K);
    }
    kind = nr;
  }
  return kind;
}

/* ---- Zts driver (src/Impedance.cpp:388-413) ---- */

typedef struct {
  const geom_t *G;
  const green_t *g;
  const double *farThresh;
  const tri_halves_t *th, *sh;
  const int *tlist, *slist;
  int ntl, nsl;
  cplx *Zpos, *Zneg;
  int64_t ld;
  int tid, nthreads;
  int tbeg, tend;
  int64_t counts[8];
  cplx sink[4]; /* timing mode (no output matrix): the scattered values are summed here */
} job_t;

/* Sum of the timing mode's sinks, so that the integration it times is kept. */
volatile double oracle_timing_checksum;

static int kind_slot(int kind) {
  switch (kind) { case 0: return 0; case 1: return 1; case 6: return 2; case 10: return 3;
    case 15: return 4; case 21: return 5; default: return 6; }
}

static void *zts_worker(void *arg) {
  job_t *J = (job_t *)arg;
  cplx L[9], K[9];
  for (int a = J->tbeg + J->tid; a < J->tend; a += J->nthreads) {
    int trit = J->tlist[a];
    const tri_halves_t *t = &J->th[trit];
    for (int b = 0; b < J->nsl; b++) {
      int tris = J->slist[b];
      const tri_halves_t *s = &J->sh[tris];
      int kind = lk_triangle(J->G, J->g, J->farThresh, trit, tris, t, s, L, K);
      J->counts[kind_slot(kind)]++;
      /* scatter, src/Impedance.cpp:365-384 */
      int ij = 0;
      for (int i = 0; i < t->nh; i++) {
        const half_t *hi = &t->h[i];
        int64_t ii = 2 * (int64_t)hi->rwg;
        cplx *Z = hi->positive ? J->Zpos : J->Zneg;
        for (int j = 0; j < s->nh; j++) {
          const half_t *hj = &s->h[j];
          int64_t jj = 2 * (int64_t)hj->rwg;
          double c = ONEOVER4PI * hi->elen * hj->elen;
          if (hi->positive != hj->positive) c = -c;
          cplx Lij = c * L[ij], Kij = c * K[ij];
          if (!Z) {
            J->sink[0] += J->g->Zeps * Lij;
            J->sink[1] += Kij;
            J->sink[2] -= Kij;
            J->sink[3] += J->g->Zmu * Lij;
            ij++;
            continue;
          }
          Z[ii + J->ld * jj] += J->g->Zeps * Lij;
          Z[ii + J->ld * (jj + 1)] += Kij;
          Z[ii + 1 + J->ld * jj] -= Kij;
          Z[ii + 1 + J->ld * (jj + 1)] += J->g->Zmu * Lij;
          ij++;
        }
      }
    }
  }
  return NULL;
}

/* Builds the per-triangle half-RWG lists of one tree (TriangleRWGMap,
 * src/Impedance.cpp:393-406): returns the triangles in first-appearance order. */
static int build_halves(const geom_t *G, const int *rwg, int nrwg, tri_halves_t *halves, int *list) {
  for (int i = 0; i < G->nt; i++) halves[i].nh = 0;
  int n = 0;
  for (int i = 0; i < nrwg; i++) {
    for (int side = 0; side < 2; side++) {
      int t = rwg[4 * i + side];
      if (t < 0 || t >= G->nt || halves[t].nh >= 3) return -1;
      if (halves[t].nh == 0) list[n++] = t;
      half_init(&halves[t].h[halves[t].nh++], G, t, rwg[4 * i + 2], rwg[4 * i + 3], side == 0, i);
    }
  }
  return n;
}

/*
 * oracle_zts: Z (column-major, ld >= 2*nrwg_t) = Zts(t, s, g) for RWG tables
 * rwg_t (rows) and rwg_s (columns) over one geometry.  Green's function built
 * from (eps, mu, omega) as GreensFunction::init does.  farThresh = Options'
 * farThresh6/10/15/21 (src/Options.cpp:23-26).  Only test triangles at
 * positions [tri_begin, tri_end) of t's triangle list are integrated (a
 * bounded sample for CPU timing; pass 0, -1 for all).  With Zout NULL
 * (timing mode) the same pairs are integrated and scaled, but the values are
 * summed into a per-thread sink instead of a matrix, so that a sample of a
 * large fill needs no n x n buffer.  Writes the number of
 * pairs integrated by each branch into counts[7] (same, neighbour, rule 6, 10,
 * 15, 21, 36) when counts is non-null.  Returns 0 or a negative error.
 */
int oracle_zts(const double *xyz, int nv, const int *tri, int nt, const int *rwg_t, int nrwg_t,
               const int *rwg_s, int nrwg_s, const double *eps_mu_omega /* re,im x3 */,
               const double *farThresh, double *Zout, int64_t ld, int tri_begin, int tri_end,
               int nthreads, int64_t *counts) {
  geom_t G = {xyz, tri, nv, nt};
  green_t g;
  green_init(&g, eps_mu_omega[0] + I * eps_mu_omega[1], eps_mu_omega[2] + I * eps_mu_omega[3],
             eps_mu_omega[4] + I * eps_mu_omega[5]);
  tri_halves_t *th = (tri_halves_t *)malloc(sizeof(tri_halves_t) * nt);
  tri_halves_t *sh = (tri_halves_t *)malloc(sizeof(tri_halves_t) * nt);
  int *tl = (int *)malloc(sizeof(int) * nt), *sl = (int *)malloc(sizeof(int) * nt);
  int ntl = build_halves(&G, rwg_t, nrwg_t, th, tl);
  int nsl = build_halves(&G, rwg_s, nrwg_s, sh, sl);
  if (ntl < 0 || nsl < 0) { free(th); free(sh); free(tl); free(sl); return -1; }
  if (tri_end < 0 || tri_end > ntl) tri_end = ntl;
  if (tri_begin < 0) tri_begin = 0;
  int64_t rows = 2 * (int64_t)nrwg_t, cols = 2 * (int64_t)nrwg_s;
  cplx *Z = (cplx *)Zout, *Zneg = NULL;
  if (Z) {
    for (int64_t j = 0; j < cols; j++) memset(Z + ld * j, 0, sizeof(cplx) * rows);
    Zneg = (cplx *)calloc((size_t)(ld * cols), sizeof(cplx));
    if (!Zneg) { free(th); free(sh); free(tl); free(sl); return -2; }
  }
  if (nthreads < 1) nthreads = 1;
  job_t *jobs = (job_t *)calloc(nthreads, sizeof(job_t));
  pthread_t *tids = (pthread_t *)malloc(sizeof(pthread_t) * nthreads);
  for (int k = 0; k < nthreads; k++) {
    job_t J = {&G, &g, farThresh, th, sh, tl, sl, ntl, nsl, Z, Zneg, ld, k, nthreads, tri_begin, tri_end, {0}, {0}};
    jobs[k] = J;
  }
  for (int k = 1; k < nthreads; k++) pthread_create(&tids[k], NULL, zts_worker, &jobs[k]);
  zts_worker(&jobs[0]);
  for (int k = 1; k < nthreads; k++) pthread_join(tids[k], NULL);
  if (Z) {
    for (int64_t j = 0; j < cols; j++)
      for (int64_t i = 0; i < rows; i++) Z[i + ld * j] += Zneg[i + ld * j];
  } else {
    double sum = 0.0;
    for (int k = 0; k < nthreads; k++)
      for (int c = 0; c < 4; c++) sum += creal(jobs[k].sink[c]) + cimag(jobs[k].sink[c]);
    oracle_timing_checksum = sum;
  }
  if (counts) {
    for (int c = 0; c < 7; c++) {
      counts[c] = 0;
      for (int k = 0; k < nthreads; k++) counts[c] += jobs[k].counts[c];
    }
  }
  free(Zneg); free(jobs); free(tids); free(th); free(sh); free(tl); free(sl);
  return 0;
}

/* GreensFunction constants for a given (eps, mu, omega): out = ksquared, k,
 * ik, k2, Zeps, Zmu as (re, im) pairs.  Lets tests compare the GPU's copy. */
void oracle_green(const double *eps_mu_omega, double *out) {
  green_t g;
  green_init(&g, eps_mu_omega[0] + I * eps_mu_omega[1], eps_mu_omega[2] + I * eps_mu_omega[3],
             eps_mu_omega[4] + I * eps_mu_omega[5]);
  cplx v[6] = {g.ksquared, g.k, g.ik, g.k2, g.Zeps, g.Zmu};
  for (int i = 0; i < 6; i++) { out[2 * i] = creal(v[i]); out[2 * i + 1] = cimag(v[i]); }
}
