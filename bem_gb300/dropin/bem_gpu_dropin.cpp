// bem_gpu_dropin.cpp — the reference-side binding of libbemgpu.so.
//
// Link this file and -lbemgpu into the reference's programs (transfer,
// transfer-mpi's single-process path) in place of the CPU definitions of
//   ComplexDenseMatrix *Zts(RWGTree*, RWGTree*, GreensFunction*, Options&)   src/Impedance.h:21
//   Real CalcHeatTransfer(Real, Real, Real, Real, RWGTree*, RWGTree*, RWGTree*, Options&)
//                                                                            src/HeatTransfer.h:33
//   Real Theta(Real omega, Real T)                                           src/HeatTransfer.cpp:3-6
// The rest of Impedance.cpp and HeatTransfer.cpp (parseShapes, LKTriangle, ...)
// stays: build those two files with -DZts=bem_cpu_Zts
// -DCalcHeatTransfer=bem_cpu_CalcHeatTransfer -DTheta=bem_cpu_Theta so that
// their CPU versions keep other names (oracle/Makefile.ref, target dropin,
// links exactly that with every symbol resolved).
//
// The reference's geometry objects are flattened into the C ABI's plain
// arrays: one geometry over every point and triangle the RWGs touch, and RWG
// tables {pos triangle, neg triangle, edge vertex 1, edge vertex 2} in the
// tree's rwg[] order (= matrix order).  Errors are thrown as
// std::runtime_error with the library's message; the reference itself has no
// error path.
#include "HeatTransfer.h"
#include "bemgpu.h"

#include <complex>
#include <map>
#include <stdexcept>
#include <vector>

namespace {

bemgpu_ctx_t ctx() {
  static bemgpu_ctx_t c = nullptr;
  if (!c && bemgpu_ctx_create(0, &c) != BEMGPU_OK) throw std::runtime_error("bemgpu: no CUDA device");
  return c;
}

void check(int rc) {
  if (rc != BEMGPU_OK) throw std::runtime_error(bemgpu_ctx_last_error(ctx()));
}

struct Flat {
  bemgpu_geom_t geom = nullptr;
  bemgpu_tree_t tree = nullptr;
  std::vector<int> rwg;
  ~Flat() {
    if (tree) bemgpu_tree_destroy(tree);
    if (geom) bemgpu_geom_destroy(geom);
  }
};

void flatten(RWGTree *tr, Flat &f) {
  std::map<Point *, int> pid;
  std::map<Triangle *, int> tid;
  std::vector<double> xyz;
  std::vector<int> tri;
  auto P = [&](Point *p) {
    auto it = pid.find(p);
    if (it != pid.end()) return it->second;
    const int i = (int)pid.size();
    pid[p] = i;
    xyz.insert(xyz.end(), {p->x, p->y, p->z});
    return i;
  };
  auto T = [&](Triangle *t) {
    auto it = tid.find(t);
    if (it != tid.end()) return it->second;
    const int i = (int)tid.size();
    tid[t] = i;
    tri.insert(tri.end(), {P(t->p1), P(t->p2), P(t->p3)});
    return i;
  };
  for (int i = 0; i < tr->rwgs; i++) {
    RWG *r = tr->rwg[i];
    f.rwg.insert(f.rwg.end(), {T(r->pos.t), T(r->neg.t), P(r->e->p1), P(r->e->p2)});
  }
  check(bemgpu_geom_create(ctx(), xyz.data(), (int)pid.size(), tri.data(), (int)tid.size(), &f.geom));
  check(bemgpu_tree_create(f.geom, f.rwg.data(), tr->rwgs, &f.tree));
}

bemgpu_options_t options_of(const Options &o) { return {o.farThresh6, o.farThresh10, o.farThresh15, o.farThresh21}; }

}  // namespace

ComplexDenseMatrix *Zts(RWGTree *t, RWGTree *s, GreensFunction *g, Options &o) {
  // t and s share one geometry only when they are the same tree; a
  // cross-tree block is a sub-block of the parent's fill
  if (t != s) throw std::runtime_error("bemgpu Zts: t and s must be the same tree (fill the parent tree)");
  Flat f;
  flatten(t, f);
  bemgpu_green_t gg;
  const double e[2] = {real(g->eps), imag(g->eps)}, m[2] = {real(g->mu), imag(g->mu)};
  const double w[2] = {real(g->omega), imag(g->omega)};
  check(bemgpu_green_init(e, m, w, g->bExternal ? 1 : 0, &gg));
  const bemgpu_options_t bo = options_of(o);
  ComplexDenseMatrix *Z = new ComplexDenseMatrix(2 * t->rwgs, 2 * s->rwgs);
  const int rc = bemgpu_zts_host(ctx(), f.tree, f.tree, &gg, &bo, BEMGPU_PREC_FP64,
                                 reinterpret_cast<double *>(Z->p + 0), Z->lda);
  if (rc != BEMGPU_OK) {
    delete Z;
    check(rc);
  }
  return Z;  // the caller deletes it, as with the reference
}

Real Theta(Real omega, Real T) { return bemgpu_theta(omega, T); }

Real CalcHeatTransfer(Real a, Real eV, Real T1, Real T2, RWGTree *top, RWGTree *s, RWGTree *t, Options &o) {
  Flat f;
  flatten(top, f);  // s's RWGs first, then t's (RWGTree::unshuffle order)
  if (s->rwgs + t->rwgs != top->rwgs) throw std::runtime_error("bemgpu CalcHeatTransfer: size(top) != size(s) + size(t)");
  // the one-body trees over the same geometry: the first s->rwgs rows of the
  // table and the last t->rwgs rows
  bemgpu_tree_t ts = nullptr, tt = nullptr;
  check(bemgpu_tree_create(f.geom, f.rwg.data(), s->rwgs, &ts));
  const int rc_t = bemgpu_tree_create(f.geom, f.rwg.data() + 4 * (size_t)s->rwgs, t->rwgs, &tt);
  if (rc_t != BEMGPU_OK) {
    bemgpu_tree_destroy(ts);
    check(rc_t);
  }
  s->diel->setTemperature(T1);
  t->diel->setTemperature(T2);
  const std::complex<double> e1 = s->diel->eps(eV), e2 = t->diel->eps(eV);
  const std::complex<double> m1 = s->diel->mu(eV), m2 = t->diel->mu(eV);
  bemgpu_solve_req_t rq = {a, eV, T1, T2, {real(e1), imag(e1)}, {real(m1), imag(m1)},
                           {real(e2), imag(e2)}, {real(m2), imag(m2)}};
  const bemgpu_options_t bo = options_of(o);
  double P = 0;
  const int rc = bemgpu_heat_transfer(ctx(), f.tree, ts, tt, &rq, &bo, BEMGPU_PREC_FP64, &P, nullptr);
  bemgpu_tree_destroy(ts);
  bemgpu_tree_destroy(tt);
  check(rc);
  return P;
}
