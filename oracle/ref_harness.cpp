// Test-infrastructure harness around the reference's own C++ (claytonotey/bem).
//
// This file is compiled together with the reference's sources, where they lie
// under the reference checkout, by oracle/Makefile.ref into oracle/_ref/.  It is
// never part of the product: it exists to pin the oracle restatement
// (oracle/bem_oracle.c) and to generate the golden fixtures in tests/golden/.
//
// What it does, per invocation:
//   1. reads two triangle meshes in the project's plain-text mesh format
//      ("nv nt", nv lines "x y z", nt lines "i j k"), builds each face through
//      the reference's FaceIndex(const char*) parser (src/FaceIndex.cpp:3-12);
//   2. translates body 1 by the gap vector exactly as parseShapes does
//      (src/HeatTransfer.cpp:67-69);
//   3. builds ShapeMesh x2 and the RWGTree with the reference's own code,
//      keeping them alive on the heap (parseShapes keeps them on its stack and
//      returns dangling pointers: src/HeatTransfer.cpp:61,105-108);
//   4. uses a fixed-parameter Lorentz dielectric with the functional form of
//      SiC::eps (src/util/SiC.cpp:16-19), parameters given in eV;
//   5. writes the RWG order chosen by the reference (RWGTree + unshuffle,
//      src/RWGTree.cpp:602-761) and, on request, the three Zts matrices of
//      CalcHeatTransfer (src/HeatTransfer.cpp:20-29) as raw complex128;
//   6. prints CalcHeatTransfer (src/HeatTransfer.cpp:8-59) for each frequency;
//   7. on request (--edges), writes each body's edges in the order ShapeMesh
//      created them (src/ShapeMesh.cpp:857-928), before any partition.
#include "HeatTransfer.h"
#include "ShapeParser.h"
#include "RWGTree.h"
#include "ShapeMesh.h"
#include "Impedance.h"
#include "SI.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include <chrono>

// X3D files are read by the reference's own ShapeParser (src/ShapeParser.cpp,
// built over the small Xerces stand-in in oracle/shim/) in --x3d mode only.

// Lorentz oscillator with SiC::eps's functional form (src/util/SiC.cpp:16-19),
// parameters fixed (no temperature dependence) and given in eV.
class FixedLorentz : public Dielectric {
 public:
  FixedLorentz(Real epsinf_, Real wTO_eV, Real wLO_eV, Real gamma_eV) {
    epsinf = epsinf_;
    wT = wTO_eV * SI::eV / SI::hbar;
    wL = wLO_eV * SI::eV / SI::hbar;
    gamma = gamma_eV * SI::eV / SI::hbar;
  }
  Complex eps(Real feV) {
    Real w = feV * SI::eV / SI::hbar;
    return epsinf * (wL * wL - w * w - Complex(0, gamma * w)) /
           (wT * wT - w * w - Complex(0, gamma * w));
  }
  Complex mu(Real) { return Complex(1., 0.); }
  Real epsinf, wT, wL, gamma;
};

static void readMesh(const char *path, Shape &shape) {
  FILE *f = fopen(path, "r");
  if (!f) { perror(path); exit(2); }
  int nv, nt;
  if (fscanf(f, "%d %d", &nv, &nt) != 2) { fprintf(stderr, "bad mesh header %s\n", path); exit(2); }
  for (int i = 0; i < nv; i++) {
    double x, y, z;
    if (fscanf(f, "%lf %lf %lf", &x, &y, &z) != 3) { fprintf(stderr, "bad vertex\n"); exit(2); }
    shape.coord.push_back(Vector3(x, y, z));
  }
  for (int i = 0; i < nt; i++) {
    int a, b, c;
    if (fscanf(f, "%d %d %d", &a, &b, &c) != 3) { fprintf(stderr, "bad face\n"); exit(2); }
    char buf[96];
    snprintf(buf, sizeof buf, "%d %d %d -1", a, b, c);
    shape.faceIndex.push_back(FaceIndex(buf));
  }
  fclose(f);
}

static void dumpMatrix(const std::string &path, ComplexDenseMatrix *Z) {
  FILE *f = fopen(path.c_str(), "wb");
  if (!f) { perror(path.c_str()); exit(2); }
  // column-major p[i + lda*j] (src/util/DenseMatrix.h:195-198), lda == m here
  for (int j = 0; j < Z->n; j++)
    fwrite(Z->p + (size_t)Z->lda * j, sizeof(Complex), Z->m, f);
  fclose(f);
}

static std::vector<double> parseList(const char *s) {
  std::vector<double> v;
  const char *p = s;
  while (*p) {
    v.push_back(atof(p));
    while (*p && *p != ',') p++;
    if (*p == ',') p++;
  }
  return v;
}

// --x3d FILE --shape-out OUT: the reference's parse of one X3D file
// (ShapeParser::parse, src/ShapeParser.cpp:83-153 with its Transform stack):
// "nv nt", the transformed coordinates, the faces' four FaceIndex integers,
// and the Dielectric's eps at 0.1 eV ("none" without one).
static int dumpX3d(const char *file, const char *out) {
  ShapeParser parser;
  Shape shape;
  Dielectric *diel = NULL;
  parser.parse((char *)file, shape, &diel);
  FILE *f = fopen(out, "w");
  if (!f) { perror(out); return 2; }
  fprintf(f, "%d %d\n", (int)shape.coord.size(), (int)shape.faceIndex.size());
  for (size_t i = 0; i < shape.coord.size(); i++)
    fprintf(f, "%.17g %.17g %.17g\n", shape.coord[i].x, shape.coord[i].y, shape.coord[i].z);
  for (size_t i = 0; i < shape.faceIndex.size(); i++)
    fprintf(f, "%d %d %d %d\n", shape.faceIndex[i].i[0], shape.faceIndex[i].i[1], shape.faceIndex[i].i[2],
            shape.faceIndex[i].i[3]);
  // ShapeParserHandler leaves its dielectric pointer unset when the file has
  // no Dielectric element, so it is read only when the file names one
  bool named = false;
  if (FILE *x = fopen(file, "rb")) {
    std::string doc;
    char buf[65536];
    size_t n;
    while ((n = fread(buf, 1, sizeof buf, x)) > 0) doc.append(buf, n);
    fclose(x);
    named = doc.find("<Dielectric") != std::string::npos;
  }
  if (named && diel) {
    Complex e = diel->eps(0.1);
    fprintf(f, "eps %.17g %.17g\n", real(e), imag(e));
  } else {
    fprintf(f, "none\n");
  }
  fclose(f);
  return 0;
}

int main(int argc, char **argv) {
  initReferenceCountingPointerLock();
  if (argc == 5 && std::string(argv[1]) == "--x3d" && std::string(argv[3]) == "--shape-out")
    return dumpX3d(argv[2], argv[4]);
  const char *mesh1 = NULL, *mesh2 = NULL, *orderOut = NULL, *zPrefix = NULL, *edgesOut = NULL;
  Vector3 gap(0., 0., 0.);
  Real a = 1e-6, T1 = 300., T2 = 0.;
  std::vector<double> l1, l2, freqs;
  bool timing = false;
  for (int i = 1; i < argc; i++) {
    std::string k = argv[i];
    if (k == "--mesh1") mesh1 = argv[++i];
    else if (k == "--mesh2") mesh2 = argv[++i];
    else if (k == "--gap") { std::vector<double> g = parseList(argv[++i]); gap = Vector3(g[0], g[1], g[2]); }
    else if (k == "--a") a = atof(argv[++i]);
    else if (k == "--T1") T1 = atof(argv[++i]);
    else if (k == "--T2") T2 = atof(argv[++i]);
    else if (k == "--lorentz1") l1 = parseList(argv[++i]);
    else if (k == "--lorentz2") l2 = parseList(argv[++i]);
    else if (k == "--freqs") freqs = parseList(argv[++i]);
    else if (k == "--order") orderOut = argv[++i];
    else if (k == "--dumpz") zPrefix = argv[++i];
    else if (k == "--edges") edgesOut = argv[++i];
    else if (k == "--time") timing = true;
    else { fprintf(stderr, "unknown argument %s\n", argv[i]); return 2; }
  }
  if (!mesh1 || !mesh2 || l1.size() != 4 || l2.size() != 4) {
    fprintf(stderr, "usage: ref_harness --mesh1 f --mesh2 f --gap x,y,z --a m --T1 K --T2 K "
                    "--lorentz1 einf,wTO,wLO,gamma --lorentz2 ... --freqs f1,f2 [--order out] [--dumpz prefix] [--edges out] "
                    "[--time]\n");
    return 2;
  }

  Options options;
  Shape body1Shape, body2Shape;
  readMesh(mesh1, body1Shape);
  readMesh(mesh2, body2Shape);
  Transform tform;
  tform.setT(gap);
  body1Shape.transform(tform);

  Real maxEdgeLength;
  ShapeMesh *m1 = new ShapeMesh(body1Shape, options.sharpThresh, options.concaveThresh,
                                options.relativeCostAngleConcave, &refineEdgeFuncBody, &maxEdgeLength);
  ShapeMesh *m2 = new ShapeMesh(body2Shape, options.sharpThresh, options.concaveThresh,
                                options.relativeCostAngleConcave, &refineEdgeFuncBody, &maxEdgeLength);
  Dielectric *d1 = new FixedLorentz(l1[0], l1[1], l1[2], l1[3]);
  Dielectric *d2 = new FixedLorentz(l2[0], l2[1], l2[2], l2[3]);
  ShapeMeshDielectricPairList meshDiel;
  PointEdgeVectorMap *eap = new PointEdgeVectorMap;
  getEdgesAtPoints(*m1, *eap);
  getEdgesAtPoints(*m2, *eap);
  meshDiel.push_back(ShapeMeshDielectricPair(m1, d1));
  meshDiel.push_back(ShapeMeshDielectricPair(m2, d2));
  RWGTree *top = new RWGTree(meshDiel, *eap, options.minSegmentSize, 0.0);
  RWGTree *s = top->sub[0];
  RWGTree *t = top->sub[1];

  if (edgesOut) {
    // One line per edge of each body's first mesh level, in creation order:
    // body, first triangle (t1, positive), second triangle (t2), p1, p2
    // (ids local to the body's mesh file).
    FILE *f = fopen(edgesOut, "w");
    ShapeMesh *mb[2] = {m1, m2};
    for (int b = 0; b < 2; b++) {
      Array<Edge> &E = *mb[b]->refinedEdge[0];
      Point *P0 = mb[b]->refinedPoint[0]->p;
      Triangle *T0 = mb[b]->refinedTriangle[0]->p;
      for (int i = 0; i < E.n; i++)
        fprintf(f, "%d %ld %ld %ld %ld\n", b, (long)(E[i].t1 - T0), (long)(E[i].t2 - T0), (long)(E[i].p1 - P0),
                (long)(E[i].p2 - P0));
    }
    fclose(f);
  }

  if (orderOut) {
    // One line per RWG in top->rwg order: body, edge p1, edge p2, pos tri, neg tri
    // (vertex and triangle ids local to the body's mesh, as read from the file).
    FILE *f = fopen(orderOut, "w");
    fprintf(f, "%d %d %d\n", top->rwgs, s->rwgs, t->rwgs);
    Point *pb[2] = {m1->refinedPoint[0]->p, m2->refinedPoint[0]->p};
    Triangle *tb[2] = {m1->refinedTriangle[0]->p, m2->refinedTriangle[0]->p};
    int np[2] = {(int)body1Shape.coord.size(), (int)body2Shape.coord.size()};
    int nt[2] = {(int)body1Shape.faceIndex.size(), (int)body2Shape.faceIndex.size()};
    for (int i = 0; i < top->rwgs; i++) {
      RWG *r = top->rwg[i];
      int body = -1;
      for (int b = 0; b < 2; b++)
        if (r->e->p1 >= pb[b] && r->e->p1 < pb[b] + np[b]) body = b;
      long tp = r->pos.t - tb[body], tn = r->neg.t - tb[body];
      if (tp < 0 || tp >= nt[body] || tn < 0 || tn >= nt[body]) { fprintf(stderr, "triangle out of range\n"); return 3; }
      fprintf(f, "%d %ld %ld %ld %ld\n", body, (long)(r->e->p1 - pb[body]), (long)(r->e->p2 - pb[body]), tp, tn);
    }
    fclose(f);
  }

  for (size_t fi = 0; fi < freqs.size(); fi++) {
    Real eV = freqs[fi];
    if (zPrefix && fi == 0) {
      // The three fills of CalcHeatTransfer (src/HeatTransfer.cpp:10-29).
      Real omegaSI = eV * SI::eV / SI::hbar;
      Real omega = omegaSI * a / SI::c;
      GreensFunction greenExt(1., 1., omega, true);
      s->g->init(s->diel->eps(eV), s->diel->mu(eV), omega);
      t->g->init(t->diel->eps(eV), t->diel->mu(eV), omega);
      auto t0 = std::chrono::steady_clock::now();
      ComplexDenseMatrix *W = Zts(top, top, &greenExt, options);
      auto t1 = std::chrono::steady_clock::now();
      ComplexDenseMatrix *G1 = Zts(s, s, s->g, options);
      ComplexDenseMatrix *G2 = Zts(t, t, t->g, options);
      auto t2 = std::chrono::steady_clock::now();
      dumpMatrix(std::string(zPrefix) + "_ext.bin", W);
      dumpMatrix(std::string(zPrefix) + "_int1.bin", G1);
      dumpMatrix(std::string(zPrefix) + "_int2.bin", G2);
      if (timing)
        fprintf(stderr, "fill ext %.3f s, int %.3f s\n",
                std::chrono::duration<double>(t1 - t0).count(),
                std::chrono::duration<double>(t2 - t1).count());
      delete W; delete G1; delete G2;
    }
    auto t0 = std::chrono::steady_clock::now();
    Real P = CalcHeatTransfer(a, eV, T1, T2, top, s, t, options);
    auto t1 = std::chrono::steady_clock::now();
    printf("P %.17g %.17g\n", eV, P);
    if (timing) fprintf(stderr, "solve %.3f s\n", std::chrono::duration<double>(t1 - t0).count());
    fflush(stdout);
  }
  return 0;
}
