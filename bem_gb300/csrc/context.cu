// Context, resident geometry and RWG trees, Green's function constants.
//
// Host-side set-up runs once per geometry: the half-RWG frames of every
// triangle are computed here in FP64 with the reference's arithmetic
// (HalfRWG::HalfRWG, src/RWG.cpp:7-39) and kept on the device.
#include "bemgpu_internal.h"

#include <cmath>
#include <complex>
#include <cstdarg>
#include <cstring>
#include <cstdlib>
#include <algorithm>
#include <unordered_map>

namespace {

// src/util/SI.cpp:3-9
const double SI_HBAR = 1.05457148e-34;
const double SI_KB = 1.3806503e-23;
const double SI_EV = 1.60217646e-19;
const double SI_C = 2.99792458e8;

struct V3 {
  double x, y, z;
};
inline V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 add(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 scale(double c, V3 a) { return {c * a.x, c * a.y, c * a.z}; }
inline V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline double norm2(V3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
inline V3 normalized(V3 a) {
  double ni = 1. / std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
  return {a.x * ni, a.y * ni, a.z * ni};
}
inline void put(double *d, V3 a) { d[0] = a.x; d[1] = a.y; d[2] = a.z; }

V3 vtx(const bemgpu_geom_s *g, int i) { return {g->xyz[3 * i], g->xyz[3 * i + 1], g->xyz[3 * i + 2]}; }

const char *kVersion = "bemgpu 0.1 (sm_103a)";

}  // namespace

int bem_fail(bemgpu_ctx_s *ctx, int code, const char *fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (ctx) ctx->last_error = buf;
  return code;
}

void bem_trace(const char *fmt, ...) {
  static const bool on = [] {
    const char *v = getenv("BEMGPU_TRACE");
    return v && v[0] && strcmp(v, "0") != 0;
  }();
  if (!on) return;
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  fprintf(stderr, "bemgpu: %s\n", buf);
}

// ---------------- deferred frees ----------------
// Destroying a tree or geometry gives its device memory (triangle records,
// near-pair lists) to this list instead of freeing it at once: cudaFree waits
// for the whole device, so a serving loop that destroys each request's
// geometry would otherwise drain every lane's work per request.  The list is
// freed in one go - one device synchronisation, so nothing in flight still
// reads the memory - when it holds DEFER_MAX_PTRS pointers or DEFER_MAX_BYTES,
// when a context is trimmed or torn down, and before an allocation that
// failed is retried.
namespace {
struct DeferredFrees {
  std::mutex mu;
  std::vector<std::pair<int, void *>> ptrs;  // (device, pointer)
  size_t bytes = 0;
};
DeferredFrees &deferred_frees() {
  static DeferredFrees d;
  return d;
}
constexpr size_t DEFER_MAX_PTRS = 96;
constexpr size_t DEFER_MAX_BYTES = (size_t)512 << 20;
}  // namespace

void bem_flush_deferred_frees() {
  std::vector<std::pair<int, void *>> v;
  {
    DeferredFrees &d = deferred_frees();
    std::lock_guard<std::mutex> lk(d.mu);
    v.swap(d.ptrs);
    d.bytes = 0;
  }
  if (v.empty()) return;
  int cur = 0;
  cudaGetDevice(&cur);
  std::sort(v.begin(), v.end());
  int dev = -1;
  for (auto &e : v) {
    if (e.first != dev) {
      dev = e.first;
      cudaSetDevice(dev);
      cudaDeviceSynchronize();
    }
    cudaFree(e.second);
  }
  cudaSetDevice(cur);
}

void bem_defer_free(int device, void *p, size_t bytes) {
  if (!p) return;
  bool flush;
  {
    DeferredFrees &d = deferred_frees();
    std::lock_guard<std::mutex> lk(d.mu);
    d.ptrs.emplace_back(device, p);
    d.bytes += bytes;
    flush = d.ptrs.size() >= DEFER_MAX_PTRS || d.bytes >= DEFER_MAX_BYTES;
  }
  if (flush) bem_flush_deferred_frees();
}

size_t bem_deferred_free_count() {
  DeferredFrees &d = deferred_frees();
  std::lock_guard<std::mutex> lk(d.mu);
  return d.ptrs.size();
}

extern "C" int64_t bemgpu_pending_free_bytes(void) {
  DeferredFrees &d = deferred_frees();
  std::lock_guard<std::mutex> lk(d.mu);
  return (int64_t)d.bytes;
}

void *bem_workspace(bemgpu_ctx_s *ctx, const std::string &name, size_t bytes) {
  auto it = ctx->ws.find(name);
  if (it != ctx->ws.end() && it->second.second >= bytes) return it->second.first;
  if (it != ctx->ws.end()) {
    cudaStreamSynchronize(ctx->stream);
    cudaFree(it->second.first);
    ctx->ws.erase(it);
  }
  void *p = nullptr;
  if (cudaMalloc(&p, bytes ? bytes : 16) != cudaSuccess) {
    cudaGetLastError();
    // memory of destroyed trees may still be waiting in the deferred list
    bem_flush_deferred_frees();
    if (cudaMalloc(&p, bytes ? bytes : 16) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
  }
  ctx->ws[name] = {p, bytes};
  return p;
}

void bem_workspace_release(bemgpu_ctx_s *ctx, const std::string &name) {
  auto it = ctx->ws.find(name);
  if (it == ctx->ws.end()) return;
  cudaStreamSynchronize(ctx->stream);
  cudaFree(it->second.first);
  ctx->ws.erase(it);
}

size_t bem_workspace_bytes(const bemgpu_ctx_s *ctx) {
  size_t b = 0;
  for (auto &kv : ctx->ws) b += kv.second.second;
  return b;
}

void bem_build_near_pairs(const bemgpu_tree_s *t, const bemgpu_tree_s *s, std::vector<NearPair> &pairs) {
  pairs.clear();
  const bemgpu_geom_s *g = t->geom;
  std::unordered_map<int, int> s_local;
  for (int i = 0; i < s->ntri; i++) s_local[s->tri_gid[i]] = i;
  std::vector<int> seen;
  for (int a = 0; a < t->ntri; a++) {
    int gt = t->tri_gid[a];
    seen.clear();
    for (int k = 0; k < 3; k++) {
      int v = g->tri[3 * gt + k];
      for (int gs : g->tris_at_vertex[v]) {
        auto f = s_local.find(gs);
        if (f == s_local.end()) continue;
        if (std::find(seen.begin(), seen.end(), f->second) != seen.end()) continue;
        seen.push_back(f->second);
      }
    }
    std::sort(seen.begin(), seen.end());
    for (int b : seen) pairs.push_back({a, b, s->tri_gid[b] == gt ? 1 : 0, 0});
  }
  // Self pairs (no neighbour-edge correction, a shorter finish) first, then
  // coplanar pairs (every outer node takes the in-plane branch of the
  // close-pair contraction), then the rest, so that the near-pair kernels'
  // CTAs, which barrier after each pair couple, take couples of one kind.
  // Each pair writes its own half-pair slots: the order changes no result.
  auto kind = [&](const NearPair &p) {
    if (p.same) return 0;
    const int *ta = &g->tri[3 * (size_t)t->tri_gid[p.t]], *sb = &g->tri[3 * (size_t)s->tri_gid[p.s]];
    const double *x = g->xyz.data();
    auto sub = [&](int a, int b, double *o) {
      for (int k = 0; k < 3; k++) o[k] = x[3 * (size_t)a + k] - x[3 * (size_t)b + k];
    };
    double e1[3], e2[3], n[3];
    sub(sb[1], sb[0], e1);
    sub(sb[2], sb[0], e2);
    n[0] = e1[1] * e2[2] - e1[2] * e2[1];
    n[1] = e1[2] * e2[0] - e1[0] * e2[2];
    n[2] = e1[0] * e2[1] - e1[1] * e2[0];
    const double nn = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    const double el = std::sqrt(e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2]);
    if (!(nn > 0)) return 2;
    // the test triangle's vertices in the source triangle's plane (the
    // contraction's plane test, |h| < 1e-8 of an edge, holds at every node)
    for (int k = 0; k < 3; k++) {
      double d[3];
      sub(ta[k], sb[0], d);
      if (std::fabs(d[0] * n[0] + d[1] * n[1] + d[2] * n[2]) / nn >= 1e-9 * el) return 2;
    }
    return 1;
  };
  std::vector<std::pair<int, NearPair>> keyed(pairs.size());
  for (size_t i = 0; i < pairs.size(); i++) keyed[i] = {kind(pairs[i]), pairs[i]};
  std::stable_sort(keyed.begin(), keyed.end(),
                   [](const std::pair<int, NearPair> &a, const std::pair<int, NearPair> &b) { return a.first < b.first; });
  for (size_t i = 0; i < pairs.size(); i++) pairs[i] = keyed[i].second;
}

const NearList *bem_near_list(bemgpu_ctx_s *ctx, const bemgpu_tree_s *t, const bemgpu_tree_s *s) {
  bemgpu_geom_s *g = t->geom;
  std::lock_guard<std::mutex> lk(g->cache_mu);
  auto key = std::make_pair(t, s);
  auto it = g->near_cache.find(key);
  if (it != g->near_cache.end()) return &it->second;
  std::vector<NearPair> pairs;
  bem_build_near_pairs(t, s, pairs);
  NearList nl;
  nl.n = (int64_t)pairs.size();
  if (nl.n) {
    if (cudaMalloc(&nl.d, sizeof(NearPair) * pairs.size()) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    // a copy from pageable memory may return before it lands; kernels on any
    // lane's stream read the list, so it must be complete on return
    if (cudaMemcpyAsync(nl.d, pairs.data(), sizeof(NearPair) * pairs.size(), cudaMemcpyHostToDevice,
                        ctx->stream) != cudaSuccess ||
        cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
      cudaGetLastError();
      cudaFree(nl.d);
      return nullptr;
    }
  }
  auto res = g->near_cache.emplace(key, nl);
  return &res.first->second;
}

static cudaEvent_t prof_event(bemgpu_ctx_s *c) {
  if (c->ev_used == c->ev_pool.size()) {
    cudaEvent_t e;
    cudaEventCreate(&e);
    c->ev_pool.push_back(e);
  }
  return c->ev_pool[c->ev_used++];
}

ProfScope::ProfScope(bemgpu_ctx_s *c, int k, cudaStream_t s, double f, double b)
    : ctx(c), kind(k), st(s), flops(f), bytes(b) {
  if (ctx && ctx->prof) {
    a = prof_event(ctx);
    cudaEventRecord(a, st);
  }
}

ProfScope::~ProfScope() {
  if (a) {
    cudaEvent_t b = prof_event(ctx);
    cudaEventRecord(b, st);
    ctx->prof_recs.push_back({kind, a, b, flops, bytes, tensor});
  }
}

const int64_t *bem_far_rule_counts(bemgpu_ctx_s *ctx, const bemgpu_tree_s *t, const bemgpu_tree_s *s,
                                   const bemgpu_options_t *opt) {
  (void)ctx;
  bemgpu_geom_s *g = t->geom;
  std::lock_guard<std::mutex> lk(g->cache_mu);
  auto key = std::make_pair(t, s);
  auto it = g->far_rule_cache.find(key);
  if (it != g->far_rule_cache.end()) return it->second.data();
  std::vector<int64_t> c(5, 0);
  for (const TriRec &T : t->host_rec)
    for (const TriRec &S : s->host_rec) {
      if (T.gid == S.gid) continue;
      int sh = 0;
      for (int i = 0; i < 3; i++) sh += (T.vid[i] == S.vid[0]) | (T.vid[i] == S.vid[1]) | (T.vid[i] == S.vid[2]);
      if (sh) continue;
      double x = T.c[0] - S.c[0], y = T.c[1] - S.c[1], z = T.c[2] - S.c[2];
      double d = x * x + y * y + z * z;
      double e = std::max(T.emax, S.emax);
      double e2 = e * e;
      int k = d * opt->farThresh6 > e2 ? 0 : d * opt->farThresh10 > e2 ? 1 : d * opt->farThresh15 > e2 ? 2
            : d * opt->farThresh21 > e2 ? 3 : 4;
      c[k]++;
    }
  auto res = g->far_rule_cache.emplace(key, c);
  return res.first->second.data();
}

extern "C" {

const char *bemgpu_version(void) { return kVersion; }

int bemgpu_prof_enable(bemgpu_ctx_t ctx, int enable) {
  if (!ctx) return BEMGPU_ERR_ARG;
  std::lock_guard<std::mutex> lk(ctx->mu);
  cudaStreamSynchronize(ctx->stream);
  ctx->prof = enable != 0;
  ctx->prof_recs.clear();
  ctx->ev_used = 0;
  return BEMGPU_OK;
}

int bemgpu_prof_query(bemgpu_ctx_t ctx, int kind, int64_t *launches, double *ms, double *flops, double *bytes) {
  if (!ctx || kind < 0 || kind >= BEMGPU_K_COUNT) return BEMGPU_ERR_ARG;
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) return bem_fail(ctx, BEMGPU_ERR_CUDA, "prof_query: sync");
  int64_t n = 0;
  double t = 0, f = 0, b = 0;
  for (auto &r : ctx->prof_recs) {
    if (r.kind != kind) continue;
    float e = 0;
    cudaEventElapsedTime(&e, r.a, r.b);
    n++;
    t += e;
    f += r.flops;
    b += r.bytes;
  }
  if (launches) *launches = n;
  if (ms) *ms = t;
  if (flops) *flops = f;
  if (bytes) *bytes = b;
  return BEMGPU_OK;
}

int bemgpu_prof_query_tensor(bemgpu_ctx_t ctx, int kind, double *tensor_flops) {
  if (!ctx || !tensor_flops || kind < 0 || kind >= BEMGPU_K_COUNT) return BEMGPU_ERR_ARG;
  std::lock_guard<std::mutex> lk(ctx->mu);
  double f = 0;
  for (auto &r : ctx->prof_recs)
    if (r.kind == kind) f += r.tensor;
  *tensor_flops = f;
  return BEMGPU_OK;
}

int bemgpu_ctx_create(int device, bemgpu_ctx_t *out) {
  if (!out) return BEMGPU_ERR_ARG;
  *out = nullptr;
  int ndev = 0;
  if (device < 0 || device >= BEM_MAX_DEVICES) return BEMGPU_ERR_ARG;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device >= ndev) {
    cudaGetLastError();
    return BEMGPU_ERR_CUDA;
  }
  if (cudaSetDevice(device) != cudaSuccess) return BEMGPU_ERR_CUDA;
  bemgpu_ctx_s *c = new bemgpu_ctx_s();
  c->device = device;
  cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return BEMGPU_ERR_CUDA;
  }
  for (auto &e : c->ev) cudaEventCreate(&e);
  *out = c;
  return BEMGPU_OK;
}

static void ctx_teardown(bemgpu_ctx_s *ctx) {
  bem_flush_deferred_frees();
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  for (auto &kv : ctx->ws) cudaFree(kv.second.first);
  for (auto &e : ctx->ev) cudaEventDestroy(e);
  for (auto &e : ctx->ev_pool) cudaEventDestroy(e);
  cudaStreamDestroy(ctx->stream);
  delete ctx;
}

// The context is torn down when its handle and every geometry created on it
// are destroyed, in whatever order a caller finalizes them.
static void ctx_release(bemgpu_ctx_s *ctx) {
  bool last;
  {
    std::lock_guard<std::mutex> lk(ctx->mu);
    last = (--ctx->refs == 0);
  }
  if (last) ctx_teardown(ctx);
}

int bemgpu_ctx_destroy(bemgpu_ctx_t ctx) {
  if (!ctx) return BEMGPU_ERR_ARG;
  ctx_release(ctx);
  return BEMGPU_OK;
}

int bemgpu_ctx_stream(bemgpu_ctx_t ctx, void **stream) {
  if (!ctx || !stream) return BEMGPU_ERR_ARG;
  *stream = (void *)ctx->stream;
  return BEMGPU_OK;
}

int64_t bemgpu_ctx_launches(bemgpu_ctx_t ctx) { return ctx ? ctx->launches : BEMGPU_ERR_ARG; }

int64_t bemgpu_ctx_workspace_bytes(bemgpu_ctx_t ctx) {
  if (!ctx) return BEMGPU_ERR_ARG;
  std::lock_guard<std::mutex> lk(ctx->mu);
  return (int64_t)bem_workspace_bytes(ctx);
}

int bemgpu_ctx_trim(bemgpu_ctx_t ctx) {
  if (!ctx) return BEMGPU_ERR_ARG;
  bem_flush_deferred_frees();
  std::lock_guard<std::mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  for (auto &kv : ctx->ws) cudaFree(kv.second.first);
  ctx->ws.clear();
  ctx->tc_err_ready = false;  // the error flag lived in the workspace
  return BEMGPU_OK;
}

const char *bemgpu_ctx_last_error(bemgpu_ctx_t ctx) {
  return ctx ? ctx->last_error.c_str() : "null context";
}

int bemgpu_geom_create(bemgpu_ctx_t ctx, const double *xyz, int nv, const int *tri, int nt,
                       bemgpu_geom_t *out) {
  if (!ctx || !xyz || !tri || !out || nv < 3 || nt < 1)
    return bem_fail(ctx, BEMGPU_ERR_ARG, "geom_create: bad arguments");
  for (int i = 0; i < 3 * nt; i++)
    if (tri[i] < 0 || tri[i] >= nv) return bem_fail(ctx, BEMGPU_ERR_MESH, "geom_create: vertex id out of range");
  for (int i = 0; i < 3 * nv; i++)
    if (!std::isfinite(xyz[i])) return bem_fail(ctx, BEMGPU_ERR_MESH, "geom_create: non-finite coordinate");
  bemgpu_geom_s *g = new bemgpu_geom_s();
  g->ctx = ctx;
  g->nv = nv;
  g->nt = nt;
  g->xyz.assign(xyz, xyz + 3 * (size_t)nv);
  g->tri.assign(tri, tri + 3 * (size_t)nt);
  g->tris_at_vertex.resize(nv);
  for (int t = 0; t < nt; t++)
    for (int k = 0; k < 3; k++) g->tris_at_vertex[tri[3 * t + k]].push_back(t);
  {
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->refs++;
  }
  *out = g;
  return BEMGPU_OK;
}

// The geometry is freed when its handle and every tree over it are destroyed,
// in whatever order a caller's garbage collector finalizes them.
// Called with ctx->mu held; returns true when the geometry was freed (the
// caller then drops the geometry's reference on the context, unlocked).
// Device memory it held goes to `dead` (the caller defers its free).
static bool geom_release(bemgpu_geom_s *g, std::vector<std::pair<void *, size_t>> &dead) {
  if (--g->refs == 0) {
    for (auto &kv : g->near_cache) dead.emplace_back(kv.second.d, sizeof(NearPair) * (size_t)kv.second.n);
    delete g;
    return true;
  }
  return false;
}

int bemgpu_geom_destroy(bemgpu_geom_t g) {
  if (!g) return BEMGPU_ERR_ARG;
  bemgpu_ctx_s *ctx = g->ctx;
  const int device = ctx->device;
  bool freed;
  std::vector<std::pair<void *, size_t>> dead;
  {
    std::lock_guard<std::mutex> lk(ctx->mu);
    freed = geom_release(g, dead);
  }
  for (auto &d : dead) bem_defer_free(device, d.first, d.second);
  if (freed) ctx_release(ctx);
  return BEMGPU_OK;
}

int bemgpu_tree_create(bemgpu_geom_t g, const int *rwg, int nrwg, bemgpu_tree_t *out) {
  if (!g || !rwg || !out || nrwg < 1) return bem_fail(g ? g->ctx : nullptr, BEMGPU_ERR_ARG, "tree_create: bad arguments");
  bemgpu_ctx_s *ctx = g->ctx;
  *out = nullptr;
  bemgpu_tree_s *t = new bemgpu_tree_s();
  t->ctx = ctx;
  t->geom = g;
  t->nrwg = nrwg;
  t->rwg.assign(rwg, rwg + 4 * (size_t)nrwg);
  std::vector<int> local(g->nt, -1);
  // TriangleRWGMap construction order (src/Impedance.cpp:397-406)
  for (int i = 0; i < nrwg; i++) {
    int tp = rwg[4 * i], tn = rwg[4 * i + 1], e1 = rwg[4 * i + 2], e2 = rwg[4 * i + 3];
    if (tp < 0 || tp >= g->nt || tn < 0 || tn >= g->nt || tp == tn || e1 == e2 || e1 < 0 || e2 < 0 ||
        e1 >= g->nv || e2 >= g->nv) {
      delete t;
      return bem_fail(ctx, BEMGPU_ERR_MESH, "tree_create: RWG %d has invalid ids", i);
    }
    for (int side = 0; side < 2; side++) {
      int tr = side == 0 ? tp : tn;
      const int *tv = &g->tri[3 * tr];
      int has1 = (tv[0] == e1) + (tv[1] == e1) + (tv[2] == e1);
      int has2 = (tv[0] == e2) + (tv[1] == e2) + (tv[2] == e2);
      if (has1 != 1 || has2 != 1) {
        delete t;
        return bem_fail(ctx, BEMGPU_ERR_MESH, "tree_create: RWG %d edge is not on triangle %d", i, tr);
      }
      if (local[tr] < 0) {
        local[tr] = t->ntri++;
        t->tri_gid.push_back(tr);
        TriRec r;
        memset(&r, 0, sizeof r);
        r.gid = tr;
        t->host_rec.push_back(r);
      }
      TriRec &r = t->host_rec[local[tr]];
      if (r.nh >= 3) {
        delete t;
        return bem_fail(ctx, BEMGPU_ERR_MESH, "tree_create: triangle %d carries more than 3 RWGs", tr);
      }
      // HalfRWG::HalfRWG (src/RWG.cpp:9-21): p0 off the edge, p1/p2 follow the
      // triangle's vertex cycle.
      int rot = (tv[0] != e1 && tv[0] != e2) ? 0 : ((tv[1] != e1 && tv[1] != e2) ? 1 : 2);
      V3 p0 = vtx(g, tv[rot]), p1 = vtx(g, tv[(rot + 1) % 3]), p2 = vtx(g, tv[(rot + 2) % 3]);
      int h = r.nh++;
      put(r.hp0[h], p0);
      r.helen[h] = std::sqrt(norm2(sub(vtx(g, e2), vtx(g, e1))));  // Edge::length
      r.hrwg[h] = i;
      r.hneg[h] = side;
      if (h == 0) {
        V3 v01 = sub(p1, p0), v12 = sub(p2, p1), v20 = sub(p0, p2), v02 = sub(p2, p0);
        r.nv01i = 1. / std::sqrt(norm2(v01));
        r.nv12i = 1. / std::sqrt(norm2(v12));
        r.nv20i = 1. / std::sqrt(norm2(v20));
        V3 n = cross(v01, v02);
        double A2 = std::sqrt(norm2(n));
        n = scale(1. / A2, n);
        r.Ai = 2.0 / A2;
        put(r.p0, p0); put(r.p1, p1); put(r.p2, p2);
        put(r.v01, v01); put(r.v12, v12); put(r.v20, v20); put(r.v02, v02);
        put(r.n, n);
        put(r.m01, normalized(cross(v01, n)));
        put(r.m12, normalized(cross(v12, n)));
        put(r.m20, normalized(cross(v20, n)));
        r.elen0 = r.helen[0];
        // center, src/Triangle.cpp:30-34; edge lengths, src/ShapeMesh.cpp:938-943
        V3 a = vtx(g, tv[0]), b = vtx(g, tv[1]), c = vtx(g, tv[2]);
        put(r.c, scale(BEM_ONETHIRD, add(add(a, b), c)));
        r.emax = std::max(std::max(std::sqrt(norm2(sub(b, a))), std::sqrt(norm2(sub(c, b)))),
                          std::sqrt(norm2(sub(a, c))));
        r.vid[0] = tv[0]; r.vid[1] = tv[1]; r.vid[2] = tv[2];
      }
    }
  }
  for (const TriRec &r : t->host_rec)
    if (!(std::isfinite(r.Ai) && r.Ai > 0)) {
      delete t;
      return bem_fail(ctx, BEMGPU_ERR_MESH, "tree_create: degenerate triangle %d", r.gid);
    }
  cudaSetDevice(ctx->device);
  if (cudaMalloc(&t->d_rec, sizeof(TriRec) * t->ntri) != cudaSuccess) {
    cudaGetLastError();
    delete t;
    return bem_fail(ctx, BEMGPU_ERR_OOM, "tree_create: device allocation failed");
  }
  // complete on return (a copy from pageable memory may return before it
  // lands, and any context's stream may read the records next)
  if (cudaMemcpyAsync(t->d_rec, t->host_rec.data(), sizeof(TriRec) * t->ntri, cudaMemcpyHostToDevice,
                      ctx->stream) != cudaSuccess ||
      cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
    cudaFree(t->d_rec);
    delete t;
    return bem_fail(ctx, BEMGPU_ERR_CUDA, "tree_create: upload failed");
  }
  {
    std::lock_guard<std::mutex> lk(ctx->mu);
    g->refs++;
  }
  *out = t;
  return BEMGPU_OK;
}

int bemgpu_tree_destroy(bemgpu_tree_t t) {
  if (!t) return BEMGPU_ERR_ARG;
  bemgpu_ctx_s *ctx = t->ctx;
  const int device = ctx->device;
  bool geom_freed;
  // any context may still have kernels in flight that read the tree: its
  // device memory is freed later, after a device synchronisation (deferred
  // frees), not here
  std::vector<std::pair<void *, size_t>> dead;
  {
    std::lock_guard<std::mutex> lk(ctx->mu);
    bemgpu_geom_s *g = t->geom;
    {
      std::lock_guard<std::mutex> lc(g->cache_mu);
      for (auto it = g->far_rule_cache.begin(); it != g->far_rule_cache.end();) {
        if (it->first.first == t || it->first.second == t) it = g->far_rule_cache.erase(it);
        else ++it;
      }
      for (auto it = g->near_cache.begin(); it != g->near_cache.end();) {
        if (it->first.first == t || it->first.second == t) {
          dead.emplace_back(it->second.d, sizeof(NearPair) * (size_t)it->second.n);
          it = g->near_cache.erase(it);
        } else {
          ++it;
        }
      }
    }
    dead.emplace_back(t->d_rec, sizeof(TriRec) * (size_t)t->ntri);
    geom_freed = geom_release(t->geom, dead);
    delete t;
  }
  for (auto &d : dead) bem_defer_free(device, d.first, d.second);
  if (geom_freed) ctx_release(ctx);
  return BEMGPU_OK;
}

int bemgpu_ctx_set_tuning(bemgpu_ctx_t ctx, int knob, int value) {
  if (!ctx) return BEMGPU_ERR_ARG;
  std::lock_guard<std::mutex> lk(ctx->mu);
  switch (knob) {
    case BEMGPU_TUNE_NEAR_MINB:
      if (value < 2 || value > 4) return bem_fail(ctx, BEMGPU_ERR_ARG, "tuning: near_minb %d not in 2..4", value);
      ctx->tune.near_minb = value;
      return BEMGPU_OK;
    case BEMGPU_TUNE_FAR_ROWS:
      if (value != 1 && value != 2 && value != 4 && value != 8)
        return bem_fail(ctx, BEMGPU_ERR_ARG, "tuning: far_rows %d not 1, 2, 4 or 8", value);
      ctx->tune.far_rows = value;
      return BEMGPU_OK;
    case BEMGPU_TUNE_RASTER:
      if (value < 1 || value > 64) return bem_fail(ctx, BEMGPU_ERR_ARG, "tuning: raster %d not in 1..64", value);
      ctx->tune.raster = value;
      return BEMGPU_OK;
    case BEMGPU_TUNE_PANEL_CTAS:
      if (value < 0 || value > 1024) return bem_fail(ctx, BEMGPU_ERR_ARG, "tuning: panel_ctas %d not in 0..1024", value);
      ctx->tune.panel_ctas = value;
      return BEMGPU_OK;
    case BEMGPU_TUNE_NEAR_SYNC:
      if (value < 0 || value > 1) return bem_fail(ctx, BEMGPU_ERR_ARG, "tuning: near_sync %d not 0 or 1", value);
      ctx->tune.near_sync = value;
      return BEMGPU_OK;
    case BEMGPU_TUNE_NEAR_GRID:
      if (value < 1 || value > 64) return bem_fail(ctx, BEMGPU_ERR_ARG, "tuning: near_grid %d not in 1..64", value);
      ctx->tune.near_grid = value;
      return BEMGPU_OK;
    case BEMGPU_TUNE_EX_WIDE:
      if (value < 0 || value > 2) return bem_fail(ctx, BEMGPU_ERR_ARG, "tuning: ex_wide %d not 0, 1 or 2", value);
      ctx->tune.ex_wide = value;
      return BEMGPU_OK;
    case BEMGPU_TUNE_LU_SUPER:
      if (value < 0 || value > 1) return bem_fail(ctx, BEMGPU_ERR_ARG, "tuning: lu_super %d not 0 or 1", value);
      ctx->tune.lu_super = value;
      return BEMGPU_OK;
    default:
      return bem_fail(ctx, BEMGPU_ERR_ARG, "tuning: unknown knob %d", knob);
  }
}

int bemgpu_ctx_get_tuning(bemgpu_ctx_t ctx, int knob, int *value) {
  if (!ctx || !value) return BEMGPU_ERR_ARG;
  switch (knob) {
    case BEMGPU_TUNE_NEAR_MINB: *value = ctx->tune.near_minb; return BEMGPU_OK;
    case BEMGPU_TUNE_FAR_ROWS: *value = ctx->tune.far_rows; return BEMGPU_OK;
    case BEMGPU_TUNE_RASTER: *value = ctx->tune.raster; return BEMGPU_OK;
    case BEMGPU_TUNE_PANEL_CTAS: *value = ctx->tune.panel_ctas; return BEMGPU_OK;
    case BEMGPU_TUNE_NEAR_SYNC: *value = ctx->tune.near_sync; return BEMGPU_OK;
    case BEMGPU_TUNE_NEAR_GRID: *value = ctx->tune.near_grid; return BEMGPU_OK;
    case BEMGPU_TUNE_EX_WIDE: *value = ctx->tune.ex_wide; return BEMGPU_OK;
    case BEMGPU_TUNE_LU_SUPER: *value = ctx->tune.lu_super; return BEMGPU_OK;
    default: return bem_fail(ctx, BEMGPU_ERR_ARG, "tuning: unknown knob %d", knob);
  }
}

int bemgpu_tree_size(bemgpu_tree_t t) { return t ? t->nrwg : BEMGPU_ERR_ARG; }

int bemgpu_tree_rwgs(bemgpu_tree_t t, int *rwg, int cap) {
  if (!t || cap < 0 || (cap > 0 && !rwg)) return BEMGPU_ERR_ARG;
  const int n = std::min(cap, t->nrwg);
  std::copy(t->rwg.begin(), t->rwg.begin() + 4 * (size_t)n, rwg);
  return t->nrwg;
}

// Edge creation of ShapeMesh::ShapeMesh (src/ShapeMesh.cpp:857-928): the
// triangles are visited in order, and each edge (v0,v1), (v1,v2), (v2,v0) of
// the current triangle whose other triangle has not been visited yet becomes
// an RWG (current triangle positive, src/RWG.cpp:5).  A triangle is visited
// before every triangle of larger index, so "not visited" is "larger index".
// The edge -> triangles map is a sort of the 3 nt directed edges by their
// undirected key instead of the reference's per-vertex edge lists.
int bemgpu_mesh_rwgs(const int *tri, int nt, int nv, int *rwg, int cap, int *nrwg) {
  if (!tri || !nrwg || nt < 1 || nv < 3 || cap < 0 || (cap > 0 && !rwg)) return BEMGPU_ERR_ARG;
  *nrwg = 0;
  const size_t ne = 3 * (size_t)nt;
  std::vector<std::pair<uint64_t, uint32_t>> e(ne);  // (undirected key, 3 t + k)
  for (size_t s = 0; s < ne; s++) {
    int u = tri[s], v = tri[s - s % 3 + (s % 3 + 1) % 3];
    if (u < 0 || u >= nv || v < 0 || v >= nv || u == v) return BEMGPU_ERR_MESH;
    uint64_t lo = (uint64_t)std::min(u, v), hi = (uint64_t)std::max(u, v);
    e[s] = {lo << 32 | hi, (uint32_t)s};
  }
  std::sort(e.begin(), e.end());
  std::vector<int> other(ne, -1);
  for (size_t i = 0; i < ne;) {
    size_t j = i;
    while (j < ne && e[j].first == e[i].first) j++;
    // a closed 2-manifold has exactly two triangles on every edge
    if (j - i != 2) return BEMGPU_ERR_MESH;
    uint32_t a = e[i].second, b = e[i + 1].second;
    if (a / 3 == b / 3) return BEMGPU_ERR_MESH;
    other[a] = (int)(b / 3);
    other[b] = (int)(a / 3);
    i = j;
  }
  int n = 0;
  for (size_t s = 0; s < ne; s++) {
    int t = (int)(s / 3), nb = other[s];
    if (nb <= t) continue;
    if (n < cap) {
      rwg[4 * (size_t)n + 0] = t;
      rwg[4 * (size_t)n + 1] = nb;
      rwg[4 * (size_t)n + 2] = tri[s];
      rwg[4 * (size_t)n + 3] = tri[s - s % 3 + (s % 3 + 1) % 3];
    }
    n++;
  }
  *nrwg = n;
  return n <= cap ? BEMGPU_OK : BEMGPU_ERR_ARG;
}

int bemgpu_green_init(const double eps[2], const double mu[2], const double omega[2], int external,
                      bemgpu_green_t *out) {
  if (!eps || !mu || !omega || !out) return BEMGPU_ERR_ARG;
  typedef std::complex<double> C;
  C e(eps[0], eps[1]), m(mu[0], mu[1]), w(omega[0], omega[1]), I(0., 1.);
  // GreensFunction::init, src/GreensFunction.cpp:17-30
  C ksq = e * m * w * w;
  C k = std::sqrt(ksq);
  C ik = I * k;
  C k2 = -0.5 * ksq;
  C Zeps = 1. / (I * w * e);
  C Zmu = 1. / (I * w * m);
  auto st = [](double *d, C v) { d[0] = v.real(); d[1] = v.imag(); };
  st(out->eps, e); st(out->mu, m); st(out->omega, w);
  st(out->ksquared, ksq); st(out->k, k); st(out->ik, ik); st(out->k2, k2);
  st(out->Zeps, Zeps); st(out->Zmu, Zmu);
  out->external = external;
  return BEMGPU_OK;
}

void bemgpu_options_default(bemgpu_options_t *opt) {
  if (!opt) return;
  opt->farThresh6 = 12.0;
  opt->farThresh10 = 8.0;
  opt->farThresh15 = 4.0;
  opt->farThresh21 = 2.0;
}

double bemgpu_theta(double omega, double T) {
  return SI_HBAR * omega / (std::exp(SI_HBAR * omega / (SI_KB * T)) - 1);
}

double bemgpu_dimensionless_omega(double a, double eV) {
  double omegaSI = eV * SI_EV / SI_HBAR;
  return omegaSI * a / SI_C;
}

}  // extern "C"
