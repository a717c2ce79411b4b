// RWG set-up on the device: the RWG table of a closed body and the half-RWG
// frames of its triangles, built from the resident geometry by kernels instead
// of on the host (ShapeMesh::ShapeMesh edge creation, src/ShapeMesh.cpp:857-928,
// and HalfRWG::HalfRWG, src/RWG.cpp:7-39).
//
// Edge creation order (the reference's): triangles in order, and for each its
// edges (v0,v1), (v1,v2), (v2,v0); an edge whose other triangle comes later
// creates the next RWG {this triangle (positive), the other (negative), the
// edge's two vertices in this triangle's order}.  On the device:
//   1. every directed edge (3 per triangle) is inserted into an open-addressing
//      hash table keyed by its undirected vertex pair; the second insertion of
//      a key finds the first and the two record each other (a third one, an
//      edge without a partner, or a repeated edge is a mesh error);
//   2. an edge is an RWG creator when its partner's triangle comes later; an
//      exclusive scan over the creator flags in (triangle, edge) order gives
//      the RWG index, which both halves of the edge record;
//   3. each triangle's first appearance in the RWG table (2 r + side of its
//      smallest RWG) orders the triangles as the host builder does (the
//      TriangleRWGMap construction order, src/Impedance.cpp:393-406), and one
//      thread per triangle writes its record: the half-RWGs in RWG order, the
//      frame of the first one, the centroid and the longest edge.
// The frame arithmetic is the host builder's operation for operation, with
// explicitly rounded operations (no contraction into FMAs), so the records
// equal an uncontracted host evaluation bit for bit.
#include "bemgpu_internal.h"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace {

constexpr int SCAN_THREADS = 512;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

// out[i] = in[0] + ... + in[i-1] within each tile of SCAN_TILE; tile sums to sums[].
__global__ void __launch_bounds__(SCAN_THREADS) scan_tiles_kernel(const int *__restrict__ in, int *__restrict__ out,
                                                                  int n, int *__restrict__ sums) {
  __shared__ int warp_tot[SCAN_THREADS / 32];
  const int base = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_ITEMS;
  int v[SCAN_ITEMS], run = 0;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; k++) {
    v[k] = base + k < n ? in[base + k] : 0;
    run += v[k];
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int incl = run;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) warp_tot[wid] = incl;
  __syncthreads();
  if (wid == 0) {
    int w = lane < SCAN_THREADS / 32 ? warp_tot[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < SCAN_THREADS / 32) warp_tot[lane] = w;  // inclusive over warps
  }
  __syncthreads();
  int excl = incl - run + (wid > 0 ? warp_tot[wid - 1] : 0);
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; k++) {
    if (base + k < n) out[base + k] = excl;
    excl += v[k];
  }
  if (threadIdx.x == SCAN_THREADS - 1 && sums) sums[blockIdx.x] = warp_tot[SCAN_THREADS / 32 - 1];
}

__global__ void scan_add_kernel(int *__restrict__ out, int n, const int *__restrict__ offs) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] += offs[i / SCAN_TILE];
}

// Exclusive scan of n ints (device), the total to *total_dev.  tmp holds
// scan_tmp_ints(n) ints.
int64_t scan_tmp_ints(int64_t n) {
  int64_t tot = 0;
  while (n > 1) {
    n = (n + SCAN_TILE - 1) / SCAN_TILE;
    tot += 2 * n + 2;
  }
  return tot + 2;
}

void exclusive_scan(const int *in, int *out, int n, int *tmp, int *total_dev, cudaStream_t st, int64_t &launches) {
  const int tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
  int *sums = tmp, *sums_scan = tmp + tiles + 1;
  scan_tiles_kernel<<<tiles, SCAN_THREADS, 0, st>>>(in, out, n, sums);
  launches++;
  if (tiles > 1) {
    exclusive_scan(sums, sums_scan, tiles, tmp + 2 * tiles + 2, nullptr, st, launches);
    scan_add_kernel<<<(n + 255) / 256, 256, 0, st>>>(out, n, sums_scan);
    launches++;
  }
  if (total_dev) {
    // total = out[n-1] + in[n-1]
    cudaMemcpyAsync(total_dev, out + (n - 1), sizeof(int), cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(total_dev + 1, in + (n - 1), sizeof(int), cudaMemcpyDeviceToDevice, st);
  }
}

__device__ __forceinline__ unsigned long long mix64(unsigned long long x) {
  x ^= x >> 33;
  x *= 0xff51afd7ed558ccdull;
  x ^= x >> 33;
  x *= 0xc4ceb9fe1a85ec53ull;
  x ^= x >> 33;
  return x;
}

constexpr int VAL_BITS = 24;  // (3 t + e) + 1 in the low bits of a slot, the undirected key above

// Error codes of the set-up kernels (first one wins).
enum { MESH_OK = 0, MESH_BAD_EDGE = 1, MESH_NONMANIFOLD = 2, MESH_TABLE_FULL = 3, MESH_OPEN = 4 };

__device__ __forceinline__ void set_err(int *err, int code) { atomicCAS(err, 0, code); }

__global__ void edge_pair_kernel(const int *__restrict__ tri, int nt, int nv, unsigned long long *tab,
                                 unsigned long long mask, int *part, int *err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 3 * nt) return;
  const int t = i / 3, e = i - 3 * t;
  const int a = tri[i], b = tri[3 * t + (e + 1) % 3];
  if (a < 0 || b < 0 || a >= nv || b >= nv || a == b) {
    set_err(err, MESH_BAD_EDGE);
    return;
  }
  const unsigned long long key = (unsigned long long)min(a, b) * (unsigned long long)nv + (unsigned long long)max(a, b) + 1ull;
  const unsigned long long packed = (key << VAL_BITS) | (unsigned long long)(i + 1);
  unsigned long long h = mix64(key) & mask;
  for (unsigned long long probe = 0; probe <= mask; probe++) {
    const unsigned long long old = atomicCAS(&tab[h], 0ull, packed);
    if (old == 0ull) return;
    if ((old >> VAL_BITS) == key) {
      const int j = (int)(old & ((1ull << VAL_BITS) - 1)) - 1;
      if (j / 3 == t || atomicExch(&part[j], i) != -1 || atomicExch(&part[i], j) != -1) set_err(err, MESH_NONMANIFOLD);
      return;
    }
    h = (h + 1) & mask;
  }
  set_err(err, MESH_TABLE_FULL);
}

__global__ void creator_flags_kernel(const int *__restrict__ part, int nt, int *__restrict__ flags, int *err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 3 * nt) return;
  const int j = part[i];
  if (j < 0) {
    set_err(err, MESH_OPEN);
    flags[i] = 0;
    return;
  }
  flags[i] = (j / 3 > i / 3) ? 1 : 0;
}

__global__ void emit_rwgs_kernel(const int *__restrict__ tri, int nt, int tri0, const int *__restrict__ part,
                                 const int *__restrict__ flags, const int *__restrict__ pos, int *__restrict__ rwg,
                                 int *__restrict__ ridx) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 3 * nt || !flags[i]) return;
  const int t = i / 3, e = i - 3 * t, j = part[i], r = pos[i];
  rwg[4 * r + 0] = tri0 + t;
  rwg[4 * r + 1] = tri0 + j / 3;
  rwg[4 * r + 2] = tri[i];
  rwg[4 * r + 3] = tri[3 * t + (e + 1) % 3];
  ridx[i] = r;
  ridx[j] = r;
}

// first appearance of triangle t in the RWG table: 2 r + side of its smallest RWG
__global__ void first_appearance_kernel(const int *__restrict__ ridx, const int *__restrict__ flags, int nt,
                                        int *__restrict__ first) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt) return;
  int key = 0x7fffffff;
  for (int e = 0; e < 3; e++) key = min(key, 2 * ridx[3 * t + e] + (flags[3 * t + e] ? 0 : 1));
  first[key] = t;
}

__global__ void occupied_kernel(const int *__restrict__ first, int n, int *__restrict__ occ) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) occ[k] = first[k] >= 0 ? 1 : 0;
}

struct D3 {
  double x, y, z;
};
__device__ __forceinline__ D3 dsub(D3 a, D3 b) { return {__dsub_rn(a.x, b.x), __dsub_rn(a.y, b.y), __dsub_rn(a.z, b.z)}; }
__device__ __forceinline__ D3 dadd(D3 a, D3 b) { return {__dadd_rn(a.x, b.x), __dadd_rn(a.y, b.y), __dadd_rn(a.z, b.z)}; }
__device__ __forceinline__ D3 dscale(double c, D3 a) { return {__dmul_rn(c, a.x), __dmul_rn(c, a.y), __dmul_rn(c, a.z)}; }
__device__ __forceinline__ D3 dcross(D3 a, D3 b) {
  return {__dsub_rn(__dmul_rn(a.y, b.z), __dmul_rn(a.z, b.y)), __dsub_rn(__dmul_rn(a.z, b.x), __dmul_rn(a.x, b.z)),
          __dsub_rn(__dmul_rn(a.x, b.y), __dmul_rn(a.y, b.x))};
}
__device__ __forceinline__ double dnorm2(D3 a) {
  return __dadd_rn(__dadd_rn(__dmul_rn(a.x, a.x), __dmul_rn(a.y, a.y)), __dmul_rn(a.z, a.z));
}
__device__ __forceinline__ D3 dnormalized(D3 a) {
  const double ni = __ddiv_rn(1.0, __dsqrt_rn(dnorm2(a)));
  return {__dmul_rn(a.x, ni), __dmul_rn(a.y, ni), __dmul_rn(a.z, ni)};
}
__device__ __forceinline__ void dput(double *d, D3 a) { d[0] = a.x; d[1] = a.y; d[2] = a.z; }
__device__ __forceinline__ D3 dvtx(const double *xyz, int i) { return {xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]}; }

// One triangle record (the host builder's bemgpu_tree_create, per triangle).
__global__ void tri_records_kernel(const double *__restrict__ xyz, const int *__restrict__ tri, int tri0,
                                   const int *__restrict__ rwg, const int *__restrict__ ridx,
                                   const int *__restrict__ flags, const int *__restrict__ first,
                                   const int *__restrict__ occ_pos, int nfirst, TriRec *__restrict__ recs,
                                   int *err) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nfirst) return;
  const int t = first[k];
  if (t < 0) return;
  TriRec r;
  memset(&r, 0, sizeof r);
  const int *tv = tri + 3 * t;  // geometry vertex ids
  // the three half-RWGs in RWG order
  int hr[3], hs[3];
  for (int e = 0; e < 3; e++) {
    hr[e] = ridx[3 * t + e];
    hs[e] = flags[3 * t + e] ? 0 : 1;
  }
  for (int a = 0; a < 2; a++)
    for (int b = 0; b < 2 - a; b++)
      if (hr[b] > hr[b + 1]) {
        int x = hr[b]; hr[b] = hr[b + 1]; hr[b + 1] = x;
        x = hs[b]; hs[b] = hs[b + 1]; hs[b + 1] = x;
      }
  r.gid = tri0 + t;
  r.nh = 3;
  for (int h = 0; h < 3; h++) {
    const int i = hr[h];
    const int e1 = rwg[4 * i + 2], e2 = rwg[4 * i + 3];
    const int rot = (tv[0] != e1 && tv[0] != e2) ? 0 : ((tv[1] != e1 && tv[1] != e2) ? 1 : 2);
    const D3 p0 = dvtx(xyz, tv[rot]), p1 = dvtx(xyz, tv[(rot + 1) % 3]), p2 = dvtx(xyz, tv[(rot + 2) % 3]);
    dput(r.hp0[h], p0);
    r.helen[h] = __dsqrt_rn(dnorm2(dsub(dvtx(xyz, e2), dvtx(xyz, e1))));
    r.hrwg[h] = i;
    r.hneg[h] = hs[h];
    if (h == 0) {
      const D3 v01 = dsub(p1, p0), v12 = dsub(p2, p1), v20 = dsub(p0, p2), v02 = dsub(p2, p0);
      r.nv01i = __ddiv_rn(1.0, __dsqrt_rn(dnorm2(v01)));
      r.nv12i = __ddiv_rn(1.0, __dsqrt_rn(dnorm2(v12)));
      r.nv20i = __ddiv_rn(1.0, __dsqrt_rn(dnorm2(v20)));
      D3 n = dcross(v01, v02);
      const double A2 = __dsqrt_rn(dnorm2(n));
      n = dscale(__ddiv_rn(1.0, A2), n);
      r.Ai = __ddiv_rn(2.0, A2);
      dput(r.p0, p0); dput(r.p1, p1); dput(r.p2, p2);
      dput(r.v01, v01); dput(r.v12, v12); dput(r.v20, v20); dput(r.v02, v02);
      dput(r.n, n);
      dput(r.m01, dnormalized(dcross(v01, n)));
      dput(r.m12, dnormalized(dcross(v12, n)));
      dput(r.m20, dnormalized(dcross(v20, n)));
      r.elen0 = r.helen[0];
      const D3 a = dvtx(xyz, tv[0]), b = dvtx(xyz, tv[1]), c = dvtx(xyz, tv[2]);
      dput(r.c, dscale(BEM_ONETHIRD, dadd(dadd(a, b), c)));
      r.emax = fmax(fmax(__dsqrt_rn(dnorm2(dsub(b, a))), __dsqrt_rn(dnorm2(dsub(c, b)))),
                    __dsqrt_rn(dnorm2(dsub(a, c))));
      r.vid[0] = tv[0]; r.vid[1] = tv[1]; r.vid[2] = tv[2];
    }
  }
  if (!(r.Ai > 0.0) || !isfinite(r.Ai)) set_err(err, MESH_BAD_EDGE);
  recs[occ_pos[k]] = r;
}

// The two-body tree's records: a's, then b's with their RWG indices moved past a's.
__global__ void concat_records_kernel(const TriRec *__restrict__ ra, int na, const TriRec *__restrict__ rb, int nb,
                                      int offset, TriRec *__restrict__ out) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < na) {
    out[k] = ra[k];
  } else if (k < na + nb) {
    TriRec r = rb[k - na];
    for (int h = 0; h < 3; h++)
      if (h < r.nh) r.hrwg[h] += offset;
    out[k] = r;
  }
}

const char *mesh_err_text(int code) {
  switch (code) {
    case MESH_BAD_EDGE: return "a triangle with a repeated or out-of-range vertex, or of zero area";
    case MESH_NONMANIFOLD: return "an edge shared by more than two triangles";
    case MESH_TABLE_FULL: return "edge hash table full";
    case MESH_OPEN: return "an edge with a single triangle (the body is not closed)";
    default: return "unknown";
  }
}

struct DevBufs {
  std::vector<void *> p;
  ~DevBufs() {
    for (void *q : p) cudaFree(q);
  }
  template <typename T>
  T *get(size_t count) {
    void *q = nullptr;
    if (cudaMalloc(&q, count * sizeof(T) + 16) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    p.push_back(q);
    return (T *)q;
  }
};

bemgpu_tree_s *new_tree(bemgpu_geom_s *g) {
  bemgpu_tree_s *t = new bemgpu_tree_s();
  t->ctx = g->ctx;
  t->geom = g;
  return t;
}

}  // namespace

extern "C" int bemgpu_tree_create_body_device(bemgpu_geom_t g, int tri0, int ntri, bemgpu_tree_t *out) {
  if (!g || !out) return BEMGPU_ERR_ARG;
  bemgpu_ctx_s *ctx = g->ctx;
  *out = nullptr;
  if (tri0 < 0 || ntri < 4 || tri0 + ntri > g->nt)
    return bem_fail(ctx, BEMGPU_ERR_ARG, "tree_create_body_device: triangles [%d, %d) outside 0..%d", tri0,
                    tri0 + ntri, g->nt);
  if (g->nv >= (1 << 20) || 3 * (int64_t)ntri >= (1 << VAL_BITS) - 1)
    return bem_fail(ctx, BEMGPU_ERR_ARG, "tree_create_body_device: at most 2^20 vertices and 5592404 triangles");
  const int ne = 3 * ntri;
  cudaSetDevice(ctx->device);
  cudaStream_t st = ctx->stream;
  std::lock_guard<std::mutex> lk(ctx->mu);
  DevBufs B;
  unsigned long long cap = 1;
  while (cap < 2ull * (unsigned long long)ne) cap <<= 1;
  const int nfirst = ne + 2;  // 2 nrwg = 3 ntri for a closed body
  double *xyz = B.get<double>(3 * (size_t)g->nv);
  int *tri = B.get<int>(ne);
  unsigned long long *tab = B.get<unsigned long long>(cap);
  int *part = B.get<int>(ne), *flags = B.get<int>(ne), *pos = B.get<int>(ne), *ridx = B.get<int>(ne);
  int *rwg = B.get<int>(2 * (size_t)ne);
  int *first = B.get<int>(nfirst), *occ = B.get<int>(nfirst), *occ_pos = B.get<int>(nfirst);
  int *tmp = B.get<int>(scan_tmp_ints(nfirst));
  int *info = B.get<int>(8);  // [0] error, [2..3] RWG count pieces, [4..5] triangle count pieces
  TriRec *recs = B.get<TriRec>(ntri);
  if (!xyz || !tri || !tab || !part || !flags || !pos || !ridx || !rwg || !first || !occ || !occ_pos || !tmp ||
      !info || !recs)
    return bem_fail(ctx, BEMGPU_ERR_OOM, "tree_create_body_device: device allocation failed");
  BEM_CUDA_TRY(ctx, cudaMemcpyAsync(xyz, g->xyz.data(), sizeof(double) * 3 * (size_t)g->nv, cudaMemcpyHostToDevice, st));
  BEM_CUDA_TRY(ctx, cudaMemcpyAsync(tri, g->tri.data() + 3 * (size_t)tri0, sizeof(int) * ne, cudaMemcpyHostToDevice, st));
  BEM_CUDA_TRY(ctx, cudaMemsetAsync(tab, 0, sizeof(unsigned long long) * cap, st));
  BEM_CUDA_TRY(ctx, cudaMemsetAsync(part, 0xff, sizeof(int) * ne, st));
  BEM_CUDA_TRY(ctx, cudaMemsetAsync(first, 0xff, sizeof(int) * nfirst, st));
  BEM_CUDA_TRY(ctx, cudaMemsetAsync(info, 0, sizeof(int) * 8, st));
  const int tb = 256;
  edge_pair_kernel<<<(ne + tb - 1) / tb, tb, 0, st>>>(tri, ntri, g->nv, tab, cap - 1, part, info);
  creator_flags_kernel<<<(ne + tb - 1) / tb, tb, 0, st>>>(part, ntri, flags, info);
  ctx->launches += 2;
  exclusive_scan(flags, pos, ne, tmp, info + 2, st, ctx->launches);
  int h_info[8];
  BEM_CUDA_TRY(ctx, cudaMemcpyAsync(h_info, info, sizeof(h_info), cudaMemcpyDeviceToHost, st));
  BEM_CUDA_TRY(ctx, cudaStreamSynchronize(st));
  if (h_info[0]) return bem_fail(ctx, BEMGPU_ERR_MESH, "tree_create_body_device: %s", mesh_err_text(h_info[0]));
  const int nrwg = h_info[2] + h_info[3];
  if (2 * nrwg != ne) return bem_fail(ctx, BEMGPU_ERR_MESH, "tree_create_body_device: %d RWGs for %d triangles", nrwg, ntri);
  emit_rwgs_kernel<<<(ne + tb - 1) / tb, tb, 0, st>>>(tri, ntri, tri0, part, flags, pos, rwg, ridx);
  first_appearance_kernel<<<(ntri + tb - 1) / tb, tb, 0, st>>>(ridx, flags, ntri, first);
  occupied_kernel<<<(nfirst + tb - 1) / tb, tb, 0, st>>>(first, nfirst, occ);
  ctx->launches += 3;
  exclusive_scan(occ, occ_pos, nfirst, tmp, info + 4, st, ctx->launches);
  // the records need the geometry's own vertex ids: tri holds them (tri0 offset only on triangle ids)
  tri_records_kernel<<<(nfirst + tb - 1) / tb, tb, 0, st>>>(xyz, tri, tri0, rwg, ridx, flags, first, occ_pos, nfirst,
                                                             recs, info);
  ctx->launches++;
  BEM_CUDA_TRY(ctx, cudaGetLastError());
  bemgpu_tree_s *t = new_tree(g);
  t->nrwg = nrwg;
  t->ntri = ntri;
  t->rwg.resize(4 * (size_t)nrwg);
  t->host_rec.resize(ntri);
  BEM_CUDA_TRY(ctx, cudaMemcpyAsync(h_info, info, sizeof(h_info), cudaMemcpyDeviceToHost, st));
  if (cudaMemcpyAsync(t->rwg.data(), rwg, sizeof(int) * 4 * (size_t)nrwg, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaMemcpyAsync(t->host_rec.data(), recs, sizeof(TriRec) * ntri, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess) {
    cudaGetLastError();
    delete t;
    return bem_fail(ctx, BEMGPU_ERR_CUDA, "tree_create_body_device: copy back failed");
  }
  if (h_info[0] || h_info[4] + h_info[5] != ntri) {
    delete t;
    return bem_fail(ctx, BEMGPU_ERR_MESH, "tree_create_body_device: %s",
                    h_info[0] ? mesh_err_text(h_info[0]) : "triangle without RWGs");
  }
  t->tri_gid.resize(ntri);
  for (int k = 0; k < ntri; k++) t->tri_gid[k] = t->host_rec[k].gid;
  // the records stay on the device: the tree takes the buffer over
  for (auto it = B.p.begin(); it != B.p.end(); ++it)
    if (*it == (void *)recs) {
      B.p.erase(it);
      break;
    }
  t->d_rec = recs;
  g->refs++;  // the tree keeps its geometry (ctx->mu is held)
  *out = t;
  return BEMGPU_OK;
}

extern "C" int bemgpu_tree_concat(bemgpu_tree_t a, bemgpu_tree_t b, bemgpu_tree_t *out) {
  if (!a || !b || !out) return BEMGPU_ERR_ARG;
  bemgpu_ctx_s *ctx = a->ctx;
  *out = nullptr;
  if (a->geom != b->geom) return bem_fail(ctx, BEMGPU_ERR_ARG, "tree_concat: the trees must share one geometry");
  for (int x : a->tri_gid)
    if (std::find(b->tri_gid.begin(), b->tri_gid.end(), x) != b->tri_gid.end())
      return bem_fail(ctx, BEMGPU_ERR_ARG, "tree_concat: the trees share triangle %d", x);
  bemgpu_tree_s *t = new_tree(a->geom);
  t->nrwg = a->nrwg + b->nrwg;
  t->ntri = a->ntri + b->ntri;
  t->rwg = a->rwg;
  t->rwg.insert(t->rwg.end(), b->rwg.begin(), b->rwg.end());
  t->tri_gid = a->tri_gid;
  t->tri_gid.insert(t->tri_gid.end(), b->tri_gid.begin(), b->tri_gid.end());
  t->host_rec = a->host_rec;
  for (TriRec r : b->host_rec) {
    for (int h = 0; h < r.nh; h++) r.hrwg[h] += a->nrwg;
    t->host_rec.push_back(r);
  }
  cudaSetDevice(ctx->device);
  if (cudaMalloc(&t->d_rec, sizeof(TriRec) * t->ntri) != cudaSuccess) {
    cudaGetLastError();
    delete t;
    return bem_fail(ctx, BEMGPU_ERR_OOM, "tree_concat: device allocation failed");
  }
  std::lock_guard<std::mutex> lk(ctx->mu);
  concat_records_kernel<<<(t->ntri + 255) / 256, 256, 0, ctx->stream>>>(a->d_rec, a->ntri, b->d_rec, b->ntri, a->nrwg,
                                                                        t->d_rec);
  ctx->launches++;
  if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
    cudaFree(t->d_rec);
    delete t;
    return bem_fail(ctx, BEMGPU_ERR_CUDA, "tree_concat: record kernel failed");
  }
  a->geom->refs++;  // ctx->mu is held
  *out = t;
  return BEMGPU_OK;
}
