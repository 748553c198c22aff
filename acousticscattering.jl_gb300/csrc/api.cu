// C ABI of libbemgpu: contexts, meshes, factors, solutions and queries.
//
// Host orchestration of the device kernels.  Every batched operation builds device
// arrays of per-instance descriptors and issues one launch sequence for all instances;
// the only host decisions are the ones the reference makes between LAPACK calls
// (promotion of the mixed-precision factor, refinement acceptance).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <thread>
#include <tuple>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "bemgpu_internal.h"
#include "linalg.cuh"
#include "nystrom.cuh"
#include "refine.cuh"
#include "condition.cuh"
#include "gemm_tc.cuh"
#include "hmatrix.cuh"
#include "hmatrix_plan.h"
#include "pressure.cuh"
#include "solve_kernels.cuh"

namespace bemgpu {
constexpr int kTcPanel = 128;  // outer panel width of the tensor-core LU
static std::atomic<long long> g_launches{0};
void count_launch(int kernels) { g_launches.fetch_add(kernels, std::memory_order_relaxed); }
long long launch_total() { return g_launches.load(std::memory_order_relaxed); }
}  // namespace bemgpu

using namespace bemgpu;

namespace {
thread_local std::string g_err;
}  // namespace

namespace bemgpu {
void bemgpu_set_process_error(const char* msg) { g_err = msg ? msg : ""; }
}  // namespace bemgpu

// ===================================================================== context + memory
constexpr int kEventPool = 512;  // ordering events of the two-stream triangular solves

struct bemgpu_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  uint64_t budget = 0;
  uint64_t live = 0;   // bytes held by this context's own allocations
  uint64_t total = 0;  // root context: bytes held by it and its lanes (against budget)
  std::string err;
  cudaError_t last_cuda = cudaSuccess;  // CUDA error of the last failed call (cuda_fail)
  std::atomic<int32_t> inject_oom{0};   // root: allocations still to fail (test hook)
  int* d_err = nullptr;
  // free device blocks of this context, reused on its own stream(s) only (stream order
  // makes a block released with work still queued safe to hand out again)
  std::multimap<size_t, void*> cache;
  uint64_t cached = 0;
  std::mutex pool_mu;  // guards cache / cached
  std::mutex acct_mu;  // root context: guards live / total of it and its lanes
  // A lane is a child context of a serving loop: its own streams, events, timeout word
  // and block pool, so that batches on different lanes run concurrently; its memory
  // counts against the parent's budget.
  bemgpu_ctx* parent = nullptr;
  std::vector<bemgpu_ctx*> lanes;  // root: live lanes (guarded by lanes_mu)
  std::mutex lanes_mu;
  bool prof = false;
  bool tensor_lu = true;  // complex64 trailing updates on the tensor cores
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  std::map<std::string, std::vector<std::pair<cudaEvent_t, cudaEvent_t>>> events;
  // launch-shape autotuner: the fastest measured choice per (kernel family, shape class)
  std::map<std::string, int> tuned;
  bool autotune = true;

  // CUDA graphs of the tensor-core LU's launch sequence, one per exact batch shape
  // (getrf_tc); a shape is captured the second time it is met
  bool graphs = true;
  std::map<std::string, std::shared_ptr<struct LuGraph>> lu_graphs;
  std::map<std::string, int> lu_seen;
  uint64_t lu_tick = 0;
  int64_t lu_captures = 0, lu_replays = 0;

  std::recursive_mutex mu;
  cudaStream_t side = nullptr;           // look-ahead stream of the triangular solves
  std::vector<cudaEvent_t> evpool;       // their ordering events
  Launch launch() const {
    return Launch{stream, d_err, side, const_cast<cudaEvent_t*>(evpool.data()),
                  (int)evpool.size()};
  }
};

namespace {

int fail(bemgpu_ctx* c, int code, const std::string& msg) {
  if (c)
    c->err = msg;
  else
    g_err = msg;
  return code;
}

int cuda_fail(bemgpu_ctx* c, cudaError_t e, const char* what) {
  std::string m = std::string(what) + ": " + cudaGetErrorString(e);
  if (c) c->last_cuda = e;
  return fail(c, BEMGPU_ECUDA, m);
}

#define CUDA_TRY(c, call)                                   \
  do {                                                      \
    cudaError_t e_ = (call);                                \
    if (e_ != cudaSuccess) return cuda_fail((c), e_, #call); \
  } while (0)
#define TRY(x)                          \
  do {                                  \
    int s_ = (x);                       \
    if (s_ != BEMGPU_OK) return s_;     \
  } while (0)

size_t round_bytes(size_t b) {
  if (b == 0) b = 1;
  const size_t kSmall = size_t(1) << 20, kLarge = size_t(2) << 20;
  if (b <= kSmall) return (b + 4095) & ~size_t(4095);
  return (b + kLarge - 1) / kLarge * kLarge;
}

// Device buffer drawn from the context's caching pool and counted against its budget.
struct Buf {
  bemgpu_ctx* c = nullptr;
  void* p = nullptr;
  size_t bytes = 0;
  Buf() = default;
  Buf(const Buf&) = delete;
  Buf& operator=(const Buf&) = delete;
  Buf(Buf&& o) noexcept : c(o.c), p(o.p), bytes(o.bytes) {
    o.p = nullptr;
    o.bytes = 0;
  }
  Buf& operator=(Buf&& o) noexcept {
    if (this != &o) {
      release();
      c = o.c;
      p = o.p;
      bytes = o.bytes;
      o.p = nullptr;
      o.bytes = 0;
    }
    return *this;
  }
  ~Buf() { release(); }
  void release();
  template <class T>
  T* as() const {
    return static_cast<T*>(p);
  }
};

bemgpu_ctx* root_of(const bemgpu_ctx* c) {
  return const_cast<bemgpu_ctx*>(c->parent ? c->parent : c);
}

// Bytes held against the budget by a context and all lanes of its root.
uint64_t total_live(const bemgpu_ctx* c) {
  bemgpu_ctx* r = root_of(c);
  std::lock_guard<std::mutex> lk(r->acct_mu);
  return r->total;
}

void account(bemgpu_ctx* c, int64_t delta) {
  bemgpu_ctx* r = root_of(c);
  std::lock_guard<std::mutex> lk(r->acct_mu);
  r->total = (uint64_t)((int64_t)r->total + delta);
  c->live = (uint64_t)((int64_t)c->live + delta);
}

void Buf::release() {
  if (p && c) {
    {
      std::lock_guard<std::mutex> lk(c->pool_mu);
      c->cache.emplace(bytes, p);
      c->cached += bytes;
    }
    account(c, -(int64_t)bytes);
  }
  p = nullptr;
  bytes = 0;
}

// Frees the free blocks of one context.  A lane's block can be released with work still
// queued on that lane's stream, so the device is synchronised before anything is freed.
void drop_cache(bemgpu_ctx* c) {
  std::multimap<size_t, void*> blocks;
  {
    std::lock_guard<std::mutex> lk(c->pool_mu);
    blocks.swap(c->cache);
    c->cached = 0;
  }
  if (blocks.empty()) return;
  // a block whose free fails (or that cannot be freed because the device could not be
  // synchronised) goes back to the pool rather than being lost
  std::multimap<size_t, void*> kept;
  if (cudaDeviceSynchronize() != cudaSuccess) {
    cudaGetLastError();
    kept.swap(blocks);
  }
  for (auto& kv : blocks)
    if (cudaFree(kv.second) != cudaSuccess) {
      cudaGetLastError();
      kept.insert(kv);
    }
  if (kept.empty()) return;
  std::lock_guard<std::mutex> lk(c->pool_mu);
  for (auto& kv : kept) {
    c->cache.insert(kv);
    c->cached += kv.first;
  }
}

// Bytes of free blocks held by the pools of a root context and its lanes.
uint64_t pooled_bytes(bemgpu_ctx* c) {
  bemgpu_ctx* r = root_of(c);
  uint64_t b = 0;
  {
    std::lock_guard<std::mutex> lk(r->pool_mu);
    b += r->cached;
  }
  std::lock_guard<std::mutex> lk(r->lanes_mu);
  for (bemgpu_ctx* l : r->lanes) {
    std::lock_guard<std::mutex> pk(l->pool_mu);
    b += l->cached;
  }
  return b;
}

// Free blocks of the root context and every lane (when a cudaMalloc fails).
void drop_all_caches(bemgpu_ctx* c) {
  bemgpu_ctx* r = root_of(c);
  drop_cache(r);
  std::lock_guard<std::mutex> lk(r->lanes_mu);
  for (bemgpu_ctx* l : r->lanes) drop_cache(l);
}

// Streams, ordering events and timeout word of a context or lane (device current).
cudaError_t init_streams(bemgpu_ctx* c) {
  cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) return e;
  e = cudaMalloc(&c->d_err, sizeof(int));
  if (e != cudaSuccess) {
    cudaStreamDestroy(c->stream);
    c->stream = nullptr;
    return e;
  }
  cudaMemsetAsync(c->d_err, 0, sizeof(int), c->stream);
  // look-ahead stream and events of the blocked triangular solves (optional: without them
  // the solves run on the main stream alone)
  if (cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking) == cudaSuccess) {
    c->evpool.resize(kEventPool, nullptr);
    for (auto& ev : c->evpool)
      if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) ev = nullptr;
    if (std::any_of(c->evpool.begin(), c->evpool.end(), [](cudaEvent_t ev) { return !ev; })) {
      for (auto& ev : c->evpool)
        if (ev) cudaEventDestroy(ev);
      c->evpool.clear();
      cudaStreamDestroy(c->side);
      c->side = nullptr;
    }
  } else {
    c->side = nullptr;
  }
  cudaGetLastError();
  return cudaStreamSynchronize(c->stream);
}

void free_streams(bemgpu_ctx* c) {
  cudaStreamSynchronize(c->stream);
  c->lu_graphs.clear();  // their descriptor buffers go back to the pool first
  for (auto& kv : c->events)
    for (auto& pr : kv.second) {
      cudaEventDestroy(pr.first);
      cudaEventDestroy(pr.second);
    }
  c->events.clear();
  if (c->side) cudaStreamSynchronize(c->side);
  drop_cache(c);
  for (auto& ev : c->evpool) cudaEventDestroy(ev);
  c->evpool.clear();
  if (c->side) {
    cudaStreamDestroy(c->side);
    c->side = nullptr;
  }
  if (c->t0) cudaEventDestroy(c->t0);
  if (c->t1) cudaEventDestroy(c->t1);
  c->t0 = c->t1 = nullptr;
  if (c->d_err) cudaFree(c->d_err);
  c->d_err = nullptr;
  cudaStreamDestroy(c->stream);
  c->stream = nullptr;
}

// A lane of `parent` (see bemgpu_ctx::parent): settings copied, memory counted against
// the parent's budget.
int make_lane(bemgpu_ctx* parent, bemgpu_ctx** out) {
  cudaSetDevice(parent->device);
  auto* l = new bemgpu_ctx();
  l->device = parent->device;
  l->parent = parent;
  l->budget = parent->budget;
  l->tensor_lu = parent->tensor_lu;
  l->autotune = parent->autotune;
  l->tuned = parent->tuned;
  // lanes do not capture graphs: served batches rarely repeat a shape, and a capture on
  // one lane would forbid the device-wide synchronisation another lane's pool release
  // needs while it lasts
  l->graphs = false;
  cudaError_t e = init_streams(l);
  if (e != cudaSuccess) {
    delete l;
    return cuda_fail(parent, e, "lane streams");
  }
  {
    std::lock_guard<std::mutex> lk(parent->lanes_mu);
    parent->lanes.push_back(l);
  }
  *out = l;
  return BEMGPU_OK;
}

// Destroys a lane; every buffer allocated through it must have been released.
void destroy_lane(bemgpu_ctx* l) {
  bemgpu_ctx* parent = l->parent;
  {
    std::lock_guard<std::mutex> lk(parent->lanes_mu);
    parent->lanes.erase(std::remove(parent->lanes.begin(), parent->lanes.end(), l),
                        parent->lanes.end());
  }
  cudaSetDevice(l->device);
  free_streams(l);
  delete l;
}

int alloc(bemgpu_ctx* c, size_t bytes, Buf* out) {
  out->release();
  size_t rb = round_bytes(bytes);
  {
    bemgpu_ctx* r = root_of(c);
    std::lock_guard<std::mutex> lk(r->acct_mu);
    if (r->total + rb > r->budget) {
      char m[200];
      std::snprintf(m, sizeof m,
                    "HBM budget exceeded: %.3f GB live + %.3f GB requested > %.3f GB",
                    r->total / 1e9, rb / 1e9, r->budget / 1e9);
      return fail(c, BEMGPU_ENOMEM_BUDGET, m);
    }
    r->total += rb;
    c->live += rb;
  }
  void* p = nullptr;
  {
    std::atomic<int32_t>& inj = root_of(c)->inject_oom;
    int32_t left = inj.load();
    while (left > 0 && !inj.compare_exchange_weak(left, left - 1)) {
    }
    if (left > 0) {  // a failure requested by bemgpu_ctx_inject_alloc_failures
      account(c, -(int64_t)rb);
      return cuda_fail(c, cudaErrorMemoryAllocation, "cudaMalloc");
    }
  }
  {
    std::lock_guard<std::mutex> lk(c->pool_mu);
    auto it = c->cache.find(rb);
    if (it != c->cache.end()) {
      p = it->second;
      c->cache.erase(it);
      c->cached -= rb;
    }
  }
  if (!p) {
    cudaError_t e = cudaMalloc(&p, rb);
    if (e == cudaErrorMemoryAllocation) {
      cudaGetLastError();
      drop_cache(c);
      e = cudaMalloc(&p, rb);
    }
    if (e == cudaErrorMemoryAllocation) {
      cudaGetLastError();
      drop_all_caches(c);
      e = cudaMalloc(&p, rb);
    }
    if (e != cudaSuccess) {
      cudaGetLastError();
      account(c, -(int64_t)rb);
      if (e != cudaErrorMemoryAllocation) return cuda_fail(c, e, "cudaMalloc");
      size_t fr = 0, tot = 0;
      cudaMemGetInfo(&fr, &tot);
      char m[240];
      std::snprintf(m, sizeof m,
                    "cudaMalloc of %.3f GB (device: %.3f GB free of %.3f GB; this library: "
                    "%.3f GB live, %.3f GB in its pools)",
                    rb / 1e9, fr / 1e9, tot / 1e9, total_live(c) / 1e9, pooled_bytes(c) / 1e9);
      return cuda_fail(c, e, m);
    }
  }
  out->c = c;
  out->p = p;
  out->bytes = rb;
  return BEMGPU_OK;
}

template <class T>
int upload(bemgpu_ctx* c, const std::vector<T>& h, Buf* out) {
  TRY(alloc(c, h.size() * sizeof(T), out));
  if (!h.empty())
    CUDA_TRY(c, cudaMemcpyAsync(out->p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice,
                                c->stream));
  return BEMGPU_OK;
}

template <class T>
int download(bemgpu_ctx* c, const Buf& b, std::vector<T>* h, size_t count) {
  h->resize(count);
  if (count)
    CUDA_TRY(c, cudaMemcpyAsync(h->data(), b.p, count * sizeof(T), cudaMemcpyDeviceToHost,
                                c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return BEMGPU_OK;
}

int check_device_error(bemgpu_ctx* c) {
  int h = 0;
  CUDA_TRY(c, cudaMemcpyAsync(&h, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  CUDA_TRY(c, cudaGetLastError());
  if (h != 0) {
    cudaMemsetAsync(c->d_err, 0, sizeof(int), c->stream);
    return fail(c, BEMGPU_ETIMEOUT, "a bounded device wait gave up (kernel returned early)");
  }
  return BEMGPU_OK;
}

// Event pair around a family of launches when profiling is on.
struct Prof {
  bemgpu_ctx* c;
  const char* fam;
  cudaEvent_t a = nullptr, b = nullptr;
  Prof(bemgpu_ctx* c_, const char* f) : c(c_), fam(f) {
    if (c->prof) {
      cudaEventCreate(&a);
      cudaEventCreate(&b);
      cudaEventRecord(a, c->stream);
    }
  }
  ~Prof() {
    if (a) {
      cudaEventRecord(b, c->stream);
      c->events[fam].emplace_back(a, b);
    }
  }
};

// Phase timer (always on): elapsed device time between construction and stop().
struct Timer {
  cudaStream_t s;
  cudaEvent_t a = nullptr, b = nullptr;
  explicit Timer(cudaStream_t st) : s(st) {
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    cudaEventRecord(a, s);
  }
  double stop() {
    cudaEventRecord(b, s);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    return ms;
  }
  ~Timer() {
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
  }
};

}  // namespace

// ===================================================================== meshes
namespace {
struct MeshData {
  bemgpu_ctx* c = nullptr;
  int64_t n = 0, nn = 0;
  double resolution = 0.0;
  char hash[65] = {0};
  double center[3] = {0, 0, 0};
  std::vector<double> panels_h;  // FP64 records
  Buf panels, panelsf, verts, near_i, near_j, near_ptr, near_lap;
  int64_t n_near = 0;
  double eta = 2.0;
  std::vector<double> nodes_h;   // the surface as supplied (3 x nn, 1-based triangles)
  std::vector<int64_t> tris_h;
  Buf surf;                      // union of several surfaces: surface of every panel
  std::vector<int64_t> offsets;  // union: first panel of every surface (+ total)
  // compressed operators: cluster tree, block partition and near-pair destinations of
  // each (leaf size, admissibility eta), built on first use
  struct HmPlanCache {
    HmPlan plan;
    Buf perm, iperm, near_dst;
    Buf ny_dst;  // Nyström node sets: full-block offsets of every same-element pair
  };
  std::map<std::pair<int32_t, double>, std::shared_ptr<HmPlanCache>> hm_plans;
  // Nyström node set: one record per quadrature node (the panel-record layout with the
  // node as centroid and all seven Gauss points, its weight as area), built on first use
  bool nystrom = false;
  std::shared_ptr<MeshData> node_mesh;
};
}  // namespace

struct bemgpu_mesh {
  std::shared_ptr<MeshData> d;
};

namespace {
// Panel records of the device layout (bemgpu_internal.h).  Host arithmetic with
// separately rounded operations (built with -ffp-contract=off).
void build_panels(const double* nodes, const int64_t* tris, int64_t M, std::vector<double>* rec,
                  std::vector<float>* recf, std::vector<double>* verts, double center[3]) {
  rec->assign(static_cast<size_t>(M * kPanelDoubles), 0.0);
  recf->assign(static_cast<size_t>(M * kPanelFloats), 0.0f);
  verts->assign(static_cast<size_t>(M * kVertDoubles), 0.0);
  double cs[3] = {0, 0, 0};
  for (int64_t t = 0; t < M; ++t) {
    double v[3][3];
    for (int a = 0; a < 3; ++a)
      for (int d = 0; d < 3; ++d) v[a][d] = nodes[3 * (tris[3 * t + a] - 1) + d];
    double e1[3], e2[3], cr[3];
    for (int d = 0; d < 3; ++d) {
      e1[d] = v[1][d] - v[0][d];
      e2[d] = v[2][d] - v[0][d];
    }
    cr[0] = e1[1] * e2[2] - e1[2] * e2[1];
    cr[1] = e1[2] * e2[0] - e1[0] * e2[2];
    cr[2] = e1[0] * e2[1] - e1[1] * e2[0];
    double len = std::sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
    double* r = rec->data() + t * kPanelDoubles;
    for (int d = 0; d < 3; ++d) {
      r[d] = (v[0][d] + v[1][d] + v[2][d]) / 3.0;
      r[3 + d] = cr[d] / len;
    }
    r[6] = 0.5 * len;
    double dm = 0.0;
    for (int a = 0; a < 3; ++a) {
      double e[3];
      for (int d = 0; d < 3; ++d) e[d] = v[(a + 1) % 3][d] - v[a][d];
      double l = std::sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]);
      if (l > dm) dm = l;
    }
    r[7] = dm;
    for (int q = 0; q < 7; ++q)
      for (int d = 0; d < 3; ++d)
        r[8 + 3 * q + d] =
            kRuleB[q][0] * v[0][d] + kRuleB[q][1] * v[1][d] + kRuleB[q][2] * v[2][d];
    double* vv = verts->data() + t * kVertDoubles;
    for (int a = 0; a < 3; ++a)
      for (int d = 0; d < 3; ++d) vv[3 * a + d] = v[a][d];
    for (int d = 0; d < 3; ++d) cs[d] += r[d];
  }
  for (int d = 0; d < 3; ++d) center[d] = M ? cs[d] / (double)M : 0.0;
  for (int64_t t = 0; t < M; ++t) {
    const double* r = rec->data() + t * kPanelDoubles;
    float* f = recf->data() + t * kPanelFloats;
    for (int d = 0; d < 3; ++d) {
      f[d] = (float)(r[d] - center[d]);
      f[3 + d] = (float)r[3 + d];
    }
    f[6] = (float)r[6];
    f[7] = (float)r[7];
    for (int q = 0; q < 7; ++q)
      for (int d = 0; d < 3; ++d) f[8 + 3 * q + d] = (float)(r[8 + 3 * q + d] - center[d]);
  }
}

int make_mesh(bemgpu_ctx* c, const double* nodes, int64_t N, const int64_t* tris, int64_t M,
              double eta, std::shared_ptr<MeshData>* out) {
  std::string err;
  double res = 0.0;
  int s = validate_surface(nodes, N, tris, M, &res, &err);
  if (s != BEMGPU_OK) return fail(c, s, err);
  auto m = std::make_shared<MeshData>();
  m->c = c;
  m->n = M;
  m->nn = N;
  m->resolution = res;
  m->eta = eta;
  mesh_hash(nodes, N, tris, M, m->hash);
  m->nodes_h.assign(nodes, nodes + 3 * N);
  m->tris_h.assign(tris, tris + 3 * M);
  std::vector<float> recf;
  std::vector<double> verts;
  build_panels(nodes, tris, M, &m->panels_h, &recf, &verts, m->center);
  std::vector<double> cent, diam;
  panel_centroids(nodes, tris, M, &cent, &diam);
  std::vector<int64_t> rowptr, cols;
  near_pairs(cent, diam, eta, &rowptr, &cols);
  std::vector<int32_t> ni(cols.size()), nj(cols.size());
  for (int64_t i = 0; i < M; ++i)
    for (int64_t p = rowptr[i]; p < rowptr[i + 1]; ++p) {
      ni[p] = (int32_t)i;
      nj[p] = (int32_t)cols[p];
    }
  m->n_near = (int64_t)cols.size();
  std::vector<int32_t> np(rowptr.begin(), rowptr.end());
  TRY(upload(c, m->panels_h, &m->panels));
  TRY(upload(c, recf, &m->panelsf));
  TRY(upload(c, verts, &m->verts));
  TRY(upload(c, ni, &m->near_i));
  TRY(upload(c, nj, &m->near_j));
  TRY(upload(c, np, &m->near_ptr));
  TRY(alloc(c, (size_t)std::max<int64_t>(1, m->n_near) * 32, &m->near_lap));
  launch_near_laplace(c->launch(), m->panels.as<double>(), m->verts.as<double>(),
                      m->near_i.as<int32_t>(), m->near_j.as<int32_t>(), m->n_near,
                      m->near_lap.as<double>());
  CUDA_TRY(c, cudaGetLastError());
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  *out = m;
  return BEMGPU_OK;
}

// Nyström node set of a panel mesh: node q of panel t is record 7 t + q, at the panel's
// Gauss point q with the panel normal and weight area * w_q (MeshData::node_mesh).
int nystrom_mesh(bemgpu_ctx* c, MeshData* m, std::shared_ptr<MeshData>* out) {
  if (m->node_mesh) {
    *out = m->node_mesh;
    return BEMGPU_OK;
  }
  auto d = std::make_shared<MeshData>();
  d->c = c;
  d->n = (int64_t)kNyNodes * m->n;
  d->resolution = m->resolution;
  d->eta = m->eta;
  std::memcpy(d->hash, m->hash, sizeof d->hash);
  for (int a = 0; a < 3; ++a) d->center[a] = m->center[a];
  d->nystrom = true;
  d->panels_h.assign((size_t)d->n * kPanelDoubles, 0.0);
  for (int64_t t = 0; t < m->n; ++t) {
    const double* r = m->panels_h.data() + t * kPanelDoubles;
    for (int q = 0; q < kNyNodes; ++q) {
      double* o = d->panels_h.data() + (t * kNyNodes + q) * kPanelDoubles;
      for (int a = 0; a < 3; ++a) {
        o[a] = r[8 + 3 * q + a];
        o[3 + a] = r[3 + a];
      }
      o[6] = r[6] * kRuleW[q];
      o[7] = r[7];
      for (int g = 0; g < 7; ++g)
        for (int a = 0; a < 3; ++a) o[8 + 3 * g + a] = o[a];
    }
  }
  // FP32 records relative to the centre (compressed operators with precision mixed)
  std::vector<float> recf((size_t)d->n * kPanelFloats, 0.0f);
  for (int64_t i = 0; i < d->n; ++i) {
    const double* r = d->panels_h.data() + i * kPanelDoubles;
    float* f = recf.data() + i * kPanelFloats;
    for (int a = 0; a < 3; ++a) {
      f[a] = (float)(r[a] - d->center[a]);
      f[3 + a] = (float)r[3 + a];
    }
    f[6] = (float)r[6];
    f[7] = (float)r[7];
    for (int q = 0; q < 7; ++q)
      for (int a = 0; a < 3; ++a) f[8 + 3 * q + a] = f[a];
  }
  TRY(upload(c, d->panels_h, &d->panels));
  TRY(upload(c, recf, &d->panelsf));
  if (m->surf.p) {  // union of several surfaces: the surface of every node, node offsets
    std::vector<int32_t> sn((size_t)d->n);
    for (size_t s = 0; s + 1 < m->offsets.size(); ++s)
      for (int64_t t = m->offsets[s]; t < m->offsets[s + 1]; ++t)
        for (int q = 0; q < kNyNodes; ++q) sn[(size_t)(t * kNyNodes + q)] = (int32_t)s;
    TRY(upload(c, sn, &d->surf));
    for (int64_t o : m->offsets) d->offsets.push_back(o * kNyNodes);
  }
  m->node_mesh = d;
  *out = d;
  return BEMGPU_OK;
}
}  // namespace

// The union of several validated surfaces as one panel set (each surface was validated
// on its own upload; the union is not one closed surface): panels in surface order, FP32
// records relative to the union's centre, near pairs over all surfaces (a close pair of
// surfaces gets its cross near pairs), the surface of every panel.
int make_union_mesh(bemgpu_ctx* c, const std::vector<const MeshData*>& parts, double eta,
                    std::shared_ptr<MeshData>* out) {
  std::vector<double> nodes;
  std::vector<int64_t> tris;
  std::vector<int32_t> surf;
  auto m = std::make_shared<MeshData>();
  int64_t base = 0;
  m->offsets.push_back(0);
  for (size_t s = 0; s < parts.size(); ++s) {
    const MeshData* p = parts[s];
    nodes.insert(nodes.end(), p->nodes_h.begin(), p->nodes_h.end());
    for (int64_t t : p->tris_h) tris.push_back(t + base);
    base += p->nn;
    for (int64_t q = 0; q < p->n; ++q) surf.push_back((int32_t)s);
    m->offsets.push_back(m->offsets.back() + p->n);
    m->resolution = std::max(m->resolution, p->resolution);
  }
  const int64_t N = base, M = (int64_t)tris.size() / 3;
  m->c = c;
  m->n = M;
  m->nn = N;
  m->eta = eta;
  mesh_hash(nodes.data(), N, tris.data(), M, m->hash);
  m->nodes_h = nodes;
  m->tris_h = tris;
  std::vector<float> recf;
  std::vector<double> verts;
  build_panels(nodes.data(), tris.data(), M, &m->panels_h, &recf, &verts, m->center);
  std::vector<double> cent, diam;
  panel_centroids(nodes.data(), tris.data(), M, &cent, &diam);
  std::vector<int64_t> rowptr, cols;
  near_pairs(cent, diam, eta, &rowptr, &cols);
  std::vector<int32_t> ni(cols.size()), nj(cols.size());
  for (int64_t i = 0; i < M; ++i)
    for (int64_t p = rowptr[i]; p < rowptr[i + 1]; ++p) {
      ni[p] = (int32_t)i;
      nj[p] = (int32_t)cols[p];
    }
  m->n_near = (int64_t)cols.size();
  std::vector<int32_t> np(rowptr.begin(), rowptr.end());
  TRY(upload(c, m->panels_h, &m->panels));
  TRY(upload(c, recf, &m->panelsf));
  TRY(upload(c, verts, &m->verts));
  TRY(upload(c, ni, &m->near_i));
  TRY(upload(c, nj, &m->near_j));
  TRY(upload(c, np, &m->near_ptr));
  TRY(upload(c, surf, &m->surf));
  TRY(alloc(c, (size_t)std::max<int64_t>(1, m->n_near) * 32, &m->near_lap));
  launch_near_laplace(c->launch(), m->panels.as<double>(), m->verts.as<double>(),
                      m->near_i.as<int32_t>(), m->near_j.as<int32_t>(), m->n_near,
                      m->near_lap.as<double>());
  CUDA_TRY(c, cudaGetLastError());
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  *out = m;
  return BEMGPU_OK;
}

// Solid angle of a closed surface (host, FP64) seen from x: 4 pi inside, 0 outside.
double host_solid_angle(const MeshData* m, const double* x) {
  double om = 0.0;
  for (int64_t t = 0; t < m->n; ++t) {
    const double* v[3];
    for (int a = 0; a < 3; ++a) v[a] = &m->nodes_h[3 * (m->tris_h[3 * t + a] - 1)];
    double R[3][3], r[3];
    for (int a = 0; a < 3; ++a) {
      for (int d = 0; d < 3; ++d) R[a][d] = v[a][d] - x[d];
      r[a] = std::sqrt(R[a][0] * R[a][0] + R[a][1] * R[a][1] + R[a][2] * R[a][2]);
    }
    const double cx = R[1][1] * R[2][2] - R[1][2] * R[2][1];
    const double cy = R[1][2] * R[2][0] - R[1][0] * R[2][2];
    const double cz = R[1][0] * R[2][1] - R[1][1] * R[2][0];
    const double num = R[0][0] * cx + R[0][1] * cy + R[0][2] * cz;
    auto dot = [&](int a, int b) { return R[a][0] * R[b][0] + R[a][1] * R[b][1] + R[a][2] * R[b][2]; };
    const double den = r[0] * r[1] * r[2] + dot(0, 1) * r[2] + dot(0, 2) * r[1] + dot(1, 2) * r[0];
    om += 2.0 * std::atan2(num, den);
  }
  return om;
}

// ===================================================================== factors
namespace {
struct FactorData {
  bemgpu_ctx* c = nullptr;
  std::shared_ptr<MeshData> mesh;  // null for dense user matrices
  bemgpu_problem prob{};
  int kind = kAsmBM;
  int64_t n = 0, N = 0;
  bool rhs_is_m2 = true;   // rigid: b = M2 q_inc; soft: b = M1 p_inc
  Buf A, Mrhs;             // system (complex128, or complex64 when a32), rhs operator
  bool a32 = false;        // system stored compact: complex64 + FP64 near corrections
  Buf dnear;               // near corrections of the compact system
  Buf dnear_rhs;           // near corrections of the compact rhs operator (a32, rigid/soft)
  Buf region_tab;          // kAsmRegion: RegionTable
  Buf outer;               // kAsmRegion: panel borders the exterior (int8)
  bool region_cbie = false;
  Buf LU, ipiv, info, perm;        // working factor (complex64 when single)
  Buf LU64, ipiv64, info64, perm64;  // complex128 factor after promotion
  Buf rows, cols, rowsum, cols_inv, rows_inv, cols_inv32;
  bool single = false;     // current factor precision
  bool mixed = false;      // requested precision
  bool fp32_regular = false;  // regular pairs assembled in FP32
  bool nystrom = false;       // Nyström operators on the node set (mesh = node mesh)
  std::shared_ptr<MeshData> base_mesh;  // Nyström: the panel mesh of the node set
  int reason = BEMGPU_REASON_NONE;
  double rcond = NAN;
  // systems of order <= condition_limit: a copy of A and its scales, whose SVD condition
  // numbers are computed on the first diagnostics read (shared with the solutions)
  std::shared_ptr<struct CondState> cond;
  double matrix_norm = 0.0, anorm = 0.0;
  int32_t info_h = 0;
  double assemble_ms = 0.0, factor_ms = 0.0;
  void* factor_ptr() const { return single ? LU.p : (mixed ? LU64.p : LU.p); }
  int32_t* ipiv_ptr() const { return single ? ipiv.as<int32_t>() : (mixed ? ipiv64.as<int32_t>() : ipiv.as<int32_t>()); }
  int32_t* info_ptr() const { return single ? info.as<int32_t>() : (mixed ? info64.as<int32_t>() : info.as<int32_t>()); }
  int32_t* perm_ptr() const { return single ? perm.as<int32_t>() : (mixed ? perm64.as<int32_t>() : perm.as<int32_t>()); }
  size_t bytes() const {
    return A.bytes + dnear.bytes + dnear_rhs.bytes + Mrhs.bytes + LU.bytes + LU64.bytes + ipiv.bytes +
           ipiv64.bytes + rows.bytes + cols.bytes + rowsum.bytes;
  }
};
}  // namespace

struct bemgpu_factor {
  std::shared_ptr<FactorData> d;
};

namespace {
struct SolutionData {
  bemgpu_ctx* c = nullptr;
  std::shared_ptr<struct CondState> cond;  // the factor's conditioning data (see FactorData)
  std::shared_ptr<MeshData> mesh;
  int boundary = 0;
  double k = 0.0, g = 1.0, h = 1.0;
  int32_t nrhs = 0;
  std::vector<double> dirs;  // incidence direction vectors, 3 per rhs
  Buf ps, qs;                // scattered traces, complex128 n x nrhs
  Buf xsol;                  // coupled regions: the solved unknowns [p; v], 2n x nrhs
  bool region = false;
  bemgpu_diagnostics diag{};
  std::vector<int32_t> parents;         // coupled regions: parent region of each surface,
  std::vector<double> region_k, region_rho;  // wavenumber and density of every region
  std::shared_ptr<MeshData> base_mesh;  // Nyström: the panel mesh (region test of points)
  bool hmatrix = false;                 // from bemgpu_hmatrix_solve
  bemgpu_hmatrix_stats hm{};
  std::vector<double> gm_hist;          // residual estimates, gm_stride per rhs
  std::vector<int32_t> gm_iters;
  int32_t gm_stride = 0;
};
}  // namespace

struct bemgpu_solution {
  std::shared_ptr<SolutionData> d;
};

namespace {

int check_problem(bemgpu_ctx* c, const bemgpu_problem& p, int* kind) {
  if (!(std::isfinite(p.k) && p.k > 0)) return fail(c, BEMGPU_EINVAL, "k must be finite and positive");
  if (p.precision != BEMGPU_DOUBLE && p.precision != BEMGPU_MIXED)
    return fail(c, BEMGPU_EINVAL, "precision must be :double or :mixed");
  if (p.precision == BEMGPU_MIXED) {
    if (!p.equilibrate) return fail(c, BEMGPU_EINVAL, "mixed precision requires equilibrate=true");
    if (!(std::isfinite(p.refine_tolerance) && p.refine_tolerance > 0 && p.refine_tolerance < 1))
      return fail(c, BEMGPU_EINVAL, "invalid refinement tolerance");
    if (p.refine_maxiter < 0) return fail(c, BEMGPU_EINVAL, "maxiter must be a nonnegative integer");
    if (!(std::isfinite(p.condition_guard) && p.condition_guard >= 0))
      return fail(c, BEMGPU_EINVAL, "invalid condition guard");
  }
  if (p.condition_limit < 0)
    return fail(c, BEMGPU_EINVAL, "condition_limit must be nonnegative");
  if (!(std::isfinite(p.norm_floor) && p.norm_floor >= 0))
    return fail(c, BEMGPU_EINVAL, "norm_floor must be finite and nonnegative");
  if (p.precision == BEMGPU_MIXED && p.norm_floor != 0.0)
    return fail(c, BEMGPU_EINVAL, "mixed precision does not support norm_floor");
  if (p.assembly < BEMGPU_ASSEMBLY_DEFAULT || p.assembly > BEMGPU_ASSEMBLY_SINGLE)
    return fail(c, BEMGPU_EINVAL, "assembly must be :default, :double or :single");
  if (!(std::isfinite(p.near_eta) && p.near_eta > 0))
    return fail(c, BEMGPU_EINVAL, "near_eta must be finite and positive");
  if (p.discretization != BEMGPU_COLLOCATION && p.discretization != BEMGPU_NYSTROM)
    return fail(c, BEMGPU_EINVAL, "discretization must be :collocation or :nystrom");
  if (p.boundary == BEMGPU_RIGID || p.boundary == BEMGPU_PRESSURE_RELEASE) {
    int f = p.formulation == BEMGPU_FORMULATION_DEFAULT ? BEMGPU_BURTON_MILLER : p.formulation;
    if (f != BEMGPU_BURTON_MILLER && f != BEMGPU_CBIE)
      return fail(c, BEMGPU_EINVAL, "formulation must be :cbie or :burton_miller");
    *kind = f == BEMGPU_BURTON_MILLER ? kAsmBM : kAsmCBIE;
  } else if (p.boundary == BEMGPU_FLUID) {
    int f = p.formulation == BEMGPU_FORMULATION_DEFAULT ? BEMGPU_MULLER : p.formulation;
    if (f != BEMGPU_MULLER && f != BEMGPU_CBIE)
      return fail(c, BEMGPU_EINVAL, "fluid formulation must be :muller or :cbie");
    const double g = p.density_contrast, h = p.soundspeed_contrast;
    if (!(std::isfinite(g) && g > 0 && std::isfinite(h) && h > 0))
      return fail(c, BEMGPU_EINVAL,
                  "fluid density and soundspeed contrasts must be finite and positive");
    *kind = f == BEMGPU_MULLER ? kAsmMuller : kAsmFluidCBIE;
  } else {
    return fail(c, BEMGPU_EINVAL, "unknown boundary condition");
  }
  return BEMGPU_OK;
}

int formulation_of(int kind) {
  switch (kind) {
    case kAsmBM: return BEMGPU_BURTON_MILLER;
    case kAsmCBIE: return BEMGPU_CBIE;
    case kAsmMuller: return BEMGPU_MULLER;
    default: return BEMGPU_CBIE;
  }
}

// Mesh and assembly precision of a factor (f->prob set): the Nyström node set for that
// discretisation (FP64 node operators; mixed precision reduces the factor only), else the
// panel mesh with FP32 regular pairs where the problem asks for them.
int bind_mesh(bemgpu_ctx* c, FactorData* f, const std::shared_ptr<MeshData>& m) {
  f->mixed = f->prob.precision == BEMGPU_MIXED;
  f->nystrom = f->prob.discretization == BEMGPU_NYSTROM;
  if (f->nystrom) {
    f->fp32_regular = false;
    f->base_mesh = m;
    return nystrom_mesh(c, m.get(), &f->mesh);
  }
  f->mesh = m;
  f->fp32_regular = f->prob.assembly == BEMGPU_ASSEMBLY_SINGLE ||
                    (f->prob.assembly == BEMGPU_ASSEMBLY_DEFAULT && f->mixed);
  return BEMGPU_OK;
}

// The nine plane-wave directions of the Nyström correction: integer vectors normalised
// by a correctly rounded square root (reproducible on any host).
void nystrom_directions(double* dirs) {
  static const int v[kNyBasis][3] = {{3, 1, -1}, {-3, -2, 2}, {-3, 1, -1}, {1, 2, -3}, {2, 2, 3},
                                     {0, 1, 2},  {0, -1, -1}, {-1, -3, 1}, {-3, -3, -1}};
  for (int s = 0; s < kNyBasis; ++s) {
    const double a = v[s][0], b = v[s][1], e = v[s][2];
    const double nr = std::sqrt(a * a + b * b + e * e);
    dirs[3 * s] = a / nr;
    dirs[3 * s + 1] = b / nr;
    dirs[3 * s + 2] = e / nr;
  }
}

template <class T>
int to_device(bemgpu_ctx* c, const std::vector<T>& h, Buf* out) {
  return upload(c, h, out);
}

// ------------------------------------------------------------------ assembly
// Operators of one Nyström instance (complex128, node order), corrected on every element:
// rigid/soft M1 and M2; fluid bodies the 2N x 2N system of their formulation.
int assemble_nystrom(bemgpu_ctx* c, FactorData* f) {
  const Launch L = c->launch();
  MeshData* m = f->mesh.get();
  const int64_t N = m->n;
  const int32_t fluid = f->kind == kAsmMuller ? 1 : f->kind == kAsmFluidCBIE ? 2
                       : f->kind == kAsmRegion ? (f->region_cbie ? 4 : 3) : 0;
  f->n = N;
  f->N = fluid ? 2 * N : N;
  f->a32 = false;
  f->rhs_is_m2 = f->prob.boundary == BEMGPU_RIGID;
  TRY(alloc(c, (size_t)f->N * f->N * 16, &f->A));
  if (!fluid) TRY(alloc(c, (size_t)N * N * 16, &f->Mrhs));
  const int32_t chunks = nystrom_chunks(N);
  const int64_t ne = N / kNyNodes;
  Buf scratch, status;
  TRY(alloc(c, (size_t)nystrom_scratch_doubles(N, chunks, fluid) * 8, &scratch));
  TRY(alloc(c, (size_t)ne * 4, &status));
  CUDA_TRY(c, cudaMemsetAsync(status.p, 0, (size_t)ne * 4, c->stream));
  NyInst I{};
  I.nodes = m->panels.as<double>();
  I.n = N;
  I.k = f->prob.k;
  I.a_re = 0.0;
  I.a_im = f->kind == kAsmBM ? 1.0 / f->prob.k : 0.0;
  nystrom_directions(I.dirs);
  const int64_t tr_doubles = 2 * (2 * (int64_t)kNyBasis * N);
  I.trace = scratch.as<double>();
  if (fluid) {
    I.fluid = fluid;
    I.k_int = f->prob.k / f->prob.soundspeed_contrast;
    I.g = f->prob.density_contrast;
    I.A = f->A.as<double>();
    I.trace_i = scratch.as<double>() + tr_doubles;
    I.part = scratch.as<double>() + 2 * tr_doubles;
    if (fluid >= 3) {  // coupled regions: surfaces of the nodes, coupling table
      I.surf = m->surf.as<int32_t>();
      I.region = f->region_tab.as<RegionTable>();
    }
  } else {
    // rigid: system M1, rhs M2; pressure release: system M2, rhs M1
    I.M1 = (f->rhs_is_m2 ? f->A : f->Mrhs).as<double>();
    I.M2 = (f->rhs_is_m2 ? f->Mrhs : f->A).as<double>();
    I.part = scratch.as<double>() + tr_doubles;
  }
  I.n_chunks = chunks;
  I.status = status.as<int32_t>();
  {
    Prof pr(c, "assemble");
    launch_nystrom(L, I);
  }
  CUDA_TRY(c, cudaGetLastError());
  std::vector<int32_t> st;
  TRY(download(c, status, &st, (size_t)ne));
  int64_t bad = 0;
  for (int32_t v : st) bad += v != 0;
  if (bad) {
    char msg[200];
    std::snprintf(msg, sizeof msg,
                  "density-interpolation fit is rank-deficient on %lld elements (k times the "
                  "panel size far below the plane-wave basis' resolution)",
                  (long long)bad);
    return fail(c, BEMGPU_EINVAL, msg);
  }
  return BEMGPU_OK;
}

int assemble_panels(bemgpu_ctx* c, std::vector<FactorData*>& fs);

int assemble_batch(bemgpu_ctx* c, std::vector<FactorData*>& fs) {
  std::vector<FactorData*> panels;
  for (FactorData* f : fs) {
    if (f->nystrom)
      TRY(assemble_nystrom(c, f));
    else
      panels.push_back(f);
  }
  return panels.empty() ? BEMGPU_OK : assemble_panels(c, panels);
}

int assemble_panels(bemgpu_ctx* c, std::vector<FactorData*>& fs) {
  const Launch L = c->launch();
  std::vector<AsmInst> ai(fs.size());
  for (size_t t = 0; t < fs.size(); ++t) {
    FactorData* f = fs[t];
    MeshData* m = f->mesh.get();
    const bool fluid = f->kind == kAsmMuller || f->kind == kAsmFluidCBIE || f->kind == kAsmRegion;
    f->n = m->n;
    f->N = fluid ? 2 * m->n : m->n;
    f->a32 = f->fp32_regular;
    TRY(alloc(c, (size_t)f->N * f->N * (f->a32 ? 8 : 16), &f->A));
    if (!fluid) TRY(alloc(c, (size_t)f->n * f->n * (f->a32 ? 8 : 16), &f->Mrhs));
    if (f->a32) {
      TRY(alloc(c, (size_t)std::max<int64_t>(1, m->n_near) * (fluid ? 4 : 1) * 16, &f->dnear));
      if (!fluid) TRY(alloc(c, (size_t)std::max<int64_t>(1, m->n_near) * 16, &f->dnear_rhs));
    }
    AsmInst& I = ai[t];
    std::memset(&I, 0, sizeof I);
    I.panels = m->panels.as<double>();
    I.panelsf = m->panelsf.as<float>();
    I.verts = m->verts.as<double>();
    I.near_i = m->near_i.as<int32_t>();
    I.near_j = m->near_j.as<int32_t>();
    I.near_lap = m->near_lap.as<double>();
    I.n = m->n;
    I.n_near = m->n_near;
    I.lda = f->N;
    I.k_e = f->prob.k;
    I.k_i = fluid ? f->prob.k / f->prob.soundspeed_contrast : f->prob.k;
    I.g = fluid ? f->prob.density_contrast : 1.0;
    I.a_re = 0.0;
    I.a_im = f->kind == kAsmBM ? 1.0 / f->prob.k : 0.0;
    I.kind = f->kind;
    if (fluid) {
      I.out1 = f->A.p;
      I.out2 = nullptr;
      I.c64 = f->a32 ? 1 : 0;
    } else {
      // rigid: system M1, rhs M2; pressure release: system M2, rhs M1
      f->rhs_is_m2 = f->prob.boundary == BEMGPU_RIGID;
      I.out1 = f->rhs_is_m2 ? f->A.p : f->Mrhs.p;
      I.out2 = f->rhs_is_m2 ? f->Mrhs.p : f->A.p;
      I.c64 = f->a32 ? 3 : 0;
    }
    if (f->kind == kAsmRegion) {
      I.surf = m->surf.as<int32_t>();
      I.region = f->region_tab.as<RegionTable>();
    }
    if (f->a32) {
      double* sysd = f->dnear.as<double>();
      double* rhsd = fluid ? nullptr : f->dnear_rhs.as<double>();
      I.dnear = (fluid || f->rhs_is_m2) ? sysd : rhsd;   // corrections of out1
      I.dnear2 = (fluid || f->rhs_is_m2) ? rhsd : sysd;  // corrections of out2
    }
  }
  // group by (kind, regular precision) so each group is one launch
  std::vector<size_t> order(fs.size());
  for (size_t t = 0; t < order.size(); ++t) order[t] = t;
  auto key = [&](size_t t) { return fs[t]->kind * 2 + (fs[t]->fp32_regular ? 1 : 0); };
  std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return key(a) < key(b); });
  std::vector<AsmInst> sorted(fs.size());
  for (size_t t = 0; t < order.size(); ++t) sorted[t] = ai[order[t]];
  Buf d_ai;
  TRY(to_device(c, sorted, &d_ai));
  {
    Prof pr(c, "assemble");
    size_t s = 0;
    while (s < order.size()) {
      size_t e = s;
      int64_t nmax = 0;
      while (e < order.size() && key(order[e]) == key(order[s])) {
        nmax = std::max(nmax, fs[order[e]]->n);
        ++e;
      }
      launch_assemble_regular(L, d_ai.as<AsmInst>() + s, (int)(e - s), nmax, fs[order[s]]->kind,
                              fs[order[s]]->fp32_regular);
      s = e;
    }
  }
  {
    Prof pr(c, "near");
    size_t s = 0;
    while (s < order.size()) {
      size_t e = s;
      int64_t nmax = 0;
      while (e < order.size() && key(order[e]) == key(order[s])) {
        nmax = std::max(nmax, fs[order[e]]->mesh->n_near);
        ++e;
      }
      launch_assemble_near(L, d_ai.as<AsmInst>() + s, (int)(e - s), nmax, fs[order[s]]->kind,
                           fs[order[s]]->fp32_regular);
      s = e;
    }
  }
  CUDA_TRY(c, cudaGetLastError());
  return BEMGPU_OK;
}

// ------------------------------------------------------------------ factorisation

// ------------------------------------------------------------------ autotuner
// Launch shapes whose choice leaves every result bit-for-bit unchanged (the rows each
// thread or CTA takes, not the order of any sum) are picked by measurement: the first
// time a (family, shape class) is met, every candidate runs on the live data (or on a
// scratch copy when the kernel works in place), timed with CUDA events on the context's
// stream, and the fastest is kept for the context's lifetime.
int log2_bucket(int64_t v) {
  int b = 0;
  while (v > 1) {
    v >>= 1;
    ++b;
  }
  return b;
}

template <class Run, class Prepare>
int tune_pick(bemgpu_ctx* c, const std::string& key, const std::vector<int>& cands, Run run,
              Prepare prepare) {
  auto it = c->tuned.find(key);
  if (it != c->tuned.end()) return it->second;
  if (!c->autotune || cands.size() < 2) return cands.front();
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best_ms = INFINITY;
  int best = cands.front();
  for (int v : cands) {
    prepare();
    cudaEventRecord(e0, c->stream);
    run(v);
    cudaEventRecord(e1, c->stream);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best_ms) {
      best_ms = ms;
      best = v;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  c->tuned[key] = best;
  return best;
}

// Cluster size of the complex64 panel kernel for this batch and panel height, measured
// on scratch copies of the panels (the kernel factors in place).
// Infinity-norm reciprocal condition of the complex64 factors (LAPACK cgecon('I'):
// zlacn2's kase 2 applies (LU)^{-1}, kase 1 applies (LU)^{-H}; rcond = 1 / (anorm
// ||A^-1||)).  Every factor's zlacn2 state lives on the device (k_lacn2); each round runs
// the batched products the states ask for and reads back only the states.
int estimate_rcond(bemgpu_ctx* c, std::vector<FactorData*>& fs) {
  if (fs.empty()) return BEMGPU_OK;
  const Launch L = c->launch();
  const size_t F = fs.size();
  std::vector<Lacn2Dev> st(F);
  std::vector<size_t> off(F + 1, 0);
  int64_t nmax = 0;
  for (size_t t = 0; t < F; ++t) {
    std::memset(&st[t], 0, sizeof st[t]);
    st[t].n = (int32_t)fs[t]->N;
    st[t].off = (int64_t)off[t];
    off[t + 1] = off[t] + (size_t)fs[t]->N;
    nmax = std::max(nmax, fs[t]->N);
  }
  Buf work, work2, d_st, d_m1, d_m2;
  TRY(alloc(c, off[F] * 8, &work));
  TRY(alloc(c, off[F] * 8, &work2));
  // one descriptor array per product: kase 1 applies (LU)^{-H}, kase 2 (LU)^{-1}; the
  // device step switches each instance's active flag
  std::vector<MatInst> mi(F);
  for (size_t t = 0; t < F; ++t) {
    MatInst& m = mi[t];
    std::memset(&m, 0, sizeof m);
    m.a = fs[t]->LU.p;
    m.n = fs[t]->N;
    m.lda = fs[t]->N;
    m.ipiv = fs[t]->ipiv.as<int32_t>();
    m.info = fs[t]->info.as<int32_t>();
    m.x = work.as<float2>() + off[t];
    m.y = work2.as<float2>() + off[t];
    m.ldx = fs[t]->N;
    m.nrhs = 1;
    m.active = 0;
  }
  TRY(upload(c, st, &d_st));
  TRY(upload(c, mi, &d_m1));
  TRY(upload(c, mi, &d_m2));
  TrsvWork tw{1};
  Lacn2Dev* ds = d_st.as<Lacn2Dev>();
  MatInst* m1 = d_m1.as<MatInst>();
  MatInst* m2 = d_m2.as<MatInst>();
  launch_lacn2(L, ds, (int)F, work.as<float2>(), m1, m2, 0);
  std::vector<int32_t> kase(F, 1);
  for (int round = 0; round < 64; ++round) {
    bool any1 = false, any2 = false;
    for (int32_t k : kase) {
      any1 |= k == 1;
      any2 |= k == 2;
    }
    if (!any1 && !any2) break;
    if (any1) {
      {
        Prof pr(c, "getrs");
        launch_getrs(L, m1, (int)F, nmax, 1, 1, 1, 0, &tw);
      }
      launch_lacn2(L, ds, (int)F, work.as<float2>(), m1, m2, 1);
      any2 = true;  // those instances usually ask for the other product next
    }
    if (any2) {
      {
        Prof pr(c, "getrs");
        launch_getrs(L, m2, (int)F, nmax, 1, 0, 1, 0, &tw);
      }
      launch_lacn2(L, ds, (int)F, work.as<float2>(), m1, m2, 2);
    }
    CUDA_TRY(c, cudaGetLastError());
    TRY(download(c, d_st, &st, F));
    for (size_t t = 0; t < F; ++t) kase[t] = st[t].kase;
  }
  for (size_t t = 0; t < F; ++t) {
    if (st[t].kase != 0) return fail(c, BEMGPU_ENOTCONVERGED, "condition estimate did not end");
    const double ainv = st[t].est;
    fs[t]->rcond = (ainv != 0.0) ? (1.0 / ainv) / fs[t]->anorm : 0.0;
  }
  return BEMGPU_OK;
}

// Complex64 LU with 256-column outer steps made of two 128-column halves.  Each half is
// factored by the SIMT panel kernels in 32-column steps; the left half's update of the
// right half, the 256-row U12 solve (through -(L11^{-1} - I) products) and the trailing
// update are tcgen05 split-BF16 GEMMs (gemm_tc.cu) on packed operand images.  The
// trailing update runs once per 256 columns with K = 256, so the matrix streams through
// HBM half as often as with 128-column steps.
//
// Per outer step (K0, halves H0 = K0 and H1 = K0 + 128, kk0 / kk1 their widths):
//   factor half 0 (columns [H0, H0 + kk0))
//   half-0 interchanges on the right half; P1: U12r = L11a^{-1} A[H0.., H1..H1 + kk1)
//   P2: A[H1.., H1..H1 + kk1) -= L21a U12r
//   factor half 1; interchanges of both halves on the columns outside [K0, K0 + 256)
//   P3: U12top = L11a^{-1} A12top            P4: A12bot -= Lmid U12top
//   P5: U12bot = L11b^{-1} A12bot            P6: A22 -= L21 U12 (K = kk0 + kk1)
}  // namespace

// A captured launch sequence of the tensor-core LU for one exact batch shape, with the
// descriptor arrays its kernels take as arguments (rewritten before every replay).
struct LuGraph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  Buf dm, dpack, dgem, dipack, digem, d_p0, d_p1;
  uint64_t last = 0;
  long long kernels = 0;  // kernel launches in the graph
  LuGraph() = default;
  LuGraph(const LuGraph&) = delete;
  LuGraph& operator=(const LuGraph&) = delete;
  ~LuGraph() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
  }
};

namespace {
constexpr size_t kLuGraphs = 16;  // captured shapes kept per context (least recently used go)

int getrf_tc(bemgpu_ctx* c, std::vector<FactorData*>& fs, const std::vector<MatInst>& mi,
             Buf& d, int64_t nmax) {
  const Launch L = c->launch();
  const int ni = (int)fs.size();
  constexpr int HB = kTcPanel;       // half width (128)
  constexpr int SB = 2 * kTcPanel;   // outer step (256)
  std::vector<Buf> apack(ni), bpack(ni), mpack(ni);
  std::vector<Buf> negn0(ni), negn1(ni), npack0(ni), npack1(ni);
  std::vector<float2*> p0(ni), p1(ni);
  for (int t = 0; t < ni; ++t) {
    const size_t bytes = tc_pack_bytes(fs[t]->N, SB);
    TRY(alloc(c, bytes, &apack[t]));
    TRY(alloc(c, bytes, &bpack[t]));
    TRY(alloc(c, tc_pack_bytes(HB, HB), &mpack[t]));
    TRY(alloc(c, (size_t)HB * HB * 8, &negn0[t]));
    TRY(alloc(c, (size_t)HB * HB * 8, &negn1[t]));
    TRY(alloc(c, tc_pack_bytes(HB, HB), &npack0[t]));
    TRY(alloc(c, tc_pack_bytes(HB, HB), &npack1[t]));
    p0[t] = negn0[t].as<float2>();
    p1[t] = negn1[t].as<float2>();
  }
  Buf d_p0, d_p1;
  TRY(to_device(c, p0, &d_p0));
  TRY(to_device(c, p1, &d_p1));
  // tensor maps of the factors for the reduction epilogue (all instances or none)
  Buf dmaps;
  bool red = true;
  std::vector<const void*> cmaps(ni, nullptr);
  {
    std::vector<uint8_t> maps((size_t)ni * kTcMapBytes + 64);
    uint8_t* hm = reinterpret_cast<uint8_t*>(
        (reinterpret_cast<uintptr_t>(maps.data()) + 63) & ~uintptr_t(63));
    for (int t = 0; t < ni && red; ++t)
      red = tc_encode_cmap(hm + (size_t)t * kTcMapBytes, mi[t].a, mi[t].lda, mi[t].n, mi[t].n);
    if (red) {
      TRY(alloc(c, (size_t)ni * kTcMapBytes, &dmaps));
      CUDA_TRY(c, cudaMemcpyAsync(dmaps.p, hm, (size_t)ni * kTcMapBytes, cudaMemcpyHostToDevice,
                                  c->stream));
      for (int t = 0; t < ni; ++t) cmaps[t] = dmaps.as<uint8_t>() + (size_t)t * kTcMapBytes;
    }
  }
  // descriptors of every outer step and phase, uploaded once
  const int64_t steps = (nmax + SB - 1) / SB;
  // pack phases; pairs launched together are adjacent
  enum { kNeg0, kP1b, kP2a, kP2b, kP3b, kP4a, kP4b, kNeg1, kP5b, kP6a, kP6b, kNPack };
  enum { kG1, kG2, kG3, kG4, kG5, kG6, kNGem };
  std::vector<TcPackInst> packs((size_t)steps * kNPack * ni);
  std::vector<TcGemmInst> gems((size_t)steps * kNGem * ni);
  std::vector<int64_t> tiles((size_t)steps * kNGem, 0), prow((size_t)steps * kNPack, 0);
  std::vector<int> pkk((size_t)steps * kNPack, 0);
  auto PK = [&](int64_t st, int ph, int t) -> TcPackInst& {
    return packs[((size_t)st * kNPack + ph) * ni + t];
  };
  auto GM = [&](int64_t st, int ph, int t) -> TcGemmInst& {
    return gems[((size_t)st * kNGem + ph) * ni + t];
  };
  // operand image of rows [r0, r0 + rows) x K [k0, k0 + kk) of `a` (trans: (r, k) at k + r lda)
  auto set_pack = [&](int64_t st, int ph, int t, const void* a, int64_t lda, int64_t r0,
                      int64_t k0, int64_t rows, int kk, int trans, void* out) {
    TcPackInst& p = PK(st, ph, t);
    std::memset(&p, 0, sizeof p);
    const bool on = rows > 0 && kk > 0;
    p.a = a;
    p.lda = lda;
    p.r0 = r0;
    p.k0 = k0;
    p.rows = on ? rows : 0;
    p.kk = on ? kk : 0;
    p.trans = trans;
    p.out = out;
    p.active = on ? 1 : 0;
    const size_t q = (size_t)st * kNPack + ph;
    if (on) {
      prow[q] = std::max(prow[q], rows);
      pkk[q] = std::max(pkk[q], kk);
    }
  };
  auto set_gemm = [&](int64_t st, int ph, int t, const void* ap, const void* bp, int64_t c_r0,
                      int64_t c_c0, int64_t m, int64_t n, int kk) {
    TcGemmInst& g = GM(st, ph, t);
    std::memset(&g, 0, sizeof g);
    const bool on = m > 0 && n > 0 && kk > 0;
    g.apack = ap;
    g.bpack = bp;
    g.c = mi[t].a;
    g.ldc = mi[t].lda;
    g.c_r0 = c_r0;
    g.c_c0 = c_c0;
    g.m = on ? m : 0;
    g.n = on ? n : 0;
    g.kk = on ? kk : 0;
    g.active = on ? 1 : 0;
    g.cmap = cmaps[t];
    if (on) tiles[(size_t)st * kNGem + ph] += ((m + 127) / 128) * ((n + 127) / 128);
  };
  for (int64_t st = 0; st < steps; ++st) {
    const int64_t K0 = st * SB, H1 = K0 + HB;
    for (int t = 0; t < ni; ++t) {
      const int64_t n = mi[t].n, lda = mi[t].lda;
      const void* A = mi[t].a;
      const int kk0 = (int)std::max<int64_t>(0, std::min<int64_t>(HB, n - K0));
      const int kk1 = (int)std::max<int64_t>(0, std::min<int64_t>(HB, n - H1));
      const int64_t m2 = std::max<int64_t>(0, n - H1);       // rows below half 0's block
      const int64_t m3 = std::max<int64_t>(0, n - K0 - SB);  // trailing extent
      void *ap = apack[t].p, *bp = bpack[t].p;
      set_pack(st, kNeg0, t, negn0[t].p, HB, 0, 0, kk1 > 0 ? kk0 : 0, kk0, 0, npack0[t].p);
      set_pack(st, kNeg1, t, negn1[t].p, HB, 0, 0, m3 > 0 ? kk1 : 0, kk1, 0, npack1[t].p);
      // P1: U12r (rows H0.., columns H1..H1 + kk1)
      set_pack(st, kP1b, t, A, lda, H1, K0, kk1, kk0, 1, bp);
      set_gemm(st, kG1, t, npack0[t].p, bp, K0, H1, kk0, kk1, kk0);
      // P2: rows [H1, n) x columns [H1, H1 + kk1) -= L21a U12r
      set_pack(st, kP2a, t, A, lda, H1, K0, kk1 > 0 ? m2 : 0, kk0, 0, ap);
      set_pack(st, kP2b, t, A, lda, H1, K0, kk1, kk0, 1, bp);
      set_gemm(st, kG2, t, ap, bp, H1, H1, m2, kk1, kk0);
      // P3: U12top (rows K0.., columns K0 + SB..)
      set_pack(st, kP3b, t, A, lda, K0 + SB, K0, m3, kk0, 1, bp);
      set_gemm(st, kG3, t, npack0[t].p, bp, K0, K0 + SB, kk0, m3, kk0);
      // P4: A12bot -= Lmid U12top
      set_pack(st, kP4a, t, A, lda, H1, K0, m3 > 0 ? kk1 : 0, kk0, 0, mpack[t].p);
      set_pack(st, kP4b, t, A, lda, K0 + SB, K0, m3, kk0, 1, bp);
      set_gemm(st, kG4, t, mpack[t].p, bp, H1, K0 + SB, kk1, m3, kk0);
      // P5: U12bot = L11b^{-1} A12bot
      set_pack(st, kP5b, t, A, lda, K0 + SB, H1, m3, kk1, 1, bp);
      set_gemm(st, kG5, t, npack1[t].p, bp, H1, K0 + SB, kk1, m3, kk1);
      // P6: trailing update with K = kk0 + kk1
      set_pack(st, kP6a, t, A, lda, K0 + SB, K0, m3, kk0 + kk1, 0, ap);
      set_pack(st, kP6b, t, A, lda, K0 + SB, K0, m3, kk0 + kk1, 1, bp);
      set_gemm(st, kG6, t, ap, bp, K0 + SB, K0 + SB, m3, m3, kk0 + kk1);
    }
  }
  // in-half updates after each 32-column panel (K = 32): rows [k0 + 32, n) x columns
  // [k0 + 32, H + 128) -= L21 U12, on the tensor cores as well
  constexpr int kInner = HB / kPanelNB - 1;  // panels with columns to their right
  const size_t nis = (size_t)steps * 2 * kInner;
  std::vector<TcPackInst> ipacks(nis * 2 * ni);
  std::vector<TcGemmInst> igems(nis * ni);
  std::vector<int64_t> itiles(nis, 0), irows(nis, 0);
  for (int64_t st = 0; st < steps; ++st)
    for (int h = 0; h < 2; ++h)
      for (int q = 0; q < kInner; ++q) {
        const size_t idx = ((size_t)st * 2 + h) * kInner + q;
        const int64_t H = st * SB + h * HB, k0 = H + (int64_t)q * kPanelNB;
        for (int t = 0; t < ni; ++t) {
          const int64_t n = mi[t].n, lda = mi[t].lda;
          const int64_t m = std::max<int64_t>(0, n - k0 - kPanelNB);
          const int64_t nc = std::max<int64_t>(0, std::min<int64_t>(H + HB, n) - k0 - kPanelNB);
          const bool on = m > 0 && nc > 0;
          TcPackInst& a = ipacks[idx * 2 * ni + t];
          TcPackInst& b = ipacks[idx * 2 * ni + ni + t];
          std::memset(&a, 0, sizeof a);
          std::memset(&b, 0, sizeof b);
          a.a = b.a = mi[t].a;
          a.lda = b.lda = lda;
          a.r0 = k0 + kPanelNB;  // rows of L21
          b.r0 = k0 + kPanelNB;  // columns of U12
          a.k0 = b.k0 = k0;
          a.rows = on ? m : 0;
          b.rows = on ? nc : 0;
          a.kk = b.kk = on ? kPanelNB : 0;
          a.trans = 0;
          b.trans = 1;
          a.out = apack[t].p;
          b.out = bpack[t].p;
          a.active = b.active = on ? 1 : 0;
          TcGemmInst& g = igems[idx * ni + t];
          std::memset(&g, 0, sizeof g);
          g.apack = apack[t].p;
          g.bpack = bpack[t].p;
          g.c = mi[t].a;
          g.ldc = lda;
          g.c_r0 = g.c_c0 = k0 + kPanelNB;
          g.m = on ? m : 0;
          g.n = on ? nc : 0;
          g.kk = on ? kPanelNB : 0;
          g.active = on ? 1 : 0;
          g.cmap = cmaps[t];
          if (on) {
            itiles[idx] += ((m + 127) / 128) * ((nc + 127) / 128);
            irows[idx] = std::max(irows[idx], std::max(m, nc));
          }
        }
      }
  // Every launch's grid and arguments follow from the batch shape (the orders of the
  // instances, the epilogue kind, profiling) and the descriptor arrays' addresses.  The
  // sequence is captured in a CUDA graph the second time a shape is met and replayed
  // from then on, with the descriptors of the new batch written into the graph's arrays.
  // (Not while profiling: the per-family event timing reads events around each group of
  // launches, which a replayed graph does not give back.)
  std::shared_ptr<LuGraph> G;
  bool capture = false;
  if (c->graphs && !c->prof) {
    std::string key = std::to_string(ni) + (red ? "r" : "s");
    for (const MatInst& m : mi) key += "/" + std::to_string(m.n) + ":" + std::to_string(m.lda);
    auto it = c->lu_graphs.find(key);
    if (it != c->lu_graphs.end()) {
      G = it->second;
    } else if (++c->lu_seen[key] >= 2) {
      if (c->lu_graphs.size() >= kLuGraphs) {  // make room: least recently used shape
        auto victim = c->lu_graphs.begin();
        for (auto jt = c->lu_graphs.begin(); jt != c->lu_graphs.end(); ++jt)
          if (jt->second->last < victim->second->last) victim = jt;
        c->lu_graphs.erase(victim);
      }
      G = std::make_shared<LuGraph>();
      c->lu_graphs[key] = G;
      capture = true;
    }
    if (G) G->last = ++c->lu_tick;
  }
  Buf dpack, dgem, dipack, digem;
  Buf* bm = nullptr;  // the MatInst array the launches take
  if (G) {
    auto put = [&](auto& host, Buf* b) -> int {
      using T = typename std::decay_t<decltype(host)>::value_type;
      const size_t bytes = host.size() * sizeof(T);
      if (!b->p) TRY(alloc(c, std::max<size_t>(bytes, 1), b));
      if (bytes)
        CUDA_TRY(c, cudaMemcpyAsync(b->p, host.data(), bytes, cudaMemcpyHostToDevice, c->stream));
      return BEMGPU_OK;
    };
    TRY(put(mi, &G->dm));
    TRY(put(packs, &G->dpack));
    TRY(put(gems, &G->dgem));
    TRY(put(ipacks, &G->dipack));
    TRY(put(igems, &G->digem));
    TRY(put(p0, &G->d_p0));
    TRY(put(p1, &G->d_p1));
    bm = &G->dm;
  } else {
    TRY(to_device(c, packs, &dpack));
    TRY(to_device(c, gems, &dgem));
    TRY(to_device(c, ipacks, &dipack));
    TRY(to_device(c, igems, &digem));
    bm = &d;
  }
  const MatInst* dm = bm->as<MatInst>();
  Buf& Dpack = G ? G->dpack : dpack;
  Buf& Dgem = G ? G->dgem : dgem;
  Buf& Dipack = G ? G->dipack : dipack;
  Buf& Digem = G ? G->digem : digem;
  Buf& Dp0 = G ? G->d_p0 : d_p0;
  Buf& Dp1 = G ? G->d_p1 : d_p1;
  auto pack = [&](int64_t st, int ph) {
    const size_t q = (size_t)st * kNPack + ph;
    if (prow[q] > 0)
      launch_tc_pack(L, Dpack.as<TcPackInst>() + q * ni, ni, prow[q], pkk[q]);
  };
  // phases ph and ph + 1 in one launch (2 ni instances)
  auto pack2 = [&](int64_t st, int ph) {
    const size_t q = (size_t)st * kNPack + ph;
    const int64_t rows = std::max(prow[q], prow[q + 1]);
    const int kk = std::max(pkk[q], pkk[q + 1]);
    if (rows > 0) launch_tc_pack(L, Dpack.as<TcPackInst>() + q * ni, 2 * ni, rows, kk);
  };
  auto gemm = [&](int64_t st, int ph) {
    const size_t q = (size_t)st * kNGem + ph;
    if (tiles[q] > 0) launch_tc_cgemm(L, Dgem.as<TcGemmInst>() + q * ni, ni, tiles[q], red);
  };
  auto any = [&](int64_t st, int ph) { return tiles[(size_t)st * kNGem + ph] > 0; };
  auto factor_half = [&](int64_t H) {
    const int64_t st = H / SB;
    const int h = (int)((H % SB) / HB);
    for (int64_t k0 = H; k0 < H + HB && k0 < nmax; k0 += kPanelNB) {
      {
        // cluster size by the batch-size rule: timing the candidates on the first panels
        // of a shape class (in place, in the order 2 4 8 8 4 2 to cancel the panels' work
        // trend) chose sizes that were slower over the whole batch (184 vs 132 ms of
        // panels per 64 x 10240 factorisation), as did timing them on scratch copies
        Prof pr(c, "getf2");
        launch_getf2(L, dm, ni, k0, kPanelNB, 1, 0);
      }
      {
        Prof pr(c, "laswp");
        launch_laswp(L, dm, ni, k0, kPanelNB, H, H + HB, k0, k0 + kPanelNB, 1);
      }
      {
        Prof pr(c, "trsm");
        launch_trsm_panel(L, dm, ni, k0, kPanelNB, k0 + kPanelNB, H + HB, 1);
      }
      const int q = (int)((k0 - H) / kPanelNB);
      if (q < kInner) {
        const size_t idx = ((size_t)st * 2 + h) * kInner + q;
        if (itiles[idx] > 0) {
          Prof pr(c, "gemm_panel");
          if (red) {  // tensor cores, reduction epilogue
            launch_tc_pack(L, Dipack.as<TcPackInst>() + idx * 2 * ni, 2 * ni, irows[idx],
                           kPanelNB);
            launch_tc_cgemm(L, Digem.as<TcGemmInst>() + idx * ni, ni, itiles[idx], true);
          } else {
            launch_gemm_update(L, dm, ni, k0, kPanelNB, nmax, k0 + kPanelNB, H + HB, 1);
          }
        }
      }
    }
  };
  auto issue = [&]() {
    for (int64_t st = 0; st < steps; ++st) {
      const int64_t K0 = st * SB, H1 = K0 + HB;
      factor_half(K0);
      if (H1 < nmax) {
        {
          Prof pr(c, "laswp");
          launch_laswp(L, dm, ni, K0, HB, H1, H1 + HB, H1, H1, 1);
        }
        {
          Prof pr(c, "trsm");
          launch_linv_neg(L, dm, ni, K0, Dp0.as<float2* const>());
          pack2(st, kNeg0);  // -N and A12r
          gemm(st, kG1);
        }
        {
          Prof pr(c, "tc_pack");
          pack2(st, kP2a);   // L21a and U12r
        }
        {
          Prof pr(c, "gemm_tc");
          gemm(st, kG2);
        }
        factor_half(H1);
      }
      {
        Prof pr(c, "laswp");
        launch_laswp(L, dm, ni, K0, HB, 0, nmax, K0, K0 + SB, 1);
        if (H1 < nmax) launch_laswp(L, dm, ni, H1, HB, 0, nmax, H1, K0 + SB, 1);
      }
      if (!any(st, kG6)) continue;
      {
        Prof pr(c, "trsm");
        pack(st, kP3b);
        gemm(st, kG3);
        pack2(st, kP4a);   // Lmid and U12top
        gemm(st, kG4);
        launch_linv_neg(L, dm, ni, H1, Dp1.as<float2* const>());
        pack2(st, kNeg1);  // -N (second half) and A12bot
        gemm(st, kG5);
      }
      {
        Prof pr(c, "tc_pack");
        pack2(st, kP6a);   // L21 and U12
      }
      {
        Prof pr(c, "gemm_tc");
        gemm(st, kG6);
      }
    }
  };
  if (!G) {
    issue();
  } else {
    if (capture) {
      CUDA_TRY(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
      const long long k0 = launch_total();
      issue();
      G->kernels = launch_total() - k0;
      cudaGraph_t g = nullptr;
      const cudaError_t ce = cudaStreamEndCapture(c->stream, &g);
      if (ce != cudaSuccess) {
        c->lu_graphs.clear();
        return cuda_fail(c, ce, "cudaStreamEndCapture");
      }
      G->graph = g;
      CUDA_TRY(c, cudaGraphInstantiate(&G->exec, g, 0));
    }
    CUDA_TRY(c, cudaGraphLaunch(G->exec, c->stream));
    if (capture) {
      c->lu_captures++;
    } else {
      c->lu_replays++;
      count_launch((int)G->kernels);  // the graph's kernels run again
    }
  }
  CUDA_TRY(c, cudaGetLastError());
  TRY(check_device_error(c));
  return BEMGPU_OK;
}

// LU of a batch of same-precision factors (prec 1: complex64 in LU, 0: complex128).
int getrf_batch(bemgpu_ctx* c, std::vector<FactorData*>& fs, int prec, bool promoted) {
  if (fs.empty()) return BEMGPU_OK;
  const Launch L = c->launch();
  std::vector<MatInst> mi(fs.size());
  int64_t nmax = 0;
  for (size_t t = 0; t < fs.size(); ++t) {
    FactorData* f = fs[t];
    MatInst& m = mi[t];
    std::memset(&m, 0, sizeof m);
    m.a = promoted ? f->LU64.p : f->LU.p;
    m.n = f->N;
    m.lda = f->N;
    m.ipiv = promoted ? f->ipiv64.as<int32_t>() : f->ipiv.as<int32_t>();
    m.info = promoted ? f->info64.as<int32_t>() : f->info.as<int32_t>();
    Buf& pb = promoted ? f->perm64 : f->perm;
    TRY(alloc(c, (size_t)f->N * 4, &pb));
    m.perm = pb.as<int32_t>();
    m.active = 1;
    CUDA_TRY(c, cudaMemsetAsync(m.info, 0, sizeof(int32_t), c->stream));
    nmax = std::max(nmax, f->N);
  }
  Buf d;
  TRY(to_device(c, mi, &d));
  if (prec == 1 && c->tensor_lu) {
    TRY(getrf_tc(c, fs, mi, d, nmax));
  } else {
    // right-looking blocked LU, 32-column panels; each kernel family timed on its own
    const MatInst* dm = d.as<MatInst>();
    const int ni = (int)fs.size();
    for (int64_t k0 = 0; k0 < nmax; k0 += kPanelNB) {
      {
        Prof pr(c, "getf2");
        launch_getf2(L, dm, ni, k0, kPanelNB, prec);
      }
      {
        Prof pr(c, "laswp");
        launch_laswp(L, dm, ni, k0, kPanelNB, 0, nmax, k0, k0 + kPanelNB, prec);
      }
      {
        Prof pr(c, "trsm");
        launch_trsm_panel(L, dm, ni, k0, kPanelNB, k0 + kPanelNB, nmax, prec);
      }
      {
        Prof pr(c, prec ? "gemm_c64" : "gemm_c128");
        launch_gemm_update(L, dm, ni, k0, kPanelNB, nmax, k0 + kPanelNB, nmax, prec);
      }
    }
  }
  launch_make_perm(L, d.as<MatInst>(), (int)fs.size(), nmax);
  CUDA_TRY(c, cudaGetLastError());
  for (size_t t = 0; t < fs.size(); ++t) {
    int32_t h = 0;
    CUDA_TRY(c, cudaMemcpyAsync(&h, mi[t].info, 4, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    fs[t]->info_h = h;
  }
  return BEMGPU_OK;
}

// Compact-storage fields of a product / sweep over the system matrix of f.
void set_compact(VecInst& v, const FactorData* f) {
  if (!f->a32) return;
  const MeshData* m = f->mesh.get();
  v.a32 = 1;
  v.nbc = f->N == 2 * f->n ? 2 : 1;
  v.n_mesh = f->n;
  v.n_near = m->n_near;
  v.near_ptr = m->near_ptr.as<int32_t>();
  v.near_i = m->near_i.as<int32_t>();
  v.near_j = m->near_j.as<int32_t>();
  v.dnear = f->dnear.as<double>();
}

// Scaled copy of A into a factor buffer (single -> LU as complex64, else complex128).
int scale_copy_batch(bemgpu_ctx* c, std::vector<FactorData*>& fs, std::vector<Buf>& part,
                     bool to_promoted, std::vector<int32_t>* flags) {
  if (fs.empty()) return BEMGPU_OK;
  const Launch L = c->launch();
  std::vector<VecInst> vi(fs.size());
  Buf d_flags, d_stats;
  TRY(alloc(c, fs.size() * 4, &d_flags));
  TRY(alloc(c, fs.size() * 2 * 8, &d_stats));
  CUDA_TRY(c, cudaMemsetAsync(d_flags.p, 0, fs.size() * 4, c->stream));
  int64_t nmax = 0;
  for (size_t t = 0; t < fs.size(); ++t) {
    FactorData* f = fs[t];
    VecInst& v = vi[t];
    std::memset(&v, 0, sizeof v);
    v.A = f->A.p;
    v.n = f->N;
    v.lda = f->N;
    v.rows = f->rows.as<double>();
    v.cols = f->cols.as<double>();
    v.rowsum = f->rowsum.as<double>();
    v.cols_inv = f->cols_inv.as<double>();
    v.cols_inv32 = f->cols_inv32.as<float>();
    v.rows_inv = f->rows_inv.as<float>();
    set_compact(v, f);
    v.part = part[t].as<double>();
    v.out = to_promoted ? f->LU64.p : f->LU.p;
    v.out_single = (!to_promoted && f->single) ? 1 : 0;
    v.flag = d_flags.as<int32_t>() + t;
    v.stats = d_stats.as<double>() + 2 * t;
    nmax = std::max(nmax, f->N);
  }
  Buf d;
  TRY(to_device(c, vi, &d));
  {
    Prof pr(c, "scale_copy");
    launch_scale_copy(L, d.as<VecInst>(), (int)fs.size(), nmax);
    if (to_promoted) {  // complex128 factor: exact near values of compact systems
      int64_t mn = 0;
      for (size_t t = 0; t < fs.size(); ++t) mn = std::max(mn, vi[t].a32 ? vi[t].n_near : 0);
      launch_near_add(L, d.as<VecInst>(), (int)fs.size(), mn, 0);
    }
  }
  std::vector<double> stats;
  std::vector<int32_t> fl;
  TRY(download(c, d_stats, &stats, fs.size() * 2));
  TRY(download(c, d_flags, &fl, fs.size()));
  for (size_t t = 0; t < fs.size(); ++t) {
    fs[t]->matrix_norm = stats[2 * t];
    if (!to_promoted) fs[t]->anorm = stats[2 * t + 1];
  }
  if (flags) *flags = fl;
  return BEMGPU_OK;
}

int promote(bemgpu_ctx* c, std::vector<FactorData*>& fs, std::vector<Buf>& part) {
  if (fs.empty()) return BEMGPU_OK;
  for (FactorData* f : fs) {
    f->LU.release();  // free the low-precision factor first (fluid_system.jl:186-190)
    f->ipiv.release();
    TRY(alloc(c, (size_t)f->N * f->N * 16, &f->LU64));
    TRY(alloc(c, (size_t)f->N * 4, &f->ipiv64));
    TRY(alloc(c, 4, &f->info64));
    f->single = false;
  }
  TRY(scale_copy_batch(c, fs, part, true, nullptr));
  TRY(getrf_batch(c, fs, 0, true));
  for (FactorData* f : fs)
    if (f->info_h > 0)
      return fail(c, BEMGPU_ESINGULAR, "double-precision factor is exactly singular");
  return BEMGPU_OK;
}

// The reference's conditioning diagnostics (full.jl:364-409) of one factor: for systems of
// order at most condition_limit, the 2-norm condition numbers of A and of the
// equilibrated A from their singular values (condition.cu).  The factorisation keeps a
// copy of A and of its scales; the SVDs run on the first diagnostics read (an FP64
// Jacobi SVD of a 500 x 500 system takes about 0.2 s on a GB300, 30 times its solve).
struct CondState {
  bemgpu_ctx* c = nullptr;
  int64_t N = 0;
  bool equilibrate = true;
  Buf A, rows, cols;  // complex128 copy of the system, its row and column scales
  bool done = false;
  double cond = NAN, scaled = NAN;
};

int prepare_conditioning(bemgpu_ctx* c, std::vector<FactorData*>& fs) {
  std::vector<VecInst> expand;
  for (FactorData* f : fs) {
    f->cond.reset();
    const int64_t N = f->N;
    if (N > f->prob.condition_limit) continue;
    auto cs = std::make_shared<CondState>();
    cs->c = c;
    cs->N = N;
    cs->equilibrate = f->prob.equilibrate != 0;
    TRY(alloc(c, (size_t)N * N * 16, &cs->A));
    TRY(alloc(c, (size_t)N * 8, &cs->rows));
    TRY(alloc(c, (size_t)N * 8, &cs->cols));
    CUDA_TRY(c, cudaMemcpyAsync(cs->rows.p, f->rows.p, (size_t)N * 8, cudaMemcpyDeviceToDevice,
                                c->stream));
    CUDA_TRY(c, cudaMemcpyAsync(cs->cols.p, f->cols.p, (size_t)N * 8, cudaMemcpyDeviceToDevice,
                                c->stream));
    if (f->a32) {  // compact storage: complex64 entries + FP64 near corrections
      VecInst v;
      std::memset(&v, 0, sizeof v);
      v.A = f->A.p;
      v.n = N;
      v.lda = N;
      v.out = cs->A.p;
      set_compact(v, f);
      expand.push_back(v);
    } else {
      CUDA_TRY(c, cudaMemcpyAsync(cs->A.p, f->A.p, (size_t)N * N * 16, cudaMemcpyDeviceToDevice,
                                  c->stream));
    }
    f->cond = cs;
  }
  if (!expand.empty()) {
    Buf de;
    TRY(to_device(c, expand, &de));
    int64_t nmax = 0, mn = 0;
    for (auto& v : expand) {
      nmax = std::max(nmax, v.n);
      mn = std::max(mn, v.n_near);
    }
    const Launch L = c->launch();
    launch_expand_a32(L, de.as<VecInst>(), (int)expand.size(), nmax);
    launch_near_add(L, de.as<VecInst>(), (int)expand.size(), mn, 1);
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));  // `de` is released on return
  }
  return BEMGPU_OK;
}

// Singular values of A and of the scaled A on working copies; cond = max / min.
int compute_conditioning(CondState* cs) {
  if (cs->done) return BEMGPU_OK;
  bemgpu_ctx* c = cs->c;
  std::lock_guard<std::recursive_mutex> lk(c->mu);
  cudaSetDevice(c->device);
  const Launch L = c->launch();
  const int64_t N = cs->N;
  Buf work[2], sig[2], flags;
  SvdInst si[2];
  TRY(alloc(c, 8, &flags));
  for (int k = 0; k < 2; ++k) {
    TRY(alloc(c, (size_t)N * N * 16, &work[k]));
    TRY(alloc(c, (size_t)N * 8, &sig[k]));
    CUDA_TRY(c, cudaMemcpyAsync(work[k].p, cs->A.p, (size_t)N * N * 16,
                                cudaMemcpyDeviceToDevice, c->stream));
    std::memset(&si[k], 0, sizeof si[k]);
    si[k].a = work[k].as<double2>();
    si[k].n = N;
    si[k].lda = N;
    if (k == 1 && cs->equilibrate) {
      si[k].rows = cs->rows.as<double>();
      si[k].cols = cs->cols.as<double>();
    }
    si[k].rotated = flags.as<int32_t>() + k;
    si[k].sigma = sig[k].as<double>();
  }
  std::vector<SvdInst> hsi(si, si + 2);
  Buf ds;
  TRY(to_device(c, hsi, &ds));
  launch_svd_scale(L, ds.as<SvdInst>(), 2, N);
  const int64_t m = (N + 1) & ~int64_t(1);
  const double tol = 4.0 * 2.220446049250313e-16 * std::sqrt((double)N);
  std::vector<int32_t> rot;
  for (int sweep = 0; sweep < 60; ++sweep) {
    CUDA_TRY(c, cudaMemsetAsync(flags.p, 0, 8, c->stream));
    for (int64_t r = 0; r < m - 1; ++r) launch_jacobi_round(L, ds.as<SvdInst>(), 2, N, r, tol);
    CUDA_TRY(c, cudaGetLastError());
    TRY(download(c, flags, &rot, 2));
    if (rot[0] == 0 && rot[1] == 0) break;
  }
  launch_column_norms(L, ds.as<SvdInst>(), 2, N);
  CUDA_TRY(c, cudaGetLastError());
  double cn[2];
  for (int k = 0; k < 2; ++k) {
    std::vector<double> sv;
    TRY(download(c, sig[k], &sv, (size_t)N));
    const double mx = *std::max_element(sv.begin(), sv.end());
    const double mn = *std::min_element(sv.begin(), sv.end());
    cn[k] = mn > 0.0 ? mx / mn : INFINITY;
  }
  cs->cond = cn[0];
  cs->scaled = cs->equilibrate ? cn[1] : cn[0];
  cs->done = true;
  return BEMGPU_OK;
}

int factorize_batch(bemgpu_ctx* c, std::vector<FactorData*>& fs) {
  const Launch L = c->launch();
  std::vector<Buf> part(fs.size());
  std::vector<VecInst> vi(fs.size());
  int64_t nmax = 0;
  for (size_t t = 0; t < fs.size(); ++t) {
    FactorData* f = fs[t];
    f->single = f->mixed;
    f->reason = BEMGPU_REASON_NONE;
    TRY(alloc(c, (size_t)f->N * 8, &f->rows));
    TRY(alloc(c, (size_t)f->N * 8, &f->cols));
    TRY(alloc(c, (size_t)f->N * 8, &f->rowsum));
    TRY(alloc(c, (size_t)f->N * 8, &f->cols_inv));
    TRY(alloc(c, (size_t)f->N * 4, &f->rows_inv));
    TRY(alloc(c, (size_t)f->N * 4, &f->cols_inv32));
    TRY(alloc(c, (size_t)kChunks * f->N * 2 * 8, &part[t]));
    TRY(alloc(c, (size_t)f->N * f->N * (f->single ? 8 : 16), &f->LU));
    TRY(alloc(c, (size_t)f->N * 4, &f->ipiv));
    TRY(alloc(c, 4, &f->info));
    VecInst& v = vi[t];
    std::memset(&v, 0, sizeof v);
    v.A = f->A.p;
    v.n = f->N;
    v.lda = f->N;
    v.rows = f->rows.as<double>();
    v.cols = f->cols.as<double>();
    v.rowsum = f->rowsum.as<double>();
    v.rows_inv = f->rows_inv.as<float>();
    set_compact(v, f);
    v.part = part[t].as<double>();
    v.norm_floor = f->prob.norm_floor;
    nmax = std::max(nmax, f->N);
  }
  Buf d;
  TRY(to_device(c, vi, &d));
  {
    Prof pr(c, "equilibrate");
    launch_equilibrate(L, d.as<VecInst>(), (int)fs.size(), nmax);
  }
  for (FactorData* f : fs)
    if (!f->prob.equilibrate) {
      launch_fill(L, f->rows.as<double>(), f->N, 1.0);
      launch_fill(L, f->cols.as<double>(), f->N, 1.0);
    }
  TRY(prepare_conditioning(c, fs));
  std::vector<int32_t> flags;
  TRY(scale_copy_batch(c, fs, part, false, &flags));
  std::vector<FactorData*> single, dbl, prom;
  for (size_t t = 0; t < fs.size(); ++t) {
    FactorData* f = fs[t];
    if (f->single && flags[t]) {
      f->reason = BEMGPU_REASON_CONVERSION;
      prom.push_back(f);
    } else if (f->single) {
      single.push_back(f);
    } else {
      dbl.push_back(f);
    }
  }
  TRY(getrf_batch(c, single, 1, false));
  TRY(getrf_batch(c, dbl, 0, false));
  for (FactorData* f : dbl)
    if (f->info_h > 0)
      return fail(c, BEMGPU_ESINGULAR, "double-precision factor is exactly singular");
  std::vector<FactorData*> ok;
  for (FactorData* f : single) {
    if (f->info_h > 0) {
      f->reason = BEMGPU_REASON_SINGLE_SINGULAR;
      prom.push_back(f);
    } else {
      ok.push_back(f);
    }
  }
  {
    Prof pr(c, "gecon");
    TRY(estimate_rcond(c, ok));
  }
  for (FactorData* f : ok)
    if (!std::isfinite(f->rcond) || f->rcond <= f->prob.condition_guard) {
      f->reason = BEMGPU_REASON_CONDITION;
      prom.push_back(f);
    }
  // promotion needs the part scratch of each promoted instance
  std::vector<Buf> ppart;
  for (FactorData* f : prom) {
    Buf b;
    TRY(alloc(c, (size_t)kChunks * f->N * 2 * 8, &b));
    ppart.push_back(std::move(b));
  }
  TRY(promote(c, prom, ppart));
  return BEMGPU_OK;
}

int factor_batch(bemgpu_ctx* c, std::vector<FactorData*>& fs, bool assemble) {
  Timer ta(c->stream);
  if (assemble) TRY(assemble_batch(c, fs));
  double asm_ms = ta.stop();
  TRY(check_device_error(c));
  Timer tf(c->stream);
  TRY(factorize_batch(c, fs));
  double fac_ms = tf.stop();
  TRY(check_device_error(c));
  for (FactorData* f : fs) {
    f->assemble_ms = assemble ? asm_ms : 0.0;
    f->factor_ms = fac_ms;
  }
  return BEMGPU_OK;
}

// ------------------------------------------------------------------ solve chain
struct RhsState {
  double final_stats[kStats] = {0};  // residual statistics of the accepted iterate
  bool have_final = false;
  double previous = INFINITY;
  int corrections = 0, attempts = 0, stalls = 0;
  bool done = false, init = true;
  double nw = INFINITY, cw = INFINITY;
  int reason = BEMGPU_REASON_NONE;
};

struct SolveInst {
  FactorData* f;
  int32_t R;
  Buf dirs, pinc, qinc, b, x, y, den, work, work2, stats, part, active, changed, tmp;
  Buf xs, xa;  // split x of compact products
  std::vector<RhsState> rs;
};

void fill_vec(VecInst& v, SolveInst& s, const void* A, int64_t N) {
  std::memset(&v, 0, sizeof v);
  v.A = A;
  v.n = N;
  v.lda = N;
  v.rows = s.f->rows.as<double>();
  v.cols = s.f->cols.as<double>();
  v.part = s.part.as<double>();
  v.nrhs = s.R;
  v.x = s.x.as<double>();
  v.ldx = N;
  v.b = s.b.as<double>();
  v.ldb = N;
  v.y = s.y.as<double>();
  v.ldy = N;
  v.den = s.den.as<double>();
  v.stats = s.stats.as<double>();
  v.active = s.active.as<int32_t>();
  v.changed = s.changed.as<int32_t>();
  v.out = s.work.p;
  v.out_single = s.f->single ? 1 : 0;
  if (s.f->a32 && (A == s.f->A.p || A == s.f->Mrhs.p)) {
    set_compact(v, s.f);
    if (A == s.f->Mrhs.p) {  // the rhs operator: n x n, its own corrections
      v.nbc = 1;
      v.dnear = s.f->dnear_rhs.as<double>();
    }
    v.xs = s.xs.as<float4>();
    v.xa = s.xa.as<float>();
  }
}

// x (mode 0) or x += (mode 1) the scaled solve of the vectors in `src` (b or residual)
// for the rhs flagged in `mask`; corrections go through the current factor precision.
int correction_pass(bemgpu_ctx* c, std::vector<SolveInst*>& ss, bool from_b,
                    const std::vector<std::vector<int32_t>>& mask, int mode) {
  const Launch L = c->launch();
  std::vector<VecInst> vi;
  std::vector<SolveInst*> who;
  for (size_t t = 0; t < ss.size(); ++t) {
    bool any = false;
    for (int32_t m : mask[t]) any |= (m != 0);
    if (!any) continue;
    SolveInst& s = *ss[t];
    CUDA_TRY(c, cudaMemcpyAsync(s.active.p, mask[t].data(), mask[t].size() * 4,
                                cudaMemcpyHostToDevice, c->stream));
    CUDA_TRY(c, cudaMemsetAsync(s.changed.p, 0, (size_t)s.R * 4, c->stream));
    VecInst v;
    fill_vec(v, s, s.f->A.p, s.f->N);
    if (from_b) v.y = s.b.as<double>();
    vi.push_back(v);
    who.push_back(&s);
  }
  if (who.empty()) return BEMGPU_OK;
  Buf d;
  TRY(to_device(c, vi, &d));
  int64_t nmax = 0;
  int32_t rmax = 0;
  for (SolveInst* s : who) {
    nmax = std::max(nmax, s->f->N);
    rmax = std::max(rmax, s->R);
  }
  launch_corr_prep(L, d.as<VecInst>(), (int)vi.size(), nmax, rmax);
  for (int prec : {1, 0}) {
    std::vector<MatInst> mi;
    int64_t pn = 0;
    int32_t pr = 0;
    for (SolveInst* s : who) {
      if ((s->f->single ? 1 : 0) != prec) continue;
      MatInst m{};
      m.a = s->f->factor_ptr();
      m.n = s->f->N;
      m.lda = s->f->N;
      m.ipiv = s->f->ipiv_ptr();
      m.info = s->f->info_ptr();
      if (!s->work2.p) TRY(alloc(c, (size_t)s->f->N * s->R * 16, &s->work2));
      m.x = s->work.p;
      m.y = s->work2.p;
      m.perm = s->f->perm_ptr();
      m.ldx = s->f->N;
      m.nrhs = s->R;
      m.active = 1;
      mi.push_back(m);
      pn = std::max(pn, s->f->N);
      pr = std::max(pr, s->R);
    }
    if (mi.empty()) continue;
    Buf dm;
    TRY(to_device(c, mi, &dm));
    TrsvWork tw{1};
    Prof p(c, "getrs");
    launch_getrs(L, dm.as<MatInst>(), (int)mi.size(), pn, pr, 0, prec, 1, &tw);
  }
  launch_corr_apply(L, d.as<VecInst>(), (int)vi.size(), nmax, rmax, mode);
  CUDA_TRY(c, cudaGetLastError());
  return BEMGPU_OK;
}

// residual y = b - A x, den, statistics for all rhs of the given instances
int residual_pass(bemgpu_ctx* c, std::vector<SolveInst*>& ss,
                  std::vector<std::vector<double>>* stats) {
  const Launch L = c->launch();
  std::vector<VecInst> vi(ss.size());
  int64_t nmax = 0;
  int32_t rmax = 0;
  for (size_t t = 0; t < ss.size(); ++t) {
    fill_vec(vi[t], *ss[t], ss[t]->f->A.p, ss[t]->f->N);
    nmax = std::max(nmax, ss[t]->f->N);
    rmax = std::max(rmax, ss[t]->R);
  }
  Buf d;
  TRY(to_device(c, vi, &d));
  {
    Prof p(c, "residual");
    // rows per thread of the compact products, measured on the live pass (idempotent: the
    // last candidate's outputs are the pass's outputs)
    bool any32 = false;
    for (auto* s : ss) any32 |= s->f->a32;
    const std::string key = "gemv/" + std::to_string(vi.size()) + "/" +
                            std::to_string(log2_bucket(nmax)) + "/" + std::to_string(rmax > 1);
    const int rows = any32 ? tune_pick(c, key, {2, 1},
                                       [&](int r) {
                                         launch_gemv(L, d.as<VecInst>(), (int)vi.size(), nmax,
                                                     rmax, 1, r);
                                       },
                                       [] {})
                           : 2;
    launch_gemv(L, d.as<VecInst>(), (int)vi.size(), nmax, rmax, 1, rows);
    launch_resid_stats(L, d.as<VecInst>(), (int)vi.size(), rmax);
  }
  stats->resize(ss.size());
  for (size_t t = 0; t < ss.size(); ++t)
    TRY(download(c, ss[t]->stats, &(*stats)[t], (size_t)ss[t]->R * kStats));
  return BEMGPU_OK;
}

// Conditioning (filled when read, see CondState) and derivative-evaluation fields of a
// factor's diagnostics.
void factor_conditioning(const FactorData* f, bemgpu_diagnostics* dg) {
  dg->conditioning = f->cond ? 1 : 0;
  dg->condition_number = dg->scaled_condition_number = NAN;
  dg->condition_limit = f->prob.condition_limit;
  const bool muller = f->kind == kAsmMuller || (f->kind == kAsmRegion && !f->region_cbie);
  dg->derivative_exterior = dg->derivative_interior = muller ? 1 : 0;
}

// The condition numbers of a diagnostics record whose conditioning data is `cs`.
int read_conditioning(const std::shared_ptr<CondState>& cs, bemgpu_diagnostics* dg) {
  if (!cs) return BEMGPU_OK;
  TRY(compute_conditioning(cs.get()));
  dg->condition_number = cs->cond;
  dg->scaled_condition_number = cs->scaled;
  return BEMGPU_OK;
}

void normwise(const double* st, double matrix_norm, double* nw, double* cw) {
  if (st[8] != 0.0) {
    *nw = *cw = INFINITY;
    return;
  }
  const double rn = st[0], xn = st[2], bn = st[3];
  const double scale = matrix_norm * xn + bn;
  if (!std::isfinite(scale))
    *nw = INFINITY;
  else if (scale == 0.0)
    *nw = rn == 0.0 ? 0.0 : INFINITY;
  else
    *nw = rn / scale;
  *cw = st[1];
}

int solve_batch(bemgpu_ctx* c, std::vector<FactorData*>& fs, const std::vector<int32_t>& nrhs,
                const std::vector<const double*>& incidence, std::vector<SolutionData*>& out) {
  const Launch L = c->launch();
  Timer tsolve(c->stream);
  const size_t F = fs.size();
  std::vector<SolveInst> si(F);
  std::vector<WaveInst> wi(F);
  int64_t nmax = 0;
  int32_t rmax = 0;
  for (size_t t = 0; t < F; ++t) {
    FactorData* f = fs[t];
    SolveInst& s = si[t];
    s.f = f;
    s.R = nrhs[t];
    if (s.R <= 0) return fail(c, BEMGPU_EINVAL, "nrhs must be positive");
    std::vector<double> dirs(3 * (size_t)s.R);
    for (int r = 0; r < s.R; ++r) {
      const double be = incidence[t][2 * r], al = incidence[t][2 * r + 1];
      if (!(std::isfinite(be) && std::isfinite(al)))
        return fail(c, BEMGPU_EINVAL, "incidence angles must be finite");
      dirs[3 * r] = std::cos(be);
      dirs[3 * r + 1] = std::sin(be) * std::cos(al);
      dirs[3 * r + 2] = std::sin(be) * std::sin(al);
    }
    out[t]->dirs = dirs;
    const int64_t n = f->n, N = f->N;
    TRY(upload(c, dirs, &s.dirs));
    TRY(alloc(c, (size_t)n * s.R * 16, &s.pinc));
    TRY(alloc(c, (size_t)n * s.R * 16, &s.qinc));
    TRY(alloc(c, (size_t)N * s.R * 16, &s.b));
    TRY(alloc(c, (size_t)N * s.R * 16, &s.x));
    TRY(alloc(c, (size_t)N * s.R * 16, &s.y));
    TRY(alloc(c, (size_t)N * s.R * 8, &s.den));
    if (f->a32) {
      TRY(alloc(c, (size_t)N * s.R * 16, &s.xs));
      TRY(alloc(c, (size_t)N * s.R * 4, &s.xa));
    }
    TRY(alloc(c, (size_t)N * s.R * 16, &s.work));
    TRY(alloc(c, (size_t)kStats * s.R * 8, &s.stats));
    TRY(alloc(c, (size_t)std::max<int64_t>(kChunks * (int64_t)s.R * N * 3, kChunks * N * 2) * 8,
              &s.part));
    TRY(alloc(c, (size_t)s.R * 4, &s.active));
    TRY(alloc(c, (size_t)s.R * 4, &s.changed));
    TRY(alloc(c, (size_t)n * s.R * 16, &out[t]->ps));
    TRY(alloc(c, (size_t)n * s.R * 16, &out[t]->qs));
    s.rs.assign((size_t)s.R, RhsState{});
    WaveInst& w = wi[t];
    std::memset(&w, 0, sizeof w);
    w.panels = f->mesh->panels.as<double>();
    w.n = n;
    w.k = f->prob.k;
    w.nrhs = s.R;
    w.dirs = s.dirs.as<double>();
    w.p = s.pinc.as<double>();
    w.q = s.qinc.as<double>();
    w.ldp = n;
    nmax = std::max(nmax, N);
    rmax = std::max(rmax, s.R);
  }
  Buf d_wi;
  TRY(to_device(c, wi, &d_wi));
  {
    Prof p(c, "incident");
    launch_incident(L, d_wi.as<WaveInst>(), (int)F, nmax, rmax);
  }
  // ---- forcing b
  {
    std::vector<VecInst> gv;  // products with a matrix
    std::vector<TraceInst> stack, cbie;
    for (size_t t = 0; t < F; ++t) {
      SolveInst& s = si[t];
      FactorData* f = s.f;
      if (f->kind == kAsmBM || f->kind == kAsmCBIE) {
        VecInst v;
        fill_vec(v, s, f->Mrhs.p, f->n);
        v.x = f->rhs_is_m2 ? s.qinc.as<double>() : s.pinc.as<double>();
        v.ldx = f->n;
        v.y = s.b.as<double>();
        v.ldy = f->N;
        gv.push_back(v);
      } else {
        TraceInst tr{};
        tr.pinc = s.pinc.as<double>();
        tr.qinc = s.qinc.as<double>();
        tr.n = f->n;
        tr.nrhs = s.R;
        tr.ps = (f->kind == kAsmMuller || f->kind == kAsmRegion) ? s.b.as<double>()
                                                                 : s.x.as<double>();
        if (f->kind == kAsmRegion) {  // plane wave on the surfaces bordering the exterior
          tr.outer = f->outer.as<int8_t>();
          tr.stack_q = f->region_cbie ? 0 : 1;
        }
        stack.push_back(tr);
        if (f->kind == kAsmFluidCBIE) {
          VecInst v;
          fill_vec(v, s, f->A.p, f->N);
          v.x = s.x.as<double>();
          v.y = s.y.as<double>();
          gv.push_back(v);
          TraceInst cb{};
          cb.x = s.y.as<double>();
          cb.n = f->n;
          cb.nrhs = s.R;
          cb.ps = s.b.as<double>();
          cbie.push_back(cb);
        }
      }
    }
    Prof p(c, "forcing");
    Buf d1, d2, d3;
    if (!stack.empty()) {
      TRY(to_device(c, stack, &d1));
      launch_stack(L, d1.as<TraceInst>(), (int)stack.size(), nmax, rmax);
    }
    if (!gv.empty()) {
      TRY(to_device(c, gv, &d2));
      launch_gemv(L, d2.as<VecInst>(), (int)gv.size(), nmax, rmax, 0);
    }
    if (!cbie.empty()) {
      TRY(to_device(c, cbie, &d3));
      launch_cbie_forcing(L, d3.as<TraceInst>(), (int)cbie.size(), nmax, rmax);
    }
  }
  // ---- solve / refine
  std::vector<SolveInst*> all;
  for (auto& s : si) all.push_back(&s);
  std::vector<std::vector<int32_t>> mask(F);
  for (size_t t = 0; t < F; ++t) mask[t].assign((size_t)si[t].R, 1);
  TRY(correction_pass(c, all, true, mask, 0));
  for (auto& s : si)
    for (auto& r : s.rs) r.init = false;
  const int kMaxRounds = 64;
  for (int round = 0; round < kMaxRounds; ++round) {
    std::vector<SolveInst*> pend;
    for (auto& s : si)
      if (s.f->mixed)
        for (auto& r : s.rs)
          if (!r.done) {
            pend.push_back(&s);
            break;
          }
    if (pend.empty()) break;
    std::vector<std::vector<double>> st;
    TRY(residual_pass(c, pend, &st));
    std::vector<FactorData*> to_promote;
    std::vector<std::vector<int32_t>> init_mask(pend.size()), corr_mask(pend.size());
    for (size_t t = 0; t < pend.size(); ++t) {
      SolveInst& s = *pend[t];
      init_mask[t].assign((size_t)s.R, 0);
      corr_mask[t].assign((size_t)s.R, 0);
      bool promote_me = false;
      for (int r = 0; r < s.R; ++r) {
        RhsState& q = s.rs[r];
        if (q.done) continue;
        double nw, cw;
        normwise(&st[t][(size_t)r * kStats], s.f->matrix_norm, &nw, &cw);
        q.nw = nw;
        q.cw = cw;
        const double metric = std::max(nw, cw);
        if (std::isfinite(metric) && metric <= s.f->prob.refine_tolerance) {
          q.done = true;
          std::memcpy(q.final_stats, &st[t][(size_t)r * kStats], sizeof q.final_stats);
          q.have_final = true;
          continue;
        }
        q.stalls = metric >= q.previous * 0.9 ? q.stalls + 1 : 0;
        int reason = !std::isfinite(metric) ? BEMGPU_REASON_NONFINITE
                     : q.attempts >= s.f->prob.refine_maxiter ? BEMGPU_REASON_ITERATION_LIMIT
                     : q.stalls >= 2 ? BEMGPU_REASON_STAGNATION
                                     : BEMGPU_REASON_NONE;
        if (reason != BEMGPU_REASON_NONE) {
          if (!s.f->single)
            return fail(c, BEMGPU_ENOTCONVERGED,
                        "double-precision fallback failed backward-error acceptance");
          if (!promote_me) s.f->reason = reason;
          promote_me = true;
          q.previous = INFINITY;
          q.attempts = 0;
          q.stalls = 0;
          init_mask[t][r] = 1;
        } else {
          corr_mask[t][r] = 1;
          q.previous = metric;
        }
      }
      if (promote_me) to_promote.push_back(s.f);
    }
    if (!to_promote.empty()) {
      std::vector<Buf> ppart;
      for (FactorData* f : to_promote) {
        Buf b;
        TRY(alloc(c, (size_t)kChunks * f->N * 2 * 8, &b));
        ppart.push_back(std::move(b));
      }
      TRY(promote(c, to_promote, ppart));
    }
    TRY(correction_pass(c, pend, true, init_mask, 0));
    TRY(correction_pass(c, pend, false, corr_mask, 1));
    // stagnation check on the corrected rhs
    for (size_t t = 0; t < pend.size(); ++t) {
      SolveInst& s = *pend[t];
      bool anyc = false;
      for (int32_t m : corr_mask[t]) anyc |= m != 0;
      if (!anyc) continue;
      std::vector<int32_t> ch;
      TRY(download(c, s.changed, &ch, (size_t)s.R));
      std::vector<FactorData*> stag;
      std::vector<int32_t> redo((size_t)s.R, 0);
      for (int r = 0; r < s.R; ++r) {
        if (!corr_mask[t][r]) continue;
        RhsState& q = s.rs[r];
        if (!ch[r]) {
          if (!s.f->single)
            return fail(c, BEMGPU_ENOTCONVERGED, "double-precision correction stagnated");
          if (stag.empty()) stag.push_back(s.f);
          s.f->reason = BEMGPU_REASON_STAGNATION;
          q.previous = INFINITY;
          q.attempts = 0;
          q.stalls = 0;
          redo[r] = 1;
        } else {
          q.corrections++;
          q.attempts++;
        }
      }
      if (!stag.empty()) {
        std::vector<Buf> ppart;
        Buf b;
        TRY(alloc(c, (size_t)kChunks * s.f->N * 2 * 8, &b));
        ppart.push_back(std::move(b));
        TRY(promote(c, stag, ppart));
        std::vector<SolveInst*> one{&s};
        std::vector<std::vector<int32_t>> m1{redo};
        TRY(correction_pass(c, one, true, m1, 0));
      }
    }
    if (round == kMaxRounds - 1)
      return fail(c, BEMGPU_ENOTCONVERGED, "refinement did not terminate");
  }
  // ---- traces and residual diagnostics
  {
    std::vector<TraceInst> ti(F);
    int64_t n_max = 0;
    for (size_t t = 0; t < F; ++t) {
      SolveInst& s = si[t];
      TraceInst& tr = ti[t];
      std::memset(&tr, 0, sizeof tr);
      tr.x = s.x.as<double>();
      tr.ldx = s.f->N;
      tr.pinc = s.pinc.as<double>();
      tr.qinc = s.qinc.as<double>();
      tr.n = s.f->n;
      tr.ps = out[t]->ps.as<double>();
      tr.qs = out[t]->qs.as<double>();
      tr.nrhs = s.R;
      tr.kind = s.f->kind == kAsmMuller ? 2
                : s.f->kind == kAsmFluidCBIE ? 3
                : s.f->kind == kAsmRegion ? 4
                : (s.f->prob.boundary == BEMGPU_RIGID ? 0 : 1);
      if (s.f->kind == kAsmRegion) tr.outer = s.f->outer.as<int8_t>();
      n_max = std::max(n_max, s.f->n);
    }
    Buf d;
    TRY(to_device(c, ti, &d));
    launch_traces(L, d.as<TraceInst>(), (int)F, n_max, rmax);
  }
  // residual diagnostics: refined right-hand sides reuse the statistics of their
  // accepted iterate; the others get one residual pass
  std::vector<SolveInst*> need;
  std::vector<size_t> need_idx;
  for (size_t t = 0; t < F; ++t) {
    bool all_final = si[t].f->mixed;
    for (auto& r : si[t].rs) all_final &= r.have_final;
    if (!all_final) {
      need.push_back(&si[t]);
      need_idx.push_back(t);
    }
  }
  std::vector<std::vector<double>> st(F);
  if (!need.empty()) {
    std::vector<std::vector<double>> st2;
    TRY(residual_pass(c, need, &st2));
    for (size_t u = 0; u < need.size(); ++u) st[need_idx[u]] = st2[u];
  }
  for (size_t t = 0; t < F; ++t)
    if (st[t].empty()) {
      st[t].resize((size_t)si[t].R * kStats);
      for (int r = 0; r < si[t].R; ++r)
        std::memcpy(&st[t][(size_t)r * kStats], si[t].rs[r].final_stats,
                    sizeof(double) * kStats);
    }
  double solve_ms = tsolve.stop();
  TRY(check_device_error(c));
  for (size_t t = 0; t < F; ++t) {
    SolveInst& s = si[t];
    FactorData* f = s.f;
    bemgpu_diagnostics& dg = out[t]->diag;
    std::memset(&dg, 0, sizeof dg);
    dg.unknown_count = f->N;
    dg.quadrature_nodes = f->n;
    dg.near_pairs = f->mesh ? f->mesh->n_near : 0;
    dg.formulation = f->kind == kAsmRegion ? (f->region_cbie ? BEMGPU_CBIE : BEMGPU_MULLER)
                                           : formulation_of(f->kind);
    dg.precision = f->prob.precision;
    dg.factor_precision = f->single ? 0 : 1;
    dg.refinement_reason = f->reason;
    dg.equilibrate = f->prob.equilibrate;
    dg.coupling_re = 0.0;
    dg.coupling_im = f->kind == kAsmBM ? 1.0 / f->prob.k : 0.0;
    dg.single_reciprocal_condition = f->rcond;
    dg.assemble_ms = f->assemble_ms;
    dg.factor_ms = f->factor_ms;
    dg.solve_ms = solve_ms;
    dg.total_ms = f->assemble_ms + f->factor_ms + solve_ms;
    dg.device_bytes = (int64_t)f->bytes();
    dg.nrhs = s.R;
    dg.info = f->info_h;
    factor_conditioning(f, &dg);
    for (int r = 0; r < s.R; ++r) {
      const double* q = &st[t][(size_t)r * kStats];
      double an = std::sqrt(q[4]), bn = std::sqrt(q[5]);
      double rel = bn == 0.0 ? (an == 0.0 ? 0.0 : INFINITY) : an / bn;
      double san = std::sqrt(q[6]), sbn = std::sqrt(q[7]);
      double srel = sbn == 0.0 ? (san == 0.0 ? 0.0 : INFINITY) : san / sbn;
      double nw, cw;
      normwise(q, f->matrix_norm, &nw, &cw);
      dg.absolute_residual = std::max(dg.absolute_residual, an);
      dg.relative_residual = std::max(dg.relative_residual, rel);
      dg.scaled_absolute_residual = std::max(dg.scaled_absolute_residual, san);
      dg.scaled_relative_residual = std::max(dg.scaled_relative_residual, srel);
      dg.normwise_backward_error = std::max(dg.normwise_backward_error, nw);
      dg.componentwise_backward_error = std::max(dg.componentwise_backward_error, cw);
      dg.refinement_iterations = std::max(dg.refinement_iterations, s.rs[r].corrections);
    }
    out[t]->nrhs = s.R;
    out[t]->mesh = f->mesh;
    out[t]->base_mesh = f->base_mesh;
    out[t]->cond = f->cond;
    out[t]->k = f->prob.k;
    out[t]->boundary = f->prob.boundary;
    out[t]->g = f->prob.density_contrast;
    out[t]->h = f->prob.soundspeed_contrast;
    if (f->kind == kAsmRegion) {  // keep the unknowns [p; v] of every interface
      out[t]->region = true;
      TRY(alloc(c, (size_t)f->N * s.R * 16, &out[t]->xsol));
      CUDA_TRY(c, cudaMemcpyAsync(out[t]->xsol.p, s.x.p, (size_t)f->N * s.R * 16,
                                  cudaMemcpyDeviceToDevice, c->stream));
    }
  }
  return BEMGPU_OK;
}

}  // namespace

// ===================================================================== serving
namespace {
using Clock = std::chrono::steady_clock;

struct ServerReq {
  int64_t id = 0;
  std::shared_ptr<MeshData> mesh;
  bemgpu_problem prob{};
  std::vector<double> ks, inc, amps;
  int32_t nfreq = 0, nangles = 0, done_freq = 0, untaken = 0;
  int status = BEMGPU_OK;
  std::string err;  // message of a failed request
  bool finished = false;
  Clock::time_point t_submit, t_done;
};

struct FKey {
  const MeshData* m;
  double k, g, h;
  int32_t b, f, p, a;
  bool operator<(const FKey& o) const {
    return std::tie(m, k, g, h, b, f, p, a) < std::tie(o.m, o.k, o.g, o.h, o.b, o.f, o.p, o.a);
  }
};

struct CacheEnt {
  std::shared_ptr<FactorData> f;
  uint64_t last = 0;
  size_t bytes = 0;
  int lane = -1;  // the lane whose running batch uses it (one at a time), or -1
};

FKey key_of(const ServerReq& r, double k) {
  const bool fl = r.prob.boundary == BEMGPU_FLUID;
  return FKey{r.mesh.get(), k, fl ? r.prob.density_contrast : 1.0,
              fl ? r.prob.soundspeed_contrast : 1.0, r.prob.boundary, r.prob.formulation,
              r.prob.precision, r.prob.assembly};
}

int64_t order_of(const ServerReq& r) {
  return r.prob.boundary == BEMGPU_FLUID ? 2 * r.mesh->n : r.mesh->n;
}

// device bytes of the solve temporaries of one item (nangles right-hand sides)
size_t solve_bytes(const ServerReq& r) {
  const size_t N = (size_t)order_of(r);
  const size_t R = (size_t)r.nangles;
  const size_t b = N * R * (16 * 6 + 8) + (size_t)kChunks * R * N * 3 * 8;
  return b + b / 20;
}

// device bytes of one factor plus the solve temporaries of its right-hand sides
size_t item_bytes(const ServerReq& r) {
  const size_t n = (size_t)r.mesh->n;
  const bool fl = r.prob.boundary == BEMGPU_FLUID;
  const size_t N = fl ? 2 * n : n;
  const bool mixed = r.prob.precision == BEMGPU_MIXED;
  const bool a32 = r.prob.assembly == BEMGPU_ASSEMBLY_SINGLE ||
                   (r.prob.assembly == BEMGPU_ASSEMBLY_DEFAULT && mixed);
  size_t b = N * N * (a32 ? 8 : 16) + N * N * (mixed ? 8 : 16) + (fl ? 0 : n * n * (a32 ? 8 : 16));
  b += a32 ? (size_t)r.mesh->n_near * (fl ? 4 : 2) * 16 : 0;
  b += 2 * tc_pack_bytes((int64_t)N, 128) + N * 64;
  return b + b / 20 + solve_bytes(r);
}

// One work item: a (request, wavenumber) pair waiting for a lane.  `retry`: its batch
// failed to allocate device memory once; it runs again when no other batch is on the
// device, and fails for good if that fails too.
struct Pending {
  std::shared_ptr<ServerReq> req;
  int32_t fi = 0;
  FKey key{};
  int64_t N = 0;
  bool retry = false;
};
}  // namespace

struct bemgpu_server {
  bemgpu_ctx* c = nullptr;
  bemgpu_server_options opt{};
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Pending> pending;                       // items in arrival order
  std::map<int64_t, std::shared_ptr<ServerReq>> all;
  std::map<FKey, CacheEnt> cache;
  std::map<FKey, int> factoring;                     // keys a running batch factors (lane)
  uint64_t tick = 0, cached_bytes = 0, reserved = 0;
  int64_t waiting = 0;                               // requests with untaken items
  int running = 0;                                   // batches on the device
  int64_t next_id = 1;
  bemgpu_server_stats st{};
  bool stop = false;
  std::vector<bemgpu_ctx*> lanes;
  std::vector<int64_t> lane_head;                    // system order heading each lane's batch
  std::vector<std::thread> workers;
};

namespace {

void finish_req(bemgpu_server* S, ServerReq& r, int status, const std::string& err = "") {
  if (r.finished) return;
  r.status = status;
  r.err = err;
  r.finished = true;
  r.t_done = Clock::now();
  if (r.untaken > 0) {
    r.untaken = 0;
    S->waiting--;
  }
  if (status == BEMGPU_OK)
    S->st.completed++;
  else
    S->st.failed++;
}

struct Item {
  std::shared_ptr<ServerReq> req;
  int32_t fi;
  FKey key;
  bool retry;
};

// One batch: factor the uncached keys, solve every item, read back backscatter.
int run_batch(bemgpu_ctx* c, std::vector<Item>& items,
              std::map<FKey, std::shared_ptr<FactorData>>& factors, int64_t* nfactored) {
  std::vector<std::shared_ptr<FactorData>> fresh;
  std::vector<FactorData*> fs;
  for (auto& kv : factors)
    if (!kv.second) {
      const ServerReq& r = *std::find_if(items.begin(), items.end(), [&](const Item& it) {
                              return !(it.key < kv.first) && !(kv.first < it.key);
                            })->req;
      auto f = std::make_shared<FactorData>();
      f->c = c;
      f->prob = r.prob;
      f->prob.k = kv.first.k;
      int kind = 0;
      TRY(check_problem(c, f->prob, &kind));
      f->kind = kind;
      TRY(bind_mesh(c, f.get(), r.mesh));
      kv.second = f;
      fresh.push_back(f);
      fs.push_back(f.get());
    }
  if (!fs.empty()) TRY(factor_batch(c, fs, true));
  std::vector<FactorData*> sf;
  std::vector<int32_t> nr;
  std::vector<const double*> inc;
  std::vector<std::shared_ptr<SolutionData>> sols;
  std::vector<SolutionData*> outs;
  for (auto& it : items) {
    sf.push_back(factors[it.key].get());
    nr.push_back(it.req->nangles);
    inc.push_back(it.req->inc.data());
    auto sd = std::make_shared<SolutionData>();
    sd->c = c;
    sols.push_back(sd);
    outs.push_back(sd.get());
  }
  TRY(solve_batch(c, sf, nr, inc, outs));
  // backscatter of every (item, angle) in one far-field launch
  std::vector<WaveInst> wi(items.size());
  std::vector<Buf> dirs(items.size()), amps(items.size()), parts(items.size());
  int32_t rmax = 0;
  int64_t nmx = 0;
  for (size_t t = 0; t < items.size(); ++t) {
    SolutionData* sd = outs[t];
    std::vector<double> d(3 * (size_t)sd->nrhs);
    for (size_t q = 0; q < d.size(); ++q) d[q] = -sd->dirs[q];
    TRY(upload(c, d, &dirs[t]));
    TRY(alloc(c, (size_t)sd->nrhs * 16, &amps[t]));
    WaveInst& w = wi[t];
    std::memset(&w, 0, sizeof w);
    w.panels = sd->mesh->panels.as<double>();
    w.n = sd->mesh->n;
    w.k = sd->k;
    w.nrhs = sd->nrhs;
    w.ndir = 1;
    w.dirs = dirs[t].as<double>();
    w.p = sd->ps.as<double>();
    w.q = sd->qs.as<double>();
    w.out = amps[t].as<double>();
    w.ldp = sd->mesh->n;
    TRY(alloc(c, far_field_scratch(w.n, 1, w.nrhs), &parts[t]));
    w.part = parts[t].as<double>();
    rmax = std::max(rmax, sd->nrhs);
    nmx = std::max(nmx, w.n);
  }
  Buf dw;
  TRY(upload(c, wi, &dw));
  {
    Prof p(c, "far_field");
    launch_far_field(c->launch(), dw.as<WaveInst>(), (int)wi.size(), rmax, 1, nmx);
  }
  CUDA_TRY(c, cudaGetLastError());
  for (size_t t = 0; t < items.size(); ++t) {
    ServerReq& r = *items[t].req;
    double* dst = r.amps.data() + 2 * (size_t)items[t].fi * r.nangles;
    CUDA_TRY(c, cudaMemcpyAsync(dst, amps[t].p, (size_t)r.nangles * 16, cudaMemcpyDeviceToHost,
                                c->stream));
  }
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  TRY(check_device_error(c));
  *nfactored = (int64_t)fresh.size();
  return BEMGPU_OK;
}

// Drops least recently used cache entries that no running batch uses until the cache
// holds at most target bytes.
void evict_lru(bemgpu_server* S, uint64_t target) {
  while (S->cached_bytes > target) {
    auto victim = S->cache.end();
    for (auto it = S->cache.begin(); it != S->cache.end(); ++it) {
      if (it->second.lane >= 0) continue;
      if (victim == S->cache.end() || it->second.last < victim->second.last) victim = it;
    }
    if (victim == S->cache.end()) break;
    S->cached_bytes -= victim->second.bytes;
    S->cache.erase(victim);
    S->st.evictions++;
  }
}

// Bytes held by the lanes' allocations (cached factors and running batches).
uint64_t lanes_live(bemgpu_server* S) {
  bemgpu_ctx* r = S->c;
  std::lock_guard<std::mutex> lk(r->acct_mu);
  uint64_t b = 0;
  for (bemgpu_ctx* l : S->lanes) b += l->live;
  return b;
}

// A batch a lane has taken: its items, the factors they use (null = to factor here),
// and the memory reserved for it.
struct Batch {
  std::vector<Item> items;
  std::map<FKey, std::shared_ptr<FactorData>> factors;
  std::vector<FKey> fresh, hits;
  size_t need = 0;
};

bool same_class(int64_t a, int64_t b) { return a <= 2 * b && b <= 2 * a; }

// Takes the next batch for lane `li` (S->mu held).  Items are considered in arrival
// order; an item is takeable when its factor is neither being computed nor in use on
// another lane.  The batch is one size class: items whose system order is within a
// factor of two of the head's (a batch lasts as long as its largest factorisation, so
// small systems do not wait behind large ones).  The head is the oldest takeable item,
// unless another lane already runs that item's class and an item of another class waits:
// then the oldest such item heads it, so that one large request cannot hold every lane
// while small ones wait.  Items join while the batch stays within max_batch
// factorisations and the memory the budget has left after the cache's unevictable part
// and the other lanes' batches.  Returns false when nothing can be taken now; *fail_head
// is set when the first item cannot fit even on an idle device with an empty cache.
bool take_batch(bemgpu_server* S, int li, Batch* B, std::shared_ptr<ServerReq>* fail_head) {
  bemgpu_ctx* c = S->c;
  // items of failed requests leave the queue
  S->pending.erase(std::remove_if(S->pending.begin(), S->pending.end(),
                                  [](const Pending& p) { return p.req->finished; }),
                   S->pending.end());
  const uint64_t usable = (uint64_t)(0.92 * (double)c->budget);
  const uint64_t total = total_live(c), lanes = lanes_live(S);
  const uint64_t outside = total > lanes ? total - lanes : 0;
  uint64_t evictable = 0;
  for (auto& kv : S->cache)
    if (kv.second.lane < 0) evictable += kv.second.bytes;
  const uint64_t held = outside + S->cached_bytes + S->reserved;
  const uint64_t avail = usable > held ? usable - held : 0;
  // an item whose batch ran out of device memory waits until no batch is on the device
  if (S->running > 0)
    for (const Pending& p : S->pending)
      if (p.retry) return false;
  auto takeable = [&](const Pending& p) {
    auto ce = S->cache.find(p.key);
    if (ce != S->cache.end()) return ce->second.lane < 0;  // else in use on another lane
    return S->factoring.count(p.key) == 0;                 // else being factored elsewhere
  };
  auto busy_class = [&](int64_t N) {
    for (size_t l = 0; l < S->lane_head.size(); ++l)
      if ((int)l != li && S->lane_head[l] > 0 && same_class(N, S->lane_head[l])) return true;
    return false;
  };
  int64_t nhead = -1, first = -1;
  for (const Pending& p : S->pending) {
    if (!takeable(p)) continue;
    if (first < 0) first = p.N;
    if (!busy_class(p.N)) {
      nhead = p.N;
      break;
    }
  }
  if (nhead < 0) nhead = first;
  if (nhead < 0) return false;
  int nnew = 0;
  bool any = false;
  std::vector<size_t> taken;  // positions in the pending deque
  for (size_t pos = 0; pos < S->pending.size(); ++pos) {
    Pending& p = S->pending[pos];
    const bool here = B->factors.count(p.key) > 0;
    auto ce = S->cache.find(p.key);
    const bool hit = !here && ce != S->cache.end();
    if (!here && !takeable(p)) continue;
    if (!same_class(p.N, nhead)) continue;
    if (!here && !hit && nnew >= S->opt.max_batch) continue;
    const size_t b = (here || hit) ? solve_bytes(*p.req) : item_bytes(*p.req);
    // a hit's factor stops counting as evictable once this batch uses it
    const uint64_t ev = evictable - (hit ? std::min<uint64_t>(evictable, ce->second.bytes) : 0);
    if (B->need + b > avail + ev) {
      if (!any) {
        // the first item does not fit: on an idle device with nothing left to evict it
        // never will
        if (S->running == 0 && S->reserved == 0 && b > (usable > outside ? usable - outside : 0))
          *fail_head = p.req;
        break;
      }
      continue;
    }
    any = true;
    B->need += b;
    if (hit) {
      ce->second.lane = li;
      ce->second.last = ++S->tick;
      evictable = ev;
      B->factors[p.key] = ce->second.f;
      B->hits.push_back(p.key);
      S->st.cache_hits++;
    } else if (!here) {
      B->factors[p.key] = nullptr;
      B->fresh.push_back(p.key);
      ++nnew;
    }
    B->items.push_back(Item{p.req, p.fi, p.key, p.retry});
    taken.push_back(pos);
  }
  if (B->items.empty()) return false;
  // make room: least recently used factors that no batch uses go first
  if (B->need > avail) {
    const uint64_t over = B->need - avail;
    evict_lru(S, S->cached_bytes > over ? S->cached_bytes - over : 0);
  }
  for (auto& k : B->fresh) S->factoring[k] = li;
  S->reserved += B->need;
  S->running++;
  S->lane_head[li] = nhead;
  for (size_t pos : taken) {
    ServerReq& r = *S->pending[pos].req;
    if (--r.untaken == 0) S->waiting--;
  }
  for (auto t = taken.rbegin(); t != taken.rend(); ++t)
    S->pending.erase(S->pending.begin() + (std::ptrdiff_t)*t);
  S->st.items += (int64_t)B->items.size();
  S->st.batches++;
  return true;
}

void lane_loop(bemgpu_server* S, int li) {
  bemgpu_ctx* lc = S->lanes[li];
  cudaSetDevice(lc->device);
  for (;;) {
    Batch B;
    {
      std::unique_lock<std::mutex> lk(S->mu);
      for (;;) {
        if (S->stop) return;
        std::shared_ptr<ServerReq> fail_head;
        if (take_batch(S, li, &B, &fail_head)) break;
        if (fail_head) {
          finish_req(S, *fail_head, BEMGPU_ENOMEM_BUDGET,
                     "the request's factor does not fit the HBM budget");
          S->cv_done.notify_all();
          continue;
        }
        S->cv_work.wait(lk);
      }
    }
    int status;
    int64_t nfactored = 0;
    std::string err;
    bool oom = false;
    Clock::time_point t0 = Clock::now();
    {
      std::lock_guard<std::recursive_mutex> ck(lc->mu);
      lc->last_cuda = cudaSuccess;
      status = run_batch(lc, B.items, B.factors, &nfactored);
      if (status != BEMGPU_OK) err = lc->err;
      oom = status == BEMGPU_ECUDA && lc->last_cuda == cudaErrorMemoryAllocation;
    }
    const double ms = std::chrono::duration<double, std::milli>(Clock::now() - t0).count();
    {
      std::lock_guard<std::mutex> lk(S->mu);
      S->st.busy_ms += ms;
      S->st.factorizations += nfactored;
      S->reserved -= std::min<uint64_t>(S->reserved, B.need);
      S->running--;
      S->lane_head[li] = -1;
      for (auto& k : B.fresh) S->factoring.erase(k);
      for (auto& k : B.hits) {
        auto it = S->cache.find(k);
        if (it == S->cache.end()) continue;
        if (status != BEMGPU_OK) {  // a factor a failed batch used is not trusted again
          S->cached_bytes -= it->second.bytes;
          S->cache.erase(it);
          continue;
        }
        // a promotion during the solve can have grown the factor
        const size_t b = it->second.f->bytes();
        S->cached_bytes = S->cached_bytes - it->second.bytes + b;
        it->second.bytes = b;
        it->second.lane = -1;
      }
      // a batch that ran out of device memory (the budget counts live blocks, not the
      // other lanes' free ones or the driver's own) goes back to the head of the queue
      // once, to run when the device holds no other batch
      std::vector<Pending> again;
      for (auto& it : B.items) {
        ServerReq& r = *it.req;
        if (status != BEMGPU_OK) {
          if (oom && !it.retry && !r.finished) {
            again.push_back(Pending{it.req, it.fi, it.key, order_of(r), true});
            if (r.untaken++ == 0) S->waiting++;
            continue;
          }
          finish_req(S, r, status, err);
          continue;
        }
        if (++r.done_freq == r.nfreq && !r.finished) finish_req(S, r, BEMGPU_OK);
      }
      S->pending.insert(S->pending.begin(), again.begin(), again.end());
      S->st.retries += (int64_t)again.size();
      if (status == BEMGPU_OK) {
        for (auto& k : B.fresh) {
          auto& f = B.factors[k];
          if (!f || S->cache.count(k)) continue;
          const size_t b = f->bytes();
          if (b > S->opt.cache_bytes) continue;
          S->cache[k] = CacheEnt{f, ++S->tick, b, -1};
          S->cached_bytes += b;
        }
      }
      evict_lru(S, S->opt.cache_bytes);
      S->st.cached_bytes = S->cached_bytes;
      // the batch's factors that did not enter the cache are freed here, before the
      // lanes that wait for memory wake up
      B.factors.clear();
      B.items.clear();
    }
    // the retry starts from a device without free blocks.  Pools are not trimmed after
    // every batch: returning blocks to the driver synchronises the device, so a lane
    // waits for the other lane's batch (measured on 300 served requests: p50 latency
    // 2.1 s -> 3.0 s, for no re-runs instead of 52)
    if (oom) drop_all_caches(lc);
    S->cv_done.notify_all();
    S->cv_work.notify_all();
  }
}
}  // namespace

// ===================================================================== C ABI
extern "C" {

namespace {
// (defined with the hierarchical-matrix build below, inside this extern "C" region)
void ras_neighbourhoods(const std::vector<double>& rec, int64_t ne, int count,
                        std::vector<int32_t>* ptr, std::vector<int32_t>* els);
}  // namespace

const char* bemgpu_version(void) { return "bemgpu 0.1.0 (sm_103a)"; }

const char* bemgpu_status_string(int s) {
  switch (s) {
    case BEMGPU_OK: return "ok";
    case BEMGPU_EINVAL: return "invalid argument";
    case BEMGPU_ETOPOLOGY: return "invalid surface topology";
    case BEMGPU_ENOMEM_BUDGET: return "HBM budget exceeded";
    case BEMGPU_ESINGULAR: return "singular matrix";
    case BEMGPU_ENOTCONVERGED: return "refinement did not converge";
    case BEMGPU_ETIMEOUT: return "device wait timed out";
    case BEMGPU_ECUDA: return "CUDA error";
    case BEMGPU_ENODEV: return "no CUDA device";
    case BEMGPU_EBUSY: return "busy";
    default: return "unknown status";
  }
}

void bemgpu_problem_init(bemgpu_problem* p) {
  if (!p) return;
  std::memset(p, 0, sizeof *p);
  p->boundary = BEMGPU_RIGID;
  p->formulation = BEMGPU_FORMULATION_DEFAULT;
  p->precision = BEMGPU_DOUBLE;
  p->equilibrate = 1;
  p->k = 1.0;
  p->density_contrast = 1.0;
  p->soundspeed_contrast = 1.0;
  p->refine_tolerance = 1e-13;
  p->refine_maxiter = 8;
  p->condition_guard = 10.0 * 1.1920928955078125e-07;
  p->near_eta = 2.0;
  p->condition_limit = 512;
  p->norm_floor = 0.0;
}

int bemgpu_schwarz_neighbourhoods(const double* nodes, int64_t n_nodes, const int64_t* triangles,
                                  int64_t n_triangles, int32_t count, int32_t* out) {
  if (!nodes || !triangles || !out || n_triangles <= 0 || count <= 0)
    return fail(nullptr, BEMGPU_EINVAL, "invalid argument");
  std::string e;
  double res = 0.0;
  int s = validate_surface(nodes, n_nodes, triangles, n_triangles, &res, &e);
  if (s != BEMGPU_OK) return fail(nullptr, s, e);
  std::vector<double> rec, verts;
  std::vector<float> recf;
  double center[3];
  build_panels(nodes, triangles, n_triangles, &rec, &recf, &verts, center);
  // node records of the Nyström node set: only the elements' first (centroid) node is read
  std::vector<double> nrec((size_t)n_triangles * kNyNodes * kPanelDoubles, 0.0);
  for (int64_t t = 0; t < n_triangles; ++t)
    for (int a = 0; a < 3; ++a)
      nrec[(size_t)t * kNyNodes * kPanelDoubles + a] = rec[(size_t)t * kPanelDoubles + 8 + a];
  std::vector<int32_t> ptr, els;
  ras_neighbourhoods(nrec, n_triangles, count, &ptr, &els);
  const int64_t m = std::min<int64_t>(count, n_triangles);
  for (int64_t t = 0; t < n_triangles; ++t)
    for (int64_t q = 0; q < m; ++q) out[t * m + q] = els[(size_t)ptr[t] + q];
  return BEMGPU_OK;
}

int bemgpu_mesh_validate(const double* nodes, int64_t n_nodes, const int64_t* triangles,
                         int64_t n_triangles, double* resolution, char* err, size_t errlen) {
  std::string e;
  int s = validate_surface(nodes, n_nodes, triangles, n_triangles, resolution, &e);
  if (err && errlen) {
    std::snprintf(err, errlen, "%s", e.c_str());
  }
  if (s != BEMGPU_OK) g_err = e;
  return s;
}

int bemgpu_mesh_hash(const double* nodes, int64_t n_nodes, const int64_t* triangles,
                     int64_t n_triangles, char out_hex[65]) {
  if (!nodes || !triangles || !out_hex || n_nodes < 0 || n_triangles < 0)
    return fail(nullptr, BEMGPU_EINVAL, "null argument");
  mesh_hash(nodes, n_nodes, triangles, n_triangles, out_hex);
  return BEMGPU_OK;
}

int bemgpu_near_pairs(const double* nodes, int64_t n_nodes, const int64_t* triangles,
                      int64_t n_triangles, double eta, int64_t* rowptr, int64_t* cols,
                      int64_t cap, int64_t* count) {
  std::string e;
  double res;
  int s = validate_surface(nodes, n_nodes, triangles, n_triangles, &res, &e);
  if (s != BEMGPU_OK) return fail(nullptr, s, e);
  std::vector<double> cent, diam;
  panel_centroids(nodes, triangles, n_triangles, &cent, &diam);
  std::vector<int64_t> rp, cl;
  near_pairs(cent, diam, eta, &rp, &cl);
  if (count) *count = (int64_t)cl.size();
  if ((int64_t)cl.size() > cap) return fail(nullptr, BEMGPU_EINVAL, "capacity too small");
  if (rowptr) std::copy(rp.begin(), rp.end(), rowptr);
  if (cols) std::copy(cl.begin(), cl.end(), cols);
  return BEMGPU_OK;
}

int bemgpu_ctx_create(int device, uint64_t hbm_budget_bytes, bemgpu_ctx** out) {
  if (!out) return fail(nullptr, BEMGPU_EINVAL, "null output");
  *out = nullptr;
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0) {
    cudaGetLastError();
    return fail(nullptr, BEMGPU_ENODEV, "no CUDA device available");
  }
  if (device < 0 || device >= count) return fail(nullptr, BEMGPU_EINVAL, "invalid device index");
  e = cudaSetDevice(device);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaSetDevice");
  auto* c = new bemgpu_ctx();
  c->device = device;
  size_t fr = 0, tot = 0;
  cudaMemGetInfo(&fr, &tot);
  c->budget = hbm_budget_bytes ? hbm_budget_bytes : (uint64_t)(0.9 * (double)fr);
  e = init_streams(c);
  if (e != cudaSuccess) {
    delete c;
    return cuda_fail(nullptr, e, "context streams");
  }
  cudaDeviceSynchronize();
  *out = c;
  return BEMGPU_OK;
}

int bemgpu_ctx_destroy(bemgpu_ctx* c) {
  if (!c) return BEMGPU_OK;
  cudaSetDevice(c->device);
  free_streams(c);
  delete c;
  return BEMGPU_OK;
}

int bemgpu_last_error(const bemgpu_ctx* c, char* buf, size_t len) {
  if (!buf || !len) return BEMGPU_EINVAL;
  std::snprintf(buf, len, "%s", c ? c->err.c_str() : g_err.c_str());
  return BEMGPU_OK;
}

int bemgpu_ctx_memory(const bemgpu_ctx* c, uint64_t* used, uint64_t* budget) {
  if (!c) return fail(nullptr, BEMGPU_EINVAL, "null context");
  if (used) *used = total_live(c);
  if (budget) *budget = root_of(c)->budget;
  return BEMGPU_OK;
}

int bemgpu_ctx_synchronize(bemgpu_ctx* c) {
  if (!c) return fail(nullptr, BEMGPU_EINVAL, "null context");
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return BEMGPU_OK;
}

int bemgpu_mesh_upload(bemgpu_ctx* c, const double* nodes, int64_t n_nodes,
                       const int64_t* triangles, int64_t n_triangles, bemgpu_mesh** out) {
  if (!c || !out) return fail(c, BEMGPU_EINVAL, "null argument");
  std::lock_guard<std::recursive_mutex> lk(c->mu);
  cudaSetDevice(c->device);
  std::shared_ptr<MeshData> m;
  TRY(make_mesh(c, nodes, n_nodes, triangles, n_triangles, 2.0, &m));
  *out = new bemgpu_mesh{m};
  return BEMGPU_OK;
}

int bemgpu_mesh_info(const bemgpu_mesh* m, int64_t* n_panels, double* resolution,
                     char hash_hex[65]) {
  if (!m) return fail(nullptr, BEMGPU_EINVAL, "null mesh");
  if (n_panels) *n_panels = m->d->n;
  if (resolution) *resolution = m->d->resolution;
  if (hash_hex) std::memcpy(hash_hex, m->d->hash, 65);
  return BEMGPU_OK;
}

int bemgpu_mesh_destroy(bemgpu_mesh* m) {
  if (m) {
    std::lock_guard<std::recursive_mutex> lk(m->d->c->mu);
    delete m;
  }
  return BEMGPU_OK;
}

int bemgpu_factor_create_batch(bemgpu_ctx* c, int32_t count, const bemgpu_mesh* const* meshes,
                               const bemgpu_problem* problems, bemgpu_factor** factors) {
  if (!c || !meshes || !problems || !factors || count <= 0)
    return fail(c, BEMGPU_EINVAL, "invalid batch arguments");
  std::lock_guard<std::recursive_mutex> lk(c->mu);
  cudaSetDevice(c->device);
  std::vector<std::shared_ptr<FactorData>> own;
  std::vector<FactorData*> fs;
  for (int32_t t = 0; t < count; ++t) {
    if (!meshes[t]) return fail(c, BEMGPU_EINVAL, "null mesh");
    int kind = 0;
    TRY(check_problem(c, problems[t], &kind));
    auto f = std::make_shared<FactorData>();
    f->c = c;
    f->prob = problems[t];
    f->kind = kind;
    TRY(bind_mesh(c, f.get(), meshes[t]->d));
    // near pairs are a mesh property; a different eta rebuilds them once
    if (!f->nystrom && std::fabs(f->prob.near_eta - f->mesh->eta) > 0) {
      return fail(c, BEMGPU_EINVAL, "near_eta differs from the mesh's (upload with that eta)");
    }
    own.push_back(f);
    fs.push_back(f.get());
  }
  TRY(factor_batch(c, fs, true));
  for (int32_t t = 0; t < count; ++t) factors[t] = new bemgpu_factor{own[t]};
  return BEMGPU_OK;
}

int bemgpu_factor_create(bemgpu_ctx* c, const bemgpu_mesh* mesh, const bemgpu_problem* problem,
                         bemgpu_factor** factor) {
  return bemgpu_factor_create_batch(c, 1, &mesh, problem, factor);
}

int bemgpu_factor_solve_batch(bemgpu_ctx* c, int32_t count, bemgpu_factor* const* factors,
                              const int32_t* nrhs, const double* const* incidence,
                              bemgpu_solution** solutions) {
  if (!c || !factors || !nrhs || !incidence || !solutions || count <= 0)
    return fail(c, BEMGPU_EINVAL, "invalid batch arguments");
  std::lock_guard<std::recursive_mutex> lk(c->mu);
  cudaSetDevice(c->device);
  std::vector<FactorData*> fs;
  std::vector<int32_t> nr;
  std::vector<const double*> inc;
  std::vector<std::shared_ptr<SolutionData>> own;
  std::vector<SolutionData*> outs;
  for (int32_t t = 0; t < count; ++t) {
    if (!factors[t] || !incidence[t]) return fail(c, BEMGPU_EINVAL, "null factor or incidence");
    if (!factors[t]->d->mesh) return fail(c, BEMGPU_EINVAL, "factor has no mesh");
    fs.push_back(factors[t]->d.get());
    nr.push_back(nrhs[t]);
    inc.push_back(incidence[t]);
    auto s = std::make_shared<SolutionData>();
    s->c = c;
    own.push_back(s);
    outs.push_back(s.get());
  }
  TRY(solve_batch(c, fs, nr, inc, outs));
  for (int32_t t = 0; t < count; ++t) solutions[t] = new bemgpu_solution{own[t]};
  return BEMGPU_OK;
}

int bemgpu_factor_solve(bemgpu_factor* f, int32_t nrhs, const double* incidence,
                        bemgpu_solution** solution) {
  if (!f) return fail(nullptr, BEMGPU_EINVAL, "null factor");
  return bemgpu_factor_solve_batch(f->d->c, 1, &f, &nrhs, &incidence, solution);
}

int bemgpu_factor_destroy(bemgpu_factor* f) {
  if (f) {
    std::lock_guard<std::recursive_mutex> lk(f->d->c->mu);
    delete f;
  }
  return BEMGPU_OK;
}

int bemgpu_factor_diagnostics(const bemgpu_factor* f, bemgpu_diagnostics* out) {
  if (!f || !out) return fail(nullptr, BEMGPU_EINVAL, "null argument");
  const FactorData* d = f->d.get();
  std::memset(out, 0, sizeof *out);
  out->unknown_count = d->N;
  out->quadrature_nodes = d->n;
  out->near_pairs = d->mesh ? d->mesh->n_near : 0;
  out->formulation = d->kind == kAsmRegion ? (d->region_cbie ? BEMGPU_CBIE : BEMGPU_MULLER)
                                           : formulation_of(d->kind);
  out->precision = d->prob.precision;
  out->factor_precision = d->single ? 0 : 1;
  out->refinement_reason = d->reason;
  out->equilibrate = d->prob.equilibrate;
  out->coupling_im = d->kind == kAsmBM ? 1.0 / d->prob.k : 0.0;
  out->single_reciprocal_condition = d->rcond;
  out->assemble_ms = d->assemble_ms;
  out->factor_ms = d->factor_ms;
  out->device_bytes = (int64_t)d->bytes();
  out->info = d->info_h;
  factor_conditioning(d, out);
  return read_conditioning(d->cond, out);
}

int bemgpu_solve(bemgpu_ctx* c, const bemgpu_mesh* mesh, const bemgpu_problem* problem,
                 int32_t nrhs, const double* incidence, bemgpu_solution** solution) {
  bemgpu_factor* f = nullptr;
  TRY(bemgpu_factor_create(c, mesh, problem, &f));
  int s = bemgpu_factor_solve(f, nrhs, incidence, solution);
  bemgpu_factor_destroy(f);
  return s;
}

int bemgpu_far_field(bemgpu_solution* sol, int32_t rhs, int64_t ndir, const double* dirs,
                     double* out) {
  if (!sol || !out) return fail(nullptr, BEMGPU_EINVAL, "null argument");
  SolutionData* s = sol->d.get();
  bemgpu_ctx* c = s->c;
  std::lock_guard<std::recursive_mutex> lk(c->mu);
  cudaSetDevice(c->device);
  if (rhs < 0 || rhs >= s->nrhs) return fail(c, BEMGPU_EINVAL, "rhs index out of range");
  std::vector<double> d;
  if (!dirs) {
    ndir = 1;
    d = {-s->dirs[3 * rhs], -s->dirs[3 * rhs + 1], -s->dirs[3 * rhs + 2]};
  } else {
    if (ndir < 0) return fail(c, BEMGPU_EINVAL, "ndir must be nonnegative");
    d.assign(dirs, dirs + 3 * ndir);
    for (int64_t i = 0; i < ndir; ++i) {
      double a = d[3 * i], b = d[3 * i + 1], e = d[3 * i + 2];
      double nr = std::sqrt(a * a + b * b + e * e);
      if (!(std::isfinite(nr) && std::fabs(nr - 1.0) < 1e-8))
        return fail(c, BEMGPU_EINVAL, "direction must be a finite unit vector with three components");
    }
  }
  if (ndir == 0) return BEMGPU_OK;
  Buf dd, dout, dw;
  TRY(upload(c, d, &dd));
  TRY(alloc(c, (size_t)ndir * 16, &dout));
  WaveInst w{};
  w.panels = s->mesh->panels.as<double>();
  w.n = s->mesh->n;
  w.k = s->k;
  w.nrhs = 1;
  w.ndir = (int32_t)ndir;
  w.dirs = dd.as<double>();
  w.p = s->ps.as<double>() + 2 * (size_t)s->mesh->n * rhs;
  w.q = s->qs.as<double>() + 2 * (size_t)s->mesh->n * rhs;
  w.out = dout.as<double>();
  w.ldp = s->mesh->n;
  Buf dpart;
  TRY(alloc(c, far_field_scratch(w.n, (int32_t)ndir, 1), &dpart));
  w.part = dpart.as<double>();
  std::vector<WaveInst> wv{w};
  TRY(upload(c, wv, &dw));
  {
    Prof p(c, "far_field");
    launch_far_field(c->launch(), dw.as<WaveInst>(), 1, 1, (int32_t)ndir, w.n);
  }
  CUDA_TRY(c, cudaGetLastError());
  CUDA_TRY(c, cudaMemcpyAsync(out, dout.p, (size_t)ndir * 16, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return BEMGPU_OK;
}

int bemgpu_target_strength(bemgpu_solution* sol, int32_t rhs, int64_t ndir, const double* dirs,
                           double* out) {
  if (!out) return fail(nullptr, BEMGPU_EINVAL, "null output");
  int64_t nd = dirs ? ndir : 1;
  std::vector<double> f((size_t)std::max<int64_t>(nd, 0) * 2);
  TRY(bemgpu_far_field(sol, rhs, ndir, dirs, f.data()));
  for (int64_t i = 0; i < nd; ++i) out[i] = 20.0 * std::log10(std::hypot(f[2 * i], f[2 * i + 1]));
  return BEMGPU_OK;
}

int bemgpu_traces(const bemgpu_solution* sol, int32_t rhs, double* p, double* q) {
  if (!sol) return fail(nullptr, BEMGPU_EINVAL, "null solution");
  SolutionData* s = sol->d.get();
  bemgpu_ctx* c = s->c;
  std::lock_guard<std::recursive_mutex> lk(c->mu);
  if (rhs < 0 || rhs >= s->nrhs) return fail(c, BEMGPU_EINVAL, "rhs index out of range");
  const size_t n = (size_t)s->mesh->n;
  if (p)
    CUDA_TRY(c, cudaMemcpyAsync(p, s->ps.as<double>() + 2 * n * rhs, n * 16, cudaMemcpyDeviceToHost,
                                c->stream));
  if (q)
    CUDA_TRY(c, cudaMemcpyAsync(q, s->qs.as<double>() + 2 * n * rhs, n * 16, cudaMemcpyDeviceToHost,
                                c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return BEMGPU_OK;
}

// ===================================================================== hierarchical matrices
namespace {

// Compressed M1 / M2 of one rigid/soft problem on one mesh.
struct HmData {
  HmPlan plan;
  std::shared_ptr<MeshData::HmPlanCache> pc;  // the mesh's plan (perm, iperm on the device)
  Buf leaf_lo, leaf_ptr, leaf_ent, dn, D1, D2, vt_items, lb_items;
  int32_t n_vt = 0, n_lb = 0;
  Buf lr[2], U[2], V[2];
  int32_t n_lr = 0, n_dense = 0, n_leaf = 0;
  int64_t tstride = 0, pstride = 0;
  bool f32 = false;  // complex64 operators, FP32 entries and products (precision mixed)
  // Nyström pressure-release systems: inverses of the element blocks of operator ny_op,
  // applied on the right inside GMRES (the node system's spectrum straddles the imaginary
  // axis, where restarted GMRES stalls without it)
  Buf ny_pinv;
  int ny_op = -1;
  // Nyström rigid systems: restricted additive Schwarz over element neighbourhoods
  // (nystrom.cu), the own-node rows of each neighbourhood inverse in ny_w
  bool ny_ras = false;
  Buf ny_nbptr, ny_nbel, ny_woff, ny_w;
  bemgpu_hmatrix_stats st{};
  size_t bytes() const {
    size_t b = leaf_lo.bytes + leaf_ptr.bytes + leaf_ent.bytes + dn.bytes + D1.bytes +
               D2.bytes + vt_items.bytes + lb_items.bytes;
    for (int o = 0; o < 2; ++o) b += lr[o].bytes + U[o].bytes + V[o].bytes;
    b += ny_pinv.bytes + ny_nbptr.bytes + ny_nbel.bytes + ny_woff.bytes + ny_w.bytes;
    return b;
  }
  size_t scratch_bytes(int32_t nr) const {  // T, P (and Xf) of a product over nr vectors
    return (size_t)nr * ((size_t)tstride * 16 + (size_t)pstride * (f32 ? 8 : 16) +
                         (f32 ? (size_t)plan.n * 8 : 0));
  }
  // s: scratch_bytes(nr) bytes for products over at most nr vectors
  HmOp op(int o, void* s, int32_t nr) const {
    double* T = static_cast<double*>(s);
    HmOp A{};
    A.lr = lr[o].as<HmLR>();
    A.dn = dn.as<HmDense>();
    A.U = U[o].p;
    A.V = V[o].p;
    A.D = (o == 0 ? D1 : D2).p;
    A.f32 = f32 ? 1 : 0;
    A.leaf_lo = leaf_lo.as<int32_t>();
    A.leaf_ptr = leaf_ptr.as<int32_t>();
    A.leaf_ent = leaf_ent.as<int32_t>();
    A.n_lr = n_lr;
    A.n_dense = n_dense;
    A.n_leaf = n_leaf;
    A.vt_items = vt_items.as<HmItem>();
    A.lb_items = lb_items.as<HmItem>();
    A.n_vt = n_vt;
    A.n_lb = n_lb;
    A.T = T;
    A.tstride = tstride;
    A.P = static_cast<char*>(s) + (size_t)nr * tstride * 16;
    A.pstride = pstride;
    A.Xf = f32 ? static_cast<char*>(A.P) + (size_t)nr * pstride * 8 : nullptr;
    A.n = plan.n;
    return A;
  }
};

int check_hm_options(bemgpu_ctx* c, const bemgpu_hmatrix_options& o) {
  if (!(std::isfinite(o.tol) && o.tol > 0 && o.tol < 1))
    return fail(c, BEMGPU_EINVAL, "compression tolerance must lie in (0, 1)");
  if (!(std::isfinite(o.eta) && o.eta > 0))
    return fail(c, BEMGPU_EINVAL, "admissibility eta must be finite and positive");
  if (o.leaf_size < 8 || o.leaf_size > 64)
    return fail(c, BEMGPU_EINVAL, "leaf_size must lie in [8, 64]");
  if (o.restart < 1 || o.restart > 500)
    return fail(c, BEMGPU_EINVAL, "restart must lie in [1, 500]");
  if (!(std::isfinite(o.reltol) && o.reltol >= 0 && std::isfinite(o.abstol) && o.abstol >= 0))
    return fail(c, BEMGPU_EINVAL, "GMRES tolerances must be finite and nonnegative");
  if (o.maxiter < 0) return fail(c, BEMGPU_EINVAL, "maxiter must be a nonnegative integer");
  if (o.neighbours < 0 || o.neighbours > 128)
    return fail(c, BEMGPU_EINVAL, "neighbours must lie in [0, 128]");
  return BEMGPU_OK;
}

// Cluster tree and blocks on the host, cross approximation of both operators, full
// blocks (regular kernel + near kernel into block storage), product lists.

// The `count` elements nearest to every element (distances between the elements'
// centroid nodes, ties by index), the element itself first: a uniform grid over the
// centroids searched in growing shells of cells until the count-th distance is covered.
void ras_neighbourhoods(const std::vector<double>& rec, int64_t ne, int count,
                        std::vector<int32_t>* ptr, std::vector<int32_t>* els) {
  count = (int)std::min<int64_t>(count, ne);
  std::vector<double> cx((size_t)ne * 3);
  double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int64_t e = 0; e < ne; ++e)
    for (int a = 0; a < 3; ++a) {
      const double v = rec[(size_t)e * kNyNodes * kPanelDoubles + a];
      cx[3 * e + a] = v;
      lo[a] = std::min(lo[a], v);
      hi[a] = std::max(hi[a], v);
    }
  const double ext = std::max({hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2], 1e-300});
  const int g = (int)std::max<double>(1.0, std::ceil(std::cbrt((double)ne)));
  const double h = ext / g * (1.0 + 1e-12);
  auto cell = [&](int64_t e, int a) {
    return std::min(g - 1, std::max(0, (int)((cx[3 * e + a] - lo[a]) / h)));
  };
  std::vector<std::vector<int32_t>> grid((size_t)g * g * g);
  for (int64_t e = 0; e < ne; ++e)
    grid[((size_t)cell(e, 0) * g + cell(e, 1)) * g + cell(e, 2)].push_back((int32_t)e);
  ptr->assign(1, 0);
  els->clear();
  els->reserve((size_t)ne * count);
  std::vector<std::pair<double, int32_t>> cand;
  for (int64_t e = 0; e < ne; ++e) {
    const int ci = cell(e, 0), cj = cell(e, 1), ck = cell(e, 2);
    cand.clear();
    for (int R = 0;; ++R) {
      for (int i = ci - R; i <= ci + R; ++i)
        for (int j = cj - R; j <= cj + R; ++j)
          for (int k = ck - R; k <= ck + R; ++k) {
            if (std::max({std::abs(i - ci), std::abs(j - cj), std::abs(k - ck)}) != R) continue;
            if (i < 0 || j < 0 || k < 0 || i >= g || j >= g || k >= g) continue;
            for (int32_t f : grid[((size_t)i * g + j) * g + k]) {
              const double dx = cx[3 * f] - cx[3 * e], dy = cx[3 * f + 1] - cx[3 * e + 1],
                           dz = cx[3 * f + 2] - cx[3 * e + 2];
              cand.emplace_back(dx * dx + dy * dy + dz * dz, f);
            }
          }
      if ((int)cand.size() >= count) {
        std::nth_element(cand.begin(), cand.begin() + (count - 1), cand.end());
        const double covered = (double)R * h;
        if (cand[count - 1].first <= covered * covered || R >= g) break;
      } else if (R >= g) {
        break;
      }
    }
    std::sort(cand.begin(), cand.end());
    for (int q = 0; q < count; ++q) els->push_back(cand[q].second);
    ptr->push_back((int32_t)els->size());
  }
}

int hm_build(bemgpu_ctx* c, MeshData* m, const bemgpu_problem& p, int kind,
             const bemgpu_hmatrix_options& o, HmData* H) {
  const Launch L = c->launch();
  Timer tb(c->stream);
  const int64_t n = m->n;
  std::shared_ptr<MeshData::HmPlanCache>& pc = m->hm_plans[{o.leaf_size, o.eta}];
  if (!pc) {  // cluster tree, partition and near-pair destinations of this mesh
    auto fresh = std::make_shared<MeshData::HmPlanCache>();
    std::vector<double> cent, diam;
    if (m->nystrom) {  // node positions, their element's longest edge
      cent.resize(3 * (size_t)n);
      diam.resize((size_t)n);
      for (int64_t i = 0; i < n; ++i) {
        const double* r = m->panels_h.data() + i * kPanelDoubles;
        for (int a = 0; a < 3; ++a) cent[3 * (size_t)i + a] = r[a];
        diam[(size_t)i] = r[7];
      }
    } else {
      panel_centroids(m->nodes_h.data(), m->tris_h.data(), n, &cent, &diam);
    }
    std::string err;
    if (hm_build_plan(cent.data(), diam.data(), n, o.leaf_size, o.eta, m->eta, &fresh->plan,
                      &err)) {
      m->hm_plans.erase({o.leaf_size, o.eta});
      return fail(c, BEMGPU_EINVAL, err);
    }
    const HmPlan& P = fresh->plan;
    // destination of a pair (original indices) inside its full leaf block: the leaf pairs
    // of the full blocks, looked up per row leaf (blocks of a row leaf sorted by column
    // leaf); -1 when the pair lies in no full block
    const int64_t nl = (int64_t)P.leaf_lo.size() - 1;
    std::vector<int32_t> leaf((size_t)n);
    for (int64_t l = 0; l < nl; ++l)
      for (int32_t t = P.leaf_lo[(size_t)l]; t < P.leaf_lo[(size_t)l + 1]; ++t) leaf[(size_t)t] = (int32_t)l;
    std::vector<std::vector<std::pair<int32_t, int64_t>>> row_blocks((size_t)nl);
    {
      int64_t off = 0;
      for (const HmBlock& B : P.dense) {  // full-block offsets as hm_build lays them out
        row_blocks[(size_t)leaf[(size_t)B.rlo]].push_back({leaf[(size_t)B.clo], off});
        off += (int64_t)B.m * B.n;
      }
    }
    for (auto& v : row_blocks) std::sort(v.begin(), v.end());
    auto pair_dst = [&](int64_t i, int64_t j) -> int64_t {
      const int32_t pi = P.iperm[(size_t)i], pj = P.iperm[(size_t)j];
      const auto& v = row_blocks[(size_t)leaf[(size_t)pi]];
      auto it = std::lower_bound(v.begin(), v.end(),
                                 std::pair<int32_t, int64_t>{leaf[(size_t)pj], INT64_MIN});
      if (it == v.end() || it->first != leaf[(size_t)pj]) return -1;
      const int32_t rlo = P.leaf_lo[(size_t)leaf[(size_t)pi]];
      const int32_t clo = P.leaf_lo[(size_t)leaf[(size_t)pj]];
      const int32_t mrows = P.leaf_lo[(size_t)leaf[(size_t)pi] + 1] - rlo;
      return it->second + (pi - rlo) + (int64_t)(pj - clo) * mrows;
    };
    std::vector<int64_t> dst((size_t)std::max<int64_t>(1, m->n_near), 0);
    if (m->n_near > 0) {
      std::vector<int64_t> rowptr, cols;
      near_pairs(cent, diam, m->eta, &rowptr, &cols);
      if ((int64_t)cols.size() != m->n_near) {
        m->hm_plans.erase({o.leaf_size, o.eta});
        return fail(c, BEMGPU_EINVAL, "internal: near-pair list differs from the mesh's");
      }
      for (int64_t i = 0; i < n; ++i)
        for (int64_t q = rowptr[i]; q < rowptr[i + 1]; ++q) {
          dst[(size_t)q] = pair_dst(i, cols[q]);
          if (dst[(size_t)q] < 0) {
            m->hm_plans.erase({o.leaf_size, o.eta});
            return fail(c, BEMGPU_EINVAL, "internal: near pair outside the full blocks");
          }
        }
    }
    if (m->nystrom) {  // every same-element pair (node i, node 7 (i / 7) + j)
      std::vector<int64_t> nd((size_t)n * kNyNodes);
      for (int64_t i = 0; i < n; ++i)
        for (int j = 0; j < kNyNodes; ++j) {
          nd[(size_t)i * kNyNodes + j] = pair_dst(i, (i / kNyNodes) * kNyNodes + j);
          if (nd[(size_t)i * kNyNodes + j] < 0) {
            m->hm_plans.erase({o.leaf_size, o.eta});
            return fail(c, BEMGPU_EINVAL, "internal: element pair outside the full blocks");
          }
        }
      TRY(upload(c, nd, &fresh->ny_dst));
    }
    TRY(upload(c, P.perm, &fresh->perm));
    TRY(upload(c, P.iperm, &fresh->iperm));
    TRY(upload(c, dst, &fresh->near_dst));
    pc = fresh;
  }
  H->plan = pc->plan;
  H->pc = pc;
  const HmPlan& P = H->plan;
  const double k = p.k;
  H->f32 = p.precision == BEMGPU_MIXED;
  const size_t es = H->f32 ? 8 : 16;  // bytes per stored complex entry
  const void* recs = H->f32 ? m->panelsf.p : m->panels.p;
  const double a_re = 0.0, a_im = kind == kAsmBM ? 1.0 / k : 0.0;  // alpha = i / k
  // admissible blocks: rank capacity below the size where a full block is cheaper
  std::vector<HmLR> lr(P.lowrank.size());
  std::vector<int32_t> normal, large;  // 256- or 512-thread CTAs
  int64_t uo = 0, vo = 0, to = 0;
  int32_t max_m = 1, max_m_large = 1;
  for (size_t b = 0; b < lr.size(); ++b) {
    const HmBlock& B = P.lowrank[b];
    const int64_t cap = (int64_t)B.m * B.n / ((int64_t)B.m + B.n);
    const int32_t kmax = (int32_t)std::max<int64_t>(1, std::min<int64_t>(kHmMaxRank, cap));
    lr[b] = HmLR{B.rlo, B.m, B.clo, B.n, uo, vo, to, kmax, 0, 0, 0, 0};
    uo += (int64_t)B.m * kmax;
    vo += (int64_t)B.n * kmax;
    to += kmax;
    if (B.m + B.n >= kHmAcaLarge) {
      large.push_back((int32_t)b);
      max_m_large = std::max(max_m_large, B.m);
    } else {
      normal.push_back((int32_t)b);
      max_m = std::max(max_m, B.m);
    }
  }
  Buf d_normal, d_large;
  TRY(upload(c, normal, &d_normal));
  TRY(upload(c, large, &d_large));
  std::vector<HmLR> lrh[2];
  for (int op = 0; op < 2; ++op) {
    TRY(upload(c, lr, &H->lr[op]));
    TRY(alloc(c, (size_t)std::max<int64_t>(1, uo) * es, &H->U[op]));
    TRY(alloc(c, (size_t)std::max<int64_t>(1, vo) * es, &H->V[op]));
    {
      Prof pr(c, "hm_aca");
      launch_hm_aca(L, H->lr[op].as<HmLR>(), d_normal.as<int32_t>(), (int32_t)normal.size(),
                    max_m, d_large.as<int32_t>(), (int32_t)large.size(), max_m_large,
                    H->U[op].p, H->V[op].p, recs, H->f32, H->pc->perm.as<int32_t>(), kind, op, k,
                    a_re, a_im, o.tol);
    }
    CUDA_TRY(c, cudaGetLastError());
  }
  for (int op = 0; op < 2; ++op) TRY(download(c, H->lr[op], &lrh[op], lr.size()));
  // blocks whose approximation did not converge within the cap are stored in full
  std::vector<HmDense> dn;
  std::vector<HmBlock> dblk = P.dense, lblk;
  std::vector<HmLR> keep[2];
  int64_t off = 0;
  int64_t poff = 0;
  for (const HmBlock& B : P.dense) {
    dn.push_back(HmDense{B.rlo, B.m, B.clo, B.n, off, poff});
    off += (int64_t)B.m * B.n;
    poff += B.m;
  }
  int64_t densified = 0, lr_entries = 0;
  int32_t max_rank = 0;
  for (size_t b = 0; b < lr.size(); ++b) {
    if (!lrh[0][b].conv || !lrh[1][b].conv) {
      const HmBlock& B = P.lowrank[b];
      dn.push_back(HmDense{B.rlo, B.m, B.clo, B.n, off, poff});
      dblk.push_back(B);
      off += (int64_t)B.m * B.n;
      poff += B.m;
      ++densified;
      continue;
    }
    lblk.push_back(P.lowrank[b]);
    for (int op = 0; op < 2; ++op) {
      keep[op].push_back(lrh[op][b]);
      keep[op].back().poff = poff;
      lr_entries += (int64_t)lrh[op][b].rank * (lrh[op][b].m + lrh[op][b].n);
      max_rank = std::max(max_rank, lrh[op][b].rank);
    }
    poff += P.lowrank[b].m;
  }
  H->pstride = std::max<int64_t>(1, poff);
  // work items of the compressed products and the coefficient offsets of the kept blocks
  std::vector<HmItem> vti, lbi;
  int64_t tof = 0;
  for (size_t b = 0; b < lblk.size(); ++b) {
    const int32_t m_ = lblk[b].m, n_ = lblk[b].n;
    const int32_t nvc = (n_ + kHmColChunk - 1) / kHmColChunk;
    for (int op = 0; op < 2; ++op) {
      keep[op][b].toff = tof;
      keep[op][b].nvc = nvc;
    }
    tof += (int64_t)nvc * keep[0][b].kmax;
    for (int32_t c = 0; c < nvc; ++c)
      vti.push_back(HmItem{(int32_t)b, c * kHmColChunk, std::min(kHmColChunk, n_ - c * kHmColChunk), c});
    for (int32_t r0 = 0; r0 < m_; r0 += kHmRowChunk)
      lbi.push_back(HmItem{(int32_t)b, r0, std::min(kHmRowChunk, m_ - r0), 0});
  }
  H->tstride = std::max<int64_t>(1, tof);
  H->n_vt = (int32_t)vti.size();
  H->n_lb = (int32_t)lbi.size();
  TRY(upload(c, vti, &H->vt_items));
  TRY(upload(c, lbi, &H->lb_items));
  H->n_dense = (int32_t)dn.size();
  H->n_lr = (int32_t)lblk.size();
  TRY(upload(c, dn, &H->dn));
  TRY(alloc(c, (size_t)std::max<int64_t>(1, off) * es, &H->D1));
  TRY(alloc(c, (size_t)std::max<int64_t>(1, off) * es, &H->D2));
  // U and V were allocated at the rank cap: move the ranks reached into tight pools
  for (int op = 0; op < 2; ++op) {
    std::vector<HmCopy> cu, cv;
    int64_t tu = 0, tv = 0;
    const int64_t w = (int64_t)es / 8;  // 8-byte words per complex entry
    for (HmLR& B : keep[op]) {
      const int64_t mu = (int64_t)B.m * B.rank, nv = (int64_t)B.n * B.rank;
      if (mu > 0) cu.push_back(HmCopy{B.uoff * w, tu * w, mu * w});
      if (nv > 0) cv.push_back(HmCopy{B.voff * w, tv * w, nv * w});
      B.uoff = tu;
      B.voff = tv;
      tu += mu;
      tv += nv;
    }
    Buf ut, vt, dcu, dcv;
    TRY(alloc(c, (size_t)std::max<int64_t>(1, tu) * es, &ut));
    TRY(alloc(c, (size_t)std::max<int64_t>(1, tv) * es, &vt));
    TRY(upload(c, cu, &dcu));
    TRY(upload(c, cv, &dcv));
    launch_hm_compact(L, dcu.as<HmCopy>(), (int32_t)cu.size(), H->U[op].p, ut.p);
    launch_hm_compact(L, dcv.as<HmCopy>(), (int32_t)cv.size(), H->V[op].p, vt.p);
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));  // the capacity pools are released next
    H->U[op] = std::move(ut);
    H->V[op] = std::move(vt);
  }
  for (int op = 0; op < 2; ++op) TRY(upload(c, keep[op], &H->lr[op]));
  {
    Prof pr(c, "hm_dense");
    launch_hm_dense(L, H->dn.as<HmDense>(), H->n_dense, H->D1.p, H->D2.p, recs, H->f32,
                    H->pc->perm.as<int32_t>(), kind, k, a_re, a_im);
  }
  // near pairs (the mesh's list, same order) into their full leaf blocks
  if (m->n_near > 0) {
    Buf d_ai, d_corr;
    if (H->f32)  // complex64 full blocks: the near values' rounding errors are not kept
      TRY(alloc(c, (size_t)m->n_near * 16, &d_corr));
    AsmInst I{};
    I.panels = m->panels.as<double>();
    I.panelsf = m->panelsf.as<float>();
    I.verts = m->verts.as<double>();
    I.near_i = m->near_i.as<int32_t>();
    I.near_j = m->near_j.as<int32_t>();
    I.near_lap = m->near_lap.as<double>();
    I.n = n;
    I.n_near = m->n_near;
    I.lda = n;
    I.k_e = I.k_i = k;
    I.g = 1.0;
    I.a_re = a_re;
    I.a_im = a_im;
    I.kind = kind;
    I.out1 = H->D1.p;
    I.out2 = H->D2.p;
    I.c64 = H->f32 ? 3 : 0;
    I.dnear = I.dnear2 = H->f32 ? d_corr.as<double>() : nullptr;
    I.near_dst = pc->near_dst.as<int64_t>();
    std::vector<AsmInst> ai{I};
    TRY(upload(c, ai, &d_ai));
    {
      Prof pr(c, "near");
      launch_assemble_near(L, d_ai.as<AsmInst>(), 1, m->n_near, kind, H->f32);
    }
    CUDA_TRY(c, cudaGetLastError());
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));  // d_ai / d_corr are released below
  }
  std::vector<int32_t> ptr, ent;
  hm_leaf_lists(P, dblk, lblk, &ptr, &ent);
  H->n_leaf = (int32_t)ptr.size() - 1;
  TRY(upload(c, P.leaf_lo, &H->leaf_lo));
  TRY(upload(c, ptr, &H->leaf_ptr));
  TRY(upload(c, ent, &H->leaf_ent));
  CUDA_TRY(c, cudaGetLastError());
  if (m->nystrom) {
    // Nyström node operators: diagonal, combined defect of the interpolants through the
    // compressed products, element corrections inside the full blocks
    const int32_t nb = kNyBasis;
    Buf trace, up, fp, y, y2, scr, status;
    TRY(alloc(c, (size_t)n * 2 * nb * 16, &trace));
    TRY(alloc(c, (size_t)n * nb * 16, &up));
    TRY(alloc(c, (size_t)n * nb * 16, &fp));
    TRY(alloc(c, (size_t)n * nb * 16, &y));
    TRY(alloc(c, (size_t)n * nb * 16, &y2));
    TRY(alloc(c, H->scratch_bytes(nb), &scr));
    TRY(alloc(c, (size_t)std::max<int64_t>(1, n / kNyNodes) * 4, &status));
    CUDA_TRY(c, cudaMemsetAsync(status.p, 0, status.bytes, c->stream));
    NyInst T{};
    T.nodes = m->panels.as<double>();
    T.n = n;
    T.k = k;
    nystrom_directions(T.dirs);
    T.trace = trace.as<double>();
    NyPoints none{};
    NyHm Y{};
    Y.trace = trace.as<double>();
    Y.Y = y2.as<double>();
    Y.iperm = pc->iperm.as<int32_t>();
    Y.dst = pc->ny_dst.as<int64_t>();
    Y.D1 = H->D1.p;
    Y.D2 = H->D2.p;
    Y.n = n;
    Y.a_re = a_re;
    Y.a_im = a_im;
    Y.f32 = H->f32 ? 1 : 0;
    Y.status = status.as<int32_t>();
    {
      Prof pr(c, "hm_dense");
      launch_nystrom_pressure(L, T, none);  // the interpolant traces only
      launch_nystrom_hm_diag(L, Y);
      launch_hm_permute(L, trace.as<double>(), n, up.as<double>(), n, pc->perm.as<int32_t>(), n,
                        nb);
      launch_hm_permute(L, trace.as<double>() + 2 * (size_t)n * nb, n, fp.as<double>(), n,
                        pc->perm.as<int32_t>(), n, nb);
      launch_hm_matvec(L, H->op(0, scr.p, nb), up.as<double>(), n, y.as<double>(), n, nullptr,
                       0, 0.0, 1.0, nb, nullptr, 0);
      launch_hm_matvec(L, H->op(1, scr.p, nb), fp.as<double>(), n, y2.as<double>(), n,
                       y.as<double>(), n, 1.0, 1.0, nb, nullptr, 0);
      launch_nystrom_hm_correct(L, Y);
    }
    CUDA_TRY(c, cudaGetLastError());
    std::vector<int32_t> st;
    TRY(download(c, status, &st, (size_t)std::max<int64_t>(1, n / kNyNodes)));
    for (int32_t v : st)
      if (v) return fail(c, BEMGPU_EINVAL, "density-interpolation fit is rank-deficient");
    if (p.boundary == BEMGPU_PRESSURE_RELEASE) {  // the system operator is M2
      TRY(alloc(c, (size_t)n * kNyNodes * 16, &H->ny_pinv));
      CUDA_TRY(c, cudaMemsetAsync(status.p, 0, status.bytes, c->stream));
      NyPrec B{};
      B.Pinv = H->ny_pinv.as<double>();
      B.iperm = pc->iperm.as<int32_t>();
      B.dst = pc->ny_dst.as<int64_t>();
      B.D = H->D2.p;
      B.n = n;
      B.f32 = H->f32 ? 1 : 0;
      B.status = status.as<int32_t>();
      launch_nystrom_prec_build(L, B);
      CUDA_TRY(c, cudaGetLastError());
      TRY(download(c, status, &st, (size_t)std::max<int64_t>(1, n / kNyNodes)));
      for (int32_t v : st)
        if (v) return fail(c, BEMGPU_ESINGULAR, "singular element block of the node system");
      H->ny_op = 1;
    } else if (p.boundary == BEMGPU_RIGID && o.neighbours > 0) {  // system M1: Schwarz
      const int64_t ne = n / kNyNodes;
      std::vector<int32_t> nptr, nel;
      ras_neighbourhoods(m->panels_h, ne, o.neighbours, &nptr, &nel);
      std::vector<int64_t> woff((size_t)ne + 1, 0);
      int32_t max_len = 0;
      for (int64_t e = 0; e < ne; ++e) {
        const int32_t len = kNyNodes * (nptr[e + 1] - nptr[e]);
        max_len = std::max(max_len, len);
        woff[e + 1] = woff[e] + (int64_t)kNyNodes * len;
      }
      TRY(upload(c, nptr, &H->ny_nbptr));
      TRY(upload(c, nel, &H->ny_nbel));
      TRY(upload(c, woff, &H->ny_woff));
      TRY(alloc(c, (size_t)std::max<int64_t>(1, woff[ne]) * 8, &H->ny_w));
      // one local system per CTA, about one wave of them at a time (the working set of
      // the eliminations then stays in L2)
      const int64_t slots = std::min<int64_t>(ne, 2 * (int64_t)device_sm_count());
      const int64_t stride = 2 * (int64_t)max_len * (max_len + kNyNodes);  // floats
      Buf work;
      TRY(alloc(c, (size_t)slots * stride * 4, &work));
      CUDA_TRY(c, cudaMemsetAsync(status.p, 0, status.bytes, c->stream));
      NyPrec B{};
      B.iperm = pc->iperm.as<int32_t>();
      B.dst = pc->ny_dst.as<int64_t>();
      B.D = H->D1.p;
      B.n = n;
      B.f32 = H->f32 ? 1 : 0;
      B.status = status.as<int32_t>();
      B.ras = 1;
      B.W = H->ny_w.as<float>();
      B.woff = H->ny_woff.as<int64_t>();
      B.nb_ptr = H->ny_nbptr.as<int32_t>();
      B.nb_el = H->ny_nbel.as<int32_t>();
      B.recf = m->panelsf.as<float>();
      B.op = 0;
      B.k = (float)k;
      B.a_re = (float)a_re;
      B.a_im = (float)a_im;
      B.work = work.as<float>();
      B.work_stride = stride;
      {
        Prof pr(c, "hm_precond");
        for (int64_t e0 = 0; e0 < ne; e0 += slots)
          launch_nystrom_ras_build(L, B, e0, std::min(slots, ne - e0), max_len);
      }
      CUDA_TRY(c, cudaGetLastError());
      TRY(download(c, status, &st, (size_t)std::max<int64_t>(1, ne)));
      for (int32_t v : st)
        if (v) return fail(c, BEMGPU_ESINGULAR, "singular neighbourhood of the node system");
      H->ny_op = 0;
      H->ny_ras = true;
    }
  }
  bemgpu_hmatrix_stats& S = H->st;
  std::memset(&S, 0, sizeof S);
  S.lowrank_blocks = H->n_lr;
  S.dense_blocks = H->n_dense;
  S.densified_blocks = densified;
  S.lowrank_entries = lr_entries;
  S.dense_entries = 2 * off;
  S.max_rank = max_rank;
  S.depth = P.depth;
  S.leaves = H->n_leaf;
  S.compression = (double)(lr_entries + 2 * off) / (2.0 * (double)n * (double)n);
  S.build_ms = tb.stop();
  return BEMGPU_OK;
}

// GMRES on A x = b for nr right-hand sides (permuted order, n x nr each), grouped so
// that the Krylov bases fit the context budget.  x receives the solutions; hist, iters,
// conv, resid receive per right-hand side the residual estimates (maxiter per rhs), the
// Arnoldi steps, the convergence flag and |b - A x| / |b|.
int hm_gmres(bemgpu_ctx* c, const HmData& H, int op, const double* b, double* x, int64_t n,
             int32_t nr, const bemgpu_hmatrix_options& o, std::vector<double>* hist,
             std::vector<int32_t>* iters, std::vector<int32_t>* conv, std::vector<double>* resid,
             std::vector<double>* absres) {
  const Launch L = c->launch();
  const int32_t R = o.restart, mi = std::max(1, o.maxiter);
  const int32_t chunks = (int32_t)((n + kGmChunk - 1) / kGmChunk);
  // bytes per right-hand side: Krylov basis, x / w vectors, Hessenberg matrix, partial
  // dots, history, the products' scratch, rotations, and the preconditioned solve's
  // P^-1 product (n complex) when the element-block preconditioner applies
  const bool precond = op == H.ny_op && (H.ny_pinv.p || H.ny_ras);
  const size_t per = ((size_t)(R + 1) * n + 2 * (size_t)n) * 16 + (size_t)(R + 1) * R * 16 +
                     (size_t)chunks * (R + 1) * 16 + (size_t)mi * 8 + H.scratch_bytes(1) +
                     (size_t)(4 * R + 8) * 16 + (precond ? (size_t)n * 16 : 0);
  const uint64_t used = total_live(c), budget = root_of(c)->budget;
  const uint64_t avail = budget > used ? budget - used : 0;
  const int32_t G = (int32_t)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)nr, avail / 2 / per));
  hist->assign((size_t)nr * mi, 0.0);
  iters->assign((size_t)nr, 0);
  conv->assign((size_t)nr, 0);
  resid->assign((size_t)nr, 0.0);
  absres->assign((size_t)nr, 0.0);
  for (int32_t r0 = 0; r0 < nr; r0 += G) {
    const int32_t g = std::min(G, nr - r0);
    Buf st, Vb, Hh, cs, sn, gg, hc, part, hb, w, T, nact;
    TRY(alloc(c, sizeof(GmState) * g, &st));
    TRY(alloc(c, (size_t)g * (R + 1) * n * 16, &Vb));
    TRY(alloc(c, (size_t)g * (R + 1) * R * 16, &Hh));
    TRY(alloc(c, (size_t)g * R * 8, &cs));
    TRY(alloc(c, (size_t)g * R * 16, &sn));
    TRY(alloc(c, (size_t)g * (R + 1) * 16, &gg));
    TRY(alloc(c, (size_t)g * (R + 1) * 16, &hc));
    TRY(alloc(c, (size_t)g * chunks * (R + 1) * 16, &part));
    TRY(alloc(c, (size_t)g * mi * 8, &hb));
    TRY(alloc(c, (size_t)g * n * 16, &w));
    TRY(alloc(c, H.scratch_bytes(g), &T));
    TRY(alloc(c, sizeof(int32_t) * (size_t)(3 + g), &nact));  // count, step, one per CTA
    CUDA_TRY(c, cudaMemsetAsync(st.p, 0, st.bytes, c->stream));
    CUDA_TRY(c, cudaMemsetAsync(Hh.p, 0, Hh.bytes, c->stream));
    CUDA_TRY(c, cudaMemsetAsync(gg.p, 0, gg.bytes, c->stream));
    CUDA_TRY(c, cudaMemsetAsync(hb.p, 0, hb.bytes, c->stream));
    double* xg = x + 2 * (size_t)r0 * n;
    const double* bg = b + 2 * (size_t)r0 * n;
    // right preconditioning (Nyström pressure-release systems): GMRES runs on A P^-1 with
    // the iterate y in W.x; every product takes P^-1 first, and x = P^-1 y at the end
    const bool prec = op == H.ny_op && (H.ny_pinv.p || H.ny_ras);
    NyPrec Pc{};
    Buf pt;
    if (prec) {
      TRY(alloc(c, (size_t)g * n * 16, &pt));
      Pc.Pinv = H.ny_pinv.as<double>();
      Pc.iperm = H.pc->iperm.as<int32_t>();
      Pc.n = n;
      if (H.ny_ras) {
        Pc.ras = 1;
        Pc.W = H.ny_w.as<float>();
        Pc.woff = H.ny_woff.as<int64_t>();
        Pc.nb_ptr = H.ny_nbptr.as<int32_t>();
        Pc.nb_el = H.ny_nbel.as<int32_t>();
      }
    }
    CUDA_TRY(c, cudaMemsetAsync(xg, 0, (size_t)g * n * 16, c->stream));
    CUDA_TRY(c, cudaMemcpyAsync(w.p, bg, (size_t)g * n * 16, cudaMemcpyDeviceToDevice, c->stream));
    GmWork W{};
    W.st = st.as<GmState>();
    W.Vb = Vb.as<double>();
    W.H = Hh.as<double>();
    W.cs = cs.as<double>();
    W.sn = sn.as<double>();
    W.g = gg.as<double>();
    W.hc = hc.as<double>();
    W.part = part.as<double>();
    W.hist = hb.as<double>();
    W.x = xg;
    W.b = bg;
    W.w = w.as<double>();
    W.n = n;
    W.nr = g;
    W.restart = R;
    W.maxiter = mi;
    W.chunks = chunks;
    W.nact = nact.as<int32_t>();
    W.jcur = nact.as<int32_t>() + 2 + g;
    const HmOp A = H.op(op, T.p, g);
    auto active = [&](int32_t* out) -> int {
      CUDA_TRY(c, cudaMemcpyAsync(out, W.nact, sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream));
      CUDA_TRY(c, cudaStreamSynchronize(c->stream));
      return BEMGPU_OK;
    };
    {
      Prof pr(c, "gmres");
      if (o.maxiter == 0) W.maxiter = 0;  // the start step marks every rhs done
      launch_gm_start(L, W, o.reltol, o.abstol, 1);
      W.maxiter = mi;
    }
    int32_t na = 0;
    TRY(active(&na));
    if (o.maxiter == 0) na = 0;
    // one Arnoldi step with the step index on the device, so that a CUDA graph of kSteps
    // steps captured once replays any kSteps consecutive steps of any cycle
    constexpr int32_t kSteps = 4;
    auto step = [&]() {
      if (prec) {
        launch_nystrom_prec_apply(L, Pc, W.Vb, (int64_t)(R + 1) * n, W.jcur, n,
                                  pt.as<double>(), n, g);
        launch_hm_matvec(L, A, pt.as<double>(), n, W.w, n, nullptr, 0, 0.0, 1.0, g, W.st, 1);
      } else {
        launch_hm_matvec(L, A, W.Vb, (int64_t)(R + 1) * n, W.w, n, nullptr, 0, 0.0, 1.0, g,
                         W.st, 1, W.jcur, n);
      }
      launch_gm_arnoldi(L, W, -1);
      launch_gm_rotate(L, W, -1);
    };
    cudaGraphExec_t steps = nullptr;
    long long graph_launches = 0;
    if (R >= kSteps) {
      cudaGraph_t graph = nullptr;
      const long long before = launch_total();
      if (cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
        for (int32_t q = 0; q < kSteps; ++q) step();
        if (cudaStreamEndCapture(c->stream, &graph) == cudaSuccess && graph) {
          if (cudaGraphInstantiate(&steps, graph, 0) != cudaSuccess) steps = nullptr;
          cudaGraphDestroy(graph);
        }
      }
      cudaGetLastError();
      graph_launches = launch_total() - before;
      count_launch(-(int)graph_launches);  // captured, not run
    }
    struct GraphGuard {
      cudaGraphExec_t& e;
      ~GraphGuard() {
        if (e) cudaGraphExecDestroy(e);
      }
    } guard{steps};
    while (na > 0) {
      {
        Prof pr(c, "gmres");
        for (int32_t j = 0; j < R;) {
          if (steps && j + kSteps <= R) {
            CUDA_TRY(c, cudaGraphLaunch(steps, c->stream));
            count_launch((int)graph_launches);
            j += kSteps;
          } else {
            step();
            ++j;
          }
          if (j % kSteps == 0 && j < R) {
            TRY(active(&na));
            if (na == 0) break;
          }
        }
        launch_gm_update_x(L, W);
        if (prec) launch_nystrom_prec_apply(L, Pc, xg, n, nullptr, 0, pt.as<double>(), n, g);
        launch_hm_matvec(L, A, prec ? pt.as<double>() : xg, n, W.w, n, bg, n, 1.0, -1.0, g,
                         W.st, 2);
        launch_gm_start(L, W, o.reltol, o.abstol, 0);
      }
      CUDA_TRY(c, cudaGetLastError());
      TRY(active(&na));
    }
    // explicit residuals b - A x (x = P^-1 y under the preconditioner, then kept in xg)
    {
      Prof pr(c, "gmres");
      if (prec) {
        launch_nystrom_prec_apply(L, Pc, xg, n, nullptr, 0, pt.as<double>(), n, g);
        CUDA_TRY(c, cudaMemcpyAsync(xg, pt.p, (size_t)g * n * 16, cudaMemcpyDeviceToDevice,
                                    c->stream));
      }
      launch_hm_matvec(L, A, xg, n, W.w, n, bg, n, 1.0, -1.0, g, nullptr, 0);
    }
    std::vector<double> wh;
    TRY(download(c, w, &wh, (size_t)g * n * 2));
    std::vector<GmState> sh;
    TRY(download(c, st, &sh, (size_t)g));
    std::vector<double> hh;
    TRY(download(c, hb, &hh, (size_t)g * mi));
    for (int32_t r = 0; r < g; ++r) {
      double s = 0.0;
      for (int64_t i = 0; i < 2 * n; ++i) s += wh[(size_t)r * 2 * n + i] * wh[(size_t)r * 2 * n + i];
      const GmState& S = sh[(size_t)r];
      (*absres)[(size_t)(r0 + r)] = std::sqrt(s);
      (*resid)[(size_t)(r0 + r)] = S.bnorm > 0 ? std::sqrt(s) / S.bnorm : 0.0;
      (*iters)[(size_t)(r0 + r)] = S.iters;
      (*conv)[(size_t)(r0 + r)] = S.converged;
      std::copy(hh.begin() + (size_t)r * mi, hh.begin() + (size_t)(r + 1) * mi,
                hist->begin() + (size_t)(r0 + r) * mi);
    }
  }
  return BEMGPU_OK;
}

int hm_problem(bemgpu_ctx* c, const bemgpu_mesh* mesh, const bemgpu_problem* problem,
               const bemgpu_hmatrix_options* opt, int* kind) {
  if (!mesh || !problem || !opt) return fail(c, BEMGPU_EINVAL, "null argument");
  TRY(check_problem(c, *problem, kind));
  if (*kind != kAsmBM && *kind != kAsmCBIE)
    return fail(c, BEMGPU_EINVAL,
                "hierarchical compression applies to Rigid and PressureRelease boundaries");
  if (std::fabs(problem->near_eta - mesh->d->eta) > 0)
    return fail(c, BEMGPU_EINVAL, "near_eta differs from the mesh's (upload with that eta)");
  return check_hm_options(c, *opt);
}

}  // namespace

void bemgpu_hmatrix_options_init(bemgpu_hmatrix_options* o) {
  if (!o) return;
  std::memset(o, 0, sizeof *o);
  o->tol = 1e-5;
  o->eta = 3.0;
  o->leaf_size = 64;
  o->restart = 150;
  o->reltol = 1e-4;
  o->abstol = 0.0;
  o->maxiter = 1200;
  // no Schwarz preconditioner unless asked for (the reference's rigid GMRES is
  // unpreconditioned).  It pays on coarse meshes -- with the oracle on the 1280-panel
  // sphere at k a = 1.6, GMRES steps to 1e-6 fall from 630 to 159, 78 and 52 with 32, 48
  // and 64 nearest elements (20 is worse than none: 1649) -- but a one-level Schwarz
  // method degrades as the mesh is refined: with 48 neighbours GMRES(150) stalls at a
  // relative residual of 1.5e-2 on a 2304-panel sphere (oracle, FP64 local inverses)
  // and of 0.95 on the 5120-panel sphere (GPU), where plain GMRES reaches 3e-6
  o->neighbours = 0;
}

int bemgpu_hmatrix_plan(const double* nodes, int64_t n_nodes, const int64_t* triangles,
                        int64_t n_triangles, double near_eta, const bemgpu_hmatrix_options* opt,
                        int64_t counts[4], int32_t* blocks, int64_t cap, int32_t* perm) {
  if (!opt || !counts) return fail(nullptr, BEMGPU_EINVAL, "null argument");
  TRY(check_hm_options(nullptr, *opt));
  if (!(std::isfinite(near_eta) && near_eta > 0))
    return fail(nullptr, BEMGPU_EINVAL, "near_eta must be finite and positive");
  std::string e;
  double res;
  int s = validate_surface(nodes, n_nodes, triangles, n_triangles, &res, &e);
  if (s != BEMGPU_OK) return fail(nullptr, s, e);
  std::vector<double> cent, diam;
  panel_centroids(nodes, triangles, n_triangles, &cent, &diam);
  HmPlan P;
  if (hm_build_plan(cent.data(), diam.data(), n_triangles, opt->leaf_size, opt->eta, near_eta,
                    &P, &e))
    return fail(nullptr, BEMGPU_EINVAL, e);
  counts[0] = (int64_t)P.lowrank.size();
  counts[1] = (int64_t)P.dense.size();
  counts[2] = (int64_t)P.leaf_lo.size() - 1;
  counts[3] = P.depth;
  if (blocks) {
    if (counts[0] + counts[1] > cap) return fail(nullptr, BEMGPU_EINVAL, "capacity too small");
    int32_t* o = blocks;
    for (const HmBlock& B : P.dense) {
      o[0] = 0; o[1] = B.rlo; o[2] = B.m; o[3] = B.clo; o[4] = B.n;
      o += 5;
    }
    for (const HmBlock& B : P.lowrank) {
      o[0] = 1; o[1] = B.rlo; o[2] = B.m; o[3] = B.clo; o[4] = B.n;
      o += 5;
    }
  }
  if (perm) std::copy(P.perm.begin(), P.perm.end(), perm);
  return BEMGPU_OK;
}

int bemgpu_hmatrix_solve(bemgpu_ctx* c, const bemgpu_mesh* mesh, const bemgpu_problem* problem,
                         const bemgpu_hmatrix_options* opt, int32_t nrhs, const double* incidence,
                         bemgpu_solution** solution) {
  if (!c) return fail(nullptr, BEMGPU_EINVAL, "null context");
  if (!incidence || !solution) return fail(c, BEMGPU_EINVAL, "null argument");
  if (nrhs <= 0) return fail(c, BEMGPU_EINVAL, "nrhs must be positive");
  std::lock_guard<std::recursive_mutex> lk(c->mu);
  cudaSetDevice(c->device);
  int kind = 0;
  TRY(hm_problem(c, mesh, problem, opt, &kind));
  const bemgpu_problem& p = *problem;
  // the Nyström discretisation compresses the node operators of the node set
  std::shared_ptr<MeshData> md = mesh->d;
  if (p.discretization == BEMGPU_NYSTROM) TRY(nystrom_mesh(c, mesh->d.get(), &md));
  MeshData* m = md.get();
  const int64_t n = m->n;
  std::vector<double> dirs(3 * (size_t)nrhs);
  for (int32_t r = 0; r < nrhs; ++r) {
    const double be = incidence[2 * r], al = incidence[2 * r + 1];
    if (!(std::isfinite(be) && std::isfinite(al)))
      return fail(c, BEMGPU_EINVAL, "incidence angles must be finite");
    dirs[3 * r] = std::cos(be);
    dirs[3 * r + 1] = std::sin(be) * std::cos(al);
    dirs[3 * r + 2] = std::sin(be) * std::sin(al);
  }
  Timer ttot(c->stream);
  HmData H;
  TRY(hm_build(c, m, p, kind, *opt, &H));
  const Launch L = c->launch();
  Timer tsol(c->stream);
  auto sd = std::make_shared<SolutionData>();
  sd->c = c;
  sd->mesh = md;
  if (m->nystrom) sd->base_mesh = mesh->d;
  sd->boundary = p.boundary;
  sd->k = p.k;
  sd->nrhs = nrhs;
  sd->dirs = dirs;
  Buf d_dirs, pinc, qinc, tp, bb, xp, xs, T, d_wi, d_ti;
  TRY(upload(c, dirs, &d_dirs));
  TRY(alloc(c, (size_t)n * nrhs * 16, &pinc));
  TRY(alloc(c, (size_t)n * nrhs * 16, &qinc));
  TRY(alloc(c, (size_t)n * nrhs * 16, &tp));
  TRY(alloc(c, (size_t)n * nrhs * 16, &bb));
  TRY(alloc(c, (size_t)n * nrhs * 16, &xp));
  TRY(alloc(c, (size_t)n * nrhs * 16, &xs));
  TRY(alloc(c, H.scratch_bytes(nrhs), &T));
  TRY(alloc(c, (size_t)n * nrhs * 16, &sd->ps));
  TRY(alloc(c, (size_t)n * nrhs * 16, &sd->qs));
  WaveInst wv{};
  wv.panels = m->panels.as<double>();
  wv.n = n;
  wv.k = p.k;
  wv.nrhs = nrhs;
  wv.dirs = d_dirs.as<double>();
  wv.p = pinc.as<double>();
  wv.q = qinc.as<double>();
  wv.ldp = n;
  std::vector<WaveInst> wi{wv};
  TRY(upload(c, wi, &d_wi));
  {
    Prof pr(c, "incident");
    launch_incident(L, d_wi.as<WaveInst>(), 1, n, nrhs);
  }
  // rigid: A = M1, b = M2 q_inc; soft: A = M2, b = M1 p_inc (full.jl:98-128, 144-152)
  const bool rigid = p.boundary == BEMGPU_RIGID;
  const int sys = rigid ? 0 : 1;
  launch_hm_permute(L, (rigid ? qinc : pinc).as<double>(), n, tp.as<double>(), n,
                    H.pc->perm.as<int32_t>(), n, nrhs);
  {
    Prof pr(c, "hm_matvec");
    launch_hm_matvec(L, H.op(1 - sys, T.p, nrhs), tp.as<double>(), n, bb.as<double>(), n,
                     nullptr, 0, 0.0, 1.0, nrhs, nullptr, 0);
  }
  CUDA_TRY(c, cudaGetLastError());
  std::vector<double> resid, absres;
  std::vector<int32_t> conv;
  TRY(hm_gmres(c, H, sys, bb.as<double>(), xp.as<double>(), n, nrhs, *opt, &sd->gm_hist,
               &sd->gm_iters, &conv, &resid, &absres));
  sd->gm_stride = std::max(1, opt->maxiter);
  launch_hm_permute(L, xp.as<double>(), n, xs.as<double>(), n, H.pc->iperm.as<int32_t>(), n, nrhs);
  TraceInst tr{};
  tr.x = xs.as<double>();
  tr.ldx = n;
  tr.pinc = pinc.as<double>();
  tr.qinc = qinc.as<double>();
  tr.n = n;
  tr.ps = sd->ps.as<double>();
  tr.qs = sd->qs.as<double>();
  tr.nrhs = nrhs;
  tr.kind = rigid ? 0 : 1;
  std::vector<TraceInst> ti{tr};
  TRY(upload(c, ti, &d_ti));
  launch_traces(L, d_ti.as<TraceInst>(), 1, n, nrhs);
  CUDA_TRY(c, cudaGetLastError());
  const double sol_ms = tsol.stop();
  TRY(check_device_error(c));
  bemgpu_hmatrix_stats& S = sd->hm;
  S = H.st;
  S.gmres_converged = 1;
  for (int32_t r = 0; r < nrhs; ++r) {
    S.gmres_iterations = std::max(S.gmres_iterations, sd->gm_iters[(size_t)r]);
    S.gmres_converged &= conv[(size_t)r];
  }
  S.gmres_ms = sol_ms;
  sd->hmatrix = true;
  bemgpu_diagnostics& dg = sd->diag;
  std::memset(&dg, 0, sizeof dg);
  dg.condition_number = dg.scaled_condition_number = NAN;  // no factor: not computed
  dg.condition_limit = p.condition_limit;
  dg.unknown_count = n;
  dg.quadrature_nodes = n;
  dg.near_pairs = m->n_near;
  dg.formulation = kind == kAsmBM ? BEMGPU_BURTON_MILLER : BEMGPU_CBIE;
  dg.precision = p.precision;
  dg.factor_precision = H.f32 ? 0 : 1;
  dg.refinement_iterations = S.gmres_iterations;
  dg.coupling_im = kind == kAsmBM ? 1.0 / p.k : 0.0;
  for (int32_t r = 0; r < nrhs; ++r) {
    dg.absolute_residual = std::max(dg.absolute_residual, absres[(size_t)r]);
    dg.relative_residual = std::max(dg.relative_residual, resid[(size_t)r]);
  }
  dg.scaled_absolute_residual = dg.absolute_residual;
  dg.scaled_relative_residual = dg.relative_residual;
  dg.assemble_ms = H.st.build_ms;
  dg.solve_ms = sol_ms;
  dg.total_ms = ttot.stop();
  dg.device_bytes = (int64_t)H.bytes();
  dg.nrhs = nrhs;
  *solution = new bemgpu_solution{sd};
  return BEMGPU_OK;
}

int bemgpu_hmatrix_stats_get(const bemgpu_solution* sol, bemgpu_hmatrix_stats* stats) {
  if (!sol || !stats) return fail(nullptr, BEMGPU_EINVAL, "null argument");
  if (!sol->d->hmatrix) return fail(sol->d->c, BEMGPU_EINVAL, "not a hierarchical-matrix solution");
  *stats = sol->d->hm;
  return BEMGPU_OK;
}

int bemgpu_gmres_history(const bemgpu_solution* sol, int32_t rhs, double* out, int32_t cap,
                         int32_t* count) {
  if (!sol || !count) return fail(nullptr, BEMGPU_EINVAL, "null argument");
  const SolutionData* s = sol->d.get();
  if (!s->hmatrix) return fail(s->c, BEMGPU_EINVAL, "not a hierarchical-matrix solution");
  if (rhs < 0 || rhs >= s->nrhs) return fail(s->c, BEMGPU_EINVAL, "rhs index out of range");
  const int32_t it = std::min(s->gm_iters[(size_t)rhs], s->gm_stride);
  *count = it;
  if (out)
    for (int32_t i = 0; i < std::min(it, cap); ++i)
      out[i] = s->gm_hist[(size_t)rhs * s->gm_stride + i];
  return BEMGPU_OK;
}

int bemgpu_hmatrix_apply(bemgpu_ctx* c, const bemgpu_mesh* mesh, const bemgpu_problem* problem,
                         const bemgpu_hmatrix_options* opt, int32_t op, int32_t nr,
                         const double* X, double* Y, bemgpu_hmatrix_stats* stats) {
  if (!c) return fail(nullptr, BEMGPU_EINVAL, "null context");
  if (op != 0 && op != 1) return fail(c, BEMGPU_EINVAL, "op must be 0 (M1) or 1 (M2)");
  if (nr < 0 || (nr > 0 && (!X || !Y))) return fail(c, BEMGPU_EINVAL, "invalid vectors");
  std::lock_guard<std::recursive_mutex> lk(c->mu);
  cudaSetDevice(c->device);
  int kind = 0;
  TRY(hm_problem(c, mesh, problem, opt, &kind));
  if (problem->discretization != BEMGPU_COLLOCATION)
    return fail(c, BEMGPU_EINVAL, "hmatrix_apply takes the collocation discretisation");
  MeshData* m = mesh->d.get();
  const int64_t n = m->n;
  HmData H;
  TRY(hm_build(c, m, *problem, kind, *opt, &H));
  if (stats) *stats = H.st;
  if (nr == 0) return BEMGPU_OK;
  const Launch L = c->launch();
  Buf xh, xp, yp, yh, T;
  TRY(alloc(c, (size_t)n * nr * 16, &xh));
  TRY(alloc(c, (size_t)n * nr * 16, &xp));
  TRY(alloc(c, (size_t)n * nr * 16, &yp));
  TRY(alloc(c, (size_t)n * nr * 16, &yh));
  TRY(alloc(c, H.scratch_bytes(nr), &T));
  CUDA_TRY(c, cudaMemcpyAsync(xh.p, X, (size_t)n * nr * 16, cudaMemcpyHostToDevice, c->stream));
  launch_hm_permute(L, xh.as<double>(), n, xp.as<double>(), n, H.pc->perm.as<int32_t>(), n, nr);
  launch_hm_matvec(L, H.op(op, T.p, nr), xp.as<double>(), n, yp.as<double>(), n, nullptr, 0,
                   0.0, 1.0, nr, nullptr, 0);
  launch_hm_permute(L, yp.as<double>(), n, yh.as<double>(), n, H.pc->iperm.as<int32_t>(), n, nr);
  CUDA_TRY(c, cudaMemcpyAsync(Y, yh.p, (size_t)n * nr * 16, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  CUDA_TRY(c, cudaGetLastError());
  return check_device_error(c);
}

int bemgpu_region_solve(bemgpu_ctx* c, int32_t count, const bemgpu_mesh* const* surfaces,
                        const double* density, const double* soundspeed, const int32_t* parents,
                        const bemgpu_problem* problem, int32_t nrhs, const double* incidence,
                        bemgpu_solution** solution) {
  if (!c) return fail(nullptr, BEMGPU_EINVAL, "null context");
  if (!surfaces || !density || !soundspeed || !parents || !problem || !incidence || !solution)
    return fail(c, BEMGPU_EINVAL, "null argument");
  if (count < 1) return fail(c, BEMGPU_EINVAL, "at least one interface is required");
  if (count > kMaxRegions) return fail(c, BEMGPU_EINVAL, "too many interfaces");
  std::lock_guard<std::recursive_mutex> lk(c->mu);
  cudaSetDevice(c->device);
  for (int32_t i = 0; i < count; ++i) {
    if (!surfaces[i]) return fail(c, BEMGPU_EINVAL, "null surface");
    if (!(parents[i] >= 0 && parents[i] <= i))
      return fail(c, BEMGPU_EINVAL, "each parent must be zero or an earlier region index");
    if (!(std::isfinite(density[i]) && density[i] > 0 && std::isfinite(soundspeed[i]) &&
          soundspeed[i] > 0))
      return fail(c, BEMGPU_EINVAL, "fluid contrasts must be finite and positive");
    if (std::fabs(problem->near_eta - surfaces[i]->d->eta) > 0)
      return fail(c, BEMGPU_EINVAL, "near_eta differs from the mesh's (upload with that eta)");
  }
  const bool nystrom = problem->discretization == BEMGPU_NYSTROM;
  bemgpu_problem q = *problem;
  q.boundary = BEMGPU_FLUID;
  q.density_contrast = q.soundspeed_contrast = 1.0;  // per region below
  int kind = 0;
  TRY(check_problem(c, q, &kind));
  // containment must match the parents (regions.jl:302-307): surface i contains surface
  // j exactly when region i + 1 is an ancestor of region j + 1
  auto ancestor = [&](int32_t region, int32_t j) {
    int32_t r = parents[j];
    while (r != 0) {
      if (r == region) return true;
      r = parents[r - 1];
    }
    return false;
  };
  for (int32_t i = 0; i < count; ++i)
    for (int32_t j = 0; j < count; ++j) {
      if (i == j) continue;
      const MeshData* mi = surfaces[i]->d.get();
      const MeshData* mj = surfaces[j]->d.get();
      const bool inside = host_solid_angle(mi, mj->nodes_h.data()) > 2.0 * M_PI;
      if (inside != ancestor(i + 1, j))
        return fail(c, BEMGPU_EINVAL, "interfaces " + std::to_string(i + 1) + " and " +
                                          std::to_string(j + 1) +
                                          " do not match the specified parents");
    }
  std::vector<const MeshData*> parts;
  for (int32_t i = 0; i < count; ++i) parts.push_back(surfaces[i]->d.get());
  std::shared_ptr<MeshData> un;
  TRY(make_union_mesh(c, parts, problem->near_eta, &un));
  // coupling table
  RegionTable tab;
  std::memset(&tab, 0, sizeof tab);
  tab.count = count;
  tab.cbie = kind == kAsmFluidCBIE ? 1 : 0;
  std::vector<double> rho(count + 1, 1.0);
  tab.kr[0] = q.k;
  for (int32_t i = 0; i < count; ++i) {
    tab.kr[i + 1] = q.k / soundspeed[i];
    rho[i + 1] = density[i];
  }
  for (int32_t si = 0; si < count; ++si)
    for (int32_t sj = 0; sj < count; ++sj) {
      RegionCoef& C = tab.c[si * kMaxRegions + sj];
      for (int32_t region : {si + 1, parents[si]}) {
        double sign;
        if (sj + 1 == region)
          sign = 1.0;
        else if (parents[sj] == region)
          sign = -1.0;
        else
          continue;
        C.kidx[C.count] = region;
        C.eq[C.count] = region == si + 1 ? 1 : 0;
        C.sign[C.count] = sign;
        C.rho[C.count] = rho[region];
        ++C.count;
      }
    }
  auto f = std::make_shared<FactorData>();
  f->c = c;
  f->prob = q;
  f->kind = kAsmRegion;
  f->region_cbie = tab.cbie != 0;
  f->mixed = q.precision == BEMGPU_MIXED;
  if (nystrom) {  // the quadrature nodes of the union (7 per panel, surface order)
    f->nystrom = true;
    f->fp32_regular = false;
    f->base_mesh = un;
    TRY(nystrom_mesh(c, un.get(), &f->mesh));
  } else {
    f->mesh = un;
    f->fp32_regular = q.assembly == BEMGPU_ASSEMBLY_SINGLE ||
                      (q.assembly == BEMGPU_ASSEMBLY_DEFAULT && f->mixed);
  }
  const MeshData* um = f->mesh.get();
  std::vector<int8_t> outer((size_t)um->n, 0);
  for (int32_t i = 0; i < count; ++i)
    if (parents[i] == 0)
      for (int64_t p = um->offsets[i]; p < um->offsets[i + 1]; ++p) outer[(size_t)p] = 1;
  std::vector<RegionTable> tv{tab};
  TRY(upload(c, tv, &f->region_tab));
  TRY(upload(c, outer, &f->outer));
  std::vector<FactorData*> fs{f.get()};
  TRY(factor_batch(c, fs, true));
  auto sd = std::make_shared<SolutionData>();
  sd->c = c;
  std::vector<SolutionData*> outs{sd.get()};
  std::vector<int32_t> nr{nrhs};
  std::vector<const double*> inc{incidence};
  TRY(solve_batch(c, fs, nr, inc, outs));
  sd->parents.assign(parents, parents + count);
  sd->region_k.assign(tab.kr, tab.kr + count + 1);
  sd->region_rho = rho;
  *solution = new bemgpu_solution{sd};
  return BEMGPU_OK;
}

int bemgpu_region_traces(const bemgpu_solution* sol, int32_t rhs, double* p, double* v) {
  if (!sol) return fail(nullptr, BEMGPU_EINVAL, "null solution");
  SolutionData* s = sol->d.get();
  bemgpu_ctx* c = s->c;
  std::lock_guard<std::recursive_mutex> lk(c->mu);
  if (!s->region) return fail(c, BEMGPU_EINVAL, "not a coupled-region solution");
  if (rhs < 0 || rhs >= s->nrhs) return fail(c, BEMGPU_EINVAL, "rhs index out of range");
  const size_t n = (size_t)s->mesh->n;
  const double* x = s->xsol.as<double>() + 4 * n * rhs;
  if (p) CUDA_TRY(c, cudaMemcpyAsync(p, x, n * 16, cudaMemcpyDeviceToHost, c->stream));
  if (v) CUDA_TRY(c, cudaMemcpyAsync(v, x + 2 * n, n * 16, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return BEMGPU_OK;
}

int bemgpu_solution_diagnostics(const bemgpu_solution* sol, bemgpu_diagnostics* out) {
  if (!sol || !out) return fail(nullptr, BEMGPU_EINVAL, "null argument");
  *out = sol->d->diag;
  return read_conditioning(sol->d->cond, out);
}

int bemgpu_solution_destroy(bemgpu_solution* sol) {
  if (sol) {
    std::lock_guard<std::recursive_mutex> lk(sol->d->c->mu);
    delete sol;
  }
  return BEMGPU_OK;
}

int bemgpu_pressure(bemgpu_solution* sol, int32_t rhs, int64_t npts, const double* points,
                    int32_t field, double* out) {
  return bemgpu_pressure_region(sol, rhs, npts, points, field, -1, out);
}

namespace {
// Field of a Nyström solution at points (validated by the caller): region and incident
// value per point from the panel kernel on the panel mesh (its exact solid angles), then
// the node sum with the nearest element recovered by the interpolant fit (nystrom.cu).
int nystrom_pressure(bemgpu_ctx* c, SolutionData* s, int32_t rhs, int64_t npts,
                     const double* points, int32_t field, double* out) {
  MeshData* base = s->base_mesh.get();
  if (!base) return fail(c, BEMGPU_EINVAL, "the solution has no panel mesh");
  const Launch L = c->launch();
  const int64_t N = s->mesh->n;
  std::vector<double> pts(points, points + 3 * npts);
  std::vector<double> dir(s->dirs.begin() + 3 * rhs, s->dirs.begin() + 3 * rhs + 3);
  const bool fluid = s->boundary == BEMGPU_FLUID;
  Buf dp, dd, dout, dreg, dst, dtr, dtri;
  TRY(upload(c, pts, &dp));
  TRY(upload(c, dir, &dd));
  TRY(alloc(c, (size_t)npts * 16, &dout));
  TRY(alloc(c, (size_t)npts * 4, &dreg));
  TRY(alloc(c, (size_t)npts * 4, &dst));
  TRY(alloc(c, (size_t)N * 2 * kNyBasis * 16, &dtr));
  if (fluid) TRY(alloc(c, (size_t)N * 2 * kNyBasis * 16, &dtri));
  CUDA_TRY(c, cudaMemsetAsync(dst.p, 0, (size_t)npts * 4, c->stream));
  PressureInst P{};
  P.panels = base->panels.as<double>();
  P.verts = base->verts.as<double>();
  P.n = base->n;
  P.dir = dd.as<double>();
  P.points = dp.as<double>();
  P.npts = npts;
  P.out = dout.as<double>();
  P.region = dreg.as<int32_t>();
  P.k = P.k_int = s->k;
  P.g = 1.0;
  P.eta = base->eta;
  P.field = BEMGPU_FIELD_INCIDENT;
  P.fluid = fluid ? 1 : 0;
  {
    Prof pr(c, "pressure");
    launch_pressure(L, P);
    if (field != BEMGPU_FIELD_INCIDENT) {
      NyInst T{};
      T.nodes = s->mesh->panels.as<double>();
      T.n = N;
      T.k = s->k;
      nystrom_directions(T.dirs);
      T.trace = dtr.as<double>();
      if (fluid) {  // the interior wavenumber's traces (k_int) through a second instance
        NyInst Ti = T;
        Ti.k = s->k / s->h;
        Ti.trace = dtri.as<double>();
        NyPoints none{};
        launch_nystrom_pressure(L, Ti, none);
      }
      NyPoints Q{};
      Q.fluid = fluid ? 1 : 0;
      Q.k_int = s->k / s->h;
      Q.g = fluid ? s->g : 1.0;
      Q.trace_i = fluid ? dtri.as<double>() : nullptr;
      for (int a = 0; a < 3; ++a) Q.dir[a] = dir[(size_t)a];
      for (int a = 0; a < 3 * kNyBasis; ++a) Q.dirs[a] = T.dirs[a];
      Q.nodes = T.nodes;
      Q.n = N;
      Q.k = s->k;
      Q.trace = dtr.as<double>();
      Q.p = s->ps.as<double>() + 2 * (size_t)N * rhs;
      Q.q = s->qs.as<double>() + 2 * (size_t)N * rhs;
      Q.points = dp.as<double>();
      Q.npts = npts;
      Q.region = dreg.as<int32_t>();
      Q.out = dout.as<double>();
      Q.field = field;
      Q.status = dst.as<int32_t>();
      launch_nystrom_pressure(L, T, Q);
    }
  }
  CUDA_TRY(c, cudaGetLastError());
  std::vector<int32_t> reg, st;
  CUDA_TRY(c, cudaMemcpyAsync(out, dout.p, (size_t)npts * 16, cudaMemcpyDeviceToHost, c->stream));
  TRY(download(c, dreg, &reg, (size_t)npts));
  TRY(download(c, dst, &st, (size_t)npts));
  for (int64_t i = 0; i < npts; ++i) {
    if (std::isnan(out[2 * i]) && field != BEMGPU_FIELD_INCIDENT) {
      if (field == BEMGPU_FIELD_INTERIOR)
        return fail(c, BEMGPU_EINVAL, "interior field requested at an exterior point");
      return fail(c, BEMGPU_EINVAL,
                  reg[(size_t)i] == 1 ? "point lies inside the body, where no exterior field exists"
                                      : "field does not exist at this point");
    }
    if (st[(size_t)i])
      return fail(c, BEMGPU_EINVAL, "density-interpolation fit is rank-deficient near a point");
  }
  return BEMGPU_OK;
}
}  // namespace

int bemgpu_pressure_region(bemgpu_solution* sol, int32_t rhs, int64_t npts, const double* points,
                           int32_t field, int32_t region, double* out) {
  if (!sol) return fail(nullptr, BEMGPU_EINVAL, "null solution");
  SolutionData* s = sol->d.get();
  bemgpu_ctx* c = s->c;
  std::lock_guard<std::recursive_mutex> lk(c->mu);
  cudaSetDevice(c->device);
  if (rhs < 0 || rhs >= s->nrhs) return fail(c, BEMGPU_EINVAL, "rhs index out of range");
  if (field < BEMGPU_FIELD_TOTAL || field > BEMGPU_FIELD_INTERIOR)
    return fail(c, BEMGPU_EINVAL, "field must be :total, :scattered, :incident or :interior");
  if (region >= 0 && !s->region)
    return fail(c, BEMGPU_EINVAL, "region selection requires a coupled fluid BEM solution");
  if (s->region && region > (int32_t)s->parents.size())
    return fail(c, BEMGPU_EINVAL, "region must be zero or an interface index");
  if (npts < 0 || (npts > 0 && (!points || !out)))
    return fail(c, BEMGPU_EINVAL, "invalid points");
  if (npts == 0) return BEMGPU_OK;
  for (int64_t i = 0; i < 3 * npts; ++i)
    if (!std::isfinite(points[i])) return fail(c, BEMGPU_EINVAL, "point coordinates must be finite");
  const bool fluid = s->boundary == BEMGPU_FLUID || s->region;
  if (field == BEMGPU_FIELD_INTERIOR && !fluid)
    return fail(c, BEMGPU_EINVAL, "interior field requires a fluid-filled body");
  if (s->mesh->nystrom && s->region)
    return fail(c, BEMGPU_EINVAL,
                "pressure of a Nyström coupled-region solution is not built (the collocation "
                "discretisation's region solutions answer it)");
  if (s->mesh->nystrom) return nystrom_pressure(c, s, rhs, npts, points, field, out);
  std::vector<double> pts(points, points + 3 * npts);
  std::vector<double> dir(s->dirs.begin() + 3 * rhs, s->dirs.begin() + 3 * rhs + 3);
  Buf dp, dd, dout, dreg;
  TRY(upload(c, pts, &dp));
  TRY(upload(c, dir, &dd));
  TRY(alloc(c, (size_t)npts * 16, &dout));
  TRY(alloc(c, (size_t)npts * 4, &dreg));
  PressureInst P{};
  P.panels = s->mesh->panels.as<double>();
  P.verts = s->mesh->verts.as<double>();
  P.n = s->mesh->n;
  P.p = s->ps.as<double>() + 2 * (size_t)s->mesh->n * rhs;
  P.q = s->qs.as<double>() + 2 * (size_t)s->mesh->n * rhs;
  P.dir = dd.as<double>();
  P.points = dp.as<double>();
  P.npts = npts;
  P.out = dout.as<double>();
  P.region = dreg.as<int32_t>();
  P.k = s->k;
  P.k_int = fluid ? s->k / s->h : s->k;
  P.g = fluid ? s->g : 1.0;
  P.eta = s->mesh->eta;
  P.field = field;
  P.fluid = fluid ? 1 : 0;
  if (s->region) {  // coupled regions: the union's surfaces and the solved unknowns
    const int32_t count = (int32_t)s->parents.size();
    P.nsurf = count;
    P.requested = region;
    P.xr = s->xsol.as<double>() + 4 * (size_t)s->mesh->n * rhs;
    for (int32_t i = 0; i <= count; ++i) {
      P.offsets[i] = s->mesh->offsets[(size_t)i];
      P.kr[i] = s->region_k[(size_t)i];
      P.rho[i] = s->region_rho[(size_t)i];
    }
    for (int32_t i = 0; i < count; ++i) P.parents[i] = s->parents[(size_t)i];
  }
  {
    Prof pr(c, "pressure");
    launch_pressure(c->launch(), P);
  }
  CUDA_TRY(c, cudaGetLastError());
  std::vector<int32_t> reg;
  CUDA_TRY(c, cudaMemcpyAsync(out, dout.p, (size_t)npts * 16, cudaMemcpyDeviceToHost, c->stream));
  TRY(download(c, dreg, &reg, (size_t)npts));
  if (s->region) {  // the reference's errors (fields/regions.jl:17-26)
    for (int64_t i = 0; i < npts; ++i)
      switch (-reg[(size_t)i]) {
        case kPrBadRegion:
          return fail(c, BEMGPU_EINVAL, "the point does not belong to the selected region");
        case kPrNeedExterior:
          return fail(c, BEMGPU_EINVAL,
                      "field=:scattered requires the unbounded exterior region");
        case kPrNeedFluid:
          return fail(c, BEMGPU_EINVAL, "field=:interior requires a bounded fluid region");
        default: break;
      }
    return BEMGPU_OK;
  }
  for (int64_t i = 0; i < npts; ++i)
    if (std::isnan(out[2 * i]) && field != BEMGPU_FIELD_INCIDENT) {
      if (field == BEMGPU_FIELD_INTERIOR)
        return fail(c, BEMGPU_EINVAL, "interior field requested at an exterior point");
      return fail(c, BEMGPU_EINVAL,
                  reg[i] == 1 ? "point lies inside the body, where no exterior field exists"
                              : "field does not exist at this point");
    }
  return BEMGPU_OK;
}


void bemgpu_server_options_init(bemgpu_server_options* o) {
  if (!o) return;
  o->max_batch = 64;
  o->queue_limit = 4096;
  o->cache_bytes = 0;
  o->lanes = 2;
  o->reserved = 0;
}

int bemgpu_server_create(bemgpu_ctx* c, const bemgpu_server_options* opts, bemgpu_server** out) {
  if (!c || !out) return fail(c, BEMGPU_EINVAL, "null argument");
  auto* S = new bemgpu_server();
  S->c = c;
  bemgpu_server_options_init(&S->opt);
  if (opts) S->opt = *opts;
  if (S->opt.max_batch <= 0) S->opt.max_batch = 64;
  if (S->opt.queue_limit <= 0) S->opt.queue_limit = 4096;
  if (!S->opt.cache_bytes) S->opt.cache_bytes = c->budget / 4;
  if (S->opt.lanes <= 0) S->opt.lanes = 2;
  if (S->opt.lanes > 8) S->opt.lanes = 8;
  for (int i = 0; i < S->opt.lanes; ++i) {
    bemgpu_ctx* l = nullptr;
    const int st = make_lane(c, &l);
    if (st != BEMGPU_OK) {
      for (bemgpu_ctx* x : S->lanes) destroy_lane(x);
      delete S;
      return st;
    }
    S->lanes.push_back(l);
  }
  S->lane_head.assign((size_t)S->opt.lanes, -1);
  for (int i = 0; i < S->opt.lanes; ++i) S->workers.emplace_back(lane_loop, S, i);
  *out = S;
  return BEMGPU_OK;
}

int bemgpu_server_submit(bemgpu_server* S, const bemgpu_mesh* mesh, const bemgpu_problem* problem,
                         int32_t nfreq, const double* ks, int32_t nangles, const double* incidence,
                         int64_t* ticket) {
  if (!S || !mesh || !problem || !ks || !incidence || !ticket || nfreq <= 0 || nangles <= 0)
    return fail(S ? S->c : nullptr, BEMGPU_EINVAL, "invalid request");
  int kind = 0;
  for (int32_t i = 0; i < nfreq; ++i) {
    bemgpu_problem p = *problem;
    p.k = ks[i];
    TRY(check_problem(S->c, p, &kind));
  }
  if (problem->discretization != BEMGPU_COLLOCATION)  // not part of the factor-cache key
    return fail(S->c, BEMGPU_EINVAL, "the server solves collocation problems");
  for (int32_t i = 0; i < 2 * nangles; ++i)
    if (!std::isfinite(incidence[i])) return fail(S->c, BEMGPU_EINVAL, "incidence angles must be finite");
  auto r = std::make_shared<ServerReq>();
  r->mesh = mesh->d;
  r->prob = *problem;
  r->ks.assign(ks, ks + nfreq);
  r->inc.assign(incidence, incidence + 2 * nangles);
  r->nfreq = nfreq;
  r->nangles = nangles;
  r->untaken = nfreq;
  r->amps.assign(2 * (size_t)nfreq * nangles, 0.0);
  r->t_submit = Clock::now();
  {
    std::lock_guard<std::mutex> lk(S->mu);
    if (S->waiting >= S->opt.queue_limit)
      return fail(S->c, BEMGPU_EBUSY, "request queue full");
    r->id = S->next_id++;
    S->all[r->id] = r;
    const int64_t N = order_of(*r);
    for (int32_t i = 0; i < nfreq; ++i) S->pending.push_back(Pending{r, i, key_of(*r, ks[i]), N});
    S->waiting++;
    S->st.submitted++;
    *ticket = r->id;
  }
  S->cv_work.notify_all();
  return BEMGPU_OK;
}

int bemgpu_server_wait(bemgpu_server* S, int64_t ticket, int32_t timeout_ms, double* amplitudes,
                       double* latency_ms) {
  if (!S) return fail(nullptr, BEMGPU_EINVAL, "null server");
  std::unique_lock<std::mutex> lk(S->mu);
  auto it = S->all.find(ticket);
  if (it == S->all.end()) return fail(S->c, BEMGPU_EINVAL, "unknown ticket");
  auto r = it->second;
  auto pred = [&] { return r->finished; };
  if (timeout_ms < 0)
    S->cv_done.wait(lk, pred);
  else if (!S->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), pred))
    return BEMGPU_ETIMEOUT;
  if (amplitudes) std::copy(r->amps.begin(), r->amps.end(), amplitudes);
  if (latency_ms)
    *latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
  const int st = r->status;
  const std::string msg = r->err.empty() ? "request failed" : "request failed: " + r->err;
  S->all.erase(it);
  if (st != BEMGPU_OK) return fail(S->c, st, msg);
  return BEMGPU_OK;
}

int bemgpu_server_stats_get(bemgpu_server* S, bemgpu_server_stats* out) {
  if (!S || !out) return fail(nullptr, BEMGPU_EINVAL, "null argument");
  std::lock_guard<std::mutex> lk(S->mu);
  *out = S->st;
  out->cached_bytes = S->cached_bytes;
  return BEMGPU_OK;
}

int bemgpu_server_destroy(bemgpu_server* S) {
  if (!S) return BEMGPU_OK;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop = true;
    for (auto& p : S->pending) finish_req(S, *p.req, BEMGPU_EBUSY, "server destroyed");
    S->pending.clear();
  }
  S->cv_work.notify_all();
  for (auto& w : S->workers)
    if (w.joinable()) w.join();
  S->cv_done.notify_all();
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->cache.clear();  // the cached factors' blocks go back to their lanes' pools
    S->cached_bytes = 0;
  }
  for (bemgpu_ctx* l : S->lanes) destroy_lane(l);
  S->lanes.clear();
  delete S;
  return BEMGPU_OK;
}

int bemgpu_dense_solve(bemgpu_ctx* c, int64_t n, const double* A, int32_t nrhs, double* B,
                       int32_t precision, int32_t equilibrate, double refine_tolerance,
                       int32_t refine_maxiter, double condition_guard,
                       bemgpu_diagnostics* diag) {
  if (!c || !A || !B || n <= 0 || nrhs <= 0) return fail(c, BEMGPU_EINVAL, "invalid arguments");
  std::lock_guard<std::recursive_mutex> lk(c->mu);
  cudaSetDevice(c->device);
  for (int64_t i = 0; i < 2 * n * n; ++i)
    if (!std::isfinite(A[i])) return fail(c, BEMGPU_EINVAL, "matrix must be finite");
  for (int64_t i = 0; i < 2 * n * nrhs; ++i)
    if (!std::isfinite(B[i])) return fail(c, BEMGPU_EINVAL, "right-hand side must be finite");
  bemgpu_problem p;
  bemgpu_problem_init(&p);
  p.precision = precision;
  p.equilibrate = equilibrate;
  p.refine_tolerance = refine_tolerance;
  p.refine_maxiter = refine_maxiter;
  p.condition_guard = condition_guard;
  p.boundary = BEMGPU_FLUID;  // no assembly; validation of the solver options only
  p.density_contrast = p.soundspeed_contrast = 1.0;
  int kind = 0;
  TRY(check_problem(c, p, &kind));
  auto f = std::make_shared<FactorData>();
  f->c = c;
  f->prob = p;
  f->kind = kAsmFluidCBIE;
  f->mixed = precision == BEMGPU_MIXED;
  f->n = n;
  f->N = n;
  TRY(alloc(c, (size_t)n * n * 16, &f->A));
  CUDA_TRY(c, cudaMemcpyAsync(f->A.p, A, (size_t)n * n * 16, cudaMemcpyHostToDevice, c->stream));
  std::vector<FactorData*> fs{f.get()};
  TRY(factor_batch(c, fs, false));
  // solve with the generic chain: b given, x out
  SolveInst s;
  s.f = f.get();
  s.R = nrhs;
  TRY(alloc(c, (size_t)n * nrhs * 16, &s.b));
  TRY(alloc(c, (size_t)n * nrhs * 16, &s.x));
  TRY(alloc(c, (size_t)n * nrhs * 16, &s.y));
  TRY(alloc(c, (size_t)n * nrhs * 8, &s.den));
  TRY(alloc(c, (size_t)n * nrhs * 16, &s.work));
  TRY(alloc(c, (size_t)kStats * nrhs * 8, &s.stats));
  TRY(alloc(c, (size_t)std::max<int64_t>(kChunks * (int64_t)nrhs * n * 3, kChunks * n * 2) * 8,
            &s.part));
  TRY(alloc(c, (size_t)nrhs * 4, &s.active));
  TRY(alloc(c, (size_t)nrhs * 4, &s.changed));
  CUDA_TRY(c, cudaMemcpyAsync(s.b.p, B, (size_t)n * nrhs * 16, cudaMemcpyHostToDevice, c->stream));
  s.rs.assign((size_t)nrhs, RhsState{});
  std::vector<SolveInst*> all{&s};
  std::vector<std::vector<int32_t>> mask{std::vector<int32_t>((size_t)nrhs, 1)};
  TRY(correction_pass(c, all, true, mask, 0));
  // refinement loop (same state machine as solve_batch, one instance)
  if (f->mixed) {
    for (int round = 0; round < 64; ++round) {
      bool pending = false;
      for (auto& r : s.rs) pending |= !r.done;
      if (!pending) break;
      std::vector<std::vector<double>> st;
      TRY(residual_pass(c, all, &st));
      std::vector<int32_t> im((size_t)nrhs, 0), cm((size_t)nrhs, 0);
      bool prom = false;
      for (int r = 0; r < nrhs; ++r) {
        RhsState& q = s.rs[r];
        if (q.done) continue;
        double nw, cw;
        normwise(&st[0][(size_t)r * kStats], f->matrix_norm, &nw, &cw);
        q.nw = nw;
        q.cw = cw;
        double metric = std::max(nw, cw);
        if (std::isfinite(metric) && metric <= refine_tolerance) {
          q.done = true;
          continue;
        }
        q.stalls = metric >= q.previous * 0.9 ? q.stalls + 1 : 0;
        int reason = !std::isfinite(metric) ? BEMGPU_REASON_NONFINITE
                     : q.attempts >= refine_maxiter ? BEMGPU_REASON_ITERATION_LIMIT
                     : q.stalls >= 2 ? BEMGPU_REASON_STAGNATION
                                     : BEMGPU_REASON_NONE;
        if (reason != BEMGPU_REASON_NONE) {
          if (!f->single)
            return fail(c, BEMGPU_ENOTCONVERGED,
                        "double-precision fallback failed backward-error acceptance");
          if (!prom) f->reason = reason;
          prom = true;
          q.previous = INFINITY;
          q.attempts = q.stalls = 0;
          im[r] = 1;
        } else {
          cm[r] = 1;
          q.previous = metric;
        }
      }
      if (prom) {
        std::vector<Buf> pp;
        Buf b;
        TRY(alloc(c, (size_t)kChunks * n * 2 * 8, &b));
        pp.push_back(std::move(b));
        TRY(promote(c, fs, pp));
      }
      std::vector<std::vector<int32_t>> m1{im}, m2{cm};
      TRY(correction_pass(c, all, true, m1, 0));
      TRY(correction_pass(c, all, false, m2, 1));
      bool anyc = false;
      for (int32_t v : cm) anyc |= v != 0;
      if (anyc) {
        std::vector<int32_t> ch;
        TRY(download(c, s.changed, &ch, (size_t)nrhs));
        for (int r = 0; r < nrhs; ++r) {
          if (!cm[r]) continue;
          if (!ch[r]) {
            if (!f->single) return fail(c, BEMGPU_ENOTCONVERGED, "double-precision correction stagnated");
            f->reason = BEMGPU_REASON_STAGNATION;
            std::vector<Buf> pp;
            Buf b;
            TRY(alloc(c, (size_t)kChunks * n * 2 * 8, &b));
            pp.push_back(std::move(b));
            TRY(promote(c, fs, pp));
            s.rs[r].previous = INFINITY;
            s.rs[r].attempts = s.rs[r].stalls = 0;
            std::vector<std::vector<int32_t>> m3{std::vector<int32_t>((size_t)nrhs, 0)};
            m3[0][r] = 1;
            TRY(correction_pass(c, all, true, m3, 0));
          } else {
            s.rs[r].corrections++;
            s.rs[r].attempts++;
          }
        }
      }
    }
  }
  std::vector<std::vector<double>> st;
  TRY(residual_pass(c, all, &st));
  CUDA_TRY(c, cudaMemcpyAsync(B, s.x.p, (size_t)n * nrhs * 16, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  TRY(check_device_error(c));
  if (diag) {
    std::memset(diag, 0, sizeof *diag);
    diag->unknown_count = n;
    diag->precision = precision;
    diag->factor_precision = f->single ? 0 : 1;
    diag->refinement_reason = f->reason;
    diag->equilibrate = equilibrate;
    diag->single_reciprocal_condition = f->rcond;
    diag->factor_ms = f->factor_ms;
    diag->nrhs = nrhs;
    diag->info = f->info_h;
    for (int r = 0; r < nrhs; ++r) {
      const double* q = &st[0][(size_t)r * kStats];
      double an = std::sqrt(q[4]), bn = std::sqrt(q[5]);
      double nw, cw;
      normwise(q, f->matrix_norm, &nw, &cw);
      diag->absolute_residual = std::max(diag->absolute_residual, an);
      diag->relative_residual = std::max(diag->relative_residual,
                                         bn == 0.0 ? (an == 0.0 ? 0.0 : INFINITY) : an / bn);
      diag->normwise_backward_error = std::max(diag->normwise_backward_error, nw);
      diag->componentwise_backward_error = std::max(diag->componentwise_backward_error, cw);
      diag->refinement_iterations = std::max(diag->refinement_iterations, s.rs[r].corrections);
    }
  }
  return BEMGPU_OK;
}

int bemgpu_assemble_dense(bemgpu_ctx* c, const bemgpu_mesh* mesh, const bemgpu_problem* problem,
                          double* M1, double* M2) {
  if (!c || !mesh || !problem || !M1) return fail(c, BEMGPU_EINVAL, "null argument");
  std::lock_guard<std::recursive_mutex> lk(c->mu);
  cudaSetDevice(c->device);
  int kind = 0;
  TRY(check_problem(c, *problem, &kind));
  auto f = std::make_shared<FactorData>();
  f->c = c;
  f->prob = *problem;
  f->kind = kind;
  TRY(bind_mesh(c, f.get(), mesh->d));
  std::vector<FactorData*> fs{f.get()};
  TRY(assemble_batch(c, fs));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  TRY(check_device_error(c));
  const bool fluid = kind == kAsmMuller || kind == kAsmFluidCBIE;
  // compact operators expanded to complex128 (value + near correction)
  Buf full, full_rhs;
  const void* sys = f->A.p;
  const void* rhs = f->Mrhs.p;
  if (f->a32) {
    std::vector<VecInst> vi;
    VecInst v;
    std::memset(&v, 0, sizeof v);
    v.A = f->A.p;
    v.n = f->N;
    v.lda = f->N;
    TRY(alloc(c, (size_t)f->N * f->N * 16, &full));
    v.out = full.p;
    set_compact(v, f.get());
    vi.push_back(v);
    if (!fluid) {
      TRY(alloc(c, (size_t)f->n * f->n * 16, &full_rhs));
      VecInst w = v;
      w.A = f->Mrhs.p;
      w.n = w.lda = f->n;
      w.out = full_rhs.p;
      w.nbc = 1;
      w.dnear = f->dnear_rhs.as<double>();
      vi.push_back(w);
    }
    Buf d;
    TRY(to_device(c, vi, &d));
    const Launch L = c->launch();
    launch_expand_a32(L, d.as<VecInst>(), (int)vi.size(), f->N);
    launch_near_add(L, d.as<VecInst>(), (int)vi.size(), v.n_near, 1);
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    sys = full.p;
    if (!fluid) rhs = full_rhs.p;
  }
  // M1 / M2 in the reference's naming: rigid system is M1, pressure release system is M2
  if (fluid) {
    CUDA_TRY(c, cudaMemcpy(M1, sys, (size_t)f->N * f->N * 16, cudaMemcpyDeviceToHost));
  } else {
    const void* m1 = f->rhs_is_m2 ? sys : rhs;
    const void* m2 = f->rhs_is_m2 ? rhs : sys;
    CUDA_TRY(c, cudaMemcpy(M1, m1, (size_t)f->n * f->n * 16, cudaMemcpyDeviceToHost));
    if (M2) CUDA_TRY(c, cudaMemcpy(M2, m2, (size_t)f->n * f->n * 16, cudaMemcpyDeviceToHost));
  }
  return BEMGPU_OK;
}

int bemgpu_profile_enable(bemgpu_ctx* c, int32_t enable) {
  if (!c) return fail(nullptr, BEMGPU_EINVAL, "null context");
  c->prof = enable != 0;
  return BEMGPU_OK;
}

int bemgpu_profile_reset(bemgpu_ctx* c) {
  if (!c) return fail(nullptr, BEMGPU_EINVAL, "null context");
  std::lock_guard<std::recursive_mutex> lk(c->mu);
  cudaStreamSynchronize(c->stream);
  for (auto& kv : c->events)
    for (auto& pr : kv.second) {
      cudaEventDestroy(pr.first);
      cudaEventDestroy(pr.second);
    }
  c->events.clear();
  return BEMGPU_OK;
}

int bemgpu_profile_read(bemgpu_ctx* c, const char* family, int64_t* launches, double* total_ms) {
  if (!c || !family) return fail(c, BEMGPU_EINVAL, "null argument");
  std::lock_guard<std::recursive_mutex> lk(c->mu);
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  int64_t cnt = 0;
  double ms = 0.0;
  auto it = c->events.find(family);
  if (it != c->events.end())
    for (auto& pr : it->second) {
      float m = 0.f;
      cudaEventElapsedTime(&m, pr.first, pr.second);
      ms += m;
      ++cnt;
    }
  if (launches) *launches = cnt;
  if (total_ms) *total_ms = ms;
  return BEMGPU_OK;
}

int bemgpu_ctx_set_graphs(bemgpu_ctx* c, int32_t enable) {
  if (!c) return fail(nullptr, BEMGPU_EINVAL, "null context");
  std::lock_guard<std::recursive_mutex> lk(c->mu);
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  c->graphs = enable != 0;
  if (!c->graphs) {
    c->lu_graphs.clear();
    c->lu_seen.clear();
  }
  return BEMGPU_OK;
}

int bemgpu_ctx_inject_alloc_failures(bemgpu_ctx* c, int32_t count) {
  if (!c || count < 0) return fail(c, BEMGPU_EINVAL, "invalid arguments");
  root_of(c)->inject_oom.store(count);
  return BEMGPU_OK;
}

int bemgpu_ctx_graph_stats(const bemgpu_ctx* c, int64_t* captures, int64_t* replays) {
  if (!c) return fail(nullptr, BEMGPU_EINVAL, "null context");
  if (captures) *captures = c->lu_captures;
  if (replays) *replays = c->lu_replays;
  return BEMGPU_OK;
}

int bemgpu_ctx_set_autotune(bemgpu_ctx* c, int32_t enable) {
  if (!c) return fail(nullptr, BEMGPU_EINVAL, "null context");
  std::lock_guard<std::recursive_mutex> lk(c->mu);
  c->autotune = enable != 0;
  if (!c->autotune) c->tuned.clear();
  return BEMGPU_OK;
}

int bemgpu_ctx_set_tensor_lu(bemgpu_ctx* c, int32_t enable) {
  if (!c) return fail(nullptr, BEMGPU_EINVAL, "null context");
  c->tensor_lu = enable != 0;
  return BEMGPU_OK;
}

int bemgpu_debug_cgemm(bemgpu_ctx* c, int64_t m, int64_t n, int32_t k, const float* A,
                       const float* B, float* C) {
  if (!c || !A || !B || !C || m <= 0 || n <= 0 || k <= 0)
    return fail(c, BEMGPU_EINVAL, "invalid arguments");
  std::lock_guard<std::recursive_mutex> lk(c->mu);
  cudaSetDevice(c->device);
  Buf dA, dB, dC, pa, pb, dpi, dgi;
  TRY(alloc(c, (size_t)m * k * 8, &dA));
  TRY(alloc(c, (size_t)k * n * 8, &dB));
  TRY(alloc(c, (size_t)m * n * 8, &dC));
  TRY(alloc(c, tc_pack_bytes(m, k), &pa));
  TRY(alloc(c, tc_pack_bytes(n, k), &pb));
  CUDA_TRY(c, cudaMemcpyAsync(dA.p, A, (size_t)m * k * 8, cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(c, cudaMemcpyAsync(dB.p, B, (size_t)k * n * 8, cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(c, cudaMemcpyAsync(dC.p, C, (size_t)m * n * 8, cudaMemcpyHostToDevice, c->stream));
  std::vector<TcPackInst> pk(2);
  std::memset(pk.data(), 0, sizeof(TcPackInst) * 2);
  pk[0].a = dA.p;
  pk[0].lda = m;
  pk[0].rows = m;
  pk[0].kk = k;
  pk[0].trans = 0;
  pk[0].out = pa.p;
  pk[0].active = 1;
  pk[1].a = dB.p;
  pk[1].lda = k;
  pk[1].rows = n;
  pk[1].kk = k;
  pk[1].trans = 1;
  pk[1].out = pb.p;
  pk[1].active = 1;
  std::vector<TcGemmInst> g(1);
  std::memset(g.data(), 0, sizeof(TcGemmInst));
  g[0].apack = pa.p;
  g[0].bpack = pb.p;
  g[0].c = dC.p;
  g[0].ldc = m;
  g[0].m = m;
  g[0].n = n;
  g[0].kk = k;
  g[0].active = 1;
  // even m: the reduction epilogue (as in the LU); odd m: the load / store epilogue
  alignas(64) uint8_t hmap[kTcMapBytes];
  Buf dmap;
  const bool red = tc_encode_cmap(hmap, dC.p, m, m, n);
  if (red) {
    TRY(alloc(c, kTcMapBytes, &dmap));
    CUDA_TRY(c, cudaMemcpyAsync(dmap.p, hmap, kTcMapBytes, cudaMemcpyHostToDevice, c->stream));
    g[0].cmap = dmap.p;
  }
  TRY(to_device(c, pk, &dpi));
  TRY(to_device(c, g, &dgi));
  const Launch L = c->launch();
  launch_tc_pack(L, dpi.as<TcPackInst>(), 2, std::max(m, n), k);
  {
    Prof pr(c, "gemm_tc");
    launch_tc_cgemm(L, dgi.as<TcGemmInst>(), 1, ((m + 127) / 128) * ((n + 127) / 128), red);
  }
  CUDA_TRY(c, cudaGetLastError());
  CUDA_TRY(c, cudaMemcpyAsync(C, dC.p, (size_t)m * n * 8, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  TRY(check_device_error(c));
  return BEMGPU_OK;
}

int bemgpu_timer_start(bemgpu_ctx* c) {
  if (!c) return fail(nullptr, BEMGPU_EINVAL, "null context");
  std::lock_guard<std::recursive_mutex> lk(c->mu);
  if (!c->t0) {
    CUDA_TRY(c, cudaEventCreate(&c->t0));
    CUDA_TRY(c, cudaEventCreate(&c->t1));
  }
  CUDA_TRY(c, cudaEventRecord(c->t0, c->stream));
  return BEMGPU_OK;
}

int bemgpu_timer_stop(bemgpu_ctx* c, double* ms) {
  if (!c || !ms || !c->t0) return fail(c, BEMGPU_EINVAL, "timer not started");
  std::lock_guard<std::recursive_mutex> lk(c->mu);
  CUDA_TRY(c, cudaEventRecord(c->t1, c->stream));
  CUDA_TRY(c, cudaEventSynchronize(c->t1));
  float m = 0.f;
  CUDA_TRY(c, cudaEventElapsedTime(&m, c->t0, c->t1));
  *ms = m;
  return BEMGPU_OK;
}

int bemgpu_launch_count(const bemgpu_ctx* c, int64_t* count) {
  (void)c;
  if (!count) return BEMGPU_EINVAL;
  *count = launch_total();
  return BEMGPU_OK;
}

}  // extern "C"
