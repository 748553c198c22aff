// Host-side surface utilities of libbemgpu: topology validation, SHA-256 fingerprint
// and the near-pair list.  No CUDA calls; every function here runs without a GPU.
//
// Compiled with -ffp-contract=off so that centroid, diameter and distance arithmetic
// rounds every operation separately on every host architecture: the near-pair set is
// then a deterministic function of the input bits.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <string>
#include <unordered_map>
#include <vector>

#include "bemgpu_internal.h"

namespace bemgpu {

namespace {

struct Vec3 {
  double x, y, z;
};
inline Vec3 sub(Vec3 a, Vec3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline double dot(Vec3 a, Vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline Vec3 cross(Vec3 a, Vec3 b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline Vec3 node(const double* nodes, int64_t i) {
  return {nodes[3 * i], nodes[3 * i + 1], nodes[3 * i + 2]};
}

std::string fmt(const char* f, long long a = 0, long long b = 0) {
  char buf[256];
  std::snprintf(buf, sizeof buf, f, a, b);
  return buf;
}

}  // namespace

// Mirrors geometry/surface.jl:275-283 (input checks) and :341-405 (topology).
int validate_surface(const double* nodes, int64_t N, const int64_t* tris, int64_t M,
                     double* resolution, std::string* err) {
  if (!nodes || !tris || N <= 0) {
    *err = "nodes must have three rows and at least one column";
    return BEMGPU_EINVAL;
  }
  if (M <= 0) {
    *err = "surface must contain triangles";
    return BEMGPU_EINVAL;
  }
  for (int64_t i = 0; i < 3 * N; ++i)
    if (!std::isfinite(nodes[i])) {
      *err = "node coordinates must be finite";
      return BEMGPU_EINVAL;
    }
  for (int64_t i = 0; i < 3 * M; ++i)
    if (tris[i] < 1 || tris[i] > N) {
      *err = "triangle connectivity contains an invalid node index";
      return BEMGPU_EINVAL;
    }
  Vec3 first = node(nodes, tris[0] - 1);
  double extent = 0.0;
  for (int64_t i = 0; i < N; ++i) {
    Vec3 d = sub(node(nodes, i), node(nodes, 0));
    extent = std::max(extent, std::sqrt(dot(d, d)));
  }
  const double eps = std::numeric_limits<double>::epsilon();
  const double tol = 100.0 * eps * extent * extent;
  double res = 0.0, volume = 0.0;
  // edge key (min, max) -> list of (triangle, orientation sign)
  std::unordered_map<uint64_t, std::vector<std::pair<int64_t, int>>> edges;
  edges.reserve(static_cast<size_t>(3 * M));
  std::vector<std::vector<int64_t>> vertex_faces(static_cast<size_t>(N));
  for (int64_t t = 0; t < M; ++t) {
    int64_t a = tris[3 * t] - 1, b = tris[3 * t + 1] - 1, c = tris[3 * t + 2] - 1;
    if (a == b || b == c || a == c) {
      *err = fmt("triangle %lld repeats a node", t + 1);
      return BEMGPU_ETOPOLOGY;
    }
    vertex_faces[a].push_back(t);
    vertex_faces[b].push_back(t);
    vertex_faces[c].push_back(t);
    Vec3 pa = node(nodes, a), pb = node(nodes, b), pc = node(nodes, c);
    Vec3 nrm = cross(sub(pb, pa), sub(pc, pa));
    if (!(std::sqrt(dot(nrm, nrm)) > tol)) {
      *err = fmt("triangle %lld is degenerate", t + 1);
      return BEMGPU_ETOPOLOGY;
    }
    volume += dot(sub(pa, first), cross(sub(pb, first), sub(pc, first))) / 6.0;
    const int64_t uv[3][2] = {{a, b}, {b, c}, {c, a}};
    for (auto& e : uv) {
      int64_t u = e[0], v = e[1];
      uint64_t key = (static_cast<uint64_t>(std::min(u, v)) << 32) |
                     static_cast<uint64_t>(std::max(u, v));
      edges[key].push_back({t, u < v ? 1 : -1});
      Vec3 d = sub(node(nodes, u), node(nodes, v));
      res = std::max(res, std::sqrt(dot(d, d)));
    }
  }
  std::vector<std::vector<int64_t>> nbr(static_cast<size_t>(M));
  for (auto& kv : edges) {
    auto& inc = kv.second;
    long long lo = static_cast<long long>(kv.first >> 32) + 1;
    long long hi = static_cast<long long>(kv.first & 0xffffffffu) + 1;
    if (inc.size() != 2) {
      char buf[160];
      std::snprintf(buf, sizeof buf,
                    "edge (%lld, %lld) has %zu incident triangles; expected two", lo, hi,
                    inc.size());
      *err = buf;
      return BEMGPU_ETOPOLOGY;
    }
    if (inc[0].second != -inc[1].second) {
      *err = fmt("triangles %lld and %lld have inconsistent orientation", inc[0].first + 1,
                 inc[1].first + 1);
      return BEMGPU_ETOPOLOGY;
    }
    nbr[inc[0].first].push_back(inc[1].first);
    nbr[inc[1].first].push_back(inc[0].first);
  }
  std::vector<char> seen(static_cast<size_t>(M), 0);
  std::vector<int64_t> stack{0};
  int64_t visited = 0;
  while (!stack.empty()) {
    int64_t i = stack.back();
    stack.pop_back();
    if (seen[i]) continue;
    seen[i] = 1;
    ++visited;
    for (int64_t j : nbr[i]) stack.push_back(j);
  }
  if (visited != M) {
    *err = "supply one connected surface; nested/disjoint regions need a multi-region solve";
    return BEMGPU_ETOPOLOGY;
  }
  for (int64_t v = 0; v < N; ++v) {
    auto& faces = vertex_faces[v];
    if (faces.empty()) continue;
    std::vector<int64_t> fan{faces[0]};
    std::vector<int64_t> st{faces[0]};
    while (!st.empty()) {
      int64_t i = st.back();
      st.pop_back();
      for (int64_t j : nbr[i]) {
        if (std::find(faces.begin(), faces.end(), j) != faces.end() &&
            std::find(fan.begin(), fan.end(), j) == fan.end()) {
          fan.push_back(j);
          st.push_back(j);
        }
      }
    }
    if (fan.size() != faces.size()) {
      *err = fmt("vertex %lld is nonmanifold", v + 1);
      return BEMGPU_ETOPOLOGY;
    }
  }
  if (!(volume > 100.0 * eps * extent * extent * extent)) {
    *err = "surface must enclose positive volume with outward orientation";
    return BEMGPU_ETOPOLOGY;
  }
  if (resolution) *resolution = res;
  return BEMGPU_OK;
}

// ------------------------------------------------------------------ SHA-256 (FIPS 180-4)
namespace {
const uint32_t K256[64] = {
    0x428a2f98, 0x71374491, 0xb5c0fbcf, 0xe9b5dba5, 0x3956c25b, 0x59f111f1, 0x923f82a4,
    0xab1c5ed5, 0xd807aa98, 0x12835b01, 0x243185be, 0x550c7dc3, 0x72be5d74, 0x80deb1fe,
    0x9bdc06a7, 0xc19bf174, 0xe49b69c1, 0xefbe4786, 0x0fc19dc6, 0x240ca1cc, 0x2de92c6f,
    0x4a7484aa, 0x5cb0a9dc, 0x76f988da, 0x983e5152, 0xa831c66d, 0xb00327c8, 0xbf597fc7,
    0xc6e00bf3, 0xd5a79147, 0x06ca6351, 0x14292967, 0x27b70a85, 0x2e1b2138, 0x4d2c6dfc,
    0x53380d13, 0x650a7354, 0x766a0abb, 0x81c2c92e, 0x92722c85, 0xa2bfe8a1, 0xa81a664b,
    0xc24b8b70, 0xc76c51a3, 0xd192e819, 0xd6990624, 0xf40e3585, 0x106aa070, 0x19a4c116,
    0x1e376c08, 0x2748774c, 0x34b0bcb5, 0x391c0cb3, 0x4ed8aa4a, 0x5b9cca4f, 0x682e6ff3,
    0x748f82ee, 0x78a5636f, 0x84c87814, 0x8cc70208, 0x90befffa, 0xa4506ceb, 0xbef9a3f7,
    0xc67178f2};

struct Sha256 {
  uint32_t h[8] = {0x6a09e667, 0xbb67ae85, 0x3c6ef372, 0xa54ff53a,
                   0x510e527f, 0x9b05688c, 0x1f83d9ab, 0x5be0cd19};
  uint8_t buf[64];
  size_t fill = 0;
  uint64_t total = 0;
  static uint32_t rotr(uint32_t x, int n) { return (x >> n) | (x << (32 - n)); }
  void block(const uint8_t* p) {
    uint32_t w[64];
    for (int i = 0; i < 16; ++i)
      w[i] = (uint32_t(p[4 * i]) << 24) | (uint32_t(p[4 * i + 1]) << 16) |
             (uint32_t(p[4 * i + 2]) << 8) | uint32_t(p[4 * i + 3]);
    for (int i = 16; i < 64; ++i) {
      uint32_t s0 = rotr(w[i - 15], 7) ^ rotr(w[i - 15], 18) ^ (w[i - 15] >> 3);
      uint32_t s1 = rotr(w[i - 2], 17) ^ rotr(w[i - 2], 19) ^ (w[i - 2] >> 10);
      w[i] = w[i - 16] + s0 + w[i - 7] + s1;
    }
    uint32_t a = h[0], b = h[1], c = h[2], d = h[3], e = h[4], f = h[5], g = h[6], hh = h[7];
    for (int i = 0; i < 64; ++i) {
      uint32_t S1 = rotr(e, 6) ^ rotr(e, 11) ^ rotr(e, 25);
      uint32_t ch = (e & f) ^ (~e & g);
      uint32_t t1 = hh + S1 + ch + K256[i] + w[i];
      uint32_t S0 = rotr(a, 2) ^ rotr(a, 13) ^ rotr(a, 22);
      uint32_t mj = (a & b) ^ (a & c) ^ (b & c);
      uint32_t t2 = S0 + mj;
      hh = g; g = f; f = e; e = d + t1; d = c; c = b; b = a; a = t1 + t2;
    }
    h[0] += a; h[1] += b; h[2] += c; h[3] += d; h[4] += e; h[5] += f; h[6] += g; h[7] += hh;
  }
  void update(const void* data, size_t len) {
    const uint8_t* p = static_cast<const uint8_t*>(data);
    total += len;
    while (len) {
      size_t take = std::min(len, size_t(64) - fill);
      std::memcpy(buf + fill, p, take);
      fill += take;
      p += take;
      len -= take;
      if (fill == 64) {
        block(buf);
        fill = 0;
      }
    }
  }
  void finish(char out[65]) {
    uint64_t bits = total * 8;
    uint8_t pad = 0x80;
    update(&pad, 1);
    uint8_t zero = 0;
    while (fill != 56) update(&zero, 1);
    uint8_t lenb[8];
    for (int i = 0; i < 8; ++i) lenb[i] = uint8_t(bits >> (56 - 8 * i));
    update(lenb, 8);
    for (int i = 0; i < 8; ++i) std::snprintf(out + 8 * i, 9, "%08x", h[i]);
    out[64] = 0;
  }
};

void put_le64(Sha256& s, uint64_t v) {
  uint8_t b[8];
  for (int i = 0; i < 8; ++i) b[i] = uint8_t(v >> (8 * i));
  s.update(b, 8);
}
}  // namespace

void mesh_hash(const double* nodes, int64_t N, const int64_t* tris, int64_t M,
               char out[65]) {
  Sha256 s;
  put_le64(s, static_cast<uint64_t>(N));
  put_le64(s, static_cast<uint64_t>(M));
  for (int64_t i = 0; i < 3 * N; ++i) {
    uint64_t v;
    std::memcpy(&v, &nodes[i], 8);
    put_le64(s, v);
  }
  for (int64_t i = 0; i < 3 * M; ++i) put_le64(s, static_cast<uint64_t>(tris[i]));
  s.finish(out);
}

// ------------------------------------------------------------------ panel geometry
void panel_centroids(const double* nodes, const int64_t* tris, int64_t M,
                     std::vector<double>* cent, std::vector<double>* diam) {
  cent->resize(static_cast<size_t>(3 * M));
  diam->resize(static_cast<size_t>(M));
  for (int64_t t = 0; t < M; ++t) {
    Vec3 v[3];
    for (int a = 0; a < 3; ++a) v[a] = node(nodes, tris[3 * t + a] - 1);
    (*cent)[3 * t] = (v[0].x + v[1].x + v[2].x) / 3.0;
    (*cent)[3 * t + 1] = (v[0].y + v[1].y + v[2].y) / 3.0;
    (*cent)[3 * t + 2] = (v[0].z + v[1].z + v[2].z) / 3.0;
    double dm = 0.0;
    for (int a = 0; a < 3; ++a) {
      Vec3 e = sub(v[(a + 1) % 3], v[a]);
      double l = std::sqrt(dot(e, e));
      if (l > dm) dm = l;
    }
    (*diam)[t] = dm;
  }
}

// Near pairs with a uniform grid: cell size = eta * max diameter, so every near pair
// lies in the 27-cell neighbourhood.  Same predicate as the oracle's O(n^2) scan.
void near_pairs(const std::vector<double>& cent, const std::vector<double>& diam,
                double eta, std::vector<int64_t>* rowptr, std::vector<int64_t>* cols) {
  const int64_t M = static_cast<int64_t>(diam.size());
  const double eta2 = eta * eta;
  double dmax = 0.0, lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (int64_t t = 0; t < M; ++t) {
    dmax = std::max(dmax, diam[t]);
    for (int d = 0; d < 3; ++d) {
      lo[d] = std::min(lo[d], cent[3 * t + d]);
      hi[d] = std::max(hi[d], cent[3 * t + d]);
    }
  }
  double cell = std::max(eta * dmax, 1e-300);
  int64_t dims[3];
  for (int d = 0; d < 3; ++d)
    dims[d] = std::max<int64_t>(1, std::min<int64_t>(
                                       1024, static_cast<int64_t>((hi[d] - lo[d]) / cell) + 1));
  auto cell_of = [&](int64_t t, int d) {
    int64_t c = static_cast<int64_t>((cent[3 * t + d] - lo[d]) / cell);
    return std::min(std::max<int64_t>(c, 0), dims[d] - 1);
  };
  std::vector<std::vector<int64_t>> grid(static_cast<size_t>(dims[0] * dims[1] * dims[2]));
  for (int64_t t = 0; t < M; ++t)
    grid[(cell_of(t, 0) * dims[1] + cell_of(t, 1)) * dims[2] + cell_of(t, 2)].push_back(t);
  rowptr->assign(static_cast<size_t>(M + 1), 0);
  cols->clear();
  std::vector<int64_t> row;
  for (int64_t i = 0; i < M; ++i) {
    (*rowptr)[i] = static_cast<int64_t>(cols->size());
    row.clear();
    int64_t ci[3] = {cell_of(i, 0), cell_of(i, 1), cell_of(i, 2)};
    for (int64_t a = std::max<int64_t>(0, ci[0] - 1); a <= std::min(dims[0] - 1, ci[0] + 1); ++a)
      for (int64_t b = std::max<int64_t>(0, ci[1] - 1); b <= std::min(dims[1] - 1, ci[1] + 1); ++b)
        for (int64_t c = std::max<int64_t>(0, ci[2] - 1); c <= std::min(dims[2] - 1, ci[2] + 1);
             ++c)
          for (int64_t j : grid[(a * dims[1] + b) * dims[2] + c]) {
            bool near = (i == j);
            if (!near) {
              double dx = cent[3 * i] - cent[3 * j];
              double dy = cent[3 * i + 1] - cent[3 * j + 1];
              double dz = cent[3 * i + 2] - cent[3 * j + 2];
              double d2 = dx * dx + dy * dy + dz * dz;
              double r2 = eta2 * (diam[j] * diam[j]);
              near = d2 < r2;
            }
            if (near) row.push_back(j);
          }
    std::sort(row.begin(), row.end());
    cols->insert(cols->end(), row.begin(), row.end());
  }
  (*rowptr)[M] = static_cast<int64_t>(cols->size());
}

}  // namespace bemgpu
