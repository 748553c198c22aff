// Cluster tree, block partition and product lists of the hierarchical-matrix operators.
// The roles follow the reference's H-matrix assembly (Inti operators compressed with
// HMatrices.jl, solvers/bem/full.jl:89-97 with compression=(method=:hmatrix, tol)):
// a geometric cluster tree over the unknowns, strong admissibility, full leaf blocks and
// low-rank admissible blocks.  The tree here is built for the GPU kernels that consume
// it: contiguous permuted ranges, balanced leaves and flat block arrays.
#include "hmatrix_plan.h"

#include <algorithm>
#include <cmath>
#include <functional>

namespace bemgpu {

namespace {

struct Cluster {
  int64_t lo, hi;
  double bmin[3], bmax[3];
  double maxdiam;  // largest panel diameter inside
  int32_t child[2];
  double size() const {
    double s = 0.0;
    for (int d = 0; d < 3; ++d) s += (bmax[d] - bmin[d]) * (bmax[d] - bmin[d]);
    return std::sqrt(s);
  }
};

double box_distance(const Cluster& a, const Cluster& b) {
  double s = 0.0;
  for (int d = 0; d < 3; ++d) {
    const double g = std::max({0.0, b.bmin[d] - a.bmax[d], a.bmin[d] - b.bmax[d]});
    s += g * g;
  }
  return std::sqrt(s);
}

}  // namespace

int hm_build_plan(const double* cent, const double* diam, int64_t n, int32_t leaf, double eta,
                  double near_eta, HmPlan* out, std::string* err) {
  if (n <= 0 || n > INT32_MAX / 2) {
    *err = "panel count out of range for the hierarchical matrix";
    return 1;
  }
  if (leaf < 8 || leaf > 64) {
    *err = "leaf_size must lie in [8, 64]";
    return 1;
  }
  if (!(std::isfinite(eta) && eta > 0)) {
    *err = "admissibility eta must be finite and positive";
    return 1;
  }
  HmPlan& P = *out;
  P = HmPlan{};
  P.n = n;
  P.perm.resize((size_t)n);
  for (int64_t i = 0; i < n; ++i) P.perm[(size_t)i] = (int32_t)i;
  std::vector<Cluster> cl;
  cl.reserve((size_t)(4 * n / leaf + 4));
  std::function<int32_t(int64_t, int64_t, int32_t)> build = [&](int64_t lo, int64_t hi,
                                                                int32_t level) -> int32_t {
    Cluster c;
    c.lo = lo;
    c.hi = hi;
    c.maxdiam = 0.0;
    c.child[0] = c.child[1] = -1;
    for (int d = 0; d < 3; ++d) {
      c.bmin[d] = 1e300;
      c.bmax[d] = -1e300;
    }
    for (int64_t t = lo; t < hi; ++t) {
      const int32_t p = P.perm[(size_t)t];
      for (int d = 0; d < 3; ++d) {
        c.bmin[d] = std::min(c.bmin[d], cent[3 * p + d]);
        c.bmax[d] = std::max(c.bmax[d], cent[3 * p + d]);
      }
      c.maxdiam = std::max(c.maxdiam, diam[p]);
    }
    P.depth = std::max(P.depth, level + 1);
    const int32_t id = (int32_t)cl.size();
    cl.push_back(c);
    if (hi - lo > leaf) {
      int axis = 0;
      for (int d = 1; d < 3; ++d)
        if (c.bmax[d] - c.bmin[d] > c.bmax[axis] - c.bmin[axis]) axis = d;
      std::sort(P.perm.begin() + lo, P.perm.begin() + hi, [&](int32_t a, int32_t b) {
        const double xa = cent[3 * a + axis], xb = cent[3 * b + axis];
        return xa < xb || (xa == xb && a < b);
      });
      const int64_t mid = lo + (hi - lo) / 2;
      const int32_t c0 = build(lo, mid, level + 1);
      const int32_t c1 = build(mid, hi, level + 1);
      cl[(size_t)id].child[0] = c0;
      cl[(size_t)id].child[1] = c1;
    } else {
      P.leaf_lo.push_back((int32_t)lo);
    }
    return id;
  };
  build(0, n, 0);
  P.leaf_lo.push_back((int32_t)n);
  P.iperm.resize((size_t)n);
  for (int64_t t = 0; t < n; ++t) P.iperm[(size_t)P.perm[(size_t)t]] = (int32_t)t;
  // block tree
  auto admissible = [&](const Cluster& a, const Cluster& b) {
    const double d = box_distance(a, b);
    if (!(d > 0.0)) return false;
    if (d < near_eta * std::max(a.maxdiam, b.maxdiam)) return false;
    const double sa = a.size() + a.maxdiam, sb = b.size() + b.maxdiam;
    return std::min(sa, sb) < eta * d;
  };
  std::vector<std::pair<int32_t, int32_t>> stack{{0, 0}};
  while (!stack.empty()) {
    const auto [ta, tb] = stack.back();
    stack.pop_back();
    const Cluster& a = cl[(size_t)ta];
    const Cluster& b = cl[(size_t)tb];
    const HmBlock blk{(int32_t)a.lo, (int32_t)(a.hi - a.lo), (int32_t)b.lo, (int32_t)(b.hi - b.lo)};
    if (admissible(a, b)) {
      P.lowrank.push_back(blk);
      continue;
    }
    const bool la = a.child[0] < 0, lb = b.child[0] < 0;
    if (la && lb) {
      P.dense.push_back(blk);
    } else if (la) {
      stack.push_back({ta, b.child[1]});
      stack.push_back({ta, b.child[0]});
    } else if (lb) {
      stack.push_back({a.child[1], tb});
      stack.push_back({a.child[0], tb});
    } else {
      for (int u = 1; u >= 0; --u)
        for (int v = 1; v >= 0; --v) stack.push_back({a.child[u], b.child[v]});
    }
  }
  return 0;
}

void hm_leaf_lists(const HmPlan& plan, const std::vector<HmBlock>& dense,
                   const std::vector<HmBlock>& lowrank, std::vector<int32_t>* ptr,
                   std::vector<int32_t>* ent) {
  const size_t nl = plan.leaf_lo.size() - 1;
  std::vector<std::vector<int32_t>> lists(nl);
  auto leaf_of = [&](int32_t row) {
    return (size_t)(std::upper_bound(plan.leaf_lo.begin(), plan.leaf_lo.end(), row) -
                    plan.leaf_lo.begin() - 1);
  };
  for (size_t b = 0; b < dense.size(); ++b) {  // full blocks may span several leaves
    const HmBlock& B = dense[b];
    for (size_t l = leaf_of(B.rlo); l < nl && plan.leaf_lo[l] < B.rlo + B.m; ++l)
      lists[l].push_back((int32_t)b);
  }
  for (size_t b = 0; b < lowrank.size(); ++b) {
    const HmBlock& B = lowrank[b];
    for (size_t l = leaf_of(B.rlo); l < nl && plan.leaf_lo[l] < B.rlo + B.m; ++l)
      lists[l].push_back(-(int32_t)b - 1);
  }
  ptr->assign(nl + 1, 0);
  ent->clear();
  for (size_t l = 0; l < nl; ++l) {
    (*ptr)[l] = (int32_t)ent->size();
    ent->insert(ent->end(), lists[l].begin(), lists[l].end());
  }
  (*ptr)[nl] = (int32_t)ent->size();
}

}  // namespace bemgpu
