// Hierarchical-matrix plan of a panel set (host only): cluster tree, block partition and
// the per-leaf block lists of the matrix-vector product.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace bemgpu {

// Admissible (low-rank) block of the permuted index space: rows [rlo, rlo + m),
// columns [clo, clo + n).
struct HmBlock {
  int32_t rlo, m, clo, n;
};

struct HmPlan {
  int64_t n = 0;
  std::vector<int32_t> perm;     // permuted position -> panel
  std::vector<int32_t> iperm;    // panel -> permuted position
  std::vector<int32_t> leaf_lo;  // row leaves in order: first position of each, plus n
  std::vector<HmBlock> dense;    // inadmissible leaf pairs (full blocks)
  std::vector<HmBlock> lowrank;  // admissible pairs (compressed)
  int32_t depth = 0;             // levels of the cluster tree
};

// Cluster tree by median bisection of the panel centroids (cent, 3 per panel) along the
// longest side of their bounding box, leaves of at most `leaf` panels; block tree by the
// standard admissibility min(diam s, diam t) < eta dist(s, t) with the centroid boxes,
// further restricted to dist(s, t) >= near_eta * (largest panel diameter of s and t) so
// that no pair integrated by the singular rules (|c_i - c_j| < near_eta diam_j) falls
// into a compressed block.  Deterministic (ties broken by panel index).
int hm_build_plan(const double* cent, const double* diam, int64_t n, int32_t leaf, double eta,
                  double near_eta, HmPlan* out, std::string* err);

// Rows of the matrix-vector product: for every row leaf, the blocks that cover its rows
// in a fixed order (full blocks as their index, low-rank ones as -(index + 1)); a block
// is listed by every leaf its row range covers (leaf ranges nest in block ranges).
void hm_leaf_lists(const HmPlan& plan, const std::vector<HmBlock>& dense,
                   const std::vector<HmBlock>& lowrank, std::vector<int32_t>* ptr,
                   std::vector<int32_t>* ent);

}  // namespace bemgpu
