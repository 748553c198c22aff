// Nyström operators on quadrature nodes with a density-interpolation correction.
//
// The reference assembles its rigid/soft system from Inti's Nyström operators on the
// surface quadrature nodes (solvers/bem/full.jl:68-128, Inti.single_double_layer and
// Inti.adj_double_layer_hypersingular with correction=(method=:dim,)), and corrects the
// singular and nearly singular quadrature with a Green-identity fit over each target's
// nearest element (the structure of solvers/bem/quadrature/fluid.jl:94-163: defect of
// the discrete identity on a basis of Helmholtz solutions, scaled minimum-norm fit of the
// element's node weights).  The basis here is kNyBasis plane waves (Faria, Perez-Arancibia
// and Bonnet 2021, doi:10.1016/j.cma.2021.113703, for the general-purpose kernel
// regularisation; plane-wave interpolants after Perez-Arancibia, Faria and Turc 2019,
// SIAM J. Sci. Comput. 41(4)).
//
// For on-surface targets every node's nearest element is its own, so the correction is a
// 7x7 block on the diagonal of each operator.  With u a plane wave (regular inside the
// body, outward normals) the identities are
//   1/2 u(x)     = S[du/dn](x)  - D[u](x)
//   1/2 du/dn(x) = K'[du/dn](x) - H[u](x)
// and the defect of the uncorrected node rule, row by row and basis function by basis
// function, is fitted by weights on the seven nodes of the row's element: pressure
// weights w_p and flux weights w_f, D += w_p and S -= w_f for the first identity, H += w_p
// and K' -= w_f for the second.  The fit is linear in the defect and only the combinations
// M1 = 1/2 I - D - alpha H and M2 = S + alpha (1/2 I + K') are kept, so one fit of the
// combined defect  e = def_1 + alpha def_2 = M2 F + M1 U - U - alpha F  (uncorrected M1,
// M2; U, F the basis traces) gives both corrections: M1 -= w_p(e), M2 -= w_f(e).
//
// Work split: k_ny_traces (basis traces at the nodes), k_ny_assemble (every pair once:
// the two system matrices and the combined defect sums, FP64-issue-bound), k_ny_correct
// (one thread per element: Householder QR of the 14 x 9 trace matrix, 7 fits, the
// corrections).
#include <climits>
#include <cmath>

#include "nystrom.cuh"
#include "quad_math.cuh"

namespace bemgpu {

namespace {

struct z2 {
  double x, y;
};
__device__ __forceinline__ z2 zmul(z2 a, z2 b) { return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
__device__ __forceinline__ z2 zconj(z2 a) { return {a.x, -a.y}; }
// acc += a * b
__device__ __forceinline__ void zfma(z2& acc, z2 a, z2 b) {
  acc.x += a.x * b.x - a.y * b.y;
  acc.y += a.x * b.y + a.y * b.x;
}
// acc -= a * b
__device__ __forceinline__ void zfms(z2& acc, z2 a, z2 b) {
  acc.x -= a.x * b.x - a.y * b.y;
  acc.y -= a.x * b.y + a.y * b.x;
}
__device__ __forceinline__ z2 zdiv(z2 a, z2 b) {
  const double d = b.x * b.x + b.y * b.y;
  return {(a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d};
}

constexpr double kInv4Pi = 0.07957747154594766788;  // 1 / (4 pi)

// ------------------------------------------------------------------ interpolant traces
// u_s(y) = exp(i k d_s . y), du_s/dn = i k (d_s . n) u_s at every node.
__global__ void k_ny_traces(NyInst I) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= I.n) return;
  const double* r = I.nodes + j * kPanelDoubles;
  z2* tr = reinterpret_cast<z2*>(I.trace);
  for (int s = 0; s < kNyBasis; ++s) {
    const double* d = I.dirs + 3 * s;
    const double ph = I.k * (d[0] * r[0] + d[1] * r[1] + d[2] * r[2]);
    const double kdn = I.k * (d[0] * r[3] + d[1] * r[4] + d[2] * r[5]);
    double sn, cs;
    sincos(ph, &sn, &cs);
    tr[(int64_t)s * I.n + j] = {cs, sn};
    tr[(int64_t)(kNyBasis + s) * I.n + j] = {-kdn * sn, kdn * cs};
  }
}

// ------------------------------------------------------------------ pair assembly
// Thread = row i (coalesced column-major stores), CTA = kNyRows rows x one column range;
// columns staged kNyTile at a time.  Per pair (i != j), with d = x_i - y_j, r = |d|,
// G = e^{ikr} / (4 pi r), G' = G (ik - 1/r), G'' = G ((ik - 1/r)^2 + 1/r^2), weight w_j:
//   S = G w,  D = -G' (d.n_j)/r w,  K' = G' (d.n_i)/r w,
//   H = -[(G'' - G'/r) (d.n_i)(d.n_j)/r^2 + G' (n_i.n_j)/r] w;
// the coincident pair (i == j) contributes zero to every operator.
__global__ void __launch_bounds__(kNyRows) k_ny_assemble(NyInst I) {
  const int64_t n = I.n;
  const int64_t i = (int64_t)blockIdx.x * kNyRows + threadIdx.x;
  const int64_t c0 = (int64_t)blockIdx.y * I.chunk_cols;
  const int64_t c1 = min(n, c0 + I.chunk_cols);
  __shared__ double s_node[kNyTile][7];           // position, normal, weight
  __shared__ z2 s_tr[2 * kNyBasis][kNyTile];      // u_s, du_s/dn
  const bool row = i < n;
  double xi[3] = {0, 0, 0}, ni[3] = {0, 0, 0};
  if (row) {
    const double* r = I.nodes + i * kPanelDoubles;
    for (int d = 0; d < 3; ++d) {
      xi[d] = r[d];
      ni[d] = r[3 + d];
    }
  }
  const double k = I.k;
  const z2 al = {I.a_re, I.a_im};
  z2 acc[kNyBasis];
#pragma unroll
  for (int t = 0; t < kNyBasis; ++t) acc[t] = {0.0, 0.0};
  const z2* tr = reinterpret_cast<const z2*>(I.trace);
  z2* M1 = reinterpret_cast<z2*>(I.M1);
  z2* M2 = reinterpret_cast<z2*>(I.M2);
  for (int64_t t0 = c0; t0 < c1; t0 += kNyTile) {
    const int cnt = (int)min((int64_t)kNyTile, c1 - t0);
    __syncthreads();
    for (int e = threadIdx.x; e < kNyTile * 7; e += kNyRows) {
      const int jj = e / 7, f = e % 7;
      s_node[jj][f] = jj < cnt ? I.nodes[(t0 + jj) * kPanelDoubles + f] : 0.0;
    }
    for (int e = threadIdx.x; e < kNyTile * 2 * kNyBasis; e += kNyRows) {
      const int jj = e % kNyTile, t = e / kNyTile;
      s_tr[t][jj] = jj < cnt ? tr[(int64_t)t * n + t0 + jj] : z2{0.0, 0.0};
    }
    __syncthreads();
    if (!row) continue;
    for (int jj = 0; jj < cnt; ++jj) {
      const int64_t j = t0 + jj;
      z2 m1, m2;
      if (j == i) {
        m1 = {0.5, 0.0};
        m2 = {0.5 * al.x, 0.5 * al.y};
      } else {
        const double dx = xi[0] - s_node[jj][0], dy = xi[1] - s_node[jj][1],
                     dz = xi[2] - s_node[jj][2];
        const double r2 = dx * dx + dy * dy + dz * dz;
        const double r = sqrt(r2);
        const double ir = 1.0 / r;
        double sn, cs;
        sincos(k * r, &sn, &cs);
        const double w = s_node[jj][6];
        const double gs = kInv4Pi * ir;
        const z2 G = {cs * gs, sn * gs};
        const z2 G1 = zmul(G, z2{-ir, k});
        const z2 G2 = zmul(G, z2{2.0 * ir * ir - k * k, -2.0 * k * ir});
        const double dny = dx * s_node[jj][3] + dy * s_node[jj][4] + dz * s_node[jj][5];
        const double dnx = dx * ni[0] + dy * ni[1] + dz * ni[2];
        const double nn = ni[0] * s_node[jj][3] + ni[1] * s_node[jj][4] + ni[2] * s_node[jj][5];
        const z2 S = {G.x * w, G.y * w};
        const double fd = -dny * ir * w, fk = dnx * ir * w;
        const z2 D = {G1.x * fd, G1.y * fd};
        const z2 K = {G1.x * fk, G1.y * fk};
        const double f2 = dnx * dny * ir * ir, f1 = nn * ir;
        const z2 H = {-((G2.x - G1.x * ir) * f2 + G1.x * f1) * w,
                      -((G2.y - G1.y * ir) * f2 + G1.y * f1) * w};
        const z2 aH = zmul(al, H), aK = zmul(al, K);
        m1 = {-D.x - aH.x, -D.y - aH.y};
        m2 = {S.x + aK.x, S.y + aK.y};
      }
      M1[i + j * n] = m1;
      M2[i + j * n] = m2;
#pragma unroll
      for (int s = 0; s < kNyBasis; ++s) {  // (M2 F + M1 U) of the row
        zfma(acc[s], m2, s_tr[kNyBasis + s][jj]);
        zfma(acc[s], m1, s_tr[s][jj]);
      }
    }
  }
  if (!row) return;
  z2* part = reinterpret_cast<z2*>(I.part);
#pragma unroll
  for (int t = 0; t < kNyBasis; ++t) part[((int64_t)blockIdx.y * kNyBasis + t) * n + i] = acc[t];
}

// ------------------------------------------------------------------ element corrections
// Element e, nodes 7e..7e+6.  Trace matrix M (14 x kNyBasis): rows u_s and du_s/dn at the
// nodes, each row scaled to unit norm (scale sc).  A = (M / sc)^T; the weights of a row's
// defect d are the minimum-norm solution of A w~ = d, w = w~ / sc, computed from the
// Householder QR A^H = Qf R: w~ = Qf R^{-H} d (equal to the pseudo-inverse solution for
// A of full row rank).  d is the combined defect of the row; its pressure weights (first
// 7) are subtracted from M1, its flux weights (last 7) from M2.
constexpr int kNyFit = 2 * kNyNodes;  // unknown weights per element
constexpr int kNyCorrT = 64;

// Scaled trace matrix of one element and its Householder QR (per thread, local memory).
struct NyFit {
  z2 B[kNyFit][kNyBasis];  // A^H, reduced in place to R
  z2 V[kNyFit][kNyBasis];  // Householder vectors (unit norm), column c from row c on
  double sc[kNyFit];       // row scales
};

// Factor the fit of the element whose nodes are b..b+6; false when R has a pivot below
// 1e-13 of the first (rank-deficient fit).
__device__ bool ny_fit_factor(NyFit& F, const z2* tr, int64_t n, int64_t b) {
  for (int j = 0; j < kNyFit; ++j) {
    const int64_t node = b + (j % kNyNodes);
    const int t = j < kNyNodes ? 0 : 1;
    double s2 = 0.0;
    for (int s = 0; s < kNyBasis; ++s) {
      const z2 v = tr[(int64_t)(t * kNyBasis + s) * n + node];
      F.B[j][s] = v;
      s2 += v.x * v.x + v.y * v.y;
    }
    F.sc[j] = fmax(sqrt(s2), 1e-300);
    for (int s = 0; s < kNyBasis; ++s) F.B[j][s] = {F.B[j][s].x / F.sc[j], -F.B[j][s].y / F.sc[j]};
  }
  for (int c = 0; c < kNyBasis; ++c) {
    double nx = 0.0;
    for (int j = c; j < kNyFit; ++j) nx += F.B[j][c].x * F.B[j][c].x + F.B[j][c].y * F.B[j][c].y;
    nx = sqrt(nx);
    const z2 x0 = F.B[c][c];
    const double ax0 = hypot(x0.x, x0.y);
    const z2 ph = ax0 > 0.0 ? z2{x0.x / ax0, x0.y / ax0} : z2{1.0, 0.0};
    const z2 alpha = {-ph.x * nx, -ph.y * nx};
    for (int j = 0; j < kNyFit; ++j) F.V[j][c] = {0.0, 0.0};
    double vn = 0.0;
    for (int j = c; j < kNyFit; ++j) {
      F.V[j][c] = j == c ? z2{x0.x - alpha.x, x0.y - alpha.y} : F.B[j][c];
      vn += F.V[j][c].x * F.V[j][c].x + F.V[j][c].y * F.V[j][c].y;
    }
    vn = sqrt(vn);
    if (!(vn > 0.0)) return false;
    for (int j = c; j < kNyFit; ++j) F.V[j][c] = {F.V[j][c].x / vn, F.V[j][c].y / vn};
    for (int q = c; q < kNyBasis; ++q) {
      z2 dot = {0.0, 0.0};
      for (int j = c; j < kNyFit; ++j) zfma(dot, zconj(F.V[j][c]), F.B[j][q]);
      for (int j = c; j < kNyFit; ++j) {
        const z2 v2 = {2.0 * F.V[j][c].x, 2.0 * F.V[j][c].y};
        zfms(F.B[j][q], v2, dot);
      }
    }
  }
  const double r00 = hypot(F.B[0][0].x, F.B[0][0].y);
  for (int c = 0; c < kNyBasis; ++c)
    if (!(hypot(F.B[c][c].x, F.B[c][c].y) > 1e-13 * r00)) return false;
  return true;
}

// Weights w (14, unscaled: pressure weights then flux weights) of a defect d (9).
__device__ void ny_fit_solve(const NyFit& F, const z2* d, z2* w) {
  z2 z[kNyBasis];  // R^{-H} d (R^H lower triangular)
  for (int q = 0; q < kNyBasis; ++q) {
    z2 v = d[q];
    for (int p = 0; p < q; ++p) zfms(v, zconj(F.B[p][q]), z[p]);
    z[q] = zdiv(v, zconj(F.B[q][q]));
  }
  for (int j = 0; j < kNyFit; ++j) w[j] = j < kNyBasis ? z[j] : z2{0.0, 0.0};
  for (int c = kNyBasis - 1; c >= 0; --c) {  // w = H_0 ... H_8 [z; 0]
    z2 dot = {0.0, 0.0};
    for (int j = c; j < kNyFit; ++j) zfma(dot, zconj(F.V[j][c]), w[j]);
    for (int j = c; j < kNyFit; ++j) {
      const z2 v2 = {2.0 * F.V[j][c].x, 2.0 * F.V[j][c].y};
      zfms(w[j], v2, dot);
    }
  }
  for (int j = 0; j < kNyFit; ++j) w[j] = {w[j].x / F.sc[j], w[j].y / F.sc[j]};
}

__global__ void __launch_bounds__(kNyCorrT) k_ny_correct(NyInst I) {
  const int64_t e = (int64_t)blockIdx.x * kNyCorrT + threadIdx.x;
  const int64_t n = I.n;
  if (e >= n / kNyNodes) return;
  const z2* tr = reinterpret_cast<const z2*>(I.trace);
  const z2* part = reinterpret_cast<const z2*>(I.part);
  z2* M1 = reinterpret_cast<z2*>(I.M1);
  z2* M2 = reinterpret_cast<z2*>(I.M2);
  const int64_t b = e * kNyNodes;
  NyFit F;
  if (!ny_fit_factor(F, tr, n, b)) {  // rank-deficient fit: the element keeps its rule
    I.status[e] = 1;
    return;
  }
  const z2 al = {I.a_re, I.a_im};
  for (int t = 0; t < kNyNodes; ++t) {
    const int64_t row = b + t;
    // combined defect e_s = (M2 F + M1 U)_s - u_s - alpha du_s/dn at the row
    z2 d[kNyBasis];
    for (int s = 0; s < kNyBasis; ++s) {
      z2 acc = {0.0, 0.0};
      for (int c = 0; c < I.n_chunks; ++c) {
        const z2 p = part[((int64_t)c * kNyBasis + s) * n + row];
        acc.x += p.x;
        acc.y += p.y;
      }
      const z2 u = tr[(int64_t)s * n + row], f = tr[(int64_t)(kNyBasis + s) * n + row];
      const z2 af = zmul(al, f);
      d[s] = {acc.x - u.x - af.x, acc.y - u.y - af.y};
    }
    z2 w[kNyFit];
    ny_fit_solve(F, d, w);
    for (int j = 0; j < kNyNodes; ++j) {
      const int64_t o = row + (b + j) * n;
      M1[o] = {M1[o].x - w[j].x, M1[o].y - w[j].y};
      M2[o] = {M2[o].x - w[kNyNodes + j].x, M2[o].y - w[kNyNodes + j].y};
    }
  }
}

// ------------------------------------------------------------------ fluid bodies
// The panel path's fluid blocks on the nodes (pair i != j; the identity parts on the
// diagonal):
//   Mueller: [I - De + Di, Se - g Si; -He + Hi/g, I + K'e - K'i]
//   CBIE:    [1/2 I - De,  Se;        1/2 I + Di,  -g Si]
// with e / i the operators at k / k_int.  Each wavenumber's operators are corrected on
// their own (the blocks mix them), so the defects of its identities are summed apart:
// slots 0 (S/D at k), 1 (K'/H at k), 2 (S/D at k_int), 3 (K'/H at k_int) for Mueller;
// 0 (S/D at k), 1 (S/D at k_int) for CBIE.
template <bool MULLER>
__global__ void __launch_bounds__(kNyRows) k_ny_assemble_fluid(NyInst I) {
  constexpr int ND = MULLER ? 4 : 2;
  const int64_t n = I.n, lda = 2 * I.n;
  const int64_t i = (int64_t)blockIdx.x * kNyRows + threadIdx.x;
  const int64_t c0 = (int64_t)blockIdx.y * I.chunk_cols;
  const int64_t c1 = min(n, c0 + I.chunk_cols);
  __shared__ double s_node[kNyTile][7];
  __shared__ z2 s_tr[4 * kNyBasis][kNyTile];  // u, du/dn at k, then at k_int
  const bool row = i < n;
  double xi[3] = {0, 0, 0}, ni[3] = {0, 0, 0};
  if (row) {
    const double* r = I.nodes + i * kPanelDoubles;
    for (int d = 0; d < 3; ++d) {
      xi[d] = r[d];
      ni[d] = r[3 + d];
    }
  }
  const double g = I.g, ginv = 1.0 / I.g;
  z2 acc[ND * kNyBasis];
#pragma unroll
  for (int t = 0; t < ND * kNyBasis; ++t) acc[t] = {0.0, 0.0};
  const z2* tre = reinterpret_cast<const z2*>(I.trace);
  const z2* tri = reinterpret_cast<const z2*>(I.trace_i);
  z2* A = reinterpret_cast<z2*>(I.A);
  for (int64_t t0 = c0; t0 < c1; t0 += kNyTile) {
    const int cnt = (int)min((int64_t)kNyTile, c1 - t0);
    __syncthreads();
    for (int e = threadIdx.x; e < kNyTile * 7; e += kNyRows) {
      const int jj = e / 7, f = e % 7;
      s_node[jj][f] = jj < cnt ? I.nodes[(t0 + jj) * kPanelDoubles + f] : 0.0;
    }
    for (int e = threadIdx.x; e < kNyTile * 4 * kNyBasis; e += kNyRows) {
      const int jj = e % kNyTile, t = e / kNyTile;
      const z2* src = t < 2 * kNyBasis ? tre : tri;
      const int tt = t < 2 * kNyBasis ? t : t - 2 * kNyBasis;
      s_tr[t][jj] = jj < cnt ? src[(int64_t)tt * n + t0 + jj] : z2{0.0, 0.0};
    }
    __syncthreads();
    if (!row) continue;
    for (int jj = 0; jj < cnt; ++jj) {
      const int64_t j = t0 + jj;
      z2 a11, a12, a21, a22;
      if (j == i) {
        a11 = {MULLER ? 1.0 : 0.5, 0.0};
        a12 = {0.0, 0.0};
        a21 = {MULLER ? 0.0 : 0.5, 0.0};
        a22 = {MULLER ? 1.0 : 0.0, 0.0};
      } else {
        const double dx = xi[0] - s_node[jj][0], dy = xi[1] - s_node[jj][1],
                     dz = xi[2] - s_node[jj][2];
        const double r = sqrt(dx * dx + dy * dy + dz * dz);
        const double ir = 1.0 / r;
        const double w = s_node[jj][6];
        const double dny = dx * s_node[jj][3] + dy * s_node[jj][4] + dz * s_node[jj][5];
        const double dnx = dx * ni[0] + dy * ni[1] + dz * ni[2];
        const double nn = ni[0] * s_node[jj][3] + ni[1] * s_node[jj][4] + ni[2] * s_node[jj][5];
        const double fd = -dny * ir * w, fk = dnx * ir * w;
        const double f2 = dnx * dny * ir * ir, f1 = nn * ir;
        z2 S[2], D[2], K[2], H[2];
#pragma unroll
        for (int side = 0; side < 2; ++side) {
          const double kk = side == 0 ? I.k : I.k_int;
          double sn, cs;
          sincos(kk * r, &sn, &cs);
          const double gs = kInv4Pi * ir;
          const z2 G = {cs * gs, sn * gs};
          const z2 G1 = zmul(G, z2{-ir, kk});
          S[side] = {G.x * w, G.y * w};
          D[side] = {G1.x * fd, G1.y * fd};
          if (MULLER) {
            const z2 G2 = zmul(G, z2{2.0 * ir * ir - kk * kk, -2.0 * kk * ir});
            K[side] = {G1.x * fk, G1.y * fk};
            H[side] = {-((G2.x - G1.x * ir) * f2 + G1.x * f1) * w,
                       -((G2.y - G1.y * ir) * f2 + G1.y * f1) * w};
          }
        }
        if (MULLER) {
          a11 = {D[1].x - D[0].x, D[1].y - D[0].y};
          a12 = {S[0].x - g * S[1].x, S[0].y - g * S[1].y};
          a21 = {ginv * H[1].x - H[0].x, ginv * H[1].y - H[0].y};
          a22 = {K[0].x - K[1].x, K[0].y - K[1].y};
        } else {
          a11 = {-D[0].x, -D[0].y};
          a12 = S[0];
          a21 = D[1];
          a22 = {-g * S[1].x, -g * S[1].y};
        }
#pragma unroll
        for (int s = 0; s < kNyBasis; ++s) {
          const z2 ue = s_tr[s][jj], fe = s_tr[kNyBasis + s][jj];
          const z2 ui = s_tr[2 * kNyBasis + s][jj], fi = s_tr[3 * kNyBasis + s][jj];
          z2& sde = acc[s];
          z2& sdi = acc[(MULLER ? 2 : 1) * kNyBasis + s];
          zfma(sde, S[0], fe);
          zfms(sde, D[0], ue);
          zfma(sdi, S[1], fi);
          zfms(sdi, D[1], ui);
          if (MULLER) {
            z2& khe = acc[kNyBasis + s];
            z2& khi = acc[3 * kNyBasis + s];
            zfma(khe, K[0], fe);
            zfms(khe, H[0], ue);
            zfma(khi, K[1], fi);
            zfms(khi, H[1], ui);
          }
        }
      }
      A[i + j * lda] = a11;
      A[i + (n + j) * lda] = a12;
      A[(n + i) + j * lda] = a21;
      A[(n + i) + (n + j) * lda] = a22;
    }
  }
  if (!row) return;
  z2* part = reinterpret_cast<z2*>(I.part);
#pragma unroll
  for (int t = 0; t < ND * kNyBasis; ++t)
    part[((int64_t)blockIdx.y * ND * kNyBasis + t) * n + i] = acc[t];
}

// One thread per element: a fit per wavenumber, then for every row of the element the
// weights of each defect (on-surface multiplier -1/2) applied to the blocks they enter:
//   S/D at k:      A11 -= w_p, A12 -= w_f          (dD = w_p, dS = -w_f)
//   K'/H at k:     A21 -= w_p, A22 -= w_f          (dH = w_p, dK' = -w_f)
//   S/D at k_int:  Mueller A11 += w_p, A12 += g w_f; CBIE A21 += w_p, A22 += g w_f
//   K'/H at k_int: A21 += w_p / g, A22 += w_f
template <bool MULLER>
__global__ void __launch_bounds__(kNyCorrT) k_ny_correct_fluid(NyInst I) {
  constexpr int ND = MULLER ? 4 : 2;
  const int64_t e = (int64_t)blockIdx.x * kNyCorrT + threadIdx.x;
  const int64_t n = I.n, lda = 2 * I.n;
  if (e >= n / kNyNodes) return;
  const z2* tre = reinterpret_cast<const z2*>(I.trace);
  const z2* tri = reinterpret_cast<const z2*>(I.trace_i);
  const z2* part = reinterpret_cast<const z2*>(I.part);
  z2* A = reinterpret_cast<z2*>(I.A);
  const int64_t b = e * kNyNodes;
  NyFit Fe, Fi;
  if (!ny_fit_factor(Fe, tre, n, b) || !ny_fit_factor(Fi, tri, n, b)) {
    I.status[e] = 1;
    return;
  }
  const double g = I.g;
  for (int t = 0; t < kNyNodes; ++t) {
    const int64_t row = b + t;
    for (int id = 0; id < ND; ++id) {
      const bool interior = MULLER ? id >= 2 : id == 1;
      const bool flux = MULLER && (id & 1);
      const z2* tr = interior ? tri : tre;
      z2 d[kNyBasis];
      for (int s = 0; s < kNyBasis; ++s) {
        z2 acc = {0.0, 0.0};
        for (int c = 0; c < I.n_chunks; ++c) {
          const z2 p = part[(((int64_t)c * ND + id) * kNyBasis + s) * n + row];
          acc.x += p.x;
          acc.y += p.y;
        }
        const z2 own = tr[(int64_t)((flux ? kNyBasis : 0) + s) * n + row];
        d[s] = {acc.x - 0.5 * own.x, acc.y - 0.5 * own.y};
      }
      z2 w[kNyFit];
      ny_fit_solve(interior ? Fi : Fe, d, w);
      // target block rows: pressure identity -> top rows, flux identity -> bottom rows
      // (Mueller); CBIE: k rows top, k_int rows bottom
      const int64_t r = (MULLER ? flux : interior) ? n + row : row;
      double cp = -1.0, cf = -1.0;  // coefficients of w_p (left block), w_f (right block)
      if (interior) {
        cp = (MULLER && flux) ? 1.0 / g : 1.0;
        cf = flux ? 1.0 : g;
      }
      for (int j = 0; j < kNyNodes; ++j) {
        const int64_t col = b + j;
        z2& L = A[r + col * lda];
        z2& R = A[r + (n + col) * lda];
        L = {L.x + cp * w[j].x, L.y + cp * w[j].y};
        R = {R.x + cf * w[kNyNodes + j].x, R.y + cf * w[kNyNodes + j].y};
      }
    }
  }
}

// ------------------------------------------------------------------ coupled regions
// Coupled fluid regions on the nodes (the reference's regions.jl:189-236 with its Nyström
// operators): the panel path's region block algebra -- for a target on surface si and a
// source on sj, every region the two surfaces share contributes its node operators at
// its wavenumber with its sign and density (RegionCoef) -- and the element corrections of
// each surface's own operators at the wavenumbers of its two sides.  Side 0 is the region
// outside a surface (its coupling entry with eq = 0), side 1 the region it encloses.

// The coupling entry of surface s with itself on `side` (eq = side).
__device__ __forceinline__ int self_entry(const RegionTable& RT, int s, int side) {
  const RegionCoef& C = RT.c[s * kMaxRegions + s];
  for (int q = 0; q < C.count; ++q)
    if (C.eq[q] == side) return q;
  return 0;
}

// Interpolant traces at the wavenumber of each node's side `side`.
__global__ void k_ny_traces_regions(NyInst I, int side) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= I.n) return;
  const RegionTable& RT = *I.region;
  const int s = I.surf[j];
  const double k = RT.kr[RT.c[s * kMaxRegions + s].kidx[self_entry(RT, s, side)]];
  const double* r = I.nodes + j * kPanelDoubles;
  z2* tr = reinterpret_cast<z2*>(side ? I.trace_i : I.trace);
  for (int t = 0; t < kNyBasis; ++t) {
    const double* d = I.dirs + 3 * t;
    const double ph = k * (d[0] * r[0] + d[1] * r[1] + d[2] * r[2]);
    const double kdn = k * (d[0] * r[3] + d[1] * r[4] + d[2] * r[5]);
    double sn, cs;
    sincos(ph, &sn, &cs);
    tr[(int64_t)t * I.n + j] = {cs, sn};
    tr[(int64_t)(kNyBasis + t) * I.n + j] = {-kdn * sn, kdn * cs};
  }
}

// Defect sums of one source node on side SIDE (slots with compile-time indices, so that
// the accumulators stay in registers).
template <bool MULLER, int SIDE>
__device__ __forceinline__ void ny_region_defects(z2* acc, z2 S, z2 D, z2 K, z2 H,
                                                  const z2 (*tr)[kNyTile], int jj) {
  constexpr int sd = MULLER ? 2 * SIDE : SIDE;
#pragma unroll
  for (int s = 0; s < kNyBasis; ++s) {
    const z2 u = tr[2 * kNyBasis * SIDE + s][jj];
    const z2 fl = tr[2 * kNyBasis * SIDE + kNyBasis + s][jj];
    zfma(acc[sd * kNyBasis + s], S, fl);
    zfms(acc[sd * kNyBasis + s], D, u);
    if (MULLER) {
      zfma(acc[(sd + 1) * kNyBasis + s], K, fl);
      zfms(acc[(sd + 1) * kNyBasis + s], H, u);
    }
  }
}

// Every node pair once (the layout of k_ny_assemble_fluid); defect slots: Mueller 2 side +
// (0 S/D, 1 K'/H), CBIE side.
template <bool MULLER>
__global__ void __launch_bounds__(kNyRows) k_ny_assemble_regions(NyInst I) {
  constexpr int ND = MULLER ? 4 : 2;
  const int64_t n = I.n, lda = 2 * I.n;
  const int64_t i = (int64_t)blockIdx.x * kNyRows + threadIdx.x;
  const int64_t c0 = (int64_t)blockIdx.y * I.chunk_cols;
  const int64_t c1 = min(n, c0 + I.chunk_cols);
  __shared__ double s_node[kNyTile][7];
  __shared__ z2 s_tr[4 * kNyBasis][kNyTile];  // u, du/dn on side 0, then on side 1
  __shared__ int32_t s_surf[kNyTile];
  const RegionTable& RT = *I.region;
  const bool row = i < n;
  double xi[3] = {0, 0, 0}, ni[3] = {0, 0, 0};
  int si = 0;
  if (row) {
    const double* r = I.nodes + i * kPanelDoubles;
    for (int d = 0; d < 3; ++d) {
      xi[d] = r[d];
      ni[d] = r[3 + d];
    }
    si = I.surf[i];
  }
  z2 acc[ND * kNyBasis];
#pragma unroll
  for (int t = 0; t < ND * kNyBasis; ++t) acc[t] = {0.0, 0.0};
  const z2* tr0 = reinterpret_cast<const z2*>(I.trace);
  const z2* tr1 = reinterpret_cast<const z2*>(I.trace_i);
  z2* A = reinterpret_cast<z2*>(I.A);
  for (int64_t t0 = c0; t0 < c1; t0 += kNyTile) {
    const int cnt = (int)min((int64_t)kNyTile, c1 - t0);
    __syncthreads();
    for (int e = threadIdx.x; e < kNyTile * 7; e += kNyRows) {
      const int jj = e / 7, f = e % 7;
      s_node[jj][f] = jj < cnt ? I.nodes[(t0 + jj) * kPanelDoubles + f] : 0.0;
    }
    for (int e = threadIdx.x; e < kNyTile * 4 * kNyBasis; e += kNyRows) {
      const int jj = e % kNyTile, t = e / kNyTile;
      const z2* src = t < 2 * kNyBasis ? tr0 : tr1;
      const int tt = t < 2 * kNyBasis ? t : t - 2 * kNyBasis;
      s_tr[t][jj] = jj < cnt ? src[(int64_t)tt * n + t0 + jj] : z2{0.0, 0.0};
    }
    for (int e = threadIdx.x; e < kNyTile; e += kNyRows) s_surf[e] = e < cnt ? I.surf[t0 + e] : 0;
    __syncthreads();
    if (!row) continue;
    for (int jj = 0; jj < cnt; ++jj) {
      const int64_t j = t0 + jj;
      z2 a11 = {0.0, 0.0}, a12 = {0.0, 0.0}, a21 = {0.0, 0.0}, a22 = {0.0, 0.0};
      if (j == i) {
        a11 = {MULLER ? 1.0 : 0.5, 0.0};
        a21 = {MULLER ? 0.0 : 0.5, 0.0};
        a22 = {MULLER ? 1.0 : 0.0, 0.0};
      } else {
        const int sj = s_surf[jj];
        const RegionCoef& C = RT.c[si * kMaxRegions + sj];
        const double dx = xi[0] - s_node[jj][0], dy = xi[1] - s_node[jj][1],
                     dz = xi[2] - s_node[jj][2];
        const double r = sqrt(dx * dx + dy * dy + dz * dz);
        const double ir = 1.0 / r;
        const double w = s_node[jj][6];
        const double dny = dx * s_node[jj][3] + dy * s_node[jj][4] + dz * s_node[jj][5];
        const double dnx = dx * ni[0] + dy * ni[1] + dz * ni[2];
        const double nn = ni[0] * s_node[jj][3] + ni[1] * s_node[jj][4] + ni[2] * s_node[jj][5];
        const double fd = -dny * ir * w, fk = dnx * ir * w;
        const double f2 = dnx * dny * ir * ir, f1 = nn * ir;
        for (int q = 0; q < C.count; ++q) {
          const double kk = RT.kr[C.kidx[q]];
          double sn, cs;
          sincos(kk * r, &sn, &cs);
          const double gs = kInv4Pi * ir;
          const z2 G = {cs * gs, sn * gs};
          const z2 G1 = zmul(G, z2{-ir, kk});
          const z2 S = {G.x * w, G.y * w};
          const z2 D = {G1.x * fd, G1.y * fd};
          z2 K = {0.0, 0.0}, H = {0.0, 0.0};
          if (MULLER) {
            const z2 G2 = zmul(G, z2{2.0 * ir * ir - kk * kk, -2.0 * kk * ir});
            K = {G1.x * fk, G1.y * fk};
            H = {-((G2.x - G1.x * ir) * f2 + G1.x * f1) * w,
                 -((G2.y - G1.y * ir) * f2 + G1.y * f1) * w};
          }
          const double sg = C.sign[q], rho = C.rho[q];
          if (MULLER) {
            a11 = {a11.x + sg * D.x, a11.y + sg * D.y};
            a12 = {a12.x - sg * rho * S.x, a12.y - sg * rho * S.y};
            a21 = {a21.x + sg / rho * H.x, a21.y + sg / rho * H.y};
            a22 = {a22.x - sg * K.x, a22.y - sg * K.y};
          } else if (C.eq[q] == 0) {
            a11 = {a11.x + sg * D.x, a11.y + sg * D.y};
            a12 = {a12.x - sg * rho * S.x, a12.y - sg * rho * S.y};
          } else {
            a21 = {a21.x + sg * D.x, a21.y + sg * D.y};
            a22 = {a22.x - sg * rho * S.x, a22.y - sg * rho * S.y};
          }
          if (sj == si) {  // the defects of surface si's identities on this side
            if (C.eq[q] == 0)
              ny_region_defects<MULLER, 0>(acc, S, D, K, H, s_tr, jj);
            else
              ny_region_defects<MULLER, 1>(acc, S, D, K, H, s_tr, jj);
          }
        }
      }
      A[i + j * lda] = a11;
      A[i + (n + j) * lda] = a12;
      A[(n + i) + j * lda] = a21;
      A[(n + i) + (n + j) * lda] = a22;
    }
  }
  if (!row) return;
  z2* part = reinterpret_cast<z2*>(I.part);
#pragma unroll
  for (int t = 0; t < ND * kNyBasis; ++t)
    part[((int64_t)blockIdx.y * ND * kNyBasis + t) * n + i] = acc[t];
}

// One thread per element: a fit per side; each defect's weights enter the blocks with the
// coefficients of the side's region for the surface with itself (sign sg, density rho):
//   S/D identity:  pressure weights x sg, flux weights x sg rho   (Mueller: top rows;
//                  CBIE: the side's equation rows)
//   K'/H identity: pressure weights x sg / rho, flux weights x sg (Mueller: bottom rows)
// which for one surface in the exterior are the coefficients of k_ny_correct_fluid.
template <bool MULLER>
__global__ void __launch_bounds__(kNyCorrT) k_ny_correct_regions(NyInst I) {
  constexpr int ND = MULLER ? 4 : 2;
  const int64_t e = (int64_t)blockIdx.x * kNyCorrT + threadIdx.x;
  const int64_t n = I.n, lda = 2 * I.n;
  if (e >= n / kNyNodes) return;
  const RegionTable& RT = *I.region;
  const z2* tr0 = reinterpret_cast<const z2*>(I.trace);
  const z2* tr1 = reinterpret_cast<const z2*>(I.trace_i);
  const z2* part = reinterpret_cast<const z2*>(I.part);
  z2* A = reinterpret_cast<z2*>(I.A);
  const int64_t b = e * kNyNodes;
  const int s = I.surf[b];
  const RegionCoef& C = RT.c[s * kMaxRegions + s];
  const int q0 = self_entry(RT, s, 0), q1 = self_entry(RT, s, 1);
  NyFit F0, F1;
  if (!ny_fit_factor(F0, tr0, n, b) || !ny_fit_factor(F1, tr1, n, b)) {
    I.status[e] = 1;
    return;
  }
  for (int t = 0; t < kNyNodes; ++t) {
    const int64_t row = b + t;
    for (int id = 0; id < ND; ++id) {
      const int side = MULLER ? (id >> 1) : id;
      const bool flux = MULLER && (id & 1);
      const z2* tr = side ? tr1 : tr0;
      z2 d[kNyBasis];
      for (int q = 0; q < kNyBasis; ++q) {
        z2 acc = {0.0, 0.0};
        for (int c = 0; c < I.n_chunks; ++c) {
          const z2 p = part[(((int64_t)c * ND + id) * kNyBasis + q) * n + row];
          acc.x += p.x;
          acc.y += p.y;
        }
        const z2 own = tr[(int64_t)((flux ? kNyBasis : 0) + q) * n + row];
        d[q] = {acc.x - 0.5 * own.x, acc.y - 0.5 * own.y};
      }
      z2 w[kNyFit];
      ny_fit_solve(side ? F1 : F0, d, w);
      const int qq = side ? q1 : q0;
      const double sg = C.sign[qq], rho = C.rho[qq];
      const int64_t r = (MULLER ? flux : side != 0) ? n + row : row;
      const double cp = flux ? sg / rho : sg, cf = flux ? sg : sg * rho;
      for (int j = 0; j < kNyNodes; ++j) {
        const int64_t col = b + j;
        z2& Lb = A[r + col * lda];
        z2& Rb = A[r + (n + col) * lda];
        Lb = {Lb.x + cp * w[j].x, Lb.y + cp * w[j].y};
        Rb = {Rb.x + cf * w[kNyNodes + j].x, Rb.y + cf * w[kNyNodes + j].y};
      }
    }
  }
}

// ------------------------------------------------------------------ compressed operators
template <typename R>
__global__ void k_ny_hm_diag(NyHm H) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= H.n) return;
  const int64_t o = H.dst[i * kNyNodes + (i % kNyNodes)];
  cx<R>* d1 = static_cast<cx<R>*>(H.D1);
  cx<R>* d2 = static_cast<cx<R>*>(H.D2);
  d1[o] = cx<R>{(R)0.5, (R)0};
  d2[o] = cx<R>{(R)(0.5 * H.a_re), (R)(0.5 * H.a_im)};
}

template <typename R>
__global__ void __launch_bounds__(kNyCorrT) k_ny_hm_correct(NyHm H) {
  const int64_t e = (int64_t)blockIdx.x * kNyCorrT + threadIdx.x;
  const int64_t n = H.n;
  if (e >= n / kNyNodes) return;
  const z2* tr = reinterpret_cast<const z2*>(H.trace);
  const z2* Y = reinterpret_cast<const z2*>(H.Y);
  cx<R>* d1 = static_cast<cx<R>*>(H.D1);
  cx<R>* d2 = static_cast<cx<R>*>(H.D2);
  const int64_t b = e * kNyNodes;
  NyFit F;
  if (!ny_fit_factor(F, tr, n, b)) {
    H.status[e] = 1;
    return;
  }
  const z2 al = {H.a_re, H.a_im};
  for (int t = 0; t < kNyNodes; ++t) {
    const int64_t row = b + t;
    const int64_t pr = H.iperm[row];
    z2 d[kNyBasis];
    for (int s = 0; s < kNyBasis; ++s) {
      const z2 y = Y[pr + (int64_t)s * n];
      const z2 u = tr[(int64_t)s * n + row], f = tr[(int64_t)(kNyBasis + s) * n + row];
      const z2 af = zmul(al, f);
      d[s] = {y.x - u.x - af.x, y.y - u.y - af.y};
    }
    z2 w[kNyFit];
    ny_fit_solve(F, d, w);
    for (int j = 0; j < kNyNodes; ++j) {
      const int64_t o = H.dst[row * kNyNodes + j];
      d1[o] = cx<R>{(R)((double)d1[o].x - w[j].x), (R)((double)d1[o].y - w[j].y)};
      d2[o] = cx<R>{(R)((double)d2[o].x - w[kNyNodes + j].x),
                    (R)((double)d2[o].y - w[kNyNodes + j].y)};
    }
  }
}

// ------------------------------------------------------------------ block preconditioner
// Gauss-Jordan inversion with partial pivoting of one element's block, FP64.
template <typename R>
__global__ void k_ny_prec_build(NyPrec P) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= P.n / kNyNodes) return;
  const cx<R>* D = static_cast<const cx<R>*>(P.D);
  z2 a[kNyNodes][2 * kNyNodes];
  for (int t = 0; t < kNyNodes; ++t)
    for (int j = 0; j < kNyNodes; ++j) {
      const cx<R> v = D[P.dst[(e * kNyNodes + t) * kNyNodes + j]];
      a[t][j] = {(double)v.x, (double)v.y};
      a[t][kNyNodes + j] = {t == j ? 1.0 : 0.0, 0.0};
    }
  for (int c = 0; c < kNyNodes; ++c) {
    int piv = c;
    double best = hypot(a[c][c].x, a[c][c].y);
    for (int t = c + 1; t < kNyNodes; ++t) {
      const double v = hypot(a[t][c].x, a[t][c].y);
      if (v > best) {
        best = v;
        piv = t;
      }
    }
    if (!(best > 0.0)) {
      P.status[e] = 1;
      return;
    }
    if (piv != c)
      for (int j = 0; j < 2 * kNyNodes; ++j) {
        const z2 tmp = a[c][j];
        a[c][j] = a[piv][j];
        a[piv][j] = tmp;
      }
    const z2 inv = zdiv(z2{1.0, 0.0}, a[c][c]);
    for (int j = 0; j < 2 * kNyNodes; ++j) a[c][j] = zmul(a[c][j], inv);
    for (int t = 0; t < kNyNodes; ++t) {
      if (t == c) continue;
      const z2 f = a[t][c];
      for (int j = 0; j < 2 * kNyNodes; ++j) zfms(a[t][j], f, a[c][j]);
    }
  }
  z2* out = reinterpret_cast<z2*>(P.Pinv) + e * kNyNodes * kNyNodes;
  for (int t = 0; t < kNyNodes; ++t)
    for (int j = 0; j < kNyNodes; ++j) out[t * kNyNodes + j] = a[t][kNyNodes + j];
}

// thread = (element, vector): the element's 7 entries gathered from their permuted
// positions, multiplied by its block inverse, scattered back
__global__ void k_ny_prec_apply(NyPrec P, const double* src, int64_t lds, const int32_t* jptr,
                                int64_t jstride, double* dst, int64_t ldd, int32_t nr) {
  const int64_t ne = P.n / kNyNodes;
  const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= ne * nr) return;
  const int64_t e = id % ne;
  const int r = (int)(id / ne);
  const z2* s = reinterpret_cast<const z2*>(src) + (int64_t)r * lds +
                (jptr ? (int64_t)(*jptr) * jstride : 0);
  z2* d = reinterpret_cast<z2*>(dst) + (int64_t)r * ldd;
  const z2* B = reinterpret_cast<const z2*>(P.Pinv) + e * kNyNodes * kNyNodes;
  z2 v[kNyNodes];
  for (int j = 0; j < kNyNodes; ++j) v[j] = s[P.iperm[e * kNyNodes + j]];
  for (int t = 0; t < kNyNodes; ++t) {
    z2 acc = {0.0, 0.0};
    for (int j = 0; j < kNyNodes; ++j) zfma(acc, B[t * kNyNodes + j], v[j]);
    d[P.iperm[e * kNyNodes + t]] = acc;
  }
}

// ------------------------------------------------------------------ Schwarz preconditioner
// Restricted additive Schwarz for the Burton-Miller node system, whose spectrum spreads as
// the mesh is refined (plain restarted GMRES needs about 300 steps at 320 panels, 640 at
// 1280 and more than 1200 at 5120): for every element e, the system restricted to the
// nodes of e's neighbourhood (its m nearest elements) is factored, and P^-1 r takes, for
// e's own seven nodes only, the neighbourhood solve of r (Cai and Sarkis, SIAM J. Sci.
// Comput. 21(2), 1999).  A one-level method (no coarse space): with 48 neighbours it cuts
// the steps eightfold at 1280 panels but stalls GMRES at 2304 and 5120 panels, so it is
// used only when asked for.  Entries between different elements are the uncorrected node
// kernel, evaluated in FP32 from the FP32 records; entries within an element are the
// corrected values of the full-block pool.  The local factorisation is FP32 as well: the
// preconditioner only steers GMRES, whose residual stays that of the true system.

// Uncorrected entry (i, j), i != j, of operator op (0: M1, 1: M2), FP32.
__device__ __forceinline__ float2 ny_entry_f32(const NyPrec& P, int64_t i, int64_t j) {
  const float* ri = P.recf + i * kPanelFloats;
  const float* rj = P.recf + j * kPanelFloats;
  const float dx = ri[0] - rj[0], dy = ri[1] - rj[1], dz = ri[2] - rj[2];
  const float r = sqrtf(dx * dx + dy * dy + dz * dz);
  const float ir = 1.0f / r;
  float sn, cs;
  sincosf(P.k * r, &sn, &cs);
  const float w = rj[6];
  const float gs = 0.07957747154594767f * ir;
  const float Gx = cs * gs, Gy = sn * gs;
  // G1 = G (-1/r + i k)
  const float G1x = -Gx * ir - Gy * P.k, G1y = Gx * P.k - Gy * ir;
  const float dny = dx * rj[3] + dy * rj[4] + dz * rj[5];
  const float dnx = dx * ri[3] + dy * ri[4] + dz * ri[5];
  if (P.op == 0) {  // M1 = -D - alpha H
    // G2 = G ((2/r^2 - k^2) - 2 i k / r)
    const float ar = 2.0f * ir * ir - P.k * P.k, ai = -2.0f * P.k * ir;
    const float G2x = Gx * ar - Gy * ai, G2y = Gx * ai + Gy * ar;
    const float nn = ri[3] * rj[3] + ri[4] * rj[4] + ri[5] * rj[5];
    const float fd = -dny * ir * w;
    const float f2 = dnx * dny * ir * ir, f1 = nn * ir;
    const float Hx = -((G2x - G1x * ir) * f2 + G1x * f1) * w;
    const float Hy = -((G2y - G1y * ir) * f2 + G1y * f1) * w;
    return make_float2(-G1x * fd - (P.a_re * Hx - P.a_im * Hy),
                       -G1y * fd - (P.a_re * Hy + P.a_im * Hx));
  }
  const float fk = dnx * ir * w;  // M2 = S + alpha K'
  const float Kx = G1x * fk, Ky = G1y * fk;
  return make_float2(Gx * w + (P.a_re * Kx - P.a_im * Ky), Gy * w + (P.a_re * Ky + P.a_im * Kx));
}

__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// One CTA per element: T = (the neighbourhood system)^T with the seven unit columns of
// e's own nodes appended, Gaussian elimination with partial pivoting (rows by |re| + |im|,
// first maximum), back substitution; W[t][q] = X[q][t].  T is column-major (L rows, L + 7
// columns) in the CTA's workspace slot.
constexpr int kRasT = 256;
template <typename R>
__global__ void __launch_bounds__(kRasT) k_ny_ras_build(NyPrec P, int64_t e0) {
  const int64_t e = e0 + blockIdx.x;
  const int32_t b0 = P.nb_ptr[e], m = P.nb_ptr[e + 1] - b0;
  const int L = kNyNodes * m;
  float2* T = reinterpret_cast<float2*>(P.work + (int64_t)blockIdx.x * P.work_stride);
  const cx<R>* D = static_cast<const cx<R>*>(P.D);
  auto node = [&](int q) -> int64_t {
    return (int64_t)P.nb_el[b0 + q / kNyNodes] * kNyNodes + q % kNyNodes;
  };
  // T(a, b) = A(node b, node a)
  for (int64_t idx = threadIdx.x; idx < (int64_t)L * L; idx += kRasT) {
    const int a = (int)(idx % L), b = (int)(idx / L);
    const int64_t i = node(b), j = node(a);
    float2 v;
    if (i / kNyNodes == j / kNyNodes) {
      const cx<R> d = D[P.dst[i * kNyNodes + j % kNyNodes]];
      v = make_float2((float)d.x, (float)d.y);
    } else {
      v = ny_entry_f32(P, i, j);
    }
    T[a + (int64_t)b * L] = v;
  }
  for (int idx = threadIdx.x; idx < L * kNyNodes; idx += kRasT) {
    const int a = idx % L, t = idx / L;
    T[a + (int64_t)(L + t) * L] = make_float2(a == t ? 1.0f : 0.0f, 0.0f);
  }
  __shared__ float s_val[kRasT / 32];
  __shared__ int s_idx[kRasT / 32];
  __shared__ int s_piv;
  __shared__ float2 s_x[kNyNodes];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int ncol = L + kNyNodes;
  for (int c = 0; c < L; ++c) {
    __syncthreads();
    // pivot: first row of maximal |re| + |im| in column c, rows c..L-1
    float bv = -1.0f;
    int bi = INT_MAX;
    for (int a = c + threadIdx.x; a < L; a += kRasT) {
      const float2 v = T[a + (int64_t)c * L];
      const float mag = fabsf(v.x) + fabsf(v.y);
      if (mag > bv || (mag == bv && a < bi)) {
        bv = mag;
        bi = a;
      }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      const float ov = __shfl_down_sync(0xffffffffu, bv, off);
      const int oi = __shfl_down_sync(0xffffffffu, bi, off);
      if (ov > bv || (ov == bv && oi < bi)) {
        bv = ov;
        bi = oi;
      }
    }
    if (lane == 0) {
      s_val[w] = bv;
      s_idx[w] = bi;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      float v = s_val[0];
      int id = s_idx[0];
      for (int q = 1; q < kRasT / 32; ++q)
        if (s_val[q] > v || (s_val[q] == v && s_idx[q] < id)) {
          v = s_val[q];
          id = s_idx[q];
        }
      s_piv = (v > 0.0f) ? id : -1;
      if (v <= 0.0f) P.status[e] = 1;
    }
    __syncthreads();
    const int p = s_piv;
    if (p < 0) return;  // every thread leaves: the neighbourhood system is singular
    if (p != c)
      for (int b = c + threadIdx.x; b < ncol; b += kRasT) {
        const float2 t0 = T[c + (int64_t)b * L];
        T[c + (int64_t)b * L] = T[p + (int64_t)b * L];
        T[p + (int64_t)b * L] = t0;
      }
    __syncthreads();
    const float2 piv = T[c + (int64_t)c * L];
    const float dd = piv.x * piv.x + piv.y * piv.y;
    const float2 inv = make_float2(piv.x / dd, -piv.y / dd);
    for (int a = c + 1 + threadIdx.x; a < L; a += kRasT)
      T[a + (int64_t)c * L] = cmulf(T[a + (int64_t)c * L], inv);
    __syncthreads();
    const int rows = L - c - 1;
    if (rows > 0) {
      const int64_t cnt = (int64_t)rows * (ncol - c - 1);
      for (int64_t idx = threadIdx.x; idx < cnt; idx += kRasT) {
        const int a = c + 1 + (int)(idx % rows);
        const int b = c + 1 + (int)(idx / rows);
        const float2 l = T[a + (int64_t)c * L], u = T[c + (int64_t)b * L];
        float2& t = T[a + (int64_t)b * L];
        t.x -= l.x * u.x - l.y * u.y;
        t.y -= l.x * u.y + l.y * u.x;
      }
    }
  }
  // back substitution with U for the seven right-hand sides
  for (int a = L - 1; a >= 0; --a) {
    __syncthreads();
    if (threadIdx.x < kNyNodes) {
      const float2 d = T[a + (int64_t)a * L];
      const float dd = d.x * d.x + d.y * d.y;
      const float2 y = T[a + (int64_t)(L + threadIdx.x) * L];
      const float2 x = cmulf(y, make_float2(d.x / dd, -d.y / dd));
      T[a + (int64_t)(L + threadIdx.x) * L] = x;
      s_x[threadIdx.x] = x;
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < a * kNyNodes; idx += kRasT) {
      const int j = idx % a, t = idx / a;
      const float2 u = T[j + (int64_t)a * L];
      float2& y = T[j + (int64_t)(L + t) * L];
      const float2 x = s_x[t];
      y.x -= u.x * x.x - u.y * x.y;
      y.y -= u.x * x.y + u.y * x.x;
    }
  }
  __syncthreads();
  float2* W = reinterpret_cast<float2*>(P.W) + P.woff[e];
  for (int idx = threadIdx.x; idx < kNyNodes * L; idx += kRasT) {
    const int t = idx / L, q = idx % L;
    W[idx] = T[q + (int64_t)(L + t) * L];
  }
}

// warp = (element, vector): the neighbourhood's L entries gathered from their permuted
// positions, the seven own-node rows of W applied, the results written at the own nodes
__global__ void k_ny_ras_apply(NyPrec P, const double* src, int64_t lds, const int32_t* jptr,
                               int64_t jstride, double* dst, int64_t ldd, int32_t nr) {
  const int64_t ne = P.n / kNyNodes;
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (gw >= ne * nr) return;
  const int64_t e = gw % ne;
  const int r = (int)(gw / ne);
  const z2* s = reinterpret_cast<const z2*>(src) + (int64_t)r * lds +
                (jptr ? (int64_t)(*jptr) * jstride : 0);
  z2* d = reinterpret_cast<z2*>(dst) + (int64_t)r * ldd;
  const int32_t b0 = P.nb_ptr[e], m = P.nb_ptr[e + 1] - b0;
  const int L = kNyNodes * m;
  const float2* W = reinterpret_cast<const float2*>(P.W) + P.woff[e];
  z2 acc[kNyNodes];
#pragma unroll
  for (int t = 0; t < kNyNodes; ++t) acc[t] = {0.0, 0.0};
  for (int q = lane; q < L; q += 32) {
    const int64_t node = (int64_t)P.nb_el[b0 + q / kNyNodes] * kNyNodes + q % kNyNodes;
    const z2 v = s[P.iperm[node]];
#pragma unroll
    for (int t = 0; t < kNyNodes; ++t) {
      const float2 wv = W[(int64_t)t * L + q];
      zfma(acc[t], z2{(double)wv.x, (double)wv.y}, v);
    }
  }
#pragma unroll
  for (int t = 0; t < kNyNodes; ++t)
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      acc[t].x += __shfl_down_sync(0xffffffffu, acc[t].x, off);
      acc[t].y += __shfl_down_sync(0xffffffffu, acc[t].y, off);
    }
  if (lane == 0)
    for (int t = 0; t < kNyNodes; ++t) d[P.iperm[e * kNyNodes + t]] = acc[t];
}

// ------------------------------------------------------------------ point evaluation
// Field at a point, one CTA per point, in the form the reference uses for point
// evaluation (fields/pressure.jl:448-467 through quadrature/fluid.jl:94-163 with
// exclude_nearest=true): the element of the nearest node is left out of the node sum and
// its contribution recovered from the fit of the interpolants' defect
//   mult u(x) + S_excl du/dn - D_excl u,   mult 0 outside the body, -1 inside.
// Outside: u_s(x) = sum_j w_j [dG/dn_y p_j - G q_j] (scattered traces, k), the element
// adding sum_{j in e} (w_p,j p_j + w_f,j q_j).  Inside a fluid body: u_i(x) = sum_j w_j
// [G g (q_j + q_inc,j) - dG/dn_y (p_j + p_inc,j)] at k_int, the element adding
// -sum_{j in e} (w_f,j g (q + q_inc)_j + w_p,j (p + p_inc)_j).  Point classes as the
// panel kernel: surface points are exterior for rigid/soft bodies, interior for fluids.
constexpr int kNyPtT = 256;
constexpr int kNyPtSums = 2 * (1 + kNyBasis);  // field + nine defects, complex

__global__ void __launch_bounds__(kNyPtT) k_ny_pressure(NyPoints P) {
  const int64_t ip = blockIdx.x;
  if (ip >= P.npts) return;
  const int32_t reg = P.region[ip];
  const bool interior = reg == 1 || (reg == 2 && P.fluid);
  if ((interior && !P.fluid) || (P.field == 3 && !interior) || (P.field == 1 && interior)) {
    if (threadIdx.x == 0) {  // no such field at this point: NaN marks it for the host
      P.out[2 * ip] = NAN;
      P.out[2 * ip + 1] = NAN;
    }
    return;
  }
  const int64_t n = P.n;
  const double x[3] = {P.points[3 * ip], P.points[3 * ip + 1], P.points[3 * ip + 2]};
  __shared__ double s_d[kNyPtT];
  __shared__ int64_t s_i[kNyPtT];
  __shared__ double s_sum[kNyPtT / 32][kNyPtSums];
  // nearest node (smallest index among equal distances)
  double best = INFINITY;
  int64_t bi = INT64_MAX;
  for (int64_t j = threadIdx.x; j < n; j += kNyPtT) {
    const double* r = P.nodes + j * kPanelDoubles;
    const double dx = x[0] - r[0], dy = x[1] - r[1], dz = x[2] - r[2];
    const double d2 = dx * dx + dy * dy + dz * dz;
    if (d2 < best) {
      best = d2;
      bi = j;
    }
  }
  s_d[threadIdx.x] = best;
  s_i[threadIdx.x] = bi;
  __syncthreads();
  for (int h = kNyPtT / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) {
      const double od = s_d[threadIdx.x + h];
      const int64_t oi = s_i[threadIdx.x + h];
      if (od < s_d[threadIdx.x] || (od == s_d[threadIdx.x] && oi < s_i[threadIdx.x])) {
        s_d[threadIdx.x] = od;
        s_i[threadIdx.x] = oi;
      }
    }
    __syncthreads();
  }
  const int64_t b = (s_i[0] / kNyNodes) * kNyNodes;
  const z2* tr = reinterpret_cast<const z2*>(interior ? P.trace_i : P.trace);
  const z2* ps = reinterpret_cast<const z2*>(P.p);
  const z2* qs = reinterpret_cast<const z2*>(P.q);
  const double k = interior ? P.k_int : P.k;
  const double ke = P.k, g = P.g;
  // interior densities: total traces p + p_inc and g (q + q_inc)
  auto dens = [&](int64_t j, z2& pj, z2& qj) {
    pj = ps[j];
    qj = qs[j];
    if (interior) {
      const double* r = P.nodes + j * kPanelDoubles;
      const double ph = ke * (P.dir[0] * r[0] + P.dir[1] * r[1] + P.dir[2] * r[2]);
      const double dn = ke * (P.dir[0] * r[3] + P.dir[1] * r[4] + P.dir[2] * r[5]);
      double sn, cs;
      sincos(ph, &sn, &cs);
      pj = {pj.x + cs, pj.y + sn};
      qj = {g * (qj.x - dn * sn), g * (qj.y + dn * cs)};
    }
  };
  z2 acc[1 + kNyBasis];
#pragma unroll
  for (int t = 0; t <= kNyBasis; ++t) acc[t] = {0.0, 0.0};
  for (int64_t j = threadIdx.x; j < n; j += kNyPtT) {
    if (j >= b && j < b + kNyNodes) continue;
    const double* r = P.nodes + j * kPanelDoubles;
    const double dx = x[0] - r[0], dy = x[1] - r[1], dz = x[2] - r[2];
    const double r2 = dx * dx + dy * dy + dz * dz;
    const double rr = sqrt(r2), ir = 1.0 / rr;
    double sn, cs;
    sincos(k * rr, &sn, &cs);
    const double w = r[6];
    const double gs = kInv4Pi * ir;
    const z2 G = {cs * gs, sn * gs};
    const z2 G1 = zmul(G, z2{-ir, k});
    const double fd = -(dx * r[3] + dy * r[4] + dz * r[5]) * ir * w;
    const z2 S = {G.x * w, G.y * w};
    const z2 D = {G1.x * fd, G1.y * fd};
    z2 pj, qj;
    dens(j, pj, qj);
    if (interior) {
      zfma(acc[0], S, qj);
      zfms(acc[0], D, pj);
    } else {
      zfma(acc[0], D, pj);
      zfms(acc[0], S, qj);
    }
#pragma unroll
    for (int s = 0; s < kNyBasis; ++s) {
      zfma(acc[1 + s], S, tr[(int64_t)(kNyBasis + s) * n + j]);
      zfms(acc[1 + s], D, tr[(int64_t)s * n + j]);
    }
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int t = 0; t <= kNyBasis; ++t) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      acc[t].x += __shfl_down_sync(0xffffffffu, acc[t].x, off);
      acc[t].y += __shfl_down_sync(0xffffffffu, acc[t].y, off);
    }
    if (lane == 0) {
      s_sum[wid][2 * t] = acc[t].x;
      s_sum[wid][2 * t + 1] = acc[t].y;
    }
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  z2 tot[1 + kNyBasis];
  for (int t = 0; t <= kNyBasis; ++t) {
    tot[t] = {0.0, 0.0};
    for (int gq = 0; gq < kNyPtT / 32; ++gq) {
      tot[t].x += s_sum[gq][2 * t];
      tot[t].y += s_sum[gq][2 * t + 1];
    }
  }
  if (interior) {  // multiplier -1: the interpolants' values at x
    for (int s = 0; s < kNyBasis; ++s) {
      const double* d = P.dirs + 3 * s;
      double sn, cs;
      sincos(k * (d[0] * x[0] + d[1] * x[1] + d[2] * x[2]), &sn, &cs);
      tot[1 + s] = {tot[1 + s].x - cs, tot[1 + s].y - sn};
    }
  }
  z2 field = tot[0];
  NyFit F;
  if (ny_fit_factor(F, tr, n, b)) {
    z2 w[kNyFit];
    ny_fit_solve(F, tot + 1, w);
    const double sg = interior ? -1.0 : 1.0;
    for (int j = 0; j < kNyNodes; ++j) {
      z2 pj, qj;
      dens(b + j, pj, qj);
      const z2 wp = {sg * w[j].x, sg * w[j].y};
      const z2 wf = {sg * w[kNyNodes + j].x, sg * w[kNyNodes + j].y};
      zfma(field, wp, pj);
      zfma(field, wf, qj);
    }
  } else {  // rank-deficient fit
    P.status[ip] = 1;
  }
  if (P.field == 0 && !interior) {  // total outside: the incident value is already in out
    field.x += P.out[2 * ip];
    field.y += P.out[2 * ip + 1];
  }
  P.out[2 * ip] = field.x;
  P.out[2 * ip + 1] = field.y;
}

}  // namespace

int32_t nystrom_defects(int32_t fluid) {
  return (fluid == 1 || fluid == 3) ? 4 : (fluid == 2 || fluid == 4) ? 2 : 1;
}

int64_t nystrom_scratch_doubles(int64_t n, int32_t n_chunks, int32_t fluid) {
  const int64_t traces = (fluid ? 2 : 1) * 2 * (2 * (int64_t)kNyBasis * n);
  return traces + 2 * ((int64_t)n_chunks * nystrom_defects(fluid) * kNyBasis * n);
}

// About four waves of resident CTAs (152 SMs x 5 CTAs of 96-register threads), so the
// last, partial wave is a small share; ranges a whole number of tiles wide.
int32_t nystrom_chunks(int64_t n) {
  const int64_t rb = (n + kNyRows - 1) / kNyRows;
  const int64_t want = std::min<int64_t>(64, std::max<int64_t>(1, (152 * 5 * 4 + rb - 1) / rb));
  const int64_t per = ((n + want - 1) / want + kNyTile - 1) / kNyTile * kNyTile;
  return (int32_t)std::max<int64_t>(1, (n + per - 1) / per);
}

void launch_nystrom_pressure(const Launch& L, const NyInst& traces, const NyPoints& P) {
  k_ny_traces<<<(unsigned)((traces.n + 127) / 128), 128, 0, L.stream>>>(traces);
  count_launch(1);
  if (P.npts > 0) {
    k_ny_pressure<<<(unsigned)P.npts, kNyPtT, 0, L.stream>>>(P);
    count_launch(1);
  }
}

void launch_nystrom_prec_build(const Launch& L, const NyPrec& P) {
  const int64_t ne = P.n / kNyNodes;
  const unsigned g = (unsigned)((ne + 127) / 128);
  if (P.f32)
    k_ny_prec_build<float><<<g, 128, 0, L.stream>>>(P);
  else
    k_ny_prec_build<double><<<g, 128, 0, L.stream>>>(P);
  count_launch(1);
}

void launch_nystrom_ras_build(const Launch& L, const NyPrec& P, int64_t e0, int64_t count,
                              int32_t max_len) {
  (void)max_len;
  if (count <= 0) return;
  if (P.f32)
    k_ny_ras_build<float><<<(unsigned)count, kRasT, 0, L.stream>>>(P, e0);
  else
    k_ny_ras_build<double><<<(unsigned)count, kRasT, 0, L.stream>>>(P, e0);
  count_launch(1);
}

void launch_nystrom_prec_apply(const Launch& L, const NyPrec& P, const double* src, int64_t lds,
                               const int32_t* jptr, int64_t jstride, double* dst, int64_t ldd,
                               int32_t nr) {
  if (P.ras) {
    const int64_t warps = P.n / kNyNodes * nr;
    k_ny_ras_apply<<<(unsigned)((warps * 32 + 127) / 128), 128, 0, L.stream>>>(
        P, src, lds, jptr, jstride, dst, ldd, nr);
    count_launch(1);
    return;
  }
  const int64_t total = P.n / kNyNodes * nr;
  k_ny_prec_apply<<<(unsigned)((total + 127) / 128), 128, 0, L.stream>>>(P, src, lds, jptr,
                                                                          jstride, dst, ldd, nr);
  count_launch(1);
}

void launch_nystrom_hm_diag(const Launch& L, const NyHm& H) {
  const unsigned g = (unsigned)((H.n + 255) / 256);
  if (H.f32)
    k_ny_hm_diag<float><<<g, 256, 0, L.stream>>>(H);
  else
    k_ny_hm_diag<double><<<g, 256, 0, L.stream>>>(H);
  count_launch(1);
}

void launch_nystrom_hm_correct(const Launch& L, const NyHm& H) {
  const int64_t ne = H.n / kNyNodes;
  const unsigned g = (unsigned)((ne + kNyCorrT - 1) / kNyCorrT);
  if (H.f32)
    k_ny_hm_correct<float><<<g, kNyCorrT, 0, L.stream>>>(H);
  else
    k_ny_hm_correct<double><<<g, kNyCorrT, 0, L.stream>>>(H);
  count_launch(1);
}

void launch_nystrom(const Launch& L, const NyInst& I0) {
  NyInst I = I0;
  const int64_t per = (I.n + I.n_chunks - 1) / I.n_chunks;
  I.chunk_cols = (per + kNyTile - 1) / kNyTile * kNyTile;
  const unsigned tb = (unsigned)((I.n + 127) / 128);
  if (I.fluid >= 3) {  // coupled regions: traces on both sides, region kernels
    k_ny_traces_regions<<<tb, 128, 0, L.stream>>>(I, 0);
    k_ny_traces_regions<<<tb, 128, 0, L.stream>>>(I, 1);
    dim3 grid((unsigned)((I.n + kNyRows - 1) / kNyRows), (unsigned)I.n_chunks);
    const unsigned cb = (unsigned)((I.n / kNyNodes + kNyCorrT - 1) / kNyCorrT);
    if (I.fluid == 3) {
      k_ny_assemble_regions<true><<<grid, kNyRows, 0, L.stream>>>(I);
      k_ny_correct_regions<true><<<cb, kNyCorrT, 0, L.stream>>>(I);
    } else {
      k_ny_assemble_regions<false><<<grid, kNyRows, 0, L.stream>>>(I);
      k_ny_correct_regions<false><<<cb, kNyCorrT, 0, L.stream>>>(I);
    }
    count_launch(4);
    return;
  }
  k_ny_traces<<<tb, 128, 0, L.stream>>>(I);
  count_launch(1);
  if (I.fluid) {  // the interior wavenumber's traces
    NyInst J = I;
    J.k = I.k_int;
    J.trace = I.trace_i;
    k_ny_traces<<<tb, 128, 0, L.stream>>>(J);
    count_launch(1);
  }
  dim3 grid((unsigned)((I.n + kNyRows - 1) / kNyRows), (unsigned)I.n_chunks);
  const int64_t ne = I.n / kNyNodes;
  const unsigned cb = (unsigned)((ne + kNyCorrT - 1) / kNyCorrT);
  if (I.fluid == 1) {
    k_ny_assemble_fluid<true><<<grid, kNyRows, 0, L.stream>>>(I);
    k_ny_correct_fluid<true><<<cb, kNyCorrT, 0, L.stream>>>(I);
  } else if (I.fluid == 2) {
    k_ny_assemble_fluid<false><<<grid, kNyRows, 0, L.stream>>>(I);
    k_ny_correct_fluid<false><<<cb, kNyCorrT, 0, L.stream>>>(I);
  } else {
    k_ny_assemble<<<grid, kNyRows, 0, L.stream>>>(I);
    k_ny_correct<<<cb, kNyCorrT, 0, L.stream>>>(I);
  }
  count_launch(2);
}

}  // namespace bemgpu
