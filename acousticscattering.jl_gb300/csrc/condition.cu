// 2-norm condition numbers of small systems: the reference's factor diagnostics
// condition_number = cond(A) and scaled_condition_number = cond(D_r^-1 A D_c^-1), computed
// by an SVD when the order is at most condition_limit (solvers/bem/full.jl:364-409).
//
// Singular values by one-sided (Hestenes) Jacobi in FP64: sweeps of round-robin rounds,
// each round rotating n/2 disjoint column pairs (one CTA per pair) so that the pair
// becomes orthogonal; the singular values are the final column norms.  The 2 x 2 step
// writes the pair's Gram matrix [a g; conj(g) b] (g = x^H y) as D [a |g|; |g| b] D^H with
// D = diag(1, e^{i arg g}) and diagonalises the real part by the symmetric Schur rotation
// (Golub & Van Loan, Matrix Computations, section 8.5): x' = c x - s e y, y' = s x + c e y,
// e = conj(g) / |g|.  Sums run in a fixed order, so the values do not depend on the batch.
#include "bemgpu_internal.h"
#include "condition.cuh"

#include <algorithm>

namespace bemgpu {

constexpr int kSvdThreads = 256;

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// Column pair (p, q) of round r among m (even) columns: the circle method (column m - 1
// stays, the others rotate), so every pair meets once in m - 1 rounds.
__device__ __forceinline__ void round_pair(int64_t m, int64_t r, int64_t k, int64_t* p,
                                           int64_t* q) {
  const int64_t mm = m - 1;
  if (k == 0) {
    *p = r % mm;
    *q = mm;
  } else {
    *p = (r + k) % mm;
    *q = (r - k + mm) % mm;
  }
}

__global__ void __launch_bounds__(kSvdThreads) k_jacobi_round(const SvdInst* __restrict__ insts,
                                                              int64_t r, double tol) {
  const SvdInst& S = insts[blockIdx.y];
  const int64_t n = S.n, m = (n + 1) & ~int64_t(1);
  if (r >= m - 1 || (int64_t)blockIdx.x >= m / 2) return;
  int64_t p, q;
  round_pair(m, r, blockIdx.x, &p, &q);
  if (p >= n || q >= n) return;  // the padding column of an odd order
  double2* x = S.a + p * S.lda;
  double2* y = S.a + q * S.lda;
  double a = 0.0, b = 0.0, gr = 0.0, gi = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += kSvdThreads) {
    const double2 u = x[i], v = y[i];
    a += u.x * u.x + u.y * u.y;
    b += v.x * v.x + v.y * v.y;
    gr += u.x * v.x + u.y * v.y;  // conj(u) v
    gi += u.x * v.y - u.y * v.x;
  }
  __shared__ double red[4][kSvdThreads / 32];
  __shared__ double rot[4];  // c, s, e (re, im); c = 2 for "no rotation"
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, off);
    b += __shfl_down_sync(0xffffffffu, b, off);
    gr += __shfl_down_sync(0xffffffffu, gr, off);
    gi += __shfl_down_sync(0xffffffffu, gi, off);
  }
  if (lane == 0) {
    red[0][w] = a;
    red[1][w] = b;
    red[2][w] = gr;
    red[3][w] = gi;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    a = b = gr = gi = 0.0;
    for (int k = 0; k < kSvdThreads / 32; ++k) {
      a += red[0][k];
      b += red[1][k];
      gr += red[2][k];
      gi += red[3][k];
    }
    const double g = hypot(gr, gi);
    if (g > tol * sqrt(a) * sqrt(b) && g > 0.0) {
      const double zeta = (b - a) / (2.0 * g);
      const double t = copysign(1.0, zeta) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
      const double c = 1.0 / sqrt(1.0 + t * t), s = c * t;
      rot[0] = c;
      rot[1] = s;
      rot[2] = gr / g;  // e = conj(g) / |g|
      rot[3] = -gi / g;
      *S.rotated = 1;
    } else {
      rot[0] = 2.0;
    }
  }
  __syncthreads();
  const double c = rot[0];
  if (c > 1.5) return;
  const double s = rot[1];
  const double2 se = make_double2(s * rot[2], s * rot[3]), ce = make_double2(c * rot[2], c * rot[3]);
  for (int64_t i = threadIdx.x; i < n; i += kSvdThreads) {
    const double2 u = x[i], v = y[i];
    const double2 sev = cmul(se, v), cev = cmul(ce, v);
    x[i] = make_double2(c * u.x - sev.x, c * u.y - sev.y);
    y[i] = make_double2(s * u.x + cev.x, s * u.y + cev.y);
  }
}

// sigma[j] = ||column j|| (fixed-order block sum)
__global__ void __launch_bounds__(kSvdThreads) k_column_norms(const SvdInst* __restrict__ insts) {
  const SvdInst& S = insts[blockIdx.y];
  const int64_t j = blockIdx.x;
  if (j >= S.n) return;
  const double2* x = S.a + j * S.lda;
  double a = 0.0;
  for (int64_t i = threadIdx.x; i < S.n; i += kSvdThreads) a += x[i].x * x[i].x + x[i].y * x[i].y;
  __shared__ double red[kSvdThreads / 32];
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) a += __shfl_down_sync(0xffffffffu, a, off);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = a;
  __syncthreads();
  if (threadIdx.x == 0) {
    a = 0.0;
    for (int k = 0; k < kSvdThreads / 32; ++k) a += red[k];
    S.sigma[j] = sqrt(a);
  }
}

// a_ij /= rows_i * cols_j (the equilibrated copy), in place; a grid-stride loop over the
// entries of each instance (blockIdx.y)
__global__ void k_svd_scale(const SvdInst* __restrict__ insts) {
  const SvdInst& S = insts[blockIdx.y];
  if (!S.rows) return;
  const int64_t total = S.n * S.n;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e % S.n, j = e / S.n;
    const double d = S.rows[i] * S.cols[j];
    double2& v = S.a[i + j * S.lda];
    v = make_double2(v.x / d, v.y / d);
  }
}

void launch_svd_scale(const Launch& L, const SvdInst* d, int ninst, int64_t nmax) {
  const int64_t blocks = std::min<int64_t>((nmax * nmax + 255) / 256, 4096);
  k_svd_scale<<<dim3((unsigned)blocks, (unsigned)ninst), 256, 0, L.stream>>>(d);
  count_launch(1);
}

void launch_jacobi_round(const Launch& L, const SvdInst* d, int ninst, int64_t nmax, int64_t r,
                         double tol) {
  const int64_t m = (nmax + 1) & ~int64_t(1);
  k_jacobi_round<<<dim3((unsigned)(m / 2), (unsigned)ninst), kSvdThreads, 0, L.stream>>>(d, r,
                                                                                         tol);
  count_launch(1);
}

void launch_column_norms(const Launch& L, const SvdInst* d, int ninst, int64_t nmax) {
  k_column_norms<<<dim3((unsigned)nmax, (unsigned)ninst), kSvdThreads, 0, L.stream>>>(d);
  count_launch(1);
}

}  // namespace bemgpu
