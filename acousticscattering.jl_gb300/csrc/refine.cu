// Matrix-vector work around the factorisation: equilibration (solvers/bem/full.jl:388-394,
// solvers/bem/fluid_system.jl:202-216), scaled low-precision copies, products with the
// complex128 system (right-hand sides, residuals, componentwise denominators), the
// backward-error statistics of fluid_system.jl:241-262 and the correction steps of
// fluid_system.jl:229-239.
//
// Column-major matrices are swept with one thread per row (consecutive threads read
// consecutive rows of a column: coalesced), and the columns are split into kChunks
// chunks whose partial results are combined by a second kernel in a fixed order, so
// every reduction here is deterministic.
#include <cfloat>
#include <cmath>

#include "bemgpu_internal.h"
#include "linalg.cuh"
#include "refine.cuh"

namespace bemgpu {

__device__ __forceinline__ cd ldc(const void* base, int64_t idx) {
  double2 v = reinterpret_cast<const double2*>(base)[idx];
  return {v.x, v.y};
}
__device__ __forceinline__ void stc(void* base, int64_t idx, cd v) {
  reinterpret_cast<double2*>(base)[idx] = make_double2(v.x, v.y);
}
__device__ __forceinline__ double cabs(cd a) { return hypot(a.x, a.y); }
// Magnitude for scales, norms and componentwise denominators: single precision is
// ample there (relative 1e-7), and GB300 issues FP64 at a small fraction of FP32.
__device__ __forceinline__ float fabs_c(cd a) {
  const float x = (float)a.x, y = (float)a.y;
  return sqrtf(fmaf(x, x, y * y));
}

__device__ __forceinline__ void chunk_range(int64_t n, int ch, int nch, int64_t* j0, int64_t* j1) {
  int64_t w = (n + nch - 1) / nch;
  *j0 = min(n, (int64_t)ch * w);
  *j1 = min(n, *j0 + w);
}

// ---------------------------------------------------------------- equilibration
__global__ void k_rowstats(const VecInst* __restrict__ insts) {
  const VecInst& V = insts[blockIdx.z];
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= V.n) return;
  int64_t j0, j1;
  chunk_range(V.n, blockIdx.y, kChunks, &j0, &j1);
  float mx = 0.f;
  double sm = 0.0;
  float sm32 = 0.f;
  int cnt = 0;
  for (int64_t j = j0; j < j1; ++j) {
    float a = fabs_c(ldc(V.A, i + j * V.lda));
    mx = fmaxf(mx, a);
    sm32 += a;
    if (++cnt == 256) {  // fold into FP64 every 256 terms
      sm += sm32;
      sm32 = 0.f;
      cnt = 0;
    }
  }
  sm += sm32;
  V.part[2 * (blockIdx.y * V.n + i)] = mx;
  V.part[2 * (blockIdx.y * V.n + i) + 1] = sm;
}

__global__ void k_rowstats_finish(const VecInst* __restrict__ insts) {
  const VecInst& V = insts[blockIdx.y];
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= V.n) return;
  double mx = 0.0, sm = 0.0;
  for (int c = 0; c < kChunks; ++c) {
    mx = fmax(mx, V.part[2 * (c * V.n + i)]);
    sm += V.part[2 * (c * V.n + i) + 1];
  }
  V.rows[i] = (mx == 0.0) ? 1.0 : mx;
  V.rows_inv[i] = (float)(1.0 / V.rows[i]);
  V.rowsum[i] = sm;
}

// columns[j] = max_i |A_ij / rows_i|, one warp per column
__global__ void k_colmax(const VecInst* __restrict__ insts) {
  const VecInst& V = insts[blockIdx.y];
  const int64_t j = (int64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (j >= V.n) return;
  float mx = 0.f;
  for (int64_t i = lane; i < V.n; i += 32) {
    cd a = ldc(V.A, i + j * V.lda);
    mx = fmaxf(mx, fabs_c(a) * V.rows_inv[i]);
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) mx = fmaxf(mx, __shfl_down_sync(0xffffffffu, mx, off));
  if (lane == 0) V.cols[j] = (mx == 0.f) ? 1.0 : (double)mx;
}

__global__ void k_cols_inv(const VecInst* __restrict__ insts) {
  const VecInst& V = insts[blockIdx.y];
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j < V.n) V.cols_inv[j] = 1.0 / V.cols[j];
}

// out_ij = A_ij / rows_i / cols_j (complex64 or complex128); partial row sums of |out|
__global__ void k_scale_copy(const VecInst* __restrict__ insts) {
  const VecInst& V = insts[blockIdx.z];
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= V.n) return;
  int64_t j0, j1;
  chunk_range(V.n, blockIdx.y, kChunks, &j0, &j1);
  const double ri = 1.0 / V.rows[i];
  double sm = 0.0;
  bool bad = false;
  for (int64_t j = j0; j < j1; ++j) {
    cd a = ldc(V.A, i + j * V.lda);
    const double sc = ri * V.cols_inv[j];
    if (V.out_single) {
      const float fs = (float)sc;
      float2 f = make_float2((float)a.x * fs, (float)a.y * fs);
      reinterpret_cast<float2*>(V.out)[i + j * V.n] = f;
      bad |= !(isfinite(f.x) && isfinite(f.y));
      sm += sqrtf(fmaf(f.x, f.x, f.y * f.y));
    } else {
      cd v = {a.x * sc, a.y * sc};
      stc(V.out, i + j * V.n, v);
      bad |= !(isfinite(v.x) && isfinite(v.y));
      sm += fabs_c(v);
    }
  }
  V.part[blockIdx.y * V.n + i] = sm;
  if (bad) atomicExch(V.flag, 1);
}

// stats[0] = max_i rowsum_i (||A||_inf), stats[1] = max_i sum_c part (||scaled||_inf)
__global__ void k_norms_finish(const VecInst* __restrict__ insts) {
  const VecInst& V = insts[blockIdx.x];
  __shared__ double s0[256], s1[256];
  double m0 = 0.0, m1 = 0.0;
  for (int64_t i = threadIdx.x; i < V.n; i += 256) {
    double t = 0.0;
    for (int c = 0; c < kChunks; ++c) t += V.part[c * V.n + i];
    m0 = fmax(m0, V.rowsum[i]);
    m1 = fmax(m1, t);
  }
  s0[threadIdx.x] = m0;
  s1[threadIdx.x] = m1;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      s0[threadIdx.x] = fmax(s0[threadIdx.x], s0[threadIdx.x + s]);
      s1[threadIdx.x] = fmax(s1[threadIdx.x], s1[threadIdx.x + s]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    V.stats[0] = s0[0];
    V.stats[1] = s1[0];
  }
}

// ---------------------------------------------------------------- products
// partial y = A x (and |A||x|) over a column chunk, up to kGemvR right-hand sides
// per pass (rhs group = blockIdx.y / kChunks).
__global__ void __launch_bounds__(256) k_gemv_part(const VecInst* __restrict__ insts, int with_abs) {
  const VecInst& V = insts[blockIdx.z];
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int ch = blockIdx.y % kChunks, grp = blockIdx.y / kChunks;
  const int r0 = grp * kGemvR;
  if (i >= V.n || r0 >= V.nrhs) return;
  const int nr = min(kGemvR, V.nrhs - r0);
  int64_t j0, j1;
  chunk_range(V.n, ch, kChunks, &j0, &j1);
  cd acc[kGemvR];
  float aacc[kGemvR];
#pragma unroll
  for (int r = 0; r < kGemvR; ++r) {
    acc[r] = cd{0.0, 0.0};
    aacc[r] = 0.f;
  }
  for (int64_t j = j0; j < j1; ++j) {
    cd a = ldc(V.A, i + j * V.lda);
    const float aa = with_abs ? fabs_c(a) : 0.f;
#pragma unroll
    for (int r = 0; r < kGemvR; ++r) {
      if (r < nr) {
        cd x = ldc(V.x, j + (int64_t)(r0 + r) * V.ldx);
        acc[r].x = fma(a.x, x.x, fma(-a.y, x.y, acc[r].x));
        acc[r].y = fma(a.x, x.y, fma(a.y, x.x, acc[r].y));
        if (with_abs) aacc[r] = fmaf(aa, fabs_c(x), aacc[r]);
      }
    }
  }
  // part layout: [chunk][rhs][row] x (re, im, abs)
  for (int r = 0; r < nr; ++r) {
    int64_t o = 3 * (((int64_t)ch * V.nrhs + r0 + r) * V.n + i);
    V.part[o] = acc[r].x;
    V.part[o + 1] = acc[r].y;
    V.part[o + 2] = (double)aacc[r];
  }
}

// mode 0: y = A x.  mode 1: y = b - A x, den = |b| + |A||x|.
__global__ void k_gemv_finish(const VecInst* __restrict__ insts, int mode) {
  const VecInst& V = insts[blockIdx.z];
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int r = blockIdx.y;
  if (i >= V.n || r >= V.nrhs) return;
  double re = 0.0, im = 0.0, ab = 0.0;
  for (int c = 0; c < kChunks; ++c) {
    int64_t o = 3 * (((int64_t)c * V.nrhs + r) * V.n + i);
    re += V.part[o];
    im += V.part[o + 1];
    ab += V.part[o + 2];
  }
  const int64_t yo = i + (int64_t)r * V.ldy;
  if (mode == 0) {
    stc(V.y, yo, cd{re, im});
  } else {
    cd b = ldc(V.b, i + (int64_t)r * V.ldb);
    stc(V.y, yo, cd{b.x - re, b.y - im});
    V.den[yo] = cabs(b) + ab;
  }
}

// Per right-hand side statistics of a residual r (in y), denominators den, solution x,
// rhs b and row scales:  [0] max|r|  [1] max |r|/den (0/0 = 0, r/0 = inf)  [2] max|x|
// [3] max|b|  [4] sum|r|^2  [5] sum|b|^2  [6] sum|r/rows|^2  [7] sum|b/rows|^2
// [8] nonfinite flag.  One CTA per (rhs, instance).
__global__ void __launch_bounds__(256) k_resid_stats(const VecInst* __restrict__ insts) {
  const VecInst& V = insts[blockIdx.y];
  const int r = blockIdx.x;
  if (r >= V.nrhs) return;
  double v[kStats];
#pragma unroll
  for (int t = 0; t < kStats; ++t) v[t] = 0.0;
  for (int64_t i = threadIdx.x; i < V.n; i += 256) {
    const int64_t o = i + (int64_t)r * V.ldy;
    cd rr = ldc(V.y, o);
    cd bb = ldc(V.b, i + (int64_t)r * V.ldb);
    cd xx = ldc(V.x, i + (int64_t)r * V.ldx);
    double ar = cabs(rr), ab = cabs(bb), ax = cabs(xx);
    double den = V.den ? V.den[o] : 0.0;
    double ratio = (den == 0.0) ? (ar == 0.0 ? 0.0 : INFINITY) : ar / den;
    double rw = V.rows ? V.rows[i] : 1.0;
    v[0] = fmax(v[0], ar);
    v[1] = fmax(v[1], ratio);
    v[2] = fmax(v[2], ax);
    v[3] = fmax(v[3], ab);
    v[4] += ar * ar;
    v[5] += ab * ab;
    v[6] += (ar / rw) * (ar / rw);
    v[7] += (ab / rw) * (ab / rw);
    if (!(isfinite(rr.x) && isfinite(rr.y) && isfinite(den) && isfinite(xx.x) && isfinite(xx.y)))
      v[8] = 1.0;
  }
  __shared__ double sh[kStats][256];
#pragma unroll
  for (int t = 0; t < kStats; ++t) sh[t][threadIdx.x] = v[t];
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
#pragma unroll
      for (int t = 0; t < kStats; ++t) {
        double a = sh[t][threadIdx.x], b = sh[t][threadIdx.x + s];
        sh[t][threadIdx.x] = (t == 4 || t == 5 || t == 6 || t == 7) ? a + b : fmax(a, b);
      }
    }
    __syncthreads();
  }
  if (threadIdx.x < kStats) V.stats[(int64_t)r * kStats + threadIdx.x] = sh[threadIdx.x][0];
}

// ---------------------------------------------------------------- correction steps
// stats[r * kStats] = max_i |v_i / rows_i| for the vectors in y (v = b or residual)
__global__ void __launch_bounds__(256) k_scaled_absmax(const VecInst* __restrict__ insts) {
  const VecInst& V = insts[blockIdx.y];
  const int r = blockIdx.x;
  if (r >= V.nrhs) return;
  double m = 0.0;
  bool bad = false;
  for (int64_t i = threadIdx.x; i < V.n; i += 256) {
    cd a = ldc(V.y, i + (int64_t)r * V.ldy);
    double s = V.rows ? V.rows[i] : 1.0;
    double t = hypot(a.x / s, a.y / s);
    if (!isfinite(t)) bad = true;
    m = fmax(m, t);
  }
  __shared__ double sh[256];
  __shared__ int sb;
  if (threadIdx.x == 0) sb = 0;
  __syncthreads();
  if (bad) sb = 1;
  sh[threadIdx.x] = m;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] = fmax(sh[threadIdx.x], sh[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) V.stats[(int64_t)r * kStats] = sb ? NAN : sh[0];
}

// work (getrs input, complex64 or complex128, ld n) = (v / rows) / mag
__global__ void k_corr_prep(const VecInst* __restrict__ insts) {
  const VecInst& V = insts[blockIdx.z];
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int r = blockIdx.y;
  if (i >= V.n || r >= V.nrhs) return;
  const double mag = V.stats[(int64_t)r * kStats];
  cd a = ldc(V.y, i + (int64_t)r * V.ldy);
  double s = V.rows ? V.rows[i] : 1.0;
  cd w = {0.0, 0.0};
  if (mag > 0.0 && isfinite(mag)) w = cd{a.x / s / mag, a.y / s / mag};
  const int64_t o = i + (int64_t)r * V.n;
  if (V.out_single)
    reinterpret_cast<float2*>(V.out)[o] = make_float2((float)w.x, (float)w.y);
  else
    stc(V.out, o, w);
}

// value = work * mag / cols;  mode 0: x = value;  mode 1: x += value (flag if changed)
__global__ void k_corr_apply(const VecInst* __restrict__ insts, int mode) {
  const VecInst& V = insts[blockIdx.z];
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int r = blockIdx.y;
  if (i >= V.n || r >= V.nrhs) return;
  if (V.active && !V.active[r]) return;
  const double mag = V.stats[(int64_t)r * kStats];
  const int64_t o = i + (int64_t)r * V.n;
  cd w;
  if (V.out_single) {
    float2 f = reinterpret_cast<const float2*>(V.out)[o];
    w = {(double)f.x, (double)f.y};
  } else {
    w = ldc(V.out, o);
  }
  const double c = V.cols ? V.cols[i] : 1.0;
  cd val;
  if (!isfinite(mag))
    val = cd{NAN, NAN};
  else if (mag == 0.0)
    val = cd{0.0, 0.0};
  else
    val = cd{w.x * mag / c, w.y * mag / c};
  double* X = const_cast<double*>(V.x);
  const int64_t xo = i + (int64_t)r * V.ldx;
  if (mode == 0) {
    stc(X, xo, val);
  } else {
    cd x = ldc(X, xo);
    cd nx = {x.x + val.x, x.y + val.y};
    if (nx.x != x.x || nx.y != x.y) V.changed[r] = 1;
    stc(X, xo, nx);
  }
}

// ---------------------------------------------------------------- launch wrappers
void launch_equilibrate(const Launch& L, const VecInst* d, int ninst, int64_t nmax) {
  dim3 g1((unsigned)((nmax + 255) / 256), kChunks, (unsigned)ninst);
  k_rowstats<<<g1, 256, 0, L.stream>>>(d); count_launch(1);
  k_rowstats_finish<<<dim3((unsigned)((nmax + 255) / 256), (unsigned)ninst), 256, 0, L.stream>>>(d); count_launch(1);
  k_colmax<<<dim3((unsigned)((nmax + 7) / 8), (unsigned)ninst), 256, 0, L.stream>>>(d); count_launch(1);
}

void launch_scale_copy(const Launch& L, const VecInst* d, int ninst, int64_t nmax) {
  k_cols_inv<<<dim3((unsigned)((nmax + 255) / 256), (unsigned)ninst), 256, 0, L.stream>>>(d);
  count_launch(1);
  dim3 g1((unsigned)((nmax + 255) / 256), kChunks, (unsigned)ninst);
  k_scale_copy<<<g1, 256, 0, L.stream>>>(d); count_launch(1);
  k_norms_finish<<<ninst, 256, 0, L.stream>>>(d); count_launch(1);
}

void launch_gemv(const Launch& L, const VecInst* d, int ninst, int64_t nmax, int32_t max_rhs,
                 int mode) {
  const int groups = (max_rhs + kGemvR - 1) / kGemvR;
  dim3 g1((unsigned)((nmax + 255) / 256), (unsigned)(kChunks * groups), (unsigned)ninst);
  k_gemv_part<<<g1, 256, 0, L.stream>>>(d, mode == 1); count_launch(1);
  dim3 g2((unsigned)((nmax + 255) / 256), (unsigned)max_rhs, (unsigned)ninst);
  k_gemv_finish<<<g2, 256, 0, L.stream>>>(d, mode); count_launch(1);
}

void launch_resid_stats(const Launch& L, const VecInst* d, int ninst, int32_t max_rhs) {
  k_resid_stats<<<dim3((unsigned)max_rhs, (unsigned)ninst), 256, 0, L.stream>>>(d); count_launch(1);
}

void launch_corr_prep(const Launch& L, const VecInst* d, int ninst, int64_t nmax,
                      int32_t max_rhs) {
  k_scaled_absmax<<<dim3((unsigned)max_rhs, (unsigned)ninst), 256, 0, L.stream>>>(d); count_launch(1);
  k_corr_prep<<<dim3((unsigned)((nmax + 255) / 256), (unsigned)max_rhs, (unsigned)ninst), 256, 0,
                L.stream>>>(d); count_launch(1);
}

void launch_corr_apply(const Launch& L, const VecInst* d, int ninst, int64_t nmax,
                       int32_t max_rhs, int mode) {
  k_corr_apply<<<dim3((unsigned)((nmax + 255) / 256), (unsigned)max_rhs, (unsigned)ninst), 256, 0,
                 L.stream>>>(d, mode); count_launch(1);
}

}  // namespace bemgpu
