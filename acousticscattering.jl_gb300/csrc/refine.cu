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

// Element access of the system: complex128, or complex64 for compact instances (a32).
__device__ __forceinline__ float2 ldf(const void* base, int64_t idx) {
  return reinterpret_cast<const float2*>(base)[idx];
}
template <bool A32>
__device__ __forceinline__ float mag_at(const VecInst& V, int64_t idx) {
  if (A32) {
    const float2 a = ldf(V.A, idx);
    return sqrtf(fmaf(a.x, a.x, a.y * a.y));
  }
  return fabs_c(ldc(V.A, idx));
}

// ---------------------------------------------------------------- equilibration
template <bool A32>
__device__ __forceinline__ void rowstats_body(const VecInst& V) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= V.n) return;
  int64_t j0, j1;
  chunk_range(V.n, blockIdx.y, kChunks, &j0, &j1);
  float mx = 0.f;
  double sm = 0.0;
  constexpr int kB = 16;
  for (int64_t jf = j0; jf < j1; jf += 256) {  // fold into FP64 every 256 terms
    float sm32 = 0.f;
    const int64_t jf1 = min(j1, jf + 256);
    for (int64_t jb = jf; jb < jf1; jb += kB) {
      const int cnt = (int)min((int64_t)kB, jf1 - jb);
      float a[kB];
#pragma unroll
      for (int q = 0; q < kB; ++q) a[q] = q < cnt ? mag_at<A32>(V, i + (jb + q) * V.lda) : 0.f;
#pragma unroll
      for (int q = 0; q < kB; ++q) {
        mx = fmaxf(mx, a[q]);
        sm32 += a[q];
      }
    }
    sm += sm32;
  }
  V.part[2 * (blockIdx.y * V.n + i)] = mx;
  V.part[2 * (blockIdx.y * V.n + i) + 1] = sm;
}
__global__ void k_rowstats(const VecInst* __restrict__ insts) {
  const VecInst& V = insts[blockIdx.z];
  if (V.a32)
    rowstats_body<true>(V);
  else
    rowstats_body<false>(V);
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
  mx = fmax(mx, V.norm_floor);  // the reference's norm_floor (full.jl:388-394)
  V.rows[i] = (mx == 0.0) ? 1.0 : mx;
  V.rows_inv[i] = (float)(1.0 / V.rows[i]);
  V.rowsum[i] = sm;
}

// columns[j] = max_i |A_ij / rows_i|, one warp per column
template <bool A32>
__device__ __forceinline__ void colmax_body(const VecInst& V) {
  const int64_t j = (int64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (j >= V.n) return;
  float mx = 0.f;
  const int64_t n = V.n, base = j * V.lda;
  int64_t i = lane;
  for (; i + 96 < n; i += 128) {
    float a[4], w[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      a[q] = mag_at<A32>(V, base + i + 32 * q);
      w[q] = V.rows_inv[i + 32 * q];
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) mx = fmaxf(mx, a[q] * w[q]);
  }
  for (; i < n; i += 32) mx = fmaxf(mx, mag_at<A32>(V, base + i) * V.rows_inv[i]);
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) mx = fmaxf(mx, __shfl_down_sync(0xffffffffu, mx, off));
  if (lane == 0) {
    const double cm = fmax((double)mx, V.norm_floor);
    V.cols[j] = (cm == 0.0) ? 1.0 : cm;
  }
}
__global__ void k_colmax(const VecInst* __restrict__ insts) {
  const VecInst& V = insts[blockIdx.y];
  if (V.a32)
    colmax_body<true>(V);
  else
    colmax_body<false>(V);
}

__global__ void k_cols_inv(const VecInst* __restrict__ insts) {
  const VecInst& V = insts[blockIdx.y];
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j < V.n) {
    V.cols_inv[j] = 1.0 / V.cols[j];
    if (V.cols_inv32) V.cols_inv32[j] = (float)V.cols_inv[j];
    if (V.rows_inv) V.rows_inv[j] = (float)(1.0 / V.rows[j]);  // rows may have been reset
  }
}

// out_ij = A_ij / rows_i / cols_j (complex64 or complex128); partial row sums of |out|.
// The complex64 copy scales in FP32 by the FP32 reciprocals (a rounding-level change of
// the scaling that the refinement, which uses the FP64 scales, absorbs).
template <bool A32>
__device__ __forceinline__ void scale_copy_body(const VecInst& V) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= V.n) return;
  int64_t j0, j1;
  chunk_range(V.n, blockIdx.y, kChunks, &j0, &j1);
  double sm = 0.0;
  float sm32 = 0.f;
  int cnt = 0;
  bool bad = false;
  if (V.out_single) {
    const float ri = V.rows_inv[i];
    constexpr int kB = 8;
    for (int64_t jb = j0; jb < j1; jb += kB) {
      const int nb = (int)min((int64_t)kB, j1 - jb);
      float2 a[kB];
#pragma unroll
      for (int q = 0; q < kB; ++q) {
        if (q < nb) {
          if (A32) {
            a[q] = ldf(V.A, i + (jb + q) * V.lda);
          } else {
            const cd d = ldc(V.A, i + (jb + q) * V.lda);
            a[q] = make_float2((float)d.x, (float)d.y);
          }
        }
      }
#pragma unroll
      for (int q = 0; q < kB; ++q) {
        if (q < nb) {
          const float fs = ri * V.cols_inv32[jb + q];
          const float2 f = make_float2(a[q].x * fs, a[q].y * fs);
          reinterpret_cast<float2*>(V.out)[i + (jb + q) * V.n] = f;
          bad |= !(isfinite(f.x) && isfinite(f.y));
          sm32 += sqrtf(fmaf(f.x, f.x, f.y * f.y));
        }
      }
      cnt += nb;
      if (cnt >= 256) {  // fold into FP64 every 256 terms
        sm += sm32;
        sm32 = 0.f;
        cnt = 0;
      }
    }
    sm += sm32;
  } else {
    const double ri = 1.0 / V.rows[i];
    for (int64_t j = j0; j < j1; ++j) {
      cd a;
      if (A32) {
        const float2 f = ldf(V.A, i + j * V.lda);
        a = cd{(double)f.x, (double)f.y};
      } else {
        a = ldc(V.A, i + j * V.lda);
      }
      const double sc = ri * V.cols_inv[j];
      cd v = {a.x * sc, a.y * sc};
      stc(V.out, i + j * V.n, v);
      bad |= !(isfinite(v.x) && isfinite(v.y));
      sm += fabs_c(v);
    }
  }
  V.part[blockIdx.y * V.n + i] = sm;
  if (bad) atomicExch(V.flag, 1);
}
__global__ void k_scale_copy(const VecInst* __restrict__ insts) {
  const VecInst& V = insts[blockIdx.z];
  if (V.a32)
    scale_copy_body<true>(V);
  else
    scale_copy_body<false>(V);
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

// ---------------------------------------------------------------- compact storage helpers
// out += near corrections (scaled unless unit); one thread per (near pair, block)
__global__ void k_near_add(const VecInst* __restrict__ insts, int unit) {
  const VecInst& V = insts[blockIdx.z];
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int b = blockIdx.y;
  if (!V.a32 || p >= V.n_near || b >= V.nbc * V.nbc) return;
  const int br = b / V.nbc, bc = b % V.nbc;
  const int64_t row = br * V.n_mesh + V.near_i[p], col = bc * V.n_mesh + V.near_j[p];
  const cd d = ldc(V.dnear, (int64_t)b * V.n_near + p);
  const double sc = unit ? 1.0 : (1.0 / V.rows[row]) * V.cols_inv[col];
  const int64_t o = row + col * V.n;
  cd v = ldc(V.out, o);
  stc(V.out, o, cd{v.x + d.x * sc, v.y + d.y * sc});
}

__global__ void k_expand_a32(const VecInst* __restrict__ insts) {
  const VecInst& V = insts[blockIdx.z];
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (!V.a32 || i >= V.n) return;
  for (int64_t j = blockIdx.y; j < V.n; j += gridDim.y) {
    const float2 f = ldf(V.A, i + j * V.lda);
    stc(V.out, i + j * V.n, cd{(double)f.x, (double)f.y});
  }
}

// x split for the compact products: hi = fl32(x), lo = fl32(x - hi)
__global__ void k_split_x(const VecInst* __restrict__ insts) {
  const VecInst& V = insts[blockIdx.z];
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int r = blockIdx.y;
  if (!V.a32 || i >= V.n || r >= V.nrhs) return;
  const cd x = ldc(V.x, i + (int64_t)r * V.ldx);
  const float hr = (float)x.x, hi = (float)x.y;
  const float lr = (float)(x.x - (double)hr), li = (float)(x.y - (double)hi);
  V.xs[i + (int64_t)r * V.n] = make_float4(hr, hi, lr, li);
  V.xa[i + (int64_t)r * V.n] = sqrtf(fmaf(hr, hr, hi * hi));
}

// ---------------------------------------------------------------- products
// Compact products in FP32 pair arithmetic.  A complex64 entry times the split x
// (hi + lo): each product a * hi is exact as p + e (round-to-nearest product and its FMA
// error), p enters a (s, t) pair by TwoSum (s + t carries the sum exactly up to the FP32
// rounding of t), and e and a * lo go into t.  Every 32 columns (128 real products) the
// pair is folded into FP64, so t holds at most that many terms' errors.  What is left is
// the FP32 rounding of t: for an exact solution the computed residual stays below about
// 6e-14 of |b| + |A||x| in every row of small Burton-Miller and Mueller systems, where a
// dominant diagonal block carries most of a row (median about 3e-15; an operation-by-
// operation emulation on the CPU), under the refinement's 1e-13 acceptance, at a small
// fraction of the FP64 instruction count of the complex128 path.  The intrinsics keep the
// compiler from contracting or reassociating the error-free steps.
struct FPair {
  float s, t;
};
__device__ __forceinline__ void pair_add_prod(FPair& a, float u, float v) {
  const float p = __fmul_rn(u, v);
  const float e = __fmaf_rn(u, v, -p);
  const float s = __fadd_rn(a.s, p);
  const float bb = __fsub_rn(s, a.s);
  const float err = __fadd_rn(__fsub_rn(a.s, __fsub_rn(s, bb)), __fsub_rn(p, bb));
  a.s = s;
  a.t = __fadd_rn(a.t, __fadd_rn(err, e));
}

template <bool A32, int NR>
__device__ __forceinline__ void gemv_body(const VecInst& V, int with_abs) {
  constexpr int kGemvR = NR;  // right-hand sides per pass of this instantiation
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
  if (A32) {
    // fold into FP64 every kFold columns; columns loaded kBatch at a time so each
    // thread keeps kBatch independent requests in flight
    constexpr int kFold = 32, kBatch = NR == 1 ? 16 : 8;
    const float2* Acol = reinterpret_cast<const float2*>(V.A) + i;
    const int64_t lda = V.lda, ldxs = V.n;
    for (int64_t jf = j0; jf < j1; jf += kFold) {
      FPair re[kGemvR], im[kGemvR];
#pragma unroll
      for (int r = 0; r < kGemvR; ++r) re[r] = im[r] = FPair{0.f, 0.f};
      const int64_t jf1 = min(j1, jf + kFold);
      for (int64_t jb = jf; jb < jf1; jb += kBatch) {
        const int cnt = (int)min((int64_t)kBatch, jf1 - jb);
        float2 a[kBatch];
#pragma unroll
        for (int q = 0; q < kBatch; ++q)
          a[q] = q < cnt ? Acol[(jb + q) * lda] : make_float2(0.f, 0.f);
#pragma unroll
        for (int q = 0; q < kBatch; ++q) {
          if (q < cnt) {
            const float aa = with_abs ? sqrtf(fmaf(a[q].x, a[q].x, a[q].y * a[q].y)) : 0.f;
#pragma unroll
            for (int r = 0; r < kGemvR; ++r) {
              if (r < nr) {
                const int64_t xo = jb + q + (int64_t)(r0 + r) * ldxs;
                const float4 x = V.xs[xo];
                // re += a.x x.re - a.y x.im ; im += a.x x.im + a.y x.re
                pair_add_prod(re[r], a[q].x, x.x);
                pair_add_prod(re[r], -a[q].y, x.y);
                pair_add_prod(im[r], a[q].x, x.y);
                pair_add_prod(im[r], a[q].y, x.x);
                re[r].t = __fmaf_rn(a[q].x, x.z, __fmaf_rn(-a[q].y, x.w, re[r].t));
                im[r].t = __fmaf_rn(a[q].x, x.w, __fmaf_rn(a[q].y, x.z, im[r].t));
                if (with_abs) aacc[r] = fmaf(aa, V.xa[xo], aacc[r]);
              }
            }
          }
        }
      }
#pragma unroll
      for (int r = 0; r < kGemvR; ++r) {
        acc[r].x += (double)re[r].s + (double)re[r].t;
        acc[r].y += (double)im[r].s + (double)im[r].t;
      }
    }
  } else {
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
  }
  // part layout: [chunk][rhs][row] x (re, im, abs)
#pragma unroll
  for (int r = 0; r < kGemvR; ++r) {
    if (r < nr) {
      int64_t o = 3 * (((int64_t)ch * V.nrhs + r0 + r) * V.n + i);
      V.part[o] = acc[r].x;
      V.part[o + 1] = acc[r].y;
      V.part[o + 2] = (double)aacc[r];
    }
  }
}

// Compact instances: ROWS rows per thread (i, i + 256, ..., all coalesced), so every x
// value loaded serves ROWS rows and each thread carries 2 ROWS independent pair-sum chains
// per right-hand side.  Columns are loaded kBatch at a time, folded into FP64 every
// kFold columns.  ROWS (1 or 2) is a launch shape of the autotuner; it does not change
// any row's arithmetic.
template <int NR, int ROWS>
__device__ __forceinline__ void gemv_a32_body(const VecInst& V, int with_abs) {
  constexpr int kA32Rows = ROWS;
  constexpr int kFold = 32, kBatch = NR == 1 ? 8 : 4;
  const int64_t n = V.n;
  const int64_t i0 = (int64_t)blockIdx.x * (256 * kA32Rows) + threadIdx.x;
  const int ch = blockIdx.y % kChunks, grp = blockIdx.y / kChunks;
  const int r0 = grp * NR;
  if (i0 >= n || r0 >= V.nrhs) return;
  const int nr = min(NR, V.nrhs - r0);
  const bool ok1 = i0 + 256 < n;
  int64_t j0, j1;
  chunk_range(n, ch, kChunks, &j0, &j1);
  const float2* A0 = reinterpret_cast<const float2*>(V.A) + i0;
  const float2* A1 = (ROWS > 1 && ok1) ? A0 + 256 : A0;
  const int64_t lda = V.lda;
  const float4* xs[NR];
  const float* xa[NR];
#pragma unroll
  for (int r = 0; r < NR; ++r) {
    const int64_t rr = (int64_t)(r0 + (r < nr ? r : 0)) * n;
    xs[r] = V.xs + rr;
    xa[r] = V.xa + rr;
  }
  cd acc[kA32Rows][NR];
  float aacc[kA32Rows][NR];
#pragma unroll
  for (int h = 0; h < kA32Rows; ++h)
#pragma unroll
    for (int r = 0; r < NR; ++r) {
      acc[h][r] = cd{0.0, 0.0};
      aacc[h][r] = 0.f;
    }
  for (int64_t jf = j0; jf < j1; jf += kFold) {
    FPair re[kA32Rows][NR], im[kA32Rows][NR];
#pragma unroll
    for (int h = 0; h < kA32Rows; ++h)
#pragma unroll
      for (int r = 0; r < NR; ++r) re[h][r] = im[h][r] = FPair{0.f, 0.f};
    const int64_t jf1 = min(j1, jf + kFold);
    for (int64_t jb = jf; jb < jf1; jb += kBatch) {
      const int cnt = (int)min((int64_t)kBatch, jf1 - jb);
      float2 a[kA32Rows][kBatch];
#pragma unroll
      for (int q = 0; q < kBatch; ++q) {
        a[0][q] = q < cnt ? A0[(jb + q) * lda] : make_float2(0.f, 0.f);
        if (ROWS > 1) a[ROWS - 1][q] = q < cnt ? A1[(jb + q) * lda] : make_float2(0.f, 0.f);
      }
#pragma unroll
      for (int q = 0; q < kBatch; ++q) {
        if (q < cnt) {
          float aa[kA32Rows];
#pragma unroll
          for (int h = 0; h < kA32Rows; ++h)
            aa[h] = with_abs ? sqrtf(fmaf(a[h][q].x, a[h][q].x, a[h][q].y * a[h][q].y)) : 0.f;
#pragma unroll
          for (int r = 0; r < NR; ++r) {
            const float4 x = xs[r][jb + q];
            const float xm = with_abs ? xa[r][jb + q] : 0.f;
#pragma unroll
            for (int h = 0; h < kA32Rows; ++h) {
              const float2 av = a[h][q];
              // re += a.x x.re - a.y x.im ; im += a.x x.im + a.y x.re
              pair_add_prod(re[h][r], av.x, x.x);
              pair_add_prod(re[h][r], -av.y, x.y);
              pair_add_prod(im[h][r], av.x, x.y);
              pair_add_prod(im[h][r], av.y, x.x);
              re[h][r].t = __fmaf_rn(av.x, x.z, __fmaf_rn(-av.y, x.w, re[h][r].t));
              im[h][r].t = __fmaf_rn(av.x, x.w, __fmaf_rn(av.y, x.z, im[h][r].t));
              aacc[h][r] = fmaf(aa[h], xm, aacc[h][r]);
            }
          }
        }
      }
    }
#pragma unroll
    for (int h = 0; h < kA32Rows; ++h)
#pragma unroll
      for (int r = 0; r < NR; ++r) {
        acc[h][r].x += (double)re[h][r].s + (double)re[h][r].t;
        acc[h][r].y += (double)im[h][r].s + (double)im[h][r].t;
      }
  }
  // part layout: [chunk][rhs][row] x (re, im, abs)
#pragma unroll
  for (int h = 0; h < kA32Rows; ++h) {
    const int64_t i = i0 + 256 * h;
    if (h == 1 && !ok1) break;
#pragma unroll
    for (int r = 0; r < NR; ++r) {
      if (r < nr) {
        const int64_t o = 3 * (((int64_t)ch * V.nrhs + r0 + r) * n + i);
        V.part[o] = acc[h][r].x;
        V.part[o + 1] = acc[h][r].y;
        V.part[o + 2] = (double)aacc[h][r];
      }
    }
  }
}

template <int NR, int ROWS>
__global__ void __launch_bounds__(256, 2) k_gemv_a32(const VecInst* __restrict__ insts, int with_abs) {
  const VecInst& V = insts[blockIdx.z];
  if (!V.a32) return;
  gemv_a32_body<NR, ROWS>(V, with_abs);
}

// partial y = A x (and |A||x|) over a column chunk, up to kGemvR right-hand sides
// per pass (rhs group = blockIdx.y / kChunks).
template <bool A32, int NR>
__global__ void __launch_bounds__(256) k_gemv_part(const VecInst* __restrict__ insts, int with_abs) {
  const VecInst& V = insts[blockIdx.z];
  if ((V.a32 != 0) != A32) return;
  gemv_body<A32, NR>(V, with_abs);
}

// mode 0: y = A x.  mode 1: y = b - A x, den = |b| + |A||x|.  Compact instances add the
// near corrections of the row (FP64, fixed CSR order).
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
  if (V.a32) {
    const int br = i >= V.n_mesh ? 1 : 0;
    const int64_t im_ = i - br * V.n_mesh;
    for (int32_t p = V.near_ptr[im_]; p < V.near_ptr[im_ + 1]; ++p) {
      const int64_t j = V.near_j[p];
      for (int bc = 0; bc < V.nbc; ++bc) {
        const cd d = ldc(V.dnear, (int64_t)(br * V.nbc + bc) * V.n_near + p);
        const cd x = ldc(V.x, j + bc * V.n_mesh + (int64_t)r * V.ldx);
        re = fma(d.x, x.x, fma(-d.y, x.y, re));
        im = fma(d.x, x.y, fma(d.y, x.x, im));
      }
    }
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
                 int mode, int rows) {
  // compact and complex128 instances by their own instantiations (each skips the others);
  // one right-hand side gets a single-rhs instantiation
  const int nr = max_rhs == 1 ? 1 : kGemvR;
  const int groups = (max_rhs + nr - 1) / nr;
  dim3 g0((unsigned)((nmax + 255) / 256), (unsigned)max_rhs, (unsigned)ninst);
  k_split_x<<<g0, 256, 0, L.stream>>>(d); count_launch(1);
  dim3 g1((unsigned)((nmax + 255) / 256), (unsigned)(kChunks * groups), (unsigned)ninst);
  const int rw = rows == 1 ? 1 : 2;
  dim3 ga((unsigned)((nmax + 256 * rw - 1) / (256 * rw)), (unsigned)(kChunks * groups),
          (unsigned)ninst);
  if (nr == 1) {
    if (rw == 1)
      k_gemv_a32<1, 1><<<ga, 256, 0, L.stream>>>(d, mode == 1);
    else
      k_gemv_a32<1, 2><<<ga, 256, 0, L.stream>>>(d, mode == 1);
    k_gemv_part<false, 1><<<g1, 256, 0, L.stream>>>(d, mode == 1);
  } else {
    if (rw == 1)
      k_gemv_a32<kGemvR, 1><<<ga, 256, 0, L.stream>>>(d, mode == 1);
    else
      k_gemv_a32<kGemvR, 2><<<ga, 256, 0, L.stream>>>(d, mode == 1);
    k_gemv_part<false, kGemvR><<<g1, 256, 0, L.stream>>>(d, mode == 1);
  }
  count_launch(2);
  dim3 g2((unsigned)((nmax + 255) / 256), (unsigned)max_rhs, (unsigned)ninst);
  k_gemv_finish<<<g2, 256, 0, L.stream>>>(d, mode); count_launch(1);
}

void launch_near_add(const Launch& L, const VecInst* d, int ninst, int64_t max_near,
                     int unit_scales) {
  if (max_near <= 0 || ninst <= 0) return;
  k_near_add<<<dim3((unsigned)((max_near + 255) / 256), 4, (unsigned)ninst), 256, 0, L.stream>>>(
      d, unit_scales);
  count_launch(1);
}

void launch_expand_a32(const Launch& L, const VecInst* d, int ninst, int64_t nmax) {
  if (nmax <= 0 || ninst <= 0) return;
  k_expand_a32<<<dim3((unsigned)((nmax + 255) / 256), 256, (unsigned)ninst), 256, 0, L.stream>>>(d);
  count_launch(1);
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
