// Small elementwise kernels of the solve chain: fluid CBIE forcing, scattered-trace
// recovery and constant fills.
#include "bemgpu_internal.h"
#include "refine.cuh"
#include "solve_kernels.cuh"

namespace bemgpu {

__device__ __forceinline__ double2 ld2(const double* p, int64_t i) {
  return reinterpret_cast<const double2*>(p)[i];
}
__device__ __forceinline__ void st2(double* p, int64_t i, double2 v) {
  reinterpret_cast<double2*>(p)[i] = v;
}

// kind: 0 rigid (p = x, q = -q_inc), 1 pressure release (p = -p_inc, q = x),
// 2 Mueller (p = x_top - p_inc, q = x_bot - q_inc), 3 fluid CBIE (p = x_top, q = x_bot),
// 4 coupled regions (as Mueller on the surfaces bordering the exterior, 0 elsewhere: the
// far field sums only those, solvers/bem/postprocessing.jl:15-31)
// (solvers/bem/full.jl:160-161, 472-477).
__global__ void k_traces(const TraceInst* __restrict__ insts) {
  const TraceInst& T = insts[blockIdx.z];
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int r = blockIdx.y;
  if (i >= T.n || r >= T.nrhs) return;
  const int64_t o = i + (int64_t)r * T.n;
  const double2 pi = ld2(T.pinc, o), qi = ld2(T.qinc, o);
  const double2 xt = ld2(T.x, i + (int64_t)r * T.ldx);
  double2 p, q;
  switch (T.kind) {
    case 0:
      p = xt;
      q = make_double2(-qi.x, -qi.y);
      break;
    case 1:
      p = make_double2(-pi.x, -pi.y);
      q = xt;
      break;
    case 4:  // regions: scattered traces on the surfaces bordering the exterior, 0 inside
      if (!T.outer[i]) {
        p = q = make_double2(0.0, 0.0);
        break;
      }
      [[fallthrough]];  // total traces minus incident, as Mueller
    case 2: {
      const double2 xb = ld2(T.x, T.n + i + (int64_t)r * T.ldx);
      p = make_double2(xt.x - pi.x, xt.y - pi.y);
      q = make_double2(xb.x - qi.x, xb.y - qi.y);
      break;
    }
    default: {
      const double2 xb = ld2(T.x, T.n + i + (int64_t)r * T.ldx);
      p = xt;
      q = xb;
      break;
    }
  }
  st2(T.ps, o, p);
  st2(T.qs, o, q);
}

// Fluid CBIE forcing (full.jl:449-453): b = [0; -y_bottom] where y = A [p_inc; q_inc].
__global__ void k_cbie_forcing(const TraceInst* __restrict__ insts) {
  const TraceInst& T = insts[blockIdx.z];
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int r = blockIdx.y;
  if (i >= T.n || r >= T.nrhs) return;
  const int64_t ld = 2 * T.n;
  const double2 y = ld2(T.x, T.n + i + (int64_t)r * ld);
  st2(T.ps, i + (int64_t)r * ld, make_double2(0.0, 0.0));
  st2(T.ps, T.n + i + (int64_t)r * ld, make_double2(-y.x, -y.y));
}

// Stack incident traces into a 2n x nrhs block [p; q].
__global__ void k_stack(const TraceInst* __restrict__ insts) {
  const TraceInst& T = insts[blockIdx.z];
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int r = blockIdx.y;
  if (i >= T.n || r >= T.nrhs) return;
  const int64_t ld = 2 * T.n;
  const bool on = T.outer ? T.outer[i] != 0 : true;  // regions: exterior surfaces only
  const bool q = T.outer ? (on && T.stack_q) : true;
  const double2 z = make_double2(0.0, 0.0);
  st2(T.ps, i + (int64_t)r * ld, on ? ld2(T.pinc, i + (int64_t)r * T.n) : z);
  st2(T.ps, T.n + i + (int64_t)r * ld, q ? ld2(T.qinc, i + (int64_t)r * T.n) : z);
}

__global__ void k_fill(double* p, int64_t count, double v) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) p[i] = v;
}

// ------------------------------------------------------------------ zlacn2 on the device
// LAPACK's zlacn2 (1-norm estimate by reverse communication, the estimator inside gecon),
// one CTA per factor: the same states and tests as LAPACK (sum of moduli, first index of
// the largest modulus, x_i / |x_i| with 1 below safmin, at most 5 iterations, the
// alternating-sign final vector), moduli and sums in FP64 from the complex64 vector, sums
// in a fixed order.
constexpr int kLacT = 256;

__device__ double lac_sum(double v, double* sh) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  for (int w = 0; w < kLacT / 32; ++w) t += sh[w];
  return t;
}

__device__ int lac_imax(const float2* x, int n, double* sv, int* si) {
  double bv = -1.0;
  int bi = INT32_MAX;
  for (int i = threadIdx.x; i < n; i += kLacT) {
    const double a = hypot((double)x[i].x, (double)x[i].y);
    if (a > bv) {  // increasing i per thread: the first index of each thread's maximum
      bv = a;
      bi = i;
    }
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const double ov = __shfl_xor_sync(0xffffffffu, bv, off);
    const int oi = __shfl_xor_sync(0xffffffffu, bi, off);
    if (ov > bv || (ov == bv && oi < bi)) {
      bv = ov;
      bi = oi;
    }
  }
  __syncthreads();
  if ((threadIdx.x & 31) == 0) {
    sv[threadIdx.x >> 5] = bv;
    si[threadIdx.x >> 5] = bi;
  }
  __syncthreads();
  bv = sv[0];
  bi = si[0];
  for (int w = 1; w < kLacT / 32; ++w)
    if (sv[w] > bv || (sv[w] == bv && si[w] < bi)) {
      bv = sv[w];
      bi = si[w];
    }
  return bi;
}

__global__ void __launch_bounds__(kLacT) k_lacn2(Lacn2Dev* __restrict__ st, float2* __restrict__ work,
                                                MatInst* __restrict__ mi1,
                                                MatInst* __restrict__ mi2, int want) {
  Lacn2Dev& S = st[blockIdx.x];
  const int kase0 = S.kase;
  if (want == 0 ? (kase0 != 0 || S.isave1 != 0) : kase0 != want) return;  // uniform
  __shared__ double sh[kLacT / 32];
  __shared__ int shi[kLacT / 32];
  float2* x = work + S.off;
  const int n = S.n;
  int kase = 0, isave1 = S.isave1, isave2 = S.isave2, isave3 = S.isave3;
  double est = S.est;
  auto sum1 = [&]() {
    double t = 0.0;
    for (int i = threadIdx.x; i < n; i += kLacT) t += hypot((double)x[i].x, (double)x[i].y);
    return lac_sum(t, sh);
  };
  auto normalise = [&]() {
    const double safmin = 2.2250738585072014e-308;
    for (int i = threadIdx.x; i < n; i += kLacT) {
      const double re = x[i].x, im = x[i].y, a = hypot(re, im);
      x[i] = a > safmin ? make_float2((float)(re / a), (float)(im / a)) : make_float2(1.f, 0.f);
    }
  };
  int go = 0;  // 1: the main loop's unit vector, 2: the final alternating vector
  if (want == 0) {
    for (int i = threadIdx.x; i < n; i += kLacT) x[i] = make_float2((float)(1.0 / n), 0.f);
    kase = 1;
    isave1 = 1;
  } else {
    switch (isave1) {
      case 1:
        if (n == 1) {
          est = hypot((double)x[0].x, (double)x[0].y);
          kase = 0;
          break;
        }
        est = sum1();
        normalise();
        kase = 2;
        isave1 = 2;
        break;
      case 2:
        isave2 = lac_imax(x, n, sh, shi);
        isave3 = 2;
        go = 1;
        break;
      case 3: {
        const double estold = est;
        est = sum1();
        if (est <= estold) {
          go = 2;
          break;
        }
        normalise();
        kase = 2;
        isave1 = 4;
        break;
      }
      case 4: {
        const int jlast = isave2;
        isave2 = lac_imax(x, n, sh, shi);
        const double a = hypot((double)x[jlast].x, (double)x[jlast].y);
        const double b = hypot((double)x[isave2].x, (double)x[isave2].y);
        if (a != b && isave3 < 5) {
          ++isave3;
          go = 1;
        } else {
          go = 2;
        }
        break;
      }
      default: {  // 5
        const double temp = 2.0 * (sum1() / (3.0 * n));
        if (temp > est) est = temp;
        kase = 0;
        break;
      }
    }
  }
  __syncthreads();  // every read of x above precedes the writes below
  if (go == 1) {
    for (int i = threadIdx.x; i < n; i += kLacT) x[i] = make_float2(i == isave2 ? 1.f : 0.f, 0.f);
    kase = 1;
    isave1 = 3;
  } else if (go == 2) {
    for (int i = threadIdx.x; i < n; i += kLacT) {
      const double v = (1.0 + (double)i / (double)(n - 1)) * ((i & 1) ? -1.0 : 1.0);
      x[i] = make_float2((float)v, 0.f);
    }
    kase = 1;
    isave1 = 5;
  }
  if (threadIdx.x == 0) {
    S.kase = kase;
    S.isave1 = isave1;
    S.isave2 = isave2;
    S.isave3 = isave3;
    S.est = est;
    mi1[blockIdx.x].active = kase == 1;
    mi2[blockIdx.x].active = kase == 2;
  }
}

void launch_lacn2(const Launch& L, Lacn2Dev* st, int ninst, float2* work, MatInst* mi1,
                  MatInst* mi2, int want) {
  k_lacn2<<<(unsigned)ninst, kLacT, 0, L.stream>>>(st, work, mi1, mi2, want);
  count_launch(1);
}

void launch_traces(const Launch& L, const TraceInst* d, int ninst, int64_t nmax, int32_t max_rhs) {
  dim3 g((unsigned)((nmax + 255) / 256), (unsigned)max_rhs, (unsigned)ninst);
  k_traces<<<g, 256, 0, L.stream>>>(d);
  count_launch(1);
}

void launch_cbie_forcing(const Launch& L, const TraceInst* d, int ninst, int64_t nmax,
                         int32_t max_rhs) {
  dim3 g((unsigned)((nmax + 255) / 256), (unsigned)max_rhs, (unsigned)ninst);
  k_cbie_forcing<<<g, 256, 0, L.stream>>>(d);
  count_launch(1);
}

void launch_stack(const Launch& L, const TraceInst* d, int ninst, int64_t nmax, int32_t max_rhs) {
  dim3 g((unsigned)((nmax + 255) / 256), (unsigned)max_rhs, (unsigned)ninst);
  k_stack<<<g, 256, 0, L.stream>>>(d);
  count_launch(1);
}

void launch_fill(const Launch& L, double* p, int64_t count, double v) {
  if (count <= 0) return;
  k_fill<<<(unsigned)((count + 255) / 256), 256, 0, L.stream>>>(p, count, v);
  count_launch(1);
}

}  // namespace bemgpu
