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
