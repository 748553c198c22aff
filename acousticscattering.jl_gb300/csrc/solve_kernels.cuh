// Descriptors and launch declarations of the elementwise solve-chain kernels.
#pragma once

#include "bemgpu_internal.h"

namespace bemgpu {

struct TraceInst {
  const double* x;     // solution (N x nrhs, ld ldx) or product y for the CBIE forcing
  int64_t ldx;
  const double* pinc;  // incident traces (n x nrhs, ld n)
  const double* qinc;
  int64_t n;
  double* ps;          // scattered traces out (n x nrhs) / forcing out (2n x nrhs)
  double* qs;
  int32_t nrhs;
  int32_t kind;            // traces: 0 rigid, 1 soft, 2 Mueller, 3 fluid CBIE, 4 regions
  const int8_t* outer;     // regions: panel borders the exterior (forcing and far field)
  int32_t stack_q;         // regions forcing: the second block gets q_inc (Mueller)
  int32_t pad;
};

// Device state of LAPACK's zlacn2 reverse communication for one factor (the 1-norm
// estimate of gecon); its vector is complex64 at work + off.
struct Lacn2Dev {
  int64_t off;
  int32_t n, kase, isave1, isave2, isave3, pad;
  double est;
};

#ifdef __CUDACC__
// One zlacn2 step for every instance whose kase == want (want = 0: the first call); the
// next product is flagged active in mi1 (kase 1) or mi2 (kase 2).
void launch_lacn2(const Launch& L, Lacn2Dev* st, int ninst, float2* work, MatInst* mi1,
                  MatInst* mi2, int want);
void launch_traces(const Launch& L, const TraceInst* d, int ninst, int64_t nmax, int32_t max_rhs);
void launch_cbie_forcing(const Launch& L, const TraceInst* d, int ninst, int64_t nmax,
                         int32_t max_rhs);
void launch_stack(const Launch& L, const TraceInst* d, int ninst, int64_t nmax, int32_t max_rhs);
void launch_fill(const Launch& L, double* p, int64_t count, double v);
#endif

}  // namespace bemgpu
