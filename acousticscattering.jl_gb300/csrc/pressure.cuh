// Descriptor and launch declaration of the point-evaluation kernel (pressure.cu).
#pragma once

#include "bemgpu_internal.h"

namespace bemgpu {

struct PressureInst {
  const double* panels;  // FP64 panel records
  const double* verts;   // vertex records
  int64_t n;             // panels
  const double* p;       // scattered pressure trace of one rhs (complex128, n)
  const double* q;       // scattered normal-derivative trace (complex128, n)
  const double* dir;     // incidence direction (3)
  const double* points;  // 3 x npts
  int64_t npts;
  double* out;           // complex128 npts
  int32_t* region;       // per point: 0 exterior, 1 interior, 2 on the surface
  double k, k_int, g, eta;
  int32_t field;         // bemgpu_field
  int32_t fluid;         // interior field exists
};

#ifdef __CUDACC__
void launch_pressure(const Launch& L, const PressureInst& P);
#endif

}  // namespace bemgpu
