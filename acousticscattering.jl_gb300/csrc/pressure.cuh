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
  // coupled regions (nsurf > 0; p, q, k_int, g, fluid unused): surface s encloses region
  // s + 1 and borders region parents[s]; xr holds the solved [p; v] (complex128, 2n)
  int32_t nsurf;
  int32_t requested;                 // region asked for, -1: the point's own
  const double* xr;
  int64_t offsets[kMaxRegions + 1];  // first panel of every surface, then n
  int32_t parents[kMaxRegions];
  double kr[kMaxRegions + 1];        // wavenumber of every region
  double rho[kMaxRegions + 1];       // density contrast of every region (region 0: 1)
};

// Region pressure status per point (PressureInst.region in region mode, as -code):
constexpr int kPrBadRegion = 1;      // the point does not belong to the requested region
constexpr int kPrNeedExterior = 2;   // field scattered outside the unbounded region
constexpr int kPrNeedFluid = 3;      // field interior in the unbounded region

#ifdef __CUDACC__
void launch_pressure(const Launch& L, const PressureInst& P);  // either mode
#endif

}  // namespace bemgpu
