// Regular 7-point rule of the collocation BEM (device): the FP64 / FP32 precision traits
// and the four Helmholtz kernels of one source panel at one collocation point.  Shared by
// the dense assembly and the hierarchical-matrix kernels so that both evaluate the same
// entries.
#pragma once

#include "bemgpu_internal.h"
#include "quad_math.cuh"

namespace bemgpu {

constexpr int kAsmCols64 = 64;     // FP64 source records per chunk (64 x 256 B = 16 KB)
constexpr int kAsmCols32 = 128;    // FP32 source records per chunk (128 x 128 B = 16 KB)

template <typename R>
struct Prec;
template <>
struct Prec<double> {
  static constexpr int kCols = kAsmCols64;
  static constexpr int kRec = kPanelDoubles;
  __device__ static __forceinline__ void sc(double z, double* s, double* c) { sincos(z, s, c); }
  __device__ static __forceinline__ double rs(double x) { return rsqrt(x); }
  __device__ static __forceinline__ const double* recs(const AsmInst& I) { return I.panels; }
};
template <>
struct Prec<float> {
  static constexpr int kCols = kAsmCols32;
  static constexpr int kRec = kPanelFloats;
  // sin/cos of pi * t with exact argument reduction
  __device__ static __forceinline__ void sc(float z, float* s, float* c) {
    sincospif(z * 0.31830988618379067154f, s, c);
  }
  __device__ static __forceinline__ float rs(float x) { return rsqrtf(x); }
  __device__ static __forceinline__ const float* recs(const AsmInst& I) { return I.panelsf; }
};

template <typename R>
struct Acc {
  cx<R> S, D, K, H;
};

// Full Helmholtz kernels of one source panel (7 points) at one wavenumber.
template <typename R, bool NEED_KH>
__device__ __forceinline__ void regular_panel(const R* rec, const R x[3], const R nx[3], R k,
                                              Acc<R>& a) {
  const R ny0 = rec[3], ny1 = rec[4], ny2 = rec[5];
  const R area = rec[6];
  const R nn = nx[0] * ny0 + nx[1] * ny1 + nx[2] * ny2;
#pragma unroll
  for (int q = 0; q < 7; ++q) {
    const R u0 = rec[8 + 3 * q] - x[0];
    const R u1 = rec[9 + 3 * q] - x[1];
    const R u2 = rec[10 + 3 * q] - x[2];
    const R r2 = u0 * u0 + u1 * u1 + u2 * u2;
    const R ir = Prec<R>::rs(r2);
    const R r = r2 * ir;
    const R z = k * r;
    R sn, cs;
    Prec<R>::sc(z, &sn, &cs);
    const R w = (R)dRuleW[q] * area * (R)kInv4Pi;
    const R wir = w * ir;
    const R ir2 = ir * ir;
    a.S += wir * cx<R>{cs, sn};
    const R uny = u0 * ny0 + u1 * ny1 + u2 * ny2;
    // e^{iz} (iz - 1) w / (4 pi r^3)
    const cx<R> gp = (wir * ir2) * cx<R>{-cs - z * sn, -sn + z * cs};
    a.D += uny * gp;
    if (NEED_KH) {
      const R unx = u0 * nx[0] + u1 * nx[1] + u2 * nx[2];
      a.K -= unx * gp;
      const R c = unx * uny * ir2;
      // e^{iz} [(nn - c (3 - z^2)) + i z (3c - nn)] w / (4 pi r^3)
      const cx<R> br = {nn - c * ((R)3 - z * z), z * ((R)3 * c - nn)};
      a.H += (wir * ir2) * (cx<R>{cs, sn} * br);
    }
  }
}

}  // namespace bemgpu
