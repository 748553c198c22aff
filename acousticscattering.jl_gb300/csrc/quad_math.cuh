// Device quadrature mathematics of the collocation BEM.
//
// Kernels (outgoing exp(ikr), time factor exp(-i w t), numerics/helmholtz.jl:6-9 of the
// reference), with u = y - x, r = |u|:
//   G  = e^{ikr} / (4 pi r)
//   D  = dG/dn_y = e^{ikr} (ikr - 1) (u.n_y) / (4 pi r^3)
//   K' = dG/dn_x = -e^{ikr} (ikr - 1) (u.n_x) / (4 pi r^3)
//   H  = d2G/dn_x dn_y = e^{ikr}/(4 pi r^3) [(1 - ikr) n_x.n_y - (3 - 3ikr - k^2 r^2) c],
//        c = (u.n_x)(u.n_y) / r^2
// Near pairs split each operator into its Laplace part on the flat source triangle,
// integrated in closed form, and a bounded remainder integrated by the 7-point rule
// (21 points on the self panel, split at the centroid):
//   S  = S0 + sum w (e^{iz} - 1)/(4 pi r)
//   D  = D0 + sum w E2(z) (u.n_y)/(4 pi r^3)            E2 = e^{iz}(iz - 1) + 1
//   K' = K0 - sum w E2(z) (u.n_x)/(4 pi r^3)
//   H  = H0 + (k^2/2)(n_x.n_y) S0 + sum w [E1(z) n_x.n_y - E3(z) c]/(4 pi r^3)
//        E1 = e^{iz}(1 - iz) - 1 - z^2/2,  E3 = e^{iz}(3 - 3iz - z^2) - 3
// with z = kr and power series below z = 0.5 to avoid cancellation.
// Closed forms (flat triangle, outward edge normals m = s x n):
//   int 1/R        = sum_e t0_e f_e + d Omega
//   grad int 1/R   = -sum_e m_e f_e + n Omega
//   grad D-layer   = -sum_e (s_e x w_e) [(L - s0)/R_b + s0/R_a] / |s_e x w_e|^2
//   Omega          = 2 atan2(R0.(R1 x R2), r0 r1 r2 + (R0.R1) r2 + (R0.R2) r1 + (R1.R2) r0)
#pragma once

#include <cuda_runtime.h>

namespace bemgpu {

constexpr double kInv4Pi = 0.079577471545947667884;  // 1 / (4 pi)
constexpr double kSeriesZ = 0.5;

// Radon's rule in constant memory (same values as kRuleW / kRuleB).
static __constant__ double dRuleW[7] = {
    0.225, 0.13239415278850618074, 0.13239415278850618074, 0.13239415278850618074,
    0.12593918054482715260, 0.12593918054482715260, 0.12593918054482715260};
static __constant__ double dRuleB[7][3] = {
    {1.0 / 3.0, 1.0 / 3.0, 1.0 / 3.0},
    {0.05971587178976982046, 0.47014206410511508977, 0.47014206410511508977},
    {0.47014206410511508977, 0.05971587178976982046, 0.47014206410511508977},
    {0.47014206410511508977, 0.47014206410511508977, 0.05971587178976982046},
    {0.79742698535308732240, 0.10128650732345633880, 0.10128650732345633880},
    {0.10128650732345633880, 0.79742698535308732240, 0.10128650732345633880},
    {0.10128650732345633880, 0.10128650732345633880, 0.79742698535308732240}};

template <typename R>
struct cx {
  R x, y;
};
using cd = cx<double>;
using cf = cx<float>;

template <typename R>
__device__ __forceinline__ cx<R> operator+(cx<R> a, cx<R> b) { return {a.x + b.x, a.y + b.y}; }
template <typename R>
__device__ __forceinline__ cx<R> operator-(cx<R> a, cx<R> b) { return {a.x - b.x, a.y - b.y}; }
template <typename R>
__device__ __forceinline__ cx<R> operator*(cx<R> a, cx<R> b) {
  return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
template <typename R>
__device__ __forceinline__ cx<R> operator*(R s, cx<R> a) { return {s * a.x, s * a.y}; }
template <typename R>
__device__ __forceinline__ cx<R>& operator+=(cx<R>& a, cx<R> b) {
  a.x += b.x;
  a.y += b.y;
  return a;
}
template <typename R>
__device__ __forceinline__ cx<R>& operator-=(cx<R>& a, cx<R> b) {
  a.x -= b.x;
  a.y -= b.y;
  return a;
}

__device__ __forceinline__ double dot3(const double* a, const double* b) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}
__device__ __forceinline__ void sub3(const double* a, const double* b, double* o) {
  o[0] = a[0] - b[0];
  o[1] = a[1] - b[1];
  o[2] = a[2] - b[2];
}
__device__ __forceinline__ void cross3(const double* a, const double* b, double* o) {
  o[0] = a[1] * b[2] - a[2] * b[1];
  o[1] = a[2] * b[0] - a[0] * b[2];
  o[2] = a[0] * b[1] - a[1] * b[0];
}

// Four operators of one panel pair at one wavenumber.
struct Ops {
  cd S, D, K, H;
};

// Power-series coefficients of the remainder functions in z (i^m folded in):
// E(z) = sum_m c_m (iz)^m, Re E = sum_j re[j] z^{2j}, Im E = z sum_j im[j] z^{2j}, with
// c_m = 1/m! (E0), (1-m)/m! (E1), (m-1)/m! (E2), (m-1)(m-3)/m! (E3), m = 0..17.
struct SeriesTab {
  double re[4][9];
  double im[4][9];
};
__host__ __device__ constexpr double series_c(int e, int m) {
  double f = 1.0;
  for (int t = 2; t <= m; ++t) f *= (double)t;
  const double num = e == 0 ? (m >= 1 ? 1.0 : 0.0)
                   : e == 1 ? (m >= 3 ? (double)(1 - m) : 0.0)
                   : e == 2 ? (m >= 2 ? (double)(m - 1) : 0.0)
                            : (m >= 2 ? (double)((m - 1) * (m - 3)) : 0.0);
  return num / f;
}
__host__ __device__ constexpr SeriesTab make_series() {
  SeriesTab t{};
  for (int e = 0; e < 4; ++e)
    for (int j = 0; j < 9; ++j) {
      const int me = 2 * j, mo = 2 * j + 1;
      t.re[e][j] = ((j & 1) ? -1.0 : 1.0) * series_c(e, me);   // i^{2j} = (-1)^j
      t.im[e][j] = ((j & 1) ? -1.0 : 1.0) * series_c(e, mo);   // i^{2j+1} = i (-1)^j
    }
  return t;
}
static __constant__ SeriesTab dSeries = make_series();

__device__ __forceinline__ cd series_eval(int e, double z, double z2) {
  double re = dSeries.re[e][8], im = dSeries.im[e][8];
#pragma unroll
  for (int j = 7; j >= 0; --j) {
    re = fma(re, z2, dSeries.re[e][j]);
    im = fma(im, z2, dSeries.im[e][j]);
  }
  return cd{re, im * z};
}

__device__ __forceinline__ void remainder_funcs(double z, cd& E0, cd& E1, cd& E2, cd& E3) {
  if (z < kSeriesZ) {
    // 18 terms: the first omitted term is below z^18/18! < 1e-21 for z < 0.5
    const double z2 = z * z;
    E0 = series_eval(0, z, z2);
    E1 = series_eval(1, z, z2);
    E2 = series_eval(2, z, z2);
    E3 = series_eval(3, z, z2);
  } else {
    double sn, cs;
    sincos(z, &sn, &cs);
    cd e = {cs, sn};
    E0 = cd{cs - 1.0, sn};
    E1 = e * cd{1.0, -z} - cd{1.0 + 0.5 * z * z, 0.0};
    E2 = e * cd{-1.0, z} + cd{1.0, 0.0};
    E3 = e * cd{3.0 - z * z, -3.0 * z} - cd{3.0, 0.0};
  }
}

// Remainder kernels at one source point (near pairs).
__device__ __forceinline__ void rem_point(double k, const double* u, const double* nx,
                                          const double* ny, double w, Ops& o) {
  double r2 = dot3(u, u);
  double r = sqrt(r2);
  double z = k * r;
  cd E0, E1, E2, E3;
  remainder_funcs(z, E0, E1, E2, E3);
  double uny = dot3(u, ny), unx = dot3(u, nx), nn = dot3(nx, ny);
  double ir = 1.0 / r, ir3 = ir * ir * ir;
  double c = unx * uny * ir * ir;
  o.S += (w * kInv4Pi * ir) * E0;
  o.D += (w * kInv4Pi * ir3 * uny) * E2;
  o.K -= (w * kInv4Pi * ir3 * unx) * E2;
  o.H += (w * kInv4Pi * ir3) * (nn * E1 - c * E3);
}

// ---- FP32 remainders (near pairs of the mixed-precision assembly).  The Laplace parts
// stay FP64; only the bounded remainders are summed in FP32, from source-to-target
// offsets formed in FP64, so their relative error is that of the FP32 regular pairs.
// The series branch is taken below z = 1, where the closed forms would lose up to a
// factor 5 to cancellation; 7 even/odd pairs leave z^14/14! < 1.2e-11 at z = 1.
constexpr float kSeriesZf = 1.0f;
constexpr int kSeriesPairsF = 7;
struct SeriesTabF {
  float re[4][kSeriesPairsF];
  float im[4][kSeriesPairsF];
};
__host__ __device__ constexpr SeriesTabF make_series_f() {
  SeriesTabF t{};
  const SeriesTab d = make_series();
  for (int e = 0; e < 4; ++e)
    for (int j = 0; j < kSeriesPairsF; ++j) {
      t.re[e][j] = (float)d.re[e][j];
      t.im[e][j] = (float)d.im[e][j];
    }
  return t;
}
static __constant__ SeriesTabF dSeriesF = make_series_f();

__device__ __forceinline__ cf series_eval_f(int e, float z, float z2) {
  float re = dSeriesF.re[e][kSeriesPairsF - 1], im = dSeriesF.im[e][kSeriesPairsF - 1];
#pragma unroll
  for (int j = kSeriesPairsF - 2; j >= 0; --j) {
    re = fmaf(re, z2, dSeriesF.re[e][j]);
    im = fmaf(im, z2, dSeriesF.im[e][j]);
  }
  return cf{re, im * z};
}

__device__ __forceinline__ void remainder_funcs_f(float z, cf& E0, cf& E1, cf& E2, cf& E3) {
  if (z < kSeriesZf) {
    const float z2 = z * z;
    E0 = series_eval_f(0, z, z2);
    E1 = series_eval_f(1, z, z2);
    E2 = series_eval_f(2, z, z2);
    E3 = series_eval_f(3, z, z2);
  } else {
    float sn, cs;
    sincosf(z, &sn, &cs);
    const cf e = {cs, sn};
    E0 = cf{cs - 1.0f, sn};
    E1 = e * cf{1.0f, -z} - cf{1.0f + 0.5f * z * z, 0.0f};
    E2 = e * cf{-1.0f, z} + cf{1.0f, 0.0f};
    E3 = e * cf{3.0f - z * z, -3.0f * z} - cf{3.0f, 0.0f};
  }
}

struct OpsF {
  cf S, D, K, H;
};

// w already carries 1/(4 pi).
__device__ __forceinline__ void rem_point_f(float k, const float* u, const float* nx,
                                            const float* ny, float w, OpsF& o) {
  const float r2 = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
  const float r = sqrtf(r2), ir = 1.0f / r;
  cf E0, E1, E2, E3;
  remainder_funcs_f(k * r, E0, E1, E2, E3);
  const float uny = u[0] * ny[0] + u[1] * ny[1] + u[2] * ny[2];
  const float unx = u[0] * nx[0] + u[1] * nx[1] + u[2] * nx[2];
  const float nn = nx[0] * ny[0] + nx[1] * ny[1] + nx[2] * ny[2];
  const float ir3 = ir * ir * ir, c = unx * uny * ir * ir;
  o.S += (w * ir) * E0;
  o.D += (w * ir3 * uny) * E2;
  o.K -= (w * ir3 * unx) * E2;
  o.H += (w * ir3) * (nn * E1 - c * E3);
}

// Closed-form Laplace parts of a flat triangle (v: 9 doubles, nT: unit normal) at x
// with target normal nx.  self: x is the triangle's own centroid (principal values).
__device__ __forceinline__ void laplace_parts(const double* v, const double* nT,
                                              const double* x, const double* nx, bool self,
                                              double& S0, double& D0, double& K0,
                                              double& H0) {
  double Pint = 0.0, gP[3] = {0.0, 0.0, 0.0}, Hs = 0.0;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const double* Pa = v + 3 * a;
    const double* Pb = v + 3 * ((a + 1) % 3);
    double e[3], s[3], m[3], w[3], wb[3], sw[3];
    sub3(Pb, Pa, e);
    double L = sqrt(dot3(e, e));
    double iL = 1.0 / L;
    s[0] = e[0] * iL;
    s[1] = e[1] * iL;
    s[2] = e[2] * iL;
    cross3(s, nT, m);
    sub3(x, Pa, w);
    sub3(x, Pb, wb);
    double s0 = dot3(w, s);
    double sm = -s0, sp = L - s0;
    double t0 = -dot3(w, m);
    double dpl = dot3(w, nT);
    double R02 = t0 * t0 + dpl * dpl;
    double Rm = sqrt(dot3(w, w)), Rp = sqrt(dot3(wb, wb));
    double f;
    if (sm >= 0.0)
      f = log((Rp + sp) / (Rm + sm));
    else if (sp <= 0.0)
      f = log((Rm - sm) / (Rp - sp));
    else
      f = log((Rp + sp) * (Rm - sm) / R02);
    Pint += t0 * f;
    gP[0] -= m[0] * f;
    gP[1] -= m[1] * f;
    gP[2] -= m[2] * f;
    cross3(s, w, sw);
    double rho2 = dot3(sw, sw);
    if (rho2 > 1e-24 * L * L) Hs += dot3(nx, sw) / rho2 * (sp / Rp - sm / Rm);
  }
  double Om = 0.0, d = 0.0;
  if (!self) {
    double R0[3], R1[3], R2[3], t[3];
    sub3(v, x, R0);
    sub3(v + 3, x, R1);
    sub3(v + 6, x, R2);
    double r0 = sqrt(dot3(R0, R0)), r1 = sqrt(dot3(R1, R1)), r2 = sqrt(dot3(R2, R2));
    cross3(R1, R2, t);
    double num = dot3(R0, t);
    double den = r0 * r1 * r2 + dot3(R0, R1) * r2 + dot3(R0, R2) * r1 + dot3(R1, R2) * r0;
    Om = 2.0 * atan2(num, den);
    double xp[3];
    sub3(x, v, xp);
    d = dot3(xp, nT);
  }
  S0 = kInv4Pi * (Pint + d * Om);
  D0 = -kInv4Pi * Om;
  K0 = kInv4Pi * (dot3(nx, gP) + dot3(nx, nT) * Om);
  H0 = -kInv4Pi * Hs;
}

// Near-pair operators of collocation point (x, nx) on source triangle (v, rec) at
// wavenumber k, given its closed-form Laplace parts.
__device__ __forceinline__ Ops near_ops(const double* v, const double* recj, const double* x,
                                        const double* nx, bool self, double k, double S0,
                                        double D0, double K0, double H0) {
  Ops o;
  o.S = o.D = o.K = o.H = cd{0.0, 0.0};
  const double* nT = recj + 3;
  const double area = recj[6];
  if (self) {
    const double* c = recj;  // centroid
    const double sa = area / 3.0;
#pragma unroll 1
    for (int a = 0; a < 3; ++a) {
      const double* Pa = v + 3 * a;
      const double* Pb = v + 3 * ((a + 1) % 3);
#pragma unroll 1
      for (int q = 0; q < 7; ++q) {
        double y[3], u[3];
        y[0] = dRuleB[q][0] * c[0] + dRuleB[q][1] * Pa[0] + dRuleB[q][2] * Pb[0];
        y[1] = dRuleB[q][0] * c[1] + dRuleB[q][1] * Pa[1] + dRuleB[q][2] * Pb[1];
        y[2] = dRuleB[q][0] * c[2] + dRuleB[q][1] * Pa[2] + dRuleB[q][2] * Pb[2];
        sub3(y, x, u);
        rem_point(k, u, nx, nT, dRuleW[q] * sa, o);
      }
    }
  } else {
#pragma unroll 1
    for (int q = 0; q < 7; ++q) {
      double u[3];
      sub3(recj + 8 + 3 * q, x, u);
      rem_point(k, u, nx, nT, dRuleW[q] * area, o);
    }
  }
  double nn = dot3(nx, nT);
  o.S += cd{S0, 0.0};
  o.D += cd{D0, 0.0};
  o.K += cd{K0, 0.0};
  o.H += cd{H0 + 0.5 * k * k * nn * S0, 0.0};
  return o;
}

// near_ops with the remainders in FP32 (same points and weights).
__device__ __forceinline__ Ops near_ops_f(const double* v, const double* recj, const double* x,
                                          const double* nx, bool self, double k, double S0,
                                          double D0, double K0, double H0) {
  OpsF o;
  o.S = o.D = o.K = o.H = cf{0.0f, 0.0f};
  const double* nT = recj + 3;
  const float nxf[3] = {(float)nx[0], (float)nx[1], (float)nx[2]};
  const float nTf[3] = {(float)nT[0], (float)nT[1], (float)nT[2]};
  const float kf = (float)k;
  const double area = recj[6];
  if (self) {
    const double* c = recj;
    const float sa = (float)(area / 3.0 * kInv4Pi);
#pragma unroll 1
    for (int a = 0; a < 3; ++a) {
      const double* Pa = v + 3 * a;
      const double* Pb = v + 3 * ((a + 1) % 3);
#pragma unroll 1
      for (int q = 0; q < 7; ++q) {
        float u[3];
#pragma unroll
        for (int t = 0; t < 3; ++t)
          u[t] = (float)(dRuleB[q][0] * c[t] + dRuleB[q][1] * Pa[t] + dRuleB[q][2] * Pb[t] -
                         x[t]);
        rem_point_f(kf, u, nxf, nTf, (float)dRuleW[q] * sa, o);
      }
    }
  } else {
    const float sa = (float)(area * kInv4Pi);
#pragma unroll
    for (int q = 0; q < 7; ++q) {
      const float u[3] = {(float)(recj[8 + 3 * q] - x[0]), (float)(recj[9 + 3 * q] - x[1]),
                          (float)(recj[10 + 3 * q] - x[2])};
      rem_point_f(kf, u, nxf, nTf, (float)dRuleW[q] * sa, o);
    }
  }
  const double nn = dot3(nx, nT);
  Ops r;
  r.S = cd{S0 + (double)o.S.x, (double)o.S.y};
  r.D = cd{D0 + (double)o.D.x, (double)o.D.y};
  r.K = cd{K0 + (double)o.K.x, (double)o.K.y};
  r.H = cd{H0 + 0.5 * k * k * nn * S0 + (double)o.H.x, (double)o.H.y};
  return r;
}

}  // namespace bemgpu
