// Field evaluation at points: the pressure query of the full-3D BEM solution
// (fields/pressure.jl:404-471 of the reference).
//
//   exterior:  u_s(x) = sum_j [ D_j(x) p_j - S_j(x) q_j ]           (scattered traces, k)
//   interior:  u_i(x) = sum_j [ S_j(x) g (q_j + q_inc,j) - D_j(x) (p_j + p_inc,j) ]  (k / h)
//   incident:  e^{ik d.x}
//
// S_j, D_j are the single- and double-layer potentials of the flat panel j with unit
// density: 7-point rule away from the panel, closed-form Laplace parts plus the
// Helmholtz remainders (quad_math.cuh) when x is within eta panel diameters.  The
// region of each point (inside / outside the closed surface) comes from the sum of the
// panels' solid angles (4 pi inside, 0 outside, 2 pi on the surface).  One CTA per
// point, fixed-order reductions, FP64 throughout.
#include "bemgpu_internal.h"
#include "pressure.cuh"
#include "quad_math.cuh"

namespace bemgpu {

constexpr int kPrThreads = 256;

__device__ __forceinline__ double solid_angle(const double* v, const double* x) {
  double R0[3], R1[3], R2[3], t[3];
  sub3(v, x, R0);
  sub3(v + 3, x, R1);
  sub3(v + 6, x, R2);
  const double r0 = sqrt(dot3(R0, R0)), r1 = sqrt(dot3(R1, R1)), r2 = sqrt(dot3(R2, R2));
  cross3(R1, R2, t);
  const double num = dot3(R0, t);
  const double den = r0 * r1 * r2 + dot3(R0, R1) * r2 + dot3(R0, R2) * r1 + dot3(R1, R2) * r0;
  return 2.0 * atan2(num, den);
}

template <int NT>
__device__ __forceinline__ double block_sum(double v, double* sh) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < NT / 32; ++w) t += sh[w];
  __syncthreads();
  if (threadIdx.x == 0) sh[0] = t;
  __syncthreads();
  return sh[0];
}

__global__ void __launch_bounds__(kPrThreads) k_pressure(const PressureInst P) {
  const int64_t ip = blockIdx.x;
  if (ip >= P.npts) return;
  __shared__ double sh[kPrThreads / 32];
  const double x[3] = {P.points[3 * ip], P.points[3 * ip + 1], P.points[3 * ip + 2]};
  const double zero3[3] = {0.0, 0.0, 0.0};
  // region by total solid angle
  double om = 0.0;
  for (int64_t j = threadIdx.x; j < P.n; j += kPrThreads)
    om += solid_angle(P.verts + j * kVertDoubles, x);
  om = block_sum<kPrThreads>(om, sh);
  const double four_pi = 12.566370614359172954;
  const bool inside = om > 0.5 * four_pi;
  const bool on_surface = fabs(om - 0.5 * four_pi) < 1e-6 * four_pi;
  int region = inside ? 1 : 0;  // 0 exterior, 1 interior
  if (on_surface) region = P.fluid ? 1 : 0;
  if (threadIdx.x == 0) P.region[ip] = on_surface ? 2 : region;
  const double* d = P.dir;
  const double ph_x = P.k * (d[0] * x[0] + d[1] * x[1] + d[2] * x[2]);
  double psn, pcs;
  sincos(ph_x, &psn, &pcs);
  if (P.field == 2) {  // incident only
    if (threadIdx.x == 0) {
      P.out[2 * ip] = pcs;
      P.out[2 * ip + 1] = psn;
    }
    return;
  }
  const bool interior = region == 1;
  if ((interior && !P.fluid) || (P.field == 3 && !interior) ||
      (P.field == 1 && interior)) {
    // the field does not exist at this point: NaN marks it for the host
    if (threadIdx.x == 0) {
      P.out[2 * ip] = NAN;
      P.out[2 * ip + 1] = NAN;
    }
    return;
  }
  const double k = interior ? P.k_int : P.k;
  double acc_r = 0.0, acc_i = 0.0;
  for (int64_t j = threadIdx.x; j < P.n; j += kPrThreads) {
    const double* rj = P.panels + j * kPanelDoubles;
    const double* nT = rj + 3;
    cd pj = {P.p[2 * j], P.p[2 * j + 1]}, qj = {P.q[2 * j], P.q[2 * j + 1]};
    if (interior) {  // total interior traces: p = p_s + p_inc, q = g (q_s + q_inc)
      const double ph = P.k * (d[0] * rj[0] + d[1] * rj[1] + d[2] * rj[2]);
      double sn, cs;
      sincos(ph, &sn, &cs);
      const double dn = P.k * (d[0] * nT[0] + d[1] * nT[1] + d[2] * nT[2]);
      pj = pj + cd{cs, sn};
      qj = P.g * (qj + cd{-dn * sn, dn * cs});
    }
    const double dx = x[0] - rj[0], dy = x[1] - rj[1], dz = x[2] - rj[2];
    const double d2 = dx * dx + dy * dy + dz * dz;
    const double lim = P.eta * rj[7];
    cd S = {0.0, 0.0}, D = {0.0, 0.0};
    if (d2 < lim * lim) {
      double v[9];
#pragma unroll
      for (int t = 0; t < 9; ++t) v[t] = P.verts[j * kVertDoubles + t];
      double S0, D0, K0, H0;
      laplace_parts(v, nT, x, zero3, false, S0, D0, K0, H0);
      Ops o;
      o.S = o.D = o.K = o.H = cd{0.0, 0.0};
#pragma unroll 1
      for (int q = 0; q < 7; ++q) {
        double u[3];
        sub3(rj + 8 + 3 * q, x, u);
        rem_point(k, u, zero3, nT, dRuleW[q] * rj[6], o);
      }
      S = o.S + cd{S0, 0.0};
      D = o.D + cd{D0, 0.0};
    } else {
#pragma unroll
      for (int q = 0; q < 7; ++q) {
        double u[3];
        sub3(rj + 8 + 3 * q, x, u);
        const double r2 = dot3(u, u);
        const double r = sqrt(r2), ir = 1.0 / r;
        const double z = k * r;
        double sn, cs;
        sincos(z, &sn, &cs);
        const double w = dRuleW[q] * rj[6] * kInv4Pi;
        const cd e = {cs, sn};
        S += (w * ir) * e;
        // dG/dn_y = e^{ikr}(ikr - 1)(u.n_y) / (4 pi r^3)
        D += (w * ir * ir * ir * dot3(u, nT)) * (e * cd{-1.0, z});
      }
    }
    cd c = interior ? (S * qj - D * pj) : (D * pj - S * qj);
    acc_r += c.x;
    acc_i += c.y;
  }
  acc_r = block_sum<kPrThreads>(acc_r, sh);
  acc_i = block_sum<kPrThreads>(acc_i, sh);
  if (threadIdx.x == 0) {
    double re = acc_r, im = acc_i;
    if (P.field == 0 && !interior) {  // total exterior = incident + scattered
      re += pcs;
      im += psn;
    }
    P.out[2 * ip] = re;
    P.out[2 * ip + 1] = im;
  }
}

// Single and double layer of panel j (unit density) at x with wavenumber k: closed-form
// Laplace parts plus remainders when x is within eta panel diameters, else the 7-point rule.
__device__ __forceinline__ void panel_layers(const PressureInst& P, int64_t j, const double* x,
                                             double k, cd& S, cd& D) {
  const double zero3[3] = {0.0, 0.0, 0.0};
  const double* rj = P.panels + j * kPanelDoubles;
  const double* nT = rj + 3;
  const double dx = x[0] - rj[0], dy = x[1] - rj[1], dz = x[2] - rj[2];
  const double d2 = dx * dx + dy * dy + dz * dz;
  const double lim = P.eta * rj[7];
  S = D = cd{0.0, 0.0};
  if (d2 < lim * lim) {
    double v[9];
#pragma unroll
    for (int t = 0; t < 9; ++t) v[t] = P.verts[j * kVertDoubles + t];
    double S0, D0, K0, H0;
    laplace_parts(v, nT, x, zero3, false, S0, D0, K0, H0);
    Ops o;
    o.S = o.D = o.K = o.H = cd{0.0, 0.0};
#pragma unroll 1
    for (int q = 0; q < 7; ++q) {
      double u[3];
      sub3(rj + 8 + 3 * q, x, u);
      rem_point(k, u, zero3, nT, dRuleW[q] * rj[6], o);
    }
    S = o.S + cd{S0, 0.0};
    D = o.D + cd{D0, 0.0};
  } else {
#pragma unroll
    for (int q = 0; q < 7; ++q) {
      double u[3];
      sub3(rj + 8 + 3 * q, x, u);
      const double r2 = dot3(u, u);
      const double r = sqrt(r2), ir = 1.0 / r;
      const double z = k * r;
      double sn, cs;
      sincos(z, &sn, &cs);
      const double w = dRuleW[q] * rj[6] * kInv4Pi;
      const cd e = {cs, sn};
      S += (w * ir) * e;
      D += (w * ir * ir * ir * dot3(u, nT)) * (e * cd{-1.0, z});
    }
  }
}

// Coupled regions (fields/regions.jl:1-65 of the reference): the region of the point by
// the reference's walk over the interfaces (an interface is tested only when its parent
// is the region found so far; the solid angle of its panels tells inside / on / outside),
// then the sum over the interfaces that border the region of S dp - D p (the region
// inside them) or D p - S dp (outside), with the region's wavenumber; in the unbounded
// region the traces are the scattered ones and the total field adds the incident wave.
__global__ void __launch_bounds__(kPrThreads) k_pressure_regions(const PressureInst P) {
  const int64_t ip = blockIdx.x;
  if (ip >= P.npts) return;
  __shared__ double sh[kPrThreads / 32];
  const double x[3] = {P.points[3 * ip], P.points[3 * ip + 1], P.points[3 * ip + 2]};
  const double four_pi = 12.566370614359172954;
  int containing = 0, adj_out = -1, adj_in = -1;
  for (int s = 0; s < P.nsurf; ++s) {
    if (P.parents[s] != containing) continue;  // uniform over the CTA
    double om = 0.0;
    for (int64_t j = P.offsets[s] + threadIdx.x; j < P.offsets[s + 1]; j += kPrThreads)
      om += solid_angle(P.verts + j * kVertDoubles, x);
    om = block_sum<kPrThreads>(om, sh);
    if (fabs(om - 0.5 * four_pi) < 1e-6 * four_pi) {
      adj_out = P.parents[s];
      adj_in = s + 1;
      break;
    }
    if (om > 0.5 * four_pi) containing = s + 1;
  }
  int region, status = 0;
  if (P.requested >= 0) {
    const bool valid = adj_in < 0 ? P.requested == containing
                                  : (P.requested == adj_out || P.requested == adj_in);
    if (!valid) status = kPrBadRegion;
    region = P.requested;
  } else if (adj_in >= 0) {
    region = P.field == 3 ? adj_in : adj_out;
  } else {
    region = containing;
  }
  if (!status && P.field == 1 && region != 0) status = kPrNeedExterior;
  if (!status && P.field == 3 && region == 0) status = kPrNeedFluid;
  const double* d = P.dir;
  double psn, pcs;
  sincos(P.k * (d[0] * x[0] + d[1] * x[1] + d[2] * x[2]), &psn, &pcs);
  if (threadIdx.x == 0) P.region[ip] = status ? -status : region;
  if (status || P.field == 2) {
    if (threadIdx.x == 0) {
      P.out[2 * ip] = status ? NAN : pcs;
      P.out[2 * ip + 1] = status ? NAN : psn;
    }
    return;
  }
  const double k = region == 0 ? P.k : P.kr[region];
  const int64_t n = P.offsets[P.nsurf];
  double acc_r = 0.0, acc_i = 0.0;
  for (int s = 0; s < P.nsurf; ++s) {
    const bool inside = s + 1 == region;
    if (!inside && P.parents[s] != region) continue;
    const double rho = inside ? P.rho[s + 1] : P.rho[P.parents[s]];
    for (int64_t j = P.offsets[s] + threadIdx.x; j < P.offsets[s + 1]; j += kPrThreads) {
      cd pj = {P.xr[2 * j], P.xr[2 * j + 1]};
      cd dp = rho * cd{P.xr[2 * (n + j)], P.xr[2 * (n + j) + 1]};
      if (region == 0) {  // scattered traces
        const double* rj = P.panels + j * kPanelDoubles;
        const double ph = P.k * (d[0] * rj[0] + d[1] * rj[1] + d[2] * rj[2]);
        double sn, cs;
        sincos(ph, &sn, &cs);
        const double dn = P.k * (d[0] * rj[3] + d[1] * rj[4] + d[2] * rj[5]);
        pj = pj - cd{cs, sn};
        dp = dp - cd{-dn * sn, dn * cs};
      }
      cd S, D;
      panel_layers(P, j, x, k, S, D);
      const cd c = inside ? (S * dp - D * pj) : (D * pj - S * dp);
      acc_r += c.x;
      acc_i += c.y;
    }
  }
  acc_r = block_sum<kPrThreads>(acc_r, sh);
  acc_i = block_sum<kPrThreads>(acc_i, sh);
  if (threadIdx.x == 0) {
    double re = acc_r, im = acc_i;
    if (P.field == 0 && region == 0) {
      re += pcs;
      im += psn;
    }
    P.out[2 * ip] = re;
    P.out[2 * ip + 1] = im;
  }
}

void launch_pressure(const Launch& L, const PressureInst& P) {
  if (P.npts <= 0) return;
  if (P.nsurf > 0)
    k_pressure_regions<<<(unsigned)P.npts, kPrThreads, 0, L.stream>>>(P);
  else
    k_pressure<<<(unsigned)P.npts, kPrThreads, 0, L.stream>>>(P);
  count_launch(1);
}

}  // namespace bemgpu
