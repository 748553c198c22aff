// Assembly, incident-field and far-field kernels of the collocation BEM.
//
// Regular pairs: each CTA owns a tile of kAsmRows collocation points (one per thread)
// and a chunk of source panels whose records (centroid, normal, area, Gauss points)
// are staged in shared memory by one bulk asynchronous copy (TMA engine).  All threads
// of a warp read the same source record (shared-memory broadcast) and write the
// column-major matrix entry of their own row, so every warp store is 32 consecutive
// complex values (256 or 512 contiguous bytes).  The mixed-precision system is stored
// as complex64 (exact for the FP32 rule); the FP64 near values it cannot hold exactly
// keep their rounding error in a sparse correction list.
// Near pairs: one thread per listed pair evaluates the FP64 singular rules and
// overwrites the regular value (stream order guarantees the regular kernel ran first).
#include <cstdio>

#include "bemgpu_internal.h"
#include "quad_math.cuh"
#include "quad_regular.cuh"
#include "tma.cuh"

namespace bemgpu {

constexpr int kAsmRows = 128;      // threads per CTA = collocation points per tile

__device__ __forceinline__ void store_c(void* base, int64_t idx, cd v) {
  reinterpret_cast<double2*>(base)[idx] = make_double2(v.x, v.y);
}
// regular entry: complex64 outputs take the value as computed (exact for the FP32 rule)
template <typename R>
__device__ __forceinline__ void store_r(void* base, bool c64, int64_t idx, cx<R> v) {
  if (c64)
    reinterpret_cast<float2*>(base)[idx] = make_float2((float)v.x, (float)v.y);
  else
    reinterpret_cast<double2*>(base)[idx] = make_double2((double)v.x, (double)v.y);
}
// near entry: complex64 outputs keep the FP64 rounding error as a correction
__device__ __forceinline__ void store_n(void* base, bool c64, double* dnear, int64_t dpos,
                                        int64_t idx, cd v) {
  if (c64) {
    const float2 f = make_float2((float)v.x, (float)v.y);
    reinterpret_cast<float2*>(base)[idx] = f;
    reinterpret_cast<double2*>(dnear)[dpos] = make_double2(v.x - (double)f.x, v.y - (double)f.y);
  } else {
    store_c(base, idx, v);
  }
}

template <typename R, int KIND>
__global__ void __launch_bounds__(kAsmRows) k_assemble_regular(const AsmInst* __restrict__ insts,
                                                               int* err) {
  constexpr int kCols = Prec<R>::kCols;
  constexpr int kRec = Prec<R>::kRec;
  __shared__ alignas(128) R srec[kCols * kRec];
  __shared__ alignas(8) uint64_t bar;
  const AsmInst& I = insts[blockIdx.z];
  const int64_t n = I.n;
  const int64_t i0 = (int64_t)blockIdx.x * kAsmRows;
  const int64_t j0 = (int64_t)blockIdx.y * kCols;
  if (i0 >= n || j0 >= n) return;  // uniform over the CTA
  const int cnt = (int)min((int64_t)kCols, n - j0);
  const R* recs = Prec<R>::recs(I);
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    mbar_fence_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const uint32_t bytes = (uint32_t)(cnt * kRec * sizeof(R));
    mbar_arrive_expect_tx(&bar, bytes);
    bulk_g2s(srec, recs + j0 * kRec, bytes, &bar);
  }
  const int64_t i = i0 + threadIdx.x;
  const bool row_ok = i < n;
  R x[3] = {0, 0, 0}, nx[3] = {0, 0, 1};
  if (row_ok) {
    const R* ri = recs + i * kRec;
    x[0] = ri[0]; x[1] = ri[1]; x[2] = ri[2];
    nx[0] = ri[3]; nx[1] = ri[4]; nx[2] = ri[5];
  }
  const bool ok = mbar_wait(&bar, 0, err);
  if (!ok || !row_ok) return;
  const R ke = (R)I.k_e, ki = (R)I.k_i;
  const int64_t lda = I.lda;
  const int si = KIND == kAsmRegion ? I.surf[i] : 0;
  for (int jj = 0; jj < cnt; ++jj) {
    const int64_t j = j0 + jj;
    if (j == i) continue;  // self pair: near kernel
    const R* rec = srec + jj * kRec;
    if (KIND == kAsmBM || KIND == kAsmCBIE) {
      Acc<R> a;
      a.S = a.D = a.K = a.H = cx<R>{0, 0};
      regular_panel<R, KIND == kAsmBM>(rec, x, nx, ke, a);
      cx<R> m1 = cx<R>{-a.D.x, -a.D.y}, m2 = a.S;
      if (KIND == kAsmBM) {
        const cx<R> al = {(R)I.a_re, (R)I.a_im};
        m1 -= al * a.H;
        m2 += al * a.K;
      }
      store_r(I.out1, (I.c64 & 1) != 0, i + j * lda, m1);
      store_r(I.out2, (I.c64 & 2) != 0, i + j * lda, m2);
    } else if (KIND == kAsmRegion) {
      const RegionTable& RT = *I.region;
      const RegionCoef& C = RT.c[si * kMaxRegions + I.surf[j]];
      cx<R> a11 = {0, 0}, a12 = {0, 0}, a21 = {0, 0}, a22 = {0, 0};
      for (int q = 0; q < C.count; ++q) {
        Acc<R> t;
        t.S = t.D = t.K = t.H = cx<R>{0, 0};
        const R kq = (R)RT.kr[C.kidx[q]];
        if (RT.cbie)
          regular_panel<R, false>(rec, x, nx, kq, t);
        else
          regular_panel<R, true>(rec, x, nx, kq, t);
        const R sg = (R)C.sign[q], rho = (R)C.rho[q];
        if (!RT.cbie) {
          a11 += sg * t.D;
          a12 -= (sg * rho) * t.S;
          a21 += (sg / rho) * t.H;
          a22 -= sg * t.K;
        } else if (C.eq[q] == 0) {
          a11 += sg * t.D;
          a12 -= (sg * rho) * t.S;
        } else {
          a21 += sg * t.D;
          a22 -= (sg * rho) * t.S;
        }
      }
      const bool c64 = (I.c64 & 1) != 0;
      store_r(I.out1, c64, i + j * lda, a11);
      store_r(I.out1, c64, i + (n + j) * lda, a12);
      store_r(I.out1, c64, (n + i) + j * lda, a21);
      store_r(I.out1, c64, (n + i) + (n + j) * lda, a22);
    } else {
      Acc<R> e, t;
      e.S = e.D = e.K = e.H = cx<R>{0, 0};
      t = e;
      constexpr bool kh = (KIND == kAsmMuller);
      regular_panel<R, kh>(rec, x, nx, ke, e);
      regular_panel<R, kh>(rec, x, nx, ki, t);
      // block combinations in the quadrature precision (no FP64 work on the FP32 path)
      const R g = (R)I.g, ginv = (R)(1.0 / I.g);
      cx<R> a11, a12, a21, a22;
      if (KIND == kAsmMuller) {
        a11 = t.D - e.D;
        a12 = e.S - g * t.S;
        a21 = ginv * t.H - e.H;
        a22 = e.K - t.K;
      } else {
        a11 = cx<R>{-e.D.x, -e.D.y};
        a12 = e.S;
        a21 = t.D;
        a22 = cx<R>{-g * t.S.x, -g * t.S.y};
      }
      const bool c64 = (I.c64 & 1) != 0;
      store_r(I.out1, c64, i + j * lda, a11);
      store_r(I.out1, c64, i + (n + j) * lda, a12);
      store_r(I.out1, c64, (n + i) + j * lda, a21);
      store_r(I.out1, c64, (n + i) + (n + j) * lda, a22);
    }
  }
}

template <int KIND, bool F32>
__device__ __forceinline__ Ops near_pair(const double* v, const double* rj, const double* x,
                                         const double* nx, bool self, double k, double S0,
                                         double D0, double K0, double H0) {
  if (F32) return near_ops_f(v, rj, x, nx, self, k, S0, D0, K0, H0);
  return near_ops(v, rj, x, nx, self, k, S0, D0, K0, H0);
}

// F32: remainders in FP32 (mixed-precision assembly); the Laplace parts and the block
// combinations stay FP64.
template <int KIND, bool F32>
__global__ void __launch_bounds__(128) k_assemble_near(const AsmInst* __restrict__ insts) {
  const AsmInst& I = insts[blockIdx.z];
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= I.n_near) return;
  const int64_t i = I.near_i[p], j = I.near_j[p];
  const double* ri = I.panels + i * kPanelDoubles;
  const double* rj = I.panels + j * kPanelDoubles;
  double v[9];
#pragma unroll
  for (int t = 0; t < 9; ++t) v[t] = I.verts[j * kVertDoubles + t];
  double x[3] = {ri[0], ri[1], ri[2]}, nx[3] = {ri[3], ri[4], ri[5]};
  const bool self = (i == j);
  const double4 lp = reinterpret_cast<const double4*>(I.near_lap)[p];
  const double S0 = lp.x, D0 = lp.y, K0 = lp.z, H0 = lp.w;
  const int64_t n = I.n, lda = I.lda;
  const double delta = self ? 1.0 : 0.0;
  if (KIND == kAsmBM || KIND == kAsmCBIE) {
    Ops o = near_pair<KIND, F32>(v, rj, x, nx, self, I.k_e, S0, D0, K0, H0);
    cd m1 = cd{0.5 * delta - o.D.x, -o.D.y};
    cd m2 = o.S;
    if (KIND == kAsmBM) {
      cd al = {I.a_re, I.a_im};
      m1 -= al * o.H;
      m2 += al * (o.K + cd{0.5 * delta, 0.0});
    }
    const int64_t dst = I.near_dst ? I.near_dst[p] : i + j * lda;
    store_n(I.out1, (I.c64 & 1) != 0, I.dnear, p, dst, m1);
    store_n(I.out2, (I.c64 & 2) != 0, I.dnear2, p, dst, m2);
  } else if (KIND == kAsmRegion) {
    const RegionTable& RT = *I.region;
    const RegionCoef& C = RT.c[I.surf[i] * kMaxRegions + I.surf[j]];
    cd a11, a12 = {0.0, 0.0}, a21, a22 = {0.0, 0.0};
    if (RT.cbie) {  // 1/2 I in both equation rows (one per region of the interface)
      a11 = cd{0.5 * delta, 0.0};
      a21 = cd{0.5 * delta, 0.0};
    } else {
      a11 = cd{delta, 0.0};
      a22 = cd{delta, 0.0};
      a21 = cd{0.0, 0.0};
    }
    for (int q = 0; q < C.count; ++q) {
      const Ops o = near_pair<KIND, F32>(v, rj, x, nx, self, RT.kr[C.kidx[q]], S0, D0, K0, H0);
      const double sg = C.sign[q], rho = C.rho[q];
      if (!RT.cbie) {
        a11 += sg * o.D;
        a12 -= (sg * rho) * o.S;
        a21 += (sg / rho) * o.H;
        a22 -= sg * o.K;
      } else if (C.eq[q] == 0) {
        a11 += sg * o.D;
        a12 -= (sg * rho) * o.S;
      } else {
        a21 += sg * o.D;
        a22 -= (sg * rho) * o.S;
      }
    }
    const bool c64 = (I.c64 & 1) != 0;
    const int64_t nn = I.n_near;
    store_n(I.out1, c64, I.dnear, p, i + j * lda, a11);
    store_n(I.out1, c64, I.dnear, nn + p, i + (n + j) * lda, a12);
    store_n(I.out1, c64, I.dnear, 2 * nn + p, (n + i) + j * lda, a21);
    store_n(I.out1, c64, I.dnear, 3 * nn + p, (n + i) + (n + j) * lda, a22);
  } else {
    Ops e = near_pair<KIND, F32>(v, rj, x, nx, self, I.k_e, S0, D0, K0, H0);
    Ops t = near_pair<KIND, F32>(v, rj, x, nx, self, I.k_i, S0, D0, K0, H0);
    const double g = I.g;
    cd a11, a12, a21, a22;
    if (KIND == kAsmMuller) {
      a11 = cd{delta - e.D.x + t.D.x, -e.D.y + t.D.y};
      a12 = e.S - g * t.S;
      a21 = cd{t.H.x / g - e.H.x, t.H.y / g - e.H.y};
      a22 = cd{delta + e.K.x - t.K.x, e.K.y - t.K.y};
    } else {
      a11 = cd{0.5 * delta - e.D.x, -e.D.y};
      a12 = e.S;
      a21 = cd{0.5 * delta + t.D.x, t.D.y};
      a22 = cd{-g * t.S.x, -g * t.S.y};
    }
    const bool c64 = (I.c64 & 1) != 0;
    const int64_t nn = I.n_near;
    store_n(I.out1, c64, I.dnear, p, i + j * lda, a11);
    store_n(I.out1, c64, I.dnear, nn + p, i + (n + j) * lda, a12);
    store_n(I.out1, c64, I.dnear, 2 * nn + p, (n + i) + j * lda, a21);
    store_n(I.out1, c64, I.dnear, 3 * nn + p, (n + i) + (n + j) * lda, a22);
  }
}

// Laplace parts of the near pairs: computed once per mesh, reused by every wavenumber.
__global__ void k_near_laplace(const double* __restrict__ panels, const double* __restrict__ verts,
                               const int32_t* __restrict__ near_i,
                               const int32_t* __restrict__ near_j, int64_t n_near, double* out) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n_near) return;
  const int64_t i = near_i[p], j = near_j[p];
  const double* ri = panels + i * kPanelDoubles;
  const double* rj = panels + j * kPanelDoubles;
  double v[9];
#pragma unroll
  for (int t = 0; t < 9; ++t) v[t] = verts[j * kVertDoubles + t];
  double x[3] = {ri[0], ri[1], ri[2]}, nx[3] = {ri[3], ri[4], ri[5]};
  double S0, D0, K0, H0;
  laplace_parts(v, rj + 3, x, nx, i == j, S0, D0, K0, H0);
  reinterpret_cast<double4*>(out)[p] = make_double4(S0, D0, K0, H0);
}

void launch_near_laplace(const Launch& L, const double* panels, const double* verts,
                         const int32_t* near_i, const int32_t* near_j, int64_t n_near,
                         double* out) {
  if (n_near <= 0) return;
  k_near_laplace<<<(unsigned)((n_near + 127) / 128), 128, 0, L.stream>>>(panels, verts, near_i,
                                                                         near_j, n_near, out);
  count_launch(1);
}

// ------------------------------------------------------------------ launch wrappers
template <typename R>
static void launch_regular_t(const Launch& L, const AsmInst* d, int ninst, int64_t nmax,
                             int kind) {
  constexpr int kCols = Prec<R>::kCols;
  dim3 grid((unsigned)((nmax + kAsmRows - 1) / kAsmRows), (unsigned)((nmax + kCols - 1) / kCols),
            (unsigned)ninst);
  switch (kind) {
    case kAsmBM: k_assemble_regular<R, kAsmBM><<<grid, kAsmRows, 0, L.stream>>>(d, L.err_flag); count_launch(1); break;
    case kAsmCBIE: k_assemble_regular<R, kAsmCBIE><<<grid, kAsmRows, 0, L.stream>>>(d, L.err_flag); count_launch(1); break;
    case kAsmMuller: k_assemble_regular<R, kAsmMuller><<<grid, kAsmRows, 0, L.stream>>>(d, L.err_flag); count_launch(1); break;
    case kAsmRegion: k_assemble_regular<R, kAsmRegion><<<grid, kAsmRows, 0, L.stream>>>(d, L.err_flag); count_launch(1); break;
    default: k_assemble_regular<R, kAsmFluidCBIE><<<grid, kAsmRows, 0, L.stream>>>(d, L.err_flag); count_launch(1); break;
  }
}

void launch_assemble_regular(const Launch& L, const AsmInst* d_inst, int ninst, int64_t nmax,
                             int kind, bool fp32) {
  if (nmax <= 0 || ninst <= 0) return;
  if (fp32)
    launch_regular_t<float>(L, d_inst, ninst, nmax, kind);
  else
    launch_regular_t<double>(L, d_inst, ninst, nmax, kind);
}

template <bool F32>
static void launch_near_t(const Launch& L, const AsmInst* d_inst, int ninst, int64_t max_near,
                          int kind) {
  dim3 grid((unsigned)((max_near + 127) / 128), 1, (unsigned)ninst);
  switch (kind) {
    case kAsmBM: k_assemble_near<kAsmBM, F32><<<grid, 128, 0, L.stream>>>(d_inst); break;
    case kAsmCBIE: k_assemble_near<kAsmCBIE, F32><<<grid, 128, 0, L.stream>>>(d_inst); break;
    case kAsmMuller: k_assemble_near<kAsmMuller, F32><<<grid, 128, 0, L.stream>>>(d_inst); break;
    case kAsmRegion: k_assemble_near<kAsmRegion, F32><<<grid, 128, 0, L.stream>>>(d_inst); break;
    default: k_assemble_near<kAsmFluidCBIE, F32><<<grid, 128, 0, L.stream>>>(d_inst); break;
  }
  count_launch(1);
}

void launch_assemble_near(const Launch& L, const AsmInst* d_inst, int ninst, int64_t max_near,
                          int kind, bool fp32) {
  if (max_near <= 0 || ninst <= 0) return;
  if (fp32)
    launch_near_t<true>(L, d_inst, ninst, max_near, kind);
  else
    launch_near_t<false>(L, d_inst, ninst, max_near, kind);
}

// ------------------------------------------------------------------ incident traces
// p = e^{ik d.c}, q = ik (d.n) p at every collocation point (core/incident.jl:64-76).
__global__ void k_incident(const WaveInst* __restrict__ insts) {
  const WaveInst& W = insts[blockIdx.z];
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int r = blockIdx.y;
  if (i >= W.n || r >= W.nrhs) return;
  const double* rec = W.panels + i * kPanelDoubles;
  const double* d = W.dirs + 3 * r;
  const double ph = W.k * (d[0] * rec[0] + d[1] * rec[1] + d[2] * rec[2]);
  double sn, cs;
  sincos(ph, &sn, &cs);
  const double dn = W.k * (d[0] * rec[3] + d[1] * rec[4] + d[2] * rec[5]);
  const int64_t o = 2 * (i + r * W.ldp);
  W.p[o] = cs;
  W.p[o + 1] = sn;
  W.q[o] = -dn * sn;
  W.q[o + 1] = dn * cs;
}

void launch_incident(const Launch& L, const WaveInst* d_inst, int ninst, int64_t nmax,
                     int32_t max_rhs) {
  if (nmax <= 0 || ninst <= 0 || max_rhs <= 0) return;
  dim3 grid((unsigned)((nmax + 255) / 256), (unsigned)max_rhs, (unsigned)ninst);
  k_incident<<<grid, 256, 0, L.stream>>>(d_inst); count_launch(1);
}

// ------------------------------------------------------------------ far field
// f(xh) = -(1/4pi) sum_j area_j (ik xh.n_j p_j + q_j) sum_g W_g e^{-ik xh.y_jg}
// (solvers/bem/full.jl:509-519).  The panels are split into chunks of kFarChunk, one CTA
// (one panel per thread) per (chunk, direction, rhs, instance), so the FP64 phase work
// of one direction is spread over the GPU; a second kernel sums the chunk partials in
// chunk order.  Every sum has a fixed order, so the result does not depend on what else
// runs on the GPU.
constexpr int kFarChunk = 128;

size_t far_field_scratch(int64_t n, int32_t ndir, int32_t nrhs) {
  const int64_t chunks = (n + kFarChunk - 1) / kFarChunk;
  return (size_t)chunks * (size_t)ndir * (size_t)nrhs * 2 * sizeof(double);
}

__global__ void __launch_bounds__(kFarChunk) k_far_field(const WaveInst* __restrict__ insts) {
  const WaveInst& W = insts[blockIdx.z];
  const int64_t dr = blockIdx.x;
  const int64_t chunk = blockIdx.y;
  const int64_t nchunks = (W.n + kFarChunk - 1) / kFarChunk;
  if (dr >= (int64_t)W.ndir * W.nrhs || chunk >= nchunks) return;
  const int r = (int)(dr / W.ndir), d = (int)(dr % W.ndir);
  const double* xh = W.dirs + 3 * ((int64_t)r * W.ndir + d);
  const double k = W.k;
  const double x0 = xh[0], x1 = xh[1], x2 = xh[2];
  double ar = 0.0, ai = 0.0;
  const int64_t j = chunk * kFarChunk + threadIdx.x;
  if (j < W.n) {
    const double* rec = W.panels + j * kPanelDoubles;
    const int64_t o = 2 * (j + r * W.ldp);
    const double pr = W.p[o], pi = W.p[o + 1];
    const double qr = W.q[o], qi = W.q[o + 1];
    const double kxn = k * (x0 * rec[3] + x1 * rec[4] + x2 * rec[5]);
    // a = i kxn p + q
    const double a_r = -kxn * pi + qr, a_i = kxn * pr + qi;
    double sr = 0.0, si = 0.0;
#pragma unroll
    for (int g = 0; g < 7; ++g) {
      const double ph = -k * (x0 * rec[8 + 3 * g] + x1 * rec[9 + 3 * g] + x2 * rec[10 + 3 * g]);
      double sn, cs;
      sincos(ph, &sn, &cs);
      sr += dRuleW[g] * cs;
      si += dRuleW[g] * sn;
    }
    const double area = rec[6];
    ar = area * (a_r * sr - a_i * si);
    ai = area * (a_r * si + a_i * sr);
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    ar += __shfl_down_sync(0xffffffffu, ar, off);
    ai += __shfl_down_sync(0xffffffffu, ai, off);
  }
  __shared__ double red[2][kFarChunk / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) {
    red[0][wid] = ar;
    red[1][wid] = ai;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double tr = 0.0, ti = 0.0;
    for (int w = 0; w < kFarChunk / 32; ++w) {
      tr += red[0][w];
      ti += red[1][w];
    }
    double* o = W.part + 2 * (dr * nchunks + chunk);
    o[0] = tr;
    o[1] = ti;
  }
}

__global__ void k_far_field_finish(const WaveInst* __restrict__ insts) {
  const WaveInst& W = insts[blockIdx.z];
  const int64_t dr = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (dr >= (int64_t)W.ndir * W.nrhs) return;
  const int64_t nchunks = (W.n + kFarChunk - 1) / kFarChunk;
  double tr = 0.0, ti = 0.0;
  for (int64_t c = 0; c < nchunks; ++c) {
    tr += W.part[2 * (dr * nchunks + c)];
    ti += W.part[2 * (dr * nchunks + c) + 1];
  }
  W.out[2 * dr] = -tr * kInv4Pi;
  W.out[2 * dr + 1] = -ti * kInv4Pi;
}

void launch_far_field(const Launch& L, const WaveInst* d_inst, int ninst, int32_t max_rhs,
                      int32_t max_dirs, int64_t max_n) {
  if (ninst <= 0 || max_dirs <= 0 || max_rhs <= 0 || max_n <= 0) return;
  const int64_t dr = (int64_t)max_dirs * max_rhs;
  dim3 grid((unsigned)dr, (unsigned)((max_n + kFarChunk - 1) / kFarChunk), (unsigned)ninst);
  k_far_field<<<grid, kFarChunk, 0, L.stream>>>(d_inst);
  k_far_field_finish<<<dim3((unsigned)((dr + 127) / 128), 1, (unsigned)ninst), 128, 0, L.stream>>>(
      d_inst);
  count_launch(2);
}

}  // namespace bemgpu
