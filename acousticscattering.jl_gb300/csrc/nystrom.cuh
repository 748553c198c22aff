// Nyström discretisation on the quadrature nodes (nystrom.cu): the rigid/soft operators of
// the reference's solve_full_bem (solvers/bem/full.jl:68-128) with unknowns at the seven
// Radon nodes of every panel, kernel values times node weights, the coincident-node entry
// zero, and a density-interpolation correction of every node's own element.
#pragma once

#include "bemgpu_internal.h"

namespace bemgpu {

constexpr int kNyNodes = 7;   // nodes per element (the panel's Radon rule)
constexpr int kNyBasis = 9;   // plane-wave interpolants of the correction
constexpr int kNyRows = 128;  // rows (threads) per assembly CTA
constexpr int kNyTile = 64;   // columns staged per shared-memory tile

// Node records use the panel-record layout (kPanelDoubles): [0..2] position, [3..5] unit
// normal of the element, [6] quadrature weight, [8..28] the position seven times, so that
// the incident-trace and far-field kernels of the panel path evaluate node sums.
struct NyInst {
  const double* nodes;  // node records, n of them (7 per element, element-major)
  int64_t n;
  double k;             // wavenumber
  double a_re, a_im;    // Burton-Miller coupling alpha (0 for CBIE)
  double* M1;           // 1/2 I - D - alpha H   (complex128, column-major, leading dim n)
  double* M2;           // S + alpha (1/2 I + K') (complex128, column-major, leading dim n)
  double dirs[3 * kNyBasis];  // unit plane-wave directions of the interpolants
  double* trace;        // interpolant traces [2][kNyBasis][n] complex: u, du/dn at the nodes
  double* part;         // defect partial sums [n_chunks][defects][kNyBasis][n] complex
  int32_t n_chunks;     // column ranges of the assembly (partial sums per range)
  int64_t chunk_cols;   // columns per range (a multiple of kNyTile)
  int32_t* status;      // per element: 0, or 1 when its correction fit met a zero pivot
  // fluid bodies (fluid != 0; M1, M2 unused): the 2n x 2n system of the panel path's
  // Mueller (1) or CBIE (2) blocks, with operators at k and at k_int, each corrected by
  // plane waves of its own wavenumber
  int32_t fluid;
  double k_int, g;      // interior wavenumber, density contrast
  double* A;            // system (complex128, column-major, leading dim 2n)
  double* trace_i;      // interpolant traces at k_int, layout of trace
  // coupled regions (fluid 3: Mueller, 4: CBIE; k, k_int, g unused): the surface of every
  // node and the regions' coupling table (the block algebra of the panel path's
  // kAsmRegion); trace / trace_i hold the interpolants at the wavenumber of the region
  // outside / inside each node's surface, and the defects sum over same-surface columns
  const int32_t* surf;
  const RegionTable* region;
};

// Defect sums per row and column range: 1 (rigid/soft, combined), 4 (Mueller: S/D and
// K'/H identities at k and k_int; regions: at the outer and inner side), 2 (fluid CBIE:
// S/D identities at k and k_int; regions: both sides).
int32_t nystrom_defects(int32_t fluid);

// Points of a Nyström solution's field evaluation (k_ny_pressure).
struct NyPoints {
  const double* nodes;   // node records (as NyInst)
  int64_t n;
  double k;
  const double* trace;   // interpolant traces [2][kNyBasis][n] complex
  const double* p;       // scattered pressure at the nodes (complex128, n)
  const double* q;       // scattered normal derivative at the nodes (complex128, n)
  const double* points;  // 3 x npts
  int64_t npts;
  const int32_t* region; // per point from the panel pass: 0 exterior, 1 interior, 2 surface
  double* out;           // complex128 npts: the incident value on entry, the field on exit
  int32_t field;         // 0 total, 1 scattered, 3 interior (bemgpu_field)
  int32_t* status;       // per point: 1 when the nearest element's fit was rank-deficient
  // fluid bodies: interior points (and surface points) take the interior field
  // S_int[g (q + q_inc)] - D_int[p + p_inc] at k_int
  int32_t fluid;
  double k_int, g;
  const double* trace_i; // interpolant traces at k_int
  double dir[3];         // incidence direction
  double dirs[3 * kNyBasis];  // plane-wave directions of the interpolants
};

// Element corrections of compressed (hierarchical) rigid/soft node operators: the same
// fit as the dense path with the combined defect  M2 F + M1 U - U - alpha F  taken from
// products of the compressed M1, M2 (nine columns, permuted order), written into the full
// leaf blocks that hold every same-element pair.
struct NyHm {
  const double* trace;   // node-order interpolant traces [2][kNyBasis][n] complex
  const double* Y;       // (M1 U + M2 F) in the tree's permuted order, n x kNyBasis complex
  const int32_t* iperm;  // node -> permuted position
  const int64_t* dst;    // n x 7: full-block offset of the pair (node i, node 7 (i / 7) + j)
  void* D1;              // full-block pools of M1 and M2 (complex64 when f32)
  void* D2;
  int64_t n;
  double a_re, a_im;     // Burton-Miller coupling
  int32_t f32;
  int32_t* status;       // per element: 1 when its fit was rank-deficient
};

// Scratch of launch_nystrom in doubles: traces (both wavenumbers for fluid bodies) and
// defect partials.
int64_t nystrom_scratch_doubles(int64_t n, int32_t n_chunks, int32_t fluid);
// Column ranges for n nodes (enough CTAs to fill the SMs a few times over).
int32_t nystrom_chunks(int64_t n);

#ifdef __CUDACC__
// Assembles M1 and M2 of one instance with the correction applied.
void launch_nystrom(const Launch& L, const NyInst& I);
// Element-block preconditioner of a compressed Nyström system: the inverse of every
// element's 7 x 7 diagonal block (node order), applied on the right inside GMRES.
struct NyPrec {
  double* Pinv;          // n / 7 blocks of 7 x 7 complex128, row-major (target, source)
  const int32_t* iperm;  // node -> permuted position
  const int64_t* dst;    // as NyHm.dst
  const void* D;         // the system operator's full-block pool (complex64 when f32)
  int64_t n;
  int32_t f32;
  int32_t* status;       // per element: 1 when its block is singular
  // Restricted additive Schwarz (ras = 1) instead of the element blocks: element e's
  // neighbourhood is the elements nb_el[nb_ptr[e] .. nb_ptr[e+1]) (e first), its L = 7 m
  // nodes in that order; W + woff[e] holds the own rows of the inverse of the system
  // restricted to those nodes (7 x L complex64, row-major).
  int32_t ras;
  float* W;
  const int64_t* woff;
  const int32_t* nb_ptr;
  const int32_t* nb_el;
  // building the local systems: FP32 node records (relative to the mesh centre), the
  // operator (0: M1 = 1/2 I - D - alpha H, 1: M2 = S + alpha (1/2 I + K')), wavenumber
  // and coupling; a workspace of `slots` local matrices of (L + 7) x L complex64
  const float* recf;
  int32_t op;
  float k, a_re, a_im;
  float* work;
  int64_t work_stride;   // floats per slot
};
// Pinv from the corrected full blocks.
void launch_nystrom_prec_build(const Launch& L, const NyPrec& P);
// Schwarz rows W of elements [e0, e0 + count) (count <= the workspace's slots).
void launch_nystrom_ras_build(const Launch& L, const NyPrec& P, int64_t e0, int64_t count,
                              int32_t max_len);
// dst[:, r] = Pinv src[:, r] for nr vectors in permuted order (ld lds / ldd complex);
// jptr (optional): src offset by (*jptr) * jstride complex entries (the Arnoldi vector).
void launch_nystrom_prec_apply(const Launch& L, const NyPrec& P, const double* src, int64_t lds,
                               const int32_t* jptr, int64_t jstride, double* dst, int64_t ldd,
                               int32_t nr);

// The diagonal of the uncorrected node operators (1/2 in M1, alpha / 2 in M2) into the
// full blocks (before the defect products), and the element corrections (after them).
void launch_nystrom_hm_diag(const Launch& L, const NyHm& H);
void launch_nystrom_hm_correct(const Launch& L, const NyHm& H);
// Interpolant traces (traces.trace, from traces.nodes / n / k / dirs), then the field at
// every point of P.
void launch_nystrom_pressure(const Launch& L, const NyInst& traces, const NyPoints& P);
#endif

}  // namespace bemgpu
