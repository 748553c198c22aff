// Internal declarations of libbemgpu (not part of the C ABI).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/bemgpu.h"

#ifdef __CUDACC__
#include <cuda_runtime.h>

#include <atomic>
#include <mutex>
#endif

namespace bemgpu {

// ------------------------------------------------------------------ host utilities
int validate_surface(const double* nodes, int64_t N, const int64_t* tris, int64_t M,
                     double* resolution, std::string* err);
void mesh_hash(const double* nodes, int64_t N, const int64_t* tris, int64_t M, char out[65]);
void panel_centroids(const double* nodes, const int64_t* tris, int64_t M,
                     std::vector<double>* cent, std::vector<double>* diam);
void near_pairs(const std::vector<double>& cent, const std::vector<double>& diam, double eta,
                std::vector<int64_t>* rowptr, std::vector<int64_t>* cols);

// Process-level error message (what bemgpu_last_error(NULL, ...) returns).
void bemgpu_set_process_error(const char* msg);

// Kernel launch accounting (every <<<>>> of the library increments the counter).
void count_launch(int kernels);
long long launch_total();

// ------------------------------------------------------------------ device records
// FP64 panel record, 32 doubles = 256 B (16-byte multiple for bulk async copies):
//   [0..2] centroid (collocation point)  [3..5] unit normal  [6] area  [7] longest edge
//   [8..28] the seven Gauss points (xyz)  [29..31] padding
constexpr int kPanelDoubles = 32;
// FP32 panel record, 32 floats = 128 B, coordinates relative to the mesh centre.
constexpr int kPanelFloats = 32;
// Vertex record, 12 doubles = 96 B: v0, v1, v2 (xyz) + padding.
constexpr int kVertDoubles = 12;

// Radon's 7-point degree-5 rule on the triangle (barycentric, weights sum to 1).
constexpr double kRuleW[7] = {0.225,
                              0.13239415278850618074, 0.13239415278850618074,
                              0.13239415278850618074, 0.12593918054482715260,
                              0.12593918054482715260, 0.12593918054482715260};
constexpr double kRuleB[7][3] = {
    {1.0 / 3.0, 1.0 / 3.0, 1.0 / 3.0},
    {0.05971587178976982046, 0.47014206410511508977, 0.47014206410511508977},
    {0.47014206410511508977, 0.05971587178976982046, 0.47014206410511508977},
    {0.47014206410511508977, 0.47014206410511508977, 0.05971587178976982046},
    {0.79742698535308732240, 0.10128650732345633880, 0.10128650732345633880},
    {0.10128650732345633880, 0.79742698535308732240, 0.10128650732345633880},
    {0.10128650732345633880, 0.10128650732345633880, 0.79742698535308732240}};

// Assembly kinds.
enum AsmKind : int32_t {
  kAsmBM = 0,        // rigid/soft Burton-Miller: M1 = 1/2 I - D - a H, M2 = S + a(1/2 I + K')
  kAsmCBIE = 1,      // rigid/soft CBIE:           M1 = 1/2 I - D,        M2 = S
  kAsmMuller = 2,    // fluid Mueller 2n x 2n
  kAsmFluidCBIE = 3, // fluid CBIE 2n x 2n
  kAsmRegion = 4     // coupled fluid regions over several surfaces, 2n x 2n (RegionTable)
};

// Coupled fluid regions (solvers/bem/regions.jl:189-236).  Surface s (0-based) encloses
// region s + 1; region 0 is the unbounded exterior.  The operators from source surface
// sj to target surface si enter the system through at most two regions, each with a
// sign (+1 when sj is the region's outer boundary, -1 when it is an inner one), the
// region's density contrast and wavenumber k / speed; Mueller adds
// [sign D, -sign rho S; sign / rho H, -sign K] to the 2 x 2 panel block, CBIE adds
// [sign D, -sign rho S] to the equation row block of the region (0: the side outside
// si, 1: inside) plus 1/2 I on the diagonal for each region.
constexpr int kMaxRegions = 16;  // interfaces per coupled problem
struct RegionCoef {
  int32_t count;    // contributing regions (0..2)
  int32_t kidx[2];  // region index of each contribution
  int32_t eq[2];    // CBIE equation row block
  int32_t pad;
  double sign[2];
  double rho[2];
};
struct RegionTable {
  int32_t count;                            // interfaces
  int32_t cbie;                             // 0 Mueller, 1 CBIE
  double kr[kMaxRegions + 1];               // wavenumber of every region
  RegionCoef c[kMaxRegions * kMaxRegions];  // [target surface * kMaxRegions + source]
};

// One assembly instance (device-resident array of these drives a batched launch).
struct AsmInst {
  const double* panels;    // FP64 panel records
  const float* panelsf;    // FP32 panel records (mixed precision regular pairs)
  const double* verts;     // vertex records
  const int32_t* near_i;   // near pair rows (collocation panel)
  const int32_t* near_j;   // near pair columns (source panel)
  const double* near_lap;  // closed-form Laplace parts S0, D0, K0, H0 per near pair
  int64_t n;               // panels
  int64_t n_near;          // near pairs
  int64_t lda;             // leading dimension of the outputs (n or 2n)
  double k_e, k_i, g;      // exterior/interior wavenumber, density contrast
  double a_re, a_im;       // Burton-Miller coupling (0 for CBIE)
  int32_t kind;            // AsmKind
  int32_t c64;             // bit 0 / bit 1: out1 / out2 stored complex64 (else complex128)
  void* out1;              // M1 (or A for fluid)
  void* out2;              // M2 (rigid/soft), null for fluid
  double* dnear;           // complex64 out1: FP64 near corrections [block][n_near]
  double* dnear2;          // complex64 out2: FP64 near corrections [n_near]
  const int32_t* surf;     // kAsmRegion: surface of every panel
  const RegionTable* region;  // kAsmRegion: coupling table
  const int64_t* near_dst;  // kAsmBM / kAsmCBIE: when set, index of near pair p in
                            // out1 / out2 (blocked storage) instead of i + j lda
};

// Incident field / far-field instance.
struct WaveInst {
  const double* panels;
  int64_t n;
  double k;
  int32_t nrhs;
  int32_t ndir;
  const double* dirs;      // incidence directions (3 * nrhs) or observation (3 * ndir)
  double* p;               // complex128 n x nrhs (traces) ...
  double* q;
  double* out;             // complex128 results
  int64_t ldp;             // leading dimension of p / q
  double* part;            // far field: per-chunk partial sums (far_field_scratch bytes)
};

// bytes of WaveInst.part for a far-field launch over n panels, ndir directions, nrhs
size_t far_field_scratch(int64_t n, int32_t ndir, int32_t nrhs);

// Dense-matrix instance for the batched factor / solve kernels.
struct MatInst {
  void* a;          // column-major matrix (complex128 or complex64)
  int64_t n;        // order
  int64_t lda;
  int32_t* ipiv;    // 0-based pivot rows
  int32_t* info;    // first zero pivot (1-based), 0 if none
  void* x;          // right-hand sides / solutions (n x nrhs, ld = ldx)
  int64_t ldx;
  int32_t nrhs;
  int32_t active;
  int32_t* perm;    // row permutation of the factor: (P b)[i] = b[perm[i]]
  void* y;          // second vector buffer of the triangular solves (n x nrhs, ld ldx)
};

// Selects the blocked triangular solves (MatInst.y / MatInst.perm provided).
struct TrsvWork {
  int32_t blocked;
};

// ------------------------------------------------------------------ launch wrappers
#ifdef __CUDACC__
constexpr int kMaxDevices = 64;

// One-time set-up per device.  Function attributes such as the dynamic shared-memory
// opt-in apply to the device that is current when they are set, so a launch helper
// keeps one of these and calls call(fn) before its launch: fn runs once for each device
// index (under a lock; later calls on that device are one atomic load).
class PerDeviceOnce {
 public:
  template <class F>
  void call(F&& fn) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
      cudaGetLastError();
      fn();
      return;
    }
    if (done_[dev].load(std::memory_order_acquire)) return;
    std::lock_guard<std::mutex> lk(mu_);
    if (done_[dev].load(std::memory_order_relaxed)) return;
    fn();
    done_[dev].store(true, std::memory_order_release);
  }

 private:
  std::mutex mu_;
  std::atomic<bool> done_[kMaxDevices]{};
};

// Streaming multiprocessors of the current device (looked up once per device).
inline int device_sm_count() {
  static std::atomic<int> sms[kMaxDevices]{};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return 1;
  }
  int v = sms[dev].load(std::memory_order_relaxed);
  if (v <= 0) {
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        v <= 0) {
      cudaGetLastError();
      return 1;
    }
    sms[dev].store(v, std::memory_order_relaxed);
  }
  return v;
}

struct Launch {
  cudaStream_t stream;
  int* err_flag;                  // device word set by bounded waits that give up
  cudaStream_t side = nullptr;    // second stream for overlapped work (joined before return)
  cudaEvent_t* events = nullptr;  // event pool for the two streams' ordering
  int n_events = 0;
};

void launch_assemble_regular(const Launch& L, const AsmInst* d_inst, int ninst, int64_t nmax,
                             int kind, bool fp32);
void launch_assemble_near(const Launch& L, const AsmInst* d_inst, int ninst, int64_t max_near,
                          int kind, bool fp32);
// closed-form Laplace parts of every near pair of a mesh (wavenumber independent)
void launch_near_laplace(const Launch& L, const double* panels, const double* verts,
                         const int32_t* near_i, const int32_t* near_j, int64_t n_near,
                         double* out);
void launch_incident(const Launch& L, const WaveInst* d_inst, int ninst, int64_t nmax,
                     int32_t max_rhs);
void launch_far_field(const Launch& L, const WaveInst* d_inst, int ninst, int32_t max_rhs,
                      int32_t max_dirs, int64_t max_n);
#endif

}  // namespace bemgpu
