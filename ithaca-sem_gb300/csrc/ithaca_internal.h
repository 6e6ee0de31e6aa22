// Internal declarations shared by the C-ABI layer and the CUDA kernels.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/ithaca_gpu.h"

namespace ithaca {

// ---------------------------------------------------------------------------
// Errors: every C-ABI entry point catches `Error` and returns its code; the message
// is kept per thread for ithaca_gpu_last_error().
struct Error {
  int code;
  std::string msg;
};
void set_last_error(const std::string& msg);
const std::string& last_error_text();  // this thread's last error message
[[noreturn]] void fail(int code, const std::string& msg);
void check_cuda(cudaError_t e, const char* what);
#define ITHACA_CUDA(x) ::ithaca::check_cuda((x), #x)

// Number of SMs of the current device (queried once per device); grids are sized from it.
int device_sm_count();

// ---------------------------------------------------------------------------
// Basis tables (host, FP64), see basis.cpp.
struct BasisTables {
  int n = 0, Q = 0;
  std::vector<double> z, w, D, B, DB;
};
BasisTables make_basis(int n, int Q);
double jacobi(int m, double a, double b, double x);

// Triangle tables (host, FP64), basis.cpp: direction 0 is make_basis(n, n + 1)
// (ModifiedA on GLL points); direction 1 the Gauss-Radau-Jacobi (alpha 1, beta 0) points
// z1 and weights w1, D1[l*Q1 + j] = l_l'(z1_j) and the ModifiedB tables B1, DB1 of the
// nc = n (n + 1) / 2 modes m(p, q) (q fastest), each Q1 = n values long.
struct TriBasisTables {
  int n = 0, Q0 = 0, Q1 = 0, nc = 0;
  BasisTables a;
  std::vector<double> z1, w1, D1, B1, DB1;
};
TriBasisTables make_tri_basis(int n);

// Packed device tables of a triangle expansion (offsets in elements):
//   B0 [p*Q0 + i]  D0 [k*Q0 + i]  w0 [i]  h0 [i] = (1 + z0_i)/2
//   B1 [m*Q1 + j]  D1 [l*Q1 + j]  w1 [j] = w1_j / 2 (the collapsed map's factor)
//   h1 [j] = 2/(1 - z1_j)          DB0 [p*Q0 + i]   DB1 [m*Q1 + j]
struct TriOff {
  int B0, D0, w0, h0, B1, D1, w1, h1, DB0, DB1, size;
};
inline __host__ __device__ constexpr int tri_nc(int n) { return n * (n + 1) / 2; }
inline __host__ __device__ constexpr TriOff tri_off(int n) {
  const int Q0 = n + 1, Q1 = n, nc = n * (n + 1) / 2;
  TriOff o{};
  o.B0 = 0;
  o.D0 = o.B0 + n * Q0;
  o.w0 = o.D0 + Q0 * Q0;
  o.h0 = o.w0 + Q0;
  o.B1 = o.h0 + Q0;
  o.D1 = o.B1 + nc * Q1;
  o.w1 = o.D1 + Q1 * Q1;
  o.h1 = o.w1 + Q1;
  o.DB0 = o.h1 + Q1;
  o.DB1 = o.DB0 + n * Q0;
  o.size = o.DB1 + nc * Q1;
  return o;
}

// Tetrahedron tables (host, FP64), basis.cpp: direction 0 make_basis(n, n + 1); direction 1
// the triangle's Gauss-Radau (alpha 1) points and ModifiedB rows (n (n+1)/2 pairs (p, q));
// direction 2 Gauss-Radau (alpha 2) points z2, weights w2, D2 and the ModifiedC rows B2,
// DB2 of the nc = n (n+1) (n+2) / 6 modes m(p, q, r) (r fastest), each n values long.
struct TetBasisTables {
  int n = 0, nc = 0;
  TriBasisTables t;
  std::vector<double> z2, w2, D2, B2, DB2;
};
TetBasisTables make_tet_basis(int n);

// Packed device tables of a tetrahedron expansion (Q0 = n + 1, Q = n; offsets in elements):
//   B0 [p*Q0+i] D0 [k*Q0+i] w0 [i] h0 [i] = (1+z0_i)/2
//   B1 [pq*Q+j] D1 [l*Q+j] w1 [j] = w1_j/2 h1 [j] = (1+z1_j)/2 h2 [j] = 2/(1-z1_j)
//   B2 [m*Q+k]  D2 [l*Q+k] w2 [k] = w2_k/4 h3 [k] = 2/(1-z2_k)
//   then DB0, DB1, DB2 (read by the diagonal kernel only; `core` ends before them)
struct TetOff {
  int B0, D0, w0, h0, B1, D1, w1, h1, h2, B2, D2, w2, h3, DB0, DB1, DB2, core, size;
};
inline __host__ __device__ constexpr int tet_nc(int n) { return n * (n + 1) * (n + 2) / 6; }
inline __host__ __device__ constexpr TetOff tet_off(int n) {
  const int Q0 = n + 1, Q = n, npq = n * (n + 1) / 2, nc = n * (n + 1) * (n + 2) / 6;
  TetOff o{};
  o.B0 = 0;
  o.D0 = o.B0 + n * Q0;
  o.w0 = o.D0 + Q0 * Q0;
  o.h0 = o.w0 + Q0;
  o.B1 = o.h0 + Q0;
  o.D1 = o.B1 + npq * Q;
  o.w1 = o.D1 + Q * Q;
  o.h1 = o.w1 + Q;
  o.h2 = o.h1 + Q;
  o.B2 = o.h2 + Q;
  o.D2 = o.B2 + nc * Q;
  o.w2 = o.D2 + Q * Q;
  o.h3 = o.w2 + Q;
  o.core = o.h3 + Q;
  o.DB0 = o.core;
  o.DB1 = o.DB0 + n * Q0;
  o.DB2 = o.DB1 + npq * Q;
  o.size = o.DB2 + nc * Q;
  return o;
}

// Packed device tables of a prism expansion (Q0 = n + 1 for directions 0 and 1, Q2 = n):
//   B0 [p*Q0+i] D0 [k*Q0+i] w0 [i] h0 [i] = (1+z0_i)/2 (directions 0 and 1 share them)
//   B2 [pr*Q2+k] (ModifiedB rows (p, r)) D2 [l*Q2+k] w2 [k] = w2_k/2 h1 [k] = 2/(1-z2_k)
//   then DB0, DB2 (diagonal kernel only; `core` ends before them)
struct PrismOff {
  int B0, D0, w0, h0, B2, D2, w2, h1, DB0, DB2, core, size;
};
inline __host__ __device__ constexpr int prism_nc(int n) { return n * n * (n + 1) / 2; }
inline __host__ __device__ constexpr PrismOff prism_off(int n) {
  const int Q0 = n + 1, Q2 = n, npr = n * (n + 1) / 2;
  PrismOff o{};
  o.B0 = 0;
  o.D0 = o.B0 + n * Q0;
  o.w0 = o.D0 + Q0 * Q0;
  o.h0 = o.w0 + Q0;
  o.B2 = o.h0 + Q0;
  o.D2 = o.B2 + npr * Q2;
  o.w2 = o.D2 + Q2 * Q2;
  o.h1 = o.w2 + Q2;
  o.core = o.h1 + Q2;
  o.DB0 = o.core;
  o.DB2 = o.DB0 + n * Q0;
  o.size = o.DB2 + npr * Q2;
  return o;
}

// Pyramid direction 2 (host, FP64), basis.cpp: Gauss-Radau (alpha 2) points and the
// ModifiedPyr_C rows of the nc = n (n+1) (2n+1) / 6 modes m(p, q, r) (r fastest,
// r < n - max(p, q)); directions 0 and 1 are make_basis(n, n + 1).
struct PyrBasisTables {
  int n = 0, nc = 0;
  BasisTables a;
  std::vector<double> z2, w2, D2, B2, DB2;
};
PyrBasisTables make_pyr_basis(int n);

// Packed device tables of a pyramid expansion (Q0 = n + 1 for directions 0 and 1, Q2 = n):
//   B0 [p*Q0+i] D0 [k*Q0+i] w0 [i] h0 [i] = (1+z0_i)/2 (directions 0 and 1 share them)
//   B2 [m*Q2+k] D2 [l*Q2+k] w2 [k] = w2_k/4 h2 [k] = 2/(1-z2_k)
//   then DB0, DB2 (diagonal kernel only)
struct PyrOff {
  int B0, D0, w0, h0, B2, D2, w2, h2, DB0, DB2, core, size;
};
inline __host__ __device__ constexpr int pyr_nc(int n) { return n * (n + 1) * (2 * n + 1) / 6; }
inline __host__ __device__ constexpr PyrOff pyr_off(int n) {
  const int Q0 = n + 1, Q2 = n, nc = n * (n + 1) * (2 * n + 1) / 6;
  PyrOff o{};
  o.B0 = 0;
  o.D0 = o.B0 + n * Q0;
  o.w0 = o.D0 + Q0 * Q0;
  o.h0 = o.w0 + Q0;
  o.B2 = o.h0 + Q0;
  o.D2 = o.B2 + nc * Q2;
  o.w2 = o.D2 + Q2 * Q2;
  o.h2 = o.w2 + Q2;
  o.core = o.h2 + Q2;
  o.DB0 = o.core;
  o.DB2 = o.DB0 + n * Q0;
  o.size = o.DB2 + nc * Q2;
  return o;
}

// Kernel family passed where the launchers below take `dim`: 2 (quads), 3 (hexes),
// kTriKernels (triangles; their geometry has the 2-D layout), kTetKernels, kPrismKernels
// and kPyrKernels (per-point geometry with the 3-D layout, 7 fields).
constexpr int kTriKernels = 23;
constexpr int kTetKernels = 33;
constexpr int kPrismKernels = 34;
constexpr int kPyrKernels = 35;

// Device copy of the 1-D tables for one (n, Q), packed for the kernels:
//   B  [p*Q + i]   Bt  [i*n + p]   DB [p*Q + i]   DBt [i*n + p]
//   D  [k*Q + i] = l_k'(z_i)        Dt  [i*Q + k] = D[k*Q + i]       w [i]
template <typename T>
struct DevTables {
  T* base = nullptr;  // one allocation, offsets below
  int n = 0, Q = 0;
  size_t size() const { return (size_t)4 * n * Q + 2 * Q * Q + Q; }
};
// Offsets (in elements) of each table inside the packed buffer.
inline __host__ __device__ int off_B(int, int) { return 0; }
inline __host__ __device__ int off_Bt(int n, int Q) { return n * Q; }
inline __host__ __device__ int off_DB(int n, int Q) { return 2 * n * Q; }
inline __host__ __device__ int off_DBt(int n, int Q) { return 3 * n * Q; }
inline __host__ __device__ int off_D(int n, int Q) { return 4 * n * Q; }
inline __host__ __device__ int off_Dt(int n, int Q) { return 4 * n * Q + Q * Q; }
inline __host__ __device__ int off_w(int n, int Q) { return 4 * n * Q + 2 * Q * Q; }

// Number of geometry fields per quadrature point used by the Helmholtz kernels:
// J*w followed by the symmetric metric J*w*g^{ab} (upper triangle, row-major).
inline __host__ __device__ constexpr int n_jg(int dim) { return 1 + dim * (dim + 1) / 2; }

// ---------------------------------------------------------------------------
// Contexts and operators are reference counted: an operator holds its context and a
// solver holds its operator, so handles may be destroyed in any order (the reference
// shares these objects through std::shared_ptr).
struct Ctx {
  std::atomic<int> refs{1};
  int device = 0;
  cudaStream_t stream = nullptr;
  long long launches = 0;
  // grow-only staging buffers for host-pointer calls
  void* stage[4] = {nullptr, nullptr, nullptr, nullptr};
  size_t stage_bytes[4] = {0, 0, 0, 0};
  void* stage_ptr(int slot, size_t bytes);
  cudaEvent_t ev_in = nullptr, ev_out = nullptr;  // ordering with the legacy default stream
  int* derr = nullptr;  // device error word set by bounded waits in kernels (0 = ok)
  void check_device_error();
  // dense eigen-solver handle of the POD offline stage, created on first use
  void* solver = nullptr;
  void (*solver_free)(void*) = nullptr;
  ~Ctx();
};

// Orders a call's work after everything already queued on the legacy default stream
// (where callers such as torch produce device inputs) and makes that stream wait for
// the call's work before it continues; no host synchronisation.
struct StreamOrder {
  Ctx* c;
  explicit StreamOrder(Ctx* ctx) : c(ctx) {
    if (c && c->ev_in) {
      cudaEventRecord(c->ev_in, cudaStreamLegacy);
      cudaStreamWaitEvent(c->stream, c->ev_in, 0);
    }
  }
  ~StreamOrder() {
    if (c && c->ev_out) {
      cudaEventRecord(c->ev_out, c->stream);
      cudaStreamWaitEvent(cudaStreamLegacy, c->ev_out, 0);
    }
  }
};

struct Op {
  std::atomic<int> refs{1};
  Ctx* ctx = nullptr;
  int shape = 0, dim = 0, n = 0, Q = 0, E = 0;
  int kdim = 0;  // kernel family for the launchers: dim, or kTriKernels for triangles
  int deformed = 1, precision = ITHACA_GPU_FP64;
  int nm = 0, nq = 0;  // modes / points per element
  DevTables<double> t64;
  DevTables<float> t32;
  // geometry: jg[e][n_jg][nq or 1], df[e][d*d][nq or 1] (FP64 always; FP32 copies for FP32 ops)
  double* jg64 = nullptr;
  double* df64 = nullptr;
  float* jg32 = nullptr;
  float* df32 = nullptr;
  std::vector<double> hB, hD;  // host copies of B[p*Q+i] and D[k*Q+i] (kernel-parameter tables)
  // Helmholtz kernel variant for FP32 hexahedra: 0 = shared-memory kernel (elem.cuh),
  // 2 or 4 = pencil kernel (elem_pencil.cuh) with that many elements per CTA and a
  // TMA-staged geometry slab, 21/22 (31/32) = persistent pipelined pencil kernel with a
  // double (single) geometry buffer (elem_pencil_pipe.cuh), 41/42 = 31/32 on packed pairs.
  int variant32 = 41;
  int variant64 = 0;  // FP64 hex apply: 0 the shared-memory kernel, 1 / 2 the even-odd pencil kernel (1 / 2 elements)
  ~Op();
};

// Padding (bytes) after geometry buffers, so a CTA's 16-byte-rounded TMA window never
// leaves the allocation.
constexpr size_t kGeoPad = 64;

// Scattered output of the gathered element kernel, one output code per local dof:
//   g | kOwnedBit  the free global row g has this single local entry ("owned" row): the
//                  kernel writes s[g] = sign * value;
//   pos >= 0       the signed local value goes to out[pos], a slot of the
//                  assembly-ordered buffer that the assembly then reads with unit stride;
//   negative       not written (Dirichlet rows).
// Every CTA also writes part[cta], its share of s.w = y.(P w) over all its local values
// (w = the gathered input, P the signed gather), i.e. the whole dot product of the
// assembled output with the input.
// The pipelined kernels (variants 21-42 and the 16-bit-geometry kernel) accept this; the
// launcher reports in ctas how many partials it wrote (-1 where it could not, and the
// output is element-ordered as usual).
constexpr int kOwnedBit = 1 << 30;
struct OwnedRows {
  float* s = nullptr;
  double* part = nullptr;
  const int* ocode = nullptr;
  int ctas = -1;
};

template <typename T>
bool launch_helm_pencil(int n, int Q, int E, int variant, const double* hB, const double* hD, const T* jg, T lambda,
                        const T* in, T* out, const int* l2g, int ndir, const int* skip, const T* lam_ptr, int* err,
                        cudaStream_t s, OwnedRows* own = nullptr);
// FP64 hexes, persistent pipelined kernel with even-odd 1-D operators (Q even); variant 1 / 2
// = one / two elements per group. False for other (n, Q).
bool launch_helm_pencil64(int n, int Q, int E, int variant, const double* hB, const double* hD, const double* jg,
                          double lambda, const double* in, double* out, const int* l2g, int ndir, const int* skip,
                          const double* lam_ptr, int* err, cudaStream_t s);
// Half-precision geometry (E x 7 x Q^3 halves) with 8 FP32 scales per element; FP32 hexes.
// variant: the FP32 kernel variant of the operator (43 and 47 have half-geometry forms at
// (n, Q) = (7, 8); any other value runs the packed-pair kernel).
bool launch_helm_pipe_geo16(int n, int Q, int E, int variant, const double* hB, const double* hD, const void* jg16,
                            const float* gscale, float lambda, const float* in, float* out, const int* l2g, int ndir,
                            const int* skip, const float* lam_ptr, int* err, cudaStream_t s,
                            OwnedRows* own = nullptr);

void retain_op(Op* op);
void release_op(Op* op);    // frees the operator (and releases its context) at zero
void release_ctx(Ctx* ctx);  // frees the context at zero

// ---------------------------------------------------------------------------
// Kernel launchers (elem_*.cu), one explicit instantiation per (T, DIM). All take
// device pointers and launch on `s`; they return false if (n, Q) is not built.
// helm: element Helmholtz. With l2g != nullptr the input is gathered from a global
// vector, in_e[m] = sign * x[g] with l2g[e*nm+m] = g (sign +1) or ~g (sign -1), and
// global ids g < ndir read as zero (homogeneous Dirichlet dofs).
template <typename T, int DIM>
struct ElemApi {
  static bool helm(int n, int Q, int E, int deformed, const T* tab, const T* jg, T lambda, const T* in, T* out,
                   const int* l2g, int ndir, const int* skip, const T* lam_ptr, const int* esolve, int skip_stride,
                   cudaStream_t s, int variant = -1);
  static bool bwd(int n, int Q, int E, const T* tab, const T* in, T* out, cudaStream_t s);
  static bool ipr(int n, int Q, int E, int deformed, const T* tab, const T* jg, const T* in, T* out, cudaStream_t s);
  static bool deriv(int n, int Q, int E, int deformed, const T* tab, const T* df, const T* in, T* d0, T* d1, T* d2,
                    cudaStream_t s);
  static bool diag(int n, int Q, int E, int deformed, const T* tab, const T* jg, T lambda, T* out, cudaStream_t s);
  static bool iprd(int n, int Q, int E, int deformed, const T* tab, const T* jg, const T* df, const T* in0,
                   const T* in1, const T* in2, T* out, cudaStream_t s);
};

// Triangles (elem_tri.cuh): the same entry points; Q is the direction-0 point count n + 1.
template <typename T>
struct TriApi {
  static bool helm(int n, int Q, int E, int deformed, const T* tab, const T* jg, T lambda, const T* in, T* out,
                   const int* l2g, int ndir, const int* skip, const T* lam_ptr, const int* esolve, int skip_stride,
                   cudaStream_t s);
  static bool bwd(int n, int Q, int E, const T* tab, const T* in, T* out, cudaStream_t s);
  static bool ipr(int n, int Q, int E, int deformed, const T* tab, const T* jg, const T* in, T* out, cudaStream_t s);
  static bool deriv(int n, int Q, int E, int deformed, const T* tab, const T* df, const T* in, T* d0, T* d1,
                    cudaStream_t s);
  static bool diag(int n, int Q, int E, int deformed, const T* tab, const T* jg, T lambda, T* out, cudaStream_t s);
  static bool iprd(int n, int Q, int E, int deformed, const T* tab, const T* jg, const T* df, const T* in0,
                   const T* in1, T* out, cudaStream_t s);
};

// Tetrahedra (elem_tet.cuh); geometry always per point.
template <typename T>
struct TetApi {
  static bool helm(int n, int Q, int E, const T* tab, const T* jg, T lambda, const T* in, T* out, const int* l2g,
                   int ndir, const int* skip, const T* lam_ptr, cudaStream_t s);
  static bool bwd(int n, int Q, int E, const T* tab, const T* in, T* out, cudaStream_t s);
  static bool ipr(int n, int Q, int E, const T* tab, const T* jg, const T* in, T* out, cudaStream_t s);
  static bool deriv(int n, int Q, int E, const T* tab, const T* df, const T* in, T* d0, T* d1, T* d2,
                    cudaStream_t s);
  static bool diag(int n, int Q, int E, const T* tab, const T* jg, T lambda, T* out, cudaStream_t s);
  static bool iprd(int n, int Q, int E, const T* tab, const T* jg, const T* df, const T* in0, const T* in1,
                   const T* in2, T* out, cudaStream_t s);
};

// Prisms (elem_prism.cuh); geometry always per point. The same entry points as TetApi.
template <typename T>
struct PrismApi {
  static bool helm(int n, int Q, int E, const T* tab, const T* jg, T lambda, const T* in, T* out, const int* l2g,
                   int ndir, const int* skip, const T* lam_ptr, cudaStream_t s);
  static bool bwd(int n, int Q, int E, const T* tab, const T* in, T* out, cudaStream_t s);
  static bool ipr(int n, int Q, int E, const T* tab, const T* jg, const T* in, T* out, cudaStream_t s);
  static bool deriv(int n, int Q, int E, const T* tab, const T* df, const T* in, T* d0, T* d1, T* d2,
                    cudaStream_t s);
  static bool diag(int n, int Q, int E, const T* tab, const T* jg, T lambda, T* out, cudaStream_t s);
  static bool iprd(int n, int Q, int E, const T* tab, const T* jg, const T* df, const T* in0, const T* in1,
                   const T* in2, T* out, cudaStream_t s);
};

// Pyramids (elem_pyr.cuh); geometry always per point. The same entry points as TetApi.
template <typename T>
struct PyrApi {
  static bool helm(int n, int Q, int E, const T* tab, const T* jg, T lambda, const T* in, T* out, const int* l2g,
                   int ndir, const int* skip, const T* lam_ptr, cudaStream_t s);
  static bool bwd(int n, int Q, int E, const T* tab, const T* in, T* out, cudaStream_t s);
  static bool ipr(int n, int Q, int E, const T* tab, const T* jg, const T* in, T* out, cudaStream_t s);
  static bool deriv(int n, int Q, int E, const T* tab, const T* df, const T* in, T* d0, T* d1, T* d2,
                    cudaStream_t s);
  static bool diag(int n, int Q, int E, const T* tab, const T* jg, T lambda, T* out, cudaStream_t s);
  static bool iprd(int n, int Q, int E, const T* tab, const T* jg, const T* df, const T* in0, const T* in1,
                   const T* in2, T* out, cudaStream_t s);
};

template <typename T>
inline bool launch_helmholtz(int dim, int n, int Q, int E, int deformed, const T* tab, const T* jg, T lambda,
                             const T* in, T* out, const int* l2g, int ndir, cudaStream_t s,
                             const int* skip = nullptr, const T* lam_ptr = nullptr, const int* esolve = nullptr,
                             int skip_stride = 0, int variant = -1) {
  if (dim == kTriKernels)
    return TriApi<T>::helm(n, Q, E, deformed, tab, jg, lambda, in, out, l2g, ndir, skip, lam_ptr, esolve,
                           skip_stride, s);
  if (dim == kTetKernels) return esolve == nullptr && TetApi<T>::helm(n, Q, E, tab, jg, lambda, in, out, l2g, ndir,
                                                                      skip, lam_ptr, s);
  if (dim == kPrismKernels)
    return esolve == nullptr && PrismApi<T>::helm(n, Q, E, tab, jg, lambda, in, out, l2g, ndir, skip, lam_ptr, s);
  if (dim == kPyrKernels)
    return esolve == nullptr && PyrApi<T>::helm(n, Q, E, tab, jg, lambda, in, out, l2g, ndir, skip, lam_ptr, s);
  return dim == 2 ? ElemApi<T, 2>::helm(n, Q, E, deformed, tab, jg, lambda, in, out, l2g, ndir, skip, lam_ptr,
                                        esolve, skip_stride, s, variant)
                  : ElemApi<T, 3>::helm(n, Q, E, deformed, tab, jg, lambda, in, out, l2g, ndir, skip, lam_ptr,
                                        esolve, skip_stride, s, variant);
}
template <typename T>
inline bool launch_bwdtrans(int dim, int n, int Q, int E, const T* tab, const T* in, T* out, cudaStream_t s) {
  if (dim == kTriKernels) return TriApi<T>::bwd(n, Q, E, tab, in, out, s);
  if (dim == kTetKernels) return TetApi<T>::bwd(n, Q, E, tab, in, out, s);
  if (dim == kPrismKernels) return PrismApi<T>::bwd(n, Q, E, tab, in, out, s);
  if (dim == kPyrKernels) return PyrApi<T>::bwd(n, Q, E, tab, in, out, s);
  return dim == 2 ? ElemApi<T, 2>::bwd(n, Q, E, tab, in, out, s) : ElemApi<T, 3>::bwd(n, Q, E, tab, in, out, s);
}
template <typename T>
inline bool launch_iproduct(int dim, int n, int Q, int E, int deformed, const T* tab, const T* jg, const T* in,
                            T* out, cudaStream_t s) {
  if (dim == kTriKernels) return TriApi<T>::ipr(n, Q, E, deformed, tab, jg, in, out, s);
  if (dim == kTetKernels) return TetApi<T>::ipr(n, Q, E, tab, jg, in, out, s);
  if (dim == kPrismKernels) return PrismApi<T>::ipr(n, Q, E, tab, jg, in, out, s);
  if (dim == kPyrKernels) return PyrApi<T>::ipr(n, Q, E, tab, jg, in, out, s);
  return dim == 2 ? ElemApi<T, 2>::ipr(n, Q, E, deformed, tab, jg, in, out, s)
                  : ElemApi<T, 3>::ipr(n, Q, E, deformed, tab, jg, in, out, s);
}
template <typename T>
inline bool launch_physderiv(int dim, int n, int Q, int E, int deformed, const T* tab, const T* df, const T* in,
                             T* d0, T* d1, T* d2, cudaStream_t s) {
  if (dim == kTriKernels) return TriApi<T>::deriv(n, Q, E, deformed, tab, df, in, d0, d1, s);
  if (dim == kTetKernels) return TetApi<T>::deriv(n, Q, E, tab, df, in, d0, d1, d2, s);
  if (dim == kPrismKernels) return PrismApi<T>::deriv(n, Q, E, tab, df, in, d0, d1, d2, s);
  if (dim == kPyrKernels) return PyrApi<T>::deriv(n, Q, E, tab, df, in, d0, d1, d2, s);
  return dim == 2 ? ElemApi<T, 2>::deriv(n, Q, E, deformed, tab, df, in, d0, d1, d2, s)
                  : ElemApi<T, 3>::deriv(n, Q, E, deformed, tab, df, in, d0, d1, d2, s);
}
template <typename T>
inline bool launch_iproduct_deriv(int dim, int n, int Q, int E, int deformed, const T* tab, const T* jg, const T* df,
                                  const T* in0, const T* in1, const T* in2, T* out, cudaStream_t s) {
  if (dim == kTriKernels) return TriApi<T>::iprd(n, Q, E, deformed, tab, jg, df, in0, in1, out, s);
  if (dim == kTetKernels) return TetApi<T>::iprd(n, Q, E, tab, jg, df, in0, in1, in2, out, s);
  if (dim == kPrismKernels) return PrismApi<T>::iprd(n, Q, E, tab, jg, df, in0, in1, in2, out, s);
  if (dim == kPyrKernels) return PyrApi<T>::iprd(n, Q, E, tab, jg, df, in0, in1, in2, out, s);
  return dim == 2 ? ElemApi<T, 2>::iprd(n, Q, E, deformed, tab, jg, df, in0, in1, in2, out, s)
                  : ElemApi<T, 3>::iprd(n, Q, E, deformed, tab, jg, df, in0, in1, in2, out, s);
}
template <typename T>
inline bool launch_helm_diag(int dim, int n, int Q, int E, int deformed, const T* tab, const T* jg, T lambda,
                             T* out, cudaStream_t s) {
  if (dim == kTriKernels) return TriApi<T>::diag(n, Q, E, deformed, tab, jg, lambda, out, s);
  if (dim == kTetKernels) return TetApi<T>::diag(n, Q, E, tab, jg, lambda, out, s);
  if (dim == kPrismKernels) return PrismApi<T>::diag(n, Q, E, tab, jg, lambda, out, s);
  if (dim == kPyrKernels) return PyrApi<T>::diag(n, Q, E, tab, jg, lambda, out, s);
  return dim == 2 ? ElemApi<T, 2>::diag(n, Q, E, deformed, tab, jg, lambda, out, s)
                  : ElemApi<T, 3>::diag(n, Q, E, deformed, tab, jg, lambda, out, s);
}

// Geometry kernels (geom.cu)
void launch_geom_factors(int dim, int Q, int E, const double* D, const double* coords, double* jac, double* df,
                         int* bad, cudaStream_t s);
template <typename T>
void launch_build_jg(int dim, int Q, int E, int deformed, const double* w, const double* jac, const double* df,
                     T* jg, T* dfo, cudaStream_t s);
// Triangles: tab = the FP64 packed tables (w0, w1, h0, h1 are read). Deformed elements get
// per point J w and J w m^{ab} with the collapsed metric of MatrixFreeOps/Helmholtz.h:
// 581-618 folded in; regular ones per element J and J g^{ab} (the kernels add the point
// factors).
template <typename T>
void launch_build_jg_tri(int n, int E, int deformed, const double* tab, const double* jac, const double* df, T* jg,
                         T* dfo, cudaStream_t s);
void launch_geom_factors_tri(int n, int E, const double* tab, const double* coords, double* jac, double* df,
                             int* bad, cudaStream_t s);
// Tetrahedra: per point J w0 w1/2 w2/4 and J w m^{ab} with the collapsed metric of
// HelmholtzTetImpl (MatrixFreeOps/Helmholtz.h:2336-2420) folded in, from per-point
// (deformed) or per-element geometry; dfo gets the 9 factors per point.
template <typename T>
void launch_build_jg_tet(int n, int E, int deformed, const double* tab, const double* jac, const double* df, T* jg,
                         T* dfo, cudaStream_t s);
void launch_geom_factors_tet(int n, int E, const double* tab, const double* coords, double* jac, double* df,
                             int* bad, cudaStream_t s);
// Prisms: per point J w0 w0 w2/2 and J w m^{ab} with the collapsed metric of
// HelmholtzPrismImpl (MatrixFreeOps/Helmholtz.h:1340-1400).
template <typename T>
void launch_build_jg_prism(int n, int E, int deformed, const double* tab, const double* jac, const double* df,
                           T* jg, T* dfo, cudaStream_t s);
void launch_geom_factors_prism(int n, int E, const double* tab, const double* coords, double* jac, double* df,
                               int* bad, cudaStream_t s);
// Pyramids: per point J w0 w0 w2/4 and J w m^{ab} with the collapsed metric of
// HelmholtzPyrImpl (MatrixFreeOps/Helmholtz.h:1841-1905).
template <typename T>
void launch_build_jg_pyr(int n, int E, int deformed, const double* tab, const double* jac, const double* df, T* jg,
                         T* dfo, cudaStream_t s);
void launch_geom_factors_pyr(int n, int E, const double* tab, const double* coords, double* jac, double* df,
                             int* bad, cudaStream_t s);

}  // namespace ithaca
