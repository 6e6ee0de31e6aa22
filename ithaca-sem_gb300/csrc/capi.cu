// C-ABI layer: contexts, element operators, geometry. No exception crosses the
// boundary; each entry point returns a status code (include/ithaca_gpu.h).
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>

#include "ithaca_internal.h"

namespace ithaca {

static thread_local std::string g_last_error;

void set_last_error(const std::string& msg) { g_last_error = msg; }
const std::string& last_error_text() { return g_last_error; }

void fail(int code, const std::string& msg) { throw Error{code, msg}; }

void check_cuda(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    cudaGetLastError();  // clear sticky-free errors so the context stays usable
    fail(e == cudaErrorMemoryAllocation ? ITHACA_GPU_ERR_NOMEM : ITHACA_GPU_ERR_CUDA,
         std::string(what) + ": " + cudaGetErrorString(e));
  }
}

int device_sm_count() {
  constexpr int kMaxDevices = 64;
  static std::atomic<int> cache[kMaxDevices] = {};
  int dev = 0;
  ITHACA_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) fail(ITHACA_GPU_ERR_ARG, "device ordinal out of range");
  int sms = cache[dev].load();
  if (sms <= 0) {
    ITHACA_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    cache[dev].store(sms);
  }
  return sms;
}

void* Ctx::stage_ptr(int slot, size_t bytes) {
  if (bytes > stage_bytes[slot]) {
    if (stage[slot]) ITHACA_CUDA(cudaFree(stage[slot]));
    stage[slot] = nullptr;
    stage_bytes[slot] = 0;
    ITHACA_CUDA(cudaMalloc(&stage[slot], bytes));
    stage_bytes[slot] = bytes;
  }
  return stage[slot];
}

// Reads and clears the device error word; raises the recorded status (e.g. a
// bounded wait that gave up). Synchronises the context stream.
void Ctx::check_device_error() {
  if (!derr) return;
  int h = 0;
  ITHACA_CUDA(cudaMemcpyAsync(&h, derr, sizeof(int), cudaMemcpyDeviceToHost, stream));
  ITHACA_CUDA(cudaStreamSynchronize(stream));
  if (h != 0) {
    ITHACA_CUDA(cudaMemsetAsync(derr, 0, sizeof(int), stream));
    fail(h, "a device-side bounded wait gave up (status " + std::to_string(h) + ")");
  }
}

Ctx::~Ctx() {
  if (solver && solver_free) solver_free(solver);
  for (auto& p : stage)
    if (p) cudaFree(p);
  if (ev_in) cudaEventDestroy(ev_in);
  if (ev_out) cudaEventDestroy(ev_out);
  if (derr) cudaFree(derr);
  if (stream) cudaStreamDestroy(stream);
}

Op::~Op() {
  cudaFree(t64.base);
  cudaFree(t32.base);
  cudaFree(jg64);
  cudaFree(df64);
  cudaFree(jg32);
  cudaFree(df32);
}

template <typename F>
static int guarded(F f) {
  try {
    f();
    return ITHACA_GPU_OK;
  } catch (const Error& e) {
    set_last_error(e.msg);
    return e.code;
  } catch (const std::bad_alloc&) {
    set_last_error("host allocation failed");
    return ITHACA_GPU_ERR_NOMEM;
  } catch (...) {
    set_last_error("unknown error");
    return ITHACA_GPU_ERR_ARG;
  }
}

static int shape_dim(int shape) {
  if (shape == ITHACA_GPU_SHAPE_QUAD || shape == ITHACA_GPU_SHAPE_TRI) return 2;
  if (shape == ITHACA_GPU_SHAPE_HEX || shape == ITHACA_GPU_SHAPE_TET || shape == ITHACA_GPU_SHAPE_PRISM ||
      shape == ITHACA_GPU_SHAPE_PYR)
    return 3;
  fail(ITHACA_GPU_ERR_UNSUPPORTED,
       "shape must be triangle (3), quadrilateral (4), tetrahedron (5), pyramid (6), prism (7) or hexahedron (8)");
}

// Packed pyramid tables (layout pyr_off in ithaca_internal.h), host FP64.
static std::vector<double> pack_pyr_tables(const PyrBasisTables& t) {
  const PyrOff o = pyr_off(t.n);
  const int n = t.n, Q0 = n + 1, Q2 = n, nc = t.nc;
  std::vector<double> h(o.size);
  for (int i = 0; i < n * Q0; ++i) {
    h[o.B0 + i] = t.a.B[i];
    h[o.DB0 + i] = t.a.DB[i];
  }
  for (int i = 0; i < Q0 * Q0; ++i) h[o.D0 + i] = t.a.D[i];
  for (int i = 0; i < Q0; ++i) {
    h[o.w0 + i] = t.a.w[i];
    h[o.h0 + i] = 0.5 * (1.0 + t.a.z[i]);
  }
  for (int i = 0; i < nc * Q2; ++i) {
    h[o.B2 + i] = t.B2[i];
    h[o.DB2 + i] = t.DB2[i];
  }
  for (int i = 0; i < Q2 * Q2; ++i) h[o.D2 + i] = t.D2[i];
  for (int k = 0; k < Q2; ++k) {
    h[o.w2 + k] = 0.25 * t.w2[k];  // MatrixFreeOps/Operator.hpp:249-251
    h[o.h2 + k] = 2.0 / (1.0 - t.z2[k]);
  }
  return h;
}

// Packed prism tables (layout prism_off in ithaca_internal.h), host FP64.
static std::vector<double> pack_prism_tables(const TriBasisTables& t) {
  const PrismOff o = prism_off(t.n);
  const int n = t.n, Q0 = n + 1, Q2 = n, npr = n * (n + 1) / 2;
  std::vector<double> h(o.size);
  for (int i = 0; i < n * Q0; ++i) {
    h[o.B0 + i] = t.a.B[i];
    h[o.DB0 + i] = t.a.DB[i];
  }
  for (int i = 0; i < Q0 * Q0; ++i) h[o.D0 + i] = t.a.D[i];
  for (int i = 0; i < Q0; ++i) {
    h[o.w0 + i] = t.a.w[i];
    h[o.h0 + i] = 0.5 * (1.0 + t.a.z[i]);
  }
  for (int i = 0; i < npr * Q2; ++i) {
    h[o.B2 + i] = t.B1[i];
    h[o.DB2 + i] = t.DB1[i];
  }
  for (int i = 0; i < Q2 * Q2; ++i) h[o.D2 + i] = t.D1[i];
  for (int k = 0; k < Q2; ++k) {
    h[o.w2 + k] = 0.5 * t.w1[k];  // MatrixFreeOps/Operator.hpp:245-248
    h[o.h1 + k] = 2.0 / (1.0 - t.z1[k]);
  }
  return h;
}

// Packed tetrahedron tables (layout tet_off in ithaca_internal.h), host FP64.
static std::vector<double> pack_tet_tables(const TetBasisTables& b) {
  const TetOff o = tet_off(b.n);
  const int n = b.n, Q0 = n + 1, Q = n, npq = n * (n + 1) / 2, nc = b.nc;
  const TriBasisTables& t = b.t;
  std::vector<double> h(o.size);
  for (int i = 0; i < n * Q0; ++i) {
    h[o.B0 + i] = t.a.B[i];
    h[o.DB0 + i] = t.a.DB[i];
  }
  for (int i = 0; i < Q0 * Q0; ++i) h[o.D0 + i] = t.a.D[i];
  for (int i = 0; i < Q0; ++i) {
    h[o.w0 + i] = t.a.w[i];
    h[o.h0 + i] = 0.5 * (1.0 + t.a.z[i]);
  }
  for (int i = 0; i < npq * Q; ++i) {
    h[o.B1 + i] = t.B1[i];
    h[o.DB1 + i] = t.DB1[i];
  }
  for (int i = 0; i < nc * Q; ++i) {
    h[o.B2 + i] = b.B2[i];
    h[o.DB2 + i] = b.DB2[i];
  }
  for (int i = 0; i < Q * Q; ++i) {
    h[o.D1 + i] = t.D1[i];
    h[o.D2 + i] = b.D2[i];
  }
  for (int j = 0; j < Q; ++j) {
    h[o.w1 + j] = 0.5 * t.w1[j];  // MatrixFreeOps/Operator.hpp:245-251
    h[o.h1 + j] = 0.5 * (1.0 + t.z1[j]);
    h[o.h2 + j] = 2.0 / (1.0 - t.z1[j]);
    h[o.w2 + j] = 0.25 * b.w2[j];
    h[o.h3 + j] = 2.0 / (1.0 - b.z2[j]);
  }
  return h;
}

template <typename T>
static void upload_packed(DevTables<T>& dt, const std::vector<double>& h, int n, int Q) {
  std::vector<T> ht(h.begin(), h.end());
  dt.n = n;
  dt.Q = Q;
  ITHACA_CUDA(cudaMalloc(&dt.base, ht.size() * sizeof(T)));
  ITHACA_CUDA(cudaMemcpy(dt.base, ht.data(), ht.size() * sizeof(T), cudaMemcpyHostToDevice));
}

// Packed triangle tables (layout tri_off in ithaca_internal.h), host FP64.
static std::vector<double> pack_tri_tables(const TriBasisTables& b) {
  const TriOff o = tri_off(b.n);
  const int n = b.n, Q0 = b.Q0, Q1 = b.Q1, nc = b.nc;
  std::vector<double> h(o.size);
  for (int i = 0; i < n * Q0; ++i) {
    h[o.B0 + i] = b.a.B[i];
    h[o.DB0 + i] = b.a.DB[i];
  }
  for (int i = 0; i < Q0 * Q0; ++i) h[o.D0 + i] = b.a.D[i];
  for (int i = 0; i < Q0; ++i) {
    h[o.w0 + i] = b.a.w[i];
    h[o.h0 + i] = 0.5 * (1.0 + b.a.z[i]);
  }
  for (int i = 0; i < nc * Q1; ++i) {
    h[o.B1 + i] = b.B1[i];
    h[o.DB1 + i] = b.DB1[i];
  }
  for (int i = 0; i < Q1 * Q1; ++i) h[o.D1 + i] = b.D1[i];
  for (int j = 0; j < Q1; ++j) {
    h[o.w1 + j] = 0.5 * b.w1[j];  // MatrixFreeOps/Operator.hpp:245-248
    h[o.h1 + j] = 2.0 / (1.0 - b.z1[j]);
  }
  return h;
}

template <typename T>
static void upload_tri_tables(DevTables<T>& dt, const TriBasisTables& b) {
  const std::vector<double> h = pack_tri_tables(b);
  std::vector<T> ht(h.begin(), h.end());
  dt.n = b.n;
  dt.Q = b.Q0;
  ITHACA_CUDA(cudaMalloc(&dt.base, ht.size() * sizeof(T)));
  ITHACA_CUDA(cudaMemcpy(dt.base, ht.data(), ht.size() * sizeof(T), cudaMemcpyHostToDevice));
}

template <typename T>
static void upload_tables(DevTables<T>& dt, const BasisTables& b) {
  const int n = b.n, Q = b.Q;
  dt.n = n;
  dt.Q = Q;
  std::vector<T> h(dt.size());
  for (int p = 0; p < n; ++p)
    for (int i = 0; i < Q; ++i) {
      h[off_B(n, Q) + p * Q + i] = (T)b.B[p * Q + i];
      h[off_Bt(n, Q) + i * n + p] = (T)b.B[p * Q + i];
      h[off_DB(n, Q) + p * Q + i] = (T)b.DB[p * Q + i];
      h[off_DBt(n, Q) + i * n + p] = (T)b.DB[p * Q + i];
    }
  for (int k = 0; k < Q; ++k)
    for (int i = 0; i < Q; ++i) {
      h[off_D(n, Q) + k * Q + i] = (T)b.D[k * Q + i];
      h[off_Dt(n, Q) + i * Q + k] = (T)b.D[k * Q + i];
    }
  for (int i = 0; i < Q; ++i) h[off_w(n, Q) + i] = (T)b.w[i];
  ITHACA_CUDA(cudaMalloc(&dt.base, h.size() * sizeof(T)));
  ITHACA_CUDA(cudaMemcpy(dt.base, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
}

// Copies `bytes` from a host or device pointer into a device buffer (returned).
static const void* to_device(Ctx* c, int slot, const void* p, size_t bytes, int on_device) {
  if (on_device) return p;
  void* d = c->stage_ptr(slot, bytes);
  ITHACA_CUDA(cudaMemcpyAsync(d, p, bytes, cudaMemcpyHostToDevice, c->stream));
  return d;
}

static void* out_buffer(Ctx* c, int slot, void* p, size_t bytes, int on_device) {
  return on_device ? p : c->stage_ptr(slot, bytes);
}

static void from_device(Ctx* c, void* host, const void* dev, size_t bytes, int on_device) {
  if (on_device) return;
  ITHACA_CUDA(cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, c->stream));
}

static void finish(Ctx* c, int on_device) {
  ITHACA_CUDA(cudaGetLastError());
  if (!on_device) ITHACA_CUDA(cudaStreamSynchronize(c->stream));
}

static void require(bool ok, const char* msg) {
  if (!ok) fail(ITHACA_GPU_ERR_ARG, msg);
}

static size_t elt(const Op* op) { return op->precision == ITHACA_GPU_FP64 ? sizeof(double) : sizeof(float); }

}  // namespace ithaca

using namespace ithaca;

struct ithaca_gpu_ctx : public Ctx {};
struct ithaca_gpu_op : public Op {};

namespace ithaca {
void retain_op(Op* op) { op->refs++; }
void release_op(Op* op) {
  if (--op->refs == 0) {
    Ctx* c = op->ctx;
    delete static_cast<ithaca_gpu_op*>(op);
    release_ctx(c);
  }
}
void release_ctx(Ctx* c) {
  if (c && --c->refs == 0) delete static_cast<ithaca_gpu_ctx*>(c);
}
}  // namespace ithaca

extern "C" {

int ithaca_gpu_last_error(char* buf, size_t len) {
  if (!buf || len == 0) return ITHACA_GPU_ERR_ARG;
  std::snprintf(buf, len, "%s", g_last_error.c_str());
  return ITHACA_GPU_OK;
}

int ithaca_gpu_version(void) { return 100; }

int ithaca_gpu_ctx_create(int device, ithaca_gpu_ctx** ctx) {
  return guarded([&] {
    require(ctx != nullptr, "ctx is null");
    int ndev = 0;
    ITHACA_CUDA(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev) fail(ITHACA_GPU_ERR_ARG, "no such CUDA device");
    ITHACA_CUDA(cudaSetDevice(device));
    auto c = std::make_unique<ithaca_gpu_ctx>();
    c->device = device;
    ITHACA_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    ITHACA_CUDA(cudaEventCreateWithFlags(&c->ev_in, cudaEventDisableTiming));
    ITHACA_CUDA(cudaEventCreateWithFlags(&c->ev_out, cudaEventDisableTiming));
    ITHACA_CUDA(cudaMalloc(&c->derr, sizeof(int)));
    ITHACA_CUDA(cudaMemset(c->derr, 0, sizeof(int)));
    *ctx = c.release();
  });
}

int ithaca_gpu_ctx_destroy(ithaca_gpu_ctx* ctx) {
  return guarded([&] {
    if (!ctx) return;
    cudaStreamSynchronize(ctx->stream);
    release_ctx(ctx);
  });
}

int ithaca_gpu_ctx_synchronize(ithaca_gpu_ctx* ctx) {
  return guarded([&] {
    require(ctx, "ctx is null");
    ITHACA_CUDA(cudaStreamSynchronize(ctx->stream));
  });
}

int ithaca_gpu_ctx_stream(ithaca_gpu_ctx* ctx, void** stream) {
  return guarded([&] {
    require(ctx && stream, "null argument");
    *stream = (void*)ctx->stream;
  });
}

int ithaca_gpu_ctx_launch_count(ithaca_gpu_ctx* ctx, long long* count) {
  return guarded([&] {
    require(ctx && count, "null argument");
    *count = ctx->launches;
  });
}

int ithaca_gpu_basis_modA(int nmodes, int npoints, double* z, double* w, double* D, double* B, double* DB) {
  return guarded([&] {
    require(nmodes >= 1 && npoints >= 2, "need nmodes >= 1 and npoints >= 2");
    BasisTables t = make_basis(nmodes, npoints);
    if (z) std::memcpy(z, t.z.data(), sizeof(double) * npoints);
    if (w) std::memcpy(w, t.w.data(), sizeof(double) * npoints);
    if (D) std::memcpy(D, t.D.data(), sizeof(double) * npoints * npoints);
    if (B) std::memcpy(B, t.B.data(), sizeof(double) * nmodes * npoints);
    if (DB) std::memcpy(DB, t.DB.data(), sizeof(double) * nmodes * npoints);
  });
}

int ithaca_gpu_basis_tri(int nmodes, double* z0, double* w0, double* D0, double* B0, double* DB0, double* z1,
                         double* w1, double* D1, double* B1, double* DB1) {
  return guarded([&] {
    require(nmodes >= 2 && nmodes <= 16, "need 2 <= nmodes <= 16");
    const TriBasisTables t = make_tri_basis(nmodes);
    const int n = nmodes, Q0 = t.Q0, Q1 = t.Q1, nc = t.nc;
    if (z0) std::memcpy(z0, t.a.z.data(), sizeof(double) * Q0);
    if (w0) std::memcpy(w0, t.a.w.data(), sizeof(double) * Q0);
    if (D0) std::memcpy(D0, t.a.D.data(), sizeof(double) * Q0 * Q0);
    if (B0) std::memcpy(B0, t.a.B.data(), sizeof(double) * n * Q0);
    if (DB0) std::memcpy(DB0, t.a.DB.data(), sizeof(double) * n * Q0);
    if (z1) std::memcpy(z1, t.z1.data(), sizeof(double) * Q1);
    if (w1) std::memcpy(w1, t.w1.data(), sizeof(double) * Q1);
    if (D1) std::memcpy(D1, t.D1.data(), sizeof(double) * Q1 * Q1);
    if (B1) std::memcpy(B1, t.B1.data(), sizeof(double) * nc * Q1);
    if (DB1) std::memcpy(DB1, t.DB1.data(), sizeof(double) * nc * Q1);
  });
}

int ithaca_gpu_basis_tet(int nmodes, double* z2, double* w2, double* D2, double* B2, double* DB2) {
  return guarded([&] {
    require(nmodes >= 2 && nmodes <= 16, "need 2 <= nmodes <= 16");
    const TetBasisTables t = make_tet_basis(nmodes);
    const int Q = nmodes, nc = t.nc;
    if (z2) std::memcpy(z2, t.z2.data(), sizeof(double) * Q);
    if (w2) std::memcpy(w2, t.w2.data(), sizeof(double) * Q);
    if (D2) std::memcpy(D2, t.D2.data(), sizeof(double) * Q * Q);
    if (B2) std::memcpy(B2, t.B2.data(), sizeof(double) * nc * Q);
    if (DB2) std::memcpy(DB2, t.DB2.data(), sizeof(double) * nc * Q);
  });
}

int ithaca_gpu_basis_pyr(int nmodes, double* z2, double* w2, double* D2, double* B2, double* DB2) {
  return guarded([&] {
    require(nmodes >= 2 && nmodes <= 16, "need 2 <= nmodes <= 16");
    const PyrBasisTables t = make_pyr_basis(nmodes);
    const int Q = nmodes, nc = t.nc;
    if (z2) std::memcpy(z2, t.z2.data(), sizeof(double) * Q);
    if (w2) std::memcpy(w2, t.w2.data(), sizeof(double) * Q);
    if (D2) std::memcpy(D2, t.D2.data(), sizeof(double) * Q * Q);
    if (B2) std::memcpy(B2, t.B2.data(), sizeof(double) * nc * Q);
    if (DB2) std::memcpy(DB2, t.DB2.data(), sizeof(double) * nc * Q);
  });
}

int ithaca_gpu_geom_factors(ithaca_gpu_ctx* ctx, int shape, int npoints, int nelmt, const double* coords,
                            double* jac, double* df, int on_device) {
  return guarded([&] {
    require(ctx && coords && jac && df, "null argument");
    StreamOrder order_(ctx);
    require(nelmt > 0 && npoints >= 2 && npoints <= 16, "bad sizes");
    const int dim = shape_dim(shape);
    if (shape == ITHACA_GPU_SHAPE_PYR) {  // npoints = Q0 = Q1 = n + 1; Q2 = n Gauss-Radau (alpha 2)
      const int n = npoints - 1;
      const size_t tot = (size_t)nelmt * npoints * npoints * n;
      const std::vector<double> h = pack_pyr_tables(make_pyr_basis(n));
      double* dtab = nullptr;
      int* dbad = nullptr;
      ITHACA_CUDA(cudaMalloc(&dtab, sizeof(double) * h.size()));
      std::unique_ptr<double, decltype(&cudaFree)> g1(dtab, cudaFree);
      ITHACA_CUDA(cudaMalloc(&dbad, sizeof(int)));
      std::unique_ptr<int, decltype(&cudaFree)> g2(dbad, cudaFree);
      ITHACA_CUDA(cudaMemcpyAsync(dtab, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice, ctx->stream));
      ITHACA_CUDA(cudaMemsetAsync(dbad, 0, sizeof(int), ctx->stream));
      const double* X = (const double*)to_device(ctx, 0, coords, sizeof(double) * 3 * tot, on_device);
      double* J = (double*)out_buffer(ctx, 1, jac, sizeof(double) * tot, on_device);
      double* F = (double*)out_buffer(ctx, 2, df, sizeof(double) * 9 * tot, on_device);
      launch_geom_factors_pyr(n, nelmt, dtab, X, J, F, dbad, ctx->stream);
      ctx->launches++;
      from_device(ctx, jac, J, sizeof(double) * tot, on_device);
      from_device(ctx, df, F, sizeof(double) * 9 * tot, on_device);
      int hbad = 0;
      ITHACA_CUDA(cudaMemcpyAsync(&hbad, dbad, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
      ITHACA_CUDA(cudaStreamSynchronize(ctx->stream));
      if (hbad) fail(ITHACA_GPU_ERR_GEOMETRY, "non-positive Jacobian at a quadrature point");
      return;
    }
    if (shape == ITHACA_GPU_SHAPE_PRISM) {  // npoints = Q0 = Q1 = n + 1; Q2 = n Gauss-Radau
      const int n = npoints - 1;
      const size_t tot = (size_t)nelmt * npoints * npoints * n;
      const std::vector<double> h = pack_prism_tables(make_tri_basis(n));
      double* dtab = nullptr;
      int* dbad = nullptr;
      ITHACA_CUDA(cudaMalloc(&dtab, sizeof(double) * h.size()));
      std::unique_ptr<double, decltype(&cudaFree)> g1(dtab, cudaFree);
      ITHACA_CUDA(cudaMalloc(&dbad, sizeof(int)));
      std::unique_ptr<int, decltype(&cudaFree)> g2(dbad, cudaFree);
      ITHACA_CUDA(cudaMemcpyAsync(dtab, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice, ctx->stream));
      ITHACA_CUDA(cudaMemsetAsync(dbad, 0, sizeof(int), ctx->stream));
      const double* X = (const double*)to_device(ctx, 0, coords, sizeof(double) * 3 * tot, on_device);
      double* J = (double*)out_buffer(ctx, 1, jac, sizeof(double) * tot, on_device);
      double* F = (double*)out_buffer(ctx, 2, df, sizeof(double) * 9 * tot, on_device);
      launch_geom_factors_prism(n, nelmt, dtab, X, J, F, dbad, ctx->stream);
      ctx->launches++;
      from_device(ctx, jac, J, sizeof(double) * tot, on_device);
      from_device(ctx, df, F, sizeof(double) * 9 * tot, on_device);
      int hbad = 0;
      ITHACA_CUDA(cudaMemcpyAsync(&hbad, dbad, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
      ITHACA_CUDA(cudaStreamSynchronize(ctx->stream));
      if (hbad) fail(ITHACA_GPU_ERR_GEOMETRY, "non-positive Jacobian at a quadrature point");
      return;
    }
    if (shape == ITHACA_GPU_SHAPE_TET) {  // npoints = Q0 = n + 1; Q1 = Q2 = n Gauss-Radau
      const int n = npoints - 1;
      const size_t tot = (size_t)nelmt * npoints * n * n;
      const std::vector<double> h = pack_tet_tables(make_tet_basis(n));
      double* dtab = nullptr;
      int* dbad = nullptr;
      ITHACA_CUDA(cudaMalloc(&dtab, sizeof(double) * h.size()));
      std::unique_ptr<double, decltype(&cudaFree)> g1(dtab, cudaFree);
      ITHACA_CUDA(cudaMalloc(&dbad, sizeof(int)));
      std::unique_ptr<int, decltype(&cudaFree)> g2(dbad, cudaFree);
      ITHACA_CUDA(cudaMemcpyAsync(dtab, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice, ctx->stream));
      ITHACA_CUDA(cudaMemsetAsync(dbad, 0, sizeof(int), ctx->stream));
      const double* X = (const double*)to_device(ctx, 0, coords, sizeof(double) * 3 * tot, on_device);
      double* J = (double*)out_buffer(ctx, 1, jac, sizeof(double) * tot, on_device);
      double* F = (double*)out_buffer(ctx, 2, df, sizeof(double) * 9 * tot, on_device);
      launch_geom_factors_tet(n, nelmt, dtab, X, J, F, dbad, ctx->stream);
      ctx->launches++;
      from_device(ctx, jac, J, sizeof(double) * tot, on_device);
      from_device(ctx, df, F, sizeof(double) * 9 * tot, on_device);
      int hbad = 0;
      ITHACA_CUDA(cudaMemcpyAsync(&hbad, dbad, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
      ITHACA_CUDA(cudaStreamSynchronize(ctx->stream));
      if (hbad) fail(ITHACA_GPU_ERR_GEOMETRY, "non-positive Jacobian at a quadrature point");
      return;
    }
    if (shape == ITHACA_GPU_SHAPE_TRI) {  // npoints = Q0 = n + 1 GLL points; Q1 = n Gauss-Radau
      const int n = npoints - 1;
      const size_t tot = (size_t)nelmt * npoints * n;
      const std::vector<double> h = pack_tri_tables(make_tri_basis(n));
      double* dtab = nullptr;
      int* dbad = nullptr;
      ITHACA_CUDA(cudaMalloc(&dtab, sizeof(double) * h.size()));
      std::unique_ptr<double, decltype(&cudaFree)> g1(dtab, cudaFree);
      ITHACA_CUDA(cudaMalloc(&dbad, sizeof(int)));
      std::unique_ptr<int, decltype(&cudaFree)> g2(dbad, cudaFree);
      ITHACA_CUDA(cudaMemcpyAsync(dtab, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice, ctx->stream));
      ITHACA_CUDA(cudaMemsetAsync(dbad, 0, sizeof(int), ctx->stream));
      const double* X = (const double*)to_device(ctx, 0, coords, sizeof(double) * 2 * tot, on_device);
      double* J = (double*)out_buffer(ctx, 1, jac, sizeof(double) * tot, on_device);
      double* F = (double*)out_buffer(ctx, 2, df, sizeof(double) * 4 * tot, on_device);
      launch_geom_factors_tri(n, nelmt, dtab, X, J, F, dbad, ctx->stream);
      ctx->launches++;
      from_device(ctx, jac, J, sizeof(double) * tot, on_device);
      from_device(ctx, df, F, sizeof(double) * 4 * tot, on_device);
      int hbad = 0;
      ITHACA_CUDA(cudaMemcpyAsync(&hbad, dbad, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
      ITHACA_CUDA(cudaStreamSynchronize(ctx->stream));
      if (hbad) fail(ITHACA_GPU_ERR_GEOMETRY, "non-positive Jacobian at a quadrature point");
      return;
    }
    const int Q = npoints;
    const size_t nq = dim == 2 ? (size_t)Q * Q : (size_t)Q * Q * Q;
    const size_t tot = (size_t)nelmt * nq;
    BasisTables b = make_basis(2, Q);
    double* dD = nullptr;
    int* dbad = nullptr;
    ITHACA_CUDA(cudaMalloc(&dD, sizeof(double) * Q * Q));
    ITHACA_CUDA(cudaMalloc(&dbad, sizeof(int)));
    std::unique_ptr<double, decltype(&cudaFree)> g1(dD, cudaFree);
    std::unique_ptr<int, decltype(&cudaFree)> g2(dbad, cudaFree);
    ITHACA_CUDA(cudaMemcpyAsync(dD, b.D.data(), sizeof(double) * Q * Q, cudaMemcpyHostToDevice, ctx->stream));
    ITHACA_CUDA(cudaMemsetAsync(dbad, 0, sizeof(int), ctx->stream));
    const double* X = (const double*)to_device(ctx, 0, coords, sizeof(double) * dim * tot, on_device);
    double* J = (double*)out_buffer(ctx, 1, jac, sizeof(double) * tot, on_device);
    double* F = (double*)out_buffer(ctx, 2, df, sizeof(double) * dim * dim * tot, on_device);
    launch_geom_factors(dim, Q, nelmt, dD, X, J, F, dbad, ctx->stream);
    ctx->launches++;
    from_device(ctx, jac, J, sizeof(double) * tot, on_device);
    from_device(ctx, df, F, sizeof(double) * dim * dim * tot, on_device);
    int hbad = 0;
    ITHACA_CUDA(cudaMemcpyAsync(&hbad, dbad, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    ITHACA_CUDA(cudaStreamSynchronize(ctx->stream));
    if (hbad) fail(ITHACA_GPU_ERR_GEOMETRY, "non-positive Jacobian at a quadrature point");
  });
}

int ithaca_gpu_op_create(ithaca_gpu_ctx* ctx, int shape, int nmodes, int npoints, int nelmt, const double* jac,
                         const double* df, int deformed, int precision, int on_device, ithaca_gpu_op** op) {
  return guarded([&] {
    require(ctx && jac && df && op, "null argument");
    StreamOrder order_(ctx);
    require(nelmt > 0, "nelmt must be positive");
    require(precision == ITHACA_GPU_FP64 || precision == ITHACA_GPU_FP32, "unknown precision");
    const int dim = shape_dim(shape);
    // triangles are built to 12 modes (P = 11, the order of 2-D snapshot sets), the rest to 10
    const int nmax = shape == ITHACA_GPU_SHAPE_TRI ? 12 : 10;
    if (!(npoints == nmodes + 1 && nmodes >= 2 && nmodes <= nmax))
      fail(ITHACA_GPU_ERR_UNSUPPORTED,
           "GPU operators are built for npoints == nmodes + 1, 2 <= nmodes <= " + std::to_string(nmax) +
               " (got nmodes=" + std::to_string(nmodes) + ", npoints=" + std::to_string(npoints) + ")");
    auto o = std::make_unique<ithaca_gpu_op>();
    o->ctx = ctx;
    o->shape = shape;
    o->dim = dim;
    o->kdim = shape == ITHACA_GPU_SHAPE_TRI ? kTriKernels : dim;
    o->n = nmodes;
    o->Q = npoints;
    o->E = nelmt;
    o->deformed = deformed ? 1 : 0;
    o->precision = precision;
    const size_t npt = o->deformed ? (size_t)(dim == 2 ? npoints * npoints : npoints * npoints * npoints) : 1;
    if (shape == ITHACA_GPU_SHAPE_PYR) {
      // ModifiedA x ModifiedA x ModifiedPyr_C: n (n+1) (2n+1) / 6 modes on (n + 1)^2 n points; the
      // geometry is expanded to per-point metric terms whatever the input kind
      o->kdim = kPyrKernels;
      o->nm = pyr_nc(nmodes);
      o->nq = npoints * npoints * nmodes;
      const std::vector<double> h = pack_pyr_tables(make_pyr_basis(nmodes));
      upload_packed(o->t64, h, nmodes, npoints);
      upload_packed(o->t32, h, nmodes, npoints);
      const size_t tp = o->deformed ? (size_t)o->nq : 1;
      const double* J = (const double*)to_device(ctx, 0, jac, sizeof(double) * nelmt * tp, on_device);
      const double* F = (const double*)to_device(ctx, 1, df, sizeof(double) * 9 * nelmt * tp, on_device);
      const int in_deformed = o->deformed;
      o->deformed = 1;
      const size_t njg = (size_t)nelmt * 7 * o->nq, ndf = (size_t)nelmt * 9 * o->nq;
      ITHACA_CUDA(cudaMalloc(&o->jg64, sizeof(double) * njg));
      ITHACA_CUDA(cudaMalloc(&o->df64, sizeof(double) * ndf));
      launch_build_jg_pyr<double>(nmodes, nelmt, in_deformed, o->t64.base, J, F, o->jg64, o->df64, ctx->stream);
      ctx->launches++;
      if (precision == ITHACA_GPU_FP32) {
        ITHACA_CUDA(cudaMalloc(&o->jg32, sizeof(float) * njg + kGeoPad));
        ITHACA_CUDA(cudaMalloc(&o->df32, sizeof(float) * ndf));
        launch_build_jg_pyr<float>(nmodes, nelmt, in_deformed, o->t64.base, J, F, o->jg32, o->df32,
                                     ctx->stream);
        ctx->launches++;
      }
    } else if (shape == ITHACA_GPU_SHAPE_PRISM) {
      // ModifiedA x ModifiedA x ModifiedB: n^2 (n+1) / 2 modes on (n + 1)^2 n points; the
      // geometry is expanded to per-point metric terms whatever the input kind
      o->kdim = kPrismKernels;
      o->nm = prism_nc(nmodes);
      o->nq = npoints * npoints * nmodes;
      const std::vector<double> h = pack_prism_tables(make_tri_basis(nmodes));
      upload_packed(o->t64, h, nmodes, npoints);
      upload_packed(o->t32, h, nmodes, npoints);
      const size_t tp = o->deformed ? (size_t)o->nq : 1;
      const double* J = (const double*)to_device(ctx, 0, jac, sizeof(double) * nelmt * tp, on_device);
      const double* F = (const double*)to_device(ctx, 1, df, sizeof(double) * 9 * nelmt * tp, on_device);
      const int in_deformed = o->deformed;
      o->deformed = 1;
      const size_t njg = (size_t)nelmt * 7 * o->nq, ndf = (size_t)nelmt * 9 * o->nq;
      ITHACA_CUDA(cudaMalloc(&o->jg64, sizeof(double) * njg));
      ITHACA_CUDA(cudaMalloc(&o->df64, sizeof(double) * ndf));
      launch_build_jg_prism<double>(nmodes, nelmt, in_deformed, o->t64.base, J, F, o->jg64, o->df64, ctx->stream);
      ctx->launches++;
      if (precision == ITHACA_GPU_FP32) {
        ITHACA_CUDA(cudaMalloc(&o->jg32, sizeof(float) * njg + kGeoPad));
        ITHACA_CUDA(cudaMalloc(&o->df32, sizeof(float) * ndf));
        launch_build_jg_prism<float>(nmodes, nelmt, in_deformed, o->t64.base, J, F, o->jg32, o->df32,
                                     ctx->stream);
        ctx->launches++;
      }
    } else if (shape == ITHACA_GPU_SHAPE_TET) {
      // ModifiedA x ModifiedB x ModifiedC: n (n+1) (n+2) / 6 modes on (n + 1) n n collapsed
      // points; the geometry is expanded to per-point metric terms whatever the input kind
      o->kdim = kTetKernels;
      o->nm = tet_nc(nmodes);
      o->nq = npoints * nmodes * nmodes;
      const std::vector<double> h = pack_tet_tables(make_tet_basis(nmodes));
      upload_packed(o->t64, h, nmodes, npoints);
      upload_packed(o->t32, h, nmodes, npoints);
      const size_t tp = o->deformed ? (size_t)o->nq : 1;
      const double* J = (const double*)to_device(ctx, 0, jac, sizeof(double) * nelmt * tp, on_device);
      const double* F = (const double*)to_device(ctx, 1, df, sizeof(double) * 9 * nelmt * tp, on_device);
      const int in_deformed = o->deformed;
      o->deformed = 1;
      const size_t njg = (size_t)nelmt * 7 * o->nq, ndf = (size_t)nelmt * 9 * o->nq;
      ITHACA_CUDA(cudaMalloc(&o->jg64, sizeof(double) * njg));
      ITHACA_CUDA(cudaMalloc(&o->df64, sizeof(double) * ndf));
      launch_build_jg_tet<double>(nmodes, nelmt, in_deformed, o->t64.base, J, F, o->jg64, o->df64, ctx->stream);
      ctx->launches++;
      if (precision == ITHACA_GPU_FP32) {
        ITHACA_CUDA(cudaMalloc(&o->jg32, sizeof(float) * njg + kGeoPad));
        ITHACA_CUDA(cudaMalloc(&o->df32, sizeof(float) * ndf));
        launch_build_jg_tet<float>(nmodes, nelmt, in_deformed, o->t64.base, J, F, o->jg32, o->df32, ctx->stream);
        ctx->launches++;
      }
    } else if (shape == ITHACA_GPU_SHAPE_TRI) {
      // ModifiedA x ModifiedB: n (n + 1) / 2 modes on (n + 1) x n collapsed points
      o->nm = tri_nc(nmodes);
      o->nq = npoints * nmodes;
      const TriBasisTables tb = make_tri_basis(nmodes);
      upload_tri_tables(o->t64, tb);
      upload_tri_tables(o->t32, tb);
      const size_t tp = o->deformed ? (size_t)o->nq : 1;
      const size_t njg = (size_t)nelmt * 4 * tp;
      const double* J = (const double*)to_device(ctx, 0, jac, sizeof(double) * nelmt * tp, on_device);
      const double* F = (const double*)to_device(ctx, 1, df, sizeof(double) * 4 * nelmt * tp, on_device);
      ITHACA_CUDA(cudaMalloc(&o->jg64, sizeof(double) * njg));
      ITHACA_CUDA(cudaMalloc(&o->df64, sizeof(double) * njg));
      launch_build_jg_tri<double>(nmodes, nelmt, o->deformed, o->t64.base, J, F, o->jg64, o->df64, ctx->stream);
      ctx->launches++;
      if (precision == ITHACA_GPU_FP32) {
        ITHACA_CUDA(cudaMalloc(&o->jg32, sizeof(float) * njg + kGeoPad));
        ITHACA_CUDA(cudaMalloc(&o->df32, sizeof(float) * njg));
        launch_build_jg_tri<float>(nmodes, nelmt, o->deformed, o->t64.base, J, F, o->jg32, o->df32, ctx->stream);
        ctx->launches++;
      }
    } else {
      o->nm = dim == 2 ? nmodes * nmodes : nmodes * nmodes * nmodes;
      o->nq = dim == 2 ? npoints * npoints : npoints * npoints * npoints;
      BasisTables b = make_basis(nmodes, npoints);
      upload_tables(o->t64, b);
      upload_tables(o->t32, b);
      o->hB = b.B;
      o->hD = b.D;
      const size_t njg = (size_t)nelmt * n_jg(dim) * npt, ndf = (size_t)nelmt * dim * dim * npt;
      const double* J = (const double*)to_device(ctx, 0, jac, sizeof(double) * nelmt * npt, on_device);
      const double* F =
          (const double*)to_device(ctx, 1, df, sizeof(double) * dim * dim * nelmt * npt, on_device);
      double* dw = nullptr;
      ITHACA_CUDA(cudaMalloc(&dw, sizeof(double) * npoints));
      std::unique_ptr<double, decltype(&cudaFree)> gw(dw, cudaFree);
      ITHACA_CUDA(cudaMemcpyAsync(dw, b.w.data(), sizeof(double) * npoints, cudaMemcpyHostToDevice, ctx->stream));
      ITHACA_CUDA(cudaMalloc(&o->jg64, sizeof(double) * njg));
      ITHACA_CUDA(cudaMalloc(&o->df64, sizeof(double) * ndf));
      launch_build_jg<double>(dim, npoints, nelmt, o->deformed, dw, J, F, o->jg64, o->df64, ctx->stream);
      ctx->launches++;
      if (precision == ITHACA_GPU_FP32) {
        ITHACA_CUDA(cudaMalloc(&o->jg32, sizeof(float) * njg + kGeoPad));
        ITHACA_CUDA(cudaMalloc(&o->df32, sizeof(float) * ndf));
        launch_build_jg<float>(dim, npoints, nelmt, o->deformed, dw, J, F, o->jg32, o->df32, ctx->stream);
        ctx->launches++;
      }
      // the stream must finish with dw before it is freed
      ITHACA_CUDA(cudaStreamSynchronize(ctx->stream));
    }
    ITHACA_CUDA(cudaGetLastError());
    ITHACA_CUDA(cudaStreamSynchronize(ctx->stream));
    ctx->refs++;  // the operator holds its context
    *op = o.release();
  });
}

int ithaca_gpu_op_destroy(ithaca_gpu_op* op) {
  return guarded([&] {
    if (!op) return;
    cudaStreamSynchronize(op->ctx->stream);
    release_op(op);
  });
}

int ithaca_gpu_op_ndof(ithaca_gpu_op* op, long long* ndof) {
  return guarded([&] {
    require(op && ndof, "null argument");
    *ndof = (long long)op->E * op->nm;
  });
}

int ithaca_gpu_bwdtrans(ithaca_gpu_op* op, const void* in, void* out, int on_device) {
  return guarded([&] {
    require(op && in && out, "null argument");
    StreamOrder order_(op->ctx);
    Ctx* c = op->ctx;
    const size_t es = elt(op), nin = (size_t)op->E * op->nm, nout = (size_t)op->E * op->nq;
    const void* din = to_device(c, 0, in, es * nin, on_device);
    void* dout = out_buffer(c, 1, out, es * nout, on_device);
    bool ok;
    if (op->precision == ITHACA_GPU_FP64)
      ok = launch_bwdtrans<double>(op->kdim, op->n, op->Q, op->E, op->t64.base, (const double*)din, (double*)dout,
                                   c->stream);
    else
      ok = launch_bwdtrans<float>(op->kdim, op->n, op->Q, op->E, op->t32.base, (const float*)din, (float*)dout,
                                  c->stream);
    if (!ok) fail(ITHACA_GPU_ERR_UNSUPPORTED, "BwdTrans: (modes, points) combination not built");
    c->launches++;
    from_device(c, out, dout, es * nout, on_device);
    finish(c, on_device);
  });
}

int ithaca_gpu_iproduct(ithaca_gpu_op* op, const void* in, void* out, int on_device) {
  return guarded([&] {
    require(op && in && out, "null argument");
    StreamOrder order_(op->ctx);
    Ctx* c = op->ctx;
    const size_t es = elt(op), nin = (size_t)op->E * op->nq, nout = (size_t)op->E * op->nm;
    const void* din = to_device(c, 0, in, es * nin, on_device);
    void* dout = out_buffer(c, 1, out, es * nout, on_device);
    bool ok;
    if (op->precision == ITHACA_GPU_FP64)
      ok = launch_iproduct<double>(op->kdim, op->n, op->Q, op->E, op->deformed, op->t64.base, op->jg64,
                                   (const double*)din, (double*)dout, c->stream);
    else
      ok = launch_iproduct<float>(op->kdim, op->n, op->Q, op->E, op->deformed, op->t32.base, op->jg32,
                                  (const float*)din, (float*)dout, c->stream);
    if (!ok) fail(ITHACA_GPU_ERR_UNSUPPORTED, "IProductWRTBase: (modes, points) combination not built");
    c->launches++;
    from_device(c, out, dout, es * nout, on_device);
    finish(c, on_device);
  });
}

int ithaca_gpu_physderiv(ithaca_gpu_op* op, const void* in, void* d0, void* d1, void* d2, int on_device) {
  return guarded([&] {
    require(op && in && d0 && d1, "null argument");
    StreamOrder order_(op->ctx);
    require(op->dim == 2 || d2, "d2 is required for hexahedra");
    Ctx* c = op->ctx;
    const size_t es = elt(op), nq = (size_t)op->E * op->nq;
    const void* din = to_device(c, 0, in, es * nq, on_device);
    void* o[3] = {out_buffer(c, 1, d0, es * nq, on_device), out_buffer(c, 2, d1, es * nq, on_device),
                  op->dim == 3 ? out_buffer(c, 3, d2, es * nq, on_device) : nullptr};
    bool ok;
    if (op->precision == ITHACA_GPU_FP64)
      ok = launch_physderiv<double>(op->kdim, op->n, op->Q, op->E, op->deformed, op->t64.base, op->df64,
                                    (const double*)din, (double*)o[0], (double*)o[1], (double*)o[2], c->stream);
    else
      ok = launch_physderiv<float>(op->kdim, op->n, op->Q, op->E, op->deformed, op->t32.base, op->df32,
                                   (const float*)din, (float*)o[0], (float*)o[1], (float*)o[2], c->stream);
    if (!ok) fail(ITHACA_GPU_ERR_UNSUPPORTED, "PhysDeriv: (modes, points) combination not built");
    c->launches++;
    from_device(c, d0, o[0], es * nq, on_device);
    from_device(c, d1, o[1], es * nq, on_device);
    if (op->dim == 3) from_device(c, d2, o[2], es * nq, on_device);
    finish(c, on_device);
  });
}

int ithaca_gpu_iproduct_deriv(ithaca_gpu_op* op, const void* in0, const void* in1, const void* in2, void* out,
                              int on_device) {
  return guarded([&] {
    require(op && in0 && in1 && out, "null argument");
    require(op->dim == 2 || in2, "in2 is required for hexahedra");
    StreamOrder order_(op->ctx);
    Ctx* c = op->ctx;
    const size_t es = elt(op), nq = (size_t)op->E * op->nq, nm = (size_t)op->E * op->nm;
    const void* di[3] = {to_device(c, 0, in0, es * nq, on_device), to_device(c, 1, in1, es * nq, on_device),
                         op->dim == 3 ? to_device(c, 2, in2, es * nq, on_device) : nullptr};
    void* dout = out_buffer(c, 3, out, es * nm, on_device);
    bool ok;
    if (op->precision == ITHACA_GPU_FP64)
      ok = launch_iproduct_deriv<double>(op->kdim, op->n, op->Q, op->E, op->deformed, op->t64.base, op->jg64,
                                         op->df64, (const double*)di[0], (const double*)di[1], (const double*)di[2],
                                         (double*)dout, c->stream);
    else
      ok = launch_iproduct_deriv<float>(op->kdim, op->n, op->Q, op->E, op->deformed, op->t32.base, op->jg32,
                                        op->df32, (const float*)di[0], (const float*)di[1], (const float*)di[2],
                                        (float*)dout, c->stream);
    if (!ok) fail(ITHACA_GPU_ERR_UNSUPPORTED, "IProductWRTDerivBase: (modes, points) combination not built");
    c->launches++;
    from_device(c, out, dout, es * nm, on_device);
    finish(c, on_device);
  });
}

int ithaca_gpu_helmholtz(ithaca_gpu_op* op, double lambda, const void* in, void* out, int on_device) {
  return guarded([&] {
    require(op && in && out, "null argument");
    StreamOrder order_(op->ctx);
    Ctx* c = op->ctx;
    const size_t es = elt(op), nm = (size_t)op->E * op->nm;
    const void* din = to_device(c, 0, in, es * nm, on_device);
    void* dout = out_buffer(c, 1, out, es * nm, on_device);
    bool ok = false;
    if (op->precision == ITHACA_GPU_FP64) {
      if (op->kdim == 3 && op->deformed && op->variant64 > 0)  // even-odd pencil kernel where it is built
        ok = launch_helm_pencil64(op->n, op->Q, op->E, op->variant64, op->hB.data(), op->hD.data(), op->jg64, lambda,
                                  (const double*)din, (double*)dout, nullptr, 0, nullptr, nullptr, c->derr,
                                  c->stream);
      if (!ok)
        ok = launch_helmholtz<double>(op->kdim, op->n, op->Q, op->E, op->deformed, op->t64.base, op->jg64, lambda,
                                      (const double*)din, (double*)dout, nullptr, 0, c->stream);
    } else if (op->kdim == 3 && op->deformed && op->variant32 > 0)
      ok = launch_helm_pencil<float>(op->n, op->Q, op->E, op->variant32, op->hB.data(), op->hD.data(), op->jg32,
                                     (float)lambda, (const float*)din, (float*)dout, nullptr, 0, nullptr, nullptr,
                                     c->derr, c->stream);
    else
      ok = launch_helmholtz<float>(op->kdim, op->n, op->Q, op->E, op->deformed, op->t32.base, op->jg32,
                                   (float)lambda, (const float*)din, (float*)dout, nullptr, 0, c->stream);
    if (!ok) fail(ITHACA_GPU_ERR_UNSUPPORTED, "Helmholtz: (modes, points) combination not built");
    c->launches++;
    from_device(c, out, dout, es * nm, on_device);
    finish(c, on_device);
    if (!on_device) c->check_device_error();
  });
}

int ithaca_gpu_op_set_variant(ithaca_gpu_op* op, int variant) {
  return guarded([&] {
    require(op != nullptr, "null argument");
    require(variant == 0 || variant == 2 || variant == 4 || variant == 21 || variant == 22 || variant == 31 ||
                variant == 32 || variant == 41 || variant == 42 || variant == 43 || variant == 44 || variant == 46 ||
                variant == 47,
            "variant must be 0, 2, 4, 21, 22, 31, 32, 41, 42, 43, 44, 46 or 47");
    op->variant32 = variant;
  });
}

int ithaca_gpu_op_set_variant64(ithaca_gpu_op* op, int variant) {
  return guarded([&] {
    require(op != nullptr, "null argument");
    require(variant >= 0 && variant <= 2, "variant must be 0, 1 or 2");
    op->variant64 = variant;
  });
}

int ithaca_gpu_op_autotune(ithaca_gpu_op* op, int reps, int* chosen, double* times_ms) {
  return guarded([&] {
    require(op && reps > 0, "bad argument");
    StreamOrder order_(op->ctx);
    Ctx* c = op->ctx;
    cudaStream_t s = c->stream;
    const size_t nm = (size_t)op->E * op->nm;
    const size_t njg = (size_t)op->E * n_jg(op->dim) * (op->deformed ? op->nq : 1);
    float* jg = op->jg32;
    float* tmp_jg = nullptr;
    float *x = nullptr, *y = nullptr;
    cudaEvent_t e0, e1;
    ITHACA_CUDA(cudaEventCreate(&e0));
    ITHACA_CUDA(cudaEventCreate(&e1));
    struct Cleanup {
      float** p[3];
      cudaEvent_t a, b;
      ~Cleanup() {
        for (auto q : p) cudaFree(*q);
        cudaEventDestroy(a);
        cudaEventDestroy(b);
      }
    } cleanup{{&tmp_jg, &x, &y}, e0, e1};
    if (!jg) {  // FP64 operator: time on an FP32 copy of its geometry
      ITHACA_CUDA(cudaMalloc(&tmp_jg, sizeof(float) * njg + kGeoPad));
      std::vector<double> h(njg);
      ITHACA_CUDA(cudaMemcpy(h.data(), op->jg64, sizeof(double) * njg, cudaMemcpyDeviceToHost));
      std::vector<float> hf(h.begin(), h.end());
      ITHACA_CUDA(cudaMemcpy(tmp_jg, hf.data(), sizeof(float) * njg, cudaMemcpyHostToDevice));
      jg = tmp_jg;
    }
    ITHACA_CUDA(cudaMalloc(&x, sizeof(float) * nm));
    ITHACA_CUDA(cudaMalloc(&y, sizeof(float) * nm));
    ITHACA_CUDA(cudaMemsetAsync(x, 0, sizeof(float) * nm, s));
    const int variants[13] = {0, 2, 4, 21, 22, 31, 32, 41, 42, 43, 44, 46, 47};
    double best = 1e300;
    int best_v = 0;
    for (int vi = 0; vi < 13; ++vi) {
      const int v = variants[vi];
      double ms_avg = -1;
      if (v == 0 || (op->kdim == 3 && op->deformed)) {
        auto run = [&] {
          bool ok = v == 0 ? launch_helmholtz<float>(op->kdim, op->n, op->Q, op->E, op->deformed, op->t32.base, jg,
                                                     1.0f, x, y, nullptr, 0, s)
                           : launch_helm_pencil<float>(op->n, op->Q, op->E, v, op->hB.data(), op->hD.data(), jg,
                                                       1.0f, x, y, nullptr, 0, nullptr, nullptr, c->derr, s);
          if (!ok) fail(ITHACA_GPU_ERR_UNSUPPORTED, "Helmholtz: (modes, points) combination not built");
          c->launches++;
        };
        run();
        ITHACA_CUDA(cudaEventRecord(e0, s));
        for (int r = 0; r < reps; ++r) run();
        ITHACA_CUDA(cudaEventRecord(e1, s));
        ITHACA_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        ITHACA_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        ms_avg = ms / reps;
        if (ms_avg < best) {
          best = ms_avg;
          best_v = v;
        }
      }
      if (times_ms) times_ms[vi] = ms_avg;
    }
    c->check_device_error();
    op->variant32 = best_v;
    if (chosen) *chosen = best_v;
  });
}

int ithaca_gpu_helmholtz_diag(ithaca_gpu_op* op, double lambda, double* out, int on_device) {
  return guarded([&] {
    require(op && out, "null argument");
    StreamOrder order_(op->ctx);
    Ctx* c = op->ctx;
    const size_t nm = (size_t)op->E * op->nm;
    double* dout = (double*)out_buffer(c, 1, out, sizeof(double) * nm, on_device);
    if (!launch_helm_diag<double>(op->kdim, op->n, op->Q, op->E, op->deformed, op->t64.base, op->jg64, lambda, dout,
                                  c->stream))
      fail(ITHACA_GPU_ERR_UNSUPPORTED, "Helmholtz diagonal: (modes, points) combination not built");
    c->launches++;
    from_device(c, out, dout, sizeof(double) * nm, on_device);
    finish(c, on_device);
  });
}

}  // extern "C"
