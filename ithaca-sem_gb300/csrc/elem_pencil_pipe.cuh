// Persistent, software-pipelined version of the register-pencil hexahedral Helmholtz
// kernel (elem_pencil.cuh holds the single-pass version and the shared helpers).
//
// One CTA per resident slot loops over groups of EB elements (group, group + gridDim.x,
// ...). While it computes group i it already has in flight
//   * the TMA copy of group i+1's geometry slab: with NB = 2 into the other half of a
//     double buffer (issued at the top of iteration i); with NB = 1 into the single
//     buffer as soon as group i's metric stage has read it (half the shared memory, so
//     about twice the resident CTAs, for a shorter lead); and
//   * the gather of group i+1's input coefficients into registers: the signed l2g codes
//     of group i+2 are loaded right after stage 1 of group i, and the dependent x loads
//     of group i+1 (whose codes arrived a group earlier) are issued after stage 5, so
//     both latencies hide behind arithmetic; the values are written to shared memory at
//     stage 1 of iteration i+1, where the sign is applied.
// The arithmetic per element is exactly that of helm3_pencil_kernel (same stages, same
// tables, same summation order), so both kernels give bit-identical results.
//
// Output: element-ordered (out[e * NM + m], unsigned), or, with per-local-dof output
// codes, scattered: owned rows (free global rows with a single local entry) are written
// straight into the assembled vector, the other signed local values into the slots of
// an assembly-ordered buffer, so that the assembly reads them with unit stride.
//
// TG = __half stores the geometry slab in half precision with one FP32 scale per element
// and field (value = half * scale, |half| <= 1): half the geometry bytes for a pointwise
// relative perturbation of the coefficients below 2^-11 of each field's element maximum.
// The operator stays symmetric positive definite and spectrally equivalent to the FP32
// one, which is what an inner solve inside FP64 iterative refinement needs.
#pragma once

#include <cuda_fp16.h>

#include <type_traits>

#include "elem_pencil.cuh"

namespace ithaca {
namespace dev {

// ---- packed FP32 pairs (fma.rn.f32x2: two FP32 FMAs per instruction) ----
__device__ __forceinline__ unsigned long long pk2(float a, float b) {
  unsigned long long r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ void upk2(unsigned long long v, float& a, float& b) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}
__device__ __forceinline__ unsigned long long ffma2(unsigned long long a, unsigned long long b, unsigned long long c) {
  unsigned long long d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}

// 1-D tables laid out for pairs of outputs: entry (input a, output o) of each table at
// [a * ld + o] with an even row length ld, so outputs (o, o + 1), o even, are one
// 8-byte-aligned constant pair. F: forward (BwdTrans / derivative), T: transposed
// (IProduct / derivative transpose).
template <int N, int Q>
struct PTabs2 {
  static constexpr int QP = Q + (Q & 1), NP = N + (N & 1);
  alignas(8) float BF[N * QP];  // BF[p * QP + i] = B(p, z_i)
  alignas(8) float DF[Q * QP];  // DF[k * QP + i] = l_k'(z_i)
  alignas(8) float BT[Q * NP];  // BT[i * NP + p] = B(p, z_i)
  alignas(8) float DT[Q * QP];  // DT[i * QP + k] = l_k'(z_i)
};

// o[x] = sum_{a < NI} W(a, x) c[a] for x < NO, the sum in increasing a (the order of the
// scalar contractions), two outputs per instruction; with INIT the sums start from o.
template <int NI, int NO, int LD, bool INIT, typename Get>
__device__ __forceinline__ void contract2(Get W, const float (&c)[NI], float (&o)[NO]) {
#pragma unroll
  for (int x = 0; x + 1 < NO; x += 2) {
    unsigned long long acc = INIT ? pk2(o[x], o[x + 1]) : pk2(0.f, 0.f);
#pragma unroll
    for (int a = 0; a < NI; ++a) acc = ffma2(pk2(W(a * LD + x), W(a * LD + x + 1)), pk2(c[a], c[a]), acc);
    upk2(acc, o[x], o[x + 1]);
  }
  if constexpr (NO & 1) {
    float acc = INIT ? o[NO - 1] : 0.f;
#pragma unroll
    for (int a = 0; a < NI; ++a) acc = fmaf(W(a * LD + NO - 1), c[a], acc);
    o[NO - 1] = acc;
  }
}

// Vector pencils (V4, Q = 8 only): plane stride 68 (= 4 mod 32) instead of 73. The pencils
// along the unit-stride index are then read and written as two 16-byte words each, and a
// quarter warp (lanes (j, k) = (t / 8, t % 8), k = 0..7) hits eight different 16-byte bank
// groups ((2 j + 17 k) mod 8 = (2 j + k) mod 8); the pencils along j run on lanes
// (i, k) = (t % 4 + 4 (t / 32), (t / 4) % 8), whose banks i + 68 k = i + 4 k (mod 32) are
// all different; the columns along k keep lanes (t % 8, t / 8), banks i + 8 j. No bank
// conflicts in any stage, and a quarter of the shared-memory instructions of the
// unit-stride stages.
template <int Q, bool V4>
__host__ __device__ constexpr int pipe_pk(void) {
  return V4 ? 68 : pk_stride(Q);
}

template <typename T, int N, int Q, int EB, int NB, typename TG = T, bool V4 = false>
struct PipeLayout {
  static constexpr int NQ = Q * Q * Q, GEO = 7 * NQ;
  static constexpr int PJ = Q, PK = pipe_pk<Q, V4>(), FS = PK * Q;
  static constexpr size_t GEO_BYTES = ((size_t)EB * GEO * sizeof(TG) + 32 + 15) / 16 * 16;  // + window slack
  static constexpr size_t bytes() { return 16 + NB * GEO_BYTES + (size_t)EB * 3 * FS * sizeof(T); }
};

// ---- even-odd contractions (EO, Q even) ----
// The GLL points are symmetric (z_{Q-1-i} = -z_i), so the collocation derivative is
// antisymmetric (l'_{Q-1-k}(z_{Q-1-i}) = -l'_k(z_i)) and the ModifiedA modes have parity
// (B_0 and B_1 swap under z -> -z, B_p(-z) = (-1)^p B_p(z) for p >= 2). Each pair of
// outputs (i, Q-1-i) then follows from half-length sums over the even and odd parts of the
// input (e_k = u_k + u_{Q-1-k}, o_k = u_k - u_{Q-1-k}), the E and O sums riding in the two
// halves of one packed FP32 pair: half the multiply-adds of the plain contraction.
//   bw[i][j] = ((B_0 + B_1) / 2, (B_0 - B_1) / 2)(z_i) for j = 0, (B_2j, B_2j+1)(z_i) else
//   d[i][k]  = (D_ki + D_(Q-1-k)i, D_ki - D_(Q-1-k)i) / 2 with D_ki = l'_k(z_i)
//   dt[i][k] = the same for the transposed derivative T_ki = l'_i(z_k)
template <typename T>
struct alignas(2 * sizeof(T)) TPair {
  T x, y;
};
template <typename T, int N, int Q>
struct PTabs3 {
  static constexpr int H = Q / 2, NE = (N + 1) / 2;
  TPair<T> bw[H][NE];
  TPair<T> d[H][H];
  TPair<T> dt[H][H];
};
__device__ __forceinline__ unsigned long long pk2f(const TPair<float>& v) {
  return *reinterpret_cast<const unsigned long long*>(&v);
}
// modes -> points: o[i], i < Q, from c[p], p < N
template <int N, int Q>
__device__ __forceinline__ void eo_bwd(const PTabs3<float, N, Q>& tb, const float (&c)[N], float (&o)[Q]) {
  constexpr int H = Q / 2, NE = (N + 1) / 2;
  unsigned long long x[NE];
  x[0] = pk2(c[0] + c[1], c[0] - c[1]);
#pragma unroll
  for (int j = 1; j < NE; ++j) x[j] = pk2(c[2 * j], 2 * j + 1 < N ? c[2 * j + 1] : 0.f);
#pragma unroll
  for (int i = 0; i < H; ++i) {
    unsigned long long acc = pk2(0.f, 0.f);
#pragma unroll
    for (int j = 0; j < NE; ++j) acc = ffma2(pk2f(tb.bw[i][j]), x[j], acc);
    float E, O;
    upk2(acc, E, O);
    o[i] = E + O;
    o[Q - 1 - i] = E - O;
  }
}
// points -> modes (IProduct): o[p], p < N, from v[i], i < Q
template <int N, int Q>
__device__ __forceinline__ void eo_ipr(const PTabs3<float, N, Q>& tb, const float (&v)[Q], float (&o)[N]) {
  constexpr int H = Q / 2, NE = (N + 1) / 2;
  unsigned long long x[H];
#pragma unroll
  for (int k = 0; k < H; ++k) x[k] = pk2(v[k] + v[Q - 1 - k], v[k] - v[Q - 1 - k]);
#pragma unroll
  for (int j = 0; j < NE; ++j) {
    unsigned long long acc = pk2(0.f, 0.f);
#pragma unroll
    for (int k = 0; k < H; ++k) acc = ffma2(pk2f(tb.bw[k][j]), x[k], acc);
    float E, O;
    upk2(acc, E, O);
    if (j == 0) {
      o[0] = E + O;
      o[1] = E - O;
    } else {
      o[2 * j] = E;
      if (2 * j + 1 < N) o[2 * j + 1] = O;
    }
  }
}
// antisymmetric Q x Q operator (derivative or its transpose); INIT adds to o
template <int Q, bool INIT>
__device__ __forceinline__ void eo_anti(const TPair<float> (&t)[Q / 2][Q / 2], const float (&u)[Q], float (&o)[Q]) {
  constexpr int H = Q / 2;
  unsigned long long x[H];
#pragma unroll
  for (int k = 0; k < H; ++k) x[k] = pk2(u[k] + u[Q - 1 - k], u[k] - u[Q - 1 - k]);
#pragma unroll
  for (int i = 0; i < H; ++i) {
    unsigned long long acc = pk2(0.f, 0.f);
#pragma unroll
    for (int k = 0; k < H; ++k) acc = ffma2(pk2f(t[i][k]), x[k], acc);
    float E, O;
    upk2(acc, E, O);
    o[i] = INIT ? o[i] + (E + O) : E + O;
    o[Q - 1 - i] = INIT ? o[Q - 1 - i] + (O - E) : O - E;
  }
}

// The same even-odd forms with scalar E and O sums (FP64 pencils).
template <typename T, int N, int Q>
__device__ __forceinline__ void eo_bwd_s(const PTabs3<T, N, Q>& tb, const T (&c)[N], T (&o)[Q]) {
  constexpr int H = Q / 2, NE = (N + 1) / 2;
  T xe[NE], xo[NE];
  xe[0] = c[0] + c[1];
  xo[0] = c[0] - c[1];
#pragma unroll
  for (int j = 1; j < NE; ++j) {
    xe[j] = c[2 * j];
    xo[j] = 2 * j + 1 < N ? c[2 * j + 1] : T(0);
  }
#pragma unroll
  for (int i = 0; i < H; ++i) {
    T E = tb.bw[i][0].x * xe[0], O = tb.bw[i][0].y * xo[0];
#pragma unroll
    for (int j = 1; j < NE; ++j) {
      E = fma(tb.bw[i][j].x, xe[j], E);
      O = fma(tb.bw[i][j].y, xo[j], O);
    }
    o[i] = E + O;
    o[Q - 1 - i] = E - O;
  }
}
template <typename T, int N, int Q>
__device__ __forceinline__ void eo_ipr_s(const PTabs3<T, N, Q>& tb, const T (&v)[Q], T (&o)[N]) {
  constexpr int H = Q / 2, NE = (N + 1) / 2;
  T xe[H], xo[H];
#pragma unroll
  for (int k = 0; k < H; ++k) {
    xe[k] = v[k] + v[Q - 1 - k];
    xo[k] = v[k] - v[Q - 1 - k];
  }
#pragma unroll
  for (int j = 0; j < NE; ++j) {
    T E = tb.bw[0][j].x * xe[0], O = tb.bw[0][j].y * xo[0];
#pragma unroll
    for (int k = 1; k < H; ++k) {
      E = fma(tb.bw[k][j].x, xe[k], E);
      O = fma(tb.bw[k][j].y, xo[k], O);
    }
    if (j == 0) {
      o[0] = E + O;
      o[1] = E - O;
    } else {
      o[2 * j] = E;
      if (2 * j + 1 < N) o[2 * j + 1] = O;
    }
  }
}
template <typename T, int Q, bool INIT>
__device__ __forceinline__ void eo_anti_s(const TPair<T> (&t)[Q / 2][Q / 2], const T (&u)[Q], T (&o)[Q]) {
  constexpr int H = Q / 2;
  T xe[H], xo[H];
#pragma unroll
  for (int k = 0; k < H; ++k) {
    xe[k] = u[k] + u[Q - 1 - k];
    xo[k] = u[k] - u[Q - 1 - k];
  }
#pragma unroll
  for (int i = 0; i < H; ++i) {
    T E = t[i][0].x * xe[0], O = t[i][0].y * xo[0];
#pragma unroll
    for (int k = 1; k < H; ++k) {
      E = fma(t[i][k].x, xe[k], E);
      O = fma(t[i][k].y, xo[k], O);
    }
    o[i] = INIT ? o[i] + (E + O) : E + O;
    o[Q - 1 - i] = INIT ? o[Q - 1 - i] + (O - E) : O - E;
  }
}

// ---- warp-level TF32 tensor-core contractions in three-term split precision (TC) ----
// A contraction of an element's 64 pencils (rows r) with a 1-D table W (8 x 8, zero padded)
// is a 64 x 8 x 8 product: four m16n8k8 tiles, two per warp of the element. Each FP32
// operand x is split into hi = tf32(x) and lo = tf32(x - hi); the product is
// hi.hi + hi.lo + lo.hi (three MMAs, smallest first, FP32 accumulation), which drops only
// lo.lo, below 2^-21 of each product: FP32-level accuracy for the inner solve.
__device__ __forceinline__ uint32_t tf32_rna(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}
struct TfFrag {
  uint32_t hi[2], lo[2];
};
// The B fragment of lane (g = lane / 4, t4 = lane % 4): W[t4][g] and W[t4 + 4][g], split.
__device__ __forceinline__ TfFrag tf_frag(float w0, float w1) {
  TfFrag f;
  f.hi[0] = tf32_rna(w0);
  f.lo[0] = tf32_rna(w0 - __uint_as_float(f.hi[0]));
  f.hi[1] = tf32_rna(w1);
  f.lo[1] = tf32_rna(w1 - __uint_as_float(f.hi[1]));
  return f;
}
__device__ __forceinline__ void mma_tf32(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}
// KIND 0: along the unit-stride index, row r = (u, v) = (r / 8, r % 8) at offset 8 u + 68 v;
// KIND 1: along j (stride 8), row r = (i, k) = (r % 8, r / 8) at offset i + 68 k (the V4
// layout). Lane (g, t4) of warp w loads A[r][t4], A[r][t4 + 4] for rows r = 16 m + g and
// r + 8 of its tiles m = 2 w, 2 w + 1 (banks t4 + 4 g and 8 t4 + g: no conflicts); rows
// failing `valid` and inputs a >= KI read as zero. All eight outputs of every row are
// written (zero where the table column is zero). src may equal dst: a tile's loads all
// precede its MMAs, and the tiles' rows are disjoint.
template <int KIND, int KI, typename Valid>
__device__ __forceinline__ void tc_contract(const float* src, float* dst, const TfFrag& w, int t, Valid valid) {
  constexpr int SA = KIND == 0 ? 1 : 8;
  const int lane = t & 31, g = lane >> 2, t4 = lane & 3;
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int m = 2 * (t >> 5) + h;
    int off[2];
    bool ok[2];
#pragma unroll
    for (int s2 = 0; s2 < 2; ++s2) {
      const int r = 16 * m + g + 8 * s2;
      const int a = KIND == 0 ? r >> 3 : r & 7, b = KIND == 0 ? r & 7 : r >> 3;
      off[s2] = KIND == 0 ? 8 * a + 68 * b : a + 68 * b;
      ok[s2] = valid(a, b);
    }
    float x[4];
    x[0] = (ok[0] && t4 < KI) ? src[t4 * SA + off[0]] : 0.f;
    x[1] = (ok[1] && t4 < KI) ? src[t4 * SA + off[1]] : 0.f;
    x[2] = (ok[0] && t4 + 4 < KI) ? src[(t4 + 4) * SA + off[0]] : 0.f;
    x[3] = (ok[1] && t4 + 4 < KI) ? src[(t4 + 4) * SA + off[1]] : 0.f;
    uint32_t ah[4], al[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      ah[i] = tf32_rna(x[i]);
      al[i] = tf32_rna(x[i] - __uint_as_float(ah[i]));
    }
    float d[4] = {0.f, 0.f, 0.f, 0.f};
    mma_tf32(d, al, w.hi);
    mma_tf32(d, ah, w.lo);
    mma_tf32(d, ah, w.hi);
    dst[2 * t4 * SA + off[0]] = d[0];
    dst[(2 * t4 + 1) * SA + off[0]] = d[1];
    dst[2 * t4 * SA + off[1]] = d[2];
    dst[(2 * t4 + 1) * SA + off[1]] = d[3];
  }
}

// 8 consecutive floats from / to 16-byte aligned shared memory as two 16-byte words; the
// first M are used (M <= 8), the rest of the store is zero.
template <int M>
__device__ __forceinline__ void lds8(const float* p, float (&c)[M]) {
  const float4 a = *reinterpret_cast<const float4*>(p), b = *reinterpret_cast<const float4*>(p + 4);
  const float v[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
#pragma unroll
  for (int i = 0; i < M; ++i) c[i] = v[i];
}
template <int M>
__device__ __forceinline__ void sts8(float* p, const float (&o)[M]) {
  float v[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = i < M ? o[i] : 0.f;
  *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
  *reinterpret_cast<float4*>(p + 4) = make_float4(v[4], v[5], v[6], v[7]);
}

template <typename T, int N, int Q, int EB, bool GATHER, int NB, typename TG = T, bool PACK = false, bool V4 = false,
          bool TC = false, bool EO = false>
__global__ void __launch_bounds__(Q* Q* EB) helm3_pipe_kernel(const T* __restrict__ in, T* __restrict__ out,
                                                               const PTabs<T, N, Q> tab, const PTabs2<N, Q> tab2,
                                                               const PTabs3<T, N, Q> tab3,
                                                               const TG* __restrict__ jg,
                                                               T lambda, int E, const int* __restrict__ l2g,
                                                               int ndir, const int* __restrict__ skip,
                                                               const T* __restrict__ lam_ptr, int* __restrict__ err,
                                                               const float* __restrict__ gscale = nullptr,
                                                               T* __restrict__ sown = nullptr,
                                                               double* __restrict__ opart = nullptr,
                                                               const int* __restrict__ ocode = nullptr) {
  static_assert(NB == 1 || NB == 2, "one or two geometry buffers");
  static_assert(!PACK || std::is_same<T, float>::value, "packed pairs are FP32");
  static_assert(!V4 || (PACK && Q == 8 && N <= 8), "vector pencils: packed FP32, Q = 8");
  static_assert(!TC || (V4 && Q * Q == 64), "tensor-core stages: the vector-pencil layout, 64 pencils");
  static_assert(!EO || ((V4 || !PACK) && !TC && Q % 2 == 0 && N >= 2),
                "even-odd stages: packed in the vector-pencil layout or scalar, Q even");
  // the 1-D operators of the packed stages: plain contractions or their even-odd forms
  auto op_bwd = [&](const T (&c)[N], T (&o)[Q]) {
    if constexpr (EO && !PACK)
      eo_bwd_s<T, N, Q>(tab3, c, o);
    else if constexpr (EO)
      eo_bwd<N, Q>(tab3, c, o);
    else
      contract2<N, Q, PTabs2<N, Q>::QP, false>([&](int i) { return tab2.BF[i]; }, c, o);
  };
  auto op_der = [&](const T (&c)[Q], T (&o)[Q]) {
    if constexpr (EO && !PACK)
      eo_anti_s<T, Q, false>(tab3.d, c, o);
    else if constexpr (EO)
      eo_anti<Q, false>(tab3.d, c, o);
    else
      contract2<Q, Q, PTabs2<N, Q>::QP, false>([&](int i) { return tab2.DF[i]; }, c, o);
  };
  auto op_dert = [&](const T (&c)[Q], T (&o)[Q]) {
    if constexpr (EO && !PACK)
      eo_anti_s<T, Q, false>(tab3.dt, c, o);
    else if constexpr (EO)
      eo_anti<Q, false>(tab3.dt, c, o);
    else
      contract2<Q, Q, PTabs2<N, Q>::QP, false>([&](int i) { return tab2.DT[i]; }, c, o);
  };
  auto op_dert_add = [&](const T (&c)[Q], T (&o)[Q]) {
    if constexpr (EO && !PACK)
      eo_anti_s<T, Q, true>(tab3.dt, c, o);
    else if constexpr (EO)
      eo_anti<Q, true>(tab3.dt, c, o);
    else
      contract2<Q, Q, PTabs2<N, Q>::QP, true>([&](int i) { return tab2.DT[i]; }, c, o);
  };
  auto op_ipr = [&](const T (&c)[Q], T (&o)[N]) {
    if constexpr (EO && !PACK)
      eo_ipr_s<T, N, Q>(tab3, c, o);
    else if constexpr (EO)
      eo_ipr<N, Q>(tab3, c, o);
    else
      contract2<Q, N, PTabs2<N, Q>::NP, false>([&](int i) { return tab2.BT[i]; }, c, o);
  };
  constexpr int QP = PTabs2<N, Q>::QP, NP = PTabs2<N, Q>::NP;
  auto BF = [&](int i) { return tab2.BF[i]; };
  auto DF = [&](int i) { return tab2.DF[i]; };
  auto BT = [&](int i) { return tab2.BT[i]; };
  auto DT = [&](int i) { return tab2.DT[i]; };
  constexpr bool HALF = !std::is_same<TG, T>::value;
  using L = PipeLayout<T, N, Q, EB, NB, TG, V4>;
  constexpr int NQ = L::NQ, NM = N * N * N, TPE = Q * Q, GEO = L::GEO;
  constexpr int PJ = L::PJ, PK = L::PK, FS = L::FS;
  constexpr int NPT = (NM + TPE - 1) / TPE;  // coefficients gathered per thread
  // Q = 8: pencils along the unit-stride index go to threads (t / 8, t % 8) rather than
  // (t % 8, t / 8). With row stride 8 and plane stride 73 (= 9 mod 32) the 32 lanes of
  // a warp then hit 32 different shared-memory banks in every stage but the two
  // j-direction derivative stages (2-way); same arithmetic per pencil either way.
  constexpr bool M8 = (Q == 8);
  // V4 lanes of the j-direction pencils: i = t % 4 + 4 (t / 32), k = (t / 4) % 8
  const int vj_i = (threadIdx.x & 3) + 4 * (threadIdx.x >> 5), vj_k = (threadIdx.x >> 2) & 7;
  // TC: this lane's B fragments of the four 1-D tables, W[a][x] zero-padded to 8 x 8:
  // BwdTrans (B(a, z_x), a < N), derivative (l_a'(z_x)), its transpose (l_x'(z_a)) and
  // IProduct (B(x, z_a), x < N)
  TfFrag wbf{}, wdf{}, wdt{}, wbt{};
  if constexpr (TC) {
    const int g = (threadIdx.x & 31) >> 2, t4 = threadIdx.x & 3;
    auto bf = [&](int a, int x) { return a < N ? tab.B[a * Q + x] : T(0); };
    auto bt = [&](int a, int x) { return x < N ? tab.B[x * Q + a] : T(0); };
    wbf = tf_frag(bf(t4, g), bf(t4 + 4, g));
    wdf = tf_frag(tab.D[t4 * Q + g], tab.D[(t4 + 4) * Q + g]);
    wdt = tf_frag(tab.D[g * Q + t4], tab.D[g * Q + t4 + 4]);
    wbt = tf_frag(bt(t4, g), bt(t4 + 4, g));
  }
  if (skip != nullptr && *skip) return;  // converged solve: the whole CTA leaves together
  if (lam_ptr != nullptr) lambda = *lam_ptr;

  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem);  // bar[0] (and bar[1] with NB = 2)
  unsigned char* geo_base = smem + 16;
  T* work = reinterpret_cast<T*>(smem + 16 + NB * L::GEO_BYTES);

  const int t = threadIdx.x, el = threadIdx.y;
  const int tid = t + el * TPE;
  const int ngroups = (E + EB - 1) / EB;
  T* SU = work + el * 3 * FS;
  T* S0 = SU + FS;
  T* S1 = S0 + FS;

  // TMA window of group `grp` into buffer `b`; returns the byte shift of its first element.
  auto issue_geometry = [&](int grp, int b) {
    const int e0 = grp * EB, ne = min(EB, E - e0);
    const uintptr_t a0 = reinterpret_cast<uintptr_t>(jg + (size_t)e0 * GEO);
    const uintptr_t lo = a0 & ~uintptr_t(15);
    const uintptr_t hi = (a0 + (size_t)ne * GEO * sizeof(TG) + 15) & ~uintptr_t(15);
    mbar_arrive_expect_tx(bar + b, static_cast<uint32_t>(hi - lo));
    // the geometry is read once per launch: evict it from L2 first
    tma_bulk_load_hint(geo_base + b * L::GEO_BYTES, reinterpret_cast<const void*>(lo), static_cast<uint32_t>(hi - lo),
                       bar + b, l2_evict_first_policy());
  };
  auto geometry_of = [&](int grp, int b) -> const TG* {
    const uintptr_t a0 = reinterpret_cast<uintptr_t>(jg + (size_t)grp * EB * GEO);
    const int shift = static_cast<int>(a0 & uintptr_t(15));
    return reinterpret_cast<const TG*>(geo_base + b * L::GEO_BYTES + shift) + el * GEO;
  };

  // Coefficient slot j of this thread is mode m = t + j TPE (every slot but the last
  // is always a mode); its shared-memory offset in the (p, q, r) work layout does not
  // depend on the element, so it is computed once here rather than per element.
  int soff[NPT];
#pragma unroll
  for (int j = 0; j < NPT; ++j) {
    const int m = t + j * TPE;
    soff[j] = m < NM ? (m % N) + PJ * ((m / N) % N) + PK * (m / (N * N)) : -1;
  }
  auto slot_ok = [&](int j) { return j < NPT - 1 || soff[j] >= 0; };

  // prefetch registers: raw gathered values and a sign mask for the next group, the
  // signed l2g codes of the next group (code) and of the one after (code2): the codes
  // are loaded two groups ahead, so the dependent value gather never waits on them
  T xv[NPT];
  int code[NPT], code2[NPT] = {};
  unsigned neg = 0;
  // scattered output (ocode != nullptr): the current group's output codes, signs and
  // gathered values; an output code is g | kOwnedBit for an owned row (a free row with a
  // single local entry, written to sown[g] here), the position of the signed local
  // value in the assembly-ordered buffer `out` otherwise, or negative (not written)
  int gcur[NPT];
  T wcur[NPT];
  unsigned neg_cur = 0;
  // this thread's share of s.w: with s = P^T y (assembly) and the gathered input P w,
  // s.w = y.(P w), the local values times their signed gathered inputs (zero on
  // Dirichlet rows), so the whole dot is summed here and the assembly needs no w
  T loc_sw = 0;
  auto load_codes = [&](int grp, int (&dst)[NPT]) {
    const int e = grp * EB + el;
    const int* lp = l2g + (size_t)min(e, E - 1) * NM + t;
#pragma unroll
    for (int j = 0; j < NPT; ++j) {
      dst[j] = 0;
      if (e < E && slot_ok(j)) {
        if constexpr (GATHER) dst[j] = __ldcs(lp + j * TPE);  // read once per launch
      }
    }
  };
  auto load_values = [&](int grp) {
    const int e = grp * EB + el;
    const T* ip = in + (size_t)min(e, E - 1) * NM + t;
    neg = 0;
#pragma unroll
    for (int j = 0; j < NPT; ++j) {
      xv[j] = T(0);
      if (e < E && slot_ok(j)) {
        if constexpr (GATHER) {
          const int c = code[j];
          const int g = c >= 0 ? c : ~c;
          if (g >= ndir) xv[j] = in[g];
          neg |= (c < 0 ? 1u : 0u) << j;
        } else {
          xv[j] = ip[j * TPE];
        }
      }
    }
  };

  int grp = blockIdx.x;
  if (grp >= ngroups) return;
  if (tid == 0) {
    mbar_init(bar, 1);
    if (NB == 2) mbar_init(bar + 1, 1);
    fence_barrier_init();
  }
  __syncthreads();
  if (tid == 0) issue_geometry(grp, 0);
  load_codes(grp, code);
  load_values(grp);
  if (grp + (int)gridDim.x < ngroups) load_codes(grp + gridDim.x, code);

  for (int it = 0; grp < ngroups; ++it, grp += gridDim.x) {
    const int b = NB == 2 ? (it & 1) : 0;
    const uint32_t parity = NB == 2 ? ((it >> 1) & 1) : (it & 1);
    const int nxt = grp + gridDim.x;
    const bool has_next = nxt < ngroups;
    const int e = grp * EB + el;
    const bool active = e < E;
    // the other buffer was last read in the previous iteration, which ended in a barrier
    if (NB == 2 && tid == 0 && has_next) issue_geometry(nxt, b ^ 1);

    // ---- 1: prefetched coefficients -> S0 as (p, q, r); then the next group's codes ----
#pragma unroll
    for (int j = 0; j < NPT; ++j)
      if (slot_ok(j)) S0[soff[j]] = (neg >> j) & 1u ? -xv[j] : xv[j];
    if (ocode != nullptr) {  // what the scattered output stage needs; the codes arrive
      neg_cur = neg;         // during the stages below
      const int* cp = ocode + (size_t)(active ? e : 0) * NM + t;
#pragma unroll
      for (int j = 0; j < NPT; ++j) {
        gcur[j] = active && slot_ok(j) ? __ldcs(cp + j * TPE) : -1;
        wcur[j] = xv[j];
      }
    }
    const int nxt2 = nxt + gridDim.x;
    if (nxt2 < ngroups) load_codes(nxt2, code2);
    T gs[7];  // per-field scales of this element (half-precision geometry), used at stage 6
    if constexpr (HALF) {
      const float* sc = gscale + (size_t)min(e, E - 1) * 8;
#pragma unroll
      for (int f = 0; f < 7; ++f) gs[f] = __ldg(sc + f);
    }
    __syncthreads();
    // ---- 2: BwdTrans along p: pencils (q, r) ----
    if constexpr (TC) {
      tc_contract<0, N>(S0, S1, wbf, t, [](int q, int r) { return q < N && r < N; });
    } else if constexpr (V4) {
      const int q = t / 8, r = t % 8;
      if (q < N && r < N) {
        T c[N], o[Q];
        lds8(S0 + PJ * q + PK * r, c);
        op_bwd(c, o);
        sts8(S1 + PJ * q + PK * r, o);
      }
    } else if (M8 ? (t / 8 < N && t % 8 < N) : t < N * N) {
      const int q = M8 ? t / 8 : t % N, r = M8 ? t % 8 : t / N;
      T c[N];
#pragma unroll
      for (int p = 0; p < N; ++p) c[p] = S0[p + PJ * q + PK * r];
      if constexpr (PACK || EO) {
        T o[Q];
        op_bwd(c, o);
#pragma unroll
        for (int i = 0; i < Q; ++i) S1[i + PJ * q + PK * r] = o[i];
      } else {
#pragma unroll
        for (int i = 0; i < Q; ++i) {
          T acc = tab.B[i] * c[0];
#pragma unroll
          for (int p = 1; p < N; ++p) acc = fma(tab.B[p * Q + i], c[p], acc);
          S1[i + PJ * q + PK * r] = acc;
        }
      }
    }
    __syncthreads();
    // ---- 3: along q: pencils (i, r) ----
    if constexpr (TC) {
      tc_contract<1, N>(S1, S0, wbf, t, [](int, int r) { return r < N; });
    } else if constexpr (V4) {
      const int i = vj_i, r = vj_k;
      if (r < N) {
        T c[N], o[Q];
#pragma unroll
        for (int q = 0; q < N; ++q) c[q] = S1[i + PJ * q + PK * r];
        op_bwd(c, o);
#pragma unroll
        for (int j = 0; j < Q; ++j) S0[i + PJ * j + PK * r] = o[j];
      }
    } else if (M8 ? t % 8 < N : t < Q * N) {
      const int i = M8 ? t / 8 : t % Q, r = M8 ? t % 8 : t / Q;
      T c[N];
#pragma unroll
      for (int q = 0; q < N; ++q) c[q] = S1[i + PJ * q + PK * r];
      if constexpr (PACK || EO) {
        T o[Q];
        op_bwd(c, o);
#pragma unroll
        for (int j = 0; j < Q; ++j) S0[i + PJ * j + PK * r] = o[j];
      } else {
#pragma unroll
        for (int j = 0; j < Q; ++j) {
          T acc = tab.B[j] * c[0];
#pragma unroll
          for (int q = 1; q < N; ++q) acc = fma(tab.B[q * Q + j], c[q], acc);
          S0[i + PJ * j + PK * r] = acc;
        }
      }
    }
    __syncthreads();
    // ---- 4: along r: columns (i, j) -> u in registers; d/dxi_2 in registers ----
    const int ci = t % Q, cj = t / Q;
    T u[Q], g2[Q];
    {
      T c[N];
#pragma unroll
      for (int r = 0; r < N; ++r) c[r] = S0[ci + PJ * cj + PK * r];
      if constexpr (PACK || EO) {
        op_bwd(c, u);
        op_der(u, g2);
      } else {
#pragma unroll
        for (int k = 0; k < Q; ++k) {
          T acc = tab.B[k] * c[0];
#pragma unroll
          for (int r = 1; r < N; ++r) acc = fma(tab.B[r * Q + k], c[r], acc);
          u[k] = acc;
        }
#pragma unroll
        for (int k = 0; k < Q; ++k) {
          T acc = tab.D[k] * u[0];
#pragma unroll
          for (int c2 = 1; c2 < Q; ++c2) acc = fma(tab.D[c2 * Q + k], u[c2], acc);
          g2[k] = acc;
        }
      }
#pragma unroll
      for (int k = 0; k < Q; ++k) SU[ci + PJ * cj + PK * k] = u[k];
    }
    __syncthreads();
    // ---- 5: d/dxi_0 on pencils (j, k) -> S0 ; d/dxi_1 on pencils (i, k) -> S1 ----
    if constexpr (TC) {
      tc_contract<0, Q>(SU, S0, wdf, t, [](int, int) { return true; });
      tc_contract<1, Q>(SU, S1, wdf, t, [](int, int) { return true; });
    } else if constexpr (V4) {
      T c[Q], o[Q];
      lds8(SU + PJ * (t / 8) + PK * (t % 8), c);
      op_der(c, o);
      sts8(S0 + PJ * (t / 8) + PK * (t % 8), o);
#pragma unroll
      for (int a = 0; a < Q; ++a) c[a] = SU[vj_i + PJ * a + PK * vj_k];
      op_der(c, o);
#pragma unroll
      for (int j = 0; j < Q; ++j) S1[vj_i + PJ * j + PK * vj_k] = o[j];
    } else {
      const int pj = M8 ? t / 8 : t % Q, pk = M8 ? t % 8 : t / Q;
      T c[Q];
#pragma unroll
      for (int a = 0; a < Q; ++a) c[a] = SU[a + PJ * pj + PK * pk];
      const int pi = t % Q, pkb = t / Q;
      if constexpr (PACK || EO) {
        T o[Q];
        op_der(c, o);
#pragma unroll
        for (int i = 0; i < Q; ++i) S0[i + PJ * pj + PK * pk] = o[i];
#pragma unroll
        for (int a = 0; a < Q; ++a) c[a] = SU[pi + PJ * a + PK * pkb];
        op_der(c, o);
#pragma unroll
        for (int j = 0; j < Q; ++j) S1[pi + PJ * j + PK * pkb] = o[j];
      } else {
#pragma unroll
        for (int i = 0; i < Q; ++i) {
          T acc = tab.D[i] * c[0];
#pragma unroll
          for (int a = 1; a < Q; ++a) acc = fma(tab.D[a * Q + i], c[a], acc);
          S0[i + PJ * pj + PK * pk] = acc;
        }
#pragma unroll
        for (int a = 0; a < Q; ++a) c[a] = SU[pi + PJ * a + PK * pkb];
#pragma unroll
        for (int j = 0; j < Q; ++j) {
          T acc = tab.D[j] * c[0];
#pragma unroll
          for (int a = 1; a < Q; ++a) acc = fma(tab.D[a * Q + j], c[a], acc);
          S1[pi + PJ * j + PK * pkb] = acc;
        }
      }
    }
    // the next group's gather: its codes were loaded a whole group ago
    if (has_next) load_values(nxt);
#pragma unroll
    for (int j = 0; j < NPT; ++j) code[j] = code2[j];  // the group after next becomes next
    // geometry of this group must have landed before the point-wise stage
    const bool ok = mbar_wait_bounded(bar + b, parity, kWaitCycles);
    if (!__syncthreads_and(ok)) {
      if (tid == 0 && err != nullptr) atomicExch(err, ITHACA_GPU_ERR_TIMEOUT);
      // give the copies in flight time to finish before the CTA's shared memory goes away
      mbar_wait_bounded(bar + b, parity, kWaitCycles);
      if (NB == 2 && has_next) mbar_wait_bounded(bar + (b ^ 1), ((it + 1) >> 1) & 1, kWaitCycles);
      return;
    }
    const TG* G = geometry_of(grp, b);
    auto geo = [&](int f, int pt) -> T {
      if constexpr (HALF)
        return __half2float(G[f * NQ + pt]) * gs[f];
      else
        return G[f * NQ + pt];
    };
    // ---- 6: point-wise metric on columns (i, j) ----
    T v[Q];
    {
      T f2[Q];
#pragma unroll
      for (int k = 0; k < Q; ++k) {
        const int s = ci + PJ * cj + PK * k;
        const int pt = ci + Q * cj + Q * Q * k;
        const T g0 = S0[s], g1 = S1[s];
        const T jw = geo(0, pt);
        const T m00 = geo(1, pt), m01 = geo(2, pt), m02 = geo(3, pt);
        const T m11 = geo(4, pt), m12 = geo(5, pt), m22 = geo(6, pt);
        S0[s] = fma(m00, g0, fma(m01, g1, m02 * g2[k]));
        S1[s] = fma(m01, g0, fma(m11, g1, m12 * g2[k]));
        f2[k] = fma(m02, g0, fma(m12, g1, m22 * g2[k]));
        v[k] = lambda * jw * u[k];
      }
      if constexpr (PACK || EO) {
        op_dert_add(f2, v);
      } else {
#pragma unroll
        for (int k = 0; k < Q; ++k) {
          T acc = v[k];
#pragma unroll
          for (int c2 = 0; c2 < Q; ++c2) acc = fma(tab.D[k * Q + c2], f2[c2], acc);
          v[k] = acc;
        }
      }
    }
    __syncthreads();
    // single buffer: stage 6 has read it, so the next group's copy can start now
    if (NB == 1 && tid == 0 && has_next) issue_geometry(nxt, 0);
    // ---- 7: D^T along i on pencils (j, k) in S0, along j on pencils (i, k) in S1 ----
    if constexpr (TC) {
      tc_contract<0, Q>(S0, S0, wdt, t, [](int, int) { return true; });
      tc_contract<1, Q>(S1, S1, wdt, t, [](int, int) { return true; });
    } else if constexpr (V4) {
      T c[Q], o[Q];
      lds8(S0 + PJ * (t / 8) + PK * (t % 8), c);
      op_dert(c, o);
      sts8(S0 + PJ * (t / 8) + PK * (t % 8), o);
#pragma unroll
      for (int a = 0; a < Q; ++a) c[a] = S1[vj_i + PJ * a + PK * vj_k];
      op_dert(c, o);
#pragma unroll
      for (int j = 0; j < Q; ++j) S1[vj_i + PJ * j + PK * vj_k] = o[j];
    } else {
      const int pj = M8 ? t / 8 : t % Q, pk = M8 ? t % 8 : t / Q;
      T c[Q], o[Q];
#pragma unroll
      for (int a = 0; a < Q; ++a) c[a] = S0[a + PJ * pj + PK * pk];
      if constexpr (PACK || EO) {
        op_dert(c, o);
      } else {
#pragma unroll
        for (int i = 0; i < Q; ++i) {
          T acc = tab.D[i * Q] * c[0];
#pragma unroll
          for (int a = 1; a < Q; ++a) acc = fma(tab.D[i * Q + a], c[a], acc);
          o[i] = acc;
        }
      }
#pragma unroll
      for (int i = 0; i < Q; ++i) S0[i + PJ * pj + PK * pk] = o[i];
      const int pi = t % Q, pkb = t / Q;
#pragma unroll
      for (int a = 0; a < Q; ++a) c[a] = S1[pi + PJ * a + PK * pkb];
      if constexpr (PACK || EO) {
        op_dert(c, o);
      } else {
#pragma unroll
        for (int j = 0; j < Q; ++j) {
          T acc = tab.D[j * Q] * c[0];
#pragma unroll
          for (int a = 1; a < Q; ++a) acc = fma(tab.D[j * Q + a], c[a], acc);
          o[j] = acc;
        }
      }
#pragma unroll
      for (int j = 0; j < Q; ++j) S1[pi + PJ * j + PK * pkb] = o[j];
    }
    __syncthreads();
    // ---- 8: sum the three directions on columns, IProduct along k -> SU as (i, j, r) ----
    {
#pragma unroll
      for (int k = 0; k < Q; ++k) {
        const int s = ci + PJ * cj + PK * k;
        v[k] += S0[s] + S1[s];
      }
      if constexpr (PACK || EO) {
        T o[N];
        op_ipr(v, o);
#pragma unroll
        for (int r = 0; r < N; ++r) SU[ci + PJ * cj + PK * r] = o[r];
      } else {
#pragma unroll
        for (int r = 0; r < N; ++r) {
          T acc = tab.B[r * Q] * v[0];
#pragma unroll
          for (int k = 1; k < Q; ++k) acc = fma(tab.B[r * Q + k], v[k], acc);
          SU[ci + PJ * cj + PK * r] = acc;
        }
      }
    }
    __syncthreads();
    // ---- 9: along j: pencils (i, r) -> S0 as (i, q, r) ----
    if constexpr (TC) {
      tc_contract<1, Q>(SU, S0, wbt, t, [](int, int r) { return r < N; });
    } else if constexpr (V4) {
      const int i = vj_i, r = vj_k;
      if (r < N) {
        T c[Q], o[N];
#pragma unroll
        for (int j = 0; j < Q; ++j) c[j] = SU[i + PJ * j + PK * r];
        op_ipr(c, o);
#pragma unroll
        for (int q = 0; q < N; ++q) S0[i + PJ * q + PK * r] = o[q];
      }
    } else if (M8 ? t % 8 < N : t < Q * N) {
      const int i = M8 ? t / 8 : t % Q, r = M8 ? t % 8 : t / Q;
      T c[Q];
#pragma unroll
      for (int j = 0; j < Q; ++j) c[j] = SU[i + PJ * j + PK * r];
      if constexpr (PACK || EO) {
        T o[N];
        op_ipr(c, o);
#pragma unroll
        for (int q = 0; q < N; ++q) S0[i + PJ * q + PK * r] = o[q];
      } else {
#pragma unroll
        for (int q = 0; q < N; ++q) {
          T acc = tab.B[q * Q] * c[0];
#pragma unroll
          for (int j = 1; j < Q; ++j) acc = fma(tab.B[q * Q + j], c[j], acc);
          S0[i + PJ * q + PK * r] = acc;
        }
      }
    }
    __syncthreads();
    // ---- 10: along i: pencils (q, r) -> S1 as (p, q, r) ----
    if constexpr (TC) {
      tc_contract<0, Q>(S0, S1, wbt, t, [](int q, int r) { return q < N && r < N; });
    } else if constexpr (V4) {
      const int q = t / 8, r = t % 8;
      if (q < N && r < N) {
        T c[Q], o[N];
        lds8(S0 + PJ * q + PK * r, c);
        op_ipr(c, o);
        sts8(S1 + PJ * q + PK * r, o);  // p = N..7 of the pencil: padding, written as zero
      }
    } else if (M8 ? (t / 8 < N && t % 8 < N) : t < N * N) {
      const int q = M8 ? t / 8 : t % N, r = M8 ? t % 8 : t / N;
      T c[Q];
#pragma unroll
      for (int i = 0; i < Q; ++i) c[i] = S0[i + PJ * q + PK * r];
      if constexpr (PACK || EO) {
        T o[N];
        op_ipr(c, o);
#pragma unroll
        for (int p = 0; p < N; ++p) S1[p + PJ * q + PK * r] = o[p];
      } else {
#pragma unroll
        for (int p = 0; p < N; ++p) {
          T acc = tab.B[p * Q] * c[0];
#pragma unroll
          for (int i = 1; i < Q; ++i) acc = fma(tab.B[p * Q + i], c[i], acc);
          S1[p + PJ * q + PK * r] = acc;
        }
      }
    }
    __syncthreads();
    if (active) {
      T* op = out + (size_t)e * NM + t;
#pragma unroll
      for (int j = 0; j < NPT; ++j) {
        if (!slot_ok(j)) continue;
        const T val = S1[soff[j]];
        if (ocode != nullptr) {
          const int oc = gcur[j];
          const T sv = (neg_cur >> j) & 1u ? -val : val;
          if (oc >= 0 && (oc & kOwnedBit))  // owned row: assembled here
            sown[oc & (kOwnedBit - 1)] = sv;
          else if (oc >= 0)
            out[oc] = sv;
          loc_sw = fma(sv, wcur[j], loc_sw);
        } else {
          op[j * TPE] = val;
        }
      }
    }
    // S0 and S1 are rewritten by the next group's stages 1-2; with NB = 2 the geometry
    // buffer read here is refilled by the copy issued at the top of the iteration after next
    __syncthreads();
  }
  if (opart != nullptr) {  // this CTA's share of s.w: warp sums in T, the CTA sum in FP64
    // Q^2 EB threads need not fill the last warp: shuffle among its existing lanes only
    constexpr int NT = Q * Q * EB, NW = (NT + 31) / 32;
    const int nl = min(32, NT - (tid & ~31)), lane = tid & 31;
    const unsigned mask = nl == 32 ? 0xffffffffu : (1u << nl) - 1u;
    T v = loc_sw;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      const T o = __shfl_down_sync(mask, v, off);
      if (lane + off < nl) v += o;
    }
    double* red = reinterpret_cast<double*>(work);  // the work area is free after the loop
    if ((tid & 31) == 0) red[tid >> 5] = (double)v;
    __syncthreads();
    if (tid == 0) {
      double sum = red[0];
      for (int w = 1; w < NW; ++w) sum += red[w];
      opart[blockIdx.x] = sum;
    }
  }
}

}  // namespace dev
}  // namespace ithaca
