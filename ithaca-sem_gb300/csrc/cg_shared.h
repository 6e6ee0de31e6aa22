// Data shared by the conjugate-gradient solvers (cg.cu) and the persistent small-system
// solver (cg_persist.cu): the scalar state of the recurrence and the assembly plan.
#pragma once

#include "ithaca_internal.h"

namespace ithaca {

// Scalar state of the reference recurrence (NekLinSysIterCG.cpp:104-263) on the device.
struct CgScalars {
  double alpha, beta, rho, mu, eps, rhs_mag, tol2, mag_override;
  double lambda;
  float lambda32, pad0;
  int iters, k, done, status, max_iter;
  int fresh;  // alpha / beta were just set by the initial step (fused inner iteration)
};

// ---- assembly plan: rows grouped by their number of local entries ----------------
// Class c < kAsmK holds the rows with exactly c + 1 local entries, stored ELL-style
// (entry j of row slot i at cols[col_off + j * n + i], entries in increasing local
// index, as the reference's scatter-add visits them); class kAsmK holds the rows with
// more entries, which are read through the CSR arrays. Inside a class the rows are in
// increasing global order, so the Dirichlet rows (numbered first) lead each class.
// The CTAs of a launch are split among the classes in proportion to their entries, so
// every CTA (and warp) handles rows of one length: no divergence, and each thread keeps
// up to kAsmK independent entry loads in flight.
constexpr int kAsmK = 8;
struct AsmPlan {
  int n[kAsmK + 1];          // rows per class
  int ndir[kAsmK + 1];       // leading Dirichlet rows per class
  int rows_off[kAsmK + 1];   // first slot of the class in the row list
  long long col_off[kAsmK];  // first ELL entry of the class
  long long tail_off;        // assembly-ordered buffer: first entry of the tail class
  int cta0[kAsmK + 2];       // CTAs [cta0[c], cta0[c + 1]) work on class c
};

// Arguments of the persistent small-system solver: the whole PCG of one system (initial
// step and iterations) in one cooperative launch, phases separated by grid barriers.
template <typename T>
struct PersistArgs {
  int N, ndir, E, deformed;
  const int* l2g;       // signed local-to-global codes
  const int* ocode;     // output codes of the scattered element output (OwnedRows)
  const int* asm_rows;  // global rows by class (AsmPlan)
  const int* tail_ptr;  // tail rows: first slot of each row's entries
  AsmPlan plan;         // the full plan (class 0 free rows are the owned rows)
  T *x, *r, *w, *s, *p, *q, *yslot;
  const T *b, *dinv, *tab, *jg;
  double* part;         // 6 x gridDim.x partial sums (slots: r.w, r.r, b.b, s.w, r.w', r.r')
  unsigned* bar;        // grid barrier: arrival count, generation (zeroed before launch)
  int* err;             // device error word
  CgScalars* sc;        // in: tol2, mag_override, max_iter, lambda; out: the final state
  // failure-path test hooks, zero in a solve: barrier poll limit (0: the default),
  // a CTA that never arrives at its first barrier (-1: none), and a pause in ns of every
  // third CTA after each barrier (0: none)
  long long dbg_polls;
  int dbg_drop_cta, dbg_delay_ns;
};

// Launches the persistent solver for quads with n modes and Q = n + 1 points; returns
// false when (n, Q) is not built or the system is not suited (the caller then runs the
// graph-captured kernels).
template <typename T>
bool launch_cg2_persistent(int n, int Q, const PersistArgs<T>& a, int sms, cudaStream_t s);

}  // namespace ithaca
