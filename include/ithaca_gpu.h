/*
 * ithaca_gpu.h -- C ABI of the GB300 (sm_103a) implementation of the spectral/hp
 * Helmholtz + conjugate-gradient + POD hot path of ITHACA-SEM (Nektar++ 5.0.0).
 *
 * Plain C: opaque handles, raw pointers and sizes, int status codes, no exceptions
 * and no C++ or torch types across the boundary. Every call returns ITHACA_GPU_OK (0)
 * or a positive ITHACA_GPU_ERR_* code; ithaca_gpu_last_error() gives the message
 * (thread-local). Pointers flagged by `on_device` are device pointers when it is 1
 * and host pointers when it is 0 (the library then stages them through device
 * buffers itself). All arrays use the reference's element-contiguous layouts:
 *
 *   coefficients  quad e*n^2 + q*n + p          hex e*n^3 + (r*n + q)*n + p
 *   physical      quad e*Q^2 + j*Q + i          hex e*Q^3 + (k*Q + j)*Q + i
 *   jac           deformed: e*Q^d + pt          regular: e
 *   df            deformed: dir*E*Q^d + e*Q^d + pt   regular: dir*E + e,
 *                 dir = k*d + j holding dxi_j/dx_k
 *                 (Collections/CoalescedGeomData.cpp:53-313 GetJac/GetDerivFactors)
 *
 * Threading: a context owns one CUDA stream; calls on one context are not
 * re-entrant (like the reference operators, which keep mutable work buffers).
 */
#ifndef ITHACA_GPU_H
#define ITHACA_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (the reference raises NekError; the adapter maps these back) ---- */
enum {
  ITHACA_GPU_OK = 0,
  ITHACA_GPU_ERR_ARG = 1,           /* invalid argument (null pointer, bad size)        */
  ITHACA_GPU_ERR_UNSUPPORTED = 2,   /* shape / (modes, points) combination not built    */
  ITHACA_GPU_ERR_CUDA = 3,          /* CUDA runtime error (message has the detail)      */
  ITHACA_GPU_ERR_NOMEM = 4,         /* device allocation failed                          */
  ITHACA_GPU_ERR_NOT_CONVERGED = 5, /* iterative solve hit max_iter (reference: efatal)  */
  ITHACA_GPU_ERR_GEOMETRY = 6,      /* non-positive Jacobian (GeomFactors.cpp:610-676)   */
  ITHACA_GPU_ERR_TIMEOUT = 7,       /* a bounded device-side wait gave up                */
  ITHACA_GPU_ERR_NUMERIC = 8        /* NaN / Inf met in a reduction                      */
};

/* LibUtilities::ShapeType values of the supported shapes (LibUtilities/BasicUtils/ShapeType.hpp). */
enum {
  ITHACA_GPU_SHAPE_TRI = 3,
  ITHACA_GPU_SHAPE_QUAD = 4,
  ITHACA_GPU_SHAPE_TET = 5,
  ITHACA_GPU_SHAPE_PYR = 6,
  ITHACA_GPU_SHAPE_PRISM = 7,
  ITHACA_GPU_SHAPE_HEX = 8
};

/* Arithmetic of an element operator. */
enum { ITHACA_GPU_FP64 = 0, ITHACA_GPU_FP32 = 1 };

/* Solver precision modes for ithaca_gpu_cg_solve. */
enum {
  ITHACA_GPU_SOLVE_FP64 = 0,        /* reference recurrence, FP64 throughout             */
  ITHACA_GPU_SOLVE_MIXED_FP32 = 1,  /* FP32 inner PCG inside FP64 iterative refinement   */
  ITHACA_GPU_SOLVE_MIXED_FP32_GEO16 = 2 /* as MIXED_FP32, with the inner applies reading
                                         * 16-bit geometry (per-element scaled halves);
                                         * curved hexahedra only (else ERR_UNSUPPORTED) */
};

typedef struct ithaca_gpu_ctx ithaca_gpu_ctx;
typedef struct ithaca_gpu_op ithaca_gpu_op;
typedef struct ithaca_gpu_cg ithaca_gpu_cg;

/* ---- errors / context ---- */

/* Copies the last error message of this thread into buf (NUL-terminated). */
int ithaca_gpu_last_error(char* buf, size_t len);
int ithaca_gpu_version(void);

/* Creates a context on `device` with its own non-blocking stream. */
int ithaca_gpu_ctx_create(int device, ithaca_gpu_ctx** ctx);
int ithaca_gpu_ctx_destroy(ithaca_gpu_ctx* ctx);
/* Blocks until all work queued on the context's stream has finished. */
int ithaca_gpu_ctx_synchronize(ithaca_gpu_ctx* ctx);
/* The context's cudaStream_t, returned as void* (for event timing by callers). */
int ithaca_gpu_ctx_stream(ithaca_gpu_ctx* ctx, void** stream);
/* Number of library kernels launched on this context so far. */
int ithaca_gpu_ctx_launch_count(ithaca_gpu_ctx* ctx, long long* count);

/* ---- 1-D tables (LibUtilities/Polylib/Polylib.cpp:195,690 zwglj/Dglj;
 *      LibUtilities/Foundations/Basis.cpp:392-421 eModified_A) ----
 * z, w: Q; D: Q*Q with D[k*Q+i] = l_k'(z_i); B, DB: n*Q with B[p*Q+i]. Host arrays. */
int ithaca_gpu_basis_modA(int nmodes, int npoints, double* z, double* w, double* D, double* B, double* DB);

/* ---- triangle basis: eModified_A on Q0 = nmodes + 1 GLL points (direction 0) and
 *      eModified_B on Q1 = nmodes Gauss-Radau-Jacobi (alpha 1, beta 0) points (direction
 *      1), the default keys of SpatialDomains/MeshGraph.cpp:1665-1681; Polylib.cpp:119-144
 *      zwgrjm, :589-626 Dgrjm; Basis.cpp:423-507 eModified_B ----
 * Direction 0 as ithaca_gpu_basis_modA(nmodes, nmodes + 1). Direction 1: z1, w1 (Q1, the
 * weights as Basis::GetW holds them, without the collapsed map's factor 1/2), D1 (Q1*Q1,
 * D1[l*Q1+j] = l_l'(z1_j)), B1 and DB1 (nc*Q1 with nc = nmodes (nmodes+1)/2, mode
 * m(p, q) with q fastest: B1[m*Q1 + j]). Host arrays; any pointer may be NULL. */
int ithaca_gpu_basis_tri(int nmodes, double* z0, double* w0, double* D0, double* B0, double* DB0, double* z1,
                         double* w1, double* D1, double* B1, double* DB1);

/* ---- tetrahedron basis, direction 2: eModified_C on Q2 = nmodes Gauss-Radau-Jacobi
 *      (alpha 2, beta 0) points (MeshGraph.cpp:1683-1716; Basis.cpp:512-566: the row of mode
 *      m(p, q, r), r fastest, is the eModified_B row (p + q, r)) ----
 * Directions 0 and 1 are those of ithaca_gpu_basis_tri(nmodes, ...). z2, w2 (Q2, weights as
 * Basis::GetW holds them, without the collapsed map's factor 1/4), D2 (Q2*Q2), B2 and DB2
 * (nc*Q2, nc = nmodes (nmodes+1) (nmodes+2) / 6). Host arrays; any pointer may be NULL. */
int ithaca_gpu_basis_tet(int nmodes, double* z2, double* w2, double* D2, double* B2, double* DB2);

/* ---- pyramid basis, direction 2: eModifiedPyr_C on Q2 = nmodes Gauss-Radau-Jacobi
 *      (alpha 2, beta 0) points (MeshGraph.cpp:1719-1745; Basis.cpp:568-672) ----
 * Directions 0 and 1 are ithaca_gpu_basis_modA(nmodes, nmodes + 1). z2, w2 (Q2, without
 * the collapsed map's factor 1/4), D2 (Q2*Q2), B2 and DB2 (nc*Q2, nc = nmodes (nmodes+1)
 * (2 nmodes+1) / 6, modes m(p, q, r) with r fastest and r < nmodes - max(p, q)). */
int ithaca_gpu_basis_pyr(int nmodes, double* z2, double* w2, double* D2, double* B2, double* DB2);

/* ---- geometry (SpatialDomains/GeomFactors.cpp:168-475 ComputeDeriv/ComputeJac/
 *      ComputeDerivFactors) ----
 * coords: d arrays of E*Q^d physical coordinates at the GLL quadrature points,
 * stored one after another (coordinate k at coords[k*E*Q^d]). Writes jac (E*Q^d)
 * and df (d*d*E*Q^d) in the deformed layout above. Returns ITHACA_GPU_ERR_GEOMETRY
 * if any Jacobian is not positive. Triangles (shape 3): npoints = Q0, the coordinates
 * at the Q0 x Q1 collapsed points (point j*Q0 + i, Q1 = Q0 - 1), 2 arrays of E*Q0*Q1;
 * the derivatives are taken in collapsed coordinates and mapped by the chain rule of
 * StdTriExp::v_PhysDeriv. Tetrahedra (shape 5): npoints = Q0, coordinates at the
 * Q0 x (Q0-1) x (Q0-1) collapsed points (point (k Q1 + j) Q0 + i), 3 arrays; chain rule of
 * StdTetExp::v_PhysDeriv. Prisms (shape 7): npoints = Q0, coordinates at the Q0 x Q0 x
 * (Q0-1) points (point (k Q0 + j) Q0 + i), chain rule of StdPrismExp::v_PhysDeriv; pyramids
 * (shape 6) the same point set with the chain rule of StdPyrExp::v_PhysDeriv. */
int ithaca_gpu_geom_factors(ithaca_gpu_ctx* ctx, int shape, int npoints, int nelmt, const double* coords,
                            double* jac, double* df, int on_device);

/* ---- element operators: one Collection of same-shape elements ----
 * Replaces Collections::Operator (Collections/Operator.h:113-165) implementations
 * BwdTrans/IProductWRTBase/PhysDeriv/Helmholtz for ImplementationType "GPU", and
 * MatrixFree::Operator (MatrixFreeOps/Operator.hpp:21-201) with its SetJac/SetDF.
 * Basis: ModifiedA with `nmodes` modes on `npoints` GLL points in every direction
 * (the homogeneous case MatrixFreeOps/Helmholtz.h:42-44 requires). Supported:
 * npoints == nmodes + 1, 2 <= nmodes <= 10 (triangles: <= 12). `precision` selects the
 * arithmetic. Triangles (shape 3): the basis of ithaca_gpu_basis_tri with npoints = Q0 = nmodes + 1;
 * per element nmodes (nmodes + 1) / 2 coefficients and Q0 (Q0 - 1) points, geometry
 * (jac, df with d = 2) per point on those points or per element (MatrixFreeOps/
 * Helmholtz.h:290-330, 505-635; BwdTrans.h:540-570; IProduct.h:560-590;
 * PhysDeriv.h:470-500; IProductWRTDerivBase.h:671-1060). Tetrahedra (shape 5): the basis of
 * ithaca_gpu_basis_tet, nmodes (nmodes+1) (nmodes+2) / 6 coefficients and Q0 (Q0-1)^2 points
 * per element, geometry (d = 3) per point or per element (MatrixFreeOps/Helmholtz.h:
 * 1970-2010, 2266-2448; BwdTrans.h:1010-1045; IProduct.h:1730-1770; PhysDeriv.h:990-1030;
 * IProductWRTDerivBase.h:2212-2630); the library keeps their metric per point either way.
 * Prisms (shape 7): eModified_A on Q0 = nmodes + 1 GLL points in directions 0 and 1,
 * eModified_B (rows (p, r), the triangle's direction 1 of ithaca_gpu_basis_tri) on nmodes
 * Gauss-Radau points in direction 2; nmodes^2 (nmodes+1) / 2 coefficients and Q0^2 (Q0-1)
 * points per element, modes m(p, q, r) with r fastest and r < nmodes - p
 * (MatrixFreeOps/Helmholtz.h:1003-1030, 1291-1440; IProductWRTDerivBase.h:1660-1760).
 * Pyramids (shape 6): eModified_A in directions 0 and 1, eModifiedPyr_C of
 * ithaca_gpu_basis_pyr in direction 2; nmodes (nmodes+1) (2 nmodes+1) / 6 coefficients and
 * Q0^2 (Q0-1) points per element (MatrixFreeOps/Helmholtz.h:1480-1510, 1770-1960;
 * IProductWRTDerivBase.h:2070-2200). */
int ithaca_gpu_op_create(ithaca_gpu_ctx* ctx, int shape, int nmodes, int npoints, int nelmt, const double* jac,
                         const double* df, int deformed, int precision, int on_device, ithaca_gpu_op** op);
int ithaca_gpu_op_destroy(ithaca_gpu_op* op);
/* Ndof() = nelmt * nmodes^d (MatrixFreeOps/Helmholtz.h:279-282); nelmt * nmodes (nmodes+1)/2
 * for triangles, nelmt * nmodes (nmodes+1) (nmodes+2)/6 for tetrahedra, nelmt * nmodes^2 (nmodes+1)/2
 * for prisms, nelmt * nmodes (nmodes+1) (2 nmodes+1)/6 for pyramids. */
int ithaca_gpu_op_ndof(ithaca_gpu_op* op, long long* ndof);

/* BwdTrans (Collections/BwdTrans.cpp:143-240): coefficients -> physical values. */
int ithaca_gpu_bwdtrans(ithaca_gpu_op* op, const void* in, void* out, int on_device);
/* IProductWRTBase (Collections/IProductWRTBase.cpp:168-262): physical -> coefficients. */
int ithaca_gpu_iproduct(ithaca_gpu_op* op, const void* in, void* out, int on_device);
/* PhysDeriv (Collections/PhysDeriv.cpp:270-415): physical -> d physical derivatives.
 * d2 may be NULL for quads. */
int ithaca_gpu_physderiv(ithaca_gpu_op* op, const void* in, void* d0, void* d1, void* d2, int on_device);
/* IProductWRTDerivBase (Collections/IProductWRTDerivBase.cpp:446-546): physical
 * components in_k (E*Q^d each; in2 may be NULL for quads) -> coefficients
 * out = sum_k (d phi / d x_k, in_k). */
int ithaca_gpu_iproduct_deriv(ithaca_gpu_op* op, const void* in0, const void* in1, const void* in2, void* out,
                              int on_device);
/* Helmholtz (Collections/Helmholtz.cpp:391-430): out = lambda M in + L in, with
 * lambda = factors[eFactorLambda]. Arrays are double for FP64 ops and float for FP32. */
int ithaca_gpu_helmholtz(ithaca_gpu_op* op, double lambda, const void* in, void* out, int on_device);
/* Kernel choice for FP32 hexahedral Helmholtz applies (also used by the FP32 inner
 * solves of a system built on this operator): 0 = shared-memory sum-factorisation
 * kernel, 2 or 4 = register-pencil kernel with a TMA-staged geometry slab and that
 * many elements per CTA, 21 or 22 = the persistent pencil kernel that
 * prefetches the next group of 1 or 2 elements (geometry by TMA into a double buffer,
 * gathered coefficients into registers) while computing the current one, 31 or 32 =
 * the same with a single geometry buffer refilled right after its metric stage, 41 or
 * 42 = 31 or 32 with the 1-D contractions on packed FP32 pairs (same results; 41 is the
 * default), 43 or 44 = 42 or 41 with the unit-stride pencils moved as 16-byte words in a
 * bank-conflict-free shared-memory layout (same results), 46 = 43 with the contractions along
 * i and j as TF32 tensor-core MMAs in three-term split precision (FP32-level accuracy, not
 * bit-identical), 47 = 43 with every 1-D operator in its even-odd form (the symmetry of
 * the GLL points and the parity of the modes: half the multiply-adds; FP32-level accuracy,
 * not bit-identical); 43, 44, 46 and 47 are built for Q = 8, other orders run 42 or 41. On
 * 16-bit geometry (ITHACA_GPU_SOLVE_MIXED_FP32_GEO16) 43 and 47 have their own forms at
 * Q = 8 and every other variant runs the packed-pair kernel with one element per group.
 * Inside the mixed solver the pipelined variants (21-47) also write the rows of
 * the global system that have a single local entry themselves, so the assembly that
 * follows skips them. */
int ithaca_gpu_op_set_variant(ithaca_gpu_op* op, int variant);
/* FP64 hex Helmholtz kernel of a deformed hexahedral operator (the FP64 apply, the FP64
 * solves and the outer residuals of the mixed solve): 0 = the shared-memory kernel (default),
 * 1 / 2 = the persistent pipelined kernel with scalar FP64 pencils and every 1-D operator in
 * its even-odd form (the symmetry of the GLL points and the parity of the ModifiedA modes:
 * half the multiply-adds of the contractions), one / two elements per group; built for
 * Q = 4, 6, 8, 10, other orders keep the shared-memory kernel. FP64-level agreement with
 * variant 0, not bit-identical. */
int ithaca_gpu_op_set_variant64(ithaca_gpu_op* op, int variant);
/* Times every variant on the operator's own data and keeps the fastest, like
 * CollectionOptimisation::SetWithTimings (Collections/CollectionOptimisation.cpp:321-469)
 * picks an implementation type. times_ms (13 entries, may be NULL) receives the average
 * FP32 apply time of variants 0, 2, 4, 21, 22, 31, 32, 41, 42, 43, 44, 46, 47 (-1 where a
 * variant does not apply). */
int ithaca_gpu_op_autotune(ithaca_gpu_op* op, int reps, int* chosen, double* times_ms);
/* Diagonals of the element Helmholtz matrices (E*n^d), the per-element input of
 * PreconditionerDiagonal::DiagonalPreconditionerSum (PreconditionerDiagonal.cpp:98-161). */
int ithaca_gpu_helmholtz_diag(ithaca_gpu_op* op, double lambda, double* out, int on_device);

/* ---- global C0 system + conjugate gradient ----
 * Replaces GlobalLinSysIterativeFull (MultiRegions/GlobalLinSysIterativeFull.cpp:110-257)
 * with NekLinSysIterCG (LibUtilities/LinearAlgebra/NekLinSysIterCG.cpp:104-263) and
 * PreconditionerDiagonal. l2g/sign: the local-to-global map and signs of
 * AssemblyMapCG (one entry per local coefficient, E*n^d), global ids < nglobal with
 * the ndir Dirichlet ids numbered first. The operator `op` must be FP64. */
int ithaca_gpu_cg_create(ithaca_gpu_op* op, const int* l2g, const double* sign, int nglobal, int ndir,
                         ithaca_gpu_cg** cg);
int ithaca_gpu_cg_destroy(ithaca_gpu_cg* cg);

/* Solver path for 2-D systems. mode -1 (default): systems of at most 2^20 global dofs run
 * the persistent solver, one cooperative launch per (inner) PCG with the phases separated
 * by bounded grid barriers; larger ones the graph-captured kernels. 0: always the
 * graph-captured kernels. 1: always the persistent solver for 2-D systems. Both paths run
 * the same recurrence (NekLinSysIterCG.cpp:104-263); 3-D systems always use the graph. */
int ithaca_gpu_cg_set_persistent(ithaca_gpu_cg* cg, int mode);
/* FP32 inner iterations of the mixed solve (no reference counterpart): 1 fuses the
 * assembly of the element kernel's scattered output with the vector update of the same
 * iteration (two launches per iteration: the update computes the iteration's scalars
 * itself), 0 (default: measured faster on the 32^3 hexes) keeps the separate assembly and
 * update (three launches). The fused form needs
 * a pipelined FP32 element kernel (hexahedra, variants 21-47, or 16-bit geometry); with
 * other kernels the separate form runs. Same recurrence; the partial sums are grouped
 * differently, so iteration counts can differ by a few. */
int ithaca_gpu_cg_set_fused_update(ithaca_gpu_cg* cg, int on);

/* Successive right-hand sides: projection onto previous solutions (P. F. Fischer,
 * Comput. Methods Appl. Mech. Engrg. 163, 1998), as GlobalLinSysIterative::DoProjection /
 * UpdateKnownSolutions (MultiRegions/GlobalLinSysIterative.cpp:156-482) with the session
 * parameter SuccessiveRHS (AssemblyMap.cpp:168-175). nsuccessive > 0 keeps that many
 * A-conjugate normalised solutions, < 0 keeps |nsuccessive| solutions with the basis
 * A x / ||A x||, 0 turns the projection off (at most 64). Each later ithaca_gpu_cg_solve /
 * ithaca_gpu_helmsolve* call projects its right-hand side onto the stored solutions,
 * runs CG on the remainder (iterations in the result count that CG) and stores the new
 * solution. The stored solutions belong to one operator: a solve with another lambda, or
 * ithaca_gpu_cg_set_varcoeff, starts the buffer afresh. Resets the buffer. */
int ithaca_gpu_cg_set_successive_rhs(ithaca_gpu_cg* cg, int nsuccessive);

/* Test hooks of the persistent solver's failure path (no reference counterpart; the
 * reference has no device waits). barrier_polls: polls of ~64 ns before a grid-barrier
 * wait gives up (0: the default, about 1 s; at most 2^24). drop_cta: that CTA never
 * arrives at its first barrier, so every wait runs out and the solve returns
 * ITHACA_GPU_ERR_TIMEOUT with the context still usable (-1: none). delay_ns: every third
 * CTA pauses that long after each barrier, so the others run ahead into the next phase
 * (a race stress; 0: none, at most 1e6). All three stay set until changed; a solve uses
 * 0, -1, 0. */
int ithaca_gpu_cg_set_wait_test(ithaca_gpu_cg* cg, long long barrier_polls, int drop_cta, int delay_ns);

typedef struct {
  double tol;          /* IterativeSolverTolerance (default 1e-9); stop when ||r||^2 < tol^2 ||b||^2 */
  int max_iter;        /* NekLinSysMaxIterations (default 5000)                                      */
  int mode;            /* ITHACA_GPU_SOLVE_*                                                         */
  double inner_tol;    /* mixed mode: relative reduction asked of each inner FP32 solve (default 1e-2) */
  int max_outer;       /* mixed mode: maximum refinement steps (default 50)                          */
  int check_every;     /* iterations per graph launch between host checks (default 16; 8 batched)    */
} ithaca_gpu_cg_opts;

typedef struct {
  int iterations;         /* total CG iterations (inner iterations in mixed mode) */
  int outer_iterations;   /* refinement steps (0 in FP64 mode)                    */
  double rel_residual;    /* ||b - A x||_2 / ||b||_2 over non-Dirichlet dofs, FP64  */
  double eps;             /* last reference-style residual r.r of the FP64 recurrence */
  double rhs_magnitude;   /* ||b||^2 with the 1e-6 -> 1 floor of NekLinSysIter.cpp:142 */
} ithaca_gpu_cg_result;

void ithaca_gpu_cg_default_opts(ithaca_gpu_cg_opts* opts);

/* Solves A(lambda) x = rhs for the non-Dirichlet global dofs (rhs, x: nglobal
 * doubles; x[0..ndir) is left untouched, the solve starts from x = 0 elsewhere as
 * the reference does). Returns ITHACA_GPU_ERR_NOT_CONVERGED past max_iter. */
int ithaca_gpu_cg_solve(ithaca_gpu_cg* cg, double lambda, const double* rhs, double* x,
                        const ithaca_gpu_cg_opts* opts, ithaca_gpu_cg_result* res, int on_device);

/* Global operator y = Assemble(Helmholtz(GlobalToLocal(x))) in FP64 (nglobal entries;
 * Dirichlet entries of x are used as given). GlobalLinSysIterativeFull::v_DoMatrixMultiply. */
int ithaca_gpu_cg_apply(ithaca_gpu_cg* cg, double lambda, const double* x, double* y, int on_device);
/* AssemblyMapCG::Assemble (MultiRegions/AssemblyMap/AssemblyMapCG.cpp:2885-2910):
 * global[g] = sum of sign * local over the local copies of g (nglobal entries). */
int ithaca_gpu_cg_assemble(ithaca_gpu_cg* cg, const double* local, double* global, int on_device);
/* AssemblyMapCG::GlobalToLocal (:2853-2876): local = sign * global[map] (E*n^d entries). */
int ithaca_gpu_cg_global_to_local(ithaca_gpu_cg* cg, const double* global, double* local, int on_device);
/* Assembled Jacobi diagonal over the non-Dirichlet dofs (nglobal - ndir entries). */
int ithaca_gpu_cg_diagonal(ithaca_gpu_cg* cg, double lambda, double* diag, int on_device);

/* ContField::v_HelmSolve (MultiRegions/ContField.cpp:878-945) for homogeneous
 * Dirichlet data: forcing f at quadrature points (E*Q^d) -> solution in local
 * coefficient space (E*n^d): rhs = Assemble(-IProductWRTBase(f)), CG, GlobalToLocal. */
int ithaca_gpu_helmsolve(ithaca_gpu_cg* cg, double lambda, const double* forcing, double* out_local,
                         const ithaca_gpu_cg_opts* opts, ithaca_gpu_cg_result* res, int on_device);
/* The same with Dirichlet data: dirichlet holds the ndir global coefficients of the
 * Dirichlet dofs (numbered first), e.g. the boundary-constrained projections of the
 * boundary condition that the reference's boundary expansions hold. The solve lifts
 * them (rhs_F -= (A x_D)_F, ContField.cpp:908-930) and they are the Dirichlet entries
 * of the result; dirichlet == NULL is homogeneous data. */
int ithaca_gpu_helmsolve_dirichlet(ithaca_gpu_cg* cg, double lambda, const double* forcing, const double* dirichlet,
                                   double* out_local, const ithaca_gpu_cg_opts* opts, ithaca_gpu_cg_result* res,
                                   int on_device);

/* ---- the ROM solvers' HelmSolve callers ----
 * VelocityCorrectionScheme_ROM::v_SolveViscous
 * (solvers/IncNavierStokesSolver/EquationSystems/VelocityCorrectionScheme_ROM.cpp:1538-1567):
 * for each of the nfields velocity fields (which share one expansion, so one system `cg`),
 * lambda = 1 / aii_dt / diff_coeff[i], HelmSolve of forcing[i] (E*Q^d values at the
 * quadrature points) with the field's Dirichlet data dirichlet[i] (ndir global coefficients,
 * NULL for homogeneous data; dirichlet == NULL for all fields homogeneous) into coeffs[i]
 * (E*n^d local coefficients), then BwdTrans into phys[i] (E*Q^d; phys == NULL or phys[i] ==
 * NULL skips it). res (NULL or nfields entries) gets each solve's result. The fields are
 * solved in order on the context stream; the first failing one stops the call and its status
 * is returned. Spectral vanishing viscosity (AppendSVVFactors) is not supported. */
int ithaca_gpu_vcs_solve_viscous(ithaca_gpu_cg* cg, int nfields, const double* const* forcing,
                                 const double* const* dirichlet, double aii_dt, const double* diff_coeff,
                                 double* const* coeffs, double* const* phys, const ithaca_gpu_cg_opts* opts,
                                 ithaca_gpu_cg_result* res, int on_device);
/* VelocityCorrectionScheme_ROM::v_SolvePressure (:1522-1534): the pressure Poisson equation,
 * HelmSolve with lambda = 0, forcing at the quadrature points -> local coefficients of the
 * pressure expansion's system. The system needs Dirichlet dofs (ITHACA_GPU_ERR_ARG
 * otherwise: without them the Poisson operator is singular). */
int ithaca_gpu_vcs_solve_pressure(ithaca_gpu_cg* cg, const double* forcing, const double* dirichlet,
                                  double* coeffs, const ithaca_gpu_cg_opts* opts, ithaca_gpu_cg_result* res,
                                  int on_device);

/* ---- batched parametric solves ----
 * Many independent C0 Helmholtz systems (own mesh, order, lambda, rhs; homogeneous
 * Dirichlet data) solved together: the parameter loop that produces the snapshots of
 * the ITHACA offline phase (CoupledLinearNS_ROM.cpp:1208-1283, one FOM HelmSolve per
 * parameter) as one graph-captured batch. Every solve follows the reference CG
 * recurrence with its own scalars. Host arrays, layouts as ithaca_gpu_cg_create. */
/* ---- statically condensed global system (GlobalSysSoln = IterativeStaticCond) ----
 * GlobalLinSysIterativeStaticCond (MultiRegions/GlobalLinSysIterativeStaticCond.cpp) with
 * GlobalLinSysStaticCond::v_Solve (GlobalLinSysStaticCond.cpp:104-238): per element the
 * Helmholtz matrix is condensed onto its boundary modes (vertex, edge, face: any modal
 * index below 2), the assembled Schur-complement system is solved by the reference CG
 * recurrence with its diagonal as Jacobi preconditioner
 * (PreconditionerDiagonal::StaticCondDiagonalPreconditionerSum, :164-189), and the
 * interior modes follow element by element. Same map arguments as ithaca_gpu_cg_create
 * (the interior modes of an element must be private to it; Dirichlet dofs are boundary
 * modes); the element blocks are built on the first solve with a given lambda, from the
 * operator's own element apply (FP64, deformed collections). */
typedef struct ithaca_gpu_sc ithaca_gpu_sc;
int ithaca_gpu_sc_create(ithaca_gpu_op* op, const int* l2g, const double* sign, int nglobal, int ndir,
                         ithaca_gpu_sc** out);
int ithaca_gpu_sc_destroy(ithaca_gpu_sc* sc);
/* Sizes: global boundary dofs, the Dirichlet ones among them, boundary and interior modes
 * per element. */
int ithaca_gpu_sc_info(ithaca_gpu_sc* sc, int* nbnd_global, int* ndir_bnd, int* nbnd_local, int* nint_local);
/* v_Solve on local (element) arrays of E*n^d entries: loc_rhs the element forcing
 * (e.g. -IProductWRTBase(f)), loc_inout the boundary values already known (Dirichlet
 * data, initial guess) in, the solution out. opts->mode must be ITHACA_GPU_SOLVE_FP64.
 * The CG's rhs magnitude is that of the assembled boundary forcing, smoothed 0.9 / 0.1
 * with the previous solve's as v_PreSolve does (:431-460); res->rel_residual is the
 * boundary system's sqrt(eps / rhs magnitude). */
int ithaca_gpu_sc_solve(ithaca_gpu_sc* sc, double lambda, const double* loc_rhs, double* loc_inout,
                        const ithaca_gpu_cg_opts* opts, ithaca_gpu_cg_result* res, int on_device);

typedef struct ithaca_gpu_batch ithaca_gpu_batch;
typedef struct {
  int nmodes, npoints, nelmt;
  const double* jac;   /* E*Q^d   (deformed layout) */
  const double* df;    /* d*d*E*Q^d                 */
  int deformed;        /* must be 1                 */
  const int* l2g;      /* E*n^d local -> global ids, Dirichlet ids first */
  const double* sign;  /* E*n^d, +1 / -1            */
  int nglobal, ndir;
  double lambda;
  const double* rhs;   /* nglobal assembled right-hand side */
} ithaca_gpu_solve_desc;
int ithaca_gpu_batch_create(ithaca_gpu_ctx* ctx, int shape, int nsolve, const ithaca_gpu_solve_desc* descs,
                            ithaca_gpu_batch** batch);
int ithaca_gpu_batch_destroy(ithaca_gpu_batch* batch);
/* Solves every system (opts->mode FP64 or mixed). x: nsolve host pointers of nglobal
 * doubles each (or NULL); iterations / outer / rel_res: nsolve entries (or NULL);
 * elapsed_ms: device time of the whole batch (CUDA events on the context stream). */
int ithaca_gpu_batch_solve(ithaca_gpu_batch* batch, const ithaca_gpu_cg_opts* opts, double* const* x,
                           int* iterations, int* outer, double* rel_res, double* elapsed_ms);
/* Launch structure of ithaca_gpu_batch_solve (the snapshot loop of
 * CoupledLinearNS_ROM.cpp:1208-1283 has no counterpart: it solves one system at a time).
 * on = 1 (default): the whole solve is one CUDA graph launch whose loops are conditional
 * graph nodes (device-side WHILE over chunks of iterations, and in mixed mode over the
 * refinement steps), so the host waits once. on = 0: the host launches a captured chunk
 * of iterations, reads the scalars and decides whether to launch again. Both run the same
 * kernels in the same order and give the same results. */
int ithaca_gpu_batch_set_one_launch(ithaca_gpu_batch* batch, int on);
/* Tile shapes per polynomial order, chosen by timing as CollectionOptimisation::
 * SetWithTimings chooses implementation types (Collections/CollectionOptimisation.cpp:
 * 321-469): for each order group and precision the gathered element apply is timed `reps`
 * times with each element-kernel variant (0 shared-memory kernel; 1 / 2 register-pencil
 * kernel with 256 / 128 threads per CTA) on the group's own data, and the fastest is used
 * from then on. Outputs (any may be NULL): the number of groups, each group's modes, the
 * chosen FP32 and FP64 variants, and the times ms[(group * 2 + precision) * 3 + variant]
 * (precision 0 FP32, 1 FP64; at most 11 groups). */
int ithaca_gpu_batch_autotune(ithaca_gpu_batch* batch, int reps, int* ngroups, int* nmodes, int* variant32,
                              int* variant64, double* ms);

/* ---- variable coefficient and adjoint gradient ----
 * Isotropic diffusion coefficient kappa at the quadrature points (E*Q^d) of a deformed
 * collection: the solver's operator becomes lambda M + L_kappa, the reference's
 * LaplacianMatrixOp_MatFree with eVarCoeffD00 = eVarCoeffD11 [= D22] = kappa
 * (StdRegions/StdExpansion.cpp:664-717). kappa == NULL restores kappa = 1. */
int ithaca_gpu_cg_set_varcoeff(ithaca_gpu_cg* cg, const double* kappa, int on_device);
/* Anisotropic coefficient: the symmetric tensor K at the quadrature points of a deformed
 * collection, d(d+1)/2 arrays of E*Q^d values in the order of the reference's
 * eVarCoeffD00, D01, (D02,) D11, (D12, D22) (StdRegions/StdExpansion.cpp:664-717, where
 * LaplacianMatrixOp_MatFree(k1, k2) scales d u / d x_k2 by the (k1, k2) component before
 * IProductWRTDerivBase(k1)). The solver's operator becomes lambda M + sum_{k1,k2}
 * (d phi / d x_k1, K_k1k2 d u / d x_k2): the metric of each point is rebuilt as
 * J w (d xi / d x)^T K (d xi / d x). ithaca_gpu_cg_set_varcoeff(cg, NULL, 1) restores K = I;
 * ithaca_gpu_kappa_gradient is defined for the isotropic coefficient only. */
int ithaca_gpu_cg_set_varcoeff_tensor(ithaca_gpu_cg* cg, const double* K, int on_device);
/* Misfit J = sum_q Jw_q (u(x_q) - u_target_q)^2 of the global vector x (Dirichlet
 * values taken as zero) and, if dJdx != NULL, its gradient w.r.t. x (nglobal entries,
 * zero on Dirichlet dofs). No reference counterpart (the reference has no adjoint). */
int ithaca_gpu_misfit(ithaca_gpu_cg* cg, const double* x, const double* u_target, double* J, double* dJdx,
                      int on_device);
/* dJ/dkappa_q = -Jw_q grad psi(x_q) . grad u(x_q) for the forward solution x and the
 * adjoint solution psi of A(kappa) psi = dJ/dx (E*Q^d entries). No reference counterpart. */
int ithaca_gpu_kappa_gradient(ithaca_gpu_cg* cg, const double* x, const double* psi, double* grad, int on_device);

/* ---- POD reduced basis (solvers/IncNavierStokesSolver/EquationSystems/CoupledLinearNS_ROM.cpp) ----
 * Column-major FP64 matrices throughout. */

/* Gram matrix C = S^T S (ns x ns) of the snapshot matrix S (N x ns). */
int ithaca_gpu_pod_gram(ithaca_gpu_ctx* ctx, int N, int ns, const double* S, double* C, int on_device);
/* ROM_offline_phase (:3916-4001) by the method of snapshots: the leading `nmodes`
 * orthonormal POD modes V (N x nmodes) and all ns singular values sigma (descending;
 * sigma is a host array whatever on_device says, S and V follow on_device).
 * *nmodes_out < nmodes when trailing modes are not resolved in FP64. */
int ithaca_gpu_pod_offline(ithaca_gpu_ctx* ctx, int N, int ns, const double* S, int nmodes, double* V,
                           double* sigma, int* nmodes_out, int on_device);
/* Reduced-basis size from the cumulative singular-value fraction (:3935-3944). Host only. */
int ithaca_gpu_pod_rb_size(int ns, const double* sigma, double pod_tolerance, int* size);
/* Affine reduced operators A_L = V^T L V, A_M = V^T M V (nmodes x nmodes) for the
 * Helmholtz system of `cg`; V holds nmodes columns over the nglobal - ndir free dofs
 * (gen_reference_matrices :3904-3911, gen_affine_mat_proj :4694-4703). */
int ithaca_gpu_pod_project(ithaca_gpu_cg* cg, int nmodes, const double* V, double* A_L, double* A_M,
                           int on_device);
/* ROM_online_phase (:4003-4100): x_r[k] solves (A_L + lambdas[k] A_M) x = f_r for each of
 * nlambda parameters (r <= 64), FP64 LU with partial pivoting; x_r is r x nlambda. */
int ithaca_gpu_pod_online(ithaca_gpu_ctx* ctx, int r, const double* A_L, const double* A_M, const double* f_r,
                          int nlambda, const double* lambdas, double* x_r, int on_device);
/* Reconstruction u = V x_r (:4054), N x nsol. */
int ithaca_gpu_pod_reconstruct(ithaca_gpu_ctx* ctx, int N, int r, const double* V, int nsol, const double* x_r,
                               double* u, int on_device);

/* Allocation-free Gram matrix C = S^T S (no counterpart in the reference). For callers
 * that cannot allocate device memory where they need it: a host application that
 * reserves its device memory up front in its own pool and forbids allocation in its
 * solve loop, or a time-stepping loop that must not stall on the device-wide
 * synchronisation that cudaFree implies.
 * S (N x ns, column-major) and C (ns x ns) are device pointers owned by the caller; work
 * is queued on `stream` (a cudaStream_t, NULL for the legacy default stream) and not
 * waited for. The split-K scratch is a fixed 2 MiB device array in the library, held on
 * every device that loads it until the process exits, so ns <= 128 (larger ns returns
 * ITHACA_GPU_ERR_ARG). Nothing in the array needs to start at zero: every partial sum is
 * written before it is read. The first call on a device looks that array up
 * (cudaGetSymbolAddress) and should come before any stream capture; the address is kept
 * for the life of the process, so calls after a cudaDeviceReset of that device are not
 * supported. All calls share the array: calls whose work overlaps on the GPU race and
 * must be serialised by the caller. A CUDA error already pending from earlier work is
 * reported (ITHACA_GPU_ERR_CUDA) and left pending, and nothing is queued. It calls no
 * cudaMalloc or cudaFree and needs no context. */
int ithaca_gpu_pod_gram_noalloc(int N, int ns, const double* S, double* C, void* stream);

/* Measurement hook (no reference counterpart): the device's FP64 FMA, FP64 tensor-core
 * (mma.sync m8n8k4 f64) and FP32 FMA throughput in TFLOP/s, each from one timed launch of
 * independent FMA / MMA chains on every SM (after a warm-up launch) on the context
 * stream; the compute roofs of the FP64 and FP32 element operators. */
int ithaca_gpu_measure_pipe_peaks(ithaca_gpu_ctx* ctx, double* fp64_fma_tflops, double* fp64_mma_tflops,
                                  double* fp32_fma_tflops);

/* Measurement hook (no reference counterpart): runs the gather + element-Helmholtz
 * kernel that ithaca_gpu_cg_solve launches for `mode` `reps` times on the context
 * stream and returns its average device time in ms (CUDA events) and the algorithmic
 * bytes of one launch: per element, the signed index (4 B) plus input and output per
 * local dof, and J w with the symmetric metric per quadrature point, at the mode's
 * element size (the scattered output's per-dof output codes are not counted). */
int ithaca_gpu_cg_profile_apply(ithaca_gpu_cg* cg, int mode, double lambda, int reps, double* avg_ms,
                                double* bytes_per_launch);

#ifdef __cplusplus
}
#endif

#endif /* ITHACA_GPU_H */
