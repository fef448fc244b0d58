/* pxg.h — C ABI of the GB300 finite-element assembly engine (proxpde_gb300).
 *
 * The engine replaces proxpde's element loop: Builder::buildLhs / buildRhs /
 * closeMatrix (include/builder.hpp:31-154, 279-371) driving AssemblyStiffness(FE),
 * AssemblyScalarMass and AssemblyRhsAnalytic / AssemblyS2SProjection over CurFE
 * geometry (include/curfe.hpp:50-103) and Gauss quadrature, on P1/P2 tetrahedra and
 * Q1/Q2 hexahedra.  Everything here is plain C: pointers, sizes and status codes.
 *
 * Conventions
 *  - Every call returns a pxg_status; pxg_last_error() gives a message for the last
 *    failing call on a context.  The reference aborts instead (assert, std::abort,
 *    std::exit(2): include/def.hpp:273-274); here nothing aborts the process.
 *  - `mem` arguments say where a buffer lives: PXG_MEM_HOST (the engine copies it
 *    through its own staging) or PXG_MEM_DEVICE (a device pointer on the context's
 *    GPU).  Assembly outputs must be device buffers unless stated otherwise.
 *  - `stream` is a cudaStream_t passed as void* (NULL = the legacy default stream).
 *    Calls are stream-ordered; host-memory variants synchronise the stream.
 *  - One context per host thread (the reference keeps a mutable CurFE inside its
 *    FESpace, include/fespace.hpp:190, so it is not thread-safe either).
 *  - Index types follow the reference: DOF and vertex ids are uint32
 *    (include/def.hpp:60-66), CSR indices are int32 like Eigen::SparseMatrix's default
 *    StorageIndex (include/sparse_matrix.hpp:38-39).
 */
#ifndef PXG_H
#define PXG_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum pxg_status
{
  PXG_OK = 0,
  PXG_ERR_INVALID_ARG = 1,   /* bad size, null pointer, out-of-range id, wrong order of calls */
  PXG_ERR_OOM = 2,           /* device or pinned-host allocation failed */
  PXG_ERR_CUDA = 3,          /* a CUDA runtime call failed (message in pxg_last_error) */
  PXG_ERR_TIMEOUT = 4,       /* a bounded device wait ran out (persistent kernels) */
  PXG_ERR_NOT_CONVERGED = 5, /* an iterative solve stopped at its iteration limit */
  PXG_ERR_UNSUPPORTED = 6,   /* element type / operator combination not provided */
  PXG_ERR_NO_DEVICE = 7,     /* no CUDA device, or the requested one is absent */
  PXG_ERR_NUMERIC = 8        /* a device procedure did not finish (the element colouring) */
} pxg_status;

/* Element types: LagrangeFE<Tetrahedron,1|2>, LagrangeFE<Hexahedron,1|2> with their
 * RecommendedQR (include/fe.hpp:96-131): Tet4, Tet11, Hex8 (2x2x2), Hex27 (3x3x3). */
typedef enum pxg_elem_type
{
  PXG_P1TET = 0,
  PXG_P2TET = 1,
  PXG_Q1HEX = 2,
  PXG_Q2HEX = 3
} pxg_elem_type;

typedef enum pxg_mem
{
  PXG_MEM_HOST = 0,
  PXG_MEM_DEVICE = 1
} pxg_mem;

/* Analytic functions evaluated on the device at the quadrature points.  The
 * reference passes a host std::function (include/assembly_rhs.hpp:50-59), which
 * cannot run on a GPU; callers pick one of these by id instead. */
typedef enum pxg_fn
{
  PXG_FN_CONST = 0,         /* f = c */
  PXG_FN_SIN3 = 1,          /* f = c sin(pi x) sin(pi y) sin(pi z) */
  PXG_FN_POISSON_RHS = 2,   /* f = c 2.5 pi^2 sin(pi x/2) sin(3 pi y/2)  (test/poisson3d*.cpp:27-33) */
  PXG_FN_POISSON_EXACT = 3, /* f = c sin(pi x/2) sin(3 pi y/2)            (test/poisson3d*.cpp:35-40) */
  PXG_FN_COORD_X = 4,       /* f = c x  (coordinates, e.g. to locate DOFs on a plane) */
  PXG_FN_COORD_Y = 5,       /* f = c y */
  PXG_FN_COORD_Z = 6        /* f = c z */
} pxg_fn;

typedef struct pxg_ctx pxg_ctx;

/* One matrix assembled by a buildLhs call (include/builder.hpp:31-154): the sum of a
 * stiffness term and a mass term.
 *   stiffness 0: none
 *             1: AssemblyStiffness(stiff_coef)          (include/assembly_lhs.hpp:36-75)
 *             2: AssemblyStiffnessFE with the per-element (P0 FEVar) coefficient set by
 *                pxg_set_coef, times stiff_coef         (include/assembly_lhs.hpp:77-113)
 *   mass      0: none, 1: AssemblyScalarMass(mass_coef) (include/assembly_lhs.hpp:191-231)
 *             2: AssemblyMassFE with the per-element coefficient set by pxg_set_coef,
 *                times mass_coef                        (include/assembly_lhs.hpp:234-277)
 *   apply_bc  condense with the context's essential BCs (include/builder.hpp:76-124);
 *             the lifted load C(-Ke h) and h at constrained DOFs go into b as the
 *             reference's buildLhs does (builder.hpp:102, 119, 137). */
typedef struct pxg_lhs_op
{
  int32_t stiffness;
  double stiff_coef;
  int32_t mass;
  double mass_coef;
  int32_t apply_bc;
} pxg_lhs_op;

/* One load vector term of a buildRhs call (include/builder.hpp:279-364).
 *   kind 0: none
 *        1: AssemblyRhsAnalytic with function `fn` scaled by `coef`
 *           (include/assembly_rhs.hpp:34-91), f evaluated at CurFE::qpoint
 *        2: AssemblyS2SProjection(coef, field) of a DOF vector on the same space
 *           (include/assembly_rhs.hpp:93-163); `field` is a device pointer (ndof)
 *        3: AssemblyRhsAnalytic with any function, evaluated by the caller at the
 *           quadrature points that pxg_get_qpoints returns: `field` is a device
 *           pointer to nelem x nq values f(qpoint) (element-major), scaled by `coef`
 *           (the reference's host std::function, assembly_rhs.hpp:50-59, cannot run on
 *           the device, so the caller evaluates it there)
 *   apply_bc  zero constrained rows (C*Fe, builder.hpp:319-347). */
typedef struct pxg_rhs_op
{
  int32_t kind;
  int32_t fn;
  double coef;
  const double * field;
  int32_t apply_bc;
} pxg_rhs_op;

/* pxg_assemble flags */
#define PXG_ACCUMULATE 1u /* add into vals0/vals1/b instead of overwriting them */

/* Scatter of the element contributions into the CSR values. */
typedef enum pxg_scatter
{
  PXG_SCATTER_REDUCE = 0, /* FP64 reductions in element order (default) */
  PXG_SCATTER_COLOUR = 1  /* one launch per element colour class: every CSR entry gets at
                             most one contribution per launch, so the sums are formed in a
                             fixed order and the matrices are bitwise reproducible */
} pxg_scatter;

/* Outcome of pxg_autotune: the chosen configuration and every candidate's time. */
typedef struct pxg_tune_report
{
  int threads;  /* threads per block of the element kernel (8 per element for Q1 hexahedra) */
  int scatter;  /* pxg_scatter */
  int ncolours; /* colour classes of the colouring (0 if it was not built) */
  int ncand;
  int cand_threads[16];
  int cand_scatter[16];
  double cand_ms[16]; /* mean time of one pxg_assemble call with the tuned operators */
} pxg_tune_report;

/* ----------------------------------------------------------------- context */
pxg_status pxg_create(pxg_ctx ** ctx, int device);
pxg_status pxg_destroy(pxg_ctx * ctx);
const char * pxg_last_error(const pxg_ctx * ctx);
const char * pxg_status_string(pxg_status s);
/* Version of this ABI (major * 10000 + minor * 100 + patch). */
int pxg_version(void);

/* ------------------------------------------------------------ mesh input
 * Mesh<Elem>{pointList, elementList} (include/mesh.hpp:74-100): node coordinates
 * xyz[nnodes][3] and vertex connectivity conn[nelem][nv] (nv = 4 tets, 8 hexes) in
 * the reference's local vertex order (include/geo.hpp:508-760).  Element ids are the
 * row indices.  Replaces any previous mesh (and drops the DOF map and pattern). */
pxg_status pxg_set_mesh(pxg_ctx * ctx, int elem_type, const double * xyz, int64_t nnodes,
                        const uint32_t * conn, int64_t nelem, int mem);
/* Overwrite the node coordinates of the current mesh (same connectivity). */
pxg_status pxg_set_coords(pxg_ctx * ctx, const double * xyz, int mem, void * stream);

/* --------------------------------------------------------------- DOF map
 * DOF::setupElemMap first-touch numbering (include/dof.hpp:111-329), computed on the
 * device: a DOF gets the next id the first time the element loop meets its entity
 * (points, then edges, then faces, then the element).  elemMap is nelem x ndofs/elem,
 * row-major, like DOF::elemMap (a Table, include/def.hpp:111-127). */
pxg_status pxg_build_dofmap(pxg_ctx * ctx, int64_t * ndof);
/* Use a caller-provided DOF map instead (e.g. proxpde's own dof.elemMap). */
pxg_status pxg_set_dofmap(pxg_ctx * ctx, const uint32_t * elem_map, int64_t ndof, int mem);
pxg_status pxg_get_dofmap(pxg_ctx * ctx, uint32_t * elem_map, int mem);

/* --------------------------------------------------------- CSR pattern
 * The structural pattern of every (idI, idJ) pair the element loop emits
 * (builder.hpp:131-152), sorted by row then column: the pattern Eigen's
 * setFromTriplets builds (builder.hpp:368) before prune.  Built on the device once
 * per mesh; it also builds the per-element scatter map used by pxg_assemble. */
pxg_status pxg_build_pattern(pxg_ctx * ctx, int64_t * nnz);
pxg_status pxg_get_pattern(pxg_ctx * ctx, int32_t * row_ptr, int32_t * col_idx, int mem);
/* Device pointers of the context-owned structural pattern (valid until the mesh
 * changes). */
pxg_status pxg_pattern_device(pxg_ctx * ctx, const int32_t ** row_ptr, const int32_t ** col_idx);

/* ----------------------------------------------------- coefficients, BCs
 * Per-element coefficient k_e (a P0 FEVar, include/var.hpp:56-127), nelem values. */
pxg_status pxg_set_coef(pxg_ctx * ctx, const double * k_e, int mem, void * stream);
/* Essential BCs: BCEss (include/bc.hpp:32-306) merged into one constrained-DOF list
 * with values; `diag` is BCEss::diag (1.0 in the reference, bc.hpp:301).  n = 0
 * clears the BCs.  A DOF listed twice keeps the last value, as the reference's
 * builder keeps the value of the last BC that constrains it (builder.hpp:85-100). */
pxg_status pxg_set_bc(pxg_ctx * ctx, const uint32_t * dofs, const double * vals, int64_t n,
                      double diag, int mem);

/* ------------------------------------------------- boundary facets and BCs
 * Device versions of proxpde's buildFacets / markFacetsCube (include/mesh.hpp:226-498)
 * and BCEss::setupDofMap (include/bc.hpp:252-295).  Markers use proxpde's side
 * numbering (mesh.hpp:178-188). */
typedef enum pxg_side
{
  PXG_SIDE_NONE = 0,
  PXG_SIDE_BOTTOM = 1, /* y = min */
  PXG_SIDE_RIGHT = 2,  /* x = max */
  PXG_SIDE_TOP = 3,    /* y = max */
  PXG_SIDE_LEFT = 4,   /* x = min */
  PXG_SIDE_BACK = 5,   /* z = min */
  PXG_SIDE_FRONT = 6   /* z = max */
} pxg_side;

/* Boundary facets of the mesh (faces of exactly one element), kept on the device in
 * the order of their sorted vertex ids; their count. */
pxg_status pxg_build_facets(pxg_ctx * ctx, int64_t * nfacets);
/* Host copies: faces[k] = element * (4 or 6) + local face (tetrahedron face i is
 * opposite vertex i; hexahedron faces are {0,3,2,1}, {3,0,4,7}, {0,1,5,4}, {1,2,6,5},
 * {2,3,7,6}, {4,5,6,7}), markers[k]; either pointer may be NULL. */
pxg_status pxg_get_facets(pxg_ctx * ctx, uint32_t * faces, int32_t * markers);
/* Markers given by the caller, one per facet in pxg_get_facets order (host array). */
pxg_status pxg_set_facet_markers(pxg_ctx * ctx, const int32_t * markers);
/* markFacetsCube: builds the facets if needed and marks those on the planes of the box
 * [origin, origin + length] (first match in the order BOTTOM, RIGHT, TOP, LEFT, BACK,
 * FRONT; tolerance 1e-6 of the length). */
pxg_status pxg_mark_facets_box(pxg_ctx * ctx, const double * origin, const double * length);
/* Dirichlet conditions from markers (replaces any earlier pxg_set_bc): condition k
 * constrains the DOFs on the facets with markers[k] to coefs[k] * fns[k](DOF point);
 * later conditions win on shared DOFs.  diag as in pxg_set_bc. */
pxg_status pxg_set_bc_markers(pxg_ctx * ctx, const int32_t * markers, const int32_t * fns,
                              const double * coefs, int nbc, double diag);

/* ------------------------------------------ systems of spaces on one mesh
 * Vector spaces and mixed (coupled) problems: FESpace<..., dim> with its offset
 * (include/fespace.hpp:15-60), Builder::buildLhs on vector spaces and
 * Builder::buildCoupling (include/builder.hpp:31-277).  The spaces are contexts with
 * DOF maps on the same mesh; space s gets dims[s] components in BLOCK ordering
 * (component d of DOF k is k + d * ndof_s) and the offset of the spaces before it. */
typedef struct pxg_sys pxg_sys;

typedef enum pxg_op_kind
{
  PXG_OP_STIFFNESS = 1,        /* AssemblyStiffness on each component (assembly_lhs.hpp:52-65) */
  PXG_OP_TENSOR_STIFFNESS = 2, /* AssemblyTensorStiffness (assembly_lhs.hpp:116-161) */
  PXG_OP_MASS = 3,             /* AssemblyMass on each component (assembly_lhs.hpp:347-365) */
  PXG_OP_GRAD = 4,             /* AssemblyGrad: rows vector space, columns scalar space (assembly_coupling.hpp:42-86) */
  PXG_OP_DIV = 5               /* AssemblyDiv: rows scalar space, columns vector space (assembly_coupling.hpp:89-132) */
} pxg_op_kind;

/* Build the system and its pattern (all DOF pairs of each element over all spaces; the
 * blocks the reference leaves empty are structural zeros that the prune removes).
 * qr_types[s]: element type whose quadrature rule space s uses (NULL: its own), e.g.
 * the pressure space of a Taylor-Hood pair on the velocity's rule. */
pxg_status pxg_sys_create(pxg_sys ** sys, pxg_ctx * const * spaces, const int * dims, const int * qr_types,
                          int nspaces, int64_t * ntot, int64_t * nnz);
pxg_status pxg_sys_destroy(pxg_sys * sys);
pxg_status pxg_sys_get_pattern(pxg_sys * sys, int32_t * row_ptr, int32_t * col_idx);
pxg_status pxg_sys_pattern_device(pxg_sys * sys, const int32_t ** row_ptr, const int32_t ** col_idx);
/* Builder::closeMatrix on the system's pattern (pxg_close_matrix for a system): the
 * pruned CSR of vals (row_ptr[ntot+1], col_idx and vals_out with capacity nnz, device
 * pointers) and its entry count; scratch is allocated on the first space's device. */
pxg_status pxg_sys_close_matrix(pxg_sys * sys, const double * vals, int32_t * row_ptr, int32_t * col_idx,
                                double * vals_out, int64_t * nnz_out, void * stream);
/* Dirichlet data of one space over its component DOFs (host arrays; the last value wins). */
pxg_status pxg_sys_set_bc(pxg_sys * sys, int space, const uint32_t * dofs, const double * vals, int64_t n,
                          double diag);
/* One Builder call: row == col is buildLhs (constrained diagonal = diag, b = h there),
 * row != col buildCoupling (no diagonal); vals (nnz) and b (ntot) are device arrays. */
pxg_status pxg_sys_assemble(pxg_sys * sys, int row, int col, const int * kinds, const double * coefs, int nops,
                            double * vals, double * b, unsigned flags, void * stream);

/* --------------------------------------------------------------- assembly
 * One fused pass over the elements: up to two matrices (vals0/vals1, each nnz long on
 * the structural pattern, device memory) and one load vector b (ndof, device).
 * Any of op0/op1/rhs may be NULL (and then its output is untouched).  b receives the
 * rhs term plus the BC lifts of the lhs ops that apply BCs. */
pxg_status pxg_assemble(pxg_ctx * ctx, const pxg_lhs_op * op0, double * vals0,
                        const pxg_lhs_op * op1, double * vals1, const pxg_rhs_op * rhs,
                        double * b, unsigned flags, void * stream);

/* Builder::closeMatrix's prune(1., 1e-16) (builder.hpp:369): count the entries of a
 * structural-pattern value array with |v| <= 1e-16.  0 means the structural pattern
 * and `vals` already are the closed matrix. */
pxg_status pxg_prune_count(pxg_ctx * ctx, const double * vals, int64_t * pruned, void * stream);
/* The same count, asynchronous: stream-ordered, it leaves the count in *pruned_dev
 * (device memory, one int64) and returns without waiting, so that assembly, the check
 * and the read-back of several steps can overlap. */
pxg_status pxg_prune_count_device(pxg_ctx * ctx, const double * vals, int64_t * pruned_dev, void * stream);

/* Scatter strategy and threads per block of the element kernels (threads = 0: the
 * kernel's default).  Valid thread counts: 64, 128, 256 (P1/P2 tetrahedra), 128, 256,
 * 512 (Q1 hexahedra), 128 (Q2 hexahedra).  PXG_SCATTER_COLOUR builds the element
 * colouring on the first use (not during a stream capture). */
pxg_status pxg_set_scatter(pxg_ctx * ctx, int scatter, int threads);
/* Arithmetic of the element kernels.  The reference computes geometry, local matrices
 * and sums in double (FVec/FMat, include/def.hpp:157-160); PXG_ARITH_FP64, the
 * default, does the same: every value is formed by IEEE binary64 operations.
 * PXG_ARITH_DFL is an opt-in alternative with a narrower significand: the geometry and
 * the local matrices run as unevaluated pairs of floats (about 48 bits) on the FP32
 * pipes, and only the coordinate differences, the final sums and the reductions into
 * the outputs stay FP64.  Changing it resets the threads per block to the default. */
typedef enum pxg_arith
{
  PXG_ARITH_FP64 = 0,
  PXG_ARITH_DFL = 1
} pxg_arith;
pxg_status pxg_set_arithmetic(pxg_ctx * ctx, int arith);
/* Element colouring of the colour-ordered scatter (built if needed): the number of
 * colour classes, and optionally the elements in colour order (nelem entries) and the
 * class offsets (ncolours + 1 entries), host arrays. */
pxg_status pxg_colouring(pxg_ctx * ctx, int * ncolours, uint32_t * order, int64_t * offsets);
/* Autotuner: times every (threads, scatter) candidate of this context's element type on
 * its own mesh with the given operators (outputs into scratch arrays), keeps the fastest
 * with pxg_set_scatter and reports the candidates.  Call it outside stream capture. */
pxg_status pxg_autotune(pxg_ctx * ctx, const pxg_lhs_op * op0, const pxg_lhs_op * op1,
                        const pxg_rhs_op * rhs, pxg_tune_report * report);
/* Compact: write the pruned CSR (row_ptr[ndof+1], col_idx, vals_out; device
 * pointers, capacity nnz) and its entry count. */
pxg_status pxg_close_matrix(pxg_ctx * ctx, const double * vals, int32_t * row_ptr,
                            int32_t * col_idx, double * vals_out, int64_t * nnz_out,
                            void * stream);

/* CurFE::qpoint (include/curfe.hpp:80) of every element and quadrature point of the
 * element type's rule: qpts[(e * nq + q) * 3 + d], nq = 4 / 11 / 8 / 27 for P1 / P2 /
 * Q1 / Q2, the point origin + J(xi_q) xi_q with origin the first vertex (tetrahedra) or
 * the vertex average (hexahedra, include/geo.hpp:721-728).  mem: where qpts lives
 * (host copies synchronise the stream).  The points rhs kind 3 expects its values at. */
pxg_status pxg_get_qpoints(pxg_ctx * ctx, double * qpts, int mem, void * stream);

/* Lagrange interpolation of an analytic function at the DOF points
 * (interpolateAnalyticFunction, include/fespace.hpp:195-271): v[ndof], device. */
pxg_status pxg_interpolate(pxg_ctx * ctx, int fn, double coef, double * v, void * stream);

/* ------------------------------------------------------------ device memory
 * Device buffers on the context's GPU for callers that have no CUDA runtime of their
 * own (the C++ Builder shim in include/proxgpu/builder.hpp uses them).  dir: 0 host
 * to device, 1 device to host, 2 device to device; synchronous when stream is NULL. */
pxg_status pxg_device_alloc(pxg_ctx * ctx, uint64_t bytes, void ** ptr);
pxg_status pxg_device_free(pxg_ctx * ctx, void * ptr);
pxg_status pxg_memcpy(pxg_ctx * ctx, void * dst, const void * src, uint64_t bytes, int dir, void * stream);

/* ------------------------------------------------------- solve and adjoint
 * Jacobi-preconditioned CG on a device CSR matrix (symmetric positive definite):
 * x = A^-1 b to ||b - A x|| <= rtol ||b|| within max_iter iterations, x starting at 0.
 * proxpde solves with UmfPackLU (include/sparse_matrix.hpp:44, include/solver.hpp:65);
 * this plain device CG is the engine's solver.  Returns PXG_ERR_NOT_CONVERGED (x holds
 * the last iterate) when the tolerance is not met.  The solve runs on a stream of the
 * context ordered after `stream`, replays its iterations as a CUDA graph and reads its
 * convergence flag on the host, so it returns with the solve complete and cannot be
 * captured into the caller's graph. */
pxg_status pxg_cg(pxg_ctx * ctx, const int32_t * row_ptr, const int32_t * col_idx,
                  const double * vals, int64_t n, const double * b, double * x, double rtol,
                  int max_iter, int * iters, double * rel_res, void * stream);
/* Adjoint gradient with respect to log k_e of a loss J(u) with K(k) u = b:
 * grad[e] = -(C u)_e^T K_e (C lambda)_e, K_e = k_e K0_e the element stiffness of the
 * context's coefficient (AssemblyStiffnessFE), C zeroing the DOFs of the essential BCs;
 * lambda solves K lambda = dJ/du.  u, lambda: device, ndof; grad: device, nelem. */
pxg_status pxg_adjoint_grad(pxg_ctx * ctx, const double * u, const double * lambda, double * grad,
                            void * stream);
/* Forward/backward operator pair (the shape of a torch.autograd.Function):
 * forward assembles K(k) (with BCs), M and b (from `rhs`, with BCs), solves K u = b by
 * CG, and returns J = 1/2 (u - u_target)^T M (u - u_target); it keeps K, M, u and
 * M (u - u_target) in the context.  backward solves K lambda = M (u - u_target) and
 * writes grad[e] = dloss * dJ/dlog k_e (and lambda if lambda_out is not NULL). */
pxg_status pxg_adjoint_forward(pxg_ctx * ctx, const pxg_rhs_op * rhs, const double * u_target,
                               double rtol, int max_iter, double * u_out, double * loss, int * iters,
                               void * stream);
pxg_status pxg_adjoint_backward(pxg_ctx * ctx, double dloss, double * grad, double * lambda_out,
                                int * iters, void * stream);

/* ---------------------------------------------------------------- batches
 * Many independent problems of one element type in one context: the mesh given to
 * pxg_set_mesh is their disjoint union with the elements grouped by problem (problem
 * p owns elements [elem_offsets[p], elem_offsets[p+1]), no node shared between
 * problems).  First-touch numbering then gives each problem a contiguous DOF range.
 * Call after pxg_build_pattern; elem_offsets is host memory (nprob + 1 values). */
pxg_status pxg_batch_set(pxg_ctx * ctx, const int64_t * elem_offsets, int64_t nprob);
/* For every problem of one or two batches (ctxs[0..nctx-1], same GPU): assemble
 * K(k) with BCs, M and b (from `rhs`), solve K u = b, J_p = 1/2 (u-ut)^T M (u-ut),
 * solve K lambda = M (u-ut), grad = dJ/dlog k_e.  The solves of all problems run in
 * one persistent cooperative kernel with per-problem convergence (relative residual
 * rtol); with use_graph the assembly, the solver and the gradient kernels are
 * captured once in a CUDA graph and replayed while the arguments stay the same.
 * u_targets[i]: device, ndof of ctxs[i]; grads[i]: device, nelem of ctxs[i];
 * losses: host, one per problem (ctxs[0]'s problems first); iters: the largest CG
 * iteration count.  PXG_ERR_TIMEOUT if a grid barrier wait of the persistent kernel
 * ran out (the context stays usable). */
pxg_status pxg_batch_adjoint(pxg_ctx * const * ctxs, int nctx, const pxg_rhs_op * rhs,
                             const double * const * u_targets, double rtol, int max_iter,
                             double * losses, double * const * grads, int * iters, int use_graph,
                             void * stream);

/* -------------------------------------------------------------- measurement
 * No counterpart in proxpde: the FP64 FMA rate of a device (FMAs per second, one FMA
 * = two floating-point operations), from an event-timed kernel of independent FMA
 * chains; the ceiling of the FP64-bound element kernels, reported beside their time.
 * ms (may be NULL) receives the timed launch's duration. */
pxg_status pxg_fp64_rate(int device, double * fma_per_s, double * ms);
/* The rate of FP64 reductions (red.global.add.f64) on `device`, by lane pattern: every
 * warp instruction adds into 32 doubles, `lanes_per_sector` (1, 2 or 4) consecutive
 * lanes sharing one 32-byte sector, the sectors hashed over an array of `bytes` (a power
 * of two, 4 KB .. 32 GB; below the 129 MB of L2 the array stays there).  Reductions per
 * second of the best of three launches after a warm-up, and that launch's ms (optional).
 * Measurement, beside pxg_fp64_rate: the bound of the element kernels' scatter.  No
 * counterpart in proxpde. */
pxg_status pxg_red_rate(int device, int lanes_per_sector, int64_t bytes, double * red_per_s, double * ms);

/* ----------------------------------------------------- allocation-free prune
 * No counterpart in proxpde: an allocation-free variant of pxg_close_matrix's
 * prune/compact for callers that cannot call cudaMalloc (code running where the
 * host application owns every device allocation, or where driver allocations are
 * forbidden, such as host callbacks and real-time sections).  It needs no context:
 * the caller passes the structural CSR (row_ptr[nrows+1], col_idx, vals) and the
 * outputs (row_ptr_out[nrows+1], col_idx_out and vals_out with the input's
 * capacity), all device pointers on the current device, and gets the kept-entry
 * count in *nnz_out (host).  Entries with |v| <= 1e-16 are dropped, as
 * Builder::closeMatrix's prune(1., 1e-16) does.
 * Limits: nrows <= 4,194,304 (else PXG_ERR_INVALID_ARG); its intermediate data live
 * in one fixed 16.8 MB device array that every GPU loading the library keeps until
 * exit.  The first call on a device looks up that array's address.  Calls that
 * overlap on the GPU share the array and race: serialise them.  Every call
 * synchronises `stream` to return the count, so it cannot be stream-captured. */
pxg_status pxg_prune_csr_noalloc(const int32_t * row_ptr, const int32_t * col_idx,
                                 const double * vals, int64_t nrows, int32_t * row_ptr_out,
                                 int32_t * col_idx_out, double * vals_out, int64_t * nnz_out,
                                 void * stream);

#ifdef __cplusplus
}
#endif

#endif /* PXG_H */
