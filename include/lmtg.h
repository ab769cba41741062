/*
 * lmtg.h -- C ABI of the GB300 finite-element hot path (element matrices -> assembly -> solve).
 *
 * This is the drop-in boundary for LMT++'s formulation/assemble/solve API.  Each entry point
 * names the reference interface it replaces (paths inside the LMTpp project):
 *
 *   FormulationAncestor<T>            include/formulation/formulation_ancestor.h:18-262
 *   Formulation<...>::allocate_matrices include/formulation/formulation.h:338-412
 *   Formulation<...>::assemble        include/formulation/formulation.h:1112-1125
 *   Formulation<...>::solve_system    include/formulation/formulation.h:1494-1504
 *   Formulation<...>::solve           include/formulation/formulation.h:1517-1568
 *   add_constraint / assemble_constraints include/formulation/formulation.h:1028-1091
 *   get_mat / get_sollicitation / get_result  formulation_ancestor.h:88-120
 *
 * Conventions: every function returns an int status (LMTG_OK == 0).  No C++ exception crosses
 * the ABI.  Host buffers are caller-owned and only read or written during the call; device
 * buffers are owned by the context.  A context is bound to one CUDA device and must not be
 * used from two host threads at once.  lmtg_last_error() gives a message for the last failure.
 */
#ifndef LMTG_H
#define LMTG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define LMTG_OK 0
#define LMTG_ERR_ARG 1           /* bad argument or size */
#define LMTG_ERR_CUDA 2          /* CUDA runtime error */
#define LMTG_ERR_STATE 3         /* call out of order (e.g. solve before assemble) */
#define LMTG_ERR_NOT_CONVERGED 4 /* iteration cap reached (reference: SolveException) */
#define LMTG_ERR_TIMEOUT 5       /* host wall-clock watchdog expired */
#define LMTG_ERR_NAN 6           /* NaN / Inf in a PCG scalar */
#define LMTG_ERR_NOMEM 7         /* device allocation failed */
#define LMTG_ERR_UNSUPPORTED 8   /* element type / size not supported */

/* ---- element types (nodes per element) ---- */
#define LMTG_ELEM_HEXA8 8    /* faces: Quad4 (4 node ids) */
#define LMTG_ELEM_TETRA10 10 /* faces: Triangle_6 (6 node ids: vertices, then mid-edges 01 12 20) */
#define LMTG_ELEM_TRIANGLE6 6 /* 2D heat diffusion (lmtg_diff_*), one unknown per node */

/* ---- lmtg_assemble flags ---- */
#define LMTG_ASM_MAT64 1        /* FP64 element matrices -> FP64 K */
#define LMTG_ASM_MAT32 2        /* FP32 copy of K rounded from the FP64 assembly (inner operator) */
#define LMTG_ASM_VEC 4          /* sollicitation vector (loads + constraint right-hand sides) */
#define LMTG_ASM_MAT32_NATIVE 8 /* FP32 element kernel -> FP32 K (no FP64 pass) */

/* ---- solve modes ---- */
#define LMTG_SOLVE_PCG_F64 0  /* plain FP64 block-Jacobi PCG */
#define LMTG_SOLVE_MIXED_IR 1 /* FP32 inner PCG wrapped in FP64 iterative refinement */

/* ---- preconditioners of the FP32 inner PCG (lmtg_set_preconditioner) ---- */
#define LMTG_PREC_BLOCK_JACOBI 0 /* inverse 3x3 diagonal blocks */
#define LMTG_PREC_AMG 1          /* aggregation multigrid W-cycle (the default) */

/* ---- stopping criteria ---- */
#define LMTG_CRIT_REL_RESIDUAL 0   /* |b - K u|_2 <= tol |b|_2 */
#define LMTG_CRIT_NORM_INF_DELTA 1 /* |alpha d|_inf <= tol (ConvergenceCriteriumNormInfDelta,
                                      include/containers/conjugate_gradient.h:100-111) */
#define LMTG_CRIT_NORM2_DELTA 2    /* |alpha d|_2 < tol (ConvergenceCriteriumNorm2, :113-123) */
#define LMTG_CRIT_ABS_RESIDUAL_INF 3 /* |r|_inf <= tol (solve_using_incomplete_chol_factorize,
                                        include/containers/matinvsparse.h:453-491) */

/* ---- adjoint objectives ---- */
#define LMTG_OBJ_COMPLIANCE 0 /* J = F . u */
#define LMTG_OBJ_MISFIT 1     /* J = 1/2 sum_i w_i (u_i - t_i)^2 */
#define LMTG_OBJ_LINEAR 2     /* J = c . u, c passed as `target` (adjoint of any upstream gradient) */

typedef struct lmtg_ctx lmtg_ctx;

typedef struct lmtg_solve_stats {
    int iterations;       /* total PCG iterations (inner iterations for the mixed mode) */
    int outer_iterations; /* FP64 refinement steps (mixed mode), 0 for plain PCG */
    int status;           /* same as the return value */
    int reserved;
    double rel_residual;  /* final |b - K u|_2 / |b|_2, recomputed in FP64 */
    double device_ms;     /* device time of the solve (CUDA events) */
} lmtg_solve_stats;

/* Context.  Replaces the construction of Problem/Formulation objects. */
int lmtg_create(int device, lmtg_ctx **ctx);
int lmtg_destroy(lmtg_ctx *ctx);
const char *lmtg_last_error(const lmtg_ctx *ctx);
const char *lmtg_status_string(int status);

/* Structured unit-box Hexa mesh on the host, identical node order and coordinates to
 * make_rect(m, Hexa(), X0, X1, nb_points) (include/mesh/make_rect.h:653-679).
 * pos: nn*3 doubles, conn: ne*8 (nn = prod nb_points, ne = prod (nb_points-1)). */
int lmtg_make_rect_hexa(const double X0[3], const double X1[3], const uint32_t nb_points[3],
                        double *pos, uint32_t *conn);

/* Structured unit-box Tetra_10 mesh on the host, identical to
 * make_rect(m, Tetra_10(), X0, X1, nb_points) (include/mesh/make_rect.h:443-545): 6 tetrahedra
 * per cube, nodes in first-creation order (the reference's distance search replaced by exact
 * half-grid coordinates: same order, same stored positions), negative-Jacobian tetrahedra
 * renumbered as permutation_if_jac_neg (include/mesh/element_Tetra_10.h:122-130).
 * Two-phase: with pos or conn NULL only *nn and *ne are written. */
int lmtg_make_rect_tetra10(const double X0[3], const double X1[3], const uint32_t nb_points[3],
                           uint64_t *nn, uint64_t *ne, double *pos, uint32_t *conn);

/* Mesh (the TM object a Formulation points to, formulation.h:2740-2745): node positions
 * (nn*3), element connectivity (ne*nodes_per_element), DOF numbering node*3 as the reference's
 * default indice_noda (formulation.h:283-325, no AMD/RCM renumbering). */
int lmtg_mesh_set(lmtg_ctx *ctx, int elem_type, uint64_t nn, const double *pos, uint64_t ne,
                  const uint32_t *conn);

/* Material: elastic_modulus (one value, or one per element) and poisson_ratio
 * (formulations/formulation_elasticity_iso.py:5-6). */
int lmtg_material_set(lmtg_ctx *ctx, const double *E, uint64_t nE, double nu);

/* allocate_matrices (formulation.h:338-412): builds the node-block sparsity pattern, the
 * element-to-block gather lists and all device buffers.  *nnz_lower (optional) receives the
 * number of stored scalar entries of the lower triangle (the SparseLine nb_nz()). */
int lmtg_allocate_matrices(lmtg_ctx *ctx, uint64_t *nnz_lower);

/* Nodal loads f_nodal (n = 3*nn doubles).  They replace the whole load vector, skin tractions
 * added before included; lmtg_add_skin_traction adds to it afterwards. */
int lmtg_set_nodal_loads(lmtg_ctx *ctx, const double *F);
/* Uniform traction f_surf on skin faces (Quad4 for Hexa8 meshes: nfaces*4 node ids; Triangle_6
 * for Tetra10 meshes: nfaces*6), accumulated into the load vector as consistent nodal loads (the
 * add_skin_elem_matrix terms, formulation.h:584-594), integrated with the rules the reference's
 * generator bakes into those routines (formal_lf/formulation.py:400-438): gauss_points[3] of
 * formulations/element_Quad.py, gauss_points[4] of formulations/element_Triangle_6.py. */
int lmtg_add_skin_traction(lmtg_ctx *ctx, uint64_t nfaces, const uint32_t *faces,
                           const double traction[3]);
/* Skin pressure p dS_normal . te dS (formulation_elasticity_iso.py:60, variable p), on the same
 * faces: the unit normal is cross(d x/d xi0, d x/d xi1) of the face's node order
 * (formal_lf/element.py:467-474); outward for the Hexa children.  Adds to the load vector. */
int lmtg_add_skin_pressure(lmtg_ctx *ctx, uint64_t nfaces, const uint32_t *faces, double p);

/* Volume force of elasticity_iso (formulations/formulation_elasticity_iso.py:49, static:
 * dep_tt = 0): F += density f_vol int N dV; f_vol global (3 doubles).  Defaults 0. */
int lmtg_set_volume_force(lmtg_ctx *ctx, double density, const double f_vol[3]);
/* Nodal springs dep_imp_coef_0 (formulation_elasticity_iso.py:55-60): K(3I+d,3I+d) += coef[I],
 * F(3I+d) += coef[I] target[3I+d] (target = lim_cond_0 dep_imp_val_0_0 + lim_cond_1
 * dep_imp_val_0_1; NULL: 0).  coef NULL removes them. */
int lmtg_set_nodal_springs(lmtg_ctx *ctx, const double *coef, const double *target);
/* The formulation's levenberg_marquadt term (formulation_ancestor.h:253, applied in
 * assemble_constraints, formulation.h:1033-1034): K(i,i) += max|diag K| * lm at every matrix
 * assembly, before the constraints; 0 by default. */
int lmtg_set_levenberg_marquadt(lmtg_ctx *ctx, double lm);
/* Constraints add_constraint("coef*node[i].dep[d] - res", penalty) for linear single-unknown
 * constraints; assembled as in assemble_constraints (formulation.h:1028-1071):
 * K(j,j) += coef^2 * max|diag K| * penalty, F(j) += coef * max|diag K| * penalty * res.
 * penalty == 0 is the reference's exact constraint (Lagrange rows, formulation.h:1072-1088),
 * applied here by elimination: u_j = res / coef exactly (one exact constraint per DOF, coef != 0;
 * needs the FP64 matrix assembly; not with the adjoint, the fit or batch solves). */
int lmtg_set_constraints(lmtg_ctx *ctx, uint64_t nc, const uint32_t *dof, const double *coef,
                         const double *res, double penalty);

/* assemble(assemble_mat, assemble_vec) (formulation.h:1112-1125), flags LMTG_ASM_*. */
int lmtg_assemble(lmtg_ctx *ctx, int flags);

/* get_mat: the assembled FP64 matrix as the reference's Sym SparseLine lower CSR (row i holds
 * columns j <= i ascending, diagonal last).  rowptr: n+1, col/val: nnz_lower. */
int lmtg_get_matrix_lower(lmtg_ctx *ctx, uint64_t *rowptr, uint32_t *col, double *val);
/* get_sollicitation: the assembled right-hand side (n doubles). */
int lmtg_get_sollicitation(lmtg_ctx *ctx, double *F);
/* Element matrices of elements [e0, e0+count) as dense row-major (3 npe) x (3 npe) blocks
 * (24x24 Hexa8, 30x30 Tetra10), for tests and inspection. */
int lmtg_get_element_matrices(lmtg_ctx *ctx, int precision, uint64_t e0, uint64_t count,
                              double *Ke);

/* solve_system(iterative_criterium) (formulation.h:1494-1504) on the assembled system.
 * The initial guess is the current result vector (zero after allocate_matrices).  maxit caps
 * the PCG iterations; timeout_s > 0 bounds the host wall clock. */
int lmtg_solve_system(lmtg_ctx *ctx, int mode, int crit_kind, double tol, int maxit,
                      double timeout_s, lmtg_solve_stats *stats);
/* solve(): assemble(mat and vec) followed by solve_system (formulation.h:1517-1568). */
int lmtg_solve(lmtg_ctx *ctx, int mode, int crit_kind, double tol, int maxit, double timeout_s,
               lmtg_solve_stats *stats);

/* get_result(0): the solution vector (n doubles); set_result: the initial guess. */
int lmtg_get_result(lmtg_ctx *ctx, double *u);
int lmtg_set_result(lmtg_ctx *ctx, const double *u);

/* Penalty scale: 0 (default) recomputes max|diag K| at every matrix assembly as the reference
 * does (formulation.h:1029-1030); a positive value is used instead, which holds the penalty fixed
 * while the material changes (the gradients below treat it as constant).
 * lmtg_get_penalty_scale returns the value used by the last assembly. */
int lmtg_set_penalty_scale(lmtg_ctx *ctx, double max_diag);
int lmtg_get_penalty_scale(lmtg_ctx *ctx, double *max_diag);

/* Adjoint gradient of an objective of the current solution u w.r.t. every element's Young's
 * modulus (ne doubles into dJdE) and the objective value J.  No counterpart in the reference,
 * which offers forward sensitivities only (solve_and_get_derivatives, formulation.h:1588-1652:
 * one solve per parameter).  Compliance needs no extra solve (the adjoint is u); the misfit
 * (target t and weights w of n doubles, NULL = 0 and 1) solves K lambda = w (u - t), the linear
 * objective (c in `target`) solves K lambda = c, with `mode`
 * (LMTG_SOLVE_*) to the relative residual `tol`.  dJ/dE_e = -lambda_e^T (K_e / E_e) u_e with the
 * element matrix recomputed, not stored; the penalty scale is held constant. */
int lmtg_adjoint_grad(lmtg_ctx *ctx, int objective, const double *target, const double *weights,
                      int mode, double tol, int maxit, double timeout_s, double *J, double *dJdE,
                      lmtg_solve_stats *stats);

/* y = K x with the assembled matrix in FP64 (precision 0) or FP32 (precision 1). */
int lmtg_spmv(lmtg_ctx *ctx, int precision, const double *x, double *y);

/* The CUDA stream (cudaStream_t) every kernel and copy of this context is issued on, so a
 * caller can order its own work or record CUDA events around calls. */
int lmtg_get_stream(lmtg_ctx *ctx, void **stream);

/* Number of kernels this context has launched since creation (all entry points). */
int lmtg_get_launch_count(lmtg_ctx *ctx, uint64_t *count);

/* Times the two PCG iteration kernels (fused SpMV kernel, update kernel) over `iters` plain
 * launches on the context's stream with CUDA events; precision 0 = FP64 system, 1 = FP32 inner
 * system.  Writes the mean milliseconds per launch of each kernel.  Needs an assembled system;
 * leaves the result vector untouched. */
int lmtg_profile_pcg_kernels(lmtg_ctx *ctx, int precision, int iters, double *spmv_ms,
                             double *update_ms);

/* Allocation-free residual: r = b - K x and *rr_host = |r|_2^2 (FP64) for a 3x3-block
 * matrix the caller already holds on the device (bptr[nn+1], bcol[nnz_blocks] as u32,
 * K[9*nnz_blocks] row-major blocks, full symmetric pattern; x, b, r of 3*nn doubles), issued
 * on `stream` (NULL = default stream).  It has no counterpart in the reference: it is for
 * callers that cannot call cudaMalloc (device memory owned by their own arena, no allocation
 * allowed between steps).  It allocates nothing: its reduction scratch is a fixed 512 KiB
 * device array, so nn is limited to 524,288 node rows (LMTG_ERR_ARG beyond).  The first call
 * on each device looks up that array's address (make it before any stream capture) and keeps
 * it for the life of the process: a cudaDeviceReset of that device reloads the library's device
 * code, so a process that resets a device must not call this entry point on it again.  All
 * calls share the array: calls that overlap on the GPU race.  rr_host may be NULL (then the
 * call does not synchronize the stream). */
int lmtg_residual_norm_noalloc(void *stream, uint64_t nn, const uint32_t *bptr,
                               const uint32_t *bcol, const double *K, const double *x,
                               const double *b, double *r, double *rr_host);

/* ---- transient heat diffusion (formulation difftherm on Triangle_6) ----
 * formulations/formulation_difftherm.py:24-30; theta scheme A T_{n+1} = B T_n with
 * A = M/dt + theta K, B = M/dt - (1 - theta) K, K = int a grad N . grad N, a = conductivity /
 * rho_c.  theta = 1/2 reproduces the reference's time integration (the residual at the interval
 * midpoint, formal_lf/formulation.py:506-509); theta = 1 is implicit Euler. */

/* Structured Triangle_6 mesh of make_rect(m, Triangle_6(), X0, X1, nb_points)
 * (include/mesh/make_rect.h:141-170): pos nn*2, conn ne*6.  Two-phase like Tetra_10. */
int lmtg_make_rect_triangle6(const double X0[2], const double X1[2], const uint32_t nb_points[2],
                             uint64_t *nn, uint64_t *ne, double *pos, uint32_t *conn);
/* 2D mesh of a diffusion context (created with lmtg_create). */
int lmtg_diff_mesh_set(lmtg_ctx *ctx, uint64_t nn, const double *pos, uint64_t ne,
                       const uint32_t *conn);
/* Conductivity (1 or ne values), rho_c, time step, theta, and T = 0 on the given nodes by the
 * reference's penalty (scale max|diag A| * penalty, or the fixed lmtg_set_penalty_scale value).
 * Builds the pattern (first call), the element matrices and A, B. */
int lmtg_diff_setup(lmtg_ctx *ctx, const double *k, uint64_t nk, double rho_c, double dt,
                    double theta, uint64_t nbnd, const uint32_t *bnd_nodes, double penalty);
/* Constant sources of difftherm (formulations/formulation_difftherm.py:26-29): the volume source
 * Q (nodal field, -Q te dV, applied as M Q) and the nodal source Qs (-Qs te dN); either may be
 * NULL (nn doubles each).  Added to the right-hand side of every step. */
int lmtg_diff_set_sources(lmtg_ctx *ctx, const double *Q, const double *Qs);
/* Skin convection H (T - t0) te dS (formulation_difftherm.py:29) on nedges Bar_3 edges
 * (3 nodes each: end, end, middle; formulations/element_Bar_3.py), H per edge (nH = nedges) or
 * one value: adds theta H Ms to A, -(1 - theta) H Ms to B and H t0 int N ds to every step's
 * right-hand side.  Call after lmtg_diff_setup (which clears it). */
int lmtg_diff_set_convection(lmtg_ctx *ctx, uint64_t nedges, const uint32_t *edges, const double *H,
                             uint64_t nH, double t0);
/* Linear solver of every time step (and of the adjoint): LMTG_SOLVE_PCG_F64 (default, FP64
 * Jacobi-PCG) or LMTG_SOLVE_MIXED_IR (FP32 Jacobi-PCG with FP64 residual replacement). */
int lmtg_diff_set_solver(lmtg_ctx *ctx, int mode);
/* Temperature state (nn doubles). */
int lmtg_diff_set_state(lmtg_ctx *ctx, const double *T);
int lmtg_diff_get_state(lmtg_ctx *ctx, double *T);
/* nsteps time steps from the current state, each solved to the relative
 * residual tol (warm start from the previous state) with the solver of lmtg_diff_set_solver. */
int lmtg_diff_run(lmtg_ctx *ctx, int nsteps, double tol, int maxit, lmtg_solve_stats *stats);
/* Final-time misfit J = 1/2 |T_N - target|^2 of nsteps steps from the current state and its
 * adjoint gradient w.r.t. every element's conductivity (ne doubles into dJdk), with forward
 * states checkpointed every `checkpoint_every` steps and recomputed per segment in the backward
 * sweep; checkpoint_every = 1 keeps all nsteps + 1 states and recomputes none (no reference
 * counterpart).  The penalty scale is held constant.  Leaves T_N as state. */
int lmtg_diff_adjoint_misfit(lmtg_ctx *ctx, int nsteps, int checkpoint_every, const double *target,
                             double tol, int maxit, double *J, double *dJdk,
                             lmtg_solve_stats *stats);
/* A and B as lower CSR (rowptr nn+1, col/A/B nnz_lower = (blocks - nn)/2 + nn entries). */
int lmtg_diff_get_matrices(lmtg_ctx *ctx, uint64_t *rowptr, uint32_t *col, double *A, double *B);

/* ---- batches of independent meshes (no reference counterpart as one call: the reference
 * solves one Formulation per mesh and one right-hand side per solve,
 * include/formulation/formulation_ancestor.h:64) ----
 * The context's mesh is the concatenation of nsys meshes: system m owns the node range
 * [node_off[m], node_off[m+1]) (node_off[0] = 0, node_off[nsys] = nn) and no element couples two
 * ranges.  The penalty scale max|diag| is then taken per system.  Call after lmtg_mesh_set. */
int lmtg_batch_set(lmtg_ctx *ctx, uint32_t nsys, const uint64_t *node_off);
/* Per-element Poisson ratios (n_nu = ne), replacing the single value of lmtg_material_set
 * (which returns the context to a single ratio: call this one after it). */
int lmtg_material_set_nu(lmtg_ctx *ctx, const double *nu, uint64_t n_nu);
/* nrhs (1..4) right-hand sides, B[r * ndof + i] (host); resets the batch solution to 0. */
int lmtg_batch_set_rhs(lmtg_ctx *ctx, int nrhs, const double *B);
/* Solves every (system, rhs) pair to |b - K x|_2 <= tol |b|_2 (FP64 true residual of that pair)
 * with block-Jacobi PCG: LMTG_SOLVE_PCG_F64 or LMTG_SOLVE_MIXED_IR (FP32 inner, FP64 residual
 * replacement; needs LMTG_ASM_MAT32).  maxit bounds the iterations of every pair.  stats: the
 * largest pair iteration count, FP32 segments, and the worst final relative residual;
 * pair_iters (optional, nsys * nrhs ints, system-major) the iterations of each pair. */
int lmtg_batch_solve(lmtg_ctx *ctx, int mode, double tol, int maxit, double timeout_s,
                     lmtg_solve_stats *stats, int *pair_iters);
/* The solutions, X[r * ndof + i] (nrhs x ndof doubles, host). */
int lmtg_batch_get_result(lmtg_ctx *ctx, double *X);
/* The autotuner's choice: rows per tile, SpMV variant (0 plain, 1 next row prefetched, 2 the
 * matrix streamed through shared memory by bulk copies, FP32 only), tile count, and the SpMV
 * time of each candidate (12 doubles, ms, variant-major over tile sizes 16, 32, 64, 128 rows
 * for variants 0, 1 and 128, 256, 512, 1024 for variant 2; 0 = not tried; optional).  A tile
 * is one warp's work (variants 0, 1); in variant 2 it is one CTA's SpMV unit, made of 128-row
 * tiles that the vector kernels take one warp each. */
int lmtg_batch_info(lmtg_ctx *ctx, int *tile_rows, int *variant, uint64_t *ntiles, double *tuned_ms);
/* Fixed rows per tile (0: autotune) and SpMV variant (-1: autotune; 0, 1, 2) of the batch
 * solver. */
int lmtg_batch_set_options(lmtg_ctx *ctx, int tile_rows, int variant);

/* Mixed-precision solvers (lmtg_solve_system, lmtg_batch_solve, the diffusion steps): the
 * recursive-residual reduction of each FP32 segment before the FP64 residual replacement,
 * in (0, 1); default 0.01 (1e-3 saved one refinement step on Hexa8 128^3 but made the
 * continued-direction segments on Tetra10 40^3 stall).  No reference counterpart. */
int lmtg_set_inner_reduction(lmtg_ctx *ctx, double inner_reduction);

/* FP32 SpMV of the single-system PCG: 0 = one warp per pair of node rows, the matrix read
 * straight into registers; 1 and 2 = the matrix streamed through shared memory by bulk copies
 * (TMA) in a ring of two stages of up to 16 rows, sized for 4 and 5 CTAs per SM; -1 (default)
 * = 2 when a node row has more than 32 blocks (Tetra10), else 1.  All give the same q; p.q is
 * summed in a different fixed order.  The diffusion step solver uses its bulk-copy SpMV unless
 * the kind is 0.  No reference counterpart. */
int lmtg_set_spmv_kind(lmtg_ctx *ctx, int kind);

/* Self-test of the device-side wait bound used by the bulk-copy SpMVs: one thread waits on an
 * mbarrier that nothing completes.  *status = LMTG_ERR_TIMEOUT when the wait gave up (about
 * 1 s, *waited_s), and the context stays usable.  No reference counterpart. */
int lmtg_selftest_bounded_wait(lmtg_ctx *ctx, int *status, double *waited_s);

/* Element fields after the solve (replaces the generated apply_on_elements_after_solve of
 * elasticity_iso, formulations/formulation_elasticity_iso.py:64-85, run by call_after_solve,
 * include/formulation/formulation.h:1867-1875): per element, at var_inter = 0.5, out[13 e + k] =
 * epsilon (k 0..5, tensor shear, 11 22 33 12 13 23), sigma (k 6..11), tr epsilon (k 12).
 * u: ndof doubles (host), or NULL for the current result. */
int lmtg_element_fields(lmtg_ctx *ctx, const double *u, double *out);

/* Identification of zone moduli by Gauss-Newton (replaces FormulationFit::exec,
 * include/formulation/FormulationFit.h:17-80, for the elastic_modulus parameter): E_e =
 * p[zone_of_elem[e]] with nz (1..4) zones; u_exp the measured displacement (ndof), w its
 * diagonal weight standing for exp_mat (NULL: 1), sens_val the weights of the
 * sensitivity_after_fit sums (NULL: 1).  Each iteration assembles, solves u (mode
 * LMTG_SOLVE_PCG_F64 or MIXED_IR, relative residual tol, maxit), solves the nz sensitivities
 * dU_i = -K^-1 dK/dp_i u, forms M_ij = (w dU_i).dU_j and V_i = (w dU_i).(u_exp - u), adds
 * levenberg_marq * max|diag M| to the diagonal and updates p += relaxation M^-1 V; it stops when
 * every |dD_i| < conv or at iteration max_iter (counted from 0, the reference's 20).  p (nz) is
 * updated in place; history (max|dD| per iteration) and residual_history ((w d).d per
 * iteration) need max_iter + 1 doubles each (optional); sensitivity (nz, optional). */
int lmtg_fit_zone_moduli(lmtg_ctx *ctx, uint32_t nz, const uint32_t *zone_of_elem, double *p,
                         const double *u_exp, const double *w, const double *sens_val,
                         double relaxation, double levenberg_marq, double conv, int max_iter,
                         int mode, double tol, int maxit, double *history,
                         double *residual_history, double *sensitivity, int *n_iter);

/* Recalage functional (replaces the generated add_elem_matrix / add_nodal_matrix of formulation
 * recalage, formulations/formulation_recalage.py:1-47, assembled by Formulation::assemble,
 * include/formulation/formulation.h:1112-1125, nodal terms by add_nodal_matrix at 467-489): the Hessian and minus the gradient at 0 of
 *   gamma a(V - U, V - U) + (1 - gamma) rho |W - U|^2_L2 + sum_nodes Ud_valid r/(1-r) E |U - Ud|^2
 * (use_test_functions = False), with the volume terms integrated by the element's Python rule of
 * order 2 (integration_totale).  Unknowns per node U, V, W then component: DOF 9 I + 3 f + d of
 * node I, field f (0 U, 1 V, 2 W), component d -- the reference's unknown order with lambd, which
 * appears in no term, left out.  Needs lmtg_mesh_set (Hexa8 or Tetra10) and lmtg_material_set with
 * one E and one poisson_ratio; replaces lmtg_allocate_matrices.  Ud: 3 nn doubles, Ud_valid: nn
 * doubles (both nodal).  omega cancels out of the functional and is only checked non-zero.  After
 * this call the context holds the 9 nn-unknown system: lmtg_set_constraints takes its DOFs, then
 * lmtg_recalage_assemble builds it, and lmtg_solve_system / lmtg_get_result /
 * lmtg_get_matrix_lower / lmtg_get_sollicitation work on it; elasticity assembly, gradients and
 * element fields refuse it (LMTG_ERR_STATE) until the next lmtg_mesh_set.  On a failure the
 * mesh must be set again. */
int lmtg_recalage_setup(lmtg_ctx *ctx, double rho, double omega, double gamma, double r, const double *Ud,
                        const double *Ud_valid);
/* Element stiffness and mass blocks, their node-pattern gather, the 9-unknown Hessian and
 * right-hand side, then the constraints (penalty or exact) and both preconditioners. */
int lmtg_recalage_assemble(lmtg_ctx *ctx);

/* Preconditioner of the FP32 inner PCG of the mixed solve (LMTG_SOLVE_MIXED_IR), standing in
 * for the reference's sequential incomplete Cholesky (include/containers/matinvsparse.h:201-261,
 * MatWithTinyBlocks.h:426-585).  LMTG_PREC_AMG (default): one W-cycle of an unsmoothed-aggregation
 * multigrid (every level above the coarsest visits the next level twice) whose coarse spaces
 * carry the six rigid-body modes per aggregate, damped block-Jacobi smoothing, a dense coarsest
 * level; used for single-system Hexa8 / Tetra10 elasticity of at
 * least 3,000 unknowns, block Jacobi otherwise (batches, recalage, small systems).  Its structure
 * is built at the first mixed solve after lmtg_allocate_matrices or lmtg_set_constraints (nodes
 * with a constraint stay out of the coarse spaces), its numeric part at the first mixed solve
 * after each matrix assembly.  LMTG_PREC_BLOCK_JACOBI: the inverse 3x3 diagonal blocks.  The
 * FP64 PCG always uses block Jacobi.
 * The diffusion step solver (lmtg_diff_set_solver LMTG_SOLVE_MIXED_IR) follows the same setting:
 * with LMTG_PREC_AMG and at least 3,000 nodes its FP32 PCG runs one cycle of a scalar
 * aggregation multigrid (piecewise-constant coarse spaces without the Dirichlet nodes, damped
 * Jacobi smoothing, the top level's coarse correction visiting level 1 twice, a dense coarsest
 * level), built at the first FP32 solve after lmtg_diff_setup or lmtg_diff_set_convection;
 * Jacobi otherwise. */
int lmtg_set_preconditioner(lmtg_ctx *ctx, int kind);
/* The multigrid hierarchy built for the last mixed solve (levels = 0 when none): per level
 * (up to 8) unknowns, stored blocks, damped-Jacobi weight and lambda_max(D^-1 K); the host time
 * of the structure setup, of the last numeric setup, and of the structure setup's phases
 * (pattern copy and rigid-body modes, aggregation, tentative prolongators, coarse patterns and
 * gather lists, uploads).  Any output may be NULL. */
int lmtg_amg_info(lmtg_ctx *ctx, int *levels, uint64_t ndof[8], uint64_t nnz_blocks[8], double omega[8],
                  double lambda_max[8], double *structure_ms, double *numeric_ms, double structure_phase_ms[5]);

/* FP32 SpMV kind in use for this context's solves (0 warp-row, 1 / 2 bulk copies with 4 / 5 CTAs
 * per SM), the autotuned kind (-1 before the first FP32 solve of the pattern, or when
 * lmtg_set_spmv_kind pinned one) and the autotuner's per-kind launch times (ms, 0 = not timed). */
int lmtg_spmv_info(lmtg_ctx *ctx, int *kind_in_use, int *tuned, double tune_ms[3]);
/* Device time (ms, CUDA events) of each stage of one multigrid-preconditioned FP32 iteration,
 * averaged over `iters` iterations on the assembled system: [0] SpMV q = K p, [1] update with
 * the first smoothing step, [2] level-0 residual, [3] restriction, [4] coarse levels, [5]
 * prolongation, [6] level-0 smoothing forming z, [7] direction update.  All 0 without a
 * hierarchy. */
int lmtg_profile_amg_kernels(lmtg_ctx *ctx, int iters, double ms[8]);

/* Sizes of the current problem. */
int lmtg_get_sizes(lmtg_ctx *ctx, uint64_t *nn, uint64_t *ne, uint64_t *ndof, uint64_t *nnz_blocks);

/* ---- mesh files next to the path (context-free host code, no GPU needed) ---- */

/* Gmsh ASCII format-2 reader (replaces read_msh_2, include/mesh/read_msh_2.h:56-235).  Nodes in
 * file order (pos: nn x dim, dim 3 for LMTG_ELEM_HEXA8 / LMTG_ELEM_TETRA10, 2 for
 * LMTG_ELEM_TRIANGLE6); elements of the mesh's dimension in file order, in LMT++'s node order
 * (Tetra_10: Gmsh's last two edge nodes swapped) and re-ordered by LMT++'s permutation when the
 * Jacobian at var_inter = 0.5 is negative (permutation_if_jac_neg); lower-dimension elements
 * (faces, edges, points) skipped; tag[e] = the element's first tag (0 without tags).  Call with
 * pos = conn = tag = NULL to get nn and ne, then with buffers of those sizes (any may be NULL).
 * LMTG_ERR_ARG: unreadable or corrupt file, unknown node number; LMTG_ERR_UNSUPPORTED: an
 * element of the mesh's dimension of another type (mixed meshes). */
int lmtg_read_msh(const char *path, int elem_type, uint64_t *nn, double *pos, uint64_t *ne, uint32_t *conn,
                  double *tag);

/* ASCII VTU file with the layout and number formatting of write_mesh_vtk<false>
 * (include/mesh/write_mesh_vtk.h:434-655): npf point arrays (pnames[f], pncomp[f] components,
 * pvals[f]: nn x pncomp[f]), then ncf cell arrays (cvals[f]: ne x cncomp[f]) of kind ckind[f]:
 * 0 = element field, 1 = global field written per element, 2 = unsigned integer (the element
 * group), each with the reference's separators; then points (z = 0 for 2D meshes), connectivity,
 * offsets and VTK cell types (12 Hexa8, 24 Tetra10, 22 Triangle6) in LMT++'s node order. */
int lmtg_write_vtu(const char *path, int elem_type, uint64_t nn, const double *pos, uint64_t ne,
                   const uint32_t *conn, int npf, const char *const *pnames, const int *pncomp,
                   const double *const *pvals, int ncf, const char *const *cnames, const int *cncomp,
                   const int *ckind, const double *const *cvals);

#ifdef __cplusplus
}
#endif
#endif /* LMTG_H */
