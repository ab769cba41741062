/*
 * fe_oracle.h -- CPU restatement of LMT++'s finite-element hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the GPU path:
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
 * load it.  The product (liblmtg.so) never links or calls it.
 *
 * Every function restates one piece of the reference, cited file:line
 * (paths inside the LMTpp project):
 *   mesh           include/mesh/make_rect.h:653-679 (Hexa), 443-545 (Tetra_10),
 *                  include/util/rectilinear_iterator.h:20-45
 *   Gauss tables   include/mesh/element_Hexa.h:5-20, include/mesh/element_Quad.h:5-12,
 *                  include/mesh/element_Tetra_10.h:5-16, include/mesh/element_Triangle_6.h:5-15
 *   element K_e    formulations/formulation_elasticity_iso.py:45-60,
 *                  formal_lf/material_help.py:116-134,175-183,
 *                  include/codegen/__init__.py:23-42,82-87,
 *                  include/formulation/formulation.h:2918-2932 (Gauss-point loop)
 *   pattern        include/formulation/formulation.h:200-241 (ResizeMat)
 *   scatter        formal_lf/calculate_matrix.py:64-98, include/containers/matsparse.h:757-770
 *   penalty        include/formulation/formulation.h:1028-1071
 *   IC(0)          include/containers/matinvsparse.h:201-261,397-423,453-491
 *   generic CG     include/containers/conjugate_gradient.h:27-68,100-123
 *   SpMV (Sym)     include/containers/matsparse.h:5368-5408
 *
 * Matrices are the reference's Mat<T,Sym<>,SparseLine<>> restated as a lower
 * CSR: row i holds the columns j <= i in ascending order, so the diagonal is
 * the last entry of each row.
 */
#ifndef FE_ORACLE_H
#define FE_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------- mesh ---------------- */
/* Structured Hexa mesh, nb_points[d] nodes along axis d; node creation order is x-fastest,
 * coordinates accumulated as the reference iterator does (pos += inc).
 * pos: nn*3, conn: ne*8.  Returns 0 on success. */
int orc_make_rect_hexa(const double X0[3], const double X1[3], const uint32_t nb_points[3],
                       double *pos, uint32_t *conn);

/* Structured Tetra_10 mesh (6 tets per cube), first-creation node order of the reference.
 * Two-phase: pos == NULL or conn == NULL only returns nn and ne. */
int orc_make_rect_tetra10(const double X0[3], const double X1[3], const uint32_t nb_points[3],
                          uint64_t *nn, uint64_t *ne, double *pos, uint32_t *conn);

/* Structured Triangle_6 mesh (2 triangles per cell), pos nn*2.  Two-phase like Tetra_10. */
int orc_make_rect_triangle6(const double X0[2], const double X1[2], const uint32_t nb_points[2],
                            uint64_t *nn, uint64_t *ne, double *pos, uint32_t *conn);

/* ---------------- Gauss tables (reference C++ tables, 12-digit constants) ---------------- */
/* Returns number of points; w[np], xi[np*dim]. */
int orc_gauss_hexa_order2(double *w, double *xi);
int orc_gauss_quad_order2(double *w, double *xi);
int orc_gauss_tetra_order2(double *w, double *xi);
int orc_gauss_triangle_order2(double *w, double *xi);

/* ---------------- element matrices ---------------- */
/* Hexa8 isotropic elasticity, one Gauss point: Ke(24x24, row-major) += w*detJ*B^T (W H) B.
 * Returns detJ. */
double orc_hexa8_elast_gp(const double *xyz, double E, double nu, double w, const double *xi,
                          double *Ke);
/* Whole element (order-2 rule, 8 points). */
void orc_hexa8_elast_ke(const double *xyz, double E, double nu, double *Ke);
/* Tetra10 isotropic elasticity: one Gauss point / whole element (order 2, 4 points), Ke 30x30. */
double orc_tetra10_elast_gp(const double *xyz, double E, double nu, double w, const double *xi,
                            double *Ke);
void orc_tetra10_elast_ke(const double *xyz, double E, double nu, double *Ke);

/* recalage (formulations/formulation_recalage.py): the element Hessian (9npe x 9npe, row-major,
 * unknowns per node U, V, W then component; the Python rule of order 2), one node's nodal part
 * (9 x 9 and 9), and the assembly of both into the lower CSR of orc_pattern_lower(nn, 9, ...). */
void orc_recalage_ke(int npe, const double *xyz, double E, double nu, double rho, double gamma, double *K);
void orc_recalage_nodal(const double ud[3], double valid, double E, double r, double *Kn, double *Fn);
int orc_assemble_recalage(int npe, uint64_t nn, uint64_t ne, const double *pos, const uint32_t *conn, double E,
                          double nu, double rho, double gamma, double r, const double *Ud, const double *Uv,
                          const uint64_t *rowptr, const uint32_t *col, double *val, double *F);

/* Triangle_6 heat diffusion: stiffness a grad.grad and mass N N (6x6 each, 6-point rule). */
int orc_gauss_triangle_6pt(double *w, double *xi);
void orc_triangle6_diff_km(const double *xy, double a, double *Ke, double *Me);

/* ---------------- pattern / assembly ---------------- */
/* Structural lower pattern (node-pair product x nnu^2, j<=i).  rowptr has n+1 entries.
 * Phase 1: col==NULL returns nnz in *nnz (rowptr filled).  Phase 2 fills col. */
int orc_pattern_lower(uint64_t nn, int nnu, uint64_t ne, int npe, const uint32_t *conn,
                      uint64_t *rowptr, uint32_t *col, uint64_t *nnz);

/* Assemble elasticity K (lower CSR, pattern from orc_pattern_lower) for an element type
 * (8 = Hexa8, 10 = Tetra10).  E has ne entries (E_per_elem=1) or 1 entry. */
int orc_assemble_elast(int npe, uint64_t nn, uint64_t ne, const double *pos, const uint32_t *conn,
                       const double *E, int E_per_elem, double nu,
                       const uint64_t *rowptr, const uint32_t *col, double *val);

/* Theta-scheme matrices A = M/dt + theta K, B = M/dt - (1-theta) K on the lower pattern of a
 * Triangle_6 mesh (nnu = 1); K uses the diffusivity conductivity / rho_c (a has ne or 1 values
 * of the conductivity). */
int orc_assemble_diff(uint64_t nn, uint64_t ne, const double *pos, const uint32_t *conn,
                      const double *a, int a_per_elem, double rho_c, double dt, double theta,
                      const uint64_t *rowptr, const uint32_t *col, double *A, double *B);

/* Consistent nodal loads of a uniform traction on Quad4 faces (4 node ids per face,
 * order-2 quad rule).  F has nn*3 entries and is accumulated. */
int orc_quad4_traction(uint64_t nfaces, const uint32_t *faces, const double *pos,
                       const double traction[3], double *F);

/* Same for Triangle_6 faces (6 node ids per face), order-2 triangle rule. */
int orc_tri6_traction(uint64_t nfaces, const uint32_t *faces, const double *pos,
                      const double traction[3], double *F);

/* Penalty constraints (include/formulation/formulation.h:1028-1071): one coefficient per
 * constraint.  max|diag| is taken over the current K.  Returns max|diag|. */
double orc_penalty(uint64_t n, const uint64_t *rowptr, const uint32_t *col, double *val, double *F,
                   uint64_t nc, const uint32_t *dof, const double *coef, const double *res,
                   double penalty);

/* y = K x for the lower-stored symmetric matrix (reference partial_mul, one thread). */
void orc_spmv_sym_lower(uint64_t n, const uint64_t *rowptr, const uint32_t *col, const double *val,
                        const double *x, double *y);

/* ---------------- solvers ---------------- */
/* Dense-envelope (skyline) Cholesky solve of the lower-stored SPD matrix.  x = K^-1 b. */
int orc_skyline_solve(uint64_t n, const uint64_t *rowptr, const uint32_t *col, const double *val,
                      const double *b, double *x);

/* IC(0) factorization in place on a copy of the lower CSR (simplified variant: diagonal
 * stores 1/sqrt(d)), reference matinvsparse.h:201-261. */
void orc_ic0_factorize(uint64_t n, const uint64_t *rowptr, const uint32_t *col, double *val);
/* Forward/backward solve with the factor, reference matinvsparse.h:397-423. */
void orc_ic0_apply(uint64_t n, const uint64_t *rowptr, const uint32_t *col, const double *fac,
                   const double *r, double *z);
/* IC-PCG with true residual each iteration and |r|_inf <= crit (matinvsparse.h:453-491).
 * Returns iterations or -1 when maxit is hit. */
int orc_ic_pcg(uint64_t n, const uint64_t *rowptr, const uint32_t *col, const double *val,
               const double *fac, const double *b, double *x, double crit, int maxit);
/* Generic preconditioned CG (conjugate_gradient.h:27-68) with IC(0) preconditioner.
 * crit_kind 0: NormInfDelta on alpha*d; 1: Norm2 on alpha*d; 2: relative residual
 * |r|_2 <= crit |b|_2 (the GPU solver's criterion).  precond 0: IC(0) (fac), 1: Jacobi. */
int orc_cg(uint64_t n, const uint64_t *rowptr, const uint32_t *col, const double *val,
           const double *fac, int precond, const double *b, double *x, int crit_kind,
           double crit, int maxit);
/* The reference's 3x3-block IC(0)-PCG (MatWithTinyBlocks<double,Sym<3> >:
 * include/containers/MatWithTinyBlocks.h:224-270 construction from the Sym SparseLine lower CSR,
 * :426-520 chol_incomp, :587-720 solve_down / solve_up, :303-350 the one-thread product,
 * :1101-1150 solve_using_incomplete_chol_factorize): |r_i| <= crit for every i (absolute),
 * recursive residual.  x holds the initial guess.  Returns the number of products A d (0 when
 * the initial residual passes, -1 at maxit, -2 on a bad size); diag_out (optional, 6 per node
 * row) receives the factor's lower diagonal blocks; t_factor (construction + factorization) and
 * t_solve (the iterations) in seconds. */
int orc_tiny_block_pcg(uint64_t n, const uint64_t *rowptr, const uint32_t *col, const double *val,
                       const double *b, double *x, double crit, int maxit, double *diag_out,
                       double *t_factor, double *t_solve);
/* int_e N_a dV per element and node (ne x npe): volume-force weights. */
int orc_volume_weights(int npe, uint64_t ne, const double *pos, const uint32_t *conn, double *w);
/* Element fields after the solve at var_inter = 0.5: out ne x 13 = epsilon[6] (tensor shear,
 * 11 22 33 12 13 23), sigma[6], tr_epsilon (formulation_elasticity_iso.py:64-85). */
int orc_elem_fields(int npe, uint64_t ne, const double *pos, const uint32_t *conn, const double *E,
                    int E_per_elem, double nu0, const double *nuv, const double *u, double *out);

#ifdef __cplusplus
}
#endif
#endif
