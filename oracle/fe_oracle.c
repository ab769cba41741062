/*
 * fe_oracle.c -- CPU restatement of LMT++'s finite-element hot path (TEST INFRASTRUCTURE).
 *
 * This is the checker the GPU path is compared against, and the "port" CPU baseline.
 * It is never linked into the product library.  See fe_oracle.h for the reference
 * file:line each function restates.  Plain C99, one thread, double precision.
 */
#define _POSIX_C_SOURCE 199309L /* clock_gettime */
#include "fe_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

/* ------------------------------------------------------------------------------------------
 * Mesh: make_rect(m, Hexa(), X0, X1, nb_points)  -- include/mesh/make_rect.h:653-679.
 * Nodes are created by Rectilinear_iterator (include/util/rectilinear_iterator.h:20-45):
 * pos[0] += inc[0]; on overflow pos[0] = lower[0] and the next axis is incremented, so the
 * coordinate along each axis is an accumulated sum X0 + inc + inc + ..., x fastest.
 * ------------------------------------------------------------------------------------------ */
static int axis_coords(double x0, double x1, uint32_t nbp, double *c) {
    double lo = x0 < x1 ? x0 : x1, hi = x0 < x1 ? x1 : x0;
    double inc = (hi - lo) / ((double)nbp - 1.0);
    double step = inc + (inc == 0.0 ? 1.0 : 0.0);
    double upper = hi + step * 0.5;
    double p = lo;
    uint32_t k = 0;
    while (p < upper) {
        if (k >= nbp) return -1; /* accumulated rounding produced an extra point */
        c[k++] = p;
        p += step;
    }
    return k == nbp ? 0 : -1;
}

int orc_make_rect_hexa(const double X0[3], const double X1[3], const uint32_t nbp[3],
                       double *pos, uint32_t *conn) {
    uint32_t nx = nbp[0], ny = nbp[1], nz = nbp[2];
    if (nx < 2 || ny < 2 || nz < 2) return -1;
    double *cx = (double *)malloc(sizeof(double) * nx), *cy = (double *)malloc(sizeof(double) * ny),
           *cz = (double *)malloc(sizeof(double) * nz);
    int bad = axis_coords(X0[0], X1[0], nx, cx) | axis_coords(X0[1], X1[1], ny, cy) |
              axis_coords(X0[2], X1[2], nz, cz);
    if (!bad) {
        uint64_t n = 0;
        for (uint32_t i = 0; i < nz; ++i)
            for (uint32_t j = 0; j < ny; ++j)
                for (uint32_t k = 0; k < nx; ++k, ++n) {
                    pos[3 * n + 0] = cx[k];
                    pos[3 * n + 1] = cy[j];
                    pos[3 * n + 2] = cz[i];
                }
        uint64_t e = 0;
        uint64_t sxy = (uint64_t)nx * ny;
        for (uint32_t i = 0; i + 1 < nz; ++i)
            for (uint32_t j = 0; j + 1 < ny; ++j)
                for (uint32_t k = 0; k + 1 < nx; ++k, ++e) {
                    uint64_t b = i * sxy + (uint64_t)j * nx + k;
                    uint32_t *c = conn + 8 * e;
                    c[0] = (uint32_t)(b);
                    c[1] = (uint32_t)(b + 1);
                    c[2] = (uint32_t)(b + 1 + nx);
                    c[3] = (uint32_t)(b + nx);
                    c[4] = (uint32_t)(b + sxy);
                    c[5] = (uint32_t)(b + sxy + 1);
                    c[6] = (uint32_t)(b + sxy + 1 + nx);
                    c[7] = (uint32_t)(b + sxy + nx);
                }
    }
    free(cx);
    free(cy);
    free(cz);
    return bad ? -1 : 0;
}

/* ------------------------------------------------------------------------------------------
 * Gauss tables.  The reference's C++ tables hold 12-significant-digit abscissae
 * (include/mesh/element_Hexa.h:5-20 order 2; include/mesh/element_Quad.h:5-12 order 2), on the
 * [0,1] reference cell.  Order 2 is the first table entry >= the formulation order.
 * ------------------------------------------------------------------------------------------ */
#define GA 0.211324865405
#define GB 0.788675134595

int orc_gauss_hexa_order2(double *w, double *xi) {
    static const double t[8][3] = {{GA, GA, GA}, {GB, GA, GA}, {GB, GB, GA}, {GA, GB, GA},
                                   {GA, GA, GB}, {GB, GA, GB}, {GB, GB, GB}, {GA, GB, GB}};
    for (int g = 0; g < 8; ++g) {
        w[g] = 0.125;
        for (int d = 0; d < 3; ++d) xi[3 * g + d] = t[g][d];
    }
    return 8;
}

/* Skin faces are integrated when the reference generates add_skin_elem_matrix
 * (formal_lf/formulation.py:400-438): with the Python rule of the face element, for Quad
 * gauss_points[3] of formulations/element_Quad.py:70-75, abscissae (1 -+ sqrt(1/3))/2 at full
 * precision, weights 1/4. */
#define QA 0.21132486540518711775
#define QB 0.78867513459481288225
int orc_gauss_quad_order2(double *w, double *xi) {
    static const double t[4][2] = {{QB, QB}, {QA, QB}, {QB, QA}, {QA, QA}};
    for (int g = 0; g < 4; ++g) {
        w[g] = 0.25;
        xi[2 * g] = t[g][0];
        xi[2 * g + 1] = t[g][1];
    }
    return 4;
}

/* Tetra_10 order 2: 4 points, weights 1/24 (include/mesh/element_Tetra_10.h:5-16; 16-digit
 * abscissae), on the unit reference tetrahedron. */
#define TA 0.1381966011250105
#define TB 0.5854101966249685
int orc_gauss_tetra_order2(double *w, double *xi) {
    static const double t[4][3] = {{TA, TA, TA}, {TB, TA, TA}, {TA, TB, TA}, {TA, TA, TB}};
    for (int g = 0; g < 4; ++g) {
        w[g] = 0.041666666666666666667;
        for (int d = 0; d < 3; ++d) xi[3 * g + d] = t[g][d];
    }
    return 4;
}

/* Triangle_6 order 2: 3 edge-midpoint points, weights 1/6 (include/mesh/element_Triangle_6.h:5-15). */
int orc_gauss_triangle_order2(double *w, double *xi) {
    static const double t[3][2] = {{0.5, 0.0}, {0.5, 0.5}, {0.0, 0.5}};
    for (int g = 0; g < 3; ++g) {
        w[g] = 0.16666666666666666667;
        xi[2 * g] = t[g][0];
        xi[2 * g + 1] = t[g][1];
    }
    return 3;
}

/* ------------------------------------------------------------------------------------------
 * Hooke law: compliance (s1, s2, s3) inverted (formal_lf/material_help.py:116-134), energy
 * trace_sym_col with the factor 2 on the shear terms (include/codegen/__init__.py:82-87),
 * Voigt order [11,22,33,12,13,23] with tensor shear (include/codegen/__init__.py:23-42).
 * Returns D = W * Kglo, W = diag(1,1,1,2,2,2).
 * ------------------------------------------------------------------------------------------ */
static void inv3(const double a[3][3], double r[3][3], double *det) {
    double c00 = a[1][1] * a[2][2] - a[1][2] * a[2][1];
    double c01 = a[1][2] * a[2][0] - a[1][0] * a[2][2];
    double c02 = a[1][0] * a[2][1] - a[1][1] * a[2][0];
    double d = a[0][0] * c00 + a[0][1] * c01 + a[0][2] * c02;
    double id = 1.0 / d;
    r[0][0] = c00 * id;
    r[1][0] = c01 * id;
    r[2][0] = c02 * id;
    r[0][1] = (a[0][2] * a[2][1] - a[0][1] * a[2][2]) * id;
    r[1][1] = (a[0][0] * a[2][2] - a[0][2] * a[2][0]) * id;
    r[2][1] = (a[0][1] * a[2][0] - a[0][0] * a[2][1]) * id;
    r[0][2] = (a[0][1] * a[1][2] - a[0][2] * a[1][1]) * id;
    r[1][2] = (a[0][2] * a[1][0] - a[0][0] * a[1][2]) * id;
    r[2][2] = (a[0][0] * a[1][1] - a[0][1] * a[1][0]) * id;
    *det = d;
}

static void hooke_energy_matrix(double E, double nu, double D[6][6]) {
    double s1 = 1.0 / E, s2 = -nu / E, s3 = (1.0 + nu) / E;
    double S[3][3] = {{s1, s2, s2}, {s2, s1, s2}, {s2, s2, s1}}, K[3][3], det;
    inv3(S, K, &det);
    memset(D, 0, sizeof(double) * 36);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) D[i][j] = K[i][j];
    for (int i = 3; i < 6; ++i) D[i][i] = 2.0 * (1.0 / s3);
}

/* Trilinear shape-function derivatives on [0,1]^3 (formulations/element_Hexa.py:61-68). */
static void hexa8_dN(const double *xi, double dN[8][3]) {
    double x = xi[0], y = xi[1], z = xi[2];
    double mx = 1 - x, my = 1 - y, mz = 1 - z;
    double v[8][3] = {{-my * mz, -mx * mz, -mx * my}, {my * mz, -x * mz, -x * my},
                      {y * mz, x * mz, -x * y},      {-y * mz, mx * mz, -mx * y},
                      {-my * z, -mx * z, mx * my},   {my * z, -x * z, x * my},
                      {y * z, x * z, x * y},         {-y * z, mx * z, mx * y}};
    memcpy(dN, v, sizeof(v));
}

/* Quadratic tetrahedron shape-function derivatives (formulations/element_Tetra_10.py:27-41):
 * X0 = 1 - x - y - z, X1 = x, X2 = y, X3 = z; vertices Xi (2 Xi - 1), edges 4 Xa Xb in the
 * node order 4:(0,1) 5:(1,2) 6:(0,2) 7:(0,3) 8:(1,3) 9:(2,3). */
static void tetra10_dN(const double *xi, double dN[10][3]) {
    const double X[4] = {1 - xi[0] - xi[1] - xi[2], xi[0], xi[1], xi[2]};
    const double dX[4][3] = {{-1, -1, -1}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    for (int i = 0; i < 4; ++i)
        for (int d = 0; d < 3; ++d) dN[i][d] = (4 * X[i] - 1) * dX[i][d];
    static const int ed[6][2] = {{0, 1}, {1, 2}, {0, 2}, {0, 3}, {1, 3}, {2, 3}};
    for (int k = 0; k < 6; ++k) {
        const int a = ed[k][0], b = ed[k][1];
        for (int d = 0; d < 3; ++d) dN[4 + k][d] = 4 * (X[b] * dX[a][d] + X[a] * dX[b][d]);
    }
}

/* One Gauss point of the isotropic-elasticity weak form for an element of npe nodes with
 * reference-cell shape-function derivatives dN[npe][3]: Ke (3npe x 3npe, row-major) +=
 * w * detJ * B^T (W Kglo) B.  Returns detJ. */
static double elast_gp(int npe, const double *xyz, const double (*dN)[3], double E, double nu,
                       double w, double *Ke) {
    const int nd = 3 * npe;
    double J[3][3] = {{0}}, Ji[3][3], det, D[6][6], g[10][3];
    for (int a = 0; a < npe; ++a)
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) J[i][j] += xyz[3 * a + i] * dN[a][j];
    inv3(J, Ji, &det);
    for (int a = 0; a < npe; ++a)
        for (int i = 0; i < 3; ++i) {
            double s = 0;
            for (int j = 0; j < 3; ++j) s += Ji[j][i] * dN[a][j];
            g[a][i] = s;
        }
    hooke_energy_matrix(E, nu, D);
    double B[6][30], DB[6][30];
    memset(B, 0, sizeof(B));
    for (int a = 0; a < npe; ++a) {
        double gx = g[a][0], gy = g[a][1], gz = g[a][2];
        B[0][3 * a + 0] = gx;
        B[1][3 * a + 1] = gy;
        B[2][3 * a + 2] = gz;
        B[3][3 * a + 0] = 0.5 * gy;
        B[3][3 * a + 1] = 0.5 * gx;
        B[4][3 * a + 0] = 0.5 * gz;
        B[4][3 * a + 2] = 0.5 * gx;
        B[5][3 * a + 1] = 0.5 * gz;
        B[5][3 * a + 2] = 0.5 * gy;
    }
    for (int k = 0; k < 6; ++k)
        for (int c = 0; c < nd; ++c) {
            double s = 0;
            for (int l = 0; l < 6; ++l) s += D[k][l] * B[l][c];
            DB[k][c] = s;
        }
    double f = w * det;
    for (int r = 0; r < nd; ++r)
        for (int c = 0; c < nd; ++c) {
            double s = 0;
            for (int k = 0; k < 6; ++k) s += B[k][r] * DB[k][c];
            Ke[nd * r + c] += f * s;
        }
    return det;
}

/* Shape functions (formulations/element_Hexa.py:61-68, element_Tetra_10.py:27-41). */
static void hexa8_N(const double *xi, double N[8]) {
    const double x = xi[0], y = xi[1], z = xi[2], mx = 1 - x, my = 1 - y, mz = 1 - z;
    const double v[8] = {mx * my * mz, x * my * mz, x * y * mz, mx * y * mz,
                         mx * my * z,  x * my * z,  x * y * z,  mx * y * z};
    memcpy(N, v, sizeof(v));
}
static void tetra10_N(const double *xi, double N[10]) {
    const double X[4] = {1 - xi[0] - xi[1] - xi[2], xi[0], xi[1], xi[2]};
    for (int i = 0; i < 4; ++i) N[i] = X[i] * (2 * X[i] - 1);
    static const int ed[6][2] = {{0, 1}, {1, 2}, {0, 2}, {0, 3}, {1, 3}, {2, 3}};
    for (int k = 0; k < 6; ++k) N[4 + k] = 4 * X[ed[k][0]] * X[ed[k][1]];
}

/* w[e npe + a] = int_e N_a dV with the order-2 rules: the weights of the volume force
 * density * f_vol . te dV (formulations/formulation_elasticity_iso.py:49). */
int orc_volume_weights(int npe, uint64_t ne, const double *pos, const uint32_t *conn, double *w) {
    if (npe != 8 && npe != 10) return 1;
    double gw[8], gx[24];
    const int ng = npe == 8 ? orc_gauss_hexa_order2(gw, gx) : orc_gauss_tetra_order2(gw, gx);
    for (uint64_t e = 0; e < ne; ++e) {
        for (int a = 0; a < npe; ++a) w[(uint64_t)npe * e + a] = 0.0;
        for (int g = 0; g < ng; ++g) {
            double N[10], dN[10][3], J[3][3] = {{0}}, Ji[3][3], det;
            if (npe == 8) {
                hexa8_N(gx + 3 * g, N);
                hexa8_dN(gx + 3 * g, dN);
            } else {
                tetra10_N(gx + 3 * g, N);
                tetra10_dN(gx + 3 * g, dN);
            }
            for (int a = 0; a < npe; ++a) {
                const uint32_t n = conn[(uint64_t)npe * e + a];
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j) J[i][j] += pos[3 * (uint64_t)n + i] * dN[a][j];
            }
            inv3(J, Ji, &det);
            for (int a = 0; a < npe; ++a) w[(uint64_t)npe * e + a] += gw[g] * det * N[a];
        }
    }
    return 0;
}

/* Element fields after the solve (apply_on_elements_after_solve,
 * formulations/formulation_elasticity_iso.py:64-85): every var_inter is set to 0.5 -- the cube
 * centre for Hexa8; for Tetra10 the same point (0.5, 0.5, 0.5), which the quadratic field
 * extrapolates to -- then epsilon = grad_sym_col(dep) (tensor shear, order 11 22 33 12 13 23,
 * include/codegen/__init__.py:23-42), tr_epsilon = e11 + e22 + e33 and sigma = Kglo epsilon with
 * Kglo the inverse compliance of hooke_isotrope (formal_lf/material_help.py:116-134).
 * out: ne x 13 = epsilon[6], sigma[6], tr_epsilon.  nuv (per element) may be NULL. */
int orc_elem_fields(int npe, uint64_t ne, const double *pos, const uint32_t *conn, const double *E,
                    int E_per_elem, double nu0, const double *nuv, const double *u, double *out) {
    if (npe != 8 && npe != 10) return 1;
    const double xi[3] = {0.5, 0.5, 0.5};
    double dN[10][3];
    if (npe == 8) hexa8_dN(xi, (double (*)[3])dN);
    else tetra10_dN(xi, (double (*)[3])dN);
    for (uint64_t e = 0; e < ne; ++e) {
        double J[3][3] = {{0}}, Ji[3][3], det, gu[3][3] = {{0}};
        for (int a = 0; a < npe; ++a) {
            const uint32_t n = conn[(uint64_t)npe * e + a];
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) J[i][j] += pos[3 * (uint64_t)n + i] * dN[a][j];
        }
        inv3(J, Ji, &det);
        for (int a = 0; a < npe; ++a) {
            const uint32_t n = conn[(uint64_t)npe * e + a];
            double g[3];
            for (int i = 0; i < 3; ++i) {
                double s = 0;
                for (int j = 0; j < 3; ++j) s += Ji[j][i] * dN[a][j];
                g[i] = s;
            }
            for (int k = 0; k < 3; ++k)
                for (int i = 0; i < 3; ++i) gu[k][i] += u[3 * (uint64_t)n + k] * g[i];  /* du_k/dx_i */
        }
        double eps[6] = {gu[0][0], gu[1][1], gu[2][2], 0.5 * (gu[0][1] + gu[1][0]),
                         0.5 * (gu[0][2] + gu[2][0]), 0.5 * (gu[1][2] + gu[2][1])};
        const double Ee = E[E_per_elem ? e : 0], nu = nuv ? nuv[e] : nu0;
        double D[6][6];
        hooke_energy_matrix(Ee, nu, D);
        double *o = out + 13 * e;
        for (int k = 0; k < 6; ++k) o[k] = eps[k];
        for (int k = 0; k < 3; ++k) o[6 + k] = D[k][0] * eps[0] + D[k][1] * eps[1] + D[k][2] * eps[2];
        for (int k = 3; k < 6; ++k) o[6 + k] = 0.5 * D[k][k] * eps[k];  /* Kglo shear = (1+nu)/E inverse */
        o[12] = eps[0] + eps[1] + eps[2];
    }
    return 0;
}

double orc_hexa8_elast_gp(const double *xyz, double E, double nu, double w, const double *xi,
                          double *Ke) {
    double dN[8][3];
    hexa8_dN(xi, dN);
    return elast_gp(8, xyz, (const double(*)[3])dN, E, nu, w, Ke);
}

double orc_tetra10_elast_gp(const double *xyz, double E, double nu, double w, const double *xi,
                            double *Ke) {
    double dN[10][3];
    tetra10_dN(xi, dN);
    return elast_gp(10, xyz, (const double(*)[3])dN, E, nu, w, Ke);
}

void orc_tetra10_elast_ke(const double *xyz, double E, double nu, double *Ke) {
    double w[4], xi[12];
    memset(Ke, 0, sizeof(double) * 900);
    orc_gauss_tetra_order2(w, xi);
    for (int g = 0; g < 4; ++g) orc_tetra10_elast_gp(xyz, E, nu, w[g], xi + 3 * g, Ke);
}

void orc_hexa8_elast_ke(const double *xyz, double E, double nu, double *Ke) {
    double w[8], xi[24];
    memset(Ke, 0, sizeof(double) * 576);
    orc_gauss_hexa_order2(w, xi);
    for (int g = 0; g < 8; ++g) orc_hexa8_elast_gp(xyz, E, nu, w[g], xi + 3 * g, Ke);
}

/* ------------------------------------------------------------------------------------------
 * recalage (formulations/formulation_recalage.py:25-47): with use_test_functions = False the
 * generated routines hold the Hessian of
 *   gamma (sigma(V) - sigma(U)) : K^-1 (sigma(V) - sigma(U)) dV + (1 - gamma) rho |W - U|^2 dV
 *   + Ud_valid r / (1 - r) E |U - Ud|^2 dN
 * (formal_lf/calculate_matrix.py:4-61), unknowns per node U, V, W then component.  Since
 * K^-1 sigma = epsilon, the first term's Hessian is 2 gamma times the elasticity matrix; the
 * second's is 2 (1 - gamma) rho N_a N_b on the matching components.  The volume part is integrated
 * by the Python rule of order 2 (integration_totale, formal_lf/formulation.py:549-551): Hexa
 * gauss_points[2] (formulations/element_Hexa.py:136-146), Tetra_10 gauss_points[2]
 * (formulations/element_Tetra_10.py:107-113).
 * ------------------------------------------------------------------------------------------ */
static uint64_t find_col(const uint64_t *rowptr, const uint32_t *col, uint64_t row, uint32_t c);

static int recal_rule(int npe, double *w, double *xi) {
    if (npe == 8) {
        const double a = 1.0 / sqrt(3.0), lo = (1 - a) / 2.0, hi = (1 + a) / 2.0;
        const double p[8][3] = {{lo, lo, lo}, {hi, lo, lo}, {hi, hi, lo}, {lo, hi, lo},
                                {lo, lo, hi}, {hi, lo, hi}, {hi, hi, hi}, {lo, hi, hi}};
        for (int g = 0; g < 8; ++g) {
            w[g] = 1.0 / 8.0;
            for (int d = 0; d < 3; ++d) xi[3 * g + d] = p[g][d];
        }
        return 8;
    }
    const double a = (5.0 - sqrt(5.0)) / 20.0, b = (5.0 + 3.0 * sqrt(5.0)) / 20.0;
    const double p[4][3] = {{a, a, a}, {b, a, a}, {a, b, a}, {a, a, b}};
    for (int g = 0; g < 4; ++g) {
        w[g] = 1.0 / 24.0;
        for (int d = 0; d < 3; ++d) xi[3 * g + d] = p[g][d];
    }
    return 4;
}

void orc_recalage_ke(int npe, const double *xyz, double E, double nu, double rho, double gamma, double *K) {
    const int nd = 9 * npe, ns = 3 * npe;
    double w[8], xi[24], Ks[900], dN[10][3], N[10], M[10][10];
    const int ngp = recal_rule(npe, w, xi);
    memset(Ks, 0, sizeof(Ks));
    memset(M, 0, sizeof(M));
    for (int g = 0; g < ngp; ++g) {
        if (npe == 8) {
            hexa8_dN(xi + 3 * g, (double (*)[3])dN);
            hexa8_N(xi + 3 * g, N);
        } else {
            tetra10_dN(xi + 3 * g, (double (*)[3])dN);
            tetra10_N(xi + 3 * g, N);
        }
        const double det = elast_gp(npe, xyz, (const double (*)[3])dN, E, nu, w[g], Ks);
        for (int a = 0; a < npe; ++a)
            for (int b = 0; b < npe; ++b) M[a][b] += w[g] * det * N[a] * N[b];
    }
    const double cK = 2.0 * gamma, cM = 2.0 * (1.0 - gamma) * rho;
    memset(K, 0, sizeof(double) * nd * nd);
    for (int a = 0; a < npe; ++a)
        for (int b = 0; b < npe; ++b)
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) {
                    const double k = Ks[ns * (3 * a + i) + 3 * b + j], m = i == j ? M[a][b] : 0.0;
                    double *r0 = K + (size_t)nd * (9 * a + i), *r1 = r0 + 3 * nd, *r2 = r0 + 6 * nd;
                    const int c = 9 * b + j;
                    r0[c] = cK * k + cM * m;   /* UU */
                    r0[c + 3] = -cK * k;       /* UV */
                    r0[c + 6] = -cM * m;       /* UW */
                    r1[c] = -cK * k;           /* VU */
                    r1[c + 3] = cK * k;        /* VV */
                    r2[c] = -cM * m;           /* WU */
                    r2[c + 6] = cM * m;        /* WW */
                }
}

void orc_recalage_nodal(const double ud[3], double valid, double E, double r, double *Kn, double *Fn) {
    const double c = 2.0 * valid * r / (1.0 - r) * E;
    memset(Kn, 0, sizeof(double) * 81);
    memset(Fn, 0, sizeof(double) * 9);
    for (int d = 0; d < 3; ++d) {
        Kn[9 * d + d] = c;
        Fn[d] = c * ud[d];
    }
}

/* Scatter of the element Hessians (upper triangle, rows max(i,j) of the Sym storage) and of the
 * nodal part of every node (add_nodal_matrix) into the lower CSR pattern of nnu = 9. */
int orc_assemble_recalage(int npe, uint64_t nn, uint64_t ne, const double *pos, const uint32_t *conn, double E,
                          double nu, double rho, double gamma, double r, const double *Ud, const double *Uv,
                          const uint64_t *rowptr, const uint32_t *col, double *val, double *F) {
    if (npe != 8 && npe != 10) return -1;
    const int nd = 9 * npe;
    double xyz[30];
    double *K = (double *)malloc(sizeof(double) * nd * nd);
    if (!K) return -3;
    memset(val, 0, sizeof(double) * rowptr[nn * 9]);
    memset(F, 0, sizeof(double) * nn * 9);
    for (uint64_t e = 0; e < ne; ++e) {
        const uint32_t *c = conn + (uint64_t)npe * e;
        for (int a = 0; a < npe; ++a)
            for (int d = 0; d < 3; ++d) xyz[3 * a + d] = pos[3 * (uint64_t)c[a] + d];
        orc_recalage_ke(npe, xyz, E, nu, rho, gamma, K);
        for (int i = 0; i < nd; ++i)
            for (int j = i; j < nd; ++j) {
                const uint64_t gi = 9 * (uint64_t)c[i / 9] + i % 9, gj = 9 * (uint64_t)c[j / 9] + j % 9;
                const uint64_t row = gi > gj ? gi : gj, cl = gi > gj ? gj : gi;
                const uint64_t p = find_col(rowptr, col, row, (uint32_t)cl);
                if (p == (uint64_t)-1) {
                    free(K);
                    return -2;
                }
                val[p] += K[(size_t)nd * i + j];
            }
    }
    free(K);
    double Kn[81], Fn[9];
    for (uint64_t n = 0; n < nn; ++n) {
        orc_recalage_nodal(Ud + 3 * n, Uv[n], E, r, Kn, Fn);
        for (int p = 0; p < 9; ++p) {
            const uint64_t q = find_col(rowptr, col, 9 * n + p, (uint32_t)(9 * n + p));
            if (q == (uint64_t)-1) return -2;
            val[q] += Kn[9 * p + p];
            F[9 * n + p] += Fn[p];
        }
    }
    return 0;
}

/* ------------------------------------------------------------------------------------------
 * Structural pattern: ResizeMat::GetNZ (include/formulation/formulation.h:200-241) -- every
 * node pair (a,b) of an element gives the nnu x nnu block of DOF pairs; indice_noda[node] =
 * node * nnu (no reordering, formulation.h:283-325).  Restated lower part only.
 * ------------------------------------------------------------------------------------------ */
static int cmp_u32(const void *a, const void *b) {
    uint32_t x = *(const uint32_t *)a, y = *(const uint32_t *)b;
    return x < y ? -1 : x > y;
}

/* node adjacency (sorted, unique, includes self) */
static int node_adjacency(uint64_t nn, uint64_t ne, int npe, const uint32_t *conn,
                          uint64_t **nptr_out, uint32_t **nbr_out) {
    uint64_t *cnt = (uint64_t *)calloc(nn + 1, sizeof(uint64_t));
    for (uint64_t e = 0; e < ne; ++e)
        for (int a = 0; a < npe; ++a) cnt[conn[e * npe + a] + 1] += (uint64_t)npe;
    for (uint64_t i = 0; i < nn; ++i) cnt[i + 1] += cnt[i];
    uint32_t *tmp = (uint32_t *)malloc(sizeof(uint32_t) * (cnt[nn] ? cnt[nn] : 1));
    uint64_t *cur = (uint64_t *)malloc(sizeof(uint64_t) * (nn ? nn : 1));
    for (uint64_t i = 0; i < nn; ++i) cur[i] = cnt[i];
    for (uint64_t e = 0; e < ne; ++e)
        for (int a = 0; a < npe; ++a) {
            uint32_t na = conn[e * npe + a];
            for (int b = 0; b < npe; ++b) tmp[cur[na]++] = conn[e * npe + b];
        }
    uint64_t *nptr = (uint64_t *)calloc(nn + 1, sizeof(uint64_t));
    uint64_t w = 0;
    for (uint64_t i = 0; i < nn; ++i) {
        uint64_t b = cnt[i], e = cnt[i + 1];
        qsort(tmp + b, (size_t)(e - b), sizeof(uint32_t), cmp_u32);
        nptr[i] = w;
        if (e == b) { /* isolated node: diagonal only */
            tmp[w++] = (uint32_t)i;
            continue;
        }
        uint32_t last = 0xffffffffu;
        for (uint64_t k = b; k < e; ++k)
            if (tmp[k] != last) last = tmp[w++] = tmp[k];
    }
    nptr[nn] = w;
    free(cnt);
    free(cur);
    *nptr_out = nptr;
    *nbr_out = tmp;
    return 0;
}

int orc_pattern_lower(uint64_t nn, int nnu, uint64_t ne, int npe, const uint32_t *conn,
                      uint64_t *rowptr, uint32_t *col, uint64_t *nnz) {
    uint64_t *nptr;
    uint32_t *nbr;
    node_adjacency(nn, ne, npe, conn, &nptr, &nbr);
    uint64_t w = 0;
    rowptr[0] = 0;
    for (uint64_t i = 0; i < nn; ++i)
        for (int c = 0; c < nnu; ++c) {
            uint64_t row = i * nnu + c;
            for (uint64_t k = nptr[i]; k < nptr[i + 1]; ++k) {
                uint32_t j = nbr[k];
                for (int d = 0; d < nnu; ++d) {
                    uint64_t cl = (uint64_t)j * nnu + d;
                    if (cl > row) break;
                    if (col) col[w] = (uint32_t)cl;
                    ++w;
                }
            }
            rowptr[row + 1] = w;
        }
    *nnz = w;
    free(nptr);
    free(nbr);
    return 0;
}

static uint64_t find_col(const uint64_t *rowptr, const uint32_t *col, uint64_t row, uint32_t c) {
    uint64_t lo = rowptr[row], hi = rowptr[row + 1];
    while (lo < hi) {
        uint64_t mid = (lo + hi) / 2;
        if (col[mid] < c) lo = mid + 1;
        else hi = mid;
    }
    return (lo < rowptr[row + 1] && col[lo] == c) ? lo : (uint64_t)-1;
}

/* Scatter: the generated code emits matrix(i,j) += tmp_i_j for j >= i (symmetric) and the
 * Sym matrix stores it in row max(i,j) (formal_lf/calculate_matrix.py:86-98,
 * include/containers/matsparse.h:757-770).  Contributions are scattered per Gauss point, as
 * add_elem_matrix calls add_local_elem_matrix once per point (formulation.h:2918-2932). */
int orc_assemble_elast(int npe, uint64_t nn, uint64_t ne, const double *pos, const uint32_t *conn,
                       const double *E, int E_per_elem, double nu,
                       const uint64_t *rowptr, const uint32_t *col, double *val) {
    (void)nn;
    if (npe != 8 && npe != 10) return -1;
    const int nd = 3 * npe;
    double w[8], xi[24];
    const int ngp = npe == 8 ? orc_gauss_hexa_order2(w, xi) : orc_gauss_tetra_order2(w, xi);
    memset(val, 0, sizeof(double) * rowptr[nn * 3]);
    double xyz[30], Ke[900];
    for (uint64_t e = 0; e < ne; ++e) {
        const uint32_t *c = conn + (uint64_t)npe * e;
        for (int a = 0; a < npe; ++a)
            for (int d = 0; d < 3; ++d) xyz[3 * a + d] = pos[3 * (uint64_t)c[a] + d];
        double Ee = E[E_per_elem ? e : 0];
        for (int g = 0; g < ngp; ++g) {
            memset(Ke, 0, sizeof(Ke));
            if (npe == 8) orc_hexa8_elast_gp(xyz, Ee, nu, w[g], xi + 3 * g, Ke);
            else orc_tetra10_elast_gp(xyz, Ee, nu, w[g], xi + 3 * g, Ke);
            for (int r = 0; r < nd; ++r)
                for (int s = r; s < nd; ++s) {
                    uint64_t gi = (uint64_t)c[r / 3] * 3 + r % 3, gj = (uint64_t)c[s / 3] * 3 + s % 3;
                    uint64_t row = gi > gj ? gi : gj, cl = gi > gj ? gj : gi;
                    uint64_t p = find_col(rowptr, col, row, (uint32_t)cl);
                    if (p == (uint64_t)-1) return -2;
                    val[p] += Ke[nd * r + s];
                }
        }
    }
    return 0;
}

/* Consistent loads of a uniform f_surf on Quad4 skin faces: the dS term of
 * formulations/formulation_elasticity_iso.py:60, V_i = int N_i t dS (formal_lf/calculate_matrix.py
 * sign convention V = -residual at u = 0). */
int orc_quad4_traction(uint64_t nfaces, const uint32_t *faces, const double *pos,
                       const double t[3], double *F) {
    double w[4], xi[8];
    orc_gauss_quad_order2(w, xi);
    for (uint64_t f = 0; f < nfaces; ++f) {
        const uint32_t *q = faces + 4 * f;
        for (int g = 0; g < 4; ++g) {
            double u = xi[2 * g], v = xi[2 * g + 1];
            double N[4] = {(1 - u) * (1 - v), u * (1 - v), u * v, (1 - u) * v};
            double dNu[4] = {-(1 - v), (1 - v), v, -v};
            double dNv[4] = {-(1 - u), -u, u, (1 - u)};
            double tu[3] = {0, 0, 0}, tv[3] = {0, 0, 0};
            for (int a = 0; a < 4; ++a)
                for (int d = 0; d < 3; ++d) {
                    tu[d] += pos[3 * (uint64_t)q[a] + d] * dNu[a];
                    tv[d] += pos[3 * (uint64_t)q[a] + d] * dNv[a];
                }
            double nx = tu[1] * tv[2] - tu[2] * tv[1], ny = tu[2] * tv[0] - tu[0] * tv[2],
                   nz = tu[0] * tv[1] - tu[1] * tv[0];
            double ds = sqrt(nx * nx + ny * ny + nz * nz) * w[g];
            for (int a = 0; a < 4; ++a)
                for (int d = 0; d < 3; ++d) F[3 * (uint64_t)q[a] + d] += N[a] * t[d] * ds;
        }
    }
    return 0;
}

/* include/formulation/formulation.h:1028-1071: max_diag = max|diag K|; for each penalty
 * constraint C = coeff * max_diag * penalty; F[j] += C * res; K(j,j) += C * coeff. */
double orc_penalty(uint64_t n, const uint64_t *rowptr, const uint32_t *col, double *val, double *F,
                   uint64_t nc, const uint32_t *dof, const double *coef, const double *res,
                   double penalty) {
    (void)col;
    double md = 0;
    for (uint64_t i = 0; i < n; ++i) {
        double d = fabs(val[rowptr[i + 1] - 1]);
        if (d > md) md = d;
    }
    for (uint64_t k = 0; k < nc; ++k) {
        double C = coef[k] * md * penalty;
        if (F) F[dof[k]] += C * res[k];
        val[rowptr[dof[k] + 1] - 1] += C * coef[k];
    }
    return md;
}

/* include/containers/matsparse.h:5368-5408 (partial_mul with one thread). */
void orc_spmv_sym_lower(uint64_t n, const uint64_t *rowptr, const uint32_t *col, const double *val,
                        const double *x, double *y) {
    memset(y, 0, sizeof(double) * n);
    for (uint64_t i = 0; i < n; ++i) {
        double r = 0;
        uint64_t b = rowptr[i], e = rowptr[i + 1];
        if (e == b) continue;
        uint64_t j;
        for (j = b; j + 1 < e; ++j) {
            r += val[j] * x[col[j]];
            y[col[j]] += val[j] * x[i];
        }
        r += val[j] * x[col[j]];
        y[i] += r;
    }
}

/* ------------------------------------------------------------------------------------------
 * make_rect(m, Tetra_10(), X0, X1, nb_points) -- include/mesh/make_rect.h:443-545.  Each cube
 * (i,j,k) of the grid (x fastest) is split into 6 tetrahedra; node t of tetrahedron s sits at
 * O + tr_s + incr * (chgt_s * rela_t), O = X0 + (k incr0, j incr1, i incr2), and nodes are
 * de-duplicated in first-creation order (BestialNodeAdder, make_rect.h:26-39; here the point's
 * exact half-grid coordinates replace the O(N^2) distance search -- same order, same first
 * stored position).  A tetrahedron with a negative Jacobian is renumbered
 * [0,1,3,2,4,8,7,6,5,9] (permutation_if_jac_neg, include/mesh/element_Tetra_10.h:122-130).
 * ------------------------------------------------------------------------------------------ */
int orc_make_rect_tetra10(const double X0_[3], const double X1_[3], const uint32_t nbp[3],
                          uint64_t *nn_out, uint64_t *ne_out, double *pos, uint32_t *conn) {
    static const double rela[10][3] = {{0, 0, 0},     {1, 0, 0},     {0, 1, 0},   {0, 0, 1},
                                       {0.5, 0, 0},   {0.5, 0.5, 0}, {0, 0.5, 0}, {0, 0, 0.5},
                                       {0.5, 0, 0.5}, {0, 0.5, 0.5}};
    /* translation (in units of incr) and basis columns of the 6 tetrahedra */
    static const int trs[6][3] = {{0, 0, 0}, {1, 1, 0}, {1, 0, 0}, {1, 0, 1}, {1, 1, 0}, {1, 1, 1}};
    static const int bas[6][3][3] = {{{1, 0, 0}, {0, 1, 0}, {0, 0, 1}},
                                     {{-1, 0, 0}, {0, -1, 0}, {0, -1, 1}},
                                     {{-1, 0, 1}, {-1, 1, 0}, {0, 0, 1}},
                                     {{-1, 0, 0}, {-1, 1, 0}, {-1, 1, -1}},
                                     {{-1, 0, 0}, {-1, 0, 1}, {0, -1, 1}},
                                     {{-1, 0, 0}, {0, -1, 0}, {0, 0, -1}}};
    uint32_t ne3[3];
    double X0[3], X1[3], incr[3];
    for (int d = 0; d < 3; ++d) {
        if (nbp[d] < 2) return -1;
        X0[d] = X0_[d] < X1_[d] ? X0_[d] : X1_[d];
        X1[d] = X0_[d] < X1_[d] ? X1_[d] : X0_[d];
        ne3[d] = nbp[d] - 1;
        incr[d] = (X1[d] - X0[d]) / ne3[d];
    }
    const uint64_t gx = 2ull * ne3[0] + 1, gy = 2ull * ne3[1] + 1, gz = 2ull * ne3[2] + 1;
    const uint64_t nn = gx * gy * gz, ne = 6ull * ne3[0] * ne3[1] * ne3[2];
    *nn_out = nn;
    *ne_out = ne;
    if (!pos || !conn) return 0;
    uint32_t *id = (uint32_t *)malloc(sizeof(uint32_t) * nn);
    for (uint64_t q = 0; q < nn; ++q) id[q] = 0xffffffffu;
    uint32_t next = 0;
    uint64_t e = 0;
    for (uint32_t i = 0; i < ne3[2]; ++i)
        for (uint32_t j = 0; j < ne3[1]; ++j)
            for (uint32_t k = 0; k < ne3[0]; ++k) {
                const double O[3] = {X0[0] + k * incr[0], X0[1] + j * incr[1], X0[2] + i * incr[2]};
                for (int s = 0; s < 6; ++s) {
                    uint32_t vn[10];
                    double vp[10][3];
                    for (int t = 0; t < 10; ++t) {
                        double wv[3];
                        for (int r = 0; r < 3; ++r)
                            wv[r] = bas[s][0][r] * rela[t][0] + bas[s][1][r] * rela[t][1] +
                                    bas[s][2][r] * rela[t][2];
                        double p[3];
                        int64_t g[3];
                        const uint32_t kk[3] = {k, j, i};
                        for (int r = 0; r < 3; ++r) {
                            const double base = s == 0 ? O[r] : O[r] + trs[s][r] * incr[r];
                            p[r] = base + incr[r] * wv[r];
                            g[r] = 2 * (int64_t)kk[r] + 2 * trs[s][r] + (int64_t)llround(2 * wv[r]);
                        }
                        const uint64_t key = ((uint64_t)g[2] * gy + (uint64_t)g[1]) * gx + (uint64_t)g[0];
                        if (id[key] == 0xffffffffu) {
                            id[key] = next;
                            for (int r = 0; r < 3; ++r) pos[3ull * next + r] = p[r];
                            ++next;
                        }
                        vn[t] = id[key];
                        for (int r = 0; r < 3; ++r) vp[t][r] = pos[3ull * vn[t] + r];
                    }
                    /* sign of the Jacobian from the vertex positions */
                    double a[3], b[3], c[3];
                    for (int r = 0; r < 3; ++r) {
                        a[r] = vp[1][r] - vp[0][r];
                        b[r] = vp[2][r] - vp[0][r];
                        c[r] = vp[3][r] - vp[0][r];
                    }
                    const double det = a[0] * (b[1] * c[2] - b[2] * c[1]) -
                                       a[1] * (b[0] * c[2] - b[2] * c[0]) +
                                       a[2] * (b[0] * c[1] - b[1] * c[0]);
                    static const int perm[10] = {0, 1, 3, 2, 4, 8, 7, 6, 5, 9};
                    for (int t = 0; t < 10; ++t) conn[10 * e + t] = det < 0 ? vn[perm[t]] : vn[t];
                    ++e;
                }
            }
    free(id);
    return next == nn ? 0 : -2;
}

int orc_gauss_triangle_6pt(double *w, double *xi);

/* Consistent loads of a uniform traction on Triangle_6 faces (6 node ids per face: vertices
 * then mid-edges (01),(12),(20)), with the Python rule the generated skin routines integrate by
 * (formal_lf/formulation.py:400-438; gauss_points[4] of formulations/element_Triangle_6.py:92-99). */
int orc_tri6_traction(uint64_t nfaces, const uint32_t *faces, const double *pos, const double t[3],
                      double *F) {
    double w[6], xi[12];
    orc_gauss_triangle_6pt(w, xi);
    for (uint64_t f = 0; f < nfaces; ++f) {
        const uint32_t *q = faces + 6 * f;
        for (int g = 0; g < 6; ++g) {
            const double u = xi[2 * g], v = xi[2 * g + 1], X0 = 1 - u - v;
            const double N[6] = {X0 * (2 * X0 - 1), u * (2 * u - 1), v * (2 * v - 1),
                                 4 * X0 * u,        4 * u * v,       4 * v * X0};
            const double dNu[6] = {-(4 * X0 - 1), 4 * u - 1, 0, 4 * (X0 - u), 4 * v, -4 * v};
            const double dNv[6] = {-(4 * X0 - 1), 0, 4 * v - 1, -4 * u, 4 * u, 4 * (X0 - v)};
            double tu[3] = {0, 0, 0}, tv[3] = {0, 0, 0};
            for (int a = 0; a < 6; ++a)
                for (int d = 0; d < 3; ++d) {
                    tu[d] += pos[3 * (uint64_t)q[a] + d] * dNu[a];
                    tv[d] += pos[3 * (uint64_t)q[a] + d] * dNv[a];
                }
            const double nx = tu[1] * tv[2] - tu[2] * tv[1], ny = tu[2] * tv[0] - tu[0] * tv[2],
                         nz = tu[0] * tv[1] - tu[1] * tv[0];
            const double ds = sqrt(nx * nx + ny * ny + nz * nz) * w[g];
            for (int a = 0; a < 6; ++a)
                for (int d = 0; d < 3; ++d) F[3 * (uint64_t)q[a] + d] += N[a] * t[d] * ds;
        }
    }
    return 0;
}

/* ------------------------------------------------------------------------------------------
 * Heat diffusion (formulations/formulation_difftherm.py:24-30) on Triangle_6.
 * make_rect(m, Triangle_6(), X0, X1, nb_points) -- include/mesh/make_rect.h:141-170: nodes on
 * the (2 nx - 1) x (2 ny - 1) half-step grid created by Rectilinear_iterator (accumulated
 * coordinates, x fastest), incr = (X1 - X0) / (nb_points - 1) * 0.5; two triangles per cell.
 * ------------------------------------------------------------------------------------------ */
int orc_make_rect_triangle6(const double X0_[2], const double X1_[2], const uint32_t nbp[2],
                            uint64_t *nn_out, uint64_t *ne_out, double *pos, uint32_t *conn) {
    const uint32_t nx = nbp[0], ny = nbp[1];
    if (nx < 2 || ny < 2) return -1;
    const uint64_t gx = 2ull * nx - 1, gy = 2ull * ny - 1;
    *nn_out = gx * gy;
    *ne_out = 2ull * (nx - 1) * (ny - 1);
    if (!pos || !conn) return 0;
    double c[2][8192 * 2];
    uint64_t cnt[2] = {0, 0};
    for (int d = 0; d < 2; ++d) {
        const double lo = X0_[d] < X1_[d] ? X0_[d] : X1_[d], hi = X0_[d] < X1_[d] ? X1_[d] : X0_[d];
        const double inc = (hi - lo) / ((double)nbp[d] - 1.0) * .5;
        const double step = inc + (inc == 0.0 ? 1.0 : 0.0), upper = hi + step * 0.5;
        for (double p = lo; p < upper; p += step) {
            if (cnt[d] >= (d ? gy : gx) || cnt[d] >= 16384) return -1;
            c[d][cnt[d]++] = p;
        }
    }
    if (cnt[0] != gx || cnt[1] != gy) return -1;
    uint64_t n = 0;
    for (uint64_t j = 0; j < gy; ++j)
        for (uint64_t i = 0; i < gx; ++i, ++n) {
            pos[2 * n] = c[0][i];
            pos[2 * n + 1] = c[1][j];
        }
    uint64_t e = 0;
    for (uint64_t i = 0; i + 1 < ny; ++i)
        for (uint64_t j = 0; j + 1 < nx; ++j) {
            const uint64_t b = 2 * i * (2 * nx - 1) + 2 * j, r = 2 * nx - 1;
            const uint64_t p[9] = {b, b + 1, b + 2, b + r, b + 1 + r, b + 2 + r, b + 2 * r, b + 1 + 2 * r, b + 2 + 2 * r};
            const uint64_t t1[6] = {p[0], p[2], p[6], p[1], p[4], p[3]};
            const uint64_t t2[6] = {p[2], p[8], p[6], p[5], p[7], p[4]};
            for (int a = 0; a < 6; ++a) conn[6 * e + a] = (uint32_t)t1[a];
            ++e;
            for (int a = 0; a < 6; ++a) conn[6 * e + a] = (uint32_t)t2[a];
            ++e;
        }
    return 0;
}

/* 6-point rule of the Python element description used when the formulation integrates the
 * element in closed form (integration_totale, formulations/element_Triangle_6.py:92-99). */
int orc_gauss_triangle_6pt(double *w, double *xi) {
    const double a = 0.445948490915965, b = 0.091576213509771;
    const double wa = 0.111690794839005, wb = 0.054975871827661;
    const double t[6][3] = {{wa, a, a}, {wa, 1.0 - 2.0 * a, a}, {wa, a, 1.0 - 2.0 * a},
                            {wb, b, b}, {wb, 1.0 - 2.0 * b, b}, {wb, b, 1.0 - 2.0 * b}};
    for (int g = 0; g < 6; ++g) {
        w[g] = t[g][0];
        xi[2 * g] = t[g][1];
        xi[2 * g + 1] = t[g][2];
    }
    return 6;
}

static void tri6_shape(double u, double v, double N[6], double dN[6][2]) {
    const double X0 = 1 - u - v;
    N[0] = X0 * (2 * X0 - 1); N[1] = u * (2 * u - 1); N[2] = v * (2 * v - 1);
    N[3] = 4 * X0 * u;        N[4] = 4 * u * v;       N[5] = 4 * v * X0;
    dN[0][0] = -(4 * X0 - 1); dN[0][1] = -(4 * X0 - 1);
    dN[1][0] = 4 * u - 1;     dN[1][1] = 0;
    dN[2][0] = 0;             dN[2][1] = 4 * v - 1;
    dN[3][0] = 4 * (X0 - u);  dN[3][1] = -4 * u;
    dN[4][0] = 4 * v;         dN[4][1] = 4 * u;
    dN[5][0] = -4 * v;        dN[5][1] = 4 * (X0 - v);
}

/* Element matrices of the diffusion weak form a grad T . grad v + T' v: stiffness
 * Ke = int a gradN_i . gradN_j (a = conductivity / (density * heat capacity), given directly)
 * and mass Me = int N_i N_j, both 6x6 row-major. */
void orc_triangle6_diff_km(const double *xy, double a, double *Ke, double *Me) {
    double w[6], xi[12];
    orc_gauss_triangle_6pt(w, xi);
    memset(Ke, 0, sizeof(double) * 36);
    memset(Me, 0, sizeof(double) * 36);
    for (int g = 0; g < 6; ++g) {
        double N[6], dN[6][2];
        tri6_shape(xi[2 * g], xi[2 * g + 1], N, dN);
        double J[2][2] = {{0, 0}, {0, 0}};
        for (int k = 0; k < 6; ++k)
            for (int i = 0; i < 2; ++i)
                for (int j = 0; j < 2; ++j) J[i][j] += xy[2 * k + i] * dN[k][j];
        const double det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
        const double Ji[2][2] = {{J[1][1] / det, -J[0][1] / det}, {-J[1][0] / det, J[0][0] / det}};
        double gx[6][2];
        for (int k = 0; k < 6; ++k)
            for (int i = 0; i < 2; ++i) gx[k][i] = Ji[0][i] * dN[k][0] + Ji[1][i] * dN[k][1];
        const double f = w[g] * det;
        for (int i = 0; i < 6; ++i)
            for (int j = 0; j < 6; ++j) {
                Ke[6 * i + j] += f * a * (gx[i][0] * gx[j][0] + gx[i][1] * gx[j][1]);
                Me[6 * i + j] += f * N[i] * N[j];
            }
    }
}

/* Theta-scheme matrices A = M/dt + theta K and B = M/dt - (1-theta) K on the structural lower
 * pattern (nnu = 1).  theta = 1/2 is the reference's time integration: the residual evaluated
 * at the midpoint of [t_n, t_n+1] with the unknown interpolated linearly
 * (formal_lf/formulation.py:506-509, formal_lf/extrapolation.py:21-40,
 * formal_lf/gauss_integration.py:52-63, left/right_time_integration 0/1). */
int orc_assemble_diff(uint64_t nn, uint64_t ne, const double *pos, const uint32_t *conn,
                      const double *a, int a_per_elem, double rho_c, double dt, double theta,
                      const uint64_t *rowptr, const uint32_t *col, double *A, double *B) {
    memset(A, 0, sizeof(double) * rowptr[nn]);
    memset(B, 0, sizeof(double) * rowptr[nn]);
    double xy[12], Ke[36], Me[36];
    for (uint64_t e = 0; e < ne; ++e) {
        const uint32_t *c = conn + 6 * e;
        for (int k = 0; k < 6; ++k) {
            xy[2 * k] = pos[2 * (uint64_t)c[k]];
            xy[2 * k + 1] = pos[2 * (uint64_t)c[k] + 1];
        }
        /* diffusivity a = conductivity / (density * heat capacity) (formulation_difftherm.py:25) */
        orc_triangle6_diff_km(xy, a[a_per_elem ? e : 0] / rho_c, Ke, Me);
        for (int i = 0; i < 6; ++i)
            for (int j = 0; j < 6; ++j) {
                const uint64_t r = c[i], s = c[j];
                if (s > r) continue;
                const uint64_t p = find_col(rowptr, col, r, (uint32_t)s);
                if (p == (uint64_t)-1) return -2;
                A[p] += Me[6 * i + j] / dt + theta * Ke[6 * i + j];
                B[p] += Me[6 * i + j] / dt - (1.0 - theta) * Ke[6 * i + j];
            }
    }
    return 0;
}

/* ------------------------------------------------------------------------------------------
 * Skyline (envelope) Cholesky, used as the oracle's direct solver in place of the vendored
 * LDL (include/util/solveLDL.cpp:44-125): same factorization mathematics, no ordering.
 * ------------------------------------------------------------------------------------------ */
int orc_skyline_solve(uint64_t n, const uint64_t *rowptr, const uint32_t *col, const double *val,
                      const double *b, double *x) {
    uint64_t *first = (uint64_t *)malloc(sizeof(uint64_t) * (n ? n : 1));
    uint64_t *off = (uint64_t *)malloc(sizeof(uint64_t) * (n + 1));
    off[0] = 0;
    for (uint64_t i = 0; i < n; ++i) {
        first[i] = rowptr[i + 1] > rowptr[i] ? col[rowptr[i]] : i;
        off[i + 1] = off[i] + (i - first[i] + 1);
    }
    double *L = (double *)calloc(off[n] ? off[n] : 1, sizeof(double));
    if (!L) {
        free(first);
        free(off);
        return -1;
    }
    for (uint64_t i = 0; i < n; ++i)
        for (uint64_t k = rowptr[i]; k < rowptr[i + 1]; ++k)
            L[off[i] + (col[k] - first[i])] = val[k];
    int rc = 0;
    for (uint64_t i = 0; i < n && !rc; ++i) {
        double *Li = L + off[i];
        for (uint64_t j = first[i]; j < i; ++j) {
            const double *Lj = L + off[j];
            uint64_t k0 = first[i] > first[j] ? first[i] : first[j];
            double s = Li[j - first[i]];
            for (uint64_t k = k0; k < j; ++k) s -= Li[k - first[i]] * Lj[k - first[j]];
            Li[j - first[i]] = s / Lj[j - first[j]];
        }
        double d = Li[i - first[i]];
        for (uint64_t k = first[i]; k < i; ++k) d -= Li[k - first[i]] * Li[k - first[i]];
        if (!(d > 0)) rc = -2;
        Li[i - first[i]] = sqrt(d);
    }
    if (!rc) {
        for (uint64_t i = 0; i < n; ++i) {
            double s = b[i];
            const double *Li = L + off[i];
            for (uint64_t k = first[i]; k < i; ++k) s -= Li[k - first[i]] * x[k];
            x[i] = s / Li[i - first[i]];
        }
        for (uint64_t ii = n; ii-- > 0;) {
            const double *Li = L + off[ii];
            x[ii] /= Li[ii - first[ii]];
            for (uint64_t k = first[ii]; k < ii; ++k) x[k] -= Li[k - first[ii]] * x[ii];
        }
    }
    free(L);
    free(first);
    free(off);
    return rc;
}

/* ------------------------------------------------------------------------------------------
 * IC(0) -- include/containers/matinvsparse.h:201-261 (simplified variant: the diagonal holds
 * 1/sqrt(d)); dot_chol_factorize matinvsparse.h:23-34.
 * ------------------------------------------------------------------------------------------ */
static double dot_chol(const uint64_t *rowptr, const uint32_t *col, const double *v, uint64_t r1,
                       uint64_t r2) {
    double res = 0;
    uint64_t b1 = rowptr[r1], e1 = rowptr[r1 + 1], b2 = rowptr[r2], e2 = rowptr[r2 + 1];
    if (e2 == b2) return 0;
    uint64_t j = b2;
    for (uint64_t i = b1; i + 1 < e1; ++i) {
        while (col[j] < col[i]) {
            ++j;
            if (j == e2) return res;
        }
        if (col[j] == col[i]) res += v[j] * v[i];
    }
    return res;
}

void orc_ic0_factorize(uint64_t n, const uint64_t *rowptr, const uint32_t *col, double *v) {
    for (uint64_t line = 0; line < n; ++line) {
        uint64_t b = rowptr[line], e = rowptr[line + 1];
        for (uint64_t ind = b; ind + 1 < e; ++ind) {
            uint32_t c = col[ind];
            v[ind] = (v[ind] - dot_chol(rowptr, col, v, c, line)) * v[rowptr[c + 1] - 1];
        }
        double d = v[e - 1];
        for (uint64_t k = b; k + 1 < e; ++k) d -= v[k] * v[k];
        v[e - 1] = 1.0 / sqrt(fabs(d) + (d == 0.0));
    }
}

void orc_ic0_apply(uint64_t n, const uint64_t *rowptr, const uint32_t *col, const double *fac,
                   const double *r, double *z) {
    for (uint64_t line = 0; line < n; ++line) {
        double v = r[line];
        uint64_t b = rowptr[line], e = rowptr[line + 1];
        for (uint64_t k = b; k + 1 < e; ++k) v -= fac[k] * z[col[k]];
        z[line] = v * fac[e - 1];
    }
    double *tmp = (double *)malloc(sizeof(double) * (n ? n : 1));
    memcpy(tmp, z, sizeof(double) * n);
    for (uint64_t line = n; line-- > 0;) {
        uint64_t b = rowptr[line], e = rowptr[line + 1];
        double t = tmp[line] * fac[e - 1];
        for (uint64_t k = b; k + 1 < e; ++k) tmp[col[k]] -= fac[k] * t;
        z[line] = t;
    }
    free(tmp);
}

static double dotv(uint64_t n, const double *a, const double *b) {
    double s = 0;
    for (uint64_t i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
}

int orc_ic_pcg(uint64_t n, const uint64_t *rowptr, const uint32_t *col, const double *val,
               const double *fac, const double *b, double *x, double crit, int maxit) {
    double *r = (double *)malloc(8 * n), *d = (double *)malloc(8 * n), *q = (double *)malloc(8 * n),
           *s = (double *)malloc(8 * n);
    int ret = -1;
    orc_spmv_sym_lower(n, rowptr, col, val, x, q);
    for (uint64_t i = 0; i < n; ++i) r[i] = b[i] - q[i];
    uint64_t i;
    for (i = 0; i < n; ++i)
        if (fabs(r[i]) > fabs(crit)) break;
    if (i == n) {
        ret = 0;
        goto done;
    }
    orc_ic0_apply(n, rowptr, col, fac, r, d);
    double deltn = dotv(n, r, d);
    for (int cpt = 0; cpt < maxit;) {
        double delto = deltn;
        orc_spmv_sym_lower(n, rowptr, col, val, d, q);
        double alpha = deltn / dotv(n, d, q);
        for (uint64_t k = 0; k < n; ++k) x[k] += alpha * d[k];
        orc_spmv_sym_lower(n, rowptr, col, val, x, q); /* true residual, as the reference */
        for (uint64_t k = 0; k < n; ++k) r[k] = b[k] - q[k];
        for (i = 0; i < n; ++i)
            if (fabs(r[i]) > fabs(crit)) break;
        if (i == n) {
            ret = cpt;
            goto done;
        }
        orc_ic0_apply(n, rowptr, col, fac, r, s);
        deltn = dotv(n, r, s);
        double beta = deltn / delto;
        for (uint64_t k = 0; k < n; ++k) d[k] = s[k] + beta * d[k];
        ++cpt;
    }
done:
    free(r);
    free(d);
    free(q);
    free(s);
    return ret;
}

int orc_cg(uint64_t n, const uint64_t *rowptr, const uint32_t *col, const double *val,
           const double *fac, int precond, const double *b, double *x, int crit_kind, double crit,
           int maxit) {
    double *r = (double *)malloc(8 * n), *d = (double *)malloc(8 * n), *q = (double *)malloc(8 * n),
           *s = (double *)malloc(8 * n);
    orc_spmv_sym_lower(n, rowptr, col, val, x, q);
    for (uint64_t i = 0; i < n; ++i) r[i] = b[i] - q[i];
    double bn = sqrt(dotv(n, b, b));
    int ret = -1;
    if (crit_kind == 2 && sqrt(dotv(n, r, r)) <= crit * bn) {
        ret = 0;
        goto done;
    }
#define PREC(in, out)                                                                              \
    do {                                                                                           \
        if (precond == 0) orc_ic0_apply(n, rowptr, col, fac, in, out);                             \
        else                                                                                       \
            for (uint64_t k = 0; k < n; ++k) out[k] = in[k] / val[rowptr[k + 1] - 1];              \
    } while (0)
    PREC(r, d);
    double deltn = dotv(n, r, d);
    for (int cpt = 1; cpt <= maxit; ++cpt) {
        double delto = deltn;
        orc_spmv_sym_lower(n, rowptr, col, val, d, q);
        double dq = dotv(n, d, q);
        double alpha = deltn / (dq + (dq == 0));
        double ninf = 0, n2 = 0;
        for (uint64_t k = 0; k < n; ++k) {
            double dx = alpha * d[k];
            x[k] += dx;
            r[k] -= alpha * q[k];
            if (fabs(dx) > ninf) ninf = fabs(dx);
            n2 += dx * dx;
        }
        int conv = crit_kind == 0   ? ninf <= crit
                   : crit_kind == 1 ? sqrt(n2) < crit
                                    : sqrt(dotv(n, r, r)) <= crit * bn;
        if (conv) {
            ret = cpt;
            goto done;
        }
        PREC(r, s);
        deltn = dotv(n, r, s);
        double beta = deltn / delto;
        for (uint64_t k = 0; k < n; ++k) d[k] = s[k] + beta * d[k];
    }
#undef PREC
done:
    free(r);
    free(d);
    free(q);
    free(s);
    return ret;
}

/* ------------------------------------------------------------------------------------------
 * 3x3-block IC(0) preconditioned CG of the reference, MatWithTinyBlocks<double,Sym<3> >
 * (include/containers/MatWithTinyBlocks.h): the reference's fastest CPU iterative path for
 * 3-DOF problems (its documentation times it at 3x the scalar IC-PCG,
 * include/mesh/exemple_probleme_elastique.txt:228-231).  TEST INFRASTRUCTURE: the CPU baseline.
 *
 * Storage: node row R holds its strictly-lower 3x3 blocks in ascending block column (the
 * reference's RowOfMatWithTinyBlocks) and a lower-stored diagonal block d00 d10 d11 d20 d21 d22
 * (DB, data[r (r + 1) / 2 + c]).  Blocks are kept row-major here; the reference's SSE2 layout
 * pairs columns 0 and 1 of a block row in one two-lane register and keeps column 2 apart, so
 * every sum below keeps that split: a "lane 0" partial over column 0, a "lane 1" partial over
 * column 1 and a separate partial over column 2, combined as (x - s0 - s1 - f).
 * ------------------------------------------------------------------------------------------ */
typedef struct {
    uint64_t nb;   /* node rows */
    uint64_t *ptr; /* nb + 1 */
    uint32_t *col; /* block columns (< row), ascending per row */
    double *blk;   /* 9 per block, B(i, j) at 3 i + j */
    double *dg;    /* 6 per row */
} orc_tiny;

#define DG(dg, i, j) ((i) >= (j) ? (dg)[(i) * ((i) + 1) / 2 + (j)] : (dg)[(j) * ((j) + 1) / 2 + (i)])

/* MatWithTinyBlocks(const Mat<T,Sym<>,SparseLine<> > &) (MatWithTinyBlocks.h:224-270): a block
 * exists when any of its nine entries is stored in the lower SparseLine rows; absent entries
 * are 0. */
static int tiny_from_lower(uint64_t n, const uint64_t *rowptr, const uint32_t *col, const double *val,
                           orc_tiny *m) {
    if (n % 3) return -1;
    const uint64_t nb = n / 3;
    m->nb = nb;
    m->ptr = (uint64_t *)calloc(nb + 1, sizeof(uint64_t));
    m->dg = (double *)calloc(6 * (nb ? nb : 1), sizeof(double));
    uint32_t *last = (uint32_t *)malloc(sizeof(uint32_t) * (nb ? nb : 1));
    /* pass 1: count the distinct block columns of each node row (entries are sorted per row) */
    for (uint64_t R = 0; R < nb; ++R) {
        uint64_t cnt = 0;
        uint32_t prev[3] = {0, 0, 0};
        uint64_t pos[3];
        for (int a = 0; a < 3; ++a) pos[a] = rowptr[3 * R + a];
        /* merge the three scalar rows by block column */
        for (;;) {
            uint32_t cmin = UINT32_MAX;
            for (int a = 0; a < 3; ++a)
                if (pos[a] < rowptr[3 * R + a + 1] && col[pos[a]] / 3 < R && col[pos[a]] / 3 < cmin)
                    cmin = col[pos[a]] / 3;
            if (cmin == UINT32_MAX) break;
            ++cnt;
            for (int a = 0; a < 3; ++a)
                while (pos[a] < rowptr[3 * R + a + 1] && col[pos[a]] / 3 == cmin) ++pos[a];
        }
        (void)prev;
        m->ptr[R + 1] = m->ptr[R] + cnt;
    }
    const uint64_t total = m->ptr[nb];
    m->col = (uint32_t *)malloc(sizeof(uint32_t) * (total ? total : 1));
    m->blk = (double *)calloc(9 * (total ? total : 1), sizeof(double));
    if (!m->col || !m->blk || !m->ptr || !m->dg) return -2;
    for (uint64_t R = 0; R < nb; ++R) {
        uint64_t w = m->ptr[R];
        uint64_t pos[3];
        for (int a = 0; a < 3; ++a) pos[a] = rowptr[3 * R + a];
        for (;;) {
            uint32_t cmin = UINT32_MAX;
            for (int a = 0; a < 3; ++a)
                if (pos[a] < rowptr[3 * R + a + 1] && col[pos[a]] / 3 < R && col[pos[a]] / 3 < cmin)
                    cmin = col[pos[a]] / 3;
            if (cmin == UINT32_MAX) break;
            m->col[w] = cmin;
            for (int a = 0; a < 3; ++a)
                while (pos[a] < rowptr[3 * R + a + 1] && col[pos[a]] / 3 == cmin) {
                    m->blk[9 * w + 3 * a + col[pos[a]] % 3] += val[pos[a]];
                    ++pos[a];
                }
            ++w;
        }
        /* the diagonal block: the rest of each scalar row (columns 3R .. 3R + a) */
        for (int a = 0; a < 3; ++a)
            for (uint64_t k = pos[a]; k < rowptr[3 * R + a + 1]; ++k) {
                const uint32_t j = col[k];
                if (j / 3 != R) continue;
                const int b = (int)(j % 3);
                m->dg[6 * R + a * (a + 1) / 2 + b] += val[k];
            }
    }
    free(last);
    return 0;
}

static void tiny_free(orc_tiny *m) {
    free(m->ptr);
    free(m->col);
    free(m->blk);
    free(m->dg);
}

/* chol_incomp (MatWithTinyBlocks.h:426-520): row by row, each existing block
 * L_RC = (A_RC - sum_k L_Rk L_Ck^T) L_CC^-T over the columns k that rows R (before this block)
 * and C share, taken from the highest down (find_corresponding_blocks), then
 * L_RR = chol(A_RR - sum_k L_Rk L_Rk^T). */
static void tiny_chol_incomp(orc_tiny *m) {
    for (uint64_t R = 0; R < m->nb; ++R) {
        const uint64_t rb = m->ptr[R], re = m->ptr[R + 1];
        for (uint64_t ic = rb; ic < re; ++ic) {
            const uint32_t C = m->col[ic];
            const double *db = m->dg + 6 * C;
            double *ob = m->blk + 9 * ic;
            double s0[3][3] = {{0}}, s1[3][3] = {{0}}, f[3][3] = {{0}};
            int found = 0;
            /* pairs (k in row C, m in row R before ic) with equal columns, highest first */
            int64_t i0 = (int64_t)(m->ptr[C + 1] - m->ptr[C]), i1 = (int64_t)(ic - rb);
            const uint32_t *c0 = m->col + m->ptr[C], *c1 = m->col + rb;
            for (;;) {
                if (--i0 < 0 || --i1 < 0) break;
                int ok = 0;
                for (;;) {
                    if (c0[i0] == c1[i1]) {
                        ok = 1;
                        break;
                    } else if (c0[i0] < c1[i1]) {
                        if (--i1 < 0) break;
                    } else {
                        if (--i0 < 0) break;
                    }
                }
                if (!ok) break;
                found = 1;
                const double *dj = m->blk + 9 * (m->ptr[C] + (uint64_t)i0);
                const double *di = m->blk + 9 * (rb + (uint64_t)i1);
                for (int a = 0; a < 3; ++a)
                    for (int b = 0; b < 3; ++b) {
                        s0[a][b] += di[3 * a + 0] * dj[3 * b + 0];
                        s1[a][b] += di[3 * a + 1] * dj[3 * b + 1];
                        f[a][b] += di[3 * a + 2] * dj[3 * b + 2];
                    }
            }
            if (found) {
#define OB(a, b) ob[3 * (a) + (b)]
#define RS(a, b) (s0[a][b]), (s1[a][b]), (f[a][b])
                for (int a = 0; a < 3; ++a)
                    OB(a, 0) = (OB(a, 0) - s0[a][0] - s1[a][0] - f[a][0]) / DG(db, 0, 0);
                for (int a = 0; a < 3; ++a)
                    OB(a, 1) = (OB(a, 1) - s0[a][1] - s1[a][1] - f[a][1] - OB(a, 0) * DG(db, 1, 0)) / DG(db, 1, 1);
                for (int a = 0; a < 3; ++a)
                    OB(a, 2) = (OB(a, 2) - s0[a][2] - s1[a][2] - f[a][2] - OB(a, 0) * DG(db, 2, 0) -
                                OB(a, 1) * DG(db, 2, 1)) / DG(db, 2, 2);
            } else {
                for (int a = 0; a < 3; ++a) OB(a, 0) = OB(a, 0) / DG(db, 0, 0);
                for (int a = 0; a < 3; ++a) OB(a, 1) = (OB(a, 1) - OB(a, 0) * DG(db, 1, 0)) / DG(db, 1, 1);
                for (int a = 0; a < 3; ++a)
                    OB(a, 2) = (OB(a, 2) - OB(a, 0) * DG(db, 2, 0) - OB(a, 1) * DG(db, 2, 1)) / DG(db, 2, 2);
            }
#undef RS
#undef OB
        }
        /* diagonal block (MatWithTinyBlocks.h:497-519) */
        double s0[3][3] = {{0}}, s1[3][3] = {{0}}, f[3][3] = {{0}};
        for (uint64_t k = rb; k < re; ++k) {
            const double *d = m->blk + 9 * k;
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b <= a; ++b) {
                    s0[a][b] += d[3 * a + 0] * d[3 * b + 0];
                    s1[a][b] += d[3 * a + 1] * d[3 * b + 1];
                    f[a][b] += d[3 * a + 2] * d[3 * b + 2];
                }
        }
        double *g = m->dg + 6 * R;
        g[0] = sqrt(g[0] - s0[0][0] - s1[0][0] - f[0][0]);
        g[1] = (g[1] - s0[1][0] - s1[1][0] - f[1][0]) / g[0];
        g[3] = (g[3] - s0[2][0] - s1[2][0] - f[2][0]) / g[0];
        g[2] = sqrt(g[2] - s0[1][1] - s1[1][1] - f[1][1] - g[1] * g[1]);
        g[4] = (g[4] - s0[2][1] - s1[2][1] - f[2][1] - g[3] * g[1]) / g[2];
        g[5] = sqrt(g[5] - s0[2][2] - s1[2][2] - f[2][2] - g[3] * g[3] - g[4] * g[4]);
    }
}

/* solve = solve_down then solve_up (MatWithTinyBlocks.h:587-720), in place */
static void tiny_solve(const orc_tiny *m, double *r) {
    for (uint64_t R = 0; R < m->nb; ++R) {
        double s0[3] = {0, 0, 0}, s1[3] = {0, 0, 0}, f[3] = {0, 0, 0};
        for (uint64_t k = m->ptr[R]; k < m->ptr[R + 1]; ++k) {
            const double *d = m->blk + 9 * k;
            const double *v = r + 3 * (uint64_t)m->col[k];
            for (int a = 0; a < 3; ++a) {
                s0[a] += d[3 * a + 0] * v[0];
                s1[a] += d[3 * a + 1] * v[1];
                f[a] += d[3 * a + 2] * v[2];
            }
        }
        const double *g = m->dg + 6 * R;
        double *x = r + 3 * R;
        x[0] -= s0[0] + s1[0] + f[0];
        x[0] /= g[0];
        x[1] -= s0[1] + s1[1] + f[1] + g[1] * x[0];
        x[1] /= g[2];
        x[2] -= s0[2] + s1[2] + f[2] + g[3] * x[0] + g[4] * x[1];
        x[2] /= g[5];
    }
    for (uint64_t R = m->nb; R-- > 0;) {
        const double *g = m->dg + 6 * R;
        double *x = r + 3 * R;
        x[2] /= g[5];
        x[0] -= g[3] * x[2];
        x[1] -= g[4] * x[2];
        x[1] /= g[2];
        x[0] -= g[1] * x[1];
        x[0] /= g[0];
        for (uint64_t k = m->ptr[R + 1]; k-- > m->ptr[R];) {
            const double *d = m->blk + 9 * k;
            double *v = r + 3 * (uint64_t)m->col[k];
            v[0] = v[0] - (x[0] * d[0] + x[1] * d[3] + x[2] * d[6]);
            v[1] = v[1] - (x[0] * d[1] + x[1] * d[4] + x[2] * d[7]);
            v[2] -= x[0] * d[2] + x[1] * d[5] + x[2] * d[8];
        }
    }
}

/* operator* = mul(v, 1) -> partial_mul (MatWithTinyBlocks.h:303-350), one thread */
static void tiny_mul(const orc_tiny *m, const double *v, double *r) {
    memset(r, 0, sizeof(double) * 3 * m->nb);
    for (uint64_t R = 0; R < m->nb; ++R) {
        const double *vR = v + 3 * R;
        double s0[3] = {0, 0, 0}, s1[3] = {0, 0, 0}, f[3] = {0, 0, 0};
        for (uint64_t k = m->ptr[R]; k < m->ptr[R + 1]; ++k) {
            const double *d = m->blk + 9 * k;
            const uint64_t c = 3 * (uint64_t)m->col[k];
            for (int a = 0; a < 3; ++a) {
                s0[a] += d[3 * a + 0] * v[c + 0];
                s1[a] += d[3 * a + 1] * v[c + 1];
                f[a] += d[3 * a + 2] * v[c + 2];
            }
            r[c + 0] += d[0] * vR[0] + d[3] * vR[1] + d[6] * vR[2];
            r[c + 1] += d[1] * vR[0] + d[4] * vR[1] + d[7] * vR[2];
            double t = 0;
            t += d[2] * vR[0];
            t += d[5] * vR[1];
            t += d[8] * vR[2];
            r[c + 2] += t;
        }
        const double *g = m->dg + 6 * R;
        for (int a = 0; a < 3; ++a)
            r[3 * R + a] += s0[a] + s1[a] + f[a] + DG(g, a, 0) * vR[0] + DG(g, a, 1) * vR[1] + DG(g, a, 2) * vR[2];
    }
}

/* solve_using_incomplete_chol_factorize for MatWithTinyBlocks (MatWithTinyBlocks.h:1101-1150):
 * r = b - A x, stop as soon as every |r_i| <= crit (absolute), recursive residual r -= alpha q.
 * Returns the number of products A d (-1 when maxit is reached), and the factor / solve times. */
int orc_tiny_block_pcg(uint64_t n, const uint64_t *rowptr, const uint32_t *col, const double *val,
                       const double *b, double *x, double crit, int maxit, double *diag_out,
                       double *t_factor, double *t_solve) {
    orc_tiny A, P;
    struct timespec t0, t1, t2;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    if (tiny_from_lower(n, rowptr, col, val, &A) || tiny_from_lower(n, rowptr, col, val, &P)) return -2;
    tiny_chol_incomp(&P);
    clock_gettime(CLOCK_MONOTONIC, &t1);
    if (diag_out) memcpy(diag_out, P.dg, sizeof(double) * 6 * P.nb);
    double *r = (double *)malloc(sizeof(double) * n), *d = (double *)malloc(sizeof(double) * n),
           *q = (double *)malloc(sizeof(double) * n), *s = (double *)malloc(sizeof(double) * n);
    int ret = -1;
    tiny_mul(&A, x, q);
    for (uint64_t i = 0; i < n; ++i) r[i] = b[i] - q[i];
    int above = 0;
    for (uint64_t i = 0; i < n; ++i)
        if (fabs(r[i]) > crit) { above = 1; break; }
    if (!above) {
        ret = 0;
        goto done;
    }
    memcpy(d, r, sizeof(double) * n);
    tiny_solve(&P, d);
    double deltn = dotv(n, r, d);
    for (int it = 1; it <= maxit; ++it) {
        const double delto = deltn;
        tiny_mul(&A, d, q);
        const double alpha = deltn / dotv(n, d, q);
        for (uint64_t i = 0; i < n; ++i) x[i] += alpha * d[i];
        for (uint64_t i = 0; i < n; ++i) r[i] -= alpha * q[i];
        above = 0;
        for (uint64_t i = 0; i < n; ++i)
            if (fabs(r[i]) > crit) { above = 1; break; }
        if (!above) {
            ret = it;
            goto done;
        }
        memcpy(s, r, sizeof(double) * n);
        tiny_solve(&P, s);
        deltn = dotv(n, r, s);
        const double beta = deltn / delto;
        for (uint64_t i = 0; i < n; ++i) d[i] = s[i] + beta * d[i];
    }
done:
    clock_gettime(CLOCK_MONOTONIC, &t2);
    if (t_factor) *t_factor = (t1.tv_sec - t0.tv_sec) + 1e-9 * (t1.tv_nsec - t0.tv_nsec);
    if (t_solve) *t_solve = (t2.tv_sec - t1.tv_sec) + 1e-9 * (t2.tv_nsec - t1.tv_nsec);
    free(r);
    free(d);
    free(q);
    free(s);
    tiny_free(&A);
    tiny_free(&P);
    return ret;
}
