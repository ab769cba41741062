/*
 * fe_oracle.c -- CPU restatement of LMT++'s finite-element hot path (TEST INFRASTRUCTURE).
 *
 * This is the checker the GPU path is compared against, and the "port" CPU baseline.
 * It is never linked into the product library.  See fe_oracle.h for the reference
 * file:line each function restates.  Plain C99, one thread, double precision.
 */
#include "fe_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

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

int orc_gauss_quad_order2(double *w, double *xi) {
    static const double t[4][2] = {{GB, GB}, {GA, GB}, {GB, GA}, {GA, GA}};
    for (int g = 0; g < 4; ++g) {
        w[g] = 0.25;
        xi[2 * g] = t[g][0];
        xi[2 * g + 1] = t[g][1];
    }
    return 4;
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

double orc_hexa8_elast_gp(const double *xyz, double E, double nu, double w, const double *xi,
                          double *Ke) {
    double dN[8][3], J[3][3] = {{0}}, Ji[3][3], det, D[6][6], g[8][3];
    hexa8_dN(xi, dN);
    for (int a = 0; a < 8; ++a)
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) J[i][j] += xyz[3 * a + i] * dN[a][j];
    inv3(J, Ji, &det);
    for (int a = 0; a < 8; ++a)
        for (int i = 0; i < 3; ++i) {
            double s = 0;
            for (int j = 0; j < 3; ++j) s += Ji[j][i] * dN[a][j];
            g[a][i] = s;
        }
    hooke_energy_matrix(E, nu, D);
    double B[6][24];
    memset(B, 0, sizeof(B));
    for (int a = 0; a < 8; ++a) {
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
    double DB[6][24];
    for (int k = 0; k < 6; ++k)
        for (int c = 0; c < 24; ++c) {
            double s = 0;
            for (int l = 0; l < 6; ++l) s += D[k][l] * B[l][c];
            DB[k][c] = s;
        }
    double f = w * det;
    for (int r = 0; r < 24; ++r)
        for (int c = 0; c < 24; ++c) {
            double s = 0;
            for (int k = 0; k < 6; ++k) s += B[k][r] * DB[k][c];
            Ke[24 * r + c] += f * s;
        }
    return det;
}

void orc_hexa8_elast_ke(const double *xyz, double E, double nu, double *Ke) {
    double w[8], xi[24];
    memset(Ke, 0, sizeof(double) * 576);
    orc_gauss_hexa_order2(w, xi);
    for (int g = 0; g < 8; ++g) orc_hexa8_elast_gp(xyz, E, nu, w[g], xi + 3 * g, Ke);
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
    if (npe != 8) return -1;
    const int nd = 24;
    double w[8], xi[24];
    orc_gauss_hexa_order2(w, xi);
    memset(val, 0, sizeof(double) * rowptr[nn * 3]);
    double xyz[24], Ke[576];
    for (uint64_t e = 0; e < ne; ++e) {
        const uint32_t *c = conn + (uint64_t)npe * e;
        for (int a = 0; a < npe; ++a)
            for (int d = 0; d < 3; ++d) xyz[3 * a + d] = pos[3 * (uint64_t)c[a] + d];
        double Ee = E[E_per_elem ? e : 0];
        for (int g = 0; g < 8; ++g) {
            memset(Ke, 0, sizeof(Ke));
            orc_hexa8_elast_gp(xyz, Ee, nu, w[g], xi + 3 * g, Ke);
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
