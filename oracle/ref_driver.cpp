/*
 * ref_driver.cpp -- runs LMT++'s own runtime on the elasticity hot path (TEST INFRASTRUCTURE).
 *
 * Compiled against the reference's headers and its vendored LDL/AMD sources by
 * oracle/build_ref.sh into oracle/_ref/ (never into the product).  What comes from the
 * reference here:
 *   - the mesh:        make_rect(m, Hexa() | Tetra_10(), X0, X1, nb_points)
 *                      include/mesh/make_rect.h:653-679, 443-545
 *   - the storage:     Mat<double,Sym<>,SparseLine<> > with its insert-on-nonzero /
 *                      erase-on-exact-zero semantics              include/containers/vecsparse.h:9-47
 *   - max|diag| penalty constraints                               include/formulation/formulation.h:1028-1071
 *   - the direct solve: LDL_solver (AMD + LDL)                     include/util/solveLDL.cpp:10-125,560
 *   - IC(0) + IC-PCG                                              include/containers/matinvsparse.h:201-261,453-491
 * The per-Gauss-point element integrand is the oracle's restatement (orc_hexa8_elast_gp),
 * because the reference's element routines are produced by a Python 2 code generator that
 * cannot run here; it is scattered exactly as the generated code does it
 * (formal_lf/calculate_matrix.py:86-98): for each Gauss point, matrix(i,j) += tmp for j >= i.
 *
 * Usage: ref_driver hexa|tetra10 <nb_points> <E> <nu> <penalty> <outdir>
 *        ref_driver tri6 <nb_points> <conductivity> <rho_c> <dt> <theta> <penalty> <outdir>
 * Writes little-endian raw arrays: pos.f64 conn.u32 rowptr.u64 col.u32 val.f64 F.f64
 * u_ldl.f64 u_icpcg.f64 lam_ldl.f64 (LDL solution of K lambda = u_ldl) and info.txt.
 */
#include "mesh/meshcaracstd.h"
#include "mesh/make_rect.h"
#include "containers/matinvsparse.h"
#include "util/solveLDL.h"
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>
#include "fe_oracle.h"

using namespace LMT;

template <class T>
static void dump(const std::string &path, const std::vector<T> &v) {
    FILE *f = fopen(path.c_str(), "wb");
    if (!f) { fprintf(stderr, "cannot write %s\n", path.c_str()); exit(2); }
    if (v.size()) fwrite(&v[0], sizeof(T), v.size(), f);
    fclose(f);
}

template <class TM>
static void read_mesh(TM &m, int npe, std::vector<double> &pos, std::vector<unsigned> &conn) {
    unsigned nn = m.node_list.size(), ne = m.elem_list.size();
    pos.resize(3 * nn);
    for (unsigned i = 0; i < nn; ++i)
        for (int d = 0; d < 3; ++d) pos[3 * i + d] = m.node_list[i].pos[d];
    conn.resize(npe * ne);
    for (unsigned e = 0; e < ne; ++e)
        for (int a = 0; a < npe; ++a)
            conn[npe * e + a] = m.node_list.number(*m.elem_list[e]->node_virtual(a));
}

/* Heat diffusion on Triangle_6: mesh, theta-scheme matrices A and B in the reference's Sym
 * SparseLine storage (oracle element integrand, per-element scatter), penalty on the boundary,
 * and one step A T1 = B T0 solved with the reference's LDL.
 * usage: ref_driver tri6 <nb_points> <conductivity> <rho_c> <dt> <theta> <penalty> <outdir> */
static int run_tri6(int argc, char **argv) {
    if (argc != 9) return 1;
    unsigned nbp = atoi(argv[2]);
    double k = atof(argv[3]), rho_c = atof(argv[4]), dt = atof(argv[5]), theta = atof(argv[6]),
           penalty = atof(argv[7]);
    std::string out = argv[8];
    typedef Mesh<MeshCaracStd<2, 2, 0, double, 2> > TM; /* nb=0, degree 2 -> Triangle_6 */
    TM m;
    make_rect(m, Triangle_6(), TM::Pvec(0, 0), TM::Pvec(1, 1), TM::Pvec(nbp, nbp));
    unsigned nn = m.node_list.size(), ne = m.elem_list.size();
    std::vector<double> pos(2 * nn);
    for (unsigned i = 0; i < nn; ++i)
        for (int d = 0; d < 2; ++d) pos[2 * i + d] = m.node_list[i].pos[d];
    std::vector<unsigned> conn(6 * ne);
    for (unsigned e = 0; e < ne; ++e)
        for (int a = 0; a < 6; ++a) conn[6 * e + a] = m.node_list.number(*m.elem_list[e]->node_virtual(a));
    Mat<double, Sym<>, SparseLine<> > A(nn, nn), B(nn, nn);
    for (unsigned e = 0; e < ne; ++e) {
        double xy[12], Ke[36], Me[36];
        for (int a = 0; a < 6; ++a)
            for (int d = 0; d < 2; ++d) xy[2 * a + d] = pos[2 * conn[6 * e + a] + d];
        orc_triangle6_diff_km(xy, k / rho_c, Ke, Me);
        for (int i = 0; i < 6; ++i)
            for (int j = i; j < 6; ++j) {
                A(conn[6 * e + i], conn[6 * e + j]) += Me[6 * i + j] / dt + theta * Ke[6 * i + j];
                B(conn[6 * e + i], conn[6 * e + j]) += Me[6 * i + j] / dt - (1 - theta) * Ke[6 * i + j];
            }
    }
    /* T = 0 on the boundary: penalty constraints node[i].temperature on A */
    double max_diag = max(abs(A.diag()));
    for (unsigned i = 0; i < nn; ++i) {
        const double x = pos[2 * i], y = pos[2 * i + 1];
        if (x < 1e-9 || y < 1e-9 || x > 1 - 1e-9 || y > 1 - 1e-9) A(i, i) += max_diag * penalty;
    }
    std::vector<double> T0(nn), T1(nn);
    for (unsigned i = 0; i < nn; ++i) {
        const double dx = pos[2 * i] - 0.5, dy = pos[2 * i + 1] - 0.5;
        T0[i] = exp(-(dx * dx + dy * dy) / (2 * 0.1 * 0.1));
    }
    Vec<double> t0, rhs;
    t0.resize(nn);
    for (unsigned i = 0; i < nn; ++i) t0[i] = T0[i];
    rhs = B * t0;
    Mat<double, Sym<>, SparseLine<> > Ac = A;
    LDL_solver ldl;
    ldl.get_factorization(Ac, false);
    ldl.solve(rhs);
    for (unsigned i = 0; i < nn; ++i) T1[i] = rhs[i];
    std::vector<unsigned long long> rowptr(nn + 1, 0), rowptrB(nn + 1, 0);
    std::vector<unsigned> col, colB;
    std::vector<double> val, valB;
    for (unsigned i = 0; i < nn; ++i) {
        for (unsigned q = 0; q < A.data[i].indices.size(); ++q) {
            col.push_back(A.data[i].indices[q]);
            val.push_back(A.data[i].data[q]);
        }
        rowptr[i + 1] = col.size();
        for (unsigned q = 0; q < B.data[i].indices.size(); ++q) {
            colB.push_back(B.data[i].indices[q]);
            valB.push_back(B.data[i].data[q]);
        }
        rowptrB[i + 1] = colB.size();
    }
    dump(out + "/pos.f64", pos);
    dump(out + "/conn.u32", conn);
    dump(out + "/rowptr.u64", rowptr);
    dump(out + "/col.u32", col);
    dump(out + "/val.f64", val);
    dump(out + "/rowptrB.u64", rowptrB);
    dump(out + "/colB.u32", colB);
    dump(out + "/valB.f64", valB);
    dump(out + "/T0.f64", T0);
    dump(out + "/T1.f64", T1);
    FILE *f = fopen((out + "/info.txt").c_str(), "w");
    fprintf(f, "nn %u\nne %u\nnnz %zu\nmax_diag %.17g\n", nn, ne, col.size(), max_diag);
    fclose(f);
    return 0;
}

int main(int argc, char **argv) {
    if (argc >= 2 && std::string(argv[1]) == "tri6") return run_tri6(argc, argv);
    if (argc != 7 || (std::string(argv[1]) != "hexa" && std::string(argv[1]) != "tetra10")) {
        fprintf(stderr, "usage: ref_driver hexa|tetra10 <nb_points> <E> <nu> <penalty> <outdir>\n");
        return 1;
    }
    const bool tet = std::string(argv[1]) == "tetra10";
    const int npe = tet ? 10 : 8, nd = 3 * npe;
    unsigned nbp = atoi(argv[2]);
    double E = atof(argv[3]), nu = atof(argv[4]), penalty = atof(argv[5]);
    std::string out = argv[6];

    std::vector<double> pos;
    std::vector<unsigned> conn;
    if (tet) {
        typedef Mesh<MeshCaracStd<3, 3, 0, double, 2> > TM; /* nb=0, degree 2 -> Tetra_10 */
        TM m;
        make_rect(m, Tetra_10(), TM::Pvec(0, 0, 0), TM::Pvec(1, 1, 1), TM::Pvec(nbp, nbp, nbp));
        read_mesh(m, npe, pos, conn);
    } else {
        typedef Mesh<MeshCaracStd<3, 3, 1, double, 1> > TM; /* nb=1, degree 1 -> Hexa */
        TM m;
        make_rect(m, Hexa(), TM::Pvec(0, 0, 0), TM::Pvec(1, 1, 1), TM::Pvec(nbp, nbp, nbp));
        read_mesh(m, npe, pos, conn);
    }
    unsigned nn = pos.size() / 3, ne = conn.size() / npe, n = 3 * nn;

    /* assembly into an empty SparseLine matrix (the preallocated pattern is cleared before
       every assembly, formulation.h:931-950) */
    Mat<double, Sym<>, SparseLine<> > K(n, n);
    double w[8], xi[24];
    const int ngp = tet ? orc_gauss_tetra_order2(w, xi) : orc_gauss_hexa_order2(w, xi);
    for (unsigned e = 0; e < ne; ++e) {
        double xyz[30];
        unsigned in[10];
        for (int a = 0; a < npe; ++a) {
            in[a] = 3 * conn[npe * e + a]; /* indice_noda = node * nnu */
            for (int d = 0; d < 3; ++d) xyz[3 * a + d] = pos[3 * conn[npe * e + a] + d];
        }
        for (int g = 0; g < ngp; ++g) {
            double Ke[900] = {0};
            if (tet) orc_tetra10_elast_gp(xyz, E, nu, w[g], xi + 3 * g, Ke);
            else orc_hexa8_elast_gp(xyz, E, nu, w[g], xi + 3 * g, Ke);
            for (int i = 0; i < nd; ++i)
                for (int j = i; j < nd; ++j)
                    K(in[i / 3] + i % 3, in[j / 3] + j % 3) += Ke[nd * i + j];
        }
    }

    /* sollicitation: uniform traction (1,0,0) on the Quad4 skin faces at x = 1 */
    std::vector<double> F(n, 0.0);
    std::vector<unsigned> faces;
    double t[3] = {1, 0, 0};
    if (!tet) {
        for (unsigned e = 0; e < ne; ++e) {
            const unsigned *c = &conn[8 * e];
            /* Hexa child face 5 is nodes [1,2,6,5] (formulations/element_Hexa.py:22-29) */
            unsigned q[4] = {c[1], c[2], c[6], c[5]};
            bool on = true;
            for (int a = 0; a < 4; ++a) on = on && pos[3 * q[a]] > 1 - 1e-6;
            if (on) faces.insert(faces.end(), q, q + 4);
        }
        orc_quad4_traction(faces.size() / 4, faces.empty() ? 0 : &faces[0], &pos[0], t, &F[0]);
    } else {
        /* Tetra_10 children (formulations/element_Tetra_10.py:16-21) */
        static const int ch[4][6] = {{0, 2, 1, 6, 5, 4}, {0, 1, 3, 4, 8, 7}, {0, 3, 2, 7, 9, 6},
                                     {1, 2, 3, 5, 9, 8}};
        for (unsigned e = 0; e < ne; ++e)
            for (int f = 0; f < 4; ++f) {
                unsigned q[6];
                bool on = true;
                for (int a = 0; a < 6; ++a) {
                    q[a] = conn[10 * e + ch[f][a]];
                    on = on && pos[3 * q[a]] > 1 - 1e-6;
                }
                if (on) faces.insert(faces.end(), q, q + 6);
            }
        orc_tri6_traction(faces.size() / 6, faces.empty() ? 0 : &faces[0], &pos[0], t, &F[0]);
    }

    /* penalty constraints: node[i].dep[d] = 0 for every node on x = 0 */
    double max_diag = max(abs(K.diag()));
    unsigned ncons = 0;
    for (unsigned i = 0; i < nn; ++i)
        if (pos[3 * i] < 1e-6)
            for (int d = 0; d < 3; ++d) {
                double C = 1.0 * max_diag * penalty;
                F[3 * i + d] += C * 0.0;
                K(3 * i + d, 3 * i + d) += C * 1.0;
                ++ncons;
            }

    /* export the lower CSR */
    std::vector<unsigned long long> rowptr(n + 1, 0);
    std::vector<unsigned> col;
    std::vector<double> val;
    for (unsigned i = 0; i < n; ++i) {
        for (unsigned k = 0; k < K.data[i].indices.size(); ++k) {
            col.push_back(K.data[i].indices[k]);
            val.push_back(K.data[i].data[k]);
        }
        rowptr[i + 1] = col.size();
    }

    /* direct solve through the reference's LDL */
    Mat<double, Sym<>, SparseLine<> > Kc = K;
    LDL_solver ldl;
    ldl.get_factorization(Kc, false);
    Vec<double> sol;
    sol.resize(n);
    for (unsigned i = 0; i < n; ++i) sol[i] = F[i];
    ldl.solve(sol);
    std::vector<double> u_ldl(n);
    for (unsigned i = 0; i < n; ++i) u_ldl[i] = sol[i];
    /* adjoint of the misfit 1/2 |u|^2 (target 0, unit weights): K lambda = u, same factorization */
    Vec<double> sol2;
    sol2.resize(n);
    for (unsigned i = 0; i < n; ++i) sol2[i] = u_ldl[i];
    ldl.solve(sol2);
    std::vector<double> lam_ldl(n);
    for (unsigned i = 0; i < n; ++i) lam_ldl[i] = sol2[i];

    /* IC(0)-PCG of the reference with |r|_inf <= 1e-10 * max|F| */
    Mat<double, Sym<>, SparseLine<> > P = K;
    incomplete_chol_factorize(P);
    Vec<double> b;
    b.resize(n);
    double fmax = 0;
    for (unsigned i = 0; i < n; ++i) {
        b[i] = F[i];
        fmax = std::max(fmax, std::abs(F[i]));
    }
    Vec<double> x;
    x.resize(n, 0.0);
    int it = solve_using_incomplete_chol_factorize(P, K, b, x, 1e-10 * fmax, false);
    std::vector<double> u_ic(n);
    for (unsigned i = 0; i < n; ++i) u_ic[i] = x[i];

    dump(out + "/pos.f64", pos);
    dump(out + "/conn.u32", conn);
    dump(out + "/rowptr.u64", rowptr);
    dump(out + "/col.u32", col);
    dump(out + "/val.f64", val);
    dump(out + "/F.f64", F);
    dump(out + "/u_ldl.f64", u_ldl);
    dump(out + "/u_icpcg.f64", u_ic);
    dump(out + "/lam_ldl.f64", lam_ldl);
    FILE *f = fopen((out + "/info.txt").c_str(), "w");
    fprintf(f, "nn %u\nne %u\nn %u\nnnz %zu\nmax_diag %.17g\nncons %u\nnfaces %zu\nicpcg_iter %d\n",
            nn, ne, n, col.size(), max_diag, ncons, faces.size() / (tet ? 6 : 4), it);
    fclose(f);
    return 0;
}
