/*
 * ref_driver.cpp -- runs LMT++'s own runtime on the hot path (TEST INFRASTRUCTURE).
 *
 * Compiled against the reference's headers and its vendored LDL/AMD sources by
 * oracle/build_ref.sh into oracle/_ref/ (never into the product).  Everything that computes a
 * value here is the reference's code:
 *   - the element routines: written by the reference's own Codegen engine (gen_elem.cpp, produced
 *     at build time by oracle/ref_codegen.cpp from the weak forms of elasticity_iso and
 *     difftherm), called once per Gauss point of the reference's table
 *     (gauss_point_for_order, include/mesh/element_Hexa.h:5-20, element_Tetra_10.h:5-16) as the
 *     default add_elem_matrix does (include/formulation/formulation.h:2918-2932), and scattered
 *     as the emitted code does (formal_lf/calculate_matrix.py:86-98): matrix(i,j) += tmp_i_j for
 *     j >= i, sollicitation[i] += vec_i;
 *   - the skin loads: the generated add_skin_elem_matrix of each child face;
 *   - the mesh:        make_rect(m, Hexa() | Tetra_10() | Triangle_6(), X0, X1, nb_points)
 *                      include/mesh/make_rect.h:653-679, 443-545, 141-170
 *   - the storage:     Mat<double,Sym<>,SparseLine<> > with its insert-on-nonzero /
 *                      erase-on-exact-zero semantics              include/containers/vecsparse.h:9-47
 *   - max|diag| penalty constraints                               include/formulation/formulation.h:1028-1071
 *   - the direct solve: LDL_solver (AMD + LDL)                     include/util/solveLDL.cpp:10-125,560
 *   - IC(0) + IC-PCG                                              include/containers/matinvsparse.h:201-261,453-491
 *   - 3x3-block IC(0) + block PCG                                 include/containers/MatWithTinyBlocks.h:224-720,1101-1150
 *
 * Usage (key=value arguments after the command):
 *   ref_driver elast elem=hexa|tetra10 nbp=N E=.. [efile=path] nu=.. penalty=.. out=dir
 *              [batch4=1 nodal=path] [icpcg=1] [block=1 crit=..] [dumpK=1]
 *       Elasticity on make_rect(0..1, nbp points per side): per-element moduli from efile (raw f64,
 *       element order) or E for all; penalty clamp of x = 0; traction (1,0,0) on x = 1, or with
 *       batch4 the four load cases traction +x, +y, +z and the nodal load of `nodal` (raw f64, n).
 *   ref_driver diff nbp=N k=.. [kfile=path] rho_c=.. dt=.. theta=0.5|1 penalty=.. steps=S out=dir
 *       Triangle_6 difftherm, T = 0 on the boundary by penalty on A, Gaussian-bump T0, S LDL steps.
 *   ref_driver elem type=hexa|tetra10 in=path E=.. nu=.. out=path
 *       One element (positions in `in`): K_e summed over the Gauss table, and the skin load of
 *       every face for f_surf = (0.7,-0.2,0.4) and p = 2.5.
 *   ref_driver elem type=tri6 in=path k=.. rho_c=.. dt=.. out=path
 *       One Triangle_6: A and B for Crank-Nicolson, then implicit Euler.
 *   ref_driver recalage elem=hexa|tetra10 nbp=N E=.. nu=.. rho=.. omega=.. gamma=.. r=.. penalty=.. out=dir
 *       The recalage functional's system (9 unknowns per node), V clamped on x = 0, LDL solve.
 *   ref_driver recal_elem type=hexa|tetra10 in=path E=.. nu=.. rho=.. omega=.. gamma=.. r=..
 *              ud0=.. ud1=.. ud2=.. valid=.. out=path
 *       One element's recalage Hessian and the nodal routine of one node.
 * Outputs are little-endian raw arrays plus info.txt.
 */
#include "mesh/meshcaracstd.h"
#include "mesh/make_rect.h"
#include "containers/matinvsparse.h"
#include "containers/MatWithTinyBlocks.h"
#include "util/solveLDL.h"
#include <cstdio>
#include <cstdlib>
#include <algorithm>
#include <cstring>
#include <iostream>
#include <map>
#include <sstream>
#include <string>
#include <sys/time.h>
#include <vector>
#include "gen_elem.h"

using namespace LMT;

typedef std::map<std::string, std::string> Args;

static Args parse(int argc, char **argv) {
    Args a;
    for (int i = 2; i < argc; ++i) {
        const char *eq = strchr(argv[i], '=');
        if (!eq) { fprintf(stderr, "bad argument %s\n", argv[i]); exit(1); }
        a[std::string(argv[i], eq - argv[i])] = eq + 1;
    }
    return a;
}
static std::string arg(const Args &a, const char *k, const char *def = 0) {
    Args::const_iterator it = a.find(k);
    if (it != a.end()) return it->second;
    if (!def) { fprintf(stderr, "missing argument %s\n", k); exit(1); }
    return def;
}
static double argd(const Args &a, const char *k, const char *def = 0) { return atof(arg(a, k, def).c_str()); }

static double now() {
    timeval tv;
    gettimeofday(&tv, 0);
    return tv.tv_sec + 1e-6 * tv.tv_usec;
}

template <class T>
static void dump(const std::string &path, const std::vector<T> &v) {
    FILE *f = fopen(path.c_str(), "wb");
    if (!f) { fprintf(stderr, "cannot write %s\n", path.c_str()); exit(2); }
    if (v.size()) fwrite(&v[0], sizeof(T), v.size(), f);
    fclose(f);
}

static std::vector<double> load_f64(const std::string &path, size_t n) {
    std::vector<double> v(n);
    FILE *f = fopen(path.c_str(), "rb");
    if (!f || fread(&v[0], sizeof(double), n, f) != n) { fprintf(stderr, "cannot read %s\n", path.c_str()); exit(2); }
    fclose(f);
    return v;
}

template <class TM>
static void read_mesh(TM &m, int dim, int npe, std::vector<double> &pos, std::vector<unsigned> &conn) {
    unsigned nn = m.node_list.size(), ne = m.elem_list.size();
    pos.resize(dim * nn);
    for (unsigned i = 0; i < nn; ++i)
        for (int d = 0; d < dim; ++d) pos[dim * i + d] = m.node_list[i].pos[d];
    conn.resize(npe * ne);
    for (unsigned e = 0; e < ne; ++e)
        for (int a = 0; a < npe; ++a) conn[npe * e + a] = m.node_list.number(*m.elem_list[e]->node_virtual(a));
}

/* lower CSR of a Sym SparseLine matrix (row i: columns j <= i ascending, diagonal last) */
static void export_lower(const Mat<double, Sym<>, SparseLine<> > &K, std::vector<unsigned long long> &rowptr,
                         std::vector<unsigned> &col, std::vector<double> &val) {
    unsigned n = K.nb_rows();
    rowptr.assign(n + 1, 0);
    col.clear();
    val.clear();
    for (unsigned i = 0; i < n; ++i) {
        for (unsigned k = 0; k < K.data[i].indices.size(); ++k) {
            col.push_back(K.data[i].indices[k]);
            val.push_back(K.data[i].data[k]);
        }
        rowptr[i + 1] = col.size();
    }
}

typedef void (*SkinFn)(const double *, const double *, double, double *);
static const SkinFn hexa_skin[6] = {gen_hexa8_elast_gp_skin0, gen_hexa8_elast_gp_skin1, gen_hexa8_elast_gp_skin2,
                                    gen_hexa8_elast_gp_skin3, gen_hexa8_elast_gp_skin4, gen_hexa8_elast_gp_skin5};
static const SkinFn tet_skin[4] = {gen_tetra10_elast_gp_skin0, gen_tetra10_elast_gp_skin1,
                                   gen_tetra10_elast_gp_skin2, gen_tetra10_elast_gp_skin3};
/* children (element_Hexa.py:22-29, element_Tetra_10.py:16-21) */
static const int hexa_face[6][4] = {{0, 3, 2, 1}, {4, 5, 6, 7}, {0, 1, 5, 4}, {3, 7, 6, 2}, {0, 4, 7, 3}, {1, 2, 6, 5}};
static const int tet_face[4][6] = {{0, 2, 1, 6, 5, 4}, {0, 1, 3, 4, 8, 7}, {0, 3, 2, 7, 9, 6}, {1, 2, 3, 5, 9, 8}};

/* one element's matrix: the generated routine at every point of the reference's Gauss table */
static void element_matrix(bool tet, const double *xyz, double E, double nu, double *Ke) {
    const int nd = tet ? 30 : 24;
    memset(Ke, 0, sizeof(double) * nd * nd);
    const double *gp0 = tet ? gauss_point_for_order(2, Tetra_10()) : gauss_point_for_order(2, Hexa());
    for (const double *gp = gp0; *gp != 0.0; gp += 3 + 1) {
        double Kg[900] = {0}, Fg[30] = {0}, fv[3] = {0, 0, 0};
        if (tet) gen_tetra10_elast_gp(xyz, gp + 1, *gp, E, nu, 0.0, fv, Kg, Fg);
        else gen_hexa8_elast_gp(xyz, gp + 1, *gp, E, nu, 0.0, fv, Kg, Fg);
        for (int i = 0; i < nd * nd; ++i) Ke[i] += Kg[i];
    }
}

static int run_elast(const Args &a) {
    const bool tet = arg(a, "elem") == "tetra10";
    const int npe = tet ? 10 : 8, nd = 3 * npe;
    unsigned nbp = atoi(arg(a, "nbp").c_str());
    double nu = argd(a, "nu"), penalty = argd(a, "penalty");
    std::string out = arg(a, "out");
    const bool batch4 = arg(a, "batch4", "0") == "1";
    std::vector<double> pos;
    std::vector<unsigned> conn;
    if (tet) {
        typedef Mesh<MeshCaracStd<3, 3, 0, double, 2> > TM; /* nb=0, degree 2 -> Tetra_10 */
        TM m;
        make_rect(m, Tetra_10(), TM::Pvec(0, 0, 0), TM::Pvec(1, 1, 1), TM::Pvec(nbp, nbp, nbp));
        read_mesh(m, 3, npe, pos, conn);
    } else {
        typedef Mesh<MeshCaracStd<3, 3, 1, double, 1> > TM; /* nb=1, degree 1 -> Hexa */
        TM m;
        make_rect(m, Hexa(), TM::Pvec(0, 0, 0), TM::Pvec(1, 1, 1), TM::Pvec(nbp, nbp, nbp));
        read_mesh(m, 3, npe, pos, conn);
    }
    unsigned nn = pos.size() / 3, ne = conn.size() / npe, n = 3 * nn;
    std::vector<double> Ee(ne, argd(a, "E", "0"));
    if (a.count("efile")) Ee = load_f64(arg(a, "efile"), ne);

    /* assembly into an empty SparseLine matrix (the preallocated pattern is cleared before
       every assembly, formulation.h:931-950) */
    double t0 = now();
    Mat<double, Sym<>, SparseLine<> > K(n, n);
    const double *gp0 = tet ? gauss_point_for_order(2, Tetra_10()) : gauss_point_for_order(2, Hexa());
    for (unsigned e = 0; e < ne; ++e) {
        double xyz[30];
        unsigned in[10];
        for (int q = 0; q < npe; ++q) {
            in[q] = 3 * conn[npe * e + q]; /* indice_noda = node * nnu */
            for (int d = 0; d < 3; ++d) xyz[3 * q + d] = pos[3 * conn[npe * e + q] + d];
        }
        for (const double *gp = gp0; *gp != 0.0; gp += 3 + 1) {
            double Kg[900] = {0}, Fg[30] = {0}, fv[3] = {0, 0, 0};
            if (tet) gen_tetra10_elast_gp(xyz, gp + 1, *gp, Ee[e], nu, 0.0, fv, Kg, Fg);
            else gen_hexa8_elast_gp(xyz, gp + 1, *gp, Ee[e], nu, 0.0, fv, Kg, Fg);
            for (int i = 0; i < nd; ++i)
                for (int j = i; j < nd; ++j)
                    K(in[i / 3] + i % 3, in[j / 3] + j % 3) += Kg[nd * i + j];
        }
    }
    double t_asm = now() - t0;

    /* load cases: skin traction on the faces at x = 1 (the generated skin routine of the child
       that lies there), or the four batch cases */
    const int nrhs = batch4 ? 4 : 1;
    std::vector<std::vector<double> > F(nrhs, std::vector<double>(n, 0.0));
    unsigned nfaces = 0;
    for (unsigned e = 0; e < ne; ++e) {
        const unsigned *c = &conn[npe * e];
        double xyz[30];
        for (int q = 0; q < npe; ++q)
            for (int d = 0; d < 3; ++d) xyz[3 * q + d] = pos[3 * c[q] + d];
        const int nf = tet ? 4 : 6, fn = tet ? 6 : 4;
        for (int f = 0; f < nf; ++f) {
            bool on = true;
            for (int q = 0; q < fn; ++q) on = on && pos[3 * c[tet ? tet_face[f][q] : hexa_face[f][q]]] > 1 - 1e-6;
            if (!on) continue;
            ++nfaces;
            for (int r = 0; r < (batch4 ? 3 : 1); ++r) {
                double t[3] = {0, 0, 0}, Fe[30] = {0};
                t[r] = 1.0;
                (tet ? tet_skin[f] : hexa_skin[f])(xyz, t, 0.0, Fe);
                for (int i = 0; i < nd; ++i)
                    if (Fe[i] != 0.0) F[r][3 * c[i / 3] + i % 3] += Fe[i];
            }
        }
    }
    if (batch4) {
        std::vector<double> g = load_f64(arg(a, "nodal"), n);
        for (unsigned i = 0; i < n; ++i) F[3][i] = g[i];
    }

    /* penalty constraints: node[i].dep[d] = 0 for every node on x = 0 */
    double max_diag = max(abs(K.diag()));
    unsigned ncons = 0;
    for (unsigned i = 0; i < nn; ++i)
        if (pos[3 * i] < 1e-6)
            for (int d = 0; d < 3; ++d) {
                double C = 1.0 * max_diag * penalty;
                for (int r = 0; r < nrhs; ++r) F[r][3 * i + d] += C * 0.0;
                K(3 * i + d, 3 * i + d) += C * 1.0;
                ++ncons;
            }

    std::vector<unsigned long long> rowptr;
    std::vector<unsigned> col;
    std::vector<double> val;
    export_lower(K, rowptr, col, val);
    if (arg(a, "dumpK", "0") == "1") {
        dump(out + "/rowptr.u64", rowptr);
        dump(out + "/col.u32", col);
        dump(out + "/val.f64", val);
    }

    /* direct solve through the reference's LDL */
    Mat<double, Sym<>, SparseLine<> > Kc = K;
    LDL_solver ldl;
    ldl.get_factorization(Kc, false);
    std::vector<double> U(nrhs * n), Fall(nrhs * n);
    for (int r = 0; r < nrhs; ++r) {
        Vec<double> sol;
        sol.resize(n);
        for (unsigned i = 0; i < n; ++i) sol[i] = Fall[r * n + i] = F[r][i];
        ldl.solve(sol);
        for (unsigned i = 0; i < n; ++i) U[r * n + i] = sol[i];
    }
    /* adjoint of the misfit 1/2 |u|^2 (target 0, unit weights): K lambda = u, same factorization */
    std::vector<double> lam(n);
    {
        Vec<double> sol;
        sol.resize(n);
        for (unsigned i = 0; i < n; ++i) sol[i] = U[i];
        ldl.solve(sol);
        for (unsigned i = 0; i < n; ++i) lam[i] = sol[i];
    }
    dump(out + "/pos.f64", pos);
    dump(out + "/conn.u32", conn);
    dump(out + "/F.f64", Fall);
    dump(out + "/u_ldl.f64", U);
    dump(out + "/lam_ldl.f64", lam);

    double fmax = 0;
    for (unsigned i = 0; i < n; ++i) fmax = std::max(fmax, std::abs(F[0][i]));
    int it = -1;
    if (arg(a, "icpcg", "0") == "1") {
        /* IC(0)-PCG of the reference with |r|_inf <= 1e-10 * max|F| */
        Mat<double, Sym<>, SparseLine<> > P = K;
        incomplete_chol_factorize(P);
        Vec<double> b, x;
        b.resize(n);
        for (unsigned i = 0; i < n; ++i) b[i] = F[0][i];
        x.resize(n, 0.0);
        it = solve_using_incomplete_chol_factorize(P, K, b, x, 1e-10 * fmax, false);
        std::vector<double> u_ic(n);
        for (unsigned i = 0; i < n; ++i) u_ic[i] = x[i];
        dump(out + "/u_icpcg.f64", u_ic);
    }
    double t_bfac = -1, t_bsolve = -1;
    int block_it = -1;
    if (arg(a, "block", "0") == "1") {
        /* 3x3-block IC(0) + block PCG (MatWithTinyBlocks.h:426-720, 1101-1150), |r|_inf <= crit */
        double crit = argd(a, "crit") * fmax;
        MatWithTinyBlocks<double, Sym<3> > C(K);
        MatWithTinyBlocks<double, Sym<3> > P(C);
        double tb = now();
        P.chol_incomp();
        t_bfac = now() - tb;
        Vec<double> b, x;
        b.resize(n);
        for (unsigned i = 0; i < n; ++i) b[i] = F[0][i];
        x.resize(n, 0.0);
        tb = now();
        solve_using_incomplete_chol_factorize(P, C, b, x, crit);
        t_bsolve = now() - tb;
        std::vector<double> u_b(n);
        for (unsigned i = 0; i < n; ++i) u_b[i] = x[i];
        dump(out + "/u_block.f64", u_b);
        /* the iteration count: the same solve again with disp_r, which prints max|r| once before
           the loop and once per product A d */
        {
            Vec<double> x2;
            x2.resize(n, 0.0);
            std::ostringstream cap;
            std::streambuf *old = std::cout.rdbuf(cap.rdbuf());
            solve_using_incomplete_chol_factorize(P, C, b, x2, crit, true);
            std::cout.rdbuf(old);
            const std::string txt = cap.str();
            block_it = (int)std::count(txt.begin(), txt.end(), '\n') - 1;
        }
        /* the factor's diagonal blocks (lower 3x3, 6 values each) for the restatement's check */
        std::vector<double> dg(6 * (n / 3));
        for (unsigned r = 0; r < n / 3; ++r)
            for (int k = 0; k < 6; ++k) dg[6 * r + k] = P.diags[r].data[k];
        dump(out + "/block_diag.f64", dg);
    }
    FILE *f = fopen((out + "/info.txt").c_str(), "w");
    fprintf(f, "nn %u\nne %u\nn %u\nnnz %zu\nmax_diag %.17g\nncons %u\nnfaces %u\nicpcg_iter %d\n"
               "t_asm %.6f\nt_block_factor %.6f\nt_block_solve %.6f\nblock_iter %d\n",
            nn, ne, n, col.size(), max_diag, ncons, nfaces, it, t_asm, t_bfac, t_bsolve, block_it);
    fclose(f);
    return 0;
}

/* Heat diffusion on Triangle_6: mesh, theta-scheme matrices A and B in the reference's Sym
 * SparseLine storage (generated element routine, per-element scatter), penalty on the boundary,
 * and `steps` LDL steps A T_{n+1} = B T_n. */
static int run_diff(const Args &a) {
    unsigned nbp = atoi(arg(a, "nbp").c_str());
    double rho_c = argd(a, "rho_c"), dt = argd(a, "dt"), theta = argd(a, "theta"), penalty = argd(a, "penalty");
    int steps = atoi(arg(a, "steps", "1").c_str());
    std::string out = arg(a, "out");
    if (theta != 0.5 && theta != 1.0) { fprintf(stderr, "theta must be 0.5 or 1\n"); return 1; }
    typedef Mesh<MeshCaracStd<2, 2, 0, double, 2> > TM; /* nb=0, degree 2 -> Triangle_6 */
    TM m;
    make_rect(m, Triangle_6(), TM::Pvec(0, 0), TM::Pvec(1, 1), TM::Pvec(nbp, nbp));
    std::vector<double> pos;
    std::vector<unsigned> conn;
    read_mesh(m, 2, 6, pos, conn);
    unsigned nn = pos.size() / 2, ne = conn.size() / 6;
    std::vector<double> ke(ne, argd(a, "k", "0"));
    if (a.count("kfile")) ke = load_f64(arg(a, "kfile"), ne);
    Mat<double, Sym<>, SparseLine<> > A(nn, nn), B(nn, nn);
    const double ts[2] = {dt, dt};
    for (unsigned e = 0; e < ne; ++e) {
        double xy[12], Ae[36] = {0}, Be[36] = {0};
        for (int q = 0; q < 6; ++q)
            for (int d = 0; d < 2; ++d) xy[2 * q + d] = pos[2 * conn[6 * e + q] + d];
        if (theta == 0.5) gen_tri6_difftherm_cn(xy, ts, ke[e], rho_c, 1.0, Ae, Be);
        else gen_tri6_difftherm_ie(xy, ts, ke[e], rho_c, 1.0, Ae, Be);
        for (int i = 0; i < 6; ++i)
            for (int j = i; j < 6; ++j) {
                A(conn[6 * e + i], conn[6 * e + j]) += Ae[6 * i + j];
                B(conn[6 * e + i], conn[6 * e + j]) += Be[6 * i + j];
            }
    }
    /* T = 0 on the boundary: penalty constraints node[i].temperature on A */
    double max_diag = max(abs(A.diag()));
    for (unsigned i = 0; i < nn; ++i) {
        const double x = pos[2 * i], y = pos[2 * i + 1];
        if (x < 1e-9 || y < 1e-9 || x > 1 - 1e-9 || y > 1 - 1e-9) A(i, i) += max_diag * penalty;
    }
    std::vector<double> T(nn), states;
    for (unsigned i = 0; i < nn; ++i) {
        const double dx = pos[2 * i] - 0.5, dy = pos[2 * i + 1] - 0.5;
        T[i] = exp(-(dx * dx + dy * dy) / (2 * 0.1 * 0.1));
    }
    if (a.count("T0file")) T = load_f64(arg(a, "T0file"), nn);
    states = T;
    Mat<double, Sym<>, SparseLine<> > Ac = A;
    LDL_solver ldl;
    ldl.get_factorization(Ac, false);
    for (int s = 0; s < steps; ++s) {
        Vec<double> t0, rhs;
        t0.resize(nn);
        for (unsigned i = 0; i < nn; ++i) t0[i] = T[i];
        rhs = B * t0;
        ldl.solve(rhs);
        for (unsigned i = 0; i < nn; ++i) T[i] = rhs[i];
        states.insert(states.end(), T.begin(), T.end());
    }
    std::vector<unsigned long long> rowptr, rowptrB;
    std::vector<unsigned> col, colB;
    std::vector<double> val, valB;
    export_lower(A, rowptr, col, val);
    export_lower(B, rowptrB, colB, valB);
    dump(out + "/pos.f64", pos);
    dump(out + "/conn.u32", conn);
    if (arg(a, "dumpAB", "1") == "1") {
        dump(out + "/rowptr.u64", rowptr);
        dump(out + "/col.u32", col);
        dump(out + "/val.f64", val);
        dump(out + "/rowptrB.u64", rowptrB);
        dump(out + "/colB.u32", colB);
        dump(out + "/valB.f64", valB);
    }
    dump(out + "/states.f64", states);
    FILE *f = fopen((out + "/info.txt").c_str(), "w");
    fprintf(f, "nn %u\nne %u\nnnz %zu\nmax_diag %.17g\n", nn, ne, col.size(), max_diag);
    fclose(f);
    return 0;
}

/* recalage (formulations/formulation_recalage.py): the generated element Hessian per element and
 * the generated nodal routine per node, scattered into the reference's Sym SparseLine with 9
 * unknowns per node (U, V, W, then component); penalty constraints V = 0 on the nodes of x = 0
 * (the functional alone leaves V - U free up to rigid motions); LDL solve.
 * Ud(x, y, z) = (0.01 x^2 + 0.002 y, 0.005 x y - 0.001 z, -0.002 z + 0.0005 x z), Ud_valid = 1. */
static int run_recalage(const Args &a) {
    const bool tet = arg(a, "elem") == "tetra10";
    const int npe = tet ? 10 : 8, nd = 9 * npe;
    unsigned nbp = atoi(arg(a, "nbp").c_str());
    const double E = argd(a, "E"), nu = argd(a, "nu"), rho = argd(a, "rho"), omega = argd(a, "omega"),
                 gamma = argd(a, "gamma"), r = argd(a, "r"), penalty = argd(a, "penalty");
    std::string out = arg(a, "out");
    std::vector<double> pos;
    std::vector<unsigned> conn;
    if (tet) {
        typedef Mesh<MeshCaracStd<3, 3, 0, double, 2> > TM;
        TM m;
        make_rect(m, Tetra_10(), TM::Pvec(0, 0, 0), TM::Pvec(1, 1, 1), TM::Pvec(nbp, nbp, nbp));
        read_mesh(m, 3, npe, pos, conn);
    } else {
        typedef Mesh<MeshCaracStd<3, 3, 1, double, 1> > TM;
        TM m;
        make_rect(m, Hexa(), TM::Pvec(0, 0, 0), TM::Pvec(1, 1, 1), TM::Pvec(nbp, nbp, nbp));
        read_mesh(m, 3, npe, pos, conn);
    }
    const unsigned nn = pos.size() / 3, ne = conn.size() / npe, n = 9 * nn;
    std::vector<double> Ud(3 * nn), valid(nn, 1.0);
    for (unsigned i = 0; i < nn; ++i) {
        const double x = pos[3 * i], y = pos[3 * i + 1], z = pos[3 * i + 2];
        Ud[3 * i] = 0.01 * x * x + 0.002 * y;
        Ud[3 * i + 1] = 0.005 * x * y - 0.001 * z;
        Ud[3 * i + 2] = -0.002 * z + 0.0005 * x * z;
    }
    Mat<double, Sym<>, SparseLine<> > K(n, n);
    std::vector<double> F(n, 0.0);
    std::vector<double> Ke(nd * nd);
    for (unsigned e = 0; e < ne; ++e) {
        double xyz[30];
        for (int q = 0; q < npe; ++q)
            for (int d = 0; d < 3; ++d) xyz[3 * q + d] = pos[3 * conn[npe * e + q] + d];
        std::fill(Ke.begin(), Ke.end(), 0.0);
        if (tet) gen_tetra10_recalage(xyz, E, nu, rho, omega, gamma, &Ke[0]);
        else gen_hexa8_recalage(xyz, E, nu, rho, omega, gamma, &Ke[0]);
        for (int i = 0; i < nd; ++i)
            for (int j = i; j < nd; ++j)
                K(9 * conn[npe * e + i / 9] + i % 9, 9 * conn[npe * e + j / 9] + j % 9) += Ke[nd * i + j];
    }
    for (unsigned i = 0; i < nn; ++i) { /* add_nodal_matrix: node 0's routine on every node */
        double Kn[81] = {0}, Fn[9] = {0};
        if (tet) gen_tetra10_recalage_nodal(&Ud[3 * i], &valid[i], E, r, Kn, Fn);
        else gen_hexa8_recalage_nodal(&Ud[3 * i], &valid[i], E, r, Kn, Fn);
        for (int p = 0; p < 9; ++p) {
            for (int q = p; q < 9; ++q) K(9 * i + p, 9 * i + q) += Kn[9 * p + q];
            F[9 * i + p] += Fn[p];
        }
    }
    double max_diag = max(abs(K.diag()));
    unsigned ncons = 0;
    for (unsigned i = 0; i < nn; ++i)
        if (pos[3 * i] < 1e-6)
            for (int d = 0; d < 3; ++d) {
                K(9 * i + 3 + d, 9 * i + 3 + d) += max_diag * penalty;
                ++ncons;
            }
    std::vector<unsigned long long> rowptr;
    std::vector<unsigned> col;
    std::vector<double> val;
    export_lower(K, rowptr, col, val);
    if (arg(a, "dumpK", "1") == "1") {
        dump(out + "/rowptr.u64", rowptr);
        dump(out + "/col.u32", col);
        dump(out + "/val.f64", val);
    }
    Mat<double, Sym<>, SparseLine<> > Kc = K;
    LDL_solver ldl;
    ldl.get_factorization(Kc, false);
    Vec<double> sol;
    sol.resize(n);
    for (unsigned i = 0; i < n; ++i) sol[i] = F[i];
    ldl.solve(sol);
    std::vector<double> u(n);
    for (unsigned i = 0; i < n; ++i) u[i] = sol[i];
    dump(out + "/pos.f64", pos);
    dump(out + "/conn.u32", conn);
    dump(out + "/F.f64", F);
    dump(out + "/u_ldl.f64", u);
    dump(out + "/Ud.f64", Ud);
    FILE *f = fopen((out + "/info.txt").c_str(), "w");
    fprintf(f, "nn %u\nne %u\nn %u\nnnz %zu\nmax_diag %.17g\nncons %u\n", nn, ne, n, col.size(), max_diag, ncons);
    fclose(f);
    return 0;
}

/* One element through the generated routines. */
static int run_elem(const Args &a) {
    std::string type = arg(a, "type"), out = arg(a, "out");
    if (type == "tri6") {
        std::vector<double> xy = load_f64(arg(a, "in"), 12);
        double dt = argd(a, "dt");
        const double ts[2] = {dt, dt};
        std::vector<double> res(4 * 36, 0.0);
        gen_tri6_difftherm_cn(&xy[0], ts, argd(a, "k"), argd(a, "rho_c"), 1.0, &res[0], &res[36]);
        gen_tri6_difftherm_ie(&xy[0], ts, argd(a, "k"), argd(a, "rho_c"), 1.0, &res[72], &res[108]);
        dump(out, res);
        return 0;
    }
    const bool tet = type == "tetra10";
    const int npe = tet ? 10 : 8, nd = 3 * npe, nf = tet ? 4 : 6;
    std::vector<double> xyz = load_f64(arg(a, "in"), 3 * npe);
    std::vector<double> res(nd * nd + nf * nd, 0.0);
    element_matrix(tet, &xyz[0], argd(a, "E"), argd(a, "nu"), &res[0]);
    const double t[3] = {0.7, -0.2, 0.4};
    for (int f = 0; f < nf; ++f) (tet ? tet_skin[f] : hexa_skin[f])(&xyz[0], t, 2.5, &res[nd * nd + nd * f]);
    dump(out, res);
    return 0;
}

/* One element through the generated recalage routines: the element Hessian (upper triangle,
 * 9 npe x 9 npe), then the nodal routine's 9 x 9 upper triangle and vector for Ud = (ud0, ud1, ud2),
 * Ud_valid = valid. */
static int run_recal_elem(const Args &a) {
    const bool tet = arg(a, "type") == "tetra10";
    const int npe = tet ? 10 : 8, nd = 9 * npe;
    std::vector<double> xyz = load_f64(arg(a, "in"), 3 * npe);
    std::vector<double> res(nd * nd + 81 + 9, 0.0);
    const double E = argd(a, "E"), nu = argd(a, "nu"), rho = argd(a, "rho"), omega = argd(a, "omega"),
                 gamma = argd(a, "gamma"), r = argd(a, "r");
    if (tet) gen_tetra10_recalage(&xyz[0], E, nu, rho, omega, gamma, &res[0]);
    else gen_hexa8_recalage(&xyz[0], E, nu, rho, omega, gamma, &res[0]);
    const double ud[3] = {argd(a, "ud0"), argd(a, "ud1"), argd(a, "ud2")}, valid = argd(a, "valid");
    if (tet) gen_tetra10_recalage_nodal(ud, &valid, E, r, &res[nd * nd], &res[nd * nd + 81]);
    else gen_hexa8_recalage_nodal(ud, &valid, E, r, &res[nd * nd], &res[nd * nd + 81]);
    dump(arg(a, "out"), res);
    return 0;
}

int main(int argc, char **argv) {
    std::string cmd = argc >= 2 ? argv[1] : "";
    Args a = parse(argc, argv);
    if (cmd == "elast") return run_elast(a);
    if (cmd == "diff") return run_diff(a);
    if (cmd == "elem") return run_elem(a);
    if (cmd == "recalage") return run_recalage(a);
    if (cmd == "recal_elem") return run_recal_elem(a);
    fprintf(stderr, "usage: ref_driver elast|diff|elem|recalage|recal_elem key=value ...\n");
    return 1;
}
