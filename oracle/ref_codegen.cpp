/*
 * ref_codegen.cpp -- runs LMT++'s own symbolic engine (include/codegen, TEST INFRASTRUCTURE) to
 * produce the element routines that LMT++'s Python 2 code generator emits for the hot path.
 *
 * The reference builds its element routines in two stages: the formal_lf Python package states
 * the weak form with Codegen expressions (through SWIG), differentiates it and hands the result to
 * Codegen's Write_code, which writes straight-line CSE'd C++.  Python 2 and SWIG are absent here,
 * but the engine itself (ex.cpp, op.cpp, exvector.cpp, exmatrix.cpp, write_code*.cpp) compiles
 * from its sources, so this program drives it from C++ with the same calls the Python layer makes
 * (the SWIG operators map one to one onto the engine's, include/codegen/codegen.i:151-171):
 *
 *   shape functions      formulations/element_Hexa.py:61-68, element_Tetra_10.py:27-41,
 *                        element_Triangle_6.py:42-47 (interpolation["nodal"])
 *   positions, jacobian  formal_lf/element.py:73-80 (pos), 141-164 (calculate_jacobian:
 *                        res[j,i] = d pos_i / d var_inter_j, determinant(), inverse())
 *   grad / grad_sym_col  formal_lf/element.py:184-242; include/codegen/__init__.py:23-34
 *   nodal unknowns       formal_lf/variable.py:50-117 (interpolation.subs(val[i] -> extrapolated
 *                        node symbol)); time extrapolation formal_lf/extrapolation.py:21-40
 *   Hooke                formal_lf/material_help.py:116-134,175-183 (compliance matrix, inverse())
 *   elasticity_iso       formulations/formulation_elasticity_iso.py:45-60
 *   difftherm            formulations/formulation_difftherm.py:19-30
 *   time integration     formal_lf/gauss_integration.py:52-63 over [left*dt1, right*dt0]
 *   volume part          formal_lf/formulation.py:548-553 (integration_totale False: form.diff(dV)
 *                        * det_jacobian * ponderation; True: element.integration(form.diff(dV)))
 *   element integration  formal_lf/element.py:97-109 with the Python Gauss rule of the element
 *   M and V              formal_lf/calculate_matrix.py:4-61 (test derivative, tests -> 0,
 *                        unknown derivative; V = -dexpr at unknowns = 0 for a linear form)
 *   code                 formal_lf/calculate_matrix.py:64-79 (Write_code('T'), tmp_i_j for
 *                        j >= i when symmetric, vec_i)
 *
 * Output: a header of plain C++ functions (one per element routine), written to the path given
 * on the command line.  The symbol names are chosen so that the emitted code compiles inside the
 * wrapper functions: P[k] = node positions (node-major), var_inter[k], ponderation, E, nu, density,
 * f_vol[d], cond, rho, cp, T1[i] (the previous time step), time_steps[k].
 * Usage: ref_codegen <out.h>
 */
#include "ex.h"
#include "exvector.h"
#include "exmatrix.h"
#include "write_code.h"
#include <cstdio>
#include <cstdlib>
#include <map>
#include <sstream>
#include <string>
#include <vector>

using namespace Codegen;
typedef std::map<Ex, Ex, Ex::ExMapCmp> MapEx;

static Ex sym(const std::string &s) { return symbol(s.c_str(), 0, 0, 0); }
static std::string idx(const char *base, int i) {
    std::ostringstream o;
    o << base << "[" << i << "]";
    return o.str();
}

/* Element data as formal_lf/element.py builds it: var_inter, val[i], interpolation["nodal"]. */
struct FElem {
    int dim, nb_nodes;
    std::vector<Ex> vi, val;
    Ex nodal;
    std::vector<ExVector> positions, base; /* base: the orthonormal frame of a face (nb_var_inter < dim) */
    ExMatrix jac, inv_jac;
    Ex det_jac;
    int nvi;
};

/* Element.__init__ (element.py:9-68): an element of formulation dimension `dim`; a face element
 * (Quad or Triangle_6 in 3D) has fewer var_inter than dim.  The symbols carry `prefix` so that a
 * face's symbols differ from its parent's, as two Element instances' do. */
static void init_elem(FElem &e, const std::string &name, int dim = 0, const char *prefix = "") {
    e.vi.clear();
    e.val.clear();
    for (int i = 0; i < 256; ++i) e.val.push_back(sym(idx("val", i)));
    std::string vname = std::string(prefix) + "var_inter", pname = std::string(prefix) + "P";
    if (name == "Hexa") {
        e.dim = 3; e.nb_nodes = 8;
        for (int i = 0; i < 3; ++i) e.vi.push_back(sym(idx(vname.c_str(), i)));
        const Ex &x = e.vi[0], &y = e.vi[1], &z = e.vi[2];
        const std::vector<Ex> &v = e.val;
        /* formulations/element_Hexa.py:61-68 */
        e.nodal = (1.0 - x) * (1.0 - y) * (1.0 - z) * v[0] +
                  x * (1.0 - y) * (1.0 - z) * v[1] +
                  x * y * (1.0 - z) * v[2] +
                  (1.0 - x) * y * (1.0 - z) * v[3] +
                  (1.0 - x) * (1.0 - y) * z * v[4] +
                  x * (1.0 - y) * z * v[5] +
                  x * y * z * v[6] +
                  (1.0 - x) * y * z * v[7];
    } else if (name == "Tetra_10") {
        e.dim = 3; e.nb_nodes = 10;
        for (int i = 0; i < 3; ++i) e.vi.push_back(sym(idx(vname.c_str(), i)));
        const std::vector<Ex> &v = e.val;
        /* formulations/element_Tetra_10.py:27-41 */
        Ex X0 = 1.0 - e.vi[0] - e.vi[1] - e.vi[2], X1 = e.vi[0], X2 = e.vi[1], X3 = e.vi[2];
        e.nodal = X0 * (2.0 * X0 - 1.0) * v[0] +
                  X1 * (2.0 * X1 - 1.0) * v[1] +
                  X2 * (2.0 * X2 - 1.0) * v[2] +
                  X3 * (2.0 * X3 - 1.0) * v[3] +
                  4.0 * X0 * X1 * v[4] +
                  4.0 * X1 * X2 * v[5] +
                  4.0 * X0 * X2 * v[6] +
                  4.0 * X0 * X3 * v[7] +
                  4.0 * X1 * X3 * v[8] +
                  4.0 * X2 * X3 * v[9];
    } else if (name == "Triangle_6") {
        e.dim = 2; e.nb_nodes = 6;
        for (int i = 0; i < 2; ++i) e.vi.push_back(sym(idx(vname.c_str(), i)));
        const std::vector<Ex> &v = e.val;
        /* formulations/element_Triangle_6.py:36-47 */
        Ex X0 = 1.0 - e.vi[0] - e.vi[1], X1 = e.vi[0], X2 = e.vi[1];
        e.nodal = (2.0 * X0 - 1.0) * X0 * v[0] +
                  (2.0 * X1 - 1.0) * X1 * v[1] +
                  (2.0 * X2 - 1.0) * X2 * v[2] +
                  4.0 * X0 * X1 * v[3] +
                  4.0 * X1 * X2 * v[4] +
                  4.0 * X2 * X0 * v[5];
    } else if (name == "Quad") {
        e.dim = 2; e.nb_nodes = 4;
        for (int i = 0; i < 2; ++i) e.vi.push_back(sym(idx(vname.c_str(), i)));
        const Ex &x = e.vi[0], &y = e.vi[1];
        const std::vector<Ex> &v = e.val;
        /* formulations/element_Quad.py:24-27 */
        e.nodal = (1.0 - x) * (1.0 - y) * v[0] +
                  x * (1.0 - y) * v[1] +
                  x * y * v[2] +
                  (1.0 - x) * y * v[3];
    } else {
        fprintf(stderr, "unknown element %s\n", name.c_str());
        exit(2);
    }
    e.nvi = e.vi.size();
    if (dim) e.dim = dim;
    /* positions elem.pos(i)[d] (element.py:56-66), named P[dim*i+d] for the wrapper */
    e.positions.clear();
    for (int i = 0; i < e.nb_nodes; ++i) {
        ExVector p(e.dim);
        for (int d = 0; d < e.dim; ++d) p[d] = sym(idx(pname.c_str(), e.dim * i + d));
        e.positions.push_back(p);
    }
    /* pos() (element.py:73-80) */
    ExVector coord(e.dim);
    for (int d = 0; d < e.dim; ++d) {
        MapEx s;
        for (int i = 0; i < e.nb_nodes; ++i) s[e.val[i]] = e.positions[i][d];
        coord[d] = e.nodal.subs(s);
    }
    e.jac = ExMatrix(e.nvi, e.nvi);
    if (e.nvi == e.dim) {
        /* calculate_jacobian, nb_var_inter == dim (element.py:141-164) */
        for (int j = 0; j < e.dim; ++j)
            for (int i = 0; i < e.dim; ++i) e.jac(j, i) = coord[i].diff(e.vi[j]);
    } else {
        /* calculate_jacobian, nb_var_inter < dim (element.py:166-182): an orthonormal frame of
         * the tangents, then the jacobian in that frame */
        e.base.clear();
        for (int v = 0; v < e.nvi; ++v) {
            ExVector cr(e.dim);
            for (int i = 0; i < e.dim; ++i) cr[i] = coord[i].diff(e.vi[v]);
            for (unsigned c = 0; c < e.base.size(); ++c) cr -= e.base[c] * dot(e.base[c], cr);
            e.base.push_back(cr / norm(cr));
        }
        for (int i = 0; i < e.nvi; ++i)
            for (int j = 0; j < e.nvi; ++j)
                for (int k = 0; k < e.dim; ++k) e.jac(j, i) += coord[k].diff(e.vi[j]) * e.base[i][k];
    }
    e.det_jac = e.jac.determinant();
    e.inv_jac = e.jac.inverse();
}

/* element.normal for a face in 3D (element.py:463-470): vectorial_product of the frame
 * (codegen/__init__.py:67-78) */
static ExVector face_normal(const FElem &c) {
    const ExVector &v1 = c.base[0], &v2 = c.base[1];
    ExVector r(3);
    r[0] = v1[1] * v2[2] - v1[2] * v2[1];
    r[1] = v1[2] * v2[0] - v1[0] * v2[2];
    r[2] = v1[0] * v2[1] - v1[1] * v2[0];
    return r;
}

/* Variable.get_scalar_expr for a nodal variable (variable.py:50-117): the interpolation with
 * val[i] replaced by the node's (extrapolated) value. */
static Ex nodal_expr(const FElem &e, const std::vector<Ex> &node_value) {
    MapEx s;
    for (int i = 0; i < e.nb_nodes; ++i) s[e.val[i]] = node_value[i];
    return e.nodal.subs(s);
}

/* element.grad for a vector (element.py:184-193) */
static ExMatrix grad_vec(const FElem &e, const ExVector &v) {
    ExMatrix res(v.size(), e.dim);
    for (unsigned k = 0; k < v.size(); ++k)
        for (int j = 0; j < e.dim; ++j)
            for (int i = 0; i < e.dim; ++i) res(k, j) += v[k].diff(e.vi[i]) * e.inv_jac(j, i);
    return res;
}

/* element.grad for a scalar (element.py:194-200) */
static ExVector grad_scal(const FElem &e, const Ex &v) {
    ExVector res(e.dim);
    for (int j = 0; j < e.dim; ++j) {
        Ex tmp = 0.0;
        for (int i = 0; i < e.dim; ++i) tmp = tmp + v.diff(e.vi[i]) * e.inv_jac(j, i);
        res[j] = tmp;
    }
    return res;
}

/* grad_sym (element.py:221-240) then mat_sym_to_vec_col (codegen/__init__.py:23-34) */
static ExVector grad_sym_col(const FElem &e, const ExVector &v) {
    ExMatrix m = grad_vec(e, v);
    int n = m.nb_rows() > m.nb_cols() ? m.nb_rows() : m.nb_cols();
    ExMatrix nm(n, n);
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
            Ex m_ij = (i < (int)m.nb_rows() && j < (int)m.nb_cols()) ? m(i, j) : Ex(0);
            Ex m_ji = (j < (int)m.nb_rows() && i < (int)m.nb_cols()) ? m(j, i) : Ex(0);
            nm(i, j) = (i == j) ? m_ij : (m_ij + m_ji) * 0.5;
        }
    ExVector r(6);
    r[0] = nm(0, 0); r[1] = nm(1, 1); r[2] = nm(2, 2);
    r[3] = nm(0, 1); r[4] = nm(0, 2); r[5] = nm(1, 2);
    return r;
}

/* hooke_isotrope_th_3d (material_help.py:116-134): Kglo = inverse of the compliance matrix */
static ExMatrix hooke_isotrope_3d(const Ex &E, const Ex &nu) {
    Ex s1 = 1.0 / E, s2 = -nu / E, s3 = (1.0 + nu) / E;
    ExMatrix H(6, 6);
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) H(i, j) = Ex(0.0);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) H(i, j) = i == j ? s1 : s2;
    for (int i = 3; i < 6; ++i) H(i, i) = s3;
    return H.inverse();
}

/* codegen/__init__.py mul(A, B) for a vector B */
static ExVector mul_mv(const ExMatrix &A, const ExVector &B) {
    ExVector r(A.nb_rows());
    for (unsigned i = 0; i < A.nb_rows(); ++i) {
        Ex tmp = 0.0;
        for (unsigned j = 0; j < A.nb_cols(); ++j) tmp = tmp + A(i, j) * B[j];
        r[i] = tmp;
    }
    return r;
}

/* trace_sym_col (codegen/__init__.py:82-87) */
static Ex trace_sym_col(const ExVector &sigma, const ExVector &epstest) {
    Ex res = 0;
    unsigned dim = (sigma.size() + 1) / 2;
    for (unsigned i = 0; i < dim; ++i) res += sigma[i] * epstest[i];
    for (unsigned i = dim; i < epstest.size(); ++i) res += 2.0 * sigma[i] * epstest[i];
    return res;
}

/* calculate_matrix (calculate_matrix.py:4-61) for a linear form, differentiation branch.  With
 * test = false (use_test_functions = False) the tests are the unknowns themselves, and the
 * substitution tests -> 0 concerns the formulation's own test symbols, which an energy does not
 * contain: nothing is substituted. */
static void calculate_matrix(const Ex &expr, const std::vector<Ex> &unk, const std::vector<Ex> &tst,
                             std::vector<std::vector<Ex> > &M, std::vector<Ex> &V, bool test = true) {
    MapEx subs_lin, subs_tes;
    for (unsigned i = 0; i < unk.size(); ++i) subs_lin[unk[i]] = number(0.0);
    if (test)
        for (unsigned i = 0; i < tst.size(); ++i) subs_tes[tst[i]] = number(0.0);
    M.assign(tst.size(), std::vector<Ex>());
    V.assign(tst.size(), Ex());
    for (unsigned i = 0; i < tst.size(); ++i) {
        Ex dexpr = expr.diff(tst[i]).subs_with_test(subs_tes);
        for (unsigned j = 0; j < unk.size(); ++j) M[i].push_back(dexpr.diff(unk[j]));
        V[i] = -dexpr.subs_with_test(subs_lin);
    }
}

/* write_matrix (calculate_matrix.py:64-79): Write_code('T'), then copies into the wrapper's out
 * arrays (the reference scatters tmp_i_j into matrix(...) at this point). */
static std::string write_matrix(const std::vector<std::vector<Ex> > &M, const std::vector<Ex> &V,
                                bool symmetric, const char *mat_out, const char *vec_out) {
    Write_code cw("T");
    unsigned n = M.size();
    std::vector<std::pair<std::string, std::string> > copies;
    for (unsigned i = 0; i < n; ++i) {
        if (mat_out)
            for (unsigned j = symmetric ? i : 0; j < M[i].size(); ++j)
                if (!M[i][j].is_zero()) {
                    std::ostringstream t, o;
                    t << "tmp_" << i << "_" << j;
                    cw.add(M[i][j], t.str(), Write_code::Declare);
                    o << mat_out << "[" << i * M[i].size() + j << "]";
                    copies.push_back(std::make_pair(o.str(), t.str()));
                }
        if (vec_out && !V[i].is_zero()) {
            std::ostringstream t, o;
            t << "vec_" << i;
            cw.add(V[i], t.str(), Write_code::Declare);
            o << vec_out << "[" << i << "]";
            copies.push_back(std::make_pair(o.str(), t.str()));
        }
    }
    std::string s = cw.to_string();
    for (unsigned k = 0; k < copies.size(); ++k)
        s += "    " + copies[k].first + " = " + copies[k].second + ";\n";
    return s;
}

/* elasticity_iso, volume part, one Gauss point (integration_totale = False):
 * dV_part = form.diff(dV) * det_jacobian * ponderation (formulation.py:552-553). */
static std::string gen_elasticity(const std::string &elem_name, const std::string &fname) {
    FElem e;
    init_elem(e, elem_name);
    const int nn = e.nb_nodes, dim = e.dim;
    /* unknowns dep (nb_der = 0: Pol_extr order 0 -> the current value) and tests */
    std::vector<Ex> unk, tst;
    std::vector<std::vector<Ex> > un(dim, std::vector<Ex>(nn)), te(dim, std::vector<Ex>(nn));
    for (int i = 0; i < nn; ++i)
        for (int d = 0; d < dim; ++d) {
            std::ostringstream su, st;
            su << "U" << i << "_" << d;
            st << "V" << i << "_" << d;
            un[d][i] = sym(su.str());
            te[d][i] = sym(st.str());
            unk.push_back(un[d][i]); /* node-major, then component (formulation.py:363-397) */
            tst.push_back(te[d][i]);
        }
    ExVector dep(dim), dep_test(dim);
    for (int d = 0; d < dim; ++d) {
        dep[d] = nodal_expr(e, un[d]);
        dep_test[d] = nodal_expr(e, te[d]);
    }
    Ex E = sym("E"), nu = sym("nu"), density = sym("density");
    ExVector f_vol(dim);
    for (int d = 0; d < dim; ++d) f_vol[d] = sym(idx("f_vol", d));
    /* formulation_elasticity_iso.py:47-53 (static: dep has no time dependence, so its second
     * time derivative is zero) */
    ExVector epsilon = grad_sym_col(e, dep), epstest = grad_sym_col(e, dep_test);
    ExMatrix H = hooke_isotrope_3d(E, nu);
    ExVector sigma = mul_mv(H, epsilon);
    ExVector acc_minus_fvol(dim);
    for (int d = 0; d < dim; ++d) acc_minus_fvol[d] = Ex(0.0) - f_vol[d];
    Ex res = density * dot(acc_minus_fvol, dep_test);
    res += trace_sym_col(sigma, epstest);
    /* time integration over [dt1 * left, dt0 * right]: one point of weight 1.0, no time symbol */
    Ex form = 0.0 + 1.0 * res;
    Ex dV_part = form * e.det_jac * sym("ponderation");
    std::vector<std::vector<Ex> > M;
    std::vector<Ex> V;
    calculate_matrix(dV_part, unk, tst, M, V);
    std::ostringstream out;
    out << "/* " << elem_name << " elasticity_iso, add_local_elem_matrix at one Gauss point: K += upper\n"
        << " * triangle (row-major " << dim * nn << "x" << dim * nn << "), F += volume force */\n"
        << "static void " << fname
        << "(const double *P, const double *var_inter, double ponderation, double E, double nu,\n"
        << "    double density, const double *f_vol, double *K, double *F) {\n"
        << "    typedef double T;\n"
        << write_matrix(M, V, true, "K", "F") << "}\n\n";

    /* skin part (formulation.py:400-438, play_with_dS_part): for each child face, the dS terms
     * -dot(f_surf, dep.test) - dot(p dS_normal, dep.test) (formulation_elasticity_iso.py:60) taken
     * onto the face, integrated by the face element with its Python Gauss rule of order >= 2 */
    ExVector f_surf(dim), dS_normal(dim);
    for (int d = 0; d < dim; ++d) {
        f_surf[d] = sym(idx("f_surf", d));
        dS_normal[d] = sym(idx("dS_normal", d));
    }
    Ex pr = sym("p");
    ExVector p_normal(dim);
    for (int d = 0; d < dim; ++d) p_normal[d] = pr * dS_normal[d];
    Ex dS_part = 0.0 - dot(f_surf, dep_test) - dot(p_normal, dep_test);
    const Ex &x = e.vi[0], &y = e.vi[1];
    const bool hexa = elem_name == "Hexa";
    /* children of element_Hexa.py:22-29 and element_Tetra_10.py:16-21 */
    static const int hexa_nodes[6][4] = {{0, 3, 2, 1}, {4, 5, 6, 7}, {0, 1, 5, 4},
                                         {3, 7, 6, 2}, {0, 4, 7, 3}, {1, 2, 6, 5}};
    static const int tet_nodes[4][6] = {{0, 2, 1, 6, 5, 4}, {0, 1, 3, 4, 8, 7},
                                        {0, 3, 2, 7, 9, 6}, {1, 2, 3, 5, 9, 8}};
    std::vector<std::vector<Ex> > cvar;
    if (hexa) {
        Ex z0 = number(0.0L), z1 = number(1.0L);
        Ex v[6][3] = {{y, x, z0}, {x, y, z1}, {x, z0, y}, {y, z1, x}, {z0, y, x}, {z1, x, y}};
        for (int c = 0; c < 6; ++c) cvar.push_back(std::vector<Ex>(v[c], v[c] + 3));
    } else {
        Ex z0 = number(0.0L);
        Ex v[4][3] = {{y, x, z0}, {y, z0, x}, {z0, x, y}, {1.0 - x - y, x, y}};
        for (int c = 0; c < 4; ++c) cvar.push_back(std::vector<Ex>(v[c], v[c] + 3));
    }
    for (unsigned c = 0; c < cvar.size(); ++c) {
        FElem ch;
        init_elem(ch, hexa ? "Quad" : "Triangle_6", dim, "C");
        MapEx s1;
        for (int i = 0; i < dim; ++i) s1[e.vi[i]] = cvar[c][i];
        Ex local = dS_part.subs(s1);
        MapEx s2;
        for (int i = 0; i < ch.nvi; ++i) s2[e.vi[i]] = ch.vi[i];
        ExVector n = face_normal(ch);
        for (int i = 0; i < dim; ++i) s2[dS_normal[i]] = n[i];
        local = local.subs(s2);
        /* element.integration (element.py:97-109) */
        Ex expr = local * ch.det_jac;
        Ex integ = 0.0;
        if (hexa) {
            /* element_Quad.py gauss_points[3] */
            Ex a = (1.0 + sqrt(Ex(1.0 / 3.0))) / 2.0, b = (1.0 - sqrt(Ex(1.0 / 3.0))) / 2.0;
            Ex a2 = (1.0 + sqrt(Ex(1.0 / 3.0))) / 2.0, b2 = (1.0 - sqrt(Ex(1.0 / 3.0))) / 2.0;
            Ex pts[4][2] = {{a, a2}, {b, a2}, {a, b2}, {b, b2}};
            for (int g = 0; g < 4; ++g) {
                MapEx mp;
                mp[ch.vi[0]] = pts[g][0];
                mp[ch.vi[1]] = pts[g][1];
                integ = integ + (1.0 / 4.0) * expr.subs(mp);
            }
        } else {
            /* element_Triangle_6.py gauss_points[4] */
            Ex ga = number("0.445948490915965"), gb = number("0.091576213509771");
            Ex wa = number("0.111690794839005"), wb = number("0.054975871827661");
            Ex pts[6][2] = {{ga, ga}, {1.0 - 2.0 * ga, ga}, {ga, 1.0 - 2.0 * ga},
                            {gb, gb}, {1.0 - 2.0 * gb, gb}, {gb, 1.0 - 2.0 * gb}};
            Ex wts[6] = {wa, wa, wa, wb, wb, wb};
            for (int g = 0; g < 6; ++g) {
                MapEx mp;
                mp[ch.vi[0]] = pts[g][0];
                mp[ch.vi[1]] = pts[g][1];
                integ = integ + wts[g] * expr.subs(mp);
            }
        }
        /* face positions -> the parent's node positions */
        MapEx sp;
        for (int i = 0; i < ch.nb_nodes; ++i)
            for (int d = 0; d < dim; ++d)
                sp[ch.positions[i][d]] = e.positions[hexa ? hexa_nodes[c][i] : tet_nodes[c][i]][d];
        integ = integ.subs(sp);
        std::vector<std::vector<Ex> > Ms;
        std::vector<Ex> Vs;
        calculate_matrix(integ, unk, tst, Ms, Vs);
        out << "/* " << elem_name << " elasticity_iso, add_skin_elem_matrix of child " << c
            << ": F += f_surf and pressure loads */\n"
            << "static void " << fname << "_skin" << c
            << "(const double *P, const double *f_surf, double p, double *F) {\n"
            << "    typedef double T;\n"
            << write_matrix(Ms, Vs, true, 0, "F") << "}\n\n";
    }
    return out.str();
}

/* difftherm on Triangle_6 (integration_totale = True, time interval [left dt1, right dt0]): the whole element; the
 * matrix is the coefficient of the new temperature, the vector is -residual at new = 0, whose
 * derivative w.r.t. the old temperature is written as B. */
static std::string gen_difftherm_tri6(const std::string &fname, double left, double right) {
    FElem e;
    init_elem(e, "Triangle_6");
    const int nn = e.nb_nodes;
    Ex time = sym("time"), ts0 = sym("time_steps[0]"), ts1 = sym("time_steps[1]");
    /* Pol_extr(1).form() (extrapolation.py:21-40) with symbols[0] = new, symbols[1] = old */
    Ex s0 = sym("S0"), s1 = sym("S1");
    Ex extr;
    {
        std::vector<Ex> t(2), s(2);
        t[0] = ts0; t[1] = ts1; s[0] = s0; s[1] = s1;
        Ex res = 0;
        Ex gact_time = t[0];
        for (int i = 0; i < 2; ++i) {
            Ex fact = number(1.0L);
            Ex act_time = t[0];
            for (int j = 0; j < 2; ++j) {
                if (i != j) fact *= time - act_time;
                act_time -= t[j];
            }
            fact /= fact.subs(time, gact_time);
            res += fact * s[i];
            gact_time -= t[i];
        }
        extr = res;
    }
    std::vector<Ex> unk, old, tst, nv(nn), tv(nn);
    for (int i = 0; i < nn; ++i) {
        Ex cur = sym(idx("T0", i)), prev = sym(idx("T1", i)), tt = sym(idx("W", i));
        MapEx m;
        m[s0] = cur;
        m[s1] = prev;
        nv[i] = extr.subs(m);
        tv[i] = tt;
        unk.push_back(cur);
        old.push_back(prev);
        tst.push_back(tt);
    }
    Ex t = nodal_expr(e, nv), te = nodal_expr(e, tv);
    Ex a = sym("cond") / (sym("rho") * sym("cp"));
    /* formulation_difftherm.py:24-30 (Q = 0: the sources are separate right-hand sides) */
    ExVector gt = grad_scal(e, t), gte = grad_scal(e, te);
    ExVector agt(2);
    for (int d = 0; d < 2; ++d) agt[d] = a * gt[d];
    Ex res = dot(agt, gte) + (t.diff(time) - Ex(0.0)) * te;
    /* gauss_integration(form, order 1, time, dt1 * left, dt0 * right): one point at the middle
     * of the interval, weight 1.0 (difftherm's left 0, right 1 give Crank-Nicolson; left = right
     * = 1 with a constant step puts the point at the end of the step, i.e. implicit Euler) */
    Ex V = sym("Vtime");
    Ex beg = ts1 * left, end = ts0 * right;
    Ex form = res.subs(time, V * (end - beg) + beg);
    form = 0.0 + 1.0 * form.subs(V, number(0.5));
    /* element.integration(form.diff(dV), 2) with the Python rule gauss_points[4] of
     * element_Triangle_6.py:81-89 (the smallest order >= 2) */
    Ex ga = number("0.445948490915965"), gb = number("0.091576213509771");
    Ex wa = number("0.111690794839005"), wb = number("0.054975871827661");
    Ex pts[6][2] = {{ga, ga}, {1.0 - 2.0 * ga, ga}, {ga, 1.0 - 2.0 * ga},
                    {gb, gb}, {1.0 - 2.0 * gb, gb}, {gb, 1.0 - 2.0 * gb}};
    Ex wts[6] = {wa, wa, wa, wb, wb, wb};
    Ex expr = form * e.det_jac;
    Ex dV_part = 0.0;
    for (int g = 0; g < 6; ++g) {
        MapEx mp;
        mp[e.vi[0]] = pts[g][0];
        mp[e.vi[1]] = pts[g][1];
        dV_part = dV_part + wts[g] * expr.subs(mp);
    }
    std::vector<std::vector<Ex> > M, Bm;
    std::vector<Ex> Vv;
    calculate_matrix(dV_part, unk, tst, M, Vv);
    /* B_ij = d V_i / d old_j: V = B T_old, the right-hand side of a step */
    Bm.assign(nn, std::vector<Ex>());
    for (int i = 0; i < nn; ++i)
        for (int j = 0; j < nn; ++j) Bm[i].push_back(Vv[i].diff(old[j]));
    std::ostringstream out;
    out << "/* Triangle_6 difftherm element (integration_totale, time interval [" << left << " dt1, " << right
        << " dt0]): A upper\n"
        << " * triangle (6x6 row-major, coefficient of the new temperature), B full (6x6, coefficient of\n"
        << " * the previous temperature in the right-hand side) */\n"
        << "static void " << fname
        << "(const double *P, const double *time_steps, double cond, double rho, double cp,\n"
        << "    double *A, double *B) {\n"
        << "    typedef double T;\n"
        << "    {\n" << write_matrix(M, Vv, true, "A", 0) << "    }\n"
        << "    {\n" << write_matrix(Bm, Vv, false, "B", 0) << "    }\n"
        << "}\n\n";
    return out.str();
}

/* recalage (formulations/formulation_recalage.py:25-47): the modified constitutive-relation-error
 * energy in the unknowns U, V, W (lambd appears in no term and is left out), minimised
 * (use_test_functions = False: calculate_matrix takes the tests to be the unknowns, so M is the
 * energy's Hessian and V minus its gradient at 0).  Unknowns per node: U, V, W, then component.
 * The volume part is integrated by the element's Python rule of order 2 (integration_totale,
 * formulation.py:549-551; element_Hexa.py gauss_points[2], element_Tetra_10.py gauss_points[2]);
 * the nodal part (norme_G, dN) is the routine of node 0 (formulation.py:538-546), applied at every
 * node by add_nodal_matrix. */
static std::string gen_recalage(const std::string &elem_name, const std::string &fname) {
    FElem e;
    init_elem(e, elem_name);
    const int nn = e.nb_nodes, dim = e.dim;
    std::vector<Ex> unk;
    std::vector<std::vector<std::vector<Ex> > > F(3, std::vector<std::vector<Ex> >(dim, std::vector<Ex>(nn)));
    const char *fld = "UVW";
    for (int i = 0; i < nn; ++i)
        for (int f = 0; f < 3; ++f)
            for (int d = 0; d < dim; ++d) {
                std::ostringstream o;
                o << fld[f] << i << "_" << d;
                F[f][d][i] = sym(o.str());
                unk.push_back(F[f][d][i]);
            }
    std::vector<std::vector<Ex> > udn(dim, std::vector<Ex>(nn));
    std::vector<Ex> udv(nn);
    for (int i = 0; i < nn; ++i) {
        for (int d = 0; d < dim; ++d) udn[d][i] = sym(idx("Ud", dim * i + d));
        udv[i] = sym(idx("Ud_valid", i));
    }
    ExVector U(dim), V(dim), W(dim), Ud(dim);
    for (int d = 0; d < dim; ++d) {
        U[d] = nodal_expr(e, F[0][d]);
        V[d] = nodal_expr(e, F[1][d]);
        W[d] = nodal_expr(e, F[2][d]);
        Ud[d] = nodal_expr(e, udn[d]);
    }
    const Ex Ud_valid = nodal_expr(e, udv);
    Ex E = sym("E"), nu = sym("nu"), rho = sym("rho"), omega = sym("omega"), gamma = sym("gamma"), r = sym("r");
    Ex dV = sym("dV"), dN = sym("dN");
    ExMatrix K = hooke_isotrope_3d(E, nu);
    ExVector epsilon_V = grad_sym_col(e, V), epsilon_U = grad_sym_col(e, U);
    ExVector sigma_V = mul_mv(K, epsilon_V), sigma_U = mul_mv(K, epsilon_U);
    ExVector gamma_w = rho * omega * W, gamma_u = rho * omega * U;
    ExMatrix Kinv = K.inverse();
    ExVector ds = sigma_V - sigma_U, dg = gamma_w - gamma_u, du = U - Ud;
    /* norme_sigma, norme_gamma, norme_G of formulation_recalage.py:27-32 */
    Ex res = gamma * (trace_sym_col(ds, mul_mv(Kinv, ds)) * dV);
    res += (1.0 - gamma) * (1.0 / (rho * pow(omega, 2)) * dot(dg, dg) * dV);
    res += Ud_valid * r / (1.0 - r) * (E * dot(du, du) * dN);
    Ex form = 0.0 + 1.0 * res;  /* time integration: no time dependence, one point of weight 1 */
    /* nodal part: var_inter -> 0, node 0's unknowns only */
    Ex dN_part = form.diff(dN);
    {
        MapEx s0;
        for (int k = 0; k < e.nvi; ++k) s0[e.vi[k]] = number(0.0L);
        dN_part = dN_part.subs(s0);
    }
    std::vector<Ex> unk0;
    for (int f = 0; f < 3; ++f)
        for (int d = 0; d < dim; ++d) unk0.push_back(F[f][d][0]);
    std::vector<std::vector<Ex> > Mn;
    std::vector<Ex> Vn;
    calculate_matrix(dN_part, unk0, unk0, Mn, Vn, false);
    form = form.subs(dN, number(0.0L));
    /* volume part, integration_totale: element.integration(form.diff(dV), 2) */
    Ex expr = form.diff(dV) * e.det_jac;
    Ex dV_part = 0.0;
    if (elem_name == "Hexa") {
        Ex a = 1.0 / sqrt(Ex(3.0));
        Ex lo = (1.0 - a) / 2.0, hi = (1.0 + a) / 2.0;
        Ex pts[8][3] = {{lo, lo, lo}, {hi, lo, lo}, {hi, hi, lo}, {lo, hi, lo},
                        {lo, lo, hi}, {hi, lo, hi}, {hi, hi, hi}, {lo, hi, hi}};
        for (int g = 0; g < 8; ++g) {
            MapEx mp;
            for (int k = 0; k < 3; ++k) mp[e.vi[k]] = pts[g][k];
            dV_part = dV_part + (1.0 / 8.0) * expr.subs(mp);
        }
    } else {
        Ex s5 = sqrt(Ex(5.0));
        Ex a = (5.0 - s5) / 20.0, b = (5.0 + 3.0 * s5) / 20.0, pw = Ex(1.0 / 24.0);
        Ex pts[4][3] = {{a, a, a}, {b, a, a}, {a, b, a}, {a, a, b}};
        for (int g = 0; g < 4; ++g) {
            MapEx mp;
            for (int k = 0; k < 3; ++k) mp[e.vi[k]] = pts[g][k];
            dV_part = dV_part + pw * expr.subs(mp);
        }
    }
    std::vector<std::vector<Ex> > M;
    std::vector<Ex> Vv;
    calculate_matrix(dV_part, unk, unk, M, Vv, false);
    std::ostringstream out;
    const int nd = 3 * dim * nn;
    out << "/* " << elem_name << " recalage: the whole element's Hessian (upper triangle of " << nd << "x" << nd
        << ", unknowns node-major then U, V, W then component) */\n"
        << "static void " << fname << "(const double *P, double E, double nu, double rho, double omega,\n"
        << "    double gamma, double *K) {\n"
        << "    typedef double T;\n"
        << write_matrix(M, Vv, true, "K", 0) << "}\n\n"
        << "/* recalage nodal part (norme_G) of one node: 9x9 upper triangle and the vector */\n"
        << "static void " << fname << "_nodal(const double *Ud, const double *Ud_valid, double E, double r,\n"
        << "    double *K, double *F) {\n"
        << "    typedef double T;\n"
        << write_matrix(Mn, Vn, true, "K", "F") << "}\n\n";
    return out.str();
}

/* Splits the generated text into a header of declarations and a source of definitions: the
 * definitions are large straight-line functions, compiled once in their own unit. */
static void split(const std::string &code, std::string &decls, std::string &defs) {
    std::string::size_type p = 0;
    defs = code;
    while ((p = defs.find("static void ", p)) != std::string::npos) {
        defs.erase(p, 7);  /* "static " */
        const std::string::size_type q = defs.find(" {\n", p);
        decls += defs.substr(p, q - p) + ";\n";
        p = q;
    }
}

int main(int argc, char **argv) {
    if (argc != 4) {
        fprintf(stderr, "usage: ref_codegen <out.h> <out.cpp> <out_recalage.cpp>\n");
        return 1;
    }
    std::string code, code_r;
    code += gen_elasticity("Hexa", "gen_hexa8_elast_gp");
    code += gen_elasticity("Tetra_10", "gen_tetra10_elast_gp");
    code += gen_difftherm_tri6("gen_tri6_difftherm_cn", 0.0, 1.0);
    code += gen_difftherm_tri6("gen_tri6_difftherm_ie", 1.0, 1.0);
    code_r += gen_recalage("Hexa", "gen_hexa8_recalage");
    code_r += gen_recalage("Tetra_10", "gen_tetra10_recalage");
    std::string decls, defs, defs_r;
    split(code, decls, defs);
    split(code_r, decls, defs_r);
    const std::string head = "/* Element routines written by LMT++'s Codegen engine (oracle/ref_codegen.cpp). */\n";
    const std::string pre = "#include <cmath>\n#include \"gen_elem.h\"\nusing std::pow;\nusing std::sqrt;\n\n";
    const std::string txt[3] = {head + "#ifndef LMTG_REF_GEN_ELEM_H\n#define LMTG_REF_GEN_ELEM_H\n" + decls + "#endif\n",
                                head + pre + defs, head + pre + defs_r};
    for (int k = 0; k < 3; ++k) {
        FILE *f = fopen(argv[1 + k], "w");
        if (!f) {
            fprintf(stderr, "cannot write %s\n", argv[1 + k]);
            return 2;
        }
        fputs(txt[k].c_str(), f);
        fclose(f);
    }
    return 0;
}
