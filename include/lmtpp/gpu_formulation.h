// gpu_formulation.h -- LMT++-side adapter: an elasticity_iso formulation whose hot path (element
// matrices, assembly, solve) runs on the GPU through liblmtg (include/lmtg.h).
//
// It is a FormulationAncestor<double> (include/formulation/formulation_ancestor.h:18-262), so code
// written against LMT++'s virtual formulation API -- main(), ProblemAncestor::iteration,
// FormulationAssembly, FormulationFit -- can hold it in place of a generated
// Formulation<TM, elasticity_iso, ...>.  It builds with the reference's own flags
// (g++ -std=gnu++98 -fpermissive -DDONT_WANT_XML -DDINT -I <LMTpp>/include) and links with
// -llmtg.
//
// What each virtual does:
//   set_mesh, allocate_matrices   mesh upload (Hexa8 or Tetra10 by the element's node count),
//                                 pattern and device buffers (lmtg_mesh_set, lmtg_allocate_matrices)
//   assemble*, solve_system,      lmtg_assemble and lmtg_solve_system: iterative_criterium == 0 is
//   solve                         the reference's direct solve, here a FP64 PCG to a 1e-14
//                                 relative residual; otherwise the mixed FP32/FP64 solver to that
//                                 relative residual (use_fp64_only = true: the FP64 PCG)
//   add_constraint                "[c*]node[i].dep[d] [+-v]" with its penalty (lmtg_set_constraints;
//                                 penalty 0 = the exact constraint)
//   get_mat / get_sollicitation / the assembled K as the reference's Sym SparseLine, F, u
//   get_result / max_diag
//   call_after_solve              epsilon, sigma, tr_epsilon per element (lmtg_element_fields),
//                                 kept in element_fields
//   levenberg_marquadt            applied at every assembly (lmtg_set_levenberg_marquadt)
// Time stepping, der_var sensitivities (the adjoint of lmtg_adjoint_grad replaces them),
// non-symmetric and other storages, XML materials and per-element residual hooks are not on the
// GPU path: those methods report it on std::cerr and return without effect.
#ifndef LMTPP_GPU_FORMULATION_H
#define LMTPP_GPU_FORMULATION_H

#include <algorithm>
#include <cstdlib>
#include <iostream>
#include <string>
#include <vector>

#include "formulation/formulation_ancestor.h"
#include "containers/matinv.h"  // SolveException
#include "lmtg.h"

namespace LMT {

template <class TM>
class GpuFormulationElasticity : public FormulationAncestor<double> {
public:
    typedef double T;

    explicit GpuFormulationElasticity(TM &m, int device = 0)
        : use_fp64_only(false), maxit(1000000), timeout_s(0.0), m_(&m), ctx_(0), nn_(0), ne_(0), npe_(0),
          allocated_(false), have_mat_(false), mesh_dirty_(true), cons_dirty_(true), E_(1, 1.0), nu_(0.33) {
        check(lmtg_create(device, &ctx_), "lmtg_create");
    }
    virtual ~GpuFormulationElasticity() {
        if (ctx_) lmtg_destroy(ctx_);
    }

    // ---- material (the elastic_modulus / poisson_ratio variables of elasticity_iso) ----
    void set_elastic_modulus(double E) { E_.assign(1, E); have_mat_ = false; }
    void set_elastic_modulus(const std::vector<double> &E_per_elem) { E_ = E_per_elem; have_mat_ = false; }
    void set_poisson_ratio(double nu) { nu_ = nu; have_mat_ = false; }
    /// f_surf on skin faces (Quad4 node ids for Hexa8 meshes, Triangle_6 ids for Tetra10 meshes)
    void add_skin_traction(const std::vector<unsigned> &faces, const double traction[3]) {
        upload_mesh();
        std::vector<uint32_t> f(faces.begin(), faces.end());
        const unsigned fn = npe_ == 8 ? 4 : 6;
        check(lmtg_add_skin_traction(ctx_, f.size() / fn, f.empty() ? 0 : &f[0], traction), "skin traction");
    }
    void set_nodal_loads(const Vec<T> &F) {
        upload_mesh();
        check(lmtg_set_nodal_loads(ctx_, F.ptr()), "nodal loads");
    }

    // ---- FormulationAncestor ----
    virtual std::string get_name() const { return "elasticity_iso (GPU, liblmtg)"; }
    virtual void set_mesh(void *m) {
        m_ = static_cast<TM *>(m);
        mesh_dirty_ = true;
        allocated_ = false;
    }
    virtual void *get_mesh() { return m_; }

    virtual void allocate_matrices(bool allocate_mat = true, bool allocate_vec = true) {
        upload_mesh();
        uint64_t nnz = 0;
        check(lmtg_allocate_matrices(ctx_, &nnz), "allocate_matrices");
        allocated_ = true;
        have_mat_ = false;
        result_.resize(3 * nn_, 0.0);
        sollicitation_.resize(3 * nn_, 0.0);
        (void)allocate_mat;
        (void)allocate_vec;
    }
    virtual void assemble(bool assemble_mat = true, bool assemble_vec = true) {
        if (!allocated_) allocate_matrices();
        sync_material_and_constraints();
        int flags = 0;
        if (assemble_mat) flags |= LMTG_ASM_MAT64 | (use_fp64_only ? 0 : LMTG_ASM_MAT32);
        if (assemble_vec) flags |= LMTG_ASM_VEC;
        check(lmtg_assemble(ctx_, flags), "assemble");
        if (assemble_mat) have_mat_ = true;
        double md = 0;
        check(lmtg_get_penalty_scale(ctx_, &md), "penalty scale");
        max_diag = md;
    }
    virtual void assemble_clean_mat(bool assemble_mat = true, bool assemble_vec = true) {
        assemble(assemble_mat, assemble_vec);
    }
    virtual void assemble_constraints(bool assemble_mat = true, bool assemble_vec = true) {
        assemble(assemble_mat, assemble_vec);
    }
    virtual void assemble_sollicitations(bool assemble_mat = true, bool assemble_vec = true) {
        assemble(assemble_mat, assemble_vec);
    }
    /// solve_system(iterative_criterium): 0 = the reference's direct solve (FP64 PCG to 1e-14 here)
    virtual bool solve_system(T iterative_criterium = T(0), bool disp_timing = false) {
        const bool direct = iterative_criterium == T(0);
        const int mode = (direct || use_fp64_only) ? LMTG_SOLVE_PCG_F64 : LMTG_SOLVE_MIXED_IR;
        lmtg_solve_stats st;
        const int s = lmtg_solve_system(ctx_, mode, LMTG_CRIT_REL_RESIDUAL, direct ? 1e-14 : iterative_criterium,
                                        maxit, timeout_s, &st);
        if (disp_timing)
            std::cout << "  solve_system (GPU) -> " << 1e-3 * st.device_ms << " s, " << st.iterations
                      << " iterations, rel. residual " << st.rel_residual << std::endl;
        if (s == LMTG_ERR_NOT_CONVERGED || s == LMTG_ERR_NAN || s == LMTG_ERR_TIMEOUT) throw SolveException();
        check(s, "solve_system");
        check(lmtg_get_result(ctx_, result_.ptr()), "get_result");
        return true;
    }
    virtual bool solve(T iterative_criterium = T(0), bool disp_timing = false) {
        if (!allocated_) allocate_matrices();
        assemble(!(assume_constant_matrix && have_mat_), true);
        solve_system(iterative_criterium ? iterative_criterium : default_iterative_criterium, disp_timing);
        call_after_solve();
        return true;
    }
    virtual void get_precond() { if (!have_mat_) assemble(true, false); }
    virtual void solve_system_using_precond(T iterative_criterium) { solve_system(iterative_criterium); }
    virtual void get_factorization_matrix() { if (!have_mat_) assemble(true, false); }
    virtual void solve_system_using_factorization_matrix() { solve_system(0); }

    virtual unsigned add_constraint(const std::string &txt, const T &penalty_value) {
        Cons c;
        if (!parse_constraint(txt, c)) {
            std::cerr << "GpuFormulationElasticity: constraint \"" << txt << "\" is not a linear nodal one" << std::endl;
            throw SolveException();
        }
        c.penalty = penalty_value;
        cons_.push_back(c);
        cons_dirty_ = true;
        return cons_.size() - 1;
    }
    virtual unsigned nb_constraints() const { return cons_.size(); }
    virtual void erase_constraints() { cons_.clear(); cons_dirty_ = true; }
    virtual void erase_constraints_from(unsigned number) {
        if (number < cons_.size()) cons_.resize(number);
        cons_dirty_ = true;
    }
    virtual Vec<LinearizedConstraint> get_linearized_constraints() {
        Vec<LinearizedConstraint> res;
        for (unsigned k = 0; k < cons_.size(); ++k) {
            LinearizedConstraint lc;
            LinearizedConstraint::Coeff cf;
            cf.val = cons_[k].coef;
            cf.num_in_vec = 3 * cons_[k].node + cons_[k].d;
            lc.coeffs.push_back(cf);
            lc.val = cons_[k].res;
            res.push_back(lc);
        }
        return res;
    }

    virtual void get_mat(Mat<T, Sym<>, SparseLine<> > *&mat) {
        const unsigned n = 3 * nn_;
        uint64_t nb = 0;
        check(lmtg_get_sizes(ctx_, 0, 0, 0, &nb), "sizes");
        std::vector<uint64_t> rowptr(n + 1);
        const uint64_t nnz_max = 9 * nb;  // upper bound of the lower part
        std::vector<uint32_t> col(nnz_max);
        std::vector<double> val(nnz_max);
        check(lmtg_get_matrix_lower(ctx_, &rowptr[0], &col[0], &val[0]), "get_matrix_lower");
        K_.resize(n, n);
        for (unsigned i = 0; i < n; ++i) {
            const unsigned b = rowptr[i], e = rowptr[i + 1];
            K_.data[i].indices.resize(e - b);
            K_.data[i].data.resize(e - b);
            for (unsigned k = b; k < e; ++k) {
                K_.data[i].indices[k - b] = col[k];
                K_.data[i].data[k - b] = val[k];
            }
        }
        mat = &K_;
    }
    virtual void get_mat(Mat<T, Gen<>, SparseLU> *&mat) { not_on_gpu("get_mat(Gen, SparseLU)"); mat = 0; }
#ifdef WITH_CHOLMOD
    virtual void get_mat(Mat<T, Sym<>, SparseCholMod> *&mat) { not_on_gpu("get_mat(SparseCholMod)"); mat = 0; }
#endif
#ifdef WITH_UMFPACK
    virtual void get_mat(Mat<T, Gen<>, SparseUMFPACK> *&mat) { not_on_gpu("get_mat(SparseUMFPACK)"); mat = 0; }
#endif
    virtual void display_mat(std::ostream &os) const { os << "(matrix on the GPU: use get_mat)" << std::endl; }
    virtual Vec<T> &get_sollicitation() {
        check(lmtg_get_sollicitation(ctx_, sollicitation_.ptr()), "get_sollicitation");
        return sollicitation_;
    }
    virtual Vec<T> &get_result(unsigned num = 0) {
        if (num != 0) not_on_gpu("get_result(num > 0): no time steps on this path");
        return result_;
    }
    virtual Vec<T> get_nodal_forces() {
        Vec<T> r;
        r.resize(3 * nn_);
        check(lmtg_spmv(ctx_, 0, result_.ptr(), r.ptr()), "spmv");
        return r;
    }
    virtual Vec<T> get_residual() const {
        Vec<T> Ku, F;
        Ku.resize(3 * nn_);
        F.resize(3 * nn_);
        lmtg_spmv(ctx_, 0, result_.ptr(), Ku.ptr());
        lmtg_get_sollicitation(ctx_, F.ptr());
        return F - Ku;
    }

    /// element fields after the solve (apply_on_elements_after_solve of elasticity_iso): 13 per
    /// element -- epsilon (6), sigma (6), tr_epsilon
    virtual void call_after_solve() {
        element_fields.resize(13 * ne_);
        check(lmtg_element_fields(ctx_, 0, &element_fields[0]), "element_fields");
    }
    virtual void call_after_solve(unsigned) { call_after_solve(); }
    virtual void call_after_solve(Vec<Vec<T> > &) { call_after_solve(); }
    virtual void call_after_solve(Vec<Vec<T> > &, unsigned) { call_after_solve(); }
    virtual void call_after_solve(const Vec<void *> &) { call_after_solve(); }
#define LMTG_NO_AFTER_SOLVE(k)                                   \
    virtual void call_after_solve_##k() {}                       \
    virtual void call_after_solve_##k(unsigned) {}               \
    virtual void call_after_solve_##k(Vec<Vec<T> > &) {}         \
    virtual void call_after_solve_##k(Vec<Vec<T> > &, unsigned) {} \
    virtual void call_after_solve_##k(const Vec<void *> &) {}
    LMTG_NO_AFTER_SOLVE(2) LMTG_NO_AFTER_SOLVE(3) LMTG_NO_AFTER_SOLVE(4) LMTG_NO_AFTER_SOLVE(5)
    LMTG_NO_AFTER_SOLVE(6) LMTG_NO_AFTER_SOLVE(7) LMTG_NO_AFTER_SOLVE(8) LMTG_NO_AFTER_SOLVE(9)
    LMTG_NO_AFTER_SOLVE(10) LMTG_NO_AFTER_SOLVE(11) LMTG_NO_AFTER_SOLVE(12) LMTG_NO_AFTER_SOLVE(13)
    LMTG_NO_AFTER_SOLVE(14) LMTG_NO_AFTER_SOLVE(15)
#undef LMTG_NO_AFTER_SOLVE

    // ---- static problem: no time stepping, identity DOF numbering node * 3 ----
    virtual void shift(int) {}
    virtual void unshift(int) {}
    virtual unsigned update_connectivity() { upload_mesh(); return 3 * nn_; }
    virtual void resize() {}
    virtual void set_initial_time_step(T) {}
    virtual T get_next_time_step() const { return T(0); }
    virtual T get_time() const { return T(0); }
    virtual void set_time(T) {}
    virtual void clean_mats() { have_mat_ = false; }
    virtual void free_matrices() { allocated_ = false; have_mat_ = false; }
    virtual unsigned get_nb_nodal_unknowns() const { return 3; }
    virtual unsigned get_nb_global_unknowns() const { return 0; }
    virtual unsigned get_nb_elem_unknowns() const { return 0; }
    virtual unsigned get_indice_noda(unsigned num_node) const { return 3 * num_node; }
    virtual void set_indice_noda(unsigned, unsigned) const { not_on_gpu("renumbering (indice_noda is node * 3)"); }
    virtual unsigned num_in_vec_unknown(const std::string &) const { return 0; }  // dep, the only unknown
    virtual unsigned get_nb_vectors() { return 1; }
    virtual unsigned nb_constrained_nodes() const { return constrained(-1).size(); }
    virtual unsigned nb_constrained_nodes_in_dim(unsigned dim) const { return constrained((int)dim).size(); }
    virtual Vec<bool> constrained_nodes() const { return constrained_mask(-1); }
    virtual Vec<bool> constrained_nodes_in_dim(unsigned dim) const { return constrained_mask((int)dim); }
    virtual void update_variables() {}
    virtual void update_variables(Vec<Vec<T> > &) {}
    virtual void update_variables(T) {}
    virtual void get_initial_conditions() {}
    virtual void get_initial_conditions(Vec<Vec<T> > &) {}
    virtual unsigned localOP_local_update() { return 0; }
    virtual void localOP_update_variables() {}

    // ---- not on the GPU path ----
    virtual bool solve_and_get_derivatives(Vec<Vec<T> > &, bool = false) {
        not_on_gpu("solve_and_get_derivatives (lmtg_adjoint_grad gives all per-element moduli gradients at once)");
        return false;
    }
    virtual void get_der_var_on_mesh(unsigned) { not_on_gpu("get_der_var_on_mesh"); }
    virtual void assemble_clean_mat(Mat<T, Sym<>, SparseLine<> > &, Vec<T> &, Vec<Vec<T> > &, bool = true, bool = true) {
        not_on_gpu("assemble_clean_mat into external storage");
    }
    virtual void assemble_constraints(Mat<T, Sym<>, SparseLine<> > &, Vec<T> &, Vec<Vec<T> > &, const T &, bool = true,
                                      bool = true) {
        not_on_gpu("assemble_constraints into external storage");
    }
    virtual void assemble_sollicitations(Mat<T, Sym<>, SparseLine<> > &, Vec<T> &, Vec<Vec<T> > &, bool = true,
                                         bool = true) {
        not_on_gpu("assemble_sollicitations into external storage");
    }
    /// assembly into caller-owned storage: the GPU assembly, copied out as Sym SparseLine and F
    virtual void assemble(Mat<T, Sym<>, SparseLine<> > &K, Vec<T> &F, Vec<Vec<T> > &, bool assemble_mat = true,
                          bool assemble_vec = true) {
        assemble(assemble_mat, assemble_vec);
        if (assemble_mat) {
            Mat<T, Sym<>, SparseLine<> > *p = 0;
            get_mat(p);
            K = *p;
        }
        if (assemble_vec) F = get_sollicitation();
    }
    virtual void assemble(Mat<T, Sym<>, SparseLine<> > &, Mat<T, Sym<>, SparseLine<> > &, Vec<Vec<T> > &, bool = true) {
        not_on_gpu("assemble(A, B): mass/stiffness split (the transient path is lmtg_diff_*)");
    }
    virtual void assemble(Mat<T, Gen<>, SparseLine<> > &, Vec<Vec<T> > &, bool = true) {
        not_on_gpu("assemble(Gen): the path is symmetric");
    }
    virtual void read_material_to_mesh(const XmlNode &) { not_on_gpu("read_material_to_mesh (XML)"); }
    virtual void set_vectors_assembly(Vec<Vec<T> > &) { not_on_gpu("set_vectors_assembly"); }
    virtual void set_indice_noda(Vec<unsigned> &) { not_on_gpu("set_indice_noda"); }
    virtual void set_indice_elem(Vec<unsigned> *) { not_on_gpu("set_indice_elem"); }
    virtual void set_indice_glob(unsigned &) { not_on_gpu("set_indice_glob"); }
    virtual void set_f_nodal(Vec<T> *) { not_on_gpu("set_f_nodal (use set_nodal_loads)"); }
    virtual void Get_Nb_UnknownByElement(unsigned *, unsigned &, unsigned *) { not_on_gpu("Get_Nb_UnknownByElement"); }
    virtual void add_elem_contribution_to_residual(Vec<T> &, const void *) const {
        not_on_gpu("add_elem_contribution_to_residual");
    }

    std::vector<double> element_fields;  ///< 13 per element after call_after_solve
    bool use_fp64_only;                   ///< solve_system with the FP64 PCG only
    int maxit;                            ///< PCG iteration cap
    double timeout_s;                     ///< host wall-clock bound of a solve (0: none)

private:
    struct Cons {
        unsigned node, d;
        double coef, res, penalty;
    };
    static void check(int s, const char *what) {
        if (s != LMTG_OK) {
            std::cerr << "lmtg " << what << ": " << lmtg_status_string(s) << std::endl;
            throw SolveException();
        }
    }
    static void not_on_gpu(const char *what) {
        std::cerr << "GpuFormulationElasticity: " << what << " is not on the GPU path" << std::endl;
    }
    /// "[c*]node[i].dep[d] [+-v]": the coefficient and right-hand side the reference's Constraint
    /// extracts by differentiation (include/formulation/constraint.h:46-93)
    static bool parse_constraint(const std::string &txt0, Cons &c) {
        std::string t;
        for (unsigned i = 0; i < txt0.size(); ++i)
            if (txt0[i] != ' ') t += txt0[i];
        c.coef = 1.0;
        c.res = 0.0;
        std::string::size_type p = t.find("node[");
        if (p == std::string::npos) return false;
        if (p > 0) {
            if (t[p - 1] != '*') return false;
            c.coef = atof(t.substr(0, p - 1).c_str());
        }
        const std::string::size_type q = t.find("].dep[", p);
        const std::string::size_type r = q == std::string::npos ? q : t.find(']', q + 6);
        if (q == std::string::npos || r == std::string::npos) return false;
        c.node = (unsigned)atoi(t.substr(p + 5, q - p - 5).c_str());
        c.d = (unsigned)atoi(t.substr(q + 6, r - q - 6).c_str());
        if (r + 1 < t.size()) {
            const char sign = t[r + 1];
            if (sign != '-' && sign != '+') return false;
            const double v = atof(t.substr(r + 2).c_str());
            c.res = sign == '-' ? v : -v;  // res = -(ex with the unknown set to 0)
        }
        return c.d < 3;
    }
    void upload_mesh() {
        if (!mesh_dirty_) return;
        nn_ = m_->node_list.size();
        ne_ = m_->elem_list.size();
        npe_ = ne_ ? m_->elem_list[0]->nb_nodes_virtual() : 8;
        std::vector<double> pos(3 * nn_);
        for (unsigned i = 0; i < nn_; ++i)
            for (int d = 0; d < 3; ++d) pos[3 * i + d] = m_->node_list[i].pos[d];
        std::vector<uint32_t> conn(npe_ * ne_);
        for (unsigned e = 0; e < ne_; ++e)
            for (unsigned a = 0; a < npe_; ++a)
                conn[npe_ * e + a] = m_->node_list.number(*m_->elem_list[e]->node_virtual(a));
        const int type = npe_ == 8 ? LMTG_ELEM_HEXA8 : LMTG_ELEM_TETRA10;
        check(lmtg_mesh_set(ctx_, type, nn_, pos.empty() ? 0 : &pos[0], ne_, conn.empty() ? 0 : &conn[0]),
              "mesh_set");
        mesh_dirty_ = false;
        have_mat_ = false;
        cons_dirty_ = true;
    }
    void sync_material_and_constraints() {
        if (!have_mat_) check(lmtg_material_set(ctx_, &E_[0], E_.size(), nu_), "material_set");
        check(lmtg_set_levenberg_marquadt(ctx_, levenberg_marquadt), "levenberg_marquadt");
        if (!cons_dirty_) return;
        // lmtg_set_constraints takes one penalty value for all the constraints of a formulation
        std::vector<uint32_t> dof;
        std::vector<double> coef, res;
        double pen = cons_.empty() ? 0.0 : cons_[0].penalty;
        for (unsigned k = 0; k < cons_.size(); ++k) {
            if (cons_[k].penalty != pen) {
                std::cerr << "GpuFormulationElasticity: one penalty value per formulation" << std::endl;
                throw SolveException();
            }
            dof.push_back(3 * cons_[k].node + cons_[k].d);
            coef.push_back(cons_[k].coef);
            res.push_back(cons_[k].res);
        }
        check(lmtg_set_constraints(ctx_, dof.size(), dof.empty() ? 0 : &dof[0], coef.empty() ? 0 : &coef[0],
                                   res.empty() ? 0 : &res[0], cons_.empty() ? 1.0 : pen),
              "set_constraints");
        cons_dirty_ = false;
    }
    std::vector<unsigned> constrained(int dim) const {
        std::vector<unsigned> r;
        for (unsigned k = 0; k < cons_.size(); ++k)
            if (dim < 0 || (int)cons_[k].d == dim) r.push_back(cons_[k].node);
        std::sort(r.begin(), r.end());
        r.erase(std::unique(r.begin(), r.end()), r.end());
        return r;
    }
    Vec<bool> constrained_mask(int dim) const {
        Vec<bool> v;
        v.resize(nn_, false);
        std::vector<unsigned> r = constrained(dim);
        for (unsigned k = 0; k < r.size(); ++k) v[r[k]] = true;
        return v;
    }

    TM *m_;
    lmtg_ctx *ctx_;
    unsigned nn_, ne_, npe_;
    bool allocated_, have_mat_, mesh_dirty_, cons_dirty_;
    std::vector<double> E_;
    double nu_;
    std::vector<Cons> cons_;
    Vec<T> result_, sollicitation_;
    Mat<T, Sym<>, SparseLine<> > K_;
};

}  // namespace LMT

#endif  // LMTPP_GPU_FORMULATION_H
