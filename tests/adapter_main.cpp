// Builds the LMT++-side adapter (include/lmtpp/gpu_formulation.h) the way the reference builds
// its own code, on the reference's make_rect mesh: the program an LMT++ user would write.  The
// CPU test compiles and links it; running it needs a GPU (it solves the Hexa8 example problem
// and prints the largest displacement).
#include "mesh/meshcaracstd.h"
#include "mesh/make_rect.h"
#include "lmtpp/gpu_formulation.h"

using namespace LMT;

int main(int argc, char **argv) {
    typedef Mesh<MeshCaracStd<3, 3, 1, double, 1> > TM;
    TM m;
    const unsigned nb = argc > 1 ? atoi(argv[1]) : 11;
    make_rect(m, Hexa(), TM::Pvec(0, 0, 0), TM::Pvec(1, 1, 1), TM::Pvec(nb, nb, nb));
    GpuFormulationElasticity<TM> gf(m);
    FormulationAncestor<double> *f = &gf;  // the reference's virtual API from here on
    gf.set_elastic_modulus(210000.0);
    gf.set_poisson_ratio(0.3);
    for (unsigned i = 0; i < m.node_list.size(); ++i)
        if (m.node_list[i].pos[0] < 1e-6)
            for (int d = 0; d < 3; ++d) f->add_constraint("node[" + to_string(i) + "].dep[" + to_string(d) + "]", 1e5);
    f->allocate_matrices();
    std::vector<unsigned> faces;  // Quad4 faces on x = 1: Hexa child 5, nodes 1 2 6 5
    static const int ch[4] = {1, 2, 6, 5};
    for (unsigned e = 0; e < m.elem_list.size(); ++e) {
        bool on = true;
        for (int a = 0; a < 4; ++a) on = on && m.elem_list[e]->node_virtual(ch[a])->pos[0] > 1 - 1e-6;
        if (on)
            for (int a = 0; a < 4; ++a) faces.push_back(m.node_list.number(*m.elem_list[e]->node_virtual(ch[a])));
    }
    const double t[3] = {1, 0, 0};
    gf.add_skin_traction(faces, t);
    f->solve(1e-12);
    Mat<double, Sym<>, SparseLine<> > *K = 0;
    f->get_mat(K);
    Vec<double> &u = f->get_result();
    std::cout << "n " << K->nb_rows() << " max|u| " << max(abs(u)) << " max_diag " << f->max_diag << std::endl;
    return 0;
}
