/*
 * ref_vtu_elast.cpp -- LMT++'s VTU writer on its elasticity mesh (TEST INFRASTRUCTURE).
 *
 * Compiled against the reference's headers by oracle/build_ref.sh into oracle/_ref/ (never
 * into the product).  The mesh type is the reference's generated elasticity mesh carac
 * (include/std_formulations/definition_probleme_elasticity_dep_static.h:72-336, node fields
 * dep, f_nodal, is_on_skin, f_surf; element fields tr_epsilon, epsilon, sigma; global
 * elastic_modulus, density, poisson_ratio, f_vol), the mesh make_rect's Hexa unit cube
 * (include/mesh/make_rect.h:653-679) and the writer write_mesh_vtk<false>
 * (include/mesh/write_mesh_vtk.h:434-655).
 *
 * Usage: ref_vtu_elast <nb_points> <fields.f64> <out.vtu>
 *   fields.f64 = dep (nn x 3), then per element epsilon (6), sigma (6), tr_epsilon (1), then
 *   elastic_modulus and poisson_ratio.
 */
#include "mesh/mesh.h"
#include "std_formulations/definition_probleme_elasticity_dep_static.h"
#include "mesh/make_rect.h"
#include "mesh/write_mesh_vtk.h"
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <vector>

using namespace LMT;

/* element fields, in element order */
struct SetElemFields {
    template <class TE>
    void operator()(TE &e) const {
        const double *v = &(*vals)[13 * (*k)];
        for (int i = 0; i < 6; ++i) e.epsilon[0][i] = v[i];  // Vec<Vec<T,6>,1>: one value per element
        for (int i = 0; i < 6; ++i) e.sigma[0][i] = v[6 + i];
        e.tr_epsilon[0] = v[12];
        ++*k;
    }
    const std::vector<double> *vals;
    unsigned *k;
};

int main(int argc, char **argv) {
    if (argc != 4) {
        fprintf(stderr, "usage: ref_vtu_elast <nb_points> <fields.f64> <out.vtu>\n");
        return 1;
    }
    typedef Mesh<Mesh_carac_pb_elasticity_dep_static<double, 3> > TM;
    TM m;
    const double nbp = atoi(argv[1]);
    make_rect(m, Hexa(), TM::Pvec(0, 0, 0), TM::Pvec(1, 1, 1), TM::Pvec(nbp, nbp, nbp));
    const unsigned nn = m.node_list.size(), ne = m.elem_list.size();
    std::vector<double> f(3 * nn + 13 * ne + 2);
    FILE *in = fopen(argv[2], "rb");
    if (!in || fread(&f[0], sizeof(double), f.size(), in) != f.size()) {
        fprintf(stderr, "cannot read %s\n", argv[2]);
        return 2;
    }
    fclose(in);
    for (unsigned i = 0; i < nn; ++i)
        for (int d = 0; d < 3; ++d) m.node_list[i].dep[d] = f[3 * i + d];
    std::vector<double> ev(f.begin() + 3 * nn, f.begin() + 3 * nn + 13 * ne);
    unsigned k = 0;
    SetElemFields s = {&ev, &k};
    apply(m.elem_list, s);
    m.elastic_modulus = f[3 * nn + 13 * ne];
    m.poisson_ratio = f[3 * nn + 13 * ne + 1];
    std::ofstream os(argv[3]);
    write_mesh_vtk<false>(os, m);
    return 0;
}
