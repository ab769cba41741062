/*
 * ref_meshio.cpp -- runs LMT++'s own mesh-file code (TEST INFRASTRUCTURE).
 *
 * Compiled against the reference's headers by oracle/build_ref.sh into oracle/_ref/ (never
 * into the product).  What comes from the reference here:
 *   - the Gmsh reader     read_msh_2                     include/mesh/read_msh_2.h:56-235, 376-383
 *   - the VTU writer      write_mesh_vtk<false>          include/mesh/write_mesh_vtk.h:434-655
 *   - the meshes          make_rect and MeshCaracStd
 *
 * Usage:
 *   ref_meshio msh hexa|tetra10|tri6 <file.msh> <outdir>
 *       reads the file, writes pos.f64 (nn x dim), conn.u32 (ne x npe) and info.txt (nn ne)
 *   ref_meshio vtu_std hexa|tetra10|tri6 <nb_points> <out.vtu>
 *       the unit cube / square of make_rect with no fields; writes the VTU file
 */
#include "mesh/meshcaracstd.h"
#include "mesh/make_rect.h"
#include "mesh/Pyramid.h"
namespace LMT {
/* read_msh_2 instantiates permutation_if_jac_neg for every Gmsh type, and the reference
 * defines none for Pyramid; this no-op lets it compile.  No test file holds a pyramid. */
template <class TNode>
void permutation_if_jac_neg(const Pyramid &, TNode **) {}
}  // namespace LMT
#include "mesh/read_msh_2.h"
#include "mesh/write_mesh_vtk.h"
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <string>
#include <vector>

using namespace LMT;

template <class T>
static void dump(const std::string &path, const std::vector<T> &v) {
    FILE *f = fopen(path.c_str(), "wb");
    if (!f) { fprintf(stderr, "cannot write %s\n", path.c_str()); exit(2); }
    if (v.size()) fwrite(&v[0], sizeof(T), v.size(), f);
    fclose(f);
}

template <class TM>
static int read_and_dump(const char *file, int npe, const std::string &out) {
    TM m;
    try {
        read_msh_2(m, std::string(file));
    } catch (const std::exception &e) {
        fprintf(stderr, "read_msh_2: %s\n", e.what());
        return 3;
    }
    const unsigned nn = m.node_list.size(), ne = m.elem_list.size(), dim = TM::dim;
    std::vector<double> pos(dim * nn);
    for (unsigned i = 0; i < nn; ++i)
        for (unsigned d = 0; d < dim; ++d) pos[dim * i + d] = m.node_list[i].pos[d];
    std::vector<unsigned> conn;
    for (unsigned e = 0; e < ne; ++e) {
        if ((int)m.elem_list[e]->nb_nodes_virtual() != npe) {
            fprintf(stderr, "element %u has %u nodes\n", e, m.elem_list[e]->nb_nodes_virtual());
            return 4;
        }
        for (int a = 0; a < npe; ++a) conn.push_back(m.node_list.number(*m.elem_list[e]->node_virtual(a)));
    }
    dump(out + "/pos.f64", pos);
    dump(out + "/conn.u32", conn);
    FILE *f = fopen((out + "/info.txt").c_str(), "w");
    fprintf(f, "%u %u\n", nn, ne);
    fclose(f);
    return 0;
}

int main(int argc, char **argv) {
    const std::string mode = argc >= 2 ? argv[1] : "";
    if (mode == "msh" && argc == 5) {
        const std::string el = argv[2];
        if (el == "hexa") return read_and_dump<Mesh<MeshCaracStd<3, 3, 1, double, 1> > >(argv[3], 8, argv[4]);
        if (el == "tetra10") return read_and_dump<Mesh<MeshCaracStd<3, 3, 0, double, 2> > >(argv[3], 10, argv[4]);
        if (el == "tri6") return read_and_dump<Mesh<MeshCaracStd<2, 2, 0, double, 2> > >(argv[3], 6, argv[4]);
    }
    if (mode == "vtu_std" && argc == 5) {
        const std::string el = argv[2];
        const double nbp = atoi(argv[3]);
        std::ofstream os(argv[4]);
        if (el == "hexa") {
            typedef Mesh<MeshCaracStd<3, 3, 1, double, 1> > TM;
            TM m;
            make_rect(m, Hexa(), TM::Pvec(0, 0, 0), TM::Pvec(1, 1, 1), TM::Pvec(nbp, nbp, nbp));
            write_mesh_vtk<false>(os, m);
            return 0;
        }
        if (el == "tetra10") {
            typedef Mesh<MeshCaracStd<3, 3, 0, double, 2> > TM;
            TM m;
            make_rect(m, Tetra_10(), TM::Pvec(0, 0, 0), TM::Pvec(1, 1, 1), TM::Pvec(nbp, nbp, nbp));
            write_mesh_vtk<false>(os, m);
            return 0;
        }
        if (el == "tri6") {
            typedef Mesh<MeshCaracStd<2, 2, 0, double, 2> > TM;
            TM m;
            make_rect(m, Triangle_6(), TM::Pvec(0, 0), TM::Pvec(1, 1), TM::Pvec(nbp, nbp));
            write_mesh_vtk<false>(os, m);
            return 0;
        }
    }
    fprintf(stderr, "usage: ref_meshio msh hexa|tetra10|tri6 <file.msh> <outdir>\n"
                    "       ref_meshio vtu_std hexa|tetra10|tri6 <nb_points> <out.vtu>\n");
    return 1;
}
