// meshio.cu -- mesh files next to the path (host code only): the Gmsh ASCII format-2 reader of
// LMT++ (read_msh_2, include/mesh/read_msh_2.h:56-235) and its ASCII VTU writer
// (write_mesh_vtk<false>, include/mesh/write_mesh_vtk.h:434-655).
//
// Reader: nodes in file order; elements of the mesh's dimension (3 for Hexa8 / Tetra10, 2 for
// Triangle_6) in file order, lower-dimension elements (faces, edges, points) skipped.  Gmsh's
// Tetra_10 lists its last two edge nodes as (3,2), (3,1); LMT++ as (1,3), (2,3), so they are
// swapped (read_msh_2.h:210).  An element whose Jacobian at var_inter = (0.5, 0.5[, 0.5]) is
// negative is re-ordered with LMT++'s permutation of its type (permutation_if_jac_neg,
// include/mesh/element_Hexa.h:269-294, element_Tetra_10.h:122-147, element_Triangle_6.h:103-115).
// The first tag of each element is returned (LMT++ stores it in the field "tag").
//
// Writer: the layout and number formatting of write_mesh_vtk<false>: C++ stream output of
// doubles (6 significant digits), point arrays then cell arrays then points and cells, one line
// per array with LMT++'s separators (node and global fields: each component followed by a
// space, and one more space after a vector; element fields: a vector's components each
// followed by a space, a scalar alone, then two spaces), cell connectivity 8 indices per line.
#include <sys/stat.h>

#include <charconv>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iterator>
#include <mutex>
#include <ostream>
#include <string>
#include <string_view>
#include <unordered_map>
#include <vector>

#include "lmtg.h"

namespace {

// nodes per element and element dimension of Gmsh element types 1..19
const int kMshNodes[19] = {2, 3, 4, 4, 8, 6, 5, 3, 6, 9, 10, 27, 18, 14, 1, 8, 20, 15, 13};
const int kMshDim[19] = {1, 2, 2, 3, 3, 3, 3, 1, 2, 2, 3, 3, 3, 3, 0, 2, 3, 3, 3};

// derivatives of the shape functions at var_inter = 0.5 (all coordinates), LMT++ node order
void dshape_half(int elem_type, double (*d)[3]) {
    if (elem_type == LMTG_ELEM_HEXA8) {
        // node a at corner (bx, by, bz) in LMT++'s order (0,0,0) (1,0,0) (1,1,0) (0,1,0) (top)
        const int bx[8] = {0, 1, 1, 0, 0, 1, 1, 0}, by[8] = {0, 0, 1, 1, 0, 0, 1, 1},
                  bz[8] = {0, 0, 0, 0, 1, 1, 1, 1};
        for (int a = 0; a < 8; ++a) {
            d[a][0] = (bx[a] ? 1 : -1) * 0.25;
            d[a][1] = (by[a] ? 1 : -1) * 0.25;
            d[a][2] = (bz[a] ? 1 : -1) * 0.25;
        }
    } else if (elem_type == LMTG_ELEM_TETRA10) {
        // barycentric X0 = 1 - x - y - z, X1 = x, X2 = y, X3 = z at (0.5, 0.5, 0.5)
        const double X[4] = {-0.5, 0.5, 0.5, 0.5};
        const double dX[4][3] = {{-1, -1, -1}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
        for (int a = 0; a < 4; ++a)
            for (int k = 0; k < 3; ++k) d[a][k] = (4 * X[a] - 1) * dX[a][k];
        const int e[6][2] = {{0, 1}, {1, 2}, {0, 2}, {0, 3}, {1, 3}, {2, 3}};  // nodes 4..9
        for (int m = 0; m < 6; ++m)
            for (int k = 0; k < 3; ++k)
                d[4 + m][k] = 4 * (dX[e[m][0]][k] * X[e[m][1]] + X[e[m][0]] * dX[e[m][1]][k]);
    } else {  // Triangle_6: X0 = 1 - u - v, X1 = u, X2 = v at (0.5, 0.5)
        const double X[3] = {0.0, 0.5, 0.5};
        const double dX[3][2] = {{-1, -1}, {1, 0}, {0, 1}};
        for (int a = 0; a < 3; ++a) {
            for (int k = 0; k < 2; ++k) d[a][k] = (4 * X[a] - 1) * dX[a][k];
            d[a][2] = 0;
        }
        const int e[3][2] = {{0, 1}, {1, 2}, {2, 0}};  // nodes 3..5
        for (int m = 0; m < 3; ++m) {
            for (int k = 0; k < 2; ++k)
                d[3 + m][k] = 4 * (dX[e[m][0]][k] * X[e[m][1]] + X[e[m][0]] * dX[e[m][1]][k]);
            d[3 + m][2] = 0;
        }
    }
}

double jacobian_det_half(int elem_type, int dim, const std::vector<double> &pos, const uint32_t *nodes, int npe) {
    double d[10][3];
    dshape_half(elem_type, d);
    double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};  // J[i][j] = d x_i / d xi_j
    for (int a = 0; a < npe; ++a)
        for (int i = 0; i < dim; ++i)
            for (int j = 0; j < dim; ++j) J[i][j] += pos[(size_t)dim * nodes[a] + i] * d[a][j];
    if (dim == 2) return J[0][0] * J[1][1] - J[0][1] * J[1][0];
    return J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) - J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
           J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
}

struct ParsedMsh {
    std::vector<double> pos;
    std::vector<uint32_t> conn;
    std::vector<double> tag;
    uint64_t nn = 0, ne = 0;
};

// numbers of one line [p, e): blanks are spaces, tabs and '\r'; false when the line has none left
inline bool next_token(const char *&p, const char *e) {
    while (p < e && (*p == ' ' || *p == '\t' || *p == '\r')) ++p;
    return p < e;
}
inline bool read_ll(const char *&p, const char *e, long long &v) {
    if (!next_token(p, e)) return false;
    char *q = nullptr;
    v = std::strtoll(p, &q, 10);
    if (q == p || q > e) return false;
    p = q;
    return true;
}
inline bool read_d(const char *&p, const char *e, double &v) {
    if (!next_token(p, e)) return false;
    char *q = nullptr;
    v = std::strtod(p, &q);  // correctly rounded, as the stream extraction of the reference
    if (q == p || q > e) return false;
    p = q;
    return true;
}

int parse_msh(const char *path, int elem_type, ParsedMsh &out) {
    int want_type, npe, dim;
    if (elem_type == LMTG_ELEM_HEXA8) { want_type = 5; npe = 8; dim = 3; }
    else if (elem_type == LMTG_ELEM_TETRA10) { want_type = 11; npe = 10; dim = 3; }
    else if (elem_type == LMTG_ELEM_TRIANGLE6) { want_type = 9; npe = 6; dim = 2; }
    else return LMTG_ERR_ARG;
    std::ifstream is(path, std::ios::binary);
    if (!is.is_open()) return LMTG_ERR_ARG;
    std::string buf((std::istreambuf_iterator<char>(is)), std::istreambuf_iterator<char>());
    std::unordered_map<long long, uint32_t> node_of;  // file number -> index in file order
    int section = 0;  // 1 nodes, 2 elements
    bool ended = false, skip_count = false;
    const char *p0 = buf.c_str(), *end = p0 + buf.size();
    for (const char *b = p0; b < end && !ended;) {
        const char *e = static_cast<const char *>(std::memchr(b, '\n', end - b));
        if (!e) e = end;
        const std::string_view line(b, e - b);
        const char *next = e < end ? e + 1 : end;
        if (skip_count) {  // the count line after $Nodes / $Elements
            skip_count = false;
        } else if (line.find("$EndNodes") != std::string_view::npos) {
            section = 0;
        } else if (line.find("$EndElements") != std::string_view::npos) {
            ended = true;
        } else if (line.find("$Nodes") != std::string_view::npos) {
            section = 1;
            skip_count = true;
        } else if (line.find("$Elements") != std::string_view::npos) {
            section = 2;
            skip_count = true;
        } else if (section == 1) {
            const char *q = b;
            long long num;
            double x[3] = {0, 0, 0};
            if (!read_ll(q, e, num)) return LMTG_ERR_ARG;
            for (int k = 0; k < dim; ++k)
                if (!read_d(q, e, x[k])) return LMTG_ERR_ARG;
            node_of[num] = (uint32_t)out.nn++;
            for (int k = 0; k < dim; ++k) out.pos.push_back(x[k]);
        } else if (section == 2) {
            const char *q = b;
            long long num, type, ntags;
            if (!read_ll(q, e, num) || !read_ll(q, e, type) || !read_ll(q, e, ntags) || type < 1 || type > 19 ||
                ntags < 0 || ntags > 64)
                return LMTG_ERR_ARG;
            double tag0 = 0.0;
            for (long long k = 0; k < ntags; ++k) {
                double t;
                if (!read_d(q, e, t)) return LMTG_ERR_ARG;
                if (k == 0) tag0 = t;
            }
            if (kMshDim[type - 1] == dim) {  // faces, edges, points of the mesh are skipped
                if (type != want_type) return LMTG_ERR_UNSUPPORTED;
                uint32_t v[10];
                for (int a = 0; a < kMshNodes[type - 1]; ++a) {
                    long long nb;
                    if (!read_ll(q, e, nb)) return LMTG_ERR_ARG;
                    auto it = node_of.find(nb);
                    if (it == node_of.end()) return LMTG_ERR_ARG;
                    v[a] = it->second;
                }
                if (type == 11) std::swap(v[8], v[9]);
                if (jacobian_det_half(elem_type, dim, out.pos, v, npe) < 0) {
                    static const int ph[8] = {0, 3, 2, 1, 4, 7, 6, 5};
                    static const int pt[10] = {0, 1, 3, 2, 4, 8, 7, 6, 5, 9};
                    static const int pr[6] = {5, 4, 3, 2, 1, 0};
                    const int *pm = type == 5 ? ph : type == 11 ? pt : pr;
                    uint32_t w[10];
                    for (int a = 0; a < npe; ++a) w[a] = v[pm[a]];
                    for (int a = 0; a < npe; ++a) v[a] = w[a];
                }
                out.conn.insert(out.conn.end(), v, v + npe);
                out.tag.push_back(tag0);
                ++out.ne;
            }
        }
        b = next;
    }
    return ended ? LMTG_OK : LMTG_ERR_ARG;
}

// The parse of the last sizing call (lmtg_read_msh with no buffers), reused by the call that
// fills the buffers when the file is unchanged (same path, element type, size and time).
struct MshCache {
    std::mutex mu;
    bool valid = false;
    std::string path;
    int elem_type = 0;
    long long size = -1, mtime_ns = -1;
    ParsedMsh m;
} g_msh_cache;

bool file_stamp(const char *path, long long &size, long long &mtime_ns) {
    struct stat st;
    if (stat(path, &st) != 0) return false;
    size = (long long)st.st_size;
    mtime_ns = (long long)st.st_mtim.tv_sec * 1000000000ll + st.st_mtim.tv_nsec;
    return true;
}

// Text written into memory and to the file at once.  Doubles are formatted as "%g" (6
// significant digits), which is what a C++ stream with default flags does (the reference's
// os << value).
struct Out {
    std::string s;
    Out &operator<<(const char *t) { s += t; return *this; }
    Out &operator<<(char c) { s += c; return *this; }
    Out &operator<<(uint64_t v) {
        char b[24];
        const int n = std::snprintf(b, sizeof b, "%llu", (unsigned long long)v);
        s.append(b, n);
        return *this;
    }
    Out &operator<<(uint32_t v) { return *this << (uint64_t)v; }
    Out &operator<<(int v) {
        char b[16];
        const int n = std::snprintf(b, sizeof b, "%d", v);
        s.append(b, n);
        return *this;
    }
};
void put(Out &os, double v) {
    char b[32];
    // std::to_chars with a precision formats as printf's "%.6g" in the "C" locale
    const auto r = std::to_chars(b, b + sizeof b, v, std::chars_format::general, 6);
    os.s.append(b, r.ptr - b);
}

}  // namespace

extern "C" int lmtg_read_msh(const char *path, int elem_type, uint64_t *nn, double *pos, uint64_t *ne,
                             uint32_t *conn, double *tag) {
    try {
        if (!path || !nn || !ne) return LMTG_ERR_ARG;
        const bool fill = pos || conn || tag;
        long long size = -1, mtime = -1;
        if (!file_stamp(path, size, mtime)) return LMTG_ERR_ARG;
        std::lock_guard<std::mutex> lock(g_msh_cache.mu);
        MshCache &C = g_msh_cache;
        if (!(C.valid && C.path == path && C.elem_type == elem_type && C.size == size && C.mtime_ns == mtime)) {
            C.valid = false;
            C.m = ParsedMsh();
            const int rc = parse_msh(path, elem_type, C.m);
            if (rc != LMTG_OK) {
                C.m = ParsedMsh();
                return rc;
            }
            C.valid = true;
            C.path = path;
            C.elem_type = elem_type;
            C.size = size;
            C.mtime_ns = mtime;
        }
        const ParsedMsh &m = C.m;
        if (fill && (*nn != m.nn || *ne != m.ne)) return LMTG_ERR_ARG;  // sizes from the first call
        *nn = m.nn;
        *ne = m.ne;
        if (pos && !m.pos.empty()) std::memcpy(pos, m.pos.data(), m.pos.size() * sizeof(double));
        if (conn && !m.conn.empty()) std::memcpy(conn, m.conn.data(), m.conn.size() * sizeof(uint32_t));
        if (tag && !m.tag.empty()) std::memcpy(tag, m.tag.data(), m.tag.size() * sizeof(double));
        if (fill) {  // the buffers are filled: drop the parse
            C.valid = false;
            C.m = ParsedMsh();
        }
        return LMTG_OK;
    } catch (...) {
        return LMTG_ERR_NOMEM;
    }
}

extern "C" int lmtg_write_vtu(const char *path, int elem_type, uint64_t nn, const double *pos, uint64_t ne,
                              const uint32_t *conn, int npf, const char *const *pnames, const int *pncomp,
                              const double *const *pvals, int ncf, const char *const *cnames, const int *cncomp,
                              const int *ckind, const double *const *cvals) {
    try {
        int npe, dim, cell_type;
        if (elem_type == LMTG_ELEM_HEXA8) { npe = 8; dim = 3; cell_type = 12; }
        else if (elem_type == LMTG_ELEM_TETRA10) { npe = 10; dim = 3; cell_type = 24; }
        else if (elem_type == LMTG_ELEM_TRIANGLE6) { npe = 6; dim = 2; cell_type = 22; }
        else return LMTG_ERR_ARG;
        if (!path || (nn && !pos) || (ne && !conn) || npf < 0 || ncf < 0) return LMTG_ERR_ARG;
        for (int f = 0; f < npf; ++f)
            if (!pnames[f] || pncomp[f] < 1 || (nn && !pvals[f])) return LMTG_ERR_ARG;
        for (int f = 0; f < ncf; ++f)
            if (!cnames[f] || cncomp[f] < 1 || ckind[f] < 0 || ckind[f] > 2 || (ne && !cvals[f])) return LMTG_ERR_ARG;
        for (uint64_t i = 0; i < ne * (uint64_t)npe; ++i)
            if (conn[i] >= nn) return LMTG_ERR_ARG;
        std::ofstream file(path, std::ios::binary);
        if (!file.is_open()) return LMTG_ERR_ARG;
        Out os;
        os << "<?xml version='1.0' ?>\n";
        os << "<VTKFile type='UnstructuredGrid' byte_order='LittleEndian'>\n";
        os << "    <UnstructuredGrid>\n";
        os << "        <Piece NumberOfPoints='" << nn << "' NumberOfCells='" << ne << "'>\n";
        os << "            <PointData>\n";
        for (int f = 0; f < (nn ? npf : 0); ++f) {  // the reference lists no arrays for an empty mesh
            os << "                <DataArray Name='" << pnames[f] << "' NumberOfComponents='" << pncomp[f]
               << "' type='Float64' format='ascii'>\n";
            for (uint64_t i = 0; i < nn; ++i) {
                for (int k = 0; k < pncomp[f]; ++k) {
                    put(os, pvals[f][(size_t)pncomp[f] * i + k]);
                    os << ' ';
                }
                if (pncomp[f] > 1) os << ' ';
            }
            os << "\n                </DataArray>\n";
        }
        os << "            </PointData> \n";
        os << "            <CellData>\n";
        for (int f = 0; f < (ne ? ncf : 0); ++f) {
            os << "                <DataArray Name='" << cnames[f] << "' NumberOfComponents='" << cncomp[f]
               << "' type='" << (ckind[f] == 2 ? "UInt32" : "Float64") << "' format='ascii'>\n";
            for (uint64_t e = 0; e < ne; ++e) {
                const double *v = cvals[f] + (size_t)cncomp[f] * e;
                if (ckind[f] == 0) {  // element field: "a b c " or "a", then two spaces
                    if (cncomp[f] > 1)
                        for (int k = 0; k < cncomp[f]; ++k) { put(os, v[k]); os << ' '; }
                    else
                        put(os, v[0]);
                    os << "  ";
                } else if (ckind[f] == 1) {  // global field repeated per element: node rule
                    for (int k = 0; k < cncomp[f]; ++k) { put(os, v[k]); os << ' '; }
                    if (cncomp[f] > 1) os << ' ';
                } else {  // integer (the element group)
                    for (int k = 0; k < cncomp[f]; ++k) os << (uint32_t)v[k] << ' ';
                }
            }
            os << "\n                </DataArray>\n";
        }
        os << "            </CellData> \n";
        os << "            <Points>\n";
        os << "                <DataArray NumberOfComponents='3' type='Float64' format='ascii'>\n";
        for (uint64_t i = 0; i < nn; ++i) {
            const double *x = pos + (size_t)dim * i;
            put(os, x[0]);
            os << ' ';
            put(os, x[1]);
            os << ' ';
            put(os, dim > 2 ? x[2] : x[0] * 0.0);  // the reference writes pos[0] * 0 for 2D meshes
            os << '\n';
        }
        os << "                </DataArray>\n";
        os << "            </Points> \n";
        os << "            <Cells>\n";
        auto list = [&](const char *name, uint64_t count, auto value) {
            os << "                <DataArray Name='" << name << "' type='Int32' format='ascii'>\n";
            for (uint64_t i = 0; i < count; ++i)
                os << (uint64_t)value(i) << ((i % 8) == 7 || i + 1 == count ? '\n' : ' ');
            os << "                </DataArray>\n";
        };
        list("connectivity", ne * (uint64_t)npe, [&](uint64_t i) { return conn[i]; });
        list("offsets", ne, [&](uint64_t i) { return (uint64_t)npe * (i + 1); });
        list("types", ne, [&](uint64_t) { return cell_type; });
        os << "            </Cells>\n";
        os << "        </Piece>\n";
        os << "    </UnstructuredGrid>\n";
        os << "    <AppendedData encoding='base64'>\n";
        os << "        _\n";
        os << "    </AppendedData>\n";
        os << "</VTKFile>\n";
        file.write(os.s.data(), (std::streamsize)os.s.size());
        file.close();
        return file ? LMTG_OK : LMTG_ERR_ARG;
    } catch (...) {
        return LMTG_ERR_NOMEM;
    }
}
