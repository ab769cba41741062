// abi.cu -- the extern "C" entry points declared in include/lmtg.h.
//
// Host-side orchestration of one formulation on one GPU, mirroring the calls a user makes on
// LMT++'s FormulationAncestor (include/formulation/formulation_ancestor.h:18-262):
// allocate_matrices -> assemble -> solve_system / solve -> get_result.  Every entry point
// catches internal errors and returns a status; nothing throws across the ABI.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <exception>
#include <new>

#include "lmtg_internal.cuh"
#include "amg.cuh"
#include "spmv_bulk.cuh"

using namespace lmtg;

namespace {

template <class F>
int guard(lmtg_ctx *c, F &&f) {
    if (!c) return LMTG_ERR_ARG;
    try {
        cudaError_t e = cudaSetDevice(c->device);
        if (e != cudaSuccess) throw Error{LMTG_ERR_CUDA, cudaGetErrorString(e)};
        int s = f();
        if (s == LMTG_OK) c->err.clear();
        return s;
    } catch (const Error &e) {
        c->err = e.msg;
        return e.status;
    } catch (const std::bad_alloc &) {
        c->err = "host allocation failed";
        return LMTG_ERR_NOMEM;
    } catch (const std::exception &e) {
        c->err = e.what();
        return LMTG_ERR_CUDA;
    }
}

template <class T>
void upload(lmtg_ctx *c, DBuf<T> &d, const T *h, size_t n) {
    d.alloc(n);
    if (n) LMTG_CUDA(cudaMemcpyAsync(d.p, h, n * sizeof(T), cudaMemcpyHostToDevice, c->stream));
}

// Quad4 consistent loads of a uniform traction.  The reference integrates skin terms when it
// generates add_skin_elem_matrix (formal_lf/formulation.py:400-438, element.integration): with the
// Python rule of the face element of order >= 2, for Quad gauss_points[3] of
// formulations/element_Quad.py:70-75, abscissae (1 -+ sqrt(1/3))/2 at full precision, weights 1/4.
void quad4_loads(const double *pos, const uint32_t *q, const double t[3], double *F, const double *pressure = nullptr) {
    const double A = 0.21132486540518711775, B = 0.78867513459481288225;
    const double gp[4][2] = {{B, B}, {A, B}, {B, A}, {A, A}};
    for (int g = 0; g < 4; ++g) {
        const double u = gp[g][0], v = gp[g][1];
        const double N[4] = {(1 - u) * (1 - v), u * (1 - v), u * v, (1 - u) * v};
        const double du[4] = {-(1 - v), 1 - v, v, -v};
        const double dv[4] = {-(1 - u), -u, u, 1 - u};
        double tu[3] = {0, 0, 0}, tv[3] = {0, 0, 0};
        for (int a = 0; a < 4; ++a)
            for (int d = 0; d < 3; ++d) {
                tu[d] += pos[3 * (uint64_t)q[a] + d] * du[a];
                tv[d] += pos[3 * (uint64_t)q[a] + d] * dv[a];
            }
        const double nx = tu[1] * tv[2] - tu[2] * tv[1], ny = tu[2] * tv[0] - tu[0] * tv[2],
                     nz = tu[0] * tv[1] - tu[1] * tv[0];
        const double nl = std::sqrt(nx * nx + ny * ny + nz * nz), ds = nl * 0.25;
        // pressure: p dS_normal, the unit normal cross(d x / d xi0, d x / d xi1) of the face's
        // node order (formal_lf/element.py:467-474)
        const double tg[3] = {pressure ? *pressure * nx / nl : t[0], pressure ? *pressure * ny / nl : t[1],
                              pressure ? *pressure * nz / nl : t[2]};
        for (int a = 0; a < 4; ++a)
            for (int d = 0; d < 3; ++d) F[3 * (uint64_t)q[a] + d] += N[a] * tg[d] * ds;
    }
}

// Triangle_6 consistent loads of a uniform traction, with the Python rule the reference's
// generated skin routines integrate by (formal_lf/formulation.py:400-438): gauss_points[4] of
// formulations/element_Triangle_6.py:92-99, 6 points.
void tri6_loads(const double *pos, const uint32_t *q, const double t[3], double *F, const double *pressure = nullptr) {
    const double a = 0.445948490915965, b = 0.091576213509771;
    const double wa = 0.111690794839005, wb = 0.054975871827661;
    const double gp[6][2] = {{a, a}, {1.0 - 2.0 * a, a}, {a, 1.0 - 2.0 * a},
                             {b, b}, {1.0 - 2.0 * b, b}, {b, 1.0 - 2.0 * b}};
    const double gw[6] = {wa, wa, wa, wb, wb, wb};
    for (int g = 0; g < 6; ++g) {
        const double u = gp[g][0], v = gp[g][1], X0 = 1 - u - v;
        const double N[6] = {X0 * (2 * X0 - 1), u * (2 * u - 1), v * (2 * v - 1),
                             4 * X0 * u,        4 * u * v,       4 * v * X0};
        const double du[6] = {-(4 * X0 - 1), 4 * u - 1, 0, 4 * (X0 - u), 4 * v, -4 * v};
        const double dv[6] = {-(4 * X0 - 1), 0, 4 * v - 1, -4 * u, 4 * u, 4 * (X0 - v)};
        double tu[3] = {0, 0, 0}, tv[3] = {0, 0, 0};
        for (int a = 0; a < 6; ++a)
            for (int d = 0; d < 3; ++d) {
                tu[d] += pos[3 * (uint64_t)q[a] + d] * du[a];
                tv[d] += pos[3 * (uint64_t)q[a] + d] * dv[a];
            }
        const double nx = tu[1] * tv[2] - tu[2] * tv[1], ny = tu[2] * tv[0] - tu[0] * tv[2],
                     nz = tu[0] * tv[1] - tu[1] * tv[0];
        const double nl = std::sqrt(nx * nx + ny * ny + nz * nz), ds = nl * gw[g];
        const double tg[3] = {pressure ? *pressure * nx / nl : t[0], pressure ? *pressure * ny / nl : t[1],
                              pressure ? *pressure * nz / nl : t[2]};
        for (int a = 0; a < 6; ++a)
            for (int d = 0; d < 3; ++d) F[3 * (uint64_t)q[a] + d] += N[a] * tg[d] * ds;
    }
}

}  // namespace

extern "C" {

const char *lmtg_status_string(int s) {
    switch (s) {
        case LMTG_OK: return "ok";
        case LMTG_ERR_ARG: return "invalid argument";
        case LMTG_ERR_CUDA: return "CUDA error";
        case LMTG_ERR_STATE: return "call out of order";
        case LMTG_ERR_NOT_CONVERGED: return "not converged";
        case LMTG_ERR_TIMEOUT: return "timeout";
        case LMTG_ERR_NAN: return "NaN or Inf in the solver";
        case LMTG_ERR_NOMEM: return "out of device memory";
        case LMTG_ERR_UNSUPPORTED: return "unsupported";
        default: return "unknown status";
    }
}

const char *lmtg_last_error(const lmtg_ctx *c) { return c ? c->err.c_str() : "null context"; }

int lmtg_create(int device, lmtg_ctx **out) {
    if (!out) return LMTG_ERR_ARG;
    *out = nullptr;
    lmtg_ctx *c = nullptr;
    try {
        c = new lmtg_ctx();
    } catch (...) {
        return LMTG_ERR_NOMEM;
    }
    c->device = device;
    int s = guard(c, [&] {
        LMTG_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
        LMTG_CUDA(cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device));
        c->scal.alloc(2);
        LMTG_CUDA(cudaMemset(c->scal.p, 0, c->scal.bytes()));
        LMTG_CUDA(cudaMallocHost(&c->h_scal, 2 * sizeof(PcgScalars)));
        memset(c->h_scal, 0, 2 * sizeof(PcgScalars));
        c->partials.alloc((size_t)5 * c->sm_count * 16);
        return LMTG_OK;
    });
    if (s != LMTG_OK) {
        lmtg_destroy(c);
        return s;
    }
    *out = c;
    return LMTG_OK;
}

int lmtg_destroy(lmtg_ctx *c) {
    if (!c) return LMTG_OK;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->h_scal) cudaFreeHost(c->h_scal);
    batch_free(c);
    recal_free(c);
    amg_free(c);
    samg_free(c);
    diff_graphs_free(c);
    if (c->aux_stream) {
        cudaStreamSynchronize(c->aux_stream);
        cudaStreamDestroy(c->aux_stream);
    }
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;  // DBuf destructors free device memory
    return LMTG_OK;
}

int lmtg_make_rect_hexa(const double X0[3], const double X1[3], const uint32_t nbp[3], double *pos,
                        uint32_t *conn) {
    if (!X0 || !X1 || !nbp || !pos || !conn) return LMTG_ERR_ARG;
    // Nodes: the reference iterator accumulates pos += inc along every axis, x fastest
    // (include/util/rectilinear_iterator.h:20-45); elements as make_rect.h:667-677.
    std::vector<double> ax[3];
    for (int d = 0; d < 3; ++d) {
        if (nbp[d] < 2) return LMTG_ERR_ARG;
        const double lo = std::fmin(X0[d], X1[d]), hi = std::fmax(X0[d], X1[d]);
        const double inc = (hi - lo) / ((double)nbp[d] - 1.0);
        const double step = inc + (inc == 0.0 ? 1.0 : 0.0), upper = hi + step * 0.5;
        for (double p = lo; p < upper; p += step) {
            if (ax[d].size() == nbp[d]) return LMTG_ERR_ARG;
            ax[d].push_back(p);
        }
        if (ax[d].size() != nbp[d]) return LMTG_ERR_ARG;
    }
    const uint64_t nx = nbp[0], ny = nbp[1], nz = nbp[2], sxy = nx * ny;
    if (nx * ny * nz >= (1ull << 32)) return LMTG_ERR_UNSUPPORTED;
    uint64_t n = 0;
    for (uint64_t i = 0; i < nz; ++i)
        for (uint64_t j = 0; j < ny; ++j)
            for (uint64_t k = 0; k < nx; ++k, ++n) {
                pos[3 * n] = ax[0][k];
                pos[3 * n + 1] = ax[1][j];
                pos[3 * n + 2] = ax[2][i];
            }
    uint64_t e = 0;
    for (uint64_t i = 0; i + 1 < nz; ++i)
        for (uint64_t j = 0; j + 1 < ny; ++j)
            for (uint64_t k = 0; k + 1 < nx; ++k, ++e) {
                const uint64_t b = i * sxy + j * nx + k;
                uint32_t *c = conn + 8 * e;
                c[0] = (uint32_t)b;
                c[1] = (uint32_t)(b + 1);
                c[2] = (uint32_t)(b + 1 + nx);
                c[3] = (uint32_t)(b + nx);
                c[4] = (uint32_t)(b + sxy);
                c[5] = (uint32_t)(b + sxy + 1);
                c[6] = (uint32_t)(b + sxy + 1 + nx);
                c[7] = (uint32_t)(b + sxy + nx);
            }
    return LMTG_OK;
}

int lmtg_make_rect_tetra10(const double X0_[3], const double X1_[3], const uint32_t nbp[3],
                           uint64_t *nn_out, uint64_t *ne_out, double *pos, uint32_t *conn) {
    if (!X0_ || !X1_ || !nbp || !nn_out || !ne_out) return LMTG_ERR_ARG;
    // vertex positions of the reference element and the 6 tetrahedra of a cube: translation (in
    // units of incr) and basis columns, as make_rect.h:466-543
    static const double rela[10][3] = {{0, 0, 0},     {1, 0, 0},     {0, 1, 0},   {0, 0, 1},
                                       {0.5, 0, 0},   {0.5, 0.5, 0}, {0, 0.5, 0}, {0, 0, 0.5},
                                       {0.5, 0, 0.5}, {0, 0.5, 0.5}};
    static const int trs[6][3] = {{0, 0, 0}, {1, 1, 0}, {1, 0, 0}, {1, 0, 1}, {1, 1, 0}, {1, 1, 1}};
    static const int bas[6][3][3] = {{{1, 0, 0}, {0, 1, 0}, {0, 0, 1}},
                                     {{-1, 0, 0}, {0, -1, 0}, {0, -1, 1}},
                                     {{-1, 0, 1}, {-1, 1, 0}, {0, 0, 1}},
                                     {{-1, 0, 0}, {-1, 1, 0}, {-1, 1, -1}},
                                     {{-1, 0, 0}, {-1, 0, 1}, {0, -1, 1}},
                                     {{-1, 0, 0}, {0, -1, 0}, {0, 0, -1}}};
    static const int perm[10] = {0, 1, 3, 2, 4, 8, 7, 6, 5, 9};
    uint64_t ne3[3];
    double X0[3], incr[3];
    for (int d = 0; d < 3; ++d) {
        if (nbp[d] < 2) return LMTG_ERR_ARG;
        X0[d] = std::fmin(X0_[d], X1_[d]);
        const double x1 = std::fmax(X0_[d], X1_[d]);
        ne3[d] = nbp[d] - 1;
        incr[d] = (x1 - X0[d]) / (double)ne3[d];
    }
    const uint64_t gx = 2 * ne3[0] + 1, gy = 2 * ne3[1] + 1, gz = 2 * ne3[2] + 1;
    const uint64_t nn = gx * gy * gz, ne = 6 * ne3[0] * ne3[1] * ne3[2];
    if (nn >= (1ull << 32)) return LMTG_ERR_UNSUPPORTED;
    *nn_out = nn;
    *ne_out = ne;
    if (!pos || !conn) return LMTG_OK;
    std::vector<uint32_t> id(nn, 0xffffffffu);
    uint32_t next = 0;
    uint64_t e = 0;
    for (uint64_t i = 0; i < ne3[2]; ++i)
        for (uint64_t j = 0; j < ne3[1]; ++j)
            for (uint64_t k = 0; k < ne3[0]; ++k) {
                const double O[3] = {X0[0] + k * incr[0], X0[1] + j * incr[1], X0[2] + i * incr[2]};
                const uint64_t kk[3] = {k, j, i};
                for (int s = 0; s < 6; ++s) {
                    uint32_t vn[10];
                    for (int t = 0; t < 10; ++t) {
                        double p[3];
                        int64_t g[3];
                        for (int r = 0; r < 3; ++r) {
                            const double w = bas[s][0][r] * rela[t][0] + bas[s][1][r] * rela[t][1] +
                                             bas[s][2][r] * rela[t][2];
                            const double base = s == 0 ? O[r] : O[r] + trs[s][r] * incr[r];
                            p[r] = base + incr[r] * w;
                            g[r] = 2 * (int64_t)kk[r] + 2 * trs[s][r] + (int64_t)std::llround(2 * w);
                        }
                        const uint64_t key = ((uint64_t)g[2] * gy + (uint64_t)g[1]) * gx + (uint64_t)g[0];
                        if (id[key] == 0xffffffffu) {
                            id[key] = next;
                            for (int r = 0; r < 3; ++r) pos[3ull * next + r] = p[r];
                            ++next;
                        }
                        vn[t] = id[key];
                    }
                    double a[3], b[3], cc[3];
                    for (int r = 0; r < 3; ++r) {
                        a[r] = pos[3ull * vn[1] + r] - pos[3ull * vn[0] + r];
                        b[r] = pos[3ull * vn[2] + r] - pos[3ull * vn[0] + r];
                        cc[r] = pos[3ull * vn[3] + r] - pos[3ull * vn[0] + r];
                    }
                    const double det = a[0] * (b[1] * cc[2] - b[2] * cc[1]) -
                                       a[1] * (b[0] * cc[2] - b[2] * cc[0]) +
                                       a[2] * (b[0] * cc[1] - b[1] * cc[0]);
                    for (int t = 0; t < 10; ++t) conn[10 * e + t] = det < 0 ? vn[perm[t]] : vn[t];
                    ++e;
                }
            }
    return next == nn ? LMTG_OK : LMTG_ERR_ARG;
}

int lmtg_mesh_set(lmtg_ctx *c, int elem_type, uint64_t nn, const double *pos, uint64_t ne,
                  const uint32_t *conn) {
    return guard(c, [&] {
        LMTG_CHECK(elem_type == LMTG_ELEM_HEXA8 || elem_type == LMTG_ELEM_TETRA10,
                   LMTG_ERR_UNSUPPORTED, "element type not supported");
        LMTG_CHECK(pos && conn && nn > 0 && ne > 0, LMTG_ERR_ARG, "empty mesh");
        LMTG_CHECK(nn < (1ull << 32), LMTG_ERR_UNSUPPORTED, "more than 2^32 nodes");
        const int npe = elem_type;
        recal_free(c);
        amg_free(c);
        c->elem_type = elem_type;
        c->npe = npe;
        c->nnu = 3;
        c->npairs = npe * (npe + 1) / 2;
        c->nn = nn;
        c->ne = ne;
        c->n = 3 * nn;
        c->h_pos.assign(pos, pos + 3 * nn);
        c->h_conn.assign(conn, conn + (uint64_t)npe * ne);
        upload(c, c->pos, pos, 3 * nn);
        upload(c, c->conn, conn, (uint64_t)npe * ne);
        // formulation defaults: elastic_modulus 1, poisson_ratio 0.33
        // (formulations/formulation_elasticity_iso.py:5-6)
        const double one = 1.0;
        upload(c, c->E, &one, 1);
        c->E_per_elem = 0;
        c->nu = 0.33;
        c->allocated = c->have64 = c->have32 = c->have_vec = false;
        c->nc = 0;
        c->h_cdof.clear();
        c->penalty = 0;
        c->h_loads.assign(c->n, 0.0);
        LMTG_CUDA(cudaStreamSynchronize(c->stream));
        return LMTG_OK;
    });
}

int lmtg_material_set(lmtg_ctx *c, const double *E, uint64_t nE, double nu) {
    return guard(c, [&] {
        LMTG_CHECK(c->ne > 0, LMTG_ERR_STATE, "mesh_set first");
        LMTG_CHECK(E && (nE == 1 || nE == c->ne), LMTG_ERR_ARG, "E needs 1 or ne values");
        LMTG_CHECK(nu > -1.0 && nu < 0.5, LMTG_ERR_ARG, "poisson_ratio out of (-1, 0.5)");
        upload(c, c->E, E, nE);
        c->E_per_elem = nE > 1 ? 1 : 0;
        c->nu = nu;
        c->nu_per_elem = 0;  // lmtg_material_set_nu afterwards for per-element ratios
        c->have64 = c->have32 = false;
        LMTG_CUDA(cudaStreamSynchronize(c->stream));
        return LMTG_OK;
    });
}

int lmtg_material_set_nu(lmtg_ctx *c, const double *nu, uint64_t n_nu) {
    return guard(c, [&] {
        LMTG_CHECK(c->ne > 0, LMTG_ERR_STATE, "mesh_set first");
        LMTG_CHECK(nu && n_nu == c->ne, LMTG_ERR_ARG, "nu needs ne values");
        for (uint64_t e = 0; e < n_nu; ++e)
            LMTG_CHECK(nu[e] > -1.0 && nu[e] < 0.5, LMTG_ERR_ARG, "poisson_ratio out of (-1, 0.5)");
        upload(c, c->nuv, nu, n_nu);
        c->nu_per_elem = 1;
        c->have64 = c->have32 = false;
        LMTG_CUDA(cudaStreamSynchronize(c->stream));
        return LMTG_OK;
    });
}

int lmtg_set_volume_force(lmtg_ctx *c, double density, const double f_vol[3]) {
    return guard(c, [&] {
        LMTG_CHECK(c->nnu == 3 && c->ne > 0, LMTG_ERR_STATE, "elasticity mesh_set first");
        LMTG_CHECK(f_vol && std::isfinite(density), LMTG_ERR_ARG, "f_vol needed");
        c->density = density;
        for (int i = 0; i < 3; ++i) c->fvol[i] = f_vol[i];
        c->have_vec = false;
        return LMTG_OK;
    });
}

int lmtg_set_nodal_springs(lmtg_ctx *c, const double *coef, const double *target) {
    return guard(c, [&] {
        LMTG_CHECK(c->nnu == 3 && c->ne > 0, LMTG_ERR_STATE, "elasticity mesh_set first");
        if (!coef) {
            c->spring_coef.release();
            c->spring_target.release();
        } else {
            upload(c, c->spring_coef, coef, c->nn);
            if (target) upload(c, c->spring_target, target, c->n);
            else c->spring_target.release();
        }
        c->have64 = c->have32 = c->have_vec = false;
        LMTG_CUDA(cudaStreamSynchronize(c->stream));
        return LMTG_OK;
    });
}

int lmtg_set_levenberg_marquadt(lmtg_ctx *c, double lm) {
    return guard(c, [&] {
        LMTG_CHECK(std::isfinite(lm), LMTG_ERR_ARG, "levenberg_marquadt must be finite");
        c->levenberg_marquadt = lm;
        c->have64 = c->have32 = false;
        return LMTG_OK;
    });
}

int lmtg_batch_set(lmtg_ctx *c, uint32_t nsys, const uint64_t *node_off) {
    return guard(c, [&] {
        amg_free(c);
        LMTG_CHECK(c->ne > 0 && c->nnu == 3, LMTG_ERR_STATE, "elasticity mesh_set first");
        LMTG_CHECK(nsys > 0 && node_off, LMTG_ERR_ARG, "nsys > 0 and node_off needed");
        LMTG_CHECK(node_off[0] == 0 && node_off[nsys] == c->nn, LMTG_ERR_ARG, "node_off must span 0..nn");
        std::vector<uint32_t> sys(c->nn);
        for (uint32_t m = 0; m < nsys; ++m) {
            LMTG_CHECK(node_off[m + 1] > node_off[m], LMTG_ERR_ARG, "empty or decreasing node range");
            for (uint64_t i = node_off[m]; i < node_off[m + 1]; ++i) sys[i] = m;
        }
        for (uint64_t e = 0; e < c->ne; ++e) {
            const uint32_t m = sys[c->h_conn[e * c->npe]];
            for (int k = 1; k < c->npe; ++k)
                LMTG_CHECK(sys[c->h_conn[e * c->npe + k]] == m, LMTG_ERR_ARG, "an element couples two systems");
        }
        c->h_sys_node_off.assign(node_off, node_off + nsys + 1);
        upload_u32(c, c->sys_of_node, sys.data(), sys.size());
        c->nsys = nsys;
        c->h_sys_max_diag.assign(nsys, 0.0);
        batch_free(c);
        c->have64 = c->have32 = false;
        LMTG_CUDA(cudaStreamSynchronize(c->stream));
        return LMTG_OK;
    });
}

int lmtg_batch_set_rhs(lmtg_ctx *c, int nrhs, const double *B) {
    return guard(c, [&] {
        LMTG_CHECK(nrhs >= 1 && nrhs <= 4 && B, LMTG_ERR_ARG, "1..4 right-hand sides");
        batch_set_rhs(c, nrhs, B);
        return LMTG_OK;
    });
}

int lmtg_batch_solve(lmtg_ctx *c, int mode, double tol, int maxit, double timeout_s, lmtg_solve_stats *st,
                     int *pair_iters) {
    lmtg_solve_stats local{};
    if (!st) st = &local;
    memset(st, 0, sizeof(*st));
    int s = guard(c, [&] {
        LMTG_CHECK(maxit > 0 && tol > 0, LMTG_ERR_ARG, "maxit > 0, tol > 0");
        cudaEvent_t e0, e1;
        LMTG_CUDA(cudaEventCreate(&e0));
        LMTG_CUDA(cudaEventCreate(&e1));
        LMTG_CUDA(cudaEventRecord(e0, c->stream));
        const int status = batch_solve(c, mode, tol, maxit, timeout_s, st, pair_iters);
        LMTG_CUDA(cudaEventRecord(e1, c->stream));
        LMTG_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        st->device_ms = ms;
        if (status != LMTG_OK) c->err = lmtg_status_string(status);
        return status;
    });
    st->status = s;
    return s;
}

int lmtg_batch_get_result(lmtg_ctx *c, double *X) {
    return guard(c, [&] {
        LMTG_CHECK(X, LMTG_ERR_ARG, "null output");
        batch_get_result(c, X);
        return LMTG_OK;
    });
}

int lmtg_batch_info(lmtg_ctx *c, int *tile_rows, int *variant, uint64_t *ntiles, double *tuned_ms) {
    return guard(c, [&] {
        batch_info(c, tile_rows, variant, ntiles, tuned_ms);
        return LMTG_OK;
    });
}

int lmtg_set_inner_reduction(lmtg_ctx *c, double inner_reduction) {
    return guard(c, [&] {
        LMTG_CHECK(inner_reduction > 0 && inner_reduction < 1, LMTG_ERR_ARG, "inner_reduction in (0, 1)");
        c->inner_reduction = inner_reduction;
        return LMTG_OK;
    });
}

// Self-test of the bound: one thread waits on an mbarrier that nothing arrives on.  out[0] =
// LMTG_ERR_TIMEOUT if the wait gave up (LMTG_OK if it completed), out[1] = ns waited.
__global__ void k_selftest_bounded_wait(long long *out) {
    using namespace lmtg::bulk;
    __shared__ uint64_t bar;
    if (threadIdx.x != 0) return;
    mbar_init(&bar, 1);
    fence_barrier_init();
    const uint64_t t0 = globaltimer_ns();
    const bool ok = mbar_wait(&bar, 0);
    out[0] = ok ? LMTG_OK : LMTG_ERR_TIMEOUT;
    out[1] = (long long)(globaltimer_ns() - t0);
}

int lmtg_selftest_bounded_wait(lmtg_ctx *c, int *status, double *waited_s) {
    return guard(c, [&] {
        DBuf<long long> out;
        out.alloc(2);
        k_selftest_bounded_wait<<<1, 32, 0, c->stream>>>(out.p);
        c->launches += 1;
        LMTG_CUDA(cudaGetLastError());
        long long h[2] = {0, 0};
        LMTG_CUDA(cudaMemcpyAsync(h, out.p, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
        LMTG_CUDA(cudaStreamSynchronize(c->stream));
        if (status) *status = (int)h[0];
        if (waited_s) *waited_s = 1e-9 * (double)h[1];
        return LMTG_OK;
    });
}

int lmtg_set_spmv_kind(lmtg_ctx *c, int kind) {
    return guard(c, [&] {
        LMTG_CHECK(kind >= -1 && kind <= 2, LMTG_ERR_ARG, "spmv kind in -1..2");
        c->spmv_kind = kind;
        if (kind == -1) c->spmv_tuned = -1;  // tune again at the next FP32 solve
        return LMTG_OK;
    });
}

int lmtg_spmv_info(lmtg_ctx *c, int *kind_in_use, int *tuned, double tune_ms[3]) {
    return guard(c, [&] {
        if (kind_in_use) *kind_in_use = spmv_kind_in_use(c);
        if (tuned) *tuned = c->spmv_tuned;
        if (tune_ms)
            for (int k = 0; k < 3; ++k) tune_ms[k] = c->spmv_tune_ms[k];
        return LMTG_OK;
    });
}

int lmtg_profile_amg_kernels(lmtg_ctx *c, int iters, double ms[8]) {
    return guard(c, [&] {
        LMTG_CHECK(ms && iters > 0, LMTG_ERR_ARG, "bad arguments");
        LMTG_CHECK(c->have_vec && c->have32, LMTG_ERR_STATE, "assemble the system (FP32 matrix) first");
        profile_amg(c, iters, ms);
        return LMTG_OK;
    });
}

int lmtg_set_preconditioner(lmtg_ctx *c, int kind) {
    return guard(c, [&] {
        LMTG_CHECK(kind == LMTG_PREC_BLOCK_JACOBI || kind == LMTG_PREC_AMG, LMTG_ERR_ARG, "unknown preconditioner");
        c->precond = kind;
        return LMTG_OK;
    });
}

int lmtg_amg_info(lmtg_ctx *c, int *levels, uint64_t *ndof, uint64_t *nnz_blocks, double *omega,
                  double *lambda_max, double *structure_ms, double *numeric_ms, double *structure_phase_ms) {
    return guard(c, [&] {
        amg_info(c, levels, ndof, nnz_blocks, omega, lambda_max, structure_ms, numeric_ms, structure_phase_ms);
        return LMTG_OK;
    });
}

int lmtg_batch_set_options(lmtg_ctx *c, int tile_rows, int variant) {
    return guard(c, [&] {
        LMTG_CHECK(variant >= -1 && variant <= 2, LMTG_ERR_ARG, "variant: -1 (autotune), 0, 1 or 2");
        const bool small = tile_rows == 16 || tile_rows == 32 || tile_rows == 64 || tile_rows == 128;
        const bool large = tile_rows == 128 || tile_rows == 256 || tile_rows == 512 || tile_rows == 1024;
        LMTG_CHECK(tile_rows == 0 || (variant == 2 ? large : variant == -1 ? (small || large) : small),
                   LMTG_ERR_ARG, "tile_rows: 0 (autotune), 16, 32, 64 or 128 (variants 0, 1), 128..1024 (2)");
        c->batch_tile_rows = tile_rows;
        c->batch_variant = variant;
        batch_free(c);  // re-tune at the next solve
        return LMTG_OK;
    });
}

int lmtg_allocate_matrices(lmtg_ctx *c, uint64_t *nnz_lower) {
    return guard(c, [&] {
        LMTG_CHECK(c->ne > 0, LMTG_ERR_STATE, "mesh_set first");
        LMTG_CHECK(c->nnu == 3, LMTG_ERR_STATE, "elasticity call on a diffusion context");
        amg_free(c);
        build_pattern(c);
        c->spmv_tuned = -1;
        c->spmv_setup_kind = -2;
        c->Ke64.alloc(c->ne * (uint64_t)c->npairs * 9);
        c->K64.alloc(c->nnzb * 9);
        c->K32.alloc(c->nnzb * 9 + 4);  // 16 bytes of slack: bulk copies round their end up
        c->F.alloc(c->n);
        c->u.alloc(c->n);
        c->Dinv64.alloc(c->nn * 9);
        c->Dinv32.alloc(c->nn * 9);
        for (auto &w : c->w64) w.alloc(c->n);
        for (auto &w : c->w32) w.alloc(4 * c->nn);  // room for 16-byte padded node vectors
        LMTG_CUDA(cudaMemsetAsync(c->u.p, 0, c->u.bytes(), c->stream));
        LMTG_CUDA(cudaMemsetAsync(c->F.p, 0, c->F.bytes(), c->stream));
        LMTG_CUDA(cudaStreamSynchronize(c->stream));
        c->allocated = true;
        c->have64 = c->have32 = c->have_vec = false;
        if (nnz_lower) *nnz_lower = c->nnz_lower;
        return LMTG_OK;
    });
}

int lmtg_set_nodal_loads(lmtg_ctx *c, const double *F) {
    return guard(c, [&] {
        LMTG_CHECK(c->n > 0 && F, LMTG_ERR_ARG, "mesh_set first / null F");
        c->h_loads.assign(F, F + c->n);
        return LMTG_OK;
    });
}

int lmtg_add_skin_pressure(lmtg_ctx *c, uint64_t nfaces, const uint32_t *faces, double p) {
    return guard(c, [&] {
        LMTG_CHECK(c->n > 0 && c->nnu == 3 && (nfaces == 0 || faces), LMTG_ERR_ARG, "bad faces");
        const int fn = c->elem_type == LMTG_ELEM_HEXA8 ? 4 : 6;
        for (uint64_t f = 0; f < nfaces; ++f)
            for (int k = 0; k < fn; ++k) LMTG_CHECK(faces[fn * f + k] < c->nn, LMTG_ERR_ARG, "face node >= nn");
        const double t0[3] = {0, 0, 0};
        for (uint64_t f = 0; f < nfaces; ++f) {
            if (fn == 4) quad4_loads(c->h_pos.data(), faces + 4 * f, t0, c->h_loads.data(), &p);
            else tri6_loads(c->h_pos.data(), faces + 6 * f, t0, c->h_loads.data(), &p);
        }
        c->have_vec = false;
        return LMTG_OK;
    });
}

int lmtg_add_skin_traction(lmtg_ctx *c, uint64_t nfaces, const uint32_t *faces,
                           const double traction[3]) {
    return guard(c, [&] {
        LMTG_CHECK(c->n > 0 && traction && (nfaces == 0 || faces), LMTG_ERR_ARG, "bad faces");
        const int fn = c->elem_type == LMTG_ELEM_HEXA8 ? 4 : 6;
        for (uint64_t f = 0; f < nfaces; ++f)
            for (int a = 0; a < fn; ++a)
                LMTG_CHECK(faces[fn * f + a] < c->nn, LMTG_ERR_ARG, "face node id >= nn");
        for (uint64_t f = 0; f < nfaces; ++f) {
            if (fn == 4) quad4_loads(c->h_pos.data(), faces + 4 * f, traction, c->h_loads.data());
            else tri6_loads(c->h_pos.data(), faces + 6 * f, traction, c->h_loads.data());
        }
        return LMTG_OK;
    });
}

int lmtg_set_constraints(lmtg_ctx *c, uint64_t nc, const uint32_t *dof, const double *coef,
                         const double *res, double penalty) {
    return guard(c, [&] {
        LMTG_CHECK(c->n > 0, LMTG_ERR_STATE, "mesh_set first");
        LMTG_CHECK(nc == 0 || (dof && coef && res), LMTG_ERR_ARG, "null constraint arrays");
        for (uint64_t k = 0; k < nc; ++k) {
            LMTG_CHECK(dof[k] < c->n, LMTG_ERR_ARG, "constraint dof >= n");
            // penalty 0: exact constraint coef u = res (the reference's Lagrange rows)
            LMTG_CHECK(penalty != 0.0 || coef[k] != 0.0, LMTG_ERR_ARG, "exact constraint with coefficient 0");
        }
        if (penalty == 0.0 && nc > 1) {  // one exact constraint per DOF
            std::vector<uint32_t> d(dof, dof + nc);
            std::sort(d.begin(), d.end());
            LMTG_CHECK(std::adjacent_find(d.begin(), d.end()) == d.end(), LMTG_ERR_ARG,
                       "two exact constraints on one DOF");
        }
        upload(c, c->cdof, dof, nc);
        c->h_cdof.assign(dof, dof + nc);
        amg_free(c);  // constrained nodes stay out of the multigrid's coarse spaces
        upload(c, c->ccoef, coef, nc);
        upload(c, c->cres, res, nc);
        c->nc = nc;
        c->penalty = penalty;
        c->have64 = c->have32 = false;
        LMTG_CUDA(cudaStreamSynchronize(c->stream));
        return LMTG_OK;
    });
}

}  // extern "C"
