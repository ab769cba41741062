// recalage.cu -- the identification functional of formulation recalage on the GPU.
//
// formulations/formulation_recalage.py:25-47 defines, for three displacement fields U, V, W of a
// mesh, the modified constitutive-relation-error energy
//   E(U,V,W) = gamma int (sigma(V) - sigma(U)) : K^-1 (sigma(V) - sigma(U)) dV        (norme_sigma)
//            + (1 - gamma) int 1 / (rho omega^2) |rho omega (W - U)|^2 dV           (norme_gamma)
//            + sum over nodes Ud_valid r / (1 - r) E |U - Ud|^2                      (norme_G, dN)
// minimised over (U, V, W): with use_test_functions = False the reference's calculate_matrix
// (formal_lf/calculate_matrix.py:4-61) takes the tests to be the unknowns, so the assembled matrix
// is the energy's Hessian and the right-hand side minus its gradient at 0.  With K_IJ the 3x3
// elasticity block of a node pair (the bilinear form of norme_sigma, since K^-1 sigma = epsilon) and
// M_IJ its scalar mass int N_I N_J dV, the Hessian's node blocks are
//   UU: 2 gamma K + 2 (1 - gamma) rho M I3 (+ nodal),   UV = VU: -2 gamma K,
//   UW = WU: -2 (1 - gamma) rho M I3,   VV: 2 gamma K,   WW: 2 (1 - gamma) rho M I3,   VW: 0;
// the nodal term adds 2 Ud_valid r / (1 - r) E to U's diagonal and the same times Ud to the
// right-hand side.  lambd, the formulation's fourth unknown, appears in no term and is left out.
// The volume integrals use the element's Python rule of order 2, as integration_totale does
// (formal_lf/formulation.py:549-551): Hexa8 2x2x2 points at (1 -+ 1/sqrt 3) / 2, weights 1/8
// (formulations/element_Hexa.py:137-147); Tetra10 4 points at (5 - sqrt 5)/20 and
// (5 + 3 sqrt 5)/20, weights 1/24 (formulations/element_Tetra_10.py:109-115).
//
// Layout: the system is a 3x3-block matrix on virtual nodes (node I, field f) -> 3 I + f, so DOF
// 3 (3 I + f) + d = 9 I + 3 f + d, and the library's solvers, penalty constraints and exports run
// on it unchanged.  The virtual row of (I, U) holds 3 blocks per neighbour node J (columns (J, U),
// (J, V), (J, W)); those of (I, V) and (I, W) hold 2 ((J, U) and their own field).
#include <new>

#include "elem_traits.cuh"

namespace lmtg {

struct RecalState {
    double rho = 0, omega = 0, gamma = 0, r = 0, E = 0, lam = 0, mu = 0;
    uint64_t nn = 0, nnzb = 0;  // the mesh's node pattern
    DBuf<uint32_t> bptr, bcol, bdiag, gptr, gsrc;
    DBuf<double> Ud, Uv, Ke, Me, Kn, Mn;
};

void recal_free(lmtg_ctx *c) {
    delete c->recal;
    c->recal = nullptr;
}

namespace {

template <class T>
void take(DBuf<T> &dst, DBuf<T> &src) {
    dst.release();
    dst.p = src.p;
    dst.n = src.n;
    src.p = nullptr;
    src.n = 0;
}

// The Python Gauss rules of order 2 (element_Hexa.py gauss_points[2], element_Tetra_10.py
// gauss_points[2]), in the same point order as the C++ tables.
template <class EL>
struct PyRule;
template <>
struct PyRule<Hexa8> {
    static constexpr int ngp = 8;
    __device__ static void point(int g, double &x, double &y, double &z, double &w) {
        const double lo = 0.21132486540518711775, hi = 0.78867513459481288225;  // (1 -+ 1/sqrt 3)/2
        x = (g == 1 || g == 2 || g == 5 || g == 6) ? hi : lo;
        y = (g == 2 || g == 3 || g == 6 || g == 7) ? hi : lo;
        z = g >= 4 ? hi : lo;
        w = 0.125;
    }
};
template <>
struct PyRule<Tetra10> {
    static constexpr int ngp = 4;
    __device__ static void point(int g, double &x, double &y, double &z, double &w) {
        const double a = 0.13819660112501051518, b = 0.58541019662496845446;  // (5 - sqrt 5)/20, (5 + 3 sqrt 5)/20
        x = g == 1 ? b : a;
        y = g == 2 ? b : a;
        z = g == 3 ? b : a;
        w = 0.041666666666666666667;
    }
};

// One thread per element: the stiffness blocks (lambda A + mu A^T + mu tr(A) I with
// A = sum_gp w detJ grad N_a (x) grad N_b, the elasticity bilinear form) and the scalar masses of
// every upper node pair, in the layout of the element blocks Ke[e][pair][3][3] / Me[e][pair].
template <class EL>
__global__ void __launch_bounds__(128)
    k_recal_elem(const double *__restrict__ pos, const uint32_t *__restrict__ conn, uint64_t ne, double lam,
                 double mu, double *__restrict__ Ke, double *__restrict__ Me) {
    constexpr int NPE = EL::npe, NGP = PyRule<EL>::ngp, NP = EL::npairs;
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < ne;
         e += (uint64_t)gridDim.x * blockDim.x) {
        double xyz[NPE][3];
        for (int a = 0; a < NPE; ++a)
            for (int i = 0; i < 3; ++i) xyz[a][i] = pos[3ull * conn[e * NPE + a] + i];
        double G[NGP][NPE][3], N[NGP][NPE], wd[NGP];
        for (int g = 0; g < NGP; ++g) {
            double x, y, z, w;
            PyRule<EL>::point(g, x, y, z, w);
            double dN[NPE][3];
            EL::dN_at(x, y, z, dN);
            EL::N_at(x, y, z, N[g]);
            double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
            for (int a = 0; a < NPE; ++a)
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j) J[i][j] += xyz[a][i] * dN[a][j];
            const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
            const double c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
            const double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
            const double det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02, id = 1.0 / det;
            const double Ji[3][3] = {
                {c00 * id, (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * id, (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id},
                {c01 * id, (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id, (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * id},
                {c02 * id, (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * id, (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id}};
            wd[g] = w * det;
            for (int a = 0; a < NPE; ++a)
                for (int i = 0; i < 3; ++i)
                    G[g][a][i] = Ji[0][i] * dN[a][0] + Ji[1][i] * dN[a][1] + Ji[2][i] * dN[a][2];
        }
        for (int a = 0; a < NPE; ++a)
            for (int b = a; b < NPE; ++b) {
                double A[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, m = 0;
                for (int g = 0; g < NGP; ++g) {
                    for (int i = 0; i < 3; ++i)
                        for (int j = 0; j < 3; ++j) A[i][j] += wd[g] * G[g][a][i] * G[g][b][j];
                    m += wd[g] * N[g][a] * N[g][b];
                }
                const uint64_t p = e * NP + pair_index(a, b, NPE);
                const double tr = mu * (A[0][0] + A[1][1] + A[2][2]);
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j) Ke[p * 9 + 3 * i + j] = lam * A[i][j] + mu * A[j][i] + (i == j ? tr : 0.0);
                Me[p] = m;
            }
    }
}

// Node-pattern gather (the atomic-free assembly of assemble.cu): one warp per node row, one lane
// per block; Kn planar per row (kidx), Mn one scalar per block.
__global__ void __launch_bounds__(256)
    k_recal_gather(const uint32_t *__restrict__ bptr, uint64_t nn, const uint32_t *__restrict__ gptr,
                   const uint32_t *__restrict__ gsrc, const double *__restrict__ Ke, const double *__restrict__ Me,
                   double *__restrict__ Kn, double *__restrict__ Mn) {
    const int lane = threadIdx.x & 31;
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t I = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; I < nn; I += nw) {
        const uint32_t rb = bptr[I], deg = bptr[I + 1] - rb;
        for (uint32_t b = lane; b < deg; b += 32) {
            double s[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, m = 0;
            for (uint32_t g = gptr[rb + b]; g < gptr[rb + b + 1]; ++g) {
                const uint32_t src = gsrc[g];
                const double *e = Ke + (uint64_t)(src >> 1) * 9;
                const bool tr = (src & 1u) != 0;
                for (int v = 0; v < 9; ++v) s[v] += tr ? e[(v % 3) * 3 + v / 3] : e[v];
                m += Me[src >> 1];
            }
            for (int v = 0; v < 9; ++v) Kn[kidx(rb, deg, b, v)] = s[v];
            Mn[rb + b] = m;
        }
    }
}

// Virtual pattern: row degrees of (I, U), (I, V), (I, W).
__global__ void k_recal_vdeg(const uint32_t *__restrict__ bptr, uint64_t nn, uint32_t *__restrict__ vdeg) {
    for (uint64_t I = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; I < nn; I += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t deg = bptr[I + 1] - bptr[I];
        vdeg[3 * I] = 3 * deg;
        vdeg[3 * I + 1] = 2 * deg;
        vdeg[3 * I + 2] = 2 * deg;
    }
}

// Virtual columns and diagonal positions (columns stay sorted: J ascending, then field).
__global__ void k_recal_vcols(const uint32_t *__restrict__ bptr, const uint32_t *__restrict__ bcol,
                              const uint32_t *__restrict__ bdiag, uint64_t nn, const uint32_t *__restrict__ vptr,
                              uint32_t *__restrict__ vcol, uint32_t *__restrict__ vdiag) {
    for (uint64_t I = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; I < nn; I += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t rb = bptr[I], deg = bptr[I + 1] - rb, d = bdiag[I] - rb;
        const uint32_t u0 = vptr[3 * I], v0 = vptr[3 * I + 1], w0 = vptr[3 * I + 2];
        for (uint32_t b = 0; b < deg; ++b) {
            const uint32_t J = bcol[rb + b];
            vcol[u0 + 3 * b] = 3 * J;
            vcol[u0 + 3 * b + 1] = 3 * J + 1;
            vcol[u0 + 3 * b + 2] = 3 * J + 2;
            vcol[v0 + 2 * b] = 3 * J;
            vcol[v0 + 2 * b + 1] = 3 * J + 1;
            vcol[w0 + 2 * b] = 3 * J;
            vcol[w0 + 2 * b + 1] = 3 * J + 2;
        }
        vdiag[3 * I] = u0 + 3 * d;
        vdiag[3 * I + 1] = v0 + 2 * d + 1;
        vdiag[3 * I + 2] = w0 + 2 * d + 1;
    }
}

// The Hessian's blocks on the virtual pattern (planar per virtual row) and the right-hand side.
__global__ void __launch_bounds__(256)
    k_recal_expand(const uint32_t *__restrict__ bptr, const uint32_t *__restrict__ bcol, uint64_t nn,
                   const double *__restrict__ Kn, const double *__restrict__ Mn, const double *__restrict__ Ud,
                   const double *__restrict__ Uv, const uint32_t *__restrict__ vptr, double cK, double cM,
                   double cG, double *__restrict__ Kv, double *__restrict__ Fv) {
    const int lane = threadIdx.x & 31;
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t I = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; I < nn; I += nw) {
        const uint32_t rb = bptr[I], deg = bptr[I + 1] - rb;
        const uint32_t ru = vptr[3 * I], rv = vptr[3 * I + 1], rw = vptr[3 * I + 2];
        const double cn = cG * Uv[I];  // 2 Ud_valid r / (1 - r) E
        for (uint32_t b = lane; b < deg; b += 32) {
            double k[9];
            for (int v = 0; v < 9; ++v) k[v] = Kn[kidx(rb, deg, b, v)];
            const double m = Mn[rb + b];
            const bool diag = bcol[rb + b] == I;
            for (int v = 0; v < 9; ++v) {
                const bool vd = v == 0 || v == 4 || v == 8;  // on the block's diagonal
                const double mv = vd ? m : 0.0;
                Kv[kidx(ru, 3 * deg, 3 * b, v)] = cK * k[v] + cM * mv + (vd && diag ? cn : 0.0);
                Kv[kidx(ru, 3 * deg, 3 * b + 1, v)] = -cK * k[v];
                Kv[kidx(ru, 3 * deg, 3 * b + 2, v)] = -cM * mv;
                Kv[kidx(rv, 2 * deg, 2 * b, v)] = -cK * k[v];
                Kv[kidx(rv, 2 * deg, 2 * b + 1, v)] = cK * k[v];
                Kv[kidx(rw, 2 * deg, 2 * b, v)] = -cM * mv;
                Kv[kidx(rw, 2 * deg, 2 * b + 1, v)] = cM * mv;
            }
        }
        if (lane < 9) Fv[9 * I + lane] = lane < 3 ? cn * Ud[3 * I + lane] : 0.0;
    }
}

}  // namespace

void recal_setup(lmtg_ctx *c, double rho, double omega, double gamma, double r, const double *Ud,
                 const double *Ud_valid) {
    LMTG_CHECK(c->ne > 0 && c->nnu == 3, LMTG_ERR_STATE, "mesh_set (Hexa8 or Tetra10) first");
    LMTG_CHECK(!c->recal, LMTG_ERR_STATE, "recalage already set up on this context (mesh_set resets it)");
    LMTG_CHECK(c->nsys == 0, LMTG_ERR_UNSUPPORTED, "recalage on a batch of systems");
    LMTG_CHECK(c->E.p && !c->E_per_elem && !c->nu_per_elem, LMTG_ERR_ARG,
               "recalage: material_set with one elastic modulus and one Poisson ratio (global variables)");
    LMTG_CHECK(rho > 0 && omega != 0 && r < 1, LMTG_ERR_ARG, "recalage: rho > 0, omega != 0, r < 1");
    LMTG_CHECK(Ud && Ud_valid, LMTG_ERR_ARG, "recalage: null Ud or Ud_valid");
    cudaStream_t s = c->stream;
    amg_free(c);
    RecalState *R = new RecalState();
    c->recal = R;
    LMTG_CUDA(cudaMemcpy(&R->E, c->E.p, sizeof(double), cudaMemcpyDeviceToHost));
    R->rho = rho;
    R->omega = omega;
    R->gamma = gamma;
    R->r = r;
    R->lam = R->E * c->nu / ((1.0 + c->nu) * (1.0 - 2.0 * c->nu));
    R->mu = R->E / (2.0 * (1.0 + c->nu));
    // the mesh's node pattern and gather lists, kept by the recalage state
    build_pattern(c);
    R->nn = c->nn;
    R->nnzb = c->nnzb;
    take(R->bptr, c->bptr);
    take(R->bcol, c->bcol);
    take(R->bdiag, c->bdiag);
    take(R->gptr, c->gptr);
    take(R->gsrc, c->gsrc);
    const uint64_t nn = R->nn, nv = 3 * nn, nnzb_v = 7 * R->nnzb;
    LMTG_CHECK(nnzb_v < (1ull << 32), LMTG_ERR_UNSUPPORTED, "recalage: pattern too large for 32-bit indices");
    R->Ud.alloc(3 * nn);
    LMTG_CUDA(cudaMemcpyAsync(R->Ud.p, Ud, sizeof(double) * 3 * nn, cudaMemcpyHostToDevice, s));
    R->Uv.alloc(nn);
    LMTG_CUDA(cudaMemcpyAsync(R->Uv.p, Ud_valid, sizeof(double) * nn, cudaMemcpyHostToDevice, s));
    R->Ke.alloc(c->ne * (uint64_t)c->npairs * 9);
    R->Me.alloc(c->ne * (uint64_t)c->npairs);
    R->Kn.alloc(9 * R->nnzb);
    R->Mn.alloc(R->nnzb);
    // the virtual pattern becomes the context's
    const int T = 256;
    DBuf<uint32_t> vdeg;
    vdeg.alloc(nv + 1);
    c->bptr.alloc(nv + 1 + 4);  // 16 bytes of slack: bulk copies round their end up
    c->bcol.alloc(nnzb_v + 4);  // 16 bytes of slack: bulk copies round their end up
    c->bdiag.alloc(nv);
    k_recal_vdeg<<<grid_for(c, nn, T), T, 0, s>>>(R->bptr.p, nn, vdeg.p);
    LMTG_CHECK(exclusive_scan_u32(c, vdeg.p, c->bptr.p, nv) == nnzb_v, LMTG_ERR_CUDA, "recalage: virtual pattern size");
    k_recal_vcols<<<grid_for(c, nn, T), T, 0, s>>>(R->bptr.p, R->bcol.p, R->bdiag.p, nn, c->bptr.p, c->bcol.p,
                                                   c->bdiag.p);
    LMTG_CUDA(cudaGetLastError());
    c->launches += 3;
    c->nn = nv;
    c->n = 3 * nv;
    c->nnzb = nnzb_v;
    c->nnz_lower = 9ull * (nnzb_v - nv) / 2 + 6ull * nv;
    c->max_row_blocks *= 3;  // above 96 the FP32 solves take the warp-row SpMV, which strides over any width
    c->spmv_setup_kind = -2;
    c->spmv_tuned = -1;
    c->K64.alloc(nnzb_v * 9);
    c->K32.alloc(nnzb_v * 9 + 4);
    c->F.alloc(c->n);
    c->u.alloc(c->n);
    c->Dinv64.alloc(nv * 9);
    c->Dinv32.alloc(nv * 9);
    for (auto &w : c->w64) w.alloc(c->n);
    for (auto &w : c->w32) w.alloc(4 * nv);
    LMTG_CUDA(cudaMemsetAsync(c->u.p, 0, c->u.bytes(), s));
    LMTG_CUDA(cudaMemsetAsync(c->F.p, 0, c->F.bytes(), s));
    c->h_loads.assign(c->n, 0.0);
    LMTG_CUDA(cudaStreamSynchronize(s));
    c->allocated = true;
    c->have64 = c->have32 = c->have_vec = false;
    c->nnu = 9;  // elasticity-only calls (assembly, gradients, fields) refuse this context
    c->nc = 0;   // constraints are given on the 9-unknown system, after this call
    c->h_cdof.clear();
}

void recal_assemble(lmtg_ctx *c) {
    Phase ph("lmtg.recalage_assemble");
    RecalState *R = c->recal;
    LMTG_CHECK(R, LMTG_ERR_STATE, "recalage_setup first");
    cudaStream_t s = c->stream;
    const int T = 128;
    if (c->elem_type == LMTG_ELEM_HEXA8)
        k_recal_elem<Hexa8><<<grid_for(c, c->ne, T), T, 0, s>>>(c->pos.p, c->conn.p, c->ne, R->lam, R->mu, R->Ke.p,
                                                                  R->Me.p);
    else
        k_recal_elem<Tetra10><<<grid_for(c, c->ne, T), T, 0, s>>>(c->pos.p, c->conn.p, c->ne, R->lam, R->mu, R->Ke.p,
                                                                    R->Me.p);
    const int G = grid_for(c, R->nn * 32, 256, 8);
    k_recal_gather<<<G, 256, 0, s>>>(R->bptr.p, R->nn, R->gptr.p, R->gsrc.p, R->Ke.p, R->Me.p, R->Kn.p, R->Mn.p);
    const double cK = 2.0 * R->gamma, cM = 2.0 * (1.0 - R->gamma) * R->rho, cG = 2.0 * R->r / (1.0 - R->r) * R->E;
    k_recal_expand<<<G, 256, 0, s>>>(R->bptr.p, R->bcol.p, R->nn, R->Kn.p, R->Mn.p, R->Ud.p, R->Uv.p, c->bptr.p, cK, cM,
                                     cG, c->K64.p, c->F.p);
    LMTG_CUDA(cudaGetLastError());
    c->launches += 3;
    c->have64 = true;
    c->have32 = false;
    c->have_vec = true;
    apply_penalty(c, true, true);
    copy_k64_to_k32(c);
    c->have32 = true;
    build_block_jacobi(c, true, true);
    ++c->mat_version;
    LMTG_CUDA(cudaStreamSynchronize(s));
}

}  // namespace lmtg

namespace {

template <class F>
int guard_r(lmtg_ctx *c, F &&f) {
    if (!c) return LMTG_ERR_ARG;
    try {
        cudaError_t e = cudaSetDevice(c->device);
        if (e != cudaSuccess) throw lmtg::Error{LMTG_ERR_CUDA, cudaGetErrorString(e)};
        f();
        c->err.clear();
        return LMTG_OK;
    } catch (const lmtg::Error &e) {
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

}  // namespace

extern "C" {

int lmtg_recalage_setup(lmtg_ctx *c, double rho, double omega, double gamma, double r, const double *Ud,
                        const double *Ud_valid) {
    const bool fresh = c && !c->recal;
    const int st = guard_r(c, [&] { lmtg::recal_setup(c, rho, omega, gamma, r, Ud, Ud_valid); });
    if (st != LMTG_OK && fresh && c->recal) {
        // the node pattern was handed over part-way: the mesh has to be set again
        lmtg::recal_free(c);
        c->allocated = c->have64 = c->have32 = c->have_vec = false;
        c->nn = c->ne = c->n = 0;
    }
    return st;
}

int lmtg_recalage_assemble(lmtg_ctx *c) {
    return guard_r(c, [&] { lmtg::recal_assemble(c); });
}

}  // extern "C"
