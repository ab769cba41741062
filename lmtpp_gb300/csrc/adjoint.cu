// adjoint.cu -- adjoint gradients of compliance and displacement misfit w.r.t. per-element E.
//
// New capability next to the reference's forward sensitivities (solve_and_get_derivatives,
// include/formulation/formulation.h:1588-1652, and the der_var vectors dV/dp - dM/dp U of
// formal_lf/formulation.py:842-901, one extra solve per parameter).  With K = sum_e E_e Khat_e
// (+ penalty terms, held at a fixed max|diag| scale), K u = F and an objective J(u):
//   compliance  J = F.u                      adjoint lambda = u (no extra solve)
//   misfit      J = 1/2 sum_i w_i (u_i - t_i)^2   K lambda = w (u - t)   (one PCG solve)
//   linear      J = c.u                      K lambda = c           (one PCG solve)
//   dJ/dE_e = -lambda_e^T Khat_e u_e.
// The element matrix is not stored: k_grad_E recomputes the geometry per Gauss point
// and evaluates the bilinear form directly,
//   a^T Khat_e b = sum_gp w detJ [lhat tr(A) tr(B) + mhat (A:B + tr(A B))],  A = grad a, B = grad b,
// with lhat = nu / ((1+nu)(1-2nu)) and mhat = 1 / (2(1+nu)) (unit modulus), the same weak form
// and Gauss rules as the element kernel (formulations/formulation_elasticity_iso.py:45-60,
// elem_traits.cuh).
#include <cmath>
#include <cstring>
#include <exception>
#include <new>

#include "elem_traits.cuh"
#include "solver_kernels.cuh"

namespace lmtg {

template <class EL>
__global__ void __launch_bounds__(128)
    k_grad_E(const double *__restrict__ pos, const uint32_t *__restrict__ conn, double nu0,
             const double *__restrict__ nuv, uint64_t ne, const double *__restrict__ a,
             const double *__restrict__ b, double *__restrict__ g) {
    constexpr int NPE = EL::npe;
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < ne;
         e += (uint64_t)gridDim.x * blockDim.x) {
        const double nu = nuv ? nuv[e] : nu0;
        const double lh = nu / ((1.0 + nu) * (1.0 - 2.0 * nu)), mh = 1.0 / (2.0 * (1.0 + nu));
        uint32_t nd[NPE];
        double xyz[NPE][3];
#pragma unroll
        for (int k = 0; k < NPE; ++k) {
            nd[k] = conn[NPE * e + k];
#pragma unroll
            for (int d = 0; d < 3; ++d) xyz[k][d] = pos[3ull * nd[k] + d];
        }
        double acc = 0.0;
#pragma unroll 1
        for (int gp = 0; gp < EL::ngp; ++gp) {
            double dN[NPE][3];
            EL::dN(gp, dN);
            double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
#pragma unroll
            for (int k = 0; k < NPE; ++k)
#pragma unroll
                for (int i = 0; i < 3; ++i)
#pragma unroll
                    for (int j = 0; j < 3; ++j) J[i][j] = fma(xyz[k][i], dN[k][j], J[i][j]);
            const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
            const double c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
            const double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
            const double det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
            const double id = 1.0 / det;
            const double Ji[3][3] = {
                {c00 * id, (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * id,
                 (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id},
                {c01 * id, (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id,
                 (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * id},
                {c02 * id, (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * id,
                 (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id}};
            double A[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, B[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
#pragma unroll
            for (int k = 0; k < NPE; ++k) {
                double gr[3];
#pragma unroll
                for (int j = 0; j < 3; ++j)
                    gr[j] = Ji[0][j] * dN[k][0] + Ji[1][j] * dN[k][1] + Ji[2][j] * dN[k][2];
                const uint64_t o = 3ull * nd[k];
                const double av[3] = {__ldg(a + o), __ldg(a + o + 1), __ldg(a + o + 2)};
                const double bv[3] = {__ldg(b + o), __ldg(b + o + 1), __ldg(b + o + 2)};
#pragma unroll
                for (int i = 0; i < 3; ++i)
#pragma unroll
                    for (int j = 0; j < 3; ++j) {
                        A[i][j] = fma(av[i], gr[j], A[i][j]);
                        B[i][j] = fma(bv[i], gr[j], B[i][j]);
                    }
            }
            const double trA = A[0][0] + A[1][1] + A[2][2], trB = B[0][0] + B[1][1] + B[2][2];
            double ddot = 0.0;
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j) ddot += A[i][j] * (B[i][j] + B[j][i]);
            acc += EL::template weight<double>(gp) * det * (lh * trA * trB + mh * ddot);
        }
        g[e] = -acc;
    }
}

void launch_grad_E(lmtg_ctx *c, const double *a, const double *b, double *g) {
    const int T = 128;
    const int grid = grid_for(c, c->ne, T, 16);
    if (c->elem_type == LMTG_ELEM_HEXA8)
        k_grad_E<Hexa8><<<grid, T, 0, c->stream>>>(c->pos.p, c->conn.p, c->nu, c->nu_per_elem ? c->nuv.p : nullptr,
                                                   c->ne, a, b, g);
    else
        k_grad_E<Tetra10><<<grid, T, 0, c->stream>>>(c->pos.p, c->conn.p, c->nu, c->nu_per_elem ? c->nuv.p : nullptr,
                                                   c->ne, a, b, g);
    LMTG_CUDA(cudaGetLastError());
    c->launches += 1;
}

// misfit right-hand side w (u - t) and the objective 1/2 sum w (u - t)^2 (partials per thread,
// grid reduction in FP64)
__global__ void k_misfit(const double *__restrict__ u, const double *__restrict__ t,
                         const double *__restrict__ w, uint64_t n, double *rhs, double *partials,
                         unsigned *ticket, double *J) {
    double v[1] = {0.0};
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const double d = u[i] - (t ? t[i] : 0.0), wi = w ? w[i] : 1.0;
        rhs[i] = wi * d;
        v[0] += 0.5 * wi * d * d;
    }
    double out[1];
    if (grid_reduce<1, 0u>(v, partials, ticket, out) && threadIdx.x == 0) *J = out[0];
}

__global__ void k_dot_small(const double *__restrict__ a, const double *__restrict__ b, uint64_t n,
                            double *partials, unsigned *ticket, double *J) {
    double v[1] = {0.0};
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x)
        v[0] += a[i] * b[i];
    double out[1];
    if (grid_reduce<1, 0u>(v, partials, ticket, out) && threadIdx.x == 0) *J = out[0];
}

}  // namespace lmtg

using namespace lmtg;

namespace {

template <class F>
int guard3(lmtg_ctx *c, F &&f) {
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

}  // namespace

extern "C" {

int lmtg_set_penalty_scale(lmtg_ctx *c, double max_diag) {
    return guard3(c, [&] {
        LMTG_CHECK(max_diag >= 0.0 && std::isfinite(max_diag), LMTG_ERR_ARG, "scale >= 0");
        c->penalty_scale = max_diag;
        return LMTG_OK;
    });
}

int lmtg_get_penalty_scale(lmtg_ctx *c, double *max_diag) {
    if (!c || !max_diag) return LMTG_ERR_ARG;
    *max_diag = c->max_diag;
    return LMTG_OK;
}

int lmtg_adjoint_grad(lmtg_ctx *c, int objective, const double *target, const double *weights,
                      int mode, double tol, int maxit, double timeout_s, double *J, double *dJdE,
                      lmtg_solve_stats *st) {
    lmtg_solve_stats local{};
    if (!st) st = &local;
    memset(st, 0, sizeof(*st));
    return guard3(c, [&] {
        LMTG_CHECK(c->have64 && c->have_vec, LMTG_ERR_STATE, "assemble (FP64) and solve first");
        LMTG_CHECK(c->nnu == 3, LMTG_ERR_STATE, "elasticity gradient on another formulation's context");
        LMTG_CHECK(dJdE && J, LMTG_ERR_ARG, "null output");
        LMTG_CHECK(c->penalty != 0.0 || c->nc == 0, LMTG_ERR_UNSUPPORTED, "adjoint gradients with exact (penalty 0) constraints");
        LMTG_CHECK(objective == LMTG_OBJ_COMPLIANCE || objective == LMTG_OBJ_MISFIT ||
                       objective == LMTG_OBJ_LINEAR,
                   LMTG_ERR_ARG, "unknown objective");
        LMTG_CHECK(objective != LMTG_OBJ_LINEAR || target, LMTG_ERR_ARG, "linear objective needs c");
        c->grad.alloc(c->ne);
        PcgScalars *o = c->scal.p + 1;
        const int T = 256;
        const int grid = grid_for(c, c->n, T, 8);
        const double *lam = c->u.p;
        if (objective == LMTG_OBJ_COMPLIANCE) {
            k_dot_small<<<grid, T, 0, c->stream>>>(c->F.p, c->u.p, c->n, c->partials.p, &o->cnt_c,
                                                   &o->rr);
            c->launches += 1;
        } else {
            DBuf<double> dt, dw;
            if (target) {
                dt.alloc(c->n);
                LMTG_CUDA(cudaMemcpyAsync(dt.p, target, c->n * 8, cudaMemcpyHostToDevice, c->stream));
            }
            if (weights) {
                dw.alloc(c->n);
                LMTG_CUDA(cudaMemcpyAsync(dw.p, weights, c->n * 8, cudaMemcpyHostToDevice, c->stream));
            }
            c->adj_rhs.alloc(c->n);
            c->adj_lam.alloc(c->n);
            if (objective == LMTG_OBJ_MISFIT) {
                k_misfit<<<grid, T, 0, c->stream>>>(c->u.p, dt.p, dw.p, c->n, c->adj_rhs.p,
                                                    c->partials.p, &o->cnt_c, &o->rr);
            } else {  // linear: rhs = c, J = c . u
                LMTG_CUDA(cudaMemcpyAsync(c->adj_rhs.p, dt.p, c->n * 8, cudaMemcpyDeviceToDevice,
                                          c->stream));
                k_dot_small<<<grid, T, 0, c->stream>>>(dt.p, c->u.p, c->n, c->partials.p, &o->cnt_c,
                                                       &o->rr);
            }
            c->launches += 1;
            double jv = 0;
            LMTG_CUDA(cudaMemcpyAsync(&jv, &o->rr, 8, cudaMemcpyDeviceToHost, c->stream));
            LMTG_CUDA(cudaMemsetAsync(c->adj_lam.p, 0, c->n * 8, c->stream));
            LMTG_CUDA(cudaStreamSynchronize(c->stream));
            *J = jv;
            int s;
            if (mode == LMTG_SOLVE_MIXED_IR) {
                if (!c->have32) {
                    copy_k64_to_k32(c);
                    build_block_jacobi(c, false, true);
                }
                s = solve_mixed(c, tol, maxit, timeout_s, st, c->adj_rhs.p, c->adj_lam.p);
            } else {
                s = solve_pcg64(c, LMTG_CRIT_REL_RESIDUAL, tol, maxit, timeout_s, st, c->adj_rhs.p,
                                c->adj_lam.p);
            }
            st->status = s;
            if (s != LMTG_OK) {
                c->err = std::string("adjoint solve: ") + lmtg_status_string(s);
                return s;
            }
            lam = c->adj_lam.p;
        }
        launch_grad_E(c, lam, c->u.p, c->grad.p);
        if (objective == LMTG_OBJ_COMPLIANCE) {
            double jv = 0;
            LMTG_CUDA(cudaMemcpyAsync(&jv, &o->rr, 8, cudaMemcpyDeviceToHost, c->stream));
            LMTG_CUDA(cudaStreamSynchronize(c->stream));
            *J = jv;
        }
        LMTG_CUDA(cudaMemcpyAsync(dJdE, c->grad.p, c->ne * 8, cudaMemcpyDeviceToHost, c->stream));
        LMTG_CUDA(cudaStreamSynchronize(c->stream));
        return LMTG_OK;
    });
}

}  // extern "C"
