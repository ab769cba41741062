// fields.cu -- element fields after the solve: strain, stress and trace of strain per element.
//
// Replaces the generated apply_on_elements_after_solve of elasticity_iso
// (formulations/formulation_elasticity_iso.py:64-85), run by call_after_solve
// (include/formulation/formulation.h:1867-1875, 2026-2035).  As there, every var_inter is set to
// 0.5: the cube centre for Hexa8, and for Tetra10 the point (0.5, 0.5, 0.5), to which the
// quadratic displacement is extrapolated.  epsilon = grad_sym_col(dep) with tensor shear in the
// order 11 22 33 12 13 23 (include/codegen/__init__.py:23-42), sigma = lambda tr(eps) I + 2 mu eps
// (the inverse compliance of hooke_isotrope, formal_lf/material_help.py:116-134).
// One thread per element, FP64; output ne x 13 = epsilon[6], sigma[6], tr_epsilon.
#include "elem_traits.cuh"

namespace lmtg {

template <class EL>
__global__ void __launch_bounds__(128)
    k_elem_fields(const double *__restrict__ pos, const uint32_t *__restrict__ conn, const double *__restrict__ E,
                  int E_per_elem, double nu0, const double *__restrict__ nuv, const double *__restrict__ u,
                  uint64_t ne, double *__restrict__ out) {
    constexpr int NPE = EL::npe;
    double dN[NPE][3];
    EL::dN_at(0.5, 0.5, 0.5, dN);
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < ne;
         e += (uint64_t)gridDim.x * blockDim.x) {
        double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, U[NPE][3];
#pragma unroll
        for (int a = 0; a < NPE; ++a) {
            const uint64_t n = conn[NPE * e + a];
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                const double x = pos[3 * n + i];
                U[a][i] = u[3 * n + i];
#pragma unroll
                for (int j = 0; j < 3; ++j) J[i][j] = fma(x, dN[a][j], J[i][j]);
            }
        }
        // inverse Jacobian (adjugate / det)
        const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
        const double c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
        const double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
        const double id = 1.0 / (J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02);
        double Ji[3][3];
        Ji[0][0] = c00 * id;
        Ji[1][0] = c01 * id;
        Ji[2][0] = c02 * id;
        Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * id;
        Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id;
        Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * id;
        Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id;
        Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * id;
        Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id;
        // gu[k][i] = du_k / dx_i
        double gu[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
#pragma unroll
        for (int a = 0; a < NPE; ++a) {
            double g[3];
#pragma unroll
            for (int i = 0; i < 3; ++i) g[i] = Ji[0][i] * dN[a][0] + Ji[1][i] * dN[a][1] + Ji[2][i] * dN[a][2];
#pragma unroll
            for (int k = 0; k < 3; ++k)
#pragma unroll
                for (int i = 0; i < 3; ++i) gu[k][i] = fma(U[a][k], g[i], gu[k][i]);
        }
        const double eps[6] = {gu[0][0], gu[1][1], gu[2][2], 0.5 * (gu[0][1] + gu[1][0]),
                               0.5 * (gu[0][2] + gu[2][0]), 0.5 * (gu[1][2] + gu[2][1])};
        const double Ee = E[E_per_elem ? e : 0], nu = nuv ? nuv[e] : nu0;
        const double lam = Ee * nu / ((1.0 + nu) * (1.0 - 2.0 * nu)), two_mu = Ee / (1.0 + nu);
        const double tr = eps[0] + eps[1] + eps[2];
        double *o = out + 13 * e;
#pragma unroll
        for (int k = 0; k < 6; ++k) o[k] = eps[k];
#pragma unroll
        for (int k = 0; k < 3; ++k) o[6 + k] = lam * tr + two_mu * eps[k];
#pragma unroll
        for (int k = 3; k < 6; ++k) o[6 + k] = two_mu * eps[k];
        o[12] = tr;
    }
}

void launch_elem_fields(lmtg_ctx *c, const double *u, double *out) {
    const int T = 128;
    const int grid = grid_for(c, c->ne, T, 16);
    const double *nuv = c->nu_per_elem ? c->nuv.p : nullptr;
    if (c->elem_type == LMTG_ELEM_HEXA8)
        k_elem_fields<Hexa8><<<grid, T, 0, c->stream>>>(c->pos.p, c->conn.p, c->E.p, c->E_per_elem, c->nu, nuv, u,
                                                        c->ne, out);
    else
        k_elem_fields<Tetra10><<<grid, T, 0, c->stream>>>(c->pos.p, c->conn.p, c->E.p, c->E_per_elem, c->nu, nuv,
                                                          u, c->ne, out);
    LMTG_CUDA(cudaGetLastError());
    c->launches += 1;
}

}  // namespace lmtg

// ---- volume force and nodal springs of elasticity_iso -------------------------------------
// density * (dep_tt - f_vol) . te dV with dep_tt = 0 (static): F += density f_vol int N_a dV
// (formulations/formulation_elasticity_iso.py:49), assembled without atomics: node I's
// elements are the contributions (a, a) of its diagonal block's gather list.
namespace lmtg {

template <class EL>
__global__ void k_volume_weights(const double *__restrict__ pos, const uint32_t *__restrict__ conn, uint64_t ne,
                                 double *__restrict__ w) {
    constexpr int NPE = EL::npe;
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < ne;
         e += (uint64_t)gridDim.x * blockDim.x) {
        double xyz[NPE][3], acc[NPE];
#pragma unroll
        for (int a = 0; a < NPE; ++a) {
            acc[a] = 0.0;
            const uint64_t n = conn[NPE * e + a];
#pragma unroll
            for (int i = 0; i < 3; ++i) xyz[a][i] = pos[3 * n + i];
        }
        for (int g = 0; g < EL::ngp; ++g) {
            double x, y, z, N[NPE], dN[NPE][3], J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
            EL::gauss_point(g, x, y, z);
            EL::N_at(x, y, z, N);
            EL::dN_at(x, y, z, dN);
#pragma unroll
            for (int a = 0; a < NPE; ++a)
#pragma unroll
                for (int i = 0; i < 3; ++i)
#pragma unroll
                    for (int j = 0; j < 3; ++j) J[i][j] = fma(xyz[a][i], dN[a][j], J[i][j]);
            const double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
                               J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                               J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
            const double wd = EL::template weight<double>(g) * det;
#pragma unroll
            for (int a = 0; a < NPE; ++a) acc[a] = fma(wd, N[a], acc[a]);
        }
#pragma unroll
        for (int a = 0; a < NPE; ++a) w[NPE * e + a] = acc[a];
    }
}

template <int NPE, int NPAIRS>
__global__ void k_volume_force(const uint32_t *__restrict__ bdiag, const uint32_t *__restrict__ gptr,
                               const uint32_t *__restrict__ gsrc, const double *__restrict__ w, uint64_t nn,
                               double f0, double f1, double f2, double *__restrict__ F) {
    for (uint64_t I = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; I < nn;
         I += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t d = bdiag[I];
        double s = 0.0;
        for (uint32_t g = gptr[d]; g < gptr[d + 1]; ++g) {
            const uint32_t q = gsrc[g] >> 1, e = q / NPAIRS, pr = q - e * NPAIRS;
            int a = 0;
            for (int k = 0; k < NPE; ++k) a = pair_index(k, k, NPE) == (int)pr ? k : a;
            s += w[(uint64_t)NPE * e + a];
        }
        F[3 * I] += f0 * s;
        F[3 * I + 1] += f1 * s;
        F[3 * I + 2] += f2 * s;
    }
}

// dep_imp_coef_0 * dep . te dN (formulation_elasticity_iso.py:55-60): K(3I+d, 3I+d) += coef_I,
// F(3I+d) += coef_I target(3I+d)
__global__ void k_springs(const uint32_t *__restrict__ bptr, const uint32_t *__restrict__ bdiag,
                          const double *__restrict__ coef, const double *__restrict__ target, uint64_t nn,
                          double *K64, float *K32, double *F, bool mat, bool vec) {
    for (uint64_t I = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; I < nn;
         I += (uint64_t)gridDim.x * blockDim.x) {
        const double k = coef[I];
        if (k == 0.0) continue;
        const uint32_t rb = bptr[I], deg = bptr[I + 1] - rb, dd = bdiag[I] - rb;
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            if (mat) {
                const uint64_t idx = kidx(rb, deg, dd, 4 * r);
                if (K64) K64[idx] += k;
                if (K32) K32[idx] = K64 ? (float)K64[idx] : K32[idx] + (float)k;
            }
            if (vec && target) F[3 * I + r] += k * target[3 * I + r];
        }
    }
}

void apply_body_terms(lmtg_ctx *c, bool mat, bool vec) {
    const int T = 256;
    cudaStream_t s = c->stream;
    if (vec && c->density != 0.0 && (c->fvol[0] != 0.0 || c->fvol[1] != 0.0 || c->fvol[2] != 0.0)) {
        DBuf<double> w;
        w.alloc(c->ne * (uint64_t)c->npe);
        if (c->elem_type == LMTG_ELEM_HEXA8) {
            k_volume_weights<Hexa8><<<grid_for(c, c->ne, 128, 16), 128, 0, s>>>(c->pos.p, c->conn.p, c->ne, w.p);
            k_volume_force<8, Hexa8::npairs><<<grid_for(c, c->nn, T), T, 0, s>>>(
                c->bdiag.p, c->gptr.p, c->gsrc.p, w.p, c->nn, c->density * c->fvol[0], c->density * c->fvol[1],
                c->density * c->fvol[2], c->F.p);
        } else {
            k_volume_weights<Tetra10><<<grid_for(c, c->ne, 128, 16), 128, 0, s>>>(c->pos.p, c->conn.p, c->ne, w.p);
            k_volume_force<10, Tetra10::npairs><<<grid_for(c, c->nn, T), T, 0, s>>>(
                c->bdiag.p, c->gptr.p, c->gsrc.p, w.p, c->nn, c->density * c->fvol[0], c->density * c->fvol[1],
                c->density * c->fvol[2], c->F.p);
        }
        c->launches += 2;
    }
    if (c->spring_coef.p && (mat || vec)) {
        k_springs<<<grid_for(c, c->nn, T), T, 0, s>>>(c->bptr.p, c->bdiag.p, c->spring_coef.p,
                                                      c->spring_target.p, c->nn, c->have64 ? c->K64.p : nullptr,
                                                      c->have32 ? c->K32.p : nullptr, c->F.p, mat, vec);
        c->launches += 1;
    }
    LMTG_CUDA(cudaGetLastError());
}

}  // namespace lmtg
