// fit.cu -- identification driver: Gauss-Newton on the elastic moduli of element zones.
//
// Replaces FormulationFit::exec (include/formulation/FormulationFit.h:17-80) for the
// elastic_modulus parameter split into nz <= 4 zones (E_e = p[zone[e]]), with a diagonal weight
// w standing for exp_mat.  Every iteration follows the reference's steps:
//   assemble (element kernel, gather, penalty with max|diag| recomputed) and u = K^-1 F;
//   dU_i = K^-1 (-dK/dp_i u), the element part of assemble_vector_der_var, one solve per zone;
//   M_ij = (w dU_i).dU_j, V_i = (w dU_i).(u_exp - u), residual (w d).d;
//   a zero diagonal becomes 1; M_ii += max|diag M| levenberg_marq; dD = M^-1 V;
//   p += relaxation dD; stop when every |dD_i| < conv or at iteration max_iter (from 0);
//   then sensitivity_i = sum_c |sens_val_c (M^-1 w dU)_ic|.
// The reference inverts K with its sparse Cholesky; here each solve is the block-Jacobi PCG
// (FP64 or mixed) to the relative residual tol, warm-started from the previous u.
//
// dK/dp_i u is formed from the stored element blocks through the gather lists: for each block
// of each row, the contributions of zone-i elements are summed (scaled by 1/p_i, as
// Ke_e = p_i Khat_e) and multiplied by u -- one pass, no atomics, a fixed summation order.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <exception>
#include <new>
#include <vector>

#include "elem_traits.cuh"
#include "solver_kernels.cuh"

namespace lmtg {

constexpr int kFitMaxZones = 4;

struct ZoneInv {
    double v[kFitMaxZones];
};

__global__ void k_zone_E(const uint32_t *__restrict__ zone, ZoneInv p, uint64_t ne, double *__restrict__ E) {
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < ne;
         e += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t z = zone[e];
        double v = p.v[0];
#pragma unroll
        for (int k = 1; k < kFitMaxZones; ++k) v = z == (uint32_t)k ? p.v[k] : v;
        E[e] = v;
    }
}

// out[z n + 3 I + r] = -(dK/dp_z u)_(3I+r) for z < nz: warp per node row, lane per block.
template <int NPAIRS>
__global__ void __launch_bounds__(256)
    k_zone_dKu(const uint32_t *__restrict__ bptr, const uint32_t *__restrict__ bcol,
               const uint32_t *__restrict__ gptr, const uint32_t *__restrict__ gsrc,
               const double *__restrict__ Ke, const uint32_t *__restrict__ zone, ZoneInv invp,
               const double *__restrict__ u, uint64_t nn, int nz, double *__restrict__ out) {
    const int lane = threadIdx.x & 31;
    const uint64_t n = 3 * nn;
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t I = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; I < nn; I += nw) {
        const uint32_t rb = bptr[I], deg = bptr[I + 1] - rb;
        double a[16];
#pragma unroll
        for (int i = 0; i < 16; ++i) a[i] = 0.0;
        for (uint32_t b = lane; b < deg; b += 32) {
            const uint32_t blk = rb + b, J = bcol[blk];
            const double u0 = u[3ull * J], u1 = u[3ull * J + 1], u2 = u[3ull * J + 2];
            for (uint32_t g = gptr[blk]; g < gptr[blk + 1]; ++g) {
                const uint32_t src = gsrc[g], q = src >> 1;
                const uint32_t z = zone[q / NPAIRS];
                const double *m = Ke + 9ull * q;
                double t[3];
                if (src & 1u) {  // transposed block
#pragma unroll
                    for (int r = 0; r < 3; ++r) t[r] = m[r] * u0 + m[3 + r] * u1 + m[6 + r] * u2;
                } else {
#pragma unroll
                    for (int r = 0; r < 3; ++r) t[r] = m[3 * r] * u0 + m[3 * r + 1] * u1 + m[3 * r + 2] * u2;
                }
#pragma unroll
                for (int zz = 0; zz < kFitMaxZones; ++zz)
#pragma unroll
                    for (int r = 0; r < 3; ++r) a[3 * zz + r] += z == (uint32_t)zz ? t[r] : 0.0;
            }
        }
        const double v = reduce_scatter16(a, lane);
        const int idx = lane >> 1, z = idx / 3;
        if ((lane & 1) == 0 && z < nz) out[(uint64_t)z * n + 3 * I + (idx - 3 * z)] = -v * invp.v[z];
    }
}

// M_ij (i <= j, row-major upper), V_i, residual: 10 + 4 + 1 sums
constexpr int kFitDots = 15;
__global__ void k_fit_dots(const double *__restrict__ dU, const double *__restrict__ u, const double *__restrict__ uexp,
                           const double *__restrict__ w, uint64_t n, int nz, double *partials, unsigned *ticket,
                           double *out) {
    double v[kFitDots];
#pragma unroll
    for (int k = 0; k < kFitDots; ++k) v[k] = 0.0;
    for (uint64_t c = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; c < n; c += (uint64_t)gridDim.x * blockDim.x) {
        const double d = uexp[c] - u[c], wc = w[c];
        double du[kFitMaxZones];
#pragma unroll
        for (int i = 0; i < kFitMaxZones; ++i) du[i] = i < nz ? dU[(uint64_t)i * n + c] : 0.0;
        int k = 0;
#pragma unroll
        for (int i = 0; i < kFitMaxZones; ++i)
#pragma unroll
            for (int j = i; j < kFitMaxZones; ++j) v[k++] += wc * du[i] * du[j];
#pragma unroll
        for (int i = 0; i < kFitMaxZones; ++i) v[10 + i] += wc * du[i] * d;
        v[14] += wc * d * d;
    }
    double o[kFitDots];
    if (grid_reduce<kFitDots, 0u>(v, partials, ticket, o) && threadIdx.x == 0)
        for (int k = 0; k < kFitDots; ++k) out[k] = o[k];
}

struct Mat4 {
    double m[kFitMaxZones][kFitMaxZones];
};

// sensitivity_i = sum_c |sv_c sum_r Minv_ir w_c dU_r(c)|
__global__ void k_fit_sens(const double *__restrict__ dU, const double *__restrict__ w, const double *__restrict__ sv,
                           Mat4 Minv, uint64_t n, int nz, double *partials, unsigned *ticket, double *out) {
    double v[kFitMaxZones] = {0.0, 0.0, 0.0, 0.0};
    for (uint64_t c = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; c < n; c += (uint64_t)gridDim.x * blockDim.x) {
        const double ws = w[c] * (sv ? sv[c] : 1.0);
        double du[kFitMaxZones];
#pragma unroll
        for (int r = 0; r < kFitMaxZones; ++r) du[r] = r < nz ? dU[(uint64_t)r * n + c] : 0.0;
#pragma unroll
        for (int i = 0; i < kFitMaxZones; ++i) {
            double t = 0.0;
#pragma unroll
            for (int r = 0; r < kFitMaxZones; ++r) t += Minv.m[i][r] * du[r];
            v[i] += fabs(ws * t);
        }
    }
    double o[kFitMaxZones];
    if (grid_reduce<kFitMaxZones, 0u>(v, partials, ticket, o) && threadIdx.x == 0)
        for (int k = 0; k < kFitMaxZones; ++k) out[k] = o[k];
}

// inverse of a small SPD-ish matrix by Gauss-Jordan with partial pivoting; false if singular
static bool invert(int n, double (*a)[kFitMaxZones], double (*r)[kFitMaxZones]) {
    double m[kFitMaxZones][2 * kFitMaxZones] = {};
    for (int i = 0; i < n; ++i) {
        for (int j = 0; j < n; ++j) m[i][j] = a[i][j];
        m[i][n + i] = 1.0;
    }
    for (int col = 0; col < n; ++col) {
        int piv = col;
        for (int i = col + 1; i < n; ++i)
            if (std::fabs(m[i][col]) > std::fabs(m[piv][col])) piv = i;
        if (m[piv][col] == 0.0) return false;
        if (piv != col)
            for (int j = 0; j < 2 * n; ++j) std::swap(m[piv][j], m[col][j]);
        const double d = m[col][col];
        for (int j = 0; j < 2 * n; ++j) m[col][j] /= d;
        for (int i = 0; i < n; ++i)
            if (i != col) {
                const double f = m[i][col];
                for (int j = 0; j < 2 * n; ++j) m[i][j] -= f * m[col][j];
            }
    }
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) r[i][j] = m[i][n + j];
    return true;
}

int fit_zone_moduli(lmtg_ctx *c, uint32_t nz, const uint32_t *zone_h, double *p, const double *uexp_h,
                    const double *w_h, const double *sv_h, double relaxation, double lm, double conv,
                    int max_iter, int mode, double tol, int maxit, double *hist, double *res_hist,
                    double *sens, int *n_iter) {
    LMTG_CHECK(c->allocated && c->nnu == 3, LMTG_ERR_STATE, "elasticity allocate_matrices first");
    LMTG_CHECK(c->penalty != 0.0 || c->nc == 0, LMTG_ERR_UNSUPPORTED, "the fit with exact (penalty 0) constraints");
    LMTG_CHECK(nz >= 1 && nz <= (uint32_t)kFitMaxZones, LMTG_ERR_ARG, "1..4 zones");
    LMTG_CHECK(zone_h && p && uexp_h && max_iter >= 0, LMTG_ERR_ARG, "zones, p and u_exp needed");
    LMTG_CHECK(mode == LMTG_SOLVE_PCG_F64 || mode == LMTG_SOLVE_MIXED_IR, LMTG_ERR_ARG, "unknown mode");
    for (uint64_t e = 0; e < c->ne; ++e) LMTG_CHECK(zone_h[e] < nz, LMTG_ERR_ARG, "zone index out of range");
    for (uint32_t i = 0; i < nz; ++i) LMTG_CHECK(p[i] > 0.0, LMTG_ERR_ARG, "moduli must be positive");
    cudaStream_t s = c->stream;
    const uint64_t n = c->n, ne = c->ne;
    DBuf<uint32_t> zone;
    DBuf<double> uexp, w, sv, rhs, dU, dots, partials;
    DBuf<unsigned> ticket;
    upload_u32(c, zone, zone_h, ne);
    uexp.alloc(n);
    w.alloc(n);
    LMTG_CUDA(cudaMemcpyAsync(uexp.p, uexp_h, n * 8, cudaMemcpyHostToDevice, s));
    if (w_h) {
        LMTG_CUDA(cudaMemcpyAsync(w.p, w_h, n * 8, cudaMemcpyHostToDevice, s));
    } else {
        std::vector<double> ones(n, 1.0);
        LMTG_CUDA(cudaMemcpyAsync(w.p, ones.data(), n * 8, cudaMemcpyHostToDevice, s));
        LMTG_CUDA(cudaStreamSynchronize(s));
    }
    if (sv_h) {
        sv.alloc(n);
        LMTG_CUDA(cudaMemcpyAsync(sv.p, sv_h, n * 8, cudaMemcpyHostToDevice, s));
    }
    rhs.alloc((uint64_t)nz * n);
    dU.alloc((uint64_t)nz * n);
    dots.alloc(kFitDots);
    const int T = 256, G = grid_for(c, n, T, 4);
    partials.alloc((uint64_t)kFitDots * G);
    ticket.alloc(1);
    LMTG_CUDA(cudaMemsetAsync(ticket.p, 0, sizeof(unsigned), s));
    // E per element
    if (!c->E_per_elem || !c->E.p) {
        c->E.alloc(ne);
        c->E_per_elem = 1;
    }
    auto set_E = [&]() {
        ZoneInv pv{};
        for (uint32_t i = 0; i < nz; ++i) pv.v[i] = p[i];
        k_zone_E<<<grid_for(c, ne, T), T, 0, s>>>(zone.p, pv, ne, c->E.p);
        LMTG_CUDA(cudaGetLastError());
        c->launches += 1;
    };
    const int asm_flags = LMTG_ASM_MAT64 | LMTG_ASM_VEC | (mode == LMTG_SOLVE_MIXED_IR ? LMTG_ASM_MAT32 : 0);
    auto solve = [&](const double *b, double *x) {
        lmtg_solve_stats st{};
        const int r = mode == LMTG_SOLVE_MIXED_IR ? solve_mixed(c, tol, maxit, 0.0, &st, b, x)
                                                  : solve_pcg64(c, LMTG_CRIT_REL_RESIDUAL, tol, maxit, 0.0, &st, b, x);
        LMTG_CHECK(r == LMTG_OK, r, "fit: a solve failed");
    };
    int status = LMTG_OK;
    for (int it = 0;; ++it) {
        set_E();
        do_assemble(c, asm_flags);
        solve(nullptr, nullptr);  // u = K^-1 F, warm start from the previous u
        ZoneInv invp{};
        for (uint32_t i = 0; i < nz; ++i) invp.v[i] = 1.0 / p[i];
        if (c->elem_type == LMTG_ELEM_HEXA8)
            k_zone_dKu<Hexa8::npairs><<<grid_for(c, c->nn * 32, T, 8), T, 0, s>>>(
                c->bptr.p, c->bcol.p, c->gptr.p, c->gsrc.p, c->Ke64.p, zone.p, invp, c->u.p, c->nn, (int)nz, rhs.p);
        else
            k_zone_dKu<Tetra10::npairs><<<grid_for(c, c->nn * 32, T, 8), T, 0, s>>>(
                c->bptr.p, c->bcol.p, c->gptr.p, c->gsrc.p, c->Ke64.p, zone.p, invp, c->u.p, c->nn, (int)nz, rhs.p);
        LMTG_CUDA(cudaGetLastError());
        c->launches += 1;
        LMTG_CUDA(cudaMemsetAsync(dU.p, 0, (uint64_t)nz * n * 8, s));
        for (uint32_t i = 0; i < nz; ++i) solve(rhs.p + (uint64_t)i * n, dU.p + (uint64_t)i * n);
        k_fit_dots<<<G, T, 0, s>>>(dU.p, c->u.p, uexp.p, w.p, n, (int)nz, partials.p, ticket.p, dots.p);
        LMTG_CUDA(cudaGetLastError());
        c->launches += 1;
        double d[kFitDots];
        LMTG_CUDA(cudaMemcpyAsync(d, dots.p, sizeof(d), cudaMemcpyDeviceToHost, s));
        LMTG_CUDA(cudaStreamSynchronize(s));
        double M[kFitMaxZones][kFitMaxZones] = {}, Minv[kFitMaxZones][kFitMaxZones] = {}, V[kFitMaxZones] = {};
        int k = 0;
        for (int i = 0; i < kFitMaxZones; ++i)
            for (int j = i; j < kFitMaxZones; ++j, ++k) M[i][j] = M[j][i] = d[k];
        for (uint32_t i = 0; i < nz; ++i) V[i] = d[10 + i];
        if (res_hist) res_hist[it] = d[14];
        double dmax = 0;
        for (uint32_t i = 0; i < nz; ++i) dmax = std::max(dmax, std::fabs(M[i][i]));
        if (dmax == 0)
            for (uint32_t i = 0; i < nz; ++i) M[i][i] = 1.0;
        if (lm != 0) {
            double mx = 0;
            for (uint32_t i = 0; i < nz; ++i) mx = std::max(mx, std::fabs(M[i][i]));
            for (uint32_t i = 0; i < nz; ++i) M[i][i] += mx * lm;
        }
        LMTG_CHECK(invert((int)nz, M, Minv), LMTG_ERR_NAN, "fit: singular Gauss-Newton matrix");
        double dD[kFitMaxZones] = {}, amax = 0;
        for (uint32_t i = 0; i < nz; ++i) {
            for (uint32_t j = 0; j < nz; ++j) dD[i] += Minv[i][j] * V[j];
            amax = std::max(amax, std::fabs(dD[i]));
        }
        if (hist) hist[it] = amax;
        for (uint32_t i = 0; i < nz; ++i) p[i] += relaxation * dD[i];
        bool all_small = true;
        for (uint32_t i = 0; i < nz; ++i) all_small = all_small && std::fabs(dD[i]) < conv;
        if (!std::isfinite(amax)) {
            status = LMTG_ERR_NAN;
            *n_iter = it + 1;
            break;
        }
        if (all_small || it == max_iter) {
            *n_iter = it + 1;
            if (sens) {
                Mat4 mi{};
                for (uint32_t i = 0; i < nz; ++i)
                    for (uint32_t j = 0; j < nz; ++j) mi.m[i][j] = Minv[i][j];
                k_fit_sens<<<G, T, 0, s>>>(dU.p, w.p, sv_h ? sv.p : nullptr, mi, n, (int)nz, partials.p, ticket.p,
                                           dots.p);
                LMTG_CUDA(cudaGetLastError());
                c->launches += 1;
                double o[kFitMaxZones];
                LMTG_CUDA(cudaMemcpyAsync(o, dots.p, sizeof(o), cudaMemcpyDeviceToHost, s));
                LMTG_CUDA(cudaStreamSynchronize(s));
                for (uint32_t i = 0; i < nz; ++i) sens[i] = o[i];
            }
            break;
        }
    }
    // the context's moduli follow the updated p; its matrices are those of the last solve
    set_E();
    c->have64 = c->have32 = false;
    LMTG_CUDA(cudaStreamSynchronize(s));
    return status;
}

}  // namespace lmtg

using namespace lmtg;

namespace {

template <class F>
int guard_f(lmtg_ctx *c, F &&f) {
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

int lmtg_fit_zone_moduli(lmtg_ctx *c, uint32_t nz, const uint32_t *zone_of_elem, double *p, const double *u_exp,
                         const double *w, const double *sens_val, double relaxation, double levenberg_marq,
                         double conv, int max_iter, int mode, double tol, int maxit, double *history,
                         double *residual_history, double *sensitivity, int *n_iter) {
    return guard_f(c, [&] {
        int it = 0;
        const int s = fit_zone_moduli(c, nz, zone_of_elem, p, u_exp, w, sens_val, relaxation, levenberg_marq, conv,
                                      max_iter, mode, tol, maxit, history, residual_history, sensitivity, &it);
        if (n_iter) *n_iter = it;
        return s;
    });
}

}  // extern "C"
