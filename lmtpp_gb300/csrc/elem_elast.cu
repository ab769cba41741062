// elem_elast.cu -- isotropic-elasticity element matrices (Hexa8, Tetra10; FP64 and FP32).
//
// Replaces the generated add_local_elem_matrix of formulation elasticity_iso, called once per
// Gauss point by add_elem_matrix (include/formulation/formulation.h:2918-2932):
//   weak form  sigma(u) : eps(v), sigma = H eps, H = inverse of the isotropic compliance
//              (formulations/formulation_elasticity_iso.py:45-60, formal_lf/material_help.py:116-134)
//   rules      the reference's order-2 tables (elem_traits.cuh)
// For an isotropic H the 3x3 block of node pair (a,b) is
//   K_ab = lambda A_ab + mu A_ab^T + mu tr(A_ab) I,   A_ab = sum_gp w detJ grad N_a (x) grad N_b,
// which is the same bilinear form as B^T H B with 9 FMAs per pair and Gauss point.
//
// Mapping: one warp per batch of 8 elements.  Phase 1 (geometry): lane = (element, Gauss
// point); the Jacobian, its inverse and the shape-function gradients go to shared memory
// (G and w*detJ*G).  Phase 2: lane = (element, node pair), accumulating A_ab over the Gauss
// points from shared memory and writing the 3x3 block.  Output layout Ke[e][pair][3][3]
// (pairs a<=b): consecutive lanes write consecutive 72/36-byte blocks.
#include "elem_traits.cuh"
#include "ffloat.cuh"

namespace lmtg {

constexpr int kElBatch = 8, kElWarps = 4;

__constant__ unsigned char c_pair_a[2][64];
__constant__ unsigned char c_pair_b[2][64];

template <class EL, class T>
struct ElSmem {
    T xyz[kElBatch][3 * EL::npe];
    T G[kElBatch][EL::ngp][EL::npe][3];   // [element][gauss point][node][dim]
    T GW[kElBatch][EL::ngp][EL::npe][3];  // w * detJ * G
    T lam[kElBatch], mu[kElBatch];
};

template <class EL, class T, int kTab>
__global__ void __launch_bounds__(kElWarps * 32)
    k_elast(const double *__restrict__ pos, const uint32_t *__restrict__ conn,
            const double *__restrict__ E, int E_per_elem, double nu0, const double *__restrict__ nuv,
            uint64_t ne, T *__restrict__ Ke) {
    constexpr int NPE = EL::npe, NGP = EL::ngp, NP = EL::npairs;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    ElSmem<EL, T> &S = reinterpret_cast<ElSmem<EL, T> *>(smem_raw)[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    const uint64_t nbatch = (ne + kElBatch - 1) / kElBatch;
    const uint64_t warp0 = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;

    for (uint64_t batch = warp0; batch < nbatch; batch += nwarps) {
        const uint64_t e0 = batch * kElBatch;
        // cooperative load of the batch's node coordinates
        for (int t = lane; t < kElBatch * 3 * NPE; t += 32) {
            const int le = t / (3 * NPE), r = t % (3 * NPE);
            const uint64_t e = e0 + le;
            T v = (T)0;
            if (e < ne) v = (T)pos[3ull * conn[e * NPE + r / 3] + r % 3];
            S.xyz[le][r] = v;
        }
        if (lane < kElBatch) {
            const uint64_t e = e0 + lane;
            const double Ee = e < ne ? E[E_per_elem ? e : 0] : 0.0;
            const double nu = (nuv && e < ne) ? nuv[e] : nu0;
            S.lam[lane] = (T)(Ee * nu / ((1.0 + nu) * (1.0 - 2.0 * nu)));
            S.mu[lane] = (T)(Ee / (2.0 * (1.0 + nu)));
        }
        __syncwarp();
        // phase 1: geometry per (element, Gauss point)
        for (int t = lane; t < kElBatch * NGP; t += 32) {
            const int le = t / NGP, g = t % NGP;
            T dN[NPE][3];
            EL::dN(g, dN);
            T J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
#pragma unroll
            for (int a = 0; a < NPE; ++a)
#pragma unroll
                for (int i = 0; i < 3; ++i)
#pragma unroll
                    for (int j = 0; j < 3; ++j) J[i][j] += S.xyz[le][3 * a + i] * dN[a][j];
            const T c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
            const T c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
            const T c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
            const T det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
            const T id = (T)1 / det;
            // Ji[j][i]: gradient g_i = sum_j Ji[j][i] dN_j
            const T Ji[3][3] = {
                {c00 * id, (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * id,
                 (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id},
                {c01 * id, (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id,
                 (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * id},
                {c02 * id, (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * id,
                 (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id}};
            const T wdet = EL::template weight<T>(g) * det;
#pragma unroll
            for (int a = 0; a < NPE; ++a)
#pragma unroll
                for (int i = 0; i < 3; ++i) {
                    const T gi = Ji[0][i] * dN[a][0] + Ji[1][i] * dN[a][1] + Ji[2][i] * dN[a][2];
                    S.G[le][g][a][i] = gi;
                    S.GW[le][g][a][i] = wdet * gi;
                }
        }
        __syncwarp();
        // phase 2: node-pair blocks
        for (int t = lane; t < kElBatch * NP; t += 32) {
            const int le = t / NP, p = t - le * NP;
            const uint64_t e = e0 + le;
            if (e >= ne) break;  // tasks are ordered by element: the rest are past the end
            const int a = c_pair_a[kTab][p], b = c_pair_b[kTab][p];
            T A[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
#pragma unroll
            for (int g = 0; g < NGP; ++g) {
                const T wa0 = S.GW[le][g][a][0], wa1 = S.GW[le][g][a][1], wa2 = S.GW[le][g][a][2];
                const T gb0 = S.G[le][g][b][0], gb1 = S.G[le][g][b][1], gb2 = S.G[le][g][b][2];
                A[0][0] += wa0 * gb0; A[0][1] += wa0 * gb1; A[0][2] += wa0 * gb2;
                A[1][0] += wa1 * gb0; A[1][1] += wa1 * gb1; A[1][2] += wa1 * gb2;
                A[2][0] += wa2 * gb0; A[2][1] += wa2 * gb1; A[2][2] += wa2 * gb2;
            }
            const T lam = S.lam[le], mu = S.mu[le];
            const T tr = mu * (A[0][0] + A[1][1] + A[2][2]);
            T *o = Ke + (e * NP + p) * 9;
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j)
                    o[3 * i + j] = lam * A[i][j] + mu * A[j][i] + (i == j ? tr : (T)0);
        }
        __syncwarp();
    }
}

// ---- FP64 element matrices in float-float arithmetic ----
// The same mapping and algebra as k_elast, every FP64 operation replaced by its float-float
// counterpart (ffloat.cuh): GB300's FP64 pipe made k_elast<double> its bound (92% busy).  The
// Jacobian is formed from the node coordinates relative to the element's first node, taken in
// FP64 (the shape-function gradients sum to zero, so this is the same Jacobian), so that no
// coordinate offset cancels in the 48-bit arithmetic; the reference-cell gradients and weights
// come from FP64 tables split on the host.  Entries reach about 1e-14 of the largest, and are
// written as FP64.

// reference-cell gradients at the Gauss points and the weights, as float-float pairs
__constant__ ff::f2 c_dNff[2][8][10][3];
__constant__ ff::f2 c_wff[2];

template <class EL>
struct ElSmemFF {
    ff::f2 d[kElBatch][3 * EL::npe];              // node coordinates minus the first node's
    ff::f2 G[kElBatch][EL::ngp][EL::npe][3];      // [element][gauss point][node][dim]
    ff::f2 GW[kElBatch][EL::ngp][EL::npe][3];     // w * detJ * G
    ff::f2 lam[kElBatch], mu[kElBatch];
};

template <class EL, int kTab>
__global__ void __launch_bounds__(kElWarps * 32)
    k_elast_ff(const double *__restrict__ pos, const uint32_t *__restrict__ conn, const double *__restrict__ E,
               int E_per_elem, ff::f2 flam, ff::f2 fmu, double nu0, const double *__restrict__ nuv, uint64_t ne,
               double *__restrict__ Ke) {
    constexpr int NPE = EL::npe, NGP = EL::ngp, NP = EL::npairs;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    ElSmemFF<EL> &S = reinterpret_cast<ElSmemFF<EL> *>(smem_raw)[threadIdx.x >> 5];
    // the gradient table in shared memory: lanes read it at different Gauss points
    __shared__ ff::f2 dN[NGP][NPE][3];
    for (int t = threadIdx.x; t < NGP * NPE * 3; t += blockDim.x) {
        const int g = t / (NPE * 3), a = (t / 3) % NPE, j = t % 3;
        dN[g][a][j] = c_dNff[kTab][g][a][j];
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const uint64_t nbatch = (ne + kElBatch - 1) / kElBatch;
    const uint64_t warp0 = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;

    for (uint64_t batch = warp0; batch < nbatch; batch += nwarps) {
        const uint64_t e0 = batch * kElBatch;
        // node coordinates relative to the element's first node
        for (int t = lane; t < kElBatch * 3 * NPE; t += 32) {
            const int le = t / (3 * NPE), r = t % (3 * NPE);
            const uint64_t e = e0 + le;
            ff::f2 v{0.f, 0.f};
            // the FP64 difference is exact for nodes within a factor 2 of the first (Sterbenz)
            if (e < ne) v = ff::split(pos[3ull * conn[e * NPE + r / 3] + r % 3] - pos[3ull * conn[e * NPE] + r % 3]);
            S.d[le][r] = v;
        }
        if (lane < kElBatch) {
            const uint64_t e = e0 + lane;
            const ff::f2 Ee = ff::split(e < ne ? E[E_per_elem ? e : 0] : 0.0);
            if (nuv && e < ne) {  // per-element Poisson ratio: the factors in FP64
                const double nu = nuv[e];
                S.lam[lane] = ff::mul(Ee, ff::split(nu / ((1.0 + nu) * (1.0 - 2.0 * nu))));
                S.mu[lane] = ff::mul(Ee, ff::split(1.0 / (2.0 * (1.0 + nu))));
            } else {
                S.lam[lane] = ff::mul(Ee, flam);
                S.mu[lane] = ff::mul(Ee, fmu);
            }
        }
        __syncwarp();
        // phase 1: geometry per (element, Gauss point)
        for (int t = lane; t < kElBatch * NGP; t += 32) {
            const int le = t / NGP, g = t % NGP;
            ff::f2 J[3][3];
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j) {
                    ff::Dot acc;
#pragma unroll
                    for (int a = 1; a < NPE; ++a) acc.add(S.d[le][3 * a + i], dN[g][a][j]);
                    J[i][j] = acc.get();
                }
            auto cof = [&](int r0, int c0, int r1, int c1) {  // J[r0][c0] J[r1][c1] - J[r0][c1] J[r1][c0]
                ff::Dot acc;
                acc.add(J[r0][c0], J[r1][c1]);
                acc.add(ff::neg(J[r0][c1]), J[r1][c0]);
                return acc.get();
            };
            const ff::f2 c00 = cof(1, 1, 2, 2), c01 = cof(1, 2, 2, 0), c02 = cof(1, 0, 2, 1);
            ff::Dot dacc;
            dacc.add(J[0][0], c00);
            dacc.add(J[0][1], c01);
            dacc.add(J[0][2], c02);
            const ff::f2 det = dacc.get();
            const ff::f2 id = ff::recip(det);
            // Ji[j][i]: gradient g_i = sum_j Ji[j][i] dN_j (the inverse's transpose, as in k_elast)
            const ff::f2 Ji[3][3] = {
                {ff::mul(c00, id), ff::mul(cof(0, 2, 2, 1), id), ff::mul(cof(0, 1, 1, 2), id)},
                {ff::mul(c01, id), ff::mul(cof(0, 0, 2, 2), id), ff::mul(cof(0, 2, 1, 0), id)},
                {ff::mul(c02, id), ff::mul(cof(0, 1, 2, 0), id), ff::mul(cof(0, 0, 1, 1), id)}};
            const ff::f2 wdet = ff::mul(c_wff[kTab], det);
#pragma unroll
            for (int a = 0; a < NPE; ++a)
#pragma unroll
                for (int i = 0; i < 3; ++i) {
                    ff::Dot acc;
                    acc.add(Ji[0][i], dN[g][a][0]);
                    acc.add(Ji[1][i], dN[g][a][1]);
                    acc.add(Ji[2][i], dN[g][a][2]);
                    const ff::f2 gi = acc.get();
                    S.G[le][g][a][i] = gi;
                    S.GW[le][g][a][i] = ff::mul(wdet, gi);
                }
        }
        __syncwarp();
        // phase 2: node-pair blocks
        for (int t = lane; t < kElBatch * NP; t += 32) {
            const int le = t / NP, p = t - le * NP;
            const uint64_t e = e0 + le;
            if (e >= ne) break;
            const int a = c_pair_a[kTab][p], b = c_pair_b[kTab][p];
            ff::Dot A[3][3];
#pragma unroll
            for (int g = 0; g < NGP; ++g) {
#pragma unroll
                for (int i = 0; i < 3; ++i) {
                    const ff::f2 wa = S.GW[le][g][a][i];
#pragma unroll
                    for (int j = 0; j < 3; ++j) A[i][j].add(wa, S.G[le][g][b][j]);
                }
            }
            ff::f2 Af[3][3];
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j) Af[i][j] = A[i][j].get();
            const ff::f2 lam = S.lam[le], mu = S.mu[le];
            const ff::f2 tr = ff::add(ff::add(Af[0][0], Af[1][1]), Af[2][2]);
            double *o = Ke + (e * NP + p) * 9;
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j) {
                    ff::Dot acc;
                    acc.add(lam, Af[i][j]);
                    acc.add(mu, Af[j][i]);
                    if (i == j) acc.add(mu, tr);
                    o[3 * i + j] = ff::to_double(acc.get());
                }
        }
        __syncwarp();
    }
}

// FP64 table of the reference-cell gradients at the Gauss points, split into float-float pairs
// on the host (hi = the float nearest to the value, lo = the float nearest to the rest)
template <class EL>
static void ff_tables(ff::f2 (&dn)[8][10][3], ff::f2 &w) {
    auto sp = [](double v) {
        const float hi = (float)v;
        return ff::f2{hi, (float)(v - (double)hi)};
    };
    for (int g = 0; g < EL::ngp; ++g) {
        double x, y, z, d[EL::npe][3];
        EL::template gauss_point<double>(g, x, y, z);
        EL::template dN_at<double>(x, y, z, d);
        for (int a = 0; a < EL::npe; ++a)
            for (int j = 0; j < 3; ++j) dn[g][a][j] = sp(d[a][j]);
    }
    w = sp(EL::template weight<double>(0));
}

static bool g_pairs_ready[64] = {false};

template <class EL, int kTab>
static void launch_t(lmtg_ctx *c, bool fp64) {
    const int threads = kElWarps * 32;
    const uint64_t nbatch = (c->ne + kElBatch - 1) / kElBatch;
    if (fp64) {
        const size_t sm = sizeof(ElSmemFF<EL>) * kElWarps;
        LMTG_CUDA(cudaFuncSetAttribute(k_elast_ff<EL, kTab>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        const double nu = c->nu;
        auto sp = [](double v) {
            const float hi = (float)v;
            return ff::f2{hi, (float)(v - (double)hi)};
        };
        k_elast_ff<EL, kTab><<<grid_for(c, nbatch * 32, threads, 2), threads, sm, c->stream>>>(
            c->pos.p, c->conn.p, c->E.p, c->E_per_elem, sp(nu / ((1.0 + nu) * (1.0 - 2.0 * nu))),
            sp(1.0 / (2.0 * (1.0 + nu))), c->nu, c->nu_per_elem ? c->nuv.p : nullptr, c->ne, c->Ke64.p);
    } else {
        const size_t sm = sizeof(ElSmem<EL, float>) * kElWarps;
        LMTG_CUDA(cudaFuncSetAttribute(k_elast<EL, float, kTab>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        k_elast<EL, float, kTab><<<grid_for(c, nbatch * 32, threads, 4), threads, sm, c->stream>>>(
            c->pos.p, c->conn.p, c->E.p, c->E_per_elem, c->nu, c->nu_per_elem ? c->nuv.p : nullptr, c->ne,
            c->Ke32.p);
    }
    LMTG_CUDA(cudaGetLastError());
    c->launches += 1;
}

void launch_elem_elast(lmtg_ctx *c, bool fp64) {
    if (!g_pairs_ready[c->device & 63]) {
        unsigned char pa[2][64] = {{0}}, pb[2][64] = {{0}};
        const int npes[2] = {8, 10};
        for (int t = 0; t < 2; ++t)
            for (int a = 0; a < npes[t]; ++a)
                for (int b = a; b < npes[t]; ++b) {
                    const int p = pair_index(a, b, npes[t]);
                    pa[t][p] = (unsigned char)a;
                    pb[t][p] = (unsigned char)b;
                }
        LMTG_CUDA(cudaMemcpyToSymbol(c_pair_a, pa, sizeof(pa)));
        LMTG_CUDA(cudaMemcpyToSymbol(c_pair_b, pb, sizeof(pb)));
        static ff::f2 dn[2][8][10][3], w[2];
        ff_tables<Hexa8>(dn[0], w[0]);
        ff_tables<Tetra10>(dn[1], w[1]);
        LMTG_CUDA(cudaMemcpyToSymbol(c_dNff, dn, sizeof(dn)));
        LMTG_CUDA(cudaMemcpyToSymbol(c_wff, w, sizeof(w)));
        g_pairs_ready[c->device & 63] = true;
    }
    if (c->elem_type == LMTG_ELEM_HEXA8) launch_t<Hexa8, 0>(c, fp64);
    else launch_t<Tetra10, 1>(c, fp64);
}

}  // namespace lmtg
