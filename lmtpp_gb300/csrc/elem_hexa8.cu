// elem_hexa8.cu -- Hexa8 isotropic-elasticity element matrices (FP64 and FP32).
//
// Replaces the generated add_local_elem_matrix of formulation elasticity_iso on Hexa, called
// once per Gauss point by add_elem_matrix (include/formulation/formulation.h:2918-2932):
//   weak form  sigma(u) : eps(v), sigma = H eps, H = inverse of the isotropic compliance
//              (formulations/formulation_elasticity_iso.py:45-60, formal_lf/material_help.py:116-134)
//   rule       order 2 = 2x2x2 points with the reference table's 12-digit abscissae
//              (include/mesh/element_Hexa.h:5-20), weights 1/8 on the [0,1]^3 cell
//   shape      trilinear (formulations/element_Hexa.py:61-68)
// For an isotropic H the 3x3 block of node pair (a,b) is
//   K_ab = lambda A_ab + mu A_ab^T + mu tr(A_ab) I,   A_ab = sum_gp w detJ grad N_a (x) grad N_b,
// which is the same bilinear form as B^T H B with 9 FMAs per pair and Gauss point.
//
// Mapping: one warp per batch of 8 elements.  Phase 1 (geometry): lane = (element, Gauss
// point); the Jacobian, its inverse and the 8 shape-function gradients go to shared memory
// (G and w*detJ*G).  Phase 2: lane = (element, node pair), 9 tasks per lane, accumulating A_ab
// over the 8 points from shared memory and writing the 3x3 block.  Output layout
// Ke[e][pair][3][3] (pairs a<=b): consecutive lanes write consecutive 72/36-byte blocks.
#include "lmtg_internal.cuh"

namespace lmtg {

constexpr int kH8Npe = 8, kH8Pairs = 36, kH8Batch = 8, kH8Warps = 4;

__constant__ unsigned char c_pair_a[kH8Pairs];
__constant__ unsigned char c_pair_b[kH8Pairs];

template <class T>
struct H8Smem {
    T xyz[kH8Batch][24];
    T G[kH8Batch][8][8][3];   // [element][gauss point][node][dim]
    T GW[kH8Batch][8][8][3];  // w * detJ * G
    T lam[kH8Batch], mu[kH8Batch];
};

template <class T>
__global__ void __launch_bounds__(kH8Warps * 32)
    k_hexa8_elast(const double *__restrict__ pos, const uint32_t *__restrict__ conn,
                  const double *__restrict__ E, int E_per_elem, double nu, uint64_t ne,
                  T *__restrict__ Ke) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    H8Smem<T> &S = reinterpret_cast<H8Smem<T> *>(smem_raw)[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    const uint64_t nbatch = (ne + kH8Batch - 1) / kH8Batch;
    const uint64_t warp0 = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    // Gauss abscissae of the reference table (12 significant digits)
    const T ga = (T)0.211324865405, gb = (T)0.788675134595;

    for (uint64_t batch = warp0; batch < nbatch; batch += nwarps) {
        const uint64_t e0 = batch * kH8Batch;
        // cooperative load of the 8 elements' node coordinates
        for (int t = lane; t < kH8Batch * 24; t += 32) {
            int le = t / 24, r = t % 24;
            uint64_t e = e0 + le;
            T v = (T)0;
            if (e < ne) v = (T)pos[3ull * conn[e * kH8Npe + r / 3] + r % 3];
            S.xyz[le][r] = v;
        }
        if (lane < kH8Batch) {
            uint64_t e = e0 + lane;
            double Ee = e < ne ? E[E_per_elem ? e : 0] : 0.0;
            S.lam[lane] = (T)(Ee * nu / ((1.0 + nu) * (1.0 - 2.0 * nu)));
            S.mu[lane] = (T)(Ee / (2.0 * (1.0 + nu)));
        }
        __syncwarp();
        // phase 1: geometry per (element, Gauss point)
        for (int t = lane; t < kH8Batch * 8; t += 32) {
            const int le = t >> 3, g = t & 7;
            const T x = (g == 1 || g == 2 || g == 5 || g == 6) ? gb : ga;
            const T y = (g == 2 || g == 3 || g == 6 || g == 7) ? gb : ga;
            const T z = (g >= 4) ? gb : ga;
            const T mx = 1 - x, my = 1 - y, mz = 1 - z;
            const T dN[8][3] = {{-my * mz, -mx * mz, -mx * my}, {my * mz, -x * mz, -x * my},
                                {y * mz, x * mz, -x * y},      {-y * mz, mx * mz, -mx * y},
                                {-my * z, -mx * z, mx * my},   {my * z, -x * z, x * my},
                                {y * z, x * z, x * y},         {-y * z, mx * z, mx * y}};
            T J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
#pragma unroll
            for (int a = 0; a < 8; ++a)
#pragma unroll
                for (int i = 0; i < 3; ++i)
#pragma unroll
                    for (int j = 0; j < 3; ++j) J[i][j] += S.xyz[le][3 * a + i] * dN[a][j];
            const T c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
            const T c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
            const T c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
            const T det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
            const T id = (T)1 / det;
            // Jinv[j][i]: gradient g_i = sum_j Jinv[j][i] dN_j
            const T Ji[3][3] = {
                {c00 * id, (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * id,
                 (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id},
                {c01 * id, (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id,
                 (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * id},
                {c02 * id, (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * id,
                 (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id}};
            const T wdet = (T)0.125 * det;
#pragma unroll
            for (int a = 0; a < 8; ++a)
#pragma unroll
                for (int i = 0; i < 3; ++i) {
                    T gi = Ji[0][i] * dN[a][0] + Ji[1][i] * dN[a][1] + Ji[2][i] * dN[a][2];
                    S.G[le][g][a][i] = gi;
                    S.GW[le][g][a][i] = wdet * gi;
                }
        }
        __syncwarp();
        // phase 2: node-pair blocks
        for (int t = lane; t < kH8Batch * kH8Pairs; t += 32) {
            const int le = t / kH8Pairs, p = t - le * kH8Pairs;
            const uint64_t e = e0 + le;
            if (e >= ne) break;  // tasks are ordered by element: the rest are past the end
            const int a = c_pair_a[p], b = c_pair_b[p];
            T A[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
#pragma unroll
            for (int g = 0; g < 8; ++g) {
                const T wa0 = S.GW[le][g][a][0], wa1 = S.GW[le][g][a][1], wa2 = S.GW[le][g][a][2];
                const T gb0 = S.G[le][g][b][0], gb1 = S.G[le][g][b][1], gb2 = S.G[le][g][b][2];
                A[0][0] += wa0 * gb0; A[0][1] += wa0 * gb1; A[0][2] += wa0 * gb2;
                A[1][0] += wa1 * gb0; A[1][1] += wa1 * gb1; A[1][2] += wa1 * gb2;
                A[2][0] += wa2 * gb0; A[2][1] += wa2 * gb1; A[2][2] += wa2 * gb2;
            }
            const T lam = S.lam[le], mu = S.mu[le];
            const T tr = mu * (A[0][0] + A[1][1] + A[2][2]);
            T *o = Ke + (e * kH8Pairs + p) * 9;
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j)
                    o[3 * i + j] = lam * A[i][j] + mu * A[j][i] + (i == j ? tr : (T)0);
        }
        __syncwarp();
    }
}

static bool g_pairs_ready[64] = {false};

void launch_hexa8_elast(lmtg_ctx *c, bool fp64) {
    if (!g_pairs_ready[c->device & 63]) {
        unsigned char pa[kH8Pairs], pb[kH8Pairs];
        for (int a = 0; a < 8; ++a)
            for (int b = a; b < 8; ++b) {
                int p = pair_index(a, b, 8);
                pa[p] = (unsigned char)a;
                pb[p] = (unsigned char)b;
            }
        LMTG_CUDA(cudaMemcpyToSymbol(c_pair_a, pa, sizeof(pa)));
        LMTG_CUDA(cudaMemcpyToSymbol(c_pair_b, pb, sizeof(pb)));
        g_pairs_ready[c->device & 63] = true;
    }
    const int threads = kH8Warps * 32;
    const uint64_t nbatch = (c->ne + kH8Batch - 1) / kH8Batch;
    if (fp64) {
        size_t sm = sizeof(H8Smem<double>) * kH8Warps;
        LMTG_CUDA(cudaFuncSetAttribute(k_hexa8_elast<double>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        int grid = grid_for(c, nbatch * 32, threads, 2);
        k_hexa8_elast<double><<<grid, threads, sm, c->stream>>>(
            c->pos.p, c->conn.p, c->E.p, c->E_per_elem, c->nu, c->ne, c->Ke64.p);
    } else {
        size_t sm = sizeof(H8Smem<float>) * kH8Warps;
        LMTG_CUDA(cudaFuncSetAttribute(k_hexa8_elast<float>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        int grid = grid_for(c, nbatch * 32, threads, 4);
        k_hexa8_elast<float><<<grid, threads, sm, c->stream>>>(
            c->pos.p, c->conn.p, c->E.p, c->E_per_elem, c->nu, c->ne, c->Ke32.p);
    }
    LMTG_CUDA(cudaGetLastError());
    c->launches += 1;
}

}  // namespace lmtg
