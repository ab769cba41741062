// diffusion.cu -- transient heat diffusion on Triangle_6 (formulation difftherm): element matrices,
// theta-scheme assembly, scalar CSR PCG, time stepping and the misfit adjoint with checkpoints.
//
// Reference: formulations/formulation_difftherm.py:24-30 (a grad T . grad v + T' v, a =
// conductivity / (density * heat capacity)); time integration: the residual evaluated at the
// midpoint of [t_n, t_n+1] with T interpolated linearly (formal_lf/formulation.py:506-509,
// formal_lf/extrapolation.py:21-40, formal_lf/gauss_integration.py:52-63), i.e. the theta
// scheme with theta = 1/2:
//     A T_{n+1} = B T_n,   A = M/dt + theta K,   B = M/dt - (1 - theta) K,
// theta = 1 gives implicit Euler.  Element rule: the 6-point triangle rule of the closed-form
// element integration (formulations/element_Triangle_6.py:92-99).  Dirichlet T = 0 uses the
// reference's penalty (formulation.h:1028-1071) on A.
//
// One unknown per node: the node-block pattern of pattern.cu is the scalar CSR pattern; a row
// holds 9 or 19 entries (11.5 on average).  The FP64 products stream a warp's 32 rows at a time
// (csr_stream32); the FP32 solver's products go through a bulk-copy (TMA) ring with a lane per
// row, and its preconditioner is Jacobi or the scalar aggregation multigrid below.
#include <algorithm>
#include <type_traits>
#include <chrono>
#include <cmath>
#include <cstring>
#include <exception>
#include <memory>
#include <new>
#include <vector>

#include "ffloat.cuh"
#include "pdl.cuh"
#include "spmv_bulk.cuh"

namespace lmtg {

constexpr int kTriPairs = 21;

__device__ __forceinline__ void tri6_point(int g, double &w, double &u, double &v) {
    const double a = 0.445948490915965, b = 0.091576213509771;
    const double wa = 0.111690794839005, wb = 0.054975871827661;
    const int k = g % 3;
    const double p = g < 3 ? a : b;
    w = g < 3 ? wa : wb;
    u = k == 1 ? 1.0 - 2.0 * p : p;
    v = k == 2 ? 1.0 - 2.0 * p : p;
}

__device__ __forceinline__ void tri6_shape(double u, double v, double (&N)[6], double (&dN)[6][2]) {
    const double X0 = 1 - u - v;
    N[0] = X0 * (2 * X0 - 1); N[1] = u * (2 * u - 1); N[2] = v * (2 * v - 1);
    N[3] = 4 * X0 * u;        N[4] = 4 * u * v;       N[5] = 4 * v * X0;
    dN[0][0] = -(4 * X0 - 1); dN[0][1] = -(4 * X0 - 1);
    dN[1][0] = 4 * u - 1;     dN[1][1] = 0;
    dN[2][0] = 0;             dN[2][1] = 4 * v - 1;
    dN[3][0] = 4 * (X0 - u);  dN[3][1] = -4 * u;
    dN[4][0] = 4 * v;         dN[4][1] = 4 * u;
    dN[5][0] = -4 * v;        dN[5][1] = 4 * (X0 - v);
}

// gradients of the 6 shape functions and w*detJ at Gauss point g
__device__ __forceinline__ double tri6_geom(const double (&xy)[6][2], int g, double (&N)[6],
                                            double (&gx)[6][2]) {
    double w, u, v, dN[6][2];
    tri6_point(g, w, u, v);
    tri6_shape(u, v, N, dN);
    double J[2][2] = {{0, 0}, {0, 0}};
#pragma unroll
    for (int k = 0; k < 6; ++k)
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
            for (int j = 0; j < 2; ++j) J[i][j] = fma(xy[k][i], dN[k][j], J[i][j]);
    const double det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
    const double id = 1.0 / det;
    const double Ji[2][2] = {{J[1][1] * id, -J[0][1] * id}, {-J[1][0] * id, J[0][0] * id}};
#pragma unroll
    for (int k = 0; k < 6; ++k)
#pragma unroll
        for (int i = 0; i < 2; ++i) gx[k][i] = Ji[0][i] * dN[k][0] + Ji[1][i] * dN[k][1];
    return w * det;
}

// element blocks of A = M/dt + theta K and B = M/dt - (1-theta) K (upper pairs, 21 each)
__global__ void k_tri6_diff(const double *__restrict__ pos, const uint32_t *__restrict__ conn,
                            const double *__restrict__ a, int a_per_elem, double inv_rho_c,
                            double dt, double theta, uint64_t ne, double *__restrict__ KA,
                            double *__restrict__ KB) {
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < ne;
         e += (uint64_t)gridDim.x * blockDim.x) {
        double xy[6][2];
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            const uint64_t n = conn[6 * e + k];
            xy[k][0] = pos[2 * n];
            xy[k][1] = pos[2 * n + 1];
        }
        const double ae = a[a_per_elem ? e : 0] * inv_rho_c;
        double K[kTriPairs], M[kTriPairs];
#pragma unroll
        for (int p = 0; p < kTriPairs; ++p) K[p] = M[p] = 0.0;
#pragma unroll 1
        for (int g = 0; g < 6; ++g) {
            double N[6], gx[6][2];
            const double wd = tri6_geom(xy, g, N, gx);
            int p = 0;
#pragma unroll
            for (int i = 0; i < 6; ++i)
#pragma unroll
                for (int j = i; j < 6; ++j, ++p) {
                    K[p] = fma(wd, gx[i][0] * gx[j][0] + gx[i][1] * gx[j][1], K[p]);
                    M[p] = fma(wd, N[i] * N[j], M[p]);
                }
        }
        const double idt = 1.0 / dt;
#pragma unroll
        for (int p = 0; p < kTriPairs; ++p) {
            KA[e * kTriPairs + p] = M[p] * idt + theta * ae * K[p];
            KB[e * kTriPairs + p] = M[p] * idt - (1.0 - theta) * ae * K[p];
        }
    }
}

// gather assembly of the scalar matrices (one value per pattern entry); A also rounded to FP32
__global__ void k_assemble_s(const uint32_t *__restrict__ gptr, const uint32_t *__restrict__ gsrc,
                             const double *__restrict__ KA, const double *__restrict__ KB,
                             uint64_t nnz, double *__restrict__ A, double *__restrict__ B,
                             float *__restrict__ A32) {
    for (uint64_t q = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; q < nnz;
         q += (uint64_t)gridDim.x * blockDim.x) {
        double sa = 0.0, sb = 0.0;
        for (uint32_t g = gptr[q]; g < gptr[q + 1]; ++g) {
            const uint32_t src = __ldg(gsrc + g) >> 1;  // 1x1 blocks: no transpose
            sa += KA[src];
            sb += KB[src];
        }
        A[q] = sa;
        B[q] = sb;
        A32[q] = (float)sa;
    }
}

__global__ void k_max_diag_s(const uint32_t *__restrict__ bdiag, const double *__restrict__ A,
                             uint64_t nn, unsigned long long *out) {
    double m = 0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < nn;
         i += (uint64_t)gridDim.x * blockDim.x)
        m = fmax(m, fabs(A[bdiag[i]]));
    m = warp_max(m);
    if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(m));
}

__global__ void k_penalty_s(const uint32_t *__restrict__ bdiag, double *A, float *A32,
                            const uint32_t *__restrict__ nodes, uint64_t nc, double penalty,
                            const unsigned long long *md_bits) {
    const double md = __longlong_as_double((long long)*md_bits);
    for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < nc;
         k += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t d = bdiag[nodes[k]];
        atomicAdd(A + d, md * penalty);
    }
}

template <class T>
__global__ void k_jacobi_s(const uint32_t *__restrict__ bdiag, const double *__restrict__ A,
                           uint64_t nn, T *Dinv, float *A32) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < nn;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const double d = A[bdiag[i]];
        Dinv[i] = (T)(d != 0.0 ? 1.0 / d : 0.0);
        if (A32) A32[bdiag[i]] = (float)d;  // constrained diagonals after the penalty
    }
}

// ---- scalar CSR kernels: one warp per 32 consecutive rows, entries streamed --------------
// The warp walks the contiguous entry range of its 32 rows in tiles of kTile entries: lane l
// takes entries t0 + 32k + l (coalesced K / col loads, every lane busy whatever the row
// lengths), all loads of a tile issued before the products are formed; the products go to a
// per-warp shared tile and each lane then sums the part of its own row inside the tile, in
// column order.  Rows average ~11.5 entries here, so 8-lanes-per-row kept too few loads in
// flight and left the kernel latency-bound.
constexpr int kTileChunks = 8;
constexpr int kTile = 32 * kTileChunks;
constexpr int kRowWarps = kRowThreads / 32;

// 32-row chunks of this CTA: a contiguous range, its warps interleaved over it
struct ChunkRange {
    uint64_t first, end;
};
__device__ __forceinline__ ChunkRange cta_chunks(uint64_t n) {
    const uint64_t nch = (n + 31) / 32;
    const uint64_t per = (nch + gridDim.x - 1) / gridDim.x;
    const uint64_t b = (uint64_t)blockIdx.x * per;
    return {b < nch ? b : nch, b + per < nch ? b + per : nch};
}

// Row sums of K x~ for rows r0 .. r0+31 (x~_j = xf(j)); returns lane l's row sum (0 past n).
template <class T, class XF>
__device__ __forceinline__ T csr_stream32(const uint32_t *__restrict__ rp, const uint32_t *__restrict__ col,
                                          const T *__restrict__ K, uint64_t r0, uint64_t n, T *tile,
                                          XF xf) {
    const int lane = threadIdx.x & 31;
    const uint64_t I = r0 + lane;
    const uint32_t rs = __ldg(rp + (I < n ? I : n));
    uint32_t re = __shfl_down_sync(0xffffffffu, rs, 1);
    if (lane == 31) re = __ldg(rp + (r0 + 32 < n ? r0 + 32 : n));
    const uint32_t e0 = __shfl_sync(0xffffffffu, rs, 0);
    const uint32_t e1 = __shfl_sync(0xffffffffu, re, 31);
    T acc = (T)0;
    for (uint32_t t0 = e0; t0 < e1; t0 += kTile) {
        const uint32_t nck = (e1 - t0 + 31) / 32;  // live chunks of this tile (warp-uniform)
        uint32_t cj[kTileChunks];
        T kv[kTileChunks];
#pragma unroll
        for (int k = 0; k < kTileChunks; ++k) {
            if (k < nck) {
                const uint32_t q = t0 + 32 * k + lane;
                const bool on = q < e1;
                cj[k] = on ? __ldcs(col + q) : 0u;  // streamed once: keep L1 for the gathers
                kv[k] = on ? __ldcs(K + q) : (T)0;
            }
        }
        T xv[kTileChunks];
#pragma unroll
        for (int k = 0; k < kTileChunks; ++k)
            if (k < nck) xv[k] = t0 + 32 * k + lane < e1 ? xf(cj[k]) : (T)0;
#pragma unroll
        for (int k = 0; k < kTileChunks; ++k)
            if (k < nck) tile[32 * k + lane] = kv[k] * xv[k];
        __syncwarp();
        const uint32_t lo = rs > t0 ? rs : t0;
        const uint32_t hi = re < t0 + kTile ? re : t0 + kTile;
        for (uint32_t q = lo; q < hi; ++q) acc += tile[q - t0];
        __syncwarp();
    }
    return acc;
}

template <class T>
__global__ void __launch_bounds__(kRowThreads)
    k_spmv_s(const uint32_t *__restrict__ rp, const uint32_t *__restrict__ col,
             const T *__restrict__ K, const T *__restrict__ x, T *__restrict__ y, uint64_t n) {
    __shared__ T tiles[kRowWarps][kTile];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const ChunkRange cr = cta_chunks(n);
    for (uint64_t ch = cr.first + w; ch < cr.end; ch += kRowWarps) {
        const T v = csr_stream32(rp, col, K, ch * 32, n, tiles[w], [&](uint32_t j) { return __ldg(x + j); });
        const uint64_t I = ch * 32 + lane;
        if (I < n) y[I] = v;
    }
}

template <class T>
__global__ void __launch_bounds__(kRowThreads)
    k_residual_s(const uint32_t *__restrict__ rp, const uint32_t *__restrict__ col,
                 const T *__restrict__ K, const T *__restrict__ x, const T *__restrict__ b,
                 T *__restrict__ r, uint64_t n, double *partials, unsigned *ticket, double *rr_out) {
    __shared__ T tiles[kRowWarps][kTile];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const ChunkRange cr = cta_chunks(n);
    T acc = (T)0;
    for (uint64_t ch = cr.first + w; ch < cr.end; ch += kRowWarps) {
        const T v = csr_stream32(rp, col, K, ch * 32, n, tiles[w], [&](uint32_t j) { return __ldg(x + j); });
        const uint64_t I = ch * 32 + lane;
        if (I < n) {
            const T ri = b[I] - v;
            r[I] = ri;
            acc = fma(ri, ri, acc);
        }
    }
    const T t[1] = {acc};
    double out[1];
    if (grid_reduce_t<1, 0u>(t, partials, ticket, out) && threadIdx.x == 0) *rr_out = out[0];
}

template <class T>
__global__ void k_pcg_start_s(const T *__restrict__ r, const T *__restrict__ b,
                              const T *__restrict__ Dinv, T *__restrict__ z, uint64_t n,
                              PcgScalars *S, double *partials) {
    T t[3] = {(T)0, (T)0, (T)0};  // rz, rr, bb
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const T ri = r[i], zi = Dinv[i] * ri;
        z[i] = zi;
        t[0] = fma(ri, zi, t[0]);
        t[1] = fma(ri, ri, t[1]);
        if (b) t[2] = fma(b[i], b[i], t[2]);
    }
    double out[3];
    if (grid_reduce_t<3, 0u>(t, partials, &S->cnt_c, out) && threadIdx.x == 0) {
        S->rz = out[0];
        S->rr = out[1];
        if (b) S->bb = out[2];
        S->beta = 0.0;
        S->iter = 0;
        S->status = LMTG_OK;
        S->done = (out[1] <= S->crit * S->crit * S->bb) ? 1 : 0;
        if (!isfinite(out[0]) || !isfinite(out[1])) {
            S->done = 1;
            S->status = LMTG_ERR_NAN;
        }
    }
}

// p = z + beta p (beta = 0 on a fresh start): its own pass, so that the SpMV gathers one vector
// and the FP64 pipe forms no z + beta p per matrix entry
template <class T>
__global__ void k_pcg_dir_s(const T *__restrict__ z, T *__restrict__ p, uint64_t n, const PcgScalars *S) {
    if (*(volatile const int *)&S->done) return;
    const T beta = (T)S->beta;
    uint64_t i0 = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
    if constexpr (std::is_same<T, float>::value) {  // four nodes per 16-byte access
        const uint64_t n4 = n / 4;
        const float4 *z4 = reinterpret_cast<const float4 *>(z);
        float4 *p4 = reinterpret_cast<float4 *>(p);
        for (uint64_t g = i0; g < n4; g += step) {
            const float4 zz = z4[g];
            if (beta != 0.f) {
                const float4 pp = p4[g];
                p4[g] = make_float4(fmaf(beta, pp.x, zz.x), fmaf(beta, pp.y, zz.y), fmaf(beta, pp.z, zz.z),
                                    fmaf(beta, pp.w, zz.w));
            } else {
                p4[g] = zz;
            }
        }
        i0 += 4 * n4;
    }
    for (uint64_t i = i0; i < n; i += step)
        p[i] = beta != (T)0 ? fma(beta, p[i], z[i]) : z[i];
}

// q = K p and p.q
template <class T>
__global__ void __launch_bounds__(kRowThreads)
    k_pcg_spmv_s(const uint32_t *__restrict__ rp, const uint32_t *__restrict__ col,
                 const T *__restrict__ K, const T *__restrict__ p, T *__restrict__ q, uint64_t n,
                 PcgScalars *S, double *partials) {
    if (*(volatile int *)&S->done) return;
    __shared__ T tiles[kRowWarps][kTile];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const ChunkRange cr = cta_chunks(n);
    T acc = (T)0;
    for (uint64_t ch = cr.first + w; ch < cr.end; ch += kRowWarps) {
        const T qi = csr_stream32(rp, col, K, ch * 32, n, tiles[w], [&](uint32_t j) { return __ldg(p + j); });
        const uint64_t I = ch * 32 + lane;
        if (I < n) {
            q[I] = qi;
            acc = fma(p[I], qi, acc);
        }
    }
    const T t[1] = {acc};
    double out[1];
    if (grid_reduce_t<1, 0u>(t, partials, &S->cnt_a, out) && threadIdx.x == 0) {
        S->pq = out[0];
        S->alpha = S->rz / (out[0] + (out[0] == 0.0 ? 1.0 : 0.0));  // once, not per thread
    }
}

// q = K p and p.q (FP32) with the matrix streamed through shared memory by bulk copies (TMA).
// Each CTA owns a contiguous range of 32-row chunks.  One producer warp copies, per stage, the
// entries (values, columns) and the row pointers of up to 8 chunks whose entries fit kCap into
// a ring of kStages stages (evict-first L2 policy).  Consumer warp w takes chunk w of a stage:
// lane l sums row l, reading the row's entries from shared memory and gathering p directly
// (four entries in flight), then the stage goes back.  Forming the products in shared memory
// first (the warp-streamed layout of csr_stream32) cost 10% more: it doubled the L1 traffic.
// Each product is rounded and then added in column order, as in csr_stream32, so q is
// bit-identical to k_pcg_spmv_s; p.q is summed in another fixed order.  Every wait is bounded; one that gives up sets
// LMTG_ERR_TIMEOUT and done in the PCG scalars.
// The epilogue Epi gives the gathered vector (x), what a row's sum becomes (row) and, with
// kReduce, the grid total of the rows' contributions (total, by the thread that finishes it):
// the PCG's q = K p with p.q, and the multigrid's level-0 residual and post-smoothing.
constexpr int kSBulkCons = 8;

struct EpiSPq {  // q = K p; p.q, alpha = rz / p.q
    const float *p;
    float *q;
    static constexpr bool kReduce = true;
    __device__ __forceinline__ float x(uint32_t j) const { return __ldg(p + j); }
    __device__ __forceinline__ void row(uint64_t I, float v, float &acc) const {
        q[I] = v;
        acc = fmaf(p[I], v, acc);
    }
    __device__ __forceinline__ unsigned *ticket(PcgScalars *S) const { return &S->cnt_a; }
    __device__ __forceinline__ void total(double v, PcgScalars *S) const {
        S->pq = v;
        S->alpha = S->rz / (v + (v == 0.0 ? 1.0 : 0.0));
    }
};
constexpr int kSBulkThreads = 32 * (kSBulkCons + 1);

// Columns are either the 32-bit indices or, when every |col - row| < 2^15 (a banded numbering,
// as the structured meshes have), 16-bit deltas col - row: a quarter fewer bytes per entry
// (values 4 + columns 2), the same products in the same order.
__device__ __forceinline__ uint32_t col_at(uint32_t c, uint64_t) { return c; }
__device__ __forceinline__ uint32_t col_at(int16_t d, uint64_t I) { return (uint32_t)((int64_t)I + d); }

template <int kCap, int kColBytes>
struct SBulkStage {
    static_assert(kCap % 8 == 0, "16-byte stage parts");
    static constexpr uint32_t kKBytes = 4u * kCap + 32u;
    static constexpr uint32_t kCBytes = (uint32_t)kColBytes * kCap + 32u;
    static constexpr uint32_t kRBytes = 4u * (32 * kSBulkCons + 1) + 32u + 12u;  // rounded to 16
    static constexpr uint32_t kBytes = kKBytes + kCBytes + kRBytes;
    static_assert(kRBytes % 16 == 0 && kBytes % 16 == 0, "16-byte stage parts");
};
template <int kStages, int kCap, int kColBytes = 4>
constexpr size_t sbulk_smem_bytes() {
    return (size_t)kStages * SBulkStage<kCap, kColBytes>::kBytes;
}

// the ring the solvers launch: two stages of up to 3072 entries (a 32-row chunk must fit one)
constexpr int kSStages = 2, kSCap = 3072;

template <int kStages, int kCap, class Epi, class CT = uint32_t>
__global__ void __launch_bounds__(kSBulkThreads, 4)
    k_pcg_spmv_s_bulk(const uint32_t *__restrict__ rp, const CT *__restrict__ col,
                      const float *__restrict__ K, Epi epi, uint64_t n, PcgScalars *S, double *partials) {
    using St = SBulkStage<kCap, (int)sizeof(CT)>;
    constexpr uint64_t kCB = sizeof(CT);
    if (*(volatile int *)&S->done) return;
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ uint64_t full[kStages], empty[kStages];
    __shared__ uint64_t meta[kStages][5];  // first row, end row, first value, rp and column index
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const ChunkRange cr = cta_chunks(n);
    const uint64_t row0 = 32 * cr.first, row_end = min(n, 32 * cr.end);
    if (threadIdx.x == 0) {
        for (int i = 0; i < kStages; ++i) {
            bulk::mbar_init(&full[i], 1);
            bulk::mbar_init(&empty[i], kSBulkCons);
        }
        bulk::fence_barrier_init();
    }
    __syncthreads();
    float acc = 0.f;
    if (warp == kSBulkCons) {
        // ---------------- producer ----------------
        uint64_t g0 = row0;
        uint32_t e0 = row0 < row_end ? rp[row0] : 0u;
        uint32_t k = 0, nissued = 0;  // stages whose full barrier got its arrival
        bool failed = false;
        for (;; ++k) {
            const int slot = k % kStages;
            if (k >= (uint32_t)kStages) {
                const bool ok = bulk::mbar_wait(&empty[slot], ((k / kStages) - 1) & 1u);
                if (!__all_sync(0xffffffffu, ok)) {
                    failed = true;
                    break;
                }
            }
            if (g0 >= row_end) {
                if (lane == 0) {
                    meta[slot][0] = g0;
                    meta[slot][1] = g0;
                    bulk::mbar_arrive(&full[slot]);
                }
                nissued = k + 1;
                break;
            }
            // chunk ends g0 + 32 (l + 1) (clamped to row_end) for lanes l < 8
            const bool in = lane < kSBulkCons && g0 + (uint64_t)(32 * lane) < row_end;
            const uint64_t ge = min(row_end, g0 + (uint64_t)(32 * (lane + 1)));
            const uint32_t ei = in ? rp[ge] : 0u;
            const unsigned fits = __ballot_sync(0xffffffffu, in && ei - e0 <= (uint32_t)kCap);
            const int nch = __popc(fits);
            if (nch == 0) {  // a chunk wider than a stage (the host checks this before launching)
                failed = true;
                break;
            }
            const uint32_t e1 = __shfl_sync(0xffffffffu, ei, nch - 1);
            const uint64_t g1 = min(row_end, g0 + (uint64_t)(32 * nch));
            if (lane == 0) {
                const uint64_t kb0 = (4ull * e0) & ~15ull, kb1 = (4ull * e1 + 15ull) & ~15ull;
                const uint64_t cb0 = (kCB * e0) & ~15ull, cb1 = (kCB * e1 + 15ull) & ~15ull;
                const uint64_t rb0 = (4ull * g0) & ~15ull, rb1 = (4ull * (g1 + 1) + 15ull) & ~15ull;
                meta[slot][0] = g0;
                meta[slot][1] = g1;
                meta[slot][2] = kb0 / 4;
                meta[slot][3] = rb0 / 4;
                meta[slot][4] = cb0 / kCB;
                unsigned char *dst = smem + (size_t)slot * St::kBytes;
                const uint64_t pol = bulk::policy_evict_first();
                __threadfence_block();
                bulk::mbar_arrive_expect_tx(&full[slot], (uint32_t)((kb1 - kb0) + (cb1 - cb0) + (rb1 - rb0)));
                bulk::copy_g2s_hint(dst, reinterpret_cast<const unsigned char *>(K) + kb0, (uint32_t)(kb1 - kb0),
                                    &full[slot], pol);
                bulk::copy_g2s_hint(dst + St::kKBytes, reinterpret_cast<const unsigned char *>(col) + cb0,
                                    (uint32_t)(cb1 - cb0), &full[slot], pol);
                bulk::copy_g2s_hint(dst + St::kKBytes + St::kCBytes, reinterpret_cast<const unsigned char *>(rp) + rb0,
                                    (uint32_t)(rb1 - rb0), &full[slot], pol);
            }
            g0 = g1;
            e0 = e1;
            nissued = k + 1;
        }
        if (lane == 0) {
            if (failed) {
                atomicExch(&S->status, LMTG_ERR_TIMEOUT);
                atomicExch(&S->done, 1);
            }
            // leave only with no copy in flight: the last stage issued on each slot (complete at
            // once when the consumers took every stage)
            const uint32_t first = nissued > (uint32_t)kStages ? nissued - kStages : 0u;
            for (uint32_t s2 = first; s2 < nissued; ++s2) bulk::mbar_wait(&full[s2 % kStages], (s2 / kStages) & 1u);
        }
    } else {
        // ---------------- consumers ----------------
        for (uint32_t k = 0;; ++k) {
            const int slot = k % kStages;
            const bool ok = bulk::mbar_wait(&full[slot], (k / kStages) & 1u);
            if (!__all_sync(0xffffffffu, ok)) {
                if (lane == 0) {
                    atomicExch(&S->status, LMTG_ERR_TIMEOUT);
                    atomicExch(&S->done, 1);
                }
                break;
            }
            const uint64_t g0 = meta[slot][0], g1 = meta[slot][1];
            if (g0 == g1) break;
            float *sK = reinterpret_cast<float *>(smem + (size_t)slot * St::kBytes);
            const CT *sC = reinterpret_cast<const CT *>(smem + (size_t)slot * St::kBytes + St::kKBytes);
            const uint32_t *sR =
                reinterpret_cast<const uint32_t *>(smem + (size_t)slot * St::kBytes + St::kKBytes + St::kCBytes);
            const uint64_t kbase = meta[slot][2], rbase = meta[slot][3], cbase = meta[slot][4];
            const uint64_t R0 = g0 + (uint64_t)(32 * warp);
            if (R0 < g1) {
                const uint64_t R1 = min(g1, R0 + (uint64_t)32);
                const uint64_t I = R0 + lane;
                float v = 0.f;
                if (I < R1) {
                    const uint32_t rs = sR[I - rbase], re = sR[I + 1 - rbase];
#pragma unroll 8
                    for (uint32_t qq = rs; qq < re; ++qq)
                        v += __fmul_rn(sK[qq - kbase], epi.x(col_at(sC[qq - cbase], I)));
                }
                __syncwarp();
                if (lane == 0) bulk::mbar_arrive(&empty[slot]);
                if (I < R1) epi.row(I, v, acc);
            } else {
                __syncwarp();
                if (lane == 0) bulk::mbar_arrive(&empty[slot]);
            }
        }
    }
    if constexpr (Epi::kReduce) {
        __syncthreads();
        const float t[1] = {acc};
        double out[1];
        if (grid_reduce_t<1, 0u>(t, partials, epi.ticket(S), out) && threadIdx.x == 0) epi.total(out[0], S);
    }
}

// grid of one resident wave of the bulk-copy kernel with epilogue Epi and column type CT (the
// function's shared-memory ceiling set on first use)
template <class Epi, class CT>
static int sbulk_grid(lmtg_ctx *c) {
    static int grid = 0;
    if (!grid) {
        constexpr size_t smem = sbulk_smem_bytes<kSStages, kSCap, (int)sizeof(CT)>();
        auto fn = k_pcg_spmv_s_bulk<kSStages, kSCap, Epi, CT>;
        LMTG_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        int nb = 0;
        LMTG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, kSBulkThreads, smem));
        grid = c->sm_count * (nb > 0 ? nb : 1);
    }
    return grid;
}

// K x through the bulk-copy kernel on the context's pattern: 16-bit column deltas when they fit
template <class Epi>
static void sbulk_launch(lmtg_ctx *c, const float *K, Epi epi, cudaStream_t s) {
    if (c->col16)
        k_pcg_spmv_s_bulk<kSStages, kSCap, Epi, int16_t>
            <<<sbulk_grid<Epi, int16_t>(c), kSBulkThreads, sbulk_smem_bytes<kSStages, kSCap, 2>(), s>>>(
                c->bptr.p, c->bcol16.p, K, epi, c->nn, c->scal.p, c->partials.p);
    else
        k_pcg_spmv_s_bulk<kSStages, kSCap, Epi, uint32_t>
            <<<sbulk_grid<Epi, uint32_t>(c), kSBulkThreads, sbulk_smem_bytes<kSStages, kSCap, 4>(), s>>>(
                c->bptr.p, c->bcol.p, K, epi, c->nn, c->scal.p, c->partials.p);
}

// column deltas col - row of the pattern as 16-bit integers; *over = 1 when one does not fit
__global__ void k_col16(const uint32_t *__restrict__ rp, const uint32_t *__restrict__ col, uint64_t n,
                        int16_t *__restrict__ c16, int *over) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        for (uint32_t e = rp[i]; e < rp[i + 1]; ++e) {
            const int64_t d = (int64_t)col[e] - (int64_t)i;
            const bool fits = d >= -32768 && d <= 32767;
            c16[e] = fits ? (int16_t)d : (int16_t)0;
            if (!fits) *over = 1;
        }
    }
}

template <class T>
__global__ void k_pcg_update_s(T *__restrict__ x, T *__restrict__ r, T *__restrict__ z,
                               const T *__restrict__ p, const T *__restrict__ q,
                               const T *__restrict__ Dinv, uint64_t n, PcgScalars *S,
                               double *partials) {
    if (*(volatile int *)&S->done) return;
    const double pq = S->pq;
    const T alpha = (T)S->alpha;
    T t[2] = {(T)0, (T)0};
    uint64_t i0 = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
    if constexpr (std::is_same<T, float>::value) {  // four nodes per 16-byte access
        const uint64_t n4 = n / 4;
        float4 *x4 = reinterpret_cast<float4 *>(x), *r4 = reinterpret_cast<float4 *>(r),
               *z4 = reinterpret_cast<float4 *>(z);
        const float4 *p4 = reinterpret_cast<const float4 *>(p), *q4 = reinterpret_cast<const float4 *>(q),
                     *d4 = reinterpret_cast<const float4 *>(Dinv);
        for (uint64_t g = i0; g < n4; g += step) {
            float xv[4], rv[4], pv[4], qv[4], dv[4], zv[4];
            *reinterpret_cast<float4 *>(xv) = x4[g];
            *reinterpret_cast<float4 *>(rv) = r4[g];
            *reinterpret_cast<float4 *>(pv) = p4[g];
            *reinterpret_cast<float4 *>(qv) = q4[g];
            *reinterpret_cast<float4 *>(dv) = d4[g];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                xv[k] = fmaf(alpha, pv[k], xv[k]);
                rv[k] = fmaf(-alpha, qv[k], rv[k]);
                zv[k] = dv[k] * rv[k];
                t[0] = fmaf(rv[k], zv[k], t[0]);
                t[1] = fmaf(rv[k], rv[k], t[1]);
            }
            x4[g] = *reinterpret_cast<const float4 *>(xv);
            r4[g] = *reinterpret_cast<const float4 *>(rv);
            z4[g] = *reinterpret_cast<const float4 *>(zv);
        }
        i0 += 4 * n4;  // the last n % 4 nodes below
    }
    for (uint64_t i = i0; i < n; i += step) {
        x[i] = fma(alpha, p[i], x[i]);
        const T ri = fma(-alpha, q[i], r[i]);
        r[i] = ri;
        const T zi = Dinv[i] * ri;
        z[i] = zi;
        t[0] = fma(ri, zi, t[0]);
        t[1] = fma(ri, ri, t[1]);
    }
    double out[2];
    if (grid_reduce_t<2, 0u>(t, partials, &S->cnt_b, out) && threadIdx.x == 0) {
        const double rz_old = S->rz;
        S->iter += 1;
        S->rr = out[1];
        S->beta = out[0] / rz_old;
        S->rz = out[0];
        if (!isfinite(out[0]) || !isfinite(out[1]) || !isfinite(pq)) {
            S->status = LMTG_ERR_NAN;
            S->done = 1;
        } else if (out[1] <= S->crit * S->crit * S->bb) {
            S->done = 1;
        } else if (S->iter >= S->maxit) {
            S->status = LMTG_ERR_NOT_CONVERGED;
            S->done = 1;
        }
    }
}

// misfit gradient accumulation for the theta scheme:
//   g_e -= lambda_e^T Khat_e (theta T_n + (1 - theta) T_{n-1})_e,  Khat_e = int gradN.gradN
__global__ void k_tri6_grad(const double *__restrict__ pos, const uint32_t *__restrict__ conn,
                            uint64_t ne, double theta, const double *__restrict__ lam,
                            const double *__restrict__ Tn, const double *__restrict__ Tm,
                            double *__restrict__ g) {
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < ne;
         e += (uint64_t)gridDim.x * blockDim.x) {
        double xy[6][2], lv[6], wv[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            const uint64_t n = conn[6 * e + k];
            xy[k][0] = pos[2 * n];
            xy[k][1] = pos[2 * n + 1];
            lv[k] = lam[n];
            wv[k] = theta * Tn[n] + (1.0 - theta) * Tm[n];
        }
        double acc = 0.0;
#pragma unroll 1
        for (int gp = 0; gp < 6; ++gp) {
            double N[6], gx[6][2];
            const double wd = tri6_geom(xy, gp, N, gx);
            double gl[2] = {0, 0}, gw[2] = {0, 0};
#pragma unroll
            for (int k = 0; k < 6; ++k)
#pragma unroll
                for (int i = 0; i < 2; ++i) {
                    gl[i] = fma(lv[k], gx[k][i], gl[i]);
                    gw[i] = fma(wv[k], gx[k][i], gw[i]);
                }
            acc = fma(wd, gl[0] * gw[0] + gl[1] * gw[1], acc);
        }
        g[e] -= acc;
    }
}

__global__ void k_axpby(const double *__restrict__ a, const double *__restrict__ b, double *c,
                        uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x)
        c[i] = a[i] - (b ? b[i] : 0.0);
}

// ---- host -----------------------------------------------------------------------------------
// row kernels: one resident wave (each CTA owns a contiguous range of 32-row chunks)
template <class KF>
static int rgrid(lmtg_ctx *c, KF kernel) {
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, kRowThreads, 0) != cudaSuccess || nb < 1)
        nb = 1;
    return grid_for(c, c->nn, kRowThreads, nb);
}
static int ngrid(lmtg_ctx *c) { return grid_for(c, c->nn, kRowThreads, 8); }

__global__ void k_dot_s(const double *__restrict__ a, const double *__restrict__ b, uint64_t n,
                        double *partials, unsigned *ticket, double *out_p) {
    double v[1] = {0.0};
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x)
        v[0] = fma(a[i], b[i], v[0]);
    double out[1];
    if (grid_reduce<1, 0u>(v, partials, ticket, out) && threadIdx.x == 0) *out_p = out[0];
}

// ---- scalar aggregation multigrid for the FP32 diffusion PCG --------------------------------
//
// Jacobi needs O(mesh side) iterations on A = M/dt + theta K (about 620 per implicit-Euler step
// of the 1024^2 workload).  With lmtg_set_preconditioner(LMTG_PREC_AMG) (the default) and at least
// kSMinUnknowns unknowns, z = M r is one cycle of an unsmoothed-aggregation multigrid built for
// the scalar matrix, the elasticity multigrid's scheme with one mode per aggregate:
//   aggregation   the node graph's greedy aggregates (a root with its free neighbours, leftovers
//                 joined to the aggregate they touch most, the rest grouped around a free node);
//                 Dirichlet (penalty) nodes stay out
//   prolongator   q_i = B_i / |B|_aggregate: the constant at level 0 (B = 1), then the previous
//                 level's normalisation (B = |B|_aggregate) -- the piecewise-constant modes
//   coarse A      Q^T A Q, thread per aggregate in a fixed order (deterministic)
//   smoother      damped Jacobi omega = 1 / theta of a degree-1 Chebyshev on [h/30, h], h = 1.2
//                 lambda_max(D^-1 A) (twelve power steps), the same before and after
//   cycle         x = omega D^-1 r; res = r - A x; restrict; the coarse correction (a dense solve
//                 on the coarsest, else the next level's cycle: twice below level 0, the second
//                 on the residual the first leaves, once deeper); x += Q e;
//                 x' = x + omega D^-1 (r - A x)
// The matrices are constant over the time steps, so the hierarchy is built once (structure on
// the host, numeric part on the device) at the first FP32 solve after diff_setup or a change of
// the convection terms.
constexpr uint64_t kSMinUnknowns = 3000, kSCoarsest = 500;
constexpr int kSMaxLevels = 10, kSGalCap = 64, kSPowerSteps = 12;
constexpr size_t kSWLevels = 1;  // levels whose coarse correction visits the next level twice
constexpr uint8_t kSNoSlot = 0xff;
constexpr uint32_t kSNone = 0xffffffffu;

// level-0 passes of the cycle on the bulk-copy pipeline
struct EpiSRes {  // res = r - A x
    const float *xv, *r;
    float *res;
    static constexpr bool kReduce = false;
    __device__ __forceinline__ float x(uint32_t j) const { return __ldg(xv + j); }
    __device__ __forceinline__ void row(uint64_t I, float v, float &) const { res[I] = r[I] - v; }
};
struct EpiSPost {  // z = x + omega D^-1 (r - A x); r.z into rz and beta (as k_s_post)
    const float *xv, *r, *D;
    float *z;
    float omega;
    int start;
    double beta_den;
    static constexpr bool kReduce = true;
    __device__ __forceinline__ float x(uint32_t j) const { return __ldg(xv + j); }
    __device__ __forceinline__ void row(uint64_t I, float v, float &acc) const {
        const float ri = r[I];
        const float zi = xv[I] + omega * D[I] * (ri - v);
        z[I] = zi;
        acc = fmaf(ri, zi, acc);
    }
    __device__ __forceinline__ unsigned *ticket(PcgScalars *S) const { return &S->cnt_d; }
    __device__ __forceinline__ void total(double v, PcgScalars *S) const {
        if (start) S->beta = beta_den > 0.0 ? v / beta_den : 0.0;
        else S->beta = v / S->rz;
        S->rz = v;
        if (!isfinite(v)) {
            S->status = LMTG_ERR_NAN;
            S->done = 1;
        }
    }
};

struct SLevel {
    uint64_t n = 0, nnz = 0;
    DBuf<uint32_t> rp, col;            // levels >= 1 (level 0: the context's pattern)
    DBuf<float> A, Dinv;               // levels >= 1 (level 0: K32, Dinv32)
    float omega = 1.f;
    double lambda = 0;
    DBuf<float> r, xa, xb, res, r2, xb2;  // right-hand side, iterates, residual, second visit
    // transfer to the next coarser level
    uint64_t nagg = 0;
    DBuf<uint32_t> agg, aptr, anode;
    DBuf<float> q;        // prolongator value per node
    DBuf<uint8_t> gslot;  // per entry: slot of agg(col) in agg(row)'s coarse row
};

struct SAmg {
    std::vector<std::unique_ptr<SLevel>> lv;
    int nc = 0;  // unknowns of the dense coarsest level
    DBuf<float> Cinv;
    DBuf<double> power;
};

void samg_free(lmtg_ctx *c) {
    if (!c->samg) return;
    diff_graphs_free(c);  // graphs captured on its buffers
    delete c->samg;
    c->samg = nullptr;
}

// slot of every fine entry's coarse column in its coarse row (rows of aggregated nodes)
__global__ void k_s_slots(const uint32_t *__restrict__ rp, const uint32_t *__restrict__ col,
                          const uint32_t *__restrict__ agg, uint64_t n, const uint32_t *__restrict__ crp,
                          const uint32_t *__restrict__ ccol, uint8_t *__restrict__ gslot) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t a = agg[i];
        for (uint32_t e = rp[i]; e < rp[i + 1]; ++e) {
            uint8_t s = kSNoSlot;
            const uint32_t J = agg[col[e]];
            if (a != kSNone && J != kSNone) {
                uint32_t lo = crp[a], hi = crp[a + 1];  // J is in the row: lower_bound finds it
                while (lo < hi) {
                    const uint32_t mid = (lo + hi) >> 1;
                    if (ccol[mid] < J) lo = mid + 1;
                    else hi = mid;
                }
                s = (uint8_t)(lo - crp[a]);
            }
            gslot[e] = s;
        }
    }
}

// coarse row a of Q^T A Q, thread per aggregate: its nodes' entries summed in order in a
// slot-major shared accumulator (conflict-free: acc[slot][thread])
constexpr int kSGalThreads = 128;
__global__ void __launch_bounds__(kSGalThreads)
    k_s_galerkin(const uint32_t *__restrict__ rp, const uint32_t *__restrict__ col, const float *__restrict__ A,
                 const uint8_t *__restrict__ gslot, const float *__restrict__ q, const uint32_t *__restrict__ aptr,
                 const uint32_t *__restrict__ anode, uint64_t na, const uint32_t *__restrict__ crp,
                 const uint32_t *__restrict__ ccol, float *__restrict__ cA) {
    __shared__ float acc[kSGalCap][kSGalThreads];
    const int t = threadIdx.x;
    for (uint64_t a = blockIdx.x * (uint64_t)blockDim.x + t; a < na; a += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t cb = crp[a], cdeg = crp[a + 1] - cb;
        for (uint32_t s = 0; s < cdeg; ++s) acc[s][t] = 0.f;
        for (uint32_t u = aptr[a]; u < aptr[a + 1]; ++u) {
            const uint32_t i = anode[u];
            const float qi = q[i];
            for (uint32_t e = rp[i]; e < rp[i + 1]; ++e) {
                const uint8_t s = gslot[e];
                if (s != kSNoSlot) acc[s][t] += qi * A[e] * q[col[e]];
            }
        }
        for (uint32_t s = 0; s < cdeg; ++s) {
            float v = acc[s][t];
            if (ccol[cb + s] == a && v == 0.f) v = 1.f;  // a decoupled unknown keeps a unit diagonal
            cA[cb + s] = v;
        }
    }
}

__global__ void k_s_dinv(const uint32_t *__restrict__ rp, const uint32_t *__restrict__ col,
                         const float *__restrict__ A, uint64_t n, float *__restrict__ Dinv) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        float d = 1.f;
        for (uint32_t e = rp[i]; e < rp[i + 1]; ++e)
            if (col[e] == i) d = A[e];
        Dinv[i] = d != 0.f ? 1.f / d : 1.f;
    }
}

__device__ __forceinline__ bool s_done(const PcgScalars *S) { return S && *(volatile const int *)&S->done; }

// one power step w = D^-1 A v / |v| (|v|^2 = the previous step's |w|^2 in prev; 1 on the first),
// |w|^2 reduced into out
__global__ void __launch_bounds__(kRowThreads)
    k_s_power(const uint32_t *__restrict__ rp, const uint32_t *__restrict__ col, const float *__restrict__ A,
              const float *__restrict__ Dinv, const float *__restrict__ v, float *__restrict__ w, uint64_t n,
              const double *prev, double *partials, unsigned *ticket, double *out) {
    __shared__ float tiles[kRowWarps][kTile];
    const int wp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float sc = 1.f;
    if (prev) {
        const float p = (float)*prev;
        sc = p > 0.f ? rsqrtf(p) : 1.f;
    }
    float acc = 0.f;
    const ChunkRange cr = cta_chunks(n);
    for (uint64_t ch = cr.first + wp; ch < cr.end; ch += kRowWarps) {
        const float y = csr_stream32(rp, col, A, ch * 32, n, tiles[wp], [&](uint32_t j) { return __ldg(v + j); });
        const uint64_t I = ch * 32 + lane;
        if (I < n) {
            const float wi = sc * Dinv[I] * y;
            w[I] = wi;
            acc = fmaf(wi, wi, acc);
        }
    }
    const float t[1] = {acc};
    double o[1];
    if (grid_reduce_t<1, 0u>(t, partials, ticket, o) && threadIdx.x == 0) *out = o[0];
}

// v = pseudo-random start in [-1, 1)
__global__ void k_s_rand(float *__restrict__ v, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t h = (uint32_t)(i * 2654435761ull) ^ 0x9e3779b9u;
        h ^= h >> 16;
        h *= 0x7feb352du;
        h ^= h >> 15;
        v[i] = (float)(h & 0xffffff) * (2.0f / 16777216.0f) - 1.0f;
    }
}

// res = r - A x; with D also the next visit's first smoothing step xpre = omega D^-1 res
__global__ void __launch_bounds__(kRowThreads)
    k_s_res(const uint32_t *__restrict__ rp, const uint32_t *__restrict__ col, const float *__restrict__ A,
            const float *__restrict__ x, const float *__restrict__ r, float *__restrict__ res, uint64_t n,
            const PcgScalars *S, const float *__restrict__ D, float omega, float *__restrict__ xpre) {
    pdl_wait_trigger();
    if (s_done(S)) return;
    __shared__ float tiles[kRowWarps][kTile];
    const int wp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const ChunkRange cr = cta_chunks(n);
    for (uint64_t ch = cr.first + wp; ch < cr.end; ch += kRowWarps) {
        const float y = csr_stream32(rp, col, A, ch * 32, n, tiles[wp], [&](uint32_t j) { return __ldg(x + j); });
        const uint64_t I = ch * 32 + lane;
        if (I < n) {
            const float ri = r[I] - y;
            res[I] = ri;
            if (D) xpre[I] = omega * D[I] * ri;
        }
    }
}

// xo = x + omega D^-1 (r - A x); with S_rz (level 0 inside the PCG) r.xo is reduced into rz and
// beta (beta = rz / rz_old, or on a start rz / beta_den when beta_den > 0, else 0)
__global__ void __launch_bounds__(kRowThreads)
    k_s_post(const uint32_t *__restrict__ rp, const uint32_t *__restrict__ col, const float *__restrict__ A,
             const float *__restrict__ Dinv, const float *__restrict__ x, const float *__restrict__ r,
             float *__restrict__ xo, float omega, uint64_t n, PcgScalars *S, bool with_rz, int start,
             double beta_den, double *partials) {
    pdl_wait_trigger();
    if (s_done(S)) return;
    __shared__ float tiles[kRowWarps][kTile];
    const int wp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float acc = 0.f;
    const ChunkRange cr = cta_chunks(n);
    for (uint64_t ch = cr.first + wp; ch < cr.end; ch += kRowWarps) {
        const float y = csr_stream32(rp, col, A, ch * 32, n, tiles[wp], [&](uint32_t j) { return __ldg(x + j); });
        const uint64_t I = ch * 32 + lane;
        if (I < n) {
            const float ri = r[I];
            const float z = x[I] + omega * Dinv[I] * (ri - y);
            xo[I] = z;
            acc = fmaf(ri, z, acc);
        }
    }
    if (!with_rz) return;
    const float t[1] = {acc};
    double out[1];
    if (grid_reduce_t<1, 0u>(t, partials, &S->cnt_d, out) && threadIdx.x == 0) {
        if (start) S->beta = beta_den > 0.0 ? out[0] / beta_den : 0.0;
        else S->beta = out[0] / S->rz;
        S->rz = out[0];
        if (!isfinite(out[0])) {
            S->status = LMTG_ERR_NAN;
            S->done = 1;
        }
    }
}

// rc = Q^T res per aggregate (thread per aggregate: its node list in order); with Dc also
// xc = omega_c Dc^-1 rc.  Streaming the lists warp-wide as matrix rows (csr_stream32) took 1.5x
// longer: the gathers of res are what costs, and fewer of them were in flight.
__global__ void k_s_restrict(const uint32_t *__restrict__ aptr, const uint32_t *__restrict__ anode,
                             const float *__restrict__ q, const float *__restrict__ res, float *__restrict__ rc,
                             uint64_t na, const float *__restrict__ Dc, float omega_c, float *__restrict__ xc,
                             const PcgScalars *S) {
    pdl_wait_trigger();
    if (s_done(S)) return;
    for (uint64_t a = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; a < na; a += (uint64_t)gridDim.x * blockDim.x) {
        float v = 0.f;
        for (uint32_t u = aptr[a]; u < aptr[a + 1]; ++u) {
            const uint32_t i = anode[u];
            v = fmaf(q[i], res[i], v);
        }
        rc[a] = v;
        if (Dc) xc[a] = omega_c * Dc[a] * v;
    }
}

// x += q (e + e2)[agg] per node (e2 may be null), four nodes per 16-byte access
__device__ __forceinline__ float s_corr(uint32_t a, float q, const float *e, const float *e2) {
    if (a == kSNone) return 0.f;
    return q * (e2 ? e[a] + e2[a] : e[a]);
}
__global__ void k_s_prolong(const uint32_t *__restrict__ agg, const float *__restrict__ q, const float *__restrict__ e,
                            const float *__restrict__ e2, float *__restrict__ x, uint64_t n, const PcgScalars *S) {
    pdl_wait_trigger();
    if (s_done(S)) return;
    const uint64_t step = (uint64_t)gridDim.x * blockDim.x, i0 = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    const uint64_t n4 = n / 4;
    for (uint64_t g = i0; g < n4; g += step) {
        const uint4 a = reinterpret_cast<const uint4 *>(agg)[g];
        const float4 qq = reinterpret_cast<const float4 *>(q)[g];
        float4 xx = reinterpret_cast<const float4 *>(x)[g];
        xx.x += s_corr(a.x, qq.x, e, e2);
        xx.y += s_corr(a.y, qq.y, e, e2);
        xx.z += s_corr(a.z, qq.z, e, e2);
        xx.w += s_corr(a.w, qq.w, e, e2);
        reinterpret_cast<float4 *>(x)[g] = xx;
    }
    for (uint64_t i = 4 * n4 + i0; i < n; i += step) x[i] += s_corr(agg[i], q[i], e, e2);
}

// The post-smoothing of a level >= 1 with its prolongation fused in: out = x~ + omega D^-1
// (r - A x~), where x~ = x + q (e + e2)[agg] is formed on the fly wherever it is read (the same
// float operations as k_s_prolong, which this replaces there; x itself is not written).  One
// launch fewer per visit of a latency-bound level.
__global__ void __launch_bounds__(kRowThreads)
    k_s_post_pro(const uint32_t *__restrict__ rp, const uint32_t *__restrict__ col, const float *__restrict__ A,
                 const float *__restrict__ Dinv, const float *__restrict__ x, const uint32_t *__restrict__ agg,
                 const float *__restrict__ q, const float *__restrict__ e, const float *__restrict__ e2,
                 const float *__restrict__ r, float *__restrict__ xo, float omega, uint64_t n, const PcgScalars *S) {
    pdl_wait_trigger();
    if (s_done(S)) return;
    __shared__ float tiles[kRowWarps][kTile];
    const int wp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    auto xt = [&](uint32_t j) { return __ldg(x + j) + s_corr(__ldg(agg + j), __ldg(q + j), e, e2); };
    const ChunkRange cr = cta_chunks(n);
    for (uint64_t ch = cr.first + wp; ch < cr.end; ch += kRowWarps) {
        const float y = csr_stream32(rp, col, A, ch * 32, n, tiles[wp], xt);
        const uint64_t I = ch * 32 + lane;
        if (I < n) xo[I] = xt((uint32_t)I) + omega * Dinv[I] * (r[I] - y);
    }
}

// e = Cinv r on the coarsest level (warp per row)
__global__ void k_s_dense(const float *__restrict__ Cinv, const float *__restrict__ r, float *__restrict__ e, int n,
                          const PcgScalars *S) {
    pdl_wait_trigger();
    if (s_done(S)) return;
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; row < n; row += nw) {
        float s = 0.f;
        for (int k = lane; k < n; k += 32) s = fmaf(Cinv[(uint64_t)row * n + k], r[k], s);
        s = warp_sum(s);
        if (lane == 0) e[row] = s;
    }
}

// AMG start / update of the FP32 PCG: the update kernel's x, r and stopping test, and the
// cycle's first smoothing step xa = omega D^-1 r; z, rz and beta come from the cycle
__global__ void k_pcg_start_s_amg(const float *__restrict__ r, const float *__restrict__ b,
                                  const float *__restrict__ Dinv, float *__restrict__ xa, float omega, uint64_t n,
                                  PcgScalars *S, double *partials) {
    float t[2] = {0.f, 0.f};  // rr, bb
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const float ri = r[i];
        xa[i] = omega * Dinv[i] * ri;
        t[0] = fmaf(ri, ri, t[0]);
        if (b) t[1] = fmaf(b[i], b[i], t[1]);
    }
    double out[2];
    if (grid_reduce_t<2, 0u>(t, partials, &S->cnt_c, out) && threadIdx.x == 0) {
        S->rr = out[0];
        if (b) S->bb = out[1];
        S->iter = 0;
        S->status = LMTG_OK;
        S->done = (out[0] <= S->crit * S->crit * S->bb) ? 1 : 0;
        if (!isfinite(out[0])) {
            S->done = 1;
            S->status = LMTG_ERR_NAN;
        }
    }
}

__global__ void k_pcg_update_s_amg(float *__restrict__ x, float *__restrict__ r, const float *__restrict__ p,
                                   const float *__restrict__ q, const float *__restrict__ Dinv, float *__restrict__ xa,
                                   float omega, uint64_t n, PcgScalars *S, double *partials) {
    if (*(volatile int *)&S->done) return;
    const double pq = S->pq;
    const float alpha = (float)S->alpha;
    float t[1] = {0.f};
    const uint64_t i0 = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x, step = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t n4 = n / 4;  // four nodes per 16-byte access, the last n % 4 below
    for (uint64_t g = i0; g < n4; g += step) {
        float4 xv = reinterpret_cast<const float4 *>(x)[g], rv = reinterpret_cast<const float4 *>(r)[g];
        const float4 pv = reinterpret_cast<const float4 *>(p)[g], qv = reinterpret_cast<const float4 *>(q)[g],
                     dv = reinterpret_cast<const float4 *>(Dinv)[g];
        xv = make_float4(fmaf(alpha, pv.x, xv.x), fmaf(alpha, pv.y, xv.y), fmaf(alpha, pv.z, xv.z),
                         fmaf(alpha, pv.w, xv.w));
        rv = make_float4(fmaf(-alpha, qv.x, rv.x), fmaf(-alpha, qv.y, rv.y), fmaf(-alpha, qv.z, rv.z),
                         fmaf(-alpha, qv.w, rv.w));
        reinterpret_cast<float4 *>(x)[g] = xv;
        reinterpret_cast<float4 *>(r)[g] = rv;
        reinterpret_cast<float4 *>(xa)[g] = make_float4(omega * dv.x * rv.x, omega * dv.y * rv.y,
                                                        omega * dv.z * rv.z, omega * dv.w * rv.w);
        t[0] = fmaf(rv.x, rv.x, t[0]);
        t[0] = fmaf(rv.y, rv.y, t[0]);
        t[0] = fmaf(rv.z, rv.z, t[0]);
        t[0] = fmaf(rv.w, rv.w, t[0]);
    }
    for (uint64_t i = 4 * n4 + i0; i < n; i += step) {
        x[i] = fmaf(alpha, p[i], x[i]);
        const float ri = fmaf(-alpha, q[i], r[i]);
        r[i] = ri;
        xa[i] = omega * Dinv[i] * ri;
        t[0] = fmaf(ri, ri, t[0]);
    }
    double out[1];
    if (grid_reduce_t<1, 0u>(t, partials, &S->cnt_b, out) && threadIdx.x == 0) {
        S->iter += 1;
        S->rr = out[0];
        if (!isfinite(out[0]) || !isfinite(pq)) {
            S->status = LMTG_ERR_NAN;
            S->done = 1;
        } else if (out[0] <= S->crit * S->crit * S->bb) {
            S->done = 1;
        } else if (S->iter >= S->maxit) {
            S->status = LMTG_ERR_NOT_CONVERGED;
            S->done = 1;
        }
    }
}

// greedy aggregation of a node graph (rows rp/col), skip[i] = nodes left out; returns aggregates
static uint64_t s_aggregate(uint64_t n, const std::vector<uint32_t> &rp, const std::vector<uint32_t> &col,
                            const std::vector<uint8_t> &skip, std::vector<uint32_t> &agg) {
    agg.assign(n, kSNone);
    std::vector<uint8_t> state(n, 0);  // 0 free, 1 aggregated, 2 skipped
    for (uint64_t i = 0; i < n; ++i)
        if (!skip.empty() && skip[i]) state[i] = 2;
    uint64_t na = 0;
    // pass 1: roots whose free neighbours are all unaggregated take them all
    for (uint64_t i = 0; i < n; ++i) {
        if (state[i] != 0) continue;
        bool ok = true;
        for (uint32_t e = rp[i]; e < rp[i + 1] && ok; ++e) ok = state[col[e]] != 1;
        if (!ok) continue;
        for (uint32_t e = rp[i]; e < rp[i + 1]; ++e) {
            const uint32_t j = col[e];
            if (state[j] == 0) {
                agg[j] = (uint32_t)na;
                state[j] = 1;
            }
        }
        agg[i] = (uint32_t)na;
        state[i] = 1;
        ++na;
    }
    // pass 2: leftovers join the neighbouring aggregate they touch most (the lowest on ties)
    std::vector<uint32_t> cand;
    for (uint64_t i = 0; i < n; ++i) {
        if (state[i] != 0) continue;
        cand.clear();
        for (uint32_t e = rp[i]; e < rp[i + 1]; ++e)
            if (agg[col[e]] != kSNone) cand.push_back(agg[col[e]]);
        if (cand.empty()) continue;
        std::sort(cand.begin(), cand.end());
        uint32_t best = cand[0];
        size_t bc = 0;
        for (size_t k = 0; k < cand.size();) {
            size_t m = k;
            while (m < cand.size() && cand[m] == cand[k]) ++m;
            if (m - k > bc) {
                bc = m - k;
                best = cand[k];
            }
            k = m;
        }
        agg[i] = best;
        state[i] = 1;
    }
    // pass 3: the rest grouped around a free node
    for (uint64_t i = 0; i < n; ++i) {
        if (state[i] != 0) continue;
        for (uint32_t e = rp[i]; e < rp[i + 1]; ++e) {
            const uint32_t j = col[e];
            if (state[j] == 0) {
                agg[j] = (uint32_t)na;
                state[j] = 1;
            }
        }
        agg[i] = (uint32_t)na;
        state[i] = 1;
        ++na;
    }
    return na;
}

template <class T>
static void s_upload(DBuf<T> &d, const std::vector<T> &h, cudaStream_t s) {
    d.alloc(h.size() ? h.size() : 1);
    if (!h.empty()) LMTG_CUDA(cudaMemcpyAsync(d.p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, s));
}

// Hierarchy of the context's scalar matrix: structure (host), then the numeric part (device)
static void samg_build(lmtg_ctx *c) {
    Phase ph("lmtg.diff.amg");
    cudaStream_t s = c->stream;
    std::unique_ptr<SAmg> M(new SAmg());
    // level 0 pattern from the device
    std::vector<uint32_t> rp(c->nn + 1), col;
    LMTG_CUDA(cudaMemcpyAsync(rp.data(), c->bptr.p, 4 * rp.size(), cudaMemcpyDeviceToHost, s));
    LMTG_CUDA(cudaStreamSynchronize(s));
    col.resize(rp.back());
    LMTG_CUDA(cudaMemcpyAsync(col.data(), c->bcol.p, 4 * col.size(), cudaMemcpyDeviceToHost, s));
    LMTG_CUDA(cudaStreamSynchronize(s));
    std::vector<uint8_t> skip(c->nn, 0);
    for (uint32_t d : c->h_cdof)
        if (d < c->nn) skip[d] = 1;
    std::vector<double> B(c->nn, 1.0);
    uint64_t n = c->nn;
    for (int l = 0;; ++l) {
        std::unique_ptr<SLevel> L(new SLevel());
        L->n = n;
        L->nnz = rp.back();
        L->r.alloc(n + 4);
        L->res.alloc(n + 4);
        L->xa.alloc(n + 4);
        L->xb.alloc(n + 4);
        if (l >= 1) {
            L->r2.alloc(n + 4);
            L->xb2.alloc(n + 4);
            s_upload(L->rp, rp, s);
            s_upload(L->col, col, s);
            L->A.alloc(L->nnz);
            L->Dinv.alloc(n);
        }
        const bool coarsest = n <= kSCoarsest || l + 1 >= kSMaxLevels;
        if (coarsest) {
            M->lv.push_back(std::move(L));
            break;
        }
        std::vector<uint32_t> agg;
        const uint64_t na = s_aggregate(n, rp, col, l == 0 ? skip : std::vector<uint8_t>(), agg);
        // aggregate lists, prolongator values, coarse modes
        std::vector<uint32_t> aptr(na + 1, 0), anode;
        for (uint64_t i = 0; i < n; ++i)
            if (agg[i] != kSNone) ++aptr[agg[i] + 1];
        for (uint64_t a = 0; a < na; ++a) aptr[a + 1] += aptr[a];
        anode.resize(aptr[na]);
        {
            std::vector<uint32_t> fill(aptr.begin(), aptr.end() - 1);
            for (uint64_t i = 0; i < n; ++i)
                if (agg[i] != kSNone) anode[fill[agg[i]]++] = (uint32_t)i;
        }
        std::vector<double> Bc(na, 0.0);
        for (uint64_t i = 0; i < n; ++i)
            if (agg[i] != kSNone) Bc[agg[i]] += B[i] * B[i];
        for (auto &v : Bc) v = std::sqrt(v);
        std::vector<float> q(n, 0.f);
        for (uint64_t i = 0; i < n; ++i)
            if (agg[i] != kSNone && Bc[agg[i]] > 0) q[i] = (float)(B[i] / Bc[agg[i]]);
        // coarse pattern: sorted distinct aggregates of each aggregate's nodes' columns
        std::vector<uint32_t> crp(na + 1, 0), ccol;
        bool wide = false;  // a coarse row beyond the Galerkin kernel's kSGalCap slots
        {
            std::vector<uint32_t> mark(na, kSNone), row;
            for (uint64_t a = 0; a < na && !wide; ++a) {
                row.clear();
                for (uint32_t u = aptr[a]; u < aptr[a + 1]; ++u) {
                    const uint32_t i = anode[u];
                    for (uint32_t e = rp[i]; e < rp[i + 1]; ++e) {
                        const uint32_t J = agg[col[e]];
                        if (J != kSNone && mark[J] != a) {
                            mark[J] = (uint32_t)a;
                            row.push_back(J);
                        }
                    }
                }
                std::sort(row.begin(), row.end());
                wide = row.size() > (size_t)kSGalCap;
                ccol.insert(ccol.end(), row.begin(), row.end());
                crp[a + 1] = (uint32_t)ccol.size();
            }
        }
        if (wide) {  // no coarser level: this one is the coarsest (dense if small enough, else Jacobi)
            M->lv.push_back(std::move(L));
            break;
        }
        L->nagg = na;
        s_upload(L->agg, agg, s);
        s_upload(L->aptr, aptr, s);
        s_upload(L->anode, anode, s);
        s_upload(L->q, q, s);
        L->gslot.alloc(L->nnz);
        M->lv.push_back(std::move(L));
        rp.swap(crp);
        col.swap(ccol);
        B.swap(Bc);
        n = na;
    }
    const size_t nl = M->lv.size();
    M->nc = (nl > 1 && M->lv.back()->n <= 2000) ? (int)M->lv.back()->n : 0;
    if (!M->nc) {  // no hierarchy (or a coarsest level too large for the dense solve): Jacobi
        c->samg = M.release();
        return;
    }
    // slots of the fine entries (every level's coarse pattern is uploaded by now)
    for (size_t l = 0; l + 1 < nl; ++l) {
        SLevel &F = *M->lv[l], &C = *M->lv[l + 1];
        k_s_slots<<<grid_for(c, F.n, 128, 8), 128, 0, s>>>(l ? F.rp.p : c->bptr.p, l ? F.col.p : c->bcol.p, F.agg.p,
                                                            F.n, C.rp.p, C.col.p, F.gslot.p);
        LMTG_CUDA(cudaGetLastError());
        c->launches += 1;
    }
    // numeric part: Galerkin products, Jacobi inverses
    for (size_t l = 0; l + 1 < nl; ++l) {
        SLevel &F = *M->lv[l], &C = *M->lv[l + 1];
        k_s_galerkin<<<grid_for(c, F.nagg, kSGalThreads, 8), kSGalThreads, 0, s>>>(
            l ? F.rp.p : c->bptr.p, l ? F.col.p : c->bcol.p, l ? F.A.p : c->K32.p, F.gslot.p, F.q.p, F.aptr.p,
            F.anode.p, F.nagg, C.rp.p, C.col.p, C.A.p);
        k_s_dinv<<<grid_for(c, C.n, 128, 8), 128, 0, s>>>(C.rp.p, C.col.p, C.A.p, C.n, C.Dinv.p);
        LMTG_CUDA(cudaGetLastError());
        c->launches += 2;
    }
    // smoother weights: twelve power steps per level, queued back to back, read once
    M->power.alloc(2 * kSPowerSteps * kSMaxLevels);
    PcgScalars *o = c->scal.p + 1;
    for (size_t l = 0; l + 1 < nl; ++l) {
        SLevel &L = *M->lv[l];
        const uint32_t *lrp = l ? L.rp.p : c->bptr.p, *lcol = l ? L.col.p : c->bcol.p;
        const float *lA = l ? L.A.p : c->K32.p, *lD = l ? L.Dinv.p : c->Dinv32.p;
        k_s_rand<<<grid_for(c, L.n, 256), 256, 0, s>>>(L.xa.p, L.n);
        const int g = grid_for(c, (L.n + 31) / 32 * 32, kRowThreads, 8);
        for (int it = 0; it < kSPowerSteps; ++it) {
            float *v = (it & 1) ? L.xb.p : L.xa.p, *w = (it & 1) ? L.xa.p : L.xb.p;
            double *out = M->power.p + (kSPowerSteps * l + it);
            k_s_power<<<g, kRowThreads, 0, s>>>(lrp, lcol, lA, lD, v, w, L.n, it ? out - 1 : nullptr, c->partials.p,
                                                &o->cnt_c, out);
        }
        LMTG_CUDA(cudaGetLastError());
        c->launches += 1 + kSPowerSteps;
    }
    std::vector<double> h(kSPowerSteps * kSMaxLevels);
    LMTG_CUDA(cudaMemcpyAsync(h.data(), M->power.p, 8 * h.size(), cudaMemcpyDeviceToHost, s));
    // coarsest: dense inverse (FP64 Gauss-Jordan on the host)
    SLevel &Cz = *M->lv.back();
    std::vector<uint32_t> zrp(Cz.n + 1), zcol(Cz.nnz);
    std::vector<float> zA(Cz.nnz);
    LMTG_CUDA(cudaMemcpyAsync(zrp.data(), Cz.rp.p, 4 * zrp.size(), cudaMemcpyDeviceToHost, s));
    LMTG_CUDA(cudaMemcpyAsync(zcol.data(), Cz.col.p, 4 * zcol.size(), cudaMemcpyDeviceToHost, s));
    LMTG_CUDA(cudaMemcpyAsync(zA.data(), Cz.A.p, 4 * zA.size(), cudaMemcpyDeviceToHost, s));
    LMTG_CUDA(cudaStreamSynchronize(s));
    for (size_t l = 0; l + 1 < nl; ++l) {
        SLevel &L = *M->lv[l];
        const double lam = std::sqrt(std::max(0.0, h[kSPowerSteps * l + kSPowerSteps - 1]));
        const double hi = 1.2 * lam, lo = hi / 30.0;
        L.lambda = lam;
        L.omega = lam > 0 ? (float)(2.0 / (hi + lo)) : 1.f;
    }
    const int nc = M->nc;
    std::vector<double> W((size_t)nc * 2 * nc, 0.0);
    const size_t w2 = 2 * (size_t)nc;
    for (int i = 0; i < nc; ++i) {
        for (uint32_t e = zrp[i]; e < zrp[i + 1]; ++e) W[i * w2 + zcol[e]] = zA[e];
        W[i * w2 + nc + i] = 1.0;
    }
    double dmax = 0;
    for (int i = 0; i < nc; ++i) dmax = std::max(dmax, std::fabs(W[i * w2 + i]));
    std::vector<char> dead(nc, 0);
    for (int cc = 0; cc < nc; ++cc) {
        int p = cc;
        for (int r = cc + 1; r < nc; ++r)
            if (std::fabs(W[r * w2 + cc]) > std::fabs(W[p * w2 + cc])) p = r;
        if (std::fabs(W[p * w2 + cc]) <= 1e-13 * dmax) {
            dead[cc] = 1;
            continue;
        }
        if (p != cc)
            for (size_t k = 0; k < w2; ++k) std::swap(W[cc * w2 + k], W[p * w2 + k]);
        const double iv = 1.0 / W[cc * w2 + cc];
        for (size_t k = 0; k < w2; ++k) W[cc * w2 + k] *= iv;
        for (int r = 0; r < nc; ++r) {
            if (r == cc) continue;
            const double f = W[r * w2 + cc];
            if (f == 0.0) continue;
            for (size_t k = cc; k < w2; ++k) W[r * w2 + k] -= f * W[cc * w2 + k];
        }
    }
    std::vector<float> Ci((size_t)nc * nc);
    for (int r = 0; r < nc; ++r)
        for (int k = 0; k < nc; ++k) Ci[(size_t)r * nc + k] = (dead[r] || dead[k]) ? 0.f : (float)W[r * w2 + nc + k];
    M->Cinv.alloc(Ci.size());
    LMTG_CUDA(cudaMemcpyAsync(M->Cinv.p, Ci.data(), 4 * Ci.size(), cudaMemcpyHostToDevice, s));
    LMTG_CUDA(cudaStreamSynchronize(s));
    c->samg = M.release();
}

// the multigrid for this context's FP32 diffusion solves, built on first use; false: Jacobi
static bool samg_prepare(lmtg_ctx *c) {
    if (c->precond != LMTG_PREC_AMG || c->nn < kSMinUnknowns) return false;
    if (!c->samg) samg_build(c);
    return c->samg && c->samg->nc > 0;
}

static void s_cycle(lmtg_ctx *c, SAmg &M, size_t l, const float *rhs, float *out, cudaStream_t s, PcgScalars *S);

// level l's coarse correction: level l+1's cycle on N.r (its first smoothing step in N.xa) --
// once on the dense coarsest (e = N.res) and below the top kSWLevels levels (e = N.xb), else
// twice, the second visit on the residual the first leaves (e = N.xb, e2 = N.xb2)
static void s_correction(lmtg_ctx *c, SAmg &M, size_t l, cudaStream_t s, PcgScalars *S, float *&e, float *&e2) {
    const size_t nl = M.lv.size();
    SLevel &N = *M.lv[l + 1];
    e2 = nullptr;
    if (l + 2 == nl) {
        e = N.res.p;
        s_cycle(c, M, l + 1, N.r.p, e, s, S);
        return;
    }
    e = N.xb.p;
    s_cycle(c, M, l + 1, N.r.p, e, s, S);
    if (l >= kSWLevels) return;
    e2 = N.xb2.p;
    launch_pdl(k_s_res, grid_for(c, (N.n + 31) / 32 * 32, kRowThreads, 8), kRowThreads, 0, s, N.rp.p, N.col.p,
               N.A.p, e, N.r.p, N.r2.p, N.n, S, N.Dinv.p, N.omega, N.xa.p);
    c->launches += 1;
    s_cycle(c, M, l + 1, N.r2.p, e2, s, S);
}

// the restriction to level l+1 (with its first smoothing step unless it is the dense coarsest)
// and the prolongation back, shared by the level-0 and deeper cycles
static void s_restrict(lmtg_ctx *c, SAmg &M, size_t l, cudaStream_t s, PcgScalars *S) {
    SLevel &L = *M.lv[l], &N = *M.lv[l + 1];
    const bool ncoarsest = l + 2 == M.lv.size();
    launch_pdl(k_s_restrict, grid_for(c, L.nagg, 256, 8), 256, 0, s, L.aptr.p, L.anode.p, L.q.p, L.res.p, N.r.p,
               L.nagg, ncoarsest ? nullptr : N.Dinv.p, N.omega, N.xa.p, S);
}
static void s_prolong(lmtg_ctx *c, SLevel &L, const float *e, const float *e2, cudaStream_t s, PcgScalars *S) {
    launch_pdl(k_s_prolong, grid_for(c, L.n / 4 + 1, 256, 8), 256, 0, s, L.agg.p, L.q.p, e, e2, L.xa.p, L.n, S);
}

// cycle of level l >= 1 on rhs (first smoothing step already in L.xa) into out
static void s_cycle(lmtg_ctx *c, SAmg &M, size_t l, const float *rhs, float *out, cudaStream_t s, PcgScalars *S) {
    SLevel &L = *M.lv[l];
    if (l + 1 == M.lv.size()) {
        launch_pdl(k_s_dense, grid_for(c, (uint64_t)M.nc * 32, 256, 4), 256, 0, s, M.Cinv.p, rhs, out, M.nc, S);
        c->launches += 1;
        return;
    }
    const int g = grid_for(c, (L.n + 31) / 32 * 32, kRowThreads, 8);
    launch_pdl(k_s_res, g, kRowThreads, 0, s, L.rp.p, L.col.p, L.A.p, L.xa.p, rhs, L.res.p, L.n, S, nullptr, 0.f,
               nullptr);
    s_restrict(c, M, l, s, S);
    float *e, *e2;
    s_correction(c, M, l, s, S, e, e2);
    launch_pdl(k_s_post_pro, g, kRowThreads, 0, s, L.rp.p, L.col.p, L.A.p, L.Dinv.p, L.xa.p, L.agg.p, L.q.p, e, e2,
               rhs, out, L.omega, L.n, S);
    c->launches += 3;
}

// the cycle after the update kernel (level 0): r -> z, rz and beta; the residual and the
// post-smoothing stream K32 by bulk copies when the PCG's SpMV does (sbulk)
static void s_cycle0(lmtg_ctx *c, const float *r, float *z, cudaStream_t s, int start, double beta_den, bool sbulk) {
    SAmg &M = *c->samg;
    PcgScalars *S = c->scal.p;
    SLevel &L = *M.lv[0];
    const int g = grid_for(c, (L.n + 31) / 32 * 32, kRowThreads, 8);
    if (sbulk)
        sbulk_launch(c, c->K32.p, EpiSRes{L.xa.p, r, L.res.p}, s);
    else
        launch_pdl(k_s_res, g, kRowThreads, 0, s, c->bptr.p, c->bcol.p, c->K32.p, L.xa.p, r, L.res.p, L.n, S,
                   nullptr, 0.f, nullptr);
    s_restrict(c, M, 0, s, S);
    float *e, *e2;
    s_correction(c, M, 0, s, S, e, e2);
    s_prolong(c, L, e, e2, s, S);
    if (sbulk)
        sbulk_launch(c, c->K32.p, EpiSPost{L.xa.p, r, c->Dinv32.p, z, L.omega, start, beta_den}, s);
    else
        launch_pdl(k_s_post, g, kRowThreads, 0, s, c->bptr.p, c->bcol.p, c->K32.p, c->Dinv32.p, L.xa.p, r, z,
                   L.omega, L.n, S, true, start, beta_den, c->partials.p);
    c->launches += 4;
    LMTG_CUDA(cudaGetLastError());
}

// PCG on K x = b in precision T, from the current x (x_zero: x is 0, r = b), preconditioned by
// Jacobi, or for FP32 with amg by the context's multigrid (K = K32).  b_norm2 >= 0 gives |b|^2 for
// the relative test; beta_den > 0 continues the search direction held in p (reliable update).
// Returns the status; *iters the iterations.
template <class T>
static int diff_pcg_t(lmtg_ctx *c, const T *K, const T *Dinv, const T *b, T *x, T *r, T *z, T *p, T *q,
                      bool x_zero, double tol, int maxit, double b_norm2, double beta_den, int *iters,
                      bool amg = false) {
    cudaStream_t s = c->stream;
    // FP32: the bulk-copy SpMV unless spmv_kind 0 or a 32-row chunk could exceed a stage
    const bool sbulk = std::is_same<T, float>::value && c->spmv_kind != 0 &&
                       32ull * c->max_row_blocks <= (uint64_t)kSCap;
    PcgScalars init{};
    init.crit = tol;
    init.crit_kind = LMTG_CRIT_REL_RESIDUAL;
    init.maxit = maxit;
    init.bb = b_norm2 >= 0 ? b_norm2 : 0.0;
    LMTG_CUDA(cudaMemcpyAsync(c->scal.p, &init, sizeof(init), cudaMemcpyHostToDevice, s));
    PcgScalars *o = c->scal.p + 1;
    if (x_zero) {
        LMTG_CUDA(cudaMemcpyAsync(r, b, sizeof(T) * c->nn, cudaMemcpyDeviceToDevice, s));
    } else {
        k_residual_s<T><<<rgrid(c, k_residual_s<T>), kRowThreads, 0, s>>>(c->bptr.p, c->bcol.p, K, x, b, r,
                                                                          c->nn, c->partials.p, &o->cnt_c,
                                                                          &o->rr);
        c->launches += 1;
    }
    if constexpr (std::is_same<T, float>::value) {
        if (amg) {
            SLevel &L0 = *c->samg->lv[0];
            k_pcg_start_s_amg<<<ngrid(c), kRowThreads, 0, s>>>(r, b_norm2 >= 0 ? nullptr : b, c->Dinv32.p,
                                                               L0.xa.p, L0.omega, c->nn, c->scal.p,
                                                               c->partials.p);
            c->launches += 1;
            s_cycle0(c, r, z, s, 1, beta_den, sbulk);  // z, rz and beta = rz / beta_den (0 on a fresh start)
        }
    }
    if (!amg) {
        k_pcg_start_s<T><<<ngrid(c), kRowThreads, 0, s>>>(r, b_norm2 >= 0 ? nullptr : b, Dinv, z, c->nn,
                                                          c->scal.p, c->partials.p);
        c->launches += 1;
    }
    LMTG_CUDA(cudaGetLastError());
    if (beta_den > 0.0 && !amg) {
        // continue the previous direction: beta = rz_new / beta_den (set after the start kernel)
        PcgScalars h{};
        LMTG_CUDA(cudaMemcpyAsync(&h, c->scal.p, sizeof(h), cudaMemcpyDeviceToHost, s));
        LMTG_CUDA(cudaStreamSynchronize(s));
        const double beta = h.rz / beta_den;
        LMTG_CUDA(cudaMemcpyAsync(&c->scal.p->beta, &beta, sizeof(double), cudaMemcpyHostToDevice, s));
        LMTG_CUDA(cudaStreamSynchronize(s));
    }
    // iterations per graph launch (a multigrid iteration is ~40 launches: fewer run on after the
    // convergence test stops the chunk)
    const int kIters = amg ? 4 : 16;
    const int gr = rgrid(c, k_pcg_spmv_s<T>);
    if (sbulk) {  // the functions' attributes and grids, set before any capture
        if (c->col16) {
            sbulk_grid<EpiSPq, int16_t>(c);
            sbulk_grid<EpiSRes, int16_t>(c);
            sbulk_grid<EpiSPost, int16_t>(c);
        } else {
            sbulk_grid<EpiSPq, uint32_t>(c);
            sbulk_grid<EpiSRes, uint32_t>(c);
            sbulk_grid<EpiSPost, uint32_t>(c);
        }
    }
    // the chunk graph of this precision, reused while it was captured on the same buffers
    DiffGraph &dg = c->diff_graph[std::is_same<T, float>::value ? 1 : 0];
    const void *key[10] = {K, Dinv, b, x, r, z, p, q, reinterpret_cast<const void *>((uintptr_t)sbulk + 2 * c->col16),
                           reinterpret_cast<const void *>((uintptr_t)amg)};
    bool cached = dg.exec != nullptr;
    for (int i = 0; i < 10 && cached; ++i) cached = dg.key[i] == key[i];
    if (!cached) {
        if (dg.exec) cudaGraphExecDestroy(dg.exec);
        if (dg.graph) cudaGraphDestroy(dg.graph);
        dg.exec = nullptr;
        dg.graph = nullptr;
    }
    cudaGraph_t graph = dg.graph;
    cudaGraphExec_t exec = dg.exec;
    if (!cached) {
        const uint64_t launches0 = c->launches;
        LMTG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        for (int k = 0; k < kIters; ++k) {
            k_pcg_dir_s<T><<<ngrid(c), kRowThreads, 0, s>>>(z, p, c->nn, c->scal.p);
            if constexpr (std::is_same<T, float>::value) {
                if (sbulk)
                    sbulk_launch(c, K, EpiSPq{p, q}, s);
                else
                    k_pcg_spmv_s<T><<<gr, kRowThreads, 0, s>>>(c->bptr.p, c->bcol.p, K, p, q, c->nn, c->scal.p,
                                                               c->partials.p);
            } else {
                k_pcg_spmv_s<T><<<gr, kRowThreads, 0, s>>>(c->bptr.p, c->bcol.p, K, p, q, c->nn, c->scal.p,
                                                           c->partials.p);
            }
            if constexpr (std::is_same<T, float>::value) {
                if (amg) {
                    SLevel &L0 = *c->samg->lv[0];
                    k_pcg_update_s_amg<<<ngrid(c), kRowThreads, 0, s>>>(x, r, p, q, c->Dinv32.p, L0.xa.p,
                                                                        L0.omega, c->nn, c->scal.p,
                                                                        c->partials.p);
                    s_cycle0(c, r, z, s, 0, 0.0, sbulk);
                }
            }
            if (!amg)
                k_pcg_update_s<T><<<ngrid(c), kRowThreads, 0, s>>>(x, r, z, p, q, Dinv, c->nn, c->scal.p,
                                                                   c->partials.p);
            c->launches += 3;
        }
        cudaError_t ce = cudaStreamEndCapture(s, &graph);
        if (ce != cudaSuccess) throw Error{LMTG_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ce)};
        ce = cudaGraphInstantiate(&exec, graph, 0);
        if (ce != cudaSuccess) {
            cudaGraphDestroy(graph);
            throw Error{LMTG_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ce)};
        }
        dg.graph = graph;
        dg.exec = exec;
        for (int i = 0; i < 10; ++i) dg.key[i] = key[i];
        dg.launches = c->launches - launches0;  // counted while capturing, run on each replay
        c->launches = launches0;
    }
    cudaError_t ce = cudaSuccess;
    LMTG_CUDA(cudaMemcpyAsync(c->h_scal, c->scal.p, sizeof(PcgScalars), cudaMemcpyDeviceToHost, s));
    LMTG_CUDA(cudaStreamSynchronize(s));
    bool finished = c->h_scal[0].done != 0;
    const int max_chunks = maxit / kIters + 2;
    for (int ch = 0; ch < max_chunks && !finished; ++ch) {
        ce = cudaGraphLaunch(exec, s);
        c->launches += dg.launches;
        if (ce == cudaSuccess)
            ce = cudaMemcpyAsync(c->h_scal, c->scal.p, sizeof(PcgScalars), cudaMemcpyDeviceToHost, s);
        if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
        if (ce != cudaSuccess) {
            diff_graphs_free(c);
            throw Error{LMTG_ERR_CUDA, std::string("pcg chunk: ") + cudaGetErrorString(ce)};
        }
        finished = c->h_scal[0].done != 0;
    }
    *iters = c->h_scal[0].iter;
    return finished ? c->h_scal[0].status : LMTG_ERR_NOT_CONVERGED;
}

void diff_graphs_free(lmtg_ctx *c) {
    for (DiffGraph &dg : c->diff_graph) {
        if (dg.exec) cudaGraphExecDestroy(dg.exec);
        if (dg.graph) cudaGraphDestroy(dg.graph);
        dg = DiffGraph{};
    }
}

static int diff_pcg64(lmtg_ctx *c, const double *b, double *x, double tol, int maxit, int *iters) {
    return diff_pcg_t<double>(c, c->K64.p, c->Dinv64.p, b, x, c->w64[0].p, c->w64[1].p, c->w64[2].p,
                              c->w64[3].p, false, tol, maxit, -1.0, 0.0, iters);
}

// Refinement residual in float-float: r = b - A x with A, x, b in FP64, each operand split into
// two floats on the integer pipe, the products formed exactly (FMA two-product of the splits)
// and summed per row in a compensated sum (Ogita, Rump and Oishi's Dot2), 48 significant bits;
// written as rs r in float, |rs r|^2 reduced.  The layout is csr_stream32's: lane l takes the
// tile's entries t0 + 32k + l, the product pairs go to per-warp shared tiles, and each lane sums
// its own row in column order.  The FP64 kernel k_residual_s<double> spends 0.53 ms at 2 x
// 1024^2 on FP64 multiplies and adds (2 lanes per clock per SM); this one runs on the FP32 and
// integer pipes.
__global__ void __launch_bounds__(kRowThreads)
    k_residual_s_ff(const uint32_t *__restrict__ rp, const uint32_t *__restrict__ col, const double *__restrict__ K,
                    const double *__restrict__ x, const double *__restrict__ b, float rs, float *__restrict__ r32,
                    uint64_t n, double *partials, unsigned *ticket, double *rr_out) {
    __shared__ float th[kRowWarps][kTile], tl[kRowWarps][kTile];
    const int wp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float acc = 0.f;
    const ChunkRange cr = cta_chunks(n);
    for (uint64_t ch = cr.first + wp; ch < cr.end; ch += kRowWarps) {
        const uint64_t r0 = ch * 32, I = r0 + lane;
        const uint32_t rs0 = __ldg(rp + (I < n ? I : n));
        uint32_t re0 = __shfl_down_sync(0xffffffffu, rs0, 1);
        if (lane == 31) re0 = __ldg(rp + (r0 + 32 < n ? r0 + 32 : n));
        const uint32_t e0 = __shfl_sync(0xffffffffu, rs0, 0);
        const uint32_t e1 = __shfl_sync(0xffffffffu, re0, 31);
        float sh = 0.f, sc = 0.f;  // the row's Dot2 sum and its compensation
        for (uint32_t t0 = e0; t0 < e1; t0 += kTile) {
            const uint32_t nck = (e1 - t0 + 31) / 32;
            uint32_t cj[kTileChunks];
            double kv[kTileChunks];
#pragma unroll
            for (int k = 0; k < kTileChunks; ++k) {
                if (k < nck) {
                    const uint32_t q = t0 + 32 * k + lane;
                    const bool on = q < e1;
                    cj[k] = on ? __ldcs(col + q) : 0u;
                    kv[k] = on ? __ldcs(K + q) : 0.0;
                }
            }
            double xv[kTileChunks];
#pragma unroll
            for (int k = 0; k < kTileChunks; ++k)
                if (k < nck) xv[k] = t0 + 32 * k + lane < e1 ? __ldg(x + cj[k]) : 0.0;
#pragma unroll
            for (int k = 0; k < kTileChunks; ++k) {
                if (k < nck) {
                    const ff::f2 a = ff::split(kv[k]), v = ff::split(xv[k]);
                    const float p = a.h * v.h;
                    float pl = fmaf(a.h, v.h, -p);
                    pl = fmaf(a.h, v.l, pl);
                    pl = fmaf(a.l, v.h, pl);
                    th[wp][32 * k + lane] = p;
                    tl[wp][32 * k + lane] = pl;
                }
            }
            __syncwarp();
            const uint32_t lo = rs0 > t0 ? rs0 : t0;
            const uint32_t hi = re0 < t0 + kTile ? re0 : t0 + kTile;
            for (uint32_t q = lo; q < hi; ++q) {
                float e;
                ff::two_sum(sh, th[wp][q - t0], sh, e);
                sc += e + tl[wp][q - t0];
            }
            __syncwarp();
        }
        if (I < n) {
            const ff::f2 r = ff::add(ff::split(b[I]), ff::neg(ff::renorm(sh, sc)));
            const float rf = (r.h + r.l) * rs;
            r32[I] = rf;
            acc = fmaf(rf, rf, acc);
        }
    }
    const float t[1] = {acc};
    double out[1];
    if (grid_reduce_t<1, 0u>(t, partials, ticket, out) && threadIdx.x == 0) *rr_out = out[0];
}

__global__ void k_scale_s32(float *__restrict__ v, float f, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        v[i] *= f;
}

// b32 = r / |r| for r = b - A x (A = K64), returns |r|^2: in float-float (ff) or in FP64 (r64)
static double diff_refinement_residual(lmtg_ctx *c, const double *x, const double *b, double bb, float *b32,
                                       double *r64, bool ff) {
    cudaStream_t st = c->stream;
    PcgScalars *o = c->scal.p + 1;
    double rr = 0;
    if (!ff) {
        k_residual_s<double><<<rgrid(c, k_residual_s<double>), kRowThreads, 0, st>>>(
            c->bptr.p, c->bcol.p, c->K64.p, x, b, r64, c->nn, c->partials.p, &o->cnt_c, &o->rr);
        LMTG_CUDA(cudaMemcpyAsync(&rr, &o->rr, 8, cudaMemcpyDeviceToHost, st));
        LMTG_CUDA(cudaStreamSynchronize(st));
        if (rr > 0 && std::isfinite(rr)) {
            k_scale_to32<<<ngrid(c), kRowThreads, 0, st>>>(r64, 1.0 / std::sqrt(rr), b32, c->nn);
            c->launches += 1;
        }
        c->launches += 1;
        return rr;
    }
    // a power of two near 1 / rms(b) keeps the squares of small residuals in the float range
    const double rms = std::sqrt(bb / (double)(c->nn ? c->nn : 1));
    const int e = (rms > 0 && std::isfinite(rms)) ? std::max(-100, std::min(100, std::ilogb(rms))) : 0;
    k_residual_s_ff<<<rgrid(c, k_residual_s_ff), kRowThreads, 0, st>>>(c->bptr.p, c->bcol.p, c->K64.p, x, b,
                                                                        std::ldexp(1.0f, -e), b32, c->nn,
                                                                        c->partials.p, &o->cnt_c, &o->rr);
    LMTG_CUDA(cudaMemcpyAsync(&rr, &o->rr, 8, cudaMemcpyDeviceToHost, st));
    LMTG_CUDA(cudaStreamSynchronize(st));
    c->launches += 1;
    if (rr > 0 && std::isfinite(rr)) {
        k_scale_s32<<<ngrid(c), kRowThreads, 0, st>>>(b32, (float)(1.0 / std::sqrt(rr)), c->nn);
        c->launches += 1;
    }
    return rr * std::ldexp(1.0, 2 * e);
}

// FP32-inner / FP64-refined solve of A x = b with reliable updates (the elasticity solver's
// scheme on the scalar matrices): FP32 PCG segments (multigrid or Jacobi) on A32 d = r / s, each ending after a
// reduction of its recursive residual by inner_reduction; x += s d and r = b - A x in FP64; the search
// direction is kept across the residual replacement.
static int diff_mixed(lmtg_ctx *c, const double *b, double *x, double tol, int maxit, int *iters) {
    cudaStream_t st = c->stream;
    double *r64 = c->w64[0].p;
    float *b32 = c->w32[0].p, *d32 = c->w32[1].p, *r32 = c->w32[2].p, *z32 = c->w32[3].p,
          *p32 = c->w32[4].p, *q32 = c->w32[5].p;
    PcgScalars *o = c->scal.p + 1;
    auto read_rr = [&]() {
        double v = 0;
        LMTG_CUDA(cudaMemcpyAsync(&v, &o->rr, 8, cudaMemcpyDeviceToHost, st));
        LMTG_CUDA(cudaStreamSynchronize(st));
        return v;
    };
    k_dot_s<<<ngrid(c), kRowThreads, 0, st>>>(b, b, c->nn, c->partials.p, &o->cnt_c, &o->rr);
    c->launches += 1;
    const double bb = read_rr();
    const bool amg = samg_prepare(c);
    const double kDelta = c->inner_reduction;
    int total = 0, status = LMTG_OK, outer = 0;
    double s_prev = 0, rz_prev = 0, rel_prev = 0;
    bool have_dir = false;
    // Float-float residuals while the residual is above kFFMinRel of |b| (their rounding stays
    // orders below it); below, to decide convergence, or when a float-float residual shows no
    // progress, the FP64 residual takes over for the rest of the solve (the elasticity solver's
    // rule)
    constexpr double kFFMinRel = 1e-9;
    bool ff = true;
    for (;;) {
        double rr = diff_refinement_residual(c, x, b, bb, b32, r64, ff);  // b32 = r / |r|
        double rel = bb > 0 ? std::sqrt(rr / bb) : std::sqrt(rr);
        if (ff && (!std::isfinite(rel) || rel <= tol || rel < kFFMinRel || rr == 0.0 ||
                   (outer > 0 && rel > 0.5 * rel_prev))) {
            ff = false;
            rr = diff_refinement_residual(c, x, b, bb, b32, r64, false);
            rel = bb > 0 ? std::sqrt(rr / bb) : std::sqrt(rr);
        }
        if (!std::isfinite(rel)) { status = LMTG_ERR_NAN; break; }
        if (rel <= tol || rr == 0.0) break;
        if (total >= maxit || outer >= 400) { status = LMTG_ERR_NOT_CONVERGED; break; }
        if (have_dir && rel > 0.5 * rel_prev) have_dir = false;
        const double sc = std::sqrt(rr);
        LMTG_CUDA(cudaMemsetAsync(d32, 0, sizeof(float) * c->nn, st));
        const double beta_den = have_dir ? rz_prev * (s_prev / sc) : 0.0;
        double eta = 0.5 * tol / rel;
        if (eta < kDelta) eta = kDelta;
        int it = 0;
        const int s2 = diff_pcg_t<float>(c, c->K32.p, c->Dinv32.p, b32, d32, r32, z32, p32, q32, true,
                                         eta, maxit - total, 1.0, beta_den, &it, amg);
        total += it;
        ++outer;
        if (s2 == LMTG_ERR_NAN) { status = s2; break; }
        // r.z of the last direction: the multigrid's cycle is skipped once the update kernel
        // stops the run, so rz is still that one; the Jacobi update forms the next rz and beta
        if (amg) rz_prev = c->h_scal[0].rz;
        else rz_prev = c->h_scal[0].beta != 0.0 ? c->h_scal[0].rz / c->h_scal[0].beta : 0.0;
        s_prev = sc;
        rel_prev = rel;
        have_dir = it > 0 && rz_prev > 0.0;
        k_axpy_64_32<<<ngrid(c), kRowThreads, 0, st>>>(x, sc, d32, c->nn);
        LMTG_CUDA(cudaGetLastError());
        c->launches += 1;
    }
    *iters = total;
    return status;
}

static int diff_pcg(lmtg_ctx *c, const double *b, double *x, double tol, int maxit, int *iters) {
    return c->diff_mode == LMTG_SOLVE_MIXED_IR ? diff_mixed(c, b, x, tol, maxit, iters)
                                               : diff_pcg64(c, b, x, tol, maxit, iters);
}

// rhs = B T (FP64)
static void diff_rhs(lmtg_ctx *c, const double *T, double *rhs) {
    k_spmv_s<double><<<rgrid(c, k_spmv_s<double>), kRowThreads, 0, c->stream>>>(c->bptr.p, c->bcol.p, c->B64.p, T, rhs,
                                                              c->nn);
    LMTG_CUDA(cudaGetLastError());
    c->launches += 1;
}

__global__ void k_add_vec(double *__restrict__ y, const double *__restrict__ a, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        y[i] += a[i];
}

// one step T_next = A^-1 (B T + s) (warm start from T); s = the constant source and convection
// loads (lmtg_diff_set_sources / lmtg_diff_set_convection)
static int diff_step(lmtg_ctx *c, const double *T, double *Tn, double tol, int maxit, int *it) {
    Phase ph("lmtg.diff.step");
    diff_rhs(c, T, c->F.p);
    if (c->diff_load.p) {
        k_add_vec<<<ngrid(c), kRowThreads, 0, c->stream>>>(c->F.p, c->diff_load.p, c->nn);
        c->launches += 1;
    }
    if (Tn != T)
        LMTG_CUDA(cudaMemcpyAsync(Tn, T, sizeof(double) * c->nn, cudaMemcpyDeviceToDevice, c->stream));
    return diff_pcg(c, c->F.p, Tn, tol, maxit, it);
}

void diff_setup(lmtg_ctx *c, const double *k, uint64_t nk, double rho_c, double dt, double theta,
                uint64_t nbnd, const uint32_t *bnd, double penalty) {
    LMTG_CHECK(c->elem_type == LMTG_ELEM_TRIANGLE6, LMTG_ERR_STATE, "diffusion needs a Triangle_6 mesh");
    LMTG_CHECK(nk == 1 || nk == c->ne, LMTG_ERR_ARG, "conductivity needs 1 or ne values");
    LMTG_CHECK(rho_c > 0 && dt > 0 && theta >= 0 && theta <= 1, LMTG_ERR_ARG, "rho_c, dt > 0, theta in [0,1]");
    c->h_diff_conv.clear();  // the matrices are rebuilt: convection has to be set again
    samg_free(c);            // and the multigrid with them, at the next FP32 solve
    cudaStream_t s = c->stream;
    if (!c->allocated) {
        build_pattern(c);
        c->nnz_lower = (c->nnzb - c->nn) / 2 + c->nn;
        c->K64.alloc(c->nnzb);
        c->B64.alloc(c->nnzb);
        c->K32.alloc(c->nnzb + 4);  // 16 bytes of slack: bulk copies round their end up
        c->Ke64.alloc(c->ne * kTriPairs);
        c->KeB64.alloc(c->ne * kTriPairs);
        c->F.alloc(c->nn);
        c->u.alloc(c->nn);
        c->Dinv64.alloc(c->nn);
        c->Dinv32.alloc(c->nn);
        for (auto &w : c->w64) w.alloc(c->nn);
        for (auto &w : c->w32) w.alloc(c->nn);
        LMTG_CUDA(cudaMemsetAsync(c->u.p, 0, c->u.bytes(), s));
        // 16-bit column deltas for the bulk-copy products when the numbering is banded enough
        c->bcol16.alloc(c->nnzb + 8);  // 16 bytes of slack: bulk copies round their end up
        DBuf<int> over;
        over.alloc(1);
        LMTG_CUDA(cudaMemsetAsync(over.p, 0, sizeof(int), s));
        k_col16<<<grid_for(c, c->nn, 256, 8), 256, 0, s>>>(c->bptr.p, c->bcol.p, c->nn, c->bcol16.p, over.p);
        LMTG_CUDA(cudaGetLastError());
        c->launches += 1;
        int h_over = 1;
        LMTG_CUDA(cudaMemcpyAsync(&h_over, over.p, sizeof(int), cudaMemcpyDeviceToHost, s));
        LMTG_CUDA(cudaStreamSynchronize(s));
        c->col16 = h_over == 0;
        if (!c->col16) c->bcol16.release();
        c->allocated = true;
    }
    c->E.alloc(nk);
    LMTG_CUDA(cudaMemcpyAsync(c->E.p, k, nk * 8, cudaMemcpyHostToDevice, s));
    c->E_per_elem = nk > 1;
    c->rho_c = rho_c;
    c->dt = dt;
    c->theta = theta;
    k_tri6_diff<<<grid_for(c, c->ne, 128, 16), 128, 0, s>>>(c->pos.p, c->conn.p, c->E.p, c->E_per_elem,
                                                            1.0 / rho_c, dt, theta, c->ne, c->Ke64.p,
                                                            c->KeB64.p);
    k_assemble_s<<<grid_for(c, c->nnzb, 256, 8), 256, 0, s>>>(c->gptr.p, c->gsrc.p, c->Ke64.p,
                                                              c->KeB64.p, c->nnzb, c->K64.p, c->B64.p,
                                                              c->K32.p);
    LMTG_CUDA(cudaGetLastError());
    c->launches += 2;
    c->h_cdof.assign(bnd, bnd + nbnd);  // penalty nodes stay out of the multigrid's aggregates
    if (nbnd) {
        upload_u32(c, c->cdof, bnd, nbnd);
        DBuf<unsigned long long> md;
        md.alloc(1);
        if (c->penalty_scale > 0.0) {
            unsigned long long bits;
            memcpy(&bits, &c->penalty_scale, sizeof(bits));
            LMTG_CUDA(cudaMemcpyAsync(md.p, &bits, sizeof(bits), cudaMemcpyHostToDevice, s));
        } else {
            LMTG_CUDA(cudaMemsetAsync(md.p, 0, 8, s));
            k_max_diag_s<<<grid_for(c, c->nn, 256), 256, 0, s>>>(c->bdiag.p, c->K64.p, c->nn, md.p);
            c->launches += 1;
        }
        k_penalty_s<<<grid_for(c, nbnd, 256), 256, 0, s>>>(c->bdiag.p, c->K64.p, c->K32.p, c->cdof.p,
                                                          nbnd, penalty, md.p);
        c->launches += 1;
        unsigned long long bits = 0;
        LMTG_CUDA(cudaMemcpyAsync(&bits, md.p, 8, cudaMemcpyDeviceToHost, s));
        LMTG_CUDA(cudaStreamSynchronize(s));
        memcpy(&c->max_diag, &bits, 8);
    }
    k_jacobi_s<double><<<grid_for(c, c->nn, 256), 256, 0, s>>>(c->bdiag.p, c->K64.p, c->nn, c->Dinv64.p,
                                                               c->K32.p);
    k_jacobi_s<float><<<grid_for(c, c->nn, 256), 256, 0, s>>>(c->bdiag.p, c->K64.p, c->nn, c->Dinv32.p,
                                                              nullptr);
    LMTG_CUDA(cudaGetLastError());
    c->launches += 2;
    LMTG_CUDA(cudaStreamSynchronize(s));
    c->have64 = true;
}

// pos += val at the given entries of A (K64 and its FP32 copy) and pos -= val_b of B
__global__ void k_add_entries(const uint64_t *__restrict__ at, const double *__restrict__ va,
                              const double *__restrict__ vb, uint64_t m, double *A, float *A32, double *B) {
    for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < m; k += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t q = at[k];
        A[q] += va[k];
        A32[q] = (float)A[q];
        B[q] += vb[k];
    }
}

// the constant loads of every step: source + convection parts
static void diff_update_load(lmtg_ctx *c) {
    const uint64_t nn = c->nn;
    const bool any = !c->h_diff_src.empty() || !c->h_diff_conv.empty();
    if (!any) {
        c->diff_load.release();
        return;
    }
    std::vector<double> v(nn, 0.0);
    for (uint64_t i = 0; i < nn && !c->h_diff_src.empty(); ++i) v[i] += c->h_diff_src[i];
    for (uint64_t i = 0; i < nn && !c->h_diff_conv.empty(); ++i) v[i] += c->h_diff_conv[i];
    upload_u32(c, c->diff_load, v.data(), nn);
    LMTG_CUDA(cudaStreamSynchronize(c->stream));
}

// s = M Q + Qs: the volume source Q (nodal, -Q te dV) and the nodal source Qs (-Qs te dN) of
// formulations/formulation_difftherm.py:26-29, M the consistent mass matrix
void diff_set_sources(lmtg_ctx *c, const double *Q, const double *Qs) {
    LMTG_CHECK(c->allocated && c->elem_type == LMTG_ELEM_TRIANGLE6, LMTG_ERR_STATE, "diff_setup first");
    cudaStream_t s = c->stream;
    const uint64_t nn = c->nn;
    std::vector<double> src(nn, 0.0);
    if (Q) {
        DBuf<double> M1, M2, Mv, Bv, q, mq;
        DBuf<float> M32;
        M1.alloc(c->ne * kTriPairs);
        M2.alloc(c->ne * kTriPairs);
        Mv.alloc(c->nnzb);
        Bv.alloc(c->nnzb);
        M32.alloc(c->nnzb);
        q.alloc(nn);
        mq.alloc(nn);
        const double one = 1.0;
        DBuf<double> a1;
        upload_u32(c, a1, &one, 1);
        // conduction 0, dt 1: the element kernel's A part is the mass matrix
        k_tri6_diff<<<grid_for(c, c->ne, 128, 16), 128, 0, s>>>(c->pos.p, c->conn.p, a1.p, 0, 0.0, 1.0, 1.0, c->ne,
                                                                M1.p, M2.p);
        k_assemble_s<<<grid_for(c, c->nnzb, 256, 8), 256, 0, s>>>(c->gptr.p, c->gsrc.p, M1.p, M2.p, c->nnzb, Mv.p,
                                                                  Bv.p, M32.p);
        LMTG_CUDA(cudaMemcpyAsync(q.p, Q, nn * 8, cudaMemcpyHostToDevice, s));
        k_spmv_s<double><<<rgrid(c, k_spmv_s<double>), kRowThreads, 0, s>>>(c->bptr.p, c->bcol.p, Mv.p, q.p, mq.p,
                                                                              nn);
        LMTG_CUDA(cudaGetLastError());
        c->launches += 3;
        LMTG_CUDA(cudaMemcpyAsync(src.data(), mq.p, nn * 8, cudaMemcpyDeviceToHost, s));
        LMTG_CUDA(cudaStreamSynchronize(s));
    }
    if (Qs)
        for (uint64_t i = 0; i < nn; ++i) src[i] += Qs[i];
    if (Q || Qs) c->h_diff_src = src;
    else c->h_diff_src.clear();
    diff_update_load(c);
}

// Skin convection H (T - t0) te dS (formulation_difftherm.py:29) on Bar_3 edges (end, end, middle;
// formulations/element_Bar_3.py), integrated with the 3-point rule of element_Bar_3.py: in the
// theta scheme A += theta H Ms, B -= (1 - theta) H Ms, and the load H t0 int N ds.
void diff_set_convection(lmtg_ctx *c, uint64_t nedges, const uint32_t *edges, const double *H, uint64_t nH,
                         double t0) {
    LMTG_CHECK(c->allocated && c->elem_type == LMTG_ELEM_TRIANGLE6, LMTG_ERR_STATE, "diff_setup first");
    LMTG_CHECK(nH == 1 || nH == nedges, LMTG_ERR_ARG, "H needs 1 or nedges values");
    cudaStream_t s = c->stream;
    const uint64_t nn = c->nn;
    std::vector<uint32_t> bp(nn + 1), bc(c->nnzb);
    LMTG_CUDA(cudaMemcpyAsync(bp.data(), c->bptr.p, (nn + 1) * 4, cudaMemcpyDeviceToHost, s));
    LMTG_CUDA(cudaMemcpyAsync(bc.data(), c->bcol.p, c->nnzb * 4, cudaMemcpyDeviceToHost, s));
    LMTG_CUDA(cudaStreamSynchronize(s));
    const double gx[3] = {0.5 - 0.5 * std::sqrt(3.0 / 5.0), 0.5, 0.5 + 0.5 * std::sqrt(3.0 / 5.0)};
    const double gw[3] = {5.0 / 18.0, 8.0 / 18.0, 5.0 / 18.0};
    std::vector<std::pair<uint64_t, double>> ent;
    std::vector<double> load(nn, 0.0);
    for (uint64_t e = 0; e < nedges; ++e) {
        const uint32_t nd[3] = {edges[3 * e], edges[3 * e + 1], edges[3 * e + 2]};
        for (int k = 0; k < 3; ++k) LMTG_CHECK(nd[k] < nn, LMTG_ERR_ARG, "edge node >= nn");
        const double h = H[nH == 1 ? 0 : e];
        double Ms[3][3] = {}, Ns[3] = {};
        for (int g = 0; g < 3; ++g) {
            const double X = gx[g];
            const double N[3] = {2 * (1 - X) * (0.5 - X), 2 * X * (X - 0.5), 4 * (1 - X) * X};
            const double dN[3] = {4 * X - 3, 4 * X - 1, 4 - 8 * X};
            double dx = 0, dy = 0;
            for (int k = 0; k < 3; ++k) {
                dx += dN[k] * c->h_pos[2 * (uint64_t)nd[k]];
                dy += dN[k] * c->h_pos[2 * (uint64_t)nd[k] + 1];
            }
            const double wj = gw[g] * std::sqrt(dx * dx + dy * dy);
            for (int a = 0; a < 3; ++a) {
                Ns[a] += wj * N[a];
                for (int b = 0; b < 3; ++b) Ms[a][b] += wj * N[a] * N[b];
            }
        }
        for (int a = 0; a < 3; ++a) {
            load[nd[a]] += h * t0 * Ns[a];
            for (int b = 0; b < 3; ++b) {
                const uint32_t i = nd[a], j = nd[b];
                uint64_t q = bp[i];
                while (q < bp[i + 1] && bc[q] != j) ++q;
                LMTG_CHECK(q < bp[i + 1], LMTG_ERR_ARG, "edge nodes are not in one element");
                ent.push_back({q, h * Ms[a][b]});
            }
        }
    }
    std::stable_sort(ent.begin(), ent.end(), [](const std::pair<uint64_t, double> &x,
                                                const std::pair<uint64_t, double> &y) {
        return x.first < y.first;
    });  // stable sums: the contributions of one entry in edge order
    std::vector<uint64_t> at;
    std::vector<double> va, vb;
    for (size_t k = 0; k < ent.size();) {
        const uint64_t q = ent[k].first;
        double v = 0;
        for (; k < ent.size() && ent[k].first == q; ++k) v += ent[k].second;
        at.push_back(q);
        va.push_back(c->theta * v);
        vb.push_back(-(1.0 - c->theta) * v);
    }
    if (!at.empty()) {
        DBuf<uint64_t> dat;
        DBuf<double> dva, dvb;
        upload_u32(c, dat, at.data(), at.size());
        upload_u32(c, dva, va.data(), va.size());
        upload_u32(c, dvb, vb.data(), vb.size());
        k_add_entries<<<grid_for(c, at.size(), 256), 256, 0, s>>>(dat.p, dva.p, dvb.p, at.size(), c->K64.p, c->K32.p,
                                                                 c->B64.p);
        k_jacobi_s<double><<<grid_for(c, nn, 256), 256, 0, s>>>(c->bdiag.p, c->K64.p, nn, c->Dinv64.p, nullptr);
        k_jacobi_s<float><<<grid_for(c, nn, 256), 256, 0, s>>>(c->bdiag.p, c->K64.p, nn, c->Dinv32.p, nullptr);
        LMTG_CUDA(cudaGetLastError());
        c->launches += 3;
        LMTG_CUDA(cudaStreamSynchronize(s));
        samg_free(c);  // A changed: the multigrid is rebuilt at the next FP32 solve
    }
    c->h_diff_conv = load;
    diff_update_load(c);
}

int diff_run(lmtg_ctx *c, int nsteps, double tol, int maxit, lmtg_solve_stats *st) {
    int total = 0, status = LMTG_OK;
    for (int n = 0; n < nsteps && status == LMTG_OK; ++n) {
        int it = 0;
        status = diff_step(c, c->u.p, c->u.p, tol, maxit, &it);
        total += it;
    }
    st->iterations = total;
    st->outer_iterations = nsteps;
    return status;
}

// Final-time misfit J = 1/2 |T_N - target|^2 and dJ/dk_e (k = conductivity; a = k / rho_c) with
// checkpoints every `ck` steps: the forward sweep keeps T at steps 0, ck, 2ck, ...; the backward
// sweep recomputes each segment's states from its checkpoint, then walks the adjoint
//   A lambda_N = T_N - target,   A lambda_n = B lambda_{n+1},
//   dJ/da_e = -sum_n lambda_n^T Khat_e (theta T_n + (1 - theta) T_{n-1}).
int diff_adjoint(lmtg_ctx *c, int nsteps, int ck, const double *target_dev, double tol, int maxit,
                 double *J, std::vector<double> &grad, lmtg_solve_stats *st) {
    cudaStream_t s = c->stream;
    const uint64_t nn = c->nn;
    const int nck = nsteps / ck + 1;
    DBuf<double> ckpt, seg, lam, lam2, g;
    ckpt.alloc((uint64_t)nck * nn);
    if (ck > 1) seg.alloc((uint64_t)(ck + 1) * nn);  // ck == 1: every state is a checkpoint
    lam.alloc(nn);
    lam2.alloc(nn);
    g.alloc(c->ne);
    LMTG_CUDA(cudaMemsetAsync(g.p, 0, c->ne * 8, s));
    int total = 0, status = LMTG_OK, it = 0;
    // forward with checkpoints (u holds T_0 on entry)
    LMTG_CUDA(cudaMemcpyAsync(ckpt.p, c->u.p, nn * 8, cudaMemcpyDeviceToDevice, s));
    for (int n = 1; n <= nsteps && status == LMTG_OK; ++n) {
        status = diff_step(c, c->u.p, c->u.p, tol, maxit, &it);
        total += it;
        if (n % ck == 0) LMTG_CUDA(cudaMemcpyAsync(ckpt.p + (uint64_t)(n / ck) * nn, c->u.p, nn * 8,
                                                   cudaMemcpyDeviceToDevice, s));
    }
    if (status != LMTG_OK) return status;
    // objective and the final adjoint
    k_axpby<<<ngrid(c), kRowThreads, 0, s>>>(c->u.p, target_dev, c->w64[5].p, nn);
    c->launches += 1;
    {
        std::vector<double> d(nn);
        LMTG_CUDA(cudaMemcpyAsync(d.data(), c->w64[5].p, nn * 8, cudaMemcpyDeviceToHost, s));
        LMTG_CUDA(cudaStreamSynchronize(s));
        double acc = 0;
        for (double v : d) acc += v * v;
        *J = 0.5 * acc;
    }
    LMTG_CUDA(cudaMemsetAsync(lam.p, 0, nn * 8, s));
    status = diff_pcg(c, c->w64[5].p, lam.p, tol, maxit, &it);
    total += it;
    if (status != LMTG_OK) return status;
    // backward over segments
    for (int seg_start = ((nsteps - 1) / ck) * ck; seg_start >= 0 && status == LMTG_OK; seg_start -= ck) {
        const int seg_end = std::min(seg_start + ck, nsteps);
        // the segment's states: recomputed from its checkpoint, or the checkpoints themselves
        const double *states = ckpt.p + (uint64_t)seg_start * nn;
        if (ck > 1) {
            LMTG_CUDA(cudaMemcpyAsync(seg.p, ckpt.p + (uint64_t)(seg_start / ck) * nn, nn * 8,
                                      cudaMemcpyDeviceToDevice, s));
            for (int n = seg_start + 1; n <= seg_end && status == LMTG_OK; ++n) {
                status = diff_step(c, seg.p + (uint64_t)(n - 1 - seg_start) * nn,
                                   seg.p + (uint64_t)(n - seg_start) * nn, tol, maxit, &it);
                total += it;
            }
            states = seg.p;
        }
        for (int n = seg_end; n > seg_start && status == LMTG_OK; --n) {
            const double *Tn = states + (uint64_t)(n - seg_start) * nn;
            const double *Tm = states + (uint64_t)(n - 1 - seg_start) * nn;
            k_tri6_grad<<<grid_for(c, c->ne, 128, 16), 128, 0, s>>>(c->pos.p, c->conn.p, c->ne,
                                                                    c->theta, lam.p, Tn, Tm, g.p);
            c->launches += 1;
            if (n > 1) {  // lambda_{n-1}: A lambda_{n-1} = B lambda_n
                diff_rhs(c, lam.p, lam2.p);
                LMTG_CUDA(cudaMemcpyAsync(lam.p, lam2.p, nn * 8, cudaMemcpyDeviceToDevice, s));
                status = diff_pcg(c, lam2.p, lam.p, tol, maxit, &it);
                total += it;
            }
        }
    }
    grad.resize(c->ne);
    LMTG_CUDA(cudaMemcpyAsync(grad.data(), g.p, c->ne * 8, cudaMemcpyDeviceToHost, s));
    LMTG_CUDA(cudaStreamSynchronize(s));
    // dJ/dk = dJ/da / rho_c
    for (double &v : grad) v /= c->rho_c;
    st->iterations = total;
    st->outer_iterations = nsteps;
    return status;
}

}  // namespace lmtg

using namespace lmtg;

namespace {

template <class F>
int guard_d(lmtg_ctx *c, F &&f) {
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

int lmtg_make_rect_triangle6(const double X0[2], const double X1[2], const uint32_t nbp[2],
                             uint64_t *nn_out, uint64_t *ne_out, double *pos, uint32_t *conn) {
    if (!X0 || !X1 || !nbp || !nn_out || !ne_out) return LMTG_ERR_ARG;
    const uint64_t nx = nbp[0], ny = nbp[1];
    if (nx < 2 || ny < 2) return LMTG_ERR_ARG;
    const uint64_t gx = 2 * nx - 1, gy = 2 * ny - 1;
    if (gx * gy >= (1ull << 32)) return LMTG_ERR_UNSUPPORTED;
    *nn_out = gx * gy;
    *ne_out = 2 * (nx - 1) * (ny - 1);
    if (!pos || !conn) return LMTG_OK;
    // half-step grid of Rectilinear_iterator (accumulated, x fastest), make_rect.h:148-150
    std::vector<double> ax[2];
    for (int d = 0; d < 2; ++d) {
        const double lo = std::fmin(X0[d], X1[d]), hi = std::fmax(X0[d], X1[d]);
        const double inc = (hi - lo) / ((double)nbp[d] - 1.0) * .5;
        const double step = inc + (inc == 0.0 ? 1.0 : 0.0), upper = hi + step * 0.5;
        const uint64_t want = d ? gy : gx;
        for (double p = lo; p < upper; p += step) {
            if (ax[d].size() == want) return LMTG_ERR_ARG;
            ax[d].push_back(p);
        }
        if (ax[d].size() != want) return LMTG_ERR_ARG;
    }
    uint64_t n = 0;
    for (uint64_t j = 0; j < gy; ++j)
        for (uint64_t i = 0; i < gx; ++i, ++n) {
            pos[2 * n] = ax[0][i];
            pos[2 * n + 1] = ax[1][j];
        }
    // two triangles per cell, make_rect.h:153-167
    uint64_t e = 0;
    const uint64_t r = 2 * nx - 1;
    for (uint64_t i = 0; i + 1 < ny; ++i)
        for (uint64_t j = 0; j + 1 < nx; ++j) {
            const uint64_t b = 2 * i * r + 2 * j;
            const uint64_t p[9] = {b, b + 1, b + 2, b + r, b + 1 + r, b + 2 + r,
                                   b + 2 * r, b + 1 + 2 * r, b + 2 + 2 * r};
            const uint64_t t1[6] = {p[0], p[2], p[6], p[1], p[4], p[3]};
            const uint64_t t2[6] = {p[2], p[8], p[6], p[5], p[7], p[4]};
            for (int a = 0; a < 6; ++a) conn[6 * e + a] = (uint32_t)t1[a];
            ++e;
            for (int a = 0; a < 6; ++a) conn[6 * e + a] = (uint32_t)t2[a];
            ++e;
        }
    return LMTG_OK;
}

int lmtg_diff_mesh_set(lmtg_ctx *c, uint64_t nn, const double *pos, uint64_t ne,
                       const uint32_t *conn) {
    return guard_d(c, [&] {
        LMTG_CHECK(pos && conn && nn > 0 && ne > 0, LMTG_ERR_ARG, "empty mesh");
        LMTG_CHECK(nn < (1ull << 32), LMTG_ERR_UNSUPPORTED, "more than 2^32 nodes");
        for (uint64_t q = 0; q < 6 * ne; ++q) LMTG_CHECK(conn[q] < nn, LMTG_ERR_ARG, "node id >= nn");
        recal_free(c);
        amg_free(c);
        samg_free(c);
        diff_graphs_free(c);
        c->elem_type = LMTG_ELEM_TRIANGLE6;
        c->npe = 6;
        c->nnu = 1;
        c->npairs = 21;
        c->nn = nn;
        c->ne = ne;
        c->n = nn;
        c->pos.alloc(2 * nn);
        LMTG_CUDA(cudaMemcpyAsync(c->pos.p, pos, 16 * nn, cudaMemcpyHostToDevice, c->stream));
        c->h_pos.assign(pos, pos + 2 * nn);  // skin integrals (convection)
        c->h_diff_src.clear();
        c->h_diff_conv.clear();
        c->diff_load.release();
        upload_u32(c, c->conn, conn, 6 * ne);
        c->allocated = c->have64 = c->have32 = c->have_vec = false;
        LMTG_CUDA(cudaStreamSynchronize(c->stream));
        return LMTG_OK;
    });
}

int lmtg_diff_setup(lmtg_ctx *c, const double *k, uint64_t nk, double rho_c, double dt,
                    double theta, uint64_t nbnd, const uint32_t *bnd, double penalty) {
    return guard_d(c, [&] {
        LMTG_CHECK(k && (nbnd == 0 || bnd), LMTG_ERR_ARG, "null arrays");
        for (uint64_t q = 0; q < nbnd; ++q) LMTG_CHECK(bnd[q] < c->nn, LMTG_ERR_ARG, "node id >= nn");
        LMTG_CHECK(nbnd == 0 || penalty > 0, LMTG_ERR_UNSUPPORTED, "penalty constraints only");
        diff_setup(c, k, nk, rho_c, dt, theta, nbnd, bnd, penalty);
        return LMTG_OK;
    });
}

int lmtg_diff_set_sources(lmtg_ctx *c, const double *Q, const double *Qs) {
    return guard_d(c, [&] {
        diff_set_sources(c, Q, Qs);
        return LMTG_OK;
    });
}

int lmtg_diff_set_convection(lmtg_ctx *c, uint64_t nedges, const uint32_t *edges, const double *H, uint64_t nH,
                             double t0) {
    return guard_d(c, [&] {
        LMTG_CHECK(nedges == 0 || (edges && H), LMTG_ERR_ARG, "null arrays");
        diff_set_convection(c, nedges, edges, H, nH, t0);
        return LMTG_OK;
    });
}

int lmtg_diff_set_solver(lmtg_ctx *c, int mode) {
    return guard_d(c, [&] {
        LMTG_CHECK(mode == LMTG_SOLVE_PCG_F64 || mode == LMTG_SOLVE_MIXED_IR, LMTG_ERR_ARG, "unknown mode");
        c->diff_mode = mode;
        return LMTG_OK;
    });
}

int lmtg_diff_set_state(lmtg_ctx *c, const double *T) {
    return guard_d(c, [&] {
        LMTG_CHECK(c->allocated && c->elem_type == LMTG_ELEM_TRIANGLE6 && T, LMTG_ERR_STATE, "setup first");
        LMTG_CUDA(cudaMemcpyAsync(c->u.p, T, c->nn * 8, cudaMemcpyHostToDevice, c->stream));
        LMTG_CUDA(cudaStreamSynchronize(c->stream));
        return LMTG_OK;
    });
}

int lmtg_diff_get_state(lmtg_ctx *c, double *T) {
    return guard_d(c, [&] {
        LMTG_CHECK(c->allocated && c->elem_type == LMTG_ELEM_TRIANGLE6 && T, LMTG_ERR_STATE, "setup first");
        LMTG_CUDA(cudaMemcpyAsync(T, c->u.p, c->nn * 8, cudaMemcpyDeviceToHost, c->stream));
        LMTG_CUDA(cudaStreamSynchronize(c->stream));
        return LMTG_OK;
    });
}

int lmtg_diff_run(lmtg_ctx *c, int nsteps, double tol, int maxit, lmtg_solve_stats *st) {
    lmtg_solve_stats local{};
    if (!st) st = &local;
    memset(st, 0, sizeof(*st));
    return guard_d(c, [&] {
        LMTG_CHECK(c->have64 && c->elem_type == LMTG_ELEM_TRIANGLE6, LMTG_ERR_STATE, "setup first");
        LMTG_CHECK(nsteps >= 0 && maxit > 0, LMTG_ERR_ARG, "nsteps >= 0, maxit > 0");
        cudaEvent_t e0, e1;
        LMTG_CUDA(cudaEventCreate(&e0));
        LMTG_CUDA(cudaEventCreate(&e1));
        LMTG_CUDA(cudaEventRecord(e0, c->stream));
        int s = diff_run(c, nsteps, tol, maxit, st);
        LMTG_CUDA(cudaEventRecord(e1, c->stream));
        LMTG_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        st->device_ms = ms;
        st->status = s;
        if (s != LMTG_OK) c->err = lmtg_status_string(s);
        return s;
    });
}

int lmtg_diff_adjoint_misfit(lmtg_ctx *c, int nsteps, int ck, const double *target, double tol,
                             int maxit, double *J, double *dJdk, lmtg_solve_stats *st) {
    lmtg_solve_stats local{};
    if (!st) st = &local;
    memset(st, 0, sizeof(*st));
    return guard_d(c, [&] {
        LMTG_CHECK(c->have64 && c->elem_type == LMTG_ELEM_TRIANGLE6, LMTG_ERR_STATE, "setup first");
        LMTG_CHECK(nsteps > 0 && ck > 0 && maxit > 0 && J && dJdk, LMTG_ERR_ARG, "bad arguments");
        DBuf<double> t;
        if (target) {
            t.alloc(c->nn);
            LMTG_CUDA(cudaMemcpyAsync(t.p, target, c->nn * 8, cudaMemcpyHostToDevice, c->stream));
        }
        cudaEvent_t e0, e1;
        LMTG_CUDA(cudaEventCreate(&e0));
        LMTG_CUDA(cudaEventCreate(&e1));
        LMTG_CUDA(cudaEventRecord(e0, c->stream));
        std::vector<double> g;
        int s = diff_adjoint(c, nsteps, ck, t.p, tol, maxit, J, g, st);
        LMTG_CUDA(cudaEventRecord(e1, c->stream));
        LMTG_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        st->device_ms = ms;
        st->status = s;
        if (s != LMTG_OK) {
            c->err = std::string("diffusion adjoint: ") + lmtg_status_string(s);
            return s;
        }
        memcpy(dJdk, g.data(), c->ne * 8);
        return LMTG_OK;
    });
}

int lmtg_diff_get_matrices(lmtg_ctx *c, uint64_t *rowptr, uint32_t *col, double *A, double *B) {
    return guard_d(c, [&] {
        LMTG_CHECK(c->have64 && c->elem_type == LMTG_ELEM_TRIANGLE6, LMTG_ERR_STATE, "setup first");
        LMTG_CHECK(rowptr && col && A && B, LMTG_ERR_ARG, "null output");
        std::vector<uint32_t> bptr(c->nn + 1), bcol(c->nnzb);
        std::vector<double> hA(c->nnzb), hB(c->nnzb);
        LMTG_CUDA(cudaMemcpy(bptr.data(), c->bptr.p, bptr.size() * 4, cudaMemcpyDeviceToHost));
        LMTG_CUDA(cudaMemcpy(bcol.data(), c->bcol.p, bcol.size() * 4, cudaMemcpyDeviceToHost));
        LMTG_CUDA(cudaMemcpy(hA.data(), c->K64.p, hA.size() * 8, cudaMemcpyDeviceToHost));
        LMTG_CUDA(cudaMemcpy(hB.data(), c->B64.p, hB.size() * 8, cudaMemcpyDeviceToHost));
        uint64_t w = 0;
        rowptr[0] = 0;
        for (uint64_t i = 0; i < c->nn; ++i) {
            for (uint32_t q = bptr[i]; q < bptr[i + 1]; ++q) {
                if (bcol[q] > i) break;
                col[w] = bcol[q];
                A[w] = hA[q];
                B[w] = hB[q];
                ++w;
            }
            rowptr[i + 1] = w;
        }
        return LMTG_OK;
    });
}

}  // extern "C"
