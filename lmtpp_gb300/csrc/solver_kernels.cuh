// solver_kernels.cuh -- BSR 3x3 SpMV and the fused PCG iteration kernels.
//
// Replaces the reference's symmetric SparseLine SpMV (include/containers/matsparse.h:5368-5408)
// and the CG loop of conjugate_gradient (include/containers/conjugate_gradient.h:27-68):
//   q = K d; alpha = deltn / d.q; x += alpha d; r -= alpha q; s = P r; deltn = r.s; d = s + beta d
// with the 3x3 block-Jacobi preconditioner P standing in for the sequential IC(0) sweeps
// (matinvsparse.h:397-423), which have no parallel form.
//
// One PCG iteration = three kernels, no host round trip:
//   A0 k_pcg_dir:    p = z + beta p
//   A  k_pcg_spmv:   q = K p, pq = p . q                   (grid reduction, last block finalises)
//   B  k_pcg_update: alpha = rz / pq; x += alpha p; r -= alpha q; z = P r;
//                    rz, rr, |alpha p|_inf, |alpha p|_2^2, |r|_inf   -> beta, stopping test
// Scalars live in device memory (PcgScalars); when the test passes, `done` is set and every
// later kernel returns at once, so the host can launch iterations in captured chunks.
#pragma once
#include "lmtg_internal.cuh"

namespace lmtg {

constexpr int kRowThreads = 256;  // SpMV / PCG block size (8 warps, one node row per warp)

// Block + grid reduction of NV doubles; max for bits set in kMaxMask, sum otherwise.
// Returns true in the last block to arrive, where `out` holds the grid result (all threads).
// Deterministic: partials are combined in a fixed order.
template <int NV, unsigned kMaxMask, bool kWarpDone = false>
__device__ __forceinline__ bool grid_reduce(double (&v)[NV], double *partials, unsigned *ticket,
                                            double (&out)[NV]) {
    __shared__ double sh[NV][32];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int i = 0; i < NV; ++i) {
        if (!kWarpDone) v[i] = ((kMaxMask >> i) & 1u) ? warp_max(v[i]) : warp_sum(v[i]);
        if (lane == 0) sh[i][wid] = v[i];
    }
    __syncthreads();
    if (wid == 0) {
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            double x = lane < nw ? sh[i][lane] : 0.0;
            x = ((kMaxMask >> i) & 1u) ? warp_max(x) : warp_sum(x);
            if (lane == 0) partials[(size_t)i * gridDim.x + blockIdx.x] = x;
        }
    }
    if (threadIdx.x == 0) {
        __threadfence();
        unsigned t = atomicInc(ticket, gridDim.x - 1);  // wraps to 0 for the next launch
        last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
#pragma unroll
    for (int i = 0; i < NV; ++i) {
        double x = 0.0;
        for (unsigned k = threadIdx.x; k < gridDim.x; k += blockDim.x) {
            double y = __ldcg(partials + (size_t)i * gridDim.x + k);
            x = ((kMaxMask >> i) & 1u) ? fmax(x, y) : x + y;
        }
        x = ((kMaxMask >> i) & 1u) ? warp_max(x) : warp_sum(x);
        __syncthreads();
        if (lane == 0) sh[i][wid] = x;
        __syncthreads();
        double y = lane < nw ? sh[i][lane] : 0.0;
        y = ((kMaxMask >> i) & 1u) ? warp_max(y) : warp_sum(y);
        out[i] = y;
    }
    return true;
}

// Grid reduction of per-thread partials held in T: the warp level runs in T (FP32 shuffles
// and adds for the FP32 solver -- GB300's FP64 pipe is ~60x narrower), block and grid levels
// in FP64.
template <int NV, unsigned kMaxMask, class T>
__device__ __forceinline__ bool grid_reduce_t(const T (&t)[NV], double *partials, unsigned *ticket,
                                              double (&out)[NV]) {
    double v[NV];
#pragma unroll
    for (int i = 0; i < NV; ++i) {
        const T w = ((kMaxMask >> i) & 1u) ? warp_max(t[i]) : warp_sum(t[i]);
        v[i] = (double)w;
    }
    return grid_reduce<NV, kMaxMask, true>(v, partials, ticket, out);
}

// Row product of node row I: acc[r] = sum_blocks sum_c K_IJ[r][c] * X(3J+c), X from a functor.
// Lanes stride over the row's 9*deg contiguous values (coalesced); block/row/col of a value
// are tracked incrementally (32 = 3*9 + 5).
template <class T, class XF>
__device__ __forceinline__ void bsr3_row(const uint32_t *__restrict__ bcol, const T *__restrict__ K,
                                         uint32_t rb, uint32_t re, int lane, XF xf, T &a0, T &a1,
                                         T &a2) {
    const T *base = K + (uint64_t)rb * 9;
    const uint32_t nv = (re - rb) * 9;
    uint32_t b = lane / 9;
    int rem = lane - 9 * (int)b;
    a0 = a1 = a2 = (T)0;
    for (uint32_t v = lane; v < nv; v += 32) {
        const uint32_t J = __ldg(bcol + rb + b);
        const int rr = rem / 3, cc = rem - 3 * (rem / 3);
        const T prod = __ldg(base + v) * xf(3 * (uint64_t)J + cc);
        if (rr == 0) a0 += prod;
        else if (rr == 1) a1 += prod;
        else a2 += prod;
        rem += 5;
        b += 3;
        if (rem >= 9) {
            rem -= 9;
            b += 1;
        }
    }
    a0 = warp_sum(a0);
    a1 = warp_sum(a1);
    a2 = warp_sum(a2);
}

// Reduce-scatter of (a0, a1, a2, 0) over the warp: returns in every lane the total of
// component (lane >> 3) & 3 (lanes 0, 8, 16 hold rows 3I, 3I+1, 3I+2); 6 shuffles instead of 15.
template <class T>
__device__ __forceinline__ T reduce_scatter3(T a0, T a1, T a2, int lane) {
    const bool hi16 = (lane & 16) != 0, hi8 = (lane & 8) != 0;
    const T s0 = hi16 ? a0 : a2, s1 = hi16 ? a1 : (T)0;
    const T k0 = hi16 ? a2 : a0, k1 = hi16 ? (T)0 : a1;
    const T b0 = k0 + __shfl_xor_sync(0xffffffffu, s0, 16);
    const T b1 = k1 + __shfl_xor_sync(0xffffffffu, s1, 16);
    T c = (hi8 ? b1 : b0) + __shfl_xor_sync(0xffffffffu, hi8 ? b0 : b1, 8);
    c += __shfl_xor_sync(0xffffffffu, c, 4);
    c += __shfl_xor_sync(0xffffffffu, c, 2);
    c += __shfl_xor_sync(0xffffffffu, c, 1);
    return c;
}

// Reduce-scatter of 16 values over the warp: afterwards lane L holds the warp total of value
// (L >> 1) & 15 (each value in two lanes); 16 shuffles instead of 16 x 5.
template <class T>
__device__ __forceinline__ T reduce_scatter16(T (&a)[16], int lane) {
#pragma unroll
    for (int s = 0; s < 4; ++s) {
        const int h = 8 >> s, bit = 16 >> s;
        const bool hi = (lane & bit) != 0;
#pragma unroll
        for (int i = 0; i < h; ++i) {
            const T send = hi ? a[i] : a[i + h];
            const T keep = hi ? a[i + h] : a[i];
            a[i] = keep + __shfl_xor_sync(0xffffffffu, send, bit);
        }
    }
    return a[0] + __shfl_xor_sync(0xffffffffu, a[0], 1);
}

// 3x3 block times a node vector, accumulated into (a0, a1, a2).
template <class T>
__device__ __forceinline__ void block_fma(const T (&m)[9], T x0, T x1, T x2, T &a0, T &a1, T &a2) {
    a0 = fma(m[0], x0, a0); a0 = fma(m[1], x1, a0); a0 = fma(m[2], x2, a0);
    a1 = fma(m[3], x0, a1); a1 = fma(m[4], x1, a1); a1 = fma(m[5], x2, a1);
    a2 = fma(m[6], x0, a2); a2 = fma(m[7], x1, a2); a2 = fma(m[8], x2, a2);
}

// Row product of node row I (any number of blocks), one 3x3 block per lane.  Rows are stored
// planar (kidx): lane b reads component k of its block at 9 rb + k deg + b, so each of the 9
// loads is one coalesced warp access straight into registers.  xnode(J, x0, x1, x2) fetches
// the three x values of node J.  Returns the reduce_scatter3 layout.
template <class T, class XN>
__device__ __forceinline__ T bsr3_row_lanes(const uint32_t *__restrict__ bcol,
                                            const T *__restrict__ K, uint32_t rb, uint32_t re,
                                            int lane, XN xnode) {
    const uint32_t deg = re - rb;
    T a0 = (T)0, a1 = (T)0, a2 = (T)0;
    for (uint32_t b0 = 0; b0 < deg; b0 += 32) {
        const uint32_t bl = b0 + lane;
        if (bl < deg) {
            T m[9];
#pragma unroll
            for (int k = 0; k < 9; ++k) m[k] = __ldcs(K + kidx(rb, deg, bl, k));
            T x0, x1, x2;
            xnode(__ldcs(bcol + rb + bl), x0, x1, x2);
            block_fma(m, x0, x1, x2, a0, a1, a2);
        }
    }
    return reduce_scatter3(a0, a1, a2, lane);
}

// Node vectors gathered by the SpMV (z, p) are stored with a stride VS per node: 3 (packed) or
// 4 (FP32, padded so that a node's three components are one aligned 16-byte load).
template <class T, int VS>
struct NodeVec {
    static __device__ __forceinline__ void load(const T *__restrict__ v, uint64_t J, T &a, T &b, T &c) {
        a = __ldg(v + VS * J);
        b = __ldg(v + VS * J + 1);
        c = __ldg(v + VS * J + 2);
    }
};
template <>
struct NodeVec<float, 4> {
    static __device__ __forceinline__ void load(const float *__restrict__ v, uint64_t J, float &a,
                                                float &b, float &c) {
        const float4 q = __ldg(reinterpret_cast<const float4 *>(v) + J);
        a = q.x;
        b = q.y;
        c = q.z;
    }
};

// y = K x
template <class T>
__global__ void __launch_bounds__(kRowThreads)
    k_spmv(const uint32_t *__restrict__ bptr, const uint32_t *__restrict__ bcol,
           const T *__restrict__ K, const T *__restrict__ x, T *__restrict__ y, uint64_t nn) {
    const int lane = threadIdx.x & 31;
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t I = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; I < nn; I += nw) {
        const T v = bsr3_row_lanes(bcol, K, bptr[I], bptr[I + 1], lane,
                                   [&](uint64_t J, T &a, T &b, T &c) { NodeVec<T, 3>::load(x, J, a, b, c); });
        if ((lane & 7) == 0 && lane < 24) y[3 * I + (lane >> 3)] = v;
    }
}

// r = b - K x (T), rr = r.r accumulated in FP64 into *rr_out (grid reduction).
template <class T>
__global__ void __launch_bounds__(kRowThreads)
    k_residual(const uint32_t *__restrict__ bptr, const uint32_t *__restrict__ bcol,
               const T *__restrict__ K, const T *__restrict__ x, const T *__restrict__ b,
               T *__restrict__ r, uint64_t nn, double *partials, unsigned *ticket,
               double *rr_out) {
    const int lane = threadIdx.x & 31;
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    double v[1] = {0.0};
    for (uint64_t I = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; I < nn; I += nw) {
        const T a = bsr3_row_lanes(bcol, K, bptr[I], bptr[I + 1], lane,
                                   [&](uint64_t J, T &p, T &q, T &w) { NodeVec<T, 3>::load(x, J, p, q, w); });
        if ((lane & 7) == 0 && lane < 24) {
            const uint64_t i = 3 * I + (lane >> 3);
            const T ri = b[i] - a;
            r[i] = ri;
            v[0] += (double)ri * (double)ri;
        }
    }
    double out[1];
    if (grid_reduce<1, 0u>(v, partials, ticket, out) && threadIdx.x == 0) *rr_out = out[0];
}

// Start of a PCG run: z = P r, rz, rr, |r|_inf; optional bb = b.b.  Initial stopping test on
// the residual criteria (the delta criteria need one step, conjugate_gradient.h:40-41).
template <class T, int VS>
__global__ void k_pcg_start(const T *__restrict__ r, const T *__restrict__ b,
                            const T *__restrict__ Dinv, T *__restrict__ z, uint64_t nn,
                            PcgScalars *S, double *partials, double beta_den) {
    T t[4] = {(T)0, (T)0, (T)0, (T)0};  // rz, rr, bb, rinf per thread (T); grid sum in FP64
    for (uint64_t I = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; I < nn;
         I += (uint64_t)gridDim.x * blockDim.x) {
        const T *D = Dinv + 9 * I;
        const T r0 = r[3 * I], r1 = r[3 * I + 1], r2 = r[3 * I + 2];
        const T z0 = D[0] * r0 + D[1] * r1 + D[2] * r2;
        const T z1 = D[3] * r0 + D[4] * r1 + D[5] * r2;
        const T z2 = D[6] * r0 + D[7] * r1 + D[8] * r2;
        z[VS * I] = z0;
        z[VS * I + 1] = z1;
        z[VS * I + 2] = z2;
        t[0] += r0 * z0 + r1 * z1 + r2 * z2;
        t[1] += r0 * r0 + r1 * r1 + r2 * r2;
        if (b) {
            const T b0 = b[3 * I], b1 = b[3 * I + 1], b2 = b[3 * I + 2];
            t[2] += b0 * b0 + b1 * b1 + b2 * b2;
        }
        t[3] = fmax(t[3], fmax(fabs(r0), fmax(fabs(r1), fabs(r2))));
    }
    double out[4];
    if (grid_reduce_t<4, 8u>(t, partials, &S->cnt_c, out) && threadIdx.x == 0) {
        S->rz = out[0];
        S->rr = out[1];
        if (b) S->bb = out[2];
        // beta_den > 0 continues a previous run after a residual replacement: the search
        // direction is kept and beta = rz_new / beta_den (the caller folds in the rescaling)
        S->beta = beta_den > 0.0 ? out[0] / beta_den : 0.0;
        S->iter = 0;
        S->status = LMTG_OK;
        S->done = 0;
        if (S->crit_kind == LMTG_CRIT_REL_RESIDUAL && out[1] <= S->crit * S->crit * S->bb)
            S->done = 1;
        if (S->crit_kind == LMTG_CRIT_ABS_RESIDUAL_INF && out[3] <= S->crit) S->done = 1;
        if (!isfinite(out[0]) || !isfinite(out[1])) {
            S->done = 1;
            S->status = LMTG_ERR_NAN;
        }
    }
}

// Kernel A0: p = z + beta p in place (beta = 0 on a fresh start: p = z), padded node stride VS
template <class T, int VS>
__global__ void k_pcg_dir(const T *__restrict__ z, T *__restrict__ p, uint64_t nn, const PcgScalars *S) {
    if (*(volatile const int *)&S->done) return;
    const T beta = (T)S->beta;
    if constexpr (sizeof(T) == 4 && VS == 4) {  // whole 16-byte nodes
        const float4 *z4 = reinterpret_cast<const float4 *>(z);
        float4 *p4 = reinterpret_cast<float4 *>(p);
        for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < nn;
             i += (uint64_t)gridDim.x * blockDim.x) {
            const float4 zv = z4[i];
            if (beta != (T)0) {
                const float4 pv = p4[i];
                p4[i] = make_float4(fmaf(beta, pv.x, zv.x), fmaf(beta, pv.y, zv.y), fmaf(beta, pv.z, zv.z),
                                    fmaf(beta, pv.w, zv.w));
            } else {
                p4[i] = zv;
            }
        }
    } else {
        for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < VS * nn;
             i += (uint64_t)gridDim.x * blockDim.x)
            p[i] = beta != (T)0 ? fma(beta, p[i], z[i]) : z[i];
    }
}

// Matrix values and column indices are read once per SpMV: they are loaded with the
// streaming hint (ld.global.cs), so that they do not evict the gathered vector from L1
// (0.487 -> 0.448 ms per FP32 launch at 128^3).
//
// Kernel A: q = K p; pq = p . q.  Each block owns a contiguous range of rows (neighbouring rows
// gather mostly the same p entries, so the range's gathers hit L1); each warp takes two adjacent
// rows per step and issues both rows' matrix loads and column indices before the dependent p
// gathers.  Only p is gathered: the direction update has its own pass (kernel A0), which costs
// one vector pass and saves one gather per block (7% per iteration at 128^3).
template <class T, int VS>
__global__ void __launch_bounds__(kRowThreads)
    k_pcg_spmv(const uint32_t *__restrict__ bptr, const uint32_t *__restrict__ bcol,
                 const T *__restrict__ K, const T *__restrict__ p, T *__restrict__ q, uint64_t nn,
                 PcgScalars *S, double *partials) {
    if (*(volatile int *)&S->done) return;
    const int lane = threadIdx.x & 31;
    auto xnode = [&](uint64_t J, T &a, T &b, T &c) { NodeVec<T, VS>::load(p, J, a, b, c); };
    T acc = (T)0;
    auto finish = [&](uint64_t I, T qi) {
        if ((lane & 7) == 0 && lane < 24) {
            q[3 * I + (lane >> 3)] = qi;
            acc = fma(p[VS * I + (lane >> 3)], qi, acc);
        }
    };
    const uint64_t per_block = (nn + gridDim.x - 1) / gridDim.x;
    const uint64_t row0 = blockIdx.x * per_block;
    const uint64_t row_end = min(nn, row0 + per_block);
    const uint64_t wid = threadIdx.x >> 5, nwb = blockDim.x >> 5;
    for (uint64_t I = row0 + 2 * wid; I < row_end; I += 2 * nwb) {
        const uint64_t I1 = I + 1;
        const uint32_t rb0 = bptr[I], re0 = bptr[I + 1];
        const uint32_t rb1 = I1 < row_end ? bptr[I1] : 0u, re1 = I1 < row_end ? bptr[I1 + 1] : 0u;
        const uint32_t d0 = re0 - rb0, d1 = re1 - rb1;
        if (d0 <= 32 && d1 <= 32) {
            T m0[9], m1[9];
            const bool on0 = (uint32_t)lane < d0, on1 = (uint32_t)lane < d1;
#pragma unroll
            for (int k = 0; k < 9; ++k) {
                m0[k] = on0 ? __ldcs(K + kidx(rb0, d0, lane, k)) : (T)0;
                m1[k] = on1 ? __ldcs(K + kidx(rb1, d1, lane, k)) : (T)0;
            }
            const uint32_t j0 = on0 ? __ldcs(bcol + rb0 + lane) : 0u;
            const uint32_t j1 = on1 ? __ldcs(bcol + rb1 + lane) : 0u;
            T x00 = 0, x01 = 0, x02 = 0, x10 = 0, x11 = 0, x12 = 0;
            if (on0) xnode(j0, x00, x01, x02);
            if (on1) xnode(j1, x10, x11, x12);
            T a00 = 0, a01 = 0, a02 = 0, a10 = 0, a11 = 0, a12 = 0;
            block_fma(m0, x00, x01, x02, a00, a01, a02);
            block_fma(m1, x10, x11, x12, a10, a11, a12);
            const T q0 = reduce_scatter3(a00, a01, a02, lane);
            const T q1 = reduce_scatter3(a10, a11, a12, lane);
            finish(I, q0);
            if (I1 < row_end) finish(I1, q1);
        } else {
            finish(I, bsr3_row_lanes(bcol, K, rb0, re0, lane, xnode));
            if (I1 < row_end) finish(I1, bsr3_row_lanes(bcol, K, rb1, re1, lane, xnode));
        }
    }
    const T tacc[1] = {acc};
    double out[1];
    if (grid_reduce_t<1, 0u>(tacc, partials, &S->cnt_a, out) && threadIdx.x == 0) {
        S->pq = out[0];
        S->alpha = S->rz / (out[0] + (out[0] == 0.0 ? 1.0 : 0.0));  // once, not per thread
    }
}

// Kernel B: alpha, updates, preconditioner, dots, beta and the stopping test.
template <class T, int VS>
__global__ void k_pcg_update(T *__restrict__ x, T *__restrict__ r, T *__restrict__ z,
                             const T *__restrict__ p, const T *__restrict__ q,
                             const T *__restrict__ Dinv, uint64_t nn, PcgScalars *S,
                             double *partials) {
    if (*(volatile int *)&S->done) return;
    const double pq = S->pq;
    const T alpha = (T)S->alpha;
    T t[5] = {(T)0, (T)0, (T)0, (T)0, (T)0};  // rz, rr, dx2, dxinf, rinf per thread (T)
    for (uint64_t I = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; I < nn;
         I += (uint64_t)gridDim.x * blockDim.x) {
        T rv[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const uint64_t i = 3 * I + c;
            const T dx = alpha * p[VS * I + c];
            x[i] += dx;
            rv[c] = fma(-alpha, q[i], r[i]);
            r[i] = rv[c];
            t[2] = fma(dx, dx, t[2]);
            t[3] = fmax(t[3], fabs(dx));
            t[4] = fmax(t[4], fabs(rv[c]));
        }
        const T *D = Dinv + 9 * I;
        const T z0 = D[0] * rv[0] + D[1] * rv[1] + D[2] * rv[2];
        const T z1 = D[3] * rv[0] + D[4] * rv[1] + D[5] * rv[2];
        const T z2 = D[6] * rv[0] + D[7] * rv[1] + D[8] * rv[2];
        z[VS * I] = z0;
        z[VS * I + 1] = z1;
        z[VS * I + 2] = z2;
        t[0] += rv[0] * z0 + rv[1] * z1 + rv[2] * z2;
        t[1] += rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2];
    }
    double out[5];
    if (grid_reduce_t<5, (8u | 16u)>(t, partials, &S->cnt_b, out) && threadIdx.x == 0) {
        const double rz_old = S->rz;
        S->iter += 1;
        S->rr = out[1];
        S->dx_2sq = out[2];
        S->dx_inf = out[3];
        S->beta = out[0] / rz_old;
        S->rz = out[0];
        bool conv = false;
        switch (S->crit_kind) {
            case LMTG_CRIT_REL_RESIDUAL: conv = out[1] <= S->crit * S->crit * S->bb; break;
            case LMTG_CRIT_NORM_INF_DELTA: conv = out[3] <= S->crit; break;
            case LMTG_CRIT_NORM2_DELTA: conv = sqrt(out[2]) < S->crit; break;
            case LMTG_CRIT_ABS_RESIDUAL_INF: conv = out[4] <= S->crit; break;
        }
        if (!isfinite(out[0]) || !isfinite(out[1]) || !isfinite(pq)) {
            S->status = LMTG_ERR_NAN;
            S->done = 1;
        } else if (conv) {
            S->done = 1;
        } else if (S->iter >= S->maxit) {
            S->status = LMTG_ERR_NOT_CONVERGED;
            S->done = 1;
        }
    }
}

// Mixed-precision helpers: r32 = r64 * s_inv ; x64 += s * d32
__global__ void k_scale_to32(const double *__restrict__ a, double s_inv, float *__restrict__ o,
                             uint64_t n);
__global__ void k_axpy_64_32(double *__restrict__ x, double s, const float *__restrict__ d,
                             uint64_t n);

}  // namespace lmtg
