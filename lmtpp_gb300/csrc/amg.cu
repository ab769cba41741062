// amg.cu -- aggregation multigrid preconditioner for the FP32 inner PCG of elasticity.
//
// The reference preconditions its CG with a sequential incomplete Cholesky
// (include/containers/matinvsparse.h:201-261, 3x3-block variant
// include/containers/MatWithTinyBlocks.h:426-585), which has no parallel form; block Jacobi, its
// stand-in here, needs O(mesh side) iterations (2,388 at Hexa8 128^3).  This file replaces z = P r
// by one W-cycle of an unsmoothed-aggregation multigrid whose coarse spaces hold the rigid-body
// modes, so that the iteration count stays nearly flat with the mesh size (41 at Hexa8 128^3).
//
// Hierarchy (structure built once per pattern and constraint set, on the host):
//   level 0   the context's 3x3-block matrix K32 (planar rows, kidx), its block-Jacobi Dinv32
//   level l+1 aggregates of level-l nodes: a root node with all its free neighbours, then the
//             leftovers joined to a neighbouring aggregate, then the rest grouped around a free
//             node.  Nodes carrying a constraint are left out (the smoother alone handles them).
//   Q_l       per level-l node a b x 6 block of the tentative prolongator: the six rigid-body modes
//             of the aggregate (three translations, three rotations about its centroid at level 0;
//             the coarse modes R at deeper levels) orthonormalised per aggregate (Gram-Schmidt in
//             FP64); a mode that the aggregate cannot carry (one node, or nodes on a line) gives a
//             zero column, and the coarse unknown it would define is a decoupled unit diagonal.
//   K_{l+1}   = Q_l^T K_l Q_l (Galerkin), 6x6 blocks: one warp per aggregate streams its nodes'
//             rows and sums every coarse entry in one fixed order (no atomics, deterministic).
//   coarsest  (<= 300 unknowns): a dense inverse, computed on the host in FP64, applied in FP32.
// Numeric setup after every matrix assembly: the Galerkin products, the 6x6 block-Jacobi
// inverses, and per level the damped-Jacobi weight omega = 1.47 / lambda_max(D^-1 K) (lambda_max by
// twelve power steps, which approach it from below; the weight of a degree-1 Chebyshev smoother on
// [h/30, h], h = 1.2 lambda).
//
// W-cycle (z = M r), per level: x = omega D^-1 r; res = r - K x; restrict Q^T res; the coarse
// correction e (the next level's cycle run twice, the second time on the residual the first
// leaves; one dense solve on the coarsest); x += 1.5 Q e; x' = x + omega D^-1 (r - K x).  The
// same smoother before and after makes M symmetric, as the conjugate gradient needs.  At level 0
// the first smoothing step is fused into the PCG's update kernel and the last one writes z and
// forms r.z and beta; at the coarser levels the first smoothing step is fused into the
// restriction (or residual) that produces the level's right-hand side.  Large 6x6 levels stream
// their matrix by bulk copies (amg_bulk6.cuh).  Every kernel returns at once once the PCG's
// `done` flag is set, so the cycle runs inside the captured iteration chunks.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <memory>
#include <thread>
#include <vector>

#include "amg.cuh"
#include "amg_bulk6.cuh"
#include "pdl.cuh"
#include "spmv_bulk.cuh"

namespace lmtg {

namespace {

constexpr uint32_t kNone = 0xffffffffu;
constexpr int kMaxLevels = 8;
constexpr int kPowerSteps = 12;  // power steps for lambda_max(D^-1 K) per level
constexpr uint64_t kCoarsestDofs = 300;
constexpr uint64_t kDenseMaxDofs = 2000;  // largest coarsest level (its dense inverse) accepted
// the coarse correction is scaled by this factor (over-correction of unsmoothed aggregation)
constexpr float kCoarseScale = 1.5f;

// planar 6x6 block rows: component v (row-major) of local block b of a row starting at block rb
__host__ __device__ __forceinline__ uint64_t kidx6(uint32_t rb, uint32_t deg, uint32_t b, int v) {
    return 36ull * rb + (uint64_t)v * deg + b;
}

template <int B>
__host__ __device__ __forceinline__ uint64_t kidxb(uint32_t rb, uint32_t deg, uint32_t b, int v) {
    return (uint64_t)(B * B) * rb + (uint64_t)v * deg + b;
}

__device__ __forceinline__ bool done(const PcgScalars *S) { return S && *(volatile const int *)&S->done; }

// ---------------------------------------------------------------------------------------------
// numeric setup kernels
// ---------------------------------------------------------------------------------------------

// Coarse row I of Q^T K Q, one warp per aggregate I.  The warp takes the fine blocks of the
// aggregate's rows 32 at a time (lane = block; aggregate-node order, then row order); each lane
// forms its block's 6x6 product Q_i^T K_ij Q_j and its slot in the coarse row (the position of
// agg(j) among the row's sorted columns) and stages them in shared memory; then the staged
// products are added to the row's accumulator in lane order, the lanes splitting the 36 entries.
// Every coarse entry is summed in one fixed order (deterministic, no atomics).  A coarse diagonal entry that sums to
// exactly zero (a mode the aggregate cannot carry) becomes 1, a decoupled unknown.
constexpr int kGalMaxDeg = 128;  // widest coarse row the shared accumulator may hold
constexpr int kGalWarps = 8;
// shared memory of one warp for coarse rows of at most cap blocks: acc[cap][36], stage[32][36], slot[32]
__host__ __device__ constexpr size_t gal_warp_bytes(int cap) { return 4u * (36u * cap + 36u * 32u + 32u); }

// Slot of every fine block (I, J) in its coarse row: the position of agg(J) among the sorted
// columns of agg(I)'s row (kNoSlot when J is in no aggregate).  Depends only on the patterns and
// the aggregation: computed once per structure, read by every Galerkin product.
constexpr uint8_t kNoSlot = 0xff;
static_assert(kGalMaxDeg < kNoSlot, "coarse slots fit a byte");

__global__ void k_gal_slots(const uint32_t *__restrict__ fbptr, const uint32_t *__restrict__ fbcol,
                            const uint32_t *__restrict__ agg, uint64_t nn, const uint32_t *__restrict__ cbptr,
                            const uint32_t *__restrict__ cbcol, uint8_t *__restrict__ gslot) {
    const int lane = threadIdx.x & 31;
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t i = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; i < nn; i += nw) {
        const uint32_t a = agg[i];
        const uint32_t rb = fbptr[i], deg = fbptr[i + 1] - rb;
        for (uint32_t bl = lane; bl < deg; bl += 32) {
            uint8_t slot = kNoSlot;
            const uint32_t J = agg[fbcol[rb + bl]];
            if (a != kNone && J != kNone) {
                const uint32_t crb = cbptr[a], cdeg = cbptr[a + 1] - crb;
                uint32_t lo = 0, hi = cdeg;  // J is in the row: lower_bound finds it
                while (lo < hi) {
                    const uint32_t mid = (lo + hi) >> 1;
                    if (cbcol[crb + mid] < J) lo = mid + 1;
                    else hi = mid;
                }
                slot = (uint8_t)lo;
            }
            gslot[rb + bl] = slot;
        }
    }
}

template <int B>
__global__ void __launch_bounds__(32 * kGalWarps)
    k_galerkin(const uint32_t *__restrict__ fbptr, const uint32_t *__restrict__ fbcol, const float *__restrict__ fK,
               const uint32_t *__restrict__ agg, const uint32_t *__restrict__ aptr, const uint32_t *__restrict__ anode,
               const float *__restrict__ Q, const uint32_t *__restrict__ cbptr, const uint32_t *__restrict__ cbcol,
               const uint8_t *__restrict__ gslot, uint64_t na, int cap, float *__restrict__ cK) {
    extern __shared__ __align__(16) unsigned char gal_raw[];
    float *wbase = reinterpret_cast<float *>(gal_raw + (threadIdx.x >> 5) * gal_warp_bytes(cap));
    float(*acc)[36] = reinterpret_cast<float(*)[36]>(wbase);
    float(*stage)[36] = reinterpret_cast<float(*)[36]>(wbase + 36 * cap);
    int *slots = reinterpret_cast<int *>(wbase + 36 * cap + 36 * 32);
    const int lane = threadIdx.x & 31;
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t a = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; a < na; a += nw) {
        const uint32_t crb = cbptr[a], cdeg = cbptr[a + 1] - crb;
        const uint32_t *crow = cbcol + crb;
        for (uint32_t t = lane; t < cdeg * 36; t += 32) (&acc[0][0])[t] = 0.f;
        __syncwarp();
        for (uint32_t u = aptr[a]; u < aptr[a + 1]; ++u) {
            const uint32_t i = anode[u];
            const uint32_t rb = fbptr[i], deg = fbptr[i + 1] - rb;
            const float *Qi = Q + (uint64_t)i * B * 6;
            for (uint32_t c0 = 0; c0 < deg; c0 += 32) {
                const uint32_t bl = c0 + lane;
                int slot = -1;
                if (bl < deg) {
                    const uint32_t j = fbcol[rb + bl], gs = gslot[rb + bl];
                    if (gs != kNoSlot) {
                        slot = (int)gs;
                        float A[B * B];
#pragma unroll
                        for (int v = 0; v < B * B; ++v) A[v] = fK[kidxb<B>(rb, deg, bl, v)];
                        const float *Qj = Q + (uint64_t)j * B * 6;
                        float T[B * 6];  // A Q_j
#pragma unroll
                        for (int r = 0; r < B; ++r)
#pragma unroll
                            for (int c = 0; c < 6; ++c) {
                                float s = 0.f;
#pragma unroll
                                for (int m = 0; m < B; ++m) s = fmaf(A[r * B + m], __ldg(Qj + m * 6 + c), s);
                                T[r * 6 + c] = s;
                            }
                        float C[36];
#pragma unroll
                        for (int v = 0; v < 36; ++v) C[v] = 0.f;
#pragma unroll
                        for (int r = 0; r < B; ++r) {
                            float q[6];
#pragma unroll
                            for (int x = 0; x < 6; ++x) q[x] = __ldg(Qi + r * 6 + x);
#pragma unroll
                            for (int x = 0; x < 6; ++x)
#pragma unroll
                                for (int c = 0; c < 6; ++c) C[x * 6 + c] = fmaf(q[x], T[r * 6 + c], C[x * 6 + c]);
                        }
#pragma unroll
                        for (int v = 0; v < 36; ++v) stage[lane][v] = C[v];
                    }
                }
                slots[lane] = slot;
                __syncwarp();
                // staged products added in lane order, the 36 entries of each by the warp's lanes
                const int nl = min(32u, deg - c0);
                for (int l = 0; l < nl; ++l) {
                    const int sl = slots[l];
                    if (sl >= 0) {
                        acc[sl][lane] += stage[l][lane];
                        if (lane < 4) acc[sl][32 + lane] += stage[l][32 + lane];
                    }
                }
                __syncwarp();
            }
        }
        for (uint32_t t = lane; t < cdeg * 36; t += 32) {
            const uint32_t sl = t / 36;
            const int v = (int)(t - 36 * sl);
            float x = acc[sl][v];
            if (crow[sl] == a && v % 7 == 0 && x == 0.f) x = 1.f;
            cK[kidx6(crb, cdeg, sl, v)] = x;
        }
        __syncwarp();
    }
}

// Tentative prolongator of one level on the device, one warp per aggregate: the aggregate's
// modes (level 0: translations and rotations about `cen` from the node positions; deeper: the
// previous level's coarse modes Bf, 6 x 6 per node) as a rows x 6 matrix, rows spread over the
// lanes (row lane + 32 k), orthonormalised by Gram-Schmidt twice in FP64 with warp sums; a column
// that falls below 1e-10 of its original norm is dropped (zero).  Writes Q (b x 6 per node, FP32)
// and the coarse modes Bc = R (6 x 6 per aggregate).  rows <= 32 kTentRows (checked on the host).
constexpr int kTentRows = 10;
template <int B>
__global__ void __launch_bounds__(128)
    k_tentative(const uint32_t *__restrict__ aptr, const uint32_t *__restrict__ anode, uint64_t na,
                const double *__restrict__ pos, double cx, double cy, double cz, const double *__restrict__ Bf,
                float *__restrict__ Q, double *__restrict__ Bc) {
    const int lane = threadIdx.x & 31;
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t a = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; a < na; a += nw) {
        const uint32_t n0 = aptr[a], rows = (aptr[a + 1] - n0) * B;
        double M[kTentRows][6];
#pragma unroll
        for (int k = 0; k < kTentRows; ++k) {
            const uint32_t r = lane + 32 * k;
#pragma unroll
            for (int c = 0; c < 6; ++c) M[k][c] = 0.0;
            if (r < rows) {
                const uint32_t i = anode[n0 + r / B];
                const int rr = (int)(r % B);
                if (B == 3) {
                    const double x = pos[3 * (uint64_t)i] - cx, y = pos[3 * (uint64_t)i + 1] - cy,
                                 z = pos[3 * (uint64_t)i + 2] - cz;
                    // columns: translations x, y, z, rotations about z, x, y
                    M[k][rr] = 1.0;
                    M[k][3] = rr == 0 ? -y : (rr == 1 ? x : 0.0);
                    M[k][4] = rr == 1 ? -z : (rr == 2 ? y : 0.0);
                    M[k][5] = rr == 0 ? z : (rr == 2 ? -x : 0.0);
                } else {
#pragma unroll
                    for (int c = 0; c < 6; ++c) M[k][c] = Bf[36 * (uint64_t)i + 6 * rr + c];
                }
            }
        }
        double R[6][6];
#pragma unroll
        for (int p = 0; p < 6; ++p)
#pragma unroll
            for (int c = 0; c < 6; ++c) R[p][c] = 0.0;
        double norm0[6];
#pragma unroll
        for (int c = 0; c < 6; ++c) {
            double t = 0.0;
#pragma unroll
            for (int k = 0; k < kTentRows; ++k) t += M[k][c] * M[k][c];
            norm0[c] = sqrt(warp_sum(t));
        }
#pragma unroll
        for (int c = 0; c < 6; ++c) {
#pragma unroll
            for (int pass = 0; pass < 2; ++pass)
#pragma unroll
                for (int p = 0; p < c; ++p) {
                    double t = 0.0;
#pragma unroll
                    for (int k = 0; k < kTentRows; ++k) t += M[k][p] * M[k][c];
                    t = warp_sum(t);
                    R[p][c] += t;
#pragma unroll
                    for (int k = 0; k < kTentRows; ++k) M[k][c] -= t * M[k][p];
                }
            double t = 0.0;
#pragma unroll
            for (int k = 0; k < kTentRows; ++k) t += M[k][c] * M[k][c];
            const double nrm = sqrt(warp_sum(t));
            const bool drop = nrm <= 1e-10 * norm0[c] || nrm == 0.0;
            R[c][c] = drop ? 0.0 : nrm;
            const double inv = drop ? 0.0 : 1.0 / nrm;
#pragma unroll
            for (int k = 0; k < kTentRows; ++k) M[k][c] *= inv;
        }
#pragma unroll
        for (int k = 0; k < kTentRows; ++k) {
            const uint32_t r = lane + 32 * k;
            if (r < rows) {
                const uint32_t i = anode[n0 + r / B];
                const int rr = (int)(r % B);
#pragma unroll
                for (int c = 0; c < 6; ++c) Q[((uint64_t)i * B + rr) * 6 + c] = (float)M[k][c];
            }
        }
        for (int v = lane; v < 36; v += 32) {
            double x = R[0][0];
#pragma unroll
            for (int u = 1; u < 36; ++u) x = v == u ? R[u / 6][u % 6] : x;
            Bc[36 * a + v] = x;
        }
    }
}

// Inverse of every 6x6 diagonal block (Gauss-Jordan with partial pivoting, FP64).
__global__ void k_block_inv6(const uint32_t *__restrict__ bptr, const uint32_t *__restrict__ bdiag,
                             const float *__restrict__ K, uint64_t nn, float *__restrict__ Dinv) {
    for (uint64_t I = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; I < nn; I += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t rb = bptr[I], deg = bptr[I + 1] - rb, d = bdiag[I] - rb;
        double a[6][12];
        for (int r = 0; r < 6; ++r)
            for (int c = 0; c < 6; ++c) {
                a[r][c] = (double)K[kidx6(rb, deg, d, 6 * r + c)];
                a[r][6 + c] = r == c ? 1.0 : 0.0;
            }
        bool ok = true;
        for (int c = 0; c < 6 && ok; ++c) {
            int p = c;
            for (int r = c + 1; r < 6; ++r)
                if (fabs(a[r][c]) > fabs(a[p][c])) p = r;
            if (a[p][c] == 0.0) {
                ok = false;
                break;
            }
            if (p != c)
                for (int k = 0; k < 12; ++k) {
                    const double t = a[c][k];
                    a[c][k] = a[p][k];
                    a[p][k] = t;
                }
            const double iv = 1.0 / a[c][c];
            for (int k = 0; k < 12; ++k) a[c][k] *= iv;
            for (int r = 0; r < 6; ++r)
                if (r != c) {
                    const double f = a[r][c];
                    if (f != 0.0)
                        for (int k = 0; k < 12; ++k) a[r][k] -= f * a[c][k];
                }
        }
        for (int r = 0; r < 6; ++r)
            for (int c = 0; c < 6; ++c) Dinv[36 * I + 6 * r + c] = ok ? (float)a[r][6 + c] : (r == c ? 1.f : 0.f);
    }
}

// ---------------------------------------------------------------------------------------------
// row products
// ---------------------------------------------------------------------------------------------

// (K x)_I for a 3x3-block row, x padded to 4 per node: returns the reduce_scatter3 layout
__device__ __forceinline__ float row3(const uint32_t *__restrict__ bcol, const float *__restrict__ K, uint32_t rb,
                                      uint32_t re, int lane, const float *__restrict__ x) {
    return bsr3_row_lanes(bcol, K, rb, re, lane, [&](uint64_t J, float &a, float &b, float &c) {
        NodeVec<float, 4>::load(x, J, a, b, c);
    });
}

// (K x)_I for a 6x6-block row, x padded to 8 per node: every lane ends with the 6 sums
__device__ __forceinline__ void row6(const uint32_t *__restrict__ bcol, const float *__restrict__ K, uint32_t rb,
                                     uint32_t re, int lane, const float *__restrict__ x, float (&a)[6]) {
    const uint32_t deg = re - rb;
#pragma unroll
    for (int k = 0; k < 6; ++k) a[k] = 0.f;
    for (uint32_t b0 = 0; b0 < deg; b0 += 32) {
        const uint32_t bl = b0 + lane;
        if (bl < deg) {
            const uint32_t J = __ldg(bcol + rb + bl);
            const float4 u = __ldg(reinterpret_cast<const float4 *>(x) + 2 * (uint64_t)J);
            const float4 w = __ldg(reinterpret_cast<const float4 *>(x) + 2 * (uint64_t)J + 1);
            const float xv[6] = {u.x, u.y, u.z, u.w, w.x, w.y};
#pragma unroll
            for (int r = 0; r < 6; ++r)
#pragma unroll
                for (int c = 0; c < 6; ++c) a[r] = fmaf(__ldg(K + kidx6(rb, deg, bl, 6 * r + c)), xv[c], a[r]);
        }
    }
#pragma unroll
    for (int k = 0; k < 6; ++k) a[k] = warp_sum(a[k]);
}

// ---------------------------------------------------------------------------------------------
// cycle kernels
// ---------------------------------------------------------------------------------------------

// res = r - K x (r == nullptr: res = -K x), warp per row; with D (6x6 levels), also the first
// smoothing step of a cycle on that residual, xpre = omega D^-1 res (padded 8)
template <int B>
__global__ void __launch_bounds__(kRowThreads)
    k_amg_res(const uint32_t *__restrict__ bptr, const uint32_t *__restrict__ bcol, const float *__restrict__ K,
              const float *__restrict__ x, const float *__restrict__ r, float *__restrict__ res, uint64_t nn,
              const PcgScalars *S, const float *__restrict__ D = nullptr, float omega = 0.f,
              float *__restrict__ xpre = nullptr) {
    pdl_wait_trigger();
    if (done(S)) return;
    const int lane = threadIdx.x & 31;
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t I = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; I < nn; I += nw) {
        if (B == 3) {
            const float a = row3(bcol, K, bptr[I], bptr[I + 1], lane, x);
            if ((lane & 7) == 0 && lane < 24) {
                const uint64_t i = 3 * I + (lane >> 3);
                res[i] = (r ? r[i] : 0.f) - a;
            }
        } else {
            float a[6];
            row6(bcol, K, bptr[I], bptr[I + 1], lane, x, a);
            if (lane < 6) {
                float v = a[0];
#pragma unroll
                for (int k = 1; k < 6; ++k) v = lane == k ? a[k] : v;
                const uint64_t i = 6 * I + lane;
                res[i] = (r ? r[i] : 0.f) - v;
                if (D) {
                    const float *Dr = D + 36 * I + 6 * lane;
                    float xp = 0.f;
#pragma unroll
                    for (int k = 0; k < 6; ++k) xp = fmaf(Dr[k], (r ? r[6 * I + k] : 0.f) - a[k], xp);
                    xpre[8 * I + lane] = omega * xp;
                }
            }
        }
    }
}

// Post-smoothing x_out = x + omega D^-1 (r - K x), warp per row.  With S_rz (level 0 inside the
// PCG) x_out is the PCG's z, and r.z is reduced: rz and beta are set (beta = rz / rz_old, or on a
// start rz / beta_den when beta_den > 0, else 0).
template <int B>
__global__ void __launch_bounds__(kRowThreads)
    k_amg_post(const uint32_t *__restrict__ bptr, const uint32_t *__restrict__ bcol, const float *__restrict__ K,
               const float *__restrict__ Dinv, const float *__restrict__ x, const float *__restrict__ r,
               float *__restrict__ xo, float omega, uint64_t nn, PcgScalars *S, bool with_rz, int start,
               double beta_den, double *partials) {
    pdl_wait_trigger();
    if (done(S)) return;
    constexpr int VS = B == 3 ? 4 : 8;
    const int lane = threadIdx.x & 31;
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    float rz = 0.f;
    for (uint64_t I = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; I < nn; I += nw) {
        float d[B];
        if (B == 3) {
            const float a = row3(bcol, K, bptr[I], bptr[I + 1], lane, x);
            d[0] = __shfl_sync(0xffffffffu, a, 0);
            d[1] = __shfl_sync(0xffffffffu, a, 8);
            d[2] = __shfl_sync(0xffffffffu, a, 16);
        } else {
            float a[6];
            row6(bcol, K, bptr[I], bptr[I + 1], lane, x, a);
#pragma unroll
            for (int k = 0; k < B; ++k) d[k] = a[k < 6 ? k : 0];
        }
#pragma unroll
        for (int k = 0; k < B; ++k) d[k] = r[(uint64_t)B * I + k] - d[k];
        if (lane < B) {
            const float *D = Dinv + (uint64_t)B * B * I + B * lane;
            float s = 0.f;
#pragma unroll
            for (int k = 0; k < B; ++k) s = fmaf(D[k], d[k], s);
            const float z = x[(uint64_t)VS * I + lane] + omega * s;
            xo[(uint64_t)VS * I + lane] = z;
            rz = fmaf(r[(uint64_t)B * I + lane], z, rz);
        }
    }
    if (!with_rz) return;
    const float t[1] = {rz};
    double out[1];
    if (grid_reduce_t<1, 0u>(t, partials, &S->cnt_d, out) && threadIdx.x == 0) {
        if (start) {
            S->beta = beta_den > 0.0 ? out[0] / beta_den : 0.0;
        } else {
            S->beta = out[0] / S->rz;
        }
        S->rz = out[0];
        if (!isfinite(out[0])) {
            S->status = LMTG_ERR_NAN;
            S->done = 1;
        }
    }
}

// rc = Q^T res per aggregate (warp per aggregate); with Dc, also the coarse level's first
// smoothing step xc = omega_c Dc^-1 rc (padded 8), which needs nothing but rc
template <int B>
__global__ void __launch_bounds__(kRowThreads)
    k_amg_restrict(const uint32_t *__restrict__ aptr, const uint32_t *__restrict__ anode, const float *__restrict__ Q,
                   const float *__restrict__ res, float *__restrict__ rc, uint64_t na, const float *__restrict__ Dc,
                   float omega_c, float *__restrict__ xc, const PcgScalars *S) {
    pdl_wait_trigger();
    if (done(S)) return;
    const int lane = threadIdx.x & 31;
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const int cc = lane >> 2;  // lane 4c ends with component c of the reduce-scatter
    const bool own = (lane & 3) == 0;
    for (uint64_t a = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; a < na; a += nw) {
        // the coarse block-Jacobi row, loaded before the products
        float d[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        if (Dc && own && cc < 6) {
#pragma unroll
            for (int k = 0; k < 6; ++k) d[k] = Dc[36 * a + 6 * cc + k];
        }
        float acc[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        for (uint32_t k = aptr[a] + lane; k < aptr[a + 1]; k += 32) {
            const uint32_t i = anode[k];
            // the node's prolongator rows as 8-byte pairs (B x 6 floats at 8-byte aligned offsets)
            const float2 *q2 = reinterpret_cast<const float2 *>(Q + (uint64_t)i * B * 6);
#pragma unroll
            for (int r = 0; r < B; ++r) {
                const float v = res[(uint64_t)B * i + r];
                const float2 q01 = q2[3 * r], q23 = q2[3 * r + 1], q45 = q2[3 * r + 2];
                acc[0] = fmaf(q01.x, v, acc[0]);
                acc[1] = fmaf(q01.y, v, acc[1]);
                acc[2] = fmaf(q23.x, v, acc[2]);
                acc[3] = fmaf(q23.y, v, acc[3]);
                acc[4] = fmaf(q45.x, v, acc[4]);
                acc[5] = fmaf(q45.y, v, acc[5]);
            }
        }
        const float t = reduce_scatter6(acc, lane);
        if (own && cc < 6) rc[6 * a + cc] = t;
        if (Dc) {
            float x = 0.f;
#pragma unroll
            for (int k = 0; k < 6; ++k) x = fmaf(d[k], __shfl_sync(0xffffffffu, t, 4 * k), x);
            if (own) xc[8 * a + cc] = cc < 6 ? omega_c * x : 0.f;  // padding too: whole 32-byte nodes
        }
    }
}

// x += Q (e + e2)[agg] per node (e, e2 with stride ES per coarse node; e2 may be null)
template <int B, int ES>
__global__ void k_amg_prolong(const uint32_t *__restrict__ agg, const float *__restrict__ Q, const float *__restrict__ e,
                              const float *__restrict__ e2, float *__restrict__ x, uint64_t nn, const PcgScalars *S) {
    pdl_wait_trigger();
    if (done(S)) return;
    constexpr int VS = B == 3 ? 4 : 8;
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < (uint64_t)B * nn;
         t += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t i = t / B;
        const int r = (int)(t - (uint64_t)B * i);
        const uint32_t a = agg[i];
        if (a == kNone) continue;
        const float2 *q2 = reinterpret_cast<const float2 *>(Q + (i * B + r) * 6);  // 8-byte aligned rows
        const float2 q01 = q2[0], q23 = q2[1], q45 = q2[2];
        const float q[6] = {q01.x, q01.y, q23.x, q23.y, q45.x, q45.y};
        const float *ev = e + (uint64_t)ES * a;
        float s = 0.f;
        if (e2) {
            const float *ev2 = e2 + (uint64_t)ES * a;
#pragma unroll
            for (int c = 0; c < 6; ++c) s = fmaf(q[c], ev[c] + ev2[c], s);
        } else {
#pragma unroll
            for (int c = 0; c < 6; ++c) s = fmaf(q[c], ev[c], s);
        }
        x[(uint64_t)VS * i + r] += kCoarseScale * s;
    }
}

// e = Cinv r on the coarsest level (warp per row)
__global__ void k_amg_dense(const float *__restrict__ Cinv, const float *__restrict__ r, float *__restrict__ e, int n,
                            const PcgScalars *S) {
    pdl_wait_trigger();
    if (done(S)) return;
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; row < n; row += nw) {
        float s = 0.f;
        for (int k = lane; k < n; k += 32) s = fmaf(Cinv[(uint64_t)row * n + k], r[k], s);
        s = warp_sum(s);
        if (lane == 0) e[row] = s;
    }
}

// 1 / |v| from the previous power step's |w|^2 (v is that w), 1 on the first step
__device__ __forceinline__ float power_scale(const double *prev) {
    if (!prev) return 1.f;
    const float p = (float)*prev;
    return p > 0.f ? rsqrtf(p) : 1.f;
}

// one power step for lambda_max(D^-1 K): w = D^-1 K v / |v| (v, w padded; |v|^2 is the previous
// step's |w|^2 in prev); |w|^2 and v.w reduced into out2
template <int B>
__global__ void __launch_bounds__(kRowThreads)
    k_amg_power(const uint32_t *__restrict__ bptr, const uint32_t *__restrict__ bcol, const float *__restrict__ K,
                const float *__restrict__ Dinv, const float *__restrict__ v, float *__restrict__ w, uint64_t nn,
                double *partials, unsigned *ticket, const double *prev, double *out2) {
    constexpr int VS = B == 3 ? 4 : 8;
    const int lane = threadIdx.x & 31;
    const float sc = power_scale(prev);
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    float ww = 0.f, vw = 0.f;
    for (uint64_t I = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; I < nn; I += nw) {
        float d[B];
        if (B == 3) {
            const float a = row3(bcol, K, bptr[I], bptr[I + 1], lane, v);
            d[0] = __shfl_sync(0xffffffffu, a, 0);
            d[1] = __shfl_sync(0xffffffffu, a, 8);
            d[2] = __shfl_sync(0xffffffffu, a, 16);
        } else {
            float a[6];
            row6(bcol, K, bptr[I], bptr[I + 1], lane, v, a);
#pragma unroll
            for (int k = 0; k < B; ++k) d[k] = a[k < 6 ? k : 0];
        }
        if (lane < B) {
            const float *D = Dinv + (uint64_t)B * B * I + B * lane;
            float s = 0.f;
#pragma unroll
            for (int k = 0; k < B; ++k) s = fmaf(D[k], d[k], s);
            s *= sc;
            w[(uint64_t)VS * I + lane] = s;
            ww = fmaf(s, s, ww);
            vw = fmaf(v[(uint64_t)VS * I + lane], s, vw);
        }
    }
    const float t[2] = {ww, vw};
    double out[2];
    if (grid_reduce_t<2, 0u>(t, partials, ticket, out) && threadIdx.x == 0) {
        out2[0] = out[0];
        out2[1] = out[1];
    }
}

// v = s w (padded vectors), or a deterministic pseudo-random start in [-1, 1) when w == nullptr
__global__ void k_amg_scale(float *__restrict__ v, const float *__restrict__ w, float s, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        if (w) {
            v[i] = s * w[i];
        } else {
            uint32_t h = (uint32_t)(i * 2654435761ull) ^ 0x9e3779b9u;
            h ^= h >> 16;
            h *= 0x7feb352du;
            h ^= h >> 15;
            v[i] = (float)(h & 0xffffff) * (2.0f / 16777216.0f) - 1.0f;
        }
    }
}

// Level-0 epilogues of the bulk-copy SpMV (spmv_bulk.cuh), which streams K32 at the HBM rate:
//   EpiRes   res = r - K x
//   EpiPost  z = x + omega D^-1 (r - K x), r.z reduced -> rz, beta (start: rz / beta_den or 0)
struct EpiRes {
    const float *r;
    float *res;
    static constexpr bool kReduce = false;
    struct Pre {
        float r;
    };
    __device__ __forceinline__ Pre pre(uint64_t I, int lane, const float *) const {
        return {((lane & 7) == 0 && lane < 24) ? r[3 * I + (lane >> 3)] : 0.f};
    }
    __device__ __forceinline__ void row(uint64_t I, float qi, int lane, const float *, float &, const Pre &pr) const {
        if ((lane & 7) == 0 && lane < 24) res[3 * I + (lane >> 3)] = pr.r - qi;
    }
    __device__ static unsigned *ticket(PcgScalars *S) { return &S->cnt_d; }
    __device__ void final(PcgScalars *, double) const {}
};

struct EpiPost {
    const float *r, *D;
    float *z;
    float omega;
    int start;
    double beta_den;
    static constexpr bool kReduce = true;
    // four registers per row: lane c < 3 holds x_c and row c of D^-1; lane 8c + 3 holds r_c
    // (its group's lanes hold the row sum's component c after the reduce-scatter).  Seven
    // registers per row (r, x and D on lanes 0-2) ran 2.5% slower; nine lanes each holding one
    // entry of D^-1 (two registers, more shuffles) 10% slower.
    struct Pre {
        float a, b, c, d;
    };
    __device__ __forceinline__ Pre pre(uint64_t I, int lane, const float *__restrict__ x) const {
        Pre p{0.f, 0.f, 0.f, 0.f};
        if (lane < 3) {
            const float *Dr = D + 9 * I + 3 * lane;
            p = {x[4 * I + lane], Dr[0], Dr[1], Dr[2]};
        } else if ((lane & 7) == 3 && lane < 24) {
            p.a = r[3 * I + (lane >> 3)];
        }
        return p;
    }
    __device__ __forceinline__ void row(uint64_t I, float qi, int lane, const float *, float &acc,
                                        const Pre &p) const {
        const float w = p.a - qi;  // r_c - (K x)_c on lane 8c + 3
        const float w0 = __shfl_sync(0xffffffffu, w, 3), w1 = __shfl_sync(0xffffffffu, w, 11),
                    w2 = __shfl_sync(0xffffffffu, w, 19);
        const float zc = p.a + omega * (p.b * w0 + p.c * w1 + p.d * w2);  // lanes 0-2
        const float zr = __shfl_sync(0xffffffffu, zc, (lane >> 3) & 3);   // z_c on lane 8c + 3
        if (lane < 3) z[4 * I + lane] = zc;
        else if (lane == 3) z[4 * I + 3] = 0.f;  // the padding too: whole 16-byte nodes, no partially written sectors
        if ((lane & 7) == 3 && lane < 24) acc = fmaf(p.a, zr, acc);
    }
    __device__ static unsigned *ticket(PcgScalars *S) { return &S->cnt_d; }
    __device__ void final(PcgScalars *S, double v) const {
        S->beta = start ? (beta_den > 0.0 ? v / beta_den : 0.0) : v / S->rz;
        S->rz = v;
        if (!isfinite(v)) {
            S->status = LMTG_ERR_NAN;
            S->done = 1;
        }
    }
};

//   EpiPower w = D^-1 K v / |v|, |w|^2 reduced into out (a power step for lambda_max, |v|^2 the
//            previous step's |w|^2 in prev; runs on the outer scalar slot, whose `done` stays 0)
struct EpiPower {
    const float *D;
    float *w;
    const double *prev;
    double *out;
    static constexpr bool kReduce = true;
    struct Pre {
        float d0, d1, d2;
    };
    __device__ __forceinline__ Pre pre(uint64_t I, int lane, const float *) const {
        Pre p{0.f, 0.f, 0.f};
        if (lane < 3) {
            const float *Dr = D + 9 * I + 3 * lane;
            p = {Dr[0], Dr[1], Dr[2]};
        }
        return p;
    }
    __device__ __forceinline__ void row(uint64_t I, float qi, int lane, const float *, float &acc,
                                        const Pre &p) const {
        const float v0 = __shfl_sync(0xffffffffu, qi, 0), v1 = __shfl_sync(0xffffffffu, qi, 8),
                    v2 = __shfl_sync(0xffffffffu, qi, 16);
        if (lane < 3) {
            const float wc = (p.d0 * v0 + p.d1 * v1 + p.d2 * v2) * power_scale(prev);
            w[4 * I + lane] = wc;
            acc = fmaf(wc, wc, acc);
        }
    }
    __device__ static unsigned *ticket(PcgScalars *S) { return &S->cnt_d; }
    __device__ void final(PcgScalars *, double v) const { *out = v; }
};

// one instance of the bulk kernel per (stage shape, epilogue); its resident grid is set up once
template <int kSt, int kCap, int kCons, bool kEF, int kMinB, class Epi>
struct Bulk0 {
    static int &grid() {
        static int g = 0;
        return g;
    }
    static void setup(lmtg_ctx *c) {
        if (grid()) return;
        constexpr size_t smem = bulk_smem_bytes<kSt, kCap>();
        auto fn = k_pcg_spmv_bulk<kSt, kCap, kCons, kEF, kMinB, Epi>;
        LMTG_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        int nb = 0;
        LMTG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, bulk_threads<kCons>(), smem));
        grid() = c->sm_count * (nb > 0 ? nb : 1);
    }
    static void launch(lmtg_ctx *c, const float *x, Epi epi, cudaStream_t s, PcgScalars *S) {
        k_pcg_spmv_bulk<kSt, kCap, kCons, kEF, kMinB, Epi><<<grid(), bulk_threads<kCons>(), bulk_smem_bytes<kSt, kCap>(), s>>>(
            c->bptr.p, c->bcol.p, c->K32.p, x, epi, c->nn, S, c->partials.p);
    }
};
// the shapes of the PCG's own SpMV: 4 CTAs per SM for rows of <= 32 blocks, 5 for wider rows
template <class Epi> using Bulk0N = Bulk0<2, 512, 8, true, 4, Epi>;
// (the smoothing and power epilogues keep 4 CTAs per SM for wide rows too: at 5 their prefetched
// operands spill)
template <class Epi> struct WideMinB { static constexpr int v = 5; };
template <> struct WideMinB<EpiPost> { static constexpr int v = 4; };
template <> struct WideMinB<EpiPower> { static constexpr int v = 4; };
template <class Epi> using Bulk0W = Bulk0<2, 512, 8, true, WideMinB<Epi>::v, Epi>;

// the level-0 residual / smoothing products follow the PCG's SpMV kind (1: 4 CTAs per SM,
// 2: 5, 0: the warp-row kernels k_amg_res<3> / k_amg_post<3>); set up outside graph capture
static void bulk0_setup(lmtg_ctx *c) {
    const int kind = spmv_kind_in_use(c);
    if (kind == 1) {
        Bulk0N<EpiRes>::setup(c);
        Bulk0N<EpiPost>::setup(c);
        Bulk0N<EpiPower>::setup(c);
    } else if (kind == 2) {
        Bulk0W<EpiRes>::setup(c);
        Bulk0W<EpiPost>::setup(c);
        Bulk0W<EpiPower>::setup(c);
    }
}

template <class Epi>
static void bulk0_launch(lmtg_ctx *c, const float *x, Epi epi, cudaStream_t s, PcgScalars *S = nullptr) {
    if (!S) S = c->scal.p;
    if (spmv_kind_in_use(c) == 2) Bulk0W<Epi>::launch(c, x, epi, s, S);
    else Bulk0N<Epi>::launch(c, x, epi, s, S);
}

// 6x6 levels of at least this many blocks stream their matrix with the bulk-copy kernel
// (amg_bulk6.cuh); smaller ones stay L2-resident and keep the warp-per-row kernels
constexpr uint64_t kBulk6MinBlocks = 1ull << 18;

template <class Epi>
struct Bulk6 {
    static constexpr int kSt = 3, kCap = 224, kCons = 8, kMinB = 2;
    static int &grid() {
        static int g = 0;
        return g;
    }
    static void setup(lmtg_ctx *c) {
        if (grid()) return;
        constexpr size_t smem = bulk6_smem_bytes<kSt, kCap>();
        auto fn = k_amg6_bulk<kSt, kCap, kCons, kMinB, Epi>;
        LMTG_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        int nb = 0;
        LMTG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, 32 * (kCons + 1), smem));
        grid() = c->sm_count * (nb > 0 ? nb : 1);
    }
    static void launch(const AmgLevel &L, const float *x, Epi epi, cudaStream_t s, PcgScalars *S) {
        launch_pdl(k_amg6_bulk<kSt, kCap, kCons, kMinB, Epi>, grid(), 32 * (kCons + 1), bulk6_smem_bytes<kSt, kCap>(),
                   s, L.bptr.p, L.bcol.p, L.K.p, x, epi, L.nn, S);
    }
};

// res = r - K x on a 6x6 level; with D also xpre = omega D^-1 res
static void level_res(lmtg_ctx *c, const AmgLevel &L, const float *x, const float *r, float *res, const float *D,
                      float omega, float *xpre, cudaStream_t s, PcgScalars *S) {
    if (L.bulk)
        Bulk6<Epi6Res>::launch(L, x, Epi6Res{r, res, D, omega, xpre}, s, S);
    else
        launch_pdl(k_amg_res<6>, grid_for(c, L.nn * 32, kRowThreads, 8), kRowThreads, 0, s, L.bptr.p, L.bcol.p,
                   L.K.p, x, r, res, L.nn, S, D, omega, xpre);
    c->launches += 1;
}

// xo = x + omega D^-1 (r - K x) on a 6x6 level
static void level_post(lmtg_ctx *c, const AmgLevel &L, const float *x, const float *r, float *xo, cudaStream_t s,
                       PcgScalars *S) {
    if (L.bulk)
        Bulk6<Epi6Post>::launch(L, x, Epi6Post{r, L.Dinv.p, x, xo, L.omega}, s, S);
    else
        launch_pdl(k_amg_post<6>, grid_for(c, L.nn * 32, kRowThreads, 8), kRowThreads, 0, s, L.bptr.p, L.bcol.p,
                   L.K.p, L.Dinv.p, x, r, xo, L.omega, L.nn, S, false, 0, 0.0, c->partials.p);
    c->launches += 1;
}

// ---------------------------------------------------------------------------------------------
// host structure setup
// ---------------------------------------------------------------------------------------------

// Host array without value-initialisation (the buffers here are filled completely, or only
// their filled part is read).
template <class T>
struct HBuf {
    std::unique_ptr<T[]> p;
    size_t n = 0;
    void alloc(size_t k) {
        p.reset(k ? new T[k] : nullptr);
        n = k;
    }
    T &operator[](size_t i) { return p[i]; }
    const T &operator[](size_t i) const { return p[i]; }
    T *data() { return p.get(); }
    const T *data() const { return p.get(); }
    size_t size() const { return n; }
};

struct HostLevel {
    int b = 3;
    uint64_t nn = 0;
    std::vector<uint32_t> bptr, bdiag;  // level pattern (level 0: copied from the device)
    HBuf<uint32_t> bcol;
};

static unsigned host_threads() { return std::max(1u, std::min(16u, std::thread::hardware_concurrency())); }

// runs f(a0, a1) on contiguous ranges of [0, n) in parallel
template <class F>
static void parallel_ranges(uint64_t n, F f) {
    const unsigned nt = host_threads();
    const uint64_t per = (n + nt - 1) / nt;
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nt; ++t) {
        const uint64_t a0 = t * per, a1 = std::min<uint64_t>(n, a0 + per);
        if (a0 < a1) th.emplace_back(f, a0, a1, t);
    }
    for (auto &t : th) t.join();
}

// standard aggregation of a node graph; skip[i] = node left out
static uint64_t aggregate(uint64_t nn, const std::vector<uint32_t> &bptr, const HBuf<uint32_t> &bcol,
                          const std::vector<uint8_t> &skip, std::vector<uint32_t> &agg) {
    agg.assign(nn, kNone);
    const uint32_t kFree = kNone, kSkip = kNone - 1;
    for (uint64_t i = 0; i < nn; ++i)
        if (!skip.empty() && skip[i]) agg[i] = kSkip;
    uint64_t na = 0;
    // pass 1: roots whose neighbours are all free
    for (uint64_t i = 0; i < nn; ++i) {
        if (agg[i] != kFree) continue;
        bool ok = true;
        for (uint32_t k = bptr[i]; k < bptr[i + 1] && ok; ++k) {
            const uint32_t j = bcol[k];
            if (j != i && agg[j] != kFree && agg[j] != kSkip) ok = false;
        }
        if (!ok) continue;
        for (uint32_t k = bptr[i]; k < bptr[i + 1]; ++k)
            if (agg[bcol[k]] == kFree) agg[bcol[k]] = (uint32_t)na;
        agg[i] = (uint32_t)na++;
    }
    // pass 2: leftovers join the neighbouring aggregate they have most links to (first on ties)
    std::vector<uint32_t> cand;
    std::vector<uint32_t> add(nn, kFree);
    for (uint64_t i = 0; i < nn; ++i) {
        if (agg[i] != kFree) continue;
        cand.clear();
        for (uint32_t k = bptr[i]; k < bptr[i + 1]; ++k) {
            const uint32_t a = agg[bcol[k]];
            if (a < kSkip) cand.push_back(a);
        }
        if (cand.empty()) continue;
        uint32_t best = cand[0];
        int bestn = 0;
        for (size_t u = 0; u < cand.size(); ++u) {
            int m = 0;
            for (size_t w = 0; w < cand.size(); ++w) m += cand[w] == cand[u];
            if (m > bestn) {
                bestn = m;
                best = cand[u];
            }
        }
        add[i] = best;
    }
    for (uint64_t i = 0; i < nn; ++i)
        if (add[i] != kFree) agg[i] = add[i];
    // pass 3: the rest, grouped around a free node with its free neighbours
    for (uint64_t i = 0; i < nn; ++i) {
        if (agg[i] != kFree) continue;
        for (uint32_t k = bptr[i]; k < bptr[i + 1]; ++k)
            if (agg[bcol[k]] == kFree) agg[bcol[k]] = (uint32_t)na;
        agg[i] = (uint32_t)na++;
    }
    for (uint64_t i = 0; i < nn; ++i)
        if (agg[i] == kSkip) agg[i] = kNone;
    return na;
}

// Tentative prolongator of one level: Q (b x 6 per aggregated node, row-major) and the coarse
// modes Bc (na x 6 x 6), from the level's modes mode(i, m) -> the b x 6 block of node i in m,
// orthonormalised per aggregate.
template <class ModeF>
static void tentative(int b, uint64_t na, const std::vector<uint32_t> &aptr, const std::vector<uint32_t> &anode,
                      ModeF mode, HBuf<float> &Q, std::vector<double> &Bc) {
    Bc.assign(na * 36, 0.0);
    parallel_ranges(na, [&](uint64_t a0, uint64_t a1, unsigned) {
        std::vector<double> M;
        for (uint64_t a = a0; a < a1; ++a) {
            const uint32_t n0 = aptr[a], m = aptr[a + 1] - n0;
            const size_t rows = (size_t)m * b;
            M.resize(rows * 6);
            for (uint32_t t = 0; t < m; ++t) mode(anode[n0 + t], &M[(size_t)t * b * 6]);
            double R[6][6] = {{0}};
            double norm0[6];
            for (int c = 0; c < 6; ++c) {
                double s = 0;
                for (size_t q = 0; q < rows; ++q) s += M[q * 6 + c] * M[q * 6 + c];
                norm0[c] = std::sqrt(s);
            }
            for (int c = 0; c < 6; ++c) {
                for (int pass = 0; pass < 2; ++pass)  // Gram-Schmidt, twice for orthogonality
                    for (int p = 0; p < c; ++p) {
                        double s = 0;
                        for (size_t q = 0; q < rows; ++q) s += M[q * 6 + p] * M[q * 6 + c];
                        R[p][c] += s;
                        for (size_t q = 0; q < rows; ++q) M[q * 6 + c] -= s * M[q * 6 + p];
                    }
                double s = 0;
                for (size_t q = 0; q < rows; ++q) s += M[q * 6 + c] * M[q * 6 + c];
                s = std::sqrt(s);
                if (s <= 1e-10 * norm0[c] || s == 0.0) {  // a mode the aggregate cannot carry
                    for (size_t q = 0; q < rows; ++q) M[q * 6 + c] = 0.0;
                    R[c][c] = 0.0;
                } else {
                    R[c][c] = s;
                    for (size_t q = 0; q < rows; ++q) M[q * 6 + c] /= s;
                }
            }
            for (uint32_t t = 0; t < m; ++t) {
                const uint32_t i = anode[n0 + t];
                for (int r = 0; r < b; ++r)
                    for (int c = 0; c < 6; ++c) Q[((size_t)i * b + r) * 6 + c] = (float)M[((size_t)t * b + r) * 6 + c];
            }
            for (int r = 0; r < 6; ++r)
                for (int c = 0; c < 6; ++c) Bc[a * 36 + r * 6 + c] = R[r][c];
        }
    });
}

// Coarse pattern: the sorted distinct aggregate columns of every aggregate row.
static void coarse_pattern(uint64_t na, const std::vector<uint32_t> &aptr, const std::vector<uint32_t> &anode,
                           const std::vector<uint32_t> &fbptr, const HBuf<uint32_t> &fbcol,
                           const std::vector<uint32_t> &agg, std::vector<uint32_t> &cbptr, HBuf<uint32_t> &cbcol,
                           std::vector<uint32_t> &cbdiag) {
    const unsigned nt = host_threads();
    std::vector<std::vector<uint32_t>> arena(nt);  // per thread: its aggregates' columns, in order
    std::vector<uint32_t> cdeg(na);
    std::vector<uint64_t> aoff(na);
    parallel_ranges(na, [&](uint64_t a0, uint64_t a1, unsigned t) {
        std::vector<uint32_t> &ar = arena[t];
        std::vector<uint32_t> mark(na, kNone), cols;
        for (uint64_t a = a0; a < a1; ++a) {
            cols.clear();
            for (uint32_t u = aptr[a]; u < aptr[a + 1]; ++u) {
                const uint32_t i = anode[u];
                for (uint32_t k = fbptr[i]; k < fbptr[i + 1]; ++k) {
                    const uint32_t J = agg[fbcol[k]];
                    if (J != kNone && mark[J] != (uint32_t)a) {
                        mark[J] = (uint32_t)a;
                        cols.push_back(J);
                    }
                }
            }
            std::sort(cols.begin(), cols.end());
            aoff[a] = ar.size();
            cdeg[a] = (uint32_t)cols.size();
            ar.insert(ar.end(), cols.begin(), cols.end());
        }
    });
    cbptr.assign(na + 1, 0);
    for (uint64_t a = 0; a < na; ++a) cbptr[a + 1] = cbptr[a] + cdeg[a];
    cbcol.alloc(cbptr[na] + 4);
    for (int k = 0; k < 4; ++k) cbcol[cbptr[na] + k] = 0;
    cbdiag.assign(na, 0);
    parallel_ranges(na, [&](uint64_t a0, uint64_t a1, unsigned t) {
        const std::vector<uint32_t> &ar = arena[t];
        for (uint64_t a = a0; a < a1; ++a)
            for (uint32_t u = 0; u < cdeg[a]; ++u) {
                const uint32_t J = ar[aoff[a] + u];
                cbcol[cbptr[a] + u] = J;
                if (J == a) cbdiag[a] = cbptr[a] + u;
            }
    });
}

template <class T>
static void upload(DBuf<T> &d, const std::vector<T> &h, cudaStream_t s) {
    d.alloc(h.size());
    if (!h.empty()) LMTG_CUDA(cudaMemcpyAsync(d.p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, s));
}
template <class T>
static void upload(DBuf<T> &d, const HBuf<T> &h, cudaStream_t s) {
    d.alloc(h.size());
    if (h.size()) LMTG_CUDA(cudaMemcpyAsync(d.p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, s));
}

}  // namespace

void amg_free(lmtg_ctx *c) {
    delete c->amg;
    c->amg = nullptr;
}

bool amg_applicable(const lmtg_ctx *c) {
    return c->precond == LMTG_PREC_AMG && c->nnu == 3 && !c->recal && c->nsys == 0 && c->n >= 3000 &&
           (c->elem_type == LMTG_ELEM_HEXA8 || c->elem_type == LMTG_ELEM_TETRA10);
}

// Structure of the hierarchy: aggregates, tentative prolongators, coarse patterns and gather lists.
static void amg_build_structure(lmtg_ctx *c) {
    Phase ph("lmtg.amg.structure");
    auto t0 = std::chrono::steady_clock::now();
    cudaStream_t s = c->stream;
    std::unique_ptr<AmgState> A(new AmgState());
    auto tp = t0;
    auto phase = [&](int k) {
        const auto now = std::chrono::steady_clock::now();
        A->phase_ms[k] += std::chrono::duration<double, std::milli>(now - tp).count();
        tp = now;
    };
    // level 0 pattern from the device
    HostLevel cur;
    cur.b = 3;
    cur.nn = c->nn;
    cur.bptr.resize(c->nn + 1);
    cur.bcol.alloc(c->nnzb);
    LMTG_CUDA(cudaMemcpyAsync(cur.bptr.data(), c->bptr.p, 4 * (c->nn + 1), cudaMemcpyDeviceToHost, s));
    LMTG_CUDA(cudaMemcpyAsync(cur.bcol.data(), c->bcol.p, 4 * c->nnzb, cudaMemcpyDeviceToHost, s));
    LMTG_CUDA(cudaStreamSynchronize(s));
    // nodes with a constraint stay out of the coarse spaces
    std::vector<uint8_t> skip(c->nn, 0);
    if (c->h_cdof.size() == c->nc)
        for (uint32_t d : c->h_cdof)
            if (d / 3 < c->nn) skip[d / 3] = 1;
    // level-0 modes: translations and rotations about the mesh centroid, per node
    double cen[3] = {0, 0, 0};
    for (uint64_t i = 0; i < c->nn; ++i)
        for (int d = 0; d < 3; ++d) cen[d] += c->h_pos[3 * i + d];
    for (int d = 0; d < 3; ++d) cen[d] /= (double)c->nn;
    const double *hp = c->h_pos.data();
    auto rigid_modes = [hp, cen](uint32_t i, double *m) {
        const double x = hp[3 * (size_t)i] - cen[0], y = hp[3 * (size_t)i + 1] - cen[1], z = hp[3 * (size_t)i + 2] - cen[2];
        // rows x, y, z; columns: translations x, y, z, rotations about z, x, y
        const double v[18] = {1, 0, 0, -y, 0, z,  //
                              0, 1, 0, x, -z, 0,  //
                              0, 0, 1, 0, y, -x};
        std::memcpy(m, v, sizeof(v));
    };
    DBuf<double> Bf_dev;  // modes of the current level (levels >= 1: 6 x 6 per node), on the device
    phase(0);
    for (int l = 0;; ++l) {
        std::unique_ptr<AmgLevel> L(new AmgLevel());
        L->b = cur.b;
        L->nn = cur.nn;
        L->nnzb = cur.bptr[cur.nn];
        const int VS = cur.b == 3 ? 4 : 8;
        L->xa.alloc(VS * cur.nn);
        L->xb.alloc(VS * cur.nn);
        L->res.alloc(cur.b * cur.nn + 4);
        if (l >= 1) {
            L->r2.alloc(cur.b * cur.nn + 4);
            L->xb2.alloc(8 * cur.nn);
        }
        if (l > 0) {
            L->r.alloc(cur.b * cur.nn + 4);
            upload(L->bptr, cur.bptr, s);
            upload(L->bcol, cur.bcol, s);
            upload(L->bdiag, cur.bdiag, s);
            L->K.alloc(36 * L->nnzb);
            L->Dinv.alloc(36 * cur.nn);
        }
        const bool coarsest = (uint64_t)cur.b * cur.nn <= kCoarsestDofs || l + 1 >= kMaxLevels;
        if (coarsest) {
            A->levels.push_back(std::move(L));
            break;
        }
        std::vector<uint32_t> agg;
        phase(4);
        const uint64_t na = aggregate(cur.nn, cur.bptr, cur.bcol, l == 0 ? skip : std::vector<uint8_t>(), agg);
        phase(1);
        if (na == 0 || na * 2 > cur.nn) {  // no useful coarsening left: this level is the coarsest
            A->levels.push_back(std::move(L));
            break;
        }
        std::vector<uint32_t> aptr(na + 1, 0), anode;
        for (uint64_t i = 0; i < cur.nn; ++i)
            if (agg[i] != kNone) ++aptr[agg[i] + 1];
        for (uint64_t a = 0; a < na; ++a) aptr[a + 1] += aptr[a];
        anode.resize(aptr[na]);
        {
            std::vector<uint32_t> pos(aptr.begin(), aptr.end() - 1);
            for (uint64_t i = 0; i < cur.nn; ++i)
                if (agg[i] != kNone) anode[pos[agg[i]]++] = (uint32_t)i;
        }
        // tentative prolongator: on the device (one warp per aggregate) when every aggregate fits
        // the kernel's 320 rows, else on the host
        uint32_t maxm = 0;
        for (uint64_t a = 0; a < na; ++a) maxm = std::max(maxm, aptr[a + 1] - aptr[a]);
        upload(L->aptr, aptr, s);
        upload(L->anode, anode, s);
        L->Q.alloc(cur.nn * cur.b * 6);  // rows of nodes in no aggregate are never read
        DBuf<double> Bc_dev;
        Bc_dev.alloc(na * 36);
        if ((uint64_t)maxm * cur.b <= 32u * kTentRows) {
            const int g = grid_for(c, na * 32, 128, 8);
            if (l == 0)
                k_tentative<3><<<g, 128, 0, s>>>(L->aptr.p, L->anode.p, na, c->pos.p, cen[0], cen[1], cen[2], nullptr,
                                                 L->Q.p, Bc_dev.p);
            else
                k_tentative<6><<<g, 128, 0, s>>>(L->aptr.p, L->anode.p, na, nullptr, 0, 0, 0, Bf_dev.p, L->Q.p,
                                                 Bc_dev.p);
            LMTG_CUDA(cudaGetLastError());
            c->launches += 1;
        } else {
            HBuf<float> Q;
            Q.alloc(cur.nn * cur.b * 6);
            std::vector<double> Bc;
            if (l == 0) {
                tentative(3, na, aptr, anode, rigid_modes, Q, Bc);
            } else {
                std::vector<double> Bf(36 * cur.nn);
                LMTG_CUDA(cudaMemcpyAsync(Bf.data(), Bf_dev.p, Bf.size() * 8, cudaMemcpyDeviceToHost, s));
                LMTG_CUDA(cudaStreamSynchronize(s));
                const double *bf = Bf.data();
                tentative(6, na, aptr, anode,
                          [bf](uint32_t i, double *m) { std::memcpy(m, bf + 36 * (size_t)i, 36 * sizeof(double)); }, Q,
                          Bc);
            }
            LMTG_CUDA(cudaMemcpyAsync(L->Q.p, Q.data(), Q.size() * sizeof(float), cudaMemcpyHostToDevice, s));
            LMTG_CUDA(cudaMemcpyAsync(Bc_dev.p, Bc.data(), Bc.size() * 8, cudaMemcpyHostToDevice, s));
            LMTG_CUDA(cudaStreamSynchronize(s));
        }
        phase(2);
        HostLevel nxt;
        nxt.b = 6;
        nxt.nn = na;
        coarse_pattern(na, aptr, anode, cur.bptr, cur.bcol, agg, nxt.bptr, nxt.bcol, nxt.bdiag);
        for (uint64_t a = 0; a < na; ++a) A->max_cdeg = std::max<uint32_t>(A->max_cdeg, nxt.bptr[a + 1] - nxt.bptr[a]);
        phase(3);
        L->nagg = na;
        upload(L->agg, agg, s);
        LMTG_CUDA(cudaStreamSynchronize(s));
        phase(4);
        A->levels.push_back(std::move(L));
        std::swap(Bf_dev.p, Bc_dev.p);
        std::swap(Bf_dev.n, Bc_dev.n);
        cur = std::move(nxt);
    }
    // coarsest dense buffers; no hierarchy (block Jacobi instead) with a single level or a
    // coarsest level too large for a dense inverse
    AmgLevel &C = *A->levels.back();
    const uint64_t nc = (uint64_t)C.b * C.nn;
    A->nc = (A->levels.size() > 1 && nc <= kDenseMaxDofs && A->max_cdeg <= (uint32_t)kGalMaxDeg) ? (int)nc : 0;
    if (A->nc) {
        // the functions' dynamic shared-memory ceilings are process-wide: set for the widest rows
        // any context may launch with, not this hierarchy's
        const int smem = (int)(kGalWarps * gal_warp_bytes(kGalMaxDeg));
        LMTG_CUDA(cudaFuncSetAttribute(k_galerkin<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        LMTG_CUDA(cudaFuncSetAttribute(k_galerkin<6>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        // large 6x6 levels (not the coarsest, which is solved densely) stream by bulk copies;
        // their rows hold at most kGalMaxDeg blocks, within a stage
        static_assert(kGalMaxDeg <= Bulk6<Epi6Res>::kCap, "a coarse row must fit a bulk-copy stage");
        for (size_t l = 1; l + 1 < A->levels.size(); ++l) {
            AmgLevel &L = *A->levels[l];
            L.bulk = L.nnzb >= kBulk6MinBlocks;
            if (L.bulk) {
                Bulk6<Epi6Res>::setup(c);
                Bulk6<Epi6Post>::setup(c);
            }
        }
    }
    if (A->nc) {
        A->Cinv.alloc((size_t)A->nc * A->nc);
        // coarse slots of every fine block, read by each numeric setup's Galerkin products
        for (size_t l = 0; l + 1 < A->levels.size(); ++l) {
            AmgLevel &F = *A->levels[l], &C = *A->levels[l + 1];
            F.gslot.alloc(F.nnzb);
            k_gal_slots<<<grid_for(c, F.nn * 32, kRowThreads, 8), kRowThreads, 0, s>>>(
                l == 0 ? c->bptr.p : F.bptr.p, l == 0 ? c->bcol.p : F.bcol.p, F.agg.p, F.nn, C.bptr.p, C.bcol.p,
                F.gslot.p);
            LMTG_CUDA(cudaGetLastError());
            c->launches += 1;
        }
    }
    A->power.alloc(2 * kPowerSteps * kMaxLevels);
    A->structure_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    c->amg = A.release();
}

// Numeric setup after an assembly: Galerkin products, block inverses, smoother weights, dense
// coarsest inverse.
static void amg_numeric(lmtg_ctx *c) {
    Phase ph("lmtg.amg.numeric");
    auto t0 = std::chrono::steady_clock::now();
    AmgState &A = *c->amg;
    cudaStream_t s = c->stream;
    const size_t nl = A.levels.size();
    // smoother weights: omega = 1 / theta of a degree-1 Chebyshev on [h/30, h], h = 1.2 lmax.
    // kPowerSteps power steps per level from a pseudo-random start, each normalising its input by
    // the previous step's norm on the device: every level's steps are queued back to back and
    // read once.  Level 0's steps need only its own matrix: they run on the auxiliary stream while
    // the Galerkin products build the coarse levels (the products' bandwidth-bound passes overlap
    // the Galerkin kernels' latency-bound ones); the coarser levels' steps follow the join.
    PcgScalars *o = c->scal.p + 1;
    auto power_steps = [&](size_t l, cudaStream_t st) {
        AmgLevel &L = *A.levels[l];
        const int VS = L.b == 3 ? 4 : 8;
        const uint64_t nv = (uint64_t)VS * L.nn;
        const uint32_t *bp = l == 0 ? c->bptr.p : L.bptr.p, *bc = l == 0 ? c->bcol.p : L.bcol.p;
        const float *K = l == 0 ? c->K32.p : L.K.p, *D = l == 0 ? c->Dinv32.p : L.Dinv.p;
        k_amg_scale<<<grid_for(c, nv, 256), 256, 0, st>>>(L.xa.p, nullptr, 1.f, nv);  // random start
        c->launches += 1;
        const bool bulk = l == 0 && spmv_kind_in_use(c) != 0;
        if (bulk) bulk0_setup(c);
        for (int it = 0; it < kPowerSteps; ++it) {
            float *v = (it & 1) ? L.xb.p : L.xa.p, *w = (it & 1) ? L.xa.p : L.xb.p;
            double *out2 = A.power.p + 2 * (kPowerSteps * l + it);
            const double *prev = it ? out2 - 2 : nullptr;
            const int g = grid_for(c, L.nn * 32, kRowThreads, 8);
            if (bulk)
                bulk0_launch(c, v, EpiPower{D, w, prev, out2}, st, o);
            else if (L.b == 3)
                k_amg_power<3><<<g, kRowThreads, 0, st>>>(bp, bc, K, D, v, w, L.nn, c->partials.p, &o->cnt_c, prev, out2);
            else
                k_amg_power<6><<<g, kRowThreads, 0, st>>>(bp, bc, K, D, v, w, L.nn, c->partials.p, &o->cnt_c, prev, out2);
            LMTG_CUDA(cudaGetLastError());
            c->launches += 1;
        }
    };
    if (!c->aux_stream) LMTG_CUDA(cudaStreamCreateWithFlags(&c->aux_stream, cudaStreamNonBlocking));
    // on an error between the fork and the join, nothing may leave with level 0's steps still
    // writing into the hierarchy's buffers
    struct AuxDrain {
        cudaStream_t st;
        ~AuxDrain() { cudaStreamSynchronize(st); }
    } drain{c->aux_stream};
    cudaEvent_t fork, join;
    LMTG_CUDA(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
    LMTG_CUDA(cudaEventCreateWithFlags(&join, cudaEventDisableTiming));
    LMTG_CUDA(cudaEventRecord(fork, s));
    LMTG_CUDA(cudaStreamWaitEvent(c->aux_stream, fork, 0));
    power_steps(0, c->aux_stream);
    LMTG_CUDA(cudaEventRecord(join, c->aux_stream));
    for (size_t l = 0; l + 1 < nl; ++l) {
        AmgLevel &F = *A.levels[l], &C = *A.levels[l + 1];
        const uint32_t *fbptr = l == 0 ? c->bptr.p : F.bptr.p;
        const uint32_t *fbcol = l == 0 ? c->bcol.p : F.bcol.p;
        const float *fK = l == 0 ? c->K32.p : F.K.p;
        const int cap = (int)((A.max_cdeg + 7) & ~7u);
        const size_t smem = kGalWarps * gal_warp_bytes(cap);
        const int g = grid_for(c, F.nagg * 32, 32 * kGalWarps, 8);
        if (F.b == 3)
            k_galerkin<3><<<g, 32 * kGalWarps, smem, s>>>(fbptr, fbcol, fK, F.agg.p, F.aptr.p, F.anode.p, F.Q.p, C.bptr.p,
                                                          C.bcol.p, F.gslot.p, F.nagg, cap, C.K.p);
        else
            k_galerkin<6><<<g, 32 * kGalWarps, smem, s>>>(fbptr, fbcol, fK, F.agg.p, F.aptr.p, F.anode.p, F.Q.p, C.bptr.p,
                                                          C.bcol.p, F.gslot.p, F.nagg, cap, C.K.p);
        k_block_inv6<<<grid_for(c, C.nn, 128), 128, 0, s>>>(C.bptr.p, C.bdiag.p, C.K.p, C.nn, C.Dinv.p);
        LMTG_CUDA(cudaGetLastError());
        c->launches += 2;
    }
    // the coarser levels' steps use the same partials and scalars as level 0's: after the join
    LMTG_CUDA(cudaStreamWaitEvent(s, join, 0));
    cudaEventDestroy(fork);
    cudaEventDestroy(join);
    for (size_t l = 1; l + 1 < nl; ++l) power_steps(l, s);
    {
        std::vector<double> h(2 * kPowerSteps * (nl - 1));
        LMTG_CUDA(cudaMemcpyAsync(h.data(), A.power.p, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, s));
        LMTG_CUDA(cudaStreamSynchronize(s));
        for (size_t l = 0; l + 1 < nl; ++l) {
            AmgLevel &L = *A.levels[l];
            const double lam = std::sqrt(std::max(0.0, h[2 * (kPowerSteps * l + kPowerSteps - 1)]));
            const double hi = 1.2 * lam, lo = hi / 30.0;
            L.lambda = lam;
            L.omega = lam > 0 ? (float)(2.0 / (hi + lo)) : 1.f;
        }
    }
    // dense inverse of the coarsest level (FP64 Gauss-Jordan with partial pivoting on the host;
    // a pivot below 1e-13 of the largest diagonal makes that unknown decoupled)
    {
        AmgLevel &C = *A.levels.back();
        const int n = A.nc;
        std::vector<uint32_t> bp(C.nn + 1), bc(C.nnzb);
        std::vector<float> K(36 * C.nnzb);
        LMTG_CUDA(cudaMemcpyAsync(bp.data(), C.bptr.p, 4 * bp.size(), cudaMemcpyDeviceToHost, s));
        LMTG_CUDA(cudaMemcpyAsync(bc.data(), C.bcol.p, 4 * bc.size(), cudaMemcpyDeviceToHost, s));
        LMTG_CUDA(cudaMemcpyAsync(K.data(), C.K.p, 4 * K.size(), cudaMemcpyDeviceToHost, s));
        LMTG_CUDA(cudaStreamSynchronize(s));
        std::vector<double> M((size_t)n * 2 * n, 0.0);
        const size_t w = 2 * (size_t)n;
        for (uint64_t I = 0; I < C.nn; ++I) {
            const uint32_t rb = bp[I], deg = bp[I + 1] - rb;
            for (uint32_t b = 0; b < deg; ++b)
                for (int r = 0; r < 6; ++r)
                    for (int cc = 0; cc < 6; ++cc)
                        M[(6 * I + r) * w + 6 * (size_t)bc[rb + b] + cc] = K[kidx6(rb, deg, b, 6 * r + cc)];
        }
        double dmax = 0;
        for (int i = 0; i < n; ++i) {
            dmax = std::max(dmax, std::fabs(M[i * w + i]));
            M[i * w + n + i] = 1.0;
        }
        std::vector<char> dead(n, 0);
        for (int col = 0; col < n; ++col) {
            int p = col;
            for (int r = col + 1; r < n; ++r)
                if (std::fabs(M[r * w + col]) > std::fabs(M[p * w + col])) p = r;
            if (std::fabs(M[p * w + col]) <= 1e-13 * dmax) {
                dead[col] = 1;
                continue;
            }
            if (p != col)
                for (size_t k = 0; k < w; ++k) std::swap(M[col * w + k], M[p * w + k]);
            const double iv = 1.0 / M[col * w + col];
            for (size_t k = 0; k < w; ++k) M[col * w + k] *= iv;
            for (int r = 0; r < n; ++r) {
                if (r == col) continue;
                const double f = M[r * w + col];
                if (f == 0.0) continue;
                for (size_t k = col; k < w; ++k) M[r * w + k] -= f * M[col * w + k];
            }
        }
        std::vector<float> Ci((size_t)n * n);
        for (int r = 0; r < n; ++r)
            for (int k = 0; k < n; ++k)
                Ci[(size_t)r * n + k] = (dead[r] || dead[k]) ? 0.f : (float)M[r * w + n + k];
        LMTG_CUDA(cudaMemcpyAsync(A.Cinv.p, Ci.data(), 4 * Ci.size(), cudaMemcpyHostToDevice, s));
        LMTG_CUDA(cudaStreamSynchronize(s));
    }
    A.version = c->mat_version;
    A.numeric_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

bool amg_prepare(lmtg_ctx *c) {
    if (!amg_applicable(c)) return false;
    LMTG_CHECK(c->have32, LMTG_ERR_STATE, "amg: FP32 matrix not assembled");
    if (!c->amg) amg_build_structure(c);
    if (c->amg->nc == 0) return false;
    if (c->amg->version != c->mat_version) amg_numeric(c);
    return true;
}

// Level-0 smoothing weight (the update kernel applies the first smoothing step itself).
float amg_omega0(const lmtg_ctx *c) { return c->amg->levels[0]->omega; }
float *amg_xa0(const lmtg_ctx *c) { return c->amg->levels[0]->xa.p; }

static void coarse_cycle(lmtg_ctx *c, AmgState &A, size_t l, const float *rhs, float *out, cudaStream_t s,
                         PcgScalars *S);

// Coarse correction of level l: level l+1's cycle on N.r (its first smoothing step already in
// N.xa, fused into the restriction).  On the dense coarsest one solve (e, packed 6); otherwise
// two cycles, the second on the residual N.r - K e the first leaves (e, e2 padded 8; a W-cycle
// below level 0, which with unsmoothed aggregation brings the multilevel cycle close to the
// two-level method's convergence).
static void coarse_correction(lmtg_ctx *c, AmgState &A, size_t l, cudaStream_t s, PcgScalars *S, float *&e,
                              float *&e2) {
    const size_t nl = A.levels.size();
    AmgLevel &N = *A.levels[l + 1];
    if (l + 2 == nl) {
        e = N.res.p;
        e2 = nullptr;
        coarse_cycle(c, A, l + 1, N.r.p, e, s, S);
        return;
    }
    e = N.xb.p;
    e2 = N.xb2.p;
    coarse_cycle(c, A, l + 1, N.r.p, e, s, S);
    level_res(c, N, e, N.r.p, N.r2.p, N.Dinv.p, N.omega, N.xa.p, s, S);
    coarse_cycle(c, A, l + 1, N.r2.p, e2, s, S);
}

// Cycle of a level l >= 1 on the right-hand side rhs (packed 6), its first smoothing step
// already in L.xa (fused into the caller's restriction or residual); the result goes to out
// (padded 8; packed 6 on the coarsest, the dense solve).
static void coarse_cycle(lmtg_ctx *c, AmgState &A, size_t l, const float *rhs, float *out, cudaStream_t s,
                         PcgScalars *S) {
    const size_t nl = A.levels.size();
    AmgLevel &L = *A.levels[l];
    if (l + 1 == nl) {
        launch_pdl(k_amg_dense, grid_for(c, (uint64_t)A.nc * 32, 256, 4), 256, 0, s, A.Cinv.p, rhs, out, A.nc, S);
        c->launches += 1;
        return;
    }
    AmgLevel &N = *A.levels[l + 1];
    const bool ncoarsest = l + 2 == nl;
    level_res(c, L, L.xa.p, rhs, L.res.p, nullptr, 0.f, nullptr, s, S);
    launch_pdl(k_amg_restrict<6>, grid_for(c, L.nagg * 32, kRowThreads, 8), kRowThreads, 0, s, L.aptr.p, L.anode.p,
               L.Q.p, L.res.p, N.r.p, L.nagg, ncoarsest ? nullptr : N.Dinv.p, N.omega, N.xa.p, S);
    float *e, *e2;
    coarse_correction(c, A, l, s, S, e, e2);
    const int tb = 256;
    if (ncoarsest)
        launch_pdl(k_amg_prolong<6, 6>, grid_for(c, 6 * L.nn, tb), tb, 0, s, L.agg.p, L.Q.p, e, nullptr, L.xa.p, L.nn,
                   S);
    else
        launch_pdl(k_amg_prolong<6, 8>, grid_for(c, 6 * L.nn, tb), tb, 0, s, L.agg.p, L.Q.p, e, e2, L.xa.p, L.nn, S);
    level_post(c, L, L.xa.p, rhs, out, s, S);
    c->launches += 2;
}

// The cycle after the update kernel: r (level-0 residual, packed) -> z (padded), rz and beta.
// ev (profiling only) receives events after the level-0 residual, the level-0 restriction, the
// coarse levels, the level-0 prolongation and the level-0 smoothing.
void amg_launch_cycle(lmtg_ctx *c, const float *r, float *z, cudaStream_t s, int start, double beta_den,
                      cudaEvent_t *ev) {
    AmgState &A = *c->amg;
    PcgScalars *S = c->scal.p;
    const size_t nl = A.levels.size();
    const bool warp_rows = spmv_kind_in_use(c) == 0;  // the level-0 products follow the PCG's kind
    if (!warp_rows) bulk0_setup(c);
    auto mark = [&](int k) {
        if (ev) LMTG_CUDA(cudaEventRecord(ev[k], s));
    };
    AmgLevel &L = *A.levels[0], &N = *A.levels[1];
    const int g0 = grid_for(c, L.nn * 32, kRowThreads, 8);
    const bool ncoarsest = nl == 2;
    // level 0: residual of the first smoothing step (written by the update kernel), restriction
    // with level 1's first smoothing step
    if (warp_rows) k_amg_res<3><<<g0, kRowThreads, 0, s>>>(c->bptr.p, c->bcol.p, c->K32.p, L.xa.p, r, L.res.p, L.nn, S);
    else bulk0_launch(c, L.xa.p, EpiRes{r, L.res.p}, s);
    mark(0);
    k_amg_restrict<3><<<grid_for(c, L.nagg * 32, kRowThreads, 8), kRowThreads, 0, s>>>(
        L.aptr.p, L.anode.p, L.Q.p, L.res.p, N.r.p, L.nagg, ncoarsest ? nullptr : N.Dinv.p, N.omega, N.xa.p, S);
    mark(1);
    c->launches += 2;
    float *e, *e2;
    coarse_correction(c, A, 0, s, S, e, e2);
    mark(2);
    const int tb = 256;
    if (ncoarsest)
        launch_pdl(k_amg_prolong<3, 6>, grid_for(c, 3 * L.nn, tb), tb, 0, s, L.agg.p, L.Q.p, e, nullptr, L.xa.p, L.nn,
                   S);
    else
        launch_pdl(k_amg_prolong<3, 8>, grid_for(c, 3 * L.nn, tb), tb, 0, s, L.agg.p, L.Q.p, e, e2, L.xa.p, L.nn, S);
    mark(3);
    if (warp_rows)
        k_amg_post<3><<<g0, kRowThreads, 0, s>>>(c->bptr.p, c->bcol.p, c->K32.p, c->Dinv32.p, L.xa.p, r, z, L.omega,
                                                 L.nn, S, true, start, beta_den, c->partials.p);
    else
        bulk0_launch(c, L.xa.p, EpiPost{r, c->Dinv32.p, z, L.omega, start, beta_den}, s);
    mark(4);
    c->launches += 2;
    LMTG_CUDA(cudaGetLastError());
}

void amg_info(const lmtg_ctx *c, int *levels, uint64_t *ndof, uint64_t *nnzb, double *omega, double *lambda,
              double *structure_ms, double *numeric_ms, double *phase_ms) {
    const AmgState *A = c->amg;
    const int nl = A ? (int)A->levels.size() : 0;
    if (levels) *levels = nl;
    for (int l = 0; l < kMaxLevels; ++l) {
        const AmgLevel *L = l < nl ? A->levels[l].get() : nullptr;
        if (ndof) ndof[l] = L ? L->b * L->nn : 0;
        if (nnzb) nnzb[l] = L ? L->nnzb : 0;
        if (omega) omega[l] = L ? L->omega : 0.0;
        if (lambda) lambda[l] = L ? L->lambda : 0.0;
    }
    if (structure_ms) *structure_ms = A ? A->structure_ms : 0.0;
    if (numeric_ms) *numeric_ms = A ? A->numeric_ms : 0.0;
    if (phase_ms)
        for (int k = 0; k < 5; ++k) phase_ms[k] = A ? A->phase_ms[k] : 0.0;
}

}  // namespace lmtg
