// batch.cu -- many independent meshes and up to four right-hand sides in one PCG.
//
// The reference solves one formulation at a time (FormulationAncestor::solve_system,
// include/formulation/formulation_ancestor.h:64; the CG loop of
// include/containers/conjugate_gradient.h:27-68) and a second right-hand side by a second solve.
// Here a batch of meshes is one block-diagonal system (the meshes concatenated, node ranges
// declared by lmtg_batch_set) and four right-hand sides share every pass over K: the SpMV
// multiplies each 3x3 block by four node vectors, so K is streamed once per iteration for all
// of them.  Every (system, rhs) pair keeps its own alpha, beta, iteration count and stopping
// test, and a system whose four pairs have stopped is skipped by every kernel.
//
// Vectors hold the four right-hand sides interleaved per node: v[12 I + 3 r + c] (node I,
// rhs r, component c), 48 bytes per node in FP32 (three aligned float4 gathers) and 96 in FP64.
//
// Work is cut into tiles of `tile_rows` consecutive node rows of one system.  A tile is one
// warp's work; the warps of persistent CTAs take tiles round-robin, so that the tiles of the
// systems still running stay spread over all SMs.  Each reduction goes per tile into a fixed
// slot; the last tile of a system to finish (a ticket per system) sums that system's slots in
// order and finalises the system's scalars.  Summation order is fixed (results are
// deterministic) and no kernel has a block-wide barrier.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <type_traits>
#include <vector>

#include "spmv_bulk.cuh"

namespace lmtg {

constexpr int kBR = 4;                // right-hand sides per node (zero-padded)
constexpr int kBV = 3 * kBR;          // values per node
constexpr int kBThreads = 256;
constexpr int kBWarps = kBThreads / 32;
constexpr int kBSlots = 8;            // partial slots per tile

struct BTile {
    uint32_t sys, row0, row1, pad;
};

struct BDev {
    const BTile *tiles;
    uint32_t ntiles;
    const uint32_t *groups;    // ngroups + 1: k_b_rows_bulk's unit g = tiles [groups[g], groups[g+1])
    uint32_t ngroups;          //   (consecutive tiles of one system)
    const uint32_t *sys_g;     // nsys + 1: the units of system m are [sys_g[m], sys_g[m+1])
    const uint32_t *tile_off;  // nsys + 1: tiles of system m are [tile_off[m], tile_off[m+1])
    double *partials;          // ntiles * kBSlots
    unsigned *tk;              // 4 ticket rows of nsys
    uint32_t nsys;
    // per (system, rhs) pair k = 4 m + r
    double *rz, *pq, *rr, *crit2, *beta, *beta_den, *scale, *out, *alpha;
    float *alpha32, *beta32;   // the same coefficients for FP32 runs (no FP64 work per entry)
    int *iter, *done, *status;
    int *sys_done;             // nsys
    int *n_active;             // systems with a pair still running
    int *fault;                // set (LMTG_ERR_TIMEOUT) when a bounded wait of a kernel gave up
    int maxit;
};

template <class T>
__device__ __forceinline__ T pair_coef(const double *d, const float *f, uint32_t k);
template <>
__device__ __forceinline__ double pair_coef<double>(const double *d, const float *, uint32_t k) { return d[k]; }
template <>
__device__ __forceinline__ float pair_coef<float>(const double *, const float *f, uint32_t k) { return f[k]; }

template <class T>
struct Node12;
template <>
struct Node12<float> {
    static __device__ __forceinline__ void load(const float *__restrict__ v, uint64_t J, float (&x)[kBV]) {
        const float4 *q = reinterpret_cast<const float4 *>(v) + 3 * J;
        const float4 a = __ldg(q), b = __ldg(q + 1), c = __ldg(q + 2);
        x[0] = a.x; x[1] = a.y; x[2] = a.z; x[3] = a.w;
        x[4] = b.x; x[5] = b.y; x[6] = b.z; x[7] = b.w;
        x[8] = c.x; x[9] = c.y; x[10] = c.z; x[11] = c.w;
    }
};
template <>
struct Node12<double> {
    static __device__ __forceinline__ void load(const double *__restrict__ v, uint64_t J, double (&x)[kBV]) {
        const double2 *q = reinterpret_cast<const double2 *>(v) + 6 * J;
#pragma unroll
        for (int i = 0; i < 6; ++i) {
            const double2 a = __ldg(q + i);
            x[2 * i] = a.x;
            x[2 * i + 1] = a.y;
        }
    }
};

// Row I of K times the four node vectors of x, any number of blocks: lane L (even, L < 24)
// returns the value of index v = L >> 1 (rhs v / 3, component v % 3).
template <class T>
__device__ __forceinline__ T brow(const uint32_t *__restrict__ bcol, const T *__restrict__ K, uint32_t rb,
                                  uint32_t re, const T *__restrict__ x, int lane) {
    const uint32_t deg = re - rb;
    T a[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) a[i] = (T)0;
    for (uint32_t b0 = 0; b0 < deg; b0 += 32) {
        const uint32_t bl = b0 + lane;
        if (bl < deg) {
            T m[9];
#pragma unroll
            for (int k = 0; k < 9; ++k) m[k] = __ldcs(K + kidx(rb, deg, bl, k));
            T xv[kBV];
            Node12<T>::load(x, __ldcs(bcol + rb + bl), xv);
#pragma unroll
            for (int r = 0; r < kBR; ++r)
                block_fma(m, xv[3 * r], xv[3 * r + 1], xv[3 * r + 2], a[3 * r], a[3 * r + 1], a[3 * r + 2]);
        }
    }
    return reduce_scatter16(a, lane);
}

// The row's first 32 blocks for one lane: the 9 planar values and the column.
template <class T>
struct RowLd {
    T m[9];
    uint32_t j;
};
template <class T>
__device__ __forceinline__ void row_load(const uint32_t *__restrict__ bptr, const uint32_t *__restrict__ bcol,
                                         const T *__restrict__ K, uint32_t I, int lane, RowLd<T> &R,
                                         uint32_t &rb, uint32_t &deg) {
    rb = __ldg(bptr + I);
    deg = __ldg(bptr + I + 1) - rb;
    const bool on = (uint32_t)lane < deg;
#pragma unroll
    for (int k = 0; k < 9; ++k) R.m[k] = on ? __ldcs(K + kidx(rb, deg, lane, k)) : (T)0;
    R.j = on ? __ldcs(bcol + rb + lane) : 0u;  // streamed once: keep L1 for the gathers
}

// Sum of the four products of a row whose blocks fit the warp (deg <= 32).
template <class T>
__device__ __forceinline__ T row_fast(const RowLd<T> &R, bool on, const T *__restrict__ x, int lane) {
    T a[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) a[i] = (T)0;
    if (on) {
        T xv[kBV];
        Node12<T>::load(x, R.j, xv);
#pragma unroll
        for (int r = 0; r < kBR; ++r)
            block_fma(R.m, xv[3 * r], xv[3 * r + 1], xv[3 * r + 2], a[3 * r], a[3 * r + 1], a[3 * r + 2]);
    }
    return reduce_scatter16(a, lane);
}

__device__ __forceinline__ uint32_t warp_id() { return (blockIdx.x * blockDim.x + threadIdx.x) >> 5; }
__device__ __forceinline__ uint32_t warp_count() { return (gridDim.x * blockDim.x) >> 5; }

template <int N>
__device__ __forceinline__ double pick(const double (&a)[N], int i) {
    double r = a[0];
#pragma unroll
    for (int k = 1; k < N; ++k) r = i == k ? a[k] : r;
    return r;
}

// Tile totals (v, the same in every lane) -> system totals.  Returns true in every lane of
// the warp that finished the system's last tile, with the system totals in tot (every lane).
template <int NV>
__device__ __forceinline__ bool warp_commit(const BDev &B, uint32_t tile, uint32_t sys, const double (&v)[NV],
                                            unsigned *ticket, double (&tot)[NV]) {
    const int lane = threadIdx.x & 31;
    const uint32_t t0 = B.tile_off[sys], t1 = B.tile_off[sys + 1];
    unsigned t = 0;
    if (lane == 0) {
#pragma unroll
        for (int i = 0; i < NV; ++i) B.partials[(size_t)tile * kBSlots + i] = v[i];
        __threadfence();
        t = atomicInc(ticket + sys, t1 - t0 - 1);  // wraps to 0 for the next launch
    }
    t = __shfl_sync(0xffffffffu, t, 0);
    if (t != t1 - t0 - 1) return false;
    __threadfence();
#pragma unroll
    for (int i = 0; i < NV; ++i) {
        double x = 0.0;
        for (uint32_t tt = t0 + lane; tt < t1; tt += 32) x += __ldcg(B.partials + (size_t)tt * kBSlots + i);
        tot[i] = warp_sum(x);
    }
    return true;
}

// Per-rhs warp totals of a value held by lanes of equal (lane & 3) -> v[off + r] in every lane.
template <class T, int NV>
__device__ __forceinline__ void rhs_totals(T x, double (&v)[NV], int off) {
    x += __shfl_xor_sync(0xffffffffu, x, 4);
    x += __shfl_xor_sync(0xffffffffu, x, 8);
    x += __shfl_xor_sync(0xffffffffu, x, 16);
#pragma unroll
    for (int r = 0; r < kBR; ++r) v[off + r] = (double)__shfl_sync(0xffffffffu, x, r);
}

// kMode 0: q = K p and p.q per pair (-> pq, alpha = rz / pq).  kMode 1: r = b - K x and r.r per
// pair (-> rr), every system.  kPipe 1: the warp loads its next row's values and columns while
// the current row's gathers and products run.
template <class T, int kMode, int kPipe>
__global__ void __launch_bounds__(kBThreads)
    k_b_rows(BDev B, const uint32_t *__restrict__ bptr, const uint32_t *__restrict__ bcol,
             const T *__restrict__ K, const T *__restrict__ x, const T *__restrict__ b, T *__restrict__ y) {
    if (kMode == 0 && *(volatile int *)B.n_active == 0) return;
    const int lane = threadIdx.x & 31;
    const int v = lane >> 1;
    const bool writer = (lane & 1) == 0 && v < kBV;
    const int my_r = writer ? v / 3 : -1;
    for (uint32_t tile = warp_id(); tile < B.ntiles; tile += warp_count()) {
        const BTile t = B.tiles[tile];
        // sys_done changes only after all of a system's tiles are done: a plain read is uniform
        if (kMode == 0 && B.sys_done[t.sys]) continue;
        T acc = (T)0;
        auto finish = [&](uint32_t I, T val) {
            if (writer) {
                const uint64_t i = (uint64_t)kBV * I + v;
                if (kMode == 0) {
                    y[i] = val;
                    acc = fma(x[i], val, acc);
                } else {
                    const T ri = b[i] - val;
                    y[i] = ri;
                    acc = fma(ri, ri, acc);
                }
            }
        };
        if (kPipe) {
            RowLd<T> cur;
            uint32_t rb = 0, deg = 0;
            row_load(bptr, bcol, K, t.row0, lane, cur, rb, deg);
            for (uint32_t I = t.row0; I < t.row1; ++I) {
                RowLd<T> nxt;
                uint32_t rb2 = 0, deg2 = 0;
                if (I + 1 < t.row1) row_load(bptr, bcol, K, I + 1, lane, nxt, rb2, deg2);
                const T val = deg <= 32 ? row_fast(cur, (uint32_t)lane < deg, x, lane)
                                        : brow(bcol, K, rb, rb + deg, x, lane);
                finish(I, val);
                cur = nxt;
                rb = rb2;
                deg = deg2;
            }
        } else {
            for (uint32_t I = t.row0; I < t.row1; ++I) finish(I, brow(bcol, K, bptr[I], bptr[I + 1], x, lane));
        }
        double s[kBR];
#pragma unroll
        for (int r = 0; r < kBR; ++r) s[r] = (double)warp_sum(my_r == r ? acc : (T)0);
        double tot[kBR];
        if (warp_commit<kBR>(B, tile, t.sys, s, B.tk + (uint64_t)kMode * B.nsys, tot) && lane < kBR) {
            const uint32_t k = kBR * t.sys + lane;
            const double val = pick(tot, lane);
            if (kMode == 0) {
                B.pq[k] = val;
                const double al = B.rz[k] / (val + (val == 0.0 ? 1.0 : 0.0));
                B.alpha[k] = al;
                B.alpha32[k] = (float)al;
            } else {
                B.rr[k] = val;
            }
        }
    }
}

// q = K p and p.q per pair (kMode 0 of k_b_rows) with the matrix streamed through shared memory
// by bulk copies (TMA): CTAs take tiles round-robin; one producer warp copies the values and
// column indices of up to 16 rows of the CTA's current tile per stage into a ring of kStages
// stages (evict-first L2 policy), eight consumer warps take two rows each (a half-warp per
// row, two blocks per lane, so that the 16-value reduce-scatter of a row runs over 16 lanes
// and serves two rows at once: 0.84 -> 0.76 ms at 256 cubes), read their blocks from shared
// memory, release the stage and gather the four right-hand sides.  At the last
// stage of a CTA unit (consecutive tiles of one system) each consumer warp commits its per-rhs
// partials to its own slot of the unit; the system's last commit sums the slots in a fixed
// order.  Every wait is bounded; one that
// gives up sets *B.fault.
constexpr int kBBulkCons = 8;
constexpr int kBBulkThreads = 32 * (kBBulkCons + 1);
constexpr int kBTileSlots = kBBulkCons * kBR;  // partial slots per tile (>= kBSlots)
static_assert(kBTileSlots >= kBSlots, "partials hold kBSlots values per tile");

// warp_commit for a CTA unit shared by kBBulkCons warps: warp w stores its per-rhs totals of
// unit g in slot (g, w); the last of the system's warps to commit sums all of the system's
// slots in order.
__device__ __forceinline__ bool warp_commit_w(const BDev &B, uint32_t g, uint32_t sys, int w,
                                              const double (&v)[kBR], unsigned *ticket, double (&tot)[kBR]) {
    const int lane = threadIdx.x & 31;
    const uint32_t t0 = B.sys_g[sys], t1 = B.sys_g[sys + 1];
    const uint32_t nslot = (t1 - t0) * kBBulkCons;
    unsigned t = 0;
    if (lane == 0) {
#pragma unroll
        for (int i = 0; i < kBR; ++i) B.partials[((size_t)g * kBBulkCons + w) * kBR + i] = v[i];
        __threadfence();
        t = atomicInc(ticket + sys, nslot - 1);  // wraps to 0 for the next launch
    }
    t = __shfl_sync(0xffffffffu, t, 0);
    if (t != nslot - 1) return false;
    __threadfence();
#pragma unroll
    for (int i = 0; i < kBR; ++i) {
        double x = 0.0;
        for (uint64_t sl = (uint64_t)t0 * kBBulkCons + lane; sl < (uint64_t)t1 * kBBulkCons; sl += 32)
            x += __ldcg(B.partials + sl * kBR + i);
        tot[i] = warp_sum(x);
    }
    return true;
}

template <int kStages, int kCap, int kMinB>
__global__ void __launch_bounds__(kBBulkThreads, kMinB)
    k_b_rows_bulk(BDev B, const uint32_t *__restrict__ bptr, const uint32_t *__restrict__ bcol,
                  const float *__restrict__ K, const float *__restrict__ x, float *__restrict__ y) {
    using St = BulkStage<kCap>;
    constexpr int kRows = 2 * kBBulkCons;
    if (*(volatile int *)B.n_active == 0) return;
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ uint64_t full[kStages], empty[kStages];
    __shared__ uint64_t meta[kStages][4];  // g0, g1, first value, first column
    __shared__ uint32_t mtile[kStages][2];  // tile, 1 = last stage of the tile
    __shared__ uint32_t sbp[kStages][kRows + 1];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int i = 0; i < kStages; ++i) {
            bulk::mbar_init(&full[i], 1);
            bulk::mbar_init(&empty[i], kBBulkCons);
        }
        bulk::fence_barrier_init();
    }
    __syncthreads();
    if (warp == kBBulkCons) {
        // ---------------- producer ----------------
        uint32_t k = 0;
        bool failed = false;
        auto next_slot = [&](int slot) -> bool {
            if (k < (uint32_t)kStages) return true;
            const bool ok = bulk::mbar_wait(&empty[slot], ((k / kStages) - 1) & 1u);
            return __all_sync(0xffffffffu, ok);
        };
        for (uint32_t tile = 0, g = blockIdx.x, gcur = 0, tile_end = 0; !failed; ++tile) {
            if (tile >= tile_end) {  // next unit of this CTA
                if (g >= B.ngroups) break;
                tile = B.groups[g];
                tile_end = B.groups[g + 1];
                gcur = g;
                g += gridDim.x;
            }
            const BTile t = B.tiles[tile];
            if (B.sys_done[t.sys]) {  // uniform for the whole launch; a unit is one system
                tile = tile_end - 1;
                continue;
            }
            uint64_t g0 = t.row0;
            uint32_t b0 = bptr[g0];
            while (g0 < t.row1) {
                const int slot = k % kStages;
                if (!next_slot(slot)) {
                    failed = true;
                    break;
                }
                const uint64_t gi = g0 + 1 + lane;
                const bool in = lane < kRows && gi <= t.row1;
                const uint32_t bi = in ? bptr[gi] : 0u;
                const unsigned fits = __ballot_sync(0xffffffffu, in && bi - b0 <= (uint32_t)kCap);
                const int nrows = __popc(fits);
                if (nrows == 0) {
                    failed = true;
                    break;
                }
                const uint32_t b1 = __shfl_sync(0xffffffffu, bi, nrows - 1);
                if (lane < nrows) sbp[slot][lane + 1] = bi;
                if (lane == 0) sbp[slot][0] = b0;
                __syncwarp();
                if (lane == 0) {
                    const uint64_t kb0 = (36ull * b0) & ~15ull, kb1 = (36ull * b1 + 15ull) & ~15ull;
                    const uint64_t cb0 = (4ull * b0) & ~15ull, cb1 = (4ull * b1 + 15ull) & ~15ull;
                    meta[slot][0] = g0;
                    meta[slot][1] = g0 + nrows;
                    meta[slot][2] = kb0 / 4;
                    meta[slot][3] = cb0 / 4;
                    mtile[slot][0] = gcur;  // the unit; 1 = its last stage
                    mtile[slot][1] = (g0 + nrows == t.row1 && tile + 1 == tile_end) ? 1u : 0u;
                    unsigned char *dst = smem + (size_t)slot * St::kBytes;
                    const uint64_t pol = bulk::policy_evict_first();
                    __threadfence_block();
                    bulk::mbar_arrive_expect_tx(&full[slot], (uint32_t)((kb1 - kb0) + (cb1 - cb0)));
                    bulk::copy_g2s_hint(dst, reinterpret_cast<const unsigned char *>(K) + kb0, (uint32_t)(kb1 - kb0),
                                        &full[slot], pol);
                    bulk::copy_g2s_hint(dst + St::kKBytes, reinterpret_cast<const unsigned char *>(bcol) + cb0,
                                        (uint32_t)(cb1 - cb0), &full[slot], pol);
                }
                g0 += nrows;
                b0 = b1;
                ++k;
            }
        }
        uint32_t nissued = k;  // stages whose full barrier got its arrival
        if (!failed) {
            const int slot = k % kStages;
            if (next_slot(slot)) {
                if (lane == 0) {  // sentinel: no rows
                    meta[slot][0] = 0;
                    meta[slot][1] = 0;
                    bulk::mbar_arrive(&full[slot]);
                }
                nissued = k + 1;
            } else {
                failed = true;
            }
        }
        if (lane == 0) {
            if (failed) atomicExch(B.fault, LMTG_ERR_TIMEOUT);
            // leave only with no copy in flight: the last stage issued on each slot (complete at
            // once when the consumers took every stage)
            const uint32_t first = nissued > (uint32_t)kStages ? nissued - kStages : 0u;
            for (uint32_t s2 = first; s2 < nissued; ++s2) bulk::mbar_wait(&full[s2 % kStages], (s2 / kStages) & 1u);
        }
    } else {
        // ---------------- consumers ----------------
        // a half-warp per row: lanes 0-15 take row I0, lanes 16-31 row I0 + 1; a lane takes the
        // row's blocks hl, hl + 16 (and further chunks of 16 for wider rows)
        const int half = lane >> 4, hl = lane & 15;
        const bool writer = hl < kBV;  // holds value hl (rhs hl / 3, component hl % 3) of its row
        const int my_r = writer ? hl / 3 : -1;
        float acc = 0.f;
        for (uint32_t k = 0;; ++k) {
            const int slot = k % kStages;
            const bool ok = bulk::mbar_wait(&full[slot], (k / kStages) & 1u);
            if (!__all_sync(0xffffffffu, ok)) {
                if (lane == 0) atomicExch(B.fault, LMTG_ERR_TIMEOUT);
                break;
            }
            const uint64_t g0 = meta[slot][0], g1 = meta[slot][1];
            if (g0 == g1) break;
            const uint32_t unit = mtile[slot][0];
            const bool last = mtile[slot][1] != 0;
            const float *sK = reinterpret_cast<const float *>(smem + (size_t)slot * St::kBytes);
            const uint32_t *sC = reinterpret_cast<const uint32_t *>(smem + (size_t)slot * St::kBytes + St::kKBytes);
            const uint64_t kbase = meta[slot][2], cbase = meta[slot][3];
            const uint64_t Ir = g0 + 2 * warp + half;
            const bool rowon = Ir < g1;
            const uint32_t rb = rowon ? sbp[slot][Ir - g0] : 0u, d = rowon ? sbp[slot][Ir - g0 + 1] - rb : 0u;
            const uint32_t dmax = max(d, __shfl_xor_sync(0xffffffffu, d, 16));
            float a[16];
#pragma unroll
            for (int i = 0; i < 16; ++i) a[i] = 0.f;
            if (dmax <= 32) {
                // the lane's two blocks into registers, then the stage goes back
                float m0[9], m1[9];
                const bool on0 = (uint32_t)hl < d, on1 = (uint32_t)hl + 16 < d;
#pragma unroll
                for (int c = 0; c < 9; ++c) {
                    m0[c] = on0 ? sK[kidx(rb, d, hl, c) - kbase] : 0.f;
                    m1[c] = on1 ? sK[kidx(rb, d, hl + 16, c) - kbase] : 0.f;
                }
                const uint32_t j0 = on0 ? sC[rb + hl - cbase] : 0u, j1 = on1 ? sC[rb + hl + 16 - cbase] : 0u;
                __syncwarp();
                if (lane == 0) bulk::mbar_arrive(&empty[slot]);
                if (on0) {
                    float xv[kBV];
                    Node12<float>::load(x, j0, xv);
#pragma unroll
                    for (int q4 = 0; q4 < kBR; ++q4)
                        block_fma(m0, xv[3 * q4], xv[3 * q4 + 1], xv[3 * q4 + 2], a[3 * q4], a[3 * q4 + 1], a[3 * q4 + 2]);
                }
                if (on1) {
                    float xv[kBV];
                    Node12<float>::load(x, j1, xv);
#pragma unroll
                    for (int q4 = 0; q4 < kBR; ++q4)
                        block_fma(m1, xv[3 * q4], xv[3 * q4 + 1], xv[3 * q4 + 2], a[3 * q4], a[3 * q4 + 1], a[3 * q4 + 2]);
                }
            } else {
                for (uint32_t c0 = 0; c0 < dmax; c0 += 16) {
                    const uint32_t bl = c0 + hl;
                    if (bl < d) {
                        float m[9];
#pragma unroll
                        for (int c = 0; c < 9; ++c) m[c] = sK[kidx(rb, d, bl, c) - kbase];
                        float xv[kBV];
                        Node12<float>::load(x, sC[rb + bl - cbase], xv);
#pragma unroll
                        for (int q4 = 0; q4 < kBR; ++q4)
                            block_fma(m, xv[3 * q4], xv[3 * q4 + 1], xv[3 * q4 + 2], a[3 * q4], a[3 * q4 + 1], a[3 * q4 + 2]);
                    }
                }
                __syncwarp();
                if (lane == 0) bulk::mbar_arrive(&empty[slot]);
            }
            // reduce-scatter of the 16 sums (12 used) over each half-warp: lane hl gets value hl
#pragma unroll
            for (int s2 = 0; s2 < 4; ++s2) {
                const int h = 8 >> s2;
                const bool hi = (hl & h) != 0;
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    if (i < h) {
                        const float send = hi ? a[i] : a[i + h];
                        const float keep = hi ? a[i + h] : a[i];
                        a[i] = keep + __shfl_xor_sync(0xffffffffu, send, h);
                    }
                }
            }
            if (writer && rowon) {
                const uint64_t i = (uint64_t)kBV * Ir + hl;
                y[i] = a[0];
                acc = fmaf(x[i], a[0], acc);
            }
            if (last) {
                // this warp's per-rhs totals of the unit, committed without a CTA barrier
                const BTile t = B.tiles[B.groups[unit]];
                double sv[kBR], tot[kBR];
#pragma unroll
                for (int r = 0; r < kBR; ++r) sv[r] = (double)warp_sum(my_r == r ? acc : 0.f);
                acc = 0.f;
                if (warp_commit_w(B, unit, t.sys, warp, sv, B.tk, tot) && lane < kBR) {
                    const uint32_t kk = kBR * t.sys + lane;
                    const double val = pick(tot, lane);
                    B.pq[kk] = val;
                    const double al = B.rz[kk] / (val + (val == 0.0 ? 1.0 : 0.0));
                    B.alpha[kk] = al;
                    B.alpha32[kk] = (float)al;
                }
            }
        }
    }
}

// Lane <-> (node, rhs) of a warp tile: the rhs is lane & 3 for the whole kernel.
// The pair (system, rhs) of a lane is fixed within a tile, so per-pair flags and coefficients
// are read once per tile, and the node loop is unrolled to keep several nodes' loads in flight.
#define BTILE_PAIRS(t)                                                                      \
    _Pragma("unroll 4") for (uint32_t I = (t).row0 + ((threadIdx.x & 31) >> 2); I < (t).row1; I += 8)

// p = z + beta p (beta = 0: p = z) for the running pairs.
template <class T>
__global__ void __launch_bounds__(kBThreads) k_b_dir(BDev B, const T *__restrict__ z, T *__restrict__ p) {
    if (*(volatile int *)B.n_active == 0) return;
    for (uint32_t tile = warp_id(); tile < B.ntiles; tile += warp_count()) {
        const BTile t = B.tiles[tile];
        if (B.sys_done[t.sys]) continue;
        const uint32_t r = threadIdx.x & 3, k = kBR * t.sys + r;
        if (B.done[k]) continue;
        const T beta = pair_coef<T>(B.beta, B.beta32, k);
        BTILE_PAIRS(t) {
            const uint64_t i = (uint64_t)kBV * I + 3 * r;
#pragma unroll
            for (int c = 0; c < 3; ++c) p[i + c] = beta != (T)0 ? fma(beta, p[i + c], z[i + c]) : z[i + c];
        }
    }
}

// 3x3 block-Jacobi: z = D r for one node and rhs.
template <class T>
__device__ __forceinline__ void bjac(const T *__restrict__ D, const T (&rv)[3], T (&zv)[3]) {
    zv[0] = D[0] * rv[0] + D[1] * rv[1] + D[2] * rv[2];
    zv[1] = D[3] * rv[0] + D[4] * rv[1] + D[5] * rv[2];
    zv[2] = D[6] * rv[0] + D[7] * rv[1] + D[8] * rv[2];
}

// Stopping test of pair k after an update (lanes 0..3 of the finalising warp), then the
// system flag and the running count (lane 0).
__device__ __forceinline__ void finish_system(const BDev &B, uint32_t sys) {
    __syncwarp();
    if ((threadIdx.x & 31) == 0) {
        const uint32_t k0 = kBR * sys;
        if (B.done[k0] && B.done[k0 + 1] && B.done[k0 + 2] && B.done[k0 + 3]) {
            B.sys_done[sys] = 1;
            atomicSub(B.n_active, 1);
        }
    }
}

// alpha; x += alpha p; r -= alpha q; z = D r; rz, rr -> beta and the stopping test.
template <class T>
__global__ void __launch_bounds__(kBThreads)
    k_b_update(BDev B, T *__restrict__ x, T *__restrict__ rv_, T *__restrict__ z, const T *__restrict__ p,
               const T *__restrict__ q, const T *__restrict__ Dinv) {
    if (*(volatile int *)B.n_active == 0) return;
    const int lane = threadIdx.x & 31;
    for (uint32_t tile = warp_id(); tile < B.ntiles; tile += warp_count()) {
        const BTile t = B.tiles[tile];
        if (B.sys_done[t.sys]) continue;  // set only after all of the system's tiles are done
        T acc0 = (T)0, acc1 = (T)0;       // rz, rr
        const uint32_t r = threadIdx.x & 3, kp = kBR * t.sys + r;
        const bool run = !B.done[kp];
        const T alpha = pair_coef<T>(B.alpha, B.alpha32, kp);
        if (run) BTILE_PAIRS(t) {
            const uint64_t i = (uint64_t)kBV * I + 3 * r;
            T rr3[3], zz[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                x[i + c] = fma(alpha, p[i + c], x[i + c]);
                rr3[c] = fma(-alpha, q[i + c], rv_[i + c]);
                rv_[i + c] = rr3[c];
            }
            bjac(Dinv + 9ull * I, rr3, zz);
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                z[i + c] = zz[c];
                acc0 = fma(rr3[c], zz[c], acc0);
                acc1 = fma(rr3[c], rr3[c], acc1);
            }
        }
        double s[2 * kBR], tot[2 * kBR];
        rhs_totals(acc0, s, 0);
        rhs_totals(acc1, s, kBR);
        if (warp_commit<2 * kBR>(B, tile, t.sys, s, B.tk + 2ull * B.nsys, tot)) {
            if (lane < kBR) {
                const uint32_t k = kBR * t.sys + lane;
                if (!B.done[k]) {
                    const double rz_new = pick(tot, lane), rr = pick(tot, kBR + lane);
                    const double beta = rz_new / B.rz[k];
                    B.iter[k] += 1;
                    B.beta[k] = beta;
                    B.beta32[k] = (float)beta;
                    B.rz[k] = rz_new;
                    B.rr[k] = rr;
                    if (!isfinite(rz_new) || !isfinite(rr) || !isfinite(B.pq[k])) {
                        B.status[k] = LMTG_ERR_NAN;
                        B.done[k] = 1;
                    } else if (rr <= B.crit2[k]) {
                        B.done[k] = 1;
                    } else if (B.iter[k] >= B.maxit) {
                        B.status[k] = LMTG_ERR_NOT_CONVERGED;
                        B.done[k] = 1;
                    }
                }
            }
            finish_system(B, t.sys);
        }
    }
}

// Start of a run from the residual r: z = D r, rz, rr per pair; beta from beta_den (> 0:
// continue the direction held in p); pairs preset done stay done.  Counts the running systems.
template <class T>
__global__ void __launch_bounds__(kBThreads)
    k_b_start(BDev B, const T *__restrict__ rv_, T *__restrict__ z, const T *__restrict__ Dinv) {
    const int lane = threadIdx.x & 31;
    for (uint32_t tile = warp_id(); tile < B.ntiles; tile += warp_count()) {
        const BTile t = B.tiles[tile];
        T acc0 = (T)0, acc1 = (T)0;
        const uint32_t r = threadIdx.x & 3;
        BTILE_PAIRS(t) {
            const uint64_t i = (uint64_t)kBV * I + 3 * r;
            T rr3[3] = {rv_[i], rv_[i + 1], rv_[i + 2]}, zz[3];
            bjac(Dinv + 9ull * I, rr3, zz);
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                z[i + c] = zz[c];
                acc0 = fma(rr3[c], zz[c], acc0);
                acc1 = fma(rr3[c], rr3[c], acc1);
            }
        }
        double s[2 * kBR], tot[2 * kBR];
        rhs_totals(acc0, s, 0);
        rhs_totals(acc1, s, kBR);
        if (warp_commit<2 * kBR>(B, tile, t.sys, s, B.tk + 3ull * B.nsys, tot)) {
            if (lane < kBR) {
                const uint32_t k = kBR * t.sys + lane;
                const double rz = pick(tot, lane), rr = pick(tot, kBR + lane);
                B.rz[k] = rz;
                B.rr[k] = rr;
                B.iter[k] = 0;
                B.status[k] = LMTG_OK;
                B.beta[k] = B.beta_den[k] > 0.0 ? rz / B.beta_den[k] : 0.0;
                B.beta32[k] = (float)B.beta[k];
                if (!isfinite(rz) || !isfinite(rr)) {
                    B.status[k] = LMTG_ERR_NAN;
                    B.done[k] = 1;
                } else if (rr <= B.crit2[k]) {
                    B.done[k] = 1;
                }
            }
            __syncwarp();
            if (lane == 0) {
                const uint32_t k0 = kBR * t.sys;
                const bool all = B.done[k0] && B.done[k0 + 1] && B.done[k0 + 2] && B.done[k0 + 3];
                B.sys_done[t.sys] = all ? 1 : 0;
                if (!all) atomicAdd(B.n_active, 1);
            }
        }
    }
}

// |v|^2 per pair -> out (FP64 vectors).
__global__ void __launch_bounds__(kBThreads) k_b_norm2(BDev B, const double *__restrict__ v) {
    const int lane = threadIdx.x & 31;
    for (uint32_t tile = warp_id(); tile < B.ntiles; tile += warp_count()) {
        const BTile t = B.tiles[tile];
        double acc = 0.0;
        const uint32_t r = threadIdx.x & 3;
        BTILE_PAIRS(t) {
            const uint64_t i = (uint64_t)kBV * I + 3 * r;
#pragma unroll
            for (int c = 0; c < 3; ++c) acc = fma(v[i + c], v[i + c], acc);
        }
        double s[kBR], tot[kBR];
        rhs_totals(acc, s, 0);
        if (warp_commit<kBR>(B, tile, t.sys, s, B.tk + 1ull * B.nsys, tot) && lane < kBR)
            B.out[kBR * t.sys + lane] = pick(tot, lane);
    }
}

// r32 = r64 / scale, d32 = 0 (scale 0: the pair is not solved, r32 = 0).
__global__ void k_b_scale(BDev B, const double *__restrict__ r64, float *__restrict__ r32, float *__restrict__ d32) {
    for (uint32_t tile = warp_id(); tile < B.ntiles; tile += warp_count()) {
        const BTile t = B.tiles[tile];
        const uint32_t r = threadIdx.x & 3;
        const double s = B.scale[kBR * t.sys + r];
        const double inv = s > 0.0 ? 1.0 / s : 0.0;
        BTILE_PAIRS(t) {
            const uint64_t i = (uint64_t)kBV * I + 3 * r;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                r32[i + c] = (float)(r64[i + c] * inv);
                d32[i + c] = 0.0f;
            }
        }
    }
}

// x64 += scale d32
__global__ void k_b_axpy(BDev B, double *__restrict__ x, const float *__restrict__ d32) {
    for (uint32_t tile = warp_id(); tile < B.ntiles; tile += warp_count()) {
        const BTile t = B.tiles[tile];
        const uint32_t r = threadIdx.x & 3;
        const double s = B.scale[kBR * t.sys + r];
        if (s == 0.0) continue;
        BTILE_PAIRS(t) {
            const uint64_t i = (uint64_t)kBV * I + 3 * r;
#pragma unroll
            for (int c = 0; c < 3; ++c) x[i + c] = fma(s, (double)d32[i + c], x[i + c]);
        }
    }
}

// host layout (nrhs x n, rhs-major) <-> interleaved node layout
__global__ void k_b_interleave(const double *__restrict__ src, double *__restrict__ dst, uint64_t nn, int nrhs) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < nn * kBV;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t I = i / kBV;
        const int v = (int)(i - I * kBV), r = v / 3, c = v - 3 * r;
        dst[i] = r < nrhs ? src[(uint64_t)r * 3 * nn + 3 * I + c] : 0.0;
    }
}
__global__ void k_b_deinterleave(const double *__restrict__ src, double *__restrict__ dst, uint64_t nn, int nrhs) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < (uint64_t)nrhs * 3 * nn;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t r = i / (3 * nn), j = i - r * 3 * nn;
        dst[i] = src[kBV * (j / 3) + 3 * r + j % 3];
    }
}

// ---- host ----------------------------------------------------------------------------------
struct BatchState {
    int tile_rows = 0;
    int unit_rows = 0;             // k_b_rows_bulk: rows per CTA unit (a multiple of tile_rows)
    std::vector<BTile> h_tiles;
    std::vector<uint32_t> h_groups, h_sys_g;
    DBuf<uint32_t> groups, sys_g;
    std::vector<uint32_t> h_tile_off;
    DBuf<BTile> tiles;
    DBuf<uint32_t> tile_off;
    DBuf<double> partials;
    DBuf<unsigned> tk;
    DBuf<double> dscal;  // 9 arrays of 4 nsys doubles
    DBuf<float> fscal;   // alpha32, beta32
    DBuf<int> iscal;     // iter, done, status (4 nsys each), sys_done (nsys), n_active, fault
    int *h_active = nullptr;  // pinned: n_active, fault
    int nrhs = 0;
    DBuf<double> F4, U4, R64, Z64, P64, Q64;
    DBuf<float> R32, Z32, P32, Q32, D32;
    int pipe = 1;                  // SpMV variant: k_b_rows kPipe 0 / 1, 2 = k_b_rows_bulk (FP32)
    int bulk_grid = 0;             // resident grid of k_b_rows_bulk
    std::vector<double> tuned_ms;  // SpMV ms per candidate (variant-major, 4 tile sizes each)
    ~BatchState() {
        if (h_active) cudaFreeHost(h_active);
    }
};

void batch_free(lmtg_ctx *c) {
    delete c->batch;
    c->batch = nullptr;
}

static BDev bdev(lmtg_ctx *c, int maxit) {
    BatchState &S = *c->batch;
    const uint64_t np = (uint64_t)kBR * c->nsys;
    BDev B{};
    B.tiles = S.tiles.p;
    B.ntiles = (uint32_t)S.h_tiles.size();
    B.groups = S.groups.p;
    B.sys_g = S.sys_g.p;
    B.ngroups = S.h_groups.empty() ? 0u : (uint32_t)S.h_groups.size() - 1;
    B.tile_off = S.tile_off.p;
    B.partials = S.partials.p;
    B.tk = S.tk.p;
    B.nsys = c->nsys;
    double *d = S.dscal.p;
    B.rz = d; B.pq = d + np; B.rr = d + 2 * np; B.crit2 = d + 3 * np;
    B.beta = d + 4 * np; B.beta_den = d + 5 * np; B.scale = d + 6 * np; B.out = d + 7 * np;
    B.alpha = d + 8 * np;
    B.alpha32 = S.fscal.p;
    B.beta32 = S.fscal.p + np;
    int *q = S.iscal.p;
    B.iter = q; B.done = q + np; B.status = q + 2 * np; B.sys_done = q + 3 * np; B.n_active = q + 3 * np + c->nsys;
    B.fault = B.n_active + 1;
    B.maxit = maxit;
    return B;
}

static void build_tiles(lmtg_ctx *c, int rows) {
    BatchState &S = *c->batch;
    S.tile_rows = rows;
    S.h_tiles.clear();
    S.h_tile_off.assign(1, 0);
    for (uint32_t m = 0; m < c->nsys; ++m) {
        for (uint64_t r0 = c->h_sys_node_off[m]; r0 < c->h_sys_node_off[m + 1]; r0 += rows)
            S.h_tiles.push_back({m, (uint32_t)r0, (uint32_t)std::min<uint64_t>(r0 + rows, c->h_sys_node_off[m + 1]), 0});
        S.h_tile_off.push_back((uint32_t)S.h_tiles.size());
    }
    upload_u32(c, S.tiles, S.h_tiles.data(), S.h_tiles.size());
    upload_u32(c, S.tile_off, S.h_tile_off.data(), S.h_tile_off.size());
    S.partials.alloc(S.h_tiles.size() * kBTileSlots);
    LMTG_CUDA(cudaStreamSynchronize(c->stream));
}

// Units of k_b_rows_bulk: runs of `per` consecutive tiles of one system.
static void build_groups(lmtg_ctx *c, int per) {
    BatchState &S = *c->batch;
    S.unit_rows = per * S.tile_rows;
    S.h_groups.clear();
    S.h_sys_g.clear();
    for (uint32_t m = 0; m < c->nsys; ++m) {
        S.h_sys_g.push_back((uint32_t)S.h_groups.size());
        for (uint32_t t = S.h_tile_off[m]; t < S.h_tile_off[m + 1]; t += per) S.h_groups.push_back(t);
    }
    S.h_sys_g.push_back((uint32_t)S.h_groups.size());
    S.h_groups.push_back((uint32_t)S.h_tiles.size());
    upload_u32(c, S.groups, S.h_groups.data(), S.h_groups.size());
    upload_u32(c, S.sys_g, S.h_sys_g.data(), S.h_sys_g.size());
    LMTG_CUDA(cudaStreamSynchronize(c->stream));
}

template <class KF>
static int bgrid(lmtg_ctx *c, KF kernel) {
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, kBThreads, 0) != cudaSuccess || nb < 1) nb = 1;
    const uint64_t nt = c->batch->h_tiles.size();  // one warp per tile
    return (int)std::max<uint64_t>(1, std::min<uint64_t>((nt + kBWarps - 1) / kBWarps, (uint64_t)c->sm_count * nb));
}

constexpr int kBBulkStages = 2, kBBulkCap = 512, kBBulkMinB = 3;

static int bulk_rows_grid(lmtg_ctx *c) {
    constexpr size_t smem = bulk_smem_bytes<kBBulkStages, kBBulkCap>();
    auto fn = k_b_rows_bulk<kBBulkStages, kBBulkCap, kBBulkMinB>;
    LMTG_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int nb = 0;
    LMTG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, kBBulkThreads, smem));
    const uint64_t nt = c->batch->h_groups.size() - 1;  // one CTA per unit at a time
    return (int)std::max<uint64_t>(1, std::min<uint64_t>(nt, (uint64_t)c->sm_count * (nb > 0 ? nb : 1)));
}

template <class T, int kMode>
static void launch_rows(lmtg_ctx *c, const BDev &B, int pipe, const T *K, const T *x, const T *b, T *y,
                        cudaStream_t s) {
    if constexpr (std::is_same<T, float>::value && kMode == 0) {
        if (pipe == 2) {
            k_b_rows_bulk<kBBulkStages, kBBulkCap, kBBulkMinB>
                <<<c->batch->bulk_grid, kBBulkThreads, bulk_smem_bytes<kBBulkStages, kBBulkCap>(), s>>>(
                    B, c->bptr.p, c->bcol.p, K, x, y);
            c->launches += 1;
            return;
        }
    }
    if (pipe)
        k_b_rows<T, kMode, 1><<<bgrid(c, k_b_rows<T, kMode, 1>), kBThreads, 0, s>>>(B, c->bptr.p, c->bcol.p, K, x,
                                                                                      b, y);
    else
        k_b_rows<T, kMode, 0><<<bgrid(c, k_b_rows<T, kMode, 0>), kBThreads, 0, s>>>(B, c->bptr.p, c->bcol.p, K, x,
                                                                                      b, y);
    c->launches += 1;
}

// Autotuner: the tile size (rows per tile) with the fastest batched SpMV on this batch, timed
// with CUDA events over a few launches with every system running.
static void autotune(lmtg_ctx *c) {
    BatchState &S = *c->batch;
    const bool f32 = c->have32;
    const uint64_t nv = (uint64_t)kBV * c->nn;
    DBuf<float> x32, y32;
    DBuf<double> x64, y64;
    if (f32) { x32.alloc(nv); y32.alloc(nv); LMTG_CUDA(cudaMemsetAsync(x32.p, 0, nv * 4, c->stream)); }
    else { x64.alloc(nv); y64.alloc(nv); LMTG_CUDA(cudaMemsetAsync(x64.p, 0, nv * 8, c->stream)); }
    // variants 0, 1: rows per warp tile; variant 2: rows per CTA unit of 128-row tiles (the
    // vector kernels keep one warp per 128-row tile)
    const int cands[3][4] = {{16, 32, 64, 128}, {16, 32, 64, 128}, {128, 256, 512, 1024}};
    constexpr int kUnitTile = 128;
    double best = 1e30;
    int best_rows = 32, best_pipe = 1;
    S.tuned_ms.clear();
    cudaEvent_t e0, e1;
    LMTG_CUDA(cudaEventCreate(&e0));
    LMTG_CUDA(cudaEventCreate(&e1));
    for (int pipe = 0; pipe < 3; ++pipe) {
        for (int rows : cands[pipe]) {
            if ((c->batch_tile_rows > 0 && rows != c->batch_tile_rows) ||
                (c->batch_variant >= 0 && pipe != c->batch_variant) || (pipe == 2 && !f32)) {
                S.tuned_ms.push_back(0.0);
                continue;
            }
            if (pipe == 2) {
                if (S.tile_rows != kUnitTile) build_tiles(c, kUnitTile);
                build_groups(c, rows / kUnitTile);
                S.bulk_grid = bulk_rows_grid(c);
            } else {
                build_tiles(c, rows);
            }
            BDev B = bdev(c, 1);
            // every system running: sys_done = 0, n_active = nsys
            LMTG_CUDA(cudaMemsetAsync(B.sys_done, 0, sizeof(int) * c->nsys, c->stream));
            const int na = (int)c->nsys;
            LMTG_CUDA(cudaMemcpyAsync(B.n_active, &na, sizeof(int), cudaMemcpyHostToDevice, c->stream));
            float ms = 0;
            for (int rep = 0; rep < 2; ++rep) {  // the first pass warms up
                LMTG_CUDA(cudaEventRecord(e0, c->stream));
                for (int it = 0; it < 3; ++it) {
                    if (f32) launch_rows<float, 0>(c, B, pipe, c->K32.p, x32.p, nullptr, y32.p, c->stream);
                    else launch_rows<double, 0>(c, B, pipe, c->K64.p, x64.p, nullptr, y64.p, c->stream);
                }
                LMTG_CUDA(cudaGetLastError());
                LMTG_CUDA(cudaEventRecord(e1, c->stream));
                LMTG_CUDA(cudaEventSynchronize(e1));
                cudaEventElapsedTime(&ms, e0, e1);
            }
            S.tuned_ms.push_back(ms / 3.0);
            if (ms < best) {
                best = ms;
                best_rows = rows;
                best_pipe = pipe;
            }
        }
    }
    S.pipe = best_pipe;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    const int tile = best_pipe == 2 ? kUnitTile : best_rows;
    if (tile != S.tile_rows) build_tiles(c, tile);
    build_groups(c, best_pipe == 2 ? best_rows / kUnitTile : 1);
    S.bulk_grid = bulk_rows_grid(c);
    LMTG_CUDA(cudaMemsetAsync(bdev(c, 1).fault, 0, sizeof(int), c->stream));
}

static void batch_prepare(lmtg_ctx *c) {
    LMTG_CHECK(c->nsys > 0, LMTG_ERR_STATE, "lmtg_batch_set first");
    LMTG_CHECK(c->have64, LMTG_ERR_STATE, "assemble the FP64 matrix first");
    if (!c->batch) c->batch = new BatchState();
    BatchState &S = *c->batch;
    if (S.tile_rows) return;
    const uint64_t np = (uint64_t)kBR * c->nsys;
    S.dscal.alloc(9 * np);
    S.fscal.alloc(2 * np);
    LMTG_CUDA(cudaMemsetAsync(S.fscal.p, 0, 2 * np * sizeof(float), c->stream));
    S.iscal.alloc(3 * np + c->nsys + 2);
    S.tk.alloc(4ull * c->nsys);
    LMTG_CUDA(cudaMemsetAsync(S.dscal.p, 0, 9 * np * sizeof(double), c->stream));
    LMTG_CUDA(cudaMemsetAsync(S.iscal.p, 0, (3 * np + c->nsys + 2) * sizeof(int), c->stream));
    LMTG_CUDA(cudaMemsetAsync(S.tk.p, 0, 4ull * c->nsys * sizeof(unsigned), c->stream));
    if (!S.h_active) LMTG_CUDA(cudaMallocHost(&S.h_active, 2 * sizeof(int)));
    const uint64_t nv = (uint64_t)kBV * c->nn;
    S.F4.alloc(nv);
    S.U4.alloc(nv);
    LMTG_CUDA(cudaMemsetAsync(S.F4.p, 0, nv * 8, c->stream));
    LMTG_CUDA(cudaMemsetAsync(S.U4.p, 0, nv * 8, c->stream));
    autotune(c);
}

static void batch_alloc_mode(lmtg_ctx *c, int mode) {
    BatchState &S = *c->batch;
    const uint64_t nv = (uint64_t)kBV * c->nn;
    S.R64.alloc(nv);
    if (mode == LMTG_SOLVE_PCG_F64) {
        S.Z64.alloc(nv);
        S.P64.alloc(nv);
        S.Q64.alloc(nv);
    } else {
        S.R32.alloc(nv);
        S.Z32.alloc(nv);
        S.P32.alloc(nv);
        S.Q32.alloc(nv);
        S.D32.alloc(nv);
    }
}

template <class T>
static void upload_pairs(lmtg_ctx *c, T *dst, const std::vector<T> &h) {
    LMTG_CUDA(cudaMemcpyAsync(dst, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, c->stream));
}
template <class T>
static void download_pairs(lmtg_ctx *c, std::vector<T> &h, const T *src) {
    LMTG_CUDA(cudaMemcpyAsync(h.data(), src, h.size() * sizeof(T), cudaMemcpyDeviceToHost, c->stream));
    LMTG_CUDA(cudaStreamSynchronize(c->stream));
}

// One PCG run in precision T on the pairs not preset done, from the residual r (x is updated in
// place); graph chunks of kBIters iterations until no system is running.
template <class T>
static int batch_pcg_run(lmtg_ctx *c, BDev B, const T *K, const T *Dinv, T *x, T *r, T *z, T *p, T *q,
                         double deadline_s, std::chrono::steady_clock::time_point t0) {
    cudaStream_t s = c->stream;
    LMTG_CUDA(cudaMemsetAsync(B.n_active, 0, 2 * sizeof(int), s));  // running count and fault word
    k_b_start<T><<<bgrid(c, k_b_start<T>), kBThreads, 0, s>>>(B, r, z, Dinv);
    c->launches += 1;
    LMTG_CUDA(cudaGetLastError());
    constexpr int kBIters = 16;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    const int g_dir = bgrid(c, k_b_dir<T>), g_upd = bgrid(c, k_b_update<T>);
    LMTG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    for (int k = 0; k < kBIters; ++k) {
        k_b_dir<T><<<g_dir, kBThreads, 0, s>>>(B, z, p);
        launch_rows<T, 0>(c, B, c->batch->pipe, K, p, nullptr, q, s);
        k_b_update<T><<<g_upd, kBThreads, 0, s>>>(B, x, r, z, p, q, Dinv);
    }
    cudaError_t ce = cudaStreamEndCapture(s, &graph);
    if (ce != cudaSuccess) throw Error{LMTG_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ce)};
    ce = cudaGraphInstantiate(&exec, graph, 0);
    if (ce != cudaSuccess) {
        cudaGraphDestroy(graph);
        throw Error{LMTG_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ce)};
    }
    int status = LMTG_OK;
    BatchState &S = *c->batch;
    LMTG_CUDA(cudaMemcpyAsync(S.h_active, B.n_active, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
    LMTG_CUDA(cudaStreamSynchronize(s));
    const int max_chunks = B.maxit / kBIters + 2;
    for (int ch = 0; ch < max_chunks && S.h_active[0] > 0; ++ch) {
        ce = cudaGraphLaunch(exec, s);
        c->launches += 2 * kBIters;  // + the SpMV launches counted at capture
        if (ce == cudaSuccess)
            ce = cudaMemcpyAsync(S.h_active, B.n_active, 2 * sizeof(int), cudaMemcpyDeviceToHost, s);
        if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
        if (ce != cudaSuccess) {
            cudaGraphExecDestroy(exec);
            cudaGraphDestroy(graph);
            throw Error{LMTG_ERR_CUDA, std::string("batched pcg: ") + cudaGetErrorString(ce)};
        }
        if (S.h_active[1] != 0) {  // a bounded wait of the SpMV gave up: results are not valid
            status = LMTG_ERR_TIMEOUT;
            break;
        }
        if (deadline_s > 0 &&
            std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count() > deadline_s) {
            status = LMTG_ERR_TIMEOUT;
            break;
        }
    }
    if (status == LMTG_OK && S.h_active[0] > 0) status = LMTG_ERR_NOT_CONVERGED;
    cudaGraphExecDestroy(exec);
    cudaGraphDestroy(graph);
    return status;
}

static int worst(int a, int b) { return a != LMTG_OK ? a : b; }

// Solves the batch: every pair (system m, rhs r < nrhs) to |b - K x| <= tol |b| in FP64.
int batch_solve(lmtg_ctx *c, int mode, double tol, int maxit, double timeout_s, lmtg_solve_stats *st,
                int *pair_iters) {
    Phase ph("lmtg.batch_solve");
    batch_prepare(c);
    BatchState &S = *c->batch;
    LMTG_CHECK(S.nrhs > 0, LMTG_ERR_STATE, "lmtg_batch_set_rhs first");
    LMTG_CHECK(c->penalty != 0.0 || c->nc == 0, LMTG_ERR_UNSUPPORTED, "batch solves with exact (penalty 0) constraints");
    batch_alloc_mode(c, mode);
    const auto t0 = std::chrono::steady_clock::now();
    cudaStream_t s = c->stream;
    const uint32_t ns = c->nsys;
    const uint64_t np = (uint64_t)kBR * ns;
    BDev B = bdev(c, maxit);
    const int g_el = bgrid(c, k_b_scale);
    // |b|^2 per pair
    k_b_norm2<<<bgrid(c, k_b_norm2), kBThreads, 0, s>>>(B, S.F4.p);
    c->launches += 1;
    std::vector<double> bb(np), rr(np), h(np);
    download_pairs(c, bb, B.out);
    std::vector<int> done(np), it_total(np, 0), it_seg(np), stat(np);
    auto residual64 = [&]() {
        launch_rows<double, 1>(c, B, S.pipe, c->K64.p, S.U4.p, S.F4.p, S.R64.p, s);
        LMTG_CUDA(cudaGetLastError());
        download_pairs(c, rr, B.rr);
    };
    int status = LMTG_OK, outer = 0;
    if (mode == LMTG_SOLVE_PCG_F64) {
        // FP64 PCG on the recursive residual; restarted from the true residual for the pairs
        // whose true residual is still above tol (a few at most)
        for (; outer < 8; ++outer) {
            residual64();
            bool all = true;
            for (uint64_t k = 0; k < np; ++k) {
                const bool conv = bb[k] == 0.0 || rr[k] <= tol * tol * bb[k];
                done[k] = conv ? 1 : 0;
                h[k] = tol * tol * bb[k];
                all = all && conv;
            }
            if (all) break;
            int itmax = 0;
            for (uint64_t k = 0; k < np; ++k) itmax = std::max(itmax, it_total[k]);
            if (itmax >= maxit) { status = LMTG_ERR_NOT_CONVERGED; break; }
            upload_pairs(c, B.done, done);
            upload_pairs(c, B.crit2, h);
            LMTG_CUDA(cudaMemsetAsync(B.beta_den, 0, np * sizeof(double), s));
            B.maxit = std::max(1, maxit - itmax);
            const int s2 = batch_pcg_run<double>(c, B, c->K64.p, c->Dinv64.p, S.U4.p, S.R64.p, S.Z64.p, S.P64.p,
                                                 S.Q64.p, timeout_s, t0);
            download_pairs(c, it_seg, B.iter);
            download_pairs(c, stat, B.status);
            for (uint64_t k = 0; k < np; ++k)
                if (!done[k]) it_total[k] += it_seg[k];
            if (s2 == LMTG_ERR_TIMEOUT) { status = s2; break; }
            bool nan = false;
            for (uint64_t k = 0; k < np; ++k) nan = nan || stat[k] == LMTG_ERR_NAN;
            if (nan) { status = LMTG_ERR_NAN; break; }
        }
        std::fill(stat.begin(), stat.end(), (int)LMTG_OK);
    } else if (mode == LMTG_SOLVE_MIXED_IR) {
        LMTG_CHECK(c->have32, LMTG_ERR_STATE, "mixed batch solve needs the FP32 matrix (assemble MAT32)");
        // FP32 segments with FP64 residual replacement, per pair (the single-system scheme):
        // each segment reduces its recursive residual by inner_reduction (or to the remaining target), the
        // direction is kept across the replacement while the true residual keeps halving.
        const double kDelta = c->inner_reduction;
        std::vector<double> s_prev(np, 0.0), rz_prev(np, 0.0), rel_prev(np, 0.0), sc(np), den(np), rzv(np), bt(np);
        std::vector<int> have_dir(np, 0);
        for (;;) {
            residual64();
            bool all = true, nan = false;
            for (uint64_t k = 0; k < np; ++k) {
                const double rel = bb[k] > 0 ? std::sqrt(rr[k] / bb[k]) : 0.0;
                if (!std::isfinite(rel)) nan = true;
                const bool conv = bb[k] == 0.0 || rel <= tol || rr[k] == 0.0;
                done[k] = conv ? 1 : 0;
                sc[k] = conv ? 0.0 : std::sqrt(rr[k]);
                if (conv) {
                    h[k] = 0.0;
                    den[k] = 0.0;
                    continue;
                }
                all = false;
                if (have_dir[k] && rel > 0.5 * rel_prev[k]) have_dir[k] = 0;
                const double eta = std::max(kDelta, 0.5 * tol / rel);
                h[k] = eta * eta;  // |b32| = 1
                den[k] = have_dir[k] ? rz_prev[k] * (s_prev[k] / sc[k]) : 0.0;
                rel_prev[k] = rel;
            }
            if (nan) { status = LMTG_ERR_NAN; break; }
            if (all) break;
            int itmax = 0;
            for (uint64_t k = 0; k < np; ++k) itmax = std::max(itmax, it_total[k]);
            if (itmax >= maxit || outer >= 400) { status = LMTG_ERR_NOT_CONVERGED; break; }
            upload_pairs(c, B.done, done);
            upload_pairs(c, B.crit2, h);
            upload_pairs(c, B.beta_den, den);
            upload_pairs(c, B.scale, sc);
            k_b_scale<<<g_el, kBThreads, 0, s>>>(B, S.R64.p, S.R32.p, S.D32.p);
            c->launches += 1;
            B.maxit = std::max(1, maxit - itmax);
            const int s2 = batch_pcg_run<float>(c, B, c->K32.p, c->Dinv32.p, S.D32.p, S.R32.p, S.Z32.p, S.P32.p,
                                                S.Q32.p, timeout_s, t0);
            ++outer;
            if (s2 == LMTG_ERR_TIMEOUT) { status = s2; }
            download_pairs(c, it_seg, B.iter);
            download_pairs(c, stat, B.status);
            download_pairs(c, rzv, B.rz);
            download_pairs(c, bt, B.beta);
            for (uint64_t k = 0; k < np; ++k) {
                if (sc[k] == 0.0) continue;
                it_total[k] += it_seg[k];
                rz_prev[k] = bt[k] != 0.0 ? rzv[k] / bt[k] : 0.0;
                s_prev[k] = sc[k];
                have_dir[k] = it_seg[k] > 0 && rz_prev[k] > 0.0;
                if (stat[k] == LMTG_ERR_NAN) status = LMTG_ERR_NAN;
            }
            k_b_axpy<<<g_el, kBThreads, 0, s>>>(B, S.U4.p, S.D32.p);
            c->launches += 1;
            LMTG_CUDA(cudaGetLastError());
            if (status != LMTG_OK) break;
        }
        std::fill(stat.begin(), stat.end(), (int)LMTG_OK);
    } else {
        throw Error{LMTG_ERR_ARG, "unknown solve mode"};
    }
    // final true residual of every pair
    residual64();
    double worst_rel = 0.0;
    int itmax = 0;
    for (uint64_t k = 0; k < np; ++k) {
        if ((int)(k % kBR) >= S.nrhs) continue;
        const double rel = bb[k] > 0 ? std::sqrt(rr[k] / bb[k]) : 0.0;
        worst_rel = std::max(worst_rel, rel);
        itmax = std::max(itmax, it_total[k]);
        status = worst(status, stat[k]);
        if (pair_iters) pair_iters[(k / kBR) * S.nrhs + k % kBR] = it_total[k];
    }
    if (status == LMTG_OK && !(worst_rel <= tol * 1.0000001)) status = LMTG_ERR_NOT_CONVERGED;
    st->iterations = itmax;
    st->outer_iterations = outer;
    st->rel_residual = worst_rel;
    return status;
}

void batch_set_rhs(lmtg_ctx *c, int nrhs, const double *B_host) {
    batch_prepare(c);
    BatchState &S = *c->batch;
    const uint64_t n = 3 * c->nn, nv = (uint64_t)kBV * c->nn;
    DBuf<double> tmp;
    tmp.alloc((uint64_t)nrhs * n);
    LMTG_CUDA(cudaMemcpyAsync(tmp.p, B_host, (uint64_t)nrhs * n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    k_b_interleave<<<grid_for(c, nv, 256), 256, 0, c->stream>>>(tmp.p, S.F4.p, c->nn, nrhs);
    LMTG_CUDA(cudaMemsetAsync(S.U4.p, 0, nv * sizeof(double), c->stream));
    LMTG_CUDA(cudaGetLastError());
    c->launches += 1;
    LMTG_CUDA(cudaStreamSynchronize(c->stream));
    S.nrhs = nrhs;
}

void batch_get_result(lmtg_ctx *c, double *X_host) {
    LMTG_CHECK(c->batch && c->batch->nrhs > 0, LMTG_ERR_STATE, "no batch solution");
    BatchState &S = *c->batch;
    const uint64_t n = 3 * c->nn;
    DBuf<double> tmp;
    tmp.alloc((uint64_t)S.nrhs * n);
    k_b_deinterleave<<<grid_for(c, (uint64_t)S.nrhs * n, 256), 256, 0, c->stream>>>(S.U4.p, tmp.p, c->nn, S.nrhs);
    LMTG_CUDA(cudaGetLastError());
    c->launches += 1;
    LMTG_CUDA(cudaMemcpyAsync(X_host, tmp.p, (uint64_t)S.nrhs * n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    LMTG_CUDA(cudaStreamSynchronize(c->stream));
}

void batch_info(lmtg_ctx *c, int *tile_rows, int *variant, uint64_t *ntiles, double *tuned_ms) {
    batch_prepare(c);
    BatchState &S = *c->batch;
    if (tile_rows) *tile_rows = S.pipe == 2 ? S.unit_rows : S.tile_rows;
    if (variant) *variant = S.pipe;
    if (ntiles) *ntiles = S.h_tiles.size();
    if (tuned_ms)
        for (size_t i = 0; i < S.tuned_ms.size(); ++i) tuned_ms[i] = S.tuned_ms[i];
}

}  // namespace lmtg
