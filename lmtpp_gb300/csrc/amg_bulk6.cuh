// Row products of the multigrid's 6x6-block levels with the matrix streamed through shared
// memory by the bulk-copy engine (TMA).
//
// At the C3 workload level 1 holds 2.05 M blocks of 144 bytes (295 MB, over twice the L2), and
// each preconditioner application streams it five times.  The warp-per-row kernels keep the
// matrix loads, the x gathers and the reductions on one dependency chain per warp and reach
// about 0.4 of HBM there; this kernel decouples the stream as the level-0 bulk-copy SpMV does.
//
// Each CTA owns a contiguous range of block rows.  The planar per-row layout (component v of
// local block b of a row starting at block rb at 36 rb + v deg + b) keeps the values of
// consecutive rows contiguous, so a run of rows is one byte range of values and one of column
// indices: one producer warp moves runs of up to kCons rows (and at most kCap blocks) into a
// ring of kStages stages with `cp.async.bulk`, completion counted on the stage's "full"
// mbarrier.  Consumer warp w takes row w of a stage, lane b its block b (rows wider than 32
// blocks in chunks of 32), reads the 36 values and the column from shared memory, gives the
// stage back (its "empty" mbarrier) and only then gathers x and multiplies.  The six row sums are
// reduce-scattered over the warp (lane 4c ends with component c) and handed to the epilogue,
// whose operands were loaded before the products.
//
// Every mbarrier wait is bounded (about a second of %globaltimer and an iteration cap); a wait
// that gives up sets LMTG_ERR_TIMEOUT and done in the PCG scalars, and the producer waits,
// bounded again, for its own copies in flight before the CTA exits.  Rows are independent and
// each is summed in a fixed order: results are deterministic.
#pragma once
#include "spmv_bulk.cuh"

namespace lmtg {

template <int kCap>
struct Bulk6Stage {
    static_assert(kCap % 4 == 0 && kCap >= 128, "a stage holds at least one coarse row of 128 blocks");
    static constexpr uint32_t kKBytes = 144u * kCap + 32u;  // values (144 * b is 16-byte aligned)
    static constexpr uint32_t kCBytes = 4u * kCap + 32u;    // column indices, rounded on both ends
    static constexpr uint32_t kBytes = kKBytes + kCBytes;
};

template <int kStages, int kCap>
constexpr size_t bulk6_smem_bytes() {
    return (size_t)kStages * Bulk6Stage<kCap>::kBytes;
}

// Sum of a[0..5] over the warp, scattered: lane 4c (c < 6) ends with the total of component c
// (lanes 4c + 1 .. 4c + 3 too).  Nine shuffles instead of thirty for six warp sums; slots 6 and 7
// are zero.
__device__ __forceinline__ float reduce_scatter6(const float (&a)[6], int lane) {
    constexpr unsigned F = 0xffffffffu;
    const bool h16 = lane & 16, h8 = lane & 8, h4 = lane & 4;
    // keep slots 0..3 (h16 clear) or 4..7, send the other four
    const float w0 = (h16 ? a[4] : a[0]) + __shfl_xor_sync(F, h16 ? a[0] : a[4], 16);
    const float w1 = (h16 ? a[5] : a[1]) + __shfl_xor_sync(F, h16 ? a[1] : a[5], 16);
    const float w2 = (h16 ? 0.f : a[2]) + __shfl_xor_sync(F, h16 ? a[2] : 0.f, 16);
    const float w3 = (h16 ? 0.f : a[3]) + __shfl_xor_sync(F, h16 ? a[3] : 0.f, 16);
    const float u0 = (h8 ? w2 : w0) + __shfl_xor_sync(F, h8 ? w0 : w2, 8);
    const float u1 = (h8 ? w3 : w1) + __shfl_xor_sync(F, h8 ? w1 : w3, 8);
    float v = (h4 ? u1 : u0) + __shfl_xor_sync(F, h4 ? u0 : u1, 4);
    v += __shfl_xor_sync(F, v, 2);
    v += __shfl_xor_sync(F, v, 1);
    return v;
}

// Epilogues of the 6x6 bulk-copy product (x padded to 8 per node, right-hand sides packed 6):
//   Epi6Res   res = r - K x (r may be null: res = -K x); with D also the first smoothing step of a
//             cycle on that residual, xpre = omega D^-1 res
//   Epi6Post  xo = x + omega D^-1 (r - K x)
// pre() runs before the row's products; row() gets the reduce-scattered sums (lane 4c holds
// component c) and is called by every lane.
struct Epi6Res {
    const float *r;
    float *res;
    const float *D;
    float omega;
    float *xpre;
    struct Pre {
        float r, d[6];
    };
    __device__ __forceinline__ Pre pre(uint64_t I, int lane) const {
        Pre p{};
        const int c = lane >> 2;
        if ((lane & 3) == 0 && c < 6) {
            p.r = r ? r[6 * I + c] : 0.f;
            if (D) {
#pragma unroll
                for (int j = 0; j < 6; ++j) p.d[j] = D[36 * I + 6 * c + j];
            }
        }
        return p;
    }
    __device__ __forceinline__ void row(uint64_t I, float t, int lane, const Pre &p) const {
        const int c = lane >> 2;
        const bool on = (lane & 3) == 0 && c < 6;
        const float dr = p.r - t;
        if (on) res[6 * I + c] = dr;
        if (D) {
            float s = 0.f;
#pragma unroll
            for (int j = 0; j < 6; ++j) s = fmaf(p.d[j], __shfl_sync(0xffffffffu, dr, 4 * j), s);
            if (on) xpre[8 * I + c] = omega * s;
        }
    }
};

struct Epi6Post {
    const float *r, *D, *x;
    float *xo;
    float omega;
    struct Pre {
        float r, x, d[6];
    };
    __device__ __forceinline__ Pre pre(uint64_t I, int lane) const {
        Pre p{};
        const int c = lane >> 2;
        if ((lane & 3) == 0 && c < 6) {
            p.r = r[6 * I + c];
            p.x = x[8 * I + c];
#pragma unroll
            for (int j = 0; j < 6; ++j) p.d[j] = D[36 * I + 6 * c + j];
        }
        return p;
    }
    __device__ __forceinline__ void row(uint64_t I, float t, int lane, const Pre &p) const {
        const int c = lane >> 2;
        const float dr = p.r - t;
        float s = 0.f;
#pragma unroll
        for (int j = 0; j < 6; ++j) s = fmaf(p.d[j], __shfl_sync(0xffffffffu, dr, 4 * j), s);
        if ((lane & 3) == 0 && c < 6) xo[8 * I + c] = p.x + omega * s;
    }
};

// kCons consumer warps (one row each per stage) + one producer warp
template <int kStages, int kCap, int kCons, int kMinBlocks, class Epi>
__global__ void __launch_bounds__(32 * (kCons + 1), kMinBlocks)
    k_amg6_bulk(const uint32_t *__restrict__ bptr, const uint32_t *__restrict__ bcol, const float *__restrict__ K,
                const float *__restrict__ x, Epi epi, uint64_t nn, PcgScalars *S) {
    static_assert(kCons >= 1 && kCons <= 31, "the producer sizes a stage with one warp of bptr loads");
    using St = Bulk6Stage<kCap>;
    // programmatic dependent launch (see the multigrid's launch_pdl): wait for the previous
    // kernel's writes.  No early trigger: its successor starts when this stream ends
    asm volatile("griddepcontrol.wait;" ::: "memory");
    if (S && *(volatile int *)&S->done) return;
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ uint64_t full[kStages], empty[kStages];
    __shared__ uint64_t meta[kStages][2];         // first and one-past-last row of the stage
    __shared__ uint32_t sbp[kStages][kCons + 1];  // bptr of the stage's rows
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint64_t per_block = (nn + gridDim.x - 1) / gridDim.x;
    const uint64_t row0 = min(nn, blockIdx.x * per_block), row_end = min(nn, row0 + per_block);
    if (threadIdx.x == 0) {
        for (int i = 0; i < kStages; ++i) {
            bulk::mbar_init(&full[i], 1);
            bulk::mbar_init(&empty[i], kCons);
        }
        bulk::fence_barrier_init();
    }
    __syncthreads();
    bool timed_out = false;
    if (warp == kCons) {
        // ---------------- producer ----------------
        uint64_t g0 = row0;
        uint32_t b0 = row0 < row_end ? bptr[row0] : 0u;
        uint32_t k = 0, nissued = 0;  // stages whose full barrier got its arrival
        for (;; ++k) {
            const int slot = k % kStages;
            if (k >= (uint32_t)kStages) {
                const bool ok = bulk::mbar_wait(&empty[slot], ((k / kStages) - 1) & 1u);
                if (!__all_sync(0xffffffffu, ok)) {
                    timed_out = true;
                    break;
                }
            }
            if (g0 >= row_end) {  // sentinel stage: no rows, no bytes
                if (lane == 0) {
                    meta[slot][0] = g0;
                    meta[slot][1] = g0;
                    bulk::mbar_arrive(&full[slot]);
                }
                nissued = k + 1;
                break;
            }
            const uint64_t gi = g0 + 1 + lane;
            const bool in = lane < kCons && gi <= row_end;
            const uint32_t bi = in ? bptr[gi] : 0u;
            const unsigned fits = __ballot_sync(0xffffffffu, in && bi - b0 <= (uint32_t)kCap);
            const int nrows = __popc(fits);  // a prefix of the lanes: bptr is non-decreasing
            if (nrows == 0) {                 // a row wider than a stage (the levels' rows hold <= 128)
                timed_out = true;
                break;
            }
            const uint32_t b1 = __shfl_sync(0xffffffffu, bi, nrows - 1);
            if (lane < nrows) sbp[slot][lane + 1] = bi;
            if (lane == 0) sbp[slot][0] = b0;
            __syncwarp();
            if (lane == 0) {
                const uint64_t kb0 = 144ull * b0, kb1 = 144ull * b1;
                const uint64_t cb0 = (4ull * b0) & ~15ull, cb1 = (4ull * b1 + 15ull) & ~15ull;
                meta[slot][0] = g0;
                meta[slot][1] = g0 + nrows;
                unsigned char *dst = smem + (size_t)slot * St::kBytes;
                __threadfence_block();
                bulk::mbar_arrive_expect_tx(&full[slot], (uint32_t)((kb1 - kb0) + (cb1 - cb0)));
                const uint64_t pol = bulk::policy_evict_first();
                if (kb1 > kb0)
                    bulk::copy_g2s_hint(dst, reinterpret_cast<const unsigned char *>(K) + kb0, (uint32_t)(kb1 - kb0),
                                        &full[slot], pol);
                if (cb1 > cb0)
                    bulk::copy_g2s_hint(dst + St::kKBytes, reinterpret_cast<const unsigned char *>(bcol) + cb0,
                                        (uint32_t)(cb1 - cb0), &full[slot], pol);
            }
            g0 += nrows;
            b0 = b1;
            nissued = k + 1;
        }
        if (lane == 0) {
            if (timed_out && S) {
                atomicExch(&S->status, LMTG_ERR_TIMEOUT);
                atomicExch(&S->done, 1);
            }
            // leave only with no copy into this CTA's shared memory in flight (bounded waits)
            const uint32_t first = nissued > (uint32_t)kStages ? nissued - kStages : 0u;
            for (uint32_t s = first; s < nissued; ++s) bulk::mbar_wait(&full[s % kStages], (s / kStages) & 1u);
        }
    } else {
        // ---------------- consumers ----------------
        const float4 *x4 = reinterpret_cast<const float4 *>(x);
        for (uint32_t k = 0;; ++k) {
            const int slot = k % kStages;
            const bool ok = bulk::mbar_wait(&full[slot], (k / kStages) & 1u);  // every lane acquires
            if (!__all_sync(0xffffffffu, ok)) {
                timed_out = true;
                break;
            }
            const uint64_t g0 = meta[slot][0], g1 = meta[slot][1];
            if (g0 == g1) break;
            const float *sK = reinterpret_cast<const float *>(smem + (size_t)slot * St::kBytes);
            const uint32_t *sC = reinterpret_cast<const uint32_t *>(smem + (size_t)slot * St::kBytes + St::kKBytes);
            const uint32_t sb0 = sbp[slot][0];
            const uint64_t I = g0 + warp;
            bool released = false;
            if (I < g1) {
                const uint32_t rb = sbp[slot][warp], d = sbp[slot][warp + 1] - rb;
                const uint32_t kofs = 36u * (rb - sb0), cofs = rb - (sb0 & ~3u);
                const typename Epi::Pre pr = epi.pre(I, lane);
                float a[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
                for (uint32_t c0 = 0; c0 < d; c0 += 32) {
                    const uint32_t bl = c0 + lane;
                    const bool on = bl < d;
                    float m[36];
                    uint32_t j = 0;
                    if (on) {
#pragma unroll
                        for (int v = 0; v < 36; ++v) m[v] = sK[kofs + v * d + bl];
                        j = sC[cofs + bl];
                    }
                    if (c0 + 32 >= d) {  // the row's last chunk: the stage is no longer read
                        __syncwarp();
                        if (lane == 0) bulk::mbar_arrive(&empty[slot]);
                        released = true;
                    }
                    if (on) {
                        const float4 u = __ldg(x4 + 2 * (uint64_t)j), w = __ldg(x4 + 2 * (uint64_t)j + 1);
                        const float xv[6] = {u.x, u.y, u.z, u.w, w.x, w.y};
#pragma unroll
                        for (int r = 0; r < 6; ++r)
#pragma unroll
                            for (int cc = 0; cc < 6; ++cc) a[r] = fmaf(m[6 * r + cc], xv[cc], a[r]);
                    }
                }
                epi.row(I, reduce_scatter6(a, lane), lane, pr);
            }
            if (!released) {
                __syncwarp();
                if (lane == 0) bulk::mbar_arrive(&empty[slot]);
            }
        }
        if (timed_out && lane == 0 && S) {
            atomicExch(&S->status, LMTG_ERR_TIMEOUT);
            atomicExch(&S->done, 1);
        }
    }
}

}  // namespace lmtg
