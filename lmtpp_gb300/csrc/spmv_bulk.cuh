// FP32 PCG SpMV with the matrix streamed through shared memory by the bulk-copy engine (TMA).
//
// Each CTA owns a contiguous range of node rows.  Since the planar per-row layout keeps the
// blocks of consecutive rows contiguous, the values and column indices of any run of rows
// are two contiguous byte ranges, so one producer warp moves them into a ring of kStages
// shared-memory stages with `cp.async.bulk` (one copy each, completion counted on the stage's
// "full" mbarrier).  Eight consumer warps take two rows each per stage, read their blocks from
// shared memory, give the stage back (its "empty" mbarrier) and only then gather p and
// multiply; a pair holding a row of more than 32 blocks (Tetra10 vertex rows) is taken as one
// list of up to 96 blocks and gives the stage back after its products.  The DRAM stream is thus
// decoupled from the latency of the p gathers, which in the warp-per-row-pair kernel sit on the
// same dependency chain as the matrix loads.
//
// Results are the ones of k_pcg_spmv (same q; pq summed in a different fixed order), and they
// are deterministic: the stage partition depends only on bptr.
//
// Every mbarrier wait is bounded (about a second of %globaltimer, and an iteration cap).  A
// wait that gives up sets LMTG_ERR_TIMEOUT and done in the PCG scalars; the producer then
// waits, bounded again, for its own copies in flight before the CTA exits.  The grid-reduction
// ticket (cnt_a) may stop part-way when a CTA gives up (later CTAs return at once on `done`):
// its count is only right because every PCG run uploads fresh scalars (tickets 0) and the host
// reads the status before trusting pq or alpha.
#pragma once
#include "solver_kernels.cuh"

namespace lmtg {

namespace bulk {

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_barrier_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    uint64_t state;
    asm volatile("mbarrier.arrive.shared::cta.b64 %0, [%1];" : "=l"(state) : "r"(smem_addr(bar)) : "memory");
    (void)state;
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    uint64_t state;
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 %0, [%1], %2;"
                 : "=l"(state)
                 : "r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
    (void)state;
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// Wait until the phase of the given parity has completed; false after ~1 s (or 2^24 polls).
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = globaltimer_ns();
    for (uint32_t it = 1; it < (1u << 24); ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((it & 63u) == 0 && globaltimer_ns() - t0 > 1000000000ull) return false;
    }
    return false;
}
// Global -> shared bulk copy; dst, src and bytes are multiples of 16.
__device__ __forceinline__ void copy_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}
// The same with an L2 cache policy (evict_first for data read once).
__device__ __forceinline__ uint64_t policy_evict_first() {
    uint64_t pol;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}
__device__ __forceinline__ void copy_g2s_hint(void *dst, const void *src, uint32_t bytes, uint64_t *bar,
                                              uint64_t pol) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, "
        "[%3], %4;" ::"r"(smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar)), "l"(pol)
        : "memory");
}

}  // namespace bulk

// kCons consumer warps (two rows each per stage) + one producer warp
template <int kCons>
constexpr int bulk_threads() {
    return 32 * (kCons + 1);
}

template <int kCap>
struct BulkStage {
    static_assert(kCap % 4 == 0 && kCap >= 96, "a stage holds at least one row of 96 blocks");
    static constexpr uint32_t kKBytes = 36u * kCap + 32u;  // values, 16-byte rounding on both ends
    static constexpr uint32_t kCBytes = 4u * kCap + 32u;   // column indices
    static constexpr uint32_t kBytes = kKBytes + kCBytes;
};

// Shared-memory bytes of one CTA for kStages stages (dynamic part).
template <int kStages, int kCap>
constexpr size_t bulk_smem_bytes() {
    return (size_t)kStages * BulkStage<kCap>::kBytes;
}

// Row epilogues of the bulk-copy SpMV.  pre() loads what the epilogue of row I needs before the
// row's products (its loads then overlap the gathers); row() receives the row sums in the
// reduce_scatter3 layout (lane 8c holds component c of row I; every lane of the warp calls it)
// and may add to the thread's partial `acc`; with kReduce the partials are reduced over the grid
// on ticket() and final() runs once with the total.
//   EpiPcg   q = K p and p.q -> pq, alpha (the PCG's SpMV)
struct EpiPcg {
    float *q;
    static constexpr bool kReduce = true;
    struct Pre {};
    __device__ __forceinline__ Pre pre(uint64_t, int, const float *) const { return {}; }
    __device__ __forceinline__ void row(uint64_t I, float qi, int lane, const float *__restrict__ p, float &acc,
                                        const Pre &) const {
        if ((lane & 7) == 0 && lane < 24) {
            q[3 * I + (lane >> 3)] = qi;
            acc = fmaf(p[4 * I + (lane >> 3)], qi, acc);
        }
    }
    __device__ static unsigned *ticket(PcgScalars *S) { return &S->cnt_a; }
    __device__ void final(PcgScalars *S, double v) const {
        S->pq = v;
        S->alpha = S->rz / (v + (v == 0.0 ? 1.0 : 0.0));
    }
};

template <int kStages, int kCap, int kCons, bool kEvictFirst, int kMinBlocks, class Epi = EpiPcg>
__global__ void __launch_bounds__(bulk_threads<kCons>(), kMinBlocks)
    k_pcg_spmv_bulk(const uint32_t *__restrict__ bptr, const uint32_t *__restrict__ bcol,
                    const float *__restrict__ K, const float *__restrict__ p, Epi epi,
                    uint64_t nn, PcgScalars *S, double *partials) {
    constexpr int VS = 4;
    constexpr int kBulkConsumers = kCons, kBulkStageRows = 2 * kCons;
    static_assert(kBulkStageRows <= 32, "the producer sizes a stage with one warp of bptr loads");
    using St = BulkStage<kCap>;
    if (*(volatile int *)&S->done) return;
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ uint64_t full[kStages], empty[kStages];
    __shared__ uint64_t meta[kStages][4];                 // g0, g1, first value, first column
    __shared__ uint32_t sbp[kStages][kBulkStageRows + 1];  // bptr of the stage's rows
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint64_t per_block = (nn + gridDim.x - 1) / gridDim.x;
    const uint64_t row0 = min(nn, blockIdx.x * per_block), row_end = min(nn, row0 + per_block);
    if (threadIdx.x == 0) {
        for (int i = 0; i < kStages; ++i) {
            bulk::mbar_init(&full[i], 1);
            bulk::mbar_init(&empty[i], kBulkConsumers);
        }
        bulk::fence_barrier_init();
    }
    __syncthreads();
    float acc = 0.f;
    bool timed_out = false;
    if (warp == kBulkConsumers) {
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
            const bool in = lane < kBulkStageRows && gi <= row_end;
            const uint32_t bi = in ? bptr[gi] : 0u;
            const unsigned fits = __ballot_sync(0xffffffffu, in && bi - b0 <= (uint32_t)kCap);
            const int nrows = __popc(fits);  // a prefix of the lanes: bptr is non-decreasing
            if (nrows == 0) {                 // a row wider than a stage (excluded by the pattern)
                timed_out = true;
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
                unsigned char *dst = smem + (size_t)slot * St::kBytes;
                __threadfence_block();
                bulk::mbar_arrive_expect_tx(&full[slot], (uint32_t)((kb1 - kb0) + (cb1 - cb0)));
                const unsigned char *srcK = reinterpret_cast<const unsigned char *>(K) + kb0;
                const unsigned char *srcC = reinterpret_cast<const unsigned char *>(bcol) + cb0;
                if (kEvictFirst) {
                    const uint64_t pol = bulk::policy_evict_first();
                    bulk::copy_g2s_hint(dst, srcK, (uint32_t)(kb1 - kb0), &full[slot], pol);
                    bulk::copy_g2s_hint(dst + St::kKBytes, srcC, (uint32_t)(cb1 - cb0), &full[slot], pol);
                } else {
                    bulk::copy_g2s(dst, srcK, (uint32_t)(kb1 - kb0), &full[slot]);
                    bulk::copy_g2s(dst + St::kKBytes, srcC, (uint32_t)(cb1 - cb0), &full[slot]);
                }
            }
            g0 += nrows;
            b0 = b1;
            nissued = k + 1;
        }
        if (lane == 0) {
            if (timed_out) {
                atomicExch(&S->status, LMTG_ERR_TIMEOUT);
                atomicExch(&S->done, 1);
            }
            // The CTA leaves only when no copy into its shared memory is in flight: wait (bounded)
            // for the last stage issued on each slot.  When the consumers took every stage these
            // phases are complete and each wait returns at once; when they gave up early (a
            // timeout) the copies are still landing here.
            const uint32_t first = nissued > (uint32_t)kStages ? nissued - kStages : 0u;
            for (uint32_t s = first; s < nissued; ++s) bulk::mbar_wait(&full[s % kStages], (s / kStages) & 1u);
        }
    } else {
        // ---------------- consumers ----------------
        auto xnode = [&](uint64_t J, float &a, float &b, float &c) { NodeVec<float, VS>::load(p, J, a, b, c); };
        using Pre = typename Epi::Pre;
        auto finish = [&](uint64_t I, float qi, const Pre &pr) { epi.row(I, qi, lane, p, acc, pr); };
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
            const uint64_t kbase = meta[slot][2], cbase = meta[slot][3];
            const uint64_t I = g0 + 2 * warp;
            bool released = false;
            if (I < g1) {
                const bool has1 = I + 1 < g1;
                const int li = (int)(I - g0);
                const uint32_t rb0 = sbp[slot][li], re0 = sbp[slot][li + 1];
                const uint32_t rb1 = has1 ? re0 : 0u, re1 = has1 ? sbp[slot][li + 2] : 0u;
                const uint32_t d0 = re0 - rb0, d1 = re1 - rb1;
                const Pre pre0 = epi.pre(I, lane, p), pre1 = has1 ? epi.pre(I + 1, lane, p) : Pre{};
                if (d0 <= 32 && d1 <= 32) {
                    float m0[9], m1[9];
                    const bool on0 = (uint32_t)lane < d0, on1 = (uint32_t)lane < d1;
#pragma unroll
                    for (int v = 0; v < 9; ++v) {
                        m0[v] = on0 ? sK[kidx(rb0, d0, lane, v) - kbase] : 0.f;
                        m1[v] = on1 ? sK[kidx(rb1, d1, lane, v) - kbase] : 0.f;
                    }
                    const uint32_t j0 = on0 ? sC[rb0 + lane - cbase] : 0u;
                    const uint32_t j1 = on1 ? sC[rb1 + lane - cbase] : 0u;
                    __syncwarp();
                    if (lane == 0) bulk::mbar_arrive(&empty[slot]);
                    released = true;
                    float x00 = 0, x01 = 0, x02 = 0, x10 = 0, x11 = 0, x12 = 0;
                    if (on0) xnode(j0, x00, x01, x02);
                    if (on1) xnode(j1, x10, x11, x12);
                    float a00 = 0, a01 = 0, a02 = 0, a10 = 0, a11 = 0, a12 = 0;
                    block_fma(m0, x00, x01, x02, a00, a01, a02);
                    block_fma(m1, x10, x11, x12, a10, a11, a12);
                    const float q0 = reduce_scatter3(a00, a01, a02, lane);
                    const float q1 = reduce_scatter3(a10, a11, a12, lane);
                    finish(I, q0, pre0);
                    if (has1) finish(I + 1, q1, pre1);
                } else if (d0 + d1 <= 96) {
                    // a wide pair (a Tetra10 vertex row of 65 blocks and its neighbour): the two
                    // rows' blocks as one list, lane l taking blocks l, l + 32, l + 64, so that
                    // all of the pair's gathers are in flight before the products
                    const uint32_t dd = d0 + d1;
                    float xs[3][3];
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        const uint32_t f = 32 * c + lane;
                        xs[c][0] = xs[c][1] = xs[c][2] = 0.f;
                        if (f < dd) {
                            const uint32_t col = f < d0 ? sC[rb0 + f - cbase] : sC[rb1 + (f - d0) - cbase];
                            xnode(col, xs[c][0], xs[c][1], xs[c][2]);
                        }
                    }
                    float a00 = 0.f, a01 = 0.f, a02 = 0.f, a10 = 0.f, a11 = 0.f, a12 = 0.f;
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        const uint32_t f = 32 * c + lane;
                        if (f < dd) {
                            const bool second = f >= d0;
                            const uint32_t rb = second ? rb1 : rb0, d = second ? d1 : d0, bl = second ? f - d0 : f;
                            float m[9];
#pragma unroll
                            for (int v = 0; v < 9; ++v) m[v] = sK[kidx(rb, d, bl, v) - kbase];
                            float t0 = 0.f, t1 = 0.f, t2 = 0.f;
                            block_fma(m, xs[c][0], xs[c][1], xs[c][2], t0, t1, t2);
                            a00 += second ? 0.f : t0;
                            a01 += second ? 0.f : t1;
                            a02 += second ? 0.f : t2;
                            a10 += second ? t0 : 0.f;
                            a11 += second ? t1 : 0.f;
                            a12 += second ? t2 : 0.f;
                        }
                    }
                    const float q0 = reduce_scatter3(a00, a01, a02, lane);
                    const float q1 = reduce_scatter3(a10, a11, a12, lane);
                    finish(I, q0, pre0);
                    if (has1) finish(I + 1, q1, pre1);
                } else {
                    for (int r = 0; r < (has1 ? 2 : 1); ++r) {
                        const uint32_t rb = r ? rb1 : rb0, d = r ? d1 : d0;
                        // rows of up to 96 blocks (the pattern's limit): the three gathers of a
                        // lane are issued before the products
                        float xs[3][3];
#pragma unroll
                        for (int c = 0; c < 3; ++c) {
                            const uint32_t bl = 32 * c + lane;
                            xs[c][0] = xs[c][1] = xs[c][2] = 0.f;
                            if (bl < d) xnode(sC[rb + bl - cbase], xs[c][0], xs[c][1], xs[c][2]);
                        }
                        float a0 = 0.f, a1 = 0.f, a2 = 0.f;
#pragma unroll
                        for (int c = 0; c < 3; ++c) {
                            const uint32_t bl = 32 * c + lane;
                            if (bl < d) {
                                float m[9];
#pragma unroll
                                for (int v = 0; v < 9; ++v) m[v] = sK[kidx(rb, d, bl, v) - kbase];
                                block_fma(m, xs[c][0], xs[c][1], xs[c][2], a0, a1, a2);
                            }
                        }
                        for (uint32_t c0 = 96; c0 < d; c0 += 32) {  // not reached: rows hold <= 96
                            const uint32_t bl = c0 + lane;
                            if (bl < d) {
                                float m[9];
#pragma unroll
                                for (int v = 0; v < 9; ++v) m[v] = sK[kidx(rb, d, bl, v) - kbase];
                                float x0, x1, x2;
                                xnode(sC[rb + bl - cbase], x0, x1, x2);
                                block_fma(m, x0, x1, x2, a0, a1, a2);
                            }
                        }
                        finish(I + r, reduce_scatter3(a0, a1, a2, lane), r ? pre1 : pre0);
                    }
                }
            }
            if (!released) {
                __syncwarp();
                if (lane == 0) bulk::mbar_arrive(&empty[slot]);
            }
        }
        if (timed_out && lane == 0) {
            atomicExch(&S->status, LMTG_ERR_TIMEOUT);
            atomicExch(&S->done, 1);
        }
    }
    __syncthreads();
    if constexpr (Epi::kReduce) {
        const float tacc[1] = {acc};
        double out[1];
        if (grid_reduce_t<1, 0u>(tacc, partials, Epi::ticket(S), out) && threadIdx.x == 0) epi.final(S, out[0]);
    }
}

}  // namespace lmtg
