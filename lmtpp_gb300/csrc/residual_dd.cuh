// FP64-accurate residual r = b - K x of the mixed solver's refinement without the FP64 pipe.
//
// GB300 issues FP64 at 2 lanes per clock per SM, so the FP64 warp-row residual (9 FMAs per
// block plus an FP64 warp reduction) is bound by that pipe, at a third of the HBM rate.  Here
// every FP64 operand is split on the integer pipe into two floats (hi + lo, 48 significant bits)
// and the row sums are formed in float-float arithmetic: each product K_ij x_j by the FMA-exact
// two-product of the high parts plus the cross terms, accumulated with the error-free two-sum
// and a running compensation (the compensated dot product of Ogita, Rump and Oishi, 2005).
// The relative error of a sum is a few units of 2^-48, against the FP64 sum's 2^-53; the mixed
// solver uses this kernel while the residual is above 1e-9 of |b|, where that rounding stays
// orders of magnitude below the residual, and the FP64 kernel below.  The residual is consumed
// only as the FP32 right-hand side of the next segment and through |r|^2, so it is written
// rounded to float.
//
// The matrix streams through shared memory by bulk copies (TMA), as in the FP32 bulk-copy SpMV:
// one producer warp moves runs of up to kCons rows (at most kCap blocks) into a ring of stages;
// consumer warp w takes row w of a stage, lane b its block b (wider rows in chunks of 32).
// Waits are bounded; a wait that gives up sets LMTG_ERR_TIMEOUT in the scalar slot's status.
#pragma once
#include "ffloat.cuh"
#include "spmv_bulk.cuh"

namespace lmtg {

namespace ff {

// running compensated sum (s, c) += (ph + pl) for a product split as ph + pl
__device__ __forceinline__ void acc(float &s, float &c, float ph, float pl) {
    float e;
    two_sum(s, ph, s, e);
    c += e + pl;
}

// (ah + al) (bh + bl) as ph + pl (the lo * lo term dropped)
__device__ __forceinline__ void mul_parts(float ah, float al, float bh, float bl, float &ph, float &pl) {
    ph = ah * bh;
    pl = fmaf(ah, bh, -ph);
    pl = fmaf(ah, bl, pl);
    pl = fmaf(al, bh, pl);
}

// reduce_scatter3 of compensated pairs: lane 8c (c < 3) ends with the warp's sum of component c
__device__ __forceinline__ void reduce_scatter3(float (&s)[3], float (&c)[3], int lane, float &rs, float &rc) {
    constexpr unsigned F = 0xffffffffu;
    const bool hi16 = (lane & 16) != 0, hi8 = (lane & 8) != 0;
    // slots 0..3 = components 0, 1, 2, 0 (zero); keep {0, 1} (hi16 clear) or {2, 3}
    const float ks0 = hi16 ? s[2] : s[0], kc0 = hi16 ? c[2] : c[0];
    const float ks1 = hi16 ? 0.f : s[1], kc1 = hi16 ? 0.f : c[1];
    const float ss0 = hi16 ? s[0] : s[2], sc0 = hi16 ? c[0] : c[2];
    const float ss1 = hi16 ? s[1] : 0.f, sc1 = hi16 ? c[1] : 0.f;
    float b0s, b0c, b1s, b1c, e;
    two_sum(ks0, __shfl_xor_sync(F, ss0, 16), b0s, e);
    b0c = kc0 + __shfl_xor_sync(F, sc0, 16) + e;
    two_sum(ks1, __shfl_xor_sync(F, ss1, 16), b1s, e);
    b1c = kc1 + __shfl_xor_sync(F, sc1, 16) + e;
    const float ts = hi8 ? b1s : b0s, tc = hi8 ? b1c : b0c;
    two_sum(ts, __shfl_xor_sync(F, hi8 ? b0s : b1s, 8), rs, e);
    rc = tc + __shfl_xor_sync(F, hi8 ? b0c : b1c, 8) + e;
#pragma unroll
    for (int m = 4; m >= 1; m >>= 1) {
        const float os = __shfl_xor_sync(F, rs, m), oc = __shfl_xor_sync(F, rc, m);
        two_sum(rs, os, rs, e);
        rc += oc + e;
    }
}

}  // namespace ff

template <int kCap>
struct Res64Stage {
    static_assert(kCap % 4 == 0 && kCap >= 96, "a stage holds at least one row of 96 blocks");
    static constexpr uint32_t kKBytes = 72u * kCap + 32u;  // FP64 values, 16-byte rounding on both ends
    static constexpr uint32_t kCBytes = 4u * kCap + 32u;   // column indices
    static constexpr uint32_t kBytes = kKBytes + kCBytes;
};

template <int kStages, int kCap>
constexpr size_t res64_smem_bytes() {
    return (size_t)kStages * Res64Stage<kCap>::kBytes;
}

// r32 = (float)(rscale (b - K x)) and |r32|^2 into o->rr (grid reduction on o->cnt_c); rscale is
// a power of two that keeps the squares of small residuals in the float range
template <int kStages, int kCap, int kCons, int kMinBlocks>
__global__ void __launch_bounds__(32 * (kCons + 1), kMinBlocks)
    k_residual_ff(const uint32_t *__restrict__ bptr, const uint32_t *__restrict__ bcol,
                  const double *__restrict__ K, const double *__restrict__ x, const double *__restrict__ b,
                  float rscale, float *__restrict__ r32, uint64_t nn, double *partials, PcgScalars *o) {
    static_assert(kCons >= 1 && kCons <= 31, "the producer sizes a stage with one warp of bptr loads");
    using St = Res64Stage<kCap>;
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ uint64_t full[kStages], empty[kStages];
    __shared__ uint64_t meta[kStages][4];         // first row, one past the last, first value, first column
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
    float racc = 0.f;
    bool timed_out = false;
    if (warp == kCons) {
        // ---------------- producer ----------------
        uint64_t g0 = row0;
        uint32_t b0 = row0 < row_end ? bptr[row0] : 0u;
        uint32_t k = 0, nissued = 0;
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
            const int nrows = __popc(fits);
            if (nrows == 0) {  // a row wider than a stage (the host keeps such patterns off this kernel)
                timed_out = true;
                break;
            }
            const uint32_t b1 = __shfl_sync(0xffffffffu, bi, nrows - 1);
            if (lane < nrows) sbp[slot][lane + 1] = bi;
            if (lane == 0) sbp[slot][0] = b0;
            __syncwarp();
            if (lane == 0) {
                const uint64_t kb0 = (72ull * b0) & ~15ull, kb1 = (72ull * b1 + 15ull) & ~15ull;
                const uint64_t cb0 = (4ull * b0) & ~15ull, cb1 = (4ull * b1 + 15ull) & ~15ull;
                meta[slot][0] = g0;
                meta[slot][1] = g0 + nrows;
                meta[slot][2] = kb0 / 8;
                meta[slot][3] = cb0 / 4;
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
            if (timed_out) atomicExch(&o->status, LMTG_ERR_TIMEOUT);
            const uint32_t first = nissued > (uint32_t)kStages ? nissued - kStages : 0u;
            for (uint32_t s = first; s < nissued; ++s) bulk::mbar_wait(&full[s % kStages], (s / kStages) & 1u);
        }
    } else {
        // ---------------- consumers ----------------
        for (uint32_t k = 0;; ++k) {
            const int slot = k % kStages;
            const bool ok = bulk::mbar_wait(&full[slot], (k / kStages) & 1u);
            if (!__all_sync(0xffffffffu, ok)) {
                timed_out = true;
                break;
            }
            const uint64_t g0 = meta[slot][0], g1 = meta[slot][1];
            if (g0 == g1) break;
            const double *sK = reinterpret_cast<const double *>(smem + (size_t)slot * St::kBytes);
            const uint32_t *sC = reinterpret_cast<const uint32_t *>(smem + (size_t)slot * St::kBytes + St::kKBytes);
            const uint64_t kbase = meta[slot][2], cbase = meta[slot][3];
            const uint64_t I = g0 + warp;
            bool released = false;
            if (I < g1) {
                const uint32_t rb = sbp[slot][warp], d = sbp[slot][warp + 1] - rb;
                // the row's right-hand side, loaded before the products
                ff::f2 bs{0.f, 0.f};
                if ((lane & 7) == 0 && lane < 24) bs = ff::split(b[3 * I + (lane >> 3)]);
                float s[3] = {0.f, 0.f, 0.f}, c[3] = {0.f, 0.f, 0.f};
                for (uint32_t c0 = 0; c0 < d; c0 += 32) {
                    const uint32_t bl_ = c0 + lane;
                    const bool on = bl_ < d;
                    double m[9];
                    uint32_t J = 0;
                    if (on) {
#pragma unroll
                        for (int v = 0; v < 9; ++v) m[v] = sK[kidx(rb, d, bl_, v) - kbase];
                        J = sC[rb + bl_ - cbase];
                    }
                    if (c0 + 32 >= d) {  // the row's last chunk: the stage is no longer read
                        __syncwarp();
                        if (lane == 0) bulk::mbar_arrive(&empty[slot]);
                        released = true;
                    }
                    if (on) {
                        ff::f2 xs[3];
#pragma unroll
                        for (int j = 0; j < 3; ++j) xs[j] = ff::split(__ldg(x + 3 * (uint64_t)J + j));
#pragma unroll
                        for (int r = 0; r < 3; ++r)
#pragma unroll
                            for (int j = 0; j < 3; ++j) {
                                const ff::f2 kv = ff::split(m[3 * r + j]);
                                float ph, pl;
                                ff::mul_parts(kv.h, kv.l, xs[j].h, xs[j].l, ph, pl);
                                ff::acc(s[r], c[r], ph, pl);
                            }
                    }
                }
                float qs, qc;
                ff::reduce_scatter3(s, c, lane, qs, qc);
                if ((lane & 7) == 0 && lane < 24) {
                    // r = b - q with b = bh + bl, q = qs + qc
                    float rh, e;
                    ff::two_sum(bs.h, -qs, rh, e);
                    const float ri = (rh + (e + (bs.l - qc))) * rscale;
                    r32[3 * I + (lane >> 3)] = ri;
                    racc = fmaf(ri, ri, racc);
                }
            }
            if (!released) {
                __syncwarp();
                if (lane == 0) bulk::mbar_arrive(&empty[slot]);
            }
        }
        if (timed_out && lane == 0) atomicExch(&o->status, LMTG_ERR_TIMEOUT);
    }
    __syncthreads();
    const float t[1] = {racc};
    double out[1];
    if (grid_reduce_t<1, 0u>(t, partials, &o->cnt_c, out) && threadIdx.x == 0) o->rr = out[0];
}

}  // namespace lmtg
