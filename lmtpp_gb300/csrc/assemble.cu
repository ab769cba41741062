// assemble.cu -- atomic-free gather assembly, penalty constraints, block-Jacobi inverses.
//
// Replaces the emitted scatter  matrix(indices[a]+o, indices[b]+o) += tmp_a_b  under the
// global assembly mutex (formal_lf/calculate_matrix.py:86-98, include/containers/vec_mt.h:39-62)
// and assemble_constraints (include/formulation/formulation.h:1028-1071).
//
// Assembly: each stored 3x3 block of K (BSR, full symmetric pattern) is the sum of the element
// blocks its gather list names (element order, built once by pattern.cu), transposed when the
// element pair is (b,a) with a > b.  No atomics, no search, a deterministic summation order.
// FP64 assembly can write the FP32 inner operator in the same pass (rounded from the FP64 sum).
#include <cstring>
#include <type_traits>

#include <algorithm>
#include <cstring>
#include "lmtg_internal.cuh"

namespace lmtg {

// IEEE round-to-nearest-even double -> float on the integer pipe (GB300 issues FP64 and its
// conversions at 2 lanes per clock per SM): finite values in the normal float range are rounded
// from the bit pattern, zeros and double subnormals give a signed zero, and the rest (float
// subnormals, overflow, inf, nan) go through the conversion instruction.  Results equal the
// conversion's.
__device__ __forceinline__ float d2f_rn(double d) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(d);
    const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
    const int ef = (int)((b >> 52) & 0x7ffu);
    if (ef == 0) return __uint_as_float(sign);
    const int e = ef - 1023 + 127;
    if (e <= 0 || e >= 255) return (float)d;
    const unsigned long long man = b & 0xfffffffffffffull;
    unsigned keep = (unsigned)(man >> 29);
    const unsigned rem = (unsigned)man & 0x1fffffffu;
    keep += (rem > 0x10000000u || (rem == 0x10000000u && (keep & 1u))) ? 1u : 0u;
    return __uint_as_float(sign | (((unsigned)e << 23) + keep));  // a mantissa carry bumps the exponent
}

template <class A>
__device__ __forceinline__ float to_f32(A v) {
    if constexpr (sizeof(A) == 8) return d2f_rn(v);
    else return v;
}

// One warp per node row, its blocks 32 at a time (a group).  The contributions of a group's
// blocks are one contiguous range of the gather list, so the warp first copies the group's
// element records (up to kAsmChunk) into shared memory -- lane t loads value t % 9 of record
// t / 9, all loads independent.  The sums are then spread evenly over the lanes: the group's
// 9 x (records) addends, ordered by (block, component, contribution), are cut into 32 equal
// ranges and each lane sums its range in order, closing every output it completes; an output
// that straddles two lanes is the earlier lane's partial plus the later lane's.  Every lane
// issues the same number of adds whatever the blocks' contribution counts (1 to 8 on a Hexa8
// grid), which matters on GB300's narrow FP64 pipe.  Groups with more records than a chunk or
// an output longer than a lane's range (Tetra10 vertex rows), or a block without contributions,
// take the per-block walk instead: lane b sums block b's records in element order.  Either way the order is fixed: results are
// deterministic.  Component v of a block goes to kidx(rb, deg, b, v): coalesced stores.
constexpr int kAsmWarps = 4, kAsmChunk = 64;  // 28 KB of static shared memory per CTA (FP64)

template <class TS, bool kW64, bool kW32>
__global__ void __launch_bounds__(32 * kAsmWarps)
    k_assemble(const uint32_t *__restrict__ bptr, uint64_t nn, const uint32_t *__restrict__ gptr,
               const uint32_t *__restrict__ gsrc, const TS *__restrict__ Ke, double *__restrict__ K64,
               float *__restrict__ K32) {
    typedef typename std::conditional<sizeof(TS) == 8, double, float>::type Acc;
    __shared__ TS rec[kAsmWarps][kAsmChunk * 9];
    __shared__ Acc outs[kAsmWarps][32 * 9];
    __shared__ uint32_t ofs[kAsmWarps][33];
    __shared__ unsigned char trf[kAsmWarps][kAsmChunk];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    TS *R = rec[warp];
    Acc *Out = outs[warp];
    uint32_t *O = ofs[warp];
    unsigned char *Tr = trf[warp];
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    auto store = [&](uint32_t rb, uint32_t deg, uint32_t b, const Acc (&s)[9]) {
#pragma unroll
        for (int v = 0; v < 9; ++v) {
            const uint64_t idx = kidx(rb, deg, b, v);
            if (kW64) K64[idx] = (double)s[v];
            if (kW32) K32[idx] = to_f32(s[v]);
        }
    };
    for (uint64_t I = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; I < nn; I += nw) {
        const uint32_t rb = __ldg(bptr + I), deg = __ldg(bptr + I + 1) - rb;
        for (uint32_t bg = 0; bg < deg; bg += 32) {
            const uint32_t nb = min(32u, deg - bg);
            const bool on = (uint32_t)lane < nb;
            const uint32_t gs = __ldg(gptr + rb + bg), ge = __ldg(gptr + rb + bg + nb);
            const uint32_t my0 = on ? __ldg(gptr + rb + bg + lane) : 0u;
            const uint32_t my1 = on ? __ldg(gptr + rb + bg + lane + 1) : 0u;
            const uint32_t nrec = ge - gs, W = 9 * nrec, P = (W + 31) / 32;
            const uint32_t maxcnt = __reduce_max_sync(0xffffffffu, my1 - my0);
            const uint32_t mincnt = __reduce_min_sync(0xffffffffu, on ? my1 - my0 : ~0u);
            if (nrec <= (uint32_t)kAsmChunk && maxcnt <= P && mincnt > 0) {
#pragma unroll 6
                for (uint32_t t = lane; t < W; t += 32) {
                    const uint32_t k = t / 9, v = t - 9 * k;
                    const uint32_t src = __ldg(gsrc + gs + k);
                    R[t] = __ldg(Ke + (uint64_t)(src >> 1) * 9 + v);
                    if (v == 0) Tr[k] = (unsigned char)(src & 1u);
                }
                if (on) O[lane] = my0 - gs;
                if (lane == 0) O[nb] = nrec;
                __syncwarp();
                // this lane's addends [j0, j1): output (b, v) holds addends 9 O[b] + v cnt_b + c
                const uint32_t j0 = min(W, lane * P), j1 = min(W, j0 + P);
                Acc s = (Acc)0, head = (Acc)0, tail = (Acc)0;
                uint32_t head_id = ~0u, tail_id = ~0u;
                if (j0 < j1) {
                    uint32_t b = 0;
                    while (9 * O[b + 1] <= j0) ++b;
                    uint32_t cnt = O[b + 1] - O[b], rel = j0 - 9 * O[b];
                    uint32_t v = rel / cnt, c = rel - v * cnt;
                    bool first_partial = c != 0;  // the first output began in the previous lane
                    for (uint32_t j = j0; j < j1; ++j) {
                        const uint32_t k = O[b] + c;
                        const uint32_t vv = Tr[k] ? (v % 3) * 3 + v / 3 : v;
                        const Acc x = (Acc)R[9 * k + vv];
                        s = c == 0 ? x : s + x;
                        if (c + 1 == cnt) {  // output (b, v) complete
                            if (first_partial) {
                                head = s;
                                head_id = 9 * b + v;
                                first_partial = false;
                            } else {
                                Out[9 * b + v] = s;
                            }
                            c = 0;
                            if (++v == 9) {
                                v = 0;
                                ++b;
                                cnt = b < nb ? O[b + 1] - O[b] : 1u;
                            }
                        } else {
                            ++c;
                        }
                    }
                    if (c != 0) {  // the last output continues in the next lane
                        tail = s;
                        tail_id = 9 * b + v;
                    }
                }
                const Acc prev = __shfl_up_sync(0xffffffffu, tail, 1);
                const uint32_t prev_id = __shfl_up_sync(0xffffffffu, tail_id, 1);
                if (lane > 0 && head_id != ~0u && prev_id == head_id) Out[head_id] = prev + head;
                __syncwarp();
                if (on) {
                    Acc o[9];
#pragma unroll
                    for (int v = 0; v < 9; ++v) o[v] = Out[9 * lane + v];
                    store(rb, deg, bg + lane, o);
                }
                __syncwarp();
            } else if (on) {
                Acc o[9];
#pragma unroll
                for (int v = 0; v < 9; ++v) o[v] = (Acc)0;
                for (uint32_t g = my0; g < my1; ++g) {
                    const uint32_t src = __ldg(gsrc + g);
                    const TS *e = Ke + (uint64_t)(src >> 1) * 9;
                    const bool tr = (src & 1u) != 0;
#pragma unroll
                    for (int v = 0; v < 9; ++v) o[v] += (Acc)__ldg(e + (tr ? (v % 3) * 3 + v / 3 : v));
                }
                store(rb, deg, bg + lane, o);
            }
        }
    }
}

void assemble_matrix(lmtg_ctx *c, bool from64, bool want64, bool want32) {
    const int T = 32 * kAsmWarps;
    const int grid = grid_for(c, c->nn * 32, T, 8);
    if (from64) {
        if (want64 && want32)
            k_assemble<double, true, true><<<grid, T, 0, c->stream>>>(c->bptr.p, c->nn, c->gptr.p, c->gsrc.p,
                                                                      c->Ke64.p, c->K64.p, c->K32.p);
        else if (want64)
            k_assemble<double, true, false><<<grid, T, 0, c->stream>>>(c->bptr.p, c->nn, c->gptr.p, c->gsrc.p,
                                                                       c->Ke64.p, c->K64.p, nullptr);
        else
            k_assemble<double, false, true><<<grid, T, 0, c->stream>>>(c->bptr.p, c->nn, c->gptr.p, c->gsrc.p,
                                                                       c->Ke64.p, nullptr, c->K32.p);
    } else {
        k_assemble<float, false, true><<<grid, T, 0, c->stream>>>(c->bptr.p, c->nn, c->gptr.p, c->gsrc.p,
                                                                  c->Ke32.p, nullptr, c->K32.p);
    }
    LMTG_CUDA(cudaGetLastError());
    c->launches += 1;
}

// ---- penalty constraints ----
// max|diag K|: diagonal entries are non-negative-signed after fabs, so the IEEE bit pattern
// orders like the value and an integer atomicMax is exact.
template <class T>
__global__ void k_max_diag(const uint32_t *__restrict__ bptr, const uint32_t *__restrict__ bdiag,
                           const T *__restrict__ K, uint64_t nn, const uint32_t *__restrict__ sys,
                           unsigned long long *out) {
    // grid-stride over whole warps so that every lane reaches the shuffles below
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i0 = blockIdx.x * (uint64_t)blockDim.x + (threadIdx.x & ~31u); i0 < nn; i0 += stride) {
        const uint64_t i = i0 + (threadIdx.x & 31);
        double m = 0;
        uint32_t s = 0;
        if (i < nn) {
            const uint32_t rb = bptr[i], deg = bptr[i + 1] - rb, d = bdiag[i] - rb;
            m = fmax(fabs((double)K[kidx(rb, deg, d, 0)]),
                     fmax(fabs((double)K[kidx(rb, deg, d, 4)]), fabs((double)K[kidx(rb, deg, d, 8)])));
            s = sys ? sys[i] : 0u;
        }
        // one system per warp (the usual case): one atomic; otherwise one per lane
        const uint32_t s0 = __shfl_sync(0xffffffffu, s, 0);
        if (__all_sync(0xffffffffu, i >= nn || s == s0)) {
            m = warp_max(m);
            if ((threadIdx.x & 31) == 0) atomicMax(out + s0, (unsigned long long)__double_as_longlong(m));
        } else if (i < nn) {
            atomicMax(out + s, (unsigned long long)__double_as_longlong(m));
        }
    }
}

template <class T>
__global__ void k_penalty(const uint32_t *__restrict__ bptr, const uint32_t *__restrict__ bdiag, T *K, double *F,
                          const uint32_t *__restrict__ dof, const double *__restrict__ coef,
                          const double *__restrict__ res, uint64_t nc, double penalty,
                          const uint32_t *__restrict__ sys, const unsigned long long *md_bits, bool mat,
                          bool vec) {
    for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < nc;
         k += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t j = dof[k];
        const double md = __longlong_as_double((long long)md_bits[sys ? sys[j / 3] : 0u]);
        const double C = coef[k] * md * penalty;
        if (vec) atomicAdd(F + j, C * res[k]);
        if (mat) {
            const uint32_t I = j / 3, rb = bptr[I];
            atomicAdd(K + kidx(rb, bptr[I + 1] - rb, bdiag[I] - rb, 4 * (j % 3)), (T)(C * coef[k]));
        }
    }
}

__global__ void k_round_constrained(const uint32_t *__restrict__ bptr,
                                    const uint32_t *__restrict__ bdiag, const double *K64,
                                    float *K32, const uint32_t *__restrict__ dof, uint64_t nc) {
    for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < nc;
         k += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t j = dof[k], I = j / 3, rb = bptr[I];
        const uint64_t idx = kidx(rb, bptr[I + 1] - rb, bdiag[I] - rb, 4 * (j % 3));
        K32[idx] = (float)K64[idx];
    }
}

// ---- exact constraints (penalty 0) ----
// The reference adds Lagrange-multiplier rows for a zero penalty (formulation.h:1072-1088) and
// needs its LDL solver for the indefinite system.  For constraints coef u_j = res on one
// unknown each, the same solution follows from elimination, which keeps K SPD for the PCG:
// u_bar_j = res / coef; F_k -= (K u_bar)_k; rows and columns j of K become zero but for the
// diagonal; F_j = K_jj u_bar_j.
__global__ void k_elim_values(const uint32_t *__restrict__ dof, const double *__restrict__ coef,
                              const double *__restrict__ res, uint64_t nc, double *__restrict__ ubar,
                              uint8_t *__restrict__ mask) {
    for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < nc; k += (uint64_t)gridDim.x * blockDim.x) {
        ubar[dof[k]] = res[k] / coef[k];
        mask[dof[k]] = 1;
    }
}

// warp per node row, lane per block: zero the constrained rows and columns but the diagonal
template <class T>
__global__ void k_eliminate(const uint32_t *__restrict__ bptr, const uint32_t *__restrict__ bcol, uint64_t nn,
                            const uint8_t *__restrict__ mask, T *__restrict__ K, float *__restrict__ K32) {
    const int lane = threadIdx.x & 31;
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t I = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; I < nn; I += nw) {
        const uint32_t rb = bptr[I], deg = bptr[I + 1] - rb;
        const bool mi[3] = {mask[3 * I] != 0, mask[3 * I + 1] != 0, mask[3 * I + 2] != 0};
        for (uint32_t b = lane; b < deg; b += 32) {
            const uint64_t J = bcol[rb + b];
            const bool mj[3] = {mask[3 * J] != 0, mask[3 * J + 1] != 0, mask[3 * J + 2] != 0};
#pragma unroll
            for (int v = 0; v < 9; ++v) {
                const int r = v / 3, cc = v % 3;
                if ((mi[r] || mj[cc]) && !(J == I && r == cc)) {
                    const uint64_t idx = kidx(rb, deg, b, v);
                    if (K) K[idx] = (T)0;
                    if (K32) K32[idx] = 0.0f;
                }
            }
        }
    }
}

__global__ void k_elim_rhs(const double *__restrict__ w, uint64_t n, double *__restrict__ F) {
    for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x)
        F[k] -= w[k];
}
__global__ void k_elim_rhs_fix(const uint32_t *__restrict__ bptr, const uint32_t *__restrict__ bdiag,
                               const double *__restrict__ K, const uint32_t *__restrict__ dof, uint64_t nc,
                               const double *__restrict__ ubar, double *__restrict__ F) {
    for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < nc; k += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t j = dof[k], I = j / 3, rb = bptr[I];
        const double kjj = K[kidx(rb, bptr[I + 1] - rb, bdiag[I] - rb, 4 * (j % 3))];
        F[j] = kjj * ubar[j];
    }
}

static void apply_elimination(lmtg_ctx *c, bool mat, bool vec) {
    LMTG_CHECK(c->have64, LMTG_ERR_UNSUPPORTED, "exact constraints need the FP64 assembly");
    cudaStream_t s = c->stream;
    const int T = 256;
    DBuf<double> ubar;
    DBuf<uint8_t> mask;
    ubar.alloc(c->n);
    mask.alloc(c->n);
    LMTG_CUDA(cudaMemsetAsync(ubar.p, 0, c->n * sizeof(double), s));
    LMTG_CUDA(cudaMemsetAsync(mask.p, 0, c->n, s));
    k_elim_values<<<grid_for(c, c->nc, T), T, 0, s>>>(c->cdof.p, c->ccoef.p, c->cres.p, c->nc, ubar.p, mask.p);
    c->launches += 1;
    if (mat) {
        // coupling of the prescribed values, from the matrix before elimination
        c->elim_w.alloc(c->n);
        spmv64(c, ubar.p, c->elim_w.p);
        k_eliminate<double><<<grid_for(c, c->nn * 32, T, 8), T, 0, s>>>(c->bptr.p, c->bcol.p, c->nn, mask.p,
                                                                        c->K64.p, c->have32 ? c->K32.p : nullptr);
        c->launches += 1;
    }
    if (vec) {
        LMTG_CHECK(c->elim_w.p, LMTG_ERR_STATE, "exact constraints: assemble the matrix first");
        k_elim_rhs<<<grid_for(c, c->n, T), T, 0, s>>>(c->elim_w.p, c->n, c->F.p);
        k_elim_rhs_fix<<<grid_for(c, c->nc, T), T, 0, s>>>(c->bptr.p, c->bdiag.p, c->K64.p, c->cdof.p, c->nc,
                                                           ubar.p, c->F.p);
        c->launches += 2;
    }
    LMTG_CUDA(cudaGetLastError());
    LMTG_CUDA(cudaStreamSynchronize(s));
}

// K(i,i) += max|diag| * levenberg_marquadt on every diagonal entry (formulation.h:1033-1034),
// with the max|diag| of the node's system
template <class T>
__global__ void k_add_diag(const uint32_t *__restrict__ bptr, const uint32_t *__restrict__ bdiag, T *K,
                           float *K32, uint64_t nn, const uint32_t *__restrict__ sys,
                           const unsigned long long *md_bits, double lm) {
    for (uint64_t I = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; I < nn;
         I += (uint64_t)gridDim.x * blockDim.x) {
        const double md = __longlong_as_double((long long)md_bits[sys ? sys[I] : 0u]);
        const uint32_t rb = bptr[I], deg = bptr[I + 1] - rb, d = bdiag[I] - rb;
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            const uint64_t idx = kidx(rb, deg, d, 4 * r);
            K[idx] = (T)((double)K[idx] + md * lm);
            if (K32) K32[idx] = (float)K[idx];
        }
    }
}

// max|diag| (one per system of a batch, nsys > 0, else one for the whole matrix), the
// Levenberg-Marquardt diagonal term, then the constraints: penalty terms, or elimination for a
// zero penalty.
void apply_penalty(lmtg_ctx *c, bool mat, bool vec) {
    const bool lm = mat && c->levenberg_marquadt != 0.0;
    if (c->nc == 0 && !lm) return;
    const bool exact = c->nc > 0 && c->penalty == 0.0;
    const uint32_t ns = c->nsys ? c->nsys : 1;
    const uint32_t *sys = c->nsys ? c->sys_of_node.p : nullptr;
    DBuf<unsigned long long> md;
    md.alloc(ns);
    const int T = 256;
    auto upload_scales = [&](const std::vector<double> &v) {
        std::vector<unsigned long long> bits(ns);
        for (uint32_t m = 0; m < ns; ++m) memcpy(&bits[m], &v[m], sizeof(double));
        LMTG_CUDA(cudaMemcpyAsync(md.p, bits.data(), ns * sizeof(unsigned long long), cudaMemcpyHostToDevice,
                                  c->stream));
        LMTG_CUDA(cudaStreamSynchronize(c->stream));
    };
    if (mat && c->penalty_scale > 0.0) {
        // caller-fixed scale (held constant for sensitivities w.r.t. the material)
        upload_scales(std::vector<double>(ns, c->penalty_scale));
    } else if (mat) {
        // max|diag| of the freshly assembled K, before any constraint (formulation.h:1029-1030)
        LMTG_CUDA(cudaMemsetAsync(md.p, 0, ns * sizeof(unsigned long long), c->stream));
        if (c->have64)
            k_max_diag<double><<<grid_for(c, c->nn, T), T, 0, c->stream>>>(c->bptr.p, c->bdiag.p, c->K64.p, c->nn,
                                                                           sys, md.p);
        else
            k_max_diag<float><<<grid_for(c, c->nn, T), T, 0, c->stream>>>(c->bptr.p, c->bdiag.p, c->K32.p, c->nn,
                                                                          sys, md.p);
        c->launches += 1;
    } else {
        // vector-only assembly reuses the max|diag| of the last matrix assembly
        upload_scales(c->nsys ? c->h_sys_max_diag : std::vector<double>(1, c->max_diag));
    }
    if (lm) {
        if (c->have64)
            k_add_diag<double><<<grid_for(c, c->nn, T), T, 0, c->stream>>>(
                c->bptr.p, c->bdiag.p, c->K64.p, c->have32 ? c->K32.p : nullptr, c->nn, sys, md.p,
                c->levenberg_marquadt);
        else
            k_add_diag<float><<<grid_for(c, c->nn, T), T, 0, c->stream>>>(c->bptr.p, c->bdiag.p, c->K32.p, nullptr,
                                                                          c->nn, sys, md.p, c->levenberg_marquadt);
        c->launches += 1;
    }
    if (exact) {
        apply_elimination(c, mat, vec);
    } else if (c->nc > 0) {
        const int g = grid_for(c, c->nc, T);
        if (c->have64) {
            k_penalty<double><<<g, T, 0, c->stream>>>(c->bptr.p, c->bdiag.p, c->K64.p, c->F.p, c->cdof.p,
                                                      c->ccoef.p, c->cres.p, c->nc, c->penalty, sys, md.p, mat, vec);
            if (mat && c->have32)
                k_round_constrained<<<g, T, 0, c->stream>>>(c->bptr.p, c->bdiag.p, c->K64.p, c->K32.p, c->cdof.p,
                                                            c->nc);
        } else {
            k_penalty<float><<<g, T, 0, c->stream>>>(c->bptr.p, c->bdiag.p, c->K32.p, c->F.p, c->cdof.p, c->ccoef.p,
                                                     c->cres.p, c->nc, c->penalty, sys, md.p, mat, vec);
        }
        c->launches += 1 + ((mat && c->have64 && c->have32) ? 1 : 0);
    }
    LMTG_CUDA(cudaGetLastError());
    std::vector<unsigned long long> bits(ns);
    LMTG_CUDA(cudaMemcpyAsync(bits.data(), md.p, ns * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                              c->stream));
    LMTG_CUDA(cudaStreamSynchronize(c->stream));
    std::vector<double> v(ns);
    double vmax = 0;
    for (uint32_t m = 0; m < ns; ++m) {
        memcpy(&v[m], &bits[m], sizeof(double));
        vmax = std::max(vmax, v[m]);
    }
    c->max_diag = vmax;
    if (c->nsys) c->h_sys_max_diag = v;
}

// ---- block-Jacobi preconditioner: inverse of every 3x3 diagonal block ----
template <class TK>
__global__ void k_block_jacobi(const uint32_t *__restrict__ bptr, const uint32_t *__restrict__ bdiag,
                               const TK *__restrict__ K, uint64_t nn, double *D64, float *D32) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < nn;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t rb = bptr[i], deg = bptr[i + 1] - rb, d = bdiag[i] - rb;
        double m[9];
        for (int k = 0; k < 9; ++k) m[k] = (double)K[kidx(rb, deg, d, k)];
        double c00 = m[4] * m[8] - m[5] * m[7], c01 = m[5] * m[6] - m[3] * m[8],
               c02 = m[3] * m[7] - m[4] * m[6];
        double det = m[0] * c00 + m[1] * c01 + m[2] * c02;
        double id = det != 0.0 ? 1.0 / det : 0.0;
        double r[9] = {c00 * id, (m[2] * m[7] - m[1] * m[8]) * id, (m[1] * m[5] - m[2] * m[4]) * id,
                       c01 * id, (m[0] * m[8] - m[2] * m[6]) * id, (m[2] * m[3] - m[0] * m[5]) * id,
                       c02 * id, (m[1] * m[6] - m[0] * m[7]) * id, (m[0] * m[4] - m[1] * m[3]) * id};
        for (int k = 0; k < 9; ++k) {
            if (D64) D64[i * 9 + k] = r[k];
            if (D32) D32[i * 9 + k] = (float)r[k];
        }
    }
}

void build_block_jacobi(lmtg_ctx *c, bool want64, bool want32) {
    const int T = 256;
    const int g = grid_for(c, c->nn, T);
    if (c->have64)
        k_block_jacobi<double><<<g, T, 0, c->stream>>>(c->bptr.p, c->bdiag.p, c->K64.p, c->nn,
                                                       want64 ? c->Dinv64.p : nullptr,
                                                       want32 ? c->Dinv32.p : nullptr);
    else
        k_block_jacobi<float><<<g, T, 0, c->stream>>>(c->bptr.p, c->bdiag.p, c->K32.p, c->nn, nullptr,
                                                      want32 ? c->Dinv32.p : nullptr);
    LMTG_CUDA(cudaGetLastError());
    c->launches += 1;
}

}  // namespace lmtg

namespace lmtg {

__global__ void k_round_all(const double *__restrict__ a, float *__restrict__ o, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x)
        o[i] = (float)a[i];
}

// FP32 inner operator rounded from the assembled FP64 matrix (used when the FP64 assembly ran
// without LMTG_ASM_MAT32 and a mixed solve is requested).
void copy_k64_to_k32(lmtg_ctx *c) {
    const uint64_t nv = c->nnzb * 9;
    k_round_all<<<grid_for(c, nv, 256), 256, 0, c->stream>>>(c->K64.p, c->K32.p, nv);
    LMTG_CUDA(cudaGetLastError());
    c->launches += 1;
    c->have32 = true;
    ++c->mat_version;
}

}  // namespace lmtg
