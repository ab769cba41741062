// pattern.cu -- sparsity pattern and element-to-block gather lists, built on the GPU.
//
// Replaces Formulation::allocate_matrices / ResizeMat (include/formulation/formulation.h:200-241,
// 338-412), which walks every element to collect the node-pair pattern, and the per-entry
// binary-search insertion of the generated scatter (formal_lf/calculate_matrix.py:86-98,
// include/containers/vecsparse.h:126-144).  Here the pattern is built once per mesh:
//   1. node -> (element, local node) incidence, sorted by element (deterministic order);
//   2. node -> sorted unique neighbour nodes (the full symmetric node-block pattern);
//   3. for every 3x3 block, the list of element blocks that sum into it, in element order.
// After that, assembly is a pure gather with no atomics and no search.
#include "lmtg_internal.cuh"

namespace lmtg {

// ------------------------------------------------------------------------------------------
// exclusive scan (u32 in, u32 out, u64 running sums; the caller checks the 32-bit total)
// ------------------------------------------------------------------------------------------
constexpr int kScanThreads = 512, kScanItems = 8, kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ unsigned long long block_exclusive_scan(unsigned long long v,
                                                                   unsigned long long *sh,
                                                                   unsigned long long *total) {
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    unsigned long long x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sh[wid] = x;
    __syncthreads();
    if (wid == 0) {
        unsigned long long s = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0ull;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            unsigned long long y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        sh[lane] = s;  // inclusive warp prefix
    }
    __syncthreads();
    unsigned long long warp_off = wid ? sh[wid - 1] : 0ull;
    *total = sh[(blockDim.x >> 5) - 1];
    __syncthreads();
    return warp_off + x - v;
}

__global__ void k_scan_tile_sums(const uint32_t *in, uint64_t count, unsigned long long *tile) {
    __shared__ unsigned long long sh[32];
    uint64_t base = (uint64_t)blockIdx.x * kScanTile;
    unsigned long long s = 0;
    for (int k = 0; k < kScanItems; ++k) {
        uint64_t i = base + (uint64_t)threadIdx.x * kScanItems + k;
        if (i < count) s += in[i];
    }
    unsigned long long tot;
    block_exclusive_scan(s, sh, &tot);
    if (threadIdx.x == 0) tile[blockIdx.x] = tot;
}

__global__ void k_scan_tiles(unsigned long long *tile, uint64_t ntiles, unsigned long long *total) {
    __shared__ unsigned long long sh[32];
    unsigned long long carry = 0;
    for (uint64_t b = 0; b < ntiles; b += blockDim.x) {
        uint64_t i = b + threadIdx.x;
        unsigned long long v = i < ntiles ? tile[i] : 0ull, tot;
        unsigned long long ex = block_exclusive_scan(v, sh, &tot);
        if (i < ntiles) tile[i] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0) *total = carry;
}

__global__ void k_scan_apply(const uint32_t *in, uint32_t *out, uint64_t count,
                             const unsigned long long *tile, const unsigned long long *total) {
    __shared__ unsigned long long sh[32];
    uint64_t base = (uint64_t)blockIdx.x * kScanTile + (uint64_t)threadIdx.x * kScanItems;
    unsigned long long loc[kScanItems], s = 0;
    for (int k = 0; k < kScanItems; ++k) {
        uint64_t i = base + k;
        loc[k] = i < count ? in[i] : 0u;
        s += loc[k];
    }
    unsigned long long tot;
    unsigned long long off = block_exclusive_scan(s, sh, &tot) + tile[blockIdx.x];
    for (int k = 0; k < kScanItems; ++k) {
        uint64_t i = base + k;
        if (i < count) out[i] = (uint32_t)off;
        off += loc[k];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) out[count] = (uint32_t)*total;
}

uint64_t exclusive_scan_u32(lmtg_ctx *c, const uint32_t *in, uint32_t *out, uint64_t count) {
    uint64_t ntiles = (count + kScanTile - 1) / kScanTile;
    if (ntiles == 0) ntiles = 1;
    DBuf<unsigned long long> tile;
    tile.alloc(ntiles + 1);
    k_scan_tile_sums<<<(unsigned)ntiles, kScanThreads, 0, c->stream>>>(in, count, tile.p);
    k_scan_tiles<<<1, 1024, 0, c->stream>>>(tile.p, ntiles, tile.p + ntiles);
    k_scan_apply<<<(unsigned)ntiles, kScanThreads, 0, c->stream>>>(in, out, count, tile.p,
                                                                   tile.p + ntiles);
    LMTG_CUDA(cudaGetLastError());
    unsigned long long total = 0;
    LMTG_CUDA(cudaMemcpyAsync(&total, tile.p + ntiles, sizeof(total), cudaMemcpyDeviceToHost,
                              c->stream));
    LMTG_CUDA(cudaStreamSynchronize(c->stream));
    LMTG_CHECK(total < (1ull << 32), LMTG_ERR_UNSUPPORTED, "pattern larger than 2^32 entries");
    return total;
}

// ------------------------------------------------------------------------------------------
// 1. incidence
// ------------------------------------------------------------------------------------------
__global__ void k_inc_count(const uint32_t *conn, uint64_t m, uint64_t nn, uint32_t *cnt,
                            int *bad) {
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < m;
         t += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t n = conn[t];
        if (n >= nn) {
            atomicExch(bad, 1);
            continue;
        }
        atomicAdd(&cnt[n], 1u);
    }
}

__global__ void k_inc_fill(const uint32_t *conn, uint64_t m, uint32_t *cursor, uint32_t *inc) {
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < m;
         t += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t p = atomicAdd(&cursor[conn[t]], 1u);
        inc[p] = (uint32_t)t;
    }
}

__global__ void k_inc_sort(const uint32_t *incptr, uint32_t *inc, uint64_t nn) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < nn;
         i += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t b = incptr[i], e = incptr[i + 1];
        for (uint32_t k = b + 1; k < e; ++k) {
            uint32_t v = inc[k], j = k;
            while (j > b && inc[j - 1] > v) {
                inc[j] = inc[j - 1];
                --j;
            }
            inc[j] = v;
        }
    }
}

// ------------------------------------------------------------------------------------------
// 2. neighbours (sorted unique node list per node, self included)
// ------------------------------------------------------------------------------------------
constexpr int kMaxNbr = 96;

template <bool kFill>
__global__ void k_nbr(const uint32_t *conn, int npe, const uint32_t *incptr, const uint32_t *inc,
                      uint64_t nn, uint32_t *deg, const uint32_t *bptr, uint32_t *bcol,
                      uint32_t *bdiag, int *bad) {
    uint32_t loc[kMaxNbr];
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < nn;
         i += (uint64_t)gridDim.x * blockDim.x) {
        int m = 0;
        bool over = false;
        for (uint32_t k = incptr[i]; k < incptr[i + 1]; ++k) {
            uint64_t e = inc[k] / npe;
            for (int b = 0; b < npe; ++b) {
                uint32_t j = conn[e * npe + b];
                int p = 0;
                while (p < m && loc[p] < j) ++p;
                if (p < m && loc[p] == j) continue;
                if (m == kMaxNbr) {
                    over = true;
                    continue;
                }
                for (int q = m; q > p; --q) loc[q] = loc[q - 1];
                loc[p] = j;
                ++m;
            }
        }
        if (m == 0) loc[m++] = (uint32_t)i;  // isolated node: diagonal block only
        if (over) atomicExch(bad, 2);
        if (!kFill) {
            deg[i] = (uint32_t)m;
            atomicMax(bad + 1, m);  // widest row
        } else {
            uint32_t o = bptr[i];
            for (int k = 0; k < m; ++k) {
                bcol[o + k] = loc[k];
                if (loc[k] == (uint32_t)i) bdiag[i] = o + k;
            }
        }
    }
}

// ------------------------------------------------------------------------------------------
// 3. gather lists: element blocks summing into each matrix block, in element order.
// gsrc = ((e * npairs + pair(min(a,b), max(a,b))) << 1) | (a > b)   (1 = read transposed)
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ int find_in_row(const uint32_t *bcol, uint32_t b, uint32_t e,
                                           uint32_t j) {
    uint32_t lo = b, hi = e;
    while (lo < hi) {
        uint32_t mid = (lo + hi) >> 1;
        if (bcol[mid] < j) lo = mid + 1;
        else hi = mid;
    }
    return (int)(lo - b);
}

template <bool kFill>
__global__ void k_gather(const uint32_t *conn, int npe, int npairs, const uint32_t *incptr,
                         const uint32_t *inc, uint64_t nn, const uint32_t *bptr,
                         const uint32_t *bcol, uint32_t *gcnt, const uint32_t *gptr,
                         uint32_t *gsrc) {
    uint32_t cur[kMaxNbr];
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < nn;
         i += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t rb = bptr[i], re = bptr[i + 1];
        int deg = (int)(re - rb);
        for (int k = 0; k < deg; ++k) cur[k] = kFill ? gptr[rb + k] : 0u;
        for (uint32_t k = incptr[i]; k < incptr[i + 1]; ++k) {
            uint32_t t = inc[k];
            uint64_t e = t / npe;
            int a = (int)(t % npe);
            for (int b = 0; b < npe; ++b) {
                uint32_t j = conn[e * npe + b];
                int slot = find_in_row(bcol, rb, re, j);
                if (slot >= deg || bcol[rb + slot] != j) continue;  // cannot happen for a
                                                                     // consistent pattern
                if (kFill) {
                    int lo = a < b ? a : b, hi = a < b ? b : a;
                    gsrc[cur[slot]++] =
                        (uint32_t)(((e * npairs + pair_index(lo, hi, npe)) << 1) | (a > b ? 1u : 0u));
                } else {
                    cur[slot]++;
                }
            }
        }
        if (!kFill)
            for (int k = 0; k < deg; ++k) gcnt[rb + k] = cur[k];
    }
}

void build_pattern(lmtg_ctx *c) {
    Phase ph("lmtg.pattern");
    const uint64_t nn = c->nn, ne = c->ne, m = ne * (uint64_t)c->npe;
    LMTG_CHECK(m < (1ull << 32), LMTG_ERR_UNSUPPORTED, "ne * nodes_per_element must be < 2^32");
    LMTG_CHECK((uint64_t)ne * c->npairs * 2 < (1ull << 32), LMTG_ERR_UNSUPPORTED,
               "too many element blocks for 32-bit gather indices");
    cudaStream_t s = c->stream;
    const int T = 256;
    DBuf<int> bad;
    bad.alloc(2);  // [0] error code, [1] blocks in the widest row
    LMTG_CUDA(cudaMemsetAsync(bad.p, 0, 2 * sizeof(int), s));

    DBuf<uint32_t> cnt, incptr, cursor, inc;
    cnt.alloc(nn + 1);
    incptr.alloc(nn + 1);
    inc.alloc(m ? m : 1);
    LMTG_CUDA(cudaMemsetAsync(cnt.p, 0, cnt.bytes(), s));
    k_inc_count<<<grid_for(c, m, T), T, 0, s>>>(c->conn.p, m, nn, cnt.p, bad.p);
    exclusive_scan_u32(c, cnt.p, incptr.p, nn);
    int hbad = 0;
    LMTG_CUDA(cudaMemcpy(&hbad, bad.p, sizeof(int), cudaMemcpyDeviceToHost));
    LMTG_CHECK(hbad == 0, LMTG_ERR_ARG, "connectivity references a node id >= nn");
    cursor.alloc(nn + 1);
    LMTG_CUDA(cudaMemcpyAsync(cursor.p, incptr.p, cursor.bytes(), cudaMemcpyDeviceToDevice, s));
    k_inc_fill<<<grid_for(c, m, T), T, 0, s>>>(c->conn.p, m, cursor.p, inc.p);
    k_inc_sort<<<grid_for(c, nn, T), T, 0, s>>>(incptr.p, inc.p, nn);
    cursor.release();

    // neighbours
    DBuf<uint32_t> deg;
    deg.alloc(nn + 1);
    k_nbr<false><<<grid_for(c, nn, 128), 128, 0, s>>>(c->conn.p, c->npe, incptr.p, inc.p, nn,
                                                       deg.p, nullptr, nullptr, nullptr, bad.p);
    c->bptr.alloc(nn + 1 + 4);  // 16 bytes of slack: bulk copies round their end up
    c->nnzb = exclusive_scan_u32(c, deg.p, c->bptr.p, nn);
    int hb2[2] = {0, 0};
    LMTG_CUDA(cudaMemcpy(hb2, bad.p, 2 * sizeof(int), cudaMemcpyDeviceToHost));
    LMTG_CHECK(hb2[0] == 0, LMTG_ERR_UNSUPPORTED, "a node has more than 96 neighbour nodes");
    c->max_row_blocks = (uint32_t)hb2[1];
    deg.release();
    c->bcol.alloc(c->nnzb + 4);  // 16 bytes of slack: bulk copies round their end up
    c->bdiag.alloc(nn);
    k_nbr<true><<<grid_for(c, nn, 128), 128, 0, s>>>(c->conn.p, c->npe, incptr.p, inc.p, nn,
                                                      nullptr, c->bptr.p, c->bcol.p, c->bdiag.p,
                                                      bad.p);
    LMTG_CUDA(cudaGetLastError());

    // gather lists
    DBuf<uint32_t> gcnt;
    gcnt.alloc(c->nnzb + 1);
    k_gather<false><<<grid_for(c, nn, 128), 128, 0, s>>>(c->conn.p, c->npe, c->npairs, incptr.p,
                                                          inc.p, nn, c->bptr.p, c->bcol.p, gcnt.p,
                                                          nullptr, nullptr);
    c->gptr.alloc(c->nnzb + 1);
    c->ngather = exclusive_scan_u32(c, gcnt.p, c->gptr.p, c->nnzb);
    LMTG_CHECK(c->ngather == m * (uint64_t)c->npe, LMTG_ERR_CUDA, "gather list size mismatch");
    gcnt.release();
    c->gsrc.alloc(c->ngather);
    k_gather<true><<<grid_for(c, nn, 128), 128, 0, s>>>(c->conn.p, c->npe, c->npairs, incptr.p,
                                                         inc.p, nn, c->bptr.p, c->bcol.p, nullptr,
                                                         c->gptr.p, c->gsrc.p);
    LMTG_CUDA(cudaGetLastError());
    LMTG_CUDA(cudaStreamSynchronize(s));
    // scalar entries of the lower triangle: off-diagonal blocks count once (9), diagonal 6
    c->nnz_lower = 9ull * (c->nnzb - nn) / 2 + 6ull * nn;
    c->launches += 1 + 3 * 3 + 2 + 2 + 2;
}

}  // namespace lmtg
