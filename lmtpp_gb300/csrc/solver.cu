// solver.cu -- host drivers of the FP64 PCG and the FP32-inner / FP64-refined solve.
//
// Replaces Formulation::solve_system's iterative branch (include/formulation/formulation.h:
// 1487-1504): the reference's IC(0)-PCG / 3x3-block IC-PCG (include/containers/matinvsparse.h:
// 453-491, include/containers/MatWithTinyBlocks.h:1101-1150).  Iterations run as captured CUDA
// graphs of kChunk iterations; the host only reads the device scalars between chunks.
#include <chrono>
#include <cmath>
#include <type_traits>
#include <vector>

#include "amg.cuh"
#include "residual_dd.cuh"
#include "spmv_bulk.cuh"

namespace lmtg {

constexpr int kChunkPairs = 16;  // iterations per graph launch = 2 * kChunkPairs

// node stride of the gathered PCG vectors: padded 16-byte nodes in FP32, packed in FP64
template <class T> struct GatherStride { static constexpr int value = 3; };
template <> struct GatherStride<float> { static constexpr int value = 4; };

__global__ void k_scale_to32(const double *__restrict__ a, double s_inv, float *__restrict__ o,
                             uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x)
        o[i] = (float)(a[i] * s_inv);
}

__global__ void k_axpy_64_32(double *__restrict__ x, double s, const float *__restrict__ d,
                             uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x)
        x[i] += s * (double)d[i];
}

__global__ void k_dot64(const double *__restrict__ a, const double *__restrict__ b, uint64_t n,
                        double *partials, unsigned *ticket, double *out_p) {
    double v[1] = {0.0};
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x)
        v[0] += a[i] * b[i];
    double out[1];
    if (grid_reduce<1, 0u>(v, partials, ticket, out) && threadIdx.x == 0) *out_p = out[0];
}

static int row_grid(lmtg_ctx *c) { return grid_for(c, c->nn * 32, kRowThreads, 8); }
static int node_grid(lmtg_ctx *c) { return grid_for(c, c->nn, kRowThreads, 8); }

// Bulk-copy SpMV instances, spmv_kind 1, 2 = (stages, blocks per stage, consumer warps,
// evict-first L2 hint, CTAs per SM the registers are sized for).  Kind 1 held 96% of the
// measured HBM copy bandwidth on Hexa8 128^3 (0.361 ms against 0.449 ms for the warp-row
// kernel, kind 0).  The dynamic shared-memory limit and the resident grid are set up
// once per kind.
#define LMTG_BULK_KINDS(X)     \
    X(1, 2, 512, 8, true, 4)   \
    X(2, 2, 512, 8, true, 5)

template <int kStages, int kCap, int kCons, bool kEF, int kMinB>
static int bulk_grid(lmtg_ctx *c) {
    constexpr size_t smem = bulk_smem_bytes<kStages, kCap>();
    auto fn = k_pcg_spmv_bulk<kStages, kCap, kCons, kEF, kMinB, EpiPcg>;
    LMTG_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int nb = 0;
    LMTG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, bulk_threads<kCons>(), smem));
    return c->sm_count * (nb > 0 ? nb : 1);
}

// the kind in use: -1 picks the 5-CTA instance for wide rows (Tetra10: 0.108 against 0.111 ms
// at 40^3) and the 4-CTA one otherwise (Hexa8: 0.363 against 0.369 ms at 128^3); rows of more
// than 96 blocks (the recalage's virtual pattern) always take the warp-row kernel
static int spmv_kind_used(const lmtg_ctx *c) {
    if (c->max_row_blocks > 96) return 0;
    if (c->spmv_kind >= 0) return c->spmv_kind;
    if (c->spmv_tuned >= 0) return c->spmv_tuned;
    return c->max_row_blocks > 32 ? 2 : 1;
}

int spmv_kind_in_use(const lmtg_ctx *c) { return spmv_kind_used(c); }

static void spmv_setup(lmtg_ctx *c) {
    const int kind = spmv_kind_used(c);
    if (kind == c->spmv_setup_kind) return;
    switch (kind) {
#define LMTG_BULK_SETUP(id, st, cap, cons, ef, minb) \
    case id: c->spmv_grid = bulk_grid<st, cap, cons, ef, minb>(c); break;
        LMTG_BULK_KINDS(LMTG_BULK_SETUP)
#undef LMTG_BULK_SETUP
        default: c->spmv_grid = row_grid(c); break;
    }
    c->spmv_setup_kind = kind;
}

// q = K p, pq and alpha of one PCG iteration (FP64: the warp-row kernel; FP32: spmv_kind)
template <class T, int VS>
static void launch_pcg_spmv(lmtg_ctx *c, const T *K, const T *p, T *q, cudaStream_t s) {
    if constexpr (std::is_same<T, float>::value) {
        switch (spmv_kind_used(c)) {
#define LMTG_BULK_LAUNCH(id, st, cap, cons, ef, minb)                                                   \
    case id:                                                                                              \
        k_pcg_spmv_bulk<st, cap, cons, ef, minb, EpiPcg><<<c->spmv_grid, bulk_threads<cons>(),              \
                                                           bulk_smem_bytes<st, cap>(), s>>>(              \
            c->bptr.p, c->bcol.p, K, p, EpiPcg{q}, c->nn, c->scal.p, c->partials.p);                       \
        return;
            LMTG_BULK_KINDS(LMTG_BULK_LAUNCH)
#undef LMTG_BULK_LAUNCH
            default: break;
        }
    }
    k_pcg_spmv<T, VS><<<row_grid(c), kRowThreads, 0, s>>>(c->bptr.p, c->bcol.p, K, p, q, c->nn, c->scal.p,
                                                          c->partials.p);
}

void spmv64(lmtg_ctx *c, const double *x, double *y) {
    k_spmv<double><<<row_grid(c), kRowThreads, 0, c->stream>>>(c->bptr.p, c->bcol.p, c->K64.p, x, y,
                                                               c->nn);
    LMTG_CUDA(cudaGetLastError());
    c->launches += 1;
}
void spmv32(lmtg_ctx *c, const float *x, float *y) {
    k_spmv<float><<<row_grid(c), kRowThreads, 0, c->stream>>>(c->bptr.p, c->bcol.p, c->K32.p, x, y,
                                                              c->nn);
    LMTG_CUDA(cudaGetLastError());
    c->launches += 1;
}

// FP32 SpMV autotuner (spmv_kind -1): at the first FP32 PCG run of a pattern every kind the
// pattern admits -- 0 the warp-row kernel, 1 and 2 the bulk-copy pipeline with the resident grid
// sized for 4 or 5 CTAs per SM -- is timed with CUDA events over three launches on the assembled
// K32 (after one untimed launch), and the fastest is kept for the context's later solves.  Runs
// with the scalars of a fresh PCG run (done = 0); p and q are scratch at that point.
static void spmv_autotune(lmtg_ctx *c, const float *K, const float *p, float *q) {
    cudaStream_t s = c->stream;
    cudaEvent_t e0, e1;
    LMTG_CUDA(cudaEventCreate(&e0));
    LMTG_CUDA(cudaEventCreate(&e1));
    int best = -1;
    double best_ms = 0;
    for (int k = 0; k < 3; ++k) {
        c->spmv_tune_ms[k] = 0;
        if (k > 0 && c->max_row_blocks > 96) continue;
        c->spmv_tuned = k;
        spmv_setup(c);
        launch_pcg_spmv<float, 4>(c, K, p, q, s);
        LMTG_CUDA(cudaEventRecord(e0, s));
        for (int r = 0; r < 3; ++r) launch_pcg_spmv<float, 4>(c, K, p, q, s);
        LMTG_CUDA(cudaEventRecord(e1, s));
        LMTG_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        LMTG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        c->spmv_tune_ms[k] = ms / 3.0;
        c->launches += 4;
        if (best < 0 || ms / 3.0 < best_ms) {
            best = k;
            best_ms = ms / 3.0;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    c->spmv_tuned = best;
    spmv_setup(c);
}

// Second scalar slot (index 1) serves the outer loop and standalone reductions.
static PcgScalars *outer_slot(lmtg_ctx *c) { return c->scal.p + 1; }

static double read_double(lmtg_ctx *c, const double *dptr) {
    double v = 0;
    LMTG_CUDA(cudaMemcpyAsync(&c->h_scal[1].rr, dptr, sizeof(double), cudaMemcpyDeviceToHost,
                              c->stream));
    LMTG_CUDA(cudaStreamSynchronize(c->stream));
    v = c->h_scal[1].rr;
    return v;
}

template <class T>
static double residual(lmtg_ctx *c, const T *K, const T *x, const T *b, T *r) {
    PcgScalars *o = outer_slot(c);
    k_residual<T><<<row_grid(c), kRowThreads, 0, c->stream>>>(c->bptr.p, c->bcol.p, K, x, b, r, c->nn,
                                                              c->partials.p, &o->cnt_c, &o->rr);
    LMTG_CUDA(cudaGetLastError());
    c->launches += 1;
    return read_double(c, &o->rr);
}

__global__ void k_scale32(float *__restrict__ v, float s, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        v[i] *= s;
}

// the float-float residual kernel's shape: 3 stages of up to 256 blocks, 8 consumer warps, 3 CTAs
// per SM (59 KB of shared memory each)
constexpr int kResStages = 3, kResCap = 256, kResCons = 8, kResMinB = 3;

// Refinement residual of the mixed solver: b32 = r / |r| for r = F - K64 u, returns |r|^2.  With
// ff the float-float bulk-copy kernel (residual_dd.cuh) forms r to ~2^-48 relative accuracy off
// the FP64 pipe; otherwise, and for patterns with rows wider than its stage, the FP64 warp-row
// kernel into r64.
static double refinement_residual(lmtg_ctx *c, const double *u, const double *Fb, double bb, float *b32,
                                  double *r64, bool ff) {
    PcgScalars *o = outer_slot(c);
    cudaStream_t s = c->stream;
    if (!ff || c->max_row_blocks > (uint32_t)kResCap) {
        const double rr = residual<double>(c, c->K64.p, u, Fb, r64);
        if (rr > 0) {
            k_scale_to32<<<node_grid(c), kRowThreads, 0, s>>>(r64, 1.0 / std::sqrt(rr), b32, c->n);
            c->launches += 1;
        }
        return rr;
    }
    static int grid = 0;
    constexpr size_t smem = res64_smem_bytes<kResStages, kResCap>();
    auto fn = k_residual_ff<kResStages, kResCap, kResCons, kResMinB>;
    if (!grid) {
        LMTG_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        int nb = 0;
        LMTG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, 32 * (kResCons + 1), smem));
        grid = c->sm_count * (nb > 0 ? nb : 1);
    }
    // a power of two near 1 / rms(F) keeps the squares of small residuals in the float range
    const double rms = std::sqrt(bb / (double)(c->n ? c->n : 1));
    const int e = (rms > 0 && std::isfinite(rms)) ? std::max(-100, std::min(100, std::ilogb(rms))) : 0;
    const float rscale = std::ldexp(1.0f, -e);
    LMTG_CUDA(cudaMemsetAsync(&o->status, 0, sizeof(int), s));
    fn<<<grid, 32 * (kResCons + 1), smem, s>>>(c->bptr.p, c->bcol.p, c->K64.p, u, Fb, rscale, b32, c->nn,
                                                c->partials.p, o);
    LMTG_CUDA(cudaGetLastError());
    c->launches += 1;
    PcgScalars h;
    LMTG_CUDA(cudaMemcpyAsync(&h, o, sizeof(h), cudaMemcpyDeviceToHost, s));
    LMTG_CUDA(cudaStreamSynchronize(s));
    LMTG_CHECK(h.status != LMTG_ERR_TIMEOUT, LMTG_ERR_TIMEOUT, "residual: a bulk-copy wait gave up");
    if (h.rr > 0) {
        k_scale32<<<node_grid(c), kRowThreads, 0, s>>>(b32, (float)(1.0 / std::sqrt(h.rr)), c->n);
        c->launches += 1;
    }
    return h.rr * std::ldexp(1.0, 2 * e);
}

static double dot64(lmtg_ctx *c, const double *a, const double *b) {
    PcgScalars *o = outer_slot(c);
    k_dot64<<<node_grid(c), kRowThreads, 0, c->stream>>>(a, b, c->n, c->partials.p, &o->cnt_c,
                                                         &o->rr);
    LMTG_CUDA(cudaGetLastError());
    c->launches += 1;
    return read_double(c, &o->rr);
}

// Multigrid-preconditioned FP32 PCG: the start and update kernels leave z to the cycle
// (amg.cu), whose last kernel forms z, r.z and beta.  Both write the cycle's first smoothing
// step xa = omega D^-1 r (padded 4 per node).
__global__ void k_pcg_start_amg(const float *__restrict__ r, const float *__restrict__ b,
                                const float *__restrict__ Dinv, float *__restrict__ xa, float omega, uint64_t nn,
                                PcgScalars *S, double *partials) {
    float t[3] = {0.f, 0.f, 0.f};  // rr, bb, rinf
    for (uint64_t I = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; I < nn;
         I += (uint64_t)gridDim.x * blockDim.x) {
        const float *D = Dinv + 9 * I;
        const float r0 = r[3 * I], r1 = r[3 * I + 1], r2 = r[3 * I + 2];
        // whole 16-byte nodes (zero padding): no partially written sectors
        reinterpret_cast<float4 *>(xa)[I] = make_float4(omega * (D[0] * r0 + D[1] * r1 + D[2] * r2),
                                                        omega * (D[3] * r0 + D[4] * r1 + D[5] * r2),
                                                        omega * (D[6] * r0 + D[7] * r1 + D[8] * r2), 0.f);
        t[0] += r0 * r0 + r1 * r1 + r2 * r2;
        if (b) {
            const float b0 = b[3 * I], b1 = b[3 * I + 1], b2 = b[3 * I + 2];
            t[1] += b0 * b0 + b1 * b1 + b2 * b2;
        }
        t[2] = fmaxf(t[2], fmaxf(fabsf(r0), fmaxf(fabsf(r1), fabsf(r2))));
    }
    double out[3];
    if (grid_reduce_t<3, 4u>(t, partials, &S->cnt_c, out) && threadIdx.x == 0) {
        S->rr = out[0];
        if (b) S->bb = out[1];
        S->iter = 0;
        S->status = LMTG_OK;
        S->done = 0;
        if (S->crit_kind == LMTG_CRIT_REL_RESIDUAL && out[0] <= S->crit * S->crit * S->bb) S->done = 1;
        if (S->crit_kind == LMTG_CRIT_ABS_RESIDUAL_INF && out[2] <= S->crit) S->done = 1;
        if (!isfinite(out[0])) {
            S->done = 1;
            S->status = LMTG_ERR_NAN;
        }
    }
}

constexpr int kUpdNodes = 2;  // nodes a thread takes per step in k_pcg_update_amg (4: 128 registers, slower)

__global__ void k_pcg_update_amg(float *__restrict__ x, float *__restrict__ r, const float *__restrict__ p,
                                 const float *__restrict__ q, const float *__restrict__ Dinv, float *__restrict__ xa,
                                 float omega, uint64_t nn, PcgScalars *S, double *partials) {
    if (*(volatile int *)&S->done) return;
    const double pq = S->pq;
    const float alpha = (float)S->alpha;
    float t[4] = {0.f, 0.f, 0.f, 0.f};  // rr, dx2, dxinf, rinf
    // kUpdNodes nodes per step (I, I + stride, ...), every load issued before the arithmetic
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t I0 = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; I0 < nn; I0 += kUpdNodes * stride) {
        uint64_t Is[kUpdNodes];
        bool on[kUpdNodes];
#pragma unroll
        for (int u = 0; u < kUpdNodes; ++u) {
            Is[u] = I0 + u * stride;
            on[u] = Is[u] < nn;
        }
        float xv[kUpdNodes][3], rv0[kUpdNodes][3], qv[kUpdNodes][3], pv[kUpdNodes][3], D[kUpdNodes][9];
#pragma unroll
        for (int u = 0; u < kUpdNodes; ++u) {
            if (!on[u]) continue;
            const uint64_t I = Is[u];
            const float4 p4 = reinterpret_cast<const float4 *>(p)[I];
            pv[u][0] = p4.x;
            pv[u][1] = p4.y;
            pv[u][2] = p4.z;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                xv[u][c] = x[3 * I + c];
                rv0[u][c] = r[3 * I + c];
                qv[u][c] = q[3 * I + c];
            }
#pragma unroll
            for (int k = 0; k < 9; ++k) D[u][k] = Dinv[9 * I + k];
        }
#pragma unroll
        for (int u = 0; u < kUpdNodes; ++u) {
            if (!on[u]) continue;
            const uint64_t I = Is[u];
            float rv[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float dx = alpha * pv[u][c];
                x[3 * I + c] = xv[u][c] + dx;
                rv[c] = fmaf(-alpha, qv[u][c], rv0[u][c]);
                r[3 * I + c] = rv[c];
                t[1] = fmaf(dx, dx, t[1]);
                t[2] = fmaxf(t[2], fabsf(dx));
                t[3] = fmaxf(t[3], fabsf(rv[c]));
            }
            const float *Du = D[u];
            reinterpret_cast<float4 *>(xa)[I] =
                make_float4(omega * (Du[0] * rv[0] + Du[1] * rv[1] + Du[2] * rv[2]),
                            omega * (Du[3] * rv[0] + Du[4] * rv[1] + Du[5] * rv[2]),
                            omega * (Du[6] * rv[0] + Du[7] * rv[1] + Du[8] * rv[2]), 0.f);
            t[0] += rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2];
        }
    }
    double out[4];
    if (grid_reduce_t<4, (4u | 8u)>(t, partials, &S->cnt_b, out) && threadIdx.x == 0) {
        S->iter += 1;
        S->rr = out[0];
        S->dx_2sq = out[1];
        S->dx_inf = out[2];
        bool conv = false;
        switch (S->crit_kind) {
            case LMTG_CRIT_REL_RESIDUAL: conv = out[0] <= S->crit * S->crit * S->bb; break;
            case LMTG_CRIT_NORM_INF_DELTA: conv = out[2] <= S->crit; break;
            case LMTG_CRIT_NORM2_DELTA: conv = sqrt(out[1]) < S->crit; break;
            case LMTG_CRIT_ABS_RESIDUAL_INF: conv = out[3] <= S->crit; break;
        }
        if (!isfinite(out[0]) || !isfinite(pq)) {
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

// A captured chunk of PCG iterations, kept across the segments of one mixed solve (its kernel
// arguments -- buffers, scalars, smoother weights -- do not change between segments).
struct ChunkGraph {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    uint64_t launches = 0;  // kernels per chunk
    ChunkGraph() = default;
    ChunkGraph(const ChunkGraph &) = delete;
    ChunkGraph &operator=(const ChunkGraph &) = delete;
    ~ChunkGraph() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
    }
};

struct PcgBufs {
    void *x, *r, *z, *p0, *p1, *q;
};

// One PCG run on K x = b from the current x.  b_norm2 >= 0 gives |b|^2 for the relative test
// (otherwise b.b is computed).  Returns the status; *iters receives the iteration count.
// beta_den > 0 continues from the search direction held in p0 (reliable update); otherwise the
// run starts fresh (p = z).
template <class T>
static int run_pcg(lmtg_ctx *c, const T *K, const T *Dinv, const T *b, T *x, T *r, T *z, T *p0,
                   T *p1, T *q, bool x_is_zero, int crit_kind, double crit, int maxit,
                   double b_norm2, std::chrono::steady_clock::time_point deadline, bool use_deadline,
                   int *iters, double beta_den = 0.0, bool use_amg = false, ChunkGraph *keep = nullptr) {
    Phase ph(sizeof(T) == 4 ? "lmtg.pcg32" : "lmtg.pcg64");
    cudaStream_t s = c->stream;
    spmv_setup(c);
    PcgScalars init{};
    init.crit = crit;
    init.crit_kind = crit_kind;
    init.maxit = maxit;
    init.bb = b_norm2 >= 0 ? b_norm2 : 0.0;
    LMTG_CUDA(cudaMemcpyAsync(c->scal.p, &init, sizeof(init), cudaMemcpyHostToDevice, s));
    if constexpr (std::is_same<T, float>::value) {
        if (c->spmv_kind < 0 && c->spmv_tuned < 0 && beta_den <= 0.0) spmv_autotune(c, K, p0, q);
    }
    if (x_is_zero) {
        LMTG_CUDA(cudaMemcpyAsync(r, b, sizeof(T) * c->n, cudaMemcpyDeviceToDevice, s));
    } else {
        PcgScalars *o = outer_slot(c);
        k_residual<T><<<row_grid(c), kRowThreads, 0, s>>>(c->bptr.p, c->bcol.p, K, x, b, r, c->nn,
                                                          c->partials.p, &o->cnt_c, &o->rr);
        c->launches += 1;
    }
    constexpr int VS = GatherStride<T>::value;
    bool amg = false;
    if constexpr (std::is_same<T, float>::value) {
        amg = use_amg;
        if (amg) {
            k_pcg_start_amg<<<node_grid(c), kRowThreads, 0, s>>>(r, b_norm2 >= 0 ? nullptr : b, Dinv, amg_xa0(c),
                                                                 amg_omega0(c), c->nn, c->scal.p, c->partials.p);
            amg_launch_cycle(c, r, z, s, 1, beta_den);
        }
    }
    if (!amg)
        k_pcg_start<T, VS><<<node_grid(c), kRowThreads, 0, s>>>(r, b_norm2 >= 0 ? nullptr : b, Dinv, z,
                                                                 c->nn, c->scal.p, c->partials.p,
                                                                 beta_den);
    if (beta_den <= 0.0) {
        LMTG_CUDA(cudaMemsetAsync(p0, 0, sizeof(T) * VS * c->nn, s));
        LMTG_CUDA(cudaMemsetAsync(p1, 0, sizeof(T) * VS * c->nn, s));
    }
    LMTG_CUDA(cudaGetLastError());
    c->launches += 1;

    // capture one chunk of iterations (or reuse the caller's): 2 kChunkPairs iterations, 8 with
    // the multigrid cycle, whose segments take fewer iterations and more kernels each
    ChunkGraph local;
    ChunkGraph &cg = keep ? *keep : local;
    const int chunk_iters = amg ? 8 : 2 * kChunkPairs;
    if (!cg.exec) {
        LMTG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        const uint64_t launches0 = c->launches;
        for (int k = 0; k < chunk_iters; ++k) {
            k_pcg_dir<T, VS><<<node_grid(c), kRowThreads, 0, s>>>(z, p0, c->nn, c->scal.p);
            launch_pcg_spmv<T, VS>(c, K, p0, q, s);
            if constexpr (std::is_same<T, float>::value) {
                if (amg) {
                    k_pcg_update_amg<<<node_grid(c), kRowThreads, 0, s>>>(x, r, p0, q, Dinv, amg_xa0(c), amg_omega0(c),
                                                                          c->nn, c->scal.p, c->partials.p);
                    amg_launch_cycle(c, r, z, s, 0, 0.0);
                    continue;
                }
            }
            k_pcg_update<T, VS><<<node_grid(c), kRowThreads, 0, s>>>(x, r, z, p0, q, Dinv, c->nn,
                                                                     c->scal.p, c->partials.p);
        }
        // kernels of one chunk (the cycle's launches were counted while capturing)
        cg.launches = 3 * chunk_iters + (c->launches - launches0);
        c->launches = launches0;
        cudaError_t ce = cudaStreamEndCapture(s, &cg.graph);
        if (ce != cudaSuccess) throw Error{LMTG_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ce)};
        ce = cudaGraphInstantiate(&cg.exec, cg.graph, 0);
        if (ce != cudaSuccess) throw Error{LMTG_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ce)};
    }
    cudaGraphExec_t exec = cg.exec;
    int status = LMTG_OK;
    const int max_chunks = maxit / chunk_iters + 2;
    bool finished = false;
    // check the initial test before the first chunk
    LMTG_CUDA(cudaMemcpyAsync(c->h_scal, c->scal.p, sizeof(PcgScalars), cudaMemcpyDeviceToHost, s));
    LMTG_CUDA(cudaStreamSynchronize(s));
    if (c->h_scal[0].done) finished = true;
    for (int ch = 0; ch < max_chunks && !finished; ++ch) {
        cudaError_t ce = cudaGraphLaunch(exec, s);
        c->launches += cg.launches;
        if (ce == cudaSuccess)
            ce = cudaMemcpyAsync(c->h_scal, c->scal.p, sizeof(PcgScalars), cudaMemcpyDeviceToHost, s);
        if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
        if (ce != cudaSuccess) throw Error{LMTG_ERR_CUDA, std::string("pcg chunk: ") + cudaGetErrorString(ce)};
        if (c->h_scal[0].done) finished = true;
        else if (use_deadline && std::chrono::steady_clock::now() > deadline) {
            status = LMTG_ERR_TIMEOUT;
            break;
        }
    }
    *iters = c->h_scal[0].iter;
    if (status == LMTG_OK) status = finished ? c->h_scal[0].status : LMTG_ERR_NOT_CONVERGED;
    return status;
}

int solve_pcg64(lmtg_ctx *c, int crit_kind, double tol, int maxit, double timeout_s,
                lmtg_solve_stats *st, const double *bvec, double *xvec) {
    Phase ph("lmtg.solve_pcg64");
    const double *Fb = bvec ? bvec : c->F.p;
    double *ux = xvec ? xvec : c->u.p;
    auto deadline = std::chrono::steady_clock::now() +
                    std::chrono::duration_cast<std::chrono::steady_clock::duration>(
                        std::chrono::duration<double>(timeout_s > 0 ? timeout_s : 0));
    double *r = c->w64[0].p, *z = c->w64[1].p, *p0 = c->w64[2].p, *p1 = c->w64[3].p,
           *q = c->w64[4].p;
    int it = 0;
    int status = run_pcg<double>(c, c->K64.p, c->Dinv64.p, Fb, ux, r, z, p0, p1, q, false,
                                 crit_kind, tol, maxit, -1.0, deadline, timeout_s > 0, &it);
    double bb = dot64(c, Fb, Fb);
    double rr = residual<double>(c, c->K64.p, ux, Fb, r);
    st->iterations = it;
    st->outer_iterations = 0;
    st->rel_residual = bb > 0 ? std::sqrt(rr / bb) : std::sqrt(rr);
    return status;
}

// FP32-inner / FP64-refined solve with reliable updates (residual replacement).
// The FP32 PCG runs in segments on the scaled system K32 d = r / s.  A segment ends when its
// recursive residual has dropped by kDelta; then u += s d in FP64, the true residual
// r = F - K64 u is recomputed in FP64 and becomes the new FP32 residual (rescaled), and the
// search direction is kept (beta folded with the rescaling), so the Krylov recurrence is not
// restarted.  A segment that fails to reduce the true residual restarts from p = z (a classic
// iterative-refinement step).  Convergence is decided on the FP64 true residual only.
int solve_mixed(lmtg_ctx *c, double tol, int maxit, double timeout_s, lmtg_solve_stats *st,
                const double *bvec, double *xvec) {
    Phase ph("lmtg.solve_mixed");
    const double *Fb = bvec ? bvec : c->F.p;
    double *ux = xvec ? xvec : c->u.p;
    auto deadline = std::chrono::steady_clock::now() +
                    std::chrono::duration_cast<std::chrono::steady_clock::duration>(
                        std::chrono::duration<double>(timeout_s > 0 ? timeout_s : 0));
    double *r64 = c->w64[0].p;
    float *b32 = c->w32[0].p, *d32 = c->w32[1].p, *r32 = c->w32[2].p, *z32 = c->w32[3].p,
          *pa = c->w32[4].p, *pb = c->w32[5].p;
    float *q32 = reinterpret_cast<float *>(c->w64[1].p);  // FP64 buffer reused as FP32 q
    const double bb = dot64(c, Fb, Fb);
    const bool amg = amg_prepare(c);
    ChunkGraph chunk;  // captured at the first segment, replayed by the others
    const double kDelta = c->inner_reduction;  // recursive-residual reduction per segment
    int total = 0, outer = 0, status = LMTG_OK;
    double rel = 0, s_prev = 0, rz_prev = 0, rel_prev = 0;
    bool have_dir = false;
    const int max_outer = 400;
    // Float-float residuals (32x the FP64 rounding) while the residual is above kFFMinRel of |F|,
    // where their rounding stays four orders below it; below, and to decide convergence or when
    // a float-float residual shows no progress, the FP64 residual takes over for the rest of the
    // solve.  (Near the float-float floor the residual is mostly rounding, and a segment that
    // continues its search direction on it can diverge.)
    constexpr double kFFMinRel = 1e-9;
    bool ff = true;
    for (;;) {
        double rr = refinement_residual(c, ux, Fb, bb, b32, r64, ff);  // b32 = r / |r|
        rel = bb > 0 ? std::sqrt(rr / bb) : std::sqrt(rr);
        if (ff && (!std::isfinite(rel) || rel <= tol || rel < kFFMinRel || rr == 0.0 ||
                   (outer > 0 && rel > 0.5 * rel_prev))) {
            ff = false;
            rr = refinement_residual(c, ux, Fb, bb, b32, r64, false);
            rel = bb > 0 ? std::sqrt(rr / bb) : std::sqrt(rr);
        }
        if (!std::isfinite(rel)) {
            status = LMTG_ERR_NAN;
            break;
        }
        if (rel <= tol || rr == 0.0) break;
        if (total >= maxit || outer >= max_outer) {
            status = LMTG_ERR_NOT_CONVERGED;
            break;
        }
        if (timeout_s > 0 && std::chrono::steady_clock::now() > deadline) {
            status = LMTG_ERR_TIMEOUT;
            break;
        }
        // a segment that did not reduce the true residual by 2x restarts the direction
        if (have_dir && rel > 0.5 * rel_prev) have_dir = false;
        const double sc = std::sqrt(rr);
        LMTG_CUDA(cudaMemsetAsync(d32, 0, sizeof(float) * c->n, c->stream));
        const double f = have_dir ? s_prev / sc : 0.0;
        const double beta_den = have_dir ? rz_prev * f : 0.0;
        // stop the segment after a kDelta reduction, or at the final target if closer
        double eta = 0.5 * tol / rel;
        if (eta < kDelta) eta = kDelta;
        int it = 0;
        int s2 = run_pcg<float>(c, c->K32.p, c->Dinv32.p, b32, d32, r32, z32, pa, pb, q32, true,
                                LMTG_CRIT_REL_RESIDUAL, eta, maxit - total, 1.0, deadline,
                                timeout_s > 0, &it, beta_den, amg, &chunk);
        total += it;
        ++outer;
        if (s2 == LMTG_ERR_NAN || s2 == LMTG_ERR_TIMEOUT) {
            status = s2;
            break;
        }
        // the latest direction stays in pa for the next segment
        // the continued recurrence needs r.z from before the segment's last update:
        // beta_k = rz_{k+1} / rz_k, so rz_k = rz / beta of the final scalars
        // (with the multigrid cycle the last update skips the cycle, so rz is still rz_k)
        if (amg) rz_prev = c->h_scal[0].rz;
        else rz_prev = c->h_scal[0].beta != 0.0 ? c->h_scal[0].rz / c->h_scal[0].beta : 0.0;
        s_prev = sc;
        rel_prev = rel;
        have_dir = it > 0 && rz_prev > 0.0;
        k_axpy_64_32<<<node_grid(c), kRowThreads, 0, c->stream>>>(ux, sc, d32, c->n);
        LMTG_CUDA(cudaGetLastError());
        c->launches += 1;
    }
    st->iterations = total;
    st->outer_iterations = outer;
    st->rel_residual = rel;
    return status;
}

template <class T>
static void profile_pcg_t(lmtg_ctx *c, const T *K, const T *Dinv, const T *b, T *x, T *r, T *z,
                          T *p0, T *p1, T *q, int iters, double *spmv_ms, double *update_ms) {
    cudaStream_t s = c->stream;
    spmv_setup(c);
    PcgScalars init{};
    init.crit = 0.0;  // never met: every launch does the full work
    init.crit_kind = LMTG_CRIT_REL_RESIDUAL;
    init.maxit = 1 << 30;
    LMTG_CUDA(cudaMemcpyAsync(c->scal.p, &init, sizeof(init), cudaMemcpyHostToDevice, s));
    LMTG_CUDA(cudaMemsetAsync(x, 0, sizeof(T) * c->n, s));
    LMTG_CUDA(cudaMemcpyAsync(r, b, sizeof(T) * c->n, cudaMemcpyDeviceToDevice, s));
    constexpr int VS = GatherStride<T>::value;
    k_pcg_start<T, VS><<<node_grid(c), kRowThreads, 0, s>>>(r, b, Dinv, z, c->nn, c->scal.p,
                                                             c->partials.p, 0.0);
    LMTG_CUDA(cudaMemsetAsync(p0, 0, sizeof(T) * VS * c->nn, s));
    LMTG_CUDA(cudaMemsetAsync(p1, 0, sizeof(T) * VS * c->nn, s));
    c->launches += 1;
    std::vector<cudaEvent_t> ev(2 * iters + 1);
    for (auto &e : ev) LMTG_CUDA(cudaEventCreate(&e));
    LMTG_CUDA(cudaEventRecord(ev[0], s));
    for (int k = 0; k < iters; ++k) {
        launch_pcg_spmv<T, VS>(c, K, p0, q, s);
        LMTG_CUDA(cudaEventRecord(ev[2 * k + 1], s));
        // the rest of the iteration: update, then the next direction
        k_pcg_update<T, VS><<<node_grid(c), kRowThreads, 0, s>>>(x, r, z, p0, q, Dinv, c->nn, c->scal.p,
                                                             c->partials.p);
        k_pcg_dir<T, VS><<<node_grid(c), kRowThreads, 0, s>>>(z, p0, c->nn, c->scal.p);
        LMTG_CUDA(cudaEventRecord(ev[2 * k + 2], s));
    }
    c->launches += 3ull * iters;
    LMTG_CUDA(cudaGetLastError());
    LMTG_CUDA(cudaEventSynchronize(ev[2 * iters]));
    double a = 0, bsum = 0;
    for (int k = 0; k < iters; ++k) {
        float m1 = 0, m2 = 0;
        cudaEventElapsedTime(&m1, ev[2 * k], ev[2 * k + 1]);
        cudaEventElapsedTime(&m2, ev[2 * k + 1], ev[2 * k + 2]);
        a += m1;
        bsum += m2;
    }
    for (auto &e : ev) cudaEventDestroy(e);
    *spmv_ms = a / iters;
    *update_ms = bsum / iters;
}

void profile_pcg(lmtg_ctx *c, bool fp32, int iters, double *spmv_ms, double *update_ms) {
    if (!fp32) {
        profile_pcg_t<double>(c, c->K64.p, c->Dinv64.p, c->F.p, c->w64[5].p, c->w64[0].p, c->w64[1].p,
                              c->w64[2].p, c->w64[3].p, c->w64[4].p, iters, spmv_ms, update_ms);
    } else {
        const double bb = dot64(c, c->F.p, c->F.p);
        float *b32 = c->w32[0].p;
        k_scale_to32<<<node_grid(c), kRowThreads, 0, c->stream>>>(c->F.p, bb > 0 ? 1.0 / std::sqrt(bb) : 1.0,
                                                                  b32, c->n);
        c->launches += 1;
        profile_pcg_t<float>(c, c->K32.p, c->Dinv32.p, b32, c->w32[1].p, c->w32[2].p, c->w32[3].p,
                             c->w32[4].p, c->w32[5].p, reinterpret_cast<float *>(c->w64[1].p), iters,
                             spmv_ms, update_ms);
    }
}

// Device time per stage of the multigrid-preconditioned FP32 iteration, averaged over `iters`
// iterations run on the scaled load vector with a criterion that never stops them: ms[0] the
// PCG's SpMV, [1] the update (with the first smoothing step), [2] the level-0 residual, [3] the
// restriction, [4] the coarse levels, [5] the prolongation, [6] the level-0 smoothing (z, r.z),
// [7] the direction update.  All zero when the context has no hierarchy.
void profile_amg(lmtg_ctx *c, int iters, double *ms) {
    Phase ph("lmtg.amg.profile");
    for (int k = 0; k < 8; ++k) ms[k] = 0;
    if (!amg_prepare(c)) return;
    cudaStream_t s = c->stream;
    spmv_setup(c);
    float *b32 = c->w32[0].p, *x = c->w32[1].p, *r = c->w32[2].p, *z = c->w32[3].p, *p0 = c->w32[4].p;
    float *q = reinterpret_cast<float *>(c->w64[1].p);
    const double bb = dot64(c, c->F.p, c->F.p);
    k_scale_to32<<<node_grid(c), kRowThreads, 0, s>>>(c->F.p, bb > 0 ? 1.0 / std::sqrt(bb) : 1.0, b32, c->n);
    PcgScalars init{};
    init.crit = 0.0;
    init.crit_kind = LMTG_CRIT_REL_RESIDUAL;
    init.maxit = 1 << 30;
    init.bb = 1.0;
    LMTG_CUDA(cudaMemcpyAsync(c->scal.p, &init, sizeof(init), cudaMemcpyHostToDevice, s));
    LMTG_CUDA(cudaMemsetAsync(x, 0, sizeof(float) * c->n, s));
    LMTG_CUDA(cudaMemcpyAsync(r, b32, sizeof(float) * c->n, cudaMemcpyDeviceToDevice, s));
    LMTG_CUDA(cudaMemsetAsync(p0, 0, sizeof(float) * 4 * c->nn, s));
    k_pcg_start_amg<<<node_grid(c), kRowThreads, 0, s>>>(r, nullptr, c->Dinv32.p, amg_xa0(c), amg_omega0(c), c->nn,
                                                         c->scal.p, c->partials.p);
    amg_launch_cycle(c, r, z, s, 1, 0.0);
    c->launches += 2;
    std::vector<cudaEvent_t> ev(9 * iters);
    for (auto &e : ev) LMTG_CUDA(cudaEventCreate(&e));
    const uint64_t l0 = c->launches;
    for (int it = 0; it < iters; ++it) {
        cudaEvent_t *e = &ev[9 * it];
        LMTG_CUDA(cudaEventRecord(e[0], s));
        k_pcg_dir<float, 4><<<node_grid(c), kRowThreads, 0, s>>>(z, p0, c->nn, c->scal.p);
        LMTG_CUDA(cudaEventRecord(e[1], s));
        launch_pcg_spmv<float, 4>(c, c->K32.p, p0, q, s);
        LMTG_CUDA(cudaEventRecord(e[2], s));
        k_pcg_update_amg<<<node_grid(c), kRowThreads, 0, s>>>(x, r, p0, q, c->Dinv32.p, amg_xa0(c), amg_omega0(c),
                                                              c->nn, c->scal.p, c->partials.p);
        LMTG_CUDA(cudaEventRecord(e[3], s));
        amg_launch_cycle(c, r, z, s, 0, 0.0, e + 4);
    }
    c->launches += 3ull * iters;
    (void)l0;
    LMTG_CUDA(cudaGetLastError());
    LMTG_CUDA(cudaEventSynchronize(ev[9 * iters - 1]));
    static const int from[8] = {1, 2, 3, 4, 5, 6, 7, 0}, to[8] = {2, 3, 4, 5, 6, 7, 8, 1};
    for (int it = 0; it < iters; ++it)
        for (int k = 0; k < 8; ++k) {
            float m = 0;
            cudaEventElapsedTime(&m, ev[9 * it + from[k]], ev[9 * it + to[k]]);
            ms[k] += m / iters;
        }
    for (auto &e : ev) cudaEventDestroy(e);
}

}  // namespace lmtg
