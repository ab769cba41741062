// noalloc.cu -- an allocation-free residual entry point for callers that cannot allocate.
//
// Some callers of this library cannot call cudaMalloc: a host application that hands every
// byte of device memory to its own arena at start-up and forbids allocation afterwards (an
// allocation there would synchronize the device, fragment the arena or fail once the arena
// holds the whole GPU), or a time-stepping loop that embeds the solver and must not touch the
// allocator between steps.  lmtg_residual_norm_noalloc gives such a caller r = b - K x and
// |r|_2^2 for a matrix it already holds on the device, without any allocation: the scratch of
// the cross-block reduction (one partial sum per thread block, a ticket counter and the result
// slot) lives in one file-scope __device__ array of fixed size.
//
// Limits and sharing: the array holds 65,536 block partials (512 KiB plus 256 bytes), so one
// call handles at most 65,536 * 8 = 524,288 node rows; larger problems are rejected.  Every GPU
// that loads the library holds this array until the process exits.  All calls share it and it
// keeps the last call's contents, so calls that overlap on the GPU (different streams, or
// different host threads) race and must be serialized by the caller.
#include "solver_kernels.cuh"

namespace {

constexpr uint64_t kNoAllocMaxBlocks = 65536;
constexpr uint64_t kNoAllocRowsPerBlock = lmtg::kRowThreads / 32;
constexpr uint64_t kNoAllocMaxRows = kNoAllocMaxBlocks * kNoAllocRowsPerBlock;
constexpr size_t kPartialsBytes = kNoAllocMaxBlocks * sizeof(double);
constexpr size_t kScratchBytes = kPartialsBytes + 256;  // + ticket (u32) and result (f64)

// Device code may name this array directly; host code must use the address obtained with
// cudaGetSymbolAddress (the host-side name is only a stand-in, not a device address).
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// One node row per warp, one block per 8 rows (no grid stride: one partial per block).
__global__ void __launch_bounds__(lmtg::kRowThreads)
    k_residual_noalloc(const uint32_t *__restrict__ bptr, const uint32_t *__restrict__ bcol,
                       const double *__restrict__ K, const double *__restrict__ x,
                       const double *__restrict__ b, double *__restrict__ r, uint64_t nn,
                       double *partials, unsigned *ticket, double *rr_out) {
    const int lane = threadIdx.x & 31;
    const uint64_t I = blockIdx.x * kNoAllocRowsPerBlock + (threadIdx.x >> 5);
    double v[1] = {0.0};
    if (I < nn) {
        double a0, a1, a2;
        lmtg::bsr3_row(bcol, K, bptr[I], bptr[I + 1], lane,
                       [&](uint64_t j) { return __ldg(x + j); }, a0, a1, a2);
        if (lane < 3) {
            const uint64_t i = 3 * I + lane;
            const double ri = b[i] - (lane == 0 ? a0 : (lane == 1 ? a1 : a2));
            r[i] = ri;
            v[0] = ri * ri;
        }
    }
    double out[1];
    if (lmtg::grid_reduce<1, 0u>(v, partials, ticket, out) && threadIdx.x == 0) *rr_out = out[0];
}

// The scratch array's address in the current device's context, looked up on every call (no
// allocation; cheap): a cached address would go stale after a device reset or a new primary
// context reloads the module.
int scratch_for_current_device(unsigned char **out) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return LMTG_ERR_CUDA;
    *out = static_cast<unsigned char *>(p);
    return LMTG_OK;
}

}  // namespace

extern "C" int lmtg_residual_norm_noalloc(void *stream, uint64_t nn, const uint32_t *bptr,
                                          const uint32_t *bcol, const double *K, const double *x,
                                          const double *b, double *r, double *rr_host) {
    if (nn == 0 || !bptr || !bcol || !K || !x || !b || !r) return LMTG_ERR_ARG;
    if (nn > kNoAllocMaxRows) return LMTG_ERR_ARG;  // scratch holds 65,536 block partials
    unsigned char *scratch = nullptr;
    int s = scratch_for_current_device(&scratch);
    if (s != LMTG_OK) return s;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    double *partials = reinterpret_cast<double *>(scratch);
    unsigned *ticket = reinterpret_cast<unsigned *>(scratch + kPartialsBytes);
    double *rr_dev = reinterpret_cast<double *>(scratch + kPartialsBytes + 8);
    // the ticket must start at zero; the partials and the result are overwritten every call
    if (cudaMemsetAsync(ticket, 0, sizeof(unsigned), st) != cudaSuccess) return LMTG_ERR_CUDA;
    const unsigned grid = (unsigned)((nn + kNoAllocRowsPerBlock - 1) / kNoAllocRowsPerBlock);
    k_residual_noalloc<<<grid, lmtg::kRowThreads, 0, st>>>(bptr, bcol, K, x, b, r, nn, partials,
                                                           ticket, rr_dev);
    if (cudaGetLastError() != cudaSuccess) return LMTG_ERR_CUDA;
    if (rr_host) {
        if (cudaMemcpyAsync(rr_host, rr_dev, sizeof(double), cudaMemcpyDeviceToHost, st) !=
            cudaSuccess)
            return LMTG_ERR_CUDA;
        if (cudaStreamSynchronize(st) != cudaSuccess) return LMTG_ERR_CUDA;
    }
    return LMTG_OK;
}
