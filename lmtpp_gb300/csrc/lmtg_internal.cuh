// lmtg_internal.cuh -- shared declarations of the GB300 finite-element hot path library.
//
// Layout in HBM (one context = one mesh/formulation on one GPU):
//   pos[nn*3] f64, conn[ne*npe] u32, E[ne or 1] f64               mesh and material
//   bptr[nn+1] u32, bcol[nnzb] u32, bdiag[nn] u32                  node-block pattern (full
//                                                                  symmetric, sorted columns)
//   gptr[nnzb+1] u32, gsrc[ne*npe*npe] u32                         gather lists: for every 3x3
//                                                                  block the element blocks that
//                                                                  sum into it, element order
//   Ke64/Ke32[ne*npairs*9]                                         element matrices, upper node
//                                                                  pairs (a<=b), 3x3 row-major
//   K64/K32[nnzb*9]                                                assembled matrix, 3x3 node
//                                                                  blocks, planar per row (kidx)
//   F, u [n] f64                                                   load vector, solution
//   Dinv64/Dinv32[nn*9]                                            block-Jacobi inverses
#pragma once
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <stdint.h>
#include <string>
#include <vector>

#include "../../include/lmtg.h"

namespace lmtg {

// NVTX range over a host phase (assembly, a PCG run, a time step...), visible in a timeline
// profiler; without one attached the calls return at once.
struct Phase {
    explicit Phase(const char *name) { nvtxRangePushA(name); }
    ~Phase() { nvtxRangePop(); }
    Phase(const Phase &) = delete;
    Phase &operator=(const Phase &) = delete;
};

constexpr int kWarp = 32;

// Thrown inside the library only; every C entry point catches and maps to a status code.
struct Error {
    int status;
    std::string msg;
};

#define LMTG_CUDA(call)                                                                          \
    do {                                                                                         \
        cudaError_t _e = (call);                                                                 \
        if (_e != cudaSuccess)                                                                   \
            throw ::lmtg::Error{_e == cudaErrorMemoryAllocation ? LMTG_ERR_NOMEM : LMTG_ERR_CUDA, \
                                std::string(#call) + ": " + cudaGetErrorString(_e)};             \
    } while (0)

#define LMTG_CHECK(cond, status, msg)                                                            \
    do {                                                                                         \
        if (!(cond)) throw ::lmtg::Error{status, msg};                                           \
    } while (0)

// Typed device buffer owned by a context.
template <class T>
struct DBuf {
    T *p = nullptr;
    size_t n = 0;
    DBuf() = default;
    DBuf(const DBuf &) = delete;
    DBuf &operator=(const DBuf &) = delete;
    ~DBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    void alloc(size_t count) {
        if (count == n && p) return;
        release();
        if (count == 0) return;
        LMTG_CUDA(cudaMalloc(&p, count * sizeof(T)));
        n = count;
    }
    size_t bytes() const { return n * sizeof(T); }
};

// Scalars of one PCG run, resident on the device so that iterations need no host round trip.
struct PcgScalars {
    double rz;       // r . z
    double pq;       // p . q
    double rr;       // r . r
    double bb;       // b . b (of the system being solved)
    double dx_inf;   // |alpha p|_inf of the last update
    double dx_2sq;   // |alpha p|_2^2 of the last update
    double beta;     // current beta (0 on the first iteration)
    double alpha;    // rz / pq of the current iteration (set with pq)
    double crit;     // threshold of the stopping test
    int crit_kind;   // LMTG_CRIT_*
    int iter;        // iterations done
    int maxit;
    int done;        // 1 = converged or stopped
    int status;      // LMTG_OK / NOT_CONVERGED / NAN
    unsigned cnt_a;  // grid-reduction tickets
    unsigned cnt_b;
    unsigned cnt_c;
    unsigned cnt_d;
};

}  // namespace lmtg

namespace lmtg {
struct BatchState;  // batch.cu
struct RecalState;  // recalage.cu
struct AmgState;    // amg.cu
struct SAmg;        // diffusion.cu
}

namespace lmtg {
// A captured chunk of the diffusion PCG, replayed by later solves while its arguments (the
// buffers it was captured on) are the same.
struct DiffGraph {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    const void *key[10] = {};
    uint64_t launches = 0;  // kernels per replay
};
}  // namespace lmtg

struct lmtg_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t aux_stream = nullptr;  // work that overlaps the main stream (created on first use)
    std::string err;
    int sm_count = 0;

    // mesh and material
    int elem_type = 0, npe = 0, nnu = 3, npairs = 0;
    uint64_t nn = 0, ne = 0, n = 0;
    lmtg::DBuf<double> pos;
    lmtg::DBuf<uint32_t> conn;
    lmtg::DBuf<double> E;
    int E_per_elem = 0;
    double nu = 0.3;
    lmtg::DBuf<double> nuv;  // per-element Poisson ratios (nu_per_elem)
    int nu_per_elem = 0;

    // batch of independent systems: node ranges [sys_node_off[m], sys_node_off[m+1]) that no
    // element couples; the penalty scale max|diag| is taken per system
    uint32_t nsys = 0;
    std::vector<uint64_t> h_sys_node_off;
    lmtg::DBuf<uint32_t> sys_of_node;
    std::vector<double> h_sys_max_diag;
    lmtg::BatchState *batch = nullptr;
    int batch_tile_rows = 0;             // 0: autotuned
    int batch_variant = -1;              // -1: autotuned
    std::vector<double> h_pos;      // host copy of positions (skin loads)
    std::vector<uint32_t> h_conn;   // host copy of connectivity

    // pattern
    bool allocated = false;
    uint64_t nnzb = 0, nnz_lower = 0, ngather = 0;
    uint32_t max_row_blocks = 0;  // blocks in the widest node row (<= 96; <= 288 on the recalage's
                                  // virtual pattern, whose FP32 SpMV is then the warp-row kernel)
    // FP32 PCG SpMV: 0 = warp per row pair, 1, 2 = bulk-copy pipeline (solver.cu) with 4 / 5 CTAs
    // per SM, -1 (default) = autotuned; the grid is set up when the kind in use changes
    int spmv_kind = -1, spmv_setup_kind = -2, spmv_grid = 0;
    // autotuned kind for spmv_kind -1 (timed at the first FP32 PCG run of a pattern; -1 = not yet)
    int spmv_tuned = -1;
    double spmv_tune_ms[3] = {0, 0, 0};
    lmtg::DBuf<uint32_t> bptr, bcol, bdiag, gptr, gsrc;

    // values
    lmtg::DBuf<double> Ke64, K64, F, u, Dinv64;
    lmtg::DBuf<double> adj_rhs, adj_lam, grad;  // adjoint workspace

    // heat diffusion (Triangle_6, one unknown per node): K64 holds A = M/dt + theta K,
    // B64 holds B = M/dt - (1 - theta) K, K32 the FP32 copy of A; Ke64 / KeB64 the element blocks
    lmtg::DBuf<double> B64, KeB64;
    double rho_c = 1.0, dt = 0.0, theta = 0.5;
    int diff_mode = LMTG_SOLVE_PCG_F64;
    std::vector<double> h_diff_src, h_diff_conv;  // constant step loads (sources, convection)
    lmtg::DBuf<double> diff_load;                  // their sum on the device (none: empty)
    // mixed solvers: recursive-residual reduction of each FP32 segment before the FP64 residual
    // replacement (lmtg_set_inner_reduction)
    double inner_reduction = 0.01;
    lmtg::DiffGraph diff_graph[2];  // the diffusion PCG's chunk graphs, [0] FP64, [1] FP32
    lmtg::SAmg *samg = nullptr;     // the diffusion FP32 PCG's multigrid (built on first use)
    lmtg::DBuf<int16_t> bcol16;     // diffusion pattern's column deltas col - row, when col16
    bool col16 = false;
    lmtg::DBuf<float> Ke32, K32, Dinv32;
    bool have64 = false, have32 = false, have_vec = false;
    double max_diag = 0;

    // loads and constraints (host side until assembly)
    std::vector<double> h_loads;  // nodal + skin loads
    uint64_t nc = 0;
    lmtg::DBuf<uint32_t> cdof;
    lmtg::DBuf<double> ccoef, cres;
    double penalty = 0;
    double penalty_scale = 0;  // > 0: fixed max|diag| used by the penalty instead of recomputing it
    lmtg::DBuf<double> elim_w;  // exact constraints: K u_bar of the last matrix assembly
    double levenberg_marquadt = 0;  // K(i,i) += max|diag| * levenberg_marquadt at assembly
    double density = 0, fvol[3] = {0, 0, 0};     // volume force density f_vol
    lmtg::DBuf<double> spring_coef, spring_target;  // nodal dep_imp_coef_0 terms

    // solver workspace
    lmtg::DBuf<double> w64[6];
    lmtg::DBuf<float> w32[6];
    lmtg::DBuf<double> partials;
    lmtg::DBuf<lmtg::PcgScalars> scal;
    lmtg::PcgScalars *h_scal = nullptr;  // pinned mirror

    // recalage functional (recalage.cu): the mesh's node pattern and element blocks, while the
    // context's pattern and matrices hold the 9-unknown system (nnu = 9)
    lmtg::RecalState *recal = nullptr;

    // preconditioner of the FP32 inner PCG (LMTG_PREC_*): the aggregation multigrid (amg.cu) is
    // built on the first mixed solve after the pattern or the constraints changed, and its
    // numeric part again after every matrix assembly (mat_version)
    int precond = LMTG_PREC_AMG;
    lmtg::AmgState *amg = nullptr;
    uint64_t mat_version = 0;
    std::vector<uint32_t> h_cdof;  // host copy of the constrained DOFs

    // number of kernels this context has launched (reported by lmtg_get_launch_count)
    uint64_t launches = 0;
};

namespace lmtg {

// ---- pattern (pattern.cu) ----
void build_pattern(lmtg_ctx *c);

// ---- element kernels (elem_elast.cu) ----
void launch_elem_elast(lmtg_ctx *c, bool fp64);

// ---- assembly (assemble.cu) ----
void assemble_matrix(lmtg_ctx *c, bool from64, bool want64, bool want32);
void apply_penalty(lmtg_ctx *c, bool mat, bool vec);
void build_block_jacobi(lmtg_ctx *c, bool want64, bool want32);
// element kernel + assembly + penalty + preconditioner for LMTG_ASM_* flags (abi_solve.cu)
void do_assemble(lmtg_ctx *c, int flags);
void copy_k64_to_k32(lmtg_ctx *c);

// ---- adjoint (adjoint.cu) ----
void launch_grad_E(lmtg_ctx *c, const double *a, const double *b, double *g);

// ---- element fields after the solve (fields.cu) ----
void launch_elem_fields(lmtg_ctx *c, const double *u, double *out);
// volume force and nodal springs into K and F at assembly, before the constraints
void apply_body_terms(lmtg_ctx *c, bool mat, bool vec);

// ---- heat diffusion (diffusion.cu) ----
void diff_setup(lmtg_ctx *c, const double *k, uint64_t nk, double rho_c, double dt, double theta,
                uint64_t nbnd, const uint32_t *bnd, double penalty);
int diff_run(lmtg_ctx *c, int nsteps, double tol, int maxit, lmtg_solve_stats *st);
int diff_adjoint(lmtg_ctx *c, int nsteps, int ck, const double *target_dev, double tol, int maxit,
                 double *J, std::vector<double> &grad, lmtg_solve_stats *st);

template <class T>
inline void upload_u32(lmtg_ctx *c, DBuf<T> &d, const T *h, size_t n) {
    d.alloc(n);
    if (n) LMTG_CUDA(cudaMemcpyAsync(d.p, h, n * sizeof(T), cudaMemcpyHostToDevice, c->stream));
}

// ---- recalage (recalage.cu) ----
void recal_free(lmtg_ctx *c);

// ---- aggregation multigrid (amg.cu) ----
void amg_free(lmtg_ctx *c);

// ---- batches (batch.cu) ----
void batch_free(lmtg_ctx *c);
// destroys the diffusion PCG's cached chunk graphs (diffusion.cu)
void diff_graphs_free(lmtg_ctx *c);
// destroys the diffusion multigrid and the chunk graphs captured on it (diffusion.cu)
void samg_free(lmtg_ctx *c);
void batch_set_rhs(lmtg_ctx *c, int nrhs, const double *B_host);
int batch_solve(lmtg_ctx *c, int mode, double tol, int maxit, double timeout_s, lmtg_solve_stats *st,
                int *pair_iters);
void batch_get_result(lmtg_ctx *c, double *X_host);
void batch_info(lmtg_ctx *c, int *tile_rows, int *variant, uint64_t *ntiles, double *tuned_ms);

// ---- solver (solver.cu) ----
void spmv64(lmtg_ctx *c, const double *x, double *y);
void spmv32(lmtg_ctx *c, const float *x, float *y);
// Solves K x = b (defaults: b = F, x = u) from the current x.
int solve_pcg64(lmtg_ctx *c, int crit_kind, double tol, int maxit, double timeout_s,
                lmtg_solve_stats *st, const double *b = nullptr, double *x = nullptr);
int solve_mixed(lmtg_ctx *c, double tol, int maxit, double timeout_s, lmtg_solve_stats *st,
                const double *b = nullptr, double *x = nullptr);
void profile_pcg(lmtg_ctx *c, bool fp32, int iters, double *spmv_ms, double *update_ms);
// FP32 SpMV kind in use (0 warp-row, 1, 2 bulk copies)
int spmv_kind_in_use(const lmtg_ctx *c);
// per-stage device times of the multigrid-preconditioned FP32 iteration (amg.cu stages)
void profile_amg(lmtg_ctx *c, int iters, double *ms);

// ---- utilities (pattern.cu) ----
// Exclusive scan of u32 counts into u32 offsets (out has count+1 entries); returns the total.
uint64_t exclusive_scan_u32(lmtg_ctx *c, const uint32_t *in, uint32_t *out, uint64_t count);

inline int grid_for(lmtg_ctx *c, uint64_t work, int threads, int per_sm = 8) {
    uint64_t want = (work + threads - 1) / threads;
    uint64_t cap = (uint64_t)c->sm_count * per_sm;
    if (want > cap) want = cap;
    return (int)(want < 1 ? 1 : want);
}

}  // namespace lmtg

// ---- device helpers ----
template <class T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
template <class T>
__device__ __forceinline__ T warp_max(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Position of component v (0..8, row-major 3x3) of local block b of a node row that starts at
// block rb and has deg blocks.  Rows are stored planar: the deg values of each component are
// contiguous, so lane b of a warp reads component v of its block with one coalesced load.
__host__ __device__ __forceinline__ uint64_t kidx(uint32_t rb, uint32_t deg, uint32_t b, int v) {
    return 9ull * rb + (uint64_t)v * deg + b;
}

// Upper node-pair index of (a, b), a <= b, among npe nodes.
__host__ __device__ __forceinline__ int pair_index(int a, int b, int npe) {
    return a * npe - (a * (a - 1)) / 2 + (b - a);
}
