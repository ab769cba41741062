// amg.cuh -- state of the aggregation multigrid preconditioner (amg.cu).
#pragma once
#include <memory>
#include <vector>

#include "solver_kernels.cuh"

namespace lmtg {

// One level of the hierarchy.  Level 0 is the context's own matrix (bptr/bcol/K32/Dinv32 of
// lmtg_ctx); deeper levels hold their 6x6-block matrices here (planar rows, 36 components).
struct AmgLevel {
    int b = 3;                        // unknowns per node: 3 at level 0, 6 below
    uint64_t nn = 0, nnzb = 0;
    DBuf<uint32_t> bptr, bcol, bdiag;  // levels >= 1
    DBuf<float> K, Dinv;               // levels >= 1: 6x6 blocks and their inverses
    float omega = 1.f;                 // damped block-Jacobi weight
    double lambda = 0;                 // lambda_max(D^-1 K) estimate
    DBuf<float> r;                     // right-hand side (packed b per node), levels >= 1
    DBuf<float> xa, xb;                // iterates, padded to 4 (level 0) or 8 per node
    DBuf<float> res;                   // residual (packed); on the coarsest, its solution
    DBuf<float> r2, xb2;               // levels >= 1: right-hand side and result of a second cycle
    bool bulk = false;                 // row products by the bulk-copy kernel (large 6x6 levels)
    // transfer to the next coarser level
    uint64_t nagg = 0;
    DBuf<uint32_t> agg;          // node -> aggregate (0xffffffff: in none)
    DBuf<uint32_t> aptr, anode;  // aggregate -> nodes
    DBuf<float> Q;               // tentative prolongator, b x 6 per node (row-major)
    DBuf<uint8_t> gslot;         // per fine block: slot of its coarse block in the coarse row
};

struct AmgState {
    std::vector<std::unique_ptr<AmgLevel>> levels;
    int nc = 0;             // unknowns of the dense coarsest level (0: no hierarchy)
    DBuf<float> Cinv;       // its inverse, row-major
    DBuf<double> power;     // |w|^2 and v.w of every power step, per level
    uint64_t version = ~0ull;  // matrix version of the numeric setup
    uint32_t max_cdeg = 0;     // widest coarse row over the levels
    double structure_ms = 0, numeric_ms = 0;
    // host time of the structure setup by phase: pattern copy and modes, aggregation, tentative
    // prolongators, coarse patterns and gather lists, uploads
    double phase_ms[5] = {0, 0, 0, 0, 0};
};

void amg_free(lmtg_ctx *c);
bool amg_applicable(const lmtg_ctx *c);
// Builds what is missing (structure, then numeric setup for the current matrix); false when the
// preconditioner is block Jacobi for this context.
bool amg_prepare(lmtg_ctx *c);
float amg_omega0(const lmtg_ctx *c);
float *amg_xa0(const lmtg_ctx *c);
void amg_launch_cycle(lmtg_ctx *c, const float *r, float *z, cudaStream_t s, int start, double beta_den,
                      cudaEvent_t *ev = nullptr);
void amg_info(const lmtg_ctx *c, int *levels, uint64_t *ndof, uint64_t *nnzb, double *omega, double *lambda,
              double *structure_ms, double *numeric_ms, double *phase_ms);

}  // namespace lmtg
