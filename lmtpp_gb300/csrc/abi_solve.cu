// abi_solve.cu -- assemble / get_mat / solve entry points of include/lmtg.h.
#include <cmath>
#include <cstring>
#include <exception>
#include <new>

#include "lmtg_internal.cuh"

using namespace lmtg;

namespace {

template <class F>
int guard2(lmtg_ctx *c, F &&f) {
    if (!c) return LMTG_ERR_ARG;
    try {
        cudaError_t e = cudaSetDevice(c->device);
        if (e != cudaSuccess) throw Error{LMTG_ERR_CUDA, cudaGetErrorString(e)};
        int s = f();
        if (s == LMTG_OK) c->err.clear();
        return s;
    } catch (const Error &e) {
        c->err = e.msg;
        return e.status;
    } catch (const std::bad_alloc &) {
        c->err = "host allocation failed";
        return LMTG_ERR_NOMEM;
    } catch (const std::exception &e) {
        c->err = e.what();
        return LMTG_ERR_CUDA;
    }
}

}  // namespace

namespace lmtg {

void do_assemble(lmtg_ctx *c, int flags) {
    Phase ph("lmtg.assemble");
    LMTG_CHECK(c->allocated, LMTG_ERR_STATE, "allocate_matrices first");
    LMTG_CHECK(c->nnu == 3, LMTG_ERR_STATE, "elasticity call on a diffusion context");
    const bool mat = (flags & (LMTG_ASM_MAT64 | LMTG_ASM_MAT32 | LMTG_ASM_MAT32_NATIVE)) != 0;
    const bool vec = (flags & LMTG_ASM_VEC) != 0;
    if (flags & (LMTG_ASM_MAT64 | LMTG_ASM_MAT32)) {
        const bool want32 = (flags & LMTG_ASM_MAT32) != 0;
        const bool want64 = (flags & LMTG_ASM_MAT64) != 0 || true;  // the FP64 sum is kept
        launch_elem_elast(c, true);
        assemble_matrix(c, true, want64, want32);
        c->have64 = true;
        c->have32 = want32;
    } else if (flags & LMTG_ASM_MAT32_NATIVE) {
        c->Ke32.alloc(c->ne * (uint64_t)c->npairs * 9);
        launch_elem_elast(c, false);
        assemble_matrix(c, false, false, true);
        c->have64 = false;
        c->have32 = true;
    }
    if (vec) {
        LMTG_CUDA(cudaMemcpyAsync(c->F.p, c->h_loads.data(), sizeof(double) * c->n,
                                  cudaMemcpyHostToDevice, c->stream));
        c->have_vec = true;
    }
    apply_body_terms(c, mat, vec);
    if (mat || vec) apply_penalty(c, mat, vec);
    if (mat) {
        build_block_jacobi(c, c->have64, c->have32);
        ++c->mat_version;
    }
    LMTG_CUDA(cudaStreamSynchronize(c->stream));
}

}  // namespace lmtg

extern "C" {

int lmtg_assemble(lmtg_ctx *c, int flags) {
    return guard2(c, [&] {
        do_assemble(c, flags);
        return LMTG_OK;
    });
}

int lmtg_get_matrix_lower(lmtg_ctx *c, uint64_t *rowptr, uint32_t *col, double *val) {
    return guard2(c, [&] {
        LMTG_CHECK(c->have64 || c->have32, LMTG_ERR_STATE, "assemble first");
        LMTG_CHECK(rowptr && col && val, LMTG_ERR_ARG, "null output");
        std::vector<uint32_t> bptr(c->nn + 1), bcol(c->nnzb);
        std::vector<double> K(c->nnzb * 9);
        LMTG_CUDA(cudaMemcpy(bptr.data(), c->bptr.p, bptr.size() * 4, cudaMemcpyDeviceToHost));
        LMTG_CUDA(cudaMemcpy(bcol.data(), c->bcol.p, bcol.size() * 4, cudaMemcpyDeviceToHost));
        if (c->have64) {
            LMTG_CUDA(cudaMemcpy(K.data(), c->K64.p, K.size() * 8, cudaMemcpyDeviceToHost));
        } else {
            std::vector<float> K32(K.size());
            LMTG_CUDA(cudaMemcpy(K32.data(), c->K32.p, K32.size() * 4, cudaMemcpyDeviceToHost));
            for (size_t i = 0; i < K.size(); ++i) K[i] = K32[i];
        }
        uint64_t w = 0;
        rowptr[0] = 0;
        for (uint64_t i = 0; i < c->nn; ++i)
            for (int r = 0; r < 3; ++r) {
                const uint32_t rb = bptr[i], deg = bptr[i + 1] - rb;
                for (uint32_t k = rb; k < rb + deg; ++k) {
                    const uint32_t J = bcol[k];
                    if (J > i) break;
                    const int dmax = (J == i) ? r : 2;
                    for (int d = 0; d <= dmax; ++d) {
                        col[w] = 3 * J + d;
                        val[w] = K[kidx(rb, deg, k - rb, 3 * r + d)];
                        ++w;
                    }
                }
                rowptr[3 * i + r + 1] = w;
            }
        return LMTG_OK;
    });
}

int lmtg_get_sollicitation(lmtg_ctx *c, double *F) {
    return guard2(c, [&] {
        LMTG_CHECK(c->have_vec && F, LMTG_ERR_STATE, "assemble the vector first");
        LMTG_CUDA(cudaMemcpy(F, c->F.p, c->n * 8, cudaMemcpyDeviceToHost));
        return LMTG_OK;
    });
}

int lmtg_get_element_matrices(lmtg_ctx *c, int precision, uint64_t e0, uint64_t count, double *Ke) {
    return guard2(c, [&] {
        LMTG_CHECK(Ke && e0 + count <= c->ne, LMTG_ERR_ARG, "element range");
        const int P = c->npairs, nd = 3 * c->npe;
        std::vector<double> blk((size_t)count * P * 9);
        if (precision == 0) {
            LMTG_CHECK(c->have64, LMTG_ERR_STATE, "no FP64 element matrices");
            LMTG_CUDA(cudaMemcpy(blk.data(), c->Ke64.p + e0 * P * 9, blk.size() * 8,
                                 cudaMemcpyDeviceToHost));
        } else {
            LMTG_CHECK(c->Ke32.p, LMTG_ERR_STATE, "no FP32 element matrices");
            std::vector<float> b32(blk.size());
            LMTG_CUDA(cudaMemcpy(b32.data(), c->Ke32.p + e0 * P * 9, b32.size() * 4,
                                 cudaMemcpyDeviceToHost));
            for (size_t i = 0; i < blk.size(); ++i) blk[i] = b32[i];
        }
        for (uint64_t e = 0; e < count; ++e)
            for (int a = 0; a < c->npe; ++a)
                for (int b = a; b < c->npe; ++b) {
                    const double *s = &blk[((size_t)e * P + pair_index(a, b, c->npe)) * 9];
                    double *o = Ke + e * nd * nd;
                    for (int i = 0; i < 3; ++i)
                        for (int j = 0; j < 3; ++j) {
                            o[(3 * a + i) * nd + 3 * b + j] = s[3 * i + j];
                            o[(3 * b + j) * nd + 3 * a + i] = s[3 * i + j];
                        }
                }
        return LMTG_OK;
    });
}

int lmtg_solve_system(lmtg_ctx *c, int mode, int crit_kind, double tol, int maxit,
                      double timeout_s, lmtg_solve_stats *st) {
    lmtg_solve_stats local{};
    if (!st) st = &local;
    memset(st, 0, sizeof(*st));
    int s = guard2(c, [&] {
        LMTG_CHECK(c->have_vec, LMTG_ERR_STATE, "assemble the vector first");
        LMTG_CHECK(maxit > 0 && tol >= 0, LMTG_ERR_ARG, "maxit > 0, tol >= 0");
        LMTG_CHECK(crit_kind >= 0 && crit_kind <= 3, LMTG_ERR_ARG, "unknown criterion");
        cudaEvent_t e0, e1;
        LMTG_CUDA(cudaEventCreate(&e0));
        LMTG_CUDA(cudaEventCreate(&e1));
        LMTG_CUDA(cudaEventRecord(e0, c->stream));
        int status;
        if (mode == LMTG_SOLVE_PCG_F64) {
            LMTG_CHECK(c->have64, LMTG_ERR_STATE, "FP64 matrix not assembled");
            status = solve_pcg64(c, crit_kind, tol, maxit, timeout_s, st);
        } else if (mode == LMTG_SOLVE_MIXED_IR) {
            LMTG_CHECK(c->have64, LMTG_ERR_STATE, "mixed solve needs the FP64 matrix");
            LMTG_CHECK(crit_kind == LMTG_CRIT_REL_RESIDUAL, LMTG_ERR_ARG,
                       "mixed solve stops on the FP64 relative residual");
            if (!c->have32) {
                copy_k64_to_k32(c);
                build_block_jacobi(c, false, true);
            }
            status = solve_mixed(c, tol, maxit, timeout_s, st);
        } else {
            throw Error{LMTG_ERR_ARG, "unknown solve mode"};
        }
        LMTG_CUDA(cudaEventRecord(e1, c->stream));
        LMTG_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        st->device_ms = ms;
        if (status != LMTG_OK) c->err = lmtg_status_string(status);
        return status;
    });
    st->status = s;
    return s;
}

int lmtg_solve(lmtg_ctx *c, int mode, int crit_kind, double tol, int maxit, double timeout_s,
               lmtg_solve_stats *st) {
    int s = guard2(c, [&] {
        do_assemble(c, LMTG_ASM_MAT64 | LMTG_ASM_VEC |
                           (mode == LMTG_SOLVE_MIXED_IR ? LMTG_ASM_MAT32 : 0));
        return LMTG_OK;
    });
    if (s != LMTG_OK) return s;
    return lmtg_solve_system(c, mode, crit_kind, tol, maxit, timeout_s, st);
}

int lmtg_get_result(lmtg_ctx *c, double *u) {
    return guard2(c, [&] {
        LMTG_CHECK(c->allocated && u, LMTG_ERR_STATE, "allocate_matrices first");
        LMTG_CUDA(cudaMemcpyAsync(u, c->u.p, c->n * 8, cudaMemcpyDeviceToHost, c->stream));
        LMTG_CUDA(cudaStreamSynchronize(c->stream));
        return LMTG_OK;
    });
}

int lmtg_element_fields(lmtg_ctx *c, const double *u, double *out) {
    return guard2(c, [&] {
        LMTG_CHECK(c->allocated && c->nnu == 3, LMTG_ERR_STATE, "elasticity allocate_matrices first");
        LMTG_CHECK(c->E.p, LMTG_ERR_STATE, "material_set first");
        LMTG_CHECK(out, LMTG_ERR_ARG, "null output");
        DBuf<double> ud, od;
        const double *up = c->u.p;
        if (u) {
            ud.alloc(c->n);
            LMTG_CUDA(cudaMemcpyAsync(ud.p, u, c->n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
            up = ud.p;
        }
        od.alloc(13 * c->ne);
        launch_elem_fields(c, up, od.p);
        LMTG_CUDA(cudaMemcpyAsync(out, od.p, 13 * c->ne * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        LMTG_CUDA(cudaStreamSynchronize(c->stream));
        return LMTG_OK;
    });
}

int lmtg_set_result(lmtg_ctx *c, const double *u) {
    return guard2(c, [&] {
        LMTG_CHECK(c->allocated && u, LMTG_ERR_STATE, "allocate_matrices first");
        LMTG_CUDA(cudaMemcpyAsync(c->u.p, u, c->n * 8, cudaMemcpyHostToDevice, c->stream));
        LMTG_CUDA(cudaStreamSynchronize(c->stream));
        return LMTG_OK;
    });
}

int lmtg_spmv(lmtg_ctx *c, int precision, const double *x, double *y) {
    return guard2(c, [&] {
        LMTG_CHECK(x && y, LMTG_ERR_ARG, "null vector");
        if (precision == 0) {
            LMTG_CHECK(c->have64, LMTG_ERR_STATE, "FP64 matrix not assembled");
            LMTG_CUDA(cudaMemcpyAsync(c->w64[0].p, x, c->n * 8, cudaMemcpyHostToDevice, c->stream));
            spmv64(c, c->w64[0].p, c->w64[1].p);
            LMTG_CUDA(cudaMemcpyAsync(y, c->w64[1].p, c->n * 8, cudaMemcpyDeviceToHost, c->stream));
            LMTG_CUDA(cudaStreamSynchronize(c->stream));
        } else {
            LMTG_CHECK(c->have32, LMTG_ERR_STATE, "FP32 matrix not assembled");
            std::vector<float> xs(x, x + c->n), ys(c->n);
            LMTG_CUDA(cudaMemcpyAsync(c->w32[0].p, xs.data(), c->n * 4, cudaMemcpyHostToDevice,
                                      c->stream));
            spmv32(c, c->w32[0].p, c->w32[1].p);
            LMTG_CUDA(cudaMemcpyAsync(ys.data(), c->w32[1].p, c->n * 4, cudaMemcpyDeviceToHost,
                                      c->stream));
            LMTG_CUDA(cudaStreamSynchronize(c->stream));
            for (uint64_t i = 0; i < c->n; ++i) y[i] = ys[i];
        }
        return LMTG_OK;
    });
}

int lmtg_get_stream(lmtg_ctx *c, void **stream) {
    if (!c || !stream) return LMTG_ERR_ARG;
    *stream = (void *)c->stream;
    return LMTG_OK;
}

int lmtg_get_launch_count(lmtg_ctx *c, uint64_t *count) {
    if (!c || !count) return LMTG_ERR_ARG;
    *count = c->launches;
    return LMTG_OK;
}

int lmtg_profile_pcg_kernels(lmtg_ctx *c, int precision, int iters, double *spmv_ms,
                             double *update_ms) {
    return guard2(c, [&] {
        LMTG_CHECK(spmv_ms && update_ms && iters > 0, LMTG_ERR_ARG, "bad arguments");
        LMTG_CHECK(c->have_vec && (precision ? c->have32 : c->have64), LMTG_ERR_STATE,
                   "assemble the system first");
        profile_pcg(c, precision != 0, iters, spmv_ms, update_ms);
        return LMTG_OK;
    });
}

int lmtg_get_sizes(lmtg_ctx *c, uint64_t *nn, uint64_t *ne, uint64_t *ndof, uint64_t *nnz_blocks) {
    if (!c) return LMTG_ERR_ARG;
    if (nn) *nn = c->nn;
    if (ne) *ne = c->ne;
    if (ndof) *ndof = c->n;
    if (nnz_blocks) *nnz_blocks = c->nnzb;
    return LMTG_OK;
}

}  // extern "C"
