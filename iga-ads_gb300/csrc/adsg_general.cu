// C-ABI of the generalised ADS solve: per-line bands along one special
// direction.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "adsg_context.cuh"

using namespace adsg;

extern "C" {

// ---------------------------------------------------------------------------
// Generalised ADS: per-line bands along one special direction.
// ---------------------------------------------------------------------------
struct adsg_line_bands {
    line_tables T;
    long long nlines = 0;
    int* line_matrix = nullptr;
    int ku = 0;
    dev_arena arena;
};

int adsg_line_bands_create(int n, int kl, int ku, int ldab, int nmat, const double* ab, const int* ipiv,
                           long long nlines, const int* line_matrix, adsg_line_bands** out) {
    if (n < 1) return fail(-1, "n must be >= 1");
    if (kl < 0 || kl > 16) return fail(-2, "kl must be in [0, 16]");
    if (ku < 0 || kl + ku > 32) return fail(-3, "ku must be >= 0 and kl + ku <= 32");
    if (ldab < 2 * kl + ku + 1) return fail(-4, "ldab < 2*kl+ku+1");
    if (nmat < 1) return fail(-5, "nmat must be >= 1");
    if (!ab) return fail(-6, "ab is NULL");
    if (!ipiv) return fail(-7, "ipiv is NULL");
    if (nlines < 1) return fail(-8, "nlines must be >= 1");
    if (!line_matrix) return fail(-9, "line_matrix is NULL");
    if (!out) return fail(-10, "out is NULL");
    for (long long l = 0; l < nlines; ++l)
        if (line_matrix[l] < 0 || line_matrix[l] >= nmat) return fail(-9, "line_matrix entry out of range");
    std::vector<double> lmul, ucol, rdiag;
    std::vector<int> piv, uext;
    int tkl = 1, tw = 1;
    for (int m = 0; m < nmat; ++m) {
        const int* pm = ipiv + static_cast<size_t>(m) * n;
        for (int j = 0; j < n; ++j)
            if (pm[j] < j + 1 || pm[j] > std::min(n, j + 1 + kl)) return fail(-7, "pivot outside the band");
        solve_tables t;
        if (make_solve_tables(n, kl, ku, ldab, ab + static_cast<size_t>(m) * ldab * n, pm, t))
            return fail(ADSG_ERR_SINGULAR, "zero diagonal in a factorised band");
        tkl = t.kl;
        tw = t.w;
        lmul.insert(lmul.end(), t.lmul.begin(), t.lmul.begin() + static_cast<long long>(n) * t.kl);
        ucol.insert(ucol.end(), t.ucol.begin(), t.ucol.end());
        rdiag.insert(rdiag.end(), t.rdiag.begin(), t.rdiag.end());
        piv.insert(piv.end(), t.piv.begin(), t.piv.end());
        uext.insert(uext.end(), t.uext.begin(), t.uext.end());
    }
    auto* b = new (std::nothrow) adsg_line_bands;
    if (!b) return fail(ADSG_ERR_NOMEM, "host allocation failed");
    b->T.n = n;
    b->T.kl = tkl;
    b->T.w = tw;
    b->T.nmat = nmat;
    b->nlines = nlines;
    b->ku = ku;
    double *dl, *du, *dr;
    int *dp, *de;
    cudaError_t e = b->arena.upload(&dl, lmul.data(), lmul.size(), nullptr);
    if (e == cudaSuccess) e = b->arena.upload(&du, ucol.data(), ucol.size(), nullptr);
    if (e == cudaSuccess) e = b->arena.upload(&dr, rdiag.data(), rdiag.size(), nullptr);
    if (e == cudaSuccess) e = b->arena.upload(&dp, piv.data(), piv.size(), nullptr);
    if (e == cudaSuccess) e = b->arena.upload(&de, uext.data(), uext.size(), nullptr);
    if (e == cudaSuccess) e = b->arena.upload(&b->line_matrix, line_matrix, static_cast<size_t>(nlines), nullptr);
    if (e == cudaSuccess) e = cudaStreamSynchronize(nullptr);
    if (e != cudaSuccess) {
        delete b;
        return fail_cuda(e, "line bands upload");
    }
    b->T.lmul = dl;
    b->T.ucol = du;
    b->T.rdiag = dr;
    b->T.piv = dp;
    b->T.uext = de;
    *out = b;
    return 0;
}

int adsg_line_bands_destroy(adsg_line_bands* b) {
    delete b;
    return 0;
}

int adsg_ads_solve_general(adsg_ctx* ctx, int special_dim, const adsg_line_bands* lines, double* rhs_dev) {
    if (!ctx) return fail(-1, "ctx is NULL");
    if (special_dim < 0 || special_dim >= ctx->ndim) return fail(-2, "special_dim out of range");
    if (!lines) return fail(-3, "lines is NULL");
    if (!rhs_dev) return fail(-4, "rhs is NULL");
    if (lines->T.n != ctx->n[special_dim]) return fail(-3, "line bands size differs from the special dimension");
    const line_layout Ls = make_line_layout(ctx->n, ctx->ndim, special_dim);
    if (lines->nlines != Ls.nlines) return fail(-3, "line_matrix length differs from the number of lines");
    {
        stage_scope sc(ctx, ADSG_STAGE_SOLVE_X + special_dim);
        ADSG_CUDA_TRY(launch_line_solve_permat(rhs_dev, lines->T, Ls, lines->line_matrix, ctx->n[0],
                                               ctx->ndim > 2 ? ctx->n[2] : 1, special_dim, ctx->ndim, ctx->stream),
                      "special direction solve");
    }
    // then the standard directions, cyclically after the special one
    for (int k = 1; k < ctx->ndim; ++k) {
        const int d = (special_dim + k) % ctx->ndim;
        const line_layout L = make_line_layout(ctx->n, ctx->ndim, d);
        stage_scope sc(ctx, ADSG_STAGE_SOLVE_X + d);
        ADSG_CUDA_TRY(launch_line_solve(rhs_dev, ctx->dims[d], L, 0, ctx->stream), "line solve");
    }
    return 0;
}

int adsg_ads_solve_general_host(adsg_ctx* ctx, int special_dim, const adsg_line_bands* lines, double* rhs_host) {
    if (!ctx) return fail(-1, "ctx is NULL");
    if (!rhs_host) return fail(-4, "rhs is NULL");
    if (!ctx->host_io) ADSG_CUDA_TRY(ctx->arena.alloc(&ctx->host_io, ctx->size), "io alloc");
    const size_t bytes = sizeof(double) * ctx->size;
    ADSG_CUDA_TRY(cudaMemcpyAsync(ctx->host_io, rhs_host, bytes, cudaMemcpyHostToDevice, ctx->stream), "H2D");
    if (int st = adsg_ads_solve_general(ctx, special_dim, lines, ctx->host_io)) return st;
    ADSG_CUDA_TRY(cudaMemcpyAsync(rhs_host, ctx->host_io, bytes, cudaMemcpyDeviceToHost, ctx->stream), "D2H");
    ADSG_CUDA_TRY(cudaStreamSynchronize(ctx->stream), "synchronize");
    return 0;
}

}  // extern "C"
