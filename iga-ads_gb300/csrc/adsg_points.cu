// C-ABI of the Gauss-point utilities: interpolation to the quadrature points,
// load vectors and L2 projection, norms and errors, non-finite counts.
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
// Gauss-point utilities
// ---------------------------------------------------------------------------
namespace {

long long quad_extent(const adsg_ctx* c, int d) { return static_cast<long long>(c->dims[d].elements) * c->dims[d].q; }

long long quad_total(const adsg_ctx* c) {
    long long t = 1;
    for (int d = 0; d < c->ndim; ++d) t *= quad_extent(c, d);
    return t;
}

int qpool_get(adsg_ctx* c, size_t doubles, double** out) {
    if (c->qpool_size < doubles) {
        if (c->qpool) {
            cudaStreamSynchronize(c->stream);
            cudaFree(c->qpool);
            c->qpool = nullptr;
            c->qpool_size = 0;
        }
        ADSG_CUDA_TRY(device_alloc(reinterpret_cast<void**>(&c->qpool), doubles * sizeof(double)),
                      "Gauss-point work space");
        c->qpool_size = doubles;
    }
    *out = c->qpool;
    return 0;
}

// interpolate u to the Gauss points: val (and the ndim derivatives in grad)
int enqueue_eval_quad(adsg_ctx* c, const double* u, double* val, double* grad) {
    const int nd = c->ndim;
    const long long n1 = nd > 1 ? c->n[1] : 1, n2 = nd > 2 ? c->n[2] : 1;
    const long long Q0 = quad_extent(c, 0), Q1 = nd > 1 ? quad_extent(c, 1) : 1, Q2 = nd > 2 ? quad_extent(c, 2) : 1;
    const long long NQ = Q0 * Q1 * Q2;
    cudaStream_t s = c->stream;
    if (nd == 1) {
        ADSG_CUDA_TRY(launch_quad_interp(u, val, grad, c->dims[0], 1, 1, s), "interp x");
        return 0;
    }
    const size_t a = static_cast<size_t>(Q0 * n1 * n2), b = static_cast<size_t>(Q0 * Q1 * n2);
    double* w = nullptr;
    if (int st = qpool_get(c, 2 * a + 3 * b, &w)) return st;
    double *A0 = w, *A1 = w + a, *B00 = w + 2 * a, *B01 = B00 + b, *B10 = B01 + b;
    const bool g = grad != nullptr;
    ADSG_CUDA_TRY(launch_quad_interp(u, A0, g ? A1 : nullptr, c->dims[0], 1, n1 * n2, s), "interp x");
    if (nd == 2) {
        ADSG_CUDA_TRY(launch_quad_interp(A0, val, g ? grad + NQ : nullptr, c->dims[1], Q0, 1, s), "interp y");
        if (g) ADSG_CUDA_TRY(launch_quad_interp(A1, grad, nullptr, c->dims[1], Q0, 1, s), "interp y");
        return 0;
    }
    ADSG_CUDA_TRY(launch_quad_interp(A0, B00, g ? B01 : nullptr, c->dims[1], Q0, n2, s), "interp y");
    if (g) ADSG_CUDA_TRY(launch_quad_interp(A1, B10, nullptr, c->dims[1], Q0, n2, s), "interp y");
    ADSG_CUDA_TRY(launch_quad_interp(B00, val, g ? grad + 2 * NQ : nullptr, c->dims[2], Q0 * Q1, 1, s), "interp z");
    if (g) {
        ADSG_CUDA_TRY(launch_quad_interp(B01, grad + NQ, nullptr, c->dims[2], Q0 * Q1, 1, s), "interp z");
        ADSG_CUDA_TRY(launch_quad_interp(B10, grad, nullptr, c->dims[2], Q0 * Q1, 1, s), "interp z");
    }
    return 0;
}

int enqueue_load_vector(adsg_ctx* c, const double* fq, double* out) {
    const int nd = c->ndim;
    const long long n0 = c->n[0], n1 = nd > 1 ? c->n[1] : 1;
    const long long Q1 = nd > 1 ? quad_extent(c, 1) : 1, Q2 = nd > 2 ? quad_extent(c, 2) : 1;
    cudaStream_t s = c->stream;
    if (nd == 1) {
        ADSG_CUDA_TRY(launch_quad_project(fq, out, c->dims[0], c->dims[0].erange, 1, 1, s), "project x");
        return 0;
    }
    const size_t a = static_cast<size_t>(n0 * Q1 * Q2), b = static_cast<size_t>(n0 * n1 * Q2);
    double* w = nullptr;
    if (int st = qpool_get(c, a + (nd == 3 ? b : 0), &w)) return st;
    ADSG_CUDA_TRY(launch_quad_project(fq, w, c->dims[0], c->dims[0].erange, 1, Q1 * Q2, s), "project x");
    if (nd == 2) {
        ADSG_CUDA_TRY(launch_quad_project(w, out, c->dims[1], c->dims[1].erange, n0, 1, s), "project y");
        return 0;
    }
    ADSG_CUDA_TRY(launch_quad_project(w, w + a, c->dims[1], c->dims[1].erange, n0, Q2, s), "project y");
    ADSG_CUDA_TRY(launch_quad_project(w + a, out, c->dims[2], c->dims[2].erange, n0 * n1, 1, s), "project z");
    return 0;
}

}  // namespace

long long adsg_quad_size(const adsg_ctx* ctx) { return ctx ? quad_total(ctx) : 0; }

int adsg_count_nonfinite(adsg_ctx* ctx, const double* u_dev, long long* count_out) {
    if (!ctx) return fail(-1, "ctx is NULL");
    if (!u_dev) return fail(-2, "u is NULL");
    if (!count_out) return fail(-3, "count is NULL");
    if (!ctx->red) ADSG_CUDA_TRY(ctx->arena.alloc(&ctx->red, 1025), "reduction alloc");
    auto* cnt = reinterpret_cast<unsigned long long*>(ctx->red + 1024);
    ADSG_CUDA_TRY(launch_count_nonfinite(u_dev, ctx->size, cnt, ctx->stream), "count");
    unsigned long long host = 0;
    ADSG_CUDA_TRY(cudaMemcpyAsync(&host, cnt, sizeof(host), cudaMemcpyDeviceToHost, ctx->stream), "D2H");
    ADSG_CUDA_TRY(cudaStreamSynchronize(ctx->stream), "synchronize");
    *count_out = static_cast<long long>(host);
    return 0;
}

int adsg_load_vector(adsg_ctx* ctx, const double* fq_dev, double* out_dev) {
    if (!ctx) return fail(-1, "ctx is NULL");
    if (!fq_dev) return fail(-2, "fq is NULL");
    if (!out_dev) return fail(-3, "out is NULL");
    return enqueue_load_vector(ctx, fq_dev, out_dev);
}

int adsg_projection(adsg_ctx* ctx, const double* fq_dev, double* out_dev) {
    if (int st = adsg_load_vector(ctx, fq_dev, out_dev)) return st;
    return ctx_solve(ctx, out_dev, 0);
}

int adsg_eval_quad(adsg_ctx* ctx, const double* u_dev, double* val_dev, double* grad_dev) {
    if (!ctx) return fail(-1, "ctx is NULL");
    if (!u_dev) return fail(-2, "u is NULL");
    if (!val_dev) return fail(-3, "val is NULL");
    return enqueue_eval_quad(ctx, u_dev, val_dev, grad_dev);
}

int adsg_norms(adsg_ctx* ctx, const double* u_dev, double* l2_out, double* h1_out) {
    if (!ctx) return fail(-1, "ctx is NULL");
    if (!u_dev) return fail(-2, "u is NULL");
    if (!l2_out) return fail(-3, "l2 is NULL");
    if (!h1_out) return fail(-4, "h1 is NULL");
    double* w = nullptr;
    if (int st = qpool_get(ctx, static_cast<size_t>(ctx->size), &w)) return st;
    if (!ctx->red) ADSG_CUDA_TRY(ctx->arena.alloc(&ctx->red, 1025), "reduction alloc");
    double vals[2];
    const double dts[2] = {0.0, -1.0};  // rhs(dt) = M u - dt K u: dt = 0 -> M u, dt = -1 -> (M + K) u
    for (int k = 0; k < 2; ++k) {
        if (int st = ctx_rhs(ctx, u_dev, w, dts[k])) return st;
        ADSG_CUDA_TRY(launch_dot(u_dev, w, ctx->size, ctx->red, ctx->red + 1024, ctx->stream), "dot");
        ADSG_CUDA_TRY(cudaMemcpyAsync(&vals[k], ctx->red + 1024, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream),
                      "D2H");
        ADSG_CUDA_TRY(cudaStreamSynchronize(ctx->stream), "synchronize");
    }
    *l2_out = std::sqrt(std::max(vals[0], 0.0));
    *h1_out = std::sqrt(std::max(vals[1], 0.0));
    return 0;
}

int adsg_errors(adsg_ctx* ctx, const double* u_dev, const double* fq_dev, const double* fgrad_dev, double* l2_out,
                double* h1_out) {
    if (!ctx) return fail(-1, "ctx is NULL");
    if (!u_dev) return fail(-2, "u is NULL");
    if (!fq_dev) return fail(-3, "fq is NULL");
    if (!l2_out) return fail(-5, "l2 is NULL");
    if (!h1_out) return fail(-6, "h1 is NULL");
    const long long NQ = quad_total(ctx);
    const int nd = ctx->ndim;
    // the interpolation's own work space first, then the point tensors after it
    const long long n1 = nd > 1 ? ctx->n[1] : 1, n2 = nd > 2 ? ctx->n[2] : 1;
    const long long Q0 = quad_extent(ctx, 0), Q1 = nd > 1 ? quad_extent(ctx, 1) : 1;
    const size_t work = nd == 1 ? 0 : static_cast<size_t>(2 * Q0 * n1 * n2 + 3 * Q0 * Q1 * n2);
    double* w = nullptr;
    if (int st = qpool_get(ctx, work + static_cast<size_t>(NQ) * (1 + nd), &w)) return st;
    double* val = w + work;
    double* grad = val + NQ;
    // enqueue_eval_quad uses the front of the pool; keep the point tensors behind it
    if (int st = enqueue_eval_quad(ctx, u_dev, val, fgrad_dev ? grad : nullptr)) return st;
    if (!ctx->red) ADSG_CUDA_TRY(ctx->arena.alloc(&ctx->red, 1025), "reduction alloc");
    double l2 = 0.0, g2 = 0.0;
    field_set F;
    F.nf = 1;
    F.a[0] = val;
    F.b[0] = fq_dev;
    ADSG_CUDA_TRY(launch_quad_wdiff(F, ctx->dims, nd, NQ, ctx->red, ctx->red + 1024, ctx->stream), "weighted sum");
    ADSG_CUDA_TRY(cudaMemcpyAsync(&l2, ctx->red + 1024, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream), "D2H");
    ADSG_CUDA_TRY(cudaStreamSynchronize(ctx->stream), "synchronize");
    if (fgrad_dev) {
        field_set G;
        G.nf = nd;
        for (int k = 0; k < nd; ++k) {
            G.a[k] = grad + k * NQ;
            G.b[k] = fgrad_dev + k * NQ;
        }
        ADSG_CUDA_TRY(launch_quad_wdiff(G, ctx->dims, nd, NQ, ctx->red, ctx->red + 1024, ctx->stream), "weighted sum");
        ADSG_CUDA_TRY(cudaMemcpyAsync(&g2, ctx->red + 1024, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream), "D2H");
        ADSG_CUDA_TRY(cudaStreamSynchronize(ctx->stream), "synchronize");
        *h1_out = std::sqrt(l2 + g2);
    } else {
        *h1_out = -1.0;
    }
    *l2_out = std::sqrt(l2);
    return 0;
}

int adsg_quad_points(const adsg_ctx* ctx, int d, double* xq_host) {
    if (!ctx) return fail(-1, "ctx is NULL");
    if (d < 0 || d >= ctx->ndim) return fail(-2, "direction out of range");
    if (!xq_host) return fail(-3, "xq is NULL");
    if (ctx->xq[d].empty()) return fail(ADSG_ERR_UNSUPPORTED, "the descriptor gave no Gauss points (xq)");
    std::memcpy(xq_host, ctx->xq[d].data(), sizeof(double) * ctx->xq[d].size());
    return 0;
}

}  // extern "C"
