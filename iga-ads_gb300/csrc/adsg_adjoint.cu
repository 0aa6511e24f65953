// C-ABI of the adjoint engine (reverse-mode gradients of the kappa-weighted
// explicit step) and of the mass-norm loss.
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
// Adjoint: reverse-mode gradients of a loss of u(T) with respect to the
// initial coefficients and the diffusion-field coefficients kappa, for the
// kappa-weighted explicit step u_{k+1} = M^{-1} R(kappa) u_k.  R is symmetric,
// so the adjoint step is lambda_k = R(kappa) M^{-T} lambda_{k+1}; dL/dkappa
// accumulates mu_{k+1}^T (dR/dkappa) u_k with mu_{k+1} = M^{-T} lambda_{k+1}.
// Forward states are checkpointed every C steps (C = ceil(sqrt(N)) by
// default) and each segment is recomputed once during the backward sweep.
// ---------------------------------------------------------------------------
struct adsg_adjoint {
    adsg_ctx* ctx = nullptr;  // null once the context is destroyed
    int nsteps = 0, every = 1, nck = 0;
    double dt = 0.0;
    bool forward_done = false;
    double* ck = nullptr;     // nck states
    double* seg = nullptr;    // every states
    double* work[2] = {nullptr, nullptr};
    double* kappa = nullptr;  // copy of the field used by the forward pass
    double* kq = nullptr;     // 3D: that field at every element's Gauss points, computed once per forward pass
    double* partial = nullptr;
    double* scalar = nullptr;
    dev_arena arena;
};

extern "C++" {
namespace adsg {

void detach_adjoints(adsg_ctx* c) {
    for (adsg_adjoint* a : c->adjoints) a->ctx = nullptr;
    c->adjoints.clear();
}

}  // namespace adsg
}

namespace {

int elem_step(adsg_adjoint* a, const double* u, double* out) {
    adsg_ctx* c = a->ctx;
    ADSG_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(double) * c->size, c->stream), "memset");
    {
        stage_scope sc(c, ADSG_STAGE_RHS_ELEM);
        // the kappa values at the Gauss points are the ones the element kernel
        // would interpolate from the coefficients, bit for bit: read them
        ADSG_CUDA_TRY(a->kq ? launch_rhs_elem_points(c->dims, u, a->kq, out, a->dt, c->stream)
                            : launch_rhs_elem(c->ndim, c->dims, u, a->kappa, out, a->dt, c->stream),
                      "element rhs");
    }
    return ctx_solve(c, out, 0);
}

}  // namespace

int adsg_adjoint_create(adsg_ctx* ctx, int nsteps, double dt, int checkpoint_every, adsg_adjoint** out) {
    if (!ctx) return fail(-1, "ctx is NULL");
    if (nsteps < 1) return fail(-2, "nsteps must be >= 1");
    if (!std::isfinite(dt)) return fail(-3, "dt must be finite");
    if (checkpoint_every < 0) return fail(-4, "checkpoint_every must be >= 0");
    if (!out) return fail(-5, "out is NULL");
    if (ctx->ndim < 2) return fail(ADSG_ERR_UNSUPPORTED, "the adjoint needs a 2D or 3D context");
    for (int d = 0; d < ctx->ndim; ++d)
        if (ctx->dims[d].p != ctx->dims[0].p || ctx->dims[d].q != ctx->dims[d].p + 1)
            return fail(ADSG_ERR_UNSUPPORTED, "the adjoint needs the same degree and p+1 Gauss points in every direction");
    auto* a = new (std::nothrow) adsg_adjoint;
    if (!a) return fail(ADSG_ERR_NOMEM, "host allocation failed");
    a->ctx = ctx;
    a->nsteps = nsteps;
    a->dt = dt;
    a->every = checkpoint_every > 0 ? checkpoint_every
                                    : std::max(1, static_cast<int>(std::ceil(std::sqrt(static_cast<double>(nsteps)))));
    a->every = std::min(a->every, nsteps);
    a->nck = (nsteps + a->every - 1) / a->every;
    const size_t n = static_cast<size_t>(ctx->size);
    cudaError_t e = a->arena.alloc(&a->ck, n * a->nck);
    if (e == cudaSuccess) e = a->arena.alloc(&a->seg, n * a->every);
    if (e == cudaSuccess) e = a->arena.alloc(&a->work[0], n);
    if (e == cudaSuccess) e = a->arena.alloc(&a->work[1], n);
    if (e == cudaSuccess) e = a->arena.alloc(&a->kappa, n);
    if (e == cudaSuccess && ctx->ndim == 3) {
        // kappa at the Gauss points: (p+1)^3 doubles per element, 1.2 to 15
        // times a state tensor; without the room the passes interpolate the
        // coefficients instead (the same bits, ~10% more time)
        if (a->arena.alloc(&a->kq, static_cast<size_t>(kappa_points_count(3, ctx->dims))) != cudaSuccess) {
            cudaGetLastError();
            a->kq = nullptr;
        }
    }
    if (e == cudaSuccess) e = a->arena.alloc(&a->partial, 1024);
    if (e == cudaSuccess) e = a->arena.alloc(&a->scalar, 1);
    if (e != cudaSuccess) {
        delete a;
        return fail_cuda(e, "adjoint allocation");
    }
    ctx->adjoints.push_back(a);
    *out = a;
    return 0;
}

int adsg_adjoint_destroy(adsg_adjoint* a) {
    if (!a) return 0;
    if (a->ctx) {
        cudaStreamSynchronize(a->ctx->stream);
        auto& v = a->ctx->adjoints;
        v.erase(std::remove(v.begin(), v.end(), a), v.end());
    }
    delete a;  // freeing device memory waits for the device
    return 0;
}

int adsg_adjoint_checkpoints(const adsg_adjoint* a, int* every, int* count) {
    if (!a) return fail(-1, "adjoint is NULL");
    if (every) *every = a->every;
    if (count) *count = a->nck;
    return 0;
}

int adsg_adjoint_forward(adsg_adjoint* a, const double* u0_dev, const double* kappa_dev, double* uT_dev) {
    if (!a) return fail(-1, "adjoint is NULL");
    if (!u0_dev) return fail(-2, "u0 is NULL");
    if (!kappa_dev) return fail(-3, "kappa is NULL");
    if (!uT_dev) return fail(-4, "uT is NULL");
    if (!a->ctx) return fail(-1, "the adjoint's context was destroyed");
    adsg_ctx* c = a->ctx;
    const size_t bytes = sizeof(double) * c->size;
    cudaStream_t s = c->stream;
    ADSG_CUDA_TRY(cudaMemcpyAsync(a->kappa, kappa_dev, bytes, cudaMemcpyDeviceToDevice, s), "copy kappa");
    if (a->kq) ADSG_CUDA_TRY(launch_kappa_points(c->dims, a->kappa, a->kq, s), "kappa at the Gauss points");
    ADSG_CUDA_TRY(cudaMemcpyAsync(a->ck, u0_dev, bytes, cudaMemcpyDeviceToDevice, s), "checkpoint 0");
    const double* cur = a->ck;
    for (int k = 0; k < a->nsteps; ++k) {
        const int kk = k + 1;
        // a state that is checkpointed is computed straight into its slot
        double* nxt = (kk < a->nsteps && kk % a->every == 0) ? a->ck + static_cast<size_t>(kk / a->every) * c->size
                                                             : a->work[k & 1];
        if (int st = elem_step(a, cur, nxt)) return st;
        cur = nxt;
    }
    ADSG_CUDA_TRY(cudaMemcpyAsync(uT_dev, cur, bytes, cudaMemcpyDeviceToDevice, s), "copy u(T)");
    a->forward_done = true;
    return 0;
}

int adsg_adjoint_backward(adsg_adjoint* a, const double* dL_duT_dev, double* grad_u0_dev, double* grad_kappa_dev) {
    if (!a) return fail(-1, "adjoint is NULL");
    if (!dL_duT_dev) return fail(-2, "dL/du(T) is NULL");
    if (!grad_u0_dev) return fail(-3, "grad_u0 is NULL");
    if (!grad_kappa_dev) return fail(-4, "grad_kappa is NULL");
    if (!a->forward_done) return fail(-1, "adsg_adjoint_forward must run first");
    if (!a->ctx) return fail(-1, "the adjoint's context was destroyed");
    adsg_ctx* c = a->ctx;
    const size_t n = static_cast<size_t>(c->size);
    const size_t bytes = sizeof(double) * n;
    cudaStream_t s = c->stream;
    double* lam = a->work[0];
    double* other = a->work[1];
    ADSG_CUDA_TRY(cudaMemcpyAsync(lam, dL_duT_dev, bytes, cudaMemcpyDeviceToDevice, s), "copy lambda");
    ADSG_CUDA_TRY(cudaMemsetAsync(grad_kappa_dev, 0, bytes, s), "zero grad kappa");
    for (int sidx = a->nck - 1; sidx >= 0; --sidx) {
        const int k0 = sidx * a->every;
        const int k1 = std::min(k0 + a->every, a->nsteps);
        // u_{k0} is the checkpoint itself; recompute u_{k0+1} .. u_{k1-1} from it
        const double* ckp = a->ck + static_cast<size_t>(sidx) * n;
        auto state = [&](int k) -> const double* {
            return k == k0 ? ckp : a->seg + static_cast<size_t>(k - k0) * n;
        };
        for (int k = k0 + 1; k < k1; ++k)
            if (int st = elem_step(a, state(k - 1), a->seg + static_cast<size_t>(k - k0) * n)) return st;
        for (int k = k1 - 1; k >= k0; --k) {
            if (int st = ctx_solve(c, lam, 1)) return st;  // lam <- mu_{k+1} = M^{-T} lambda_{k+1}
            ADSG_CUDA_TRY(cudaMemsetAsync(other, 0, bytes, s), "memset");
            {
                // grad kappa += mu^T (dR/dkappa) u_k and other = R^T mu (R is symmetric)
                stage_scope sc(c, ADSG_STAGE_RHS_ELEM);
                ADSG_CUDA_TRY(launch_adjoint_pair(c->ndim, c->dims, state(k), lam, a->kq ? a->kq : a->kappa, other,
                                                  grad_kappa_dev, a->dt, s, a->kq != nullptr),
                              "kappa gradient and R^T mu");
            }
            std::swap(lam, other);  // lam <- lambda_k = R mu_{k+1}
        }
    }
    ADSG_CUDA_TRY(cudaMemcpyAsync(grad_u0_dev, lam, bytes, cudaMemcpyDeviceToDevice, s), "copy grad u0");
    return 0;
}

int adsg_mass_loss(adsg_ctx* ctx, const double* u_dev, const double* target_dev, double* scratch_dev, double* loss_host,
                   double* grad_dev) {
    if (!ctx) return fail(-1, "ctx is NULL");
    if (!u_dev) return fail(-2, "u is NULL");
    if (!target_dev) return fail(-3, "target is NULL");
    if (!scratch_dev) return fail(-4, "scratch is NULL");
    if (!loss_host) return fail(-5, "loss is NULL");
    if (!grad_dev) return fail(-6, "grad is NULL");
    if (grad_dev == scratch_dev) return fail(-6, "grad must not alias scratch");
    const long long n = ctx->size;
    cudaStream_t s = ctx->stream;
    // scratch <- u - target ; grad <- M scratch (the factored mass operator, dt = 0)
    ADSG_CUDA_TRY(cudaMemcpyAsync(scratch_dev, u_dev, sizeof(double) * n, cudaMemcpyDeviceToDevice, s), "copy");
    ADSG_CUDA_TRY(launch_axpby(scratch_dev, -1.0, target_dev, 1.0, n, s), "difference");
    if (int st = ctx_rhs(ctx, scratch_dev, grad_dev, 0.0)) return st;
    if (!ctx->red) ADSG_CUDA_TRY(ctx->arena.alloc(&ctx->red, 1025), "reduction alloc");
    ADSG_CUDA_TRY(launch_dot(scratch_dev, grad_dev, n, ctx->red, ctx->red + 1024, s), "dot");
    ADSG_CUDA_TRY(cudaMemcpyAsync(loss_host, ctx->red + 1024, sizeof(double), cudaMemcpyDeviceToHost, s), "D2H");
    ADSG_CUDA_TRY(launch_axpby(grad_dev, 0.0, grad_dev, 2.0, n, s), "scale");
    ADSG_CUDA_TRY(cudaStreamSynchronize(s), "synchronize");
    return 0;
}

}  // extern "C"
