// ads/gpu.hpp -- header-only C++ bridge from the reference's types to the
// GB300 engine (include/ads_gb300.h).
//
// A C++ program written against marcinlos/iga-ads keeps its ads::dimension
// objects (src/ads/simulation/dimension.cpp) and swaps the two hot calls:
//
//     ads::gpu::context gpu{x, y, z};             // once, after prepare_matrices()
//     gpu.compute_rhs_heat(u_prev, u, steps.dt);  // instead of heat_3d::compute_rhs
//     gpu.solve(u);                               // instead of ads_solve(u, buffer, x, y, z)
//
// where u / u_prev are ads::lin::tensor objects (anything with data() and
// size()).  The bridge is duck-typed: a Dimension needs `basis` (basis_data:
// elements, quad_order, degree, dofs, b[e][q][d][a], w, J, first_dof(e)), `M`
// (the factorised lin::band_matrix: kl, ku, cols, column_size(),
// full_buffer()) and `ctx` (lin::solver_ctx: pivot_vector), which is what the
// reference's ads::dimension has after factorize_matrix().
//
// The heavy data stays on the GPU between calls; the host-tensor overloads
// copy in and out (adsg_*_host).  Device-pointer overloads are available for
// callers that keep their state in HBM.
#ifndef ADS_GPU_HPP
#define ADS_GPU_HPP

#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../../../include/ads_gb300.h"

namespace ads::gpu {

inline void check(int code) {
    if (code != 0) throw std::runtime_error("ads_gb300: " + std::to_string(code) + ": " + adsg_last_error());
}

// Flattened copy of one dimension's tables (basis_data keeps b as nested
// pointers; the C-ABI takes contiguous arrays).
struct flat_dim {
    std::vector<double> btab, w, J, lu;
    std::vector<int> first, ipiv;
    int p = 0, elements = 0, quad_order = 0, n = 0, kl = 0, ku = 0, ldab = 0;

    template <typename Dimension>
    explicit flat_dim(const Dimension& d) {
        const auto& B = d.basis;
        elements = B.elements;
        quad_order = B.quad_order;
        p = B.degree;
        n = B.dofs;
        btab.resize(static_cast<size_t>(elements) * quad_order * 2 * (p + 1));
        for (int e = 0; e < elements; ++e)
            for (int q = 0; q < quad_order; ++q)
                for (int k = 0; k < 2; ++k)
                    for (int a = 0; a <= p; ++a)
                        btab[((static_cast<size_t>(e) * quad_order + q) * 2 + k) * (p + 1) + a] = B.b[e][q][k][a];
        w.assign(B.w, B.w + quad_order);
        J.assign(B.J, B.J + elements);
        first.resize(elements);
        for (int e = 0; e < elements; ++e) first[e] = B.first_dof(e);
        const auto& M = d.M;
        ldab = M.column_size();
        kl = M.kl;
        ku = M.ku;
        lu.assign(M.full_buffer(), M.full_buffer() + static_cast<size_t>(ldab) * M.cols);
        ipiv = d.ctx.pivot_vector;
    }

    // Descriptor pointing into this object's arrays (valid while it lives).
    adsg_dim_desc desc() const {
        adsg_dim_desc d{};
        d.p = p;
        d.elements = elements;
        d.quad_order = quad_order;
        d.n = n;
        d.btab = btab.data();
        d.w = w.data();
        d.J = J.data();
        d.first_dofs = first.data();
        d.kl = kl;
        d.ku = ku;
        d.ldab = ldab;
        d.lu = lu.data();
        d.ipiv = ipiv.data();
        return d;
    }
};

class context {
public:
    template <typename... Dims>
    explicit context(const Dims&... dims) {
        std::vector<flat_dim> flat;
        (flat.emplace_back(dims), ...);
        std::vector<adsg_dim_desc> descs;
        for (const auto& f : flat) descs.push_back(f.desc());
        check(adsg_ctx_create(static_cast<int>(descs.size()), descs.data(), &ctx_));
    }
    explicit context(const std::vector<adsg_dim_desc>& descs) {
        check(adsg_ctx_create(static_cast<int>(descs.size()), descs.data(), &ctx_));
    }
    context(const context&) = delete;
    context& operator=(const context&) = delete;
    ~context() { adsg_ctx_destroy(ctx_); }

    long long size() const { return adsg_ctx_size(ctx_); }
    adsg_ctx* handle() { return ctx_; }

    // host tensors (reference lin::tensor or anything with data()/size())
    template <typename Tensor>
    void compute_rhs_heat(const Tensor& u_prev, Tensor& rhs, double dt) {
        require(u_prev.size());
        require(rhs.size());
        check(adsg_heat_rhs_host(ctx_, u_prev.data(), rhs.data(), dt));
    }
    template <typename Tensor>
    void solve(Tensor& rhs) {
        require(rhs.size());
        check(adsg_ads_solve_host(ctx_, rhs.data()));
    }
    template <typename Tensor>
    void heat_steps(Tensor& u, double dt, int nsteps) {
        require(u.size());
        check(adsg_heat_steps_host(ctx_, u.data(), dt, nsteps));
    }

    // device buffers
    void compute_rhs_heat_dev(const double* u_prev, double* rhs, double dt) { check(adsg_heat_rhs(ctx_, u_prev, rhs, dt)); }
    void solve_dev(double* rhs) { check(adsg_ads_solve(ctx_, rhs, nullptr)); }
    void heat_step_dev(const double* u_prev, double* u_next, double dt) {
        check(adsg_heat_step(ctx_, u_prev, u_next, dt));
    }
    void heat_steps_dev(double* u, double dt, int nsteps) { check(adsg_heat_steps(ctx_, u, dt, nsteps)); }
    // the element-wise RHS with a diffusion field kappa (spline coefficients;
    // nullptr: kappa = 1), and with kappa evaluated once at the Gauss points
    // (3D; kappa_points_count() doubles) for many right-hand sides
    void compute_rhs_kappa_dev(const double* u_prev, const double* kappa, double* rhs, double dt) {
        check(adsg_heat_rhs_elem(ctx_, u_prev, kappa, rhs, dt));
    }
    long long kappa_points_count() const { return adsg_kappa_points_count(ctx_); }
    void kappa_points_dev(const double* kappa, double* kq) { check(adsg_kappa_points(ctx_, kappa, kq)); }
    void compute_rhs_kappa_points_dev(const double* u_prev, const double* kq, double* rhs, double dt) {
        check(adsg_heat_rhs_elem_points(ctx_, u_prev, kq, rhs, dt));
    }
    // L = (u - target)^T M (u - target) and dL/du = 2 M (u - target)
    double mass_loss_dev(const double* u, const double* target, double* scratch, double* grad) {
        double loss = 0.0;
        check(adsg_mass_loss(ctx_, u, target, scratch, &loss, grad));
        return loss;
    }
    void synchronize() { check(adsg_ctx_synchronize(ctx_)); }

private:
    void require(long long n) const {
        if (n != adsg_ctx_size(ctx_)) throw std::invalid_argument("ads::gpu: tensor size does not match the context");
    }
    adsg_ctx* ctx_ = nullptr;
};

// Reverse mode of the kappa-weighted explicit run u_{k+1} = M^-1 R(kappa) u_k
// (adsg_adjoint_*): the C++ counterpart of a torch.autograd.Function.
// forward() runs nsteps from u0 keeping checkpoints (every ceil(sqrt(nsteps))
// steps unless checkpoint_every says otherwise; 1 keeps every state) and
// returns u(T); backward() takes dL/du(T) and returns dL/du0 and dL/dkappa.
// Device buffers of the context's size.
class adjoint {
public:
    adjoint(context& ctx, int nsteps, double dt, int checkpoint_every = 0) {
        check(adsg_adjoint_create(ctx.handle(), nsteps, dt, checkpoint_every, &a_));
    }
    adjoint(const adjoint&) = delete;
    adjoint& operator=(const adjoint&) = delete;
    ~adjoint() { adsg_adjoint_destroy(a_); }

    void forward(const double* u0, const double* kappa, double* uT) { check(adsg_adjoint_forward(a_, u0, kappa, uT)); }
    void backward(const double* dL_duT, double* grad_u0, double* grad_kappa) {
        check(adsg_adjoint_backward(a_, dL_duT, grad_u0, grad_kappa));
    }
    // (steps between checkpoints, checkpoints kept)
    std::pair<int, int> checkpoints() const {
        int every = 0, count = 0;
        check(adsg_adjoint_checkpoints(a_, &every, &count));
        return {every, count};
    }

private:
    adsg_adjoint* a_ = nullptr;
};

// ads_solve(rhs, buf, dims...) of the reference with a GPU context in place
// of the dim_data pack: the solution is left in rhs (buf is not needed).
template <typename Tensor>
void ads_solve(context& gpu, Tensor& rhs) {
    gpu.solve(rhs);
}

}  // namespace ads::gpu

#endif  // ADS_GPU_HPP
