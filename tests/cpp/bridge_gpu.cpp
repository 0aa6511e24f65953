// The C++ bridge (ads/gpu.hpp) on the GPU, driven through stand-ins of the
// reference's own types that carry exactly the members the bridge reads:
//   ads::basis_data        (include/ads/basis_data.hpp:21-86): degree,
//                          elements, dofs, quad_order, b[e][q][d][a] as
//                          double****, w as const double*, J as double*,
//                          first_dof(e);
//   ads::lin::band_matrix  (include/ads/lin/band_matrix.hpp:18-79): kl, ku,
//                          cols, column_size(), full_buffer();
//   ads::lin::solver_ctx   (include/ads/lin/solver_ctx.hpp:14-30): pivot_vector;
//   ads::dimension         (include/ads/simulation/dimension.hpp): basis, M
//                          (factorised), ctx.
// The tables come from the CPU oracle (its B-spline tables, mass band and
// dgbtrf factors are bit-identical to the reference's, pinned by the golden
// fixtures), and the bridge's compute_rhs_heat, solve and heat_steps are
// checked against the oracle's step.  Test code: prints "ok" when every
// check holds, the errors either way.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <memory>
#include <random>
#include <string>
#include <vector>

#include "ads/gpu.hpp"
#include "ads_oracle.h"

namespace standin {

struct basis_data {
    int degree = 0, elements = 0, dofs = 0, quad_order = 0;
    double**** b = nullptr;
    const double* w = nullptr;
    double* J = nullptr;
    std::vector<int> first_dofs;
    int first_dof(int e) const { return first_dofs[e]; }

    // storage behind the reference-shaped pointers
    std::vector<double> btab_, w_, J_;
    std::vector<double*> lvl3_;
    std::vector<double**> lvl2_;
    std::vector<double***> lvl1_;
};

struct band_matrix {
    int kl = 0, ku = 0, rows = 0, cols = 0, row_offset = 0;
    std::vector<double> data_;
    int column_size() const { return row_offset + ku + 1 + kl; }
    const double* full_buffer() const { return data_.data(); }
};

struct solver_ctx {
    std::vector<int> pivot_vector;
};

struct dimension {
    basis_data basis;
    band_matrix M;
    solver_ctx ctx;
};

// Dimension d of an oracle problem, in the reference's shapes.
std::unique_ptr<dimension> from_oracle(const orc_problem* pr, int d, int p, int elements) {
    auto dim = std::make_unique<dimension>();
    basis_data& B = dim->basis;
    const int q = p + 1, n = elements + p, ldab = 3 * p + 1;
    B.degree = p;
    B.elements = elements;
    B.dofs = n;
    B.quad_order = q;
    B.btab_.resize(static_cast<size_t>(elements) * q * 2 * (p + 1));
    B.w_.resize(q);
    B.J_.resize(elements);
    B.first_dofs.resize(elements);
    dim->M.data_.resize(static_cast<size_t>(ldab) * n);
    dim->ctx.pivot_vector.resize(n);
    orc_problem_dim(pr, d, B.btab_.data(), B.w_.data(), B.J_.data(), B.first_dofs.data(), nullptr,
                    dim->M.data_.data(), dim->ctx.pivot_vector.data());
    // b[e][q][k] points at the p+1 values of basis_data's layout
    B.lvl3_.resize(static_cast<size_t>(elements) * q * 2);
    B.lvl2_.resize(static_cast<size_t>(elements) * q);
    B.lvl1_.resize(elements);
    for (size_t i = 0; i < B.lvl3_.size(); ++i) B.lvl3_[i] = B.btab_.data() + i * (p + 1);
    for (size_t i = 0; i < B.lvl2_.size(); ++i) B.lvl2_[i] = B.lvl3_.data() + i * 2;
    for (int e = 0; e < elements; ++e) B.lvl1_[e] = B.lvl2_.data() + static_cast<size_t>(e) * q;
    B.b = B.lvl1_.data();
    B.w = B.w_.data();
    B.J = B.J_.data();
    dim->M.kl = p;
    dim->M.ku = p;
    dim->M.rows = n;
    dim->M.cols = n;
    dim->M.row_offset = p;
    return dim;
}

}  // namespace standin

// stand-in for lin::tensor: data() and size()
struct tensor {
    std::vector<double> v;
    double* data() { return v.data(); }
    const double* data() const { return v.data(); }
    long long size() const { return static_cast<long long>(v.size()); }
};

static double rel_l2(const std::vector<double>& a, const std::vector<double>& b) {
    double s = 0;
    for (size_t i = 0; i < a.size(); ++i) s = std::fmax(s, std::fmax(std::fabs(a[i]), std::fabs(b[i])));
    if (s == 0) return 0;
    double num = 0, den = 0;
    for (size_t i = 0; i < a.size(); ++i) {
        num += (a[i] - b[i]) / s * ((a[i] - b[i]) / s);
        den += a[i] / s * (a[i] / s);
    }
    return std::sqrt(num / den);
}

static bool report(const char* what, double err, double bound) {
    std::printf("%s: rel L2 %.3e (bound %.1e)\n", what, err, bound);
    return err <= bound;
}

template <typename... Dims>
static bool run_case(const char* name, const orc_problem* pr, double dt, int nsteps, const Dims&... dims) {
    const long long size = orc_problem_size(pr);
    std::mt19937_64 gen(42);
    std::uniform_real_distribution<double> U(-1.0, 1.0);
    tensor u0{std::vector<double>(size)};
    for (auto& x : u0.v) x = U(gen);

    ads::gpu::context gpu{dims...};
    bool ok = true;
    char label[128];

    tensor rhs{std::vector<double>(size)};
    gpu.compute_rhs_heat(u0, rhs, dt);
    std::vector<double> ref(size);
    orc_heat_rhs(pr, u0.data(), ref.data(), dt);
    std::snprintf(label, sizeof label, "%s compute_rhs_heat", name);
    ok &= report(label, rel_l2(rhs.v, ref), 1e-13);

    tensor x = u0;
    gpu.solve(x);
    ref = u0.v;
    orc_ads_solve(pr, ref.data());
    std::snprintf(label, sizeof label, "%s solve", name);
    ok &= report(label, rel_l2(x.v, ref), 1e-13);

    tensor s = u0;
    gpu.heat_steps(s, dt, nsteps);
    ref = u0.v;
    orc_heat_steps(pr, ref.data(), dt, nsteps, 1);
    std::snprintf(label, sizeof label, "%s %d heat steps", name, nsteps);
    ok &= report(label, rel_l2(s.v, ref), 1e-12 * nsteps);
    return ok;
}

// The reverse-mode class on device buffers: the dot-product identity of the
// linear map u0 -> u(T) and central differences of the mass-norm loss along a
// seeded direction in u0 (the loss is quadratic in u0, so the difference is
// exact up to rounding).
template <typename... Dims>
static bool run_adjoint(const char* name, const Dims&... dims) {
    ads::gpu::context gpu{dims...};
    const long long n = gpu.size();
    const size_t bytes = sizeof(double) * static_cast<size_t>(n);
    std::mt19937_64 gen(7);
    std::uniform_real_distribution<double> U(-1.0, 1.0);
    auto host = [&](double lo, double scale) {
        std::vector<double> v(n);
        for (auto& x : v) x = lo + scale * U(gen);
        return v;
    };
    const std::vector<double> u0 = host(0.0, 1.0), kap = host(1.0, 0.3), tgt = host(0.0, 1.0), x = host(0.0, 1.0),
                              y = host(0.0, 1.0), d = host(0.0, 1.0);
    double* buf[10];
    for (auto& b : buf)
        if (cudaMalloc(&b, bytes) != cudaSuccess) return false;
    double *du0 = buf[0], *dk = buf[1], *dt_ = buf[2], *uT = buf[3], *gu = buf[4], *gk = buf[5], *sc = buf[6],
           *dL = buf[7], *dx = buf[8], *dy = buf[9];
    cudaMemcpy(du0, u0.data(), bytes, cudaMemcpyHostToDevice);
    cudaMemcpy(dk, kap.data(), bytes, cudaMemcpyHostToDevice);
    cudaMemcpy(dt_, tgt.data(), bytes, cudaMemcpyHostToDevice);
    cudaMemcpy(dx, x.data(), bytes, cudaMemcpyHostToDevice);
    cudaMemcpy(dy, y.data(), bytes, cudaMemcpyHostToDevice);
    ads::gpu::adjoint adj(gpu, 4, 1e-5);
    auto dot = [&](const double* a, const std::vector<double>& b) {
        std::vector<double> h(n);
        cudaMemcpy(h.data(), a, bytes, cudaMemcpyDeviceToHost);
        double s = 0;
        for (long long i = 0; i < n; ++i) s += h[i] * b[i];
        return s;
    };
    // <A x, y> against <x, A^T y>
    adj.forward(dx, dk, uT);
    const double lhs = dot(uT, y);
    adj.backward(dy, gu, gk);
    const double rhs = dot(gu, x);
    bool ok = report((std::string(name) + " adjoint dot-product identity").c_str(),
                     std::fabs(lhs - rhs) / std::fmax(std::fabs(lhs), std::fabs(rhs)), 1e-12);
    // dL/du0 . d against central differences of the loss
    adj.forward(du0, dk, uT);
    gpu.mass_loss_dev(uT, dt_, sc, dL);
    adj.backward(dL, gu, gk);
    const double an = dot(gu, d);
    const double h = 1e-4;
    auto loss_at = [&](double s) {
        std::vector<double> v(u0);
        for (long long i = 0; i < n; ++i) v[i] += s * d[i];
        cudaMemcpy(dx, v.data(), bytes, cudaMemcpyHostToDevice);
        adj.forward(dx, dk, uT);
        return gpu.mass_loss_dev(uT, dt_, sc, dL);
    };
    const double num = (loss_at(h) - loss_at(-h)) / (2 * h);
    ok &= report((std::string(name) + " adjoint dL/du0 against central differences").c_str(),
                 std::fabs(num - an) / std::fmax(std::fabs(num), std::fabs(an)), 1e-7);
    const auto ck = adj.checkpoints();
    ok &= ck.first == 2 && ck.second == 2;  // ceil(sqrt(4)) steps apart, 2 kept
    for (auto b : buf) cudaFree(b);
    return ok;
}

int main() {
    bool ok = true;
    {
        const int p[3] = {2, 2, 2}, E[3] = {20, 16, 12};
        orc_problem* pr = orc_problem_create(3, p, E);
        auto x = standin::from_oracle(pr, 0, p[0], E[0]);
        auto y = standin::from_oracle(pr, 1, p[1], E[1]);
        auto z = standin::from_oracle(pr, 2, p[2], E[2]);
        ok &= run_case("3D p=2 20x16x12", pr, 1e-5, 4, *x, *y, *z);
        ok &= run_adjoint("3D p=2 20x16x12", *x, *y, *z);
        orc_problem_destroy(pr);
    }
    {
        const int p[2] = {3, 2}, E[2] = {30, 25};
        orc_problem* pr = orc_problem_create(2, p, E);
        auto x = standin::from_oracle(pr, 0, p[0], E[0]);
        auto y = standin::from_oracle(pr, 1, p[1], E[1]);
        ok &= run_case("2D p=3,2 30x25", pr, 1e-5, 3, *x, *y);
        orc_problem_destroy(pr);
    }
    std::printf("%s\n", ok ? "ok" : "FAILED");
    return ok ? 0 : 1;
}
