// Driver around the reference's OWN compiled code (built by oracle/Makefile
// from the reference sources where they lie; output only into oracle/_ref/).
// TEST INFRASTRUCTURE ONLY: it exists to pin the C restatement in
// ads_oracle.c and to generate the golden fixtures under tests/golden/.
//
// Exposes a small extern "C" surface so Python can load it with ctypes.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <iostream>
#include <memory>
#include <string>
#include <utility>
#include <vector>

#include <atomic>
#include <mutex>
#include <thread>

#include "ads/executor/sequential.hpp"
#include "ads/lin/band_solve.hpp"
#include "ads/simulation.hpp"

// Galois 6.0 is not installed, so executor/galois.hpp declares nothing here
// (its body is under ADS_USE_GALOIS).  This stand-in has the interface of
// galois_executor (executor/galois.hpp:19-46): for_each runs the function on
// every item of a range from a pool of threads, in no fixed order, and
// synchronized runs a function under one lock.  Written on std::thread and
// std::mutex; with one thread it visits the items in range order.
namespace ads {
class galois_executor {
    mutable std::mutex lock_;
    int threads_ = 1;

public:
    explicit galois_executor(int threads) { thread_count(threads); }
    void thread_count(int threads) { threads_ = threads < 1 ? 1 : threads; }

    template <typename Fun>
    void synchronized(Fun fun) const {
        std::lock_guard<std::mutex> guard{lock_};
        fun();
    }

    template <typename Range, typename Fun>
    void for_each(Range range, Fun&& fun) const {
        using std::begin;
        using std::end;
        using item = typename std::decay<decltype(*begin(range))>::type;
        std::vector<item> items;
        for (auto it = begin(range); it != end(range); ++it) items.push_back(*it);
        std::atomic<std::size_t> next{0};
        const std::size_t chunk = 16;
        auto work = [&] {
            for (;;) {
                std::size_t i = next.fetch_add(chunk);
                if (i >= items.size()) return;
                std::size_t stop = std::min(items.size(), i + chunk);
                for (; i < stop; ++i) fun(items[i]);
            }
        };
        std::vector<std::thread> pool;
        for (int t = 1; t < threads_; ++t) pool.emplace_back(work);
        work();
        for (auto& t : pool) t.join();
    }
};
}  // namespace ads

// The reference's examples/heat/heat_3d.hpp keeps compute_rhs private; open
// it up so the literal reference loop (eval_fun inside the dof loop) runs.
#define private public
#include "heat/heat_3d.hpp"
#undef private

// The reference's heat_2d (Dirichlet row at x = 0, heat_2d.hpp:40-52) and
// validation (Dirichlet on every side, exact solution, validation.hpp) examples
// write files through ads::output_manager, whose headers need boost::format;
// this stand-in of output_manager<2> (constructor and to_file, the interface
// those examples use) writes nothing, and its header is skipped.  Their
// galois_executor is the stand-in above; galois/Timer.h comes from refshim/.
#define ADS_OUTPUT_MANAGER_HPP
namespace ads {
template <std::size_t Dim>
struct output_manager;
template <>
struct output_manager<2> {
    template <typename... A>
    explicit output_manager(const A&...) { }
    template <typename... A>
    void to_file(const A&...) { }
};
}  // namespace ads
#define private public
#include "heat/heat_2d.hpp"
#include "validation/validation.hpp"
#undef private

// The reference's flow environment (random channel paths, mt19937-seeded) is
// header-only; its flow.hpp include is skipped (the flow class needs Galois).
#define FLOW_FLOW_HPP
#include "flow/environment.hpp"
#undef FLOW_FLOW_HPP

namespace {

// 3D heat step in the executor form of heat_2d.hpp:80-106 /
// scalability/test3d.hpp:66-95 (eval_fun hoisted, local element tile,
// synchronized scatter), driven by the reference's sequential_executor or by
// the galois_executor stand-in above on several threads.
template <typename Exec>
class heat3_driver_t : public ads::simulation_3d {
public:
    vector_type u, u_prev;
    Exec executor;

    template <typename... Args>
    explicit heat3_driver_t(const ads::config_3d& c, Args... exec_args)
    : simulation_3d{c}
    , u{shape()}
    , u_prev{shape()}
    , executor{exec_args...} { }

    void compute_rhs() {
        auto& rhs = u;
        zero(rhs);
        executor.for_each(elements(), [&](index_type e) {
            auto U = element_rhs();
            double J = jacobian(e);
            for (auto q : quad_points()) {
                double w = weight(q);
                value_type uu = eval_fun(u_prev, e, q);
                for (auto a : dofs_on_element(e)) {
                    auto aa = dof_global_to_local(e, a);
                    value_type v = eval_basis(e, q, a);
                    double gradient_prod = grad_dot(uu, v);
                    double val = uu.val * v.val - steps.dt * gradient_prod;
                    U(aa[0], aa[1], aa[2]) += val * w * J;
                }
            }
            executor.synchronized([&]() { update_global_rhs(rhs, U, e); });
        });
    }

    void prepare() { prepare_matrices(); }
    void do_solve(vector_type& v) { solve(v); }
    void step() {
        std::swap(u, u_prev);
        compute_rhs();
        solve(u);
    }
};

template <typename Exec>
class heat2_driver_t : public ads::simulation_2d {
public:
    vector_type u, u_prev;
    Exec executor;

    template <typename... Args>
    explicit heat2_driver_t(const ads::config_2d& c, Args... exec_args)
    : simulation_2d{c}
    , u{shape()}
    , u_prev{shape()}
    , executor{exec_args...} { }

    void compute_rhs() {
        auto& rhs = u;
        zero(rhs);
        executor.for_each(elements(), [&](index_type e) {
            auto U = element_rhs();
            double J = jacobian(e);
            for (auto q : quad_points()) {
                double w = weight(q);
                for (auto a : dofs_on_element(e)) {
                    auto aa = dof_global_to_local(e, a);
                    value_type v = eval_basis(e, q, a);
                    value_type uu = eval_fun(u_prev, e, q);
                    double gradient_prod = grad_dot(uu, v);
                    double val = uu.val * v.val - steps.dt * gradient_prod;
                    U(aa[0], aa[1]) += val * w * J;
                }
            }
            executor.synchronized([&]() { update_global_rhs(rhs, U, e); });
        });
    }

    void prepare() { prepare_matrices(); }
    void do_solve(vector_type& v) { solve(v); }
    template <typename F>
    void do_projection(vector_type& v, F f) {
        projection(v, f);
    }
    void step() {
        std::swap(u, u_prev);
        compute_rhs();
        solve(u);
    }
};

using heat3_driver = heat3_driver_t<ads::sequential_executor>;
using heat2_driver = heat2_driver_t<ads::sequential_executor>;

// scalability_3d::compute_rhs (examples/scalability/test3d.hpp:66-95) and
// flow::compute_rhs (examples/flow/flow.hpp:77-98), loop for loop, on the
// reference's own simulation_3d helpers with its sequential_executor in place
// of galois_executor; forcing terms as test3d.hpp:56-63 and flow.hpp:128-132.
class forms3_driver : public ads::simulation_3d {
public:
    vector_type u, u_prev;
    ads::sequential_executor executor;
    ads::problems::environment env{1};

    explicit forms3_driver(const ads::config_3d& c)
    : simulation_3d{c}
    , u{shape()}
    , u_prev{shape()} { }

    double scal_forcing(double x, double y, double z) const {
        double dx = x - 0.5, dy = y - 0.5, dz = z - 0.5;
        double r = std::sqrt(dx * dx + dy * dy + dz * dz);
        return std::exp(-r) + 1 + std::cos(M_PI * x) * std::cos(M_PI * y) * std::cos(M_PI * z);
    }

    void scalability_rhs() {
        auto& rhs = u;
        zero(rhs);
        executor.for_each(elements(), [&](index_type e) {
            auto U = element_rhs();
            double J = jacobian(e);
            for (auto q : quad_points()) {
                double w = weight(q);
                auto x = point(e, q);
                value_type uu = eval_fun(u_prev, e, q);
                for (auto a : dofs_on_element(e)) {
                    auto aa = dof_global_to_local(e, a);
                    value_type v = eval_basis(e, q, a);
                    double gradient_prod = grad_dot(uu, v);
                    double val = uu.val * v.val - steps.dt * (gradient_prod - scal_forcing(x[0], x[1], x[2]));
                    U(aa[0], aa[1], aa[2]) += val * w * J;
                }
            }
            executor.synchronized([&]() { update_global_rhs(rhs, U, e); });
        });
    }

    double flow_forcing(point_type x) const {
        double pi2 = 2 * M_PI;
        return 1 + std::sin(pi2 * x[0]) * std::sin(pi2 * x[1]) * std::sin(pi2 * x[2]);
    }

    // also returns k and u at every Gauss point (x-fastest over e_d q + k_d)
    void flow_rhs(double* kq, double* uq) {
        const long Qx = static_cast<long>(x.basis.elements) * x.basis.quad_order;
        const long Qy = static_cast<long>(y.basis.elements) * y.basis.quad_order;
        auto& rhs = u;
        zero(rhs);
        executor.for_each(elements(), [&](index_type e) {
            auto U = element_rhs();
            double J = jacobian(e);
            for (auto q : quad_points()) {
                double w = weight(q);
                auto x = point(e, q);
                double mi = 10;
                double k = env.permeability(x[0], x[1], x[2]);
                value_type uu = eval_fun(u_prev, e, q);
                double h = flow_forcing(x);
                const long pq = (static_cast<long>(e[0]) * this->x.basis.quad_order + q[0]) +
                                Qx * ((static_cast<long>(e[1]) * this->y.basis.quad_order + q[1]) +
                                      Qy * (static_cast<long>(e[2]) * this->z.basis.quad_order + q[2]));
                kq[pq] = k;
                uq[pq] = uu.val;
                for (auto a : dofs_on_element(e)) {
                    auto aa = dof_global_to_local(e, a);
                    value_type v = eval_basis(e, q, a);
                    double val = -k * std::exp(mi * uu.val) * grad_dot(uu, v) + h * v.val;
                    U(aa[0], aa[1], aa[2]) += (uu.val * v.val + steps.dt * val) * w * J;
                }
            }
            executor.synchronized([&] { update_global_rhs(rhs, U, e); });
        });
    }
};

template <typename T>
void load(T& t, const double* src) {
    std::copy(src, src + t.size(), t.data());
}

template <typename T>
void store(const T& t, double* dst) {
    std::copy(t.data(), t.data() + t.size(), dst);
}

}  // namespace

extern "C" {

// Per-dimension tables exactly as the reference builds them (dimension ctor,
// dimension.cpp:8-17) and the factorised matrix (dimension::factorize_matrix).
int ref_dim_tables(int p, int elements, double* btab, double* xq, double* w, double* J,
                   int* first_dofs, double* mass_ab, double* lu_ab, int* ipiv) {
    ads::dim_config cfg{p, elements};
    ads::dimension d{cfg, 1};
    const auto& bd = d.basis;
    int q = bd.quad_order;
    for (int e = 0; e < bd.elements; ++e) {
        for (int k = 0; k < q; ++k) {
            xq[e * q + k] = bd.x[e][k];
            for (int dd = 0; dd < 2; ++dd)
                for (int a = 0; a <= p; ++a) btab[((e * q + k) * 2 + dd) * (p + 1) + a] = bd.b[e][k][dd][a];
        }
        J[e] = bd.J[e];
        first_dofs[e] = bd.first_dof(e);
    }
    for (int k = 0; k < q; ++k) w[k] = bd.w[k];
    int ldab = d.M.column_size();
    int n = d.dofs();
    std::copy(d.M.full_buffer(), d.M.full_buffer() + ldab * n, mass_ab);
    d.factorize_matrix();
    std::copy(d.M.full_buffer(), d.M.full_buffer() + ldab * n, lu_ab);
    std::copy(d.ctx.pivot_vector.begin(), d.ctx.pivot_vector.end(), ipiv);
    return d.ctx.info;
}

// Stiffness matrix of the same basis (form_matrix.cpp:26-42).
int ref_stiffness(int p, int elements, double* ab) {
    ads::dim_config cfg{p, elements};
    ads::dimension d{cfg, 1};
    ads::lin::band_matrix K{p, p, d.dofs()};
    ads::stiffness_matrix_1d(K, d.basis);
    std::copy(K.full_buffer(), K.full_buffer() + K.column_size() * d.dofs(), ab);
    return 0;
}

// LAPACK band factorisation + solve through the reference's lin:: wrappers
// (band_solve.hpp:16-31). ab is a kl/ku band in the layout of band_matrix.
int ref_band_solve(int kl, int ku, int n, const double* ab_in, int nrhs, double* b, double* lu_out,
                   int* ipiv_out) {
    ads::lin::band_matrix M{kl, ku, n};
    std::copy(ab_in, ab_in + M.column_size() * n, M.full_buffer());
    ads::lin::solver_ctx ctx{M};
    ads::lin::factorize(M, ctx);
    if (ctx.info != 0) return ctx.info;
    ads::lin::solve_with_factorized(M, b, ctx, nrhs);
    if (lu_out) std::copy(M.full_buffer(), M.full_buffer() + M.column_size() * n, lu_out);
    if (ipiv_out) std::copy(ctx.pivot_vector.begin(), ctx.pivot_vector.end(), ipiv_out);
    return ctx.info;
}

// ads_solve (solver.hpp:222-226) on the factorised mass matrices of a
// uniform p / elements grid in ndim dimensions.
int ref_ads_solve(int ndim, int p, int elements, double* rhs) {
    ads::dim_config dim{p, elements};
    ads::timesteps_config steps{1, 0.0};
    if (ndim == 3) {
        heat3_driver s{ads::config_3d{dim, dim, dim, steps, 1}};
        s.prepare();
        load(s.u, rhs);
        s.do_solve(s.u);
        store(s.u, rhs);
    } else if (ndim == 2) {
        heat2_driver s{ads::config_2d{dim, dim, steps, 1}};
        s.prepare();
        load(s.u, rhs);
        s.do_solve(s.u);
        store(s.u, rhs);
    } else {
        return -1;
    }
    return 0;
}

// nsteps explicit heat steps from u (in/out). mode 0: executor form with the
// hoisted eval_fun; mode 1 (3D only): the literal heat_3d::compute_rhs.
int ref_heat_steps(int ndim, int p, int elements, double dt, int nsteps, double* u, int mode) {
    ads::dim_config dim{p, elements};
    ads::timesteps_config steps{nsteps, dt};
    if (ndim == 3) {
        ads::config_3d c{dim, dim, dim, steps, 1};
        if (mode == 1) {
            ads::problems::heat_3d s{c};
            s.prepare_matrices();
            load(s.u, u);
            for (int i = 0; i < nsteps; ++i) {
                s.before_step(i, i * dt);
                s.step(i, i * dt);
            }
            store(s.u, u);
        } else {
            heat3_driver s{c};
            s.prepare();
            load(s.u, u);
            for (int i = 0; i < nsteps; ++i) s.step();
            store(s.u, u);
        }
    } else if (ndim == 2) {
        heat2_driver s{ads::config_2d{dim, dim, steps, 1}};
        s.prepare();
        load(s.u, u);
        for (int i = 0; i < nsteps; ++i) s.step();
        store(s.u, u);
    } else {
        return -1;
    }
    return 0;
}

// nsteps explicit heat steps from u (in/out) in the executor form, with the
// element loop on nthreads threads of the galois_executor stand-in (the
// scatter order, and so the rounding, varies from run to run as under Galois).
int ref_heat_steps_mt(int ndim, int p, int elements, double dt, int nsteps, double* u, int nthreads) {
    ads::dim_config dim{p, elements};
    ads::timesteps_config steps{nsteps, dt};
    if (ndim == 3) {
        heat3_driver_t<ads::galois_executor> s{ads::config_3d{dim, dim, dim, steps, 1}, nthreads};
        s.prepare();
        load(s.u, u);
        for (int i = 0; i < nsteps; ++i) s.step();
        store(s.u, u);
    } else if (ndim == 2) {
        heat2_driver_t<ads::galois_executor> s{ads::config_2d{dim, dim, steps, 1}, nthreads};
        s.prepare();
        load(s.u, u);
        for (int i = 0; i < nsteps; ++i) s.step();
        store(s.u, u);
    } else {
        return -1;
    }
    return 0;
}

// normL2 / normH1 of a spline and errorL2 / errorH1 against
// f = prod_d sin(pi x_d) (with its gradient), and normL2 / normH1 of f itself,
// by basic_simulation_2d/3d's own quadrature loops
// (basic_simulation_3d.hpp:281-397): out = {normL2(u), normH1(u),
// errorL2(u, f), errorH1(u, f), normL2(f), normH1(f)}.
class norms3_driver : public ads::simulation_3d {
public:
    using simulation_3d::simulation_3d;
    void norms(const double* uin, double* out) {
        vector_type u{shape()};
        load(u, uin);
        auto f = [](point_type p) {
            const double sx = std::sin(M_PI * p[0]), sy = std::sin(M_PI * p[1]), sz = std::sin(M_PI * p[2]);
            const double cx = M_PI * std::cos(M_PI * p[0]), cy = M_PI * std::cos(M_PI * p[1]),
                         cz = M_PI * std::cos(M_PI * p[2]);
            return value_type{sx * sy * sz, cx * sy * sz, sx * cy * sz, sx * sy * cz};
        };
        out[0] = normL2(u, x, y, z);
        out[1] = normH1(u, x, y, z);
        out[2] = errorL2(u, x, y, z, f);
        out[3] = errorH1(u, x, y, z, f);
        out[4] = normL2(x, y, z, f);
        out[5] = normH1(x, y, z, f);
    }
    void step() { }
};

class norms2_driver : public ads::simulation_2d {
public:
    using simulation_2d::simulation_2d;
    void norms(const double* uin, double* out) {
        vector_type u{shape()};
        load(u, uin);
        auto f = [](point_type p) {
            const double sx = std::sin(M_PI * p[0]), sy = std::sin(M_PI * p[1]);
            return value_type{sx * sy, M_PI * std::cos(M_PI * p[0]) * sy, sx * M_PI * std::cos(M_PI * p[1])};
        };
        out[0] = normL2(u, x, y);
        out[1] = normH1(u, x, y);
        out[2] = errorL2(u, x, y, f);
        out[3] = errorH1(u, x, y, f);
        out[4] = normL2(x, y, f);
        out[5] = normH1(x, y, f);
    }
    void step() { }
};

int ref_norms(int ndim, int p, int elements, const double* u, double* out) {
    ads::dim_config dim{p, elements};
    ads::timesteps_config steps{1, 0.0};
    if (ndim == 3) {
        norms3_driver s{ads::config_3d{dim, dim, dim, steps, 1}};
        s.norms(u, out);
    } else if (ndim == 2) {
        norms2_driver s{ads::config_2d{dim, dim, steps, 1}};
        s.norms(u, out);
    } else {
        return -1;
    }
    return 0;
}

// examples/validation: the 2D heat problem with Dirichlet rows on all four
// sides (fix_left/fix_right in x and y, boundary rows of the right-hand side
// zeroed before every solve) from the projection of sin(pi x) sin(pi y),
// against its exact solution e^{-2 pi^2 t} sin(pi x) sin(pi y).  Runs the
// reference's own class: before(), then nsteps x (before_step, step); writes
// the state and errorL2(T), errorH1(T) in percent of the exact solution's
// norms (validation.hpp:121-129), T = nsteps dt.
int ref_validation(int p, int elements, double dt, int nsteps, double* u_out, double* err_out) {
    ads::dim_config dim{p, elements};
    ads::timesteps_config steps{nsteps, dt};
    ads::problems::validation s{ads::config_2d{dim, dim, steps, 1}};
    s.before();
    for (int i = 0; i < nsteps; ++i) {
        s.before_step(i, i * dt);
        s.step(i, i * dt);
    }
    store(s.u, u_out);
    err_out[0] = s.errorL2(nsteps * dt);
    err_out[1] = s.errorH1(nsteps * dt);
    return 0;
}

// examples/heat/heat_2d: x.fix_left(), and before every solve row x = 0 of
// the right-hand side replaced by the load vector of sin(pi y) on the y basis
// (heat_2d.hpp:40-52).  Runs the reference's own class from its before()
// state (the projection of init_state = 0, then that solve) through nsteps
// steps; writes the state and the load vector it imposes (ny values).
struct heat2d_open : ads::problems::heat_2d {
    using heat_2d::heat_2d;
    using simulation_2d::projection;
    const ads::dimension& ydim() const { return y; }
};

int ref_heat2d_dirichlet(int p, int elements, double dt, int nsteps, double* u_out, double* row_out) {
    ads::dim_config dim{p, elements};
    ads::timesteps_config steps{nsteps, dt};
    heat2d_open s{ads::config_2d{dim, dim, steps, 1}};
    s.prepare_matrices();
    s.projection(s.u, [&s](double x, double y) { return s.init_state(x, y); });
    s.solve(s.u);
    for (int i = 0; i < nsteps; ++i) {
        s.before_step(i, i * dt);
        s.step(i, i * dt);
    }
    store(s.u, u_out);
    const ads::dimension& y = s.ydim();
    ads::lin::vector buf{{y.dofs()}};
    ads::compute_projection(buf, y.basis, [](double t) { return std::sin(t * M_PI); });
    for (int i = 0; i < y.dofs(); ++i) row_out[i] = buf(i);
    return 0;
}

// One RHS evaluation (no solve) from u_prev into rhs, executor form.
int ref_heat_rhs(int ndim, int p, int elements, double dt, const double* u_prev, double* rhs) {
    ads::dim_config dim{p, elements};
    ads::timesteps_config steps{1, dt};
    if (ndim == 3) {
        heat3_driver s{ads::config_3d{dim, dim, dim, steps, 1}};
        load(s.u_prev, u_prev);
        s.compute_rhs();
        store(s.u, rhs);
    } else if (ndim == 2) {
        heat2_driver s{ads::config_2d{dim, dim, steps, 1}};
        load(s.u_prev, u_prev);
        s.compute_rhs();
        store(s.u, rhs);
    } else {
        return -1;
    }
    return 0;
}

// scalability_3d's RHS (which = 0) or flow's RHS (which = 1, also filling
// kq and uq, each of the Gauss-point count) from u_prev.
int ref_form_rhs(int which, int p, int elements, double dt, const double* u_prev, double* rhs, double* kq,
                 double* uq) {
    ads::dim_config dim{p, elements};
    ads::timesteps_config steps{1, dt};
    forms3_driver s{ads::config_3d{dim, dim, dim, steps, 1}};
    load(s.u_prev, u_prev);
    if (which == 0)
        s.scalability_rhs();
    else
        s.flow_rhs(kq, uq);
    store(s.u, rhs);
    return 0;
}

// compute_projection of prod_d sin(pi x_d) (projection.hpp:148-153), unsolved.
int ref_projection_sin(int ndim, int p, int elements, double* out) {
    ads::dim_config dim{p, elements};
    ads::timesteps_config steps{1, 0.0};
    if (ndim == 3) {
        heat3_driver s{ads::config_3d{dim, dim, dim, steps, 1}};
        s.projection(s.u, [](double x, double y, double z) {
            return std::sin(M_PI * x) * std::sin(M_PI * y) * std::sin(M_PI * z);
        });
        store(s.u, out);
    } else if (ndim == 2) {
        heat2_driver s{ads::config_2d{dim, dim, steps, 1}};
        s.do_projection(s.u, [](double x, double y) { return std::sin(M_PI * x) * std::sin(M_PI * y); });
        store(s.u, out);
    } else {
        return -1;
    }
    return 0;
}

}  // extern "C"
