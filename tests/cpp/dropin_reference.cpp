// Drop-in check against the reference's OWN classes: an ads::simulation_3d
// heat problem (examples/heat/heat_3d.hpp's form) whose step runs through
// ads/gpu.hpp.  Built by oracle/Makefile (target dropin) where the reference
// sources are present.  Without a GPU the context cannot be created and the
// program reports "no-gpu"; with one it compares a GPU step with the
// reference's own CPU step and prints the relative difference.
#include <cmath>
#include <cstdio>
#include <exception>
#include <vector>

#include "ads/gpu.hpp"
#include "ads/simulation.hpp"

namespace {

class heat_cpu : public ads::simulation_3d {
public:
    vector_type u, u_prev;
    explicit heat_cpu(const ads::config_3d& c)
    : simulation_3d{c}
    , u{shape()}
    , u_prev{shape()} { }

    void prepare() { prepare_matrices(); }

    // heat_3d::compute_rhs with eval_fun hoisted (identical arithmetic)
    void compute_rhs() {
        auto& rhs = u;
        zero(rhs);
        for (auto e : elements()) {
            double J = jacobian(e);
            for (auto q : quad_points()) {
                double w = weight(q);
                value_type uu = eval_fun(u_prev, e, q);
                for (auto a : dofs_on_element(e)) {
                    value_type v = eval_basis(e, q, a);
                    double val = uu.val * v.val - steps.dt * grad_dot(uu, v);
                    rhs(a[0], a[1], a[2]) += val * w * J;
                }
            }
        }
    }
    void step() {
        std::swap(u, u_prev);
        compute_rhs();
        solve(u);
    }
};

}  // namespace

int main() {
    ads::dim_config dim{2, 8};
    ads::timesteps_config steps{1, 1e-4};
    ads::config_3d c{dim, dim, dim, steps, 1};
    heat_cpu cpu{c};
    cpu.prepare();
    for (int i = 0; i < cpu.u.size(); ++i) cpu.u.data()[i] = std::sin(0.37 * i) + 0.1 * std::cos(1.3 * i);
    auto gpu_state = cpu.u;  // the same initial tensor (lin::tensor)
    try {
        ads::gpu::context gpu{cpu.x, cpu.y, cpu.z};  // the reference's own ads::dimension objects
        auto prev = gpu_state;
        gpu.compute_rhs_heat(prev, gpu_state, steps.dt);
        ads::gpu::ads_solve(gpu, gpu_state);
    } catch (const std::exception& ex) {
        std::printf("no-gpu: %s\n", ex.what());
        return 0;
    }
    cpu.step();
    double num = 0, den = 0;
    for (int i = 0; i < cpu.u.size(); ++i) {
        double d = cpu.u.data()[i] - gpu_state.data()[i];
        num += d * d;
        den += cpu.u.data()[i] * cpu.u.data()[i];
    }
    std::printf("ok rel_l2=%.3e\n", std::sqrt(num / den));
    return std::sqrt(num / den) < 1e-12 ? 0 : 1;
}
