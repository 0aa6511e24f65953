// Standalone C++ host program over the C-ABI and ads/gpu.hpp (no reference
// sources needed): the 3D known-answer ADS system of the reference test
// tests/ads/solver_test.cpp:164-255 (tridiagonal Mx, My, Mz; solution 1..24),
// and one heat step through the context.  Prints "ok" and exits 0 on success.
#include <cmath>
#include <cstdio>
#include <vector>

#include "ads/gpu.hpp"

namespace {

// LAPACK band layout kl = ku = 1, ldab = 4, filled row by row from the first
// in-band column (the reference test's make_matrix)
std::vector<double> band(int n, const std::vector<std::vector<double>>& rows) {
    std::vector<double> ab(4 * n, 0.0);
    for (int i = 0; i < n; ++i) {
        int j = i > 0 ? i - 1 : 0;
        for (double v : rows[i]) {
            ab[j * 4 + 2 + i - j] = v;
            ++j;
        }
    }
    return ab;
}

// no-pivot LU is what dgbtrf produces for these diagonally placed systems?
// Not in general: factorise with the engine's own host code via adsg_dgbtrs_-
// compatible layout is unavailable, so the factors are computed here with
// partial pivoting (a small dgbtf2).
void factor(int n, std::vector<double>& ab, std::vector<int>& ipiv) {
    const int kl = 1, ku = 1, kv = 2, ldab = 4;
    auto A = [&](int r, int c) -> double& { return ab[c * ldab + r]; };
    ipiv.assign(n, 0);
    int reach = 0;
    for (int j = 0; j < n; ++j) {
        if (j + kv < n) A(0, j + kv) = 0;
        const int km = std::min(kl, n - 1 - j);
        int jp = 0;
        double big = std::fabs(A(kv, j));
        for (int i = 1; i <= km; ++i)
            if (std::fabs(A(kv + i, j)) > big) {
                big = std::fabs(A(kv + i, j));
                jp = i;
            }
        ipiv[j] = j + jp + 1;
        reach = std::max(reach, std::min(j + ku + jp, n - 1));
        if (jp)
            for (int c = 0; c <= reach - j; ++c) std::swap(A(kv + jp - c, j + c), A(kv - c, j + c));
        if (km > 0) {
            const double inv = 1.0 / A(kv, j);
            for (int i = 1; i <= km; ++i) A(kv + i, j) *= inv;
            for (int c = 1; c <= reach - j; ++c) {
                const double y = A(kv - c, j + c);
                for (int i = 1; i <= km; ++i) A(kv + i - c, j + c) -= A(kv + i, j) * y;
            }
        }
    }
}

adsg_dim_desc desc(int n, std::vector<double>& lu, std::vector<int>& ipiv, std::vector<double>& btab,
                   std::vector<double>& w, std::vector<double>& J, std::vector<int>& first) {
    const int E = n - 1;
    btab.assign(E * 2 * 2 * 2, 0.5);
    w.assign(2, 1.0);
    J.assign(E, 0.5);
    first.resize(E);
    for (int e = 0; e < E; ++e) first[e] = e;
    adsg_dim_desc d{};
    d.p = 1;
    d.elements = E;
    d.quad_order = 2;
    d.n = n;
    d.btab = btab.data();
    d.w = w.data();
    d.J = J.data();
    d.first_dofs = first.data();
    d.kl = 1;
    d.ku = 1;
    d.ldab = 4;
    d.lu = lu.data();
    d.ipiv = ipiv.data();
    return d;
}

}  // namespace

int main() {
    std::vector<double> mx = band(4, {{1, 2}, {2, 3, 1}, {-1, 4}, {1, 3}});
    std::vector<double> my = band(3, {{2, 3}, {1, 2, -3}, {2, 2}});
    std::vector<double> mz = band(2, {{1, 2}, {3, 4}});
    std::vector<int> px, py, pz;
    factor(4, mx, px);
    factor(3, my, py);
    factor(2, mz, pz);
    std::vector<double> b1, w1, j1, b2, w2, j2, b3, w3, j3;
    std::vector<int> f1, f2, f3;
    std::vector<adsg_dim_desc> d = {desc(4, mx, px, b1, w1, j1, f1), desc(3, my, py, b2, w2, j2, f2),
                                    desc(2, mz, pz, b3, w3, j3, f3)};
    std::vector<double> rhs = {543, 1101, 618, 849, -144, -288, -144, -192, 564, 1140, 624, 852,
                               1147, 2329, 1322, 1821, -336, -672, -336, -448, 1220, 2468, 1360, 1860};
    try {
        ads::gpu::context gpu{d};
        gpu.solve(rhs);
    } catch (const std::exception& ex) {
        std::printf("failed: %s\n", ex.what());
        return 2;
    }
    for (int i = 0; i < 24; ++i)
        if (std::fabs(rhs[i] - (i + 1)) > 1e-12 * (i + 1)) {
            std::printf("mismatch at %d: %.17g\n", i, rhs[i]);
            return 1;
        }
    // a heat step on a p = 2 grid through engine-built dimensions
    adsg_dim* dims[3];
    std::vector<adsg_dim_desc> hd(3);
    for (int k = 0; k < 3; ++k) {
        ads::gpu::check(adsg_dim_create(2, 6, 0.0, 1.0, 0, &dims[k]));
        ads::gpu::check(adsg_dim_describe(dims[k], &hd[k]));
    }
    ads::gpu::context heat{hd};
    std::vector<double> u(heat.size(), 1.0);
    heat.heat_steps(u, 1e-4, 3);  // the constant field stays (nearly) constant under diffusion
    double dev = 0;
    for (double v : u) dev = std::max(dev, std::fabs(v - 1.0));
    for (auto* p : dims) adsg_dim_destroy(p);
    if (dev > 1e-12) {
        std::printf("heat: constant field drifted by %.3e\n", dev);
        return 1;
    }
    std::printf("ok\n");
    return 0;
}
