// Host-side tables of one direction, built once per context: row-format
// bands, the symmetric row range of the pair-sum passes, the LAPACK-order
// solve tables from dgbtrf factors, and the two-ended (twisted) factorisation
// with its row-scaled form.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "adsg_internal.hpp"

namespace adsg {

// Row-format band (n rows x (2p+1)) of sum_e sum_q B_a B_b w_q J_e with the
// basis values (which = 0) or derivatives (which = 1) of a descriptor.
std::vector<double> row_band(const adsg_dim_desc& d, int which) {
    const int p = d.p, bw = 2 * p + 1;
    std::vector<double> rows(static_cast<size_t>(d.n) * bw, 0.0);
    for (int e = 0; e < d.elements; ++e) {
        const int f = d.first_dofs[e];
        for (int k = 0; k < d.quad_order; ++k) {
            const double* v = d.btab + ((static_cast<size_t>(e) * d.quad_order + k) * 2 + which) * (p + 1);
            for (int a = 0; a <= p; ++a)
                for (int b = 0; b <= p; ++b) rows[static_cast<size_t>(f + a) * bw + (b - a + p)] += v[a] * v[b] * d.w[k] * d.J[e];
        }
    }
    return rows;
}

// The widest range [lo, hi) of rows that are symmetric in both row-format
// bands (coefficients of columns r-t and r+t equal to 1e-13 of the row's
// size), grown from the middle row: with uniform open knots every row 2p-1 or
// more away from the ends is a translate of one symmetric row, up to the
// rounding of its quadrature (measured 14-220 ulp of the row's largest
// entry, <= 5e-14 relative, on grids of 32-512 elements, p = 2..4).  The
// pair-sum passes use the left coefficient of each pair on these rows, which
// moves the operator by that relative amount; lo = hi when the middle row
// itself is not symmetric.
void symmetric_row_range(const std::vector<double>& m, const std::vector<double>& k, int n, int p, int& lo, int& hi) {
    const int bw = 2 * p + 1;
    auto sym = [&](int r) {
        for (const std::vector<double>* rows : {&m, &k}) {
            const double* row = rows->data() + static_cast<size_t>(r) * bw;
            double mx = 0.0;
            for (int t = 0; t < bw; ++t) mx = std::max(mx, std::fabs(row[t]));
            for (int t = 1; t <= p; ++t)
                if (!(std::fabs(row[p - t] - row[p + t]) <= 1e-13 * mx)) return false;
        }
        return true;
    };
    lo = hi = n / 2;
    if (n < 2 * p + 1 || !sym(n / 2)) return;
    while (lo > p && sym(lo - 1)) --lo;
    hi = n / 2 + 1;
    while (hi < n - p && sym(hi)) ++hi;
}

bool valid_desc(const adsg_dim_desc& d) {
    if (d.p < 1 || d.p > ADSG_MAX_DEGREE || d.elements < 1 || d.quad_order < 1 || d.n < 1) return false;
    if (!d.btab || !d.w || !d.J || !d.first_dofs || !d.lu || !d.ipiv) return false;
    if (d.kl < 0 || d.ku < 0 || d.ldab < 2 * d.kl + d.ku + 1) return false;
    if (d.kl > 16 || d.kl + d.ku > 32) return false;
    for (int e = 0; e < d.elements; ++e)
        if (d.first_dofs[e] < 0 || d.first_dofs[e] + d.p >= d.n) return false;
    for (int j = 0; j < d.n; ++j)
        if (d.ipiv[j] < j + 1 || d.ipiv[j] > std::min(d.n, j + 1 + d.kl)) return false;
    return true;
}

// Solve tables extracted from a dgbtrf band.

int make_solve_tables(int n, int kl, int ku, int ldab, const double* ab, const int* ipiv, solve_tables& t) {
    const int kv = kl + ku;
    t.kl = std::max(kl, 1);
    t.w = std::max(kv, 1);
    t.lmul.assign(static_cast<size_t>(n + 16) * t.kl, 0.0);  // padded for block-wise prefetch
    t.ucol.assign(static_cast<size_t>(n) * t.w, 0.0);
    t.rdiag.assign(n, 0.0);
    t.piv.assign(n, 0);
    t.uext.assign(n, 0);
    for (int j = 0; j < n; ++j) {
        const double* col = ab + static_cast<size_t>(j) * ldab;
        const double diag = col[kv];
        if (diag == 0.0) return j + 1;
        t.rdiag[j] = 1.0 / diag;
        t.piv[j] = ipiv[j] - 1;
        for (int i = 1; i <= kl && j + i < n; ++i) t.lmul[static_cast<size_t>(j) * t.kl + i - 1] = col[kv + i];
        int ext = 0;
        for (int d = 1; d <= kv && d <= j; ++d) {
            const double u = col[kv - d];
            t.ucol[static_cast<size_t>(j) * t.w + d - 1] = u;
            if (u != 0.0) ext = d;
        }
        t.uext[j] = ext;
    }
    // columns from which the sweeps need no exchange / no extra U terms
    t.fwd_fast = 0;
    for (int j = 0; j < n; ++j)
        if (t.piv[j] != j) t.fwd_fast = j + 1;
    t.bwd_fast = 0;
    for (int j = 0; j < n; ++j)
        if (t.uext[j] > ku) t.bwd_fast = j + 1;
    return 0;
}

namespace {

// LAPACK dgbtrs order ('N') on one right-hand side, for the twisted self-check.
void host_band_solve(int n, int kl, int ku, int ldab, const double* ab, const int* ipiv, double* b) {
    const int kv = kl + ku;
    for (int j = 0; j + 1 < n; ++j) {
        const int p = ipiv[j] - 1;
        if (p != j) std::swap(b[p], b[j]);
        for (int i = 1; i <= kl && j + i < n; ++i) b[j + i] -= ab[static_cast<size_t>(j) * ldab + kv + i] * b[j];
    }
    for (int j = n - 1; j >= 0; --j) {
        const double* col = ab + static_cast<size_t>(j) * ldab;
        b[j] /= col[kv];
        for (int d = 1; d <= kv && d <= j; ++d) b[j - d] -= col[kv - d] * b[j];
    }
}

// One chain of the twisted solve, in the kernel's operation order: x points
// at chain-local row 0, rows advance by es.  own/other: the chains' tails.
void host_twisted_forward(const twisted_tables& t, int chain, double* x, long long es) {
    const int k = t.k, nc = chain ? t.n2 : t.n1;
    const double* l = t.lmul.data() + static_cast<size_t>(chain) * t.rows * k;
    for (int j = 0; j < nc; ++j)
        for (int i = 1; i <= k && j + i < nc; ++i) x[(j + i) * es] -= l[static_cast<size_t>(j) * k + i - 1] * x[j * es];
}

void host_twisted_backward(const twisted_tables& t, int chain, double* x, long long es, const double* other_tail) {
    const int k = t.k, nc = chain ? t.n2 : t.n1;
    const double* u = t.ucol.data() + static_cast<size_t>(chain) * t.rows * k;
    const double* r = t.rdiag.data() + static_cast<size_t>(chain) * t.rows;
    const double* g = t.g.data() + static_cast<size_t>(chain) * 2 * k * k;
    std::vector<double> own(k), z(k);
    for (int i = 0; i < k; ++i) own[i] = x[(nc - k + i) * es];
    for (int a = 0; a < k; ++a) {
        double s = 0.0;
        for (int i = 0; i < k; ++i) s += g[a * 2 * k + i] * own[i];
        for (int i = 0; i < k; ++i) s += g[a * 2 * k + k + i] * other_tail[i];
        z[a] = s;
    }
    for (int c = nc - 1; c >= 0; --c) {
        const double v = c >= nc - k ? z[c - (nc - k)] : x[c * es] * r[c];
        x[c * es] = v;
        for (int d = 1; d <= k && c - d >= 0; ++d) x[(c - d) * es] -= v * u[static_cast<size_t>(c) * k + d - 1];
    }
}

}  // namespace

void scale_twisted(const twisted_tables& t, int n, twisted_tables& o, std::vector<double>& scale) {
    const int k = t.k, rows = t.rows;
    o = t;
    scale.assign(n, 1.0);
    for (int chain = 0; chain < 2; ++chain) {
        const int nc = chain ? t.n2 : t.n1;
        const size_t off = static_cast<size_t>(chain) * rows;
        const double* sc = t.rdiag.data() + off;  // 1 / U(i, i), chain-local row i
        for (int i = 0; i < nc; ++i) scale[chain ? n - 1 - i : i] = sc[i];
        for (int j = 0; j < nc; ++j)
            for (int q = 1; q <= k; ++q) {
                const size_t at = (off + j) * k + q - 1;
                o.lmul[at] = j + q < nc ? sc[j + q] * t.lmul[at] / sc[j] : 0.0;
                o.ucol[at] = j - q >= 0 ? t.ucol[at] * sc[j - q] : 0.0;
            }
        for (int i = 0; i < nc; ++i) o.rdiag[off + i] = 1.0;
        const int no = chain ? t.n1 : t.n2;
        const double* so = t.rdiag.data() + static_cast<size_t>(1 - chain) * rows;
        double* g = o.g.data() + static_cast<size_t>(chain) * 2 * k * k;
        for (int a = 0; a < k; ++a)
            for (int i = 0; i < k; ++i) {
                g[a * 2 * k + i] /= sc[nc - k + i];
                g[a * 2 * k + k + i] /= so[no - k + i];
            }
    }
}

int make_twisted_tables(int n, int kl, int ku, int ldab, const double* ab, const int* ipiv, twisted_tables& t) {
    const int k = kl;
    if (kl != ku || k < 1 || k > 4 || n < 4 * k + 2) return 1;
    const int kv = kl + ku;
    // 1. the matrix itself, A = P0 L0 P1 L1 ... U, rebuilt densely from the factors
    std::vector<double> A(static_cast<size_t>(n) * n, 0.0);
    auto at = [&](int i, int j) -> double& { return A[static_cast<size_t>(i) * n + j]; };
    for (int j = 0; j < n; ++j)
        for (int d = 0; d <= kv && d <= j; ++d) at(j - d, j) = ab[static_cast<size_t>(j) * ldab + kv - d];
    for (int j = n - 1; j >= 0; --j) {
        const double* col = ab + static_cast<size_t>(j) * ldab;
        for (int i = 1; i <= kl && j + i < n; ++i) {
            const double l = col[kv + i];
            if (l == 0.0) continue;
            for (int c = j; c < n && c <= j + kv; ++c) at(j + i, c) += l * at(j, c);
        }
        const int p = ipiv[j] - 1;
        if (p != j)
            for (int c = 0; c < n; ++c) std::swap(at(j, c), at(p, c));
    }
    double amax = 0.0, outside = 0.0;
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
            const double v = std::fabs(at(i, j));
            if (j - i > ku || i - j > kl) {
                outside = std::max(outside, v);
                at(i, j) = 0.0;
            } else {
                amax = std::max(amax, v);
            }
        }
    if (!(amax > 0.0) || outside > 1e-12 * amax) return 2;

    // 2. chain 0: rows [0, n1) eliminated top-down over columns [0, n1 + k)
    const int n1 = n / 2, n2 = n - n1, rows = n2 + 16;
    t.k = k;
    t.n1 = n1;
    t.n2 = n2;
    t.rows = rows;
    t.lmul.assign(2 * static_cast<size_t>(rows) * k, 0.0);
    t.ucol.assign(2 * static_cast<size_t>(rows) * k, 0.0);
    t.rdiag.assign(2 * static_cast<size_t>(rows), 0.0);
    t.g.assign(2 * static_cast<size_t>(k) * 2 * k, 0.0);
    std::vector<double> S(static_cast<size_t>(2 * k) * 2 * k, 0.0);  // interface rows over x[n1-k .. n1+k)
    for (int chain = 0; chain < 2; ++chain) {
        const int nc = chain ? n2 : n1;
        const int width = nc + k;
        // B(i, j): chain-local entries; chain 1 reads A with rows and columns reversed
        std::vector<double> B(static_cast<size_t>(nc) * width, 0.0);
        for (int i = 0; i < nc; ++i)
            for (int j = std::max(0, i - k); j < width && j <= i + k; ++j)
                B[static_cast<size_t>(i) * width + j] = chain ? at(n - 1 - i, n - 1 - j) : at(i, j);
        double* l = t.lmul.data() + static_cast<size_t>(chain) * rows * k;
        double* u = t.ucol.data() + static_cast<size_t>(chain) * rows * k;
        double* r = t.rdiag.data() + static_cast<size_t>(chain) * rows;
        for (int j = 0; j < nc; ++j) {
            const double piv = B[static_cast<size_t>(j) * width + j];
            if (!(std::fabs(piv) > 1e-8 * amax)) return 3;
            for (int i = j + 1; i < nc && i <= j + k; ++i) {
                const double m = B[static_cast<size_t>(i) * width + j] / piv;
                l[static_cast<size_t>(j) * k + (i - j - 1)] = m;
                B[static_cast<size_t>(i) * width + j] = 0.0;
                for (int c = j + 1; c < width && c <= j + k; ++c)
                    B[static_cast<size_t>(i) * width + c] -= m * B[static_cast<size_t>(j) * width + c];
            }
        }
        double umax = 0.0;
        for (int c = 0; c < nc; ++c) {
            r[c] = 1.0 / B[static_cast<size_t>(c) * width + c];
            for (int d = 0; d <= k && c - d >= 0; ++d) {
                const double v = B[static_cast<size_t>(c - d) * width + c];
                umax = std::max(umax, std::fabs(v));
                if (d > 0) u[static_cast<size_t>(c) * k + d - 1] = v;
            }
        }
        if (umax > 1e4 * amax) return 4;  // element growth: unpivoted elimination not trusted
        // tail rows -> interface rows; chain-local column c is x[c] (chain 0) or x[n-1-c] (chain 1)
        for (int rr = 0; rr < k; ++rr) {
            const int i = nc - k + rr;
            for (int c = nc - k; c < nc + k; ++c) {
                const int xi = chain ? n - 1 - c : c;
                S[static_cast<size_t>(chain * k + rr) * 2 * k + (xi - (n1 - k))] = B[static_cast<size_t>(i) * width + c];
            }
        }
    }
    // 3. inverse of the 2k x 2k interface matrix (Gauss-Jordan, partial pivoting)
    const int m2 = 2 * k;
    std::vector<double> W(S), Inv(static_cast<size_t>(m2) * m2, 0.0);
    for (int i = 0; i < m2; ++i) Inv[static_cast<size_t>(i) * m2 + i] = 1.0;
    double smax = 0.0;
    for (double v : S) smax = std::max(smax, std::fabs(v));
    for (int c = 0; c < m2; ++c) {
        int pr = c;
        for (int i = c + 1; i < m2; ++i)
            if (std::fabs(W[static_cast<size_t>(i) * m2 + c]) > std::fabs(W[static_cast<size_t>(pr) * m2 + c])) pr = i;
        if (!(std::fabs(W[static_cast<size_t>(pr) * m2 + c]) > 1e-10 * smax)) return 5;
        for (int j = 0; j < m2; ++j) {
            std::swap(W[static_cast<size_t>(c) * m2 + j], W[static_cast<size_t>(pr) * m2 + j]);
            std::swap(Inv[static_cast<size_t>(c) * m2 + j], Inv[static_cast<size_t>(pr) * m2 + j]);
        }
        const double d = W[static_cast<size_t>(c) * m2 + c];
        for (int j = 0; j < m2; ++j) {
            W[static_cast<size_t>(c) * m2 + j] /= d;
            Inv[static_cast<size_t>(c) * m2 + j] /= d;
        }
        for (int i = 0; i < m2; ++i) {
            if (i == c) continue;
            const double f = W[static_cast<size_t>(i) * m2 + c];
            if (f == 0.0) continue;
            for (int j = 0; j < m2; ++j) {
                W[static_cast<size_t>(i) * m2 + j] -= f * W[static_cast<size_t>(c) * m2 + j];
                Inv[static_cast<size_t>(i) * m2 + j] -= f * Inv[static_cast<size_t>(c) * m2 + j];
            }
        }
    }
    // z = Inv [tail0; tail1] with z over x[n1-k .. n1+k).  Chain 0 owns z[0..k)
    // (its rows n1-k..n1-1); chain 1 owns z[k..2k) in reverse (its local row
    // n2-k+a is x[n1+k-1-a] = z[2k-1-a]).  Each chain's g row lists its own
    // tail's coefficients first.
    for (int a = 0; a < k; ++a)
        for (int i = 0; i < k; ++i) {
            t.g[static_cast<size_t>(a) * m2 + i] = Inv[static_cast<size_t>(a) * m2 + i];
            t.g[static_cast<size_t>(a) * m2 + k + i] = Inv[static_cast<size_t>(a) * m2 + k + i];
            const size_t row1 = static_cast<size_t>(m2 - 1 - a) * m2;
            t.g[static_cast<size_t>(k) * m2 + static_cast<size_t>(a) * m2 + i] = Inv[row1 + k + i];
            t.g[static_cast<size_t>(k) * m2 + static_cast<size_t>(a) * m2 + k + i] = Inv[row1 + i];
        }
    // 4. self-check against the LAPACK-order solve on a fixed pseudo-random right-hand side
    std::vector<double> b(n), x(n);
    unsigned long long state = 0x9E3779B97F4A7C15ULL;
    for (int i = 0; i < n; ++i) {
        state = state * 6364136223846793005ULL + 1442695040888963407ULL;
        b[i] = static_cast<double>(state >> 11) * 0x1.0p-53 - 0.5;
    }
    x = b;
    host_band_solve(n, kl, ku, ldab, ab, ipiv, b.data());
    host_twisted_forward(t, 0, x.data(), 1);
    host_twisted_forward(t, 1, x.data() + n - 1, -1);
    std::vector<double> tail0(k), tail1(k);
    for (int i = 0; i < k; ++i) {
        tail0[i] = x[n1 - k + i];
        tail1[i] = x[n - 1 - (n2 - k + i)];
    }
    host_twisted_backward(t, 0, x.data(), 1, tail1.data());
    host_twisted_backward(t, 1, x.data() + n - 1, -1, tail0.data());
    double num = 0.0, den = 0.0;
    for (int i = 0; i < n; ++i) {
        num += (x[i] - b[i]) * (x[i] - b[i]);
        den += b[i] * b[i];
    }
    if (!(num <= 1e-24 * den)) return 6;
    return 0;
}

}  // namespace adsg
