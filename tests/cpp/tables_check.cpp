// Host-side direction tables, checked on the CPU (no device call): for the
// reference's uniform open-knot spaces of degree 1-4 and several lengths,
// the dgbtrf factors give LAPACK-order solve tables; the two-ended
// factorisation is built exactly when the line is long enough (n >= 4k + 2)
// and passes its own accuracy check against the LAPACK-order solve; its
// row-scaled form has a unit diagonal and finite, non-zero scales; the band
// rows are symmetric away from the ends, where the pair-sum passes use them.
#include <cmath>
#include <cstdio>
#include <vector>

#include "adsg_internal.hpp"

using namespace adsg;

// adsg_host.cpp's C-ABI entries record errors through the engine's fail();
// this program calls none of them
namespace adsg {
int fail(int code, const char*) { return code; }
}  // namespace adsg

static int failures = 0;

static void check(bool ok, const char* what, int p, int e) {
    if (!ok) {
        std::printf("FAIL p=%d elements=%d: %s\n", p, e, what);
        ++failures;
    }
}

// row-format band [n][2p+1] of a LAPACK band with kl = ku = p (ldab = 3p+1)
static std::vector<double> rows_of(const dim_host& d, const std::vector<double>& ab) {
    const int p = d.p, n = d.n, bw = 2 * p + 1;
    std::vector<double> r(static_cast<size_t>(n) * bw, 0.0);
    for (int i = 0; i < n; ++i)
        for (int t = 0; t < bw; ++t) {
            const int c = i - p + t;
            if (c >= 0 && c < n) r[static_cast<size_t>(i) * bw + t] = ab[static_cast<size_t>(c) * d.ldab + 2 * p + i - c];
        }
    return r;
}

int main() {
    for (int p = 1; p <= 4; ++p)
        for (int e : {1, 3, 8, 20, 61}) {
            dim_host d;
            check(build_dimension(d, p, e, 0.0, 1.0, p + 1), "build_dimension", p, e);
            const int n = d.n;
            check(n == e + p, "n = elements + p", p, e);

            solve_tables st;
            check(make_solve_tables(n, p, p, d.ldab, d.lu.data(), d.ipiv.data(), st) == 0, "solve tables", p, e);

            int lo = -1, hi = -1;
            symmetric_row_range(rows_of(d, d.mass), rows_of(d, d.stiff), n, p, lo, hi);
            check(0 <= lo && lo <= hi && hi <= n, "symmetric range inside the line", p, e);
            if (e >= 4 * p + 2)
                check(lo <= 2 * p - 1 && hi >= n - (2 * p - 1), "rows 2p-1 or more from the ends are symmetric", p, e);

            twisted_tables tw;
            const int rc = make_twisted_tables(n, p, p, d.ldab, d.lu.data(), d.ipiv.data(), tw);
            check((rc == 0) == (n >= 4 * p + 2), "two-ended tables exactly for n >= 4k+2", p, e);
            if (rc != 0) continue;
            check(tw.k == p && tw.n1 + tw.n2 == n && tw.n1 == n / 2, "chain split", p, e);
            check(tw.lmul.size() == 2 * static_cast<size_t>(tw.rows) * p && tw.ucol.size() == tw.lmul.size() &&
                      tw.rdiag.size() == 2 * static_cast<size_t>(tw.rows) && tw.g.size() == 4 * static_cast<size_t>(p) * p,
                  "table sizes", p, e);
            twisted_tables u;
            std::vector<double> scale;
            scale_twisted(tw, n, u, scale);
            bool finite = scale.size() == static_cast<size_t>(n);
            for (double s : scale) finite = finite && std::isfinite(s) && s != 0.0;
            check(finite, "finite non-zero row scales", p, e);
            bool unit = true;
            for (int chain = 0; chain < 2; ++chain)
                for (int i = 0; i < (chain ? tw.n2 : tw.n1); ++i) unit = unit && u.rdiag[chain * tw.rows + i] == 1.0;
            check(unit, "unit diagonal after scaling", p, e);
        }
    // a band that is not square in shape has no two-ended form
    dim_host d;
    build_dimension(d, 2, 20, 0.0, 1.0, 3);
    twisted_tables tw;
    check(make_twisted_tables(d.n, 2, 1, d.ldab, d.lu.data(), d.ipiv.data(), tw) != 0, "kl != ku rejected", 2, 20);
    if (failures) return 1;
    std::printf("ok\n");
    return 0;
}
