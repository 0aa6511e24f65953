// Host-side set-up of one dimension: knot vector, Gauss rule, basis tables,
// 1D mass/stiffness bands and the pivoted band LU of the mass matrix.  This is
// the set-up the reference performs once per dimension on the CPU
// (src/ads/simulation/dimension.cpp:8-21, dimension::factorize_matrix); the
// GPU never runs it.  Everything here is the product's own code.
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "adsg_internal.hpp"

namespace adsg {

// Gauss-Legendre rule on [-1, 1] (the reference tabulates the same rule in
// include/ads/quad/gauss.hpp for 2..64 points).  Newton on P_q with the
// derivative from the recurrence, in extended precision, ascending order.
bool gauss_legendre(int q, double* x, double* w) {
    if (q < 2 || q > 64) return false;
    const long double pi = 3.141592653589793238462643383279502884L;
    for (int k = 0; k < (q + 1) / 2; ++k) {
        long double z = std::cos(pi * (k + 0.75L) / (q + 0.5L));
        long double pd = 1;
        for (int it = 0; it < 100; ++it) {
            long double pm = 1, pc = z;
            for (int m = 2; m <= q; ++m) {
                long double pn = ((2 * m - 1) * z * pc - (m - 1) * pm) / m;
                pm = pc;
                pc = pn;
            }
            pd = q * (z * pc - pm) / (z * z - 1);
            long double step = pc / pd;
            z -= step;
            if (std::fabs(static_cast<double>(step)) < 1e-300 || std::fabs(step) < 1e-30L) break;
        }
        long double pm = 1, pc = z;
        for (int m = 2; m <= q; ++m) {
            long double pn = ((2 * m - 1) * z * pc - (m - 1) * pm) / m;
            pm = pc;
            pc = pn;
        }
        pd = q * (z * pc - pm) / (z * z - 1);
        long double wk = 2.0L / ((1 - z * z) * pd * pd);
        x[q - 1 - k] = static_cast<double>(z);
        x[k] = -static_cast<double>(z);
        w[q - 1 - k] = static_cast<double>(wk);
        w[k] = static_cast<double>(wk);
    }
    if (q % 2 == 1) x[q / 2] = 0.0;
    return true;
}

namespace {

double interp(double t, double a, double b) { return (1 - t) * a + t * b; }

// Open (clamped) uniform knot vector with p+1 repeated end knots and simple
// interior knots, as bspline::create_basis(a, b, p, elements, 0) builds it.
std::vector<double> open_knots(int p, int elements, double a, double b) {
    int size = elements + 2 * p + 1;
    std::vector<double> k(size);
    for (int i = 0; i <= p; ++i) {
        k[i] = a;
        k[size - 1 - i] = b;
    }
    for (int i = 1; i < elements; ++i) k[p + i] = interp(static_cast<double>(i) / elements, a, b);
    return k;
}

int span_of(double x, const std::vector<double>& k, int p) {
    int lo = p;
    int hi = static_cast<int>(k.size()) - p - 1;
    if (x >= k[hi]) return hi - 1;
    if (x <= k[lo]) return lo;
    int mid = (lo + hi) / 2;
    while (x < k[mid] || x >= k[mid + 1]) {
        if (x < k[mid])
            hi = mid;
        else
            lo = mid;
        mid = (lo + hi) / 2;
    }
    return mid;
}

// Values and first derivatives of the p+1 non-zero B-splines at x: the
// triangular Cox-de Boor scheme with derivative coefficients (Piegl & Tiller,
// The NURBS Book, algorithm A2.3), first derivative only.
void eval_ders(int span, double x, const std::vector<double>& k, int p, double* val, double* der) {
    double tri[ADSG_MAX_DEGREE + 1][ADSG_MAX_DEGREE + 1];
    double lft[ADSG_MAX_DEGREE + 1];
    double rgt[ADSG_MAX_DEGREE + 1];
    tri[0][0] = 1;
    for (int j = 1; j <= p; ++j) {
        lft[j] = x - k[span + 1 - j];
        rgt[j] = k[span + j] - x;
        double acc = 0;
        for (int r = 0; r < j; ++r) {
            tri[j][r] = rgt[r + 1] + lft[j - r];
            double t = tri[r][j - 1] / tri[j][r];
            tri[r][j] = acc + rgt[r + 1] * t;
            acc = lft[j - r] * t;
        }
        tri[j][j] = acc;
    }
    for (int j = 0; j <= p; ++j) val[j] = tri[j][p];
    for (int r = 0; r <= p; ++r) {
        // first-derivative coefficients a_{1,0} and a_{1,1}
        double d = 0;
        double c0 = 0;
        if (r >= 1) {
            c0 = 1.0 / tri[p][r - 1];
            d = c0 * tri[r - 1][p - 1];
        }
        if (r <= p - 1) {
            double c1 = -1.0 / tri[p][r];
            d += c1 * tri[r][p - 1];
        }
        der[r] = d * p;
    }
}

}  // namespace

// Band entry (i, j) in the factorisable LAPACK layout.
static inline double& band_at(std::vector<double>& ab, int ldab, int kl, int ku, int i, int j) {
    return ab[static_cast<size_t>(j) * ldab + kl + ku + i - j];
}

bool build_dimension(dim_host& d, int p, int elements, double a, double b, int q) {
    if (p < 1 || p > ADSG_MAX_DEGREE || elements < 1 || q < 2 || q > 64) return false;
    d.p = p;
    d.elements = elements;
    d.q = q;
    d.n = elements + p;
    d.kl = p;
    d.ku = p;
    d.ldab = 2 * d.kl + d.ku + 1;
    d.knots = open_knots(p, elements, a, b);
    std::vector<double> gx(q);
    d.w.assign(q, 0.0);
    gauss_legendre(q, gx.data(), d.w.data());

    // element break points = distinct knots
    std::vector<double> pts;
    pts.push_back(d.knots[0]);
    for (size_t i = 1; i < d.knots.size(); ++i)
        if (d.knots[i] != d.knots[i - 1]) pts.push_back(d.knots[i]);

    d.btab.assign(static_cast<size_t>(elements) * q * 2 * (p + 1), 0.0);
    d.xq.assign(static_cast<size_t>(elements) * q, 0.0);
    d.J.assign(elements, 0.0);
    d.first_dofs.assign(elements, 0);
    for (int e = 0; e < elements; ++e) {
        double x1 = pts[e], x2 = pts[e + 1];
        d.J[e] = 0.5 * (x2 - x1);
        for (int k = 0; k < q; ++k) {
            double t = 0.5 * (gx[k] + 1);
            double x = interp(t, x1, x2);
            d.xq[static_cast<size_t>(e) * q + k] = x;
            double* row = &d.btab[(static_cast<size_t>(e) * q + k) * 2 * (p + 1)];
            eval_ders(span_of(x, d.knots, p), x, d.knots, p, row, row + (p + 1));
        }
    }
    int e = 0;
    for (int i = p; i + 1 < static_cast<int>(d.knots.size()) - p; ++i)
        if (d.knots[i] != d.knots[i + 1]) d.first_dofs[e++] = i - p;

    form_band(d, 0, d.mass);
    form_band(d, 1, d.stiff);
    d.lu = d.mass;
    return factorize(d) == 0;
}

// gram_matrix_1d / stiffness_matrix_1d: M(a,b) += B_a B_b w_q J_e over
// elements and points, with the reference's association ((Ba*Bb)*w)*J.
void form_band(const dim_host& d, int which, std::vector<double>& ab) {
    int p = d.p;
    ab.assign(static_cast<size_t>(d.ldab) * d.n, 0.0);
    for (int e = 0; e < d.elements; ++e) {
        for (int k = 0; k < d.q; ++k) {
            const double* v = &d.btab[((static_cast<size_t>(e) * d.q + k) * 2 + which) * (p + 1)];
            int f = d.first_dofs[e];
            for (int r = 0; r <= p; ++r)
                for (int c = 0; c <= p; ++c) band_at(ab, d.ldab, d.kl, d.ku, f + r, f + c) += v[r] * v[c] * d.w[k] * d.J[e];
        }
    }
}

// Pivoted band LU of d.lu in place (LAPACK's unblocked dgbtf2 schedule, the
// one dgbtrf uses for narrow bands).  Returns the 1-based column of the first
// zero pivot, 0 on success.
int factorize(dim_host& d) {
    int n = d.n, kl = d.kl, ku = d.ku, ldab = d.ldab;
    int kv = kl + ku;
    d.ipiv.assign(n, 0);
    auto A = [&](int r, int c) -> double& { return d.lu[static_cast<size_t>(c) * ldab + r]; };  // 0-based
    for (int j = ku + 1; j < std::min(kv, n); ++j)
        for (int i = kv - j; i < kl; ++i) A(i, j) = 0;
    int reach = 0;  // last column (0-based) touched by row swaps so far
    int info = 0;
    for (int j = 0; j < n; ++j) {
        if (j + kv < n)
            for (int i = 0; i < kl; ++i) A(i, j + kv) = 0;
        int km = std::min(kl, n - 1 - j);
        int jp = 0;
        double big = std::fabs(A(kv, j));
        for (int i = 1; i <= km; ++i) {
            double v = std::fabs(A(kv + i, j));
            if (v > big) {
                big = v;
                jp = i;
            }
        }
        d.ipiv[j] = jp + j + 1;
        if (A(kv + jp, j) != 0) {
            reach = std::max(reach, std::min(j + ku + jp, n - 1));
            if (jp != 0)
                for (int c = 0; c <= reach - j; ++c) std::swap(A(kv + jp - c, j + c), A(kv - c, j + c));
            if (km > 0) {
                double inv = 1.0 / A(kv, j);
                for (int i = 1; i <= km; ++i) A(kv + i, j) *= inv;
                for (int c = 1; c <= reach - j; ++c) {
                    double y = A(kv - c, j + c);
                    if (y != 0) {
                        double t = -y;
                        for (int i = 1; i <= km; ++i) A(kv + i - c, j + c) += A(kv + i, j) * t;
                    }
                }
            }
        } else if (info == 0) {
            info = j + 1;
        }
    }
    return info;
}

}  // namespace adsg

using adsg::dim_host;

struct adsg_dim {
    dim_host h;
};

extern "C" {

int adsg_dim_create(int p, int elements, double a, double b, int quad_order, adsg_dim** out) {
    if (p < 1 || p > ADSG_MAX_DEGREE) return adsg::fail(-1, "degree out of range");
    if (elements < 1) return adsg::fail(-2, "elements must be >= 1");
    if (!(b > a)) return adsg::fail(-4, "interval must satisfy b > a");
    if (quad_order <= 0) quad_order = p + 1;
    if (quad_order < 2 || quad_order > 64) return adsg::fail(-5, "quad_order out of range");
    if (!out) return adsg::fail(-6, "out is NULL");
    auto* d = new (std::nothrow) adsg_dim;
    if (!d) return adsg::fail(ADSG_ERR_NOMEM, "host allocation failed");
    if (!adsg::build_dimension(d->h, p, elements, a, b, quad_order)) {
        delete d;
        return adsg::fail(ADSG_ERR_SINGULAR, "mass matrix factorisation failed");
    }
    *out = d;
    return 0;
}

void adsg_dim_destroy(adsg_dim* d) { delete d; }

int adsg_dim_describe(const adsg_dim* d, adsg_dim_desc* out) {
    if (!d) return adsg::fail(-1, "dim is NULL");
    if (!out) return adsg::fail(-2, "out is NULL");
    const dim_host& h = d->h;
    out->p = h.p;
    out->elements = h.elements;
    out->quad_order = h.q;
    out->n = h.n;
    out->btab = h.btab.data();
    out->w = h.w.data();
    out->J = h.J.data();
    out->first_dofs = h.first_dofs.data();
    out->kl = h.kl;
    out->ku = h.ku;
    out->ldab = h.ldab;
    out->lu = h.lu.data();
    out->ipiv = h.ipiv.data();
    out->xq = h.xq.data();
    return 0;
}

int adsg_dim_fix_dof(adsg_dim* d, int k) {
    if (!d) return adsg::fail(-1, "dim is NULL");
    dim_host& h = d->h;
    if (k < 0 || k >= h.n) return adsg::fail(-2, "dof index out of range");
    // identity row k of the unfactorised mass matrix, then refactorise
    int lo = std::max(k - h.p, 0), hi = std::min(k + h.p, h.n - 1);
    for (int i = lo; i <= hi; ++i) adsg::band_at(h.mass, h.ldab, h.kl, h.ku, k, i) = 0;
    adsg::band_at(h.mass, h.ldab, h.kl, h.ku, k, k) = 1;
    h.lu = h.mass;
    if (adsg::factorize(h) != 0) return adsg::fail(ADSG_ERR_SINGULAR, "refactorisation failed");
    return 0;
}

int adsg_dim_form_band(const adsg_dim* d, int which, double* ab) {
    if (!d) return adsg::fail(-1, "dim is NULL");
    if (which != 0 && which != 1) return adsg::fail(-2, "which must be 0 (mass) or 1 (stiffness)");
    if (!ab) return adsg::fail(-3, "ab is NULL");
    const dim_host& h = d->h;
    const std::vector<double>& src = which ? h.stiff : h.mass;
    std::memcpy(ab, src.data(), sizeof(double) * src.size());
    return 0;
}

}  // extern "C"
