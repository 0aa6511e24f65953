/* The CPU oracle's entry points on small problems, for a build under
 * AddressSanitizer + UndefinedBehaviorSanitizer (no recovery): every entry
 * the tests call, on 1D/2D/3D grids of degree 1-4 with uneven sizes, with
 * consistency checks that need no fixture -- the threaded RHS against the
 * sequential one, the solve against the mass apply (the heat RHS at dt = 0),
 * the transposed solve against the plain one (the mass matrix is symmetric),
 * threaded against sequential steps, a unit kappa field and the general form
 * against the heat RHS, and banded LU residuals in 'N' and 'T' with pivoting.
 * Test code: prints "ok" when every check holds. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "ads_oracle.h"

static int failures = 0;

static void check(int ok, const char* what, const char* label) {
    if (!ok) {
        printf("FAIL %s: %s\n", label, what);
        ++failures;
    }
}

static unsigned long long rng_state = 0x9e3779b97f4a7c15ULL;
static double uniform(void) { /* in [-1, 1) */
    rng_state = rng_state * 6364136223846793005ULL + 1442695040888963407ULL;
    return (double)(rng_state >> 11) * (2.0 / 9007199254740992.0) - 1.0;
}

static double rel_l2(const double* a, const double* b, long n) {
    double num = 0, den = 0;
    for (long i = 0; i < n; ++i) {
        num += (a[i] - b[i]) * (a[i] - b[i]);
        den += b[i] * b[i];
    }
    return den > 0 ? sqrt(num / den) : sqrt(num);
}

static int all_finite(const double* a, long n) {
    for (long i = 0; i < n; ++i)
        if (!isfinite(a[i])) return 0;
    return 1;
}

static void problem_case(int ndim, const int* p, const int* E) {
    char label[96];
    snprintf(label, sizeof label, "%dD p=%d,%d,%d E=%d,%d,%d", ndim, p[0], ndim > 1 ? p[1] : 0, ndim > 2 ? p[2] : 0,
             E[0], ndim > 1 ? E[1] : 0, ndim > 2 ? E[2] : 0);
    orc_problem* pr = orc_problem_create(ndim, p, E);
    check(pr != NULL, "create", label);
    if (!pr) return;
    const long size = orc_problem_size(pr);
    const double dt = 1e-5;
    double* u = malloc(sizeof(double) * size);
    double* r0 = malloc(sizeof(double) * size);
    double* r1 = malloc(sizeof(double) * size);
    double* t = malloc(sizeof(double) * size);
    for (long i = 0; i < size; ++i) u[i] = uniform();

    /* every dimension's tables copied out */
    for (int d = 0; d < ndim; ++d) {
        const int n = orc_problem_dofs(pr, d), q = p[d] + 1, ldab = 3 * p[d] + 1;
        double* btab = malloc(sizeof(double) * E[d] * q * 2 * (p[d] + 1));
        double* w = malloc(sizeof(double) * q);
        double* J = malloc(sizeof(double) * E[d]);
        int* fd = malloc(sizeof(int) * E[d]);
        double* mab = malloc(sizeof(double) * ldab * n);
        double* lab = malloc(sizeof(double) * ldab * n);
        int* ipiv = malloc(sizeof(int) * n);
        check(orc_problem_dim(pr, d, btab, w, J, fd, mab, lab, ipiv) == 0, "problem_dim", label);
        check(n == E[d] + p[d] && fd[E[d] - 1] == E[d] - 1, "dofs and first dofs", label);
        free(btab), free(w), free(J), free(fd), free(mab), free(lab), free(ipiv);
    }

    check(orc_heat_rhs(pr, u, r0, dt) == 0 && all_finite(r0, size), "heat_rhs", label);
    check(orc_heat_rhs_mt(pr, u, r1, dt, 3) == 0, "heat_rhs_mt", label);
    check(rel_l2(r1, r0, size) <= 1e-12, "threaded RHS against sequential", label);

    /* mass apply then solve returns the input */
    check(orc_heat_rhs(pr, u, t, 0.0) == 0 && orc_ads_solve(pr, t) == 0, "mass apply + solve", label);
    check(rel_l2(t, u, size) <= 1e-9, "solve inverts the mass apply", label);
    memcpy(r1, r0, sizeof(double) * size);
    memcpy(t, r0, sizeof(double) * size);
    check(orc_ads_solve(pr, r1) == 0 && orc_ads_solve_t(pr, t) == 0, "solve / solve_t", label);
    check(rel_l2(t, r1, size) <= 1e-9, "transposed solve of the symmetric mass", label);

    /* a unit kappa field (partition of unity) and the general form reduce to the heat RHS */
    for (long i = 0; i < size; ++i) t[i] = 1.0;
    check(orc_heat_rhs_kappa(pr, u, t, r1, dt) == 0, "heat_rhs_kappa", label);
    check(rel_l2(r1, r0, size) <= 1e-12, "unit kappa against heat RHS", label);
    if (ndim >= 2) {
        const double cst[4] = {1.0, -dt, 0.0, 0.0};
        check(orc_form_rhs(pr, u, cst, NULL, NULL, NULL, NULL, r1) == 0, "form_rhs", label);
        check(rel_l2(r1, r0, size) <= 1e-12, "general form against heat RHS", label);
    }
    memset(t, 0, sizeof(double) * size);
    if (ndim >= 2) check(orc_kappa_grad(pr, u, r0, t, dt) == 0 && all_finite(t, size), "kappa_grad", label);
    else check(orc_kappa_grad(pr, u, r0, t, dt) == -1, "kappa_grad refuses 1D", label);
    check(orc_projection_sin(pr, t) == 0 && all_finite(t, size), "projection_sin", label);

    /* two steps, sequential and threaded */
    memcpy(r0, u, sizeof(double) * size);
    memcpy(r1, u, sizeof(double) * size);
    check(orc_heat_steps(pr, r0, dt, 2, 1) == 0 && orc_heat_steps(pr, r1, dt, 2, 3) == 0, "heat_steps", label);
    check(rel_l2(r1, r0, size) <= 1e-11, "threaded steps against sequential", label);

    free(u), free(r0), free(r1), free(t);
    orc_problem_destroy(pr);
}

/* pivoted banded LU against a dense product */
static void band_case(int n, int kl, int ku, int nrhs, int ldb) {
    char label[64];
    snprintf(label, sizeof label, "dgbtrf/dgbtrs n=%d kl=%d ku=%d", n, kl, ku);
    const int ldab = 2 * kl + ku + 1;
    double* A = calloc((size_t)n * n, sizeof(double));
    double* ab = calloc((size_t)ldab * n, sizeof(double));
    int* ipiv = malloc(sizeof(int) * n);
    for (int j = 0; j < n; ++j)
        for (int i = j - ku < 0 ? 0 : j - ku; i <= j + kl && i < n; ++i) {
            const double v = uniform();  /* no dominance: pivoting happens */
            A[(size_t)j * n + i] = v;
            ab[(size_t)j * ldab + kl + ku + i - j] = v;
        }
    check(orc_dgbtrf(n, kl, ku, ab, ldab, ipiv) == 0, "dgbtrf info", label);
    for (int tr = 0; tr < 2; ++tr) {
        double* x = malloc(sizeof(double) * ldb * nrhs);
        double* b = malloc(sizeof(double) * ldb * nrhs);
        for (int i = 0; i < ldb * nrhs; ++i) b[i] = x[i] = uniform();
        check(orc_dgbtrs(tr ? 'T' : 'N', n, kl, ku, nrhs, ab, ldab, ipiv, x, ldb) == 0, "dgbtrs info", label);
        double worst = 0;
        for (int c = 0; c < nrhs; ++c)
            for (int i = 0; i < n; ++i) {
                double s = 0;
                for (int k = 0; k < n; ++k) s += (tr ? A[(size_t)i * n + k] : A[(size_t)k * n + i]) * x[c * ldb + k];
                worst = fmax(worst, fabs(s - b[c * ldb + i]));
            }
        check(worst <= 1e-9, tr ? "residual 'T'" : "residual 'N'", label);
        for (int c = 0; c < nrhs; ++c)  /* rows past n untouched */
            for (int i = n; i < ldb; ++i) check(x[c * ldb + i] == b[c * ldb + i], "ldb padding", label);
        free(x), free(b);
    }
    free(A), free(ab), free(ipiv);
}

int main(void) {
    for (int q = 2; q <= 64; ++q) {
        double x[64], w[64], s = 0;
        check(orc_gauss(q, x, w) == 0, "gauss", "gauss");
        for (int i = 0; i < q; ++i) s += w[i];
        check(fabs(s - 2.0) <= 1e-13, "gauss weights sum to 2", "gauss");
    }
    for (int p = 1; p <= 4; ++p) {
        const int E = 7, q = p + 1;
        double knots[7 + 2 * 4 + 1];
        double* btab = malloc(sizeof(double) * E * q * 2 * (p + 1));
        double* xq = malloc(sizeof(double) * E * q);
        double J[7];
        int fd[7];
        check(orc_knots(p, E, 0.0, 1.0, knots) == 0, "knots", "basis");
        check(orc_basis_tables(p, E, 0.0, 1.0, q, btab, xq, J, fd) == 0, "basis tables", "basis");
        for (int e = 0; e < E; ++e)
            for (int k = 0; k < q; ++k) {  /* partition of unity; derivatives sum to zero */
                double v = 0, dv = 0;
                for (int a = 0; a <= p; ++a) {
                    v += btab[((e * q + k) * 2 + 0) * (p + 1) + a];
                    dv += btab[((e * q + k) * 2 + 1) * (p + 1) + a];
                }
                check(fabs(v - 1.0) <= 1e-14 && fabs(dv) <= 1e-11, "partition of unity", "basis");
            }
        free(btab), free(xq);
    }
    {
        const int p[1] = {3}, E[1] = {12};
        problem_case(1, p, E);
    }
    {
        const int p[2] = {2, 4}, E[2] = {9, 6};
        problem_case(2, p, E);
    }
    {
        const int p[2] = {1, 1}, E[2] = {5, 1};
        problem_case(2, p, E);
    }
    {
        const int p[3] = {2, 3, 4}, E[3] = {5, 4, 3};
        problem_case(3, p, E);
    }
    {
        const int p[3] = {4, 4, 4}, E[3] = {4, 5, 6};
        problem_case(3, p, E);
    }
    band_case(37, 2, 3, 3, 40);
    band_case(20, 4, 4, 2, 20);
    band_case(9, 1, 1, 1, 9);
    printf("%s\n", failures ? "FAILED" : "ok");
    return failures ? 1 : 0;
}
