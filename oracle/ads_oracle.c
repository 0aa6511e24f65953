/*
 * CPU oracle for the IGA-ADS explicit heat step -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain C restatement of the reference algorithm (marcinlos/iga-ads), each
 * function citing the reference file:line it follows.  Only tests/, the smoke
 * check and the CPU-baseline leg of bench.py call it; the product never does.
 * The restatement is pinned against the reference's own compiled code
 * (oracle/_ref) and the reference tests' known answers via tests/golden/.
 *
 * Third-party algorithm restated here: LAPACK dgbtf2/dgbtrs/dtbsv (the
 * reference links whatever LAPACK find_package(LAPACK) finds, unpinned; the
 * comparison build here uses OpenBLAS 0.3.31.dev bundled with scipy 1.18.1).
 */
#include "ads_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define ORC_MAXD 3
#define ORC_MAXP 8

/* ------------------------------------------------------------------------ */
/* Gauss-Legendre nodes (quad/gauss.hpp: gauss_data<N>::X/W, N = 2..64).     */
/* Computed by Newton iteration on the Legendre three-term recurrence in     */
/* long double, then rounded; the middle node of an odd rule is exactly 0.   */
/* ------------------------------------------------------------------------ */
int orc_gauss(int q, double* x, double* w) {
    if (q < 2 || q > 64) return -1;
    const long double pi = 3.141592653589793238462643383279502884L;
    for (int k = 0; k < (q + 1) / 2; ++k) {
        long double z = cosl(pi * (k + 0.75L) / (q + 0.5L));
        long double dp = 0;
        for (int it = 0; it < 100; ++it) {
            long double p0 = 1, p1 = z;
            for (int n = 2; n <= q; ++n) {
                long double p2 = ((2 * n - 1) * z * p1 - (n - 1) * p0) / n;
                p0 = p1;
                p1 = p2;
            }
            dp = q * (z * p1 - p0) / (z * z - 1);
            long double dz = p1 / dp;
            z -= dz;
            if (fabsl(dz) < 1e-30L) break;
        }
        {
            long double p0 = 1, p1 = z;
            for (int n = 2; n <= q; ++n) {
                long double p2 = ((2 * n - 1) * z * p1 - (n - 1) * p0) / n;
                p0 = p1;
                p1 = p2;
            }
            dp = q * (z * p1 - p0) / (z * z - 1);
        }
        long double wk = 2.0L / ((1 - z * z) * dp * dp);
        /* z is the k-th largest root */
        x[q - 1 - k] = (double)z;
        x[k] = -(double)z;
        w[q - 1 - k] = (double)wk;
        w[k] = (double)wk;
    }
    if (q % 2 == 1) x[q / 2] = 0.0;
    return 0;
}

/* util.hpp:16-26 lerp(t, a, b) = (1 - t) * a + t * b; lerp(i, n, a, b) with t = i/n */
static double lerp_t(double t, double a, double b) { return (1 - t) * a + t * b; }
static double lerp_in(int i, int n, double a, double b) { return lerp_t((double)i / (double)n, a, b); }

/* bspline.cpp:26-43, repeated_nodes = 0 (r = 1) */
int orc_knots(int p, int elements, double a, double b, double* knots) {
    if (p < 1 || elements < 1) return -1;
    int points = elements + 1;
    int size = 2 * (p + 1) + (points - 2);
    for (int i = 0; i <= p; ++i) {
        knots[i] = a;
        knots[size - i - 1] = b;
    }
    for (int i = 1; i < points - 1; ++i) knots[p + 1 + (i - 1)] = lerp_in(i, elements, a, b);
    return 0;
}

/* bspline.cpp:61-81: span search between begin_idx = p and end_idx = size-p-1 */
static int find_span(double x, const double* knots, int size, int p) {
    int low = p, high = size - p - 1;
    if (x >= knots[high]) return high - 1;
    if (x <= knots[low]) return low;
    int idx = (low + high) / 2;
    while (x < knots[idx] || x >= knots[idx + 1]) {
        if (x < knots[idx])
            high = idx;
        else
            low = idx;
        idx = (low + high) / 2;
    }
    return idx;
}

/* Basis functions and first derivatives at x (bspline.cpp:102-160), the
 * Cox-de Boor triangle with derivative coefficients of The NURBS Book A2.3,
 * specialised to n = 1 derivative: out0[j] = N_{span-p+j,p}(x), out1[j] = N'. */
static void basis_ders1(int span, double x, const double* knots, int p, double* out0, double* out1) {
    double ndu[ORC_MAXP + 1][ORC_MAXP + 1];
    double left[ORC_MAXP + 1], right[ORC_MAXP + 1];
    double a[2][ORC_MAXP + 1];
    ndu[0][0] = 1;
    for (int j = 1; j <= p; ++j) {
        left[j] = x - knots[span + 1 - j];
        right[j] = knots[span + j] - x;
        double saved = 0;
        for (int r = 0; r < j; ++r) {
            ndu[j][r] = right[r + 1] + left[j - r]; /* lower triangle: knot differences */
            double tmp = ndu[r][j - 1] / ndu[j][r];
            ndu[r][j] = saved + right[r + 1] * tmp;
            saved = left[j - r] * tmp;
        }
        ndu[j][j] = saved;
    }
    for (int j = 0; j <= p; ++j) out0[j] = ndu[j][p];
    for (int r = 0; r <= p; ++r) {
        int s1 = 0, s2 = 1;
        a[0][0] = 1;
        /* k = 1 only */
        int k = 1;
        double d = 0;
        int rk = r - k, pk = p - k;
        if (r >= k) {
            a[s2][0] = a[s1][0] / ndu[pk + 1][rk];
            d = a[s2][0] * ndu[rk][pk];
        }
        int j1 = (rk >= -1) ? 1 : -rk;
        int j2 = (r - 1 <= pk) ? k - 1 : p - r;
        for (int j = j1; j <= j2; ++j) {
            a[s2][j] = (a[s1][j] - a[s1][j - 1]) / ndu[pk + 1][rk + j];
            d += a[s2][j] * ndu[rk + j][pk];
        }
        if (r <= pk) {
            a[s2][k] = -a[s1][k - 1] / ndu[pk + 1][r];
            d += a[s2][k] * ndu[r][pk];
        }
        out1[r] = d;
    }
    for (int j = 0; j <= p; ++j) out1[j] *= p;
}

/* basis_data.cpp:63-114 with derivatives = 1, elem_division = 1 and the
 * first_nonzero_dofs scan of bspline.cpp:162-172. */
int orc_basis_tables(int p, int elements, double a, double b, int q, double* btab, double* xq,
                     double* J, int* first_dofs) {
    if (p < 1 || p > ORC_MAXP || elements < 1 || q < 2 || q > 64) return -1;
    int size = elements + 2 * p + 1;
    double* knots = (double*)malloc(sizeof(double) * size);
    double* X = (double*)malloc(sizeof(double) * q);
    double* W = (double*)malloc(sizeof(double) * q);
    orc_knots(p, elements, a, b, knots);
    orc_gauss(q, X, W);
    /* element break points: the distinct knots (bspline.hpp basis ctor) */
    double* pts = (double*)malloc(sizeof(double) * (elements + 1));
    int np = 0;
    pts[np++] = knots[0];
    for (int i = 1; i < size; ++i)
        if (knots[i] != knots[i - 1]) pts[np++] = knots[i];
    for (int e = 0; e < elements; ++e) {
        double x1 = pts[e], x2 = pts[e + 1];
        if (J) J[e] = 0.5 * (x2 - x1);
        for (int k = 0; k < q; ++k) {
            double t = 0.5 * (X[k] + 1);
            double xx = lerp_t(t, x1, x2);
            if (xq) xq[e * q + k] = xx;
            int span = find_span(xx, knots, size, p);
            double* o0 = btab + ((long)(e * q + k) * 2 + 0) * (p + 1);
            double* o1 = btab + ((long)(e * q + k) * 2 + 1) * (p + 1);
            basis_ders1(span, xx, knots, p, o0, o1);
        }
    }
    if (first_dofs) {
        int e = 0;
        for (int i = p; i + 1 < size - p; ++i)
            if (knots[i] != knots[i + 1]) first_dofs[e++] = i - p;
    }
    free(pts);
    free(knots);
    free(X);
    free(W);
    return 0;
}

/* band entry (i,j) of a kl/ku band with LAPACK factorisable layout (band_matrix.hpp:66-73) */
#define BAND(ab, ldab, kl, ku, i, j) ((ab)[(long)(j) * (ldab) + (kl) + (ku) + (i) - (j)])

/* form_matrix.cpp:8-24 (mass) and :26-42 (stiffness) */
int orc_form_band(int which, int p, int elements, int q, const double* btab, const double* w,
                  const double* J, const int* first_dofs, double* ab) {
    int n = elements + p;
    int ldab = 3 * p + 1;
    memset(ab, 0, sizeof(double) * ldab * n);
    int d = which ? 1 : 0;
    for (int e = 0; e < elements; ++e) {
        for (int k = 0; k < q; ++k) {
            int first = first_dofs[e];
            int last = first + p;
            const double* bv = btab + ((long)(e * q + k) * 2 + d) * (p + 1);
            for (int a = 0; a + first <= last; ++a) {
                for (int b = 0; b + first <= last; ++b) {
                    BAND(ab, ldab, p, p, a + first, b + first) += bv[a] * bv[b] * w[k] * J[e];
                }
            }
        }
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* LAPACK band LU (dgbtf2) and band solve (dgbtrs + dtbsv), restated from the */
/* published reference LAPACK algorithms. 1-based pivots.                     */
/* ------------------------------------------------------------------------ */
int orc_dgbtrf(int n, int kl, int ku, double* ab, int ldab, int* ipiv) {
    int kv = ku + kl;
    int info = 0;
    /* AB(r, c) 1-based -> ab[(c-1)*ldab + (r-1)] */
#define AB1(r, c) ab[(long)((c)-1) * ldab + ((r)-1)]
    for (int j = ku + 2; j <= (kv < n ? kv : n); ++j)
        for (int i = kv - j + 2; i <= kl; ++i) AB1(i, j) = 0;
    int ju = 1;
    for (int j = 1; j <= n; ++j) {
        if (j + kv <= n)
            for (int i = 1; i <= kl; ++i) AB1(i, j + kv) = 0;
        int km = kl < n - j ? kl : n - j;
        /* idamax over AB(kv+1 .. kv+1+km, j): first index of the largest |.| */
        int jp = 1;
        double best = fabs(AB1(kv + 1, j));
        for (int i = 2; i <= km + 1; ++i) {
            double v = fabs(AB1(kv + i, j));
            if (v > best) {
                best = v;
                jp = i;
            }
        }
        ipiv[j - 1] = jp + j - 1;
        if (AB1(kv + jp, j) != 0) {
            int cand = j + ku + jp - 1;
            if (cand > n) cand = n;
            if (cand > ju) ju = cand;
            if (jp != 1) {
                /* swap rows across columns j..ju (stride ldab-1 walks a matrix row) */
                for (int c = 0; c <= ju - j; ++c) {
                    double t = AB1(kv + jp - c, j + c);
                    AB1(kv + jp - c, j + c) = AB1(kv + 1 - c, j + c);
                    AB1(kv + 1 - c, j + c) = t;
                }
            }
            if (km > 0) {
                double r = 1.0 / AB1(kv + 1, j);
                for (int i = 1; i <= km; ++i) AB1(kv + 1 + i, j) *= r;
                if (ju > j) {
                    /* dger: A(kv+1+i-c, j+c) -= x(i) * y(c) */
                    for (int c = 1; c <= ju - j; ++c) {
                        double y = AB1(kv + 1 - c, j + c);
                        if (y != 0) {
                            double t = -y;
                            for (int i = 1; i <= km; ++i) AB1(kv + 1 + i - c, j + c) += AB1(kv + 1 + i, j) * t;
                        }
                    }
                }
            }
        } else if (info == 0) {
            info = j;
        }
    }
#undef AB1
    return info;
}

int orc_dgbtrs(char trans, int n, int kl, int ku, int nrhs, const double* ab, int ldab,
               const int* ipiv, double* b, int ldb) {
    int kd = ku + kl + 1;
    int k = kl + ku;
#define AB1(r, c) ab[(long)((c)-1) * ldab + ((r)-1)]
    if (trans == 'N' || trans == 'n') {
        for (int c = 0; c < nrhs; ++c) {
            double* x = b + (long)c * ldb;
            if (kl > 0) {
                for (int j = 1; j <= n - 1; ++j) {
                    int lm = kl < n - j ? kl : n - j;
                    int l = ipiv[j - 1];
                    if (l != j) {
                        double t = x[l - 1];
                        x[l - 1] = x[j - 1];
                        x[j - 1] = t;
                    }
                    double y = x[j - 1];
                    if (y != 0) {
                        double t = -y;
                        for (int i = 1; i <= lm; ++i) x[j - 1 + i] += AB1(kd + i, j) * t;
                    }
                }
            }
            /* dtbsv Upper, No transpose, Non-unit, bandwidth k */
            for (int j = n; j >= 1; --j) {
                if (x[j - 1] != 0) {
                    int l = k + 1 - j;
                    x[j - 1] = x[j - 1] / AB1(k + 1, j);
                    double t = x[j - 1];
                    int lo = j - k > 1 ? j - k : 1;
                    for (int i = j - 1; i >= lo; --i) x[i - 1] -= t * AB1(l + i, j);
                }
            }
        }
    } else {
        for (int c = 0; c < nrhs; ++c) {
            double* x = b + (long)c * ldb;
            /* dtbsv Upper, Transpose, Non-unit */
            for (int j = 1; j <= n; ++j) {
                double t = x[j - 1];
                int l = k + 1 - j;
                int lo = j - k > 1 ? j - k : 1;
                for (int i = lo; i <= j - 1; ++i) t -= AB1(l + i, j) * x[i - 1];
                t = t / AB1(k + 1, j);
                x[j - 1] = t;
            }
            if (kl > 0) {
                for (int j = n - 1; j >= 1; --j) {
                    int lm = kl < n - j ? kl : n - j;
                    /* dgemv 'T': x(j) += -sum_i AB(kd+i, j) * x(j+i) */
                    double t = 0;
                    for (int i = 1; i <= lm; ++i) t += x[j - 1 + i] * AB1(kd + i, j);
                    x[j - 1] += -t;
                    int l = ipiv[j - 1];
                    if (l != j) {
                        double s = x[l - 1];
                        x[l - 1] = x[j - 1];
                        x[j - 1] = s;
                    }
                }
            }
        }
    }
#undef AB1
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Problem setup (dimension.cpp:8-21, heat_3d::before -> prepare_matrices).   */
/* ------------------------------------------------------------------------ */
typedef struct {
    int p, elements, n, q, ldab;
    double *btab, *xq, *J, *w, *mass, *lu;
    int *first_dofs, *ipiv;
} orc_dim;

struct orc_problem {
    int ndim;
    orc_dim d[ORC_MAXD];
    long size;
};

orc_problem* orc_problem_create(int ndim, const int* p, const int* elements) {
    if (ndim < 1 || ndim > ORC_MAXD) return NULL;
    orc_problem* pr = (orc_problem*)calloc(1, sizeof(orc_problem));
    pr->ndim = ndim;
    pr->size = 1;
    for (int i = 0; i < ndim; ++i) {
        orc_dim* D = &pr->d[i];
        D->p = p[i];
        D->elements = elements[i];
        D->n = elements[i] + p[i];
        D->q = p[i] + 1;
        D->ldab = 3 * p[i] + 1;
        if (D->p < 1 || D->p > ORC_MAXP || D->elements < 1) {
            orc_problem_destroy(pr);
            return NULL;
        }
        int E = D->elements, Q = D->q, P1 = D->p + 1;
        D->btab = (double*)malloc(sizeof(double) * E * Q * 2 * P1);
        D->xq = (double*)malloc(sizeof(double) * E * Q);
        D->J = (double*)malloc(sizeof(double) * E);
        D->w = (double*)malloc(sizeof(double) * Q);
        D->first_dofs = (int*)malloc(sizeof(int) * E);
        D->mass = (double*)malloc(sizeof(double) * D->ldab * D->n);
        D->lu = (double*)malloc(sizeof(double) * D->ldab * D->n);
        D->ipiv = (int*)malloc(sizeof(int) * D->n);
        double* X = (double*)malloc(sizeof(double) * Q);
        orc_gauss(Q, X, D->w);
        free(X);
        orc_basis_tables(D->p, E, 0.0, 1.0, Q, D->btab, D->xq, D->J, D->first_dofs);
        orc_form_band(0, D->p, E, Q, D->btab, D->w, D->J, D->first_dofs, D->mass);
        memcpy(D->lu, D->mass, sizeof(double) * D->ldab * D->n);
        if (orc_dgbtrf(D->n, D->p, D->p, D->lu, D->ldab, D->ipiv) != 0) {
            orc_problem_destroy(pr);
            return NULL;
        }
        pr->size *= D->n;
    }
    return pr;
}

void orc_problem_destroy(orc_problem* pr) {
    if (!pr) return;
    for (int i = 0; i < ORC_MAXD; ++i) {
        orc_dim* D = &pr->d[i];
        free(D->btab);
        free(D->xq);
        free(D->J);
        free(D->w);
        free(D->first_dofs);
        free(D->mass);
        free(D->lu);
        free(D->ipiv);
    }
    free(pr);
}

int orc_problem_dofs(const orc_problem* pr, int d) { return (d >= 0 && d < pr->ndim) ? pr->d[d].n : 1; }
long orc_problem_size(const orc_problem* pr) { return pr->size; }

int orc_problem_dim(const orc_problem* pr, int d, double* btab, double* w, double* J,
                    int* first_dofs, double* mass_ab, double* lu_ab, int* ipiv) {
    if (d < 0 || d >= pr->ndim) return -2;
    const orc_dim* D = &pr->d[d];
    int E = D->elements, Q = D->q, P1 = D->p + 1;
    if (btab) memcpy(btab, D->btab, sizeof(double) * E * Q * 2 * P1);
    if (w) memcpy(w, D->w, sizeof(double) * Q);
    if (J) memcpy(J, D->J, sizeof(double) * E);
    if (first_dofs) memcpy(first_dofs, D->first_dofs, sizeof(int) * E);
    if (mass_ab) memcpy(mass_ab, D->mass, sizeof(double) * D->ldab * D->n);
    if (lu_ab) memcpy(lu_ab, D->lu, sizeof(double) * D->ldab * D->n);
    if (ipiv) memcpy(ipiv, D->ipiv, sizeof(int) * D->n);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Heat RHS (heat_3d.hpp:49-67; 2D heat_2d.hpp:80-106).                      */
/* Loop order of util/iter/product.hpp: the last index runs fastest, so     */
/* elements, quadrature points and dofs iterate with z (or y in 2D) inner.  */
/* ------------------------------------------------------------------------ */
#define BT(D_, e_, q_, d_, a_) ((D_)->btab[(((long)(e_) * (D_)->q + (q_)) * 2 + (d_)) * ((D_)->p + 1) + (a_)])

/* One element's contribution; accumulates into out (global rhs when local==0,
 * else an element tile of (p+1)^ndim entries, x fastest). kappa may be NULL. */
static void heat_element(const orc_problem* pr, const int* e, const double* u_prev,
                         const double* kappa, double dt, double* out, int local) {
    const orc_dim* X = &pr->d[0];
    if (pr->ndim == 3) {
        const orc_dim* Y = &pr->d[1];
        const orc_dim* Z = &pr->d[2];
        long nx = X->n, ny = Y->n;
        int fx = X->first_dofs[e[0]], fy = Y->first_dofs[e[1]], fz = Z->first_dofs[e[2]];
        int px = X->p, py = Y->p, pz = Z->p;
        double J = X->J[e[0]] * Y->J[e[1]] * Z->J[e[2]];
        for (int qx = 0; qx < X->q; ++qx)
            for (int qy = 0; qy < Y->q; ++qy)
                for (int qz = 0; qz < Z->q; ++qz) {
                    double w = X->w[qx] * Y->w[qy] * Z->w[qz];
                    /* eval_fun (simulation_3d.hpp:120-128) */
                    double uv = 0, ux = 0, uy = 0, uz = 0, kv = 0;
                    for (int bx = 0; bx <= px; ++bx)
                        for (int by = 0; by <= py; ++by)
                            for (int bz = 0; bz <= pz; ++bz) {
                                long g = (fx + bx) + nx * ((fy + by) + ny * (long)(fz + bz));
                                double c = u_prev[g];
                                double B1 = BT(X, e[0], qx, 0, bx), B2 = BT(Y, e[1], qy, 0, by),
                                       B3 = BT(Z, e[2], qz, 0, bz);
                                double dB1 = BT(X, e[0], qx, 1, bx), dB2 = BT(Y, e[1], qy, 1, by),
                                       dB3 = BT(Z, e[2], qz, 1, bz);
                                double v = B1 * B2 * B3;
                                uv += c * v;
                                ux += c * (dB1 * B2 * B3);
                                uy += c * (B1 * dB2 * B3);
                                uz += c * (B1 * B2 * dB3);
                                if (kappa) kv += kappa[g] * v;
                            }
                    double kd = kappa ? dt * kv : dt;
                    for (int ax = 0; ax <= px; ++ax)
                        for (int ay = 0; ay <= py; ++ay)
                            for (int az = 0; az <= pz; ++az) {
                                double B1 = BT(X, e[0], qx, 0, ax), B2 = BT(Y, e[1], qy, 0, ay),
                                       B3 = BT(Z, e[2], qz, 0, az);
                                double dB1 = BT(X, e[0], qx, 1, ax), dB2 = BT(Y, e[1], qy, 1, ay),
                                       dB3 = BT(Z, e[2], qz, 1, az);
                                double v = B1 * B2 * B3;
                                double vx = dB1 * B2 * B3, vy = B1 * dB2 * B3, vz = B1 * B2 * dB3;
                                double gp = ux * vx + uy * vy + uz * vz;
                                double val = uv * v - kd * gp;
                                long idx = local ? ax + (px + 1) * (ay + (py + 1) * (long)az)
                                                 : (fx + ax) + nx * ((fy + ay) + ny * (long)(fz + az));
                                out[idx] += val * w * J;
                            }
                }
    } else if (pr->ndim == 2) {
        const orc_dim* Y = &pr->d[1];
        long nx = X->n;
        int fx = X->first_dofs[e[0]], fy = Y->first_dofs[e[1]];
        int px = X->p, py = Y->p;
        double J = X->J[e[0]] * Y->J[e[1]];
        for (int qx = 0; qx < X->q; ++qx)
            for (int qy = 0; qy < Y->q; ++qy) {
                double w = X->w[qx] * Y->w[qy];
                double uv = 0, ux = 0, uy = 0, kv = 0;
                for (int bx = 0; bx <= px; ++bx)
                    for (int by = 0; by <= py; ++by) {
                        long g = (fx + bx) + nx * (long)(fy + by);
                        double c = u_prev[g];
                        double B1 = BT(X, e[0], qx, 0, bx), B2 = BT(Y, e[1], qy, 0, by);
                        double dB1 = BT(X, e[0], qx, 1, bx), dB2 = BT(Y, e[1], qy, 1, by);
                        double v = B1 * B2;
                        uv += c * v;
                        ux += c * (dB1 * B2);
                        uy += c * (B1 * dB2);
                        if (kappa) kv += kappa[g] * v;
                    }
                double kd = kappa ? dt * kv : dt;
                for (int ax = 0; ax <= px; ++ax)
                    for (int ay = 0; ay <= py; ++ay) {
                        double B1 = BT(X, e[0], qx, 0, ax), B2 = BT(Y, e[1], qy, 0, ay);
                        double dB1 = BT(X, e[0], qx, 1, ax), dB2 = BT(Y, e[1], qy, 1, ay);
                        double v = B1 * B2;
                        double gp = ux * (dB1 * B2) + uy * (B1 * dB2);
                        double val = uv * v - kd * gp;
                        long idx = local ? ax + (px + 1) * (long)ay : (fx + ax) + nx * (long)(fy + ay);
                        out[idx] += val * w * J;
                    }
            }
    } else {
        int fx = X->first_dofs[e[0]];
        int px = X->p;
        double J = X->J[e[0]];
        for (int qx = 0; qx < X->q; ++qx) {
            double w = X->w[qx];
            double uv = 0, ux = 0, kv = 0;
            for (int bx = 0; bx <= px; ++bx) {
                double c = u_prev[fx + bx];
                uv += c * BT(X, e[0], qx, 0, bx);
                ux += c * BT(X, e[0], qx, 1, bx);
                if (kappa) kv += kappa[fx + bx] * BT(X, e[0], qx, 0, bx);
            }
            double kd = kappa ? dt * kv : dt;
            for (int ax = 0; ax <= px; ++ax) {
                double val = uv * BT(X, e[0], qx, 0, ax) - kd * (ux * BT(X, e[0], qx, 1, ax));
                out[local ? ax : fx + ax] += val * w * J;
            }
        }
    }
}

static long n_elements(const orc_problem* pr) {
    long ne = 1;
    for (int i = 0; i < pr->ndim; ++i) ne *= pr->d[i].elements;
    return ne;
}

/* element linear id -> (ex, ey, ez) with the LAST index fastest (product.hpp:103-123) */
static void element_of(const orc_problem* pr, long id, int* e) {
    for (int i = pr->ndim - 1; i >= 0; --i) {
        e[i] = (int)(id % pr->d[i].elements);
        id /= pr->d[i].elements;
    }
}

static int heat_rhs_seq(const orc_problem* pr, const double* u_prev, const double* kappa,
                        double* rhs, double dt) {
    memset(rhs, 0, sizeof(double) * pr->size);
    long ne = n_elements(pr);
    int e[ORC_MAXD];
    for (long id = 0; id < ne; ++id) {
        element_of(pr, id, e);
        heat_element(pr, e, u_prev, kappa, dt, rhs, 0);
    }
    return 0;
}

int orc_heat_rhs(const orc_problem* pr, const double* u_prev, double* rhs, double dt) {
    return heat_rhs_seq(pr, u_prev, NULL, rhs, dt);
}

int orc_heat_rhs_kappa(const orc_problem* pr, const double* u_prev, const double* kappa,
                       double* rhs, double dt) {
    return heat_rhs_seq(pr, u_prev, kappa, rhs, dt);
}

/* ------------------------------------------------------------------------ */
/* General pointwise form of the element loop, the pattern the reference's  */
/* other problems share: scalability_3d::compute_rhs (examples/scalability/ */
/* test3d.hpp:66-95: val = u v - dt (grad u . grad v - f(x)), the forcing   */
/* added without a test function) and flow::compute_rhs (examples/flow/     */
/* flow.hpp:77-98: (u v + dt (-k e^{mi u} grad u . grad v + h v)) w J).     */
/* Per Gauss point: val = A u v + B grad u . grad v + G v + D, each of A, B, */
/* G, D a constant plus an optional point field (Gauss grid, x fastest over  */
/* e_d q + k_d).  2D and 3D; loops in the reference's order.                */
/* ------------------------------------------------------------------------ */
static double pf(double c, const double* f, long pq) { return f ? c + f[pq] : c; }

int orc_form_rhs(const orc_problem* pr, const double* u, const double* cst, const double* aq, const double* bq,
                 const double* gq, const double* dq, double* rhs) {
    if (pr->ndim < 2) return -1;
    memset(rhs, 0, sizeof(double) * pr->size);
    const orc_dim* X = &pr->d[0];
    const orc_dim* Y = &pr->d[1];
    const orc_dim* Z = pr->ndim == 3 ? &pr->d[2] : NULL;
    const long nx = X->n, ny = Y->n;
    const long Qx = (long)X->elements * X->q, Qy = (long)Y->elements * Y->q;
    const int ez_n = Z ? Z->elements : 1, qz_n = Z ? Z->q : 1, pz = Z ? Z->p : 0;
    for (int ex = 0; ex < X->elements; ++ex)
        for (int ey = 0; ey < Y->elements; ++ey)
            for (int ez = 0; ez < ez_n; ++ez) {
                const int fx = X->first_dofs[ex], fy = Y->first_dofs[ey], fz = Z ? Z->first_dofs[ez] : 0;
                const double J = X->J[ex] * Y->J[ey] * (Z ? Z->J[ez] : 1.0);
                for (int qx = 0; qx < X->q; ++qx)
                    for (int qy = 0; qy < Y->q; ++qy)
                        for (int qz = 0; qz < qz_n; ++qz) {
                            const double w = X->w[qx] * Y->w[qy] * (Z ? Z->w[qz] : 1.0);
                            const long pq = ((long)ex * X->q + qx) +
                                            Qx * (((long)ey * Y->q + qy) + Qy * ((long)ez * qz_n + qz));
                            const double A = pf(cst[0], aq, pq), B = pf(cst[1], bq, pq), G = pf(cst[2], gq, pq),
                                         D = pf(cst[3], dq, pq);
                            double uv = 0, ux = 0, uy = 0, uz = 0;
                            if (u)
                                for (int bx = 0; bx <= X->p; ++bx)
                                    for (int by = 0; by <= Y->p; ++by)
                                        for (int bz = 0; bz <= pz; ++bz) {
                                            const long g = (fx + bx) + nx * ((fy + by) + ny * (long)(fz + bz));
                                            const double B1 = BT(X, ex, qx, 0, bx), B2 = BT(Y, ey, qy, 0, by);
                                            const double dB1 = BT(X, ex, qx, 1, bx), dB2 = BT(Y, ey, qy, 1, by);
                                            const double B3 = Z ? BT(Z, ez, qz, 0, bz) : 1.0;
                                            const double dB3 = Z ? BT(Z, ez, qz, 1, bz) : 0.0;
                                            uv += u[g] * (B1 * B2 * B3);
                                            ux += u[g] * (dB1 * B2 * B3);
                                            uy += u[g] * (B1 * dB2 * B3);
                                            uz += u[g] * (B1 * B2 * dB3);
                                        }
                            for (int ax = 0; ax <= X->p; ++ax)
                                for (int ay = 0; ay <= Y->p; ++ay)
                                    for (int az = 0; az <= pz; ++az) {
                                        const double B1 = BT(X, ex, qx, 0, ax), B2 = BT(Y, ey, qy, 0, ay);
                                        const double dB1 = BT(X, ex, qx, 1, ax), dB2 = BT(Y, ey, qy, 1, ay);
                                        const double B3 = Z ? BT(Z, ez, qz, 0, az) : 1.0;
                                        const double dB3 = Z ? BT(Z, ez, qz, 1, az) : 0.0;
                                        const double v = B1 * B2 * B3;
                                        const double gp = ux * (dB1 * B2 * B3) + uy * (B1 * dB2 * B3) + uz * (B1 * B2 * dB3);
                                        const double val = A * uv * v + B * gp + G * v + D;
                                        rhs[(fx + ax) + nx * ((fy + ay) + ny * (long)(fz + az))] += val * w * J;
                                    }
                        }
            }
    return 0;
}

/* ---- executor stand-in: for_each over elements + synchronized scatter ---- */
typedef struct {
    const orc_problem* pr;
    const double* u_prev;
    double* rhs;
    double dt;
    long ne;
    long next;
    pthread_mutex_t work_lock;
    pthread_mutex_t scatter_lock; /* galois_executor::synchronized (galois.hpp:27-32) */
} mt_job;

static void* mt_worker(void* arg) {
    mt_job* job = (mt_job*)arg;
    const orc_problem* pr = job->pr;
    long tile = 1;
    for (int i = 0; i < pr->ndim; ++i) tile *= pr->d[i].p + 1;
    double* U = (double*)malloc(sizeof(double) * tile);
    int e[ORC_MAXD];
    const long chunk = 16;
    for (;;) {
        pthread_mutex_lock(&job->work_lock);
        long begin = job->next;
        job->next += chunk;
        pthread_mutex_unlock(&job->work_lock);
        if (begin >= job->ne) break;
        long end = begin + chunk < job->ne ? begin + chunk : job->ne;
        for (long id = begin; id < end; ++id) {
            element_of(pr, id, e);
            memset(U, 0, sizeof(double) * tile);
            heat_element(pr, e, job->u_prev, NULL, job->dt, U, 1);
            /* update_global_rhs (simulation_3d.hpp:140-145) under the lock */
            pthread_mutex_lock(&job->scatter_lock);
            const orc_dim* X = &pr->d[0];
            int px = X->p;
            int fx = X->first_dofs[e[0]];
            if (pr->ndim == 3) {
                const orc_dim* Y = &pr->d[1];
                const orc_dim* Z = &pr->d[2];
                long nx = X->n, ny = Y->n;
                int fy = Y->first_dofs[e[1]], fz = Z->first_dofs[e[2]];
                for (int ax = 0; ax <= px; ++ax)
                    for (int ay = 0; ay <= Y->p; ++ay)
                        for (int az = 0; az <= Z->p; ++az)
                            job->rhs[(fx + ax) + nx * ((fy + ay) + ny * (long)(fz + az))] +=
                                U[ax + (px + 1) * (ay + (Y->p + 1) * (long)az)];
            } else if (pr->ndim == 2) {
                const orc_dim* Y = &pr->d[1];
                long nx = X->n;
                int fy = Y->first_dofs[e[1]];
                for (int ax = 0; ax <= px; ++ax)
                    for (int ay = 0; ay <= Y->p; ++ay)
                        job->rhs[(fx + ax) + nx * (long)(fy + ay)] += U[ax + (px + 1) * (long)ay];
            } else {
                for (int ax = 0; ax <= px; ++ax) job->rhs[fx + ax] += U[ax];
            }
            pthread_mutex_unlock(&job->scatter_lock);
        }
    }
    free(U);
    return NULL;
}

int orc_heat_rhs_mt(const orc_problem* pr, const double* u_prev, double* rhs, double dt,
                    int nthreads) {
    if (nthreads <= 1) return orc_heat_rhs(pr, u_prev, rhs, dt);
    memset(rhs, 0, sizeof(double) * pr->size);
    mt_job job;
    job.pr = pr;
    job.u_prev = u_prev;
    job.rhs = rhs;
    job.dt = dt;
    job.ne = n_elements(pr);
    job.next = 0;
    pthread_mutex_init(&job.work_lock, NULL);
    pthread_mutex_init(&job.scatter_lock, NULL);
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * nthreads);
    for (int t = 0; t < nthreads; ++t) pthread_create(&th[t], NULL, mt_worker, &job);
    for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
    free(th);
    pthread_mutex_destroy(&job.work_lock);
    pthread_mutex_destroy(&job.scatter_lock);
    return 0;
}

/* Adjoint support (no reference counterpart): g_c += -dt sum_e sum_q W B_c(x_q)
 * grad u(x_q) . grad mu(x_q), the derivative of mu^T R(kappa) u with respect to
 * the kappa coefficients, element by element in the reference loop order. */
int orc_kappa_grad(const orc_problem* pr, const double* u, const double* mu, double* g, double dt) {
    if (pr->ndim < 2) return -1;
    long ne = n_elements(pr);
    int e[ORC_MAXD];
    for (long id = 0; id < ne; ++id) {
        element_of(pr, id, e);
        const orc_dim* X = &pr->d[0];
        const orc_dim* Y = &pr->d[1];
        const orc_dim* Z = pr->ndim == 3 ? &pr->d[2] : NULL;
        int nz = Z ? Z->p + 1 : 1, qzn = Z ? Z->q : 1;
        long nx = X->n, ny = Y->n;
        int fx = X->first_dofs[e[0]], fy = Y->first_dofs[e[1]], fz = Z ? Z->first_dofs[e[2]] : 0;
        double J = X->J[e[0]] * Y->J[e[1]] * (Z ? Z->J[e[2]] : 1.0);
        for (int qx = 0; qx < X->q; ++qx)
            for (int qy = 0; qy < Y->q; ++qy)
                for (int qz = 0; qz < qzn; ++qz) {
                    double w = X->w[qx] * Y->w[qy] * (Z ? Z->w[qz] : 1.0);
                    double gu[3] = {0, 0, 0}, gm[3] = {0, 0, 0};
                    for (int bx = 0; bx <= X->p; ++bx)
                        for (int by = 0; by <= Y->p; ++by)
                            for (int bz = 0; bz < nz; ++bz) {
                                long gi = (fx + bx) + nx * ((fy + by) + ny * (long)(fz + bz));
                                double B1 = BT(X, e[0], qx, 0, bx), B2 = BT(Y, e[1], qy, 0, by);
                                double dB1 = BT(X, e[0], qx, 1, bx), dB2 = BT(Y, e[1], qy, 1, by);
                                double B3 = Z ? BT(Z, e[2], qz, 0, bz) : 1.0, dB3 = Z ? BT(Z, e[2], qz, 1, bz) : 0.0;
                                double v[3] = {dB1 * B2 * B3, B1 * dB2 * B3, B1 * B2 * dB3};
                                for (int k = 0; k < 3; ++k) {
                                    gu[k] += u[gi] * v[k];
                                    gm[k] += mu[gi] * v[k];
                                }
                            }
                    double sdot = (gu[0] * gm[0] + gu[1] * gm[1] + gu[2] * gm[2]) * w * J * (-dt);
                    for (int ax = 0; ax <= X->p; ++ax)
                        for (int ay = 0; ay <= Y->p; ++ay)
                            for (int az = 0; az < nz; ++az) {
                                double B = BT(X, e[0], qx, 0, ax) * BT(Y, e[1], qy, 0, ay) * (Z ? BT(Z, e[2], qz, 0, az) : 1.0);
                                g[(fx + ax) + nx * ((fy + ay) + ny * (long)(fz + az))] += sdot * B;
                            }
                }
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* ADS solve (solver.hpp:35-41, 149-160, 199-203). The reference solves all  */
/* lines of the leading dimension with one dgbtrs (nrhs = size/n0) and then  */
/* cyclically transposes; the transposes only move data, so solving each    */
/* line of each direction in place performs the same arithmetic per line.   */
/* ------------------------------------------------------------------------ */
static int ads_solve_impl(const orc_problem* pr, double* rhs, char trans) {
    int nd = pr->ndim;
    long n[ORC_MAXD] = {1, 1, 1};
    for (int i = 0; i < nd; ++i) n[i] = pr->d[i].n;
    long maxn = 0;
    for (int i = 0; i < nd; ++i)
        if (n[i] > maxn) maxn = n[i];
    double* line = (double*)malloc(sizeof(double) * maxn);
    for (int d = 0; d < nd; ++d) {
        const orc_dim* D = &pr->d[d];
        long stride = 1;
        for (int i = 0; i < d; ++i) stride *= n[i];
        long nlines = pr->size / n[d];
        if (d == 0) {
            orc_dgbtrs(trans, D->n, D->p, D->p, (int)nlines, D->lu, D->ldab, D->ipiv, rhs, D->n);
            continue;
        }
        for (long l = 0; l < nlines; ++l) {
            long lo = l % stride, hi = l / stride;
            long base = lo + hi * stride * n[d];
            for (long t = 0; t < n[d]; ++t) line[t] = rhs[base + t * stride];
            orc_dgbtrs(trans, D->n, D->p, D->p, 1, D->lu, D->ldab, D->ipiv, line, D->n);
            for (long t = 0; t < n[d]; ++t) rhs[base + t * stride] = line[t];
        }
    }
    free(line);
    return 0;
}

int orc_ads_solve(const orc_problem* pr, double* rhs) { return ads_solve_impl(pr, rhs, 'N'); }
int orc_ads_solve_t(const orc_problem* pr, double* rhs) { return ads_solve_impl(pr, rhs, 'T'); }

int orc_heat_steps(const orc_problem* pr, double* u, double dt, int nsteps, int nthreads) {
    double* prev = (double*)malloc(sizeof(double) * pr->size);
    for (int s = 0; s < nsteps; ++s) {
        memcpy(prev, u, sizeof(double) * pr->size); /* swap(u, u_prev) */
        if (nthreads > 1)
            orc_heat_rhs_mt(pr, prev, u, dt, nthreads);
        else
            orc_heat_rhs(pr, prev, u, dt);
        orc_ads_solve(pr, u);
    }
    free(prev);
    return 0;
}

/* projection.hpp:55-107: rhs(idx) += f(x) * B * w * J, B = prod_d b[e_d][q_d][0][a_d] */
int orc_projection_sin(const orc_problem* pr, double* out) {
    const double pi = 3.14159265358979323846;
    memset(out, 0, sizeof(double) * pr->size);
    int nd = pr->ndim;
    long ne = n_elements(pr);
    int e[ORC_MAXD];
    for (long id = 0; id < ne; ++id) {
        element_of(pr, id, e);
        double J = 1;
        for (int i = 0; i < nd; ++i) J *= pr->d[i].J[e[i]];
        long nq = 1;
        for (int i = 0; i < nd; ++i) nq *= pr->d[i].q;
        for (long qi = 0; qi < nq; ++qi) {
            int q[ORC_MAXD];
            long t = qi;
            for (int i = nd - 1; i >= 0; --i) {
                q[i] = (int)(t % pr->d[i].q);
                t /= pr->d[i].q;
            }
            double w = 1, f = 1;
            for (int i = 0; i < nd; ++i) w *= pr->d[i].w[q[i]];
            for (int i = 0; i < nd; ++i) f *= sin(pi * pr->d[i].xq[e[i] * pr->d[i].q + q[i]]);
            long na = 1;
            for (int i = 0; i < nd; ++i) na *= pr->d[i].p + 1;
            for (long ai = 0; ai < na; ++ai) {
                int a[ORC_MAXD];
                long s = ai;
                for (int i = nd - 1; i >= 0; --i) {
                    a[i] = (int)(s % (pr->d[i].p + 1));
                    s /= pr->d[i].p + 1;
                }
                double B = 1;
                long idx = 0, stride = 1;
                for (int i = 0; i < nd; ++i) {
                    B *= BT(&pr->d[i], e[i], q[i], 0, a[i]);
                    idx += (pr->d[i].first_dofs[e[i]] + a[i]) * stride;
                    stride *= pr->d[i].n;
                }
                out[idx] += f * B * w * J;
            }
        }
    }
    return 0;
}
