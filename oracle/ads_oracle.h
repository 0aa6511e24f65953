/*
 * CPU oracle for the explicit heat step of IGA-ADS: a plain C restatement of
 * the reference algorithm, used ONLY as a checker (tests, the smoke check and
 * the CPU-baseline leg of the benchmark).  No product code links it.
 *
 * Parity pin: the restatement is checked against the reference's own compiled
 * code (oracle/_ref, built from the reference sources by oracle/Makefile) and
 * against the known answers in the reference tests (tests/ads/solver_test.cpp,
 * tests/ads/lin/band_solve_test.cpp), through the golden fixtures committed in
 * tests/golden/.
 *
 * Layout conventions follow the reference:
 *  - tensors are x-fastest: u[i + nx*(j + ny*k)]  (util/multi_array/ordering/reverse.hpp:27-31)
 *  - basis tables b[e][q][d][a] flattened as ((e*Q + q)*2 + d)*(p+1) + a  (basis_data.hpp:35)
 *  - band matrices in LAPACK band storage with ldab = 2*kl+ku+1, entry (i,j) at
 *    (kl+ku+i-j) + j*ldab  (lin/band_matrix.hpp:66-73, row_offset = kl)
 *  - pivots are 1-based as produced by dgbtrf.
 */
#ifndef ADS_ORACLE_H
#define ADS_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- 1D building blocks ------------------------------------------------ */

/* Gauss-Legendre nodes/weights on [-1,1], q in [2,64] (quad/gauss.hpp tables). */
int orc_gauss(int q, double* x, double* w);

/* Knot vector of create_basis(a, b, p, elements, repeated_nodes=0)
 * (bspline.cpp:26-43); knots has elements + 2p + 1 entries. */
int orc_knots(int p, int elements, double a, double b, double* knots);

/* basis_data(B, derivatives=1, q, elem_division=1) (basis_data.cpp:63-114):
 * btab [E][q][2][p+1], xq [E][q], J [E], first_dofs [E]. */
int orc_basis_tables(int p, int elements, double a, double b, int q, double* btab, double* xq,
                     double* J, int* first_dofs);

/* gram_matrix_1d / stiffness_matrix_1d (form_matrix.cpp:8-42) into LAPACK band
 * storage with kl = ku = p, ldab = 3p+1 (the factorisable layout). which=0: mass,
 * which=1: stiffness. */
int orc_form_band(int which, int p, int elements, int q, const double* btab, const double* w,
                  const double* J, const int* first_dofs, double* ab);

/* Banded LU with partial pivoting: LAPACK dgbtf2 algorithm, the path dgbtrf
 * takes for kl < 32 (lin/band_solve.hpp:16-18 -> dgbtrf_). Returns info. */
int orc_dgbtrf(int n, int kl, int ku, double* ab, int ldab, int* ipiv);

/* LAPACK dgbtrs: trans 'N' or 'T' (lin/band_solve.hpp:20-31). */
int orc_dgbtrs(char trans, int n, int kl, int ku, int nrhs, const double* ab, int ldab,
               const int* ipiv, double* b, int ldb);

/* ---- the simulation ----------------------------------------------------- */

typedef struct orc_problem orc_problem;

/* A 1-, 2- or 3-D tensor-product problem on [0,1]^ndim with open uniform knots,
 * quad_order = p+1 per dimension (dim_config defaults, config.hpp:11-29), the
 * mass matrix of every dimension assembled and factorised as in
 * heat_3d::before -> prepare_matrices (heat_3d.hpp:31-37). */
orc_problem* orc_problem_create(int ndim, const int* p, const int* elements);
void orc_problem_destroy(orc_problem* pr);
int orc_problem_dofs(const orc_problem* pr, int d);
long orc_problem_size(const orc_problem* pr);

/* Copy out dimension d's tables (any pointer may be NULL). */
int orc_problem_dim(const orc_problem* pr, int d, double* btab, double* w, double* J,
                    int* first_dofs, double* mass_ab, double* lu_ab, int* ipiv);

/* heat_3d::compute_rhs (heat_3d.hpp:49-67) / heat_2d (heat_2d.hpp:80-106),
 * with eval_fun hoisted out of the dof loop as in scalability/test3d.hpp:79
 * (same arithmetic).  Sequential, in the reference's loop order. */
int orc_heat_rhs(const orc_problem* pr, const double* u_prev, double* rhs, double dt);

/* The same RHS with the executor pattern (for_each over elements + a local
 * element tile + synchronized scatter, executor/galois.hpp:27-44 with
 * heat_2d.hpp:86-104), on nthreads host threads. */
int orc_heat_rhs_mt(const orc_problem* pr, const double* u_prev, double* rhs, double dt,
                    int nthreads);

/* heat RHS with a diffusion coefficient field kappa given as spline
 * coefficients on the same basis: u.v - dt * kappa(x_q) grad u . grad v.
 * Reduces to orc_heat_rhs for kappa == 1. */
int orc_heat_rhs_kappa(const orc_problem* pr, const double* u_prev, const double* kappa,
                       double* rhs, double dt);
/* General pointwise form (scalability test3d.hpp:66-95, flow.hpp:77-98):
 * rhs_a = sum_e sum_q w J [A u v_a + B grad u . grad v_a + G v_a + D], with
 * cst = {A, B, G, D} constants and aq..dq optional Gauss-point fields added
 * to them (NULL = none).  u may be NULL (then the u terms vanish).  2D/3D. */
int orc_form_rhs(const orc_problem* pr, const double* u, const double* cst, const double* aq, const double* bq,
                 const double* gq, const double* dq, double* rhs);

/* Adjoint support (no reference counterpart): g += mu^T (dR/dkappa) u, i.e.
 * g_c += -dt sum_e sum_q w J B_c(x_q) grad u . grad mu at the quadrature points. */
int orc_kappa_grad(const orc_problem* pr, const double* u, const double* mu, double* g, double dt);

/* ads_solve(rhs, buf, x.data(), y.data(), z.data()) (solver.hpp:149-160,
 * 199-203): one dgbtrs per grid line, direction by direction; result in rhs. */
int orc_ads_solve(const orc_problem* pr, double* rhs);

/* The adjoint-direction solve: M^T in every dimension (dgbtrs 'T'). */
int orc_ads_solve_t(const orc_problem* pr, double* rhs);

/* simulation_base::run's loop (simulation_base.cpp:11-20) with heat_3d's
 * before_step/step (heat_3d.hpp:39-47): nsteps x (swap, compute_rhs, solve).
 * nthreads <= 1 uses the sequential RHS. u holds the state in and out. */
int orc_heat_steps(const orc_problem* pr, double* u, double dt, int nsteps, int nthreads);

/* compute_projection (projection.hpp:55-107, 148-153) of
 * f = prod_d sin(pi x_d) into out (not solved; apply orc_ads_solve after). */
int orc_projection_sin(const orc_problem* pr, double* out);

#ifdef __cplusplus
}
#endif

#endif
