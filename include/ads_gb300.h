/*
 * ads_gb300.h -- C-ABI of the GB300 (sm_103a) explicit-step engine for
 * IGA-ADS: Gauss-quadrature heat RHS assembly over tensor-product B-spline
 * elements and the alternating-directions (Kronecker) banded mass solve.
 *
 * Conventions shared by every entry point:
 *  - plain C types only; every function returns an int status:
 *      0                   success
 *      -k  (k >= 1)        the k-th argument is invalid (LAPACK's convention)
 *      ADSG_ERR_* (> 0)    runtime or numerical failure; adsg_last_error()
 *                          returns a message for the calling thread
 *  - tensors are x-fastest: u[i + nx*(j + ny*k)], the layout of ads::lin::tensor
 *    (reference include/ads/util/multi_array/ordering/reverse.hpp:27-31);
 *  - band matrices use LAPACK band storage (dgbtrf/dgbtrs layout): entry (i,j)
 *    of a kl/ku band is ab[(kl+ku+i-j) + j*ldab], ldab >= 2*kl+ku+1
 *    (reference include/ads/lin/band_matrix.hpp:66-73 with row_offset = kl);
 *    pivots are 1-based as dgbtrf writes them;
 *  - "_dev" pointers are device (HBM) addresses; everything else is host memory.
 *    Device work runs on the context's stream and is asynchronous unless the
 *    function's comment says it synchronises.
 *
 * A context is not thread-safe: use one context per host thread, or serialise.
 */
#ifndef ADS_GB300_H
#define ADS_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define ADSG_ERR_CUDA 1001      /* a CUDA runtime call failed */
#define ADSG_ERR_NOMEM 1002     /* host or device allocation failed */
#define ADSG_ERR_SINGULAR 1003  /* zero pivot in a band factorisation */
#define ADSG_ERR_DEVICE 1004    /* a kernel reported an error word (bounds, timeout) */
#define ADSG_ERR_UNSUPPORTED 1005

/* Maximum degree handled by the device kernels. */
#define ADSG_MAX_DEGREE 8

typedef struct adsg_ctx adsg_ctx;
typedef struct adsg_dim adsg_dim;

/* ---- one dimension: the data of ads::dimension -------------------------
 * Replaces what reference include/ads/simulation/dimension.hpp:20-59 holds:
 * basis_data tables (basis_data.hpp:21-86, derivatives = 1) and the
 * factorised mass matrix with its pivots (dim_data{M, ctx}, solver.hpp:17-20).
 */
typedef struct adsg_dim_desc {
    int p;                  /* B-spline degree */
    int elements;           /* number of elements */
    int quad_order;         /* Gauss points per element */
    int n;                  /* number of dofs */
    const double* btab;     /* [elements][quad_order][2][p+1]: b[e][q][d][a] */
    const double* w;        /* [quad_order] Gauss weights on [-1,1] */
    const double* J;        /* [elements] element Jacobians (x2-x1)/2 */
    const int* first_dofs;  /* [elements] basis_data::first_dofs */
    int kl, ku, ldab;       /* band parameters of the factorised matrix */
    const double* lu;       /* dgbtrf output, ldab*n doubles */
    const int* ipiv;        /* [n] 1-based pivots */
    const double* xq;       /* [elements][quad_order] Gauss points (basis_data::x);
                               optional (NULL): only adsg_quad_points needs it */
} adsg_dim_desc;

/* Build a dimension on the host exactly as the reference's dimension ctor
 * does (dimension.cpp:8-21 -> bspline::create_basis, basis_data,
 * gram_matrix_1d) and factorise its mass matrix (dimension::factorize_matrix,
 * dimension.hpp:52 -> dgbtrf).  Open uniform knots on [a, b],
 * repeated_nodes = 0.  quad_order <= 0 means p + 1.  No GPU needed. */
int adsg_dim_create(int p, int elements, double a, double b, int quad_order, adsg_dim** out);
void adsg_dim_destroy(adsg_dim* d);
/* Descriptor pointing into d's arrays (valid while d lives). */
int adsg_dim_describe(const adsg_dim* d, adsg_dim_desc* out);
/* dimension::fix_dof (dimension.cpp:23-29): identity row k in M, then the
 * matrix is refactorised.  Affects only the solve, as in the reference. */
int adsg_dim_fix_dof(adsg_dim* d, int k);
/* Unfactorised 1D mass (which = 0, gram_matrix_1d, form_matrix.cpp:8-24) or
 * stiffness (which = 1, stiffness_matrix_1d, form_matrix.cpp:26-42) band with
 * kl = ku = p in the layout above (ldab = 3p+1). ab has (3p+1)*n doubles. */
int adsg_dim_form_band(const adsg_dim* d, int which, double* ab);

/* ---- contexts ------------------------------------------------------------
 * A context owns the device copies of ndim (1..3) dimension descriptors, the
 * 1D mass/stiffness bands derived from their quadrature tables, scratch
 * tensors and a CUDA stream.  The host descriptors may be freed afterwards.
 * The context's own stream is a blocking stream: it is ordered with work on
 * the legacy default stream (e.g. torch's default stream). */
int adsg_ctx_create(int ndim, const adsg_dim_desc* dims, adsg_ctx** out);
int adsg_ctx_destroy(adsg_ctx* ctx);
/* Number of dofs of the whole tensor (product of the dimension sizes). */
long long adsg_ctx_size(const adsg_ctx* ctx);
/* Make the context enqueue on an existing cudaStream_t (NULL: its own). */
int adsg_ctx_set_stream(adsg_ctx* ctx, void* cuda_stream);
/* Wait for all work of the context and report any device error word. */
int adsg_ctx_synchronize(adsg_ctx* ctx);
/* Thread-local message describing the last failure (never NULL). */
const char* adsg_last_error(void);

/* ---- the hot path (device buffers) ---------------------------------------- */

/* heat_3d::compute_rhs (reference examples/heat/heat_3d.hpp:49-67; 2D:
 * heat_2d.hpp:80-106): rhs_a = sum_e sum_q w_q J_e (u v_a - dt grad u . grad v_a)
 * with u from u_prev.  Computed by the factored quadrature: the tensor-product
 * Gauss rule and the separable Jacobian make the element sum equal to
 * (Mx(x)My(x)Mz - dt (Kx(x)My(x)Mz + Mx(x)Ky(x)Mz + Mx(x)My(x)Kz)) u_prev with the
 * 1D quadrature-assembled mass/stiffness bands.  u_prev and rhs must not alias. */
int adsg_heat_rhs(adsg_ctx* ctx, const double* u_prev_dev, double* rhs_dev, double dt);

/* The same RHS by element-wise sum-factorised quadrature over the basis
 * tables, optionally with a diffusion field kappa given as spline
 * coefficients on the same space (kappa_dev may be NULL for kappa = 1):
 * rhs_a = sum_e sum_q w J (u v_a - dt kappa(x_q) grad u . grad v_a). */
int adsg_heat_rhs_elem(adsg_ctx* ctx, const double* u_prev_dev, const double* kappa_dev,
                       double* rhs_dev, double dt);

/* For many right-hand sides with one kappa field (a time loop, the adjoint),
 * 3D contexts: adsg_kappa_points evaluates the field at every element's Gauss
 * points once, into kq_dev (adsg_kappa_points_count doubles, (p+1)^3 per
 * element, in the element kernel's own order: by element colour, so that a
 * warp's elements are contiguous), and adsg_heat_rhs_elem_points takes those
 * values instead of interpolating the coefficients on every call.  The values are the ones adsg_heat_rhs_elem
 * interpolates, bit for bit, so both give the same rhs.  count: 0 for a 2D
 * context (ADSG_ERR_UNSUPPORTED from the other two). */
long long adsg_kappa_points_count(const adsg_ctx* ctx);
int adsg_kappa_points(adsg_ctx* ctx, const double* kappa_dev, double* kq_dev);
int adsg_heat_rhs_elem_points(adsg_ctx* ctx, const double* u_prev_dev, const double* kq_dev, double* rhs_dev,
                              double dt);

/* ads_solve(rhs, buf, dims...) (reference include/ads/solver.hpp:222-226,
 * standard ADS, 1D case :199-203): solves (M_x (x) M_y (x) M_z) x = rhs with the
 * factorised bands, one pivoted band substitution (dgbtrs) per grid line and
 * direction, with no transpose passes.  The solution is left in rhs_dev;
 * buf_dev is accepted for signature parity and may be NULL. */
int adsg_ads_solve(adsg_ctx* ctx, double* rhs_dev, double* buf_dev);

/* The transposed solve (dgbtrs 'T' along every direction): the adjoint of
 * adsg_ads_solve. */
int adsg_ads_solve_t(adsg_ctx* ctx, double* rhs_dev);

/* One explicit step, heat_3d::step (heat_3d.hpp:39-47: compute_rhs then
 * ads_solve): u_next = M^-1 R u_prev.  u_prev_dev and u_next_dev must not
 * overlap.  Because the right-hand side stays internal, directions solved
 * with the two-ended sweep receive it row-scaled by their factors' diagonal
 * (folded into the band rows) and skip the backward sweep's multiply, and
 * the directions are solved outermost first and x last (x first when the x
 * band pass is fused with the x solve); the result equals adsg_heat_rhs +
 * adsg_ads_solve up to rounding. */
int adsg_heat_step(adsg_ctx* ctx, const double* u_prev_dev, double* u_next_dev, double dt);

/* nsteps of simulation_base::run's loop with heat_3d's step
 * (simulation_base.cpp:11-20, heat_3d.hpp:39-47): swap, compute_rhs, solve.
 * u_dev holds the state in and out.  Steps are adsg_heat_step's, replayed
 * from a CUDA graph. */
int adsg_heat_steps(adsg_ctx* ctx, double* u_dev, double dt, int nsteps);

/* ---- stage timers (observability) -----------------------------------------
 * Stages of a step, in launch order.  With timers enabled every kernel launch
 * of the context is bracketed by CUDA events on the context's stream (not
 * while a CUDA graph replays).  adsg_ctx_stage_times synchronises, adds the
 * elapsed times to ms[stage] and launch counts to launches[stage] (arrays of
 * ADSG_NSTAGES entries, accumulated since the last call) and resets them.
 * adsg_ctx_stage_work gives each stage's algorithmic work per launch: the FP64
 * operations of the algorithm the stage's kernel implements in the step path
 * (pair sums on symmetric band rows, two-ended unit-diagonal sweeps where the
 * context chose them), each FMA, multiply or add counted as 2 flops since
 * each takes one DFMA issue slot (the element stage: FMA = 2, others = 1), and
 * compulsory HBM bytes (each input read and each output written once). */
#define ADSG_STAGE_RHS_OUTER 0  /* band pass along z (3D) or y (2D) */
#define ADSG_STAGE_RHS_MIDDLE 1 /* band pass along y (3D) */
#define ADSG_STAGE_RHS_X 2      /* band pass along x, writes the RHS */
#define ADSG_STAGE_SOLVE_X 3
#define ADSG_STAGE_SOLVE_Y 4
#define ADSG_STAGE_SOLVE_Z 5
#define ADSG_STAGE_RHS_ELEM 6   /* element-wise sum-factorised quadrature */
#define ADSG_STAGE_RHS_SOLVE_X 7 /* x band pass fused with the x solve (adsg_heat_step) */
#define ADSG_STAGE_STEP_1BLOCK 8 /* a whole small 2D step in one block (adsg_heat_step) */
#define ADSG_NSTAGES 9
int adsg_ctx_enable_stage_timers(adsg_ctx* ctx, int enable);
int adsg_ctx_stage_times(adsg_ctx* ctx, double* ms, long long* launches);
int adsg_ctx_stage_work(const adsg_ctx* ctx, double* flops, double* bytes);
/* Line-solve kernel chosen per direction when the context was created (the
 * autotuner times each applicable variant on the context's own buffers):
 * 0 one 32-line tile per block staged in shared memory, 1 and 2 the same with
 * two / four tiles per block, 3 lines swept in place in global memory, four
 * warps per block (0-3 follow dgbtrs's operation order and agree bitwise);
 * 4 the two-ended sweep (each line swept from both ends by two lanes, the
 * meeting unknowns from a small dense inverse) in global memory, 5 the same
 * with contiguous lines staged whole through shared memory, 6 the same with
 * contiguous lines streamed through shared memory in 32-row chunks, 7 the
 * same as 5 with the tile moved by the copy engine (one bulk copy in and one
 * out per 16 lines; 4-7 agree bitwise).  variants has 3 entries
 * (-1 for absent dimensions).  The environment variable ADSG_SOLVE_VARIANT
 * forces a variant where it applies; ADSG_AUTOTUNE_LOG=1 prints the timings.
 * Decisions are cached per shape for the process. */
int adsg_ctx_solve_variants(const adsg_ctx* ctx, int* variants);
/* Line-solve variant per direction of the explicit step (adsg_heat_step,
 * adsg_heat_steps*): the variant above, or, where that is 0-3 and a
 * two-ended variant with the pivots folded into the right-hand side is at
 * least 5% faster on this shape, that variant (4-6).  Same layout as
 * adsg_ctx_solve_variants. */
int adsg_ctx_step_solve_variants(const adsg_ctx* ctx, int* variants);
/* 1 when the step's kernels use programmatic dependent launch (chosen at
 * creation by timing a few steps both ways; ADSG_PDL=0/1 forces it), 0 when
 * not, -1 for a NULL context.  Results do not depend on it. */
int adsg_ctx_launch_pdl(const adsg_ctx* ctx);
/* 1 when adsg_heat_step fuses the x band pass into the x solve (possible when
 * x uses solve variant 5; chosen at creation by timing, ADSG_FUSE_X=0/1
 * forces it), 0 when not, -1 for a NULL context.  The fused step solves x
 * first, the unfused one x last: results agree to rounding. */
int adsg_ctx_fused_x(const adsg_ctx* ctx);
/* 1 when adsg_heat_step runs a whole 2D step in one block (grids whose four
 * working tensors fit in 200 KB of shared memory, both directions on the
 * two-ended sweep; chosen at creation by timing, ADSG_STEP_1BLOCK=0/1 forces
 * it), 0 when not, -1 for a NULL context.  Results do not depend on it. */
int adsg_ctx_step_1block(const adsg_ctx* ctx);
/* 1 when that one-launch step runs on a thread-block cluster (8 CTAs: the
 * band passes spread over their SMs through distributed shared memory, the
 * sweeps in the first CTA), 0 when on one block or not used; chosen at
 * creation by timing both, ADSG_STEP_CLUSTER=0/1 forces it; -1 for NULL.
 * Results do not depend on it. */
int adsg_ctx_step_cluster(const adsg_ctx* ctx);
/* 1 when adsg_heat_step replays a cached single-step CUDA graph per
 * (u_prev, u_next, dt) (up to four, the least recently used replaced; steps
 * issued into a stream under capture, with stage timers on, or with buffers
 * that change faster than the cache serves are launched directly), 0 when it
 * always launches directly; chosen at creation by timing both,
 * ADSG_STEP_GRAPHS=0/1 forces it; -1 for a NULL context.  Results do not
 * depend on it. */
int adsg_ctx_step_graphs(const adsg_ctx* ctx);

/* ---- Dirichlet rows -----------------------------------------------------------
 * The reference imposes Dirichlet data in two steps: the dimension's mass
 * matrix gets identity rows (dimension::fix_dof, adsg_dim_fix_dof here) and,
 * before every solve, those rows of the right-hand side are overwritten with
 * the boundary values -- examples/heat/heat_2d.hpp:40-45 sets row x = 0 to the
 * load vector of sin(pi y); examples/validation/validation.hpp:31-41 zeroes
 * all four sides.  A plane is the set of dofs whose index along direction dim
 * equals index; values (device) holds its dofs x-fastest over the other
 * directions, or is NULL for zeros. */
typedef struct adsg_plane {
    int dim;
    int index;
    const double* values;
} adsg_plane;
/* Overwrite planes of a device tensor (asynchronous). */
int adsg_set_planes(adsg_ctx* ctx, double* u_dev, int nplanes, const adsg_plane* planes);
/* One step of those examples: compute_rhs (the heat form, as adsg_heat_rhs),
 * the planes overwritten in the right-hand side, then ads_solve with the
 * context's (fixed-row) factorisations: heat_2d::step / validation::step
 * (heat_2d.hpp:66-69 with its solve at :40-45).  u_prev and u_next must not
 * overlap.  Asynchronous. */
int adsg_heat_step_dirichlet(adsg_ctx* ctx, const double* u_prev_dev, double* u_next_dev, double dt, int nplanes,
                             const adsg_plane* planes);

/* ---- host-buffer entry points (the reference-facing boundary) ------------- */

/* adsg_heat_steps on a host tensor: copies u_host to the device, runs nsteps,
 * copies the result back; synchronises. */
int adsg_heat_steps_host(adsg_ctx* ctx, double* u_host, double dt, int nsteps);

/* adsg_ads_solve on a host tensor (copy in, solve, copy out; synchronises). */
int adsg_ads_solve_host(adsg_ctx* ctx, double* rhs_host);

/* adsg_heat_rhs on host tensors (synchronises). */
int adsg_heat_rhs_host(adsg_ctx* ctx, const double* u_prev_host, double* rhs_host, double dt);

/* Drop-in for LAPACK dgbtrs_ as the reference declares it
 * (include/ads/lin/lapack.hpp:27-39, called from lin/band_solve.hpp:26-31):
 * same arguments, by pointer, host memory, column-major B with ldb >= n.
 * Solves on the GPU (all nrhs columns in parallel) and synchronises.  Any n;
 * kl <= 16 and kl + ku <= 32.
 * *info = 0 on success, -k for an invalid k-th argument (as LAPACK), and
 * positive whenever B is left unsolved for another reason: the 1-based column
 * of an exactly zero U diagonal (dgbtrf's meaning), or n + 1 when the GPU
 * solve could not run (band wider than the limits above, a CUDA failure;
 * adsg_last_error() has the reason).  Every nonzero info is also reported on
 * stderr.  The return value is 0 or the ADSG status. */
int adsg_dgbtrs_(const char* trans, const int* n, const int* kl, const int* ku, const int* nrhs,
                 const double* ab, const int* ldab, const int* ipiv, double* b, const int* ldb,
                 int* info);

/* adsg_dgbtrs_ for callers that never read info, such as the reference's own
 * lin::solve_with_factorized (band_solve.hpp:26-31 ignores it): on any
 * nonzero info it prints the reason and aborts the process, as reference
 * LAPACK's xerbla stops on a bad argument, instead of letting the program go
 * on with unsolved right-hand sides.  Bind the reference to this one
 * (-Ddgbtrs_=adsg_dgbtrs_checked_).  Returns 0. */
int adsg_dgbtrs_checked_(const char* trans, const int* n, const int* kl, const int* ku, const int* nrhs,
                         const double* ab, const int* ldab, const int* ipiv, double* b, const int* ldb,
                         int* info);

/* ---- general pointwise forms (the other problems' compute_rhs) -------------
 * rhs_a = sum_e sum_q w_q J_e [ A u v_a + B grad u . grad v_a + G v_a + D ]
 * where each of A, B, G, D is a constant plus an optional per-point field
 * (device, the Gauss-point layout of adsg_eval_quad; NULL = none) and D is
 * added to every dof of the element without a test function.  Covers:
 *  - heat_3d::compute_rhs (heat_3d.hpp:49-67): A = 1, B = -dt;
 *  - scalability_3d::compute_rhs (scalability/test3d.hpp:66-95): A = 1,
 *    B = -dt, D_q = dt f(x_q) (the reference adds its forcing this way);
 *  - flow::compute_rhs (flow/flow.hpp:77-98): A = 1,
 *    B_q = -dt k(x_q) exp(mi u(x_q)), G_q = dt h(x_q, t), with u(x_q) from
 *    adsg_eval_quad and x_q from adsg_quad_points.
 * u_dev may be NULL when A and B are zero (a pure load).  2D and 3D, the
 * same degree and q = p + 1 in every direction.  rhs_dev is overwritten. */
typedef struct adsg_point_form {
    double alpha, beta, gamma, delta;
    const double* alpha_q;
    const double* beta_q;
    const double* gamma_q;
    const double* delta_q;
} adsg_point_form;
int adsg_form_rhs(adsg_ctx* ctx, const double* u_dev, const adsg_point_form* form, double* rhs_dev);

/* ---- Gauss-point utilities: projection, norms, errors -----------------------
 * Point tensors are x-fastest over the Gauss points of all elements of every
 * direction: point (rx, ry, rz) with rd = e_d * q_d + k_d.
 *  - adsg_load_vector: b_a = sum_e sum_q f(x_q) B_a(x_q) w_q J_e, the load
 *    vector of compute_projection (reference include/ads/projection.hpp:55-107);
 *  - adsg_projection: the load vector followed by adsg_ads_solve (the
 *    reference's projection(u, f); solve(u), heat_3d.hpp:35-36);
 *  - adsg_eval_quad: values and (grad_dev != NULL) the ndim first derivatives
 *    of a spline at every Gauss point (eval / eval_fun of simulation_3d.hpp);
 *  - adsg_norms: normL2 and normH1 of a spline (basic_simulation_3d.hpp:309-335),
 *    computed as sqrt(u^T M u) and sqrt(u^T (M + K) u) with the Kronecker
 *    mass/stiffness operators of the heat RHS;
 *  - adsg_errors: errorL2 / errorH1 against point values (and gradients) of a
 *    reference function (basic_simulation_3d.hpp:337-397); h1_out is set to -1
 *    when fgrad_dev is NULL;
 *  - adsg_quad_points: the Gauss points of direction d (needs desc.xq).
 * All synchronise except adsg_load_vector, adsg_projection, adsg_eval_quad. */
long long adsg_quad_size(const adsg_ctx* ctx);
/* Failure detection: the number of NaN / Inf coefficients of a device tensor
 * of the context's size (an explicit step that is unstable for its dt grows
 * until it overflows).  Synchronises. */
int adsg_count_nonfinite(adsg_ctx* ctx, const double* u_dev, long long* count_out);
int adsg_load_vector(adsg_ctx* ctx, const double* fq_dev, double* out_dev);
int adsg_projection(adsg_ctx* ctx, const double* fq_dev, double* out_dev);
int adsg_eval_quad(adsg_ctx* ctx, const double* u_dev, double* val_dev, double* grad_dev);
int adsg_norms(adsg_ctx* ctx, const double* u_dev, double* l2_out, double* h1_out);
int adsg_errors(adsg_ctx* ctx, const double* u_dev, const double* fq_dev, const double* fgrad_dev, double* l2_out,
                double* h1_out);
int adsg_quad_points(const adsg_ctx* ctx, int d, double* xq_host);

/* ---- generalised ADS --------------------------------------------------------
 * ads_solve(rhs, buf, dims..., callable, dims...) with one special dimension
 * (reference include/ads/solver.hpp:47-195, used by
 * examples/implicit/implicit.hpp:104-110): along the special direction each
 * grid line has its own factorised band.  A line-bands object holds nmat
 * dgbtrf factorisations of one size n (ab: nmat consecutive ldab*n bands,
 * ipiv: nmat*n 1-based pivots) and line_matrix[l] = the band of line l, with
 * lines numbered as the reference hands them to its callable: over the
 * directions that follow the special one cyclically, the first fastest.
 * adsg_ads_solve_general solves the special direction first, then the other
 * directions with the context's bands, as the reference does. */
typedef struct adsg_line_bands adsg_line_bands;
int adsg_line_bands_create(int n, int kl, int ku, int ldab, int nmat, const double* ab, const int* ipiv,
                           long long nlines, const int* line_matrix, adsg_line_bands** out);
int adsg_line_bands_destroy(adsg_line_bands* b);
int adsg_ads_solve_general(adsg_ctx* ctx, int special_dim, const adsg_line_bands* lines, double* rhs_dev);
int adsg_ads_solve_general_host(adsg_ctx* ctx, int special_dim, const adsg_line_bands* lines, double* rhs_host);

/* ---- adjoint (reverse mode) ------------------------------------------------
 * No counterpart in the reference.  For the kappa-weighted explicit step
 *     u_{k+1} = M^{-1} R(kappa) u_k,
 *     R(kappa)_ab = sum_e sum_q w_q J_e (B_a B_b - dt kappa(x_q) grad B_a . grad B_b)
 * (adsg_heat_rhs_elem followed by adsg_ads_solve), an adjoint object runs
 * nsteps forward from u0 with kappa (spline coefficients on the same space),
 * keeping checkpoints every checkpoint_every steps (0: ceil(sqrt(nsteps))),
 * then returns dL/du0 and dL/dkappa for a given dL/du(T).  The backward sweep
 * recomputes each segment once from its checkpoint and applies
 *     mu = M^{-T} lambda (transposed line solves),  dL/dkappa += mu^T dR/dkappa u_k,
 *     lambda <- R(kappa) mu (R is symmetric).
 * Needs a 2D or 3D context with one degree p <= 4 and p+1 Gauss points.
 * kappa is copied at forward time; buffers are device pointers of ctx's size.
 * In 3D the forward call also evaluates kappa at every element's Gauss points
 * ((p+1)^3 doubles per element, as adsg_kappa_points) and every element pass
 * reads those values; where that memory cannot be had at creation, the passes
 * interpolate the coefficients instead, with the same results bit for bit. */
typedef struct adsg_adjoint adsg_adjoint;
int adsg_adjoint_create(adsg_ctx* ctx, int nsteps, double dt, int checkpoint_every, adsg_adjoint** out);
int adsg_adjoint_destroy(adsg_adjoint* a);
int adsg_adjoint_checkpoints(const adsg_adjoint* a, int* every, int* count);
int adsg_adjoint_forward(adsg_adjoint* a, const double* u0_dev, const double* kappa_dev, double* uT_dev);
int adsg_adjoint_backward(adsg_adjoint* a, const double* dL_duT_dev, double* grad_u0_dev, double* grad_kappa_dev);
/* Mass-norm loss L = (u - target)^T (Mx (x) My (x) Mz) (u - target) on the host,
 * and dL/du = 2 M (u - target) into grad_dev; scratch_dev holds u - target.
 * Synchronises. */
int adsg_mass_loss(adsg_ctx* ctx, const double* u_dev, const double* target_dev, double* scratch_dev,
                   double* loss_host, double* grad_dev);

/* ---- batched simulations ---------------------------------------------------
 * No single counterpart in the reference, whose unit of work is one
 * simulation object run by simulation_base::run (simulation_base.cpp:11-20):
 * here many independent heat problems -- each 2D or 3D, cubic (the same
 * elements and degree in every direction), 1 <= p <= 4, its own dt, open
 * uniform knots on [0,1] -- advance together.  adsg_batch_steps runs nsteps
 * of every instance as ONE persistent cooperative launch (all RHS passes and
 * line solves of all instances as work items taken in order from a counter,
 * each instance's stages ordered by bounded waits on its own completion
 * counts), replayed from a CUDA graph; the grid size is chosen at creation by
 * timing every feasible blocks-per-SM count on the batch.  States start at
 * zero.  adsg_batch_steps_looped advances the same states with the plain
 * per-instance entry points (adsg_heat_rhs + adsg_ads_solve per instance and
 * step), the reference point for the batched launch. */
typedef struct adsg_batch adsg_batch;
int adsg_batch_create(int count, const int* ndim, const int* p, const int* elements, const double* dt,
                      adsg_batch** out);
int adsg_batch_destroy(adsg_batch* b);
long long adsg_batch_dofs(const adsg_batch* b, int i);
int adsg_batch_set_state(adsg_batch* b, int i, const double* u_host);  /* synchronises */
int adsg_batch_get_state(adsg_batch* b, int i, double* u_host);        /* synchronises */
int adsg_batch_steps(adsg_batch* b, int nsteps);
int adsg_batch_steps_looped(adsg_batch* b, int nsteps);
/* Waits for the batch's work; ADSG_ERR_DEVICE if a wait of the persistent kernel timed out. */
int adsg_batch_synchronize(adsg_batch* b);
/* Autotuned blocks per SM and whether the launch is replayed from a graph. */
int adsg_batch_tuning(const adsg_batch* b, int* blocks_per_sm, int* graph_captured);
/* The engine the batch chose at creation by timing both on itself: 0 the
 * persistent cooperative kernel (one launch per call: every stage of every
 * instance as a sequence of work items taken from a counter, each instance's
 * stages ordered by its own completion counts), 1 a CUDA graph of independent
 * per-instance chains (each instance's own tuned step kernels, run side by
 * side); -1 for a NULL batch.  ADSG_BATCH_ENGINE=0/1 forces it. */
int adsg_batch_engine(const adsg_batch* b);
/* The order in which the persistent kernel hands out a step's work, chosen
 * with its grid by timing: 0 stage-major (every instance's first stage, then
 * every instance's second, ...), 1 a wavefront over groups of instances whose
 * tensors fit in L2 together (group g runs stage w - g in wave w, so few
 * groups' tensors are live at once); -1 for a NULL batch.  Results do not
 * depend on it.  ADSG_BATCH_ORDER=0/1 forces it. */
int adsg_batch_order(const adsg_batch* b);
/* Test hook for failure detection (no reference counterpart): every wait of
 * the persistent kernel for an instance's previous stage expects
 * extra_items completed work items beyond those that exist (nonzero: no
 * such wait can end) and a waiting block gives up after spin_limit polls,
 * sets the batch's error word and the kernel winds down.
 * The next adsg_batch_synchronize returns ADSG_ERR_DEVICE and clears the
 * word; adsg_batch_test_waits(b, 0, 1 << 26) restores the defaults. */
int adsg_batch_test_waits(adsg_batch* b, int extra_items, long long spin_limit);

/* ---- debug build: device-side bounds checks ----------------------------------
 * No reference counterpart (the reference's debug builds assert in
 * band_matrix::operator(), lin/band_matrix.hpp:43).  In the library built
 * with -DADSG_BOUNDS_CHECK=1 (libads_gb300_checked.so: python
 * iga-ads_gb300/build.py --checked) the step, solve, batch, element and
 * Gauss-point kernels compare every global index with the extent of the
 * buffer it addresses, and every shared-memory tile with the launch's
 * dynamic shared memory; a violation skips the access (never traps) and is
 * counted.  This returns the count since the last reset and the first
 * violation's file (0 adsg_kernels.cu, 1 adsg_elem.cu, 2 adsg_quad.cu), source
 * line, index and extent; reset != 0 clears them.  Synchronises the device.
 * ADSG_ERR_UNSUPPORTED in the release build. */
int adsg_debug_bounds(long long* violations, int* file, int* line, long long* index, long long* extent, int reset);

/* ---- test hook: a device allocation that fails ---------------------------
 * No reference counterpart.  Makes the k-th device allocation of the library
 * from now on (k >= 0, counted across threads) fail as cudaMalloc does on a
 * full device, after which the hook turns itself off; k = -1 turns it off.
 * Every allocation goes through it: contexts (tables, state and work
 * tensors, the launch-mode tuner's buffer), Gauss-point work space,
 * adjoints and batches.  The call that meets the failure returns
 * ADSG_ERR_NOMEM with nothing leaked, and the next call works.  Returns the
 * previous setting (how many allocations were still to pass, -1 if none was
 * pending). */
int adsg_test_fail_device_alloc(int k);

/* ---- the heat RHS without any allocation --------------------------------
 * No counterpart in the reference: an addition for callers that cannot call
 * cudaMalloc -- code running inside a host application that owns every
 * device allocation through its own pool, or a latency-critical loop that
 * must not hit cudaMalloc's implicit device synchronisation.
 * Computes exactly what adsg_heat_rhs computes, but needs no context: the
 * dimensions are passed as host descriptors on every call, and the scratch
 * (four intermediate tensors and the 1D band tables) lives in a file-scope
 * device array of fixed size (about 17.6 MiB) that every GPU which loads the
 * library holds until the process exits.  The call enqueues on cuda_stream
 * (NULL: the legacy default stream) and allocates nothing, neither device nor
 * host memory.
 *  - The first call on a device looks up the array's device address
 *    (cudaGetSymbolAddress) with that device current and creates one event
 *    for that device.
 *  - All calls share the array: calls whose work overlaps on the GPU race and
 *    must be serialised by the caller.  Nothing carries over between calls.
 *    Calls on one stream need no synchronisation between them: a call waits
 *    on the host until the previous call's upload of the band tables has
 *    read the library's host staging buffer before it rewrites it.
 *  - Tensors above ADSG_NOALLOC_MAX_DOFS dofs or dimensions above
 *    ADSG_NOALLOC_MAX_N dofs are rejected with -2 and a message. */
#define ADSG_NOALLOC_MAX_DOFS (1 << 19)
#define ADSG_NOALLOC_MAX_N 1024
int adsg_heat_rhs_noalloc(int ndim, const adsg_dim_desc* dims, const double* u_prev_dev, double* rhs_dev,
                          double dt, void* cuda_stream);

#ifdef __cplusplus
}
#endif

#endif /* ADS_GB300_H */
