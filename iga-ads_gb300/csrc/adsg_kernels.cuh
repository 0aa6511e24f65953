// Device-side data of a context and the kernel launchers.
#ifndef ADSG_KERNELS_CUH
#define ADSG_KERNELS_CUH

#include <cuda_runtime.h>

namespace adsg {

// Per-dimension device tables.  Band rows hold the 2p+1 coefficients of row r
// for columns r-p .. r+p (zero outside the matrix).
// Line-solve kernel variants chosen per direction by the context's autotuner.
// SOLVE_TWISTED* sweep each line from both ends (a two-chain factorisation of
// the same band; on contiguous lines the staged form copies whole lines
// through shared memory and the chunked form streams 32-row chunks; both
// equal the plain form on strided lines, and all three give bitwise equal
// results); the others follow LAPACK dgbtrs's column order and give bitwise
// equal results.
enum solve_variant_id {
    SOLVE_STAGED_1 = 0,
    SOLVE_STAGED_2 = 1,
    SOLVE_STAGED_4 = 2,
    SOLVE_GLOBAL_4 = 3,
    SOLVE_TWISTED = 4,
    SOLVE_TWISTED_STAGED = 5,
    SOLVE_TWISTED_CHUNKED = 6,
    SOLVE_TWISTED_BULK = 7,  // the staged tile moved by the copy engine (cp.async.bulk) both ways
    SOLVE_NVARIANTS = 8
};
inline bool solve_variant_twisted(int v) {
    return v == SOLVE_TWISTED || v == SOLVE_TWISTED_STAGED || v == SOLVE_TWISTED_CHUNKED || v == SOLVE_TWISTED_BULK;
}
// Bulk-copy waits of the x-line tiles that ran out (their lines were left
// unsolved); nonzero never happens in a healthy run.  reset != 0 clears it.
int bulk_wait_timeouts(int reset);

struct dim_dev {
    int n = 0, p = 0, kl = 0, w = 0;  // w = kl + ku: widest upper extent of U
    int ku_regular = 0;               // U extent of all columns but a few (row-exchange fill)
    int fwd_fast = 0;                 // no row exchange in columns >= fwd_fast
    int bwd_fast = 0;                 // U extent <= ku_regular in columns >= bwd_fast
    int solve_variant = SOLVE_STAGED_1;
    int elements = 0, q = 0;
    const double* mrow = nullptr;   // [n][2p+1] 1D mass matrix
    const double* krow = nullptr;   // [n][2p+1] 1D stiffness matrix
    const double* nrow = nullptr;   // [n][2p+1] M - dt K     (per dt)
    const double* kdt = nullptr;    // [n][2p+1] -dt K        (per dt)
    const double* lmul = nullptr;   // [n + 16][kl] L multipliers of column j (dgbtrf), zero padded
    const int* piv = nullptr;       // [n] 0-based row exchanged with row j
    const double* ucol = nullptr;   // [n][w] U(j-d, j), d = 1..w
    const int* uext = nullptr;      // [n] number of non-zero U(j-d, j) to apply
    const double* rdiag = nullptr;  // [n] 1 / U(j, j)
    const double* btab = nullptr;   // [E][q][2][p+1] basis values / derivatives
    const double* wq = nullptr;     // [q]
    const double* jac = nullptr;    // [E]
    const int* first = nullptr;     // [E]
    const int* erange = nullptr;    // [n][2] first and last element supporting each dof
    // Twisted factorisation (0 = not available): rows [0, tw_n1) form chain 0,
    // rows [tw_n1, n) chain 1 in reverse order; tables per chain, stride tw_rows.
    int tw_k = 0, tw_n1 = 0, tw_n2 = 0, tw_rows = 0;
    int tw_unit = 0;  // tables of the row-scaled system (unit upper diagonal)
    int sym_lo = 0, sym_hi = 0;  // rows [sym_lo, sym_hi) of the M and K bands are symmetric (pair sums allowed)
    const double* tw_lmul = nullptr;   // [2][tw_rows][k] multipliers of chain-local column j
    const double* tw_ucol = nullptr;   // [2][tw_rows][k] U(j-d, j), d = 1..k
    const double* tw_rdiag = nullptr;  // [2][tw_rows] 1 / U(j, j)
    const double* tw_g = nullptr;      // [2][k][2k] interface rows: own tail, then the other chain's tail
};

// Where the grid lines of one direction sit in a tensor of extents n[0..2]
// (x fastest): element j of line g is at base(g) + j*elem_stride with
// base(g) = (g % a) * sa + (g / a) * sb.
struct line_layout {
    long long nlines = 0;
    long long a = 1, sa = 0, sb = 0, elem_stride = 1;
    int contiguous = 0;  // lines are consecutive blocks of n doubles
    long long total = 0;  // doubles in the tensor the lines belong to (bounds-checked build)
};

line_layout make_line_layout(const int* n, int ndim, int d);

// Programmatic dependent launch for the step kernels issued by the calling
// thread (0 = off, 1 = on).
void set_launch_pdl(int on);
int launch_pdl_mode();
struct pdl_scope {
    int saved;
    explicit pdl_scope(int on) : saved(launch_pdl_mode()) { set_launch_pdl(on); }
    ~pdl_scope() { set_launch_pdl(saved); }
};

// Stacked solve tables of several factorised bands of one size (generalised ADS).
struct line_tables {
    int n = 0, kl = 0, w = 0, nmat = 0;
    const double* lmul = nullptr;   // [nmat][n][kl]
    const double* ucol = nullptr;   // [nmat][n][w]
    const double* rdiag = nullptr;  // [nmat][n]
    const int* piv = nullptr;       // [nmat][n]
    const int* uext = nullptr;      // [nmat][n]
};

cudaError_t launch_line_solve_permat(double* data, const line_tables& T, const line_layout& L, const int* line_matrix,
                                     int nx, int nz, int special, int ndim, cudaStream_t s);

// One instance of the batched engine (cubic: the same dimension in every direction).
struct batch_inst {
    int ndim = 0, p = 0, n = 0;
    int twisted = 0;  // 1: row-scaled bands and unit two-ended tables in dim; 0: LAPACK-order sweeps
    long long size = 0;
    long long units[6] = {};  // outputs (passes) or lines (solves) per stage; 0 = no work
    int items[6] = {};        // work items per stage (batch_units_per_item units each)
    double* buf[2] = {nullptr, nullptr};
    double* T[4] = {nullptr, nullptr, nullptr, nullptr};
    dim_dev dim;
};

struct batch_dev {
    int count = 0;
    const batch_inst* inst = nullptr;  // device array [count]
    // one step's (stage, instance) pairs in the order their items are handed
    // out: pair[k] = stage * count + instance at position k, prefix[k] the
    // step's items before position k
    const int* pair = nullptr;          // device array [6 count]
    const long long* prefix = nullptr;  // device array [6 count + 1]
    long long per_step = 0;             // items of one step
    unsigned* done = nullptr;           // device array [count][6]: items completed in this launch
    unsigned long long* next = nullptr;  // the work counter (zeroed before each launch)
    int* err = nullptr;
    // bounded wait: polls of a completion count before a waiting block gives
    // up (sets *err and winds down)
    long long spin_limit = 1LL << 26;
    // test hook (failure detection): items every wait expects beyond those
    // that exist; nonzero makes every wait run out
    unsigned wait_extra = 0;
};

const void* batch_kernel_symbol();
int batch_max_blocks_per_sm();
size_t batch_smem_bytes();
int batch_units_per_item(int stage, int twisted);
cudaError_t batch_prepare_kernel();

// rhs passes -------------------------------------------------------------
// out0 = A0 (.) in0 [+ A1 (.) in1],  out1 = B0 (.) in0  along one axis, where
// (.) applies a band with rows of 2p+1 coefficients.  Rows sym_lo .. sym_hi-1
// of every band are symmetric (dim_dev::sym_lo/hi; an empty range for none),
// so a two-output pass may share pair sums between its outputs there.
cudaError_t launch_band_pass(int p, const double* in0, const double* in1, double* out0, double* out1,
                             const double* A0, const double* A1, const double* B0, int n_axis,
                             long long stride, long long total, cudaStream_t s, int sym_lo = 0, int sym_hi = 0);
// The first pass of a step (out0 = A0 (.) in, out1 = B0 (.) in along the
// outermost axis) as column sweeps that read every input value once: for an
// input in pinned host memory, read over the host link while the pass
// computes.  Same operations in the same order as launch_band_pass; p <= 4.
bool outer_pass_columns_ok(int p);
// row_begin / row_end restrict the outputs to rows [row_begin, row_end) of the
// outer axis (the rows around them are still read for the band); -1 = all.
cudaError_t launch_outer_pass_columns(int p, const double* in, double* out0, double* out1, const double* A0,
                                      const double* B0, int n_axis, long long stride, cudaStream_t s, int sym_lo,
                                      int sym_hi, int row_begin = 0, int row_end = -1);

// Set the plane {index along d == k} of an x-fastest tensor with dofs n[0..ndim)
// to values (device, x-fastest over the other directions) or to 0 (NULL).
cudaError_t launch_set_plane(double* u, const double* values, const int* n, int ndim, int d, int k, cudaStream_t s);

// nrow = mrow - dt*krow, kdt = -dt*krow for one dimension
cudaError_t launch_dt_bands(const dim_dev& d, double dt, double* nrow, double* kdt, cudaStream_t s);

// line solves ------------------------------------------------------------
// trans = 0: dgbtrs 'N', trans = 1: dgbtrs 'T', along every line of layout L.
cudaError_t launch_line_solve(double* data, const dim_dev& d, const line_layout& L, int trans,
                              cudaStream_t s);
// The same solve of contiguous lines with the result written to out (e.g.
// mapped pinned host memory) instead of in place; only the tiled two-ended
// sweep (variant 5) does this (line_solve_out_ok).
bool line_solve_out_ok(const dim_dev& d, const line_layout& L);
cudaError_t launch_line_solve_out(const double* data, double* out, const dim_dev& d, const line_layout& L,
                                  cudaStream_t s);
size_t line_solve_smem_per_warp(int n);
bool line_solve_variant_ok(int variant, const dim_dev& d);
// x band pass (out = A0 (.) in0 [+ A1 (.) in1]) fused with the two-ended x
// solve on contiguous lines; out holds the solved lines.
bool rhs_x_solve_ok(const dim_dev& d, const line_layout& L);
// A whole 2D step (the step view's passes and two-ended unit-diagonal sweeps)
// in one block, for grids whose four working tensors fit in shared memory.
bool small2d_step_ok(const dim_dev& x, const dim_dev& y);
// Whether launch_small2d_step runs on a thread-block cluster (1, default) or one block (0),
// per calling thread.
void set_small2d_cluster(int on);
int small2d_cluster_mode();
cudaError_t launch_small2d_step(const double* u, double* out, const dim_dev& x, const dim_dev& y, cudaStream_t s);
cudaError_t launch_rhs_x_solve(const double* in0, const double* in1, double* out, const double* A0, const double* A1,
                               const dim_dev& d, const line_layout& L, cudaStream_t s);

// General pointwise form of the element quadrature: per Gauss point, a
// constant plus an optional field (Gauss-grid layout, x-fastest over
// e_d * q + k_d) for each coefficient of
//     rhs_a = sum_e sum_q w J [alpha u v_a + beta grad u . grad v_a + gamma v_a + delta]
// where delta is added to every dof of the element (no test function).
struct point_form {
    double alpha = 0.0, beta = 0.0, gamma = 0.0, delta = 0.0;
    const double* alpha_q = nullptr;
    const double* beta_q = nullptr;
    const double* gamma_q = nullptr;
    const double* delta_q = nullptr;
};
// rhs += the form applied to u (u may be NULL when alpha = beta = 0)
cudaError_t launch_form_elem(int ndim, const dim_dev* dims, const double* u, const point_form& F, double* rhs,
                             cudaStream_t s);

// element-wise sum-factorised quadrature (optional kappa field) -----------
// g += mu^T (dR/dkappa) u  (gradient of the element operator w.r.t. kappa
// coefficients), 2D; in 3D the gradient runs inside launch_adjoint_pair
cudaError_t launch_kappa_grad(int ndim, const dim_dev* dims, const double* u, const double* mu, double* g, double dt,
                              cudaStream_t s);
// both element operations of one adjoint backward step on mu:
// rmu += R(kappa) mu and g += mu^T (dR/dkappa) u, in one pass in 3D (the
// R(kappa) mu part bitwise launch_rhs_elem's), in two kernels in 2D
cudaError_t launch_adjoint_pair(int ndim, const dim_dev* dims, const double* u, const double* mu,
                                const double* kappa, double* rmu, double* g, double dt, cudaStream_t s,
                                bool kappa_points = false);  // kappa_points: kappa at the Gauss points (3D)

// small vector kernels of the adjoint driver
cudaError_t launch_axpby(double* y, double a, const double* x, double b, long long n, cudaStream_t s);  // y = a*x + b*y
cudaError_t launch_dot(const double* x, const double* y, long long n, double* partial, double* out, cudaStream_t s);

cudaError_t launch_sum(const double* partial, int m, double* out, cudaStream_t s);  // deterministic sum
cudaError_t launch_count_nonfinite(const double* x, long long n, unsigned long long* count, cudaStream_t s);

// quadrature-point passes (adsg_quad.cu); tensors are x-fastest, the pass acts
// on the axis with `inner` faster entries and `outer` slower ones
cudaError_t launch_quad_interp(const double* in, double* out0, double* out1, const dim_dev& d, long long inner,
                               long long outer, cudaStream_t s);
cudaError_t launch_quad_project(const double* in, double* out, const dim_dev& d, const int* erange, long long inner,
                                long long outer, cudaStream_t s);
struct field_set {
    int nf = 0;
    const double* a[4] = {nullptr, nullptr, nullptr, nullptr};
    const double* b[4] = {nullptr, nullptr, nullptr, nullptr};  // NULL: compare with zero
};
// sum over Gauss points of W * sum_k (a_k - b_k)^2 into out (device scalar)
cudaError_t launch_quad_wdiff(const field_set& F, const dim_dev* dims, int ndim, long long total, double* partial,
                              double* out, cudaStream_t s);

// kappa at every Gauss point of every element of a 3D grid
// (kappa_points_count doubles, by element colour in the element kernel's
// launch order), and the kappa RHS from those values: bitwise launch_rhs_elem
// with the coefficients
long long kappa_points_count(int ndim, const dim_dev* dims);
cudaError_t launch_kappa_points(const dim_dev* dims, const double* kappa, double* kq, cudaStream_t s);
cudaError_t launch_rhs_elem_points(const dim_dev* dims, const double* u_prev, const double* kq, double* rhs,
                                   double dt, cudaStream_t s);
cudaError_t launch_rhs_elem(int ndim, const dim_dev* dims, const double* u_prev, const double* kappa,
                            double* rhs, double dt, cudaStream_t s);

}  // namespace adsg

#endif
