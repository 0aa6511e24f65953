// Internal declarations shared by the host set-up, the kernels and the C-ABI.
#ifndef ADSG_INTERNAL_HPP
#define ADSG_INTERNAL_HPP

#include <cstddef>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/ads_gb300.h"

namespace adsg {

// One dimension on the host: what the reference's ads::dimension holds.
struct dim_host {
    int p = 0, elements = 0, q = 0, n = 0;
    int kl = 0, ku = 0, ldab = 0;
    std::vector<double> knots;
    std::vector<double> btab;  // [E][q][2][p+1]
    std::vector<double> xq;    // [E][q]
    std::vector<double> w;     // [q]
    std::vector<double> J;     // [E]
    std::vector<int> first_dofs;
    std::vector<double> mass;   // unfactorised, LAPACK band layout kl = ku = p
    std::vector<double> stiff;  // same layout
    std::vector<double> lu;     // factorised copy of mass
    std::vector<int> ipiv;      // 1-based
};

bool gauss_legendre(int q, double* x, double* w);
bool build_dimension(dim_host& d, int p, int elements, double a, double b, int q);
void form_band(const dim_host& d, int which, std::vector<double>& ab);
int factorize(dim_host& d);

// Solve tables extracted from a dgbtrf band (see make_solve_tables).
struct solve_tables {
    std::vector<double> lmul, ucol, rdiag;  // lmul padded by 16 columns
    std::vector<int> piv, uext;
    int kl = 0, w = 0;
    int fwd_fast = 0, bwd_fast = 0;
};

// Twisted (two-ended) factorisation of a band matrix with kl == ku == k:
// rows [0, n1) are eliminated top-down, rows [n1, n) bottom-up, and the 2k
// unknowns where the chains meet come from a dense 2k x 2k inverse.  Tables
// are laid out as dim_dev's tw_* members (see make_twisted_tables).
struct twisted_tables {
    int k = 0, n1 = 0, n2 = 0, rows = 0;
    std::vector<double> lmul, ucol, rdiag, g;
};

// Row-scaled form of twisted tables for a right-hand side that arrives
// multiplied by scale[r] = 1 / U(r, r) (r the global row along the line):
// the upper factors get a unit diagonal (rdiag = 1, unused), the multipliers
// and the meeting-point rows absorb the scaling.  Solving the scaled system
// gives the same x.
void scale_twisted(const twisted_tables& t, int n, twisted_tables& out, std::vector<double>& scale);

// Row-format band [n][2p+1] of sum_e sum_q B_a B_b w_q J_e (which: 0 values, 1 derivatives).
std::vector<double> row_band(const adsg_dim_desc& d, int which);
bool valid_desc(const adsg_dim_desc& d);
void symmetric_row_range(const std::vector<double>& m, const std::vector<double>& k, int n, int p, int& lo, int& hi);
// 0 on success, else the 1-based column of a zero diagonal.
int make_solve_tables(int n, int kl, int ku, int ldab, const double* ab, const int* ipiv, solve_tables& t);

// Builds the twisted tables of the matrix whose dgbtrf factors (ab, ipiv) are
// given.  Returns 0 when built; non-zero when the band is not symmetric in
// shape, too short, or the unpivoted elimination is not accurate enough
// (the LAPACK-order sweeps are used then).
int make_twisted_tables(int n, int kl, int ku, int ldab, const double* ab, const int* ipiv, twisted_tables& t);

// A context's stream, and its dt-dependent bands built ahead of a stream
// capture (used by the batched engine).
cudaStream_t ctx_stream(adsg_ctx* c);
int ctx_prepare_dt(adsg_ctx* c, double dt);

// Records msg as the calling thread's last error and returns code.
int fail(int code, const char* msg);
// A CUDA error: ADSG_ERR_NOMEM for a failed allocation, else ADSG_ERR_CUDA.
int fail_cuda(int err, const char* where);

// Every device allocation of the library: cudaMalloc, unless the test hook
// (adsg_test_fail_device_alloc) makes this one fail as a full device would.
cudaError_t device_alloc(void** p, size_t bytes);

}  // namespace adsg

#endif
