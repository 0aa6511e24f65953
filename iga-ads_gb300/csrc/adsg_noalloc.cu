// adsg_heat_rhs_noalloc: the heat RHS of adsg_heat_rhs for callers that may
// not allocate device memory -- for example code that runs inside a host
// application which owns every device allocation through its own pool, or
// that must not trigger cudaMalloc's implicit device synchronisation in a
// latency-critical loop.  It needs no context: the four intermediate tensors
// of the band passes and the 1D band tables live in one file-scope device
// array of fixed size, which every GPU that loads this library holds until
// the process exits.
//
// Limits: at most ADSG_NOALLOC_MAX_DOFS dofs in the tensor, at most
// ADSG_NOALLOC_MAX_N dofs along a dimension, degree <= ADSG_MAX_DEGREE.
//
// Calls share the array: two calls whose work overlaps on the GPU (different
// streams, or different host threads) race on it and must be serialised by
// the caller.  Calls on one stream are ordered and need nothing more: each
// call waits, on the host, until the previous call's table upload has read
// the host staging buffer before rewriting it.  Every element of the array that a call reads is written
// earlier in the same call (band tables are uploaded whole, every
// intermediate tensor is written by the pass before the one that reads it),
// so nothing has to start at zero and no content of a previous call is used.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>

#include "adsg_internal.hpp"
#include "adsg_kernels.cuh"

namespace adsg {
namespace {

constexpr long long kMaxDofs = ADSG_NOALLOC_MAX_DOFS;
constexpr int kMaxN = ADSG_NOALLOC_MAX_N;
constexpr int kMaxBand = 2 * ADSG_MAX_DEGREE + 1;
constexpr long long kTableDoubles = 3LL * 4 * kMaxN * kMaxBand;  // 3 dims x {M, K, M-dtK, -dtK}
constexpr long long kScratchDoubles = 4 * kMaxDofs + kTableDoubles;

// The device array.  In host code its name is only a host-side handle: the
// address the kernels use comes from cudaGetSymbolAddress below.
static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

// Host staging of the band tables (static: the entry point allocates nothing).
// The upload from it is asynchronous, and on a host whose memory the GPU
// reads directly the copy may read the buffer after the call has returned; so
// an event recorded after each upload is waited for before the next call
// rewrites the buffer.
static double g_host_tables[kTableDoubles];
static std::mutex g_lock;

constexpr int kMaxDevices = 64;
static double* g_dev_ptr[kMaxDevices] = {};
static cudaEvent_t g_upload_done[kMaxDevices] = {};
static cudaEvent_t g_pending = nullptr;  // the upload that last read g_host_tables

// Per-device set-up, once per device with that device current.
int scratch_address(double** out, cudaEvent_t* event) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail_cuda(e, "cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices) return fail(ADSG_ERR_UNSUPPORTED, "device index above 63");
    if (!g_dev_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return fail_cuda(e, "cudaGetSymbolAddress(scratch)");
        e = cudaEventCreateWithFlags(&g_upload_done[dev], cudaEventDisableTiming);
        if (e != cudaSuccess) return fail_cuda(e, "cudaEventCreate(upload)");
        g_dev_ptr[dev] = static_cast<double*>(p);
    }
    *out = g_dev_ptr[dev];
    *event = g_upload_done[dev];
    return 0;
}

bool desc_ok(const adsg_dim_desc& d) {
    if (d.p < 1 || d.p > ADSG_MAX_DEGREE || d.elements < 1 || d.quad_order < 1 || d.n < 1) return false;
    if (!d.btab || !d.w || !d.J || !d.first_dofs) return false;
    for (int e = 0; e < d.elements; ++e)
        if (d.first_dofs[e] < 0 || d.first_dofs[e] + d.p >= d.n) return false;
    return true;
}

// Row band [n][2p+1] of sum_e sum_q B_a B_b w_q J_e (which = 0: values,
// 1: derivatives), the same assembly the context performs.
void row_band_into(const adsg_dim_desc& d, int which, double* rows) {
    const int p = d.p, bw = 2 * p + 1;
    std::memset(rows, 0, sizeof(double) * static_cast<size_t>(d.n) * bw);
    for (int e = 0; e < d.elements; ++e) {
        const int f = d.first_dofs[e];
        for (int k = 0; k < d.quad_order; ++k) {
            const double* v = d.btab + ((static_cast<size_t>(e) * d.quad_order + k) * 2 + which) * (p + 1);
            for (int a = 0; a <= p; ++a)
                for (int b = 0; b <= p; ++b) rows[static_cast<size_t>(f + a) * bw + (b - a + p)] += v[a] * v[b] * d.w[k] * d.J[e];
        }
    }
}

}  // namespace
}  // namespace adsg

using namespace adsg;

extern "C" int adsg_heat_rhs_noalloc(int ndim, const adsg_dim_desc* dims, const double* u_prev_dev, double* rhs_dev,
                                     double dt, void* cuda_stream) {
    if (ndim < 1 || ndim > 3) return fail(-1, "ndim must be 1, 2 or 3");
    if (!dims) return fail(-2, "dims is NULL");
    if (!u_prev_dev) return fail(-3, "u_prev is NULL");
    if (!rhs_dev) return fail(-4, "rhs is NULL");
    if (u_prev_dev == rhs_dev) return fail(-4, "rhs must not alias u_prev");
    if (!std::isfinite(dt)) return fail(-5, "dt must be finite");
    long long size = 1;
    for (int d = 0; d < ndim; ++d) {
        if (!desc_ok(dims[d])) return fail(-2, "invalid dimension descriptor");
        if (dims[d].n > kMaxN)
            return fail(-2, "adsg_heat_rhs_noalloc: a dimension has more than ADSG_NOALLOC_MAX_N (1024) dofs");
        size *= dims[d].n;
    }
    if (size > kMaxDofs)
        return fail(-2, "adsg_heat_rhs_noalloc: tensor larger than ADSG_NOALLOC_MAX_DOFS (524288) dofs");
    cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);

    std::lock_guard<std::mutex> guard(g_lock);
    double* base = nullptr;
    cudaEvent_t upload_done = nullptr;
    int st = scratch_address(&base, &upload_done);
    if (st) return st;
    if (g_pending) {
        // the previous call's upload must have read the staging buffer
        const cudaError_t w = cudaEventSynchronize(g_pending);
        if (w != cudaSuccess) return fail_cuda(w, "wait for the previous upload");
        g_pending = nullptr;
    }
    double* T[4] = {base, base + kMaxDofs, base + 2 * kMaxDofs, base + 3 * kMaxDofs};
    double* tables_dev = base + 4 * kMaxDofs;

    // band tables of every dimension: M, K, M - dt K, -dt K (as the context computes them)
    const double* mrow[3] = {};
    const double* nrow[3] = {};
    const double* kdt[3] = {};
    size_t off = 0;
    for (int d = 0; d < ndim; ++d) {
        const size_t cnt = static_cast<size_t>(dims[d].n) * (2 * dims[d].p + 1);
        double* hm = g_host_tables + off;
        double* hk = hm + cnt;
        double* hn = hk + cnt;
        double* hd = hn + cnt;
        row_band_into(dims[d], 0, hm);
        row_band_into(dims[d], 1, hk);
        for (size_t i = 0; i < cnt; ++i) {
            hn[i] = std::fma(-dt, hk[i], hm[i]);
            hd[i] = -dt * hk[i];
        }
        mrow[d] = tables_dev + off;
        nrow[d] = tables_dev + off + 2 * cnt;
        kdt[d] = tables_dev + off + 3 * cnt;
        off += 4 * cnt;
    }
    cudaError_t e = cudaMemcpyAsync(tables_dev, g_host_tables, off * sizeof(double), cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return fail_cuda(e, "upload band tables");
    e = cudaEventRecord(upload_done, s);
    if (e != cudaSuccess) {
        // without the event the buffer cannot be rewritten safely: finish the copy now
        cudaStreamSynchronize(s);
        return fail_cuda(e, "record the upload");
    }
    g_pending = upload_done;

    const int nx = dims[0].n;
    if (ndim == 1) {
        e = launch_band_pass(dims[0].p, u_prev_dev, nullptr, rhs_dev, nullptr, nrow[0], nullptr, nullptr, nx, 1, size, s);
    } else if (ndim == 2) {
        e = launch_band_pass(dims[1].p, u_prev_dev, nullptr, T[0], T[1], mrow[1], nullptr, nrow[1], dims[1].n, nx,
                             size, s);
        if (e == cudaSuccess)
            e = launch_band_pass(dims[0].p, T[0], T[1], rhs_dev, nullptr, kdt[0], mrow[0], nullptr, nx, 1, size, s);
    } else {
        const long long sz = static_cast<long long>(nx) * dims[1].n;
        e = launch_band_pass(dims[2].p, u_prev_dev, nullptr, T[0], T[1], mrow[2], nullptr, nrow[2], dims[2].n, sz,
                             size, s);
        if (e == cudaSuccess)
            e = launch_band_pass(dims[1].p, T[0], T[1], T[2], T[3], kdt[1], mrow[1], mrow[1], dims[1].n, nx, size, s);
        if (e == cudaSuccess)
            e = launch_band_pass(dims[0].p, T[3], T[2], rhs_dev, nullptr, kdt[0], mrow[0], nullptr, nx, 1, size, s);
    }
    if (e != cudaSuccess) return fail_cuda(e, "adsg_heat_rhs_noalloc launch");
    return 0;
}
