// sm_103a kernels of the explicit heat step.
//
// GB300 executes FP64 at ~1.2 TFLOP/s (measured: 2 DFMA/clk/SM, 64-cycle
// dependent latency), about 1/60 of its FP32 rate and far below what HBM can
// feed.  Every kernel here is therefore organised around the FP64 pipe: the
// work is arranged so that no FP64 operation is redundant, and loads, index
// arithmetic and shared-memory traffic (which run on other pipes) are spent
// freely to keep it busy.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "adsg_kernels.cuh"

namespace adsg {

// ---------------------------------------------------------------------------
// Band pass: one output per thread, 2p+1 neighbours along one axis.
// out0 = A0 (.) in0 [+ A1 (.) in1]; out1 = B0 (.) in0.
// Threads of a warp take consecutive x, so every neighbour load is coalesced;
// along y/z the band row is the same for the whole warp (broadcast loads).
// ---------------------------------------------------------------------------
template <int P, bool IN1, bool OUT1>
__global__ void __launch_bounds__(256) band_pass_kernel(const double* __restrict__ in0,
                                                         const double* __restrict__ in1,
                                                         double* __restrict__ out0,
                                                         double* __restrict__ out1,
                                                         const double* __restrict__ A0,
                                                         const double* __restrict__ A1,
                                                         const double* __restrict__ B0, int n_axis,
                                                         long long stride, long long total) {
    constexpr int BW = 2 * P + 1;
    long long g = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (g >= total) return;
    const int r = static_cast<int>((g / stride) % n_axis);
    const double* a0 = A0 + static_cast<long long>(r) * BW;
    const double* a1 = IN1 ? A1 + static_cast<long long>(r) * BW : nullptr;
    const double* b0 = OUT1 ? B0 + static_cast<long long>(r) * BW : nullptr;
    double acc0 = 0.0, acc1 = 0.0;
#pragma unroll
    for (int t = 0; t < BW; ++t) {
        const int c = r - P + t;
        if (c >= 0 && c < n_axis) {
            const long long at = g + static_cast<long long>(t - P) * stride;
            const double v0 = __ldg(in0 + at);
            acc0 = fma(__ldg(a0 + t), v0, acc0);
            if (OUT1) acc1 = fma(__ldg(b0 + t), v0, acc1);
            if (IN1) acc0 = fma(__ldg(a1 + t), __ldg(in1 + at), acc0);
        }
    }
    out0[g] = acc0;
    if (OUT1) out1[g] = acc1;
}

template <int P>
static cudaError_t band_pass_p(const double* in0, const double* in1, double* out0, double* out1,
                               const double* A0, const double* A1, const double* B0, int n_axis,
                               long long stride, long long total, cudaStream_t s) {
    const int threads = 256;
    const long long blocks = (total + threads - 1) / threads;
    if (in1 && out1)
        band_pass_kernel<P, true, true><<<blocks, threads, 0, s>>>(in0, in1, out0, out1, A0, A1, B0, n_axis, stride, total);
    else if (in1)
        band_pass_kernel<P, true, false><<<blocks, threads, 0, s>>>(in0, in1, out0, out1, A0, A1, B0, n_axis, stride, total);
    else if (out1)
        band_pass_kernel<P, false, true><<<blocks, threads, 0, s>>>(in0, in1, out0, out1, A0, A1, B0, n_axis, stride, total);
    else
        band_pass_kernel<P, false, false><<<blocks, threads, 0, s>>>(in0, in1, out0, out1, A0, A1, B0, n_axis, stride, total);
    return cudaGetLastError();
}

cudaError_t launch_band_pass(int p, const double* in0, const double* in1, double* out0, double* out1,
                             const double* A0, const double* A1, const double* B0, int n_axis,
                             long long stride, long long total, cudaStream_t s) {
    if (total <= 0) return cudaSuccess;
    switch (p) {
        case 1: return band_pass_p<1>(in0, in1, out0, out1, A0, A1, B0, n_axis, stride, total, s);
        case 2: return band_pass_p<2>(in0, in1, out0, out1, A0, A1, B0, n_axis, stride, total, s);
        case 3: return band_pass_p<3>(in0, in1, out0, out1, A0, A1, B0, n_axis, stride, total, s);
        case 4: return band_pass_p<4>(in0, in1, out0, out1, A0, A1, B0, n_axis, stride, total, s);
        case 5: return band_pass_p<5>(in0, in1, out0, out1, A0, A1, B0, n_axis, stride, total, s);
        case 6: return band_pass_p<6>(in0, in1, out0, out1, A0, A1, B0, n_axis, stride, total, s);
        case 7: return band_pass_p<7>(in0, in1, out0, out1, A0, A1, B0, n_axis, stride, total, s);
        case 8: return band_pass_p<8>(in0, in1, out0, out1, A0, A1, B0, n_axis, stride, total, s);
        default: return cudaErrorInvalidValue;
    }
}

__global__ void dt_bands_kernel(const double* __restrict__ mrow, const double* __restrict__ krow,
                                double* __restrict__ nrow, double* __restrict__ kdt, double dt, int count) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const double k = krow[i];
    nrow[i] = fma(-dt, k, mrow[i]);
    kdt[i] = -dt * k;
}

cudaError_t launch_dt_bands(const dim_dev& d, double dt, double* nrow, double* kdt, cudaStream_t s) {
    const int count = d.n * (2 * d.p + 1);
    dt_bands_kernel<<<(count + 255) / 256, 256, 0, s>>>(d.mrow, d.krow, nrow, kdt, dt, count);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Line solves.  One warp owns 32 grid lines; the lines are staged in shared
// memory as s[j*33 + lane] (row j of all 32 lines; the odd pitch keeps both
// the coalesced staging of contiguous x-lines and the sweeps conflict-free),
// swept in place column by column exactly as LAPACK's dgbtrs/dtbsv order the
// updates, and written back.  No transpose pass: the staging reads each
// direction's lines where they lie.
// ---------------------------------------------------------------------------
constexpr int kPitch = 33;

size_t line_solve_smem_per_warp(int n) { return static_cast<size_t>(n) * kPitch * sizeof(double); }

line_layout make_line_layout(const int* n, int ndim, int d) {
    long long nx = n[0], ny = ndim > 1 ? n[1] : 1, nz = ndim > 2 ? n[2] : 1;
    line_layout L;
    if (d == 0) {
        L.nlines = ny * nz;
        L.a = L.nlines;
        L.sa = nx;
        L.sb = 0;
        L.elem_stride = 1;
        L.contiguous = 1;
    } else if (d == 1) {
        L.nlines = nx * nz;
        L.a = nx;
        L.sa = 1;
        L.sb = nx * ny;
        L.elem_stride = nx;
    } else {
        L.nlines = nx * ny;
        L.a = nx * ny;
        L.sa = 1;
        L.sb = 0;
        L.elem_stride = nx * ny;
    }
    return L;
}

__device__ __forceinline__ void stage_in(const double* __restrict__ data, double* s, const line_layout& L,
                                         int n, long long line0, int nvalid, int lane) {
    if (L.contiguous) {
        const double* src = data + line0 * n;
        for (int l = 0; l < 32; ++l) {
            if (l < nvalid) {
                for (int j = lane; j < n; j += 32) s[j * kPitch + l] = src[static_cast<long long>(l) * n + j];
            } else {
                for (int j = lane; j < n; j += 32) s[j * kPitch + l] = 0.0;
            }
        }
    } else {
        const long long g = line0 + lane;
        const bool ok = lane < nvalid;
        const long long base = ok ? (g % L.a) * L.sa + (g / L.a) * L.sb : 0;
        for (int j = 0; j < n; ++j) s[j * kPitch + lane] = ok ? data[base + j * L.elem_stride] : 0.0;
    }
}

__device__ __forceinline__ void stage_out(double* __restrict__ data, const double* s, const line_layout& L,
                                          int n, long long line0, int nvalid, int lane) {
    if (L.contiguous) {
        double* dst = data + line0 * n;
        for (int l = 0; l < nvalid; ++l)
            for (int j = lane; j < n; j += 32) dst[static_cast<long long>(l) * n + j] = s[j * kPitch + l];
    } else {
        if (lane < nvalid) {
            const long long g = line0 + lane;
            const long long base = (g % L.a) * L.sa + (g / L.a) * L.sb;
            for (int j = 0; j < n; ++j) data[base + j * L.elem_stride] = s[j * kPitch + lane];
        }
    }
}

// dgbtrs 'N': L-solve with row exchanges (dgbtrs forward loop + dger), then
// U-solve (dtbsv 'Upper','N','Non-unit') with the diagonal as a reciprocal.
__device__ __forceinline__ void sweep_n(double* x, const dim_dev& D) {
    const int n = D.n, kl = D.kl, w = D.w;
    for (int j = 0; j < n - 1; ++j) {
        const int l = __ldg(D.piv + j);
        if (l != j) {
            const double t = x[l * kPitch];
            x[l * kPitch] = x[j * kPitch];
            x[j * kPitch] = t;
        }
        const double y = -x[j * kPitch];
        const int lm = min(kl, n - 1 - j);
        const double* lj = D.lmul + static_cast<long long>(j) * kl;
        for (int i = 1; i <= lm; ++i) x[(j + i) * kPitch] = fma(y, __ldg(lj + i - 1), x[(j + i) * kPitch]);
    }
    for (int j = n - 1; j >= 0; --j) {
        const double v = x[j * kPitch] * __ldg(D.rdiag + j);
        x[j * kPitch] = v;
        const int ext = __ldg(D.uext + j);
        const double* uj = D.ucol + static_cast<long long>(j) * w;
        const double nv = -v;
        for (int dd = 1; dd <= ext; ++dd) x[(j - dd) * kPitch] = fma(nv, __ldg(uj + dd - 1), x[(j - dd) * kPitch]);
    }
}

// dgbtrs 'T': U^T-solve (dtbsv 'Upper','T'), then L^T with the row exchanges
// undone in reverse order.
__device__ __forceinline__ void sweep_t(double* x, const dim_dev& D) {
    const int n = D.n, kl = D.kl, w = D.w;
    for (int j = 0; j < n; ++j) {
        double t = x[j * kPitch];
        const int ext = __ldg(D.uext + j);
        const double* uj = D.ucol + static_cast<long long>(j) * w;
        for (int dd = ext; dd >= 1; --dd) t = fma(-__ldg(uj + dd - 1), x[(j - dd) * kPitch], t);
        x[j * kPitch] = t * __ldg(D.rdiag + j);
    }
    for (int j = n - 2; j >= 0; --j) {
        const int lm = min(kl, n - 1 - j);
        const double* lj = D.lmul + static_cast<long long>(j) * kl;
        double t = 0.0;
        for (int i = 1; i <= lm; ++i) t = fma(x[(j + i) * kPitch], __ldg(lj + i - 1), t);
        x[j * kPitch] -= t;
        const int l = __ldg(D.piv + j);
        if (l != j) {
            const double s = x[l * kPitch];
            x[l * kPitch] = x[j * kPitch];
            x[j * kPitch] = s;
        }
    }
}

__global__ void __launch_bounds__(32) line_solve_kernel(double* __restrict__ data, dim_dev D, line_layout L,
                                                        int trans) {
    extern __shared__ double smem[];
    const int lane = threadIdx.x & 31;
    const long long line0 = static_cast<long long>(blockIdx.x) * 32;
    if (line0 >= L.nlines) return;
    const int nvalid = static_cast<int>(min(32LL, L.nlines - line0));
    double* s = smem;
    stage_in(data, s, L, D.n, line0, nvalid, lane);
    __syncwarp();
    if (trans)
        sweep_t(s + lane, D);
    else
        sweep_n(s + lane, D);
    __syncwarp();
    stage_out(data, s, L, D.n, line0, nvalid, lane);
}

cudaError_t launch_line_solve(double* data, const dim_dev& d, const line_layout& L, int trans, cudaStream_t s) {
    if (L.nlines <= 0) return cudaSuccess;
    const size_t smem = line_solve_smem_per_warp(d.n);
    static thread_local size_t configured = 0;
    if (smem > 48 * 1024 && smem > configured) {
        cudaError_t e = cudaFuncSetAttribute(line_solve_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             static_cast<int>(smem));
        if (e != cudaSuccess) return e;
        configured = smem;
    }
    const long long blocks = (L.nlines + 31) / 32;
    line_solve_kernel<<<blocks, 32, smem, s>>>(data, d, L, trans);
    return cudaGetLastError();
}

}  // namespace adsg
