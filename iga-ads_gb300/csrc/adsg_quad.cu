// Quadrature-point passes: interpolation of spline coefficients to the Gauss
// points of every element (values and first derivatives), and its transpose,
// the weighted projection of point values onto the basis (the load vector of
// compute_projection, reference include/ads/projection.hpp:55-107).  Both act
// along one axis at a time on x-fastest tensors: the tensor-product rule
// factors the element/point/dof loops into three 1D passes, each output a
// (p+1)- or (p+1)q-term sum.
#include <cuda_runtime.h>

#include "adsg_check.cuh"
#include "adsg_kernels.cuh"

namespace adsg {

ADSG_BOUNDS_TU(quad)

namespace {

// out(ii, r, oo) = sum_a T[e][qq][which][a] in(ii, first[e] + a, oo), r = e*q + qq
__global__ void quad_interp_kernel(const double* __restrict__ in, double* __restrict__ out0, double* __restrict__ out1,
                                   const double* __restrict__ btab, const int* __restrict__ first, int p, int q, int E,
                                   int n_axis, long long inner, long long outer) {
    const long long Qa = static_cast<long long>(E) * q;
    const long long total = inner * Qa * outer;
    for (long long g = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; g < total;
         g += static_cast<long long>(gridDim.x) * blockDim.x) {
        const long long ii = g % inner;
        const long long r = (g / inner) % Qa;
        const long long oo = g / (inner * Qa);
        const int e = static_cast<int>(r / q), qq = static_cast<int>(r % q);
        const double* row = btab + (static_cast<long long>(e) * q + qq) * 2 * (p + 1);
        const long long base = ii + inner * (static_cast<long long>(__ldg(first + e)) + n_axis * oo);
        // bounds-checked build: the element, and its p+1 input rows inside the tensor
        if (!(ADSG_IN(e, E) && ADSG_IN(base, inner * n_axis * outer) &&
              ADSG_IN(base + inner * p, inner * n_axis * outer)))
            continue;
        double a0 = 0.0, a1 = 0.0;
        for (int a = 0; a <= p; ++a) {
            const double v = in[base + inner * a];
            a0 = fma(__ldg(row + a), v, a0);
            if (out1) a1 = fma(__ldg(row + p + 1 + a), v, a1);
        }
        out0[g] = a0;
        if (out1) out1[g] = a1;
    }
}

// out(ii, a, oo) = sum_{e supporting a} sum_qq T[e][qq][0][a-first[e]] w[qq] J[e] in(ii, e*q+qq, oo)
__global__ void quad_project_kernel(const double* __restrict__ in, double* __restrict__ out,
                                    const double* __restrict__ btab, const int* __restrict__ first,
                                    const int* __restrict__ erange, const double* __restrict__ w,
                                    const double* __restrict__ J, int p, int q, int E, int n_axis, long long inner,
                                    long long outer) {
    const long long Qa = static_cast<long long>(E) * q;
    const long long total = inner * n_axis * outer;
    for (long long g = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; g < total;
         g += static_cast<long long>(gridDim.x) * blockDim.x) {
        const long long ii = g % inner;
        const int a = static_cast<int>((g / inner) % n_axis);
        const long long oo = g / (inner * n_axis);
        double acc = 0.0;
        const int lo = __ldg(erange + 2 * a), hi = __ldg(erange + 2 * a + 1);
        // bounds-checked build: the supporting elements, and the point rows they read
        if (!(ADSG_IN(lo, E) && ADSG_IN(hi, E) && ADSG_IN(ii + inner * (static_cast<long long>(lo) * q + Qa * oo), inner * Qa * outer) &&
              ADSG_IN(ii + inner * (static_cast<long long>(hi) * q + q - 1 + Qa * oo), inner * Qa * outer)))
            continue;
        for (int e = lo; e <= hi; ++e) {
            const int loc = a - __ldg(first + e);
            const double je = __ldg(J + e);
            for (int qq = 0; qq < q; ++qq) {
                const double b = __ldg(btab + (static_cast<long long>(e) * q + qq) * 2 * (p + 1) + loc);
                acc = fma(b * __ldg(w + qq) * je, in[ii + inner * (static_cast<long long>(e) * q + qq + Qa * oo)], acc);
            }
        }
        out[g] = acc;
    }
}

// partial sums of W(point) * (sum_k (a_k - b_k)^2) over the quadrature grid
__global__ void quad_wdiff_kernel(field_set F, dim_dev X, dim_dev Y, dim_dev Z, int ndim, long long total,
                                  double* __restrict__ partial) {
    __shared__ double sh[256];
    const long long Qx = static_cast<long long>(X.elements) * X.q;
    const long long Qy = ndim > 1 ? static_cast<long long>(Y.elements) * Y.q : 1;
    double acc = 0.0;
    for (long long g = blockIdx.x * 256LL + threadIdx.x; g < total; g += 256LL * gridDim.x) {
        const long long rx = g % Qx, ry = (g / Qx) % Qy, rz = g / (Qx * Qy);
        double W = __ldg(X.wq + rx % X.q) * __ldg(X.jac + rx / X.q);
        if (ndim > 1) W *= __ldg(Y.wq + ry % Y.q) * __ldg(Y.jac + ry / Y.q);
        if (ndim > 2) W *= __ldg(Z.wq + rz % Z.q) * __ldg(Z.jac + rz / Z.q);
        double s = 0.0;
        for (int k = 0; k < F.nf; ++k) {
            const double d = F.a[k][g] - (F.b[k] ? F.b[k][g] : 0.0);
            s = fma(d, d, s);
        }
        acc = fma(W, s, acc);
    }
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int wdt = 128; wdt > 0; wdt >>= 1) {
        if (threadIdx.x < wdt) sh[threadIdx.x] += sh[threadIdx.x + wdt];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

int grid_for(long long total) {
    long long b = (total + 255) / 256;
    return static_cast<int>(b < 152 * 32 ? (b > 0 ? b : 1) : 152 * 32);
}

}  // namespace

cudaError_t launch_quad_interp(const double* in, double* out0, double* out1, const dim_dev& d, long long inner,
                               long long outer, cudaStream_t s) {
    const long long total = inner * static_cast<long long>(d.elements) * d.q * outer;
    quad_interp_kernel<<<grid_for(total), 256, 0, s>>>(in, out0, out1, d.btab, d.first, d.p, d.q, d.elements, d.n,
                                                        inner, outer);
    return cudaGetLastError();
}

cudaError_t launch_quad_project(const double* in, double* out, const dim_dev& d, const int* erange, long long inner,
                                long long outer, cudaStream_t s) {
    const long long total = inner * static_cast<long long>(d.n) * outer;
    quad_project_kernel<<<grid_for(total), 256, 0, s>>>(in, out, d.btab, d.first, erange, d.wq, d.jac, d.p, d.q,
                                                         d.elements, d.n, inner, outer);
    return cudaGetLastError();
}

cudaError_t launch_quad_wdiff(const field_set& F, const dim_dev* dims, int ndim, long long total, double* partial,
                              double* out, cudaStream_t s) {
    quad_wdiff_kernel<<<1024, 256, 0, s>>>(F, dims[0], ndim > 1 ? dims[1] : dims[0], ndim > 2 ? dims[2] : dims[0], ndim,
                                           total, partial);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return launch_sum(partial, 1024, out, s);
}

}  // namespace adsg
