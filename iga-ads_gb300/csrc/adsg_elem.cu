// Element-wise sum-factorised quadrature of the heat form
//     rhs_a += sum_q w_q J_e ( u v_a - dt kappa(x_q) grad u . grad v_a )
// (reference examples/heat/heat_3d.hpp:49-67 with an optional coefficient
// field).  One warp per group of elements (several when an element has fewer
// items per stage than a warp has lanes, see elems_per_warp): each element's
// coefficient tile and its 1D basis/derivative rows (basis_data::b) are
// staged in shared memory, u and
// grad u are interpolated to the q^d points one direction at a time, the
// pointwise form is applied and the result is projected back with the
// transposed 1D factors.  Elements are processed in (p+1)^d colours so that no
// two concurrently processed elements share a dof: the scatter into the
// global RHS is a plain read-modify-write, with no atomics, in a fixed order.
#include <cuda_runtime.h>

#include "adsg_check.cuh"
#include "adsg_kernels.cuh"

namespace adsg {

ADSG_BOUNDS_TU(elem)

// Bounds-checked build: element e[d] inside the grid and its dof box
// first[e] .. first[e] + N - 1 inside the tensor along direction d; every
// gather and scatter of a valid element then stays inside the tensor.
#define ADSG_ELEM_OK(S, X, d)                                                             \
    (ADSG_IN((S).e[d], (X).elements) && ADSG_IN((X).first[(S).e[d]], (X).n) &&           \
     ADSG_IN((X).first[(S).e[d]] + N - 1, (X).n))

namespace {

constexpr int kNoKappa = 0, kKappaCoef = 1, kKappaPoints = 2;

// One element's buffers (the kappa buffers have one entry without KAPPA).
// SHARED lays them out so that buffers whose lives do not overlap share
// storage: the coefficients and the x-contracted T0/T1/K0 ([bz][by][qx]) are
// dead from the pointwise stage until the y back-projection rewrites T0/T1,
// which is exactly while the point values f/g* live.  The smaller tile keeps
// more warps per SM; which layout is faster depends on the form (see
// elem_p).
template <int N, int Q, bool KAPPA, bool SHARED>
struct elem3_smem;

template <int N, int Q, bool KAPPA>
struct elem3_smem<N, Q, KAPPA, false> {
    static constexpr int NK = KAPPA ? 1 : 0;
    double c[N * N * N];
    double kc[NK * N * N * N + 1 - NK];
    double B[3][Q * N];  // B[d][q*N + a]
    double dB[3][Q * N];
    double T0[N * N * Q], T1[N * N * Q];
    double V00[N * Q * Q], V01[N * Q * Q], V10[N * Q * Q];  // [bz][qy][qx]
    double f[Q * Q * Q], gx[Q * Q * Q], gy[Q * Q * Q], gz[Q * Q * Q];
    double K0[NK * N * N * Q + 1 - NK], K1[NK * N * Q * Q + 1 - NK];
    double J;
    long long id;  // index in the colour launch
    int e[3], f0[3];
    int valid;
};

template <int N, int Q, bool KAPPA>
struct elem3_smem<N, Q, KAPPA, true> {
    static constexpr int NK = KAPPA ? 1 : 0;
    double B[3][Q * N];
    double dB[3][Q * N];
    double V00[N * Q * Q], V01[N * Q * Q], V10[N * Q * Q];
    double K1[NK * N * Q * Q + 1 - NK];
    union {
        struct {
            double c[N * N * N], kc[NK * N * N * N + 1 - NK];
            double T0[N * N * Q], T1[N * N * Q], K0[NK * N * N * Q + 1 - NK];
        };
        struct {
            double f[Q * Q * Q], gx[Q * Q * Q], gy[Q * Q * Q], gz[Q * Q * Q];
        };
    };
    double J;
    long long id;  // index in the colour launch
    int e[3], f0[3];
    int valid;
};

// Elements per warp: every stage of the sum factorisation has (p+1)^d or
// (p+1)^a q^b items per element, 27 at p = 2 in 3D; one element per warp
// leaves 5 of 32 lanes idle in every FP64 instruction.  Several elements per
// warp (their items dealt to the lanes in turn) fill the lanes: 7 x 27 = 189
// of 192 lane slots at p = 2.
template <int ITEMS>
constexpr int elems_per_warp() {
    // 27 -> 7 (189 of 192 lane slots), 25 -> 5 (125/128), 16 -> 2, 9 -> 7
    // (63/64), 8 -> 4, 4 -> 8; 64 and 125 items already fill the lanes
    return ITEMS == 27 ? 7
                       : (ITEMS == 25 ? 5
                                      : (ITEMS == 16 ? 2 : (ITEMS == 9 ? 7 : (ITEMS == 8 ? 4 : (ITEMS == 4 ? 8 : 1)))));
}

// warps per block so that the static shared memory stays within 48 KB
template <typename S>
constexpr int warps_for() {
    return sizeof(S) * 4 <= 48 * 1024 ? 4 : (sizeof(S) * 3 <= 48 * 1024 ? 3 : (sizeof(S) * 2 <= 48 * 1024 ? 2 : 1));
}

template <typename S, int EPW>
struct elem_group {
    S el[EPW];
};

// f(S, t) for every item t < ITEMS of every valid element of the warp
// (unrolled: a lane's items are independent, so their loads and FMA chains
// overlap, which is what hides latency with few warps per SM)
template <int ITEMS, int EPW, typename S, typename F>
__device__ __forceinline__ void each_item(S* el, int lane, F&& f) {
    constexpr int kIters = (EPW * ITEMS + 31) / 32;
#pragma unroll
    for (int k = 0; k < kIters; ++k) {
        const int it = lane + 32 * k;
        if (it < EPW * ITEMS) {
            S& e = el[it / ITEMS];
            if (e.valid) f(e, it % ITEMS);
        }
    }
}

// FORM: the general pointwise form of point_form (kappa and dt unused; one
// element per warp, whose D terms are summed across the warp).
// KAPPA: kNoKappa; kKappaCoef, kappa holds the field's spline coefficients,
// interpolated to the Gauss points alongside u; kKappaPoints, kappa holds the
// field's values at every element's Gauss points (kappa_points_kernel, the
// same operations), read in the pointwise stage.
template <int P, int Q, bool FORM, int KAPPA, bool SHARED, int EPW, int kWarpsPerBlock>
__global__ void __launch_bounds__(32 * kWarpsPerBlock)
    elem3_kernel(const double* __restrict__ u, const double* __restrict__ kappa, double* __restrict__ rhs,
                 dim_dev X, dim_dev Y, dim_dev Z, int cx, int cy, int cz, int mx, int my, int mz, double dt,
                 point_form F) {
    constexpr int N = P + 1;
    using S_t = elem3_smem<N, Q, KAPPA == kKappaCoef, SHARED>;
    __shared__ elem_group<S_t, EPW> sm_all[kWarpsPerBlock];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const long long wid = static_cast<long long>(blockIdx.x) * kWarpsPerBlock + warp;
    const long long count = static_cast<long long>(mx) * my * mz;
    if (wid * EPW >= count) return;
    S_t* el = sm_all[warp].el;
    if (lane < EPW) {
        S_t& S = el[lane];
        const long long id = wid * EPW + lane;
        S.id = id;
        S.valid = id < count;
        if (S.valid) {
            const int iz = static_cast<int>(id % mz);
            const int iy = static_cast<int>((id / mz) % my);
            const int ix = static_cast<int>(id / (static_cast<long long>(mz) * my));
            S.e[0] = cx + ix * N;
            S.e[1] = cy + iy * N;
            S.e[2] = cz + iz * N;
            S.valid = ADSG_ELEM_OK(S, X, 0) && ADSG_ELEM_OK(S, Y, 1) && ADSG_ELEM_OK(S, Z, 2);
        }
        if (S.valid) {
            S.f0[0] = X.first[S.e[0]];
            S.f0[1] = Y.first[S.e[1]];
            S.f0[2] = Z.first[S.e[2]];
            S.J = X.jac[S.e[0]] * Y.jac[S.e[1]] * Z.jac[S.e[2]];
        }
    }
    __syncwarp();
    const long long nx = X.n, nxy = static_cast<long long>(X.n) * Y.n;

    // stage coefficients and tables
    each_item<N * N * N, EPW>(el, lane, [&](S_t& S, int t) {
        const int ax = t % N, ay = (t / N) % N, az = t / (N * N);
        const long long g = (S.f0[0] + ax) + nx * (S.f0[1] + ay) + nxy * (S.f0[2] + az);
        S.c[t] = u ? u[g] : 0.0;
        if constexpr (KAPPA == kKappaCoef) S.kc[t] = kappa[g];
    });
    each_item<Q * N, EPW>(el, lane, [&](S_t& S, int t) {
        const int q = t / N, a = t % N;
        const double* bx = X.btab + ((static_cast<long long>(S.e[0]) * Q + q) * 2) * N;
        const double* by = Y.btab + ((static_cast<long long>(S.e[1]) * Q + q) * 2) * N;
        const double* bz = Z.btab + ((static_cast<long long>(S.e[2]) * Q + q) * 2) * N;
        S.B[0][t] = bx[a];
        S.dB[0][t] = bx[N + a];
        S.B[1][t] = by[a];
        S.dB[1][t] = by[N + a];
        S.B[2][t] = bz[a];
        S.dB[2][t] = bz[N + a];
    });
    __syncwarp();
    // x: T0/T1[bz][by][qx]
    each_item<N * N * Q, EPW>(el, lane, [&](S_t& S, int t) {
        const int qx = t % Q, byz = t / Q;
        double a0 = 0.0, a1 = 0.0, k0 = 0.0;
#pragma unroll
        for (int b = 0; b < N; ++b) {
            const double cv = S.c[byz * N + b];
            a0 = fma(S.B[0][qx * N + b], cv, a0);
            a1 = fma(S.dB[0][qx * N + b], cv, a1);
            if constexpr (KAPPA == kKappaCoef) k0 = fma(S.B[0][qx * N + b], S.kc[byz * N + b], k0);
        }
        S.T0[t] = a0;
        S.T1[t] = a1;
        if constexpr (KAPPA == kKappaCoef) S.K0[t] = k0;
    });
    __syncwarp();
    // y: V..[bz][qy][qx]
    each_item<N * Q * Q, EPW>(el, lane, [&](S_t& S, int t) {
        const int qx = t % Q, qy = (t / Q) % Q, bz = t / (Q * Q);
        double v00 = 0.0, v01 = 0.0, v10 = 0.0, k1 = 0.0;
#pragma unroll
        for (int b = 0; b < N; ++b) {
            const int src = (bz * N + b) * Q + qx;
            const double by = S.B[1][qy * N + b], dby = S.dB[1][qy * N + b];
            v00 = fma(by, S.T0[src], v00);
            v01 = fma(dby, S.T0[src], v01);
            v10 = fma(by, S.T1[src], v10);
            if constexpr (KAPPA == kKappaCoef) k1 = fma(by, S.K0[src], k1);
        }
        S.V00[t] = v00;
        S.V01[t] = v01;
        S.V10[t] = v10;
        if constexpr (KAPPA == kKappaCoef) S.K1[t] = k1;
    });
    __syncwarp();
    // z + pointwise form: f = W u, g* = -dt kappa W d*u
    // (FORM: f = W (alpha u + gamma), g* = W beta d*u, and W delta summed)
    double dsum = 0.0;
    each_item<Q * Q * Q, EPW>(el, lane, [&](S_t& S, int t) {
        const int qx = t % Q, qy = (t / Q) % Q, qz = t / (Q * Q);
        double uv = 0.0, ux = 0.0, uy = 0.0, uz = 0.0, kv = 0.0;
        // this colour's block: the warp's elements are consecutive; issued
        // before the contraction so that it arrives during it
        if constexpr (KAPPA == kKappaPoints) kv = kappa[S.id * (Q * Q * Q) + t];
#pragma unroll
        for (int b = 0; b < N; ++b) {
            const int src = (b * Q + qy) * Q + qx;
            const double bz = S.B[2][qz * N + b], dbz = S.dB[2][qz * N + b];
            uv = fma(bz, S.V00[src], uv);
            uz = fma(dbz, S.V00[src], uz);
            uy = fma(bz, S.V01[src], uy);
            ux = fma(bz, S.V10[src], ux);
            if constexpr (KAPPA == kKappaCoef) kv = fma(bz, S.K1[src], kv);
        }
        const double W = X.wq[qx] * Y.wq[qy] * Z.wq[qz] * S.J;
        if (FORM) {
            const long long Qx = static_cast<long long>(X.elements) * Q, Qy = static_cast<long long>(Y.elements) * Q;
            const long long pq = (static_cast<long long>(S.e[0]) * Q + qx) +
                                 Qx * ((static_cast<long long>(S.e[1]) * Q + qy) +
                                       Qy * (static_cast<long long>(S.e[2]) * Q + qz));
            const double al = F.alpha + (F.alpha_q ? F.alpha_q[pq] : 0.0);
            const double be = F.beta + (F.beta_q ? F.beta_q[pq] : 0.0);
            const double ga = F.gamma + (F.gamma_q ? F.gamma_q[pq] : 0.0);
            const double de = F.delta + (F.delta_q ? F.delta_q[pq] : 0.0);
            const double g = be * W;
            S.f[t] = fma(al, uv, ga) * W;
            S.gx[t] = ux * g;
            S.gy[t] = uy * g;
            S.gz[t] = uz * g;
            dsum = fma(de, W, dsum);
        } else {
            const double g = (KAPPA != kNoKappa ? -dt * kv : -dt) * W;
            S.f[t] = uv * W;
            S.gx[t] = ux * g;
            S.gy[t] = uy * g;
            S.gz[t] = uz * g;
        }
    });
    if (FORM) {  // one element per warp
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) dsum += __shfl_xor_sync(0xffffffffu, dsum, off);
    }
    __syncwarp();
    // z back: V00 <- S0[az][qy][qx], V01 <- Sx, V10 <- Sy
    each_item<N * Q * Q, EPW>(el, lane, [&](S_t& S, int t) {
        const int qx = t % Q, qy = (t / Q) % Q, az = t / (Q * Q);
        double s0 = 0.0, sx = 0.0, sy = 0.0;
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            const int src = (q * Q + qy) * Q + qx;
            const double bz = S.B[2][q * N + az], dbz = S.dB[2][q * N + az];
            s0 = fma(bz, S.f[src], s0);
            s0 = fma(dbz, S.gz[src], s0);
            sx = fma(bz, S.gx[src], sx);
            sy = fma(bz, S.gy[src], sy);
        }
        S.V00[t] = s0;
        S.V01[t] = sx;
        S.V10[t] = sy;
    });
    __syncwarp();
    // y back: T0 <- R0[az][ay][qx], T1 <- Rx
    each_item<N * N * Q, EPW>(el, lane, [&](S_t& S, int t) {
        const int qx = t % Q, ay = (t / Q) % N, az = t / (Q * N);
        double r0 = 0.0, rx = 0.0;
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            const int src = (az * Q + q) * Q + qx;
            const double by = S.B[1][q * N + ay], dby = S.dB[1][q * N + ay];
            r0 = fma(by, S.V00[src], r0);
            r0 = fma(dby, S.V10[src], r0);
            rx = fma(by, S.V01[src], rx);
        }
        S.T0[t] = r0;
        S.T1[t] = rx;
    });
    __syncwarp();
    // x back and scatter (this colour owns every dof of the element)
    each_item<N * N * N, EPW>(el, lane, [&](S_t& S, int t) {
        const int ax = t % N, ay = (t / N) % N, az = t / (N * N);
        double o = 0.0;
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            const int src = (az * N + ay) * Q + q;
            o = fma(S.B[0][q * N + ax], S.T0[src], o);
            o = fma(S.dB[0][q * N + ax], S.T1[src], o);
        }
        const long long g = (S.f0[0] + ax) + nx * (S.f0[1] + ay) + nxy * (S.f0[2] + az);
        rhs[g] += FORM ? o + dsum : o;
    });
}

template <int N, int Q>
struct elem2_smem {
    double c[N * N], kc[N * N];
    double B[2][Q * N], dB[2][Q * N];
    double T0[N * Q], T1[N * Q], K0[N * Q];  // [by][qx]
    double f[Q * Q], gx[Q * Q], gy[Q * Q];
    double J;
    int e[2], f0[2];
    int valid;
};

template <int P, int Q, bool FORM = false, int EPW = (FORM ? 1 : elems_per_warp<(P + 1) * (P + 1)>()),
          int kWarpsPerBlock = warps_for<elem_group<elem2_smem<P + 1, Q>, EPW>>()>
__global__ void __launch_bounds__(32 * kWarpsPerBlock)
    elem2_kernel(const double* __restrict__ u, const double* __restrict__ kappa, double* __restrict__ rhs,
                 dim_dev X, dim_dev Y, int cx, int cy, int mx, int my, double dt, point_form F) {
    constexpr int N = P + 1;
    using S_t = elem2_smem<N, Q>;
    __shared__ elem_group<S_t, EPW> sm_all[kWarpsPerBlock];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const long long wid = static_cast<long long>(blockIdx.x) * kWarpsPerBlock + warp;
    const long long count = static_cast<long long>(mx) * my;
    if (wid * EPW >= count) return;
    S_t* el = sm_all[warp].el;
    if (lane < EPW) {
        S_t& S = el[lane];
        const long long id = wid * EPW + lane;
        S.valid = id < count;
        if (S.valid) {
            S.e[0] = cx + static_cast<int>(id / my) * N;
            S.e[1] = cy + static_cast<int>(id % my) * N;
            S.valid = ADSG_ELEM_OK(S, X, 0) && ADSG_ELEM_OK(S, Y, 1);
        }
        if (S.valid) {
            S.f0[0] = X.first[S.e[0]];
            S.f0[1] = Y.first[S.e[1]];
            S.J = X.jac[S.e[0]] * Y.jac[S.e[1]];
        }
    }
    __syncwarp();
    const long long nx = X.n;
    each_item<N * N, EPW>(el, lane, [&](S_t& S, int t) {
        const long long g = (S.f0[0] + t % N) + nx * (S.f0[1] + t / N);
        S.c[t] = u ? u[g] : 0.0;
        S.kc[t] = kappa ? kappa[g] : 0.0;
    });
    each_item<Q * N, EPW>(el, lane, [&](S_t& S, int t) {
        const int q = t / N, a = t % N;
        const double* bx = X.btab + ((static_cast<long long>(S.e[0]) * Q + q) * 2) * N;
        const double* by = Y.btab + ((static_cast<long long>(S.e[1]) * Q + q) * 2) * N;
        S.B[0][t] = bx[a];
        S.dB[0][t] = bx[N + a];
        S.B[1][t] = by[a];
        S.dB[1][t] = by[N + a];
    });
    __syncwarp();
    each_item<N * Q, EPW>(el, lane, [&](S_t& S, int t) {
        const int qx = t % Q, by = t / Q;
        double a0 = 0.0, a1 = 0.0, k0 = 0.0;
#pragma unroll
        for (int b = 0; b < N; ++b) {
            a0 = fma(S.B[0][qx * N + b], S.c[by * N + b], a0);
            a1 = fma(S.dB[0][qx * N + b], S.c[by * N + b], a1);
            if (kappa) k0 = fma(S.B[0][qx * N + b], S.kc[by * N + b], k0);
        }
        S.T0[t] = a0;
        S.T1[t] = a1;
        if (kappa) S.K0[t] = k0;
    });
    __syncwarp();
    double dsum = 0.0;
    each_item<Q * Q, EPW>(el, lane, [&](S_t& S, int t) {
        const int qx = t % Q, qy = t / Q;
        double uv = 0.0, ux = 0.0, uy = 0.0, kv = 0.0;
#pragma unroll
        for (int b = 0; b < N; ++b) {
            const double by = S.B[1][qy * N + b], dby = S.dB[1][qy * N + b];
            uv = fma(by, S.T0[b * Q + qx], uv);
            uy = fma(dby, S.T0[b * Q + qx], uy);
            ux = fma(by, S.T1[b * Q + qx], ux);
            if (kappa) kv = fma(by, S.K0[b * Q + qx], kv);
        }
        const double W = X.wq[qx] * Y.wq[qy] * S.J;
        if (FORM) {
            const long long Qx = static_cast<long long>(X.elements) * Q;
            const long long pq =
                (static_cast<long long>(S.e[0]) * Q + qx) + Qx * (static_cast<long long>(S.e[1]) * Q + qy);
            const double al = F.alpha + (F.alpha_q ? F.alpha_q[pq] : 0.0);
            const double be = F.beta + (F.beta_q ? F.beta_q[pq] : 0.0);
            const double ga = F.gamma + (F.gamma_q ? F.gamma_q[pq] : 0.0);
            const double de = F.delta + (F.delta_q ? F.delta_q[pq] : 0.0);
            const double g = be * W;
            S.f[t] = fma(al, uv, ga) * W;
            S.gx[t] = ux * g;
            S.gy[t] = uy * g;
            dsum = fma(de, W, dsum);
        } else {
            const double g = (kappa ? -dt * kv : -dt) * W;
            S.f[t] = uv * W;
            S.gx[t] = ux * g;
            S.gy[t] = uy * g;
        }
    });
    if (FORM) {  // one element per warp
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) dsum += __shfl_xor_sync(0xffffffffu, dsum, off);
    }
    __syncwarp();
    // y back: T0 <- S0[ay][qx], T1 <- Sx
    each_item<N * Q, EPW>(el, lane, [&](S_t& S, int t) {
        const int qx = t % Q, ay = t / Q;
        double s0 = 0.0, sx = 0.0;
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            const double by = S.B[1][q * N + ay], dby = S.dB[1][q * N + ay];
            s0 = fma(by, S.f[q * Q + qx], s0);
            s0 = fma(dby, S.gy[q * Q + qx], s0);
            sx = fma(by, S.gx[q * Q + qx], sx);
        }
        S.T0[t] = s0;
        S.T1[t] = sx;
    });
    __syncwarp();
    each_item<N * N, EPW>(el, lane, [&](S_t& S, int t) {
        const int ax = t % N, ay = t / N;
        double o = 0.0;
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            o = fma(S.B[0][q * N + ax], S.T0[ay * Q + q], o);
            o = fma(S.dB[0][q * N + ax], S.T1[ay * Q + q], o);
        }
        rhs[(S.f0[0] + ax) + nx * (S.f0[1] + ay)] += FORM ? o + dsum : o;
    });
}

// ---------------------------------------------------------------------------
// One backward step of the adjoint in one pass over the elements: both
// element operations that read mu = M^-T lambda,
//     r_a += sum_q W (mu v_a - dt kappa grad mu . grad v_a)        (R(kappa) mu)
//     g_a += sum_q -dt W (grad u . grad mu) v_a                     (dL/dkappa)
// share mu's interpolation to the Gauss points (value and gradient), which
// a separate gradient pass would repeat.  The R(kappa) mu accumulators take
// elem3_kernel's operations (with kappa) in its order, so that part is
// bitwise elem3_kernel's; the gradient interpolates grad u and grad mu
// direction by direction and projects the pointwise product onto the value
// factors (kgrad2_kernel's scheme in 3D).  Buffers whose
// lives do not overlap share storage: the coefficients with the y
// back-projection's results, the x stage's results with the point values,
// the y stage's results with the z back-projection's.
// ---------------------------------------------------------------------------
template <int N, int Q>
struct adj3_smem {
    double B[3][Q * N], dB[3][Q * N];
    union {
        struct {
            double cm[N * N * N], cu[N * N * N], kc[N * N * N];
        };
        struct {
            double R0[N * N * Q], Rx[N * N * Q], Ra[N * N * Q];  // [az][ay][qx]
        };
    };
    union {
        struct {
            double Tm0[N * N * Q], Tm1[N * N * Q], Tu0[N * N * Q], Tu1[N * N * Q], K0[N * N * Q];  // [bz][by][qx]
        };
        struct {
            double f[Q * Q * Q], gx[Q * Q * Q], gy[Q * Q * Q], gz[Q * Q * Q], sk[Q * Q * Q];
        };
    };
    union {
        struct {
            double Vm00[N * Q * Q], Vm01[N * Q * Q], Vm10[N * Q * Q];  // [bz][qy][qx]
            double Vu00[N * Q * Q], Vu01[N * Q * Q], Vu10[N * Q * Q], K1[N * Q * Q];
        };
        struct {
            double S0[N * Q * Q], Sx[N * Q * Q], Sy[N * Q * Q], Sa[N * Q * Q];  // [az][qy][qx]
        };
    };
    double J;
    long long id;  // index in the colour launch
    int e[3], f0[3];
    int valid;
};

// KP: kappa holds the field's values at the Gauss points (this colour's block
// of kappa_points_kernel's output) instead of its coefficients.
template <int P, int Q, bool KP = false, int EPW = elems_per_warp<(P + 1) * (P + 1) * (P + 1)>(),
          int kWarpsPerBlock = warps_for<elem_group<adj3_smem<P + 1, Q>, EPW>>()>
__global__ void __launch_bounds__(32 * kWarpsPerBlock)
    adj3_kernel(const double* __restrict__ u, const double* __restrict__ mu, const double* __restrict__ kappa,
                double* __restrict__ rmu, double* __restrict__ g, dim_dev X, dim_dev Y, dim_dev Z, int cx, int cy,
                int cz, int mx, int my, int mz, double dt) {
    constexpr int N = P + 1;
    using S_t = adj3_smem<N, Q>;
    __shared__ elem_group<S_t, EPW> sm_all[kWarpsPerBlock];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const long long wid = static_cast<long long>(blockIdx.x) * kWarpsPerBlock + warp;
    const long long count = static_cast<long long>(mx) * my * mz;
    if (wid * EPW >= count) return;
    S_t* el = sm_all[warp].el;
    if (lane < EPW) {
        S_t& S = el[lane];
        const long long id = wid * EPW + lane;
        S.id = id;
        S.valid = id < count;
        if (S.valid) {
            const int iz = static_cast<int>(id % mz);
            const int iy = static_cast<int>((id / mz) % my);
            const int ix = static_cast<int>(id / (static_cast<long long>(mz) * my));
            S.e[0] = cx + ix * N;
            S.e[1] = cy + iy * N;
            S.e[2] = cz + iz * N;
            S.valid = ADSG_ELEM_OK(S, X, 0) && ADSG_ELEM_OK(S, Y, 1) && ADSG_ELEM_OK(S, Z, 2);
        }
        if (S.valid) {
            S.f0[0] = X.first[S.e[0]];
            S.f0[1] = Y.first[S.e[1]];
            S.f0[2] = Z.first[S.e[2]];
            S.J = X.jac[S.e[0]] * Y.jac[S.e[1]] * Z.jac[S.e[2]];
        }
    }
    __syncwarp();
    const long long nx = X.n, nxy = static_cast<long long>(X.n) * Y.n;
    each_item<N * N * N, EPW>(el, lane, [&](S_t& S, int t) {
        const int ax = t % N, ay = (t / N) % N, az = t / (N * N);
        const long long gi = (S.f0[0] + ax) + nx * (S.f0[1] + ay) + nxy * (S.f0[2] + az);
        S.cm[t] = mu[gi];
        S.cu[t] = u[gi];
        if constexpr (!KP) S.kc[t] = kappa[gi];
    });
    each_item<Q * N, EPW>(el, lane, [&](S_t& S, int t) {
        const int q = t / N, a = t % N;
        const double* bx = X.btab + ((static_cast<long long>(S.e[0]) * Q + q) * 2) * N;
        const double* by = Y.btab + ((static_cast<long long>(S.e[1]) * Q + q) * 2) * N;
        const double* bz = Z.btab + ((static_cast<long long>(S.e[2]) * Q + q) * 2) * N;
        S.B[0][t] = bx[a];
        S.dB[0][t] = bx[N + a];
        S.B[1][t] = by[a];
        S.dB[1][t] = by[N + a];
        S.B[2][t] = bz[a];
        S.dB[2][t] = bz[N + a];
    });
    __syncwarp();
    // x: mu's value/derivative factors (elem3_kernel's T0/T1), kappa's (K0), u's (Tu0/Tu1)
    each_item<N * N * Q, EPW>(el, lane, [&](S_t& S, int t) {
        const int qx = t % Q, byz = t / Q;
        double a0 = 0.0, a1 = 0.0, k0 = 0.0, b0 = 0.0, b1 = 0.0;
#pragma unroll
        for (int b = 0; b < N; ++b) {
            const double bv = S.B[0][qx * N + b], dv = S.dB[0][qx * N + b];
            const double cv = S.cm[byz * N + b], uv = S.cu[byz * N + b];
            a0 = fma(bv, cv, a0);
            a1 = fma(dv, cv, a1);
            if constexpr (!KP) k0 = fma(bv, S.kc[byz * N + b], k0);
            b0 = fma(bv, uv, b0);
            b1 = fma(dv, uv, b1);
        }
        S.Tm0[t] = a0;
        S.Tm1[t] = a1;
        if constexpr (!KP) S.K0[t] = k0;
        S.Tu0[t] = b0;
        S.Tu1[t] = b1;
    });
    __syncwarp();
    // y
    each_item<N * Q * Q, EPW>(el, lane, [&](S_t& S, int t) {
        const int qx = t % Q, qy = (t / Q) % Q, bz = t / (Q * Q);
        double v00 = 0.0, v01 = 0.0, v10 = 0.0, k1 = 0.0, u00 = 0.0, u01 = 0.0, u10 = 0.0;
#pragma unroll
        for (int b = 0; b < N; ++b) {
            const int src = (bz * N + b) * Q + qx;
            const double by = S.B[1][qy * N + b], dby = S.dB[1][qy * N + b];
            v00 = fma(by, S.Tm0[src], v00);
            v01 = fma(dby, S.Tm0[src], v01);
            v10 = fma(by, S.Tm1[src], v10);
            if constexpr (!KP) k1 = fma(by, S.K0[src], k1);
            u00 = fma(by, S.Tu0[src], u00);
            u01 = fma(dby, S.Tu0[src], u01);
            u10 = fma(by, S.Tu1[src], u10);
        }
        S.Vm00[t] = v00;
        S.Vm01[t] = v01;
        S.Vm10[t] = v10;
        if constexpr (!KP) S.K1[t] = k1;
        S.Vu00[t] = u00;
        S.Vu01[t] = u01;
        S.Vu10[t] = u10;
    });
    __syncwarp();
    // z + both pointwise forms
    each_item<Q * Q * Q, EPW>(el, lane, [&](S_t& S, int t) {
        const int qx = t % Q, qy = (t / Q) % Q, qz = t / (Q * Q);
        double mv = 0.0, mx_ = 0.0, my_ = 0.0, mz_ = 0.0, kv = 0.0, ux = 0.0, uy = 0.0, uz = 0.0;
#pragma unroll
        for (int b = 0; b < N; ++b) {
            const int src = (b * Q + qy) * Q + qx;
            const double bz = S.B[2][qz * N + b], dbz = S.dB[2][qz * N + b];
            mv = fma(bz, S.Vm00[src], mv);
            mz_ = fma(dbz, S.Vm00[src], mz_);
            my_ = fma(bz, S.Vm01[src], my_);
            mx_ = fma(bz, S.Vm10[src], mx_);
            if constexpr (!KP) kv = fma(bz, S.K1[src], kv);
            uz = fma(dbz, S.Vu00[src], uz);
            uy = fma(bz, S.Vu01[src], uy);
            ux = fma(bz, S.Vu10[src], ux);
        }
        if constexpr (KP) kv = kappa[S.id * (Q * Q * Q) + t];
        const double W = X.wq[qx] * Y.wq[qy] * Z.wq[qz] * S.J;
        const double gk = (-dt * kv) * W;
        S.f[t] = mv * W;
        S.gx[t] = mx_ * gk;
        S.gy[t] = my_ * gk;
        S.gz[t] = mz_ * gk;
        S.sk[t] = -dt * W * (ux * mx_ + uy * my_ + uz * mz_);
    });
    __syncwarp();
    // z back: R(kappa) mu with value and derivative factors, the kappa gradient with value factors
    each_item<N * Q * Q, EPW>(el, lane, [&](S_t& S, int t) {
        const int qx = t % Q, qy = (t / Q) % Q, az = t / (Q * Q);
        double s0 = 0.0, sx = 0.0, sy = 0.0, sa = 0.0;
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            const int src = (q * Q + qy) * Q + qx;
            const double bz = S.B[2][q * N + az], dbz = S.dB[2][q * N + az];
            s0 = fma(bz, S.f[src], s0);
            s0 = fma(dbz, S.gz[src], s0);
            sx = fma(bz, S.gx[src], sx);
            sy = fma(bz, S.gy[src], sy);
            sa = fma(bz, S.sk[src], sa);
        }
        S.S0[t] = s0;
        S.Sx[t] = sx;
        S.Sy[t] = sy;
        S.Sa[t] = sa;
    });
    __syncwarp();
    // y back
    each_item<N * N * Q, EPW>(el, lane, [&](S_t& S, int t) {
        const int qx = t % Q, ay = (t / Q) % N, az = t / (Q * N);
        double r0 = 0.0, rx = 0.0, ra = 0.0;
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            const int src = (az * Q + q) * Q + qx;
            const double by = S.B[1][q * N + ay], dby = S.dB[1][q * N + ay];
            r0 = fma(by, S.S0[src], r0);
            r0 = fma(dby, S.Sy[src], r0);
            rx = fma(by, S.Sx[src], rx);
            ra = fma(by, S.Sa[src], ra);
        }
        S.R0[t] = r0;
        S.Rx[t] = rx;
        S.Ra[t] = ra;
    });
    __syncwarp();
    // x back and both scatters (this colour owns every dof of the element)
    each_item<N * N * N, EPW>(el, lane, [&](S_t& S, int t) {
        const int ax = t % N, ay = (t / N) % N, az = t / (N * N);
        double o = 0.0, a = 0.0;
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            const int src = (az * N + ay) * Q + q;
            o = fma(S.B[0][q * N + ax], S.R0[src], o);
            o = fma(S.dB[0][q * N + ax], S.Rx[src], o);
            a = fma(S.B[0][q * N + ax], S.Ra[src], a);
        }
        const long long gi = (S.f0[0] + ax) + nx * (S.f0[1] + ay) + nxy * (S.f0[2] + az);
        rmu[gi] += o;
        g[gi] += a;
    });
}

// ---------------------------------------------------------------------------
// Gradient of a quadratic functional with respect to the diffusion field, 2D:
//     g_c += -dt sum_e sum_q W B_c(x_q) grad u(x_q) . grad mu(x_q)
// i.e. mu^T (dR/dkappa_c) u for the operator R(kappa) applied by the element
// kernels above.  Same sum factorisation and colouring: gradients of u and
// mu are interpolated direction by direction, the pointwise product is formed
// and projected onto the value factors.  (3D runs this inside adj3_kernel.)
// ---------------------------------------------------------------------------
template <int N, int Q>
struct kg2_smem {
    double c[N * N], m[N * N];
    double B[2][Q * N], dB[2][Q * N];
    double Tu0[N * Q], Tu1[N * Q], Tm0[N * Q], Tm1[N * Q];
    double s[Q * Q];
    double J;
    int e[2], f0[2];
    int valid;
};

template <int P, int Q, int EPW = elems_per_warp<(P + 1) * (P + 1)>(),
          int kWarpsPerBlock = warps_for<elem_group<kg2_smem<P + 1, Q>, EPW>>()>
__global__ void __launch_bounds__(32 * kWarpsPerBlock)
    kgrad2_kernel(const double* __restrict__ u, const double* __restrict__ mu, double* __restrict__ g, dim_dev X,
                  dim_dev Y, int cx, int cy, int mx, int my, double dt) {
    constexpr int N = P + 1;
    using S_t = kg2_smem<N, Q>;
    __shared__ elem_group<S_t, EPW> sm_all[kWarpsPerBlock];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const long long wid = static_cast<long long>(blockIdx.x) * kWarpsPerBlock + warp;
    const long long count = static_cast<long long>(mx) * my;
    if (wid * EPW >= count) return;
    S_t* el = sm_all[warp].el;
    if (lane < EPW) {
        S_t& S = el[lane];
        const long long id = wid * EPW + lane;
        S.valid = id < count;
        if (S.valid) {
            S.e[0] = cx + static_cast<int>(id / my) * N;
            S.e[1] = cy + static_cast<int>(id % my) * N;
            S.valid = ADSG_ELEM_OK(S, X, 0) && ADSG_ELEM_OK(S, Y, 1);
        }
        if (S.valid) {
            S.f0[0] = X.first[S.e[0]];
            S.f0[1] = Y.first[S.e[1]];
            S.J = X.jac[S.e[0]] * Y.jac[S.e[1]];
        }
    }
    __syncwarp();
    const long long nx = X.n;
    each_item<N * N, EPW>(el, lane, [&](S_t& S, int t) {
        const long long gi = (S.f0[0] + t % N) + nx * (S.f0[1] + t / N);
        S.c[t] = u[gi];
        S.m[t] = mu[gi];
    });
    each_item<Q * N, EPW>(el, lane, [&](S_t& S, int t) {
        const int q = t / N, a = t % N;
        const double* bx = X.btab + ((static_cast<long long>(S.e[0]) * Q + q) * 2) * N;
        const double* by = Y.btab + ((static_cast<long long>(S.e[1]) * Q + q) * 2) * N;
        S.B[0][t] = bx[a];
        S.dB[0][t] = bx[N + a];
        S.B[1][t] = by[a];
        S.dB[1][t] = by[N + a];
    });
    __syncwarp();
    each_item<N * Q, EPW>(el, lane, [&](S_t& S, int t) {
        const int qx = t % Q, by = t / Q;
        double a0 = 0.0, a1 = 0.0, b0 = 0.0, b1 = 0.0;
#pragma unroll
        for (int b = 0; b < N; ++b) {
            const double bv = S.B[0][qx * N + b], dv = S.dB[0][qx * N + b];
            a0 = fma(bv, S.c[by * N + b], a0);
            a1 = fma(dv, S.c[by * N + b], a1);
            b0 = fma(bv, S.m[by * N + b], b0);
            b1 = fma(dv, S.m[by * N + b], b1);
        }
        S.Tu0[t] = a0;
        S.Tu1[t] = a1;
        S.Tm0[t] = b0;
        S.Tm1[t] = b1;
    });
    __syncwarp();
    each_item<Q * Q, EPW>(el, lane, [&](S_t& S, int t) {
        const int qx = t % Q, qy = t / Q;
        double ux = 0.0, uy = 0.0, mx_ = 0.0, my_ = 0.0;
#pragma unroll
        for (int b = 0; b < N; ++b) {
            const double by = S.B[1][qy * N + b], dby = S.dB[1][qy * N + b];
            uy = fma(dby, S.Tu0[b * Q + qx], uy);
            ux = fma(by, S.Tu1[b * Q + qx], ux);
            my_ = fma(dby, S.Tm0[b * Q + qx], my_);
            mx_ = fma(by, S.Tm1[b * Q + qx], mx_);
        }
        const double W = X.wq[qx] * Y.wq[qy] * S.J;
        S.s[t] = -dt * W * (ux * mx_ + uy * my_);
    });
    __syncwarp();
    each_item<N * Q, EPW>(el, lane, [&](S_t& S, int t) {
        const int qx = t % Q, ay = t / Q;
        double a = 0.0;
#pragma unroll
        for (int q = 0; q < Q; ++q) a = fma(S.B[1][q * N + ay], S.s[q * Q + qx], a);
        S.Tu0[t] = a;
    });
    __syncwarp();
    each_item<N * N, EPW>(el, lane, [&](S_t& S, int t) {
        const int ax = t % N, ay = t / N;
        double a = 0.0;
#pragma unroll
        for (int q = 0; q < Q; ++q) a = fma(S.B[0][q * N + ax], S.Tu0[ay * Q + q], a);
        g[(S.f0[0] + ax) + nx * (S.f0[1] + ay)] += a;
    });
}

__host__ __device__ inline int colour_count(int E, int c, int N) { return E > c ? (E - c + N - 1) / N : 0; }

// Elements before colour (cx, cy, cz) in the launch order of the colours (cx
// outermost, cz innermost): where that colour's block of Gauss-point kappa
// values starts, in elements.
__host__ __device__ inline long long colour_base(int Ex, int Ey, int Ez, int N, int cx, int cy, int cz) {
    long long sx = 0, sy = 0, sz = 0;
    for (int c = 0; c < cx; ++c) sx += colour_count(Ex, c, N);
    for (int c = 0; c < cy; ++c) sy += colour_count(Ey, c, N);
    for (int c = 0; c < cz; ++c) sz += colour_count(Ez, c, N);
    const long long mx = colour_count(Ex, cx, N), my = colour_count(Ey, cy, N);
    return sx * Ey * Ez + mx * (sy * Ez + my * sz);
}

// kappa_points: kappa holds the field at the Gauss points (3D only).
template <int P, bool FORM>
cudaError_t elem_p(int ndim, const dim_dev* d, const double* u, const double* kappa, double* rhs, double dt,
                   const point_form& F, cudaStream_t s, bool kappa_points = false) {
    if (kappa_points && (ndim != 3 || FORM || !kappa)) return cudaErrorNotSupported;
    constexpr int N = P + 1, Q = P + 1;
    constexpr int E3 = FORM ? 1 : elems_per_warp<N * N * N>();
    constexpr int E2 = FORM ? 1 : elems_per_warp<N * N>();
    // tile layouts and block shapes by measurement, one warp per block: shared
    // storage without kappa (128^3 p=2: 6.68 ms per evaluation, against 6.95
    // with three warps per block and 7.83 with separate buffers); with kappa
    // separate buffers (200 adjoint forward steps at 96^3 p=2: 713 ms, against
    // 742 with two warps per block, 785-796 with shared storage, 840 with 4
    // elements per warp)
    constexpr bool kShared = true, kSharedKappa = false;
    constexpr int E3k = FORM ? 1 : elems_per_warp<N * N * N>();
    constexpr int W3 = FORM ? warps_for<elem_group<elem3_smem<N, Q, false, kShared>, E3>>() : 1;
    constexpr int W3k = 1;
    constexpr int W2 = warps_for<elem_group<elem2_smem<N, Q>, E2>>();
    if (ndim == 3) {
        for (int cx = 0; cx < N; ++cx)
            for (int cy = 0; cy < N; ++cy)
                for (int cz = 0; cz < N; ++cz) {
                    const int mx = colour_count(d[0].elements, cx, N), my = colour_count(d[1].elements, cy, N),
                              mz = colour_count(d[2].elements, cz, N);
                    const long long work = static_cast<long long>(mx) * my * mz;
                    if (!work) continue;
                    if (kappa_points) {
                        // the tile without kappa buffers, as without kappa
                        const long long blocks = ((work + E3 - 1) / E3 + W3 - 1) / W3;
                        const double* kc = kappa + colour_base(d[0].elements, d[1].elements, d[2].elements, N, cx, cy,
                                                               cz) * (Q * Q * Q);
                        elem3_kernel<P, Q, FORM, kKappaPoints, kShared, E3, W3><<<blocks, 32 * W3, 0, s>>>(
                            u, kc, rhs, d[0], d[1], d[2], cx, cy, cz, mx, my, mz, dt, F);
                    } else if (!FORM && kappa) {
                        const long long blocks = ((work + E3k - 1) / E3k + W3k - 1) / W3k;
                        elem3_kernel<P, Q, FORM, kKappaCoef, kSharedKappa, E3k, W3k><<<blocks, 32 * W3k, 0, s>>>(
                            u, kappa, rhs, d[0], d[1], d[2], cx, cy, cz, mx, my, mz, dt, F);
                    } else {
                        const long long blocks = ((work + E3 - 1) / E3 + W3 - 1) / W3;
                        elem3_kernel<P, Q, FORM, kNoKappa, kShared, E3, W3><<<blocks, 32 * W3, 0, s>>>(
                            u, kappa, rhs, d[0], d[1], d[2], cx, cy, cz, mx, my, mz, dt, F);
                    }
                }
    } else {
        for (int cx = 0; cx < N; ++cx)
            for (int cy = 0; cy < N; ++cy) {
                const int mx = colour_count(d[0].elements, cx, N), my = colour_count(d[1].elements, cy, N);
                const long long work = static_cast<long long>(mx) * my;
                if (!work) continue;
                const long long blocks = ((work + E2 - 1) / E2 + W2 - 1) / W2;
                elem2_kernel<P, Q, FORM><<<blocks, 32 * W2, 0, s>>>(u, kappa, rhs, d[0], d[1], cx, cy, mx, my, dt, F);
            }
    }
    return cudaGetLastError();
}

template <int P>
cudaError_t kgrad2_p(const dim_dev* d, const double* u, const double* mu, double* g, double dt, cudaStream_t s) {
    constexpr int N = P + 1, Q = P + 1;
    constexpr int E2 = elems_per_warp<N * N>();
    constexpr int W2 = warps_for<elem_group<kg2_smem<N, Q>, E2>>();
    for (int cx = 0; cx < N; ++cx)
        for (int cy = 0; cy < N; ++cy) {
            const int mx = colour_count(d[0].elements, cx, N), my = colour_count(d[1].elements, cy, N);
            const long long work = static_cast<long long>(mx) * my;
            if (!work) continue;
            kgrad2_kernel<P, Q><<<((work + E2 - 1) / E2 + W2 - 1) / W2, 32 * W2, 0, s>>>(u, mu, g, d[0], d[1], cx, cy, mx,
                                                                                       my, dt);
        }
    return cudaGetLastError();
}

template <int P>
cudaError_t adj3_p(const dim_dev* d, const double* u, const double* mu, const double* kappa, double* rmu, double* g,
                   double dt, cudaStream_t s, bool kappa_points) {
    constexpr int N = P + 1, Q = P + 1;
    constexpr int E3 = elems_per_warp<N * N * N>();
    constexpr int W3 = warps_for<elem_group<adj3_smem<N, Q>, E3>>();
    for (int cx = 0; cx < N; ++cx)
        for (int cy = 0; cy < N; ++cy)
            for (int cz = 0; cz < N; ++cz) {
                const int mx = colour_count(d[0].elements, cx, N), my = colour_count(d[1].elements, cy, N),
                          mz = colour_count(d[2].elements, cz, N);
                const long long work = static_cast<long long>(mx) * my * mz;
                if (!work) continue;
                const long long blocks = ((work + E3 - 1) / E3 + W3 - 1) / W3;
                if (kappa_points)
                    adj3_kernel<P, Q, true><<<blocks, 32 * W3, 0, s>>>(
                        u, mu,
                        kappa + colour_base(d[0].elements, d[1].elements, d[2].elements, N, cx, cy, cz) * (Q * Q * Q),
                        rmu, g, d[0], d[1], d[2], cx, cy, cz, mx, my, mz, dt);
                else
                    adj3_kernel<P, Q><<<blocks, 32 * W3, 0, s>>>(u, mu, kappa, rmu, g, d[0], d[1], d[2], cx, cy, cz,
                                                                 mx, my, mz, dt);
            }
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_adjoint_pair(int ndim, const dim_dev* dims, const double* u, const double* mu,
                                const double* kappa, double* rmu, double* g, double dt, cudaStream_t s,
                                bool kappa_points) {
    if (ndim != 3) {
        if (kappa_points) return cudaErrorNotSupported;
        cudaError_t e = launch_kappa_grad(ndim, dims, u, mu, g, dt, s);
        return e != cudaSuccess ? e : launch_rhs_elem(ndim, dims, mu, kappa, rmu, dt, s);
    }
    const int p = dims[0].p;
    for (int d = 0; d < ndim; ++d)
        if (dims[d].p != p || dims[d].q != p + 1) return cudaErrorNotSupported;
    switch (p) {
        case 1: return adj3_p<1>(dims, u, mu, kappa, rmu, g, dt, s, kappa_points);
        case 2: return adj3_p<2>(dims, u, mu, kappa, rmu, g, dt, s, kappa_points);
        case 3: return adj3_p<3>(dims, u, mu, kappa, rmu, g, dt, s, kappa_points);
        case 4: return adj3_p<4>(dims, u, mu, kappa, rmu, g, dt, s, kappa_points);
        default: return cudaErrorNotSupported;
    }
}

cudaError_t launch_kappa_grad(int ndim, const dim_dev* dims, const double* u, const double* mu, double* g, double dt,
                              cudaStream_t s) {
    if (ndim != 2) return cudaErrorNotSupported;  // 3D: launch_adjoint_pair
    const int p = dims[0].p;
    for (int d = 0; d < ndim; ++d)
        if (dims[d].p != p || dims[d].q != p + 1) return cudaErrorNotSupported;
    switch (p) {
        case 1: return kgrad2_p<1>(dims, u, mu, g, dt, s);
        case 2: return kgrad2_p<2>(dims, u, mu, g, dt, s);
        case 3: return kgrad2_p<3>(dims, u, mu, g, dt, s);
        case 4: return kgrad2_p<4>(dims, u, mu, g, dt, s);
        default: return cudaErrorNotSupported;
    }
}

// kappa at every Gauss point of every element, one thread per point, stored
// by element colour in the element kernel's launch order (colour blocks,
// elements in their launch index within a block, then the point
// qx + Q (qy + Q qz)): a warp of the element kernel reads its elements'
// values as one contiguous run.
// The contractions are elem3_kernel's (x, then y, then z, each an FMA chain
// from zero over the element's coefficients in the same order), so the values
// equal the ones that kernel interpolates alongside u, bit for bit.
template <int P>
__global__ void __launch_bounds__(256) kappa_points_kernel(const double* __restrict__ kappa, double* __restrict__ kq,
                                                           dim_dev X, dim_dev Y, dim_dev Z) {
    constexpr int N = P + 1, Q = P + 1, Q3 = Q * Q * Q;
    const long long ne = static_cast<long long>(X.elements) * Y.elements * Z.elements;
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= ne * Q3) return;
    const long long el = i / Q3;
    const int t = static_cast<int>(i - el * Q3);
    const int qx = t % Q, qy = (t / Q) % Q, qz = t / (Q * Q);
    const int e0 = static_cast<int>(el % X.elements), e1 = static_cast<int>((el / X.elements) % Y.elements),
              e2 = static_cast<int>(el / (static_cast<long long>(X.elements) * Y.elements));
    const long long nx = X.n, nxy = static_cast<long long>(X.n) * Y.n;
    const int f0 = X.first[e0], f1 = Y.first[e1], f2 = Z.first[e2];
    if (!(ADSG_IN(f0 + N - 1, X.n) && ADSG_IN(f1 + N - 1, Y.n) && ADSG_IN(f2 + N - 1, Z.n) && f0 >= 0 && f1 >= 0 &&
          f2 >= 0))
        return;
    const double* bx = X.btab + ((static_cast<long long>(e0) * Q + qx) * 2) * N;  // value row of qx
    const double* by = Y.btab + ((static_cast<long long>(e1) * Q + qy) * 2) * N;
    const double* bz = Z.btab + ((static_cast<long long>(e2) * Q + qz) * 2) * N;
    double kv = 0.0;
#pragma unroll
    for (int cz = 0; cz < N; ++cz) {
        double k1 = 0.0;
#pragma unroll
        for (int cy = 0; cy < N; ++cy) {
            const double* row = kappa + (f0 + nx * (f1 + cy) + nxy * (f2 + cz));
            double k0 = 0.0;
#pragma unroll
            for (int cx = 0; cx < N; ++cx) k0 = fma(bx[cx], row[cx], k0);
            k1 = fma(by[cy], k0, k1);
        }
        kv = fma(bz[cz], k1, kv);
    }
    const int cx = e0 % N, cy = e1 % N, cz = e2 % N;
    const long long my = colour_count(Y.elements, cy, N), mz = colour_count(Z.elements, cz, N);
    const long long id = (static_cast<long long>(e0 / N) * my + e1 / N) * mz + e2 / N;
    kq[(colour_base(X.elements, Y.elements, Z.elements, N, cx, cy, cz) + id) * Q3 + t] = kv;
}

cudaError_t launch_kappa_points(const dim_dev* dims, const double* kappa, double* kq, cudaStream_t s) {
    const int p = dims[0].p;
    for (int d = 0; d < 3; ++d)
        if (dims[d].p != p || dims[d].q != p + 1) return cudaErrorNotSupported;
    const long long total = kappa_points_count(3, dims);
    if (total <= 0) return cudaSuccess;
    const unsigned blocks = static_cast<unsigned>((total + 255) / 256);
    switch (p) {
        case 1: kappa_points_kernel<1><<<blocks, 256, 0, s>>>(kappa, kq, dims[0], dims[1], dims[2]); break;
        case 2: kappa_points_kernel<2><<<blocks, 256, 0, s>>>(kappa, kq, dims[0], dims[1], dims[2]); break;
        case 3: kappa_points_kernel<3><<<blocks, 256, 0, s>>>(kappa, kq, dims[0], dims[1], dims[2]); break;
        case 4: kappa_points_kernel<4><<<blocks, 256, 0, s>>>(kappa, kq, dims[0], dims[1], dims[2]); break;
        default: return cudaErrorNotSupported;
    }
    return cudaGetLastError();
}

long long kappa_points_count(int ndim, const dim_dev* dims) {
    if (ndim != 3) return 0;
    const long long q = dims[0].q;
    return static_cast<long long>(dims[0].elements) * dims[1].elements * dims[2].elements * q * q * q;
}

cudaError_t launch_rhs_elem_points(const dim_dev* dims, const double* u_prev, const double* kq, double* rhs,
                                   double dt, cudaStream_t s) {
    const int p = dims[0].p;
    for (int d = 0; d < 3; ++d)
        if (dims[d].p != p || dims[d].q != p + 1) return cudaErrorNotSupported;
    const point_form none;
    switch (p) {
        case 1: return elem_p<1, false>(3, dims, u_prev, kq, rhs, dt, none, s, true);
        case 2: return elem_p<2, false>(3, dims, u_prev, kq, rhs, dt, none, s, true);
        case 3: return elem_p<3, false>(3, dims, u_prev, kq, rhs, dt, none, s, true);
        case 4: return elem_p<4, false>(3, dims, u_prev, kq, rhs, dt, none, s, true);
        default: return cudaErrorNotSupported;
    }
}

cudaError_t launch_rhs_elem(int ndim, const dim_dev* dims, const double* u_prev, const double* kappa, double* rhs,
                            double dt, cudaStream_t s) {
    if (ndim < 2) return cudaErrorNotSupported;
    const int p = dims[0].p;
    for (int d = 0; d < ndim; ++d)
        if (dims[d].p != p || dims[d].q != p + 1) return cudaErrorNotSupported;
    const point_form none;
    switch (p) {
        case 1: return elem_p<1, false>(ndim, dims, u_prev, kappa, rhs, dt, none, s);
        case 2: return elem_p<2, false>(ndim, dims, u_prev, kappa, rhs, dt, none, s);
        case 3: return elem_p<3, false>(ndim, dims, u_prev, kappa, rhs, dt, none, s);
        case 4: return elem_p<4, false>(ndim, dims, u_prev, kappa, rhs, dt, none, s);
        default: return cudaErrorNotSupported;
    }
}

cudaError_t launch_form_elem(int ndim, const dim_dev* dims, const double* u, const point_form& F, double* rhs,
                             cudaStream_t s) {
    if (ndim < 2) return cudaErrorNotSupported;
    const int p = dims[0].p;
    for (int d = 0; d < ndim; ++d)
        if (dims[d].p != p || dims[d].q != p + 1) return cudaErrorNotSupported;
    switch (p) {
        case 1: return elem_p<1, true>(ndim, dims, u, nullptr, rhs, 0.0, F, s);
        case 2: return elem_p<2, true>(ndim, dims, u, nullptr, rhs, 0.0, F, s);
        case 3: return elem_p<3, true>(ndim, dims, u, nullptr, rhs, 0.0, F, s);
        case 4: return elem_p<4, true>(ndim, dims, u, nullptr, rhs, 0.0, F, s);
        default: return cudaErrorNotSupported;
    }
}

}  // namespace adsg
