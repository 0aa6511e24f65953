// sm_103a kernels of the explicit heat step.
//
// GB300 executes FP64 at ~1.2 TFLOP/s (measured: 2 DFMA/clk/SM, 64-cycle
// dependent latency), about 1/60 of its FP32 rate and far below what HBM can
// feed.  Every kernel here is therefore organised around the FP64 pipe: the
// work is arranged so that no FP64 operation is redundant, and loads, index
// arithmetic and shared-memory traffic (which run on other pipes) are spent
// freely to keep it busy.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <mutex>
#include <vector>

#include "adsg_check.cuh"
#include "adsg_kernels.cuh"

namespace adsg {

ADSG_BOUNDS_TU(kernels)

// Bounds-checked build: whether the rows 0 .. n-1 of a line, x[r * es],
// lie inside the buffer of `total` doubles at base (a line's accesses are
// all of that form, with the row index kept in [0, n) by the sweeps' loops).
#define ADSG_LINE_OK(base, x, n, es, total)                                                               \
    (!ADSG_BOUNDS_CHECK || (ADSG_IN((x) - (base), (total)) &&                                            \
                            ADSG_IN(((x) - (base)) + static_cast<long long>((n) - 1) * (es), (total))))

// ---------------------------------------------------------------------------
// Programmatic dependent launch.  The step's kernels are launched with
// programmatic stream serialisation: the next kernel on the stream may be
// scheduled once every block of the current one has started, and waits in
// griddepcontrol.wait (before its first global memory access) until the
// current kernel has completed and its writes are visible.  This hides the
// launch latency between the six kernels of a step behind the last wave of
// the previous one.  Without the attribute both instructions are no-ops.
// Whether the attribute is set is chosen per context (set_launch_pdl): it
// pays on small, launch-bound grids, while on large ones the early-placed
// blocks of a one-wave solve kernel can land unevenly across the SMs.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void pdl_wait_and_release() {
    asm volatile("griddepcontrol.wait;\n" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
}

// Kernels that run as one wave of long-lived warps (the line solves) only
// wait: their dependents launch when the last block exits, so the next
// kernel's blocks do not sit on the SMs beside the sweeps, while the launch
// still overlaps the grid's completion.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }

static thread_local int t_pdl_mode = 0;  // set per context around its launches

void set_launch_pdl(int on) { t_pdl_mode = on ? 1 : 0; }
int launch_pdl_mode() { return t_pdl_mode; }

static bool pdl_enabled() { return t_pdl_mode == 1; }

static thread_local int t_small2d_cluster = 1;  // the small 2D step on a cluster (1) or one block (0)
void set_small2d_cluster(int on) { t_small2d_cluster = on ? 1 : 0; }
int small2d_cluster_mode() { return t_small2d_cluster; }

template <typename... KArgs, typename... Args>
static cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                              Args... args) {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = pdl_enabled() ? 1 : 0;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaError_t e = cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
    return e != cudaSuccess ? e : cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Band pass: one output per thread, 2p+1 neighbours along one axis.
// out0 = A0 (.) in0 [+ A1 (.) in1]; out1 = B0 (.) in0.
// Threads of a warp take consecutive x, so every neighbour load is coalesced;
// along y/z the band row is the same for the whole warp (broadcast loads).
// ---------------------------------------------------------------------------
// SYM (used where a pass has two outputs, OUT1): rows sym_lo .. sym_hi-1 are
// symmetric (the host finds the range; uniform open knots make every row
// 2p-1 or more away from the ends a translate of one symmetric row, up to
// rounding), so the pair sums in(r-t) + in(r+t) are formed once and shared by
// both outputs, with the left coefficient of each pair: 3p+2 FP64 operations
// instead of 2(2p+1) for out0/out1 = A0/B0 (.) in0, and 5p+3 instead of
// 3(2p+1) with a second input.  Other rows take the full band.
// One output of a band pass (the body of band_pass_kernel, shared with the
// one-block small-grid step so that both perform the same operations in the
// same order).  GIN: the inputs are in global memory (read through the
// read-only path); otherwise in shared memory.
template <int GIN>
__device__ __forceinline__ double ldin(const double* p) {
    if (GIN == 2) return __ldcg(p);  // written earlier in the same launch (batched engine)
    if (GIN == 1) return __ldg(p);
    return *p;
}

// GIN: 0 inputs in shared memory, 1 in global memory (read-only path), 2 in
// global memory written earlier in the same launch (L2 loads).
template <int P, bool IN1, bool OUT1, bool SYM, int GIN>
__device__ __forceinline__ void band_out(long long g, const double* in0, const double* in1, double* out0,
                                         double* out1, const double* __restrict__ A0,
                                         const double* __restrict__ A1, const double* __restrict__ B0, int n_axis,
                                         long long stride, int sym_lo, int sym_hi, long long total) {
    constexpr int BW = 2 * P + 1;
    const int r = static_cast<int>((g / stride) % n_axis);
    // bounds-checked build: the output, and the rows r-P .. r+P the band
    // reaches (those inside the axis), inside the tensors of `total` doubles
    if (!(ADSG_IN(g, total) && ADSG_IN(g - static_cast<long long>(min(r, P)) * stride, total) &&
          ADSG_IN(g + static_cast<long long>(min(n_axis - 1 - r, P)) * stride, total)))
        return;
    const double* a0 = A0 + static_cast<long long>(r) * BW;
    const double* a1 = IN1 ? A1 + static_cast<long long>(r) * BW : nullptr;
    const double* b0 = OUT1 ? B0 + static_cast<long long>(r) * BW : nullptr;
    double acc0 = 0.0, acc1 = 0.0;
    if (SYM && r >= sym_lo && r < sym_hi) {
        const double c0 = ldin<GIN>(in0 + g);
        acc0 = __ldg(a0 + P) * c0;
        if (OUT1) acc1 = __ldg(b0 + P) * c0;
        if (IN1) acc0 = fma(__ldg(a1 + P), ldin<GIN>(in1 + g), acc0);
#pragma unroll
        for (int t = 1; t <= P; ++t) {
            const long long off = static_cast<long long>(t) * stride;
            const double s0 = ldin<GIN>(in0 + g - off) + ldin<GIN>(in0 + g + off);
            acc0 = fma(__ldg(a0 + P - t), s0, acc0);
            if (OUT1) acc1 = fma(__ldg(b0 + P - t), s0, acc1);
            if (IN1) acc0 = fma(__ldg(a1 + P - t), ldin<GIN>(in1 + g - off) + ldin<GIN>(in1 + g + off), acc0);
        }
        out0[g] = acc0;
        if (OUT1) out1[g] = acc1;
        return;
    }
#pragma unroll
    for (int t = 0; t < BW; ++t) {
        const int c = r - P + t;
        if (c >= 0 && c < n_axis) {
            const long long at = g + static_cast<long long>(t - P) * stride;
            const double v0 = ldin<GIN>(in0 + at);
            acc0 = fma(__ldg(a0 + t), v0, acc0);
            if (OUT1) acc1 = fma(__ldg(b0 + t), v0, acc1);
            if (IN1) acc0 = fma(__ldg(a1 + t), ldin<GIN>(in1 + at), acc0);
        }
    }
    out0[g] = acc0;
    if (OUT1) out1[g] = acc1;
}

template <int P, bool IN1, bool OUT1, bool SYM = false>
__global__ void __launch_bounds__(256) band_pass_kernel(const double* __restrict__ in0,
                                                         const double* __restrict__ in1,
                                                         double* __restrict__ out0,
                                                         double* __restrict__ out1,
                                                         const double* __restrict__ A0,
                                                         const double* __restrict__ A1,
                                                         const double* __restrict__ B0, int n_axis,
                                                         long long stride, long long total, int sym_lo, int sym_hi) {
    long long g = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (g >= total) return;
    pdl_wait_and_release();
    band_out<P, IN1, OUT1, SYM, true>(g, in0, in1, out0, out1, A0, A1, B0, n_axis, stride, sym_lo, sym_hi, total);
}

template <int P>
static cudaError_t band_pass_p(const double* in0, const double* in1, double* out0, double* out1,
                               const double* A0, const double* A1, const double* B0, int n_axis,
                               long long stride, long long total, cudaStream_t s, int lo, int hi) {
    const int threads = 256;
    const bool sym = hi > lo;
    const dim3 grid(static_cast<unsigned>((total + threads - 1) / threads));
    if (in1 && out1) {
        if (sym)
            return launch_pdl(band_pass_kernel<P, true, true, true>, grid, dim3(threads), 0, s, in0, in1, out0, out1,
                              A0, A1, B0, n_axis, stride, total, lo, hi);
        return launch_pdl(band_pass_kernel<P, true, true>, grid, dim3(threads), 0, s, in0, in1, out0, out1, A0, A1, B0,
                          n_axis, stride, total, lo, hi);
    }
    if (in1)
        return launch_pdl(band_pass_kernel<P, true, false>, grid, dim3(threads), 0, s, in0, in1, out0, out1, A0, A1, B0,
                          n_axis, stride, total, lo, hi);
    if (out1) {
        if (sym)
            return launch_pdl(band_pass_kernel<P, false, true, true>, grid, dim3(threads), 0, s, in0, in1, out0, out1,
                              A0, A1, B0, n_axis, stride, total, lo, hi);
        return launch_pdl(band_pass_kernel<P, false, true>, grid, dim3(threads), 0, s, in0, in1, out0, out1, A0, A1, B0,
                          n_axis, stride, total, lo, hi);
    }
    return launch_pdl(band_pass_kernel<P, false, false>, grid, dim3(threads), 0, s, in0, in1, out0, out1, A0, A1, B0,
                      n_axis, stride, total, lo, hi);
}

cudaError_t launch_band_pass(int p, const double* in0, const double* in1, double* out0, double* out1,
                             const double* A0, const double* A1, const double* B0, int n_axis,
                             long long stride, long long total, cudaStream_t s, int sym_lo, int sym_hi) {
    if (total <= 0) return cudaSuccess;
    // a single output gains nothing from pair sums; the range must keep the
    // pair's rows inside the axis
    const int lo = std::max(sym_lo, p), hi = std::min(sym_hi, n_axis - p);
    const bool sym = out1 != nullptr && hi > lo;
    const int L = sym ? lo : 0, H = sym ? hi : 0;
    switch (p) {
        case 1: return band_pass_p<1>(in0, in1, out0, out1, A0, A1, B0, n_axis, stride, total, s, L, H);
        case 2: return band_pass_p<2>(in0, in1, out0, out1, A0, A1, B0, n_axis, stride, total, s, L, H);
        case 3: return band_pass_p<3>(in0, in1, out0, out1, A0, A1, B0, n_axis, stride, total, s, L, H);
        case 4: return band_pass_p<4>(in0, in1, out0, out1, A0, A1, B0, n_axis, stride, total, s, L, H);
        case 5: return band_pass_p<5>(in0, in1, out0, out1, A0, A1, B0, n_axis, stride, total, s, L, H);
        case 6: return band_pass_p<6>(in0, in1, out0, out1, A0, A1, B0, n_axis, stride, total, s, L, H);
        case 7: return band_pass_p<7>(in0, in1, out0, out1, A0, A1, B0, n_axis, stride, total, s, L, H);
        case 8: return band_pass_p<8>(in0, in1, out0, out1, A0, A1, B0, n_axis, stride, total, s, L, H);
        default: return cudaErrorInvalidValue;
    }
}

// ---------------------------------------------------------------------------
// Outer-axis pass as column sweeps.  Thread (column, segment) walks the rows
// of one segment of one column of the outermost axis with a window of the
// 2P+1 neighbouring inputs, so every input value is read once (plus a 2P-row
// halo per segment) instead of 2P+1 times.  That matters when the input sits
// in pinned host memory, whose lines the GPU does not keep in L2: the pass
// then streams its input over the host link once while it computes.  The
// rows ahead are prefetched PRE deep to keep enough host reads in flight.
// Per output the operations and their order are band_pass_kernel's
// (out0 = A0 (.) in, out1 = B0 (.) in), so the results are bitwise equal.
// ---------------------------------------------------------------------------
template <int P, bool SYM>
__global__ void __launch_bounds__(128) outer_columns_kernel(const double* __restrict__ in, double* __restrict__ out0,
                                                            double* __restrict__ out1, const double* __restrict__ A0,
                                                            const double* __restrict__ B0, int n, long long so,
                                                            int seg, int sym_lo, int sym_hi, int row_begin,
                                                            int row_end) {
    constexpr int BW = 2 * P + 1, PRE = 8;
    const long long t = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    const long long nseg = (row_end - row_begin + seg - 1) / seg;
    if (t >= so * nseg) return;
    pdl_wait_and_release();
    const long long col = t % so;
    const int r0 = row_begin + static_cast<int>(t / so) * seg, r1 = min(row_end, r0 + seg);
    const double* src = in + col;
    if (!(ADSG_IN(col, so) && ADSG_IN(col + static_cast<long long>(n - 1) * so, static_cast<long long>(n) * so)))
        return;  // bounds-checked build: the column inside the n x so tensor
    auto ld = [&](int r) -> double { return (r >= 0 && r < n) ? src[r * so] : 0.0; };
    double w[BW];
#pragma unroll
    for (int q = 0; q < BW; ++q) w[q] = ld(r0 - P + q);
    double pre[PRE];
#pragma unroll
    for (int q = 0; q < PRE; ++q) pre[q] = ld(r0 + P + 1 + q);
    // one row: the host read PRE rows ahead is issued first, so that the
    // link keeps PRE reads per thread in flight while the row computes
    auto row = [&](int r, bool sym) {
        const double incoming = ld(r + P + 1 + PRE);
        const double* a0 = A0 + static_cast<long long>(r) * BW;
        const double* b0 = B0 + static_cast<long long>(r) * BW;
        double acc0 = 0.0, acc1 = 0.0;
        if (sym) {  // band_pass_kernel's SYM order
            acc0 = __ldg(a0 + P) * w[P];
            acc1 = __ldg(b0 + P) * w[P];
#pragma unroll
            for (int t = 1; t <= P; ++t) {
                const double s0 = w[P - t] + w[P + t];
                acc0 = fma(__ldg(a0 + P - t), s0, acc0);
                acc1 = fma(__ldg(b0 + P - t), s0, acc1);
            }
        } else {
#pragma unroll
            for (int q = 0; q < BW; ++q) {
                const int c = r - P + q;
                if (c >= 0 && c < n) {
                    acc0 = fma(__ldg(a0 + q), w[q], acc0);
                    acc1 = fma(__ldg(b0 + q), w[q], acc1);
                }
            }
        }
        out0[col + r * so] = acc0;
        out1[col + r * so] = acc1;
#pragma unroll
        for (int q = 0; q < BW - 1; ++q) w[q] = w[q + 1];
        w[BW - 1] = pre[0];
#pragma unroll
        for (int q = 0; q < PRE - 1; ++q) pre[q] = pre[q + 1];
        pre[PRE - 1] = incoming;
    };
    const int lo = SYM ? max(r0, min(r1, sym_lo)) : r1, hi = SYM ? max(lo, min(r1, sym_hi)) : r1;
    int r = r0;
    for (; r < lo; ++r) row(r, false);
    for (; r < hi; ++r) row(r, true);
    for (; r < r1; ++r) row(r, false);
}

bool outer_pass_columns_ok(int p) { return p >= 1 && p <= 4; }

cudaError_t launch_outer_pass_columns(int p, const double* in, double* out0, double* out1, const double* A0,
                                      const double* B0, int n_axis, long long stride, cudaStream_t s, int sym_lo,
                                      int sym_hi, int row_begin, int row_end) {
    if (!outer_pass_columns_ok(p)) return cudaErrorInvalidValue;
    if (row_end < 0) row_end = n_axis;
    if (row_begin < 0 || row_end > n_axis || row_begin >= row_end) return cudaErrorInvalidValue;
    const int rows = row_end - row_begin;
    // whole columns (each input read exactly once) unless there are too few
    // columns to give every sub-partition a few warps; segments re-read a
    // 2p-row halo each
    const long long want = 16384;
    int seg = rows;
    if (stride < want) seg = static_cast<int>(std::max<long long>(32, (rows * stride + want - 1) / want));
    const long long threads = stride * ((rows + seg - 1) / seg);
    if (threads <= 0) return cudaSuccess;
    const dim3 grid(static_cast<unsigned>((threads + 127) / 128)), block(128);
    const int lo = std::max(sym_lo, p), hi = std::min(sym_hi, n_axis - p);
    const bool sym = hi > lo;
#define ADSG_COLS(P_)                                                                                          \
    (sym ? launch_pdl(outer_columns_kernel<P_, true>, grid, block, 0, s, in, out0, out1, A0, B0, n_axis, stride, seg, \
                      lo, hi, row_begin, row_end)                                                               \
         : launch_pdl(outer_columns_kernel<P_, false>, grid, block, 0, s, in, out0, out1, A0, B0, n_axis, stride, seg, \
                      0, 0, row_begin, row_end))
    switch (p) {
        case 1: return ADSG_COLS(1);
        case 2: return ADSG_COLS(2);
        case 3: return ADSG_COLS(3);
        default: return ADSG_COLS(4);
    }
#undef ADSG_COLS
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
// Shared-memory rows reserved above and below each staged line (zeros): the
// register sweeps read up to UNR + KL + 1 rows past the end and UNR + KL + KU
// + 1 rows before the start (at most 8 + 2 + 1 and 4 + 8 + 1 for p <= 4).
constexpr int kPadLo = 16, kPadHi = 16;

// Raise a kernel's dynamic shared-memory limit on the current device once
// (the attribute is per device; a small table remembers what was set).
cudaError_t ensure_smem_attribute(const void* func, size_t bytes) {
    struct entry {
        const void* func;
        int device;
        size_t bytes;
    };
    static std::mutex lock;
    static std::vector<entry> done;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> g(lock);
    for (const entry& x : done)
        if (x.func == func && x.device == dev && x.bytes >= bytes) return cudaSuccess;
    e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(bytes));
    if (e == cudaSuccess) done.push_back({func, dev, bytes});
    return e;
}


line_layout make_line_layout(const int* n, int ndim, int d) {
    long long nx = n[0], ny = ndim > 1 ? n[1] : 1, nz = ndim > 2 ? n[2] : 1;
    line_layout L;
    L.total = nx * ny * nz;
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

// Asynchronous 8-byte global->shared copies (cp.async): every lane issues the
// copies of its whole tile before waiting once, so the staging of a tile
// keeps hundreds of loads in flight instead of one per loop iteration.
__device__ __forceinline__ void async_copy8(double* dst_smem, const double* src) {
    const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(dst_smem));
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
}

__device__ __forceinline__ void async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

__device__ __forceinline__ void stage_in(const double* __restrict__ data, double* s, const line_layout& L,
                                         int n, long long line0, int nvalid, int lane) {
    // bounds-checked build: the lines inside the tensor (the kernels check
    // their tiles against the launch's shared memory)
    if (L.contiguous) {
        if (!(ADSG_IN(line0 * n, L.total) && ADSG_IN((line0 + nvalid) * n - 1, L.total))) return;
        const double* src = data + line0 * n;
        for (int l = 0; l < 32; ++l) {
            if (l < nvalid) {
                for (int j = lane; j < n; j += 32) async_copy8(s + j * kPitch + l, src + static_cast<long long>(l) * n + j);
            } else {
                for (int j = lane; j < n; j += 32) s[j * kPitch + l] = 0.0;
            }
        }
    } else {
        const long long g = line0 + lane;
        if (lane < nvalid) {
            const double* src = data + (g % L.a) * L.sa + (g / L.a) * L.sb;
            if (!ADSG_LINE_OK(data, src, n, L.elem_stride, L.total)) return;
            for (int j = 0; j < n; ++j) async_copy8(s + j * kPitch + lane, src + j * L.elem_stride);
        } else {
            for (int j = 0; j < n; ++j) s[j * kPitch + lane] = 0.0;
        }
    }
    async_wait_all();
}

__device__ __forceinline__ void stage_out(double* __restrict__ data, const double* s, const line_layout& L,
                                          int n, long long line0, int nvalid, int lane) {
    if (L.contiguous) {
        double* dst = data + line0 * n;
        if (!(ADSG_IN(line0 * n, L.total) && ADSG_IN((line0 + nvalid) * n - 1, L.total))) return;
        for (int l = 0; l < nvalid; ++l)
            for (int j = lane; j < n; j += 32) dst[static_cast<long long>(l) * n + j] = s[j * kPitch + l];
    } else {
        if (lane < nvalid) {
            const long long g = line0 + lane;
            double* dst = data + (g % L.a) * L.sa + (g / L.a) * L.sb;
            if (!ADSG_LINE_OK(data, dst, n, L.elem_stride, L.total)) return;
#pragma unroll 8
            for (int j = 0; j < n; ++j) dst[j * L.elem_stride] = s[j * kPitch + lane];
        }
    }
}

// dgbtrs 'N' on one line x[j*es] (generic bands): the L-solve with row
// exchanges (dgbtrs's forward loop), then the U-solve (dtbsv 'Upper','N',
// 'Non-unit') with the diagonal applied as a reciprocal, column by column in
// LAPACK's order.  es is kPitch for a line staged in shared memory, or the
// line's element stride in global memory.
__device__ __forceinline__ void sweep_n_generic(double* x, const dim_dev& D, const long long es = kPitch) {
    const int n = D.n, kl = D.kl, w = D.w;
    for (int j = 0; j < n - 1; ++j) {
        const int l = __ldg(D.piv + j);
        if (l != j) {
            const double t = x[l * es];
            x[l * es] = x[j * es];
            x[j * es] = t;
        }
        const double y = -x[j * es];
        const int lm = min(kl, n - 1 - j);
        const double* lj = D.lmul + static_cast<long long>(j) * kl;
        for (int i = 1; i <= lm; ++i) x[(j + i) * es] = fma(y, __ldg(lj + i - 1), x[(j + i) * es]);
    }
    for (int j = n - 1; j >= 0; --j) {
        const double v = x[j * es] * __ldg(D.rdiag + j);
        x[j * es] = v;
        const int ext = __ldg(D.uext + j);
        const double* uj = D.ucol + static_cast<long long>(j) * w;
        for (int dd = 1; dd <= ext; ++dd) x[(j - dd) * es] = fma(-v, __ldg(uj + dd - 1), x[(j - dd) * es]);
    }
}

// The same substitution with both sweeps held in registers.  One warp-wide
// FP64 instruction occupies a GB300 SM sub-partition's FP64 unit for ~64
// cycles, and a line solve has one warp per sub-partition at typical sizes,
// so every latency on the recurrence stalls the pipe: the forward sweep keeps
// rows j..j+KL, the backward sweep rows j..j-WW, in registers, the next row
// is loaded from shared memory (zero padding above and below the line makes
// every step identical) and the next column's coefficients are fetched a
// step ahead.  The order of the updates is LAPACK's: row i receives its
// forward updates from columns i-KL..i-1 and its backward updates from
// columns i+WW..i+1, in that order.  Columns whose U extent exceeds KU (fill
// from row exchanges) take a warp-uniform branch for the extra terms.
template <int KL, int KU, int UNR>
__device__ __forceinline__ void sweep_n_reg(double* x, const dim_dev& D) {
    constexpr int WW = KL + KU;
    // every row the sweep touches lies in [-kPadLo, n + kPadHi): the tile
    static_assert(UNR + KL + 1 <= kPadHi && UNR + WW + 1 <= kPadLo, "staged tile padding too small");
    const int n = D.n;
    const int w = D.w;  // U table stride (>= KU); the L table stride equals KL
    // ---- forward: window f[t] = x[j+t] ----
    double f[KL + 1];
#pragma unroll
    for (int t = 0; t <= KL; ++t) f[t] = x[t * kPitch];
    int j = 0;
    // head: columns with row exchanges
    for (; j < D.fwd_fast; ++j) {
        const int pc = __ldg(D.piv + j);
        const double incoming = x[(j + KL + 1) * kPitch];
        if (pc != j) {
            const int dsw = pc - j;
#pragma unroll
            for (int t = 1; t <= KL; ++t)
                if (t == dsw) {
                    const double tmp = f[0];
                    f[0] = f[t];
                    f[t] = tmp;
                }
        }
        x[j * kPitch] = f[0];
        const double ny = -f[0];
#pragma unroll
        for (int t = 1; t <= KL; ++t) f[t] = fma(ny, __ldg(D.lmul + static_cast<long long>(j) * KL + t - 1), f[t]);
#pragma unroll
        for (int t = 0; t < KL; ++t) f[t] = f[t + 1];
        f[KL] = incoming;
    }
    // body: no exchanges; UNR columns per iteration, coefficients a block ahead
    {
        double lnx[UNR * KL];
        const double* lp = D.lmul + static_cast<long long>(j) * KL;
#pragma unroll
        for (int k = 0; k < UNR * KL; ++k) lnx[k] = __ldg(lp + k);  // table padded by UNR columns
        for (; j + UNR <= n; j += UNR) {
            double lc[UNR * KL];
#pragma unroll
            for (int k = 0; k < UNR * KL; ++k) lc[k] = lnx[k];
            lp += UNR * KL;
#pragma unroll
            for (int k = 0; k < UNR * KL; ++k) lnx[k] = __ldg(lp + k);
            double inc[UNR];
#pragma unroll
            for (int u = 0; u < UNR; ++u) inc[u] = x[(j + u + KL + 1) * kPitch];
#pragma unroll
            for (int u = 0; u < UNR; ++u) {
                x[(j + u) * kPitch] = f[0];
                const double ny = -f[0];
#pragma unroll
                for (int t = 1; t <= KL; ++t) f[t] = fma(ny, lc[u * KL + t - 1], f[t]);
#pragma unroll
                for (int t = 0; t < KL; ++t) f[t] = f[t + 1];
                f[KL] = inc[u];
            }
        }
    }
    for (; j < n; ++j) {
        const double incoming = x[(j + KL + 1) * kPitch];
        x[j * kPitch] = f[0];
        const double ny = -f[0];
#pragma unroll
        for (int t = 1; t <= KL; ++t) f[t] = fma(ny, __ldg(D.lmul + static_cast<long long>(j) * KL + t - 1), f[t]);
#pragma unroll
        for (int t = 0; t < KL; ++t) f[t] = f[t + 1];
        f[KL] = incoming;
    }
    // ---- backward: window b[d] = x[j-d] (pending) ----
    double b[WW + 1];
#pragma unroll
    for (int d = 0; d <= WW; ++d) b[d] = x[(n - 1 - d) * kPitch];
    j = n - 1;
    // body: columns whose U extent is <= KU, UNR per iteration
    {
        double rnx[UNR], unx[UNR * KU];
        auto load_block = [&](int jj, double* r, double* uu) {
#pragma unroll
            for (int u = 0; u < UNR; ++u) {
                const int c = max(jj - u, 0);
                r[u] = __ldg(D.rdiag + c);
#pragma unroll
                for (int d = 0; d < KU; ++d) uu[u * KU + d] = __ldg(D.ucol + static_cast<long long>(c) * w + d);
            }
        };
        load_block(j, rnx, unx);
        for (; j - UNR + 1 >= D.bwd_fast; j -= UNR) {
            double rc[UNR], uc[UNR * KU];
#pragma unroll
            for (int u = 0; u < UNR; ++u) rc[u] = rnx[u];
#pragma unroll
            for (int k = 0; k < UNR * KU; ++k) uc[k] = unx[k];
            load_block(j - UNR, rnx, unx);
            double inc[UNR];
#pragma unroll
            for (int u = 0; u < UNR; ++u) inc[u] = x[(j - u - WW - 1) * kPitch];
#pragma unroll
            for (int u = 0; u < UNR; ++u) {
                const double v = b[0] * rc[u];
                x[(j - u) * kPitch] = v;
                const double nv = -v;
#pragma unroll
                for (int d = 1; d <= KU; ++d) b[d] = fma(nv, uc[u * KU + d - 1], b[d]);
#pragma unroll
                for (int d = 0; d < WW; ++d) b[d] = b[d + 1];
                b[WW] = inc[u];
            }
        }
    }
    // tail: remaining columns, including the ones with row-exchange fill
    for (; j >= 0; --j) {
        const double incoming = x[(j - WW - 1) * kPitch];
        const double v = b[0] * __ldg(D.rdiag + j);
        x[j * kPitch] = v;
        const double nv = -v;
        const int ec = __ldg(D.uext + j);
        const double* uj = D.ucol + static_cast<long long>(j) * w;
#pragma unroll
        for (int d = 1; d <= KU; ++d) b[d] = fma(nv, __ldg(uj + d - 1), b[d]);
        if (ec > KU) {
#pragma unroll
            for (int d = KU + 1; d <= WW; ++d)
                if (d <= ec) b[d] = fma(nv, __ldg(uj + d - 1), b[d]);
        }
#pragma unroll
        for (int d = 0; d < WW; ++d) b[d] = b[d + 1];
        b[WW] = incoming;
    }
}

// dgbtrs 'T': U^T-solve (dtbsv 'Upper','T'), then L^T with the row exchanges
// undone in reverse order.
__device__ __forceinline__ void sweep_t(double* x, const dim_dev& D, const long long es = kPitch) {
    const int n = D.n, kl = D.kl, w = D.w;
    for (int j = 0; j < n; ++j) {
        double t = x[j * es];
        const int ext = __ldg(D.uext + j);
        const double* uj = D.ucol + static_cast<long long>(j) * w;
        for (int dd = ext; dd >= 1; --dd) t = fma(-__ldg(uj + dd - 1), x[(j - dd) * es], t);
        x[j * es] = t * __ldg(D.rdiag + j);
    }
    for (int j = n - 2; j >= 0; --j) {
        const int lm = min(kl, n - 1 - j);
        const double* lj = D.lmul + static_cast<long long>(j) * kl;
        double t = 0.0;
        for (int i = 1; i <= lm; ++i) t = fma(x[(j + i) * es], __ldg(lj + i - 1), t);
        x[j * es] -= t;
        const int l = __ldg(D.piv + j);
        if (l != j) {
            const double s = x[l * es];
            x[l * es] = x[j * es];
            x[j * es] = s;
        }
    }
}


// KL/KU > 0: register sweeps for bands with kl <= KL, regular U extent <= KU;
// KL == 0: generic shared-memory sweeps.
template <int KL, int KU>
__global__ void __launch_bounds__(32) line_solve_kernel(double* __restrict__ data, dim_dev D, line_layout L,
                                                        int trans) {
    extern __shared__ double smem[];
    const int lane = threadIdx.x & 31;
    const long long line0 = static_cast<long long>(blockIdx.x) * 32;
    if (line0 >= L.nlines) return;
    pdl_wait();
    const int nvalid = static_cast<int>(min(32LL, L.nlines - line0));
    double* s = smem + kPadLo * kPitch;
    if (!ADSG_SMEM_RANGE(smem, static_cast<long long>(D.n + kPadLo + kPadHi) * kPitch)) return;
    for (int r = 0; r < kPadLo; ++r) smem[r * kPitch + lane] = 0.0;
    for (int r = 0; r < kPadHi; ++r) s[(D.n + r) * kPitch + lane] = 0.0;
    stage_in(data, s, L, D.n, line0, nvalid, lane);
    __syncwarp();
    if (trans)
        sweep_t(s + lane, D);
    else if (KL > 0)
        sweep_n_reg<(KL > 0 ? KL : 1), (KU > 0 ? KU : 1), (KL > 2 ? 4 : 8)>(s + lane, D);
    else
        sweep_n_generic(s + lane, D);
    __syncwarp();
    stage_out(data, s, L, D.n, line0, nvalid, lane);
}

size_t line_solve_smem_per_warp(int n) { return static_cast<size_t>(n + kPadLo + kPadHi) * kPitch * sizeof(double); }

// Lines too long for a shared-memory tile (more than ~850 rows): each lane
// sweeps its own line in place in global memory with the generic sweeps, 'N'
// or 'T', any band.  Same operations in the same order as the staged generic
// kernel, so the results are bitwise those of line_solve_kernel<0, 0>.
__global__ void __launch_bounds__(128) line_solve_long_kernel(double* __restrict__ data, dim_dev D, line_layout L,
                                                              int trans) {
    const long long g = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (g >= L.nlines) return;
    pdl_wait();
    double* x = data + (L.contiguous ? g * D.n : (g % L.a) * L.sa + (g / L.a) * L.sb);
    if (!ADSG_LINE_OK(data, x, D.n, L.elem_stride, L.total)) return;
    if (trans)
        sweep_t(x, D, L.elem_stride);
    else
        sweep_n_generic(x, D, L.elem_stride);
}

// ---------------------------------------------------------------------------
// Line solve without shared memory: each lane sweeps its own line directly in
// global memory (forward results written in place and read back by the same
// lane in the backward sweep), with the same register windows and column
// order as sweep_n_reg and the incoming rows prefetched UNR rows ahead.  No
// shared memory means no occupancy limit from long lines, so short lines and
// long lines alike fill every sub-partition.
// ---------------------------------------------------------------------------
// CG: read the line with L1-bypassing loads (for data written by other blocks
// earlier in the same launch).
template <int KL, int KU, int UNR, bool CG = false>
__device__ __forceinline__ void sweep_global(double* __restrict__ x, const long long es, const dim_dev& D) {
    constexpr int WW = KL + KU;
    const int n = D.n;
    const int w = D.w;
    auto ld = [&](int r) -> double {
        if (r < 0 || r >= n) return 0.0;
        return CG ? __ldcg(x + r * es) : x[r * es];
    };

    // ---- forward ----
    double f[KL + 1];
#pragma unroll
    for (int t = 0; t <= KL; ++t) f[t] = ld(t);
    int j = 0;
    for (; j < D.fwd_fast; ++j) {
        const int pc = __ldg(D.piv + j);
        const double incoming = ld(j + KL + 1);
        if (pc != j) {
            const int dsw = pc - j;
#pragma unroll
            for (int t = 1; t <= KL; ++t)
                if (t == dsw) {
                    const double tmp = f[0];
                    f[0] = f[t];
                    f[t] = tmp;
                }
        }
        x[j * es] = f[0];
        const double ny = -f[0];
#pragma unroll
        for (int t = 1; t <= KL; ++t) f[t] = fma(ny, __ldg(D.lmul + static_cast<long long>(j) * KL + t - 1), f[t]);
#pragma unroll
        for (int t = 0; t < KL; ++t) f[t] = f[t + 1];
        f[KL] = incoming;
    }
    {
        double pre[UNR];
#pragma unroll
        for (int u = 0; u < UNR; ++u) pre[u] = ld(j + KL + 1 + u);
        const double* lp = D.lmul + static_cast<long long>(j) * KL;
        double lnx[UNR * KL];
#pragma unroll
        for (int k = 0; k < UNR * KL; ++k) lnx[k] = __ldg(lp + k);
        for (; j + UNR <= n; j += UNR) {
            double inc[UNR], lc[UNR * KL];
#pragma unroll
            for (int u = 0; u < UNR; ++u) inc[u] = pre[u];
#pragma unroll
            for (int k = 0; k < UNR * KL; ++k) lc[k] = lnx[k];
#pragma unroll
            for (int u = 0; u < UNR; ++u) pre[u] = ld(j + UNR + KL + 1 + u);
            lp += UNR * KL;
#pragma unroll
            for (int k = 0; k < UNR * KL; ++k) lnx[k] = __ldg(lp + k);
#pragma unroll
            for (int u = 0; u < UNR; ++u) {
                x[(j + u) * es] = f[0];
                const double ny = -f[0];
#pragma unroll
                for (int t = 1; t <= KL; ++t) f[t] = fma(ny, lc[u * KL + t - 1], f[t]);
#pragma unroll
                for (int t = 0; t < KL; ++t) f[t] = f[t + 1];
                f[KL] = inc[u];
            }
        }
    }
    for (; j < n; ++j) {
        const double incoming = ld(j + KL + 1);
        x[j * es] = f[0];
        const double ny = -f[0];
#pragma unroll
        for (int t = 1; t <= KL; ++t) f[t] = fma(ny, __ldg(D.lmul + static_cast<long long>(j) * KL + t - 1), f[t]);
#pragma unroll
        for (int t = 0; t < KL; ++t) f[t] = f[t + 1];
        f[KL] = incoming;
    }
    // ---- backward ----
    double b[WW + 1];
#pragma unroll
    for (int d = 0; d <= WW; ++d) b[d] = ld(n - 1 - d);
    j = n - 1;
    {
        double pre[UNR];
#pragma unroll
        for (int u = 0; u < UNR; ++u) pre[u] = ld(j - WW - 1 - u);
        double rnx[UNR], unx[UNR * KU];
        auto load_block = [&](int jj, double* r, double* uu) {
#pragma unroll
            for (int u = 0; u < UNR; ++u) {
                const int c = max(jj - u, 0);
                r[u] = __ldg(D.rdiag + c);
#pragma unroll
                for (int d = 0; d < KU; ++d) uu[u * KU + d] = __ldg(D.ucol + static_cast<long long>(c) * w + d);
            }
        };
        load_block(j, rnx, unx);
        for (; j - UNR + 1 >= D.bwd_fast; j -= UNR) {
            double inc[UNR], rc[UNR], uc[UNR * KU];
#pragma unroll
            for (int u = 0; u < UNR; ++u) {
                inc[u] = pre[u];
                rc[u] = rnx[u];
            }
#pragma unroll
            for (int k = 0; k < UNR * KU; ++k) uc[k] = unx[k];
#pragma unroll
            for (int u = 0; u < UNR; ++u) pre[u] = ld(j - UNR - WW - 1 - u);
            load_block(j - UNR, rnx, unx);
#pragma unroll
            for (int u = 0; u < UNR; ++u) {
                const double v = b[0] * rc[u];
                x[(j - u) * es] = v;
                const double nv = -v;
#pragma unroll
                for (int d = 1; d <= KU; ++d) b[d] = fma(nv, uc[u * KU + d - 1], b[d]);
#pragma unroll
                for (int d = 0; d < WW; ++d) b[d] = b[d + 1];
                b[WW] = inc[u];
            }
        }
    }
    for (; j >= 0; --j) {
        const double incoming = ld(j - WW - 1);
        const double v = b[0] * __ldg(D.rdiag + j);
        x[j * es] = v;
        const double nv = -v;
        const int ec = __ldg(D.uext + j);
        const double* uj = D.ucol + static_cast<long long>(j) * w;
#pragma unroll
        for (int d = 1; d <= KU; ++d) b[d] = fma(nv, __ldg(uj + d - 1), b[d]);
        if (ec > KU) {
#pragma unroll
            for (int d = KU + 1; d <= WW; ++d)
                if (d <= ec) b[d] = fma(nv, __ldg(uj + d - 1), b[d]);
        }
#pragma unroll
        for (int d = 0; d < WW; ++d) b[d] = b[d + 1];
        b[WW] = incoming;
    }
}

template <int KL, int KU, int UNR>
__global__ void __launch_bounds__(128) line_solve_global_kernel(double* __restrict__ data, dim_dev D, line_layout L) {
    const int lane = threadIdx.x & 31;
    const long long g = static_cast<long long>(blockIdx.x) * (blockDim.x >> 5) * 32 + (threadIdx.x >> 5) * 32 + lane;
    if (g >= L.nlines) return;
    pdl_wait();
    double* x = data + (L.contiguous ? g * D.n : (g % L.a) * L.sa + (g / L.a) * L.sb);
    if (!ADSG_LINE_OK(data, x, D.n, L.elem_stride, L.total)) return;
    sweep_global<KL, KU, UNR>(x, L.elem_stride, D);
}

// 8-byte global -> shared copy that completes asynchronously (zero-filled
// when !valid, src then only has to be a mapped address); a lane's copies
// are all in flight until cp_async_wait_all().
__device__ __forceinline__ void cp_async8(double* dst, const double* src, bool valid) {
    const unsigned sa = static_cast<unsigned>(__cvta_generic_to_shared(dst));
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(sa), "l"(src), "r"(valid ? 8 : 0) : "memory");
}

__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// ---------------------------------------------------------------------------
// Twisted line solve.  Each line is split at n1 = n/2: lanes 0-15 of a warp
// sweep rows [0, n1) of 16 lines top-down, lanes 16-31 rows [n1, n) of the
// same lines bottom-up, each with its own unpivoted factors (the same band,
// eliminated from its end).  Where the chains meet, the k last forward
// results of both (exchanged by one shuffle) give the 2k unknowns
// x[n1-k .. n1+k) through a precomputed 2k x 2k inverse; each chain then
// back-substitutes outward from there.  Same FP64 work per row as the
// LAPACK-order sweep, twice the independent chains per line.
// ---------------------------------------------------------------------------
// UNIT: the right-hand side arrives row-scaled by 1 / U(r, r) and the tables
// have a unit upper diagonal (no multiply in the backward sweep).
// xo: where the backward sweep stores the solution (x itself, or another
// buffer with the same layout, e.g. mapped host memory); the forward results
// stay in x.
// TAIL: keep the last K+1 forward results in registers for the meeting point
// and the backward sweep's start instead of reading them back from the line
// (pays where the line is a shared-memory tile: 28.5 -> 26.8 us for the x
// sweep at 130^3, 312 -> 303 us at 260^3 p=4; costs the global-memory sweep
// its occupancy at p = 4: 245 -> 257 us).
// CG: read the line through L2 (it was written by other blocks earlier in
// the same launch: the batched engine).
template <int K, int UNR, bool UNIT, bool TAIL = false, bool CG = false>
__device__ __forceinline__ void twisted_chain(double* __restrict__ x, double* __restrict__ xo, const long long es,
                                              const int nc, const double* __restrict__ lmul,
                                              const double* __restrict__ ucol, const double* __restrict__ rdiag,
                                              const double* __restrict__ G, const unsigned mask) {
    auto ld = [&](int r) -> double {
        if (r < 0 || r >= nc) return 0.0;
        return CG ? __ldcg(x + r * es) : x[r * es];
    };
    // ---- forward (unit lower factor, no row exchanges) ----
    double f[K + 1];
#pragma unroll
    for (int t = 0; t <= K; ++t) f[t] = ld(t);
    // the last K+1 forward results stay in registers for the meeting point and
    // the backward sweep's start (no round trip through the line just written)
    double tail[TAIL ? K + 1 : 1];
#pragma unroll
    for (int t = 0; t < (TAIL ? K + 1 : 1); ++t) tail[t] = 0.0;
    auto keep = [&](double v) {
        if constexpr (TAIL) {
#pragma unroll
            for (int t = 0; t < K; ++t) tail[t] = tail[t + 1];
            tail[K] = v;
        }
    };
    int j = 0;
    {
        double pre[UNR];
#pragma unroll
        for (int u = 0; u < UNR; ++u) pre[u] = ld(K + 1 + u);
        const double* lp = lmul;
        double lnx[UNR * K];
#pragma unroll
        for (int q = 0; q < UNR * K; ++q) lnx[q] = __ldg(lp + q);
        for (; j + UNR <= nc; j += UNR) {
            double inc[UNR], lc[UNR * K];
#pragma unroll
            for (int u = 0; u < UNR; ++u) inc[u] = pre[u];
#pragma unroll
            for (int q = 0; q < UNR * K; ++q) lc[q] = lnx[q];
#pragma unroll
            for (int u = 0; u < UNR; ++u) pre[u] = ld(j + UNR + K + 1 + u);
            lp += UNR * K;  // tables carry 16 rows of zero padding past the chain
#pragma unroll
            for (int q = 0; q < UNR * K; ++q) lnx[q] = __ldg(lp + q);
#pragma unroll
            for (int u = 0; u < UNR; ++u) {
                x[(j + u) * es] = f[0];
                keep(f[0]);
                const double ny = -f[0];
#pragma unroll
                for (int t = 1; t <= K; ++t) f[t] = fma(ny, lc[u * K + t - 1], f[t]);
#pragma unroll
                for (int t = 0; t < K; ++t) f[t] = f[t + 1];
                f[K] = inc[u];
            }
        }
    }
    for (; j < nc; ++j) {
        const double incoming = ld(j + K + 1);
        x[j * es] = f[0];
        keep(f[0]);
        const double ny = -f[0];
#pragma unroll
        for (int t = 1; t <= K; ++t) f[t] = fma(ny, __ldg(lmul + static_cast<long long>(j) * K + t - 1), f[t]);
#pragma unroll
        for (int t = 0; t < K; ++t) f[t] = f[t + 1];
        f[K] = incoming;
    }
    // ---- meeting point ----
    double own[K], oth[K], z[K];
#pragma unroll
    for (int i = 0; i < K; ++i) own[i] = TAIL ? tail[TAIL ? 1 + i : 0] : ld(nc - K + i);  // rows nc-K .. nc-1
#pragma unroll
    for (int i = 0; i < K; ++i) oth[i] = __shfl_xor_sync(mask, own[i], 16);
#pragma unroll
    for (int a = 0; a < K; ++a) {
        double acc = 0.0;
#pragma unroll
        for (int i = 0; i < K; ++i) acc = fma(__ldg(G + a * 2 * K + i), own[i], acc);
#pragma unroll
        for (int i = 0; i < K; ++i) acc = fma(__ldg(G + a * 2 * K + K + i), oth[i], acc);
        z[a] = acc;
    }
    // ---- backward (upper factor, bandwidth K), columns nc-1 .. 0 ----
    double b[K + 1];
#pragma unroll
    for (int d = 0; d <= K; ++d) b[d] = TAIL ? tail[TAIL ? K - d : 0] : ld(nc - 1 - d);  // rows nc-1 .. nc-1-K
    int c = nc - 1;
#pragma unroll
    for (int a = K - 1; a >= 0; --a, --c) {  // the chain's K interface rows
        const double v = z[a];
        xo[c * es] = v;
        const double nv = -v;
#pragma unroll
        for (int d = 1; d <= K; ++d) b[d] = fma(nv, __ldg(ucol + static_cast<long long>(c) * K + d - 1), b[d]);
#pragma unroll
        for (int d = 0; d < K; ++d) b[d] = b[d + 1];
        b[K] = ld(c - K - 1);
    }
    {
        double pre[UNR];
#pragma unroll
        for (int u = 0; u < UNR; ++u) pre[u] = ld(c - K - 1 - u);
        double rnx[UNR], unx[UNR * K];
        auto load_block = [&](int jj, double* r, double* uu) {
#pragma unroll
            for (int u = 0; u < UNR; ++u) {
                const int cc = max(jj - u, 0);
                r[u] = UNIT ? 1.0 : __ldg(rdiag + cc);
#pragma unroll
                for (int d = 0; d < K; ++d) uu[u * K + d] = __ldg(ucol + static_cast<long long>(cc) * K + d);
            }
        };
        load_block(c, rnx, unx);
        for (; c - UNR + 1 >= 0; c -= UNR) {
            double inc[UNR], rc[UNR], uc[UNR * K];
#pragma unroll
            for (int u = 0; u < UNR; ++u) {
                inc[u] = pre[u];
                rc[u] = rnx[u];
            }
#pragma unroll
            for (int q = 0; q < UNR * K; ++q) uc[q] = unx[q];
#pragma unroll
            for (int u = 0; u < UNR; ++u) pre[u] = ld(c - UNR - K - 1 - u);
            load_block(c - UNR, rnx, unx);
#pragma unroll
            for (int u = 0; u < UNR; ++u) {
                const double v = UNIT ? b[0] : b[0] * rc[u];
                xo[(c - u) * es] = v;
                const double nv = -v;
#pragma unroll
                for (int d = 1; d <= K; ++d) b[d] = fma(nv, uc[u * K + d - 1], b[d]);
#pragma unroll
                for (int d = 0; d < K; ++d) b[d] = b[d + 1];
                b[K] = inc[u];
            }
        }
    }
    for (; c >= 0; --c) {
        const double incoming = ld(c - K - 1);
        const double v = UNIT ? b[0] : b[0] * __ldg(rdiag + c);
        xo[c * es] = v;
        const double nv = -v;
#pragma unroll
        for (int d = 1; d <= K; ++d) b[d] = fma(nv, __ldg(ucol + static_cast<long long>(c) * K + d - 1), b[d]);
#pragma unroll
        for (int d = 0; d < K; ++d) b[d] = b[d + 1];
        b[K] = incoming;
    }
}

template <int K, int UNR, bool UNIT>
__global__ void __launch_bounds__(128) line_solve_twisted_kernel(double* __restrict__ data, dim_dev D, line_layout L) {
    const int lane = threadIdx.x & 31, chain = lane >> 4;
    const long long g = (static_cast<long long>(blockIdx.x) * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 16 + (lane & 15);
    double* x = data + (L.contiguous ? g * D.n : (g % L.a) * L.sa + (g / L.a) * L.sb);
    const long long es = L.elem_stride;
    // bounds-checked build: the line inside the tensor (both chains of a line
    // decide alike, so a skipped line leaves no partner waiting in the shuffle)
    const bool active = g < L.nlines && ADSG_LINE_OK(data, x, D.n, es, L.total);
    const unsigned mask = __ballot_sync(0xffffffffu, active);  // lanes g and g^16 share a line
    if (!active) return;
    pdl_wait();
    const long long off = static_cast<long long>(chain) * D.tw_rows;
    if (chain) x += static_cast<long long>(D.n - 1) * es;
    twisted_chain<K, UNR, UNIT>(x, x, chain ? -es : es, chain ? D.tw_n2 : D.tw_n1, D.tw_lmul + off * K, D.tw_ucol + off * K,
                          D.tw_rdiag + off, D.tw_g + chain * 2 * K * K, mask);
}

// The same sweep for contiguous lines (the x direction), where a lane walking
// its own line would touch a different cache line per lane and row: each
// warp first copies its 16 lines (16 n consecutive doubles) into a shared
// tile with coalesced loads, sweeps there, and copies the tile back.  The
// tile pitch is odd so that the 16 lines of one row fall in distinct banks.
__host__ __device__ inline int twisted_pitch(int n) { return n | 1; }

template <int K, int UNR, bool UNIT>
// out: where the solved tile is written (data itself, or another buffer of
// the same layout such as mapped pinned host memory: the write-back is
// coalesced, 256 contiguous bytes per warp instruction)
__global__ void __launch_bounds__(128) line_solve_twisted_staged_kernel(const double* data, double* out, dim_dev D,
                                                                        line_layout L) {
    extern __shared__ double smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, chain = lane >> 4;
    const int n = D.n, pitch = twisted_pitch(n);
    const long long g0 = (static_cast<long long>(blockIdx.x) * (blockDim.x >> 5) + warp) * 16;
    if (g0 >= L.nlines) return;  // whole warp
    pdl_wait();
    const int nv = static_cast<int>(min(16LL, L.nlines - g0));
    double* tile = smem + static_cast<size_t>(warp) * 16 * pitch;
    const double* src = data + g0 * n;
    const int count = nv * n;
    // bounds-checked build: the warp's tile and its 16 lines (warp-uniform)
    if (!(ADSG_SMEM_RANGE(tile, 16LL * pitch) && ADSG_IN(g0 * n, L.total) && ADSG_IN(g0 * n + count - 1, L.total)))
        return;
#pragma unroll 4
    for (int e = lane; e < count; e += 32) {
        const int line = e / n;
        cp_async8(tile + line * pitch + (e - line * n), src + e, true);
    }
    cp_async_wait_all();
    __syncwarp();
    const int line = lane & 15;
    const bool active = line < nv;
    const unsigned mask = __ballot_sync(0xffffffffu, active);
    if (active) {
        double* x = tile + line * pitch + (chain ? n - 1 : 0);
        const long long off = static_cast<long long>(chain) * D.tw_rows;
        twisted_chain<K, UNR, UNIT, true>(x, x, chain ? -1 : 1, chain ? D.tw_n2 : D.tw_n1, D.tw_lmul + off * K,
                                          D.tw_ucol + off * K, D.tw_rdiag + off, D.tw_g + chain * 2 * K * K, mask);
    }
    __syncwarp();
    double* dst = out + g0 * n;
    for (int e = lane; e < count; e += 32) {
        const int ln = e / n;
        dst[e] = tile[ln * pitch + (e - ln * n)];
    }
}

size_t twisted_staged_smem_per_warp(int n) { return static_cast<size_t>(16) * twisted_pitch(n) * sizeof(double); }

// ---------------------------------------------------------------------------
// The staged two-ended sweep with its tile moved by the copy engine.  A warp's
// 16 contiguous x-lines are 16 n consecutive doubles in global memory; one
// lane issues a single bulk copy (cp.async.bulk) of them into the warp's
// shared tile, completing on an mbarrier the warp waits on, and after the
// sweeps one bulk copy writes the tile back.  The tile keeps the lines' own
// pitch n (a bulk copy moves contiguous bytes, 16 at a time); for even n that
// costs the sweep's 16-lane shared loads a two-way bank conflict, which an
// FP64-bound sweep does not feel.  Same operations in the same order as the
// other two-ended variants: bitwise equal results.
// The wait for the copy is bounded: past the limit the warp records it in
// g_bulk_wait_timeouts, waits (bounded again) for its copy and returns with
// its lines unsolved; the context reports ADSG_ERR_DEVICE.
// ---------------------------------------------------------------------------
__device__ int g_bulk_wait_timeouts;

__device__ __forceinline__ unsigned smem_u32(const void* p) {
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* bar, unsigned bytes) {
    asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n}" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
    unsigned done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return done != 0;
}

__device__ __forceinline__ void bulk_load(void* dst_smem, const void* src, unsigned bytes, unsigned long long* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst_smem)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void bulk_store(void* dst, const void* src_smem, unsigned bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(smem_u32(src_smem)),
                 "r"(bytes)
                 : "memory");
    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}

__device__ __forceinline__ void bulk_store_wait() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

constexpr long long kBulkWaitPolls = 1LL << 22;

template <int K, int UNR, bool UNIT>
__global__ void __launch_bounds__(128) line_solve_twisted_bulk_kernel(double* __restrict__ data, dim_dev D,
                                                                      line_layout L) {
    extern __shared__ __align__(16) double smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, chain = lane >> 4, wpb = blockDim.x >> 5;
    const int n = D.n;
    const long long g0 = (static_cast<long long>(blockIdx.x) * wpb + warp) * 16;
    if (g0 >= L.nlines) return;  // whole warp
    pdl_wait();
    const int nv = static_cast<int>(min(16LL, L.nlines - g0));
    double* tile = smem + static_cast<size_t>(warp) * 16 * n;  // 128 n bytes per warp: 16-byte aligned
    unsigned long long* bar = reinterpret_cast<unsigned long long*>(smem + static_cast<size_t>(wpb) * 16 * n) + warp;
    const long long count = static_cast<long long>(nv) * n;
    const unsigned bytes = static_cast<unsigned>((count * 8) & ~15LL);  // whole 16-byte units by the engine
    double* src = data + g0 * n;                                         // 128 g0 n bytes in: 16-byte aligned
    // bounds-checked build: the warp's tile and barrier, and its 16 lines (warp-uniform)
    if (!(ADSG_SMEM_RANGE(tile, 16LL * n) && ADSG_SMEM_RANGE(reinterpret_cast<double*>(bar), 1) &&
          ADSG_IN(g0 * n, L.total) && ADSG_IN(g0 * n + count - 1, L.total)))
        return;
    if (lane == 0) {
        mbar_init(bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_arrive_expect_tx(bar, bytes);
        bulk_load(tile, src, bytes, bar);
    }
    if (lane == 1 && bytes < count * 8) tile[count - 1] = src[count - 1];  // an odd last double
    bool arrived = false;
    for (long long it = 0; it < kBulkWaitPolls && !arrived; ++it) arrived = mbar_try_wait(bar, 0);
    if (!__all_sync(0xffffffffu, arrived)) {
        if (lane == 0) atomicAdd(&g_bulk_wait_timeouts, 1);
        for (long long it = 0; it < kBulkWaitPolls && !arrived; ++it) arrived = mbar_try_wait(bar, 0);
        return;  // lines left unsolved; reported to the host
    }
    __syncwarp();
    const int line = lane & 15;
    const bool active = line < nv;
    const unsigned mask = __ballot_sync(0xffffffffu, active);
    if (active) {
        double* x = tile + line * n + (chain ? n - 1 : 0);
        const long long off = static_cast<long long>(chain) * D.tw_rows;
        twisted_chain<K, UNR, UNIT, true>(x, x, chain ? -1 : 1, chain ? D.tw_n2 : D.tw_n1, D.tw_lmul + off * K,
                                          D.tw_ucol + off * K, D.tw_rdiag + off, D.tw_g + chain * 2 * K * K, mask);
    }
    __syncwarp();
    // the sweeps' shared-memory writes are made visible to the copy engine, then one bulk store
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncwarp();
    if (lane == 0) {
        bulk_store(src, tile, bytes);
        bulk_store_wait();  // the tile must be read before the warp's shared memory goes away
        asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
    }
    if (lane == 1 && bytes < count * 8) src[count - 1] = tile[count - 1];
}

size_t twisted_bulk_smem_per_warp(int n) { return static_cast<size_t>(16) * n * sizeof(double) + 8; }

int bulk_wait_timeouts(int reset) {
    int v = 0;
    if (cudaMemcpyFromSymbol(&v, g_bulk_wait_timeouts, sizeof(int)) != cudaSuccess) return -1;
    if (reset && v) {
        const int zero = 0;
        cudaMemcpyToSymbol(g_bulk_wait_timeouts, &zero, sizeof(int));
    }
    return v;
}

// Warps per block (1, 2 or 4) for kernels whose warps each hold a tile of
// per_warp bytes: the one that keeps the most warps resident per SM (228 KB
// of shared memory, 1 KB reserved per block), the smaller on a tie (finer
// blocks spread the warps over the SMs more evenly); 0 when one warp's tile
// does not fit.
int tile_warps_per_block(size_t per_warp) {
    int best = 0, best_res = 0;
    for (int w : {1, 2, 4}) {
        const size_t blk = per_warp * w;
        if (blk > 227 * 1024) continue;
        const int res = static_cast<int>((228 * 1024) / (blk + 1024)) * w;
        if (res > best_res) {
            best_res = res;
            best = w;
        }
    }
    return best;
}

// ---------------------------------------------------------------------------
// The two-ended sweep for contiguous lines, streamed in chunks.  A warp owns
// 16 consecutive lines (lanes 0-15 chain 0, lanes 16-31 chain 1, as above)
// and a shared buffer of 2 chains x 16 lines x kChunk rows.  Before each
// chunk of a sweep, the whole warp copies the rows the chunk will read
// (kChunk consecutive rows of one line and chain per warp-wide load: 256
// coalesced bytes); the chunk then runs in registers, leaving its results in
// the same slots, which the warp writes back the same way.  The forward
// results make one round trip through memory (L2 at these sizes) for the
// backward sweep.  Unlike the tile of variant 5 the buffer does not grow
// with the line, so long lines keep many warps per SM.  Same operations in
// the same order as twisted_chain.
// ---------------------------------------------------------------------------
constexpr int kChunk = 32, kChunkPitch = kChunk + 1;

struct chunk_lines {
    double* data;    // first line of the warp
    int n, n1, n2;   // line length and the chains' lengths
    int nv;          // valid lines of the warp (<= 16)
};

// chain-local row r of chain c lies at offset c ? n-1-r : r of its line
__device__ __forceinline__ long long chunk_offset(const chunk_lines& W, int line, int c, int r) {
    return static_cast<long long>(line) * W.n + (c ? W.n - 1 - r : r);
}

// buf[c][l][t] <- chain-local row (first[c] + dir * t) of line l, chain c
// (0 outside the chain); dir = +1 (forward) or -1 (backward).  (Plain loads:
// asynchronous copies measured slower here, unlike in the whole-line tile.)
template <bool CG = false>
__device__ __forceinline__ void chunk_stage(double* buf, const chunk_lines& W, const int first[2], int dir) {
    const int lane = threadIdx.x & 31;
    for (int idx = lane; idx < 2 * 16 * kChunk; idx += 32) {
        const int c = idx / (16 * kChunk), l = (idx / kChunk) % 16, t = idx % kChunk;
        const int r = first[c] + dir * t, nc = c ? W.n2 : W.n1;
        double v = 0.0;
        if (l < W.nv && r >= 0 && r < nc) {
            const double* src = W.data + chunk_offset(W, l, c, r);
            v = CG ? __ldcg(src) : *src;
        }
        buf[(c * 16 + l) * kChunkPitch + t] = v;
    }
}

__device__ __forceinline__ void chunk_flush(const double* buf, const chunk_lines& W, const int first[2], int dir) {
    const int lane = threadIdx.x & 31;
    for (int idx = lane; idx < 2 * 16 * kChunk; idx += 32) {
        const int c = idx / (16 * kChunk), l = (idx / kChunk) % 16, t = idx % kChunk;
        const int r = first[c] + dir * t, nc = c ? W.n2 : W.n1;
        if (l < W.nv && r >= 0 && r < nc) W.data[chunk_offset(W, l, c, r)] = buf[(c * 16 + l) * kChunkPitch + t];
    }
}

// The body of the chunked two-ended sweep for one warp: W.nv (<= 16) contiguous
// lines starting at W.data, lanes 0-15 chain 0 and 16-31 chain 1 of line
// lane & 15, buf this warp's 2 x 16 x kChunkPitch shared slots.  CG: the lines
// were written by other blocks earlier in the same launch.
template <int K, bool UNIT, bool CG = false>
__device__ __forceinline__ void chunked_twisted_warp(const chunk_lines& W, const dim_dev& D, double* buf) {
    const int lane = threadIdx.x & 31, chain = lane >> 4, line = lane & 15;
    double* mine = buf + (chain * 16 + line) * kChunkPitch;  // this lane's slots
    const bool active = line < W.nv;  // every lane stays to the end: the staging is warp-wide
    const int nc = chain ? W.n2 : W.n1, nmax = max(W.n1, W.n2);
    const long long off = static_cast<long long>(chain) * D.tw_rows;
    const double* lmul = D.tw_lmul + off * K;
    const double* ucol = D.tw_ucol + off * K;
    const double* rdiag = D.tw_rdiag + off;
    const double* G = D.tw_g + chain * 2 * K * K;
    auto ld = [&](int r) -> double {
        if (!(active && r >= 0 && r < nc)) return 0.0;
        const double* src = W.data + chunk_offset(W, line, chain, r);
        return CG ? __ldcg(src) : *src;
    };

    // ---- forward: rows j0 .. j0+kChunk-1 read rows j+K+1 from the chunk ----
    double f[K + 1];
#pragma unroll
    for (int t = 0; t <= K; ++t) f[t] = ld(t);
    double own[K], pre_tail = 0.0;  // y rows nc-K .. nc-1 and nc-K-1
#pragma unroll
    for (int i = 0; i < K; ++i) own[i] = 0.0;
    for (int j0 = 0; j0 < nmax; j0 += kChunk) {
        const int first[2] = {j0 + K + 1, j0 + K + 1};
        __syncwarp();
        chunk_stage<CG>(buf, W, first, +1);
        __syncwarp();
        if (active) {
            const int tend = min(kChunk, nc - j0);
            for (int t = 0; t < tend; ++t) {
                const int j = j0 + t;
                const double incoming = mine[t];
                const double yv = f[0];
                mine[t] = yv;
                if (j == nc - K - 1) pre_tail = yv;
#pragma unroll
                for (int i = 0; i < K; ++i)
                    if (j == nc - K + i) own[i] = yv;
                const double ny = -yv;
#pragma unroll
                for (int q = 1; q <= K; ++q) f[q] = fma(ny, __ldg(lmul + static_cast<long long>(j) * K + q - 1), f[q]);
#pragma unroll
                for (int q = 0; q < K; ++q) f[q] = f[q + 1];
                f[K] = incoming;
            }
        }
        __syncwarp();
        const int out_first[2] = {j0, j0};
        chunk_flush(buf, W, out_first, +1);
    }
    __syncwarp();  // the flushed forward results are visible to the whole warp
    // ---- meeting point ----
    double oth[K], z[K];
#pragma unroll
    for (int i = 0; i < K; ++i) oth[i] = __shfl_xor_sync(0xffffffffu, own[i], 16);
#pragma unroll
    for (int a = 0; a < K; ++a) {
        double acc = 0.0;
#pragma unroll
        for (int i = 0; i < K; ++i) acc = fma(__ldg(G + a * 2 * K + i), own[i], acc);
#pragma unroll
        for (int i = 0; i < K; ++i) acc = fma(__ldg(G + a * 2 * K + K + i), oth[i], acc);
        z[a] = acc;
    }
    // ---- backward: columns nc-1 .. 0 ----
    double b[K + 1];
#pragma unroll
    for (int d = 0; d < K; ++d) b[d] = own[K - 1 - d];
    b[K] = pre_tail;
    int c = nc - 1;
#pragma unroll
    for (int a = K - 1; a >= 0; --a, --c) {  // the chain's K interface rows
        const double v = z[a];
        if (active) W.data[chunk_offset(W, line, chain, c)] = v;
        const double nv = -v;
#pragma unroll
        for (int d = 1; d <= K; ++d) b[d] = fma(nv, __ldg(ucol + static_cast<long long>(c) * K + d - 1), b[d]);
#pragma unroll
        for (int d = 0; d < K; ++d) b[d] = b[d + 1];
        b[K] = ld(c - K - 1);
    }
    // chunks of columns c_hi, c_hi-1, ..., c_hi-kChunk+1, reading rows c-K-1
    const int chi0[2] = {W.n1 - K - 1, W.n2 - K - 1};
    const int steps = (max(chi0[0], chi0[1]) + kChunk) / kChunk;
    for (int s = 0; s < steps; ++s) {
        const int in_first[2] = {chi0[0] - s * kChunk - K - 1, chi0[1] - s * kChunk - K - 1};
        __syncwarp();
        chunk_stage<CG>(buf, W, in_first, -1);
        __syncwarp();
        if (active) {
            const int chi = chi0[chain] - s * kChunk;
            for (int t = 0; t < kChunk; ++t) {
                const int cc = chi - t;
                if (cc < 0) break;
                const double incoming = mine[t];
                const double v = UNIT ? b[0] : b[0] * __ldg(rdiag + cc);
                mine[t] = v;
                const double nv = -v;
#pragma unroll
                for (int d = 1; d <= K; ++d) b[d] = fma(nv, __ldg(ucol + static_cast<long long>(cc) * K + d - 1), b[d]);
#pragma unroll
                for (int d = 0; d < K; ++d) b[d] = b[d + 1];
                b[K] = incoming;
            }
        }
        __syncwarp();
        const int out_first[2] = {chi0[0] - s * kChunk, chi0[1] - s * kChunk};
        chunk_flush(buf, W, out_first, -1);
    }
}


template <int K, bool UNIT>
__global__ void __launch_bounds__(128) line_solve_twisted_chunked_kernel(double* __restrict__ data, dim_dev D,
                                                                         line_layout L) {
    extern __shared__ double smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, chain = lane >> 4, line = lane & 15;
    const long long g0 = (static_cast<long long>(blockIdx.x) * (blockDim.x >> 5) + warp) * 16;
    if (g0 >= L.nlines) return;  // whole warp
    pdl_wait();
    chunk_lines W;
    W.data = data + g0 * D.n;
    W.n = D.n;
    W.n1 = D.tw_n1;
    W.n2 = D.tw_n2;
    W.nv = static_cast<int>(min(16LL, L.nlines - g0));
    double* buf = smem + static_cast<size_t>(warp) * 2 * 16 * kChunkPitch;
    // bounds-checked build: the warp's buffer and its 16 lines (warp-uniform)
    if (!(ADSG_SMEM_RANGE(buf, 2LL * 16 * kChunkPitch) && ADSG_IN(g0 * D.n, L.total) &&
          ADSG_IN((g0 + W.nv) * D.n - 1, L.total)))
        return;
    chunked_twisted_warp<K, UNIT>(W, D, buf);
}

size_t twisted_chunked_smem_per_warp() { return sizeof(double) * 2 * 16 * kChunkPitch; }

// ---------------------------------------------------------------------------
// The x band pass of the right-hand side fused with the x line solve.  Both
// work on the same contiguous x-lines: each warp computes the band pass of its
// 16 lines straight into its shared tile (out = A0 (.) in0 [+ A1 (.) in1],
// the same operations in the same order as band_pass_kernel, so the tile
// holds bitwise the values that kernel would store), sweeps the tile with the
// two-ended solve and writes the solved lines once.
// ---------------------------------------------------------------------------
template <int K, int UNR, bool UNIT, bool IN1>
__global__ void __launch_bounds__(128) rhs_x_solve_kernel(const double* __restrict__ in0,
                                                          const double* __restrict__ in1,
                                                          double* __restrict__ out, const double* __restrict__ A0,
                                                          const double* __restrict__ A1, dim_dev D, line_layout L) {
    extern __shared__ double smem[];
    constexpr int BW = 2 * K + 1;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, chain = lane >> 4;
    const int n = D.n, pitch = twisted_pitch(n);
    const long long g0 = (static_cast<long long>(blockIdx.x) * (blockDim.x >> 5) + warp) * 16;
    if (g0 >= L.nlines) return;  // whole warp
    pdl_wait();
    const int nv = static_cast<int>(min(16LL, L.nlines - g0));
    double* tile = smem + static_cast<size_t>(warp) * 16 * pitch;
    const long long base = g0 * n;
    const int count = nv * n;
    // bounds-checked build: the warp's tile and its 16 lines (warp-uniform)
    if (!(ADSG_SMEM_RANGE(tile, 16LL * pitch) && ADSG_IN(base, L.total) && ADSG_IN(base + count - 1, L.total))) return;
    // unrolled so that several outputs' loads are in flight at once: few warps
    // per SM hold these tiles
#pragma unroll 4
    for (int e = lane; e < count; e += 32) {
        const int line = e / n, r = e - line * n;
        const double* a0 = A0 + static_cast<long long>(r) * BW;
        const double* a1 = IN1 ? A1 + static_cast<long long>(r) * BW : nullptr;
        const long long g = base + e;
        double acc = 0.0;
#pragma unroll
        for (int t = 0; t < BW; ++t) {
            const int c = r - K + t;
            if (c >= 0 && c < n) {
                const long long at = g + (t - K);
                acc = fma(__ldg(a0 + t), __ldg(in0 + at), acc);
                if (IN1) acc = fma(__ldg(a1 + t), __ldg(in1 + at), acc);
            }
        }
        tile[line * pitch + r] = acc;
    }
    __syncwarp();
    const int line = lane & 15;
    const bool active = line < nv;
    const unsigned mask = __ballot_sync(0xffffffffu, active);
    if (active) {
        double* x = tile + line * pitch + (chain ? n - 1 : 0);
        const long long off = static_cast<long long>(chain) * D.tw_rows;
        twisted_chain<K, UNR, UNIT, true>(x, x, chain ? -1 : 1, chain ? D.tw_n2 : D.tw_n1, D.tw_lmul + off * K,
                                          D.tw_ucol + off * K, D.tw_rdiag + off, D.tw_g + chain * 2 * K * K, mask);
    }
    __syncwarp();
    for (int e = lane; e < count; e += 32) {
        const int ln = e / n;
        out[base + e] = tile[ln * pitch + (e - ln * n)];
    }
}

template <int K, bool UNIT, bool IN1>
static cudaError_t rhs_x_solve_t(const double* in0, const double* in1, double* out, const double* A0,
                                 const double* A1, const dim_dev& d, const line_layout& L, cudaStream_t s) {
    constexpr int UNR = K > 2 ? 4 : 8;
    const size_t per_warp = twisted_staged_smem_per_warp(d.n);
    const int wpb = tile_warps_per_block(per_warp);
    if (wpb == 0) return cudaErrorInvalidConfiguration;
    const size_t smem = per_warp * wpb;
    auto kern = rhs_x_solve_kernel<K, UNR, UNIT, IN1>;
    if (smem > 48 * 1024) {
        cudaError_t e = ensure_smem_attribute(reinterpret_cast<const void*>(kern), smem);
        if (e != cudaSuccess) return e;
    }
    const long long per = 16LL * wpb;
    return launch_pdl(kern, dim3(static_cast<unsigned>((L.nlines + per - 1) / per)), dim3(32 * wpb), smem, s, in0, in1,
                      out, A0, A1, d, L);
}

// ---------------------------------------------------------------------------
// One-block step for small 2D grids: adsg_heat_step's y pass, x pass, y sweep
// and x sweep in one launch, separated by block barriers, on a grid whose
// four working tensors fit in shared memory.  Launch latency, not work,
// bounds such grids (four dependent launches of a few microseconds each).
// The passes are band_out and the sweeps twisted_chain, so the operations and
// their order are those of the separate kernels.
// ---------------------------------------------------------------------------
template <int K, int UNR>
__device__ __forceinline__ void small_sweeps(double* R, const dim_dev& D, int nlines, long long line_stride,
                                             long long es) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5, chain = lane >> 4;
    for (int grp = warp; grp * 16 < nlines; grp += nwarps) {
        const int line = grp * 16 + (lane & 15);
        const bool active = line < nlines;
        const unsigned mask = __ballot_sync(0xffffffffu, active);
        if (active) {
            double* x = R + line * line_stride + (chain ? static_cast<long long>(D.n - 1) * es : 0);
            const long long off = static_cast<long long>(chain) * D.tw_rows;
            twisted_chain<K, UNR, true, true>(x, x, chain ? -es : es, chain ? D.tw_n2 : D.tw_n1, D.tw_lmul + off * K,
                                        D.tw_ucol + off * K, D.tw_rdiag + off, D.tw_g + chain * 2 * K * K, mask);
        }
    }
}

// Issue L1 prefetches of `count` doubles from p (one per 128-byte line,
// spread over the block's threads); nothing waits for them.
__device__ __forceinline__ void prefetch_l1(const double* p, long long count) {
    const char* c = reinterpret_cast<const char*>(p);
    const long long bytes = count * static_cast<long long>(sizeof(double));
    for (long long off = static_cast<long long>(threadIdx.x) * 128; off < bytes; off += static_cast<long long>(blockDim.x) * 128)
        asm volatile("prefetch.global.L1 [%0];" ::"l"(c + off));
}

// every table the one-block step reads, so that its phases find them in L1
// rather than each taking its own trip to memory
template <int K>
__device__ __forceinline__ void prefetch_step_tables(const dim_dev& D, bool x_pass) {
    const long long band = static_cast<long long>(D.n) * (2 * K + 1);
    prefetch_l1(D.mrow, band);
    prefetch_l1(x_pass ? D.kdt : D.nrow, band);
    prefetch_l1(D.tw_lmul, 2LL * D.tw_rows * K);
    prefetch_l1(D.tw_ucol, 2LL * D.tw_rows * K);
    prefetch_l1(D.tw_g, 4LL * K * K);
}

template <int K>
__global__ void __launch_bounds__(512) small2d_step_kernel(const double* __restrict__ u, double* __restrict__ out,
                                                           dim_dev X, dim_dev Y) {
    extern __shared__ double sm[];
    constexpr int UNR = K > 2 ? 4 : 8;
    const int nx = X.n, ny = Y.n, N = nx * ny;
    double* U = sm;
    double* A = sm + N;
    double* C = sm + 2 * N;
    double* R = sm + 3 * N;
    if (!ADSG_SMEM_RANGE(sm, 4LL * N)) return;
    pdl_wait_and_release();  // the tables may come from the previous launch (the dt bands)
    prefetch_step_tables<K>(X, true);
    prefetch_step_tables<K>(Y, false);
    for (int g = threadIdx.x; g < N; g += blockDim.x) U[g] = u[g];
    __syncthreads();
    // y pass: A = My u, C = Ny u (pair sums on the symmetric rows, as launch_band_pass)
    const int ylo = max(Y.sym_lo, K), yhi = min(Y.sym_hi, ny - K);
    for (int g = threadIdx.x; g < N; g += blockDim.x) {
        if (yhi > ylo)
            band_out<K, false, true, true, false>(g, U, nullptr, A, C, Y.mrow, nullptr, Y.nrow, ny, nx, ylo, yhi, N);
        else
            band_out<K, false, true, false, false>(g, U, nullptr, A, C, Y.mrow, nullptr, Y.nrow, ny, nx, 0, 0, N);
    }
    __syncthreads();
    // x pass: R = (-dt Kx) A + Mx C
    for (int g = threadIdx.x; g < N; g += blockDim.x)
        band_out<K, true, false, false, false>(g, A, C, R, nullptr, X.kdt, X.mrow, nullptr, nx, 1, 0, 0, N);
    __syncthreads();
    // the step's solve order: the outer direction first, x last
    small_sweeps<K, UNR>(R, Y, nx, 1, nx);  // y-lines: columns of R
    __syncthreads();
    small_sweeps<K, UNR>(R, X, ny, nx, 1);  // x-lines: rows of R
    __syncthreads();
    for (int g = threadIdx.x; g < N; g += blockDim.x) out[g] = R[g];
}

// The same step on a thread-block cluster of kSmallClusterCtas CTAs: the four
// tensors live in the shared memory of the cluster's first CTA, every CTA
// computes a share of the two band passes reading and writing them through
// distributed shared memory (cluster barriers between the phases), and the
// first CTA then runs both sweeps on its own shared memory and writes the
// result.  The passes get the FP64 pipes of kSmallClusterCtas SMs instead of
// one; the sweeps, latency-bound chains, stay on one SM.  Same device
// functions as the separate kernels: the same bits.
constexpr int kSmallClusterCtas = 8;

template <int K>
__global__ void __launch_bounds__(256) small2d_cluster_step_kernel(const double* __restrict__ u, double* __restrict__ out,
                                                                   dim_dev X, dim_dev Y) {
    namespace cg = cooperative_groups;
    extern __shared__ double sm[];
    constexpr int UNR = K > 2 ? 4 : 8;
    cg::cluster_group cluster = cg::this_cluster();
    const unsigned rank = cluster.block_rank(), nblk = cluster.num_blocks();
    const int nx = X.n, ny = Y.n, N = nx * ny;
    // every CTA has the same dynamic shared memory: all decide alike, before any barrier
    if (!ADSG_SMEM_RANGE(sm, 4LL * N)) return;
    double* home = cluster.map_shared_rank(sm, 0);  // the first CTA's tensors
    double* U = home;
    double* A = home + N;
    double* C = home + 2 * N;
    double* R = home + 3 * N;
    pdl_wait_and_release();  // the tables may come from the previous launch (the dt bands)
    if (rank == 0) {
        prefetch_step_tables<K>(X, true);
        prefetch_step_tables<K>(Y, false);
    }
    const int tid = static_cast<int>(rank * blockDim.x + threadIdx.x), stride = static_cast<int>(nblk * blockDim.x);
    for (int g = tid; g < N; g += stride) U[g] = u[g];
    cluster.sync();
    // y pass: A = My u, C = Ny u (pair sums on the symmetric rows, as launch_band_pass)
    const int ylo = max(Y.sym_lo, K), yhi = min(Y.sym_hi, ny - K);
    for (int g = tid; g < N; g += stride) {
        if (yhi > ylo)
            band_out<K, false, true, true, 0>(g, U, nullptr, A, C, Y.mrow, nullptr, Y.nrow, ny, nx, ylo, yhi, N);
        else
            band_out<K, false, true, false, 0>(g, U, nullptr, A, C, Y.mrow, nullptr, Y.nrow, ny, nx, 0, 0, N);
    }
    cluster.sync();
    // x pass: R = (-dt Kx) A + Mx C
    for (int g = tid; g < N; g += stride)
        band_out<K, true, false, false, 0>(g, A, C, R, nullptr, X.kdt, X.mrow, nullptr, nx, 1, 0, 0, N);
    cluster.sync();  // nothing reads another CTA's shared memory after this
    if (rank != 0) return;
    double* Rl = sm + 3 * N;
    small_sweeps<K, UNR>(Rl, Y, nx, 1, nx);  // y-lines: columns of R
    __syncthreads();
    small_sweeps<K, UNR>(Rl, X, ny, nx, 1);  // x-lines: rows of R
    __syncthreads();
    for (int g = threadIdx.x; g < N; g += blockDim.x) out[g] = Rl[g];
}

template <int K>
static cudaError_t launch_small2d_cluster(const double* u, double* out, const dim_dev& x, const dim_dev& y, size_t smem,
                                          cudaStream_t s) {
    auto kern = small2d_cluster_step_kernel<K>;
    if (smem > 48 * 1024) {
        cudaError_t e = ensure_smem_attribute(reinterpret_cast<const void*>(kern), smem);
        if (e != cudaSuccess) return e;
    }
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(kSmallClusterCtas);
    cfg.blockDim = dim3(256);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[2];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = kSmallClusterCtas;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[1].val.programmaticStreamSerializationAllowed = pdl_enabled() ? 1 : 0;
    cfg.attrs = attr;
    cfg.numAttrs = 2;
    cudaError_t e = cudaLaunchKernelEx(&cfg, kern, u, out, x, y);
    return e != cudaSuccess ? e : cudaGetLastError();
}

size_t small2d_smem(const dim_dev& x, const dim_dev& y) { return sizeof(double) * 4 * static_cast<size_t>(x.n) * y.n; }

bool small2d_step_ok(const dim_dev& x, const dim_dev& y) {
    auto tw = [](const dim_dev& d) {
        return solve_variant_twisted(d.solve_variant) && d.tw_unit && d.tw_k == d.p && d.tw_k >= 1 && d.tw_k <= 4 &&
               d.tw_lmul != nullptr;
    };
    return tw(x) && tw(y) && x.p == y.p && small2d_smem(x, y) <= 200 * 1024;
}

cudaError_t launch_small2d_step(const double* u, double* out, const dim_dev& x, const dim_dev& y, cudaStream_t s) {
    if (!small2d_step_ok(x, y)) return cudaErrorInvalidValue;
    const size_t smem = small2d_smem(x, y);
    if (small2d_cluster_mode()) {
        switch (x.p) {
            case 1: return launch_small2d_cluster<1>(u, out, x, y, smem, s);
            case 2: return launch_small2d_cluster<2>(u, out, x, y, smem, s);
            case 3: return launch_small2d_cluster<3>(u, out, x, y, smem, s);
            default: return launch_small2d_cluster<4>(u, out, x, y, smem, s);
        }
    }
    auto go = [&](auto kern) -> cudaError_t {
        if (smem > 48 * 1024) {
            cudaError_t e = ensure_smem_attribute(reinterpret_cast<const void*>(kern), smem);
            if (e != cudaSuccess) return e;
        }
        return launch_pdl(kern, dim3(1), dim3(512), smem, s, u, out, x, y);
    };
    switch (x.p) {
        case 1: return go(small2d_step_kernel<1>);
        case 2: return go(small2d_step_kernel<2>);
        case 3: return go(small2d_step_kernel<3>);
        default: return go(small2d_step_kernel<4>);
    }
}

template <int K>
static cudaError_t rhs_x_solve_k(const double* in0, const double* in1, double* out, const double* A0,
                                 const double* A1, const dim_dev& d, const line_layout& L, cudaStream_t s) {
    if (d.tw_unit)
        return in1 ? rhs_x_solve_t<K, true, true>(in0, in1, out, A0, A1, d, L, s)
                   : rhs_x_solve_t<K, true, false>(in0, in1, out, A0, A1, d, L, s);
    return in1 ? rhs_x_solve_t<K, false, true>(in0, in1, out, A0, A1, d, L, s)
               : rhs_x_solve_t<K, false, false>(in0, in1, out, A0, A1, d, L, s);
}

bool rhs_x_solve_ok(const dim_dev& d, const line_layout& L) {
    return L.contiguous && d.tw_k >= 1 && d.tw_k <= 4 && d.tw_k == d.p && d.tw_lmul != nullptr &&
           twisted_staged_smem_per_warp(d.n) <= 227 * 1024;
}

cudaError_t launch_rhs_x_solve(const double* in0, const double* in1, double* out, const double* A0, const double* A1,
                               const dim_dev& d, const line_layout& L, cudaStream_t s) {
    if (!rhs_x_solve_ok(d, L)) return cudaErrorInvalidValue;
    if (L.nlines <= 0) return cudaSuccess;
    switch (d.tw_k) {
        case 1: return rhs_x_solve_k<1>(in0, in1, out, A0, A1, d, L, s);
        case 2: return rhs_x_solve_k<2>(in0, in1, out, A0, A1, d, L, s);
        case 3: return rhs_x_solve_k<3>(in0, in1, out, A0, A1, d, L, s);
        default: return rhs_x_solve_k<4>(in0, in1, out, A0, A1, d, L, s);
    }
}

template <int K, bool UNIT>
static cudaError_t twisted_t(double* data, const dim_dev& d, const line_layout& L, int variant, cudaStream_t s,
                             double* out = nullptr) {
    constexpr int UNR = K > 2 ? 4 : 8;
    if (!out) out = data;
    // one warp (16 lines) per block: the FP64 pipe is per SM, and single-warp
    // blocks spread the warps over the SMs most evenly
    if (variant == SOLVE_TWISTED_CHUNKED && L.contiguous) {
        return launch_pdl(line_solve_twisted_chunked_kernel<K, UNIT>,
                          dim3(static_cast<unsigned>((L.nlines + 15) / 16)), dim3(32),
                          twisted_chunked_smem_per_warp(), s, data, d, L);
    }
    if (variant == SOLVE_TWISTED_BULK && L.contiguous && out == data &&
        reinterpret_cast<uintptr_t>(data) % 16 == 0) {
        const size_t per_warp = twisted_bulk_smem_per_warp(d.n);
        const int wpb = tile_warps_per_block(per_warp);
        if (wpb == 0) return cudaErrorInvalidConfiguration;
        const size_t smem = per_warp * wpb;
        auto kern = line_solve_twisted_bulk_kernel<K, UNR, UNIT>;
        if (smem > 48 * 1024) {
            cudaError_t e = ensure_smem_attribute(reinterpret_cast<const void*>(kern), smem);
            if (e != cudaSuccess) return e;
        }
        const long long per = 16LL * wpb;
        return launch_pdl(kern, dim3(static_cast<unsigned>((L.nlines + per - 1) / per)), dim3(32 * wpb), smem, s, data,
                          d, L);
    }
    const bool staged = variant == SOLVE_TWISTED_STAGED || variant == SOLVE_TWISTED_BULK;  // bulk: unaligned fallback
    if (staged && L.contiguous) {
        const size_t per_warp = twisted_staged_smem_per_warp(d.n);
        const int wpb = tile_warps_per_block(per_warp);
        if (wpb == 0) return cudaErrorInvalidConfiguration;
        const size_t smem = per_warp * wpb;
        if (smem > 48 * 1024) {
            cudaError_t e =
                ensure_smem_attribute(reinterpret_cast<const void*>(line_solve_twisted_staged_kernel<K, UNR, UNIT>), smem);
            if (e != cudaSuccess) return e;
        }
        const long long per = 16LL * wpb;
        return launch_pdl(line_solve_twisted_staged_kernel<K, UNR, UNIT>, dim3(static_cast<unsigned>((L.nlines + per - 1) / per)),
                          dim3(32 * wpb), smem, s, static_cast<const double*>(data), out, d, L);
    }
    if (out != data) return cudaErrorNotSupported;  // only the tiled sweep writes elsewhere
    return launch_pdl(line_solve_twisted_kernel<K, UNR, UNIT>, dim3(static_cast<unsigned>((L.nlines + 15) / 16)),
                      dim3(32), 0, s, data, d, L);
}

template <int KL, int KU>
static cudaError_t line_solve_t(double* data, const dim_dev& d, const line_layout& L, int trans, cudaStream_t s) {
    const size_t smem = line_solve_smem_per_warp(d.n);
    if (smem > 48 * 1024) {
        cudaError_t e = ensure_smem_attribute(reinterpret_cast<const void*>(line_solve_kernel<KL, KU>), smem);
        if (e != cudaSuccess) return e;
    }
    const long long blocks = (L.nlines + 31) / 32;
    return launch_pdl(line_solve_kernel<KL, KU>, dim3(static_cast<unsigned>(blocks)), dim3(32), smem, s, data, d, L,
                      trans);
}

// staged kernel with several warps (one tile each) per block
template <int KL, int KU, int WPB>
__global__ void __launch_bounds__(32 * WPB) line_solve_staged_kernel(double* __restrict__ data, dim_dev D, line_layout L) {
    extern __shared__ double smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const long long line0 = (static_cast<long long>(blockIdx.x) * WPB + warp) * 32;
    if (line0 >= L.nlines) return;
    pdl_wait();
    const int nvalid = static_cast<int>(min(32LL, L.nlines - line0));
    double* base = smem + static_cast<size_t>(warp) * (D.n + kPadLo + kPadHi) * kPitch;
    double* s = base + kPadLo * kPitch;
    if (!ADSG_SMEM_RANGE(base, static_cast<long long>(D.n + kPadLo + kPadHi) * kPitch)) return;
    for (int r = 0; r < kPadLo; ++r) base[r * kPitch + lane] = 0.0;
    for (int r = 0; r < kPadHi; ++r) s[(D.n + r) * kPitch + lane] = 0.0;
    stage_in(data, s, L, D.n, line0, nvalid, lane);
    __syncwarp();
    sweep_n_reg<KL, KU, (KL > 2 ? 4 : 8)>(s + lane, D);
    __syncwarp();
    stage_out(data, s, L, D.n, line0, nvalid, lane);
}

template <int KL, int KU, int WPB>
static cudaError_t staged_t(double* data, const dim_dev& d, const line_layout& L, cudaStream_t s) {
    const size_t smem = line_solve_smem_per_warp(d.n) * WPB;
    if (smem > 227 * 1024) return cudaErrorInvalidConfiguration;
    if (smem > 48 * 1024) {
        cudaError_t e = ensure_smem_attribute(reinterpret_cast<const void*>(line_solve_staged_kernel<KL, KU, WPB>), smem);
        if (e != cudaSuccess) return e;
    }
    const long long per = 32LL * WPB;
    return launch_pdl(line_solve_staged_kernel<KL, KU, WPB>, dim3(static_cast<unsigned>((L.nlines + per - 1) / per)),
                      dim3(32 * WPB), smem, s, data, d, L);
}

template <int KL, int KU>
static cudaError_t line_solve_variant(int variant, double* data, const dim_dev& d, const line_layout& L, cudaStream_t s) {
    switch (variant) {
        case SOLVE_STAGED_1:
            return line_solve_t<KL, KU>(data, d, L, 0, s);
        case SOLVE_STAGED_2:
            return staged_t<KL, KU, 2>(data, d, L, s);
        case SOLVE_STAGED_4:
            return staged_t<KL, KU, 4>(data, d, L, s);
        case SOLVE_GLOBAL_4:
        default: {
            const long long per = 128;
            return launch_pdl(line_solve_global_kernel<KL, KU, (KL > 2 ? 4 : 8)>,
                              dim3(static_cast<unsigned>((L.nlines + per - 1) / per)), dim3(128), 0, s, data, d, L);
        }
    }
}

bool line_solve_variant_ok(int variant, const dim_dev& d) {
    if (variant == SOLVE_TWISTED || variant == SOLVE_TWISTED_CHUNKED)
        return d.tw_k >= 1 && d.tw_k <= 4 && d.tw_lmul != nullptr;
    if (variant == SOLVE_TWISTED_STAGED)
        return d.tw_k >= 1 && d.tw_k <= 4 && d.tw_lmul != nullptr && twisted_staged_smem_per_warp(d.n) <= 227 * 1024;
    if (variant == SOLVE_TWISTED_BULK)
        return d.tw_k >= 1 && d.tw_k <= 4 && d.tw_lmul != nullptr && twisted_bulk_smem_per_warp(d.n) <= 227 * 1024 &&
               twisted_staged_smem_per_warp(d.n) <= 227 * 1024;
    const int kl = d.kl, ku = d.ku_regular, w = d.w;
    const bool reg = (kl == 1 && ku <= 2 && w <= 3 && w >= 1) || (kl == 2 && ku <= 2 && w <= 4 && w >= 2) ||
                     (kl == 3 && ku <= 3 && w <= 6 && w >= 3) || (kl == 4 && ku <= 4 && w <= 8 && w >= 4);
    if (variant == SOLVE_STAGED_1) return line_solve_smem_per_warp(d.n) <= 227 * 1024;
    if (!reg) return false;
    if (variant == SOLVE_STAGED_2) return line_solve_smem_per_warp(d.n) * 2 <= 227 * 1024;
    if (variant == SOLVE_STAGED_4) return line_solve_smem_per_warp(d.n) * 4 <= 227 * 1024;
    return true;
}

// The x sweep that writes its tiles to another buffer (mapped host memory)
// is the whole-line staged one (variant 5, plain coalesced stores); it serves
// variant 7 too, whose results it equals bitwise.
bool line_solve_out_ok(const dim_dev& d, const line_layout& L) {
    return L.contiguous && (d.solve_variant == SOLVE_TWISTED_STAGED || d.solve_variant == SOLVE_TWISTED_BULK) &&
           line_solve_variant_ok(SOLVE_TWISTED_STAGED, d);
}

cudaError_t launch_line_solve_out(const double* data, double* out, const dim_dev& d, const line_layout& L,
                                  cudaStream_t s) {
    if (!line_solve_out_ok(d, L)) return cudaErrorNotSupported;
    if (L.nlines <= 0) return cudaSuccess;
    double* in = const_cast<double*>(data);  // read only: the tiled sweep writes out
    if (d.tw_unit) {
        switch (d.tw_k) {
            case 1: return twisted_t<1, true>(in, d, L, SOLVE_TWISTED_STAGED, s, out);
            case 2: return twisted_t<2, true>(in, d, L, SOLVE_TWISTED_STAGED, s, out);
            case 3: return twisted_t<3, true>(in, d, L, SOLVE_TWISTED_STAGED, s, out);
            default: return twisted_t<4, true>(in, d, L, SOLVE_TWISTED_STAGED, s, out);
        }
    }
    switch (d.tw_k) {
        case 1: return twisted_t<1, false>(in, d, L, SOLVE_TWISTED_STAGED, s, out);
        case 2: return twisted_t<2, false>(in, d, L, SOLVE_TWISTED_STAGED, s, out);
        case 3: return twisted_t<3, false>(in, d, L, SOLVE_TWISTED_STAGED, s, out);
        default: return twisted_t<4, false>(in, d, L, SOLVE_TWISTED_STAGED, s, out);
    }
}

cudaError_t launch_line_solve(double* data, const dim_dev& d, const line_layout& L, int trans, cudaStream_t s) {
    if (L.nlines <= 0) return cudaSuccess;
    // the register sweeps need the L table stride to equal KL and a regular
    // U extent (columns beyond it take the wide-column branch)
    const int kl = d.kl, ku = d.ku_regular, w = d.w;
    const int v = trans ? SOLVE_STAGED_1 : d.solve_variant;
    if (!trans && solve_variant_twisted(v) && line_solve_variant_ok(v, d)) {
        if (d.tw_unit) {
            switch (d.tw_k) {
                case 1: return twisted_t<1, true>(data, d, L, v, s);
                case 2: return twisted_t<2, true>(data, d, L, v, s);
                case 3: return twisted_t<3, true>(data, d, L, v, s);
                default: return twisted_t<4, true>(data, d, L, v, s);
            }
        }
        switch (d.tw_k) {
            case 1: return twisted_t<1, false>(data, d, L, v, s);
            case 2: return twisted_t<2, false>(data, d, L, v, s);
            case 3: return twisted_t<3, false>(data, d, L, v, s);
            default: return twisted_t<4, false>(data, d, L, v, s);
        }
    }
    if (!trans && v != SOLVE_STAGED_1 && !solve_variant_twisted(v) && line_solve_variant_ok(v, d)) {
        if (kl == 1 && ku <= 1 && w <= 2) return line_solve_variant<1, 1>(v, data, d, L, s);
        if (kl == 1 && ku <= 2 && w <= 3) return line_solve_variant<1, 2>(v, data, d, L, s);
        if (kl == 2) return line_solve_variant<2, 2>(v, data, d, L, s);
        if (kl == 3) return line_solve_variant<3, 3>(v, data, d, L, s);
        if (kl == 4) return line_solve_variant<4, 4>(v, data, d, L, s);
    }
    if (line_solve_smem_per_warp(d.n) > 227 * 1024)
        return launch_pdl(line_solve_long_kernel, dim3(static_cast<unsigned>((L.nlines + 127) / 128)), dim3(128), 0, s,
                          data, d, L, trans);
    if (kl == 1 && ku <= 1 && w <= 2 && w >= 1) return line_solve_t<1, 1>(data, d, L, trans, s);
    if (kl == 1 && ku <= 2 && w <= 3 && w >= 2) return line_solve_t<1, 2>(data, d, L, trans, s);
    if (kl == 2 && ku <= 2 && w <= 4 && w >= 2) return line_solve_t<2, 2>(data, d, L, trans, s);
    if (kl == 3 && ku <= 3 && w <= 6 && w >= 3) return line_solve_t<3, 3>(data, d, L, trans, s);
    if (kl == 4 && ku <= 4 && w <= 8 && w >= 4) return line_solve_t<4, 4>(data, d, L, trans, s);
    return line_solve_t<0, 0>(data, d, L, trans, s);
}

// ---------------------------------------------------------------------------
// Generalised ADS (reference include/ads/solver.hpp:47-195): along one
// "special" direction every grid line has its own factorised band.  Each lane
// sweeps one line in global memory with that line's tables, in LAPACK's
// column order (forward with row exchanges, backward over the full kl+ku U
// band, reciprocal diagonal).  Line l is numbered as the reference numbers
// the lines handed to its special-dimension callable: over the directions
// that follow the special one cyclically, the first of them fastest.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) line_solve_permat_kernel(double* __restrict__ data, line_tables T,
                                                                line_layout L, const int* __restrict__ line_matrix,
                                                                int nx, int nz, int special, int ndim) {
    const long long g = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (g >= L.nlines) return;
    // reference line number of my line
    long long ref = g;
    if (ndim == 3 && special == 1) ref = (g / nx) + static_cast<long long>(nz) * (g % nx);
    const long long m = line_matrix[ref];
    const int n = T.n, kl = T.kl, w = T.w;
    const double* lmul = T.lmul + m * static_cast<long long>(n) * kl;
    const double* ucol = T.ucol + m * static_cast<long long>(n) * w;
    const double* rdiag = T.rdiag + m * static_cast<long long>(n);
    const int* piv = T.piv + m * static_cast<long long>(n);
    const int* uext = T.uext + m * static_cast<long long>(n);
    double* x = data + (L.contiguous ? g * n : (g % L.a) * L.sa + (g / L.a) * L.sb);
    const long long es = L.elem_stride;
    if (!ADSG_LINE_OK(data, x, n, es, L.total)) return;
    for (int j = 0; j < n - 1; ++j) {
        const int l = __ldg(piv + j);
        if (l != j) {
            const double t = x[l * es];
            x[l * es] = x[j * es];
            x[j * es] = t;
        }
        const double y = -x[j * es];
        const int lm = min(kl, n - 1 - j);
        for (int i = 1; i <= lm; ++i) x[(j + i) * es] = fma(y, __ldg(lmul + static_cast<long long>(j) * kl + i - 1), x[(j + i) * es]);
    }
    for (int j = n - 1; j >= 0; --j) {
        const double v = x[j * es] * __ldg(rdiag + j);
        x[j * es] = v;
        const int ext = __ldg(uext + j);
        for (int d = 1; d <= ext; ++d) x[(j - d) * es] = fma(-v, __ldg(ucol + static_cast<long long>(j) * w + d - 1), x[(j - d) * es]);
    }
}

cudaError_t launch_line_solve_permat(double* data, const line_tables& T, const line_layout& L, const int* line_matrix,
                                     int nx, int nz, int special, int ndim, cudaStream_t s) {
    if (L.nlines <= 0) return cudaSuccess;
    line_solve_permat_kernel<<<(L.nlines + 127) / 128, 128, 0, s>>>(data, T, L, line_matrix, nx, nz, special, ndim);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Vector helpers of the adjoint driver.  The dot product is deterministic: a
// fixed grid writes block partial sums in a fixed order, one block adds them.
// ---------------------------------------------------------------------------
__global__ void axpby_kernel(double* __restrict__ y, double a, const double* __restrict__ x, double b, long long n) {
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x)
        y[i] = fma(a, x[i], b * y[i]);
}

cudaError_t launch_axpby(double* y, double a, const double* x, double b, long long n, cudaStream_t s) {
    const long long blocks = std::min<long long>((n + 255) / 256, 152 * 16);
    axpby_kernel<<<static_cast<int>(std::max<long long>(blocks, 1)), 256, 0, s>>>(y, a, x, b, n);
    return cudaGetLastError();
}

constexpr int kDotBlocks = 1024;

__global__ void dot_partial_kernel(const double* __restrict__ x, const double* __restrict__ y, long long n,
                                   double* __restrict__ partial) {
    __shared__ double sh[256];
    double acc = 0.0;
    for (long long i = blockIdx.x * 256LL + threadIdx.x; i < n; i += 256LL * gridDim.x) acc = fma(x[i], y[i], acc);
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

__global__ void dot_final_kernel(const double* __restrict__ partial, int m, double* __restrict__ out) {
    __shared__ double sh[256];
    double acc = 0.0;
    for (int i = threadIdx.x; i < m; i += 256) acc += partial[i];
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = sh[0];
}

__global__ void count_nonfinite_kernel(const double* __restrict__ x, long long n, unsigned long long* __restrict__ count) {
    unsigned long long local = 0;
    for (long long i = blockIdx.x * 256LL + threadIdx.x; i < n; i += 256LL * gridDim.x) local += isfinite(x[i]) ? 0 : 1;
    for (int o = 16; o > 0; o >>= 1) local += __shfl_down_sync(0xffffffffu, local, o);
    if ((threadIdx.x & 31) == 0 && local) atomicAdd(count, local);
}

// Dirichlet planes: the dofs of an x-fastest nx x ny x nz tensor whose index
// along direction d is k, set to values[t] (t over the plane's dofs, x-fastest
// over the other directions) or to 0 when values is NULL.
__global__ void set_plane_kernel(double* __restrict__ u, const double* __restrict__ values, long long nx, long long ny,
                                 long long nz, int d, long long k, long long count) {
    const long long t = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= count) return;
    long long i, j, l;
    if (d == 0) {
        i = k;
        j = t % ny;
        l = t / ny;
    } else if (d == 1) {
        j = k;
        i = t % nx;
        l = t / nx;
    } else {
        l = k;
        i = t % nx;
        j = t / nx;
    }
    const long long g = i + nx * (j + ny * l);
    if (ADSG_IN(g, nx * ny * nz)) u[g] = values ? values[t] : 0.0;
}

cudaError_t launch_set_plane(double* u, const double* values, const int* n, int ndim, int d, int k, cudaStream_t s) {
    const long long nx = n[0], ny = ndim > 1 ? n[1] : 1, nz = ndim > 2 ? n[2] : 1;
    const long long count = nx * ny * nz / n[d];
    if (count <= 0) return cudaSuccess;
    set_plane_kernel<<<static_cast<unsigned>((count + 255) / 256), 256, 0, s>>>(u, values, nx, ny, nz, d, k, count);
    return cudaGetLastError();
}

cudaError_t launch_count_nonfinite(const double* x, long long n, unsigned long long* count, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(count, 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
    const long long blocks = std::min<long long>((n + 255) / 256, 152 * 8);
    count_nonfinite_kernel<<<static_cast<int>(std::max<long long>(blocks, 1)), 256, 0, s>>>(x, n, count);
    return cudaGetLastError();
}

cudaError_t launch_sum(const double* partial, int m, double* out, cudaStream_t s) {
    dot_final_kernel<<<1, 256, 0, s>>>(partial, m, out);
    return cudaGetLastError();
}

cudaError_t launch_dot(const double* x, const double* y, long long n, double* partial, double* out, cudaStream_t s) {
    dot_partial_kernel<<<kDotBlocks, 256, 0, s>>>(x, y, n, partial);
    dot_final_kernel<<<1, 256, 0, s>>>(partial, kDotBlocks, out);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Batched engine: many independent cubic heat problems (2D or 3D, p <= 4)
// advanced by one persistent cooperative launch.  A step is six stages per
// instance (RHS passes outer / middle / x, then the x, y, z line solves).
// The work of every stage of every instance is cut into items (2048 outputs
// of a pass; 128 lines of a two-ended solve, 256 of a LAPACK-order one), and
// the items of all steps, stages and instances form one sequence (step-major,
// then stage, then instance).  Blocks take the next item from a global
// counter; before working on it they wait until the same instance has
// finished its previous stage (a per-instance, per-stage count of completed
// items), so each instance runs its stages in order while the instances
// overlap freely -- no grid-wide barrier, no stage waits for the slowest
// instance.  Items are handed out in sequence order and every dependency lies
// earlier in the sequence, so with all blocks resident (cooperative launch)
// the earliest unfinished item can always proceed.  Waits are bounded: past
// the spin limit a block sets the error word and the launch winds down.
// The kernels are those of the single-instance step: pair-sum band passes,
// row-scaled right-hand sides and unit-diagonal two-ended sweeps (chunked
// through shared memory on the contiguous x-lines), reading data written
// earlier in the launch through L2.
// ---------------------------------------------------------------------------
namespace {

// Work per item: outputs of a band pass, lines of a two-ended sweep (8 warps
// x 16), lines of a LAPACK-order sweep (one per thread).  Larger pass items
// spread the per-item cost (the counter, the wait, the completion count) over
// more work: 1.54 / 1.37 / 1.33 / 1.47 ms per step of the 64-instance set at
// 2048 / 8192 / 16384 / 32768 outputs (stage-major order); two rounds of
// sweeps per warp and item took 1.53 ms against 1.33.
constexpr int kBatchPassUnits = 16384, kBatchTwistedLines = 128, kBatchLapackLines = 256;

// One item of a band pass: kBatchPassUnits consecutive outputs, 256 at a
// time.  The buffers of a pass never overlap (each stage reads the tensors the
// one before wrote and writes others), which the restrict qualifiers tell the
// compiler: the loads of later outputs can then be issued before the stores
// of earlier ones, several outputs' loads in flight per thread -- what keeps
// the FP64 pipe fed at the kernel's 16 resident warps per SM.
template <int P, bool IN1, bool OUT1, bool SYM>
__device__ __forceinline__ void batch_pass_run(long long first, long long size, const double* __restrict__ in0,
                                               const double* __restrict__ in1, double* __restrict__ out0,
                                               double* __restrict__ out1, const double* __restrict__ A0,
                                               const double* __restrict__ A1, const double* __restrict__ B0,
                                               int n_axis, long long stride, int lo, int hi) {
#pragma unroll 4
    for (int k = 0; k < kBatchPassUnits / 256; ++k) {
        const long long g = first + k * 256 + threadIdx.x;
        if (g < size) band_out<P, IN1, OUT1, SYM, 2>(g, in0, in1, out0, out1, A0, A1, B0, n_axis, stride, lo, hi, size);
    }
}

template <int P>
__device__ __forceinline__ void batch_pass(const batch_inst& I, int stage, long long first, int par) {
    const double* cur = I.buf[par];
    double* nxt = I.buf[par ^ 1];
    const int n = I.n;
    const dim_dev& D = I.dim;
    const long long nn = static_cast<long long>(n) * n, size = I.size;
    const int lo = max(D.sym_lo, P), hi = min(D.sym_hi, n - P);
    const bool sym = hi > lo;
    // the outer axis (z in 3D, y in 2D), then y in 3D, then x
    const long long outer = I.ndim == 3 ? nn : n;
    if (stage == 0) {
        if (sym)
            batch_pass_run<P, false, true, true>(first, size, cur, nullptr, I.T[0], I.T[1], D.mrow, nullptr, D.nrow, n,
                                                 outer, lo, hi);
        else
            batch_pass_run<P, false, true, false>(first, size, cur, nullptr, I.T[0], I.T[1], D.mrow, nullptr, D.nrow, n,
                                                  outer, 0, 0);
    } else if (stage == 1) {  // 3D only
        if (sym)
            batch_pass_run<P, true, true, true>(first, size, I.T[0], I.T[1], I.T[2], I.T[3], D.kdt, D.mrow, D.mrow, n, n,
                                                lo, hi);
        else
            batch_pass_run<P, true, true, false>(first, size, I.T[0], I.T[1], I.T[2], I.T[3], D.kdt, D.mrow, D.mrow, n,
                                                 n, 0, 0);
    } else if (I.ndim == 3) {
        batch_pass_run<P, true, false, false>(first, size, I.T[3], I.T[2], nxt, nullptr, D.kdt, D.mrow, nullptr, n, 1,
                                              0, 0);
    } else {
        batch_pass_run<P, true, false, false>(first, size, I.T[0], I.T[1], nxt, nullptr, D.kdt, D.mrow, nullptr, n, 1,
                                              0, 0);
    }
}

// Where line g of direction dir (0 x, 1 y, 2 z) of an instance starts, and
// its element stride.
__device__ __forceinline__ long long batch_line(const batch_inst& I, int dir, long long g, long long* es) {
    const long long n = I.n, nn = n * n;
    if (dir == 0) {
        *es = 1;
        return g * n;
    }
    if (dir == 1) {
        *es = n;
        return I.ndim == 3 ? (g % n) + (g / n) * nn : g;
    }
    *es = nn;
    return g;
}

// Two-ended unit-diagonal sweeps of 128 lines: 8 warps x 16 lines.
template <int K>
__device__ __forceinline__ void batch_solve_twisted(const batch_inst& I, int stage, long long first, int par,
                                                    double* wbuf) {
    double* x = I.buf[par ^ 1];
    const dim_dev& D = I.dim;
    const int n = I.n, dir = stage - 3;
    const long long lines = I.units[stage];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const long long g0 = first + static_cast<long long>(warp) * 16;
    if (g0 >= lines) return;  // whole warp
    if (dir == 0) {
        // contiguous x-lines: streamed through this warp's shared chunk buffer
        chunk_lines W;
        W.data = x + g0 * n;
        W.n = n;
        W.n1 = D.tw_n1;
        W.n2 = D.tw_n2;
        W.nv = static_cast<int>(min(16LL, lines - g0));
        if (!(ADSG_SMEM_RANGE(wbuf, 2LL * 16 * kChunkPitch) && ADSG_IN(g0 * n, I.size) &&
              ADSG_IN((g0 + W.nv) * n - 1, I.size)))
            return;
        chunked_twisted_warp<K, true, true>(W, D, wbuf);
        return;
    }
    const int chain = lane >> 4;
    const long long g = g0 + (lane & 15);
    long long es = 1;
    double* xl = x + batch_line(I, dir, g < lines ? g : 0, &es);
    const bool active = g < lines && ADSG_LINE_OK(x, xl, n, es, I.size);
    const unsigned mask = __ballot_sync(0xffffffffu, active);  // lanes g and g^16 share a line
    if (!active) return;
    const long long off = static_cast<long long>(chain) * D.tw_rows;
    if (chain) xl += static_cast<long long>(n - 1) * es;
    twisted_chain<K, (K > 2 ? 4 : 8), true, false, true>(xl, xl, chain ? -es : es, chain ? D.tw_n2 : D.tw_n1,
                                                         D.tw_lmul + off * K, D.tw_ucol + off * K, D.tw_rdiag + off,
                                                         D.tw_g + chain * 2 * K * K, mask);
}

// LAPACK-order sweeps (instances without two-ended tables): one line per thread.
template <int P>
__device__ __forceinline__ void batch_solve_lapack(const batch_inst& I, int stage, long long g, int par) {
    if (g >= I.units[stage]) return;
    double* x = I.buf[par ^ 1];
    long long es = 1;
    double* xl = x + batch_line(I, stage - 3, g, &es);
    if (ADSG_LINE_OK(x, xl, I.n, es, I.size)) sweep_global<P, P, (P > 2 ? 4 : 8), true>(xl, es, I.dim);
}

// Thread 0: wait until instance i has finished the stage before (stage, step
// t) -- the nearest earlier stage with work, in this step or the last.
// Returns 0 when the wait ran out (or another block's did): the error word is
// set and the launch winds down.
__device__ __noinline__ int batch_wait(const batch_dev& B, const batch_inst& I, int i, int stage, int t) {
    int ps = stage, pt = t;
    do {
        if (ps == 0) {
            if (pt == 0) return 1;  // the launch's first stage of this instance
            ps = 5;
            --pt;
        } else {
            --ps;
        }
    } while (I.items[ps] == 0);
    const unsigned target = static_cast<unsigned>((pt + 1) * I.items[ps]) + B.wait_extra;
    const volatile unsigned* c = B.done + i * 6 + ps;
    long long spins = 0;
    while (*c < target) {
        if (++spins > B.spin_limit || *reinterpret_cast<volatile int*>(B.err) != 0) {
            atomicExch(B.err, 1);
            return 0;
        }
        __nanosleep(64);
    }
    __threadfence();
    return 1;
}

__global__ void __launch_bounds__(256) batch_steps_kernel(batch_dev B, int nsteps, int par0) {
    extern __shared__ double smem[];  // per warp: 2 x 16 x kChunkPitch doubles for the x-lines
    __shared__ long long s_item;
    __shared__ int s_go;
    double* wbuf = smem + static_cast<size_t>(threadIdx.x >> 5) * 2 * 16 * kChunkPitch;
    const long long total = static_cast<long long>(nsteps) * B.per_step;
    const int pairs = 6 * B.count;
    for (;;) {
        if (threadIdx.x == 0) s_item = static_cast<long long>(atomicAdd(B.next, 1ULL));
        __syncthreads();
        const long long item = s_item;
        if (item >= total) return;
        const int t = static_cast<int>(item / B.per_step);
        const long long r = item - static_cast<long long>(t) * B.per_step;
        int lo = 0, hi = pairs;  // the position k with prefix[k] <= r < prefix[k+1]
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (B.prefix[mid] <= r) lo = mid; else hi = mid;
        }
        const int k = B.pair[lo], stage = k / B.count, i = k - stage * B.count;
        const batch_inst& I = B.inst[i];
        const long long it = r - B.prefix[lo];
        if (threadIdx.x == 0) s_go = batch_wait(B, I, i, stage, t);
        __syncthreads();
        if (!s_go) return;
        const int par = (par0 + t) & 1;
        if (stage < 3) {
            switch (I.p) {
                case 1: batch_pass<1>(I, stage, it * kBatchPassUnits, par); break;
                case 2: batch_pass<2>(I, stage, it * kBatchPassUnits, par); break;
                case 3: batch_pass<3>(I, stage, it * kBatchPassUnits, par); break;
                default: batch_pass<4>(I, stage, it * kBatchPassUnits, par); break;
            }
        } else if (I.twisted) {
            switch (I.p) {
                case 1: batch_solve_twisted<1>(I, stage, it * kBatchTwistedLines, par, wbuf); break;
                case 2: batch_solve_twisted<2>(I, stage, it * kBatchTwistedLines, par, wbuf); break;
                case 3: batch_solve_twisted<3>(I, stage, it * kBatchTwistedLines, par, wbuf); break;
                default: batch_solve_twisted<4>(I, stage, it * kBatchTwistedLines, par, wbuf); break;
            }
        } else {
            const long long g = it * kBatchLapackLines + threadIdx.x;
            switch (I.p) {
                case 1: batch_solve_lapack<1>(I, stage, g, par); break;
                case 2: batch_solve_lapack<2>(I, stage, g, par); break;
                case 3: batch_solve_lapack<3>(I, stage, g, par); break;
                default: batch_solve_lapack<4>(I, stage, g, par); break;
            }
        }
        __syncthreads();  // every thread's writes of the item precede its completion count
        if (threadIdx.x == 0) {
            __threadfence();
            atomicAdd(B.done + i * 6 + stage, 1u);
        }
    }
}

}  // namespace

const void* batch_kernel_symbol() { return reinterpret_cast<const void*>(batch_steps_kernel); }

size_t batch_smem_bytes() { return sizeof(double) * 8 * 2 * 16 * kChunkPitch; }

int batch_units_per_item(int stage, int twisted) {
    return stage < 3 ? kBatchPassUnits : (twisted ? kBatchTwistedLines : kBatchLapackLines);
}

cudaError_t batch_prepare_kernel() {
    return ensure_smem_attribute(batch_kernel_symbol(), batch_smem_bytes());
}

int batch_max_blocks_per_sm() {
    int nb = 0;
    if (batch_prepare_kernel() != cudaSuccess) return 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, batch_steps_kernel, 256, batch_smem_bytes());
    return nb;
}

}  // namespace adsg
