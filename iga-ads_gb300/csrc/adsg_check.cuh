// Device-side bounds checks of the debug build (compiled with
// -DADSG_BOUNDS_CHECK=1 into libads_gb300_checked.so by build.py --checked).
//
// In that build every global-memory index of the step, solve, batch and
// element kernels is compared with the extent of the buffer it addresses,
// and every shared-memory tile a kernel sweeps is compared with the dynamic
// shared memory the launch was given.  A violation does not trap: the access
// is skipped (a load reads 0), a counter and the first offending index,
// extent and source line are recorded in a per-translation-unit __device__
// record, and adsg_debug_bounds() reports them to the host.  In the release
// build every check is the constant true and compiles away.
#ifndef ADSG_CHECK_CUH
#define ADSG_CHECK_CUH

#include <cuda_runtime.h>

#ifndef ADSG_BOUNDS_CHECK
#define ADSG_BOUNDS_CHECK 0
#endif

namespace adsg {

struct bounds_record {
    unsigned long long count;  // violations since the last reset
    long long index, extent;   // the first one
    int line;
    int pad;
};

#if ADSG_BOUNDS_CHECK
// One record per translation unit (the engine is built without relocatable
// device code); ADSG_BOUNDS_TU below defines the host function that reads it.
static __device__ bounds_record g_bounds_record;

static __device__ __noinline__ void bounds_violation(long long i, long long n, int line) {
    if (atomicAdd(&g_bounds_record.count, 1ULL) == 0ULL) {
        g_bounds_record.index = i;
        g_bounds_record.extent = n;
        g_bounds_record.line = line;
        __threadfence();
    }
}

static __device__ __forceinline__ bool bounds_ok(long long i, long long n, int line) {
    if (i >= 0 && i < n) return true;
    bounds_violation(i, n, line);
    return false;
}

// Whether [p, p + count) lies inside the launch's dynamic shared memory.
static __device__ __forceinline__ bool smem_range_ok(const double* p, long long count, int line) {
    extern __shared__ double adsg_dynamic_smem[];
    unsigned bytes;
    asm volatile("mov.u32 %0, %%dynamic_smem_size;" : "=r"(bytes));
    const long long lo = p - adsg_dynamic_smem;
    const long long cap = static_cast<long long>(bytes / sizeof(double));
    if (lo >= 0 && lo + count <= cap) return true;
    bounds_violation(lo < 0 ? lo : lo + count - 1, cap, line);
    return false;
}

#define ADSG_IN(i, n) ::adsg::bounds_ok(static_cast<long long>(i), static_cast<long long>(n), __LINE__)
#define ADSG_SMEM_RANGE(p, count) ::adsg::smem_range_ok((p), static_cast<long long>(count), __LINE__)
#define ADSG_BOUNDS_TU(name)                                                                       \
    int bounds_read_##name(::adsg::bounds_record* out, int reset) {                                \
        cudaError_t e = cudaMemcpyFromSymbol(out, g_bounds_record, sizeof(::adsg::bounds_record)); \
        if (e == cudaSuccess && reset) {                                                           \
            const ::adsg::bounds_record zero{};                                                     \
            e = cudaMemcpyToSymbol(g_bounds_record, &zero, sizeof(zero));                          \
        }                                                                                          \
        return e == cudaSuccess ? 1 : -static_cast<int>(e);                                        \
    }
#else
#define ADSG_IN(i, n) (true)
#define ADSG_SMEM_RANGE(p, count) (true)
#define ADSG_BOUNDS_TU(name)                                             \
    int bounds_read_##name(::adsg::bounds_record* out, int) {            \
        *out = ::adsg::bounds_record{};                                  \
        return 0;                                                        \
    }
#endif

// The per-translation-unit readers (1: read, 0: not a checked build, < 0: a
// CUDA error).
int bounds_read_kernels(bounds_record* out, int reset);
int bounds_read_elem(bounds_record* out, int reset);
int bounds_read_quad(bounds_record* out, int reset);

}  // namespace adsg

#endif
