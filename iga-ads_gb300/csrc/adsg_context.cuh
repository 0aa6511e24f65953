// The engine's context (the opaque adsg_ctx of the C-ABI) and the helpers
// shared by the translation units that implement its entry points.
#ifndef ADSG_CONTEXT_CUH
#define ADSG_CONTEXT_CUH

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "adsg_internal.hpp"
#include "adsg_kernels.cuh"

// returns from the enclosing entry point with ADSG_ERR_CUDA (and the error
// recorded) when a CUDA call fails
#define ADSG_CUDA_TRY(expr, where)                          \
    do {                                                    \
        cudaError_t e_ = (expr);                            \
        if (e_ != cudaSuccess) return fail_cuda(e_, where); \
    } while (0)

namespace adsg {

// Device allocations of one context, freed together.
struct dev_arena {
    std::vector<void*> blocks;
    ~dev_arena() {
        for (void* p : blocks) cudaFree(p);
    }
    template <typename T>
    cudaError_t alloc(T** out, size_t count) {
        void* p = nullptr;
        cudaError_t e = device_alloc(&p, std::max<size_t>(count, 1) * sizeof(T));
        if (e != cudaSuccess) return e;
        blocks.push_back(p);
        *out = static_cast<T*>(p);
        return cudaSuccess;
    }
    template <typename T>
    cudaError_t upload(T** out, const T* src, size_t count, cudaStream_t s) {
        cudaError_t e = alloc(out, count);
        if (e != cudaSuccess) return e;
        return cudaMemcpyAsync(*out, src, count * sizeof(T), cudaMemcpyHostToDevice, s);
    }
};

void detach_adjoints(adsg_ctx* c);

}  // namespace adsg

using adsg::dev_arena;
using adsg::dim_dev;

struct adsg_ctx {
    int ndim = 0;
    int n[3] = {1, 1, 1};
    long long size = 0;
    dim_dev dims[3];
    double* nrow[3] = {nullptr, nullptr, nullptr};
    double* kdt[3] = {nullptr, nullptr, nullptr};
    // The explicit step's own view of each direction.  Where the direction is
    // solved with a two-ended sweep, its band rows are pre-multiplied by
    // 1 / U(r, r) of that sweep's factors and the solve tables are the unit-
    // diagonal ones: the RHS passes deliver the row-scaled right-hand side at
    // no extra cost and the backward sweeps drop their multiply.  Elsewhere
    // sdims[d] equals dims[d].
    dim_dev sdims[3];
    double* snrow[3] = {nullptr, nullptr, nullptr};
    double* skdt[3] = {nullptr, nullptr, nullptr};
    double band_dt = std::nan("");
    double* scratch[4] = {nullptr, nullptr, nullptr, nullptr};
    double* ping = nullptr;  // second state buffer of the step loop
    double uext_sum[3] = {0, 0, 0};  // sum over columns of the applied U extents
    double* host_io = nullptr;
    double* red = nullptr;  // 1025 doubles: dot-product partials + result
    std::vector<double> xq[3];  // Gauss points per direction (empty if not described)
    double* qpool = nullptr;    // Gauss-point work space (grown on demand)
    size_t qpool_size = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    // second stream and fork/join events of the host entry's slab-chunked
    // first and last steps (created on first use)
    cudaStream_t aux = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    cudaEvent_t ev_chunk[16] = {};  // one per slab chunk
    int host_chunks = -1;  // slab chunks of the host entry (1 = none); -1 = not chosen yet
    dev_arena arena;
    // graph of two steps u -> ping -> u, specialised on (u, dt)
    cudaGraphExec_t graph = nullptr;
    double graph_dt = std::nan("");
    double* graph_u = nullptr;
    // single-step graphs of adsg_heat_step, specialised on (prev, next, dt):
    // a replayed graph runs the step's kernels back to back with shorter gaps
    // than stream launches (130^3 p=2: 191.5 against 201.6 us per step)
    struct step_graph {
        const double* prev;
        double* next;
        double dt;
        cudaGraphExec_t exec;
    };
    std::vector<step_graph> step_graphs;  // most recently used last
    long long step_graph_hits = 0, step_graph_misses = 0;
    int step_graphs_on = 1;  // chosen at creation: replay pays on all but launch-bound grids
    // the host-buffer steps (upload pass, steps, download) of one pinned buffer
    cudaGraphExec_t host_graph = nullptr;
    const double* host_graph_u = nullptr;
    double host_graph_dt = std::nan("");
    int host_graph_steps = 0;
    void drop_step_graphs() {
        for (auto& g : step_graphs) cudaGraphExecDestroy(g.exec);
        step_graphs.clear();
        if (host_graph) cudaGraphExecDestroy(host_graph);
        host_graph = nullptr;
        host_graph_u = nullptr;
    }
    // stage timers
    bool timing = false;
    bool capturing = false;
    struct timed { int stage; cudaEvent_t a, b; };
    std::vector<timed> pending;
    std::vector<cudaEvent_t> spare;
    double stage_ms[ADSG_NSTAGES] = {};
    long long stage_launches[ADSG_NSTAGES] = {};
    // adjoints created on this context (detached when the context goes first)
    std::vector<adsg_adjoint*> adjoints;
    int pdl = 0;     // programmatic dependent launch for the step kernels (chosen at creation)
    int fuse_x = 0;  // the step fuses the x band pass with the x solve (chosen at creation)
    int step_1block = 0;  // small 2D grids: the whole step in one launch (chosen at creation)
    int step_cluster = 0;  // ... on a thread-block cluster rather than one block (chosen at creation)

    cudaEvent_t take_event() {
        if (!spare.empty()) {
            cudaEvent_t e = spare.back();
            spare.pop_back();
            return e;
        }
        cudaEvent_t e = nullptr;
        cudaEventCreate(&e);
        return e;
    }
    void drain() {
        for (auto& t : pending) {
            float ms = 0.f;
            if (cudaEventElapsedTime(&ms, t.a, t.b) == cudaSuccess) {
                stage_ms[t.stage] += ms;
                stage_launches[t.stage] += 1;
            }
            spare.push_back(t.a);
            spare.push_back(t.b);
        }
        pending.clear();
    }

    ~adsg_ctx() {
        if (graph) cudaGraphExecDestroy(graph);
        drop_step_graphs();
        if (stream) cudaStreamSynchronize(stream);
        if (qpool) cudaFree(qpool);
        for (auto& t : pending) {
            cudaEventDestroy(t.a);
            cudaEventDestroy(t.b);
        }
        for (auto e : spare) cudaEventDestroy(e);
        if (aux) {
            cudaStreamSynchronize(aux);
            cudaStreamDestroy(aux);
        }
        if (ev_fork) cudaEventDestroy(ev_fork);
        if (ev_join) cudaEventDestroy(ev_join);
        for (auto e : ev_chunk)
            if (e) cudaEventDestroy(e);
        if (own_stream && stream) cudaStreamDestroy(stream);
    }
};

// Brackets one kernel launch with timer events when timers are on.
struct stage_scope {
    adsg_ctx* c;
    int stage;
    cudaEvent_t a = nullptr;
    stage_scope(adsg_ctx* ctx, int st) : c(ctx), stage(st) {
        if (c->timing && !c->capturing) {
            a = c->take_event();
            cudaEventRecord(a, c->stream);
        }
    }
    ~stage_scope() {
        if (a) {
            cudaEvent_t b = c->take_event();
            cudaEventRecord(b, c->stream);
            c->pending.push_back({stage, a, b});
        }
    }
};

namespace adsg {

// the context's heat RHS (the plain view) and ADS solve, for the entry points
// outside adsg_capi.cu
int ctx_rhs(adsg_ctx* c, const double* u, double* rhs, double dt);
int ctx_solve(adsg_ctx* c, double* x, int trans);

}  // namespace adsg

#endif
