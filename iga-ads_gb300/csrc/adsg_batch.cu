// Batched engine: many independent heat simulations of uneven sizes and
// degrees advanced together, by one of two engines chosen at creation by
// timing both on the batch itself:
//  - persistent: ONE cooperative launch per run of steps (all stages of all
//    instances as one sequence of work items taken from a counter, each
//    instance's stages ordered by per-instance completion counts), replayed
//    from a CUDA graph, its grid size autotuned;
//  - concurrent: every instance has a plain context (its own tuned kernels:
//    two-ended sweeps, pair sums, row-scaled step) on its own stream, and one
//    step of all instances is a CUDA graph of independent per-instance
//    chains forked from and joined to the batch stream, so the hardware runs
//    the instances side by side.
// The reference has no batched form: its unit of work is one simulation
// object driven by simulation_base::run (src/ads/simulation/simulation_base.cpp:11-20).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <new>
#include <vector>

#include "adsg_internal.hpp"
#include "adsg_kernels.cuh"

using namespace adsg;

namespace {

struct arena {
    std::vector<void*> blocks;
    ~arena() {
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

}  // namespace

struct adsg_batch {
    int count = 0;
    std::vector<dim_host> dims;
    std::vector<batch_inst> inst;  // host copies (device pointers inside)
    std::vector<double> dt;
    batch_dev B;
    arena mem;
    cudaStream_t stream = nullptr;
    int par = 0;            // which buffer holds the state
    int blocks_per_sm = 1;  // autotuned
    int order = 0;          // autotuned: 0 stage-major, 1 wavefront over instance groups (pair_order)
    int sms = 0;
    cudaGraphExec_t graph = nullptr;
    int graph_steps = -1, graph_par = -1;
    bool graph_ok = true;
    int engine = 0;                    // 0 persistent kernel, 1 concurrent per-instance graph
    std::vector<adsg_ctx*> ctxs;       // plain per-instance contexts (own streams)
    std::vector<cudaEvent_t> events;   // fork/join and chaining events, one per instance + 1
    cudaGraphExec_t step_graph[2] = {nullptr, nullptr};  // one concurrent step from parity 0 / 1

    ~adsg_batch() {
        if (stream) cudaStreamSynchronize(stream);
        for (auto* c : ctxs) adsg_ctx_destroy(c);
        for (auto g : step_graph)
            if (g) cudaGraphExecDestroy(g);
        for (auto e : events) cudaEventDestroy(e);
        if (graph) cudaGraphExecDestroy(graph);
        if (stream) cudaStreamDestroy(stream);
    }
};

#define ADSG_BATCH_TRY(expr, where)                         \
    do {                                                    \
        cudaError_t e_ = (expr);                            \
        if (e_ != cudaSuccess) return fail_cuda(e_, where); \
    } while (0)

namespace {

// Bytes of the L2 that one dof of a wavefront group may take: up to six
// groups are in flight (one per stage), each with about three live tensors.
constexpr long long kWavefrontBytesPerDof = 6 * 3 * 8;

// The order in which one step's (stage, instance) pairs are handed out
// (entries stage * count + instance).  0, stage-major: every instance's stage
// 0, then every instance's stage 1, and so on; all instances' tensors are live
// at once.  1, wavefront: the instances in consecutive groups of at most
// group_dofs dofs (an instance above that is a group of its own), group g
// running stage w - g in wave w, the groups further along first within a wave,
// so that only the groups of six consecutive waves hold live tensors.  In both
// a pair comes after the pair it waits for (the same instance's stage before,
// or the last stage of the step before), which is all the kernel's waits need;
// the items compute the same outputs in either order.
std::vector<int> pair_order(const std::vector<batch_inst>& inst, int wavefront, long long group_dofs) {
    const int count = static_cast<int>(inst.size());
    std::vector<int> order;
    order.reserve(6 * static_cast<size_t>(count));
    if (!wavefront) {
        for (int k = 0; k < 6 * count; ++k) order.push_back(k);
        return order;
    }
    std::vector<std::vector<int>> groups;
    long long acc = 0;
    for (int i = 0; i < count; ++i) {
        if (groups.empty() || (acc > 0 && acc + inst[i].size > group_dofs)) {
            groups.emplace_back();
            acc = 0;
        }
        groups.back().push_back(i);
        acc += inst[i].size;
    }
    const int G = static_cast<int>(groups.size());
    for (int w = 0; w < G + 5; ++w)
        for (int g = std::max(0, w - 5); g <= std::min(G - 1, w); ++g)
            for (int i : groups[g]) order.push_back((w - g) * count + i);
    return order;
}

int launch_steps(adsg_batch* b, int nsteps, int blocks_per_sm) {
    // completion counts and the work counter start at zero in every launch
    cudaError_t e = cudaMemsetAsync(b->B.done, 0, sizeof(unsigned) * 6 * b->count, b->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->B.next, 0, sizeof(unsigned long long), b->stream);
    if (e != cudaSuccess) return fail_cuda(e, "reset the work counters");
    void* args[] = {&b->B, &nsteps, &b->par};
    const dim3 grid(b->sms * blocks_per_sm), block(256);
    e = cudaLaunchCooperativeKernel(batch_kernel_symbol(), grid, block, args, batch_smem_bytes(), b->stream);
    if (e != cudaSuccess) return fail_cuda(e, "cooperative launch");
    return 0;
}

int check_error_word(adsg_batch* b) {
    int err = 0;
    cudaError_t e = cudaMemcpyAsync(&err, b->B.err, sizeof(int), cudaMemcpyDeviceToHost, b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) return fail_cuda(e, "batch synchronize");
    if (err) {
        cudaMemsetAsync(b->B.err, 0, sizeof(int), b->stream);
        cudaStreamSynchronize(b->stream);
        return fail(ADSG_ERR_DEVICE, "a wait of the batched kernel timed out");
    }
    return 0;
}

// Per-instance contexts on their own streams, and the events that fork,
// join or chain their work.
int ensure_contexts(adsg_batch* b) {
    if (!b->ctxs.empty()) return 0;
    b->ctxs.assign(b->count, nullptr);
    for (int i = 0; i < b->count; ++i) {
        const dim_host& h = b->dims[i];
        adsg_dim_desc d{};
        d.p = h.p;
        d.elements = h.elements;
        d.quad_order = h.q;
        d.n = h.n;
        d.btab = h.btab.data();
        d.w = h.w.data();
        d.J = h.J.data();
        d.first_dofs = h.first_dofs.data();
        d.kl = h.kl;
        d.ku = h.ku;
        d.ldab = h.ldab;
        d.lu = h.lu.data();
        d.ipiv = h.ipiv.data();
        const adsg_dim_desc descs[3] = {d, d, d};
        if (int st = adsg_ctx_create(b->inst[i].ndim, descs, &b->ctxs[i])) {
            b->ctxs[i] = nullptr;
            return st;
        }
    }
    while (b->events.size() < static_cast<size_t>(b->count) + 1) {
        cudaEvent_t e = nullptr;
        ADSG_BATCH_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event");
        b->events.push_back(e);
    }
    return 0;
}

// One step of every instance from parity par on its own context's stream:
// fork from the batch stream, join back into it.
int enqueue_concurrent_step(adsg_batch* b, int par) {
    cudaEvent_t fork = b->events[b->count];
    ADSG_BATCH_TRY(cudaEventRecord(fork, b->stream), "event");
    for (int i = 0; i < b->count; ++i) {
        cudaStream_t s = ctx_stream(b->ctxs[i]);
        ADSG_BATCH_TRY(cudaStreamWaitEvent(s, fork, 0), "fork");
        if (int st = adsg_heat_step(b->ctxs[i], b->inst[i].buf[par], b->inst[i].buf[par ^ 1], b->dt[i])) return st;
        ADSG_BATCH_TRY(cudaEventRecord(b->events[i], s), "event");
        ADSG_BATCH_TRY(cudaStreamWaitEvent(b->stream, b->events[i], 0), "join");
    }
    return 0;
}

int concurrent_steps(adsg_batch* b, int nsteps) {
    for (int s = 0; s < nsteps; ++s) {
        const int par = b->par;
        if (!b->step_graph[par]) {
            // prime each context's dt bands outside the capture
            for (int i = 0; i < b->count; ++i)
                if (int st = ctx_prepare_dt(b->ctxs[i], b->dt[i])) return st;
            cudaGraph_t g = nullptr;
            ADSG_BATCH_TRY(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
            const int st = enqueue_concurrent_step(b, par);
            const cudaError_t ec = cudaStreamEndCapture(b->stream, &g);
            if (st) {
                if (g) cudaGraphDestroy(g);
                return st;
            }
            if (ec != cudaSuccess) return fail_cuda(ec, "end capture");
            const cudaError_t ei = cudaGraphInstantiate(&b->step_graph[par], g, 0);
            cudaGraphDestroy(g);
            if (ei != cudaSuccess) {
                b->step_graph[par] = nullptr;
                return fail_cuda(ei, "graph instantiate");
            }
        }
        ADSG_BATCH_TRY(cudaGraphLaunch(b->step_graph[par], b->stream), "graph launch");
        b->par ^= 1;
    }
    return 0;
}

}  // namespace

extern "C" {

int adsg_batch_create(int count, const int* ndim, const int* p, const int* elements, const double* dt,
                      adsg_batch** out) {
    if (count < 1) return fail(-1, "count must be >= 1");
    if (!ndim) return fail(-2, "ndim is NULL");
    if (!p) return fail(-3, "p is NULL");
    if (!elements) return fail(-4, "elements is NULL");
    if (!dt) return fail(-5, "dt is NULL");
    if (!out) return fail(-6, "out is NULL");
    *out = nullptr;
    for (int i = 0; i < count; ++i) {
        if (ndim[i] != 2 && ndim[i] != 3) return fail(-2, "batched instances are 2D or 3D");
        if (p[i] < 1 || p[i] > 4) return fail(-3, "batched instances need 1 <= p <= 4");
        if (elements[i] < 1) return fail(-4, "elements must be >= 1");
        if (!std::isfinite(dt[i])) return fail(-5, "dt must be finite");
    }
    auto* b = new (std::nothrow) adsg_batch;
    if (!b) return fail(ADSG_ERR_NOMEM, "host allocation failed");
    b->count = count;
    b->dims.resize(count);
    b->inst.resize(count);
    b->dt.assign(dt, dt + count);
    auto bail = [&](int code) {
        delete b;
        return code;
    };
    cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamDefault);
    if (e != cudaSuccess) return bail(fail_cuda(e, "stream"));
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev);
    int coop = 0;
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
    if (!coop) return bail(fail(ADSG_ERR_UNSUPPORTED, "device lacks cooperative launch"));

    if ((e = batch_prepare_kernel()) != cudaSuccess) return bail(fail_cuda(e, "batched kernel shared memory"));
    for (int i = 0; i < count; ++i) {
        dim_host& h = b->dims[i];
        if (!build_dimension(h, p[i], elements[i], 0.0, 1.0, p[i] + 1))
            return bail(fail(ADSG_ERR_SINGULAR, "dimension set-up failed"));
        adsg_dim_desc d{};
        d.p = h.p;
        d.elements = h.elements;
        d.quad_order = h.q;
        d.n = h.n;
        d.btab = h.btab.data();
        d.w = h.w.data();
        d.J = h.J.data();
        d.first_dofs = h.first_dofs.data();
        d.kl = h.kl;
        d.ku = h.ku;
        d.ldab = h.ldab;
        d.lu = h.lu.data();
        d.ipiv = h.ipiv.data();
        solve_tables t;
        if (make_solve_tables(h.n, h.kl, h.ku, h.ldab, h.lu.data(), h.ipiv.data(), t))
            return bail(fail(ADSG_ERR_SINGULAR, "zero pivot"));
        std::vector<double> m = row_band(d, 0), k = row_band(d, 1);
        batch_inst& I = b->inst[i];
        int sym_lo = 0, sym_hi = 0;
        symmetric_row_range(m, k, h.n, h.p, sym_lo, sym_hi);
        // two-ended unit-diagonal sweeps where the band allows them: the rows
        // of every band are pre-multiplied by 1 / U(r, r) of the sweep
        // (symmetric rows stay symmetric), as in a context's step view
        twisted_tables tw, tu;
        std::vector<double> scale;
        I.twisted = make_twisted_tables(h.n, h.kl, h.ku, h.ldab, h.lu.data(), h.ipiv.data(), tw) == 0 ? 1 : 0;
        if (I.twisted) {
            scale_twisted(tw, h.n, tu, scale);
            const int bw = 2 * h.p + 1;
            for (int r = 0; r < h.n; ++r)
                for (int c = 0; c < bw; ++c) {
                    m[static_cast<size_t>(r) * bw + c] *= scale[r];
                    k[static_cast<size_t>(r) * bw + c] *= scale[r];
                }
        }
        std::vector<double> nr(m.size()), kd(m.size());
        for (size_t q = 0; q < m.size(); ++q) {
            nr[q] = std::fma(-dt[i], k[q], m[q]);
            kd[q] = -dt[i] * k[q];
        }
        I.ndim = ndim[i];
        I.p = p[i];
        I.n = h.n;
        I.size = ndim[i] == 3 ? static_cast<long long>(h.n) * h.n * h.n : static_cast<long long>(h.n) * h.n;
        dim_dev& D = I.dim;
        D.n = h.n;
        D.p = h.p;
        D.kl = t.kl;
        D.w = t.w;
        D.ku_regular = h.ku;
        D.fwd_fast = t.fwd_fast;
        D.bwd_fast = t.bwd_fast;
        D.elements = h.elements;
        D.q = h.q;
        D.sym_lo = sym_lo;
        D.sym_hi = sym_hi;
        double *mrow, *krow, *nrow, *kdt, *lmul, *ucol, *rdiag;
        double *tw_l = nullptr, *tw_u = nullptr, *tw_r = nullptr, *tw_g = nullptr;
        int *piv, *uext;
        arena& A = b->mem;
        cudaStream_t s = b->stream;
        e = A.upload(&mrow, m.data(), m.size(), s);
        if (e == cudaSuccess) e = A.upload(&krow, k.data(), k.size(), s);
        if (e == cudaSuccess) e = A.upload(&nrow, nr.data(), nr.size(), s);
        if (e == cudaSuccess) e = A.upload(&kdt, kd.data(), kd.size(), s);
        if (e == cudaSuccess) e = A.upload(&lmul, t.lmul.data(), t.lmul.size(), s);
        if (e == cudaSuccess) e = A.upload(&ucol, t.ucol.data(), t.ucol.size(), s);
        if (e == cudaSuccess) e = A.upload(&rdiag, t.rdiag.data(), t.rdiag.size(), s);
        if (e == cudaSuccess) e = A.upload(&piv, t.piv.data(), t.piv.size(), s);
        if (e == cudaSuccess) e = A.upload(&uext, t.uext.data(), t.uext.size(), s);
        if (I.twisted) {
            if (e == cudaSuccess) e = A.upload(&tw_l, tu.lmul.data(), tu.lmul.size(), s);
            if (e == cudaSuccess) e = A.upload(&tw_u, tu.ucol.data(), tu.ucol.size(), s);
            if (e == cudaSuccess) e = A.upload(&tw_r, tu.rdiag.data(), tu.rdiag.size(), s);
            if (e == cudaSuccess) e = A.upload(&tw_g, tu.g.data(), tu.g.size(), s);
        }
        if (e == cudaSuccess) e = A.alloc(&I.buf[0], I.size);
        if (e == cudaSuccess) e = A.alloc(&I.buf[1], I.size);
        for (int q = 0; q < (ndim[i] == 3 ? 4 : 2) && e == cudaSuccess; ++q) e = A.alloc(&I.T[q], I.size);
        if (e == cudaSuccess) e = cudaMemsetAsync(I.buf[0], 0, sizeof(double) * I.size, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);  // host staging above dies with this iteration
        if (e != cudaSuccess) return bail(fail_cuda(e, "batch set-up"));
        D.mrow = mrow;
        D.krow = krow;
        D.nrow = nrow;
        D.kdt = kdt;
        D.lmul = lmul;
        D.ucol = ucol;
        D.rdiag = rdiag;
        D.piv = piv;
        D.uext = uext;
        if (I.twisted) {
            D.tw_k = tu.k;
            D.tw_n1 = tu.n1;
            D.tw_n2 = tu.n2;
            D.tw_rows = tu.rows;
            D.tw_unit = 1;
            D.tw_lmul = tw_l;
            D.tw_ucol = tw_u;
            D.tw_rdiag = tw_r;
            D.tw_g = tw_g;
        }
        const long long lines = I.size / I.n;
        if (I.ndim == 3) {
            const long long u[6] = {I.size, I.size, I.size, lines, lines, lines};
            std::copy(u, u + 6, I.units);
        } else {
            const long long u[6] = {I.size, 0, I.size, lines, lines, 0};
            std::copy(u, u + 6, I.units);
        }
    }
    for (int st = 0; st < 6; ++st)
        for (int i = 0; i < count; ++i) {
            batch_inst& I = b->inst[i];
            const long long per = batch_units_per_item(st, I.twisted);
            I.items[st] = static_cast<int>((I.units[st] + per - 1) / per);
        }
    // the two orders of a step's pairs, and their item prefixes
    int l2 = 0;
    cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev);
    std::vector<int> order[2];
    std::vector<long long> prefix[2];
    for (int o = 0; o < 2; ++o) {
        order[o] = pair_order(b->inst, o, std::max(1LL, static_cast<long long>(l2) / kWavefrontBytesPerDof));
        prefix[o].assign(order[o].size() + 1, 0);
        for (size_t k = 0; k < order[o].size(); ++k) {
            const int st = order[o][k] / count, i = order[o][k] % count;
            prefix[o][k + 1] = prefix[o][k] + b->inst[i].items[st];
        }
    }
    batch_inst* dinst = nullptr;
    int* dorder[2] = {nullptr, nullptr};
    long long* dprefix[2] = {nullptr, nullptr};
    unsigned* done = nullptr;
    unsigned long long* next = nullptr;
    int* err = nullptr;
    e = b->mem.upload(&dinst, b->inst.data(), b->inst.size(), b->stream);
    for (int o = 0; o < 2; ++o) {
        if (e == cudaSuccess) e = b->mem.upload(&dorder[o], order[o].data(), order[o].size(), b->stream);
        if (e == cudaSuccess) e = b->mem.upload(&dprefix[o], prefix[o].data(), prefix[o].size(), b->stream);
    }
    if (e == cudaSuccess) e = b->mem.alloc(&done, 6 * static_cast<size_t>(count));
    if (e == cudaSuccess) e = b->mem.alloc(&next, 1);
    if (e == cudaSuccess) e = b->mem.alloc(&err, 1);
    if (e == cudaSuccess) e = cudaMemsetAsync(err, 0, sizeof(int), b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) return bail(fail_cuda(e, "batch set-up"));
    b->B.count = count;
    b->B.inst = dinst;
    b->B.per_step = prefix[0].back();  // the same items in either order
    b->B.done = done;
    b->B.next = next;
    b->B.err = err;
    auto use_order = [&](int o) {
        b->order = o;
        b->B.pair = dorder[o];
        b->B.prefix = dprefix[o];
    };

    // autotune the persistent grid and the order on the zero state (the state
    // is reset after); ADSG_BATCH_ORDER=0/1 forces the order
    const int maxb = std::max(1, batch_max_blocks_per_sm());
    const char* fo = std::getenv("ADSG_BATCH_ORDER");
    const int forced_order = fo && (*fo == '0' || *fo == '1') ? *fo - '0' : -1;
    cudaEvent_t t0, t1;
    cudaEventCreate(&t0);
    cudaEventCreate(&t1);
    float best = 1e30f;
    int best_order = forced_order >= 0 ? forced_order : 0;
    for (int o = 0; o < 2; ++o) {
        if (forced_order >= 0 && o != forced_order) continue;
        use_order(o);
        for (int bps = 1; bps <= maxb; ++bps) {
            int st = launch_steps(b, 1, bps);  // warm-up
            if (st) break;
            cudaEventRecord(t0, b->stream);
            st = launch_steps(b, 2, bps);
            cudaEventRecord(t1, b->stream);
            if (st || cudaEventSynchronize(t1) != cudaSuccess) break;
            float ms = 0.f;
            cudaEventElapsedTime(&ms, t0, t1);
            if (ms < best) {
                best = ms;
                b->blocks_per_sm = bps;
                best_order = o;
            }
        }
    }
    use_order(best_order);
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    if (int st = check_error_word(b)) return bail(st);
    for (int i = 0; i < count; ++i) {
        cudaMemsetAsync(b->inst[i].buf[0], 0, sizeof(double) * b->inst[i].size, b->stream);
        cudaMemsetAsync(b->inst[i].buf[1], 0, sizeof(double) * b->inst[i].size, b->stream);
    }
    b->par = 0;
    if ((e = cudaStreamSynchronize(b->stream)) != cudaSuccess) return bail(fail_cuda(e, "batch set-up"));
    // engine: the persistent kernel (best grid above) against the concurrent
    // per-instance graph, timed on the zero state
    {
        const char* force = std::getenv("ADSG_BATCH_ENGINE");
        if (force && (*force == '0' || *force == '1')) {
            b->engine = *force - '0';
        } else if (ensure_contexts(b) == 0) {
            cudaEventCreate(&t0);
            cudaEventCreate(&t1);
            // the faster of two timings of six steps each, after a warm-up:
            // the engines can be within a few percent of each other, and the
            // persistent launch's fixed cost spreads over the steps of a call
            float tp = 1e30f, tc = 1e30f;
            for (int eng = 0; eng < 2; ++eng) {
                auto run = [&]() { return eng == 0 ? launch_steps(b, 6, b->blocks_per_sm) : concurrent_steps(b, 6); };
                if (run() != 0) continue;  // warm-up (the concurrent one builds both graphs)
                for (int rep = 0; rep < 2; ++rep) {
                    cudaEventRecord(t0, b->stream);
                    if (run() != 0) break;
                    cudaEventRecord(t1, b->stream);
                    float ms = 1e30f;
                    if (cudaEventSynchronize(t1) == cudaSuccess) cudaEventElapsedTime(&ms, t0, t1);
                    float& t = eng == 0 ? tp : tc;
                    t = std::min(t, ms);
                }
            }
            cudaEventDestroy(t0);
            cudaEventDestroy(t1);
            cudaGetLastError();
            b->engine = tc < tp ? 1 : 0;
            if (int st = check_error_word(b)) return bail(st);
            for (int i = 0; i < count; ++i) {
                cudaMemsetAsync(b->inst[i].buf[0], 0, sizeof(double) * b->inst[i].size, b->stream);
                cudaMemsetAsync(b->inst[i].buf[1], 0, sizeof(double) * b->inst[i].size, b->stream);
            }
            b->par = 0;
            if ((e = cudaStreamSynchronize(b->stream)) != cudaSuccess) return bail(fail_cuda(e, "batch set-up"));
        }
        cudaGetLastError();
    }
    *out = b;
    return 0;
}

int adsg_batch_destroy(adsg_batch* b) {
    delete b;
    return 0;
}

long long adsg_batch_dofs(const adsg_batch* b, int i) {
    if (!b || i < 0 || i >= b->count) return -1;
    return b->inst[i].size;
}

int adsg_batch_set_state(adsg_batch* b, int i, const double* u_host) {
    if (!b) return fail(-1, "batch is NULL");
    if (i < 0 || i >= b->count) return fail(-2, "instance index out of range");
    if (!u_host) return fail(-3, "u is NULL");
    cudaError_t e = cudaMemcpyAsync(b->inst[i].buf[b->par], u_host, sizeof(double) * b->inst[i].size,
                                    cudaMemcpyHostToDevice, b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    return e == cudaSuccess ? 0 : fail_cuda(e, "set state");
}

int adsg_batch_get_state(adsg_batch* b, int i, double* u_host) {
    if (!b) return fail(-1, "batch is NULL");
    if (i < 0 || i >= b->count) return fail(-2, "instance index out of range");
    if (!u_host) return fail(-3, "u is NULL");
    cudaError_t e = cudaMemcpyAsync(u_host, b->inst[i].buf[b->par], sizeof(double) * b->inst[i].size,
                                    cudaMemcpyDeviceToHost, b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    return e == cudaSuccess ? 0 : fail_cuda(e, "get state");
}

int adsg_batch_steps(adsg_batch* b, int nsteps) {
    if (!b) return fail(-1, "batch is NULL");
    if (nsteps < 0) return fail(-2, "nsteps must be >= 0");
    if (nsteps == 0) return 0;
    if (b->engine == 1) {
        if (int st = ensure_contexts(b)) return st;
        return concurrent_steps(b, nsteps);
    }
    if (b->graph_ok && !(b->graph && b->graph_steps == nsteps && b->graph_par == b->par)) {
        if (b->graph) {
            cudaGraphExecDestroy(b->graph);
            b->graph = nullptr;
        }
        cudaGraph_t g = nullptr;
        if (cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
            const int st = launch_steps(b, nsteps, b->blocks_per_sm);
            const cudaError_t ec = cudaStreamEndCapture(b->stream, &g);
            if (st == 0 && ec == cudaSuccess && g && cudaGraphInstantiate(&b->graph, g, 0) == cudaSuccess) {
                b->graph_steps = nsteps;
                b->graph_par = b->par;
            } else {
                b->graph = nullptr;
                b->graph_ok = false;  // fall back to direct cooperative launches
            }
            if (g) cudaGraphDestroy(g);
        } else {
            b->graph_ok = false;
        }
        cudaGetLastError();
    }
    if (b->graph) {
        cudaError_t e = cudaGraphLaunch(b->graph, b->stream);
        if (e != cudaSuccess) return fail_cuda(e, "graph launch");
    } else {
        if (int st = launch_steps(b, nsteps, b->blocks_per_sm)) return st;
    }
    b->par ^= (nsteps & 1);
    return 0;
}

int adsg_batch_steps_looped(adsg_batch* b, int nsteps) {
    if (!b) return fail(-1, "batch is NULL");
    if (nsteps < 0) return fail(-2, "nsteps must be >= 0");
    if (int st = ensure_contexts(b)) return st;
    // one instance after the other: each context's stream waits for the
    // previous instance (or the batch stream), the batch stream for the last
    for (int s = 0; s < nsteps; ++s) {
        cudaEvent_t prev = b->events[b->count];
        ADSG_BATCH_TRY(cudaEventRecord(prev, b->stream), "event");
        for (int i = 0; i < b->count; ++i) {
            cudaStream_t st_i = ctx_stream(b->ctxs[i]);
            ADSG_BATCH_TRY(cudaStreamWaitEvent(st_i, prev, 0), "chain");
            double* cur = b->inst[i].buf[b->par];
            double* nxt = b->inst[i].buf[b->par ^ 1];
            if (int st = adsg_heat_step(b->ctxs[i], cur, nxt, b->dt[i])) return st;
            ADSG_BATCH_TRY(cudaEventRecord(b->events[i], st_i), "event");
            prev = b->events[i];
        }
        ADSG_BATCH_TRY(cudaStreamWaitEvent(b->stream, prev, 0), "chain");
        b->par ^= 1;
    }
    return 0;
}

int adsg_batch_synchronize(adsg_batch* b) {
    if (!b) return fail(-1, "batch is NULL");
    return check_error_word(b);
}

int adsg_batch_tuning(const adsg_batch* b, int* blocks_per_sm, int* graph_captured) {
    if (!b) return fail(-1, "batch is NULL");
    if (blocks_per_sm) *blocks_per_sm = b->blocks_per_sm;
    if (graph_captured) *graph_captured = b->graph || b->step_graph[0] || b->step_graph[1] ? 1 : 0;
    return 0;
}

int adsg_batch_engine(const adsg_batch* b) { return b ? b->engine : -1; }

int adsg_batch_order(const adsg_batch* b) { return b ? b->order : -1; }

int adsg_batch_test_waits(adsg_batch* b, int extra_items, long long spin_limit) {
    if (!b) return fail(-1, "batch is NULL");
    if (extra_items < 0) return fail(-2, "extra_items < 0");
    if (spin_limit < 1) return fail(-3, "spin_limit < 1");
    if (b->stream) {
        cudaError_t e = cudaStreamSynchronize(b->stream);
        if (e != cudaSuccess) return fail_cuda(e, "batch synchronize");
    }
    // the launch arguments are baked into a captured graph: drop it
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    b->graph_steps = b->graph_par = -1;
    b->B.wait_extra = static_cast<unsigned>(extra_items);
    b->B.spin_limit = spin_limit;
    return 0;
}

}  // extern "C"
