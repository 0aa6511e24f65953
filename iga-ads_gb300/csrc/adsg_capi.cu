// C-ABI of the engine: contexts, device tables, the heat RHS, the ADS solve,
// the graph-replayed step loop and the LAPACK-compatible dgbtrs_.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "adsg_internal.hpp"
#include "adsg_kernels.cuh"

namespace adsg {

static thread_local std::string g_last_error = "no error";

int fail(int code, const char* msg) {
    g_last_error = msg;
    return code;
}

int fail_cuda(int err, const char* where) {
    g_last_error = std::string(where) + ": " + cudaGetErrorString(static_cast<cudaError_t>(err));
    return err == cudaErrorMemoryAllocation ? ADSG_ERR_NOMEM : ADSG_ERR_CUDA;
}

// Allocation-failure hook: the k-th device allocation from now fails (k >= 0,
// counted across threads), then the hook turns itself off; -1 = off.
std::atomic<int> g_alloc_fail_in{-1};

cudaError_t device_alloc(void** p, size_t bytes) {
    int k = g_alloc_fail_in.load();
    while (k >= 0 && !g_alloc_fail_in.compare_exchange_weak(k, k - 1)) {
    }
    if (k == 0) {
        *p = nullptr;
        return cudaErrorMemoryAllocation;
    }
    return cudaMalloc(p, bytes);
}

}  // namespace adsg

using namespace adsg;

#include "adsg_check.cuh"
#include "adsg_context.cuh"

namespace {

int ensure_dt_bands(adsg_ctx* c, double dt) {
    if (c->band_dt == dt) return 0;
    for (int d = 0; d < c->ndim; ++d) {
        ADSG_CUDA_TRY(launch_dt_bands(c->dims[d], dt, c->nrow[d], c->kdt[d], c->stream), "dt bands");
        c->dims[d].nrow = c->nrow[d];
        c->dims[d].kdt = c->kdt[d];
        if (c->snrow[d]) {
            ADSG_CUDA_TRY(launch_dt_bands(c->sdims[d], dt, c->snrow[d], c->skdt[d], c->stream), "dt bands");
            c->sdims[d].nrow = c->snrow[d];
            c->sdims[d].kdt = c->skdt[d];
        } else {
            c->sdims[d].nrow = c->nrow[d];
            c->sdims[d].kdt = c->kdt[d];
        }
    }
    c->band_dt = dt;
    return 0;
}

// rhs = (M(x)M(x)M - dt (K(x)M(x)M + M(x)K(x)M + M(x)M(x)K)) u_prev as a sequence of
// band passes along z, y, x (3D), y, x (2D) or x (1D).
// fused_x: the x pass is issued fused with the x solve (rhs then holds the
// x-solved right-hand side); the caller checks fusion_ok first.
// outer_done: the first (outermost-axis) pass has already been issued into
// scratch[0..1] (the host entry overlaps it with the upload).
int enqueue_rhs_with(adsg_ctx* c, const dim_dev* D, const double* u, double* rhs, double dt, bool fused_x = false,
                     bool outer_done = false) {
    pdl_scope pdl(c->pdl);
    int st = ensure_dt_bands(c, dt);
    if (st) return st;
    const long long total = c->size;
    cudaStream_t s = c->stream;
    double** T = c->scratch;
    const line_layout Lx = make_line_layout(c->n, c->ndim, 0);
    // the last pass, along x: out = A0 (.) in0 [+ A1 (.) in1]
    auto x_pass = [&](const double* in0, const double* in1, const double* A0, const double* A1) -> int {
        if (fused_x) {
            stage_scope sc(c, ADSG_STAGE_RHS_SOLVE_X);
            ADSG_CUDA_TRY(launch_rhs_x_solve(in0, in1, rhs, A0, A1, D[0], Lx, s), "rhs pass x + x solve");
            return 0;
        }
        stage_scope sc(c, ADSG_STAGE_RHS_X);
        ADSG_CUDA_TRY(launch_band_pass(D[0].p, in0, in1, rhs, nullptr, A0, A1, nullptr, D[0].n, 1, total, s),
                      "rhs pass x");
        return 0;
    };
    if (c->ndim == 1) {
        if (int st2 = x_pass(u, nullptr, D[0].nrow, nullptr)) return st2;
    } else if (c->ndim == 2) {
        const long long sy = c->n[0];
        // A = My u, C = Ny u
        if (!outer_done) {
            stage_scope s1(c, ADSG_STAGE_RHS_OUTER);
            ADSG_CUDA_TRY(launch_band_pass(D[1].p, u, nullptr, T[0], T[1], D[1].mrow, nullptr, D[1].nrow, D[1].n, sy,
                                           total, s, D[1].sym_lo, D[1].sym_hi),
                          "rhs pass y");
        }
        // rhs = (-dt Kx) A + Mx C
        if (int st2 = x_pass(T[0], T[1], D[0].kdt, D[0].mrow)) return st2;
    } else {
        const long long sy = c->n[0], sz = static_cast<long long>(c->n[0]) * c->n[1];
        // A = Mz u, C = Nz u
        if (!outer_done) {
            stage_scope s1(c, ADSG_STAGE_RHS_OUTER);
            ADSG_CUDA_TRY(launch_band_pass(D[2].p, u, nullptr, T[0], T[1], D[2].mrow, nullptr, D[2].nrow, D[2].n, sz,
                                           total, s, D[2].sym_lo, D[2].sym_hi),
                          "rhs pass z");
        }
        // F = (-dt Ky) A + My C,  G = My A
        { stage_scope s2(c, ADSG_STAGE_RHS_MIDDLE);
        ADSG_CUDA_TRY(launch_band_pass(D[1].p, T[0], T[1], T[2], T[3], D[1].kdt, D[1].mrow, D[1].mrow, D[1].n, sy,
                                       total, s, D[1].sym_lo, D[1].sym_hi),
                      "rhs pass y"); }
        // rhs = (-dt Kx) G + Mx F
        if (int st2 = x_pass(T[3], T[2], D[0].kdt, D[0].mrow)) return st2;
    }
    return 0;
}

int enqueue_rhs(adsg_ctx* c, const double* u, double* rhs, double dt) { return enqueue_rhs_with(c, c->dims, u, rhs, dt); }

int enqueue_solve_with(adsg_ctx* c, const dim_dev* D, double* x, int trans, int first_dim = 0, int end_dim = 3) {
    pdl_scope pdl(c->pdl);
    for (int d = first_dim; d < c->ndim && d < end_dim; ++d) {
        line_layout L = make_line_layout(c->n, c->ndim, d);
        stage_scope sc(c, ADSG_STAGE_SOLVE_X + d);
        ADSG_CUDA_TRY(launch_line_solve(x, D[d], L, trans, c->stream), "line solve");
    }
    return 0;
}

int enqueue_solve(adsg_ctx* c, double* x, int trans) { return enqueue_solve_with(c, c->dims, x, trans); }

// The explicit step's solves (the step's own view, sdims).  After the fused x
// pass + x solve: y, then z.  Otherwise the outer directions first and x
// last, so that the last sweep runs over contiguous lines and its tile can
// be written anywhere: into `out` when given (e.g. the caller's pinned
// buffer, mapped), in place otherwise.  The order differs from ads_solve's
// x, y, z only by rounding (the directions' inverses commute).
bool step_x_out_ok(const adsg_ctx* c) {
    return line_solve_out_ok(c->sdims[0], make_line_layout(c->n, c->ndim, 0));
}

int enqueue_step_solves(adsg_ctx* c, double* x, bool fused, double* out = nullptr) {
    if (fused) return enqueue_solve_with(c, c->sdims, x, 0, 1);
    pdl_scope pdl(c->pdl);
    for (int d = c->ndim - 1; d >= 0; --d) {
        const line_layout L = make_line_layout(c->n, c->ndim, d);
        stage_scope sc(c, ADSG_STAGE_SOLVE_X + d);
        if (d == 0 && out && out != x) {
            ADSG_CUDA_TRY(launch_line_solve_out(x, out, c->sdims[0], L, c->stream), "line solve (to output)");
        } else {
            ADSG_CUDA_TRY(launch_line_solve(x, c->sdims[d], L, 0, c->stream), "line solve");
        }
    }
    return 0;
}

std::mutex g_autotune_lock;
std::map<std::string, int> g_autotune_cache;

// Device time of three line solves of direction D on the context's state
// buffer, after one warm-up launch; a launch error is returned.
cudaError_t time_line_solve(adsg_ctx* c, const dim_dev& D, const line_layout& L, cudaEvent_t a, cudaEvent_t b,
                            float* ms) {
    cudaGetLastError();
    cudaError_t e = launch_line_solve(c->ping, D, L, 0, c->stream);
    if (e == cudaSuccess) e = cudaEventRecord(a, c->stream);
    for (int r = 0; r < 3 && e == cudaSuccess; ++r) e = launch_line_solve(c->ping, D, L, 0, c->stream);
    if (e == cudaSuccess) e = cudaEventRecord(b, c->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(b);
    if (e == cudaSuccess) e = cudaEventElapsedTime(ms, a, b);
    return e;
}

std::string autotune_key(const adsg_ctx* c, int d) {
    const dim_dev& D = c->dims[d];
    int dev = 0;
    cudaGetDevice(&dev);
    char key[192];
    std::snprintf(key, sizeof key, "%d|%d|%d,%d,%d|%d|%d,%d,%d,%d,%d,%d,%d", dev, c->ndim, c->n[0], c->n[1], c->n[2], d,
                  D.p, D.kl, D.w, D.ku_regular, D.fwd_fast, D.bwd_fast, D.tw_k);
    return key;
}

// Autotuner: time every applicable line-solve variant per direction on the
// context's own state buffer (zeros) and keep the fastest.  ADSG_SOLVE_VARIANT
// (0..7) forces one variant where applicable; ADSG_AUTOTUNE_LOG=1 prints each
// candidate's time to stderr.  A candidate whose launch reports an error is
// dropped (the error is cleared so that it cannot leak into the next one).
int autotune_solves(adsg_ctx* c) {
    const char* force = std::getenv("ADSG_SOLVE_VARIANT");
    int forced = -1;
    if (force && *force) forced = std::atoi(force);
    const char* logv = std::getenv("ADSG_AUTOTUNE_LOG");
    const bool log = logv && *logv && *logv != '0';
    ADSG_CUDA_TRY(cudaMemsetAsync(c->ping, 0, sizeof(double) * c->size, c->stream), "autotune memset");
    ADSG_CUDA_TRY(cudaStreamSynchronize(c->stream), "autotune memset");
    cudaEvent_t a, b;
    ADSG_CUDA_TRY(cudaEventCreate(&a), "event");
    if (cudaEventCreate(&b) != cudaSuccess) {
        cudaEventDestroy(a);
        return fail_cuda(cudaGetLastError(), "event");
    }
    int rc = 0;
    for (int d = 0; d < c->ndim && rc == 0; ++d) {
        dim_dev& D = c->dims[d];
        const line_layout L = make_line_layout(c->n, c->ndim, d);
        if (forced >= 0 && forced < SOLVE_NVARIANTS && line_solve_variant_ok(forced, D)) {
            D.solve_variant = forced;
            if (log) std::fprintf(stderr, "ads_gb300 autotune: dim %d n=%d forced variant %d\n", d, D.n, forced);
            continue;
        }
        // one decision per (device, shape, direction) and process, so that
        // contexts of the same shape run the same kernels (bitwise equal results)
        const std::string key = autotune_key(c, d);
        {
            std::lock_guard<std::mutex> g(g_autotune_lock);
            auto it = g_autotune_cache.find(key);
            if (it != g_autotune_cache.end() && line_solve_variant_ok(it->second, D)) {
                D.solve_variant = it->second;
                if (log) std::fprintf(stderr, "ads_gb300 autotune: dim %d n=%d cached variant %d\n", d, D.n, it->second);
                continue;
            }
        }
        float best = 1e30f, best_tw = 1e30f;
        int best_v = SOLVE_STAGED_1, best_twv = SOLVE_TWISTED;
        for (int v = 0; v < SOLVE_NVARIANTS; ++v) {
            if (!line_solve_variant_ok(v, D)) continue;
            D.solve_variant = v;
            float ms = 0.f;
            cudaError_t e = time_line_solve(c, D, L, a, b, &ms);
            if (e == cudaSuccess && v == SOLVE_TWISTED_BULK && bulk_wait_timeouts(1) != 0)
                e = cudaErrorLaunchTimeout;  // a copy wait ran out: not a candidate
            if (e != cudaSuccess) {
                if (log)
                    std::fprintf(stderr, "ads_gb300 autotune: dim %d n=%d variant %d dropped: %s\n", d, D.n, v,
                                 cudaGetErrorString(e));
                cudaGetLastError();
                // an error that persists (the context is unusable) ends set-up
                const cudaError_t e2 = cudaStreamSynchronize(c->stream);
                if (e2 != cudaSuccess) {
                    rc = fail_cuda(e2, "autotune");
                    break;
                }
                continue;
            }
            if (log) std::fprintf(stderr, "ads_gb300 autotune: dim %d n=%d variant %d %.2f us\n", d, D.n, v, ms * 1000.f / 3);
            if (solve_variant_twisted(v)) {
                if (ms < best_tw) {
                    best_tw = ms;
                    best_twv = v;
                }
            } else if (ms < best) {
                best = ms;
                best_v = v;
            }
        }
        // the two-ended sweep rounds differently from the LAPACK-order ones:
        // take it only for a clear gain, so that the choice does not flip
        // between runs on timing noise
        if (best_tw < 0.9f * best) best_v = best_twv;
        D.solve_variant = best_v;
        std::lock_guard<std::mutex> g(g_autotune_lock);
        g_autotune_cache[key] = best_v;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaGetLastError();
    return rc;
}

// One explicit step prev -> next through the step's own view (sdims): the
// row-scaled right-hand side, then the solves.
bool fusion_ok(const adsg_ctx* c) {
    return c->sdims[0].solve_variant == SOLVE_TWISTED_STAGED &&
           rhs_x_solve_ok(c->sdims[0], make_line_layout(c->n, c->ndim, 0));
}

bool step_1block_ok(const adsg_ctx* c) { return c->ndim == 2 && small2d_step_ok(c->sdims[0], c->sdims[1]); }

int enqueue_step(adsg_ctx* c, const double* prev, double* next, double dt) {
    int st = ensure_dt_bands(c, dt);  // before the view is read
    if (st) return st;
    if (c->step_1block && step_1block_ok(c)) {
        pdl_scope pdl(c->pdl);
        stage_scope sc(c, ADSG_STAGE_STEP_1BLOCK);
        set_small2d_cluster(c->step_cluster);
        ADSG_CUDA_TRY(launch_small2d_step(prev, next, c->sdims[0], c->sdims[1], c->stream), "one-launch step");
        return 0;
    }
    const bool fused = c->fuse_x && fusion_ok(c);
    st = enqueue_rhs_with(c, c->sdims, prev, next, dt, fused);
    if (st) return st;
    return enqueue_step_solves(c, next, fused);
}

// Builds the step's view of direction d once the solve variant of ads_solve
// is chosen.  With the two-ended tables at hand the step divides the right-hand
// side's rows by the pivots (folded into the band rows), which lets the
// two-ended sweeps skip their diagonal multiplies; where ads_solve kept a
// LAPACK-order variant, those unit-diagonal sweeps are timed against it and
// the step takes them when they are at least 5% faster.
int build_step_dim(adsg_ctx* c, int d, const adsg_dim_desc& h, const twisted_tables* tw) {
    c->sdims[d] = c->dims[d];
    if (!tw) return 0;
    const bool tw_chosen = solve_variant_twisted(c->dims[d].solve_variant);
    const char* force = std::getenv("ADSG_SOLVE_VARIANT");
    if (!tw_chosen && force && *force) return 0;  // a forced variant rules both views
    twisted_tables u;
    std::vector<double> scale;
    scale_twisted(*tw, h.n, u, scale);
    std::vector<double> m = row_band(h, 0), k = row_band(h, 1);
    const int bw = 2 * h.p + 1;
    for (int r = 0; r < h.n; ++r)
        for (int t = 0; t < bw; ++t) {
            m[static_cast<size_t>(r) * bw + t] *= scale[r];
            k[static_cast<size_t>(r) * bw + t] *= scale[r];
        }
    double *sm = nullptr, *sk = nullptr, *l = nullptr, *uc = nullptr, *rd = nullptr, *g = nullptr;
    dev_arena& A = c->arena;
    cudaStream_t s = c->stream;
    cudaError_t e = A.upload(&sm, m.data(), m.size(), s);
    if (e == cudaSuccess) e = A.upload(&sk, k.data(), k.size(), s);
    if (e == cudaSuccess) e = A.alloc(&c->snrow[d], m.size());
    if (e == cudaSuccess) e = A.alloc(&c->skdt[d], m.size());
    if (e == cudaSuccess) e = A.upload(&l, u.lmul.data(), u.lmul.size(), s);
    if (e == cudaSuccess) e = A.upload(&uc, u.ucol.data(), u.ucol.size(), s);
    if (e == cudaSuccess) e = A.upload(&rd, u.rdiag.data(), u.rdiag.size(), s);
    if (e == cudaSuccess) e = A.upload(&g, u.g.data(), u.g.size(), s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);  // the host vectors die here
    if (e != cudaSuccess) return fail_cuda(e, "step tables");
    dim_dev S = c->dims[d];
    S.mrow = sm;
    S.krow = sk;
    S.tw_lmul = l;
    S.tw_ucol = uc;
    S.tw_rdiag = rd;
    S.tw_g = g;
    S.tw_unit = 1;
    if (!tw_chosen) {
        const std::string key = autotune_key(c, d) + "|step";
        int pick = -1;
        {
            std::lock_guard<std::mutex> lk(g_autotune_lock);
            auto it = g_autotune_cache.find(key);
            if (it != g_autotune_cache.end()) pick = it->second;
        }
        if (pick < 0) {
            const char* logv = std::getenv("ADSG_AUTOTUNE_LOG");
            const bool log = logv && *logv && *logv != '0';
            const line_layout L = make_line_layout(c->n, c->ndim, d);
            cudaEvent_t a, b;
            ADSG_CUDA_TRY(cudaEventCreate(&a), "event");
            if (cudaEventCreate(&b) != cudaSuccess) {
                cudaEventDestroy(a);
                return fail_cuda(cudaGetLastError(), "event");
            }
            float plain = 1e30f, best = 1e30f;
            pick = c->dims[d].solve_variant;
            if (time_line_solve(c, c->dims[d], L, a, b, &plain) != cudaSuccess) plain = 1e30f;
            for (int v : {SOLVE_TWISTED, SOLVE_TWISTED_STAGED, SOLVE_TWISTED_CHUNKED, SOLVE_TWISTED_BULK}) {
                S.solve_variant = v;
                if (!line_solve_variant_ok(v, S)) continue;
                float ms = 0.f;
                cudaError_t te = time_line_solve(c, S, L, a, b, &ms);
                if (te == cudaSuccess && v == SOLVE_TWISTED_BULK && bulk_wait_timeouts(1) != 0)
                    te = cudaErrorLaunchTimeout;
                if (log)
                    std::fprintf(stderr, "ads_gb300 autotune: dim %d n=%d step view variant %d %s %.2f us (plain %.2f)\n",
                                 d, S.n, v, te == cudaSuccess ? "" : cudaGetErrorString(te), ms * 1000.f / 3,
                                 plain * 1000.f / 3);
                if (te != cudaSuccess) {
                    cudaGetLastError();
                    const cudaError_t e2 = cudaStreamSynchronize(c->stream);
                    if (e2 != cudaSuccess) {
                        cudaEventDestroy(a);
                        cudaEventDestroy(b);
                        return fail_cuda(e2, "step autotune");
                    }
                    continue;
                }
                if (ms < best && ms < 0.95f * plain) {
                    best = ms;
                    pick = v;
                }
            }
            cudaEventDestroy(a);
            cudaEventDestroy(b);
            cudaGetLastError();
            std::lock_guard<std::mutex> lk(g_autotune_lock);
            g_autotune_cache[key] = pick;
        }
        if (!solve_variant_twisted(pick)) {  // the plain view stays, with the plain dt bands
            c->snrow[d] = c->skdt[d] = nullptr;
            return 0;
        }
        S.solve_variant = pick;
    }
    c->sdims[d] = S;
    c->band_dt = std::nan("");  // the scaled dt bands are built on the next step
    return 0;
}

// adsg_heat_step through a cached single-step graph.  Steps issued while the
// stream is being captured (a batch recording its own graph), with stage
// timers on, or by a caller that keeps changing buffers (more misses than the
// small cache can serve) are enqueued directly.  The same kernels run either
// way, so results do not depend on the path.
constexpr size_t kStepGraphs = 4;

int step_via_graph(adsg_ctx* c, const double* prev, double* next, double dt) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(c->stream, &cs) != cudaSuccess) {
        cudaGetLastError();
        cs = cudaStreamCaptureStatusActive;  // unknown: take the direct path
    }
    const bool thrashing = c->step_graph_misses > 2 * c->step_graph_hits + 16;
    if (cs != cudaStreamCaptureStatusNone || c->timing || thrashing || !c->step_graphs_on)
        return enqueue_step(c, prev, next, dt);
    int st = ensure_dt_bands(c, dt);  // the graph reads the dt bands in place
    if (st) return st;
    auto& v = c->step_graphs;
    for (size_t i = 0; i < v.size(); ++i)
        if (v[i].prev == prev && v[i].next == next && v[i].dt == dt) {
            const adsg_ctx::step_graph g = v[i];
            v.erase(v.begin() + static_cast<long>(i));
            v.push_back(g);
            ++c->step_graph_hits;
            ADSG_CUDA_TRY(cudaGraphLaunch(g.exec, c->stream), "step graph launch");
            return 0;
        }
    ++c->step_graph_misses;
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        cudaGetLastError();
        return enqueue_step(c, prev, next, dt);
    }
    c->capturing = true;
    st = enqueue_step(c, prev, next, dt);
    c->capturing = false;
    const cudaError_t ec = cudaStreamEndCapture(c->stream, &g);
    cudaGraphExec_t exec = nullptr;
    const cudaError_t ei = (st == 0 && ec == cudaSuccess) ? cudaGraphInstantiate(&exec, g, 0) : cudaErrorUnknown;
    if (g) cudaGraphDestroy(g);
    if (st) return st;
    if (ei != cudaSuccess) {  // capture not possible here: the direct path
        cudaGetLastError();
        return enqueue_step(c, prev, next, dt);
    }
    if (v.size() >= kStepGraphs) {
        cudaGraphExecDestroy(v.front().exec);
        v.erase(v.begin());
    }
    v.push_back({prev, next, dt, exec});
    ADSG_CUDA_TRY(cudaGraphLaunch(exec, c->stream), "step graph launch");
    return 0;
}

// Step tuner: time a few explicit steps under each launch mode and keep the
// fastest; then time the chosen mode replayed from single-step graphs against
// direct launches.  None of the switches changes any result bit: programmatic
// dependent launch (ADSG_PDL=0/1 forces it), fusing the x band pass into the
// staged two-ended x solve where that is the x variant (ADSG_FUSE_X), the
// one-launch step of small 2D grids (ADSG_STEP_1BLOCK), that step on a
// thread-block cluster rather than one block (ADSG_STEP_CLUSTER) and the graph
// replay (ADSG_STEP_GRAPHS).
int autotune_launch_mode(adsg_ctx* c) {
    auto forced = [](const char* name) -> int {
        const char* v = std::getenv(name);
        return v && (*v == '0' || *v == '1') ? *v - '0' : -1;
    };
    const int f_pdl = forced("ADSG_PDL"), f_fuse = forced("ADSG_FUSE_X"), f_one = forced("ADSG_STEP_1BLOCK"),
              f_graph = forced("ADSG_STEP_GRAPHS"), f_cluster = forced("ADSG_STEP_CLUSTER");
    const bool can_fuse = fusion_ok(c), can_one = step_1block_ok(c);
    // bit 0: pdl, bit 1: fuse, bit 2: one-launch step, bit 3: graph replay, bit 4: that step on a cluster
    std::vector<int> modes;
    for (int m = 0; m < 32; ++m) {
        const int pdl = m & 1, fuse = (m >> 1) & 1, one = (m >> 2) & 1, graph = (m >> 3) & 1, cl = (m >> 4) & 1;
        if (fuse && !can_fuse) continue;
        if (one && !can_one) continue;
        if (one && fuse) continue;  // the one-launch step has no separate x pass
        if (cl && !one) continue;
        if (f_pdl >= 0 && pdl != f_pdl) continue;
        if (f_fuse >= 0 && fuse != (f_fuse && can_fuse)) continue;
        if (f_one >= 0 && one != (f_one && can_one)) continue;
        if (f_graph >= 0 && graph != f_graph) continue;
        if (f_cluster >= 0 && one && cl != f_cluster) continue;
        modes.push_back(m);
    }
    if (modes.empty()) modes.push_back(0);
    auto apply = [&](int m) {
        c->drop_step_graphs();  // a graph holds the launches of the mode it was captured under
        c->step_graph_hits = c->step_graph_misses = 0;
        c->pdl = m & 1;
        c->fuse_x = (m >> 1) & 1;
        c->step_1block = (m >> 2) & 1;
        c->step_graphs_on = (m >> 3) & 1;
        c->step_cluster = (m >> 4) & 1;
    };
    if (modes.size() == 1) {
        apply(modes[0]);
        return 0;
    }
    double* tmp = nullptr;
    if (device_alloc(reinterpret_cast<void**>(&tmp), sizeof(double) * c->size) != cudaSuccess) {  // no room: keep plain launches
        cudaGetLastError();
        apply(modes[0]);
        return 0;
    }
    cudaEvent_t a = nullptr, b = nullptr;
    cudaError_t e = cudaEventCreate(&a);
    if (e == cudaSuccess) e = cudaEventCreate(&b);
    float best = 1e30f;
    int best_mode = modes[0], rc = 0;
    // steps of small grids take tens of microseconds: time enough of them
    // that launch jitter does not pick the mode
    const int reps = c->size < (1 << 20) ? 32 : 4;
    const char* logv = std::getenv("ADSG_AUTOTUNE_LOG");
    const bool log = logv && *logv == '1';
    for (size_t i = 0; i < modes.size() && e == cudaSuccess && rc == 0; ++i) {
        apply(modes[i]);
        auto step = [&](const double* p, double* q) {
            return c->step_graphs_on ? step_via_graph(c, p, q, 1e-6) : enqueue_step(c, p, q, 1e-6);
        };
        rc = step(c->ping, tmp);  // warm-up (also builds the dt bands and captures the graphs)
        if (rc == 0) rc = step(tmp, c->ping);
        if (rc != 0 && c->step_cluster) {
            // a cluster launch the device refuses drops the mode, not the context
            cudaGetLastError();
            if (cudaStreamSynchronize(c->stream) == cudaSuccess) {
                rc = 0;
                continue;
            }
        }
        if (rc == 0) e = cudaEventRecord(a, c->stream);
        for (int r = 0; r < reps && rc == 0 && e == cudaSuccess; ++r) {
            rc = step(c->ping, tmp);
            if (rc == 0) rc = step(tmp, c->ping);
        }
        if (rc == 0 && e == cudaSuccess) e = cudaEventRecord(b, c->stream);
        if (rc == 0 && e == cudaSuccess) e = cudaEventSynchronize(b);
        float ms = 0.f;
        if (rc == 0 && e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
        if (rc == 0 && e == cudaSuccess && log)
            std::fprintf(stderr, "ads_gb300 autotune: launch mode pdl=%d fuse_x=%d one_launch=%d graphs=%d cluster=%d %.2f us/step\n",
                         modes[i] & 1, (modes[i] >> 1) & 1, (modes[i] >> 2) & 1, (modes[i] >> 3) & 1,
                         (modes[i] >> 4) & 1, 1e3 * ms / (2 * reps));
        if (rc == 0 && e == cudaSuccess && ms < best) {
            best = ms;
            best_mode = modes[i];
        }
    }
    apply(best_mode);  // also drops the graphs, which name the tuner's buffers
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    cudaFree(tmp);
    if (rc) return rc;
    if (e != cudaSuccess) return fail_cuda(e, "launch-mode tuner");
    // the tuner ran on the context's own (zeroed) state buffer; leave it zero
    ADSG_CUDA_TRY(cudaMemsetAsync(c->ping, 0, sizeof(double) * c->size, c->stream), "launch-mode tuner");
    return 0;
}

// Host-buffer steps (2D and 3D).  The host link moves ~200 GB/s either way,
// so each step's state costs about as long to move as to compute.  When the
// input is pinned host memory (mapped into the device's address space), the
// first step's first band pass, the only reader of that input, reads it
// there directly as column sweeps: the upload runs under the pass's
// arithmetic instead of before it.  The result is copied back once after the
// last step (stores to host memory from the solve kernels were measured
// slower than one copy).
// Host entry, slab-chunked first step.  The first step's right-hand side
// reads the pinned input over the host link (outer-axis column sweeps), and
// its later passes need only their own slab of the outer axis.  So that step's
// passes run in chunks of outer-axis slabs as a two-stage pipeline on two
// streams: the host-reading column sweeps of all chunks on one, the y and x
// passes of each chunk on the other as soon as that chunk's sweep is done
// (an event per chunk), which overlaps the link transfer with FP64 passes.
// Every output takes the same operations as unchunked: the same bits.  (The
// last step's line solves are not chunked: a sweep's time is set by its line
// length, not by the number of lines, so chunks of lines would run one after
// another where they now run side by side.)
constexpr int kMaxHostChunks = 16;

int ensure_aux(adsg_ctx* c) {
    if (c->aux) return 0;
    ADSG_CUDA_TRY(cudaStreamCreateWithFlags(&c->aux, cudaStreamNonBlocking), "aux stream");
    ADSG_CUDA_TRY(cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming), "fork event");
    ADSG_CUDA_TRY(cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming), "join event");
    for (auto& e : c->ev_chunk) ADSG_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "chunk event");
    return 0;
}

int host_chunks(adsg_ctx* c) {
    if (c->host_chunks < 0) {
        const char* v = std::getenv("ADSG_HOST_CHUNKS");
        int k = v && *v ? std::atoi(v) : 2;
        c->host_chunks = std::max(1, std::min({k, kMaxHostChunks, c->n[c->ndim - 1] / 4}));
    }
    return c->ndim >= 2 ? c->host_chunks : 1;
}

// aux waits for everything issued so far on the context's stream
int fork_aux(adsg_ctx* c) {
    ADSG_CUDA_TRY(cudaEventRecord(c->ev_fork, c->stream), "fork");
    ADSG_CUDA_TRY(cudaStreamWaitEvent(c->aux, c->ev_fork, 0), "fork");
    return 0;
}

// rows [r0, r1) of chunk k of K over an outer axis of n rows
void chunk_rows(int n, int k, int K, int* r0, int* r1) {
    *r0 = static_cast<int>(static_cast<long long>(n) * k / K);
    *r1 = static_cast<int>(static_cast<long long>(n) * (k + 1) / K);
}

// The whole right-hand side of the first step from the pinned input (device
// view in_dev): the host-reading column sweeps of all chunks on aux, the
// chunks' y and x passes on the context's stream.
int enqueue_rhs_from_host_chunked(adsg_ctx* c, const dim_dev* D, const double* in_dev, double* rhs, int K) {
    pdl_scope pdl(c->pdl);
    const int o = c->ndim - 1;
    const long long so = c->size / c->n[o];
    double** T = c->scratch;
    if (int st = fork_aux(c)) return st;
    for (int k = 0; k < K; ++k) {
        int r0, r1;
        chunk_rows(c->n[o], k, K, &r0, &r1);
        ADSG_CUDA_TRY(launch_outer_pass_columns(D[o].p, in_dev, T[0], T[1], D[o].mrow, D[o].nrow, c->n[o], so, c->aux,
                                                D[o].sym_lo, D[o].sym_hi, r0, r1),
                      "rhs pass (outer, from host, chunk)");
        ADSG_CUDA_TRY(cudaEventRecord(c->ev_chunk[k], c->aux), "chunk event");
    }
    for (int k = 0; k < K; ++k) {
        int r0, r1;
        chunk_rows(c->n[o], k, K, &r0, &r1);
        const long long off = r0 * so, cnt = (r1 - r0) * so;
        ADSG_CUDA_TRY(cudaStreamWaitEvent(c->stream, c->ev_chunk[k], 0), "chunk wait");
        if (c->ndim == 3) {
            // F = (-dt Ky) A + My C, G = My A on the chunk's slabs
            ADSG_CUDA_TRY(launch_band_pass(D[1].p, T[0] + off, T[1] + off, T[2] + off, T[3] + off, D[1].kdt, D[1].mrow,
                                           D[1].mrow, D[1].n, c->n[0], cnt, c->stream, D[1].sym_lo, D[1].sym_hi),
                          "rhs pass y (chunk)");
            ADSG_CUDA_TRY(launch_band_pass(D[0].p, T[3] + off, T[2] + off, rhs + off, nullptr, D[0].kdt, D[0].mrow,
                                           nullptr, D[0].n, 1, cnt, c->stream),
                          "rhs pass x (chunk)");
        } else {
            ADSG_CUDA_TRY(launch_band_pass(D[0].p, T[0] + off, T[1] + off, rhs + off, nullptr, D[0].kdt, D[0].mrow,
                                           nullptr, D[0].n, 1, cnt, c->stream),
                          "rhs pass x (chunk)");
        }
    }
    return 0;  // the context's stream waited for every chunk's sweep on aux
}

int heat_steps_host_direct(adsg_ctx* c, const double* u_in, double* u_out, double dt, int nsteps) {
    const int o = c->ndim - 1;  // outermost axis
    const long long so = c->size / c->n[o];
    int st = ensure_dt_bands(c, dt);
    if (st) return st;
    const dim_dev* D = c->sdims;
    double* cur = c->host_io;
    double* nxt = c->ping;
    const double* in_dev = nullptr;
    {
        cudaPointerAttributes attr{};
        if (cudaPointerGetAttributes(&attr, u_in) == cudaSuccess && attr.type == cudaMemoryTypeHost)
            in_dev = static_cast<const double*>(attr.devicePointer);
        cudaGetLastError();
    }
    // below ~2 MB the copy is a few microseconds and the column sweeps would
    // run nearly serially
    const bool direct_in = in_dev && outer_pass_columns_ok(D[o].p) && c->size >= (1LL << 18);
    // slab chunks on two streams (not with stage timers, which time one stream)
    const int K = c->timing ? 1 : host_chunks(c);
    if (K > 1)
        if (int st2 = ensure_aux(c)) return st2;
    const bool chunked_in = direct_in && K > 1 && !(c->fuse_x && fusion_ok(c));
    if (chunked_in) {
        // the first step's whole right-hand side, below
    } else if (direct_in) {
        pdl_scope pdl(c->pdl);
        stage_scope sc(c, ADSG_STAGE_RHS_OUTER);
        ADSG_CUDA_TRY(launch_outer_pass_columns(D[o].p, in_dev, c->scratch[0], c->scratch[1], D[o].mrow, D[o].nrow,
                                                c->n[o], so, c->stream, D[o].sym_lo, D[o].sym_hi),
                      "rhs pass (outer, from host)");
    } else {
        ADSG_CUDA_TRY(cudaMemcpyAsync(cur, u_in, sizeof(double) * c->size, cudaMemcpyHostToDevice, c->stream), "H2D");
    }
    // a pinned u_out (mapped) takes the last step's x sweep straight from its
    // tiles: the download runs under that sweep instead of after it
    double* out_dev = nullptr;
    {
        cudaPointerAttributes attr{};
        if (cudaPointerGetAttributes(&attr, u_out) == cudaSuccess && attr.type == cudaMemoryTypeHost)
            out_dev = static_cast<double*>(attr.devicePointer);
        cudaGetLastError();
    }
    for (int step = 0; step < nsteps; ++step) {
        const bool fused = c->fuse_x && fusion_ok(c);
        if (step == 0 && chunked_in)
            st = enqueue_rhs_from_host_chunked(c, D, in_dev, nxt, K);
        else
            st = enqueue_rhs_with(c, D, cur, nxt, dt, fused, /*outer_done=*/step == 0 && direct_in);
        if (st) return st;
        const bool to_host = step + 1 == nsteps && !fused && out_dev && step_x_out_ok(c) && c->size >= (1LL << 18);
        st = enqueue_step_solves(c, nxt, fused, to_host ? out_dev : nullptr);
        if (st) return st;
        if (to_host) return 0;
        std::swap(cur, nxt);
    }
    ADSG_CUDA_TRY(cudaMemcpyAsync(u_out, cur, sizeof(double) * c->size, cudaMemcpyDeviceToHost, c->stream), "D2H");
    return 0;
}

// The same, replayed from a graph cached per (pinned buffer, dt, nsteps) when
// the context replays its steps from graphs; pageable buffers (which a graph
// cannot copy to), a stream under capture and stage timers take the direct
// path.  Same operations either way.
int heat_steps_host_graph(adsg_ctx* c, double* u, double dt, int nsteps) {
    bool pinned = false;
    {
        cudaPointerAttributes attr{};
        pinned = cudaPointerGetAttributes(&attr, u) == cudaSuccess && attr.type == cudaMemoryTypeHost;
        cudaGetLastError();
    }
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(c->stream, &cs) != cudaSuccess) {
        cudaGetLastError();
        cs = cudaStreamCaptureStatusActive;
    }
    if (!pinned || !c->step_graphs_on || c->timing || cs != cudaStreamCaptureStatusNone)
        return heat_steps_host_direct(c, u, u, dt, nsteps);
    int st = ensure_dt_bands(c, dt);
    if (st) return st;
    if (host_chunks(c) > 1 && (st = ensure_aux(c)) != 0) return st;  // created outside the capture
    if (!(c->host_graph && c->host_graph_u == u && c->host_graph_dt == dt && c->host_graph_steps == nsteps)) {
        if (c->host_graph) cudaGraphExecDestroy(c->host_graph);
        c->host_graph = nullptr;
        cudaGraph_t g = nullptr;
        if (cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
            cudaGetLastError();
            return heat_steps_host_direct(c, u, u, dt, nsteps);
        }
        c->capturing = true;
        st = heat_steps_host_direct(c, u, u, dt, nsteps);
        c->capturing = false;
        const cudaError_t ec = cudaStreamEndCapture(c->stream, &g);
        cudaGraphExec_t exec = nullptr;
        const cudaError_t ei = (st == 0 && ec == cudaSuccess) ? cudaGraphInstantiate(&exec, g, 0) : cudaErrorUnknown;
        if (g) cudaGraphDestroy(g);
        if (st) return st;
        if (ei != cudaSuccess) {
            cudaGetLastError();
            return heat_steps_host_direct(c, u, u, dt, nsteps);
        }
        c->host_graph = exec;
        c->host_graph_u = u;
        c->host_graph_dt = dt;
        c->host_graph_steps = nsteps;
    }
    ADSG_CUDA_TRY(cudaGraphLaunch(c->host_graph, c->stream), "host step graph launch");
    return 0;
}

}  // namespace

namespace adsg {
cudaStream_t ctx_stream(adsg_ctx* c) { return c->stream; }
int ctx_prepare_dt(adsg_ctx* c, double dt) { return ensure_dt_bands(c, dt); }
int ctx_rhs(adsg_ctx* c, const double* u, double* rhs, double dt) { return enqueue_rhs(c, u, rhs, dt); }
int ctx_solve(adsg_ctx* c, double* x, int trans) { return enqueue_solve(c, x, trans); }
}  // namespace adsg

extern "C" {

const char* adsg_last_error(void) { return g_last_error.c_str(); }

int adsg_ctx_create(int ndim, const adsg_dim_desc* dims, adsg_ctx** out) {
    if (ndim < 1 || ndim > 3) return fail(-1, "ndim must be 1, 2 or 3");
    if (!dims) return fail(-2, "dims is NULL");
    if (!out) return fail(-3, "out is NULL");
    *out = nullptr;
    for (int d = 0; d < ndim; ++d)
        if (!valid_desc(dims[d])) return fail(-2, "invalid dimension descriptor");
    auto* c = new (std::nothrow) adsg_ctx;
    if (!c) return fail(ADSG_ERR_NOMEM, "host allocation failed");
    c->ndim = ndim;
    c->size = 1;
    for (int d = 0; d < ndim; ++d) {
        c->n[d] = dims[d].n;
        c->size *= dims[d].n;
    }
    if (c->size >= (1LL << 31)) {
        delete c;
        return fail(-2, "tensor larger than 2^31 dofs");
    }
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamDefault);
    if (e != cudaSuccess) {
        delete c;
        return fail_cuda(e, "cudaStreamCreate");
    }
    twisted_tables tw_keep[3];
    bool tw_ok[3] = {false, false, false};
    c->own_stream = true;

    auto bail = [&](cudaError_t err, const char* where) {
        int r = fail_cuda(err, where);
        delete c;
        return r;
    };
    for (int d = 0; d < ndim; ++d) {
        const adsg_dim_desc& h = dims[d];
        dim_dev& D = c->dims[d];
        D.n = h.n;
        D.p = h.p;
        D.elements = h.elements;
        D.q = h.quad_order;
        solve_tables t;
        if (make_solve_tables(h.n, h.kl, h.ku, h.ldab, h.lu, h.ipiv, t)) {
            delete c;
            return fail(ADSG_ERR_SINGULAR, "zero diagonal in the factorised band");
        }
        D.kl = t.kl;
        D.w = t.w;
        D.ku_regular = h.ku;
        D.fwd_fast = t.fwd_fast;
        D.bwd_fast = t.bwd_fast;
        for (int v : t.uext) c->uext_sum[d] += v;
        twisted_tables& tw = tw_keep[d];
        const bool have_tw = make_twisted_tables(h.n, h.kl, h.ku, h.ldab, h.lu, h.ipiv, tw) == 0;
        tw_ok[d] = have_tw;
        const std::vector<double> m = row_band(h, 0);
        const std::vector<double> k = row_band(h, 1);
        symmetric_row_range(m, k, h.n, h.p, D.sym_lo, D.sym_hi);
        {
            // ADSG_PAIR_SUMS=0: full-band passes on every row (no symmetric
            // range), to measure what the pair sums change
            const char* ps = std::getenv("ADSG_PAIR_SUMS");
            if (ps && *ps == '0') D.sym_lo = D.sym_hi = 0;
        }
        const size_t nb = static_cast<size_t>(h.elements) * h.quad_order * 2 * (h.p + 1);
        double *mrow = nullptr, *krow = nullptr, *lmul = nullptr, *ucol = nullptr, *rdiag = nullptr;
        double *btab = nullptr, *wq = nullptr, *jac = nullptr;
        int *piv = nullptr, *uext = nullptr, *first = nullptr;
        dev_arena& A = c->arena;
        cudaStream_t s = c->stream;
        e = A.upload(&mrow, m.data(), m.size(), s);
        if (e == cudaSuccess) e = A.upload(&krow, k.data(), k.size(), s);
        if (e == cudaSuccess) e = A.alloc(&c->nrow[d], m.size());
        if (e == cudaSuccess) e = A.alloc(&c->kdt[d], m.size());
        if (e == cudaSuccess) e = A.upload(&lmul, t.lmul.data(), t.lmul.size(), s);
        if (e == cudaSuccess) e = A.upload(&ucol, t.ucol.data(), t.ucol.size(), s);
        if (e == cudaSuccess) e = A.upload(&rdiag, t.rdiag.data(), t.rdiag.size(), s);
        if (e == cudaSuccess) e = A.upload(&piv, t.piv.data(), t.piv.size(), s);
        if (e == cudaSuccess) e = A.upload(&uext, t.uext.data(), t.uext.size(), s);
        if (e == cudaSuccess) e = A.upload(&btab, h.btab, nb, s);
        if (e == cudaSuccess) e = A.upload(&wq, h.w, h.quad_order, s);
        if (e == cudaSuccess) e = A.upload(&jac, h.J, h.elements, s);
        if (e == cudaSuccess) e = A.upload(&first, h.first_dofs, h.elements, s);
        std::vector<int> er(2 * static_cast<size_t>(h.n));
        for (int a = 0; a < h.n; ++a) {
            er[2 * a] = h.elements;
            er[2 * a + 1] = -1;
        }
        for (int el = 0; el < h.elements; ++el)
            for (int a = h.first_dofs[el]; a <= h.first_dofs[el] + h.p; ++a) {
                er[2 * a] = std::min(er[2 * a], el);
                er[2 * a + 1] = std::max(er[2 * a + 1], el);
            }
        int* erange = nullptr;
        if (e == cudaSuccess) e = A.upload(&erange, er.data(), er.size(), s);
        double *tw_l = nullptr, *tw_u = nullptr, *tw_r = nullptr, *tw_g = nullptr;
        if (have_tw) {
            if (e == cudaSuccess) e = A.upload(&tw_l, tw.lmul.data(), tw.lmul.size(), s);
            if (e == cudaSuccess) e = A.upload(&tw_u, tw.ucol.data(), tw.ucol.size(), s);
            if (e == cudaSuccess) e = A.upload(&tw_r, tw.rdiag.data(), tw.rdiag.size(), s);
            if (e == cudaSuccess) e = A.upload(&tw_g, tw.g.data(), tw.g.size(), s);
        }
        if (h.xq) c->xq[d].assign(h.xq, h.xq + static_cast<size_t>(h.elements) * h.quad_order);
        // the host staging vectors above die at the end of this iteration
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return bail(e, "set-up upload");
        D.mrow = mrow;
        D.krow = krow;
        D.lmul = lmul;
        D.ucol = ucol;
        D.rdiag = rdiag;
        D.piv = piv;
        D.uext = uext;
        D.btab = btab;
        D.wq = wq;
        D.jac = jac;
        D.first = first;
        D.erange = erange;
        if (have_tw) {
            D.tw_k = tw.k;
            D.tw_n1 = tw.n1;
            D.tw_n2 = tw.n2;
            D.tw_rows = tw.rows;
            D.tw_lmul = tw_l;
            D.tw_ucol = tw_u;
            D.tw_rdiag = tw_r;
            D.tw_g = tw_g;
        }
    }
    const int nscratch = ndim == 3 ? 4 : (ndim == 2 ? 2 : 0);
    for (int i = 0; i < nscratch; ++i)
        if ((e = c->arena.alloc(&c->scratch[i], c->size)) != cudaSuccess) return bail(e, "scratch alloc");
    if ((e = c->arena.alloc(&c->ping, c->size)) != cudaSuccess) return bail(e, "state alloc");
    if ((e = cudaStreamSynchronize(c->stream)) != cudaSuccess) return bail(e, "set-up copies");
    if (int st = autotune_solves(c)) {
        delete c;
        return st;
    }
    for (int d = 0; d < ndim; ++d)
        if (int st = build_step_dim(c, d, dims[d], tw_ok[d] ? &tw_keep[d] : nullptr)) {
            delete c;
            return st;
        }
    if (int st = autotune_launch_mode(c)) {
        delete c;
        return st;
    }
    *out = c;
    return 0;
}

int adsg_ctx_destroy(adsg_ctx* ctx) {
    if (!ctx) return 0;
    cudaStreamSynchronize(ctx->stream);
    detach_adjoints(ctx);
    delete ctx;
    return 0;
}

long long adsg_ctx_size(const adsg_ctx* ctx) { return ctx ? ctx->size : 0; }

int adsg_ctx_set_stream(adsg_ctx* ctx, void* cuda_stream) {
    if (!ctx) return fail(-1, "ctx is NULL");
    if (ctx->graph) {
        cudaGraphExecDestroy(ctx->graph);
        ctx->graph = nullptr;
    }
    ctx->drop_step_graphs();
    if (ctx->own_stream) {
        cudaStreamSynchronize(ctx->stream);
        cudaStreamDestroy(ctx->stream);
        ctx->own_stream = false;
        ctx->stream = nullptr;
    }
    if (cuda_stream) {
        ctx->stream = static_cast<cudaStream_t>(cuda_stream);
    } else {
        ADSG_CUDA_TRY(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamDefault), "cudaStreamCreate");
        ctx->own_stream = true;
    }
    return 0;
}

int adsg_ctx_synchronize(adsg_ctx* ctx) {
    if (!ctx) return fail(-1, "ctx is NULL");
    ADSG_CUDA_TRY(cudaStreamSynchronize(ctx->stream), "synchronize");
    if (solve_variant_twisted(ctx->dims[0].solve_variant) || solve_variant_twisted(ctx->sdims[0].solve_variant))
        if (bulk_wait_timeouts(1) > 0)
            return fail(ADSG_ERR_DEVICE, "a bulk-copy wait of an x-line solve ran out (lines left unsolved)");
    return 0;
}

int adsg_heat_rhs(adsg_ctx* ctx, const double* u_prev_dev, double* rhs_dev, double dt) {
    if (!ctx) return fail(-1, "ctx is NULL");
    if (!u_prev_dev) return fail(-2, "u_prev is NULL");
    if (!rhs_dev) return fail(-3, "rhs is NULL");
    if (u_prev_dev == rhs_dev) return fail(-3, "rhs must not alias u_prev");
    if (!std::isfinite(dt)) return fail(-4, "dt must be finite");
    return enqueue_rhs(ctx, u_prev_dev, rhs_dev, dt);
}

int adsg_heat_rhs_elem(adsg_ctx* ctx, const double* u_prev_dev, const double* kappa_dev, double* rhs_dev,
                       double dt) {
    if (!ctx) return fail(-1, "ctx is NULL");
    if (!u_prev_dev) return fail(-2, "u_prev is NULL");
    if (!rhs_dev) return fail(-4, "rhs is NULL");
    if (u_prev_dev == rhs_dev || kappa_dev == rhs_dev) return fail(-4, "rhs must not alias an input");
    if (!std::isfinite(dt)) return fail(-5, "dt must be finite");
    ADSG_CUDA_TRY(cudaMemsetAsync(rhs_dev, 0, sizeof(double) * ctx->size, ctx->stream), "memset rhs");
    stage_scope sc(ctx, ADSG_STAGE_RHS_ELEM);
    ADSG_CUDA_TRY(launch_rhs_elem(ctx->ndim, ctx->dims, u_prev_dev, kappa_dev, rhs_dev, dt, ctx->stream),
                  "element rhs");
    return 0;
}

long long adsg_kappa_points_count(const adsg_ctx* ctx) { return ctx ? kappa_points_count(ctx->ndim, ctx->dims) : 0; }

int adsg_kappa_points(adsg_ctx* ctx, const double* kappa_dev, double* kq_dev) {
    if (!ctx) return fail(-1, "ctx is NULL");
    if (!kappa_dev) return fail(-2, "kappa is NULL");
    if (!kq_dev) return fail(-3, "kq is NULL");
    if (ctx->ndim != 3) return fail(ADSG_ERR_UNSUPPORTED, "Gauss-point kappa values are for 3D contexts");
    ADSG_CUDA_TRY(launch_kappa_points(ctx->dims, kappa_dev, kq_dev, ctx->stream), "kappa at the Gauss points");
    return 0;
}

int adsg_heat_rhs_elem_points(adsg_ctx* ctx, const double* u_prev_dev, const double* kq_dev, double* rhs_dev,
                              double dt) {
    if (!ctx) return fail(-1, "ctx is NULL");
    if (!u_prev_dev) return fail(-2, "u_prev is NULL");
    if (!kq_dev) return fail(-3, "kq is NULL");
    if (!rhs_dev) return fail(-4, "rhs is NULL");
    if (u_prev_dev == rhs_dev || kq_dev == rhs_dev) return fail(-4, "rhs must not alias an input");
    if (!std::isfinite(dt)) return fail(-5, "dt must be finite");
    if (ctx->ndim != 3) return fail(ADSG_ERR_UNSUPPORTED, "Gauss-point kappa values are for 3D contexts");
    ADSG_CUDA_TRY(cudaMemsetAsync(rhs_dev, 0, sizeof(double) * ctx->size, ctx->stream), "memset rhs");
    stage_scope sc(ctx, ADSG_STAGE_RHS_ELEM);
    ADSG_CUDA_TRY(launch_rhs_elem_points(ctx->dims, u_prev_dev, kq_dev, rhs_dev, dt, ctx->stream), "element rhs");
    return 0;
}

int adsg_ads_solve(adsg_ctx* ctx, double* rhs_dev, double* buf_dev) {
    (void)buf_dev;
    if (!ctx) return fail(-1, "ctx is NULL");
    if (!rhs_dev) return fail(-2, "rhs is NULL");
    return enqueue_solve(ctx, rhs_dev, 0);
}

int adsg_ads_solve_t(adsg_ctx* ctx, double* rhs_dev) {
    if (!ctx) return fail(-1, "ctx is NULL");
    if (!rhs_dev) return fail(-2, "rhs is NULL");
    return enqueue_solve(ctx, rhs_dev, 1);
}

int adsg_form_rhs(adsg_ctx* ctx, const double* u_dev, const adsg_point_form* form, double* rhs_dev) {
    if (!ctx) return fail(-1, "ctx is NULL");
    if (!form) return fail(-3, "form is NULL");
    if (!rhs_dev) return fail(-4, "rhs is NULL");
    const bool needs_u = form->alpha != 0.0 || form->beta != 0.0 || form->alpha_q || form->beta_q;
    if (needs_u && !u_dev) return fail(-2, "u is NULL but the form has u terms");
    if (ctx->ndim < 2) return fail(ADSG_ERR_UNSUPPORTED, "forms need a 2D or 3D context");
    for (int d = 0; d < ctx->ndim; ++d)
        if (ctx->dims[d].p != ctx->dims[0].p || ctx->dims[d].q != ctx->dims[d].p + 1 || ctx->dims[d].p > 4)
            return fail(ADSG_ERR_UNSUPPORTED, "forms need the same degree p <= 4 and p+1 Gauss points in every direction");
    point_form F;
    F.alpha = form->alpha;
    F.beta = form->beta;
    F.gamma = form->gamma;
    F.delta = form->delta;
    F.alpha_q = form->alpha_q;
    F.beta_q = form->beta_q;
    F.gamma_q = form->gamma_q;
    F.delta_q = form->delta_q;
    ADSG_CUDA_TRY(cudaMemsetAsync(rhs_dev, 0, sizeof(double) * ctx->size, ctx->stream), "memset");
    stage_scope sc(ctx, ADSG_STAGE_RHS_ELEM);
    ADSG_CUDA_TRY(launch_form_elem(ctx->ndim, ctx->dims, needs_u ? u_dev : nullptr, F, rhs_dev, ctx->stream),
                  "form rhs");
    return 0;
}

int adsg_heat_step(adsg_ctx* ctx, const double* u_prev_dev, double* u_next_dev, double dt) {
    if (!ctx) return fail(-1, "ctx is NULL");
    if (!u_prev_dev) return fail(-2, "u_prev is NULL");
    if (!u_next_dev) return fail(-3, "u_next is NULL");
    if (!std::isfinite(dt)) return fail(-4, "dt must be finite");
    const char* a = reinterpret_cast<const char*>(u_prev_dev);
    const char* b = reinterpret_cast<const char*>(u_next_dev);
    const size_t bytes = sizeof(double) * static_cast<size_t>(ctx->size);
    if (a < b + bytes && b < a + bytes) return fail(-3, "u_prev and u_next overlap");
    return step_via_graph(ctx, u_prev_dev, u_next_dev, dt);
}

int adsg_set_planes(adsg_ctx* ctx, double* u_dev, int nplanes, const adsg_plane* planes) {
    if (!ctx) return fail(-1, "ctx is NULL");
    if (!u_dev) return fail(-2, "u is NULL");
    if (nplanes < 0) return fail(-3, "nplanes < 0");
    if (nplanes > 0 && !planes) return fail(-4, "planes is NULL");
    for (int i = 0; i < nplanes; ++i)
        if (planes[i].dim < 0 || planes[i].dim >= ctx->ndim || planes[i].index < 0 ||
            planes[i].index >= ctx->n[planes[i].dim])
            return fail(-4, "a plane's direction or index is outside the tensor");
    for (int i = 0; i < nplanes; ++i)
        ADSG_CUDA_TRY(launch_set_plane(u_dev, planes[i].values, ctx->n, ctx->ndim, planes[i].dim, planes[i].index,
                                       ctx->stream),
                      "set plane");
    return 0;
}

int adsg_heat_step_dirichlet(adsg_ctx* ctx, const double* u_prev_dev, double* u_next_dev, double dt, int nplanes,
                             const adsg_plane* planes) {
    if (!ctx) return fail(-1, "ctx is NULL");
    if (!u_prev_dev) return fail(-2, "u_prev is NULL");
    if (!u_next_dev) return fail(-3, "u_next is NULL");
    if (!std::isfinite(dt)) return fail(-4, "dt must be finite");
    if (nplanes < 0) return fail(-5, "nplanes < 0");
    if (nplanes > 0 && !planes) return fail(-6, "planes is NULL");
    const char* a = reinterpret_cast<const char*>(u_prev_dev);
    const char* b = reinterpret_cast<const char*>(u_next_dev);
    const size_t bytes = sizeof(double) * static_cast<size_t>(ctx->size);
    if (a < b + bytes && b < a + bytes) return fail(-3, "u_prev and u_next overlap");
    for (int i = 0; i < nplanes; ++i)
        if (planes[i].dim < 0 || planes[i].dim >= ctx->ndim || planes[i].index < 0 ||
            planes[i].index >= ctx->n[planes[i].dim])
            return fail(-6, "a plane's direction or index is outside the tensor");
    if (int st = enqueue_rhs(ctx, u_prev_dev, u_next_dev, dt)) return st;
    if (int st = adsg_set_planes(ctx, u_next_dev, nplanes, planes)) return st;
    return enqueue_solve(ctx, u_next_dev, 0);
}

int adsg_heat_steps(adsg_ctx* ctx, double* u_dev, double dt, int nsteps) {
    if (!ctx) return fail(-1, "ctx is NULL");
    if (!u_dev) return fail(-2, "u is NULL");
    if (!std::isfinite(dt)) return fail(-3, "dt must be finite");
    if (nsteps < 0) return fail(-4, "nsteps must be >= 0");
    if (nsteps == 0) return 0;
    int st = ensure_dt_bands(ctx, dt);
    if (st) return st;
    if (nsteps >= 2 && !(ctx->graph && ctx->graph_dt == dt && ctx->graph_u == u_dev)) {
        if (ctx->graph) {
            cudaGraphExecDestroy(ctx->graph);
            ctx->graph = nullptr;
        }
        cudaGraph_t g = nullptr;
        ADSG_CUDA_TRY(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
        ctx->capturing = true;
        int s1 = enqueue_step(ctx, u_dev, ctx->ping, dt);
        int s2 = s1 ? s1 : enqueue_step(ctx, ctx->ping, u_dev, dt);
        ctx->capturing = false;
        cudaError_t ec = cudaStreamEndCapture(ctx->stream, &g);
        if (s2) {
            if (g) cudaGraphDestroy(g);
            return s2;
        }
        if (ec != cudaSuccess) return fail_cuda(ec, "end capture");
        cudaError_t ei = cudaGraphInstantiate(&ctx->graph, g, 0);
        cudaGraphDestroy(g);
        if (ei != cudaSuccess) {
            ctx->graph = nullptr;
            return fail_cuda(ei, "graph instantiate");
        }
        ctx->graph_dt = dt;
        ctx->graph_u = u_dev;
    }
    for (int i = 0; i + 1 < nsteps; i += 2) ADSG_CUDA_TRY(cudaGraphLaunch(ctx->graph, ctx->stream), "graph launch");
    if (nsteps % 2) {
        st = enqueue_step(ctx, u_dev, ctx->ping, dt);
        if (st) return st;
        ADSG_CUDA_TRY(cudaMemcpyAsync(u_dev, ctx->ping, sizeof(double) * ctx->size, cudaMemcpyDeviceToDevice,
                                      ctx->stream),
                      "copy state");
    }
    return 0;
}

int adsg_ctx_enable_stage_timers(adsg_ctx* ctx, int enable) {
    if (!ctx) return fail(-1, "ctx is NULL");
    ctx->timing = enable != 0;
    return 0;
}

int adsg_ctx_stage_times(adsg_ctx* ctx, double* ms, long long* launches) {
    if (!ctx) return fail(-1, "ctx is NULL");
    ADSG_CUDA_TRY(cudaStreamSynchronize(ctx->stream), "synchronize");
    ctx->drain();
    for (int i = 0; i < ADSG_NSTAGES; ++i) {
        if (ms) ms[i] = ctx->stage_ms[i];
        if (launches) launches[i] = ctx->stage_launches[i];
        ctx->stage_ms[i] = 0.0;
        ctx->stage_launches[i] = 0;
    }
    return 0;
}

int adsg_ctx_solve_variants(const adsg_ctx* ctx, int* variants) {
    if (!ctx) return fail(-1, "ctx is NULL");
    if (!variants) return fail(-2, "variants is NULL");
    for (int d = 0; d < 3; ++d) variants[d] = d < ctx->ndim ? ctx->dims[d].solve_variant : -1;
    return 0;
}

int adsg_ctx_step_solve_variants(const adsg_ctx* ctx, int* variants) {
    if (!ctx) return fail(-1, "ctx is NULL");
    if (!variants) return fail(-2, "variants is NULL");
    for (int d = 0; d < 3; ++d) variants[d] = d < ctx->ndim ? ctx->sdims[d].solve_variant : -1;
    return 0;
}

int adsg_ctx_launch_pdl(const adsg_ctx* ctx) { return ctx ? ctx->pdl : -1; }

int adsg_ctx_fused_x(const adsg_ctx* ctx) { return ctx ? ctx->fuse_x : -1; }

int adsg_ctx_step_1block(const adsg_ctx* ctx) { return ctx ? ctx->step_1block : -1; }

int adsg_ctx_step_graphs(const adsg_ctx* ctx) { return ctx ? ctx->step_graphs_on : -1; }

int adsg_ctx_stage_work(const adsg_ctx* ctx, double* flops, double* bytes) {
    if (!ctx) return fail(-1, "ctx is NULL");
    if (!flops) return fail(-2, "flops is NULL");
    if (!bytes) return fail(-3, "bytes is NULL");
    for (int i = 0; i < ADSG_NSTAGES; ++i) flops[i] = bytes[i] = 0.0;
    const double total = static_cast<double>(ctx->size);
    // FP64 operations of the algorithm each step kernel implements (the
    // step's view, sdims), each counted as 2 flops: an add or a multiply
    // takes a DFMA issue slot like an FMA, so the rate compares with the
    // DGEMM roof as pipe utilisation.
    const dim_dev* S = ctx->sdims;
    // one band pass along direction d with `outs` outputs and `ins` inputs:
    // full band rows take ins*outs... FMAs per in-band term; symmetric rows
    // (two outputs) take the pair-sum form
    auto pass_ops = [&](int d, int products, bool pair_form) {
        const int n = S[d].n, p = S[d].p;
        const int lo = std::max(S[d].sym_lo, p), hi = std::min(S[d].sym_hi, n - p);
        double ops = 0.0;
        for (int r = 0; r < n; ++r) {
            const int inband = std::min(n - 1, r + p) - std::max(0, r - p) + 1;
            if (pair_form && r >= lo && r < hi)
                ops += products == 2 ? 3.0 * p + 2 : 5.0 * p + 3;  // p (2p) adds, 2 (3) centre terms, 2p (3p) FMAs
            else
                ops += static_cast<double>(products) * inband;
        }
        return ops / n * total;  // rows are equally populated
    };
    if (ctx->ndim == 3) {
        flops[ADSG_STAGE_RHS_OUTER] = 2.0 * pass_ops(2, 2, true);  // Mz, Nz
        bytes[ADSG_STAGE_RHS_OUTER] = 8.0 * total * 3;
        flops[ADSG_STAGE_RHS_MIDDLE] = 2.0 * pass_ops(1, 3, true);  // -dtKy, My (F); My (G)
        bytes[ADSG_STAGE_RHS_MIDDLE] = 8.0 * total * 4;
        flops[ADSG_STAGE_RHS_X] = 2.0 * pass_ops(0, 2, false);
        bytes[ADSG_STAGE_RHS_X] = 8.0 * total * 3;
    } else if (ctx->ndim == 2) {
        flops[ADSG_STAGE_RHS_OUTER] = 2.0 * pass_ops(1, 2, true);
        bytes[ADSG_STAGE_RHS_OUTER] = 8.0 * total * 3;
        flops[ADSG_STAGE_RHS_X] = 2.0 * pass_ops(0, 2, false);
        bytes[ADSG_STAGE_RHS_X] = 8.0 * total * 3;
    } else {
        flops[ADSG_STAGE_RHS_X] = 2.0 * pass_ops(0, 1, false);
        bytes[ADSG_STAGE_RHS_X] = 8.0 * total * 2;
    }
    for (int d = 0; d < ctx->ndim; ++d) {
        const dim_dev& D = S[d];
        const int n = D.n;
        const double lines = total / n;
        double ops = 0.0;
        if (solve_variant_twisted(D.solve_variant) && D.tw_k > 0) {
            // two chains: forward min(k, nc-1-j) FMAs, backward min(k, j) FMAs
            // (+1 multiply unless unit-diagonal), 2k^2 FMAs each at the meeting
            const int k = D.tw_k;
            for (int nc : {D.tw_n1, D.tw_n2}) {
                for (int j = 0; j < nc; ++j) ops += std::min(k, nc - 1 - j) + std::min(k, j) + (D.tw_unit ? 0 : 1);
                ops += 2.0 * k * k;
            }
        } else {
            // LAPACK order: forward sum_j min(kl, n-1-j) FMAs, backward sum_j
            // (uext_j FMAs + 1 multiply)
            for (int j = 0; j + 1 < n; ++j) ops += std::min(D.kl, n - 1 - j);
            ops += ctx->uext_sum[d] + n;
        }
        flops[ADSG_STAGE_SOLVE_X + d] = 2.0 * lines * ops;
        bytes[ADSG_STAGE_SOLVE_X + d] = 16.0 * total;
    }
    {
        // element quadrature: sum-factorised contractions per element (3D/2D, p = q - 1)
        const int nd = ctx->ndim;
        if (nd >= 2) {
            const double n = ctx->dims[0].p + 1, q = ctx->dims[0].q;
            double elems = 1;
            for (int d = 0; d < nd; ++d) elems *= ctx->dims[d].elements;
            double f;
            if (nd == 3)
                f = 2 * (2 * n * n * q * n + 3 * n * q * q * n + 4 * q * q * q * n + 4 * n * q * q * q +
                         3 * n * n * q * q + 2 * n * n * n * q) +
                    6 * q * q * q;
            else
                f = 2 * (2 * n * q * n + 3 * q * q * n + 3 * n * q * q + 2 * n * n * q) + 5 * q * q;
            flops[ADSG_STAGE_RHS_ELEM] = elems * f;
            bytes[ADSG_STAGE_RHS_ELEM] = 16.0 * total;
        }
    }
    // fused x pass + x solve: both works, the pass's inputs and the solved output
    flops[ADSG_STAGE_RHS_SOLVE_X] = flops[ADSG_STAGE_RHS_X] + flops[ADSG_STAGE_SOLVE_X];
    bytes[ADSG_STAGE_RHS_SOLVE_X] = bytes[ADSG_STAGE_RHS_X];
    // one-block step: the whole step's work, the state read and written once
    flops[ADSG_STAGE_STEP_1BLOCK] = flops[ADSG_STAGE_RHS_OUTER] + flops[ADSG_STAGE_RHS_MIDDLE] +
                                    flops[ADSG_STAGE_RHS_X] + flops[ADSG_STAGE_SOLVE_X] + flops[ADSG_STAGE_SOLVE_Y] +
                                    flops[ADSG_STAGE_SOLVE_Z];
    bytes[ADSG_STAGE_STEP_1BLOCK] = 16.0 * total;
    return 0;
}

int adsg_ctx_step_cluster(const adsg_ctx* ctx) {
    if (!ctx) return -1;
    return ctx->step_1block && ctx->step_cluster && step_1block_ok(ctx) ? 1 : 0;
}

int adsg_heat_steps_host(adsg_ctx* ctx, double* u_host, double dt, int nsteps) {
    if (!ctx) return fail(-1, "ctx is NULL");
    if (!u_host) return fail(-2, "u is NULL");
    if (!std::isfinite(dt)) return fail(-3, "dt must be finite");
    if (nsteps < 0) return fail(-4, "nsteps must be >= 0");
    if (nsteps == 0) return 0;
    if (!ctx->host_io) ADSG_CUDA_TRY(ctx->arena.alloc(&ctx->host_io, ctx->size), "io alloc");
    const size_t bytes = sizeof(double) * ctx->size;
    if (ctx->ndim >= 2) {
        int st = heat_steps_host_graph(ctx, u_host, dt, nsteps);
        if (st) return st;
        ADSG_CUDA_TRY(cudaStreamSynchronize(ctx->stream), "synchronize");
        return 0;
    }
    ADSG_CUDA_TRY(cudaMemcpyAsync(ctx->host_io, u_host, bytes, cudaMemcpyHostToDevice, ctx->stream), "H2D");
    int st = adsg_heat_steps(ctx, ctx->host_io, dt, nsteps);
    if (st) return st;
    ADSG_CUDA_TRY(cudaMemcpyAsync(u_host, ctx->host_io, bytes, cudaMemcpyDeviceToHost, ctx->stream), "D2H");
    ADSG_CUDA_TRY(cudaStreamSynchronize(ctx->stream), "synchronize");
    return 0;
}

int adsg_ads_solve_host(adsg_ctx* ctx, double* rhs_host) {
    if (!ctx) return fail(-1, "ctx is NULL");
    if (!rhs_host) return fail(-2, "rhs is NULL");
    if (!ctx->host_io) ADSG_CUDA_TRY(ctx->arena.alloc(&ctx->host_io, ctx->size), "io alloc");
    const size_t bytes = sizeof(double) * ctx->size;
    ADSG_CUDA_TRY(cudaMemcpyAsync(ctx->host_io, rhs_host, bytes, cudaMemcpyHostToDevice, ctx->stream), "H2D");
    int st = enqueue_solve(ctx, ctx->host_io, 0);
    if (st) return st;
    ADSG_CUDA_TRY(cudaMemcpyAsync(rhs_host, ctx->host_io, bytes, cudaMemcpyDeviceToHost, ctx->stream), "D2H");
    ADSG_CUDA_TRY(cudaStreamSynchronize(ctx->stream), "synchronize");
    return 0;
}

int adsg_heat_rhs_host(adsg_ctx* ctx, const double* u_prev_host, double* rhs_host, double dt) {
    if (!ctx) return fail(-1, "ctx is NULL");
    if (!u_prev_host) return fail(-2, "u_prev is NULL");
    if (!rhs_host) return fail(-3, "rhs is NULL");
    if (!ctx->host_io) ADSG_CUDA_TRY(ctx->arena.alloc(&ctx->host_io, ctx->size), "io alloc");
    const size_t bytes = sizeof(double) * ctx->size;
    ADSG_CUDA_TRY(cudaMemcpyAsync(ctx->host_io, u_prev_host, bytes, cudaMemcpyHostToDevice, ctx->stream), "H2D");
    int st = enqueue_rhs(ctx, ctx->host_io, ctx->ping, dt);
    if (st) return st;
    ADSG_CUDA_TRY(cudaMemcpyAsync(rhs_host, ctx->ping, bytes, cudaMemcpyDeviceToHost, ctx->stream), "D2H");
    ADSG_CUDA_TRY(cudaStreamSynchronize(ctx->stream), "synchronize");
    return 0;
}

int adsg_dgbtrs_(const char* trans, const int* n, const int* kl, const int* ku, const int* nrhs, const double* ab,
                 const int* ldab, const int* ipiv, double* b, const int* ldb, int* info) {
    // info as LAPACK defines it for a bad argument (-k = k-th argument).  Where
    // b is left unsolved for any other reason, info is positive as well, so a
    // caller that reads only info sees the failure: the 1-based column of a
    // zero U diagonal (dgbtrf's meaning of a positive info), or n + 1 when the
    // GPU solve could not run (band too wide, CUDA failure).  The message is
    // also written to stderr, as LAPACK's xerbla does.
    const int n_unsolved = (n ? *n : 0) + 1;
    auto ret = [&](int code, const char* msg, int pos_info = -1) {
        const int v = code < 0 ? code : (pos_info > 0 ? pos_info : n_unsolved);
        if (info) *info = v;
        std::fprintf(stderr, "adsg_dgbtrs_: %s (info %d)\n", msg, v);
        return fail(code, msg);
    };
    if (!trans) return ret(-1, "trans is NULL");
    const char t = *trans;
    const bool tr = (t == 'T' || t == 't' || t == 'C' || t == 'c');
    if (!tr && t != 'N' && t != 'n') return ret(-1, "trans must be N or T");
    if (!n || *n < 0) return ret(-2, "n < 0");
    if (!kl || *kl < 0) return ret(-3, "kl < 0");
    if (!ku || *ku < 0) return ret(-4, "ku < 0");
    if (!nrhs || *nrhs < 0) return ret(-5, "nrhs < 0");
    if (!ldab || *ldab < 2 * *kl + *ku + 1) return ret(-7, "ldab < 2*kl+ku+1");
    if (!ldb || *ldb < std::max(1, *n)) return ret(-10, "ldb < max(1, n)");
    if (!ab) return ret(-6, "ab is NULL");
    if (!ipiv) return ret(-8, "ipiv is NULL");
    if (!b) return ret(-9, "b is NULL");
    if (*kl > 16 || *kl + *ku > 32) return ret(ADSG_ERR_UNSUPPORTED, "band wider than kl=16, kl+ku=32");
    if (info) *info = 0;
    if (*n == 0 || *nrhs == 0) return 0;
    for (int j = 0; j < *n; ++j)
        if (ipiv[j] < j + 1 || ipiv[j] > std::min(*n, j + 1 + *kl)) return ret(-8, "pivot outside the band of a dgbtrf factorisation");
    for (int j = 0; j < *n; ++j)
        if (ab[static_cast<size_t>(j) * *ldab + *kl + *ku] == 0.0) return ret(ADSG_ERR_SINGULAR, "zero diagonal in U", j + 1);
    solve_tables tb;
    if (make_solve_tables(*n, *kl, *ku, *ldab, ab, ipiv, tb)) return ret(ADSG_ERR_SINGULAR, "zero diagonal in U");

    cudaStream_t s = nullptr;
    ADSG_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "stream");
    dev_arena ar;
    dim_dev D;
    D.n = *n;
    D.kl = tb.kl;
    D.w = tb.w;
    D.ku_regular = *ku;
    D.fwd_fast = tb.fwd_fast;
    D.bwd_fast = tb.bwd_fast;
    double *lmul, *ucol, *rdiag, *x;
    int *piv, *uext;
    cudaError_t e = cudaSuccess;
    const size_t cols = static_cast<size_t>(*nrhs);
    const size_t n_ = static_cast<size_t>(*n);
    if (e == cudaSuccess) e = ar.upload(&lmul, tb.lmul.data(), tb.lmul.size(), s);
    if (e == cudaSuccess) e = ar.upload(&ucol, tb.ucol.data(), tb.ucol.size(), s);
    if (e == cudaSuccess) e = ar.upload(&rdiag, tb.rdiag.data(), tb.rdiag.size(), s);
    if (e == cudaSuccess) e = ar.upload(&piv, tb.piv.data(), tb.piv.size(), s);
    if (e == cudaSuccess) e = ar.upload(&uext, tb.uext.data(), tb.uext.size(), s);
    if (e == cudaSuccess) e = ar.alloc(&x, n_ * cols);
    // gather the columns densely (ldb may exceed n)
    if (e == cudaSuccess)
        e = cudaMemcpy2DAsync(x, n_ * sizeof(double), b, static_cast<size_t>(*ldb) * sizeof(double), n_ * sizeof(double),
                              cols, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        D.lmul = lmul;
        D.ucol = ucol;
        D.rdiag = rdiag;
        D.piv = piv;
        D.uext = uext;
        int nn = *n;
        line_layout L;
        L.nlines = static_cast<long long>(cols);
        L.a = L.nlines;
        L.sa = nn;
        L.contiguous = 1;
        L.total = L.nlines * nn;
        e = launch_line_solve(x, D, L, tr ? 1 : 0, s);
    }
    if (e == cudaSuccess)
        e = cudaMemcpy2DAsync(b, static_cast<size_t>(*ldb) * sizeof(double), x, n_ * sizeof(double), n_ * sizeof(double),
                              cols, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
    if (e != cudaSuccess) {
        if (info) *info = n_unsolved;
        std::fprintf(stderr, "adsg_dgbtrs_: CUDA failure: %s (info %d)\n", cudaGetErrorString(e), n_unsolved);
        return fail_cuda(e, "dgbtrs");
    }
    return 0;
}

int adsg_test_fail_device_alloc(int k) { return g_alloc_fail_in.exchange(k < 0 ? -1 : k); }

int adsg_debug_bounds(long long* violations, int* file, int* line, long long* index, long long* extent, int reset) {
    if (!violations) return fail(-1, "violations is NULL");
    if (!ADSG_BOUNDS_CHECK) return fail(ADSG_ERR_UNSUPPORTED, "not the bounds-checked build (ADSG_BOUNDS_CHECK)");
    {
        const cudaError_t e = cudaDeviceSynchronize();  // every kernel's records are complete
        if (e != cudaSuccess) return fail_cuda(e, "synchronize before reading the bounds records");
    }
    bounds_record r[3] = {};
    const int st[3] = {bounds_read_kernels(&r[0], 0), bounds_read_elem(&r[1], 0), bounds_read_quad(&r[2], 0)};
    for (int k = 0; k < 3; ++k) {
        if (st[k] == 0) return fail(ADSG_ERR_UNSUPPORTED, "not the bounds-checked build (ADSG_BOUNDS_CHECK)");
        if (st[k] < 0) return fail_cuda(static_cast<cudaError_t>(-st[k]), "read the bounds records");
    }
    *violations = 0;
    int first = -1;
    for (int k = 0; k < 3; ++k) {
        *violations += static_cast<long long>(r[k].count);
        if (first < 0 && r[k].count) first = k;
    }
    if (file) *file = first;
    if (line) *line = first >= 0 ? r[first].line : 0;
    if (index) *index = first >= 0 ? r[first].index : 0;
    if (extent) *extent = first >= 0 ? r[first].extent : 0;
    if (reset) {
        bounds_record tmp;
        bounds_read_kernels(&tmp, 1);
        bounds_read_elem(&tmp, 1);
        bounds_read_quad(&tmp, 1);
    }
    return 0;
}

int adsg_dgbtrs_checked_(const char* trans, const int* n, const int* kl, const int* ku, const int* nrhs,
                         const double* ab, const int* ldab, const int* ipiv, double* b, const int* ldb, int* info) {
    int local = 0;
    int* ip = info ? info : &local;
    const int rc = adsg_dgbtrs_(trans, n, kl, ku, nrhs, ab, ldab, ipiv, b, ldb, ip);
    if (rc != 0 || *ip != 0) {
        std::fprintf(stderr, "adsg_dgbtrs_checked_: the right-hand sides were not solved (info %d, %s); aborting\n", *ip,
                     adsg_last_error());
        std::abort();
    }
    return 0;
}

}  // extern "C"
