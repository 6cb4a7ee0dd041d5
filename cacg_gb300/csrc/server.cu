// server.cu -- persistent request loop for SPD solves (no reference
// counterpart: sclc/cacg solves one system per process launch,
// src/main.c:22-221).
//
// Continuous batching on one GPU (the default, CACG_SERVER_BATCHED):
//   * submit() copies the request (CSR, RHS block, params) and queues it;
//   * one engine thread admits queued requests whenever their device
//     footprint fits in what the memory budget has left and a slot is free:
//     first fit in arrival order, so a large request at the head does not
//     block smaller ones behind it (a request passed over 16 times blocks
//     further admissions until it fits, so it cannot starve);
//   * every engine step advances ALL admitted requests by one outer
//     iteration: each phase (basis steps, Gram products, LU, Q update, A Q,
//     X/R update) is one launch per precision class over every request's
//     tiles (k_batch.cu), and the step's launch sequence is captured once in
//     a CUDA graph per batch shape (which classes are present, longest basis)
//     and replayed: the host only rewrites the pinned descriptor block the
//     graph's first copy reads;
//   * requests join and leave between steps (iteration-level batching);
//     convergence checks, residual replacements and final residuals are
//     batched the same way;
//   * the grid size of each batched kernel is chosen by a measurement-driven
//     autotuner (once per device and class), and never changes a result:
//     a request's iterates are bit-identical alone and in any mix.
// Requests outside the batched kernels' limits (k = s m > 64, m > 32,
// s > 16, Lanczos bounds, block CG) and large requests (more rows than
// batch_max_rows: their phases are long enough to keep the GPU busy alone,
// and the single-request solver's DIA / tensor-core kernels stream them at a
// higher fraction of HBM than the generic batched kernels) run on per-request
// stream workers; CACG_SERVER_STREAMS sends every request there (the
// previous design, kept for comparison).  max_active bounds the requests in
// flight on both paths together.
//
// Stream priorities: small requests (the engine's stream, or a stream worker
// serving a request of at most batch_max_rows rows) run at the device's
// highest priority and large ones at its lowest, so the CTAs of a small
// request's short kernels are scheduled ahead of the pending CTAs of a large
// request's long ones.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <tuple>
#include <vector>

#include "batch.h"
#include "cacg_internal.cuh"
#include "cacg_solver.h"

namespace cacg {

struct Request {
    int64_t ticket;
    int64_t n, nnz;
    int m;
    std::vector<int32_t> rp, ci;
    std::vector<double> val, B;
    cacg_params p;
    double *X_out;
    size_t cost;
    bool batched = false;
    int skips = 0;  // admissions that passed this request over
    int state = 0;  // 0 queued, 1 running, 2 done
    int status = CACG_PENDING;
    cacg_result res{};
    std::vector<double> relres;
};

static double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

// ------------------------------------------------- batched request layout
static size_t a256(size_t b) { return (b + 255) & ~size_t(255); }

struct BLayout {
    size_t rp, ci, val, val32, B, X, R, R32, S, Q, AQ, small, gpart, npart, gws, total;
};

static BLayout blayout(int64_t n, int64_t nnz, int m, int s, bool f32) {
    const int k = s * m;
    const size_t es = f32 ? 4 : 8;
    const int pr = bpiece_rows(f32);
    const int64_t ntile = (n + kBRows - 1) / kBRows, npiece = (n + pr - 1) / pr;
    BLayout L{};
    size_t o = 0;
    auto put = [&](size_t &field, size_t bytes) {
        field = o;
        o += a256(bytes);
    };
    put(L.rp, (size_t)(n + 1) * 4);
    put(L.ci, (size_t)std::max<int64_t>(nnz, 1) * 4);
    put(L.val, (size_t)std::max<int64_t>(nnz, 1) * 8);
    put(L.val32, f32 ? (size_t)std::max<int64_t>(nnz, 1) * 4 : 0);
    put(L.B, (size_t)n * m * 8);
    put(L.X, (size_t)n * m * 8);
    put(L.R, (size_t)n * m * 8);
    put(L.R32, f32 ? (size_t)n * m * 4 : 0);
    put(L.S, (size_t)n * k * es);
    put(L.Q, (size_t)n * k * es);
    put(L.AQ, (size_t)n * k * es);
    // QtAS, QtAQ, beta k x k; F 2 k x k + k; QtR, alpha k x m; bounds 2
    put(L.small, sizeof(double) * ((size_t)5 * k * k + k + (size_t)2 * k * m + 2));
    put(L.gpart, sizeof(double) * (size_t)npiece * k * (k + m));
    put(L.npart, sizeof(double) * (size_t)ntile * m);
    put(L.gws, sizeof(double) * 2 * 320);  // Gerschgorin partials
    L.total = o;
    return L;
}

static bool batch_eligible(const cacg_params &p, int m) {
    return p.algorithm == CACG_ALG_CACG && p.s >= 2 && p.s <= kBMaxS && m >= 1 &&
           m <= kBMaxM && p.s * m <= kBMaxK &&
           (p.bounds_mode == CACG_BOUNDS_GERSCHGORIN || p.bounds_mode == CACG_BOUNDS_GIVEN) &&
           (p.precision == CACG_FP64 || p.precision == CACG_MIXED) && p.maxit >= 0;
}

// ----------------------------------------------------------- autotuner
// Per device and class: blocks per SM of each batched kernel kind, measured
// on a synthetic batch (eight 2-D Laplacians of 36,864 rows, 8 RHS, s = 4)
// and kept for the process.  The grid size never changes results.
static std::mutex g_tune_mu;
static std::map<std::pair<int, int>, BTune> g_tunes;

struct Engine;

// ------------------------------------------------------------- server
struct Server {
    cacg_server_config cfg;
    int device = 0;
    std::mutex mu;
    std::condition_variable cv_work, cv_done, cv_engine;
    std::deque<std::shared_ptr<Request>> queue;   // batched engine
    std::deque<std::shared_ptr<Request>> lqueue;  // per-request stream workers
    std::map<int64_t, std::shared_ptr<Request>> all;
    int64_t next_ticket = 1;
    int64_t bytes_in_use = 0;
    int64_t active = 0;
    bool stop = false;
    std::vector<std::thread> workers;
    std::thread engine_thread;
    std::unique_ptr<Engine> engine;
    std::atomic<int64_t> engine_steps{0}, engine_graph_replays{0};

    int64_t small_rows() const {
        return cfg.batch_max_rows == 0 ? 65536
               : cfg.batch_max_rows < 0 ? INT64_MAX
                                        : (int64_t)cfg.batch_max_rows;
    }

    void finish_request(Request *r, int status) {
        {
            std::lock_guard<std::mutex> lk(mu);
            bytes_in_use -= (int64_t)r->cost;
            active--;
            r->status = status;
            r->res.status = status;
            r->state = 2;
            std::vector<int32_t>().swap(r->rp);
            std::vector<int32_t>().swap(r->ci);
            std::vector<double>().swap(r->val);
            std::vector<double>().swap(r->B);
        }
        cv_done.notify_all();
        cv_work.notify_all();
        cv_engine.notify_all();
    }

    // ---------------------------------------- per-request stream workers
    void worker() {
        cudaSetDevice(device);
        int lo = 0, hi = 0;
        cudaDeviceGetStreamPriorityRange(&lo, &hi);
        cudaStream_t st_small, st_large;
        cudaStreamCreateWithPriority(&st_small, cudaStreamNonBlocking, hi);
        cudaStreamCreateWithPriority(&st_large, cudaStreamNonBlocking, lo);
        for (;;) {
            std::shared_ptr<Request> r;
            {
                std::unique_lock<std::mutex> lk(mu);
                cv_work.wait(lk, [&] {
                    return stop || (!lqueue.empty() &&
                                    bytes_in_use + (int64_t)lqueue.front()->cost <=
                                        cfg.mem_budget_bytes &&
                                    active < cfg.max_active);
                });
                if (stop) break;
                r = lqueue.front();
                lqueue.pop_front();
                bytes_in_use += (int64_t)r->cost;
                active++;
                r->state = 1;
            }
            const int rc = run_one(r.get(), r->n <= small_rows() ? st_small : st_large);
            finish_request(r.get(), rc);
        }
        cudaStreamDestroy(st_small);
        cudaStreamDestroy(st_large);
    }

    int run_one(Request *r, cudaStream_t st) {
        const double t0 = now_s();
        const int64_t l0 = g_launches.load();
        cacg_csr A{r->n, r->nnz, r->rp.data(), r->ci.data(), r->val.data()};
        DevMatrix M;
        int rc = DevMatrix::create(&A, r->p.precision == CACG_MIXED, &M, st);
        size_t bx = (size_t)r->n * r->m * sizeof(double);
        size_t wsb = solve_workspace_bytes(r->n, r->m, r->p.s, r->p.precision,
                                           r->p.bounds_mode == CACG_BOUNDS_LANCZOS);
        double *dB = nullptr, *dX = nullptr;
        void *ws = nullptr;
        if (rc == CACG_OK && cudaMallocAsync((void **)&dB, bx, st) != cudaSuccess) rc = CACG_ERR_OOM;
        if (rc == CACG_OK && cudaMallocAsync((void **)&dX, bx, st) != cudaSuccess) rc = CACG_ERR_OOM;
        if (rc == CACG_OK && cudaMallocAsync(&ws, wsb, st) != cudaSuccess) rc = CACG_ERR_OOM;
        if (rc == CACG_OK) {
            cudaMemcpyAsync(dB, r->B.data(), bx, cudaMemcpyHostToDevice, st);
            cudaMemsetAsync(dX, 0, bx, st);
            cacg_params p = r->p;
            p.stream = st;
            r->relres.assign(r->m, 0.0);
            r->res.true_relres = r->relres.data();
            rc = solve_on_device(&M, dB, dX, r->m, &p, &r->res, ws, wsb);
            if (rc >= 0 || rc == CACG_ERR_BREAKDOWN) {
                if (cudaMemcpyAsync(r->X_out, dX, bx, cudaMemcpyDeviceToHost, st) != cudaSuccess)
                    rc = CACG_ERR_CUDA;
            }
        }
        if (dB) cudaFreeAsync(dB, st);
        if (dX) cudaFreeAsync(dX, st);
        if (ws) cudaFreeAsync(ws, st);
        cudaStreamSynchronize(st);
        M.release();
        cudaGetLastError();
        r->res.seconds = now_s() - t0;
        r->res.launches = g_launches.load() - l0;
        return rc;
    }

    void engine_main();
};

// ------------------------------------------------------------- engine
struct BSlot {
    std::shared_ptr<Request> req;
    int cls = 0;  // 0: FP64, 1: FP32 (mixed)
    char *mem = nullptr;
    BLayout L{};
    BDesc d{};
    double *bounds = nullptr;  // device, 2 doubles
    double *gws = nullptr;
    double bn[kBMaxM];
    int since_rr = 0;
    bool resid = false;        // in the next residual launch
    bool r_true = false;       // R holds B - A X for the current X
    bool done = false;
    int final_status = CACG_OK;
    double t_admit = 0;
    int64_t l_admit = 0;
};

struct Engine {
    Server *srv;
    cudaStream_t st = nullptr;
    BBatch *h_b[2] = {nullptr, nullptr}, *d_b[2] = {nullptr, nullptr};
    double *h_norms = nullptr, *d_norms = nullptr;  // [2][kBMax][kBMaxM]
    int *h_status = nullptr, *d_status = nullptr;   // [2][kBMax]
    BTune tune[2];
    bool tuned[2] = {false, false};
    std::vector<std::unique_ptr<BSlot>> slots[2];
    bool graphs = true;
    struct G {
        cudaGraphExec_t exec = nullptr;
        int64_t kernels = 0;
    };
    std::map<std::tuple<int, int>, G> gcache;  // (longest basis FP64, FP32; 0 = class absent)

    ~Engine() {
        for (auto &pm : marks) {
            cudaEventDestroy(pm.a);
            cudaEventDestroy(pm.b);
        }
        for (auto e : event_pool) cudaEventDestroy(e);
        for (auto &kv : gcache)
            if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
        for (int c = 0; c < 2; ++c)
            for (auto &s : slots[c])
                if (s->mem) cudaFreeAsync(s->mem, st);
        if (st) cudaStreamSynchronize(st);
        for (int c = 0; c < 2; ++c) {
            if (h_b[c]) cudaFreeHost(h_b[c]);
            if (d_b[c]) cudaFree(d_b[c]);
        }
        if (h_norms) cudaFreeHost(h_norms);
        if (d_norms) cudaFree(d_norms);
        if (h_status) cudaFreeHost(h_status);
        if (d_status) cudaFree(d_status);
        if (st) cudaStreamDestroy(st);
        cudaGetLastError();
    }

    int init() {
        int lo = 0, hi = 0;
        cudaDeviceGetStreamPriorityRange(&lo, &hi);
        if (cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, hi) != cudaSuccess)
            return CACG_ERR_CUDA;
        for (int c = 0; c < 2; ++c) {
            if (cudaMallocHost((void **)&h_b[c], sizeof(BBatch)) != cudaSuccess ||
                cudaMalloc((void **)&d_b[c], sizeof(BBatch)) != cudaSuccess)
                return CACG_ERR_OOM;
            memset(h_b[c], 0, sizeof(BBatch));
        }
        const size_t nb = sizeof(double) * 2 * kBMax * kBMaxM, sb = sizeof(int) * 2 * kBMax;
        if (cudaMallocHost((void **)&h_norms, nb) != cudaSuccess ||
            cudaMalloc((void **)&d_norms, nb) != cudaSuccess ||
            cudaMallocHost((void **)&h_status, sb) != cudaSuccess ||
            cudaMalloc((void **)&d_status, sb) != cudaSuccess)
            return CACG_ERR_OOM;
        cudaMemset(d_status, 0, sb);
        return cudaDeviceSynchronize() == cudaSuccess ? CACG_OK : CACG_ERR_CUDA;
    }

    double *norms_of(int cls, int pos) { return d_norms + ((size_t)cls * kBMax + pos) * kBMaxM; }
    double *hnorms_of(int cls, int pos) { return h_norms + ((size_t)cls * kBMax + pos) * kBMaxM; }

    // the class's descriptor block: every slot, flags per `flag_of`
    template <class F>
    int fill_batch(int cls, F &&flag_of) {
        BBatch *b = h_b[cls];
        const int nr = (int)slots[cls].size();
        b->nr = nr;
        int tiles = 0, pieces = 0;
        for (int i = 0; i < nr; ++i) {
            BSlot &s = *slots[cls][i];
            b->tile_start[i] = tiles;
            b->piece_start[i] = pieces;
            tiles += s.d.ntile;
            pieces += s.d.npiece;
            b->d[i] = s.d;
            b->d[i].norms = norms_of(cls, i);
            b->d[i].status = d_status + cls * kBMax + i;
            b->d[i].flags = flag_of(s);
        }
        b->tile_start[nr] = tiles;
        b->piece_start[nr] = pieces;
        b->total_tiles = tiles;
        b->total_pieces = pieces;
        return nr;
    }

    int smax(int cls) {
        int v = 0;
        for (auto &s : slots[cls]) v = std::max(v, s->d.s);
        return v;
    }

    // phase timing of direct (not graph-replayed) steps while the profiler is
    // on: events around each phase, read after the step's synchronisation
    struct PhaseMark {
        int phase;
        cudaEvent_t a, b;
    };
    std::vector<PhaseMark> marks;
    std::vector<cudaEvent_t> event_pool;
    bool timing = false;
    cudaEvent_t ev() {
        if (!event_pool.empty()) {
            cudaEvent_t e = event_pool.back();
            event_pool.pop_back();
            return e;
        }
        cudaEvent_t e;
        cudaEventCreate(&e);
        return e;
    }
    template <class F>
    int timed(int phase, F &&f) {
        if (!timing) return f();
        PhaseMark pm{phase, ev(), ev()};
        cudaEventRecord(pm.a, st);
        const int rc = f();
        cudaEventRecord(pm.b, st);
        marks.push_back(pm);
        return rc;
    }
    void harvest_marks() {
        for (auto &pm : marks) {
            float ms = 0.f;
            if (cudaEventElapsedTime(&ms, pm.a, pm.b) == cudaSuccess)
                profile_accumulate(pm.phase, ms, 0);
            cudaGetLastError();
            event_pool.push_back(pm.a);
            event_pool.push_back(pm.b);
        }
        marks.clear();
    }

    // one outer iteration of every slot of class `cls` (T: its precision)
    template <typename T>
    int iteration_launches(int cls, int sm) {
        const BBatch *b = d_b[cls];
        const BTune &tu = tune[cls];
        int rc = CACG_OK;
        for (int j = 1; j < sm && rc == CACG_OK; ++j)
            rc = timed(CACG_PHASE_BASIS, [&] { return bl_basis_step<T>(st, b, j, tu); });
        if (rc == CACG_OK) rc = timed(CACG_PHASE_GRAM, [&] { return bl_gram<T>(st, b, 0, tu); });
        if (rc == CACG_OK) rc = timed(CACG_PHASE_LU, [&] { return bl_lu_solve(st, b, 0); });
        if (rc == CACG_OK) rc = timed(CACG_PHASE_QUPDATE, [&] { return bl_qupdate<T>(st, b, tu); });
        if (rc == CACG_OK) rc = timed(CACG_PHASE_AQ, [&] { return bl_aq<T>(st, b, tu); });
        if (rc == CACG_OK) rc = timed(CACG_PHASE_GRAM, [&] { return bl_gram<T>(st, b, 1, tu); });
        if (rc == CACG_OK) rc = timed(CACG_PHASE_LU, [&] { return bl_lu_factor(st, b); });
        if (rc == CACG_OK) rc = timed(CACG_PHASE_LU, [&] { return bl_lu_solve(st, b, 1); });
        if (rc == CACG_OK) rc = timed(CACG_PHASE_XRUPDATE, [&] { return bl_xrupdate<T>(st, b, tu); });
        return rc;
    }

    int step_launches(int sm0, int sm1) {
        int rc = CACG_OK;
        for (int c = 0; c < 2 && rc == CACG_OK; ++c) {
            if ((c == 0 ? sm0 : sm1) == 0) continue;
            if (cudaMemcpyAsync(d_b[c], h_b[c], sizeof(BBatch), cudaMemcpyHostToDevice, st) !=
                cudaSuccess)
                rc = CACG_ERR_CUDA;
        }
        if (rc == CACG_OK && cudaMemsetAsync(d_status, 0, sizeof(int) * 2 * kBMax, st) != cudaSuccess)
            rc = CACG_ERR_CUDA;
        if (rc == CACG_OK && sm0) rc = iteration_launches<double>(0, sm0);
        if (rc == CACG_OK && sm1) rc = iteration_launches<float>(1, sm1);
        if (rc == CACG_OK &&
            (cudaMemcpyAsync(h_norms, d_norms, sizeof(double) * 2 * kBMax * kBMaxM,
                             cudaMemcpyDeviceToHost, st) != cudaSuccess ||
             cudaMemcpyAsync(h_status, d_status, sizeof(int) * 2 * kBMax, cudaMemcpyDeviceToHost,
                             st) != cudaSuccess))
            rc = CACG_ERR_CUDA;
        return rc;
    }

    // one engine step: every slot advances one outer iteration
    int step() {
        for (int c = 0; c < 2; ++c) fill_batch(c, [](BSlot &) { return kBActive; });
        const int sm0 = slots[0].empty() ? 0 : smax(0), sm1 = slots[1].empty() ? 0 : smax(1);
        int rc;
        if (graphs) {
            G &g = gcache[std::make_tuple(sm0, sm1)];
            if (!g.exec) {
                const int64_t l0 = g_launches.load();
                if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
                    return CACG_ERR_CUDA;
                rc = step_launches(sm0, sm1);
                cudaGraph_t gr = nullptr;
                const cudaError_t e = cudaStreamEndCapture(st, &gr);
                g.kernels = g_launches.load() - l0;
                g_launches -= g.kernels;
                if (rc != CACG_OK || e != cudaSuccess || !gr) {
                    if (gr) cudaGraphDestroy(gr);
                    cudaGetLastError();
                    return rc != CACG_OK ? rc : CACG_ERR_CUDA;
                }
                const cudaError_t ei = cudaGraphInstantiate(&g.exec, gr, 0);
                cudaGraphDestroy(gr);
                if (ei != cudaSuccess) {
                    g.exec = nullptr;
                    cudaGetLastError();
                    return CACG_ERR_CUDA;
                }
            }
            if (cudaGraphLaunch(g.exec, st) != cudaSuccess) return CACG_ERR_CUDA;
            g_launches += g.kernels;
            srv->engine_graph_replays++;
            rc = CACG_OK;
        } else {
            timing = profile_enabled();
            rc = step_launches(sm0, sm1);
            timing = false;
        }
        if (rc != CACG_OK) return rc;
        if (cudaStreamSynchronize(st) != cudaSuccess) return CACG_ERR_CUDA;
        harvest_marks();
        srv->engine_steps++;
        return CACG_OK;
    }

    // residual launch for the slots with s.resid set; norms to h_norms
    int residual_pass() {
        bool any = false;
        for (int c = 0; c < 2; ++c) {
            bool anyc = false;
            fill_batch(c, [&](BSlot &s) {
                anyc = anyc || s.resid;
                return s.resid ? kBResid : 0;
            });
            if (!anyc) continue;
            any = true;
            if (cudaMemcpyAsync(d_b[c], h_b[c], sizeof(BBatch), cudaMemcpyHostToDevice, st) !=
                cudaSuccess)
                return CACG_ERR_CUDA;
            timing = profile_enabled();
            const int rc = timed(CACG_PHASE_RESIDUAL, [&] {
                return c == 0 ? bl_residual<double>(st, d_b[c], tune[c])
                              : bl_residual<float>(st, d_b[c], tune[c]);
            });
            timing = false;
            if (rc) return rc;
        }
        if (!any) return CACG_OK;
        if (cudaMemcpyAsync(h_norms, d_norms, sizeof(double) * 2 * kBMax * kBMaxM,
                            cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess)
            return CACG_ERR_CUDA;
        harvest_marks();
        return CACG_OK;
    }

    // ------------------------------------------------------- admission
    int setup_slot(BSlot &s) {
        Request *r = s.req.get();
        const bool f32 = r->p.precision == CACG_MIXED;
        s.cls = f32 ? 1 : 0;
        s.L = blayout(r->n, r->nnz, r->m, r->p.s, f32);
        if (cudaMallocAsync((void **)&s.mem, s.L.total, st) != cudaSuccess) {
            cudaGetLastError();
            s.mem = nullptr;
            return CACG_ERR_OOM;
        }
        char *base = s.mem;
        const int m = r->m, k = r->p.s * m;
        BDesc &d = s.d;
        memset(&d, 0, sizeof d);
        d.rp = (const int32_t *)(base + s.L.rp);
        d.ci = (const int32_t *)(base + s.L.ci);
        d.val = (const double *)(base + s.L.val);
        d.val32 = f32 ? (const float *)(base + s.L.val32) : nullptr;
        d.B = (const double *)(base + s.L.B);
        d.X = (double *)(base + s.L.X);
        d.R = (double *)(base + s.L.R);
        d.R32 = f32 ? (float *)(base + s.L.R32) : nullptr;
        d.S = base + s.L.S;
        d.Qold = base + s.L.Q;
        d.AQ = base + s.L.AQ;
        double *sm = (double *)(base + s.L.small);
        d.QtAS = sm; sm += (size_t)k * k;
        d.QtAQ = sm; sm += (size_t)k * k;
        d.beta = sm; sm += (size_t)k * k;
        d.F = sm; sm += (size_t)2 * k * k + k;
        d.QtR = sm; sm += (size_t)k * m;
        d.alpha = sm; sm += (size_t)k * m;
        s.bounds = sm;
        d.gpart = (double *)(base + s.L.gpart);
        d.npart = (double *)(base + s.L.npart);
        s.gws = (double *)(base + s.L.gws);
        d.n = r->n;
        d.m = m;
        d.s = r->p.s;
        d.k = k;
        d.it = 0;
        d.ntile = (int)((r->n + kBRows - 1) / kBRows);
        d.npiece = (int)((r->n + bpiece_rows(f32) - 1) / bpiece_rows(f32));
        const size_t bx = (size_t)r->n * m * 8;
        if (cudaMemcpyAsync((void *)d.rp, r->rp.data(), (size_t)(r->n + 1) * 4,
                            cudaMemcpyHostToDevice, st) != cudaSuccess ||
            (r->nnz > 0 && (cudaMemcpyAsync((void *)d.ci, r->ci.data(), (size_t)r->nnz * 4,
                                            cudaMemcpyHostToDevice, st) != cudaSuccess ||
                            cudaMemcpyAsync((void *)d.val, r->val.data(), (size_t)r->nnz * 8,
                                            cudaMemcpyHostToDevice, st) != cudaSuccess)) ||
            cudaMemcpyAsync((void *)d.B, r->B.data(), bx, cudaMemcpyHostToDevice, st) !=
                cudaSuccess ||
            cudaMemsetAsync(d.X, 0, bx, st) != cudaSuccess)
            return CACG_ERR_CUDA;
        if (f32 && r->nnz > 0) {
            int rc = launch_cast_f64_f32(st, r->nnz, d.val, (float *)d.val32);
            if (rc) return rc;
        }
        if (r->p.bounds_mode == CACG_BOUNDS_GERSCHGORIN) {
            int rc = launch_gerschgorin(st, r->n, d.rp, d.ci, d.val, s.bounds, s.gws);
            if (rc) return rc;
        }
        s.t_admit = now_s();
        s.l_admit = g_launches.load();
        return CACG_OK;
    }

    void tune_class(int cls);

    // admit what fits; device set-up of the new slots; R = B, ||B||
    int admit() {
        std::vector<std::unique_ptr<BSlot>> fresh;
        {
            std::lock_guard<std::mutex> lk(srv->mu);
            int64_t free_slots = srv->cfg.max_active - srv->active;
            std::vector<Request *> passed;  // earlier requests that did not fit
            for (auto it = srv->queue.begin(); it != srv->queue.end() && free_slots > 0;) {
                Request *r = it->get();
                const int cls = r->p.precision == CACG_MIXED ? 1 : 0;
                int in_cls = (int)slots[cls].size();
                for (auto &f : fresh) in_cls += f->cls == cls;
                if (srv->bytes_in_use + (int64_t)r->cost <= srv->cfg.mem_budget_bytes &&
                    in_cls < kBMax) {
                    // a request passed over 16 times holds back the ones behind it
                    bool starving = false;
                    for (Request *q : passed) starving = starving || q->skips >= 16;
                    if (starving) break;
                    for (Request *q : passed) ++q->skips;
                    auto s = std::make_unique<BSlot>();
                    s->req = *it;
                    s->cls = cls;
                    srv->bytes_in_use += (int64_t)r->cost;
                    srv->active++;
                    r->state = 1;
                    fresh.push_back(std::move(s));
                    it = srv->queue.erase(it);
                    --free_slots;
                } else {
                    passed.push_back(r);
                    ++it;
                }
            }
        }
        if (fresh.empty()) return CACG_OK;
        for (auto &s : fresh) {
            if (!tuned[s->cls]) tune_class(s->cls);
            const int rc = setup_slot(*s);
            if (rc != CACG_OK) {
                if (s->mem) cudaFreeAsync(s->mem, st);
                s->mem = nullptr;
                cudaStreamSynchronize(st);
                cudaGetLastError();
                srv->finish_request(s->req.get(), rc);
                s.reset();
            }
        }
        // bounds to the host, then R = B - A 0 and ||B(:,c)||^2
        std::vector<BSlot *> added;
        for (auto &s : fresh)
            if (s) {
                s->resid = true;
                added.push_back(s.get());
                slots[s->cls].push_back(std::move(s));
            }
        if (added.empty()) return CACG_OK;
        std::vector<double> hb(2 * added.size());
        for (size_t i = 0; i < added.size(); ++i) {
            const cacg_params &p = added[i]->req->p;
            if (p.bounds_mode == CACG_BOUNDS_GERSCHGORIN) {
                if (cudaMemcpyAsync(&hb[2 * i], added[i]->bounds, 16, cudaMemcpyDeviceToHost,
                                    st) != cudaSuccess)
                    return CACG_ERR_CUDA;
            } else {
                hb[2 * i] = p.lambda_min;
                hb[2 * i + 1] = p.lambda_max;
            }
        }
        int rc = residual_pass();  // synchronises the stream
        if (rc) return rc;
        for (size_t i = 0; i < added.size(); ++i) {
            BSlot &s = *added[i];
            s.resid = false;
            s.r_true = true;
            const double lmin = hb[2 * i], lmax = hb[2 * i + 1];
            s.req->res.lambda_min = lmin;
            s.req->res.lambda_max = lmax;
            s.d.sa = 2.0 / (lmax - lmin);             // src/bcbcgKernel.c:113
            s.d.sb = -(lmax + lmin) / (lmax - lmin);  // src/bcbcgKernel.c:114-115
            const int pos = position(s);
            const double *nr = hnorms_of(s.cls, pos);
            for (int c = 0; c < s.d.m; ++c) s.bn[c] = nr[c] > 0 ? sqrt(nr[c]) : 1.0;
            if (!(lmax > lmin)) {
                s.done = true;
                s.final_status = CACG_ERR_ARG;
            } else if (s.req->p.maxit == 0) {
                s.done = true;
                s.final_status = CACG_NOT_CONVERGED;
            }
        }
        return CACG_OK;
    }

    int position(const BSlot &s) {
        auto &v = slots[s.cls];
        for (size_t i = 0; i < v.size(); ++i)
            if (v[i].get() == &s) return (int)i;
        return -1;
    }

    // -------------------------------------------- after an engine step
    void after_step() {
        for (int c = 0; c < 2; ++c) {
            for (size_t i = 0; i < slots[c].size(); ++i) {
                BSlot &s = *slots[c][i];
                Request *r = s.req.get();
                const cacg_params &p = r->p;
                std::swap(s.d.S, s.d.Qold);  // Q is in S's buffer; the next T_0 in Q_old's
                s.d.it++;
                s.since_rr++;
                s.r_true = false;
                r->res.iterations = s.d.it;
                const double *nr = hnorms_of(c, (int)i);
                r->res.recurrence_norm0 = sqrt(std::max(nr[0], 0.0));
                if (h_status[c * kBMax + i] & kStatusBreakdown) {
                    s.done = true;
                    s.final_status = CACG_ERR_BREAKDOWN;
                    continue;
                }
                bool finite = true;
                for (int q = 0; q < s.d.m; ++q) finite = finite && std::isfinite(nr[q]);
                if (!finite) {
                    s.done = true;
                    s.final_status = CACG_ERR_BREAKDOWN;
                    continue;
                }
                const bool mixed = p.precision == CACG_MIXED;
                const bool rr_due = mixed && p.rr_period > 0 && s.since_rr >= p.rr_period;
                if (p.tol_mode == CACG_TOL_ABS_COL0) {
                    if (sqrt(nr[0]) < p.tol) {  // src/bcbcgKernel.c:524
                        s.done = true;
                        s.final_status = CACG_OK;
                        continue;
                    }
                    if (rr_due) s.resid = true;
                } else {
                    double mx = 0.0;
                    for (int q = 0; q < s.d.m; ++q) {
                        const double v = sqrt(std::max(nr[q], 0.0)) / s.bn[q];
                        if (!(v <= mx)) mx = v;
                    }
                    if (mx <= p.tol || rr_due) s.resid = true;
                }
                if (!s.resid && s.d.it >= p.maxit) {
                    s.done = true;
                    s.final_status = CACG_NOT_CONVERGED;
                }
            }
        }
    }

    // replacements and convergence checks (true residuals, FP64)
    int check_round() {
        bool any = false;
        for (int c = 0; c < 2; ++c)
            for (auto &s : slots[c]) any = any || s->resid;
        if (!any) return CACG_OK;
        int rc = residual_pass();
        if (rc) return rc;
        for (int c = 0; c < 2; ++c) {
            for (size_t i = 0; i < slots[c].size(); ++i) {
                BSlot &s = *slots[c][i];
                if (!s.resid) continue;
                s.resid = false;
                s.r_true = true;
                s.since_rr = 0;
                Request *r = s.req.get();
                r->res.residual_replacements++;
                const double *nr = hnorms_of(c, (int)i);
                double mx = 0.0;
                for (int q = 0; q < s.d.m; ++q) {
                    const double v = sqrt(std::max(nr[q], 0.0)) / s.bn[q];
                    if (!(v <= mx)) mx = v;
                }
                if (r->p.tol_mode == CACG_TOL_REL_ALL && mx <= r->p.tol) {
                    s.done = true;
                    s.final_status = CACG_OK;
                } else if (s.d.it >= r->p.maxit) {
                    s.done = true;
                    s.final_status = CACG_NOT_CONVERGED;
                }
            }
        }
        return CACG_OK;
    }

    // final true residuals, X to the caller, slots released
    int retire() {
        bool any = false;
        for (int c = 0; c < 2; ++c)
            for (auto &s : slots[c])
                if (s->done) {
                    any = true;
                    s->resid = !s->r_true;
                }
        if (!any) return CACG_OK;
        int rc = residual_pass();
        if (rc) return rc;
        std::vector<std::unique_ptr<BSlot>> out;
        for (int c = 0; c < 2; ++c) {
            for (size_t i = 0; i < slots[c].size(); ++i) {
                BSlot &s = *slots[c][i];
                if (!s.done) continue;
                Request *r = s.req.get();
                const double *nr = hnorms_of(c, (int)i);
                r->relres.assign(s.d.m, 0.0);
                double mx = 0.0;
                for (int q = 0; q < s.d.m; ++q) {
                    const double v = sqrt(std::max(nr[q], 0.0)) / s.bn[q];
                    r->relres[q] = v;
                    if (!(v <= mx)) mx = v;
                }
                r->res.true_relres_max = mx;
                r->res.m = s.d.m;
                cudaMemcpyAsync(r->X_out, s.d.X, (size_t)r->n * s.d.m * 8, cudaMemcpyDeviceToHost,
                                st);
            }
            for (auto it = slots[c].begin(); it != slots[c].end();) {
                if ((*it)->done) {
                    out.push_back(std::move(*it));
                    it = slots[c].erase(it);
                } else {
                    ++it;
                }
            }
        }
        const bool ok = cudaStreamSynchronize(st) == cudaSuccess;
        for (auto &s : out) {
            cudaFreeAsync(s->mem, st);
            s->mem = nullptr;
            Request *r = s->req.get();
            r->res.seconds = now_s() - s->t_admit;
            r->res.launches = g_launches.load() - s->l_admit;
            srv->finish_request(r, ok ? s->final_status : CACG_ERR_CUDA);
        }
        return ok ? CACG_OK : CACG_ERR_CUDA;
    }

    // a device error ends every request in flight with it
    void fail_all(int rc) {
        cudaStreamSynchronize(st);
        cudaGetLastError();
        for (int c = 0; c < 2; ++c) {
            for (auto &s : slots[c]) {
                if (s->mem) cudaFreeAsync(s->mem, st);
                s->mem = nullptr;
                srv->finish_request(s->req.get(), rc);
            }
            slots[c].clear();
        }
        cudaStreamSynchronize(st);
        cudaGetLastError();
    }

    bool empty() const { return slots[0].empty() && slots[1].empty(); }
};

// Synthetic batch for the autotuner: eight 2-D 5-point Laplacians (192^2
// rows), 8 right-hand sides, s = 4, in the class's precision.
void Engine::tune_class(int cls) {
    int dev = 0;
    cudaGetDevice(&dev);
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tunes.find({dev, cls});
        if (it != g_tunes.end()) {
            tune[cls] = it->second;
            tuned[cls] = true;
            return;
        }
    }
    for (int q = 0; q < kBKNumKinds; ++q) tune[cls].blocks_per_sm[q] = 2;
    const int N = 192, m = 8, s = 4, nreq = 8;
    const int64_t n = (int64_t)N * N, nnz = 5 * n - 4 * N;
    std::vector<int32_t> rp(n + 1), ci(nnz);
    std::vector<double> val(nnz), B((size_t)n * m);
    if (cacg_gen_matrix(CACG_GEN_LAPLACE2D_5PT, N, 0.01, 0.0, 1, rp.data(), ci.data(),
                        val.data()) != CACG_OK ||
        cacg_gen_rhs(CACG_RHS_NORMAL, n, m, 1, 0.0, 1.0, B.data()) != CACG_OK) {
        tuned[cls] = true;
        return;
    }
    std::vector<std::unique_ptr<BSlot>> saved;
    saved.swap(slots[cls]);
    bool ok = true;
    for (int i = 0; i < nreq && ok; ++i) {
        auto sl = std::make_unique<BSlot>();
        sl->req = std::make_shared<Request>();
        Request *r = sl->req.get();
        r->n = n;
        r->nnz = nnz;
        r->m = m;
        r->rp = rp;
        r->ci = ci;
        r->val = val;
        r->B = B;
        cacg_params_default(&r->p);
        r->p.s = s;
        r->p.precision = cls ? CACG_MIXED : CACG_FP64;
        r->p.bounds_mode = CACG_BOUNDS_GIVEN;
        ok = setup_slot(*sl) == CACG_OK;
        sl->d.it = 1;
        sl->d.sa = 0.25;
        sl->d.sb = -1.0;
        slots[cls].push_back(std::move(sl));
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int cand[4] = {1, 2, 4, 8};
    if (ok) {
        fill_batch(cls, [](BSlot &) { return kBActive | kBResid; });
        ok = cudaMemcpyAsync(d_b[cls], h_b[cls], sizeof(BBatch), cudaMemcpyHostToDevice, st) ==
             cudaSuccess;
        ok = ok && (cls ? bl_residual<float>(st, d_b[cls], tune[cls])
                        : bl_residual<double>(st, d_b[cls], tune[cls])) == CACG_OK;
        ok = ok && cudaStreamSynchronize(st) == cudaSuccess;
    }
    for (int kind = 0; kind < kBKNumKinds && ok; ++kind) {
        float best = 1e30f;
        int best_c = 2;
        for (int ci_ = 0; ci_ < 4 && ok; ++ci_) {
            BTune tu = tune[cls];
            tu.blocks_per_sm[kind] = cand[ci_];
            auto run = [&]() {
                const BBatch *b = d_b[cls];
                switch (kind) {
                    case kBKSpmm:
                        return cls ? bl_aq<float>(st, b, tu) : bl_aq<double>(st, b, tu);
                    case kBKGram:
                        return cls ? bl_gram<float>(st, b, 1, tu) : bl_gram<double>(st, b, 1, tu);
                    case kBKQupd:
                        return cls ? bl_qupdate<float>(st, b, tu) : bl_qupdate<double>(st, b, tu);
                    default:
                        return cls ? bl_xrupdate<float>(st, b, tu) : bl_xrupdate<double>(st, b, tu);
                }
            };
            ok = run() == CACG_OK;  // warm-up
            cudaEventRecord(e0, st);
            for (int rep = 0; rep < 3 && ok; ++rep) ok = run() == CACG_OK;
            cudaEventRecord(e1, st);
            ok = ok && cudaEventSynchronize(e1) == cudaSuccess;
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (ok && ms < best) {
                best = ms;
                best_c = cand[ci_];
            }
        }
        tune[cls].blocks_per_sm[kind] = best_c;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    for (auto &sl : slots[cls])
        if (sl->mem) cudaFreeAsync(sl->mem, st);
    slots[cls].clear();
    slots[cls].swap(saved);
    cudaStreamSynchronize(st);
    cudaGetLastError();
    tuned[cls] = true;
    if (ok) {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tunes[{dev, cls}] = tune[cls];
    }
}

void Server::engine_main() {
    cudaSetDevice(device);
    for (;;) {
        {
            std::unique_lock<std::mutex> lk(mu);
            cv_engine.wait(lk, [&] { return stop || !queue.empty() || !engine->empty(); });
            if (stop) break;
        }
        int rc = engine->admit();
        if (rc == CACG_OK) rc = engine->retire();  // maxit == 0, bad bounds
        if (rc == CACG_OK && !engine->empty()) {
            rc = engine->step();
            if (rc == CACG_OK) {
                engine->after_step();
                rc = engine->check_round();
            }
            if (rc == CACG_OK) rc = engine->retire();
        }
        if (rc != CACG_OK) engine->fail_all(rc);
        if (engine->empty()) {
            // nothing admitted: wait for a completion elsewhere or a submission
            std::unique_lock<std::mutex> lk(mu);
            cv_engine.wait_for(lk, std::chrono::milliseconds(2));
        }
    }
    engine->fail_all(CACG_ERR_CUDA);
}

}  // namespace cacg

using namespace cacg;

extern "C" {

int cacg_server_create(const cacg_server_config *cfg, cacg_server **out) {
    if (!cfg || !out || cfg->mem_budget_bytes <= 0 || cfg->max_active <= 0) return CACG_ERR_ARG;
    if (cfg->engine != CACG_SERVER_BATCHED && cfg->engine != CACG_SERVER_STREAMS)
        return CACG_ERR_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) {
        cudaGetLastError();
        return CACG_ERR_NODEV;
    }
    keep_pool_memory();
    Server *s = new Server();
    s->cfg = *cfg;
    cudaGetDevice(&s->device);
    if (cfg->engine == CACG_SERVER_BATCHED) {
        s->engine = std::make_unique<Engine>();
        s->engine->srv = s;
        s->engine->graphs = cfg->no_graphs == 0;
        const int rc = s->engine->init();
        if (rc != CACG_OK) {
            delete s;
            return rc;
        }
        s->engine_thread = std::thread([s] { s->engine_main(); });
    }
    for (int i = 0; i < cfg->max_active; ++i) s->workers.emplace_back([s] { s->worker(); });
    *out = reinterpret_cast<cacg_server *>(s);
    return CACG_OK;
}

int cacg_server_submit(cacg_server *srv, const cacg_csr *A, const double *B, int32_t m,
                       const cacg_params *p, double *X_out, int64_t *ticket) {
    if (!srv || !A || !B || !p || !X_out || !ticket || m <= 0 || A->n <= 0 || A->nnz < 0 ||
        A->n > INT32_MAX || A->nnz > INT32_MAX)
        return CACG_ERR_ARG;
    if (p->s < 2 || (int64_t)p->s * m > 256) return CACG_ERR_UNSUPPORTED;
    Server *s = reinterpret_cast<Server *>(srv);
    auto r = std::make_shared<Request>();
    r->n = A->n;
    r->nnz = A->nnz;
    r->m = m;
    r->rp.assign(A->row_ptr, A->row_ptr + A->n + 1);
    r->ci.assign(A->col_idx, A->col_idx + A->nnz);
    r->val.assign(A->val, A->val + A->nnz);
    r->B.assign(B, B + (size_t)A->n * m);
    r->p = *p;
    r->X_out = X_out;
    r->batched = s->engine && batch_eligible(*p, m) && A->n <= s->small_rows();
    if (r->batched) {
        r->cost = blayout(A->n, A->nnz, m, p->s, p->precision == CACG_MIXED).total;
    } else {
        // CSR (+ FP32 values) and, for diagonal-structured matrices, the DIA
        // view (at most 1.5 x nnz entries of FP64 + FP32 values)
        size_t mat = (size_t)(A->n + 1) * 4 + (size_t)A->nnz * (4 + 8 + 16) +
                     (p->precision == CACG_MIXED ? (size_t)A->nnz * 4 : 0) +
                     (size_t)A->nnz * 18 + (size_t)(A->n + 64) * 12 * 2;
        r->cost = mat + 2 * (size_t)A->n * m * 8 +
                  solve_workspace_bytes(A->n, m, p->s, p->precision,
                                        p->bounds_mode == CACG_BOUNDS_LANCZOS);
    }
    if ((int64_t)r->cost > s->cfg.mem_budget_bytes) return CACG_ERR_BUSY;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        r->ticket = s->next_ticket++;
        s->all[r->ticket] = r;
        (r->batched ? s->queue : s->lqueue).push_back(r);
        *ticket = r->ticket;
    }
    s->cv_work.notify_all();
    s->cv_engine.notify_all();
    return CACG_OK;
}

static int fill(const std::shared_ptr<Request> &r, cacg_result *res) {
    if (res) {
        double *keep = res->true_relres;
        *res = r->res;
        res->true_relres = keep;
        if (keep)
            for (int c = 0; c < r->m && c < (int)r->relres.size(); ++c) keep[c] = r->relres[c];
    }
    return r->status;
}

int cacg_server_poll(cacg_server *srv, int64_t ticket, cacg_result *res) {
    Server *s = reinterpret_cast<Server *>(srv);
    if (!s) return CACG_ERR_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->all.find(ticket);
    if (it == s->all.end()) return CACG_ERR_ARG;
    if (it->second->state != 2) return CACG_PENDING;
    auto r = it->second;
    s->all.erase(it);
    return fill(r, res);
}

int cacg_server_wait(cacg_server *srv, int64_t ticket, cacg_result *res) {
    Server *s = reinterpret_cast<Server *>(srv);
    if (!s) return CACG_ERR_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->all.find(ticket);
    if (it == s->all.end()) return CACG_ERR_ARG;
    auto r = it->second;
    s->cv_done.wait(lk, [&] { return r->state == 2; });
    s->all.erase(ticket);
    return fill(r, res);
}

int cacg_server_stats(cacg_server *srv, int64_t *queued, int64_t *active, int64_t *bytes) {
    Server *s = reinterpret_cast<Server *>(srv);
    if (!s) return CACG_ERR_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    if (queued) *queued = (int64_t)(s->queue.size() + s->lqueue.size());
    if (active) *active = s->active;
    if (bytes) *bytes = s->bytes_in_use;
    return CACG_OK;
}

int cacg_server_engine_stats(cacg_server *srv, int64_t *steps, int64_t *graph_replays,
                             int32_t *blocks_per_sm, int32_t nvals) {
    Server *s = reinterpret_cast<Server *>(srv);
    if (!s) return CACG_ERR_ARG;
    if (steps) *steps = s->engine_steps.load();
    if (graph_replays) *graph_replays = s->engine_graph_replays.load();
    if (blocks_per_sm) {
        int dev = 0;
        cudaGetDevice(&dev);
        std::lock_guard<std::mutex> lk(g_tune_mu);
        for (int c = 0; c < 2; ++c) {
            auto it = g_tunes.find({dev, c});
            for (int q = 0; q < kBKNumKinds; ++q)
                if (c * kBKNumKinds + q < nvals)
                    blocks_per_sm[c * kBKNumKinds + q] =
                        it != g_tunes.end() ? it->second.blocks_per_sm[q] : 0;
        }
    }
    return CACG_OK;
}

int cacg_server_destroy(cacg_server *srv) {
    Server *s = reinterpret_cast<Server *>(srv);
    if (!s) return CACG_ERR_ARG;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    s->cv_engine.notify_all();
    if (s->engine_thread.joinable()) s->engine_thread.join();
    for (auto &t : s->workers) t.join();
    delete s;
    return CACG_OK;
}

}  // extern "C"
