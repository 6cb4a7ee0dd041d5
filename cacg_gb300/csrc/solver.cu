// solver.cu -- CBCG / BCBCG outer loop on one GPU, the extended solver API
// and the drop-in cbcg_v1 / bcbcg_v1 entry points.
//
// Reference (sclc/cacg): bcbcg_v1 src/bcbcgKernel.c:27-556, cbcg_v1
// src/cbcgKernel.c:23-250.  One outer iteration, as in the reference:
//   S  = Chebyshev basis of R (s blocks of width m)        src/bcbcgKernel.c:180
//   it == 0: Q = S                                          :199-203
//   else:    QtAS = AQ^T S; beta = (QtAQ)^-1 QtAS; Q = S - Q beta   :214-262
//   AQ = A Q; QtAQ = Q^T AQ; QtR = Q^T R; alpha = (QtAQ)^-1 QtR     :284-344
//   X += Q alpha; R -= AQ alpha; stop when ||R(:,0)|| < eps        :376-526
//
// GB300 layout: everything stays resident in HBM for the whole solve; only
// the m residual norms (and a status word) cross to the host per iteration.
// S, Q, AQ are n x k row-major (k = s*m), the reference's post-transpose
// layout, written in place by the basis kernel (no transpose pass).  Q and S
// swap buffers: Q_new = S - Q_old beta is written over S, so no n x k
// temporary exists (the reference allocates Qbeta, Qalpha, AQalpha).
// The factor of QtAQ is computed once and serves both alpha (this iteration)
// and beta (next iteration).
//
// Precision modes:
//   CACG_FP64   all FP64 (parity mode with the reference).
//   CACG_MIXED  A, S, Q, AQ in FP32 (SpMM and basis in FP32); Gram products
//               and Q = S - Q beta on the tcgen05 tensor cores (bf16x3 slices,
//               FP32 accumulation, Gram group sums in float-float, split-K in
//               FP64); LU, alpha, beta, X, R in FP64; R = B - A X recomputed in
//               FP64 every rr_period iterations and before convergence is
//               declared.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <set>
#include <string>
#include <vector>

#include "cacg_internal.cuh"
#include "cacg_solver.h"

namespace cacg {

std::atomic<int64_t> g_launches{0};

static std::mutex g_err_mu;
static std::string g_err_text;

void record_cuda_error(cudaError_t e, const char *what, const char *file, int line) {
    std::lock_guard<std::mutex> lk(g_err_mu);
    char buf[512];
    snprintf(buf, sizeof buf, "%s: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
    g_err_text = buf;
}

const char *last_cuda_error_text() { return g_err_text.c_str(); }

int sm_count() {
    static int cached[64] = {0};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) dev = 0;
    if (!cached[dev]) {
        int v = 0;
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        cached[dev] = v > 0 ? v : 1;
    }
    return cached[dev];
}

size_t max_smem_optin() {
    static size_t cached[64] = {0};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) dev = 0;
    if (!cached[dev]) {
        int v = 0;
        cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        cached[dev] = v > 0 ? (size_t)v : 49152;
    }
    return cached[dev];
}

void set_smem_attr_fn(const void *fn, int bytes) {
    static std::mutex mu;
    static std::set<std::pair<int, const void *>> done;
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(mu);
    if (done.insert({dev, fn}).second)
        cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

// --------------------------------------------------------------- matrices
int DevMatrix::create(const cacg_csr *A, bool want_f32, DevMatrix *M, cudaStream_t st) {
    if (!A || A->n <= 0 || A->nnz < 0 || A->n > INT32_MAX || A->nnz > INT32_MAX ||
        !A->row_ptr || !A->col_idx || !A->val)
        return CACG_ERR_ARG;
    M->n = A->n;
    M->nnz = A->nnz;
    M->avg_nnz = (double)A->nnz / (double)A->n;
    size_t b_rp = (size_t)(A->n + 1) * 4, b_ci = (size_t)A->nnz * 4, b_v = (size_t)A->nnz * 8;
    size_t b_v32 = want_f32 ? (size_t)A->nnz * 4 : 0;
    M->st = st;
    CACG_CUDA_TRY(cudaMallocAsync((void **)&M->rp, b_rp, st));
    M->owned_bytes = b_rp;
    CACG_CUDA_TRY(cudaMallocAsync((void **)&M->ci, b_ci + 16, st));
    M->owned_bytes += b_ci;
    CACG_CUDA_TRY(cudaMallocAsync((void **)&M->val, b_v + 16, st));
    M->owned_bytes += b_v;
    CACG_CUDA_TRY(cudaMemcpyAsync(M->rp, A->row_ptr, b_rp, cudaMemcpyHostToDevice, st));
    CACG_CUDA_TRY(cudaMemcpyAsync(M->ci, A->col_idx, b_ci, cudaMemcpyHostToDevice, st));
    CACG_CUDA_TRY(cudaMemcpyAsync(M->val, A->val, b_v, cudaMemcpyHostToDevice, st));
    if (want_f32) {
        CACG_CUDA_TRY(cudaMallocAsync((void **)&M->val32, b_v32 + 16, st));
        M->owned_bytes += b_v32;
        int rc = launch_cast_f64_f32(st, A->nnz, M->val, M->val32);
        if (rc) return rc;
    }
    return M->build_dia(A, want_f32, st);
}

int DevMatrix::ensure_f32(cudaStream_t st) {
    if (!val32) {
        CACG_CUDA_TRY(cudaMallocAsync((void **)&val32, (size_t)nnz * 4 + 16, st));
        owned_bytes += (size_t)nnz * 4;
        int rc = launch_cast_f64_f32(st, nnz, val, val32);
        if (rc) return rc;
    }
    if (dia_ndiag > 0 && !dia32) {
        const int64_t cnt = (int64_t)dia_ndiag * dia_npad;
        CACG_CUDA_TRY(cudaMallocAsync((void **)&dia32, (size_t)cnt * 8, st));
        owned_bytes += (size_t)cnt * 8;
        dia32lo = dia32 + cnt;
        return launch_dia_hilo(st, cnt, dia64, dia32, dia32lo);
    }
    return CACG_OK;
}

void DevMatrix::release() {
    if (rp) cudaFreeAsync(rp, st);
    if (ci) cudaFreeAsync(ci, st);
    if (val) cudaFreeAsync(val, st);
    if (val32) cudaFreeAsync(val32, st);
    if (dia64) cudaFreeAsync(dia64, st);
    if (dia32) cudaFreeAsync(dia32, st);
    rp = nullptr;
    ci = nullptr;
    val = nullptr;
    val32 = nullptr;
    dia64 = nullptr;
    dia32 = nullptr;
    dia32lo = nullptr;
    dia_ndiag = 0;
    owned_bytes = 0;
}

// --------------------------------------------------------------- workspace
static size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

struct Layout {
    size_t S, Q, AQ, R, R32, R32p, Xff, Rff, Bnorm, small, gram, norm, lanczos, total;
    size_t o_S, o_Q, o_AQ, o_R, o_R32, o_R32p, o_Xff, o_Rff, o_small, o_gram, o_norm, o_lanczos;
    size_t Ssl, R32sl, o_Ssl, o_Qsl, o_AQsl, o_R32sl;
    bool slices;
};

// With gram_variant CACG_GRAM_TC_SLICES the mixed mode carries bf16 slice
// planes of S, Q, AQ and R32, written by their producers and read by the
// tensor-core Gram (needs 16-byte slice rows: m a multiple of 8).
static bool use_slice_planes(int m, int s, int prec, int gram_variant, int exact_updates) {
    const int k = s * m;
    return prec == CACG_MIXED && gram_variant == CACG_GRAM_TC_SLICES && !exact_updates &&
           m % 8 == 0 && (size_t)k * k * sizeof(float) <= 160 * 1024;
}

static Layout layout(int64_t n, int m, int s, int prec, bool lanczos, bool slices = false) {
    Layout L{};
    const int k = s * m;
    const size_t es = prec == CACG_MIXED ? 4 : 8;
    L.slices = slices;
    L.S = L.Q = L.AQ = align256((size_t)n * k * es + 64);
    L.R = align256((size_t)n * m * 8);
    L.R32 = prec == CACG_MIXED ? align256((size_t)n * m * 4) : 0;
    // R32 again with its rows padded to 16 bytes, for the TMA-fed Gram when m
    // is not a multiple of 4 (R32's own rows are m values)
    L.R32p = prec == CACG_MIXED && m % 4 != 0 && k % 4 == 0
                 ? align256((size_t)n * (size_t)((m + 3) & ~3) * 4)
                 : 0;
    L.Xff = prec == CACG_MIXED ? align256((size_t)n * m * 8) : 0;  // X as FP32 hi, lo
    L.Rff = prec == CACG_MIXED ? align256((size_t)n * m * 8) : 0;  // R as FP32 hi, lo
    L.Ssl = slices ? align256((size_t)3 * n * k * 2) : 0;
    L.R32sl = slices ? align256((size_t)3 * n * m * 2) : 0;
    // small: QtAS k*k, QtAQ k*k, QtR k*m, F 2*k*k + k, alpha k*m, beta k*k, norms m,
    //        bnorm m, true norms m, bounds 2, scalars 16, status (int) 16
    L.small = align256(sizeof(double) * ((size_t)5 * k * k + k + (size_t)2 * k * m +
                                         3 * (size_t)m + 64));
    L.gram = align256(std::max(
        gram_workspace_bytes(n, k, k + m),
        prec == CACG_MIXED ? std::max(std::max(gram_tc_workspace_bytes(n, k, k + m),
                                               gram_tcs_workspace_bytes(n, k, k + m)),
                                      gram_tc5_workspace_bytes(n, k, k + m))
                           : (size_t)0));
    L.norm = align256(norm_workspace_doubles(n, std::max(m, 2)) * sizeof(double) + 4096);
    L.lanczos = lanczos ? align256((size_t)3 * n * 8) : 0;
    size_t o = 0;
    L.o_S = o; o += L.S;
    L.o_Q = o; o += L.Q;
    L.o_AQ = o; o += L.AQ;
    L.o_R = o; o += L.R;
    L.o_R32 = o; o += L.R32;
    L.o_R32p = o; o += L.R32p;
    L.o_Xff = o; o += L.Xff;
    L.o_Rff = o; o += L.Rff;
    L.o_small = o; o += L.small;
    L.o_gram = o; o += L.gram;
    L.o_norm = o; o += L.norm;
    L.o_lanczos = o; o += L.lanczos;
    L.o_Ssl = o; o += L.Ssl;
    L.o_Qsl = o; o += L.Ssl;
    L.o_AQsl = o; o += L.Ssl;
    L.o_R32sl = o; o += L.R32sl;
    L.total = o;
    return L;
}

size_t solve_workspace_bytes(int64_t n, int m, int s, int prec, bool lanczos) {
    return layout(n, m, s, prec, lanczos, use_slice_planes(m, s, prec, CACG_GRAM_TC_SLICES, 0))
        .total;
}

// A growable cache of one device workspace per thread-less use (the bench
// and the drop-ins call repeatedly; cudaMalloc of GBs per call would dominate).
static std::mutex g_ws_mu;
static void *g_ws_ptr = nullptr;
static size_t g_ws_bytes = 0;
static bool g_ws_busy = false;

static int ws_acquire(size_t bytes, void **out, bool *from_cache) {
    std::lock_guard<std::mutex> lk(g_ws_mu);
    if (!g_ws_busy) {
        if (g_ws_bytes < bytes) {
            if (g_ws_ptr) cudaFree(g_ws_ptr);
            g_ws_ptr = nullptr;
            g_ws_bytes = 0;
            cudaError_t e = cudaMalloc(&g_ws_ptr, bytes);
            if (e != cudaSuccess) {
                cudaGetLastError();
                return CACG_ERR_OOM;
            }
            g_ws_bytes = bytes;
        }
        g_ws_busy = true;
        *out = g_ws_ptr;
        *from_cache = true;
        return CACG_OK;
    }
    cudaError_t e = cudaMalloc(out, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return CACG_ERR_OOM;
    }
    *from_cache = false;
    return CACG_OK;
}

static void ws_release(void *p, bool from_cache) {
    if (from_cache) {
        std::lock_guard<std::mutex> lk(g_ws_mu);
        g_ws_busy = false;
    } else if (p) {
        cudaFree(p);
    }
}

// Per-thread pinned host scratch for the per-iteration norm read-back.
struct PinnedScratch {
    double *p = nullptr;
    size_t bytes = 0;
    ~PinnedScratch() {
        if (p) cudaFreeHost(p);
    }
};
double *pinned_scratch(size_t bytes) {
    static thread_local PinnedScratch ps;
    if (ps.bytes < bytes) {
        if (ps.p) cudaFreeHost(ps.p);
        ps.p = nullptr;
        ps.bytes = 0;
        if (cudaMallocHost((void **)&ps.p, bytes) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        ps.bytes = bytes;
    }
    return ps.p;
}

// Keep freed stream-ordered allocations in the device pool (process-local).
// Set once per device (each device has its own default pool).
void keep_pool_memory() {
    static std::atomic<uint64_t> done{0};
    int dev = 0;
    cudaGetDevice(&dev);
    const uint64_t bit = 1ull << (dev & 63);
    if (done.load() & bit) return;
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
        uint64_t thr = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    cudaGetLastError();
    done.fetch_or(bit);
}

// ------------------------------------------------------- phase profiling
static std::atomic<int> g_prof_on{0};
static std::mutex g_prof_mu;
struct PhaseAcc {
    double ms = 0, bytes = 0, flops = 0;
    int64_t launches = 0;
    int64_t calls = 0;  // timed begin/end pairs (one product, one update, ...)
};
static PhaseAcc g_prof[CACG_NUM_PHASES];

bool profile_enabled() { return g_prof_on.load() != 0; }

// a timed call of `phase` measured outside the solver (the serving engine)
void profile_accumulate(int phase, double ms, int64_t launches) {
    if (phase < 0 || phase >= CACG_NUM_PHASES) return;
    std::lock_guard<std::mutex> lk(g_prof_mu);
    g_prof[phase].ms += ms;
    g_prof[phase].launches += launches;
    g_prof[phase].calls += 1;
}

struct PendingEv {
    cudaEvent_t a, b;
    int phase;
    double bytes, flops;
    int64_t launches;
};

struct Profiler {
    bool on = false;
    cudaStream_t st = nullptr;
    std::vector<PendingEv> pend;
    std::vector<cudaEvent_t> pool;
    PendingEv cur{};
    int64_t l0 = 0;
    cudaEvent_t get() {
        if (!pool.empty()) {
            cudaEvent_t e = pool.back();
            pool.pop_back();
            return e;
        }
        cudaEvent_t e;
        cudaEventCreate(&e);
        return e;
    }
    void begin(int phase, double bytes, double flops) {
        if (!on) return;
        cur.a = get();
        cur.b = get();
        cur.phase = phase;
        cur.bytes = bytes;
        cur.flops = flops;
        l0 = g_launches.load();
        cudaEventRecord(cur.a, st);
    }
    void end() {
        if (!on) return;
        cudaEventRecord(cur.b, st);
        cur.launches = g_launches.load() - l0;
        pend.push_back(cur);
    }
    // call after a stream synchronisation
    void harvest() {
        if (pend.empty()) return;
        std::lock_guard<std::mutex> lk(g_prof_mu);
        for (auto &p : pend) {
            float ms = 0.f;
            if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
                PhaseAcc &a = g_prof[p.phase];
                a.ms += ms;
                a.bytes += p.bytes;
                a.flops += p.flops;
                a.launches += p.launches;
                a.calls += 1;
            }
            cudaGetLastError();
            pool.push_back(p.a);
            pool.push_back(p.b);
        }
        pend.clear();
    }
    ~Profiler() {
        for (auto e : pool) cudaEventDestroy(e);
        for (auto &p : pend) {
            cudaEventDestroy(p.a);
            cudaEventDestroy(p.b);
        }
    }
};

// Two captured outer iterations (one per buffer parity), replayed with
// cudaGraphLaunch; launches inside a replay are added to the launch count.
struct GraphPair {
    cudaGraphExec_t exec[2] = {nullptr, nullptr};
    int64_t kernels[2] = {0, 0};
    template <class F>
    int capture(cudaStream_t st, int par, F &&body) {
        const int64_t l0 = g_launches.load();
        if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
            cudaGetLastError();
            return CACG_ERR_CUDA;
        }
        const int rc = body();
        cudaGraph_t g = nullptr;
        const cudaError_t e = cudaStreamEndCapture(st, &g);
        kernels[par] = g_launches.load() - l0;
        if (rc != CACG_OK || e != cudaSuccess || !g) {
            if (g) cudaGraphDestroy(g);
            cudaGetLastError();
            return rc != CACG_OK ? rc : CACG_ERR_CUDA;
        }
        const cudaError_t ei = cudaGraphInstantiate(&exec[par], g, 0);
        cudaGraphDestroy(g);
        if (ei != cudaSuccess) {
            exec[par] = nullptr;
            cudaGetLastError();
            return CACG_ERR_CUDA;
        }
        // the capture recorded the launches; run them
        g_launches -= kernels[par];
        return replay(st, par);
    }
    int replay(cudaStream_t st, int par) {
        if (cudaGraphLaunch(exec[par], st) != cudaSuccess) {
            cudaGetLastError();
            return CACG_ERR_CUDA;
        }
        g_launches += kernels[par];
        return CACG_OK;
    }
    ~GraphPair() {
        for (auto &e : exec)
            if (e) cudaGraphExecDestroy(e);
    }
};

// ----------------------------------------------------------- the solver
struct SolveBuffers {
    void *S, *Q, *AQ;
    double *R;
    float *R32;
    float *R32p;  // R32 with rows of ldr32p >= m values (nullptr: not needed)
    int ldr32p;
    double *QtAS, *QtAQ, *QtR, *F, *alpha, *beta, *norms, *bnorm, *tnorm, *bounds, *scal;
    int *status;
    double *gram_ws;
    size_t gram_ws_bytes;
    double *norm_ws;
    int64_t norm_ws_doubles;
    float *Xff;  // n x m hi, then n x m lo (mixed mode's float-float residual)
    float *Rff;  // the same for R (the float-float state of the mixed mode)
    double *lz;  // 3 x n (Lanczos)
    Slices Ssl, Qsl, AQsl, R32sl;  // bf16 slice planes (mixed mode, when enabled)
};

static void carve(char *base, const Layout &L, int m, int k, SolveBuffers *b) {
    b->S = base + L.o_S;
    b->Q = base + L.o_Q;
    b->AQ = base + L.o_AQ;
    b->R = (double *)(base + L.o_R);
    b->R32 = L.R32 ? (float *)(base + L.o_R32) : nullptr;
    b->R32p = L.R32p ? (float *)(base + L.o_R32p) : nullptr;
    b->ldr32p = (m + 3) & ~3;
    b->Xff = L.Xff ? (float *)(base + L.o_Xff) : nullptr;
    b->Rff = L.Rff ? (float *)(base + L.o_Rff) : nullptr;
    double *sm = (double *)(base + L.o_small);
    b->QtAS = sm; sm += (size_t)k * k;
    b->QtAQ = sm; sm += (size_t)k * k;
    b->F = sm; sm += (size_t)2 * k * k + k;  // factors, pivot reciprocals, factors transposed
    b->beta = sm; sm += (size_t)k * k;
    b->QtR = sm; sm += (size_t)k * m;
    b->alpha = sm; sm += (size_t)k * m;
    b->norms = sm; sm += m;
    b->bnorm = sm; sm += m;
    b->tnorm = sm; sm += m;
    b->bounds = sm; sm += 2;
    b->scal = sm; sm += 16;
    b->status = (int *)sm;
    b->gram_ws = (double *)(base + L.o_gram);
    b->gram_ws_bytes = L.gram;
    b->norm_ws = (double *)(base + L.o_norm);
    b->norm_ws_doubles = (int64_t)((L.norm - 4096) / sizeof(double));
    b->lz = L.lanczos ? (double *)(base + L.o_lanczos) : nullptr;
}

static void carve_slices(char *base, const Layout &L, int64_t n, int m, int k, SolveBuffers *b) {
    if (!L.slices) return;
    b->Ssl = Slices{(__nv_bfloat16 *)(base + L.o_Ssl), n * k};
    b->Qsl = Slices{(__nv_bfloat16 *)(base + L.o_Qsl), n * k};
    b->AQsl = Slices{(__nv_bfloat16 *)(base + L.o_AQsl), n * k};
    b->R32sl = Slices{(__nv_bfloat16 *)(base + L.o_R32sl), n * m};
}

// Symmetric tridiagonal eigenvalues (diag a[0..k), off b[1..k)) by bisection
// on the Sturm count: returns the smallest and largest.
static void tridiag_extremes(const std::vector<double> &a, const std::vector<double> &b,
                             double *lo, double *hi) {
    const int k = (int)a.size();
    double gl = 1e300, gu = -1e300;
    for (int i = 0; i < k; ++i) {
        double r = (i > 0 ? fabs(b[i]) : 0.0) + (i + 1 < k ? fabs(b[i + 1]) : 0.0);
        gl = std::min(gl, a[i] - r);
        gu = std::max(gu, a[i] + r);
    }
    auto count_below = [&](double x) {
        int c = 0;
        double d = 1.0;
        for (int i = 0; i < k; ++i) {
            double bb = i > 0 ? b[i] * b[i] : 0.0;
            d = a[i] - x - (i > 0 ? bb / d : 0.0);
            if (d == 0.0) d = -1e-300;
            if (d < 0) ++c;
        }
        return c;
    };
    auto kth = [&](int idx) {  // idx-th smallest eigenvalue (0-based)
        double l = gl, u = gu;
        for (int it = 0; it < 200 && u - l > 1e-15 * std::max(fabs(l), fabs(u)); ++it) {
            double mid = 0.5 * (l + u);
            if (count_below(mid) > idx)
                u = mid;
            else
                l = mid;
        }
        return 0.5 * (l + u);
    };
    *lo = kth(0);
    *hi = kth(k - 1);
}

struct Solver {
    const DevMatrix *A;
    int m, s, k, prec;
    cacg_params p;
    cudaStream_t st;
    SolveBuffers b;
    double *h_pin = nullptr;  // pinned: norms m, status, bounds, misc
    double avg_nnz;
    Profiler prof;

    // algorithmic traffic of one SpMM of width w (A once, X once, extra
    // streamed operands once, Y written once)
    // (over the DIA view: ndiag * n values, no indices)
    double spmm_bytes(int w, int extra) const {
        double vb = prec == CACG_MIXED ? 4.0 : 8.0;
        const double xyz = (double)A->n * w * (double)es() * (2.0 + extra);
        if (uses_dia()) return (double)A->dia_ndiag * (double)A->n * vb + xyz;
        return (double)A->nnz * (vb + 4.0) + 4.0 * (double)(A->n + 1) + xyz;
    }
    bool uses_dia() const { return p.spmm_format != CACG_SPMM_CSR && A->dia_ndiag > 0; }

    const void *val_t() const { return prec == CACG_MIXED ? (const void *)A->val32 : A->val; }
    size_t es() const { return prec == CACG_MIXED ? 4 : 8; }

    // Y = ca A X + cb Z1 + cc Z2 in precision T: over the DIA view when the
    // matrix has one (bit-identical to the CSR kernel), else over CSR.
    template <typename T>
    int spmm(const T *X, int64_t ldx, T *Y, int64_t ldy, int w, const T *Z1, int64_t ldz1,
             const T *Z2, int64_t ldz2, double ca, double cb, double cc) {
        if (uses_dia()) {
            if constexpr (std::is_same<T, float>::value) {
                if (p.spmm_format == CACG_SPMM_AUTO) {
                    int rc = launch_dia_ring(st, A, w, X, ldx, Y, ldy, Z1, ldz1, Z2, ldz2, ca, cb,
                                             cc, b.status);
                    if (rc != CACG_ERR_UNSUPPORTED) return rc;
                    rc = launch_dia_wide(st, A, w, X, ldx, Y, ldy, Z1, ldz1, Z2, ldz2, ca, cb, cc);
                    if (rc != CACG_ERR_UNSUPPORTED) return rc;
                }
            }
            int rc = launch_dia_spmm<T>(st, A, w, X, ldx, Y, ldy, Z1, ldz1, Z2, ldz2, ca, cb, cc);
            if (rc != CACG_ERR_UNSUPPORTED) return rc;
        }
        const T *v = std::is_same<T, float>::value ? (const T *)(const void *)A->val32
                                                   : (const T *)(const void *)A->val;
        return launch_spmm<T>(st, A->n, A->rp, A->ci, v, w, X, ldx, Y, ldy, Z1, ldz1, Z2, ldz2,
                              ca, cb, cc, avg_nnz);
    }

    int bounds(double *lmin, double *lmax) {
        if (p.bounds_mode == CACG_BOUNDS_GIVEN) {
            *lmin = p.lambda_min;
            *lmax = p.lambda_max;
            return CACG_OK;
        }
        if (p.bounds_mode == CACG_BOUNDS_GERSCHGORIN) {
            int rc = launch_gerschgorin(st, A->n, A->rp, A->ci, A->val, b.bounds, b.norm_ws);
            if (rc) return rc;
            CACG_CUDA_TRY(cudaMemcpyAsync(h_pin, b.bounds, 2 * sizeof(double),
                                          cudaMemcpyDeviceToHost, st));
            CACG_CUDA_TRY(cudaStreamSynchronize(st));
            *lmin = h_pin[0];
            *lmax = h_pin[1];
            return CACG_OK;
        }
        if (p.bounds_mode == CACG_BOUNDS_LANCZOS) return lanczos(lmin, lmax);
        return CACG_ERR_ARG;
    }

    // lanczos_steps-step Lanczos (FP64) from a seeded N(0,1) start vector;
    // Ritz extremes theta_min, theta_max -> [theta_min, 1.05 theta_max].
    int lanczos(double *lmin, double *lmax) {
        const int64_t n = A->n;
        int steps = p.lanczos_steps > 0 ? p.lanczos_steps : 50;
        if (steps > n) steps = (int)n;
        double *v0 = b.lz, *v1 = b.lz + n, *w = b.lz + 2 * n;
        std::vector<double> h(n);
        cacg_gen_rhs(CACG_RHS_NORMAL, n, 1, p.lanczos_seed, 0.0, 1.0, h.data());
        CACG_CUDA_TRY(cudaMemcpyAsync(v1, h.data(), n * 8, cudaMemcpyHostToDevice, st));
        CACG_CUDA_TRY(cudaMemsetAsync(v0, 0, n * 8, st));
        int rc = launch_dot(st, n, v1, v1, b.scal, b.norm_ws);
        if (rc) return rc;
        CACG_CUDA_TRY(cudaMemcpyAsync(h_pin, b.scal, 8, cudaMemcpyDeviceToHost, st));
        CACG_CUDA_TRY(cudaStreamSynchronize(st));
        double nrm = sqrt(h_pin[0]);
        rc = launch_axpby(st, n, 0.0, v1, 1.0 / nrm, v1);
        if (rc) return rc;
        std::vector<double> al, be(1, 0.0);
        double beta_prev = 0.0;
        for (int j = 0; j < steps; ++j) {
            // w = A v1 - beta_prev v0
            rc = spmm<double>(v1, 1, w, 1, 1, v0, 1, nullptr, 0, 1.0, -beta_prev, 0.0);
            if (rc) return rc;
            rc = launch_dot(st, n, w, v1, b.scal, b.norm_ws);
            if (rc) return rc;
            CACG_CUDA_TRY(cudaMemcpyAsync(h_pin, b.scal, 8, cudaMemcpyDeviceToHost, st));
            CACG_CUDA_TRY(cudaStreamSynchronize(st));
            double a = h_pin[0];
            al.push_back(a);
            rc = launch_axpby(st, n, -a, v1, 1.0, w);
            if (rc) return rc;
            rc = launch_dot(st, n, w, w, b.scal + 1, b.norm_ws);
            if (rc) return rc;
            CACG_CUDA_TRY(cudaMemcpyAsync(h_pin, b.scal + 1, 8, cudaMemcpyDeviceToHost, st));
            CACG_CUDA_TRY(cudaStreamSynchronize(st));
            double bn = sqrt(h_pin[0]);
            if (j + 1 == steps || bn <= 1e-14 * fabs(a)) break;
            be.push_back(bn);
            // v0 <- v1 ; v1 <- w / bn
            CACG_CUDA_TRY(cudaMemcpyAsync(v0, v1, n * 8, cudaMemcpyDeviceToDevice, st));
            rc = launch_axpby(st, n, 1.0 / bn, w, 0.0, v1);
            if (rc) return rc;
            beta_prev = bn;
        }
        be.resize(al.size());
        double lo, hi;
        tridiag_extremes(al, be, &lo, &hi);
        *lmin = lo;
        *lmax = 1.05 * hi;
        return CACG_OK;
    }

    // R = B - A X (FP64); S0 = cast(R); R32; norms.  Used at start and for
    // residual replacement / true-residual checks.
    bool slices = false;
    // the X whose FP64 residual b.R holds (nullptr once X may have changed):
    // the final true residual then needs only its norms
    const double *r_fp64_of = nullptr;
    // float-float state (mixed mode, m = 16, DIA view): X and R live in Xff,
    // Rff between FP64 checks; x_dirty: the FP64 X lags Xff
    bool ffx = false, x_dirty = false, xff_valid = false;

    // R = B - A X.  ff: in the mixed mode over a DIA view, float-float
    // arithmetic (FP32 pipe) instead of FP64 -- used for the periodic residual
    // replacements; convergence checks and the reported residual use FP64.
    int residual(const double *B, const double *X, double *R, bool write_s0, double *norms,
                 bool ff = false) {
        const double dn = (double)A->n;
        ff = ff && prec == CACG_MIXED && uses_dia() && !slices && b.Xff &&
             p.residual_precision != CACG_RESID_FP64;
        prof.begin(CACG_PHASE_RESIDUAL,
                   (uses_dia() ? (double)A->dia_ndiag * dn * 8.0  // FP64, or FP32 hi + lo
                               : (double)A->nnz * 12.0 + 4.0 * (dn + 1)) +
                       dn * m * (8.0 * 3 + (double)es()),
                   2.0 * (double)A->nnz * m);
        int rc;
        if (ff) {
            // on the float-float state X is already split and R goes to Rff
            rc = launch_dia_residual_ff(st, A, m, ffx && xff_valid ? nullptr : X, B,
                                        ffx ? nullptr : R, b.Xff, b.Xff + (size_t)A->n * m,
                                        write_s0 ? (float *)b.S : nullptr, k,
                                        write_s0 ? b.R32 : nullptr, norms, b.norm_ws,
                                        b.norm_ws_doubles, ffx ? b.Rff : nullptr);
            if (rc != CACG_ERR_UNSUPPORTED) {
                if (rc == CACG_OK && ffx) xff_valid = true;
                prof.end();
                return rc;
            }
            if (ffx && xff_valid) {
                prof.end();
                return CACG_ERR_CUDA;  // the float-float state cannot leave the ff kernels
            }
            ffx = false;  // not supported for this matrix: FP64 state from the start
        }
        if (ffx && x_dirty) {  // an FP64 residual of the float-float X
            rc = launch_ff_join(st, A->n * (int64_t)m, b.Xff, b.Xff + (size_t)A->n * m,
                                const_cast<double *>(X));
            if (rc) {
                prof.end();
                return rc;
            }
            x_dirty = false;
        }
        if (slices && write_s0) {
            rc = launch_residual_sl(st, A->n, A->rp, A->ci, A->val, m, X, B, R, (float *)b.S, k,
                                    b.R32, norms, b.norm_ws, avg_nnz, b.Ssl, b.R32sl);
        } else {
            rc = spmm<double>(X, m, R, m, m, B, m, nullptr, 0, -1.0, 1.0, 0.0);
            if (rc == CACG_OK)
                rc = launch_residual_post(st, A->n, m, R, write_s0 ? b.S : nullptr,
                                          prec == CACG_MIXED, k, norms, b.norm_ws);
            if (rc == CACG_OK && write_s0 && b.R32)
                rc = launch_cast_f64_f32(st, A->n * m, R, b.R32);
            // the iterations continue from this R on the float-float state
            if (rc == CACG_OK && ffx && R == b.R)
                rc = launch_ff_split(st, A->n * (int64_t)m, R, b.Rff, b.Rff + (size_t)A->n * m);
            if (rc == CACG_OK && R == b.R) r_fp64_of = X;
        }
        prof.end();
        return rc;
    }

    static Slices at(Slices S, int64_t off) { return Slices{S.p ? S.p + off : nullptr, S.plane}; }

    template <typename T>
    int iterate_once(int it, double *X) {
        const int64_t n = A->n;
        T *S = (T *)b.S;
        // basis T_1 .. T_{s-1} (T_0 = S[:, 0:m] already holds R)
        const double dn = (double)n, ees = (double)es();
        for (int j = 1; j < s; ++j) {
            const T *Tm1 = S + (size_t)(j - 1) * m;
            const T *Tm2 = j >= 2 ? S + (size_t)(j - 2) * m : nullptr;
            double ca = j == 1 ? sa : 2.0 * sa, cb = j == 1 ? sb : 2.0 * sb;
            prof.begin(CACG_PHASE_BASIS, spmm_bytes(m, j >= 2 ? 1 : 0),
                       2.0 * (double)A->nnz * m + 5.0 * dn * m);
            int rc;
            if constexpr (std::is_same<T, float>::value) {
                if (slices)
                    rc = launch_spmm_sl<float>(st, n, A->rp, A->ci, A->val32, m, Tm1, k,
                                               S + (size_t)j * m, k, Tm1, k, Tm2, k, ca, cb,
                                               -1.0, avg_nnz, at(b.Ssl, (int64_t)j * m));
                else
                    rc = spmm<T>(Tm1, k, S + (size_t)j * m, k, m, Tm1, k, Tm2, k, ca, cb, -1.0);
            } else {
                rc = spmm<T>(Tm1, k, S + (size_t)j * m, k, m, Tm1, k, Tm2, k, ca, cb, -1.0);
            }
            prof.end();
            if (rc) return rc;
        }
        if (it == 0) {
            std::swap(b.Q, b.S);
            std::swap(b.Qsl, b.Ssl);
        } else {
            prof.begin(CACG_PHASE_GRAM, dn * 2.0 * k * ees, 2.0 * dn * k * k);
            int rc;
            if (slices)
                rc = launch_gram_tcs(st, n, b.AQsl, k, k, b.Ssl, k, k, Slices(), 0, 0, b.QtAS, k,
                                     nullptr, 0, b.gram_ws, b.gram_ws_bytes);
            else
                rc = gram<T>((const T *)b.AQ, k, (const T *)b.S, k, k, nullptr, 0, 0, b.QtAS, k,
                             nullptr, 0);
            prof.end();
            if (rc) return rc;
            prof.begin(CACG_PHASE_LU, 16.0 * k * k, 2.0 * (double)k * k * k);
            rc = launch_lu_solve(st, k, b.F, k, b.QtAS, b.beta);
            prof.end();
            if (rc) return rc;
            // Q_new = S - Q_old beta, written over S; then S <-> Q
            prof.begin(CACG_PHASE_QUPDATE, 3.0 * dn * k * ees, 2.0 * dn * k * k);
            if constexpr (std::is_same<T, float>::value) {
                if (slices) {
                    rc = launch_qupdate_sl(st, n, k, (float *)b.S, k, (const float *)b.Q, k,
                                           (const float *)b.S, k, b.beta, b.Ssl);
                } else {
                    rc = CACG_ERR_UNSUPPORTED;
                    if (tensor_cores5())
                        rc = launch_qupdate_tc5(st, n, k, (float *)b.S, k, (const float *)b.Q, k,
                                                (const float *)b.S, k, b.beta, b.status);
                    if (rc == CACG_ERR_UNSUPPORTED)
                        rc = launch_qupdate<T>(st, n, k, (T *)b.S, k, (const T *)b.Q, k,
                                               (const T *)b.S, k, b.beta);
                }
            } else {
                rc = launch_qupdate<T>(st, n, k, (T *)b.S, k, (const T *)b.Q, k, (const T *)b.S,
                                       k, b.beta);
            }
            prof.end();
            if (rc) return rc;
            std::swap(b.Q, b.S);
            std::swap(b.Qsl, b.Ssl);
        }
        const T *Q = (const T *)b.Q;
        T *AQ = (T *)b.AQ;
        prof.begin(CACG_PHASE_AQ, spmm_bytes(k, 0), 2.0 * (double)A->nnz * k);
        int rc;
        if constexpr (std::is_same<T, float>::value) {
            if (slices)
                rc = launch_spmm_sl<float>(st, n, A->rp, A->ci, A->val32, k, Q, k, AQ, k, nullptr,
                                           0, nullptr, 0, 1.0, 0.0, 0.0, avg_nnz, b.AQsl);
            else
                rc = spmm<T>(Q, k, AQ, k, k, nullptr, 0, nullptr, 0, 1.0, 0.0, 0.0);
        } else {
            rc = spmm<T>(Q, k, AQ, k, k, nullptr, 0, nullptr, 0, 1.0, 0.0, 0.0);
        }
        prof.end();
        if (rc) return rc;
        const T *Rp = prec == CACG_MIXED ? (const T *)(const void *)b.R32
                                         : (const T *)(const void *)b.R;
        int64_t ldrp = m;
        prof.begin(CACG_PHASE_GRAM, dn * (2.0 * k + m) * ees, 2.0 * dn * k * (k + m));
        if constexpr (std::is_same<T, float>::value) {
            // rows of m % 4 != 0 FP32 values are not 16-byte aligned: a padded
            // copy lets the Gram take TMA boxes (the tensor-map width stays m)
            if (!slices && b.R32p && gram_tc5_supported(k, k + m) &&
                (p.gram_variant == CACG_GRAM_AUTO || p.gram_variant == CACG_GRAM_TC5)) {
                rc = launch_copy_rows_f32(st, n, m, b.R32, m, b.R32p, b.ldr32p);
                if (rc) {
                    prof.end();
                    return rc;
                }
                Rp = b.R32p;
                ldrp = b.ldr32p;
            }
        }
        if (slices)
            rc = launch_gram_tcs(st, n, b.Qsl, k, k, b.AQsl, k, k, b.R32sl, m, m, b.QtAQ, k,
                                 b.QtR, m, b.gram_ws, b.gram_ws_bytes);
        else
            rc = gram<T>(Q, k, AQ, k, k, Rp, ldrp, m, b.QtAQ, k, b.QtR, m, true);
        prof.end();
        if (rc) return rc;
        prof.begin(CACG_PHASE_LU, 16.0 * k * k, (2.0 / 3.0) * k * k * k + 2.0 * k * k * m);
        rc = launch_lu_factor(st, k, b.QtAQ, b.F, b.status);
        if (rc == CACG_OK) rc = launch_lu_solve(st, k, b.F, m, b.QtR, b.alpha);
        prof.end();
        if (rc) return rc;
        // X += Q alpha; R -= AQ alpha; next T_0 into the spare buffer (S)
        prof.begin(CACG_PHASE_XRUPDATE,
                   dn * (2.0 * k * ees + 32.0 * m + ees * m + (b.R32 ? 4.0 * m : 0.0)),
                   4.0 * dn * k * m);
        rc = xrupdate<T>(Q, AQ, X);
        prof.end();
        return rc;
    }

    double sa = 0, sb = 0;

    // mixed mode on the tcgen05 kernels (Gram, Q update) unless a CUDA-core
    // or mma.sync Gram variant is requested
    bool tensor_cores5() const {
        return p.gram_variant == CACG_GRAM_AUTO || p.gram_variant == CACG_GRAM_TC5;
    }

    // Gram with the variant for this precision: the mixed mode uses the
    // tensor-core kernel unless a CUDA-core variant is requested.
    template <typename T>
    // symmetric: L^T R1 with R1 = A L (Q^T A Q), only its upper triangle is
    // computed and mirrored (FP64 CUDA-core Gram)
    int gram(const T *Lm, int ka, const T *R1, int64_t ldr1, int kb1, const T *R2, int64_t ldr2,
             int kb2, double *C1, int ldc1, double *C2, int ldc2, bool symmetric = false) {
        const int64_t n = A->n;
        if constexpr (std::is_same<T, float>::value) {
            if ((p.gram_variant == CACG_GRAM_AUTO || p.gram_variant == CACG_GRAM_TC5) &&
                gram_tc5_supported(ka, kb1 + kb2))
                return launch_gram_tc5(st, n, Lm, k, ka, R1, ldr1, kb1, R2, ldr2, kb2, C1, ldc1,
                                       C2, ldc2, b.gram_ws, b.gram_ws_bytes, b.status);
            if (p.gram_variant == CACG_GRAM_AUTO || p.gram_variant == CACG_GRAM_TC ||
                p.gram_variant == CACG_GRAM_TC5)
                return launch_gram_tc(st, n, Lm, k, ka, R1, ldr1, kb1, R2, ldr2, kb2, C1, ldc1,
                                      C2, ldc2, b.gram_ws, b.gram_ws_bytes);
        }
        int v = p.gram_variant == CACG_GRAM_TC ? CACG_GRAM_FMA : p.gram_variant;
        return launch_gram<T>(st, v, n, Lm, k, ka, R1, ldr1, kb1, R2, ldr2, kb2, C1, ldc1, C2,
                              ldc2, b.gram_ws, b.gram_ws_bytes,
                              symmetric && std::is_same<T, double>::value);
    }

    template <typename T>
    int xrupdate(const T *Q, const T *AQ, double *X) {
        if constexpr (std::is_same<T, float>::value) {
            if (slices)
                return launch_xrupdate_sl(st, A->n, k, m, Q, AQ, k, b.alpha, X, b.R, (float *)b.S,
                                          k, b.R32, b.norms, b.norm_ws, b.Ssl, b.R32sl);
        }
        if (prec == CACG_MIXED && p.exact_updates)
            return launch_xrupdate<T>(st, A->n, k, m, Q, AQ, k, b.alpha, X, b.R, (T *)b.S, k,
                                      b.R32, b.norms, b.norm_ws);
        // (the tcgen05 X/R update, launch_xrupdate_tc5, is slower than the
        // CUDA-core kernels at m = 16: its N = 16 MMAs are latency-bound)
        if constexpr (std::is_same<T, float>::value) {
            if (ffx)
                return launch_xrupdate_m16_ff(st, A->n, k, Q, AQ, k, b.alpha, b.Xff, b.Rff,
                                              (float *)b.S, k, b.R32, b.norms, b.norm_ws,
                                              b.status);
            if (m == 16) {
                int rc = launch_xrupdate_m16_tma(st, A->n, k, Q, AQ, k, b.alpha, X, b.R,
                                                 (float *)b.S, k, b.R32, b.norms, b.norm_ws,
                                                 b.status);
                if (rc != CACG_ERR_UNSUPPORTED) return rc;
            }
        }
        return launch_xrupdate_fast<T>(st, A->n, k, m, Q, AQ, k, b.alpha, X, b.R, (T *)b.S, k,
                                       b.R32, b.norms, b.norm_ws);
    }

    int fetch_norms(int *status_out) {
        CACG_CUDA_TRY(cudaMemcpyAsync(h_pin, b.norms, m * sizeof(double),
                                      cudaMemcpyDeviceToHost, st));
        CACG_CUDA_TRY(cudaMemcpyAsync(h_pin + m, b.status, sizeof(int), cudaMemcpyDeviceToHost,
                                      st));
        CACG_CUDA_TRY(cudaStreamSynchronize(st));
        prof.harvest();
        int stv;
        memcpy(&stv, h_pin + m, sizeof(int));
        *status_out = stv;
        return CACG_OK;
    }

    int run(const double *B, double *X, cacg_result *res) {
        const int64_t n = A->n;
        int rc;
        r_fp64_of = nullptr;
        res->status = CACG_OK;
        res->iterations = 0;
        res->residual_replacements = 0;
        res->m = m;
        CACG_CUDA_TRY(cudaMemsetAsync(b.status, 0, sizeof(int), st));
        double lmin, lmax;
        rc = bounds(&lmin, &lmax);
        if (rc) return rc;
        res->lambda_min = lmin;
        res->lambda_max = lmax;
        if (!(lmax > lmin)) return CACG_ERR_ARG;
        sa = 2.0 / (lmax - lmin);              // src/bcbcgKernel.c:113
        sb = -(lmax + lmin) / (lmax - lmin);   // src/bcbcgKernel.c:114-115

        std::vector<double> bn(m, 1.0);
        if (p.tol_mode == CACG_TOL_REL_ALL) {
            rc = launch_colnorm(st, n, m, B, b.bnorm, b.norm_ws);
            if (rc) return rc;
            CACG_CUDA_TRY(cudaMemcpyAsync(h_pin, b.bnorm, m * 8, cudaMemcpyDeviceToHost, st));
            CACG_CUDA_TRY(cudaStreamSynchronize(st));
            for (int c = 0; c < m; ++c) bn[c] = h_pin[c] > 0 ? sqrt(h_pin[c]) : 1.0;
        }
        // float-float state for the mixed mode's 16-column blocks over a DIA view
        xff_valid = false;
        x_dirty = false;
        ffx = prec == CACG_MIXED && m == 16 && uses_dia() && !slices && b.Xff && b.Rff &&
              A->dia32 && A->dia32lo && p.residual_precision != CACG_RESID_FP64 &&
              !p.exact_updates && k % 4 == 0 && k <= 128 && n < (int64_t)INT32_MAX - 256;
        rc = residual(B, X, b.R, true, b.norms, true);
        if (rc) return rc;

        auto rel_max = [&](const double *nr) {
            double mx = 0.0;
            for (int c = 0; c < m; ++c) {
                double v = sqrt(std::max(nr[c], 0.0)) / bn[c];
                if (!(v <= mx)) mx = v;  // NaN propagates as "not converged"
            }
            return mx;
        };

        int since_rr = 0;
        bool converged = false;
        int it = 0;
        // CUDA graphs (use_graph, on a non-default stream): from iteration 2 on,
        // an outer iteration's launch sequence is captured once per parity
        // (Q and S swap buffers every iteration, so even and odd iterations
        // differ only in which buffer is which) and replayed; the host repeats
        // the buffer swap the captured iteration made.  Iterations 0 and 1 run
        // uncaptured (iteration 0 differs, and every kernel's one-time setup
        // happens outside a capture).
        const bool graphs = p.use_graph != 0 && st != nullptr;
        GraphPair gp;
        const bool prof_on = prof.on;
        for (it = 0; it < p.maxit; ++it) {
            r_fp64_of = nullptr;  // this iteration updates X
            if (ffx) x_dirty = true;  // (in Xff; the FP64 X is joined on demand)
            if (graphs && it >= 2) {
                const int par = it & 1;
                prof.on = false;
                if (!gp.exec[par]) {
                    rc = gp.capture(st, par, [&] {
                        return prec == CACG_MIXED ? iterate_once<float>(it, X)
                                                  : iterate_once<double>(it, X);
                    });
                } else {
                    std::swap(b.Q, b.S);
                    std::swap(b.Qsl, b.Ssl);
                    rc = gp.replay(st, par);
                }
                prof.on = prof_on;
            } else {
                rc = prec == CACG_MIXED ? iterate_once<float>(it, X) : iterate_once<double>(it, X);
            }
            if (rc) return rc;
            int stv = 0;
            rc = fetch_norms(&stv);
            if (rc) return rc;
            ++since_rr;
            res->iterations = it + 1;
            res->recurrence_norm0 = sqrt(std::max(h_pin[0], 0.0));
            // an early stop leaves the caller's X at the last iterate, as the
            // FP64 state does (the float-float X is joined back first)
            auto stop = [&](int code) {
                if (ffx && x_dirty &&
                    launch_ff_join(st, n * (int64_t)m, b.Xff, b.Xff + (size_t)n * m, X) ==
                        CACG_OK)
                    cudaStreamSynchronize(st);
                res->status = code;
                return code;
            };
            if (stv & kStatusTimeout) return stop(CACG_ERR_TIMEOUT);
            if (stv & kStatusBreakdown) return stop(CACG_ERR_BREAKDOWN);
            bool finite = true;
            for (int c = 0; c < m; ++c) finite = finite && std::isfinite(h_pin[c]);
            if (!finite) return stop(CACG_ERR_BREAKDOWN);
            if (p.tol_mode == CACG_TOL_ABS_COL0) {
                // the reference's test, src/bcbcgKernel.c:524
                if (sqrt(h_pin[0]) < p.tol) {
                    converged = true;
                    break;
                }
                if (prec == CACG_MIXED && p.rr_period > 0 && since_rr >= p.rr_period) {
                    rc = residual(B, X, b.R, true, b.norms, true);
                    if (rc) return rc;
                    res->residual_replacements++;
                    since_rr = 0;
                }
                continue;
            }
            // relative, all columns, confirmed on the true residual
            bool rec_ok = rel_max(h_pin) <= p.tol;
            bool rr_due = prec == CACG_MIXED && p.rr_period > 0 && since_rr >= p.rr_period;
            if (rec_ok || rr_due) {
                // a convergence check runs in FP64; a periodic replacement
                // may run in float-float
                rc = residual(B, X, b.R, true, b.norms, !rec_ok);
                if (rc) return rc;
                res->residual_replacements++;
                since_rr = 0;
                int stv2;
                rc = fetch_norms(&stv2);
                if (rc) return rc;
                if (rel_max(h_pin) <= p.tol) {
                    converged = true;
                    break;
                }
            }
        }
        // the float-float X back to FP64 (the caller's X)
        if (ffx && x_dirty) {
            rc = launch_ff_join(st, n * (int64_t)m, b.Xff, b.Xff + (size_t)n * m, X);
            if (rc) return rc;
            x_dirty = false;
        }
        // final true residual per column (FP64); after a converged FP64 check
        // b.R already holds B - A X for this X
        rc = r_fp64_of == X ? CACG_OK
                            : spmm<double>(X, m, b.R, m, m, B, m, nullptr, 0, -1.0, 1.0, 0.0);
        if (rc == CACG_OK)
            rc = launch_residual_post(st, n, m, b.R, nullptr, 0, k, b.tnorm, b.norm_ws);
        if (rc) return rc;
        if (p.tol_mode != CACG_TOL_REL_ALL) {
            rc = launch_colnorm(st, n, m, B, b.bnorm, b.norm_ws);
            if (rc) return rc;
        }
        CACG_CUDA_TRY(cudaMemcpyAsync(h_pin, b.tnorm, m * 8, cudaMemcpyDeviceToHost, st));
        CACG_CUDA_TRY(cudaMemcpyAsync(h_pin + m, b.bnorm, m * 8, cudaMemcpyDeviceToHost, st));
        CACG_CUDA_TRY(cudaStreamSynchronize(st));
        double mx = 0.0;
        for (int c = 0; c < m; ++c) {
            double den = h_pin[m + c] > 0 ? sqrt(h_pin[m + c]) : 1.0;
            double v = sqrt(std::max(h_pin[c], 0.0)) / den;
            if (res->true_relres) res->true_relres[c] = v;
            if (!(v <= mx)) mx = v;
        }
        res->true_relres_max = mx;
        res->status = converged ? CACG_OK : CACG_NOT_CONVERGED;
        return res->status;
    }
};

int solve_on_device(const DevMatrix *A, const double *B, double *X, int m,
                    const cacg_params *pin, cacg_result *res, void *ws_external,
                    size_t ws_external_bytes) {
    if (!A || !B || !X || m <= 0 || m > 256 || !pin || !res) return CACG_ERR_ARG;
    if (pin->algorithm == CACG_ALG_BCG) return solve_bcg_on_device(A, B, X, m, pin, res);
    if (pin->algorithm != CACG_ALG_CACG) return CACG_ERR_ARG;
    keep_pool_memory();
    cacg_params p = *pin;
    if (p.s < 2 || p.maxit < 0 || (p.precision != CACG_FP64 && p.precision != CACG_MIXED))
        return CACG_ERR_ARG;
    if ((int64_t)p.s * m > 256) return CACG_ERR_UNSUPPORTED;
    Solver S;
    S.A = A;
    S.m = m;
    S.s = p.s;
    S.k = p.s * m;
    S.prec = p.precision;
    S.p = p;
    S.avg_nnz = A->avg_nnz;
    S.st = (cudaStream_t)p.stream;
    S.prof.on = g_prof_on.load() != 0;
    S.prof.st = S.st;
    if (S.prec == CACG_MIXED && !A->val32) return CACG_ERR_ARG;
    bool lz = p.bounds_mode == CACG_BOUNDS_LANCZOS;
    const bool sl = use_slice_planes(m, p.s, p.precision, p.gram_variant, p.exact_updates);
    Layout L = layout(A->n, m, p.s, p.precision, lz, sl);
    S.slices = sl;
    void *ws = ws_external;
    bool from_cache = false;
    if (ws) {
        if (ws_external_bytes < L.total) return CACG_ERR_ARG;
    } else {
        int rc = ws_acquire(L.total, &ws, &from_cache);
        if (rc) return rc;
    }
    carve((char *)ws, L, m, S.k, &S.b);
    carve_slices((char *)ws, L, A->n, m, S.k, &S.b);
    double *pin_host = pinned_scratch(sizeof(double) * (2 * (size_t)m + 64));
    if (!pin_host) {
        if (!ws_external) ws_release(ws, from_cache);
        return CACG_ERR_OOM;
    }
    S.h_pin = pin_host;
    int64_t l0 = g_launches.load();
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, S.st);
    int rc = S.run(B, X, res);
    cudaEventRecord(e1, S.st);
    cudaEventSynchronize(e1);
    S.prof.harvest();
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    res->seconds = ms * 1e-3;
    res->launches = g_launches.load() - l0;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (!ws_external) ws_release(ws, from_cache);
    if (rc < 0) res->status = rc;
    return rc;
}

}  // namespace cacg

// ======================================================================
//                                 C ABI
// ======================================================================
using namespace cacg;

extern "C" {

void cacg_params_default(cacg_params *p) {
    if (!p) return;
    memset(p, 0, sizeof *p);
    p->s = 4;
    p->bounds_mode = CACG_BOUNDS_GERSCHGORIN;
    p->lanczos_steps = 50;
    p->tol_mode = CACG_TOL_REL_ALL;
    p->tol = 1e-8;
    p->maxit = 1000;
    p->precision = CACG_FP64;
    p->rr_period = 5;
    p->gram_variant = CACG_GRAM_AUTO;
    p->lanczos_seed = 12345;
}

const char *cacg_status_string(int s) {
    switch (s) {
    case CACG_OK: return "ok";
    case CACG_NOT_CONVERGED: return "not converged";
    case CACG_PENDING: return "pending";
    case CACG_ERR_ARG: return "invalid argument";
    case CACG_ERR_OOM: return "out of device memory";
    case CACG_ERR_CUDA: return last_cuda_error_text();
    case CACG_ERR_BREAKDOWN: return "breakdown (zero/non-finite pivot or residual)";
    case CACG_ERR_TIMEOUT: return "device wait timed out";
    case CACG_ERR_UNSUPPORTED: return "unsupported configuration";
    case CACG_ERR_BUSY: return "admission refused";
    case CACG_ERR_NODEV: return "no CUDA device";
    default: return "unknown";
    }
}

int64_t cacg_launch_count(void) { return g_launches.load(); }

void cacg_profile_enable(int on) { g_prof_on.store(on ? 1 : 0); }

void cacg_profile_reset(void) {
    std::lock_guard<std::mutex> lk(g_prof_mu);
    for (auto &a : g_prof) a = PhaseAcc();
}

int cacg_profile_get(int phase, double *ms, int64_t *launches, double *bytes, double *flops) {
    if (phase < 0 || phase >= CACG_NUM_PHASES) return CACG_ERR_ARG;
    std::lock_guard<std::mutex> lk(g_prof_mu);
    const PhaseAcc &a = g_prof[phase];
    if (ms) *ms = a.ms;
    if (launches) *launches = a.launches;
    if (bytes) *bytes = a.bytes;
    if (flops) *flops = a.flops;
    return CACG_OK;
}

int64_t cacg_profile_calls(int phase) {
    if (phase < 0 || phase >= CACG_NUM_PHASES) return 0;
    std::lock_guard<std::mutex> lk(g_prof_mu);
    return g_prof[phase].calls;
}

const char *cacg_profile_name(int phase) {
    static const char *names[CACG_NUM_PHASES] = {"basis_spmm", "aq_spmm", "gram", "qupdate",
                                                 "xrupdate", "lu", "residual", "bounds"};
    return (phase >= 0 && phase < CACG_NUM_PHASES) ? names[phase] : "?";
}

static int have_device() {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) {
        cudaGetLastError();
        return 0;
    }
    return 1;
}

int cacg_matrix_create(const cacg_csr *A, int32_t want_fp32, cacg_matrix **out) {
    if (!out) return CACG_ERR_ARG;
    if (!have_device()) return CACG_ERR_NODEV;
    DevMatrix *M = new DevMatrix();
    int rc = DevMatrix::create(A, want_fp32 != 0, M, nullptr);
    if (rc == CACG_OK && cudaStreamSynchronize(nullptr) != cudaSuccess) rc = CACG_ERR_CUDA;
    if (rc != CACG_OK) {
        M->release();
        delete M;
        return rc;
    }
    *out = reinterpret_cast<cacg_matrix *>(M);
    return CACG_OK;
}

int cacg_matrix_destroy(cacg_matrix *A) {
    if (!A) return CACG_ERR_ARG;
    DevMatrix *M = reinterpret_cast<DevMatrix *>(A);
    M->release();
    delete M;
    return CACG_OK;
}

int64_t cacg_matrix_device_bytes(const cacg_matrix *A) {
    return A ? (int64_t)reinterpret_cast<const DevMatrix *>(A)->owned_bytes : 0;
}

int32_t cacg_matrix_diagonals(const cacg_matrix *A) {
    if (!A) return 0;
    return reinterpret_cast<const DevMatrix *>(A)->dia_ndiag;
}

int64_t cacg_workspace_bytes(int64_t n, int32_t m, int32_t s, int32_t precision) {
    return (int64_t)solve_workspace_bytes(n, m, s, precision, true);
}

int cacg_solve_device(cacg_matrix *A, const double *B_dev, double *X_dev, int32_t m,
                      const cacg_params *p, cacg_result *res) {
    if (!A || !p || !res) return CACG_ERR_ARG;
    DevMatrix *M = reinterpret_cast<DevMatrix *>(A);
    if (p->precision == CACG_MIXED && !M->val32) {
        int rc = M->ensure_f32((cudaStream_t)p->stream);
        if (rc) return rc;
    }
    return solve_on_device(M, B_dev, X_dev, m, p, res, nullptr, 0);
}

int cacg_solve(const cacg_csr *A, const double *B, double *X, int32_t m, const cacg_params *p,
               cacg_result *res) {
    if (!A || !B || !X || !p || !res || m <= 0) return CACG_ERR_ARG;
    if (!have_device()) return CACG_ERR_NODEV;
    cudaStream_t st = (cudaStream_t)p->stream;
    DevMatrix M;
    int rc = DevMatrix::create(A, p->precision == CACG_MIXED, &M, st);
    double *dB = nullptr, *dX = nullptr;
    size_t bytes = (size_t)A->n * m * sizeof(double);
    if (rc == CACG_OK && cudaMallocAsync((void **)&dB, bytes, st) != cudaSuccess) rc = CACG_ERR_OOM;
    if (rc == CACG_OK && cudaMallocAsync((void **)&dX, bytes, st) != cudaSuccess) rc = CACG_ERR_OOM;
    if (rc == CACG_OK) {
        cudaMemcpyAsync(dB, B, bytes, cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(dX, X, bytes, cudaMemcpyHostToDevice, st);
        int r2 = solve_on_device(&M, dB, dX, m, p, res, nullptr, 0);
        if (r2 >= 0 || r2 == CACG_ERR_BREAKDOWN) {
            // the reference leaves X at the last iterate in every case
            if (cudaMemcpyAsync(X, dX, bytes, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                cudaStreamSynchronize(st) != cudaSuccess)
                r2 = CACG_ERR_CUDA;
        }
        rc = r2;
    }
    if (dB) cudaFreeAsync(dB, st);
    if (dX) cudaFreeAsync(dX, st);
    M.release();
    cudaStreamSynchronize(st);
    cudaGetLastError();
    res->status = rc;
    return rc;
}

// ---------------------------------------------------------------- drop-ins
static thread_local int t_last_status = CACG_OK;
static thread_local int t_last_iters = 0;
static std::atomic<int> g_dropin_maxit{0};

int cacg_last_status(void) { return t_last_status; }
int cacg_last_iterations(void) { return t_last_iters; }
void cacg_set_dropin_maxit(int maxit) { g_dropin_maxit.store(maxit > 0 ? maxit : 0); }

static void dropin(csrType_local mat, denseType B, denseType X, long s, double epsilon,
                   int numprocs, int default_maxit, const char *name,
                   int algorithm = CACG_ALG_CACG) {
    t_last_iters = 0;
    if (numprocs != 1) {
        fprintf(stderr, "%s (libcacg): one rank per GPU only; numprocs=%d unsupported\n", name,
                numprocs);
        t_last_status = CACG_ERR_UNSUPPORTED;
        return;
    }
    const long n = mat.num_rows;
    const long m = B.local_num_col;
    if (n <= 0 || mat.num_cols != n || mat.start != 0 || B.local_num_row != n ||
        X.local_num_row != n || X.local_num_col != m || m <= 0 || !mat.row_start ||
        !mat.col_idx || !mat.csrdata || !B.data || !X.data || s < 2) {
        t_last_status = CACG_ERR_ARG;
        return;
    }
    const long nnz = mat.row_start[n] - mat.row_start[0];
    if (nnz < 0 || nnz > INT32_MAX || n > INT32_MAX) {
        t_last_status = CACG_ERR_UNSUPPORTED;
        return;
    }
    // long -> int32 indices (rebased to row_start[0])
    std::vector<int32_t> rp(n + 1), ci(nnz);
    for (long i = 0; i <= n; ++i) rp[i] = (int32_t)(mat.row_start[i] - mat.row_start[0]);
    for (long e = 0; e < nnz; ++e) {
        long c = mat.col_idx[mat.row_start[0] + e];
        if (c < 0 || c >= n) {
            t_last_status = CACG_ERR_ARG;
            return;
        }
        ci[e] = (int32_t)c;
    }
    cacg_csr A{n, nnz, rp.data(), ci.data(), mat.csrdata + mat.row_start[0]};
    cacg_params p;
    cacg_params_default(&p);
    p.s = (int32_t)s;
    p.bounds_mode = CACG_BOUNDS_GERSCHGORIN;  // src/bcbcgKernel.c:106
    p.tol_mode = CACG_TOL_ABS_COL0;           // src/bcbcgKernel.c:445-447, 524
    p.tol = epsilon;
    int ov = g_dropin_maxit.load();
    p.maxit = ov > 0 ? ov : default_maxit;
    p.precision = CACG_FP64;
    p.algorithm = algorithm;
    cacg_result r;
    memset(&r, 0, sizeof r);
    int rc = cacg_solve(&A, B.data, X.data, (int32_t)m, &p, &r);
    t_last_status = rc;
    t_last_iters = r.iterations;
}

void cbcg_v1(csrType_local mat, denseType B, denseType X, long s, double epsilon, int myid,
             int numprocs) {
    (void)myid;
    dropin(mat, B, X, s, epsilon, numprocs, 1000, "cbcg_v1");  // src/cbcgKernel.c:2
}

void bcbcg_v1(csrType_local mat, denseType B, denseType X, long s, double epsilon, int myid,
              int numprocs) {
    (void)myid;
    dropin(mat, B, X, s, epsilon, numprocs, 100, "bcbcg_v1");  // src/bcbcgKernel.c:3
}

void bcg_v1(csrType_local mat, denseType B, denseType X, double epsilon, int myid,
            int numprocs) {
    (void)myid;
    // s is not a bcg_v1 argument; 2 passes the drop-in's argument check only
    dropin(mat, B, X, 2, epsilon, numprocs, 1000, "bcg_v1", CACG_ALG_BCG);  // src/bcgKernel.c:2
}

}  // extern "C"
