// server.cu -- persistent request loop for SPD solves (no reference
// counterpart: sclc/cacg solves one system per process launch,
// src/main.c:22-221).
//
// Continuous batching on one GPU:
//   * submit() copies the request (CSR, RHS block, params) and queues it;
//   * max_active worker slots each own a CUDA stream; a slot takes the queue
//     head as soon as the head's device footprint (matrix + B/X + solver
//     workspace, from cacg_workspace_bytes) fits in what the memory budget
//     has left, so requests are admitted while others run, and freed memory
//     admits the next one;
//   * admitted requests run concurrently on their streams, so their SpMM /
//     Gram / LU kernels overlap on the device;
//   * every kernel of a request sees only that request's buffers and its grid
//     and reduction order depend only on the request's own shape, so a result
//     is bit-identical whether the request ran alone or in the mix.
#include <cuda_runtime.h>

#include <atomic>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

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
    int state = 0;  // 0 queued, 1 running, 2 done
    int status = CACG_PENDING;
    cacg_result res{};
    std::vector<double> relres;
};

struct Server {
    cacg_server_config cfg;
    int device = 0;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<std::shared_ptr<Request>> queue;
    std::map<int64_t, std::shared_ptr<Request>> all;
    int64_t next_ticket = 1;
    int64_t bytes_in_use = 0;
    int64_t active = 0;
    bool stop = false;
    std::vector<std::thread> workers;

    void worker() {
        cudaSetDevice(device);
        cudaStream_t st;
        cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
        for (;;) {
            std::shared_ptr<Request> r;
            {
                std::unique_lock<std::mutex> lk(mu);
                cv_work.wait(lk, [&] {
                    return stop || (!queue.empty() &&
                                    bytes_in_use + (int64_t)queue.front()->cost <=
                                        cfg.mem_budget_bytes);
                });
                if (stop && queue.empty()) break;
                if (stop) break;
                r = queue.front();
                queue.pop_front();
                bytes_in_use += (int64_t)r->cost;
                active++;
                r->state = 1;
            }
            run_one(r.get(), st);
            {
                std::lock_guard<std::mutex> lk(mu);
                bytes_in_use -= (int64_t)r->cost;
                active--;
                r->state = 2;
                // drop the host copies of the inputs once solved
                std::vector<int32_t>().swap(r->rp);
                std::vector<int32_t>().swap(r->ci);
                std::vector<double>().swap(r->val);
                std::vector<double>().swap(r->B);
            }
            cv_done.notify_all();
            cv_work.notify_all();
        }
        cudaStreamDestroy(st);
    }

    void run_one(Request *r, cudaStream_t st) {
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
        r->status = rc;
        r->res.status = rc;
    }
};

}  // namespace cacg

using namespace cacg;

extern "C" {

int cacg_server_create(const cacg_server_config *cfg, cacg_server **out) {
    if (!cfg || !out || cfg->mem_budget_bytes <= 0 || cfg->max_active <= 0) return CACG_ERR_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) {
        cudaGetLastError();
        return CACG_ERR_NODEV;
    }
    Server *s = new Server();
    s->cfg = *cfg;
    cudaGetDevice(&s->device);
    for (int i = 0; i < cfg->max_active; ++i) s->workers.emplace_back([s] { s->worker(); });
    *out = reinterpret_cast<cacg_server *>(s);
    return CACG_OK;
}

int cacg_server_submit(cacg_server *srv, const cacg_csr *A, const double *B, int32_t m,
                       const cacg_params *p, double *X_out, int64_t *ticket) {
    if (!srv || !A || !B || !p || !X_out || !ticket || m <= 0 || A->n <= 0 || A->nnz < 0)
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
    // CSR (+ FP32 values) and, for diagonal-structured matrices, the DIA view
    // (at most 1.5 x nnz entries of FP64 + FP32 values)
    size_t mat = (size_t)(A->n + 1) * 4 + (size_t)A->nnz * (4 + 8 + 16) +
                 (p->precision == CACG_MIXED ? (size_t)A->nnz * 4 : 0) + (size_t)A->nnz * 18 +
                 (size_t)(A->n + 64) * 12 * 2;
    r->cost = mat + 2 * (size_t)A->n * m * 8 +
              solve_workspace_bytes(A->n, m, p->s, p->precision,
                                    p->bounds_mode == CACG_BOUNDS_LANCZOS);
    if ((int64_t)r->cost > s->cfg.mem_budget_bytes) return CACG_ERR_BUSY;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        r->ticket = s->next_ticket++;
        s->all[r->ticket] = r;
        s->queue.push_back(r);
        *ticket = r->ticket;
    }
    s->cv_work.notify_all();
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
    return fill(it->second, res);
}

int cacg_server_wait(cacg_server *srv, int64_t ticket, cacg_result *res) {
    Server *s = reinterpret_cast<Server *>(srv);
    if (!s) return CACG_ERR_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->all.find(ticket);
    if (it == s->all.end()) return CACG_ERR_ARG;
    auto r = it->second;
    s->cv_done.wait(lk, [&] { return r->state == 2; });
    return fill(r, res);
}

int cacg_server_stats(cacg_server *srv, int64_t *queued, int64_t *active, int64_t *bytes) {
    Server *s = reinterpret_cast<Server *>(srv);
    if (!s) return CACG_ERR_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    if (queued) *queued = (int64_t)s->queue.size();
    if (active) *active = s->active;
    if (bytes) *bytes = s->bytes_in_use;
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
    for (auto &t : s->workers) t.join();
    delete s;
    return CACG_OK;
}

}  // extern "C"
