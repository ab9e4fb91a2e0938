// Many independent solves on one GPU: batched problems (many generalized
// problems of uneven n and nev) and a serving loop (requests that arrive
// while others run).  The reference solves one problem per process
// (file-static solver state, src/ops_eig_sol_gcg.c:44-55); here every solve
// has its own OPS, solver context and host thread, and every host thread its
// own stream, so solves overlap on the device.
//
// A server owns `workers` host threads.  Submitted requests wait in FIFO
// order; a worker takes the next one when its estimated device footprint fits
// the memory budget (or when nothing else is running, so a request larger than
// the budget still runs, alone), solves it through GCGE_Solve and releases the
// footprint.  Each worker's solves take a 1/workers share of the persistent
// PCG kernel's grid, so the cooperative kernels of concurrent solves always
// fit on the device together.  Results do not depend on what else runs: every
// kernel's work split depends on the problem (and the share), not on timing.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>
#include <vector>

#include "common.cuh"

struct gcge_server {
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<gcge_request *> queue;
    std::vector<std::thread> threads;
    size_t budget = 0, used = 0;
    int active = 0;
    int workers = 1;
    bool stop = false;
};

namespace {

double now_s() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

// Device bytes a solve needs at most: the basis V = [X P W] and the Ritz
// vectors, the solver's n-length work blocks, the FP64 and FP32 block-PCG
// blocks, and the matrices (CSR, SELL and the union pattern) with slack.
size_t footprint(const gcge_request *r) {
    const size_t ld = ((size_t)r->n + 31) / 32 * 32;
    const size_t cols = (size_t)r->nev_max + 2 * (size_t)r->block_size;
    const size_t nnz_a = (size_t)r->a_colptr[r->n];
    const size_t nnz_b = r->b_colptr ? (size_t)r->b_colptr[r->n] : 0;
    const size_t kp = 40;
    size_t b = 8 * ld * (cols + r->nev_max);          // V, Ritz vectors
    b += 8 * ld * (3 * cols + 4 * r->block_size);     // workspaces, T1/T2, b, r
    b += 5 * ld * kp * (8 + 4);                       // PCG blocks (FP64 and FP32)
    b += 2 * 8 * ld * std::min<size_t>(50, (size_t)r->nev_max);  // A x, B x of the check
    b += 64 * (nnz_a + nnz_b + r->n);                 // CSR, SELL, union, staging
    return b + ((size_t)64 << 20);
}

void worker_loop(gcge_server *s) {
    gcge::t_pcg_share = s->workers;
    for (;;) {
        gcge_request *r = nullptr;
        size_t fp = 0;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv_work.wait(lk, [&] {
                if (s->stop && s->queue.empty()) return true;
                if (s->queue.empty()) return false;
                const size_t need = footprint(s->queue.front());
                return s->active == 0 || s->used + need <= s->budget;
            });
            if (s->queue.empty()) return;  // stopping
            r = s->queue.front();
            s->queue.pop_front();
            fp = footprint(r);
            s->used += fp;
            s->active++;
        }
        r->t_start = now_s();
        const int st = GCGE_Solve(r->n, r->a_colptr, r->a_rowind, r->a_val, r->b_colptr,
                                  r->b_rowind, r->b_val, r->nev, r->block_size, r->nev_init,
                                  r->nev_max, r->max_iter, r->tol, r->gap_min, r->auto_shift,
                                  r->precision, r->X0, r->nev_given, r->eval, r->evec, &r->info);
        r->t_end = now_s();
        {
            std::lock_guard<std::mutex> lk(s->mu);
            r->status = st;
            r->done = 1;
            s->used -= fp;
            s->active--;
        }
        s->cv_done.notify_all();
        s->cv_work.notify_all();
    }
}

}  // namespace

extern "C" {

gcge_server *GCGE_ServerCreate(int workers, size_t device_budget_bytes) {
    if (workers < 1) {
        gcge::set_error(GCGE_ERR_ARG, "GCGE_ServerCreate: workers >= 1");
        return nullptr;
    }
    try {
        gcge::lib_stream();  // fails without a device
        size_t budget = device_budget_bytes;
        if (budget == 0) {
            size_t fr = 0, tot = 0;
            GCGE_CUDA(cudaMemGetInfo(&fr, &tot));
            budget = fr / 10 * 8;
        }
        gcge_server *s = new gcge_server();
        s->budget = budget;
        s->workers = workers;
        for (int i = 0; i < workers; ++i) s->threads.emplace_back(worker_loop, s);
        return s;
    } catch (const gcge::CudaError &e) {
        gcge::set_error(e.status, e.where.c_str());
        return nullptr;
    }
}

int GCGE_ServerSubmit(gcge_server *s, gcge_request *r) {
    if (!s || !r || r->n <= 0 || !r->a_colptr || !r->eval) return GCGE_ERR_ARG;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->stop) return GCGE_ERR_ARG;
        r->done = 0;
        r->status = GCGE_OK;
        r->t_submit = now_s();
        r->t_start = r->t_end = 0.0;
        s->queue.push_back(r);
    }
    s->cv_work.notify_all();
    return GCGE_OK;
}

int GCGE_ServerWait(gcge_server *s, gcge_request *r) {
    if (!s || !r) return GCGE_ERR_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    s->cv_done.wait(lk, [&] { return r->done != 0; });
    return r->status;
}

void GCGE_ServerDestroy(gcge_server **sp) {
    if (!sp || !*sp) return;
    gcge_server *s = *sp;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    for (auto &t : s->threads) t.join();
    delete s;
    *sp = nullptr;
}

int GCGE_SolveBatch(gcge_request *reqs, int count, int workers, size_t device_budget_bytes) {
    if (count < 0 || (count > 0 && !reqs)) return GCGE_ERR_ARG;
    gcge_server *s = GCGE_ServerCreate(workers, device_budget_bytes);
    if (!s) return GCGE_ERR_CUDA;
    int first_err = GCGE_OK;
    for (int i = 0; i < count; ++i) {
        const int st = GCGE_ServerSubmit(s, &reqs[i]);
        if (st != GCGE_OK) {
            reqs[i].status = st;
            reqs[i].done = 1;
            if (first_err == GCGE_OK) first_err = st;
        }
    }
    GCGE_ServerDestroy(&s);  // drains the queue
    for (int i = 0; i < count; ++i)
        if (first_err == GCGE_OK && reqs[i].status != GCGE_OK &&
            reqs[i].status != GCGE_ERR_NOT_CONVERGED)
            first_err = reqs[i].status;
    return first_err;
}

}  // extern "C"
