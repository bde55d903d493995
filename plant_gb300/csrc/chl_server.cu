// Continuous-batching distance-query server over labels resident in HBM.
//
// No reference counterpart: the reference answers one batch per process run
// (query mode 1, distributed_memory/query.hpp:82-91, over batchLocalQuery,
// distributed_memory/query_funcs.hpp:23-30).  Here requests of any size
// arrive at any time:
//   * admission by memory: every admitted pair holds 12 bytes of staging
//     (8 for the pair, 4 for its answer) until it is answered; a request is
//     admitted once its pairs fit in the budget (max_inflight_pairs) and a
//     request entry is free, and a request larger than the budget is
//     rejected with CHL_ERR_OOM.  The budget is released when the request's
//     answers are complete, whether or not its client has collected them;
//     an answered request keeps only its entry until chl_server_wait;
//   * batching: the server thread packs the pending pairs of many requests
//     (splitting large ones) into one launch of up to max_batch_pairs;
//   * overlap: kPipes batches are in flight at once, each on its own stream
//     (copy in, kernel, copy out), so new requests are admitted and launched
//     while earlier ones are still on the device;
//   * completion: answers are scattered back per request; chl_server_wait
//     returns them with the request's submit-to-completion latency.
// Every answer is computed by the same kernel as chl_query_batch, so a
// request's answers do not depend on what it was batched with.
#include "chl_dev.cuh"

#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

namespace chl {
int query_launch(const chl_labels *l, const uint32_t *d_pairs, size_t k, int32_t *d_out,
                 cudaStream_t s);
}

namespace {

constexpr int kPipes = 4;
using Clock = std::chrono::steady_clock;

struct Request {
    uint64_t id;
    size_t k;
    std::vector<uint32_t> pairs;
    std::vector<int32_t> out;
    size_t next = 0;        // next pair to batch
    size_t done = 0;        // answered pairs
    bool complete = false;
    Clock::time_point t0, t1;
};

struct Piece {
    Request *r;
    size_t off, cnt, pos;   // request offset, count, position in batch
};

struct Pipe {
    cudaStream_t st = nullptr;
    cudaEvent_t ev = nullptr;
    uint32_t *h_in = nullptr, *d_in = nullptr;
    int32_t *h_out = nullptr, *d_out = nullptr;
    std::vector<Piece> pieces;
    size_t count = 0;
    bool busy = false;
    uint64_t seq = 0;
};

}  // namespace

struct chl_server {
    const chl_labels *labels = nullptr;
    chl_server_opts opts{};
    std::mutex mu;
    std::condition_variable cv_work, cv_done, cv_space;
    std::deque<Request *> pending;
    std::unordered_map<uint64_t, Request *> table;
    size_t inflight_pairs = 0;      // admitted pairs not yet answered
    uint64_t next_id = 1;
    bool stop = false;
    int blocked = 0;                // callers inside submit / wait
    std::condition_variable cv_quit;
    Pipe pipes[kPipes];
    uint64_t launch_seq = 0;
    std::thread worker;
    uint64_t n_launch = 0, n_pairs = 0, n_req = 0;
    int error = CHL_OK;
};

namespace {

void finish_pipe(chl_server *s, Pipe &p) {
    // caller holds no lock; event already complete
    std::lock_guard<std::mutex> g(s->mu);
    for (const Piece &pc : p.pieces) {
        std::memcpy(pc.r->out.data() + pc.off, p.h_out + pc.pos, pc.cnt * 4);
        pc.r->done += pc.cnt;
        if (pc.r->done == pc.r->k) {
            pc.r->complete = true;
            pc.r->t1 = Clock::now();
            s->inflight_pairs -= pc.r->k;   // its staging is free again
        }
    }
    p.pieces.clear();
    p.busy = false;
    s->cv_done.notify_all();
    s->cv_space.notify_all();
}

void server_loop(chl_server *s) {
    int rr = 0;
    while (true) {
        // retire finished pipes
        for (Pipe &p : s->pipes)
            if (p.busy && cudaEventQuery(p.ev) == cudaSuccess) finish_pipe(s, p);
        std::unique_lock<std::mutex> lk(s->mu);
        bool any_busy = false;
        for (Pipe &p : s->pipes) any_busy |= p.busy;
        if (s->stop) {
            // requests not yet on the device are dropped (their callers were
            // told so by chl_server_free); batches in flight are retired
            s->pending.clear();
            if (!any_busy) break;
        }
        if (s->pending.empty()) {
            if (any_busy) {
                lk.unlock();
                // wait on the oldest busy pipe
                Pipe *old = nullptr;
                for (Pipe &p : s->pipes)
                    if (p.busy && (!old || p.seq < old->seq)) old = &p;
                cudaEventSynchronize(old->ev);
                continue;
            }
            s->cv_work.wait(lk, [&] { return s->stop || !s->pending.empty(); });
            continue;
        }
        // free pipe?
        Pipe *pp = nullptr;
        for (int i = 0; i < kPipes; ++i) {
            Pipe &p = s->pipes[(rr + i) % kPipes];
            if (!p.busy) {
                pp = &p;
                rr = (rr + i + 1) % kPipes;
                break;
            }
        }
        if (!pp) {
            lk.unlock();
            Pipe *old = nullptr;
            for (Pipe &p : s->pipes)
                if (p.busy && (!old || p.seq < old->seq)) old = &p;
            cudaEventSynchronize(old->ev);
            continue;
        }
        // form a batch from the pending queue (FIFO, splitting large requests)
        Pipe &p = *pp;
        p.count = 0;
        p.pieces.clear();
        const size_t cap = s->opts.max_batch_pairs;
        while (!s->pending.empty() && p.count < cap) {
            Request *r = s->pending.front();
            size_t take = std::min(r->k - r->next, cap - p.count);
            p.pieces.push_back(Piece{r, r->next, take, p.count});
            std::memcpy(p.h_in + 2 * p.count, r->pairs.data() + 2 * r->next, take * 8);
            r->next += take;
            p.count += take;
            if (r->next == r->k) s->pending.pop_front();
        }
        p.busy = true;
        p.seq = ++s->launch_seq;
        s->n_launch++;
        s->n_pairs += p.count;
        lk.unlock();
        cudaMemcpyAsync(p.d_in, p.h_in, p.count * 8, cudaMemcpyHostToDevice, p.st);
        int rc = chl::query_launch(s->labels, p.d_in, p.count, p.d_out, p.st);
        cudaMemcpyAsync(p.h_out, p.d_out, p.count * 4, cudaMemcpyDeviceToHost, p.st);
        cudaEventRecord(p.ev, p.st);
        if (rc != CHL_OK) {
            std::lock_guard<std::mutex> g(s->mu);
            s->error = rc;
        }
    }
}

}  // namespace

extern "C" void chl_server_opts_default(chl_server_opts *o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->max_inflight_pairs = 1u << 22;
    o->max_requests = 1u << 16;
    o->max_batch_pairs = 1u << 20;
}

extern "C" int chl_server_create(const chl_labels *l, const chl_server_opts *opts, chl_server **out) {
    if (!l || !out) return CHL_ERR_INVALID;
    int rc0 = chl::labels_ensure_device(l);
    if (rc0) return rc0;
    chl_server *s = new (std::nothrow) chl_server();
    if (!s) return CHL_ERR_OOM;
    s->labels = l;
    if (opts) s->opts = *opts;
    else chl_server_opts_default(&s->opts);
    if (s->opts.max_batch_pairs == 0 || s->opts.max_inflight_pairs == 0 || s->opts.max_requests == 0) {
        delete s;
        return CHL_ERR_INVALID;
    }
    const size_t B = s->opts.max_batch_pairs;
    for (Pipe &p : s->pipes) {
        cudaError_t e = cudaStreamCreateWithFlags(&p.st, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p.ev, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaMallocHost(&p.h_in, B * 8);
        if (e == cudaSuccess) e = cudaMallocHost(&p.h_out, B * 4);
        if (e == cudaSuccess) e = cudaMalloc(&p.d_in, B * 8);
        if (e == cudaSuccess) e = cudaMalloc(&p.d_out, B * 4);
        if (e != cudaSuccess) {
            int rc = chl::cuda_status(e, "server setup", __FILE__, __LINE__);
            chl_server_free(s);
            return rc;
        }
    }
    s->worker = std::thread(server_loop, s);
    *out = s;
    return CHL_OK;
}

extern "C" int chl_server_submit(chl_server *s, const uint32_t *pairs, size_t k, uint64_t *req_id) {
    if (!s || !req_id || (k && !pairs)) return CHL_ERR_INVALID;
    if (k > s->opts.max_inflight_pairs) return CHL_ERR_OOM;
    for (size_t i = 0; i < 2 * k; ++i)
        if (pairs[i] >= s->labels->n) return CHL_ERR_INVALID;
    Request *r = new (std::nothrow) Request();
    if (!r) return CHL_ERR_OOM;
    r->k = k;
    r->pairs.assign(pairs, pairs + 2 * k);
    r->out.assign(k, 0);
    std::unique_lock<std::mutex> lk(s->mu);
    if (s->stop) {
        delete r;
        return CHL_ERR_INVALID;
    }
    ++s->blocked;
    s->cv_space.wait(lk, [&] {
        return s->stop || (s->inflight_pairs + k <= s->opts.max_inflight_pairs &&
                           s->table.size() < s->opts.max_requests);
    });
    if (--s->blocked == 0 && s->stop) s->cv_quit.notify_all();
    if (s->stop) {
        delete r;
        return CHL_ERR_INVALID;   // the server is being freed
    }
    r->id = s->next_id++;
    r->t0 = Clock::now();
    s->inflight_pairs += k;
    s->table[r->id] = r;
    s->n_req++;
    if (k == 0) {
        r->complete = true;
        r->t1 = r->t0;
    } else {
        s->pending.push_back(r);
        s->cv_work.notify_one();
    }
    *req_id = r->id;
    return CHL_OK;
}

extern "C" int chl_server_wait(chl_server *s, uint64_t req_id, int32_t *out, double timeout_ms,
                               double *latency_ms) {
    if (!s) return CHL_ERR_INVALID;
    std::unique_lock<std::mutex> lk(s->mu);
    if (s->stop) return CHL_ERR_INVALID;
    auto it = s->table.find(req_id);
    if (it == s->table.end()) return CHL_ERR_INVALID;
    Request *r = it->second;
    auto ready = [&] { return s->stop || r->complete || s->error != CHL_OK; };
    ++s->blocked;
    bool timed_out = false;
    if (timeout_ms < 0) {
        s->cv_done.wait(lk, ready);
    } else {
        timed_out = !s->cv_done.wait_for(lk, std::chrono::duration<double, std::milli>(timeout_ms), ready);
    }
    if (--s->blocked == 0 && s->stop) s->cv_quit.notify_all();
    if (s->stop) return CHL_ERR_INVALID;   // the server is being freed: r may be gone
    if (timed_out) return CHL_ERR_TIMEOUT;
    if (!r->complete) return s->error;
    if (out && r->k) std::memcpy(out, r->out.data(), r->k * 4);
    if (latency_ms) *latency_ms = std::chrono::duration<double, std::milli>(r->t1 - r->t0).count();
    s->table.erase(it);
    delete r;
    s->cv_space.notify_all();
    return CHL_OK;
}

extern "C" int chl_server_blocked(chl_server *s, uint32_t *callers) {
    if (!s || !callers) return CHL_ERR_INVALID;
    std::lock_guard<std::mutex> g(s->mu);
    *callers = (uint32_t)s->blocked;
    return CHL_OK;
}

extern "C" int chl_server_stats(chl_server *s, uint64_t *launches, uint64_t *pairs, uint64_t *requests) {
    if (!s) return CHL_ERR_INVALID;
    std::lock_guard<std::mutex> g(s->mu);
    if (launches) *launches = s->n_launch;
    if (pairs) *pairs = s->n_pairs;
    if (requests) *requests = s->n_req;
    return CHL_OK;
}

extern "C" void chl_server_free(chl_server *s) {
    if (!s) return;
    {
        // fail every caller blocked in submit or wait, and wait until they
        // have left (after that, nothing of this server is touched by them)
        std::unique_lock<std::mutex> lk(s->mu);
        s->stop = true;
        s->cv_work.notify_all();
        s->cv_space.notify_all();
        s->cv_done.notify_all();
        s->cv_quit.wait(lk, [&] { return s->blocked == 0; });
    }
    if (s->worker.joinable()) s->worker.join();
    for (Pipe &p : s->pipes) {
        if (p.st) cudaStreamSynchronize(p.st);
        if (p.st) cudaStreamDestroy(p.st);
        if (p.ev) cudaEventDestroy(p.ev);
        cudaFreeHost(p.h_in);
        cudaFreeHost(p.h_out);
        cudaFree(p.d_in);
        cudaFree(p.d_out);
    }
    for (auto &kv : s->table) delete kv.second;
    delete s;
}
