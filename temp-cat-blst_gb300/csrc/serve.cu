// Serving engine: continuous batching of MSM and G1 FFT requests on one GPU
// (no reference counterpart; the reference is a synchronous library).
//
// State kept resident in HBM: the basis and its fixed-base tables (a Basis
// from batch.cu).  Requests arrive from any host thread:
//   MSM  over the first k basis points with k 32-byte scalars;
//   FFT  of n Jacobian points with a prepared domain (forward / inverse /
//        inverse unscaled), in place.
// W worker threads each own a CUDA stream and a workspace.  Whenever a worker
// is free it takes the OLDEST queued request and, as one batch, every other
// queued request of the same size class (MSMs: k in the same power-of-four
// band; FFTs: the same n), up to a point cap -- so requests that arrived
// while other batches ran join at the next batch boundary, a small MSM never
// waits inside a batch of large ones, and batches of different workers
// overlap on the device.  Worker 0 runs on the device's highest-priority
// stream and takes the oldest large request first (see is_large); while a
// large batch runs, other batches start only after a short hold (kHoldMs).  MSMs of at
// least kPlainMinPoints points, and a batch of a single MSM, run through the
// plain pipeline (GLV split, batch-affine rounds) over the basis points,
// which beats the fixed-base tables there; batches of several smaller ones
// run as one batched launch over the tables.  Admission is by HBM budget: a batch starts only while the
// estimated device memory of all in-flight batches stays within the budget
// (a single request above the budget runs alone).  Every request records
// submit/start/done times on the host's steady clock.
#include "common.cuh"
#include "catmsm_internal.h"
#include "catmsm_gpu.h"

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <new>
#include <thread>
#include <unordered_map>
#include <vector>

namespace catmsm {

namespace {

double now_ms()
{
    using namespace std::chrono;
    return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

struct Request {
    int64_t id = 0;
    int type = 0;                       // 0 MSM, 1 FFT
    const uint8_t* scalars = nullptr;   // MSM
    size_t k = 0;
    blst_p1 result;
    blst_p1* values = nullptr;          // FFT
    size_t n = 0;
    const blst_fr* domain = nullptr;
    int mode = 0;
    size_t mem = 0;                     // admission estimate, bytes
    double t_submit = 0, t_start = 0, t_done = 0;
    int status = 0;
    bool done = false;
    bool claimed = false;               // a wait call owns it (a ticket is waited once)
};

struct Server;

struct Worker {
    Server* s = nullptr;
    std::thread th;
    BatchWork* work = nullptr;
    int index = 0;
};

struct Server {
    Basis* basis = nullptr;
    int device = 0;
    size_t budget = 0, inflight = 0;
    size_t msm_cap = 0, fft_cap = 0;    // points per batch
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Request*> queue;
    std::unordered_map<int64_t, Request*> reqs;
    int64_t next_id = 1;
    bool stop = false;
    std::vector<Worker*> workers;
    // stats
    long batches = 0, batched_reqs = 0, max_batch = 0;
    long running = 0, max_running = 0;   // batches executing at once
    long large_running = 0;              // of those, batches of large requests
};

// While a large batch runs, another batch starts only once its oldest request
// has waited this long: at light load a large job (the latency tail) then
// runs without co-resident work slowing it, and under load the queue still
// drains concurrently after a bounded delay.
constexpr double kHoldMs = 10.0;

// MSMs of at least this many points take the plain pipeline (msm.cu), and
// so does a batch of one MSM of any size: for a lone request the fixed-base
// tables' batched launch sequence is slower (measured on the 2^22-point basis,
// c = 13: 2^12 points 0.66 against 0.44 ms, 2^16 1.61 against 0.98, 2^17 2.58
// against 1.51); the tables win once several MSMs share one batch.
constexpr size_t kPlainMinPoints = size_t(1) << 18;

// Large requests (FFTs of at least 2^14 points, MSMs of at least 2^20):
// worker 0 runs on the device's highest-priority stream and takes the oldest
// large request first, so the longest jobs -- the latency tail -- get SMs
// ahead of the small batches that share the GPU with them.
bool is_large(const Request* r) { return r->type == 0 ? r->k >= (size_t(1) << 20) : r->n >= (size_t(1) << 14); }

// Size class: requests of one class are batched together.
int req_class(const Request* r)
{
    size_t x = r->type == 0 ? r->k : r->n;
    int lg = 0;
    while (x > 1) {
        x >>= 1;
        lg++;
    }
    return r->type == 0 ? lg / 2 : 64 + lg;
}

size_t msm_mem(const Basis* b, size_t k)
{
    // the plain pipeline's workspace: ~14 bucket entries per point (GLV halves
    // over 7-8 windows), each with its index/key/rank words, its slots in the
    // two batch-affine lists and a share of the prefix products (~240 B)
    const size_t plain = k * 3400 + ((size_t)64 << 20);
    if (k >= kPlainMinPoints) return plain;
    // a smaller MSM runs over the tables in a batch, or through the plain
    // pipeline alone: the larger of the two
    const size_t D = 256 / basis_window(b) + 1;
    const size_t table = k * D * 24 + ((size_t)1 << (basis_window(b) - 1)) * 192 * 2 + k * 32 + (1 << 20);
    return std::max(plain, table);
}

size_t fft_mem(size_t n) { return n * 144 * 2 + n * 64 + (1 << 20); }

// A large MSM through the plain pipeline over the basis points: the scalars
// are copied to the worker context's device buffer first.
int run_plain_msm(Server* s, Ctx* ctx, Request* r)
{
    uint8_t* d_sc = (uint8_t*)ctx->msm.scalars.get(r->k * 32);
    if (!d_sc) return (int)cudaErrorMemoryAllocation;
    cudaError_t err = cudaMemcpyAsync(d_sc, r->scalars, r->k * 32, cudaMemcpyHostToDevice, ctx->stream);
    uint64_t out[18];
    if (err == cudaSuccess) err = msm_device(ctx, basis_points_device(s->basis), d_sc, 32, r->k, 256, 0, out);
    if (err != cudaSuccess) return (int)err;
    std::memcpy(&r->result, out, sizeof(blst_p1));
    return 0;
}

void worker_main(Worker* wk)
{
    Server* s = wk->s;
    cudaSetDevice(s->device);
    Ctx* ctx = get_ctx();
    if (ctx && wk->index == 0) {
        int least = 0, greatest = 0;
        cudaStream_t ps = nullptr;
        if (cudaDeviceGetStreamPriorityRange(&least, &greatest) == cudaSuccess &&
            cudaStreamCreateWithPriority(&ps, cudaStreamNonBlocking, greatest) == cudaSuccess) {
            cudaStreamSynchronize(ctx->stream);
            cudaStreamDestroy(ctx->stream);
            ctx->stream = ps;
        }
    }
    for (;;) {
        std::vector<Request*> batch;
        size_t mem = 0;
        bool large = false;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            const Request* head = nullptr;
            for (;;) {
                if (s->stop && s->queue.empty()) return;
                head = nullptr;
                if (!s->queue.empty()) {
                    head = s->queue.front();
                    if (wk->index == 0)
                        for (const Request* r : s->queue)
                            if (is_large(r)) {
                                head = r;
                                break;
                            }
                    const bool fits = s->inflight + head->mem <= s->budget || s->inflight == 0;
                    const double waited = now_ms() - head->t_submit;
                    if (fits && (s->large_running == 0 || waited >= kHoldMs)) break;
                    if (fits) {
                        s->cv_work.wait_for(lk, std::chrono::microseconds((long)((kHoldMs - waited) * 1000) + 100));
                        continue;
                    }
                }
                s->cv_work.wait(lk);
            }
            large = is_large(head);
            const int type = head->type, cls = req_class(head);
            const size_t cap = type == 0 ? s->msm_cap : s->fft_cap;
            size_t pts = 0;
            for (auto it = s->queue.begin(); it != s->queue.end();) {
                Request* r = *it;
                const size_t rp = type == 0 ? r->k : r->n;
                if (r->type != type || req_class(r) != cls) {
                    ++it;
                    continue;
                }
                const bool first = batch.empty();
                if (!first && (pts + rp > cap || s->inflight + mem + r->mem > s->budget)) break;
                batch.push_back(r);
                pts += rp;
                mem += r->mem;
                it = s->queue.erase(it);
            }
            s->inflight += mem;
            s->batches++;
            s->batched_reqs += (long)batch.size();
            s->max_batch = std::max<long>(s->max_batch, (long)batch.size());
            s->running++;
            s->max_running = std::max(s->max_running, s->running);
            if (large) s->large_running++;
        }
        const double t0 = now_ms();
        for (Request* r : batch) r->t_start = t0;
        int rc = 0;
        if (!ctx) {
            rc = (int)cudaErrorInitializationError;
        } else if (batch[0]->type == 0 && (batch[0]->k >= kPlainMinPoints || batch.size() == 1)) {
            for (Request* r : batch) {
                const int e = run_plain_msm(s, ctx, r);
                if (e && !rc) rc = e;
            }
        } else if (batch[0]->type == 0) {
            std::vector<size_t> counts(batch.size());
            size_t total = 0;
            for (size_t j = 0; j < batch.size(); j++) {
                counts[j] = batch[j]->k;
                total += batch[j]->k;
            }
            std::vector<uint8_t> sc(total * 32 + 32);
            size_t off = 0;
            for (Request* r : batch) {
                std::memcpy(sc.data() + off, r->scalars, r->k * 32);
                off += r->k * 32;
            }
            std::vector<blst_p1> out(batch.size());
            rc = (int)batch_run(s->basis, wk->work, ctx->stream, out.data(), (uint32_t)batch.size(), counts.data(),
                                sc.data());
            for (size_t j = 0; j < batch.size(); j++) batch[j]->result = out[j];
        } else {
            std::vector<blst_p1*> vals;
            std::vector<size_t> ns;
            std::vector<const blst_fr*> doms;
            std::vector<int> modes;
            for (Request* r : batch) {
                vals.push_back(r->values);
                ns.push_back(r->n);
                doms.push_back(r->domain);
                modes.push_back(r->mode);
            }
            rc = catmsm_p1_fft_batch(vals.data(), ns.data(), doms.data(), modes.data(), batch.size());
        }
        const double t1 = now_ms();
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->inflight -= mem;
            s->running--;
            if (large) s->large_running--;
            for (Request* r : batch) {
                r->status = rc;
                r->t_done = t1;
                r->done = true;
            }
        }
        s->cv_done.notify_all();
        s->cv_work.notify_all();
    }
}

int64_t submit(Server* s, Request* r)
{
    r->t_submit = now_ms();
    int64_t id;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        id = s->next_id++;
        r->id = id;
        s->reqs[id] = r;
        s->queue.push_back(r);
    }
    s->cv_work.notify_one();
    return id;
}

}  // namespace
}  // namespace catmsm

using namespace catmsm;

extern "C" {

void* catmsm_server_create(void* basis, size_t workers, size_t hbm_budget_bytes)
{
    if (!basis || workers == 0 || workers > 64) return nullptr;
    Server* s = new (std::nothrow) Server();
    if (!s) return nullptr;
    s->basis = (Basis*)basis;
    s->device = basis_device(s->basis);
    s->budget = hbm_budget_bytes ? hbm_budget_bytes : ((size_t)64 << 30);
    s->msm_cap = std::max<size_t>(basis_points(s->basis), (size_t)1 << 22);
    s->fft_cap = (size_t)1 << 20;
    for (size_t i = 0; i < workers; i++) {
        Worker* w = new (std::nothrow) Worker();
        if (!w) break;
        w->s = s;
        w->work = batch_work_new();
        if (!w->work) {
            delete w;
            break;
        }
        s->workers.push_back(w);
    }
    if (s->workers.empty()) {
        delete s;
        return nullptr;
    }
    for (size_t i = 0; i < s->workers.size(); i++) s->workers[i]->index = (int)i;
    for (Worker* w : s->workers) w->th = std::thread(worker_main, w);
    return s;
}

void catmsm_server_destroy(void* server)
{
    Server* s = (Server*)server;
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    for (Worker* w : s->workers) {
        if (w->th.joinable()) w->th.join();
        batch_work_free(w->work);
        delete w;
    }
    for (auto& kv : s->reqs) delete kv.second;
    delete s;
}

int64_t catmsm_server_submit_msm(void* server, const blst_byte* scalars, size_t k)
{
    Server* s = (Server*)server;
    if (!s || !scalars || k == 0 || k > basis_points(s->basis)) return -1;
    Request* r = new (std::nothrow) Request();
    if (!r) return -1;
    r->type = 0;
    r->scalars = scalars;
    r->k = k;
    r->mem = msm_mem(s->basis, k);
    return submit(s, r);
}

int64_t catmsm_server_submit_fft(void* server, blst_p1* values, size_t n, const blst_fr* domain, int mode)
{
    Server* s = (Server*)server;
    if (!s || !values || !domain || n == 0 || (n & (n - 1)) || mode < 0 || mode > 2) return -1;
    Request* r = new (std::nothrow) Request();
    if (!r) return -1;
    r->type = 1;
    r->values = values;
    r->n = n;
    r->domain = domain;
    r->mode = mode;
    r->mem = fft_mem(n);
    return submit(s, r);
}

int catmsm_server_wait(void* server, int64_t ticket, blst_p1* msm_out, double* times_ms)
{
    Server* s = (Server*)server;
    if (!s) return (int)cudaErrorInvalidValue;
    Request* r = nullptr;
    {
        // The lock is released while waiting and a submit may rehash the
        // map, so the entry is erased by key afterwards, not by iterator.
        std::unique_lock<std::mutex> lk(s->mu);
        auto it = s->reqs.find(ticket);
        if (it == s->reqs.end() || it->second->claimed) return (int)cudaErrorInvalidValue;
        r = it->second;
        r->claimed = true;
        s->cv_done.wait(lk, [&] { return r->done; });
        s->reqs.erase(ticket);
    }
    if (msm_out && r->type == 0) *msm_out = r->result;
    if (times_ms) {
        times_ms[0] = r->t_start - r->t_submit;   // queueing
        times_ms[1] = r->t_done - r->t_submit;    // latency
    }
    const int rc = r->status;
    delete r;
    return rc;
}

int catmsm_server_stats(void* server, long* batches, long* batched_requests, long* max_batch,
                        long* max_concurrent)
{
    Server* s = (Server*)server;
    if (!s) return (int)cudaErrorInvalidValue;
    std::lock_guard<std::mutex> lk(s->mu);
    if (batches) *batches = s->batches;
    if (batched_requests) *batched_requests = s->batched_reqs;
    if (max_batch) *max_batch = s->max_batch;
    if (max_concurrent) *max_concurrent = s->max_running;
    return 0;
}

}  // extern "C"
