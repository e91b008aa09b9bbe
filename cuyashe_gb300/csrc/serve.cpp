// serve.cpp -- continuous-batching request loop for YASHE homomorphic multiplies.
//
// The reference has no serving layer: each Ciphertext::operator* runs alone and
// synchronises the device (src/ciphertext.cpp:38-73, src/common.h:223). Here a
// dispatcher thread owns `streams` slots. It
//   * admits pending requests into a batch of one YASHE context and relin flag
//     (the oldest request's first, up to max_batch requests, FIFO within them)
//     when a slot is free and the device-memory budget has room for their
//     inputs, outputs and residue scratch;
//   * copies the batch's host ciphertexts into pinned staging (spread over a
//     small pool of copy threads, so that host copies do not serialise on the
//     dispatcher), then on the
//     slot's stream: one host-to-device copy, cy_yashe_mul_ws on the slot's own
//     workspace, one device-to-host copy, an event;
//   * retires batches whose event has completed, copies the results to the
//     callers' buffers, records latencies and frees the budget.
// Requests on device-resident ciphertexts (cy_server_submit_device) form their
// own batches: their inputs are gathered on the device into the slot's buffers
// and their products scattered to the callers' device buffers, with no host copy.
// Batches of different contexts and sizes run concurrently on different
// streams while new requests keep arriving. Evaluation keys stay resident in
// each cy_yashe. Waits are host-side and bounded (cy_server_wait takes a
// timeout); nothing on the GPU waits on anything.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "host.h"

namespace cy {

static double now_us() {
    return std::chrono::duration<double, std::micro>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

cy_status move_polys(uint64_t* const* d_ptrs, uint64_t* flat, int count, size_t words, bool gather,
                     cudaStream_t st);

struct Request {
    int cls = 0;
    int relin = 1;
    bool dev = false;                // buffers are device memory (cy_server_submit_device)
    const uint64_t* h_c1 = nullptr;  // host or device pointers, as `dev` says
    const uint64_t* h_c2 = nullptr;
    uint64_t* h_out = nullptr;
    double t_submit = 0;
    bool done = false;
    bool taken = false;  // admitted into a batch
    cy_status status = CY_OK;
    size_t bytes = 0;
};

// Host copies of a batch, spread over a few threads (the caller takes part).
struct CopyTask {
    void* dst;
    const void* src;
    size_t bytes;
};

class CopyPool {
   public:
    explicit CopyPool(int threads) {
        for (int i = 0; i < threads; i++) th_.emplace_back([this] { loop(); });
    }
    ~CopyPool() {
        {
            std::lock_guard<std::mutex> l(mu_);
            stop_ = true;
        }
        cv_.notify_all();
        for (auto& t : th_) t.join();
    }
    // Copies every task; returns when all are done.
    void run(const std::vector<CopyTask>& tasks) {
        if (tasks.size() < 4 || th_.empty()) {
            for (const CopyTask& t : tasks) std::memcpy(t.dst, t.src, t.bytes);
            return;
        }
        std::unique_lock<std::mutex> l(mu_);
        tasks_ = &tasks;
        next_.store(0);
        busy_ = (int)th_.size();
        gen_++;
        l.unlock();
        cv_.notify_all();
        work();
        l.lock();
        cv_done_.wait(l, [this] { return busy_ == 0; });
        tasks_ = nullptr;
    }

   private:
    void work() {
        const std::vector<CopyTask>& t = *tasks_;
        for (size_t i = next_.fetch_add(1); i < t.size(); i = next_.fetch_add(1)) std::memcpy(t[i].dst, t[i].src, t[i].bytes);
    }
    void loop() {
        uint64_t seen = 0;
        std::unique_lock<std::mutex> l(mu_);
        for (;;) {
            cv_.wait(l, [&] { return stop_ || gen_ != seen; });
            if (stop_) return;
            seen = gen_;
            l.unlock();
            work();
            l.lock();
            if (--busy_ == 0) cv_done_.notify_all();
        }
    }
    std::vector<std::thread> th_;
    std::mutex mu_;
    std::condition_variable cv_, cv_done_;
    const std::vector<CopyTask>* tasks_ = nullptr;
    std::atomic<size_t> next_{0};
    int busy_ = 0;
    uint64_t gen_ = 0;
    bool stop_ = false;
};

struct Slot {
    cudaStream_t st = nullptr;
    cudaEvent_t ev = nullptr;
    cudaEvent_t ev_start = nullptr;  // timing of the batch (time per request of its context)
    cy_workspace ws;
    bool busy = false;
    int cls = -1;
    std::vector<uint64_t> ids;
    size_t bytes = 0;
    size_t cap_words = 0;  // uint64 words of one device output buffer (inputs hold twice as many)
    size_t cap_host_words = 0;  // the same for the page-locked staging (host-buffer batches)
    uint64_t *d_in = nullptr, *d_out = nullptr, *h_in = nullptr, *h_out = nullptr;
    bool dev = false;            // the batch in flight is of device-resident requests
    size_t cap_ptrs = 0;         // pointer lists of device-resident batches
    uint64_t** h_ptrs = nullptr;  // page-locked: c1 of each request, then c2, then out
    uint64_t** d_ptrs = nullptr;
    ~Slot() {
        if (h_ptrs) cudaFreeHost(h_ptrs);
        if (d_ptrs) cudaFree(d_ptrs);
        if (d_in) cudaFree(d_in);
        if (d_out) cudaFree(d_out);
        if (h_in) cudaFreeHost(h_in);
        if (h_out) cudaFreeHost(h_out);
        if (ev) cudaEventDestroy(ev);
        if (ev_start) cudaEventDestroy(ev_start);
        if (st) cudaStreamDestroy(st);
    }
};

}  // namespace cy

using namespace cy;

struct cy_server {
    cy_server_config cfg{};
    int device = 0;
    std::vector<cy_yashe*> classes;
    std::vector<double> us_per_req;  // per context: running estimate (0: none yet)
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    // pending requests: one FIFO per (context, relin, device-resident) batch key,
    // and the submission order of all of them (the oldest request's key forms
    // the next batch; ids already taken are skipped lazily)
    std::map<int, std::deque<uint64_t>> queues;
    std::deque<uint64_t> order;
    size_t n_pending = 0;
    static int batch_key(const cy::Request& r) { return 4 * r.cls + 2 * r.relin + (r.dev ? 1 : 0); }
    void enqueue(uint64_t id, const cy::Request& r) {
        queues[batch_key(r)].push_back(id);
        order.push_back(id);
        n_pending++;
    }
    std::unordered_map<uint64_t, Request> reqs;
    uint64_t next_id = 1;
    std::vector<std::unique_ptr<Slot>> slots;
    std::unique_ptr<CopyPool> copies;
    size_t in_use = 0, peak = 0;
    bool stop = false;
    std::thread worker;
    // statistics
    std::vector<double> lat_us;
    uint64_t completed = 0, rejected = 0, batches = 0, failed = 0;
    double t_first = 0, t_last = 0;
    ~cy_server();
};

namespace cy {

static size_t request_bytes(const cy_yashe* y) {
    const size_t poly = (size_t)y->ring->n * y->ring->l64 * sizeof(uint64_t);
    const size_t resid = (size_t)std::max(y->tensor.h.k, y->relin.h.k) * y->ring->n * sizeof(uint32_t);
    return 3 * poly + resid;
}

// Slots serve every registered context, whose polynomials differ in size:
// capacity is counted in words, not polynomials.
// Growing frees and allocates (cudaFree waits for the whole device), so a slot
// grows to twice what the batch needs: few growths once the load settles.
static cy_status grow_slot(Slot& s, size_t polys, size_t poly_words, bool host) {
    const size_t need = polys * poly_words;
    if (need > s.cap_words) {  // device buffers
        const size_t words = std::max(2 * need, 2 * s.cap_words);
        if (s.d_in) cudaFree(s.d_in);
        if (s.d_out) cudaFree(s.d_out);
        s.d_in = s.d_out = nullptr;
        s.cap_words = 0;
        CY_CUDA(cudaMalloc(&s.d_in, 2 * words * sizeof(uint64_t)));
        CY_CUDA(cudaMalloc(&s.d_out, words * sizeof(uint64_t)));
        s.cap_words = words;
    }
    if (host && need > s.cap_host_words) {  // page-locked staging: host-buffer batches only
        const size_t words = std::max(2 * need, 2 * s.cap_host_words);
        if (s.h_in) cudaFreeHost(s.h_in);
        if (s.h_out) cudaFreeHost(s.h_out);
        s.h_in = s.h_out = nullptr;
        s.cap_host_words = 0;
        CY_CUDA(cudaMallocHost(&s.h_in, 2 * words * sizeof(uint64_t)));
        CY_CUDA(cudaMallocHost(&s.h_out, words * sizeof(uint64_t)));
        s.cap_host_words = words;
    }
    return CY_OK;
}

static cy_status grow_ptrs(Slot& s, size_t n) {
    if (n <= s.cap_ptrs) return CY_OK;
    const size_t want = std::max(2 * n, 2 * s.cap_ptrs);
    if (s.h_ptrs) cudaFreeHost(s.h_ptrs);
    if (s.d_ptrs) cudaFree(s.d_ptrs);
    s.h_ptrs = s.d_ptrs = nullptr;
    s.cap_ptrs = 0;
    CY_CUDA(cudaMallocHost(&s.h_ptrs, want * sizeof(uint64_t*)));
    CY_CUDA(cudaMalloc(&s.d_ptrs, want * sizeof(uint64_t*)));
    s.cap_ptrs = want;
    return CY_OK;
}

// One pass of the dispatcher. Bookkeeping happens under the lock; copies into
// and out of the callers' buffers and the launches happen without it, so that
// submitters are never held up by a batch being prepared. Only this thread
// touches the slots.
static void dispatch_once(cy_server* S, std::unique_lock<std::mutex>& lock) {
    // 1. completed batches: collect under the lock, copy out without it
    struct Done {
        Slot* s;
        cy_status st;
        std::vector<uint64_t*> outs;
        size_t poly;
    };
    std::vector<Done> done;
    for (auto& sp : S->slots) {
        Slot& s = *sp;
        if (!s.busy) continue;
        const cudaError_t q = cudaEventQuery(s.ev);
        if (q == cudaErrorNotReady) continue;
        Done d{&s, q == cudaSuccess ? CY_OK : cuda_error(q, "serving batch"), {}, 0};
        float ms = 0;
        if (q == cudaSuccess && cudaEventElapsedTime(&ms, s.ev_start, s.ev) == cudaSuccess && !s.ids.empty()) {
            const double per = 1000.0 * ms / (double)s.ids.size();
            double& est = S->us_per_req[s.cls];
            est = est > 0 ? 0.8 * est + 0.2 * per : per;
        }
        const cy_yashe* y = S->classes[s.cls];
        d.poly = (size_t)y->ring->n * y->ring->l64;
        if (s.ids.size() * d.poly > (s.dev ? s.cap_words : s.cap_host_words))
            d.st = set_error(CY_ERR_INTERNAL, "serving slot too small");
        if (!s.dev)  // device-resident results are already in the callers' buffers
            for (uint64_t id : s.ids) d.outs.push_back(S->reqs[id].h_out);
        done.push_back(std::move(d));
    }
    if (!done.empty()) {
        lock.unlock();
        std::vector<CopyTask> tasks;
        for (const Done& d : done)
            if (d.st == CY_OK)
                for (size_t i = 0; i < d.outs.size(); i++)
                    tasks.push_back({d.outs[i], d.s->h_out + i * d.poly, d.poly * sizeof(uint64_t)});
        S->copies->run(tasks);
        lock.lock();
        const double t = now_us();
        for (const Done& d : done) {
            for (uint64_t id : d.s->ids) {
                Request& r = S->reqs[id];
                r.status = d.st;
                r.done = true;
                S->lat_us.push_back(t - r.t_submit);
                if (d.st == CY_OK) S->completed++;
                else S->failed++;
            }
            S->t_last = t;
            S->in_use -= d.s->bytes;
            d.s->busy = false;
            d.s->ids.clear();
        }
        S->cv_done.notify_all();
    }

    // 2. new batches on free slots: choose under the lock, stage and launch without it
    for (auto& sp : S->slots) {
        Slot& s = *sp;
        if (s.busy || S->n_pending == 0) continue;
        while (!S->order.empty()) {  // drop ids already admitted (or already waited for)
            auto f = S->reqs.find(S->order.front());
            if (f != S->reqs.end() && !f->second.taken) break;
            S->order.pop_front();
        }
        if (S->order.empty()) continue;
        const Request& oldest = S->reqs[S->order.front()];
        const int cls = oldest.cls;
        const int relin = oldest.relin;
        const bool dev = oldest.dev;
        std::deque<uint64_t>& q = S->queues[cy_server::batch_key(oldest)];
        cy_yashe* y = S->classes[cls];
        const size_t per = request_bytes(y);
        int cap = S->cfg.max_batch;  // requests of this batch
        if (S->cfg.batch_budget_us > 0 && S->us_per_req[cls] > 0)
            cap = std::max(1, std::min(cap, (int)(S->cfg.batch_budget_us / S->us_per_req[cls])));
        std::vector<uint64_t> take;
        std::vector<const uint64_t*> in1, in2;
        std::vector<uint64_t*> outs;
        size_t bytes = 0;
        while (!q.empty() && (int)take.size() < cap) {
            Request& r = S->reqs[q.front()];
            if (S->in_use + bytes + per > S->cfg.device_budget_bytes) break;  // admission by device memory
            take.push_back(q.front());
            in1.push_back(r.h_c1);
            in2.push_back(r.h_c2);
            outs.push_back(r.h_out);
            r.taken = true;
            bytes += per;
            q.pop_front();
            S->n_pending--;
        }
        if (take.empty()) break;  // the budget is full until a batch retires
        s.busy = true;  // reserved: not retired before its event is recorded below
        s.dev = dev;
        s.cls = cls;
        s.ids = take;
        s.bytes = bytes;
        S->in_use += bytes;
        S->peak = std::max(S->peak, S->in_use);
        S->batches++;
        lock.unlock();
        const int nb = (int)take.size();
        const size_t poly = (size_t)y->ring->n * y->ring->l64;
        cy_status st = grow_slot(s, nb, poly, !dev);
        if (st == CY_OK && ((size_t)nb * poly > s.cap_words || (!dev && (size_t)nb * poly > s.cap_host_words)))
            st = set_error(CY_ERR_INTERNAL, "serving slot too small");
        if (st == CY_OK && dev) {
            // device-resident: pointer lists in, gather, multiply, scatter
            st = grow_ptrs(s, 3 * (size_t)nb);
            if (st == CY_OK) {
                for (int i = 0; i < nb; i++) {
                    s.h_ptrs[i] = const_cast<uint64_t*>(in1[i]);
                    s.h_ptrs[nb + i] = const_cast<uint64_t*>(in2[i]);
                    s.h_ptrs[2 * nb + i] = outs[i];
                }
                cudaError_t e = cudaEventRecord(s.ev_start, s.st);
                if (e == cudaSuccess)
                    e = cudaMemcpyAsync(s.d_ptrs, s.h_ptrs, 3 * nb * sizeof(uint64_t*), cudaMemcpyHostToDevice, s.st);
                if (e != cudaSuccess) st = cuda_error(e, "serving pointer lists");
            }
            if (st == CY_OK) st = move_polys(s.d_ptrs, s.d_in, 2 * nb, poly, true, s.st);
            if (st == CY_OK) st = cy_yashe_mul_ws(y, &s.ws, s.d_in, s.d_in + nb * poly, s.d_out, nb, relin, s.st);
            if (st == CY_OK) st = move_polys(s.d_ptrs + 2 * nb, s.d_out, nb, poly, false, s.st);
            if (st == CY_OK) {
                const cudaError_t e = cudaEventRecord(s.ev, s.st);
                if (e != cudaSuccess) st = cuda_error(e, "serving event");
            }
        } else if (st == CY_OK) {
            std::vector<CopyTask> tasks;
            tasks.reserve(2 * nb);
            for (int i = 0; i < nb; i++) {
                tasks.push_back({s.h_in + i * poly, in1[i], poly * sizeof(uint64_t)});
                tasks.push_back({s.h_in + (nb + i) * poly, in2[i], poly * sizeof(uint64_t)});
            }
            S->copies->run(tasks);
            cudaError_t e = cudaEventRecord(s.ev_start, s.st);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(s.d_in, s.h_in, 2 * nb * poly * sizeof(uint64_t), cudaMemcpyHostToDevice, s.st);
            if (e != cudaSuccess) st = cuda_error(e, "serving H2D");
            if (st == CY_OK) st = cy_yashe_mul_ws(y, &s.ws, s.d_in, s.d_in + nb * poly, s.d_out, nb, relin, s.st);
            if (st == CY_OK) {
                e = cudaMemcpyAsync(s.h_out, s.d_out, nb * poly * sizeof(uint64_t), cudaMemcpyDeviceToHost, s.st);
                if (e == cudaSuccess) e = cudaEventRecord(s.ev, s.st);
                if (e != cudaSuccess) st = cuda_error(e, "serving D2H");
            }
        }
        lock.lock();
        if (st != CY_OK) {  // fail the batch on the host
            for (uint64_t id : take) {
                Request& r = S->reqs[id];
                r.status = st;
                r.done = true;
                S->failed++;
            }
            S->in_use -= bytes;
            s.busy = false;
            s.ids.clear();
            S->cv_done.notify_all();
        }
    }
}

static void worker_loop(cy_server* S) {
    cudaSetDevice(S->device);
    std::unique_lock<std::mutex> lock(S->mu);
    while (!S->stop) {
        dispatch_once(S, lock);
        bool busy = false;
        for (auto& s : S->slots) busy |= s->busy;
        if (busy || S->n_pending > 0) {
            // poll the slots' events without holding the lock
            lock.unlock();
            std::this_thread::sleep_for(std::chrono::microseconds(S->cfg.poll_us));
            lock.lock();
        } else {
            S->cv_work.wait_for(lock, std::chrono::milliseconds(5));
        }
    }
}

}  // namespace cy

cy_server::~cy_server() {
    {
        std::lock_guard<std::mutex> lock(mu);
        stop = true;
    }
    cv_work.notify_all();
    if (worker.joinable()) worker.join();
    for (auto& s : slots)
        if (s->busy) cudaEventSynchronize(s->ev);
}

extern "C" {

cy_status cy_server_create(const cy_server_config* cfg, cy_server** out) {
    if (!cfg || !out) return set_error(CY_ERR_INVALID_ARGUMENT, "NULL argument");
    if (cfg->streams < 1 || cfg->streams > 32 || cfg->max_batch < 1 || cfg->device_budget_bytes == 0 ||
        cfg->batch_budget_us < 0)
        return set_error(CY_ERR_INVALID_ARGUMENT,
                         "streams must be 1..32, max_batch >= 1, budget > 0, batch_budget_us >= 0");
    std::unique_ptr<cy_server> S(new cy_server());
    S->cfg = *cfg;
    if (S->cfg.poll_us <= 0) S->cfg.poll_us = 20;
    CY_CUDA(cudaGetDevice(&S->device));
    for (int i = 0; i < cfg->streams; i++) {
        std::unique_ptr<Slot> s(new Slot());
        CY_CUDA(cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking));
        CY_CUDA(cudaEventCreate(&s->ev));  // timed: batch time per request of its context
        CY_CUDA(cudaEventCreate(&s->ev_start));
        s->ws.ws.device = S->device;
        S->slots.push_back(std::move(s));
    }
    S->copies.reset(new CopyPool(3));
    S->worker = std::thread(worker_loop, S.get());
    *out = S.release();
    return CY_OK;
}

cy_status cy_server_destroy(cy_server* s) {
    delete s;
    return CY_OK;
}

cy_status cy_server_register(cy_server* S, cy_yashe* y, int* class_id) {
    if (!S || !y || !class_id) return set_error(CY_ERR_INVALID_ARGUMENT, "NULL argument");
    if (!y->has_keys) return set_error(CY_ERR_NO_KEYS, "context has no keys");
    std::lock_guard<std::mutex> lock(S->mu);
    S->classes.push_back(y);
    S->us_per_req.push_back(0.0);
    *class_id = (int)S->classes.size() - 1;
    return CY_OK;
}

cy_status cy_server_submit(cy_server* S, const cy_serve_request* req, uint64_t* ticket) {
    if (!S || !req || !ticket) return set_error(CY_ERR_INVALID_ARGUMENT, "NULL argument");
    std::lock_guard<std::mutex> lock(S->mu);
    if (req->class_id < 0 || req->class_id >= (int)S->classes.size() || !req->h_c1 || !req->h_c2 || !req->h_out) {
        S->rejected++;
        return set_error(CY_ERR_INVALID_ARGUMENT, "request with an unknown class or NULL buffers");
    }
    const size_t bytes = request_bytes(S->classes[req->class_id]);
    if (bytes > S->cfg.device_budget_bytes) {
        S->rejected++;
        return set_error(CY_ERR_OUT_OF_MEMORY, "one request needs more device memory than the whole budget");
    }
    Request r;
    r.cls = req->class_id;
    r.relin = req->relin ? 1 : 0;
    r.h_c1 = req->h_c1;
    r.h_c2 = req->h_c2;
    r.h_out = req->h_out;
    r.t_submit = now_us();
    r.bytes = bytes;
    if (S->t_first == 0) S->t_first = r.t_submit;
    const uint64_t id = S->next_id++;
    S->reqs[id] = r;
    S->enqueue(id, r);
    *ticket = id;
    S->cv_work.notify_one();
    return CY_OK;
}

cy_status cy_server_submit_device(cy_server* S, const cy_serve_request_dev* reqs, int n, uint64_t* tickets) {
    if (!S || (n > 0 && (!reqs || !tickets)) || n < 0) return set_error(CY_ERR_INVALID_ARGUMENT, "NULL argument");
    std::lock_guard<std::mutex> lock(S->mu);
    const double t = now_us();
    for (int i = 0; i < n; i++) {
        const cy_serve_request_dev& q = reqs[i];
        if (q.class_id < 0 || q.class_id >= (int)S->classes.size() || !q.d_c1 || !q.d_c2 || !q.d_out ||
            (((uintptr_t)q.d_c1 | (uintptr_t)q.d_c2 | (uintptr_t)q.d_out) & 15)) {
            S->rejected++;
            return set_error(CY_ERR_INVALID_ARGUMENT,
                             "device request with an unknown class, NULL or unaligned buffers (index " +
                                 std::to_string(i) + ")");
        }
        const size_t bytes = request_bytes(S->classes[q.class_id]);
        if (bytes > S->cfg.device_budget_bytes) {
            S->rejected++;
            return set_error(CY_ERR_OUT_OF_MEMORY, "one request needs more device memory than the whole budget");
        }
        Request r;
        r.cls = q.class_id;
        r.relin = q.relin ? 1 : 0;
        r.dev = true;
        r.h_c1 = q.d_c1;
        r.h_c2 = q.d_c2;
        r.h_out = q.d_out;
        r.t_submit = t;
        r.bytes = bytes;
        if (S->t_first == 0) S->t_first = t;
        const uint64_t id = S->next_id++;
        S->reqs[id] = r;
        S->enqueue(id, r);
        tickets[i] = id;
    }
    S->cv_work.notify_one();
    return CY_OK;
}

cy_status cy_server_poll(cy_server* S, uint64_t ticket, int* done) {
    if (!S || !done) return set_error(CY_ERR_INVALID_ARGUMENT, "NULL argument");
    std::lock_guard<std::mutex> lock(S->mu);
    auto it = S->reqs.find(ticket);
    if (it == S->reqs.end()) return set_error(CY_ERR_INVALID_ARGUMENT, "unknown ticket");
    *done = it->second.done ? 1 : 0;
    return CY_OK;
}

cy_status cy_server_wait(cy_server* S, uint64_t ticket, int timeout_ms) {
    if (!S) return set_error(CY_ERR_INVALID_ARGUMENT, "NULL argument");
    std::unique_lock<std::mutex> lock(S->mu);
    auto it = S->reqs.find(ticket);
    if (it == S->reqs.end()) return set_error(CY_ERR_INVALID_ARGUMENT, "unknown ticket");
    const bool ok = S->cv_done.wait_for(lock, std::chrono::milliseconds(timeout_ms),
                                        [&] { return S->reqs[ticket].done; });
    if (!ok) return set_error(CY_ERR_TIMEOUT, "request not finished before the deadline");
    const cy_status st = S->reqs[ticket].status;
    S->reqs.erase(ticket);
    return st;
}

cy_status cy_server_drain(cy_server* S, int timeout_ms) {
    if (!S) return set_error(CY_ERR_INVALID_ARGUMENT, "NULL argument");
    std::unique_lock<std::mutex> lock(S->mu);
    const bool ok = S->cv_done.wait_for(lock, std::chrono::milliseconds(timeout_ms), [&] {
        if (S->n_pending > 0) return false;
        for (auto& s : S->slots)
            if (s->busy) return false;
        return true;
    });
    return ok ? CY_OK : set_error(CY_ERR_TIMEOUT, "requests still running at the deadline");
}

cy_status cy_server_get_stats(cy_server* S, cy_server_stats* out) {
    if (!S || !out) return set_error(CY_ERR_INVALID_ARGUMENT, "NULL argument");
    std::lock_guard<std::mutex> lock(S->mu);
    std::memset(out, 0, sizeof(*out));
    out->completed = S->completed;
    out->rejected = S->rejected;
    out->failed = S->failed;
    out->batches = S->batches;
    out->peak_device_bytes = S->peak;
    std::vector<double> v = S->lat_us;
    if (!v.empty()) {
        std::sort(v.begin(), v.end());
        auto pct = [&](double p) { return v[std::min(v.size() - 1, (size_t)(p * (v.size() - 1) + 0.5))]; };
        out->p50_us = pct(0.50);
        out->p99_us = pct(0.99);
        double sum = 0;
        for (double x : v) sum += x;
        out->mean_us = sum / v.size();
    }
    if (S->t_last > S->t_first) out->throughput_per_s = S->completed / ((S->t_last - S->t_first) * 1e-6);
    return CY_OK;
}

cy_status cy_server_reset_stats(cy_server* S) {
    if (!S) return set_error(CY_ERR_INVALID_ARGUMENT, "NULL argument");
    std::lock_guard<std::mutex> lock(S->mu);
    S->lat_us.clear();
    S->completed = S->rejected = S->batches = S->failed = 0;
    S->t_first = S->t_last = 0;
    S->peak = S->in_use;
    return CY_OK;
}

}  // extern "C"
