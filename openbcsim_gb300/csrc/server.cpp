// server.cpp -- continuous-batching request server.
//
// Phantoms (configured simulators: scatterers, beam, excitation, parameters)
// stay resident on the device.  A request asks for some scan lines of one
// phantom (origins, directions, timestamps, line length, decimation).  One worker
// thread admits queued requests in arrival order as soon as a simulator slot of
// their phantom is free -- creating slots while the device-memory budget allows
// -- prepares them on the host and enqueues their device work on the slot's own
// stream, so requests that arrive while others are on the GPU overlap with them.
// The same thread polls completion events, copies results out and records the
// submit-to-result latency.  A request's result depends only on its phantom and
// its own lines, never on what else is in flight.
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
#include <vector>

#include "../../include/bcsim_gb300.h"
#include "engine.hpp"

struct bcsim_handle;
namespace bcsim_gb300 {
Simulator& simulator_of(bcsim_handle* h);
}
using bcsim_gb300::SimError;
using bcsim_gb300::Simulator;
using Clock = std::chrono::steady_clock;

namespace {

struct Request {
    int64_t id;
    int phantom;
    std::vector<float> origins, dirs, lats, ts;
    int num_lines;
    float line_length;
    int decimation;
    Clock::time_point submitted;
    // result
    bool done = false;
    int status = BCSIM_OK;
    std::string error;
    std::vector<float2> iq;
    int64_t nd = 0;
    double latency_ms = 0.0;
    int64_t projections = 0;
};

struct Slot {
    std::unique_ptr<Simulator> sim;
    bool busy = false;
    size_t bytes = 0;
    float2* host = nullptr;         // pinned staging for the result
    size_t host_bytes = 0;
    cudaEvent_t done = nullptr;
    std::shared_ptr<Request> req;
};

struct Phantom {
    std::unique_ptr<Simulator> base;   // resident copy of the configuration
    std::vector<std::unique_ptr<Slot>> slots;
};

}  // namespace

struct bcsim_server {
    int device = 0;
    int64_t budget = 0;
    int max_slots = 4;
    std::atomic<int64_t> in_use{0};
    // phantoms: fixed capacity so that the worker can read entries while
    // add_phantom appends (entries never move)
    static constexpr int kMaxPhantoms = 256;
    std::unique_ptr<Phantom> phantoms[kMaxPhantoms];
    std::atomic<int> num_phantoms{0};
    std::mutex mu;
    std::condition_variable cv;        // wakes the worker (new request, stop)
    std::condition_variable done_cv;   // wakes waiters (a request finished)
    std::deque<std::shared_ptr<Request>> pending;
    std::map<int64_t, std::shared_ptr<Request>> requests;
    int64_t next_id = 1;
    int64_t completed = 0, failed = 0, projections = 0;
    std::vector<double> latencies;
    bool stop = false;
    std::thread worker;
    std::string last_error;

    void run();
    bool dispatch(const std::shared_ptr<Request>& r);
    void poll();
};

bool bcsim_server::dispatch(const std::shared_ptr<Request>& r) {
    Phantom& ph = *phantoms[r->phantom];
    Slot* slot = nullptr;
    for (auto& s : ph.slots)
        if (!s->busy) { slot = s.get(); break; }
    const int64_t ns = ph.base->samples_for(r->line_length);
    if (!slot) {
        const size_t need = ph.base->footprint_bytes(r->num_lines, ns);
        if ((int)ph.slots.size() >= max_slots || (!ph.slots.empty() && in_use + (int64_t)need > budget)) return false;
        auto s = std::make_unique<Slot>();
        s->sim = std::make_unique<Simulator>();
        s->sim->clone_from(*ph.base);
        s->bytes = need;
        in_use += (int64_t)need;
        if (cudaEventCreateWithFlags(&s->done, cudaEventDisableTiming) != cudaSuccess)
            throw SimError(BCSIM_E_CUDA, "cudaEventCreate failed");
        ph.slots.push_back(std::move(s));
        slot = ph.slots.back().get();
    }
    slot->busy = true;
    slot->req = r;
    try {
        Simulator& sim = *slot->sim;
        sim.set_parameter("radial_decimation", std::to_string(r->decimation));
        sim.set_scan_sequence(r->origins.data(), r->dirs.data(), r->lats.data(), r->ts.data(), r->num_lines,
                              r->line_length);
        sim.prepare();
        const size_t bytes = (size_t)sim.num_lines() * sim.num_out_samples() * sizeof(float2);
        if (bytes > slot->host_bytes) {
            if (slot->host) cudaFreeHost(slot->host);
            slot->host = nullptr;
            if (cudaMallocHost(&slot->host, bytes) != cudaSuccess) throw SimError(BCSIM_E_MEMORY, "pinned host allocation failed");
            slot->host_bytes = bytes;
        }
        cudaStream_t st = sim.stream();
        sim.enqueue(st, sim.internal_output(), false);
        if (cudaMemcpyAsync(slot->host, sim.internal_output(), bytes, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaEventRecord(slot->done, st) != cudaSuccess)
            throw SimError(BCSIM_E_CUDA, "enqueue failed");
        r->nd = sim.num_out_samples();
        r->projections = sim.total_num_scatterers() * (int64_t)r->num_lines;
    } catch (const std::exception& e) {
        std::lock_guard<std::mutex> lock(mu);
        r->done = true;
        r->status = dynamic_cast<const SimError*>(&e) ? static_cast<const SimError&>(e).code : BCSIM_E_INTERNAL;
        r->error = e.what();
        failed++;
        slot->busy = false;
        slot->req.reset();
        done_cv.notify_all();
    }
    return true;
}

void bcsim_server::poll() {
    const int np = num_phantoms.load();
    for (int pi = 0; pi < np; pi++) {
        for (auto& s : phantoms[pi]->slots) {
            if (!s->busy || !s->req) continue;
            const cudaError_t q = cudaEventQuery(s->done);
            if (q == cudaErrorNotReady) continue;
            std::shared_ptr<Request> r = s->req;
            const size_t n = (size_t)r->num_lines * r->nd;
            std::vector<float2> iq(s->host, s->host + n);
            std::lock_guard<std::mutex> lock(mu);
            if (q == cudaSuccess) {
                r->iq.swap(iq);
                r->latency_ms = std::chrono::duration<double, std::milli>(Clock::now() - r->submitted).count();
                latencies.push_back(r->latency_ms);
                completed++;
                projections += r->projections;
            } else {
                r->status = BCSIM_E_CUDA;
                r->error = cudaGetErrorString(q);
                failed++;
            }
            r->done = true;
            s->busy = false;
            s->req.reset();
            done_cv.notify_all();
        }
    }
}

void bcsim_server::run() {
    cudaSetDevice(device);
    for (;;) {
        std::vector<std::shared_ptr<Request>> todo;
        bool any_busy = false;
        {
            std::unique_lock<std::mutex> lock(mu);
            const int np = num_phantoms.load();
            for (int pi = 0; pi < np; pi++)
                for (auto& s : phantoms[pi]->slots) any_busy = any_busy || s->busy;
            if (!any_busy && pending.empty() && !stop) cv.wait(lock, [&] { return stop || !pending.empty(); });
            if (stop && pending.empty() && !any_busy) return;
            todo.assign(pending.begin(), pending.end());
        }
        // admit in arrival order; a request whose phantom has no free slot waits
        std::vector<int64_t> admitted;
        for (auto& r : todo) {
            bool ok = false;
            try {
                ok = dispatch(r);
            } catch (const std::exception& e) {
                std::lock_guard<std::mutex> lock(mu);
                r->done = true;
                r->status = BCSIM_E_INTERNAL;
                r->error = e.what();
                failed++;
                ok = true;
                done_cv.notify_all();
            }
            if (ok) admitted.push_back(r->id);
        }
        if (!admitted.empty()) {
            std::lock_guard<std::mutex> lock(mu);
            pending.erase(std::remove_if(pending.begin(), pending.end(),
                                         [&](const std::shared_ptr<Request>& r) {
                                             return std::find(admitted.begin(), admitted.end(), r->id) != admitted.end();
                                         }),
                          pending.end());
        }
        poll();
        if (admitted.empty()) std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
}

namespace {
template <typename F>
int guarded(bcsim_server* s, F&& f) {
    if (!s) return BCSIM_E_INVALID;
    try {
        f();
        return BCSIM_OK;
    } catch (const SimError& e) {
        std::lock_guard<std::mutex> lock(s->mu);
        s->last_error = e.what();
        return e.code;
    } catch (const std::exception& e) {
        std::lock_guard<std::mutex> lock(s->mu);
        s->last_error = e.what();
        return BCSIM_E_INTERNAL;
    }
}
}  // namespace

extern "C" {

int bcsim_server_create(int64_t hbm_budget_bytes, int max_slots_per_phantom, bcsim_server** out) {
    if (!out || hbm_budget_bytes <= 0 || max_slots_per_phantom <= 0) return BCSIM_E_INVALID;
    auto* s = new bcsim_server();
    s->budget = hbm_budget_bytes;
    s->max_slots = max_slots_per_phantom;
    if (cudaGetDevice(&s->device) != cudaSuccess) {
        delete s;
        return BCSIM_E_CUDA;
    }
    s->worker = std::thread([s] { s->run(); });
    *out = s;
    return BCSIM_OK;
}

int bcsim_server_destroy(bcsim_server* s) {
    if (!s) return BCSIM_OK;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        s->stop = true;
    }
    s->cv.notify_all();
    if (s->worker.joinable()) s->worker.join();
    for (int pi = 0; pi < s->num_phantoms.load(); pi++)
        for (auto& sl : s->phantoms[pi]->slots) {
            if (sl->host) cudaFreeHost(sl->host);
            if (sl->done) cudaEventDestroy(sl->done);
        }
    delete s;
    return BCSIM_OK;
}

const char* bcsim_server_last_error(const bcsim_server* s) { return s ? s->last_error.c_str() : "null server"; }

int bcsim_server_add_phantom(bcsim_server* s, bcsim_handle* configured, int* phantom_id) {
    return guarded(s, [&] {
        if (!configured || !phantom_id) throw SimError(BCSIM_E_INVALID, "null argument");
        auto ph = std::make_unique<Phantom>();
        ph->base = std::make_unique<Simulator>();
        ph->base->clone_from(bcsim_gb300::simulator_of(configured));
        std::lock_guard<std::mutex> lock(s->mu);
        const int id = s->num_phantoms.load();
        if (id >= bcsim_server::kMaxPhantoms) throw SimError(BCSIM_E_CAPACITY, "too many phantoms (256)");
        s->phantoms[id] = std::move(ph);
        s->num_phantoms.store(id + 1);
        *phantom_id = id;
    });
}

int bcsim_server_submit(bcsim_server* s, int phantom_id, const float* origins, const float* directions,
                        const float* lateral_dirs, const float* timestamps, int num_lines, float line_length,
                        int decimation, int64_t* request_id) {
    return guarded(s, [&] {
        if (num_lines <= 0 || !origins || !directions || !lateral_dirs || !timestamps || decimation <= 0)
            throw SimError(BCSIM_E_INVALID, "invalid request");
        auto r = std::make_shared<Request>();
        r->phantom = phantom_id;
        r->origins.assign(origins, origins + 3 * num_lines);
        r->dirs.assign(directions, directions + 3 * num_lines);
        r->lats.assign(lateral_dirs, lateral_dirs + 3 * num_lines);
        r->ts.assign(timestamps, timestamps + num_lines);
        r->num_lines = num_lines;
        r->line_length = line_length;
        r->decimation = decimation;
        {
            std::lock_guard<std::mutex> lock(s->mu);
            if (phantom_id < 0 || phantom_id >= s->num_phantoms.load()) throw SimError(BCSIM_E_INVALID, "unknown phantom");
            r->id = s->next_id++;
            r->submitted = Clock::now();
            s->requests[r->id] = r;
            s->pending.push_back(r);
            if (request_id) *request_id = r->id;
        }
        s->cv.notify_all();
    });
}

int bcsim_server_wait(bcsim_server* s, int64_t request_id, float* out, int64_t cap_complex, int64_t* num_lines,
                      int64_t* num_samples, double* latency_ms, int timeout_ms) {
    if (!s) return BCSIM_E_INVALID;
    std::shared_ptr<Request> r;
    {
        std::unique_lock<std::mutex> lock(s->mu);
        auto it = s->requests.find(request_id);
        if (it == s->requests.end()) {
            s->last_error = "unknown request";
            return BCSIM_E_INVALID;
        }
        r = it->second;
        const bool ok = s->done_cv.wait_for(lock, std::chrono::milliseconds(timeout_ms < 0 ? 1 << 30 : timeout_ms),
                                            [&] { return r->done; });
        if (!ok) return BCSIM_E_PENDING;
        s->requests.erase(request_id);
        if (r->status != BCSIM_OK) {
            s->last_error = r->error;
            return r->status;
        }
    }
    if (num_lines) *num_lines = r->num_lines;
    if (num_samples) *num_samples = r->nd;
    if (latency_ms) *latency_ms = r->latency_ms;
    const int64_t n = (int64_t)r->num_lines * r->nd;
    if (out) {
        if (cap_complex < n) return BCSIM_E_CAPACITY;
        std::memcpy(out, r->iq.data(), (size_t)n * sizeof(float2));
    }
    return BCSIM_OK;
}

int bcsim_server_stats(bcsim_server* s, int64_t* completed, int64_t* failed, double* p50_ms, double* p99_ms,
                       int64_t* projections, int64_t* hbm_in_use, int64_t* queue_depth) {
    if (!s) return BCSIM_E_INVALID;
    std::lock_guard<std::mutex> lock(s->mu);
    std::vector<double> l = s->latencies;
    std::sort(l.begin(), l.end());
    auto pct = [&](double q) { return l.empty() ? 0.0 : l[std::min(l.size() - 1, (size_t)(q * (l.size() - 1) + 0.5))]; };
    if (completed) *completed = s->completed;
    if (failed) *failed = s->failed;
    if (p50_ms) *p50_ms = pct(0.50);
    if (p99_ms) *p99_ms = pct(0.99);
    if (projections) *projections = s->projections;
    if (hbm_in_use) *hbm_in_use = s->in_use;
    if (queue_depth) *queue_depth = (int64_t)s->pending.size();
    return BCSIM_OK;
}

}  // extern "C"
