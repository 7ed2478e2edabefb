// server.cpp -- continuous-batching request server.
//
// Phantoms (configured simulators: scatterers, beam, excitation, parameters)
// stay resident on the device.  A request asks for some scan lines of one
// phantom (origins, directions, timestamps, line length, decimation).  One worker
// thread admits queued requests in arrival order as soon as a simulator slot of
// their phantom is free and the device memory the request needs is available --
// creating slots while the budget allows -- prepares them on the host and
// enqueues their device work on the slot's own stream, so requests that arrive
// while others are on the GPU overlap with them.
//
// Admission by device memory: a request needs its slot's footprint for its
// lines (bins, records, output); the growth beyond what the slot already holds
// must fit in the memory available now -- the driver's free memory plus what
// the device's stream-ordered pool holds reserved but unused (slots grow from
// that pool) -- less a reserve.  A request that does not fit waits while others
// are in flight (their completion can free slots for reuse); one that cannot
// fit even with nothing in flight, or that exceeds the whole budget, fails with
// BCSIM_E_MEMORY and the stream goes on.
// The same thread polls completion events, hands each result (the pinned buffer
// the device copied it to) to its request and records the submit-to-result
// latency; the waiter copies it out.  Device buffers grow in stream order and
// pinned buffers are recycled, so the steady state allocates nothing.  A
// request's result depends only on its phantom and its own lines, never on what
// else is in flight.
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
    // result: the pinned staging buffer the device copied it to, handed over
    // by the slot (returned to the server's free list by the waiter)
    bool done = false;
    int status = BCSIM_OK;
    std::string error;
    float2* iq = nullptr;
    size_t iq_bytes = 0;
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
    int* flag = nullptr;            // pinned copy of the slot's device error flag, read with the result
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
    std::atomic<int> max_in_flight{3};
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
    std::vector<std::pair<float2*, size_t>> free_pinned;   // result buffers returned by waiters
    bool stop = false;
    std::thread worker;
    std::string last_error;
    // host-side fault injection for tests (bcsim_server_debug_inject)
    std::atomic<int> inject_wait_flag{0};     // raise the next admitted request's wait flag
    std::atomic<int> inject_throw{0};         // make the next dispatch throw inside the worker
    std::atomic<int64_t> free_cap{-1};        // cap on the available device memory admission sees
    static constexpr size_t kReserve = (size_t)256 << 20;   // kept free for the driver and the pool's slack

    void run();
    bool dispatch(const std::shared_ptr<Request>& r);
    void poll();
    int busy_slots();
    size_t available_memory();
    void fail_request(const std::shared_ptr<Request>& r, int code, const std::string& msg);
};

namespace {
// A slot: a simulator holding a copy of the phantom, its result staging and its
// completion event.
std::unique_ptr<Slot> make_slot(Simulator& base, size_t bytes) {
    auto s = std::make_unique<Slot>();
    s->sim = std::make_unique<Simulator>();
    s->sim->clone_from(base);
    s->bytes = bytes;
    if (cudaEventCreateWithFlags(&s->done, cudaEventDisableTiming) != cudaSuccess)
        throw SimError(BCSIM_E_CUDA, "cudaEventCreate failed");
    const size_t pinned = (size_t)8 << 20;
    if (cudaMallocHost(&s->host, pinned) != cudaSuccess) throw SimError(BCSIM_E_MEMORY, "pinned host allocation failed");
    s->host_bytes = pinned;
    if (cudaMallocHost(&s->flag, sizeof(int)) != cudaSuccess) throw SimError(BCSIM_E_MEMORY, "pinned host allocation failed");
    *s->flag = 0;
    return s;
}
}  // namespace

// Device memory a request can still take: the driver's free memory plus the
// default pool's reserved-but-unused bytes (stream-ordered buffers are carved
// from that pool, which keeps freed memory for reuse), less a reserve.
size_t bcsim_server::available_memory() {
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
        cudaGetLastError();
        free_b = 0;
    }
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
        uint64_t reserved = 0, used = 0;
        if (cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &reserved) == cudaSuccess &&
            cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &used) == cudaSuccess && reserved > used)
            free_b += (size_t)(reserved - used);
    }
    free_b = free_b > kReserve ? free_b - kReserve : 0;
    const int64_t cap = free_cap.load();
    if (cap >= 0 && (size_t)cap < free_b) free_b = (size_t)cap;
    return free_b;
}

void bcsim_server::fail_request(const std::shared_ptr<Request>& r, int code, const std::string& msg) {
    std::lock_guard<std::mutex> lock(mu);
    r->done = true;
    r->status = code;
    r->error = msg;
    failed++;
    done_cv.notify_all();
}

int bcsim_server::busy_slots() {
    int n = 0;
    const int np = num_phantoms.load();
    for (int pi = 0; pi < np; pi++)
        for (auto& s : phantoms[pi]->slots) n += s->busy ? 1 : 0;
    return n;
}

bool bcsim_server::dispatch(const std::shared_ptr<Request>& r) {
    Phantom& ph = *phantoms[r->phantom];
    Slot* slot = nullptr;
    for (auto& s : ph.slots)
        if (!s->busy) { slot = s.get(); break; }
    const int64_t ns = ph.base->samples_for(r->line_length);
    const size_t need = ph.base->footprint_bytes(r->num_lines, ns);
    if (need > (size_t)budget) {
        fail_request(r, BCSIM_E_MEMORY, "request needs " + std::to_string(need) + " bytes of device memory, above the "
                                        "server's budget of " + std::to_string(budget));
        return true;
    }
    // device memory this admission takes: a new slot's footprint, or the growth
    // of a free slot's buffers
    const size_t grow = slot ? (need > slot->bytes ? need - slot->bytes : 0) : need;
    if (!slot && ((int)ph.slots.size() >= max_slots || (!ph.slots.empty() && in_use + (int64_t)need > budget)))
        return false;   // wait for a slot of this phantom
    if (grow > 0) {
        const size_t avail = available_memory();
        if (grow > avail) {
            if (busy_slots() > 0) return false;   // completions may free slots to reuse
            fail_request(r, BCSIM_E_MEMORY, "request needs " + std::to_string(grow) + " more bytes of device memory; " +
                                            std::to_string(avail) + " available");
            return true;
        }
    }
    if (!slot) {
        ph.slots.push_back(make_slot(*ph.base, need));
        in_use += (int64_t)need;
        slot = ph.slots.back().get();
    } else if (need > slot->bytes) {
        in_use += (int64_t)(need - slot->bytes);
        slot->bytes = need;
    }
    slot->busy = true;
    slot->req = r;
    try {
        if (inject_throw.exchange(0)) throw std::runtime_error("injected worker failure");
        Simulator& sim = *slot->sim;
        sim.set_parameter("radial_decimation", std::to_string(r->decimation));
        sim.set_scan_sequence(r->origins.data(), r->dirs.data(), r->lats.data(), r->ts.data(), r->num_lines,
                              r->line_length);
        sim.prepare();
        const size_t bytes = (size_t)sim.num_lines() * sim.num_out_samples() * sizeof(float2);
        if (bytes > slot->host_bytes) {
            // pinned staging grows rarely (at least 8 MiB, then doubling): freeing
            // pinned memory can wait for the device
            const size_t grow_h = std::max({bytes, slot->host_bytes * 2, (size_t)8 << 20});
            if (slot->host) cudaFreeHost(slot->host);
            slot->host = nullptr;
            slot->host_bytes = 0;
            if (cudaMallocHost(&slot->host, grow_h) != cudaSuccess) throw SimError(BCSIM_E_MEMORY, "pinned host allocation failed");
            slot->host_bytes = grow_h;
        }
        cudaStream_t st = sim.stream();
        sim.enqueue(st, sim.internal_output(), false);
        if (inject_wait_flag.exchange(0)) sim.raise_device_flag();   // as a bounded wait that gave up would
        if (cudaMemcpyAsync(slot->host, sim.internal_output(), bytes, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            sim.enqueue_flag_read(slot->flag, st) != cudaSuccess || cudaEventRecord(slot->done, st) != cudaSuccess)
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
            std::string flag_error;
            if (q == cudaSuccess && *s->flag) {
                // a bounded device wait of this request's kernels gave up: the
                // result is incomplete (the check clears the slot's flag)
                try {
                    s->sim->check_device_flag();
                } catch (const std::exception& e) {
                    flag_error = e.what();
                }
                *s->flag = 0;
                if (flag_error.empty()) flag_error = "a bounded device wait gave up; results are incomplete";
            }
            std::lock_guard<std::mutex> lock(mu);
            if (q == cudaSuccess && !flag_error.empty()) {
                r->status = BCSIM_E_INTERNAL;
                r->error = flag_error;
                failed++;
            } else if (q == cudaSuccess) {
                // hand the staging buffer to the request; the slot takes a
                // returned one (or allocates at its next dispatch)
                r->iq = s->host;
                r->iq_bytes = s->host_bytes;
                s->host = nullptr;
                s->host_bytes = 0;
                if (!free_pinned.empty()) {
                    s->host = free_pinned.back().first;
                    s->host_bytes = free_pinned.back().second;
                    free_pinned.pop_back();
                }
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
        // admit strictly in arrival order while fewer than max_in_flight
        // requests are on the GPU: the GPU works on the oldest requests (their
        // kernels overlap, and the host prepares the next request meanwhile)
        // instead of sharing itself among every queued one
        std::vector<int64_t> admitted;
        int in_flight = busy_slots();
        for (auto& r : todo) {
            if (in_flight >= max_in_flight.load()) break;
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
            if (!ok) break;   // its phantom has no free slot: later requests wait too
            admitted.push_back(r->id);
            in_flight++;
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
        if (admitted.empty()) std::this_thread::sleep_for(std::chrono::microseconds(20));
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
            if (sl->flag) cudaFreeHost(sl->flag);
            if (sl->done) cudaEventDestroy(sl->done);
        }
    for (auto& b : s->free_pinned) cudaFreeHost(b.first);
    for (auto& kv : s->requests)   // results never collected
        if (kv.second->iq) cudaFreeHost(kv.second->iq);
    delete s;
    return BCSIM_OK;
}

const char* bcsim_server_last_error(const bcsim_server* s) { return s ? s->last_error.c_str() : "null server"; }

int bcsim_server_set_max_in_flight(bcsim_server* s, int max_in_flight) {
    if (!s || max_in_flight <= 0) return BCSIM_E_INVALID;
    s->max_in_flight.store(max_in_flight);
    return BCSIM_OK;
}

int bcsim_server_add_phantom(bcsim_server* s, bcsim_handle* configured, int* phantom_id) {
    return guarded(s, [&] {
        if (!configured || !phantom_id) throw SimError(BCSIM_E_INVALID, "null argument");
        auto ph = std::make_unique<Phantom>();
        Simulator& src = bcsim_gb300::simulator_of(configured);
        ph->base = std::make_unique<Simulator>();
        ph->base->clone_from(src);
        // slots made now, and prepared once with the handle's scan (when it has
        // one): device buffers, tables and staging exist before the first request
        const int warm = std::min(s->max_slots, 3);
        for (int k = 0; k < warm; k++) {
            const size_t need = ph->base->footprint_bytes(1, 1);
            if (k > 0 && s->in_use + (int64_t)need > s->budget) break;
            ph->slots.push_back(make_slot(*ph->base, need));
            s->in_use += (int64_t)need;
            Simulator& sim = *ph->slots.back()->sim;
            sim.copy_scan_from(src);
            try {
                sim.prepare();
            } catch (const SimError&) {
                // a scan that does not suit (e.g. none): the first request prepares
            }
        }
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
    int rc = BCSIM_OK;
    if (out) {
        if (cap_complex < n) rc = BCSIM_E_CAPACITY;
        else std::memcpy(out, r->iq, (size_t)n * sizeof(float2));
    }
    if (r->iq) {
        std::lock_guard<std::mutex> lock(s->mu);
        s->free_pinned.emplace_back(r->iq, r->iq_bytes);
        r->iq = nullptr;
    }
    return rc;
}

int bcsim_server_debug_inject(bcsim_server* s, int what, int64_t value) {
    if (!s) return BCSIM_E_INVALID;
    switch (what) {
        case BCSIM_SERVER_INJECT_WAIT_FLAG: s->inject_wait_flag.store(1); return BCSIM_OK;
        case BCSIM_SERVER_INJECT_WORKER_THROW: s->inject_throw.store(1); return BCSIM_OK;
        case BCSIM_SERVER_INJECT_FREE_MEMORY_CAP: s->free_cap.store(value); return BCSIM_OK;
        default: return BCSIM_E_INVALID;
    }
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
