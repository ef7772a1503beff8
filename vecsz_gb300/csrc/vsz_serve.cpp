// Request server: continuous admission of compress / decompress requests under a device-memory
// budget, with their work overlapping on the device.
//
// Requests queue in arrival order.  A dispatcher thread admits the request at the head of the
// queue as soon as a stream slot is free and the request's workspace and output fit in the
// budget; its work (vsz_compress or vsz_decompress) is enqueued on the slot's stream, followed by
// an async copy of the result record to pinned memory and an event.  A completer thread polls the
// events of the running requests (spinning only while some request runs) and completes each as
// soon as its event has passed -- sooner than a stream host function, whose dispatch took tens
// of microseconds.
// Workspaces and outputs are carved from one pre-allocated device arena by a host-side first-fit
// allocator, so admission never calls cudaMalloc.  A completed request frees its workspace at
// once and keeps its output (compress: shrunk to the archive's real size) until released.
#include <chrono>
#include <algorithm>
#include <condition_variable>
#include <cstdint>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "vsz_types.h"

namespace {

double now_s() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

// First-fit allocator over [0, size): offsets only, 256-byte granules.
class Arena {
public:
    explicit Arena(size_t size) { free_[0] = size; }
    static size_t round(size_t n) { return (n + 255) & ~(size_t)255; }
    bool alloc(size_t n, size_t* off) {
        n = round(n);
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= n) {
                *off = it->first;
                size_t rest = it->second - n, at = it->first + n;
                free_.erase(it);
                if (rest) free_[at] = rest;
                used_ += n;
                return true;
            }
        }
        return false;
    }
    void release(size_t off, size_t n) {
        n = round(n);
        if (!n) return;
        used_ -= n;
        auto it = free_.emplace(off, n).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }
    size_t used() const { return used_; }

private:
    std::map<size_t, size_t> free_;
    size_t used_ = 0;
};

struct Job {
    uint64_t ticket = 0;
    vsz_request req{};
    size_t ws_bytes = 0, out_bytes = 0;  // requested
    size_t ws_off = 0, out_off = 0;
    int slot = -1;
    int state = 0;  // 0 queued, 1 running, 2 done
    int status = VSZ_OK;
    double t_submit = 0, t_start = 0, t_done = 0;
    uint64_t result[8] = {};
    size_t out_keep = 0;  // output bytes kept after completion
};

struct Slot {
    cudaStream_t stream = nullptr;
    uint64_t* h_result = nullptr;  // pinned: 8 u64 result record + 1 status word
    cudaEvent_t done   = nullptr;  // recorded after the job's work and its result copy
    Job* job           = nullptr;  // the job whose event the completer waits for
    int busy = 0;
};

}  // namespace

struct vsz_server {
    int device = 0;
    uint8_t* base = nullptr;
    size_t budget = 0;
    Arena* arena = nullptr;
    std::vector<Slot> slots;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<Job*> queue;
    std::unordered_map<uint64_t, Job*> jobs;
    uint64_t next_ticket = 1;
    bool stop = false;
    bool stop_completer = false;
    std::condition_variable cv_run;  // a job was launched (or the completer is to stop)
    std::thread dispatcher, completer;
    uint64_t n_done = 0, bytes_in_done = 0;
};

namespace {

size_t request_bytes(const vsz_request& r) {
    if (r.kind == VSZ_REQ_COMPRESS) {
        size_t n = 1;
        for (int i = 0; i < r.ndim; i++) n *= r.dims[i];
        return 4 * n;
    }
    return 4 * r.desc.dims[0] * r.desc.dims[1] * r.desc.dims[2];
}

// Completes a job whose slot event has passed (lock held).  stream_failed: the event reported an
// error, so the result copy may not have run.
void complete_job(vsz_server* s, Job* j, bool stream_failed) {
    Slot& sl = s->slots[(size_t)j->slot];
    j->t_done = now_s();
    if (stream_failed) {
        j->status   = VSZ_ERR_CUDA;
        j->out_keep = 0;
    } else if (j->req.kind == VSZ_REQ_COMPRESS) {
        memcpy(j->result, sl.h_result, sizeof(j->result));
        j->status   = (int)j->result[5];
        j->out_keep = j->status == VSZ_OK ? (size_t)(j->result[0] + j->result[1]) : 0;
    } else {
        j->status   = (int)(int32_t)sl.h_result[8];
        j->out_keep = j->status == VSZ_OK ? j->out_bytes : 0;
    }
    // the workspace goes back at once; a compress output keeps its real size only
    s->arena->release(j->ws_off, j->ws_bytes);
    const size_t keep = Arena::round(j->out_keep);
    if (Arena::round(j->out_bytes) > keep) s->arena->release(j->out_off + keep, Arena::round(j->out_bytes) - keep);
    j->out_bytes = keep;
    j->state     = 2;
    sl.busy      = 0;
    s->n_done++;
    if (j->status == VSZ_OK) s->bytes_in_done += request_bytes(j->req);
    s->cv.notify_all();
}

// The completer: polls the events of the launched jobs without the lock and completes the ones
// that have passed.  It sleeps while no job runs and exits once stopped with none left.
void complete_loop(vsz_server* s) {
    cudaSetDevice(s->device);
    std::vector<int> running, ready, failed;
    std::unique_lock<std::mutex> lk(s->mu);
    for (;;) {
        auto any_running = [&] {
            for (auto& sl : s->slots)
                if (sl.job) return true;
            return false;
        };
        s->cv_run.wait(lk, [&] { return s->stop_completer || any_running(); });
        if (!any_running()) break;  // stopped, nothing left
        running.clear();
        for (size_t i = 0; i < s->slots.size(); i++)
            if (s->slots[i].job) running.push_back((int)i);
        lk.unlock();
        ready.clear();
        failed.clear();
        for (int i : running) {
            const cudaError_t e = cudaEventQuery(s->slots[(size_t)i].done);  // the handle never changes
            if (e == cudaSuccess) ready.push_back(i);
            else if (e != cudaErrorNotReady) failed.push_back(i);
        }
        if (ready.empty() && failed.empty()) std::this_thread::yield();
        lk.lock();
        // only this thread clears a slot's job, and the dispatcher sets one only on a free slot
        for (int i : ready) {
            Job* j = s->slots[(size_t)i].job;
            s->slots[(size_t)i].job = nullptr;
            complete_job(s, j, false);
        }
        for (int i : failed) {
            Job* j = s->slots[(size_t)i].job;
            s->slots[(size_t)i].job = nullptr;
            cudaGetLastError();
            complete_job(s, j, true);
        }
    }
}

// Enqueue one admitted job on its slot's stream (dispatcher thread, lock not held).
int launch_job(vsz_server* s, Job* j) {
    Slot& sl        = s->slots[(size_t)j->slot];
    uint8_t* ws     = s->base + j->ws_off;
    uint8_t* out    = s->base + j->out_off;
    uint64_t* d_rec = reinterpret_cast<uint64_t*>(ws);  // first 256 bytes of the workspace: result record
    int rc;
    if (j->req.kind == VSZ_REQ_COMPRESS) {
        rc = vsz_compress(&j->req.params, j->req.ndim, j->req.dims, static_cast<const float*>(j->req.d_in), ws + 256,
                          j->ws_bytes - 256, out, j->out_bytes, d_rec, sl.stream);
        if (rc == VSZ_OK && cudaMemcpyAsync(sl.h_result, d_rec, 64, cudaMemcpyDeviceToHost, sl.stream) != cudaSuccess)
            rc = VSZ_ERR_CUDA;
    } else {
        int* d_status = reinterpret_cast<int*>(ws);
        rc = vsz_decompress(&j->req.desc, &j->req.opts, static_cast<const uint8_t*>(j->req.d_in), ws + 256,
                            j->ws_bytes - 256, reinterpret_cast<float*>(out), d_status, sl.stream);
        if (rc == VSZ_OK && cudaMemcpyAsync(sl.h_result + 8, d_status, 4, cudaMemcpyDeviceToHost, sl.stream) != cudaSuccess)
            rc = VSZ_ERR_CUDA;
    }
    if (rc != VSZ_OK) return rc;
    return cudaEventRecord(sl.done, sl.stream) == cudaSuccess ? VSZ_OK : VSZ_ERR_CUDA;
}

void dispatch_loop(vsz_server* s) {
    cudaSetDevice(s->device);
    std::unique_lock<std::mutex> lk(s->mu);
    while (true) {
        s->cv.wait(lk, [&] {
            if (s->stop) return true;
            if (s->queue.empty()) return false;
            for (auto& sl : s->slots)
                if (!sl.busy) return true;
            return false;
        });
        if (s->stop) break;
        Job* j = s->queue.front();
        int slot = -1;
        for (size_t i = 0; i < s->slots.size(); i++)
            if (!s->slots[i].busy) {
                slot = (int)i;
                break;
            }
        size_t wo = 0, oo = 0;
        if (!s->arena->alloc(j->ws_bytes, &wo)) {
            s->cv.wait(lk);  // memory frees up when a running request completes
            continue;
        }
        if (!s->arena->alloc(j->out_bytes, &oo)) {
            s->arena->release(wo, j->ws_bytes);
            s->cv.wait(lk);
            continue;
        }
        s->queue.pop_front();
        j->ws_off  = wo;
        j->out_off = oo;
        j->slot    = slot;
        j->state   = 1;
        j->t_start = now_s();
        s->slots[(size_t)slot].busy = 1;
        lk.unlock();
        int rc = launch_job(s, j);
        // A failed launch may have queued some of its kernels and copies before the step that
        // failed: let them finish before the job's arena memory goes to the next request.
        if (rc != VSZ_OK) cudaStreamSynchronize(s->slots[(size_t)slot].stream);
        lk.lock();
        if (rc == VSZ_OK) {  // the completer takes it from here
            s->slots[(size_t)slot].job = j;
            s->cv_run.notify_one();
        } else {  // no event was recorded: complete it here
            s->arena->release(j->ws_off, j->ws_bytes);
            s->arena->release(j->out_off, j->out_bytes);
            j->out_bytes = 0;
            j->status    = rc;
            j->state     = 2;
            j->t_done    = now_s();
            s->slots[(size_t)slot].busy = 0;
            s->cv.notify_all();
        }
    }
}

}  // namespace

extern "C" {

vsz_status vsz_server_create(size_t budget_bytes, int nslots, vsz_server** out) {
    if (!out || budget_bytes < (1u << 20) || nslots < 1 || nslots > 64) return VSZ_ERR_INVALID;
    *out = nullptr;
    vsz_server* s = new vsz_server();
    cudaGetDevice(&s->device);
    if (cudaMalloc(reinterpret_cast<void**>(&s->base), budget_bytes) != cudaSuccess) {
        delete s;
        return VSZ_ERR_NOMEM;
    }
    s->budget = budget_bytes;
    s->arena  = new Arena(budget_bytes);
    s->slots.resize((size_t)nslots);
    for (auto& sl : s->slots) {
        if (cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaHostAlloc(reinterpret_cast<void**>(&sl.h_result), 128, cudaHostAllocDefault) != cudaSuccess ||
            cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming) != cudaSuccess) {
            vsz_server_destroy(s);
            return VSZ_ERR_CUDA;
        }
    }
    s->dispatcher = std::thread(dispatch_loop, s);
    s->completer  = std::thread(complete_loop, s);
    *out          = s;
    return VSZ_OK;
}

vsz_status vsz_server_submit(vsz_server* s, const vsz_request* r, uint64_t* ticket) {
    if (!s || !r || !ticket || !r->d_in) return VSZ_ERR_INVALID;
    Job* j = new Job();
    j->req = *r;
    size_t ws = 0, out = 0;
    int rc;
    if (r->kind == VSZ_REQ_COMPRESS) {
        rc = vsz_compress_bounds(&r->params, r->ndim, r->dims, &ws, &out);
    } else if (r->kind == VSZ_REQ_DECOMPRESS) {
        rc  = vsz_decompress_bounds(&r->desc, &r->opts, &ws);
        out = 4 * (size_t)(r->desc.dims[0] * r->desc.dims[1] * r->desc.dims[2]);
    } else {
        rc = VSZ_ERR_INVALID;
    }
    if (rc != VSZ_OK) {
        delete j;
        return rc;
    }
    j->ws_bytes  = ws + 256;
    j->out_bytes = out;
    if (Arena::round(j->ws_bytes) + Arena::round(out) > s->budget) {
        delete j;
        return VSZ_ERR_CAPACITY;  // would never fit
    }
    std::lock_guard<std::mutex> g(s->mu);
    j->ticket   = s->next_ticket++;
    j->t_submit = now_s();
    s->jobs[j->ticket] = j;
    s->queue.push_back(j);
    *ticket = j->ticket;
    s->cv.notify_all();
    return VSZ_OK;
}

vsz_status vsz_server_wait(vsz_server* s, uint64_t ticket, double timeout_s, vsz_completion* c) {
    if (!s || !c) return VSZ_ERR_INVALID;
    std::unique_lock<std::mutex> lk(s->mu);
    if (s->jobs.find(ticket) == s->jobs.end()) return VSZ_ERR_INVALID;
    // The job is looked up again on every wake-up: another thread may release the ticket while
    // this one waits, and then the job no longer exists.
    Job* j = nullptr;
    const auto until = std::chrono::steady_clock::now() + std::chrono::duration<double>(timeout_s);
    const bool woke  = s->cv.wait_until(lk, until, [&] {
        auto it = s->jobs.find(ticket);
        j       = it == s->jobs.end() ? nullptr : it->second;
        return !j || j->state == 2;
    });
    if (!woke) return VSZ_ERR_TIMEOUT;
    if (!j) return VSZ_ERR_INVALID;  // released by another thread meanwhile
    c->status    = j->status;
    c->d_out     = j->out_bytes ? s->base + j->out_off : nullptr;
    c->out_bytes = j->out_keep;
    c->t_submit  = j->t_submit;
    c->t_start   = j->t_start;
    c->t_done    = j->t_done;
    memcpy(c->result, j->result, sizeof(c->result));
    return VSZ_OK;
}

vsz_status vsz_server_release(vsz_server* s, uint64_t ticket) {
    if (!s) return VSZ_ERR_INVALID;
    std::lock_guard<std::mutex> g(s->mu);
    auto it = s->jobs.find(ticket);
    if (it == s->jobs.end() || it->second->state != 2) return VSZ_ERR_INVALID;
    Job* j = it->second;
    s->arena->release(j->out_off, j->out_bytes);
    s->jobs.erase(it);
    delete j;
    s->cv.notify_all();
    return VSZ_OK;
}

vsz_status vsz_server_cancel(vsz_server* s, uint64_t ticket) {
    if (!s) return VSZ_ERR_INVALID;
    std::lock_guard<std::mutex> g(s->mu);
    auto it = s->jobs.find(ticket);
    if (it == s->jobs.end()) return VSZ_ERR_INVALID;
    Job* j = it->second;
    if (j->state != 0) return VSZ_ERR_UNSUPPORTED;  // admitted: its work is on the device
    auto q = std::find(s->queue.begin(), s->queue.end(), j);
    if (q != s->queue.end()) s->queue.erase(q);
    j->status    = VSZ_ERR_CANCELLED;
    j->out_bytes = 0;  // nothing was allocated for it
    j->out_keep  = 0;
    j->state     = 2;
    j->t_start = j->t_done = now_s();
    s->cv.notify_all();
    return VSZ_OK;
}

vsz_status vsz_server_stats(vsz_server* s, uint64_t* done, uint64_t* bytes_in_done, size_t* bytes_in_use,
                            int* queued) {
    if (!s) return VSZ_ERR_INVALID;
    std::lock_guard<std::mutex> g(s->mu);
    if (done) *done = s->n_done;
    if (bytes_in_done) *bytes_in_done = s->bytes_in_done;
    if (bytes_in_use) *bytes_in_use = s->arena->used();
    if (queued) *queued = (int)s->queue.size();
    return VSZ_OK;
}

void vsz_server_destroy(vsz_server* s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> g(s->mu);
        s->stop = true;
        s->cv.notify_all();
    }
    if (s->dispatcher.joinable()) s->dispatcher.join();
    for (auto& sl : s->slots)
        if (sl.stream) cudaStreamSynchronize(sl.stream);
    {  // every launched job's event has passed: the completer completes them and exits
        std::lock_guard<std::mutex> g(s->mu);
        s->stop_completer = true;
        s->cv_run.notify_all();
    }
    if (s->completer.joinable()) s->completer.join();
    for (auto& sl : s->slots) {
        if (sl.stream) cudaStreamDestroy(sl.stream);
        if (sl.done) cudaEventDestroy(sl.done);
        if (sl.h_result) cudaFreeHost(sl.h_result);
    }
    for (auto& kv : s->jobs) delete kv.second;
    if (s->base) cudaFree(s->base);
    delete s->arena;
    delete s;
}

}  // extern "C"
