// Request loop on one GPU with continuous batching (declared in
// include/chaos_gb300.h, chaos_server_*).
//
// Threads: the caller submits; a scheduler thread admits requests into
// device-resident slots (descriptor table + output buffers, bounded by the
// HBM budget and maxActive) and launches iterations; a pool of completion
// workers (one copy stream each) copies finished requests back, runs the
// basins clustering when asked, frees their memory and records latency. A
// request's descriptor slot is released as soon as its device work is done;
// its memory counts against the budget until the worker frees it. An iteration is a list of block-sized
// chunks shared fairly among the resident requests up to a work budget, run
// by the grouped persistent kernels of batched mode; two
// iterations are in flight on two streams, so new requests enter the next
// iteration while the current one runs. All waits on the host are bounded.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <new>
#include <thread>
#include <unordered_map>
#include <vector>

#include "batch_util.h"
#include "dbscan.h"

using namespace chaos;
using Clock = std::chrono::steady_clock;

namespace {

struct Request {
    long long id = 0;
    chaos_job job{};
    std::vector<double> ic, ranges, values;
    std::vector<int> mut;
    JobDesc desc{};
    std::vector<HostOut> outs;  // device -> host copies (host-memory servers)
    std::vector<std::pair<void*, size_t>> want;  // requested device buffers: (host pointer, bytes)
    char* devBlock = nullptr;   // one device allocation for all outputs
    size_t bytes = 0;
    int* dLabels = nullptr;     // basins clustering output (device)
    long long nPoints = 0, next = 0, done = 0;
    int chunk = 0;
    int slot = -1;
    int state = CHAOS_REQ_PENDING;
    long long steps = 0;
    long long perPoint = 0;
    Clock::time_point tSubmit;
    double latency = -1;
};

struct Iteration {
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    Chunk* dChunks = nullptr;
    Chunk* hChunks = nullptr;  // pinned staging
    int* dCounters = nullptr;
    int capacity = 0;
    std::vector<cudaStream_t> aux;
    std::vector<cudaEvent_t> events;
    std::vector<std::pair<Request*, long long>> work;
    bool busy = false;
};

constexpr int kAuxPerIteration = 8;

double seconds(Clock::duration d) { return std::chrono::duration<double>(d).count(); }

}  // namespace

struct chaos_server {
    int device = 0;
    int memory = CHAOS_MEM_HOST;
    size_t budget = 0, used = 0, peakUsed = 0;
    int maxActive = 0;
    double iterationSteps = 0;
    cudaMemPool_t pool = nullptr;
    cudaStream_t setup = nullptr;
    std::vector<cudaStream_t> copy;  // one per completion worker
    cudaEvent_t setupDone = nullptr;
    JobDesc* dTable = nullptr;
    std::vector<int> freeSlots;
    Iteration it[2];

    std::mutex mu;
    std::condition_variable cvWork, cvDone, cvComplete;
    std::deque<Request*> pending;
    std::vector<Request*> active;  // admitted, in admission order
    std::deque<Request*> completed;  // waiting for the completion thread
    std::unordered_map<long long, std::unique_ptr<Request>> all;
    long long nextId = 1;
    bool stop = false, schedulerDone = false;
    int error = CHAOS_OK;
    std::vector<double> latencies;
    long long stepsDone = 0, iterations = 0, failed = 0;
    bool started = false;
    Clock::time_point tFirst;
    std::thread scheduler;
    std::vector<std::thread> completers;
    int completersRunning = 0;
};

constexpr int kCompleters = 4;

namespace {

// Admits pending requests while slots and budget allow (called with mu held).
// Allocations and descriptor uploads go to the setup stream; iterations wait
// for its event before they start.
bool admit_locked(chaos_server* S) {
    bool any = false;
    while (!S->pending.empty() && !S->freeSlots.empty()) {
        Request* r = S->pending.front();
        if (S->used + r->bytes > S->budget && S->used > 0) break;  // a request alone on the device may exceed it
        void* block = nullptr;
        if (r->bytes && cudaMallocFromPoolAsync(&block, r->bytes, S->pool, S->setup) != cudaSuccess) break;
        S->pending.pop_front();
        r->devBlock = (char*)block;
        size_t off = 0;
        std::vector<HostOut> outs;
        auto carve = [&](size_t b) -> void* {
            void* p = r->devBlock + off;
            off += (b + 255) & ~size_t(255);
            return p;
        };
        prepare_job(r->job, S->memory, r->desc, outs, carve);
        r->outs = outs;
        if (r->job.kind == CHAOS_JOB_BASINS && r->job.labels && r->job.eps > 0)
            r->dLabels = S->memory == CHAOS_MEM_DEVICE ? r->job.labels : (int*)carve(r->nPoints * sizeof(int));
        r->slot = S->freeSlots.back();
        S->freeSlots.pop_back();
        cudaMemcpyAsync(S->dTable + r->slot, &r->desc, sizeof(JobDesc), cudaMemcpyHostToDevice, S->setup);
        r->state = CHAOS_REQ_RUNNING;
        S->used += r->bytes;
        S->peakUsed = std::max(S->peakUsed, S->used);
        S->active.push_back(r);
        any = true;
    }
    if (any) {
        cudaEventRecord(S->setupDone, S->setup);
        cudaStreamSynchronize(S->setup);  // the descriptor copies read request-owned host memory
    }
    return any;
}

// Chunks of this iteration (called with mu held): first every resident
// request with points left gets an equal share of the work budget (at least
// one chunk), in admission order; what is left of the budget then goes to
// the oldest requests first. Small requests therefore finish within a few
// iterations even while large ones are resident (processor sharing).
void take_chunks_locked(chaos_server* S, Iteration& I, std::vector<Chunk>& chunks) {
    I.work.clear();
    int waiting = 0;
    for (Request* r : S->active)
        if (r->next < r->nPoints) ++waiting;
    if (!waiting) return;
    double budget = S->iterationSteps;
    const double share = budget / waiting;
    std::vector<long long> taken(S->active.size(), 0);
    auto take = [&](size_t idx, double limit) {
        Request* r = S->active[idx];
        double used = 0;
        while (r->next < r->nPoints && used < limit && budget > 0) {
            const int cnt = (int)std::min<long long>(r->chunk, r->nPoints - r->next);
            chunks.push_back(Chunk{r->slot, cnt, r->next});
            r->next += cnt;
            taken[idx] += cnt;
            const double w = (double)cnt * (double)r->perPoint;
            used += w;
            budget -= w;
        }
    };
    for (size_t i = 0; i < S->active.size() && budget > 0; ++i) take(i, share);
    for (size_t i = 0; i < S->active.size() && budget > 0; ++i) take(i, budget);
    for (size_t i = 0; i < S->active.size(); ++i)
        if (taken[i]) I.work.push_back({S->active[i], taken[i]});
}

// Marks an iteration's work finished; hands completed requests over.
void finalize(chaos_server* S, Iteration& I) {
    std::lock_guard<std::mutex> lk(S->mu);
    for (auto& w : I.work) {
        w.first->done += w.second;
        if (w.first->done == w.first->nPoints) {
            S->active.erase(std::find(S->active.begin(), S->active.end(), w.first));
            S->freeSlots.push_back(w.first->slot);  // its descriptor is no longer read
            S->completed.push_back(w.first);
        }
    }
    I.work.clear();
    I.busy = false;
    S->cvComplete.notify_all();
}

int launch_iteration(chaos_server* S, Iteration& I, std::vector<Chunk>& chunks,
                     const std::vector<Request*>& slotOwner) {
    // group by (kind, system) of the owning requests, keeping FIFO order inside a group
    std::stable_sort(chunks.begin(), chunks.end(), [&](const Chunk& a, const Chunk& b) {
        const JobDesc& A = slotOwner[a.job]->desc;
        const JobDesc& B = slotOwner[b.job]->desc;
        if (A.kind != B.kind) return A.kind < B.kind;
        return A.system < B.system;
    });
    std::vector<Group> groups;
    for (int i = 0; i < (int)chunks.size(); ++i) {
        const JobDesc& J = slotOwner[chunks[i].job]->desc;
        if (groups.empty() || groups.back().kind != J.kind || groups.back().system != J.system)
            groups.push_back(Group{J.kind, J.system, i, 0});
        groups.back().count++;
    }
    if ((int)chunks.size() > I.capacity) {
        if (I.dChunks) cudaFree(I.dChunks);
        if (I.hChunks) cudaFreeHost(I.hChunks);
        I.capacity = std::max((int)chunks.size(), 2 * I.capacity);
        if (cudaMalloc(&I.dChunks, I.capacity * sizeof(Chunk)) != cudaSuccess ||
            cudaMallocHost(&I.hChunks, I.capacity * sizeof(Chunk)) != cudaSuccess)
            return set_error(CHAOS_E_NOMEM, "iteration buffers");
    }
    memcpy(I.hChunks, chunks.data(), chunks.size() * sizeof(Chunk));
    cudaStreamWaitEvent(I.stream, S->setupDone, 0);
    cudaError_t e = cudaMemcpyAsync(I.dChunks, I.hChunks, chunks.size() * sizeof(Chunk), cudaMemcpyHostToDevice,
                                    I.stream);
    if (e != cudaSuccess) return cuda_error(e, "iteration upload");
    if ((int)I.events.size() < 1 + (int)groups.size()) {
        destroy_events(I.events);
        I.events = make_events(1 + kMaxGroups);
    }
    int rc = launch_groups(groups, group_grids(groups, S->device), S->dTable, I.dChunks, I.dCounters, I.stream,
                           I.aux, I.events);
    if (rc) return rc;
    e = cudaEventRecord(I.done, I.stream);
    return e == cudaSuccess ? CHAOS_OK : cuda_error(e, "iteration event");
}

void scheduler_main(chaos_server* S) {
    cudaSetDevice(S->device);
    int k = 0;
    std::vector<Chunk> chunks;
    std::vector<Request*> slotOwner(S->maxActive, nullptr);
    for (;;) {
        Iteration& I = S->it[k & 1];
        Iteration& other = S->it[(k + 1) & 1];
        if (I.busy) {
            cudaEventSynchronize(I.done);
            finalize(S, I);
        }
        chunks.clear();
        bool quit = false, idleWait = false, drainOther = false;
        {
            std::unique_lock<std::mutex> lk(S->mu);
            admit_locked(S);
            for (Request* r : S->active) slotOwner[r->slot] = r;
            take_chunks_locked(S, I, chunks);
            if (chunks.empty()) {
                if (other.busy) drainOther = true;
                else if (S->stop && S->active.empty()) quit = true;
                else idleWait = true;
            }
            if (idleWait) {
                S->cvWork.wait_for(lk, std::chrono::milliseconds(5));
                continue;
            }
        }
        if (quit) break;
        if (drainOther) {
            cudaEventSynchronize(other.done);
            finalize(S, other);
            continue;
        }
        int rc = launch_iteration(S, I, chunks, slotOwner);
        if (rc != CHAOS_OK) {
            std::lock_guard<std::mutex> lk(S->mu);
            S->error = rc;
            for (auto& w : I.work) w.first->state = CHAOS_REQ_FAILED;
            I.work.clear();
            S->cvDone.notify_all();
            continue;
        }
        I.busy = true;
        {
            std::lock_guard<std::mutex> lk(S->mu);
            S->iterations++;
        }
        ++k;
    }
    for (Iteration& I : S->it)
        if (I.busy) {
            cudaEventSynchronize(I.done);
            finalize(S, I);
        }
    std::lock_guard<std::mutex> lk(S->mu);
    S->schedulerDone = true;
    S->cvComplete.notify_all();
}

void completer_main(chaos_server* S, int worker) {
    cudaSetDevice(S->device);
    cudaStream_t copy = S->copy[worker];
    for (;;) {
        Request* r = nullptr;
        {
            std::unique_lock<std::mutex> lk(S->mu);
            S->cvComplete.wait_for(lk, std::chrono::milliseconds(5),
                                   [&] { return !S->completed.empty() || S->schedulerDone; });
            if (S->completed.empty()) {
                if (S->schedulerDone) {
                    S->completersRunning--;
                    S->cvComplete.notify_all();
                    break;
                }
                continue;
            }
            r = S->completed.front();
            S->completed.pop_front();
        }
        int rc = CHAOS_OK;
        if (r->dLabels) {  // the reference clustering of a basins map
            chaos_exec ex{CHAOS_FP64, CHAOS_MEM_DEVICE, copy, S->device};
            Call c;
            rc = c.begin(&ex);
            if (!rc) rc = dbscan_compat_device(c, r->desc.bas.avgPeaks, r->desc.bas.avgIntervals, r->desc.bas.flags,
                                               r->nPoints, r->job.eps, r->dLabels);
            rc = c.finish(rc);
            if (!rc && S->memory == CHAOS_MEM_HOST)
                cudaMemcpyAsync(r->job.labels, r->dLabels, r->nPoints * sizeof(int), cudaMemcpyDeviceToHost, copy);
        }
        for (const HostOut& o : r->outs) cudaMemcpyAsync(o.host, o.dev, o.bytes, cudaMemcpyDeviceToHost, copy);
        if (r->devBlock) cudaFreeAsync(r->devBlock, copy);
        cudaError_t e = cudaStreamSynchronize(copy);
        if (e != cudaSuccess && !rc) rc = cuda_error(e, "completion");
        std::lock_guard<std::mutex> lk(S->mu);
        r->state = rc == CHAOS_OK ? CHAOS_REQ_DONE : CHAOS_REQ_FAILED;
        r->latency = seconds(Clock::now() - r->tSubmit);
        S->used -= r->bytes;
        if (rc == CHAOS_OK) {
            S->latencies.push_back(r->latency);
            S->stepsDone += r->steps;
        } else {
            S->failed++;
        }
        S->cvDone.notify_all();
        S->cvWork.notify_all();
    }
}

double percentile(std::vector<double> v, double q) {
    if (v.empty()) return 0.0;
    std::sort(v.begin(), v.end());
    const double pos = q * (v.size() - 1);
    const size_t i = (size_t)pos;
    const double f = pos - i;
    return i + 1 < v.size() ? v[i] * (1 - f) + v[i + 1] * f : v[i];
}

}  // namespace

extern "C" {

int chaos_server_create(const chaos_exec* ex, size_t hbmBudgetBytes, int maxActive, double iterationSteps,
                        chaos_server** server) {
    if (!server || maxActive < 1 || maxActive > (1 << 20) || !(iterationSteps > 0) || hbmBudgetBytes == 0)
        return set_error(CHAOS_E_ARGS, "bad server arguments");
    *server = nullptr;
    Call c;
    int rc = c.begin(ex);
    if (rc) return rc;
    c.finish(CHAOS_OK);
    chaos_server* S = new (std::nothrow) chaos_server;
    if (!S) return set_error(CHAOS_E_NOMEM, "host allocation");
    S->device = c.device;
    S->memory = c.ex.memory;
    S->budget = hbmBudgetBytes;
    S->maxActive = maxActive;
    S->iterationSteps = iterationSteps;
    S->pool = c.pool;
    cudaError_t e = cudaStreamCreateWithFlags(&S->setup, cudaStreamNonBlocking);
    for (int w = 0; w < kCompleters && e == cudaSuccess; ++w) {
        cudaStream_t cs;
        e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
        if (e == cudaSuccess) S->copy.push_back(cs);
    }
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&S->setupDone, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMalloc(&S->dTable, (size_t)maxActive * sizeof(JobDesc));
    for (Iteration& I : S->it) {
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&I.stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&I.done, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaMalloc(&I.dCounters, kMaxGroups * sizeof(int));
        for (int a = 0; a < kAuxPerIteration && e == cudaSuccess; ++a) {
            cudaStream_t s;
            e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
            if (e == cudaSuccess) I.aux.push_back(s);
        }
    }
    if (e != cudaSuccess) {
        rc = cuda_error(e, "server setup");
        chaos_server_destroy(S);
        return rc;
    }
    cudaEventRecord(S->setupDone, S->setup);
    for (int i = maxActive - 1; i >= 0; --i) S->freeSlots.push_back(i);
    S->scheduler = std::thread(scheduler_main, S);
    S->completersRunning = kCompleters;
    for (int w = 0; w < kCompleters; ++w) S->completers.emplace_back(completer_main, S, w);
    *server = S;
    return CHAOS_OK;
}

int chaos_server_submit(chaos_server* S, const chaos_job* job, long long* requestId) {
    if (!S || !job) return set_error(CHAOS_E_ARGS, "null server or job");
    std::unique_ptr<Request> r(new (std::nothrow) Request);
    if (!r) return set_error(CHAOS_E_NOMEM, "host allocation");
    r->job = *job;
    const int nx = system_supported(job->system) ? system_nx(job->system) : 0;
    const int na = system_supported(job->system) ? system_na(job->system) : 0;
    const int nr = job->kind == CHAOS_JOB_BIF1D ? 2 : 4, nm = job->kind == CHAOS_JOB_BIF1D ? 1 : 2;
    if (job->initialConditions) r->ic.assign(job->initialConditions, job->initialConditions + nx);
    if (job->ranges) r->ranges.assign(job->ranges, job->ranges + nr);
    if (job->values) r->values.assign(job->values, job->values + na);
    if (job->indicesOfMutVars) r->mut.assign(job->indicesOfMutVars, job->indicesOfMutVars + nm);
    r->job.initialConditions = job->initialConditions ? r->ic.data() : nullptr;
    r->job.ranges = job->ranges ? r->ranges.data() : nullptr;
    r->job.values = job->values ? r->values.data() : nullptr;
    r->job.indicesOfMutVars = job->indicesOfMutVars ? r->mut.data() : nullptr;
    // validate and size the device block with a counting allocator
    size_t bytes = 0;
    std::vector<HostOut> outs;
    auto count = [&](size_t b) -> void* {
        bytes += (b + 255) & ~size_t(255);
        return (void*)(uintptr_t)256;  // never dereferenced
    };
    int rc = prepare_job(r->job, S->memory, r->desc, outs, count);
    if (rc) return rc;
    r->nPoints = r->desc.nPoints;
    if (job->kind == CHAOS_JOB_BASINS && job->labels && job->eps > 0 && S->memory == CHAOS_MEM_HOST)
        bytes += ((size_t)r->nPoints * sizeof(int) + 255) & ~size_t(255);
    r->bytes = bytes;
    r->perPoint = work_per_point(r->desc);
    r->steps = r->perPoint * r->nPoints;
    // two points per thread for the RK4 systems, as in batches
    r->chunk = (job->system <= SYS_CHEN_RK4 ? 2 : 1) * batch_block_size();
    std::lock_guard<std::mutex> lk(S->mu);
    if (S->stop) return set_error(CHAOS_E_BUSY, "server is shutting down");
    if (!S->started) {
        S->started = true;
        S->tFirst = Clock::now();
    }
    r->id = S->nextId++;
    r->tSubmit = Clock::now();
    if (requestId) *requestId = r->id;
    S->pending.push_back(r.get());
    S->all[r->id] = std::move(r);
    S->cvWork.notify_all();
    return CHAOS_OK;
}

int chaos_server_poll(chaos_server* S, long long id, int* state) {
    if (!S || !state) return set_error(CHAOS_E_ARGS, "null argument");
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->all.find(id);
    if (it == S->all.end()) return set_error(CHAOS_E_ARGS, "unknown request %lld", id);
    *state = it->second->state;
    return CHAOS_OK;
}

int chaos_server_wait(chaos_server* S, long long id, double timeoutSeconds, int* state) {
    if (!S) return set_error(CHAOS_E_ARGS, "null server");
    std::unique_lock<std::mutex> lk(S->mu);
    auto it = S->all.find(id);
    if (it == S->all.end()) return set_error(CHAOS_E_ARGS, "unknown request %lld", id);
    Request* r = it->second.get();
    const auto deadline = Clock::now() + std::chrono::duration_cast<Clock::duration>(
                                             std::chrono::duration<double>(std::max(timeoutSeconds, 0.0)));
    while (r->state != CHAOS_REQ_DONE && r->state != CHAOS_REQ_FAILED) {
        if (S->cvDone.wait_until(lk, deadline) == std::cv_status::timeout &&
            r->state != CHAOS_REQ_DONE && r->state != CHAOS_REQ_FAILED) {
            if (state) *state = r->state;
            return set_error(CHAOS_E_TIMEOUT, "request %lld not done within %.3f s", id, timeoutSeconds);
        }
    }
    if (state) *state = r->state;
    return r->state == CHAOS_REQ_DONE ? CHAOS_OK : (S->error ? S->error : CHAOS_E_CUDA);
}

double chaos_server_latency(chaos_server* S, long long id) {
    if (!S) return -1;
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->all.find(id);
    return it == S->all.end() ? -1 : it->second->latency;
}

int chaos_server_stats(chaos_server* S, double* st, int n) {
    if (!S || !st) return set_error(CHAOS_E_ARGS, "null argument");
    std::lock_guard<std::mutex> lk(S->mu);
    double v[12];
    v[0] = (double)S->latencies.size();
    v[1] = (double)S->failed;
    v[2] = (double)S->pending.size();
    v[3] = (double)S->active.size();
    v[4] = percentile(S->latencies, 0.50);
    v[5] = percentile(S->latencies, 0.99);
    double sum = 0;
    for (double x : S->latencies) sum += x;
    v[6] = S->latencies.empty() ? 0 : sum / S->latencies.size();
    v[7] = (double)S->stepsDone;
    v[8] = S->started ? seconds(Clock::now() - S->tFirst) : 0.0;
    v[9] = (double)S->iterations;
    v[10] = (double)S->peakUsed;
    v[11] = S->latencies.empty() ? 0 : *std::max_element(S->latencies.begin(), S->latencies.end());
    for (int i = 0; i < n && i < 12; ++i) st[i] = v[i];
    return CHAOS_OK;
}

int chaos_server_destroy(chaos_server* S) {
    if (!S) return CHAOS_OK;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stop = true;
        for (Request* r : S->pending) r->state = CHAOS_REQ_FAILED;
        S->pending.clear();
        S->cvWork.notify_all();
        S->cvDone.notify_all();
    }
    if (S->scheduler.joinable()) S->scheduler.join();
    else S->schedulerDone = true;
    for (std::thread& t : S->completers)
        if (t.joinable()) t.join();
    cudaSetDevice(S->device);
    for (Iteration& I : S->it) {
        if (I.stream) cudaStreamSynchronize(I.stream);
        destroy_events(I.events);
        if (I.done) cudaEventDestroy(I.done);
        if (I.dChunks) cudaFree(I.dChunks);
        if (I.hChunks) cudaFreeHost(I.hChunks);
        if (I.dCounters) cudaFree(I.dCounters);
        for (cudaStream_t s : I.aux) cudaStreamDestroy(s);
        if (I.stream) cudaStreamDestroy(I.stream);
    }
    if (S->setup) cudaStreamSynchronize(S->setup);
    for (cudaStream_t cs : S->copy) cudaStreamSynchronize(cs);
    if (S->dTable) cudaFree(S->dTable);
    if (S->setupDone) cudaEventDestroy(S->setupDone);
    if (S->setup) cudaStreamDestroy(S->setup);
    for (cudaStream_t cs : S->copy) cudaStreamDestroy(cs);
    delete S;
    return CHAOS_OK;
}

}  // extern "C"
