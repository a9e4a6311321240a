// Host side of batched sweeps: job validation, descriptors, chunk lists, the
// persistent launch and its CUDA-graph replay (declared in include/chaos_gb300.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/chaos_gb300.h"
#include "batch.h"
#include "capi_internal.h"
#include "systems.h"

using namespace chaos;

namespace {

struct HostOut {  // a device output of one job and where it goes on the host
    void* host;
    void* dev;
    size_t bytes;
};

// Work per point of a job (trajectory-steps), the key of the longest-first order.
long long work_per_point(const JobDesc& J) {
    if (J.kind == CHAOS_JOB_LLE2D) return J.lp.trans + 2LL * J.lp.ntp * (J.lp.calcBlocks + 1);
    return (long long)J.sp.S + (long long)J.sp.B * J.sp.preScaller;
}

// Validates one job and fills its descriptor; device buffers for its outputs
// come from `alloc` (host-memory batches) or are the caller's pointers.
template <class Alloc>
int prepare_job(const chaos_job& j, int memory, JobDesc& J, std::vector<HostOut>& outs, Alloc alloc) {
    memset(&J, 0, sizeof J);
    J.kind = j.kind;
    J.system = j.system;
    auto out = [&](void* user, size_t bytes) -> void* {
        if (!user) return nullptr;
        if (memory == CHAOS_MEM_DEVICE) return user;
        void* d = alloc(bytes);
        if (d) outs.push_back({user, d, bytes});
        return d;
    };
    const int nx = system_supported(j.system) ? system_nx(j.system) : 0;
    const int na = system_supported(j.system) ? system_na(j.system) : 0;
    int rc;
    switch (j.kind) {
        case CHAOS_JOB_BIF1D: {
            rc = fill_sweep(J.sp, j.system, 1, j.tMax, j.nPts, j.h, nx, j.initialConditions, j.ranges,
                            j.indicesOfMutVars, j.writableVar, j.maxValue, j.transientTime, j.values, na,
                            j.preScaller, false);
            if (rc) return rc;
            if (!j.counts || !j.flags) return set_error(CHAOS_E_ARGS, "bifurcation job needs counts and flags");
            if ((j.peaks || j.intervals) && j.peakCapacity < 1) return set_error(CHAOS_E_ARGS, "peakCapacity < 1");
            const long long n = J.sp.nPoints;
            J.nPoints = n;
            J.bif.cap = j.peakCapacity;
            J.bif.counts = (int*)out(j.counts, n * sizeof(int));
            J.bif.flags = (int*)out(j.flags, n * sizeof(int));
            J.bif.first = (double*)out(j.first, n * sizeof(double));
            J.bif.peaks = (double*)out(j.peaks, (size_t)n * j.peakCapacity * sizeof(double));
            J.bif.intervals = (double*)out(j.intervals, (size_t)n * j.peakCapacity * sizeof(double));
            break;
        }
        case CHAOS_JOB_BASINS: {
            rc = fill_sweep(J.sp, j.system, 2, j.tMax, j.nPts, j.h, nx, j.initialConditions, j.ranges,
                            j.indicesOfMutVars, j.writableVar, j.maxValue, j.transientTime, j.values, na,
                            j.preScaller, true);
            if (rc) return rc;
            if (!j.flags || !j.avgPeaks || !j.avgIntervals)
                return set_error(CHAOS_E_ARGS, "basins job needs flags, avgPeaks and avgIntervals");
            const long long n = J.sp.nPoints;
            J.nPoints = n;
            J.bas.flags = (int*)out(j.flags, n * sizeof(int));
            J.bas.avgPeaks = (double*)out(j.avgPeaks, n * sizeof(double));
            J.bas.avgIntervals = (double*)out(j.avgIntervals, n * sizeof(double));
            J.bas.counts = (int*)out(j.counts, n * sizeof(int));
            J.bas.last = nullptr;
            break;
        }
        case CHAOS_JOB_LLE2D: {
            rc = fill_lle(J.lp, j.system, j.tMax, j.NT, j.nPts, j.h, j.eps, j.initialConditions, nx, j.ranges,
                          j.indicesOfMutVars, j.transientTime, j.values, na);
            if (rc) return rc;
            if (!system_has_difference_form(j.system))
                return set_error(CHAOS_E_UNSUPPORTED, "batched LLE jobs need a quadratic RK4 system (0-2)");
            if (!j.lle) return set_error(CHAOS_E_ARGS, "LLE job needs lle");
            J.nPoints = J.lp.nPoints;
            J.lle = (double*)out(j.lle, J.nPoints * sizeof(double));
            break;
        }
        default:
            return set_error(CHAOS_E_ARGS, "unknown job kind %d", j.kind);
    }
    return CHAOS_OK;
}

struct Group {
    int kind, system;
    int begin, count;  // range in the chunk list
};

// Block-sized chunks of point ranges, grouped by (kind, system); inside a
// group the jobs with the most work per point come first.
void make_chunks(const std::vector<JobDesc>& jobs, std::vector<Chunk>& chunks, std::vector<Group>& groups) {
    const int block = batch_block_size();
    std::vector<int> order(jobs.size());
    for (size_t i = 0; i < jobs.size(); ++i) order[i] = (int)i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        if (jobs[a].kind != jobs[b].kind) return jobs[a].kind < jobs[b].kind;
        if (jobs[a].system != jobs[b].system) return jobs[a].system < jobs[b].system;
        return work_per_point(jobs[a]) > work_per_point(jobs[b]);
    });
    chunks.clear();
    groups.clear();
    for (int j : order) {
        const JobDesc& J = jobs[j];
        if (groups.empty() || groups.back().kind != J.kind || groups.back().system != J.system)
            groups.push_back(Group{J.kind, J.system, (int)chunks.size(), 0});
        const int size = J.kind == CHAOS_JOB_LLE2D ? 2 * block : block;
        for (long long b = 0; b < J.nPoints; b += size)
            chunks.push_back(Chunk{j, (int)std::min<long long>(size, J.nPoints - b), b});
        groups.back().count = (int)chunks.size() - groups.back().begin;
    }
}

// Resets the group counters on `st`, forks one branch per group onto the
// auxiliary streams, launches each group's persistent kernel and joins the
// branches back into `st` (works the same inside a stream capture).
// Grid of every group's persistent kernel: resident blocks, at most one per chunk
// (queried before any capture: occupancy queries are not allowed inside one).
std::vector<int> group_grids(const std::vector<Group>& groups, int device) {
    std::vector<int> grid(groups.size());
    for (size_t g = 0; g < groups.size(); ++g)
        grid[g] = std::max(1, std::min(groups[g].count, group_resident_blocks(groups[g].kind, groups[g].system, device)));
    return grid;
}

int launch_groups(const std::vector<Group>& groups, const std::vector<int>& grids, const JobDesc* dJobs,
                  const Chunk* dChunks, int* dCounters, cudaStream_t st, const std::vector<cudaStream_t>& aux,
                  const std::vector<cudaEvent_t>& events) {
    cudaError_t e = reset_counters(dCounters, (int)groups.size(), st);
    if (e == cudaSuccess) e = cudaEventRecord(events[0], st);
    for (size_t g = 0; g < groups.size() && e == cudaSuccess; ++g) {
        cudaStream_t s = aux[g % aux.size()];
        e = cudaStreamWaitEvent(s, events[0], 0);
        if (e == cudaSuccess)
            e = launch_group(groups[g].kind, groups[g].system, dJobs, dChunks + groups[g].begin, groups[g].count,
                             dCounters + g, grids[g], s);
        if (e == cudaSuccess) e = cudaEventRecord(events[1 + g], s);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(st, events[1 + g], 0);
    }
    return e == cudaSuccess ? CHAOS_OK : cuda_error(e, "batch launch");
}

constexpr int kMaxGroups = 32;

std::vector<cudaEvent_t> make_events(int n) {
    std::vector<cudaEvent_t> ev(n);
    for (auto& x : ev) cudaEventCreateWithFlags(&x, cudaEventDisableTiming);
    return ev;
}

void destroy_events(std::vector<cudaEvent_t>& ev) {
    for (auto x : ev) cudaEventDestroy(x);
    ev.clear();
}

}  // namespace

struct chaos_batch {
    chaos_exec ex{};
    int device = 0;
    cudaStream_t user = nullptr;    // the caller's stream: runs are ordered after its earlier work
    cudaStream_t stream = nullptr;  // the plan's own stream (a default stream cannot be captured)
    cudaEvent_t in = nullptr, out = nullptr;
    std::vector<void*> buffers;  // cudaMalloc'd, freed by destroy
    std::vector<HostOut> outs;
    JobDesc* dJobs = nullptr;
    Chunk* dChunks = nullptr;
    int* dCounters = nullptr;
    std::vector<Group> groups;
    std::vector<cudaStream_t> aux;
    std::vector<cudaEvent_t> events;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

extern "C" {

int chaos_run_batch(const chaos_exec* ex, const chaos_job* jobs, int nJobs) {
    if (nJobs < 0 || (nJobs > 0 && !jobs)) return set_error(CHAOS_E_ARGS, "bad job list");
    Call c;
    int rc = c.begin(ex);
    if (rc) return rc;
    std::vector<JobDesc> desc(nJobs);
    std::vector<HostOut> outs;
    for (int i = 0; i < nJobs; ++i) {
        rc = prepare_job(jobs[i], c.ex.memory, desc[i], outs, [&](size_t b) { return c.alloc(b); });
        if (rc) return c.finish(rc);
        if (c.failed) return c.finish(CHAOS_E_NOMEM);
    }
    std::vector<Chunk> chunks;
    std::vector<Group> groups;
    make_chunks(desc, chunks, groups);
    if ((int)groups.size() > kMaxGroups) return c.finish(set_error(CHAOS_E_ARGS, "too many (kind, system) groups"));
    JobDesc* dJobs = (JobDesc*)c.alloc(desc.size() * sizeof(JobDesc) + 16);
    Chunk* dChunks = (Chunk*)c.alloc(chunks.size() * sizeof(Chunk) + 16);
    int* counters = (int*)c.alloc(kMaxGroups * sizeof(int));
    if (c.failed) return c.finish(CHAOS_E_NOMEM);
    cudaError_t e = cudaMemcpyAsync(dJobs, desc.data(), desc.size() * sizeof(JobDesc), cudaMemcpyHostToDevice, c.stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(dChunks, chunks.data(), chunks.size() * sizeof(Chunk), cudaMemcpyHostToDevice, c.stream);
    if (e != cudaSuccess) return c.finish(cuda_error(e, "batch upload"));
    std::vector<cudaStream_t> aux;
    if ((rc = aux_streams(c.device, aux))) return c.finish(rc);
    std::vector<cudaEvent_t> events = make_events(1 + (int)groups.size());
    rc = launch_groups(groups, group_grids(groups, c.device), dJobs, dChunks, counters, c.stream, aux, events);
    for (const HostOut& o : outs)
        if (!rc) rc = c.to_host(o.host, o.dev, o.bytes);
    // the host-side descriptor arrays are copied asynchronously: wait before they go out of scope
    if (!rc) {
        e = cudaStreamSynchronize(c.stream);
        if (e != cudaSuccess) rc = cuda_error(e, "batch");
    }
    destroy_events(events);
    return c.finish(rc);
}

int chaos_batch_create(const chaos_exec* ex, const chaos_job* jobs, int nJobs, chaos_batch** plan) {
    if (!plan || nJobs < 0 || (nJobs > 0 && !jobs)) return set_error(CHAOS_E_ARGS, "bad batch arguments");
    *plan = nullptr;
    Call c;  // resolves device and stream only; the plan owns its memory
    int rc = c.begin(ex);
    if (rc) return rc;
    chaos_batch* b = new (std::nothrow) chaos_batch;
    if (!b) return c.finish(set_error(CHAOS_E_NOMEM, "host allocation"));
    b->ex = c.ex;
    b->device = c.device;
    b->user = c.stream;
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->in, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->out, cudaEventDisableTiming) != cudaSuccess) {
        chaos_batch_destroy(b);
        return c.finish(set_error(CHAOS_E_CUDA, "stream or event create"));
    }
    auto dalloc = [&](size_t bytes) -> void* {
        void* p = nullptr;
        if (cudaMalloc(&p, bytes ? bytes : 16) != cudaSuccess) return nullptr;
        b->buffers.push_back(p);
        return p;
    };
    std::vector<JobDesc> desc(nJobs);
    for (int i = 0; i < nJobs && rc == CHAOS_OK; ++i) {
        size_t before = b->outs.size();
        rc = prepare_job(jobs[i], b->ex.memory, desc[i], b->outs, dalloc);
        if (rc == CHAOS_OK && b->ex.memory == CHAOS_MEM_HOST) {
            for (size_t k = before; k < b->outs.size(); ++k)
                if (!b->outs[k].dev) rc = set_error(CHAOS_E_NOMEM, "device allocation");
        }
    }
    std::vector<Chunk> chunks;
    if (rc == CHAOS_OK) {
        make_chunks(desc, chunks, b->groups);
        if ((int)b->groups.size() > kMaxGroups) rc = set_error(CHAOS_E_ARGS, "too many (kind, system) groups");
    }
    if (rc == CHAOS_OK) {
        b->dJobs = (JobDesc*)dalloc(desc.size() * sizeof(JobDesc));
        b->dChunks = (Chunk*)dalloc(chunks.size() * sizeof(Chunk));
        b->dCounters = (int*)dalloc(kMaxGroups * sizeof(int));
        if (!b->dJobs || !b->dChunks || !b->dCounters) rc = set_error(CHAOS_E_NOMEM, "device allocation");
    }
    if (rc == CHAOS_OK) rc = aux_streams(b->device, b->aux);
    if (rc == CHAOS_OK) {
        cudaMemcpy(b->dJobs, desc.data(), desc.size() * sizeof(JobDesc), cudaMemcpyHostToDevice);
        cudaMemcpy(b->dChunks, chunks.data(), chunks.size() * sizeof(Chunk), cudaMemcpyHostToDevice);
        b->events = make_events(1 + (int)b->groups.size());
        const std::vector<int> grids = group_grids(b->groups, b->device);
        cudaError_t e = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            int lrc = launch_groups(b->groups, grids, b->dJobs, b->dChunks, b->dCounters, b->stream, b->aux,
                                    b->events);
            e = cudaStreamEndCapture(b->stream, &b->graph);
            if (lrc != CHAOS_OK && e == cudaSuccess) e = cudaErrorUnknown;
        }
        if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, b->graph, 0);
        if (e != cudaSuccess) rc = cuda_error(e, "batch graph capture");
    }
    if (rc != CHAOS_OK) {
        chaos_batch_destroy(b);
        return c.finish(rc);
    }
    *plan = b;
    return c.finish(CHAOS_OK);
}

int chaos_batch_run(chaos_batch* b) {
    if (!b) return set_error(CHAOS_E_ARGS, "null plan");
    int prev = 0;
    cudaGetDevice(&prev);
    if (prev != b->device) cudaSetDevice(b->device);
    cudaError_t e = cudaEventRecord(b->in, b->user);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(b->stream, b->in, 0);
    if (e == cudaSuccess) e = cudaGraphLaunch(b->exec, b->stream);
    if (e == cudaSuccess) e = cudaEventRecord(b->out, b->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(b->user, b->out, 0);
    for (const HostOut& o : b->outs)
        if (e == cudaSuccess) e = cudaMemcpyAsync(o.host, o.dev, o.bytes, cudaMemcpyDeviceToHost, b->user);
    if (e == cudaSuccess && b->ex.memory == CHAOS_MEM_HOST) e = cudaStreamSynchronize(b->user);
    if (prev != b->device) cudaSetDevice(prev);
    return e == cudaSuccess ? CHAOS_OK : cuda_error(e, "batch run");
}

int chaos_batch_destroy(chaos_batch* b) {
    if (!b) return CHAOS_OK;
    int prev = 0;
    cudaGetDevice(&prev);
    if (prev != b->device) cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->in) cudaEventDestroy(b->in);
    if (b->out) cudaEventDestroy(b->out);
    if (b->stream) cudaStreamDestroy(b->stream);
    if (b->graph) cudaGraphDestroy(b->graph);
    destroy_events(b->events);
    for (void* p : b->buffers) cudaFree(p);
    if (prev != b->device) cudaSetDevice(prev);
    delete b;
    return CHAOS_OK;
}

}  // extern "C"
