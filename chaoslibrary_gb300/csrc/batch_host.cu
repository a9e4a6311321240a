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
#include "batch_util.h"

using namespace chaos;

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
    long long kernels = 0;  // kernel nodes of the graph (launches per replay)
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
        if (e == cudaSuccess) {
            // captured launches ran nothing: count them at each replay instead
            size_t nodes = 0;
            cudaGraphGetNodes(b->graph, nullptr, &nodes);
            std::vector<cudaGraphNode_t> list(nodes);
            if (nodes) cudaGraphGetNodes(b->graph, list.data(), &nodes);
            for (cudaGraphNode_t nd : list) {
                cudaGraphNodeType t;
                if (cudaGraphNodeGetType(nd, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++b->kernels;
            }
            note_launch(-b->kernels);
        }
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
    if (e == cudaSuccess) note_launch(b->kernels);
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
