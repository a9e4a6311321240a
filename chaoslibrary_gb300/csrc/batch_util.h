// Host helpers shared by batched runs (batch_host.cu) and the server (server.cu):
// job validation into device descriptors, chunk lists grouped by (kind,
// system), and the forked launch of the group kernels.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "../../include/chaos_gb300.h"
#include "batch.h"
#include "capi_internal.h"
#include "systems.h"

namespace chaos {

struct HostOut {  // a device output of one job and where it goes on the host
    void* host;
    void* dev;
    size_t bytes;
};

// Work per point of a job (trajectory-steps), the key of the longest-first order.
inline long long work_per_point(const JobDesc& J) {
    if (J.kind == CHAOS_JOB_LLE2D || J.kind == CHAOS_JOB_LLE2D_FF32)
        return J.lp.trans + 2LL * J.lp.ntp * (J.lp.calcBlocks + 1);
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
    if (j.system == SYS_USER)
        return set_error(CHAOS_E_UNSUPPORTED, "batched and served jobs use the built-in systems");
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
        case CHAOS_JOB_LLE2D:
        case CHAOS_JOB_LLE2D_FF32: {
            rc = fill_lle(J.lp, j.system, j.tMax, j.NT, j.nPts, j.h, j.eps, j.initialConditions, nx, j.ranges,
                          j.indicesOfMutVars, j.transientTime, j.values, na);
            if (rc) return rc;
            if (j.kind == CHAOS_JOB_LLE2D_FF32 && !system_has_difference_form(j.system))
                return set_error(CHAOS_E_UNSUPPORTED, "float-float LLE jobs need an RK4 system (0-2)");
            if (!system_has_fp32_lle(j.system))
                return set_error(CHAOS_E_UNSUPPORTED, "batched LLE jobs need a quadratic RK4 system (0-2) or Chameleon");
            if (J.lp.twin != 0)
                return set_error(CHAOS_E_UNSUPPORTED, "batched LLE jobs are FP32: the reference twin start is FP64 only");
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
inline void make_chunks(const std::vector<JobDesc>& jobs, std::vector<Chunk>& chunks, std::vector<Group>& groups) {
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
        // two points per thread for the RK4 systems
        const int size = J.system <= SYS_CHEN_RK4 ? 2 * block : block;
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
inline std::vector<int> group_grids(const std::vector<Group>& groups, int device) {
    std::vector<int> grid(groups.size());
    for (size_t g = 0; g < groups.size(); ++g)
        grid[g] = std::max(1, std::min(groups[g].count, group_resident_blocks(groups[g].kind, groups[g].system, device)));
    return grid;
}

inline int launch_groups(const std::vector<Group>& groups, const std::vector<int>& grids, const JobDesc* dJobs,
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

inline std::vector<cudaEvent_t> make_events(int n) {
    std::vector<cudaEvent_t> ev(n);
    for (auto& x : ev) cudaEventCreateWithFlags(&x, cudaEventDisableTiming);
    return ev;
}

inline void destroy_events(std::vector<cudaEvent_t>& ev) {
    for (auto x : ev) cudaEventDestroy(x);
    ev.clear();
}

}  // namespace chaos
