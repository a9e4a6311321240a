// Device-side description of a batch of sweeps (batch.cu, batch_host.cu).
#pragma once

#include <cuda_runtime.h>

#include "launch.h"

namespace chaos {

// One job of a batch: its kind (CHAOS_JOB_*), system, parameters and outputs
// (device pointers).
struct JobDesc {
    int kind;
    int system;
    long long nPoints;
    SweepParams sp;  // bifurcation / basins jobs
    BifOut bif;
    BasinsOut bas;
    LleParams lp;    // LLE jobs
    double* lle;
};

// A contiguous range of one job's points, processed by one block.
struct Chunk {
    int job;
    int count;
    long long begin;
};

int batch_block_size();
// resident blocks of the group kernel of (kind, system) on a device; 0 = no such kernel
int group_resident_blocks(int kind, int system, int device);
cudaError_t reset_counters(int* counters, int n, cudaStream_t st);  // n <= 32
cudaError_t launch_group(int kind, int system, const JobDesc* jobs, const Chunk* chunks, int count, int* counter,
                         int gridBlocks, cudaStream_t st);
// the float-float LLE group (CHAOS_JOB_LLE2D_FF32; kern_ff.cu): resident blocks and launch
int group_ff_resident_blocks(int system, int device);
cudaError_t launch_group_ff(int system, const JobDesc* jobs, const Chunk* chunks, int count, int* counter,
                            int gridBlocks, cudaStream_t st);

}  // namespace chaos
