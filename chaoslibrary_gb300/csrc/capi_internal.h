// Internal helpers of the C-ABI layer shared by its translation units.
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "../../include/chaos_gb300.h"

namespace chaos {

int set_error(int code, const char* fmt, ...);
int cuda_error(cudaError_t e, const char* what);

// One C-ABI call: resolves the device and stream, hands out stream-ordered
// device buffers from the library's pool (freed when the call finishes),
// stages host inputs and outputs, and synchronises host-memory calls.
struct Call {
    chaos_exec ex{};
    int device = 0, prevDevice = 0;
    cudaStream_t stream = nullptr;
    cudaMemPool_t pool = nullptr;
    std::vector<void*> owned;
    bool failed = false;

    int begin(const chaos_exec* e);
    void* alloc(size_t bytes);  // device scratch, freed at finish()
    const void* input(const void* user, size_t bytes);  // device view of a caller input
    void* output(void* user, size_t bytes);             // device buffer for a caller output
    int to_host(void* host, const void* dev, size_t bytes);  // copy back (host-memory calls)
    int finish(int rc);
};

}  // namespace chaos
