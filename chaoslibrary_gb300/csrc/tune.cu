// Self-timing tuner of the FP32 sweeps (chaos_autotune, declared in
// include/chaos_gb300.h). For each RK4 system and each of the 1-D
// bifurcation, basins and LLE map kernels it times the candidate launch
// shapes -- one or two points per thread (packed FP32x2 lanes), the LLE map's
// register shapes, and the block size 64 / 128 / 256 -- on a probe sweep that
// fills the GPU eight times over, keeps the fastest, and installs it for
// every later call in the process. Results never depend on the shape (the
// paired and single-point kernels are bit-identical); only speed does.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "../../include/chaos_gb300.h"
#include "capi_internal.h"
#include "launch.h"
#include "systems.h"

using namespace chaos;

namespace {

struct SystemProbe {
    int system;
    double values[3], ic[3];
    double bifRange[2];  // swept parameter values[bifMut]
    int bifMut;
};

// the RK4 systems at the parameters of their benchmarks
const SystemProbe kProbes[3] = {
    {SYS_LORENZ_RK4, {10.0, 28.0, 8.0 / 3.0}, {0.1, 0.1, 0.1}, {20.0, 200.0}, 1},
    {SYS_ROSSLER_RK4, {0.2, 0.2, 5.7}, {1.0, 1.0, 1.0}, {2.0, 10.0}, 2},
    {SYS_CHEN_RK4, {35.0, 3.0, 28.0}, {-10.0, 0.0, 37.0}, {20.0, 30.0}, 2},
};

// candidate shapes per kind (form * 1024 + block)
std::vector<int> candidates(int kind) {
    std::vector<int> c;
    for (int block : {64, 128, 256}) {
        c.push_back(1 * 1024 + block);
        c.push_back(2 * 1024 + block);
    }
    if (kind <= 1)  // bifurcation and basins: also the hybrid (packed transient, recorded part lane by lane)
        for (int block : {64, 128, 256}) c.push_back(3 * 1024 + block);
    if (kind == 2) {  // the LLE map: one point per thread exists only as the 12 / 16 register shapes
        c.erase(std::remove_if(c.begin(), c.end(), [](int s) { return s / 1024 == 1; }), c.end());
        c.push_back(12 * 1024 + 128);
        c.push_back(16 * 1024 + 128);
    }
    return c;
}

}  // namespace

extern "C" int chaos_autotune(const chaos_exec* ex, double* table, int nTable) {
    Call c;
    int rc = c.begin(ex);
    if (rc) return rc;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c.device);
    const long long n = 8LL * std::max(sms, 1) * 1024;  // points of a probe sweep
    const int side = (int)std::ceil(std::sqrt((double)n));
    const long long n2 = (long long)side * side;
    int* i1 = (int*)c.alloc(n * sizeof(int));
    int* i2 = (int*)c.alloc(n2 * sizeof(int));
    double* d1 = (double*)c.alloc(n2 * sizeof(double));
    double* d2 = (double*)c.alloc(n2 * sizeof(double));
    int* i3 = (int*)c.alloc(n2 * sizeof(int));
    if (c.failed) return c.finish(CHAOS_E_NOMEM);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    int row = 0;
    cudaError_t err = cudaSuccess;
    for (int kind = 0; kind < 3 && err == cudaSuccess; ++kind) {
        for (const SystemProbe& sp : kProbes) {
            SweepParams P;
            LleParams L;
            if (kind == 0) {
                rc = fill_sweep(P, sp.system, 1, 20.0, (int)n, 0.01, 3, sp.ic, sp.bifRange, &sp.bifMut, 0, 1e4, 20.0,
                                sp.values, 3, 1, false);
            } else if (kind == 1) {
                const double r[4] = {-20.0, 20.0, -20.0, 20.0};
                const int mut[2] = {0, 1};
                rc = fill_sweep(P, sp.system, 2, 20.0, side, 0.01, 3, sp.ic, r, mut, 0, 1e8, 20.0, sp.values, 3, 1,
                                true);
            } else {
                const double r[4] = {sp.values[0] * 0.8, sp.values[0] * 1.2, sp.values[2] * 0.8, sp.values[2] * 1.2};
                const int mut[2] = {0, 2};
                rc = fill_lle(L, sp.system, 10.0, 0.1, side, 0.01, 1e-8, sp.ic, 3, r, mut, 5.0, sp.values, 3);
                L.twin = 0;
            }
            if (rc) break;
            const int keep = get_launch_shape(kind, sp.system);
            auto run = [&]() -> cudaError_t {
                if (kind == 0) return launch_bif_f32(P, BifOut{i1, i3, nullptr, nullptr, nullptr, 0}, c.stream);
                if (kind == 1) return launch_basins_f32(P, BasinsOut{i2, d1, d2, nullptr, nullptr}, c.stream);
                return launch_lle_f32(L, d1, c.stream);
            };
            auto time_shape = [&](int code, float& best) -> cudaError_t {
                set_launch_shape(kind, sp.system, code);
                best = 1e30f;
                cudaError_t e = run();  // warm-up
                for (int rep = 0; rep < 3 && e == cudaSuccess; ++rep) {
                    cudaEventRecord(e0, c.stream);
                    e = run();
                    cudaEventRecord(e1, c.stream);
                    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
                    float ms = 0.f;
                    if (e == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
                    best = std::min(best, ms);
                }
                return e;
            };
            float msDefault = 0.f;
            err = time_shape(0, msDefault);
            int bestCode = 0;
            float bestMs = msDefault;
            for (int code : candidates(kind)) {
                if (err != cudaSuccess) break;
                float ms = 0.f;
                err = time_shape(code, ms);
                if (ms < bestMs * 0.99f) {  // a shape must beat the rule by 1 % to replace it
                    bestMs = ms;
                    bestCode = code;
                }
            }
            set_launch_shape(kind, sp.system, err == cudaSuccess ? bestCode : keep);
            if (table && row < nTable) {
                double* t = table + 6 * row++;
                t[0] = kind;
                t[1] = sp.system;
                t[2] = bestCode / 1024;
                t[3] = bestCode % 1024;
                t[4] = bestMs;
                t[5] = msDefault;
            }
        }
        if (rc) break;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return c.finish(rc);
    if (err != cudaSuccess) return c.finish(cuda_error(err, "autotune probe"));
    return c.finish(CHAOS_OK);
}
