// C-ABI layer: argument checks, device buffers from a stream-ordered pool,
// host<->device copies and kernel launches. Declared in include/chaos_gb300.h.
#include <cuda_runtime.h>

#include <atomic>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "../../include/chaos_gb300.h"
#include "capi_internal.h"
#include "dbscan.h"
#include "order_keys.h"
#include "launch.h"
#include "systems.h"

namespace chaos {

namespace {
thread_local std::string g_err;

struct DeviceCtx {
    bool ready = false;
    cudaStream_t stream = nullptr;
    cudaMemPool_t pool = nullptr;
    std::vector<cudaStream_t> aux;  // for concurrent branches of one call (batched groups)
};
std::mutex g_mu;
std::vector<DeviceCtx> g_dev;
std::atomic<long long> g_launches{0};
int env_flag(const char* name) {
    const char* s = getenv(name);
    return s && atoi(s) == 1 ? 1 : 0;
}
std::atomic<int> g_grid_fma{env_flag("CHAOS_GRID_FMA")};  // CHAOS_TUNE_GRID_FMA
// an environment value in [0, hi], else 0
int env_level(const char* name, int hi) {
    const char* s = getenv(name);
    const int v = s ? atoi(s) : 0;
    return v >= 0 && v <= hi ? v : 0;
}
std::atomic<int> g_lle_twin{env_level("CHAOS_LLE_TWIN", 2)};  // CHAOS_TUNE_LLE_TWIN
std::atomic<int> g_bif2d_cap{0};                          // CHAOS_TUNE_BIF2D_CAP
}  // namespace

void note_launch(long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
long long launch_count() { return g_launches.load(std::memory_order_relaxed); }

int set_error(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

int cuda_error(cudaError_t e, const char* what) {
    if (e == cudaErrorMemoryAllocation) return set_error(CHAOS_E_NOMEM, "%s: %s", what, cudaGetErrorString(e));
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver)
        return set_error(CHAOS_E_NODEV, "%s: %s", what, cudaGetErrorString(e));
    return set_error(CHAOS_E_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

// Per-device stream and memory pool, created on first use. The pool keeps
// freed blocks (release threshold = max) so repeated calls do not go back to
// the driver.
static int device_ctx(int dev, DeviceCtx** out) {
    std::lock_guard<std::mutex> lk(g_mu);
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count <= 0) return cuda_error(e == cudaSuccess ? cudaErrorNoDevice : e, "device count");
    if (dev < 0 || dev >= count) return set_error(CHAOS_E_ARGS, "device %d out of range (%d devices)", dev, count);
    if ((int)g_dev.size() < count) g_dev.resize(count);
    DeviceCtx& c = g_dev[dev];
    if (!c.ready) {
        if ((e = cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking)) != cudaSuccess)
            return cuda_error(e, "stream create");
        cudaMemPoolProps props;
        memset(&props, 0, sizeof props);
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        if ((e = cudaMemPoolCreate(&c.pool, &props)) != cudaSuccess) return cuda_error(e, "pool create");
        uint64_t thr = UINT64_MAX;
        cudaMemPoolSetAttribute(c.pool, cudaMemPoolAttrReleaseThreshold, &thr);
        c.ready = true;
    }
    *out = &c;
    return CHAOS_OK;
}

int aux_streams(int dev, std::vector<cudaStream_t>& out) {
    DeviceCtx* c = nullptr;
    int rc = device_ctx(dev, &c);
    if (rc) return rc;
    std::lock_guard<std::mutex> lk(g_mu);
    while (c->aux.size() < 8) {
        cudaStream_t s = nullptr;
        cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
        if (e != cudaSuccess) return cuda_error(e, "stream create");
        c->aux.push_back(s);
    }
    out = c->aux;
    return CHAOS_OK;
}

int Call::begin(const chaos_exec* e) {
    ex = e ? *e : chaos_exec{CHAOS_FP64, CHAOS_MEM_HOST, nullptr, -1};
    if (ex.precision != CHAOS_FP64 && ex.precision != CHAOS_FP32 && ex.precision != CHAOS_FF32)
        return set_error(CHAOS_E_ARGS, "precision must be CHAOS_FP64, CHAOS_FP32 or CHAOS_FF32");
    if (ex.memory != CHAOS_MEM_HOST && ex.memory != CHAOS_MEM_DEVICE)
        return set_error(CHAOS_E_ARGS, "memory must be CHAOS_MEM_HOST or CHAOS_MEM_DEVICE");
    cudaError_t err = cudaGetDevice(&prevDevice);
    if (err != cudaSuccess) return cuda_error(err, "get device");
    device = ex.device >= 0 ? ex.device : prevDevice;
    if (device != prevDevice && (err = cudaSetDevice(device)) != cudaSuccess) return cuda_error(err, "set device");
    DeviceCtx* c = nullptr;
    int rc = device_ctx(device, &c);
    if (rc) return rc;
    pool = c->pool;
    stream = ex.stream ? (cudaStream_t)ex.stream : c->stream;
    return CHAOS_OK;
}

void* Call::alloc(size_t bytes) {
    if (bytes == 0) bytes = 16;
    void* p = nullptr;
    cudaError_t e = cudaMallocFromPoolAsync(&p, bytes, pool, stream);
    if (e != cudaSuccess) {
        cuda_error(e, "device allocation");
        failed = true;
        return nullptr;
    }
    owned.push_back(p);
    return p;
}

int Call::finish(int rc) {
    for (void* p : owned) cudaFreeAsync(p, stream);
    owned.clear();
    if (rc == CHAOS_OK) {
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess && ex.memory == CHAOS_MEM_HOST) e = cudaStreamSynchronize(stream);
        if (e != cudaSuccess) rc = cuda_error(e, "execution");
    }
    if (device != prevDevice) cudaSetDevice(prevDevice);
    return rc;
}

int Call::to_host(void* host, const void* dev, size_t bytes) {
    if (ex.memory != CHAOS_MEM_HOST || !host || bytes == 0) return CHAOS_OK;
    cudaError_t e = cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, stream);
    return e == cudaSuccess ? CHAOS_OK : cuda_error(e, "copy to host");
}

const void* Call::input(const void* user, size_t bytes) {
    if (!user) return nullptr;
    if (ex.memory == CHAOS_MEM_DEVICE) return user;
    void* d = alloc(bytes);
    if (!d) return nullptr;
    cudaError_t e = cudaMemcpyAsync(d, user, bytes, cudaMemcpyHostToDevice, stream);
    if (e != cudaSuccess) {
        cuda_error(e, "copy to device");
        failed = true;
        return nullptr;
    }
    return d;
}

void* Call::output(void* user, size_t bytes) {
    if (!user) return nullptr;
    if (ex.memory == CHAOS_MEM_DEVICE) return user;
    return alloc(bytes);
}

// ---------------------------------------------------------------------------
// argument checks shared by the sweeps

static void sizes_of(int system, int* nx, int* na) {
    if (system == SYS_USER) {
        user_system_sizes(nx, na);
    } else {
        *nx = system_nx(system);
        *na = system_na(system);
    }
}

static int check_system(int system, int nIC, int nValues) {
    if (system == SYS_USER && !user_system_available())
        return set_error(CHAOS_E_UNSUPPORTED, "the library was built without a user plug-in (CHAOS_USER_SYSTEMS at build time)");
    if (!system_supported(system)) return set_error(CHAOS_E_ARGS, "unknown system %d", system);
    int nx, na;
    sizes_of(system, &nx, &na);
    if (nx > kMaxState || na > kMaxParams)
        return set_error(CHAOS_E_UNSUPPORTED, "plug-in sizes %d/%d exceed %d/%d", nx, na, kMaxState, kMaxParams);
    if (nIC != nx)
        return set_error(CHAOS_E_ARGS, "amountOfInitialConditions %d != SIZE_X %d of system %d", nIC, nx, system);
    if (nValues != na)
        return set_error(CHAOS_E_ARGS, "amountOfValues %d != SIZE_A %d of system %d", nValues, na, system);
    return CHAOS_OK;
}

// CHAOS_FF32 is implemented for the LLE maps and trajectories of the RK4
// systems; the other sweeps refuse it instead of running another precision.
static int no_ff32(const chaos_exec* ex, const char* what) {
    if (ex && ex->precision == CHAOS_FF32)
        return set_error(CHAOS_E_UNSUPPORTED, "CHAOS_FF32 runs the LLE maps (chaos_lle2d, chaos_lle_sweep) and "
                                              "chaos_trajectory of the RK4 systems; %s takes CHAOS_FP64 or CHAOS_FP32",
                         what);
    return CHAOS_OK;
}
// CHAOS_FF32 LLE: the RK4 systems (the twin as an exact difference) with the twin at x + eps e_x.
static int check_ff32_lle(const chaos_exec* ex, int system, const LleParams& L) {
    if (!ex || ex->precision != CHAOS_FF32) return CHAOS_OK;
    if (system == SYS_USER || !system_has_difference_form(system))
        return set_error(CHAOS_E_UNSUPPORTED, "CHAOS_FF32 LLE needs an RK4 system (0-2); use CHAOS_FP64");
    if (L.twin != 0) return set_error(CHAOS_E_UNSUPPORTED, "the reference twin starts (CHAOS_TUNE_LLE_TWIN 1, 2) are FP64 only");
    return CHAOS_OK;
}

// precision / plug-in dispatch of the sweep kernels
// The legacy per-point loop runs in FP64, the legacy library's arithmetic.
static cudaError_t run_bif(int prec, const SweepParams& P, const BifOut& O, cudaStream_t st) {
    if (P.legacyLoop) prec = CHAOS_FP64;
    if (P.system == SYS_USER) return prec == CHAOS_FP32 ? cudaErrorNotSupported : launch_bif_user(P, O, st);
    return prec == CHAOS_FP32 ? launch_bif_f32(P, O, st) : launch_bif_f64(P, O, st);
}
static cudaError_t run_bif_list(int prec, const SweepParams& P, const BifOut& O, const int* list, int count,
                                cudaStream_t st) {
    if (P.legacyLoop) prec = CHAOS_FP64;
    return prec == CHAOS_FP32 ? launch_bif_list_f32(P, O, list, count, st) : launch_bif_list_f64(P, O, list, count, st);
}
static cudaError_t run_basins(int prec, const SweepParams& P, const BasinsOut& O, cudaStream_t st) {
    if (P.system == SYS_USER) return prec == CHAOS_FP32 ? cudaErrorNotSupported : launch_basins_user(P, O, st);
    return prec == CHAOS_FP32 ? launch_basins_f32(P, O, st) : launch_basins_f64(P, O, st);
}
static cudaError_t run_lle(int prec, const LleParams& L, double* out, cudaStream_t st) {
    if (L.legacyLoop) prec = CHAOS_FP64;  // the legacy kernels' arithmetic
    if (L.system == SYS_USER) return prec != CHAOS_FP64 ? cudaErrorNotSupported : launch_lle_user(L, out, st);
    if (prec == CHAOS_FF32) return launch_lle_ff(L, out, st);
    return prec == CHAOS_FP32 ? launch_lle_f32(L, out, st) : launch_lle_f64(L, out, st);
}

// Values of a log-scale axis: the legacy getValueByIdxLog exponent
// log10(r0) + n*((log10(r1) - log10(r0)) / (nPts - 1)) (debri/cudaLibrary.cu:1191-1196),
// then 10^x in FP64, or (double)powf(10, (float)x) as the legacy step-size
// sweep rounds it (debri/cudaLibrary.cu:1001).
void log_axis_values(double r0, double r1, int nPts, bool f32, std::vector<double>& out) {
    out.resize(nPts);
    const double l0 = std::log10(r0);
    const double step = (std::log10(r1) - l0) / (double)(nPts - 1);
    for (int n = 0; n < nPts; ++n) {
        const double x = l0 + (double)n * step;
        out[n] = f32 ? (double)powf(10.0f, (float)x) : std::pow(10.0, x);
    }
}

// Checks a grid mode against the ranges: log-scale axes need positive ends and nPts >= 2.
static int check_grid_mode(int gridMode, int dim, int nPts, const double* ranges) {
    if (gridMode & ~(CHAOS_GRID_STATE | CHAOS_GRID_LOG0 | CHAOS_GRID_LOG1 | CHAOS_GRID_LOG_F32 | CHAOS_GRID_LEGACY_LOOP))
        return set_error(CHAOS_E_ARGS, "unknown grid mode bits 0x%x", gridMode);
    if ((gridMode & CHAOS_GRID_LOG1) && dim < 2) return set_error(CHAOS_E_ARGS, "CHAOS_GRID_LOG1 needs dim 2");
    for (int d = 0; d < dim; ++d) {
        if (!(gridMode & (d ? CHAOS_GRID_LOG1 : CHAOS_GRID_LOG0))) continue;
        if (nPts < 2) return set_error(CHAOS_E_ARGS, "a log-scale axis needs nPts >= 2");
        if (!(ranges[2 * d] > 0) || !(ranges[2 * d + 1] > 0) || std::isinf(ranges[2 * d]) ||
            std::isinf(ranges[2 * d + 1]))
            return set_error(CHAOS_E_ARGS, "a log-scale axis needs finite positive ranges");
    }
    return CHAOS_OK;
}

// Uploads the log-scale axes of a grid mode to scratch of the call; table[d]
// receives the device array (untouched for linear axes).
static int upload_log_axes(Call& c, int gridMode, int dim, int nPts, const double* ranges, const double** table) {
    for (int d = 0; d < dim; ++d) {
        if (!(gridMode & (d ? CHAOS_GRID_LOG1 : CHAOS_GRID_LOG0))) continue;
        std::vector<double> v;
        try {
            log_axis_values(ranges[2 * d], ranges[2 * d + 1], nPts, (gridMode & CHAOS_GRID_LOG_F32) != 0, v);
        } catch (const std::bad_alloc&) {
            return set_error(CHAOS_E_NOMEM, "host allocation of a log-scale axis failed");
        }
        double* dv = (double*)c.alloc(v.size() * sizeof(double));
        if (c.failed) return CHAOS_E_NOMEM;
        cudaError_t e = cudaMemcpyAsync(dv, v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice, c.stream);
        // (a copy from pageable memory has read v when it returns)
        if (e != cudaSuccess) return cuda_error(e, "grid table upload");
        table[d] = dv;
    }
    return CHAOS_OK;
}

// With CHAOS_TUNE_GRID_FMA, the linear axes of an LLE grid take start + i*step
// fused into one FMA. The reference's host linspace (LLE/src/LLECUDA.cu:195-200)
// computes them that way where its host compiler contracts the expression
// (aarch64 by default). They are uploaded as value tables, like the log-scale
// axes, so the kernels are unchanged.
static int upload_fused_axes(Call& c, int gridMode, int dim, int nPts, const double* ranges, const double** table) {
    if (!g_grid_fma.load(std::memory_order_relaxed) || nPts < 2) return CHAOS_OK;
    for (int d = 0; d < dim; ++d) {
        if (gridMode & (d ? CHAOS_GRID_LOG1 : CHAOS_GRID_LOG0)) continue;
        std::vector<double> v;
        try {
            v.resize(nPts);
        } catch (const std::bad_alloc&) {
            return set_error(CHAOS_E_NOMEM, "host allocation of a grid axis failed");
        }
        const double step = (ranges[2 * d + 1] - ranges[2 * d]) / (double)(nPts - 1);
        for (int i = 0; i < nPts; ++i) v[i] = std::fma((double)i, step, ranges[2 * d]);
        double* dv = (double*)c.alloc(v.size() * sizeof(double));
        if (c.failed) return CHAOS_E_NOMEM;
        cudaError_t e = cudaMemcpyAsync(dv, v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice, c.stream);
        // (a copy from pageable memory has read v when it returns)
        if (e != cudaSuccess) return cuda_error(e, "grid table upload");
        table[d] = dv;
    }
    return CHAOS_OK;
}

int fill_sweep(SweepParams& P, int system, int dim, double tMax, int nPts, double h, int nIC, const double* ic,
               const double* ranges, const int* mut, int wv, double maxValue, double transientTime,
               const double* values, int nValues, int preScaller, bool basins, int gridMode) {
    int rc = check_system(system, nIC, nValues);
    if (rc) return rc;
    if (!ic || !ranges || !mut || !values) return set_error(CHAOS_E_ARGS, "null parameter array");
    const bool state = basins || (gridMode & CHAOS_GRID_STATE);
    const bool stepAxis = (gridMode & kGridStepAxis) && mut[0] == CHAOS_MUT_STEP;
    if (stepAxis) {  // the step sweeps dimension 0; the caller's h is not used
        if (dim != 1 || basins) return set_error(CHAOS_E_ARGS, "the step-size sweep is a 1-D bifurcation");
        if (!(ranges[0] > 0) || !(ranges[1] > 0) || std::isinf(ranges[0]) || std::isinf(ranges[1]))
            return set_error(CHAOS_E_ARGS, "the step-size range must be finite and positive");
        h = std::min(ranges[0], ranges[1]) * (1.0 - 1e-9);  // below every step on the axis: bounds the step counts
    }
    if (!(h > 0) || !(tMax > 0) || !(transientTime >= 0)) return set_error(CHAOS_E_ARGS, "need h > 0, tMax > 0, transientTime >= 0");
    if (nPts < 2) return set_error(CHAOS_E_ARGS, "nPts must be >= 2");
    if (preScaller < 1) return set_error(CHAOS_E_ARGS, "preScaller must be >= 1");
    if (wv < 0 || wv >= nIC) return set_error(CHAOS_E_ARGS, "writableVar %d out of range", wv);
    if ((rc = check_grid_mode(gridMode & ~kGridStepAxis, dim, nPts, ranges))) return rc;
    const int lim = state ? nIC : nValues;
    for (int d = stepAxis ? 1 : 0; d < dim; ++d)
        if (mut[d] < 0 || mut[d] >= lim) return set_error(CHAOS_E_ARGS, "indicesOfMutVars[%d] = %d out of range", d, mut[d]);
    const double Bd = tMax / h / preScaller, Sd = transientTime / h;
    if (!(Bd >= 1) || Bd > 2.0e9 || Sd > 2.0e9) return set_error(CHAOS_E_ARGS, "tMax/h/preScaller must be in [1, 2e9]");
    memset(&P, 0, sizeof P);
    P.system = system;
    P.dim = dim;
    P.B = (int)Bd;
    P.S = (int)Sd;
    P.preScaller = basins ? preScaller : 1;
    P.wv = wv;
    P.checkMax = maxValue != 0;
    P.mutateState = state ? 1 : 0;
    P.h = h;
    P.hInterval = h * (double)preScaller;
    P.maxValue = maxValue;
    P.maxValueF = (float)maxValue;
    if ((double)P.maxValueF > maxValue) P.maxValueF = nextafterf(P.maxValueF, -INFINITY);
    // For a double v, float(v) (round to nearest, ties to even) exceeds maxValueF
    // exactly when |v| is above the midpoint m of maxValueF and the next float
    // up (or at m, when that next float is the even one, or infinity).
    if (!(maxValue == maxValue) || maxValue == INFINITY) {
        P.maxBits = ~0ull;  // never
        P.maxTie = 0;
    } else if (maxValue < 0) {
        P.maxBits = 0;  // always (|float(v)| >= 0 > maxValue)
        P.maxTie = 1;
    } else {
        const float up = nextafterf(P.maxValueF, INFINITY);
        const double m = up == INFINITY ? 340282356779733661637539395458142568448.0  // 2^128 - 2^103
                                        : ((double)P.maxValueF + (double)up) * 0.5;
        uint32_t upBits;
        memcpy(&upBits, &up, sizeof upBits);
        memcpy(&P.maxBits, &m, sizeof P.maxBits);
        P.maxTie = (up == INFINITY || (upBits & 1u) == 0) ? 1 : 0;
    }
    for (int i = 0; i < nIC; ++i) P.ic[i] = ic[i];
    for (int i = 0; i < nValues; ++i) P.values[i] = values[i];
    P.mut[0] = mut[0];
    P.mut[1] = dim > 1 ? mut[1] : -1;
    P.grid.nPts = nPts;
    P.grid.fused = g_grid_fma.load(std::memory_order_relaxed);
    for (int d = 0; d < dim; ++d) {
        P.grid.start[d] = ranges[2 * d];
        P.grid.scale[d] = (ranges[2 * d + 1] - ranges[2 * d]) / (double)(nPts - 1);
    }
    P.pBegin = 0;
    P.nPoints = dim == 1 ? (long long)nPts : (long long)nPts * nPts;
    P.sweepStep = stepAxis ? 1 : 0;
    P.bPre = preScaller;
    P.tMax = tMax;
    P.transientTime = transientTime;
    if (gridMode & CHAOS_GRID_LEGACY_LOOP) {
        if (basins) return set_error(CHAOS_E_ARGS, "CHAOS_GRID_LEGACY_LOOP belongs to the bifurcation sweep");
        P.legacyLoop = stepAxis ? 2 : 1;
    }
    return CHAOS_OK;
}

int fill_lle(LleParams& L, int system, double tMax, double NT, int nPts, double h, double eps,
             const double* initialConditions, int amountOfInitialConditions, const double* ranges,
             const int* indicesOfMutVars, double transientTime, const double* values, int amountOfValues, int dim,
             int gridMode) {
    const int mutateState = gridMode & CHAOS_GRID_STATE;
    if (gridMode & CHAOS_GRID_LEGACY_LOOP)
        return set_error(CHAOS_E_ARGS, "CHAOS_GRID_LEGACY_LOOP belongs to the bifurcation sweep");
    int rc = check_system(system, amountOfInitialConditions, amountOfValues);
    if (rc) return rc;
    if (!initialConditions || !ranges || !indicesOfMutVars || !values) return set_error(CHAOS_E_ARGS, "null argument");
    if (nPts < 1) return set_error(CHAOS_E_ARGS, "nPts must be >= 1");
    if (!(h > 0) || !(tMax > 0) || !(NT > 0) || !(transientTime >= 0) || !(eps > 0))
        return set_error(CHAOS_E_ARGS, "need h, tMax, NT, eps > 0 and transientTime >= 0");
    if (dim != 1 && dim != 2) return set_error(CHAOS_E_ARGS, "dim must be 1 or 2");
    if ((rc = check_grid_mode(gridMode, dim, nPts, ranges))) return rc;
    const int lim = mutateState ? amountOfInitialConditions : amountOfValues;
    for (int d = 0; d < dim; ++d)
        if (indicesOfMutVars[d] < 0 || indicesOfMutVars[d] >= lim)
            return set_error(CHAOS_E_ARGS, "indicesOfMutVars[%d] out of range", d);
    if (dim == 2 && (double)nPts * nPts > 2.0e9) return set_error(CHAOS_E_ARGS, "nPts^2 must be < 2e9");
    if (NT / h > 2.0e9 || tMax / h > 2.0e9 || transientTime / h > 2.0e9)
        return set_error(CHAOS_E_ARGS, "step counts must fit in int");
    memset(&L, 0, sizeof L);
    L.system = system;
    L.nPts = nPts;
    L.ntp = static_cast<int>(NT / h);
    L.trans = static_cast<int>(transientTime / h);
    const int all = static_cast<int>(tMax / h);
    if (L.ntp < 1) return set_error(CHAOS_E_ARGS, "NT / h must be >= 1");
    L.calcBlocks = all / L.ntp + 1;
    L.h = h;
    L.eps = eps;
    L.tMax = tMax;
    for (int i = 0; i < amountOfInitialConditions; ++i) L.ic[i] = initialConditions[i];
    for (int i = 0; i < amountOfValues; ++i) L.values[i] = values[i];
    L.mut[0] = indicesOfMutVars[0];
    L.mut[1] = dim == 2 ? indicesOfMutVars[1] : -1;
    L.rangeA[0] = ranges[0];
    L.rangeA[1] = ranges[1];
    L.rangeB[0] = dim == 2 ? ranges[2] : 0.0;
    L.rangeB[1] = dim == 2 ? ranges[3] : 0.0;
    L.stepA = nPts > 1 ? (ranges[1] - ranges[0]) / (nPts - 1) : 0.0;
    L.stepB = nPts > 1 && dim == 2 ? (ranges[3] - ranges[2]) / (nPts - 1) : 0.0;
    L.pBegin = 0;
    L.nPoints = dim == 2 ? (long long)nPts * nPts : nPts;
    L.twin = g_lle_twin.load(std::memory_order_relaxed);
    L.dim = dim;
    L.mutateState = mutateState ? 1 : 0;
    return CHAOS_OK;
}

size_t scratch_budget_bytes() {
    const char* s = getenv("CHAOS_SCRATCH_BUDGET_MB");
    size_t mb = s ? (size_t)strtoull(s, nullptr, 10) : 8192;
    return std::max<size_t>(mb, 1) << 20;
}

}  // namespace chaos

using namespace chaos;

extern "C" {

int chaos_abi_version(void) { return CHAOS_ABI_VERSION; }
const char* chaos_last_error(void) { return g_err.c_str(); }

int chaos_launch_count(long long* count) {
    if (!count) return set_error(CHAOS_E_ARGS, "null count");
    *count = launch_count();
    return CHAOS_OK;
}

int chaos_system_info(int system, int* sizeX, int* sizeA) {
    if (system == SYS_USER && !user_system_available())
        return set_error(CHAOS_E_UNSUPPORTED, "the library was built without a user plug-in");
    if (!system_supported(system)) return set_error(CHAOS_E_ARGS, "unknown system %d", system);
    int nx, na;
    sizes_of(system, &nx, &na);
    if (sizeX) *sizeX = nx;
    if (sizeA) *sizeA = na;
    return CHAOS_OK;
}

int chaos_synchronize(const chaos_exec* ex) {
    Call c;
    int rc = c.begin(ex);
    if (rc) return rc;
    cudaError_t e = cudaStreamSynchronize(c.stream);
    rc = e == cudaSuccess ? CHAOS_OK : cuda_error(e, "synchronize");
    return c.finish(rc);
}

}  // extern "C"

// The 1-D bifurcation of a filled parameter block (log-scale axes of gridMode
// uploaded here).
static int bif1d_run(const chaos_exec* ex, SweepParams P, int gridMode, const double* ranges, int peakCapacity,
                     int* counts, int* flags, double* firstSample, double* peaks, double* intervals) {
    int rc = CHAOS_OK;
    if (!counts || !flags) return set_error(CHAOS_E_ARGS, "counts and flags are required");
    if (peakCapacity < 0 || ((peaks || intervals) && peakCapacity == 0))
        return set_error(CHAOS_E_ARGS, "peakCapacity must be > 0 when peaks or intervals are requested");
    if (!P.legacyLoop && (rc = no_ff32(ex, "the bifurcation sweep"))) return rc;
    Call c;
    if ((rc = c.begin(ex))) return rc;
    if ((rc = upload_log_axes(c, gridMode, P.dim, (int)P.grid.nPts, ranges, P.grid.table))) return c.finish(rc);
    const long long n = P.nPoints;
    const size_t rowBytes = (size_t)n * peakCapacity * sizeof(double);
    BifOut O;
    O.cap = peakCapacity;
    O.counts = (int*)c.output(counts, n * sizeof(int));
    O.flags = (int*)c.output(flags, n * sizeof(int));
    O.first = (double*)c.output(firstSample, n * sizeof(double));
    O.peaks = (double*)c.output(peaks, rowBytes);
    O.intervals = (double*)c.output(intervals, rowBytes);
    if (c.failed) return c.finish(CHAOS_E_NOMEM);
    cudaError_t e = run_bif(c.ex.precision, P, O, c.stream);
    if (e != cudaSuccess) return c.finish(cuda_error(e, "bifurcation kernel"));
    rc = c.to_host(counts, O.counts, n * sizeof(int));
    if (!rc) rc = c.to_host(flags, O.flags, n * sizeof(int));
    if (!rc) rc = c.to_host(firstSample, O.first, n * sizeof(double));
    if (!rc) rc = c.to_host(peaks, O.peaks, rowBytes);
    if (!rc) rc = c.to_host(intervals, O.intervals, rowBytes);
    return c.finish(rc);
}

// The 2-D bifurcation with per-point clustering of a filled parameter block.
static int bif2d_run(const chaos_exec* ex, SweepParams P, int gridMode, const double* ranges, double eps,
                     int* labels, int* counts) {
    int rc = CHAOS_OK;
    if (!labels) return set_error(CHAOS_E_ARGS, "labels is required");
    if (!P.legacyLoop && (rc = no_ff32(ex, "the bifurcation sweep"))) return rc;
    Call c;
    if ((rc = c.begin(ex))) return rc;
    if ((rc = upload_log_axes(c, gridMode, P.dim, (int)P.grid.nPts, ranges, P.grid.table))) return c.finish(rc);
    const long long n = P.nPoints;
    // every detected peak sits at least two samples after the previous one,
    // so B/2 rows hold all kept intervals of a point
    const int capFull = std::max(P.B / 2, 1);
    // Peak-buffer capacity. B/2 rows when the whole grid fits the scratch
    // budget with them; else as many rows as let the grid run as one chunk,
    // when that is at least 512; else the kept-peak counts of up to 4096
    // evenly spread points, 25 % + 16 above their maximum (a probe whose cost
    // is one full trajectory). CHAOS_TUNE_BIF2D_CAP: > 0 a fixed capacity, -1
    // always B/2. Points with more peaks than the capacity are run again with
    // B/2 rows, so the capacity changes memory and speed, never results.
    int cap = capFull;
    const int capKnob = g_bif2d_cap.load(std::memory_order_relaxed);
    const bool adapt = capKnob >= 0 && P.system != SYS_USER && n <= 0x7fffffffLL && capFull > 64;
    const long long capBudget = (long long)(scratch_budget_bytes() / ((size_t)n * (sizeof(double) + 2 * sizeof(int))));
    if (adapt && capKnob > 0) {
        cap = std::min(capKnob, capFull);
    } else if (adapt && capBudget >= 512) {
        cap = (int)std::min<long long>(capFull, capBudget);
    } else if (adapt) {
        const int S = (int)std::min<long long>(n, 4096);
        std::vector<int> idx(S), hc(S);
        for (int s = 0; s < S; ++s) idx[s] = (int)(n * s / S);
        int* dIdx = (int*)c.alloc(S * sizeof(int));
        int* dPc = (int*)c.alloc(S * sizeof(int));
        int* dPf = (int*)c.alloc(S * sizeof(int));
        if (c.failed) return c.finish(CHAOS_E_NOMEM);
        cudaError_t e = cudaMemcpyAsync(dIdx, idx.data(), S * sizeof(int), cudaMemcpyHostToDevice, c.stream);
        BifOut Op{dPc, dPf, nullptr, nullptr, nullptr, 0};
        if (e == cudaSuccess) e = run_bif_list(c.ex.precision, P, Op, dIdx, S, c.stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(hc.data(), dPc, S * sizeof(int), cudaMemcpyDeviceToHost, c.stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
        if (e != cudaSuccess) return c.finish(cuda_error(e, "bifurcation 2-D capacity probe"));
        const int mx = std::max(0, *std::max_element(hc.begin(), hc.end()));
        cap = (int)std::min<long long>(capFull, (long long)mx + mx / 4 + 16);
    }
    const size_t perPoint = (size_t)cap * (sizeof(double) + 2 * sizeof(int));
    long long chunk = (long long)std::max<size_t>(scratch_budget_bytes() / perPoint, 1);
    chunk = std::min(chunk, n);
    int* dLabels = (int*)c.output(labels, n * sizeof(int));
    int* dCounts = counts ? (int*)c.output(counts, n * sizeof(int)) : (int*)c.alloc(n * sizeof(int));
    int* dFlags = (int*)c.alloc(chunk * sizeof(int));
    double* dIv = (double*)c.alloc((size_t)chunk * cap * sizeof(double));
    int* dLab = (int*)c.alloc((size_t)chunk * cap * sizeof(int));
    int* dSlot = (int*)c.alloc((size_t)chunk * cap * sizeof(int));
    if (c.failed) return c.finish(CHAOS_E_NOMEM);
    for (long long b = 0; b < n; b += chunk) {
        SweepParams Q = P;
        Q.pBegin = b;
        Q.nPoints = std::min(chunk, n - b);
        BifOut O{dCounts + b, dFlags, nullptr, nullptr, dIv, cap};
        cudaError_t e = run_bif(c.ex.precision, Q, O, c.stream);
        if (e == cudaSuccess)
            e = launch_point_dbscan(dIv, dCounts + b, Q.nPoints, cap, eps, dLab, dSlot, dLabels + b, c.stream);
        if (e != cudaSuccess) return c.finish(cuda_error(e, "bifurcation 2-D kernels"));
    }
    if (cap < capFull) {  // the points with more kept peaks than the capacity, again with B/2 rows
        int* dList = (int*)c.alloc(n * sizeof(int));
        int* dNum = (int*)c.alloc(sizeof(int));
        if (c.failed) return c.finish(CHAOS_E_NOMEM);
        int hNum = 0;
        cudaError_t e = cudaMemsetAsync(dNum, 0, sizeof(int), c.stream);
        if (e == cudaSuccess) e = launch_overflow_select(dCounts, n, cap, dList, dNum, c.stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&hNum, dNum, sizeof(int), cudaMemcpyDeviceToHost, c.stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
        if (e != cudaSuccess) return c.finish(cuda_error(e, "bifurcation 2-D overflow selection"));
        if (hNum > 0) {
            const size_t perFull = (size_t)capFull * (sizeof(double) + 2 * sizeof(int)) + 2 * sizeof(int);
            const int chunk2 = (int)std::min<long long>(hNum, std::max<size_t>(scratch_budget_bytes() / perFull, 1));
            int* rCounts = (int*)c.alloc(chunk2 * sizeof(int));
            int* rFlags = (int*)c.alloc(chunk2 * sizeof(int));
            double* rIv = (double*)c.alloc((size_t)chunk2 * capFull * sizeof(double));
            int* rLab = (int*)c.alloc((size_t)chunk2 * capFull * sizeof(int));
            int* rSlot = (int*)c.alloc((size_t)chunk2 * capFull * sizeof(int));
            if (c.failed) return c.finish(CHAOS_E_NOMEM);
            for (int b = 0; b < hNum && e == cudaSuccess; b += chunk2) {
                const int m = std::min(chunk2, hNum - b);
                BifOut Or{rCounts, rFlags, nullptr, nullptr, rIv, capFull};
                e = run_bif_list(c.ex.precision, P, Or, dList + b, m, c.stream);
                if (e == cudaSuccess)
                    e = launch_point_dbscan(rIv, rCounts, m, capFull, eps, rLab, rSlot, dLabels, c.stream, dList + b);
            }
            if (e != cudaSuccess) return c.finish(cuda_error(e, "bifurcation 2-D overflow pass"));
        }
    }
    rc = c.to_host(labels, dLabels, n * sizeof(int));
    if (!rc && counts) rc = c.to_host(counts, dCounts, n * sizeof(int));
    return c.finish(rc);
}

extern "C" {

int chaos_bifurcation1d(const chaos_exec* ex, int system, double tMax, int nPts, double h,
                        int amountOfInitialConditions, const double* initialConditions, const double* ranges,
                        const int* indicesOfMutVars, int writableVar, double maxValue, double transientTime,
                        const double* values, int amountOfValues, int preScaller, int peakCapacity, int* counts,
                        int* flags, double* firstSample, double* peaks, double* intervals) {
    SweepParams P;
    int rc = fill_sweep(P, system, 1, tMax, nPts, h, amountOfInitialConditions, initialConditions, ranges,
                        indicesOfMutVars, writableVar, maxValue, transientTime, values, amountOfValues, preScaller,
                        false);
    if (rc) return rc;
    return bif1d_run(ex, P, 0, ranges, peakCapacity, counts, flags, firstSample, peaks, intervals);
}

int chaos_bifurcation2d(const chaos_exec* ex, int system, double tMax, int nPts, double h,
                        int amountOfInitialConditions, const double* initialConditions, const double* ranges,
                        const int* indicesOfMutVars, int writableVar, double maxValue, double transientTime,
                        const double* values, int amountOfValues, int preScaller, double eps, int* labels,
                        int* counts) {
    SweepParams P;
    int rc = fill_sweep(P, system, 2, tMax, nPts, h, amountOfInitialConditions, initialConditions, ranges,
                        indicesOfMutVars, writableVar, maxValue, transientTime, values, amountOfValues, preScaller,
                        false);
    if (rc) return rc;
    return bif2d_run(ex, P, 0, ranges, eps, labels, counts);
}

int chaos_bifurcation_sweep(const chaos_exec* ex, int system, int dim, int gridMode, double tMax, int nPts,
                            double h, int amountOfInitialConditions, const double* initialConditions,
                            const double* ranges, const int* indicesOfMutVars, int writableVar, double maxValue,
                            double transientTime, const double* values, int amountOfValues, int preScaller,
                            double eps, int peakCapacity, int* counts, int* flags, double* firstSample,
                            double* peaks, double* intervals, int* labels) {
    if (dim != 1 && dim != 2) return set_error(CHAOS_E_ARGS, "dim must be 1 or 2");
    if (gridMode & kGridStepAxis) return set_error(CHAOS_E_ARGS, "unknown grid mode bits 0x%x", gridMode);
    SweepParams P;
    int rc = fill_sweep(P, system, dim, tMax, nPts, h, amountOfInitialConditions, initialConditions, ranges,
                        indicesOfMutVars, writableVar, maxValue, transientTime, values, amountOfValues, preScaller,
                        false, gridMode | kGridStepAxis);
    if (rc) return rc;
    if (dim == 1) {
        if (labels) return set_error(CHAOS_E_ARGS, "labels belong to the 2-D sweep");
        return bif1d_run(ex, P, gridMode, ranges, peakCapacity, counts, flags, firstSample, peaks, intervals);
    }
    if (flags || firstSample || peaks || intervals || peakCapacity)
        return set_error(CHAOS_E_ARGS, "the 2-D sweep returns labels and counts only");
    return bif2d_run(ex, P, gridMode, ranges, eps, labels, counts);
}

int chaos_lle2d(const chaos_exec* ex, int system, double tMax, double NT, int nPts, double h, double eps,
                const double* initialConditions, int amountOfInitialConditions, const double* ranges,
                const int* indicesOfMutVars, int writableVar, double maxValue, double transientTime,
                const double* values, int amountOfValues, double* lle) {
    (void)writableVar;
    (void)maxValue;
    int rc = CHAOS_OK;
    if (!lle) return set_error(CHAOS_E_ARGS, "null argument");
    LleParams L;
    if ((rc = fill_lle(L, system, tMax, NT, nPts, h, eps, initialConditions, amountOfInitialConditions, ranges,
                       indicesOfMutVars, transientTime, values, amountOfValues)))
        return rc;
    if (ex && ex->precision == CHAOS_FP32 && (system == SYS_USER || !system_has_fp32_lle(system)))
        return set_error(CHAOS_E_UNSUPPORTED, "FP32 LLE needs a quadratic RK4 system (0-2) or Chameleon; use CHAOS_FP64");
    if (ex && ex->precision == CHAOS_FP32 && L.twin != 0)
        return set_error(CHAOS_E_UNSUPPORTED, "the reference twin starts (CHAOS_TUNE_LLE_TWIN 1, 2) are FP64 only");
    if ((rc = check_ff32_lle(ex, system, L))) return rc;
    Call c;
    if ((rc = c.begin(ex))) return rc;
    if ((rc = upload_fused_axes(c, 0, 2, nPts, ranges, L.table))) return c.finish(rc);
    double* dOut = (double*)c.output(lle, L.nPoints * sizeof(double));
    if (c.failed) return c.finish(CHAOS_E_NOMEM);
    cudaError_t e = run_lle(c.ex.precision, L, dOut, c.stream);
    if (e != cudaSuccess) return c.finish(cuda_error(e, "LLE kernel"));
    rc = c.to_host(lle, dOut, L.nPoints * sizeof(double));
    return c.finish(rc);
}

// The legacy LLE kernels' scheme (legacy_lle.cuh), FP64: the LLE (spectrum
// false, out[p]) or the spectrum (out[p*SIZE_X + j]). draws: the raw twin
// draws (SIZE_X per point, SIZE_X^2 for the spectrum), host or device memory, or null.
static int run_legacy_scheme(const chaos_exec* ex, bool spectrum, int system, int dim, int gridMode, double tMax,
                             double NT, int nPts, double h, double eps, const double* initialConditions,
                             int amountOfInitialConditions, const double* ranges, const int* indicesOfMutVars,
                             double maxValue, double transientTime, const double* values, int amountOfValues,
                             const double* draws, double* out) {
    int rc = CHAOS_OK;
    if (!out) return set_error(CHAOS_E_ARGS, "null argument");
    LleParams L;
    if ((rc = fill_lle(L, system, tMax, NT, nPts, h, eps, initialConditions, amountOfInitialConditions, ranges,
                       indicesOfMutVars, transientTime, values, amountOfValues, dim, gridMode)))
        return rc;
    L.legacyLoop = 1;
    L.legacyBlocks = (int)(tMax / NT);  // <= tMax / h, which fill_lle bounds
    L.maxValue = maxValue;
    L.twin = 0;
    const int nx = amountOfInitialConditions;
    Call c;
    if ((rc = c.begin(ex))) return rc;
    if ((rc = upload_log_axes(c, gridMode, dim, nPts, ranges, L.table))) return c.finish(rc);
    if (draws) {
        const size_t bytes = (size_t)L.nPoints * nx * (spectrum ? nx : 1) * sizeof(double);
        double* dDraws = (double*)c.alloc(bytes);
        if (c.failed) return c.finish(CHAOS_E_NOMEM);
        cudaError_t e = cudaMemcpyAsync(dDraws, draws, bytes, cudaMemcpyDefault, c.stream);
        if (e != cudaSuccess) return c.finish(cuda_error(e, "twin draws upload"));
        L.draws = dDraws;
    }
    const size_t outBytes = (size_t)L.nPoints * (spectrum ? nx : 1) * sizeof(double);
    double* dOut = (double*)c.output(out, outBytes);
    if (c.failed) return c.finish(CHAOS_E_NOMEM);
    cudaError_t e = spectrum ? launch_spectrum_f64(L, dOut, c.stream) : run_lle(CHAOS_FP64, L, dOut, c.stream);
    if (e != cudaSuccess) return c.finish(cuda_error(e, "legacy LLE kernel"));
    rc = c.to_host(out, dOut, outBytes);
    return c.finish(rc);
}

int chaos_lle_sweep(const chaos_exec* ex, int system, int dim, int gridMode, double tMax, double NT, int nPts,
                    double h, double eps, const double* initialConditions, int amountOfInitialConditions,
                    const double* ranges, const int* indicesOfMutVars, double transientTime, const double* values,
                    int amountOfValues, double* lle) {
    int rc = CHAOS_OK;
    if (!lle) return set_error(CHAOS_E_ARGS, "null argument");
    LleParams L;
    if ((rc = fill_lle(L, system, tMax, NT, nPts, h, eps, initialConditions, amountOfInitialConditions, ranges,
                       indicesOfMutVars, transientTime, values, amountOfValues, dim, gridMode)))
        return rc;
    if (ex && ex->precision == CHAOS_FP32 && (system == SYS_USER || !system_has_fp32_lle(system)))
        return set_error(CHAOS_E_UNSUPPORTED, "FP32 LLE needs a quadratic RK4 system (0-2) or Chameleon; use CHAOS_FP64");
    if (ex && ex->precision == CHAOS_FP32 && L.twin != 0)
        return set_error(CHAOS_E_UNSUPPORTED, "the reference twin starts (CHAOS_TUNE_LLE_TWIN 1, 2) are FP64 only");
    if ((rc = check_ff32_lle(ex, system, L))) return rc;
    Call c;
    if ((rc = c.begin(ex))) return rc;
    if ((rc = upload_log_axes(c, gridMode, dim, nPts, ranges, L.table))) return c.finish(rc);
    double* dOut = (double*)c.output(lle, L.nPoints * sizeof(double));
    if (c.failed) return c.finish(CHAOS_E_NOMEM);
    cudaError_t e = run_lle(c.ex.precision, L, dOut, c.stream);
    if (e != cudaSuccess) return c.finish(cuda_error(e, "LLE kernel"));
    rc = c.to_host(lle, dOut, L.nPoints * sizeof(double));
    return c.finish(rc);
}

int chaos_lle_sweep_legacy(const chaos_exec* ex, int system, int dim, int gridMode, double tMax, double NT,
                           int nPts, double h, double eps, const double* initialConditions,
                           int amountOfInitialConditions, const double* ranges, const int* indicesOfMutVars,
                           double maxValue, double transientTime, const double* values, int amountOfValues,
                           const double* draws, double* lle) {
    return run_legacy_scheme(ex, false, system, dim, gridMode, tMax, NT, nPts, h, eps, initialConditions,
                             amountOfInitialConditions, ranges, indicesOfMutVars, maxValue, transientTime, values,
                             amountOfValues, draws, lle);
}

int chaos_lyapunov_spectrum_legacy(const chaos_exec* ex, int system, int dim, int gridMode, double tMax, double NT,
                                   int nPts, double h, double eps, const double* initialConditions,
                                   int amountOfInitialConditions, const double* ranges, const int* indicesOfMutVars,
                                   double maxValue, double transientTime, const double* values, int amountOfValues,
                                   const double* draws, double* spectrum) {
    if (system == SYS_USER) return set_error(CHAOS_E_UNSUPPORTED, "the spectrum runs on the built-in systems");
    return run_legacy_scheme(ex, true, system, dim, gridMode, tMax, NT, nPts, h, eps, initialConditions,
                             amountOfInitialConditions, ranges, indicesOfMutVars, maxValue, transientTime, values,
                             amountOfValues, draws, spectrum);
}

int chaos_legacy_lle_draws(const chaos_exec* ex, int kind, long long n, int nx, double* draws) {
    if (kind < 0 || kind > 2 || n < 0 || nx < 1 || nx > kMaxState || (n > 0 && !draws))
        return set_error(CHAOS_E_ARGS, "bad twin-draw arguments");
    if (n == 0) return CHAOS_OK;
    const size_t bytes = (size_t)n * nx * (kind == 2 ? nx : 1) * sizeof(double);
    Call c;
    int rc = c.begin(ex);
    if (rc) return rc;
    double* d = (double*)c.output(draws, bytes);
    if (c.failed) return c.finish(CHAOS_E_NOMEM);
    cudaError_t e = launch_legacy_draws(kind, n, nx, d, c.stream);
    if (e != cudaSuccess) return c.finish(cuda_error(e, "twin draws"));
    rc = c.to_host(draws, d, bytes);
    return c.finish(rc);
}

int chaos_lle_from_states(const chaos_exec* ex, int system, long long n, const double* states, double tMax,
                          double NT, double h, double eps, double* lle) {
    if (system == SYS_USER) return set_error(CHAOS_E_UNSUPPORTED, "starting states run on the built-in systems");
    if (!system_supported(system)) return set_error(CHAOS_E_ARGS, "unknown system %d", system);
    if (n < 0 || (n > 0 && (!states || !lle))) return set_error(CHAOS_E_ARGS, "bad starting-state arguments");
    if (!(h > 0) || !(tMax > 0) || !(NT > 0) || !(eps > 0)) return set_error(CHAOS_E_ARGS, "need h, tMax, NT, eps > 0");
    if (NT / h > 2.0e9 || tMax / h > 2.0e9) return set_error(CHAOS_E_ARGS, "step counts must fit in int");
    const int prec = ex ? ex->precision : CHAOS_FP64;
    if (prec == CHAOS_FP32)
        return set_error(CHAOS_E_UNSUPPORTED, "starting states run in CHAOS_FP64 or CHAOS_FF32");
    if (prec == CHAOS_FF32 && !system_has_difference_form(system))
        return set_error(CHAOS_E_UNSUPPORTED, "CHAOS_FF32 LLE needs an RK4 system (0-2)");
    LleParams L;
    memset(&L, 0, sizeof L);
    L.system = system;
    L.ntp = static_cast<int>(NT / h);
    if (L.ntp < 1) return set_error(CHAOS_E_ARGS, "NT / h must be >= 1");
    L.calcBlocks = static_cast<int>(tMax / h) / L.ntp + 1;
    L.h = h;
    L.eps = eps;
    L.tMax = tMax;
    L.nPoints = n;
    int nx, na;
    sizes_of(system, &nx, &na);
    const size_t rowBytes = (size_t)(2 * nx + na) * sizeof(double);
    Call c;
    int rc = c.begin(ex);
    if (rc) return rc;
    if (n == 0) return c.finish(CHAOS_OK);
    const double* dStates = (const double*)c.input(states, (size_t)n * rowBytes);
    double* dOut = (double*)c.output(lle, (size_t)n * sizeof(double));
    if (c.failed) return c.finish(CHAOS_E_NOMEM);
    cudaError_t e = prec == CHAOS_FF32 ? launch_lle_states_ff(L, dStates, dOut, c.stream)
                                       : launch_lle_states_f64(L, dStates, dOut, c.stream);
    if (e != cudaSuccess) return c.finish(cuda_error(e, "LLE kernel"));
    rc = c.to_host(lle, dOut, (size_t)n * sizeof(double));
    return c.finish(rc);
}

int chaos_lyapunov_spectrum(const chaos_exec* ex, int system, int dim, int gridMode, double tMax, double NT,
                            int nPts, double h, double eps, const double* initialConditions,
                            int amountOfInitialConditions, const double* ranges, const int* indicesOfMutVars,
                            double transientTime, const double* values, int amountOfValues, double* spectrum) {
    int rc = CHAOS_OK;
    if (!spectrum) return set_error(CHAOS_E_ARGS, "null argument");
    if (system == SYS_USER) return set_error(CHAOS_E_UNSUPPORTED, "the spectrum runs on the built-in systems");
    LleParams L;
    if ((rc = fill_lle(L, system, tMax, NT, nPts, h, eps, initialConditions, amountOfInitialConditions, ranges,
                       indicesOfMutVars, transientTime, values, amountOfValues, dim, gridMode)))
        return rc;
    if ((rc = no_ff32(ex, "the Lyapunov spectrum"))) return rc;
    const bool fp32 = ex && ex->precision == CHAOS_FP32;
    if (fp32 && !system_has_fp32_lle(system))
        return set_error(CHAOS_E_UNSUPPORTED,
                         "the FP32 spectrum needs a quadratic RK4 system (0-2) or Chameleon; use CHAOS_FP64");
    Call c;
    if ((rc = c.begin(ex))) return rc;
    if ((rc = upload_log_axes(c, gridMode, dim, nPts, ranges, L.table))) return c.finish(rc);
    const size_t bytes = (size_t)L.nPoints * system_nx(system) * sizeof(double);
    double* dOut = (double*)c.output(spectrum, bytes);
    if (c.failed) return c.finish(CHAOS_E_NOMEM);
    cudaError_t e = fp32 ? launch_spectrum_f32(L, dOut, c.stream) : launch_spectrum_f64(L, dOut, c.stream);
    if (e != cudaSuccess) return c.finish(cuda_error(e, "Lyapunov spectrum kernel"));
    rc = c.to_host(spectrum, dOut, bytes);
    return c.finish(rc);
}

int chaos_lle2d_checked(const chaos_exec* ex, int system, double tMax, double NT, int nPts, double h, double eps,
                        const double* initialConditions, int amountOfInitialConditions, const double* ranges,
                        const int* indicesOfMutVars, double transientTime, const double* values, int amountOfValues,
                        double band, double checkTMax, double* lle, long long* nChecked, long long* nReplaced) {
    int rc = CHAOS_OK;
    if (!lle) return set_error(CHAOS_E_ARGS, "null argument");
    if (!(band >= 0) || !(checkTMax > 0)) return set_error(CHAOS_E_ARGS, "need band >= 0 and checkTMax > 0");
    LleParams L, Lc;
    if ((rc = fill_lle(L, system, tMax, NT, nPts, h, eps, initialConditions, amountOfInitialConditions, ranges,
                       indicesOfMutVars, transientTime, values, amountOfValues)))
        return rc;
    const bool fullCheck = checkTMax >= tMax;
    if ((rc = fill_lle(Lc, system, fullCheck ? tMax : checkTMax, NT, nPts, h, eps, initialConditions,
                       amountOfInitialConditions, ranges, indicesOfMutVars, transientTime, values, amountOfValues)))
        return rc;
    if (system == SYS_USER || !system_has_fp32_lle(system))
        return set_error(CHAOS_E_UNSUPPORTED, "FP32 LLE needs a quadratic RK4 system (0-2) or Chameleon");
    if (L.twin != 0) return set_error(CHAOS_E_UNSUPPORTED, "the reference twin starts (CHAOS_TUNE_LLE_TWIN 1, 2) are FP64 only");
    if (L.nPoints > 0x7fffffffLL) return set_error(CHAOS_E_ARGS, "nPts^2 must be < 2^31");
    Call c;
    if ((rc = c.begin(ex))) return rc;
    const long long n = L.nPoints;
    double* dOut = (double*)c.output(lle, n * sizeof(double));
    int* counts = (int*)c.alloc(2 * sizeof(int));
    int* list = (int*)c.alloc(n * sizeof(int));
    if (c.failed) return c.finish(CHAOS_E_NOMEM);
    cudaError_t e = launch_lle_f32(L, dOut, c.stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(counts, 0, 2 * sizeof(int), c.stream);
    if (e == cudaSuccess) e = launch_lle_select(dOut, n, band, list, counts, c.stream);
    int h0[2] = {0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(h0, counts, sizeof(int), cudaMemcpyDeviceToHost, c.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
    if (e != cudaSuccess) return c.finish(cuda_error(e, "FP32 LLE map and selection"));
    const long long checked = h0[0];
    long long replaced = 0;
    if (checked > 0) {
        double* check = (double*)c.alloc(checked * sizeof(double));
        int* list2 = fullCheck ? nullptr : (int*)c.alloc(checked * sizeof(int));
        if (c.failed) return c.finish(CHAOS_E_NOMEM);
        e = launch_lle_list_f64(Lc, list, counts, checked, check, false, c.stream);
        if (e == cudaSuccess)
            e = launch_lle_flip(dOut, list, counts, checked, check, fullCheck, dOut, list2, counts + 1, c.stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(h0 + 1, counts + 1, sizeof(int), cudaMemcpyDeviceToHost, c.stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
        if (e == cudaSuccess && !fullCheck && h0[1] > 0)
            e = launch_lle_list_f64(L, list2, counts + 1, h0[1], dOut, true, c.stream);
        if (e != cudaSuccess) return c.finish(cuda_error(e, "FP64 re-check"));
        replaced = h0[1];
    }
    if (nChecked) *nChecked = checked;
    if (nReplaced) *nReplaced = replaced;
    rc = c.to_host(lle, dOut, n * sizeof(double));
    return c.finish(rc);
}

int chaos_basins_features(const chaos_exec* ex, int system, double tMax, int nPts, double h,
                          int amountOfInitialConditions, const double* initialConditions, const double* ranges,
                          const int* indicesOfMutVars, int writableVar, double maxValue, double transientTime,
                          const double* values, int amountOfValues, int preScaller, int* flags, double* avgPeaks,
                          double* avgIntervals, int* counts) {
    SweepParams P;
    int rc = fill_sweep(P, system, 2, tMax, nPts, h, amountOfInitialConditions, initialConditions, ranges,
                        indicesOfMutVars, writableVar, maxValue, transientTime, values, amountOfValues, preScaller,
                        true);
    if (rc) return rc;
    if (!flags || !avgPeaks || !avgIntervals) return set_error(CHAOS_E_ARGS, "flags, avgPeaks and avgIntervals are required");
    if ((rc = no_ff32(ex, "the basins sweep"))) return rc;
    Call c;
    if ((rc = c.begin(ex))) return rc;
    const long long n = P.nPoints;
    BasinsOut O;
    O.flags = (int*)c.output(flags, n * sizeof(int));
    O.avgPeaks = (double*)c.output(avgPeaks, n * sizeof(double));
    O.avgIntervals = (double*)c.output(avgIntervals, n * sizeof(double));
    O.counts = (int*)c.output(counts, n * sizeof(int));
    O.last = nullptr;
    if (c.failed) return c.finish(CHAOS_E_NOMEM);
    cudaError_t e = run_basins(c.ex.precision, P, O, c.stream);
    if (e != cudaSuccess) return c.finish(cuda_error(e, "basins kernel"));
    rc = c.to_host(flags, O.flags, n * sizeof(int));
    if (!rc) rc = c.to_host(avgPeaks, O.avgPeaks, n * sizeof(double));
    if (!rc) rc = c.to_host(avgIntervals, O.avgIntervals, n * sizeof(double));
    if (!rc) rc = c.to_host(counts, O.counts, n * sizeof(int));
    return c.finish(rc);
}

int chaos_basins(const chaos_exec* ex, int system, double tMax, int nPts, double h, int amountOfInitialConditions,
                 const double* initialConditions, const double* ranges, const int* indicesOfMutVars,
                 int writableVar, double maxValue, double transientTime, const double* values, int amountOfValues,
                 int preScaller, double eps, int* labels, double* avgPeaks, double* avgIntervals, int* flags) {
    SweepParams P;
    int rc = fill_sweep(P, system, 2, tMax, nPts, h, amountOfInitialConditions, initialConditions, ranges,
                        indicesOfMutVars, writableVar, maxValue, transientTime, values, amountOfValues, preScaller,
                        true);
    if (rc) return rc;
    if (!labels) return set_error(CHAOS_E_ARGS, "labels is required");
    if (!(eps >= 0)) return set_error(CHAOS_E_ARGS, "eps must be >= 0");
    if ((rc = no_ff32(ex, "the basins sweep"))) return rc;
    Call c;
    if ((rc = c.begin(ex))) return rc;
    const long long n = P.nPoints;
    BasinsOut O;
    O.flags = flags ? (int*)c.output(flags, n * sizeof(int)) : (int*)c.alloc(n * sizeof(int));
    O.avgPeaks = avgPeaks ? (double*)c.output(avgPeaks, n * sizeof(double)) : (double*)c.alloc(n * sizeof(double));
    O.avgIntervals = avgIntervals ? (double*)c.output(avgIntervals, n * sizeof(double)) : (double*)c.alloc(n * sizeof(double));
    O.counts = nullptr;
    O.last = nullptr;
    int* dLabels = (int*)c.output(labels, n * sizeof(int));
    if (c.failed) return c.finish(CHAOS_E_NOMEM);
    cudaError_t e = run_basins(c.ex.precision, P, O, c.stream);
    if (e != cudaSuccess) return c.finish(cuda_error(e, "basins kernel"));
    rc = dbscan_compat_device(c, O.avgPeaks, O.avgIntervals, O.flags, n, eps, dLabels);
    if (!rc) rc = c.to_host(labels, dLabels, n * sizeof(int));
    if (!rc && flags) rc = c.to_host(flags, O.flags, n * sizeof(int));
    if (!rc && avgPeaks) rc = c.to_host(avgPeaks, O.avgPeaks, n * sizeof(double));
    if (!rc && avgIntervals) rc = c.to_host(avgIntervals, O.avgIntervals, n * sizeof(double));
    return c.finish(rc);
}

int chaos_basins_dbscan(const chaos_exec* ex, int system, double tMax, int nPts, double h,
                        int amountOfInitialConditions, const double* initialConditions, const double* ranges,
                        const int* indicesOfMutVars, int writableVar, double maxValue, double transientTime,
                        const double* values, int amountOfValues, int preScaller, double eps, int minPts,
                        int* labels, double* features, int* flags) {
    SweepParams P;
    int rc = fill_sweep(P, system, 2, tMax, nPts, h, amountOfInitialConditions, initialConditions, ranges,
                        indicesOfMutVars, writableVar, maxValue, transientTime, values, amountOfValues, preScaller,
                        true);
    if (rc) return rc;
    if (!labels) return set_error(CHAOS_E_ARGS, "labels is required");
    if (!(eps > 0) || minPts < 1) return set_error(CHAOS_E_ARGS, "need eps > 0 and minPts >= 1");
    if ((rc = no_ff32(ex, "the basins sweep"))) return rc;
    Call c;
    if ((rc = c.begin(ex))) return rc;
    const long long n = P.nPoints;
    BasinsOut O;
    O.flags = flags ? (int*)c.output(flags, n * sizeof(int)) : (int*)c.alloc(n * sizeof(int));
    O.avgPeaks = (double*)c.alloc(n * sizeof(double));
    O.avgIntervals = (double*)c.alloc(n * sizeof(double));
    O.counts = (int*)c.alloc(n * sizeof(int));
    O.last = (double*)c.alloc(n * sizeof(double));
    // the integration kernels fold the features' minima and maxima into
    // these keys; the clustering normalises the features on the fly and
    // writes the row-major matrix only when the caller asks for it
    O.mm = (unsigned long long*)c.alloc(6 * kKeyReplicas * sizeof(unsigned long long));
    double* F = features ? (double*)c.output(features, (size_t)n * 3 * sizeof(double)) : nullptr;
    int* dLabels = (int*)c.output(labels, n * sizeof(int));
    if (c.failed) return c.finish(CHAOS_E_NOMEM);
    cudaError_t e = cudaMemsetAsync(O.mm, 0xff, 3 * kKeyReplicas * sizeof(unsigned long long), c.stream);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(O.mm + 3 * kKeyReplicas, 0, 3 * kKeyReplicas * sizeof(unsigned long long), c.stream);
    if (e == cudaSuccess) e = run_basins(c.ex.precision, P, O, c.stream);
    unsigned long long hm[6 * kKeyReplicas], keys[6];
    if (e == cudaSuccess) e = cudaMemcpyAsync(hm, O.mm, sizeof hm, cudaMemcpyDeviceToHost, c.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
    if (e != cudaSuccess) return c.finish(cuda_error(e, "basins kernels"));
    for (int k = 0; k < 6; ++k) {
        keys[k] = hm[k * kKeyReplicas];
        for (int r = 1; r < kKeyReplicas; ++r)
            keys[k] = k < 3 ? std::min(keys[k], hm[k * kKeyReplicas + r]) : std::max(keys[k], hm[k * kKeyReplicas + r]);
    }
    rc = dbscan_basins_device(c, O, n, keys, eps, minPts, F, dLabels);
    if (!rc) rc = c.to_host(labels, dLabels, n * sizeof(int));
    if (!rc && features) rc = c.to_host(features, F, (size_t)n * 3 * sizeof(double));
    if (!rc && flags) rc = c.to_host(flags, O.flags, n * sizeof(int));
    return c.finish(rc);
}

int chaos_dbscan_compat(const chaos_exec* ex, const double* avgPeaks, const double* avgIntervals, const int* flags,
                        long long n, double eps, int* labels) {
    if (n < 0 || (n > 0 && (!avgPeaks || !avgIntervals || !flags || !labels)))
        return set_error(CHAOS_E_ARGS, "null array or negative n");
    if (!(eps >= 0)) return set_error(CHAOS_E_ARGS, "eps must be >= 0");
    if (n > 0x7fffffffLL) return set_error(CHAOS_E_ARGS, "n must be < 2^31");
    Call c;
    int rc = c.begin(ex);
    if (rc) return rc;
    if (n == 0) return c.finish(CHAOS_OK);
    const double* dP = (const double*)c.input(avgPeaks, n * sizeof(double));
    const double* dI = (const double*)c.input(avgIntervals, n * sizeof(double));
    const int* dF = (const int*)c.input(flags, n * sizeof(int));
    int* dL = (int*)c.output(labels, n * sizeof(int));
    if (c.failed) return c.finish(CHAOS_E_NOMEM);
    rc = dbscan_compat_device(c, dP, dI, dF, n, eps, dL);
    if (!rc) rc = c.to_host(labels, dL, n * sizeof(int));
    return c.finish(rc);
}

int chaos_dbscan(const chaos_exec* ex, const double* features, long long n, int dims, double eps, int minPts,
                 const int* mask, int* labels) {
    if (n < 0 || (n > 0 && (!features || !labels))) return set_error(CHAOS_E_ARGS, "null array or negative n");
    if (dims < 1 || dims > 3) return set_error(CHAOS_E_ARGS, "dims must be 1..3");
    if (!(eps > 0) || minPts < 1) return set_error(CHAOS_E_ARGS, "need eps > 0 and minPts >= 1");
    if (n > 0x7fffffffLL) return set_error(CHAOS_E_ARGS, "n must be < 2^31");
    Call c;
    int rc = c.begin(ex);
    if (rc) return rc;
    if (n == 0) return c.finish(CHAOS_OK);
    const double* dF = (const double*)c.input(features, (size_t)n * dims * sizeof(double));
    const int* dM = (const int*)c.input(mask, n * sizeof(int));
    int* dL = (int*)c.output(labels, n * sizeof(int));
    if (c.failed) return c.finish(CHAOS_E_NOMEM);
    rc = dbscan_device(c, dF, n, dims, eps, minPts, dM, dL);
    if (!rc) rc = c.to_host(labels, dL, n * sizeof(int));
    return c.finish(rc);
}

int chaos_peak_finder(const chaos_exec* ex, const double* data, long long nSeries, int len, double h,
                      int peakCapacity, int* counts, double* peaks, double* intervals) {
    if (nSeries < 0 || len < 0 || peakCapacity < 1 || (nSeries > 0 && (!data || !counts || !peaks || !intervals)))
        return set_error(CHAOS_E_ARGS, "bad peak finder arguments");
    Call c;
    int rc = c.begin(ex);
    if (rc) return rc;
    if (nSeries == 0) return c.finish(CHAOS_OK);
    const size_t rows = (size_t)nSeries * peakCapacity * sizeof(double);
    const double* dD = (const double*)c.input(data, (size_t)nSeries * len * sizeof(double));
    int* dC = (int*)c.output(counts, nSeries * sizeof(int));
    double* dP = (double*)c.output(peaks, rows);
    double* dI = (double*)c.output(intervals, rows);
    if (c.failed) return c.finish(CHAOS_E_NOMEM);
    cudaError_t e = launch_peak_finder(dD, nSeries, len, h, peakCapacity, dC, dP, dI, c.stream);
    if (e != cudaSuccess) return c.finish(cuda_error(e, "peak finder kernel"));
    rc = c.to_host(counts, dC, nSeries * sizeof(int));
    if (!rc) rc = c.to_host(peaks, dP, rows);
    if (!rc) rc = c.to_host(intervals, dI, rows);
    return c.finish(rc);
}

int chaos_point_dbscan(const chaos_exec* ex, const double* intervals, const int* counts, long long n, int stride,
                       double eps, int* labels) {
    if (n < 0 || stride < 1 || (n > 0 && (!intervals || !counts || !labels)))
        return set_error(CHAOS_E_ARGS, "bad point dbscan arguments");
    Call c;
    int rc = c.begin(ex);
    if (rc) return rc;
    if (n == 0) return c.finish(CHAOS_OK);
    const double* dI = (const double*)c.input(intervals, (size_t)n * stride * sizeof(double));
    const int* dC = (const int*)c.input(counts, n * sizeof(int));
    int* dL = (int*)c.output(labels, n * sizeof(int));
    int* lab = (int*)c.alloc((size_t)n * stride * sizeof(int));
    int* slot = (int*)c.alloc((size_t)n * stride * sizeof(int));
    if (c.failed) return c.finish(CHAOS_E_NOMEM);
    cudaError_t e = launch_point_dbscan(dI, dC, n, stride, eps, lab, slot, dL, c.stream);
    if (e != cudaSuccess) return c.finish(cuda_error(e, "point dbscan kernel"));
    rc = c.to_host(labels, dL, n * sizeof(int));
    return c.finish(rc);
}

int chaos_set_tuning(int knob, int value) {
    if (knob == CHAOS_TUNE_LLE_F32_VARIANT)
        return set_lle_variant(value) == 0 ? CHAOS_OK : set_error(CHAOS_E_ARGS, "LLE variant must be 0, 2, 12 or 16");
    if (knob == CHAOS_TUNE_SWEEP_PAIRS)
        return set_sweep_pairs(value) ? set_error(CHAOS_E_ARGS, "sweep-pairs mode %d (0, 1, 2 or 3)", value) : CHAOS_OK;
    if (knob == CHAOS_TUNE_LLE_RENORM)
        return set_lle_renorm(value) ? set_error(CHAOS_E_ARGS, "LLE renormalisation mode %d (0, 1 or 2)", value)
                                     : CHAOS_OK;
    if (knob == CHAOS_TUNE_FF_PAIRS)
        return set_ff_pairs(value) ? set_error(CHAOS_E_ARGS, "float-float pairs mode %d (0 or 1)", value) : CHAOS_OK;
    if (knob == CHAOS_TUNE_SHAPES) {
        if (value != 0) return set_error(CHAOS_E_ARGS, "CHAOS_TUNE_SHAPES takes 0 (forget tuned shapes)");
        for (int k = 0; k < 3; ++k)
            for (int s = 0; s <= SYS_CHEN_RK4; ++s) set_launch_shape(k, s, 0);
        return CHAOS_OK;
    }
    if (knob == CHAOS_TUNE_BIF2D_CAP) {
        if (value < -1) return set_error(CHAOS_E_ARGS, "bifurcation 2-D capacity: -1, 0 or a row size");
        g_bif2d_cap.store(value);
        return CHAOS_OK;
    }
    if (knob == CHAOS_TUNE_GRID_FMA || knob == CHAOS_TUNE_LLE_TWIN) {
        const int hi = knob == CHAOS_TUNE_LLE_TWIN ? 2 : 1;
        if (value < 0 || value > hi) return set_error(CHAOS_E_ARGS, "knob %d takes 0 to %d", knob, hi);
        (knob == CHAOS_TUNE_GRID_FMA ? g_grid_fma : g_lle_twin).store(value);
        return CHAOS_OK;
    }
    return set_error(CHAOS_E_ARGS, "unknown tuning knob %d", knob);
}

int chaos_get_tuning(int knob) {
    if (knob == CHAOS_TUNE_LLE_F32_VARIANT) return get_lle_variant();
    if (knob == CHAOS_TUNE_SWEEP_PAIRS) return sweep_pairs();
    if (knob == CHAOS_TUNE_GRID_FMA) return g_grid_fma.load();
    if (knob == CHAOS_TUNE_LLE_TWIN) return g_lle_twin.load();
    if (knob == CHAOS_TUNE_BIF2D_CAP) return g_bif2d_cap.load();
    if (knob == CHAOS_TUNE_LLE_RENORM) return get_lle_renorm();
    if (knob == CHAOS_TUNE_FF_PAIRS) return get_ff_pairs();
    return set_error(CHAOS_E_ARGS, "unknown tuning knob %d", knob);
}

int chaos_trajectory(const chaos_exec* ex, int system, long long nTraj, const double* x0, const double* a, double h,
                     int nSteps, double* out) {
    if (system == SYS_USER && !user_system_available())
        return set_error(CHAOS_E_UNSUPPORTED, "the library was built without a user plug-in");
    if (!system_supported(system)) return set_error(CHAOS_E_ARGS, "unknown system %d", system);
    if (nTraj < 0 || nSteps < 0 || !(h == h) || (nTraj > 0 && (!x0 || !a || !out)))
        return set_error(CHAOS_E_ARGS, "bad trajectory arguments");
    if (ex && ex->precision == CHAOS_FF32 && !system_has_difference_form(system))
        return set_error(CHAOS_E_UNSUPPORTED, "CHAOS_FF32 trajectories need an RK4 system (0-2)");
    Call c;
    int rc = c.begin(ex);
    if (rc) return rc;
    if (nTraj == 0) return c.finish(CHAOS_OK);
    int nx, na;
    sizes_of(system, &nx, &na);
    const size_t outBytes = (size_t)nTraj * (nSteps + 1) * nx * sizeof(double);
    const double* dX = (const double*)c.input(x0, (size_t)nTraj * nx * sizeof(double));
    const double* dA = (const double*)c.input(a, (size_t)nTraj * na * sizeof(double));
    double* dO = (double*)c.output(out, outBytes);
    if (c.failed) return c.finish(CHAOS_E_NOMEM);
    cudaError_t e;
    if (system == SYS_USER)
        e = c.ex.precision != CHAOS_FP64 ? cudaErrorNotSupported
                                         : launch_trajectory_user(dX, dA, h, nSteps, dO, nTraj, c.stream);
    else if (c.ex.precision == CHAOS_FF32)
        e = launch_trajectory_ff(system, dX, dA, h, nSteps, dO, nTraj, c.stream);
    else
        e = c.ex.precision == CHAOS_FP32 ? launch_trajectory_f32(system, dX, dA, h, nSteps, dO, nTraj, c.stream)
                                         : launch_trajectory_f64(system, dX, dA, h, nSteps, dO, nTraj, c.stream);
    if (e != cudaSuccess) return c.finish(cuda_error(e, "trajectory kernel"));
    rc = c.to_host(out, dO, outBytes);
    return c.finish(rc);
}

}  // extern "C"
