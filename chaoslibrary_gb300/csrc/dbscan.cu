// Grid clustering on the device, cell first.
//
// Both clusterings (textbook DBSCAN and the reference's eps-components) run
// one pipeline over points in a D-dimensional feature space (D = 1..3). The
// points are read from a feature source: feature columns, a row-major matrix,
// or the basin map's per-point outputs normalised on the fly. The work is
// arranged so that a map's millions of points are read once and touched
// again only through 4-byte cell slots, while exact point tests run on the
// few cells that need them:
//   1. one pass over the points: the cell of every point (floor(f / side) per
//      dimension, side = eps / sqrt(D) shrunk by 1e-9, so two points of one
//      cell are always within eps and a neighbour within eps is at most R = 2
//      cells away per dimension) goes into an open-addressing hash table; the
//      runs of equal cells along a warp fold into it, with one atomic per
//      quantity, their point count, bounding box (float bounds rounded
//      outward: still a box around the points), smallest and largest index
//      (the cell's representatives) and smallest fixed-point index, and a
//      clamped/NaN mark; the point keeps its slot;
//   2. per cell: dense (a safe cell with >= minPts points -- every included
//      point in the reference mode: all its points are core) or not; the
//      occupied neighbour cells; per neighbouring pair, the bounding boxes
//      settle most pairs (farther than eps: nothing; every point within eps:
//      joined), the representatives join most other pairs of dense cells;
//      the joined pairs' components come from one block's union-find in
//      shared memory;
//   3. the points of the cells that are not dense are sorted by cell (one
//      pass over the slots) and their core flags counted: whole cells by
//      their boxes, dense cells' representatives as a lower bound, sorted
//      cells exactly; core points join dense neighbours the same way;
//   4. the cells that some pair, core count or border label still has to
//      scan -- pairs of dense cells that the unions so far leave apart, dense
//      neighbours of points whose count or label the shortcuts cannot settle
//      -- are sorted in a second pass, and their point pairs tested exactly;
//   5. union-find over nodes: a safe cell's core points are one node (they
//      are within eps of each other), a core point of a clamped/NaN cell is
//      a node of its own; lock-free hooking with atomicCAS, parent[v] <= v;
//   6. components numbered by their smallest core index (and, in the
//      reference mode, their smallest fixed-point index); one pass over the
//      slots writes the labels of the dense cells' points, a kernel over the
//      sorted points those of the others (border points: the component of
//      the smallest index among the core points within eps).
// Distances are sqrt(sum of squared differences) <= eps in FP64, in dimension
// order, each operation rounded on its own (this file is compiled with
// --fmad=false), as the reference computes them (Basins/src/basinsCUDA.cu:918);
// the square root is skipped where the squared distance is clear of eps^2 by
// 1e-7. Cells whose coordinates had to be clamped (|f| / side >= 2^19) or that
// hold a NaN feature lose the one-cell-is-connected shortcut and are resolved
// by exact pair tests. Every box test keeps a relative margin of 1e-7 on
// squared distances, and a representative is a real point of its cell, so the
// shortcuts skip work without changing a label.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "dbscan.h"
#include "order_keys.h"

namespace chaos {

namespace {

constexpr int kTPB = 256;
constexpr unsigned long long kEmpty = ~0ull;
constexpr long long kLim = 1LL << 19;  // clamp of cell coordinates (21-bit packing for D = 3)
constexpr int kR = 2;                  // neighbour reach in cells
constexpr int kReps = 2;               // representatives per cell: its smallest and largest point index

__device__ __forceinline__ unsigned long long pack(const long long* c, int D) {
    if (D <= 2) {
        const unsigned long long a = (unsigned long long)(c[0] + 2147483648LL);
        const unsigned long long b = (unsigned long long)((D == 2 ? c[1] : 0) + 2147483648LL);
        return (a << 32) | (b & 0xffffffffull);
    }
    return (((unsigned long long)c[0] & 0x1FFFFFull) << 42) | (((unsigned long long)c[1] & 0x1FFFFFull) << 21) |
           ((unsigned long long)c[2] & 0x1FFFFFull);
}

__device__ __forceinline__ void unpack(unsigned long long k, int D, long long* c) {
    if (D <= 2) {
        c[0] = (long long)(k >> 32) - 2147483648LL;
        c[1] = (long long)(k & 0xffffffffull) - 2147483648LL;
        c[2] = 0;
        return;
    }
    for (int d = 0; d < 3; ++d) {
        long long v = (long long)((k >> (42 - 21 * d)) & 0x1FFFFFull);
        if (v & 0x100000) v -= 0x200000;
        c[d] = v;
    }
}

__device__ __forceinline__ unsigned long long mix(unsigned long long k) {
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdull;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ull;
    k ^= k >> 33;
    return k;
}

__device__ __forceinline__ double dist2(const double* a, const double* b, int D) {
    double s = 0.0;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        if (d >= D) continue;
        const double df = a[d] - b[d];
        s = s + df * df;
    }
    return s;
}

// ---- prefix sum ------------------------------------------------------------
constexpr int kScanItems = 4096;  // 1024 threads x 4

template <class T>
__global__ void __launch_bounds__(1024) scan_block_kernel(const T* in, T* out, T* blockSums, long long n) {
    __shared__ T warpSums[32];
    const long long base = (long long)blockIdx.x * kScanItems + threadIdx.x * 4;
    T v[4], s = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        v[j] = base + j < n ? in[base + j] : 0;
        s += v[j];
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    T x = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const T y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warpSums[w] = x;
    __syncthreads();
    if (w == 0) {
        T ws = warpSums[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const T y = __shfl_up_sync(0xffffffffu, ws, o);
            if (lane >= o) ws += y;
        }
        warpSums[lane] = ws;
    }
    __syncthreads();
    T prefix = (w > 0 ? warpSums[w - 1] : 0) + x - s;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        if (base + j < n) out[base + j] = prefix;
        prefix += v[j];
    }
    if (threadIdx.x == 1023) blockSums[blockIdx.x] = warpSums[31];
}

template <class T>
__global__ void add_offsets_kernel(T* out, const T* offsets, long long n) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] += offsets[i / kScanItems];
}

inline unsigned blocks(long long n, int tpb = kTPB) { return (unsigned)((n + tpb - 1) / tpb); }

// ---- order keys (order_keys.h: okey, unkey, group_min64, group_max64) ------------
// Order keys of floats: the cell boxes are kept in float, each bound rounded
// outward (minima down, maxima up), so a box still holds all its points and
// every box test stays one-sided; 32-bit keys take the native atomics.
__device__ __forceinline__ unsigned fkey(float f) {
    const unsigned b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float unfkey(unsigned k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}
constexpr unsigned kFKeyPosInf = 0xff800000u;  // fkey(+inf)
constexpr unsigned kFKeyNegInf = 0x007fffffu;  // fkey(-inf)

// ---- cell boxes ------------------------------------------------------------------
// A cell's box holds all its points, so a box farther than eps from a point
// (or from another box) holds no point within eps, and a box whose farthest
// corner is within eps holds only points within eps. Both tests keep a
// relative margin of 1e-7 on the squared distance (far above the rounding of
// the exact test), so they never change a result, only skip work.
constexpr double kBoxOut = 1.0000001, kBoxIn = 0.9999999;

// sqrt(d2) <= eps, the reference's test, with the square root taken only near
// the boundary: a squared distance below eps^2 (1 - 1e-7) has its root below
// eps and one above eps^2 (1 + 1e-7) above it, far outside the roundings of
// the square, the product and the root; NaN is never within.
__device__ __forceinline__ bool within_eps(double d2, double eps) {
    const double eps2 = eps * eps;
    if (d2 <= eps2 * kBoxIn) return true;
    if (d2 > eps2 * kBoxOut) return false;
    return sqrt(d2) <= eps;
}

__device__ __forceinline__ void box_dist2(const double* v, const double* lo, const double* hi, int D, double& near2,
                                          double& far2) {
    near2 = 0.0;
    far2 = 0.0;
    for (int d = 0; d < D; ++d) {
        double g = 0.0;
        if (v[d] < lo[d]) g = lo[d] - v[d];
        else if (v[d] > hi[d]) g = v[d] - hi[d];
        near2 = near2 + g * g;
        const double f = fmax(fabs(v[d] - lo[d]), fabs(hi[d] - v[d]));
        far2 = far2 + f * f;
    }
}

// ---- union-find (parent[v] <= v) --------------------------------------------
__device__ __forceinline__ int uf_find(int* parent, int x) {
    int cur = __ldcg(parent + x);
    if (cur != x) {
        int prev = x, next;
        while (cur > (next = __ldcg(parent + cur))) {
            parent[prev] = next;
            prev = cur;
            cur = next;
        }
    }
    return cur;
}

__device__ __forceinline__ void uf_unite(int* parent, int a, int b) {
    int ra = uf_find(parent, a), rb = uf_find(parent, b);
    while (ra != rb) {
        if (ra < rb) { const int t = ra; ra = rb; rb = t; }
        const int old = atomicCAS(parent + ra, ra, rb);
        if (old == ra) break;
        ra = old;
        rb = uf_find(parent, rb);
        ra = uf_find(parent, ra);
    }
}

// warp-aggregated append of p to list (one atomic per warp)
__device__ __forceinline__ void list_append(bool take, int p, int* list, int* count) {
    const unsigned m = __ballot_sync(0xffffffffu, take);
    if (!m) return;
    const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(count, __popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (take) list[base + __popc(m & ((1u << lane) - 1))] = p;
}

// ---- feature sources ---------------------------------------------------------
// Where the clustering reads point i: whether it takes part, its features
// (FP64) and, for the reference-compatible numbering, whether it is a fixed
// point (flag -1).
struct ColSrc {  // feature columns
    const double* f[3];
    const int* mask;   // textbook mode: the points with mask[i] != 0 (all when null)
    const int* flags;  // reference mode: the points with flags[i] != 0
    int D;
    bool compat;
    __device__ __forceinline__ bool included(long long i) const {
        return compat ? flags[i] != 0 : (mask ? mask[i] != 0 : true);
    }
    __device__ __forceinline__ bool fix(long long i) const { return compat && flags[i] == -1; }
    __device__ __forceinline__ void load(long long i, double* v) const {
#pragma unroll
        for (int d = 0; d < 3; ++d)
            if (d < D) v[d] = f[d][i];
    }
};

struct RowSrc {  // row-major n x D matrix, textbook mode
    const double* F;
    const int* mask;
    int D;
    __device__ __forceinline__ bool included(long long i) const { return mask ? mask[i] != 0 : true; }
    __device__ __forceinline__ bool fix(long long) const { return false; }
    __device__ __forceinline__ void load(long long i, double* v) const {
#pragma unroll
        for (int d = 0; d < 3; ++d)
            if (d < D) v[d] = F[i * D + d];
    }
};

// The basin map's outputs, normalised on the fly: per point (amplitude, kept
// peak count, mean interval) -- the amplitude is the mean peak value, or the
// last recorded sample for a point without peaks -- min-max scaled per
// feature over the points with flag != 0: (f - lo) * (1 / (hi - lo)), 0 for a
// feature whose points are all equal.
struct BasinSrc {
    const int* flags;
    const int* counts;
    const double* avgPeaks;
    const double* avgIntervals;
    const double* last;
    double lo[3], inv[3];
    int ok[3];
    int D;
    __device__ __forceinline__ bool included(long long i) const { return flags[i] != 0; }
    __device__ __forceinline__ bool fix(long long) const { return false; }
    __device__ __forceinline__ void load(long long i, double* v) const {
        const int c = counts[i];
        const double f[3] = {c > 0 ? avgPeaks[i] : last[i], (double)c, c > 0 ? avgIntervals[i] : 0.0};
#pragma unroll
        for (int d = 0; d < 3; ++d) v[d] = ok[d] ? (f[d] - lo[d]) * inv[d] : 0.0;
    }
};

// ---- the cell table: slot-indexed statistics of the occupied cells ---------------
struct Table {
    unsigned long long* key;  // packed cell coordinates, kEmpty for a free slot
    unsigned long long mask;  // capacity - 1 (a power of two)
    int* cnt;                 // points
    unsigned* lo;             // 3 per slot: order keys of the feature minima rounded down to float
    unsigned* hi;             // 3 per slot: order keys of the feature maxima rounded up to float
    int* minIdx;              // smallest point index
    int* maxIdx;              // largest point index
    int* minFix;              // smallest fixed-point index (reference mode)
    int* bad;                 // a clamped or NaN point
};

__global__ void table_init_kernel(Table T, long long cap) {
    const long long h = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= cap) return;
    T.key[h] = kEmpty;
    T.cnt[h] = 0;
    for (int d = 0; d < 3; ++d) {
        T.lo[3 * h + d] = kFKeyPosInf;
        T.hi[3 * h + d] = kFKeyNegInf;
    }
    T.minIdx[h] = INT_MAX;
    T.maxIdx[h] = -1;
    T.minFix[h] = INT_MAX;
    T.bad[h] = 0;
}

__device__ __forceinline__ long long table_insert(unsigned long long* tab, unsigned long long mask,
                                                  unsigned long long k) {
    unsigned long long g = mix(k) & mask;
    for (unsigned long long probe = 0; probe <= mask; ++probe) {
        const unsigned long long prev = atomicCAS(&tab[g], kEmpty, k);
        if (prev == kEmpty || prev == k) return (long long)g;
        g = (g + 1) & mask;
    }
    return -1;  // only if the table were full (it has twice as many slots as cells)
}

__device__ __forceinline__ int hash_find(const unsigned long long* tab, unsigned long long mask, const int* slotCell,
                                         unsigned long long k) {
    unsigned long long h = mix(k) & mask;
    for (unsigned long long probe = 0; probe <= mask; ++probe) {
        const unsigned long long t = tab[h];
        if (t == k) return slotCell[h];
        if (t == kEmpty) return -1;
        h = (h + 1) & mask;
    }
    return -1;
}

// NaN test on the bits (the integer pipe; a double compare takes the FP64 pipe)
__device__ __forceinline__ bool is_nan(double v) {
    return ((unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull) > 0x7ff0000000000000ull;
}

// Cell coordinates of a feature vector; true when the point is clamped or NaN.
// q = f * (1/side): the rounding of the product (|q| < 2^19: below 1e-10 of a
// cell) stays far inside the 1e-9 by which the side is shrunk, so two points
// of one cell are still within eps. floor(q) is one conversion rounding down
// (saturating for infinities), clamped on the integer.
__device__ __forceinline__ bool cell_coords(const double* v, int D, double invSide, long long* c) {
    bool bad = false, nan = false;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        if (d >= D) continue;
        const double q = v[d] * invSide;
        nan = nan || is_nan(q);
        long long k = __double2ll_rd(q);
        if (k >= kLim) { k = kLim; bad = true; }
        else if (k < -kLim) { k = -kLim; bad = true; }
        c[d] = k;
    }
    if (nan) {
        c[0] = c[1] = c[2] = kLim + 5;
        return true;
    }
    return bad;
}

// Extent of the cell coordinates of the ordinary points (ext[d] = -min,
// ext[3 + d] = max) and the number of clamped or NaN ones (ext[6]): the
// occupied cells are at most the product of the extents plus that count,
// which sizes the table. Warps reduce with shuffles into shared memory, one
// global atomic per block and quantity. (Sources whose features have known
// bounds skip this pass.)
template <class Src>
__global__ void extent_kernel(Src S, long long n, double invSide, long long* ext) {
    __shared__ long long sext[7];
    if (threadIdx.x < 7) sext[threadIdx.x] = threadIdx.x < 6 ? LLONG_MIN : 0;
    __syncthreads();
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long c[3] = {0, 0, 0};
    bool bad = false, ok = false;
    if (i < n && S.included(i)) {
        double v[3];
        S.load(i, v);
        bad = cell_coords(v, S.D, invSide, c);
        ok = !bad;
    }
    const int lane = threadIdx.x & 31;
    const unsigned nbad = __popc(__ballot_sync(0xffffffffu, bad));
    if (lane == 0 && nbad) atomicAdd((unsigned long long*)&sext[6], (unsigned long long)nbad);
    if (__any_sync(0xffffffffu, ok)) {
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            if (d >= S.D) continue;
            long long lo = ok ? -c[d] : LLONG_MIN, hi = ok ? c[d] : LLONG_MIN;  // max of -c and of c
            for (int o = 16; o > 0; o >>= 1) {
                lo = max(lo, __shfl_xor_sync(0xffffffffu, lo, o));
                hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
            }
            if (lane == 0) {
                atomicMax(&sext[d], lo);
                atomicMax(&sext[3 + d], hi);
            }
        }
    }
    __syncthreads();
    if (threadIdx.x < 6 && sext[threadIdx.x] != LLONG_MIN) atomicMax(&ext[threadIdx.x], sext[threadIdx.x]);
    if (threadIdx.x == 6 && sext[6]) atomicAdd((unsigned long long*)&ext[6], (unsigned long long)sext[6]);
}

// The slot of a cell key: found by reading the table (no atomics once the
// cell is in it), inserted with atomicCAS otherwise.
__device__ __forceinline__ long long table_slot(unsigned long long* tab, unsigned long long mask,
                                                unsigned long long k) {
    unsigned long long g = mix(k) & mask;
    for (unsigned long long probe = 0; probe <= mask; ++probe) {
        const unsigned long long t = __ldcg(tab + g);
        if (t == k) return (long long)g;
        if (t == kEmpty) return table_insert(tab, mask, k);  // from here on, with atomics
        g = (g + 1) & mask;
    }
    return -1;
}

// Step 1, one point per thread. Consecutive grid points mostly share a cell,
// so a warp's lanes form runs of equal keys; each run's statistics are
// reduced to its first lane (warp-wide reductions when the whole row is one
// run, shuffles otherwise), which finds the slot (a read once the cell is in
// the table) and folds the run in with one 32-bit atomic per quantity: a
// run's smallest and largest index are its end lanes', its smallest
// fixed-point index and its clamped/NaN mark come from ballots, its box from
// the reductions. (Folding each block's runs into a shared-memory table
// first, or keeping extreme points as representatives with 64-bit atomics,
// measured slower on a 2048^2 basin map: 338 and 494 against 267 us.) Fout
// (basin maps, when the caller asks for the normalised features) receives
// each point's row.
template <class Src>
__global__ void __launch_bounds__(kTPB) cells_kernel(Src S, long long n, double invSide, Table T, int* slot,
                                                     double* Fout, int* err) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    unsigned long long key = kEmpty;
    double v[3] = {0.0, 0.0, 0.0};
    bool bad = false, fix = false;
    if (i < n && S.included(i)) {
        S.load(i, v);
        long long c[3] = {0, 0, 0};
        bad = cell_coords(v, S.D, invSide, c);
        key = pack(c, S.D);
        fix = S.fix(i);
    }
    if (Fout && i < n)
        for (int d = 0; d < 3; ++d) Fout[i * 3 + d] = v[d];
    // runs of equal keys: heads, and each lane's run [head, tail]
    const unsigned long long prevKey = __shfl_up_sync(0xffffffffu, key, 1);
    const unsigned heads = __ballot_sync(0xffffffffu, lane == 0 || prevKey != key);
    const unsigned upTo = 0xffffffffu >> (31 - lane);  // lanes 0..lane
    const int head = 31 - __clz(heads & upTo);
    const unsigned after = heads & ~upTo;               // heads above this lane
    const int tail = after ? __ffs(after) - 2 : 31;
    const bool isHead = lane == head;
    long long h = -1;
    if (isHead && key != kEmpty) {
        h = table_slot(T.key, T.mask, key);
        if (h < 0) atomicAdd(err, 1);
    }
    h = __shfl_sync(0xffffffffu, h, head);
    if (i < n) slot[i] = key == kEmpty || h < 0 ? -1 : (int)h;
    // box (float, rounded outward), reduced toward the head
    unsigned lo[3], hi[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const bool skip = d >= S.D || is_nan(v[d]) || key == kEmpty;
        lo[d] = skip ? kFKeyPosInf : fkey(__double2float_rd(v[d]));
        hi[d] = skip ? kFKeyNegInf : fkey(__double2float_ru(v[d]));
    }
    if (heads == 1u) {  // the whole row is one run (the common case)
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            if (d >= S.D) continue;
            lo[d] = __reduce_min_sync(0xffffffffu, lo[d]);
            hi[d] = __reduce_max_sync(0xffffffffu, hi[d]);
        }
    } else {
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const bool in = lane + o <= tail;
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                if (d >= S.D) continue;
                const unsigned a = __shfl_down_sync(0xffffffffu, lo[d], o);
                const unsigned b = __shfl_down_sync(0xffffffffu, hi[d], o);
                if (in) {
                    lo[d] = a < lo[d] ? a : lo[d];
                    hi[d] = b > hi[d] ? b : hi[d];
                }
            }
        }
    }
    const unsigned fixes = __ballot_sync(0xffffffffu, fix);
    const unsigned bads = __ballot_sync(0xffffffffu, bad);
    if (!isHead || key == kEmpty || h < 0) return;
    const unsigned run = (tail == 31 ? 0xffffffffu : ((1u << (tail + 1)) - 1u)) & ~((1u << head) - 1u);
    const long long base = i - lane;  // index of lane 0
    atomicAdd(&T.cnt[h], tail - head + 1);
    atomicMin(&T.minIdx[h], (int)i);
    atomicMax(&T.maxIdx[h], (int)(base + tail));
    if (fixes & run) atomicMin(&T.minFix[h], (int)(base + __ffs(fixes & run) - 1));
    if (bads & run) atomicOr(&T.bad[h], 1);
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        if (d >= S.D) continue;
        atomicMin(&T.lo[3 * h + d], lo[d]);
        atomicMax(&T.hi[3 * h + d], hi[d]);
    }
}

__global__ void occupied_kernel(const unsigned long long* tab, long long cap, int* occ) {
    const long long h = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (h < cap) occ[h] = tab[h] != kEmpty;
}

__global__ void cell_ids_kernel(const unsigned long long* tab, long long cap, const int* occScan, int* slotCell,
                                unsigned long long* cellKey, int* cellSlot) {
    const long long h = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= cap) return;
    if (tab[h] != kEmpty) {
        const int c = occScan[h];
        slotCell[h] = c;
        cellKey[c] = tab[h];
        cellSlot[c] = (int)h;
    } else {
        slotCell[h] = -1;
    }
}

// ---- step 2: cells -------------------------------------------------------------
struct Cells {
    int C, D;
    const unsigned long long* key;
    int* cnt;
    double* lo;  // 3 per cell
    double* hi;
    unsigned char* unsafe;  // clamped / NaN points (or eps == 0): exact point tests only
    unsigned char* dense;   // safe, and every point core
    int* minIdx;
    int* minFix;
    double* repV;  // kReps x 3 per cell
    int* repN;
    int* hasCore;  // a core point (safe cells)
    int* minCore;  // smallest core index (safe cells that are not dense)
    int* sb;       // sorted range [sb, se) (empty for a cell that was not sorted)
    int* se;
    int* need;     // to be sorted in the second pass
};

template <class Src>
__global__ void finalize_kernel(Src S, Cells K, const int* cellSlot, Table T, int compat, int zeroEps, int minPts) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= K.C) return;
    const long long h = cellSlot[c];
    const int n = T.cnt[h];
    K.cnt[c] = n;
    for (int d = 0; d < 3; ++d) {
        K.lo[3 * c + d] = d < K.D ? (double)unfkey(T.lo[3 * h + d]) : 0.0;
        K.hi[3 * c + d] = d < K.D ? (double)unfkey(T.hi[3 * h + d]) : 0.0;
    }
    const bool unsafe = T.bad[h] != 0 || zeroEps;
    const bool dense = !unsafe && (compat || n >= minPts);
    K.unsafe[c] = unsafe ? 1 : 0;
    K.dense[c] = dense ? 1 : 0;
    K.minIdx[c] = T.minIdx[h];
    K.minFix[c] = T.minFix[h];
    K.hasCore[c] = dense ? 1 : 0;
    K.minCore[c] = INT_MAX;
    K.sb[c] = 0;
    K.se[c] = 0;
    K.need[c] = 0;
    int idx[kReps], m = 0;
    idx[m++] = T.minIdx[h];
    if (T.maxIdx[h] != T.minIdx[h]) idx[m++] = T.maxIdx[h];
    K.repN[c] = m;
    for (int j = 0; j < m; ++j) {
        double v[3] = {0.0, 0.0, 0.0};
        S.load(idx[j], v);
        for (int d = 0; d < 3; ++d) K.repV[((long long)c * kReps + j) * 3 + d] = v[d];
    }
}

// Warp per cell: number (pass 0) or list (pass 1) of its occupied neighbour
// cells, the lanes looking up 32 of the (2R+1)^D - 1 offsets at a time (in
// the order dx, dy, dz).
__global__ void neighbours_kernel(const unsigned long long* cellKey, int C, int D, const unsigned long long* tab,
                                  unsigned long long mask, const int* slotCell, int* nbCount, const int* nbStart,
                                  int* nbList, int* nbOwner) {
    const long long c = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (c >= C) return;
    long long base[3];
    unpack(cellKey[c], D, base);
    const int ry = D >= 2 ? kR : 0, rz = D >= 3 ? kR : 0;
    const int ny = 2 * ry + 1, nz = 2 * rz + 1, total = (2 * kR + 1) * ny * nz;
    const int w0 = nbStart ? nbStart[c] : 0;
    int k = 0;
    for (int o0 = 0; o0 < total; o0 += 32) {
        const int o = o0 + lane;
        int c2 = -1;
        if (o < total) {
            const int dz = o % nz - rz, dy = (o / nz) % ny - ry, dx = o / (nz * ny) - kR;
            if (dx != 0 || dy != 0 || dz != 0) {
                long long q[3] = {base[0] + dx, base[1] + dy, base[2] + dz};
                c2 = hash_find(tab, mask, slotCell, pack(q, D));
            }
        }
        const unsigned m = __ballot_sync(0xffffffffu, c2 >= 0);
        if (nbList && c2 >= 0) {
            const int pos = w0 + k + __popc(m & ((1u << lane) - 1u));
            nbList[pos] = c2;
            nbOwner[pos] = (int)c;
        }
        k += __popc(m);
    }
    if (!nbList && lane == 0) nbCount[c] = k;
}

// Pair states (one per neighbour entry with owner < neighbour).
enum : unsigned char {
    kFar = 0,       // boxes farther than eps apart (or the mirrored entry)
    kJoined = 1,    // settled: joined, or already in one component
    kDenseOpen = 2, // two dense cells the shortcuts did not join
    kWhole = 3,     // every point of one within eps of every point of the other (a cell not dense)
    kPoints = 4,    // point tests (a cell not dense or unsafe, boxes partly within eps)
    kDensePts = 5,  // two dense cells still apart after the shortcuts: point tests
};

__device__ __forceinline__ void pair_boxes(const Cells& K, int a, int b, double& gap2, double& span2) {
    const double* loA = K.lo + 3 * (long long)a;
    const double* hiA = K.hi + 3 * (long long)a;
    const double* loB = K.lo + 3 * (long long)b;
    const double* hiB = K.hi + 3 * (long long)b;
    gap2 = 0.0;
    span2 = 0.0;
    for (int d = 0; d < K.D; ++d) {
        double g = 0.0;
        if (hiA[d] < loB[d]) g = loB[d] - hiA[d];
        else if (hiB[d] < loA[d]) g = loA[d] - hiB[d];
        gap2 = gap2 + g * g;
        const double f = fmax(hiA[d], hiB[d]) - fmin(loA[d], loB[d]);
        span2 = span2 + f * f;
    }
}

// a representative of cell b within eps of v
__device__ __forceinline__ bool rep_within(const Cells& K, int b, const double* v, double eps) {
    for (int j = 0; j < K.repN[b]; ++j)
        if (within_eps(dist2(v, K.repV + ((long long)b * kReps + j) * 3, K.D), eps)) return true;
    return false;
}

// Thread per neighbour entry (owner < neighbour): the box tests; pairs of
// dense cells that the boxes leave open are listed for the representatives.
__global__ void pair_kernel(Cells K, const int* nbOwner, const int* nbList, long long E, double eps,
                            unsigned char* st, int* open, int* nOpen, int* joined, int* nJoined) {
    const long long w = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    bool take = false, join = false;
    if (w < E) {
        const int a = nbOwner[w], b = nbList[w];
        unsigned char state = kFar;
        if (b > a) {
            const double eps2 = eps * eps;
            double gap2, span2;
            pair_boxes(K, a, b, gap2, span2);
            if (gap2 > eps2 * kBoxOut) state = kFar;
            else if (K.dense[a] && K.dense[b]) {
                if (span2 < eps2 * kBoxIn) {
                    state = kJoined;  // joined by cell_components_kernel
                    join = true;
                } else {
                    state = kDenseOpen;
                    take = true;
                }
            } else {
                state = !K.unsafe[a] && !K.unsafe[b] && span2 < eps2 * kBoxIn ? kWhole : kPoints;
            }
        }
        st[w] = state;
    }
    list_append(take, (int)w, open, nOpen);
    list_append(join, (int)w, joined, nJoined);
}

// Warp per listed pair of dense cells: the lanes share the representative
// pairs; one within eps marks the two cells joined.
__global__ void rep_pairs_kernel(Cells K, const int* nbOwner, const int* nbList, const int* open, int nOpen,
                                 double eps, unsigned char* st, int* joined, int* nJoined) {
    const long long wi = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (wi >= nOpen) return;
    const int w = open[wi];
    const int a = nbOwner[w], b = nbList[w];
    const int na = K.repN[a], nb = K.repN[b];
    bool hit = false;
    for (int k = lane; k < na * nb && !hit; k += 32) {
        const double* ra = K.repV + ((long long)a * kReps + k / nb) * 3;
        const double* rb = K.repV + ((long long)b * kReps + k % nb) * 3;
        hit = within_eps(dist2(ra, rb, K.D), eps);
    }
    if (__any_sync(0xffffffffu, hit) && lane == 0) {
        st[w] = kJoined;
        joined[atomicAdd(nJoined, 1)] = w;
    }
}

// The components of the dense cells over the joined pairs. Thousands of
// concurrent unions into one growing component make a global union-find
// chase pointers through L2; with up to kSharedCells cells one block runs it
// in shared memory (hooking with atomicCAS, path halving) and writes every
// cell's root, so later finds take one step. joinAll: the same over the
// global array, a thread per entry (more cells).
constexpr int kSharedCells = 40960;

__device__ __forceinline__ int sh_find(int* par, int x) {
    int cur = par[x];
    if (cur != x) {
        int prev = x, next;
        while (cur > (next = par[cur])) {
            par[prev] = next;
            prev = cur;
            cur = next;
        }
    }
    return cur;
}

__global__ void __launch_bounds__(1024) cell_components_kernel(int C, const int* nbOwner, const int* nbList,
                                                               const int* joined, const int* nJoined, int* parent) {
    extern __shared__ int par[];
    for (int v = threadIdx.x; v < C; v += blockDim.x) par[v] = v;
    __syncthreads();
    const int J = *nJoined;
    for (int k = threadIdx.x; k < J; k += blockDim.x) {
        const int e = joined[k];
        int ra = sh_find(par, nbOwner[e]), rb = sh_find(par, nbList[e]);
        while (ra != rb) {
            if (ra < rb) { const int t = ra; ra = rb; rb = t; }
            const int old = atomicCAS(par + ra, ra, rb);
            if (old == ra) break;
            ra = sh_find(par, old);
            rb = sh_find(par, rb);
        }
    }
    __syncthreads();
    for (int v = threadIdx.x; v < C; v += blockDim.x) parent[v] = sh_find(par, v);
}

__global__ void join_all_kernel(const int* nbOwner, const int* nbList, const int* joined, const int* nJoined,
                                int* parent) {
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < *nJoined) uf_unite(parent, nbOwner[joined[k]], nbList[joined[k]]);
}

// ---- step 3: sorting ----------------------------------------------------------
// Counting sort of the points of the cells with begin[c] >= 0 (one phase):
// one pass over the slots; only those points' features are read.
struct Sorted {
    double* s[3];
    int* order;
    int* cell;
    unsigned char* core;  // 0 / 1, 2 = not decided yet
    unsigned char* fix;   // reference mode
    const int* sb;
    const int* se;
    int D;
    __device__ __forceinline__ void load(int pos, double* v) const {
#pragma unroll
        for (int d = 0; d < 3; ++d)
            if (d < D) v[d] = s[d][pos];
    }
};

template <class Src>
__global__ void sort_kernel(Src S, long long n, const int* slot, const int* slotCell, const int* begin, int* cursor,
                            Sorted Q, const unsigned char* dense, int compat) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    const int h = i < n ? slot[i] : -1;
    const int c0 = h >= 0 ? slotCell[h] : -1;
    const int base = c0 >= 0 ? begin[c0] : -1;
    const int c = base >= 0 ? c0 : -1;
    const unsigned grp = __match_any_sync(0xffffffffu, c);
    const int leader = __ffs(grp) - 1;
    int off = 0;
    if (c >= 0 && lane == leader) off = atomicAdd(&cursor[c], __popc(grp));
    off = __shfl_sync(0xffffffffu, off, leader);
    if (c < 0) return;
    const int pos = base + off + __popc(grp & ((1u << lane) - 1u));
    Q.order[pos] = (int)i;
    Q.cell[pos] = c;
    double v[3] = {0.0, 0.0, 0.0};
    S.load(i, v);
#pragma unroll
    for (int d = 0; d < 3; ++d)
        if (d < Q.D) Q.s[d][pos] = v[d];
    Q.core[pos] = compat || dense[c] ? 1 : 0;
    if (Q.fix) Q.fix[pos] = S.fix(i) ? 1 : 0;
}

__global__ void phase_begin_kernel(int C, const int* scan, const int* take, int offset, int* begin, int* sb, int* se,
                                   const int* cnt) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= C) return;
    if (take[c]) {
        begin[c] = offset + scan[c];
        sb[c] = offset + scan[c];
        se[c] = offset + scan[c] + cnt[c];
    } else {
        begin[c] = -1;
    }
}

__global__ void take_sparse_kernel(Cells K, int* take) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c < K.C) take[c] = K.dense[c] ? 0 : K.cnt[c];
}

__global__ void take_needed_kernel(Cells K, int* take) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c < K.C) take[c] = K.need[c] && K.se[c] == K.sb[c] ? K.cnt[c] : 0;
}

// ---- step 3/4: point-level work on the sorted points ---------------------------------
// node of sorted point p in cell c: the cell for a safe cell, C + p otherwise
__device__ __forceinline__ int node_of(const Cells& K, int c, int p) { return K.unsafe[c] ? K.C + p : c; }

__device__ __forceinline__ bool sorted_cell(const Sorted& Q, int c) { return Q.se[c] > Q.sb[c]; }

// Warp per sorted point of a cell that is not dense (textbook mode), in
// [0, M1): the lanes classify the neighbour cells (at most 124, four per
// lane) by their boxes -- beyond eps: nothing; wholly within eps: counted
// whole; partly: scanned if sorted, otherwise (a dense cell) its
// representatives within eps counted, a lower bound -- then the sorted cells
// are scanned 32 points at a time until minPts. A point that stays below
// minPts with a lower-bound cell is left undecided (core = 2) and those cells
// are marked for the second sort. redo: only the undecided points, counted
// exactly; one found core joins the dense cells wholly within eps of it.
constexpr int kNbPerLane = 4;  // (2R+1)^3 - 1 = 124 neighbour cells at most

__global__ void core_kernel(Sorted Q, Cells K, const int* nbStart, const int* nbList, int M1, double eps, int minPts,
                            int redo, int* parent) {
    const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= M1) return;
    const int p = (int)w;
    if (redo && Q.core[p] != 2) return;
    const int c = Q.cell[p];
    double me[3] = {0, 0, 0};
    Q.load(p, me);
    const double eps2 = eps * eps;
    const int e0 = nbStart[c], e1 = nbStart[c + 1];
    int cls[kNbPerLane];  // 0 nothing, 1 whole, 2 scan, 3 representatives (a lower bound)
    int local = 0;
    bool lower = false;
#pragma unroll
    for (int j = 0; j < kNbPerLane; ++j) {
        const int e = e0 + lane + 32 * j;
        cls[j] = 0;
        if (e >= e1) continue;
        const int b = nbList[e];
        if (K.unsafe[b]) {
            cls[j] = 2;
            continue;
        }
        double near2, far2;
        box_dist2(me, K.lo + 3 * (long long)b, K.hi + 3 * (long long)b, K.D, near2, far2);
        if (near2 > eps2 * kBoxOut) continue;
        if (far2 < eps2 * kBoxIn) {
            cls[j] = 1;
            local += K.cnt[b];
            continue;
        }
        if (sorted_cell(Q, b)) {
            cls[j] = 2;
            continue;
        }
        cls[j] = 3;
        lower = true;
        for (int r = 0; r < K.repN[b]; ++r)
            if (within_eps(dist2(me, K.repV + ((long long)b * kReps + r) * 3, K.D), eps)) ++local;
    }
    int cnt = (K.unsafe[c] ? 0 : K.cnt[c]) + (int)__reduce_add_sync(0xffffffffu, (unsigned)local);
    const bool inexact = __any_sync(0xffffffffu, lower);
    auto scan_cell = [&](int cell) {
        const int end = Q.se[cell];
        for (int q0 = Q.sb[cell]; q0 < end && cnt < minPts; q0 += 32) {
            const int q = q0 + lane;
            bool hit = false;
            if (q < end) {
                double v[3];
                Q.load(q, v);
                hit = within_eps(dist2(me, v, K.D), eps);
            }
            cnt += __popc(__ballot_sync(0xffffffffu, hit));
        }
    };
    if (K.unsafe[c] && cnt < minPts) scan_cell(c);
#pragma unroll
    for (int j = 0; j < kNbPerLane; ++j) {
        unsigned m = __ballot_sync(0xffffffffu, cls[j] == 2);
        while (m && cnt < minPts) {
            const int src = __ffs(m) - 1;
            m &= m - 1;
            scan_cell(nbList[e0 + src + 32 * j]);
        }
    }
    const int core = cnt >= minPts ? 1 : (inexact && !redo ? 2 : 0);
    if (lane == 0) {
        Q.core[p] = (unsigned char)core;
        if (core == 1 && !K.unsafe[c]) {
            atomicOr(&K.hasCore[c], 1);
            atomicMin(&K.minCore[c], Q.order[p]);
        }
    }
#pragma unroll
    for (int j = 0; j < kNbPerLane; ++j) {
        if (cls[j] == 3 && core == 2) K.need[nbList[e0 + lane + 32 * j]] = 1;  // to be sorted
        if (cls[j] == 1 && redo && core == 1 && K.dense[nbList[e0 + lane + 32 * j]])
            uf_unite(parent, node_of(K, c, p), nbList[e0 + lane + 32 * j]);
    }
}

// Warp per sorted point of a cell that is not dense, in [0, M1), after the
// core flags, lanes over the neighbour cells: a core point of a safe cell
// joins its cell to every dense neighbour that is whole within eps of it or
// holds a representative within eps; an entry (cell -> dense neighbour) that
// none of the cell's core points settled that way is marked open. A point
// that is not core marks the dense neighbours its border label would have to
// scan (partly within eps, no representative within eps), and a point of an
// unsafe cell every dense neighbour within reach: those are sorted in the
// second pass.
__global__ void dense_links_kernel(Sorted Q, Cells K, const int* nbStart, const int* nbList, int M1, double eps,
                                   int* parent, unsigned char* openE, unsigned char* settledE) {
    const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= M1) return;
    const int p = (int)w;
    const int c = Q.cell[p];
    const int core = Q.core[p];
    if (core == 2) return;  // its neighbours are sorted in the second pass
    double me[3] = {0, 0, 0};
    Q.load(p, me);
    const double eps2 = eps * eps;
    for (int e = nbStart[c] + lane; e < nbStart[c + 1]; e += 32) {
        const int b = nbList[e];
        if (!K.dense[b]) continue;
        double near2, far2;
        box_dist2(me, K.lo + 3 * (long long)b, K.hi + 3 * (long long)b, K.D, near2, far2);
        if (near2 > eps2 * kBoxOut) continue;
        if (K.unsafe[c]) {
            K.need[b] = 1;
            continue;
        }
        const bool reach = far2 < eps2 * kBoxIn || rep_within(K, b, me, eps);
        if (core == 1) {
            if (reach) {
                uf_unite(parent, c, b);
                settledE[e] = 1;
            } else {
                openE[e] = 1;
            }
        } else if (!reach) {
            K.need[b] = 1;
        }
    }
}

// Entry pass after the shortcuts' unions: two dense cells still apart, and
// open entries of a cell whose core points did not reach a dense neighbour,
// get point tests (both cells sorted) when they are in two components; pairs
// with an unsafe cell are tested point by point.
__global__ void open_pairs_kernel(Cells K, const int* nbOwner, const int* nbList, long long E, int* parent,
                                  unsigned char* st, const unsigned char* openE, const unsigned char* settledE) {
    const long long w = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= E) return;
    const int a = nbOwner[w], b = nbList[w];
    if (st[w] == kDenseOpen) {
        if (uf_find(parent, a) != uf_find(parent, b)) {
            st[w] = kDensePts;
            K.need[a] = 1;
            K.need[b] = 1;
        } else {
            st[w] = kJoined;
        }
    }
    if (openE[w] && !settledE[w] && uf_find(parent, a) != uf_find(parent, b)) K.need[b] = 1;
    if (st[w] == kPoints && (K.unsafe[a] || K.unsafe[b])) {
        K.need[a] = 1;
        K.need[b] = 1;
    }
}

// ---- step 5: unions ------------------------------------------------------------

__global__ void whole_pairs_kernel(Cells K, const int* nbOwner, const int* nbList, long long E,
                                   const unsigned char* st, int* parent) {
    const long long w = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= E || st[w] != kWhole) return;
    const int a = nbOwner[w], b = nbList[w];
    if (K.hasCore[a] && K.hasCore[b]) uf_unite(parent, a, b);
}

// warp per unsafe cell: exact pair tests between its core points
__global__ void unsafe_cell_kernel(Sorted Q, Cells K, double eps, int* parent) {
    const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= K.C || !K.unsafe[w]) return;
    const int b = Q.sb[w], e = Q.se[w];
    for (int p = b; p < e; ++p) {
        if (Q.core[p] != 1) continue;
        double a[3];
        Q.load(p, a);
        for (int q = p + 1 + lane; q < e; q += 32) {
            if (Q.core[q] != 1) continue;
            double v[3];
            Q.load(q, v);
            if (within_eps(dist2(a, v, K.D), eps)) uf_unite(parent, K.C + p, K.C + q);
        }
    }
}

// warp per entry in state kPoints / kDensePts whose two cells are sorted:
// unite the two cells' core points if any core pair is within eps. The
// smaller cell's points are walked one by one, the larger cell's 32 at a
// time.
//
// Three passes of growing budget. Pass 0 probes every pair with a small
// amount of work (kPassOuter points of the smaller cell against kPassChunks
// x 32 points of the larger one) and marks the pairs it could not settle;
// each later pass takes the marked pairs only, first skips those whose two
// cells earlier unions already put into one component, and the last pass
// scans exhaustively. The components found do not depend on the order of
// the unions.
constexpr int kCrossPasses = 3;
__constant__ int kPassOuter[kCrossPasses] = {2, 32, 0x7fffffff};
__constant__ int kPassChunks[kCrossPasses] = {2, 8, 0x7fffffff};

__global__ void cross_cell_kernel(Sorted Q, Cells K, const int* nbOwner, const int* nbList, long long E,
                                  const unsigned char* st, double eps, int* parent, int pass, unsigned char* deferred) {
    const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= E) return;
    if (st[w] != kPoints && st[w] != kDensePts) return;
    int ca = nbOwner[w], cb = nbList[w];
    if (!sorted_cell(Q, ca) || !sorted_cell(Q, cb)) return;
    const bool last = pass == kCrossPasses - 1;
    if (pass > 0) {
        const bool todo = deferred[w] != 0;
        __syncwarp();  // every lane has read the mark before lane 0 clears it
        if (!todo) return;
        if (lane == 0) deferred[w] = 0;
    }
    const bool safe = !K.unsafe[ca] && !K.unsafe[cb];
    if (safe && (!K.hasCore[ca] || !K.hasCore[cb])) return;
    if (!safe && !last) {  // unsafe cells unite every core pair within eps: last pass only
        if (lane == 0) deferred[w] = 1;
        return;
    }
    if (safe && uf_find(parent, ca) == uf_find(parent, cb)) return;
    const double eps2 = eps * eps;
    double gap2, span2;
    pair_boxes(K, ca, cb, gap2, span2);
    if (gap2 > eps2 * kBoxOut) return;
    if (Q.se[ca] - Q.sb[ca] > Q.se[cb] - Q.sb[cb]) {
        const int t = ca;
        ca = cb;
        cb = t;
    }
    const double* lo = K.lo + 3 * (long long)cb;
    const double* hi = K.hi + 3 * (long long)cb;
    int outerLeft = kPassOuter[pass];
    const int chunkBudget = kPassChunks[pass];
    bool cut = false, stop = false;
    const int endA = Q.se[ca], endB = Q.se[cb];
    for (int p0 = Q.sb[ca]; p0 < endA && !stop; p0 += 32) {
        const int p = p0 + lane;
        double a[3] = {0, 0, 0};
        bool inReach = false, allIn = false;
        if (p < endA && Q.core[p] == 1) {
            Q.load(p, a);
            double near2, far2;
            box_dist2(a, lo, hi, K.D, near2, far2);
            inReach = near2 <= eps2 * kBoxOut;
            allIn = safe && far2 < eps2 * kBoxIn;
        }
        const unsigned mAll = __ballot_sync(0xffffffffu, inReach && allIn);
        if (mAll) {  // every core point of cb is within eps of this one
            if (lane == __ffs(mAll) - 1) uf_unite(parent, ca, cb);
            return;
        }
        unsigned todo = __ballot_sync(0xffffffffu, inReach);
        while (todo) {
            const int src = __ffs(todo) - 1;
            todo &= todo - 1;
            if (outerLeft-- == 0) {
                cut = stop = true;
                break;
            }
            const int pp = p0 + src;
            double aa[3];
            for (int d = 0; d < 3; ++d) aa[d] = __shfl_sync(0xffffffffu, a[d], src);
            int chunks = 0;
            for (int q0 = Q.sb[cb]; q0 < endB; q0 += 32) {
                if (chunks++ == chunkBudget) {
                    cut = true;
                    break;
                }
                const int q = q0 + lane;
                bool hit = false;
                if (q < endB && Q.core[q] == 1) {
                    double v[3];
                    Q.load(q, v);
                    hit = within_eps(dist2(aa, v, K.D), eps);
                }
                const unsigned bal = __ballot_sync(0xffffffffu, hit);
                if (bal) {
                    if (safe) {
                        if (lane == __ffs(bal) - 1) uf_unite(parent, ca, cb);
                        return;
                    }
                    if (hit) uf_unite(parent, node_of(K, ca, pp), node_of(K, cb, q));
                }
            }
        }
    }
    if (cut && lane == 0) deferred[w] = 1;
}

// ---- step 6: components and labels ------------------------------------------------
__global__ void iota_kernel(int* p, long long n) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = (int)i;
}

__global__ void fill_kernel(int* p, long long n, int v) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = v;
}

// node's smallest core (and fixed-point) index, folded into its component's root
__device__ __forceinline__ bool node_keys(const Sorted& Q, const Cells& K, int v, int& key, int& fixKey) {
    if (v < K.C) {
        if (K.unsafe[v] || !K.hasCore[v]) return false;
        key = K.dense[v] ? K.minIdx[v] : K.minCore[v];
        fixKey = K.minFix[v];
        return true;
    }
    const int p = v - K.C;
    if (!K.unsafe[Q.cell[p]] || Q.core[p] != 1) return false;
    key = Q.order[p];
    fixKey = Q.fix && Q.fix[p] ? Q.order[p] : INT_MAX;
    return true;
}

__global__ void comp_kernel(Sorted Q, Cells K, long long N, int* parent, int* compMin, int* compFix) {
    const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= N) return;
    int key, fixKey;
    if (!node_keys(Q, K, (int)v, key, fixKey)) return;
    const int r = uf_find(parent, (int)v);
    atomicMin(&compMin[r], key);
    if (fixKey != INT_MAX) atomicMin(&compFix[r], fixKey);
}

__global__ void roots_kernel(Sorted Q, Cells K, long long N, int* parent, const int* compMin, const int* compFix,
                             int* rootList, int* rootMin, int* rootFix, int* nRoots) {
    const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    bool take = false;
    int key, fixKey;
    if (v < N && node_keys(Q, K, (int)v, key, fixKey)) take = uf_find(parent, (int)v) == (int)v;
    const unsigned m = __ballot_sync(0xffffffffu, take);
    if (!m) return;
    const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(nRoots, __popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (!take) return;
    const int k = base + __popc(m & ((1u << lane) - 1));
    rootList[k] = (int)v;
    rootMin[k] = compMin[v];
    rootFix[k] = compFix[v];
}

__global__ void scatter_labels_kernel(const int* rootList, const int* lab, int K, int* compLabel) {
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < K) compLabel[rootList[k]] = lab[k];
}

// Numbering on the device for many components: marks over the point indices,
// then prefix sums (textbook: by smallest core index; reference: fixed-point
// components by their smallest fixed-point index, the others by smallest index).
__global__ void rank_marks_kernel(const int* rootMin, const int* rootFix, int K, int compat, int* markMin,
                                  int* markFix) {
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= K) return;
    if (compat && rootFix[k] != INT_MAX) markFix[rootFix[k]] = 1;
    else markMin[rootMin[k]] = 1;
}

__global__ void rank_labels_kernel(const int* rootList, const int* rootMin, const int* rootFix, int K, int compat,
                                   const int* rankMin, const int* rankFix, int* compLabel) {
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= K) return;
    int lab;
    if (compat) lab = rootFix[k] != INT_MAX ? -(rankFix[rootFix[k]] + 1) : rankMin[rootMin[k]] + 1;
    else lab = rankMin[rootMin[k]];
    compLabel[rootList[k]] = lab;
}

__global__ void cell_labels_kernel(Cells K, int* parent, const int* compLabel, int* cellLabel) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= K.C) return;
    cellLabel[c] = !K.unsafe[c] && K.hasCore[c] ? compLabel[uf_find(parent, (int)c)] : -1;
}

// one pass over the slots: excluded points, and every point of a dense cell
__global__ void labels_kernel(const int* slot, const int* slotCell, long long n, const unsigned char* dense,
                              const int* cellLabel, int compat, int* labels) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int h = slot[i];
    if (h < 0) {
        labels[i] = compat ? 0 : -2;
        return;
    }
    const int c = slotCell[h];
    if (dense[c]) labels[i] = cellLabel[c];
}

// Warp per sorted point of a cell that is not dense, in [0, M1): a core
// point takes its component's label; a border point the component with the
// smallest core index among the core points within eps (lanes settle the
// neighbour cells by box or representatives, the rest are scanned by the
// warp, a safe cell only while it could still lower the answer); the rest
// are noise (-1).
__global__ void sorted_labels_kernel(Sorted Q, Cells K, const int* nbStart, const int* nbList, int M1, double eps,
                                     int* parent, const int* compMin, const int* compLabel, int* labels) {
    const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= M1) return;
    const int p = (int)w;
    const int c = Q.cell[p];
    if (Q.core[p] == 1) {
        if (lane == 0) labels[Q.order[p]] = compLabel[uf_find(parent, node_of(K, c, p))];
        return;
    }
    double me[3] = {0, 0, 0};
    Q.load(p, me);
    const double eps2 = eps * eps;
    const int e0 = nbStart[c], e1 = nbStart[c + 1];
    // candidates as (smallest core index of the component, root): the smallest wins
    auto key_of = [&](int r) { return ((unsigned long long)(unsigned)compMin[r] << 32) | (unsigned)r; };
    unsigned long long best = ~0ull;
    if (lane == 0 && !K.unsafe[c] && K.hasCore[c]) best = key_of(uf_find(parent, c));  // own cell: within eps
    bool scanIt[kNbPerLane];
#pragma unroll
    for (int j = 0; j < kNbPerLane; ++j) {
        const int e = e0 + lane + 32 * j;
        scanIt[j] = false;
        if (e >= e1) continue;
        const int b = nbList[e];
        if (K.unsafe[b]) {
            scanIt[j] = true;
            continue;
        }
        if (!K.hasCore[b]) continue;
        double near2, far2;
        box_dist2(me, K.lo + 3 * (long long)b, K.hi + 3 * (long long)b, K.D, near2, far2);
        if (near2 > eps2 * kBoxOut) continue;
        if (far2 < eps2 * kBoxIn || (K.dense[b] && rep_within(K, b, me, eps))) {
            const unsigned long long k = key_of(uf_find(parent, b));
            best = k < best ? k : best;
            continue;
        }
        scanIt[j] = true;  // sorted: a dense cell here was marked for the second pass
    }
    best = group_min64(0xffffffffu, best);
    auto scan = [&](int cell) {
        const int end = Q.se[cell];
        if (!K.unsafe[cell]) {  // all its core points share one root
            const unsigned long long k = key_of(uf_find(parent, cell));
            if (k >= best) return;
            for (int q0 = Q.sb[cell]; q0 < end; q0 += 32) {
                const int q = q0 + lane;
                bool hit = false;
                if (q < end && Q.core[q] == 1) {
                    double v[3];
                    Q.load(q, v);
                    hit = within_eps(dist2(me, v, K.D), eps);
                }
                if (__any_sync(0xffffffffu, hit)) {
                    best = k;
                    return;
                }
            }
            return;
        }
        for (int q0 = Q.sb[cell]; q0 < end; q0 += 32) {
            const int q = q0 + lane;
            unsigned long long k = ~0ull;
            if (q < end && Q.core[q] == 1) {
                double v[3];
                Q.load(q, v);
                if (within_eps(dist2(me, v, K.D), eps)) k = key_of(uf_find(parent, node_of(K, cell, q)));
            }
            k = group_min64(0xffffffffu, k);
            best = k < best ? k : best;
        }
    };
    if (K.unsafe[c]) scan(c);
#pragma unroll
    for (int j = 0; j < kNbPerLane; ++j) {
        unsigned m = __ballot_sync(0xffffffffu, scanIt[j]);
        while (m) {
            const int src = __ffs(m) - 1;
            m &= m - 1;
            scan(nbList[e0 + src + 32 * j]);
        }
    }
    if (lane == 0) labels[Q.order[p]] = best == ~0ull ? -1 : compLabel[(int)(best & 0xffffffffull)];
}

#define CK(x)                                                   \
    do {                                                        \
        cudaError_t e_ = (x);                                   \
        if (e_ != cudaSuccess) return cuda_error(e_, #x);       \
    } while (0)
#define CKL() CK(cudaGetLastError())
#define NEED(p) \
    if (!(p)) return CHAOS_E_NOMEM

// Components numbered on the host when there are few (their keys copied
// back), on the device otherwise.
constexpr int kHostRankMax = 1 << 18;

int number_components(Call& c, long long n, int K, bool compat, const int* rootList, const int* rootMin,
                      const int* rootFix, int* compLabel) {
    cudaStream_t st = c.stream;
    if (K <= 0) return CHAOS_OK;
    if (K <= kHostRankMax) {
        std::vector<int> hMin(K), hFix(K), lab(K), idx(K);
        CK(cudaMemcpyAsync(hMin.data(), rootMin, K * sizeof(int), cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(hFix.data(), rootFix, K * sizeof(int), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        for (int k = 0; k < K; ++k) idx[k] = k;
        if (compat) {
            // fixed-point components by smallest fixed-point index (-1, -2, ...), the others by smallest index
            std::vector<int> neg, pos;
            for (int k = 0; k < K; ++k) (hFix[k] != INT_MAX ? neg : pos).push_back(k);
            std::sort(neg.begin(), neg.end(), [&](int a, int b) { return hFix[a] < hFix[b]; });
            std::sort(pos.begin(), pos.end(), [&](int a, int b) { return hMin[a] < hMin[b]; });
            for (size_t r = 0; r < neg.size(); ++r) lab[neg[r]] = -(int)(r + 1);
            for (size_t r = 0; r < pos.size(); ++r) lab[pos[r]] = (int)(r + 1);
        } else {
            std::sort(idx.begin(), idx.end(), [&](int a, int b) { return hMin[a] < hMin[b]; });
            for (int r = 0; r < K; ++r) lab[idx[r]] = r;
        }
        int* dLab = (int*)c.alloc((size_t)K * sizeof(int));
        NEED(dLab);
        CK(cudaMemcpyAsync(dLab, lab.data(), K * sizeof(int), cudaMemcpyHostToDevice, st));
        scatter_labels_kernel<<<blocks(K), kTPB, 0, st>>>(rootList, dLab, K, compLabel);
        note_launch();
        CKL();
        CK(cudaStreamSynchronize(st));  // lab is released on return
        return CHAOS_OK;
    }
    int* markMin = (int*)c.alloc(n * sizeof(int));
    int* markFix = (int*)c.alloc(n * sizeof(int));
    NEED(!c.failed);
    CK(cudaMemsetAsync(markMin, 0, n * sizeof(int), st));
    CK(cudaMemsetAsync(markFix, 0, n * sizeof(int), st));
    rank_marks_kernel<<<blocks(K), kTPB, 0, st>>>(rootMin, rootFix, K, compat ? 1 : 0, markMin, markFix);
    note_launch();
    CKL();
    int t = 0, rc;
    if ((rc = exclusive_scan(c, markMin, markMin, n, &t))) return rc;
    if (compat && (rc = exclusive_scan(c, markFix, markFix, n, &t))) return rc;
    rank_labels_kernel<<<blocks(K), kTPB, 0, st>>>(rootList, rootMin, rootFix, K, compat ? 1 : 0, markMin, markFix,
                                                   compLabel);
    note_launch();
    CKL();
    return CHAOS_OK;
}

// The pipeline. compat: the reference's eps-components (every included point
// core, numbering by fixed points); otherwise textbook DBSCAN with minPts.
// bound > 0: a bound on the occupied cells known from the source (else one
// pass over the features measures their extent). Fout (basin maps) receives
// the normalised features.
template <class Src>
int cell_cluster(Call& c, const Src& S, long long n, double eps, int minPts, bool compat, double bound, double* Fout,
                 int* labels) {
    cudaStream_t st = c.stream;
    const int D = S.D;
    const bool zeroEps = !(eps > 0);
    const double side = zeroEps ? 1.0 : eps / sqrt((double)D) * (1.0 - 1e-9);
    const double invSide = 1.0 / side;
    int* err = (int*)c.alloc(sizeof(int));
    NEED(err);
    CK(cudaMemsetAsync(err, 0, sizeof(int), st));
    if (!(bound > 0)) {
        long long* ext = (long long*)c.alloc(8 * sizeof(long long));
        NEED(ext);
        const long long init[8] = {LLONG_MIN, LLONG_MIN, LLONG_MIN, LLONG_MIN, LLONG_MIN, LLONG_MIN, 0, 0};
        CK(cudaMemcpyAsync(ext, init, sizeof init, cudaMemcpyHostToDevice, st));
        extent_kernel<Src><<<blocks(n), kTPB, 0, st>>>(S, n, invSide, ext);
        note_launch();
        long long hx[8];
        CK(cudaMemcpyAsync(hx, ext, sizeof hx, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        bound = (double)hx[6];
        if (hx[3] != LLONG_MIN) {  // some ordinary point
            double prod = 1.0;
            for (int d = 0; d < D; ++d) prod *= (double)(hx[3 + d] + hx[d] + 1);
            bound += prod;
        }
    }
    bound = std::min(bound, (double)n);
    unsigned long long cap = 1024;
    while ((double)cap < 2.0 * bound + 2.0) cap <<= 1;
    Table T;
    T.mask = cap - 1;
    T.key = (unsigned long long*)c.alloc(cap * sizeof(unsigned long long));
    T.cnt = (int*)c.alloc(cap * sizeof(int));
    T.lo = (unsigned*)c.alloc(cap * 3 * sizeof(unsigned));
    T.hi = (unsigned*)c.alloc(cap * 3 * sizeof(unsigned));
    T.minIdx = (int*)c.alloc(cap * sizeof(int));
    T.maxIdx = (int*)c.alloc(cap * sizeof(int));
    T.minFix = (int*)c.alloc(cap * sizeof(int));
    T.bad = (int*)c.alloc(cap * sizeof(int));
    int* slot = (int*)c.alloc(n * sizeof(int));
    int* occ = (int*)c.alloc(cap * sizeof(int));
    int* slotCell = (int*)c.alloc(cap * sizeof(int));
    NEED(!c.failed);
    table_init_kernel<<<blocks(cap), kTPB, 0, st>>>(T, (long long)cap);
    note_launch();
    cells_kernel<Src><<<blocks(n), kTPB, 0, st>>>(S, n, invSide, T, slot, Fout, err);
    note_launch();
    occupied_kernel<<<blocks(cap), kTPB, 0, st>>>(T.key, cap, occ);
    note_launch();
    CKL();
    int C = 0;
    int rc = exclusive_scan(c, occ, occ, (long long)cap, &C);
    if (rc) return rc;
    {
        int hErr = 0;
        CK(cudaMemcpyAsync(&hErr, err, sizeof(int), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        if (hErr) return set_error(CHAOS_E_CUDA, "clustering: cell table full");
    }
    Cells K;
    K.C = C;
    K.D = D;
    unsigned long long* cellKey = (unsigned long long*)c.alloc((size_t)(C + 1) * sizeof(unsigned long long));
    int* cellSlot = (int*)c.alloc((size_t)(C + 1) * sizeof(int));
    K.key = cellKey;
    K.cnt = (int*)c.alloc((size_t)(C + 1) * sizeof(int));
    K.lo = (double*)c.alloc((size_t)(C + 1) * 3 * sizeof(double));
    K.hi = (double*)c.alloc((size_t)(C + 1) * 3 * sizeof(double));
    K.unsafe = (unsigned char*)c.alloc((size_t)C + 1);
    K.dense = (unsigned char*)c.alloc((size_t)C + 1);
    K.minIdx = (int*)c.alloc((size_t)(C + 1) * sizeof(int));
    K.minFix = (int*)c.alloc((size_t)(C + 1) * sizeof(int));
    K.repV = (double*)c.alloc((size_t)(C + 1) * kReps * 3 * sizeof(double));
    K.repN = (int*)c.alloc((size_t)(C + 1) * sizeof(int));
    K.hasCore = (int*)c.alloc((size_t)(C + 1) * sizeof(int));
    K.minCore = (int*)c.alloc((size_t)(C + 1) * sizeof(int));
    K.sb = (int*)c.alloc((size_t)(C + 1) * sizeof(int));
    K.se = (int*)c.alloc((size_t)(C + 1) * sizeof(int));
    K.need = (int*)c.alloc((size_t)(C + 1) * sizeof(int));
    int* nbStart = (int*)c.alloc((size_t)(C + 1) * sizeof(int));
    int* take = (int*)c.alloc((size_t)(C + 1) * sizeof(int));
    int* begin = (int*)c.alloc((size_t)(C + 1) * sizeof(int));
    int* cursor = (int*)c.alloc((size_t)(C + 1) * sizeof(int));
    int* parentC = (int*)c.alloc((size_t)(C + 1) * sizeof(int));
    NEED(!c.failed);
    if (C > 0) {
        cell_ids_kernel<<<blocks(cap), kTPB, 0, st>>>(T.key, cap, occ, slotCell, cellKey, cellSlot);
        note_launch();
        finalize_kernel<Src><<<blocks(C), kTPB, 0, st>>>(S, K, cellSlot, T, compat ? 1 : 0, zeroEps ? 1 : 0, minPts);
        note_launch();
        neighbours_kernel<<<blocks((long long)C * 32), kTPB, 0, st>>>(cellKey, C, D, T.key, T.mask, slotCell,
                                                                      nbStart, nullptr, nullptr, nullptr);
        note_launch();
        iota_kernel<<<blocks(C), kTPB, 0, st>>>(parentC, C);
        note_launch();
        CKL();
    }
    CK(cudaMemsetAsync(nbStart + C, 0, sizeof(int), st));
    int E = 0;
    if ((rc = exclusive_scan(c, nbStart, nbStart, C + 1, &E))) return rc;
    int* nbList = (int*)c.alloc((size_t)(E + 1) * sizeof(int));
    int* nbOwner = (int*)c.alloc((size_t)(E + 1) * sizeof(int));
    unsigned char* pst = (unsigned char*)c.alloc((size_t)E + 1);
    unsigned char* openE = (unsigned char*)c.alloc((size_t)E + 1);
    unsigned char* settledE = (unsigned char*)c.alloc((size_t)E + 1);
    unsigned char* deferred = (unsigned char*)c.alloc((size_t)E + 1);
    int* openList = (int*)c.alloc((size_t)(E + 1) * sizeof(int));
    int* nOpen = (int*)c.alloc(sizeof(int));
    int* joinList = (int*)c.alloc((size_t)(E + 1) * sizeof(int));
    int* nJoined = (int*)c.alloc(sizeof(int));
    NEED(!c.failed);
    if (E > 0) {
        neighbours_kernel<<<blocks((long long)C * 32), kTPB, 0, st>>>(cellKey, C, D, T.key, T.mask, slotCell,
                                                                      nullptr, nbStart, nbList, nbOwner);
        note_launch();
        CK(cudaMemsetAsync(openE, 0, (size_t)E, st));
        CK(cudaMemsetAsync(settledE, 0, (size_t)E, st));
        CK(cudaMemsetAsync(deferred, 0, (size_t)E, st));
        CK(cudaMemsetAsync(nOpen, 0, sizeof(int), st));
        CK(cudaMemsetAsync(nJoined, 0, sizeof(int), st));
        pair_kernel<<<blocks(E), kTPB, 0, st>>>(K, nbOwner, nbList, E, eps, pst, openList, nOpen, joinList, nJoined);
        note_launch();
        CKL();
        int hOpen = 0;
        CK(cudaMemcpyAsync(&hOpen, nOpen, sizeof(int), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        if (hOpen > 0) {
            rep_pairs_kernel<<<blocks((long long)hOpen * 32), kTPB, 0, st>>>(K, nbOwner, nbList, openList, hOpen, eps,
                                                                             pst, joinList, nJoined);
            note_launch();
            CKL();
        }
        if (C <= kSharedCells) {
            const size_t shm = (size_t)C * sizeof(int);
            if (shm > 48 * 1024)
                CK(cudaFuncSetAttribute(cell_components_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm));
            cell_components_kernel<<<1, 1024, shm, st>>>(C, nbOwner, nbList, joinList, nJoined, parentC);
        } else {
            join_all_kernel<<<blocks(E), kTPB, 0, st>>>(nbOwner, nbList, joinList, nJoined, parentC);
        }
        note_launch();
        CKL();
    }
    // first sort: the points of the cells that are not dense
    Sorted Q;
    Q.order = (int*)c.alloc((size_t)(n + 1) * sizeof(int));
    Q.cell = (int*)c.alloc((size_t)(n + 1) * sizeof(int));
    Q.core = (unsigned char*)c.alloc((size_t)n + 1);
    Q.fix = compat ? (unsigned char*)c.alloc((size_t)n + 1) : nullptr;
    for (int d = 0; d < 3; ++d) Q.s[d] = d < D ? (double*)c.alloc((size_t)(n + 1) * sizeof(double)) : nullptr;
    Q.sb = K.sb;
    Q.se = K.se;
    Q.D = D;
    NEED(!c.failed);
    int M1 = 0;
    if (C > 0) {
        take_sparse_kernel<<<blocks(C), kTPB, 0, st>>>(K, take);
        note_launch();
        CKL();
        if ((rc = exclusive_scan(c, take, cursor, C, &M1))) return rc;
        if (M1 > 0) {
            phase_begin_kernel<<<blocks(C), kTPB, 0, st>>>(C, cursor, take, 0, begin, K.sb, K.se, K.cnt);
            note_launch();
            CK(cudaMemsetAsync(cursor, 0, (size_t)C * sizeof(int), st));
            sort_kernel<Src><<<blocks(n), kTPB, 0, st>>>(S, n, slot, slotCell, begin, cursor, Q, K.dense,
                                                         compat ? 1 : 0);
            note_launch();
            CKL();
        }
    }
    // core flags and the shortcuts' links of the points that are not in dense cells
    if (M1 > 0) {
        if (!compat) {
            core_kernel<<<blocks((long long)M1 * 32), kTPB, 0, st>>>(Q, K, nbStart, nbList, M1, eps, minPts, 0,
                                                                     nullptr);
            note_launch();
        }
        dense_links_kernel<<<blocks((long long)M1 * 32), kTPB, 0, st>>>(Q, K, nbStart, nbList, M1, eps, parentC,
                                                                        openE, settledE);
        note_launch();
        CKL();
    }
    if (E > 0) {
        open_pairs_kernel<<<blocks(E), kTPB, 0, st>>>(K, nbOwner, nbList, E, parentC, pst, openE, settledE);
        note_launch();
        CKL();
    }
    // second sort: the cells some pair, count or label still has to scan
    int M2 = 0;
    if (C > 0) {
        take_needed_kernel<<<blocks(C), kTPB, 0, st>>>(K, take);
        note_launch();
        CKL();
        if ((rc = exclusive_scan(c, take, cursor, C, &M2))) return rc;
        if (M2 > 0) {
            phase_begin_kernel<<<blocks(C), kTPB, 0, st>>>(C, cursor, take, M1, begin, K.sb, K.se, K.cnt);
            note_launch();
            CK(cudaMemsetAsync(cursor, 0, (size_t)C * sizeof(int), st));
            sort_kernel<Src><<<blocks(n), kTPB, 0, st>>>(S, n, slot, slotCell, begin, cursor, Q, K.dense,
                                                         compat ? 1 : 0);
            note_launch();
            CKL();
        }
    }
    // union-find over nodes: cells, then the sorted points (unsafe cells' core points)
    const long long M = (long long)M1 + M2;
    const long long N = (long long)C + M;
    int* parent = (int*)c.alloc((size_t)(N + 1) * sizeof(int));
    int* compMin = (int*)c.alloc((size_t)(N + 1) * sizeof(int));
    int* compFix = (int*)c.alloc((size_t)(N + 1) * sizeof(int));
    int* compLabel = (int*)c.alloc((size_t)(N + 1) * sizeof(int));
    int* cellLabel = (int*)c.alloc((size_t)(C + 1) * sizeof(int));
    int* rootList = (int*)c.alloc((size_t)(N + 1) * sizeof(int));
    int* rootMin = (int*)c.alloc((size_t)(N + 1) * sizeof(int));
    int* rootFix = (int*)c.alloc((size_t)(N + 1) * sizeof(int));
    int* nRoots = (int*)c.alloc(sizeof(int));
    NEED(!c.failed);
    iota_kernel<<<blocks(N + 1), kTPB, 0, st>>>(parent, N + 1);
    note_launch();
    if (C > 0) CK(cudaMemcpyAsync(parent, parentC, (size_t)C * sizeof(int), cudaMemcpyDeviceToDevice, st));
    if (M1 > 0 && !compat) {  // the undecided counts, exactly (their neighbours are sorted now)
        core_kernel<<<blocks((long long)M1 * 32), kTPB, 0, st>>>(Q, K, nbStart, nbList, M1, eps, minPts, 1,
                                                                 parent);
        note_launch();
        CKL();
    }
    if (E > 0) {
        whole_pairs_kernel<<<blocks(E), kTPB, 0, st>>>(K, nbOwner, nbList, E, pst, parent);
        note_launch();
    }
    if (C > 0 && M > 0) {
        unsafe_cell_kernel<<<blocks((long long)C * 32), kTPB, 0, st>>>(Q, K, eps, parent);
        note_launch();
    }
    if (E > 0 && M > 0)
        for (int pass = 0; pass < kCrossPasses; ++pass) {
            cross_cell_kernel<<<blocks((long long)E * 32), kTPB, 0, st>>>(Q, K, nbOwner, nbList, E, pst, eps, parent,
                                                                          pass, deferred);
            note_launch();
        }
    CKL();
    // components, numbered
    CK(cudaMemsetAsync(nRoots, 0, sizeof(int), st));
    if (N > 0) {
        fill_kernel<<<blocks(N), kTPB, 0, st>>>(compMin, N, INT_MAX);
        note_launch();
        fill_kernel<<<blocks(N), kTPB, 0, st>>>(compFix, N, INT_MAX);
        note_launch();
        comp_kernel<<<blocks(N), kTPB, 0, st>>>(Q, K, N, parent, compMin, compFix);
        note_launch();
        roots_kernel<<<blocks(N), kTPB, 0, st>>>(Q, K, N, parent, compMin, compFix, rootList, rootMin, rootFix,
                                                 nRoots);
        note_launch();
        CKL();
    }
    int nK = 0;
    CK(cudaMemcpyAsync(&nK, nRoots, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if ((rc = number_components(c, n, nK, compat, rootList, rootMin, rootFix, compLabel))) return rc;
    if (C > 0) {
        cell_labels_kernel<<<blocks(C), kTPB, 0, st>>>(K, parent, compLabel, cellLabel);
        note_launch();
    }
    labels_kernel<<<blocks(n), kTPB, 0, st>>>(slot, slotCell, n, K.dense, cellLabel, compat ? 1 : 0, labels);
    note_launch();
    if (M1 > 0) {
        sorted_labels_kernel<<<blocks((long long)M1 * 32), kTPB, 0, st>>>(Q, K, nbStart, nbList, M1, eps, parent,
                                                                          compMin, compLabel, labels);
        note_launch();
    }
    CKL();
    return CHAOS_OK;
}

}  // namespace

template <class T>
static int exclusive_scan_t(Call& c, const T* in, T* out, long long n, T* total) {
    if (n <= 0) {
        if (total) *total = 0;
        return CHAOS_OK;
    }
    const long long nb = (n + kScanItems - 1) / kScanItems;
    T* sums = (T*)c.alloc((size_t)(nb + 1) * sizeof(T));
    if (!sums) return CHAOS_E_NOMEM;
    scan_block_kernel<T><<<(unsigned)nb, 1024, 0, c.stream>>>(in, out, sums, n);
    note_launch();
    CK(cudaGetLastError());
    if (nb > 1) {
        int rc = exclusive_scan_t<T>(c, sums, sums, nb, total);
        if (rc) return rc;
        add_offsets_kernel<T><<<blocks(n), kTPB, 0, c.stream>>>(out, sums, n);
        note_launch();
        CK(cudaGetLastError());
    } else if (total) {
        CK(cudaMemcpyAsync(total, sums, sizeof(T), cudaMemcpyDeviceToHost, c.stream));
        CK(cudaStreamSynchronize(c.stream));
    }
    return CHAOS_OK;
}

int exclusive_scan(Call& c, const int* in, int* out, long long n, int* total) {
    return exclusive_scan_t<int>(c, in, out, n, total);
}

int exclusive_scan64(Call& c, const long long* in, long long* out, long long n, long long* total) {
    return exclusive_scan_t<long long>(c, in, out, n, total);
}

int dbscan_compat_device(Call& c, const double* avgPeaks, const double* avgIntervals, const int* flags, long long n,
                         double eps, int* labels) {
    ColSrc S;
    S.f[0] = avgPeaks;
    S.f[1] = avgIntervals;
    S.f[2] = avgIntervals;
    S.mask = nullptr;
    S.flags = flags;
    S.D = 2;
    S.compat = true;
    return cell_cluster(c, S, n, eps, 1, true, 0.0, nullptr, labels);
}

int dbscan_device(Call& c, const double* features, long long n, int dims, double eps, int minPts, const int* mask,
                  int* labels) {
    RowSrc S;
    S.F = features;
    S.mask = mask;
    S.D = dims;
    return cell_cluster(c, S, n, eps, minPts, false, 0.0, nullptr, labels);
}

int dbscan_basins_device(Call& c, const BasinsOut& O, long long n, const unsigned long long* minmaxKeys, double eps,
                         int minPts, double* features, int* labels) {
    BasinSrc S;
    S.flags = O.flags;
    S.counts = O.counts;
    S.avgPeaks = O.avgPeaks;
    S.avgIntervals = O.avgIntervals;
    S.last = O.last;
    S.D = 3;
    for (int d = 0; d < 3; ++d) {
        const bool any = minmaxKeys[d] != ~0ull;
        auto unk = [](unsigned long long k) {
            const unsigned long long b = (k & 0x8000000000000000ull) ? (k & 0x7fffffffffffffffull) : ~k;
            double v;
            memcpy(&v, &b, sizeof v);
            return v;
        };
        const double lo = any ? unk(minmaxKeys[d]) : 0.0, hi = any ? unk(minmaxKeys[3 + d]) : 0.0;
        S.lo[d] = lo;
        S.ok[d] = any && hi > lo;
        S.inv[d] = S.ok[d] ? 1.0 / (hi - lo) : 0.0;
    }
    // normalised features lie in [0, 1]: at most floor(1 / side) + 1 cells per
    // dimension (one more for the rounding of (f - lo) * inv), and one cell
    // of NaN features
    const double side = eps / sqrt(3.0) * (1.0 - 1e-9);
    const double per = floor(1.0 / side) + 2.0;
    const double bound = per * per * per + 1.0;
    return cell_cluster(c, S, n, eps, minPts, false, bound, features, labels);
}

}  // namespace chaos
