// Grid clustering on the device.
//
// Both clusterings share one pipeline over points in a D-dimensional feature
// space (D = 1..3), all integer/FP64 and bound by memory traffic:
//   1. cell of every point: floor(f * (1/side)) per dimension, side = eps/sqrt(D)
//      shrunk by 1e-9, so two points of one cell are always within eps and a
//      neighbour within eps is at most R = 2 cells away per dimension;
//   2. an open-addressing hash table of the occupied cells (64-bit packed
//      coordinates), their dense numbering and a counting sort of the points
//      by cell, with the features gathered into cell order (coalesced reads
//      for everything that follows);
//   3. per cell: bounding box and the list of occupied neighbour cells;
//   4. (DBSCAN) core flags: a cell holding >= minPts points makes all of them
//      core; otherwise neighbours are counted exactly, with early exit, whole
//      cells counted or skipped by their bounding boxes;
//   5. union-find over points (parent[v] <= v, lock-free hooking with
//      atomicCAS): every cell's core points are linked to its smallest one,
//      then one warp per neighbouring cell pair looks for a core pair within
//      eps (lanes stride over the larger cell, box tests per cell pair and per
//      point, early exit) in two passes: bounded probes first, then
//      exhaustive scans of the pairs that still separate two components. The
//      root of a component is its smallest core index;
//   6. numbering by prefix sums over the root indices.
// Distances are sqrt(sum of squared differences) <= eps in FP64, in dimension
// order, each operation rounded on its own (this file is compiled with
// --fmad=false), as the reference computes them (Basins/src/basinsCUDA.cu:918).
// Cells whose coordinates had to be clamped (|f| / side >= 2^19) or that hold
// a NaN feature lose the one-cell-is-connected shortcut and are resolved by
// exact pair tests.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>

#include "dbscan.h"

namespace chaos {

namespace {

constexpr int kTPB = 256;
constexpr unsigned long long kEmpty = ~0ull;
constexpr long long kLim = 1LL << 19;  // clamp of cell coordinates (21-bit packing for D = 3)
constexpr int kR = 2;                  // neighbour reach in cells

struct Feat {
    const double* f[3];
    int D;
};

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
    for (int d = 0; d < D; ++d) {
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

// ---- grid construction -----------------------------------------------------
// q = f * (1/side): the rounding of the product (|q| < 2^19: below 1e-10 of a
// cell) stays far inside the 1e-9 by which the side is shrunk, so two points
// of one cell are still within eps (a division here would cost the FP64 pipe
// three divides per point for the same guarantee).
// The kernel also reduces the extent of the cell coordinates of its ordinary
// points (ext[d] = -min, ext[3 + d] = max, per dimension) and counts the
// clamped or NaN ones (ext[6]): the number of occupied cells is at most the
// product of the extents plus that count, which sizes the hash table (a
// basin map's normalised features occupy at most ~35^3 cells of its 4.2 M
// points). Warps reduce with shuffles into shared memory, one global atomic
// per block and quantity.
__global__ void cell_key_kernel(Feat F, const int* include, long long n, double invSide, unsigned long long* key,
                                unsigned char* unsafe, long long* ext) {
    __shared__ long long sext[7];
    if (threadIdx.x < 7) sext[threadIdx.x] = threadIdx.x < 6 ? LLONG_MIN : 0;
    __syncthreads();
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long c[3] = {0, 0, 0};
    bool bad = false, ok = false;
    if (i < n) {
        if (!include[i]) {
            key[i] = kEmpty;
            unsafe[i] = 0;
        } else {
            for (int d = 0; d < F.D; ++d) {
                const double q = F.f[d][i] * invSide;
                if (q != q) { c[0] = kLim + 5; c[1] = kLim + 5; c[2] = kLim + 5; bad = true; break; }
                long long v;
                if (q >= (double)kLim) { v = kLim; bad = true; }
                else if (q < -(double)kLim) { v = -kLim; bad = true; }
                else v = (long long)floor(q);
                c[d] = v;
            }
            key[i] = pack(c, F.D);
            unsafe[i] = bad ? 1 : 0;
            ok = !bad;
        }
    }
    const int lane = threadIdx.x & 31;
    const unsigned nbad = __popc(__ballot_sync(0xffffffffu, bad));
    if (lane == 0 && nbad) atomicAdd((unsigned long long*)&sext[6], (unsigned long long)nbad);
    if (__any_sync(0xffffffffu, ok)) {
        for (int d = 0; d < F.D; ++d) {
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

// The lanes of a warp that carry the same cell key are served by one lane
// (__match_any_sync): a basin map puts up to 225,000 points in one cell, and
// neighbouring grid points mostly share theirs, so the hot cells' table slot,
// counter and cursor see one access per warp instead of one per point.
__global__ void hash_insert_kernel(const unsigned long long* key, long long n, unsigned long long* tab,
                                   unsigned long long mask, long long* slot) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    const unsigned long long k = i < n ? key[i] : kEmpty;
    const unsigned grp = __match_any_sync(0xffffffffu, k);
    const int leader = __ffs(grp) - 1;
    long long h = -1;
    if (k != kEmpty && lane == leader) {
        unsigned long long g = mix(k) & mask;
        for (unsigned long long probe = 0; probe <= mask; ++probe) {
            const unsigned long long prev = atomicCAS(&tab[g], kEmpty, k);
            if (prev == kEmpty || prev == k) { h = (long long)g; break; }
            g = (g + 1) & mask;
        }  // the table has at least twice as many slots as occupied cells: a free slot is always found
    }
    h = __shfl_sync(0xffffffffu, h, leader);
    if (i < n) slot[i] = k == kEmpty ? -1 : h;
}

__global__ void occupied_kernel(const unsigned long long* tab, long long cap, int* occ) {
    const long long h = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (h < cap) occ[h] = tab[h] != kEmpty;
}

__global__ void cell_ids_kernel(const unsigned long long* tab, long long cap, const int* occScan, int* slotCell,
                                unsigned long long* cellKey) {
    const long long h = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= cap) return;
    if (tab[h] != kEmpty) {
        slotCell[h] = occScan[h];
        cellKey[occScan[h]] = tab[h];
    } else {
        slotCell[h] = -1;
    }
}

__global__ void point_cell_kernel(const long long* slot, long long n, const int* slotCell, int* cellOf, int* cnt) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    const long long sl = i < n ? slot[i] : -1;
    const int c = sl >= 0 ? slotCell[sl] : -1;
    if (i < n) cellOf[i] = c;
    const unsigned grp = __match_any_sync(0xffffffffu, c);
    if (c >= 0 && lane == __ffs(grp) - 1) atomicAdd(&cnt[c], __popc(grp));
}

__global__ void scatter_kernel(Feat F, long long n, const int* cellOf, const int* start, int* cursor, int* order,
                               double* s0, double* s1, double* s2) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    const int c = i < n ? cellOf[i] : -1;
    const unsigned grp = __match_any_sync(0xffffffffu, c);
    const int leader = __ffs(grp) - 1;
    int base = 0;
    if (c >= 0 && lane == leader) base = atomicAdd(&cursor[c], __popc(grp));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (c < 0) return;
    const int pos = start[c] + base + __popc(grp & ((1u << lane) - 1u));
    order[pos] = (int)i;
    s0[pos] = F.f[0][i];
    if (F.D > 1) s1[pos] = F.f[1][i];
    if (F.D > 2) s2[pos] = F.f[2][i];
}

struct Sorted {
    const double* s[3];
    const int* order;
    const int* start;  // C + 1 entries
    int D;
    __device__ __forceinline__ void load(int pos, double* v) const {
        for (int d = 0; d < D; ++d) v[d] = s[d][pos];
    }
};

// ---- per-cell reductions over the cell-sorted points ---------------------------
// One thread per sorted position; a cell's positions are contiguous, so a warp
// reduces each run of equal cells with shuffles and the run's first lane
// folds it into the cell with one atomic. Work is even however unequal the
// cells are (a basin map can put a quarter of a million points in one cell).
__device__ __forceinline__ unsigned long long okey(double v) {  // order-preserving, for atomicMin/atomicMax
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    return (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double unkey(unsigned long long k) {
    const unsigned long long b = (k & 0x8000000000000000ull) ? (k & 0x7fffffffffffffffull) : ~k;
    return __longlong_as_double((long long)b);
}

// reduction of the lanes [lane, end of its run) holding the same cell
template <class T, class Op> __device__ __forceinline__ T run_reduce(T v, int cell, Op op) {
    const int lane = threadIdx.x & 31;
    for (int o = 1; o < 32; o <<= 1) {
        const T u = __shfl_down_sync(0xffffffffu, v, o);
        const int c2 = __shfl_down_sync(0xffffffffu, cell, o);
        if (lane + o < 32 && c2 == cell) v = op(v, u);
    }
    return v;
}

__device__ __forceinline__ bool run_head(int cell) {
    const int lane = threadIdx.x & 31;
    const int prev = __shfl_up_sync(0xffffffffu, cell, 1);
    return cell >= 0 && (lane == 0 || prev != cell);
}

__global__ void cell_init_kernel(int C, unsigned long long* keyLo, unsigned long long* keyHi, int* bad, int* rep) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= C) return;
    for (int d = 0; d < 3; ++d) {
        keyLo[3 * c + d] = ~0ull;
        keyHi[3 * c + d] = 0ull;
    }
    bad[c] = 0;
    rep[c] = 0x7fffffff;
}

// bounding box (NaN features ignored) and unsafe flag of every cell
__global__ void box_reduce_kernel(Sorted S, long long used, const int* cellOf, const unsigned char* unsafePt,
                                  unsigned long long* keyLo, unsigned long long* keyHi, int* bad) {
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    int c = -1, b = 0;
    double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    if (p < used) {
        const int i = S.order[p];
        c = cellOf[i];
        b = unsafePt[i];
        for (int d = 0; d < S.D; ++d) {
            const double v = S.s[d][p];
            lo[d] = v != v ? INFINITY : v;
            hi[d] = v != v ? -INFINITY : v;
        }
    }
    for (int d = 0; d < S.D; ++d) {
        lo[d] = run_reduce(lo[d], c, [](double x, double y) { return fmin(x, y); });
        hi[d] = run_reduce(hi[d], c, [](double x, double y) { return fmax(x, y); });
    }
    b = run_reduce(b, c, [](int x, int y) { return x | y; });
    if (run_head(c)) {
        for (int d = 0; d < S.D; ++d) {
            atomicMin(&keyLo[3 * (long long)c + d], okey(lo[d]));
            atomicMax(&keyHi[3 * (long long)c + d], okey(hi[d]));
        }
        if (b) atomicOr(&bad[c], 1);
    }
}

__global__ void box_final_kernel(int C, int D, const unsigned long long* keyLo, const unsigned long long* keyHi,
                                 const int* bad, double* boxLo, double* boxHi, unsigned char* unsafeCell) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= C) return;
    for (int d = 0; d < 3; ++d) {
        boxLo[3 * c + d] = d < D ? unkey(keyLo[3 * c + d]) : 0.0;
        boxHi[3 * c + d] = d < D ? unkey(keyHi[3 * c + d]) : 0.0;
    }
    unsafeCell[c] = bad[c] ? 1 : 0;
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

// per cell: number (pass 0) or list (pass 1) of occupied neighbour cells
__global__ void neighbours_kernel(const unsigned long long* cellKey, int C, int D, const unsigned long long* tab,
                                  unsigned long long mask, const int* slotCell, int* nbCount, const int* nbStart,
                                  int* nbList, int* nbOwner) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= C) return;
    long long base[3];
    unpack(cellKey[c], D, base);
    const int ry = D >= 2 ? kR : 0, rz = D >= 3 ? kR : 0;
    int k = 0;
    const int w0 = nbStart ? nbStart[c] : 0;
    for (int dx = -kR; dx <= kR; ++dx)
        for (int dy = -ry; dy <= ry; ++dy)
            for (int dz = -rz; dz <= rz; ++dz) {
                if (dx == 0 && dy == 0 && dz == 0) continue;
                long long q[3] = {base[0] + dx, base[1] + dy, base[2] + dz};
                const int c2 = hash_find(tab, mask, slotCell, pack(q, D));
                if (c2 < 0) continue;
                if (nbList) {
                    nbList[w0 + k] = c2;
                    nbOwner[w0 + k] = (int)c;
                }
                ++k;
            }
    if (!nbList) nbCount[c] = k;
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

// ---- cell bounding boxes ---------------------------------------------------------
// A cell's box holds all its points, so a box farther than eps from a point
// (or from another box) holds no point within eps, and a box whose farthest
// corner is within eps holds only points within eps. Both tests keep a
// relative margin of 1e-7 on the squared distance (far above the rounding of
// the exact test), so they never change a result, only skip work.
constexpr double kBoxOut = 1.0000001, kBoxIn = 0.9999999;

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

// ---- core points (DBSCAN) ----------------------------------------------------
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

// points of a safe cell holding >= minPts points are core; every other
// included point is listed for the exact count below
__global__ void core_kernel(Sorted S, const int* cellOf, long long n, const unsigned char* unsafeCell, int minPts,
                            unsigned char* core, int* sparse, int* nSparse) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    bool take = false;
    if (i < n) {
        const int c = cellOf[i];
        if (c < 0) core[i] = 0;
        else if (!unsafeCell[c] && S.start[c + 1] - S.start[c] >= minPts) core[i] = 1;
        else take = true;
    }
    list_append(take, (int)i, sparse, nSparse);
}

// block per listed point: neighbours within eps counted blockDim at a time
// (__syncthreads_count), whole safe cells counted or skipped by their
// bounding boxes, early exit at minPts. A point at the edge of a dense cell
// (the basin maps put up to 225,000 points in one cell) may have to test
// every point of it: a block spreads that scan over 8 warps. The cells whose
// box the ball contains are counted before any cell is scanned.
__global__ void core_sparse_kernel(Feat F, Sorted S, const int* cellOf, const int* sparse, int nSparse,
                                   const int* nbStart, const int* nbList, const unsigned char* unsafeCell,
                                   const double* boxLo, const double* boxHi, double eps, int minPts,
                                   unsigned char* core) {
    const int w = blockIdx.x;
    if (w >= nSparse) return;
    const int i = sparse[w];
    const int c = cellOf[i];
    double me[3] = {0, 0, 0};
    for (int d = 0; d < F.D; ++d) me[d] = F.f[d][i];
    const double eps2 = eps * eps;
    // box test of a safe cell: 0 skip, 1 count whole, 2 scan
    auto classify = [&](int cell) {
        if (unsafeCell[cell]) return 2;
        double near2, far2;
        box_dist2(me, boxLo + 3 * (long long)cell, boxHi + 3 * (long long)cell, S.D, near2, far2);
        if (near2 > eps2 * kBoxOut) return 0;
        if (far2 < eps2 * kBoxIn) return 1;
        return 2;
    };
    int cnt = 0;  // the same in every thread
    if (!unsafeCell[c]) cnt = S.start[c + 1] - S.start[c];  // one cell is within eps of itself
    for (int e = nbStart[c]; e < nbStart[c + 1] && cnt < minPts; ++e) {
        const int cell = nbList[e];
        if (classify(cell) == 1) cnt += S.start[cell + 1] - S.start[cell];
    }
    auto scan_cell = [&](int cell) {
        const int end = S.start[cell + 1];
        for (int p0 = S.start[cell]; p0 < end && cnt < minPts; p0 += blockDim.x) {
            const int p = p0 + threadIdx.x;
            bool hit = false;
            if (p < end) {
                double v[3];
                S.load(p, v);
                hit = sqrt(dist2(me, v, S.D)) <= eps;
            }
            cnt += __syncthreads_count(hit);
        }
    };
    if (unsafeCell[c] && cnt < minPts) scan_cell(c);
    for (int e = nbStart[c]; e < nbStart[c + 1] && cnt < minPts; ++e) {
        const int cell = nbList[e];
        if (classify(cell) == 2) scan_cell(cell);
    }
    if (threadIdx.x == 0) core[i] = cnt >= minPts ? 1 : 0;
}

// rep[c] = smallest core index of cell c (or -1); every core point of a safe
// cell is linked to it, the core points of an unsafe cell by exact pair tests.
__global__ void rep_reduce_kernel(Sorted S, long long used, const int* cellOf, const unsigned char* core,
                                  int* rep) {
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    int c = -1, m = 0x7fffffff;
    if (p < used) {
        const int i = S.order[p];
        c = cellOf[i];
        if (core[i]) m = i;
    }
    m = run_reduce(m, c, [](int x, int y) { return min(x, y); });
    if (run_head(c) && m != 0x7fffffff) atomicMin(&rep[c], m);
}

__global__ void rep_final_kernel(int C, int* rep) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c < C && rep[c] == 0x7fffffff) rep[c] = -1;
}

__global__ void link_kernel(const int* cellOf, long long n, const unsigned char* core,
                            const unsigned char* unsafeCell, const int* rep, int* parent) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !core[i]) return;
    const int c = cellOf[i];
    if (c < 0 || unsafeCell[c]) return;
    const int m = rep[c];
    if (m != (int)i) parent[i] = m;  // i is still a root: nothing else has linked it yet
}

// warp per unsafe cell: exact pair tests between its core points
__global__ void unsafe_cell_kernel(Sorted S, int C, const unsigned char* core, const unsigned char* unsafeCell,
                                   double eps, int* parent) {
    const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= C || !unsafeCell[w]) return;
    const int b = S.start[w], e = S.start[w + 1];
    for (int p = b; p < e; ++p) {
        const int i = S.order[p];
        if (!core[i]) continue;
        double a[3];
        S.load(p, a);
        for (int q = p + 1 + lane; q < e; q += 32) {
            const int j = S.order[q];
            if (!core[j]) continue;
            double v[3];
            S.load(q, v);
            if (sqrt(dist2(a, v, S.D)) <= eps) uf_unite(parent, i, j);
        }
    }
}

// warp per (cell, neighbour cell) entry with neighbour > cell: unite the two
// cells' core points if any core pair is within eps. The smaller cell's points
// are walked one by one, the larger cell's 32 at a time.
//
// Three passes of growing budget. Pass 0 probes every pair with a small
// amount of work (kPassOuter points of the smaller cell against kPassChunks
// x 32 points of the larger one) and marks the pairs it could not settle;
// each later pass takes the marked pairs only, first skips those whose two
// cells earlier unions already put into one component, and the last pass
// scans exhaustively. Inside a dense cluster almost every pair is settled by a
// probe or joined through other pairs, so the exhaustive scans are left to
// pairs that really separate two components. The components found do not
// depend on the order of the unions.
constexpr int kCrossPasses = 3;
__constant__ int kPassOuter[kCrossPasses] = {2, 32, 0x7fffffff};
__constant__ int kPassChunks[kCrossPasses] = {2, 8, 0x7fffffff};

__global__ void cross_cell_kernel(Sorted S, const int* nbOwner, const int* nbList, long long E,
                                  const unsigned char* core, const unsigned char* unsafeCell, const int* rep,
                                  const double* boxLo, const double* boxHi, double eps, int* parent, int pass,
                                  unsigned char* deferred) {
    const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= E) return;
    int ca = nbOwner[w], cb = nbList[w];
    if (cb <= ca) return;
    const bool last = pass == kCrossPasses - 1;
    if (pass > 0) {
        const bool todo = deferred[w] != 0;
        __syncwarp();  // every lane has read the mark before lane 0 clears it
        if (!todo) return;
        if (lane == 0) deferred[w] = 0;
    }
    if (rep[ca] < 0 || rep[cb] < 0) return;
    const bool safe = !unsafeCell[ca] && !unsafeCell[cb];
    if (!safe && !last) {  // unsafe cells unite every core pair within eps: last pass only
        if (lane == 0) deferred[w] = 1;
        return;
    }
    if (safe && uf_find(parent, rep[ca]) == uf_find(parent, rep[cb])) return;
    const double eps2 = eps * eps;
    const double* loA = boxLo + 3 * (long long)ca;
    const double* hiA = boxHi + 3 * (long long)ca;
    const double* loB = boxLo + 3 * (long long)cb;
    const double* hiB = boxHi + 3 * (long long)cb;
    double gap2 = 0.0, span2 = 0.0;
    for (int d = 0; d < S.D; ++d) {
        double g = 0.0;
        if (hiA[d] < loB[d]) g = loB[d] - hiA[d];
        else if (hiB[d] < loA[d]) g = loA[d] - hiB[d];
        gap2 = gap2 + g * g;
        const double f = fmax(hiA[d], hiB[d]) - fmin(loA[d], loB[d]);
        span2 = span2 + f * f;
    }
    if (gap2 > eps2 * kBoxOut) return;
    if (safe && span2 < eps2 * kBoxIn) {  // every point of one cell is within eps of every point of the other
        if (lane == 0) uf_unite(parent, rep[ca], rep[cb]);
        return;
    }
    if (S.start[ca + 1] - S.start[ca] > S.start[cb + 1] - S.start[cb]) {
        const int t = ca;
        ca = cb;
        cb = t;
    }
    const double* lo = boxLo + 3 * (long long)cb;
    const double* hi = boxHi + 3 * (long long)cb;
    int outerLeft = kPassOuter[pass];
    const int chunkBudget = kPassChunks[pass];
    bool cut = false, stop = false;
    // lanes test 32 points of the smaller cell against cb's box at a time;
    // the points in reach are then taken one by one against cb's points
    const int endA = S.start[ca + 1], endB = S.start[cb + 1];
    for (int p0 = S.start[ca]; p0 < endA && !stop; p0 += 32) {
        const int p = p0 + lane;
        int i = -1;
        double a[3] = {0, 0, 0};
        bool inReach = false, allIn = false;
        if (p < endA) {
            i = S.order[p];
            if (core[i]) {
                S.load(p, a);
                double near2, far2;
                box_dist2(a, lo, hi, S.D, near2, far2);
                inReach = near2 <= eps2 * kBoxOut;
                allIn = safe && far2 < eps2 * kBoxIn;
            }
        }
        const unsigned mAll = __ballot_sync(0xffffffffu, inReach && allIn);
        if (mAll) {  // every core point of cb is within eps of this one
            if (lane == __ffs(mAll) - 1) uf_unite(parent, i, rep[cb]);
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
            const int ii = __shfl_sync(0xffffffffu, i, src);
            double aa[3];
            for (int d = 0; d < 3; ++d) aa[d] = __shfl_sync(0xffffffffu, a[d], src);
            int chunks = 0;
            for (int q0 = S.start[cb]; q0 < endB; q0 += 32) {
                if (chunks++ == chunkBudget) {
                    cut = true;
                    break;
                }
                const int q = q0 + lane;
                bool hit = false;
                int j = -1;
                if (q < endB) {
                    j = S.order[q];
                    if (core[j]) {
                        double v[3];
                        S.load(q, v);
                        hit = sqrt(dist2(aa, v, S.D)) <= eps;
                    }
                }
                const unsigned bal = __ballot_sync(0xffffffffu, hit);
                if (bal) {
                    if (safe) {
                        if (lane == __ffs(bal) - 1) uf_unite(parent, ii, j);
                        return;
                    }
                    if (hit) uf_unite(parent, ii, j);
                }
            }
        }
    }
    if (cut && lane == 0) deferred[w] = 1;
}

__global__ void roots_kernel(int* parent, const unsigned char* core, long long n, int* root) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    root[i] = core[i] ? uf_find(parent, (int)i) : -1;
}

// ---- numbering: reference-compatible ----------------------------------------
__global__ void compat_minfix_kernel(const int* root, const int* flags, long long n, int* minFix) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (root[i] >= 0 && flags[i] == -1) atomicMin(&minFix[root[i]], (int)i);
}

__global__ void compat_marks_kernel(const int* root, const int* minFix, long long n, int* negMark, int* posMark) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (root[i] == (int)i) {
        if (minFix[i] < n) negMark[minFix[i]] = 1;  // several roots never share a minFix
        else posMark[i] = 1;
    }
}

__global__ void compat_labels_kernel(const int* root, const int* minFix, long long n, const int* negRank,
                                     const int* posRank, int* labels) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int r = root[i];
    if (r < 0) { labels[i] = 0; return; }
    const int mf = minFix[r];
    labels[i] = mf < n ? -(negRank[mf] + 1) : posRank[r] + 1;
}

// ---- numbering: DBSCAN ------------------------------------------------------
__global__ void root_marks_kernel(const int* root, long long n, int* mark) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    mark[i] = root[i] == (int)i ? 1 : 0;
}

__global__ void dbscan_labels_kernel(Feat F, Sorted S, const int* cellOf, const int* include, long long n,
                                     const int* nbStart, const int* nbList, const unsigned char* unsafeCell,
                                     const double* boxLo, const double* boxHi, const unsigned char* core,
                                     const int* root, const int* rep, const int* rank, double eps, int* labels) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (!include[i]) { labels[i] = -2; return; }
    if (core[i]) { labels[i] = rank[root[i]]; return; }
    const int c = cellOf[i];
    double me[3] = {0, 0, 0};
    for (int d = 0; d < F.D; ++d) me[d] = F.f[d][i];
    int best = 0x7fffffff;
    if (!unsafeCell[c] && rep[c] >= 0) best = root[rep[c]];
    const double eps2 = eps * eps;
    auto scan = [&](int cell) {
        if (!unsafeCell[cell]) {  // all core points of a safe cell share one root
            if (rep[cell] < 0) return;
            const int r = root[rep[cell]];
            if (r >= best) return;
            double near2, far2;
            box_dist2(me, boxLo + 3 * (long long)cell, boxHi + 3 * (long long)cell, S.D, near2, far2);
            if (near2 > eps2 * kBoxOut) return;
            if (far2 < eps2 * kBoxIn) {
                best = r;
                return;
            }
        }
        for (int p = S.start[cell]; p < S.start[cell + 1]; ++p) {
            const int j = S.order[p];
            if (!core[j]) continue;
            const int r = root[j];
            if (r >= best) continue;
            double v[3];
            S.load(p, v);
            if (sqrt(dist2(me, v, S.D)) <= eps) best = r;
        }
    };
    if (unsafeCell[c]) scan(c);
    for (int e = nbStart[c]; e < nbStart[c + 1]; ++e) scan(nbList[e]);
    labels[i] = best == 0x7fffffff ? -1 : rank[best];
}

__global__ void soa_kernel(const double* F, long long n, int D, double* a, double* b, double* c) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    a[i] = F[i * D];
    if (D > 1) b[i] = F[i * D + 1];
    if (D > 2) c[i] = F[i * D + 2];
}

__global__ void include_kernel(const int* flags, const int* mask, long long n, int compat, int* include) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    include[i] = compat ? (flags[i] != 0) : (mask ? mask[i] != 0 : 1);
}

__global__ void core_from_include_kernel(const int* include, long long n, unsigned char* core) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) core[i] = include[i] ? 1 : 0;
}

__global__ void iota_kernel(int* p, long long n) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = (int)i;
}

__global__ void fill_kernel(int* p, long long n, int v) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = v;
}

#define CK(x)                                                   \
    do {                                                        \
        cudaError_t e_ = (x);                                   \
        if (e_ != cudaSuccess) return cuda_error(e_, #x);       \
    } while (0)
#define CKL() CK(cudaGetLastError())
#define NEED(p) \
    if (!(p)) return CHAOS_E_NOMEM

// The shared pipeline. compat: flags select the points (flag != 0) and every
// selected point is core; otherwise mask (may be null) selects them and core
// points are computed with minPts.
int grid_cluster(Call& c, Feat F, long long n, double eps, int minPts, bool compat, const int* flags, const int* mask,
                 int* labels) {
    cudaStream_t st = c.stream;
    const int D = F.D;
    const bool zeroEps = !(eps > 0);
    const double side = zeroEps ? 1.0 : eps / sqrt((double)D) * (1.0 - 1e-9);

    int* include = (int*)c.alloc(n * sizeof(int));
    unsigned long long* key = (unsigned long long*)c.alloc(n * sizeof(unsigned long long));
    unsigned char* unsafePt = (unsigned char*)c.alloc(n);
    long long* slot = (long long*)c.alloc(n * sizeof(long long));
    long long* ext = (long long*)c.alloc(8 * sizeof(long long));
    NEED(!c.failed);
    include_kernel<<<blocks(n), kTPB, 0, st>>>(flags, mask, n, compat ? 1 : 0, include);
    note_launch();
    {
        const long long init[8] = {LLONG_MIN, LLONG_MIN, LLONG_MIN, LLONG_MIN, LLONG_MIN, LLONG_MIN, 0, 0};
        CK(cudaMemcpyAsync(ext, init, sizeof init, cudaMemcpyHostToDevice, st));
    }
    cell_key_kernel<<<blocks(n), kTPB, 0, st>>>(F, include, n, 1.0 / side, key, unsafePt, ext);
    note_launch();
    // table capacity: a power of two >= twice a bound on the occupied cells
    long long hx[8];
    CK(cudaMemcpyAsync(hx, ext, sizeof hx, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    double bound = (double)hx[6];
    if (hx[3] != LLONG_MIN) {  // some ordinary point
        double prod = 1.0;
        for (int d = 0; d < D; ++d) prod *= (double)(hx[3 + d] + hx[d] + 1);
        bound += prod;
    }
    bound = std::min(bound, (double)n);
    unsigned long long cap = 1024;
    while ((double)cap < 2.0 * bound + 2.0) cap <<= 1;
    unsigned long long* tab = (unsigned long long*)c.alloc(cap * sizeof(unsigned long long));
    int* occ = (int*)c.alloc(cap * sizeof(int));
    int* slotCell = (int*)c.alloc(cap * sizeof(int));
    NEED(!c.failed);
    CK(cudaMemsetAsync(tab, 0xff, cap * sizeof(unsigned long long), st));
    hash_insert_kernel<<<blocks(n), kTPB, 0, st>>>(key, n, tab, cap - 1, slot);
    note_launch();
    occupied_kernel<<<blocks(cap), kTPB, 0, st>>>(tab, cap, occ);
    note_launch();
    CKL();
    int C = 0;
    int rc = exclusive_scan(c, occ, occ, (long long)cap, &C);
    if (rc) return rc;
    unsigned long long* cellKey = (unsigned long long*)c.alloc((size_t)(C + 1) * sizeof(unsigned long long));
    int* cnt = (int*)c.alloc((size_t)(C + 1) * sizeof(int));
    int* cellOf = (int*)c.alloc(n * sizeof(int));
    NEED(!c.failed);
    cell_ids_kernel<<<blocks(cap), kTPB, 0, st>>>(tab, cap, occ, slotCell, cellKey);
    note_launch();
    CK(cudaMemsetAsync(cnt, 0, (size_t)(C + 1) * sizeof(int), st));
    point_cell_kernel<<<blocks(n), kTPB, 0, st>>>(slot, n, slotCell, cellOf, cnt);
    note_launch();
    CKL();
    int used = 0;
    if ((rc = exclusive_scan(c, cnt, cnt, C + 1, &used))) return rc;  // cnt -> start (C+1 entries)
    int* start = cnt;
    int* cursor = (int*)c.alloc((size_t)(C + 1) * sizeof(int));
    int* order = (int*)c.alloc((size_t)(used + 1) * sizeof(int));
    double* s0 = (double*)c.alloc((size_t)(used + 1) * sizeof(double));
    double* s1 = (double*)c.alloc((size_t)(used + 1) * sizeof(double));
    double* s2 = (double*)c.alloc((size_t)(used + 1) * sizeof(double));
    NEED(!c.failed);
    CK(cudaMemsetAsync(cursor, 0, (size_t)(C + 1) * sizeof(int), st));
    scatter_kernel<<<blocks(n), kTPB, 0, st>>>(F, n, cellOf, start, cursor, order, s0, s1, s2);
    note_launch();
    CKL();
    Sorted S;
    S.s[0] = s0;
    S.s[1] = s1;
    S.s[2] = s2;
    S.order = order;
    S.start = start;
    S.D = D;
    double* boxLo = (double*)c.alloc((size_t)(C + 1) * 3 * sizeof(double));
    double* boxHi = (double*)c.alloc((size_t)(C + 1) * 3 * sizeof(double));
    unsigned char* unsafeCell = (unsigned char*)c.alloc((size_t)C + 1);
    int* nbStart = (int*)c.alloc((size_t)(C + 1) * sizeof(int));
    NEED(!c.failed);
    unsigned long long* keyLo = (unsigned long long*)c.alloc((size_t)(C + 1) * 3 * sizeof(unsigned long long));
    unsigned long long* keyHi = (unsigned long long*)c.alloc((size_t)(C + 1) * 3 * sizeof(unsigned long long));
    int* bad = (int*)c.alloc((size_t)(C + 1) * sizeof(int));
    int* rep = (int*)c.alloc((size_t)(C + 1) * sizeof(int));
    NEED(!c.failed);
    if (C > 0) {
        cell_init_kernel<<<blocks(C), kTPB, 0, st>>>(C, keyLo, keyHi, bad, rep);
        note_launch();
        box_reduce_kernel<<<blocks(used), kTPB, 0, st>>>(S, used, cellOf, unsafePt, keyLo, keyHi, bad);
        note_launch();
        box_final_kernel<<<blocks(C), kTPB, 0, st>>>(C, D, keyLo, keyHi, bad, boxLo, boxHi, unsafeCell);
        note_launch();
        neighbours_kernel<<<blocks(C), kTPB, 0, st>>>(cellKey, C, D, tab, cap - 1, slotCell, nbStart, nullptr,
                                                      nullptr, nullptr);
        note_launch();
        CKL();
    }
    if (zeroEps && C > 0) CK(cudaMemsetAsync(unsafeCell, 1, (size_t)C, st));
    CK(cudaMemsetAsync(nbStart + C, 0, sizeof(int), st));
    int E = 0;
    if ((rc = exclusive_scan(c, nbStart, nbStart, C + 1, &E))) return rc;
    int* nbList = (int*)c.alloc((size_t)(E + 1) * sizeof(int));
    int* nbOwner = (int*)c.alloc((size_t)(E + 1) * sizeof(int));
    unsigned char* core = (unsigned char*)c.alloc(n);
    int* parent = (int*)c.alloc(n * sizeof(int));
    int* root = (int*)c.alloc(n * sizeof(int));
    unsigned char* deferred = (unsigned char*)c.alloc((size_t)E + 1);
    NEED(!c.failed);
    if (C > 0) {
        neighbours_kernel<<<blocks(C), kTPB, 0, st>>>(cellKey, C, D, tab, cap - 1, slotCell, nullptr, nbStart, nbList,
                                                      nbOwner);
        note_launch();
    }
    if (compat) {
        core_from_include_kernel<<<blocks(n), kTPB, 0, st>>>(include, n, core);
        note_launch();
    } else {
        int* sparse = (int*)c.alloc((n + 1) * sizeof(int));
        int* nSparse = (int*)c.alloc(sizeof(int));
        NEED(!c.failed);
        CK(cudaMemsetAsync(nSparse, 0, sizeof(int), st));
        core_kernel<<<blocks(n), kTPB, 0, st>>>(S, cellOf, n, unsafeCell, minPts, core, sparse, nSparse);
        note_launch();
        int hSparse = 0;
        CK(cudaMemcpyAsync(&hSparse, nSparse, sizeof(int), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        if (hSparse > 0) {
            core_sparse_kernel<<<hSparse, kTPB, 0, st>>>(
                F, S, cellOf, sparse, hSparse, nbStart, nbList, unsafeCell, boxLo, boxHi, eps, minPts, core);
            note_launch();
        }
    }
    iota_kernel<<<blocks(n), kTPB, 0, st>>>(parent, n);
    note_launch();
    if (C > 0) {
        rep_reduce_kernel<<<blocks(used), kTPB, 0, st>>>(S, used, cellOf, core, rep);
        note_launch();
        rep_final_kernel<<<blocks(C), kTPB, 0, st>>>(C, rep);
        note_launch();
        link_kernel<<<blocks(n), kTPB, 0, st>>>(cellOf, n, core, unsafeCell, rep, parent);
        note_launch();
        unsafe_cell_kernel<<<blocks((long long)C * 32), kTPB, 0, st>>>(S, C, core, unsafeCell, eps, parent);
        note_launch();
    }
    if (E > 0) {
        CK(cudaMemsetAsync(deferred, 0, (size_t)E, st));
        for (int pass = 0; pass < kCrossPasses; ++pass) {
            cross_cell_kernel<<<blocks((long long)E * 32), kTPB, 0, st>>>(S, nbOwner, nbList, E, core, unsafeCell,
                                                                          rep, boxLo, boxHi, eps, parent, pass,
                                                                          deferred);
            note_launch();
        }
    }
    roots_kernel<<<blocks(n), kTPB, 0, st>>>(parent, core, n, root);
    note_launch();
    CKL();
    if (compat) {
        int* minFix = (int*)c.alloc(n * sizeof(int));
        int* negRank = (int*)c.alloc(n * sizeof(int));
        int* posRank = (int*)c.alloc(n * sizeof(int));
        NEED(!c.failed);
        fill_kernel<<<blocks(n), kTPB, 0, st>>>(minFix, n, (int)n);
        note_launch();
        compat_minfix_kernel<<<blocks(n), kTPB, 0, st>>>(root, flags, n, minFix);
        note_launch();
        CK(cudaMemsetAsync(negRank, 0, n * sizeof(int), st));
        CK(cudaMemsetAsync(posRank, 0, n * sizeof(int), st));
        compat_marks_kernel<<<blocks(n), kTPB, 0, st>>>(root, minFix, n, negRank, posRank);
        note_launch();
        CKL();
        int t = 0;
        if ((rc = exclusive_scan(c, negRank, negRank, n, &t))) return rc;
        if ((rc = exclusive_scan(c, posRank, posRank, n, &t))) return rc;
        compat_labels_kernel<<<blocks(n), kTPB, 0, st>>>(root, minFix, n, negRank, posRank, labels);
        note_launch();
        CKL();
    } else {
        int* rank = (int*)c.alloc(n * sizeof(int));
        NEED(!c.failed);
        root_marks_kernel<<<blocks(n), kTPB, 0, st>>>(root, n, rank);
        note_launch();
        CKL();
        int t = 0;
        if ((rc = exclusive_scan(c, rank, rank, n, &t))) return rc;
        dbscan_labels_kernel<<<blocks(n), kTPB, 0, st>>>(F, S, cellOf, include, n, nbStart, nbList, unsafeCell,
                                                         boxLo, boxHi, core, root, rep, rank, eps, labels);
        ::chaos::note_launch();
        CKL();
    }
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
    Feat F;
    F.f[0] = avgPeaks;
    F.f[1] = avgIntervals;
    F.f[2] = avgIntervals;
    F.D = 2;
    return grid_cluster(c, F, n, eps, 1, true, flags, nullptr, labels);
}

int dbscan_device_soa(Call& c, const double* const* columns, long long n, int dims, double eps, int minPts,
                      const int* mask, int* labels) {
    Feat F;
    for (int d = 0; d < 3; ++d) F.f[d] = columns[d < dims ? d : dims - 1];
    F.D = dims;
    return grid_cluster(c, F, n, eps, minPts, false, nullptr, mask, labels);
}

int dbscan_device(Call& c, const double* features, long long n, int dims, double eps, int minPts, const int* mask,
                  int* labels) {
    double* a = (double*)c.alloc(n * sizeof(double));
    double* b = (double*)c.alloc(n * sizeof(double));
    double* d = (double*)c.alloc(n * sizeof(double));
    if (c.failed) return CHAOS_E_NOMEM;
    soa_kernel<<<blocks(n), kTPB, 0, c.stream>>>(features, n, dims, a, b, d);
    note_launch();
    CK(cudaGetLastError());
    Feat F;
    F.f[0] = a;
    F.f[1] = b;
    F.f[2] = d;
    F.D = dims;
    return grid_cluster(c, F, n, eps, minPts, false, nullptr, mask, labels);
}

}  // namespace chaos
