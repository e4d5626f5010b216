// Device primitives: block-decomposed scans, a stable LSD radix sort of
// (key, value) pairs and the dataset bounding-box reduction.
#include <float.h>

#include "vdb_internal.cuh"

namespace vdb {

std::atomic<unsigned long long> g_launches{0};

namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

struct OpSum {
    template <class T>
    __device__ static T apply(T a, T b) { return a + b; }
    template <class T>
    __device__ static T identity() { return T(0); }
};
struct OpMin {
    template <class T>
    __device__ static T apply(T a, T b) { return a < b ? a : b; }
    template <class T>
    __device__ static T identity() { return T(~T(0)); }
};

// Inclusive block scan of one value per thread; returns the inclusive prefix
// and writes the block aggregate to *total.
template <class T, class Op>
__device__ T block_inclusive(T v, T* total) {
    __shared__ T warp_tot[kScanThreads / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        T o = __shfl_up_sync(0xffffffffu, v, d);
        if (lane >= d) v = Op::apply(o, v);
    }
    if (lane == 31) warp_tot[wid] = v;
    __syncthreads();
    if (wid == 0) {
        T w = lane < kScanThreads / 32 ? warp_tot[lane] : Op::template identity<T>();
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            T o = __shfl_up_sync(0xffffffffu, w, d);
            if (lane >= d) w = Op::apply(o, w);
        }
        if (lane < kScanThreads / 32) warp_tot[lane] = w;
    }
    __syncthreads();
    if (wid > 0) v = Op::apply(warp_tot[wid - 1], v);
    *total = warp_tot[kScanThreads / 32 - 1];
    __syncthreads();
    return v;
}

// Exclusive block scan built on the inclusive one; *total = block aggregate.
template <class T, class Op>
__device__ T block_exclusive(T v, T* total) {
    __shared__ T wl[kScanThreads / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    T inc = block_inclusive<T, Op>(v, total);
    T prev = __shfl_up_sync(0xffffffffu, inc, 1);
    if (lane == 31) wl[wid] = inc;
    __syncthreads();
    T exc = lane > 0 ? prev : (wid > 0 ? wl[wid - 1] : Op::template identity<T>());
    __syncthreads();
    return exc;
}

template <bool Rev>
__device__ __forceinline__ uint64_t phys(uint64_t i, uint64_t n) { return Rev ? n - 1 - i : i; }

template <class TIn, class TOut, class Op, bool Rev>
__global__ void scan_reduce_kernel(const TIn* in, uint64_t n, TOut* part) {
    uint64_t base = (uint64_t)blockIdx.x * kScanTile;
    TOut acc = Op::template identity<TOut>();
    for (int k = 0; k < kScanItems; k++) {
        uint64_t i = base + (uint64_t)k * kScanThreads + threadIdx.x;
        if (i < n) acc = Op::apply(acc, (TOut)in[phys<Rev>(i, n)]);
    }
    TOut tot;
    block_inclusive<TOut, Op>(acc, &tot);
    if (threadIdx.x == 0) part[blockIdx.x] = tot;
}

// Exclusive scan of the per-block aggregates (one block, loops with a carry).
template <class TOut, class Op>
__global__ void scan_parts_kernel(TOut* part, uint64_t nparts, TOut* total_out) {
    TOut carry = Op::template identity<TOut>();
    for (uint64_t b = 0; b < nparts; b += kScanThreads) {
        uint64_t i = b + threadIdx.x;
        TOut v = i < nparts ? part[i] : Op::template identity<TOut>();
        TOut tot;
        TOut exc = block_exclusive<TOut, Op>(v, &tot);
        if (i < nparts) part[i] = Op::apply(carry, exc);
        carry = Op::apply(carry, tot);
    }
    if (threadIdx.x == 0 && total_out) *total_out = carry;
}

template <class TIn, class TOut, class Op, bool Rev, bool Inclusive>
__global__ void scan_apply_kernel(const TIn* in, uint64_t n, const TOut* part, TOut* out) {
    uint64_t base = (uint64_t)blockIdx.x * kScanTile + (uint64_t)threadIdx.x * kScanItems;
    TOut v[kScanItems];
    TOut acc = Op::template identity<TOut>();
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        uint64_t i = base + k;
        TOut x = i < n ? (TOut)in[phys<Rev>(i, n)] : Op::template identity<TOut>();
        v[k] = x;
        acc = Op::apply(acc, x);
    }
    TOut tot;
    TOut run = Op::apply(part[blockIdx.x], block_exclusive<TOut, Op>(acc, &tot));
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        uint64_t i = base + k;
        if (Inclusive) run = Op::apply(run, v[k]);
        if (i < n) out[phys<Rev>(i, n)] = run;
        if (!Inclusive) run = Op::apply(run, v[k]);
    }
}

uint64_t num_scan_blocks(uint64_t n) { return (n + kScanTile - 1) / kScanTile; }

template <class TIn, class TOut, class Op, bool Rev, bool Inclusive>
void scan_run(const TIn* in, TOut* out, uint64_t n, void* scratch, TOut* total_out,
              cudaStream_t s) {
    uint64_t nb = num_scan_blocks(n);
    TOut* part = (TOut*)scratch;
    if (nb == 0) {
        VDB_COUNT_LAUNCH();
        scan_parts_kernel<TOut, Op><<<1, kScanThreads, 0, s>>>(part, 0, total_out);
        return;
    }
    VDB_COUNT_LAUNCH();
    scan_reduce_kernel<TIn, TOut, Op, Rev><<<(unsigned)nb, kScanThreads, 0, s>>>(in, n, part);
    VDB_COUNT_LAUNCH();
    scan_parts_kernel<TOut, Op><<<1, kScanThreads, 0, s>>>(part, nb, total_out);
    VDB_COUNT_LAUNCH();
    scan_apply_kernel<TIn, TOut, Op, Rev, Inclusive>
        <<<(unsigned)nb, kScanThreads, 0, s>>>(in, n, part, out);
}

}  // namespace

size_t scan_u32_to_u64_scratch_bytes(uint64_t n) { return (num_scan_blocks(n) + 1) * 8; }
size_t scan_u32_scratch_bytes(uint64_t n) { return (num_scan_blocks(n) + 1) * 4; }
size_t suffix_min_u32_scratch_bytes(uint64_t n) { return (num_scan_blocks(n) + 1) * 4; }

void scan_u32_to_u64(const uint32_t* in, unsigned long long* out, uint64_t n, void* scratch,
                     cudaStream_t s) {
    scan_run<uint32_t, unsigned long long, OpSum, false, false>(in, out, n, scratch, out + n, s);
}

void scan_u32(const uint32_t* in, uint32_t* out, uint64_t n, void* scratch, cudaStream_t s) {
    scan_run<uint32_t, uint32_t, OpSum, false, false>(in, out, n, scratch, out + n, s);
}

void suffix_min_u32(uint32_t* a, uint64_t n, void* scratch, cudaStream_t s) {
    scan_run<uint32_t, uint32_t, OpMin, true, true>(a, a, n, scratch, (uint32_t*)nullptr, s);
}

// ------------------------------------------------------------------ radix sort

namespace {

constexpr int kSortThreads = 256;
constexpr int kSortRounds = 16;                 // items per thread per tile
constexpr int kSortRoundsSmall = 4;             // the same for sorts of <= 2^18 keys
constexpr uint32_t kSortSmall = 1u << 18;
constexpr int kRadix = 256;

// Rounds per tile: small sorts take short tiles, so that their few blocks
// become more blocks with a quarter of the serial rounds each.
int sort_rounds(uint32_t n) { return n <= kSortSmall ? kSortRoundsSmall : kSortRounds; }

__global__ void radix_hist_kernel(const uint32_t* keys, uint32_t n, int shift, uint32_t nblocks,
                                  int rounds, uint32_t* hist) {
    __shared__ uint32_t h[kRadix];
    h[threadIdx.x] = 0;
    __syncthreads();
    uint32_t base = blockIdx.x * (uint32_t)(kSortThreads * rounds);
    for (int r = 0; r < rounds; r++) {
        uint32_t i = base + r * kSortThreads + threadIdx.x;
        if (i < n) atomicAdd(&h[(keys[i] >> shift) & (kRadix - 1)], 1u);
    }
    __syncthreads();
    hist[threadIdx.x * nblocks + blockIdx.x] = h[threadIdx.x];
}

// Stable scatter: inside a tile, items keep their order (rounds of 256
// consecutive items; ranks within a warp from __match_any_sync, across warps
// from a per-digit prefix over the warps).
__global__ void radix_scatter_kernel(const uint32_t* keys, const uint32_t* vals, uint32_t n,
                                     int shift, uint32_t nblocks, int rounds,
                                     const uint32_t* hist_scan, uint32_t* okeys,
                                     uint32_t* ovals) {
    constexpr int W = kSortThreads / 32;
    __shared__ uint32_t gbase[kRadix];
    __shared__ uint32_t base[kRadix];
    __shared__ uint32_t wcnt[W][kRadix];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    gbase[threadIdx.x] = hist_scan[threadIdx.x * nblocks + blockIdx.x];
    base[threadIdx.x] = 0;
    const uint32_t lt = (1u << lane) - 1u;
    uint32_t tile = blockIdx.x * (uint32_t)(kSortThreads * rounds);
    for (int r = 0; r < rounds; r++) {
#pragma unroll
        for (int w = 0; w < W; w++) wcnt[w][threadIdx.x] = 0;
        __syncthreads();
        uint32_t i = tile + r * kSortThreads + threadIdx.x;
        bool valid = i < n;
        uint32_t k = valid ? keys[i] : 0u;
        uint32_t v = valid ? vals[i] : 0u;
        uint32_t d = valid ? ((k >> shift) & (kRadix - 1)) : (kRadix + lane);
        uint32_t peers = __match_any_sync(0xffffffffu, d);
        uint32_t rank = __popc(peers & lt);
        if (valid && rank == 0) wcnt[wid][d] = __popc(peers);
        __syncthreads();
        {
            uint32_t acc = base[threadIdx.x];
#pragma unroll
            for (int w = 0; w < W; w++) {
                uint32_t c = wcnt[w][threadIdx.x];
                wcnt[w][threadIdx.x] = acc;
                acc += c;
            }
            base[threadIdx.x] = acc;
        }
        __syncthreads();
        if (valid) {
            uint32_t dst = gbase[d] + wcnt[wid][d] + rank;
            okeys[dst] = k;
            ovals[dst] = v;
        }
        __syncthreads();
    }
}

}  // namespace

size_t radix_sort_scratch_bytes(uint32_t n) {
    const uint64_t tile = (uint64_t)kSortThreads * sort_rounds(n);
    uint64_t nb = ((uint64_t)n + tile - 1) / tile;
    uint64_t h = nb * kRadix;
    size_t b = 0;
    b += (size_t)n * 8;                     // alternate key/value buffers
    b += (h + 1) * 4 * 2;                   // histogram + its scan
    b += scan_u32_scratch_bytes(h);
    return b + 256;
}

void radix_sort_pairs(uint32_t* keys, uint32_t* vals, uint32_t n, int bits, void* scratch,
                      cudaStream_t s) {
    if (n <= 1 || bits <= 0) return;
    const int rounds = sort_rounds(n);
    const uint32_t tile = (uint32_t)(kSortThreads * rounds);
    uint32_t nb = (uint32_t)(((uint64_t)n + tile - 1) / tile);
    uint64_t h = (uint64_t)nb * kRadix;
    char* p = (char*)scratch;
    uint32_t* k2 = (uint32_t*)p; p += (size_t)n * 4;
    uint32_t* v2 = (uint32_t*)p; p += (size_t)n * 4;
    uint32_t* hist = (uint32_t*)p; p += (h + 1) * 4;
    uint32_t* hscan = (uint32_t*)p; p += (h + 1) * 4;
    void* sscratch = p;
    int passes = (bits + 7) / 8;
    uint32_t *ka = keys, *va = vals, *kb = k2, *vb = v2;
    for (int ps = 0; ps < passes; ps++) {
        int shift = ps * 8;
        VDB_COUNT_LAUNCH();
        radix_hist_kernel<<<nb, kSortThreads, 0, s>>>(ka, n, shift, nb, rounds, hist);
        scan_u32(hist, hscan, h, sscratch, s);
        VDB_COUNT_LAUNCH();
        radix_scatter_kernel<<<nb, kSortThreads, 0, s>>>(ka, va, n, shift, nb, rounds, hscan, kb,
                                                         vb);
        uint32_t* t;
        t = ka; ka = kb; kb = t;
        t = va; va = vb; vb = t;
    }
    if (ka != keys) {
        cudaMemcpyAsync(keys, ka, (size_t)n * 4, cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(vals, va, (size_t)n * 4, cudaMemcpyDeviceToDevice, s);
    }
}

// ------------------------------------------------------------------ bounding box

namespace {

constexpr int kBoxThreads = 256;

struct BoxAcc {
    double minx, maxx, miny, maxy;
    uint32_t bad;
};

__device__ BoxAcc box_merge(BoxAcc a, BoxAcc b) {
    a.minx = fmin(a.minx, b.minx);
    a.maxx = fmax(a.maxx, b.maxx);
    a.miny = fmin(a.miny, b.miny);
    a.maxy = fmax(a.maxy, b.maxy);
    a.bad |= b.bad;
    return a;
}

__device__ BoxAcc box_block_reduce(BoxAcc v) {
    __shared__ BoxAcc sh[kBoxThreads / 32];
    for (int d = 16; d > 0; d >>= 1) {
        BoxAcc o;
        o.minx = __shfl_down_sync(0xffffffffu, v.minx, d);
        o.maxx = __shfl_down_sync(0xffffffffu, v.maxx, d);
        o.miny = __shfl_down_sync(0xffffffffu, v.miny, d);
        o.maxy = __shfl_down_sync(0xffffffffu, v.maxy, d);
        o.bad = __shfl_down_sync(0xffffffffu, v.bad, d);
        v = box_merge(v, o);
    }
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < kBoxThreads / 32; w++) v = box_merge(v, sh[w]);
    }
    return v;
}

__global__ void bbox_partial_kernel(const double* x, const double* y, uint32_t n, BoxAcc* part) {
    BoxAcc a{DBL_MAX, -DBL_MAX, DBL_MAX, -DBL_MAX, 0u};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double xi = x[i], yi = y[i];
        if (!isfinite(xi) || !isfinite(yi)) a.bad = 1u;
        a.minx = fmin(a.minx, xi);
        a.maxx = fmax(a.maxx, xi);
        a.miny = fmin(a.miny, yi);
        a.maxy = fmax(a.maxy, yi);
    }
    a = box_block_reduce(a);
    if (threadIdx.x == 0) part[blockIdx.x] = a;
}

__global__ void bbox_final_kernel(const BoxAcc* part, int nparts, BBox* out) {
    BoxAcc a{DBL_MAX, -DBL_MAX, DBL_MAX, -DBL_MAX, 0u};
    for (int i = threadIdx.x; i < nparts; i += blockDim.x) a = box_merge(a, part[i]);
    a = box_block_reduce(a);
    if (threadIdx.x == 0) {
        // src/main.cpp:465-488: min starts at DBL_MAX, max at DBL_MIN
        out->minx = fmin(a.minx, DBL_MAX);
        out->miny = fmin(a.miny, DBL_MAX);
        out->maxx = fmax(a.maxx, DBL_MIN);
        out->maxy = fmax(a.maxy, DBL_MIN);
        out->tmaxx = a.maxx;
        out->tmaxy = a.maxy;
        out->nonfinite = a.bad;
        out->pad = 0;
    }
}

constexpr int kBoxBlocks = 1024;

}  // namespace

size_t bbox_scratch_bytes(uint32_t) { return sizeof(BoxAcc) * kBoxBlocks; }

void launch_bbox(const double* x, const double* y, uint32_t n, BBox* out, void* scratch,
                 cudaStream_t s) {
    int nb = (int)((n + kBoxThreads - 1) / kBoxThreads);
    if (nb > kBoxBlocks) nb = kBoxBlocks;
    if (nb < 1) nb = 1;
    BoxAcc* part = (BoxAcc*)scratch;
    VDB_COUNT_LAUNCH();
    bbox_partial_kernel<<<nb, kBoxThreads, 0, s>>>(x, y, n, part);
    VDB_COUNT_LAUNCH();
    bbox_final_kernel<<<1, kBoxThreads, 0, s>>>(part, nb, out);
}

}  // namespace vdb
