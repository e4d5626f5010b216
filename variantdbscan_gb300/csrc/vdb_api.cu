// Host driver and C ABI of libSharedVDBSCAN.so.
//
// Per dataset: bounding box, the reference's visit order and multiple-point
// boxes (shared by all variants), then per group of variants with the same
// epsilon: the grid, the count pass, the CSR neighbour table (whole, or in
// row chunks when it exceeds the memory budget) and, for each minpts of the
// group, union-find and labelling from scratch.  Several datasets of one call
// run concurrently on worker streams.
#include <float.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <map>
#include <mutex>
#include <numeric>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "../../include/vdbscan.h"
#include "vdb_internal.cuh"

using namespace vdb;

// ------------------------------------------------------------------ memory pool

namespace {

struct Pool {
    std::multimap<size_t, void*> free_blocks;
    std::map<void*, size_t> sizes;
    size_t held = 0;

    static size_t round(size_t b) {
        if (b < (1u << 20)) {
            size_t r = 256;
            while (r < b) r <<= 1;
            return r;
        }
        const size_t g = (size_t)2 << 20;
        return (b + g - 1) / g * g;
    }
    void* get(size_t bytes, cudaError_t* err) {
        size_t b = round(bytes ? bytes : 1);
        auto it = free_blocks.lower_bound(b);
        if (it != free_blocks.end() && it->first <= b + b / 4 + ((size_t)4 << 20)) {
            void* p = it->second;
            free_blocks.erase(it);
            return p;
        }
        void* p = nullptr;
        cudaError_t e = cudaMalloc(&p, b);
        if (e != cudaSuccess) {
            cudaGetLastError();
            trim();
            e = cudaMalloc(&p, b);
            if (e != cudaSuccess) {
                cudaGetLastError();
                *err = e;
                return nullptr;
            }
        }
        sizes[p] = b;
        held += b;
        return p;
    }
    void put(void* p) {
        if (!p) return;
        auto it = sizes.find(p);
        if (it == sizes.end()) return;
        free_blocks.emplace(it->second, p);
    }
    size_t cached_free() const {
        size_t b = 0;
        for (auto& kv : free_blocks) b += kv.first;
        return b;
    }
    void trim() {
        for (auto& kv : free_blocks) {
            cudaFree(kv.second);
            held -= sizes[kv.second];
            sizes.erase(kv.second);
        }
        free_blocks.clear();
    }
    void release_all() {
        for (auto& kv : sizes) cudaFree(kv.first);
        sizes.clear();
        free_blocks.clear();
        held = 0;
    }
};

}  // namespace

// Tile-shape decision of one table: dataset buffers, size and bounding box,
// epsilon and cells per epsilon.
struct TuneKey {
    const void *x, *y;
    uint32_t n;
    double minx, maxx, miny, maxy, eps;
    int r;
    bool operator<(const TuneKey& o) const {
        return std::tie(x, y, n, minx, maxx, miny, maxy, eps, r) <
               std::tie(o.x, o.y, o.n, o.minx, o.maxx, o.miny, o.maxy, o.eps, o.r);
    }
};

struct GraphEntry;

struct vdb_context {
    std::vector<GraphEntry*> graphs;         // captured calls (vdb_options.graph), oldest first
    std::map<TuneKey, uint32_t> tune_cache;  // autotuned tiles per table
    std::mutex tune_mu;
    vdb_context* tune_owner = nullptr;       // workers share their caller's cache
    int device = 0;
    int nsm = 1;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    Pool pool;
    std::string err;
    cudaEvent_t box_ready = nullptr;   // the bounding box has reached h_pinned
    DeviceStatus* d_status = nullptr;  // device status block, read back through h_status
    DeviceStatus* h_status = nullptr;  // pinned host mirror
    void* h_pinned = nullptr;          // pinned staging (EpsParams, scalars)
    size_t h_pinned_bytes = 0;
    int mem_share = 1;                 // contexts sharing the device memory budget
    std::vector<vdb_context*> workers; // stream contexts of concurrent batches
    std::mutex mu;
};

namespace {

struct VdbError {
    int code;
    std::string msg;
};

#define CK(call)                                                                         \
    do {                                                                                 \
        cudaError_t e_ = (call);                                                         \
        if (e_ != cudaSuccess)                                                           \
            throw VdbError{VDB_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)}; \
    } while (0)

// Allocations of one call, returned to the context pool when it ends.
// The bytes it holds (as the pool rounds them) and their peak: the call's
// device footprint.
struct Arena {
    vdb_context* ctx;
    std::vector<void*> ptrs;
    size_t cur = 0, peak = 0;
    // keep: nothing returns to the pool before the arena ends.  The arenas of
    // a captured graph (one per branch of concurrent datasets) reuse their
    // own returned blocks only: work within a branch is ordered, across
    // branches it is not.
    bool keep = false;
    std::multimap<size_t, void*> own_free;
    explicit Arena(vdb_context* c) : ctx(c) {}
    ~Arena() {
        for (void* p : ptrs) ctx->pool.put(p);
    }
    template <class T>
    T* get(size_t count) {
        if (keep) {
            const size_t b = Pool::round(count * sizeof(T) ? count * sizeof(T) : 1);
            auto it = own_free.lower_bound(b);
            if (it != own_free.end() && it->first <= b + b / 4 + ((size_t)4 << 20)) {
                void* p = it->second;
                own_free.erase(it);
                return (T*)p;
            }
        }
        cudaError_t e = cudaSuccess;
        void* p = ctx->pool.get(count * sizeof(T), &e);
        if (!p) {
            char buf[160];
            snprintf(buf, sizeof buf, "device allocation of %zu bytes failed: %s",
                     count * sizeof(T), cudaGetErrorString(e));
            throw VdbError{VDB_ERR_NOMEM, buf};
        }
        ptrs.push_back(p);
        cur += ctx->pool.sizes[p];
        peak = std::max(peak, cur);
        return (T*)p;
    }
    void put(void* p) {
        if (keep) {
            if (p) own_free.emplace(ctx->pool.sizes[p], p);
            return;
        }
        auto it = std::find(ptrs.begin(), ptrs.end(), p);
        if (it != ptrs.end()) {
            ptrs.erase(it);
            cur -= ctx->pool.sizes[p];
            ctx->pool.put(p);
        }
    }
};

// ------------------------------------------------------------ host parameters

// Largest double t with sqrt(t) <= eps (src/DBScan.cpp:687, 699-702 compare
// sqrt(d2) <= eps; sqrt is correctly rounded and monotone).
double eps_sq_threshold(double eps) {
    if (!(eps >= 0.0)) return -1.0;
    if (isinf(eps)) return INFINITY;
    double t = eps * eps;
    while (t > 0.0 && sqrt(t) > eps) t = nextafter(t, 0.0);
    for (;;) {
        double u = nextafter(t, INFINITY);
        if (isinf(u) || sqrt(u) > eps) break;
        t = u;
    }
    return t;
}

// Rounds w up to 12 significant bits: multiples k*w with |k| < 2^12 are then
// exact in FP32 (and FP64).
double round_up_12bits(double w) {
    int e = 0;
    double m = frexp(w, &e);
    double m12 = ceil(m * 4096.0) / 4096.0;
    return ldexp(m12, e);
}

constexpr uint64_t kMaxCells = (uint64_t)1 << 28;

struct HostBox {
    double minx, maxx, miny, maxy;  // true extremes
};

GridParams make_grid(const HostBox& hb, double w_target, uint32_t G,
                     uint64_t max_cells = kMaxCells) {
    GridParams g;
    memset(&g, 0, sizeof g);
    double rx = hb.maxx - hb.minx, ry = hb.maxy - hb.miny;
    if (!isfinite(rx) || !isfinite(ry) || !(w_target >= 0.0))
        throw VdbError{VDB_ERR_INVALID_ARG, "coordinate range is not finite"};
    // cells no finer than the target (padded), than range/2^26 (cell indices
    // stay far from FP64 rounding trouble) or than 2^-1000
    double w = std::max({w_target * (1.0 + 0x1p-12), rx * 0x1p-26, ry * 0x1p-26, 0x1p-1000});
    w = round_up_12bits(w);
    // at most kMaxCells cells
    for (int it = 0; it < 64; it++) {
        double fx = floor(rx / w) + 1.0, fy = floor(ry / w) + 1.0;
        double padx = ceil(fx / G) * G;
        if (padx * fy <= (double)max_cells) break;
        w = round_up_12bits(w * 2.0);
    }
    {
        double fx = floor(rx / w) + 1.0, fy = floor(ry / w) + 1.0;
        if (!(fx >= 1.0 && fy >= 1.0 && ceil(fx / G) * G * fy <= (double)max_cells))
            throw VdbError{VDB_ERR_INVALID_ARG, "grid cannot cover the coordinate range"};
    }
    g.x0 = hb.minx;
    g.y0 = hb.miny;
    g.w = w;
    g.ncx = (uint32_t)(floor((hb.maxx - hb.minx) / w) + 1.0);
    g.ncy = (uint32_t)(floor((hb.maxy - hb.miny) / w) + 1.0);
    g.G = G;
    g.ncx_pad = (g.ncx + G - 1) / G * G;
    g.ncells = (uint64_t)g.ncx_pad * g.ncy;
    return g;
}

int bits_for(uint64_t v) {
    int b = 0;
    while (b < 32 && (((uint64_t)1 << b) <= v)) b++;
    return b;
}

// Distance-test parameters of eps on grid g.  Cells (i, j) relative to a query
// cell are scanned when their nearest points can be within eps:
// (max(|i|-1,0)^2 + max(|j|-1,0)^2) * w^2 <= eps^2 (1 + 2^-16).  The margin
// covers the FP64 rounding of the cell index; w carries a 2^-12 padding so
// that cells exactly eps away are not scanned.
EpsParams make_eps(double eps, const GridParams& g, const HostBox& hb, bool want_mixed) {
    EpsParams p;
    memset(&p, 0, sizeof p);
    p.eps = eps;
    p.thr = eps_sq_threshold(eps);
    const double rho = eps / g.w;
    const double lim = rho * rho * (1.0 + 0x1p-16);
    int R = 0;
    while (R + 1 < (kMaxRows - 1) / 2 + 1) {
        double gy = (double)std::max(R + 1 - 1, 0);
        if (gy * gy <= lim) R++;
        else break;
    }
    p.rho = R;
    int maxreach = 0;
    for (int dy = -R; dy <= R; dy++) {
        double gy = (double)std::max(std::abs(dy) - 1, 0);
        int gx = 0;
        while ((double)(gx + 1) * (gx + 1) + gy * gy <= lim) gx++;
        p.reach[dy + R] = gx + 1;
        maxreach = std::max(maxreach, gx + 1);
    }
    // |coordinates| and |cell origins|
    const double C = std::max(std::max(fabs(hb.minx), fabs(hb.maxx)),
                              std::max(fabs(hb.miny), fabs(hb.maxy))) + 2.0 * g.w;
    {
        double ulpC = nextafter(C + eps, INFINITY) - (C + eps);
        double tb = eps - 4.0 * ulpC;
        p.tbox = tb > 0.0 ? tb * tb * (1.0 - 0x1p-40) : -1.0;
    }
    // FP32 error bound of the squared distance on tile-relative coordinates
    const double u = 0x1p-24, ud = 0x1p-52;
    const double w = g.w;
    const double Rm = ((double)g.G + std::max(maxreach, R) + 1.0) * w;
    const double e_loc = u * 1.01 * w + 2.0 * ud * C;
    const double e_rel = e_loc + u * Rm;
    const double Edx = 2.0 * e_rel + 2.0 * u * Rm;
    const double D = eps;
    double band = 8.0 * (4.0 * D * Edx + 2.0 * Edx * Edx + 4.0 * u * D * D) + 0x1p-22 * eps * eps;
    const double e2 = eps * eps;
    p.mixed = 0;
    if (want_mixed && isfinite(e2) && e2 > 1e-30 && e2 < 1e30 && band < 0.25 * e2) {
        if (e2 - band > p.tbox) band = e2 - p.tbox;
        if (band < 0.25 * e2) {
            float lo = (float)(e2 - band), hi = (float)(e2 + band);
            lo = nextafterf(lo, 0.0f);
            hi = nextafterf(hi, INFINITY);
            p.lo32 = lo;
            p.hi32 = hi;
            p.mixed = 1;
            // Count-pass filter on the quadratic form: with q, c the FP32
            // cell-relative coordinates (|q|, |c| <= Rm per coordinate),
            // nS = fl(hc - fl(qx*cx + fl(qy*cy - hq))), hc = fl(|c|^2/2),
            // hq = fl((|q|^2 - L)/2) differs from (d2_f - L)/2 (d2_f the
            // squared distance of the FP32 coordinates) by at most the sum of
            // its roundings, < 13.5 u Rm^2 + 2 u L; dS doubles that.  Then
            //   nS <= 0  =>  d2_f <= L + 2 dS = lo32 (1 - 2^-20)
            //            =>  FP32 d2 < lo32 (its rounding is < 5u relative): in;
            //   nS > W   =>  d2_f > hi32 (1 + 2^-20)  =>  FP32 d2 > hi32: out.
            const double dS = 32.0 * u * (Rm * Rm + e2);
            const double L = (double)lo * (1.0 - 0x1p-20) - 2.0 * dS;
            float L32 = (float)L;
            if ((double)L32 > L) L32 = nextafterf(L32, 0.0f);
            const double W = 0.5 * ((double)hi * (1.0 + 0x1p-20) - (double)L32) + dS;
            p.L32 = L32;
            float w32 = (float)W;
            if ((double)w32 < W) w32 = nextafterf(w32, INFINITY);
            p.w32 = w32;
            if (!(L > 0.5 * e2)) p.mixed = 0;  // bound too loose for these coordinates
        }
    }
    return p;
}

struct Options {
    int precision = VDB_PRECISION_MIXED;
    int schedule = VDB_SCHEDULE_BATCHED;
    int location = VDB_LOC_HOST;
    int cells_per_eps = 0;
    int verbose = 0;
    int64_t budget = 0;
    int streams = 0;
    int table_rows = VDB_TABLE_ALL;
    int table_hash = 0;
    int entry_bytes = 0;  // 0 / 2: compact entries where they fit; 4: always 32-bit
    bool reuse = true;    // labellings start from earlier variants' components
    int tile_cells = 0;   // cells per tile group G; 0 = autotuned per table
    int unit_words = 0;   // work-unit size in bitmap words; 0 = by dataset size
    bool graph = false;   // repeated calls replayed as one CUDA graph
};

struct Timer {
    std::vector<cudaEvent_t> evs;
    cudaStream_t s;
    bool off;  // no events (stream capture into conditional bodies takes none)
    explicit Timer(cudaStream_t st, bool off_ = false) : s(st), off(off_) {}
    ~Timer() {
        for (auto e : evs)
            if (e) cudaEventDestroy(e);
    }
    size_t mark() {
        cudaEvent_t e = nullptr;
        if (!off) {
            CK(cudaEventCreate(&e));
            CK(cudaEventRecord(e, s));
        }
        evs.push_back(e);
        return evs.size() - 1;
    }
    double ms(size_t a, size_t b) {
        float f = 0.f;
        if (!off) cudaEventElapsedTime(&f, evs[a], evs[b]);
        return (double)f;
    }
};

struct Group {
    double eps;
    std::vector<std::pair<uint32_t, uint32_t>> vars;  // (minpts, variant index), minpts desc
};

// Grid cells per eps when the caller leaves it open: two.  The cells are then
// cliques (cell union instead of one union per core-core edge) and a one-cell
// tile scans 25 cells of (eps/2)^2, 1.99x the disc's area, against 2.86x for
// cells of width eps.  Three cells per eps scan 1.6x the disc but multiply the
// cell pairs the clustering searches (measured slower at every eps of the
// variant sweep and the lattice), so the cell size is a fixed choice and the
// tile shape is the tuned one (choose_tile_cells).
constexpr int kCellsPerEps = 2;

// Tile-shape autotuner.  A tile is up to 64 consecutive cell-ordered points of
// one group of G cells of a grid row; its candidates are the cells within
// reach of the whole group.  Larger groups put more queries in a tile (sparse
// grids leave most of a warp's 64 query slots empty with G = 1) at the price
// of more candidates per query.  The cost of shape G is modelled from the
// statistics of launch_tile_costs, measured on the grid itself:
//   lane-slot tests  C * 32 * ceil(P/32)  x kCostSlot   (count and expand
//                                                         passes scale with it)
//   tiles            ceil(P/64)           x kCostTile   (per-tile fixed work)
// The weights are a non-negative least-squares fit of the count + expand time
// of single tables measured for every G on 17 tables (2M-point sweep at 4 eps,
// 1M uniform points at 4 eps, blob datasets of 2e4-4e5 points at 3 eps, each
// G timed 3 times); a bitmap-word term fitted to zero weight and was dropped.
// The fitted model picks the fastest shape on every table of >= 4e5 points
// and recovers 97% of the time the best shapes save over G = 1; below about
// 1e5 points the shapes differ by a few percent and the model's picks are no
// better than G = 1, so small datasets keep G = 1 (kTuneMinPoints).  A shape
// replaces G = 1 only when it models at least 5% cheaper.  The statistics come
// from about 65,536 sampled non-empty cells in runs of 64 (launch_tile_costs),
// which track the exact sums within a few percent on the tables above.
constexpr double kCostSlot = 6.9e-13, kCostTile = 2.8e-9;  // seconds
constexpr uint32_t kTuneMinPoints = 131072;
constexpr uint32_t kSmallUnitPoints = 1u << 18;  // smaller work units below this many points

uint32_t choose_tile_cells(const unsigned long long* sums) {
    double best = 0.0, base = 0.0;
    uint32_t G = 1;
    for (int i = 0; i < kTuneShapes; i++) {
        const double c = kCostSlot * (double)sums[2 * i] + kCostTile * (double)sums[2 * i + 1];
        if (i == 0) base = best = c;
        else if (c < best) {
            best = c;
            G = 1u << i;
        }
    }
    return best < 0.95 * base ? G : 1u;
}

// Worker streams of a multi-dataset call: datasets run concurrently so that
// one dataset's host waits and small grids are covered by the others, but
// every worker adds a memory pool and a host thread, and beyond 4 workers the
// variant-throughput of the 64-dataset batch fell (1 / 4 / 8 / 16 workers:
// 1.4 / 2.0 / 1.1 / 0.5 x 10^8 variant-points/s).  The work of a dataset is
// taken as points x distinct epsilons (its tables); with W the total and M the
// largest, no more than W / M workers can be kept busy.
int autotune_streams(const vdb_dataset* ds, int nds) {
    double W = 0.0, M = 0.0;
    for (int i = 0; i < nds; i++) {
        std::vector<double> e(ds[i].eps, ds[i].eps + (ds[i].eps ? ds[i].nv : 0));
        std::sort(e.begin(), e.end());
        const double tables = (double)(std::unique(e.begin(), e.end()) - e.begin());
        const double w = (double)ds[i].n * std::max(tables, 1.0);
        W += w;
        M = std::max(M, w);
    }
    if (nds <= 1 || M <= 0.0) return std::max(nds, 0) > 0 ? 1 : 0;
    const int k = (int)std::floor(W / M);
    return std::max(1, std::min({k, 4, nds}));
}

void read_status(vdb_context* ctx, cudaStream_t s) {
    CK(cudaMemcpyAsync(ctx->h_status, ctx->d_status, sizeof(DeviceStatus),
                       cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
}

void check_flags(const DeviceStatus& st) {
    const uint32_t f = st.flags;
    if (f & kStatGuard) {
        char buf[160];
        snprintf(buf, sizeof buf, "index guard %u failed (value %llu)", st.guard_site,
                 (unsigned long long)st.guard_value);
        throw VdbError{VDB_ERR_CUDA, buf};
    }
    if (f & kStatNonFinite)
        throw VdbError{VDB_ERR_INVALID_ARG, "non-finite coordinate"};
    if (f & kStatDegenerate)
        throw VdbError{VDB_ERR_DEGENERATE,
                       "zero-width bounding box: the reference reports bins out of range"};
    if (f & kStatAsymOverflow)
        throw VdbError{VDB_ERR_CAPACITY, "asymmetric pair list overflowed"};
    if (f & kStatResolveOverflow)
        throw VdbError{VDB_ERR_CAPACITY, "too many one-way core-core edges"};
    if (f & kStatRowOverflow)
        throw VdbError{VDB_ERR_CUDA, "fill pass disagrees with count pass"};
    if (f & kStatUnionStall)
        throw VdbError{VDB_ERR_CUDA, "union-find retry limit reached"};
}

constexpr uint32_t kAsymCap = 1u << 20;

// Free device memory plus blocks this context holds in its pool.
// Free device memory plus blocks this context holds in its pool, divided
// among the contexts that run concurrently on the device.
double avail_bytes(vdb_context* ctx) {
    size_t fb = 0, tb = 0;
    CK(cudaMemGetInfo(&fb, &tb));
    return ((double)fb + (double)ctx->pool.cached_free()) / ctx->mem_share;
}

// Rows [r_lo, r_hi) of the neighbour table = tiles [t_lo, t_hi) = work units
// [u_lo, u_hi), entries [e_lo, e_hi).  The whole table: t_hi = 0xffffffff and
// u_hi = 0 (no limits).
struct RowChunk {
    uint32_t t_lo, t_hi, u_lo, u_hi, r_lo, r_hi;
    uint64_t e_lo, e_hi;
};

// Union-find state of one variant.
struct UfState {
    uint32_t *parent, *seed, *cstart, *best, *cluster_no, *pos_flag;
};

// Splits the table into row chunks of whole tiles holding at most cap
// entries each (greedy, in tile order).
std::vector<RowChunk> plan_row_chunks(vdb_context* ctx, const uint32_t* tiles,
                                      const uint32_t* ntiles_dev, const uint32_t* tuoff,
                                      const unsigned long long* off, uint32_t n, uint64_t cap,
                                      cudaStream_t s) {
    uint32_t nt = 0;
    CK(cudaMemcpyAsync(ctx->h_pinned, ntiles_dev, 4, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    memcpy(&nt, ctx->h_pinned, 4);
    std::vector<uint32_t> ht((size_t)nt + 1), hu((size_t)nt + 1);
    std::vector<unsigned long long> ho((size_t)n + 1);
    CK(cudaMemcpyAsync(ht.data(), tiles, ((size_t)nt + 1) * 4, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(hu.data(), tuoff, ((size_t)nt + 1) * 4, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(ho.data(), off, ((size_t)n + 1) * 8, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (ht[nt] != n) throw VdbError{VDB_ERR_CUDA, "tile list does not end at n"};
    std::vector<RowChunk> out;
    uint32_t t = 0;
    while (t < nt) {
        const uint64_t e0 = ho[ht[t]];
        uint32_t t1 = t;
        while (t1 < nt && ho[ht[t1 + 1]] - e0 <= cap) t1++;
        if (t1 == t)
            throw VdbError{VDB_ERR_NOMEM, "the rows of one tile exceed the table budget"};
        out.push_back(RowChunk{t, t1, hu[t], hu[t1], ht[t], ht[t1], e0, ho[ht[t1]]});
        t = t1;
    }
    if (out.empty()) out.push_back(RowChunk{0, 0, 0, 0, 0, 0, 0, 0});
    return out;
}

// ------------------------------------------------------------- graph replay
//
// vdb_options.graph: the first call with a given key (datasets, variants,
// options) runs directly and records every value the host reads back from the
// device (bounding box, bitmap and work-unit sizes, neighbour and one-way
// pair counts) and every decision taken from free memory.  The same host code
// then runs once more under stream capture, taking those values from the
// record instead of waiting for the device.  Each read-back becomes a
// checkpoint: a one-thread kernel compares the device value with the record
// (the box must be equal; sizes at most the recorded ones, for which the
// buffers were sized) and sets the condition of the IF node that holds the
// work up to the next checkpoint.  Later calls with the key replay the
// instantiated graph: one launch and one host wait per call, the datasets of
// a batch in concurrent branches of the graph.  A failed checkpoint skips
// the rest of the replay and the call runs directly.

struct GraphBuild {
    cudaGraph_t top = nullptr;
    uint32_t* d_bad = nullptr;  // 1-based index of the first failed checkpoint
    uint32_t nchk = 0;
};

struct GraphRec {
    bool capture = false;       // false: recording a direct run
    bool graphable = true;      // false: the run took a path that is not captured
    std::vector<uint64_t> vals; // values read back and decisions, in order
    size_t pos = 0;
    // capture
    GraphBuild* gb = nullptr;
    Arena* ar = nullptr;                 // buffers of this dataset's branch of the graph
    std::vector<cudaGraphNode_t> tails;  // last top-level nodes of this dataset's branch
    bool in_body = false;                // capturing into an IF body (else the top graph)
    DeviceStatus* d_status = nullptr;    // this dataset's status block
    DeviceStatus* h_status = nullptr;    // its pinned copy, written by each replay
    double *hx = nullptr, *hy = nullptr; // pinned sources of host inputs
    uint32_t* hlabels = nullptr;         // pinned destination of host labels
    // the copy nodes of host inputs and labels, and their device ends: a
    // replay points them at the caller's buffers when those are page-locked
    cudaGraphNode_t n_x = nullptr, n_y = nullptr, n_labels = nullptr;
    const void *dx = nullptr, *dy = nullptr, *dlabels = nullptr;
    uint64_t launches = 0;               // kernels of one replay of this dataset
    vdb_stats fixed;                     // per-call statistics fixed by the record

    void put(uint64_t v) { vals.push_back(v); }
    uint64_t take() {
        if (pos >= vals.size()) throw VdbError{VDB_ERR_CUDA, "graph capture: record exhausted"};
        return vals[pos++];
    }
};

// Capacity of a captured buffer whose recorded size was v: a replay may need
// up to a quarter more.
uint64_t graph_room(uint64_t v) { return v + v / 4 + 4096; }

// The same for a neighbour table of v entries of esz bytes, kept within the
// caller's table budget (the record fitted it, so v does).
uint64_t graph_table_room(uint64_t v, uint64_t esz, int64_t budget) {
    const uint64_t r = graph_room(v);
    if (budget <= 0) return r;
    return std::max(v, std::min(r, (uint64_t)budget / esz));
}

GraphCond graph_cond(const void* p, uint32_t kind, uint64_t a, uint64_t b = 0,
                     unsigned long long* sum = nullptr) {
    GraphCond c;
    memset(&c, 0, sizeof c);
    c.ptr = p;
    c.sum = sum;
    c.a = a;
    c.b = b;
    c.kind = kind;
    return c;
}

std::vector<cudaGraphNode_t> capture_deps(cudaStream_t s) {
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    unsigned long long id = 0;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    const cudaGraphEdgeData* ed = nullptr;
    size_t nd = 0;
    CK(cudaStreamGetCaptureInfo(s, &st, &id, &g, &deps, &ed, &nd));
    return std::vector<cudaGraphNode_t>(deps, deps + nd);
}

void capture_top(GraphRec& r, cudaStream_t s) {
    CK(cudaStreamBeginCaptureToGraph(s, r.gb->top, r.tails.empty() ? nullptr : r.tails.data(),
                                     nullptr, r.tails.size(), cudaStreamCaptureModeRelaxed));
    r.in_body = false;
}

void capture_end(GraphRec& r, cudaStream_t s) {
    if (!r.in_body) r.tails = capture_deps(s);  // (an IF body ends in its IF node)
    cudaGraph_t g = nullptr;
    CK(cudaStreamEndCapture(s, &g));
    r.in_body = false;
}

// Ends the current segment, appends the check kernel and an IF node to the
// dataset's branch of the top graph, and continues the capture in its body.
void capture_checkpoint(GraphRec& r, cudaStream_t s, GraphCheck chk) {
    GraphBuild& b = *r.gb;
    capture_end(r, s);
    chk.index = ++b.nchk;
    cudaGraphConditionalHandle h;
    CK(cudaGraphConditionalHandleCreate(&h, b.top, 0, cudaGraphCondAssignDefault));
    capture_top(r, s);
    launch_graph_check(chk, b.d_bad, h, s);
    CK(cudaGetLastError());
    capture_end(r, s);
    cudaGraphNodeParams p = {};
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = h;
    p.conditional.type = cudaGraphCondTypeIf;
    p.conditional.size = 1;
    cudaGraphNode_t node = nullptr;
    CK(cudaGraphAddNode(&node, b.top, r.tails.empty() ? nullptr : r.tails.data(), nullptr,
                        r.tails.size(), &p));
    r.tails.assign(1, node);
    CK(cudaStreamBeginCaptureToGraph(s, p.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                     cudaStreamCaptureModeRelaxed));
    r.in_body = true;
}

void run_dataset(vdb_context* ctx, const vdb_dataset& ds, const Options& o, vdb_stats* stats,
                 GraphRec* rec = nullptr) {
    cudaStream_t s = ctx->stream;
    const uint32_t n = ds.n, V = ds.nv;
    if (n == 0 || V == 0) return;
    if (!ds.x || !ds.y || !ds.eps || !ds.minpts || !ds.labels)
        throw VdbError{VDB_ERR_INVALID_ARG, "null pointer"};
    if (ds.mbb_size <= 0) throw VdbError{VDB_ERR_INVALID_ARG, "MBBsize must be positive"};
    if (o.tile_cells < 0 || o.tile_cells > 64)
        throw VdbError{VDB_ERR_INVALID_ARG, "tile_cells must be 0 (autotuned) or 1..64"};
    if (o.unit_words != 0 && o.unit_words != (int)kUnitWordsSmall && o.unit_words != 64 &&
        o.unit_words != (int)kUnitWords)
        throw VdbError{VDB_ERR_INVALID_ARG, "unit_candidates must be 0, 1024, 2048 or 4096"};
    // work units: 1024 candidates for datasets below 2^18 points (few units:
    // the longest one bounds the count and expand passes), else 4096
    const uint32_t unit_words = o.unit_words > 0 ? (uint32_t)o.unit_words
                                : n < kSmallUnitPoints ? kUnitWordsSmall
                                                       : kUnitWords;
    if (n > 0x7fffffffu) throw VdbError{VDB_ERR_TOO_LARGE, "more than 2^31-1 points"};

    // graph replay: recording a direct run, or capturing one from its record
    const bool capturing = rec && rec->capture;
    const bool recording = rec && !rec->capture;
    Arena local_ar(ctx);
    Arena& ar = capturing ? *rec->ar : local_ar;
    Timer tm(s, capturing);
    DeviceStatus* const d_st = capturing ? rec->d_status : ctx->d_status;
    const unsigned long long launches0 = g_launches.load();
    if (capturing) capture_top(*rec, s);
    const size_t t0 = tm.mark();
    const bool host = o.location == VDB_LOC_HOST;

    const double *x = ds.x, *y = ds.y;
    if (host) {
        double* dx = ar.get<double>(n);
        double* dy = ar.get<double>(n);
        CK(cudaMemcpyAsync(dx, capturing ? rec->hx : ds.x, (size_t)n * 8,
                           cudaMemcpyHostToDevice, s));
        if (capturing) {
            rec->n_x = capture_deps(s).at(0);
            rec->dx = dx;
        }
        CK(cudaMemcpyAsync(dy, capturing ? rec->hy : ds.y, (size_t)n * 8,
                           cudaMemcpyHostToDevice, s));
        if (capturing) {
            rec->n_y = capture_deps(s).at(0);
            rec->dy = dy;
        }
        x = dx;
        y = dy;
    }
    uint32_t* labels = host ? ar.get<uint32_t>((size_t)n * V) : ds.labels;

    // scratch sized for the largest primitive call
    size_t scr = std::max({radix_sort_scratch_bytes(n), scan_u32_to_u64_scratch_bytes(n + 1),
                           bbox_scratch_bytes(n),
                           resolve_scratch_bytes() + scan_u32_scratch_bytes(n)});
    char* scratch = ar.get<char>(scr);

    CK(cudaMemsetAsync(d_st, 0, sizeof(DeviceStatus), s));
    BBox* d_bb = ar.get<BBox>(1);
    launch_bbox(x, y, n, d_bb, scratch, s);
    if (!capturing) {
        CK(cudaMemcpyAsync(ctx->h_pinned, d_bb, sizeof(BBox), cudaMemcpyDeviceToHost, s));
        CK(cudaEventRecord(ctx->box_ready, s));
    }

    // visit order (shared by all variants): it reads the box on the device, so
    // it is queued before the host waits for the box's copy (the grid needs
    // it); the GPU sorts while the host sets up the grid
    uint32_t* vkey = ar.get<uint32_t>(n);
    uint32_t* vorder = ar.get<uint32_t>(n);
    uint32_t* pos = ar.get<uint32_t>(n);
    const uint32_t nmpb = (uint32_t)(((uint64_t)n + (uint32_t)ds.mbb_size - 1) / (uint32_t)ds.mbb_size);
    MpbBox* mpb = ar.get<MpbBox>(nmpb);
    launch_visit_keys(x, y, n, d_bb, vkey, vorder, d_st, s);
    radix_sort_pairs(vkey, vorder, n, bits_for(kVisitBins * kVisitBins - 1), scratch, s);
    launch_invert(vorder, n, pos, s);
    launch_mpb_boxes(x, y, vorder, n, ds.mbb_size, mpb, s);
    BBox hb_ref;
    memset(&hb_ref, 0, sizeof hb_ref);
    double* const box_f[6] = {&hb_ref.minx, &hb_ref.maxx, &hb_ref.miny,
                              &hb_ref.maxy, &hb_ref.tmaxx, &hb_ref.tmaxy};
    if (capturing) {
        // the replay goes on with points inside the recorded box: the host
        // builds the grid and the error bounds from the box (min x, true max
        // x, min y, true max y), and both stay valid (the bounds conservative)
        // for points inside it
        GraphCheck chk;
        memset(&chk, 0, sizeof chk);
        for (int i = 0; i < 6; i++) {
            const uint64_t v = rec->take();
            memcpy(box_f[i], &v, 8);
        }
        uint64_t b[4];
        memcpy(&b[0], &hb_ref.minx, 8);
        memcpy(&b[1], &hb_ref.tmaxx, 8);
        memcpy(&b[2], &hb_ref.miny, 8);
        memcpy(&b[3], &hb_ref.tmaxy, 8);
        chk.c[0] = graph_cond(&d_bb->minx, kGcGeF64, b[0]);
        chk.c[1] = graph_cond(&d_bb->tmaxx, kGcLeF64, b[1]);
        chk.c[2] = graph_cond(&d_bb->miny, kGcGeF64, b[2]);
        chk.c[3] = graph_cond(&d_bb->tmaxy, kGcLeF64, b[3]);
        hb_ref.nonfinite = (uint32_t)rec->take();
        chk.c[4] = graph_cond(&d_bb->nonfinite, kGcMask32, 0xffffffffu, hb_ref.nonfinite);
        chk.n = 5;
        capture_checkpoint(*rec, s, chk);
    } else {
        CK(cudaEventSynchronize(ctx->box_ready));
        memcpy(&hb_ref, ctx->h_pinned, sizeof(BBox));
        if (recording) {
            for (int i = 0; i < 6; i++) {
                uint64_t v;
                memcpy(&v, box_f[i], 8);
                rec->put(v);
            }
            rec->put(hb_ref.nonfinite);
        }
    }
    if (hb_ref.nonfinite) throw VdbError{VDB_ERR_INVALID_ARG, "non-finite coordinate"};
    HostBox hb{hb_ref.minx, hb_ref.tmaxx, hb_ref.miny, hb_ref.tmaxy};
    ar.put(vkey);

    // variant groups
    std::vector<Group> groups;
    {
        std::vector<uint32_t> idx(V);
        for (uint32_t v = 0; v < V; v++) idx[v] = v;
        // epsilon descending (NaN last), minpts descending
        std::sort(idx.begin(), idx.end(), [&](uint32_t a, uint32_t b) {
            double ea = ds.eps[a], eb = ds.eps[b];
            bool na = ea != ea, nb2 = eb != eb;
            if (na != nb2) return nb2;
            if (!na && ea != eb) return ea > eb;
            if (ds.minpts[a] != ds.minpts[b]) return ds.minpts[a] > ds.minpts[b];
            return a < b;
        });
        for (uint32_t v : idx) {
            double e = ds.eps[v];
            bool sameg = !groups.empty() &&
                         (o.schedule == VDB_SCHEDULE_BATCHED
                              ? (groups.back().eps == e || (e != e && groups.back().eps !=
                                                                          groups.back().eps))
                              : false);
            if (!sameg) groups.push_back(Group{e, {}});
            groups.back().vars.push_back({ds.minpts[v], v});
        }
    }

    const size_t t_index = tm.mark();
    double ms_count = 0, ms_table = 0, ms_cluster = 0, ms_index_extra = 0;

    uint32_t* deg = ar.get<uint32_t>(n);
    unsigned long long* off = ar.get<unsigned long long>((size_t)n + 1);
    uint32_t* parent = ar.get<uint32_t>(n);
    uint32_t* seed = ar.get<uint32_t>(n);
    uint32_t* cstart = ar.get<uint32_t>(n);
    uint32_t* best = ar.get<uint32_t>(n);
    uint32_t* cluster_no = ar.get<uint32_t>((size_t)n + 1);
    uint32_t* pos_flag = ar.get<uint32_t>(n);
    uint32_t asym_cap = kAsymCap;  // grows when a count pass finds more one-way pairs
    AsymPair* asym = ar.get<AsymPair>(asym_cap);
    uint32_t* asym_n = ar.get<uint32_t>(4);
    uint32_t* tile_counter = asym_n + 1;
    EpsParams* d_ep = ar.get<EpsParams>(1);
    unsigned long long* tune_sums = ar.get<unsigned long long>(2 * kTuneShapes);
    uint32_t tile_cells_hist[8] = {0, 0, 0, 0, 0, 0, 0, 0};  // tables per log2(G)
    uint32_t* gkey = ar.get<uint32_t>(n);
    uint32_t* gorig = ar.get<uint32_t>(n);
    double2* gxy = ar.get<double2>(n);
    float2* glocal = ar.get<float2>(n);
    uint32_t* gpos = ar.get<uint32_t>(n);
    MpbBox* gbox = ar.get<MpbBox>(n);
    uint32_t* tflags = ar.get<uint32_t>(n);
    uint32_t* tscan = ar.get<uint32_t>((size_t)n + 1);
    uint32_t* tiles = ar.get<uint32_t>((size_t)n + 1);
    uint32_t* cscan = ar.get<uint32_t>((size_t)n + 1);
    uint32_t* clist = ar.get<uint32_t>((size_t)n + 1);
    uint32_t* crep = ar.get<uint32_t>(n);
    unsigned long long* tboff = ar.get<unsigned long long>((size_t)n + 1);
    uint32_t* tunits = ar.get<uint32_t>(n);
    uint32_t* tuoff = ar.get<uint32_t>((size_t)n + 1);
    uint32_t* bitmap = nullptr;
    uint64_t bitmap_cap = 0;
    uint32_t* unit_tile = nullptr;
    uint32_t* parts = nullptr;
    uint64_t unit_cap = 0;
    uint32_t* nbr = nullptr;
    size_t nbr_cap_bytes = 0;
    size_t table_alloc_max = 0;  // largest neighbour-table (or chunk) allocation
    uint32_t* ptile = nullptr;  // compact tables: tile of every cell-ordered point
    uint32_t* cell_start = nullptr;
    uint64_t cell_cap = 0;
    uint32_t* crow = nullptr;   // sparse grids: row directory
    uint64_t crow_cap = 0;
    uint32_t* ccx = nullptr;
    uint32_t *trow_s = nullptr, *trow_e = nullptr;  // tile row ranges (sparse grids, compact tables)
    size_t trow_cap = 0;

    const bool want_mixed = o.precision == VDB_PRECISION_MIXED;
    const int tq = table_tile_queries();
    const int nb_count = ctx->nsm * table_blocks_per_sm(false, want_mixed);
    const int nb_fill = ctx->nsm * table_blocks_per_sm(true, want_mixed);
    const int nb_expand16 = ctx->nsm * expand_blocks_per_sm(true);
    const int nb_expand32 = ctx->nsm * expand_blocks_per_sm(false);
    const int nb_warps = ctx->nsm * 8;
    uint64_t pairs = 0, asym_total = 0, entry_bytes = 0;
    uint32_t compact_tables = 0;
    uint32_t tables = 0, chunks = 0;
    std::vector<RowChunk> chunk_list;
    std::vector<std::pair<size_t, size_t>> table_marks;  // timer marks around table builds
    std::vector<UfState> states;                           // per-variant states (row chunks)
    struct GroupSpan {
        size_t cl0, cl1;                                   // timer marks around the clustering
        std::vector<std::pair<size_t, size_t>> tables;     // table builds of the group
        size_t first_cluster_table;                        // first build inside [cl0, cl1]
    };
    std::vector<GroupSpan> group_spans;
    // nested-epsilon reuse: components (seed per visit position) of the latest
    // labelled variant of each minpts, with the index of its epsilon group
    struct SavedComp {
        size_t group;
        uint32_t* comp;
    };
    std::map<uint64_t, SavedComp> saved_comp;
    size_t group_index = 0;
    // components from an earlier (larger) epsilon with the largest minpts <= mp
    auto comp_source = [&](uint64_t mp) -> const uint32_t* {
        if (!o.reuse) return nullptr;
        for (auto it = saved_comp.upper_bound(mp); it != saved_comp.begin();) {
            --it;
            if (it->second.group < group_index) return it->second.comp;
        }
        return nullptr;
    };
    auto save_comp = [&](const ClusterArgs& ca, uint64_t mp) {
        // (nothing reads the components of the last epsilon group)
        if (!o.reuse || mp == ~0ull || group_index + 1 >= groups.size()) return;
        auto it = saved_comp.find(mp);
        if (it == saved_comp.end())
            it = saved_comp.emplace(mp, SavedComp{group_index, ar.get<uint32_t>(n)}).first;
        it->second.group = group_index;
        launch_save_components(ca, it->second.comp, s);
    };
    // builds the rows of chunk c into nbr (expand from the bitmap, or the
    // fill pass when there is no bitmap)
    auto build_chunk = [&](TableArgs& t, const RowChunk& c, uint32_t nasym) {
        const size_t m0 = tm.mark();
        t.off_base = c.e_lo;
        t.tile_lo = c.t_lo;
        t.tile_end = c.t_hi;
        t.unit_lo = c.u_lo;
        t.unit_hi = c.u_hi;
        t.row_lo = c.r_lo;
        t.row_hi = c.r_hi;
        CK(cudaMemsetAsync(t.tile_counter, 0, 4, s));
        if (t.bitmap) {
            launch_expand(t, t.compact ? nb_expand16 : nb_expand32, s);
            if (nasym) launch_asym_flags(t, s);
        } else {
            launch_fill(t, nb_fill, s);
        }
        // hash of the rows just built (tables written in full only)
        if (o.table_hash && t.row_deg_lim == 0) launch_table_hash(t, gorig, nb_warps, s);
        CK(cudaGetLastError());
        table_marks.push_back({m0, tm.mark()});
        chunks++;
    };

    for (const Group& gr : groups) {
        const double eps = gr.eps;
        const bool none = !(eps >= 0.0);  // negative or NaN epsilon: empty neighbourhoods
        CK(cudaMemsetAsync(asym_n, 0, 4 * sizeof(uint32_t), s));
        uint64_t E = 0;
        GridParams g;
        bool clique = false;
        memset(&g, 0, sizeof g);
        TableArgs ta_args;
        memset(&ta_args, 0, sizeof ta_args);
        uint32_t group_asym = 0;
        bool chunked = false;
        bool compact = false;  // 16-bit table entries for this group's table
        chunk_list.assign(1, RowChunk{0, 0xffffffffu, 0, 0, 0, n, 0, 0});
        table_marks.clear();
        // unique minpts of the group, largest first; a repeated minpts copies
        // the labels of the variant before it
        std::vector<std::pair<uint32_t, uint64_t>> slots;    // (variant, minpts)
        std::vector<std::pair<uint32_t, uint32_t>> copies;   // (variant, source variant)
        for (auto& mv : gr.vars) {
            const uint64_t mp = mv.first > 0x7fffffffu ? ~0ull : (uint64_t)mv.first;
            if (!slots.empty() && slots.back().second == mp)
                copies.push_back({mv.second, slots.back().first});
            else
                slots.push_back({mv.second, mp});
        }
        EpsParams ep;
        memset(&ep, 0, sizeof ep);
        if (none) {
            // (an empty-neighbourhood group uploads its order from the host:
            // not captured)
            if (capturing) throw VdbError{VDB_ERR_CUDA, "graph capture: path not captured"};
            if (recording) rec->graphable = false;
            CK(cudaMemsetAsync(deg, 0, (size_t)n * 4, s));
            CK(cudaMemsetAsync(off, 0, ((size_t)n + 1) * 8, s));
            // grid order = input order
            std::vector<uint32_t> iota(n);
            for (uint32_t i = 0; i < n; i++) iota[i] = i;
            CK(cudaMemcpyAsync(gorig, iota.data(), (size_t)n * 4, cudaMemcpyHostToDevice, s));
            CK(cudaStreamSynchronize(s));
            GridParams g1 = make_grid(hb, 1.0, 1);
            g1.w = 1.0;
            launch_grid_gather(x, y, gorig, pos, n, g1, gorig, gxy, glocal, gpos, s);
            launch_point_boxes(gpos, n, mpb, ds.mbb_size, gbox, s);
        } else {
            const size_t ta = tm.mark();
            const int r = o.cells_per_eps > 0 ? o.cells_per_eps : kCellsPerEps;
            if (isinf(eps)) {
                g = make_grid(hb, 1.0, 1);
                g.w = INFINITY;
                g.ncx = g.ncy = g.ncx_pad = 1;
                g.ncells = 1;
                ep.eps = eps;
                ep.thr = INFINITY;
                ep.tbox = INFINITY;
                ep.rho = 0;
                ep.reach[0] = 0;
                ep.mixed = 0;
            } else {
                // tile groups of G cells: fixed by the caller, or 1 until the
                // autotuner below has measured the grid
                g = make_grid(hb, eps / r, o.tile_cells > 0 ? (uint32_t)o.tile_cells : 1u);
                ep = make_eps(eps, g, hb, want_mixed);
            }
            // grid
            // far more cells than points (small eps over a wide box): a row
            // directory of the non-empty cells instead of a dense cell array,
            // so that the grid costs O(points + rows), not O(cells)
            g.sparse = g.ncells > 32ull * n + (1ull << 22) ? 1u : 0u;
            launch_grid_keys(x, y, n, g, gkey, gorig, s);
            radix_sort_pairs(gkey, gorig, n, bits_for(g.ncells - 1), scratch, s);
            launch_grid_gather(x, y, gorig, pos, n, g, gkey, gxy, glocal, gpos, s);
            launch_point_boxes(gpos, n, mpb, ds.mbb_size, gbox, s);
            auto build_cell_start = [&]() {
                if (g.sparse) return;
                if (g.ncells + 1 > cell_cap) {
                    if (cell_start) ar.put(cell_start);
                    cell_start = ar.get<uint32_t>(g.ncells + 1);
                    cell_cap = g.ncells + 1;
                }
                CK(cudaMemsetAsync(cell_start, 0xff, (g.ncells + 1) * 4, s));
                launch_cell_marks(gkey, n, cell_start, g.ncells, s);
                size_t need = suffix_min_u32_scratch_bytes(g.ncells + 1);
                char* sm = need <= scr ? scratch : ar.get<char>(need);
                suffix_min_u32(cell_start, g.ncells + 1, sm, s);
            };
            build_cell_start();
            // non-empty cells (clist) and the cell index of each cell's first point
            launch_tile_flags(gkey, n, 1, 0xffffffffu, tflags, s);
            scan_u32(tflags, cscan, n, scratch, s);
            launch_tile_write(tflags, cscan, n, clist, s);
            if (g.sparse) {
                if ((uint64_t)g.ncy + 1 > crow_cap) {
                    if (crow) ar.put(crow);
                    crow = ar.get<uint32_t>((size_t)g.ncy + 1);
                    crow_cap = (uint64_t)g.ncy + 1;
                }
                if (!ccx) ccx = ar.get<uint32_t>(n);
                CK(cudaMemsetAsync(crow, 0xff, ((size_t)g.ncy + 1) * 4, s));
                launch_cell_rows(gkey, clist, cscan + n, n, g, crow, ccx, s);
                size_t need = suffix_min_u32_scratch_bytes((uint64_t)g.ncy + 1);
                char* sm = need <= scr ? scratch : ar.get<char>(need);
                suffix_min_u32(crow, (uint64_t)g.ncy + 1, sm, s);
            }
            // tile shape: the cost model of choose_tile_cells on the grid's
            // own statistics (sampled non-empty cells); a new G only re-pads
            // the rows, so the keys are rewritten without sorting again (the
            // row directory of sparse grids does not depend on the padding)
            if (o.tile_cells <= 0 && isfinite(g.w) && n >= kTuneMinPoints) {
                // decisions are kept per dataset (its buffers, size and box)
                // and epsilon: a repeated call measures nothing
                const TuneKey key{ds.x, ds.y, n, hb.minx, hb.maxx, hb.miny, hb.maxy, eps, r};
                vdb_context* tc = ctx->tune_owner ? ctx->tune_owner : ctx;
                uint32_t G = 0;
                {
                    std::lock_guard<std::mutex> lk(tc->tune_mu);
                    auto it = tc->tune_cache.find(key);
                    if (it != tc->tune_cache.end()) G = it->second;
                }
                if (G == 0) {
                    if (capturing)
                        throw VdbError{VDB_ERR_CUDA, "graph capture: tile shape not recorded"};
                    memcpy(ctx->h_pinned, &ep, sizeof ep);
                    CK(cudaMemcpyAsync(d_ep, ctx->h_pinned, sizeof ep, cudaMemcpyHostToDevice, s));
                    CK(cudaMemsetAsync(tune_sums, 0, 2 * kTuneShapes * sizeof(unsigned long long),
                                       s));
                    launch_tile_costs(g, d_ep, gkey, cell_start, crow, ccx, clist, cscan + n, n,
                                      tune_sums, s);
                    char* hs = (char*)ctx->h_pinned + 2048;
                    CK(cudaMemcpyAsync(hs, tune_sums, 2 * kTuneShapes * sizeof(unsigned long long),
                                       cudaMemcpyDeviceToHost, s));
                    CK(cudaStreamSynchronize(s));
                    unsigned long long sums[2 * kTuneShapes];
                    memcpy(sums, hs, sizeof sums);
                    G = choose_tile_cells(sums);
                    std::lock_guard<std::mutex> lk(tc->tune_mu);
                    if (tc->tune_cache.size() >= 4096) tc->tune_cache.clear();
                    tc->tune_cache[key] = G;
                }
                GridParams g2 = make_grid(hb, eps / r, G);
                // (a padding that would exceed the cell limit coarsens the
                // cells: such a shape is not taken)
                if (G != g.G && g2.ncx == g.ncx && g2.ncy == g.ncy && g2.w == g.w) {
                    g2.sparse = g.sparse;
                    launch_grid_rekey(gkey, n, g.ncx_pad, g2.ncx_pad, s);
                    g = g2;
                    build_cell_start();
                    ep = make_eps(eps, g, hb, want_mixed);
                }
            }
            if (isfinite(g.w)) {
                int lg = 0;
                while ((1u << lg) < g.G && lg < 7) lg++;
                tile_cells_hist[lg]++;
            }
            const bool mixed = ep.mixed != 0;
            launch_tile_flags(gkey, n, g.G, (uint32_t)tq, tflags, s);
            scan_u32(tflags, tscan, n, scratch, s);
            launch_tile_write(tflags, tscan, n, tiles, s);
            // cells are cliques when two points of one cell always pass the
            // distance test without a box check: 2 w^2 below thr and tbox
            clique = isfinite(g.w) && 2.0 * g.w * g.w * (1.0 + 0x1p-20) <= std::min(ep.thr, ep.tbox);
            if (capturing) {
                launch_store_eps(d_ep, ep, s);
            } else {
                memcpy(ctx->h_pinned, &ep, sizeof ep);
                CK(cudaMemcpyAsync(d_ep, ctx->h_pinned, sizeof ep, cudaMemcpyHostToDevice, s));
            }
            const size_t tb = tm.mark();

            ta_args.g = g;
            ta_args.ep = d_ep;
            ta_args.mixed = mixed ? 1 : 0;
            ta_args.tiles = tiles;
            ta_args.ntiles = tscan + n;
            ta_args.tile_end = 0xffffffffu;
            ta_args.tile_counter = tile_counter;
            ta_args.cell_start = cell_start;
            // compact entries are possible when the caller allows them and a
            // warp can hold the tile's row segments; their tile row ranges
            // are then kept for every tile.  By default, tables of border rows
            // only (small, read entry by entry) keep 32-bit entries.
            const bool compact_ok = o.entry_bytes != 4 && 2 * ep.rho + 1 <= 32 &&
                                    (o.entry_bytes == 2 || o.table_rows != VDB_TABLE_BORDER);
            if (g.sparse || compact_ok) {
                const size_t nr = (size_t)n * (size_t)(2 * ep.rho + 1);
                if (nr > trow_cap) {
                    if (trow_s) ar.put(trow_s);
                    if (trow_e) ar.put(trow_e);
                    trow_s = ar.get<uint32_t>(nr);
                    trow_e = ar.get<uint32_t>(nr);
                    trow_cap = nr;
                }
                ta_args.trow_s = trow_s;
                ta_args.trow_e = trow_e;
            }
            ta_args.crow = crow;
            ta_args.ccx = ccx;
            ta_args.clist = clist;
            ta_args.gkey = gkey;
            ta_args.glocal = glocal;
            ta_args.gxy = gxy;
            ta_args.gpos = gpos;
            ta_args.gbox = gbox;
            ta_args.n = n;
            ta_args.deg = deg;
            ta_args.off = off;
            ta_args.asym = asym;
            ta_args.asym_n = asym_n;
            ta_args.asym_cap = asym_cap;
            ta_args.st = d_st;
            // layout of the count pass's test bitmap (one word per query and
            // 32 candidates of its tile), which the table pass expands
            ta_args.unit_words = unit_words;
            launch_tile_words(ta_args, tflags, tunits, nb_warps, s);
            scan_u32_to_u64(tflags, tboff, n, scratch, s);
            scan_u32(tunits, tuoff, n, scratch, s);
            uint64_t bm_words = 0;
            uint32_t nunits = 0;
            uint32_t st_flags = 0;
            DeviceStatus status_before_count;
            memset(&status_before_count, 0, sizeof status_before_count);
            if (capturing) {
                // buffers sized with headroom over the record, checked
                // against what they hold
                bm_words = graph_room(rec->take());
                nunits = (uint32_t)std::min<uint64_t>(graph_room(rec->take()), 0xfffffffeu);
                st_flags = (uint32_t)rec->take();
                GraphCheck chk;
                memset(&chk, 0, sizeof chk);
                chk.c[0] = graph_cond(tboff + n, kGcLe64, bm_words);
                chk.c[1] = graph_cond(tuoff + n, kGcLe32, nunits);
                chk.c[2] = graph_cond(&d_st->flags, kGcMask32, kStatBitmapTooLarge, st_flags);
                chk.n = 3;
                capture_checkpoint(*rec, s, chk);
            } else {
                CK(cudaMemcpyAsync(ctx->h_pinned, tboff + n, 8, cudaMemcpyDeviceToHost, s));
                CK(cudaMemcpyAsync((char*)ctx->h_pinned + 8, tuoff + n, 4,
                                   cudaMemcpyDeviceToHost, s));
                read_status(ctx, s);
                status_before_count = *ctx->h_status;
                memcpy(&bm_words, ctx->h_pinned, 8);
                memcpy(&nunits, (char*)ctx->h_pinned + 8, 4);
                st_flags = ctx->h_status->flags & kStatBitmapTooLarge;
                if (recording) {
                    rec->put(bm_words);
                    rec->put(nunits);
                    rec->put(st_flags);
                }
            }
            // 16-bit entries (positions within work units)
            compact = compact_ok;
            ta_args.compact = compact ? 1 : 0;
            if (compact) {
                if (!ptile) ptile = ar.get<uint32_t>(n);
                ta_args.ptile = ptile;
                launch_tile_owner(ta_args, ptile, nb_warps, s);
            }
            // work units: (tile, chunk of unit_words bitmap words)
            if ((uint64_t)nunits + 1 > unit_cap) {
                if (unit_tile) ar.put(unit_tile);
                if (parts) ar.put(parts);
                unit_cap = (uint64_t)nunits + 1;
                unit_tile = ar.get<uint32_t>(unit_cap);
                parts = ar.get<uint32_t>(unit_cap * kUnitQ);
            }
            ta_args.tile_uoff = tuoff;
            ta_args.nunits = tuoff + n;
            ta_args.unit_tile = unit_tile;
            ta_args.parts = parts;
            launch_unit_list(ta_args, unit_tile, nb_warps, s);
            CK(cudaMemsetAsync(deg, 0, (size_t)n * 4, s));
            ta_args.bitmap = nullptr;
            ta_args.tile_boff = tboff;
            if (capturing) {
                // the recorded choice between the bitmap and the fill pass
                const bool want = rec->take() != 0;
                if (want && bm_words > bitmap_cap) {
                    if (bitmap) ar.put(bitmap);
                    bitmap = ar.get<uint32_t>(bm_words ? bm_words : 1);
                    bitmap_cap = bm_words;
                }
                if (want) ta_args.bitmap = bitmap;
            } else if (!(st_flags & kStatBitmapTooLarge)) {
                if (bm_words > bitmap_cap) {
                    if (bitmap) ar.put(bitmap);
                    bitmap = nullptr;
                    bitmap_cap = 0;
                    // the test bitmap is kept when it fits 35% of the memory
                    // (and the caller's table budget); else the fill pass
                    // re-tests the candidates instead
                    double cap = 0.35 * avail_bytes(ctx);
                    if (o.budget > 0) cap = std::min(cap, (double)o.budget);
                    if ((double)bm_words * 4.0 <= cap) {
                        bitmap = ar.get<uint32_t>(bm_words ? bm_words : 1);
                        bitmap_cap = bm_words;
                    }
                }
                if (bitmap && bm_words <= bitmap_cap) ta_args.bitmap = bitmap;
            }
            if (recording) rec->put(ta_args.bitmap ? 1 : 0);
            size_t tc = 0;
            for (;;) {
                CK(cudaMemsetAsync(tile_counter, 0, 4, s));
                launch_count(ta_args, nb_count, s);
                CK(cudaGetLastError());
                tc = tm.mark();
                scan_u32_to_u64(deg, off, n, scratch, s);
                if (capturing) break;
                CK(cudaMemcpyAsync(ctx->h_pinned, off + n, 8, cudaMemcpyDeviceToHost, s));
                CK(cudaMemcpyAsync((char*)ctx->h_pinned + 8, asym_n, 4, cudaMemcpyDeviceToHost, s));
                read_status(ctx, s);
                if (!(ctx->h_status->flags & kStatAsymOverflow)) break;
                if (recording) rec->graphable = false;  // (the re-count is not captured)
                // more one-way pairs than the list holds: grow it past the
                // counted number and run the count pass again
                uint32_t want = 0;
                memcpy(&want, (char*)ctx->h_pinned + 8, 4);
                uint64_t cap2 = (uint64_t)asym_cap * 2;
                while (cap2 < (uint64_t)want + want / 4) cap2 *= 2;
                if (cap2 > 0x7fffffffull)
                    throw VdbError{VDB_ERR_CAPACITY, "asymmetric pair list overflowed"};
                ar.put(asym);
                asym_cap = (uint32_t)cap2;
                asym = ar.get<AsymPair>(asym_cap);
                ta_args.asym = asym;
                ta_args.asym_cap = asym_cap;
                memcpy(ctx->h_pinned, &status_before_count, sizeof status_before_count);
                CK(cudaMemcpyAsync(ctx->d_status, ctx->h_pinned, sizeof(DeviceStatus),
                                   cudaMemcpyHostToDevice, s));
                CK(cudaMemsetAsync(asym_n, 0, sizeof(uint32_t), s));
                CK(cudaMemsetAsync(deg, 0, (size_t)n * 4, s));
                CK(cudaStreamSynchronize(s));
            }
            if (capturing) {
                E = graph_table_room(rec->take(), compact ? 2 : 4, o.budget);
                group_asym = (uint32_t)rec->take();
                // at most the recorded neighbours (the table's size); one-way
                // pairs only if the record had some (their flag pass runs then)
                GraphCheck chk;
                memset(&chk, 0, sizeof chk);
                chk.c[0] = graph_cond(off + n, kGcLe64, E, 0, &d_st->pairs);
                chk.c[1] = graph_cond(asym_n, kGcLe32, group_asym ? asym_cap : 0u);
                chk.c[2] = graph_cond(&d_st->flags, kGcMask32, kStatAsymOverflow, 0);
                chk.n = 3;
                capture_checkpoint(*rec, s, chk);
            } else {
                check_flags(*ctx->h_status);
                memcpy(&E, ctx->h_pinned, 8);
                memcpy(&group_asym, (char*)ctx->h_pinned + 8, 4);
                if (recording) {
                    rec->put(E);
                    rec->put(group_asym);
                }
            }
            asym_total += group_asym;
            ms_index_extra += tm.ms(ta, tb);
            ms_count += tm.ms(tb, tc);
            // rows to write: all, or (VDB_TABLE_BORDER, cells that are
            // cliques) those of points that are not core for the group's
            // largest minpts: the border pulls of every minpts read only
            // those, and off becomes the scan of their degrees
            uint64_t Erows = E;
            if (o.table_rows == VDB_TABLE_BORDER && clique && !slots.empty() &&
                slots.front().second > 0) {
                const uint64_t mp_max = slots.front().second;
                const uint32_t lim = mp_max >= 0xffffffffull ? 0xffffffffu : (uint32_t)mp_max;
                launch_masked_degrees(deg, n, lim, tflags, s);
                scan_u32_to_u64(tflags, off, n, scratch, s);
                if (capturing) {
                    Erows = graph_table_room(rec->take(), compact ? 2 : 4, o.budget);
                    GraphCheck chk;
                    memset(&chk, 0, sizeof chk);
                    chk.c[0] = graph_cond(off + n, kGcLe64, Erows);
                    chk.n = 1;
                    capture_checkpoint(*rec, s, chk);
                } else {
                    CK(cudaMemcpyAsync(ctx->h_pinned, off + n, 8, cudaMemcpyDeviceToHost, s));
                    CK(cudaStreamSynchronize(s));
                    memcpy(&Erows, ctx->h_pinned, 8);
                    if (recording) rec->put(Erows);
                }
                ta_args.row_deg_lim = lim;
            }
            chunk_list[0].e_hi = Erows;
            // neighbour table: whole when its entries (2 or 4 bytes each)
            // fit the budget (free device memory plus blocks cached by this
            // context, or the caller's table_budget_bytes); otherwise in row
            // chunks of whole tiles, each built and consumed before the next
            const uint64_t esz = compact ? 2 : 4;
            auto words_for = [&](uint64_t entries) { return (size_t)((entries * esz + 3) / 4); };
            chunked = o.budget > 0 && (int64_t)(Erows * esz) > o.budget;
            if (!chunked && Erows * esz > nbr_cap_bytes) {
                if (nbr) ar.put(nbr);
                nbr = nullptr;
                nbr_cap_bytes = 0;
                // (a captured call was recorded unchunked: its table fits)
                const int64_t budget = o.budget > 0 ? o.budget
                                       : capturing  ? INT64_MAX
                                                    : (int64_t)(avail_bytes(ctx) * 0.9);
                if ((int64_t)(Erows * esz) <= budget) {
                    const size_t w = std::max<size_t>(words_for(Erows), 1);
                    nbr = ar.get<uint32_t>(w);
                    nbr_cap_bytes = w * 4;
                } else {
                    chunked = true;
                }
            }
            if (chunked && capturing)
                throw VdbError{VDB_ERR_CUDA, "graph capture: chunked table not captured"};
            if (chunked && recording) rec->graphable = false;
            if (chunked) {
                // one union-find state per minpts of the group (the rows of
                // every chunk serve all of them), then the largest chunk
                // that the remaining memory allows
                while (states.size() < slots.size()) {
                    UfState u;
                    u.parent = ar.get<uint32_t>(n);
                    u.seed = ar.get<uint32_t>(n);
                    u.cstart = ar.get<uint32_t>(n);
                    u.best = ar.get<uint32_t>(n);
                    u.cluster_no = ar.get<uint32_t>((size_t)n + 1);
                    u.pos_flag = ar.get<uint32_t>(n);
                    states.push_back(u);
                }
                if (nbr) ar.put(nbr);
                nbr = nullptr;
                nbr_cap_bytes = 0;
                const int64_t budget = o.budget > 0 ? o.budget : (int64_t)(avail_bytes(ctx) * 0.9);
                const uint64_t cap = (uint64_t)std::max<int64_t>(budget / (int64_t)esz, 1);
                chunk_list = plan_row_chunks(ctx, tiles, tscan + n, tuoff, off, n, cap, s);
                uint64_t mx = 1;
                for (const RowChunk& c : chunk_list) mx = std::max<uint64_t>(mx, c.e_hi - c.e_lo);
                const size_t w = std::max<size_t>(words_for(mx), 1);
                nbr = ar.get<uint32_t>(w);
                nbr_cap_bytes = w * 4;
            }
            ta_args.nbr = nbr;
            table_alloc_max = std::max(table_alloc_max, nbr_cap_bytes);
            if (!chunked) {
                build_chunk(ta_args, chunk_list[0], group_asym);
            }
            tables++;
            pairs += E;
            entry_bytes += Erows * esz;
            compact_tables += compact ? 1u : 0u;
        }

        // clustering, minpts descending
        const size_t tcl0 = tm.mark();
        const size_t table_marks_before = table_marks.size();
        auto cluster_args = [&](size_t si) {
            ClusterArgs ca;
            memset(&ca, 0, sizeof ca);
            ca.n = n;
            ca.deg = deg;
            ca.minpts = slots[si].second;
            ca.minpts_prev = ~0ull;
            ca.off = off;
            ca.off_base = 0;
            ca.row_lo = 0;
            ca.row_hi = n;
            ca.nbr = nbr;
            ca.compact = compact ? 1 : 0;
            ca.ptile = ptile;
            ca.trow_s = trow_s;
            ca.trow_e = trow_e;
            ca.tiles = tiles;
            ca.tile_uoff = tuoff;
            ca.parts = parts;
            ca.unit_words = unit_words;
            ca.gpos = gpos;
            ca.gorig = gorig;
            if (chunked) {
                const UfState& u = states[si];
                ca.parent = u.parent;
                ca.seed = u.seed;
                ca.cstart = u.cstart;
                ca.best = u.best;
                ca.cluster_no = u.cluster_no;
                ca.pos_flag = u.pos_flag;
            } else {
                ca.parent = parent;
                ca.seed = seed;
                ca.cstart = cstart;
                ca.best = best;
                ca.cluster_no = cluster_no;
                ca.pos_flag = pos_flag;
            }
            ca.asym = asym;
            ca.asym_count = asym_n;
            ca.asym_cap = asym_cap;
            ca.labels_out = labels + (size_t)slots[si].first * n;
            ca.st = d_st;
            ca.g = g;
            ca.ep = d_ep;
            ca.gkey = gkey;
            ca.cell_start = cell_start;
            ca.crow = crow;
            ca.ccx = ccx;
            ca.clist = clist;
            ca.ncl = cscan + n;
            ca.cscan = cscan;
            ca.crep = crep;
            ca.glocal = glocal;
            ca.gxy = gxy;
            ca.gbox = gbox;
            return ca;
        };
        auto chunk_rows = [&](ClusterArgs& ca, const RowChunk& c) {
            ca.off_base = c.e_lo;
            ca.row_lo = c.r_lo;
            ca.row_hi = c.r_hi;
        };
        if (!chunked) {
            // the whole table is resident: one variant after the other on one
            // state; with reuse, a variant starts from the components of the
            // one before it (a larger minpts of the same epsilon: its cores
            // and edges are a subset of this variant's, so its unions hold)
            for (size_t si = 0; si < slots.size(); si++) {
                ClusterArgs ca = cluster_args(si);
                const bool chain = o.reuse && si > 0 && !none;
                if (chain) ca.minpts_prev = slots[si - 1].second;
                if (!none) ca.comp_prev = comp_source(slots[si].second);
                launch_uf_init(ca, !chain, s);
                if (!none) {
                    if (clique)
                        launch_cell_union(ca, nb_warps, s);
                    else
                        launch_uf_union(ca, nb_warps, s);
                }
                launch_uf_finish(ca, scratch, scratch + resolve_scratch_bytes(), s);
                if (!none) save_comp(ca, slots[si].second);
                launch_border_and_write(ca, nb_warps, s);
                CK(cudaGetLastError());
            }
        } else {
            // row chunks: every variant keeps its own state while the chunks
            // pass.  Cells that are cliques are united without the table;
            // otherwise every chunk is built once for the unions and once
            // more for the border pull.
            std::vector<ClusterArgs> cas;
            for (size_t si = 0; si < slots.size(); si++) {
                cas.push_back(cluster_args(si));
                cas.back().comp_prev = comp_source(slots[si].second);
                launch_uf_init(cas.back(), true, s);
                if (clique) launch_cell_union(cas.back(), nb_warps, s);
            }
            if (!clique) {
                for (const RowChunk& c : chunk_list) {
                    build_chunk(ta_args, c, group_asym);
                    for (ClusterArgs& ca : cas) {
                        chunk_rows(ca, c);
                        launch_uf_union(ca, nb_warps, s);
                    }
                }
            }
            for (size_t si = 0; si < cas.size(); si++) {
                launch_uf_finish(cas[si], scratch, scratch + resolve_scratch_bytes(), s);
                save_comp(cas[si], slots[si].second);
            }
            for (const RowChunk& c : chunk_list) {
                build_chunk(ta_args, c, group_asym);
                for (ClusterArgs& ca : cas) {
                    chunk_rows(ca, c);
                    launch_border_pull(ca, nb_warps, s);
                }
            }
            for (ClusterArgs& ca : cas) launch_label_write(ca, s);
            CK(cudaGetLastError());
        }
        for (auto& cp : copies)
            CK(cudaMemcpyAsync(labels + (size_t)cp.first * n, labels + (size_t)cp.second * n,
                               (size_t)n * 4, cudaMemcpyDeviceToDevice, s));
        // the group's status flags and times are read once the dataset ends
        // (no host wait between groups)
        const size_t tcl1 = tm.mark();
        group_spans.push_back(GroupSpan{tcl0, tcl1, table_marks, table_marks_before});
        group_index++;
    }
    launch_count_clusters(labels, n, V, ar.get<uint32_t>(V), d_st, s);
    if (capturing) {
        // the labels and the status block come back through pinned buffers
        // of the graph, after the last IF body
        capture_end(*rec, s);
        capture_top(*rec, s);
        if (host) {
            CK(cudaMemcpyAsync(rec->hlabels, labels, (size_t)n * V * 4, cudaMemcpyDeviceToHost, s));
            rec->n_labels = capture_deps(s).at(0);
            rec->dlabels = labels;
        }
        CK(cudaMemcpyAsync(rec->h_status, d_st, sizeof(DeviceStatus), cudaMemcpyDeviceToHost, s));
        capture_end(*rec, s);
        rec->launches = g_launches.load() - launches0;
        return;
    }
    if (host) {
        CK(cudaMemcpyAsync(ds.labels, labels, (size_t)n * V * 4, cudaMemcpyDeviceToHost, s));
    }
    const size_t tend = tm.mark();
    CK(cudaStreamSynchronize(s));
    read_status(ctx, s);
    check_flags(*ctx->h_status);
    for (const GroupSpan& gs : group_spans) {
        double in_cluster_tables = 0;
        for (size_t i = 0; i < gs.tables.size(); i++) {
            const double t = tm.ms(gs.tables[i].first, gs.tables[i].second);
            ms_table += t;
            if (i >= gs.first_cluster_table) in_cluster_tables += t;
        }
        ms_cluster += tm.ms(gs.cl0, gs.cl1) - in_cluster_tables;
    }
    if (recording) {
        // statistics a replay reports as recorded (the rest come from its
        // own status block)
        vdb_stats& f = rec->fixed;
        memset(&f, 0, sizeof f);
        f.tables = tables;
        f.table_chunks = chunks;
        f.asymmetric_pairs = asym_total;
        f.entry_bytes = entry_bytes;
        f.compact_tables = compact_tables;
        f.table_bytes = table_alloc_max;
        for (int i = 0; i < 8; i++) f.tables_by_tile_cells[i] = tile_cells_hist[i];
    }
    if (stats) {
        stats->pairs += pairs;
        stats->candidates += ctx->h_status->candidates;
        stats->retested += ctx->h_status->retested;
        stats->tables += tables;
        stats->kernel_launches += (uint32_t)(g_launches.load() - launches0);
        stats->asymmetric_pairs += asym_total;
        stats->table_chunks += chunks;
        stats->clusters += (uint32_t)ctx->h_status->clusters;
        stats->table_hash += ctx->h_status->table_hash;
        stats->entry_bytes += entry_bytes;
        stats->compact_tables += compact_tables;
        stats->reuse_skipped_pairs += ctx->h_status->reuse_skips;
        stats->device_bytes = std::max<uint64_t>(stats->device_bytes, ar.peak);
        stats->table_bytes = std::max<uint64_t>(stats->table_bytes, table_alloc_max);
        for (int i = 0; i < 8; i++) stats->tables_by_tile_cells[i] += tile_cells_hist[i];
        stats->ms_index += tm.ms(t0, t_index) + ms_index_extra;
        stats->ms_count += ms_count;
        stats->ms_table += ms_table;
        stats->ms_cluster += ms_cluster;
        stats->ms_total += tm.ms(t0, tend);
    }
}

Options to_options(const vdb_options* opts) {
    Options o;
    if (opts) {
        o.precision = opts->precision;
        o.schedule = opts->schedule;
        o.location = opts->location;
        o.cells_per_eps = opts->cells_per_eps;
        o.verbose = opts->verbose;
        o.budget = opts->table_budget_bytes;
        o.streams = opts->streams;
        o.table_rows = opts->table_rows;
        o.table_hash = opts->table_hash;
        o.entry_bytes = opts->table_entry_bytes;
        o.reuse = opts->no_reuse == 0;
        o.tile_cells = opts->tile_cells;
        o.unit_words = opts->unit_candidates / 32;
        if (opts->unit_candidates % 32) o.unit_words = -1;
        o.graph = opts->graph != 0;
    }
    // the plain schedule is the one-variant-at-a-time comparison path
    if (o.schedule == VDB_SCHEDULE_PLAIN) o.reuse = false;
    return o;
}

int init_context(vdb_context* ctx, void* stream) {
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        ctx->err = "no CUDA device";
        return VDB_ERR_NO_DEVICE;
    }
    cudaGetDevice(&ctx->device);
    cudaDeviceGetAttribute(&ctx->nsm, cudaDevAttrMultiProcessorCount, ctx->device);
    if (stream) {
        ctx->stream = (cudaStream_t)stream;
        ctx->own_stream = false;
    } else {
        if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess)
            return VDB_ERR_CUDA;
        ctx->own_stream = true;
    }
    if (cudaEventCreateWithFlags(&ctx->box_ready, cudaEventDisableTiming) != cudaSuccess)
        return VDB_ERR_CUDA;
    if (cudaMalloc(&ctx->d_status, sizeof(DeviceStatus)) != cudaSuccess) return VDB_ERR_NOMEM;
    if (cudaMallocHost(&ctx->h_status, sizeof(DeviceStatus)) != cudaSuccess) return VDB_ERR_NOMEM;
    ctx->h_pinned_bytes = 4096;
    if (cudaMallocHost(&ctx->h_pinned, ctx->h_pinned_bytes) != cudaSuccess) return VDB_ERR_NOMEM;
    return VDB_OK;
}

void add_stats(vdb_stats* a, const vdb_stats& b) {
    a->pairs += b.pairs;
    a->candidates += b.candidates;
    a->retested += b.retested;
    a->asymmetric_pairs += b.asymmetric_pairs;
    a->tables += b.tables;
    a->table_chunks += b.table_chunks;
    a->kernel_launches += b.kernel_launches;
    a->clusters += b.clusters;
    a->table_hash += b.table_hash;
    a->entry_bytes += b.entry_bytes;
    a->compact_tables += b.compact_tables;
    a->reuse_skipped_pairs += b.reuse_skipped_pairs;
    a->device_bytes = std::max(a->device_bytes, b.device_bytes);
    a->table_bytes = std::max(a->table_bytes, b.table_bytes);
    for (int i = 0; i < 8; i++) a->tables_by_tile_cells[i] += b.tables_by_tile_cells[i];
    a->ms_index += b.ms_index;
    a->ms_count += b.ms_count;
    a->ms_table += b.ms_table;
    a->ms_cluster += b.ms_cluster;
    a->ms_total += b.ms_total;
}

// Runs the datasets of one call on nw worker contexts, each with its own
// stream, memory pool and host thread, largest datasets first: while one
// dataset waits on a host read-back or runs a small grid, the others keep the
// GPU busy.  The workers share the device memory budget (mem_share).  The
// caller's stream is ordered before and after the work with events.
void run_concurrent(vdb_context* ctx, const vdb_dataset* ds, int nds, const Options& o, int nw,
                    vdb_stats* stats) {
    CK(cudaSetDevice(ctx->device));
    while ((int)ctx->workers.size() < nw) {
        vdb_context* w = new vdb_context();
        const int rc = init_context(w, nullptr);
        ctx->workers.push_back(w);  // destroyed with ctx, also after a failed init
        if (rc != VDB_OK) throw VdbError{rc, "cannot create a worker stream"};
    }
    for (int i = 0; i < nw; i++) {
        ctx->workers[i]->mem_share = nw;
        ctx->workers[i]->tune_owner = ctx;
    }
    cudaEvent_t ready = nullptr;
    CK(cudaEventCreateWithFlags(&ready, cudaEventDisableTiming));
    CK(cudaEventRecord(ready, ctx->stream));
    for (int i = 0; i < nw; i++) CK(cudaStreamWaitEvent(ctx->workers[i]->stream, ready, 0));
    std::vector<int> order(nds);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        return (uint64_t)ds[a].n * ds[a].nv > (uint64_t)ds[b].n * ds[b].nv;
    });
    std::atomic<int> next{0};
    std::atomic<bool> stop{false};
    std::vector<vdb_stats> part(nw);
    std::vector<int> codes(nw, VDB_OK);
    std::vector<std::string> errs(nw);
    auto body = [&](int wi) {
        vdb_context* w = ctx->workers[wi];
        memset(&part[wi], 0, sizeof(vdb_stats));
        try {
            CK(cudaSetDevice(ctx->device));
            while (!stop.load()) {
                const int k = next.fetch_add(1);
                if (k >= nds) break;
                run_dataset(w, ds[order[k]], o, &part[wi]);
            }
        } catch (const VdbError& e) {
            codes[wi] = e.code;
            errs[wi] = e.msg;
            stop = true;
            cudaStreamSynchronize(w->stream);
            cudaGetLastError();
        }
    };
    std::vector<std::thread> threads;
    for (int i = 1; i < nw; i++) threads.emplace_back(body, i);
    body(0);
    for (auto& t : threads) t.join();
    for (int i = 0; i < nw; i++) {
        cudaEvent_t e = nullptr;
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) == cudaSuccess) {
            cudaEventRecord(e, ctx->workers[i]->stream);
            cudaStreamWaitEvent(ctx->stream, e, 0);
            cudaEventDestroy(e);
        }
    }
    cudaEventDestroy(ready);
    for (int i = 0; i < nw; i++)
        if (codes[i] != VDB_OK) throw VdbError{codes[i], errs[i]};
    if (stats)
        for (const vdb_stats& p : part) add_stats(stats, p);
}

}  // namespace

// A captured call (vdb_options.graph).
struct GraphEntry {
    std::vector<uint64_t> key;       // datasets, variants and options of the call
    bool ok = false;                 // false: recorded as not captured (calls run directly)
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::vector<Arena*> ars;         // device buffers of the graph, one arena per branch
    std::vector<void*> pinned;       // pinned host buffers of the graph
    std::vector<GraphRec> recs;      // per dataset: staging buffers, status copy, statistics
    uint32_t* h_bad = nullptr;       // first failed checkpoint of the last replay (0: none)
    uint32_t checks = 0;
    uint64_t launches = 0;           // kernels of one replay
    cudaEvent_t e0 = nullptr, e1 = nullptr;
};

namespace {

constexpr size_t kMaxGraphs = 4;  // captured calls kept per context

void free_graph(GraphEntry* ge) {
    if (!ge) return;
    if (ge->exec) cudaGraphExecDestroy(ge->exec);
    if (ge->graph) cudaGraphDestroy(ge->graph);
    for (Arena* a : ge->ars) delete a;  // returns the buffers to the context's pool
    for (void* p : ge->pinned) cudaFreeHost(p);
    if (ge->e0) cudaEventDestroy(ge->e0);
    if (ge->e1) cudaEventDestroy(ge->e1);
    delete ge;
}

void* graph_pinned(GraphEntry* ge, size_t bytes) {
    void* p = nullptr;
    CK(cudaMallocHost(&p, bytes ? bytes : 1));
    ge->pinned.push_back(p);
    return p;
}

// Datasets (device buffers, sizes, variants) and the options that shape the
// work; empty when a dataset is malformed (the direct path reports it).
std::vector<uint64_t> graph_key(const vdb_dataset* ds, int nds, const Options& o) {
    std::vector<uint64_t> k;
    auto add = [&](uint64_t v) { k.push_back(v); };
    add((uint64_t)nds);
    add((uint64_t)o.precision);
    add((uint64_t)o.schedule);
    add((uint64_t)o.location);
    add((uint64_t)(int64_t)o.cells_per_eps);
    add((uint64_t)o.budget);
    add((uint64_t)o.table_rows);
    add((uint64_t)o.table_hash);
    add((uint64_t)o.entry_bytes);
    add(o.reuse ? 1u : 0u);
    add((uint64_t)(int64_t)o.tile_cells);
    add((uint64_t)(int64_t)o.unit_words);
    for (int i = 0; i < nds; i++) {
        const vdb_dataset& d = ds[i];
        if (d.nv && (!d.eps || !d.minpts)) return {};
        if (d.n && d.nv && (!d.x || !d.y || !d.labels)) return {};
        // device buffers are read and written by the graph itself; host
        // buffers are copied through the graph's pinned buffers at each call
        if (o.location == VDB_LOC_DEVICE) {
            add((uint64_t)(uintptr_t)d.x);
            add((uint64_t)(uintptr_t)d.y);
            add((uint64_t)(uintptr_t)d.labels);
        }
        add(d.n);
        add((uint64_t)(int64_t)d.mbb_size);
        add(d.nv);
        for (uint32_t v = 0; v < d.nv; v++) {
            uint64_t e;
            memcpy(&e, &d.eps[v], 8);
            add(e);
            add(d.minpts[v]);
        }
    }
    return k;
}

// Captures the recorded call into ge (recs: one record per dataset, filled by
// the direct run).  The datasets run in up to autotune_streams() branches of
// the graph (largest first, each to the branch with the least work so far);
// within a branch they run one after the other and reuse its buffers.  False
// when the capture fails or its buffers would hold more than half of the
// device: the call then stays direct.
bool build_graph(vdb_context* ctx, GraphEntry* ge, const vdb_dataset* ds, int nds,
                 const Options& o, std::vector<GraphRec>& recs) {
    cudaStream_t s = ctx->stream;
    GraphBuild gb;
    try {
        const int nb = std::max(1, o.streams > 0 ? std::min(nds, o.streams)
                                                 : autotune_streams(ds, nds));
        for (int i = 0; i < nb; i++) {
            ge->ars.push_back(new Arena(ctx));
            ge->ars.back()->keep = true;
        }
        CK(cudaGraphCreate(&gb.top, 0));
        uint32_t* d_bad = ge->ars[0]->get<uint32_t>(1);
        gb.d_bad = d_bad;
        cudaMemsetParams mp;
        memset(&mp, 0, sizeof mp);
        mp.dst = d_bad;
        mp.value = 0;
        mp.elementSize = 4;
        mp.width = 1;
        mp.height = 1;
        mp.pitch = 4;
        cudaGraphNode_t root = nullptr;
        CK(cudaGraphAddMemsetNode(&root, gb.top, nullptr, 0, &mp));
        std::vector<int> order(nds);
        std::iota(order.begin(), order.end(), 0);
        auto work = [&](int i) {
            std::vector<double> e(ds[i].eps, ds[i].eps + (ds[i].eps ? ds[i].nv : 0));
            std::sort(e.begin(), e.end());
            const double t = (double)(std::unique(e.begin(), e.end()) - e.begin());
            return (double)ds[i].n * std::max(t, 1.0);
        };
        std::stable_sort(order.begin(), order.end(),
                         [&](int a, int b) { return work(a) > work(b); });
        std::vector<double> load(nb, 0.0);
        std::vector<std::vector<cudaGraphNode_t>> btails(nb, std::vector<cudaGraphNode_t>(1, root));
        const bool host = o.location == VDB_LOC_HOST;
        const unsigned long long l0 = g_launches.load();
        for (int i : order) {
            const int b = (int)(std::min_element(load.begin(), load.end()) - load.begin());
            load[b] += work(i);
            GraphRec& r = recs[i];
            r.capture = true;
            r.pos = 0;
            r.gb = &gb;
            r.ar = ge->ars[b];
            r.tails = btails[b];
            r.d_status = r.ar->get<DeviceStatus>(1);
            r.h_status = (DeviceStatus*)graph_pinned(ge, sizeof(DeviceStatus));
            memset(r.h_status, 0, sizeof(DeviceStatus));
            if (host && ds[i].n && ds[i].nv) {
                r.hx = (double*)graph_pinned(ge, (size_t)ds[i].n * 8);
                r.hy = (double*)graph_pinned(ge, (size_t)ds[i].n * 8);
                r.hlabels = (uint32_t*)graph_pinned(ge, (size_t)ds[i].n * ds[i].nv * 4);
            }
            run_dataset(ctx, ds[i], o, nullptr, &r);
            if (r.pos != r.vals.size())
                throw VdbError{VDB_ERR_CUDA, "graph capture: record not consumed"};
            r.gb = nullptr;
            btails[b] = r.tails;
        }
        // the failed-checkpoint flag comes back after every branch
        ge->h_bad = (uint32_t*)graph_pinned(ge, 4);
        *ge->h_bad = 0;
        std::vector<cudaGraphNode_t> deps;
        for (const auto& t : btails) deps.insert(deps.end(), t.begin(), t.end());
        CK(cudaStreamBeginCaptureToGraph(s, gb.top, deps.empty() ? nullptr : deps.data(), nullptr,
                                         deps.size(), cudaStreamCaptureModeRelaxed));
        CK(cudaMemcpyAsync(ge->h_bad, gb.d_bad, 4, cudaMemcpyDeviceToHost, s));
        cudaGraph_t g = nullptr;
        CK(cudaStreamEndCapture(s, &g));
        ge->launches = g_launches.load() - l0;
        size_t fb = 0, tb = 0, held = 0;
        CK(cudaMemGetInfo(&fb, &tb));
        for (Arena* a : ge->ars) held += a->cur;
        if ((double)held > 0.5 * (double)tb)
            throw VdbError{VDB_ERR_NOMEM, "graph buffers above half of the device"};
        CK(cudaGraphInstantiate(&ge->exec, gb.top, 0));
        CK(cudaEventCreate(&ge->e0));
        CK(cudaEventCreate(&ge->e1));
        ge->graph = gb.top;
        ge->checks = gb.nchk;
        ge->recs = std::move(recs);
        return true;
    } catch (const VdbError& e) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(s, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone) {
            cudaGraph_t g = nullptr;
            cudaStreamEndCapture(s, &g);
        }
        cudaGetLastError();
        if (ge->exec) cudaGraphExecDestroy(ge->exec);
        ge->exec = nullptr;
        if (gb.top) cudaGraphDestroy(gb.top);
        ge->graph = nullptr;
        for (Arena* a : ge->ars) delete a;
        ge->ars.clear();
        for (void* p : ge->pinned) cudaFreeHost(p);
        ge->pinned.clear();
        if (ge->e0) cudaEventDestroy(ge->e0);
        if (ge->e1) cudaEventDestroy(ge->e1);
        ge->e0 = ge->e1 = nullptr;
        if (o.verbose) fprintf(stderr, "vdbscan: call not captured: %s\n", e.msg.c_str());
        return false;
    }
}

// Page-locked host memory (cudaMallocHost, cudaHostAlloc, cudaHostRegister).
bool page_locked(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

// Points a captured host copy at the caller's buffer when it is page-locked
// (the copy then runs straight from or to it, as a direct call's does), else
// at the graph's pinned buffer.  True when the caller's buffer is used.
bool point_copy(GraphEntry* ge, cudaGraphNode_t node, void* dst, const void* src, size_t bytes,
                cudaMemcpyKind kind, const void* user, void* staged) {
    if (page_locked(user)) {
        void* d = kind == cudaMemcpyDeviceToHost ? const_cast<void*>(user) : dst;
        const void* s = kind == cudaMemcpyDeviceToHost ? src : user;
        if (cudaGraphExecMemcpyNodeSetParams1D(ge->exec, node, d, s, bytes, kind) == cudaSuccess)
            return true;
        cudaGetLastError();
    }
    void* d = kind == cudaMemcpyDeviceToHost ? staged : dst;
    const void* s = kind == cudaMemcpyDeviceToHost ? src : staged;
    CK(cudaGraphExecMemcpyNodeSetParams1D(ge->exec, node, d, s, bytes, kind));
    return false;
}

// One replay.  False when a checkpoint failed (nothing is returned then).
bool replay_graph(vdb_context* ctx, GraphEntry* ge, const vdb_dataset* ds, int nds,
                  const Options& o, vdb_stats* stats) {
    cudaStream_t s = ctx->stream;
    const bool host = o.location == VDB_LOC_HOST;
    std::vector<char> labels_direct(nds, 0);
    for (int i = 0; i < nds; i++) {
        const GraphRec& r = ge->recs[i];
        if (!host || !r.hx) continue;
        const size_t nb = (size_t)ds[i].n * 8;
        if (!point_copy(ge, r.n_x, (void*)r.dx, nullptr, nb, cudaMemcpyHostToDevice, ds[i].x, r.hx))
            memcpy(r.hx, ds[i].x, nb);
        if (!point_copy(ge, r.n_y, (void*)r.dy, nullptr, nb, cudaMemcpyHostToDevice, ds[i].y, r.hy))
            memcpy(r.hy, ds[i].y, nb);
        labels_direct[i] = point_copy(ge, r.n_labels, nullptr, r.dlabels,
                                      (size_t)ds[i].n * ds[i].nv * 4, cudaMemcpyDeviceToHost,
                                      ds[i].labels, r.hlabels);
    }
    // a launch that fails (the graph, not the data) is treated like a failed
    // checkpoint: the call runs directly and the graph is dropped
    if (cudaEventRecord(ge->e0, s) != cudaSuccess || cudaGraphLaunch(ge->exec, s) != cudaSuccess ||
        cudaEventRecord(ge->e1, s) != cudaSuccess) {
        cudaGetLastError();
        CK(cudaStreamSynchronize(s));
        return false;
    }
    CK(cudaStreamSynchronize(s));
    g_launches.fetch_add(ge->launches, std::memory_order_relaxed);
    if (*ge->h_bad != 0) return false;
    for (int i = 0; i < nds; i++) check_flags(*ge->recs[i].h_status);
    for (int i = 0; i < nds; i++) {
        const GraphRec& r = ge->recs[i];
        if (host && r.hlabels && !labels_direct[i])
            memcpy(ds[i].labels, r.hlabels, (size_t)ds[i].n * ds[i].nv * 4);
    }
    if (stats) {
        for (int i = 0; i < nds; i++) {
            const GraphRec& r = ge->recs[i];
            vdb_stats p = r.fixed;
            p.pairs = r.h_status->pairs;
            p.candidates = r.h_status->candidates;
            p.retested = r.h_status->retested;
            p.clusters = (uint32_t)r.h_status->clusters;
            p.table_hash = r.h_status->table_hash;
            p.reuse_skipped_pairs = r.h_status->reuse_skips;
            add_stats(stats, p);
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ge->e0, ge->e1);
        stats->ms_total = ms;
        stats->kernel_launches = (uint32_t)ge->launches;
        uint64_t held = 0;
        for (const Arena* a : ge->ars) held += a->cur;
        stats->device_bytes = held;
        stats->worker_streams = (uint32_t)ge->ars.size();
    }
    return true;
}

void drop_graph(vdb_context* ctx, GraphEntry* ge) {
    auto it = std::find(ctx->graphs.begin(), ctx->graphs.end(), ge);
    if (it != ctx->graphs.end()) ctx->graphs.erase(it);
    free_graph(ge);
}

size_t graph_bytes(const GraphEntry* ge) {
    size_t b = 0;
    for (const Arena* a : ge->ars) b += a->cur;
    return b;
}

// vdb_options.graph: replays the call's graph, or records and captures it.
// Returns VDB_GRAPH_REPLAYED or VDB_GRAPH_CAPTURED when the call is done, or
// VDB_GRAPH_FALLBACK / VDB_GRAPH_UNSUPPORTED when it is to run directly.
int run_graph(vdb_context* ctx, const vdb_dataset* ds, int nds, const Options& o,
              vdb_stats* stats) {
    const std::vector<uint64_t> key = graph_key(ds, nds, o);
    if (key.empty()) return VDB_GRAPH_UNSUPPORTED;
    GraphEntry* ge = nullptr;
    for (GraphEntry* e : ctx->graphs)
        if (e->key == key) ge = e;
    if (ge) {
        // most recently used last
        ctx->graphs.erase(std::find(ctx->graphs.begin(), ctx->graphs.end(), ge));
        ctx->graphs.push_back(ge);
        if (!ge->ok) return VDB_GRAPH_UNSUPPORTED;
        if (replay_graph(ctx, ge, ds, nds, o, stats)) {
            if (stats) stats->graph_checks = ge->checks;
            return VDB_GRAPH_REPLAYED;
        }
        // other data: drop the graph (the next call records the new data)
        drop_graph(ctx, ge);
        if (stats) memset(stats, 0, sizeof *stats);
        return VDB_GRAPH_FALLBACK;
    }
    // blocks cached by the worker contexts of earlier direct calls go back
    // to the device (the capture allocates through this context's pool),
    // and the cached graphs keep at most a quarter of the device before a
    // new recording (least recently used dropped first)
    for (vdb_context* w : ctx->workers) w->pool.trim();
    {
        size_t fb = 0, tb = 0, held = 0;
        CK(cudaMemGetInfo(&fb, &tb));
        for (const GraphEntry* e : ctx->graphs) held += graph_bytes(e);
        while (!ctx->graphs.empty() && (double)held > 0.25 * (double)tb) {
            held -= graph_bytes(ctx->graphs.front());
            drop_graph(ctx, ctx->graphs.front());
        }
    }
    // record (direct runs, one dataset after the other), then capture; out of
    // memory with graphs cached: release them and record again
    std::vector<GraphRec> recs(nds);
    try {
        for (int i = 0; i < nds; i++) run_dataset(ctx, ds[i], o, stats, &recs[i]);
    } catch (const VdbError& e) {
        if (e.code != VDB_ERR_NOMEM || ctx->graphs.empty()) throw;
        CK(cudaStreamSynchronize(ctx->stream));
        while (!ctx->graphs.empty()) drop_graph(ctx, ctx->graphs.front());
        if (stats) memset(stats, 0, sizeof *stats);
        recs.assign(nds, GraphRec());
        for (int i = 0; i < nds; i++) run_dataset(ctx, ds[i], o, stats, &recs[i]);
    }
    if (stats) stats->worker_streams = 1;
    bool ok = true;
    for (const GraphRec& r : recs) ok = ok && r.graphable;
    ge = new GraphEntry();
    ge->key = key;
    ge->ok = ok && build_graph(ctx, ge, ds, nds, o, recs);
    if (ok && !ge->ok && !ctx->graphs.empty()) {
        // once more without the other graphs' buffers
        while (!ctx->graphs.empty()) drop_graph(ctx, ctx->graphs.front());
        ge->ok = build_graph(ctx, ge, ds, nds, o, recs);
    }
    while (ctx->graphs.size() >= kMaxGraphs) drop_graph(ctx, ctx->graphs.front());
    ctx->graphs.push_back(ge);
    if (stats) stats->graph_checks = ge->checks;
    return ge->ok ? VDB_GRAPH_CAPTURED : VDB_GRAPH_UNSUPPORTED;
}

}  // namespace

// ====================================================================== C ABI

extern "C" {

void vdb_default_options(vdb_options* opts) {
    if (!opts) return;
    memset(opts, 0, sizeof *opts);
    opts->precision = VDB_PRECISION_MIXED;
    opts->schedule = VDB_SCHEDULE_BATCHED;
    opts->location = VDB_LOC_HOST;
}

int vdb_context_create(vdb_context** out, void* stream) {
    if (!out) return VDB_ERR_INVALID_ARG;
    *out = nullptr;
    vdb_context* ctx = new vdb_context();
    int rc = init_context(ctx, stream);
    if (rc != VDB_OK) {
        vdb_context_destroy(ctx);
        return rc;
    }
    *out = ctx;
    return VDB_OK;
}

void vdb_context_destroy(vdb_context* ctx) {
    if (!ctx) return;
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    for (GraphEntry* ge : ctx->graphs) free_graph(ge);
    ctx->graphs.clear();
    for (vdb_context* w : ctx->workers) vdb_context_destroy(w);
    ctx->workers.clear();
    ctx->pool.release_all();
    if (ctx->box_ready) cudaEventDestroy(ctx->box_ready);
    if (ctx->d_status) cudaFree(ctx->d_status);
    if (ctx->h_status) cudaFreeHost(ctx->h_status);
    if (ctx->h_pinned) cudaFreeHost(ctx->h_pinned);
    if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

int vdb_run_batch(vdb_context* ctx, const vdb_dataset* ds, int nds, const vdb_options* opts,
                  vdb_stats* stats) {
    if (!ctx) return VDB_ERR_INVALID_ARG;
    if (nds < 0 || (nds > 0 && !ds)) {
        ctx->err = "invalid dataset list";
        return VDB_ERR_INVALID_ARG;
    }
    std::lock_guard<std::mutex> lk(ctx->mu);
    Options o = to_options(opts);
    if (stats) memset(stats, 0, sizeof *stats);
    try {
        int gstate = VDB_GRAPH_NONE;
        if (o.graph) {
            gstate = run_graph(ctx, ds, nds, o, stats);
        }
        if (gstate != VDB_GRAPH_CAPTURED && gstate != VDB_GRAPH_REPLAYED) {
            const int nw = o.streams > 0 ? std::min(nds, o.streams) : autotune_streams(ds, nds);
            if (stats) stats->worker_streams = (uint32_t)std::max(nw, 1);
            if (nw > 1) {
                run_concurrent(ctx, ds, nds, o, nw, stats);
            } else {
                for (int i = 0; i < nds; i++) run_dataset(ctx, ds[i], o, stats);
            }
        }
        if (stats) stats->graph = (uint32_t)gstate;
    } catch (const VdbError& e) {
        ctx->err = e.msg;
        cudaStreamSynchronize(ctx->stream);
        cudaGetLastError();
        if (o.verbose) fprintf(stderr, "vdbscan: %s\n", e.msg.c_str());
        return e.code;
    }
    ctx->err.clear();
    return VDB_OK;
}

const char* vdb_last_error(vdb_context* ctx) { return ctx ? ctx->err.c_str() : ""; }

const char* vdb_version(void) { return "vdbscan-gb300 0.1 (sm_103a)"; }

}  // extern "C"

// ======================================================== allocation-free call
//
// vdb_run_noalloc clusters one small device-resident dataset for one variant
// without allocating: every temporary is carved out of g_noalloc_scratch, a
// fixed array that the CUDA runtime reserves on each device when it loads this
// library's device code, and that stays reserved until the process exits.
// It serves callers that may not allocate device memory inside a call: code
// whose device memory is all reserved up front (latency-bound services, a
// framework whose own allocator owns the heap), and code that cannot afford
// the implicit device-wide synchronisation of cudaMalloc and cudaFree.

namespace {

constexpr size_t kNoallocBytes = (size_t)64 << 20;      // 64 MiB per device
constexpr uint32_t kNoallocMaxPoints = 65536;
constexpr uint64_t kNoallocMaxCells = (uint64_t)1 << 20;
// pairs accepted in one direction only (4 MiB of the array; 4 per point at
// the largest n): an input with more returns VDB_ERR_CAPACITY
constexpr uint32_t kNoallocAsymCap = 1u << 18;
constexpr int kNoallocMaxDevices = 64;

}  // namespace

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocBytes];

namespace {

std::mutex g_noalloc_mu;
void* g_noalloc_ptr[kNoallocMaxDevices];  // device address of g_noalloc_scratch per device

// Bump carving of the fixed array (256-byte aligned pieces).
struct Carve {
    char* base;
    size_t cap;
    size_t used;
    template <class T>
    T* take(size_t count) {
        const size_t b = (count * sizeof(T) + 255) & ~(size_t)255;
        if (used + b > cap)
            throw VdbError{VDB_ERR_TOO_LARGE, "input needs more than the fixed scratch array"};
        T* p = (T*)(base + used);
        used += b;
        return p;
    }
};

void run_noalloc(const double* x, const double* y, uint32_t n, double eps, uint32_t minpts,
                 int mbb, uint32_t* labels, cudaStream_t s, char* base) {
    int dev = 0, nsm = 1;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    Carve cv{base, kNoallocBytes, 0};
    DeviceStatus* st = cv.take<DeviceStatus>(1);
    BBox* d_bb = cv.take<BBox>(1);
    const size_t scr = std::max({radix_sort_scratch_bytes(n), scan_u32_to_u64_scratch_bytes(n + 1),
                                 bbox_scratch_bytes(n),
                                 resolve_scratch_bytes() + scan_u32_scratch_bytes(n),
                                 suffix_min_u32_scratch_bytes(kNoallocMaxCells + 1)});
    char* scratch = cv.take<char>(scr);
    // the array keeps the previous call's contents: clear what starts at zero
    CK(cudaMemsetAsync(st, 0, sizeof(DeviceStatus), s));
    launch_bbox(x, y, n, d_bb, scratch, s);
    BBox bb;
    CK(cudaMemcpyAsync(&bb, d_bb, sizeof bb, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (bb.nonfinite) throw VdbError{VDB_ERR_INVALID_ARG, "non-finite coordinate"};
    const HostBox hb{bb.minx, bb.tmaxx, bb.miny, bb.tmaxy};

    uint32_t* vkey = cv.take<uint32_t>(n);
    uint32_t* vorder = cv.take<uint32_t>(n);
    uint32_t* pos = cv.take<uint32_t>(n);
    launch_visit_keys(x, y, n, d_bb, vkey, vorder, st, s);
    radix_sort_pairs(vkey, vorder, n, bits_for(kVisitBins * kVisitBins - 1), scratch, s);
    launch_invert(vorder, n, pos, s);
    const uint32_t nmpb = (uint32_t)(((uint64_t)n + (uint32_t)mbb - 1) / (uint32_t)mbb);
    MpbBox* mpb = cv.take<MpbBox>(nmpb);
    launch_mpb_boxes(x, y, vorder, n, mbb, mpb, s);

    const GridParams g = make_grid(hb, eps / kCellsPerEps, 1,
                                   kNoallocMaxCells);
    const EpsParams ep = make_eps(eps, g, hb, true);
    uint32_t* gkey = cv.take<uint32_t>(n);
    uint32_t* gorig = cv.take<uint32_t>(n);
    double2* gxy = cv.take<double2>(n);
    float2* glocal = cv.take<float2>(n);
    uint32_t* gpos = cv.take<uint32_t>(n);
    MpbBox* gbox = cv.take<MpbBox>(n);
    uint32_t* cell_start = cv.take<uint32_t>(g.ncells + 1);
    uint32_t* tflags = cv.take<uint32_t>(n);
    uint32_t* tscan = cv.take<uint32_t>((size_t)n + 1);
    uint32_t* tiles = cv.take<uint32_t>((size_t)n + 1);
    uint32_t* cscan = cv.take<uint32_t>((size_t)n + 1);
    uint32_t* clist = cv.take<uint32_t>((size_t)n + 1);
    uint32_t* crep = cv.take<uint32_t>(n);
    EpsParams* d_ep = cv.take<EpsParams>(1);
    uint32_t* deg = cv.take<uint32_t>(n);
    unsigned long long* off = cv.take<unsigned long long>((size_t)n + 1);
    AsymPair* asym = cv.take<AsymPair>(kNoallocAsymCap);
    uint32_t* asym_n = cv.take<uint32_t>(4);
    uint32_t* tile_counter = asym_n + 1;
    uint32_t* parent = cv.take<uint32_t>(n);
    uint32_t* seed = cv.take<uint32_t>(n);
    uint32_t* cstart = cv.take<uint32_t>(n);
    uint32_t* best = cv.take<uint32_t>(n);
    uint32_t* cluster_no = cv.take<uint32_t>((size_t)n + 1);
    uint32_t* pos_flag = cv.take<uint32_t>(n);

    launch_grid_keys(x, y, n, g, gkey, gorig, s);
    radix_sort_pairs(gkey, gorig, n, bits_for(g.ncells - 1), scratch, s);
    launch_grid_gather(x, y, gorig, pos, n, g, gkey, gxy, glocal, gpos, s);
    launch_point_boxes(gpos, n, mpb, mbb, gbox, s);
    CK(cudaMemsetAsync(cell_start, 0xff, (g.ncells + 1) * 4, s));
    launch_cell_marks(gkey, n, cell_start, g.ncells, s);
    suffix_min_u32(cell_start, g.ncells + 1, scratch, s);
    const int tq = table_tile_queries();
    launch_tile_flags(gkey, n, g.G, (uint32_t)tq, tflags, s);
    scan_u32(tflags, tscan, n, scratch, s);
    launch_tile_write(tflags, tscan, n, tiles, s);
    launch_tile_flags(gkey, n, 1, 0xffffffffu, tflags, s);
    scan_u32(tflags, cscan, n, scratch, s);
    launch_tile_write(tflags, cscan, n, clist, s);
    CK(cudaMemcpyAsync(d_ep, &ep, sizeof ep, cudaMemcpyHostToDevice, s));
    CK(cudaMemsetAsync(asym_n, 0, 4 * sizeof(uint32_t), s));

    TableArgs ta;
    memset(&ta, 0, sizeof ta);
    ta.g = g;
    ta.ep = d_ep;
    ta.mixed = ep.mixed;
    ta.tiles = tiles;
    ta.ntiles = tscan + n;
    ta.tile_end = 0xffffffffu;
    ta.tile_counter = tile_counter;
    ta.cell_start = cell_start;
    ta.gkey = gkey;
    ta.glocal = glocal;
    ta.gxy = gxy;
    ta.gpos = gpos;
    ta.gbox = gbox;
    ta.n = n;
    ta.deg = deg;
    ta.off = off;
    ta.asym = asym;
    ta.asym_n = asym_n;
    ta.asym_cap = kNoallocAsymCap;
    ta.st = st;
    ta.unit_words = kUnitWords;
    // work units of the count pass (no bitmap here: the fill pass writes the table)
    uint32_t* twords = cv.take<uint32_t>(n);
    uint32_t* tunits = cv.take<uint32_t>(n);
    uint32_t* tuoff = cv.take<uint32_t>((size_t)n + 1);
    launch_tile_words(ta, twords, tunits, nsm * 8, s);
    scan_u32(tunits, tuoff, n, scratch, s);
    uint32_t nunits = 0;
    CK(cudaMemcpyAsync(&nunits, tuoff + n, 4, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    uint32_t* unit_tile = cv.take<uint32_t>((size_t)nunits + 1);
    ta.tile_uoff = tuoff;
    ta.nunits = tuoff + n;
    ta.unit_tile = unit_tile;
    ta.parts = nullptr;
    ta.bitmap = nullptr;
    launch_unit_list(ta, unit_tile, nsm * 8, s);
    CK(cudaMemsetAsync(deg, 0, (size_t)n * 4, s));
    CK(cudaMemsetAsync(tile_counter, 0, 4, s));
    launch_count(ta, nsm * table_blocks_per_sm(false, ep.mixed != 0), s);
    scan_u32_to_u64(deg, off, n, scratch, s);
    unsigned long long E = 0;
    DeviceStatus hs;
    CK(cudaMemcpyAsync(&E, off + n, 8, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(&hs, st, sizeof hs, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    check_flags(hs);
    // the neighbour table takes the rest of the array
    const size_t room = (kNoallocBytes - cv.used) / sizeof(uint32_t);
    if (E > room)
        throw VdbError{VDB_ERR_TOO_LARGE, "neighbour table exceeds the fixed scratch array"};
    uint32_t* nbr = cv.take<uint32_t>(E ? E : 1);
    ta.nbr = nbr;
    ta.off_base = 0;
    CK(cudaMemsetAsync(tile_counter, 0, 4, s));
    launch_fill(ta, nsm * table_blocks_per_sm(true, ep.mixed != 0), s);

    ClusterArgs ca;
    memset(&ca, 0, sizeof ca);
    ca.n = n;
    ca.deg = deg;
    ca.unit_words = kUnitWords;
    ca.minpts = minpts > 0x7fffffffu ? ~0ull : (unsigned long long)minpts;
    ca.minpts_prev = ~0ull;
    ca.off = off;
    ca.row_lo = 0;
    ca.row_hi = n;
    ca.nbr = nbr;
    ca.gpos = gpos;
    ca.gorig = gorig;
    ca.parent = parent;
    ca.seed = seed;
    ca.cstart = cstart;
    ca.best = best;
    ca.cluster_no = cluster_no;
    ca.pos_flag = pos_flag;
    ca.asym = asym;
    ca.asym_count = asym_n;
    ca.asym_cap = kNoallocAsymCap;
    ca.labels_out = labels;
    ca.st = st;
    ca.g = g;
    ca.ep = d_ep;
    ca.gkey = gkey;
    ca.cell_start = cell_start;
    ca.clist = clist;
    ca.ncl = cscan + n;
    ca.cscan = cscan;
    ca.crep = crep;
    ca.glocal = glocal;
    ca.gxy = gxy;
    ca.gbox = gbox;
    const int nb_warps = nsm * 8;
    launch_uf_init(ca, true, s);
    const bool clique = 2.0 * g.w * g.w * (1.0 + 0x1p-20) <= std::min(ep.thr, ep.tbox);
    if (clique)
        launch_cell_union(ca, nb_warps, s);
    else
        launch_uf_union(ca, nb_warps, s);
    launch_uf_finish(ca, scratch, scratch + resolve_scratch_bytes(), s);
    launch_border_and_write(ca, nb_warps, s);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(&hs, st, sizeof hs, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    check_flags(hs);
}

}  // namespace

extern "C" {

int vdb_run_noalloc(const double* x, const double* y, uint32_t n, double eps, uint32_t minpts,
                    int32_t mbb_size, uint32_t* labels, void* stream) {
    if (!x || !y || !labels || mbb_size <= 0) return VDB_ERR_INVALID_ARG;
    if (!(eps >= 0.0) || isinf(eps)) return VDB_ERR_INVALID_ARG;
    if (n == 0) return VDB_OK;
    if (n > kNoallocMaxPoints) return VDB_ERR_TOO_LARGE;
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    cudaStream_t s = (cudaStream_t)stream;
    try {
        int dev = 0;
        CK(cudaGetDevice(&dev));
        if (dev < 0 || dev >= kNoallocMaxDevices)
            throw VdbError{VDB_ERR_INVALID_ARG, "device ordinal out of range"};
        if (!g_noalloc_ptr[dev]) {
            // set-up, once per device with that device current: the host-side
            // name g_noalloc_scratch is not a device address
            void* p = nullptr;
            CK(cudaGetSymbolAddress(&p, g_noalloc_scratch));
            g_noalloc_ptr[dev] = p;
        }
        run_noalloc(x, y, n, eps, minpts, mbb_size, labels, s, (char*)g_noalloc_ptr[dev]);
    } catch (const VdbError& e) {
        cudaStreamSynchronize(s);
        cudaGetLastError();
        return e.code;
    }
    return VDB_OK;
}

}  // extern "C"

extern "C" {

static std::mutex g_mu;
static vdb_context* g_ctx = nullptr;

int libVDBSCAN(double* inputx, double* inputy, unsigned int datasetSize, double* inputEpsilon,
               unsigned int* inputMinpts, unsigned int numVariants, int MBBsize,
               unsigned int* retArr, bool verbose) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (verbose) printf("Verbose mode on");
    if (datasetSize == 0 || numVariants == 0) return VDB_OK;
    if (!g_ctx) {
        int rc = vdb_context_create(&g_ctx, nullptr);
        if (rc != VDB_OK) return rc;
    }
    vdb_dataset d;
    d.x = inputx;
    d.y = inputy;
    d.n = datasetSize;
    d.mbb_size = MBBsize;
    d.eps = inputEpsilon;
    d.minpts = inputMinpts;
    d.nv = numVariants;
    d.labels = retArr;
    vdb_options o;
    vdb_default_options(&o);
    o.verbose = verbose ? 1 : 0;
    vdb_stats st;
    int rc = vdb_run_batch(g_ctx, &d, 1, &o, &st);
    if (verbose) {
        printf("\nvdbscan-gb300: %u points, %u variants, rc=%d, %.3f ms, %llu pairs\n",
               datasetSize, numVariants, rc, st.ms_total, (unsigned long long)st.pairs);
    }
    return rc;
}

}  // extern "C"
