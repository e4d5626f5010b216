// Internal declarations shared by the CUDA translation units of
// libSharedVDBSCAN.so (GB300, sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <string>
#include <vector>

namespace vdb {

// Kernels launched by this library since it was loaded.
extern std::atomic<unsigned long long> g_launches;
#define VDB_COUNT_LAUNCH() (::vdb::g_launches.fetch_add(1, std::memory_order_relaxed))

constexpr int kVisitBins = 300;          // src/main.cpp:107 (binDataset(&dataPoints, 300, ...))
constexpr int kMaxRows = 65;             // neighbour rows per tile: 2*rho+1 <= 65
constexpr uint32_t kAsymFlag = 0x80000000u;  // neighbour-table entry accepted in one direction only
constexpr uint32_t kIdMask = 0x7fffffffu;
// Compact tables: 16-bit entries.  A row lists its neighbours work unit by
// work unit (units of 1024 to 4096 candidates of the row's tile, in
// order; the count pass's per-unit counts give each unit's share of the row);
// an entry holds the neighbour's position within its unit's candidates (12
// bits) and, in the top bit, the one-way flag.  Positions map to cell-ordered
// indices through the tile's 2*rho+1 row segments.
constexpr uint16_t kAsymFlag16 = 0x8000u;
constexpr uint16_t kPosMask16 = 0x0fffu;

// Status bits written by kernels into DeviceStatus::flags.
enum : uint32_t {
    kStatNonFinite = 1u << 0,    // NaN or inf coordinate
    kStatDegenerate = 1u << 1,   // reference binDataset would report bins out of range
    kStatAsymOverflow = 1u << 2, // asymmetric-pair list full
    kStatResolveOverflow = 1u << 3,  // too many directed component edges
    kStatRowOverflow = 1u << 4,      // fill pass found more neighbours than the count pass
    kStatUnionStall = 1u << 5,       // union-find retry limit reached
    kStatGuard = 1u << 6,            // an index guard failed (see guard_site)
    kStatBitmapTooLarge = 1u << 7,   // a tile's test bitmap exceeds 2^32 words (use the fill pass)
};

constexpr uint32_t kResolveCap = 4096;   // directed component edges per variant

struct DeviceStatus {
    uint32_t flags;
    uint32_t guard_site;           // first failed index guard: site code
    unsigned long long retested;   // FP64 re-tests
    unsigned long long candidates; // candidate pairs tested
    unsigned long long asym_count; // asymmetric pairs recorded
    unsigned long long guard_value; // first failed index guard: the index
    unsigned long long clusters;   // clusters summed over the variants written
    unsigned long long table_hash; // hash of the tables built (vdb_stats.table_hash)
    unsigned long long reuse_skips; // cell pairs not searched: different components at a
                                    // larger epsilon
    unsigned long long pairs;      // neighbour pairs counted (graph replays only)
};

// Index guards: a data-derived index outside its array is recorded (site and
// value of the first one) and the access is skipped.
__device__ __forceinline__ void guard_fail(DeviceStatus* st, uint32_t site,
                                           unsigned long long v) {
    if (atomicOr(&st->flags, 1u << 6) & (1u << 6)) return;
    st->guard_site = site;
    st->guard_value = v;
}
#define VDB_GUARD(st, cond, site, val) ((cond) ? true : (guard_fail((st), (site), (val)), false))

// Bounding box with the reference's initial values (src/main.cpp:465-468):
// min starts at DBL_MAX, max at DBL_MIN (the smallest positive double).
struct BBox {
    double minx, maxx, miny, maxy;      // reference semantics (max >= DBL_MIN)
    double tmaxx, tmaxy;                // true maxima
    uint32_t nonfinite;
    uint32_t pad;
};

// Grid over a dataset: cells of width w (exactly representable with 12
// significant bits, so small multiples of w are exact in FP32), row-major keys
// key = cy*ncx_pad + cx.  A tile covers up to kTileQueries consecutive points of
// one group of G cells of one row.
struct GridParams {
    double x0, y0, w;
    uint32_t ncx, ncy, ncx_pad, G;
    uint64_t ncells;                    // ncx_pad*ncy
    // 0: cells are looked up in a dense cell_start array (ncells+1 entries);
    // 1: many more cells than points - a row directory of the non-empty
    //    cells (crow, ccx, clist) replaces it
    uint32_t sparse;
    uint32_t pad;
};

// Points [*s, *e) of the cells lo_c..hi_c of grid row ry (cell order).
// Dense grids: cell_start[key] = first point of the first non-empty cell with
// a key >= key.  Sparse grids: crow[ry]..crow[ry+1] are the non-empty cells of
// row ry (sorted by column ccx), clist[c] the first point of cell c.
static __device__ __forceinline__ uint32_t cx_lower_bound(const uint32_t* __restrict__ ccx,
                                                          uint32_t b, uint32_t e, uint32_t v) {
    while (b < e) {
        const uint32_t m = (b + e) >> 1;
        if (ccx[m] < v) b = m + 1;
        else e = m;
    }
    return b;
}
static __device__ __forceinline__ void cell_row_range(const GridParams& g,
                                                      const uint32_t* __restrict__ cell_start,
                                                      const uint32_t* __restrict__ crow,
                                                      const uint32_t* __restrict__ ccx,
                                                      const uint32_t* __restrict__ clist,
                                                      uint32_t ry, uint32_t lo_c, uint32_t hi_c,
                                                      uint32_t* s, uint32_t* e) {
    if (g.sparse) {
        const uint32_t rb = crow[ry], re = crow[ry + 1];
        const uint32_t c0 = cx_lower_bound(ccx, rb, re, lo_c);
        const uint32_t c1 = cx_lower_bound(ccx, c0, re, hi_c + 1);
        *s = clist[c0];
        *e = clist[c1];
    } else {
        const uint32_t base = ry * g.ncx_pad;
        *s = cell_start[base + lo_c];
        *e = cell_start[base + hi_c + 1];
    }
}

// Distance test of one epsilon.
struct EpsParams {
    double eps;
    double thr;     // largest double t with sqrt(t) <= eps
    double tbox;    // d2 <= tbox guarantees the candidate lies in the query box
    float lo32;     // FP32 d2 < lo32: neighbour (no FP64 re-test)
    float hi32;     // FP32 d2 > hi32: not a neighbour
    // count pass filter on the quadratic form nS = |c|^2/2 + (|q|^2 - L32)/2 - q.c
    // (= (d2 - L32)/2 up to rounding): nS < 0 => d2 < lo32 (in); nS > w32 =>
    // d2 > hi32 (out); every nS in between is re-tested in FP64
    float L32;
    float w32;
    int rho;        // rows above/below the tile row to scan
    int mixed;      // 1: FP32 filter + FP64 band re-test; 0: FP64 only
    int reach[kMaxRows];  // columns left/right of the tile's cells to scan, per row offset+rho
};

// Bounding box of one group of MBBsize consecutive visit-ordered points
// (the reference's MPBRect, src/structs.h:70-125).
struct __align__(32) MpbBox {
    double x0, x1, y0, y1;   // min x, max x, min y, max y
};

struct AsymPair {
    uint32_t a, b;     // grid indices, a < b
    uint32_t dir;      // bit0: b in N(a); bit1: a in N(b)
    uint32_t pad;
};

// ------------------------------------------------- the reference's predicate
// q in N(p)  <=>  sqrt(fl(fl(dx*dx)+fl(dy*dy))) <= eps with dx = fl(px-qx) in
// FP64 (src/DBScan.cpp:687, 699-702) and q's multiple-point box overlaps the
// query box [p-eps, p+eps]^2 (R-tree candidates, src/RTree.h:1613-1625).

// q inside the query box of p (DBScan::generateMBB, src/DBScan.cpp:722-731);
// a point inside the box makes its multiple-point box overlap it.
static __device__ __forceinline__ bool in_query_box(double qx, double qy, double px, double py,
                                                    double eps) {
    const double x0 = __dsub_rn(px, eps), x1 = __dadd_rn(px, eps);
    const double y0 = __dsub_rn(py, eps), y1 = __dadd_rn(py, eps);
    return !(x0 > qx || qx > x1 || y0 > qy || qy > y1);
}

static __device__ __forceinline__ bool box_overlap(MpbBox m, double px, double py, double eps) {
    const double x0 = __dsub_rn(px, eps), x1 = __dadd_rn(px, eps);
    const double y0 = __dsub_rn(py, eps), y1 = __dadd_rn(py, eps);
    return !(x0 > m.x1 || m.x0 > x1 || y0 > m.y1 || m.y0 > y1);
}

// Bounds of the exact predicate as ordered integers.  For doubles >= +0 the
// order of the values is the order of their bit patterns read as integers, so
// the predicate compares d2 and |d| with integer instructions and leaves
// GB300's narrow FP64 pipe to the subtractions and products.  A negative or
// NaN bound becomes -1, which no value passes (as with the FP64 comparison).
struct ExactBounds {
    double eps;
    long long thr, tbox, ax;  // thr, tbox and ax_in = sqrt(tbox), ordered
};
static __device__ __forceinline__ long long ordered_bits(double v) {
    return v > 0.0 ? __double_as_longlong(v) : (v == 0.0 ? 0ll : -1ll);
}
static __device__ __forceinline__ ExactBounds exact_bounds(double eps, double thr, double tbox) {
    ExactBounds b;
    b.eps = eps;
    b.thr = ordered_bits(thr);
    b.tbox = ordered_bits(tbox);
    b.ax = ordered_bits(sqrt(tbox));
    return b;
}

// Exact predicate in both directions: bit0 = q in N(p), bit1 = p in N(q).
// thr: largest double whose square root is <= eps; tbox: below it the pair is
// inside both query boxes; ax_in = sqrt(tbox): an axis along which
// |d| <= ax_in keeps each point inside the other's query box whatever the
// roundings of p +- eps (the margin behind tbox is per axis), so the box
// arithmetic is done only along the other axis.  d2 >= +0 and |d| >= +0 are
// compared as ordered integers (ExactBounds).  kp, kq: cell-ordered indices;
// gbox[k]: the multiple-point box holding cell-ordered point k (one load, no
// index chain).
static __device__ __noinline__ uint32_t exact_pair(double2 P, double2 Q, uint32_t kp,
                                                   uint32_t kq, const ExactBounds b,
                                                   const MpbBox* __restrict__ gbox) {
    const double dx = __dsub_rn(P.x, Q.x), dy = __dsub_rn(P.y, Q.y);
    const double d2 = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
    const long long d2b = __double_as_longlong(d2);
    if (!(d2b <= b.thr)) return 0u;
    if (d2b <= b.tbox) return 3u;
    const long long mag = 0x7fffffffffffffffll;
    const bool inx = (__double_as_longlong(dx) & mag) <= b.ax;
    const bool iny = (__double_as_longlong(dy) & mag) <= b.ax;
    if (inx && iny) return 3u;
    const double eps = b.eps;
    uint32_t r = 0u;
    // q inside the query box of p (DBScan::generateMBB, src/DBScan.cpp:722-731)
    const bool qin = (inx || !(__dsub_rn(P.x, eps) > Q.x || Q.x > __dadd_rn(P.x, eps))) &&
                     (iny || !(__dsub_rn(P.y, eps) > Q.y || Q.y > __dadd_rn(P.y, eps)));
    if (qin || box_overlap(gbox[kq], P.x, P.y, eps)) r |= 1u;
    const bool pin = (inx || !(__dsub_rn(Q.x, eps) > P.x || P.x > __dadd_rn(Q.x, eps))) &&
                     (iny || !(__dsub_rn(Q.y, eps) > P.y || P.y > __dadd_rn(Q.y, eps)));
    if (pin || box_overlap(gbox[kp], Q.x, Q.y, eps)) r |= 2u;
    return r;
}

// Compact-table decoding, one warp per row (every lane must call both, with
// the same t): lane i < nrows holds the start of segment i of tile t's
// candidate list and the number of candidates before it.
struct TileSegs {
    uint32_t start, before;
};
static __device__ __forceinline__ TileSegs load_tile_segs(const uint32_t* __restrict__ trow_s,
                                                          const uint32_t* __restrict__ trow_e,
                                                          uint32_t t, int nrows, int lane) {
    uint32_t st = 0, len = 0;
    if (lane < nrows) {
        const unsigned long long k = (unsigned long long)t * (uint32_t)nrows + (uint32_t)lane;
        st = trow_s[k];
        len = trow_e[k] - st;
    }
    uint32_t incl = len;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t v = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl += v;
    }
    return TileSegs{st, incl - len};
}
// Cell-ordered index of candidate position g (g below the tile's total).
static __device__ __forceinline__ uint32_t decode_candidate(const TileSegs& sg, int nrows,
                                                            uint32_t g) {
    uint32_t id = 0;
    for (int i = 0; i < nrows; i++) {
        const uint32_t b = __shfl_sync(0xffffffffu, sg.before, i);
        const uint32_t s0 = __shfl_sync(0xffffffffu, sg.start, i);
        if (g >= b) id = s0 + (g - b);
    }
    return id;
}

// ----------------------------------------------------------------- primitives
// All launches go to `s`; temporaries come from the caller-provided scratch.

// Exclusive scan of n uint32 values into uint64 (out has n+1 entries; out[n] = total).
size_t scan_u32_to_u64_scratch_bytes(uint64_t n);
void scan_u32_to_u64(const uint32_t* in, unsigned long long* out, uint64_t n, void* scratch,
                     cudaStream_t s);
// Exclusive scan of n uint32 values into uint32 (out has n+1 entries).
size_t scan_u32_scratch_bytes(uint64_t n);
void scan_u32(const uint32_t* in, uint32_t* out, uint64_t n, void* scratch, cudaStream_t s);
// Reverse inclusive min-scan in place: a[i] = min(a[i..n-1]).
size_t suffix_min_u32_scratch_bytes(uint64_t n);
void suffix_min_u32(uint32_t* a, uint64_t n, void* scratch, cudaStream_t s);

// Stable LSD radix sort of (key, value) pairs on the low `bits` key bits.
size_t radix_sort_scratch_bytes(uint32_t n);
void radix_sort_pairs(uint32_t* keys, uint32_t* vals, uint32_t n, int bits, void* scratch,
                      cudaStream_t s);

// ------------------------------------------------------------------ index
void launch_bbox(const double* x, const double* y, uint32_t n, BBox* out, void* scratch,
                 cudaStream_t s);
size_t bbox_scratch_bytes(uint32_t n);
void launch_visit_keys(const double* x, const double* y, uint32_t n, const BBox* bb,
                       uint32_t* keys, uint32_t* idx, DeviceStatus* st, cudaStream_t s);
void launch_invert(const uint32_t* order, uint32_t n, uint32_t* inv, cudaStream_t s);
void launch_mpb_boxes(const double* x, const double* y, const uint32_t* vorder, uint32_t n,
                      int mbb, MpbBox* boxes, cudaStream_t s);
void launch_grid_keys(const double* x, const double* y, uint32_t n, GridParams g,
                      uint32_t* keys, uint32_t* idx, cudaStream_t s);
// gbox[k] = mpb[gpos[k] / mbb]: the multiple-point box of cell-ordered point k
void launch_point_boxes(const uint32_t* gpos, uint32_t n, const MpbBox* mpb, int mbb,
                        MpbBox* gbox, cudaStream_t s);
void launch_grid_gather(const double* x, const double* y, const uint32_t* gorig,
                        const uint32_t* pos, uint32_t n, GridParams g, const uint32_t* gkey,
                        double2* gxy, float2* glocal, uint32_t* gpos, cudaStream_t s);
// Row directory of a sparse grid: ccx[c] = column of non-empty cell c,
// crow[r] = first non-empty cell of row >= r (crow[ncy] = number of cells;
// crow must hold 0xffffffff before the call, then is completed by a suffix min).
void launch_cell_rows(const uint32_t* gkey, const uint32_t* clist, const uint32_t* ncl,
                      uint32_t n, const GridParams& g, uint32_t* crow, uint32_t* ccx,
                      cudaStream_t s);
void launch_cell_marks(const uint32_t* gkey, uint32_t n, uint32_t* cell_start,
                       uint64_t ncells, cudaStream_t s);
void launch_tile_flags(const uint32_t* gkey, uint32_t n, uint32_t G, uint32_t tq,
                       uint32_t* flags, cudaStream_t s);
// Autotuner statistics of tile shapes: for each candidate G = 2^i (cells
// per tile group), over the non-empty cells that start a group of G cells
// among about kTuneSamples sampled cells (runs of kTuneRun consecutive
// non-empty cells spread evenly over the grid's non-empty cells):
// out[2i] += candidate tests in lane slots (C * 32 * ceil(P/32)),
// out[2i+1] += tiles (ceil(P/64)), with P the group's points and C its
// candidates (cells within reach of the group in rows cy-rho..cy+rho).  Cell
// structures of the grid g (any G), keys in its layout; out must hold
// 2*kTuneShapes zeroed u64.
constexpr int kTuneShapes = 5;   // G = 1, 2, 4, 8, 16
constexpr uint32_t kTuneSamples = 65536;
constexpr uint32_t kTuneRun = 64;
void launch_tile_costs(const GridParams& g, const EpsParams* ep, const uint32_t* gkey,
                       const uint32_t* cell_start, const uint32_t* crow, const uint32_t* ccx,
                       const uint32_t* clist, const uint32_t* ncl, uint32_t n,
                       unsigned long long* out, cudaStream_t s);
// Keys of grid `from` rewritten in the layout of grid `to` (same cells, other
// padding of the rows: the cell order, hence the sort, is unchanged).
void launch_grid_rekey(uint32_t* gkey, uint32_t n, uint32_t ncx_pad_from, uint32_t ncx_pad_to,
                       cudaStream_t s);
void launch_tile_write(const uint32_t* flags, const uint32_t* scan, uint32_t n,
                       uint32_t* tiles, cudaStream_t s);

// ------------------------------------------------------------------ tables
struct TableArgs {
    GridParams g;
    const EpsParams* ep;        // device copy
    int mixed;                  // 1: FP32 filter kernels, 0: FP64 kernels
    const uint32_t* tiles;      // tile start indices (ntiles+1 entries, last = n)
    const uint32_t* ntiles;     // device scalar
    uint32_t tile_end;          // 0xffffffff: use *ntiles
    uint32_t* tile_counter;     // device scalar: first tile to take (set before launch)
    const uint32_t* cell_start; // ncells+1 entries (dense grids)
    const uint32_t* crow;       // sparse grids: row directory (see cell_row_range)
    const uint32_t* ccx;
    const uint32_t* clist;      // first point of each non-empty cell (ncl+1 entries)
    // sparse grids and compact tables: candidate range of row i of tile t at
    // [t*(2*rho+1) + i] (written by the tile-words pass, read by the count and
    // expand passes and, for compact tables, by every reader of the table)
    uint32_t* trow_s;
    uint32_t* trow_e;
    const uint32_t* ptile;      // compact tables: tile of every cell-ordered point
    int compact;                // nonzero: nbr holds 16-bit entries (kAsymFlag16)
    const uint32_t* gkey;
    const float2* glocal;
    const double2* gxy;
    const uint32_t* gpos;
    const MpbBox* gbox;         // multiple-point box of each cell-ordered point
    uint32_t n;
    uint32_t* deg;              // count pass output
    const unsigned long long* off;  // fill pass: row offsets (n+1)
    unsigned long long off_base;    // fill pass: first entry held by nbr
    uint32_t* nbr;                  // fill pass output (uint16_t entries when compact)
    AsymPair* asym;
    uint32_t* asym_n;
    uint32_t asym_cap;
    DeviceStatus* st;
    uint32_t* bitmap;               // count pass: per-tile test bitmaps (nullptr: none)
    const unsigned long long* tile_boff;  // first bitmap word of each tile
    // work units of the count and table passes: (tile, chunk of unit_words
    // bitmap words); unit u belongs to tile unit_tile[u], chunk u - tile_uoff[tile]
    uint32_t unit_words;            // kUnitWords or kUnitWordsSmall
    const uint32_t* unit_tile;
    const uint32_t* tile_uoff;
    const uint32_t* nunits;         // device scalar
    uint32_t* parts;                // per unit and query slot: neighbours in that chunk
    // one row chunk of the table (zero: the whole table): the fill pass takes
    // tiles from tile_lo on, the expand pass units [unit_lo, unit_hi), and the
    // asymmetric flags touch rows [row_lo, row_hi) only
    uint32_t tile_lo;
    uint32_t unit_lo, unit_hi;
    uint32_t row_lo, row_hi;
    // nonzero: the table holds only the rows of points with deg < row_deg_lim
    // (off is the scan of those rows' degrees); the other rows are skipped
    uint32_t row_deg_lim;
};
// Work units hold 4096 candidates of a tile (kUnitWords bitmap words) or, for
// small datasets, 1024 (kUnitWordsSmall): a warp's longest unit bounds the
// count and expand passes of a table with few units.  Compact entries are
// positions within a unit (12 bits) either way.
constexpr uint32_t kUnitWords = 128;
constexpr uint32_t kUnitWordsSmall = 32;
constexpr uint32_t kUnitQ = 64;        // query slots per unit (tiles hold <= 64 queries)

// Walks row k of a compact table (nb16, the row's entries [row0, row1)) unit
// by unit, 32 entries at a time: fn(neighbour cell-ordered index, one-way
// flag, valid) on every lane (the decoding shuffles need the whole warp; lanes
// past the end get valid = false).  parts[u * kUnitQ + slot]: the row's
// entries in unit u; unit_words: the table's unit size in bitmap words.
template <class Fn>
static __device__ __forceinline__ void walk_compact_row(
    const uint16_t* __restrict__ nb16, unsigned long long row0, unsigned long long row1, uint32_t k,
    const uint32_t* __restrict__ ptile, const uint32_t* __restrict__ tiles,
    const uint32_t* __restrict__ tile_uoff, const uint32_t* __restrict__ parts,
    const uint32_t* __restrict__ trow_s, const uint32_t* __restrict__ trow_e, int nrows,
    uint32_t unit_words, int lane, Fn&& fn) {
    const uint32_t t = ptile[k];
    const uint32_t slot = k - tiles[t];
    const uint32_t u0 = tile_uoff[t], u1 = tile_uoff[t + 1];
    const TileSegs sg = load_tile_segs(trow_s, trow_e, t, nrows, lane);
    unsigned long long j = row0;
    for (uint32_t ub = u0; ub < u1; ub += 32) {
        const uint32_t u = ub + (uint32_t)lane;
        const uint32_t c = (u < u1 && slot < kUnitQ) ? parts[(unsigned long long)u * kUnitQ + slot] : 0u;
        uint32_t incl = c;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t v = __shfl_up_sync(0xffffffffu, incl, d);
            if (lane >= d) incl += v;
        }
        const unsigned long long jb = j + (incl - c);
        for (uint32_t nz = __ballot_sync(0xffffffffu, c != 0u); nz; nz &= nz - 1u) {
            const int src = __ffs(nz) - 1;
            const uint32_t cu = __shfl_sync(0xffffffffu, c, src);
            const unsigned long long js = __shfl_sync(0xffffffffu, jb, src);
            const uint32_t gbase = (ub + (uint32_t)src - u0) * (unit_words * 32u);
            for (uint32_t e0 = 0; e0 < cu; e0 += 32) {
                const bool valid = e0 + (uint32_t)lane < cu && js + e0 + (uint32_t)lane < row1;
                const uint16_t ev = valid ? nb16[js + e0 + (uint32_t)lane] : (uint16_t)0;
                const uint32_t id = decode_candidate(sg, nrows, gbase + (ev & kPosMask16));
                fn(id, (ev & kAsymFlag16) != 0, valid);
            }
        }
        j += __shfl_sync(0xffffffffu, incl, 31);
    }
}
void launch_count(const TableArgs& a, int nblocks, cudaStream_t s);
void launch_fill(const TableArgs& a, int nblocks, cudaStream_t s);
void launch_tile_words(const TableArgs& a, uint32_t* words, uint32_t* units, int nblocks,
                       cudaStream_t s);
void launch_unit_list(const TableArgs& a, uint32_t* unit_tile, int nblocks, cudaStream_t s);
// adds the hash of rows [row_lo, row_hi) of the table to st->table_hash
// (gorig: input index of every cell-ordered point)
void launch_table_hash(const TableArgs& a, const uint32_t* gorig, int nblocks, cudaStream_t s);
// out[k] = deg[k] < lim ? deg[k] : 0
void launch_masked_degrees(const uint32_t* deg, uint32_t n, uint32_t lim, uint32_t* out,
                           cudaStream_t s);
void launch_expand(const TableArgs& a, int nblocks, cudaStream_t s);
// ptile[k] = t for the points [tiles[t], tiles[t+1]) of every tile t
void launch_tile_owner(const TableArgs& a, uint32_t* ptile, int nblocks, cudaStream_t s);
void launch_asym_flags(const TableArgs& a, cudaStream_t s);
int table_block_threads();
int table_tile_queries();
int table_blocks_per_sm(bool fill, bool mixed);
int expand_blocks_per_sm(bool compact);

// ------------------------------------------------------------------ clustering
struct ClusterArgs {
    uint32_t n;
    const uint32_t* deg;
    unsigned long long minpts;      // ~0ull: no core points
    unsigned long long minpts_prev; // ~0ull: union-find starts from scratch; else the
                                    // cores of minpts_prev are already united in parent
    const unsigned long long* off;
    unsigned long long off_base;
    uint32_t row_lo, row_hi;
    const uint32_t* nbr;        // uint16_t entries when compact
    int compact;                // compact table: entries decoded through ptile, trow_s/e,
    const uint32_t* ptile;      // the tiles' first points and work units, and the count
    const uint32_t* trow_s;     // pass's per-unit counts
    const uint32_t* trow_e;
    const uint32_t* tiles;
    const uint32_t* tile_uoff;
    const uint32_t* parts;
    uint32_t unit_words;        // the table's work-unit size in bitmap words
    const uint32_t* gpos;
    const uint32_t* gorig;
    uint32_t* parent;
    uint32_t* seed;             // per root: min visit position of its cores
    uint32_t* cstart;           // per root: root of the component that starts its cluster
    uint32_t* best;             // per point: earliest cluster start among adjacent cores
    uint32_t* cluster_no;       // per visit position: clusters started before it (n+1)
    uint32_t* pos_flag;         // per visit position: a cluster starts there
    const AsymPair* asym;
    const uint32_t* asym_count;
    uint32_t asym_cap;
    uint32_t* labels_out;       // n labels in input order
    DeviceStatus* st;
    // cell structure (cell union): cells of width <= eps/sqrt(2) are cliques
    GridParams g;
    const EpsParams* ep;        // reach pattern of the grid
    const uint32_t* gkey;
    const uint32_t* cell_start;
    const uint32_t* crow;       // sparse grids: row directory (see cell_row_range)
    const uint32_t* ccx;
    const uint32_t* clist;      // first point of every non-empty cell (ncl+1 entries)
    const uint32_t* ncl;        // device scalar
    const uint32_t* cscan;      // cell index of the first point of each cell
    uint32_t* crep;             // per non-empty cell: its first core point or ~0
    const float2* glocal;       // FP32 coordinates relative to the own cell's origin
    const double2* gxy;         // FP64 coordinates, cell order
    const MpbBox* gbox;         // multiple-point box of each cell-ordered point
    // nested-epsilon reuse: comp_prev[pos] = component (its seed) of the core
    // at visit position pos in a variant with a larger or equal epsilon and a
    // smaller or equal minpts (nullptr: none); cores of different components
    // there cannot be connected here
    const uint32_t* comp_prev;
};
size_t resolve_scratch_bytes();
// comp[gpos[k]] = seed of the component of core k, kNone for other points
// (after launch_uf_finish)
void launch_save_components(const ClusterArgs& a, uint32_t* comp, cudaStream_t s);

// Graph replay (vdb_options.graph).  A checkpoint re-checks device values
// that the host read while recording the call: each condition compares one
// value with what the host planned for (kGcEq64: equal 64-bit word; kGcLe64 /
// kGcLe32: at most a, and kGcLe64 adds the value to *sum when sum is set;
// kGcMask32: (value & a) == b; kGcGeF64 / kGcLeF64: a double at least / at
// most the double whose bits are a).  If all hold and no earlier checkpoint
// failed the conditional node after it runs; otherwise *bad = index (first
// failure) and the rest of the replay is skipped.
enum : uint32_t { kGcEq64 = 1, kGcLe64 = 2, kGcLe32 = 3, kGcMask32 = 4, kGcGeF64 = 5,
                  kGcLeF64 = 6 };
constexpr int kGraphConds = 8;
struct GraphCond {
    const void* ptr;
    unsigned long long* sum;
    unsigned long long a, b;
    uint32_t kind;
    uint32_t pad;
};
struct GraphCheck {
    GraphCond c[kGraphConds];
    int n;
    uint32_t index;  // 1-based checkpoint number
};
void launch_graph_check(const GraphCheck& chk, uint32_t* bad, cudaGraphConditionalHandle next,
                        cudaStream_t s);
// *dst = v by a kernel (a captured host-to-device copy would read the host
// buffer at replay time).
void launch_store_eps(EpsParams* dst, const EpsParams& v, cudaStream_t s);
void launch_cell_union(const ClusterArgs& a, int nblocks, cudaStream_t s);
void launch_uf_init(const ClusterArgs& a, bool fresh, cudaStream_t s);
void launch_uf_union(const ClusterArgs& a, int nblocks, cudaStream_t s);
void launch_uf_finish(const ClusterArgs& a, void* resolve_ws, void* scan_scratch,
                      cudaStream_t s);
void launch_border_and_write(const ClusterArgs& a, int nblocks, cudaStream_t s);
// the two halves of launch_border_and_write: border pull over rows
// [row_lo, row_hi) of the table held in nbr (from off_base), then the
// one-way in-edges and the label write (after every row has been pulled)
void launch_border_pull(const ClusterArgs& a, int nblocks, cudaStream_t s);
// st->clusters += sum over the V variants of their largest label (labels[v*n + i])
void launch_count_clusters(const uint32_t* labels, uint32_t n, uint32_t V, uint32_t* vmax,
                           DeviceStatus* st, cudaStream_t s);
void launch_label_write(const ClusterArgs& a, cudaStream_t s);

}  // namespace vdb
