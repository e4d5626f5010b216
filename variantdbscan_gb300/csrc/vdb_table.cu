// Epsilon-neighbourhood kernels: the count pass (|N_eps(p)| for every point,
// plus a bitmap of every candidate test) and the table pass (CSR neighbour
// table written from that bitmap).
//
// Work is split into units: a tile is up to 64 consecutive cell-ordered points
// of one cell; its candidates are the points of the cells within reach in the
// rows cy-rho..cy+rho, i.e. 2*rho+1 contiguous ranges of the cell-ordered
// arrays; a unit is one tile and one chunk of unit_words*32 of its
// candidates.  Persistent warps take units from a global counter; each warp
// holds one tile's queries (lane l: queries l and l+32) and stages its
// candidates in its own slice of shared memory.
//
// The neighbour predicate is the reference's (src/DBScan.cpp:665-702 with the
// R-tree candidate rule of src/RTree.h:1613-1625):
//   q in N(p)  <=>  sqrt(fl(fl(dx*dx)+fl(dy*dy))) <= eps     (dx = fl(px-qx), FP64)
//                   and q's multiple-point box overlaps [p-eps, p+eps]^2.
// sqrt is monotone and correctly rounded, so the first part is d2 <= thr with
// thr the largest double whose square root is <= eps.  The box part can only
// fail when d2 > tbox (a pair that deep inside the circle lies inside the query
// box).  Mixed precision: an FP32 quadratic form on cell-relative coordinates
// classifies a pair as in, out or within an error band around eps^2 whose
// width the host derives from the FP32 rounding bounds; only band pairs are
// re-tested with the FP64 predicate above, so membership is that of FP64.
//
// Table pass: the count pass stores, per tile, one 32-bit word per query and
// per 32 consecutive candidates (bit j: candidate j is a neighbour), laid out
// [word][query] so that a warp's 32 queries store 128 contiguous bytes.  The
// table pass turns each word into table entries (lane = bit), in candidate
// order, so every row comes out sorted.  An entry is 16 bits (the neighbour's
// position within its work unit of 1024 to 4096 candidates; readers decode it
// through the tile's row segments and the count pass's per-unit counts) or 32 bits (the
// cell-ordered index).  Entries accepted in one direction only are flagged
// afterwards from the asymmetric-pair list.  When the bitmap does not fit in
// device memory, the fill kernel (blocks of kTT threads, kQPT queries each)
// re-tests the candidates and writes the table directly.
#include "vdb_internal.cuh"

namespace vdb {

namespace {

constexpr int kTT = 256;              // threads per block
constexpr int kQPT = 2;               // queries per thread
constexpr int kChunk = 1024;          // candidates staged per round
constexpr unsigned kFull = 0xffffffffu;

// Row i (offset dy = i - rho) of the tile whose group starts at cell (cy, cx0):
// the candidate range [*st, *st + *len) and the key of the group's first cell
// in that row (so that key - base is the candidate's cell offset in x).
// Tile t's ranges come from a.trow_s / a.trow_e when those hold them (sparse
// grids, filled by the tile-words pass), else from the cell index.
__device__ __forceinline__ void tile_row(const TableArgs& a, const EpsParams* __restrict__ ep,
                                         int rho, uint32_t cy, uint32_t cx0, int i,
                                         uint32_t* st, uint32_t* len, uint32_t* base,
                                         uint32_t t = 0xffffffffu) {
    const int ry = (int)cy + i - rho;
    *st = 0;
    *len = 0;
    *base = 0;
    if (ry < 0 || ry >= (int)a.g.ncy) return;
    const int reach = ep->reach[i];
    const int lo_c = max((int)cx0 - reach, 0);
    const int hi_c = min((int)(cx0 + a.g.G - 1) + reach, (int)a.g.ncx - 1);
    const uint32_t rb = (uint32_t)ry * a.g.ncx_pad;
    uint32_t s = 0, e = 0;
    if (t != 0xffffffffu && a.trow_s) {
        const unsigned long long k = (unsigned long long)t * (uint32_t)(2 * rho + 1) + (uint32_t)i;
        s = a.trow_s[k];
        e = a.trow_e[k];
    } else {
        cell_row_range(a.g, a.cell_start, a.crow, a.ccx, a.clist, (uint32_t)ry, (uint32_t)lo_c,
                       (uint32_t)hi_c, &s, &e);
    }
    if (VDB_GUARD(a.st, s <= e && e <= a.n, 2, ((unsigned long long)s << 32) | e)) {
        *st = s;
        *len = e - s;
    }
    *base = rb + cx0;
}

// Cell-ordered index of candidate g of the tile (segments in shared memory).
__device__ __forceinline__ uint32_t tile_candidate(const uint32_t* s_seg_start,
                                                   const uint32_t* s_seg_off, int nrows,
                                                   uint32_t g, int* row) {
    int i = 0;
    while (i < nrows - 1 && s_seg_off[i + 1] <= g) i++;
    *row = i;
    return s_seg_start[i] + (g - s_seg_off[i]);
}

// Packed FP32 pairs (Blackwell f32x2 arithmetic): element-wise IEEE
// round-to-nearest, the same results as __fsub_rn / __fmaf_rn.
__device__ __forceinline__ unsigned long long f2_pack(float lo, float hi) {
    return ((unsigned long long)__float_as_uint(hi) << 32) | __float_as_uint(lo);
}
__device__ __forceinline__ unsigned long long f2_sub(unsigned long long a, unsigned long long b) {
    unsigned long long r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ unsigned long long f2_fma(unsigned long long a, unsigned long long b,
                                                     unsigned long long c) {
    unsigned long long r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}

// ------------------------------------------------------ warp-granular kernels
// The count and table passes give every warp its own tile of at most kWQ
// queries (one group of cells): the warp stages its candidates in its own
// slice of shared memory and synchronises with __syncwarp only, so small
// tiles (the common case with cells of eps/2) keep every warp busy.

constexpr int kWPB = 8;               // warps per block
constexpr int kWQ = 64;               // queries per warp tile (lane l: queries l and l+32)
constexpr int kWC = 128;              // candidates staged per warp round
constexpr int kWXW = 16;              // bitmap words per round of the table pass
constexpr int kRQ = 128;              // band pairs queued per warp for FP64 re-tests

struct WarpRows {
    uint32_t start[kMaxRows];
    uint32_t off[kMaxRows + 1];
    uint32_t base[kMaxRows];
    float dyw[kMaxRows];
};

// Row segments of the tile whose group starts at cell (cy, cx0), prefix of
// their lengths in r.off (r.off[nrows] = number of candidates).
__device__ __forceinline__ void warp_rows(const TableArgs& a, const EpsParams* __restrict__ ep,
                                          int rho, int nrows, uint32_t cy, uint32_t cx0,
                                          float wf, WarpRows& r, int lane, uint32_t t) {
    for (int i = lane; i < nrows; i += 32) {
        uint32_t st, len, base;
        tile_row(a, ep, rho, cy, cx0, i, &st, &len, &base, t);
        r.start[i] = st;
        r.off[i + 1] = len;
        r.base[i] = base;
        r.dyw[i] = __fmul_rn((float)(i - rho), wf);
    }
    __syncwarp();
    if (lane == 0) {
        uint32_t acc = 0;
        r.off[0] = 0;
        for (int i = 0; i < nrows; i++) {
            acc += r.off[i + 1];
            r.off[i + 1] = acc;
        }
    }
    __syncwarp();
}

// Count pass over work units (tile, chunk of unit_words*32 candidates): adds
// each query's neighbours in the chunk to deg, records them in parts (for the
// table pass) and, when a.bitmap is set, stores the chunk's test bitmap
// ([word][query] words; bit j of word w: candidate 32w+j is a neighbour).
template <bool MIXED>
__global__ void __launch_bounds__(kWPB * 32, 3) count_kernel(TableArgs a) {
    __shared__ WarpRows s_rows[kWPB];
    __shared__ double2 s_xy[kWPB][MIXED ? 1 : kWC];
    __shared__ uint32_t s_id[kWPB][kWC];
    __shared__ float4 s_relp[kWPB][MIXED ? kWC / 2 : 1];
    __shared__ float2 s_hcp[kWPB][MIXED ? kWC / 2 : 1];
    // band pairs of a word are re-tested in FP64 32 at a time, whatever query
    // they belong to: queue of (query slot, candidate) entries, the queries'
    // FP64 coordinates and the accepted bits per query slot
    __shared__ uint16_t s_rq[kWPB][kRQ];
    __shared__ double2 s_qd[kWPB][kWQ];
    __shared__ uint32_t s_madd[kWPB][kWQ];

    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    WarpRows& rows = s_rows[wib];
    uint16_t* rq = s_rq[wib];
    double2* sqd = s_qd[wib];
    uint32_t* madd = s_madd[wib];
    madd[lane] = 0u;
    madd[lane + 32] = 0u;
    float4* relp = s_relp[wib];
    float2* hcp = s_hcp[wib];
    double2* cxy = s_xy[wib];
    uint32_t* ids = s_id[wib];
    const EpsParams* __restrict__ ep = a.ep;
    const double eps = ep->eps, thr = ep->thr, tbox = ep->tbox;
    const ExactBounds xb = exact_bounds(eps, thr, tbox);
    const float L = ep->L32, wq = ep->w32;
    const int rho = ep->rho;
    const int nrows = 2 * rho + 1;
    const float wf = (float)a.g.w;
    const uint32_t nunits = *a.nunits;
    const uint32_t ncx_pad = a.g.ncx_pad, G = a.g.G;
    const float fnan = __int_as_float(0x7fc00000);
    const double dnan = __longlong_as_double(0x7ff8000000000000ll);
    unsigned long long my_retest = 0;

    for (;;) {
        uint32_t u = 0;
        if (lane == 0) u = atomicAdd(a.tile_counter, 1u);
        u = __shfl_sync(kFull, u, 0);
        if (u >= nunits) break;
        const uint32_t t = a.unit_tile[u];
        const uint32_t chunk = u - a.tile_uoff[t];
        const uint32_t qs = a.tiles[t], qe = a.tiles[t + 1];
        if (!(qs < qe && qe <= a.n && qe - qs <= kUnitQ)) {
            if (lane == 0) guard_fail(a.st, 1, ((unsigned long long)qs << 32) | qe);
            continue;
        }
        const uint32_t Q = qe - qs;
        const uint32_t key0 = a.gkey[qs];
        const uint32_t cy = key0 / ncx_pad;
        const uint32_t cx0 = (key0 - cy * ncx_pad) / G * G;
        const uint32_t tile_base = cy * ncx_pad + cx0;
        warp_rows(a, ep, rho, nrows, cy, cx0, wf, rows, lane, t);
        const uint32_t C = rows.off[nrows];
        const uint32_t cbeg = chunk * a.unit_words * 32u;
        const uint32_t cend = min(C, cbeg + a.unit_words * 32u);
        if (cbeg >= cend) continue;
        if (lane == 0) atomicAdd(&a.st->candidates, (unsigned long long)(cend - cbeg) * Q);
        const unsigned long long bm0 = a.bitmap ? a.tile_boff[t] : 0ull;

        float qx[2], qy[2];
        double2 qd[2];
        uint32_t qk[2], cnt[2];
#pragma unroll
        for (int q = 0; q < 2; q++) {
            const uint32_t k = qs + (uint32_t)lane + 32u * q;
            qk[q] = k;
            cnt[q] = 0;
            if (k < qe) {
                const float2 loc = a.glocal[k];
                const int dcx = (int)(a.gkey[k] - tile_base);
                qx[q] = __fmaf_rn((float)dcx, wf, loc.x);
                qy[q] = loc.y;
                qd[q] = a.gxy[k];
            } else {
                qx[q] = qy[q] = fnan;
                qd[q] = make_double2(dnan, dnan);
            }
        }
        const bool two = Q > 32;  // second query slot used by some lane
        sqd[lane] = qd[0];
        sqd[lane + 32] = qd[1];
        unsigned long long qxx[2], qyy[2], nhq2[2];
#pragma unroll
        for (int q = 0; q < 2; q++) {
            qxx[q] = f2_pack(qx[q], qx[q]);
            qyy[q] = f2_pack(qy[q], qy[q]);
            // -(|q|^2 - L)/2 (halving and negation are exact)
            const float q2 = __fmaf_rn(qx[q], qx[q], __fmul_rn(qy[q], qy[q]));
            const float nhq = -0.5f * __fsub_rn(q2, L);
            nhq2[q] = f2_pack(nhq, nhq);
        }
        // the float above w (w > 0)
        const float wup = __uint_as_float(__float_as_uint(wq) + 1u);
        const unsigned long long w2p = f2_pack(wup, wup);

        for (uint32_t cb = cbeg; cb < cend; cb += kWC) {
            const uint32_t len = min((uint32_t)kWC, cend - cb);
#pragma unroll
            for (int s = 0; s < kWC / 32; s++) {
                const uint32_t j = (uint32_t)lane + 32u * s;
                uint32_t k = 0xffffffffu;
                int i = 0;
                if (j < len) {
                    k = tile_candidate(rows.start, rows.off, nrows, cb + j, &i);
                    if (!VDB_GUARD(a.st, k < a.n, 3, k)) k = 0xffffffffu;
                }
                // pair slot of candidate j: (j>>5)*16 + (j&15), element j>>4 & 1
                float* pslot = reinterpret_cast<float*>(&relp[(j >> 5) * 16 + (j & 15)]) +
                               ((j >> 4) & 1);
                float* hslot = reinterpret_cast<float*>(&hcp[(j >> 5) * 16 + (j & 15)]) +
                               ((j >> 4) & 1);
                if (k != 0xffffffffu) {
                    if (MIXED) {
                        const float2 loc = a.glocal[k];
                        const int dcx = (int)(a.gkey[k] - rows.base[i]);
                        const float rx = __fmaf_rn((float)dcx, wf, loc.x);
                        const float ry = __fadd_rn(loc.y, rows.dyw[i]);
                        pslot[0] = rx;
                        pslot[2] = ry;
                        hslot[0] = 0.5f * __fmaf_rn(rx, rx, __fmul_rn(ry, ry));
                    } else {
                        cxy[j] = a.gxy[k];
                    }
                    ids[j] = k;
                } else {
                    if (MIXED) {
                        pslot[0] = fnan;
                        pslot[2] = fnan;
                        hslot[0] = fnan;
                    } else {
                        cxy[j] = make_double2(dnan, dnan);
                    }
                    ids[j] = 0;
                }
            }
            __syncwarp();
            for (uint32_t j0 = 0; j0 < len; j0 += 32) {
                uint32_t m[2] = {0u, 0u}, amb[2] = {0u, 0u};
                if (MIXED) {
                    // Candidates jj and jj+16 are tested together with packed FP32
                    // pair instructions (each element rounds exactly like the
                    // scalar __f*_rn operations of the fill pass); sign bits are
                    // gathered by funnel shifts (bit 31-jj, reversed below).
                    // nS =|c|^2/2 - (q.c - (|q|^2 - L)/2) = (d2 - L)/2: two
                    // fma and one subtraction per test; its sign is the
                    // in-mask.  The sign of nS - w' (w' the float above w, so
                    // negative <=> nS <= w; a difference of floats is zero only
                    // for equal operands, so its sign is exact) marks the tests
                    // that are not out; band = not out and not in.  NaN (empty
                    // query or candidate slots) has both signs clear.
                    uint32_t ma[2] = {0u, 0u}, mb[2] = {0u, 0u}, oa[2] = {0u, 0u}, ob[2] = {0u, 0u};
                    const ulonglong2* pr = reinterpret_cast<const ulonglong2*>(relp) + (j0 >> 5) * 16;
                    const unsigned long long* ph =
                        reinterpret_cast<const unsigned long long*>(hcp) + (j0 >> 5) * 16;
#pragma unroll
                    for (int jj = 0; jj < 16; jj++) {
                        const ulonglong2 c = pr[jj];  // (x_a, x_b), (y_a, y_b)
                        const unsigned long long hc = ph[jj];  // (|c_a|^2/2, |c_b|^2/2)
#pragma unroll
                        for (int q = 0; q < 2; q++) {
                            if (q == 1 && !two) break;
                            const unsigned long long ay = f2_fma(qyy[q], c.y, nhq2[q]);
                            const unsigned long long qc = f2_fma(qxx[q], c.x, ay);
                            const unsigned long long s = f2_sub(hc, qc);
                            const unsigned long long nw = f2_sub(s, w2p);
                            ma[q] = __funnelshift_l((uint32_t)s, ma[q], 1);
                            mb[q] = __funnelshift_l((uint32_t)(s >> 32), mb[q], 1);
                            oa[q] = __funnelshift_l((uint32_t)nw, oa[q], 1);
                            ob[q] = __funnelshift_l((uint32_t)(nw >> 32), ob[q], 1);
                        }
                    }
#pragma unroll
                    for (int q = 0; q < 2; q++) {
                        m[q] = __brev((ma[q] << 16) | (mb[q] & 0xffffu));
                        amb[q] = __brev((oa[q] << 16) | (ob[q] & 0xffffu)) & ~m[q];
                    }
                } else {
                    uint32_t hm[2] = {0u, 0u};
#pragma unroll
                    for (int jj = 0; jj < 32; jj++) {
                        const double2 c = cxy[j0 + jj];
#pragma unroll
                        for (int q = 0; q < 2; q++) {
                            if (q == 1 && !two) break;
                            const double dx = __dsub_rn(qd[q].x, c.x);
                            const double dy = __dsub_rn(qd[q].y, c.y);
                            const double d2 = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
                            m[q] |= (d2 <= tbox) ? (1u << jj) : 0u;
                            hm[q] |= (d2 <= thr) ? (1u << jj) : 0u;
                        }
                    }
                    amb[0] = hm[0] & ~m[0];
                    amb[1] = hm[1] & ~m[1];
                }
                // pairs in the band: exact FP64 predicate, 32 pairs per step
                // of the warp (queued in shared memory, whatever their query)
                if (__any_sync(kFull, (amb[0] | amb[1]) != 0u)) {
                    const uint32_t c = __popc(amb[0]) + __popc(amb[1]);
                    uint32_t incl = c;
#pragma unroll
                    for (int d = 1; d < 32; d <<= 1) {
                        const uint32_t v = __shfl_up_sync(kFull, incl, d);
                        if (lane >= d) incl += v;
                    }
                    const uint32_t excl = incl - c;
                    const uint32_t total = __shfl_sync(kFull, incl, 31);
                    for (uint32_t pb = 0; pb < total; pb += kRQ) {
                        uint32_t idx = excl;
#pragma unroll
                        for (int q = 0; q < 2; q++) {
                            for (uint32_t bits = amb[q]; bits; bits &= bits - 1u, idx++) {
                                if (idx >= pb && idx < pb + kRQ)
                                    rq[idx - pb] = (uint16_t)(((uint32_t)lane << 6) |
                                                              ((uint32_t)q << 5) |
                                                              (uint32_t)(__ffs(bits) - 1));
                            }
                        }
                        __syncwarp();
                        const uint32_t ne = min((uint32_t)kRQ, total - pb);
                        for (uint32_t e = lane; e < ne; e += 32) {
                            const uint32_t ent = rq[e];
                            const uint32_t slot_q = (ent >> 6) + 32u * ((ent >> 5) & 1u);
                            const uint32_t jj = ent & 31u;
                            const uint32_t kp = qs + slot_q;
                            const uint32_t kq = ids[j0 + jj];
                            const uint32_t r =
                                exact_pair(sqd[slot_q], a.gxy[kq], kp, kq, xb, a.gbox);
                            my_retest++;
                            if (r & 1u) atomicOr(&madd[slot_q], 1u << jj);
                            if ((r == 1u || r == 2u) && kp < kq) {
                                const uint32_t slot = atomicAdd(a.asym_n, 1u);
                                if (slot < a.asym_cap) {
                                    AsymPair ap;
                                    ap.a = kp;
                                    ap.b = kq;
                                    ap.dir = r;
                                    ap.pad = 0u;
                                    a.asym[slot] = ap;
                                } else {
                                    atomicOr(&a.st->flags, kStatAsymOverflow);
                                }
                            }
                        }
                        __syncwarp();
                    }
                    m[0] |= madd[lane];
                    m[1] |= madd[lane + 32];
                    madd[lane] = 0u;
                    madd[lane + 32] = 0u;
                    __syncwarp();
                }
                const unsigned long long wrow = bm0 + (unsigned long long)((cb + j0) >> 5) * Q;
#pragma unroll
                for (int q = 0; q < 2; q++) {
                    if (qk[q] < qe) {
                        cnt[q] += __popc(m[q]);
                        if (a.bitmap) a.bitmap[wrow + (qk[q] - qs)] = m[q];
                    }
                }
            }
            __syncwarp();
        }
#pragma unroll
        for (int q = 0; q < 2; q++) {
            if (qk[q] < qe) {
                if (cnt[q]) atomicAdd(&a.deg[qk[q]], cnt[q]);
                if (a.parts) a.parts[(unsigned long long)u * kUnitQ + lane + 32u * q] = cnt[q];
            }
        }
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) my_retest += __shfl_down_sync(kFull, my_retest, d);
    if (lane == 0 && my_retest) atomicAdd(&a.st->retested, my_retest);
}

// Table pass over the same work units: neighbour ids from the count pass's
// bitmap.  A unit's rows start at the row offsets plus the neighbours of the
// tile's earlier units (parts).  The warp expands the unit in rounds of kWXW
// words.  Each lane keeps the ids of its bit of the round's words in
// registers.  The round's words are transposed through the warp's shared
// memory, 32 queries at a time: lane q loads query q's words (coalesced over
// q), adds up their popcounts into the in-row offset of every word and takes
// its row cursor forward; every query's slot (words, offsets, cursor, count)
// is then read back with a few broadcast vector loads.  Lane l shifts each word
// left by 31-l: the sign bit is its own bit and the popcount is its rank among
// the word's neighbours plus one, so the entry goes to the word's staging
// address (that of the entry before its first) plus 4 * popcount.  Rows come
// out in candidate order, which is increasing neighbour index.
//
// Stores: a query's ids of a round are first placed in a shared-memory
// staging buffer (one store per word, lane = bit, at the same position modulo
// 16 bytes as their place in the table); the 16-byte-aligned middle of the
// segment then goes to the table as one asynchronous bulk copy, and the at
// most 3 + 3 entries before and after it as plain stores.  The warp's stores
// thus become shared-memory stores that do not wait on the memory system, and
// the copies run while the warp expands the next queries.  Two staging buffers
// per warp, used in turn: before a buffer is refilled, the copy last issued
// from it (if any) must have read it.
//
// A round writes a query's segment only up to its last 32-byte boundary; the
// at most 7 entries after it are kept in shared memory and staged again in
// front of the query's next round (the unit's last round writes everything).
// The row's next segment follows a whole round over the tile's other queries
// later, and a sector left half written for that long was measured to cost
// about a third of the write bandwidth.
constexpr int kXS = 36;  // words per query slot: 16 words, 16 staging addresses, cursor, counts
constexpr int kXPB = 3;        // warps per block

// Entry layout of a table with entries of type E (uint32_t: cell-ordered
// index; uint16_t: position in the tile's candidate list): entries per 16
// bytes (the bulk-copy granule) and per 32-byte sector (carry alignment), and
// staging entries per buffer (phase + carried entries + one round's entries,
// rounded up to a granule).
template <typename E>
struct XFmt {
    static constexpr uint32_t kVec = 16 / sizeof(E);
    static constexpr uint32_t kSec = 32 / sizeof(E);
    static constexpr uint32_t kStage = ((kVec - 1) + (kSec - 1) + kWXW * 32 + kVec - 1) / kVec * kVec;
};

// Stores v at shared-memory address addr if x is negative (one predicated store).
__device__ __forceinline__ void st_shared_if_neg(int x, uint32_t addr, uint32_t v) {
    asm volatile("{ .reg .pred p; setp.lt.s32 p, %0, 0; @p st.shared.u32 [%1], %2; }"
                 ::"r"(x), "r"(addr), "r"(v) : "memory");
}
__device__ __forceinline__ void st_shared_if_neg(int x, uint32_t addr, uint16_t v) {
    asm volatile("{ .reg .pred p; setp.lt.s32 p, %0, 0; @p st.shared.u16 [%1], %2; }"
                 ::"r"(x), "r"(addr), "h"(v) : "memory");
}

__device__ __forceinline__ void bulk_copy_to_global(void* gdst, const void* ssrc,
                                                    uint32_t bytes) {
    const uint32_t s = (uint32_t)__cvta_generic_to_shared(ssrc);
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;"
                 ::"l"(gdst), "r"(s), "r"(bytes) : "memory");
    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}

template <typename E>
__global__ void __launch_bounds__(kXPB * 32, 6) expand_kernel(TableArgs a) {
    constexpr uint32_t kVec = XFmt<E>::kVec, kSec = XFmt<E>::kSec, kStage = XFmt<E>::kStage;
    constexpr bool kCompact = sizeof(E) == 2;
    static_assert(kWXW == 16, "the query slot layout holds 16 words");
    static_assert(kSec <= 16, "carry counts take 4 bits of the slot");
    __shared__ WarpRows s_rows[kXPB];
    __shared__ __align__(16) uint32_t s_slot[kXPB][32 * kXS];
    __shared__ __align__(16) E s_stage[kXPB][2][kStage];
    __shared__ E s_carry[kXPB][kWQ][kSec];
    E* const nbr = reinterpret_cast<E*>(a.nbr);

    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const uint32_t lsh = 31u - (uint32_t)lane;
    WarpRows& rows = s_rows[wib];
    uint32_t* slots = s_slot[wib];
    const EpsParams* __restrict__ ep = a.ep;
    const int rho = ep->rho;
    const int nrows = 2 * rho + 1;
    const float wf = (float)a.g.w;
    // units of the row chunk (all units when unit_hi is 0)
    const uint32_t nunits = a.unit_hi ? min(*a.nunits, a.unit_hi) : *a.nunits;
    const uint32_t ncx_pad = a.g.ncx_pad, G = a.g.G;
    uint32_t par = 0;        // staging buffer of the next query
    uint32_t pending = 0;    // bit b: a copy from buffer b may still be reading it
    uint32_t last_copy = 0;  // buffer of the most recent copy
    const uint32_t stage_s = (uint32_t)__cvta_generic_to_shared(&s_stage[wib][0][0]);

    for (;;) {
        uint32_t u = 0;
        if (lane == 0) u = a.unit_lo + atomicAdd(a.tile_counter, 1u);
        u = __shfl_sync(kFull, u, 0);
        if (u >= nunits) break;
        const uint32_t t = a.unit_tile[u];
        const uint32_t u0 = a.tile_uoff[t];
        const uint32_t qs = a.tiles[t], qe = a.tiles[t + 1];
        if (!(qs < qe && qe <= a.n && qe - qs <= kUnitQ && u0 <= u)) {
            if (lane == 0) guard_fail(a.st, 4, ((unsigned long long)qs << 32) | qe);
            continue;
        }
        const uint32_t Q = qe - qs;
        const uint32_t key0 = a.gkey[qs];
        const uint32_t cy = key0 / ncx_pad;
        const uint32_t cx0 = (key0 - cy * ncx_pad) / G * G;
        warp_rows(a, ep, rho, nrows, cy, cx0, wf, rows, lane, t);
        const uint32_t C = rows.off[nrows];
        const uint32_t words = (C + 31u) >> 5;
        const uint32_t wbeg = (u - u0) * a.unit_words;
        const uint32_t wend = min(words, wbeg + a.unit_words);
        const unsigned long long bm0 = a.tile_boff[t];
        // row cursors: lane l holds queries l and l+32
        const bool v0 = qs + lane < qe, v1 = qs + lane + 32 < qe;
        // rows written: all, or (row_deg_lim) those of points with deg < lim
        const uint32_t lim = a.row_deg_lim;
        const bool w0row = v0 && (!lim || a.deg[qs + lane] < lim);
        const bool w1row = v1 && (!lim || a.deg[qs + lane + 32] < lim);
        if (!__any_sync(kFull, w0row || w1row)) continue;
        unsigned long long cur0 = v0 ? a.off[qs + lane] - a.off_base : 0;
        unsigned long long cur1 = v1 ? a.off[qs + lane + 32] - a.off_base : 0;
        for (uint32_t uu = u0; uu < u; uu++) {
            if (v0) cur0 += a.parts[(unsigned long long)uu * kUnitQ + lane];
            if (v1) cur1 += a.parts[(unsigned long long)uu * kUnitQ + lane + 32];
        }
        // entries staged but not yet written (carried to the next round)
        uint32_t nc0 = 0, nc1 = 0;
        for (uint32_t w0 = wbeg; w0 < wend; w0 += kWXW) {
            const uint32_t nw = min((uint32_t)kWXW, wend - w0);
            const bool last = w0 + kWXW >= wend;  // the unit's last round: write everything
            // entry of each lane's candidate of the round's words: its
            // cell-ordered index, or (compact) its position in the unit
            E id[kWXW];
#pragma unroll
            for (int s = 0; s < kWXW; s++) {
                const uint32_t g = (w0 + (uint32_t)s) * 32u + (uint32_t)lane;
                id[s] = 0;
                if (g < C) {
                    if (kCompact) {
                        id[s] = (E)((w0 - wbeg + (uint32_t)s) * 32u + (uint32_t)lane);
                    } else {
                        int i;
                        id[s] = (E)tile_candidate(rows.start, rows.off, nrows, g, &i);
                    }
                }
            }
            const uint32_t* bw = a.bitmap + bm0 + (unsigned long long)w0 * Q;
            for (uint32_t qh = 0; qh < Q; qh += 32) {
                const uint32_t q = qh + (uint32_t)lane;
                __syncwarp();  // the previous slots have been read
                const bool wrow = qh == 0 ? w0row : w1row;
                uint32_t todo = __ballot_sync(kFull, wrow);  // queries whose rows are written
                if (wrow) {
                    uint32_t wd[kWXW], pm[kWXW];
#pragma unroll
                    for (int s = 0; s < kWXW; s++)
                        wd[s] = ((uint32_t)s < nw) ? __ldg(bw + (unsigned long long)s * Q + q) : 0u;
                    const unsigned long long cur = qh == 0 ? cur0 : cur1;
                    const uint32_t nc = qh == 0 ? nc0 : nc1;
                    // table entry wcur + k sits at staging position
                    // (wcur mod kVec) + k: the carried entries first, then this round's
                    const unsigned long long wcur = cur - nc;
                    uint32_t acc = ((uint32_t)wcur & (kVec - 1u)) + nc;
                    // the staging buffer of this query (queries take the two
                    // buffers in turn, in increasing order); pm[s] = shared
                    // address of the entry before word s's first
                    const uint32_t bq = par ^ (__popc(todo & ((1u << lane) - 1u)) & 1u);
                    const uint32_t sbase = stage_s + bq * (uint32_t)(kStage * sizeof(E));
#pragma unroll
                    for (int s = 0; s < kWXW; s++) {
                        pm[s] = sbase + (uint32_t)sizeof(E) * (acc - 1u);
                        acc += __popc(wd[s]);
                    }
                    const uint32_t nstage = acc - ((uint32_t)wcur & (kVec - 1u));  // carried + new
                    const unsigned long long end = wcur + nstage;
                    // written this round: up to the last 32-byte boundary (all at
                    // the unit's last round), never before wcur
                    unsigned long long wto = last ? end : (end & ~(unsigned long long)(kSec - 1u));
                    if (wto < wcur) wto = wcur;
                    const uint32_t nwrite = (uint32_t)(wto - wcur);
                    uint4* sl = reinterpret_cast<uint4*>(slots + lane * kXS);
#pragma unroll
                    for (int v = 0; v < 4; v++) {
                        sl[v] = make_uint4(wd[4 * v], wd[4 * v + 1], wd[4 * v + 2], wd[4 * v + 3]);
                        sl[4 + v] = make_uint4(pm[4 * v], pm[4 * v + 1], pm[4 * v + 2], pm[4 * v + 3]);
                    }
                    sl[8] = make_uint4((uint32_t)wcur, (uint32_t)(wcur >> 32), nstage, nc | (nwrite << 4));
                    if (qh == 0) {
                        cur0 = end;
                        nc0 = nstage - nwrite;
                    } else {
                        cur1 = end;
                        nc1 = nstage - nwrite;
                    }
                }
                __syncwarp();
                for (; todo; todo &= todo - 1u) {
                    const uint32_t qi = (uint32_t)__ffs(todo) - 1u;
                    const uint4* sl = reinterpret_cast<const uint4*>(slots + qi * kXS);
                    uint32_t W[kWXW], P[kWXW];
#pragma unroll
                    for (int v = 0; v < 4; v++) {
                        const uint4 w4 = sl[v], p4 = sl[4 + v];
                        W[4 * v] = w4.x; W[4 * v + 1] = w4.y; W[4 * v + 2] = w4.z; W[4 * v + 3] = w4.w;
                        P[4 * v] = p4.x; P[4 * v + 1] = p4.y; P[4 * v + 2] = p4.z; P[4 * v + 3] = p4.w;
                    }
                    const uint4 cc = sl[8];
                    const unsigned long long wcur = ((unsigned long long)cc.y << 32) | cc.x;
                    const uint32_t nstage = cc.z, nc = cc.w & 15u, nwrite = cc.w >> 4;
                    E* const carry = s_carry[wib][qh + qi];
                    // a copy from this buffer must have read it: if it is the
                    // latest copy, wait for all copies, else for all but one
                    const uint32_t b = par;
                    E* const buf = s_stage[wib][b];
                    par ^= 1u;
                    if (pending & (1u << b)) {
                        if (lane == 0) {
                            if (last_copy == b)
                                asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
                            else
                                asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory");
                        }
                        pending &= ~(1u << b);
                    }
                    __syncwarp();
                    // table entry wcur + k sits at buf[phase + k]
                    const uint32_t phase = (uint32_t)wcur & (kVec - 1u);
                    if ((uint32_t)lane < nc) buf[phase + lane] = carry[lane];
#pragma unroll
                    for (int wi = 0; wi < kWXW; wi++) {
                        const uint32_t x = W[wi] << lsh;
                        st_shared_if_neg((int)x, P[wi] + (uint32_t)sizeof(E) * __popc(x), id[wi]);
                    }
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                    __syncwarp();
                    const unsigned long long wto = wcur + nwrite;
                    const unsigned long long A = (wcur + (kVec - 1u)) & ~(unsigned long long)(kVec - 1u);
                    const unsigned long long B = wto & ~(unsigned long long)(kVec - 1u);
                    E* const sb = buf + phase;
                    if (B > A) {
                        if (lane == 0)
                            bulk_copy_to_global(nbr + A, sb + (uint32_t)(A - wcur),
                                                (uint32_t)(B - A) * (uint32_t)sizeof(E));
                        pending |= 1u << b;
                        last_copy = b;
                        const uint32_t nh = (uint32_t)(A - wcur), nt = (uint32_t)(wto - B);
                        if ((uint32_t)lane < nh)
                            nbr[wcur + (uint32_t)lane] = sb[lane];
                        else if ((uint32_t)lane >= kVec && (uint32_t)lane - kVec < nt)
                            nbr[B + ((uint32_t)lane - kVec)] = sb[(uint32_t)(B - wcur) + ((uint32_t)lane - kVec)];
                    } else if ((uint32_t)lane < nwrite) {
                        nbr[wcur + (uint32_t)lane] = sb[lane];  // fewer than 2 kVec - 1 entries
                    }
                    // entries after the last 32-byte boundary wait for the next round
                    if ((uint32_t)lane < nstage - nwrite) carry[lane] = sb[nwrite + (uint32_t)lane];
                }
            }
        }
    }
    if (lane == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}

// 16-bit tables: two queries per pass.  The round's words are transposed
// into the query slots as above (lane = query); then lanes 0-15 expand one
// query of a pair and lanes 16-31 the other, lane j of a half taking bits j
// and j + 16 of every word.  The work of a query that does not depend on its
// words (slot reads, barriers, the proxy fence, the bulk copy, the head and
// tail stores, the carry) is thus done once per two queries.  One staging
// buffer per half: before a half stages its next query, its first lane waits
// until its copies have read the buffer (bulk async-groups belong to the
// issuing thread).  With one buffer per half and no per-warp row table (the
// 16-bit entries need only the tile's candidate count), 8 blocks of 3 warps
// (80 registers, 26.4 KB of shared memory) share an SM; the extra warps hide
// more of the kernel's dependency latency (2M sweep: 34.7 ms of tables against
// 40.3 with two buffers per half at 6 blocks).
__global__ void __launch_bounds__(kXPB * 32, 8) expand16_kernel(TableArgs a) {
    using E = uint16_t;
    constexpr uint32_t kVec = XFmt<E>::kVec, kSec = XFmt<E>::kSec, kStage = XFmt<E>::kStage;
    static_assert(kWXW == 16, "the query slot layout holds 16 words");
    static_assert(kSec <= 16 && 2 * kVec <= 16, "head, tail and carry fit a half-warp");
    __shared__ __align__(16) uint32_t s_slot[kXPB][32 * kXS];
    __shared__ __align__(16) E s_stage[kXPB][2][kStage];
    __shared__ E s_carry[kXPB][kWQ][kSec];
    E* const nbr = reinterpret_cast<E*>(a.nbr);

    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const uint32_t hj = (uint32_t)lane & 15u, half = (uint32_t)lane >> 4;
    const uint32_t lsh_a = 31u - hj, lsh_b = 15u - hj;  // bit hj, bit hj + 16 to the sign
    uint32_t* slots = s_slot[wib];
    const EpsParams* __restrict__ ep = a.ep;
    const int rho = ep->rho;
    const int nrows = 2 * rho + 1;
    const uint32_t nunits = a.unit_hi ? min(*a.nunits, a.unit_hi) : *a.nunits;
    const uint32_t ncx_pad = a.g.ncx_pad, G = a.g.G;
    uint32_t pending = 0;    // nonzero: a copy from this half's buffer may be reading it
    const uint32_t stage_s = (uint32_t)__cvta_generic_to_shared(&s_stage[wib][0][0]);

    for (;;) {
        uint32_t u = 0;
        if (lane == 0) u = a.unit_lo + atomicAdd(a.tile_counter, 1u);
        u = __shfl_sync(kFull, u, 0);
        if (u >= nunits) break;
        const uint32_t t = a.unit_tile[u];
        const uint32_t u0 = a.tile_uoff[t];
        const uint32_t qs = a.tiles[t], qe = a.tiles[t + 1];
        if (!(qs < qe && qe <= a.n && qe - qs <= kUnitQ && u0 <= u)) {
            if (lane == 0) guard_fail(a.st, 4, ((unsigned long long)qs << 32) | qe);
            continue;
        }
        const uint32_t Q = qe - qs;
        const uint32_t key0 = a.gkey[qs];
        const uint32_t cy = key0 / ncx_pad;
        const uint32_t cx0 = (key0 - cy * ncx_pad) / G * G;
        // candidates of the tile (16-bit entries are positions: the rows'
        // starts are not needed here)
        uint32_t Cl = 0;
        for (int i = lane; i < nrows; i += 32) {
            uint32_t st, len, base;
            tile_row(a, ep, rho, cy, cx0, i, &st, &len, &base, t);
            Cl += len;
        }
        const uint32_t C = __reduce_add_sync(kFull, Cl);
        const uint32_t words = (C + 31u) >> 5;
        const uint32_t wbeg = (u - u0) * a.unit_words;
        const uint32_t wend = min(words, wbeg + a.unit_words);
        const unsigned long long bm0 = a.tile_boff[t];
        const bool v0 = qs + lane < qe, v1 = qs + lane + 32 < qe;
        const uint32_t lim = a.row_deg_lim;
        const bool w0row = v0 && (!lim || a.deg[qs + lane] < lim);
        const bool w1row = v1 && (!lim || a.deg[qs + lane + 32] < lim);
        if (!__any_sync(kFull, w0row || w1row)) continue;
        unsigned long long cur0 = v0 ? a.off[qs + lane] - a.off_base : 0;
        unsigned long long cur1 = v1 ? a.off[qs + lane + 32] - a.off_base : 0;
        for (uint32_t uu = u0; uu < u; uu++) {
            if (v0) cur0 += a.parts[(unsigned long long)uu * kUnitQ + lane];
            if (v1) cur1 += a.parts[(unsigned long long)uu * kUnitQ + lane + 32];
        }
        uint32_t nc0 = 0, nc1 = 0;
        for (uint32_t w0 = wbeg; w0 < wend; w0 += kWXW) {
            const uint32_t nw = min((uint32_t)kWXW, wend - w0);
            const bool last = w0 + kWXW >= wend;
            // position in the unit of bit hj of the round's word s (bit hj + 16:
            // + 16); bits past the candidates are never set
            const uint32_t idbase = (w0 - wbeg) * 32u + hj;
            const uint32_t* bw = a.bitmap + bm0 + (unsigned long long)w0 * Q;
            for (uint32_t qh = 0; qh < Q; qh += 32) {
                const uint32_t q = qh + (uint32_t)lane;
                __syncwarp();  // the previous slots have been read
                const bool wrow = qh == 0 ? w0row : w1row;
                uint32_t todo = __ballot_sync(kFull, wrow);
                if (wrow) {
                    uint32_t wd[kWXW], pm[kWXW];
#pragma unroll
                    for (int s = 0; s < kWXW; s++)
                        wd[s] = ((uint32_t)s < nw) ? __ldg(bw + (unsigned long long)s * Q + q) : 0u;
                    const unsigned long long cur = qh == 0 ? cur0 : cur1;
                    const uint32_t nc = qh == 0 ? nc0 : nc1;
                    const unsigned long long wcur = cur - nc;
                    uint32_t acc = ((uint32_t)wcur & (kVec - 1u)) + nc;
                    // the k-th query of todo is expanded in pass k / 2 by half
                    // k % 2, in that half's buffer
                    const uint32_t k = __popc(todo & ((1u << lane) - 1u));
                    const uint32_t bq = k & 1u;
                    const uint32_t sbase = stage_s + bq * (uint32_t)(kStage * sizeof(E));
#pragma unroll
                    for (int s = 0; s < kWXW; s++) {
                        pm[s] = sbase + (uint32_t)sizeof(E) * (acc - 1u);
                        acc += __popc(wd[s]);
                    }
                    const uint32_t nstage = acc - ((uint32_t)wcur & (kVec - 1u));
                    const unsigned long long end = wcur + nstage;
                    unsigned long long wto = last ? end : (end & ~(unsigned long long)(kSec - 1u));
                    if (wto < wcur) wto = wcur;
                    const uint32_t nwrite = (uint32_t)(wto - wcur);
                    uint4* sl = reinterpret_cast<uint4*>(slots + lane * kXS);
#pragma unroll
                    for (int v = 0; v < 4; v++) {
                        sl[v] = make_uint4(wd[4 * v], wd[4 * v + 1], wd[4 * v + 2], wd[4 * v + 3]);
                        sl[4 + v] = make_uint4(pm[4 * v], pm[4 * v + 1], pm[4 * v + 2], pm[4 * v + 3]);
                    }
                    sl[8] = make_uint4((uint32_t)wcur, (uint32_t)(wcur >> 32), nstage, nc | (nwrite << 4));
                    if (qh == 0) {
                        cur0 = end;
                        nc0 = nstage - nwrite;
                    } else {
                        cur1 = end;
                        nc1 = nstage - nwrite;
                    }
                }
                __syncwarp();
                while (todo) {
                    const uint32_t qa = (uint32_t)__ffs(todo) - 1u;
                    todo &= todo - 1u;
                    const bool has_b = todo != 0u;
                    const uint32_t qb = has_b ? (uint32_t)__ffs(todo) - 1u : qa;
                    if (has_b) todo &= todo - 1u;
                    const bool act = half == 0u || has_b;  // the second half idles on an odd count
                    const uint32_t qi = half ? qb : qa;
                    const uint4* sl = reinterpret_cast<const uint4*>(slots + qi * kXS);
                    uint32_t W[kWXW], P[kWXW];
#pragma unroll
                    for (int v = 0; v < 4; v++) {
                        const uint4 w4 = sl[v], p4 = sl[4 + v];
                        W[4 * v] = w4.x; W[4 * v + 1] = w4.y; W[4 * v + 2] = w4.z; W[4 * v + 3] = w4.w;
                        P[4 * v] = p4.x; P[4 * v + 1] = p4.y; P[4 * v + 2] = p4.z; P[4 * v + 3] = p4.w;
                    }
                    const uint4 cc = sl[8];
                    const unsigned long long wcur = ((unsigned long long)cc.y << 32) | cc.x;
                    const uint32_t nstage = cc.z, nc = cc.w & 15u, nwrite = cc.w >> 4;
                    E* const carry = s_carry[wib][qh + qi];
                    E* const buf = s_stage[wib][half];
                    // the half's copies must have read its buffer
                    if (act && pending) {
                        if (hj == 0) asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
                        pending = 0;
                    }
                    __syncwarp();
                    const uint32_t phase = (uint32_t)wcur & (kVec - 1u);
                    if (act) {
                        if (hj < nc) buf[phase + hj] = carry[hj];
#pragma unroll
                        for (int wi = 0; wi < kWXW; wi++) {
                            const uint32_t xa = W[wi] << lsh_a, xb = W[wi] << lsh_b;
                            const uint32_t id = idbase + 32u * (uint32_t)wi;
                            st_shared_if_neg((int)xa, P[wi] + (uint32_t)sizeof(E) * __popc(xa), (E)id);
                            st_shared_if_neg((int)xb, P[wi] + (uint32_t)sizeof(E) * __popc(xb),
                                             (E)(id + 16u));
                        }
                    }
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                    __syncwarp();
                    if (act) {
                        const unsigned long long wto = wcur + nwrite;
                        const unsigned long long A = (wcur + (kVec - 1u)) & ~(unsigned long long)(kVec - 1u);
                        const unsigned long long B = wto & ~(unsigned long long)(kVec - 1u);
                        E* const sb = buf + phase;
                        if (B > A) {
                            if (hj == 0)
                                bulk_copy_to_global(nbr + A, sb + (uint32_t)(A - wcur),
                                                    (uint32_t)(B - A) * (uint32_t)sizeof(E));
                            pending = 1u;
                            const uint32_t nh = (uint32_t)(A - wcur), nt = (uint32_t)(wto - B);
                            if (hj < nh)
                                nbr[wcur + hj] = sb[hj];
                            else if (hj >= kVec && hj - kVec < nt)
                                nbr[B + (hj - kVec)] = sb[(uint32_t)(B - wcur) + (hj - kVec)];
                        } else if (hj < nwrite) {
                            nbr[wcur + hj] = sb[hj];  // fewer than 2 kVec - 1 entries
                        }
                        if (hj < nstage - nwrite) carry[hj] = sb[nwrite + hj];
                    }
                }
            }
        }
    }
    if (hj == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}

template <bool MIXED, bool FILL>
__global__ void __launch_bounds__(kTT) table_kernel(TableArgs a) {
    __shared__ float2 s_rel[kChunk];
    __shared__ double2 s_xy[kChunk];
    __shared__ uint32_t s_id[kChunk];
    __shared__ uint32_t s_seg_start[kMaxRows];
    __shared__ uint32_t s_seg_off[kMaxRows + 1];
    __shared__ uint32_t s_seg_base[kMaxRows];
    __shared__ float s_seg_dyw[kMaxRows];
    __shared__ uint32_t s_tile;

    const int tid = threadIdx.x, lane = tid & 31;
    const uint32_t lt = (1u << lane) - 1u;
    const EpsParams* __restrict__ ep = a.ep;
    const double eps = ep->eps, thr = ep->thr, tbox = ep->tbox;
    const ExactBounds xb = exact_bounds(eps, thr, tbox);
    const float lo = ep->lo32, hi = ep->hi32;
    const int rho = ep->rho;
    const int nrows = 2 * rho + 1;
    const float wf = (float)a.g.w;
    const uint32_t tile_end = a.tile_end != 0xffffffffu ? a.tile_end : *a.ntiles;
    const uint32_t ncx_pad = a.g.ncx_pad, G = a.g.G;
    unsigned long long my_retest = 0;

    for (;;) {
        if (tid == 0) s_tile = a.tile_lo + atomicAdd(a.tile_counter, 1u);
        __syncthreads();
        const uint32_t t = s_tile;
        if (t >= tile_end) break;
        const uint32_t qs = a.tiles[t], qe = a.tiles[t + 1];
        if (!(qs < qe && qe <= a.n)) {
            if (tid == 0) guard_fail(a.st, 1, ((unsigned long long)qs << 32) | qe);
            __syncthreads();
            continue;
        }
        const uint32_t Q = qe - qs;
        const uint32_t key0 = a.gkey[qs];
        const uint32_t cy = key0 / ncx_pad;
        const uint32_t cx0 = (key0 - cy * ncx_pad) / G * G;
        const uint32_t tile_base = cy * ncx_pad + cx0;
        // bitmap of this tile (count pass only)
        const unsigned long long bm0 = (!FILL && a.bitmap) ? a.tile_boff[t] : 0ull;

        if (tid < nrows) {
            uint32_t st, len, base;
            tile_row(a, ep, rho, cy, cx0, tid, &st, &len, &base);
            s_seg_start[tid] = st;
            s_seg_off[tid + 1] = len;
            s_seg_base[tid] = base;
            s_seg_dyw[tid] = __fmul_rn((float)(tid - rho), wf);
        }
        __syncthreads();
        if (tid == 0) {
            uint32_t acc = 0;
            s_seg_off[0] = 0;
            for (int i = 0; i < nrows; i++) {
                acc += s_seg_off[i + 1];
                s_seg_off[i + 1] = acc;
            }
            if (!FILL) atomicAdd(&a.st->candidates, (unsigned long long)acc * Q);
        }
        __syncthreads();
        const uint32_t C = s_seg_off[nrows];

        // queries of this thread: tile queries tid*kQPT .. tid*kQPT+kQPT-1, so a
        // small tile fills the slots of its first warps and the other warps
        // skip the tests
        const bool warp_active = qs + (uint32_t)(tid & ~31) * kQPT < qe;
        float qx[kQPT], qy[kQPT];
        double2 qd[kQPT];
        uint32_t qk[kQPT], cnt[kQPT];
        unsigned long long cur[kQPT], rend[kQPT];
        bool wr[kQPT];
#pragma unroll
        for (int q = 0; q < kQPT; q++) {
            const uint32_t k = qs + (uint32_t)tid * kQPT + q;
            qk[q] = k;
            cnt[q] = 0;
            cur[q] = rend[q] = 0;
            wr[q] = false;
            if (k < qe) {
                const float2 loc = a.glocal[k];
                const int dcx = (int)(a.gkey[k] - tile_base);
                qx[q] = __fmaf_rn((float)dcx, wf, loc.x);
                qy[q] = loc.y;
                qd[q] = a.gxy[k];
                if (FILL) {
                    cur[q] = a.off[k] - a.off_base;
                    rend[q] = a.off[k + 1] - a.off_base;
                    // rows of points with deg >= row_deg_lim are not written
                    wr[q] = !a.row_deg_lim || a.deg[k] < a.row_deg_lim;
                }
            } else {
                qx[q] = qy[q] = __int_as_float(0x7fc00000);
                qd[q] = make_double2(__longlong_as_double(0x7ff8000000000000ll),
                                     __longlong_as_double(0x7ff8000000000000ll));
            }
        }

        for (uint32_t cb = 0; cb < C; cb += kChunk) {
            const uint32_t len = min((uint32_t)kChunk, C - cb);
            const uint32_t len32 = (len + 31u) & ~31u;
            for (uint32_t j = tid; j < len32; j += kTT) {
                uint32_t k = 0xffffffffu;
                int i = 0;
                if (j < len) {
                    k = tile_candidate(s_seg_start, s_seg_off, nrows, cb + j, &i);
                    if (!VDB_GUARD(a.st, k < a.n, 3, k)) k = 0xffffffffu;
                }
                if (k != 0xffffffffu) {
                    if (MIXED) {
                        const float2 loc = a.glocal[k];
                        const int dcx = (int)(a.gkey[k] - s_seg_base[i]);
                        s_rel[j] = make_float2(__fmaf_rn((float)dcx, wf, loc.x),
                                               __fadd_rn(loc.y, s_seg_dyw[i]));
                    }
                    s_xy[j] = a.gxy[k];
                    s_id[j] = k;
                } else {
                    // padding: NaN fails every comparison (also against thr = inf)
                    s_rel[j] = make_float2(__int_as_float(0x7fc00000), __int_as_float(0x7fc00000));
                    s_xy[j] = make_double2(__longlong_as_double(0x7ff8000000000000ll),
                                           __longlong_as_double(0x7ff8000000000000ll));
                    s_id[j] = 0;
                }
            }
            __syncthreads();

            for (uint32_t j0 = 0; warp_active && j0 < len; j0 += 32) {
                uint32_t m[kQPT], hm[kQPT];
#pragma unroll
                for (int q = 0; q < kQPT; q++) m[q] = hm[q] = 0u;
#pragma unroll
                for (int jj = 0; jj < 32; jj++) {
                    if (MIXED) {
                        const float2 c = s_rel[j0 + jj];
#pragma unroll
                        for (int q = 0; q < kQPT; q++) {
                            const float dx = __fsub_rn(qx[q], c.x);
                            const float dy = __fsub_rn(qy[q], c.y);
                            const float d2 = __fmaf_rn(dx, dx, __fmul_rn(dy, dy));
                            m[q] |= (d2 < lo) ? (1u << jj) : 0u;
                            hm[q] |= (d2 <= hi) ? (1u << jj) : 0u;
                        }
                    } else {
                        const double2 c = s_xy[j0 + jj];
#pragma unroll
                        for (int q = 0; q < kQPT; q++) {
                            const double dx = __dsub_rn(qd[q].x, c.x);
                            const double dy = __dsub_rn(qd[q].y, c.y);
                            const double d2 = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
                            m[q] |= (d2 <= tbox) ? (1u << jj) : 0u;
                            hm[q] |= (d2 <= thr) ? (1u << jj) : 0u;
                        }
                    }
                }
                // pairs in the band: exact FP64 predicate
                uint32_t amb[kQPT], asy[kQPT], any = 0u;
#pragma unroll
                for (int q = 0; q < kQPT; q++) {
                    amb[q] = hm[q] & ~m[q];
                    asy[q] = 0u;
                    any |= amb[q];
                }
                if (__any_sync(kFull, any != 0u)) {
#pragma unroll
                    for (int q = 0; q < kQPT; q++) {
                        while (amb[q]) {
                            const int jj = __ffs(amb[q]) - 1;
                            amb[q] &= amb[q] - 1u;
                            const uint32_t kq = s_id[j0 + jj];
                            const uint32_t r = exact_pair(qd[q], s_xy[j0 + jj], qk[q], kq, xb,
                                                          a.gbox);
                            my_retest++;
                            if (r & 1u) {
                                m[q] |= 1u << jj;
                                if (!(r & 2u)) asy[q] |= 1u << jj;
                            }
                            if (!FILL && (r == 1u || r == 2u) && qk[q] < kq) {
                                const uint32_t slot = atomicAdd(a.asym_n, 1u);
                                if (slot < a.asym_cap) {
                                    AsymPair ap;
                                    ap.a = qk[q];
                                    ap.b = kq;
                                    ap.dir = r;
                                    ap.pad = 0u;
                                    a.asym[slot] = ap;
                                } else {
                                    atomicOr(&a.st->flags, kStatAsymOverflow);
                                }
                            }
                        }
                    }
                }
                if (FILL) {
#pragma unroll
                    for (int q = 0; q < kQPT; q++) {
                        uint32_t act = __ballot_sync(kFull, m[q] != 0u && wr[q]);
                        while (act) {
                            const int src = __ffs(act) - 1;
                            act &= act - 1u;
                            const uint32_t mm = __shfl_sync(kFull, m[q], src);
                            const uint32_t am = __shfl_sync(kFull, asy[q], src);
                            const unsigned long long c0 = __shfl_sync(kFull, cur[q], src);
                            const unsigned long long ce = __shfl_sync(kFull, rend[q], src);
                            if ((mm >> lane) & 1u) {
                                const unsigned long long dst = c0 + __popc(mm & lt);
                                if (dst < ce) {
                                    const bool one_way = (am >> lane) & 1u;
                                    if (a.compact)  // position in its work unit's candidates
                                        reinterpret_cast<uint16_t*>(a.nbr)[dst] =
                                            (uint16_t)(((cb + j0 + (uint32_t)lane) &
                                                        (a.unit_words * 32u - 1u)) |
                                                       (one_way ? kAsymFlag16 : 0u));
                                    else
                                        a.nbr[dst] = s_id[j0 + lane] | (one_way ? kAsymFlag : 0u);
                                } else {
                                    atomicOr(&a.st->flags, kStatRowOverflow);
                                }
                            }
                            if (lane == src) cur[q] += __popc(mm);
                        }
                    }
                } else {
                    const unsigned long long wrow = bm0 + (unsigned long long)((cb + j0) >> 5) * Q;
#pragma unroll
                    for (int q = 0; q < kQPT; q++) {
                        cnt[q] += __popc(m[q]);
                        if (a.bitmap && qk[q] < qe) a.bitmap[wrow + (qk[q] - qs)] = m[q];
                    }
                }
            }
            __syncthreads();
        }
        if (!FILL) {
#pragma unroll
            for (int q = 0; q < kQPT; q++)
                if (qk[q] < qe) a.deg[qk[q]] = cnt[q];
        }
        __syncthreads();
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) my_retest += __shfl_down_sync(kFull, my_retest, d);
    if (lane == 0 && my_retest) atomicAdd(&a.st->retested, my_retest);
}

// Per tile (one warp per tile; lanes over rows): the bitmap size
// ceil(C/32) words per query and the number of work units
// ceil(ceil(C/32) / unit_words).  Tiles past the end write 0 so that scans
// over n entries give the offsets.
__global__ void tile_words_kernel(TableArgs a, uint32_t* words, uint32_t* units) {
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const EpsParams* __restrict__ ep = a.ep;
    const int rho = ep->rho, nrows = 2 * rho + 1;
    const uint32_t ntiles = *a.ntiles;
    for (uint64_t t = warp; t < a.n; t += nwarps) {
        uint64_t w = 0;
        uint32_t nu = 0;
        if (t < ntiles) {
            const uint32_t qs = a.tiles[t], qe = a.tiles[t + 1];
            const uint32_t key0 = a.gkey[qs];
            const uint32_t cy = key0 / a.g.ncx_pad;
            const uint32_t cx0 = (key0 - cy * a.g.ncx_pad) / a.g.G * a.g.G;
            uint32_t c = 0;
            for (int i = lane; i < nrows; i += 32) {
                uint32_t st, len, base;
                tile_row(a, ep, rho, cy, cx0, i, &st, &len, &base);
                c += len;
                if (a.trow_s) {
                    const unsigned long long k = t * (uint32_t)nrows + (uint32_t)i;
                    a.trow_s[k] = st;
                    a.trow_e[k] = st + len;
                }
            }
#pragma unroll
            for (int d = 16; d > 0; d >>= 1) c += __shfl_down_sync(kFull, c, d);
            const uint32_t tw = (c + 31u) >> 5;
            w = (uint64_t)tw * (qe - qs);
            nu = (tw + a.unit_words - 1) / a.unit_words;
        }
        if (lane == 0) {
            if (w > 0xffffffffull) {
                atomicOr(&a.st->flags, kStatBitmapTooLarge);
                w = 0;
            }
            words[t] = (uint32_t)w;
            units[t] = nu;
        }
    }
}

// ptile[k] = t for the points [tiles[t], tiles[t+1]) of every tile t.
__global__ void tile_owner_kernel(TableArgs a, uint32_t* __restrict__ ptile) {
    const uint32_t ntiles = *a.ntiles;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < ntiles;
         t += gridDim.x * blockDim.x) {
        const uint32_t qs = a.tiles[t], qe = min(a.tiles[t + 1], a.n);
        for (uint32_t k = qs; k < qe; k++) ptile[k] = t;
    }
}

__global__ void masked_degrees_kernel(const uint32_t* __restrict__ deg, uint32_t n, uint32_t lim,
                                      uint32_t* __restrict__ out) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) out[k] = deg[k] < lim ? deg[k] : 0u;
}

// unit_tile[u] = t for the units [tile_uoff[t], tile_uoff[t+1]) of tile t.
__global__ void unit_list_kernel(TableArgs a, uint32_t* unit_tile) {
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const uint32_t ntiles = *a.ntiles;
    for (uint64_t t = warp; t < ntiles; t += nwarps) {
        const uint32_t b = a.tile_uoff[t], e = a.tile_uoff[t + 1];
        for (uint32_t u = b + lane; u < e; u += 32) unit_tile[u] = (uint32_t)t;
    }
}

// splitmix64 finaliser (a published 64-bit mixer).
__device__ __forceinline__ unsigned long long mix64(unsigned long long x) {
    x ^= x >> 30;
    x *= 0xbf58476d1ce4e5b9ull;
    x ^= x >> 27;
    x *= 0x94d049bb133111ebull;
    x ^= x >> 31;
    return x;
}

// Hash of the rows [row_lo, row_hi) of a table (a warp per row): the sum over
// entries q of row p of mix64(p << 32 | q), plus a constant for entries
// flagged one-way, p and q input indices.
__global__ void table_hash_kernel(TableArgs a, const uint32_t* __restrict__ gorig) {
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const int nrows = 2 * a.ep->rho + 1;
    const uint16_t* const nb16 = reinterpret_cast<const uint16_t*>(a.nbr);
    unsigned long long acc = 0;
    for (uint64_t r = a.row_lo + warp; r < a.row_hi; r += nwarps) {
        const uint32_t k = (uint32_t)r;
        const unsigned long long s = a.off[k] - a.off_base, e = a.off[k + 1] - a.off_base;
        const unsigned long long p = (unsigned long long)gorig[k] << 32;
        auto add = [&](uint32_t q, bool one_way) {
            if (!VDB_GUARD(a.st, q < a.n, 17, q)) return;
            acc += mix64(p | gorig[q]) + (one_way ? 0x9e3779b97f4a7c15ull : 0ull);
        };
        if (a.compact) {
            walk_compact_row(nb16, s, e, k, a.ptile, a.tiles, a.tile_uoff, a.parts, a.trow_s,
                             a.trow_e, nrows, a.unit_words, (int)lane,
                             [&](uint32_t q, bool one_way, bool valid) {
                                 if (valid) add(q, one_way);
                             });
        } else {
            for (unsigned long long j = s + lane; j < e; j += 32) {
                const uint32_t ev = a.nbr[j];
                add(ev & kIdMask, (ev & kAsymFlag) != 0);
            }
        }
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) acc += __shfl_down_sync(kFull, acc, d);
    if (lane == 0 && acc) atomicAdd(&a.st->table_hash, acc);
}

// Flags the table entries accepted in one direction only (the count pass
// recorded them): b in row a when dir == 1, a in row b when dir == 2.  Rows are
// sorted by neighbour index.
__global__ void asym_flags_kernel(TableArgs a) {
    uint32_t na = *a.asym_n;
    if (na > a.asym_cap) na = a.asym_cap;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < na;
         i += gridDim.x * blockDim.x) {
        const AsymPair p = a.asym[i];
        const uint32_t row = p.dir == 1u ? p.a : p.b;
        const uint32_t target = p.dir == 1u ? p.b : p.a;
        if (a.row_hi && (row < a.row_lo || row >= a.row_hi)) continue;  // row not in this chunk
        if (a.row_deg_lim && a.deg[row] >= a.row_deg_lim) continue;     // row not written
        unsigned long long lo = a.off[row] - a.off_base, hi = a.off[row + 1] - a.off_base;
        const unsigned long long end = hi;
        if (a.compact) {
            // the target's position in the candidate list of the row's tile,
            // then its unit and the unit's share of the row
            const uint32_t t = a.ptile[row];
            const uint32_t slot = row - a.tiles[t];
            const uint32_t nr = 2u * (uint32_t)a.ep->rho + 1u;
            uint32_t before = 0, g = 0xffffffffu;
            for (uint32_t i = 0; i < nr; i++) {
                const unsigned long long k = (unsigned long long)t * nr + i;
                const uint32_t s0 = a.trow_s[k], e0 = a.trow_e[k];
                if (target >= s0 && target < e0) g = before + (target - s0);
                before += e0 - s0;
            }
            const uint32_t u0 = a.tile_uoff[t], nu = a.tile_uoff[t + 1] - u0;
            const uint32_t c = g / (a.unit_words * 32u), pos = g % (a.unit_words * 32u);
            if (!VDB_GUARD(a.st, g != 0xffffffffu && c < nu && slot < kUnitQ, 5, target)) continue;
            for (uint32_t u = u0; u < u0 + c; u++) lo += a.parts[(unsigned long long)u * kUnitQ + slot];
            hi = lo + a.parts[(unsigned long long)(u0 + c) * kUnitQ + slot];
            if (hi > end) hi = end;
            if (lo > hi) lo = hi;
            const unsigned long long seg_end = hi;
            uint16_t* const nb = reinterpret_cast<uint16_t*>(a.nbr);
            while (lo < hi) {
                const unsigned long long mid = (lo + hi) >> 1;
                if ((uint32_t)(nb[mid] & kPosMask16) < pos) lo = mid + 1;
                else hi = mid;
            }
            if (VDB_GUARD(a.st, lo < seg_end && (uint32_t)(nb[lo] & kPosMask16) == pos,
                          5, target))
                nb[lo] |= kAsymFlag16;
            continue;
        }
        while (lo < hi) {
            const unsigned long long mid = (lo + hi) >> 1;
            if ((a.nbr[mid] & kIdMask) < target) lo = mid + 1;
            else hi = mid;
        }
        if (VDB_GUARD(a.st, lo < end && (a.nbr[lo] & kIdMask) == target, 5, target))
            a.nbr[lo] |= kAsymFlag;
    }
}

}  // namespace
int table_block_threads() { return kTT; }
// tiles hold at most one warp tile of queries (the count and table passes
// give each warp one tile; the fill pass's blocks accept up to kTT * kQPT)
int table_tile_queries() {
    static_assert(kWQ <= kTT * kQPT, "fill blocks must hold a whole tile");
    return kWQ;
}

void launch_count(const TableArgs& a, int nblocks, cudaStream_t s) {
    VDB_COUNT_LAUNCH();
    if (a.mixed)
        count_kernel<true><<<nblocks, kWPB * 32, 0, s>>>(a);
    else
        count_kernel<false><<<nblocks, kWPB * 32, 0, s>>>(a);
}

void launch_fill(const TableArgs& a, int nblocks, cudaStream_t s) {
    VDB_COUNT_LAUNCH();
    if (a.mixed)
        table_kernel<true, true><<<nblocks, kTT, 0, s>>>(a);
    else
        table_kernel<false, true><<<nblocks, kTT, 0, s>>>(a);
}

void launch_tile_words(const TableArgs& a, uint32_t* words, uint32_t* units, int nblocks,
                       cudaStream_t s) {
    VDB_COUNT_LAUNCH();
    tile_words_kernel<<<nblocks, kTT, 0, s>>>(a, words, units);
}

void launch_unit_list(const TableArgs& a, uint32_t* unit_tile, int nblocks, cudaStream_t s) {
    VDB_COUNT_LAUNCH();
    unit_list_kernel<<<nblocks, kTT, 0, s>>>(a, unit_tile);
}

void launch_masked_degrees(const uint32_t* deg, uint32_t n, uint32_t lim, uint32_t* out,
                           cudaStream_t s) {
    if (!n) return;
    VDB_COUNT_LAUNCH();
    masked_degrees_kernel<<<(n + kTT - 1) / kTT, kTT, 0, s>>>(deg, n, lim, out);
}

void launch_expand(const TableArgs& a, int nblocks, cudaStream_t s) {
    VDB_COUNT_LAUNCH();
    if (a.compact)
        expand16_kernel<<<nblocks, kXPB * 32, 0, s>>>(a);
    else
        expand_kernel<uint32_t><<<nblocks, kXPB * 32, 0, s>>>(a);
}

void launch_tile_owner(const TableArgs& a, uint32_t* ptile, int nblocks, cudaStream_t s) {
    VDB_COUNT_LAUNCH();
    tile_owner_kernel<<<nblocks, kTT, 0, s>>>(a, ptile);
}

void launch_table_hash(const TableArgs& a, const uint32_t* gorig, int nblocks, cudaStream_t s) {
    if (a.row_hi <= a.row_lo) return;
    VDB_COUNT_LAUNCH();
    table_hash_kernel<<<nblocks, kTT, 0, s>>>(a, gorig);
}

void launch_asym_flags(const TableArgs& a, cudaStream_t s) {
    VDB_COUNT_LAUNCH();
    asym_flags_kernel<<<64, kTT, 0, s>>>(a);
}

int table_blocks_per_sm(bool fill, bool mixed) {
    int nb = 0;
    if (fill) {
        if (mixed)
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, table_kernel<true, true>, kTT, 0);
        else
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, table_kernel<false, true>, kTT, 0);
    } else {
        if (mixed)
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, count_kernel<true>, kWPB * 32, 0);
        else
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, count_kernel<false>, kWPB * 32, 0);
    }
    return nb > 0 ? nb : 1;
}

int expand_blocks_per_sm(bool compact) {
    int nb = 0;
    if (compact)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, expand16_kernel, kXPB * 32, 0);
    else
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, expand_kernel<uint32_t>, kXPB * 32, 0);
    return nb > 0 ? nb : 1;
}

}  // namespace vdb
