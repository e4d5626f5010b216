// Epsilon-neighbourhood kernels: the count pass (|N_eps(p)| for every point,
// plus a bitmap of every candidate test) and the table pass (CSR neighbour
// table written from that bitmap).
//
// Each persistent block takes query tiles from a global counter.  A tile is up
// to kTileQ consecutive cell-ordered points of one group of G cells of one grid
// row; its candidates are the points of the cells within reach in the rows
// cy-rho..cy+rho, which are 2*rho+1 contiguous ranges of the cell-ordered
// arrays.  Candidates are staged through shared memory in chunks (coalesced
// float2 + key loads, shifted to the tile's cell origin with exact FP32
// offsets) and every thread tests its kQPT queries against each staged
// candidate (lane = query, candidate = shared-memory broadcast).
//
// The neighbour predicate is the reference's (src/DBScan.cpp:665-702 with the
// R-tree candidate rule of src/RTree.h:1613-1625):
//   q in N(p)  <=>  sqrt(fl(fl(dx*dx)+fl(dy*dy))) <= eps     (dx = fl(px-qx), FP64)
//                   and q's multiple-point box overlaps [p-eps, p+eps]^2.
// sqrt is monotone and correctly rounded, so the first part is d2 <= thr with
// thr the largest double whose square root is <= eps.  The box part can only
// fail when d2 > tbox (a pair that deep inside the circle lies inside the query
// box).  Mixed precision: the FP32 squared distance on cell-local coordinates
// classifies a pair as in (d2 < lo32), out (d2 > hi32) or ambiguous; only
// ambiguous pairs are re-tested with the FP64 predicate above.  The band
// [lo32, hi32] is derived from the FP32 error bound on the host.
//
// Table pass: the count pass stores, per tile, one 32-bit word per query and
// per 32 consecutive candidates (bit j: candidate j is a neighbour), laid out
// [word][query] so that a warp's 32 queries store 128 contiguous bytes.  The
// table pass turns each word into neighbour ids with one coalesced store
// (lane = bit), in candidate order, so every row comes out sorted by
// neighbour index.  Entries accepted in one direction only are flagged
// afterwards from the asymmetric-pair list.  When the bitmap does not fit in
// device memory, the fill variant of the tile kernel re-tests the candidates
// and writes the table directly.
#include "vdb_internal.cuh"

namespace vdb {

namespace {

constexpr int kTT = 256;              // threads per block
constexpr int kQPT = 2;               // queries per thread
constexpr int kTileQ = kTT * kQPT;    // queries per tile (must match the host's tile size)
constexpr int kChunk = 1024;          // candidates staged per round
constexpr int kXW = 16;               // bitmap words staged per round of the table pass
constexpr unsigned kFull = 0xffffffffu;

// Row i (offset dy = i - rho) of the tile whose group starts at cell (cy, cx0):
// the candidate range [*st, *st + *len) and the key of the group's first cell
// in that row (so that key - base is the candidate's cell offset in x).
__device__ __forceinline__ void tile_row(const TableArgs& a, const EpsParams* __restrict__ ep,
                                         int rho, uint32_t cy, uint32_t cx0, int i,
                                         uint32_t* st, uint32_t* len, uint32_t* base) {
    const int ry = (int)cy + i - rho;
    *st = 0;
    *len = 0;
    *base = 0;
    if (ry < 0 || ry >= (int)a.g.ncy) return;
    const int reach = ep->reach[i];
    const int lo_c = max((int)cx0 - reach, 0);
    const int hi_c = min((int)(cx0 + a.g.G - 1) + reach, (int)a.g.ncx - 1);
    const uint32_t rb = (uint32_t)ry * a.g.ncx_pad;
    const uint32_t s = a.cell_start[rb + lo_c];
    const uint32_t e = a.cell_start[rb + hi_c + 1];
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
    const float lo = ep->lo32, hi = ep->hi32;
    const int rho = ep->rho;
    const int nrows = 2 * rho + 1;
    const float wf = (float)a.g.w;
    const uint32_t tile_end = a.tile_end != 0xffffffffu ? a.tile_end : *a.ntiles;
    const uint32_t ncx_pad = a.g.ncx_pad, G = a.g.G;
    unsigned long long my_retest = 0;

    for (;;) {
        if (tid == 0) s_tile = atomicAdd(a.tile_counter, 1u);
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
#pragma unroll
        for (int q = 0; q < kQPT; q++) {
            const uint32_t k = qs + (uint32_t)tid * kQPT + q;
            qk[q] = k;
            cnt[q] = 0;
            cur[q] = rend[q] = 0;
            if (k < qe) {
                const float2 loc = a.glocal[k];
                const int dcx = (int)(a.gkey[k] - tile_base);
                qx[q] = __fmaf_rn((float)dcx, wf, loc.x);
                qy[q] = loc.y;
                qd[q] = a.gxy[k];
                if (FILL) {
                    cur[q] = a.off[k] - a.off_base;
                    rend[q] = a.off[k + 1] - a.off_base;
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
                            const uint32_t r = exact_pair(qd[q], s_xy[j0 + jj], qk[q], kq, eps,
                                                          thr, tbox, a.gpos, a.mpb, a.mbb);
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
                        uint32_t act = __ballot_sync(kFull, m[q] != 0u);
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
                                    a.nbr[dst] = s_id[j0 + lane] |
                                                 (((am >> lane) & 1u) ? kAsymFlag : 0u);
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

// Bitmap words of every tile: ceil(C/32) words per query (one warp per tile;
// lanes over rows).  Tiles past the end write 0 so that a scan over n entries
// gives the offsets.
__global__ void tile_words_kernel(TableArgs a, uint32_t* words) {
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const EpsParams* __restrict__ ep = a.ep;
    const int rho = ep->rho, nrows = 2 * rho + 1;
    const uint32_t ntiles = *a.ntiles;
    for (uint64_t t = warp; t < a.n; t += nwarps) {
        uint64_t w = 0;
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
            }
#pragma unroll
            for (int d = 16; d > 0; d >>= 1) c += __shfl_down_sync(kFull, c, d);
            w = (uint64_t)((c + 31u) >> 5) * (qe - qs);
        }
        if (lane == 0) {
            if (w > 0xffffffffull) {
                atomicOr(&a.st->flags, kStatBitmapTooLarge);
                w = 0;
            }
            words[t] = (uint32_t)w;
        }
    }
}

// Table pass: neighbour ids from the count pass's bitmap.  Per tile, rounds of
// kXW words: the round's candidate ids and bitmap words are staged in shared
// memory, then each warp expands its queries' words (lane = bit, one
// coalesced store per non-zero word).
__global__ void __launch_bounds__(kTT) expand_kernel(TableArgs a) {
    __shared__ uint32_t s_bm[kXW][kTileQ + 1];
    __shared__ uint32_t s_id[kXW * 32];
    __shared__ unsigned long long s_cur[kTileQ];
    __shared__ uint32_t s_seg_start[kMaxRows];
    __shared__ uint32_t s_seg_off[kMaxRows + 1];
    __shared__ uint32_t s_tile;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t lt = (1u << lane) - 1u;
    const EpsParams* __restrict__ ep = a.ep;
    const int rho = ep->rho;
    const int nrows = 2 * rho + 1;
    const uint32_t tile_end = a.tile_end != 0xffffffffu ? a.tile_end : *a.ntiles;
    const uint32_t ncx_pad = a.g.ncx_pad, G = a.g.G;

    for (;;) {
        if (tid == 0) s_tile = atomicAdd(a.tile_counter, 1u);
        __syncthreads();
        const uint32_t t = s_tile;
        if (t >= tile_end) break;
        const uint32_t qs = a.tiles[t], qe = a.tiles[t + 1];
        if (!(qs < qe && qe <= a.n)) {
            if (tid == 0) guard_fail(a.st, 4, ((unsigned long long)qs << 32) | qe);
            __syncthreads();
            continue;
        }
        const uint32_t Q = qe - qs;
        const uint32_t key0 = a.gkey[qs];
        const uint32_t cy = key0 / ncx_pad;
        const uint32_t cx0 = (key0 - cy * ncx_pad) / G * G;
        if (tid < nrows) {
            uint32_t st, len, base;
            tile_row(a, ep, rho, cy, cx0, tid, &st, &len, &base);
            s_seg_start[tid] = st;
            s_seg_off[tid + 1] = len;
        }
        for (uint32_t q = tid; q < Q; q += kTT) s_cur[q] = a.off[qs + q] - a.off_base;
        __syncthreads();
        if (tid == 0) {
            uint32_t acc = 0;
            s_seg_off[0] = 0;
            for (int i = 0; i < nrows; i++) {
                acc += s_seg_off[i + 1];
                s_seg_off[i + 1] = acc;
            }
        }
        __syncthreads();
        const uint32_t C = s_seg_off[nrows];
        const uint32_t words = (C + 31u) >> 5;
        const unsigned long long bm0 = a.tile_boff[t];
        for (uint32_t w0 = 0; w0 < words; w0 += kXW) {
            const uint32_t nw = min((uint32_t)kXW, words - w0);
            for (uint32_t j = tid; j < nw * 32u; j += kTT) {
                const uint32_t g = w0 * 32u + j;
                uint32_t id = 0;
                if (g < C) {
                    int i;
                    id = tile_candidate(s_seg_start, s_seg_off, nrows, g, &i);
                }
                s_id[j] = id;
            }
            for (uint32_t wi = 0; wi < nw; wi++) {
                const unsigned long long src = bm0 + (unsigned long long)(w0 + wi) * Q;
                for (uint32_t q = tid; q < Q; q += kTT) s_bm[wi][q] = a.bitmap[src + q];
            }
            __syncthreads();
            for (uint32_t q = warp; q < Q; q += kTT / 32) {
                unsigned long long cur = s_cur[q];
                for (uint32_t wi = 0; wi < nw; wi++) {
                    const uint32_t word = s_bm[wi][q];
                    if (!word) continue;
                    if ((word >> lane) & 1u) a.nbr[cur + __popc(word & lt)] = s_id[wi * 32u + lane];
                    cur += __popc(word);
                }
                if (lane == 0) s_cur[q] = cur;
            }
            __syncthreads();
        }
    }
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
        unsigned long long lo = a.off[row] - a.off_base, hi = a.off[row + 1] - a.off_base;
        while (lo < hi) {
            const unsigned long long mid = (lo + hi) >> 1;
            if ((a.nbr[mid] & kIdMask) < target) lo = mid + 1;
            else hi = mid;
        }
        const unsigned long long end = a.off[row + 1] - a.off_base;
        if (VDB_GUARD(a.st, lo < end && (a.nbr[lo] & kIdMask) == target, 5, target))
            a.nbr[lo] |= kAsymFlag;
    }
}

}  // namespace

int table_block_threads() { return kTT; }
int table_tile_queries() { return kTileQ; }

template <bool FILL>
static void launch_table(const TableArgs& a, int nblocks, cudaStream_t s) {
    VDB_COUNT_LAUNCH();
    if (a.mixed)
        table_kernel<true, FILL><<<nblocks, kTT, 0, s>>>(a);
    else
        table_kernel<false, FILL><<<nblocks, kTT, 0, s>>>(a);
}

void launch_count(const TableArgs& a, int nblocks, cudaStream_t s) {
    launch_table<false>(a, nblocks, s);
}

void launch_fill(const TableArgs& a, int nblocks, cudaStream_t s) {
    launch_table<true>(a, nblocks, s);
}

void launch_tile_words(const TableArgs& a, uint32_t* words, int nblocks, cudaStream_t s) {
    VDB_COUNT_LAUNCH();
    tile_words_kernel<<<nblocks, kTT, 0, s>>>(a, words);
}

void launch_expand(const TableArgs& a, int nblocks, cudaStream_t s) {
    VDB_COUNT_LAUNCH();
    expand_kernel<<<nblocks, kTT, 0, s>>>(a);
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
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, table_kernel<true, false>, kTT, 0);
        else
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, table_kernel<false, false>, kTT,
                                                          0);
    }
    return nb > 0 ? nb : 1;
}

int expand_blocks_per_sm() {
    int nb = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, expand_kernel, kTT, 0);
    return nb > 0 ? nb : 1;
}

}  // namespace vdb
