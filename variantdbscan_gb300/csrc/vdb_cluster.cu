// Cluster labelling from the neighbour table, reproducing the labels of the
// reference's sequential expansion (DBScan::algDBScanParallel,
// src/DBScan.cpp:523-609) without running it sequentially.
//
// With pos(p) the reference's visit position (binDataset order):
//   core(p)   <=> |N(p)| >= minpts (N(p) contains p);
//   components of the core points under the symmetric core-core edges are
//   found by lock-free union-find (link the larger root under the smaller);
//   seed(C) = min pos over the cores of C.  The reference's main loop reaches
//   the cores of C first at seed(C) and its expansion then visits every point
//   reachable from C, so a cluster starts at seed(C) and numbers follow seeds.
//   A core-core edge accepted in one direction only (the R-tree box rule,
//   see vdb_table.cu) lets the cluster started by one component absorb
//   another; resolve_kernel replays that on the component graph in seed order.
//   A non-core point p joins the cluster with the earliest start among the
//   cores u with p in N(u), if that start precedes pos(p); otherwise the main
//   loop visited p first and labelled it noise (src/DBScan.cpp:552-554,
//   573-577).
#include <algorithm>

#include "vdb_internal.cuh"

namespace vdb {

namespace {

constexpr int kThreads = 256;
constexpr uint32_t kNone = 0xffffffffu;
constexpr unsigned kFull = 0xffffffffu;

inline unsigned nblk(uint64_t n) { return (unsigned)((n + kThreads - 1) / kThreads); }

__device__ __forceinline__ bool is_core(uint32_t d, unsigned long long minpts) {
    return (unsigned long long)d >= minpts;
}

// Root of x.  Ends after at most x steps: every parent is at most its child
// (unions link the larger root under the smaller one, path halving stores an
// ancestor), so the chain strictly decreases until it meets a root.
__device__ __forceinline__ uint32_t uf_find(uint32_t* parent, uint32_t x) {
    volatile uint32_t* vp = parent;
    uint32_t p = vp[x];
    while (p != x) {
        const uint32_t gp = vp[p];
        if (gp != p) vp[x] = gp;  // path halving; parents only decrease
        x = p;
        p = gp;
    }
    return x;
}

__device__ __forceinline__ void uf_union(uint32_t* parent, uint32_t a, uint32_t b,
                                         DeviceStatus* st) {
    for (int it = 0; it < (1 << 24); it++) {
        a = uf_find(parent, a);
        b = uf_find(parent, b);
        if (a == b) return;
        if (a > b) {
            const uint32_t t = a;
            a = b;
            b = t;
        }
        const uint32_t old = atomicCAS(&parent[b], b, a);
        if (old == b) return;
        b = old;
    }
    atomicOr(&st->flags, kStatUnionStall);
}

__global__ void uf_init_kernel(uint32_t n, int fresh, uint32_t* parent, uint32_t* seed,
                               uint32_t* best, uint32_t* cstart, uint32_t* pos_flag) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    if (fresh) parent[k] = k;
    seed[k] = kNone;
    best[k] = kNone;
    cstart[k] = k;
    pos_flag[k] = 0u;
}

// One warp per row.  From scratch, an edge (k, v) of two cores is united from
// its smaller end; when the parent array already holds the components of a
// larger minpts, only rows of the new cores are read and all their core
// neighbours are united.
__global__ void uf_union_kernel(ClusterArgs a) {
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const bool reuse = a.minpts_prev != ~0ull;
    for (uint64_t r = a.row_lo + warp; r < a.row_hi; r += nwarps) {
        const uint32_t k = (uint32_t)r;
        const uint32_t dk = a.deg[k];
        if (!is_core(dk, a.minpts)) continue;
        if (reuse && is_core(dk, a.minpts_prev)) continue;
        const unsigned long long s = a.off[k] - a.off_base, e = a.off[k + 1] - a.off_base;
        auto edge = [&](uint32_t v) {
            if (!VDB_GUARD(a.st, v < a.n, 10, v)) return;
            if (v == k || (!reuse && v < k)) return;
            if (!is_core(a.deg[v], a.minpts)) return;
            uf_union(a.parent, k, v, a.st);
        };
        if (a.compact) {
            walk_compact_row(reinterpret_cast<const uint16_t*>(a.nbr), s, e, k, a.ptile, a.tiles,
                             a.tile_uoff, a.parts, a.trow_s, a.trow_e, 2 * a.ep->rho + 1,
                             a.unit_words, (int)lane, [&](uint32_t v, bool one_way, bool valid) {
                                 if (valid && !one_way) edge(v);
                             });
        } else {
            for (unsigned long long j = s + lane; j < e; j += 32) {
                const uint32_t ev = a.nbr[j];
                if (!(ev & kAsymFlag)) edge(ev & kIdMask);
            }
        }
    }
}

// Read-only find: while the flatten pass stores roots, a path-halving write of
// another thread could replace a stored root by an intermediate ancestor.
__device__ __forceinline__ uint32_t uf_find_ro(const uint32_t* parent, uint32_t x) {
    const volatile uint32_t* vp = parent;
    uint32_t p = vp[x];
    while (p != x) {
        x = p;
        p = vp[x];
    }
    return x;
}

// Cell union, step 1.  With cells of width <= eps/sqrt(2), every two points
// of a cell are neighbours in both directions, so the cell's cores form a
// clique: all of them are linked to the cell's first core (the smallest index,
// so parents still only decrease).  Point-parallel: crep[c] = first core of
// cell c (one atomic per cell and warp), then every other core links to it.
// The cell of point k is cscan[k + 1] - 1 (cscan: exclusive scan of the
// cell-start flags).
__global__ void cell_rep_min_kernel(ClusterArgs a) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    const bool core = k < a.n && is_core(a.deg[k], a.minpts);
    const uint32_t c = core ? a.cscan[k + 1] - 1u : kNone;
    const uint32_t act = __ballot_sync(kFull, core);
    if (!core) return;
    const uint32_t same = __match_any_sync(act, c);
    // lanes are in point order: the lowest lane of a cell holds its first core
    if ((threadIdx.x & 31) == (uint32_t)(__ffs(same) - 1) && VDB_GUARD(a.st, c < a.n, 15, c))
        atomicMin(&a.crep[c], k);
}

// From scratch every other core of the cell takes the first core as parent
// (rep <= k, so parents still only decrease).  When parent holds the
// components of a larger minpts (minpts_prev), a core that is new at this
// minpts is still a root of its own and is linked the same way; the cores
// that were already cores form one component, which is united with the first
// core only when that first core is new.
__global__ void cell_rep_link_kernel(ClusterArgs a) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= a.n || !is_core(a.deg[k], a.minpts)) return;
    const uint32_t c = a.cscan[k + 1] - 1u;
    if (!VDB_GUARD(a.st, c < a.n, 16, c)) return;
    const uint32_t rep = a.crep[c];
    if (rep == k) return;
    if (a.minpts_prev == ~0ull || !is_core(a.deg[k], a.minpts_prev))
        a.parent[k] = rep;
    else if (!is_core(a.deg[rep], a.minpts_prev))
        uf_union(a.parent, k, rep, a.st);
}

// Cell union, step 2 (one warp per cell A with cores): for every cell B within
// reach with a larger key that also has cores and is not yet in A's
// component, look for one core-core pair (a, b) accepted in both directions
// and unite the two cells on the first one.  One edge per connected cell pair
// replaces the union of every edge.  The lanes first screen up to 32
// neighbour cells at once (range, cores, roots); then, for each cell still to
// test, lanes hold A's cores and B's points are broadcast; the test is the
// table kernels' (FP32 on cell-relative coordinates, exact FP64 predicate
// inside the error band).
__global__ void cell_pairs_kernel(ClusterArgs a) {
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const uint32_t ncl = *a.ncl;
    const EpsParams* __restrict__ ep = a.ep;
    const int R = ep->rho;
    const bool mixed = ep->mixed != 0;
    const float lo = ep->lo32, hi = ep->hi32;
    const double eps = ep->eps, thr = ep->thr, tbox = ep->tbox;
    const ExactBounds xb = exact_bounds(eps, thr, tbox);
    const float wf = (float)a.g.w;
    const uint32_t ncx_pad = a.g.ncx_pad;
    const float fnan = __int_as_float(0x7fc00000);
    const float near2 = (float)(eps * eps * (1.0 + 0x1p-8));
    // neighbours of the half neighbourhood: row dy = 0 to the right, rows
    // dy = 1..R across their reach
    int nnb = 0;
    for (int dy = 0; dy <= R; dy++) nnb += dy == 0 ? ep->reach[R] : 2 * ep->reach[dy + R] + 1;
    uint32_t skipped = 0;  // lane 0: cell pairs of different components at a larger epsilon
    for (uint64_t c = warp; c < ncl; c += nwarps) {
        const uint32_t repA = a.crep[c];
        if (repA == kNone) continue;
        const uint32_t compA = a.comp_prev ? a.comp_prev[a.gpos[repA]] : kNone;
        const uint32_t sA = a.clist[c], eA = a.clist[c + 1];
        const uint32_t keyA = a.gkey[sA];
        const int cy = (int)(keyA / ncx_pad), cx = (int)(keyA - (uint32_t)cy * ncx_pad);
        // A's first 32 points, kept for every neighbour cell
        const bool va0 = sA + lane < eA && is_core(a.deg[sA + lane], a.minpts);
        float2 pa0 = make_float2(fnan, fnan);
        double2 Pa0 = make_double2(0.0, 0.0);
        if (va0) {
            pa0 = a.glocal[sA + lane];
            Pa0 = a.gxy[sA + lane];
        }
        for (int base = 0; base < nnb; base += 32) {
            // lane -> neighbour (dy, dx) number base + lane
            int my_dy = 0, my_dx = 0;
            bool valid = false;
            {
                int idx = base + (int)lane, acc = 0;
                for (int dy = 0; dy <= R && !valid; dy++) {
                    const int reach = ep->reach[dy + R];
                    const int cnt = dy == 0 ? reach : 2 * reach + 1;
                    if (idx < acc + cnt) {
                        my_dy = dy;
                        my_dx = (dy == 0 ? 1 : -reach) + (idx - acc);
                        valid = true;
                    }
                    acc += cnt;
                }
            }
            const int ry = cy + my_dy, rx = cx + my_dx;
            uint32_t sB = 0, eB = 0, repB = kNone;
            bool need = false;
            if (valid && ry < (int)a.g.ncy && rx >= 0 && rx < (int)a.g.ncx) {
                cell_row_range(a.g, a.cell_start, a.crow, a.ccx, a.clist, (uint32_t)ry,
                               (uint32_t)rx, (uint32_t)rx, &sB, &eB);
                if (sB < eB) {
                    repB = a.crep[a.cscan[sB]];
                    need = repB != kNone && uf_find(a.parent, repA) != uf_find(a.parent, repB);
                    // cores in different components at the larger epsilon are
                    // not connected at this one (its components refine those)
                    if (need && a.comp_prev && a.comp_prev[a.gpos[repB]] != compA) need = false;
                }
            }
            if (a.comp_prev) {
                const bool skip = valid && repB != kNone && !need && sB < eB &&
                                  a.comp_prev[a.gpos[repB]] != compA;
                skipped += __popc(__ballot_sync(kFull, skip));
            }
            // nearest cells first (their pairs are found soonest, and the unions
            // they make often connect the farther cells already): squared gap
            // between the cells in cell widths, then lane
            const int gx = max(abs(my_dx) - 1, 0), gy = max(my_dy - 1, 0);
            const uint32_t order = ((uint32_t)(gx * gx + gy * gy) << 5) | lane;
            for (uint32_t todo = __ballot_sync(kFull, need); todo;) {
                const uint32_t pick = __reduce_min_sync(kFull, (todo >> lane) & 1u ? order : 0xffffffffu);
                const int src = (int)(pick & 31u);
                todo &= ~(1u << src);
                const uint32_t sBb = __shfl_sync(kFull, sB, src), eBb = __shfl_sync(kFull, eB, src);
                const int dx = __shfl_sync(kFull, my_dx, src), dy = __shfl_sync(kFull, my_dy, src);
                // unions made since the screen may have joined the two cells
                const uint32_t repBb = __shfl_sync(kFull, repB, src);
                if (uf_find(a.parent, repA) == uf_find(a.parent, repBb)) continue;
                const float dyw = __fmul_rn((float)dy, wf);
                const float dxw = __fmul_rn((float)dx, wf);
                bool found = false;
                for (uint32_t b = sA; b < eA && !found; b += 32) {
                    const uint32_t ka = b + lane;
                    bool va = va0;
                    float2 pa = pa0;
                    double2 Pa = Pa0;
                    if (b != sA) {  // cells of more than 32 points: the next 32
                        va = ka < eA && is_core(a.deg[ka], a.minpts);
                        pa = make_float2(fnan, fnan);
                        if (va) {
                            pa = a.glocal[ka];
                            Pa = a.gxy[ka];
                        }
                    }
                    // only points within eps of the other cell's square can pair
                    // (cell-relative FP32 coordinates, eps^2 widened by 2^-8)
                    if (mixed && va) {
                        const float ex = fmaxf(fmaxf(dxw - pa.x, pa.x - (dxw + wf)), 0.0f);
                        const float ey = fmaxf(fmaxf(dyw - pa.y, pa.y - (dyw + wf)), 0.0f);
                        va = __fmaf_rn(ex, ex, ey * ey) <= near2;
                    }
                    if (!__any_sync(kFull, va)) continue;
                    // B's points 32 at a time: one coalesced load of their
                    // core flags and coordinates, then broadcast core by core
                    for (uint32_t kb0 = sBb; kb0 < eBb && !found; kb0 += 32) {
                        const uint32_t kbl = kb0 + lane;
                        bool vb = kbl < eBb && is_core(a.deg[kbl], a.minpts);
                        float2 lbl = make_float2(fnan, fnan);
                        if (vb && mixed) {
                            lbl = a.glocal[kbl];
                            const float bx = __fmaf_rn((float)dx, wf, lbl.x);
                            const float by = __fadd_rn(lbl.y, dyw);
                            const float ex = fmaxf(fmaxf(-bx, bx - wf), 0.0f);
                            const float ey = fmaxf(fmaxf(-by, by - wf), 0.0f);
                            vb = __fmaf_rn(ex, ex, ey * ey) <= near2;
                        }
                        for (uint32_t cm = __ballot_sync(kFull, vb); cm; cm &= cm - 1u) {
                            const int t = __ffs(cm) - 1;
                            const uint32_t kb = kb0 + (uint32_t)t;
                            const float lbx = __shfl_sync(kFull, lbl.x, t);
                            const float lby = __shfl_sync(kFull, lbl.y, t);
                            bool in = false;
                            if (va) {
                                uint32_t cls;  // 0 out, 1 in (both directions), 2 band
                                double2 Qb = make_double2(0.0, 0.0);  // FP64 tests only
                                if (mixed) {
                                    const float bx = __fmaf_rn((float)dx, wf, lbx);
                                    const float by = __fadd_rn(lby, dyw);
                                    const float ddx = __fsub_rn(pa.x, bx), ddy = __fsub_rn(pa.y, by);
                                    const float d2 = __fmaf_rn(ddx, ddx, __fmul_rn(ddy, ddy));
                                    cls = d2 < lo ? 1u : (d2 <= hi ? 2u : 0u);
                                } else {
                                    Qb = a.gxy[kb];
                                    const double ddx = __dsub_rn(Pa.x, Qb.x), ddy = __dsub_rn(Pa.y, Qb.y);
                                    const double d2 = __dadd_rn(__dmul_rn(ddx, ddx), __dmul_rn(ddy, ddy));
                                    cls = d2 <= tbox ? 1u : (d2 <= thr ? 2u : 0u);
                                }
                                if (cls == 2u) {
                                    if (mixed) Qb = a.gxy[kb];
                                    cls = exact_pair(Pa, Qb, ka, kb, xb, a.gbox) == 3u
                                              ? 1u : 0u;
                                }
                                in = cls == 1u;
                            }
                            const uint32_t hit = __ballot_sync(kFull, in);
                            if (hit) {
                                const uint32_t u = __shfl_sync(kFull, ka, __ffs(hit) - 1);
                                if (lane == 0) uf_union(a.parent, u, kb, a.st);
                                found = true;
                                break;
                            }
                        }
                    }
                }
            }
        }
    }
    if (lane == 0 && skipped) atomicAdd(&a.st->reuse_skips, (unsigned long long)skipped);
}

__global__ void save_components_kernel(ClusterArgs a, uint32_t* __restrict__ comp) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= a.n) return;
    const uint32_t p = a.gpos[k];
    if (!VDB_GUARD(a.st, p < a.n, 18, p)) return;
    comp[p] = is_core(a.deg[k], a.minpts) ? a.seed[a.parent[k]] : kNone;
}

__global__ void uf_flatten_kernel(ClusterArgs a) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= a.n || !is_core(a.deg[k], a.minpts)) return;
    const uint32_t r = uf_find_ro(a.parent, k);
    a.parent[k] = r;
    // cell-ordered neighbours mostly share a root: one atomic per root and warp
    const uint32_t same = __match_any_sync(__activemask(), r);
    const uint32_t mn = __reduce_min_sync(same, a.gpos[k]);
    if ((threadIdx.x & 31) == (uint32_t)(__ffs(same) - 1)) atomicMin(&a.seed[r], mn);
}

// Directed core-core edges between different components (single thread; the
// list is empty unless the box rule broke the symmetry of a core pair).
__global__ void resolve_kernel(ClusterArgs a, uint32_t* ws, uint32_t cap) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    uint32_t na = *a.asym_count;
    if (na > a.asym_cap) na = a.asym_cap;
    uint32_t* efrom = ws;
    uint32_t* eto = ws + cap;
    uint32_t* nodes = ws + 2 * cap;
    uint32_t* stack = ws + 4 * cap;  // 2*cap entries
    uint32_t ne = 0;
    for (uint32_t i = 0; i < na; i++) {
        const AsymPair p = a.asym[i];
        if (!is_core(a.deg[p.a], a.minpts) || !is_core(a.deg[p.b], a.minpts)) continue;
        const uint32_t ra = a.parent[p.a], rb = a.parent[p.b];
        if (ra == rb) continue;
        if (ne >= cap) {
            atomicOr(&a.st->flags, kStatResolveOverflow);
            return;
        }
        if (p.dir == 1u) {  // b in N(a) only: a's expansion reaches b
            efrom[ne] = ra;
            eto[ne] = rb;
        } else {
            efrom[ne] = rb;
            eto[ne] = ra;
        }
        ne++;
    }
    if (ne == 0) return;
    // distinct endpoint components in seed order
    uint32_t nn = 0;
    for (uint32_t i = 0; i < 2 * ne; i++) {
        const uint32_t r = i < ne ? efrom[i] : eto[i - ne];
        bool dup = false;
        for (uint32_t j = 0; j < nn && !dup; j++) dup = nodes[j] == r;
        if (dup) continue;
        uint32_t j = nn++;
        while (j > 0 && a.seed[nodes[j - 1]] > a.seed[r]) {
            nodes[j] = nodes[j - 1];
            j--;
        }
        nodes[j] = r;
    }
    for (uint32_t i = 0; i < nn; i++) a.cstart[nodes[i]] = kNone;
    for (uint32_t i = 0; i < nn; i++) {
        const uint32_t u = nodes[i];
        if (a.cstart[u] != kNone) continue;
        a.cstart[u] = u;
        uint32_t top = 0;
        stack[top++] = u;
        while (top) {
            const uint32_t x = stack[--top];
            for (uint32_t e = 0; e < ne; e++) {
                if (efrom[e] != x) continue;
                const uint32_t y = eto[e];
                if (a.cstart[y] != kNone) continue;
                a.cstart[y] = u;
                stack[top++] = y;
            }
        }
    }
}

__global__ void start_flags_kernel(ClusterArgs a) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= a.n || !is_core(a.deg[k], a.minpts)) return;
    if (a.parent[k] == k && a.cstart[k] == k && VDB_GUARD(a.st, a.seed[k] < a.n, 12, a.seed[k]))
        a.pos_flag[a.seed[k]] = 1u;
}

__device__ __forceinline__ uint32_t start_time(const ClusterArgs& a, uint32_t u) {
    return a.seed[a.cstart[a.parent[u]]];
}

// Non-core rows (shorter than minpts): earliest cluster start among the core
// neighbours that hold the point in their own neighbourhood.  (32 registers:
// the launch's 8 blocks of 256 threads per SM all stay resident.)
__global__ void __launch_bounds__(kThreads, 8) border_pull_kernel(ClusterArgs a) {
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t r = a.row_lo + warp; r < a.row_hi; r += nwarps) {
        const uint32_t k = (uint32_t)r;
        if (is_core(a.deg[k], a.minpts)) continue;
        const unsigned long long s = a.off[k] - a.off_base, e = a.off[k + 1] - a.off_base;
        uint32_t mn = kNone;
        auto pull = [&](uint32_t v) {
            if (!VDB_GUARD(a.st, v < a.n, 11, v)) return;
            if (v == k || !is_core(a.deg[v], a.minpts)) return;
            mn = min(mn, start_time(a, v));
        };
        // one-way entries (k reaches v, v does not reach k) are skipped
        if (a.compact) {
            walk_compact_row(reinterpret_cast<const uint16_t*>(a.nbr), s, e, k, a.ptile, a.tiles,
                             a.tile_uoff, a.parts, a.trow_s, a.trow_e, 2 * a.ep->rho + 1,
                             a.unit_words, (int)lane, [&](uint32_t v, bool one_way, bool valid) {
                                 if (valid && !one_way) pull(v);
                             });
        } else {
            for (unsigned long long j = s + lane; j < e; j += 32) {
                const uint32_t ev = a.nbr[j];
                if (!(ev & kAsymFlag)) pull(ev & kIdMask);
            }
        }
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) mn = min(mn, __shfl_down_sync(kFull, mn, d));
        if (lane == 0) a.best[k] = mn;
    }
}

// In-edges that the non-core row does not list: pairs accepted only towards
// the non-core point.
__global__ void asym_push_kernel(ClusterArgs a) {
    uint32_t na = *a.asym_count;
    if (na > a.asym_cap) na = a.asym_cap;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < na;
         i += gridDim.x * blockDim.x) {
    const AsymPair p = a.asym[i];
    uint32_t from, to;
    if (p.dir == 1u) {
        from = p.a;
        to = p.b;
    } else {
        from = p.b;
        to = p.a;
    }
    if (!is_core(a.deg[from], a.minpts) || is_core(a.deg[to], a.minpts)) continue;
    atomicMin(&a.best[to], start_time(a, from));
    }
}

__global__ void write_labels_kernel(ClusterArgs a) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= a.n) return;
    uint32_t lab;
    if (is_core(a.deg[k], a.minpts)) {
        const uint32_t t = start_time(a, k);
        lab = VDB_GUARD(a.st, t < a.n, 14, t) ? a.cluster_no[t] + 1u : 0u;
    } else {
        const uint32_t b = a.best[k];
        lab = (b != kNone && b < a.gpos[k]) ? a.cluster_no[b] + 1u : 0u;
    }
    if (VDB_GUARD(a.st, a.gorig[k] < a.n, 13, a.gorig[k])) a.labels_out[a.gorig[k]] = lab;
}

// vmax[v] = largest label of variant v (one atomic per variant and warp)
// Largest label of each variant: block b reduces part b % bpv of variant
// b / bpv and raises vmax[v] once.
__global__ void label_max_kernel(const uint32_t* __restrict__ labels, uint32_t n, uint32_t bpv,
                                 uint32_t* __restrict__ vmax) {
    __shared__ uint32_t s_max[kThreads / 32];
    const uint32_t v = blockIdx.x / bpv, part = blockIdx.x % bpv;
    const uint32_t* __restrict__ lv = labels + (size_t)v * n;
    uint32_t mx = 0;
    for (unsigned long long i = (unsigned long long)part * kThreads + threadIdx.x; i < n;
         i += (unsigned long long)bpv * kThreads)
        mx = max(mx, lv[i]);
    mx = __reduce_max_sync(kFull, mx);
    if ((threadIdx.x & 31) == 0) s_max[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x < 32) {
        mx = threadIdx.x < kThreads / 32 ? s_max[threadIdx.x] : 0u;
        mx = __reduce_max_sync(kFull, mx);
        if (threadIdx.x == 0 && mx) atomicMax(&vmax[v], mx);
    }
}

__global__ void sum_clusters_kernel(const uint32_t* __restrict__ vmax, uint32_t V,
                                    DeviceStatus* st) {
    unsigned long long acc = 0;
    for (uint32_t v = threadIdx.x; v < V; v += blockDim.x) acc += vmax[v];
    for (int d = 16; d > 0; d >>= 1) acc += __shfl_down_sync(kFull, acc, d);
    if ((threadIdx.x & 31) == 0 && acc) atomicAdd(&st->clusters, acc);
}

}  // namespace

void launch_count_clusters(const uint32_t* labels, uint32_t n, uint32_t V, uint32_t* vmax,
                           DeviceStatus* st, cudaStream_t s) {
    if (!n || !V) return;
    cudaMemsetAsync(vmax, 0, (size_t)V * sizeof(uint32_t), s);
    // about 8 labels per thread, at most 64 blocks per variant
    const uint32_t bpv = (uint32_t)std::min<unsigned long long>(
        64, std::max<unsigned long long>(1, ((unsigned long long)n + 8 * kThreads - 1) / (8 * kThreads)));
    VDB_COUNT_LAUNCH();
    label_max_kernel<<<bpv * V, kThreads, 0, s>>>(labels, n, bpv, vmax);
    VDB_COUNT_LAUNCH();
    sum_clusters_kernel<<<1, kThreads, 0, s>>>(vmax, V, st);
}

size_t resolve_scratch_bytes() { return (size_t)kResolveCap * 6 * sizeof(uint32_t); }

void launch_uf_init(const ClusterArgs& a, bool fresh, cudaStream_t s) {
    if (a.n) VDB_COUNT_LAUNCH();
    if (a.n)
        uf_init_kernel<<<nblk(a.n), kThreads, 0, s>>>(a.n, fresh ? 1 : 0, a.parent, a.seed,
                                                      a.best, a.cstart, a.pos_flag);
}

void launch_uf_union(const ClusterArgs& a, int nblocks, cudaStream_t s) {
    if (a.row_hi > a.row_lo) { VDB_COUNT_LAUNCH(); uf_union_kernel<<<nblocks, kThreads, 0, s>>>(a); }
}

void launch_cell_union(const ClusterArgs& a, int nblocks, cudaStream_t s) {
    if (!a.n) return;
    // crep[c] starts as "no core" for every cell (ncl <= n)
    cudaMemsetAsync(a.crep, 0xff, (size_t)a.n * sizeof(uint32_t), s);
    VDB_COUNT_LAUNCH();
    cell_rep_min_kernel<<<nblk(a.n), kThreads, 0, s>>>(a);
    VDB_COUNT_LAUNCH();
    cell_rep_link_kernel<<<nblk(a.n), kThreads, 0, s>>>(a);
    VDB_COUNT_LAUNCH();
    cell_pairs_kernel<<<nblocks, kThreads, 0, s>>>(a);
}

void launch_uf_finish(const ClusterArgs& a, void* resolve_ws, void* scan_scratch,
                      cudaStream_t s) {
    if (!a.n) return;
    VDB_COUNT_LAUNCH();
    uf_flatten_kernel<<<nblk(a.n), kThreads, 0, s>>>(a);
    VDB_COUNT_LAUNCH();
    resolve_kernel<<<1, 32, 0, s>>>(a, (uint32_t*)resolve_ws, kResolveCap);
    VDB_COUNT_LAUNCH();
    start_flags_kernel<<<nblk(a.n), kThreads, 0, s>>>(a);
    scan_u32(a.pos_flag, a.cluster_no, a.n, scan_scratch, s);
}

void launch_save_components(const ClusterArgs& a, uint32_t* comp, cudaStream_t s) {
    if (!a.n) return;
    VDB_COUNT_LAUNCH();
    save_components_kernel<<<nblk(a.n), kThreads, 0, s>>>(a, comp);
}

void launch_border_pull(const ClusterArgs& a, int nblocks, cudaStream_t s) {
    if (a.row_hi <= a.row_lo) return;
    VDB_COUNT_LAUNCH();
    border_pull_kernel<<<nblocks, kThreads, 0, s>>>(a);
}

void launch_label_write(const ClusterArgs& a, cudaStream_t s) {
    if (!a.n) return;
    VDB_COUNT_LAUNCH();
    asym_push_kernel<<<64, kThreads, 0, s>>>(a);
    VDB_COUNT_LAUNCH();
    write_labels_kernel<<<nblk(a.n), kThreads, 0, s>>>(a);
}

void launch_border_and_write(const ClusterArgs& a, int nblocks, cudaStream_t s) {
    if (!a.n) return;
    launch_border_pull(a, nblocks, s);
    launch_label_write(a, s);
}

}  // namespace vdb
