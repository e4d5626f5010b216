// Index construction on the device:
//  * the reference's visit order (binDataset, src/main.cpp:459-605),
//  * its multiple-point boxes (createEntryMBBMultiplePoints, src/main.cpp:404-436;
//    MPBRect::CreateMBB, src/structs.h:79-120),
//  * the uniform grid that replaces its R-tree for candidate generation:
//    cell keys, cell-ordered coordinates, cell start offsets and query tiles.
#include <float.h>

#include "vdb_internal.cuh"

namespace vdb {

namespace {

constexpr int kThreads = 256;

inline unsigned nblk(uint64_t n) { return (unsigned)((n + kThreads - 1) / kThreads); }

// Bin key of src/main.cpp:491-540 evaluated with the same FP64 operations:
// width = (max-min)*1.01, offset = -min (or fabs(min)), bin = floor(((x+offset)/width)*300).
__global__ void visit_keys_kernel(const double* __restrict__ x, const double* __restrict__ y,
                                  uint32_t n, const BBox* __restrict__ bb,
                                  uint32_t* __restrict__ keys, uint32_t* __restrict__ idx,
                                  DeviceStatus* st) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double minx = bb->minx, maxx = bb->maxx, miny = bb->miny, maxy = bb->maxy;
    const double xw = __dmul_rn(__dsub_rn(maxx, minx), 1.01);
    const double yw = __dmul_rn(__dsub_rn(maxy, miny), 1.01);
    const double xo = (minx > 0) ? -minx : fabs(minx);
    const double yo = (miny > 0) ? -miny : fabs(miny);
    double fx = floor(__dmul_rn(__ddiv_rn(__dadd_rn(x[i], xo), xw), (double)kVisitBins));
    double fy = floor(__dmul_rn(__ddiv_rn(__dadd_rn(y[i], yo), yw), (double)kVisitBins));
    bool ok = fx >= 0.0 && fx <= (double)(kVisitBins - 1) && fy >= 0.0 &&
              fy <= (double)(kVisitBins - 1);
    if (!ok) {
        atomicOr(&st->flags, kStatDegenerate);
        fx = 0.0;
        fy = 0.0;
    }
    keys[i] = (uint32_t)fx * kVisitBins + (uint32_t)fy;
    idx[i] = i;
}

__global__ void invert_kernel(const uint32_t* __restrict__ order, uint32_t n,
                              uint32_t* __restrict__ inv) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n && order[k] < n) inv[order[k]] = k;
}

// One warp per box: the bounding box of visit positions [b*mbb, b*mbb+mbb)
// (the lanes gather the box's points 32 at a time, then reduce).
__global__ void mpb_kernel(const double* __restrict__ x, const double* __restrict__ y,
                           const uint32_t* __restrict__ vorder, uint32_t n, int mbb,
                           uint32_t nboxes, MpbBox* __restrict__ boxes) {
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t b = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (b >= nboxes) return;  // (whole warps)
    const uint64_t s = b * (uint32_t)mbb;
    uint64_t e = s + (uint32_t)mbb;
    if (e > n) e = n;
    double x0 = INFINITY, x1 = -INFINITY, y0 = INFINITY, y1 = -INFINITY;
    for (uint64_t k = s + lane; k < e; k += 32) {
        const uint32_t o = vorder[k];
        const double xv = x[o], yv = y[o];
        if (xv < x0) x0 = xv;
        if (xv > x1) x1 = xv;
        if (yv < y0) y0 = yv;
        if (yv > y1) y1 = yv;
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        const double a0 = __shfl_xor_sync(0xffffffffu, x0, d);
        const double a1 = __shfl_xor_sync(0xffffffffu, x1, d);
        const double b0 = __shfl_xor_sync(0xffffffffu, y0, d);
        const double b1 = __shfl_xor_sync(0xffffffffu, y1, d);
        if (a0 < x0) x0 = a0;
        if (a1 > x1) x1 = a1;
        if (b0 < y0) y0 = b0;
        if (b1 > y1) y1 = b1;
    }
    if (lane == 0) boxes[b] = MpbBox{x0, x1, y0, y1};
}

__device__ __forceinline__ uint32_t cell_of(double v, double v0, double w, uint32_t nc) {
    double f = floor(__ddiv_rn(__dsub_rn(v, v0), w));
    if (!(f >= 0.0)) f = 0.0;
    if (f > (double)(nc - 1)) f = (double)(nc - 1);
    return (uint32_t)f;
}

__global__ void grid_keys_kernel(const double* __restrict__ x, const double* __restrict__ y,
                                 uint32_t n, GridParams g, uint32_t* __restrict__ keys,
                                 uint32_t* __restrict__ idx) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t cx = cell_of(x[i], g.x0, g.w, g.ncx);
    uint32_t cy = cell_of(y[i], g.y0, g.w, g.ncy);
    keys[i] = cy * g.ncx_pad + cx;
    idx[i] = i;
}

// Cell-ordered copies: FP64 coordinates, FP32 coordinates relative to the own
// cell's origin (the FP64 shift is exact up to one rounding; the FP32
// conversion adds one more), and the visit position of every point.
__global__ void grid_gather_kernel(const double* __restrict__ x, const double* __restrict__ y,
                                   const uint32_t* __restrict__ gorig,
                                   const uint32_t* __restrict__ pos, uint32_t n, GridParams g,
                                   const uint32_t* __restrict__ gkey, double2* __restrict__ gxy,
                                   float2* __restrict__ glocal, uint32_t* __restrict__ gpos) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    uint32_t o = gorig[k];
    double xv = x[o], yv = y[o];
    uint32_t key = gkey[k];
    uint32_t cy = key / g.ncx_pad, cx = key - cy * g.ncx_pad;
    double ox = __dadd_rn(g.x0, __dmul_rn((double)cx, g.w));
    double oy = __dadd_rn(g.y0, __dmul_rn((double)cy, g.w));
    gxy[k] = make_double2(xv, yv);
    glocal[k] = make_float2(__double2float_rn(__dsub_rn(xv, ox)),
                            __double2float_rn(__dsub_rn(yv, oy)));
    gpos[k] = pos[o];
}

// cell_start[key] = first sorted index of each non-empty cell; the rest is
// filled by a suffix-min so that empty cells point at the next non-empty one.
__global__ void cell_marks_kernel(const uint32_t* __restrict__ gkey, uint32_t n,
                                  uint32_t* __restrict__ cell_start, uint64_t ncells) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k == 0) cell_start[ncells] = n;
    if (k >= n) return;
    if ((k == 0 || gkey[k] != gkey[k - 1]) && gkey[k] < ncells) cell_start[gkey[k]] = k;
}

__global__ void tile_flags_kernel(const uint32_t* __restrict__ gkey, uint32_t n, uint32_t G,
                                  uint32_t tq, uint32_t* __restrict__ flags) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    flags[k] = (k == 0 || (gkey[k] / G) != (gkey[k - 1] / G) || (k % tq) == 0) ? 1u : 0u;
}

__global__ void tile_write_kernel(const uint32_t* __restrict__ flags,
                                  const uint32_t* __restrict__ scan, uint32_t n,
                                  uint32_t* __restrict__ tiles) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k == 0) tiles[scan[n]] = n;
    if (k < n && flags[k]) tiles[scan[k]] = k;
}

__global__ void cell_rows_kernel(const uint32_t* __restrict__ gkey,
                                 const uint32_t* __restrict__ clist,
                                 const uint32_t* __restrict__ ncl, uint32_t n, uint32_t ncx_pad,
                                 uint32_t ncy, uint32_t* __restrict__ crow,
                                 uint32_t* __restrict__ ccx) {
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t nc = *ncl;
    if (c == 0) crow[ncy] = nc;
    if (c >= nc || c >= n) return;
    const uint32_t key = gkey[clist[c]];
    const uint32_t cy = key / ncx_pad;
    ccx[c] = key - cy * ncx_pad;
    if (cy < ncy && (c == 0 || gkey[clist[c - 1]] / ncx_pad != cy)) crow[cy] = c;
}

__global__ void point_boxes_kernel(const uint32_t* __restrict__ gpos, uint32_t n,
                                   const MpbBox* __restrict__ mpb, uint32_t mbb,
                                   MpbBox* __restrict__ gbox) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) gbox[k] = mpb[gpos[k] / mbb];
}

__global__ void tile_costs_kernel(GridParams g, const EpsParams* __restrict__ ep,
                                  const uint32_t* __restrict__ gkey,
                                  const uint32_t* __restrict__ cell_start,
                                  const uint32_t* __restrict__ crow,
                                  const uint32_t* __restrict__ ccx,
                                  const uint32_t* __restrict__ clist,
                                  const uint32_t* __restrict__ ncl, uint32_t n,
                                  unsigned long long* __restrict__ out) {
    __shared__ unsigned long long s_acc[2 * kTuneShapes];
    for (int i = threadIdx.x; i < 2 * kTuneShapes; i += blockDim.x) s_acc[i] = 0ull;
    __syncthreads();
    const uint32_t nc = min(*ncl, n);
    const int rho = ep->rho;
    // sampled cells: about kTuneSamples of them, in runs of kTuneRun
    // consecutive non-empty cells spread evenly over all of them (a regular
    // stride of single cells would alias with the period G of the groups of
    // dense rows and count some shapes' groups more often than others)
    const uint64_t per = ((uint64_t)nc + kTuneSamples - 1) / kTuneSamples;
    const uint64_t stride = per ? per : 1;
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t c = (t / kTuneRun) * kTuneRun * stride + t % kTuneRun;
    if (c < nc) {
        const uint32_t key = gkey[clist[c]];
        const uint32_t cy = key / g.ncx_pad, cx = key - cy * g.ncx_pad;
        uint32_t pcy = 0xffffffffu, pcx = 0;
        if (c > 0) {
            const uint32_t pk = gkey[clist[c - 1]];
            pcy = pk / g.ncx_pad;
            pcx = pk - pcy * g.ncx_pad;
        }
#pragma unroll 1
        for (int i = 0; i < kTuneShapes; i++) {
            const uint32_t G = 1u << i;
            if (pcy == cy && pcx / G == cx / G) continue;  // not the group's first cell
            const uint32_t gx0 = cx / G * G;
            const uint32_t gx1 = min(gx0 + G - 1, g.ncx - 1);
            uint32_t s0, e0;
            cell_row_range(g, cell_start, crow, ccx, clist, cy, gx0, gx1, &s0, &e0);
            const unsigned long long P = e0 - s0;
            unsigned long long C = 0;
            for (int r = 0; r <= 2 * rho; r++) {
                const int ry = (int)cy + r - rho;
                if (ry < 0 || ry >= (int)g.ncy) continue;
                const int reach = ep->reach[r];
                const uint32_t lo = (uint32_t)max((int)gx0 - reach, 0);
                const uint32_t hi = (uint32_t)min((int)gx1 + reach, (int)g.ncx - 1);
                uint32_t s1, e1;
                cell_row_range(g, cell_start, crow, ccx, clist, (uint32_t)ry, lo, hi, &s1, &e1);
                C += e1 - s1;
            }
            atomicAdd(&s_acc[2 * i], C * 32ull * ((P + 31) / 32));
            atomicAdd(&s_acc[2 * i + 1], (P + 63) / 64);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 2 * kTuneShapes; i += blockDim.x)
        if (s_acc[i]) atomicAdd(&out[i], s_acc[i]);
}

__global__ void grid_rekey_kernel(uint32_t* __restrict__ gkey, uint32_t n, uint32_t from,
                                  uint32_t to) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint32_t key = gkey[k];
    const uint32_t cy = key / from;
    gkey[k] = cy * to + (key - cy * from);
}

}  // namespace

void launch_tile_costs(const GridParams& g, const EpsParams* ep, const uint32_t* gkey,
                       const uint32_t* cell_start, const uint32_t* crow, const uint32_t* ccx,
                       const uint32_t* clist, const uint32_t* ncl, uint32_t n,
                       unsigned long long* out, cudaStream_t s) {
    if (!n) return;
    const uint64_t threads = (uint64_t)kTuneSamples + kTuneRun;
    VDB_COUNT_LAUNCH();
    tile_costs_kernel<<<nblk(threads), kThreads, 0, s>>>(g, ep, gkey, cell_start, crow, ccx,
                                                        clist, ncl, n, out);
}

void launch_grid_rekey(uint32_t* gkey, uint32_t n, uint32_t ncx_pad_from, uint32_t ncx_pad_to,
                       cudaStream_t s) {
    if (!n || ncx_pad_from == ncx_pad_to) return;
    VDB_COUNT_LAUNCH();
    grid_rekey_kernel<<<nblk(n), kThreads, 0, s>>>(gkey, n, ncx_pad_from, ncx_pad_to);
}

void launch_point_boxes(const uint32_t* gpos, uint32_t n, const MpbBox* mpb, int mbb,
                        MpbBox* gbox, cudaStream_t s) {
    if (!n) return;
    VDB_COUNT_LAUNCH();
    point_boxes_kernel<<<nblk(n), kThreads, 0, s>>>(gpos, n, mpb, (uint32_t)mbb, gbox);
}

void launch_cell_rows(const uint32_t* gkey, const uint32_t* clist, const uint32_t* ncl,
                      uint32_t n, const GridParams& g, uint32_t* crow, uint32_t* ccx,
                      cudaStream_t s) {
    VDB_COUNT_LAUNCH();
    cell_rows_kernel<<<nblk(n ? n : 1), kThreads, 0, s>>>(gkey, clist, ncl, n, g.ncx_pad, g.ncy,
                                                         crow, ccx);
}

void launch_visit_keys(const double* x, const double* y, uint32_t n, const BBox* bb,
                       uint32_t* keys, uint32_t* idx, DeviceStatus* st, cudaStream_t s) {
    if (n) { VDB_COUNT_LAUNCH(); visit_keys_kernel<<<nblk(n), kThreads, 0, s>>>(x, y, n, bb, keys, idx, st); }
}

void launch_invert(const uint32_t* order, uint32_t n, uint32_t* inv, cudaStream_t s) {
    if (n) { VDB_COUNT_LAUNCH(); invert_kernel<<<nblk(n), kThreads, 0, s>>>(order, n, inv); }
}

void launch_mpb_boxes(const double* x, const double* y, const uint32_t* vorder, uint32_t n,
                      int mbb, MpbBox* boxes, cudaStream_t s) {
    uint32_t nb = (uint32_t)(((uint64_t)n + (uint32_t)mbb - 1) / (uint32_t)mbb);
    if (nb) {
        VDB_COUNT_LAUNCH();
        mpb_kernel<<<nblk((uint64_t)nb * 32u), kThreads, 0, s>>>(x, y, vorder, n, mbb, nb,
                                                                  boxes);
    }
}

void launch_grid_keys(const double* x, const double* y, uint32_t n, GridParams g,
                      uint32_t* keys, uint32_t* idx, cudaStream_t s) {
    if (n) { VDB_COUNT_LAUNCH(); grid_keys_kernel<<<nblk(n), kThreads, 0, s>>>(x, y, n, g, keys, idx); }
}

void launch_grid_gather(const double* x, const double* y, const uint32_t* gorig,
                        const uint32_t* pos, uint32_t n, GridParams g, const uint32_t* gkey,
                        double2* gxy, float2* glocal, uint32_t* gpos, cudaStream_t s) {
    if (n) VDB_COUNT_LAUNCH();
    if (n)
        grid_gather_kernel<<<nblk(n), kThreads, 0, s>>>(x, y, gorig, pos, n, g, gkey, gxy,
                                                        glocal, gpos);
}

void launch_cell_marks(const uint32_t* gkey, uint32_t n, uint32_t* cell_start,
                       uint64_t ncells, cudaStream_t s) {
    VDB_COUNT_LAUNCH();
    cell_marks_kernel<<<nblk(n ? n : 1), kThreads, 0, s>>>(gkey, n, cell_start, ncells);
}

void launch_tile_flags(const uint32_t* gkey, uint32_t n, uint32_t G, uint32_t tq,
                       uint32_t* flags, cudaStream_t s) {
    if (n) { VDB_COUNT_LAUNCH(); tile_flags_kernel<<<nblk(n), kThreads, 0, s>>>(gkey, n, G, tq, flags); }
}

void launch_tile_write(const uint32_t* flags, const uint32_t* scan, uint32_t n,
                       uint32_t* tiles, cudaStream_t s) {
    VDB_COUNT_LAUNCH();
    tile_write_kernel<<<nblk(n ? n : 1), kThreads, 0, s>>>(flags, scan, n, tiles);
}

}  // namespace vdb
