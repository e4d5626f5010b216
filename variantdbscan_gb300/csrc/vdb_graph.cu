// Device side of graph replay (vdb_options.graph): the checkpoint kernel that
// re-checks, on each replay of a captured call, the device values the host
// read while recording it, and the kernel that stores per-table parameters
// (a captured call cannot copy them from host memory that changes later).
#include "vdb_internal.cuh"

namespace vdb {

namespace {

__global__ void graph_check_kernel(GraphCheck chk, uint32_t* bad,
                                   cudaGraphConditionalHandle next) {
    if (threadIdx.x != 0) return;
    // an earlier checkpoint failed: everything after it is skipped
    bool ok = *bad == 0u;
    for (int i = 0; i < chk.n && i < kGraphConds; i++) {
        const GraphCond& c = chk.c[i];
        switch (c.kind) {
            case kGcEq64:
                ok = ok && *(const unsigned long long*)c.ptr == c.a;
                break;
            case kGcLe64: {
                const unsigned long long v = *(const unsigned long long*)c.ptr;
                ok = ok && v <= c.a;
                if (c.sum) *c.sum += v;
                break;
            }
            case kGcLe32:
                ok = ok && (unsigned long long)*(const uint32_t*)c.ptr <= c.a;
                break;
            case kGcMask32:
                ok = ok && (*(const uint32_t*)c.ptr & (uint32_t)c.a) == (uint32_t)c.b;
                break;
            case kGcGeF64:
                ok = ok && *(const double*)c.ptr >= __longlong_as_double((long long)c.a);
                break;
            case kGcLeF64:
                ok = ok && *(const double*)c.ptr <= __longlong_as_double((long long)c.a);
                break;
            default:
                ok = false;
        }
    }
    if (!ok && *bad == 0u) *bad = chk.index;
    cudaGraphSetConditional(next, ok ? 1u : 0u);
}

__global__ void store_eps_kernel(EpsParams* dst, EpsParams v) {
    if (threadIdx.x == 0 && blockIdx.x == 0) *dst = v;
}

}  // namespace

void launch_graph_check(const GraphCheck& chk, uint32_t* bad, cudaGraphConditionalHandle next,
                        cudaStream_t s) {
    VDB_COUNT_LAUNCH();
    graph_check_kernel<<<1, 32, 0, s>>>(chk, bad, next);
}

void launch_store_eps(EpsParams* dst, const EpsParams& v, cudaStream_t s) {
    VDB_COUNT_LAUNCH();
    store_eps_kernel<<<1, 32, 0, s>>>(dst, v);
}

}  // namespace vdb
