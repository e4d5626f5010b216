/*
 * vdbscan.h - C ABI of the GB300 VariantDBSCAN library (libSharedVDBSCAN.so).
 *
 * The library is a drop-in for the reference's CPU shared library of the same
 * name.  Every buffer is owned by the caller; no entry point prints unless
 * asked to (verbose); all entry points return 0 on success and a negative
 * VDB_ERR_* code otherwise.
 *
 * Labels: 0 = noise, 1..K = clusters numbered in the order in which the
 * reference's sequential DBSCAN meets their seeds (its visit order), so the
 * values are identical to the reference's, not just the partition.  Each
 * variant is clustered on its own (the reference's from-scratch path,
 * src/DBScan.cpp:523-609); the reference's multi-variant cluster reuse
 * (src/DBScan.cpp:272-416) is not reproduced because its result depends on
 * thread timing.
 *
 * Thread safety: calls on different vdb_context objects may run concurrently
 * from different host threads.  libVDBSCAN uses one process-wide context and
 * serialises its callers.
 */
#ifndef VDBSCAN_GB300_H
#define VDBSCAN_GB300_H

#include <stddef.h>
#include <stdint.h>
#ifndef __cplusplus
#include <stdbool.h>
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ errors */
#define VDB_OK 0
#define VDB_ERR_INVALID_ARG (-1)   /* null pointer, MBBsize <= 0, NaN/inf input */
#define VDB_ERR_DEGENERATE (-2)    /* zero-width bounding box: the reference's binDataset
                                      prints "bins out of range" and leaves its mapping short
                                      (src/main.cpp:559-563) */
#define VDB_ERR_CUDA (-3)          /* a CUDA runtime call failed */
#define VDB_ERR_NOMEM (-4)         /* device memory could not be allocated */
#define VDB_ERR_CAPACITY (-5)      /* an internal fixed-size list overflowed */
#define VDB_ERR_NO_DEVICE (-6)     /* no CUDA device is visible */
#define VDB_ERR_TOO_LARGE (-7)     /* N*V or N exceeds what the ABI can index */

/* ------------------------------------------------------------ reference ABI */

/* Replaces libVDBSCAN of the reference (src/main.cpp:50; prototype
 * src/c_test_prog.h:26; ctypes binding python_package/vdbscan/variantdbscan.py:66-69).
 * inputx/inputy: datasetSize FP64 coordinates (host memory).
 * inputEpsilon/inputMinpts: numVariants variants (host memory).
 * MBBsize: points per R-tree box in the reference; it decides which candidate
 *   pairs the reference tests (src/main.cpp:404-436), so it is honoured.
 * retArr: datasetSize*numVariants labels, retArr[v*datasetSize + i] (host),
 *   variant v in the caller's order, point i in the caller's order
 *   (src/main.cpp:273-284).
 * Returns 0 on success (the reference always returns 0), VDB_ERR_* otherwise. */
int libVDBSCAN(double *inputx, double *inputy, unsigned int datasetSize,
               double *inputEpsilon, unsigned int *inputMinpts, unsigned int numVariants,
               int MBBsize, unsigned int *retArr, bool verbose);

/* ------------------------------------------------------------ batched API */

typedef struct vdb_context vdb_context;

/* Distance-test precision of the neighbour search. */
#define VDB_PRECISION_MIXED 0  /* FP32 filter on cell-local coordinates, FP64 re-test
                                  of pairs within the error band (default) */
#define VDB_PRECISION_FP64 1   /* every candidate pair tested in FP64 */

/* Variant scheduling. */
#define VDB_SCHEDULE_BATCHED 0 /* variants of equal epsilon share one neighbour table and
                                  one grid; each minpts is then labelled on its own */
#define VDB_SCHEDULE_PLAIN 1   /* one neighbour table and one clustering per variant */

#define VDB_TABLE_ALL 0        /* every row of each neighbour table is written */
#define VDB_TABLE_BORDER 1     /* only the rows the labelling reads: points that are not
                                  core for some minpts of their epsilon (labels only;
                                  needs cells that are cliques, else all rows) */

typedef struct {
    const double *x;        /* n coordinates; host or device pointer (see location) */
    const double *y;
    uint32_t n;
    int32_t mbb_size;       /* the reference's MBBsize (70 in its examples) */
    const double *eps;      /* nv epsilons (host memory) */
    const uint32_t *minpts; /* nv minpts (host memory) */
    uint32_t nv;
    uint32_t *labels;       /* nv*n labels, labels[v*n + i]; host or device pointer */
} vdb_dataset;

#define VDB_LOC_HOST 0
#define VDB_LOC_DEVICE 1

typedef struct {
    int32_t precision;      /* VDB_PRECISION_* */
    int32_t schedule;       /* VDB_SCHEDULE_* */
    int32_t location;       /* VDB_LOC_*: where x, y and labels live */
    int32_t cells_per_eps;  /* grid cells per epsilon (1..4); 0 = the library's choice (2) */
    int32_t verbose;
    int64_t table_budget_bytes; /* neighbour-table budget; 0 = derived from free memory */
    int32_t streams;        /* datasets of one call run concurrently on this many CUDA
                               streams (one host thread each); 0 = autotuned: at most 4,
                               and no more than (total work) / (largest dataset's work),
                               work = points x distinct epsilons */
    int32_t table_rows;     /* VDB_TABLE_* */
    int32_t table_hash;     /* nonzero: fill vdb_stats.table_hash (reads every table once
                               more; meaningful with VDB_TABLE_ALL) */
    int32_t table_entry_bytes; /* neighbour-table entries: 2 = 16 bits (the position within
                               a work unit (unit_candidates) of the row's tile; half the
                               table bytes); 4 = 32 bits (the cell-ordered index);
                               0 = 16 bits with VDB_TABLE_ALL, 32 with VDB_TABLE_BORDER */
    int32_t no_reuse;       /* nonzero: label every variant from scratch.  By default
                               (batched schedule) a variant's union-find starts from the
                               components of the larger minpts before it at the same
                               epsilon, and cell pairs whose cores lie in different
                               components at a larger epsilon (and a smaller or equal
                               minpts) are not searched: both only save work, the labels
                               are those of a from-scratch run */
    int32_t tile_cells;     /* grid cells per tile group of the neighbour search (1, 2, 4,
                               8, 16); 0 = autotuned per table from a lane-slot cost model
                               of the grid's own occupancy (sampled cells) */
    int32_t unit_candidates; /* candidates of a tile per work unit of the neighbour search
                               (1024, 2048 or 4096); 0 = 1024 for datasets of fewer than
                               2^18 points (a table with few units is bounded by its
                               longest unit), else 4096.  Labels and tables do not
                               depend on it */
    int32_t graph;          /* nonzero: replay repeated calls as one CUDA graph.  The first
                               call with given datasets (buffers, sizes, variants) and
                               options runs directly, records the sizes the host reads back
                               and captures the call; later calls with the same key replay
                               it (one launch, one host wait; the datasets of a batch run in
                               concurrent branches of the graph, as many as the streams
                               option or its autotuned value gives, largest datasets first,
                               each branch reusing its buffers).  A replay serves points
                               inside the recorded bounding box whose sizes (test bitmap,
                               work units, neighbours) fit the graph's buffers, which hold
                               the recorded sizes plus a quarter; other data stop the
                               replay at its first failed checkpoint and the call runs
                               directly; the graph is then dropped and recorded again at
                               the next call.  The graph keeps its device buffers until the
                               context is destroyed or the graph is replaced (at most 4 per
                               context).  Not captured, so always direct: chunked tables,
                               empty-neighbourhood epsilons (< 0 or NaN) and recounts after
                               a one-way pair list overflow */
} vdb_options;

/* vdb_stats.graph */
#define VDB_GRAPH_NONE 0        /* vdb_options.graph not set */
#define VDB_GRAPH_CAPTURED 1    /* the call ran directly and captured its graph */
#define VDB_GRAPH_REPLAYED 2    /* the call replayed the graph */
#define VDB_GRAPH_FALLBACK 3    /* a checkpoint of the replay failed: the call ran directly */
#define VDB_GRAPH_UNSUPPORTED 4 /* the call takes a path that is not captured: ran directly */

typedef struct {
    uint64_t pairs;            /* sum over neighbour tables built of |N_eps(p)| */
    uint64_t candidates;       /* candidate pairs tested by the table kernels */
    uint64_t retested;         /* candidate pairs re-tested in FP64 */
    uint64_t asymmetric_pairs; /* pairs accepted in one direction only (box rule) */
    uint32_t tables;           /* neighbour tables built */
    uint32_t table_chunks;     /* table chunks (> tables when a table exceeded the budget) */
    uint32_t kernel_launches;  /* kernels launched by the call */
    uint32_t clusters;         /* clusters summed over variants */
    double ms_index;           /* device time: visit order, boxes, grid */
    double ms_count;           /* device time: neighbour counting */
    double ms_table;           /* device time: neighbour-table fill */
    double ms_cluster;         /* device time: union-find and labelling */
    double ms_total;           /* device time of the whole call */
    /* With vdb_options.table_hash: hash of the neighbour tables built, the sum
     * modulo 2^64 over tables, rows p and entries q in N(p) of
     * mix64(p << 32 | q) + (p not in N(q) ? 0x9e3779b97f4a7c15 : 0), p and q
     * input indices, mix64 the splitmix64 finaliser (x ^= x >> 30;
     * x *= 0xbf58476d1ce4e5b9; x ^= x >> 27; x *= 0x94d049bb133111eb;
     * x ^= x >> 31).  Equal hashes: equal neighbour sets, one-way entries
     * included (up to hash collisions). */
    uint64_t table_hash;
    uint64_t entry_bytes;      /* bytes of neighbour-table entries written */
    uint32_t compact_tables;   /* tables built with 16-bit entries */
    uint32_t pad;
    uint64_t reuse_skipped_pairs; /* cell pairs not searched because their cores lie in
                                     different components at a larger epsilon */
    uint32_t tables_by_tile_cells[8]; /* tables built with tile groups of 2^i cells */
    uint32_t worker_streams;   /* concurrent dataset streams the call used */
    uint32_t pad2;
    uint64_t device_bytes;     /* device footprint: the most device memory one dataset of the
                                  call held at once (index, tables, labelling state) */
    uint64_t table_bytes;      /* of which the largest neighbour-table allocation */
    uint32_t graph;            /* VDB_GRAPH_* */
    uint32_t graph_checks;     /* checkpoints in the call's graph */
} vdb_stats;

/* Fills opts with the defaults (mixed precision, batched, host buffers,
 * autotuned grid). */
void vdb_default_options(vdb_options *opts);

/* Creates a context on the current CUDA device; *ctx = NULL on failure.
 * stream: a cudaStream_t (NULL = the context creates its own stream). */
int vdb_context_create(vdb_context **ctx, void *stream);
void vdb_context_destroy(vdb_context *ctx);

/* Clusters nds datasets with all their variants.  Batched extension of the
 * reference ABI (no counterpart in the reference; each dataset gets the labels
 * libVDBSCAN would return for it).  stats may be NULL. */
int vdb_run_batch(vdb_context *ctx, const vdb_dataset *ds, int nds, const vdb_options *opts,
                  vdb_stats *stats);

/* Allocation-free clustering of one small dataset for one variant (no
 * counterpart in the reference).  For callers that may not allocate device
 * memory while they run: programs that reserve all their device memory up
 * front, frameworks whose own allocator owns the device heap, and
 * latency-bound code that cannot take the device-wide synchronisation that
 * cudaMalloc and cudaFree imply.  Every temporary lives in one fixed 64 MiB
 * array inside the library, which each GPU that loads the library reserves
 * until the process exits; the call allocates nothing.
 * x, y: n FP64 coordinates in device memory; labels: n labels written to
 * device memory (same values as libVDBSCAN for this variant).  stream: a
 * cudaStream_t or NULL; the call returns after the stream has finished.
 * Limits: n <= 65536 and the neighbour table must fit what the other
 * temporaries leave of the 64 MiB (about 12 million pairs at n = 65536);
 * larger inputs return VDB_ERR_TOO_LARGE.  More than 262,144 pairs accepted
 * in one direction only (pairs at almost exactly eps along an axis whose
 * multiple-point box misses the other point's query box) return
 * VDB_ERR_CAPACITY.  eps must be finite and >= 0.
 * The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress) and keeps it for the life of the process.  The kept
 * address does not survive a cudaDeviceReset of that device: do not call this
 * entry point after one.
 * All calls share the one array: calls are serialised by a process-wide lock,
 * and work that overlaps a call on the GPU through the same array would
 * race. */
int vdb_run_noalloc(const double *x, const double *y, uint32_t n, double eps, uint32_t minpts,
                    int32_t mbb_size, uint32_t *labels, void *stream);

/* ------------------------------------------------------------ file ingest */

/* Reads a dataset file as the reference's GPU prototype does (importDataset,
 * src/gpu/import_dataset.cpp:63-134): one point per line,
 * "longitude,latitude[,value...]"; x[i] = the latitude mapped to [0, 180]
 * (((90 - lat) / 90) * 90 for lat > 0, ((-lat) / 90) * 90 + 90 otherwise),
 * y[i] = the longitude.  Blank lines are skipped.  x and y hold cap points
 * (both NULL: count only); *n receives the number of points in the file.
 * Returns VDB_ERR_INVALID_ARG for an unreadable file or a line with fewer
 * than two fields, VDB_ERR_CAPACITY when the file holds more than cap points
 * (the first cap are stored).  Host code only: no device is needed. */
int vdb_import_dataset(const char *path, double *x, double *y, uint32_t cap, uint32_t *n);

/* Reads a variant file as the reference's GPU prototype does
 * (importDBScanInstances, src/gpu/import_dataset.cpp:232-262): "epsilon,minpts"
 * per line, sorted by compareByEpsilon (import_dataset.cpp:41-49): epsilon
 * descending, then minpts ascending (NaN epsilons last).  eps and minpts hold
 * cap variants (both NULL: count only); *nv receives the number of variants.
 * Negative minpts is VDB_ERR_INVALID_ARG; otherwise as vdb_import_dataset. */
int vdb_import_variants(const char *path, double *eps, uint32_t *minpts, uint32_t cap,
                        uint32_t *nv);

/* Message of the last failing call on ctx (thread-local for libVDBSCAN). */
const char *vdb_last_error(vdb_context *ctx);

/* Library version string. */
const char *vdb_version(void);

#ifdef __cplusplus
}
#endif

#endif /* VDBSCAN_GB300_H */
