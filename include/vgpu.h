/*
 * vgpu.h -- libvgpu: GB300 (sm_103a) operator nodes for vectra's columnar
 * execution path: predicate evaluation into selection vectors, hash grouped
 * aggregation, hash-join build and probe, and the arithmetic projections
 * that feed them.
 *
 * DROP-IN BOUNDARY.  The four constructors below have exactly the names,
 * signatures, ownership rules and output schemas of the reference's node
 * constructors, so linking libvgpu in place of src/filter.c, src/project.c,
 * src/group_agg.c and src/join.c hands every plan the R front end and the
 * optimizer build to the GPU.  The nodes they return keep the reference's
 * struct prefixes and `kind` strings (include/vectra_abi.h), which the
 * optimizer and explain() read through casts.  Construction touches no
 * device (the library initialises on the first next_batch), so the
 * optimizer can rewrite a plan of libvgpu nodes on any host.
 *
 * Batches crossing the boundary are host memory owned by the receiver and
 * released with free(), as in the reference.  Columns stay resident on the
 * device inside a chain of libvgpu nodes: a group-agg node over a filter,
 * a projection and/or a join runs the whole chain as one fused kernel.
 *
 * Errors: every failure releases the node's device state and then calls
 * vectra_error() (src/error.c), which does not return.  Without the
 * reference engine linked in, libvgpu's own vectra_error reports through
 * the vgpu_guard_* entry points below.  Nothing falls back to the CPU: an
 * input the GPU path does not support (string keys, string expressions) is
 * an explicit error.
 */
#ifndef VGPU_H
#define VGPU_H

#include "vectra_abi.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- drop-in node constructors -------------------------------------- */

/* replaces src/filter.h:14 (FilterNode *filter_node_create).  Predicates
 * over int64, double, bool and string columns (comparisons, Kleene logic,
 * is.na, arithmetic, nchar, substr, grepl with a fixed pattern). */
FilterNode *filter_node_create(VecNode *child, VecExpr *predicate);

/* replaces src/project.h:23 (ProjectNode *project_node_create) */
ProjectNode *project_node_create(VecNode *child, int n_entries,
                                 ProjEntry *entries);

/* replaces src/group_agg.h:28-31 (GroupAggNode *group_agg_node_create).
 * temp_dir != NULL with n_keys > 0 emits groups in ascending key order with
 * NA last (what the reference's sort path produces); otherwise groups come
 * in first-seen order (the reference's hash path).  No spill directory is
 * used: group state lives in device memory. */
GroupAggNode *group_agg_node_create(VecNode *child, int n_keys,
                                    char **key_names, int n_aggs,
                                    AggSpec *agg_specs, const char *temp_dir);

/* replaces src/join.h:76-78 (JoinNode *join_node_create).  Keys of any
 * type, string keys included (compared byte for byte); string columns are
 * carried on both sides. */
JoinNode *join_node_create(VecNode *left, VecNode *right, JoinKind kind,
                           int n_keys, JoinKey *keys,
                           const char *suffix_x, const char *suffix_y);

/* replaces src/scan.h:22 (ScanNode *scan_node_create): a .vtr scan with
 * the reference's ScanNode prefix and kind, so the optimizer prunes its
 * columns and pushes a filter's predicate into it as before; row groups the
 * predicate's min / max statistics rule out are skipped (src/scan.c:12-105).
 * libvgpu nodes above it read each row group straight into page-locked
 * staging and copy it to the device asynchronously; other consumers get
 * malloc-owned batches as from src/vtr1.c:306-392.  col_indices: NULL = all
 * columns. */
ScanNode *scan_node_create(const char *path, int *col_indices, int n_selected);

/* replaces src/sort.h:31-32 (SortNode *sort_node_create): arrange() on the
 * GPU.  The node keeps the reference's SortNode prefix and kind, reads its
 * keys (col_index, descending) only when it runs, and returns every row of
 * the child stably sorted -- NA last ascending, first descending, ties in
 * input order (src/sort.c:32-116); strings in memcmp order, the shorter
 * first -- as one batch (an empty one for no rows), then NULL.  An input
 * larger than a third of the free device memory (or VGPU_SORT_RUN_ROWS
 * rows) is sorted in runs kept in host memory and merged back on the
 * device by key range; temp_dir is kept for the struct's sake (nothing is
 * written to disk).  Takes ownership of keys. */
SortNode *sort_node_create(VecNode *child, int n_keys, SortKey *keys, const char *temp_dir);

/* ---- data sources (no reference counterpart beyond ScanNode's role) -- */

#define VGPU_SRC_COPY    0   /* copy the host columns at creation          */
#define VGPU_SRC_BORROW  1   /* borrow host columns (caller keeps them)     */
#define VGPU_SRC_DEVICE  2   /* borrow device-resident columns              */
#define VGPU_SRC_MAPPED  4   /* borrow page-locked host columns that libvgpu
                                kernels read in place (cudaHostAlloc /
                                cudaHostRegister memory; over NVLink-C2C on
                                Grace systems) -- no staging copy            */

/* The largest batch a table source emits: row ids inside a batch are
 * int32, as the reference's selection vectors are (src/types.h:70-85). */
#define VGPU_MAX_BATCH_ROWS ((int64_t)2147483647)

/* A table as a source node, emitting batches of batch_rows rows (any count
 * from 1 to VGPU_MAX_BATCH_ROWS; 0 or less = the whole table, clamped to
 * VGPU_MAX_BATCH_ROWS; a larger value fails with NULL and vgpu_last_error).
 * Its kind string is "VgpuTableSource", not "ScanNode": the reference
 * optimizer reads a .vtr file header through every "ScanNode".  data[c]: n_rows int64 / double values or bool bytes;
 * validity[c]: the reference bitmap (bit i%8 of byte i/8), NULL = all
 * valid.  With VGPU_SRC_DEVICE both are device pointers and libvgpu nodes
 * read the batches in place; any other consumer gets host copies.  With
 * VGPU_SRC_BORROW from page-locked memory, libvgpu nodes copy each batch to
 * the device asynchronously.  With VGPU_SRC_MAPPED, data and validity must
 * be memory the device can address; each validity bitmap 4-byte aligned
 * and padded to whole 32-bit words (as for VGPU_SRC_DEVICE); creation fails
 * (NULL, vgpu_last_error) otherwise. */
VecNode *vgpu_table_source_create(int n_cols, const char *const *names,
                                  const int *types, const void *const *data,
                                  const uint8_t *const *validity,
                                  int64_t n_rows, int64_t batch_rows,
                                  int flags);

/* ---- runtime --------------------------------------------------------- */

int         vgpu_init(int device);          /* 0 on success */
const char *vgpu_last_error(void);
/* The CUDA stream (cudaStream_t) libvgpu launches on; NULL = its own. */
void        vgpu_set_stream(void *cuda_stream);
void       *vgpu_get_stream(void);
int         vgpu_synchronize(void);
/* Kernels launched by libvgpu since load. */
unsigned long long vgpu_kernel_launches(void);
/* Warnings the reference would raise through Rf_warning (all-NA min/max
 * with na.rm), counted since load. */
long        vgpu_warning_count(void);
/* Group-aggregations that took the partitioned path (many groups, one
 * int64 key, key-ordered output), counted since load.  The path is chosen
 * on the first input batch; environment: VGPU_PAGG=0 never, =1 whenever
 * the plan allows it, VGPU_PAGG_MIN_ROWS / VGPU_PAGG_MIN_GROUPS the
 * thresholds otherwise (4Mi rows, 256Ki estimated groups). */
unsigned long long vgpu_pagg_runs(void);
/* Fan-out (bucket count) and reducer shape of the partitioned path, tuned
 * per shape class (rows of the first batch, estimated groups, record
 * words, accumulators, each as a power of two).  With tuning on
 * (vgpu_pagg_tune(1), or VGPU_PAGG_TUNE=1), the first seven queries of a
 * shape class without a record run, one per query (each a complete,
 * correct query): the sketch's bucket count x1, x2, x4 with one reducer
 * CTA of 1024 threads per SM, x1 and x2 with two CTAs of 512 threads per
 * SM (each holding half the groups), x1 with four of 256 threads and x1
 * with eight of 128 (a quarter / an eighth each); they are timed by the
 * device
 * time of their partition and reducer launches, the fastest is kept for
 * the rest of the process and appended to the file named by
 * VGPU_TUNE_FILE, from which later processes read it.  vgpu_pagg_tuned:
 * the last decision -- its doublings over the sketch's count (-1: none
 * yet), shape class, reducer CTAs per SM and measured milliseconds. */
void        vgpu_pagg_tune(int on);
int         vgpu_pagg_tuned(char *shape, int shape_bytes, int *ctas, double *ms);

/* arrange() beyond device memory: sorted runs kept in host memory since
 * load (returned) and key ranges merged back on the device (*ranges).  A
 * sort spills when its input passes a share of the free device memory, or
 * VGPU_SORT_RUN_ROWS rows when that is set. */
long        vgpu_sort_spill_stats(long *ranges);
/* Host wall time (ms, summed since load) of the partitioned path's phases:
 * 0 sketch, 1 partition pass, 2 bucket reducer, 3 compaction into the
 * output columns, 4 waiting for the host result buffers, 5 copy to host,
 * 6 the whole next_batch call of the aggregation. */
double      vgpu_pagg_phase_ms(int phase);
/* The same for the hash-table aggregation path: 0 planning before the
 * first batch (join build included), 1 the join build alone, 2 the
 * aggregation launches and their synchronisations, 3 the result
 * (compaction, order, finish, copy to host), 4 the whole next_batch call.
 * The launches over a dense group cache are not waited for batch by batch:
 * their status is read back with the result's first read-back, so the
 * wait for them counts in 3. */
double      vgpu_agg_phase_ms(int phase);

/* Optional kernel timing: CUDA events recorded on the launching stream
 * around each kernel class (VGPU_PROF_*), read back in milliseconds. */
#define VGPU_PROF_AGG         0   /* fused filter / probe / group-agg kernel */
#define VGPU_PROF_FILTER      1   /* filter into a selection vector */
#define VGPU_PROF_JOIN_BUILD  2   /* hash-join build insert */
#define VGPU_PROF_JOIN_PROBE  3   /* hash-join probe count */
#define VGPU_PROF_FINISH      4   /* group results */
#define VGPU_PROF_PAGG        5   /* partitioned aggregation: bucket reducer */
void   vgpu_profile_enable(int on);
void   vgpu_profile_reset(void);
double vgpu_profile_ms(int kernel_class, unsigned long long *launches);

/* ---- diagnostics (no reference counterpart) ---------------------------- */
/* Bytes the device's default memory pool (where libvgpu allocates) has
 * handed out and not taken back, or -1: a failed call leaves it where it
 * was before the call. */
long long vgpu_device_bytes_in_use(void);
/* Fault injection: the n-th device allocation from now on fails (0: none);
 * also read once from the environment, VGPU_FAIL_ALLOC=n. */
void      vgpu_debug_fail_alloc(long n);
/* Runs the device's bounded wait on a word nothing changes for `limit`
 * polls: returns -1 with vgpu_last_error describing the expired wait (the
 * device stays usable), as any wait of a libvgpu kernel that runs out does. */
int       vgpu_wait_selftest(long long limit);

/* ---- guarded entry points for callers without an R error handler ----- */
/* Each returns NULL (and sets vgpu_last_error) where the unguarded call
 * would raise vectra_error. */
VecBatch     *vgpu_guard_next_batch(VecNode *node);
FilterNode   *vgpu_guard_filter(VecNode *child, VecExpr *predicate);
ProjectNode  *vgpu_guard_project(VecNode *child, int n, ProjEntry *entries);
GroupAggNode *vgpu_guard_group_agg(VecNode *child, int n_keys, char **key_names,
                                   int n_aggs, AggSpec *specs,
                                   const char *temp_dir);
ScanNode     *vgpu_guard_scan(const char *path, int *col_indices, int n_selected);
SortNode     *vgpu_guard_sort(VecNode *child, int n_keys, SortKey *keys, const char *temp_dir);
JoinNode     *vgpu_guard_join(VecNode *left, VecNode *right, JoinKind kind,
                              int n_keys, JoinKey *keys, const char *suffix_x,
                              const char *suffix_y);
void          vgpu_batch_free(VecBatch *batch);

/* ---- query sets: many small queries at once (no reference counterpart) */
/* Many small independent queries run together: a plan prepared once
 * captures persistent kernels over all of them in one CUDA graph, and
 * every run replays it.  Two kinds, on one int64 key column (no NA):
 *   VGPU_SET_GROUP  group_by(key) |> summarise(sum(value), mean(value),
 *                   n()): one output row per distinct key (table order, not
 *                   sorted), double sums correctly rounded;
 *   VGPU_SET_JOIN   inner_join over unique build keys: the (probe row,
 *                   build row) pairs in probe row order.
 * All pointers are device memory the caller keeps alive while the plan
 * exists; outputs are sized by the caller (group: max_groups rows, join: n
 * rows) and *out_rows receives the output row count. */
#define VGPU_SET_GROUP 0
#define VGPU_SET_JOIN  1
typedef struct {
    int32_t kind;
    int32_t pad;
    int64_t n;                  /* group rows / probe rows */
    const int64_t *key;         /* group keys / probe keys */
    const double *value;        /* group values */
    int64_t n_build;            /* join build rows */
    const int64_t *build_key;   /* join build keys (unique) */
    int64_t max_groups;         /* group: bound on distinct keys (output rows) */
    int64_t *out_key;           /* group outputs */
    double *out_sum;
    double *out_mean;
    int64_t *out_n;
    int32_t *out_probe;         /* join outputs */
    int32_t *out_build;
    int64_t *out_rows;          /* output row count (device) */
} VgpuSetQuery;
/* 0 on success (*plan set), -1 with vgpu_last_error set. */
int  vgpu_queryset_prepare(const VgpuSetQuery *queries, int n_queries, void **plan);
/* Runs every query of the plan and waits: 0, or -1 (a table or output too
 * small, repeated build keys) with vgpu_last_error set. */
int  vgpu_queryset_run(void *plan);
void vgpu_queryset_free(void *plan);
/* Autotuning of a set's launch parameters: every candidate (threads per
 * CTA 256 / 512 / 1024, rows per work item 16Ki / 64Ki / 256Ki, table load
 * <= 1/2 or 1/4) is prepared and timed on the set itself (best of `reps`
 * runs after a warm-up; outputs are rewritten), and the fastest is
 * recorded for the set's shape (instance counts per kind, total and
 * largest instance rows, mean group cardinality, each as a power of two).
 * vgpu_queryset_prepare then uses the recorded parameters for any set of
 * that shape.  VGPU_TUNE_FILE names a file that keeps the records across
 * processes.  vgpu_queryset_tuning: 1 and the record for the set's shape,
 * or 0 and the defaults. */
typedef struct {
    int32_t threads;            /* per CTA */
    int32_t table_mult;         /* table capacity >= table_mult x keys */
    int64_t chunk_rows;         /* rows per work item */
    double  ms;                 /* measured time of one run (0: defaults) */
    int32_t candidates;         /* configurations timed */
    char    shape[60];
} VgpuSetTuning;
int  vgpu_queryset_tune(const VgpuSetQuery *queries, int n_queries, int reps, VgpuSetTuning *out);
int  vgpu_queryset_tuning(const VgpuSetQuery *queries, int n_queries, VgpuSetTuning *out);
/* vgpu_queryset_prepare with explicit launch parameters (threads,
 * chunk_rows, table_mult of `params`; NULL: the defaults 512, 64Ki, 2). */
int  vgpu_queryset_prepare_with(const VgpuSetQuery *queries, int n_queries, const VgpuSetTuning *params,
                                void **plan);

/* ---- serving loop over resident tables (no reference counterpart) ---- */
/* A server keeps tables resident (device pointers the caller keeps alive)
 * and runs requests as they arrive: vgpu_server_poll admits queued
 * requests in arrival order while their estimated memory fits the budget,
 * launches the admitted ones as one wave on a free stream (waves on
 * different streams overlap) and retires finished waves.  Kinds:
 *   VGPU_SERVE_FILTER_SUM  rows with a valid val > threshold: count, exact sum
 *   VGPU_SERVE_GROUP_SUM   group_by(key) |> summarise(sum(val, na.rm = TRUE),
 *                          n()): NA keys form one group
 *   VGPU_SERVE_SEMI / ANTI rows of `table` whose key has / has no match in
 *                          `build_table` (NA keys never match), ascending
 * Bitmaps use the reference layout, 4-byte aligned, padded to 32-bit words;
 * NULL means all valid.  Results stay valid until vgpu_server_release. */
#define VGPU_SERVE_FILTER_SUM 0
#define VGPU_SERVE_GROUP_SUM  1
#define VGPU_SERVE_SEMI       2
#define VGPU_SERVE_ANTI       3
typedef struct {
    int32_t kind;
    int32_t table;
    int32_t build_table;
    int32_t pad;
    double  threshold;
} VgpuServeQuery;
typedef struct {
    int64_t rows;                 /* filter: rows kept; group: groups; semi / anti: rows */
    double  sum;                  /* filter: exact sum */
    const int64_t *key;           /* group (device): keys ... */
    const uint8_t *key_valid;     /* ... 0 for the NA group ... */
    const double  *group_sum;     /* ... exact sums ... */
    const int64_t *group_n;       /* ... n() */
    const int32_t *sel;           /* semi / anti (device): selected rows */
} VgpuServeResult;
void   *vgpu_server_create(int n_streams, int64_t budget_bytes);
int     vgpu_server_add_table(void *server, const int64_t *key, const uint8_t *key_valid,
                              const double *val, const uint8_t *val_valid, int64_t n);
int64_t vgpu_server_submit(void *server, const VgpuServeQuery *query);   /* request id, or -1 */
int     vgpu_server_poll(void *server);          /* requests not yet done, or -1 */
int     vgpu_server_done(void *server, int64_t id);
int     vgpu_server_result(void *server, int64_t id, VgpuServeResult *result);
void    vgpu_server_release(void *server, int64_t id);
/* Withdraws a request still waiting for admission (submitted, not yet
 * admitted by a poll): 0, its id is then unknown to the server; -1 if it
 * is unknown or already admitted (release it once done).  A request whose
 * estimate alone exceeds the budget is refused at submit (-1). */
int     vgpu_server_cancel(void *server, int64_t id);
/* Builds a table's key set now (it is built at the first request that
 * needs it otherwise): 0 or -1. */
int     vgpu_server_warm(void *server, int table);
void    vgpu_server_free(void *server);
/* Copies bytes of device memory (a result) to host memory; 0 or -1. */
int     vgpu_copy_to_host(void *dst_host, const void *src_device, int64_t bytes);

/* ---- allocation-free filter (no counterpart in the reference) -------- */
/* For callers that may not allocate device memory during a query: a host
 * whose device memory is fully reserved by another framework's pool, a
 * latency-bound serving loop that must never wait on the allocator, or an
 * embedding with a fixed memory budget.  Every other entry point allocates
 * its working space (stream-ordered, from the device's default pool).
 *
 * Writes the ascending indices of the rows of n_rows device-resident rows
 * that satisfy `predicate` (filter_node_create's semantics: NA and NaN
 * comparisons drop the row) to d_sel_out (device, room for n_rows int32),
 * and their number to *n_selected.  d_data[c]: device int64 / double
 * values or bool bytes; d_validity[c]: device bitmap in the reference
 * layout, 4-byte aligned and padded to whole 32-bit words, NULL = all valid
 * (d_validity itself may be NULL).  Runs on the vgpu_set_stream stream if
 * one is set, else libvgpu's own stream if the library is initialised,
 * else the legacy default stream, and synchronises that stream before it
 * returns.  Returns 0, or -1 with vgpu_last_error set: more than
 * VGPU_STATIC_MAX_ROWS rows, more than 24 columns, a string column or an
 * unsupported predicate.  If the library's own stream belongs to another
 * device than the current one (vgpu_init chose a device, the caller has
 * since switched), the call runs on the current device's legacy default
 * stream instead.
 *
 * Working space is one fixed device array of 1 MiB + 64 KiB compiled into
 * libvgpu; nothing in it needs to be zero beforehand (each call writes
 * what it reads).  Because that array is shared, calls must not overlap:
 * two calls at once, from two threads or on two streams, race on it.  The
 * first call on each device looks up the array's address
 * (cudaGetSymbolAddress), and its first launches load the filter kernels'
 * module (CUDA loads modules lazily by default), which takes a little
 * device memory once: make one call on each device as a warm-up before a
 * memory budget is fixed or a stream is captured. */
#define VGPU_STATIC_MAX_ROWS 8388608LL
int vgpu_filter_select_static(int n_cols, const char *const *names,
                              const int *types, const void *const *d_data,
                              const void *const *d_validity, int64_t n_rows,
                              const VecExpr *predicate, int32_t *d_sel_out,
                              int64_t *n_selected);

#ifdef __cplusplus
}
#endif

#endif /* VGPU_H */
