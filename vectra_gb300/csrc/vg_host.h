/*
 * vg_host.h -- internal declarations of libvgpu's C11 host layer.
 */
#ifndef VG_HOST_H
#define VG_HOST_H

#include <stdint.h>
#include <stddef.h>
#include "vgpu.h"
#include "vgpu_internal.h"

/* ---- errors ---- */
/* Records the message and raises it through vectra_error (no return). */
void vg_fail(const char *fmt, ...);
void vg_warn_count(long n);
/* Records a message for vgpu_last_error() without raising. */
void vg_set_error(const char *fmt, ...);
/* Fails with the last kernel-side message if rc != 0. */
void vg_check_rc(int rc, const char *what);

/* ---- device memory / stream ---- */
void vg_ensure_init(void);
vg_stream_t vg_stream(void);
vg_stream_t vg_stream_noinit(void);
void *vg_dmalloc(size_t bytes);          /* stream-ordered, fails loudly; a temporary of the current call */
void *vg_dmalloc_kept(size_t bytes);     /* the same, for state a node keeps across calls */
void vg_dkeep(void *p);                  /* a temporary becomes state a node keeps */
void vg_dfree(void *p);
/* The node API call scope: temporaries still allocated when a call fails
 * are released before the error is raised. */
void vg_scope_enter(void);
void vg_scope_leave(void);
void vg_h2d(void *dst, const void *src, size_t bytes);
void vg_d2h(void *dst, const void *src, size_t bytes);
void vg_dmemset(void *dst, int v, size_t bytes);
void vg_sync(void);
/* A page-locked host buffer of at least `bytes` for small read-backs:
 * copies into it do not wait, so several go out before one vg_sync().
 * Kept for the process; a larger request replaces it (after a sync), so
 * a caller reads what it copied before asking again. */
void *vg_pinned_scratch(size_t bytes);
uint32_t *vg_pinned_status(void);

/* ---- host batches ---- */
void *vg_xmalloc(size_t n);
void *vg_xcalloc(size_t n, size_t s);
char *vg_xstrdup(const char *s);
VecBatch *vg_batch_alloc(int n_cols, int64_t n_rows);
void vg_batch_free(VecBatch *b);
VecSchema vg_schema_make(int n, char *const *names, const VecType *types);
VecSchema vg_schema_copy(const VecSchema *s);
void vg_schema_free(VecSchema *s);
int vg_schema_find(const VecSchema *s, const char *name);
static inline int64_t vg_vbytes(int64_t n) { return (n + 7) / 8; }

/* ---- device batches ---- */
/* A batch whose needed columns are resident on the device. */
typedef struct {
    int64_t n_rows;            /* physical rows */
    int n_cols;
    VgCol *cols;               /* n_cols entries; data == NULL if not present */
    const int32_t *d_sel;      /* device selection vector or NULL */
    int64_t sel_n;
    VecBatch *host;            /* the host batch it came from (owned) or NULL */
    void *block;               /* device allocation holding uploaded data */
    int64_t row_base;          /* stream position of physical row 0 */
    int in_host;               /* columns are page-locked host memory read in place */
    int64_t *str_chars;        /* n_cols: bytes of characters of each string column (or NULL) */
} VgDBatch;

/* Pulls the next batch of `child` with the columns flagged in need[]
 * resident on the device.  Returns 0 at end of stream.  keep_host: keep the
 * host batch in out->host (otherwise it is freed after the upload). */
int vg_pull(VecNode *child, const uint8_t *need, int keep_host, VgDBatch *out);
void vg_dbatch_release(VgDBatch *b);

/* Device column -> newly malloc'd host VecArray of n values. */
VecArray vg_download_column(int type, const void *d_data, const uint32_t *d_valid, int64_t n);
/* Rows [lo, lo + n) of a host column on the device (one new block *blk). */
VgCol vg_upload_slice(const VecArray *a, int64_t lo, int64_t n, void **blk);
/* Device string column (views) -> host VecArray of rows d_idx[j] (or j). */
VecArray vg_download_strings(const VgCol *c, const int32_t *d_idx, int64_t n);
VecArray vg_host_column(int type, int64_t n, void *values, const uint32_t *d_valid);
/* Newly malloc'd host VecArray of n values copied from host memory (values
 * of value_bytes(type, n), validity as the device's 32-bit words). */
VecArray vg_column_from_host(int type, const void *values, const void *valid, int64_t n);
void vg_copy_after_main(void);
void vg_d2h_copy(void *dst, const void *src, size_t bytes);
void vg_copy_sync(void);
/* n host buffers of `bytes` each, faulted in by background threads */
/* kernel timing (k_prof.cu): classes 0 the aggregation kernel, 5 the
 * partitioned path's bucket reducer */
int vg_prof_force_on(void);
void vg_prof_restore(int prev);
double vgpu_profile_ms(int cls, unsigned long long *launches);
#define VG_PROF_CLASS_AGG 0
#define VG_PROF_CLASS_PAGG 5

typedef struct VgHostBufs VgHostBufs;
VgHostBufs *vg_host_bufs_begin(int n, size_t bytes);
void vg_host_bufs_wait(VgHostBufs *h);
void vg_host_bufs_wait_upto(VgHostBufs *h, size_t bytes);   /* the first `bytes` of every buffer */
void *vg_host_bufs_take(VgHostBufs *h, int b, size_t need);   /* NULL: too small or taken */
void vg_host_bufs_free(VgHostBufs *h);

/* ---- string dictionaries (strdict.c) ---- */
typedef struct VgDict VgDict;
VgDict *vg_dict_new(void);
VgDict *vg_dict_new_kept(void);
void vg_dict_free(VgDict *D);
/* d_codes[p] for the logical rows p of string column c (insert: new
 * strings get the next codes; otherwise absent strings get -1).
 * chars_ub: an upper bound of the characters of those rows when the
 * caller knows one (then room is made without reading the device's
 * counters back), else -1. */
void vg_dict_encode(VgDict *D, const VgCol *c, const int32_t *d_sel, int64_t n_logical, int insert,
                    int64_t *d_codes, int64_t chars_ub);
int64_t vg_dict_size(VgDict *D);
const VgStrDict *vg_dict_device(VgDict *D);
void vg_dict_order(VgDict *D, int32_t **d_perm, int64_t **d_rank);
VecArray vg_dict_strings(VgDict *D, const int64_t *d_codes, const uint32_t *d_valid, const int32_t *d_perm,
                         int64_t n);

/* ---- .vtr scan (scan_vtr.c) ---- */
int vg_is_vtr_scan(const VecNode *n);
int vg_scan_pull(VecNode *n, const uint8_t *need, VgDBatch *out);

/* ---- table source (source.c) ---- */
int vg_is_table_source(const VecNode *n);
int vg_source_pull(VecNode *n, const uint8_t *need, VgDBatch *out);

/* ---- expression compilation (compile.c) ---- */
/* Column lookup: returns the index of `name` in the launch's column table
 * (uploading it on demand) or -1 if unknown. */
typedef int (*vg_colmap_fn)(void *ctx, const char *name, int *type);
/* 1 if expr is a conjunction of column-vs-constant terms (filled into out),
 * 0 if it needs the general program, -1 on error (message set). */
int vg_compile_pred(const VecExpr *e, vg_colmap_fn map, void *ctx, VgPred *out);
/* general program; returns 0 or -1 (message set) */
int vg_compile_prog(const VecExpr *e, vg_colmap_fn map, void *ctx, VgProg *out);
/* a value for fused kernels: a column, a literal, or a binary arithmetic of
 * those; returns 1 if representable, 0 if not, -1 on error. */
int vg_compile_value(const VecExpr *e, vg_colmap_fn map, void *ctx, int side, VgValue *out);
const char *vg_compile_error(void);
/* reference type of an expression (src/r_bridge.c parse rules) */
int vg_expr_type(const VecExpr *e);
/* frees an expression tree allocated with malloc (src/expr.c:16-27) */
void vg_expr_free(VecExpr *e);
/* 1 if the expression mentions column `name` */
int vg_expr_refs(const VecExpr *e, const char *name);

/* ---- compact column tables for kernels (at most VG_MAX_COLS) ---- */
typedef struct { int n; int idx[VG_MAX_COLS]; } VgColSet;
/* index of column i in the set, adding it if new; -1 if the set is full */
static inline int vg_colset_add(VgColSet *s, int i) {
    for (int j = 0; j < s->n; j++) if (s->idx[j] == i) return j;
    if (s->n >= VG_MAX_COLS) return -1;
    s->idx[s->n] = i;
    return s->n++;
}

/* ---- node identification ---- */
int vg_is_filter(const VecNode *n);
int vg_is_project(const VecNode *n);
int vg_is_join(const VecNode *n);

/* filter internals used by fusion */
const VgPred *vg_filter_cnf(VecNode *n, VecNode **child_out, const VgColSet **set);
const VgProg *vg_filter_program(VecNode *n, VecNode **child_out, const VgColSet **set);
/* project internals: the expression producing column `name`, or NULL if it
 * is a pass-through (then *pass_name is the child column name) */
int vg_project_lookup(VecNode *n, const char *name, const VecExpr **expr, const char **pass_name);
VecNode *vg_project_child(VecNode *n);

/* join internals used by the fused aggregation */
typedef struct {
    VgJoinTable jt;
    int n_keys;
    int32_t lkey[VG_MAX_KEYS];       /* probe-side key columns */
    int32_t rkey[VG_MAX_KEYS];       /* build-side key columns (index into bcols) */
    int32_t conv[VG_MAX_KEYS];       /* probe key int/bool -> double */
    VgCol *bcols;                    /* device build columns (all right columns) */
    int n_bcols;
    int kind;
    /* payload copy columns (right column indices) and, when pay_mm_ok, the
     * min / max / count of their valid values for int64 columns */
    int pay_n;
    int32_t pay_col[2];
    int pay_mm_ok;
    int64_t pay_mm[6];
    /* the payload copy's entries: -2 VgJPay; -1 VgJPay16 of one column;
     * 0 / 1 VgJPay16 narrowing that payload column (minimum pay_min) */
    int pay_layout;
    int64_t pay_min;
} VgJoinBuilt;
const VgJoinBuilt *vg_join_build_now(VecNode *n);
/* builds with a payload copy of right columns cols[0..n_cols) (n_cols <= 2);
 * *pay = the copy, or NULL when it does not apply (duplicate or composite
 * keys, table already built) */
const VgJoinBuilt *vg_join_build_payload(VecNode *n, const int32_t *cols, int n_cols, const VgJPay **pay);
int vg_join_right_type(VecNode *n, int col);
/* the join table's slots, filled (a build with a payload copy defers them) */
void vg_join_ensure_slots(VecNode *n);
VecNode *vg_join_left(VecNode *n);
int vg_join_kind(VecNode *n);
int vg_join_has_string_keys(VecNode *n);
/* resolves an output column name of the join: side 0 = left column index,
 * side 1 = right column index; returns 0 if not found */
int vg_join_resolve(VecNode *n, const char *name, int *side, int *col);

#endif
