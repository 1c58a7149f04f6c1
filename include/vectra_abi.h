/*
 * vectra_abi.h -- the data and node contract that vectra's C engine uses
 * between plan nodes, restated so that libvgpu can be compiled without the
 * reference sources.  Every type here is layout-identical to its counterpart
 * in gcol33/vectra (checked by oracle/abi_check.c against the reference
 * headers):
 *
 *   VecType, VecArray, VecBatch, VecSchema, VecNode   src/types.h:7-104
 *   VecExprKind, VecExpr                               src/expr.h:6-63
 *   AggKind                                            src/agg_ops.h:7-14
 *   AggSpec, GroupAggNode (prefix)                     src/group_agg.h:7-23
 *   JoinKind, JoinKey, JoinNode (prefix)               src/join.h:6-56
 *   FilterNode                                         src/filter.h:7-11
 *   ProjEntry, ProjectNode                             src/project.h:7-18
 *
 * Memory rules of the contract (src/batch.c:19-29, src/array.c:41-58):
 * every buffer reachable from a VecBatch handed across a node boundary is
 * plain malloc memory and is released with free() by the consumer.
 *
 * If the reference's own types.h has already been included, its definitions
 * are used and the duplicates below are skipped.
 */
#ifndef VGPU_VECTRA_ABI_H
#define VGPU_VECTRA_ABI_H

#ifdef __CUDACC_RTC__
#include "vg_rtc_types.h"   /* run-time compiled device code: no libc headers */
#else
#include <stdint.h>
#include <stdio.h>
#include <stddef.h>
#endif

#ifdef __cplusplus
extern "C" {
#endif

#ifndef VECTRA_TYPES_H
#define VECTRA_TYPES_H

typedef enum {
    VEC_INT64  = 0,
    VEC_DOUBLE = 1,
    VEC_BOOL   = 2,
    VEC_STRING = 3
} VecType;

/* One column.  validity: bit i%8 of byte i/8 set = row i is valid (not NA). */
typedef struct {
    VecType   type;
    int64_t   length;
    uint8_t  *validity;
    uint8_t   owns_data;          /* only meaningful for VEC_STRING */
    union {
        int64_t  *i64;
        double   *dbl;
        uint8_t  *bln;            /* one byte per row, 0/1 */
        struct {
            int64_t *offsets;     /* length+1 entries */
            char    *data;
            int64_t  data_len;
        } str;
    } buf;
} VecArray;

/* A batch of rows.  If sel is non-NULL the logical rows are the physical
 * row ids sel[0..sel_n). */
typedef struct {
    int64_t    n_rows;
    int        n_cols;
    char     **col_names;
    VecArray  *columns;
    int32_t   *sel;
    int32_t    sel_n;
} VecBatch;

typedef struct {
    int       n_cols;
    char    **col_names;
    VecType  *col_types;
    char    **col_annotations;
} VecSchema;

typedef struct VecNode VecNode;
typedef VecBatch* (*NextBatchFn)(VecNode *self);
typedef void      (*FreeFn)(VecNode *self);

/* Pull-based plan node: next_batch returns an owned batch or NULL at end of
 * stream (and keeps returning NULL afterwards); free_node frees the node and
 * its children. */
struct VecNode {
    NextBatchFn   next_batch;
    FreeFn        free_node;
    VecSchema     output_schema;
    const char   *kind;
};

#endif /* VECTRA_TYPES_H */

#ifndef VECTRA_EXPR_H
#define VECTRA_EXPR_H

typedef enum {
    EXPR_COL_REF,
    EXPR_LIT_INT64,
    EXPR_LIT_DOUBLE,
    EXPR_LIT_BOOL,
    EXPR_LIT_STRING,
    EXPR_LIT_NA,
    EXPR_ARITH,
    EXPR_CMP,
    EXPR_BOOL,
    EXPR_IS_NA,
    EXPR_IF_ELSE,
    EXPR_CAST,
    EXPR_NEGATE,
    EXPR_NCHAR,
    EXPR_SUBSTR,
    EXPR_GREPL
} VecExprKind;

typedef struct VecExpr VecExpr;

/* Expression tree node.  op/op2 encode the operator: arith '+','-','*','/',
 * '%'; compare ('=','='), ('!','='), ('<',' '), ('<','='), ('>',' '),
 * ('>','='); bool '&', '|', '!' (unary, uses operand). */
struct VecExpr {
    VecExprKind kind;
    VecType     result_type;
    char       *col_name;
    int64_t     lit_i64;
    double      lit_dbl;
    uint8_t     lit_bln;
    char       *lit_str;
    char        op;
    char        op2;
    VecExpr    *left;
    VecExpr    *right;
    VecExpr    *operand;
    VecExpr    *cond;
    VecExpr    *then_expr;
    VecExpr    *else_expr;
    VecType     cast_to;
};

#endif /* VECTRA_EXPR_H */

#ifndef VECTRA_AGG_OPS_H
#define VECTRA_AGG_OPS_H
typedef enum {
    AGG_COUNT,        /* count of non-NA values */
    AGG_COUNT_STAR,   /* n(): count of all rows */
    AGG_SUM,
    AGG_MEAN,
    AGG_MIN,
    AGG_MAX
} AggKind;
#endif

#ifndef VECTRA_GROUP_AGG_H
#define VECTRA_GROUP_AGG_H
typedef struct {
    char    *output_name;
    AggKind  kind;
    char    *input_col;     /* NULL for AGG_COUNT_STAR */
    int      na_rm;
} AggSpec;

/* Fields read by the reference optimizer and explain() through casts
 * (src/optimize.c:243-259, src/r_bridge.c:540-543). */
typedef struct {
    VecNode     base;
    VecNode    *child;
    int         n_keys;
    char      **key_names;
    int         n_aggs;
    AggSpec    *agg_specs;
    int         done;
    int         use_sorted;
} GroupAggNode;
#endif

#ifndef VECTRA_JOIN_H
#define VECTRA_JOIN_H
typedef enum {
    JOIN_INNER,
    JOIN_LEFT,
    JOIN_FULL,
    JOIN_SEMI,
    JOIN_ANTI
} JoinKind;

typedef struct {
    int   left_col;
    int   right_col;
} JoinKey;

/* Prefix read by the reference optimizer and explain()
 * (src/optimize.c:313-333, src/r_bridge.c:552-557). */
typedef struct {
    VecNode   base;
    VecNode  *left;
    VecNode  *right;
    JoinKind  kind;
    int       n_keys;
    JoinKey  *keys;
    char     *suffix_x;
    char     *suffix_y;
} JoinNodePrefix;
typedef JoinNodePrefix JoinNode;
#endif

#ifndef VECTRA_FILTER_H
#define VECTRA_FILTER_H
/* Read by the optimizer's pruning and predicate pushdown
 * (src/optimize.c:102-125, 356-371), which borrows `predicate`. */
typedef struct {
    VecNode   base;
    VecNode  *child;
    VecExpr  *predicate;
} FilterNode;
#endif

#ifndef VECTRA_PROJECT_H
#define VECTRA_PROJECT_H
typedef struct {
    char    *output_name;
    VecExpr *expr;          /* NULL: pass the column named output_name through */
} ProjEntry;

typedef struct {
    VecNode     base;
    VecNode    *child;
    int         n_entries;
    ProjEntry  *entries;
} ProjectNode;
#endif

#ifndef VECTRA_SORT_H
#define VECTRA_SORT_H
/* src/sort.h:6-26: read by the optimizer, which re-points col_index after
 * pruning the child (src/optimize.c:141-178). */
typedef struct {
    int   col_index;
    int   descending;   /* 1 = DESC, 0 = ASC */
} SortKey;

typedef struct {
    VecNode   base;
    VecNode  *child;
    int       n_keys;
    SortKey  *keys;
    int       phase;
    int64_t   mem_budget;
    char     *temp_dir;
    int       n_runs;
    int       runs_cap;
    char    **run_paths;
    VecBatch *mem_result;
    void     *merge;
} SortNode;
#endif

#ifndef __CUDACC_RTC__   /* host-only: the file handle holds a FILE * */
#ifndef VECTRA_VTR1_H
#define VECTRA_VTR1_H
/* .vtr file handle (src/vtr1.h): read by the optimizer's pruning and
 * pushdown through ScanNode->file (src/optimize.c:38-41, 360-363). */
typedef struct {
    uint16_t  version;
    VecSchema schema;
    uint32_t  n_rowgroups;
} Vtr1Header;

/* per-column per-row-group min / max (version 3) */
typedef struct {
    uint8_t has_stats;
    union {
        struct { int64_t min, max; } i64;
        struct { double min, max; } dbl;
        struct { uint8_t min, max; } bln;
    };
} Vtr1ColStat;

typedef struct {
    int64_t      file_offset;
    int64_t      n_rows;
    Vtr1ColStat *col_stats;     /* n_cols entries; NULL before version 3 */
} Vtr1RowGroup;

typedef struct {
    FILE         *fp;
    Vtr1Header    header;
    Vtr1RowGroup *rowgroups;
} Vtr1File;
#endif

#ifndef VECTRA_SCAN_H
#define VECTRA_SCAN_H
/* Read by the optimizer (src/optimize.c:38-77 prunes col_mask and the
 * output schema; 356-371 attaches a FilterNode's predicate, borrowed). */
typedef struct {
    VecNode    base;
    Vtr1File  *file;
    int       *col_mask;        /* file columns read */
    uint32_t   next_rg;
    VecExpr   *predicate;       /* pushed-down predicate, NULL = none */
    int        pred_borrowed;   /* 1: owned by the filter node */
} ScanNode;
#endif
#endif /* __CUDACC_RTC__ */

#ifdef __cplusplus
}
#endif

#endif /* VGPU_VECTRA_ABI_H */
