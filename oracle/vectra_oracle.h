/*
 * vectra_oracle.h -- CPU restatement of gcol33/vectra's filter / project /
 * group-agg / join path, used as the correctness oracle for libvgpu and as
 * the timed CPU baseline where the reference engine itself cannot be built.
 *
 * TEST INFRASTRUCTURE ONLY: only tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py load it.  The product (libvgpu) never does.
 *
 * The node constructors take and return the reference's own node contract
 * (include/vectra_abi.h), with the same ownership rules, so the same Python
 * plan builder drives the reference library, this port and libvgpu.
 */
#ifndef VGPU_VECTRA_ORACLE_H
#define VGPU_VECTRA_ORACLE_H

#include "vectra_abi.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Error reporting: every error longjmps to the innermost orc_guard_* frame,
 * which returns NULL; the message is in orc_last_error(). */
const char *orc_last_error(void);
long        orc_warning_count(void);
void        orc_reset(void);

/* 1 (default): reproduce the reference's chain walk for LEFT/FULL joins,
 * which compares the uncoerced probe key column (src/join.c:408-410).
 * 0: compare the coerced key, i.e. what INNER joins do (src/join.c:392-394). */
void        orc_set_join_quirk(int on);

/* In-memory source node: emits the table in batches of batch_rows rows as
 * malloc-owned deep copies (what ScanNode does per row group,
 * src/scan.c:107-127).  sel_mode 0: no selection vector; 1: every batch
 * carries sel = the even physical rows (exercises sel composition).
 * data[c] points at n_rows values (int64/double/uint8) or, for strings, at
 * an int64 offsets array of n_rows+1 entries with str_data[c] the bytes.
 * validity[c] may be NULL (all valid).  The node copies everything it needs. */
VecNode *orc_table_source_create(int n_cols, const char *const *names,
                                 const int *types, const void *const *data,
                                 const char *const *str_data,
                                 const uint8_t *const *validity,
                                 int64_t n_rows, int64_t batch_rows,
                                 int sel_mode);

VecNode *orc_filter_node_create(VecNode *child, VecExpr *predicate);
VecNode *orc_project_node_create(VecNode *child, int n_entries,
                                 ProjEntry *entries);
/* temp_dir != NULL and n_keys > 0 selects the sort-based path (ascending
 * keys, NA last), as the R front end always does (src/r_bridge.c:990,
 * src/group_agg.c:625-638); otherwise the hash path (first-seen order). */
VecNode *orc_group_agg_node_create(VecNode *child, int n_keys,
                                   char **key_names, int n_aggs,
                                   AggSpec *agg_specs, const char *temp_dir);
/* arrange(): every logical row, stably sorted by the keys, as one batch
 * (the in-memory path of src/sort.c). */
VecNode *orc_sort_node_create(VecNode *child, int n_keys, SortKey *keys, const char *temp_dir);
VecNode *orc_guard_sort(VecNode *child, int n_keys, SortKey *keys, const char *temp_dir);
VecNode *orc_join_node_create(VecNode *left, VecNode *right, JoinKind kind,
                              int n_keys, JoinKey *keys,
                              const char *suffix_x, const char *suffix_y);

/* Guarded entry points (setjmp frames). */
VecBatch *orc_guard_next_batch(VecNode *n);
VecNode  *orc_guard_filter(VecNode *child, VecExpr *pred);
VecNode  *orc_guard_project(VecNode *child, int n, ProjEntry *entries);
VecNode  *orc_guard_group_agg(VecNode *child, int n_keys, char **key_names,
                              int n_aggs, AggSpec *specs, const char *temp_dir);
VecNode  *orc_guard_join(VecNode *l, VecNode *r, JoinKind kind, int n_keys,
                         JoinKey *keys, const char *sx, const char *sy);

void orc_batch_free(VecBatch *b);

/* Exactly rounded sum of n doubles (Shewchuk's adaptive expansion
 * arithmetic, as in Python's math.fsum).  Non-finite inputs follow IEEE. */
double orc_exact_sum(const double *x, int64_t n);

/* Exactly rounded sum of fl(a[i]*b[i]) (each product rounded once). */
double orc_exact_sum_products(const double *a, const double *b, int64_t n);

#ifdef __cplusplus
}
#endif

#endif
