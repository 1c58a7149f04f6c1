/*
 * Host shim linked into oracle/_ref/libvectra_ref.so (the reference vectra
 * engine compiled from its own C sources).  TEST INFRASTRUCTURE ONLY.
 *
 *  - Rf_error: the reference reports every error through vectra_error ->
 *    Rf_error (src/error.c:4-11), which in R never returns (longjmp).  Here
 *    it longjmps to the innermost vref_guard_* frame, which returns NULL and
 *    leaves the message in vref_last_error().
 *  - Rf_warning: counted (src/agg_ops.c:219,239 warn on all-NA min/max).
 *  - vref_guard_*: setjmp frames around the reference entry points that the
 *    Python test harness calls through ctypes, so a reference error never
 *    unwinds through Python frames.
 */
#include <setjmp.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "types.h"
#include "expr.h"
#include "filter.h"
#include "group_agg.h"
#include "join.h"
#include "project.h"
#include "scan.h"
#include "sort.h"

static jmp_buf *g_jmp = NULL;
static char g_msg[1024];
static long g_warnings = 0;

void Rf_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_msg, sizeof(g_msg), fmt, ap);
    va_end(ap);
    if (g_jmp) longjmp(*g_jmp, 1);
    fprintf(stderr, "vectra reference error outside a guard: %s\n", g_msg);
    abort();
}

void Rf_warning(const char *fmt, ...) {
    (void)fmt;
    g_warnings++;
}

const char *vref_last_error(void) { return g_msg; }
long vref_warning_count(void) { return g_warnings; }
void vref_reset(void) { g_msg[0] = 0; g_warnings = 0; }

#define GUARD_BEGIN                        \
    jmp_buf jb; jmp_buf *prev = g_jmp;     \
    g_msg[0] = 0;                          \
    if (setjmp(jb)) { g_jmp = prev; return NULL; } \
    g_jmp = &jb;
#define GUARD_END g_jmp = prev;

VecBatch *vref_guard_next_batch(VecNode *n) {
    GUARD_BEGIN
    VecBatch *b = n->next_batch(n);
    GUARD_END
    return b;
}

FilterNode *vref_guard_filter(VecNode *child, VecExpr *pred) {
    GUARD_BEGIN
    FilterNode *r = filter_node_create(child, pred);
    GUARD_END
    return r;
}

GroupAggNode *vref_guard_group_agg(VecNode *child, int n_keys, char **key_names,
                                   int n_aggs, AggSpec *specs,
                                   const char *temp_dir) {
    GUARD_BEGIN
    GroupAggNode *r = group_agg_node_create(child, n_keys, key_names, n_aggs,
                                            specs, temp_dir);
    GUARD_END
    return r;
}

JoinNode *vref_guard_join(VecNode *l, VecNode *r, JoinKind kind, int n_keys,
                          JoinKey *keys, const char *sx, const char *sy) {
    GUARD_BEGIN
    JoinNode *j = join_node_create(l, r, kind, n_keys, keys, sx, sy);
    GUARD_END
    return j;
}

SortNode *vref_guard_sort(VecNode *child, int n_keys, SortKey *keys, const char *temp_dir) {
    GUARD_BEGIN
    SortNode *r = sort_node_create(child, n_keys, keys, temp_dir);
    GUARD_END
    return r;
}

ScanNode *vref_guard_scan(const char *path, int *col_indices, int n_selected) {
    GUARD_BEGIN
    ScanNode *r = scan_node_create(path, col_indices, n_selected);
    GUARD_END
    return r;
}

ProjectNode *vref_guard_project(VecNode *child, int n, ProjEntry *entries) {
    GUARD_BEGIN
    ProjectNode *p = project_node_create(child, n, entries);
    GUARD_END
    return p;
}
