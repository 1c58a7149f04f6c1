/*
 * node_filter.c -- FilterNode on the GPU (replaces src/filter.c).
 *
 * next_batch pulls a host batch from the child, moves only the columns the
 * predicate reads to the device, computes the selection vector there and
 * returns the same batch with its `sel` replaced (composed with any sel the
 * batch already had), exactly as apply_mask_sel does (src/filter.c:13-39).
 * Batches left empty are dropped (src/filter.c:56-60).
 *
 * A group-agg node directly above this node does not call next_batch: it
 * reads the compiled predicate (vg_filter_cnf) and evaluates it inside its
 * own kernel, so the selection vector never exists; or, for a general
 * program (vg_filter_program), runs this node's filter kernels on the
 * batch it already holds on the device and keeps the selection there.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "vg_host.h"

typedef struct {
    FilterNode fn;            /* reference prefix: base, child, predicate */
    int compiled;             /* 0 not yet, 1 CNF, 2 program */
    VgPred pred;
    VgProg prog;
    uint8_t *need;            /* child columns the predicate reads */
    VgColSet set;             /* kernel column table -> child column */
    char err[512];            /* deferred compile error (raised at next_batch) */
} VgFilter;

static VecBatch *filter_next(VecNode *self);
static void filter_free(VecNode *self);

int vg_is_filter(const VecNode *n) { return n && n->next_batch == filter_next; }

typedef struct { const VecSchema *s; uint8_t *need; VgColSet *set; } MapCtx;

static int map_schema(void *ctx, const char *name, int *type) {
    MapCtx *m = (MapCtx *)ctx;
    int i = vg_schema_find(m->s, name);
    if (i < 0) return -1;
    *type = m->s->col_types[i];
    if (m->need) m->need[i] = 1;
    int j = vg_colset_add(m->set, i);
    if (j < 0) return -1;
    return j;
}

static void compile_filter(VgFilter *f) {
    if (f->compiled) return;
    const VecSchema *cs = &f->fn.child->output_schema;
    f->need = (uint8_t *)vg_xcalloc((size_t)(cs->n_cols ? cs->n_cols : 1), 1);
    MapCtx mc = {cs, f->need, &f->set};
    int r = vg_compile_pred(f->fn.predicate, map_schema, &mc, &f->pred);
    if (r == 1) { f->compiled = 1; return; }
    if (r < 0) { snprintf(f->err, sizeof(f->err), "%s", vg_compile_error()); f->compiled = 3; return; }
    memset(f->need, 0, (size_t)(cs->n_cols ? cs->n_cols : 1));
    memset(&f->set, 0, sizeof(f->set));
    if (vg_compile_prog(f->fn.predicate, map_schema, &mc, &f->prog) != 0) {
        snprintf(f->err, sizeof(f->err), "%s", vg_compile_error());
        f->compiled = 3;
        return;
    }
    if (f->prog.result_type != VEC_BOOL) {
        snprintf(f->err, sizeof(f->err), "filter predicate must evaluate to boolean");
        f->compiled = 3;
        return;
    }
    f->compiled = 2;
}

/* The general program this filter compiled to (its columns index the
 * child columns listed in *set), or NULL if it is a conjunction or does not
 * compile. */
const VgProg *vg_filter_program(VecNode *n, VecNode **child_out, const VgColSet **set) {
    VgFilter *f = (VgFilter *)n;
    compile_filter(f);
    *child_out = f->fn.child;
    *set = &f->set;
    return f->compiled == 2 ? &f->prog : NULL;
}

/* The conjunction this filter compiled to (term columns index the child
 * columns listed in *set), or NULL if it needs the general program. */
const VgPred *vg_filter_cnf(VecNode *n, VecNode **child_out, const VgColSet **set) {
    VgFilter *f = (VgFilter *)n;
    compile_filter(f);
    *child_out = f->fn.child;
    *set = &f->set;
    return f->compiled == 1 ? &f->pred : NULL;
}

static VecBatch *filter_next_body(VecNode *self) {
    VgFilter *f = (VgFilter *)self;
    compile_filter(f);
    if (f->compiled == 3) {
        /* the reference evaluates the predicate on each batch: its errors
         * come with the first batch, and an empty input has none */
        VecBatch *b = f->fn.child->next_batch(f->fn.child);
        if (!b) return NULL;
        vg_batch_free(b);
        vg_fail("%s", f->err);
    }
    VgDBatch db;
    while (vg_pull(f->fn.child, f->need, 1, &db)) {
        VgCol cols[VG_MAX_COLS];
        int nc = f->set.n;
        for (int j = 0; j < nc; j++) cols[j] = db.cols[f->set.idx[j]];
        int64_t n_logical = db.d_sel ? db.sel_n : db.n_rows;
        size_t scratch_bytes = vgk_filter_scratch_bytes(n_logical);
        char *scratch = (char *)vg_dmalloc(scratch_bytes + (size_t)(n_logical > 0 ? n_logical : 1) * 4);
        int32_t *d_out = (int32_t *)(scratch + scratch_bytes);
        int64_t cnt = 0;
        int rc = (f->compiled == 1)
            ? vgk_filter_pred(cols, nc, &f->pred, db.n_rows, db.d_sel, db.sel_n, d_out, &cnt,
                              scratch, scratch_bytes, vg_stream())
            : vgk_filter_prog(cols, nc, &f->prog, db.n_rows, db.d_sel, db.sel_n, d_out, &cnt,
                              scratch, scratch_bytes, vg_stream());
        if (rc) { vg_dfree(scratch); vg_dbatch_release(&db); vg_check_rc(rc, "filter"); }
        VecBatch *b = db.host;
        if (cnt > 0) {
            int32_t *sel = (int32_t *)vg_xmalloc((size_t)cnt * 4);
            vg_d2h(sel, d_out, (size_t)cnt * 4);
            vg_sync();
            vg_dfree(scratch);
            free(b->sel);
            b->sel = sel;
            b->sel_n = (int32_t)cnt;
            db.host = NULL;
            vg_dbatch_release(&db);
            return b;
        }
        vg_dfree(scratch);
        vg_dbatch_release(&db);   /* empty after filtering: drop and pull the next */
    }
    return NULL;
}

/* one node API call: its temporary device memory is released if it fails */
static VecBatch *filter_next(VecNode *self) {
    vg_scope_enter();
    VecBatch *b = filter_next_body(self);
    vg_scope_leave();
    return b;
}

static void filter_free(VecNode *self) {
    VgFilter *f = (VgFilter *)self;
    f->fn.child->free_node(f->fn.child);
    vg_expr_free(f->fn.predicate);
    vg_schema_free(&f->fn.base.output_schema);
    free(f->need);
    free(f);
}

FilterNode *filter_node_create(VecNode *child, VecExpr *predicate) {
    VgFilter *f = (VgFilter *)vg_xcalloc(1, sizeof(VgFilter));
    f->fn.child = child;
    f->fn.predicate = predicate;
    f->fn.base.output_schema = vg_schema_copy(&child->output_schema);
    f->fn.base.next_batch = filter_next;
    f->fn.base.free_node = filter_free;
    f->fn.base.kind = "FilterNode";
    return &f->fn;
}
