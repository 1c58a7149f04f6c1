/*
 * node_project.c -- ProjectNode (select / mutate) on the GPU
 * (replaces src/project.c).
 *
 * next_batch evaluates every expression entry over the logical rows of the
 * child batch on the device and returns a dense batch (no sel), as
 * project_mutate_path does (src/project.c:51-252): pass-through columns are
 * gathered, expression columns computed, and an expression may refer to the
 * outputs of earlier entries.
 *
 * Under a group-agg node the projection is not run on its own: the
 * aggregate reads `value * weight`-style entries directly (vg_project_lookup)
 * and computes them inside its kernel.  This is how the hidden mutate that
 * the R front end inserts for summarise(s = sum(x * y)) (R/verbs.R:255-283)
 * costs nothing.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "vg_host.h"

typedef struct {
    ProjectNode pn;           /* reference prefix: base, child, n_entries, entries */
} VgProject;

static VecBatch *project_next(VecNode *self);

int vg_is_project(const VecNode *n) { return n && n->next_batch == project_next; }
VecNode *vg_project_child(VecNode *n) { return ((VgProject *)n)->pn.child; }

int vg_project_lookup(VecNode *n, const char *name, const VecExpr **expr, const char **pass_name) {
    VgProject *p = (VgProject *)n;
    for (int i = 0; i < p->pn.n_entries; i++) {
        if (strcmp(p->pn.entries[i].output_name, name) != 0) continue;
        *expr = p->pn.entries[i].expr;
        *pass_name = p->pn.entries[i].expr ? NULL : p->pn.entries[i].output_name;
        return 1;
    }
    return 0;
}

/* working columns: the child's, then each computed entry in turn */
typedef struct {
    int n;
    char **names;
    VgCol *cols;
    const VecSchema *child;
    uint8_t *need;            /* child columns referenced (first pass) */
} Work;

static int map_work(void *ctx, const char *name, int *type) {
    Work *w = (Work *)ctx;
    for (int i = 0; i < w->n; i++) {
        if (strcmp(w->names[i], name) == 0) {
            *type = w->cols[i].type;
            if (w->need && i < w->child->n_cols) w->need[i] = 1;
            return i;
        }
    }
    return -1;
}

/* column references of one program, as a compact kernel table */
typedef struct { Work *w; int idx[VG_MAX_COLS]; int n; } Compact;

static int map_compact(void *ctx, const char *name, int *type) {
    Compact *c = (Compact *)ctx;
    int i = map_work(c->w, name, type);
    if (i < 0) return -1;
    for (int j = 0; j < c->n; j++) if (c->idx[j] == i) return j;
    if (c->n >= VG_MAX_COLS) return -1;
    c->idx[c->n] = i;
    return c->n++;
}

static VecBatch *project_next_body(VecNode *self) {
    VgProject *p = (VgProject *)self;
    const VecSchema *cs = &p->pn.child->output_schema;
    int nc = cs->n_cols, ne = p->pn.n_entries;
    /* which child columns are needed: pass-throughs and expression refs */
    Work w;
    memset(&w, 0, sizeof(w));
    w.child = cs;
    w.names = (char **)vg_xcalloc((size_t)(nc + ne), sizeof(char *));
    w.cols = (VgCol *)vg_xcalloc((size_t)(nc + ne), sizeof(VgCol));
    w.need = (uint8_t *)vg_xcalloc((size_t)(nc ? nc : 1), 1);
    for (int c = 0; c < nc; c++) {
        w.names[c] = cs->col_names[c];
        w.cols[c].type = cs->col_types[c];
    }
    w.n = nc;
    for (int i = 0; i < ne; i++) {
        ProjEntry *pe = &p->pn.entries[i];
        if (!pe->expr) {
            int t;
            if (map_work(&w, pe->output_name, &t) < 0) vg_fail("select: column not found: %s", pe->output_name);
        } else {
            VgProg tmp;
            if (vg_compile_prog(pe->expr, map_work, &w, &tmp) != 0) vg_fail("%s", vg_compile_error());
            w.names[w.n] = pe->output_name;
            w.cols[w.n].type = tmp.result_type;
            w.n++;
        }
    }
    VgDBatch db;
    if (!vg_pull(p->pn.child, w.need, 0, &db)) {
        free(w.names); free(w.cols); free(w.need);
        return NULL;
    }
    int64_t n = db.d_sel ? db.sel_n : db.n_rows;
    /* dense copies of the needed child columns over the logical rows */
    size_t wb = (size_t)((n + 31) / 32) * 4;
    /* room for the widest value: a string column is one 16-byte view per row */
    const size_t vbytes = ((size_t)n * 16 + 255) & ~(size_t)255;
    size_t per = vbytes + ((wb + 255) & ~(size_t)255);
    char *blk = (char *)vg_dmalloc(per * (size_t)(nc + ne) + 256);
    for (int c = 0; c < nc; c++) {
        if (!w.need[c]) { w.cols[c].data = NULL; continue; }
        char *dv = blk + per * (size_t)c;
        uint32_t *dm = (uint32_t *)(dv + vbytes);
        vg_check_rc(vgk_gather(&db.cols[c], db.d_sel, n, 0, dv, dm, vg_stream()), "project gather");
        w.cols[c].data = dv;
        w.cols[c].valid = dm;
    }
    VecBatch *out = vg_batch_alloc(ne, n);
    int k = nc;
    for (int i = 0; i < ne; i++) {
        ProjEntry *pe = &p->pn.entries[i];
        out->col_names[i] = vg_xstrdup(pe->output_name);
        int src;
        if (!pe->expr) {
            int t;
            src = map_work(&w, pe->output_name, &t);
        } else {
            VgProg prog;
            Work w2 = w;
            w2.n = k;
            w2.need = NULL;
            Compact cm = {&w2, {0}, 0};
            if (vg_compile_prog(pe->expr, map_compact, &cm, &prog) != 0) vg_fail("%s", vg_compile_error());
            VgCol cols[VG_MAX_COLS];
            for (int j = 0; j < cm.n; j++) cols[j] = w.cols[cm.idx[j]];
            char *dv = blk + per * (size_t)k;
            uint32_t *dm = (uint32_t *)(dv + vbytes);
            vg_check_rc(vgk_eval_prog(cols, cm.n, &prog, n, NULL, n, dv, dm, vg_stream()), "project eval");
            w.cols[k].data = dv;
            w.cols[k].valid = dm;
            src = k++;
        }
        out->columns[i] = w.cols[src].type == VEC_STRING
                              ? vg_download_strings(&w.cols[src], NULL, n)
                              : vg_download_column(w.cols[src].type, w.cols[src].data, w.cols[src].valid, n);
    }
    vg_sync();
    vg_dfree(blk);
    vg_dbatch_release(&db);
    free(w.names); free(w.cols); free(w.need);
    return out;
}

/* one node API call: its temporary device memory is released if it fails */
static VecBatch *project_next(VecNode *self) {
    vg_scope_enter();
    VecBatch *b = project_next_body(self);
    vg_scope_leave();
    return b;
}

static void project_free(VecNode *self) {
    VgProject *p = (VgProject *)self;
    p->pn.child->free_node(p->pn.child);
    for (int i = 0; i < p->pn.n_entries; i++) {
        free(p->pn.entries[i].output_name);
        vg_expr_free(p->pn.entries[i].expr);
    }
    free(p->pn.entries);
    vg_schema_free(&p->pn.base.output_schema);
    free(p);
}

ProjectNode *project_node_create(VecNode *child, int n_entries, ProjEntry *entries) {
    VgProject *p = (VgProject *)vg_xcalloc(1, sizeof(VgProject));
    p->pn.child = child;
    p->pn.n_entries = n_entries;
    p->pn.entries = entries;
    char **names = (char **)vg_xcalloc((size_t)(n_entries ? n_entries : 1), sizeof(char *));
    VecType *types = (VecType *)vg_xcalloc((size_t)(n_entries ? n_entries : 1), sizeof(VecType));
    for (int i = 0; i < n_entries; i++) {
        names[i] = entries[i].output_name;
        if (entries[i].expr) {
            types[i] = entries[i].expr->result_type;
        } else {
            int idx = vg_schema_find(&child->output_schema, entries[i].output_name);
            if (idx < 0) vg_fail("project: column not found in child: %s", entries[i].output_name);
            types[i] = child->output_schema.col_types[idx];
        }
    }
    p->pn.base.output_schema = vg_schema_make(n_entries, names, types);
    free(names);
    free(types);
    p->pn.base.next_batch = project_next;
    p->pn.base.free_node = project_free;
    p->pn.base.kind = "ProjectNode";
    return &p->pn;
}
