"""libvgpu nodes inside the reference engine's own plan machinery, on the CPU.

A C host compiled against the reference's headers writes a .vtr file with
the reference's own writer (vtr1_write_header / vtr1_write_rowgroup,
src/vtr1.c), opens it with the reference's ScanNode (src/scan.c), puts
libvgpu's FilterNode / GroupAggNode / JoinNode on top (the constructors the
R bridge calls, linked from libvgpu.so in place of src/filter.c,
src/group_agg.c and src/join.c) and runs the reference optimizer,
vec_optimize (src/optimize.c), over the plans:

- filter -> group_agg over a scan: predicate pushdown borrows the filter's
  predicate into the scan (src/optimize.c:356-371) and the filter keeps it
  intact; column pruning reaches the scan through the filter and the
  group-agg (src/optimize.c:85-125, 243-259) and the filter's schema follows
  the pruned scan; the scan then skips the row groups whose v3 min/max
  statistics rule the predicate out (src/scan.c:12-105);
- a join of two scans (src/optimize.c:313-333): both sides stay whole;
- a filter over libvgpu's table source: its kind is not "ScanNode", so the
  optimizer neither casts it to a ScanNode nor pushes anything into it;
- the first plan again over libvgpu's own scan node (its scan_node_create,
  the drop-in for src/scan.c): the optimizer prunes and pushes into it
  through the same struct fields, and it skips the same row groups.

Nothing here touches a device: node construction is host work only, and the
plans are freed without being run.  The reference objects come from
oracle/_ref (built from the reference checkout), so the test is skipped
where that checkout is absent.
"""
import os
import shutil
import subprocess

import pytest

from engines import ORACLE_DIR, REF_SRC, ref_available

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

HOST = r"""
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <stdarg.h>
#include <dlfcn.h>

#include "types.h"
#include "array.h"
#include "batch.h"
#include "schema.h"
#include "expr.h"
#include "vtr1.h"
#include "scan.h"
#include "filter.h"
#include "group_agg.h"
#include "join.h"
#include "optimize.h"

/* the R API the reference's error.c needs */
void Rf_error(const char *fmt, ...) {
    va_list ap; va_start(ap, fmt); vfprintf(stderr, fmt, ap); va_end(ap);
    fprintf(stderr, "\n"); exit(90);
}
void Rf_warning(const char *fmt, ...) { (void)fmt; }

/* libvgpu's table source (include/vgpu.h) */
VecNode *vgpu_table_source_create(int n_cols, const char *const *names, const int *types,
                                  const void *const *data, const uint8_t *const *validity,
                                  int64_t n_rows, int64_t batch_rows, int flags);

static int fails = 0;
#define CHECK(c) do { if (!(c)) { fprintf(stderr, "check failed: %s (line %d)\n", #c, __LINE__); fails++; } } while (0)

static char *dup(const char *s) { char *r = malloc(strlen(s) + 1); strcpy(r, s); return r; }

static VecExpr *colref(const char *n) { VecExpr *e = vec_expr_alloc(EXPR_COL_REF); e->col_name = dup(n); return e; }
static VecExpr *lit_d(double v) { VecExpr *e = vec_expr_alloc(EXPR_LIT_DOUBLE); e->result_type = VEC_DOUBLE; e->lit_dbl = v; return e; }
static VecExpr *cmp(VecExpr *l, char op, char op2, VecExpr *r) {
    VecExpr *e = vec_expr_alloc(EXPR_CMP); e->result_type = VEC_BOOL; e->op = op; e->op2 = op2; e->left = l; e->right = r; return e;
}
static VecExpr *and_(VecExpr *l, VecExpr *r) {
    VecExpr *e = vec_expr_alloc(EXPR_BOOL); e->result_type = VEC_BOOL; e->op = '&'; e->op2 = ' '; e->left = l; e->right = r; return e;
}

/* row group g of the weather table: station, temperature, year, extra;
 * temperature stays below 25 in the even row groups */
static VecBatch *weather_rg(int g, int64_t n) {
    VecBatch *b = vec_batch_alloc(4, n);
    const char *names[4] = {"station", "temperature", "year", "extra"};
    VecType types[4] = {VEC_INT64, VEC_DOUBLE, VEC_INT64, VEC_DOUBLE};
    for (int c = 0; c < 4; c++) {
        b->columns[c] = vec_array_alloc(types[c], n);
        vec_array_set_all_valid(&b->columns[c]);
        b->col_names[c] = dup(names[c]);
    }
    for (int64_t i = 0; i < n; i++) {
        b->columns[0].buf.i64[i] = (i * 7 + g) % 100;
        b->columns[1].buf.dbl[i] = (g % 2 == 0) ? (double)(i % 25) : (double)(i % 40);
        b->columns[2].buf.i64[i] = 2000 + (i + g) % 26;
        b->columns[3].buf.dbl[i] = 0.5 * (double)i;
    }
    return b;
}

static void write_weather(const char *path, int n_rg, int64_t n) {
    FILE *fp = fopen(path, "wb");
    VecBatch *b0 = weather_rg(0, n);
    VecSchema s;
    memset(&s, 0, sizeof(s));
    s.n_cols = 4;
    s.col_names = b0->col_names;
    VecType t[4] = {VEC_INT64, VEC_DOUBLE, VEC_INT64, VEC_DOUBLE};
    s.col_types = t;
    vtr1_write_header(fp, &s, (uint32_t)n_rg);
    vec_batch_free(b0);
    for (int g = 0; g < n_rg; g++) {
        VecBatch *b = weather_rg(g, n);
        vtr1_write_rowgroup(fp, b);
        vec_batch_free(b);
    }
    fclose(fp);
}

/* filter -> group_agg over a scan made by `mk`: pushdown, pruning and the
 * row groups the scan then returns */
static void filter_agg_plan(ScanNode *(*mk)(const char *, int *, int), const char *path, const char *tmp) {
    ScanNode *sn = mk(path, NULL, 0);
    CHECK(strcmp(sn->base.kind, "ScanNode") == 0 && sn->base.output_schema.n_cols == 4);
    CHECK(sn->file->header.version == 3 && sn->file->header.n_rowgroups == 6);
    VecExpr *pred = and_(cmp(colref("temperature"), '>', ' ', lit_d(30.0)),
                         cmp(colref("year"), '>', '=', lit_d(2020.0)));
    FilterNode *fn = filter_node_create(&sn->base, pred);
    char **keys = malloc(sizeof(char *));
    keys[0] = dup("station");
    AggSpec *specs = calloc(2, sizeof(AggSpec));
    specs[0].kind = AGG_MEAN; specs[0].input_col = dup("temperature"); specs[0].output_name = dup("avg");
    specs[1].kind = AGG_COUNT_STAR; specs[1].input_col = NULL; specs[1].output_name = dup("n");
    GroupAggNode *ga = group_agg_node_create(&fn->base, 1, keys, 2, specs, tmp);
    vec_optimize(&ga->base);
    CHECK(sn->predicate == pred && sn->pred_borrowed == 1 && fn->predicate == pred);
    CHECK(sn->col_mask[0] == 1 && sn->col_mask[1] == 1 && sn->col_mask[2] == 1 && sn->col_mask[3] == 0);
    CHECK(sn->base.output_schema.n_cols == 3 && fn->base.output_schema.n_cols == 3);
    int n_batches = 0;
    for (VecBatch *b; (b = sn->base.next_batch(&sn->base)) != NULL; n_batches++) {
        CHECK(b->n_cols == 3 && b->n_rows == 1000);
        CHECK(strcmp(b->col_names[2], "year") == 0);
        vec_batch_free(b);
    }
    CHECK(n_batches == 3);
    ga->base.free_node(&ga->base);
}

int main(int argc, char **argv) {
    if (argc < 3) return 2;
    char path[4096], path2[4096];
    snprintf(path, sizeof(path), "%s/weather.vtr", argv[1]);
    snprintf(path2, sizeof(path2), "%s/dim.vtr", argv[1]);
    write_weather(path, 6, 1000);

    /* --- filter -> group_agg over a scan ------------------------------- */
    ScanNode *sn = scan_node_create(path, NULL, 0);
    CHECK(sn->base.output_schema.n_cols == 4);
    VecExpr *pred = and_(cmp(colref("temperature"), '>', ' ', lit_d(30.0)),
                         cmp(colref("year"), '>', '=', lit_d(2020.0)));
    FilterNode *fn = filter_node_create(&sn->base, pred);
    CHECK(strcmp(fn->base.kind, "FilterNode") == 0);
    CHECK(fn->child == &sn->base && fn->predicate == pred);
    char **keys = malloc(sizeof(char *));
    keys[0] = dup("station");
    AggSpec *specs = calloc(2, sizeof(AggSpec));
    specs[0].kind = AGG_MEAN; specs[0].input_col = dup("temperature"); specs[0].output_name = dup("avg");
    specs[1].kind = AGG_COUNT_STAR; specs[1].input_col = NULL; specs[1].output_name = dup("n");
    GroupAggNode *ga = group_agg_node_create(&fn->base, 1, keys, 2, specs, argv[1]);
    CHECK(strcmp(ga->base.kind, "GroupAggNode") == 0);
    CHECK(ga->child == &fn->base && ga->n_keys == 1 && ga->n_aggs == 2 && ga->use_sorted == 1);

    vec_optimize(&ga->base);

    /* pushdown: the scan borrows the filter's predicate, which stays whole */
    CHECK(sn->predicate == pred && sn->pred_borrowed == 1);
    CHECK(fn->predicate == pred && pred->kind == EXPR_BOOL && pred->op == '&');
    CHECK(pred->left->kind == EXPR_CMP && strcmp(pred->left->left->col_name, "temperature") == 0);
    CHECK(pred->right->kind == EXPR_CMP && strcmp(pred->right->left->col_name, "year") == 0);
    /* pruning reached the scan: 'extra' is no longer read */
    CHECK(sn->col_mask[0] == 1 && sn->col_mask[1] == 1 && sn->col_mask[2] == 1 && sn->col_mask[3] == 0);
    CHECK(sn->base.output_schema.n_cols == 3);
    CHECK(fn->base.output_schema.n_cols == 3);
    CHECK(strcmp(fn->base.output_schema.col_names[2], "year") == 0);
    /* the pushed predicate prunes row groups: only the odd ones (temperature
     * up to 39) can hold temperature > 30 */
    int n_batches = 0;
    for (VecBatch *b; (b = sn->base.next_batch(&sn->base)) != NULL; n_batches++) {
        CHECK(b->n_cols == 3 && b->n_rows == 1000);
        vec_batch_free(b);
    }
    CHECK(n_batches == 3);
    ga->base.free_node(&ga->base);

    /* --- a join of two scans ------------------------------------------ */
    write_weather(path2, 2, 100);
    ScanNode *l = scan_node_create(path, NULL, 0);
    ScanNode *r = scan_node_create(path2, NULL, 0);
    JoinKey *jk = malloc(sizeof(JoinKey));
    jk[0].left_col = 0; jk[0].right_col = 0;
    JoinNode *jn = join_node_create(&l->base, &r->base, JOIN_LEFT, 1, jk, ".x", ".y");
    CHECK(strcmp(jn->base.kind, "JoinNode") == 0);
    CHECK(jn->left == &l->base && jn->right == &r->base && jn->kind == JOIN_LEFT && jn->n_keys == 1);
    CHECK(jn->base.output_schema.n_cols == 7);
    vec_optimize(&jn->base);
    CHECK(l->col_mask[3] == 1 && r->col_mask[3] == 1);
    CHECK(l->predicate == NULL && r->predicate == NULL);
    CHECK(jn->base.output_schema.n_cols == 7);
    jn->base.free_node(&jn->base);

    /* --- a filter over libvgpu's table source -------------------------- */
    int64_t kv[4] = {1, 2, 3, 4};
    double xv[4] = {0.5, 40.0, 31.0, 2.0};
    const char *nm[2] = {"k", "temperature"};
    int ty[2] = {VEC_INT64, VEC_DOUBLE};
    const void *dv[2] = {kv, xv};
    VecNode *src = vgpu_table_source_create(2, nm, ty, dv, NULL, 4, 0, 0);
    CHECK(src != NULL && strcmp(src->kind, "ScanNode") != 0);
    VecExpr *p2 = cmp(colref("temperature"), '>', ' ', lit_d(30.0));
    FilterNode *f2 = filter_node_create(src, p2);
    vec_optimize(&f2->base);
    CHECK(f2->predicate == p2 && f2->base.output_schema.n_cols == 2);
    f2->base.free_node(&f2->base);

    /* the same plan over libvgpu's own scan node (scan_node_create from
     * libvgpu.so, looked up by name: the reference's scan.o, linked into this
     * program, defines the same symbol) */
    void *h = dlopen(argv[2], RTLD_NOW | RTLD_LOCAL);
    CHECK(h != NULL);
    if (h) {
        ScanNode *(*vg_scan)(const char *, int *, int) = (ScanNode * (*)(const char *, int *, int))dlsym(h, "scan_node_create");
        CHECK(vg_scan != NULL && vg_scan != scan_node_create);
        if (vg_scan && vg_scan != scan_node_create) filter_agg_plan(vg_scan, path, argv[1]);
    }
    filter_agg_plan(scan_node_create, path, argv[1]);

    remove(path);
    remove(path2);
    if (fails) return 1;
    printf("plans ok\n");
    return 0;
}
"""

REF_OBJS = ["optimize", "scan", "vtr1", "array", "batch", "schema", "expr", "scalar_ops", "coerce", "error"]


def test_libvgpu_nodes_under_the_reference_optimizer(tmp_path):
    if not ref_available():
        pytest.skip("reference checkout absent: its optimizer, scan and writer cannot be built")
    gcc = shutil.which("gcc")
    if not gcc:
        pytest.skip("no gcc")
    import vectra_gb300
    vectra_gb300.load()   # built
    src = tmp_path / "host.c"
    src.write_text(HOST)
    exe = tmp_path / "host"
    objs = [os.path.join(ORACLE_DIR, "_ref", o + ".o") for o in REF_OBJS]
    libdir = os.path.join(ROOT, "vectra_gb300")
    r = subprocess.run([gcc, "-std=gnu11", "-O1", "-o", str(exe), str(src), *objs,
                        "-I", REF_SRC, "-I", os.path.join(ORACLE_DIR, "rshim"),
                        os.path.join(libdir, "libvgpu.so"), "-Wl,-rpath," + libdir, "-lm", "-ldl"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    nm = subprocess.run(["nm", str(exe)], capture_output=True, text=True, check=True).stdout
    # the node constructors come from libvgpu, not from the reference's objects
    for sym in ("filter_node_create", "group_agg_node_create", "join_node_create"):
        assert any(l.split()[-1] == sym and " U " in l for l in nm.splitlines()), sym
    out = subprocess.run([str(exe), str(tmp_path), os.path.join(libdir, "libvgpu.so")], capture_output=True,
                         text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "plans ok" in out.stdout
