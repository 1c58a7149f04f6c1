/*
 * node_agg.c -- GroupAggNode on the GPU (replaces src/group_agg.c and the
 * sort-based path it builds through src/sort.c).
 *
 * The node looks at the chain below it and fuses what it can into one
 * kernel per batch (vgk_agg_launch):
 *
 *     GroupAgg <- [Project] <- [Join (INNER/LEFT)] <- [Filter] <- source
 *
 * the filter's conjunction is evaluated per row, the join probe runs per row
 * against the build-side table, the projection's arithmetic (e.g. the
 * hidden `.vectra_tmp_s = value * weight` mutate that summarise(sum(value *
 * weight)) inserts, R/verbs.R:255-283) is computed per matched row, and the
 * result feeds the group accumulators.  The intermediate nodes are never
 * asked for batches.  Any other child is consumed batch by batch through
 * next_batch.
 *
 * Output (src/group_agg.c:240-281, 466-585): one batch, group keys with
 * their input types, then every aggregate as double.  Groups come in
 * ascending key order with NA last when temp_dir is given (what the R front
 * end always requests, src/r_bridge.c:990), otherwise in first-seen order
 * (the reference's hash path).  Ungrouped aggregation of zero rows yields
 * zero rows, as in the reference.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "vg_host.h"

typedef struct {
    GroupAggNode ga;          /* reference prefix */
    int sorted;               /* emit in key order */
} VgAgg;

/* ------------------------------------------------------------------ */
/* plan                                                                */
/* ------------------------------------------------------------------ */

typedef struct {
    VecNode *src;             /* pulled batch by batch */
    VecNode *project, *join, *filter;
    const VgPred *pred;       /* over the filter child's columns (set fset) */
    const VgColSet *fset;
    VgColSet pset;            /* kernel probe column table -> src column */
    VgColSet bset;            /* kernel build column table -> right column */
    int n_keys, n_accs, n_out;
    VgValue key[VG_MAX_KEYS];
    int32_t key_type[VG_MAX_KEYS];
    VgAccSpec acc[VG_MAX_ACCS];
    VgFinish fin[VG_MAX_OUTS];
    int fail;                 /* resolution failed: not fusable */
} Plan;

typedef struct {
    Plan *P;
    int side;                 /* layer being resolved: 0 probe (src / left), 1 build */
    int below_join;
} Res;

static int add_probe(Plan *P, VecNode *at, const char *name, int *type);

/* Resolves `name` as seen at node `at` (a node of the fused chain, or the
 * source) into an operand. */
static int resolve_operand(Plan *P, VecNode *at, const char *name, VgOperand *o) {
    memset(o, 0, sizeof(*o));
    if (at == P->project) {
        const VecExpr *e = NULL;
        const char *pass = NULL;
        if (!vg_project_lookup(at, name, &e, &pass)) return 0;
        if (!e) return resolve_operand(P, vg_project_child(at), pass, o);
        return 0;   /* expressions are handled one level up (resolve_value) */
    }
    if (at == P->join) {
        int side, col;
        if (!vg_join_resolve(at, name, &side, &col)) return 0;
        if (side == 0) {
            VecNode *l = vg_join_left(at);
            return resolve_operand(P, l, l->output_schema.col_names[col], o);
        }
        int j = vg_colset_add(&P->bset, col);
        if (j < 0) return 0;
        o->side = VG_SIDE_BUILD;
        o->col = j;
        o->type = vg_join_right_type(at, col);
        return o->type != VEC_STRING;
    }
    if (at == P->filter) {
        VecNode *child = P->src;
        return resolve_operand(P, child, name, o);
    }
    /* the source */
    int t;
    int j = add_probe(P, at, name, &t);
    if (j < 0) return 0;
    o->side = VG_SIDE_PROBE;
    o->col = j;
    o->type = t;
    return t != VEC_STRING;
}

static int add_probe(Plan *P, VecNode *at, const char *name, int *type) {
    int i = vg_schema_find(&at->output_schema, name);
    if (i < 0) return -1;
    *type = at->output_schema.col_types[i];
    return vg_colset_add(&P->pset, i);
}

/* colmap used when compiling a projection expression: names resolve at the
 * projection's child */
typedef struct { Plan *P; VecNode *at; VgOperand last; } ExprCtx;

static int map_expr(void *ctx, const char *name, int *type) {
    ExprCtx *c = (ExprCtx *)ctx;
    VgOperand o;
    if (!resolve_operand(c->P, c->at, name, &o)) return -1;
    *type = o.type;
    c->last = o;
    /* encode side in the returned index: build columns offset by 1000 */
    return o.side == VG_SIDE_BUILD ? 1000 + o.col : o.col;
}

static int resolve_value(Plan *P, const char *name, VgValue *v) {
    memset(v, 0, sizeof(*v));
    VecNode *top = P->project ? P->project : (P->join ? P->join : (P->filter ? P->filter : P->src));
    if (top == P->project) {
        const VecExpr *e = NULL;
        const char *pass = NULL;
        if (!vg_project_lookup(top, name, &e, &pass)) return 0;
        if (e) {
            /* every column the expression reads must be a column of the
             * projection's child (the reference looks those up first) */
            VecNode *pc = vg_project_child(top);
            ExprCtx ctx = {P, pc, {0}};
            int r = vg_compile_value(e, map_expr, &ctx, VG_SIDE_PROBE, v);
            if (r <= 0) return 0;
            /* fix up sides: indices >= 1000 are build columns */
            VgOperand *ops[2] = {&v->a, &v->b};
            for (int i = 0; i < 2; i++) {
                if (ops[i]->side == VG_SIDE_PROBE && ops[i]->col >= 1000) {
                    ops[i]->side = VG_SIDE_BUILD;
                    ops[i]->col -= 1000;
                }
            }
            return 1;
        }
        if (!resolve_operand(P, vg_project_child(top), pass, &v->a)) return 0;
        v->type = v->a.type;
        return 1;
    }
    if (!resolve_operand(P, top, name, &v->a)) return 0;
    v->type = v->a.type;
    return 1;
}

static int acc_class(AggKind k, int t) {
    switch (k) {
    case AGG_COUNT_STAR: return VG_ACC_COUNT_ALL;
    case AGG_COUNT: return VG_ACC_COUNT_VALID;
    case AGG_SUM:
    case AGG_MEAN: return t == VEC_DOUBLE ? VG_ACC_SUM_F64 : VG_ACC_SUM_I64;
    case AGG_MIN: return t == VEC_DOUBLE ? VG_ACC_MIN_F64 : t == VEC_INT64 ? VG_ACC_MIN_I64 : VG_ACC_NA_ONLY;
    default: return t == VEC_DOUBLE ? VG_ACC_MAX_F64 : t == VEC_INT64 ? VG_ACC_MAX_I64 : VG_ACC_NA_ONLY;
    }
}

static int same_value(const VgValue *a, const VgValue *b) { return memcmp(a, b, sizeof(*a)) == 0; }

/* Resolves keys and aggregates for the chain chosen in P; 0 if some name
 * does not resolve through it. */
static int plan_resolve(VgAgg *A, Plan *P) {
    GroupAggNode *ga = &A->ga;
    P->n_keys = ga->n_keys;
    for (int k = 0; k < ga->n_keys; k++) {
        if (!resolve_value(P, ga->key_names[k], &P->key[k])) return 0;
        P->key_type[k] = P->key[k].type;
    }
    P->n_accs = 0;
    P->n_out = ga->n_aggs;
    for (int a = 0; a < ga->n_aggs; a++) {
        AggSpec *s = &ga->agg_specs[a];
        VgAccSpec acc;
        memset(&acc, 0, sizeof(acc));
        int in_type = VEC_INT64;
        if (s->kind == AGG_COUNT_STAR) {
            acc.cls = VG_ACC_COUNT_ALL;
        } else {
            if (!s->input_col) return 0;
            if (!resolve_value(P, s->input_col, &acc.in)) return 0;
            in_type = acc.in.type;
            acc.cls = acc_class(s->kind, in_type);
            acc.na_rm = (acc.cls == VG_ACC_COUNT_VALID) ? 0 : (s->na_rm != 0);
        }
        int idx = -1;
        for (int i = 0; i < P->n_accs; i++)
            if (P->acc[i].cls == acc.cls && P->acc[i].na_rm == acc.na_rm &&
                (acc.cls == VG_ACC_COUNT_ALL || same_value(&P->acc[i].in, &acc.in))) { idx = i; break; }
        if (idx < 0) {
            if (P->n_accs >= VG_MAX_ACCS) vg_fail("too many aggregates for the GPU group-agg (max %d)", VG_MAX_ACCS);
            idx = P->n_accs++;
            P->acc[idx] = acc;
        }
        P->fin[a].acc = idx;
        P->fin[a].finish = s->kind;
        P->fin[a].in_type = in_type;
        P->fin[a].na_rm = s->na_rm;
    }
    return 1;
}

static void plan_build(VgAgg *A, Plan *P) {
    memset(P, 0, sizeof(*P));
    VecNode *n = A->ga.child;
    if (vg_is_project(n)) { P->project = n; n = vg_project_child(n); }
    if (vg_is_join(n) && (vg_join_kind(n) == JOIN_INNER || vg_join_kind(n) == JOIN_LEFT)) {
        P->join = n;
        n = vg_join_left(n);
    }
    if (vg_is_filter(n)) {
        VecNode *fc;
        const VgColSet *fs;
        const VgPred *pr = vg_filter_cnf(n, &fc, &fs);
        if (pr) { P->filter = n; P->pred = pr; P->fset = fs; n = fc; }
    }
    P->src = n;
    if (plan_resolve(A, P)) return;
    /* fall back to consuming the child's batches */
    memset(P, 0, sizeof(*P));
    P->src = A->ga.child;
    if (!plan_resolve(A, P)) {
        for (int k = 0; k < A->ga.n_keys; k++)
            if (vg_schema_find(&P->src->output_schema, A->ga.key_names[k]) < 0)
                vg_fail("group_by: column not found: %s", A->ga.key_names[k]);
        for (int a = 0; a < A->ga.n_aggs; a++)
            if (A->ga.agg_specs[a].input_col &&
                vg_schema_find(&P->src->output_schema, A->ga.agg_specs[a].input_col) < 0)
                vg_fail("summarise: column not found: %s", A->ga.agg_specs[a].input_col);
        vg_fail("group-agg inputs not supported by the GPU path (string or too many columns)");
    }
}

/* ------------------------------------------------------------------ */
/* device group table                                                  */
/* ------------------------------------------------------------------ */

typedef struct {
    VgGroupTable gt;
    void *block;
} Table;

static size_t a256(size_t x) { return (x + 255) & ~(size_t)255; }

static void table_alloc(Table *T, const Plan *P, int64_t cap) {
    memset(T, 0, sizeof(*T));
    int nk = P->n_keys > 0 ? P->n_keys : 1;
    size_t bytes = a256((size_t)cap * 4) * 2 + a256((size_t)cap * 8 * (size_t)nk) + a256((size_t)cap * 8) + 512;
    for (int a = 0; a < P->n_accs; a++) {
        bytes += a256((size_t)cap * 8) * 2 + a256((size_t)cap * 4);
        if (P->acc[a].cls == VG_ACC_SUM_F64) bytes += a256(vgk_lacc_bytes(cap));
    }
    char *b = (char *)vg_dmalloc(bytes);
    T->block = b;
    size_t o = 0;
    VgGroupTable *g = &T->gt;
    g->cap = cap;
    g->state = (uint32_t *)(b + o); o += a256((size_t)cap * 4);
    g->nullmask = (uint32_t *)(b + o); o += a256((size_t)cap * 4);
    g->keys = (uint64_t *)(b + o); o += a256((size_t)cap * 8 * (size_t)nk);
    g->first_row = (uint64_t *)(b + o); o += a256((size_t)cap * 8);
    g->n_used = (uint32_t *)(b + o); o += 256;
    g->err = (uint32_t *)(b + o); o += 256;
    int32_t cls[VG_MAX_ACCS];
    for (int a = 0; a < P->n_accs; a++) {
        cls[a] = P->acc[a].cls;
        g->cnt[a] = (uint64_t *)(b + o); o += a256((size_t)cap * 8);
        g->val[a] = (int64_t *)(b + o); o += a256((size_t)cap * 8);
        g->flags[a] = (uint32_t *)(b + o); o += a256((size_t)cap * 4);
        if (P->acc[a].cls == VG_ACC_SUM_F64) { g->lacc[a] = (int64_t *)(b + o); o += a256(vgk_lacc_bytes(cap)); }
    }
    vg_check_rc(vgk_group_table_init(g, P->n_keys, cls, P->n_accs, vg_stream()), "group table init");
}

/* Rows per aggregation launch while the group table is still growing; once
 * a launch needed no growth, the rest of the batch goes in one launch (the
 * spill list is sized for a launch). */
static const int64_t kChunk = (int64_t)1 << 24;

/* column view of rows [off, ...) of c */
static VgCol vg_col_slice(const VgCol *c, int64_t off) {
    VgCol o = *c;
    if (off == 0 || !c->data) return o;
    o.data = (const char *)c->data + (size_t)off * (c->type == VEC_BOOL ? 1 : 8);
    if (c->valid) {
        const int64_t b = (int64_t)c->voff + off;
        o.valid = c->valid + (b >> 5);
        o.voff = (int32_t)(b & 31);
    }
    return o;
}

static int64_t pow2_at_least(int64_t x) {
    int64_t c = 1024;
    while (c < x) c <<= 1;
    return c;
}

/* ------------------------------------------------------------------ */
/* execution                                                           */
/* ------------------------------------------------------------------ */

typedef struct {
    int64_t *rows;            /* spilled rows */
    uint32_t *counters;       /* [0] rows, [1] cache entries */
    char *cache;
    int64_t rows_cap, cache_cap;
} Spill;

/* The spill list is sized for a whole launch and kept between queries (the
 * node API runs one query at a time), so a large batch does not allocate
 * gigabytes per query. */
static int64_t *g_spill_rows;
static int64_t g_spill_rows_cap;

static int cache_slots_for(const VgAggLaunch *L) {
    /* largest power of two <= 2048 whose shared layout fits in 96 KB */
    VgAggLaunch tmp = *L;
    for (int s = 2048; s >= 256; s >>= 1) {
        tmp.cache_slots = s;
        if (vgk_agg_smem_bytes(&tmp) <= 96 * 1024) return s;
    }
    return 0;
}

/* one launch over n_logical rows (+ growth and replay); 1 if the table grew */
static int run_batch(Plan *P, Table *T, VgAggLaunch *L, Spill *S, int64_t n_logical) {
    int sms = vgk_num_sms();
    /* spill space for this launch */
    int64_t need_rows = n_logical + 65536;
    if (!S->counters) S->counters = (uint32_t *)vg_dmalloc(256);
    if (g_spill_rows_cap < need_rows) {
        vg_dfree(g_spill_rows);
        g_spill_rows = (int64_t *)vg_dmalloc((size_t)need_rows * 16);
        g_spill_rows_cap = need_rows;
    }
    S->rows = g_spill_rows;
    S->rows_cap = g_spill_rows_cap;
    int64_t cc = (int64_t)sms * 2 * (L->cache_slots > 0 ? L->cache_slots : 1);
    if (L->cache_slots > 0 && S->cache_cap < cc) {
        vg_dfree(S->cache);
        S->cache = (char *)vg_dmalloc(vgk_agg_cache_bytes(L, cc) + 256);
        S->cache_cap = cc;
    }
    for (;;) {
        vg_dmemset(S->counters, 0, 8);
        L->gt = T->gt;
        L->spill_rows = S->rows;
        L->spill_rows_n = S->counters;
        L->spill_rows_cap = S->rows_cap;
        L->spill_cache = S->cache;
        L->spill_cache_n = S->counters + 1;
        L->spill_cache_cap = S->cache_cap;
        L->replay = NULL;
        L->replay_n = 0;
        vg_check_rc(vgk_agg_launch(L, vg_stream()), "group-agg");
        uint32_t c[2] = {0, 0}, err = 0, used = 0;
        vg_d2h(c, S->counters, 8);
        vg_d2h(&err, T->gt.err, 4);
        vg_d2h(&used, T->gt.n_used, 4);
        vg_sync();
        if (err & (VG_ERR_WAIT | VG_ERR_PROG)) vg_fail("group-agg kernel error (code %u)", err);
        if (err & (VG_ERR_FULL | VG_ERR_SPILL))
            vg_fail("group-agg: spill capacity exceeded (%u rows, %u entries)", c[0], c[1]);
        if (c[0] == 0 && c[1] == 0) {
            /* keep the load factor at or below 1/2 for the next batch */
            if ((int64_t)used * 2 > T->gt.cap) {
                Table T2;
                table_alloc(&T2, P, pow2_at_least(4 * (int64_t)used));
                int32_t cls[VG_MAX_ACCS];
                for (int a = 0; a < P->n_accs; a++) cls[a] = P->acc[a].cls;
                vg_check_rc(vgk_group_table_rehash(&T->gt, &T2.gt, P->n_keys, P->key_type, cls, P->n_accs,
                                                   vg_stream()), "group table rehash");
                vg_dfree(T->block);
                *T = T2;
                return 1;
            }
            return 0;
        }
        /* grow the table, move the groups, then replay what spilled */
        int64_t ncap = pow2_at_least(2 * ((int64_t)used + c[0] + c[1]) + 1024);
        Table T2;
        table_alloc(&T2, P, ncap);
        int32_t cls[VG_MAX_ACCS];
        for (int a = 0; a < P->n_accs; a++) cls[a] = P->acc[a].cls;
        vg_check_rc(vgk_group_table_rehash(&T->gt, &T2.gt, P->n_keys, P->key_type, cls, P->n_accs, vg_stream()),
                    "group table rehash");
        vg_dfree(T->block);
        *T = T2;
        L->gt = T->gt;
        if (c[1]) vg_check_rc(vgk_agg_merge_spilled_cache(L, c[1], vg_stream()), "group-agg merge");
        if (c[0]) {
            if (P->join) vg_join_ensure_slots(P->join);   /* the replay kernel probes slots */
            L->replay = S->rows;
            L->replay_n = c[0];
            L->spill_rows_cap = 0;           /* a replay must not spill again */
            vg_dmemset(S->counters, 0, 8);
            vg_check_rc(vgk_agg_launch(L, vg_stream()), "group-agg replay");
        }
        err = 0;
        vg_d2h(&err, T->gt.err, 4);
        vg_sync();
        if (err) vg_fail("group-agg: table still full after growing (code %u)", err);
        return 1;
    }
}

static VecBatch *emit_result(VgAgg *A, Plan *P, Table *T) {
    GroupAggNode *ga = &A->ga;
    uint32_t n = 0;
    int32_t *d_slots = (int32_t *)vg_dmalloc((size_t)T->gt.cap * 4 + 16);
    vg_check_rc(vgk_group_table_compact(&T->gt, d_slots, &n, vg_stream()), "group compact");
    int64_t ng = n;
    if (ng > 1 && ga->n_keys > 0) {
        size_t sb = vgk_order_scratch_bytes(ng);
        void *scratch = vg_dmalloc(sb);
        vg_check_rc(vgk_order_groups(&T->gt, P->n_keys, P->key_type, d_slots, ng, A->sorted ? 0 : 1, scratch, sb,
                                     vg_stream()), "group order");
        vg_dfree(scratch);
    }
    int n_out = ga->n_keys + ga->n_aggs;
    VecBatch *res = vg_batch_alloc(n_out, ng);
    size_t wb = (size_t)((ng + 31) / 32) * 4;
    size_t per = a256((size_t)ng * 8 + 8) + a256(wb + 8);
    char *blk = (char *)vg_dmalloc(per * (size_t)(n_out ? n_out : 1) + 256);
    uint64_t *kout[VG_MAX_KEYS];
    uint32_t *kval[VG_MAX_KEYS];
    double *aout[VG_MAX_OUTS];
    uint32_t *aval[VG_MAX_OUTS];
    for (int k = 0; k < ga->n_keys; k++) {
        kout[k] = (uint64_t *)(blk + per * (size_t)k);
        kval[k] = (uint32_t *)((char *)kout[k] + a256((size_t)ng * 8 + 8));
    }
    for (int a = 0; a < ga->n_aggs; a++) {
        aout[a] = (double *)(blk + per * (size_t)(ga->n_keys + a));
        aval[a] = (uint32_t *)((char *)aout[a] + a256((size_t)ng * 8 + 8));
    }
    uint32_t *d_warn = (uint32_t *)(blk + per * (size_t)n_out);
    vg_dmemset(d_warn, 0, 4);
    vg_check_rc(vgk_group_finish(&T->gt, P->n_keys, P->key_type, d_slots, ng, P->fin, ga->n_aggs, kout, kval,
                                 aout, aval, d_warn, vg_stream()), "group finish");
    for (int k = 0; k < ga->n_keys; k++) {
        int t = P->key_type[k];
        VecArray arr = vg_download_column(VEC_INT64, kout[k], kval[k], ng);
        if (t == VEC_BOOL) {
            vg_sync();
            uint8_t *bv = (uint8_t *)vg_xcalloc((size_t)ng + 1, 1);
            for (int64_t i = 0; i < ng; i++) bv[i] = (uint8_t)(arr.buf.i64[i] & 1);
            free(arr.buf.i64);
            arr.buf.bln = bv;
        }
        arr.type = (VecType)t;
        res->columns[k] = arr;
        res->col_names[k] = vg_xstrdup(ga->key_names[k]);
    }
    for (int a = 0; a < ga->n_aggs; a++) {
        res->columns[ga->n_keys + a] = vg_download_column(VEC_DOUBLE, aout[a], aval[a], ng);
        res->col_names[ga->n_keys + a] = vg_xstrdup(ga->agg_specs[a].output_name);
    }
    uint32_t warn = 0;
    vg_d2h(&warn, d_warn, 4);
    vg_sync();
    vg_warn_count((long)warn);
    vg_dfree(blk);
    vg_dfree(d_slots);
    return res;
}

static VecBatch *agg_next(VecNode *self) {
    VgAgg *A = (VgAgg *)self;
    if (A->ga.done) return NULL;
    A->ga.done = 1;
    Plan P;
    plan_build(A, &P);
    /* columns to move to the device for each source batch */
    int nsrc = P.src->output_schema.n_cols;
    uint8_t *need = (uint8_t *)vg_xcalloc((size_t)(nsrc ? nsrc : 1), 1);
    VgAggLaunch *L = (VgAggLaunch *)vg_xcalloc(1, sizeof(VgAggLaunch));
    /* predicate terms index the filter child's columns through fset */
    if (P.pred) {
        L->pred = *P.pred;
        for (int t = 0; t < L->pred.n_terms; t++) {
            if (L->pred.term[t].kind == VG_TERM_NONE) continue;
            int j = vg_colset_add(&P.pset, P.fset->idx[L->pred.term[t].col]);
            if (j < 0) vg_fail("too many columns for the GPU group-agg");
            L->pred.term[t].col = j;
        }
    }
    const VgJoinBuilt *B = NULL;
    if (P.join) {
        /* up to two build columns travel in a payload copy of the join
         * table (one sector per probe row in the specialised kernel) */
        const VgJPay *pay = NULL;
        B = vg_join_build_payload(P.join, P.bset.idx, P.bset.n, &pay);
        L->jpay = pay;
        L->jpay_n = pay ? P.bset.n : 0;
        L->has_join = 1;
        L->join_kind = vg_join_kind(P.join);
        L->n_jkeys = B->n_keys;
        L->jt = B->jt;
        for (int k = 0; k < B->n_keys; k++) {
            /* probe key columns are columns of the join's left input */
            VecNode *l = vg_join_left(P.join);
            VgOperand o;
            if (!resolve_operand(&P, P.filter ? P.filter : l, l->output_schema.col_names[B->lkey[k]], &o) ||
                o.side != VG_SIDE_PROBE)
                vg_fail("GPU join+aggregate: cannot resolve join key");
            L->jkey_col[k] = o.col;
            L->jkey_conv[k] = B->conv[k];
        }
        L->n_bcols = P.bset.n;
        for (int j = 0; j < P.bset.n; j++) L->bcols[j] = B->bcols[P.bset.idx[j]];
    }
    for (int j = 0; j < P.pset.n; j++) need[P.pset.idx[j]] = 1;
    L->n_pcols = P.pset.n;
    L->n_keys = P.n_keys;
    L->n_accs = P.n_accs;
    for (int k = 0; k < P.n_keys; k++) L->key[k] = P.key[k];
    for (int a = 0; a < P.n_accs; a++) L->acc[a] = P.acc[a];
    L->track_first = (!A->sorted && P.n_keys > 0);
    L->cache_slots = cache_slots_for(L);
    /* sum accumulators whose row counts no output reads (no mean) */
    for (int a = 0; a < P.n_accs; a++) {
        if (P.acc[a].cls != VG_ACC_SUM_F64 && P.acc[a].cls != VG_ACC_SUM_I64) continue;
        int counted = 0;
        for (int o = 0; o < P.n_out; o++)
            if (P.fin[o].acc == a && P.fin[o].finish != AGG_SUM) counted = 1;
        if (!counted) L->skip_count_mask |= 1u << a;
    }
    /* one int64 group key read straight from a build-side column: if the
     * build side's values span fewer slots than the cache holds, every
     * group has a fixed cache slot (key - min; NA in the last one) */
    if (B && P.n_keys == 1 && L->cache_slots > 0 && P.key[0].op == 0 &&
        P.key[0].a.side == VG_SIDE_BUILD && P.key[0].a.type == VEC_INT64) {
        int64_t mm[3];
        const int rcol = P.bset.idx[P.key[0].a.col];
        int q = -1;
        if (B->pay_mm_ok)
            for (int i = 0; i < B->pay_n; i++)
                if (B->pay_col[i] == rcol) q = i;
        if (q >= 0) {
            /* the join build's payload pass measured this column */
            mm[0] = B->pay_mm[3 * q];
            mm[1] = B->pay_mm[3 * q + 1];
            mm[2] = B->pay_mm[3 * q + 2];
        } else {
            int64_t *d = (int64_t *)vg_dmalloc(256);
            vg_check_rc(vgk_col_minmax_i64(&L->bcols[P.key[0].a.col], B->jt.n_build, d, mm, vg_stream()),
                        "build key range");
            vg_dfree(d);
        }
        if (mm[2] == 0) {
            L->dense = 1;
            L->dense_n = 0;
            L->dense_min = 0;
        } else if ((uint64_t)mm[1] - (uint64_t)mm[0] < (uint64_t)(L->cache_slots - 1)) {
            L->dense = 1;
            L->dense_n = (int32_t)(mm[1] - mm[0] + 1);
            L->dense_min = mm[0];
        }
    }

    /* only the specialised kernel reads the payload copy instead of slots */
    if (P.join && !(L->jpay && vgk_agg_jit_ok(L))) {
        vg_join_ensure_slots(P.join);
        L->jt = B->jt;
    }

    Table T;
    table_alloc(&T, &P, 8192);
    Spill S;
    memset(&S, 0, sizeof(S));
    VgDBatch db;
    int64_t batch_idx = 0, stream_pos = 0;
    while (vg_pull(P.src, need, 0, &db)) {
        int64_t n_logical = db.d_sel ? db.sel_n : db.n_rows;
        L->batch_idx = batch_idx;
        /* launches of at most kChunk logical rows, so that everything one
         * launch can spill fits the spill list (a batch of any size) */
        int settled = 0;
        for (int64_t off = 0, n = 0; off < n_logical; off += n) {
            n = n_logical - off;
            if (!settled && n > kChunk) n = kChunk;
            if (db.d_sel) {
                for (int j = 0; j < P.pset.n; j++) L->pcols[j] = db.cols[P.pset.idx[j]];
                L->n_rows = db.n_rows;
                L->sel = db.d_sel + off;
                L->sel_n = n;
            } else {
                for (int j = 0; j < P.pset.n; j++) L->pcols[j] = vg_col_slice(&db.cols[P.pset.idx[j]], off);
                L->n_rows = n;
                L->sel = NULL;
                L->sel_n = 0;
            }
            L->row_base = stream_pos + off;   /* logical position of the launch's first row */
            L->li_base = off;
            settled = !run_batch(&P, &T, L, &S, n);
        }
        vg_dbatch_release(&db);
        stream_pos += n_logical;
        batch_idx++;
    }
    VecBatch *res = emit_result(A, &P, &T);
    vg_dfree(T.block);
    vg_dfree(S.cache);
    vg_dfree(S.counters);
    free(L);
    free(need);
    return res;
}

static void agg_free(VecNode *self) {
    VgAgg *A = (VgAgg *)self;
    A->ga.child->free_node(A->ga.child);
    for (int k = 0; k < A->ga.n_keys; k++) free(A->ga.key_names[k]);
    free(A->ga.key_names);
    for (int a = 0; a < A->ga.n_aggs; a++) {
        free(A->ga.agg_specs[a].output_name);
        free(A->ga.agg_specs[a].input_col);
    }
    free(A->ga.agg_specs);
    vg_schema_free(&A->ga.base.output_schema);
    free(A);
}

GroupAggNode *group_agg_node_create(VecNode *child, int n_keys, char **key_names, int n_aggs,
                                    AggSpec *agg_specs, const char *temp_dir) {
    vg_ensure_init();
    if (n_keys > VG_MAX_KEYS) vg_fail("GPU group-agg supports at most %d key columns", VG_MAX_KEYS);
    if (n_aggs > VG_MAX_OUTS) vg_fail("GPU group-agg supports at most %d aggregates", VG_MAX_OUTS);
    const VecSchema *cs = &child->output_schema;
    for (int k = 0; k < n_keys; k++) {
        int idx = vg_schema_find(cs, key_names[k]);
        if (temp_dir && idx < 0) vg_fail("group_by: column not found: %s", key_names[k]);
        if (idx >= 0 && cs->col_types[idx] == VEC_STRING)
            vg_fail("string group keys are not supported by the GPU group-agg (%s)", key_names[k]);
    }
    VgAgg *A = (VgAgg *)vg_xcalloc(1, sizeof(VgAgg));
    A->ga.child = child;
    A->ga.n_keys = n_keys;
    A->ga.key_names = key_names;
    A->ga.n_aggs = n_aggs;
    A->ga.agg_specs = agg_specs;
    A->sorted = (temp_dir != NULL && n_keys > 0);
    A->ga.use_sorted = A->sorted;
    int n_out = n_keys + n_aggs;
    char **names = (char **)vg_xcalloc((size_t)(n_out ? n_out : 1), sizeof(char *));
    VecType *types = (VecType *)vg_xcalloc((size_t)(n_out ? n_out : 1), sizeof(VecType));
    for (int k = 0; k < n_keys; k++) {
        names[k] = key_names[k];
        int idx = vg_schema_find(cs, key_names[k]);
        types[k] = idx >= 0 ? cs->col_types[idx] : VEC_DOUBLE;
    }
    for (int a = 0; a < n_aggs; a++) {
        names[n_keys + a] = agg_specs[a].output_name;
        types[n_keys + a] = VEC_DOUBLE;
    }
    A->ga.base.output_schema = vg_schema_make(n_out, names, types);
    free(names);
    free(types);
    A->ga.base.next_batch = agg_next;
    A->ga.base.free_node = agg_free;
    A->ga.base.kind = "GroupAggNode";
    return &A->ga;
}
