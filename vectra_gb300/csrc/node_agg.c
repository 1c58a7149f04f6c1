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
#include <time.h>
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
    const VgProg *prog;       /* or a general program over them, run per batch */
    int prog_col[VG_MAX_COLS];/* its columns as source columns */
    const VgColSet *fset;
    VgColSet pset;            /* kernel probe column table -> src column */
    VgColSet bset;            /* kernel build column table -> right column */
    int n_keys, n_accs, n_out;
    VgValue key[VG_MAX_KEYS];
    int32_t key_type[VG_MAX_KEYS];
    VgAccSpec acc[VG_MAX_ACCS];
    VgFinish fin[VG_MAX_OUTS];
    int fail;                 /* resolution failed: not fusable */
    /* string group keys: grouped by their dictionary codes (strdict.c) */
    int allow_str;            /* resolving a key: a string source column is allowed */
    int n_str;
    int str_key[VG_MAX_KEYS]; /* key k is a string column of the source */
    int str_col[VG_MAX_KEYS]; /* that source column */
    VgDict *dict[VG_MAX_KEYS];
    int dict_owner[VG_MAX_KEYS];
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
    return t != VEC_STRING || P->allow_str;
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
        P->allow_str = 1;
        const int ok = resolve_value(P, ga->key_names[k], &P->key[k]);
        P->allow_str = 0;
        if (!ok) return 0;
        if (P->key[k].type == VEC_STRING) {
            /* a plain column of the source, grouped by its codes */
            if (P->key[k].op != 0 || P->key[k].a.side != VG_SIDE_PROBE) return 0;
            P->key[k].type = P->key[k].a.type = VEC_INT64;
            P->str_key[k] = 1;
            P->str_col[k] = P->pset.idx[P->key[k].a.col];
            P->n_str++;
        }
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
    if (vg_is_join(n) && (vg_join_kind(n) == JOIN_INNER || vg_join_kind(n) == JOIN_LEFT) &&
        !vg_join_has_string_keys(n)) {
        P->join = n;
        n = vg_join_left(n);
    }
    if (vg_is_filter(n)) {
        VecNode *fc;
        const VgColSet *fs;
        const VgPred *pr = vg_filter_cnf(n, &fc, &fs);
        const VgProg *pg = pr ? NULL : vg_filter_program(n, &fc, &fs);
        if (pr) { P->filter = n; P->pred = pr; P->fset = fs; n = fc; }
        else if (pg) { P->filter = n; P->prog = pg; P->fset = fs; n = fc; }
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
    int deferred;             /* launches not yet checked (dense cache) */
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
/* The dense cache's deferred-row marks (see VgAggLaunch.defer_bits): a
 * count word, then one bit per row and double-sum accumulator; kept and
 * reused by later calls, cleared before every launch. */
static void *g_defer;
static size_t g_defer_cap;

static void defer_prepare(VgAggLaunch *L, int64_t n_logical) {
    L->defer_bits = NULL;
    L->defer_n = NULL;
    L->defer_words = 0;
    if (!L->dense || L->part) return;
    int nf = 0;
    for (int a = 0; a < L->n_accs; a++) nf += L->acc[a].cls == VG_ACC_SUM_F64;
    if (nf == 0) return;
    const int64_t words = (n_logical + 31) / 32;
    const size_t bytes = 256 + (size_t)nf * (size_t)words * 4;
    if (g_defer_cap < bytes) {
        vg_dfree(g_defer);
        g_defer = NULL;
        g_defer_cap = 0;
        g_defer = vg_dmalloc_kept(bytes);
        g_defer_cap = bytes;
    }
    vg_dmemset(g_defer, 0, bytes);
    L->defer_n = (uint32_t *)g_defer;
    L->defer_bits = (uint32_t *)((char *)g_defer + 256);
    L->defer_words = words;
}

static int run_batch(Plan *P, Table *T, VgAggLaunch *L, Spill *S, int64_t n_logical) {
    int sms = vgk_num_sms();
    defer_prepare(L, n_logical);
    /* spill space for this launch */
    /* a dense cache holds every group: nothing misses it, so rows never
     * spill (a spill would be reported, not lost) */
    int64_t need_rows = L->dense ? 65536 : n_logical + 65536;
    if (!S->counters) S->counters = (uint32_t *)vg_dmalloc(256);
    if (g_spill_rows_cap < need_rows) {
        vg_dfree(g_spill_rows);
        g_spill_rows = (int64_t *)vg_dmalloc_kept((size_t)need_rows * 16);   /* reused by later calls */
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
    /* a dense cache holds every group and the table cannot outgrow its
     * first allocation: nothing spills, so a stream of batches is checked
     * once, after its last launch (check_deferred), and the host does not
     * wait for each batch's kernel before pulling the next batch */
    const int deferred = L->dense != 0;
    for (;;) {
        if (!deferred || !S->deferred) vg_dmemset(S->counters, 0, 8);
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
        if (deferred) {
            S->deferred = 1;
            return 0;
        }
        /* spill counters, error word and groups used: three copies, one wait */
        uint32_t *hw = (uint32_t *)vg_pinned_scratch(16);
        vg_d2h(hw, S->counters, 8);
        vg_d2h(hw + 2, T->gt.err, 4);
        vg_d2h(hw + 3, T->gt.n_used, 4);
        vg_sync();
        uint32_t c[2] = {hw[0], hw[1]}, err = hw[2], used = hw[3];
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

/* The status of deferred launches (dense cache): queued for the host
 * behind them (no wait here); check_deferred reads it once the stream has
 * synchronised -- the result's first read-back waits for it. */
static uint32_t *queue_deferred_status(Table *T, Spill *S) {
    uint32_t *hw = vg_pinned_status();
    vg_d2h(hw, S->counters, 8);
    vg_d2h(hw + 2, T->gt.err, 4);
    S->deferred = 0;
    return hw;
}

/* an error, or rows that left the cache (which a dense cache cannot lose),
 * fails the call */
static void check_deferred(const uint32_t *hw) {
    const uint32_t err = hw[2];
    if (err & (VG_ERR_WAIT | VG_ERR_PROG)) vg_fail("group-agg kernel error (code %u)", err);
    if ((err & (VG_ERR_FULL | VG_ERR_SPILL)) || hw[0] || hw[1])
        vg_fail("group-agg: rows left a dense group cache (%u rows, %u entries, code %u)", hw[0], hw[1], err);
}

/* results up to this size are read back in one page-locked copy */
#define kSmallResultBytes ((size_t)8 << 20)

/* ------------------------------------------------------------------ */
/* string group keys                                                   */
/* ------------------------------------------------------------------ */

/* one dictionary per distinct string key column */
static void str_dicts_begin(Plan *P) {
    for (int k = 0; k < P->n_keys; k++) {
        if (!P->str_key[k]) continue;
        for (int k2 = 0; k2 < k; k2++)
            if (P->str_key[k2] && P->str_col[k2] == P->str_col[k]) P->dict[k] = P->dict[k2];
        if (!P->dict[k]) {
            P->dict[k] = vg_dict_new();
            P->dict_owner[k] = 1;
        }
    }
}

static void str_dicts_free(Plan *P) {
    for (int k = 0; k < P->n_keys; k++)
        if (P->dict_owner[k]) vg_dict_free(P->dict[k]);
}

/* The filter program over the batch: its selection (composed with any
 * the batch had) replaces the batch's, on the device.  Returns the device
 * block holding it, freed by the caller after the batch's launches. */
static void *filter_batch(Plan *P, VgDBatch *db) {
    VgCol cols[VG_MAX_COLS];
    const int nc = P->fset->n;
    for (int j = 0; j < nc; j++) cols[j] = db->cols[P->prog_col[j]];
    const int64_t n_in = db->d_sel ? db->sel_n : db->n_rows;
    const size_t sb = vgk_filter_scratch_bytes(n_in);
    char *blk = (char *)vg_dmalloc(sb + (size_t)(n_in > 0 ? n_in : 1) * 4 + 256);
    int32_t *out = (int32_t *)(blk + sb);
    int64_t cnt = 0;
    vg_check_rc(vgk_filter_prog(cols, nc, P->prog, db->n_rows, db->d_sel, db->sel_n, out, &cnt, blk, sb, vg_stream()),
                "filter");
    db->d_sel = out;
    db->sel_n = cnt;
    return blk;
}

/* Each string key column of the batch replaced by the int64 codes of its
 * logical rows (validity unchanged); returns the device block of the
 * codes, freed by the caller after the batch's launches. */
static void *str_encode_batch(Plan *P, VgDBatch *db) {
    const int64_t n = db->n_rows, n_logical = db->d_sel ? db->sel_n : db->n_rows;
    const size_t per = a256((size_t)(n ? n : 1) * 8);
    char *blk = (char *)vg_dmalloc(per * (size_t)P->n_keys);
    for (int k = 0; k < P->n_keys; k++) {
        if (!P->dict_owner[k]) continue;
        VgCol *c = &db->cols[P->str_col[k]];
        if (c->type != VEC_STRING) vg_fail("group_by: key column %d is not a string column", P->str_col[k]);
        int64_t *codes = (int64_t *)(blk + per * (size_t)k);
        vg_dict_encode(P->dict[k], c, db->d_sel, n_logical, 1, codes,
                       db->str_chars ? db->str_chars[P->str_col[k]] : -1);
        c->type = VEC_INT64;
        c->data = codes;
    }
    return blk;
}

static VecBatch *emit_result(VgAgg *A, Plan *P, Table *T, const uint32_t *deferred) {
    GroupAggNode *ga = &A->ga;
    uint32_t n = 0;
    int32_t *d_slots = (int32_t *)vg_dmalloc((size_t)T->gt.cap * 4 + 16);
    vg_check_rc(vgk_group_table_compact(&T->gt, d_slots, &n, vg_stream()), "group compact");
    if (deferred) check_deferred(deferred);     /* read back behind the launches, before the count */
    int64_t ng = n;
    /* key order of string keys: each group's code becomes the rank of its
     * string, then the groups sort as integer keys do */
    int32_t *sperm[VG_MAX_KEYS] = {0};
    int64_t *srank[VG_MAX_KEYS] = {0};
    const int str_ranked = A->sorted && ng > 1;
    for (int k = 0; str_ranked && k < P->n_keys; k++) {
        if (!P->str_key[k]) continue;
        vg_dict_order(P->dict[k], &sperm[k], &srank[k]);
        vg_check_rc(vgk_group_keys_remap(&T->gt, k, d_slots, ng, srank[k], vg_stream()), "string key order");
    }
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
    /* a small result comes back in one copy of the whole output block
     * (page-locked, one wait); a large one column by column */
    const size_t out_bytes = per * (size_t)n_out + 4;
    const char *hb = NULL;
    if (out_bytes <= kSmallResultBytes) {
        char *pin = (char *)vg_pinned_scratch(out_bytes);
        vg_d2h(pin, blk, out_bytes);
        vg_sync();
        hb = pin;
    }
    for (int k = 0; k < ga->n_keys; k++) {
        if (P->str_key[k]) {
            if (!str_ranked) (void)vg_dict_size(P->dict[k]);    /* its error word, read back once */
            res->columns[k] = vg_dict_strings(P->dict[k], (const int64_t *)kout[k], kval[k],
                                              str_ranked ? sperm[k] : NULL, ng);
            res->col_names[k] = vg_xstrdup(ga->key_names[k]);
            vg_dfree(sperm[k]);
            vg_dfree(srank[k]);
            continue;
        }
        int t = P->key_type[k];
        VecArray arr = hb ? vg_column_from_host(VEC_INT64, hb + per * (size_t)k,
                                                hb + per * (size_t)k + a256((size_t)ng * 8 + 8), ng)
                          : vg_download_column(VEC_INT64, kout[k], kval[k], ng);
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
        const size_t o = per * (size_t)(ga->n_keys + a);
        res->columns[ga->n_keys + a] = hb ? vg_column_from_host(VEC_DOUBLE, hb + o, hb + o + a256((size_t)ng * 8 + 8), ng)
                                          : vg_download_column(VEC_DOUBLE, aout[a], aval[a], ng);
        res->col_names[ga->n_keys + a] = vg_xstrdup(ga->agg_specs[a].output_name);
    }
    uint32_t warn = 0;
    if (hb) {
        memcpy(&warn, hb + per * (size_t)n_out, 4);
    } else {
        vg_d2h(&warn, d_warn, 4);
        vg_sync();
    }
    vg_warn_count((long)warn);
    vg_dfree(blk);
    vg_dfree(d_slots);
    return res;
}

/* ------------------------------------------------------------------ */
/* partitioned aggregation (many groups, one int64 key, key order)     */
/* ------------------------------------------------------------------ */

/* For key-ordered output of a single int64 key with very many groups, the
 * group table does not fit on chip and every update would be a random
 * atomic in HBM.  Instead (k_pagg.cu, k_jit_pagg.cuh):
 *   1. the first batch's key column is sketched: distinct-key estimate D
 *      and key range; buckets = 2^p contiguous key ranges with about 3/4 of
 *      the groups one reducer CTA holds in each;
 *   2. per batch: rows per bucket (hist), bucket ranges (scan), and the
 *      fused kernel in partition mode writes each row with a valid key as
 *      a record into its bucket (NA keys go to a one-group table);
 *   3. the reducer aggregates every bucket in shared memory, orders its
 *      groups by key and stages their results; buckets with too many
 *      groups are split by their own key range (recursively);
 *   4. the staged results are compacted into the output columns, NA group
 *      last.
 * Buckets ascend with the key, so the output needs no global sort. */

typedef struct {
    uint64_t *rec;
    uint64_t *off;                 /* n_buckets + 1 */
    unsigned long long *cursor;    /* record ends after the partition pass */
} PRegion;

typedef struct {
    int G;                         /* groups per reducer CTA */
    int ctas;                      /* reducer CTAs per SM (1, 2, 4 or 8) */
    int rw;                        /* record words */
    int nb;                        /* buckets */
    int shift;
    uint64_t omin;
    int n_regions;
    PRegion reg[VG_PAGG_MAX_REGIONS];
    uint32_t *cnt;                 /* nb: rows per bucket (hist scratch) */
    unsigned long long *pcur;      /* nb cursors of the partition pass, VG_PAGG_CURSOR_STRIDE apart */
    uint32_t *err;
    Table na;                      /* the NA-key group */
    uint32_t *counters;            /* spill counters of the partition launch (never used) */
    uint64_t rows;                 /* records written (upper bound) */
    VgHostBufs *hb;                /* result columns, faulted in while the device works */
    size_t hb_bytes;               /* bytes of each */
    struct PTune *tune;            /* fan-out being tuned by this query, or NULL */
    int prof_prev;                 /* kernel timing state before the tuning query */
    double prof_base;              /* partition + reducer milliseconds before it */
} PAgg;

/* Host wall time of the partitioned path's phases, summed since load
 * (each phase ends in a device synchronisation, so its time includes its
 * device work): 0 sketch and setup, 1 partition (hist, scan, partition
 * kernel), 2 bucket reducer (and splits), 3 NA group and compaction into
 * the output columns, 4 waiting for the host result buffers, 5 copying
 * the result to the host; 6 the whole aggregation (its next_batch call). */
static double g_pagg_ms[7];

/* Host wall time of the hash-table aggregation path, summed since load:
 * 0 planning before the first batch (join build included), 1 the join
 * build alone, 2 the aggregation launches and their synchronisations, 3
 * the result (compaction, order, finish, copy to host), 4 the whole
 * next_batch call.  A dense cache's launches are waited for in 3 (their
 * status comes back with the result's first read-back). */
static double g_agg_ms[5];

double vgpu_agg_phase_ms(int phase) { return phase >= 0 && phase < 5 ? g_agg_ms[phase] : 0.0; }

static double now_ms(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec * 1e3 + (double)ts.tv_nsec * 1e-6;
}

double vgpu_pagg_phase_ms(int phase) { return phase >= 0 && phase < 7 ? g_pagg_ms[phase] : 0.0; }

static int env_int(const char *name, int dflt) {
    const char *e = getenv(name);
    return (e && *e) ? atoi(e) : dflt;
}

static int bitlen64(uint64_t x) {
    int b = 0;
    while (x) { b++; x >>= 1; }
    return b;
}

/* Whether this aggregation takes the partitioned path; decided on the
 * first batch.  VGPU_PAGG=0 never, =1 always when the plan allows it
 * (tests); otherwise when the batch has at least VGPU_PAGG_MIN_ROWS
 * logical rows and an estimated VGPU_PAGG_MIN_GROUPS distinct keys. */
/* ---- fan-out and reducer shape of the partitioned path, tuned per shape
 * class --------------------------------------------------------------
 *
 * The bucket count follows the key sketch: the fewest powers of two that
 * keep each bucket's groups at 3/4 of a reducer CTA's capacity, one
 * reducer CTA of 1024 threads per SM.  Tuning (vgpu_pagg_tune(1) or
 * VGPU_PAGG_TUNE=1) tries, one per query on the first queries of a shape
 * class (rows of the first batch, estimated groups, record words,
 * accumulators: powers of two), that count x1, x2 and x4 with one reducer
 * CTA per SM, x1 and x2 with two reducer CTAs of 512 threads per SM (each
 * holding half the groups, so the count itself doubles), and x1 with four
 * of 256 threads or eight of 128 (a quarter or an eighth of the groups
 * each) -- timed by
 * the device time of their partition and reducer launches -- and keeps the
 * fastest.  Fewer buckets than the sketch's count overflow the reducer's
 * capacity and are not tried.  The choice is appended to the file named by
 * VGPU_TUNE_FILE (the query sets' tuning file; a line
 * "pagg.<shape> <reducer CTAs per SM> <doublings> 0 <ms> <candidates>")
 * and read back by later processes. */
#define PT_CANDS 7
static const int kPtDoublings[PT_CANDS] = {0, 1, 2, 0, 1, 0, 0};
static const int kPtCtas[PT_CANDS] = {1, 1, 1, 2, 2, 4, 8};
typedef struct PTune {
    char shape[96];
    int recorded, cand, next;
    double ms[PT_CANDS];
} PTune;
static PTune g_pt[64];
static int g_pt_n, g_pt_loaded, g_pt_armed = -1;
static int g_pt_last = -1;
static double g_pt_last_ms;
static char g_pt_last_shape[96];

void vgpu_pagg_tune(int on) { g_pt_armed = on ? 1 : 0; }

/* The last decision: the shape class, the reducer CTAs per SM, the
 * measured milliseconds; returns the doublings over the sketch's bucket
 * count (-1: none yet). */
int vgpu_pagg_tuned(char *shape, int shape_bytes, int *ctas, double *ms) {
    if (shape && shape_bytes > 0) snprintf(shape, (size_t)shape_bytes, "%s", g_pt_last_shape);
    if (ms) *ms = g_pt_last_ms;
    if (ctas) *ctas = g_pt_last >= 0 ? kPtCtas[g_pt_last] : 0;
    return g_pt_last >= 0 ? kPtDoublings[g_pt_last] : -1;
}

static PTune *pt_find(const char *shape, int create) {
    for (int i = 0; i < g_pt_n; i++)
        if (strcmp(g_pt[i].shape, shape) == 0) return &g_pt[i];
    if (!create || g_pt_n == (int)(sizeof(g_pt) / sizeof(g_pt[0]))) return NULL;
    PTune *t = &g_pt[g_pt_n++];
    memset(t, 0, sizeof(*t));
    snprintf(t->shape, sizeof(t->shape), "%s", shape);
    return t;
}

static void pt_load(void) {
    if (g_pt_loaded) return;
    g_pt_loaded = 1;
    const char *path = getenv("VGPU_TUNE_FILE");
    if (!path || !*path) return;
    FILE *f = fopen(path, "r");
    if (!f) return;
    char shape[96];
    int threads = 0, mult = 0, cands = 0;
    long long chunk = 0;
    double ms = 0;
    while (fscanf(f, "%95s %d %lld %d %lf %d", shape, &threads, &chunk, &mult, &ms, &cands) == 6) {
        if (strncmp(shape, "pagg.", 5) != 0) continue;
        int c = -1;
        for (int k = 0; k < PT_CANDS; k++)
            if (kPtCtas[k] == threads && kPtDoublings[k] == chunk) c = k;
        if (c < 0) continue;
        PTune *t = pt_find(shape, 1);
        if (!t) break;
        t->recorded = 1;           /* the last line of a shape wins */
        t->cand = c;
        t->ms[c] = ms;
    }
    fclose(f);
}

static void pt_save(const PTune *t, double ms) {
    const char *path = getenv("VGPU_TUNE_FILE");
    if (!path || !*path) return;
    FILE *f = fopen(path, "a");
    if (!f) return;
    fprintf(f, "%s %d %d 0 %.6f %d\n", t->shape, kPtCtas[t->cand], kPtDoublings[t->cand], ms, PT_CANDS);
    fclose(f);
}

static int lg2d(double x) {
    int b = 0;
    while (x >= 2.0 && b < 62) { x /= 2.0; b++; }
    return b;
}

/* the partition and reducer launches' device time so far (events around
 * each launch, recorded after its kernel is compiled) */
static double pt_kernel_ms(void) {
    return vgpu_profile_ms(VG_PROF_CLASS_AGG, NULL) + vgpu_profile_ms(VG_PROF_CLASS_PAGG, NULL);
}

static void pt_start(PAgg *pg) {
    pg->prof_prev = vg_prof_force_on();
    pg->prof_base = pt_kernel_ms();
}

/* after the query's last launch: its time for the candidate it ran */
static void pt_finish(PAgg *pg) {
    if (!pg->tune) return;
    const double ms = pt_kernel_ms() - pg->prof_base;
    vg_prof_restore(pg->prof_prev);
    PTune *t = pg->tune;
    pg->tune = NULL;
    t->ms[t->next] = ms;
    g_pt_last = t->next;
    g_pt_last_ms = ms;
    if (++t->next == PT_CANDS) {
        int best = 0;
        for (int c = 1; c < PT_CANDS; c++)
            if (t->ms[c] < t->ms[best]) best = c;
        t->cand = best;
        t->recorded = 1;
        pt_save(t, t->ms[best]);
    }
}

/* a tuning query that failed: its candidate is tried again next time */
static void pt_free(PAgg *pg) {
    if (pg->tune) vg_prof_restore(pg->prof_prev);
    pg->tune = NULL;
}

static PAgg *pagg_begin(VgAgg *A, Plan *P, VgAggLaunch *L, const VgDBatch *db) {
    const int mode = env_int("VGPU_PAGG", -1);
    if (mode == 0 || !A->sorted || P->n_keys != 1 || P->key[0].op != 0 || P->key[0].a.side != VG_SIDE_PROBE ||
        P->key[0].a.type != VEC_INT64 || L->dense || L->track_first)
        return NULL;
    const int64_t n = db->d_sel ? db->sel_n : db->n_rows;
    if (mode != 1 && n < (int64_t)env_int("VGPU_PAGG_MIN_ROWS", 1 << 22)) return NULL;
    L->part = 1;
    const int ok = vgk_agg_jit_ok(L);
    const int G = ok ? vgk_pagg_groups(L) : 0;
    L->part = 0;
    if (!G) return NULL;
    const VgCol *kc = &db->cols[P->pset.idx[P->key[0].a.col]];
    uint32_t *regs = (uint32_t *)vg_dmalloc(4096 * 4 + 256);
    unsigned long long *mm = (unsigned long long *)((char *)regs + 4096 * 4);
    double d = 0.0;
    uint64_t hmm[3];
    vg_check_rc(vgk_pagg_sketch(kc, n, db->d_sel, regs, mm, &d, hmm, vg_stream()), "partitioned aggregation sketch");
    vg_dfree(regs);
    if (mode != 1 && d < (double)env_int("VGPU_PAGG_MIN_GROUPS", 1 << 18)) return NULL;
    PAgg *pg = (PAgg *)vg_xcalloc(1, sizeof(PAgg));
    pg->G = env_int("VGPU_PAGG_G", G);          /* a smaller G exercises the bucket split (tests) */
    if (pg->G < 1 || pg->G > G) pg->G = G;
    pg->ctas = 1;
    L->part = 1;
    pg->rw = vgk_pagg_record_words(L);
    L->part = 0;
    /* the recorded (or, while tuning, the next) fan-out and reducer shape
     * of this shape class, unless a test forces the buckets or G */
    const int forced = env_int("VGPU_PAGG_BUCKETS", 0) > 1 || env_int("VGPU_PAGG_G", 0) > 0;
    int doublings = 0;
    if (!forced) {
        char shape[96];
        snprintf(shape, sizeof(shape), "pagg.r%d.d%d.w%d.a%d", lg2d((double)n), lg2d(d), pg->rw, P->n_accs);
        if (g_pt_armed < 0) g_pt_armed = env_int("VGPU_PAGG_TUNE", 0) != 0;
        pt_load();
        PTune *t = pt_find(shape, g_pt_armed);
        int c = 0;
        if (t && t->recorded) {
            c = t->cand;
            g_pt_last = c;
            g_pt_last_ms = t->ms[c];
        } else if (t) {
            c = t->next;
            pg->tune = t;
            pt_start(pg);
        }
        snprintf(g_pt_last_shape, sizeof(g_pt_last_shape), "%s", shape);
        doublings = kPtDoublings[c];
        if (kPtCtas[c] > 1) {
            L->part = 1;
            const int Gc = vgk_pagg_groups_for(L, kPtCtas[c]);
            L->part = 0;
            if (Gc > 0) {
                pg->ctas = kPtCtas[c];
                pg->G = Gc;
            }
        }
    }
    /* buckets: about 3/4 of G groups each */
    const double want = d / (0.75 * (double)pg->G);
    int nb = 2;
    while ((double)nb < want && nb < (1 << 20)) nb <<= 1;
    if (env_int("VGPU_PAGG_BUCKETS", 0) > 1) nb = env_int("VGPU_PAGG_BUCKETS", 0);
    for (int k = 0; k < doublings && nb < (1 << 20); k++) nb <<= 1;
    pg->omin = hmm[2] ? hmm[0] : 0;
    const int bits = hmm[2] ? bitlen64(hmm[1] - hmm[0]) : 0;
    int lb = 0;
    while ((1 << lb) < nb) lb++;
    if (bits < lb) {            /* fewer distinct key values than buckets */
        lb = bits > 0 ? bits : 1;
        nb = 1 << lb;
    }
    pg->nb = nb;
    pg->shift = bits > lb ? bits - lb : 0;
    pg->cnt = (uint32_t *)vg_dmalloc((size_t)nb * 4 + 256);
    pg->pcur = (unsigned long long *)vg_dmalloc((size_t)nb * VG_PAGG_CURSOR_STRIDE * 8 + 256);
    pg->err = (uint32_t *)vg_dmalloc(256);
    vg_dmemset(pg->err, 0, 4);
    pg->counters = (uint32_t *)vg_dmalloc(256);
    table_alloc(&pg->na, P, 1024);
    /* the host result columns (key + outputs) for about the estimated
     * number of groups: their fresh pages are faulted in by background
     * threads during the device passes */
    const double est = d * 1.04 + 4096.0;
    if (est * 8.0 >= (double)(4 << 20) && est < 4e9)
    {
        pg->hb_bytes = (size_t)est * 8;
        pg->hb = vg_host_bufs_begin(1 + A->ga.n_aggs, pg->hb_bytes);
    }
    return pg;
}

/* Step 2 for one batch: its rows become records of a new region.  With at
 * most VG_PAGG_CTA_BUCKETS buckets, each CTA of the partition kernel
 * owns a range of every bucket, counted beforehand over exactly its rows,
 * and hands positions out with shared-memory counters; otherwise the rows
 * claim positions with global atomics on per-bucket cursors. */
static void pagg_batch(PAgg *pg, Plan *P, VgAggLaunch *L, const VgDBatch *db, int64_t stream_pos, int64_t batch_idx) {
    if (pg->n_regions == VG_PAGG_MAX_REGIONS)
        vg_fail("partitioned aggregation: more than %d input batches", VG_PAGG_MAX_REGIONS);
    const int64_t n = db->d_sel ? db->sel_n : db->n_rows;
    const VgCol *kc = &db->cols[P->pset.idx[P->key[0].a.col]];
    const int nb = pg->nb;
    PRegion *R = &pg->reg[pg->n_regions++];
    R->off = (uint64_t *)vg_dmalloc((size_t)(nb + 1) * 8 + 256);
    R->cursor = (unsigned long long *)vg_dmalloc((size_t)nb * 8 + 256);

    for (int j = 0; j < P->pset.n; j++) L->pcols[j] = db->cols[P->pset.idx[j]];
    if (db->d_sel) {
        L->n_rows = db->n_rows;
        L->sel = db->d_sel;
        L->sel_n = n;
    } else {
        L->n_rows = n;
        L->sel = NULL;
        L->sel_n = 0;
    }
    L->row_base = stream_pos;
    L->li_base = 0;
    L->batch_idx = batch_idx;
    L->part = 1;
    L->gt = pg->na.gt;
    vg_dmemset(pg->counters, 0, 8);
    L->spill_rows = NULL;
    L->spill_rows_n = pg->counters;
    L->spill_rows_cap = 0;
    L->spill_cache = NULL;
    L->spill_cache_n = pg->counters + 1;
    L->spill_cache_cap = 0;
    L->replay = NULL;
    L->replay_n = 0;
    L->po.omin = pg->omin;
    L->po.shift = pg->shift;
    L->po.n_buckets = nb;
    L->po.rec_words = pg->rw;
    L->po.n_vals = pg->rw - 2;
    L->po.err = pg->err;
    L->po.cursor = NULL;
    L->po.cta_off = NULL;
    L->po.start = R->off;
    L->po.end = R->off + 1;

    /* per-CTA ranges: every position below 2^32 (n rows or fewer records) */
    const int cta = nb <= VG_PAGG_CTA_BUCKETS && (uint64_t)n < ((uint64_t)1 << 32) &&
                    env_int("VGPU_PAGG_ATOMIC", 0) == 0;
    uint64_t *cta_off = NULL;
    if (cta) {
        /* the kernel's geometry decides which rows each CTA counts */
        L->po.cta_off = (const uint64_t *)R->off;   /* non-null: selects the per-CTA kernel */
        int grid = 0;
        int64_t tile = 0;
        if (vgk_agg_jit_geometry(L, n, &grid, &tile) != 0) vg_fail("partitioned aggregation: %s", vgk_jit_error());
        const int64_t cells = (int64_t)nb * grid;
        uint32_t *m = (uint32_t *)vg_dmalloc((size_t)cells * 4 + 256);
        cta_off = (uint64_t *)vg_dmalloc((size_t)(cells + 1) * 8 + 256);
        unsigned long long *sums = (unsigned long long *)vg_dmalloc((size_t)(cells / 16384 + 2) * 8 + 256);
        vg_check_rc(vgk_pagg_hist_cta(kc, n, db->d_sel, pg->omin, pg->shift, nb, grid, tile, m, vg_stream()),
                    "partitioned aggregation hist");
        vg_check_rc(vgk_scan_u32_u64(m, cells, cta_off, sums, vg_stream()), "partitioned aggregation scan");
        /* bucket starts: the offsets of each bucket's first CTA (and the total) */
        vg_check_rc(vgk_pagg_cursor_compact((const unsigned long long *)cta_off, grid, nb + 1,
                                            (unsigned long long *)R->off, vg_stream()),
                    "partitioned aggregation offsets");
        vg_dfree(sums);
        vg_dfree(m);
        L->po.cta_off = cta_off;
    } else {
        vg_check_rc(vgk_pagg_hist(kc, n, db->d_sel, pg->omin, pg->shift, nb, pg->cnt, vg_stream()),
                    "partitioned aggregation hist");
        vg_check_rc(vgk_pagg_scan(pg->cnt, NULL, nb, R->off, pg->pcur, VG_PAGG_CURSOR_STRIDE, vg_stream()),
                    "partitioned aggregation scan");
        L->po.cursor = pg->pcur;
    }
    uint64_t total = 0;
    vg_d2h(&total, R->off + nb, 8);
    vg_sync();
    R->rec = (uint64_t *)vg_dmalloc((size_t)(total ? total : 1) * (size_t)pg->rw * 8 + 256);
    if ((uintptr_t)R->rec & 31)       /* records are written and read as aligned 32-byte words */
        vg_fail("partitioned aggregation: record area not 32-byte aligned");
    pg->rows += total;
    L->po.rec = R->rec;
    L->po.total = total;
    if (n > 0) {
        const int rc = vgk_agg_launch_jit(L, n, vg_stream());
        if (rc <= 0) vg_fail("partitioned aggregation: %s", rc < 0 ? vgk_jit_error() : "plan not covered");
    }
    L->part = 0;
    /* record ends: the whole bucket (holes marked) or the cursors */
    if (cta)
        vg_check_rc(vgk_pagg_cursor_compact((const unsigned long long *)(R->off + 1), 1, nb, R->cursor, vg_stream()),
                    "partitioned aggregation cursors");
    else
        vg_check_rc(vgk_pagg_cursor_compact(pg->pcur, VG_PAGG_CURSOR_STRIDE, nb, R->cursor, vg_stream()),
                    "partitioned aggregation cursors");
    uint32_t err[2] = {0, 0};
    vg_d2h(&err[0], pg->err, 4);
    vg_d2h(&err[1], pg->na.gt.err, 4);
    vg_sync();
    vg_dfree(cta_off);
    if (err[0] | err[1]) vg_fail("partitioned aggregation: partition kernel error (codes %u, %u)", err[0], err[1]);
}

typedef struct {
    uint64_t *stage;               /* host leaf arrays (refinement) */
    uint64_t *gc;
    int64_t n, cap;
} Leaves;

static void leaves_push(Leaves *lv, uint64_t stage, uint64_t gc) {
    if (lv->n == lv->cap) {
        lv->cap = lv->cap ? 2 * lv->cap : 1024;
        lv->stage = (uint64_t *)realloc(lv->stage, (size_t)lv->cap * 8);
        lv->gc = (uint64_t *)realloc(lv->gc, (size_t)lv->cap * 8);
        if (!lv->stage || !lv->gc) vg_fail("out of host memory");
    }
    lv->stage[lv->n] = stage;
    lv->gc[lv->n] = gc;
    lv->n++;
}

/* The reducer over buckets [b0, b0 + n) of B (a level of nb buckets;
 * gc: 2 nb words of device scratch, groups then overflow flags). */
static void pagg_reduce_launch(PAgg *pg, VgAggLaunch *L, const Plan *P, VgPaggReduce *B, const uint64_t *d_stage_off,
                               uint32_t *gc, int nb, unsigned int *ticket, int b0, int n) {
    vg_dmemset(ticket, 0, 4);
    B->bucket_base = b0;
    B->n_buckets = n;
    B->stage_off = d_stage_off;
    B->gc = gc;
    B->ovf = gc + nb;
    B->ticket = ticket;
    if (vgk_pagg_reduce(L, P->fin, P->n_out, pg->G, pg->ctas, B, vg_stream()) != 0)
        vg_fail("partitioned aggregation reduce: %s", vgk_jit_error());
}

static void pagg_reduce_level(PAgg *pg, VgAggLaunch *L, const Plan *P, VgPaggReduce *B, int nb,
                              const uint64_t *d_stage_off, Leaves *lv, int depth);

/* After the launch over [b0, b0 + n): the leaves of those buckets in key
 * order; a bucket with more groups than a CTA holds is split by its own
 * key range into up to 256 sub-buckets, reduced in turn (recursively). */
static void pagg_reduce_collect(PAgg *pg, VgAggLaunch *L, const Plan *P, VgPaggReduce *B,
                                const uint64_t *d_stage_off, const uint32_t *gc, int nb, int b0, int n, Leaves *lv,
                                int depth) {
    uint32_t *h = (uint32_t *)vg_xcalloc((size_t)n * 2 + 1, 4);
    uint64_t *hs = (uint64_t *)vg_xcalloc((size_t)n + 1, 8);
    uint32_t err = 0;
    vg_d2h(h, gc + b0, (size_t)n * 4);
    vg_d2h(h + n, gc + nb + b0, (size_t)n * 4);
    vg_d2h(hs, d_stage_off + b0, (size_t)n * 8);
    vg_d2h(&err, B->err, 4);
    vg_sync();
    if (err) vg_fail("partitioned aggregation: reduce kernel error (code %u)", err);
    for (int i = 0; i < n; i++) {
        const int b = b0 + i;
        if (!h[n + i]) {
            leaves_push(lv, hs[i], h[i]);
            continue;
        }
        if (depth > 16) vg_fail("partitioned aggregation: bucket split did not converge");
        uint64_t rows = 0;
        for (int r = 0; r < B->n_regions; r++) {
            uint64_t ra = 0, re = 0;
            vg_d2h(&ra, B->roff[r] + b, 8);
            vg_d2h(&re, B->rend[r] + b, 8);
            vg_sync();
            rows += re - ra;
        }
        unsigned long long *mm = (unsigned long long *)vg_dmalloc(256);
        uint64_t hmm[3];
        vg_check_rc(vgk_pagg_rec_minmax(B, b, rows, mm, hmm, vg_stream()), "partitioned aggregation split range");
        vg_dfree(mm);
        const int bits = bitlen64(hmm[1] - hmm[0]);
        if (bits == 0) vg_fail("partitioned aggregation: one key overflowed a bucket");
        const int lb = bits < 8 ? bits : 8;
        const int nb2 = 1 << lb;
        const int shift2 = bits - lb;
        uint32_t *cnt2 = (uint32_t *)vg_dmalloc((size_t)nb2 * 4 + 256);
        uint64_t *off2 = (uint64_t *)vg_dmalloc((size_t)(nb2 + 1) * 8 + 256);
        unsigned long long *cur2 = (unsigned long long *)vg_dmalloc((size_t)nb2 * 8 + 256);
        uint64_t *rec2 = (uint64_t *)vg_dmalloc((size_t)(rows ? rows : 1) * (size_t)pg->rw * 8 + 256);
        if ((uintptr_t)rec2 & 31) vg_fail("partitioned aggregation: record area not 32-byte aligned");
        vg_check_rc(vgk_pagg_rec_split(B, b, rows, hmm[0], shift2, nb2, cnt2, off2, cur2, rec2, pg->err, vg_stream()),
                    "partitioned aggregation split");
        uint64_t *hoff = (uint64_t *)vg_xcalloc((size_t)nb2 + 1, 8);
        vg_d2h(hoff, off2, (size_t)(nb2 + 1) * 8);
        vg_d2h(&err, pg->err, 4);
        vg_sync();
        if (err) vg_fail("partitioned aggregation: split kernel error (code %u)", err);
        for (int j = 0; j < nb2; j++) hoff[j] += hs[i];
        uint64_t *st2 = (uint64_t *)vg_dmalloc((size_t)nb2 * 8 + 256);
        vg_h2d(st2, hoff, (size_t)nb2 * 8);
        VgPaggReduce B2 = *B;
        B2.n_regions = 1;
        for (int r = 1; r < VG_PAGG_MAX_REGIONS; r++) { B2.rec[r] = NULL; B2.roff[r] = NULL; B2.rend[r] = NULL; }
        B2.omin = hmm[0];
        B2.shift = shift2;
        B2.rec[0] = rec2;
        B2.roff[0] = off2;
        B2.rend[0] = cur2;
        pagg_reduce_level(pg, L, P, &B2, nb2, st2, lv, depth + 1);
        vg_sync();
        free(hoff);
        vg_dfree(st2);
        vg_dfree(rec2);
        vg_dfree(cur2);
        vg_dfree(off2);
        vg_dfree(cnt2);
    }
    free(h);
    free(hs);
}

/* Every bucket of a level, in one launch. */
static void pagg_reduce_level(PAgg *pg, VgAggLaunch *L, const Plan *P, VgPaggReduce *B, int nb,
                              const uint64_t *d_stage_off, Leaves *lv, int depth) {
    uint32_t *gc = (uint32_t *)vg_dmalloc((size_t)nb * 8 + 256);
    unsigned int *ticket = (unsigned int *)vg_dmalloc(256);
    pagg_reduce_launch(pg, L, P, B, d_stage_off, gc, nb, ticket, 0, nb);
    pagg_reduce_collect(pg, L, P, B, d_stage_off, gc, nb, 0, nb, lv, depth);
    vg_dfree(ticket);
    vg_dfree(gc);
}

/* Staging positions and output rows of the leaves [l0, l1) on the device:
 * n + 1 staging positions, then n + 1 output rows relative to the first
 * leaf's; *rows: their groups. */
static uint64_t *leaf_arrays(const Leaves *lv, int64_t l0, int64_t l1, int64_t *rows) {
    const int64_t n = l1 - l0;
    uint64_t *h = (uint64_t *)vg_xcalloc((size_t)(2 * n + 2), 8);
    int64_t run = 0;
    for (int64_t i = 0; i < n; i++) {
        h[i] = lv->stage[l0 + i];
        h[n + 1 + i] = (uint64_t)run;
        run += (int64_t)lv->gc[l0 + i];
    }
    h[2 * n + 1] = (uint64_t)run;
    uint64_t *d = (uint64_t *)vg_dmalloc((size_t)(2 * n + 2) * 8 + 256);
    vg_h2d(d, h, (size_t)(2 * n + 2) * 8);
    vg_sync();
    free(h);
    *rows = run;
    return d;
}

/* Steps 3 and 4: the result batch. */
static VecBatch *pagg_end(PAgg *pg, VgAgg *A, Plan *P, VgAggLaunch *L) {
    GroupAggNode *ga = &A->ga;
    const int nb = pg->nb;
    const int n_out = ga->n_aggs;
    VgPaggReduce B;
    memset(&B, 0, sizeof(B));
    B.n_regions = pg->n_regions;
    B.rec_words = pg->rw;
    B.n_out = n_out;
    B.omin = pg->omin;
    B.shift = pg->shift;
    for (int r = 0; r < pg->n_regions; r++) {
        B.rec[r] = pg->reg[r].rec;
        B.roff[r] = pg->reg[r].off;
        B.rend[r] = pg->reg[r].cursor;
    }
    uint64_t *stage_off = (uint64_t *)vg_dmalloc((size_t)(nb + 1) * 8 + 256);
    vg_check_rc(vgk_pagg_scan(NULL, &B, nb, stage_off, NULL, 1, vg_stream()), "partitioned aggregation stage scan");
    uint64_t total = 0;
    vg_d2h(&total, stage_off + nb, 8);
    vg_sync();
    /* staging: one position per record plus the NA group's */
    const uint64_t cap = total + 1;
    size_t bytes = a256(cap * 8) + a256(cap * 4) + (size_t)n_out * a256(cap * 8);
    int n_fb = 0;
    for (int a = 0; a < P->n_accs; a++)
        if (P->acc[a].cls == VG_ACC_SUM_F64) n_fb++;
    bytes += (size_t)n_fb * 2 * a256(cap * 8);
    char *blk = (char *)vg_dmalloc(bytes + 256);
    size_t o = 0;
    B.st_key = (uint64_t *)(blk + o); o += a256(cap * 8);
    B.st_ok = (uint32_t *)(blk + o); o += a256(cap * 4);
    for (int j = 0; j < n_out; j++) { B.st_out[j] = (double *)(blk + o); o += a256(cap * 8); }
    for (int a = 0; a < P->n_accs; a++) {
        if (P->acc[a].cls != VG_ACC_SUM_F64) continue;
        B.fs[a] = (double *)(blk + o); o += a256(cap * 8);
        B.fc[a] = (double *)(blk + o); o += a256(cap * 8);
    }
    uint32_t *warn = (uint32_t *)vg_dmalloc(256);
    vg_dmemset(warn, 0, 4);
    B.warn = warn;
    B.err = pg->err;

    Leaves lv;
    memset(&lv, 0, sizeof(lv));
    const int n_cols = 1 + n_out;
    int64_t n_groups = 0;
    VecBatch *res = NULL;
    void *hcol[VG_MAX_OUTS + 1];
    memset(hcol, 0, sizeof(hcol));
    /* output validity: one bitmap per column for every possible row; each
     * emit ORs its bits in from its first output row */
    const size_t vwords = (size_t)((cap + 31) / 32) + 2;
    uint32_t *dval = (uint32_t *)vg_dmalloc((size_t)n_cols * a256(vwords * 4) + 256);
    vg_dmemset(dval, 0, (size_t)n_cols * a256(vwords * 4));
    uint32_t *vcol[VG_MAX_OUTS + 1];
    for (int c = 0; c < n_cols; c++) vcol[c] = (uint32_t *)((char *)dval + (size_t)c * a256(vwords * 4));

    /* The buckets in W runs.  Run w's groups are emitted into a device
     * buffer and copied into the host result columns on the copy stream
     * while run w + 1 is reduced.  The host columns were faulted in during
     * the earlier passes, sized from the distinct-key estimate (grown if the
     * count turns out larger). */
    const int W = (pg->hb && nb >= 2048) ? 8 : 1;
    uint64_t *hso = (uint64_t *)vg_xcalloc((size_t)nb + 1, 8);
    vg_d2h(hso, stage_off, (size_t)(nb + 1) * 8);
    vg_sync();
    uint64_t wmax = 1;
    for (int w = 0; w < W; w++) {
        const int b0 = (int)((int64_t)nb * w / W), b1 = (int)((int64_t)nb * (w + 1) / W);
        if (hso[b1] - hso[b0] > wmax) wmax = hso[b1] - hso[b0];
    }
    double *wbuf = (double *)vg_dmalloc((size_t)2 * n_cols * a256(wmax * 8) + 256);
    size_t hcap = 0;
    if (W > 1) {
        /* the columns are taken now and filled from the front; each run's
         * copy waits only for the pages it writes */
        for (int c = 0; c < n_cols; c++) hcol[c] = vg_host_bufs_take(pg->hb, c, 0);
        hcap = pg->hb_bytes / 8;
    }
    uint32_t *gc = (uint32_t *)vg_dmalloc((size_t)nb * 8 + 256);
    unsigned int *tickets = (unsigned int *)vg_dmalloc((size_t)W * 4 + 256);
    double t0 = now_ms();
    double t_emit = 0.0, t_copy = 0.0;
    pagg_reduce_launch(pg, L, P, &B, stage_off, gc, nb, tickets, 0, (int)((int64_t)nb / W));
    for (int w = 0; w < W; w++) {
        const int b0 = (int)((int64_t)nb * w / W), b1 = (int)((int64_t)nb * (w + 1) / W);
        const int64_t l0 = lv.n;
        pagg_reduce_collect(pg, L, P, &B, stage_off, gc, nb, b0, b1 - b0, &lv, 0);
        if (W == 1) break;
        const double te = now_ms();
        int64_t rows = 0;
        uint64_t *d_leaf = leaf_arrays(&lv, l0, lv.n, &rows);
        double *wb[VG_MAX_OUTS + 1];
        for (int c = 0; c < n_cols; c++)
            wb[c] = (double *)((char *)wbuf + (size_t)((w & 1) * n_cols + c) * a256(wmax * 8));
        vg_check_rc(vgk_pagg_emit(lv.n - l0, d_leaf, d_leaf + (lv.n - l0) + 1, rows, 0, 0, B.st_key, B.st_ok,
                                  (const double *const *)B.st_out, n_out, (uint64_t *)wb[0], vcol[0], wb + 1, vcol + 1,
                                  (uint64_t)n_groups, vg_stream()),
                    "partitioned aggregation emit");
        vg_copy_after_main();                         /* the copies below wait for this emit only */
        if (w + 1 < W) {
            const int c0 = b1, c1 = (int)((int64_t)nb * (w + 2) / W);
            pagg_reduce_launch(pg, L, P, &B, stage_off, gc, nb, tickets + w + 1, c0, c1 - c0);
        }
        t_emit += now_ms() - te;
        double tc = now_ms();
        if ((size_t)(n_groups + rows) <= hcap) {
            vg_host_bufs_wait_upto(pg->hb, (size_t)(n_groups + rows) * 8);
            g_pagg_ms[4] += now_ms() - tc;
            tc = now_ms();
        } else {                                     /* more groups than estimated: grow the host columns */
            vg_host_bufs_wait(pg->hb);
            size_t ncap = (size_t)(n_groups + rows) * 5 / 4 + 4096;
            for (int c = 0; c < n_cols; c++) {
                void *q = realloc(hcol[c], ncap * 8);
                if (!q) vg_fail("out of host memory for the result");
                hcol[c] = q;
            }
            hcap = ncap;
        }
        for (int c = 0; c < n_cols; c++)
            vg_d2h_copy((char *)hcol[c] + (size_t)n_groups * 8, wb[c], (size_t)rows * 8);
        vg_copy_sync();
        vg_dfree(d_leaf);
        t_copy += now_ms() - tc;
        n_groups += rows;
    }
    vg_host_bufs_wait(pg->hb);        /* every page touched: the threads are done with the buffers */
    g_pagg_ms[2] += now_ms() - t0 - t_emit - t_copy;
    g_pagg_ms[3] += t_emit;
    g_pagg_ms[5] += t_copy;
    t0 = now_ms();

    /* the NA-key group, last */
    uint32_t na_n = 0;
    vg_d2h(&na_n, pg->na.gt.n_used, 4);
    vg_sync();
    int has_na = 0;
    if (na_n) {
        int32_t *slots = (int32_t *)vg_dmalloc((size_t)pg->na.gt.cap * 4 + 16);
        uint32_t ns = 0;
        vg_check_rc(vgk_group_table_compact(&pg->na.gt, slots, &ns, vg_stream()), "group compact");
        int32_t slot = 0;
        vg_d2h(&slot, slots, 4);
        vg_sync();
        vg_dfree(slots);
        if (ns != 1) vg_fail("partitioned aggregation: NA group table holds %u groups", ns);
        vg_check_rc(vgk_group_stage(&pg->na.gt, P->fin, n_out, slot, B.st_key, B.st_ok, B.st_out, total, warn,
                                    vg_stream()),
                    "NA group");
        has_na = 1;
    }
    if (W == 1) {
        /* one run: every group (and the NA group) emitted at once */
        int64_t rows = 0;
        uint64_t *d_leaf = leaf_arrays(&lv, 0, lv.n, &rows);
        const int64_t ng = rows + has_na;
        size_t per = a256((size_t)ng * 8 + 8);
        char *ob = (char *)vg_dmalloc(per * (size_t)n_cols + 256);
        double *oc[VG_MAX_OUTS + 1];
        for (int c = 0; c < n_cols; c++) oc[c] = (double *)(ob + per * (size_t)c);
        vg_check_rc(vgk_pagg_emit(lv.n, d_leaf, d_leaf + lv.n + 1, ng, has_na, total, B.st_key, B.st_ok,
                                  (const double *const *)B.st_out, n_out, (uint64_t *)oc[0], vcol[0], oc + 1, vcol + 1,
                                  0, vg_stream()),
                    "partitioned aggregation emit");
        vg_sync();
        g_pagg_ms[3] += now_ms() - t0;
        t0 = now_ms();
        vg_host_bufs_wait(pg->hb);
        g_pagg_ms[4] += now_ms() - t0;
        t0 = now_ms();
        n_groups = ng;
        res = vg_batch_alloc(n_cols, n_groups);
        const size_t need = (size_t)n_groups * 8;
        for (int c = 0; c < n_cols; c++) {
            void *dst = vg_host_bufs_take(pg->hb, c, need);
            if (!dst) dst = vg_xcalloc(need ? need : 1, 1);
            vg_d2h(dst, oc[c], need);
            res->columns[c] = vg_host_column(c == 0 ? VEC_INT64 : VEC_DOUBLE, n_groups, dst, vcol[c]);
        }
        vg_sync();
        vg_dfree(d_leaf);
        vg_dfree(ob);
    } else {
        if (has_na) {
            /* one more run: the NA group alone */
            double *wb[VG_MAX_OUTS + 1];
            for (int c = 0; c < n_cols; c++) wb[c] = (double *)((char *)wbuf + (size_t)c * a256(wmax * 8));
            uint64_t *d_leaf = (uint64_t *)vg_dmalloc(256);
            vg_dmemset(d_leaf, 0, 16);
            vg_check_rc(vgk_pagg_emit(0, d_leaf, d_leaf, 1, 1, total, B.st_key, B.st_ok,
                                      (const double *const *)B.st_out, n_out, (uint64_t *)wb[0], vcol[0], wb + 1,
                                      vcol + 1, (uint64_t)n_groups, vg_stream()),
                        "partitioned aggregation emit");
            if ((size_t)(n_groups + 1) > hcap) {
                for (int c = 0; c < n_cols; c++) {
                    void *q = realloc(hcol[c], (size_t)(n_groups + 1) * 8);
                    if (!q) vg_fail("out of host memory for the result");
                    hcol[c] = q;
                }
            }
            for (int c = 0; c < n_cols; c++) vg_d2h((char *)hcol[c] + (size_t)n_groups * 8, wb[c], 8);
            vg_sync();
            vg_dfree(d_leaf);
            n_groups += 1;
        }
        res = vg_batch_alloc(n_cols, n_groups);
        for (int c = 0; c < n_cols; c++) {
            res->columns[c] = vg_host_column(c == 0 ? VEC_INT64 : VEC_DOUBLE, n_groups, hcol[c], vcol[c]);
            hcol[c] = NULL;
        }
    }
    res->col_names[0] = vg_xstrdup(ga->key_names[0]);
    for (int j = 0; j < n_out; j++) res->col_names[1 + j] = vg_xstrdup(ga->agg_specs[j].output_name);
    uint32_t w = 0;
    vg_d2h(&w, warn, 4);
    vg_sync();
    g_pagg_ms[5] += now_ms() - t0;
    vg_warn_count((long)w);
    vg_dfree(tickets);
    vg_dfree(gc);
    vg_dfree(wbuf);
    vg_dfree(dval);
    free(hso);
    vg_dfree(warn);
    vg_dfree(blk);
    vg_dfree(stage_off);
    free(lv.stage);
    free(lv.gc);
    return res;
}

static unsigned long long g_pagg_runs;
unsigned long long vgpu_pagg_runs(void) { return g_pagg_runs; }

static void pagg_free(PAgg *pg) {
    if (!pg) return;
    pt_free(pg);
    for (int r = 0; r < pg->n_regions; r++) {
        vg_dfree(pg->reg[r].rec);
        vg_dfree(pg->reg[r].off);
        vg_dfree(pg->reg[r].cursor);
    }
    vg_dfree(pg->cnt);
    vg_dfree(pg->pcur);
    vg_dfree(pg->err);
    vg_dfree(pg->counters);
    vg_dfree(pg->na.block);
    vg_host_bufs_free(pg->hb);
    free(pg);
}

static VecBatch *agg_next_body(VecNode *self) {
    VgAgg *A = (VgAgg *)self;
    if (A->ga.done) return NULL;
    A->ga.done = 1;
    const double t_start = now_ms();
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
        const double tb = now_ms();
        B = vg_join_build_payload(P.join, P.bset.idx, P.bset.n, &pay);
        g_agg_ms[1] += now_ms() - tb;
        L->jpay = pay;
        L->jpay_n = pay ? P.bset.n : 0;
        L->jpay16 = pay && B->pay_layout != -2;
        L->jpay_narrow = pay ? (B->pay_layout >= 0 ? B->pay_layout : -1) : -1;
        L->jpay_min = pay ? B->pay_min : 0;
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
    /* a general filter program: its columns come with every batch, and its
     * selection is made on the device before the batch's launches */
    if (P.prog)
        for (int j = 0; j < P.fset->n; j++) {
            P.prog_col[j] = P.fset->idx[j];
            need[P.fset->idx[j]] = 1;
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
    PAgg *pg = NULL;
    double t_loop = now_ms();
    g_agg_ms[0] += t_loop - t_start;
    if (P.n_str) str_dicts_begin(&P);
    while (vg_pull(P.src, need, 0, &db)) {
        void *fsel = P.prog ? filter_batch(&P, &db) : NULL;
        if (P.prog && db.sel_n == 0) {                /* no row passes: as if the batch were dropped */
            vg_dfree(fsel);
            vg_dbatch_release(&db);
            continue;
        }
        int64_t n_logical = db.d_sel ? db.sel_n : db.n_rows;
        void *codes = P.n_str ? str_encode_batch(&P, &db) : NULL;
        if (batch_idx == 0 && !P.n_str) {
            const double t0 = now_ms();
            pg = pagg_begin(A, &P, L, &db);
            if (pg) g_pagg_ms[0] += now_ms() - t0;
        }
        if (pg) {
            const double t0 = now_ms();
            pagg_batch(pg, &P, L, &db, stream_pos, batch_idx);
            g_pagg_ms[1] += now_ms() - t0;
            vg_dfree(fsel);
            vg_dbatch_release(&db);
            stream_pos += n_logical;
            batch_idx++;
            continue;
        }
        L->batch_idx = batch_idx;
        /* launches of at most kChunk logical rows, so that everything one
         * launch can spill fits the spill list (a batch of any size) */
        int settled = 0;
        for (int64_t off = 0, n = 0; off < n_logical; off += n) {
            n = n_logical - off;
            if (!settled && n > kChunk && !L->dense) n = kChunk;   /* dense: the table cannot grow */
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
        vg_dfree(codes);
        vg_dfree(fsel);
        vg_dbatch_release(&db);
        stream_pos += n_logical;
        batch_idx++;
    }
    const uint32_t *deferred = S.deferred ? queue_deferred_status(&T, &S) : NULL;
    const double t_emit = now_ms();
    if (!pg) g_agg_ms[2] += t_emit - t_loop;
    VecBatch *res = pg ? pagg_end(pg, A, &P, L) : emit_result(A, &P, &T, deferred);
    str_dicts_free(&P);
    if (pg) pt_finish(pg);
    if (!pg) g_agg_ms[3] += now_ms() - t_emit;
    if (pg) g_pagg_runs++;
    const int was_pagg = pg != NULL;
    pagg_free(pg);
    vg_dfree(T.block);
    vg_dfree(S.cache);
    vg_dfree(S.counters);
    free(L);
    free(need);
    if (was_pagg) g_pagg_ms[6] += now_ms() - t_start;
    else g_agg_ms[4] += now_ms() - t_start;
    return res;
}

/* one node API call: its temporary device memory is released if it fails */
static VecBatch *agg_next(VecNode *self) {
    vg_scope_enter();
    VecBatch *b = agg_next_body(self);
    vg_scope_leave();
    return b;
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
    if (n_keys > VG_MAX_KEYS) vg_fail("GPU group-agg supports at most %d key columns", VG_MAX_KEYS);
    if (n_aggs > VG_MAX_OUTS) vg_fail("GPU group-agg supports at most %d aggregates", VG_MAX_OUTS);
    const VecSchema *cs = &child->output_schema;
    for (int k = 0; k < n_keys; k++) {
        int idx = vg_schema_find(cs, key_names[k]);
        if (temp_dir && idx < 0) vg_fail("group_by: column not found: %s", key_names[k]);
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
