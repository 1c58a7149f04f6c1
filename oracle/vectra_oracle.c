/*
 * vectra_oracle.c -- CPU restatement of gcol33/vectra's columnar hot path.
 *
 * TEST INFRASTRUCTURE ONLY (the correctness oracle and the CPU baseline of
 * the benchmark).  The product library never links or calls this file.
 *
 * Each part restates the reference algorithm it cites (paths are within the
 * reference project).  It is written from the reference's behaviour, with
 * its own data structures; only the node contract (include/vectra_abi.h) and
 * the semantics are shared:
 *   expression evaluation      src/expr.c:91-281
 *   compare / arith / Kleene   src/scalar_ops.c:11-226, src/coerce.c:7-71
 *   filter + sel composition   src/filter.c:13-64
 *   project (mutate)           src/project.c:51-252
 *   hashing                    src/hash.c:9-78, src/hash.h:11-14
 *   aggregate semantics        src/agg_ops.c:10-255
 *   hash group-agg             src/group_agg.c:155-281
 *   sort group-agg             src/group_agg.c:466-585, src/sort.c:32-116
 *   hash join                  src/join.c:23-599
 */
#include "vectra_oracle.h"

#include <math.h>
#include <setjmp.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------ */
/* errors                                                              */
/* ------------------------------------------------------------------ */

static jmp_buf *g_jmp = NULL;
static char g_msg[1024];
static long g_warn = 0;
static int g_join_quirk = 1;

const char *orc_last_error(void) { return g_msg; }
long orc_warning_count(void) { return g_warn; }
void orc_reset(void) { g_msg[0] = 0; g_warn = 0; }
void orc_set_join_quirk(int on) { g_join_quirk = on; }

static void orc_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_msg, sizeof(g_msg), fmt, ap);
    va_end(ap);
    if (g_jmp) longjmp(*g_jmp, 1);
    fprintf(stderr, "oracle error outside a guard: %s\n", g_msg);
    abort();
}

static void *xmalloc(size_t n) {
    void *p = malloc(n ? n : 1);
    if (!p) orc_error("oracle: out of memory (%zu bytes)", n);
    return p;
}
static void *xcalloc(size_t n, size_t s) {
    void *p = calloc(n ? n : 1, s ? s : 1);
    if (!p) orc_error("oracle: out of memory");
    return p;
}
static char *xstrdup(const char *s) {
    size_t n = strlen(s) + 1;
    char *p = (char *)xmalloc(n);
    memcpy(p, s, n);
    return p;
}

/* ------------------------------------------------------------------ */
/* arrays, batches, schemas (the node contract's memory rules)         */
/* ------------------------------------------------------------------ */

static inline int is_valid(const VecArray *a, int64_t i) {
    return a->validity ? (a->validity[i >> 3] >> (i & 7)) & 1 : 1;
}
static inline void set_valid(VecArray *a, int64_t i) {
    a->validity[i >> 3] |= (uint8_t)(1u << (i & 7));
}
static inline void set_null(VecArray *a, int64_t i) {
    a->validity[i >> 3] &= (uint8_t)~(1u << (i & 7));
}
static inline int64_t vbytes(int64_t n) { return (n + 7) / 8; }

/* zeroed values, all-NA validity (src/array.c:6-39) */
static VecArray arr_alloc(VecType t, int64_t n) {
    VecArray a;
    memset(&a, 0, sizeof(a));
    a.type = t;
    a.length = n;
    a.owns_data = 1;
    a.validity = (uint8_t *)xcalloc((size_t)vbytes(n), 1);
    switch (t) {
    case VEC_INT64: a.buf.i64 = (int64_t *)xcalloc((size_t)n, 8); break;
    case VEC_DOUBLE: a.buf.dbl = (double *)xcalloc((size_t)n, 8); break;
    case VEC_BOOL: a.buf.bln = (uint8_t *)xcalloc((size_t)n, 1); break;
    case VEC_STRING:
        a.buf.str.offsets = (int64_t *)xcalloc((size_t)n + 1, 8);
        a.buf.str.data = NULL;
        a.buf.str.data_len = 0;
        break;
    }
    return a;
}

static void arr_free(VecArray *a) {
    free(a->validity);
    a->validity = NULL;
    switch (a->type) {
    case VEC_INT64: free(a->buf.i64); break;
    case VEC_DOUBLE: free(a->buf.dbl); break;
    case VEC_BOOL: free(a->buf.bln); break;
    case VEC_STRING:
        free(a->buf.str.offsets);
        if (a->owns_data) free(a->buf.str.data);
        break;
    }
    memset(&a->buf, 0, sizeof(a->buf));
    a->length = 0;
}

static void set_all_valid(VecArray *a) {
    memset(a->validity, 0xFF, (size_t)vbytes(a->length));
}

static VecBatch *batch_alloc(int n_cols, int64_t n_rows) {
    VecBatch *b = (VecBatch *)xcalloc(1, sizeof(VecBatch));
    b->n_cols = n_cols;
    b->n_rows = n_rows;
    b->columns = (VecArray *)xcalloc((size_t)n_cols, sizeof(VecArray));
    b->col_names = (char **)xcalloc((size_t)n_cols, sizeof(char *));
    return b;
}

void orc_batch_free(VecBatch *b) {
    if (!b) return;
    for (int i = 0; i < b->n_cols; i++) {
        arr_free(&b->columns[i]);
        free(b->col_names[i]);
    }
    free(b->columns);
    free(b->col_names);
    free(b->sel);
    free(b);
}

static inline int64_t logical_rows(const VecBatch *b) {
    return b->sel ? (int64_t)b->sel_n : b->n_rows;
}
static inline int64_t phys_row(const VecBatch *b, int64_t li) {
    return b->sel ? (int64_t)b->sel[li] : li;
}

static VecSchema schema_make(int n, char *const *names, const VecType *types) {
    VecSchema s;
    s.n_cols = n;
    s.col_names = (char **)xcalloc((size_t)n, sizeof(char *));
    s.col_types = (VecType *)xcalloc((size_t)n, sizeof(VecType));
    s.col_annotations = (char **)xcalloc((size_t)n, sizeof(char *));
    for (int i = 0; i < n; i++) {
        s.col_names[i] = xstrdup(names[i]);
        s.col_types[i] = types[i];
    }
    return s;
}
static void schema_free(VecSchema *s) {
    for (int i = 0; i < s->n_cols; i++) {
        free(s->col_names[i]);
        if (s->col_annotations) free(s->col_annotations[i]);
    }
    free(s->col_names);
    free(s->col_types);
    free(s->col_annotations);
    memset(s, 0, sizeof(*s));
}
static int schema_find(const VecSchema *s, const char *name) {
    for (int i = 0; i < s->n_cols; i++)
        if (strcmp(s->col_names[i], name) == 0) return i;
    return -1;
}

/* deep copy (same type) or numeric widening (src/coerce.c:18-71) */
static VecArray arr_coerce(const VecArray *a, VecType t) {
    VecArray o = arr_alloc(t, a->length);
    if (a->validity) memcpy(o.validity, a->validity, (size_t)vbytes(a->length));
    else set_all_valid(&o);
    int64_t n = a->length;
    if (a->type == t) {
        switch (t) {
        case VEC_INT64: memcpy(o.buf.i64, a->buf.i64, (size_t)n * 8); break;
        case VEC_DOUBLE: memcpy(o.buf.dbl, a->buf.dbl, (size_t)n * 8); break;
        case VEC_BOOL: memcpy(o.buf.bln, a->buf.bln, (size_t)n); break;
        case VEC_STRING: {
            memcpy(o.buf.str.offsets, a->buf.str.offsets, (size_t)(n + 1) * 8);
            o.buf.str.data_len = a->buf.str.data_len;
            o.buf.str.data = (char *)xmalloc((size_t)a->buf.str.data_len);
            if (a->buf.str.data_len)
                memcpy(o.buf.str.data, a->buf.str.data, (size_t)a->buf.str.data_len);
            break;
        }
        }
        return o;
    }
    if (a->type == VEC_BOOL && t == VEC_INT64) {
        for (int64_t i = 0; i < n; i++) o.buf.i64[i] = (int64_t)a->buf.bln[i];
    } else if (a->type == VEC_BOOL && t == VEC_DOUBLE) {
        for (int64_t i = 0; i < n; i++) o.buf.dbl[i] = (double)a->buf.bln[i];
    } else if (a->type == VEC_INT64 && t == VEC_DOUBLE) {
        for (int64_t i = 0; i < n; i++) o.buf.dbl[i] = (double)a->buf.i64[i];
    } else {
        arr_free(&o);
        orc_error("unsupported coercion: %d -> %d", a->type, t);
    }
    return o;
}

/* bool < int64 < double; strings do not mix (src/coerce.c:7-16) */
static VecType common_type(VecType a, VecType b) {
    if (a == b) return a;
    if (a == VEC_STRING || b == VEC_STRING)
        orc_error("cannot coerce string in arithmetic/comparison");
    if (a == VEC_DOUBLE || b == VEC_DOUBLE) return VEC_DOUBLE;
    if (a == VEC_INT64 || b == VEC_INT64) return VEC_INT64;
    return VEC_BOOL;
}

/* gather logical rows into a dense array (src/array.c:66-135) */
static VecArray arr_gather(const VecArray *src, const int32_t *sel, int32_t n) {
    VecArray d = arr_alloc(src->type, n);
    if (src->type == VEC_STRING) {
        int64_t total = 0;
        for (int32_t j = 0; j < n; j++)
            if (is_valid(src, sel[j]))
                total += src->buf.str.offsets[sel[j] + 1] - src->buf.str.offsets[sel[j]];
        d.buf.str.data = (char *)xmalloc((size_t)total);
        d.buf.str.data_len = total;
        int64_t off = 0;
        for (int32_t j = 0; j < n; j++) {
            int64_t p = sel[j];
            d.buf.str.offsets[j] = off;
            if (is_valid(src, p)) {
                set_valid(&d, j);
                int64_t s = src->buf.str.offsets[p], l = src->buf.str.offsets[p + 1] - s;
                if (l) memcpy(d.buf.str.data + off, src->buf.str.data + s, (size_t)l);
                off += l;
            }
        }
        d.buf.str.offsets[n] = off;
        return d;
    }
    for (int32_t j = 0; j < n; j++) {
        int64_t p = sel[j];
        if (!is_valid(src, p)) continue;
        set_valid(&d, j);
        switch (src->type) {
        case VEC_INT64: d.buf.i64[j] = src->buf.i64[p]; break;
        case VEC_DOUBLE: d.buf.dbl[j] = src->buf.dbl[p]; break;
        case VEC_BOOL: d.buf.bln[j] = src->buf.bln[p]; break;
        default: break;
        }
    }
    return d;
}

/* ------------------------------------------------------------------ */
/* growable column builder (what src/builder.c provides)               */
/* ------------------------------------------------------------------ */

typedef struct {
    VecType type;
    int64_t len, cap;
    uint8_t *valid;
    union { int64_t *i64; double *dbl; uint8_t *bln; } v;
    int64_t *offs;
    char *sdata;
    int64_t slen, scap;
} Bld;

static Bld bld_init(VecType t) {
    Bld b;
    memset(&b, 0, sizeof(b));
    b.type = t;
    return b;
}
static void bld_reserve(Bld *b, int64_t extra) {
    int64_t need = b->len + extra;
    if (need <= b->cap) return;
    int64_t nc = b->cap ? b->cap : 1024;
    while (nc < need) nc *= 2;
    int64_t ovb = vbytes(b->cap), nvb = vbytes(nc);
    b->valid = (uint8_t *)realloc(b->valid, (size_t)nvb);
    memset(b->valid + ovb, 0, (size_t)(nvb - ovb));
    switch (b->type) {
    case VEC_INT64: b->v.i64 = (int64_t *)realloc(b->v.i64, (size_t)nc * 8);
        memset(b->v.i64 + b->cap, 0, (size_t)(nc - b->cap) * 8); break;
    case VEC_DOUBLE: b->v.dbl = (double *)realloc(b->v.dbl, (size_t)nc * 8);
        memset(b->v.dbl + b->cap, 0, (size_t)(nc - b->cap) * 8); break;
    case VEC_BOOL: b->v.bln = (uint8_t *)realloc(b->v.bln, (size_t)nc);
        memset(b->v.bln + b->cap, 0, (size_t)(nc - b->cap)); break;
    case VEC_STRING: b->offs = (int64_t *)realloc(b->offs, (size_t)(nc + 1) * 8);
        if (b->cap == 0) b->offs[0] = 0;
        break;
    }
    b->cap = nc;
}
static void bld_put_str(Bld *b, const char *p, int64_t l) {
    if (b->slen + l > b->scap) {
        int64_t nc = b->scap ? b->scap : 256;
        while (nc < b->slen + l) nc *= 2;
        b->sdata = (char *)realloc(b->sdata, (size_t)nc);
        b->scap = nc;
    }
    if (l) memcpy(b->sdata + b->slen, p, (size_t)l);
    b->slen += l;
}
static void bld_append_one(Bld *b, const VecArray *a, int64_t row) {
    bld_reserve(b, 1);
    int64_t j = b->len;
    if (is_valid(a, row)) {
        b->valid[j >> 3] |= (uint8_t)(1u << (j & 7));
        switch (b->type) {
        case VEC_INT64: b->v.i64[j] = a->buf.i64[row]; break;
        case VEC_DOUBLE: b->v.dbl[j] = a->buf.dbl[row]; break;
        case VEC_BOOL: b->v.bln[j] = a->buf.bln[row]; break;
        case VEC_STRING: {
            int64_t s = a->buf.str.offsets[row], e = a->buf.str.offsets[row + 1];
            bld_put_str(b, a->buf.str.data + s, e - s);
            break;
        }
        }
    }
    if (b->type == VEC_STRING) b->offs[j + 1] = b->slen;
    b->len++;
}
static void bld_append_na(Bld *b) {
    bld_reserve(b, 1);
    if (b->type == VEC_STRING) b->offs[b->len + 1] = b->slen;
    b->len++;
}
static void bld_append_i64(Bld *b, int64_t v) {
    bld_reserve(b, 1);
    b->valid[b->len >> 3] |= (uint8_t)(1u << (b->len & 7));
    b->v.i64[b->len++] = v;
}
static void bld_append_dbl(Bld *b, double v, int valid) {
    bld_reserve(b, 1);
    if (valid) b->valid[b->len >> 3] |= (uint8_t)(1u << (b->len & 7));
    b->v.dbl[b->len++] = valid ? v : 0.0;
}
static VecArray bld_finish(Bld *b) {
    VecArray a;
    memset(&a, 0, sizeof(a));
    a.type = b->type;
    a.length = b->len;
    a.owns_data = 1;
    a.validity = b->valid ? b->valid : (uint8_t *)xcalloc(1, 1);
    switch (b->type) {
    case VEC_INT64: a.buf.i64 = b->v.i64 ? b->v.i64 : (int64_t *)xcalloc(1, 8); break;
    case VEC_DOUBLE: a.buf.dbl = b->v.dbl ? b->v.dbl : (double *)xcalloc(1, 8); break;
    case VEC_BOOL: a.buf.bln = b->v.bln ? b->v.bln : (uint8_t *)xcalloc(1, 1); break;
    case VEC_STRING:
        if (!b->offs) { b->offs = (int64_t *)xcalloc(1, 8); }
        a.buf.str.offsets = b->offs;
        a.buf.str.data = b->sdata ? b->sdata : (char *)xmalloc(1);
        a.buf.str.data_len = b->slen;
        break;
    }
    memset(b, 0, sizeof(*b));
    return a;
}
static void bld_free(Bld *b) {
    free(b->valid); free(b->v.i64); free(b->offs); free(b->sdata);
    memset(b, 0, sizeof(*b));
}

/* ------------------------------------------------------------------ */
/* source node                                                         */
/* ------------------------------------------------------------------ */

typedef struct {
    VecNode base;
    int n_cols;
    VecArray *cols;    /* owned full-length copies */
    int64_t n_rows, batch_rows, cursor;
    int sel_mode;
} SrcNode;

static VecBatch *src_next(VecNode *self) {
    SrcNode *s = (SrcNode *)self;
    if (s->cursor >= s->n_rows) return NULL;
    int64_t lo = s->cursor, n = s->n_rows - lo;
    if (n > s->batch_rows) n = s->batch_rows;
    s->cursor += n;
    VecBatch *b = batch_alloc(s->n_cols, n);
    for (int c = 0; c < s->n_cols; c++) {
        const VecArray *src = &s->cols[c];
        VecArray d = arr_alloc(src->type, n);
        for (int64_t i = 0; i < n; i++)
            if (is_valid(src, lo + i)) set_valid(&d, i);
        switch (src->type) {
        case VEC_INT64: memcpy(d.buf.i64, src->buf.i64 + lo, (size_t)n * 8); break;
        case VEC_DOUBLE: memcpy(d.buf.dbl, src->buf.dbl + lo, (size_t)n * 8); break;
        case VEC_BOOL: memcpy(d.buf.bln, src->buf.bln + lo, (size_t)n); break;
        case VEC_STRING: {
            int64_t base = src->buf.str.offsets[lo];
            int64_t len = src->buf.str.offsets[lo + n] - base;
            for (int64_t i = 0; i <= n; i++)
                d.buf.str.offsets[i] = src->buf.str.offsets[lo + i] - base;
            d.buf.str.data = (char *)xmalloc((size_t)len);
            if (len) memcpy(d.buf.str.data, src->buf.str.data + base, (size_t)len);
            d.buf.str.data_len = len;
            break;
        }
        }
        b->columns[c] = d;
        b->col_names[c] = xstrdup(self->output_schema.col_names[c]);
    }
    if (s->sel_mode == 1) {
        int32_t k = (int32_t)((n + 1) / 2);
        b->sel = (int32_t *)xmalloc((size_t)k * 4);
        for (int32_t j = 0; j < k; j++) b->sel[j] = 2 * j;
        b->sel_n = k;
    }
    return b;
}

static void src_free(VecNode *self) {
    SrcNode *s = (SrcNode *)self;
    for (int c = 0; c < s->n_cols; c++) arr_free(&s->cols[c]);
    free(s->cols);
    schema_free(&self->output_schema);
    free(s);
}

VecNode *orc_table_source_create(int n_cols, const char *const *names,
                                 const int *types, const void *const *data,
                                 const char *const *str_data,
                                 const uint8_t *const *validity,
                                 int64_t n_rows, int64_t batch_rows,
                                 int sel_mode) {
    SrcNode *s = (SrcNode *)xcalloc(1, sizeof(SrcNode));
    s->n_cols = n_cols;
    s->n_rows = n_rows;
    s->batch_rows = batch_rows > 0 ? batch_rows : (n_rows > 0 ? n_rows : 1);
    s->sel_mode = sel_mode;
    s->cols = (VecArray *)xcalloc((size_t)n_cols, sizeof(VecArray));
    VecType *ts = (VecType *)xcalloc((size_t)n_cols, sizeof(VecType));
    for (int c = 0; c < n_cols; c++) {
        VecType t = (VecType)types[c];
        ts[c] = t;
        VecArray a = arr_alloc(t, n_rows);
        if (validity && validity[c]) memcpy(a.validity, validity[c], (size_t)vbytes(n_rows));
        else set_all_valid(&a);
        switch (t) {
        case VEC_INT64: memcpy(a.buf.i64, data[c], (size_t)n_rows * 8); break;
        case VEC_DOUBLE: memcpy(a.buf.dbl, data[c], (size_t)n_rows * 8); break;
        case VEC_BOOL: memcpy(a.buf.bln, data[c], (size_t)n_rows); break;
        case VEC_STRING: {
            const int64_t *offs = (const int64_t *)data[c];
            memcpy(a.buf.str.offsets, offs, (size_t)(n_rows + 1) * 8);
            int64_t len = offs[n_rows];
            a.buf.str.data = (char *)xmalloc((size_t)len);
            if (len) memcpy(a.buf.str.data, str_data[c], (size_t)len);
            a.buf.str.data_len = len;
            break;
        }
        }
        s->cols[c] = a;
    }
    s->base.output_schema = schema_make(n_cols, (char *const *)names, ts);
    free(ts);
    s->base.next_batch = src_next;
    s->base.free_node = src_free;
    s->base.kind = "ScanNode";
    return &s->base;
}

/* ------------------------------------------------------------------ */
/* expression evaluation (src/expr.c:91-281, src/scalar_ops.c)         */
/* ------------------------------------------------------------------ */

static const VecArray *find_col(const VecBatch *b, const char *name) {
    for (int i = 0; i < b->n_cols; i++)
        if (strcmp(b->col_names[i], name) == 0) return &b->columns[i];
    orc_error("column not found: %s", name);
    return NULL;
}

static int cmp_result(int cmp, char op, char op2) {
    if (op == '=' && op2 == '=') return cmp == 0;
    if (op == '!' && op2 == '=') return cmp != 0;
    if (op == '<' && op2 == ' ') return cmp < 0;
    if (op == '<' && op2 == '=') return cmp <= 0;
    if (op == '>' && op2 == ' ') return cmp > 0;
    if (op == '>' && op2 == '=') return cmp >= 0;
    return 0;
}

static VecArray eval(const VecExpr *e, const VecBatch *b);

/* src/scalar_ops.c:11-66 */
static VecArray eval_arith(const VecArray *l, const VecArray *r, char op) {
    if (l->length != r->length) orc_error("arith: mismatched lengths");
    VecType t = common_type(l->type, r->type);
    if (t == VEC_BOOL) t = VEC_INT64;
    VecArray cl = arr_coerce(l, t), cr = arr_coerce(r, t);
    int64_t n = l->length;
    VecArray o = arr_alloc(t, n);
    for (int64_t i = 0; i < n; i++) {
        if (!is_valid(&cl, i) || !is_valid(&cr, i)) continue;
        set_valid(&o, i);
        if (t == VEC_INT64) {
            /* wrap-around as two's complement, like the reference on every
             * target it builds for */
            uint64_t a = (uint64_t)cl.buf.i64[i], bb = (uint64_t)cr.buf.i64[i];
            int64_t sa = cl.buf.i64[i], sb = cr.buf.i64[i];
            switch (op) {
            case '+': o.buf.i64[i] = (int64_t)(a + bb); break;
            case '-': o.buf.i64[i] = (int64_t)(a - bb); break;
            case '*': o.buf.i64[i] = (int64_t)(a * bb); break;
            case '/':
                if (sb == 0) set_null(&o, i);
                else if (sb == -1) o.buf.i64[i] = (int64_t)(0 - a);
                else o.buf.i64[i] = sa / sb;
                break;
            case '%':
                if (sb == 0) set_null(&o, i);
                else if (sb == -1) o.buf.i64[i] = 0;
                else o.buf.i64[i] = sa % sb;
                break;
            default: orc_error("unknown arith op: %c", op);
            }
        } else {
            double a = cl.buf.dbl[i], bb = cr.buf.dbl[i];
            switch (op) {
            case '+': o.buf.dbl[i] = a + bb; break;
            case '-': o.buf.dbl[i] = a - bb; break;
            case '*': o.buf.dbl[i] = a * bb; break;
            case '/': o.buf.dbl[i] = a / bb; break;
            case '%': o.buf.dbl[i] = fmod(a, bb); break;
            default: orc_error("unknown arith op: %c", op);
            }
        }
    }
    arr_free(&cl);
    arr_free(&cr);
    return o;
}

/* src/scalar_ops.c:70-147 */
static VecArray eval_cmp(const VecArray *l, const VecArray *r, char op, char op2) {
    if (l->length != r->length) orc_error("cmp: mismatched lengths");
    int64_t n = l->length;
    VecArray o = arr_alloc(VEC_BOOL, n);
    if (l->type == VEC_STRING && r->type == VEC_STRING) {
        for (int64_t i = 0; i < n; i++) {
            if (!is_valid(l, i) || !is_valid(r, i)) continue;
            set_valid(&o, i);
            int64_t ls = l->buf.str.offsets[i], ll = l->buf.str.offsets[i + 1] - ls;
            int64_t rs = r->buf.str.offsets[i], rl = r->buf.str.offsets[i + 1] - rs;
            int64_t m = ll < rl ? ll : rl;
            int c = memcmp(l->buf.str.data + ls, r->buf.str.data + rs, (size_t)m);
            if (c == 0) c = (ll > rl) - (ll < rl);
            o.buf.bln[i] = (uint8_t)cmp_result(c, op, op2);
        }
        return o;
    }
    VecType t = common_type(l->type, r->type);
    if (t == VEC_BOOL) t = VEC_INT64;
    VecArray cl = arr_coerce(l, t), cr = arr_coerce(r, t);
    for (int64_t i = 0; i < n; i++) {
        if (!is_valid(&cl, i) || !is_valid(&cr, i)) continue;
        set_valid(&o, i);
        int c;
        if (t == VEC_INT64) {
            int64_t a = cl.buf.i64[i], bb = cr.buf.i64[i];
            c = (a > bb) - (a < bb);
        } else {
            double a = cl.buf.dbl[i], bb = cr.buf.dbl[i];
            c = (a > bb) - (a < bb);   /* NaN compares as equal */
        }
        o.buf.bln[i] = (uint8_t)cmp_result(c, op, op2);
    }
    arr_free(&cl);
    arr_free(&cr);
    return o;
}

/* R's three-valued logic (src/scalar_ops.c:151-185) */
static VecArray eval_bool2(const VecArray *l, const VecArray *r, char op) {
    if (l->length != r->length) orc_error("bool: mismatched lengths");
    if (l->type != VEC_BOOL || r->type != VEC_BOOL)
        orc_error("bool: operands must be boolean");
    int64_t n = l->length;
    VecArray o = arr_alloc(VEC_BOOL, n);
    for (int64_t i = 0; i < n; i++) {
        int lv = is_valid(l, i), rv = is_valid(r, i);
        int lb = lv ? l->buf.bln[i] : -1, rb = rv ? r->buf.bln[i] : -1;
        if (op == '&') {
            if ((lv && !lb) || (rv && !rb)) { set_valid(&o, i); o.buf.bln[i] = 0; }
            else if (lv && rv) { set_valid(&o, i); o.buf.bln[i] = (uint8_t)(lb && rb); }
        } else {
            if ((lv && lb) || (rv && rb)) { set_valid(&o, i); o.buf.bln[i] = 1; }
            else if (lv && rv) { set_valid(&o, i); o.buf.bln[i] = (uint8_t)(lb || rb); }
        }
    }
    return o;
}

static VecArray eval(const VecExpr *e, const VecBatch *b) {
    int64_t n = b->n_rows;
    switch (e->kind) {
    case EXPR_COL_REF: {
        const VecArray *c = find_col(b, e->col_name);
        return arr_coerce(c, c->type);
    }
    case EXPR_LIT_INT64: {
        VecArray o = arr_alloc(VEC_INT64, n);
        set_all_valid(&o);
        for (int64_t i = 0; i < n; i++) o.buf.i64[i] = e->lit_i64;
        return o;
    }
    case EXPR_LIT_DOUBLE: {
        VecArray o = arr_alloc(VEC_DOUBLE, n);
        set_all_valid(&o);
        for (int64_t i = 0; i < n; i++) o.buf.dbl[i] = e->lit_dbl;
        return o;
    }
    case EXPR_LIT_BOOL: {
        VecArray o = arr_alloc(VEC_BOOL, n);
        set_all_valid(&o);
        memset(o.buf.bln, e->lit_bln, (size_t)n);
        return o;
    }
    case EXPR_LIT_NA:
        return arr_alloc(e->result_type, n);
    case EXPR_ARITH: {
        VecArray l = eval(e->left, b), r = eval(e->right, b);
        VecArray o = eval_arith(&l, &r, e->op);
        arr_free(&l); arr_free(&r);
        return o;
    }
    case EXPR_CMP: {
        VecArray l = eval(e->left, b), r = eval(e->right, b);
        VecArray o = eval_cmp(&l, &r, e->op, e->op2);
        arr_free(&l); arr_free(&r);
        return o;
    }
    case EXPR_BOOL: {
        if (e->op == '!') {
            VecArray x = eval(e->operand, b);
            if (x.type != VEC_BOOL) { arr_free(&x); orc_error("bool not: operand must be boolean"); }
            VecArray o = arr_alloc(VEC_BOOL, x.length);
            memcpy(o.validity, x.validity, (size_t)vbytes(x.length));
            for (int64_t i = 0; i < x.length; i++)
                if (is_valid(&x, i)) o.buf.bln[i] = (uint8_t)!x.buf.bln[i];
            arr_free(&x);
            return o;
        }
        VecArray l = eval(e->left, b), r = eval(e->right, b);
        VecArray o = eval_bool2(&l, &r, e->op);
        arr_free(&l); arr_free(&r);
        return o;
    }
    case EXPR_IS_NA: {
        VecArray x = eval(e->operand, b);
        VecArray o = arr_alloc(VEC_BOOL, x.length);
        set_all_valid(&o);
        for (int64_t i = 0; i < x.length; i++) o.buf.bln[i] = (uint8_t)!is_valid(&x, i);
        arr_free(&x);
        return o;
    }
    case EXPR_NEGATE: {
        VecArray x = eval(e->operand, b);
        VecArray o = arr_alloc(x.type, x.length);
        memcpy(o.validity, x.validity, (size_t)vbytes(x.length));
        if (x.type == VEC_INT64) {
            for (int64_t i = 0; i < x.length; i++)
                o.buf.i64[i] = (int64_t)(0 - (uint64_t)x.buf.i64[i]);
        } else if (x.type == VEC_DOUBLE) {
            for (int64_t i = 0; i < x.length; i++) o.buf.dbl[i] = -x.buf.dbl[i];
        } else {
            arr_free(&x); arr_free(&o);
            orc_error("negate: unsupported type %d", (int)e->operand->result_type);
        }
        arr_free(&x);
        return o;
    }
    case EXPR_LIT_STRING: {   /* the literal repeated per row (src/expr.c:64-77) */
        const char *lit = e->lit_str ? e->lit_str : "";
        const int64_t l = (int64_t)strlen(lit);
        VecArray o = arr_alloc(VEC_STRING, n);
        set_all_valid(&o);
        o.buf.str.data = (char *)xmalloc((size_t)(l * n > 0 ? l * n : 1));
        o.buf.str.data_len = l * n;
        for (int64_t i = 0; i < n; i++) {
            o.buf.str.offsets[i] = i * l;
            memcpy(o.buf.str.data + i * l, lit, (size_t)l);
        }
        o.buf.str.offsets[n] = l * n;
        return o;
    }
    case EXPR_NCHAR: {        /* byte length (src/expr.c:153-170) */
        VecArray x = eval(e->operand, b);
        if (x.type != VEC_STRING) { arr_free(&x); orc_error("nchar: argument must be string"); }
        VecArray o = arr_alloc(VEC_INT64, x.length);
        for (int64_t i = 0; i < x.length; i++) {
            if (!is_valid(&x, i)) continue;
            set_valid(&o, i);
            o.buf.i64[i] = x.buf.str.offsets[i + 1] - x.buf.str.offsets[i];
        }
        arr_free(&x);
        return o;
    }
    case EXPR_SUBSTR: {       /* 1-based, inclusive stop (src/expr.c:172-235) */
        VecArray x = eval(e->operand, b);
        VecArray a0 = eval(e->left, b), a1 = eval(e->right, b);
        if (x.type != VEC_STRING) {
            arr_free(&x); arr_free(&a0); arr_free(&a1);
            orc_error("substr: first argument must be string");
        }
        /* start and stop as int64: doubles truncated toward zero */
        VecArray st = arr_coerce(&a0, a0.type == VEC_DOUBLE ? VEC_DOUBLE : VEC_INT64);
        VecArray sp = arr_coerce(&a1, a1.type == VEC_DOUBLE ? VEC_DOUBLE : VEC_INT64);
        const int64_t m = x.length;
        VecArray o = arr_alloc(VEC_STRING, m);
        int64_t cap = x.buf.str.data_len > 0 ? x.buf.str.data_len : 1, at = 0;
        o.buf.str.data = (char *)xmalloc((size_t)cap);
        for (int64_t i = 0; i < m; i++) {
            o.buf.str.offsets[i] = at;
            if (!is_valid(&x, i) || !is_valid(&st, i) || !is_valid(&sp, i)) continue;
            set_valid(&o, i);
            const int64_t so = x.buf.str.offsets[i], sl = x.buf.str.offsets[i + 1] - so;
            int64_t from = (st.type == VEC_DOUBLE ? (int64_t)st.buf.dbl[i] : st.buf.i64[i]) - 1;
            int64_t to = sp.type == VEC_DOUBLE ? (int64_t)sp.buf.dbl[i] : sp.buf.i64[i];
            if (from < 0) from = 0;
            if (to > sl) to = sl;
            if (to > from) {
                memcpy(o.buf.str.data + at, x.buf.str.data + so + from, (size_t)(to - from));
                at += to - from;
            }
        }
        o.buf.str.offsets[m] = at;
        o.buf.str.data_len = at;
        arr_free(&x); arr_free(&a0); arr_free(&a1); arr_free(&st); arr_free(&sp);
        return o;
    }
    case EXPR_GREPL: {        /* fixed substring search (src/expr.c:237-268) */
        VecArray x = eval(e->operand, b);
        if (x.type != VEC_STRING) { arr_free(&x); orc_error("grepl: argument must be string"); }
        const char *pat = e->lit_str ? e->lit_str : "";
        const int64_t pl = (int64_t)strlen(pat);
        VecArray o = arr_alloc(VEC_BOOL, x.length);
        for (int64_t i = 0; i < x.length; i++) {
            if (!is_valid(&x, i)) continue;
            set_valid(&o, i);
            const char *sv = x.buf.str.data + x.buf.str.offsets[i];
            const int64_t sl = x.buf.str.offsets[i + 1] - x.buf.str.offsets[i];
            int hit = 0;
            for (int64_t j = 0; !hit && j + pl <= sl; j++) hit = memcmp(sv + j, pat, (size_t)pl) == 0;
            o.buf.bln[i] = (uint8_t)hit;
        }
        arr_free(&x);
        return o;
    }
    case EXPR_IF_ELSE:
    case EXPR_CAST:
        orc_error("if_else/cast not yet implemented");
        break;
    }
    orc_error("unknown expr kind: %d", (int)e->kind);
    VecArray dummy;
    memset(&dummy, 0, sizeof(dummy));
    return dummy;
}

static void expr_free(VecExpr *e) {
    if (!e) return;
    free(e->col_name);
    free(e->lit_str);
    expr_free(e->left);
    expr_free(e->right);
    expr_free(e->operand);
    expr_free(e->cond);
    expr_free(e->then_expr);
    expr_free(e->else_expr);
    free(e);
}

static int expr_refs(const VecExpr *e, const char *name) {
    if (!e) return 0;
    if (e->kind == EXPR_COL_REF) return strcmp(e->col_name, name) == 0;
    return expr_refs(e->left, name) || expr_refs(e->right, name) ||
           expr_refs(e->operand, name) || expr_refs(e->cond, name) ||
           expr_refs(e->then_expr, name) || expr_refs(e->else_expr, name);
}

/* ------------------------------------------------------------------ */
/* filter (src/filter.c)                                               */
/* ------------------------------------------------------------------ */

typedef struct {
    VecNode base;
    VecNode *child;
    VecExpr *predicate;
} OFilter;

static VecBatch *filter_next(VecNode *self) {
    OFilter *f = (OFilter *)self;
    VecBatch *b;
    while ((b = f->child->next_batch(f->child)) != NULL) {
        VecArray m = eval(f->predicate, b);
        if (m.type != VEC_BOOL) {
            arr_free(&m);
            orc_batch_free(b);
            orc_error("filter predicate must evaluate to boolean");
        }
        /* count then fill, over logical rows (src/filter.c:13-39) */
        int64_t nl = logical_rows(b);
        int32_t k = 0;
        for (int64_t li = 0; li < nl; li++) {
            int64_t p = phys_row(b, li);
            if (is_valid(&m, p) && m.buf.bln[p]) k++;
        }
        int32_t *sel = (int32_t *)xmalloc((size_t)(k > 0 ? k : 1) * 4);
        int32_t j = 0;
        for (int64_t li = 0; li < nl; li++) {
            int64_t p = phys_row(b, li);
            if (is_valid(&m, p) && m.buf.bln[p]) sel[j++] = (int32_t)p;
        }
        arr_free(&m);
        free(b->sel);
        b->sel = sel;
        b->sel_n = k;
        if (k > 0) return b;
        orc_batch_free(b);   /* empty batches are dropped */
    }
    return NULL;
}

static void filter_free(VecNode *self) {
    OFilter *f = (OFilter *)self;
    f->child->free_node(f->child);
    expr_free(f->predicate);
    schema_free(&self->output_schema);
    free(f);
}

VecNode *orc_filter_node_create(VecNode *child, VecExpr *predicate) {
    OFilter *f = (OFilter *)xcalloc(1, sizeof(OFilter));
    f->child = child;
    f->predicate = predicate;
    f->base.output_schema = schema_make(child->output_schema.n_cols,
                                        child->output_schema.col_names,
                                        child->output_schema.col_types);
    f->base.next_batch = filter_next;
    f->base.free_node = filter_free;
    f->base.kind = "FilterNode";
    return &f->base;
}

/* ------------------------------------------------------------------ */
/* project (src/project.c:19-252)                                      */
/* ------------------------------------------------------------------ */

typedef struct {
    VecNode base;
    VecNode *child;
    int n;
    ProjEntry *entries;
} OProject;

static VecBatch *project_next(VecNode *self) {
    OProject *p = (OProject *)self;
    VecBatch *in = p->child->next_batch(p->child);
    if (!in) return NULL;
    int64_t nl = logical_rows(in);
    /* dense working copy of the logical rows of every input column */
    int wcap = in->n_cols + p->n;
    VecBatch work;
    memset(&work, 0, sizeof(work));
    work.n_rows = nl;
    work.columns = (VecArray *)xcalloc((size_t)wcap, sizeof(VecArray));
    work.col_names = (char **)xcalloc((size_t)wcap, sizeof(char *));
    for (int c = 0; c < in->n_cols; c++) {
        work.columns[c] = in->sel ? arr_gather(&in->columns[c], in->sel, in->sel_n)
                                  : arr_coerce(&in->columns[c], in->columns[c].type);
        work.col_names[c] = xstrdup(in->col_names[c]);
    }
    work.n_cols = in->n_cols;
    orc_batch_free(in);

    VecBatch *out = batch_alloc(p->n, nl);
    for (int i = 0; i < p->n; i++) {
        ProjEntry *pe = &p->entries[i];
        out->col_names[i] = xstrdup(pe->output_name);
        if (!pe->expr) {
            const VecArray *src = NULL;
            for (int c = 0; c < work.n_cols; c++)
                if (strcmp(work.col_names[c], pe->output_name) == 0) { src = &work.columns[c]; break; }
            if (!src) orc_error("select: column not found: %s", pe->output_name);
            out->columns[i] = arr_coerce(src, src->type);
        } else {
            out->columns[i] = eval(pe->expr, &work);
            /* later entries see the new column (appended; lookups take the
             * first match, as src/project.c:180-227 does) */
            work.columns[work.n_cols] = arr_coerce(&out->columns[i], out->columns[i].type);
            work.col_names[work.n_cols] = xstrdup(pe->output_name);
            work.n_cols++;
        }
    }
    for (int c = 0; c < work.n_cols; c++) {
        arr_free(&work.columns[c]);
        free(work.col_names[c]);
    }
    free(work.columns);
    free(work.col_names);
    return out;
}

static void project_free(VecNode *self) {
    OProject *p = (OProject *)self;
    p->child->free_node(p->child);
    for (int i = 0; i < p->n; i++) {
        free(p->entries[i].output_name);
        expr_free(p->entries[i].expr);
    }
    free(p->entries);
    schema_free(&self->output_schema);
    free(p);
}

VecNode *orc_project_node_create(VecNode *child, int n, ProjEntry *entries) {
    OProject *p = (OProject *)xcalloc(1, sizeof(OProject));
    p->child = child;
    p->n = n;
    p->entries = entries;
    char **names = (char **)xcalloc((size_t)n, sizeof(char *));
    VecType *types = (VecType *)xcalloc((size_t)n, sizeof(VecType));
    for (int i = 0; i < n; i++) {
        names[i] = entries[i].output_name;
        if (entries[i].expr) {
            types[i] = entries[i].expr->result_type;
        } else {
            int idx = schema_find(&child->output_schema, entries[i].output_name);
            if (idx < 0) orc_error("project: column not found in child: %s", entries[i].output_name);
            types[i] = child->output_schema.col_types[idx];
        }
    }
    p->base.output_schema = schema_make(n, names, types);
    free(names);
    free(types);
    p->base.next_batch = project_next;
    p->base.free_node = project_free;
    p->base.kind = "ProjectNode";
    return &p->base;
}

/* ------------------------------------------------------------------ */
/* hashing (src/hash.c:9-78)                                           */
/* ------------------------------------------------------------------ */

#define FNV_OFF 14695981039346656037ULL
#define FNV_PRM 1099511628211ULL
#define NA_HASH (FNV_OFF ^ 0xFFULL)

static inline uint64_t fnv_bytes(const uint8_t *p, int64_t n) {
    uint64_t h = FNV_OFF;
    for (int64_t k = 0; k < n; k++) { h ^= p[k]; h *= FNV_PRM; }
    return h;
}
static uint64_t hash_value(const VecArray *a, int64_t r) {
    if (!is_valid(a, r)) return NA_HASH;
    switch (a->type) {
    case VEC_INT64: {
        int64_t v = a->buf.i64[r];
        uint8_t bytes[8];
        memcpy(bytes, &v, 8);   /* little-endian byte order on every target */
        return fnv_bytes(bytes, 8);
    }
    case VEC_DOUBLE: {
        double v = a->buf.dbl[r];
        if (v == 0.0) v = 0.0;  /* -0 hashes as +0 */
        uint8_t bytes[8];
        memcpy(bytes, &v, 8);
        return fnv_bytes(bytes, 8);
    }
    case VEC_BOOL: {
        uint64_t h = FNV_OFF;
        h ^= a->buf.bln[r];
        return h * FNV_PRM;
    }
    case VEC_STRING: {
        int64_t s = a->buf.str.offsets[r], e = a->buf.str.offsets[r + 1];
        return fnv_bytes((const uint8_t *)a->buf.str.data + s, e - s);
    }
    }
    return 0;
}
static inline uint64_t hash_combine(uint64_t h1, uint64_t h2) {
    return ((h1 << 5) | (h1 >> 59)) ^ h2;
}

/* NA equals NA; doubles by == (src/hash.c:48-69) */
static int val_equal(const VecArray *a, int64_t ra, const VecArray *b, int64_t rb) {
    int va = is_valid(a, ra), vb = is_valid(b, rb);
    if (!va && !vb) return 1;
    if (!va || !vb) return 0;
    switch (a->type) {
    case VEC_INT64: return a->buf.i64[ra] == b->buf.i64[rb];
    case VEC_DOUBLE: return a->buf.dbl[ra] == b->buf.dbl[rb];
    case VEC_BOOL: return a->buf.bln[ra] == b->buf.bln[rb];
    case VEC_STRING: {
        int64_t as = a->buf.str.offsets[ra], al = a->buf.str.offsets[ra + 1] - as;
        int64_t bs = b->buf.str.offsets[rb], bl = b->buf.str.offsets[rb + 1] - bs;
        return al == bl && memcmp(a->buf.str.data + as, b->buf.str.data + bs, (size_t)al) == 0;
    }
    }
    return 0;
}

/* ------------------------------------------------------------------ */
/* aggregate accumulators (src/agg_ops.c:10-255)                       */
/* ------------------------------------------------------------------ */

typedef struct {
    AggKind kind;
    VecType in_type;
    int na_rm;
    int64_t cap;
    int64_t *count;
    double *sum_d;
    int64_t *sum_i;
    double *min_d, *max_d;
    int64_t *min_i, *max_i;
    uint8_t *has_value, *has_na;
} Acc;

static void acc_ensure(Acc *a, int64_t n) {
    if (n <= a->cap) return;
    int64_t nc = a->cap ? a->cap : 64;
    while (nc < n) nc *= 2;
#define GROW(p, T) do { p = (T *)realloc(p, (size_t)nc * sizeof(T)); \
        memset(p + a->cap, 0, (size_t)(nc - a->cap) * sizeof(T)); } while (0)
    GROW(a->count, int64_t);
    GROW(a->sum_d, double);
    GROW(a->sum_i, int64_t);
    GROW(a->min_d, double);
    GROW(a->max_d, double);
    GROW(a->min_i, int64_t);
    GROW(a->max_i, int64_t);
    GROW(a->has_value, uint8_t);
    GROW(a->has_na, uint8_t);
#undef GROW
    a->cap = nc;
}

static void acc_free(Acc *a) {
    free(a->count); free(a->sum_d); free(a->sum_i); free(a->min_d);
    free(a->max_d); free(a->min_i); free(a->max_i); free(a->has_value);
    free(a->has_na);
    memset(a, 0, sizeof(*a));
}

static void acc_feed(Acc *a, int64_t g, const VecArray *col, int64_t row) {
    int valid = col ? is_valid(col, row) : 0;
    switch (a->kind) {
    case AGG_COUNT_STAR: a->count[g]++; break;
    case AGG_COUNT: if (valid) a->count[g]++; break;
    case AGG_SUM:
    case AGG_MEAN:
        if (!valid) { if (!a->na_rm) a->has_na[g] = 1; break; }
        a->count[g]++;
        if (a->in_type == VEC_DOUBLE) a->sum_d[g] += col->buf.dbl[row];
        else if (a->in_type == VEC_INT64)
            a->sum_i[g] = (int64_t)((uint64_t)a->sum_i[g] + (uint64_t)col->buf.i64[row]);
        else if (a->in_type == VEC_BOOL) a->sum_d[g] += (double)col->buf.bln[row];
        break;
    case AGG_MIN:
        if (!valid) { if (!a->na_rm) a->has_na[g] = 1; break; }
        if (a->in_type == VEC_DOUBLE) {
            double v = col->buf.dbl[row];
            if (!a->has_value[g] || v < a->min_d[g]) { a->min_d[g] = v; a->has_value[g] = 1; }
        } else if (a->in_type == VEC_INT64) {
            int64_t v = col->buf.i64[row];
            if (!a->has_value[g] || v < a->min_i[g]) { a->min_i[g] = v; a->has_value[g] = 1; }
        }
        break;
    case AGG_MAX:
        if (!valid) { if (!a->na_rm) a->has_na[g] = 1; break; }
        if (a->in_type == VEC_DOUBLE) {
            double v = col->buf.dbl[row];
            if (!a->has_value[g] || v > a->max_d[g]) { a->max_d[g] = v; a->has_value[g] = 1; }
        } else if (a->in_type == VEC_INT64) {
            int64_t v = col->buf.i64[row];
            if (!a->has_value[g] || v > a->max_i[g]) { a->max_i[g] = v; a->has_value[g] = 1; }
        }
        break;
    }
}

/* result of group g as (value, valid); every output is double */
static void acc_result(Acc *a, int64_t g, double *v, int *valid) {
    *valid = 1;
    *v = 0.0;
    switch (a->kind) {
    case AGG_COUNT:
    case AGG_COUNT_STAR: *v = (double)a->count[g]; return;
    case AGG_SUM:
        if (a->has_na[g]) { *valid = 0; return; }
        *v = (a->in_type == VEC_INT64) ? (double)a->sum_i[g] : a->sum_d[g];
        return;
    case AGG_MEAN:
        if (a->has_na[g]) { *valid = 0; return; }
        if (a->count[g] == 0) { *v = NAN; return; }
        *v = ((a->in_type == VEC_INT64) ? (double)a->sum_i[g] : a->sum_d[g]) / (double)a->count[g];
        return;
    case AGG_MIN:
        if (a->has_na[g]) { *valid = 0; return; }
        if (!a->has_value[g]) { *v = INFINITY; g_warn++; return; }
        *v = (a->in_type == VEC_DOUBLE) ? a->min_d[g] : (double)a->min_i[g];
        return;
    case AGG_MAX:
        if (a->has_na[g]) { *valid = 0; return; }
        if (!a->has_value[g]) { *v = -INFINITY; g_warn++; return; }
        *v = (a->in_type == VEC_DOUBLE) ? a->max_d[g] : (double)a->max_i[g];
        return;
    }
}

/* ------------------------------------------------------------------ */
/* group-agg node                                                      */
/* ------------------------------------------------------------------ */

typedef struct {
    VecNode base;
    VecNode *child;
    int n_keys;
    char **key_names;
    int n_aggs;
    AggSpec *specs;
    int done;
    int use_sorted;
} OGroupAgg;

typedef struct {
    int *key_idx;
    VecType *key_types;
    int *agg_idx;
    VecType *agg_types;
} Resolved;

static Resolved resolve(OGroupAgg *ga) {
    const VecSchema *cs = &ga->child->output_schema;
    Resolved r;
    r.key_idx = (int *)xcalloc((size_t)ga->n_keys, sizeof(int));
    r.key_types = (VecType *)xcalloc((size_t)ga->n_keys, sizeof(VecType));
    r.agg_idx = (int *)xcalloc((size_t)ga->n_aggs, sizeof(int));
    r.agg_types = (VecType *)xcalloc((size_t)ga->n_aggs, sizeof(VecType));
    for (int k = 0; k < ga->n_keys; k++) {
        r.key_idx[k] = schema_find(cs, ga->key_names[k]);
        if (r.key_idx[k] < 0) orc_error("group_by: column not found: %s", ga->key_names[k]);
        r.key_types[k] = cs->col_types[r.key_idx[k]];
    }
    for (int a = 0; a < ga->n_aggs; a++) {
        if (ga->specs[a].kind == AGG_COUNT_STAR) {
            r.agg_idx[a] = -1;
            r.agg_types[a] = VEC_INT64;
        } else {
            r.agg_idx[a] = schema_find(cs, ga->specs[a].input_col);
            if (r.agg_idx[a] < 0) orc_error("summarise: column not found: %s", ga->specs[a].input_col);
            r.agg_types[a] = cs->col_types[r.agg_idx[a]];
        }
    }
    return r;
}
static void resolved_free(Resolved *r) {
    free(r->key_idx); free(r->key_types); free(r->agg_idx); free(r->agg_types);
}

/* Hash path (src/group_agg.c:155-281): linear-probing table of group ids
 * keyed by the combined FNV-1a hash, groups numbered in first-seen order,
 * one copy of each distinct key kept in builders. */
static VecBatch *hash_agg(OGroupAgg *ga) {
    Resolved R = resolve(ga);
    Acc *acc = (Acc *)xcalloc((size_t)ga->n_aggs, sizeof(Acc));
    for (int a = 0; a < ga->n_aggs; a++) {
        acc[a].kind = ga->specs[a].kind;
        acc[a].in_type = R.agg_types[a];
        acc[a].na_rm = ga->specs[a].na_rm;
    }
    Bld *kb = (Bld *)xcalloc((size_t)(ga->n_keys ? ga->n_keys : 1), sizeof(Bld));
    for (int k = 0; k < ga->n_keys; k++) kb[k] = bld_init(R.key_types[k]);
    VecArray *arena = (VecArray *)xcalloc((size_t)(ga->n_keys ? ga->n_keys : 1), sizeof(VecArray));

    int64_t n_slots = 64, n_groups = 0;
    int64_t *slot = (int64_t *)xmalloc((size_t)n_slots * 8);
    uint64_t *shash = (uint64_t *)xmalloc((size_t)n_slots * 8);
    memset(slot, -1, (size_t)n_slots * 8);

    VecBatch *b;
    while ((b = ga->child->next_batch(ga->child)) != NULL) {
        int64_t nl = logical_rows(b);
        for (int64_t li = 0; li < nl; li++) {
            int64_t r = phys_row(b, li);
            uint64_t h = 0;
            for (int k = 0; k < ga->n_keys; k++) {
                uint64_t kh = hash_value(&b->columns[R.key_idx[k]], r);
                h = k == 0 ? kh : hash_combine(h, kh);
            }
            if (n_groups * 10 > n_slots * 7) {   /* grow at 70% load */
                int64_t ns = n_slots * 2;
                int64_t *s2 = (int64_t *)xmalloc((size_t)ns * 8);
                uint64_t *h2 = (uint64_t *)xmalloc((size_t)ns * 8);
                memset(s2, -1, (size_t)ns * 8);
                for (int64_t i = 0; i < n_slots; i++) {
                    if (slot[i] < 0) continue;
                    int64_t j = (int64_t)(shash[i] & (uint64_t)(ns - 1));
                    while (s2[j] >= 0) j = (j + 1) & (ns - 1);
                    s2[j] = slot[i];
                    h2[j] = shash[i];
                }
                free(slot); free(shash);
                slot = s2; shash = h2; n_slots = ns;
            }
            int64_t j = (int64_t)(h & (uint64_t)(n_slots - 1)), gid = -1;
            for (;;) {
                if (slot[j] < 0) {
                    gid = n_groups++;
                    slot[j] = gid;
                    shash[j] = h;
                    for (int k = 0; k < ga->n_keys; k++) {
                        bld_append_one(&kb[k], &b->columns[R.key_idx[k]], r);
                        /* refresh the arena view used for key equality */
                        arena[k].type = kb[k].type;
                        arena[k].validity = kb[k].valid;
                        arena[k].buf.i64 = kb[k].v.i64;
                        if (kb[k].type == VEC_STRING) {
                            arena[k].buf.str.offsets = kb[k].offs;
                            arena[k].buf.str.data = kb[k].sdata;
                        }
                    }
                    for (int a = 0; a < ga->n_aggs; a++) acc_ensure(&acc[a], n_groups);
                    break;
                }
                if (shash[j] == h) {
                    int eq = 1;
                    for (int k = 0; k < ga->n_keys && eq; k++)
                        eq = val_equal(&arena[k], slot[j], &b->columns[R.key_idx[k]], r);
                    if (eq) { gid = slot[j]; break; }
                }
                j = (j + 1) & (n_slots - 1);
            }
            for (int a = 0; a < ga->n_aggs; a++)
                acc_feed(&acc[a], gid, R.agg_idx[a] >= 0 ? &b->columns[R.agg_idx[a]] : NULL, r);
        }
        orc_batch_free(b);
    }

    VecBatch *res = batch_alloc(ga->n_keys + ga->n_aggs, n_groups);
    for (int k = 0; k < ga->n_keys; k++) {
        res->columns[k] = bld_finish(&kb[k]);
        res->columns[k].length = n_groups;
        res->col_names[k] = xstrdup(ga->key_names[k]);
    }
    for (int a = 0; a < ga->n_aggs; a++) {
        VecArray o = arr_alloc(VEC_DOUBLE, n_groups);
        for (int64_t g = 0; g < n_groups; g++) {
            double v; int valid;
            acc_result(&acc[a], g, &v, &valid);
            if (valid) { set_valid(&o, g); o.buf.dbl[g] = v; }
        }
        res->columns[ga->n_keys + a] = o;
        res->col_names[ga->n_keys + a] = xstrdup(ga->specs[a].output_name);
        acc_free(&acc[a]);
    }
    free(acc); free(kb); free(arena); free(slot); free(shash);
    resolved_free(&R);
    return res;
}

/* key comparison with NA last, NaN equal to everything (src/sort.c:32-71) */
static int cmp_key(const VecArray *a, int64_t ra, const VecArray *b, int64_t rb) {
    int va = is_valid(a, ra), vb = is_valid(b, rb);
    if (!va && !vb) return 0;
    if (!va) return 1;
    if (!vb) return -1;
    switch (a->type) {
    case VEC_DOUBLE: {
        double x = a->buf.dbl[ra], y = b->buf.dbl[rb];
        return x < y ? -1 : x > y ? 1 : 0;
    }
    case VEC_INT64: {
        int64_t x = a->buf.i64[ra], y = b->buf.i64[rb];
        return x < y ? -1 : x > y ? 1 : 0;
    }
    case VEC_BOOL: return (int)a->buf.bln[ra] - (int)b->buf.bln[rb];
    case VEC_STRING: {
        int64_t sa = a->buf.str.offsets[ra], la = a->buf.str.offsets[ra + 1] - sa;
        int64_t sb = b->buf.str.offsets[rb], lb = b->buf.str.offsets[rb + 1] - sb;
        int c = memcmp(a->buf.str.data + sa, b->buf.str.data + sb, (size_t)(la < lb ? la : lb));
        if (c == 0) c = la < lb ? -1 : la > lb ? 1 : 0;
        return c;
    }
    }
    return 0;
}

typedef struct { VecArray *cols; const int *kidx; int nk; } SortCtx;

static int cmp_rows(const SortCtx *c, int64_t x, int64_t y) {
    for (int k = 0; k < c->nk; k++) {
        int r = cmp_key(&c->cols[c->kidx[k]], x, &c->cols[c->kidx[k]], y);
        if (r) return r;
    }
    return 0;
}

/* stable top-down merge sort of row indices (src/sort.c:97-116) */
static void msort(int64_t *idx, int64_t *tmp, int64_t n, const SortCtx *c) {
    if (n <= 1) return;
    int64_t m = n / 2;
    msort(idx, tmp, m, c);
    msort(idx + m, tmp, n - m, c);
    int64_t i = 0, j = m, k = 0;
    while (i < m && j < n)
        tmp[k++] = cmp_rows(c, idx[i], idx[j]) <= 0 ? idx[i++] : idx[j++];
    while (i < m) tmp[k++] = idx[i++];
    while (j < n) tmp[k++] = idx[j++];
    memcpy(idx, tmp, (size_t)n * 8);
}

/* Sort path (src/group_agg.c:466-585 over a SortNode, src/sort.c):
 * materialise every logical row, stable-sort by the keys, then one linear
 * scan with group boundaries where the key tuple changes. */
static VecBatch *sorted_agg(OGroupAgg *ga) {
    Resolved R = resolve(ga);
    const VecSchema *cs = &ga->child->output_schema;
    int nc = cs->n_cols;
    Bld *all = (Bld *)xcalloc((size_t)nc, sizeof(Bld));
    for (int c = 0; c < nc; c++) all[c] = bld_init(cs->col_types[c]);
    VecBatch *b;
    while ((b = ga->child->next_batch(ga->child)) != NULL) {
        int64_t nl = logical_rows(b);
        for (int c = 0; c < nc; c++) bld_reserve(&all[c], nl);
        for (int64_t li = 0; li < nl; li++) {
            int64_t r = phys_row(b, li);
            for (int c = 0; c < nc; c++) bld_append_one(&all[c], &b->columns[c], r);
        }
        orc_batch_free(b);
    }
    int64_t n = all[0].len;
    VecArray *cols = (VecArray *)xcalloc((size_t)nc, sizeof(VecArray));
    for (int c = 0; c < nc; c++) cols[c] = bld_finish(&all[c]);
    free(all);
    int64_t *idx = (int64_t *)xmalloc((size_t)n * 8), *tmp = (int64_t *)xmalloc((size_t)n * 8);
    for (int64_t i = 0; i < n; i++) idx[i] = i;
    SortCtx sc = { cols, R.key_idx, ga->n_keys };
    msort(idx, tmp, n, &sc);
    free(tmp);

    Bld *kb = (Bld *)xcalloc((size_t)ga->n_keys, sizeof(Bld));
    for (int k = 0; k < ga->n_keys; k++) kb[k] = bld_init(R.key_types[k]);
    Bld *ab = (Bld *)xcalloc((size_t)ga->n_aggs, sizeof(Bld));
    for (int a = 0; a < ga->n_aggs; a++) ab[a] = bld_init(VEC_DOUBLE);
    Acc *acc = (Acc *)xcalloc((size_t)ga->n_aggs, sizeof(Acc));
    for (int a = 0; a < ga->n_aggs; a++) {
        acc[a].kind = ga->specs[a].kind;
        acc[a].in_type = R.agg_types[a];
        acc[a].na_rm = ga->specs[a].na_rm;
        acc_ensure(&acc[a], 1);
    }
    int64_t cur = -1;
    for (int64_t i = 0; i <= n; i++) {
        int boundary = (i == n);
        if (!boundary && cur >= 0) {
            /* snapshot comparison: NA == NA, values by == (src/group_agg.c:338-373) */
            for (int k = 0; k < ga->n_keys && !boundary; k++)
                boundary = !val_equal(&cols[R.key_idx[k]], cur, &cols[R.key_idx[k]], idx[i]);
        }
        if ((boundary || i == n) && cur >= 0) {
            for (int k = 0; k < ga->n_keys; k++) bld_append_one(&kb[k], &cols[R.key_idx[k]], cur);
            for (int a = 0; a < ga->n_aggs; a++) {
                double v; int valid;
                acc_result(&acc[a], 0, &v, &valid);
                bld_append_dbl(&ab[a], v, valid);
                AggKind kd = acc[a].kind; VecType t = acc[a].in_type; int nr = acc[a].na_rm;
                acc_free(&acc[a]);
                acc[a].kind = kd; acc[a].in_type = t; acc[a].na_rm = nr;
                acc_ensure(&acc[a], 1);
            }
        }
        if (i == n) break;
        if (cur < 0 || boundary) cur = idx[i];
        for (int a = 0; a < ga->n_aggs; a++)
            acc_feed(&acc[a], 0, R.agg_idx[a] >= 0 ? &cols[R.agg_idx[a]] : NULL, idx[i]);
    }
    int64_t ng = ga->n_keys ? kb[0].len : 0;
    VecBatch *res = batch_alloc(ga->n_keys + ga->n_aggs, ng);
    for (int k = 0; k < ga->n_keys; k++) {
        res->columns[k] = bld_finish(&kb[k]);
        res->col_names[k] = xstrdup(ga->key_names[k]);
    }
    for (int a = 0; a < ga->n_aggs; a++) {
        res->columns[ga->n_keys + a] = bld_finish(&ab[a]);
        res->col_names[ga->n_keys + a] = xstrdup(ga->specs[a].output_name);
        acc_free(&acc[a]);
    }
    for (int c = 0; c < nc; c++) arr_free(&cols[c]);
    free(cols); free(idx); free(kb); free(ab); free(acc);
    resolved_free(&R);
    return res;
}

static VecBatch *group_agg_next(VecNode *self) {
    OGroupAgg *ga = (OGroupAgg *)self;
    if (ga->done) return NULL;
    ga->done = 1;
    return ga->use_sorted ? sorted_agg(ga) : hash_agg(ga);
}

static void group_agg_free(VecNode *self) {
    OGroupAgg *ga = (OGroupAgg *)self;
    ga->child->free_node(ga->child);
    for (int k = 0; k < ga->n_keys; k++) free(ga->key_names[k]);
    free(ga->key_names);
    for (int a = 0; a < ga->n_aggs; a++) {
        free(ga->specs[a].output_name);
        free(ga->specs[a].input_col);
    }
    free(ga->specs);
    schema_free(&self->output_schema);
    free(ga);
}

VecNode *orc_group_agg_node_create(VecNode *child, int n_keys, char **key_names,
                                   int n_aggs, AggSpec *specs, const char *temp_dir) {
    OGroupAgg *ga = (OGroupAgg *)xcalloc(1, sizeof(OGroupAgg));
    const VecSchema *cs = &child->output_schema;
    if (temp_dir && n_keys > 0) {
        for (int k = 0; k < n_keys; k++)
            if (schema_find(cs, key_names[k]) < 0)
                orc_error("group_by: column not found: %s", key_names[k]);
        ga->use_sorted = 1;
    }
    ga->child = child;
    ga->n_keys = n_keys;
    ga->key_names = key_names;
    ga->n_aggs = n_aggs;
    ga->specs = specs;
    int no = n_keys + n_aggs;
    char **names = (char **)xcalloc((size_t)(no ? no : 1), sizeof(char *));
    VecType *types = (VecType *)xcalloc((size_t)(no ? no : 1), sizeof(VecType));
    for (int k = 0; k < n_keys; k++) {
        names[k] = key_names[k];
        int idx = schema_find(cs, key_names[k]);
        types[k] = idx >= 0 ? cs->col_types[idx] : VEC_DOUBLE;
    }
    for (int a = 0; a < n_aggs; a++) {
        names[n_keys + a] = specs[a].output_name;
        types[n_keys + a] = VEC_DOUBLE;
    }
    ga->base.output_schema = schema_make(no, names, types);
    free(names);
    free(types);
    ga->base.next_batch = group_agg_next;
    ga->base.free_node = group_agg_free;
    ga->base.kind = "GroupAggNode";
    return &ga->base;
}

/* ------------------------------------------------------------------ */
/* sort node (src/sort.c, the in-memory path)                           */
/* ------------------------------------------------------------------ */

/* compare_value (src/sort.c:32-71): NA last ascending, first descending
 * (its sign is not flipped), values compared by < and >, so NaN is equal to
 * everything and -0 to +0; descending flips the value comparison. */
static int sort_cmp_value(const VecArray *a, int64_t ra, int64_t rb, int desc) {
    int va = is_valid(a, ra), vb = is_valid(a, rb);
    if (!va && !vb) return 0;
    if (!va) return desc ? -1 : 1;
    if (!vb) return desc ? 1 : -1;
    int c = 0;
    switch (a->type) {
    case VEC_DOUBLE: {
        double x = a->buf.dbl[ra], y = a->buf.dbl[rb];
        c = x < y ? -1 : x > y ? 1 : 0;
        break;
    }
    case VEC_INT64: {
        int64_t x = a->buf.i64[ra], y = a->buf.i64[rb];
        c = x < y ? -1 : x > y ? 1 : 0;
        break;
    }
    case VEC_BOOL: c = (int)a->buf.bln[ra] - (int)a->buf.bln[rb]; break;
    case VEC_STRING: {
        int64_t sa = a->buf.str.offsets[ra], la = a->buf.str.offsets[ra + 1] - sa;
        int64_t sb = a->buf.str.offsets[rb], lb = a->buf.str.offsets[rb + 1] - sb;
        c = memcmp(a->buf.str.data + sa, a->buf.str.data + sb, (size_t)(la < lb ? la : lb));
        if (c == 0) c = la < lb ? -1 : la > lb ? 1 : 0;
        break;
    }
    }
    return desc ? -c : c;
}

typedef struct { VecArray *cols; const SortKey *keys; int nk; } OSortCtx;

static int sort_cmp_rows(const OSortCtx *c, int64_t x, int64_t y) {
    for (int k = 0; k < c->nk; k++) {
        int r = sort_cmp_value(&c->cols[c->keys[k].col_index], x, y, c->keys[k].descending);
        if (r) return r;
    }
    return 0;
}

/* stable top-down merge sort (src/sort.c:97-116) */
static void sort_msort(int64_t *idx, int64_t *tmp, int64_t n, const OSortCtx *c) {
    if (n <= 1) return;
    int64_t m = n / 2;
    sort_msort(idx, tmp, m, c);
    sort_msort(idx + m, tmp, n - m, c);
    int64_t i = 0, j = m, k = 0;
    while (i < m && j < n) tmp[k++] = sort_cmp_rows(c, idx[i], idx[j]) <= 0 ? idx[i++] : idx[j++];
    while (i < m) tmp[k++] = idx[i++];
    while (j < n) tmp[k++] = idx[j++];
    memcpy(idx, tmp, (size_t)n * 8);
}

typedef struct {
    SortNode sn;              /* the reference's prefix */
} OSort;

/* every logical row of the child, then one stably sorted batch (an empty
 * input gives one batch of no rows, src/sort.c:488-504) */
static VecBatch *sort_next(VecNode *self) {
    OSort *o = (OSort *)self;
    if (o->sn.phase) return NULL;
    o->sn.phase = 1;
    const VecSchema *cs = &o->sn.base.output_schema;
    int nc = cs->n_cols;
    Bld *all = (Bld *)xcalloc((size_t)(nc ? nc : 1), sizeof(Bld));
    for (int c = 0; c < nc; c++) all[c] = bld_init(cs->col_types[c]);
    VecBatch *b;
    while ((b = o->sn.child->next_batch(o->sn.child)) != NULL) {
        int64_t nl = logical_rows(b);
        for (int c = 0; c < nc; c++) bld_reserve(&all[c], nl);
        for (int64_t li = 0; li < nl; li++) {
            int64_t r = phys_row(b, li);
            for (int c = 0; c < nc; c++) bld_append_one(&all[c], &b->columns[c], r);
        }
        orc_batch_free(b);
    }
    int64_t n = nc ? all[0].len : 0;
    VecArray *cols = (VecArray *)xcalloc((size_t)(nc ? nc : 1), sizeof(VecArray));
    for (int c = 0; c < nc; c++) cols[c] = bld_finish(&all[c]);
    free(all);
    int64_t *idx = (int64_t *)xmalloc((size_t)(n ? n : 1) * 8), *tmp = (int64_t *)xmalloc((size_t)(n ? n : 1) * 8);
    for (int64_t i = 0; i < n; i++) idx[i] = i;
    OSortCtx sc = {cols, o->sn.keys, o->sn.n_keys};
    sort_msort(idx, tmp, n, &sc);
    free(tmp);
    VecBatch *res = batch_alloc(nc, n);
    for (int c = 0; c < nc; c++) {
        Bld ob = bld_init(cs->col_types[c]);
        bld_reserve(&ob, n);
        for (int64_t i = 0; i < n; i++) bld_append_one(&ob, &cols[c], idx[i]);
        res->columns[c] = bld_finish(&ob);
        res->col_names[c] = xstrdup(cs->col_names[c]);
        arr_free(&cols[c]);
    }
    free(cols);
    free(idx);
    return res;
}

static void sort_free(VecNode *self) {
    OSort *o = (OSort *)self;
    o->sn.child->free_node(o->sn.child);
    free(o->sn.keys);
    free(o->sn.temp_dir);
    schema_free(&self->output_schema);
    free(o);
}

VecNode *orc_sort_node_create(VecNode *child, int n_keys, SortKey *keys, const char *temp_dir) {
    OSort *o = (OSort *)xcalloc(1, sizeof(OSort));
    o->sn.child = child;
    o->sn.n_keys = n_keys;
    o->sn.keys = keys;
    o->sn.mem_budget = 1024LL * 1024 * 1024;
    o->sn.temp_dir = temp_dir ? xstrdup(temp_dir) : NULL;
    const VecSchema *cs = &child->output_schema;
    o->sn.base.output_schema = schema_make(cs->n_cols, cs->col_names, cs->col_types);
    o->sn.base.next_batch = sort_next;
    o->sn.base.free_node = sort_free;
    o->sn.base.kind = "SortNode";
    return &o->sn.base;
}

/* ------------------------------------------------------------------ */
/* hash join (src/join.c)                                              */
/* ------------------------------------------------------------------ */

typedef struct {
    VecNode base;
    VecNode *left, *right;
    JoinKind kind;
    int n_keys;
    JoinKey *keys;
    char *sx, *sy;
    int state;                 /* 0 build, 1 probe, 2 finalize, 3 done */
    int r_ncols;
    VecArray *r_cols;
    int64_t n_build, n_slots;
    int64_t *head, *next;
    uint64_t *shash;
    int *lk, *rk;
    int *r_nonkey;
    int r_nonkey_n;
    uint8_t *build_matched;
    int64_t fin_cursor;
} OJoin;

static uint64_t join_hash(const VecArray *cols, const int *kidx, int nk, int64_t r) {
    uint64_t h = 0;
    for (int k = 0; k < nk; k++) {
        uint64_t kh = hash_value(&cols[kidx[k]], r);
        h = k == 0 ? kh : hash_combine(h, kh);
    }
    return h;
}

/* NA never matches (src/join.c:77-113).  The switch is on the probe
 * column's type, as in the reference. */
static int join_eq(const VecArray *pc, const int *pk, const VecArray *bc,
                   const int *bk, int nk, int64_t pr, int64_t br) {
    for (int k = 0; k < nk; k++) {
        const VecArray *pa = &pc[pk[k]], *ba = &bc[bk[k]];
        if (!is_valid(pa, pr) || !is_valid(ba, br)) return 0;
        switch (pa->type) {
        case VEC_INT64: if (pa->buf.i64[pr] != ba->buf.i64[br]) return 0; break;
        case VEC_DOUBLE: if (pa->buf.dbl[pr] != ba->buf.dbl[br]) return 0; break;
        case VEC_BOOL: if (pa->buf.bln[pr] != ba->buf.bln[br]) return 0; break;
        case VEC_STRING: {
            int64_t ps = pa->buf.str.offsets[pr], pl = pa->buf.str.offsets[pr + 1] - ps;
            int64_t bs = ba->buf.str.offsets[br], bl = ba->buf.str.offsets[br + 1] - bs;
            if (pl != bl || memcmp(pa->buf.str.data + ps, ba->buf.str.data + bs, (size_t)pl)) return 0;
            break;
        }
        }
    }
    return 1;
}

static void join_build(OJoin *j) {
    const VecSchema *rs = &j->right->output_schema;
    j->r_ncols = rs->n_cols;
    Bld *rb = (Bld *)xcalloc((size_t)j->r_ncols, sizeof(Bld));
    for (int c = 0; c < j->r_ncols; c++) rb[c] = bld_init(rs->col_types[c]);
    VecBatch *b;
    while ((b = j->right->next_batch(j->right)) != NULL) {
        int64_t nl = logical_rows(b);
        for (int c = 0; c < j->r_ncols; c++) bld_reserve(&rb[c], nl);
        for (int64_t li = 0; li < nl; li++) {
            int64_t p = phys_row(b, li);
            for (int c = 0; c < j->r_ncols; c++) bld_append_one(&rb[c], &b->columns[c], p);
        }
        orc_batch_free(b);
    }
    int64_t n = j->r_ncols ? rb[0].len : 0;
    j->r_cols = (VecArray *)xcalloc((size_t)j->r_ncols, sizeof(VecArray));
    for (int c = 0; c < j->r_ncols; c++) j->r_cols[c] = bld_finish(&rb[c]);
    free(rb);
    /* build keys take the common type with the probe key (src/join.c:190-205) */
    const VecSchema *ls = &j->left->output_schema;
    for (int k = 0; k < j->n_keys; k++) {
        VecType lt = ls->col_types[j->lk[k]], rt = j->r_cols[j->rk[k]].type;
        if (lt != rt) {
            VecType ct = common_type(lt, rt);
            if (rt != ct) {
                VecArray co = arr_coerce(&j->r_cols[j->rk[k]], ct);
                arr_free(&j->r_cols[j->rk[k]]);
                j->r_cols[j->rk[k]] = co;
            }
        }
    }
    /* slots: 64 * 2^k >= 2 * n_build; chains by head insertion, so equal
     * hashes chain in descending build-row order (src/join.c:23-61) */
    int64_t nb = n > 0 ? n : 1;
    int64_t ns = 64;
    while (ns < nb * 2) ns *= 2;
    j->n_slots = ns;
    j->n_build = nb;
    j->head = (int64_t *)xmalloc((size_t)ns * 8);
    j->shash = (uint64_t *)xmalloc((size_t)ns * 8);
    j->next = (int64_t *)xmalloc((size_t)nb * 8);
    memset(j->head, -1, (size_t)ns * 8);
    memset(j->next, -1, (size_t)nb * 8);
    for (int64_t r = 0; r < n; r++) {
        uint64_t h = join_hash(j->r_cols, j->rk, j->n_keys, r);
        int64_t s = (int64_t)(h & (uint64_t)(ns - 1));
        for (;;) {
            if (j->head[s] == -1) { j->head[s] = r; j->shash[s] = h; break; }
            if (j->shash[s] == h) { j->next[r] = j->head[s]; j->head[s] = r; break; }
            s = (s + 1) & (ns - 1);
        }
    }
    if (j->kind == JOIN_FULL) j->build_matched = (uint8_t *)xcalloc((size_t)vbytes(nb), 1);
}

static int64_t chain_first(OJoin *j, uint64_t h, const VecArray *pc, int64_t pr) {
    int64_t s = (int64_t)(h & (uint64_t)(j->n_slots - 1));
    for (;;) {
        if (j->head[s] == -1) return -1;
        if (j->shash[s] == h) {
            for (int64_t br = j->head[s]; br >= 0; br = j->next[br])
                if (join_eq(pc, j->lk, j->r_cols, j->rk, j->n_keys, pr, br)) return br;
        }
        s = (s + 1) & (j->n_slots - 1);
    }
}
static int64_t chain_next(OJoin *j, int64_t br, const VecArray *pc, int64_t pr) {
    for (br = j->next[br]; br >= 0; br = j->next[br])
        if (join_eq(pc, j->lk, j->r_cols, j->rk, j->n_keys, pr, br)) return br;
    return -1;
}

static VecBatch *emit(OJoin *j, Bld *out, int oc) {
    int64_t n = out[0].len;
    if (n == 0) {
        for (int c = 0; c < oc; c++) bld_free(&out[c]);
        return NULL;
    }
    VecBatch *r = batch_alloc(oc, n);
    for (int c = 0; c < oc; c++) {
        r->columns[c] = bld_finish(&out[c]);
        r->col_names[c] = xstrdup(j->base.output_schema.col_names[c]);
    }
    return r;
}

static VecBatch *join_probe(OJoin *j, VecBatch *pb) {
    int lc = j->left->output_schema.n_cols, oc = j->base.output_schema.n_cols;
    int64_t nl = logical_rows(pb);
    /* probe keys coerced to the build key type for hashing and compare */
    VecArray *pcols = pb->columns;
    VecArray *tmp = NULL;
    int *coerced = (int *)xcalloc((size_t)(j->n_keys ? j->n_keys : 1), sizeof(int));
    for (int k = 0; k < j->n_keys; k++) {
        if (pb->columns[j->lk[k]].type != j->r_cols[j->rk[k]].type) {
            if (!tmp) {
                tmp = (VecArray *)xmalloc((size_t)lc * sizeof(VecArray));
                memcpy(tmp, pb->columns, (size_t)lc * sizeof(VecArray));
            }
            tmp[j->lk[k]] = arr_coerce(&pb->columns[j->lk[k]], j->r_cols[j->rk[k]].type);
            coerced[k] = 1;
        }
    }
    if (tmp) pcols = tmp;
    /* the chain walk of LEFT/FULL joins reads the uncoerced probe columns
     * in the reference (src/join.c:408-410, 427-429) */
    const VecArray *walk_cols = (g_join_quirk && (j->kind == JOIN_LEFT || j->kind == JOIN_FULL))
                                ? pb->columns : pcols;
    Bld *out = (Bld *)xcalloc((size_t)oc, sizeof(Bld));
    for (int c = 0; c < oc; c++) {
        out[c] = bld_init(j->base.output_schema.col_types[c]);
        bld_reserve(&out[c], nl);
    }
    uint8_t *matched = (uint8_t *)xcalloc((size_t)vbytes(nl > 0 ? nl : 1), 1);
    for (int64_t li = 0; li < nl; li++) {
        int64_t pr = phys_row(pb, li);
        uint64_t h = join_hash(pcols, j->lk, j->n_keys, pr);
        int64_t br = chain_first(j, h, pcols, pr);
        switch (j->kind) {
        case JOIN_SEMI:
            if (br >= 0) for (int c = 0; c < lc; c++) bld_append_one(&out[c], &pb->columns[c], pr);
            break;
        case JOIN_ANTI:
            if (br < 0) for (int c = 0; c < lc; c++) bld_append_one(&out[c], &pb->columns[c], pr);
            break;
        default: {
            const VecArray *wc = (j->kind == JOIN_INNER) ? pcols : walk_cols;
            if (br >= 0) matched[li >> 3] |= (uint8_t)(1u << (li & 7));
            while (br >= 0) {
                if (j->kind == JOIN_FULL) j->build_matched[br >> 3] |= (uint8_t)(1u << (br & 7));
                for (int c = 0; c < lc; c++) bld_append_one(&out[c], &pb->columns[c], pr);
                for (int q = 0; q < j->r_nonkey_n; q++)
                    bld_append_one(&out[lc + q], &j->r_cols[j->r_nonkey[q]], br);
                br = chain_next(j, br, wc, pr);
            }
            break;
        }
        }
    }
    /* unmatched probe rows after all matches of the batch (src/join.c:438-450) */
    if (j->kind == JOIN_LEFT || j->kind == JOIN_FULL) {
        for (int64_t li = 0; li < nl; li++) {
            if (matched[li >> 3] & (1u << (li & 7))) continue;
            int64_t pr = phys_row(pb, li);
            for (int c = 0; c < lc; c++) bld_append_one(&out[c], &pb->columns[c], pr);
            for (int q = 0; q < j->r_nonkey_n; q++) bld_append_na(&out[lc + q]);
        }
    }
    free(matched);
    if (tmp) {
        for (int k = 0; k < j->n_keys; k++)
            if (coerced[k]) arr_free(&tmp[j->lk[k]]);
        free(tmp);
    }
    free(coerced);
    VecBatch *r = emit(j, out, oc);
    free(out);
    return r;
}

/* FULL join: unmatched build rows in chunks of 65536 (src/join.c:489-551) */
static VecBatch *join_finalize(OJoin *j) {
    int lc = j->left->output_schema.n_cols, oc = j->base.output_schema.n_cols;
    Bld *out = (Bld *)xcalloc((size_t)oc, sizeof(Bld));
    for (int c = 0; c < oc; c++) out[c] = bld_init(j->base.output_schema.col_types[c]);
    int64_t nb = j->r_ncols ? j->r_cols[0].length : 0;
    int64_t emitted = 0, br = j->fin_cursor;
    for (; br < nb && emitted < 65536; br++) {
        if (j->build_matched[br >> 3] & (1u << (br & 7))) continue;
        for (int c = 0; c < lc; c++) {
            int rkc = -1;
            for (int k = 0; k < j->n_keys; k++)
                if (j->lk[k] == c) { rkc = j->rk[k]; break; }
            if (rkc >= 0) bld_append_one(&out[c], &j->r_cols[rkc], br);
            else bld_append_na(&out[c]);
        }
        for (int q = 0; q < j->r_nonkey_n; q++)
            bld_append_one(&out[lc + q], &j->r_cols[j->r_nonkey[q]], br);
        emitted++;
    }
    j->fin_cursor = br;
    VecBatch *r = emit(j, out, oc);
    free(out);
    return r;
}

static VecBatch *join_next(VecNode *self) {
    OJoin *j = (OJoin *)self;
    if (j->state == 0) { join_build(j); j->state = 1; }
    while (j->state == 1) {
        VecBatch *pb = j->left->next_batch(j->left);
        if (!pb) { j->state = j->kind == JOIN_FULL ? 2 : 3; break; }
        VecBatch *r = join_probe(j, pb);
        orc_batch_free(pb);
        if (r) return r;
    }
    while (j->state == 2) {
        VecBatch *r = join_finalize(j);
        if (r) return r;
        j->state = 3;
    }
    return NULL;
}

static void join_free(VecNode *self) {
    OJoin *j = (OJoin *)self;
    j->left->free_node(j->left);
    j->right->free_node(j->right);
    free(j->keys); free(j->sx); free(j->sy); free(j->lk); free(j->rk);
    free(j->r_nonkey); free(j->build_matched);
    if (j->r_cols) {
        for (int c = 0; c < j->r_ncols; c++) arr_free(&j->r_cols[c]);
        free(j->r_cols);
    }
    free(j->head); free(j->shash); free(j->next);
    schema_free(&self->output_schema);
    free(j);
}

VecNode *orc_join_node_create(VecNode *left, VecNode *right, JoinKind kind,
                              int n_keys, JoinKey *keys,
                              const char *sx, const char *sy) {
    static const char *kn[] = { "inner_join", "left_join", "full_join", "semi_join", "anti_join" };
    const VecSchema *ls = &left->output_schema, *rs = &right->output_schema;
    for (int k = 0; k < n_keys; k++) {
        VecType lt = ls->col_types[keys[k].left_col], rt = rs->col_types[keys[k].right_col];
        if (lt != rt && (lt == VEC_STRING || rt == VEC_STRING))
            orc_error("%s key type mismatch: x.%s (%s) vs y.%s (%s)", kn[kind],
                      ls->col_names[keys[k].left_col],
                      lt == VEC_STRING ? "string" : lt == VEC_DOUBLE ? "double" : lt == VEC_INT64 ? "int64" : "bool",
                      rs->col_names[keys[k].right_col],
                      rt == VEC_STRING ? "string" : rt == VEC_DOUBLE ? "double" : rt == VEC_INT64 ? "int64" : "bool");
    }
    OJoin *j = (OJoin *)xcalloc(1, sizeof(OJoin));
    j->left = left; j->right = right; j->kind = kind; j->n_keys = n_keys; j->keys = keys;
    j->sx = xstrdup(sx); j->sy = xstrdup(sy);
    j->lk = (int *)xcalloc((size_t)(n_keys ? n_keys : 1), sizeof(int));
    j->rk = (int *)xcalloc((size_t)(n_keys ? n_keys : 1), sizeof(int));
    for (int k = 0; k < n_keys; k++) { j->lk[k] = keys[k].left_col; j->rk[k] = keys[k].right_col; }
    int *is_rkey = (int *)xcalloc((size_t)(rs->n_cols ? rs->n_cols : 1), sizeof(int));
    for (int k = 0; k < n_keys; k++) is_rkey[keys[k].right_col] = 1;
    j->r_nonkey = (int *)xcalloc((size_t)(rs->n_cols ? rs->n_cols : 1), sizeof(int));
    if (kind == JOIN_INNER || kind == JOIN_LEFT || kind == JOIN_FULL)
        for (int c = 0; c < rs->n_cols; c++)
            if (!is_rkey[c]) j->r_nonkey[j->r_nonkey_n++] = c;
    /* output schema: left ++ right non-key columns, suffixes on name
     * collisions (src/join.c:703-784); SEMI/ANTI keep the left schema */
    int on = ls->n_cols + ((kind == JOIN_SEMI || kind == JOIN_ANTI) ? 0 : j->r_nonkey_n);
    char **names = (char **)xcalloc((size_t)(on ? on : 1), sizeof(char *));
    VecType *types = (VecType *)xcalloc((size_t)(on ? on : 1), sizeof(VecType));
    for (int i = 0; i < ls->n_cols; i++) { names[i] = xstrdup(ls->col_names[i]); types[i] = ls->col_types[i]; }
    if (!(kind == JOIN_SEMI || kind == JOIN_ANTI)) {
        for (int q = 0; q < j->r_nonkey_n; q++) {
            int c = j->r_nonkey[q];
            const char *rn = rs->col_names[c];
            int coll = -1;
            for (int li = 0; li < ls->n_cols; li++)
                if (strcmp(ls->col_names[li], rn) == 0) { coll = li; break; }
            if (coll >= 0) {
                size_t l1 = strlen(rn) + strlen(sy) + 1;
                names[ls->n_cols + q] = (char *)xmalloc(l1);
                snprintf(names[ls->n_cols + q], l1, "%s%s", rn, sy);
                size_t l2 = strlen(ls->col_names[coll]) + strlen(sx) + 1;
                free(names[coll]);
                names[coll] = (char *)xmalloc(l2);
                snprintf(names[coll], l2, "%s%s", ls->col_names[coll], sx);
            } else {
                names[ls->n_cols + q] = xstrdup(rn);
            }
            types[ls->n_cols + q] = rs->col_types[c];
        }
    }
    j->base.output_schema = schema_make(on, names, types);
    for (int i = 0; i < on; i++) free(names[i]);
    free(names); free(types); free(is_rkey);
    j->base.next_batch = join_next;
    j->base.free_node = join_free;
    j->base.kind = "JoinNode";
    return &j->base;
}

/* ------------------------------------------------------------------ */
/* guards                                                              */
/* ------------------------------------------------------------------ */

#define GUARD_BEGIN \
    jmp_buf jb; jmp_buf *prev = g_jmp; g_msg[0] = 0; \
    if (setjmp(jb)) { g_jmp = prev; return NULL; } \
    g_jmp = &jb;
#define GUARD_END g_jmp = prev;

VecBatch *orc_guard_next_batch(VecNode *n) {
    GUARD_BEGIN
    VecBatch *b = n->next_batch(n);
    GUARD_END
    return b;
}
VecNode *orc_guard_filter(VecNode *child, VecExpr *pred) {
    GUARD_BEGIN
    VecNode *r = orc_filter_node_create(child, pred);
    GUARD_END
    return r;
}
VecNode *orc_guard_project(VecNode *child, int n, ProjEntry *entries) {
    GUARD_BEGIN
    VecNode *r = orc_project_node_create(child, n, entries);
    GUARD_END
    return r;
}
VecNode *orc_guard_group_agg(VecNode *child, int n_keys, char **key_names,
                             int n_aggs, AggSpec *specs, const char *temp_dir) {
    GUARD_BEGIN
    VecNode *r = orc_group_agg_node_create(child, n_keys, key_names, n_aggs, specs, temp_dir);
    GUARD_END
    return r;
}
VecNode *orc_guard_sort(VecNode *child, int n_keys, SortKey *keys, const char *temp_dir) {
    GUARD_BEGIN
    VecNode *r = orc_sort_node_create(child, n_keys, keys, temp_dir);
    GUARD_END
    return r;
}
VecNode *orc_guard_join(VecNode *l, VecNode *r, JoinKind kind, int n_keys,
                        JoinKey *keys, const char *sx, const char *sy) {
    GUARD_BEGIN
    VecNode *x = orc_join_node_create(l, r, kind, n_keys, keys, sx, sy);
    GUARD_END
    return x;
}

/* ------------------------------------------------------------------ */
/* exactly rounded summation                                           */
/* ------------------------------------------------------------------ */

/* Shewchuk, "Adaptive Precision Floating-Point Arithmetic and Fast Robust
 * Geometric Predicates" (1997): keep the running sum as a list of
 * non-overlapping partials, each update an exact TwoSum; the final
 * rounding follows the half-even correction used by Python's math.fsum. */
typedef struct { double *p; int64_t n, cap; double special; int has_special; } FSum;

static void fsum_add(FSum *s, double x) {
    if (!isfinite(x)) {
        s->special = s->has_special ? s->special + x : x;
        s->has_special = 1;
        return;
    }
    int64_t i = 0;
    for (int64_t j = 0; j < s->n; j++) {
        double y = s->p[j];
        if (fabs(x) < fabs(y)) { double t = x; x = y; y = t; }
        double hi = x + y;
        double lo = y - (hi - x);
        if (lo != 0.0) s->p[i++] = lo;
        x = hi;
    }
    s->n = i;
    if (x != 0.0) {
        if (s->n >= s->cap) {
            s->cap = s->cap ? s->cap * 2 : 32;
            s->p = (double *)realloc(s->p, (size_t)s->cap * sizeof(double));
        }
        s->p[s->n++] = x;
    }
}

static double fsum_result(FSum *s) {
    if (s->has_special) return s->special;
    int64_t n = s->n;
    if (n == 0) return 0.0;
    double hi = s->p[--n], lo = 0.0;
    while (n > 0) {
        double x = hi, y = s->p[--n];
        hi = x + y;
        double yr = hi - x;
        lo = y - yr;
        if (lo != 0.0) break;
    }
    if (n > 0 && ((lo < 0.0 && s->p[n - 1] < 0.0) || (lo > 0.0 && s->p[n - 1] > 0.0))) {
        double y = lo * 2.0, x = hi + y, yr = x - hi;
        if (y == yr) hi = x;
    }
    return hi;
}

double orc_exact_sum(const double *x, int64_t n) {
    FSum s;
    memset(&s, 0, sizeof(s));
    for (int64_t i = 0; i < n; i++) fsum_add(&s, x[i]);
    double r = fsum_result(&s);
    free(s.p);
    return r;
}

double orc_exact_sum_products(const double *a, const double *b, int64_t n) {
    FSum s;
    memset(&s, 0, sizeof(s));
    for (int64_t i = 0; i < n; i++) {
        volatile double prod = a[i] * b[i];   /* one rounding, no contraction */
        fsum_add(&s, prod);
    }
    double r = fsum_result(&s);
    free(s.p);
    return r;
}
