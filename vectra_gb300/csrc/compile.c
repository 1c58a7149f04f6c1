/*
 * compile.c -- turns the reference's expression trees (VecExpr,
 * src/expr.h:27-63) into what the kernels execute:
 *
 *  - vg_compile_pred: a conjunction of column-vs-constant comparisons,
 *    each folded into an integer range on the column's own values.  The
 *    reference compares an int64 column with a double literal by converting
 *    the column to double (src/scalar_ops.c:110-142); since that conversion
 *    is monotone, the set of int64 values passing `(double)v OP c` is an
 *    integer interval, found here once per query by binary search.  Double
 *    columns compare on the order-preserving integer image of their bits.
 *    The kernel then needs no floating-point work at all, and the answer is
 *    exactly the reference's, NaN included (NaN compares as equal there,
 *    src/scalar_ops.c:130-131).
 *  - vg_compile_prog: any other supported expression, as a postfix program
 *    that applies the reference's coercion (bool < int64 < double,
 *    src/coerce.c:7-16) and R's three-valued logic (src/scalar_ops.c:151-203).
 *  - vg_compile_value: columns, constants and one arithmetic operation on
 *    them, read directly by the fused aggregation kernel.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "vg_host.h"

static char g_cerr[512];
const char *vg_compile_error(void) { return g_cerr; }

static int cerr(const char *fmt, const char *arg) {
    snprintf(g_cerr, sizeof(g_cerr), fmt, arg ? arg : "");
    return -1;
}

void vg_expr_free(VecExpr *e) {
    if (!e) return;
    free(e->col_name);
    free(e->lit_str);
    vg_expr_free(e->left);
    vg_expr_free(e->right);
    vg_expr_free(e->operand);
    vg_expr_free(e->cond);
    vg_expr_free(e->then_expr);
    vg_expr_free(e->else_expr);
    free(e);
}

int vg_expr_refs(const VecExpr *e, const char *name) {
    if (!e) return 0;
    if (e->kind == EXPR_COL_REF) return e->col_name && strcmp(e->col_name, name) == 0;
    return vg_expr_refs(e->left, name) || vg_expr_refs(e->right, name) ||
           vg_expr_refs(e->operand, name) || vg_expr_refs(e->cond, name) ||
           vg_expr_refs(e->then_expr, name) || vg_expr_refs(e->else_expr, name);
}

static int common_type(int a, int b) {
    if (a == b) return a;
    if (a == VEC_STRING || b == VEC_STRING) return -1;
    if (a == VEC_DOUBLE || b == VEC_DOUBLE) return VEC_DOUBLE;
    if (a == VEC_INT64 || b == VEC_INT64) return VEC_INT64;
    return VEC_BOOL;
}

static int cmp_code(char op, char op2) {
    if (op == '=' && op2 == '=') return VG_CMP_EQ;
    if (op == '!' && op2 == '=') return VG_CMP_NE;
    if (op == '<' && op2 == '=') return VG_CMP_LE;
    if (op == '<') return VG_CMP_LT;
    if (op == '>' && op2 == '=') return VG_CMP_GE;
    if (op == '>') return VG_CMP_GT;
    return -1;
}

static int flip_code(int c) {
    switch (c) {
    case VG_CMP_LT: return VG_CMP_GT;
    case VG_CMP_LE: return VG_CMP_GE;
    case VG_CMP_GT: return VG_CMP_LT;
    case VG_CMP_GE: return VG_CMP_LE;
    default: return c;
    }
}

/* type of an expression under the reference's rules; -1 if unsupported */
static int type_of(const VecExpr *e, vg_colmap_fn map, void *ctx) {
    switch (e->kind) {
    case EXPR_COL_REF: {
        int t = -1;
        if (map(ctx, e->col_name, &t) < 0) return -2;
        return t;
    }
    case EXPR_LIT_INT64: return VEC_INT64;
    case EXPR_LIT_DOUBLE: return VEC_DOUBLE;
    case EXPR_LIT_BOOL: return VEC_BOOL;
    case EXPR_LIT_STRING: return VEC_STRING;
    case EXPR_LIT_NA: return e->result_type;
    case EXPR_ARITH: {
        int l = type_of(e->left, map, ctx), r = type_of(e->right, map, ctx);
        if (l < 0) return l;
        if (r < 0) return r;
        int c = common_type(l, r);
        if (c == VEC_BOOL) c = VEC_INT64;
        return c;
    }
    case EXPR_CMP: case EXPR_BOOL: case EXPR_IS_NA: case EXPR_GREPL: return VEC_BOOL;
    case EXPR_NEGATE: return type_of(e->operand, map, ctx);
    case EXPR_NCHAR: return VEC_INT64;
    case EXPR_SUBSTR: return VEC_STRING;
    default: return -1;
    }
}

int vg_expr_type(const VecExpr *e) { return e ? (int)e->result_type : -1; }

/* ------------------------------------------------------------------ */
/* range folding                                                       */
/* ------------------------------------------------------------------ */

static int64_t ord_of(double d) {
    int64_t s;
    memcpy(&s, &d, 8);
    return s >= 0 ? s : (int64_t)((uint64_t)s ^ 0x7FFFFFFFFFFFFFFFull);
}

/* smallest v in [lo, hi] with (double)v >= c (ge=1) or > c (ge=0);
 * returns 0 if none.  (double) is monotone non-decreasing in v. */
static int min_int_passing(double c, int ge, int64_t *out) {
    int64_t lo = INT64_MIN, hi = INT64_MAX;
#define PASS(v) (ge ? ((double)(v) >= c) : ((double)(v) > c))
    if (!PASS(hi)) return 0;
    if (PASS(lo)) { *out = lo; return 1; }
    /* invariant: !PASS(lo), PASS(hi) */
    while ((uint64_t)hi - (uint64_t)lo > 1) {
        int64_t mid = (int64_t)((uint64_t)lo + (((uint64_t)hi - (uint64_t)lo) >> 1));
        if (PASS(mid)) hi = mid; else lo = mid;
    }
#undef PASS
    *out = hi;
    return 1;
}

/* Fills t (column index set by caller) for `col <code> literal`. */
static void fold_term(int col_type, int lit_type, int64_t li, double ld, int code, VgTerm *t) {
    t->nan_keep = 0;
    int common = common_type(col_type, lit_type);
    if (common == VEC_BOOL) common = VEC_INT64;
    if (common == VEC_INT64) {
        int64_t L = (lit_type == VEC_BOOL) ? (li ? 1 : 0) : li;
        t->domain = col_type == VEC_BOOL ? VG_DOM_BOOL : VG_DOM_INT64;
        t->kind = VG_TERM_RANGE;
        switch (code) {
        case VG_CMP_EQ: t->lo = L; t->hi = L; break;
        case VG_CMP_NE: t->lo = L; t->hi = L; t->kind = VG_TERM_NOT_RANGE; break;
        case VG_CMP_LT:
            if (L == INT64_MIN) { t->kind = VG_TERM_NONE; break; }
            t->lo = INT64_MIN; t->hi = L - 1; break;
        case VG_CMP_LE: t->lo = INT64_MIN; t->hi = L; break;
        case VG_CMP_GT:
            if (L == INT64_MAX) { t->kind = VG_TERM_NONE; break; }
            t->lo = L + 1; t->hi = INT64_MAX; break;
        default: t->lo = L; t->hi = INT64_MAX; break;
        }
        return;
    }
    /* common type double */
    double c = (lit_type == VEC_DOUBLE) ? ld : (lit_type == VEC_BOOL ? (li ? 1.0 : 0.0) : (double)li);
    int eq_like = (code == VG_CMP_EQ || code == VG_CMP_LE || code == VG_CMP_GE);
    if (isnan(c)) {           /* every comparison with NaN has cmp == 0 */
        t->kind = eq_like ? VG_TERM_NOT_NA : VG_TERM_NONE;
        return;
    }
    if (col_type == VEC_DOUBLE) {
        int64_t lo_c = (c == 0.0) ? -1 : ord_of(c);
        int64_t hi_c = (c == 0.0) ? 0 : ord_of(c);
        t->domain = VG_DOM_DOUBLE;
        t->nan_keep = eq_like;   /* a NaN value compares as equal */
        t->kind = VG_TERM_RANGE;
        switch (code) {
        case VG_CMP_EQ: t->lo = lo_c; t->hi = hi_c; break;
        case VG_CMP_NE: t->lo = lo_c; t->hi = hi_c; t->kind = VG_TERM_NOT_RANGE; break;
        case VG_CMP_LT: t->lo = INT64_MIN; t->hi = lo_c - 1; break;
        case VG_CMP_LE: t->lo = INT64_MIN; t->hi = hi_c; break;
        case VG_CMP_GT: t->lo = hi_c + 1; t->hi = INT64_MAX; break;
        default: t->lo = lo_c; t->hi = INT64_MAX; break;
        }
        return;
    }
    /* int64 / bool column against a double: (double)v OP c */
    t->domain = col_type == VEC_BOOL ? VG_DOM_BOOL : VG_DOM_INT64;
    int64_t a, b;
    int has_a, has_b;
    t->kind = VG_TERM_RANGE;
    switch (code) {
    case VG_CMP_GE:
        if (!min_int_passing(c, 1, &a)) { t->kind = VG_TERM_NONE; return; }
        t->lo = a; t->hi = INT64_MAX; return;
    case VG_CMP_GT:
        if (!min_int_passing(c, 0, &a)) { t->kind = VG_TERM_NONE; return; }
        t->lo = a; t->hi = INT64_MAX; return;
    case VG_CMP_LE:   /* max v with (double)v <= c  = (min v with > c) - 1 */
        has_b = min_int_passing(c, 0, &b);
        if (!has_b) { t->lo = INT64_MIN; t->hi = INT64_MAX; return; }
        if (b == INT64_MIN) { t->kind = VG_TERM_NONE; return; }
        t->lo = INT64_MIN; t->hi = b - 1; return;
    case VG_CMP_LT:
        has_b = min_int_passing(c, 1, &b);
        if (!has_b) { t->lo = INT64_MIN; t->hi = INT64_MAX; return; }
        if (b == INT64_MIN) { t->kind = VG_TERM_NONE; return; }
        t->lo = INT64_MIN; t->hi = b - 1; return;
    default: {  /* EQ / NE: [min v with >= c, max v with <= c] */
        has_a = min_int_passing(c, 1, &a);
        has_b = min_int_passing(c, 0, &b);
        int64_t hi_v = has_b ? b - 1 : INT64_MAX;
        int empty = !has_a || (has_b && b == INT64_MIN) || a > hi_v;
        if (code == VG_CMP_EQ) {
            if (empty) { t->kind = VG_TERM_NONE; return; }
            t->lo = a; t->hi = hi_v; return;
        }
        if (empty) { t->kind = VG_TERM_NOT_NA; return; }
        t->kind = VG_TERM_NOT_RANGE; t->lo = a; t->hi = hi_v; return;
    }
    }
}

static int is_lit(const VecExpr *e) {
    return e->kind == EXPR_LIT_INT64 || e->kind == EXPR_LIT_DOUBLE || e->kind == EXPR_LIT_BOOL;
}
static int lit_type(const VecExpr *e) {
    return e->kind == EXPR_LIT_INT64 ? VEC_INT64 : e->kind == EXPR_LIT_DOUBLE ? VEC_DOUBLE : VEC_BOOL;
}

/* returns 1 ok, 0 not a conjunction of simple terms, -1 error */
static int pred_rec(const VecExpr *e, vg_colmap_fn map, void *ctx, VgPred *out, int negate) {
    if (out->n_terms >= VG_MAX_TERMS) return 0;
    VgTerm *t = &out->term[out->n_terms];
    memset(t, 0, sizeof(*t));
    switch (e->kind) {
    case EXPR_BOOL:
        if (e->op == '&' && !negate) {
            int a = pred_rec(e->left, map, ctx, out, 0);
            if (a <= 0) return a;
            return pred_rec(e->right, map, ctx, out, 0);
        }
        if (e->op == '!') return pred_rec(e->operand, map, ctx, out, !negate);
        return 0;
    case EXPR_LIT_BOOL:
        if ((e->lit_bln != 0) != (negate != 0)) return 1;    /* TRUE: no term */
        t->kind = VG_TERM_NONE; out->n_terms++; return 1;
    case EXPR_LIT_NA:
        t->kind = VG_TERM_NONE; out->n_terms++; return 1;
    case EXPR_COL_REF: {
        int ty = -1;
        int ci = map(ctx, e->col_name, &ty);
        if (ci < 0) return cerr("column not found: %s", e->col_name);
        if (ty != VEC_BOOL) return 0;
        t->col = ci;
        t->domain = VG_DOM_BOOL;
        t->lo = 0; t->hi = 0;
        t->kind = negate ? VG_TERM_RANGE : VG_TERM_NOT_RANGE;
        out->n_terms++;
        return 1;
    }
    case EXPR_IS_NA: {
        if (e->operand->kind != EXPR_COL_REF) return 0;
        int ty = -1;
        int ci = map(ctx, e->operand->col_name, &ty);
        if (ci < 0) return cerr("column not found: %s", e->operand->col_name);
        if (ty == VEC_STRING) return 0;
        t->col = ci;
        t->kind = negate ? VG_TERM_NOT_NA : VG_TERM_IS_NA;
        out->n_terms++;
        return 1;
    }
    case EXPR_CMP: {
        const VecExpr *c = e->left, *l = e->right;
        int code = cmp_code(e->op, e->op2);
        if (code < 0) return 0;
        if (c->kind != EXPR_COL_REF) {
            const VecExpr *x = c; c = l; l = x;
            code = flip_code(code);
        }
        if (c->kind != EXPR_COL_REF) return 0;
        if (l->kind == EXPR_LIT_NA) {
            int ty = -1;
            if (map(ctx, c->col_name, &ty) < 0) return cerr("column not found: %s", c->col_name);
            t->kind = VG_TERM_NONE; out->n_terms++; return 1;
        }
        if (!is_lit(l)) return 0;
        int ty = -1;
        int ci = map(ctx, c->col_name, &ty);
        if (ci < 0) return cerr("column not found: %s", c->col_name);
        if (ty == VEC_STRING) return 0;
        fold_term(ty, lit_type(l), l->kind == EXPR_LIT_BOOL ? (int64_t)(l->lit_bln != 0) : l->lit_i64,
                  l->lit_dbl, code, t);
        t->col = ci;
        if (negate) {   /* Kleene NOT keeps NA as NA */
            switch (t->kind) {
            case VG_TERM_RANGE: t->kind = VG_TERM_NOT_RANGE; break;
            case VG_TERM_NOT_RANGE: t->kind = VG_TERM_RANGE; break;
            case VG_TERM_NONE: t->kind = VG_TERM_NOT_NA; break;   /* !FALSE over valid rows */
            case VG_TERM_NOT_NA: t->kind = VG_TERM_NONE; break;
            default: return 0;
            }
            t->nan_keep = !t->nan_keep;
        }
        out->n_terms++;
        return 1;
    }
    default:
        return 0;
    }
}

int vg_compile_pred(const VecExpr *e, vg_colmap_fn map, void *ctx, VgPred *out) {
    memset(out, 0, sizeof(*out));
    g_cerr[0] = 0;
    int r = pred_rec(e, map, ctx, out, 0);
    if (r <= 0) memset(out, 0, sizeof(*out));
    return r;
}

/* ------------------------------------------------------------------ */
/* general programs                                                    */
/* ------------------------------------------------------------------ */

typedef struct {
    VgProg *p;
    int depth;
    vg_colmap_fn map;
    void *ctx;
} PC;

static int emit(PC *pc, int op, int a, int64_t imm, int push) {
    if (pc->p->n >= VG_MAX_INSNS) return cerr("expression too large for the GPU program%s", "");
    VgInsn *in = &pc->p->insn[pc->p->n++];
    in->op = op;
    in->a = a;
    in->imm = imm;
    pc->depth += push;
    if (pc->depth > pc->p->max_depth) pc->p->max_depth = pc->depth;
    if (pc->depth > 15) return cerr("expression too deep for the GPU program%s", "");
    return 0;
}

static int coerce_top(PC *pc, int from, int to) {
    if (from == to) return 0;
    if (to == VEC_DOUBLE) return emit(pc, VI_I2F, 0, 0, 0);   /* int64 / bool -> double */
    return 0;                                                /* bool -> int64: payload is 0/1 */
}

/* a string literal's bytes into the program's pool: its offset, or -1 */
static int64_t pool_add(PC *pc, const char *str, int *len) {
    const size_t n = str ? strlen(str) : 0;
    if ((size_t)pc->p->pool_n + n > VG_PROG_POOL)
        return cerr("string literals too long for the GPU program%s", "");
    memcpy(pc->p->pool + pc->p->pool_n, str ? str : "", n);
    const int64_t off = pc->p->pool_n;
    pc->p->pool_n += (int32_t)n;
    *len = (int)n;
    return off;
}

static int prog_rec(PC *pc, const VecExpr *e);

/* an argument that must be a string (nchar, substr, grepl) */
static int prog_string_arg(PC *pc, const VecExpr *e, const char *what) {
    int t = prog_rec(pc, e);
    if (t < 0) return -1;
    if (t != VEC_STRING) return cerr("%s: argument must be string", what);
    return 0;
}

/* substr's start / stop: int64 (a double is truncated toward zero, as the
 * reference's (int64_t) cast does, src/expr.c:186-193) */
static int prog_int_arg(PC *pc, const VecExpr *e) {
    int t = prog_rec(pc, e);
    if (t < 0) return -1;
    if (t == VEC_STRING) return cerr("substr: start and stop must be numeric%s", "");
    if (t == VEC_DOUBLE) return emit(pc, VI_F2I, 0, 0, 0);
    return 0;
}

/* returns the type of the value pushed, or -1 */
static int prog_rec(PC *pc, const VecExpr *e) {
    switch (e->kind) {
    case EXPR_COL_REF: {
        int ty = -1;
        int ci = pc->map(pc->ctx, e->col_name, &ty);
        if (ci < 0) return cerr("column not found: %s", e->col_name);
        if (ty == VEC_STRING) {
            if (emit(pc, VI_COL_STR, ci, 0, 1)) return -1;
            return VEC_STRING;
        }
        if (emit(pc, ty == VEC_DOUBLE ? VI_COL_F64 : ty == VEC_BOOL ? VI_COL_BOOL : VI_COL_I64, ci, 0, 1)) return -1;
        return ty;
    }
    case EXPR_LIT_STRING: {
        int len = 0;
        int64_t off = pool_add(pc, e->lit_str, &len);
        if (off < 0) return -1;
        if (emit(pc, VI_LIT_STR, len, off, 1)) return -1;
        return VEC_STRING;
    }
    case EXPR_NCHAR:   /* bytes of the string (src/expr.c:153-170) */
        if (prog_string_arg(pc, e->operand, "nchar")) return -1;
        if (emit(pc, VI_NCHAR, 0, 0, 0)) return -1;
        return VEC_INT64;
    case EXPR_SUBSTR:  /* src/expr.c:172-235 */
        if (prog_string_arg(pc, e->operand, "substr")) return -1;
        if (prog_int_arg(pc, e->left) || prog_int_arg(pc, e->right)) return -1;
        if (emit(pc, VI_SUBSTR, 0, 0, -2)) return -1;
        return VEC_STRING;
    case EXPR_GREPL: { /* fixed pattern (src/expr.c:237-268) */
        if (prog_string_arg(pc, e->operand, "grepl")) return -1;
        int len = 0;
        int64_t off = pool_add(pc, e->lit_str, &len);
        if (off < 0) return -1;
        if (emit(pc, VI_GREPL, len, off, 0)) return -1;
        return VEC_BOOL;
    }
    case EXPR_LIT_INT64:
        if (emit(pc, VI_LIT_I64, 0, e->lit_i64, 1)) return -1;
        return VEC_INT64;
    case EXPR_LIT_DOUBLE: {
        int64_t b;
        memcpy(&b, &e->lit_dbl, 8);
        if (emit(pc, VI_LIT_F64, 0, b, 1)) return -1;
        return VEC_DOUBLE;
    }
    case EXPR_LIT_BOOL:
        if (emit(pc, VI_LIT_BOOL, 0, e->lit_bln ? 1 : 0, 1)) return -1;
        return VEC_BOOL;
    case EXPR_LIT_NA:
        if (emit(pc, VI_LIT_NA, 0, 0, 1)) return -1;
        return e->result_type;
    case EXPR_ARITH: {
        int lt = type_of(e->left, pc->map, pc->ctx), rt = type_of(e->right, pc->map, pc->ctx);
        if (lt == -2 || rt == -2) return cerr("column not found%s", "");
        int c = common_type(lt, rt);
        if (c < 0 || lt == VEC_STRING || rt == VEC_STRING)
            return cerr("cannot coerce string in arithmetic/comparison%s", "");
        if (c == VEC_BOOL) c = VEC_INT64;
        if (prog_rec(pc, e->left) < 0 || coerce_top(pc, lt, c)) return -1;
        if (prog_rec(pc, e->right) < 0 || coerce_top(pc, rt, c)) return -1;
        if (e->op != '+' && e->op != '-' && e->op != '*' && e->op != '/' && e->op != '%')
            return cerr("unknown arith op%s", "");
        if (emit(pc, c == VEC_DOUBLE ? VI_ARITH_F64 : VI_ARITH_I64, e->op, 0, -1)) return -1;
        return c;
    }
    case EXPR_CMP: {
        int lt = type_of(e->left, pc->map, pc->ctx), rt = type_of(e->right, pc->map, pc->ctx);
        if (lt == -2 || rt == -2) return cerr("column not found%s", "");
        if (lt == VEC_STRING && rt == VEC_STRING) {   /* src/scalar_ops.c:78-107 */
            int code = cmp_code(e->op, e->op2);
            if (code < 0) return cerr("unknown comparison%s", "");
            if (prog_rec(pc, e->left) < 0 || prog_rec(pc, e->right) < 0) return -1;
            if (emit(pc, VI_CMP_STR, code, 0, -1)) return -1;
            return VEC_BOOL;
        }
        if (lt == VEC_STRING || rt == VEC_STRING)
            return cerr("cannot coerce string in arithmetic/comparison%s", "");
        int c = common_type(lt, rt);
        if (c == VEC_BOOL) c = VEC_INT64;
        int code = cmp_code(e->op, e->op2);
        if (code < 0) return cerr("unknown comparison%s", "");
        if (prog_rec(pc, e->left) < 0 || coerce_top(pc, lt, c)) return -1;
        if (prog_rec(pc, e->right) < 0 || coerce_top(pc, rt, c)) return -1;
        if (emit(pc, c == VEC_DOUBLE ? VI_CMP_F64 : VI_CMP_I64, code, 0, -1)) return -1;
        return VEC_BOOL;
    }
    case EXPR_BOOL: {
        if (e->op == '!') {
            int t = prog_rec(pc, e->operand);
            if (t < 0) return -1;
            if (t != VEC_BOOL) return cerr("bool not: operand must be boolean%s", "");
            if (emit(pc, VI_NOT, 0, 0, 0)) return -1;
            return VEC_BOOL;
        }
        int l = prog_rec(pc, e->left);
        if (l < 0) return -1;
        int r = prog_rec(pc, e->right);
        if (r < 0) return -1;
        if (l != VEC_BOOL || r != VEC_BOOL) return cerr("bool: operands must be boolean%s", "");
        if (emit(pc, e->op == '&' ? VI_AND : VI_OR, 0, 0, -1)) return -1;
        return VEC_BOOL;
    }
    case EXPR_IS_NA: {
        int t = prog_rec(pc, e->operand);
        if (t < 0) return -1;
        if (emit(pc, VI_IS_NA, 0, 0, 0)) return -1;
        return VEC_BOOL;
    }
    case EXPR_NEGATE: {
        int t = prog_rec(pc, e->operand);
        if (t < 0) return -1;
        if (t == VEC_INT64) { if (emit(pc, VI_NEG_I64, 0, 0, 0)) return -1; }
        else if (t == VEC_DOUBLE) { if (emit(pc, VI_NEG_F64, 0, 0, 0)) return -1; }
        else return cerr("negate: unsupported type%s", "");
        return t;
    }
    case EXPR_IF_ELSE:
    case EXPR_CAST:
        return cerr("if_else/cast not yet implemented%s", "");
    default:
        return cerr("unknown expression kind%s", "");
    }
}

int vg_compile_prog(const VecExpr *e, vg_colmap_fn map, void *ctx, VgProg *out) {
    memset(out, 0, sizeof(*out));
    g_cerr[0] = 0;
    PC pc = {out, 0, map, ctx};
    int t = prog_rec(&pc, e);
    if (t < 0) return -1;
    out->result_type = t;
    return 0;
}

/* ------------------------------------------------------------------ */
/* values for fused kernels                                            */
/* ------------------------------------------------------------------ */

static int operand_of(const VecExpr *e, vg_colmap_fn map, void *ctx, int side, VgOperand *o) {
    memset(o, 0, sizeof(*o));
    switch (e->kind) {
    case EXPR_COL_REF: {
        int ty = -1;
        int ci = map(ctx, e->col_name, &ty);
        if (ci < 0) return cerr("column not found: %s", e->col_name);
        if (ty == VEC_STRING) return 0;
        o->side = side;
        o->col = ci;
        o->type = ty;
        return 1;
    }
    case EXPR_LIT_INT64: o->side = VG_SIDE_LIT; o->type = VEC_INT64; o->lit = e->lit_i64; return 1;
    case EXPR_LIT_BOOL: o->side = VG_SIDE_LIT; o->type = VEC_BOOL; o->lit = e->lit_bln ? 1 : 0; return 1;
    case EXPR_LIT_DOUBLE: o->side = VG_SIDE_LIT; o->type = VEC_DOUBLE; memcpy(&o->lit, &e->lit_dbl, 8); return 1;
    case EXPR_LIT_NA: o->side = VG_SIDE_NA; o->type = e->result_type; return o->type != VEC_STRING;
    default: return 0;
    }
}

int vg_compile_value(const VecExpr *e, vg_colmap_fn map, void *ctx, int side, VgValue *out) {
    memset(out, 0, sizeof(*out));
    g_cerr[0] = 0;
    if (e->kind != EXPR_ARITH) {
        int r = operand_of(e, map, ctx, side, &out->a);
        if (r <= 0) return r;
        out->type = out->a.type;
        return 1;
    }
    int ra = operand_of(e->left, map, ctx, side, &out->a);
    if (ra <= 0) return ra;
    int rb = operand_of(e->right, map, ctx, side, &out->b);
    if (rb <= 0) return rb;
    int c = common_type(out->a.type, out->b.type);
    if (c < 0) return 0;
    if (c == VEC_BOOL) c = VEC_INT64;
    out->type = c;
    out->op = e->op;
    return 1;
}
