/*
 * node_join.c -- JoinNode on the GPU (replaces src/join.c).
 *
 * Same state machine as the reference (src/join.c:569-599): BUILD pulls the
 * whole right side (applying any sel, src/join.c:166-182) into device
 * columns and builds the hash table; PROBE turns each left batch into one
 * output batch (skipping empty ones); FINALIZE (FULL joins) emits the build
 * rows nothing matched, 65536 at a time (src/join.c:487-551).
 *
 * Keys are compared after the reference's coercion: the build key takes the
 * common type of both sides and the probe key is converted to it
 * (src/join.c:190-205, 270-293).  NA (and NaN) keys never match
 * (src/join.c:85).
 *
 * Output batches are host memory, columns ordered left ++ right non-key with
 * the reference's suffix rule; SEMI/ANTI return the probe batch itself with
 * a selection vector of the kept rows.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "vg_host.h"

typedef struct {
    JoinNodePrefix jn;        /* reference prefix: base, left, right, kind, n_keys, keys, suffixes */
    int state;                /* 0 build, 1 probe, 2 finalize, 3 done */
    int built;
    VgJoinBuilt B;
    int64_t n_build;
    int32_t key_type[VG_MAX_KEYS];
    int32_t conv_build[VG_MAX_KEYS];
    void *build_block;        /* device build columns */
    VgDBatch kept;            /* the one build batch, used in place */
    int has_kept;
    int slots_ready;          /* the slot table is filled (else derive it from pay) */
    VgJPay *pay;              /* payload copy requested by a fused aggregation */
    int pay_n;
    int32_t pay_col[2];
    void *table_block;        /* device hash table */
    int *r_nonkey;
    int r_nonkey_n;
    uint32_t *d_matched;      /* FULL: build rows matched so far */
    int32_t *d_unmatched;
    int64_t n_unmatched, fin_cursor;
    int64_t batch_idx;
    /* string keys: both sides' key strings as codes of one dictionary (the
     * build side's inserted, the probe side's looked up: a string the build
     * side does not hold gets -1 and matches nothing) */
    VgDict *dict;
    int str_key[VG_MAX_KEYS];
    VgCol bkey_codes[VG_MAX_KEYS];
    void *codes_block;
    /* build batches kept whole: the build columns' string views point into them */
    VgDBatch *bkeep;
    int bkeep_n;
} VgJoin;

static VecBatch *join_next(VecNode *self);

int vg_is_join(const VecNode *n) { return n && n->next_batch == join_next; }
VecNode *vg_join_left(VecNode *n) { return ((VgJoin *)n)->jn.left; }
int vg_join_kind(VecNode *n) { return ((VgJoin *)n)->jn.kind; }

int vg_join_resolve(VecNode *n, const char *name, int *side, int *col) {
    VgJoin *j = (VgJoin *)n;
    int i = vg_schema_find(&j->jn.base.output_schema, name);
    if (i < 0) return 0;
    int nl = j->jn.left->output_schema.n_cols;
    if (i < nl) { *side = 0; *col = i; }
    else { *side = 1; *col = j->r_nonkey[i - nl]; }
    return 1;
}

static int common_type(int a, int b) {
    if (a == b) return a;
    if (a == VEC_DOUBLE || b == VEC_DOUBLE) return VEC_DOUBLE;
    if (a == VEC_INT64 || b == VEC_INT64) return VEC_INT64;
    return VEC_BOOL;
}

static size_t a256(size_t x) { return (x + 255) & ~(size_t)255; }
static size_t elem(int t) { return t == VEC_BOOL ? 1 : t == VEC_STRING ? 16 : 8; }

int vg_join_has_string_keys(VecNode *n) {
    VgJoin *j = (VgJoin *)n;
    for (int k = 0; k < j->jn.n_keys; k++)
        if (j->str_key[k]) return 1;
    return 0;
}

/* a host string column of n NA rows */
static VecArray na_strings(int64_t n) {
    VecArray a;
    memset(&a, 0, sizeof(a));
    a.type = VEC_STRING;
    a.length = n;
    a.owns_data = 1;
    a.validity = (uint8_t *)vg_xcalloc((size_t)vg_vbytes(n) + 1, 1);
    a.buf.str.offsets = (int64_t *)vg_xcalloc((size_t)n + 1, 8);
    a.buf.str.data = (char *)vg_xcalloc(1, 1);
    return a;
}

/* n rows of a device column gathered by idx (-1: NA) to the host; dv/dm
 * hold 16 bytes and one validity bit per row */
static VecArray gather_down(const VgCol *src, const int32_t *idx, int64_t n, char *dv, uint32_t *dm) {
    vg_check_rc(vgk_gather(src, idx, n, 1, dv, dm, vg_stream()), "join gather");
    if (src->type != VEC_STRING) return vg_download_column(src->type, dv, dm, n);
    VgCol v;
    memset(&v, 0, sizeof(v));
    v.type = VEC_STRING;
    v.data = dv;
    v.valid = dm;
    return vg_download_strings(&v, NULL, n);
}

/* BUILD: materialise the right side on the device, then the hash table
 * (and, when a fused aggregation asked for it, the payload copy of up to
 * two right columns: pay_n / pay_col set before the build) */
static void join_build(VgJoin *j) {
    if (j->built) return;
    const VecSchema *rs = &j->jn.right->output_schema;
    int nr = rs->n_cols;
    uint8_t *need = (uint8_t *)vg_xcalloc((size_t)(nr ? nr : 1), 1);
    for (int k = 0; k < j->jn.n_keys; k++) need[j->jn.keys[k].right_col] = 1;
    for (int q = 0; q < j->r_nonkey_n; q++) need[j->r_nonkey[q]] = 1;
    int has_str = 0;
    for (int c = 0; c < nr; c++) has_str |= need[c] && rs->col_types[c] == VEC_STRING;
    /* pull every batch, keeping them on the device until the total is known */
    int cap = 16, nb = 0;
    VgDBatch *bs = (VgDBatch *)vg_xcalloc((size_t)cap, sizeof(VgDBatch));
    int64_t total = 0;
    for (;;) {
        if (nb == cap) {
            cap *= 2;
            bs = (VgDBatch *)realloc(bs, (size_t)cap * sizeof(VgDBatch));
            if (!bs) vg_fail("host allocation failed");
        }
        if (!vg_pull(j->jn.right, need, 0, &bs[nb])) break;
        total += bs[nb].d_sel ? bs[nb].sel_n : bs[nb].n_rows;
        nb++;
    }
    j->n_build = total;
    j->B.n_bcols = nr;
    j->B.bcols = (VgCol *)vg_xcalloc((size_t)(nr ? nr : 1), sizeof(VgCol));
    if (nb == 1 && !bs[0].d_sel && !bs[0].in_host) {
        /* one device batch without a selection: its columns are the build
         * columns as they are (kept until the node is freed) */
        for (int c = 0; c < nr; c++) {
            j->B.bcols[c].type = rs->col_types[c];
            if (need[c]) j->B.bcols[c] = bs[0].cols[c];
        }
        j->kept = bs[0];
        j->has_kept = 1;
        vg_dkeep(j->kept.block);   /* the node owns it now */
        nb = 0;
    }
    /* otherwise a dense device copy of the logical rows (one gather per batch) */
    size_t wbytes = (size_t)((total + 31) / 32) * 4 + 8;
    size_t bytes = 0;
    for (int c = 0; c < nr && !j->has_kept; c++)
        if (need[c]) bytes += a256((size_t)total * elem(rs->col_types[c]) + 8) + a256(wbytes);
    char *blk = j->has_kept ? NULL : (char *)vg_dmalloc_kept(bytes ? bytes : 256);
    j->build_block = blk;
    size_t off = 0;
    for (int c = 0; c < nr && !j->has_kept; c++) {
        j->B.bcols[c].type = rs->col_types[c];
        if (!need[c]) continue;
        char *dv = blk + off;
        off += a256((size_t)total * elem(rs->col_types[c]) + 8);
        uint32_t *dm = (uint32_t *)(blk + off);
        off += a256(wbytes);
        vg_dmemset(dm, 0, wbytes);
        int64_t at = 0;
        for (int b = 0; b < nb; b++) {
            int64_t n = bs[b].d_sel ? bs[b].sel_n : bs[b].n_rows;
            if (n == 0) continue;
            if ((at & 31) == 0)   /* word-aligned: whole validity words per warp */
                vg_check_rc(vgk_gather(&bs[b].cols[c], bs[b].d_sel, n, 0, dv + (size_t)at * elem(rs->col_types[c]),
                                       dm + at / 32, vg_stream()), "join build gather");
            else
                vg_check_rc(vgk_gather_into(&bs[b].cols[c], bs[b].d_sel, n, dv, dm, at, vg_stream()),
                            "join build gather");
            at += n;
        }
        j->B.bcols[c].data = dv;
        j->B.bcols[c].valid = dm;
    }
    if (has_str && nb > 0) {
        /* the gathered string views point into the batches' blocks */
        for (int b = 0; b < nb; b++) vg_dkeep(bs[b].block);
        j->bkeep = bs;
        j->bkeep_n = nb;
    } else {
        for (int b = 0; b < nb; b++) vg_dbatch_release(&bs[b]);
        free(bs);
    }
    free(need);

    /* string keys: the build key columns as dictionary codes */
    int n_skeys = 0;
    for (int k = 0; k < j->jn.n_keys; k++) n_skeys += j->str_key[k];
    if (n_skeys) {
        j->dict = vg_dict_new_kept();
        const size_t per = a256((size_t)(total > 0 ? total : 1) * 8);
        j->codes_block = vg_dmalloc_kept(per * (size_t)j->jn.n_keys);
        for (int k = 0; k < j->jn.n_keys; k++) {
            if (!j->str_key[k]) continue;
            const VgCol *sc = &j->B.bcols[j->jn.keys[k].right_col];
            int64_t *codes = (int64_t *)((char *)j->codes_block + per * (size_t)k);
            vg_dict_encode(j->dict, sc, NULL, total, 1, codes, -1);
            j->bkey_codes[k] = *sc;
            j->bkey_codes[k].type = VEC_INT64;
            j->bkey_codes[k].data = codes;
        }
    }

    /* hash table, or a direct-addressed one when the only key is an int64
     * column whose values span at most twice the build rows (dense ids) */
    int nk = j->jn.n_keys;
    VgCol kc[VG_MAX_KEYS];
    for (int k = 0; k < nk; k++) kc[k] = j->str_key[k] ? j->bkey_codes[k] : j->B.bcols[j->jn.keys[k].right_col];
    int direct = 0;
    int64_t dmin = 0, drange = 0;
    if (nk == 1 && j->key_type[0] == VEC_INT64 && kc[0].type == VEC_INT64 && total > 0) {
        int64_t mm[3];
        int64_t *d = (int64_t *)vg_dmalloc(256);
        vg_check_rc(vgk_col_minmax_i64(&kc[0], total, d, mm, vg_stream()), "join key range");
        vg_dfree(d);
        uint64_t limit = (uint64_t)(2 * total > 65536 ? 2 * total : 65536);
        if (mm[2] > 0 && (uint64_t)mm[1] - (uint64_t)mm[0] < limit) {
            direct = 1;
            dmin = mm[0];
            drange = (int64_t)((uint64_t)mm[1] - (uint64_t)mm[0]) + 1;
        }
    }
    int64_t tcap = direct ? drange : vgk_join_cap(total);
    size_t rows_b = a256((size_t)(total > 0 ? total : 1) * 4);
    size_t tb = (nk == 1) ? a256((size_t)(tcap + 1) * sizeof(VgJSlot)) + rows_b + 256
                          : a256((size_t)tcap * 4) * 3 + a256((size_t)tcap * 8 * (size_t)nk) + rows_b + 256;
    char *t = (char *)vg_dmalloc_kept(tb);
    j->table_block = t;
    VgJoinTable *jt = &j->B.jt;
    memset(jt, 0, sizeof(*jt));
    jt->cap = tcap;
    jt->direct = direct;
    jt->dmin = dmin;
    jt->n_keys = nk;
    for (int k = 0; k < nk; k++) jt->key_types[k] = j->key_type[k];
    size_t o = 0;
    if (nk == 1) {
        /* one 16-byte {key, start, count} slot per key, claimed lock-free */
        jt->slots = (VgJSlot *)(t + o); o += a256((size_t)(tcap + 1) * sizeof(VgJSlot));
    } else {
        jt->state = (uint32_t *)(t + o); o += a256((size_t)tcap * 4);
        jt->start = (int32_t *)(t + o); o += a256((size_t)tcap * 4);
        jt->count = (int32_t *)(t + o); o += a256((size_t)tcap * 4);
        jt->keys = (uint64_t *)(t + o); o += a256((size_t)tcap * 8 * (size_t)nk);
    }
    jt->rows = (int32_t *)(t + o); o += rows_b;
    jt->err = (uint32_t *)(t + o);
    jt->n_build = total;
    VgCol pc[2];
    memset(pc, 0, sizeof(pc));
    if (j->pay_n > 0 && nk == 1) {
        for (int q = 0; q < j->pay_n; q++) pc[q] = j->B.bcols[j->pay_col[q]];
        j->pay = (VgJPay *)vg_dmalloc_kept((size_t)(tcap + 1) * sizeof(VgJPay));
    }
    size_t sb = vgk_join_build_scratch_bytes(total);
    void *scratch = vg_dmalloc(sb);
    int64_t distinct = 0, maxdup = 0;
    j->B.pay_layout = -2;
    int rc = vgk_join_build(jt, kc, nk, j->conv_build, total, scratch, sb, &distinct, &maxdup, pc,
                            j->pay ? j->pay_n : 0, j->pay, j->B.pay_mm, &j->B.pay_layout, &j->B.pay_min,
                            &j->slots_ready, vg_stream());
    if (j->pay) {
        j->B.pay_n = j->pay_n;
        for (int q = 0; q < j->pay_n; q++) j->B.pay_col[q] = j->pay_col[q];
        j->B.pay_mm_ok = jt->direct;   /* the claim pass computed them */
    }
    vg_dfree(scratch);
    vg_check_rc(rc, "join build");
    if (j->jn.kind == JOIN_FULL) {
        size_t mb = (size_t)((total + 31) / 32) * 4 + 8;
        j->d_matched = (uint32_t *)vg_dmalloc_kept(mb);
        vg_dmemset(j->d_matched, 0, mb);
    }
    j->built = 1;
}

const VgJoinBuilt *vg_join_build_now(VecNode *n) {
    VgJoin *j = (VgJoin *)n;
    join_build(j);
    return &j->B;
}

const VgJoinBuilt *vg_join_build_payload(VecNode *n, const int32_t *cols, int n_cols, const VgJPay **pay) {
    VgJoin *j = (VgJoin *)n;
    *pay = NULL;
    if (!j->built && n_cols >= 1 && n_cols <= 2) {
        j->pay_n = n_cols;
        for (int q = 0; q < n_cols; q++) j->pay_col[q] = cols[q];
    }
    join_build(j);
    /* usable only for unique single keys built with the same columns */
    if (j->pay && !j->B.jt.rows && j->pay_n == n_cols &&
        (n_cols < 1 || j->pay_col[0] == cols[0]) && (n_cols < 2 || j->pay_col[1] == cols[1]))
        *pay = j->pay;
    return &j->B;
}

void vg_join_ensure_slots(VecNode *n) {
    VgJoin *j = (VgJoin *)n;
    join_build(j);
    if (j->slots_ready) return;
    if (j->B.pay_layout == -2) {
        vg_check_rc(vgk_join_slots_from_payload(&j->B.jt, j->pay, vg_stream()), "join slots");
    } else {
        /* compact entries hold neither keys nor build rows: the slots come
         * from the key column */
        void *scratch = vg_dmalloc((size_t)(j->B.jt.n_build > 0 ? j->B.jt.n_build : 1) * 4 + 256);
        const VgCol kc = j->str_key[0] ? j->bkey_codes[0] : j->B.bcols[j->jn.keys[0].right_col];
        const int rc = vgk_join_slots_from_keys(&j->B.jt, &kc, j->conv_build[0], j->B.jt.n_build, scratch,
                                                vg_stream());
        vg_dfree(scratch);
        vg_check_rc(rc, "join slots");
    }
    j->slots_ready = 1;
}

int vg_join_right_type(VecNode *n, int col) {
    VgJoin *j = (VgJoin *)n;
    return j->jn.right->output_schema.col_types[col];
}

/* one probe batch -> one output batch (NULL if empty) */
static VecBatch *probe_one(VgJoin *j) {
    vg_join_ensure_slots(&j->jn.base);
    const VecSchema *ls = &j->jn.left->output_schema;
    int nl = ls->n_cols, nk = j->jn.n_keys;
    int semi = (j->jn.kind == JOIN_SEMI || j->jn.kind == JOIN_ANTI);
    uint8_t *need = (uint8_t *)vg_xcalloc((size_t)(nl ? nl : 1), 1);
    for (int k = 0; k < nk; k++) need[j->jn.keys[k].left_col] = 1;
    if (!semi)
        for (int c = 0; c < nl; c++) need[c] = 1;
    for (;;) {
        VgDBatch db;
        if (!vg_pull(j->jn.left, need, semi, &db)) { free(need); return NULL; }
        j->batch_idx++;
        int64_t n = db.d_sel ? db.sel_n : db.n_rows;
        VgCol pk[VG_MAX_KEYS];
        for (int k = 0; k < nk; k++) pk[k] = db.cols[j->jn.keys[k].left_col];
        /* string keys: the probe strings' codes (looked up, not inserted) */
        char *pcodes = NULL;
        if (j->dict) {
            const size_t per = a256((size_t)(db.n_rows > 0 ? db.n_rows : 1) * 8);
            pcodes = (char *)vg_dmalloc(per * (size_t)nk);
            for (int k = 0; k < nk; k++) {
                if (!j->str_key[k]) continue;
                int64_t *codes = (int64_t *)(pcodes + per * (size_t)k);
                vg_dict_encode(j->dict, &pk[k], db.d_sel, n, 0, codes, -1);
                pk[k].type = VEC_INT64;
                pk[k].data = codes;
            }
        }
        size_t sb = vgk_join_probe_scratch_bytes(n);
        void *scratch = vg_dmalloc(sb);
        int64_t total = 0;
        int rc = vgk_join_probe_count(&j->B.jt, pk, nk, j->B.conv, db.n_rows, db.d_sel, db.sel_n,
                                      j->jn.kind, scratch, sb, &total, vg_stream());
        if (rc) { vg_dfree(scratch); vg_dbatch_release(&db); vg_check_rc(rc, "join probe"); }
        if (total == 0) { vg_dfree(scratch); vg_dfree(pcodes); vg_dbatch_release(&db); continue; }
        int32_t *pairs = (int32_t *)vg_dmalloc((size_t)total * 8 + 16);
        int32_t *op = pairs, *ob = semi ? NULL : pairs + total;
        rc = vgk_join_probe_emit(&j->B.jt, db.n_rows, db.d_sel, db.sel_n, j->jn.kind, scratch, sb, op, ob,
                                 j->d_matched, vg_stream());
        vg_dfree(scratch);
        if (rc) { vg_dfree(pairs); vg_dbatch_release(&db); vg_check_rc(rc, "join emit"); }
        VecBatch *out;
        if (semi) {
            /* the probe batch itself, with the kept rows as its selection */
            out = db.host;
            int32_t *sel = (int32_t *)vg_xmalloc((size_t)total * 4);
            vg_d2h(sel, op, (size_t)total * 4);
            vg_sync();
            free(out->sel);
            out->sel = sel;
            out->sel_n = (int32_t)total;
            db.host = NULL;
        } else {
            int oc = j->jn.base.output_schema.n_cols;
            out = vg_batch_alloc(oc, total);
            size_t wb = (size_t)((total + 31) / 32) * 4;
            size_t per = a256((size_t)total * 16) + a256(wb);
            char *blk = (char *)vg_dmalloc(per * (size_t)oc + 256);
            for (int c = 0; c < oc; c++) {
                char *dv = blk + per * (size_t)c;
                uint32_t *dm = (uint32_t *)(dv + a256((size_t)total * 16));
                const VgCol *src;
                const int32_t *idx;
                if (c < nl) { src = &db.cols[c]; idx = op; }
                else { src = &j->B.bcols[j->r_nonkey[c - nl]]; idx = ob; }
                out->columns[c] = gather_down(src, idx, total, dv, dm);
                out->col_names[c] = vg_xstrdup(j->jn.base.output_schema.col_names[c]);
            }
            vg_sync();
            vg_dfree(blk);
        }
        vg_dfree(pairs);
        vg_dfree(pcodes);
        vg_dbatch_release(&db);
        free(need);
        return out;
    }
}

static VecBatch *finalize_one(VgJoin *j) {
    if (!j->d_unmatched) {
        j->d_unmatched = (int32_t *)vg_dmalloc_kept((size_t)(j->n_build > 0 ? j->n_build : 1) * 4);
        size_t sb = vgk_join_probe_scratch_bytes(j->n_build);
        void *scratch = vg_dmalloc(sb);
        int rc = vgk_join_unmatched_build(j->d_matched, j->n_build, j->d_unmatched, &j->n_unmatched, scratch, sb,
                                          vg_stream());
        vg_dfree(scratch);
        vg_check_rc(rc, "join finalize");
        j->fin_cursor = 0;
    }
    int64_t left = j->n_unmatched - j->fin_cursor;
    if (left <= 0) return NULL;
    int64_t n = left < 65536 ? left : 65536;
    const int32_t *idx = j->d_unmatched + j->fin_cursor;
    j->fin_cursor += n;
    const VecSchema *ls = &j->jn.left->output_schema;
    int nl = ls->n_cols, oc = j->jn.base.output_schema.n_cols;
    VecBatch *out = vg_batch_alloc(oc, n);
    size_t wb = (size_t)((n + 31) / 32) * 4;
    size_t per = a256((size_t)n * 16) + a256(wb);
    char *blk = (char *)vg_dmalloc(per * (size_t)oc + 256);
    for (int c = 0; c < oc; c++) {
        char *dv = blk + per * (size_t)c;
        uint32_t *dm = (uint32_t *)(dv + a256((size_t)n * 16));
        out->col_names[c] = vg_xstrdup(j->jn.base.output_schema.col_names[c]);
        if (c < nl) {
            int rk = -1;
            for (int k = 0; k < j->jn.n_keys; k++)
                if (j->jn.keys[k].left_col == c) { rk = j->jn.keys[k].right_col; break; }
            if (rk < 0 && ls->col_types[c] == VEC_STRING) {
                out->columns[c] = na_strings(n);
                continue;
            }
            if (rk < 0) {   /* non-key left column: NA */
                VecArray a;
                memset(&a, 0, sizeof(a));
                a.type = ls->col_types[c];
                a.length = n;
                a.owns_data = 1;
                a.validity = (uint8_t *)vg_xcalloc((size_t)vg_vbytes(n), 1);
                a.buf.i64 = (int64_t *)vg_xcalloc((size_t)n * elem(a.type) + 1, 1);
                out->columns[c] = a;
                continue;
            }
            if (j->B.bcols[rk].type == VEC_STRING) {
                out->columns[c] = gather_down(&j->B.bcols[rk], idx, n, dv, dm);
                continue;
            }
            vg_check_rc(vgk_gather(&j->B.bcols[rk], idx, n, 0, dv, dm, vg_stream()), "join finalize gather");
            out->columns[c] = vg_download_column(ls->col_types[c], dv, dm, n);
        } else {
            out->columns[c] = gather_down(&j->B.bcols[j->r_nonkey[c - nl]], idx, n, dv, dm);
        }
    }
    vg_sync();
    vg_dfree(blk);
    return out;
}

static VecBatch *join_next_body(VecNode *self) {
    VgJoin *j = (VgJoin *)self;
    if (j->state == 0) { join_build(j); j->state = 1; }
    if (j->state == 1) {
        VecBatch *b = probe_one(j);
        if (b) return b;
        j->state = (j->jn.kind == JOIN_FULL) ? 2 : 3;
    }
    if (j->state == 2) {
        VecBatch *b = finalize_one(j);
        if (b) return b;
        j->state = 3;
    }
    return NULL;
}

/* one node API call: its temporary device memory is released if it fails */
static VecBatch *join_next(VecNode *self) {
    vg_scope_enter();
    VecBatch *b = join_next_body(self);
    vg_scope_leave();
    return b;
}

static void join_free(VecNode *self) {
    VgJoin *j = (VgJoin *)self;
    j->jn.left->free_node(j->jn.left);
    j->jn.right->free_node(j->jn.right);
    free(j->jn.keys);
    free(j->jn.suffix_x);
    free(j->jn.suffix_y);
    free(j->r_nonkey);
    free(j->B.bcols);
    vg_dfree(j->build_block);
    if (j->has_kept) vg_dbatch_release(&j->kept);
    vg_dfree(j->pay);
    vg_dfree(j->table_block);
    vg_dfree(j->d_matched);
    vg_dfree(j->d_unmatched);
    vg_dict_free(j->dict);
    vg_dfree(j->codes_block);
    for (int b = 0; b < j->bkeep_n; b++) vg_dbatch_release(&j->bkeep[b]);
    free(j->bkeep);
    vg_schema_free(&j->jn.base.output_schema);
    free(j);
}

static const char *type_name(int t) {
    switch (t) {
    case VEC_INT64: return "int64";
    case VEC_DOUBLE: return "double";
    case VEC_BOOL: return "bool";
    default: return "string";
    }
}

JoinNode *join_node_create(VecNode *left, VecNode *right, JoinKind kind, int n_keys, JoinKey *keys,
                           const char *suffix_x, const char *suffix_y) {
    static const char *kind_names[] = {"inner_join", "left_join", "full_join", "semi_join", "anti_join"};
    const VecSchema *ls = &left->output_schema, *rs = &right->output_schema;
    if (n_keys < 1 || n_keys > VG_MAX_KEYS) vg_fail("GPU join supports 1 to %d key columns", VG_MAX_KEYS);
    for (int k = 0; k < n_keys; k++) {
        int lt = ls->col_types[keys[k].left_col], rt = rs->col_types[keys[k].right_col];
        if (lt != rt && (lt == VEC_STRING || rt == VEC_STRING))
            vg_fail("%s key type mismatch: x.%s (%s) vs y.%s (%s)", kind_names[kind],
                    ls->col_names[keys[k].left_col], type_name(lt), rs->col_names[keys[k].right_col],
                    type_name(rt));
        if (kind == JOIN_FULL && lt != rt)
            vg_fail("full_join with key columns of different types (x.%s %s, y.%s %s) is not supported by the GPU join",
                    ls->col_names[keys[k].left_col], type_name(lt), rs->col_names[keys[k].right_col], type_name(rt));
    }
    VgJoin *j = (VgJoin *)vg_xcalloc(1, sizeof(VgJoin));
    j->jn.left = left;
    j->jn.right = right;
    j->jn.kind = kind;
    j->jn.n_keys = n_keys;
    j->jn.keys = keys;
    j->jn.suffix_x = vg_xstrdup(suffix_x);
    j->jn.suffix_y = vg_xstrdup(suffix_y);
    j->B.n_keys = n_keys;
    j->B.kind = kind;
    for (int k = 0; k < n_keys; k++) {
        int lt = ls->col_types[keys[k].left_col], rt = rs->col_types[keys[k].right_col];
        int c = common_type(lt, rt);
        if (lt == VEC_STRING) {   /* both strings: joined on dictionary codes */
            j->str_key[k] = 1;
            c = VEC_INT64;
        }
        j->key_type[k] = c;
        j->conv_build[k] = (rt != c && c == VEC_DOUBLE);
        j->B.conv[k] = (lt != c && c == VEC_DOUBLE);
        j->B.lkey[k] = keys[k].left_col;
        j->B.rkey[k] = keys[k].right_col;
    }
    /* output schema (src/join.c:703-784) */
    int *is_rkey = (int *)vg_xcalloc((size_t)(rs->n_cols ? rs->n_cols : 1), sizeof(int));
    for (int k = 0; k < n_keys; k++) is_rkey[keys[k].right_col] = 1;
    j->r_nonkey = (int *)vg_xcalloc((size_t)(rs->n_cols ? rs->n_cols : 1), sizeof(int));
    if (kind == JOIN_INNER || kind == JOIN_LEFT || kind == JOIN_FULL)
        for (int c = 0; c < rs->n_cols; c++)
            if (!is_rkey[c]) j->r_nonkey[j->r_nonkey_n++] = c;
    int on = ls->n_cols + j->r_nonkey_n;
    char **names = (char **)vg_xcalloc((size_t)(on ? on : 1), sizeof(char *));
    VecType *types = (VecType *)vg_xcalloc((size_t)(on ? on : 1), sizeof(VecType));
    for (int i = 0; i < ls->n_cols; i++) { names[i] = vg_xstrdup(ls->col_names[i]); types[i] = ls->col_types[i]; }
    for (int q = 0; q < j->r_nonkey_n; q++) {
        int c = j->r_nonkey[q];
        const char *rn = rs->col_names[c];
        int coll = vg_schema_find(ls, rn);
        if (coll >= 0) {
            size_t l1 = strlen(rn) + strlen(suffix_y) + 1;
            names[ls->n_cols + q] = (char *)vg_xmalloc(l1);
            snprintf(names[ls->n_cols + q], l1, "%s%s", rn, suffix_y);
            size_t l2 = strlen(ls->col_names[coll]) + strlen(suffix_x) + 1;
            free(names[coll]);
            names[coll] = (char *)vg_xmalloc(l2);
            snprintf(names[coll], l2, "%s%s", ls->col_names[coll], suffix_x);
        } else {
            names[ls->n_cols + q] = vg_xstrdup(rn);
        }
        types[ls->n_cols + q] = rs->col_types[c];
    }
    j->jn.base.output_schema = vg_schema_make(on, names, types);
    for (int i = 0; i < on; i++) free(names[i]);
    free(names);
    free(types);
    free(is_rkey);
    j->jn.base.next_batch = join_next;
    j->jn.base.free_node = join_free;
    j->jn.base.kind = "JoinNode";
    return (JoinNode *)&j->jn;
}
